"""Builds the Python extension over the C++17 host API (added with the host
API headers)."""


def build_bindings(verbose: bool = False) -> None:
    return None
