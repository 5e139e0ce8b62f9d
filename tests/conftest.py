import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def pytest_sessionstart(session):
    """Builds the native libraries (nvcc cross-compiles without a GPU) when a
    fresh checkout runs the tests before build()."""
    import glob
    import importlib.util

    pkg = os.path.join(REPO, "jet_gb300")
    if os.path.exists(os.path.join(pkg, "libjetgpu.so")) and glob.glob(
            os.path.join(pkg, "_jet_bindings*.so")):
        return
    spec = importlib.util.spec_from_file_location("jet_gb300_build",
                                                  os.path.join(pkg, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build_all()


@pytest.fixture(scope="session")
def cuda():
    """The CUDA device for `gpu` tests; the native library must load."""
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import jet_gb300.capi  # noqa: F401  (fails loudly when the library is missing)

    return torch.device("cuda:0")


@pytest.fixture(scope="session")
def golden():
    import json

    d = os.path.join(REPO, "tests", "golden")
    with open(os.path.join(d, "permuter_vectors.json")) as f:
        perm = json.load(f)
    with open(os.path.join(d, "ref_cases.json")) as f:
        cases = json.load(f)
    with open(os.path.join(d, "qflex_plans.json")) as f:
        qflex = json.load(f)
    return {"permuter": perm, "ref": cases, "qflex_plans": qflex}
