"""Tensor-network files (reference: include/jet/TensorNetworkIO.hpp:67-293,
python/src/TensorNetworkIO.hpp).

JSON layout:
    {"path": [[i, j], ...],            # optional
     "tensors": [[tags, indices, shape, [[re, im], ...]], ...]}
Data are row-major; with col_major=True the indices and shape of every
tensor are reversed on load, as the reference does for files written from
column-major tensors. Loading builds the GPU TensorNetwork directly, so the
reference's benchmark networks (m10.json / m12.json) load straight into
device memory.
"""
from __future__ import annotations

import json
from typing import Optional

import numpy as np

from . import factory
from ._jet_bindings import PathInfo


class TensorFileException(Exception):
    """Invalid tensor-network file (TensorNetworkIO.hpp:37-53)."""


class TensorNetworkFile:
    """A loaded network and its optional contraction path."""

    def __init__(self, tensors=None, path: Optional[PathInfo] = None, dtype="complex128"):
        self.tensors = tensors if tensors is not None else factory.TensorNetwork(dtype=dtype)
        self.path = path


class TensorNetworkSerializer:
    """Callable (de)serializer: (tn[, path]) -> str, (str[, col_major]) -> TensorNetworkFile."""

    def __init__(self, indent: int = -1, dtype="complex128"):
        self.indent = indent
        self.dtype = np.dtype(dtype)

    def __call__(self, *args, **kwargs):
        if args and isinstance(args[0], str):
            return self._load(*args, **kwargs)
        return self._dump(*args, **kwargs)

    def _dump(self, tn, path: Optional[PathInfo] = None) -> str:
        js = {}
        if path is not None:
            js["path"] = [list(p) for p in path.path]
        tensors = []
        for node in tn.nodes:
            t = node.tensor
            tensors.append([list(node.tags), list(t.indices), list(t.shape),
                            [[float(np.real(x)), float(np.imag(x))] for x in t.data]])
        js["tensors"] = tensors
        if self.indent is None or self.indent < 0:
            return json.dumps(js, sort_keys=True, separators=(",", ":"))
        return json.dumps(js, sort_keys=True, indent=self.indent)

    def _load(self, js_str: str, col_major: bool = False) -> TensorNetworkFile:
        js = json.loads(js_str)
        if not isinstance(js, dict):
            raise TensorFileException("root element must be an object.")
        if "tensors" not in js:
            raise TensorFileException("root object must contain 'tensors' key")
        tn = factory.TensorNetwork(dtype=self.dtype)
        for i, entry in enumerate(js["tensors"]):
            tags, indices, shape, raw = entry[0], entry[1], entry[2], entry[3]
            data = []
            for j, x in enumerate(raw):
                try:
                    data.append(complex(float(x[0]), float(x[1])))
                except (TypeError, ValueError, IndexError):
                    raise TensorFileException(
                        "Invalid element at index %d of tensor %d: Could not parse %s as "
                        "complex." % (j, i, json.dumps(x)))
            if col_major:
                indices, shape = list(reversed(indices)), list(reversed(shape))
            tn.add_tensor(factory.Tensor(indices=list(indices), shape=[int(s) for s in shape],
                                         data=data, dtype=self.dtype), list(tags))
        path = PathInfo(tn, [tuple(p) for p in js["path"]]) if "path" in js else None
        return TensorNetworkFile(tn, path)


def load(filename: str, dtype="complex64", col_major: bool = False) -> TensorNetworkFile:
    with open(filename) as f:
        return TensorNetworkSerializer(dtype=dtype)(f.read(), col_major)
