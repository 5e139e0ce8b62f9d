"""The Permuter<Backend> front-end (permute/Permuter.hpp:36-126): its
validation runs on the host before any device work, with the reference's
messages (Test_Permuter.cpp:344-456). The GPU-backed transposes of the
golden vectors are in test_permuter_api_gpu below."""
import numpy as np
import pytest

import jet_gb300._jet_bindings as b

X30 = [complex(i, i) for i in range(30)]


@pytest.mark.parametrize("shape,old,new,msg", [
    ([2, 3, 5, 2], "cab", "abc", "Tensor shape does not match number of indices."),
    ([2, 3, 5, 2], "cabd", "abcd", "Tensor shape does not match given tensor data."),
    ([2, 3, 5], "abb", "abc", "Duplicate existing indices found"),
    ([2, 3, 5], "abc", "abb", "Duplicate transpose indices found"),
    ([2, 3, 5], "abc", "abd", "New indices are an invalid permutation"),
    ([], "", "", "Tensor shape does not match given tensor data"),
])
def test_permuter_messages(shape, old, new, msg):
    with pytest.raises(RuntimeError, match=msg):
        b.permuter_transpose(X30, shape, list(old), list(new))


@pytest.mark.gpu
def test_permuter_golden_vectors_gpu(cuda, golden):
    for c in golden["permuter"]["cases"]:
        x = [complex(a, bb) for a, bb in c["input"]]
        got = b.permuter_transpose(x, c["shape"], c["old"], c["new"])
        assert got == [complex(a, bb) for a, bb in c["expected"]], c["source"]
