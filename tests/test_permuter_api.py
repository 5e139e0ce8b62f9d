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


@pytest.mark.parametrize("shape,old", [([3, 5, 2], "bca"), ([5, 3, 2], "cba"), ([5, 2, 3], "cab")])
def test_qflex_rejects_non_power_of_2(shape, old):
    """Test_Permuter.cpp:344-387: QFlexPermuter plans binary indices only."""
    with pytest.raises(RuntimeError, match="Fast transpose expects power-of-2 data"):
        b.permuter_transpose(X30, shape, list(old), list("abc"), backend="qflex")


def test_qflex_insufficient_blocksize(golden):
    """Test_Permuter.cpp:492-519: the 9-index example needs a larger BLOCKSIZE
    than 64 in the reference's three-pass plan; QFlexPermuter<64> rejects it
    with the reference's message, before any device work."""
    c = [c for c in golden["permuter"]["cases"] if c["source"].endswith("large_example")][0]
    x = [complex(a, bb) for a, bb in c["input"]]
    with pytest.raises(RuntimeError, match="Consider increasing the BLOCKSIZE"):
        b.permuter_transpose(x, c["shape"], c["old"], c["new"], backend="qflex64")


def test_unknown_backend():
    with pytest.raises(ValueError, match="backend"):
        b.permuter_transpose(X30, [2, 3, 5], list("abc"), list("cba"), backend="nope")


@pytest.mark.gpu
def test_permuter_golden_vectors_gpu(cuda, golden):
    """Every golden transpose through DefaultPermuter, and the power-of-2 ones
    through QFlexPermuter (including the 9-index example that QFlexPermuter<>
    plans and QFlexPermuter<64> rejects)."""
    for c in golden["permuter"]["cases"]:
        x = [complex(a, bb) for a, bb in c["input"]]
        want = [complex(a, bb) for a, bb in c["expected"]]
        assert b.permuter_transpose(x, c["shape"], c["old"], c["new"], backend="default") == want
        if all(d & (d - 1) == 0 for d in c["shape"]):
            got = b.permuter_transpose(x, c["shape"], c["old"], c["new"], backend="qflex")
            assert got == want, c["source"]


def test_qflex_plan_decisions_match_reference(golden):
    """QFlexPermuter<BLOCKSIZE, MIN_DIMS> accepts and rejects exactly what the
    compiled reference's plan does, on 160 seeded power-of-2 transposes for
    seven instantiations (tests/golden/qflex_plans.json), with the same
    message."""
    n_reject = 0
    for c in golden["qflex_plans"]:
        for key, decision in c["decisions"].items():
            block, min_dims = (int(v) for v in key.split(","))
            if decision is True:
                b.qflex_check_plan(c["shape"], c["old"], c["new"], block, min_dims)
            else:
                n_reject += 1
                with pytest.raises(RuntimeError) as e:
                    b.qflex_check_plan(c["shape"], c["old"], c["new"], block, min_dims)
                assert decision in str(e.value), (c["case"], key)
    assert n_reject > 100


@pytest.mark.gpu
def test_qflex_accepted_transposes_bit_exact_gpu(cuda, golden):
    """Accepted fixture transposes through Permuter<QFlexPermuter<>> on the GPU
    equal the reference's output bit for bit (SHA-256 of the bytes)."""
    import hashlib

    import cases

    for c in golden["qflex_plans"][:40]:
        n = int(np.prod(c["shape"]))
        x = cases.tensor_data(c["seed"], [n], np.complex64)
        got = np.array(b.permuter_transpose(list(x), c["shape"], c["old"], c["new"]),
                       dtype=np.complex64)
        assert hashlib.sha256(got.tobytes()).hexdigest() == c["sha256"], c["case"]
