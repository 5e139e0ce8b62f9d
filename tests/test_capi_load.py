"""The C-ABI library loads on the host and exports every declared entry point;
argument validation happens on the host before any device work."""
import ctypes

import pytest


def test_library_exports_every_declared_symbol():
    from jet_gb300 import capi

    declared = capi.declared_symbols()
    assert len(declared) >= 14
    missing = [s for s in declared if not hasattr(capi.lib, s)]
    assert missing == []


def test_version():
    from jet_gb300 import capi

    assert capi.lib.jetgpu_version() == 1


@pytest.mark.parametrize("perm", [[0, 0, 1], [0, 1, 3], [2, 1, -1]])
def test_permute_rejects_bad_permutation(perm):
    from jet_gb300 import capi

    shape = [2, 2, 2]
    rc = capi.lib.jetgpu_permute(None, None, 3, capi.u64(shape), capi.i32(perm), capi.C64, None)
    assert rc == capi.ERR_INVALID
    assert b"permutation" in capi.lib.jetgpu_last_error()


def test_contract_rejects_inconsistent_sizes():
    from jet_gb300 import capi

    rc = capi.lib.jetgpu_contract(None, 2, capi.u64([2, 2]), capi.i32([0, 1]), None, 2,
                                  capi.u64([2, 2]), capi.i32([0, 1]), None, 4, 2, 2,
                                  capi.C64, capi.PREC_FP32, capi.ALGO_4M, 0, 0, None, 0, None)
    assert rc == capi.ERR_INVALID
    assert b"size does not match" in capi.lib.jetgpu_last_error()


def test_contract_rejects_tf32_for_complex128():
    from jet_gb300 import capi

    rc = capi.lib.jetgpu_contract(None, 1, capi.u64([2]), capi.i32([0]), None, 1,
                                  capi.u64([2]), capi.i32([0]), None, 1, 1, 2, capi.C128,
                                  capi.PREC_TF32X3, capi.ALGO_4M, 0, 0, None, 0, None)
    assert rc == capi.ERR_UNSUPPORTED


@pytest.mark.parametrize("depth", [-1, 4097])
def test_chunk_depth_rejects_out_of_range(depth):
    from jet_gb300 import capi

    assert capi.lib.jetgpu_set_tc_chunk_depth(depth) == capi.ERR_INVALID
    assert b"chunk depth" in capi.lib.jetgpu_last_error()
    assert capi.lib.jetgpu_set_tc_chunk_depth(0) == capi.OK
