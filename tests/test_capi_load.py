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


@pytest.mark.parametrize("form,ok", [(1, True), (3, True), (4, True), (0, False), (2, False),
                                     (5, False)])
def test_auto_form_accepts_split_forms_only(form, ok):
    from jet_gb300 import capi

    rc = capi.lib.jetgpu_set_auto_form(form)
    try:
        if ok:
            assert rc == capi.OK
        else:
            assert rc == capi.ERR_INVALID
            assert b"AUTO form" in capi.lib.jetgpu_last_error()
    finally:
        capi.lib.jetgpu_set_auto_form(capi.PREC_FP16X3)


def test_split_forms_need_complex64_and_fp16_scale_range():
    """Host-side checks of jetgpu_contract before any device work: the split
    forms reject complex128, FP16x3 rejects |scale_a + scale_b| > 126."""
    from jet_gb300 import capi

    sh = capi.u64([256, 256])
    pm = capi.i32([0, 1])
    for prec in (capi.PREC_TF32X3, capi.PREC_BF16X3, capi.PREC_FP16X3):
        rc = capi.lib.jetgpu_contract(None, 2, sh, pm, None, 2, sh, pm, None, 256, 256, 256,
                                      capi.C128, prec, capi.ALGO_4M, 0, 0, None, 0, None)
        assert rc == capi.ERR_UNSUPPORTED
        assert b"complex64" in capi.lib.jetgpu_last_error()
    rc = capi.lib.jetgpu_contract(None, 2, sh, pm, None, 2, sh, pm, None, 256, 256, 256,
                                  capi.C64, 9, capi.ALGO_4M, 0, 0, None, 0, None)
    assert rc == capi.ERR_INVALID and b"precision" in capi.lib.jetgpu_last_error()


def test_fp16_stage_entry_points_need_exponents():
    from jet_gb300 import capi

    sh = capi.u64([16, 8])
    pm = capi.i32([0, 1])
    rc = capi.lib.jetgpu_split_fp16(None, 2, sh, pm, 16, 8, 8, 128, None, None, None)
    assert rc == capi.ERR_INVALID and b"exponent" in capi.lib.jetgpu_last_error()
    rc = capi.lib.jetgpu_gemm_fp16x3(None, None, None, 128, 128, 64, 64, None, 1.0, None)
    assert rc == capi.ERR_INVALID and b"null" in capi.lib.jetgpu_last_error()


def test_pool_limit_fails_allocations_on_the_host():
    """A capped pool turns an allocation past the cap into ERR_MEMORY before
    any CUDA call (host-side injection of device memory exhaustion)."""
    from jet_gb300 import capi

    assert capi.pool_bytes_in_use() == 0
    capi.set_pool_limit(1)
    try:
        p = ctypes.c_void_p(0)
        rc = capi.lib.jetgpu_malloc(1024, ctypes.byref(p))
        assert rc == capi.ERR_MEMORY
        assert p.value is None
        msg = capi.lib.jetgpu_last_error().decode()
        assert "device memory limit of 1 bytes reached" in msg
        assert "1024 requested" in msg
        # A zero-byte request needs no memory and passes.
        assert capi.lib.jetgpu_malloc(0, ctypes.byref(p)) == capi.OK
        with pytest.raises(capi.JetGpuError) as e:
            capi.malloc(4096)
        assert e.value.code == capi.ERR_MEMORY
    finally:
        capi.set_pool_limit(0)
    assert capi.pool_bytes_in_use() == 0


def test_nvtx_ranges_nest_without_a_tool():
    from jet_gb300 import capi

    with capi.nvtx_range("outer"):
        with capi.nvtx_range("inner"):
            pass


def test_tuned_precision_accepted_and_workspace_covers_every_form():
    """TUNED is a valid precision code; its workspace is at least that of each
    form it may pick (host arithmetic only)."""
    from jet_gb300 import capi

    shape, perm = [2] * 12, list(range(12))
    sizes = {p: capi.contract_workspace_size(shape, perm[::-1], shape, perm, 64, 64, 64,
                                             capi.C64, p)
             for p in (capi.PREC_FP32, capi.PREC_AUTO, capi.PREC_TF32X3, capi.PREC_FP16X3,
                       capi.PREC_TUNED)}
    assert sizes[capi.PREC_TUNED] == max(sizes.values())
    rc = capi.lib.jetgpu_contract(None, 12, capi.u64(shape), capi.i32(perm), None, 12,
                                  capi.u64(shape), capi.i32(perm), None, 64, 64, 64, capi.C64,
                                  6, capi.ALGO_4M, 0, 0, None, 0, None)
    assert rc == capi.ERR_INVALID and b"bad precision" in capi.lib.jetgpu_last_error()
    assert capi.lib.jetgpu_autotune_count() == 0
    assert capi.lib.jetgpu_autotune_entry(0, None, None, None, None, None) == capi.ERR_INVALID


def test_skinny_products_need_no_workspace():
    """A gate on any axes of a large tensor (one side <= 16 wide, k <= 64) is
    read in place by the skinny kernel: no transpose buffers. Wider products
    keep the transposing path's workspace (host arithmetic only)."""
    from jet_gb300 import capi

    shape = [2] * 16
    a_perm = [0, 1, 2, 4, 5, 6, 7, 8, 9, 10, 11, 13, 14, 15, 3, 12]  # gate on axes 3, 12
    for n, prec in ((4, capi.PREC_FP32), (16, capi.PREC_FP32), (4, capi.PREC_AUTO)):
        assert capi.contract_workspace_size(shape, a_perm, [4, n], [0, 1], 2 ** 14, n, 4,
                                            capi.C64, prec) == 0
        assert capi.contract_workspace_size([4, n], [1, 0], shape, a_perm[14:] + a_perm[:14],
                                            n, 2 ** 14, 4, capi.C128, capi.PREC_FP32) == 0
    assert capi.contract_workspace_size(shape, a_perm, [4, 32], [0, 1], 2 ** 14, 32, 4,
                                        capi.C64, capi.PREC_FP32) > 0


def test_group_offset_tables_match_numpy_views():
    """capi.view_offsets (the grouped launch's batch / row / column tables):
    element (b, i, j) of a view is the tensor's flat element at
    bat[b] + row[i] + col[j], as numpy's transpose + reshape says."""
    import numpy as np

    from jet_gb300 import capi

    rng = np.random.default_rng(4)
    for shape in ([3, 2, 4, 5], [2, 2, 2, 2, 2, 2], [7, 1, 3], [6]):
        x = np.arange(int(np.prod(shape))).reshape(shape)
        axes = list(rng.permutation(len(shape)))
        cut1 = int(rng.integers(0, len(axes) + 1))
        cut2 = int(rng.integers(cut1, len(axes) + 1))
        g = [axes[:cut1], axes[cut1:cut2], axes[cut2:]]
        bat, row, col = (capi.view_offsets(shape, a) for a in g)
        view = np.transpose(x, g[0] + g[1] + g[2]).reshape(len(bat), len(row), len(col))
        flat = x.reshape(-1)
        got = flat[bat[:, None, None] + row[None, :, None] + col[None, None, :]]
        assert np.array_equal(got, view)


def test_batched_operand_forms_are_checked_on_the_host():
    """a_batched / b_batched take 0, 1 or 2; in form 2 the permutation must
    lead with axes whose extents multiply to the batch (host checks, no
    device work)."""
    from jet_gb300 import capi

    shape = [2, 4, 3, 5]  # batch 2 at axis 0 in the layout below
    a_perm_ok = [0, 1, 2, 3]
    args = lambda a_batched, a_perm: (2, None, 4, capi.u64(shape), capi.i32(a_perm), a_batched,
                                      None, 2, capi.u64([5, 6]), capi.i32([0, 1]), 0, None,
                                      12, 6, 5, capi.C64, 0, capi.ALGO_4M, 0, 0, None, 0, None)
    rc = capi.lib.jetgpu_contract_batched(*args(3, a_perm_ok))
    assert rc == capi.ERR_INVALID and b"batched flags" in capi.lib.jetgpu_last_error()
    # Form 2 with a permutation that leads with the 4-axis: no batch split.
    rc = capi.lib.jetgpu_contract_batched(*args(2, [1, 0, 2, 3]))
    assert rc == capi.ERR_INVALID


def test_tensor_core_settings_reject_out_of_range_values():
    from jet_gb300 import capi

    assert capi.lib.jetgpu_set_tc_group_m(0) == capi.ERR_INVALID
    assert capi.lib.jetgpu_set_tc_group_m(1025) == capi.ERR_INVALID
    assert capi.lib.jetgpu_set_tc_persistent(2) == capi.ERR_INVALID
    assert capi.lib.jetgpu_set_tc_group_m(8) == capi.OK
    assert capi.lib.jetgpu_set_tc_persistent(1) == capi.OK


def test_group_launch_checks_on_the_host():
    from jet_gb300 import capi

    assert capi.lib.jetgpu_contract_group(None, 257, 1, capi.C64, None) == capi.ERR_INVALID
    assert capi.lib.jetgpu_contract_group(None, 0, 0, capi.C64, None) == capi.OK
    assert capi.lib.jetgpu_contract_group(None, 1, 1, 7, None) == capi.ERR_INVALID
    assert capi.lib.jetgpu_group_tiles(3, 33, 64) == 3 * 2 * 2
