"""Failure detection without a GPU fault: the bounded device waits of the
tensor-core kernels give up, record JETGPU_ERR_TIMEOUT in the device status
word and return, and the context stays usable. The probe waits on an
mbarrier that nothing completes, with a 20 ms limit."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_reports(cuda):
    import torch

    from jet_gb300 import capi

    capi.take_device_status()  # clear any earlier status
    t0 = time.perf_counter()
    capi.check(capi.lib.jetgpu_probe_bounded_wait(20000, None))
    torch.cuda.synchronize()
    elapsed = time.perf_counter() - t0
    assert capi.take_device_status() == capi.ERR_TIMEOUT
    assert capi.take_device_status() == 0  # reading clears it
    assert elapsed < 5.0
    # The context is still usable: a tensor-core contraction runs and is right.
    m, n, k = 256, 128, 64
    rng = np.random.default_rng(0)
    a = (rng.standard_normal((m, k)) + 1j * rng.standard_normal((m, k))).astype(np.complex64)
    b = (rng.standard_normal((k, n)) + 1j * rng.standard_normal((k, n))).astype(np.complex64)
    got = capi.contract(torch.from_numpy(a.reshape(-1)).to(cuda), [m, k], [0, 1],
                        torch.from_numpy(b.reshape(-1)).to(cuda), [k, n], [0, 1], m, n, k,
                        precision=capi.PREC_TF32X3).cpu().numpy().reshape(m, n)
    want = a.astype(np.complex128) @ b.astype(np.complex128)
    assert np.linalg.norm(got - want) <= 1e-5 * np.linalg.norm(want)
    assert capi.take_device_status() == 0


def test_probe_limit_is_validated_on_the_host(cuda):
    from jet_gb300 import capi

    assert capi.lib.jetgpu_probe_bounded_wait(0, None) == capi.ERR_INVALID
    assert capi.lib.jetgpu_probe_bounded_wait(2000000, None) == capi.ERR_INVALID
