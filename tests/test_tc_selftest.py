"""tcgen05 tensor-core GEMM self-test through the C ABI: one M=128 MMA chain
with bf16 operands in 128-byte-swizzled shared memory and the accumulator in
tensor memory must reproduce A B^T exactly (bf16-exact inputs, sums well
inside fp32)."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import __graft_entry__ as g
    g.build()
    from magic_gb300 import _lib
    return _lib.load()


@pytest.mark.parametrize("n,kc", [(128, 1), (64, 1), (32, 1), (256, 2), (128, 2)])
def test_tc_gemm_exact(lib, n, kc):
    from magic_gb300._lib import check
    v = ctypes.c_double()
    check(lib.magic_sht_tc_selftest(0, n, kc, ctypes.byref(v)))
    assert v.value < 1e-6, v.value


@pytest.mark.parametrize("n,kc", [(128, 1), (64, 1), (256, 2), (128, 2)])
def test_tc_gemm_exact_tf32(lib, n, kc):
    """The same GEMM with tf32 operands (kind::tf32, K = 8 per MMA)."""
    from magic_gb300._lib import check
    v = ctypes.c_double()
    check(lib.magic_sht_tc_selftest_tf32(0, n, kc, ctypes.byref(v)))
    assert v.value < 1e-6, v.value


def test_bounded_wait_gives_up_and_device_stays_usable(lib):
    """Failure detection without a GPU fault: a wait on an mbarrier that
    nothing completes gives up after its cycle limit, the library reports
    MAGIC_SHT_ERR_TIMEOUT, and the device keeps working (a completed wait and
    a transform afterwards)."""
    import numpy as np
    from magic_gb300 import _lib, SHT
    assert lib.magic_sht_wait_selftest(0, 1 << 20, 0) == _lib.ERR_TIMEOUT
    assert lib.magic_sht_wait_selftest(0, 1 << 20, 1) == _lib.OK
    s = SHT(31, 1, 48, 96, precision="fp64", device=0)
    S = np.zeros(s.lm_max, dtype=np.complex128)
    S[0] = 1.0
    f = s.scal_to_spat(S)
    np.testing.assert_allclose(f[:, :48], 1.0 / np.sqrt(4.0 * np.pi), rtol=1e-12)
