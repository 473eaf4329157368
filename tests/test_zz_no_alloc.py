"""The allocation-free scal_to_spat entry point (magic_sht_scal_to_spat_noalloc),
called through the C ABI, against the ordinary magic_sht_scal_to_spat.

It serves callers that must not allocate device memory while they run (GPU
memory owned by a pool allocator, time-critical loops that cannot absorb the
device synchronisation of cudaMalloc/cudaFree): its only scratch is a static
device array shared by all calls.  Two calls in a row must both reproduce the
ordinary entry point (FP64 form and FP64-accurate tensor-core form: 1e-12
relative, the tolerance of the parity tests; the 3xBF16 form: its own 2e-6), and oversized grids and host pointers
are rejected with an error code.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import __graft_entry__ as g
    g.build()
    return torch


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("bf16x3", 2e-6), ("fp64tc", 1e-12)])
def test_noalloc_matches_ordinary_entry_point(torch, prec, tol):
    from magic_gb300 import SHT, _lib
    from magic_gb300.workload import spectra
    lib = _lib.load()
    s = SHT(255, 1, 384, 768, precision=prec, device=0)
    S = [torch.from_numpy(x).cuda() for x in spectra(255, 1, 2, seed=31)]
    # Calls in a row share the static scratch.  The first one (lcut = l_max)
    # leaves non-zero half-spectrum entries at every order, including the
    # orders above 250 that the later calls (lcut = 250) must overwrite with
    # zeros; stale entries would show up as a mismatch there.
    for call, (Sk, lc) in enumerate(((S[0], 255), (S[1], 250), (S[0], 250))):
        ref = s.scal_to_spat(Sk, lc)  # ordinary entry point, same stream
        out = torch.full((s.n_phi_max, s.nlat_padded), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        s.set_stream(None)
        n0, n1 = ctypes.c_longlong(0), ctypes.c_longlong(0)
        _lib.check(lib.magic_sht_launch_count(s._h, ctypes.byref(n0)))
        _lib.check(lib.magic_sht_scal_to_spat_noalloc(s._h, Sk.data_ptr(), out.data_ptr(), lc))
        _lib.check(lib.magic_sht_launch_count(s._h, ctypes.byref(n1)))
        s.synchronize()
        err = float(torch.linalg.vector_norm(out - ref) / torch.linalg.vector_norm(ref))
        assert err <= tol, (call, err)
        # the call counts its two kernels (Legendre sums, inverse FFT) in the
        # handle's launch counters like the ordinary entry points do
        assert n1.value - n0.value == 2, (call, n0.value, n1.value)
    s.close()


def test_noalloc_rejects_host_pointers_and_oversized_grids(torch):
    from magic_gb300 import SHT, _lib
    lib = _lib.load()
    s = SHT(31, 1, 48, 96, precision="fp64", device=0)
    host_in = np.zeros(s.lm_max, dtype=np.complex128)
    host_out = np.zeros((s.n_phi_max, s.nlat_padded))
    rc = lib.magic_sht_scal_to_spat_noalloc(s._h, host_in.ctypes.data, host_out.ctypes.data, 31)
    assert rc == _lib.ERR_ARG
    big = SHT(300, 1, 1024, 640, precision="fp64", device=0)  # 301*1024*16 B > 4 MiB
    d_in = torch.zeros(big.lm_max, dtype=torch.complex128, device="cuda")
    d_out = torch.zeros((big.n_phi_max, big.nlat_padded), dtype=torch.float64, device="cuda")
    rc = lib.magic_sht_scal_to_spat_noalloc(big._h, d_in.data_ptr(), d_out.data_ptr(), 300)
    assert rc == _lib.ERR_SIZE
    assert b"4194304" in lib.magic_sht_last_error()
