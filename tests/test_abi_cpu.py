"""The C-ABI library loads and exports every entry point include/magic_sht.h
declares; argument validation that happens before any CUDA call returns the
documented error codes.  No compute is launched (no GPU here)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "magic_sht.h")


@pytest.fixture(scope="module")
def lib():
    from magic_gb300 import build
    build.build()
    from magic_gb300 import _lib
    return _lib.load()


def declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(magic_sht_\w+)\s*\(", src)))


def test_header_declares_entry_points():
    names = declared()
    assert "magic_sht_init" in names and "magic_sht_transform_to_grid_space" in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol(lib):
    for name in declared():
        assert hasattr(lib, name), name


def test_binding_table_matches_header():
    from magic_gb300 import _lib
    assert sorted(_lib.SIGNATURES) == declared()


def test_phase_numbers_match_python_names():
    """MAGIC_SHT_PHASE_* in the header index _lib.PHASES (the names
    SHT.phase_times returns), and MAGIC_SHT_N_PHASES is their count."""
    from magic_gb300 import _lib
    src = open(HEADER).read()
    ph = {m.group(1).lower(): int(m.group(2)) for m in re.finditer(r"#define MAGIC_SHT_PHASE_(\w+)\s+(\d+)", src)}
    n = int(re.search(r"#define MAGIC_SHT_N_PHASES\s+(\d+)", src).group(1))
    assert n == len(_lib.PHASES) == len(ph)
    assert sorted(ph.values()) == list(range(n))
    for name, i in ph.items():
        assert _lib.PHASES[i] == name, (name, i)


def test_reference_names_all_present():
    # public names of src/sht_native.f90:16-20
    names = ["scal_to_spat", "scal_to_grad_spat", "pol_to_grad_spat", "torpol_to_spat",
             "pol_to_curlr_spat", "torpol_to_curl_spat", "torpol_to_dphspat", "scal_to_SH",
             "spat_to_sphertor", "torpol_to_spat_IC", "torpol_to_curl_spat_IC", "axi_to_spat",
             "spat_to_qst", "sphtor_to_spat", "toraxi_to_spat"]
    d = declared()
    for n in names:
        assert "magic_sht_" + n in d
    from magic_gb300 import SHT
    for n in names:
        assert callable(getattr(SHT, n))


def _init(lib, **kw):
    from magic_gb300 import _lib
    args = dict(l_max=31, m_max=0, minc=1, n_theta_max=48, n_phi_max=96, nlat_padded=0,
                precision=0, device=0)
    args.update(kw)
    d = _lib.Desc(*[args[k] for k, _ in _lib.Desc._fields_])
    h = ctypes.c_void_p()
    rc = lib.magic_sht_init(ctypes.byref(d), ctypes.byref(h))
    return rc, h


@pytest.mark.parametrize("kw,code", [
    (dict(n_theta_max=50), 2),        # not a multiple of 4 (truncation.f90:150)
    (dict(n_phi_max=98), 2),          # not a multiple of 4 (truncation.f90:137)
    (dict(n_phi_max=28), 2),          # 7 is not a factor of the FFT (fft.f90:73)
    (dict(minc=0), 2),                # minc < 1 (truncation.f90:131)
    (dict(l_max=0), 2),
    (dict(l_max=40000, n_theta_max=60000, n_phi_max=120000), 2),   # l | m << 16 packing of the lm tables
    (dict(n_phi_max=32), 2),          # m_max/minc+1 > n_phi/2: aliasing
    (dict(nlat_padded=40), 2),        # padding smaller than n_theta
    (dict(precision=9), 1),
])
def test_init_rejects_bad_grids_before_touching_cuda(lib, kw, code):
    rc, h = _init(lib, **kw)
    assert rc == code
    assert not h.value
    assert lib.magic_sht_last_error()


def test_null_arguments(lib):
    h = ctypes.c_void_p()
    assert lib.magic_sht_init(None, ctypes.byref(h)) == 1
    assert lib.magic_sht_scal_to_spat(None, None, None, 0) == 1
    assert lib.magic_sht_finalize(None) == 0
