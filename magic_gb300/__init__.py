"""GB300-native (sm_103a) spherical-harmonic transforms for MagIC's radial loop.

`SHT` mirrors the public names of MagIC's ``module sht``
(src/sht_native.f90:16-20) over the C ABI of ``libmagic_sht.so``
(include/magic_sht.h).
"""
from .sht import SHT, SHTGroup, truncation, prime_decomposition, measure_gflops, dt_courant  # noqa: F401
