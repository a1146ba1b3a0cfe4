"""GB300-native (sm_103a) ADC(2)-s hot path of mschuurman/ADC_ottawa.

The compute lives in libadcgpu.so (csrc/, C ABI in include/adcgpu.h);
this package is its host-side mirror (api.py) and build recipe (build.py).
"""
from .api import (  # noqa: F401
    ADCGPU_DIRECT, ADCGPU_FP64, ADCGPU_MIXED, PRECON_DPR, PRECON_FOLD, PRECON_MLP, PRECON_OLSEN, AdcGpu, AdcGpuError, adc2s_dim,
    chebyshev_auto_order_domain, eri_packed_size, fortran_e, select_adc2s, synth_eri_packed, synth_orbitals,
    synth_system, synth_uniform_block, write_cheby1h1p, write_chebyshev_auto, write_davidson_file,
    read_davidson_file, synth_dipole, fill_stvc, lanczos_guess_vecs, cvs_dim, select_adc2s_cvs,
)
