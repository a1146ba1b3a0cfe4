"""The allocation-free sigma product (adcgpu_sigma_device_noalloc).

It exists for callers that must not allocate device memory while they run,
such as a host application working inside a device-memory budget fixed in
advance, or a host thread that must not stall on cudaFree.  It must
give the same product as the regular entry point (adcgpu_sigma_device) on
the same device buffers, on consecutive calls that reuse its static scratch,
and it must refuse sizes beyond that scratch.  This file is collected after
the builder, learned-preconditioner and solver tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MIXED_TOL = 5e-3   # relative tolerance of the mixed-precision sigma tests


def test_noalloc_sigma_matches_regular_entry_point(gpu):
    import torch

    from adc_ottawa_gb300 import ADCGPU_MIXED, AdcGpu, synth_system
    from adc_ottawa_gb300._native import lib

    no, nv = 6, 30
    e, eri = synth_system(no, nv, 11)
    g = AdcGpu(0)
    g.set_orbitals(no, nv, e)
    g.set_eri_packed(eri)
    g.write_fspace_adc2_1(None, precision=ADCGPU_MIXED)
    N = g.ndim
    gen = torch.Generator(device="cuda").manual_seed(5)
    for m in (5, 3):       # two calls in a row sharing the static scratch
        x = torch.randn(m, N, device="cuda", dtype=torch.float32, generator=gen)   # N x m column-major
        w_ref = torch.zeros_like(x)
        w_na = torch.full_like(x, float("nan"))
        torch.cuda.synchronize()
        assert lib().adcgpu_sigma_device(g._h, m, C.c_void_p(x.data_ptr()), C.c_void_p(w_ref.data_ptr()), N) == 0
        assert lib().adcgpu_sigma_device_noalloc(g._h, m, C.c_void_p(x.data_ptr()),
                                                 C.c_void_p(w_na.data_ptr()), N) == 0
        ref = w_ref.cpu().numpy()
        got = w_na.cpu().numpy()
        assert np.isfinite(got).all()
        assert np.abs(got - ref).max() <= MIXED_TOL * np.abs(ref).max()
        assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()
    # beyond the static scratch: refused before any device work
    m_big = 1048576 // (no * nv) + 1
    st = lib().adcgpu_sigma_device_noalloc(g._h, m_big, C.c_void_p(x.data_ptr()), C.c_void_p(w_na.data_ptr()), N)
    assert st == 12
    assert b"static scratch" in lib().adcgpu_last_error(g._h)
    g.close()


@pytest.mark.parametrize("m,pad", [(16, 0), (24, 7), (3, 5)])
def test_noalloc_sigma_wide_blocks_and_padded_ld(gpu, m, pad):
    """From 16 columns on, the regular entry point switches to the tiled
    tensor-core pass while the allocation-free one keeps the per-warp pass:
    the two products agree within 1e-5 relative (BF16 values in both; FP32
    vectors against BF16 hi+lo vector pairs).  A leading dimension larger
    than N (padded columns) is honoured by both, and the padding rows of the
    output are left untouched.  Two calls in a row per case."""
    import torch

    from adc_ottawa_gb300 import ADCGPU_MIXED, AdcGpu, synth_system
    from adc_ottawa_gb300._native import lib

    no, nv = 5, 36
    e, eri = synth_system(no, nv, 23)
    g = AdcGpu(0)
    g.set_orbitals(no, nv, e)
    g.set_eri_packed(eri)
    g.write_fspace_adc2_1(None, precision=ADCGPU_MIXED)
    N = g.ndim
    ld = N + pad
    assert no * nv * m <= 1048576
    gen = torch.Generator(device="cuda").manual_seed(m + pad)
    for _ in range(2):
        x = torch.randn(m, ld, device="cuda", dtype=torch.float32, generator=gen)
        w_ref = torch.full_like(x, 7.0)
        w_na = torch.full_like(x, 7.0)
        torch.cuda.synchronize()
        assert lib().adcgpu_sigma_device(g._h, m, C.c_void_p(x.data_ptr()), C.c_void_p(w_ref.data_ptr()), ld) == 0
        assert lib().adcgpu_sigma_device_noalloc(g._h, m, C.c_void_p(x.data_ptr()),
                                                 C.c_void_p(w_na.data_ptr()), ld) == 0
        ref = w_ref.cpu().numpy()[:, :N]
        got = w_na.cpu().numpy()
        assert np.isfinite(got).all()
        assert np.all(got[:, N:] == 7.0)
        got = got[:, :N]
        assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()
    g.close()
