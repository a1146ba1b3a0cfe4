"""The tensor-core (tcgen05) sigma pass for BF16 matrix values.

The mixed-precision sigma product with BF16 values runs its C|D segments on
the tensor cores (csrc/sigma_umma.cu) from 1 to 48 columns per matrix pass.
It is checked against the same product on the previous path (mma.sync tile
for 16 columns and more, per-warp pass below) at 1e-5 relative, and against
the oracle's FP64 product (hxvec_incore, block_davidson.f90:844-883) at the
BF16 value tolerance, for column counts that exercise every operand width
(16, 32, 48 padded columns), several passes (56 columns), C-only and C|D
classes, one to six 64-value boxes per row, and a leading dimension larger
than N.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from tests.conftest import system

pytestmark = pytest.mark.gpu

BF16_TOL = 5e-3     # BF16 matrix values against the exact FP64 product
SAME_TOL = 1e-5     # two FP32-vector paths over the same BF16 values


def _mixed(no, nv, seed):
    from adc_ottawa_gb300 import ADCGPU_MIXED, AdcGpu

    e, eri = system(no, nv, seed)
    g = AdcGpu(0)
    g.set_orbitals(no, nv, e)
    g.set_eri_packed(eri)
    g.write_fspace_adc2_1(None, precision=ADCGPU_MIXED)
    return g, e, eri


def _sigma(g, x, ld, umma):
    import torch

    from adc_ottawa_gb300._native import lib

    # the previous path: flag 64 turns the tensor-core pass off
    assert lib().adcgpu_sigma_set_shape(g._h, 64, 2, 4 if umma else 4 | 64) == 0
    w = torch.full_like(x, 3.0)
    torch.cuda.synchronize()
    st = lib().adcgpu_sigma_device(g._h, x.shape[0], C.c_void_p(x.data_ptr()), C.c_void_p(w.data_ptr()), ld)
    assert st == 0, lib().adcgpu_last_error(g._h)
    return w.cpu().numpy().T


@pytest.mark.parametrize("no,nv,seed", [(6, 40, 3), (4, 180, 5), (10, 110, 2024)])
def test_umma_sigma_matches_previous_path_and_oracle(gpu, no, nv, seed):
    import torch

    g, e, eri = _mixed(no, nv, seed)
    N = g.ndim
    ref = oracle.Matrix.build(no, nv, e, eri)
    gen = torch.Generator(device="cuda").manual_seed(no * 1000 + nv)
    for m, pad in ((1, 0), (7, 3), (16, 0), (24, 0), (40, 5), (48, 0), (56, 0)):
        ld = N + pad
        x = torch.randn(m, ld, device="cuda", dtype=torch.float32, generator=gen)
        w_new = _sigma(g, x, ld, True)
        w_old = _sigma(g, x, ld, False)
        assert np.all(w_new[N:] == 3.0), "padding rows written"
        w_new, w_old = w_new[:N], w_old[:N]
        assert np.isfinite(w_new).all()
        scale = np.abs(w_old).max()
        assert np.abs(w_new - w_old).max() <= SAME_TOL * scale, (m, np.abs(w_new - w_old).max() / scale)
        if m in (7, 40):
            xs = x.cpu().numpy().T[:N].astype(np.float64)
            w64 = ref.matvec(xs)
            assert np.abs(w_new - w64).max() <= BF16_TOL * np.abs(w64).max()
    g.close()


def test_umma_mixed_davidson_matches_oracle(gpu):
    """The mixed ladder with the folded preconditioner (its BF16 phase and
    preconditioner run on the tensor-core pass) reaches the oracle's FP64
    eigenvalues within 1e-6 Ha."""
    from adc_ottawa_gb300 import ADCGPU_MIXED, PRECON_FOLD

    g, e, eri = _mixed(6, 40, 3)
    res = g.davdiag_block(10, 1e-6, precision=ADCGPU_MIXED, precon=PRECON_FOLD, want_vectors=False)
    st, ev, _, _ = oracle.Matrix.build(6, 40, e, eri).davidson(10, 1e-9, precon=1)
    assert res.status == 0 and st == 0
    assert np.abs(res.evals - ev).max() < 1e-6
    g.close()


def _sigma_flags(g, x, ld, flags):
    import torch

    from adc_ottawa_gb300._native import lib

    assert lib().adcgpu_sigma_set_shape(g._h, 64, 2, 4 | flags) == 0
    w = torch.full_like(x, 3.0)
    torch.cuda.synchronize()
    st = lib().adcgpu_sigma_device(g._h, x.shape[0], C.c_void_p(x.data_ptr()), C.c_void_p(w.data_ptr()), ld)
    assert st == 0, lib().adcgpu_last_error(g._h)
    out = w.cpu().numpy().T
    assert lib().adcgpu_sigma_set_shape(g._h, 64, 2, 4) == 0
    return out


@pytest.mark.parametrize("no,nv,seed", [(6, 40, 3), (10, 110, 2024), (3, 37, 9)])
def test_compact_segments_match_pass2_and_oracle(gpu, no, nv, seed, capsys):
    """Segments A and B in compact form (csrc/sigma_ab.cu: per-slab tables
    of the entries that do not depend on the other virtual index, plus the
    stored coincident entries) against the per-(slab, b') pass 2 and the
    per-run pass 3 over the same values: BF16 values on the tensor-core pass
    (flag 128 switches the compact kernels off) and FP32 values on the tiled
    pass (flag 256), at 1e-5 relative; both against the oracle's FP64
    product at the value precision.  FP32 values on the two tcgen05 passes
    over their BF16 slices (flag 1024, off by default) are held to the same
    bounds.  Column counts cover partial 4-column
    groups, more than one 48-column pass and a padded leading dimension;
    (3, 37) gives noP = 8 and an odd number of virtuals."""
    import torch

    g, e, eri = _mixed(no, nv, seed)
    N = g.ndim
    ref = oracle.Matrix.build(no, nv, e, eri)
    gen = torch.Generator(device="cuda").manual_seed(7 * no + nv)
    for fp32_values, base in ((False, 0), (True, 256), (True, 256 | 1024)):
        for m, pad in ((1, 0), (6, 2), (16, 0), (21, 3), (40, 0), (53, 1)):
            ld = N + pad
            x = torch.randn(m, ld, device="cuda", dtype=torch.float32, generator=gen)
            w_ab = _sigma_flags(g, x, ld, base)
            w_p2 = _sigma_flags(g, x, ld, base | 128)
            assert np.all(w_ab[N:] == 3.0), "padding rows written"
            w_ab, w_p2 = w_ab[:N], w_p2[:N]
            assert np.isfinite(w_ab).all()
            scale = np.abs(w_p2).max()
            assert np.abs(w_ab - w_p2).max() <= SAME_TOL * scale, (fp32_values, m, np.abs(w_ab - w_p2).max() / scale)
            if m in (6, 40):
                xs = x.cpu().numpy().T[:N].astype(np.float64)
                w64 = ref.matvec(xs)
                tol = 1e-5 if fp32_values else BF16_TOL
                err = np.abs(w_ab - w64).max() / np.abs(w64).max()
                err_p2 = np.abs(w_p2 - w64).max() / np.abs(w64).max()
                with capsys.disabled():
                    print(f"\nno={no} nv={nv} flags={base} m={m}: max error / max |W| {err:.2e} "
                          f"(pass-2 route {err_p2:.2e})")
                assert err <= tol, (fp32_values, m)
    g.close()
