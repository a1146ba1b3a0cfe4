"""The solvers' tall-skinny Gram product C = A^T B of FP32 vectors on the
tensor cores (csrc/dense_umma.cu, reached through adcgpu_gram_f32): the
Rayleigh matrix and orthogonalisation products of calcrmat / qrortho
(block_davidson.f90:954-967, 1423-1465) on the mixed-precision phases.

Each FP32 value is split into three BF16 slices and six slice products are
accumulated, so the result must match the FP64 product of the same FP32
inputs to FP32 accuracy: 1e-6 of sum |a_i b_i| per entry (the FP32 rounding
of a few hundred partial sums), the same bound the CUDA-core kernel meets.
Shapes cover one and two 128-column tiles, 16/32/48-column operand widths,
row counts that are not multiples of the 64-row stage, padded leading
dimensions and a vector length of the benchmarked matrix.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _gram(g, A, B, lda, ldb, cuda_cores=False):
    import torch

    from adc_ottawa_gb300._native import lib

    N = A.shape[1]
    p, q = A.shape[0], B.shape[0]
    assert lib().adcgpu_sigma_set_shape(g._h, 64, 2, 4 | (512 if cuda_cores else 0)) == 0
    out = torch.full((q, p), 7.0, device="cuda", dtype=torch.float64)
    st = lib().adcgpu_gram_f32(g._h, N, p, q, C.c_void_p(A.data_ptr()), lda, C.c_void_p(B.data_ptr()), ldb,
                               C.c_void_p(out.data_ptr()), p)
    assert st == 0, lib().adcgpu_last_error(g._h)
    assert lib().adcgpu_sigma_set_shape(g._h, 64, 2, 4) == 0
    return out.cpu().numpy().T


@pytest.mark.parametrize("N,p,q,pad", [(4655, 10, 5, 0), (20000, 130, 40, 3), (131071, 160, 48, 1),
                                        (64 * 37, 33, 17, 0), (4151520, 120, 40, 0)])
def test_gram_f32_tensor_cores(gpu, N, p, q, pad):
    import torch

    from adc_ottawa_gb300 import AdcGpu, synth_system

    e, eri = synth_system(4, 12, 7)
    g = AdcGpu(0)
    g.set_orbitals(4, 12, e)
    g.set_eri_packed(eri)
    g.write_fspace_adc2_1(None)   # the launch-shape switches act on a built matrix
    gen = torch.Generator(device="cuda").manual_seed(N + p + q)
    lda, ldb = N + pad, N + 2 * pad
    A = torch.randn(p, lda, device="cuda", dtype=torch.float32, generator=gen)
    B = torch.randn(q, ldb, device="cuda", dtype=torch.float32, generator=gen) * 1e-3
    c_tc = _gram(g, A[:, :N], B[:, :N], lda, ldb)
    c_cc = _gram(g, A[:, :N], B[:, :N], lda, ldb, cuda_cores=True)
    a = A[:, :N].double()
    b = B[:, :N].double()
    ref = (a @ b.T).cpu().numpy()
    bound = (a.abs() @ b.abs().T).cpu().numpy()
    err_tc = np.abs(c_tc - ref) / bound
    err_cc = np.abs(c_cc - ref) / bound
    assert err_tc.max() < 1e-6, err_tc.max()
    assert err_cc.max() < 1e-6, err_cc.max()
    g.close()
