"""The direct (matrix-free) path, ADCGPU_DIRECT: the matvec keyword's
get_matvec_adc2s_omp (dmatvec_davidson.f90:1031-1230) with hiivec (:888-978)
and the Ca1/Cb1/Cc1/Cc2 ph-ph formulas (adc_ph.f90:98-303).  The coupling
block is not stored; every sigma product recomputes it chunk by chunk."""
import numpy as np
import pytest

import oracle
from tests.conftest import system

pytestmark = pytest.mark.gpu


def _direct(no, nv, seed):
    from adc_ottawa_gb300 import ADCGPU_DIRECT, AdcGpu

    e, eri = system(no, nv, seed)
    g = AdcGpu(0)
    g.set_orbitals(no, nv, e)
    g.set_eri_packed(eri)
    noffd = g.write_fspace_adc2_1(None, precision=ADCGPU_DIRECT)
    return g, e, eri, noffd


@pytest.mark.parametrize("no,nv,seed", [(5, 19, 1234), (6, 40, 3)])
def test_direct_matches_oracle(gpu, no, nv, seed):
    """hiivec diagonal bit for bit, the kept count of the coupling block, and
    the FP64 sigma product within 1e-13 of the oracle's direct matrix."""
    g, e, eri, noffd = _direct(no, nv, seed)
    ref = oracle.Matrix.build_direct(no, nv, e, eri)
    d_ref, _, _, _ = ref.coo()
    assert np.array_equal(g.get_diag(), d_ref)
    assert noffd == ref.nnz
    x = np.random.RandomState(no).rand(g.ndim, 21)      # 16-column tile + per-warp pass
    y = g.sigma(x)
    y_ref = ref.matvec(x)
    assert np.abs(y - y_ref).max() <= 1e-13 * np.abs(y_ref).max()
    g.close()


def test_direct_davidson_and_memory(gpu):
    """Davidson on the direct path converges to the oracle's eigenvalues
    (1e-8 Ha); the context holds only one chunk of the coupling block, so it
    needs less device memory than the stored path; the COO export, which
    needs the stored block, is refused."""
    from adc_ottawa_gb300 import ADCGPU_FP64, AdcGpu, AdcGpuError

    no, nv, seed = 6, 40, 3
    g, e, eri, _ = _direct(no, nv, seed)
    res = g.davdiag_block(8, 1e-8)
    st, ev, _, _ = oracle.Matrix.build_direct(no, nv, e, eri).davidson(8, 1e-8)
    assert res.status == 0 and st == 0
    assert np.abs(res.evals - ev).max() < 1e-8
    h = AdcGpu(0)
    h.set_orbitals(no, nv, e)
    h.set_eri_packed(eri)
    h.write_fspace_adc2_1(None, precision=ADCGPU_FP64)
    assert g.device_bytes() < h.device_bytes()
    with pytest.raises(AdcGpuError) as ei:
        g.export_coo()
    assert ei.value.code == 16
    h.close()
    g.close()
