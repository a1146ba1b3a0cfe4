"""Chebyshev order-domain autocorrelation on the GPU against the oracle.

chebyshev_auto (chebyspec.f90:246-330), project_psi0 (:398-470) and
spectral_bounds_davlanc (specbounds.f90:121-205).  Tolerances: C_k within
1e-7 of C_0 (the autocorrelation bar), vectors within 1e-9 of their largest
element, spectral bounds within 1e-8 Ha (the eigenvalue bar).
"""
import numpy as np
import pytest

import oracle
from tests.conftest import system

pytestmark = pytest.mark.gpu


def make(no, nv, seed):
    from adc_ottawa_gb300 import AdcGpu, select_adc2s

    e, eri = system(no, nv, seed)
    g = AdcGpu(0)
    g.set_orbitals(no, nv, e)
    g.set_eri_packed(eri)
    g.write_fspace_adc2_1(select_adc2s(no, nv))
    return g, e, eri


@pytest.fixture(scope="module")
def cfg1(gpu):
    no, nv = 5, 19
    g, e, eri = make(no, nv, 1234)
    M = oracle.Matrix.build(no, nv, e, eri)
    w = np.linalg.eigvalsh(M.dense())
    yield g, M, w, no * nv
    g.close()


@pytest.mark.parametrize("chebyord", [60, 61])
def test_chebyshev_auto_matches_oracle(cfg1, chebyord):
    """Three start vectors in one expansion; an odd order is rounded down."""
    g, M, w, n1 = cfg1
    bounds = np.array([w[0] - 0.2, 1.1 * w[-1]])
    Q = np.random.RandomState(7).uniform(size=(M.ndim, 3))
    auto, q1 = g.chebyshev_auto(Q, bounds, chebyord, save1h1p=True)
    assert auto.shape == (3, 121) and q1.shape == (3, 61, n1)
    for p in range(3):
        ref, rq1 = M.chebyshev_auto(Q[:, p], bounds, chebyord, n1=n1)
        assert np.abs(auto[p] - ref).max() <= 1e-7 * ref[0], np.abs(auto[p] - ref).max() / ref[0]
        assert np.abs(q1[p] - rq1.T).max() <= 1e-9 * np.abs(rq1).max()


def test_chebyshev_df_matches_oracle(cfg1):
    """16 vectors (the tiled sigma pass) with double-float arithmetic."""
    g, M, w, n1 = cfg1
    bounds = np.array([w[0] - 0.2, 1.1 * w[-1]])
    Q = np.random.RandomState(11).uniform(size=(M.ndim, 16))
    auto, _ = g.chebyshev_auto(Q, bounds, 40, df=True)
    nat, _ = g.chebyshev_auto(Q, bounds, 40)
    for p in (0, 7, 15):
        ref, _ = M.chebyshev_auto(Q[:, p], bounds, 40)
        assert np.abs(auto[p] - ref).max() <= 1e-7 * ref[0]
    assert np.abs(auto - nat).max() <= 1e-10 * nat[:, 0].max()
    pq = g.project_psi0(Q[:, :16], bounds, 40, 0.5 * (w[0] + w[-1]), df=True)
    ref = M.chebyshev_project(Q[:, 3], bounds, 40, 0.5 * (w[0] + w[-1]))
    assert np.abs(pq[:, 3] - ref).max() <= 1e-9 * np.abs(ref).max()


def test_project_psi0_matches_oracle(cfg1):
    g, M, w, n1 = cfg1
    bounds = np.array([w[0] - 0.2, 1.1 * w[-1]])
    projen = 0.5 * (w[0] + w[-1])
    Q = np.random.RandomState(8).uniform(size=(M.ndim, 2))
    pq = g.project_psi0(Q, bounds, 60, projen)
    for p in range(2):
        ref = M.chebyshev_project(Q[:, p], bounds, 60, projen)
        assert np.abs(pq[:, p] - ref).max() <= 1e-9 * np.abs(ref).max()


def test_spectral_bounds_match_oracle(cfg1):
    g, M, w, n1 = cfg1
    b = g.spectral_bounds()
    st, ref = M.spectral_bounds()
    assert st == 0
    assert np.abs(b - ref).max() <= 1e-8
    assert abs(b[0] - w[0]) <= 1e-8 and abs(b[1] - w[-1]) <= 1e-8


def test_driver_widens_bounds_and_writes_files(cfg1, tmp_path):
    from adc_ottawa_gb300 import chebyshev_auto_order_domain

    g, M, w, n1 = cfg1
    q0 = np.random.RandomState(9).uniform(size=M.ndim)
    raw = np.array([w[0] - 0.2, w[-1]])
    auto, q1, b = chebyshev_auto_order_domain(g, q0, 20, bounds=raw, save1h1p=True, outdir=str(tmp_path))
    assert np.array_equal(b, [0.9 * raw[0], 1.1 * raw[1]])
    ref, _ = M.chebyshev_auto(q0, b, 20)
    assert np.abs(auto[0] - ref).max() <= 1e-7 * ref[0]
    lines = (tmp_path / "chebyauto").read_text().split("\n")
    assert lines[2] == "#    Order [k]    C_k" and len(lines) == 3 + 41 + 1
    assert (tmp_path / "cheby1h1p").stat().st_size == 21 * (8 * n1 + 8)


def test_identities_at_larger_size(gpu):
    """N = 51,680: with bounds that contain the spectrum |C_k| <= C_0; the
    doubling formulas of an order-40 run equal the direct products of an
    order-80 run; a block of 4 vectors equals 4 single-vector runs."""
    g, e, eri = make(8, 40, 5)
    b = g.spectral_bounds()
    width = b[1] - b[0]
    bounds = np.array([b[0] - 0.05 * width, b[1] + 0.05 * width])
    Q = np.random.RandomState(10).uniform(size=(g.ndim, 4))
    a80, _ = g.chebyshev_auto(Q, bounds, 80)
    a40, _ = g.chebyshev_auto(Q, bounds, 40)
    c0 = a80[:, :1]
    assert np.all(np.abs(a80) <= c0 * (1 + 1e-10))
    assert np.abs(a40 - a80[:, :81]).max() <= 1e-9 * c0.max()
    for p in range(4):
        single, _ = g.chebyshev_auto(Q[:, p], bounds, 80)
        assert np.abs(single[0] - a80[p]).max() <= 1e-12 * c0[p, 0]
    g.close()


def test_rejects_bad_bounds(cfg1):
    from adc_ottawa_gb300 import AdcGpuError

    g, M, w, n1 = cfg1
    q0 = np.ones(M.ndim)
    with pytest.raises(AdcGpuError) as ei:
        g.chebyshev_auto(q0, [1.0, -1.0], 10)
    assert ei.value.code == 12
    with pytest.raises(AdcGpuError) as ei:
        g.project_psi0(q0, [w[0] - 0.2, 1.1 * w[-1]], 10, 10.0 * w[-1])
    assert ei.value.code == 12


def test_device_bytes_released_after_solvers(cfg1):
    """adcgpu_device_bytes counts what the context holds: the FP64 solvers'
    work spaces are released when they return."""
    g, M, w, n1 = cfg1
    b0 = g.device_bytes()
    assert b0 > 8 * M.ndim
    g.davdiag_block(4, 1e-8, want_vectors=False)
    g.lancdiag_block(np.random.RandomState(1).uniform(size=(M.ndim, 2)), 10, orthotype=1)
    g.chebyshev_auto(np.ones(M.ndim), [w[0] - 0.2, 1.1 * w[-1]], 10)
    g.spectral_bounds()
    assert g.device_bytes() == b0


def test_matches_golden_fixture(cfg1):
    """tests/golden/chebyshev.json (written by the oracle): bounds within
    1e-8 Ha, C_k within 1e-7 C_0."""
    import json
    import os

    from adc_ottawa_gb300 import synth_uniform_block
    from tests.conftest import ROOT

    g, M, w, n1 = cfg1
    c = json.load(open(os.path.join(ROOT, "tests", "golden", "chebyshev.json")))
    assert (c["nocc"], c["nvirt"], c["seed"]) == (5, 19, 1234)
    assert np.abs(g.spectral_bounds() - np.array(c["spectral_bounds"])).max() <= 1e-8
    q0 = synth_uniform_block(g.ndim, 1, c["vector_seed"])[:, 0]
    auto, _ = g.chebyshev_auto(q0, c["bounds"], c["chebyord"])
    ref = np.array(c["auto"])
    assert np.abs(auto[0] - ref).max() <= 1e-7 * ref[0]
