"""Parity at the shapes of the larger workloads, against the oracle.

* block Lanczos on the nocc=10/nvirt=110 matrix, b = 10, 30 cycles,
  orthotype 0 and 1 (run_block_lanczos, block_lanczos.f90:947-1256);
* SIL autocorrelation of 32 wavepackets on the same matrix, Krylov
  dimension 15, step tout/2 = 0.05 au, 20 outer steps (propagate_sillib,
  fvecprop.f90:365-564), two packets checked;
* independent systems solved concurrently by the batch driver, each against
  the oracle's Davidson;
* the davname eigenpair file of a GPU solve (wreigenpairs,
  block_davidson.f90:1469-1532).

The nocc=10/nvirt=110 references are committed fixtures
(tests/golden/config2.json, written by make_golden.py --config2-solvers).
"""
import json
import os

import numpy as np
import pytest

import oracle
from tests.conftest import ROOT
from tests.test_gpu_build import make

pytestmark = pytest.mark.gpu

GOLD = os.path.join(ROOT, "tests", "golden", "config2.json")


@pytest.fixture(scope="module")
def cfg2(gpu):
    gold = json.load(open(GOLD))
    g, e, eri = make(gold["nocc"], gold["nvirt"], gold["seed"])
    yield g, gold
    g.close()


@pytest.mark.slow
@pytest.mark.parametrize("orthotype", [0, 1])
def test_lanczos_config2_golden(cfg2, orthotype):
    """b = 10, ncycles = 30: the first-block moments tr (T^k)[:b,:b], k < 60,
    within 1e-7 relative of the oracle's, and the five lowest and highest
    eigenvalues of T within 1e-7 relative (T itself is defined up to the
    block-diagonal sign similarity of the QR factors)."""
    from adc_ottawa_gb300 import synth_uniform_block

    g, gold = cfg2
    ref = [x for x in gold["lanczos"] if x["orthotype"] == orthotype][0]
    b, ncyc = ref["b"], ref["ncycles"]
    q0 = synth_uniform_block(g.ndim, b, ref["seed"])
    T, ev, _ = g.lancdiag_block(q0, ncyc, orthotype=orthotype)
    mom, Tk = [], np.eye(b * ncyc)[:, :b]
    for k in range(1, 2 * ncyc):
        Tk = T @ Tk
        mom.append(np.trace(Tk[:b]))
    mom, mref = np.array(mom), np.array(ref["trace_moments"])
    assert np.all(np.abs(mom - mref) <= 1e-7 * np.abs(mref)), np.abs(mom / mref - 1).max()
    evr = np.array(ref["evals"])
    scale = np.abs(evr).max()
    assert np.abs(ev[:5] - evr[:5]).max() <= 1e-7 * scale
    assert np.abs(ev[-5:] - evr[-5:]).max() <= 1e-7 * scale


@pytest.mark.slow
def test_sil_config4_golden(cfg2):
    """32 wavepackets propagated together (Krylov dimension 15, step 0.05 au,
    20 outer steps, autotol 1e-8): packets 0 and 1 match the oracle's
    one-packet propagation within 1e-7 relative to max |a(t)|."""
    from adc_ottawa_gb300 import synth_uniform_block

    g, gold = cfg2
    s = gold["sil"]
    f = synth_uniform_block(g.ndim, s["npackets"], s["seed"])
    a, _ = g.propagate_fvec(f, s["tout"], s["tfinal"], s["kdim"], s["tol"])
    assert a.shape[0] == s["npackets"]
    for j, p in enumerate(s["packets"]):
        ar = np.array(s["auto_re"][j]) + 1j * np.array(s["auto_im"][j])
        assert a.shape[1] == ar.shape[0]
        assert np.abs(a[p] - ar).max() <= 1e-7 * np.abs(ar).max()


@pytest.mark.parametrize("mode", ["mixed", "fp64"])
def test_batched_systems_vs_oracle(gpu, mode):
    """The four smallest of the 64 seeded batch systems, solved concurrently
    (one context and stream each), 8 roots: mixed ladder + fold within
    1e-6 Ha, FP64 + DPR within 1e-8 Ha of the oracle's FP64 Davidson."""
    from adc_ottawa_gb300 import ADCGPU_FP64, ADCGPU_MIXED, PRECON_DPR, PRECON_FOLD, adc2s_dim, batch
    from tests.conftest import system

    systems = sorted(batch.seeded_systems(64), key=lambda s: adc2s_dim(s[0], s[1])[0])[:4]
    if mode == "mixed":
        res, _ = batch.solve_many(systems, nroots=8, tol=1e-6, precision=ADCGPU_MIXED, precon=PRECON_FOLD,
                                  workers=4)
        tol_e = 1e-6
    else:
        res, _ = batch.solve_many(systems, nroots=8, tol=1e-8, precision=ADCGPU_FP64, precon=PRECON_DPR,
                                  workers=4)
        tol_e = 1e-8
    for (no, nv, seed), r in zip(systems, res):
        assert r["status"] == 0
        e, eri = system(no, nv, seed)
        st, ev, _, _ = oracle.Matrix.build(no, nv, e, eri).davidson(8, 1e-9, precon=1)
        assert st == 0
        assert np.abs(np.array(r["evals"]) - ev).max() < tol_e, (no, nv, seed)


def test_davname_file_of_gpu_solve(gpu, tmp_path):
    """The eigenpairs of a GPU Davidson written as davname records read back
    bit for bit, in ascending order, as readdavvc would see them."""
    from adc_ottawa_gb300 import read_davidson_file, write_davidson_file

    g, e, eri = make(5, 19, 1234)
    res = g.davdiag_block(6, 1e-8)
    path = str(tmp_path / "davname")
    write_davidson_file(path, res.evals, res.evecs)
    idx, ev, X = read_davidson_file(path, g.ndim)
    assert np.array_equal(idx, np.arange(1, 7))
    assert np.array_equal(ev, res.evals) and np.all(np.diff(ev) >= 0)
    assert np.array_equal(X, res.evecs)
    g.close()
