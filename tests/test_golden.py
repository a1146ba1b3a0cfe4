"""Committed golden fixtures (tests/golden/make_golden.py) re-checked on this
host: the generator is bit-identical across hosts and the oracle reproduces
its recorded structure, eigenvalues, Lanczos spectra and autocorrelation."""
import json
import os

import numpy as np
import pytest

import oracle
from tests.conftest import ROOT, system

GOLD = os.path.join(ROOT, "tests", "golden")


def load(name):
    with open(os.path.join(GOLD, name)) as f:
        return json.load(f)


def cases():
    return load("small_cases.json")


def fingerprint(M):
    import hashlib

    d, h, oi, oj = M.coo()
    k = np.lexsort((oj, oi))
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
    return M.nnz, [str(x) for x in oracle.structure_hash(oi, oj)], sha(d), sha(h[k])


@pytest.mark.parametrize("idx", range(4))
def test_generator_and_oracle_structure(built, idx):
    import hashlib

    c = cases()[idx]
    e, eri = system(c["nocc"], c["nvirt"], c["seed"])
    assert hashlib.sha256(e.tobytes()).hexdigest() == c["e_sha"]
    assert hashlib.sha256(eri.tobytes()).hexdigest() == c["eri_sha"]
    M = oracle.Matrix.build(c["nocc"], c["nvirt"], e, eri)
    nnz, sh, dsha, vsha = fingerprint(M)
    assert nnz == c["nnz"] and sh == c["structure_hash"] and dsha == c["diag_sha"] and vsha == c["values_sorted_sha"]


def test_oracle_solvers_reproduce(built):
    from adc_ottawa_gb300 import synth_uniform_block

    c = cases()[2]
    e, eri = system(c["nocc"], c["nvirt"], c["seed"])
    M = oracle.Matrix.build(c["nocc"], c["nvirt"], e, eri)
    st, ev, _, _ = M.davidson(c["davidson"]["nstates"], c["davidson"]["tol"])
    assert np.abs(ev - np.array(c["davidson"]["evals"])).max() < 1e-10
    L = c["lanczos"]
    q0 = synth_uniform_block(M.ndim, L["b"], L["seed"])
    T, lev = M.block_lanczos(q0, L["ncycles"])
    assert np.abs(lev - np.array(L["evals"])).max() < 1e-9
    S = c["sil"]
    f = synth_uniform_block(M.ndim, 1, S["seed"])[:, 0]
    st, a, _ = M.autocorr(f, S["tout"], S["tfinal"], S["kdim"], S["tol"])
    ref = np.array(S["auto_re"]) + 1j * np.array(S["auto_im"])
    assert np.abs(a - ref).max() <= 1e-9 * np.abs(ref).max()


def test_oracle_chebyshev_reproduces(built):
    """chebyshev.json: the oracle's 'davlanc' bounds and C_0..C_80."""
    from adc_ottawa_gb300 import synth_uniform_block

    c = load("chebyshev.json")
    e, eri = system(c["nocc"], c["nvirt"], c["seed"])
    M = oracle.Matrix.build(c["nocc"], c["nvirt"], e, eri)
    st, raw = M.spectral_bounds()
    assert st == 0 and np.abs(raw - np.array(c["spectral_bounds"])).max() <= 1e-9
    q0 = synth_uniform_block(M.ndim, 1, c["vector_seed"])[:, 0]
    a, _ = M.chebyshev_auto(q0, np.array(c["bounds"]), c["chebyord"])
    ref = np.array(c["auto"])
    assert np.abs(a - ref).max() <= 1e-12 * ref[0]
