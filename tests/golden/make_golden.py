"""Generate the golden fixtures in tests/golden/ from the oracle.

Run on a CPU host:  python tests/golden/make_golden.py [--config2]
                    python tests/golden/make_golden.py --config2-solvers
                    python tests/golden/make_golden.py --chebyshev

The fixtures pin (i) the seeded synthetic generator bit for bit across
hosts (SHA-256 of the orbital energies and packed ERIs), (ii) the oracle's
kept structure (count and an order-independent hash), diagonal and values,
and (iii) the oracle's eigenvalues, Lanczos spectra and SIL autocorrelation
on small systems.  --chebyshev writes chebyshev.json alone (the
order-domain autocorrelation and spectral bounds).  --config2 adds the nocc=10, nvirt=110 system (about
137 M kept elements; the oracle Davidson takes tens of minutes there).
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from adc_ottawa_gb300 import synth_system, synth_uniform_block  # noqa: E402


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def matrix_fingerprint(M: oracle.Matrix) -> dict:
    d, h, oi, oj = M.coo()
    k = np.lexsort((oj, oi))
    return {
        "ndim": int(M.ndim),
        "nnz": int(M.nnz),
        "structure_hash": [str(x) for x in oracle.structure_hash(oi, oj)],
        "diag_sha": sha(d),
        "values_sorted_sha": sha(h[k]),
    }


def small_case(no, nv, seed, dav=None, lanczos=None, sil=None) -> dict:
    e, eri = synth_system(no, nv, seed)
    M = oracle.Matrix.build(no, nv, e, eri)
    out = {"nocc": no, "nvirt": nv, "seed": seed, "e_sha": sha(e), "eri_sha": sha(eri)}
    out.update(matrix_fingerprint(M))
    if dav:
        st, ev, _, info = M.davidson(dav["nstates"], dav["tol"], precon=dav.get("precon", 1))
        assert st == 0, st
        out["davidson"] = {**dav, "evals": ev.tolist(), "iterations": info["iterations"]}
    if lanczos:
        q0 = synth_uniform_block(M.ndim, lanczos["b"], lanczos["seed"])
        T, ev = M.block_lanczos(q0, lanczos["ncycles"], orthotype=lanczos.get("orthotype", 0))
        b = lanczos["b"]
        mom, Tk = [], np.eye(T.shape[0])[:, :b]
        for k in range(1, 2 * lanczos["ncycles"]):
            Tk = T @ Tk
            mom.append(np.trace(Tk[:b]))
        out["lanczos"] = {**lanczos, "evals": ev.tolist(), "trace_moments": mom}
    if sil:
        f = synth_uniform_block(M.ndim, 1, sil["seed"])[:, 0]
        st, a, nm = M.autocorr(f, sil["tout"], sil["tfinal"], sil["kdim"], sil["tol"])
        assert st == 0
        out["sil"] = {**sil, "auto_re": a.real.tolist(), "auto_im": a.imag.tolist()}
    return out


def chebyshev_case() -> dict:
    """Chebyshev order-domain autocorrelation on nocc=5 nvirt=19 (seed 1234):
    the oracle's 'davlanc' bounds, and C_0..C_80 of a seeded uniform start
    vector with bounds [Emin - 0.2, 1.1 Emax] (which contain the spectrum)."""
    no, nv, seed = 5, 19, 1234
    e, eri = synth_system(no, nv, seed)
    M = oracle.Matrix.build(no, nv, e, eri)
    st, raw = M.spectral_bounds()
    assert st == 0
    bounds = [float(raw[0]) - 0.2, 1.1 * float(raw[1])]
    q0 = synth_uniform_block(M.ndim, 1, 79)[:, 0]
    auto, _ = M.chebyshev_auto(q0, np.array(bounds), 40)
    return {"nocc": no, "nvirt": nv, "seed": seed, "vector_seed": 79, "spectral_bounds": raw.tolist(),
            "bounds": bounds, "chebyord": 40, "auto": auto.tolist()}


def config2_solvers() -> dict:
    """Block Lanczos and SIL on the nocc=10/nvirt=110 matrix (seed 2024),
    the shapes of the nocc=10/nvirt=110 workloads:

    * block Lanczos, b = 10 seeded uniform start vectors (seed 99), 30
      cycles, orthotype 0 and 1 (run_block_lanczos, block_lanczos.f90
      :947-1256): the eigenvalues of T and the first-block trace moments
      tr (T^k)[:b,:b], k = 1..59 (stable under the sign freedom of the QR);
    * SIL autocorrelation (propagate_sillib, fvecprop.f90:365-564) of the
      first two of 32 seeded wavepackets (synth_uniform_block seed 77),
      Krylov dimension 15, tout = 0.1 au (step tout/2 = 0.05 au), 20 outer
      steps (tfinal = 1.0 au), autotol 1e-8."""
    no, nv, seed = 10, 110, 2024
    e, eri = synth_system(no, nv, seed)
    M = oracle.Matrix.build(no, nv, e, eri)
    out = {"lanczos": [], "sil": None}
    b, ncyc = 10, 30
    q0 = synth_uniform_block(M.ndim, b, 99)
    for ot in (0, 1):
        t = time.time()
        T, ev = M.block_lanczos(q0, ncyc, orthotype=ot)
        mom, Tk = [], np.eye(T.shape[0])[:, :b]
        for k in range(1, 2 * ncyc):
            Tk = T @ Tk
            mom.append(float(np.trace(Tk[:b])))
        out["lanczos"].append({"b": b, "ncycles": ncyc, "seed": 99, "orthotype": ot, "evals": ev.tolist(),
                               "trace_moments": mom})
        print("lanczos orthotype", ot, time.time() - t, flush=True)
    f = synth_uniform_block(M.ndim, 32, 77)
    sil = {"npackets": 32, "seed": 77, "packets": [0, 1], "tout": 0.1, "tfinal": 1.0, "kdim": 15, "tol": 1e-8,
           "auto_re": [], "auto_im": [], "nmult": []}
    for p in sil["packets"]:
        t = time.time()
        st, a, nm = M.autocorr(f[:, p], sil["tout"], sil["tfinal"], sil["kdim"], sil["tol"])
        assert st == 0, st
        sil["auto_re"].append(a.real.tolist())
        sil["auto_im"].append(a.imag.tolist())
        sil["nmult"].append(int(nm))
        print("sil packet", p, time.time() - t, flush=True)
    out["sil"] = sil
    return out


def main():
    if "--config2-solvers" in sys.argv:
        path = os.path.join(HERE, "config2.json")
        gold = json.load(open(path))
        gold.update(config2_solvers())
        with open(path, "w") as f:
            json.dump(gold, f, indent=1)
        print("updated config2.json")
        return
    if "--chebyshev" in sys.argv:
        with open(os.path.join(HERE, "chebyshev.json"), "w") as f:
            json.dump(chebyshev_case(), f, indent=1)
        print("wrote chebyshev.json")
        return
    cases = [
        small_case(2, 3, 5),
        small_case(4, 9, 7, dav={"nstates": 4, "tol": 1e-8}),
        small_case(5, 19, 1234, dav={"nstates": 6, "tol": 1e-8},
                   lanczos={"b": 4, "ncycles": 10, "seed": 77},
                   sil={"seed": 78, "tout": 0.5, "tfinal": 5.0, "kdim": 12, "tol": 1e-9}),
        small_case(6, 30, 11, dav={"nstates": 5, "tol": 1e-8, "precon": 2}),
    ]
    with open(os.path.join(HERE, "small_cases.json"), "w") as f:
        json.dump(cases, f, indent=1)
    print("wrote small_cases.json")
    if "--config2" in sys.argv:
        t = time.time()
        no, nv, seed = 10, 110, 2024
        e, eri = synth_system(no, nv, seed)
        M = oracle.Matrix.build(no, nv, e, eri)
        out = {"nocc": no, "nvirt": nv, "seed": seed, "e_sha": sha(e), "eri_sha": sha(eri)}
        out.update(matrix_fingerprint(M))
        print("config2 matrix", out["nnz"], time.time() - t, flush=True)
        st, ev, _, info = M.davidson(10, 1e-8, precon=1)
        out["davidson"] = {"nstates": 10, "tol": 1e-8, "precon": 1, "status": int(st), "evals": ev.tolist(),
                           "iterations": info["iterations"], "nmult": info["nmult"], "seconds": time.time() - t}
        with open(os.path.join(HERE, "config2.json"), "w") as f:
            json.dump(out, f, indent=1)
        print("wrote config2.json", time.time() - t)


if __name__ == "__main__":
    main()
