"""Iteration structure of the reference Davidson algorithm on the
nocc=16/nvirt=180 workload (N = 4,151,520, 20 roots, tol 1e-6, DPR, FP64,
reference default blocksize/maxvec, deflation on).

Needs a GPU: the reference algorithm (davdiag_block, block_davidson.f90
:33-145) is run by the library's plain FP64 path, which follows it step for
step (its two differences, cached W = HV and block CGS2 + Cholesky QR, are
exact in exact arithmetic; tests/test_gpu_solvers.py checks at
nocc=10/nvirt=110 that its iterations and its sum of currdim equal the
oracle's).  A full CPU run of the reference algorithm on this workload takes
hours, so the CPU timings of bench.py scale a measured sample of the
reference sigma product (hxvec_incore, :844-883) by the number of sigma
columns recorded here: sum over iterations of currdim, the columns the
reference recomputes every iteration (:855).

    python tests/golden/make_config3.py      # writes tests/golden/config3.json
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from adc_ottawa_gb300 import ADCGPU_FP64, PRECON_DPR, AdcGpu, synth_system  # noqa: E402

NO, NV, SEED, NROOTS, TOL = 16, 180, 7, 20, 1e-6


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main():
    e, eri = synth_system(NO, NV, SEED)
    g = AdcGpu(0)
    g.set_orbitals(NO, NV, e)
    g.set_eri_packed(eri)
    nnz = g.write_fspace_adc2_1(None, precision=ADCGPU_FP64)
    t = time.perf_counter()
    r = g.davdiag_block(NROOTS, TOL, precon=PRECON_DPR, precision=ADCGPU_FP64, want_vectors=False)
    sec = time.perf_counter() - t
    out = {"nocc": NO, "nvirt": NV, "seed": SEED, "e_sha": sha(e), "eri_sha": sha(eri), "ndim": g.ndim,
           "noffd": nnz, "davidson": {"nstates": NROOTS, "tol": TOL, "precon": PRECON_DPR, "status": r.status,
                                      "iterations": r.iterations, "nmult_reference": r.nmult_reference,
                                      "evals": r.evals.tolist(), "gpu_seconds": sec}}
    g.close()
    with open(os.path.join(HERE, "config3.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote config3.json", {k: v for k, v in out["davidson"].items() if k != "evals"})


if __name__ == "__main__":
    main()
