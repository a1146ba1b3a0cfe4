"""Batched execution of independent ADC(2)-s problems on one GPU.

Many seeded systems of uneven size (and many SIL wavepackets) are solved
concurrently: every system owns a context with its own CUDA stream, the host
drives them from a thread pool (the C ABI releases the GIL), so builds,
sigma products and dense kernels of different systems overlap on the device.
Wavepackets on one matrix share every sigma product (adcgpu_autocorr runs
them as one block of 2P real columns).
"""
from __future__ import annotations

import concurrent.futures as cf
import time

import numpy as np

from . import api


def seeded_systems(n: int = 64, seed: int = 4242, nocc=(4, 12), nvirt=(30, 120)):
    """n systems with nocc ~ U{nocc}, nvirt ~ U{nvirt} and seeds seed + i."""
    rs = np.random.RandomState(seed)
    return [(int(rs.randint(nocc[0], nocc[1] + 1)), int(rs.randint(nvirt[0], nvirt[1] + 1)), seed + i)
            for i in range(n)]


def _solve_one(args):
    no, nv, seed, nroots, tol, precision, precon = args
    t0 = time.perf_counter()
    e, eri = api.synth_system(no, nv, seed, nthreads=2)
    g = api.AdcGpu(0)
    g.set_orbitals(no, nv, e)
    g.set_eri_packed(eri)
    g.write_fspace_adc2_1(None, precision=precision)
    r = g.davdiag_block(nroots, tol, precision=precision, precon=precon, want_vectors=False,
                        raise_on_nonconv=False)
    g.close()
    return {"nocc": no, "nvirt": nv, "seed": seed, "N": int(api.adc2s_dim(no, nv)[0]), "status": r.status,
            "iterations": r.iterations, "evals": r.evals.tolist(), "seconds": time.perf_counter() - t0}


def solve_many(systems, nroots: int = 8, tol: float = 1e-6, precision: int = api.ADCGPU_MIXED,
               precon: int = api.PRECON_DPR, workers: int = 8):
    """Solves all systems concurrently; returns per-system results and the
    wall time of the whole batch."""
    t = time.perf_counter()
    jobs = [(no, nv, seed, nroots, tol, precision, precon) for no, nv, seed in systems]
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        res = list(ex.map(_solve_one, jobs))
    return res, time.perf_counter() - t


def wavepackets(g: api.AdcGpu, npackets: int, seed: int = 77) -> np.ndarray:
    """Seeded positive 'dipole-like' start vectors (ndim x npackets)."""
    return api.synth_uniform_block(g.ndim, npackets, seed)
