"""Training pipeline of the learned Davidson preconditioner (ADCGPU_PRECON_MLP).

Data: residual -> correction pairs generated by the FP64 GPU Davidson itself
(adcgpu_davidson_trace) on seeded small synthetic systems.  For root i at
iteration k the residual r, Ritz vector x and Ritz value lambda are recorded;
the target correction is the part of the converged eigenvector x* orthogonal
to x, e = x* - (x*.x) x: the direction that completes the subspace.

Model: t_j = m_j r_j / (lambda - h_jj), m = MLP(features_j) (the library's
16 -> 256 -> 256 -> 1 SiLU network, BF16 weights, FP32 accumulation), trained
with the scale- and sign-invariant loss 1 - cos^2(t, e) by the library's own
forward/backward/Adam kernels (adcgpu_mlp_train_step).  The last layer starts
at w3 = 0, b3 = 1, i.e. at the diagonal preconditioner.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import api
from ._native import DavParams, lib, ptr

NIN, H = 16, 256
_fp = C.POINTER(C.c_float)


def num_params() -> int:
    return int(lib().adcgpu_mlp_num_params())


def init_params(seed: int = 0) -> np.ndarray:
    rs = np.random.RandomState(seed)
    W1 = rs.standard_normal((H, NIN)) * np.sqrt(2.0 / NIN)
    b1 = np.zeros(H)
    W2 = rs.standard_normal((H, H)) * np.sqrt(2.0 / H)
    b2 = np.zeros(H)
    w3 = np.zeros(H)
    b3 = np.ones(1)
    p = np.concatenate([W1.ravel(), b1, W2.ravel(), b2, w3, b3]).astype(np.float32)
    assert p.size == num_params()
    return p


def unpack(p: np.ndarray):
    o = 0
    W1 = p[o:o + H * NIN].reshape(H, NIN); o += H * NIN
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    w3 = p[o:o + H]; o += H
    b3 = p[o]
    return W1, b1, W2, b2, w3, b3


def config_info(nocc: int, nvirt: int, e: np.ndarray):
    """Per configuration j: zeroth-order energy d0 and class (-1 single, 0..3)."""
    kpq = api.select_adc2s(nocc, nvirt)[1:]
    n1 = nocc * nvirt
    d0 = np.empty(len(kpq))
    cls = np.empty(len(kpq), np.int32)
    j = kpq[:, 2] - 1
    a = kpq[:, 4] - 1
    d0[:n1] = e[a[:n1]] - e[j[:n1]]
    cls[:n1] = -1
    k = kpq[n1:, 3] - 1
    b = kpq[n1:, 5] - 1
    d0[n1:] = ((e[a[n1:]] + e[b]) - e[j[n1:]]) - e[k]
    cls[n1:] = np.minimum(kpq[n1:, 6] - 1, 3)
    return d0, cls


def features(lam: float, h: np.ndarray, d0: np.ndarray, cls: np.ndarray) -> np.ndarray:
    """Same features as mlp_feature in csrc/mlp.cu (FP32)."""
    g = lam - h
    F = np.zeros((len(h), NIN), np.float32)
    F[:, 0] = g.astype(np.float32)
    F[:, 1] = np.where(g >= 0, 1.0, -1.0).astype(np.float32) * np.exp(-np.abs(g.astype(np.float32)))
    F[:, 2] = 1.0 / (1.0 + np.abs(g.astype(np.float32)))
    F[:, 3] = cls < 0
    for c in range(4):
        F[:, 4 + c] = cls == c
    F[:, 8] = (d0 / 10.0).astype(np.float32)
    F[:, 9] = ((h - d0) / 10.0).astype(np.float32)
    F[:, 10] = np.float32(lam / 10.0)
    return F


def trace(g: api.AdcGpu, nstates: int, tol: float, every: int = 2, max_records: int = 40, maxiter: int = 200):
    N = g.ndim
    p = DavParams(davstates=nstates, dmain=0, maxsubdim=-1, maxiter=maxiter, precon=1, ldfl=0, lsubdiag=0,
                  guessdim=800, davtol=tol, precision=0, refine=0, tol_bf16=0.0, tol_fp32=0.0)
    R = np.empty((max_records, nstates, N))
    X = np.empty((max_records, nstates, N))
    lam = np.empty((max_records, nstates))
    ev = np.empty(nstates)
    vec = np.empty((nstates, N))
    n = C.c_int(0)
    st = lib().adcgpu_davidson_trace(g._h, C.byref(p), every, max_records, ptr(R), ptr(X), ptr(lam), ptr(ev),
                                     ptr(vec), C.byref(n))
    if st not in (0, 10):
        g._check(st, "davidson_trace")
    k = n.value
    return R[:k], X[:k], lam[:k], ev, vec


def make_samples(nocc, nvirt, seed, nstates=6, tol=1e-6, S=2048, rs=None):
    """Training samples of one seeded system: list of (F[S,16], t0[S], e[S])."""
    rs = rs or np.random.RandomState(seed)
    e, eri = api.synth_system(nocc, nvirt, seed)
    g = api.AdcGpu(0)
    g.set_orbitals(nocc, nvirt, e)
    g.set_eri_packed(eri)
    g.write_fspace_adc2_1(None)
    h = g.get_diag()
    d0, cls = config_info(nocc, nvirt, e)
    R, X, lam, ev, vec = trace(g, nstates, tol)
    g.close()
    N = len(h)
    out = []
    for k in range(len(R)):
        for i in range(nstates):
            x = X[k, i]
            ov = vec @ x
            m = int(np.argmax(np.abs(ov)))
            tgt = vec[m] - ov[m] * x
            if np.linalg.norm(tgt) < 1e-8:
                continue
            gap = lam[k, i] - h
            t0 = np.where(gap == 0.0, 0.0, R[k, i] / np.where(gap == 0.0, 1.0, gap))
            idx = rs.choice(N, size=min(S, N), replace=False) if N > S else np.arange(N)
            if len(idx) < S:
                idx = np.concatenate([idx, rs.choice(N, size=S - len(idx), replace=True)])
            F = features(lam[k, i], h[idx], d0[idx], cls[idx])
            ts, es = t0[idx], tgt[idx]
            nt, ne = np.linalg.norm(ts), np.linalg.norm(es)
            if not (np.isfinite(nt) and nt > 0 and ne > 0):
                continue
            # the loss is scale invariant: normalise so FP32 sums cannot overflow
            out.append((F, (ts / nt).astype(np.float32), (es / ne).astype(np.float32)))
    return out


def random_systems(n: int, seed: int = 1000):
    rs = np.random.RandomState(seed)
    return [(int(rs.randint(3, 7)), int(rs.randint(10, 31)), seed + 17 * i) for i in range(n)]


def train(samples, steps: int = 400, G: int = 64, lr: float = 1e-3, seed: int = 0, params=None, log=None):
    """Trains on the GPU with the library's kernels; returns (params, losses)."""
    S = samples[0][0].shape[0]
    g = api.AdcGpu(0)
    p = init_params(seed) if params is None else params.astype(np.float32)
    st = lib().adcgpu_mlp_set_params(g._h, p.ctypes.data_as(_fp), p.size)
    g._check(st, "mlp_set_params")
    rs = np.random.RandomState(seed)
    losses = []
    for it in range(steps):
        pick = rs.choice(len(samples), size=min(G, len(samples)), replace=False)
        F = np.ascontiguousarray(np.concatenate([samples[i][0] for i in pick]))
        T0 = np.ascontiguousarray(np.concatenate([samples[i][1] for i in pick]))
        E = np.ascontiguousarray(np.concatenate([samples[i][2] for i in pick]))
        loss = C.c_float(0.0)
        st = lib().adcgpu_mlp_train_step(g._h, len(pick), S, F.ctypes.data_as(_fp), T0.ctypes.data_as(_fp),
                                         E.ctypes.data_as(_fp), lr, C.byref(loss), None)
        g._check(st, "mlp_train_step")
        losses.append(loss.value)
        if log and it % 50 == 0:
            log(f"step {it} loss {loss.value:.5f}")
    out = np.empty(num_params(), np.float32)
    g._check(lib().adcgpu_mlp_get_params(g._h, out.ctypes.data_as(_fp), out.size), "mlp_get_params")
    g.close()
    return out, np.array(losses)


def gradient(params: np.ndarray, F, T0, E, G: int, S: int):
    """Library gradient (summed over groups) and mean loss for one batch."""
    g = api.AdcGpu(0)
    p = params.astype(np.float32)
    g._check(lib().adcgpu_mlp_set_params(g._h, p.ctypes.data_as(_fp), p.size), "mlp_set_params")
    grad = np.empty(num_params(), np.float32)
    loss = C.c_float(0.0)
    st = lib().adcgpu_mlp_train_step(g._h, G, S, np.ascontiguousarray(F, np.float32).ctypes.data_as(_fp),
                                     np.ascontiguousarray(T0, np.float32).ctypes.data_as(_fp),
                                     np.ascontiguousarray(E, np.float32).ctypes.data_as(_fp), 0.0, C.byref(loss),
                                     grad.ctypes.data_as(_fp))
    g._check(st, "mlp_train_step")
    g.close()
    return grad, loss.value


def load_into(g: api.AdcGpu, params: np.ndarray):
    p = np.ascontiguousarray(params, np.float32)
    g._check(lib().adcgpu_mlp_set_params(g._h, p.ctypes.data_as(_fp), p.size), "mlp_set_params")


def save(path: str, params: np.ndarray):
    np.save(path, params.astype(np.float32))


def load(path: str) -> np.ndarray:
    return np.load(path).astype(np.float32)


DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "mlp_weights.npy")


def evaluate(params, systems, nstates=6, tol=1e-6, maxiter=300):
    """Davidson iterations and time with the diagonal and the learned
    preconditioner on the given (nocc, nvirt, seed) systems (FP64 path)."""
    import time

    rows = []
    for no, nv, seed in systems:
        e, eri = api.synth_system(no, nv, seed)
        g = api.AdcGpu(0)
        g.set_orbitals(no, nv, e)
        g.set_eri_packed(eri)
        g.write_fspace_adc2_1(None)
        t = time.perf_counter()
        r0 = g.davdiag_block(nstates, tol, precon=api.PRECON_DPR, maxiter=maxiter, want_vectors=False,
                             raise_on_nonconv=False)
        t0 = time.perf_counter() - t
        load_into(g, params)
        t = time.perf_counter()
        r1 = g.davdiag_block(nstates, tol, precon=api.PRECON_MLP, maxiter=maxiter, want_vectors=False,
                             raise_on_nonconv=False)
        t1 = time.perf_counter() - t
        g.close()
        rows.append({"nocc": no, "nvirt": nv, "seed": seed, "iters_dpr": r0.iterations, "iters_mlp": r1.iterations,
                     "s_dpr": t0, "s_mlp": t1, "status": [r0.status, r1.status],
                     "max_dE": float(np.abs(r0.evals - r1.evals).max())})
    return rows


def main(argv=None):
    import argparse
    import json
    import time

    ap = argparse.ArgumentParser(description="train the learned Davidson preconditioner on the GPU")
    ap.add_argument("--systems", type=int, default=200)
    ap.add_argument("--steps", type=int, default=600)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--out", default=DEFAULT_WEIGHTS)
    ap.add_argument("--eval", type=int, default=6)
    a = ap.parse_args(argv)
    t = time.time()
    samples = []
    for no, nv, seed in random_systems(a.systems):
        samples += make_samples(no, nv, seed)
    print(f"{len(samples)} samples from {a.systems} systems in {time.time() - t:.1f} s", flush=True)
    t = time.time()
    params, losses = train(samples, steps=a.steps, lr=a.lr, log=print)
    print(f"trained in {time.time() - t:.1f} s: loss {losses[:20].mean():.4f} -> {losses[-20:].mean():.4f}",
          flush=True)
    save(a.out, params)
    held = random_systems(a.eval, seed=99991)
    rows = evaluate(params, held)
    for r in rows:
        print(json.dumps(r), flush=True)
    it0 = sum(r["iters_dpr"] for r in rows)
    it1 = sum(r["iters_mlp"] for r in rows)
    print(json.dumps({"held_out_iters_dpr": it0, "held_out_iters_mlp": it1, "ratio": it1 / max(it0, 1)}), flush=True)


if __name__ == "__main__":
    main()
