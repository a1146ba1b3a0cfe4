"""The compact form of segments A and B that csrc/sigma_ab.cu relies on,
checked on the CPU against the oracle's stored matrix (COO of
get_offdiag_adc2_save_omp, get_matrix.f90:705-1186).

1. In a slab (fixed k', l', class) of the classes with a' < b', the coupling
   of double (a', b', k', l') with single (a', k), k outside {k', l'}, does
   not depend on a' (the coincidence tests of C1/C2/C4_ph_2p2h,
   adc_ph.f90:974-1054, leave only the term in (b', k, k', l')); the
   coupling with (b', k) does not depend on b'.  Entries dropped by the minc
   threshold are dropped for every a' (b') alike.
2. A numpy restatement of the kernels' index arithmetic (slab enumeration,
   the Y/Z tables copied from rows (0, b) and (a, nv-1), the coincident
   entries per row, the storage order of class 2 with its kpq index, phase 1
   over a' < b and phase 2 over the run of a, the row-by-row classes 1 and 3)
   reproduces the segment-A/B part of the oracle's matrix-vector product.
"""
from collections import defaultdict

import numpy as np
import pytest

import oracle


def _matrix(no, nv, seed):
    e, eri = oracle.synth_system(no, nv, seed)
    M = oracle.Matrix.build(no, nv, e, eri)
    d, h, oi, oj = M.coo()
    return oracle.select(no, nv), h, oi, oj


@pytest.mark.parametrize("no,nv,seed", [(5, 19, 3), (4, 12, 7), (3, 9, 11)])
def test_segments_depend_on_one_virtual(no, nv, seed):
    kpq, h, oi, oj = _matrix(no, nv, seed)
    n1 = no * nv
    groups = defaultdict(set)
    for val, i, j in zip(h, oi, oj):
        if not (i <= n1 < j):
            continue
        si, dj = kpq[i], kpq[j]
        a, k = si[4] - no - 1, si[2] - 1
        kp, lp, ap, bp, typ = dj[2] - 1, dj[3] - 1, dj[4] - no - 1, dj[5] - no - 1, dj[6]
        if ap == bp or k in (kp, lp):
            continue
        if a == ap:
            groups[("A", typ, kp, lp, bp, k)].add(val)
        elif a == bp:
            groups[("B", typ, kp, lp, ap, k)].add(val)
    assert groups
    assert all(len(v) == 1 for v in groups.values())


class Geo:
    """The storage geometry of csrc/internal.h (0-based)."""

    def __init__(self, no, nv):
        self.no, self.nv = no, nv
        self.n1 = no * nv
        self.npv, self.npo = nv * (nv - 1) // 2, no * (no - 1) // 2
        c1, c2, c3, c4 = no * nv, self.npv * no, self.npo * nv, self.npo * self.npv
        self.start = [0, c1, c1 + c2, c1 + c2 + c3, c1 + c2 + c3 + c4, c1 + c2 + c3 + 2 * c4]

    @staticmethod
    def pidx(x, y, n):
        return x * n - x * (x + 1) // 2 + (y - x - 1)

    def pdec(self, p, n):
        for x in range(n - 1):
            if self.pidx(x, x + 1, n) <= p < self.pidx(x, x + 1, n) + (n - 1 - x):
                return x, p - self.pidx(x, x + 1, n) + x + 1
        raise ValueError(p)

    def decode_double(self, d):
        no, nv, st = self.no, self.nv, self.start
        if d < st[1]:
            return d % nv, d % nv, d // nv, d // nv, 0
        if d < st[2]:
            t = d - st[1]
            a, b = self.pdec(t // no, nv)
            return a, b, t % no, t % no, 1
        if d < st[3]:
            t = d - st[2]
            k, l = self.pdec(t // nv, no)
            return t % nv, t % nv, k, l, 2
        t, cls = d - st[3], 3
        if t >= st[4] - st[3]:
            t, cls = t - (st[4] - st[3]), 4
        k, l = self.pdec(t // self.npv, no)
        a, b = self.pdec(t % self.npv, nv)
        return a, b, k, l, cls

    def decode_row(self, row):
        if self.start[1] <= row < self.start[2]:
            t = row - self.start[1]
            a, b = self.pdec(t % self.npv, self.nv)
            return a, b, t // self.npv, t // self.npv, 1
        return self.decode_double(row)

    def row_to_d(self, r, row):
        a, b, k, _, cls = r
        return self.start[1] + self.pidx(a, b, self.nv) * self.no + k if cls == 1 else row


@pytest.mark.parametrize("no,nv,seed", [(4, 9, 5), (3, 7, 2)])
def test_compact_kernels_restated_match_oracle(no, nv, seed):
    kpq, h, oi, oj = _matrix(no, nv, seed)
    G = Geo(no, nv)
    n1, n2 = G.n1, G.start[5]
    N = n1 + n2
    H = np.zeros((N, N))
    H[oi - 1, oj - 1] = h
    H[oj - 1, oi - 1] = h
    for d in range(n2):   # the doubles order is select_atom_d's
        a, b, k, l, _ = G.decode_double(d)
        q = kpq[n1 + 1 + d]
        assert (q[2] - 1, q[3] - 1, q[4] - no - 1, q[5] - no - 1) == (k, l, a, b)
    noP = 8 * ((no + 7) // 8)
    segA = np.zeros((n2, noP))
    segB = np.zeros((n2, noP))
    for row in range(n2):
        r = G.decode_row(row)
        a, b = r[0], r[1]
        d = G.row_to_d(r, row)
        for k in range(no):
            segA[row, k] = H[a * no + k, n1 + d]
            if a != b:
                segB[row, k] = H[b * no + k, n1 + d]
    nslab = no + 2 * G.npo

    def pair_slab(s):
        if s < no:
            return 1, s, s, G.start[1] + s * G.npv
        t = s - no
        cls, p = 3 + t // G.npo, t % G.npo
        k, l = G.pdec(p, no)
        return cls, k, l, G.start[cls] + p * G.npv

    Y = np.zeros((nslab, nv, noP))
    Z = np.zeros((nslab, nv, noP))
    for s in range(nslab):
        _, kp, lp, row0 = pair_slab(s)
        for x in range(nv):
            for k in range(no):
                if k in (kp, lp):
                    continue
                if x >= 1:
                    Y[s, x, k] = segA[row0 + G.pidx(0, x, nv), k]
                if x <= nv - 2:
                    Z[s, x, k] = segB[row0 + G.pidx(x, nv - 1, nv), k]
    c2 = G.start[2] - G.start[1]
    nrow = c2 + (G.start[5] - G.start[3])
    coin = np.zeros((nrow, 4))
    for t in range(nrow):
        row = G.start[1] + t if t < c2 else G.start[3] + (t - c2)
        _, _, kp, lp, _ = G.decode_row(row)
        coin[t] = [segA[row, kp], segA[row, lp] if kp != lp else 0.0,
                   segB[row, kp], segB[row, lp] if kp != lp else 0.0]

    def pri(cls, row):
        return row - G.start[1] if cls == 1 else c2 + (row - G.start[3])

    m = 3
    V = np.random.RandomState(seed).standard_normal((N, m))
    V1 = np.zeros((nv, noP, m))
    V1[:, :no] = V[:n1].reshape(nv, no, m)
    W2 = np.zeros((n2, m))
    W1 = np.zeros((n1, m))
    for s in range(nslab):
        cls, kp, lp, row0 = pair_slab(s)
        for b in range(1, nv):                       # phase 1
            accB = np.zeros((noP, m))
            accR = np.zeros(m)
            accS = np.zeros(m)
            for a in range(b):
                pr = G.pidx(a, b, nv)
                row = row0 + pr
                d = G.start[1] + pr * no + kp if cls == 1 else row
                q = coin[pri(cls, row)]
                v2 = V[n1 + d]
                W2[d] += (Z[s, a] @ V1[b] + Y[s, b] @ V1[a] + q[2] * V1[b, kp] + q[3] * V1[b, lp]
                          + q[0] * V1[a, kp] + q[1] * V1[a, lp])
                accB += np.outer(Z[s, a], v2)
                accR += q[2] * v2
                accS += q[3] * v2
            accB[kp] += accR
            accB[lp] += accS
            W1[b * no:(b + 1) * no] += accB[:no]
        for a in range(nv - 1):                      # phase 2
            acc = np.zeros((noP, m))
            pr0 = G.pidx(a, a + 1, nv)
            for b in range(a + 1, nv):
                pr = pr0 + (b - a - 1)
                row = row0 + pr
                d = G.start[1] + pr * no + kp if cls == 1 else row
                q = coin[pri(cls, row)]
                v2 = V[n1 + d]
                acc += np.outer(Y[s, b], v2)
                acc[kp] += q[0] * v2
                acc[lp] += q[1] * v2
            W1[a * no:(a + 1) * no] += acc[:no]
    for a in range(nv):                              # classes 1 and 3, row by row
        for qq in range(no + G.npo):
            row = qq * nv + a if qq < no else G.start[2] + (qq - no) * nv + a
            W2[row] += segA[row, :no] @ V[a * no:(a + 1) * no]
            W1[a * no:(a + 1) * no] += np.outer(segA[row, :no], V[n1 + row])
    # the segment-A/B part of H V, straight from the oracle's matrix
    ref2 = np.zeros((n2, m))
    ref1 = np.zeros((n1, m))
    for row in range(n2):
        r = G.decode_row(row)
        a, b = r[0], r[1]
        d = G.row_to_d(r, row)
        for k in range(no):
            ref2[d] += H[a * no + k, n1 + d] * V[a * no + k]
            ref1[a * no + k] += H[a * no + k, n1 + d] * V[n1 + d]
            if a != b:
                ref2[d] += H[b * no + k, n1 + d] * V[b * no + k]
                ref1[b * no + k] += H[b * no + k, n1 + d] * V[n1 + d]
    assert np.abs(W2 - ref2).max() <= 1e-13 * np.abs(ref2).max()
    assert np.abs(W1 - ref1).max() <= 1e-13 * np.abs(ref1).max()
