// ADC(2)-s matrix build on the GPU (compiled with --fmad=false).
//
// Replaces get_diag_adc2_save (get_matrix.f90:267-311) and
// get_offdiag_adc2_save_omp (get_matrix.f90:705-1186).  Every matrix element
// is evaluated with the reference's operation order (adc_ph.f90), each
// product and sum rounded separately, so an element lands on the same side
// of minc = 1e-12 as in the reference and the kept structure is bit-exact.
//
// ERIs are read from four dense blocks gathered once from the caller's
// integrals (8-fold symmetry makes every (pq|rs) the reference touches one of
// (vo|vo), (vv|oo), (oo|ov), (vv|ov)).
#include <cub/cub.cuh>

#include "internal.h"

namespace adcgpu {

namespace {

struct Eri {
  const double* vovo;
  const double* vvoo;
  const double* ooov;
  const double* vvov;
  int no, nv;
  __device__ double VOVO(int a, int i, int b, int j) const {
    return vovo[(((int64_t)a * no + i) * nv + b) * no + j];
  }
  __device__ double VVOO(int a, int b, int i, int j) const {
    return vvoo[(((int64_t)a * nv + b) * no + i) * no + j];
  }
  __device__ double OOOV(int i, int j, int k, int a) const {
    return ooov[(((int64_t)i * no + j) * no + k) * nv + a];
  }
  __device__ double VVOV(int a, int b, int i, int c) const {
    return vvov[(((int64_t)a * nv + b) * no + i) * nv + c];
  }
};

__host__ __device__ inline int64_t canon(int64_t p, int64_t q, int64_t r, int64_t s) {
  int64_t pq = p >= q ? p * (p + 1) / 2 + q : q * (q + 1) / 2 + p;
  int64_t rs = r >= s ? r * (r + 1) / 2 + s : s * (s + 1) / 2 + r;
  return pq >= rs ? pq * (pq + 1) / 2 + rs : rs * (rs + 1) / 2 + pq;
}

// (P, Q) with P >= Q from the triangular index t = P(P+1)/2 + Q.
__host__ __device__ inline void untri(int64_t t, int64_t& P, int64_t& Q) {
  P = (int64_t)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
  while (P * (P + 1) / 2 > t) --P;
  while ((P + 1) * (P + 2) / 2 <= t) ++P;
  Q = t - P * (P + 1) / 2;
}

// Gather one ERI block from the canonical packed array.
// kind 0: (a i|b j) 1: (a b|i j) 2: (i j|k a) 3: (a b|i c) 4: (i j|k l)
// 5: (a c|b d) packed over virtual pairs, index tri(pair(a,c), pair(b,d))
__global__ void k_gather_block(const double* __restrict__ packed, double* __restrict__ out, int kind,
                               int no, int nv, int64_t total) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    int64_t x = t;
    int p, q, r, s;
    switch (kind) {
      case 4: { int l = x % no; x /= no; int k = x % no; x /= no; int j = x % no; int i = (int)(x / no);
                p = i; q = j; r = k; s = l; } break;
      case 5: { int64_t P, Q, a, c, b, d;
                untri(x, P, Q); untri(P, a, c); untri(Q, b, d);
                p = no + (int)a; q = no + (int)c; r = no + (int)b; s = no + (int)d; } break;
      case 0: { int j = x % no; x /= no; int b = x % nv; x /= nv; int i = x % no; int a = (int)(x / no);
                p = no + a; q = i; r = no + b; s = j; } break;
      case 1: { int j = x % no; x /= no; int i = x % no; x /= no; int b = x % nv; int a = (int)(x / nv);
                p = no + a; q = no + b; r = i; s = j; } break;
      case 2: { int a = x % nv; x /= nv; int k = x % no; x /= no; int j = x % no; int i = (int)(x / no);
                p = i; q = j; r = k; s = no + a; } break;
      default: { int c = x % nv; x /= nv; int i = x % no; x /= no; int b = x % nv; int a = (int)(x / nv);
                 p = no + a; q = no + b; r = i; s = no + c; } break;
    }
    out[t] = packed[canon(p, q, r, s)];
  }
}

// CA_ph_ph(a,a1), adc_ph.f90:769-812, for a <= a1 (0-based virtuals).
__global__ void k_ca(Eri E, const double* __restrict__ e, double* __restrict__ ca) {
  const int no = E.no, nv = E.nv;
  int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= (int64_t)nv * nv) return;
  int a = (int)(t / nv), a1 = (int)(t % nv);
  if (a > a1) return;
  const double ea = e[no + a], ea1 = e[no + a1];
  double acc = 0.0;
  for (int r = 0; r < nv; ++r)
    for (int u = 0; u < no; ++u)
      for (int v = 0; v < no; ++v) {
        double eijc = e[u] + e[v] - e[no + r];
        double DA = (eijc - 0.5 * (ea + ea1)) / ((eijc - ea) * (eijc - ea1));
        double term = 0.0;
        term = term + E.VOVO(a, u, r, v) * (2.0 * E.VOVO(a1, u, r, v) - E.VOVO(r, u, a1, v));
        term = term + E.VOVO(a, v, r, u) * (2.0 * E.VOVO(r, u, a1, v) - E.VOVO(a1, u, r, v));
        term = DA * term;
        acc = acc + term;
      }
  double x = -0.5 * acc;
  ca[(int64_t)a * nv + a1] = x;
  ca[(int64_t)a1 * nv + a] = x;
}

// CB_ph_ph(k,k1), adc_ph.f90:819-912 ("dumbed down" branch), k <= k1, in two
// passes: every term of the (r, s, u) sum of one pair evaluated in parallel
// (the reference's expression, operation by operation), then the terms summed
// in the reference's loop order by one thread per pair.  The result is bit
// for bit that of the serial loop while the divisions run on all SMs.
// terms: [pair][(r*nv + s)*no + u], pairs k <= k1 enumerated row by row.
__global__ void k_cb_terms(Eri E, const double* __restrict__ e, const int2* __restrict__ pairs, int npairs,
                           double* __restrict__ terms) {
  const int no = E.no, nv = E.nv;
  const int64_t nt = (int64_t)nv * nv * no;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < npairs * nt;
       x += (int64_t)gridDim.x * blockDim.x) {
    const int pi = (int)(x / nt);
    const int64_t t = x % nt;
    const int u = (int)(t % no), s = (int)((t / no) % nv), r = (int)(t / ((int64_t)no * nv));
    const int k = pairs[pi].x, k1 = pairs[pi].y;
    const double ek = e[k], ek1 = e[k1];
    double eicd = e[u] - e[no + r] - e[no + s];
    double DB = (eicd + 0.5 * (ek + ek1)) / ((eicd + ek) * (eicd + ek1));
    double term = 0.0;
    term = term + E.VOVO(r, k, s, u) * (2.0 * E.VOVO(r, k1, s, u) - E.VOVO(s, k1, r, u));
    term = term + E.VOVO(r, u, s, k) * (2.0 * E.VOVO(s, k1, r, u) - E.VOVO(r, k1, s, u));
    terms[x] = DB * term;
  }
}

__global__ void k_cb_sum(const double* __restrict__ terms, const int2* __restrict__ pairs, int npairs, int64_t nt,
                         int no, double* __restrict__ cb) {
  const int pi = blockIdx.x * blockDim.x + threadIdx.x;
  if (pi >= npairs) return;
  const double* tp = terms + (int64_t)pi * nt;
  double acc = 0.0;
  for (int64_t t = 0; t < nt; ++t) acc = acc + tp[t];
  const double x = -0.5 * acc;
  const int k = pairs[pi].x, k1 = pairs[pi].y;
  cb[k * no + k1] = x;
  cb[k1 * no + k] = x;
}

// The direct path's intermediates (get_interm_adc2_save, get_matrix.f90
// :625-701): Ca1_ph_ph(a,a1) (adc_ph.f90:98-152) for a <= a1 and
// Cb1_ph_ph(k,k1) (:158-211) for k <= k1, in the reference's operation order.
__global__ void k_ca1(Eri E, const double* __restrict__ e, double* __restrict__ ca) {
  const int no = E.no, nv = E.nv;
  int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= (int64_t)nv * nv) return;
  int a = (int)(t / nv), a1 = (int)(t % nv);
  if (a > a1) return;
  const double ea = e[no + a], ea1 = e[no + a1];
  double acc = 0.0;
  for (int r = 0; r < nv; ++r)
    for (int u = 0; u < no; ++u)
      for (int v = 0; v < no; ++v) {
        const double er = e[no + r];
        double eija = er + ea - e[u] - e[v];
        double eijc = er + ea1 - e[u] - e[v];
        double DA = 1.0 / ((er + ea - e[u] - e[v]) * (er + ea1 - e[u] - e[v]));
        double term = 0.0;
        term = term + eijc * E.VOVO(a1, u, r, v) * (2.0 * E.VOVO(a, u, r, v) - E.VOVO(r, u, a, v));
        term = term + eija * E.VOVO(a, v, r, u) * (2.0 * E.VOVO(r, u, a1, v) - E.VOVO(a1, u, r, v));
        term = DA * term;
        acc = acc + term;
      }
  double x = 0.5 * acc;
  ca[(int64_t)a * nv + a1] = x;
  ca[(int64_t)a1 * nv + a] = x;
}

__global__ void k_cb1(Eri E, const double* __restrict__ e, double* __restrict__ cb) {
  const int no = E.no, nv = E.nv;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= no * no) return;
  int k = t / no, k1 = t % no;
  if (k > k1) return;
  const double ek = e[k], ek1 = e[k1];
  double acc = 0.0;
  for (int r = 0; r < nv; ++r)
    for (int s = 0; s < nv; ++s)
      for (int u = 0; u < no; ++u) {
        const double er = e[no + r], es = e[no + s];
        double eicd = er + es - e[u] - ek;
        double ejcd = er + es - e[u] - ek1;
        double DB = 1.0 / ((er + es - e[u] - ek) * (er + es - e[u] - ek1));
        double term = 0.0;
        term = term + ejcd * E.VOVO(r, k1, s, u) * (2.0 * E.VOVO(r, k, s, u) - E.VOVO(s, k, r, u));
        term = term + eicd * E.VOVO(r, u, s, k) * (2.0 * E.VOVO(s, k1, r, u) - E.VOVO(r, k1, s, u));
        term = DB * term;
        acc = acc + term;
      }
  double x = 0.5 * acc;
  cb[k * no + k1] = x;
  cb[k1 * no + k] = x;
}

// Per (single, (c,i)) tables for CC_ph_ph (adc_ph.f90:918-957):
//   X[s][t]  = 2 (a k|c i) - (a i|c k)       the first factor of term
//   D1[s][t] = e(k) - e(a) + (e(i) - e(c))   one factor of the DC denominator
// with t = c*no + i (c outer, i inner: the reference's loop order).
// DIRECT: D1[s][t] = 1 / (e(c) + e(a) - e(i) - e(k)), the DC factor of
// Cc1_ph_ph / Cc2_ph_ph (adc_ph.f90:214-303) for the single s = (a,k).
template <bool DIRECT>
__global__ void k_cc_tables(Eri E, const double* __restrict__ e, double* __restrict__ X,
                            double* __restrict__ D1) {
  const int no = E.no, nv = E.nv;
  const int64_t n1 = (int64_t)no * nv, nt = n1;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n1 * nt;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t s = idx / nt, t = idx % nt;
    int a = (int)(s / no), k = (int)(s % no);
    int c = (int)(t / no), i = (int)(t % no);
    X[idx] = 2.0 * E.VOVO(a, k, c, i) - E.VOVO(a, i, c, k);
    if (DIRECT) {
      D1[idx] = 1.0 / (e[no + c] + e[no + a] - e[i] - e[k]);
    } else {
      double eic = e[i] - e[no + c];
      D1[idx] = e[k] - e[no + a] + eic;
    }
  }
}

constexpr int PT = 16;   // ph-ph tile (PT x PT elements per block)
constexpr int TK = 32;   // t-chunk staged in shared memory

// ph-ph block (get_matrix.f90:848-884) and singles diagonal (:286-294).
// Each thread evaluates one element (s1 <= s2) with the exact serial CC sum.
// DIRECT: the direct path's ph-ph block (dmatvec_davidson.f90:1100-1107)
// and singles diagonal (hiivec :917-924): Ca1/Cb1 intermediates and the two
// serial sums Cc1_ph_ph and Cc2_ph_ph instead of CC_ph_ph.
template <bool DIRECT>
__global__ void __launch_bounds__(PT * PT) k_phph(Eri E, const double* __restrict__ e,
                                                  const double* __restrict__ X, const double* __restrict__ D1,
                                                  const double* __restrict__ ca, const double* __restrict__ cb,
                                                  double* __restrict__ A, double* __restrict__ hii,
                                                  unsigned long long* __restrict__ kept) {
  const int no = E.no, nv = E.nv;
  const int n1 = no * nv, nt = n1;
  const int bi = blockIdx.y, bj = blockIdx.x;
  if (bj < bi) return;                 // upper-triangle tiles only
  __shared__ double sX1[PT][TK + 1], sD1[PT][TK + 1], sX2[PT][TK + 1], sD2[PT][TK + 1], sEic[TK];
  const int ty = threadIdx.y, tx = threadIdx.x;
  const int s1 = bi * PT + ty, s2 = bj * PT + tx;
  const int tid = ty * PT + tx;
  double hv = 0.0;
  if (s1 < n1 && s2 < n1) {
    int a = s1 / no, k = s1 % no, a1 = s2 / no, k1 = s2 % no;
    hv = 0.5 * (e[k] + e[k1] - e[no + a] - e[no + a1]);
  }
  double cc = 0.0, cc2 = 0.0;
  for (int t0 = 0; t0 < nt; t0 += TK) {
    __syncthreads();
    for (int l = tid; l < PT * TK; l += PT * PT) {
      int r = l / TK, c = l % TK;
      int t = t0 + c;
      int r1 = bi * PT + r, r2 = bj * PT + r;
      bool ok = t < nt;
      sX1[r][c] = (ok && r1 < n1) ? X[(int64_t)r1 * nt + t] : 0.0;
      sD1[r][c] = (ok && r1 < n1) ? D1[(int64_t)r1 * nt + t] : 1.0;
      sX2[r][c] = (ok && r2 < n1) ? X[(int64_t)r2 * nt + t] : 0.0;
      sD2[r][c] = (ok && r2 < n1) ? D1[(int64_t)r2 * nt + t] : 1.0;
    }
    for (int l = tid; l < TK; l += PT * PT) {
      int t = t0 + l;
      sEic[l] = t < nt ? (e[t % no] - e[no + t / no]) : 0.0;
    }
    __syncthreads();
    const int tl = min(TK, nt - t0);
    if (DIRECT) {
      for (int c = 0; c < tl; ++c) {
        const double term = sX1[ty][c] * sX2[tx][c];
        cc = cc + term * sD1[ty][c];     // Cc1: DC of (a, k)
        cc2 = cc2 + term * sD2[tx][c];   // Cc2: DC of (a1, k1)
      }
    } else {
      for (int c = 0; c < tl; ++c) {
        double DC = (hv + sEic[c]) / (sD1[ty][c] * sD2[tx][c]);
        double term = sX1[ty][c] * sX2[tx][c];
        term = term * DC;
        cc = cc + term;
      }
    }
  }
  if (s1 >= n1 || s2 >= n1 || s2 < s1) return;
  const int a = s1 / no, k = s1 % no, a1 = s2 / no, k1 = s2 % no;
  if (s1 == s2) {
    double x = e[no + a] - e[k];                                   // K_ph_ph
    x = x + (2.0 * E.VOVO(a, k, a, k) - E.VVOO(a, a, k, k));       // C1_ph_ph
    x = x + ca[(int64_t)a * nv + a];                               // CA (Ca1)(a,a)
    x = x + cb[k * no + k];                                        // CB (Cb1)(k,k)
    if (DIRECT) {
      x = x + -0.5 * cc;                                           // Cc1_ph_ph
      x = x + -0.5 * cc2;                                          // Cc2_ph_ph
    } else {
      x = x + cc;                                                  // CC_ph_ph
    }
    hii[s1] = x;
    A[(int64_t)s1 * n1 + s1] = 0.0;
    return;
  }
  double x = 2.0 * E.VOVO(a, k, a1, k1) - E.VVOO(a, a1, k, k1);  // C1_ph_ph
  if (k == k1) x = x + ca[(int64_t)a * nv + a1];
  if (a == a1) x = x + cb[k * no + k1];
  if (DIRECT) {
    x = x + -0.5 * cc;
    x = x + -0.5 * cc2;
  } else {
    x = x + cc;
  }
  double keep = fabs(x) > MINC ? x : 0.0;
  A[(int64_t)s1 * n1 + s2] = keep;
  A[(int64_t)s2 * n1 + s1] = keep;
  if (keep != 0.0) atomicAdd(kept, 1ull);
}

// ADC(1) (TDA) matrix of the singles, dense n1 x n1: get_diag_tda_direct
// (K_ph_ph + C1_ph_ph(a,k,a,k)) and get_offdiag_tda_direct (C1_ph_ph), the
// matrix whose eigenvectors adc1_guessvecs writes for initvec_adc1
// (get_matrix.f90:17-82, guessvecs.f90:9-84).
__global__ void k_tda(Eri E, const double* __restrict__ e, double* __restrict__ M) {
  const int no = E.no, nv = E.nv;
  const int64_t n1 = (int64_t)no * nv;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n1 * n1;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s1 = t / n1, s2 = t % n1;
    const int a = (int)(s1 / no), k = (int)(s1 % no), a1 = (int)(s2 / no), k1 = (int)(s2 % no);
    double x = 2.0 * E.VOVO(a, k, a1, k1) - E.VVOO(a, a1, k, k1);   // C1_ph_ph
    if (s1 == s2) x = (e[no + a] - e[k]) + x;                        // K_ph_ph + C1_ph_ph
    M[t] = x;
  }
}

// 2p2h diagonal K_2p2h_2p2h (get_matrix.f90:303-306, adc_ph.f90:1090-1096).
__global__ void k_diag2(GeomDev g, const double* __restrict__ e, double* __restrict__ hii) {
  for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < g.n2;
       d += (int64_t)gridDim.x * blockDim.x) {
    Double r = decode_double(g, d);
    const int no = g.no;
    hii[g.n1 + d] = e[no + r.ap] + e[no + r.bp] - e[r.kp] - e[r.lp];
  }
}

// ph-2p2h coupling value of single (a,k) with double r (adc_ph.f90:974-1073),
// in the argument mapping of get_matrix.f90:900,931,964,997,1030.
__device__ inline double coupling(const Eri& E, int a, int k, const Double& r) {
  const int ap = r.ap, bp = r.bp, kp = r.kp, lp = r.lp;
  double f = 0.0;
  switch (r.cls) {
    case 0:   // C5_ph_2p2h(a,k,a',k')
      if (a == ap) f = f + E.OOOV(kp, k, kp, ap);
      if (k == kp) f = f - E.VVOV(a, ap, kp, ap);
      return sqrt(2.0) * f;
    case 1:   // C4_ph_2p2h(a,k,a',b',k')
      if (a == ap) f = f + E.OOOV(kp, k, kp, bp);
      if (a == bp) f = f + E.OOOV(kp, k, kp, ap);
      if (k == kp) f = f - (E.VVOV(a, ap, kp, bp) + E.VVOV(a, bp, kp, ap));
      return f;
    case 2:   // C3_ph_2p2h(a,k,a',k',l')
      if (a == ap) f = f - (E.OOOV(kp, k, lp, ap) + E.OOOV(lp, k, kp, ap));
      if (k == kp) f = f + E.VVOV(a, ap, lp, ap);
      if (k == lp) f = f + E.VVOV(a, ap, kp, ap);
      return f;
    case 3:   // C1_ph_2p2h(a,k,a',b',k',l')
      if (a == ap) f = f - (E.OOOV(kp, k, lp, bp) + E.OOOV(lp, k, kp, bp));
      if (a == bp) f = f - (E.OOOV(kp, k, lp, ap) + E.OOOV(lp, k, kp, ap));
      if (k == kp) f = f + (E.VVOV(a, ap, lp, bp) + E.VVOV(a, bp, lp, ap));
      if (k == lp) f = f + (E.VVOV(a, ap, kp, bp) + E.VVOV(a, bp, kp, ap));
      return f / sqrt(2.0);
    default:  // C2_ph_2p2h(a,k,a',b',k',l')
      if (a == ap) f = f - (E.OOOV(kp, k, lp, bp) - E.OOOV(lp, k, kp, bp));
      if (a == bp) f = f + (E.OOOV(kp, k, lp, ap) - E.OOOV(lp, k, kp, ap));
      if (k == kp) f = f + (E.VVOV(a, ap, lp, bp) - E.VVOV(a, bp, lp, ap));
      if (k == lp) f = f - (E.VVOV(a, ap, kp, bp) - E.VVOV(a, bp, kp, ap));
      return sqrt(3.0) * f / sqrt(2.0);
  }
}

// One warp per stored row of B^T: evaluates its structural entries, applies
// the minc threshold (get_matrix.f90:904 etc.), zeroes the padding and counts
// the kept entries.
// Rows [row_begin, row_end) of the store; Bt holds the values from the
// value offset vbase on (the whole store: vbase = 0; one chunk of the direct
// path: vbase = the chunk's first value).  rowcount may be null.
__global__ void k_coupling(Eri E, GeomDev g, double* __restrict__ Bt, int64_t vbase, int64_t row_begin,
                           int64_t row_end, int64_t* __restrict__ rowcount) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t row_i = row_begin + warp; row_i < row_end; row_i += nwarps) {
    Double r = decode_row(g, row_i);
    const int64_t L = g.len[r.cls];
    double* row = Bt + (g.off[r.cls] + (row_i - g.start[r.cls]) * L - vbase);
    int cnt = 0;
    for (int e = lane; e < L; e += 32) {
      int64_t s = entry_single(g, r, e);
      double x = 0.0;
      if (s >= 0) {
        int a = (int)(s / g.no), k = (int)(s % g.no);
        x = coupling(E, a, k, r);
      }
      bool keep = s >= 0 && fabs(x) > MINC;
      row[e] = keep ? x : 0.0;
      cnt += keep;
    }
    for (int o = 16; o; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if (lane == 0 && rowcount) rowcount[row_i] = cnt;
  }
}

// CVS build ------------------------------------------------------------------
// ph-ph block of the core singles (get_offdiag_adc2_save_cvs_omp, get_matrix.f90
// :1452-1478) and their diagonal (get_diag_adc2_save :286-294).  The element
// (i, j < i) is evaluated with row i's indices first, as the reference's loop
// (j = 1..i-1) does; CC_ph_ph is the same serial sum over (c, i) as k_phph.
// sidx[i] is the ADC(2)-s single index of CVS single i.
__global__ void k_phph_cvs(Eri E, const double* __restrict__ e, const double* __restrict__ X,
                           const double* __restrict__ D1, const double* __restrict__ ca,
                           const double* __restrict__ cb, const int32_t* __restrict__ sidx, int cn1,
                           double* __restrict__ Ac, double* __restrict__ hii, unsigned long long* __restrict__ kept) {
  const int no = E.no, nv = E.nv;
  const int64_t n1 = (int64_t)no * nv;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)cn1 * cn1;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t / cn1), j = (int)(t % cn1);
    if (j > i) continue;
    const int64_t s1 = sidx[i], s2 = sidx[j];
    const int a = (int)(s1 / no), k = (int)(s1 % no), a1 = (int)(s2 / no), k1 = (int)(s2 % no);
    const double hv = 0.5 * (e[k] + e[k1] - e[no + a] - e[no + a1]);
    double cc = 0.0;
    for (int64_t u = 0; u < n1; ++u) {
      const double eic = e[u % no] - e[no + u / no];
      const double DC = (hv + eic) / (D1[s1 * n1 + u] * D1[s2 * n1 + u]);
      double term = X[s1 * n1 + u] * X[s2 * n1 + u];
      term = term * DC;
      cc = cc + term;
    }
    if (i == j) {
      double x = e[no + a] - e[k];                                   // K_ph_ph
      x = x + (2.0 * E.VOVO(a, k, a, k) - E.VVOO(a, a, k, k));       // C1_ph_ph
      x = x + ca[(int64_t)a * nv + a];
      x = x + cb[k * no + k];
      x = x + cc;
      hii[i] = x;
      Ac[(int64_t)i * cn1 + i] = x;
      continue;
    }
    double x = 2.0 * E.VOVO(a, k, a1, k1) - E.VVOO(a, a1, k, k1);
    if (k == k1) x = x + ca[(int64_t)a * nv + a1];
    if (a == a1) x = x + cb[k * no + k1];
    x = x + cc;
    const double keep = fabs(x) > MINC ? x : 0.0;
    Ac[(int64_t)i * cn1 + j] = keep;
    Ac[(int64_t)j * cn1 + i] = keep;
    if (keep != 0.0) atomicAdd(kept, 1ull);
  }
}

// A CVS double row from its kpq column (7 int32: cnf, spin, k, l, a, b, type;
// 1-based orbitals); type 3, 4, 5 map to the classes a=b,i<j / 4I / 4II.
__device__ inline Double cvs_row(const int32_t* q, int no) {
  Double r;
  r.kp = q[2] - 1; r.lp = q[3] - 1;
  r.ap = q[4] - no - 1; r.bp = q[5] - no - 1;
  r.cls = q[6] - 1;
  return r;
}

// Candidate e of a CVS double row: the core singles that the coincidence
// tests of C1/C2/C3_ph_2p2h can reach, (a',k), (b',k) for core k, then
// (a,k') and (a,l') for the core one of k', l' (a not in {a',b'}).  Returns
// the CVS single index a*ncore + corepos[k], or -1.
__device__ inline int cvs_candidate(const Double& r, int e, int nv, int ncore, const int* __restrict__ corepos,
                                    const int* __restrict__ coreorb, int& a, int& k) {
  if (e < ncore) { a = r.ap; k = coreorb[e]; }
  else if (e < 2 * ncore) { if (r.ap == r.bp) return -1; a = r.bp; k = coreorb[e - ncore]; }
  else if (e < 2 * ncore + nv) { a = e - 2 * ncore; k = r.kp; if (corepos[k] < 0 || a == r.ap || a == r.bp) return -1; }
  else { a = e - 2 * ncore - nv; k = r.lp; if (corepos[k] < 0 || a == r.ap || a == r.bp) return -1; }
  return a * ncore + corepos[k];
}

// One warp per CVS double row: count (FILL = false) or write (FILL = true)
// the kept coupling entries (|x| > minc, get_matrix.f90:1503-1620).
template <bool FILL>
__global__ void k_cvs_coupling(Eri E, const int32_t* __restrict__ cols, int64_t n2, int ncore,
                               const int* __restrict__ corepos, const int* __restrict__ coreorb,
                               int64_t* __restrict__ rowcnt, const int64_t* __restrict__ rowptr,
                               int32_t* __restrict__ ccol, double* __restrict__ cval) {
  const int lane = threadIdx.x & 31;
  const int no = E.no, nv = E.nv;
  const int L = 2 * ncore + 2 * nv;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t row = warp; row < n2; row += nwarps) {
    const Double r = cvs_row(cols + 7 * row, no);
    int cnt = 0;
    int64_t base = FILL ? rowptr[row] : 0;
    for (int e0 = 0; e0 < L; e0 += 32) {
      const int e = e0 + lane;
      int a = 0, k = 0, j = -1;
      double x = 0.0;
      if (e < L) j = cvs_candidate(r, e, nv, ncore, corepos, coreorb, a, k);
      if (j >= 0) x = coupling(E, a, k, r);
      const bool keep = j >= 0 && fabs(x) > MINC;
      const unsigned m = __ballot_sync(0xffffffffu, keep);
      if (FILL && keep) {
        const int64_t o = base + __popc(m & ((1u << lane) - 1));
        ccol[o] = j;
        cval[o] = x;
      }
      base += __popc(m);
      cnt += __popc(m);
    }
    if (!FILL && lane == 0) rowcnt[row] = cnt;
  }
}

// K_2p2h_2p2h of the CVS doubles (get_diag_adc2_save :298-301)
__global__ void k_cvs_diag2(const int32_t* __restrict__ cols, int64_t n2, int no, const double* __restrict__ e,
                            double* __restrict__ hii) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n2; t += (int64_t)gridDim.x * blockDim.x) {
    const Double r = cvs_row(cols + 7 * t, no);
    hii[t] = e[no + r.ap] + e[no + r.bp] - e[r.kp] - e[r.lp];
  }
}

// COO export -----------------------------------------------------------------
__global__ void k_count_phph_rows(const double* __restrict__ A, int n1, int64_t* __restrict__ cnt) {
  int s1 = blockIdx.x;
  int c = 0;
  for (int s2 = s1 + 1 + threadIdx.x; s2 < n1; s2 += blockDim.x) c += A[(int64_t)s1 * n1 + s2] != 0.0;
  __shared__ int red[32];
  for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    cnt[s1] = t;
  }
}

__global__ void k_export_phph(const double* __restrict__ A, int n1, const int64_t* __restrict__ pos,
                              double* __restrict__ h, int32_t* __restrict__ oi, int32_t* __restrict__ oj) {
  // one block per row; the block compacts in order with a warp-ballot scan
  int s1 = blockIdx.x;
  __shared__ int64_t base;
  __shared__ int wsum[32];
  if (threadIdx.x == 0) base = pos[s1];
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int s0 = s1 + 1; s0 < n1; s0 += blockDim.x) {
    int s2 = s0 + threadIdx.x;
    double x = s2 < n1 ? A[(int64_t)s1 * n1 + s2] : 0.0;
    bool k = s2 < n1 && x != 0.0;
    unsigned m = __ballot_sync(0xffffffffu, k);
    int before = __popc(m & ((1u << lane) - 1));
    if (lane == 0) wsum[w] = __popc(m);
    __syncthreads();
    int64_t off = base;
    for (int q = 0; q < w; ++q) off += wsum[q];
    if (k) { h[off + before] = x; oi[off + before] = s1 + 1; oj[off + before] = s2 + 1; }
    __syncthreads();
    if (threadIdx.x == 0) { int64_t t = 0; for (int q = 0; q < nw; ++q) t += wsum[q]; base += t; }
    __syncthreads();
  }
}

__global__ void k_export_coupling(GeomDev g, const double* __restrict__ Bt, const int64_t* __restrict__ pos,
                                  double* __restrict__ h, int32_t* __restrict__ oi, int32_t* __restrict__ oj) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t row_i = warp; row_i < g.n2; row_i += nwarps) {
    Double r = decode_row(g, row_i);
    const int64_t d = row_to_d(g, r, row_i);
    const int64_t L = g.len[r.cls];
    const double* row = Bt + g.off[r.cls] + (row_i - g.start[r.cls]) * L;
    int64_t base = pos[row_i];
    for (int e0 = 0; e0 < L; e0 += 32) {
      int e = e0 + lane;
      double x = e < L ? row[e] : 0.0;
      bool k = e < L && x != 0.0;
      unsigned m = __ballot_sync(0xffffffffu, k);
      if (k) {
        int64_t o = base + __popc(m & ((1u << lane) - 1));
        h[o] = x;
        oi[o] = (int32_t)(entry_single(g, r, e) + 1);
        oj[o] = (int32_t)(g.n1 + d + 1);
      }
      base += __popc(m);
    }
  }
}

inline int grid_for(const Ctx* c, int64_t n, int block) {
  int64_t g = (n + block - 1) / block;
  return (int)std::min<int64_t>(std::max<int64_t>(g, 1), (int64_t)c->nsm * 32);
}

}  // namespace

int build_eri_blocks_from_packed(Ctx* c, const double* d_packed) {
  const int no = c->geom.no, nv = c->geom.nv;
  const int64_t npv = (int64_t)nv * (nv + 1) / 2;
  const int64_t sz[6] = {(int64_t)nv * no * nv * no, (int64_t)nv * nv * no * no,
                         (int64_t)no * no * no * nv, (int64_t)nv * nv * no * nv,
                         (int64_t)no * no * no * no, npv * (npv + 1) / 2};
  double** dst[6] = {&c->d_vovo, &c->d_vvoo, &c->d_ooov, &c->d_vvov, &c->d_oooo, &c->d_vvvv};
  for (int k = 0; k < 6; ++k) {
    if (*dst[k]) { dfree(c, *dst[k], 0); *dst[k] = nullptr; }
    int st = dmalloc(c, (void**)dst[k], sizeof(double) * sz[k]);
    if (st) return st;
    k_gather_block<<<grid_for(c, sz[k], 256), 256, 0, c->stream>>>(d_packed, *dst[k], k, no, nv, sz[k]); ADC_COUNT_LAUNCH();
    ADC_CUDA(c, cudaGetLastError());
  }
  ADC_CUDA(c, cudaStreamSynchronize(c->stream));
  return ADCGPU_OK;
}

int build_adc1_matrix(Ctx* c, double* d_M) {
  if (!c->d_vovo || !c->d_vvoo) return set_err(c, ADCGPU_NO_MATRIX, "ADC(1) matrix: integrals missing");
  Eri E{c->d_vovo, c->d_vvoo, c->d_ooov, c->d_vvov, c->geom.no, c->geom.nv};
  k_tda<<<grid_for(c, c->geom.n1 * c->geom.n1, 256), 256, 0, c->stream>>>(E, c->d_e, d_M); ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  return ADCGPU_OK;
}

int coupling_values(Ctx* c, double* buf, int64_t vbase, int64_t row0, int64_t row1, int64_t* rowcount) {
  Eri E{c->d_vovo, c->d_vvoo, c->d_ooov, c->d_vvov, c->geom.no, c->geom.nv};
  k_coupling<<<c->nsm * 8, 256, 0, c->stream>>>(E, to_dev(c->geom), buf, vbase, row0, row1, rowcount);
  ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  return ADCGPU_OK;
}

// CB_ph_ph for all k <= k1 (two passes: k_cb_terms + k_cb_sum; pairs in
// batches that keep the term buffer near 1 GiB)
static int compute_cb(Ctx* c, const Eri& E, double* d_cb) {
  const int no = E.no, nv = E.nv;
  const int64_t nt = (int64_t)nv * nv * no;
  std::vector<int2> pairs;
  for (int k = 0; k < no; ++k)
    for (int k1 = k; k1 < no; ++k1) pairs.push_back(make_int2(k, k1));
  const int np = (int)pairs.size();
  const int batch = (int)std::max<int64_t>(1, std::min<int64_t>(np, ((int64_t)1 << 27) / nt));
  int2* d_pairs = nullptr;
  double* d_terms = nullptr;
  int st = dmalloc(c, (void**)&d_pairs, sizeof(int2) * np);
  if (!st) st = dmalloc(c, (void**)&d_terms, sizeof(double) * (size_t)batch * nt);
  if (!st && cudaMemcpyAsync(d_pairs, pairs.data(), sizeof(int2) * np, cudaMemcpyHostToDevice, c->stream) != cudaSuccess)
    st = set_err(c, ADCGPU_CUDA_ERROR, "CB pairs");
  for (int p0 = 0; !st && p0 < np; p0 += batch) {
    const int nb = std::min(batch, np - p0);
    k_cb_terms<<<grid_for(c, (int64_t)nb * nt, 256), 256, 0, c->stream>>>(E, c->d_e, d_pairs + p0, nb, d_terms);
    ADC_COUNT_LAUNCH();
    k_cb_sum<<<(nb + 31) / 32, 32, 0, c->stream>>>(d_terms, d_pairs + p0, nb, nt, no, d_cb);
    ADC_COUNT_LAUNCH();
    if (cudaGetLastError() != cudaSuccess) st = set_err(c, ADCGPU_CUDA_ERROR, "CB kernels");
  }
  if (!st && cudaStreamSynchronize(c->stream) != cudaSuccess) st = set_err(c, ADCGPU_CUDA_ERROR, "CB kernels");
  dfree(c, d_terms);
  dfree(c, d_pairs);
  return st;
}

int build_matrix(Ctx* c) {
  const Geometry& G = c->geom;
  const int no = G.no, nv = G.nv;
  const int64_t n1 = G.n1;
  GeomDev g = to_dev(G);
  Eri E{c->d_vovo, c->d_vvoo, c->d_ooov, c->d_vvov, no, nv};
  cudaStream_t s = c->stream;
  double *d_ca = nullptr, *d_cb = nullptr, *d_X = nullptr, *d_D1 = nullptr;
  unsigned long long* d_kept = nullptr;
  int st;
  if ((st = dmalloc(c, (void**)&d_ca, sizeof(double) * nv * nv))) return st;
  if ((st = dmalloc(c, (void**)&d_cb, sizeof(double) * no * no))) return st;
  if ((st = dmalloc(c, (void**)&d_X, sizeof(double) * n1 * n1))) return st;
  if ((st = dmalloc(c, (void**)&d_D1, sizeof(double) * n1 * n1))) return st;
  if ((st = dmalloc(c, (void**)&d_kept, sizeof(unsigned long long)))) return st;
  ADC_CUDA(c, cudaMemsetAsync(d_kept, 0, sizeof(unsigned long long), s));
  if (!c->d_diag && (st = dmalloc(c, (void**)&c->d_diag, sizeof(double) * G.N))) return st;
  if (!c->d_A && (st = dmalloc(c, (void**)&c->d_A, sizeof(double) * n1 * n1))) return st;
  // the stored path keeps all of B^T; the direct path one chunk at a time
  int64_t bt_values = G.off[5];
  if (c->direct) {
    c->dchunks = direct_chunk_rows(G, direct_budget(G));
    bt_values = 0;
    for (const DirectChunk& dc : c->dchunks) bt_values = std::max(bt_values, dc.vlen);
  }
  if (!c->d_Bt && (st = dmalloc(c, (void**)&c->d_Bt, sizeof(double) * bt_values))) return st;
  if (!c->d_rowcount && (st = dmalloc(c, (void**)&c->d_rowcount, sizeof(int64_t) * (G.n2 + n1 + 1))))
    return st;

  dim3 tiles((unsigned)((n1 + PT - 1) / PT), (unsigned)((n1 + PT - 1) / PT));
  if (c->direct) {
    // the direct path's formulas (get_interm_adc2_save, hiivec, get_matvec_adc2s_omp)
    k_ca1<<<(int)((nv * (int64_t)nv + 127) / 128), 128, 0, s>>>(E, c->d_e, d_ca); ADC_COUNT_LAUNCH();
    k_cb1<<<(no * no + 63) / 64, 64, 0, s>>>(E, c->d_e, d_cb); ADC_COUNT_LAUNCH();
    k_cc_tables<true><<<grid_for(c, n1 * n1, 256), 256, 0, s>>>(E, c->d_e, d_X, d_D1); ADC_COUNT_LAUNCH();
    ADC_CUDA(c, cudaGetLastError());
    k_phph<true><<<tiles, dim3(PT, PT), 0, s>>>(E, c->d_e, d_X, d_D1, d_ca, d_cb, c->d_A, c->d_diag, d_kept);
    ADC_COUNT_LAUNCH();
  } else {
    k_ca<<<(int)((nv * (int64_t)nv + 127) / 128), 128, 0, s>>>(E, c->d_e, d_ca); ADC_COUNT_LAUNCH();
    ST(compute_cb(c, E, d_cb));
    k_cc_tables<false><<<grid_for(c, n1 * n1, 256), 256, 0, s>>>(E, c->d_e, d_X, d_D1); ADC_COUNT_LAUNCH();
    ADC_CUDA(c, cudaGetLastError());
    k_phph<false><<<tiles, dim3(PT, PT), 0, s>>>(E, c->d_e, d_X, d_D1, d_ca, d_cb, c->d_A, c->d_diag, d_kept);
    ADC_COUNT_LAUNCH();
  }
  ADC_CUDA(c, cudaGetLastError());
  k_diag2<<<grid_for(c, G.n2, 256), 256, 0, s>>>(g, c->d_e, c->d_diag); ADC_COUNT_LAUNCH();
  if (c->direct) {
    // the kept count (noffd) from one pass over the chunks; no values stay
    for (const DirectChunk& dc : c->dchunks)
      ST(coupling_values(c, c->d_Bt, dc.vbase, dc.row0, dc.row1, c->d_rowcount + n1));
  } else {
    ST(coupling_values(c, c->d_Bt, 0, 0, G.n2, c->d_rowcount + n1));
  }
  ADC_CUDA(c, cudaGetLastError());
  unsigned long long kept_ph = 0;
  ADC_CUDA(c, cudaMemcpyAsync(&kept_ph, d_kept, sizeof(kept_ph), cudaMemcpyDeviceToHost, s));
  // total kept coupling entries
  int64_t* d_sum = nullptr;
  if ((st = dmalloc(c, (void**)&d_sum, sizeof(int64_t)))) return st;
  size_t tmp_bytes = 0;
  cub::DeviceReduce::Sum(nullptr, tmp_bytes, c->d_rowcount + n1, d_sum, G.n2, s);
  void* d_tmp = nullptr;
  if ((st = dmalloc(c, &d_tmp, tmp_bytes))) return st;
  cub::DeviceReduce::Sum(d_tmp, tmp_bytes, c->d_rowcount + n1, d_sum, G.n2, s);
  int64_t kept_b = 0;
  ADC_CUDA(c, cudaMemcpyAsync(&kept_b, d_sum, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  ADC_CUDA(c, cudaStreamSynchronize(s));
  c->nnz_ph = (int64_t)kept_ph;
  c->nnz_kept = (int64_t)kept_ph + kept_b;
  dfree(c, d_tmp, tmp_bytes);
  dfree(c, d_sum, sizeof(int64_t));
  dfree(c, d_ca, sizeof(double) * nv * nv);
  dfree(c, d_cb, sizeof(double) * no * no);
  dfree(c, d_X, sizeof(double) * n1 * n1);
  dfree(c, d_D1, sizeof(double) * n1 * n1);
  dfree(c, d_kept, sizeof(unsigned long long));
  return ADCGPU_OK;
}

int export_coo_device(Ctx* c, double* d_h, int32_t* d_oi, int32_t* d_oj) {
  const Geometry& G = c->geom;
  const int n1 = (int)G.n1;
  GeomDev g = to_dev(G);
  cudaStream_t s = c->stream;
  int64_t* d_cnt = c->d_rowcount;      // [0,n1): ph-ph rows, [n1, n1+n2): doubles
  k_count_phph_rows<<<n1, 256, 0, s>>>(c->d_A, n1, d_cnt); ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  int64_t* d_pos = nullptr;
  int st;
  const int64_t nrows = G.n1 + G.n2;
  if ((st = dmalloc(c, (void**)&d_pos, sizeof(int64_t) * (nrows + 1)))) return st;
  size_t tmp_bytes = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, d_cnt, d_pos, nrows, s);
  void* d_tmp = nullptr;
  if ((st = dmalloc(c, &d_tmp, tmp_bytes))) return st;
  cub::DeviceScan::ExclusiveSum(d_tmp, tmp_bytes, d_cnt, d_pos, nrows, s);
  k_export_phph<<<n1, 256, 0, s>>>(c->d_A, n1, d_pos, d_h, d_oi, d_oj); ADC_COUNT_LAUNCH();
  k_export_coupling<<<c->nsm * 8, 256, 0, s>>>(g, c->d_Bt, d_pos + n1, d_h, d_oi, d_oj); ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  ADC_CUDA(c, cudaStreamSynchronize(s));
  dfree(c, d_tmp, tmp_bytes);
  dfree(c, d_pos, sizeof(int64_t) * (nrows + 1));
  return ADCGPU_OK;
}


int build_matrix_cvs(Ctx* c, const int32_t* kpq, int64_t ndim, int ncore, const int32_t* core) {
  const Geometry& G = c->geom;
  const int no = G.no, nv = G.nv;
  const int64_t n1 = G.n1;
  const int cn1 = kpq[0];
  const int64_t n2 = ndim - cn1;
  Eri E{c->d_vovo, c->d_vvoo, c->d_ooov, c->d_vvov, no, nv};
  cudaStream_t s = c->stream;
  std::vector<int> corepos(no, -1), coreorb(ncore);
  {
    // core holes in hcentre (ascending) order, the order of the CVS singles
    std::vector<int> sorted(core, core + ncore);
    std::sort(sorted.begin(), sorted.end());
    for (int i = 0; i < ncore; ++i) { coreorb[i] = sorted[i] - 1; corepos[sorted[i] - 1] = i; }
  }
  std::vector<int32_t> sidx(cn1);
  for (int i = 0; i < cn1; ++i) {
    const int32_t* q = kpq + 7 * (i + 1);
    sidx[i] = (q[4] - no - 1) * no + (q[2] - 1);
  }
  double *d_ca = nullptr, *d_cb = nullptr, *d_X = nullptr, *d_D1 = nullptr;
  int32_t *d_sidx = nullptr, *d_cols = nullptr;
  int *d_corepos = nullptr, *d_coreorb = nullptr;
  unsigned long long* d_kept = nullptr;
  int64_t* d_cnt = nullptr;
  void* d_tmp = nullptr;
  size_t tmp_bytes = 0;
  auto cleanup = [&]() {
    dfree(c, d_ca); dfree(c, d_cb); dfree(c, d_X); dfree(c, d_D1); dfree(c, d_sidx); dfree(c, d_cols);
    dfree(c, d_corepos); dfree(c, d_coreorb); dfree(c, d_kept); dfree(c, d_cnt); dfree(c, d_tmp);
  };
  auto run = [&]() -> int {
    ST(dmalloc(c, (void**)&d_ca, sizeof(double) * nv * nv));
    ST(dmalloc(c, (void**)&d_cb, sizeof(double) * no * no));
    ST(dmalloc(c, (void**)&d_X, sizeof(double) * n1 * n1));
    ST(dmalloc(c, (void**)&d_D1, sizeof(double) * n1 * n1));
    ST(dmalloc(c, (void**)&d_sidx, sizeof(int32_t) * cn1));
    ST(dmalloc(c, (void**)&d_cols, sizeof(int32_t) * 7 * std::max<int64_t>(n2, 1)));
    ST(dmalloc(c, (void**)&d_corepos, sizeof(int) * no));
    ST(dmalloc(c, (void**)&d_coreorb, sizeof(int) * ncore));
    ST(dmalloc(c, (void**)&d_kept, sizeof(unsigned long long)));
    ST(dmalloc(c, (void**)&d_cnt, sizeof(int64_t) * (n2 + 1)));
    ST(dmalloc(c, (void**)&c->d_diag, sizeof(double) * ndim));
    ST(dmalloc(c, (void**)&c->d_Ac, sizeof(double) * (size_t)cn1 * cn1));
    ST(dmalloc(c, (void**)&c->d_crow, sizeof(int64_t) * (n2 + 1)));
    ADC_CUDA(c, cudaMemsetAsync(d_kept, 0, sizeof(unsigned long long), s));
    ADC_CUDA(c, cudaMemsetAsync(d_cnt, 0, sizeof(int64_t) * (n2 + 1), s));
    ADC_CUDA(c, cudaMemsetAsync(c->d_Ac, 0, sizeof(double) * (size_t)cn1 * cn1, s));
    ADC_CUDA(c, cudaMemcpyAsync(d_sidx, sidx.data(), sizeof(int32_t) * cn1, cudaMemcpyHostToDevice, s));
    ADC_CUDA(c, cudaMemcpyAsync(d_corepos, corepos.data(), sizeof(int) * no, cudaMemcpyHostToDevice, s));
    ADC_CUDA(c, cudaMemcpyAsync(d_coreorb, coreorb.data(), sizeof(int) * ncore, cudaMemcpyHostToDevice, s));
    if (n2 > 0)
      ADC_CUDA(c, cudaMemcpyAsync(d_cols, kpq + 7 * (cn1 + 1), sizeof(int32_t) * 7 * n2, cudaMemcpyHostToDevice, s));
    k_ca<<<(int)((nv * (int64_t)nv + 127) / 128), 128, 0, s>>>(E, c->d_e, d_ca); ADC_COUNT_LAUNCH();
    ST(compute_cb(c, E, d_cb));
    k_cc_tables<false><<<grid_for(c, n1 * n1, 256), 256, 0, s>>>(E, c->d_e, d_X, d_D1); ADC_COUNT_LAUNCH();
    k_phph_cvs<<<grid_for(c, (int64_t)cn1 * cn1, 128), 128, 0, s>>>(E, c->d_e, d_X, d_D1, d_ca, d_cb, d_sidx, cn1,
                                                                     c->d_Ac, c->d_diag, d_kept);
    ADC_COUNT_LAUNCH();
    k_cvs_diag2<<<grid_for(c, n2, 256), 256, 0, s>>>(d_cols, n2, no, c->d_e, c->d_diag + cn1); ADC_COUNT_LAUNCH();
    k_cvs_coupling<false><<<c->nsm * 8, 256, 0, s>>>(E, d_cols, n2, ncore, d_corepos, d_coreorb, d_cnt, nullptr,
                                                      nullptr, nullptr);
    ADC_COUNT_LAUNCH();
    ADC_CUDA(c, cudaGetLastError());
    cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, d_cnt, c->d_crow, n2 + 1, s);
    ST(dmalloc(c, &d_tmp, tmp_bytes));
    cub::DeviceScan::ExclusiveSum(d_tmp, tmp_bytes, d_cnt, c->d_crow, n2 + 1, s);
    int64_t nnz = 0;
    unsigned long long kept_ph = 0;
    ADC_CUDA(c, cudaMemcpyAsync(&nnz, c->d_crow + n2, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    ADC_CUDA(c, cudaMemcpyAsync(&kept_ph, d_kept, sizeof(kept_ph), cudaMemcpyDeviceToHost, s));
    ADC_CUDA(c, cudaStreamSynchronize(s));
    ST(dmalloc(c, (void**)&c->d_ccol, sizeof(int32_t) * std::max<int64_t>(nnz, 1)));
    ST(dmalloc(c, (void**)&c->d_cval, sizeof(double) * std::max<int64_t>(nnz, 1)));
    k_cvs_coupling<true><<<c->nsm * 8, 256, 0, s>>>(E, d_cols, n2, ncore, d_corepos, d_coreorb, nullptr, c->d_crow,
                                                     c->d_ccol, c->d_cval);
    ADC_COUNT_LAUNCH();
    ADC_CUDA(c, cudaGetLastError());
    ADC_CUDA(c, cudaStreamSynchronize(s));
    c->cvs_n1 = cn1;
    c->cvs_N = ndim;
    c->cvs_nnz = nnz;
    c->nnz_ph = (int64_t)kept_ph;
    c->nnz_kept = (int64_t)kept_ph + nnz;
    return ADCGPU_OK;
  };
  int st = run();
  cleanup();
  return st;
}

}  // namespace adcgpu
