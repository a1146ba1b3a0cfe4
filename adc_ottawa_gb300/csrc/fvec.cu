// The ADC(2) f-vector F_J = <Psi_J|D|Psi_0> of one dipole component
// (get_modifiedtm_adc2, source/adclib/get_moment.f90:153-442, with the terms
// of source/adclib/dipole_ph.f90), computed on the device in FP64.
//
// 2h2p block: one thread per configuration evaluates FI/FII/FIII/FIV1/FIV2
// (dipole_ph.f90:662-846) in the reference's loop and expression order.  The
// file is compiled with --fmad=false, so these entries equal the reference's
// IEEE FP64 values bit for bit.
//
// 1h1p block: the reference evaluates each of F25_ph..F210_ph as a 4- or
// 5-fold loop per single (O(n1^3) and O(n1 no nv^2) terms with 4-8 ERI
// gathers each).  Here the same sums are regrouped into dense contractions
// over pair matrices indexed by singles s = (a,k), t = (b,l) (0-based
// virtual a, occupied k; s = a*no + k, the select_atom_is order):
//
//   D(ak,bl)  = e_k + e_l - e_a - e_b
//   T(ak,bl)  = (2(ak|bl) - (al|bk)) / D        (first-order amplitudes)
//   K(ak,bl)  = 2(ak|bl) - (ab|kl)
//   A1(ak,bl) = (ak|bl) / D,  L2(ak,bl) = (al|bk) / D
//   X2(ak,bl) = (ab|kl),  Tsw(ak,bl) = T(al,bk),  J(ak,bl) = 2(ba|kl) - (ak|bl)
//
//   F25 + F26 (:390-469) = sum_cm [K T + T K](ak,cm) d(c,m) / D(ak,cm)
//   F27 + F28 (:473-557) = -sum_lb [E T + X2 Tsw + A1 K + L2 J](al,bk) d(b,l) / D(ak,bl)
//   F29 + F210 (:561-656) = sum_lb W(ab,kl) d(b,l) / D(ak,bl),
//       W(ab,kl) = sum_cd (ac|bd) T(ck,dl) + sum_mn (am|bn)/(e_m+e_n-e_a-e_b) (2(mk|nl) - (ml|nk))
//   F0 (:24-46) = (T d)(ak);  tauC (:1181-1209) = 0.5 T d;  FC_ph_new (:1213-1242) = T tauC
//   tauA (:896-935)  = -0.5 sum_{l,bm} T(cl,bm) A1(al,bm)
//   tauB (:939-981)  = -0.5 sum_{b,cl} T(bm,cl) A1(bk,cl)
//   tau21..tau24 (:985-1177): contractions of A1, T with (vv|ov) and (oo|ov)
//
// where E = (ak|bl) itself.  The reference's restricted sums (m > l, c > b,
// d > c plus the diagonal term) are the halves of symmetric full sums, which
// the matrices above run over.  The dense products are FP64 GEMMs on the
// CUDA cores (GB300 has no fast FP64 tensor path); the result differs from
// the reference's loop order only by FP64 rounding (about 1e-15 relative).
#include <algorithm>
#include <cmath>
#include <vector>

#include "internal.h"

namespace adcgpu {
namespace {

constexpr int FV_MAXNO = 32;   // adcgpu_set_orbitals caps nocc at 32

inline int fv_grid(const Ctx* c, int64_t n, int block) {
  int64_t g = (n + block - 1) / block;
  int64_t cap = (int64_t)c->nsm * 16;
  return (int)std::max<int64_t>(1, std::min<int64_t>(g, cap));
}

// ---------------------------------------------------------------------------
// FP64 GEMM, row-major: C[z] = alpha * A * op(B) + beta * C[z], where
// op(B) = B (K x N, ldb) or, with BT, B^T for B given as N x K (ldb).
// Split K: blockIdx.z covers [z*kchunk, min(K, (z+1)*kchunk)) and writes the
// slice C + z*cstride.  64 x 64 tiles, K steps of 16, 256 threads with a 4x4
// register tile each; explicit __fma_rn (the file is built with --fmad=false).
// ---------------------------------------------------------------------------
template <bool BT>
__global__ void __launch_bounds__(256) k_dgemm(int M, int N, int K, double alpha, const double* __restrict__ A,
                                               int64_t lda, const double* __restrict__ B, int64_t ldb, double beta,
                                               double* __restrict__ C, int64_t ldc, int kchunk, int64_t cstride) {
  __shared__ double As[16][65];
  __shared__ double Bs[16][65];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
  const int kbeg = blockIdx.z * kchunk;
  const int kend = min(K, kbeg + kchunk);
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
  for (int k0 = kbeg; k0 < kend; k0 += 16) {
    for (int i = tid; i < 1024; i += 256) {
      const int r = i >> 4, kk = i & 15;
      const int gm = m0 + r, gk = k0 + kk;
      As[kk][r] = (gm < M && gk < kend) ? A[(int64_t)gm * lda + gk] : 0.0;
    }
    for (int i = tid; i < 1024; i += 256) {
      if (!BT) {
        const int kk = i >> 6, cc = i & 63;
        const int gk = k0 + kk, gn = n0 + cc;
        Bs[kk][cc] = (gk < kend && gn < N) ? B[(int64_t)gk * ldb + gn] : 0.0;
      } else {
        const int cc = i >> 4, kk = i & 15;
        const int gk = k0 + kk, gn = n0 + cc;
        Bs[kk][cc] = (gk < kend && gn < N) ? B[(int64_t)gn * ldb + gk] : 0.0;
      }
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = __fma_rn(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  double* Cz = C + (int64_t)blockIdx.z * cstride;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gm = m0 + ty + 16 * i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gn = n0 + tx + 16 * j;
      if (gn >= N) continue;
      double* cp = Cz + (int64_t)gm * ldc + gn;
      double v = alpha * acc[i][j];
      if (beta != 0.0) v = __fma_rn(beta, *cp, v);
      *cp = v;
    }
  }
}

// sum of nsplit slices of length n into out (out may be slice 0)
__global__ void k_sum_slices(const double* __restrict__ part, int nsplit, int64_t stride, int64_t n,
                             double* __restrict__ out) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int z = 0; z < nsplit; ++z) s += part[(int64_t)z * stride + t];
    out[t] = s;
  }
}

// ---------------------------------------------------------------------------
// Pair matrices over (ak, bl), n1 x n1 row-major; vovo is (ak|bl) in the same
// layout, vvoo is (ab|kl) as [a][b][k][l].
// ---------------------------------------------------------------------------
__global__ void k_fv_pairs(int no, int nv, const double* __restrict__ e, const double* __restrict__ vovo,
                           const double* __restrict__ vvoo, double* __restrict__ T, double* __restrict__ Km,
                           double* __restrict__ X2, double* __restrict__ Tsw, double* __restrict__ A1,
                           double* __restrict__ L2, double* __restrict__ J) {
  const int64_t n1 = (int64_t)no * nv, total = n1 * n1;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < total;
       x += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = x / n1, t = x % n1;
    const int a = (int)(s / no), k = (int)(s % no), b = (int)(t / no), l = (int)(t % no);
    const double D = e[k] + e[l] - e[no + a] - e[no + b];
    const double akbl = vovo[x];
    const double albk = vovo[((int64_t)a * no + l) * n1 + (int64_t)b * no + k];
    const double abkl = vvoo[(((int64_t)a * nv + b) * no + k) * no + l];
    const double bakl = vvoo[(((int64_t)b * nv + a) * no + k) * no + l];
    T[x] = (2.0 * akbl - albk) / D;
    Tsw[x] = (2.0 * albk - akbl) / D;
    Km[x] = 2.0 * akbl - abkl;
    X2[x] = abkl;
    A1[x] = akbl / D;
    L2[x] = albk / D;
    J[x] = 2.0 * bakl - akbl;
  }
}

// Tcd[(c,d),(k,l)] = T[(c,k),(d,l)]
__global__ void k_fv_tcd(int no, int nv, const double* __restrict__ T, double* __restrict__ Tcd) {
  const int64_t n1 = (int64_t)no * nv, total = n1 * n1;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < total;
       x += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = x;
    const int l = (int)(r % no); r /= no;
    const int k = (int)(r % no); r /= no;
    const int d = (int)(r % nv);
    const int c = (int)(r / nv);
    Tcd[x] = T[((int64_t)c * no + k) * n1 + (int64_t)d * no + l];
  }
}

__device__ __forceinline__ int64_t tri_idx(int64_t p, int64_t q) {
  return p >= q ? p * (p + 1) / 2 + q : q * (q + 1) / 2 + p;
}

// Ablk[(a - a0, b), (c, d)] = (ac|bd) for a in [a0, a0 + na), from the
// virtual-pair packed (vv|vv) block
__global__ void k_fv_vvvv_rows(int nv, int a0, int na, const double* __restrict__ vvvv, double* __restrict__ Ablk) {
  const int64_t nv2 = (int64_t)nv * nv, total = (int64_t)na * nv * nv2;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < total;
       x += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = x / nv2, col = x % nv2;
    const int a = a0 + (int)(row / nv), b = (int)(row % nv);
    const int c = (int)(col / nv), d = (int)(col % nv);
    Ablk[x] = vvvv[tri_idx(tri_idx(a, c), tri_idx(b, d))];
  }
}

// A'[(a,b),(m,n)] = (am|bn)/(e_m+e_n-e_a-e_b);  B'[(m,n),(k,l)] = 2(mk|nl) - (ml|nk)
__global__ void k_fv_hole_ladder(int no, int nv, const double* __restrict__ e, const double* __restrict__ vovo,
                                 const double* __restrict__ oooo, double* __restrict__ Ap, double* __restrict__ Bp) {
  const int64_t no2 = (int64_t)no * no, n1 = (int64_t)no * nv;
  const int64_t na = (int64_t)nv * nv * no2, nb = no2 * no2;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < na + nb;
       x += (int64_t)gridDim.x * blockDim.x) {
    if (x < na) {
      int64_t r = x;
      const int n = (int)(r % no); r /= no;
      const int m = (int)(r % no); r /= no;
      const int b = (int)(r % nv);
      const int a = (int)(r / nv);
      Ap[x] = vovo[((int64_t)a * no + m) * n1 + (int64_t)b * no + n] / (e[m] + e[n] - e[no + a] - e[no + b]);
    } else {
      int64_t r = x - na;
      const int l = (int)(r % no); r /= no;
      const int k = (int)(r % no); r /= no;
      const int n = (int)(r % no);
      const int m = (int)(r / no);
      const double mknl = oooo[(((int64_t)m * no + k) * no + n) * no + l];
      const double mlnk = oooo[(((int64_t)m * no + l) * no + n) * no + k];
      Bp[x - na] = 2.0 * mknl - mlnk;
    }
  }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// y(s) = alpha * sum_t M(s,t) x(t), one warp per row (M n1 x n1)
__global__ void k_fv_matvec(int64_t n1, double alpha, const double* __restrict__ M, const double* __restrict__ x,
                            double* __restrict__ y) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t s = w0; s < n1; s += nw) {
    double acc = 0.0;
    for (int64_t t = lane; t < n1; t += 32) acc = __fma_rn(M[s * n1 + t], x[t], acc);
    acc = warp_sum(acc);
    if (lane == 0) y[s] = alpha * acc;
  }
}

// dvo(a,k) = dpl(no+a, k)  [nv][no];  dpl is column-major: dpl(p,q) = dpl[q*nb + p]
__device__ __forceinline__ double dp(const double* dpl, int nb, int p, int q) { return dpl[(int64_t)q * nb + p]; }

// x(b,l) = dpl(b,l) over the singles
__global__ void k_fv_dvo(int no, int nv, const double* __restrict__ dpl, double* __restrict__ x) {
  const int64_t n1 = (int64_t)no * nv;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n1; t += (int64_t)gridDim.x * blockDim.x)
    x[t] = dp(dpl, no + nv, no + (int)(t / no), (int)(t % no));
}

// Per single (a,k), one warp:
//   f2526 = sum_cm Z(ak,cm) d(c,m) / D(ak,cm)
//   f2728 = -sum_lb Y(al,bk) d(b,l) / D(ak,bl)
//   f29   = sum_lb W(ab,kl) d(b,l) / D(ak,bl)
__global__ void k_fv_contract(int no, int nv, const double* __restrict__ e, const double* __restrict__ dpl,
                              const double* __restrict__ Z, const double* __restrict__ Y,
                              const double* __restrict__ W, double* __restrict__ f2526, double* __restrict__ f2728,
                              double* __restrict__ f29) {
  const int lane = threadIdx.x & 31;
  const int64_t n1 = (int64_t)no * nv;
  const int nb = no + nv;
  const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t s = w0; s < n1; s += nw) {
    const int a = (int)(s / no), k = (int)(s % no);
    const double ek_a = e[k] - e[no + a];
    double z = 0.0, y = 0.0, w = 0.0;
    for (int64_t t = lane; t < n1; t += 32) {
      const int b = (int)(t / no), l = (int)(t % no);
      const double D = ek_a + e[l] - e[no + b];
      const double r = dp(dpl, nb, l, no + b) / D;   // d(m,c), d(l,b), d(m,b) of F25..F210
      z = __fma_rn(Z[s * n1 + t], r, z);
      y = __fma_rn(Y[((int64_t)a * no + l) * n1 + (int64_t)b * no + k], r, y);
      w = __fma_rn(W[((int64_t)a * nv + b) * no * no + (int64_t)k * no + l], r, w);
    }
    z = warp_sum(z); y = warp_sum(y); w = warp_sum(w);
    if (lane == 0) { f2526[s] = z; f2728[s] = -y; f29[s] = w; }
  }
}

// tauB(m,k) = -0.5 sum_b sum_cl T[(b,m),(cl)] A1[(b,k),(cl)], one block per (m,k)
__global__ void k_fv_taub(int no, int nv, const double* __restrict__ T, const double* __restrict__ A1,
                          double* __restrict__ tauB) {
  __shared__ double red[32];
  const int64_t n1 = (int64_t)no * nv;
  const int m = blockIdx.x / no, k = blockIdx.x % no;
  double acc = 0.0;
  for (int64_t x = threadIdx.x; x < (int64_t)nv * n1; x += blockDim.x) {
    const int b = (int)(x / n1);
    const int64_t cl = x % n1;
    acc = __fma_rn(T[((int64_t)b * no + m) * n1 + cl], A1[((int64_t)b * no + k) * n1 + cl], acc);
  }
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    v = warp_sum(v);
    if (threadIdx.x == 0) tauB[blockIdx.x] = -0.5 * v;
  }
}

// One block per virtual v, accumulating over items (l,b,c) for all holes:
//   mode 0 (tau21): out(v,m) = -1/(e_m - e_v) sum_{lbc} A1[(b,l),(c,m)] (2(vc|lb) - (vb|lc))
//   mode 1 (tau24): out(v,k) =  1/(e_k - e_v) sum_{lbc} A1[(c,l),(b,k)] (2(vb|lc) - (vc|lb))
// (A1 is symmetric, so A1[(c,l),(b,k)] = A1[(b,k),(c,l)]); vvov = (ab|ic) [a][b][i][c].
__global__ void __launch_bounds__(256) k_fv_tau_vo(int mode, int no, int nv, const double* __restrict__ e,
                                                   const double* __restrict__ A1, const double* __restrict__ vvov,
                                                   double* __restrict__ out) {
  __shared__ double red[FV_MAXNO][8];
  const int64_t n1 = (int64_t)no * nv;
  const int v = blockIdx.x;
  double acc[FV_MAXNO];
#pragma unroll
  for (int m = 0; m < FV_MAXNO; ++m) acc[m] = 0.0;
  const int64_t items = (int64_t)no * nv * nv;
  for (int64_t x = threadIdx.x; x < items; x += blockDim.x) {
    const int c = (int)(x % nv);
    const int b = (int)((x / nv) % nv);
    const int l = (int)(x / ((int64_t)nv * nv));
    double g;
    const double* arow;
    if (mode == 0) {
      g = 2.0 * vvov[(((int64_t)v * nv + c) * no + l) * nv + b] - vvov[(((int64_t)v * nv + b) * no + l) * nv + c];
      arow = A1 + ((int64_t)b * no + l) * n1 + (int64_t)c * no;
    } else {
      g = 2.0 * vvov[(((int64_t)v * nv + b) * no + l) * nv + c] - vvov[(((int64_t)v * nv + c) * no + l) * nv + b];
      arow = A1 + ((int64_t)c * no + l) * n1 + (int64_t)b * no;
    }
#pragma unroll
    for (int m = 0; m < FV_MAXNO; ++m)
      if (m < no) acc[m] = __fma_rn(arow[m], g, acc[m]);
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int m = 0; m < FV_MAXNO; ++m) {
    if (m >= no) break;
    double s = warp_sum(acc[m]);
    if (lane == 0) red[m][warp] = s;
  }
  __syncthreads();
  if (threadIdx.x < no) {
    const int m = threadIdx.x;
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[m][w];
    const double den = e[m] - e[no + v];
    out[(int64_t)v * no + m] = mode == 0 ? -s / den : s / den;
  }
}

// One warp per (v,o):
//   mode 0 (tau22): out(a,n) =  1/(e_n - e_a) sum_{l,m,b} (mn|lb) T[(b,l),(a,m)]
//   mode 1 (tau23): out(b,k) = -1/(e_k - e_b) sum_{c,l,m} A1[(b,l),(c,m)] (2(lk|mc) - (mk|lc))
// ooov = (ij|ka) [i][j][k][a].
__global__ void k_fv_tau_oo(int mode, int no, int nv, const double* __restrict__ e, const double* __restrict__ T,
                            const double* __restrict__ A1, const double* __restrict__ ooov, double* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t n1 = (int64_t)no * nv;
  const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t items = (int64_t)no * no * nv;
  for (int64_t s = w0; s < n1; s += nw) {
    const int v = (int)(s / no), o = (int)(s % no);
    double acc = 0.0;
    for (int64_t x = lane; x < items; x += 32) {
      if (mode == 0) {
        const int b = (int)(x % nv);
        const int m = (int)((x / nv) % no);
        const int l = (int)(x / ((int64_t)nv * no));
        acc = __fma_rn(ooov[(((int64_t)m * no + o) * no + l) * nv + b], T[((int64_t)b * no + l) * n1 + (int64_t)v * no + m],
                       acc);
      } else {
        const int c = (int)(x % nv);
        const int m = (int)((x / nv) % no);
        const int l = (int)(x / ((int64_t)nv * no));
        const double g = 2.0 * ooov[(((int64_t)l * no + o) * no + m) * nv + c] - ooov[(((int64_t)m * no + o) * no + l) * nv + c];
        acc = __fma_rn(A1[((int64_t)v * no + l) * n1 + (int64_t)c * no + m], g, acc);
      }
    }
    acc = warp_sum(acc);
    if (lane == 0) {
      const double den = e[o] - e[no + v];
      out[s] = mode == 0 ? acc / den : -acc / den;
    }
  }
}

// The 1h1p entries, in the reference's order of terms:
//   mtm = -sqrt(2) (d(a,k) + F0 + F25..F210 + FA + FB + FC + F21 + F22 + F23 + F24)
// written to the kpq positions of the singles (s = a*no + k is kpq column s+1).
__global__ void k_fv_singles(int no, int nv, const double* __restrict__ dpl, const double* __restrict__ f0,
                             const double* __restrict__ f2526, const double* __restrict__ f2728,
                             const double* __restrict__ f29, const double* __restrict__ fc,
                             const double* __restrict__ tauA, const double* __restrict__ tauB,
                             const double* __restrict__ tau21, const double* __restrict__ tau22,
                             const double* __restrict__ tau23, const double* __restrict__ tau24,
                             double* __restrict__ mtm) {
  const int64_t n1 = (int64_t)no * nv;
  const int nb = no + nv;
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n1; s += (int64_t)gridDim.x * blockDim.x) {
    const int a = (int)(s / no), k = (int)(s % no);
    double fa = 0.0, fb = 0.0, f21 = 0.0, f22 = 0.0, f23 = 0.0, f24 = 0.0;
    for (int c = 0; c < nv; ++c) {
      fa = __fma_rn(tauA[(int64_t)c * nv + a], dp(dpl, nb, no + c, k), fa);
      const double dac = dp(dpl, nb, no + a, no + c);
      f23 = __fma_rn(dac, tau23[(int64_t)c * no + k], f23);
      f24 = __fma_rn(dac, tau24[(int64_t)c * no + k], f24);
    }
    for (int l = 0; l < no; ++l) {
      fb = __fma_rn(dp(dpl, nb, no + a, l), tauB[l * no + k], fb);
      const double dlk = dp(dpl, nb, l, k);
      f21 = __fma_rn(tau21[(int64_t)a * no + l], dlk, f21);
      f22 = __fma_rn(tau22[(int64_t)a * no + l], dlk, f22);
    }
    double x = dp(dpl, nb, no + a, k);
    x = x + f0[s];
    x = x + f2526[s];
    x = x + f2728[s];
    x = x + f29[s];
    x = x + fa;
    x = x + fb;
    x = x + fc[s];
    x = x + f21;
    x = x + f22;
    x = x + f23;
    x = x + f24;
    mtm[s] = -sqrt(2.0) * x;
  }
}

// ---------------------------------------------------------------------------
// 2h2p block: FI_2p2h .. FIV1_2p2h (dipole_ph.f90:662-846), one thread per
// kpq column, in the reference's order.  (pq|rs) of the classes (vo|vo) only.
// ---------------------------------------------------------------------------
struct FvEri {
  const double* vovo;
  int no, nv;
  // (p q|r s) for p, r virtual and q, s occupied (0-based orbitals)
  __device__ double vo(int p, int q, int r, int s) const {
    return vovo[(((int64_t)(p - no) * no + q) * nv + (r - no)) * no + s];
  }
};

__global__ void k_fv_doubles(FvEri V, const double* __restrict__ e, const double* __restrict__ dpl,
                             const int32_t* __restrict__ cols, int64_t n2, double* __restrict__ mtm) {
  const int no = V.no, nb = V.no + V.nv;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n2; t += (int64_t)gridDim.x * blockDim.x) {
    const int32_t* q = cols + 7 * t;
    // kpq(3) = k, kpq(4) = j, kpq(5) = a, kpq(6) = b, kpq(7) = type; 1-based
    const int k = q[2] - 1, j = q[3] - 1, a = q[4] - 1, b = q[5] - 1, type = q[6];
    double f = 0.0;
    if (type == 1) {                    // FI_2p2h(a,k) :662-690
      for (int m = 0; m < no; ++m) {
        double e_mkaa = e[m] + e[k] - e[a] - e[a];
        f = f - dp(dpl, nb, m, k) / e_mkaa * V.vo(a, k, a, m);
      }
      for (int c = no; c < nb; ++c) {
        double e_kkac = e[k] + e[k] - e[a] - e[c];
        f = f + dp(dpl, nb, a, c) / e_kkac * V.vo(c, k, a, k);
      }
      f = 2.0 * f;
    } else if (type == 2) {             // FII_2p2h(a,b,k) :694-727
      for (int m = 0; m < no; ++m) {
        double e_mkab = e[m] + e[k] - e[a] - e[b];
        f = f - dp(dpl, nb, m, k) / e_mkab * (V.vo(a, m, b, k) + V.vo(a, k, b, m));
      }
      for (int c = no; c < nb; ++c) {
        double e_kkbc = e[k] + e[k] - e[b] - e[c];
        f = f + dp(dpl, nb, a, c) / e_kkbc * V.vo(c, k, b, k);
        double e_kkac = e[k] + e[k] - e[a] - e[c];
        f = f + dp(dpl, nb, b, c) / e_kkac * V.vo(c, k, a, k);
      }
      f = sqrt(2.0) * f;
    } else if (type == 3) {             // FIII_2p2h(a,k,l), l = kpq(4) :731-764
      const int l = j;
      for (int m = 0; m < no; ++m) {
        double e_mlaa = e[m] + e[l] - e[a] - e[a];
        f = f + dp(dpl, nb, m, k) / e_mlaa * V.vo(a, m, a, l);
        double e_kmaa = e[k] + e[m] - e[a] - e[a];
        f = f + dp(dpl, nb, m, l) / e_kmaa * V.vo(a, k, a, m);
      }
      for (int c = no; c < nb; ++c) {
        double e_klac = e[k] + e[l] - e[a] - e[c];
        f = f - dp(dpl, nb, a, c) / e_klac * (V.vo(c, k, a, l) + V.vo(c, l, a, k));
      }
      f = sqrt(2.0) * f;
    } else {                            // FIV1 (type 4) / FIV2 (type 5), l = kpq(4) :768-846
      const int l = j;
      for (int m = 0; m < no; ++m) {
        // (a l|m b) = (a l|b m), (a m|b k), (a k|m b) = (a k|b m)
        double e_mlab = e[m] + e[l] - e[a] - e[b];
        double x1 = type == 4 ? V.vo(a, m, b, l) + V.vo(a, l, b, m) : V.vo(a, m, b, l) - V.vo(a, l, b, m);
        f = f + dp(dpl, nb, m, k) / e_mlab * x1;
        double e_kmab = e[k] + e[m] - e[a] - e[b];
        double x2 = type == 4 ? V.vo(a, k, b, m) + V.vo(a, m, b, k) : V.vo(a, k, b, m) - V.vo(a, m, b, k);
        f = f + dp(dpl, nb, m, l) / e_kmab * x2;
      }
      for (int c = no; c < nb; ++c) {
        double e_klbc = e[k] + e[l] - e[b] - e[c];
        double x3 = type == 4 ? V.vo(c, k, b, l) + V.vo(c, l, b, k) : V.vo(c, k, b, l) - V.vo(c, l, b, k);
        f = f - dp(dpl, nb, a, c) / e_klbc * x3;
        double e_klac = e[k] + e[l] - e[a] - e[c];
        double x4 = type == 4 ? V.vo(c, l, a, k) + V.vo(c, k, a, l) : V.vo(c, l, a, k) - V.vo(c, k, a, l);
        f = f - dp(dpl, nb, b, c) / e_klac * x4;
      }
      if (type == 5) f = sqrt(3.0) * f;
    }
    mtm[t] = f;
  }
}

}  // namespace

// Launch helper: C = alpha A op(B) + beta C with optional split-K into scratch.
static int dgemm(Ctx* c, bool bt, int M, int N, int K, double alpha, const double* A, int64_t lda, const double* B,
                 int64_t ldb, double beta, double* C, int64_t ldc, double* split_ws = nullptr, int nsplit = 1) {
  dim3 grid((N + 63) / 64, (M + 63) / 64, 1);
  if (nsplit > 1 && split_ws && beta == 0.0 && ldc == N) {
    const int kchunk = ((K + nsplit - 1) / nsplit + 15) / 16 * 16;
    const int nz = (K + kchunk - 1) / kchunk;
    grid.z = nz;
    const int64_t stride = (int64_t)M * N;
    if (bt) k_dgemm<true><<<grid, 256, 0, c->stream>>>(M, N, K, alpha, A, lda, B, ldb, 0.0, split_ws, ldc, kchunk, stride);
    else k_dgemm<false><<<grid, 256, 0, c->stream>>>(M, N, K, alpha, A, lda, B, ldb, 0.0, split_ws, ldc, kchunk, stride);
    ADC_COUNT_LAUNCH();
    k_sum_slices<<<fv_grid(c, stride, 256), 256, 0, c->stream>>>(split_ws, nz, stride, stride, C);
    ADC_COUNT_LAUNCH();
  } else {
    if (bt) k_dgemm<true><<<grid, 256, 0, c->stream>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, K, 0);
    else k_dgemm<false><<<grid, 256, 0, c->stream>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, K, 0);
    ADC_COUNT_LAUNCH();
  }
  ADC_CUDA(c, cudaGetLastError());
  return ADCGPU_OK;
}

int modified_tm_adc2(Ctx* c, int64_t ndim, const int32_t* kpq, double* mtm) {
  const int no = c->geom.no, nv = c->geom.nv;
  if (no > FV_MAXNO) return set_err(c, ADCGPU_UNSUPPORTED, "f-vector: nocc above 32");
  if (!c->d_oooo || !c->d_vvvv) return set_err(c, ADCGPU_BAD_INPUT, "f-vector: (oo|oo) and (vv|vv) blocks missing");
  // kpq: the ADC(2)-s list or a CVS list (singles on core holes, no i=j
  // doubles); the 1h1p block is evaluated for all singles and gathered
  const int64_t n1 = c->geom.n1, nn = n1 * n1, ns = kpq[0], n2 = ndim - ns;
  const int64_t nv2 = (int64_t)nv * nv, no2 = (int64_t)no * no;
  cudaStream_t s = c->stream;
  // a-batch of the (vv|vv) rows: at most ~1 GiB of rows
  const int64_t row_bytes = nv * nv2 * (int64_t)sizeof(double);
  const int na = (int)std::max<int64_t>(1, std::min<int64_t>(nv, ((int64_t)1 << 30) / row_bytes));
  const int nsplit_a = std::max(1, std::min<int>(c->nsm, (int)((int64_t)no * n1 / 2048)));
  // device scratch: 7 pair matrices, Z, Y, W (= n1 x n1 as (ab) x (kl)), Tcd,
  // the (vv|vv) row batch, the hole-ladder operands and small vectors
  struct Buf { double** p; int64_t n; };
  double *T, *Km, *X2, *Tsw, *A1, *L2, *J, *Z, *Y, *W, *Tcd, *Ab, *Ap, *Bp, *vec, *ws, *dout;
  int32_t* dcols = nullptr;
  const int64_t nvec = 6 * n1 + nv2 + no2 + 4 * n1;
  const int64_t nws = std::max<int64_t>((int64_t)nsplit_a * nv2, 1);
  Buf bufs[] = {{&T, nn}, {&Km, nn}, {&X2, nn}, {&Tsw, nn}, {&A1, nn}, {&L2, nn}, {&J, nn}, {&Z, nn}, {&Y, nn},
                {&W, nn}, {&Tcd, nn}, {&Ab, (int64_t)na * nv * nv2}, {&Ap, nv2 * no2}, {&Bp, no2 * no2},
                {&vec, nvec}, {&ws, nws}, {&dout, n1 + n2}};
  const int nbuf = (int)(sizeof(bufs) / sizeof(bufs[0]));
  for (Buf& b : bufs) *b.p = nullptr;
  int st = ADCGPU_OK;
  for (Buf& b : bufs)
    if (!st) st = dmalloc(c, (void**)b.p, sizeof(double) * (size_t)b.n);
  if (!st) st = dmalloc(c, (void**)&dcols, sizeof(int32_t) * 7 * (size_t)std::max<int64_t>(n2, 1));
  auto cleanup = [&]() {
    for (int i = 0; i < nbuf; ++i) dfree(c, *bufs[i].p);
    dfree(c, dcols);
  };
  if (st) { cleanup(); return st; }
  double* f0 = vec;
  double* fc = vec + n1;
  double* f2526 = vec + 2 * n1;
  double* f2728 = vec + 3 * n1;
  double* f29 = vec + 4 * n1;
  double* tauA = vec + 6 * n1;
  double* tauB = tauA + nv2;
  double* tau21 = tauB + no2;
  double* tau22 = tau21 + n1;
  double* tau23 = tau22 + n1;
  double* tau24 = tau23 + n1;
  const double* e = c->d_e;
  const double* dpl = c->d_dpl;
  auto run = [&]() -> int {
    k_fv_pairs<<<fv_grid(c, nn, 256), 256, 0, s>>>(no, nv, e, c->d_vovo, c->d_vvoo, T, Km, X2, Tsw, A1, L2, J);
    ADC_COUNT_LAUNCH();
    ADC_CUDA(c, cudaGetLastError());
    const int N1 = (int)n1;
    // Z = K T + T K ;  Y = E T + X2 Tsw + A1 K + L2 J
    ST(dgemm(c, false, N1, N1, N1, 1.0, Km, n1, T, n1, 0.0, Z, n1));
    ST(dgemm(c, false, N1, N1, N1, 1.0, T, n1, Km, n1, 1.0, Z, n1));
    ST(dgemm(c, false, N1, N1, N1, 1.0, c->d_vovo, n1, T, n1, 0.0, Y, n1));
    ST(dgemm(c, false, N1, N1, N1, 1.0, X2, n1, Tsw, n1, 1.0, Y, n1));
    ST(dgemm(c, false, N1, N1, N1, 1.0, A1, n1, Km, n1, 1.0, Y, n1));
    ST(dgemm(c, false, N1, N1, N1, 1.0, L2, n1, J, n1, 1.0, Y, n1));
    // W(ab,kl) = sum_cd (ac|bd) T(ck,dl) + hole ladder
    k_fv_tcd<<<fv_grid(c, nn, 256), 256, 0, s>>>(no, nv, T, Tcd);
    ADC_COUNT_LAUNCH();
    for (int a0 = 0; a0 < nv; a0 += na) {
      const int nb = std::min(na, nv - a0);
      k_fv_vvvv_rows<<<fv_grid(c, (int64_t)nb * nv * nv2, 256), 256, 0, s>>>(nv, a0, nb, c->d_vvvv, Ab);
      ADC_COUNT_LAUNCH();
      ST(dgemm(c, false, nb * nv, (int)no2, (int)nv2, 1.0, Ab, nv2, Tcd, no2, 0.0, W + (int64_t)a0 * nv * no2, no2));
    }
    k_fv_hole_ladder<<<fv_grid(c, nv2 * no2 + no2 * no2, 256), 256, 0, s>>>(no, nv, e, c->d_vovo, c->d_oooo, Ap, Bp);
    ADC_COUNT_LAUNCH();
    ST(dgemm(c, false, (int)nv2, (int)no2, (int)no2, 1.0, Ap, no2, Bp, no2, 1.0, W, no2));
    k_fv_contract<<<fv_grid(c, n1 * 32, 256), 256, 0, s>>>(no, nv, e, dpl, Z, Y, W, f2526, f2728, f29);
    ADC_COUNT_LAUNCH();
    // u = T d  (F0 = u, tauC = u/2),  FC = T tauC
    k_fv_dvo<<<fv_grid(c, n1, 256), 256, 0, s>>>(no, nv, dpl, fc);   // fc holds d(b,l) until overwritten
    ADC_COUNT_LAUNCH();
    k_fv_matvec<<<fv_grid(c, n1 * 32, 256), 256, 0, s>>>(n1, 1.0, T, fc, f0);
    ADC_COUNT_LAUNCH();
    k_fv_matvec<<<fv_grid(c, n1 * 32, 256), 256, 0, s>>>(n1, 0.5, T, f0, fc);
    ADC_COUNT_LAUNCH();
    // tauA(c,a) = -0.5 T_m A1_m^T over K = (l, bm): split-K into ws
    ST(dgemm(c, true, nv, nv, (int)(no * n1), -0.5, T, (int64_t)no * n1, A1, (int64_t)no * n1, 0.0, tauA, nv, ws,
             nsplit_a));
    k_fv_taub<<<(int)no2, 256, 0, s>>>(no, nv, T, A1, tauB);
    ADC_COUNT_LAUNCH();
    k_fv_tau_vo<<<nv, 256, 0, s>>>(0, no, nv, e, A1, c->d_vvov, tau21);
    ADC_COUNT_LAUNCH();
    k_fv_tau_vo<<<nv, 256, 0, s>>>(1, no, nv, e, A1, c->d_vvov, tau24);
    ADC_COUNT_LAUNCH();
    k_fv_tau_oo<<<fv_grid(c, n1 * 32, 256), 256, 0, s>>>(0, no, nv, e, T, A1, c->d_ooov, tau22);
    ADC_COUNT_LAUNCH();
    k_fv_tau_oo<<<fv_grid(c, n1 * 32, 256), 256, 0, s>>>(1, no, nv, e, T, A1, c->d_ooov, tau23);
    ADC_COUNT_LAUNCH();
    k_fv_singles<<<fv_grid(c, n1, 128), 128, 0, s>>>(no, nv, dpl, f0, f2526, f2728, f29, fc, tauA, tauB, tau21, tau22,
                                                     tau23, tau24, dout);
    ADC_COUNT_LAUNCH();
    // 2h2p block over kpq columns n1+1 .. ndim
    if (n2 > 0) {
      ADC_CUDA(c, h2d(c, dcols, kpq + 7 * (ns + 1), sizeof(int32_t) * 7 * (size_t)n2));
      FvEri V{c->d_vovo, no, nv};
      k_fv_doubles<<<fv_grid(c, n2, 128), 128, 0, s>>>(V, e, dpl, dcols, n2, dout + n1);
      ADC_COUNT_LAUNCH();
    }
    ADC_CUDA(c, cudaGetLastError());
    if (ns == n1) {
      ADC_CUDA(c, d2h(c, mtm, dout, sizeof(double) * (size_t)ndim));
    } else {
      std::vector<double> full((size_t)(n1 + n2));
      ADC_CUDA(c, d2h(c, full.data(), dout, sizeof(double) * full.size()));
      for (int64_t i = 0; i < ns; ++i) {
        const int32_t* q = kpq + 7 * (i + 1);
        mtm[i] = full[(size_t)(q[4] - no - 1) * no + (q[2] - 1)];
      }
      std::copy(full.begin() + n1, full.end(), mtm + ns);
    }
    return ADCGPU_OK;
  };
  st = run();
  cleanup();
  return st;
}

}  // namespace adcgpu

using namespace adcgpu;

extern "C" int adcgpu_fill_stvc(int ndim, const double* vctr, int lmain, int32_t* stvc_lbl) {
  if (ndim <= 0 || lmain <= 0 || lmain > ndim || !vctr || !stvc_lbl) return ADCGPU_BAD_INPUT;
  // dsortindxa1('D') on vctr^2: the ascending heapsort with every comparison
  // reversed, i.e. the ascending one on the negated keys
  std::vector<double> neg((size_t)ndim);
  for (int i = 0; i < ndim; ++i) neg[i] = -(vctr[i] * vctr[i]);
  std::vector<int64_t> indx;
  host_heapsort_index(ndim, neg.data(), indx);
  for (int i = 0; i < lmain; ++i) stvc_lbl[i] = (int32_t)indx[i];
  return ADCGPU_OK;
}
