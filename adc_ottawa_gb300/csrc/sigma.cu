// Sigma-vector product W = H V for a block of m vectors.
//
// Replaces hxvec_incore (block_davidson.f90:844-883), hxq_incore
// (block_lanczos.f90:1325-1361) and matxvec_treal_incore (tdselib.f90:352-437).
// The reference streams its 16-byte COO triples once per vector column with
// scattered updates; here the matrix is read once per block of columns:
//
//   W1 = diag1 . V1 + A V1 + B V2       (A dense n1 x n1, B index-free)
//   W2 = diag2 . V2 + B^T V1
//
// k_doubles: one warp per row of B^T (a double).  Lanes stride over the
// row's entries (coalesced value loads); W2[d] is a warp reduction of
// val * V1[s]; the B V2 contributions val * V2[d] go to a per-CTA partial of W1
// in shared memory, flushed to global memory once per CTA.  V1 (n1 x m) is
// tiny and stays in L1/L2.
// k_singles: W1 = diag1 . V1 + A V1 as a tiled dense product (n1 <= ~5000).
#include <cuda_bf16.h>

#include <mutex>
#include <type_traits>

#include "df.h"
#include "internal.h"

namespace adcgpu {

namespace {

// 8 consecutive stored values -> T (one 16-byte load for BF16, two for FP32,
// four for FP64; segments start on 16-byte boundaries).
template <typename T, typename TV> struct Load8;
template <> struct Load8<float, __nv_bfloat16> {
  __device__ __forceinline__ static void go(const __nv_bfloat16* p, float (&v)[8]) {
    uint4 q = __ldg(reinterpret_cast<const uint4*>(p));
    const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&q);
#pragma unroll
    for (int i = 0; i < 4; ++i) { float2 f = __bfloat1622float2(h[i]); v[2 * i] = f.x; v[2 * i + 1] = f.y; }
  }
};
template <> struct Load8<float, float> {
  __device__ __forceinline__ static void go(const float* p, float (&v)[8]) {
    float4 a = __ldg(reinterpret_cast<const float4*>(p)), b = __ldg(reinterpret_cast<const float4*>(p) + 1);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
  }
};
template <> struct Load8<double, double> {
  __device__ __forceinline__ static void go(const double* p, double (&v)[8]) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      double2 d = __ldg(reinterpret_cast<const double2*>(p) + i);
      v[2 * i] = d.x; v[2 * i + 1] = d.y;
    }
  }
};

// Advance (a',b') to the next row of a slab in storage order.
__device__ __forceinline__ void next_pair(int& ap, int& bp, bool twoa, int nv) {
  if (!twoa) { ++ap; bp = ap; return; }
  if (++bp == nv) { ++ap; bp = ap + 1; }
}

// Pass 1: one warp per work item (rows of one slab: fixed k', l', class).
// The row's A, C and D segments are split in 8-value chunks; lane l owns
// chunks l and l + 32 for the whole item (role A: singles (a', 8q..8q+7);
// C: (8q..8q+7, k'); D: (8q..8q+7, l')).  Products with V2 accumulate in
// registers (C/D: fixed targets; A: while a' is unchanged); W2 rows are
// written complete except for segment B, which pass 2 adds.  The next row's
// values and V2 entries are loaded before the current row is reduced.
template <typename T, typename TV, typename TA, int MC>
__global__ void __launch_bounds__(128) k_sigma_p1(GeomDev g, const int2* __restrict__ chunks, int nchunks,
                                                  const TV* __restrict__ Bt, const T* __restrict__ diag,
                                                  const T* __restrict__ V, int64_t ldv, T* __restrict__ W,
                                                  int64_t ldw, TA* __restrict__ W1, int64_t ld1) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int no = g.no, nv = g.nv;
  const int64_t n1 = g.n1;
  const int nA = g.noP / 8, nC = g.nvP / 8;
  for (int ci = warp; ci < nchunks; ci += nwarps) {
    const int2 ch = chunks[ci];
    Double r = decode_row(g, ch.x);
    const int cls = r.cls;
    const bool twoa = (cls == 1 || cls >= 3);
    const bool hasD = cls >= 2;
    const int64_t L = g.len[cls];
    const int offC = twoa ? 2 * g.noP : g.noP;
    const int kp = r.kp, lp = r.lp;
    const int nCh = nA + nC + (hasD ? nC : 0);
    // roles of the two owned chunks: 0 A, 1 C, 2 D, -1 none
    int role[2], base[2], moff[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const int q = lane + 32 * k;
      if (q >= nCh) { role[k] = -1; base[k] = 0; moff[k] = 0; }
      else if (q < nA) { role[k] = 0; base[k] = 8 * q; moff[k] = 8 * q; }
      else if (q < nA + nC) { role[k] = 1; base[k] = 8 * (q - nA); moff[k] = offC + 8 * (q - nA); }
      else { role[k] = 2; base[k] = 8 * (q - nA - nC); moff[k] = offC + g.nvP + 8 * (q - nA - nC); }
    }
    T xq[2][8][MC], yq[2][8][MC];
#pragma unroll
    for (int k = 0; k < 2; ++k)
#pragma unroll
      for (int u = 0; u < 8; ++u)
#pragma unroll
        for (int c = 0; c < MC; ++c) {
          yq[k][u][c] = T(0);
          const int a = base[k] + u;
          T x = T(0);
          if ((role[k] == 1 || role[k] == 2) && a < nv)
            x = V[(int64_t)c * ldv + (int64_t)a * no + (role[k] == 1 ? kp : lp)];
          xq[k][u][c] = x;
        }
    int cur_ap = -1;
    const TV* rowp = Bt + g.off[cls] + (int64_t)(ch.x - g.start[cls]) * L;
    int ap = r.ap, bp = r.bp;
    T cv[2][8], cx2[MC];
    int64_t cd;
    {
      Double rr{ap, bp, kp, lp, cls};
      cd = row_to_d(g, rr, ch.x);
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        if (role[k] >= 0) Load8<T, TV>::go(rowp + moff[k], cv[k]);
        else {
#pragma unroll
          for (int u = 0; u < 8; ++u) cv[k][u] = T(0);
        }
      }
#pragma unroll
      for (int c = 0; c < MC; ++c) cx2[c] = V[(int64_t)c * ldv + n1 + cd];
    }
    for (int row = ch.x; row < ch.y; ++row) {
      // prefetch the next row
      int nap = ap, nbp = bp;
      next_pair(nap, nbp, twoa, nv);
      T nv_[2][8], nx2[MC];
      int64_t nd = 0;
      const bool more = row + 1 < ch.y;
      if (more) {
        Double rr{nap, nbp, kp, lp, cls};
        nd = row_to_d(g, rr, row + 1);
      }
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        if (more && role[k] >= 0) Load8<T, TV>::go(rowp + L + moff[k], nv_[k]);
        else {
#pragma unroll
          for (int u = 0; u < 8; ++u) nv_[k][u] = T(0);
        }
      }
#pragma unroll
      for (int c = 0; c < MC; ++c) nx2[c] = more ? V[(int64_t)c * ldv + n1 + nd] : T(0);
      // segment A targets change with a'
      if (ap != cur_ap) {
#pragma unroll
        for (int k = 0; k < 2; ++k) {
          if (role[k] == 0) {
#pragma unroll
            for (int u = 0; u < 8; ++u) {
              const int kk = base[k] + u;
#pragma unroll
              for (int c = 0; c < MC; ++c) {
                if (cur_ap >= 0 && kk < no && yq[k][u][c] != T(0))
                  atomicAdd(&W1[(int64_t)c * ld1 + (int64_t)cur_ap * no + kk], (TA)yq[k][u][c]);
                yq[k][u][c] = T(0);
                xq[k][u][c] = kk < no ? V[(int64_t)c * ldv + (int64_t)ap * no + kk] : T(0);
              }
            }
          }
        }
        cur_ap = ap;
      }
      T z[MC];
#pragma unroll
      for (int c = 0; c < MC; ++c) z[c] = T(0);
#pragma unroll
      for (int k = 0; k < 2; ++k)
#pragma unroll
        for (int u = 0; u < 8; ++u)
#pragma unroll
          for (int c = 0; c < MC; ++c) {
            yq[k][u][c] += cv[k][u] * cx2[c];
            z[c] += cv[k][u] * xq[k][u][c];
          }
#pragma unroll
      for (int c = 0; c < MC; ++c) {
        T v = z[c];
#pragma unroll
        for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) W[(int64_t)c * ldw + n1 + cd] = diag[n1 + cd] * cx2[c] + v;
      }
      ap = nap; bp = nbp; rowp += L; cd = nd;
#pragma unroll
      for (int k = 0; k < 2; ++k)
#pragma unroll
        for (int u = 0; u < 8; ++u) cv[k][u] = nv_[k][u];
#pragma unroll
      for (int c = 0; c < MC; ++c) cx2[c] = nx2[c];
    }
    // flush the register accumulators
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      if (role[k] < 0) continue;
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int idx = base[k] + u;
        int64_t tgt = -1;
        if (role[k] == 0) { if (idx < no) tgt = (int64_t)cur_ap * no + idx; }
        else if (idx < nv) tgt = (int64_t)idx * no + (role[k] == 1 ? kp : lp);
        if (tgt < 0) continue;
#pragma unroll
        for (int c = 0; c < MC; ++c)
          if (yq[k][u][c] != T(0)) atomicAdd(&W1[(int64_t)c * ld1 + tgt], (TA)yq[k][u][c]);
      }
    }
  }
}

// Pass 1, staged variant: the same computation, but each lane copies the
// 16-byte pieces of its two chunks of the next NS-1 rows (and lanes < MC the
// row's V2 entries) into a per-warp shared-memory ring with cp.async, so NS
// rows per warp are in flight without holding them in registers.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
template <int BYTES>
__device__ __forceinline__ void cp_async_small(void* smem, const void* gmem) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(s), "l"(gmem), "n"(BYTES));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

template <typename T, typename TV> struct FromSmem8;
template <> struct FromSmem8<float, __nv_bfloat16> {
  __device__ __forceinline__ static void go(const void* p, float (&v)[8]) {
    uint4 q = *reinterpret_cast<const uint4*>(p);
    const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&q);
#pragma unroll
    for (int i = 0; i < 4; ++i) { float2 f = __bfloat1622float2(h[i]); v[2 * i] = f.x; v[2 * i + 1] = f.y; }
  }
};
template <> struct FromSmem8<float, float> {
  __device__ __forceinline__ static void go(const void* p, float (&v)[8]) {
    const float4* q = reinterpret_cast<const float4*>(p);
    float4 a = q[0], b = q[1];
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
  }
};
template <> struct FromSmem8<double, double> {
  __device__ __forceinline__ static void go(const void* p, double (&v)[8]) {
    const double2* q = reinterpret_cast<const double2*>(p);
#pragma unroll
    for (int i = 0; i < 4; ++i) { double2 d = q[i]; v[2 * i] = d.x; v[2 * i + 1] = d.y; }
  }
};

template <typename T, typename TV, typename TA, int MC, int NS>
__global__ void __launch_bounds__(128) k_sigma_p1s(GeomDev g, const int2* __restrict__ chunks, int nchunks,
                                                   const TV* __restrict__ Bt, const T* __restrict__ diag,
                                                   const T* __restrict__ V, int64_t ldv, T* __restrict__ W,
                                                   int64_t ldw, TA* __restrict__ W1, int64_t ld1) {
  constexpr int CB = 8 * sizeof(TV);              // bytes of one 8-value chunk
  constexpr int LANE_B = 2 * CB;                  // per lane per stage
  constexpr int STAGE_B = 32 * LANE_B + 16 * MC;  // + V2 entries (padded)
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  unsigned char* ring = smem_raw + (size_t)(threadIdx.x >> 5) * NS * STAGE_B;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int no = g.no, nv = g.nv;
  const int64_t n1 = g.n1;
  const int nA = g.noP / 8, nC = g.nvP / 8;
  for (int ci = warp; ci < nchunks; ci += nwarps) {
    const int2 ch = chunks[ci];
    Double r = decode_row(g, ch.x);
    const int cls = r.cls;
    const bool twoa = (cls == 1 || cls >= 3);
    const bool hasD = cls >= 2;
    const int64_t L = g.len[cls];
    const int offC = twoa ? 2 * g.noP : g.noP;
    const int kp = r.kp, lp = r.lp;
    const int nCh = nA + nC + (hasD ? nC : 0);
    int role[2], base[2], moff[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const int q = lane + 32 * k;
      if (q >= nCh) { role[k] = -1; base[k] = 0; moff[k] = 0; }
      else if (q < nA) { role[k] = 0; base[k] = 8 * q; moff[k] = 8 * q; }
      else if (q < nA + nC) { role[k] = 1; base[k] = 8 * (q - nA); moff[k] = offC + 8 * (q - nA); }
      else { role[k] = 2; base[k] = 8 * (q - nA - nC); moff[k] = offC + g.nvP + 8 * (q - nA - nC); }
    }
    T xq[2][8][MC], yq[2][8][MC];
#pragma unroll
    for (int k = 0; k < 2; ++k)
#pragma unroll
      for (int u = 0; u < 8; ++u)
#pragma unroll
        for (int c = 0; c < MC; ++c) {
          yq[k][u][c] = T(0);
          const int a = base[k] + u;
          T x = T(0);
          if ((role[k] == 1 || role[k] == 2) && a < nv)
            x = V[(int64_t)c * ldv + (int64_t)a * no + (role[k] == 1 ? kp : lp)];
          xq[k][u][c] = x;
        }
    const TV* row0p = Bt + g.off[cls] + (int64_t)(ch.x - g.start[cls]) * L;
    // issue iterator
    int iap = r.ap, ibp = r.bp;
    int irow = ch.x;
    auto issue = [&](int slot) {
      if (irow < ch.y) {
        unsigned char* st = ring + slot * STAGE_B;
        const TV* rp = row0p + (int64_t)(irow - ch.x) * L;
#pragma unroll
        for (int k = 0; k < 2; ++k)
          if (role[k] >= 0) {
#pragma unroll
            for (int b = 0; b < CB; b += 16) cp_async16(st + lane * LANE_B + k * CB + b, (const char*)(rp + moff[k]) + b);
          }
        if (lane < MC) {
          Double rr{iap, ibp, kp, lp, cls};
          const int64_t d = row_to_d(g, rr, irow);
          cp_async_small<sizeof(T)>(st + 32 * LANE_B + lane * 16, &V[(int64_t)lane * ldv + n1 + d]);
        }
        next_pair(iap, ibp, twoa, nv);
        ++irow;
      }
      cp_async_commit();
    };
#pragma unroll
    for (int s0 = 0; s0 < NS - 1; ++s0) issue(s0);
    int cur_ap = -1;
    int ap = r.ap, bp = r.bp;
    int i = 0;
    for (int row = ch.x; row < ch.y; ++row, ++i) {
      issue((i + NS - 1) % NS);
      cp_async_wait<NS - 1>();
      __syncwarp();
      const unsigned char* st = ring + (i % NS) * STAGE_B;
      Double rr{ap, bp, kp, lp, cls};
      const int64_t cd = row_to_d(g, rr, row);
      T cx2[MC];
#pragma unroll
      for (int c = 0; c < MC; ++c) cx2[c] = *reinterpret_cast<const T*>(st + 32 * LANE_B + c * 16);
      if (ap != cur_ap) {
#pragma unroll
        for (int k = 0; k < 2; ++k) {
          if (role[k] == 0) {
#pragma unroll
            for (int u = 0; u < 8; ++u) {
              const int kk = base[k] + u;
#pragma unroll
              for (int c = 0; c < MC; ++c) {
                if (cur_ap >= 0 && kk < no && yq[k][u][c] != T(0))
                  atomicAdd(&W1[(int64_t)c * ld1 + (int64_t)cur_ap * no + kk], (TA)yq[k][u][c]);
                yq[k][u][c] = T(0);
                xq[k][u][c] = kk < no ? V[(int64_t)c * ldv + (int64_t)ap * no + kk] : T(0);
              }
            }
          }
        }
        cur_ap = ap;
      }
      T z[MC];
#pragma unroll
      for (int c = 0; c < MC; ++c) z[c] = T(0);
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        if (role[k] < 0) continue;
        T v[8];
        FromSmem8<T, TV>::go(st + lane * LANE_B + k * CB, v);
#pragma unroll
        for (int u = 0; u < 8; ++u)
#pragma unroll
          for (int c = 0; c < MC; ++c) {
            yq[k][u][c] += v[u] * cx2[c];
            z[c] += v[u] * xq[k][u][c];
          }
      }
#pragma unroll
      for (int c = 0; c < MC; ++c) {
        T v = z[c];
#pragma unroll
        for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) W[(int64_t)c * ldw + n1 + cd] = diag[n1 + cd] * cx2[c] + v;
      }
      __syncwarp();
      next_pair(ap, bp, twoa, nv);
    }
    cp_async_wait<0>();
    __syncwarp();
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      if (role[k] < 0) continue;
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int idx = base[k] + u;
        int64_t tgt = -1;
        if (role[k] == 0) { if (idx < no) tgt = (int64_t)cur_ap * no + idx; }
        else if (idx < nv) tgt = (int64_t)idx * no + (role[k] == 1 ? kp : lp);
        if (tgt < 0) continue;
#pragma unroll
        for (int c = 0; c < MC; ++c)
          if (yq[k][u][c] != T(0)) atomicAdd(&W1[(int64_t)c * ld1 + tgt], (TA)yq[k][u][c]);
      }
    }
  }
}

// Pass 2: segment B (classes 2, 4I, 4II).  One warp per (slab, b'): rows
// (a', b') for a' < b' share the target singles (b', k).  Lanes form groups
// of GS (>= noP/8 chunks of segment B): group slot = row, lane in group =
// 8-value chunk.  32/GS rows are in flight per step; partial W1 sums reduce
// across groups at the end, W2 sums within a group.
template <typename T, typename TV, typename TA, int MC, int GS>
__global__ void __launch_bounds__(256) k_sigma_p2(GeomDev g, const int2* __restrict__ items, int nitems,
                                                  const TV* __restrict__ Bt, const T* __restrict__ V, int64_t ldv,
                                                  T* __restrict__ W, int64_t ldw, TA* __restrict__ W1, int64_t ld1) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int no = g.no, nv = g.nv;
  const int64_t n1 = g.n1;
  const int nB = g.noP / 8;
  const int slot = lane / GS, h = lane % GS;
  constexpr int RPS = 32 / GS;   // rows per step
  for (int it = warp; it < nitems; it += nwarps) {
    const int2 item = items[it];
    const int slab0 = item.x, bp = item.y;
    Double r = decode_row(g, slab0);
    const int cls = r.cls;
    const int64_t L = g.len[cls];
    const bool act = h < nB;
    T xb[8][MC], yb[8][MC];
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
      for (int c = 0; c < MC; ++c) {
        const int kk = 8 * h + u;
        xb[u][c] = (act && kk < no) ? V[(int64_t)c * ldv + (int64_t)bp * no + kk] : T(0);
        yb[u][c] = T(0);
      }
    for (int a0 = 0; a0 < bp; a0 += RPS) {
      const int ap = a0 + slot;
      const bool rv = ap < bp;
      T v[8], x2[MC], w2[MC];
      int64_t d = 0;
      if (rv) {
        const int64_t row = slab0 + pair_index(ap, bp, nv);
        Double rr{ap, bp, r.kp, r.lp, cls};
        d = row_to_d(g, rr, row);
        if (act) Load8<T, TV>::go(Bt + g.off[cls] + (row - g.start[cls]) * L + g.noP + 8 * h, v);
      }
      if (!(rv && act)) {
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = T(0);
      }
#pragma unroll
      for (int c = 0; c < MC; ++c) {
        x2[c] = rv ? V[(int64_t)c * ldv + n1 + d] : T(0);
        w2[c] = (rv && h == 0) ? W[(int64_t)c * ldw + n1 + d] : T(0);
      }
#pragma unroll
      for (int c = 0; c < MC; ++c) {
        T z = T(0);
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          yb[u][c] += v[u] * x2[c];
          z += v[u] * xb[u][c];
        }
#pragma unroll
        for (int o = 1; o < GS; o <<= 1) z += __shfl_xor_sync(0xffffffffu, z, o);
        if (rv && h == 0) W[(int64_t)c * ldw + n1 + d] = w2[c] + z;
      }
    }
    // sum yb over the row slots (lanes with equal h), then flush
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
      for (int c = 0; c < MC; ++c) {
        T y = yb[u][c];
#pragma unroll
        for (int o = GS; o < 32; o <<= 1) y += __shfl_xor_sync(0xffffffffu, y, o);
        yb[u][c] = y;
      }
    if (slot == 0 && act) {
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int kk = 8 * h + u;
        if (kk >= no) continue;
#pragma unroll
        for (int c = 0; c < MC; ++c)
          if (yb[u][c] != T(0)) atomicAdd(&W1[(int64_t)c * ld1 + (int64_t)bp * no + kk], (TA)yb[u][c]);
      }
    }
  }
}

// Pass 3: the W1 part of segment A, W1[(a', k), c] += sum over the rows of
// (a', b') of A[row, k] V2[row, c], for the tensor-core pass (which does the
// W2 part of segment A itself).  One warp per run of rows with equal a' in
// one slab (contiguous in storage: item = (first row, row count)).  Lanes
// form groups of GS (>= noP/8 chunks of segment A); 32/GS rows per step; the
// sums reduce across groups at the end, one atomic per (single, column).
template <typename TV, int MC, int GS>
__global__ void __launch_bounds__(256) k_sigma_p3(GeomDev g, const int2* __restrict__ runs, int nruns,
                                                  const TV* __restrict__ Bt, const float* __restrict__ V,
                                                  int64_t ldv, double* __restrict__ W1, int64_t ld1) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int no = g.no;
  const int64_t n1 = g.n1;
  const int nA = g.noP / 8;
  const int slot = lane / GS, h = lane % GS;
  constexpr int RPS = 32 / GS;
  for (int it = warp; it < nruns; it += nwarps) {
    const int2 run = runs[it];
    const Double r0 = decode_row(g, run.x);
    const int cls = r0.cls, ap = r0.ap;
    const bool twoa = (cls == 1 || cls >= 3);
    const int64_t L = g.len[cls];
    const bool act = h < nA;
    float ya[8][MC];
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
      for (int c = 0; c < MC; ++c) ya[u][c] = 0.f;
    for (int r = slot; r < run.y; r += RPS) {
      const int64_t row = run.x + r;
      // rows of one run: (a', a' + 1 + r) for a' < b' classes, (a', a') otherwise
      const Double rr{ap, twoa ? ap + 1 + r : ap, r0.kp, r0.lp, cls};
      const int64_t d = row_to_d(g, rr, row);
      float v[8];
      if (act) Load8<float, TV>::go(Bt + g.off[cls] + (row - g.start[cls]) * L + 8 * h, v);
      else {
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = 0.f;
      }
#pragma unroll
      for (int c = 0; c < MC; ++c) {
        const float x2 = V[(int64_t)c * ldv + n1 + d];
#pragma unroll
        for (int u = 0; u < 8; ++u) ya[u][c] += v[u] * x2;
      }
    }
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
      for (int c = 0; c < MC; ++c) {
        float y = ya[u][c];
#pragma unroll
        for (int o = GS; o < 32; o <<= 1) y += __shfl_xor_sync(0xffffffffu, y, o);
        ya[u][c] = y;
      }
    if (slot == 0 && act) {
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int kk = 8 * h + u;
        if (kk >= no) continue;
#pragma unroll
        for (int c = 0; c < MC; ++c)
          if (ya[u][c] != 0.f) atomicAdd(&W1[(int64_t)c * ld1 + (int64_t)ap * no + kk], (double)ya[u][c]);
      }
    }
  }
}

// Arithmetic of the tiled pass 1.  Native: values, vectors and sums in T.
// DF (FP64 inputs only): the C|D values and the vectors are held in shared
// memory as double-float pairs and multiplied on the FP32 pipe (df.h), and so
// are segment A and the per-item W1 sums; only the diagonal term is FP64.
template <typename T> struct NativeArith {
  typedef T S;
  __device__ __forceinline__ static S from(T x) { return x; }
  __device__ __forceinline__ static S zero() { return T(0); }
  __device__ __forceinline__ static void fma(S& acc, S a, S b) { acc += a * b; }
  __device__ __forceinline__ static S add(S a, S b) { return a + b; }
  __device__ __forceinline__ static S shfl_add(S a, int off) { return a + __shfl_xor_sync(0xffffffffu, a, off); }
  __device__ __forceinline__ static T value(S a) { return a; }
  __device__ __forceinline__ static bool nonzero(S a) { return a != T(0); }
};
struct DfArith {
  typedef df S;
  __device__ __forceinline__ static S from(double x) { return df_split(x); }
  __device__ __forceinline__ static S zero() { return df{0.f, 0.f}; }
  __device__ __forceinline__ static void fma(S& acc, S a, S b) { df_fma(acc, a, b); }
  __device__ __forceinline__ static S add(S a, S b) { return df_add(a, b); }
  __device__ __forceinline__ static S shfl_add(S a, int off) {
    return df_add(a, df{__shfl_xor_sync(0xffffffffu, a.hi, off), __shfl_xor_sync(0xffffffffu, a.lo, off)});
  }
  __device__ __forceinline__ static double value(S a) { return df_value(a); }
  __device__ __forceinline__ static bool nonzero(S a) { return a.hi != 0.f || a.lo != 0.f; }
};

template <typename T> struct DfArithSel { typedef NativeArith<T> type; };
template <> struct DfArithSel<double> { typedef DfArith type; };
template <typename T> using DfArithFor = typename DfArithSel<T>::type;

// 4 consecutive values from 16-byte aligned shared memory
template <typename S> struct Vec4;
template <> struct Vec4<float> {
  __device__ __forceinline__ static void ld(const float* p, float (&v)[4]) {
    const float4 q = *reinterpret_cast<const float4*>(p);
    v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
  }
};
template <> struct Vec4<double> {
  __device__ __forceinline__ static void ld(const double* p, double (&v)[4]) {
    const double2 q0 = reinterpret_cast<const double2*>(p)[0], q1 = reinterpret_cast<const double2*>(p)[1];
    v[0] = q0.x; v[1] = q0.y; v[2] = q1.x; v[3] = q1.y;
  }
};
template <> struct Vec4<df> {
  __device__ __forceinline__ static void ld(const df* p, df (&v)[4]) {
    const float4 q0 = reinterpret_cast<const float4*>(p)[0], q1 = reinterpret_cast<const float4*>(p)[1];
    v[0] = df{q0.x, q0.y}; v[1] = df{q0.z, q0.w}; v[2] = df{q1.x, q1.y}; v[3] = df{q1.z, q1.w};
  }
};

// Vec4 with the two 16-byte halves of a double-float group loaded in the
// order given by h (0: first half first).  Lanes that read the same bank set
// are given opposite h, so each quarter-warp's 16-byte loads fall on disjoint
// banks; for the one-word types the load is Vec4::ld.
template <typename S> struct Vec4h {
  __device__ __forceinline__ static void ld(const S* p, S (&v)[4], int) { Vec4<S>::ld(p, v); }
};
template <> struct Vec4h<df> {
  __device__ __forceinline__ static void ld(const df* p, df (&v)[4], int h) {
    const float4* q = reinterpret_cast<const float4*>(p);
    const float4 first = q[h], second = q[1 - h];
    const float4 q0 = h ? second : first, q1 = h ? first : second;
    v[0] = df{q0.x, q0.y}; v[1] = df{q0.z, q0.w}; v[2] = df{q1.x, q1.y}; v[3] = df{q1.z, q1.w};
  }
};

// 8 values to 16-byte aligned shared memory as vector stores
template <typename S> struct Store8;
template <> struct Store8<float> {
  __device__ __forceinline__ static void go(float* d, const float (&v)[8]) {
    reinterpret_cast<float4*>(d)[0] = make_float4(v[0], v[1], v[2], v[3]);
    reinterpret_cast<float4*>(d)[1] = make_float4(v[4], v[5], v[6], v[7]);
  }
};
template <> struct Store8<double> {
  __device__ __forceinline__ static void go(double* d, const double (&v)[8]) {
#pragma unroll
    for (int i = 0; i < 4; ++i) reinterpret_cast<double2*>(d)[i] = make_double2(v[2 * i], v[2 * i + 1]);
  }
};
template <> struct Store8<df> {
  __device__ __forceinline__ static void go(df* d, const df (&v)[8]) {
#pragma unroll
    for (int i = 0; i < 4; ++i)
      reinterpret_cast<float4*>(d)[i] = make_float4(v[2 * i].hi, v[2 * i].lo, v[2 * i + 1].hi, v[2 * i + 1].lo);
  }
};

// ---------------------------------------------------------------------------
// Tiled pass 1: one block per work item (up to TILE_ITEM_ROWS consecutive
// rows of one slab), all MT columns of a column group at once, so the matrix
// is streamed once per MT columns instead of once per MC.
//
// For a slab (fixed k', l') the C and D segments of its rows form a dense
// rows x nvP block each, coupling to the fixed singles (a, k') and (a, l'):
//   W2[r, c] += sum_a C[r, a] Xk[a, c] + D[r, a] Xl[a, c]     (Xk = V[(a,k'), c])
//   W1[(a, k'), c] += sum_r C[r, a] V2[r, c]   (and D with l')
// Xk and Xl stay in shared memory for the whole item; each 32-row tile of
// C|D values is staged once and used for every column.  W2: 4 x CT output
// tiles, the K sum of each split over S lanes and reduced by shuffles.  W1:
// 4 k x 4 columns per thread over the tile's rows, added per tile to the
// item's sums in shared memory (T), which go to the TA accumulators of W1
// once at the end of the item.  Segment A (singles (a', k)) is handled per
// tile: its W2 part gathers V through L1, its W1 part is reduced over runs
// of equal a' and added atomically.  Segment B stays with pass 2.
// Shared memory (bytes): S sW1[nseg*nvP*MT] | S sX[MT*(2nvP+4)] (column-major)
// | S sCD[RT*(2nvP+4)] | S sA[RT*(noP+4)] | S sV2[RT*MT] | int64 sD[RT] |
// int sAp[RT] (row strides are multiples of 16 bytes, so the staging stores
// are 16-byte vector stores, and 4 rows read in one warp fall into
// different banks).
// ---------------------------------------------------------------------------
constexpr int TILE_RT = 32;
constexpr int TILE_ITEM_ROWS = 1024;

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) / 16 * 16; }

inline size_t tile_smem_bytes(int nvP, int noP, int MT, size_t sT, size_t sS) {
  size_t b = align16((size_t)2 * nvP * MT * sT);
  b += align16((size_t)MT * (2 * nvP + 4) * sS);
  b += align16((size_t)TILE_RT * (2 * nvP + 4) * sS);
  b += align16((size_t)TILE_RT * (noP + 4) * sS);
  b += align16((size_t)TILE_RT * MT * sS);
  b += align16((size_t)TILE_RT * 8);
  b += align16((size_t)TILE_RT * 4);
  return b;
}

template <typename T, typename TV, typename TA, int MT, typename AR>
__global__ void __launch_bounds__(256, 1) k_sigma_tile(GeomDev g, const int2* __restrict__ titems, int ntitems,
                                                    const TV* __restrict__ Bt, const T* __restrict__ diag,
                                                    const T* __restrict__ V, int64_t ldv, int mcols,
                                                    T* __restrict__ W, int64_t ldw, TA* __restrict__ W1,
                                                    int64_t ld1) {
  typedef typename AR::S S;
  constexpr int RT = TILE_RT;
  static_assert((MT & (MT - 1)) == 0, "the W1 accumulator swizzle needs a power-of-two column tile");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int no = g.no, nv = g.nv, noP = g.noP, nvP = g.nvP;
  const int64_t n1 = g.n1;
  const int CDS = 2 * nvP + 4, AS = noP + 4, KP = 2 * nvP + 4;
  unsigned char* p = smem_raw;
  S* sW1 = reinterpret_cast<S*>(p); p += align16((size_t)2 * nvP * MT * sizeof(S));
  S* sX = reinterpret_cast<S*>(p); p += align16((size_t)MT * (2 * nvP + 4) * sizeof(S));
  S* sCD = reinterpret_cast<S*>(p); p += align16((size_t)RT * CDS * sizeof(S));
  S* sA = reinterpret_cast<S*>(p); p += align16((size_t)RT * AS * sizeof(S));
  S* sV2 = reinterpret_cast<S*>(p); p += align16((size_t)RT * MT * sizeof(S));
  int64_t* sD = reinterpret_cast<int64_t*>(p); p += align16((size_t)RT * 8);
  int* sAp = reinterpret_cast<int*>(p);
  const int tid = threadIdx.x;
  for (int it = blockIdx.x; it < ntitems; it += gridDim.x) {
    const int2 item = titems[it];
    const Double r0 = decode_row(g, item.x);
    const int cls = r0.cls;
    const bool twoa = (cls == 1 || cls >= 3);
    const int nseg = cls >= 2 ? 2 : 1;
    const int K = nseg * nvP;
    const int64_t L = g.len[cls];
    const int offC = twoa ? 2 * noP : noP;
    const int kp = r0.kp, lp = r0.lp;
    const TV* base = Bt + g.off[cls];   // row r starts at base + (r - start[cls]) * L
    __syncthreads();
    for (int o = tid; o < K * MT; o += 256) {
      const int k = o % K, c = o / K;
      const int seg = k / nvP, a = k - seg * nvP;
      sX[c * KP + k] =
          AR::from((a < nv && c < mcols) ? V[(int64_t)c * ldv + (int64_t)a * no + (seg ? lp : kp)] : T(0));
      sW1[k * MT + c] = AR::zero();
    }
    for (int row0 = item.x; row0 < item.y; row0 += RT) {
      const int nrow = min(RT, item.y - row0);
      __syncthreads();
      if (tid < RT) {
        int ap = -1;
        int64_t d = 0;
        if (tid < nrow) {
          const Double rr = decode_row(g, row0 + tid);
          ap = rr.ap;
          d = row_to_d(g, rr, row0 + tid);
        }
        sAp[tid] = ap;
        sD[tid] = d;
      }
      // C|D and A values, 8 at a time (segments start on 8-value boundaries)
      const int nchK = K / 8, nchA = noP / 8;
      for (int o = tid; o < RT * (nchK + nchA); o += 256) {
        const int rr = o / (nchK + nchA), q = o - rr * (nchK + nchA);
        T v[8];
        if (rr < nrow) {
          const TV* rp = base + (int64_t)(row0 + rr - g.start[cls]) * L + (q < nchK ? offC + 8 * q : 8 * (q - nchK));
          Load8<T, TV>::go(rp, v);
        } else {
#pragma unroll
          for (int u = 0; u < 8; ++u) v[u] = T(0);
        }
        S w[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) w[u] = AR::from(v[u]);
        Store8<S>::go(q < nchK ? sCD + rr * CDS + 8 * q : sA + rr * AS + 8 * (q - nchK), w);
      }
      __syncthreads();
      for (int o = tid; o < RT * MT; o += 256) {
        const int rr = o % RT, c = o / RT;
        sV2[rr * MT + c] = AR::from((rr < nrow && c < mcols) ? V[(int64_t)c * ldv + n1 + sD[rr]] : T(0));
      }
      __syncthreads();
      // W2 rows of the tile: 4 x CT output tiles (CT = 4 for FP32 values, 2
      // for 8-byte ones, to stay within registers)
      {
        constexpr int CT = sizeof(S) == 4 ? 4 : 2;
        constexpr int NMT = (RT / 4) * (MT / CT);
        constexpr int SPL = 256 / NMT;
        const int mt = tid / SPL, ks = tid % SPL;
        const int r0 = 4 * (mt % (RT / 4)), c0 = CT * (mt / (RT / 4));
        S acc[4][CT];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int cc = 0; cc < CT; ++cc) acc[i][cc] = AR::zero();
        for (int k4 = ks; k4 < K / 4; k4 += SPL) {
          S a[4][4], x[CT][4];
#pragma unroll
          for (int i = 0; i < 4; ++i) Vec4h<S>::ld(sCD + (r0 + i) * CDS + 4 * k4, a[i], mt & 1);
#pragma unroll
          for (int cc = 0; cc < CT; ++cc) Vec4<S>::ld(sX + (c0 + cc) * KP + 4 * k4, x[cc]);
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int cc = 0; cc < CT; ++cc)
#pragma unroll
              for (int jj = 0; jj < 4; ++jj) AR::fma(acc[i][cc], a[i][jj], x[cc][jj]);
        }
#pragma unroll
        for (int off = SPL / 2; off > 0; off >>= 1)
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int cc = 0; cc < CT; ++cc) acc[i][cc] = AR::shfl_add(acc[i][cc], off);
#pragma unroll
        for (int q = 0; q < 4 * CT; ++q) {
          if (q % SPL != ks) continue;
          const int rr = r0 + q / CT, c = c0 + q % CT;
          if (rr >= nrow || c >= mcols) continue;
          const int ap = sAp[rr];
          const int64_t d = sD[rr];
          const S* arow = sA + rr * AS;
          const T* vs = V + (int64_t)c * ldv + (int64_t)ap * no;
          S sa = acc[q / CT][q % CT];
          // padded A entries are zero; (ap, kk >= no) stays inside the V column
#pragma unroll 8
          for (int kk = 0; kk < noP; ++kk) AR::fma(sa, arow[kk], AR::from(vs[kk]));
          W[(int64_t)c * ldw + n1 + d] = diag[n1 + d] * AR::value(sV2[rr * MT + c]) + AR::value(sa);
        }
      }
      // W1 (C|D): thread owns 4 k x 4 columns; sums over the tile's rows
      for (int o = tid; o < (K / 4) * (MT / 4); o += 256) {
        const int kq = o % (K / 4), cg = o / (K / 4);
        S sm[4][4];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int cc = 0; cc < 4; ++cc) sm[i][cc] = AR::zero();
#pragma unroll 2
        for (int rr = 0; rr < RT; ++rr) {
          S a[4], v[4];
          Vec4h<S>::ld(sCD + rr * CDS + 4 * kq, a, (kq >> 2) & 1);
          Vec4<S>::ld(sV2 + rr * MT + 4 * cg, v);
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int cc = 0; cc < 4; ++cc) AR::fma(sm[i][cc], a[i], v[cc]);
        }
        // sW1 row k holds column c at c ^ (k/4 mod MT): consecutive kq of a
        // warp then touch different banks
        const int swz = kq & (MT - 1);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          S* w = sW1 + (4 * kq + i) * MT;
#pragma unroll
          for (int cc = 0; cc < 4; ++cc) {
            const int pos = (4 * cg + cc) ^ swz;
            w[pos] = AR::add(w[pos], sm[i][cc]);
          }
        }
      }
      // W1 (A): runs of equal a' reduced, then added atomically
      for (int o = tid; o < noP * MT; o += 256) {
        const int kk = o % noP, c = o / noP;
        if (kk >= no || c >= mcols) continue;
        S sacc = AR::zero();
        int prev = sAp[0];
        for (int rr = 0; rr < nrow; ++rr) {
          const int ap = sAp[rr];
          if (ap != prev) {
            if (AR::nonzero(sacc)) atomicAdd(&W1[(int64_t)c * ld1 + (int64_t)prev * no + kk], (TA)AR::value(sacc));
            sacc = AR::zero();
            prev = ap;
          }
          AR::fma(sacc, sA[rr * AS + kk], sV2[rr * MT + c]);
        }
        if (AR::nonzero(sacc)) atomicAdd(&W1[(int64_t)c * ld1 + (int64_t)prev * no + kk], (TA)AR::value(sacc));
      }
    }
    __syncthreads();
    for (int o = tid; o < K * MT; o += 256) {
      const int k = o / MT, c = (o - k * MT) ^ ((k >> 2) & (MT - 1));
      const int seg = k / nvP, a = k - seg * nvP;
      const T v = AR::value(sW1[o]);
      if (a < nv && c < mcols && v != T(0))
        atomicAdd(&W1[(int64_t)c * ld1 + (int64_t)a * no + (seg ? lp : kp)], (TA)v);
    }
  }
}

// ---------------------------------------------------------------------------
// Tiled pass 1 on the tensor cores (BF16 values, FP32 vectors): the same
// work items and tiles as k_sigma_tile, 16 columns per pass.  The vectors
// enter as BF16 hi + lo pairs (x = hi + lo to ~2^-17), each product is two
// mma.sync m16n8k16 (BF16 in, FP32 accumulate).
//   warps 0-3: W2[32 x 16] = C|D[32 x K] . X[K x 16]   (one 16 x 8 tile each)
//   warps 4-7: W1^T[16 x K] += V2^T[16 x 32] . C|D[32 x K], the item's sums
//              held in the accumulators, added to W1 (FP64) at the end.
// K is rounded up to 16 with zero padding.  Segment A and the diagonal term
// stay on the CUDA cores as in k_sigma_tile; segment B stays with pass 2.
// The raw C|D and A values of tile t+1 stream into a second stage with
// cp.async (zero-filled past K and past the item's rows) while tile t is
// multiplied; the transposed copy used by W1 is built in shared memory.
// Shared memory: see tile_mma_smem_bytes.
// ---------------------------------------------------------------------------
constexpr int MMA_MT = 16;
constexpr int MMA_RTP = TILE_RT + 8;

inline size_t tile_mma_smem_bytes(int nvP, int noP) {
  const size_t KP = (size_t)2 * nvP + 8;
  size_t b = 2 * align16((size_t)TILE_RT * KP * 2);           // raw C|D tiles (2 stages)
  b += 2 * align16((size_t)TILE_RT * noP * 2);                // raw A tiles (2 stages)
  b += align16(KP * MMA_RTP * 2);                             // transposed C|D
  b += 2 * align16((size_t)MMA_MT * KP * 2);                  // X hi, lo
  b += 2 * align16((size_t)MMA_MT * MMA_RTP * 2);             // V2^T hi, lo
  b += align16((size_t)TILE_RT * MMA_MT * 4);                 // V2 (f32)
  b += align16((size_t)TILE_RT * (noP + 4) * 4);              // A (f32)
  b += 2 * align16((size_t)TILE_RT * 8);                      // d (2 stages)
  b += 2 * align16((size_t)TILE_RT * 4);                      // a' (2 stages)
  return b;
}

__device__ __forceinline__ void mma16816(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t ld_u32(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

// 16-byte cp.async that reads src_bytes (16 or 0) and zero-fills the rest
__device__ __forceinline__ void cp_async16_zf(void* smem, const void* gmem, int src_bytes) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(src_bytes));
}

template <typename TA>
__global__ void __launch_bounds__(256, 2) k_sigma_tile_mma(GeomDev g, const int2* __restrict__ titems, int ntitems,
                                                           const __nv_bfloat16* __restrict__ Bt,
                                                           const float* __restrict__ diag,
                                                           const float* __restrict__ V, int64_t ldv, int mcols,
                                                           float* __restrict__ W, int64_t ldw, TA* __restrict__ W1,
                                                           int64_t ld1) {
  constexpr int RT = TILE_RT, MT = MMA_MT, RTP = MMA_RTP;
  constexpr int NT1 = 16;                  // W1 n-tile slots per warp (K/8 <= 64)
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int no = g.no, nv = g.nv, noP = g.noP, nvP = g.nvP;
  const int64_t n1 = g.n1;
  // row stride 4 nvP + 16 bytes: an odd multiple of 16, so the 8 rows of a
  // fragment load fall into 8 different 16-byte bank groups
  const int KP = 2 * nvP + 8, AS = noP + 4;
  unsigned char* p = smem_raw;
  __nv_bfloat16* const sCDr0 = reinterpret_cast<__nv_bfloat16*>(p); p += align16((size_t)RT * KP * 2);
  __nv_bfloat16* const sCDr1 = reinterpret_cast<__nv_bfloat16*>(p); p += align16((size_t)RT * KP * 2);
  __nv_bfloat16* const sAr0 = reinterpret_cast<__nv_bfloat16*>(p); p += align16((size_t)RT * noP * 2);
  __nv_bfloat16* const sAr1 = reinterpret_cast<__nv_bfloat16*>(p); p += align16((size_t)RT * noP * 2);
  __nv_bfloat16* sCDt = reinterpret_cast<__nv_bfloat16*>(p); p += align16((size_t)KP * RTP * 2);
  __nv_bfloat16* sXh = reinterpret_cast<__nv_bfloat16*>(p); p += align16((size_t)MT * KP * 2);
  __nv_bfloat16* sXl = reinterpret_cast<__nv_bfloat16*>(p); p += align16((size_t)MT * KP * 2);
  __nv_bfloat16* sV2h = reinterpret_cast<__nv_bfloat16*>(p); p += align16((size_t)MT * RTP * 2);
  __nv_bfloat16* sV2l = reinterpret_cast<__nv_bfloat16*>(p); p += align16((size_t)MT * RTP * 2);
  float* sV2f = reinterpret_cast<float*>(p); p += align16((size_t)RT * MT * 4);
  float* sA = reinterpret_cast<float*>(p); p += align16((size_t)RT * AS * 4);
  int64_t* const sD0 = reinterpret_cast<int64_t*>(p); p += align16((size_t)RT * 8);
  int64_t* const sD1 = reinterpret_cast<int64_t*>(p); p += align16((size_t)RT * 8);
  int* const sAp0 = reinterpret_cast<int*>(p); p += align16((size_t)RT * 4);
  int* const sAp1 = reinterpret_cast<int*>(p);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int gid = lane >> 2, tig = lane & 3;
  for (int it = blockIdx.x; it < ntitems; it += gridDim.x) {
    const int2 item = titems[it];
    const Double r0 = decode_row(g, item.x);
    const int cls = r0.cls;
    const bool twoa = (cls == 1 || cls >= 3);
    const int nseg = cls >= 2 ? 2 : 1;
    const int K = nseg * nvP, K16 = (K + 15) / 16 * 16;
    const int64_t L = g.len[cls];
    const int offC = twoa ? 2 * noP : noP;
    const int kp = r0.kp, lp = r0.lp;
    const __nv_bfloat16* base = Bt + g.off[cls];   // row r starts at base + (r - start[cls]) * L
    const int nch16 = K16 / 8, nchK = K / 8, nchA = noP / 8;
    // raw C|D (row-major, zero past K) and A values of rows [r, r + RT) into stage b
    auto issue = [&](int rbeg, int b) {
      const int nr = min(RT, item.y - rbeg);
      for (int o = tid; o < RT * (nch16 + nchA); o += 256) {
        const int rr = o % RT, q = o / RT;
        const int64_t roff = (int64_t)(rbeg + rr - g.start[cls]) * L;
        if (q < nch16) {
          const bool ok = rr < nr && q < nchK;
          cp_async16_zf((b ? sCDr1 : sCDr0) + rr * KP + 8 * q, ok ? (const void*)(base + roff + offC + 8 * q) : (const void*)base,
                        ok ? 16 : 0);
        } else {
          const int qa = q - nch16;
          const bool ok = rr < nr;
          cp_async16_zf((b ? sAr1 : sAr0) + rr * noP + 8 * qa, ok ? (const void*)(base + roff + 8 * qa) : (const void*)base,
                        ok ? 16 : 0);
        }
      }
    };
    float acc1[NT1][4];
#pragma unroll
    for (int j = 0; j < NT1; ++j) acc1[j][0] = acc1[j][1] = acc1[j][2] = acc1[j][3] = 0.f;
    __syncthreads();   // the previous item is done with every buffer
    issue(item.x, 0);
    cp_async_commit();
    for (int o = tid; o < K16 * MT; o += 256) {
      const int k = o % K16, c = o / K16;
      const int seg = k / nvP, a = k - seg * nvP;
      const float x = (k < K && a < nv && c < mcols) ? V[(int64_t)c * ldv + (int64_t)a * no + (seg ? lp : kp)] : 0.f;
      const __nv_bfloat16 h = __float2bfloat16(x);
      sXh[c * KP + k] = h;
      sXl[c * KP + k] = __float2bfloat16(x - __bfloat162float(h));
    }
    int t = 0;
    for (int row0 = item.x; row0 < item.y; row0 += RT, ++t) {
      const int b = t & 1;
      const int nrow = min(RT, item.y - row0);
      int64_t* sD = b ? sD1 : sD0;
      int* sAp = b ? sAp1 : sAp0;
      if (tid < RT) {   // stage b's row data is not read by the previous tile
        int ap = -1;
        int64_t d = 0;
        if (tid < nrow) {
          const Double rr = decode_row(g, row0 + tid);
          ap = rr.ap;
          d = row_to_d(g, rr, row0 + tid);
        }
        sAp[tid] = ap;
        sD[tid] = d;
      }
      cp_async_wait<0>();
      __syncthreads();
      // prefetch the next tile into the other stage (its last readers, the
      // previous tile's products, are past the barrier above)
      if (row0 + RT < item.y) issue(row0 + RT, b ^ 1);
      cp_async_commit();
      const __nv_bfloat16* sCD = b ? sCDr1 : sCDr0;
      for (int o = tid; o < RT * nch16; o += 256) {
        const int rr = o % RT, q = o / RT;
        const uint4 u = *reinterpret_cast<const uint4*>(sCD + rr * KP + 8 * q);
        const __nv_bfloat16* e = reinterpret_cast<const __nv_bfloat16*>(&u);
#pragma unroll
        for (int v = 0; v < 8; ++v) sCDt[(8 * q + v) * RTP + rr] = e[v];
      }
      for (int o = tid; o < RT * nchA; o += 256) {
        const int rr = o % RT, qa = o / RT;
        float v[8];
        FromSmem8<float, __nv_bfloat16>::go((b ? sAr1 : sAr0) + rr * noP + 8 * qa, v);
        Store8<float>::go(sA + rr * AS + 8 * qa, v);
      }
      for (int o = tid; o < RT * MT; o += 256) {
        const int rr = o % RT, c = o / RT;
        const float x = (rr < nrow && c < mcols) ? V[(int64_t)c * ldv + n1 + sD[rr]] : 0.f;
        sV2f[rr * MT + c] = x;
        const __nv_bfloat16 h = __float2bfloat16(x);
        sV2h[c * RTP + rr] = h;
        sV2l[c * RTP + rr] = __float2bfloat16(x - __bfloat162float(h));
      }
      __syncthreads();
      if (warp < 4) {
        // W2 tile: rows 16 (warp & 1).., columns 8 (warp >> 1)..
        const int m0 = 16 * (warp & 1), n0 = 8 * (warp >> 1);
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        for (int k0 = 0; k0 < K16; k0 += 16) {
          uint32_t a[4];
          a[0] = ld_u32(sCD + (m0 + gid) * KP + k0 + 2 * tig);
          a[1] = ld_u32(sCD + (m0 + gid + 8) * KP + k0 + 2 * tig);
          a[2] = ld_u32(sCD + (m0 + gid) * KP + k0 + 2 * tig + 8);
          a[3] = ld_u32(sCD + (m0 + gid + 8) * KP + k0 + 2 * tig + 8);
          const int xo = (n0 + gid) * KP + k0 + 2 * tig;
          mma16816(acc, a, ld_u32(sXh + xo), ld_u32(sXh + xo + 8));
          mma16816(acc, a, ld_u32(sXl + xo), ld_u32(sXl + xo + 8));
        }
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          const int rr = m0 + gid + 8 * (h >> 1), c = n0 + 2 * tig + (h & 1);
          if (rr >= nrow || c >= mcols) continue;
          const int ap = sAp[rr];
          const int64_t d = sD[rr];
          const float* arow = sA + rr * AS;
          const float* vs = V + (int64_t)c * ldv + (int64_t)ap * no;
          float sa = 0.f;
          // padded A entries are zero; (ap, kk >= no) stays inside the V column
#pragma unroll 8
          for (int kk = 0; kk < noP; ++kk) sa += arow[kk] * vs[kk];
          W[(int64_t)c * ldw + n1 + d] = diag[n1 + d] * sV2f[rr * MT + c] + (sa + acc[h]);
        }
      } else {
        // W1^T += V2^T . C|D: n-tiles nt = (warp - 4) + 4 j over K/8
        const int w4 = warp - 4;
#pragma unroll
        for (int ks = 0; ks < RT; ks += 16) {
          uint32_t ah[4], al[4];
          ah[0] = ld_u32(sV2h + gid * RTP + ks + 2 * tig);
          ah[1] = ld_u32(sV2h + (gid + 8) * RTP + ks + 2 * tig);
          ah[2] = ld_u32(sV2h + gid * RTP + ks + 2 * tig + 8);
          ah[3] = ld_u32(sV2h + (gid + 8) * RTP + ks + 2 * tig + 8);
          al[0] = ld_u32(sV2l + gid * RTP + ks + 2 * tig);
          al[1] = ld_u32(sV2l + (gid + 8) * RTP + ks + 2 * tig);
          al[2] = ld_u32(sV2l + gid * RTP + ks + 2 * tig + 8);
          al[3] = ld_u32(sV2l + (gid + 8) * RTP + ks + 2 * tig + 8);
#pragma unroll
          for (int j = 0; j < NT1; ++j) {
            const int nt = w4 + 4 * j;
            if (nt < K / 8) {
              const int bo = (8 * nt + gid) * RTP + ks + 2 * tig;
              const uint32_t b0 = ld_u32(sCDt + bo), b1 = ld_u32(sCDt + bo + 8);
              mma16816(acc1[j], ah, b0, b1);
              mma16816(acc1[j], al, b0, b1);
            }
          }
        }
      }
      // W1 (A): runs of equal a' reduced, then added atomically
      for (int o = tid; o < noP * MT; o += 256) {
        const int kk = o % noP, c = o / noP;
        if (kk >= no || c >= mcols) continue;
        float sacc = 0.f;
        int prev = sAp[0];
        for (int rr = 0; rr < nrow; ++rr) {
          const int ap = sAp[rr];
          if (ap != prev) {
            if (sacc != 0.f) atomicAdd(&W1[(int64_t)c * ld1 + (int64_t)prev * no + kk], (TA)sacc);
            sacc = 0.f;
            prev = ap;
          }
          sacc += sA[rr * AS + kk] * sV2f[rr * MT + c];
        }
        if (sacc != 0.f) atomicAdd(&W1[(int64_t)c * ld1 + (int64_t)prev * no + kk], (TA)sacc);
      }
      // sCDt, sA and the V2 arrays are rebuilt after the next barrier
      __syncthreads();
    }
    // the item's W1 (C|D) sums: accumulator (c = gid + 8 (h >> 1), k = 8 nt + 2 tig + (h & 1))
    if (warp >= 4) {
      const int w4 = warp - 4;
#pragma unroll
      for (int j = 0; j < NT1; ++j) {
        const int nt = w4 + 4 * j;
        if (nt >= K / 8) continue;
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          const int c = gid + 8 * (h >> 1), k = 8 * nt + 2 * tig + (h & 1);
          const int seg = k / nvP, a = k - seg * nvP;
          const float v = acc1[j][h];
          if (c < mcols && a < nv && v != 0.f)
            atomicAdd(&W1[(int64_t)c * ld1 + (int64_t)a * no + (seg ? lp : kp)], (TA)v);
        }
      }
    }
  }
  cp_async_wait<0>();
}

// W1 = diag1 . V1 + A V1 (A symmetric n1 x n1, row-major == column-major).
template <typename T>
__global__ void __launch_bounds__(256) k_singles(int n1, const T* __restrict__ A, const T* __restrict__ diag,
                                                 const T* __restrict__ V, int64_t ldv, T* __restrict__ W,
                                                 int64_t ldw, int m) {
  // tile: 64 rows x 4 columns per block; each thread one (row, col) pair
  // reading A row-wise through L1 (A^T = A).
  __shared__ T sV[64][4];
  const int r = blockIdx.x * 64 + (threadIdx.x & 63);
  const int c = blockIdx.y * 4 + (threadIdx.x >> 6);
  T acc = T(0);
  for (int k0 = 0; k0 < n1; k0 += 64) {
    __syncthreads();
    {
      int kk = threadIdx.x & 63, cc = threadIdx.x >> 6;
      int k = k0 + kk, col = blockIdx.y * 4 + cc;
      sV[kk][cc] = (k < n1 && col < m) ? V[(int64_t)col * ldv + k] : T(0);
    }
    __syncthreads();
    if (r < n1) {
      const int kl = min(64, n1 - k0);
      const T* Ar = A + (int64_t)r * n1 + k0;   // row r of A == column r
      for (int kk = 0; kk < kl; ++kk) acc += Ar[kk] * sV[kk][threadIdx.x >> 6];
    }
  }
  if (r < n1 && c < m) W[(int64_t)c * ldw + r] = diag[r] * V[(int64_t)c * ldv + r] + acc;
}

// W1 = diag1 . V1 + A V1 as a register-tiled GEMM: block tile 32 rows x 32
// columns, K staged 32 at a time, 128 threads with 4 x 2 outputs each.
// Used by the sigma product and by the folded preconditioner's MINRES.
template <typename T>
__global__ void __launch_bounds__(128) k_singles_gemm(int n1, const T* __restrict__ A, const T* __restrict__ diag,
                                                      const T* __restrict__ V, int64_t ldv, T* __restrict__ W,
                                                      int64_t ldw, int m, T* __restrict__ part = nullptr,
                                                      int kchunk = 0) {
  __shared__ __align__(16) T sA[32][36];   // sA[k][r]
  __shared__ T sV[32][33];                 // sV[k][c]
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;   // columns 2tx, 2tx+1; rows 4ty..4ty+3
  const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  T acc[4][2];
#pragma unroll
  for (int i = 0; i < 4; ++i) { acc[i][0] = T(0); acc[i][1] = T(0); }
  // split K (part != null): this block sums k in [kbeg, kend) into part
  const int kbeg = part ? blockIdx.z * kchunk : 0;
  const int kend = part ? min(n1, kbeg + kchunk) : n1;
  for (int k0 = kbeg; k0 < kend; k0 += 32) {
    __syncthreads();
#pragma unroll
    for (int l = tid; l < 32 * 32; l += 128) {
      const int kk = l & 31, rr = l >> 5;
      const int r = r0 + rr, k = k0 + kk;
      sA[kk][rr] = (r < n1 && k < kend) ? A[(int64_t)r * n1 + k] : T(0);
      const int c = c0 + rr;
      sV[kk][rr] = (c < m && k < kend) ? V[(int64_t)c * ldv + k] : T(0);
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < 32; ++kk) {
      T a[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = sA[kk][4 * ty + i];
      const T b0 = sV[kk][2 * tx], b1 = sV[kk][2 * tx + 1];
#pragma unroll
      for (int i = 0; i < 4; ++i) { acc[i][0] += a[i] * b0; acc[i][1] += a[i] * b1; }
    }
  }
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    const int c = c0 + 2 * tx + j;
    if (c >= m) continue;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int r = r0 + 4 * ty + i;
      if (r >= n1) continue;
      if (part) part[((int64_t)blockIdx.z * m + c) * n1 + r] = acc[i][j];
      else W[(int64_t)c * ldw + r] = diag[r] * V[(int64_t)c * ldv + r] + acc[i][j];
    }
  }
}

// W1 = diag V1 + the split-K partials, summed in a fixed order
template <typename T>
__global__ void k_singles_reduce(int n1, int m, int ks, const T* __restrict__ part, const T* __restrict__ diag,
                                 const T* __restrict__ V, int64_t ldv, T* __restrict__ W, int64_t ldw) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (int64_t)n1 * m;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(i / n1), r = (int)(i - (int64_t)c * n1);
    T acc = diag[r] * V[(int64_t)c * ldv + r];
    for (int z = 0; z < ks; ++z) acc += part[((int64_t)z * m + c) * n1 + r];
    W[(int64_t)c * ldw + r] = acc;
  }
}

template <typename T>
void launch_singles(Ctx* c, int m, const T* A, const T* diag, const T* V, int64_t ldv, T* W, int64_t ldw) {
  const int n1 = (int)c->geom.n1;
  dim3 grid((n1 + 31) / 32, (m + 31) / 32);
  k_singles_gemm<T><<<grid, 128, 0, c->stream>>>(n1, A, diag, V, ldv, W, ldw, m); ADC_COUNT_LAUNCH();
}

// FP32 singles block with K split over about four blocks per SM: the
// unsplit grid has only (n1/32) x (m/32) blocks, each walking all n1 values
// of k, which leaves the product latency-bound.  The partials go to the
// plan's scratch and are summed in a fixed order.
int launch_singles_split(Ctx* c, int m, const float* A, const float* diag, const float* V, int64_t ldv, float* W,
                         int64_t ldw) {
  const int n1 = (int)c->geom.n1;
  const int base = ((n1 + 31) / 32) * ((m + 31) / 32);
  const int ks = std::max(1, std::min(16, (4 * c->nsm + base - 1) / base));
  SigmaPlan* plan = reinterpret_cast<SigmaPlan*>(c->sigma_plan);
  if (ks == 1 || !plan) {
    launch_singles<float>(c, m, A, diag, V, ldv, W, ldw);
    return ADCGPU_OK;
  }
  const int kchunk = ((n1 + ks - 1) / ks + 31) / 32 * 32;
  const int ksu = (n1 + kchunk - 1) / kchunk;
  const size_t need = sizeof(float) * (size_t)ksu * m * n1;
  if (plan->sk_bytes < need) {
    dfree(c, plan->d_sk);
    plan->d_sk = nullptr;
    plan->sk_bytes = 0;
    ST(dmalloc(c, &plan->d_sk, need));
    plan->sk_bytes = need;
  }
  float* part = reinterpret_cast<float*>(plan->d_sk);
  dim3 grid((n1 + 31) / 32, (m + 31) / 32, ksu);
  k_singles_gemm<float><<<grid, 128, 0, c->stream>>>(n1, A, diag, V, ldv, W, ldw, m, part, kchunk);
  ADC_COUNT_LAUNCH();
  k_singles_reduce<float><<<std::min((n1 * m + 255) / 256, c->nsm * 8), 256, 0, c->stream>>>(n1, m, ksu, part, diag,
                                                                                          V, ldv, W, ldw);
  ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  return ADCGPU_OK;
}

// Close the statistics window of the previous sigma call (its stop event
// has completed by the time the next call or a read of the stats happens).
void sigma_stats_flush(Ctx* c) {
  if (!c->st_pending) return;
  cudaEventSynchronize(c->st_ev1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, c->st_ev0, c->st_ev1);
  c->st_ms += ms;
  c->st_bytes += c->st_pending_bytes;
  c->st_cols += c->st_pending_cols;
  c->st_calls += 1;
  double* by = c->st_by[c->st_pending_kind];
  by[0] += 1.0; by[1] += ms; by[2] += c->st_pending_bytes; by[3] += c->st_pending_cols;
  c->st_pending = false;
}

// W1 += accumulated coupling part (FP64 accumulator of the FP32 path)
__global__ void k_w1_finalize(int n1, int m, const double* __restrict__ acc, float* __restrict__ W, int64_t ldw) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n1 * m; i += gridDim.x * blockDim.x) {
    const int c = i / n1, s = i - c * n1;
    W[(int64_t)c * ldw + s] += (float)acc[i];
  }
}

template <typename T, typename TV, typename TA, int MT>
int launch_tile(Ctx* c, const GeomDev& g, const SigmaPlan* plan, const TV* Bt, const T* diag, const T* V,
                int64_t ldv, int ncols, T* W, int64_t ldw, TA* W1, int64_t ld1, size_t smem) {
  // FP64 inputs in the mixed ladder's refinement: double-float arithmetic
  auto kern = (sizeof(T) == 8 && c->dense_df) ? k_sigma_tile<T, TV, TA, MT, DfArithFor<T>>
                                              : k_sigma_tile<T, TV, TA, MT, NativeArith<T>>;
  // the cap is a property of the kernel, shared by every context and host
  // thread: set it to the device's opt-in maximum, never to this call's size
  ADC_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_optin_max(c)));
  ADC_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  const int grid = std::min(plan->ntitems, c->nsm * 2);
  kern<<<grid, 256, smem, c->stream>>>(g, plan->d_titems, plan->ntitems, Bt, diag, V, ldv, ncols, W, ldw, W1,
                                       ld1); ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  return ADCGPU_OK;
}

template <typename TA>
int launch_tile_mma(Ctx* c, const GeomDev& g, const SigmaPlan* plan, const __nv_bfloat16* Bt, const float* diag,
                    const float* V, int64_t ldv, int ncols, float* W, int64_t ldw, TA* W1, int64_t ld1) {
  const size_t smem = tile_mma_smem_bytes(g.nvP, g.noP);
  auto kern = k_sigma_tile_mma<TA>;
  ADC_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_optin_max(c)));
  ADC_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  const int grid = std::min(plan->ntitems, c->nsm * 2);
  kern<<<grid, 256, smem, c->stream>>>(g, plan->d_titems, plan->ntitems, Bt, diag, V, ldv, ncols, W, ldw, W1,
                                       ld1); ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  return ADCGPU_OK;
}

// pass 2 (segment B) for mc <= 4 columns (8 with FP32 vectors)
template <typename T, typename TV, typename TA>
int launch_p2(Ctx* c, const GeomDev& g, const SigmaPlan* plan, int mc, const TV* Bt, const T* V, int64_t ldv,
              T* W, int64_t ldw, TA* W1, int64_t ld1) {
  const int g2 = std::min(plan->nitems, c->nsm * 8 * 8) / 8 + 1;
  const int gs = g.noP <= 8 ? 1 : (g.noP <= 16 ? 2 : 4);
  cudaStream_t s = c->stream;
#define P2(MC, GS) \
  k_sigma_p2<T, TV, TA, MC, GS><<<g2, 256, 0, s>>>(g, plan->d_items, plan->nitems, Bt, V, ldv, W, ldw, W1, ld1)
  if constexpr (sizeof(T) == 4) {
    if (mc == 8) {
      if (gs == 1) P2(8, 1); else if (gs == 2) P2(8, 2); else P2(8, 4);
      ADC_COUNT_LAUNCH();
      ADC_CUDA(c, cudaGetLastError());
      return ADCGPU_OK;
    }
  }
  if (mc == 4) { if (gs == 1) P2(4, 1); else if (gs == 2) P2(4, 2); else P2(4, 4); }
  else if (mc == 2) { if (gs == 1) P2(2, 1); else if (gs == 2) P2(2, 2); else P2(2, 4); }
  else { if (gs == 1) P2(1, 1); else if (gs == 2) P2(1, 2); else P2(1, 4); }
#undef P2
  ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  return ADCGPU_OK;
}

// pass 3 (segment A's W1 part, after the tensor-core pass) for mc <= 8 columns
template <typename TV>
int launch_p3(Ctx* c, const GeomDev& g, const int2* runs, int nruns, int mc, const TV* Bt, const float* V,
              int64_t ldv, double* W1, int64_t ld1) {
  const int g3 = std::min(nruns, c->nsm * 8 * 8) / 8 + 1;
  const int gs = g.noP <= 8 ? 1 : (g.noP <= 16 ? 2 : 4);
  cudaStream_t s = c->stream;
#define P3(MC, GS) k_sigma_p3<TV, MC, GS><<<g3, 256, 0, s>>>(g, runs, nruns, Bt, V, ldv, W1, ld1)
  if (mc == 8) { if (gs == 1) P3(8, 1); else if (gs == 2) P3(8, 2); else P3(8, 4); }
  else if (mc == 4) { if (gs == 1) P3(4, 1); else if (gs == 2) P3(4, 2); else P3(4, 4); }
  else if (mc == 2) { if (gs == 1) P3(2, 1); else if (gs == 2) P3(2, 2); else P3(2, 4); }
  else { if (gs == 1) P3(1, 1); else if (gs == 2) P3(1, 2); else P3(1, 4); }
#undef P3
  ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  return ADCGPU_OK;
}

template <typename T, typename TV>
int sigma_impl(Ctx* c, int m, const T* dV, int64_t ldv, T* dW, int64_t ldw, const T* A, const T* diag,
               const TV* Bt) {
  const Geometry& G = c->geom;
  const int n1 = (int)G.n1;
  cudaStream_t s = c->stream;
  if (!c->st_ev0) {
    ADC_CUDA(c, cudaEventCreate(&c->st_ev0));
    ADC_CUDA(c, cudaEventCreate(&c->st_ev1));
  }
  sigma_stats_flush(c);
  ADC_CUDA(c, cudaEventRecord(c->st_ev0, s));
  GeomDev g = to_dev(G);
  // singles block first (plain stores), then the coupling adds atomically
  if constexpr (sizeof(T) == 4) ST(launch_singles_split(c, m, A, diag, dV, ldv, dW, ldw));
  else launch_singles<T>(c, m, A, diag, dV, ldv, dW, ldw);
  ADC_CUDA(c, cudaGetLastError());
  SigmaPlan* plan = reinterpret_cast<SigmaPlan*>(c->sigma_plan);
  if (!plan) return set_err(c, ADCGPU_NO_MATRIX, "sigma plan missing");
  // FP64 path: coupling contributions to W1 go straight into W.  FP32 path:
  // into an FP64 n1 x m accumulator, added to W1 at the end (a singles row
  // sums ~ n2 n1 / N products; FP32 atomics there would floor the residual).
  typedef typename std::conditional<sizeof(T) == 8, T, double>::type TAcc;
  TAcc* W1base = nullptr;
  if (sizeof(T) == 4) {
    const size_t need = sizeof(double) * (size_t)n1 * m;
    if (plan->acc_bytes < need) {
      dfree(c, plan->d_acc);
      plan->d_acc = nullptr; plan->acc_bytes = 0;
      int st2 = dmalloc(c, (void**)&plan->d_acc, need);
      if (st2) return st2;
      plan->acc_bytes = need;
    }
    ADC_CUDA(c, cudaMemsetAsync(plan->d_acc, 0, need, s));
    W1base = reinterpret_cast<TAcc*>(plan->d_acc);
  }
  // The coupling part over the work lists of P (the whole store, or the
  // rows of one chunk of the direct path) with the values at BtP.
  bool umma_used = false;
  auto coupling = [&](const SigmaPlan* P, const TV* BtP, bool allow_umma) -> int {
    int c0 = 0;
    // tiled pass 1 (k_sigma_tile) when its shared memory fits: widest column
    // group first; segment B still runs through pass 2 in groups of <= 4
    // FP32: 16 columns keep two blocks per SM (their loads overlap the other's
    // arithmetic); FP64 is bound by the FP64 pipe at one block per SM
    constexpr int MTMAX = 16;
    const size_t smax = (size_t)smem_optin_max(c);
    int mt_fit = 0;
    for (int mt = MTMAX; mt >= 8 && !mt_fit; mt /= 2)
      if (tile_smem_bytes(G.nvP, G.noP, mt, sizeof(T), sizeof(T)) <= smax) mt_fit = mt;
    // a column tile always computes MT columns: below 16 columns the per-warp
    // pass 1 is faster
    const bool tiled = P->tiled && P->d_titems && mt_fit > 0 && m >= 16;
    if constexpr (std::is_same<TV, __nv_bfloat16>::value) {
      // tensor-core pass (tcgen05, sigma_umma.cu) for the C|D segments and the
      // W2 part of segment A, then segment B (pass 2) and the W1 part of
      // segment A (pass 3), up to 48 columns per matrix pass
      if (allow_umma && P->tiled == 1 && !P->umma_off && umma_supported(c)) {
        ST(umma_prepare(c, plan->umma, plan->umma_item_rows));
        const int2* runs = nullptr;
        int nruns = 0;
        ST(umma_runs(plan->umma, &runs, &nruns));
        const bool ab = !P->ab_off && ab_supported(c);
        for (; c0 < m;) {
          const int nc = std::min(m - c0, 48);
          const T* V = dV + (int64_t)c0 * ldv;
          T* W = dW + (int64_t)c0 * ldw;
          TAcc* W1 = W1base + (int64_t)c0 * n1;
          ST(umma_launch(c, plan->umma, V, ldv, nc, W, ldw, W1, n1, ab ? 0 : 1));
          if (ab) {
            // segments A and B in compact form, W2 rows updated in place
            ST(ab_launch<TV>(c, plan->ab, BtP, true, V, ldv, nc, W, ldw, W1, n1));
            c0 += nc;
            continue;
          }
          for (int b0 = 0; P->nitems && b0 < nc;) {
            const int lb = nc - b0, mc = lb >= 8 ? 8 : (lb >= 4 ? 4 : (lb >= 2 ? 2 : 1));
            ST((launch_p2<T, TV, TAcc>(c, g, P, mc, BtP, V + (int64_t)b0 * ldv, ldv, W + (int64_t)b0 * ldw, ldw,
                                       W1 + (int64_t)b0 * n1, n1)));
            b0 += mc;
          }
          for (int b0 = 0; b0 < nc;) {
            const int lb = nc - b0, mc = lb >= 8 ? 8 : (lb >= 4 ? 4 : (lb >= 2 ? 2 : 1));
            ST((launch_p3<TV>(c, g, runs, nruns, mc, BtP, V + (int64_t)b0 * ldv, ldv, W1 + (int64_t)b0 * n1, n1)));
            b0 += mc;
          }
          c0 += nc;
        }
        umma_used = true;
      }
    }
    if constexpr (std::is_same<T, float>::value && std::is_same<TV, float>::value) {
      // FP32 values on the tensor cores: the values and vectors as three BF16
      // slices each (sigma_umma.cu), segments A/B in compact form from the
      // FP32 store, up to 32 columns per matrix pass
      if (allow_umma && P->umma3_on && P->tiled == 1 && !P->umma_off && !P->ab_off && !c->direct &&
          umma3_supported(c) && ab_supported(c)) {
        ST(umma_prepare(c, plan->umma, plan->umma_item_rows));
        for (; c0 < m;) {
          const int nc = std::min(m - c0, 32);
          const T* V = dV + (int64_t)c0 * ldv;
          T* W = dW + (int64_t)c0 * ldw;
          TAcc* W1 = W1base + (int64_t)c0 * n1;
          ST(umma3_launch(c, plan->umma, V, ldv, nc, W, ldw, W1, n1));
          ST(ab_launch<TV>(c, plan->ab, BtP, true, V, ldv, nc, W, ldw, W1, n1));
          c0 += nc;
        }
        umma_used = true;
      }
    }
    while (tiled && c0 < m) {
      const int left = m - c0;
      const int mt = left > 8 && mt_fit >= 16 ? 16 : 8;
      const int ncols = std::min(left, mt);
      const T* V = dV + (int64_t)c0 * ldv;
      T* W = dW + (int64_t)c0 * ldw;
      TAcc* W1 = sizeof(T) == 8 ? reinterpret_cast<TAcc*>(W) : W1base + (int64_t)c0 * n1;
      const int64_t ld1 = sizeof(T) == 8 ? ldw : (int64_t)n1;
      const size_t smem = tile_smem_bytes(G.nvP, G.noP, mt, sizeof(T), sizeof(T));
      if constexpr (std::is_same<TV, __nv_bfloat16>::value) {
        if (P->tiled == 1 && tile_mma_smem_bytes(G.nvP, G.noP) <= smax) {
          // tensor-core tile: 16 columns per pass
          const int nc = std::min(left, MMA_MT);
          ST((launch_tile_mma<TAcc>(c, g, P, BtP, diag, V, ldv, nc, W, ldw, W1, ld1)));
          for (int b0 = 0; P->nitems && b0 < nc;) {
            const int lb = nc - b0, mc = lb >= 8 ? 8 : (lb >= 4 ? 4 : (lb >= 2 ? 2 : 1));
            ST((launch_p2<T, TV, TAcc>(c, g, P, mc, BtP, V + (int64_t)b0 * ldv, ldv, W + (int64_t)b0 * ldw, ldw,
                                       W1 + (int64_t)b0 * ld1, ld1)));
            b0 += mc;
          }
          c0 += nc;
          continue;
        }
      }
      if (mt == 16) ST((launch_tile<T, TV, TAcc, 16>(c, g, P, BtP, diag, V, ldv, ncols, W, ldw, W1, ld1, smem)));
      else ST((launch_tile<T, TV, TAcc, 8>(c, g, P, BtP, diag, V, ldv, ncols, W, ldw, W1, ld1, smem)));
      ADC_CUDA(c, cudaGetLastError());
      if constexpr (std::is_same<T, float>::value && std::is_same<TV, float>::value) {
        if (!P->ab_off && !c->direct && ab_supported(c)) {
          // segment B (the tile did segment A) in compact form
          ST(ab_launch<TV>(c, plan->ab, BtP, false, V, ldv, ncols, W, ldw, W1, ld1));
          c0 += ncols;
          continue;
        }
      }
      // segment B: pass 2 over the same columns
      int b0 = 0;
      while (P->nitems && b0 < ncols) {
        const int lb = ncols - b0;
        const int mc = (sizeof(T) == 4 && lb >= 8) ? 8 : (lb >= 4 ? 4 : (lb >= 2 ? 2 : 1));
        const T* Vb = V + (int64_t)b0 * ldv;
        T* Wb = W + (int64_t)b0 * ldw;
        TAcc* W1b = W1 + (int64_t)b0 * ld1;
        ST((launch_p2<T, TV, TAcc>(c, g, P, mc, BtP, Vb, ldv, Wb, ldw, W1b, ld1)));
        ADC_CUDA(c, cudaGetLastError());
        b0 += mc;
      }
      c0 += ncols;
    }
    while (c0 < m) {
      const int left = m - c0;
      const T* V = dV + (int64_t)c0 * ldv;
      T* W = dW + (int64_t)c0 * ldw;
      TAcc* W1 = sizeof(T) == 8 ? reinterpret_cast<TAcc*>(W) : W1base + (int64_t)c0 * n1;
      const int64_t ld1 = sizeof(T) == 8 ? ldw : (int64_t)n1;
      int cap = P->mc_cap[sizeof(T) == 8 ? 0 : 1];
      if (sizeof(T) == 8) cap = std::min(cap, 2);
      const int mc = (left >= 4 && cap >= 4) ? 4 : ((left >= 2 && cap >= 2) ? 2 : 1);
      const int g1 = std::min(P->nchunks, c->nsm * 4 * 16) / 4 + 1;   // 4 warps per block
      const int g2 = std::min(P->nitems, c->nsm * 8 * 8) / 8 + 1;
  #define LAUNCH_P2(MC, GS) \
    k_sigma_p2<T, TV, TAcc, MC, GS><<<g2, 256, 0, s>>>(g, P->d_items, P->nitems, BtP, V, ldv, W, ldw, W1, ld1); ADC_COUNT_LAUNCH();
  #define LAUNCH(MC)                                                                                              \
    if (P->staged) {                                                                                           \
      constexpr int NS = sizeof(TV) == 2 ? 8 : 4;                                                                 \
      const size_t smem = (size_t)4 * NS * (32 * 16 * sizeof(TV) + 16 * MC);                                    \
      auto kern = k_sigma_p1s<T, TV, TAcc, MC, NS>;                                                               \
      ADC_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));            \
      kern<<<g1, 128, smem, s>>>(g, P->d_chunks, P->nchunks, BtP, diag, V, ldv, W, ldw, W1, ld1); ADC_COUNT_LAUNCH();                   \
    } else {                                                                                                      \
      k_sigma_p1<T, TV, TAcc, MC><<<g1, 128, 0, s>>>(g, P->d_chunks, P->nchunks, BtP, diag, V, ldv, W, ldw, W1, ld1); ADC_COUNT_LAUNCH(); \
    }                                                                                                             \
    if (P->nitems) {                                                                                           \
      if (G.noP <= 8) { LAUNCH_P2(MC, 1) } else if (G.noP <= 16) { LAUNCH_P2(MC, 2) } else { LAUNCH_P2(MC, 4) }   \
    }
      if (mc == 4) { LAUNCH(4) } else if (mc == 2) { LAUNCH(2) } else { LAUNCH(1) }
  #undef LAUNCH
  #undef LAUNCH_P2
      ADC_CUDA(c, cudaGetLastError());
      c0 += mc;
    }
    return ADCGPU_OK;
  };
  if (c->direct) {
    // direct (matrix-free) path: the coupling values are recomputed for each
    // chunk of whole slabs into the chunk buffer and used at once
    if constexpr (std::is_same<TV, double>::value) {
      for (const DirectChunk& dc : plan->dchunks) {
        ST(coupling_values(c, c->d_Bt, dc.vbase, dc.row0, dc.row1, nullptr));
        SigmaPlan view = *plan;
        view.d_titems = plan->d_titems + dc.ti0; view.ntitems = dc.ti1 - dc.ti0;
        view.d_chunks = plan->d_chunks + dc.ch0; view.nchunks = dc.ch1 - dc.ch0;
        view.d_items = plan->d_items + dc.it0; view.nitems = dc.it1 - dc.it0;
        // the kernels address row r at Bt + off[cls] + (r - start[cls]) L;
        // shifting the base by the chunk's first value puts its rows in the buffer
        const TV* BtP = reinterpret_cast<const TV*>(reinterpret_cast<uintptr_t>(c->d_Bt) -
                                                    (uintptr_t)dc.vbase * sizeof(TV));
        ST(coupling(&view, BtP, false));
      }
    } else {
      return set_err(c, ADCGPU_UNSUPPORTED, "the direct path computes in FP64");
    }
  } else {
    ST(coupling(plan, Bt, true));
  }
  if (sizeof(T) == 4) {
    k_w1_finalize<<<(n1 * m + 255) / 256, 256, 0, s>>>(n1, m, reinterpret_cast<const double*>(W1base),
                                                       reinterpret_cast<float*>(dW), ldw); ADC_COUNT_LAUNCH();
  }
  ADC_CUDA(c, cudaEventRecord(c->st_ev1, s));
  if (umma_used) ST(umma_check(c, plan->umma));
  c->st_pending = true;
  c->st_pending_cols = m;
  c->st_pending_kind = std::is_same<TV, __nv_bfloat16>::value ? 0 : (std::is_same<TV, float>::value ? 1 : 2);
  // algorithmic bytes of one sparse product of m columns, counted as for a
  // CSR matrix: every kept coupling value once with a 4-byte column index,
  // the dense singles block as n1^2 values, n1+1 row pointers, the FP64
  // diagonal, V read and W written once.  The index-free layout here reads
  // no indices (and the zero padding of its segments instead).
  c->st_pending_bytes = (double)(c->nnz_kept - c->nnz_ph) * (sizeof(TV) + 4) + (double)G.n1 * G.n1 * sizeof(TV) +
                        4.0 * (double)(G.n1 + 1) + 8.0 * (double)G.N + 2.0 * (double)m * G.N * sizeof(T);
  return ADCGPU_OK;
}

__global__ void k_to_f32(const double* __restrict__ x, float* __restrict__ y, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = (float)x[i];
}
// mid and lo BF16 slices of the FP32 values: x32 = hi + mid + lo to ~2^-25
// relative, hi the BF16 store (x32 - hi is exact in FP32)
__global__ void k_bf16_slices(const float* __restrict__ x32, const __nv_bfloat16* __restrict__ hi,
                              __nv_bfloat16* __restrict__ mid, __nv_bfloat16* __restrict__ lo, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float r = x32[i] - __bfloat162float(hi[i]);
    const __nv_bfloat16 m = __float2bfloat16(r);
    mid[i] = m;
    lo[i] = __float2bfloat16(r - __bfloat162float(m));
  }
}

__global__ void k_to_bf16(const double* __restrict__ x, __nv_bfloat16* __restrict__ y, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = __double2bfloat16(x[i]);
}

}  // namespace

// Work lists of the sigma kernels: pass-1 chunks (row ranges of at most
// 'chunk' rows inside one slab) and pass-2 items (slab, b') of the classes
// with a' < b'.
int build_chunks(Ctx* c, int chunk) {
  const Geometry& G = c->geom;
  std::vector<int2> chunks, items, titems;
  // direct path: the work-list ranges of each chunk of slabs
  std::vector<DirectChunk> dch = c->direct ? c->dchunks : std::vector<DirectChunk>();
  size_t di = 0;
  for (int cls = 0; cls < 5; ++cls) {
    const int64_t r0 = G.start[cls], r1 = G.start[cls + 1], sl = G.slab_len(cls);
    for (int64_t s0 = r0; s0 < r1; s0 += sl) {
      if (di < dch.size() && s0 == dch[di].row0) {
        dch[di].ti0 = (int)titems.size(); dch[di].ch0 = (int)chunks.size(); dch[di].it0 = (int)items.size();
      }
      for (int64_t a = s0; a < s0 + sl; a += chunk)
        chunks.push_back(make_int2((int)a, (int)std::min<int64_t>(a + chunk, s0 + sl)));
      // tiled pass 1: equal pieces of at most TILE_ITEM_ROWS rows per slab
      const int64_t npc = (sl + TILE_ITEM_ROWS - 1) / TILE_ITEM_ROWS, per = (sl + npc - 1) / npc;
      for (int64_t a = s0; a < s0 + sl; a += per)
        titems.push_back(make_int2((int)a, (int)std::min<int64_t>(a + per, s0 + sl)));
      if (cls == 1 || cls >= 3)
        for (int bp = 1; bp < G.nv; ++bp) items.push_back(make_int2((int)s0, bp));
      if (di < dch.size() && s0 + sl == dch[di].row1) {
        dch[di].ti1 = (int)titems.size(); dch[di].ch1 = (int)chunks.size(); dch[di].it1 = (int)items.size();
        ++di;
      }
    }
  }
  SigmaPlan* plan = reinterpret_cast<SigmaPlan*>(c->sigma_plan);
  if (!plan) { plan = new SigmaPlan; c->sigma_plan = plan; }
  dfree(c, plan->d_chunks);
  dfree(c, plan->d_items);
  dfree(c, plan->d_titems);
  plan->d_chunks = plan->d_items = plan->d_titems = nullptr;
  int st;
  if ((st = dmalloc(c, (void**)&plan->d_titems, sizeof(int2) * titems.size()))) return st;
  ADC_CUDA(c, h2d(c, plan->d_titems, titems.data(), sizeof(int2) * titems.size()));
  plan->ntitems = (int)titems.size();
  if ((st = dmalloc(c, (void**)&plan->d_chunks, sizeof(int2) * chunks.size()))) return st;
  if ((st = dmalloc(c, (void**)&plan->d_items, sizeof(int2) * std::max<size_t>(items.size(), 1)))) return st;
  ADC_CUDA(c, h2d(c, plan->d_chunks, chunks.data(), sizeof(int2) * chunks.size()));
  if (!items.empty())
    ADC_CUDA(c, h2d(c, plan->d_items, items.data(), sizeof(int2) * items.size()));
  plan->nchunks = (int)chunks.size();
  plan->nitems = (int)items.size();
  plan->chunk = chunk;
  plan->dchunks = dch;
  return ADCGPU_OK;
}

int prepare_desc(Ctx* c) {
  SigmaPlan* plan = reinterpret_cast<SigmaPlan*>(c->sigma_plan);
  return build_chunks(c, plan ? plan->chunk : 64);
}

void free_sigma_plan(Ctx* c) {
  SigmaPlan* plan = reinterpret_cast<SigmaPlan*>(c->sigma_plan);
  if (!plan) return;
  dfree(c, plan->d_chunks);
  dfree(c, plan->d_items);
  dfree(c, plan->d_titems);
  dfree(c, plan->d_acc);
  dfree(c, plan->d_sk);
  umma_free(c, plan->umma);
  ab_free(c, plan->ab);
  delete plan;
  c->sigma_plan = nullptr;
}

int prepare_mixed(Ctx* c) {
  const Geometry& G = c->geom;
  int st;
  if (!c->d_A32 && (st = dmalloc(c, (void**)&c->d_A32, sizeof(float) * G.n1 * G.n1))) return st;
  if (!c->d_diag32 && (st = dmalloc(c, (void**)&c->d_diag32, sizeof(float) * G.N))) return st;
  if (!c->d_Bt16 && (st = dmalloc(c, (void**)&c->d_Bt16, sizeof(uint16_t) * G.off[5]))) return st;
  if (!c->d_Bt32 && (st = dmalloc(c, (void**)&c->d_Bt32, sizeof(float) * G.off[5]))) return st;
  k_to_f32<<<c->nsm * 8, 256, 0, c->stream>>>(c->d_A, c->d_A32, G.n1 * G.n1); ADC_COUNT_LAUNCH();
  k_to_f32<<<c->nsm * 8, 256, 0, c->stream>>>(c->d_diag, c->d_diag32, G.N); ADC_COUNT_LAUNCH();
  k_to_bf16<<<c->nsm * 8, 256, 0, c->stream>>>(c->d_Bt, (__nv_bfloat16*)c->d_Bt16, G.off[5]); ADC_COUNT_LAUNCH();
  k_to_f32<<<c->nsm * 8, 256, 0, c->stream>>>(c->d_Bt, c->d_Bt32, G.off[5]); ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  // the FP32 values as three BF16 slices for the tcgen05 FP32-value pass
  // (shapes the tensor-core pass takes only)
  if (umma_geometry_ok(G)) {
    for (int t = 0; t < 2; ++t)
      if (!c->d_Bt16s[t] && (st = dmalloc(c, (void**)&c->d_Bt16s[t], sizeof(uint16_t) * G.off[5]))) return st;
    k_bf16_slices<<<c->nsm * 8, 256, 0, c->stream>>>(c->d_Bt32, (const __nv_bfloat16*)c->d_Bt16,
                                                     (__nv_bfloat16*)c->d_Bt16s[0], (__nv_bfloat16*)c->d_Bt16s[1],
                                                     G.off[5]);
    ADC_COUNT_LAUNCH();
    ADC_CUDA(c, cudaGetLastError());
  }
  // the value stores were rewritten: the compact segment-A/B tables follow
  if (SigmaPlan* plan = reinterpret_cast<SigmaPlan*>(c->sigma_plan)) ab_invalidate(plan->ab);
  return ADCGPU_OK;
}

extern "C" int adcgpu_sigma_stats_by_store(adcgpu_ctx* h, double* out, int reset) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c || !out) return ADCGPU_BAD_INPUT;
  cudaSetDevice(c->device);
  sigma_stats_flush(c);
  for (int k = 0; k < 3; ++k)
    for (int j = 0; j < 4; ++j) out[4 * k + j] = c->st_by[k][j];
  if (reset)
    for (auto& b : c->st_by) for (double& x : b) x = 0.0;
  return ADCGPU_OK;
}

extern "C" int adcgpu_sigma_stats(adcgpu_ctx* h, double* out, int reset) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c || !out) return ADCGPU_BAD_INPUT;
  cudaSetDevice(c->device);
  sigma_stats_flush(c);
  out[0] = (double)c->st_calls; out[1] = c->st_ms; out[2] = c->st_bytes; out[3] = (double)c->st_cols;
  if (reset) {
    c->st_calls = 0; c->st_cols = 0; c->st_ms = 0.0; c->st_bytes = 0.0;
    for (auto& b : c->st_by) for (double& x : b) x = 0.0;
  }
  return ADCGPU_OK;
}

// Autotuner: times the sigma product for m columns over the launch shapes
// (pass-1 chunk rows x columns per pass) with CUDA events on the context's
// stream and keeps the fastest.  Results are cached by the caller.
extern "C" int adcgpu_sigma_autotune(adcgpu_ctx* h, int m, int* best_chunk, int* best_mc, double* best_ms) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c || m <= 0) return ADCGPU_BAD_INPUT;
  cudaSetDevice(c->device);
  if (!c->have_matrix) return set_err(c, ADCGPU_NO_MATRIX, "build the matrix first");
  SigmaPlan* plan = reinterpret_cast<SigmaPlan*>(c->sigma_plan);
  const int64_t N = c->geom.N;
  const bool mixed = c->precision == ADCGPU_MIXED;
  const size_t esz = mixed ? sizeof(float) : sizeof(double);
  void *dv = nullptr, *dw = nullptr;
  int st;
  if ((st = dmalloc(c, &dv, esz * N * m))) return st;
  if ((st = dmalloc(c, &dw, esz * N * m))) { dfree(c, dv, 0); return st; }
  ADC_CUDA(c, cudaMemsetAsync(dv, 0, esz * N * m, c->stream));
  const int chunks[] = {16, 64, 256};
  const int mcs[] = {1, 2, 4};
  double best = 1e30;
  int bc = plan->chunk, bm = plan->mc_cap[mixed ? 1 : 0], bs = plan->staged, bt = plan->tiled;
  auto time_once = [&]() {
    double t = 1e30;
    for (int rep = 0; rep < 3; ++rep) {
      cudaEventRecord(c->ev0, c->stream);
      st = mixed ? sigma_fp32(c, m, (const float*)dv, N, (float*)dw, N)
                 : sigma_fp64(c, m, (const double*)dv, N, (double*)dw, N);
      cudaEventRecord(c->ev1, c->stream);
      cudaEventSynchronize(c->ev1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, c->ev0, c->ev1);
      if (rep > 0) t = std::min(t, (double)ms);
    }
    return t;
  };
  // the tiled pass 1 (one candidate), then the per-warp shapes
  plan->tiled = 1;
  {
    const double t = time_once();
    if (t < best) { best = t; bt = 1; }
  }
  plan->tiled = 0;
  for (int ch : chunks) {
    if (st || (st = build_chunks(c, ch))) break;
    for (int stg = 0; stg < 2; ++stg)
    for (int mc : mcs) {
      if (!mixed && mc > 2) continue;
      plan->mc_cap[mixed ? 1 : 0] = mc;
      plan->staged = stg;
      const double t = time_once();
      if (t < best) { best = t; bc = ch; bm = mc; bs = stg; bt = 0; }
    }
  }
  sigma_stats_flush(c);
  c->st_calls = 0; c->st_cols = 0; c->st_ms = 0.0; c->st_bytes = 0.0;
  for (auto& b : c->st_by) for (double& x : b) x = 0.0;
  plan->mc_cap[mixed ? 1 : 0] = bm;
  plan->staged = bs;
  plan->tiled = bt;
  if (!st) st = build_chunks(c, bc);
  dfree(c, dv, 0);
  dfree(c, dw, 0);
  if (best_chunk) *best_chunk = bc;
  // bit 3: staged pass-1 variant; bit 4: per-warp pass 1 instead of the tiled one
  if (best_mc) *best_mc = bm + 8 * bs + 16 * (bt ? 0 : 1);
  if (best_ms) *best_ms = best;
  return st;
}

// Applies a cached tuning result.
extern "C" int adcgpu_sigma_set_shape(adcgpu_ctx* h, int chunk, int mc_fp64, int mc_fp32) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c || chunk < 1 || mc_fp64 < 1 || mc_fp32 < 1) return ADCGPU_BAD_INPUT;
  cudaSetDevice(c->device);
  if (!c->have_matrix) return set_err(c, ADCGPU_NO_MATRIX, "build the matrix first");
  SigmaPlan* plan = reinterpret_cast<SigmaPlan*>(c->sigma_plan);
  plan->staged = ((mc_fp64 | mc_fp32) & 8) ? 1 : 0;
  plan->tiled = ((mc_fp64 | mc_fp32) & 16) ? 0 : (((mc_fp64 | mc_fp32) & 32) ? 2 : 1);
  plan->umma_off = ((mc_fp64 | mc_fp32) & 64) ? 1 : 0;
  // 128: segments A/B through pass 2 and pass 3 instead of the compact kernels
  plan->ab_off = ((mc_fp64 | mc_fp32) & 128) ? 1 : 0;
  // 256: a mixed-precision matrix's sigma product reads the FP32 value store
  // (the Davidson ladder's FP32 phase) instead of the BF16 one
  c->mixed_bf16 = ((mc_fp64 | mc_fp32) & 256) ? 0 : 1;
  // 512: the FP32 Gram products (V^T W) on the CUDA cores instead of the
  // tensor cores
  gram_set_off(c, ((mc_fp64 | mc_fp32) & 512) ? 1 : 0);
  // 1024: FP32 values on the two tcgen05 passes over their BF16 slices
  // instead of the CUDA-core tile.  As accurate as the tile and 3x faster
  // per call, but off by default: with it as the FP32 phase's product the
  // folded-preconditioner solve of one seeded system (nocc=12, nvirt=120,
  // 20 roots) converged to a wrong root set
  plan->umma3_on = ((mc_fp64 | mc_fp32) & 1024) ? 1 : 0;
  plan->mc_cap[0] = std::min(mc_fp64 & 7, 2);
  plan->mc_cap[1] = std::min(mc_fp32 & 7, 4);
  return build_chunks(c, chunk);
}

int sigma_fp64(Ctx* c, int m, const double* dV, int64_t ldv, double* dW, int64_t ldw) {
  if (c->cvs) return sigma_cvs(c, m, dV, ldv, dW, ldw);
  return sigma_impl<double, double>(c, m, dV, ldv, dW, ldw, c->d_A, c->d_diag, c->d_Bt);
}

// W = Hss V for the dense singles block alone (diag1 + A), m columns of n1
// rows: the inner product of the folded preconditioner's MINRES solve.
int singles_block_product(Ctx* c, int m, const double* V, int64_t ldv, double* W, int64_t ldw) {
  launch_singles<double>(c, m, c->d_A, c->d_diag, V, ldv, W, ldw);
  ADC_CUDA(c, cudaGetLastError());
  return ADCGPU_OK;
}
int singles_block_product(Ctx* c, int m, const float* V, int64_t ldv, float* W, int64_t ldw) {
  if (!c->d_A32 || !c->d_diag32) return set_err(c, ADCGPU_NO_MATRIX, "FP32 singles block missing");
  ST(launch_singles_split(c, m, c->d_A32, c->d_diag32, V, ldv, W, ldw));
  ADC_CUDA(c, cudaGetLastError());
  return ADCGPU_OK;
}

int sigma_fp32(Ctx* c, int m, const float* dV, int64_t ldv, float* dW, int64_t ldw) {
  if (c->cvs) return set_err(c, ADCGPU_UNSUPPORTED, "the CVS matrix is held in FP64 only");
  if (c->mixed_bf16)
    return sigma_impl<float, __nv_bfloat16>(c, m, dV, ldv, dW, ldw, c->d_A32, c->d_diag32,
                                            (const __nv_bfloat16*)c->d_Bt16);
  return sigma_impl<float, float>(c, m, dV, ldv, dW, ldw, c->d_A32, c->d_diag32, c->d_Bt32);
}

}  // namespace adcgpu

// ---------------------------------------------------------------------------
// Allocation-free sigma product.
//
// Some callers must not allocate device memory while they run: a host
// application that gives the library a device-memory budget up front and
// needs it not to grow in the middle of a solve (another library, or the
// host's own caching allocator, already owns the rest of the device), and a
// host thread that must not stall on the allocator (cudaFree waits for the
// whole device to go idle).  adcgpu_sigma_device grows a context-owned FP64
// accumulator on demand, so it may call cudaMalloc.  This variant uses a
// statically sized device array instead and calls no allocating routine.
// Its first call on a device does a one-time address lookup (below), so it
// should come before any stream capture.
//
// The array belongs to the library image: every device that loads the
// library holds it until the process exits, and all calls share it, so the
// product of one call must not overlap another call on the GPU (calls on
// one stream, or separated by synchronisation, are safe; concurrent calls
// race).  Its contents persist between calls; the part a call uses is zeroed
// at the start of that call.
// ---------------------------------------------------------------------------
namespace adcgpu {

constexpr size_t NOALLOC_ACC_DOUBLES = size_t(1) << 20;   // 8 MiB: n1 * m <= 1,048,576
static __device__ __align__(256) double g_noalloc_acc[NOALLOC_ACC_DOUBLES];

namespace {

// Device address of g_noalloc_acc, looked up once per device with that device
// current (the host-side symbol is only a stand-in, never a device address).
// std::call_once orders the lookup against every later reader, so host
// threads that make their first call on a device at the same time are safe.
constexpr int NOALLOC_MAX_DEVICES = 64;
double* noalloc_scratch(Ctx* c) {
  static std::once_flag once[NOALLOC_MAX_DEVICES];
  static double* ptrs[NOALLOC_MAX_DEVICES] = {nullptr};
  if (c->device < 0 || c->device >= NOALLOC_MAX_DEVICES) return nullptr;
  std::call_once(once[c->device], [c]() {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_acc) != cudaSuccess) {
      cudaGetLastError();
      return;
    }
    ptrs[c->device] = reinterpret_cast<double*>(p);
  });
  return ptrs[c->device];
}

template <typename TV>
int sigma_fp32_with_acc(Ctx* c, int m, const float* dV, int64_t ldv, float* dW, int64_t ldw, const TV* Bt,
                        double* acc) {
  typedef float T;
  typedef double TAcc;
  const Geometry& G = c->geom;
  const int n1 = (int)G.n1;
  cudaStream_t s = c->stream;
  GeomDev g = to_dev(G);
  const float* A = c->d_A32;
  const float* diag = c->d_diag32;
  dim3 gs((n1 + 63) / 64, (m + 3) / 4);
  k_singles<T><<<gs, 256, 0, s>>>(n1, A, diag, dV, ldv, dW, ldw, m); ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  SigmaPlan* plan = reinterpret_cast<SigmaPlan*>(c->sigma_plan);
  if (!plan) return set_err(c, ADCGPU_NO_MATRIX, "sigma plan missing");
  const int2* chunks = plan->d_chunks;
  const int2* items = plan->d_items;
  ADC_CUDA(c, cudaMemsetAsync(acc, 0, sizeof(double) * (size_t)n1 * m, s));
  int c0 = 0;
  while (c0 < m) {
    const int left = m - c0;
    const T* V = dV + (int64_t)c0 * ldv;
    T* W = dW + (int64_t)c0 * ldw;
    TAcc* W1 = acc + (int64_t)c0 * n1;
    const int64_t ld1 = (int64_t)n1;
    const int cap = plan->mc_cap[1];
    const int mc = (left >= 4 && cap >= 4) ? 4 : ((left >= 2 && cap >= 2) ? 2 : 1);
    const int g1 = std::min(plan->nchunks, c->nsm * 4 * 16) / 4 + 1;
    const int g2 = std::min(plan->nitems, c->nsm * 8 * 8) / 8 + 1;
#define NA_P2(MC, GS) \
  k_sigma_p2<T, TV, TAcc, MC, GS><<<g2, 256, 0, s>>>(g, items, plan->nitems, Bt, V, ldv, W, ldw, W1, ld1); ADC_COUNT_LAUNCH();
#define NA_LAUNCH(MC)                                                                                           \
  k_sigma_p1<T, TV, TAcc, MC><<<g1, 128, 0, s>>>(g, chunks, plan->nchunks, Bt, diag, V, ldv, W, ldw, W1, ld1); ADC_COUNT_LAUNCH(); \
  if (plan->nitems) {                                                                                           \
    if (G.noP <= 8) { NA_P2(MC, 1) } else if (G.noP <= 16) { NA_P2(MC, 2) } else { NA_P2(MC, 4) }             \
  }
    if (mc == 4) { NA_LAUNCH(4) } else if (mc == 2) { NA_LAUNCH(2) } else { NA_LAUNCH(1) }
#undef NA_LAUNCH
#undef NA_P2
    ADC_CUDA(c, cudaGetLastError());
    c0 += mc;
  }
  k_w1_finalize<<<(n1 * m + 255) / 256, 256, 0, s>>>(n1, m, acc, dW, ldw); ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  return ADCGPU_OK;
}

}  // namespace
}  // namespace adcgpu

extern "C" int adcgpu_sigma_device_noalloc(adcgpu_ctx* h, int m, const void* dv, void* dw, int64_t ld) {
  using namespace adcgpu;
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c) return ADCGPU_BAD_INPUT;
  if (cudaSetDevice(c->device) != cudaSuccess) { cudaGetLastError(); return ADCGPU_CUDA_ERROR; }
  if (!c->have_matrix) return set_err(c, ADCGPU_NO_MATRIX, "no matrix");
  if (c->precision != ADCGPU_MIXED)
    return set_err(c, ADCGPU_UNSUPPORTED, "sigma_device_noalloc needs a matrix built with ADCGPU_MIXED");
  if (m <= 0 || ld < c->geom.N || !dv || !dw) return set_err(c, ADCGPU_BAD_INPUT, "sigma arguments");
  if ((size_t)c->geom.n1 * (size_t)m > NOALLOC_ACC_DOUBLES)
    return set_err(c, ADCGPU_BAD_INPUT,
                   "sigma_device_noalloc: nocc*nvirt*m exceeds the 1,048,576-entry static scratch; "
                   "use fewer columns per call");
  double* acc = noalloc_scratch(c);
  if (!acc) return set_err(c, ADCGPU_CUDA_ERROR, "cudaGetSymbolAddress of the static scratch failed");
  int st = c->mixed_bf16
               ? sigma_fp32_with_acc<__nv_bfloat16>(c, m, (const float*)dv, ld, (float*)dw, ld,
                                                    (const __nv_bfloat16*)c->d_Bt16, acc)
               : sigma_fp32_with_acc<float>(c, m, (const float*)dv, ld, (float*)dw, ld, c->d_Bt32, acc);
  if (st) return st;
  ADC_CUDA(c, cudaStreamSynchronize(c->stream));
  return ADCGPU_OK;
}
