// Segments A and B of the coupling block (the singles (a', k) and (b', k) of
// a double (a', b', k', l'); layout in internal.h) in compact form, for the
// mixed-precision sigma product.  Replaces the per-(slab, b') pass 2 and the
// per-run pass 3 of sigma.cu on the BF16 tensor-core path and the FP32-value
// tiled path; the product is that of hxvec_incore (block_davidson.f90:
// 844-883) restricted to these entries.
//
// The compact form.  In a slab of a class with a' < b' (classes 2, 4I, 4II,
// fixed k', l') the segment-A entry of row (a', b') at a hole k outside
// {k', l'} is the coupling of (a', k) with the double, and the coincidence
// tests of C1, C2 and C4_ph_2p2h (adc_ph.f90:974-1054) leave only the term
// that depends on (b', k, k', l'): the same FP64 value, thresholded the same
// way, for every a'.  Likewise the segment-B entry depends on (a', k) only.
// So per slab
//     segA[(a',b'), k] = Y[b', k] + [k = k'] P(a',b') + [k = l'] Q(a',b')
//     segB[(a',b'), k] = Z[a', k] + [k = k'] R(a',b') + [k = l'] S(a',b')
// with Y, Z zero at k', l' and P, Q, R, S the stored coincident entries
// (Q = S = 0 when k' = l').  The tables are copied out of the value store, so
// they reproduce it exactly.  With them the slab's products are small dense
// contractions over k (16 values) and over a' or b', and the rows are read
// in storage order:
//   W2[(a',b'), c] += sum_k segA[k] V[(a',k), c] + sum_k segB[k] V[(b',k), c]
//   W1[(b',k), c]  += sum_{a'<b'} segB[(a',b'), k] V2[(a',b'), c]     (phase 1)
//   W1[(a',k), c]  += sum_{b'>a'} segA[(a',b'), k] V2[(a',b'), c]     (phase 2)
// Rows of the classes with a' = b' (1 and 3) carry segment A only and are
// handled row by row by k_ab_diag.
#include <cuda_bf16.h>

#include <algorithm>
#include <type_traits>
#include <vector>

#include "internal.h"

namespace adcgpu {

namespace {

// slab s of the classes with a' < b': s < no -> class 2 (k' = l' = s);
// otherwise classes 4I / 4II, hole pair s - no (mod npair_o)
struct PairSlab {
  int cls, kp, lp;
  int64_t row0;
};

__host__ __device__ inline PairSlab pair_slab(const GeomDev& g, int s) {
  PairSlab r;
  if (s < g.no) {
    r.cls = 1; r.kp = r.lp = s;
    r.row0 = g.start[1] + (int64_t)s * g.npair_v;
  } else {
    const int64_t t = s - g.no;
    r.cls = 3 + (int)(t / g.npair_o);
    const int64_t p = t % g.npair_o;
    pair_decode(p, g.no, r.kp, r.lp);
    r.row0 = g.start[r.cls] + p * g.npair_v;
  }
  return r;
}

// index of a pair-class row in the coincident-entry table
__host__ __device__ inline int64_t pair_row_index(const GeomDev& g, int cls, int64_t row) {
  return cls == 1 ? row - g.start[1] : (g.start[2] - g.start[1]) + (row - g.start[3]);
}

template <typename TV> __device__ inline float to_f(TV x);
template <> __device__ inline float to_f<__nv_bfloat16>(__nv_bfloat16 x) { return __bfloat162float(x); }
template <> __device__ inline float to_f<float>(float x) { return x; }

// Copies Y, Z and the coincident entries out of the value store.
template <typename TV>
__global__ void k_ab_extract(GeomDev g, const TV* __restrict__ Bt, int nslab, float* __restrict__ Y,
                             float* __restrict__ Z, float4* __restrict__ coin) {
  const int nv = g.nv, no = g.no, noP = g.noP;
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, nth = (int64_t)gridDim.x * blockDim.x;
  // Y[s][b][k], Z[s][a][k]
  const int64_t ntab = (int64_t)nslab * nv * noP;
  for (int64_t i = tid; i < ntab; i += nth) {
    const int k = (int)(i % noP);
    const int x = (int)((i / noP) % nv);
    const int s = (int)(i / ((int64_t)noP * nv));
    const PairSlab ps = pair_slab(g, s);
    const int64_t L = g.len[ps.cls];
    const bool kin = k < no && k != ps.kp && k != ps.lp;
    float y = 0.f, z = 0.f;
    if (kin && x >= 1) {           // row (0, x): segment A at k
      const int64_t row = ps.row0 + pair_index(0, x, nv);
      y = to_f(Bt[g.off[ps.cls] + (row - g.start[ps.cls]) * L + k]);
    }
    if (kin && x <= nv - 2) {      // row (x, nv - 1): segment B at k
      const int64_t row = ps.row0 + pair_index(x, nv - 1, nv);
      z = to_f(Bt[g.off[ps.cls] + (row - g.start[ps.cls]) * L + noP + k]);
    }
    Y[i] = y;
    Z[i] = z;
  }
  // coincident entries of every pair-class row
  const int64_t c2 = g.start[2] - g.start[1], nrow = c2 + (g.start[5] - g.start[3]);
  for (int64_t t = tid; t < nrow; t += nth) {
    const int64_t row = t < c2 ? g.start[1] + t : g.start[3] + (t - c2);
    const int cls = t < c2 ? 1 : (row < g.start[4] ? 3 : 4);
    const int64_t L = g.len[cls];
    const int64_t rl = row - g.start[cls];
    int kp, lp;
    if (cls == 1) {
      kp = lp = (int)(rl / g.npair_v);
    } else {
      pair_decode(rl / g.npair_v, no, kp, lp);
    }
    const TV* rp = Bt + g.off[cls] + rl * L;
    float4 q;
    q.x = to_f(rp[kp]);
    q.y = kp != lp ? to_f(rp[lp]) : 0.f;
    q.z = to_f(rp[noP + kp]);
    q.w = kp != lp ? to_f(rp[noP + lp]) : 0.f;
    coin[t] = q;
  }
}

// swizzled 16-byte slot of (b, k) in the V1 table: the 8 lanes of a
// quarter-warp with consecutive b read 8 different bank groups
__device__ __forceinline__ int v1_slot(int b, int k, int NOPv) { return b * NOPv + (k ^ (b & 7)); }

// One CTA per (pair-class slab, 4 columns); thread b <-> virtual b.
// Phase 1 (every a' < b): W2 of row (a', b) and, in registers, the segment-B
// sums of single (b, k).  Phase 2 (DO_A; thread a): the segment-A sums of
// single (a, k) over its run of rows (a, a+1 .. nv-1).  Dynamic shared
// memory: V1 of the block's columns [nvS][NOP] float4, Z [nv][NOP], Y [NOP][nvS].
template <int NOP, bool DO_A>
__global__ void __launch_bounds__(256) k_ab_pairs(GeomDev g, const float* __restrict__ Yt,
                                                  const float* __restrict__ Zt, const float4* __restrict__ coin,
                                                  const float* __restrict__ V, int64_t ldv, int m,
                                                  float* __restrict__ W, int64_t ldw, double* __restrict__ W1,
                                                  int64_t ld1) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int nv = g.nv, no = g.no;
  const int nvS = blockDim.x;
  float4* sV1 = reinterpret_cast<float4*>(smem);
  float* sZ = reinterpret_cast<float*>(sV1 + (size_t)nvS * NOP);
  float* sY = sZ + (size_t)nv * NOP;
  const int s = blockIdx.x;
  const int c0 = blockIdx.y * 4;
  const int ncol = min(4, m - c0);
  const PairSlab ps = pair_slab(g, s);
  const int64_t n1 = g.n1;
  const int tid = threadIdx.x;
  // phase 0: tables of this slab and V1 of the four columns
  for (int i = tid; i < nv * NOP; i += nvS) {
    const int b = i / NOP, k = i - b * NOP;
    float4 v;
    float* pv = reinterpret_cast<float*>(&v);
#pragma unroll
    for (int c = 0; c < 4; ++c)
      pv[c] = (k < no && c < ncol) ? V[(int64_t)(c0 + c) * ldv + (int64_t)b * no + k] : 0.f;
    sV1[v1_slot(b, k, NOP)] = v;
    sZ[i] = Zt[((int64_t)s * nv) * NOP + i];
    if (DO_A) sY[k * nvS + b] = Yt[((int64_t)s * nv) * NOP + i];
  }
  __syncthreads();
  const int kp = ps.kp, lp = ps.lp;
  const int cls = ps.cls;
  const bool cls2 = cls == 1;
  // ------------------------------------------------------------- phase 1
  {
    const int b = tid;
    const bool act = b < nv && b >= 1;
    float accB[NOP][4];
#pragma unroll
    for (int k = 0; k < NOP; ++k)
#pragma unroll
      for (int c = 0; c < 4; ++c) accB[k][c] = 0.f;
    float accR[4] = {0.f, 0.f, 0.f, 0.f}, accS[4] = {0.f, 0.f, 0.f, 0.f};
    const int amax = act ? b : 0;
    for (int a = 0; a < amax; ++a) {
      const int64_t pr = pair_index(a, b, nv);
      const int64_t row = ps.row0 + pr;
      const int64_t d = cls2 ? g.start[1] + pr * no + kp : row;
      const float4 q = coin[pair_row_index(g, cls, row)];
      float v2[4], w2[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        v2[c] = c < ncol ? V[(int64_t)(c0 + c) * ldv + n1 + d] : 0.f;
        w2[c] = c < ncol ? W[(int64_t)(c0 + c) * ldw + n1 + d] : 0.f;
      }
      // sum_k segA[k] V1[(a,k)] + sum_k segB[k] V1[(b,k)]
#pragma unroll
      for (int k = 0; k < NOP; ++k) {
        const float zk = sZ[a * NOP + k];
        const float4 xb = sV1[v1_slot(b, k, NOP)];
        w2[0] = fmaf(zk, xb.x, w2[0]);
        w2[1] = fmaf(zk, xb.y, w2[1]);
        w2[2] = fmaf(zk, xb.z, w2[2]);
        w2[3] = fmaf(zk, xb.w, w2[3]);
        if (DO_A) {
          const float yk = sY[k * nvS + b];              // consecutive b: no bank conflicts
          const float4 xa = sV1[v1_slot(a, k, NOP)];   // the same for the whole CTA: broadcast
          w2[0] = fmaf(yk, xa.x, w2[0]);
          w2[1] = fmaf(yk, xa.y, w2[1]);
          w2[2] = fmaf(yk, xa.z, w2[2]);
          w2[3] = fmaf(yk, xa.w, w2[3]);
        }
#pragma unroll
        for (int c = 0; c < 4; ++c) accB[k][c] = fmaf(zk, v2[c], accB[k][c]);
      }
      // coincident entries
      {
        const float4 bk = sV1[v1_slot(b, kp, NOP)], bl = sV1[v1_slot(b, lp, NOP)];
        const float* pbk = reinterpret_cast<const float*>(&bk);
        const float* pbl = reinterpret_cast<const float*>(&bl);
#pragma unroll
        for (int c = 0; c < 4; ++c) w2[c] = fmaf(q.z, pbk[c], fmaf(q.w, pbl[c], w2[c]));
        if (DO_A) {
          const float4 ak = sV1[v1_slot(a, kp, NOP)], al = sV1[v1_slot(a, lp, NOP)];
          const float* pak = reinterpret_cast<const float*>(&ak);
          const float* pal = reinterpret_cast<const float*>(&al);
#pragma unroll
          for (int c = 0; c < 4; ++c) w2[c] = fmaf(q.x, pak[c], fmaf(q.y, pal[c], w2[c]));
        }
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          accR[c] = fmaf(q.z, v2[c], accR[c]);
          accS[c] = fmaf(q.w, v2[c], accS[c]);
        }
      }
#pragma unroll
      for (int c = 0; c < 4; ++c)
        if (c < ncol) W[(int64_t)(c0 + c) * ldw + n1 + d] = w2[c];
    }
    if (act) {
#pragma unroll
      for (int k = 0; k < NOP; ++k) {
        if (k >= no) break;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          if (c >= ncol) break;
          const float v = accB[k][c] + (k == kp ? accR[c] : 0.f) + (k == lp ? accS[c] : 0.f);
          if (v != 0.f) atomicAdd(&W1[(int64_t)(c0 + c) * ld1 + (int64_t)b * no + k], (double)v);
        }
      }
    }
  }
  if (!DO_A) return;
  // ------------------------------------------------------------- phase 2
  {
    const int a = tid;
    if (a >= nv - 1) return;
    float acc[NOP][4];
#pragma unroll
    for (int k = 0; k < NOP; ++k)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[k][c] = 0.f;
    float accP[4] = {0.f, 0.f, 0.f, 0.f}, accQ[4] = {0.f, 0.f, 0.f, 0.f};
    const int64_t pr0 = pair_index(a, a + 1, nv);
    for (int b = a + 1; b < nv; ++b) {
      const int64_t pr = pr0 + (b - a - 1);
      const int64_t row = ps.row0 + pr;
      const int64_t d = cls2 ? g.start[1] + pr * no + kp : row;
      const float4 q = coin[pair_row_index(g, cls, row)];
      float v2[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) v2[c] = c < ncol ? V[(int64_t)(c0 + c) * ldv + n1 + d] : 0.f;
#pragma unroll
      for (int k = 0; k < NOP; ++k) {
        const float yk = sY[k * nvS + b];
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[k][c] = fmaf(yk, v2[c], acc[k][c]);
      }
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        accP[c] = fmaf(q.x, v2[c], accP[c]);
        accQ[c] = fmaf(q.y, v2[c], accQ[c]);
      }
    }
#pragma unroll
    for (int k = 0; k < NOP; ++k) {
      if (k >= no) break;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        if (c >= ncol) break;
        const float v = acc[k][c] + (k == kp ? accP[c] : 0.f) + (k == lp ? accQ[c] : 0.f);
        if (v != 0.f) atomicAdd(&W1[(int64_t)(c0 + c) * ld1 + (int64_t)a * no + k], (double)v);
      }
    }
  }
}

// Segment A of the rows with a' = b' (classes 1 and 3: one row per virtual a
// in each slab).  Thread <-> (a, 4 columns) over a group of AB_DIAG_SLABS slabs
// (class-1 slabs k' = 0..no-1, then the class-3 hole pairs): V1[(a, k)] of its
// columns in registers, W2 of each row updated, the W1 sums of single (a, k)
// accumulated over the group.
constexpr int AB_DIAG_SLABS = 8;

template <typename TV, int NOP>
__global__ void __launch_bounds__(256) k_ab_diag(GeomDev g, const TV* __restrict__ Bt, const float* __restrict__ V,
                                                 int64_t ldv, int m, float* __restrict__ W, int64_t ldw,
                                                 double* __restrict__ W1, int64_t ld1) {
  const int nv = g.nv, no = g.no;
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  const int c0 = blockIdx.y * 4;
  const int ncol = min(4, m - c0);
  if (a >= nv) return;
  const int nslab = no + (int)g.npair_o;
  const int q0 = blockIdx.z * AB_DIAG_SLABS, q1 = min(nslab, q0 + AB_DIAG_SLABS);
  const int64_t n1 = g.n1;
  float x1[NOP][4], acc[NOP][4];
#pragma unroll
  for (int k = 0; k < NOP; ++k)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      x1[k][c] = (k < no && c < ncol) ? V[(int64_t)(c0 + c) * ldv + (int64_t)a * no + k] : 0.f;
      acc[k][c] = 0.f;
    }
  for (int q = q0; q < q1; ++q) {
    const int cls = q < no ? 0 : 2;
    const int64_t row = q < no ? (int64_t)q * nv + a : g.start[2] + (int64_t)(q - no) * nv + a;
    const TV* rp = Bt + g.off[cls] + (row - g.start[cls]) * g.len[cls];
    float va[NOP];
#pragma unroll
    for (int k = 0; k < NOP; ++k) va[k] = to_f(rp[k]);
    float v2[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      v2[c] = c < ncol ? V[(int64_t)(c0 + c) * ldv + n1 + row] : 0.f;
      float w = 0.f;
#pragma unroll
      for (int k = 0; k < NOP; ++k) w = fmaf(va[k], x1[k][c], w);
      if (c < ncol) W[(int64_t)(c0 + c) * ldw + n1 + row] += w;
    }
#pragma unroll
    for (int k = 0; k < NOP; ++k)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[k][c] = fmaf(va[k], v2[c], acc[k][c]);
  }
#pragma unroll
  for (int k = 0; k < NOP; ++k) {
    if (k >= no) break;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      if (c >= ncol) break;
      if (acc[k][c] != 0.f) atomicAdd(&W1[(int64_t)(c0 + c) * ld1 + (int64_t)a * no + k], (double)acc[k][c]);
    }
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
struct AbTables {
  const void* made_from = nullptr;   // the value store the tables were copied from
  float* Y = nullptr;                // [nslab][nv][noP]
  float* Z = nullptr;
  float4* coin = nullptr;            // [pair-class rows]
};

struct AbPlan {
  AbTables t[2];                     // 0: from the BF16 store, 1: from the FP32 store
};

bool ab_supported(const Ctx* c) {
  const Geometry& G = c->geom;
  return (G.noP == 8 || G.noP == 16 || G.noP == 24 || G.noP == 32) && G.nv >= 2 && G.nv <= 256 && G.no >= 1;
}

// The value store was rewritten (a new matrix): the tables are copied again
// on their next use.
void ab_invalidate(void* handle) {
  AbPlan* p = reinterpret_cast<AbPlan*>(handle);
  if (p)
    for (auto& t : p->t) t.made_from = nullptr;
}

void ab_free(Ctx* c, void*& handle) {
  AbPlan* p = reinterpret_cast<AbPlan*>(handle);
  if (!p) return;
  for (auto& t : p->t) {
    dfree(c, t.Y);
    dfree(c, t.Z);
    dfree(c, t.coin);
  }
  delete p;
  handle = nullptr;
}

static int ab_tables(Ctx* c, void*& handle, int which, const void* Bt) {
  if (!handle) handle = new AbPlan;
  AbTables& t = reinterpret_cast<AbPlan*>(handle)->t[which];
  if (t.made_from == Bt && t.Y) return ADCGPU_OK;
  const Geometry& G = c->geom;
  const GeomDev g = to_dev(G);
  const int nslab = G.no + 2 * (int)G.npair_o;
  const size_t ntab = (size_t)nslab * G.nv * G.noP;
  const size_t nrow = (size_t)((G.start[2] - G.start[1]) + (G.start[5] - G.start[3]));
  int st;
  if (!t.Y && (st = dmalloc(c, (void**)&t.Y, sizeof(float) * ntab))) return st;
  if (!t.Z && (st = dmalloc(c, (void**)&t.Z, sizeof(float) * ntab))) return st;
  if (!t.coin && (st = dmalloc(c, (void**)&t.coin, sizeof(float4) * std::max<size_t>(nrow, 1)))) return st;
  if (which == 0)
    k_ab_extract<__nv_bfloat16><<<c->nsm * 8, 256, 0, c->stream>>>(g, (const __nv_bfloat16*)Bt, nslab, t.Y, t.Z,
                                                                   t.coin);
  else
    k_ab_extract<float><<<c->nsm * 8, 256, 0, c->stream>>>(g, (const float*)Bt, nslab, t.Y, t.Z, t.coin);
  ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  t.made_from = Bt;
  return ADCGPU_OK;
}

// Segments A (when do_a) and B of the pair classes, and (when do_a) segment A
// of the classes with a' = b', for m columns of FP32 vectors; W2 rows are
// updated in place, the singles sums go to the FP64 accumulator W1 (ld1).
template <typename TV>
int ab_launch(Ctx* c, void*& handle, const TV* Bt, bool do_a, const float* V, int64_t ldv, int m, float* W,
              int64_t ldw, double* W1, int64_t ld1) {
  const int which = std::is_same<TV, float>::value ? 1 : 0;
  ST(ab_tables(c, handle, which, Bt));
  const AbTables& t = reinterpret_cast<AbPlan*>(handle)->t[which];
  const Geometry& G = c->geom;
  const GeomDev g = to_dev(G);
  const int nslab = G.no + 2 * (int)G.npair_o;
  const int nvS = (G.nv + 31) / 32 * 32;
  const int ncb = (m + 3) / 4;
  const size_t smem = (size_t)nvS * G.noP * 16 + (size_t)G.nv * G.noP * 4 + (do_a ? (size_t)G.noP * nvS * 4 : 0);
  // the cap is a per-function attribute shared by every host thread: set it
  // to the device maximum, not to this launch's size
  const int smax = smem_optin_max(c);
  if (smem > (size_t)smax) return set_err(c, ADCGPU_UNSUPPORTED, "segment A/B kernels: shared memory too small");
  auto pairs = [&](auto kern) -> int {
    ADC_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smax));
    kern<<<dim3(nslab, ncb), nvS, smem, c->stream>>>(g, t.Y, t.Z, t.coin, V, ldv, m, W, ldw, W1, ld1);
    ADC_COUNT_LAUNCH();
    ADC_CUDA(c, cudaGetLastError());
    return ADCGPU_OK;
  };
  if (nslab > 0) {
    switch (G.noP) {
      case 8: ST(do_a ? pairs(k_ab_pairs<8, true>) : pairs(k_ab_pairs<8, false>)); break;
      case 16: ST(do_a ? pairs(k_ab_pairs<16, true>) : pairs(k_ab_pairs<16, false>)); break;
      case 24: ST(do_a ? pairs(k_ab_pairs<24, true>) : pairs(k_ab_pairs<24, false>)); break;
      default: ST(do_a ? pairs(k_ab_pairs<32, true>) : pairs(k_ab_pairs<32, false>)); break;
    }
  }
  if (do_a) {
    const int nq = G.no + (int)G.npair_o;
    const dim3 grid((G.nv + 127) / 128, ncb, (nq + AB_DIAG_SLABS - 1) / AB_DIAG_SLABS);
    switch (G.noP) {
      case 8: k_ab_diag<TV, 8><<<grid, 128, 0, c->stream>>>(g, Bt, V, ldv, m, W, ldw, W1, ld1); break;
      case 16: k_ab_diag<TV, 16><<<grid, 128, 0, c->stream>>>(g, Bt, V, ldv, m, W, ldw, W1, ld1); break;
      case 24: k_ab_diag<TV, 24><<<grid, 128, 0, c->stream>>>(g, Bt, V, ldv, m, W, ldw, W1, ld1); break;
      default: k_ab_diag<TV, 32><<<grid, 128, 0, c->stream>>>(g, Bt, V, ldv, m, W, ldw, W1, ld1); break;
    }
    ADC_COUNT_LAUNCH();
    ADC_CUDA(c, cudaGetLastError());
  }
  return ADCGPU_OK;
}

template int ab_launch<__nv_bfloat16>(Ctx*, void*&, const __nv_bfloat16*, bool, const float*, int64_t, int, float*,
                                      int64_t, double*, int64_t);
template int ab_launch<float>(Ctx*, void*&, const float*, bool, const float*, int64_t, int, float*, int64_t, double*,
                              int64_t);

}  // namespace adcgpu
