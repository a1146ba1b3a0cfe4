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

#include "internal.h"

namespace adcgpu {

namespace {

template <typename TV> __device__ __forceinline__ float tofloat(TV x);
template <> __device__ __forceinline__ float tofloat<float>(float x) { return x; }
template <> __device__ __forceinline__ float tofloat<__nv_bfloat16>(__nv_bfloat16 x) { return __bfloat162float(x); }

template <typename T, typename TV> struct Acc;
template <> struct Acc<double, double> { __device__ static double v(double x) { return x; } };
template <> struct Acc<float, float> { __device__ static float v(float x) { return x; } };
template <> struct Acc<float, __nv_bfloat16> { __device__ static float v(__nv_bfloat16 x) { return __bfloat162float(x); } };

// Virtual index a = lane + 32 t, t < NT (template: 4, 6 or 8 for nv <= 128,
// 192, 256).

// Advance (a',b') to the next row of a slab in storage order.
__device__ __forceinline__ void next_pair(int& ap, int& bp, bool twoa, int nv) {
  if (!twoa) { ++ap; bp = ap; return; }
  if (++bp == nv) { ++ap; bp = ap + 1; }
}

// Pass 1: one warp per chunk of rows inside one slab (fixed k', l', class).
// Segment C/D products with V2 accumulate in registers (lane owns virtual a),
// segment A products accumulate while a' is unchanged; W2 rows are complete
// except for segment B, which pass 2 adds.
template <typename T, typename TV, int MC, int NTMAX>
__global__ void __launch_bounds__(256) k_sigma_p1(GeomDev g, const int2* __restrict__ chunks, int nchunks,
                                                  const TV* __restrict__ Bt, const T* __restrict__ diag,
                                                  const T* __restrict__ V, int64_t ldv, T* __restrict__ W,
                                                  int64_t ldw) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int no = g.no, nv = g.nv;
  const int64_t n1 = g.n1;
  for (int ci = warp; ci < nchunks; ci += nwarps) {
    const int2 ch = chunks[ci];
    Double r = decode_row(g, ch.x);
    const int cls = r.cls;
    const bool twoa = (cls == 1 || cls >= 3);
    const bool hasD = cls >= 2;
    const int64_t L = g.len[cls];
    const int offC = twoa ? 2 * no : no;
    const int kp = r.kp, lp = r.lp;
    T xk[NTMAX][MC], xl[NTMAX][MC], yk[NTMAX][MC], yl[NTMAX][MC];
#pragma unroll
    for (int t = 0; t < NTMAX; ++t) {
      const int a = lane + 32 * t;
#pragma unroll
      for (int c = 0; c < MC; ++c) {
        xk[t][c] = (a < nv) ? V[(int64_t)c * ldv + (int64_t)a * no + kp] : T(0);
        xl[t][c] = (a < nv && hasD) ? V[(int64_t)c * ldv + (int64_t)a * no + lp] : T(0);
        yk[t][c] = T(0);
        yl[t][c] = T(0);
      }
    }
    int cur_ap = -1;
    T xa[MC], ya[MC];
#pragma unroll
    for (int c = 0; c < MC; ++c) { xa[c] = T(0); ya[c] = T(0); }
    const TV* rowp = Bt + g.off[cls] + (int64_t)(ch.x - g.start[cls]) * L;
    int ap = r.ap, bp = r.bp;
    for (int row = ch.x; row < ch.y; ++row, rowp += L) {
      if (ap != cur_ap) {
        if (cur_ap >= 0 && lane < no) {
#pragma unroll
          for (int c = 0; c < MC; ++c) atomicAdd(&W[(int64_t)c * ldw + (int64_t)cur_ap * no + lane], ya[c]);
        }
        cur_ap = ap;
#pragma unroll
        for (int c = 0; c < MC; ++c) {
          xa[c] = lane < no ? V[(int64_t)c * ldv + (int64_t)ap * no + lane] : T(0);
          ya[c] = T(0);
        }
      }
      Double rr{ap, bp, kp, lp, cls};
      const int64_t d = row_to_d(g, rr, row);
      T x2[MC], z[MC];
#pragma unroll
      for (int c = 0; c < MC; ++c) { x2[c] = V[(int64_t)c * ldv + n1 + d]; z[c] = T(0); }
      // issue the row's loads first
      T vA = lane < no ? (T)Acc<T, TV>::v(rowp[lane]) : T(0);
      T vC[NTMAX], vD[NTMAX];
#pragma unroll
      for (int t = 0; t < NTMAX; ++t) {
        const int a = lane + 32 * t;
        vC[t] = a < nv ? (T)Acc<T, TV>::v(rowp[offC + a]) : T(0);
        vD[t] = (a < nv && hasD) ? (T)Acc<T, TV>::v(rowp[offC + nv + a]) : T(0);
      }
#pragma unroll
      for (int c = 0; c < MC; ++c) {
        ya[c] += vA * x2[c];
        z[c] += vA * xa[c];
#pragma unroll
        for (int t = 0; t < NTMAX; ++t) {
          yk[t][c] += vC[t] * x2[c];
          z[c] += vC[t] * xk[t][c];
          yl[t][c] += vD[t] * x2[c];
          z[c] += vD[t] * xl[t][c];
        }
      }
#pragma unroll
      for (int c = 0; c < MC; ++c) {
        T v = z[c];
#pragma unroll
        for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) W[(int64_t)c * ldw + n1 + d] = diag[n1 + d] * x2[c] + v;
      }
      next_pair(ap, bp, twoa, nv);
    }
    if (lane < no) {
#pragma unroll
      for (int c = 0; c < MC; ++c) atomicAdd(&W[(int64_t)c * ldw + (int64_t)cur_ap * no + lane], ya[c]);
    }
#pragma unroll
    for (int t = 0; t < NTMAX; ++t) {
      const int a = lane + 32 * t;
      if (a < nv) {
#pragma unroll
        for (int c = 0; c < MC; ++c) {
          atomicAdd(&W[(int64_t)c * ldw + (int64_t)a * no + kp], yk[t][c]);
          if (hasD) atomicAdd(&W[(int64_t)c * ldw + (int64_t)a * no + lp], yl[t][c]);
        }
      }
    }
  }
}

// Pass 2: segment B (classes 2, 4I, 4II).  One warp per (slab, b'): rows
// (a',b') for a' < b' share the target singles (b', k), accumulated in
// registers; W2 rows receive the segment-B part of their sums.
template <typename T, typename TV, int MC>
__global__ void __launch_bounds__(256) k_sigma_p2(GeomDev g, const int2* __restrict__ items, int nitems,
                                                  const TV* __restrict__ Bt, const T* __restrict__ V, int64_t ldv,
                                                  T* __restrict__ W, int64_t ldw) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int no = g.no, nv = g.nv;
  const int64_t n1 = g.n1;
  for (int it = warp; it < nitems; it += nwarps) {
    const int2 item = items[it];
    const int slab0 = item.x, bp = item.y;
    Double r = decode_row(g, slab0);
    const int cls = r.cls;
    const int64_t L = g.len[cls];
    T xb[MC], yb[MC];
#pragma unroll
    for (int c = 0; c < MC; ++c) {
      xb[c] = lane < no ? V[(int64_t)c * ldv + (int64_t)bp * no + lane] : T(0);
      yb[c] = T(0);
    }
    for (int ap = 0; ap < bp; ++ap) {
      const int64_t row = slab0 + pair_index(ap, bp, nv);
      Double rr{ap, bp, r.kp, r.lp, cls};
      const int64_t d = row_to_d(g, rr, row);
      const TV* rowp = Bt + g.off[cls] + (row - g.start[cls]) * L;
      T v = lane < no ? (T)Acc<T, TV>::v(rowp[no + lane]) : T(0);
#pragma unroll
      for (int c = 0; c < MC; ++c) {
        const T x2 = V[(int64_t)c * ldv + n1 + d];
        yb[c] += v * x2;
        T z = v * xb[c];
#pragma unroll
        for (int o = 16; o; o >>= 1) z += __shfl_xor_sync(0xffffffffu, z, o);
        if (lane == 0) W[(int64_t)c * ldw + n1 + d] += z;
      }
    }
    if (lane < no) {
#pragma unroll
      for (int c = 0; c < MC; ++c) atomicAdd(&W[(int64_t)c * ldw + (int64_t)bp * no + lane], yb[c]);
    }
  }
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
  c->st_pending = false;
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
  dim3 gs((n1 + 63) / 64, (m + 3) / 4);
  k_singles<T><<<gs, 256, 0, s>>>(n1, A, diag, dV, ldv, dW, ldw, m);
  ADC_CUDA(c, cudaGetLastError());
  const SigmaPlan* plan = reinterpret_cast<const SigmaPlan*>(c->sigma_plan);
  if (!plan) return set_err(c, ADCGPU_NO_MATRIX, "sigma plan missing");
  const int2* chunks = plan->d_chunks;
  const int2* items = plan->d_items;
  int c0 = 0;
  while (c0 < m) {
    const int left = m - c0;
    const T* V = dV + (int64_t)c0 * ldv;
    T* W = dW + (int64_t)c0 * ldw;
    const int mc = (sizeof(T) == 8 || G.nv > 192) ? (left >= 2 ? 2 : 1) : (left >= 4 ? 4 : (left >= 2 ? 2 : 1));
    const int g1 = std::min(plan->nchunks, 152 * 8 * 8) / 8 + 1;
    const int g2 = std::min(plan->nitems, 152 * 8 * 8) / 8 + 1;
#define LAUNCH(MC, NT)                                                                                  \
  k_sigma_p1<T, TV, MC, NT><<<g1, 256, 0, s>>>(g, chunks, plan->nchunks, Bt, diag, V, ldv, W, ldw);    \
  if (plan->nitems) k_sigma_p2<T, TV, MC><<<g2, 256, 0, s>>>(g, items, plan->nitems, Bt, V, ldv, W, ldw);
#define LAUNCH_NT(MC)                                     \
  if (G.nv <= 128) { LAUNCH(MC, 4) }                      \
  else if (G.nv <= 192) { LAUNCH(MC, 6) }                 \
  else { LAUNCH(MC, 8) }
    if (mc == 4) { LAUNCH_NT(4) } else if (mc == 2) { LAUNCH_NT(2) } else { LAUNCH_NT(1) }
#undef LAUNCH_NT
#undef LAUNCH
    ADC_CUDA(c, cudaGetLastError());
    c0 += mc;
  }
  ADC_CUDA(c, cudaEventRecord(c->st_ev1, s));
  c->st_pending = true;
  c->st_pending_cols = m;
  // algorithmic bytes: every stored value once, A once, diagonal once,
  // V read and W written once
  c->st_pending_bytes = (double)G.off[5] * sizeof(TV) + (double)G.n1 * G.n1 * sizeof(T) +
                        (double)G.N * sizeof(T) + 2.0 * (double)m * G.N * sizeof(T);
  return ADCGPU_OK;
}

__global__ void k_to_f32(const double* __restrict__ x, float* __restrict__ y, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = (float)x[i];
}
__global__ void k_to_bf16(const double* __restrict__ x, __nv_bfloat16* __restrict__ y, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = __double2bfloat16(x[i]);
}

}  // namespace

// Work lists of the sigma kernels: pass-1 chunks (row ranges inside one
// slab) and pass-2 items (slab, b') of the classes with a' < b'.
int prepare_desc(Ctx* c) {
  const Geometry& G = c->geom;
  std::vector<int2> chunks, items;
  const int64_t CH = 64;
  for (int cls = 0; cls < 5; ++cls) {
    const int64_t r0 = G.start[cls], r1 = G.start[cls + 1], sl = G.slab_len(cls);
    for (int64_t s0 = r0; s0 < r1; s0 += sl) {
      for (int64_t a = s0; a < s0 + sl; a += CH) chunks.push_back(make_int2((int)a, (int)std::min(a + CH, s0 + sl)));
      if (cls == 1 || cls >= 3)
        for (int bp = 1; bp < G.nv; ++bp) items.push_back(make_int2((int)s0, bp));
    }
  }
  SigmaPlan* plan = reinterpret_cast<SigmaPlan*>(c->sigma_plan);
  if (!plan) { plan = new SigmaPlan; c->sigma_plan = plan; }
  if (plan->d_chunks) cudaFree(plan->d_chunks);
  if (plan->d_items) cudaFree(plan->d_items);
  plan->d_chunks = plan->d_items = nullptr;
  int st;
  if ((st = dmalloc(c, (void**)&plan->d_chunks, sizeof(int2) * chunks.size()))) return st;
  if ((st = dmalloc(c, (void**)&plan->d_items, sizeof(int2) * std::max<size_t>(items.size(), 1)))) return st;
  ADC_CUDA(c, cudaMemcpy(plan->d_chunks, chunks.data(), sizeof(int2) * chunks.size(), cudaMemcpyHostToDevice));
  if (!items.empty())
    ADC_CUDA(c, cudaMemcpy(plan->d_items, items.data(), sizeof(int2) * items.size(), cudaMemcpyHostToDevice));
  plan->nchunks = (int)chunks.size();
  plan->nitems = (int)items.size();
  return ADCGPU_OK;
}

void free_sigma_plan(Ctx* c) {
  SigmaPlan* plan = reinterpret_cast<SigmaPlan*>(c->sigma_plan);
  if (!plan) return;
  if (plan->d_chunks) cudaFree(plan->d_chunks);
  if (plan->d_items) cudaFree(plan->d_items);
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
  k_to_f32<<<152 * 8, 256, 0, c->stream>>>(c->d_A, c->d_A32, G.n1 * G.n1);
  k_to_f32<<<152 * 8, 256, 0, c->stream>>>(c->d_diag, c->d_diag32, G.N);
  k_to_bf16<<<152 * 8, 256, 0, c->stream>>>(c->d_Bt, (__nv_bfloat16*)c->d_Bt16, G.off[5]);
  k_to_f32<<<152 * 8, 256, 0, c->stream>>>(c->d_Bt, c->d_Bt32, G.off[5]);
  ADC_CUDA(c, cudaGetLastError());
  return ADCGPU_OK;
}

extern "C" int adcgpu_sigma_stats(adcgpu_ctx* h, double* out, int reset) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c || !out) return ADCGPU_BAD_INPUT;
  cudaSetDevice(c->device);
  sigma_stats_flush(c);
  out[0] = (double)c->st_calls; out[1] = c->st_ms; out[2] = c->st_bytes; out[3] = (double)c->st_cols;
  if (reset) { c->st_calls = 0; c->st_cols = 0; c->st_ms = 0.0; c->st_bytes = 0.0; }
  return ADCGPU_OK;
}

int sigma_fp64(Ctx* c, int m, const double* dV, int64_t ldv, double* dW, int64_t ldw) {
  return sigma_impl<double, double>(c, m, dV, ldv, dW, ldw, c->d_A, c->d_diag, c->d_Bt);
}

int sigma_fp32(Ctx* c, int m, const float* dV, int64_t ldv, float* dW, int64_t ldw) {
  if (c->mixed_bf16)
    return sigma_impl<float, __nv_bfloat16>(c, m, dV, ldv, dW, ldw, c->d_A32, c->d_diag32,
                                            (const __nv_bfloat16*)c->d_Bt16);
  return sigma_impl<float, float>(c, m, dV, ldv, dW, ldw, c->d_A32, c->d_diag32, c->d_Bt32);
}

}  // namespace adcgpu
