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

// Row descriptor: a' | b'<<16 in .x; k' | l'<<8 | cls<<16 in .y.
__device__ __forceinline__ void unpack(uint2 q, int& ap, int& bp, int& kp, int& lp, int& cls) {
  ap = q.x & 0xFFFF; bp = q.x >> 16; kp = q.y & 0xFF; lp = (q.y >> 8) & 0xFF; cls = q.y >> 16;
}

constexpr int MAXC = 8;   // columns per pass held in registers

template <typename T, typename TV>
__global__ void __launch_bounds__(256) k_doubles(GeomDev g, const uint2* __restrict__ desc,
                                                 const TV* __restrict__ Bt, const T* __restrict__ diag,
                                                 const T* __restrict__ V, int64_t ldv, T* __restrict__ W,
                                                 int64_t ldw, int mc, int c0) {
  extern __shared__ unsigned char smem_raw[];
  T* sW1 = reinterpret_cast<T*>(smem_raw);          // [mc][n1]
  const int n1 = (int)g.n1, no = g.no, nv = g.nv;
  for (int i = threadIdx.x; i < mc * n1; i += blockDim.x) sW1[i] = T(0);
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const T* V1 = V + (int64_t)c0 * ldv;
  const T* V2 = V1 + n1;
  for (int64_t d = warp; d < g.n2; d += nwarps) {
    int ap, bp, kp, lp, cls;
    unpack(desc[d], ap, bp, kp, lp, cls);
    const int64_t L = g.len[cls];
    const TV* row = Bt + g.off[cls] + (d - g.start[cls]) * L;
    T x2[MAXC], acc[MAXC];
#pragma unroll
    for (int c = 0; c < MAXC; ++c) {
      x2[c] = c < mc ? V2[d + c * ldv] : T(0);
      acc[c] = T(0);
    }
    const bool twoa = ap != bp;
    const int nseg = nv - (twoa ? 2 : 1);
    for (int e = lane; e < L; e += 32) {
      // single index of entry e (segments A, B, C, D)
      int s;
      if (e < no) s = ap * no + e;
      else if (twoa && e < 2 * no) s = bp * no + (e - no);
      else {
        int t = e - (twoa ? 2 * no : no);
        int seg = t >= nseg;
        t -= seg * nseg;
        int a = t + (t >= ap);
        if (twoa) a += (a >= bp);
        s = a * no + (seg ? lp : kp);
      }
      const T h = Acc<T, TV>::v(row[e]);
#pragma unroll
      for (int c = 0; c < MAXC; ++c) {
        if (c < mc) {
          acc[c] += h * V1[s + c * ldv];
          atomicAdd(&sW1[c * n1 + s], h * x2[c]);
        }
      }
    }
#pragma unroll
    for (int c = 0; c < MAXC; ++c) {
      if (c < mc) {
        T v = acc[c];
        for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) W[(int64_t)(c0 + c) * ldw + n1 + d] = diag[n1 + d] * x2[c] + v;
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < mc * n1; i += blockDim.x) {
    int c = i / n1, s = i - c * n1;
    T v = sW1[i];
    if (v != T(0)) atomicAdd(&W[(int64_t)(c0 + c) * ldw + s], v);
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

template <typename T, typename TV>
int sigma_impl(Ctx* c, int m, const T* dV, int64_t ldv, T* dW, int64_t ldw, const T* A, const T* diag,
               const TV* Bt) {
  const Geometry& G = c->geom;
  const int n1 = (int)G.n1;
  cudaStream_t s = c->stream;
  GeomDev g = to_dev(G);
  // singles block first (plain stores), then the coupling adds atomically
  dim3 gs((n1 + 63) / 64, (m + 3) / 4);
  k_singles<T><<<gs, 256, 0, s>>>(n1, A, diag, dV, ldv, dW, ldw, m);
  ADC_CUDA(c, cudaGetLastError());
  const size_t per_col = sizeof(T) * (size_t)n1;
  int mc_max = (int)std::min<size_t>(MAXC, (200u * 1024u) / per_col);
  if (mc_max < 1) return set_err(c, ADCGPU_UNSUPPORTED, "n1 too large for the shared-memory W1 partial");
  const uint2* desc = reinterpret_cast<const uint2*>(c->d_ws);
  for (int c0 = 0; c0 < m; c0 += mc_max) {
    int mc = std::min(mc_max, m - c0);
    size_t smem = per_col * mc;
    auto kern = k_doubles<T, TV>;
    ADC_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = smem > 110 * 1024 ? 1 : 2;
    kern<<<152 * per_sm, 256, smem, s>>>(g, desc, Bt, diag, dV, ldv, dW, ldw, mc, c0);
    ADC_CUDA(c, cudaGetLastError());
  }
  return ADCGPU_OK;
}

__global__ void k_make_desc(GeomDev g, uint2* desc) {
  for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < g.n2; d += (int64_t)gridDim.x * blockDim.x) {
    Double r = decode_double(g, d);
    desc[d] = make_uint2((unsigned)r.ap | ((unsigned)r.bp << 16),
                         (unsigned)r.kp | ((unsigned)r.lp << 8) | ((unsigned)r.cls << 16));
  }
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

// Row descriptors live at the start of the workspace d_ws.
int prepare_desc(Ctx* c) {
  const Geometry& G = c->geom;
  size_t need = sizeof(uint2) * (size_t)G.n2;
  if (c->ws_bytes < need) {
    if (c->d_ws) dfree(c, c->d_ws, c->ws_bytes);
    c->d_ws = nullptr; c->ws_bytes = 0;
    int st = dmalloc(c, &c->d_ws, need);
    if (st) return st;
    c->ws_bytes = need;
  }
  GeomDev g = to_dev(G);
  k_make_desc<<<152 * 8, 256, 0, c->stream>>>(g, (uint2*)c->d_ws);
  ADC_CUDA(c, cudaGetLastError());
  return ADCGPU_OK;
}

int prepare_mixed(Ctx* c) {
  const Geometry& G = c->geom;
  int st;
  if (!c->d_A32 && (st = dmalloc(c, (void**)&c->d_A32, sizeof(float) * G.n1 * G.n1))) return st;
  if (!c->d_diag32 && (st = dmalloc(c, (void**)&c->d_diag32, sizeof(float) * G.N))) return st;
  k_to_f32<<<152 * 8, 256, 0, c->stream>>>(c->d_A, c->d_A32, G.n1 * G.n1);
  k_to_f32<<<152 * 8, 256, 0, c->stream>>>(c->d_diag, c->d_diag32, G.N);
  if (c->mixed_bf16) {
    if (!c->d_Bt16 && (st = dmalloc(c, (void**)&c->d_Bt16, sizeof(uint16_t) * G.off[5]))) return st;
    k_to_bf16<<<152 * 8, 256, 0, c->stream>>>(c->d_Bt, (__nv_bfloat16*)c->d_Bt16, G.off[5]);
  } else {
    if (!c->d_Bt32 && (st = dmalloc(c, (void**)&c->d_Bt32, sizeof(float) * G.off[5]))) return st;
    k_to_f32<<<152 * 8, 256, 0, c->stream>>>(c->d_Bt, c->d_Bt32, G.off[5]);
  }
  ADC_CUDA(c, cudaGetLastError());
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
