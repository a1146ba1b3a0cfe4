// The CVS ADC(2)-s matrix (write_fspace_adc2_1_cvs, fspacetrial.f90:566-596)
// on the device: FP64 sigma product, COO export and release.  The matrix is
// built in build_kernels.cu (build_matrix_cvs):
//
//   H = | Ac   B |   Ac : dense ph-ph block of the core singles (diagonal included)
//       | B^T  D |   B^T: CSR over the doubles rows, kept entries only, column
//                         = CVS single index; D: the 2p2h diagonal
//
// The CVS space is small in its singles (ncore * nvirt) and its rows couple
// to at most 2 ncore + nvirt singles, so W1 = B V2 is accumulated per block
// in shared memory (one slot per single and column) and added to W1 once per
// block; W2 = B^T V1 + D V2 reads each row's entries once for a group of
// columns.  The reference's counterpart is the COO product hxvec_incore
// (block_davidson.f90:844-883) over the hmlt.off records the CVS builder
// writes.
#include <algorithm>
#include <vector>

#include "internal.h"

namespace adcgpu {
namespace {

// W1(i,q) = sum_j Ac(i,j) V1(j,q), one thread per (i, q)
__global__ void k_cvs_singles(int cn1, int m, const double* __restrict__ Ac, const double* __restrict__ V,
                              int64_t ldv, double* __restrict__ W, int64_t ldw) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)cn1 * m;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % cn1), q = (int)(t / cn1);
    const double* a = Ac + (int64_t)i * cn1;
    const double* v = V + q * ldv;
    double acc = 0.0;
    for (int j = 0; j < cn1; ++j) acc = fma(a[j], v[j], acc);
    W[i + q * ldw] = acc;
  }
}

// Doubles rows for MG columns [q0, q0 + MG): one warp per row.
//   W2(r,q) = D(r) V2(r,q) + sum_e val_e V1(col_e, q)
//   W1(col_e, q) += val_e V2(r, q)   (shared accumulator, added once per block)
template <int MG>
__global__ void __launch_bounds__(256) k_cvs_rows(int64_t n2, int cn1, int q0, const int64_t* __restrict__ rowptr,
                                                  const int32_t* __restrict__ col, const double* __restrict__ val,
                                                  const double* __restrict__ diag, const double* __restrict__ V,
                                                  int64_t ldv, double* __restrict__ W, int64_t ldw) {
  extern __shared__ double sh[];
  double* sV1 = sh;                       // [cn1][MG]
  double* sW1 = sh + (int64_t)cn1 * MG;   // [cn1][MG]
  for (int t = threadIdx.x; t < cn1 * MG; t += blockDim.x) {
    const int j = t / MG, q = t % MG;
    sV1[t] = V[j + (int64_t)(q0 + q) * ldv];
    sW1[t] = 0.0;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = w0; r < n2; r += nw) {
    const int64_t R = cn1 + r;
    double v2[MG], acc[MG];
#pragma unroll
    for (int q = 0; q < MG; ++q) {
      v2[q] = V[R + (int64_t)(q0 + q) * ldv];
      acc[q] = 0.0;
    }
    const int64_t e1 = rowptr[r + 1];
    for (int64_t e = rowptr[r] + lane; e < e1; e += 32) {
      const double x = val[e];
      const int j = col[e];
#pragma unroll
      for (int q = 0; q < MG; ++q) {
        acc[q] = fma(x, sV1[j * MG + q], acc[q]);
        atomicAdd(&sW1[j * MG + q], x * v2[q]);
      }
    }
#pragma unroll
    for (int q = 0; q < MG; ++q) {
      double a = acc[q];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
      if (lane == q % 32) W[R + (int64_t)(q0 + q) * ldw] = fma(diag[R], v2[q], a);
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < cn1 * MG; t += blockDim.x) {
    const double x = sW1[t];
    if (x != 0.0) atomicAdd(&W[t / MG + (int64_t)(q0 + t % MG) * ldw], x);
  }
}

template <int MG>
int launch_rows(Ctx* c, int q0, const double* dV, int64_t ldv, double* dW, int64_t ldw) {
  const size_t smem = sizeof(double) * 2 * (size_t)c->cvs_n1 * MG;
  if (smem > 48 * 1024)
    ADC_CUDA(c, cudaFuncSetAttribute(k_cvs_rows<MG>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t n2 = c->cvs_N - c->cvs_n1;
  k_cvs_rows<MG><<<c->nsm * 2, 256, smem, c->stream>>>(n2, (int)c->cvs_n1, q0, c->d_crow, c->d_ccol, c->d_cval,
                                                         c->d_diag, dV, ldv, dW, ldw);
  ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  return ADCGPU_OK;
}

// COO export: the ph-ph pairs (i > j, row i first as the reference's loop
// writes them) from the dense block, then the coupling entries by rows.
__global__ void k_cvs_export_phph(const double* __restrict__ Ac, int cn1, const int64_t* __restrict__ pos,
                                  double* __restrict__ h, int32_t* __restrict__ oi, int32_t* __restrict__ oj) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cn1; i += gridDim.x * blockDim.x) {
    int64_t o = pos[i];
    for (int j = 0; j < i; ++j) {
      const double x = Ac[(int64_t)i * cn1 + j];
      if (x != 0.0) { h[o] = x; oi[o] = i + 1; oj[o] = j + 1; ++o; }
    }
  }
}

__global__ void k_cvs_count_phph(const double* __restrict__ Ac, int cn1, int64_t* __restrict__ cnt) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cn1; i += gridDim.x * blockDim.x) {
    int64_t n = 0;
    for (int j = 0; j < i; ++j) n += Ac[(int64_t)i * cn1 + j] != 0.0;
    cnt[i] = n;
  }
}

__global__ void k_cvs_export_coupling(int64_t n2, int cn1, int64_t base, const int64_t* __restrict__ rowptr,
                                      const int32_t* __restrict__ col, const double* __restrict__ val,
                                      double* __restrict__ h, int32_t* __restrict__ oi, int32_t* __restrict__ oj) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n2; r += (int64_t)gridDim.x * blockDim.x)
    for (int64_t e = rowptr[r]; e < rowptr[r + 1]; ++e) {
      h[base + e] = val[e];
      oi[base + e] = col[e] + 1;
      oj[base + e] = (int32_t)(cn1 + r + 1);
    }
}

}  // namespace

int sigma_cvs(Ctx* c, int m, const double* dV, int64_t ldv, double* dW, int64_t ldw) {
  const int cn1 = (int)c->cvs_n1;
  k_cvs_singles<<<std::max(1, std::min(c->nsm * 8, (cn1 * m + 255) / 256)), 256, 0, c->stream>>>(cn1, m, c->d_Ac, dV,
                                                                                                  ldv, dW, ldw);
  ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  // columns per pass: both shared arrays within 200 KiB
  const int64_t cap = (int64_t)200 * 1024 / (2 * (int64_t)sizeof(double) * cn1);
  for (int q0 = 0; q0 < m;) {
    const int left = m - q0;
    int mg = 1;
    for (int t : {16, 8, 4, 2})
      if (t <= left && t <= cap) { mg = t; break; }
    switch (mg) {
      case 16: ST(launch_rows<16>(c, q0, dV, ldv, dW, ldw)); break;
      case 8: ST(launch_rows<8>(c, q0, dV, ldv, dW, ldw)); break;
      case 4: ST(launch_rows<4>(c, q0, dV, ldv, dW, ldw)); break;
      case 2: ST(launch_rows<2>(c, q0, dV, ldv, dW, ldw)); break;
      default: ST(launch_rows<1>(c, q0, dV, ldv, dW, ldw)); break;
    }
    q0 += mg;
  }
  return ADCGPU_OK;
}

int export_coo_cvs(Ctx* c, double* d_h, int32_t* d_oi, int32_t* d_oj) {
  const int cn1 = (int)c->cvs_n1;
  const int64_t n2 = c->cvs_N - cn1;
  int64_t* d_cnt = nullptr;
  ST(dmalloc(c, (void**)&d_cnt, sizeof(int64_t) * (cn1 + 1)));
  std::vector<int64_t> cnt(cn1 + 1, 0);
  k_cvs_count_phph<<<(cn1 + 127) / 128, 128, 0, c->stream>>>(c->d_Ac, cn1, d_cnt);
  ADC_COUNT_LAUNCH();
  int st = ADCGPU_OK;
  if (cudaMemcpyAsync(cnt.data(), d_cnt, sizeof(int64_t) * cn1, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
      cudaStreamSynchronize(c->stream) != cudaSuccess)
    st = set_err(c, ADCGPU_CUDA_ERROR, "CVS export: row counts");
  int64_t tot = 0;
  for (int i = 0; i < cn1; ++i) { const int64_t x = cnt[i]; cnt[i] = tot; tot += x; }
  if (!st && cudaMemcpyAsync(d_cnt, cnt.data(), sizeof(int64_t) * cn1, cudaMemcpyHostToDevice, c->stream) != cudaSuccess)
    st = set_err(c, ADCGPU_CUDA_ERROR, "CVS export: offsets");
  if (!st) {
    k_cvs_export_phph<<<(cn1 + 127) / 128, 128, 0, c->stream>>>(c->d_Ac, cn1, d_cnt, d_h, d_oi, d_oj);
    ADC_COUNT_LAUNCH();
    k_cvs_export_coupling<<<c->nsm * 4, 256, 0, c->stream>>>(n2, cn1, tot, c->d_crow, c->d_ccol, c->d_cval, d_h,
                                                             d_oi, d_oj);
    ADC_COUNT_LAUNCH();
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(c->stream) != cudaSuccess)
      st = set_err(c, ADCGPU_CUDA_ERROR, "CVS export");
  }
  dfree(c, d_cnt);
  return st;
}

void free_cvs(Ctx* c) {
  dfree(c, c->d_Ac); c->d_Ac = nullptr;
  dfree(c, c->d_crow); c->d_crow = nullptr;
  dfree(c, c->d_ccol); c->d_ccol = nullptr;
  dfree(c, c->d_cval); c->d_cval = nullptr;
  c->cvs = 0;
  c->cvs_n1 = c->cvs_N = c->cvs_nnz = 0;
  c->cvs_kpq.clear();
}

}  // namespace adcgpu
