// Declarations of the tall-skinny dense kernels (dense.cu).
#pragma once
#include "internal.h"

namespace adcgpu {

// Reusable device scratch owned by a solver call.
struct Workspace {
  Ctx* ctx = nullptr;
  void* p = nullptr;
  size_t bytes = 0;
  ~Workspace();
  void release();
  int reserve(Ctx* c, size_t need);
};

// C(p x q, ldc) = beta C + alpha A^T B, A: N x p (lda), B: N x q (ldb).
// TA is the accumulation type, TC the output type.
template <typename T, typename TA, typename TC>
int gemm_tn(Ctx* c, Workspace& ws, int64_t N, int p, int q, const T* A, int64_t lda, const T* B, int64_t ldb,
            TC* C, int ldc, TC alpha, TC beta);

// C(N x q) = beta C + alpha A(N x p) B(p x q); C must not alias A.
template <typename T, typename TB>
int gemm_nn(Ctx* c, int64_t N, int p, int q, T alpha, const T* A, int64_t lda, const TB* B, int ldb, T beta, T* C,
            int64_t ldc);

template <typename T, typename TD>
int precond_dpr(Ctx* c, int64_t N, int nb, const T* R, int64_t ldr, const double* d_lam, const TD* hii, T* Tout,
                int64_t ldt);

template <typename T, typename TD>
int precond_olsen(Ctx* c, Workspace& ws, int64_t N, int nb, const T* X, const T* R, int64_t ld, const double* d_lam,
                  const TD* hii, T* Tout, int64_t ldt, double* h_alpha_out);

// Folded singles-block preconditioner (precond_fold.cu): Tout = correction of
// the residual block R; Z (N x 2nb, leading dimension N) is scratch.
template <typename T>
int precond_fold(Ctx* c, Workspace& ws, int64_t N, int nb, const T* R, int64_t ldr, const double* d_lam,
                 const T* hii, T* Tout, int64_t ldt, T* Z, int64_t ldz);

// Rout = lambda X - WY (column-wise); h_norm2 receives ||Rout_i||^2 (FP64 sums).
template <typename T>
int residuals(Ctx* c, Workspace& ws, int64_t N, int nb, const T* X, const T* WY, int64_t ld, const double* d_lam,
              T* Rout, double* h_norm2);

template <typename TS, typename TD>
int convert(Ctx* c, const TS* x, TD* y, int64_t n);

// Tensor-core Gram product of FP32 inputs (dense_umma.cu): C(p x q, FP64,
// ldc) = beta C + alpha A^T B for q <= 48, FP32-accurate products.
bool gram_umma_usable(Ctx* c, int64_t N, int p, int q);
int gram_umma(Ctx* c, Workspace& ws, int64_t N, int p, int q, const float* A, int64_t lda, const float* B,
              int64_t ldb, double* C, int ldc, double alpha, double beta);


}  // namespace adcgpu
