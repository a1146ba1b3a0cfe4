// Davidson driver and the learned preconditioner interface.
#pragma once
#include "internal.h"

namespace adcgpu {

// Learned correction t = MLP(features of the residual) used in place of the
// diagonal preconditioner (block_davidson.f90:1288-1342).  Weights are BF16
// on the device, activations FP32.  See mlp.cu.
struct MlpPrecond {
  int nin = 0, nhid = 0, nout = 0;
  const uint16_t* W1 = nullptr;   // [nhid][nin]  bf16
  const float* b1 = nullptr;      // [nhid]
  const uint16_t* W2 = nullptr;   // [nhid][nhid]
  const float* b2 = nullptr;
  const uint16_t* W3 = nullptr;   // [nout][nhid]
  const float* b3 = nullptr;
  const float* feat_scale = nullptr;  // [nin] input normalisation
  float out_scale = 1.f;
};

template <typename T>
int mlp_apply(Ctx* c, const MlpPrecond& m, int64_t N, int nb, const T* R, const T* X, const double* d_lam,
              const T* hii, T* Tout);

int davidson_solve(Ctx* c, const adcgpu_dav_params* p, double* evals, double* evecs, adcgpu_dav_info* info,
                   const MlpPrecond* mlp);

}  // namespace adcgpu
