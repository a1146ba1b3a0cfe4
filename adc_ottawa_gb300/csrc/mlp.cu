// Learned preconditioner (placeholder translation unit; filled in with the
// MLP kernels).  Until a network is loaded the Davidson driver falls back to
// the diagonal preconditioner.
#include "davidson.h"
#include "dense.h"

namespace adcgpu {

template <typename T>
int mlp_apply(Ctx* c, const MlpPrecond&, int64_t N, int nb, const T* R, const T*, const double* d_lam, const T* hii,
              T* Tout) {
  return precond_dpr<T, T>(c, N, nb, R, N, d_lam, hii, Tout, N);
}

template int mlp_apply<double>(Ctx*, const MlpPrecond&, int64_t, int, const double*, const double*, const double*,
                               const double*, double*);
template int mlp_apply<float>(Ctx*, const MlpPrecond&, int64_t, int, const float*, const float*, const double*,
                              const float*, float*);

}  // namespace adcgpu
