// Block Lanczos on the GPU: lancdiag_block (block_lanczos.f90:28-81),
// init_vecs_random (:402-439), run_block_lanczos (:947-1256) with PRO
// (:1474-1706, orthotype 1), calc_pseudospec / diagmat_banded (:1941-2052)
// and ritzvecs_incore (:2237-2316).
//
// The block QR of R_j (dgeqrf/dorgqr, :1146-1168) is Cholesky QR applied
// twice; its triangular factor has a positive diagonal, so B_j and Q_{j+1}
// differ from Householder QR by a diagonal sign matrix S_j.  T is then
// S T S for a block-diagonal sign matrix S with S_1 = I: eigenvalues and
// the first-block moments E_1^T T^k E_1 are identical.
// All Lanczos blocks stay resident in HBM (the reference pages them through
// SCRATCH/lanvecs and lanvecs2).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "dense.h"
#include "internal.h"

namespace adcgpu {

namespace {

__global__ void k_colnorm2_part(int64_t N, int ncol, const double* __restrict__ X, int64_t ld,
                                double* __restrict__ part) {
  __shared__ double red[8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int cidx = 0; cidx < ncol; ++cidx) {
    double s = 0.0;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < N; r += (int64_t)gridDim.x * blockDim.x) {
      double v = X[(int64_t)cidx * ld + r];
      s += v * v;
    }
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) red[w] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += red[q];
      part[(int64_t)blockIdx.x * ncol + cidx] = t;
    }
    __syncthreads();
  }
}

__global__ void k_scale_cols(int64_t N, int ncol, double* __restrict__ X, int64_t ld, const double* __restrict__ s) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < N; r += (int64_t)gridDim.x * blockDim.x)
    for (int c = 0; c < ncol; ++c) X[(int64_t)c * ld + r] *= s[c];
}

}  // namespace


struct LanczosGPU {
  Ctx* c;
  int64_t N;
  int b, ncycles, nvec;
  Workspace ws;
  double *Qall = nullptr, *Q1 = nullptr, *Q2 = nullptr, *U = nullptr, *Tmp = nullptr;
  double *d_s = nullptr, *d_s2 = nullptr, *d_part = nullptr;

  ~LanczosGPU() {
    double* ps[] = {Qall, Q1, Q2, U, Tmp, d_s, d_s2, d_part};
    for (double* p : ps) dfree(c, p);
  }

  int colnorms(double* X, int ncol, std::vector<double>& out) {
    const int nblk = c->nsm * 2;
    k_colnorm2_part<<<nblk, 256, 0, c->stream>>>(N, ncol, X, N, d_part); ADC_COUNT_LAUNCH();
    std::vector<double> part((size_t)nblk * ncol);
    ADC_CUDA(c, cudaMemcpyAsync(part.data(), d_part, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, c->stream));
    ADC_CUDA(c, cudaStreamSynchronize(c->stream));
    out.assign(ncol, 0.0);
    for (int bl = 0; bl < nblk; ++bl)
      for (int i = 0; i < ncol; ++i) out[i] += part[(size_t)bl * ncol + i];
    for (int i = 0; i < ncol; ++i) out[i] = std::sqrt(out[i]);
    return ADCGPU_OK;
  }

  int scale_cols(double* X, int ncol, const std::vector<double>& s) {
    ADC_CUDA(c, cudaMemcpyAsync(d_s2, s.data(), sizeof(double) * ncol, cudaMemcpyHostToDevice, c->stream));
    k_scale_cols<<<c->nsm * 4, 256, 0, c->stream>>>(N, ncol, X, N, d_s2); ADC_COUNT_LAUNCH();
    ADC_CUDA(c, cudaGetLastError());
    return ADCGPU_OK;
  }

  int normalise(double* X, int ncol) {
    std::vector<double> nr;
    ST(colnorms(X, ncol, nr));
    for (auto& v : nr) v = 1.0 / v;
    return scale_cols(X, ncol, nr);
  }

  // X(:,i) -= Q(:,0:nq) (Q^T X(:,i)) for all i (one block CGS step)
  int project(const double* Qb, int nq, double* X, int nx) {
    ST((gemm_tn<double, double, double>(c, ws, N, nq, nx, Qb, N, X, N, d_s, nq, 1.0, 0.0)));
    ST((gemm_nn<double, double>(c, N, nq, nx, -1.0, Qb, N, d_s, nq, 1.0, X, N)));
    return ADCGPU_OK;
  }

  // Cholesky QR twice: X <- X R^{-1}, R = R2 R1 (upper, positive diagonal).
  int cholqr2(double* X, std::vector<double>& Rout) {
    std::vector<double> G, R1((size_t)b * b), Ri((size_t)b * b), Racc((size_t)b * b, 0.0);
    for (int i = 0; i < b; ++i) Racc[(size_t)i * b + i] = 1.0;
    for (int pass = 0; pass < 2; ++pass) {
      ST((gemm_tn<double, double, double>(c, ws, N, b, b, X, N, X, N, d_s, b, 1.0, 0.0)));
      G.resize((size_t)b * b);
      ADC_CUDA(c, cudaMemcpyAsync(G.data(), d_s, sizeof(double) * b * b, cudaMemcpyDeviceToHost, c->stream));
      ADC_CUDA(c, cudaStreamSynchronize(c->stream));
      if (host_cholesky_upper(b, G.data(), R1.data(), 1e-30) >= 0)
        return set_err(c, ADCGPU_EIGEN_FAILED, "block Lanczos breakdown: rank-deficient residual block");
      host_triu_inverse(b, R1.data(), Ri.data());
      ADC_CUDA(c, cudaMemcpyAsync(d_s2, Ri.data(), sizeof(double) * b * b, cudaMemcpyHostToDevice, c->stream));
      ST((gemm_nn<double, double>(c, N, b, b, 1.0, X, N, d_s2, b, 0.0, Tmp, N)));
      ADC_CUDA(c, cudaMemcpyAsync(X, Tmp, sizeof(double) * N * b, cudaMemcpyDeviceToDevice, c->stream));
      // Racc = R1 * Racc
      std::vector<double> nr((size_t)b * b, 0.0);
      for (int j = 0; j < b; ++j)
        for (int i = 0; i < b; ++i) {
          double s = 0.0;
          for (int k = 0; k < b; ++k) s += R1[(size_t)k * b + i] * Racc[(size_t)j * b + k];
          nr[(size_t)j * b + i] = s;
        }
      Racc.swap(nr);
    }
    Rout = Racc;
    return ADCGPU_OK;
  }

  // localro (:1430-1470): Q2 against each vector of Q1, then normalise Q2.
  int localro() {
    ST(project(Q1, b, Q2, b));
    return normalise(Q2, b);
  }

  int run(int orthotype, const double* q0_host, double* tmat_out, double* evals_out, double* ritz_out) {
    nvec = b * ncycles;
    ST(dmalloc(c, (void**)&Qall, sizeof(double) * (size_t)N * nvec));
    ST(dmalloc(c, (void**)&Q1, sizeof(double) * (size_t)N * b));
    ST(dmalloc(c, (void**)&Q2, sizeof(double) * (size_t)N * b));
    ST(dmalloc(c, (void**)&U, sizeof(double) * (size_t)N * b));
    ST(dmalloc(c, (void**)&Tmp, sizeof(double) * (size_t)N * b));
    ST(dmalloc(c, (void**)&d_s, sizeof(double) * (size_t)std::max(b * b, 4096)));
    ST(dmalloc(c, (void**)&d_s2, sizeof(double) * (size_t)std::max(b * b, 4096)));
    ST(dmalloc(c, (void**)&d_part, sizeof(double) * c->nsm * 2 * (size_t)std::max(b, 64)));
    ADC_CUDA(c, cudaMemsetAsync(Q1, 0, sizeof(double) * N * b, c->stream));
    ADC_CUDA(c, cudaMemcpyAsync(Q2, q0_host, sizeof(double) * N * b, cudaMemcpyHostToDevice, c->stream));
    // init_vecs_random: normalise, then modified Gram-Schmidt twice
    ST(normalise(Q2, b));
    for (int pass = 0; pass < 2; ++pass)
      for (int i = 0; i < b; ++i) {
        for (int j = 0; j < i; ++j) ST(project(Q2 + (size_t)j * N, 1, Q2 + (size_t)i * N, 1));
        ST(normalise(Q2 + (size_t)i * N, 1));
      }
    double epmach = 1.0;
    while (1.0 + 0.5 * epmach != 1.0) epmach = 0.5 * epmach;   // machine_precision :927-943
    const double orthlim = std::sqrt(epmach);
    double eps = epmach;
    std::vector<double> T((size_t)nvec * nvec, 0.0), A((size_t)b * b), B((size_t)b * b, 0.0), Bt((size_t)b * b);
    std::vector<std::vector<double>> Aall(ncycles), Ball(ncycles);
    const int nom = ncycles + 2;
    std::vector<double> om((size_t)nom * nom, 0.0), anorm(nom, 0.0), bnorm(nom, 0.0);
    auto OM = [&](int r, int cc) -> double& { return om[(size_t)cc * nom + r]; };
    auto norms = [&](const std::vector<double>& M, double& smax, double& smin) {
      // singular values from the eigenvalues of M^T M
      std::vector<double> G((size_t)b * b), w(b);
      for (int i = 0; i < b; ++i)
        for (int j = 0; j < b; ++j) {
          double s = 0.0;
          for (int k = 0; k < b; ++k) s += M[(size_t)i * b + k] * M[(size_t)j * b + k];
          G[(size_t)j * b + i] = s;
        }
      host_syev(b, G.data(), b, w.data(), nullptr);
      smax = std::sqrt(std::max(w[b - 1], 0.0));
      smin = std::sqrt(std::max(w[0], 0.0));
    };
    for (int j = 1; j <= ncycles; ++j) {
      double* Qj = Qall + (size_t)(j - 1) * b * N;
      ADC_CUDA(c, cudaMemcpyAsync(Qj, Q2, sizeof(double) * N * b, cudaMemcpyDeviceToDevice, c->stream));
      // U = H Q_j - Q_{j-1} B_{j-1}^T   (:1111-1122)
      ST(sigma_fp64(c, b, Q2, N, U, N));
      for (int r = 0; r < b; ++r)
        for (int cc = 0; cc < b; ++cc) Bt[(size_t)cc * b + r] = B[(size_t)r * b + cc];
      ADC_CUDA(c, cudaMemcpyAsync(d_s2, Bt.data(), sizeof(double) * b * b, cudaMemcpyHostToDevice, c->stream));
      ST((gemm_nn<double, double>(c, N, b, b, -1.0, Q1, N, d_s2, b, 1.0, U, N)));
      // A_j = Q_j^T U   (:1124-1127)
      ST((gemm_tn<double, double, double>(c, ws, N, b, b, Q2, N, U, N, d_s, b, 1.0, 0.0)));
      ADC_CUDA(c, cudaMemcpyAsync(A.data(), d_s, sizeof(double) * b * b, cudaMemcpyDeviceToHost, c->stream));
      ADC_CUDA(c, cudaStreamSynchronize(c->stream));
      Aall[j - 1] = A;
      // R = U - Q_j A_j   (:1132-1135), in place in U
      ADC_CUDA(c, cudaMemcpyAsync(d_s2, A.data(), sizeof(double) * b * b, cudaMemcpyHostToDevice, c->stream));
      ST((gemm_nn<double, double>(c, N, b, b, -1.0, Q2, N, d_s2, b, 1.0, U, N)));
      // QR (:1141-1168)
      ST(cholqr2(U, B));
      Ball[j - 1] = B;
      std::swap(Q1, Q2);          // Q1 <- Q_j
      std::swap(Q2, U);           // Q2 <- Q_{j+1}; U becomes scratch
      bool lro = false;
      if (j > 1 && j < ncycles && orthotype == 1) {
        // update_omega (:1530-1639)
        double smax, smin;
        if (j == 2) {
          norms(Aall[0], smax, smin); anorm[1] = smax;
          norms(Ball[0], smax, smin); bnorm[1] = smax;
          norms(Ball[1], smax, smin); bnorm[2] = smax;
          eps = epmach * b * std::sqrt((double)N);
          OM(1, 1) = eps; OM(2, 2) = eps;
          OM(1, 2) = eps / smin; OM(2, 1) = OM(1, 2);
        }
        norms(Aall[j - 1], smax, smin); anorm[j] = smax;
        norms(Ball[j - 1], smax, smin); bnorm[j] = smax;
        const double invssvb = 1.0 / smin;
        OM(j, j + 1) = eps; OM(j + 1, j) = eps; OM(j + 1, j + 1) = eps;
        for (int k = 1; k <= j - 1; ++k) {
          if (k == 1)
            OM(j + 1, k) = bnorm[k + 1] * OM(j, k + 1) + bnorm[j] * OM(j - 1, k) + (anorm[j] + anorm[k]) * OM(j, k);
          else
            OM(j + 1, k) = bnorm[k + 1] * OM(j, k + 1) + bnorm[k] * OM(j, k - 1) + bnorm[j] * OM(j - 1, k) +
                           (anorm[j] + anorm[k]) * OM(j, k);
          OM(j + 1, k) = invssvb * OM(j + 1, k);
          OM(k, j + 1) = OM(j + 1, k);
        }
        for (int k = 1; k <= j - 1; ++k) if (OM(j + 1, k) >= orthlim) lro = true;
        if (lro) {
          // pro_mgs (:1643-1706): Q_j and Q_{j+1} against Q_1..Q_{j-1}
          for (int k = 1; k <= j - 1; ++k) {
            const double* Qk = Qall + (size_t)(k - 1) * b * N;
            ST(project(Qk, b, Q1, b));
            ST(project(Qk, b, Q2, b));
          }
          ST(normalise(Q1, b));
          ST(localro());
          for (int k = 1; k <= j; ++k) { OM(j + 1, k) = eps; OM(j, k) = eps; }
        }
      }
      if (!lro && orthotype == 1) ST(localro());
      // T assembly (:1197-1219)
      int i1 = 0;
      for (int m = (j - 1) * b + 1; m <= j * b; ++m) {
        ++i1;
        const int upper = (j < ncycles) ? (j + 1) * b : j * b;
        int j1 = 0, k1 = 0, k2 = 0;
        for (int n = (j - 1) * b + 1; n <= upper; ++n) {
          ++j1;
          double v;
          if (j1 <= b) { ++k1; v = A[(size_t)(i1 - 1) * b + (k1 - 1)]; }
          else { ++k2; v = B[(size_t)(i1 - 1) * b + (k2 - 1)]; }
          T[(size_t)(m - 1) * nvec + (n - 1)] = v;
          T[(size_t)(n - 1) * nvec + (m - 1)] = v;
        }
      }
    }
    if (tmat_out) std::memcpy(tmat_out, T.data(), sizeof(double) * T.size());
    if (evals_out && !ritz_out) {
      // diagmat_banded with eigenvalues only: band reduction, O(nvec^2 b)
      if (!host_sbev_values(nvec, b, T.data(), nvec, evals_out))
        return set_err(c, ADCGPU_EIGEN_FAILED, "diagonalisation of the Lanczos T matrix failed");
    } else if (evals_out || ritz_out) {
      // diagmat_banded: dsbev('V','L') on the lower band (kd = b)
      std::vector<double> Tb((size_t)nvec * nvec, 0.0), w(nvec), E;
      for (int cc = 0; cc < nvec; ++cc)
        for (int r = cc; r < std::min(nvec, cc + b + 1); ++r) {
          double x = T[(size_t)cc * nvec + r];
          Tb[(size_t)cc * nvec + r] = x;
          Tb[(size_t)r * nvec + cc] = x;
        }
      if (ritz_out) E.resize((size_t)nvec * nvec);
      if (!host_syev(nvec, Tb.data(), nvec, w.data(), ritz_out ? E.data() : nullptr))
        return set_err(c, ADCGPU_EIGEN_FAILED, "diagonalisation of the Lanczos T matrix failed");
      if (evals_out) std::memcpy(evals_out, w.data(), sizeof(double) * nvec);
      if (ritz_out) {
        // ritzvecs_incore: Q E, columns normalised
        double* d_E = nullptr;
        double* d_R = nullptr;
        ST(dmalloc(c, (void**)&d_E, sizeof(double) * E.size()));
        ST(dmalloc(c, (void**)&d_R, sizeof(double) * (size_t)N * nvec));
        ADC_CUDA(c, cudaMemcpyAsync(d_E, E.data(), sizeof(double) * E.size(), cudaMemcpyHostToDevice, c->stream));
        const int PC = 128, QC = 16;
        for (int q0 = 0; q0 < nvec; q0 += QC) {
          int qn = std::min(QC, nvec - q0);
          for (int p0 = 0; p0 < nvec; p0 += PC) {
            int pn = std::min(PC, nvec - p0);
            ST((gemm_nn<double, double>(c, N, pn, qn, 1.0, Qall + (size_t)p0 * N, N, d_E + (size_t)q0 * nvec + p0,
                                        nvec, p0 == 0 ? 0.0 : 1.0, d_R + (size_t)q0 * N, N)));
          }
        }
        dfree(c, d_part, 0);   // grow the norm partials to nvec columns
        d_part = nullptr;
        ST(dmalloc(c, (void**)&d_part, sizeof(double) * c->nsm * 2 * (size_t)nvec));
        std::vector<double> nr;
        ST(colnorms(d_R, nvec, nr));
        for (auto& v : nr) v = 1.0 / v;
        double* d_sc = nullptr;
        ST(dmalloc(c, (void**)&d_sc, sizeof(double) * nvec));
        ADC_CUDA(c, cudaMemcpyAsync(d_sc, nr.data(), sizeof(double) * nvec, cudaMemcpyHostToDevice, c->stream));
        k_scale_cols<<<c->nsm * 4, 256, 0, c->stream>>>(N, nvec, d_R, N, d_sc); ADC_COUNT_LAUNCH();
        ADC_CUDA(c, cudaMemcpyAsync(ritz_out, d_R, sizeof(double) * (size_t)N * nvec, cudaMemcpyDeviceToHost, c->stream));
        ADC_CUDA(c, cudaStreamSynchronize(c->stream));
        dfree(c, d_E, 0);
        dfree(c, d_R, 0);
        dfree(c, d_sc, 0);
      }
    }
    return ADCGPU_OK;
  }
};

}  // namespace adcgpu

extern "C" int adcgpu_block_lanczos(adcgpu_ctx* h, int lmain, int ncycles, int orthotype, const double* q0,
                                    double* tmat, double* evals, double* ritz) {
  using namespace adcgpu;
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c) return ADCGPU_BAD_INPUT;
  cudaSetDevice(c->device);
  if (!c->have_matrix) return set_err(c, ADCGPU_NO_MATRIX, "build the matrix first");
  if (c->precision != ADCGPU_FP64 && c->precision != ADCGPU_MIXED) return ADCGPU_BAD_INPUT;
  if (lmain <= 0 || ncycles <= 0 || !q0 || (orthotype != 0 && orthotype != 1))
    return set_err(c, ADCGPU_BAD_INPUT, "lmain, ncycles, q0 and orthotype in {0,1} required");
  if ((int64_t)lmain * ncycles > mat_dim(c)) return set_err(c, ADCGPU_BAD_INPUT, "nvec exceeds the dimension");
  LanczosGPU L;
  L.c = c; L.N = mat_dim(c); L.b = lmain; L.ncycles = ncycles;
  return L.run(orthotype, q0, tmat, evals, ritz);
}
