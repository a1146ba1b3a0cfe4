// Block Davidson on the GPU: davdiag_block (block_davidson.f90:33-145) and
// run_block_davidson (:690-774) with the same parameters, guess vectors,
// preconditioners (dpr :1288, olsen :1346), deflation (:1147-1222), collapse
// rule (:1109-1116), convergence count (:1073-1083) and output order
// (wreigenpairs :1469-1532).
//
// Two algorithmic differences, both exact in exact arithmetic:
//  * W = H V is cached: each iteration multiplies only the new block (the
//    reference recomputes all currdim columns, :855).  After a collapse the
//    Ritz block's products W Y are reused; after a deflation the collapsed
//    block is projected against the converged vectors and re-multiplied.
//  * Orthonormalisation is block classical Gram-Schmidt applied twice plus
//    Cholesky QR applied twice on the new block, instead of Householder QR
//    of the whole subspace (:1448-1454): the old columns are already
//    orthonormal and stay fixed, which is what makes W reusable.
//
// T is the storage/compute type of the N-length vectors (double for the
// FP64 path, float for the mixed path).  The Rayleigh matrix, its
// eigendecomposition, residual norms and all convergence decisions are FP64.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "dense.h"
#include "internal.h"
#include "davidson.h"

namespace adcgpu {

namespace {

__global__ void k_fill_random(double* x, int64_t n, uint64_t seed) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(i + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    x[i] = ((double)(z >> 11) * (1.0 / 9007199254740992.0)) - 0.5;
  }
}
__global__ void k_fill_random_f(float* x, int64_t n, uint64_t seed) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(i + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    x[i] = (float)(((double)(z >> 11) * (1.0 / 9007199254740992.0)) - 0.5);
  }
}

template <typename T> void fill_random(Ctx* c, T* x, int64_t n, uint64_t seed);
template <> void fill_random<double>(Ctx* c, double* x, int64_t n, uint64_t seed) {
  k_fill_random<<<c->nsm * 4, 256, 0, c->stream>>>(x, n, seed); ADC_COUNT_LAUNCH();
}
template <> void fill_random<float>(Ctx* c, float* x, int64_t n, uint64_t seed) {
  k_fill_random_f<<<c->nsm * 4, 256, 0, c->stream>>>(x, n, seed); ADC_COUNT_LAUNCH();
}

template <typename T> int sigma_t(Ctx* c, int m, const T* V, int64_t ldv, T* W, int64_t ldw);
template <> int sigma_t<double>(Ctx* c, int m, const double* V, int64_t ldv, double* W, int64_t ldw) {
  return sigma_fp64(c, m, V, ldv, W, ldw);
}
template <> int sigma_t<float>(Ctx* c, int m, const float* V, int64_t ldv, float* W, int64_t ldw) {
  return sigma_fp32(c, m, V, ldv, W, ldw);
}

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace


template <typename T>
struct DavidsonGPU {
  Ctx* c;
  int64_t N;
  int nstates, blocksize, maxvec, niter, ipre;
  bool ldeflate;
  double tol;
  // lower-precision phases of the mixed ladder: stop (not converged) when
  // the largest residual of the unconverged roots has not fallen by 10 %
  // within this many iterations (0: never), i.e. at the phase's floor
  int stall_iters = 0;
  const T* hii;            // device diagonal in T
  const MlpPrecond* mlp = nullptr;
  // device arrays
  T *V = nullptr, *W = nullptr, *X = nullptr, *R = nullptr, *WY = nullptr, *Tn = nullptr, *Tmp = nullptr;
  T* Cv = nullptr;         // deflated (converged) vectors
  double *d_lam = nullptr, *d_small = nullptr, *d_small2 = nullptr;
  Workspace ws;
  std::vector<double> Rm;  // host Rayleigh matrix, maxvec x maxvec col-major
  std::vector<double> Cval;
  int nconv_store = 0;
  int64_t nmult = 0;
  double sigma_s = 0.0;
  size_t bytes_v = 0;

  int alloc() {
    bytes_v = sizeof(T) * (size_t)N;
    ST(dmalloc(c, (void**)&V, bytes_v * maxvec));
    ST(dmalloc(c, (void**)&W, bytes_v * maxvec));
    ST(dmalloc(c, (void**)&X, bytes_v * blocksize));
    ST(dmalloc(c, (void**)&R, bytes_v * blocksize));
    ST(dmalloc(c, (void**)&WY, bytes_v * blocksize));
    ST(dmalloc(c, (void**)&Tn, bytes_v * blocksize));
    ST(dmalloc(c, (void**)&Tmp, bytes_v * 2 * blocksize));   // orthonormalise handles up to 2 blocks
    ST(dmalloc(c, (void**)&Cv, bytes_v * std::max(1, nstates)));
    ST(dmalloc(c, (void**)&d_lam, sizeof(double) * blocksize));
    ST(dmalloc(c, (void**)&d_small, sizeof(double) * (size_t)maxvec * maxvec));
    ST(dmalloc(c, (void**)&d_small2, sizeof(double) * (size_t)maxvec * maxvec));
    ADC_CUDA(c, cudaMemsetAsync(V, 0, bytes_v * maxvec, c->stream));
    Rm.assign((size_t)maxvec * maxvec, 0.0);
    return ADCGPU_OK;
  }
  void release() {
    T* ps[] = {V, W, X, R, WY, Tn, Tmp, Cv};
    for (T* p : ps) dfree(c, p);
    dfree(c, d_lam);
    dfree(c, d_small);
    dfree(c, d_small2);
    V = W = X = R = WY = Tn = Tmp = Cv = nullptr;
    d_lam = d_small = d_small2 = nullptr;
    ws.release();
  }
  ~DavidsonGPU() { release(); }

  T* col(T* base, int j) { return base + (size_t)j * N; }

  int sigma_cols(int j0, int j1) {
    if (j1 <= j0) return ADCGPU_OK;
    double t0 = now_s();
    ST(sigma_t<T>(c, j1 - j0, col(V, j0), N, col(W, j0), N));
    ADC_CUDA(c, cudaStreamSynchronize(c->stream));
    sigma_s += now_s() - t0;
    nmult += j1 - j0;
    return ADCGPU_OK;
  }

  // S(p x q) = A^T B into d_small; copied to host h (p x q col-major).
  int tn_to_host(int p, int q, const T* A, const T* B, std::vector<double>& h) {
    ST((gemm_tn<T, double, double>(c, ws, N, p, q, A, N, B, N, d_small, p, 1.0, 0.0)));
    h.resize((size_t)p * q);
    ADC_CUDA(c, cudaMemcpyAsync(h.data(), d_small, sizeof(double) * p * q, cudaMemcpyDeviceToHost, c->stream));
    ADC_CUDA(c, cudaStreamSynchronize(c->stream));
    return ADCGPU_OK;
  }

  // Tcols -= Q (Q^T Tcols), Q = ncq columns at Qb, nt columns at Tb.
  int project_out(const T* Qb, int ncq, T* Tb, int nt) {
    if (ncq <= 0 || nt <= 0) return ADCGPU_OK;
    ST((gemm_tn<T, double, double>(c, ws, N, ncq, nt, Qb, N, Tb, N, d_small, ncq, 1.0, 0.0)));
    ST((gemm_nn<T, double>(c, N, ncq, nt, T(-1), Qb, N, d_small, ncq, T(1), Tb, N)));
    return ADCGPU_OK;
  }

  // Orthonormalise nt columns at Tb against Q1 (nq1 cols), Q2 (nq2 cols)
  // and among themselves: block CGS twice, then Cholesky QR twice on the
  // column-scaled Gram matrix.  A column whose norm drops below 1e-10 of its
  // norm before projection (numerically inside the span) is replaced by a
  // random vector, as Householder QR would complete the basis.
  int orthonormalise(T* Tb, int nt, const T* Q1, int nq1, const T* Q2, int nq2, int* nreplaced) {
    *nreplaced = 0;
    if (nt > 2 * blocksize || nt > maxvec) return set_err(c, ADCGPU_BAD_INPUT, "orthonormalise: block too wide");
    std::vector<double> G, Gs((size_t)nt * nt), Rc((size_t)nt * nt), Ri((size_t)nt * nt), n0(nt), sc(nt);
    ST(tn_to_host(nt, nt, Tb, Tb, G));
    for (int j = 0; j < nt; ++j) n0[j] = std::sqrt(std::max(G[(size_t)j * nt + j], 0.0));
    for (int attempt = 0; attempt < nt + 3; ++attempt) {
      for (int pass = 0; pass < 2; ++pass) {
        ST(project_out(Q2, nq2, Tb, nt));
        ST(project_out(Q1, nq1, Tb, nt));
      }
      bool ok = true;
      for (int pass = 0; pass < 2 && ok; ++pass) {
        ST(tn_to_host(nt, nt, Tb, Tb, G));
        int bad = -1;
        for (int j = 0; j < nt && bad < 0; ++j) {
          double nj = std::sqrt(std::max(G[(size_t)j * nt + j], 0.0));
          if (!(nj > 0.0) || (pass == 0 && nj <= 1e-10 * n0[j])) bad = j;
          else sc[j] = 1.0 / nj;
        }
        if (bad < 0) {
          for (int j = 0; j < nt; ++j)
            for (int i = 0; i < nt; ++i) Gs[(size_t)j * nt + i] = G[(size_t)j * nt + i] * sc[i] * sc[j];
          bad = host_cholesky_upper(nt, Gs.data(), Rc.data(), 1e-12);
        }
        if (bad >= 0) {
          fill_random<T>(c, Tb + (size_t)bad * N, N, 0xC0FFEEull + 7919ull * (attempt + 1) + bad);
          n0[bad] = 1.0;
          ++*nreplaced;
          ok = false;
          break;
        }
        // R = Rs S^{-1}  =>  R^{-1} = S Rs^{-1}
        host_triu_inverse(nt, Rc.data(), Ri.data());
        for (int j = 0; j < nt; ++j)
          for (int i = 0; i < nt; ++i) Ri[(size_t)j * nt + i] *= sc[i];
        ADC_CUDA(c, cudaMemcpyAsync(d_small2, Ri.data(), sizeof(double) * nt * nt, cudaMemcpyHostToDevice, c->stream));
        ST((gemm_nn<T, double>(c, N, nt, nt, T(1), Tb, N, d_small2, nt, T(0), Tmp, N)));
        ADC_CUDA(c, cudaMemcpyAsync(Tb, Tmp, bytes_v * nt, cudaMemcpyDeviceToDevice, c->stream));
      }
      if (ok) return ADCGPU_OK;
    }
    return set_err(c, ADCGPU_EIGEN_FAILED, "orthonormalisation failed: new block linearly dependent");
  }

  // initvec_ondiag (block_davidson.f90:463-532): unit vectors at the
  // blocksize smallest |hii| in heapsort order.
  int guess_ondiag(const std::vector<double>& hdiag) {
    (void)hdiag;
    const std::vector<int64_t>& indx = diag_order(c);   // heapsort of |hii|, from the build
    if ((int64_t)indx.size() != N) return set_err(c, ADCGPU_NO_MATRIX, "diagonal order missing");
    const T one = T(1);
    for (int i = 0; i < blocksize; ++i) {
      int64_t k = indx[i] - 1;
      ADC_CUDA(c, cudaMemcpyAsync(V + (size_t)i * N + k, &one, sizeof(T), cudaMemcpyHostToDevice, c->stream));
    }
    ADC_CUDA(c, cudaStreamSynchronize(c->stream));
    return ADCGPU_OK;
  }

  // initvec_subdiag (:293-459): eigenvectors of H on the subdim lowest-hii
  // configurations.
  int guess_subdiag(const std::vector<double>& hdiag, int subdim);

  // initvec_adc1 (:246-289): the blocksize lowest eigenvectors of the ADC(1)
  // singles matrix (adc1_guessvecs, guessvecs.f90:9-84) in the singles rows
  // of V, the doubles rows zero.
  int guess_adc1() {
    const int n1 = (int)c->geom.n1;
    if (blocksize > n1) return set_err(c, ADCGPU_BAD_INPUT, "ADC(1) guess: blocksize exceeds the singles space");
    double* d_M = nullptr;
    ST(dmalloc(c, (void**)&d_M, sizeof(double) * (size_t)n1 * n1));
    int st = build_adc1_matrix(c, d_M);
    std::vector<double> M((size_t)n1 * n1), w(n1), Vs((size_t)n1 * n1);
    if (!st) st = d2h(c, M.data(), d_M, sizeof(double) * M.size()) == cudaSuccess ? ADCGPU_OK : ADCGPU_CUDA_ERROR;
    dfree(c, d_M, 0);
    if (st) return set_err(c, st, "ADC(1) guess: matrix");
    if (!host_syev(n1, M.data(), n1, w.data(), Vs.data()))
      return set_err(c, ADCGPU_EIGEN_FAILED, "ADC(1) matrix diagonalisation failed");
    std::vector<T> colbuf(n1);
    for (int i = 0; i < blocksize; ++i) {
      for (int j = 0; j < n1; ++j) colbuf[j] = (T)Vs[(size_t)i * n1 + j];
      ADC_CUDA(c, h2d(c, V + (size_t)i * N, colbuf.data(), sizeof(T) * n1));
    }
    return ADCGPU_OK;
  }

  // Guess from given vectors (device, ncols columns, T type): orthonormalised.
  int guess_vectors(const T* G, int ncols) {
    int nb = std::min(ncols, blocksize);
    ADC_CUDA(c, cudaMemcpyAsync(V, G, bytes_v * nb, cudaMemcpyDeviceToDevice, c->stream));
    if (nb < blocksize) fill_random<T>(c, V + (size_t)nb * N, (int64_t)N * (blocksize - nb), 0xABCDEFull);
    int nrep;
    ST(orthonormalise(V, blocksize, nullptr, 0, nullptr, 0, &nrep));
    return ADCGPU_OK;
  }

  // optional trace of (residual, Ritz vector, Ritz value) of the first
  // nstates roots every trace_every iterations (training data of the MLP)
  double *tr_R = nullptr, *tr_X = nullptr, *tr_lam = nullptr;
  int tr_every = 0, tr_max = 0, tr_n = 0;
  int64_t nmult_ref = 0;       // sum of currdim over iterations (reference hxvec columns)
  double max_res = 0.0;        // largest residual norm among the returned roots
  std::vector<double> Cnorm;   // residual norms of the deflated roots

  // evecs_dev: capacity ncap >= nstates columns; receives the nstates roots
  // (ascending) followed by the other current Ritz vectors; *nout = count.
  int run(const std::vector<double>& hdiag, int guess_kind, int guessdim, const T* guess_dev, int nguess,
          std::vector<double>& evals_out, T* evecs_dev, int ncap, int* nout, int* iters_out, int* nconv_out) {
    ST(alloc());
    if (guess_kind == 1) ST(guess_subdiag(hdiag, guessdim));
    else if (guess_kind == 2) ST(guess_vectors(guess_dev, nguess));
    else if (guess_kind == 3) ST(guess_adc1());
    else ST(guess_ondiag(hdiag));

    int currdim = blocksize, bs_curr = blocksize, maxvec_curr = maxvec, nstates_curr = nstates;
    int nconv = 0, nconv_prev = 0, nW = 0, iters = 0;
    double stall_best = 1e300;
    int stall_since = 0;
    std::vector<double> val(maxvec), vec((size_t)maxvec * maxvec), lam(blocksize), norm(blocksize), Y;
    std::vector<double> S;
    for (int k = 1; k <= niter; ++k) {
      iters = k;
      nmult_ref += currdim;
      // hxvec: only the columns without a product
      ST(sigma_cols(nW, currdim));
      // calcrmat: new columns of the Rayleigh matrix (upper triangle)
      if (nW < currdim) {
        ST(tn_to_host(currdim, currdim - nW, V, col(W, nW), S));
        for (int j = nW; j < currdim; ++j)
          for (int i = 0; i <= j; ++i) Rm[(size_t)j * maxvec + i] = S[(size_t)(j - nW) * currdim + i];
      }
      nW = currdim;
      // diagrmat (dsyev 'U')
      if (!host_syev(currdim, Rm.data(), maxvec, val.data(), vec.data()))
        return set_err(c, ADCGPU_EIGEN_FAILED, "Rayleigh matrix diagonalisation failed");
      Y.assign((size_t)currdim * bs_curr, 0.0);
      for (int j = 0; j < bs_curr; ++j) {
        lam[j] = val[j];
        std::memcpy(&Y[(size_t)j * currdim], &vec[(size_t)j * currdim], sizeof(double) * currdim);
      }
      ADC_CUDA(c, cudaMemcpyAsync(d_small, Y.data(), sizeof(double) * currdim * bs_curr, cudaMemcpyHostToDevice, c->stream));
      ADC_CUDA(c, cudaMemcpyAsync(d_lam, lam.data(), sizeof(double) * bs_curr, cudaMemcpyHostToDevice, c->stream));
      // calcritzvec, calcres
      ST((gemm_nn<T, double>(c, N, currdim, bs_curr, T(1), V, N, d_small, currdim, T(0), X, N)));
      ST((gemm_nn<T, double>(c, N, currdim, bs_curr, T(1), W, N, d_small, currdim, T(0), WY, N)));
      std::vector<double> n2(bs_curr);
      ST(residuals<T>(c, ws, N, bs_curr, X, WY, N, d_lam, R, n2.data()));
      for (int i = 0; i < bs_curr; ++i) norm[i] = std::sqrt(n2[i]);
      if (tr_every > 0 && (k - 1) % tr_every == 0 && tr_n < tr_max && nstates_curr == nstates) {
        const size_t blk = sizeof(T) * (size_t)N * nstates;
        ADC_CUDA(c, cudaMemcpyAsync(tr_R + (size_t)tr_n * N * nstates, R, blk, cudaMemcpyDeviceToHost, c->stream));
        ADC_CUDA(c, cudaMemcpyAsync(tr_X + (size_t)tr_n * N * nstates, X, blk, cudaMemcpyDeviceToHost, c->stream));
        for (int i = 0; i < nstates; ++i) tr_lam[(size_t)tr_n * nstates + i] = lam[i];
        ADC_CUDA(c, cudaStreamSynchronize(c->stream));
        ++tr_n;
      }
      if (!ldeflate) nconv = 0;
      for (int i = 0; i < nstates_curr; ++i)
        if (norm[i] < tol) ++nconv;
      if (nconv == nstates) break;
      if (stall_iters > 0) {
        double cur = 0.0;
        for (int i = 0; i < nstates_curr; ++i)
          if (!(norm[i] < tol)) cur = std::max(cur, norm[i]);
        if (cur < 0.9 * stall_best) { stall_best = cur; stall_since = 0; }
        else if (++stall_since >= stall_iters) break;
      }

      // subspace_expansion
      const bool deflated = ldeflate && nconv > nconv_prev;
      if (deflated) {
        // deflate (:1147-1222): converged roots to the tail, same swaps
        std::vector<int> convmap;
        for (int i = 0; i < bs_curr; ++i) if (norm[i] < tol) convmap.push_back(i);
        for (int i = 1; i <= nconv - nconv_prev; ++i) {
          int indx = blocksize - nconv_prev - i;   // 0-based column of the active block tail
          int src = convmap[i - 1];
          // store the converged vector and value
          ADC_CUDA(c, cudaMemcpyAsync(col(Cv, nconv_store), col(X, src), bytes_v, cudaMemcpyDeviceToDevice, c->stream));
          Cval.push_back(lam[src]);
          Cnorm.push_back(norm[src]);
          ++nconv_store;
          if (indx != src) {
            ADC_CUDA(c, cudaMemcpyAsync(col(X, src), col(X, indx), bytes_v, cudaMemcpyDeviceToDevice, c->stream));
            ADC_CUDA(c, cudaMemcpyAsync(col(R, src), col(R, indx), bytes_v, cudaMemcpyDeviceToDevice, c->stream));
            ADC_CUDA(c, cudaMemcpyAsync(col(WY, src), col(WY, indx), bytes_v, cudaMemcpyDeviceToDevice, c->stream));
            std::swap(lam[src], lam[indx]);
            std::swap(norm[src], norm[indx]);
          }
        }
        const int dn = nconv - nconv_prev;
        bs_curr -= dn; maxvec_curr -= dn; nstates_curr -= dn; currdim -= dn;
        ADC_CUDA(c, cudaMemcpyAsync(d_lam, lam.data(), sizeof(double) * bs_curr, cudaMemcpyHostToDevice, c->stream));
      }
      bool lcollapse = !(currdim <= maxvec_curr - bs_curr) || deflated;
      int ilast;
      if (lcollapse) {
        ADC_CUDA(c, cudaMemcpyAsync(V, X, bytes_v * bs_curr, cudaMemcpyDeviceToDevice, c->stream));
        ADC_CUDA(c, cudaMemcpyAsync(W, WY, bytes_v * bs_curr, cudaMemcpyDeviceToDevice, c->stream));
        ilast = bs_curr;
        nW = bs_curr;
        std::fill(Rm.begin(), Rm.end(), 0.0);
        for (int i = 0; i < bs_curr; ++i) Rm[(size_t)i * maxvec + i] = lam[i];
      } else {
        ilast = currdim;
      }
      // new vectors from the residuals
      T* Tb = col(V, ilast);
      if (ipre == ADCGPU_PRECON_OLSEN) {
        ST((precond_olsen<T, T>(c, ws, N, bs_curr, X, R, N, d_lam, hii, Tb, N, nullptr)));
      } else if (ipre == ADCGPU_PRECON_FOLD) {
        ST((precond_fold<T>(c, ws, N, bs_curr, R, N, d_lam, hii, Tb, N, Tmp, N)));
        nmult += bs_curr;   // the folding sigma product
      } else if (ipre == ADCGPU_PRECON_MLP && c->mlp) {
        MlpPrecond none;
        ST(mlp_apply(c, mlp ? *mlp : none, N, bs_curr, R, X, d_lam, hii, Tb));
      } else {
        ST((precond_dpr<T, T>(c, N, bs_curr, R, N, d_lam, hii, Tb, N)));
      }
      int nrep = 0;
      if (deflated) {
        // subspace_projection of the whole collapsed subspace, then a fresh
        // orthonormal basis and fresh products (:1226-1284, :1423-1465)
        ST(orthonormalise(V, 2 * bs_curr, nullptr, 0, Cv, nconv_store, &nrep));
        nW = 0;
        std::fill(Rm.begin(), Rm.end(), 0.0);
      } else {
        ST(orthonormalise(Tb, bs_curr, V, ilast, (ldeflate && nconv_store > 0) ? Cv : nullptr,
                          (ldeflate ? nconv_store : 0), &nrep));
        if (lcollapse) {
          // Rayleigh block of the kept Ritz vectors from their products
          ST(tn_to_host(bs_curr, bs_curr, V, W, S));
          for (int j = 0; j < bs_curr; ++j)
            for (int i = 0; i <= j; ++i) Rm[(size_t)j * maxvec + i] = S[(size_t)j * bs_curr + i];
        }
      }
      currdim = lcollapse ? 2 * bs_curr : currdim + bs_curr;
      nconv_prev = nconv;
    }
    // wreigenpairs: converged-and-deflated roots join the current ones
    std::vector<double> ev(nstates);
    std::vector<int> src_col(nstates);   // >= 0: X column; < 0: -(1+Cv column)
    for (int i = 0; i < nstates_curr; ++i) { ev[i] = lam[i]; src_col[i] = i; }
    for (int t = 0; t < nconv_store && nstates_curr + t < nstates; ++t) {
      ev[nstates_curr + t] = Cval[t];
      src_col[nstates_curr + t] = -(1 + t);
    }
    std::vector<int64_t> indx;
    if (nstates > 1) host_heapsort_index(nstates, ev.data(), indx);
    else indx.assign(1, 1);
    evals_out.resize(nstates);
    max_res = 0.0;
    for (int i = 0; i < nstates_curr; ++i) max_res = std::max(max_res, norm[i]);
    for (double v : Cnorm) max_res = std::max(max_res, v);
    int nw = 0;
    for (int i = 0; i < nstates; ++i) {
      int k = (int)indx[i] - 1;
      evals_out[i] = ev[k];
      if (evecs_dev) {
        const T* src = src_col[k] >= 0 ? col(X, src_col[k]) : col(Cv, -src_col[k] - 1);
        ADC_CUDA(c, cudaMemcpyAsync(evecs_dev + (size_t)i * N, src, bytes_v, cudaMemcpyDeviceToDevice, c->stream));
        ++nw;
      }
    }
    // the remaining current Ritz vectors (useful as a warm start)
    for (int i = nstates_curr; evecs_dev && i < bs_curr && nw < ncap; ++i, ++nw)
      ADC_CUDA(c, cudaMemcpyAsync(evecs_dev + (size_t)nw * N, col(X, i), bytes_v, cudaMemcpyDeviceToDevice, c->stream));
    if (nout) *nout = nw;
    ADC_CUDA(c, cudaStreamSynchronize(c->stream));
    *iters_out = iters;
    *nconv_out = nconv;
    return nconv == nstates ? ADCGPU_OK : ADCGPU_NOT_CONVERGED;
  }
};

// ---------------------------------------------------------------------------
// initvec_subdiag: the H sub-block on the subdim lowest-hii configurations
// is gathered on the device, diagonalised on the host, and its lowest
// blocksize eigenvectors scattered into V.
// ---------------------------------------------------------------------------
namespace {

__global__ void k_gather_sub(GeomDev g, const double* __restrict__ A, const double* __restrict__ Bt,
                             const uint2* __restrict__ desc, const int64_t* __restrict__ sub, int m,
                             double* __restrict__ Hs) {
  // Hs(i,j) for i != j; the diagonal is filled on the host
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)m * m;
       t += (int64_t)gridDim.x * blockDim.x) {
    int i = (int)(t % m), j = (int)(t / m);
    int64_t p = sub[i], q = sub[j];
    double v = 0.0;
    if (p != q) {
      if (p < g.n1 && q < g.n1) v = A[p * g.n1 + q];
      else if (p < g.n1 || q < g.n1) {
        int64_t s = p < g.n1 ? p : q, dd = (p < g.n1 ? q : p) - g.n1;
        Double r = decode_double(g, dd);
        // storage row of the double (class 2 is stored hole-outer)
        int64_t rw = r.cls == 1 ? g.start[1] + (int64_t)r.kp * g.npair_v + pair_index(r.ap, r.bp, g.nv) : dd;
        const int64_t L = g.len[r.cls];
        const double* row = Bt + g.off[r.cls] + (rw - g.start[r.cls]) * L;
        for (int e = 0; e < L; ++e)
          if (entry_single(g, r, e) == s) { v = row[e]; break; }
      }
    }
    Hs[t] = v;
  }
}

}  // namespace

template <typename T>
int DavidsonGPU<T>::guess_subdiag(const std::vector<double>& hdiag, int subdim) {
  if (c->direct)
    return set_err(c, ADCGPU_UNSUPPORTED, "initvec_subdiag reads the stored coupling block; the direct path has none");
  if (subdim > N) subdim = (int)N;
  std::vector<int64_t> indx;
  host_heapsort_index(N, hdiag.data(), indx);
  while (subdim < N && std::fabs(hdiag[indx[subdim - 1] - 1] - hdiag[indx[subdim] - 1]) < 1e-6) ++subdim;
  if (subdim < blocksize) subdim = std::min<int64_t>(N, blocksize);
  std::vector<int64_t> sub(subdim);
  for (int i = 0; i < subdim; ++i) sub[i] = indx[i] - 1;
  int64_t* d_sub = nullptr;
  double* d_H = nullptr;
  ST(dmalloc(c, (void**)&d_sub, sizeof(int64_t) * subdim));
  ST(dmalloc(c, (void**)&d_H, sizeof(double) * (size_t)subdim * subdim));
  ADC_CUDA(c, cudaMemcpyAsync(d_sub, sub.data(), sizeof(int64_t) * subdim, cudaMemcpyHostToDevice, c->stream));
  k_gather_sub<<<c->nsm * 4, 256, 0, c->stream>>>(to_dev(c->geom), c->d_A, c->d_Bt, nullptr, d_sub,
                                               subdim, d_H); ADC_COUNT_LAUNCH();
  std::vector<double> H((size_t)subdim * subdim), w(subdim), Vs((size_t)subdim * subdim);
  ADC_CUDA(c, cudaMemcpyAsync(H.data(), d_H, sizeof(double) * H.size(), cudaMemcpyDeviceToHost, c->stream));
  ADC_CUDA(c, cudaStreamSynchronize(c->stream));
  dfree(c, d_sub, 0);
  dfree(c, d_H, 0);
  for (int i = 0; i < subdim; ++i) H[(size_t)i * subdim + i] = hdiag[sub[i]];
  if (!host_syev(subdim, H.data(), subdim, w.data(), Vs.data()))
    return set_err(c, ADCGPU_EIGEN_FAILED, "subspace Hamiltonian diagonalisation failed");
  std::vector<T> colbuf(N);
  for (int i = 0; i < blocksize; ++i) {
    std::fill(colbuf.begin(), colbuf.end(), T(0));
    for (int j = 0; j < subdim; ++j) colbuf[sub[j]] = (T)Vs[(size_t)i * subdim + j];
    ADC_CUDA(c, h2d(c, V + (size_t)i * N, colbuf.data(), bytes_v));
  }
  return ADCGPU_OK;
}

template struct DavidsonGPU<double>;
template struct DavidsonGPU<float>;

// ---------------------------------------------------------------------------
// Driver used by the C ABI.
//   FP64  : one FP64 Davidson (the plain drop-in path).
//   MIXED : a precision ladder, each phase warm-started with the previous
//           phase's block of Ritz vectors:
//             1. BF16 matrix values, FP32 vectors, to residual tol_bf16
//             2. FP32 matrix values, FP32 vectors, to residual tol_fp32
//             3. FP64 refinement to davtol: the FP64 residual norm decides
//           Rayleigh-Ritz, Gram-Schmidt and residual norms are FP64 in every
//           phase (davidson.cu DavidsonGPU).
// ---------------------------------------------------------------------------
int davidson_solve(Ctx* c, const adcgpu_dav_params* p, double* evals, double* evecs, adcgpu_dav_info* info,
                   const MlpPrecond* mlp) {
  const double t_start = now_s();
  const int64_t N = mat_dim(c);
  int nstates = p->davstates;
  if (nstates <= 0 || nstates > N) return set_err(c, ADCGPU_BAD_INPUT, "davstates");
  if (c->cvs) {
    // the CVS matrix is FP64 with the reference's own preconditioners and guess
    if (p->precision != ADCGPU_FP64) return set_err(c, ADCGPU_UNSUPPORTED, "CVS matrix: FP64 iterations only");
    if (p->precon != ADCGPU_PRECON_DPR && p->precon != ADCGPU_PRECON_OLSEN)
      return set_err(c, ADCGPU_UNSUPPORTED, "CVS matrix: DPR or Olsen preconditioner");
    if (p->lsubdiag) return set_err(c, ADCGPU_UNSUPPORTED, "CVS matrix: initvec_ondiag guess");
  }
  int blocksize = p->dmain > 0 ? p->dmain : std::max(nstates + 5, 2 * nstates);
  int maxvec = p->maxsubdim >= 0 ? p->maxsubdim : 4 * blocksize;
  {
    float ftmp = (float)maxvec / (float)blocksize;     // davinitialise :203-205
    maxvec = (int)std::floor(ftmp) * blocksize;
  }
  if (blocksize > N || maxvec < 2 * blocksize || maxvec > N)
    return set_err(c, ADCGPU_BAD_INPUT, "blocksize/maxvec incompatible with the matrix dimension");
  std::vector<double> hdiag(N);
  ADC_CUDA(c, d2h(c, hdiag.data(), c->d_diag, sizeof(double) * N));
  // lsubdiag: 1 initvec_subdiag, 2 initvec_adc1, 0 initvec_ondiag
  const int guess_kind = p->lsubdiag == 2 ? 3 : (p->lsubdiag ? 1 : 0);
  const int precon64 = p->precon;
  int st = ADCGPU_OK;
  adcgpu_dav_info inf{};
  std::vector<double> ev;
  double* out64 = nullptr;
  ST(dmalloc(c, (void**)&out64, sizeof(double) * (size_t)N * blocksize));
  if (p->precision == ADCGPU_MIXED) {
    if (c->precision != ADCGPU_MIXED) { dfree(c, out64, 0); return set_err(c, ADCGPU_BAD_INPUT, "matrix was not built for MIXED"); }
    const double tol_b = p->tol_bf16 == 0.0 ? 1e-2 : p->tol_bf16;
    // the folded preconditioner makes FP64 iterations cheap and few, so it
    // hands over earlier
    const double tol_f = p->tol_fp32 != 0.0 ? p->tol_fp32 : (p->precon == ADCGPU_PRECON_FOLD ? 1e-5 : 5e-6);
    // Deflation (locking converged roots, block_davidson.f90:1147-1222) is
    // kept for the reference preconditioners.  With the folded one it lost
    // roots: on 9 seeded systems (nocc 10-14, 20 roots) the solve converged to
    // a wrong set on 3 with deflation and on none without, and without it the
    // solve is also faster (fewer, better-conditioned iterations).
    const bool deflate = p->ldfl != 0 && p->precon != ADCGPU_PRECON_FOLD;
    float* g32 = nullptr;
    ST(dmalloc(c, (void**)&g32, sizeof(float) * (size_t)N * blocksize));
    int nguess = 0;
    for (int phase = 0; phase < 2; ++phase) {
      if (phase == 0 && tol_b < 0) continue;
      c->mixed_bf16 = phase == 0 ? 1 : 0;
      DavidsonGPU<float> D;
      D.c = c; D.N = N; D.nstates = nstates; D.blocksize = blocksize; D.maxvec = maxvec;
      D.niter = p->maxiter; D.ipre = p->precon;
      D.ldeflate = deflate;
      D.tol = std::max(p->davtol, phase == 0 ? tol_b : tol_f);
      D.hii = c->d_diag32; D.mlp = mlp;
      D.stall_iters = 12;
      int it = 0, nc = 0;
      st = D.run(hdiag, nguess ? 2 : guess_kind, p->guessdim, g32, nguess, ev, g32, blocksize, &nguess, &it, &nc);
      inf.iterations += it; inf.nmult += D.nmult; inf.sigma_seconds += D.sigma_s;
      inf.nmult_reference += D.nmult_ref;
      if (phase == 0) inf.iters_bf16 = it; else inf.iters_fp32 = it;
      D.release();
      if (st && st != ADCGPU_NOT_CONVERGED) { dfree(c, g32, 0); dfree(c, out64, 0); return st; }
    }
    c->mixed_bf16 = 1;
    // FP64 refinement from the mixed-precision Ritz block
    double* g64 = nullptr;
    ST(dmalloc(c, (void**)&g64, sizeof(double) * (size_t)N * blocksize));
    ST((convert<float, double>(c, g32, g64, (int64_t)N * nguess)));
    dfree(c, g32, 0);
    DavidsonGPU<double> F;
    // refinement block: fewer columns than the solver's block (FP64 columns
    // are the expensive ones), but with room above the wanted roots; a block
    // of exactly davstates can lose a root (measured: 20 roots at
    // nocc=16/nvirt=180 converged to a wrong set)
    const int rdef = std::min(blocksize, std::max(nstates + 10, nstates + nstates / 2));
    const int rblock = p->refine_block == 0 ? rdef
                       : ((p->refine_block >= nstates && p->refine_block <= blocksize) ? p->refine_block : blocksize);
    F.c = c; F.N = N; F.nstates = nstates; F.blocksize = rblock;
    F.maxvec = (p->refine > 1 ? p->refine : 4) * rblock;
    // the learned correction is trained on whole FP64 solves; from the FP32
    // phase's Ritz block (residuals near 1e-5) it stalled (100 FP64
    // iterations without convergence at nocc=16/nvirt=180), so the
    // refinement uses its DPR fallback
    F.niter = p->maxiter; F.ipre = precon64 == ADCGPU_PRECON_MLP ? ADCGPU_PRECON_DPR : precon64;
    F.ldeflate = deflate; F.tol = p->davtol; F.hii = c->d_diag;
    int it2 = 0, nc2 = 0, nout = 0;
    // the refinement's subspace GEMMs run in double-float on the FP32 pipe
    // (FP64-accurate to ~1e-14 relative); the plain FP64 path keeps DFMA
    const int df_caller = c->dense_df;
    c->dense_df = 1;
    st = F.run(hdiag, 2, 0, g64, nguess, ev, out64, blocksize, &nout, &it2, &nc2);
    c->dense_df = df_caller;
    inf.iterations += it2; inf.iters_fp64 = it2; inf.nmult += F.nmult; inf.sigma_seconds += F.sigma_s;
    inf.nmult_reference += F.nmult_ref; inf.nconv = nc2; inf.max_residual = F.max_res;
    F.release();
    dfree(c, g64, 0);
  } else {
    DavidsonGPU<double> D;
    D.c = c; D.N = N; D.nstates = nstates; D.blocksize = blocksize; D.maxvec = maxvec;
    D.niter = p->maxiter; D.ipre = precon64;
    D.ldeflate = p->ldfl != 0 && precon64 != ADCGPU_PRECON_FOLD; D.tol = p->davtol; D.hii = c->d_diag;
    int it = 0, nc = 0, nout = 0;
    st = D.run(hdiag, guess_kind, p->guessdim, nullptr, 0, ev, out64, blocksize, &nout, &it, &nc);
    inf.iterations = it; inf.iters_fp64 = it; inf.nmult = D.nmult; inf.sigma_seconds = D.sigma_s; inf.nconv = nc;
    inf.nmult_reference = D.nmult_ref; inf.max_residual = D.max_res;
    D.release();
  }
  if (evecs && (st == ADCGPU_OK || st == ADCGPU_NOT_CONVERGED))
    d2h(c, evecs, out64, sizeof(double) * (size_t)N * nstates);
  dfree(c, out64, 0);
  if (st && st != ADCGPU_NOT_CONVERGED) return st;
  for (int i = 0; i < nstates; ++i) evals[i] = ev[i];
  inf.seconds = now_s() - t_start;
  if (info) *info = inf;
  return st;
}

}  // namespace adcgpu

extern "C" int adcgpu_davidson(adcgpu_ctx* h, const adcgpu_dav_params* p, double* evals, double* evecs,
                               adcgpu_dav_info* info) {
  using namespace adcgpu;
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c || !p || !evals) return ADCGPU_BAD_INPUT;
  cudaSetDevice(c->device);
  if (!c->have_matrix) return set_err(c, ADCGPU_NO_MATRIX, "build the matrix first");
  return davidson_solve(c, p, evals, evecs, info, nullptr);
}

extern "C" int adcgpu_davidson_trace(adcgpu_ctx* h, const adcgpu_dav_params* p, int every, int max_records,
                                     double* R_out, double* X_out, double* lam_out, double* evals, double* evecs,
                                     int* nrec) {
  using namespace adcgpu;
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c || !p || every <= 0 || max_records <= 0 || !R_out || !X_out || !lam_out || !evals || !evecs)
    return ADCGPU_BAD_INPUT;
  cudaSetDevice(c->device);
  if (!c->have_matrix) return set_err(c, ADCGPU_NO_MATRIX, "build the matrix first");
  const int64_t N = mat_dim(c);
  const int nstates = p->davstates;
  int blocksize = p->dmain > 0 ? p->dmain : std::max(nstates + 5, 2 * nstates);
  int maxvec = p->maxsubdim >= 0 ? p->maxsubdim : 4 * blocksize;
  maxvec = (maxvec / blocksize) * blocksize;
  std::vector<double> hdiag(N), ev;
  ADC_CUDA(c, d2h(c, hdiag.data(), c->d_diag, sizeof(double) * N));
  DavidsonGPU<double> D;
  D.c = c; D.N = N; D.nstates = nstates; D.blocksize = blocksize; D.maxvec = maxvec;
  D.niter = p->maxiter; D.ipre = p->precon; D.ldeflate = false; D.tol = p->davtol; D.hii = c->d_diag;
  D.tr_R = R_out; D.tr_X = X_out; D.tr_lam = lam_out; D.tr_every = every; D.tr_max = max_records;
  double* out = nullptr;
  int st = dmalloc(c, (void**)&out, sizeof(double) * (size_t)N * blocksize);
  if (st) return st;
  int it = 0, nc = 0, nout = 0;
  st = D.run(hdiag, p->lsubdiag == 2 ? 3 : (p->lsubdiag ? 1 : 0), p->guessdim, nullptr, 0, ev, out, blocksize,
             &nout, &it, &nc);
  if (st == ADCGPU_OK || st == ADCGPU_NOT_CONVERGED) {
    d2h(c, evecs, out, sizeof(double) * (size_t)N * nstates);
    for (int i = 0; i < nstates; ++i) evals[i] = ev[i];
  }
  if (nrec) *nrec = D.tr_n;
  D.release();
  dfree(c, out, 0);
  return st;
}

extern "C" int adcgpu_write_davidson_file(const char* path, int ndim, int nstates, const double* evals,
                                          const double* evecs) {
  if (!path || !evals || !evecs || ndim <= 0 || nstates <= 0) return ADCGPU_BAD_INPUT;
  FILE* f = fopen(path, "wb");
  if (!f) return ADCGPU_BAD_INPUT;
  for (int i = 0; i < nstates; ++i) {
    // record (i, E_i, vec_i): int32 + real8 + real8(ndim) (:1521-1523)
    int64_t bytes = 4 + 8 + 8 * (int64_t)ndim;
    if (bytes > 0x7FFFFFFF) { fclose(f); return ADCGPU_UNSUPPORTED; }
    int32_t len = (int32_t)bytes, idx = i + 1;
    fwrite(&len, 4, 1, f);
    fwrite(&idx, 4, 1, f);
    fwrite(&evals[i], 8, 1, f);
    fwrite(evecs + (size_t)i * ndim, 8, ndim, f);
    fwrite(&len, 4, 1, f);
  }
  fclose(f);
  return ADCGPU_OK;
}
