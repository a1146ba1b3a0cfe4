// Short-iterative-Lanczos propagation on the GPU.
//
// SILStep (sillib.f90:108-393) with Func = matxvec_treal (tdselib.f90:323-437,
// v2 = -i H v1) and the propagate_sillib driver (fvecprop.f90:365-564), run
// for P wavepackets at once.  Complex N-vectors are stored split: a block of
// 2P real columns [Re_0..Re_{P-1}, Im_0..Im_{P-1}], so one sigma call
// (H times 2P real columns) is the matvec of every packet, and
// -iH v = H Im v - i H Re v.
//
// Each packet keeps its own Lanczos order, error estimate, step size and
// interval progress; the per-order scalars (alpha, beta) come back to the host
// where the reference's branch logic (:236-338) is applied per packet.
// Packets that have finished an order or an interval are masked out.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#include "dense.h"
#include "internal.h"

namespace adcgpu {

typedef std::complex<double> cplx;

namespace {

// blocks of the reduction passes: two per SM (c: the context in scope)
#define SIL_BLK (c->nsm * 2)

// per-packet partials: conj(x).y (2 sums) for active packets
__global__ void k_cdot(int64_t N, int P, const double* __restrict__ X, const double* __restrict__ Y,
                       const int* __restrict__ mask, double* __restrict__ part) {
  __shared__ double red[8][2];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t ld = N;
  for (int p = 0; p < P; ++p) {
    if (!mask[p]) continue;
    double sr = 0.0, si = 0.0;
    const double *xr = X + (int64_t)p * ld, *xi = X + (int64_t)(P + p) * ld;
    const double *yr = Y + (int64_t)p * ld, *yi = Y + (int64_t)(P + p) * ld;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < N; r += (int64_t)gridDim.x * blockDim.x) {
      double a = xr[r], b = xi[r], c = yr[r], d = yi[r];
      sr += a * c + b * d;
      si += a * d - b * c;
    }
    for (int o = 16; o; o >>= 1) {
      sr += __shfl_xor_sync(0xffffffffu, sr, o);
      si += __shfl_xor_sync(0xffffffffu, si, o);
    }
    if (lane == 0) { red[w][0] = sr; red[w][1] = si; }
    __syncthreads();
    if (threadIdx.x == 0) {
      double a = 0.0, b = 0.0;
      for (int q = 0; q < (int)(blockDim.x >> 5); ++q) { a += red[q][0]; b += red[q][1]; }
      part[((int64_t)blockIdx.x * P + p) * 2 + 0] = a;
      part[((int64_t)blockIdx.x * P + p) * 2 + 1] = b;
    }
    __syncthreads();
  }
}

// K = K - alpha K1 - cbeta K2 (complex per packet), then ||K||^2 partials.
// coef layout: [p][4] = (alpha.re, alpha.im, cbeta.re, cbeta.im)
__global__ void k_recur(int64_t N, int P, double* __restrict__ K, const double* __restrict__ K1,
                        const double* __restrict__ K2, const double* __restrict__ coef, const int* __restrict__ mask,
                        double* __restrict__ part) {
  __shared__ double red[8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int p = 0; p < P; ++p) {
    if (!mask[p]) continue;
    const double ar = coef[4 * p], ai = coef[4 * p + 1], br = coef[4 * p + 2], bi = coef[4 * p + 3];
    double* kr = K + (int64_t)p * N;
    double* ki = K + (int64_t)(P + p) * N;
    const double *k1r = K1 + (int64_t)p * N, *k1i = K1 + (int64_t)(P + p) * N;
    const double *k2r = K2 + (int64_t)p * N, *k2i = K2 + (int64_t)(P + p) * N;
    double s = 0.0;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < N; r += (int64_t)gridDim.x * blockDim.x) {
      double xr = k1r[r], xi = k1i[r], yr = k2r[r], yi = k2i[r];
      double vr = kr[r] - (ar * xr - ai * xi) - (br * yr - bi * yi);
      double vi = ki[r] - (ar * xi + ai * xr) - (br * yi + bi * yr);
      kr[r] = vr; ki[r] = vi;
      s += vr * vr + vi * vi;
    }
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) red[w] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double a = 0.0;
      for (int q = 0; q < (int)(blockDim.x >> 5); ++q) a += red[q];
      part[(int64_t)blockIdx.x * P + p] = a;
    }
    __syncthreads();
  }
}

// K *= s (complex per packet): s layout [p][2]
__global__ void k_cscale(int64_t N, int P, double* __restrict__ K, const double* __restrict__ s,
                         const int* __restrict__ mask) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < N; r += (int64_t)gridDim.x * blockDim.x)
    for (int p = 0; p < P; ++p) {
      if (!mask[p]) continue;
      double sr = s[2 * p], si = s[2 * p + 1];
      double xr = K[(int64_t)p * N + r], xi = K[(int64_t)(P + p) * N + r];
      K[(int64_t)p * N + r] = sr * xr - si * xi;
      K[(int64_t)(P + p) * N + r] = sr * xi + si * xr;
    }
}

// Y := -i Y for active packets (Y holds H X): (re, im) <- (im, -re)
__global__ void k_minus_i(int64_t N, int P, double* __restrict__ Y, const int* __restrict__ mask) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < N; r += (int64_t)gridDim.x * blockDim.x)
    for (int p = 0; p < P; ++p) {
      if (!mask[p]) continue;
      double re = Y[(int64_t)p * N + r], im = Y[(int64_t)(P + p) * N + r];
      Y[(int64_t)p * N + r] = im;
      Y[(int64_t)(P + p) * N + r] = -re;
    }
}

// Psi = sum_{q=0..order} coef_q K_q, K_0 = Psi.  Kptr[q] for q >= 1.
__global__ void k_combine(int64_t N, int P, double* __restrict__ Psi, const double* const* __restrict__ Kptr,
                          const double* __restrict__ coef, const int* __restrict__ order, int maxord,
                          const int* __restrict__ mask) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < N; r += (int64_t)gridDim.x * blockDim.x)
    for (int p = 0; p < P; ++p) {
      if (!mask[p]) continue;
      const double* cp = coef + (int64_t)p * 2 * (maxord + 1);
      double xr = Psi[(int64_t)p * N + r], xi = Psi[(int64_t)(P + p) * N + r];
      double vr = cp[0] * xr - cp[1] * xi, vi = cp[0] * xi + cp[1] * xr;
      for (int q = 1; q <= order[p]; ++q) {
        const double* K = Kptr[q];
        double kr = K[(int64_t)p * N + r], ki = K[(int64_t)(P + p) * N + r];
        vr += cp[2 * q] * kr - cp[2 * q + 1] * ki;
        vi += cp[2 * q] * ki + cp[2 * q + 1] * kr;
      }
      Psi[(int64_t)p * N + r] = vr;
      Psi[(int64_t)(P + p) * N + r] = vi;
    }
}

// sum_j psi_j^2 (no conjugate) per packet: part[blk][p][2]
__global__ void k_csquare(int64_t N, int P, const double* __restrict__ Psi, double* __restrict__ part) {
  __shared__ double red[8][2];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int p = 0; p < P; ++p) {
    double sr = 0.0, si = 0.0;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < N; r += (int64_t)gridDim.x * blockDim.x) {
      double a = Psi[(int64_t)p * N + r], b = Psi[(int64_t)(P + p) * N + r];
      sr += a * a - b * b;
      si += 2.0 * a * b;
    }
    for (int o = 16; o; o >>= 1) {
      sr += __shfl_xor_sync(0xffffffffu, sr, o);
      si += __shfl_xor_sync(0xffffffffu, si, o);
    }
    if (lane == 0) { red[w][0] = sr; red[w][1] = si; }
    __syncthreads();
    if (threadIdx.x == 0) {
      double a = 0.0, b = 0.0;
      for (int q = 0; q < (int)(blockDim.x >> 5); ++q) { a += red[q][0]; b += red[q][1]; }
      part[((int64_t)blockIdx.x * P + p) * 2 + 0] = a;
      part[((int64_t)blockIdx.x * P + p) * 2 + 1] = b;
    }
    __syncthreads();
  }
}

}  // namespace


// Per-packet SILStep state (host side).
struct SilPacket {
  int TrueOrder = 0;
  double Stepsize = 0.0, Error = 0.0, MinStepsize = 0.0;
  cplx CBeta;
  std::vector<double> Diagonal, OffDiag, EigVal, EigVec;
  bool building = false;   // Krylov build in progress
  int err = 0;
  adcgpu_sil_state save;   // OldOrder / OldError / OldStepsize
};

struct SilEngine {
  Ctx* c;
  int64_t N;
  int P, kdim;
  double *Psi = nullptr, *Kbase = nullptr, *d_part = nullptr, *d_coef = nullptr;
  int *d_mask = nullptr, *d_order = nullptr;
  double** d_kptr = nullptr;
  int64_t nmult = 0;

  ~SilEngine() {
    dfree(c, Psi);
    dfree(c, Kbase);
    dfree(c, d_part);
    dfree(c, d_coef);
    dfree(c, d_mask);
    dfree(c, d_order);
    dfree(c, d_kptr);
  }
  double* K(int q) { return Kbase + (size_t)(q - 1) * N * 2 * P; }   // q = 1..kdim (K_1 = DtPsi)

  int alloc() {
    ST(dmalloc(c, (void**)&Psi, sizeof(double) * (size_t)N * 2 * P));
    ST(dmalloc(c, (void**)&Kbase, sizeof(double) * (size_t)N * 2 * P * kdim));
    ST(dmalloc(c, (void**)&d_part, sizeof(double) * SIL_BLK * 2 * (size_t)P));
    ST(dmalloc(c, (void**)&d_coef, sizeof(double) * 2 * (size_t)P * (kdim + 2) + 64));
    ST(dmalloc(c, (void**)&d_mask, sizeof(int) * P));
    ST(dmalloc(c, (void**)&d_order, sizeof(int) * P));
    ST(dmalloc(c, (void**)&d_kptr, sizeof(double*) * (kdim + 2)));
    std::vector<double*> kp(kdim + 2, nullptr);
    for (int q = 1; q <= kdim; ++q) kp[q] = K(q);
    ADC_CUDA(c, h2d(c, d_kptr, kp.data(), sizeof(double*) * (kdim + 2)));
    return ADCGPU_OK;
  }

  int set_mask(const std::vector<int>& m) {
    ADC_CUDA(c, cudaMemcpyAsync(d_mask, m.data(), sizeof(int) * P, cudaMemcpyHostToDevice, c->stream));
    return ADCGPU_OK;
  }

  // Y = -i H X for all packets (masked rotation; H applied to every column)
  int minus_i_H(const double* X, double* Y, const std::vector<int>& mask) {
    ST(sigma_fp64(c, 2 * P, X, N, Y, N));
    ST(set_mask(mask));
    k_minus_i<<<c->nsm * 4, 256, 0, c->stream>>>(N, P, Y, d_mask); ADC_COUNT_LAUNCH();
    ADC_CUDA(c, cudaGetLastError());
    int na = 0;
    for (int v : mask) na += v;
    nmult += na;
    return ADCGPU_OK;
  }

  int cdots(const double* X, const double* Y, const std::vector<int>& mask, std::vector<cplx>& out) {
    ST(set_mask(mask));
    k_cdot<<<SIL_BLK, 256, 0, c->stream>>>(N, P, X, Y, d_mask, d_part); ADC_COUNT_LAUNCH();
    std::vector<double> h((size_t)SIL_BLK * P * 2);
    ADC_CUDA(c, cudaMemcpyAsync(h.data(), d_part, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c->stream));
    ADC_CUDA(c, cudaStreamSynchronize(c->stream));
    out.assign(P, cplx(0, 0));
    for (int p = 0; p < P; ++p) {
      if (!mask[p]) continue;
      double a = 0.0, b = 0.0;
      for (int bl = 0; bl < SIL_BLK; ++bl) { a += h[((size_t)bl * P + p) * 2]; b += h[((size_t)bl * P + p) * 2 + 1]; }
      out[p] = cplx(a, b);
    }
    return ADCGPU_OK;
  }

  int recur(double* Kn, const double* K1, const double* K2, const std::vector<cplx>& alpha,
            const std::vector<cplx>& cbeta, const std::vector<int>& mask, std::vector<double>& norm2) {
    std::vector<double> coef(4 * (size_t)P, 0.0);
    for (int p = 0; p < P; ++p) {
      coef[4 * p] = alpha[p].real(); coef[4 * p + 1] = alpha[p].imag();
      coef[4 * p + 2] = cbeta[p].real(); coef[4 * p + 3] = cbeta[p].imag();
    }
    ADC_CUDA(c, cudaMemcpyAsync(d_coef, coef.data(), sizeof(double) * coef.size(), cudaMemcpyHostToDevice, c->stream));
    ST(set_mask(mask));
    k_recur<<<SIL_BLK, 256, 0, c->stream>>>(N, P, Kn, K1, K2, d_coef, d_mask, d_part); ADC_COUNT_LAUNCH();
    std::vector<double> h((size_t)SIL_BLK * P);
    ADC_CUDA(c, cudaMemcpyAsync(h.data(), d_part, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c->stream));
    ADC_CUDA(c, cudaStreamSynchronize(c->stream));
    norm2.assign(P, 0.0);
    for (int p = 0; p < P; ++p) {
      if (!mask[p]) continue;
      for (int bl = 0; bl < SIL_BLK; ++bl) norm2[p] += h[(size_t)bl * P + p];
    }
    return ADCGPU_OK;
  }

  int cscale(double* Kn, const std::vector<cplx>& s, const std::vector<int>& mask) {
    std::vector<double> coef(2 * (size_t)P, 0.0);
    for (int p = 0; p < P; ++p) { coef[2 * p] = s[p].real(); coef[2 * p + 1] = s[p].imag(); }
    ADC_CUDA(c, cudaMemcpyAsync(d_coef, coef.data(), sizeof(double) * coef.size(), cudaMemcpyHostToDevice, c->stream));
    ST(set_mask(mask));
    k_cscale<<<c->nsm * 4, 256, 0, c->stream>>>(N, P, Kn, d_coef, d_mask); ADC_COUNT_LAUNCH();
    ADC_CUDA(c, cudaGetLastError());
    return ADCGPU_OK;
  }

  // One SILStep for the packets in 'mask' (restart mode, StdForm, no relax
  // unless 'relax'); DtPsi = K(1) must hold -iH Psi.  Sets stepsize/order.
  int silstep(const std::vector<int>& mask_in, std::vector<SilPacket>& pk, const std::vector<double>& intperiod,
              double tol, bool relax) {
    const double RelativeMinStep = 1.0e-10;
    const cplx PreFactor = relax ? cplx(-1.0, 0.0) : cplx(0.0, -1.0);
    std::vector<int> mask = mask_in;
    if (kdim < 2) {
      for (int p = 0; p < P; ++p) if (mask[p]) pk[p].err = ADCGPU_SIL_BAD_ORDER;
      return ADCGPU_OK;
    }
    // first diagonal element and basis vector (:189-221)
    std::vector<cplx> alpha, cbeta(P, cplx(0, 0)), inv(P, cplx(0, 0));
    ST(cdots(Psi, K(1), mask, alpha));
    for (int p = 0; p < P; ++p) {
      if (!mask[p]) continue;
      SilPacket& s = pk[p];
      s.Stepsize = intperiod[p];
      s.MinStepsize = std::fabs(RelativeMinStep * intperiod[p]);
      s.Diagonal.assign(kdim + 1, 0.0);
      s.OffDiag.assign(kdim + 1, 0.0);
      s.save.old_error = 0.0; s.save.old_order = 0; s.save.old_stepsize = 0.0;
      s.TrueOrder = 1;
      s.Diagonal[0] = (alpha[p] / PreFactor).real();
    }
    // DtPsi -= Alpha Psi; Beta = ||DtPsi||  (K2 unused: cbeta = 0)
    std::vector<double> n2;
    ST(recur(K(1), Psi, Psi, alpha, cbeta, mask, n2));
    for (int p = 0; p < P; ++p) {
      if (!mask[p]) continue;
      SilPacket& s = pk[p];
      double Beta = std::sqrt(n2[p]);
      s.OffDiag[1] = Beta;
      s.CBeta = PreFactor * Beta;
      if (Beta < 1.0e-20) { Beta = 0.0; inv[p] = cplx(0, 0); }
      else inv[p] = 1.0 / s.CBeta;
      s.Error = std::fabs(Beta * s.Stepsize);
    }
    ST(cscale(K(1), inv, mask));
    // build the Krylov space (:225-326)
    std::vector<int> active = mask;
    for (;;) {
      bool any = false;
      for (int p = 0; p < P; ++p) {
        if (!active[p]) continue;
        SilPacket& s = pk[p];
        if (std::fabs(s.Stepsize) < std::fabs(s.MinStepsize)) { s.err = ADCGPU_SIL_STEP_UNDERFLOW; active[p] = 0; continue; }
        s.TrueOrder += 1;
        any = true;
      }
      if (!any) break;
      // all active packets are at the same order (they advance in lockstep)
      int ord = 0;
      for (int p = 0; p < P; ++p) if (active[p]) { ord = pk[p].TrueOrder; break; }
      ST(minus_i_H(K(ord - 1), K(ord), active));
      ST(cdots(K(ord - 1), K(ord), active, alpha));
      for (int p = 0; p < P; ++p) {
        if (!active[p]) continue;
        pk[p].Diagonal[ord - 1] = (alpha[p] / PreFactor).real();
        cbeta[p] = pk[p].CBeta;
      }
      const double* Kprev2 = ord == 2 ? Psi : K(ord - 2);
      ST(recur(K(ord), K(ord - 1), Kprev2, alpha, cbeta, active, n2));
      for (int p = 0; p < P; ++p) {
        if (!active[p]) continue;
        SilPacket& s = pk[p];
        double Beta = std::sqrt(n2[p]);
        s.OffDiag[ord] = Beta;
        s.CBeta = PreFactor * Beta;
        if (Beta < 1.0e-20) { s.OffDiag[ord] = 0.0; Beta = 0.0; inv[p] = cplx(0, 0); }
        else inv[p] = 1.0 / s.CBeta;
        s.Error = std::fabs(s.Error * Beta * s.Stepsize / (double)ord);
        s.building = (ord < kdim) && (s.Error > tol) && (Beta > 1.0e-20);
      }
      ST(cscale(K(ord), inv, active));
      for (int p = 0; p < P; ++p) if (active[p] && !pk[p].building) active[p] = 0;
    }
    // finish each packet: step size, tridiagonal eigenproblem, propagation
    int maxord = 0;
    for (int p = 0; p < P; ++p) if (mask[p] && !pk[p].err) maxord = std::max(maxord, pk[p].TrueOrder);
    std::vector<double> coef((size_t)P * 2 * (kdim + 1), 0.0);
    std::vector<int> ordv(P, 0), pmask(P, 0);
    for (int p = 0; p < P; ++p) {
      if (!mask[p] || pk[p].err) continue;
      SilPacket& s = pk[p];
      const int to = s.TrueOrder;
      s.Diagonal[to] = s.Diagonal[to - 1];
      if (s.Error > tol) s.Stepsize = s.Stepsize * std::pow(tol / s.Error, 1.0 / (double)to);
      s.save.old_order = to; s.save.old_stepsize = s.Stepsize; s.save.old_error = s.Error;
      // dsteqr on the (to+1) x (to+1) tridiagonal
      const int n = to + 1;
      std::vector<double> Tm((size_t)n * n, 0.0);
      for (int i = 0; i < n; ++i) Tm[(size_t)i * n + i] = s.Diagonal[i];
      for (int i = 0; i + 1 < n; ++i) { Tm[(size_t)i * n + i + 1] = s.OffDiag[i + 1]; Tm[(size_t)(i + 1) * n + i] = s.OffDiag[i + 1]; }
      s.EigVal.assign(n, 0.0);
      s.EigVec.assign((size_t)n * n, 0.0);
      if (!host_syev(n, Tm.data(), n, s.EigVal.data(), s.EigVec.data())) { s.err = ADCGPU_SIL_DIAG_FAILED; continue; }
      for (int P2 = 0; P2 <= to; ++P2) {
        cplx sum(0.0, 0.0);
        for (int Q = 0; Q <= to; ++Q)
          sum += std::exp(PreFactor * s.EigVal[Q] * s.Stepsize) * s.EigVec[(size_t)Q * n + 0] * s.EigVec[(size_t)Q * n + P2];
        coef[(size_t)p * 2 * (kdim + 1) + 2 * P2] = sum.real();
        coef[(size_t)p * 2 * (kdim + 1) + 2 * P2 + 1] = sum.imag();
      }
      ordv[p] = to;
      pmask[p] = 1;
    }
    ADC_CUDA(c, cudaMemcpyAsync(d_coef, coef.data(), sizeof(double) * coef.size(), cudaMemcpyHostToDevice, c->stream));
    ADC_CUDA(c, cudaMemcpyAsync(d_order, ordv.data(), sizeof(int) * P, cudaMemcpyHostToDevice, c->stream));
    ST(set_mask(pmask));
    k_combine<<<c->nsm * 4, 256, 0, c->stream>>>(N, P, Psi, d_kptr, d_coef, d_order, kdim, d_mask); ADC_COUNT_LAUNCH();
    ADC_CUDA(c, cudaGetLastError());
    (void)maxord;
    return ADCGPU_OK;
  }

  int csquare(std::vector<cplx>& out) {
    k_csquare<<<SIL_BLK, 256, 0, c->stream>>>(N, P, Psi, d_part); ADC_COUNT_LAUNCH();
    std::vector<double> h((size_t)SIL_BLK * P * 2);
    ADC_CUDA(c, cudaMemcpyAsync(h.data(), d_part, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c->stream));
    ADC_CUDA(c, cudaStreamSynchronize(c->stream));
    out.assign(P, cplx(0, 0));
    for (int p = 0; p < P; ++p) {
      double a = 0.0, b = 0.0;
      for (int bl = 0; bl < SIL_BLK; ++bl) { a += h[((size_t)bl * P + p) * 2]; b += h[((size_t)bl * P + p) * 2 + 1]; }
      out[p] = cplx(a, b);
    }
    return ADCGPU_OK;
  }
};

}  // namespace adcgpu

using namespace adcgpu;

extern "C" int adcgpu_autocorr(adcgpu_ctx* h, int nwp, const double* f, double tout, double tfinal, int kdim,
                               double tol, double* auto_out, int* ntimes_out, int64_t* nmult_out) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c) return ADCGPU_BAD_INPUT;
  cudaSetDevice(c->device);
  if (!c->have_matrix) return set_err(c, ADCGPU_NO_MATRIX, "build the matrix first");
  if (c->precision != ADCGPU_FP64) return set_err(c, ADCGPU_BAD_INPUT, "SIL runs on the FP64 matrix");
  if (nwp <= 0 || !f || !auto_out || tout <= 0.0 || tfinal < 0.0 || kdim < 2)
    return set_err(c, ADCGPU_BAD_INPUT, "autocorr arguments");
  const int64_t N = mat_dim(c);
  SilEngine E;
  E.c = c; E.N = N; E.P = nwp; E.kdim = kdim;
  ST(E.alloc());
  // init_wavepacket: psi0 = f / ||f|| (complex, zero imaginary part)
  std::vector<double> norm0(nwp);
  {
    std::vector<double> blk((size_t)N * 2 * nwp, 0.0);
    for (int p = 0; p < nwp; ++p) {
      double s = 0.0;
      for (int64_t i = 0; i < N; ++i) s += f[(size_t)p * N + i] * f[(size_t)p * N + i];
      norm0[p] = std::sqrt(s);
      for (int64_t i = 0; i < N; ++i) blk[(size_t)p * N + i] = f[(size_t)p * N + i] / norm0[p];
    }
    ADC_CUDA(c, h2d(c, E.Psi, blk.data(), sizeof(double) * blk.size()));
  }
  const double intperiod = 0.5 * tout, tiny = 1e-9;
  const int nsteps = (int)(tfinal / intperiod);
  const int ntimes = nsteps + 1;
  // t = 0: dot_product(psi0,psi0)*norm0^2 = norm0^2
  for (int p = 0; p < nwp; ++p) {
    auto_out[((size_t)p * ntimes) * 2] = norm0[p] * norm0[p];
    auto_out[((size_t)p * ntimes) * 2 + 1] = 0.0;
  }
  std::vector<SilPacket> pk(nwp);
  std::vector<double> inttime(nwp), period(nwp);
  for (int i = 1; i <= nsteps; ++i) {
    std::fill(inttime.begin(), inttime.end(), 0.0);
    std::vector<int> todo(nwp, 1);
    for (;;) {
      bool any = false;
      for (int p = 0; p < nwp; ++p) {
        if (!todo[p]) continue;
        any = true;
        period[p] = intperiod - inttime[p];
      }
      if (!any) break;
      ST(E.minus_i_H(E.Psi, E.K(1), todo));
      ST(E.silstep(todo, pk, period, tol, false));
      for (int p = 0; p < nwp; ++p) {
        if (!todo[p]) continue;
        if (pk[p].err) {
          if (ntimes_out) *ntimes_out = i;
          return set_err(c, pk[p].err, "SIL integration failed");
        }
        inttime[p] += pk[p].Stepsize;
        if (!(std::fabs(intperiod - inttime[p]) > std::fabs(tiny * intperiod))) todo[p] = 0;
      }
    }
    std::vector<cplx> a;
    ST(E.csquare(a));
    for (int p = 0; p < nwp; ++p) {
      cplx v = a[p] * (norm0[p] * norm0[p]);
      auto_out[((size_t)p * ntimes + i) * 2] = v.real();
      auto_out[((size_t)p * ntimes + i) * 2 + 1] = v.imag();
    }
  }
  if (ntimes_out) *ntimes_out = ntimes;
  if (nmult_out) *nmult_out = E.nmult / std::max(1, nwp);
  return ADCGPU_OK;
}

extern "C" int adcgpu_silstep(adcgpu_ctx* h, double* psi, double* dtpsi, int psidim, double intperiod, int intorder,
                              double tol, int relax, int restart, int stdform, double* stepsize_out,
                              int* trueorder_out, adcgpu_sil_state* st) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c) return ADCGPU_BAD_INPUT;
  cudaSetDevice(c->device);
  if (!c->have_matrix) return set_err(c, ADCGPU_NO_MATRIX, "build the matrix first");
  if (psidim != mat_dim(c) || !psi || !dtpsi) return set_err(c, ADCGPU_BAD_INPUT, "psi dimension");
  if (intorder < 2) return ADCGPU_SIL_BAD_ORDER;
  if (!restart) return set_err(c, ADCGPU_UNSUPPORTED, "non-restart SILStep calls keep Krylov vectors; use restart");
  if (!stdform) return set_err(c, ADCGPU_UNSUPPORTED, "Func must be -iH (StdForm) on this path");
  const int64_t N = mat_dim(c);
  SilEngine E;
  E.c = c; E.N = N; E.P = 1; E.kdim = intorder;
  ST(E.alloc());
  std::vector<double> blk((size_t)N * 2);
  for (int64_t i = 0; i < N; ++i) { blk[i] = psi[2 * i]; blk[N + i] = psi[2 * i + 1]; }
  ADC_CUDA(c, h2d(c, E.Psi, blk.data(), sizeof(double) * 2 * N));
  for (int64_t i = 0; i < N; ++i) { blk[i] = dtpsi[2 * i]; blk[N + i] = dtpsi[2 * i + 1]; }
  ADC_CUDA(c, h2d(c, E.K(1), blk.data(), sizeof(double) * 2 * N));
  std::vector<SilPacket> pk(1);
  std::vector<int> mask(1, 1);
  std::vector<double> period(1, intperiod);
  ST(E.silstep(mask, pk, period, tol, relax != 0));
  ADC_CUDA(c, cudaStreamSynchronize(c->stream));
  if (pk[0].err) return pk[0].err;
  ADC_CUDA(c, d2h(c, blk.data(), E.Psi, sizeof(double) * 2 * N));
  for (int64_t i = 0; i < N; ++i) { psi[2 * i] = blk[i]; psi[2 * i + 1] = blk[N + i]; }
  ADC_CUDA(c, d2h(c, blk.data(), E.K(1), sizeof(double) * 2 * N));
  for (int64_t i = 0; i < N; ++i) { dtpsi[2 * i] = blk[i]; dtpsi[2 * i + 1] = blk[N + i]; }
  if (stepsize_out) *stepsize_out = pk[0].Stepsize;
  if (trueorder_out) *trueorder_out = pk[0].TrueOrder;
  if (st) *st = pk[0].save;
  return ADCGPU_OK;
}
