// prop_gnlse.cu -- fused split-step kernel of Chi3GNLSE (solvers/Chi3GNLSE.cpp:39-92).
//
// Each RK4 stage of the generalised NLSE needs two convolutions of the whole field:
//     k = IFFT[(g0 + g1 w) FFT[ y * IFFT[R~ FFT[rel |y|^2]] ]]
// so a z step is 16 transforms inside the nonlinear step plus the dispersion pair.  The
// field state and the RK4 accumulator of each propagation are kept in a per-CTA slot of
// global scratch memory (each thread only touches its own points, so the slot stays in L1/L2);
// registers hold the stage input y and the transform in flight.
#include <vector>

#include "nlm_propagate.cuh"

namespace nlm {

// GEN: the general plan (any N, padded ownership); the scratch slot then holds T R >= N values per part.
// FS: the RK4 sum kept in the frequency domain, as in k_propagate_gnlse_pair: each stage's k is formed
// as a spectrum by the self-steepening operator and transformed back only as the next stage's input
// (the fourth stage's inverse transform drops out), and the state's spectrum is kept from the previous
// dispersion step, so FFT[x + sum / 6] = N (X + A / 6) needs no transform: 16 transforms per step
// instead of 18, three scratch parts (X, its spectrum XF, the sum A) instead of two.  Without FS (the
// allocation-free entry point, whose static array is sized for two parts) the sum stays in time.
template <int R, bool GEN = false, bool FS = true>
__global__ void __launch_bounds__(kMaxThreads) k_propagate_gnlse(const PropArgs a, double2* __restrict__ scratch) {
  extern __shared__ double2 smem[];
  const FFTPlanH& plan = a.plan;
  const int N = plan.N, T = plan.T;
  const int g = threadIdx.x / T, j = threadIdx.x - g * T;
  double2* bufs;
  const double2* tw = stage_twiddles<R>(a.tw, smem, N, &bufs);
  double2* buf = bufs + (long long)g * N;
  const long long NS = (long long)T * R;                                          // N for a power-of-two plan
  double2* X = scratch + ((long long)blockIdx.x * a.ipc + g) * (FS ? 3 : 2) * NS;  // state (time domain)
  double2* ACC = X + NS;                       // k1 + 2 k2 + 2 k3 + k4 (time domain; the spectrum with FS)
  double2* XF = X + 2 * NS;                    // FS: the state's spectrum
  const long long nGroups = (a.nInst + a.ipc - 1) / a.ipc;
  __shared__ long long s_group;
  for (long long cg = blockIdx.x; cg < nGroups; cg = next_group(a, cg, &s_group)) {
    const long long local = cg * a.ipc + g;
    const bool active = local < a.nInst;
    const long long inst = a.instBase + local;
    double2 x[1][R];
    load_input<1, R, GEN>(a, inst, active, j, x, buf, plan, tw);
    const long long ms = (long long)a.nZ * N;
    if (a.gridF) store_rows<1, R, GEN>(a.gridF, ms, 0, N, T, j, x, (double)N, active);
    if (FS) {
#pragma unroll
      for (int v = 0; v < R; v++) XF[j + v * T] = x[0][v];
    }
    fft_any<R, true, GEN>(x[0], buf, tw, plan, j);
    if (a.gridT) store_rows<1, R, GEN>(a.gridT, ms, 0, N, T, j, x, 1.0, active);
#pragma unroll
    for (int v = 0; v < R; v++) X[j + v * T] = x[0][v];
    if (a.ckpt && a.nZ > 1) store_rows<1, R, GEN>(a.ckpt + inst * a.ckN * (long long)N, N, 0, N, T, j, x, 1.0, active);
    for (int i = 1; i < a.nZ; i++) {
      const double* rel = a.relInt + (long long)(i - 1) * 3;
      double2 k[R];
#pragma unroll
      for (int v = 0; v < R; v++) k[v] = czero();
      for (int s = 0; s < 4; s++) {
        const double fac = s == 0 ? 0.0 : (s == 3 ? 1.0 : 0.5);
        const double wgt = (s == 1 || s == 2) ? 2.0 : 1.0;
        const double ri = __ldg(rel + (s == 0 ? 0 : (s == 3 ? 2 : 1)));
        double2 y[R], u[R];
#pragma unroll
        for (int v = 0; v < R; v++) {
          y[v] = caxpy(X[j + v * T], fac, k[v]);
          u[v] = make_double2(ri * cabs2(y[v]), 0.0);
        }
        // Raman convolution R~ * (rel |y|^2)
        fft_any<R, false, GEN>(u, buf, tw, plan, j);
#pragma unroll
        for (int v = 0; v < R; v++) u[v] = cmul(u[v], __ldg(a.raman + j + v * T));
        fft_any<R, true, GEN>(u, buf, tw, plan, j);
        // times the field, then the self-steepening operator (g0 + g1 w)
#pragma unroll
        for (int v = 0; v < R; v++) u[v] = cmul(u[v], y[v]);
        fft_any<R, false, GEN>(u, buf, tw, plan, j);
#pragma unroll
        for (int v = 0; v < R; v++) u[v] = cmul(u[v], __ldg(a.steep + j + v * T));
        if (FS) {
#pragma unroll
          for (int v = 0; v < R; v++) {
            const int t = j + v * T;
            ACC[t] = s == 0 ? u[v] : caxpy(ACC[t], wgt, u[v]);
          }
          if (s < 3) {
            fft_any<R, true, GEN>(u, buf, tw, plan, j);
#pragma unroll
            for (int v = 0; v < R; v++) k[v] = u[v];
          }
        } else {
          fft_any<R, true, GEN>(u, buf, tw, plan, j);
#pragma unroll
          for (int v = 0; v < R; v++) {
            k[v] = u[v];
            const int t = j + v * T;
            ACC[t] = s == 0 ? u[v] : caxpy(ACC[t], wgt, u[v]);
          }
        }
      }
      const bool last = i == a.nZ - 1;
      if (FS) {
        // the dispersion step on the spectrum of x + sum / 6 (the tables carry each pair's 1/N)
        const double2* table = last ? a.dlast : a.dstep;
#pragma unroll
        for (int v = 0; v < R; v++) {
          const int t = j + v * T;
          x[0][v] = cmul(cscale(caxpy(XF[t], 1.0 / 6.0, ACC[t]), (double)N), __ldg(table + t));
        }
        if (a.gridF) store_rows<1, R, GEN>(a.gridF, ms, i, N, T, j, x, (double)N, active);
        if (!last) {
#pragma unroll
          for (int v = 0; v < R; v++) XF[j + v * T] = x[0][v];
        }
        if (!last || a.inTime || a.gridT) {
          fft_any<R, true, GEN>(x[0], buf, tw, plan, j);
          if (a.gridT) store_rows<1, R, GEN>(a.gridT, ms, i, N, T, j, x, 1.0, active);
        }
      } else {
#pragma unroll
        for (int v = 0; v < R; v++) x[0][v] = caxpy(X[j + v * T], 1.0 / 6.0, ACC[j + v * T]);
        dispersion_step<1, R, GEN>(a, i, last, j, x, buf, plan, active, last ? a.dlast : a.dstep, tw);
      }
      if (!last) {
#pragma unroll
        for (int v = 0; v < R; v++) X[j + v * T] = x[0][v];
        if (a.ckpt && i % a.ckK == 0)
          store_rows<1, R, GEN>(a.ckpt + (inst * a.ckN + i / a.ckK) * (long long)N, N, 0, N, T, j, x, 1.0, active);
      }
    }
    if (a.nZ == 1) {
      fft_any<R, false, GEN>(x[0], buf, tw, plan, j);
#pragma unroll
      for (int v = 0; v < R; v++) x[0][v] = cmul(x[0][v], __ldg(a.back + j + v * T));
      if (a.gridF) store_rows<1, R, GEN>(a.gridF, ms, 0, N, T, j, x, (double)N, active);
      if (a.inTime || a.gridT) {
        fft_any<R, true, GEN>(x[0], buf, tw, plan, j);
        if (a.gridT) store_rows<1, R, GEN>(a.gridT, ms, 0, N, T, j, x, 1.0, active);
      }
    }
    store_output<1, R, GEN>(a, inst, active, j, x, a.inTime ? 1.0 : (double)N);
    __syncthreads();
  }
}

// Two rows per thread group (rows 2q and 2q+1 of the launch).  The Raman convolution acts on the real
// intensity rel |y|^2 with the transform of a real response, R~ (Hermitian), so the two rows'
// convolutions run as one complex convolution: IFFT[R~ FFT[uA + i uB]] = conv(uA) + i conv(uB); the
// Raman result is taken real, as it is in exact arithmetic.
// The RK4 sum is kept in the frequency domain: each stage's k is formed there (the self-steepening
// operator) and needed back in time only as the next stage's input, so the last stage's inverse
// transform is skipped; and the state's spectrum is kept from the previous step's dispersion, so the
// step's end FFT[x + sum / 6] = X + FFT[sum] / 6 needs no transform.  A row then costs 12 transforms
// per step instead of 18 (4 stages x (1 shared Raman pair / 2 + 2 steepening) - 1, + 1 inverse for the
// dispersion step); in exact arithmetic the same step.  A second row past the end of the launch
// propagates zeros and is not stored.
// Scratch per slot: the two rows' states in time (X) and frequency (XF), RK4 sums in frequency (A) and
// stage results in time (K), and their real Raman results (9 N complex values).
template <int R>
__global__ void __launch_bounds__(kMaxThreads) k_propagate_gnlse_pair(const PropArgs a, double2* __restrict__ scratch) {
  extern __shared__ double2 smem[];
  const FFTPlanH& plan = a.plan;
  const int N = plan.N, T = plan.T;
  const int g = threadIdx.x / T, j = threadIdx.x - g * T;
  double2* bufs;
  const double2* tw = stage_twiddles<R>(a.tw, smem, N, &bufs);
  double2* buf = bufs + (long long)g * N;
  // slot: X, XF, A, K of row 0 and 1 (N values each), then the two rows' real Raman results (N reals
  // each, in the space of N complex values)
  double2* slot = scratch + ((long long)blockIdx.x * a.ipc + g) * 9 * N;
  auto U = [&](int r) { return reinterpret_cast<double*>(slot + 8 * N) + (long long)r * N; };
  auto X = [&](int r) { return slot + (long long)r * N; };
  auto XF = [&](int r) { return slot + (long long)(2 + r) * N; };
  auto A = [&](int r) { return slot + (long long)(4 + r) * N; };
  auto K = [&](int r) { return slot + (long long)(6 + r) * N; };
  const long long nPairs = (a.nInst + 1) / 2;
  const long long nGroups = (nPairs + a.ipc - 1) / a.ipc;
  __shared__ long long s_group;
  for (long long cg = blockIdx.x; cg < nGroups; cg = next_group(a, cg, &s_group)) {
    const long long pair = cg * a.ipc + g;
    auto active = [&](int r) { return pair < nPairs && 2 * pair + r < a.nInst; };
    auto inst = [&](int r) { return a.instBase + 2 * pair + r; };
#pragma unroll 1
    for (int r = 0; r < 2; r++) {
      double2 x[1][R];
      load_input<1, R>(a, inst(r), active(r), j, x, buf, plan, tw);
#pragma unroll
      for (int v = 0; v < R; v++) XF(r)[j + v * T] = x[0][v];
      fft_regs<R, true>(x[0], buf, tw, plan, j);
#pragma unroll
      for (int v = 0; v < R; v++) X(r)[j + v * T] = x[0][v];
      if (a.ckpt && a.nZ > 1) store_rows<1, R>(a.ckpt + inst(r) * a.ckN * (long long)N, N, 0, N, T, j, x, 1.0, active(r));
    }
    for (int i = 1; i < a.nZ; i++) {
      const double* rel = a.relInt + (long long)(i - 1) * 3;
      for (int s = 0; s < 4; s++) {
        const double fac = s == 0 ? 0.0 : (s == 3 ? 1.0 : 0.5);
        const double wgt = (s == 1 || s == 2) ? 2.0 : 1.0;
        const double ri = __ldg(rel + (s == 0 ? 0 : (s == 3 ? 2 : 1)));
        // both rows' Raman convolutions in one complex transform pair
        double2 u[R];
#pragma unroll
        for (int v = 0; v < R; v++) {
          const int t = j + v * T;
          const double2 yA = s == 0 ? X(0)[t] : caxpy(X(0)[t], fac, K(0)[t]);
          const double2 yB = s == 0 ? X(1)[t] : caxpy(X(1)[t], fac, K(1)[t]);
          u[v] = make_double2(ri * cabs2(yA), ri * cabs2(yB));
        }
        fft_regs<R, false>(u, buf, tw, plan, j);
#pragma unroll
        for (int v = 0; v < R; v++) u[v] = cmul(u[v], __ldg(a.raman + j + v * T));
        fft_regs<R, true>(u, buf, tw, plan, j);
        // the two real results wait in scratch (each thread reads back its own points)
#pragma unroll
        for (int v = 0; v < R; v++) {
          U(0)[j + v * T] = u[v].x;
          U(1)[j + v * T] = u[v].y;
        }
        // per row: times the field, then the self-steepening operator (g0 + g1 w): the stage's k in
        // the frequency domain, added to the sum there; back in time for the next stage's input
#pragma unroll 1
        for (int r = 0; r < 2; r++) {
          double2 w[R];
#pragma unroll
          for (int v = 0; v < R; v++) {
            const int t = j + v * T;
            const double2 y = s == 0 ? X(r)[t] : caxpy(X(r)[t], fac, K(r)[t]);
            const double c = U(r)[t];
            w[v] = make_double2(c * y.x, c * y.y);
          }
          fft_regs<R, false>(w, buf, tw, plan, j);
#pragma unroll
          for (int v = 0; v < R; v++) {
            const int t = j + v * T;
            w[v] = cmul(w[v], __ldg(a.steep + t));
            A(r)[t] = s == 0 ? w[v] : caxpy(A(r)[t], wgt, w[v]);
          }
          if (s < 3) {
            fft_regs<R, true>(w, buf, tw, plan, j);
#pragma unroll
            for (int v = 0; v < R; v++) K(r)[j + v * T] = w[v];
          }
        }
      }
      // the dispersion step on the spectrum of x + sum / 6: N (X + A / 6), X and A holding spectra whose
      // unscaled inverse transform is the time-domain field (the tables carry the 1/N of each
      // transform pair); then back to time
      const bool last = i == a.nZ - 1;
      const double2* table = last ? a.dlast : a.dstep;
#pragma unroll 1
      for (int r = 0; r < 2; r++) {
        double2 x[1][R];
#pragma unroll
        for (int v = 0; v < R; v++) {
          const int t = j + v * T;
          x[0][v] = cmul(cscale(caxpy(XF(r)[t], 1.0 / 6.0, A(r)[t]), (double)N), __ldg(table + t));
        }
        if (!last) {
#pragma unroll
          for (int v = 0; v < R; v++) XF(r)[j + v * T] = x[0][v];
        }
        if (!last || a.inTime) fft_regs<R, true>(x[0], buf, tw, plan, j);
        if (!last) {
#pragma unroll
          for (int v = 0; v < R; v++) X(r)[j + v * T] = x[0][v];
          if (a.ckpt && i % a.ckK == 0)
            store_rows<1, R>(a.ckpt + (inst(r) * a.ckN + i / a.ckK) * (long long)N, N, 0, N, T, j, x, 1.0, active(r));
        } else {
          store_output<1, R>(a, inst(r), active(r), j, x, a.inTime ? 1.0 : (double)N);
        }
      }
    }
    if (a.nZ == 1) {
#pragma unroll 1
      for (int r = 0; r < 2; r++) {
        double2 x[1][R];
#pragma unroll
        for (int v = 0; v < R; v++) x[0][v] = X(r)[j + v * T];
        fft_regs<R, false>(x[0], buf, tw, plan, j);
#pragma unroll
        for (int v = 0; v < R; v++) x[0][v] = cmul(x[0][v], __ldg(a.back + j + v * T));
        if (a.inTime) fft_regs<R, true>(x[0], buf, tw, plan, j);
        store_output<1, R>(a, inst(r), active(r), j, x, a.inTime ? 1.0 : (double)N);
      }
    }
    __syncthreads();
  }
}

void add_kernels_gnlse(std::vector<KernelEntry>& t) {
  t.push_back({kKindGnlse, kChi3GNLSE, 8, (const void*)k_propagate_gnlse<8>});
  // key + 700: the RK4 sum in time (two scratch parts), for the allocation-free entry point
  t.push_back({kKindGnlse, kChi3GNLSE + 700, 8, (const void*)k_propagate_gnlse<8, false, false>});
  // key + kGenKey: grids that are not powers of two (general plan), up to 4096 and 8192 points
  t.push_back({kKindGnlse, kChi3GNLSE + kGenKey, 8, (const void*)k_propagate_gnlse<8, true>});
  t.push_back({kKindGnlse, kChi3GNLSE + kGenKey, 16, (const void*)k_propagate_gnlse<16, true>});
  // key + 400: two rows per thread group, shared Raman transforms
  t.push_back({kKindGnlse, kChi3GNLSE + 400, 8, (const void*)k_propagate_gnlse_pair<8>});
}

}  // namespace nlm
