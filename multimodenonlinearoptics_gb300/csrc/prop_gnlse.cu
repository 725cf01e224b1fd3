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

template <int R>
__global__ void __launch_bounds__(kMaxThreads) k_propagate_gnlse(const PropArgs a, double2* __restrict__ scratch) {
  extern __shared__ double2 smem[];
  const FFTPlanH& plan = a.plan;
  const int N = plan.N, T = plan.T;
  const int g = threadIdx.x / T, j = threadIdx.x - g * T;
  double2* bufs;
  const double2* tw = stage_twiddles<R>(a.tw, smem, N, &bufs);
  double2* buf = bufs + (long long)g * N;
  double2* X = scratch + ((long long)blockIdx.x * a.ipc + g) * 2 * N;   // state (time domain)
  double2* ACC = X + N;                                                 // k1 + 2 k2 + 2 k3 + k4
  const long long nGroups = (a.nInst + a.ipc - 1) / a.ipc;
  __shared__ long long s_group;
  for (long long cg = blockIdx.x; cg < nGroups; cg = next_group(a, cg, &s_group)) {
    const long long local = cg * a.ipc + g;
    const bool active = local < a.nInst;
    const long long inst = a.instBase + local;
    double2 x[1][R];
    load_input<1, R>(a, inst, active, j, x, buf, plan, tw);
    const long long ms = (long long)a.nZ * N;
    if (a.gridF) store_rows<1, R>(a.gridF, ms, 0, N, T, j, x, (double)N, active);
    fft_regs<R, true>(x[0], buf, tw, plan, j);
    if (a.gridT) store_rows<1, R>(a.gridT, ms, 0, N, T, j, x, 1.0, active);
#pragma unroll
    for (int v = 0; v < R; v++) X[j + v * T] = x[0][v];
    if (a.ckpt && a.nZ > 1) store_rows<1, R>(a.ckpt + inst * a.ckN * (long long)N, N, 0, N, T, j, x, 1.0, active);
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
        fft_regs<R, false>(u, buf, tw, plan, j);
#pragma unroll
        for (int v = 0; v < R; v++) u[v] = cmul(u[v], __ldg(a.raman + j + v * T));
        fft_regs<R, true>(u, buf, tw, plan, j);
        // times the field, then the self-steepening operator (g0 + g1 w)
#pragma unroll
        for (int v = 0; v < R; v++) u[v] = cmul(u[v], y[v]);
        fft_regs<R, false>(u, buf, tw, plan, j);
#pragma unroll
        for (int v = 0; v < R; v++) u[v] = cmul(u[v], __ldg(a.steep + j + v * T));
        fft_regs<R, true>(u, buf, tw, plan, j);
#pragma unroll
        for (int v = 0; v < R; v++) {
          k[v] = u[v];
          const int t = j + v * T;
          ACC[t] = s == 0 ? u[v] : caxpy(ACC[t], wgt, u[v]);
        }
      }
#pragma unroll
      for (int v = 0; v < R; v++) x[0][v] = caxpy(X[j + v * T], 1.0 / 6.0, ACC[j + v * T]);
      const bool last = i == a.nZ - 1;
      dispersion_step<1, R>(a, i, last, j, x, buf, plan, active, last ? a.dlast : a.dstep, tw);
      if (!last) {
#pragma unroll
        for (int v = 0; v < R; v++) X[j + v * T] = x[0][v];
        if (a.ckpt && i % a.ckK == 0)
          store_rows<1, R>(a.ckpt + (inst * a.ckN + i / a.ckK) * (long long)N, N, 0, N, T, j, x, 1.0, active);
      }
    }
    if (a.nZ == 1) {
      fft_regs<R, false>(x[0], buf, tw, plan, j);
#pragma unroll
      for (int v = 0; v < R; v++) x[0][v] = cmul(x[0][v], __ldg(a.back + j + v * T));
      if (a.gridF) store_rows<1, R>(a.gridF, ms, 0, N, T, j, x, (double)N, active);
      if (a.inTime || a.gridT) {
        fft_regs<R, true>(x[0], buf, tw, plan, j);
        if (a.gridT) store_rows<1, R>(a.gridT, ms, 0, N, T, j, x, 1.0, active);
      }
    }
    store_output<1, R>(a, inst, active, j, x, a.inTime ? 1.0 : (double)N);
    __syncthreads();
  }
}

void add_kernels_gnlse(std::vector<KernelEntry>& t) {
  t.push_back({kKindGnlse, kChi3GNLSE, 8, (const void*)k_propagate_gnlse<8>});
}

}  // namespace nlm
