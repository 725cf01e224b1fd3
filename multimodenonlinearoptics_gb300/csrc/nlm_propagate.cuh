// nlm_propagate.cuh -- the fused split-step kernels.
//
// One thread group of T = N/R threads owns one propagation (one impulse of
// computeGreensFunction, one row of batchSignalSimulation, or the single signal of
// runSignalSimulation).  A CTA holds `ipc` groups; a persistent grid walks over the
// groups.  Per z step (src/_NonlinearMedium.hpp:204-233) each group does, without
// leaving registers except for the FFT exchanges:
//     RK4 nonlinear step (point-wise)  ->  FFT  ->  x dispStep/N  ->  inverse FFT
// The RK4 step is either the solver's DiffEq evaluated four times per point
// (k_propagate_direct) or, for the pump-driven ("linear") solvers, the exact real-linear
// map that one RK4 step applies to (Re a, Im a) at a point, precomputed once per pump
// and shared by every propagation (k_propagate_linear).
#pragma once
#include "nlm_device.cuh"
#include "nlm_kernels.h"
#include "nlm_solvers.cuh"

namespace nlm {

constexpr int kMaxThreads = 512;   // launch bound of every propagation kernel

// Next group of propagations for this CTA: static round robin, or the next free group of a
// work counter shared by the grid (first group = blockIdx.x, then atomically claimed ones).
// Called by all threads of the CTA in uniform control flow.
__device__ __forceinline__ long long next_group(const PropArgs& a, long long cg, long long* slot) {
  if (a.work == nullptr) return cg + gridDim.x;
  __syncthreads();   // everyone has read the previous value of *slot
  if (threadIdx.x == 0) *slot = (long long)atomicAdd(a.work, 1ULL) + gridDim.x;
  __syncthreads();
  return *slot;
}

// Twiddle table of the transforms: staged in shared memory (in front of the exchange buffers) for
// R <= 8, i.e. N <= 4096, so that the passes read it with shared-memory loads instead of loading it
// through the L1/texture path, whose queue otherwise throttles the warps; left in global memory for
// R = 16 (N = 8192), where the table would not fit next to the buffer.
template <int R>
__device__ __forceinline__ const double2* stage_twiddles(const double2* __restrict__ tw, double2* smem, int N,
                                                         double2** bufs) {
  if constexpr (R != 16) {
    for (int k = threadIdx.x; k < N; k += blockDim.x) smem[k] = tw[k];
    __syncthreads();
    *bufs = smem + N;
    return smem;
  } else {
    *bufs = smem;
    return tw;
  }
}

// Input of one propagation, in the frequency domain and pre-multiplied by exp(+i dz/2 D)/N
// (src/_NonlinearMedium.hpp:169-192).
// GEN: the general plan (padded ownership): points j + v*T at or past N are not loaded or stored.
template <int M, int R, bool GEN = false>
__device__ __forceinline__ void load_input(const PropArgs& a, long long inst, bool active, int j,
                                           double2 (&x)[M][R], double2* buf, const FFTPlanH& plan,
                                           const double2* tw) {
  const int N = plan.N, T = plan.T;
  if (a.inKind == 0) {
    // impulses: instance = ((im * N) + bin) * 2 + which; value 1 (which 0) or i (which 1)
    const long long pair = inst >> 1;
    const int bin = (int)(pair % N);
    const int im = (int)(pair / N);
    const int mode = active ? a.impModes[im < kMaxModes ? im : 0] : -1;
    const double2 val = (inst & 1) ? make_double2(0.0, 1.0) : make_double2(1.0, 0.0);
#pragma unroll
    for (int m = 0; m < M; m++)
#pragma unroll
      for (int v = 0; v < R; v++) x[m][v] = (m == mode && j + v * T == bin) ? val : czero();
  } else {
    const double2* row = a.in + (active ? inst : 0) * a.inStride;
#pragma unroll
    for (int m = 0; m < M; m++) {
      int seg = -1;
      if (m == a.inputMode) seg = 0;
      else if (a.inputMode < 1 && m < a.inChannels) seg = m;
#pragma unroll
      for (int v = 0; v < R; v++)
        x[m][v] = (active && seg >= 0 && (!GEN || j + v * T < N)) ? row[(long long)seg * N + j + v * T] : czero();
    }
  }
#pragma unroll
  for (int m = 0; m < M; m++) {
    if (a.inTime) fft_any<R, false, GEN>(x[m], buf, tw, plan, j);
    const double2* h = a.half + (long long)m * N;
#pragma unroll
    for (int v = 0; v < R; v++) x[m][v] = cmul(x[m][v], __ldg(h + j + v * T));
  }
}

template <int M, int R, bool GEN = false>
__device__ __forceinline__ void store_rows(double2* base, long long modeStride, int row, int N, int T, int j,
                                           const double2 (&x)[M][R], double scale, bool active) {
  if (!active) return;
#pragma unroll
  for (int m = 0; m < M; m++)
#pragma unroll
    for (int v = 0; v < R; v++)
      if (!GEN || j + v * T < N) base[m * modeStride + (long long)row * N + j + v * T] = cscale(x[m][v], scale);
}

template <int M, int R, bool GEN = false>
__device__ __forceinline__ void store_output(const PropArgs& a, long long inst, bool active, int j,
                                             const double2 (&x)[M][R], double scale) {
  if (!active || a.out == nullptr) return;
  const int N = a.plan.N, T = a.plan.T;
  double2* o = a.out + inst * a.outStride;
  for (int om = 0; om < a.nOut; om++) {
    const int mode = a.outModes[om];
#pragma unroll
    for (int m = 0; m < M; m++) {
      if (m != mode) continue;
#pragma unroll
      for (int v = 0; v < R; v++)
        if (!GEN || j + v * T < N) o[(long long)om * N + j + v * T] = cscale(x[m][v], scale);
    }
  }
}

// Dispersion half of a step for all modes: FFT, multiply, optional inverse FFT and grid rows.
template <int M, int R, bool GEN = false>
__device__ __forceinline__ void dispersion_step(const PropArgs& a, int i, bool last, int j, double2 (&x)[M][R],
                                                double2* buf, const FFTPlanH& plan, bool active, const double2* table,
                                                const double2* tw) {
  const int N = plan.N, T = plan.T;
  const bool wantTime = !last || a.inTime || a.gridT != nullptr;
#pragma unroll
  for (int m = 0; m < M; m++) {
    fft_any<R, false, GEN>(x[m], buf, tw, plan, j);
    const double2* d = table + (long long)m * N;
#pragma unroll
    for (int v = 0; v < R; v++) x[m][v] = cmul(x[m][v], __ldg(d + j + v * T));
  }
  const long long ms = (long long)a.nZ * N;
  if (a.gridF) store_rows<M, R, GEN>(a.gridF, ms, i, N, T, j, x, (double)N, active);
  if (wantTime) {
#pragma unroll
    for (int m = 0; m < M; m++) fft_any<R, true, GEN>(x[m], buf, tw, plan, j);
    if (a.gridT) store_rows<M, R, GEN>(a.gridT, ms, i, N, T, j, x, 1.0, active);
  }
}

// One RK4 step at a point with the solver's right-hand side (src/_NonlinearMedium.hpp:207-210).
template <class S>
__device__ __forceinline__ void rk4_point(double2 (&x)[S::kM], const double2 (&p)[3][S::kP > 0 ? S::kP : 1],
                                          const double2* __restrict__ c) {
  constexpr int M = S::kM, C = S::kC;
  double2 k[M], y[M], acc[M];
  S::f(x, p[0], c, k);
#pragma unroll
  for (int m = 0; m < M; m++) {
    acc[m] = k[m];
    y[m] = caxpy(x[m], 0.5, k[m]);
  }
  S::f(y, p[1], c + C, k);
#pragma unroll
  for (int m = 0; m < M; m++) {
    acc[m] = caxpy(acc[m], 2.0, k[m]);
    y[m] = caxpy(x[m], 0.5, k[m]);
  }
  S::f(y, p[1], c + C, k);
#pragma unroll
  for (int m = 0; m < M; m++) {
    acc[m] = caxpy(acc[m], 2.0, k[m]);
    y[m] = cadd(x[m], k[m]);
  }
  S::f(y, p[2], c + 2 * C, k);
#pragma unroll
  for (int m = 0; m < M; m++) {
    acc[m] = cadd(acc[m], k[m]);
    x[m] = caxpy(x[m], 1.0 / 6.0, acc[m]);
  }
}

// --------------------------------------------------------------------------------------------
// Direct kernel: every solver except Chi3GNLSE.
// --------------------------------------------------------------------------------------------
template <class S, int R, bool GEN = false>
__global__ void __launch_bounds__(kMaxThreads) k_propagate_direct(const PropArgs a) {
  constexpr int M = S::kM, P = S::kP > 0 ? S::kP : 1;
  extern __shared__ double2 smem[];
  const FFTPlanH& plan = a.plan;
  const int N = plan.N, T = plan.T;
  const int g = threadIdx.x / T, j = threadIdx.x - g * T;
  double2* bufs;
  const double2* tw = stage_twiddles<R>(a.tw, smem, N, &bufs);
  double2* buf = bufs + (long long)g * N;
  const long long nGroups = (a.nInst + a.ipc - 1) / a.ipc;
  __shared__ long long s_group;
  for (long long cg = blockIdx.x; cg < nGroups; cg = next_group(a, cg, &s_group)) {
    const long long local = cg * a.ipc + g;
    const bool active = local < a.nInst;
    const long long inst = a.instBase + local;
    double2 x[M][R];
    load_input<M, R, GEN>(a, inst, active, j, x, buf, plan, tw);
    const long long ms = (long long)a.nZ * N;
    if (a.gridF) store_rows<M, R, GEN>(a.gridF, ms, 0, N, T, j, x, (double)N, active);
#pragma unroll
    for (int m = 0; m < M; m++) fft_any<R, true, GEN>(x[m], buf, tw, plan, j);
    if (a.gridT) store_rows<M, R, GEN>(a.gridT, ms, 0, N, T, j, x, 1.0, active);
    if (a.ckpt && a.nZ > 1) store_rows<M, R, GEN>(a.ckpt + inst * a.ckN * M * (long long)N, N, 0, N, T, j, x, 1.0, active);
    for (int i = 1; i < a.nZ; i++) {
      const double2* c = a.coef + (long long)(i - 1) * 3 * a.nCoef;
#pragma unroll
      for (int v = 0; v < R; v++) {
        const int t = j + v * T;
        double2 p[3][P];
#pragma unroll
        for (int q = 0; q < P; q++) {
          if (S::kP > 0) {
            const double2* pr = a.pump + q * a.pumpStride + (long long)(2 * i - 2) * N + t;
            p[0][q] = __ldg(pr);
            p[1][q] = __ldg(pr + N);
            p[2][q] = __ldg(pr + 2 * N);
          } else {
            p[0][q] = p[1][q] = p[2][q] = czero();
          }
        }
        double2 xm[M];
#pragma unroll
        for (int m = 0; m < M; m++) xm[m] = x[m][v];
        rk4_point<S>(xm, p, c);
#pragma unroll
        for (int m = 0; m < M; m++) x[m][v] = xm[m];
      }
      const bool last = i == a.nZ - 1;
      dispersion_step<M, R, GEN>(a, i, last, j, x, buf, plan, active, last ? a.dlast : a.dstep, tw);
      if (a.ckpt && !last && i % a.ckK == 0)
        store_rows<M, R, GEN>(a.ckpt + (inst * a.ckN + i / a.ckK) * M * (long long)N, N, 0, N, T, j, x, 1.0, active);
    }
    if (a.nZ == 1) {
#pragma unroll
      for (int m = 0; m < M; m++) fft_any<R, false, GEN>(x[m], buf, tw, plan, j);
      // x now holds X_in * exp(+i dz/2 D); the factor tables are pre-divided by N
#pragma unroll
      for (int m = 0; m < M; m++)
#pragma unroll
        for (int v = 0; v < R; v++) x[m][v] = cmul(x[m][v], __ldg(a.back + (long long)m * N + j + v * T));
      if (a.gridF) store_rows<M, R, GEN>(a.gridF, ms, 0, N, T, j, x, (double)N, active);
      if (a.inTime || a.gridT) {
#pragma unroll
        for (int m = 0; m < M; m++) fft_any<R, true, GEN>(x[m], buf, tw, plan, j);
        if (a.gridT) store_rows<M, R, GEN>(a.gridT, ms, 0, N, T, j, x, 1.0, active);
      }
    }
    store_output<M, R, GEN>(a, inst, active, j, x, a.inTime ? 1.0 : (double)N);
    __syncthreads();
  }
}

// --------------------------------------------------------------------------------------------
// Linear kernel: pump-driven solvers with the precomputed per-point RK4 map.
// prop layout: [step][E/2][N] double2, word w = row * M + c holding the entries (row, 2c), (row, 2c+1)
// of the (2M)x(2M) real matrix over (Re a0, Im a0, Re a1, ...).
// --------------------------------------------------------------------------------------------
// CK: the forward checkpoints of the adjoint (PropArgs::ckpt) are written; a separate instantiation,
// so that the other launches carry no per-step test.
template <int M, int R, bool CK = false, bool GEN = false>
__device__ __forceinline__ void linear_body(const PropArgs& a) {
  constexpr int D = 2 * M, E = D * D;
  extern __shared__ double2 smem[];
  const FFTPlanH& plan = a.plan;
  const int N = plan.N, T = plan.T;
  const int g = threadIdx.x / T, j = threadIdx.x - g * T;
  double2* bufs;
  const double2* tw = stage_twiddles<R>(a.tw, smem, N, &bufs);
  double2* buf = bufs + (long long)g * N;
  const long long nGroups = (a.nInst + a.ipc - 1) / a.ipc;
  __shared__ long long s_group;
  for (long long cg = blockIdx.x; cg < nGroups; cg = next_group(a, cg, &s_group)) {
    const long long local = cg * a.ipc + g;
    const bool active = local < a.nInst;
    const long long inst = a.instBase + local;
    double2 x[M][R];
    load_input<M, R, GEN>(a, inst, active, j, x, buf, plan, tw);
    const long long ms = (long long)a.nZ * N;
    if (a.gridF) store_rows<M, R, GEN>(a.gridF, ms, 0, N, T, j, x, (double)N, active);
#pragma unroll
    for (int m = 0; m < M; m++) fft_any<R, true, GEN>(x[m], buf, tw, plan, j);
    if (a.gridT) store_rows<M, R, GEN>(a.gridT, ms, 0, N, T, j, x, 1.0, active);
    if (CK && a.nZ > 1) store_rows<M, R, GEN>(a.ckpt + inst * a.ckN * M * (long long)N, N, 0, N, T, j, x, 1.0, active);
    for (int i = 1; i < a.nZ; i++) {
      // entries stored as pairs (row r, columns 2c and 2c+1) so a point loads D*D/2 16-byte words
      const double2* mat = reinterpret_cast<const double2*>(a.prop) + (long long)(i - 1) * (E / 2) * N;
#pragma unroll
      for (int v = 0; v < R; v++) {
        const int t = j + v * T;
        double in[D], outv[D];
#pragma unroll
        for (int m = 0; m < M; m++) {
          in[2 * m] = x[m][v].x;
          in[2 * m + 1] = x[m][v].y;
        }
#pragma unroll
        for (int r = 0; r < D; r++) {
          const double2 e0 = __ldg(mat + (long long)(r * (D / 2)) * N + t);
          double s = fma(e0.y, in[1], e0.x * in[0]);
#pragma unroll
          for (int c = 1; c < D / 2; c++) {
            const double2 e = __ldg(mat + (long long)(r * (D / 2) + c) * N + t);
            s = fma(e.x, in[2 * c], s);
            s = fma(e.y, in[2 * c + 1], s);
          }
          outv[r] = s;
        }
#pragma unroll
        for (int m = 0; m < M; m++) x[m][v] = make_double2(outv[2 * m], outv[2 * m + 1]);
      }
      const bool last = i == a.nZ - 1;
      dispersion_step<M, R, GEN>(a, i, last, j, x, buf, plan, active, last ? a.dlast : a.dstep, tw);
      if (CK && !last && i % a.ckK == 0)
        store_rows<M, R, GEN>(a.ckpt + (inst * a.ckN + i / a.ckK) * M * (long long)N, N, 0, N, T, j, x, 1.0, active);
    }
    if (a.nZ == 1) {
#pragma unroll
      for (int m = 0; m < M; m++) fft_any<R, false, GEN>(x[m], buf, tw, plan, j);
#pragma unroll
      for (int m = 0; m < M; m++)
#pragma unroll
        for (int v = 0; v < R; v++) x[m][v] = cmul(x[m][v], __ldg(a.back + (long long)m * N + j + v * T));
      if (a.inTime) {
#pragma unroll
        for (int m = 0; m < M; m++) fft_any<R, true, GEN>(x[m], buf, tw, plan, j);
      }
    }
    store_output<M, R, GEN>(a, inst, active, j, x, a.inTime ? 1.0 : (double)N);
    __syncthreads();
  }
}

template <int M, int R, bool CK = false, bool GEN = false>
__global__ void __launch_bounds__(kMaxThreads) k_propagate_linear(const PropArgs a) {
  linear_body<M, R, CK, GEN>(a);
}

// The same kernel compiled for 128-thread CTAs with at least MINB of them resident per SM: fewer
// registers per thread, more warps to hide the shared-memory phases of the transforms.  The
// autotuner times it against k_propagate_linear where a CTA has 128 threads.
template <int M, int R, int MINB>
__global__ void __launch_bounds__(128, MINB) k_propagate_linear_occ(const PropArgs a) {
  linear_body<M, R>(a);
}

// --------------------------------------------------------------------------------------------
// Propagator build: for every (step, point), apply one RK4 step to the 2M real unit vectors.
// One thread per (step, point).
// --------------------------------------------------------------------------------------------
template <class S>
__global__ void k_build_propagator(const PropArgs a) {
  constexpr int M = S::kM, P = S::kP > 0 ? S::kP : 1, D = 2 * M, E = D * D;
  const int N = a.plan.N;
  const long long total = (long long)(a.nZ - 1) * N;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(idx / N) + 1;
    const int t = (int)(idx - (long long)(i - 1) * N);
    double2 p[3][P];
#pragma unroll
    for (int q = 0; q < P; q++) {
      const double2* pr = a.pump + q * a.pumpStride + (long long)(2 * i - 2) * N + t;
      p[0][q] = pr[0];
      p[1][q] = pr[N];
      p[2][q] = pr[2 * N];
    }
    const double2* c = a.coef + (long long)(i - 1) * 3 * a.nCoef;
    double cols[D][D];   // cols[col][row]
#pragma unroll
    for (int col = 0; col < D; col++) {
      double2 xm[M];
#pragma unroll
      for (int m = 0; m < M; m++) xm[m] = czero();
      xm[col / 2] = (col & 1) ? make_double2(0.0, 1.0) : make_double2(1.0, 0.0);
      rk4_point<S>(xm, p, c);
#pragma unroll
      for (int m = 0; m < M; m++) {
        cols[col][2 * m] = xm[m].x;
        cols[col][2 * m + 1] = xm[m].y;
      }
    }
    double2* mat = reinterpret_cast<double2*>(const_cast<double*>(a.prop)) + (long long)(i - 1) * (E / 2) * N + t;
#pragma unroll
    for (int r = 0; r < D; r++)
#pragma unroll
      for (int cc = 0; cc < D / 2; cc++)
        mat[(long long)(r * (D / 2) + cc) * N] = make_double2(cols[2 * cc][r], cols[2 * cc + 1][r]);
  }
}

}  // namespace nlm
