// nlm_cluster.cuh -- one propagation spread over a thread-block cluster of C CTAs (C SMs).
//
// A single propagation is a sequential z march; on one SM it runs at that SM's FP64 rate (2 DFMA
// lanes per clock on this part), no faster than a CPU core.  Here the N-point field is split over
// the C CTAs of a cluster and every transform is a four-step FFT (N = C M):
//   time domain:       CTA c, thread j, register v  <->  point n = c + C (j + v T)       (T = M / C)
//   frequency domain:  CTA c, thread j, register v  <->  bin   k = j + c T + M v
// forward:  M-point FFT of the CTA's strided points (register Stockham, as in the one-CTA kernels),
//           twiddle exp(-2 pi i c k2 / N), transpose over the cluster (thread j of CTA c sends its
//           register v to thread j of CTA v through distributed shared memory), C-point DFT over the
//           registers;
// inverse:  the same steps in reverse order with conjugate twiddles (unscaled, 1/N is in the tables).
// With R = C points per thread the transpose is one value per (thread, CTA) pair.  Each transpose
// writes a receive buffer of the destination CTA and ends with one cluster barrier (hardware,
// release/acquire at cluster scope); the buffers alternate between two halves, so a CTA never
// overwrites a half that another CTA is still reading (that CTA passed the barrier in between).
// Point-wise work (RK4 with the solver's DiffEq, or the precomputed RK4 matrices of the pump-driven
// solvers; dispersion tables) indexes the global arrays with the maps above.
#pragma once
#include <cooperative_groups.h>

#include "nlm_propagate.cuh"

namespace cg = cooperative_groups;

namespace nlm {

template <int C>
struct ClusterFFT {
  const double2* twM;   // [M] exp(-2 pi i m / M)
  const double2* twC;   // [M] exp(-2 pi i c k2 / N) of this CTA's rank c
  double2* buf;         // [M] Stockham exchange buffer of the local transforms
  double2* recv;        // [2][C][T] transpose receive buffers
  const FFTPlanH* plan; // the local M-point plan (R = C): the kernel parameter's, indexed in place
  int rank, j, phase;
  int base = 0;         // cluster rank of the group's first CTA (clusters holding several groups)
};

template <int C>
__device__ __forceinline__ void cluster_transpose(ClusterFFT<C>& f, double2 (&x)[C], cg::cluster_group& cl) {
  const int T = f.plan->T;
  double2* half = f.recv + (long long)f.phase * C * T;
#pragma unroll
  for (int v = 0; v < C; v++) {
    double2* dst = cl.map_shared_rank(half + f.rank * T + f.j, f.base + v);
    *dst = x[v];
  }
  cl.sync();
#pragma unroll
  for (int c = 0; c < C; c++) x[c] = half[c * T + f.j];
  f.phase ^= 1;
}

// n bare cluster barriers: the slots of a group that has no transform to do while the other group of
// the same cluster does (every transpose ends with a barrier of the whole cluster)
__device__ __forceinline__ void cluster_idle(cg::cluster_group& cl, int n) {
  for (int q = 0; q < n; q++) cl.sync();
}

// time-domain ownership -> frequency-domain ownership
template <int C>
__device__ __forceinline__ void cluster_fft_fwd(ClusterFFT<C>& f, double2 (&x)[C], cg::cluster_group& cl) {
  fft_regs<C, false>(x, f.buf, f.twM, *f.plan, f.j);
#pragma unroll
  for (int v = 0; v < C; v++) x[v] = cmul(x[v], f.twC[f.j + v * f.plan->T]);
  cluster_transpose<C>(f, x, cl);
  dft_r<C, false>(x, 0, 1);
}

// frequency-domain ownership -> time-domain ownership (unscaled)
template <int C>
__device__ __forceinline__ void cluster_fft_inv(ClusterFFT<C>& f, double2 (&x)[C], cg::cluster_group& cl) {
  dft_r<C, true>(x, 0, 1);
  cluster_transpose<C>(f, x, cl);
#pragma unroll
  for (int v = 0; v < C; v++) x[v] = cmulc(x[v], f.twC[f.j + v * f.plan->T]);
  fft_regs<C, true>(x, f.buf, f.twM, *f.plan, f.j);
}

// a.plan is the local M-point plan; a.tw the N-point table.  One propagation per cluster at a time.
template <class S, int C>
__global__ void __launch_bounds__(kMaxThreads) k_propagate_cluster(const PropArgs a) {
  constexpr int MD = S::kM, P = S::kP > 0 ? S::kP : 1, R = C;
  extern __shared__ double2 smem[];
  cg::cluster_group cl = cg::this_cluster();
  ClusterFFT<C> f;
  f.plan = &a.plan;
  const int M = a.plan.N, T = a.plan.T;
  const int N = M * C;
  f.rank = (int)cl.block_rank();
  f.j = threadIdx.x;
  f.phase = 0;
  double2* twM = smem;
  double2* twC = smem + M;
  f.buf = smem + 2 * M;
  f.recv = smem + 3 * M;
  for (int k = threadIdx.x; k < M; k += blockDim.x) {
    twM[k] = a.tw[(long long)k * C];
    twC[k] = a.tw[(long long)f.rank * k];
  }
  __syncthreads();
  f.twM = twM;
  f.twC = twC;
  const int j = f.j, rank = f.rank;
  const long long clusterId = blockIdx.x / C, nClusters = gridDim.x / C;
  const long long ms = (long long)a.nZ * N;
  // global index of register v in the time / frequency domain
  auto tn = [&](int v) { return rank + C * (j + v * T); };
  auto fk = [&](int v) { return j + rank * T + M * v; };
  for (long long local = clusterId; local < a.nInst; local += nClusters) {
    const long long inst = a.instBase + local;
    double2 x[MD][R];
    const double2* row = a.in + inst * a.inStride;
#pragma unroll
    for (int m = 0; m < MD; m++) {
      int seg = -1;
      if (m == a.inputMode) seg = 0;
      else if (a.inputMode < 1 && m < a.inChannels) seg = m;
#pragma unroll
      for (int v = 0; v < R; v++)
        x[m][v] = seg >= 0 ? row[(long long)seg * N + (a.inTime ? tn(v) : fk(v))] : czero();
      if (a.inTime) cluster_fft_fwd<C>(f, x[m], cl);
#pragma unroll
      for (int v = 0; v < R; v++) x[m][v] = cmul(x[m][v], __ldg(a.half + (long long)m * N + fk(v)));
    }
    if (a.gridF) {
#pragma unroll
      for (int m = 0; m < MD; m++)
#pragma unroll
        for (int v = 0; v < R; v++) a.gridF[m * ms + fk(v)] = cscale(x[m][v], (double)N);
    }
#pragma unroll
    for (int m = 0; m < MD; m++) cluster_fft_inv<C>(f, x[m], cl);
    if (a.gridT) {
#pragma unroll
      for (int m = 0; m < MD; m++)
#pragma unroll
        for (int v = 0; v < R; v++) a.gridT[m * ms + tn(v)] = x[m][v];
    }
    // checkpoints for the reverse sweep: the time-domain state before steps 1, K + 1, 2 K + 1, ...
    double2* ckRow = a.ckpt ? a.ckpt + inst * a.ckN * MD * (long long)N : nullptr;
    if (ckRow && a.nZ > 1) {
#pragma unroll
      for (int m = 0; m < MD; m++)
#pragma unroll
        for (int v = 0; v < R; v++) ckRow[(long long)m * N + tn(v)] = x[m][v];
    }
    for (int i = 1; i < a.nZ; i++) {
      if (a.prop) {
        // pump-driven solvers: the RK4 step as its per-point real (2M)x(2M) matrix, stored as pairs
        // (row r, columns 2c and 2c+1) at [step][r * M + c][N]
        constexpr int D = 2 * MD;
        const double2* mat = reinterpret_cast<const double2*>(a.prop) + (long long)(i - 1) * (D * D / 2) * N;
#pragma unroll
        for (int v = 0; v < R; v++) {
          const int t = tn(v);
          double in[D], outv[D];
#pragma unroll
          for (int m = 0; m < MD; m++) {
            in[2 * m] = x[m][v].x;
            in[2 * m + 1] = x[m][v].y;
          }
#pragma unroll
          for (int r = 0; r < D; r++) {
            double acc = 0.0;
#pragma unroll
            for (int cc = 0; cc < D / 2; cc++) {
              const double2 e = __ldg(mat + (long long)(r * (D / 2) + cc) * N + t);
              acc = fma(e.x, in[2 * cc], acc);
              acc = fma(e.y, in[2 * cc + 1], acc);
            }
            outv[r] = acc;
          }
#pragma unroll
          for (int m = 0; m < MD; m++) x[m][v] = make_double2(outv[2 * m], outv[2 * m + 1]);
        }
      } else {
        const double2* c = a.coef + (long long)(i - 1) * 3 * a.nCoef;
#pragma unroll
        for (int v = 0; v < R; v++) {
          const int t = tn(v);
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
          double2 xm[MD];
#pragma unroll
          for (int m = 0; m < MD; m++) xm[m] = x[m][v];
          rk4_point<S>(xm, p, c);
#pragma unroll
          for (int m = 0; m < MD; m++) x[m][v] = xm[m];
        }
      }
      const bool last = i == a.nZ - 1;
      const double2* table = last ? a.dlast : a.dstep;
      const bool wantTime = !last || a.inTime || a.gridT != nullptr;
#pragma unroll
      for (int m = 0; m < MD; m++) {
        cluster_fft_fwd<C>(f, x[m], cl);
#pragma unroll
        for (int v = 0; v < R; v++) x[m][v] = cmul(x[m][v], __ldg(table + (long long)m * N + fk(v)));
        if (a.gridF) {
#pragma unroll
          for (int v = 0; v < R; v++) a.gridF[m * ms + (long long)i * N + fk(v)] = cscale(x[m][v], (double)N);
        }
        if (wantTime) {
          cluster_fft_inv<C>(f, x[m], cl);
          if (a.gridT) {
#pragma unroll
            for (int v = 0; v < R; v++) a.gridT[m * ms + (long long)i * N + tn(v)] = x[m][v];
          }
        }
        if (ckRow && !last && i % a.ckK == 0) {
#pragma unroll
          for (int v = 0; v < R; v++) ckRow[((long long)(i / a.ckK) * MD + m) * N + tn(v)] = x[m][v];
        }
      }
    }
    if (a.nZ == 1) {
#pragma unroll
      for (int m = 0; m < MD; m++) {
        cluster_fft_fwd<C>(f, x[m], cl);
#pragma unroll
        for (int v = 0; v < R; v++) x[m][v] = cmul(x[m][v], __ldg(a.back + (long long)m * N + fk(v)));
        if (a.gridF) {
#pragma unroll
          for (int v = 0; v < R; v++) a.gridF[m * ms + fk(v)] = cscale(x[m][v], (double)N);
        }
        if (a.inTime || a.gridT) {
          cluster_fft_inv<C>(f, x[m], cl);
          if (a.gridT) {
#pragma unroll
            for (int v = 0; v < R; v++) a.gridT[m * ms + tn(v)] = x[m][v];
          }
        }
      }
    }
    // the last row is in the time domain when the input was, else in the frequency domain
    if (a.out) {
      double2* o = a.out + inst * a.outStride;
      const double sc = a.inTime ? 1.0 : (double)N;
      for (int om = 0; om < a.nOut; om++) {
#pragma unroll
        for (int m = 0; m < MD; m++) {
          if (m != a.outModes[om]) continue;
#pragma unroll
          for (int v = 0; v < R; v++) o[(long long)om * N + (a.inTime ? tn(v) : fk(v))] = cscale(x[m][v], sc);
        }
      }
    }
  }
}

}  // namespace nlm
