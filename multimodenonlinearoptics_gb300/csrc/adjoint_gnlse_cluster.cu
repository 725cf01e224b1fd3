// adjoint_gnlse_cluster.cu -- the pipelined Chi3GNLSE reverse sweep (solvers/Chi3GNLSE.cpp:39-92 run
// backwards) on clusters of eight CTAs: two groups of four, each group doing the four-step transforms
// of nlm_cluster.cuh over its four SMs.
//
//   group 1 (cluster ranks 4..7) marches segment j-1 forward from its checkpoint, keeping the state in
//           registers, and stores the stage inputs y_s and convolutions u2_s of every step;
//   group 0 (cluster ranks 0..3) runs the reverse steps of segment j from the stored stages, keeping
//           the gradient and the per-stage accumulators in registers.
// The adjoint algebra of a stage is the one of k_adjoint_gnlse (adjoint_gnlse.cu).  Both groups pass
// every cluster barrier of the other: a transpose ends with a barrier of the whole cluster.  So that
// the barrier counts agree by construction, both groups execute, per segment iteration, exactly K step
// slots of 18 transposes each (a forward step: 4 stages x 4 transforms + the dispersion pair; a reverse
// step: the dispersion pair + 4 x 4) followed by one barrier; a slot without a step (the idle group in
// the first and last iteration, a short last segment, the frequency-domain start of the reverse sweep)
// passes the same number of bare barriers.  The final forward transform of the input gradient is
// matched by one bare barrier in group 1.
// Scratch per cluster: STG[2][K][8][N] (double-buffered stage values).
// When the forward stored the stage values of every step (memory permitting), k_adjoint_gnlse_stored
// runs the reverse steps alone on clusters of four CTAs.
#include <vector>

#include "nlm_cluster.cuh"

namespace nlm {

namespace {

constexpr int kStepSyncs = 18;   // cluster barriers of one forward or reverse step

// Forward step i from the state x (time domain): stores y_s at Yi[s][N] and u2_s at Yi[4 + s][N] and
// advances x by the step (RK4, then the dispersion step).  18 transposes.
template <int C>
__device__ __forceinline__ void forward_step(const PropArgs& a, int i, int N, ClusterFFT<C>& f, cg::cluster_group& cl,
                                             const int (&tn)[C], const int (&fk)[C], double2 (&x)[C],
                                             double2* Yi) {
  const double* rel = a.relInt + (long long)(i - 1) * 3;
  double2 k[C], acc[C];
#pragma unroll
  for (int v = 0; v < C; v++) k[v] = czero();
  for (int s = 0; s < 4; s++) {
    const double fac = s == 0 ? 0.0 : (s == 3 ? 1.0 : 0.5);
    const double wgt = (s == 1 || s == 2) ? 2.0 : 1.0;
    const double ri = __ldg(rel + (s == 0 ? 0 : (s == 3 ? 2 : 1)));
    double2 y[C], u[C];
#pragma unroll
    for (int v = 0; v < C; v++) {
      y[v] = caxpy(x[v], fac, k[v]);
      Yi[(long long)s * N + tn[v]] = y[v];
      u[v] = make_double2(ri * cabs2(y[v]), 0.0);
    }
    cluster_fft_fwd<C>(f, u, cl);
#pragma unroll
    for (int v = 0; v < C; v++) u[v] = cmul(u[v], __ldg(a.raman + fk[v]));
    cluster_fft_inv<C>(f, u, cl);
#pragma unroll
    for (int v = 0; v < C; v++) {
      Yi[(long long)(4 + s) * N + tn[v]] = u[v];
      u[v] = cmul(u[v], y[v]);
    }
    cluster_fft_fwd<C>(f, u, cl);
#pragma unroll
    for (int v = 0; v < C; v++) u[v] = cmul(u[v], __ldg(a.steep + fk[v]));
    cluster_fft_inv<C>(f, u, cl);
#pragma unroll
    for (int v = 0; v < C; v++) {
      k[v] = u[v];
      acc[v] = s == 0 ? u[v] : caxpy(acc[v], wgt, u[v]);
    }
  }
#pragma unroll
  for (int v = 0; v < C; v++) x[v] = caxpy(x[v], 1.0 / 6.0, acc[v]);
  cluster_fft_fwd<C>(f, x, cl);
#pragma unroll
  for (int v = 0; v < C; v++) x[v] = cmul(x[v], __ldg(a.dstep + fk[v]));
  cluster_fft_inv<C>(f, x, cl);
}

// Reverse step i: g (time domain after the step; frequency domain for the last step) becomes the
// gradient with respect to the state before the step.  18 transposes (one bare barrier in place of
// the forward transform of the last step).
template <int C>
__device__ __forceinline__ void reverse_step(const PropArgs& a, int i, int N, ClusterFFT<C>& f, cg::cluster_group& cl,
                                             const int (&tn)[C], const int (&fk)[C], double2 (&g)[C],
                                             const double2* Yi) {
  const bool lastStep = i == a.nZ - 1;
  if (lastStep) cl.sync();
  else cluster_fft_fwd<C>(f, g, cl);
  const double2* tab = lastStep ? a.dlast : a.dstep;
#pragma unroll
  for (int v = 0; v < C; v++) g[v] = cmulc(g[v], __ldg(tab + fk[v]));
  cluster_fft_inv<C>(f, g, cl);
  const double* rel = a.relInt + (long long)(i - 1) * 3;
  double2 gxp[C], gke[C];
#pragma unroll
  for (int v = 0; v < C; v++) {
    gxp[v] = g[v];
    gke[v] = czero();
  }
  for (int s = 3; s >= 0; s--) {
    const double w = (s == 1 || s == 2) ? 2.0 / 6.0 : 1.0 / 6.0;
    const double fac = s == 0 ? 0.0 : (s == 3 ? 1.0 : 0.5);
    const double ri = __ldg(rel + (s == 0 ? 0 : (s == 3 ? 2 : 1)));
    double2 u[C], gy[C];
#pragma unroll
    for (int v = 0; v < C; v++) u[v] = caxpy(gke[v], w, gxp[v]);   // g_k_s
    cluster_fft_fwd<C>(f, u, cl);
#pragma unroll
    for (int v = 0; v < C; v++) u[v] = cmulc(u[v], __ldg(a.steep + fk[v]));
    cluster_fft_inv<C>(f, u, cl);                                   // g_u3
#pragma unroll
    for (int v = 0; v < C; v++) {
      const double2 y = Yi[(long long)s * N + tn[v]], u2 = Yi[(long long)(4 + s) * N + tn[v]];
      gy[v] = cmulc(u[v], u2);     // conj(u2) g_u3
      u[v] = cmulc(u[v], y);       // g_u2 = conj(y) g_u3
    }
    cluster_fft_fwd<C>(f, u, cl);
#pragma unroll
    for (int v = 0; v < C; v++) u[v] = cmulc(u[v], __ldg(a.raman + fk[v]));
    cluster_fft_inv<C>(f, u, cl);                                   // g_u1 (real part)
#pragma unroll
    for (int v = 0; v < C; v++) {
      const double2 y = Yi[(long long)s * N + tn[v]];
      gy[v] = caxpy(gy[v], 2.0 * ri * u[v].x, y);
      g[v] = cadd(g[v], gy[v]);
      gke[v] = cscale(gy[v], fac);
    }
  }
}

// Reverse step i in the frequency domain, for the sweep over stored stages: g (this thread's bins of
// the gradient with respect to the spectrum after the step) becomes the gradient with respect to the
// spectrum before it.  The transpose of the forward's frequency-domain RK4 sum: with h = N conj(D) g
// (D the dispersion factors, which carry the 1/N of a transform pair), stage s's spectrum gets w_s h
// plus the transform of the gradient its time-domain value takes through the next stage's input, and
// the spectrum before the step h plus the transform of the stage inputs' gradient.  16 transposes.
template <int C>
__device__ __forceinline__ void reverse_step_fs(const PropArgs& a, int i, int N, ClusterFFT<C>& f,
                                                cg::cluster_group& cl, const int (&tn)[C], const int (&fk)[C],
                                                double2 (&g)[C], const double2* Yi) {
  const double2* tab = i == a.nZ - 1 ? a.dlast : a.dstep;
  double2 h[C], gx[C], gke[C];
#pragma unroll
  for (int v = 0; v < C; v++) {
    h[v] = cscale(cmulc(g[v], __ldg(tab + fk[v])), (double)N);
    gx[v] = czero();
    gke[v] = czero();
  }
  const double* rel = a.relInt + (long long)(i - 1) * 3;
  for (int s = 3; s >= 0; s--) {
    const double w = (s == 1 || s == 2) ? 2.0 / 6.0 : 1.0 / 6.0;
    const double fac = s == 0 ? 0.0 : (s == 3 ? 1.0 : 0.5);
    const double ri = __ldg(rel + (s == 0 ? 0 : (s == 3 ? 2 : 1)));
    double2 u[C], gy[C];
    if (s < 3) {
#pragma unroll
      for (int v = 0; v < C; v++) u[v] = gke[v];
      cluster_fft_fwd<C>(f, u, cl);
#pragma unroll
      for (int v = 0; v < C; v++) u[v] = caxpy(u[v], w, h[v]);     // g_k_s (spectrum)
    } else {
#pragma unroll
      for (int v = 0; v < C; v++) u[v] = cscale(h[v], w);
    }
#pragma unroll
    for (int v = 0; v < C; v++) u[v] = cmulc(u[v], __ldg(a.steep + fk[v]));
    cluster_fft_inv<C>(f, u, cl);                                   // g_u3
#pragma unroll
    for (int v = 0; v < C; v++) {
      const double2 y = Yi[(long long)s * N + tn[v]], u2 = Yi[(long long)(4 + s) * N + tn[v]];
      gy[v] = cmulc(u[v], u2);     // conj(u2) g_u3
      u[v] = cmulc(u[v], y);       // g_u2 = conj(y) g_u3
    }
    cluster_fft_fwd<C>(f, u, cl);
#pragma unroll
    for (int v = 0; v < C; v++) u[v] = cmulc(u[v], __ldg(a.raman + fk[v]));
    cluster_fft_inv<C>(f, u, cl);                                   // g_u1 (real part)
#pragma unroll
    for (int v = 0; v < C; v++) {
      const double2 y = Yi[(long long)s * N + tn[v]];
      gy[v] = caxpy(gy[v], 2.0 * ri * u[v].x, y);
      gx[v] = cadd(gx[v], gy[v]);
      gke[v] = cscale(gy[v], fac);
    }
  }
  cluster_fft_fwd<C>(f, gx, cl);
#pragma unroll
  for (int v = 0; v < C; v++) g[v] = cadd(gx[v], h[v]);
}

}  // namespace

// a.plan: the local M-point plan (M = N / C, C points per thread); a.tw: the N-point table.
template <int C>
__global__ void __launch_bounds__(kMaxThreads) k_adjoint_gnlse_cluster(const PropArgs a, const AdjArgs d) {
  extern __shared__ double2 smem[];
  cg::cluster_group cl = cg::this_cluster();
  const int crank = (int)cl.block_rank();
  const int role = crank / C;   // 0: reverse sweep, 1: forward recomputation
  ClusterFFT<C> f;
  f.plan = &a.plan;
  const int M = a.plan.N, T = a.plan.T;
  const int N = M * C;
  f.rank = crank - role * C;
  f.base = role * C;
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
  int tn[C], fk[C];
#pragma unroll
  for (int v = 0; v < C; v++) {
    tn[v] = f.rank + C * (f.j + v * T);
    fk[v] = f.j + f.rank * T + M * v;
  }
  const int K = d.K;
  const long long clusterId = blockIdx.x / (2 * C), nClusters = gridDim.x / (2 * C);
  const long long stepStride = 8LL * N, bufStride = (long long)K * stepStride;
  double2* STG = d.seg + clusterId * 2 * bufStride;
  const int nSeg = (a.nZ - 2) / K + 1;
  for (long long local = clusterId; local < a.nInst; local += nClusters) {
    const long long inst = a.instBase + local;
    const double2* ck = d.ckpt + inst * (long long)d.nCk * N;
    double2 g[C];
    if (role == 0) {
      const double2* go = d.gout + inst * (long long)N;
#pragma unroll
      for (int v = 0; v < C; v++) g[v] = cscale(go[fk[v]], (double)N);
    }
    for (int it = 0; it <= nSeg; it++) {
      if (role == 1) {
        if (it < nSeg) {
          const int jseg = nSeg - 1 - it, s0 = jseg * K, segEnd = min(s0 + K, a.nZ - 1);
          double2* stg = STG + (long long)(it & 1) * bufStride;
          double2 x[C];
#pragma unroll
          for (int v = 0; v < C; v++) x[v] = ck[(long long)jseg * N + tn[v]];
          for (int q = 0; q < K; q++) {
            const int i = s0 + 1 + q;
            if (i <= segEnd) forward_step<C>(a, i, N, f, cl, tn, fk, x, stg + (long long)q * stepStride);
            else cluster_idle(cl, kStepSyncs);
          }
        } else {
          cluster_idle(cl, kStepSyncs * K);
        }
      } else {
        if (it >= 1) {
          const int jseg = nSeg - it, s0 = jseg * K, segEnd = min(s0 + K, a.nZ - 1);
          const double2* stg = STG + (long long)((it - 1) & 1) * bufStride;
          for (int q = 0; q < K; q++) {
            const int i = segEnd - q;
            if (i > s0) reverse_step<C>(a, i, N, f, cl, tn, fk, g, stg + (long long)(i - 1 - s0) * stepStride);
            else cluster_idle(cl, kStepSyncs);
          }
        } else {
          cluster_idle(cl, kStepSyncs * K);
        }
      }
      cl.sync();
    }
    if (role == 0) {
      cluster_fft_fwd<C>(f, g, cl);
#pragma unroll
      for (int v = 0; v < C; v++) d.gin[inst * (long long)N + fk[v]] = cmulc(g[v], __ldg(a.half + fk[v]));
    } else {
      cl.sync();
    }
  }
}

// Reverse sweep from stages stored by the forward (PropArgs::stages, written by the cluster forward
// kernel): nothing is recomputed; one propagation per cluster of C CTAs at a time.
template <int C>
__global__ void __launch_bounds__(kMaxThreads) k_adjoint_gnlse_stored(const PropArgs a, const AdjArgs d) {
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
  int tn[C], fk[C];
#pragma unroll
  for (int v = 0; v < C; v++) {
    tn[v] = f.rank + C * (f.j + v * T);
    fk[v] = f.j + f.rank * T + M * v;
  }
  const long long clusterId = blockIdx.x / C, nClusters = gridDim.x / C;
  for (long long local = clusterId; local < a.nInst; local += nClusters) {
    const long long inst = a.instBase + local;
    const double2* stg = a.stages + inst * (long long)(a.nZ - 1) * 8 * N;
    double2 g[C];
    const double2* go = d.gout + inst * (long long)N;
#pragma unroll
    for (int v = 0; v < C; v++) g[v] = cscale(go[fk[v]], (double)N);
    for (int i = a.nZ - 1; i >= 1; i--)
      reverse_step_fs<C>(a, i, N, f, cl, tn, fk, g, stg + (long long)(i - 1) * 8 * N);
    // g: the gradient of the input spectrum, times half a dispersion step
#pragma unroll
    for (int v = 0; v < C; v++) d.gin[inst * (long long)N + fk[v]] = cmulc(g[v], __ldg(a.half + fk[v]));
  }
}

void add_kernels_adjoint_gnlse_cluster(std::vector<KernelEntry>& t) {
  // key + 200: eight-CTA clusters, two groups of four
  t.push_back({kKindAdjoint, kChi3GNLSE + 200, 4, (const void*)k_adjoint_gnlse_cluster<4>});
  // key + 300: four-CTA clusters over stored stages
  t.push_back({kKindAdjoint, kChi3GNLSE + 300, 4, (const void*)k_adjoint_gnlse_stored<4>});
}

}  // namespace nlm
