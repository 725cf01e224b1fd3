// adjoint_cluster.cu -- the Chi2PDC reverse sweep (adjoint.cu) with each propagation spread over a
// cluster of C CTAs, the transforms being the four-step FFTs of nlm_cluster.cuh.  Used with the
// forwards that run on clusters (few rows on grids of 1024 to 8192 points), whose checkpoints it reads.
// Per segment between checkpoints the states are recomputed into per-cluster scratch (K > 1; nothing
// for K = 1), then the reverse steps run: the dispersion pair as cluster transforms, the transposed
// RK4 step point-wise in the time-domain ownership, with the stage-factor gradients added to d.ga.
// The state and gradient of a point are read and written by the thread that owns the point in the
// time domain, so the per-thread order of the scratch accesses is all the ordering they need.
#include <vector>

#include "nlm_adjoint_pdc.cuh"
#include "nlm_cluster.cuh"

namespace nlm {

// a.plan: the local M-point plan (M = N / C, C points per thread); a.tw: the N-point table.
// d.seg: [cluster][K][N] scratch when d.K > 1.
template <int C>
__global__ void __launch_bounds__(kMaxThreads) k_adjoint_pdc_cluster(const PropArgs a, const AdjArgs d) {
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
  const int K = d.K;
  const long long clusterId = blockIdx.x / C, nClusters = gridDim.x / C;
  double2* seg = K > 1 ? d.seg + clusterId * (long long)K * N : nullptr;
  for (long long local = clusterId; local < a.nInst; local += nClusters) {
    const long long inst = a.instBase + local;
    const double2* ck = d.ckpt + inst * (long long)d.nCk * N;
    double2 g[C];
    const double2* go = d.gout + inst * (long long)N;
#pragma unroll
    for (int v = 0; v < C; v++) g[v] = cscale(go[fk[v]], (double)N);
    int segEnd = a.nZ - 1;
    while (segEnd >= 1) {
      const int jseg = (segEnd - 1) / K, s0 = jseg * K;
      const double2* states = ck + (long long)s0 * N;   // K = 1: checkpoint i-1 is the state s_{i-1}
      if (K > 1) {
        // states s_{s0} .. s_{segEnd-1} into seg[0 ..]
        double2 x[C];
#pragma unroll
        for (int v = 0; v < C; v++) {
          x[v] = ck[(long long)jseg * N + tn[v]];
          seg[tn[v]] = x[v];
        }
        for (int i = s0 + 1; i < segEnd; i++) {
#pragma unroll
          for (int v = 0; v < C; v++) x[v] = pdc_step_point(a, N, i, tn[v], x[v]);
          cluster_fft_fwd<C>(f, x, cl);
#pragma unroll
          for (int v = 0; v < C; v++) x[v] = cmul(x[v], __ldg(a.dstep + fk[v]));
          cluster_fft_inv<C>(f, x, cl);
#pragma unroll
          for (int v = 0; v < C; v++) seg[(long long)(i - s0) * N + tn[v]] = x[v];
        }
        states = seg;
      }
      for (int i = segEnd; i > s0; i--) {
        const double2* prev = states + (long long)(i - 1 - s0) * N;
        if (i < a.nZ - 1) cluster_fft_fwd<C>(f, g, cl);
        const double2* tab = (i == a.nZ - 1) ? a.dlast : a.dstep;
#pragma unroll
        for (int v = 0; v < C; v++) g[v] = cmulc(g[v], __ldg(tab + fk[v]));
        cluster_fft_inv<C>(f, g, cl);
        if (d.gp) {   // marching form: P^T per point, the stage-factor gradients afterwards in parallel
#pragma unroll
          for (int v = 0; v < C; v++) g[v] = pdc_march_point(a, d, N, i, tn[v], inst, g[v], true);
          continue;
        }
        const double2* c = a.coef + (long long)(i - 1) * 3 * a.nCoef;
        const double2 c0 = c[0], c1 = c[1], c2 = c[2];
#pragma unroll
        for (int v = 0; v < C; v++) g[v] = pdc_reverse_point(a, d, N, i, tn[v], c0, c1, c2, prev[tn[v]], g[v], true);
      }
      segEnd = s0;
    }
    // gradient of the input spectrum: s_0 = IFFT(half X_in)
    cluster_fft_fwd<C>(f, g, cl);
#pragma unroll
    for (int v = 0; v < C; v++) d.gin[inst * (long long)N + fk[v]] = cmulc(g[v], __ldg(a.half + fk[v]));
  }
}

// Pipelined form for checkpoint intervals K > 1, on clusters of 2 C CTAs (two groups of C, as in
// k_adjoint_gnlse_cluster): ranks C..2C-1 recompute the states of segment j-1 from its checkpoint
// into one half of STG while ranks 0..C-1 reverse segment j from the other half.  Every transpose
// ends with a barrier of the whole cluster, so both groups run, per segment iteration, exactly K
// step slots of 2 transposes (a recomputed step: the forward and inverse transform of the dispersion
// step; a reverse step: the same pair, with a bare barrier in place of the forward transform for the
// last step, whose gradient starts in the frequency domain) and then one barrier; a slot without a
// step passes 2 bare barriers.  The final forward transform of the input gradient is matched by one
// bare barrier in the recomputing group.  d.seg: [cluster][2][K][N].
template <int C>
__global__ void __launch_bounds__(kMaxThreads) k_adjoint_pdc_cluster_pipe(const PropArgs a, const AdjArgs d) {
  extern __shared__ double2 smem[];
  cg::cluster_group cl = cg::this_cluster();
  const int crank = (int)cl.block_rank();
  const int role = crank / C;   // 0: reverse sweep, 1: recomputation
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
  const long long bufStride = (long long)K * N;
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
          for (int v = 0; v < C; v++) {
            x[v] = ck[(long long)jseg * N + tn[v]];
            stg[tn[v]] = x[v];
          }
          for (int q = 1; q <= K; q++) {
            const int i = s0 + q;
            if (i < segEnd) {
#pragma unroll
              for (int v = 0; v < C; v++) x[v] = pdc_step_point(a, N, i, tn[v], x[v]);
              cluster_fft_fwd<C>(f, x, cl);
#pragma unroll
              for (int v = 0; v < C; v++) x[v] = cmul(x[v], __ldg(a.dstep + fk[v]));
              cluster_fft_inv<C>(f, x, cl);
#pragma unroll
              for (int v = 0; v < C; v++) stg[(long long)q * N + tn[v]] = x[v];
            } else {
              cluster_idle(cl, 2);
            }
          }
        } else {
          cluster_idle(cl, 2 * K);
        }
      } else {
        if (it >= 1) {
          const int jseg = nSeg - it, s0 = jseg * K, segEnd = min(s0 + K, a.nZ - 1);
          const double2* stg = STG + (long long)((it - 1) & 1) * bufStride;
          for (int q = 0; q < K; q++) {
            const int i = segEnd - q;
            if (i > s0) {
              const double2* prev = stg + (long long)(i - 1 - s0) * N;
              if (i < a.nZ - 1) cluster_fft_fwd<C>(f, g, cl);
              else cl.sync();
              const double2* tab = (i == a.nZ - 1) ? a.dlast : a.dstep;
#pragma unroll
              for (int v = 0; v < C; v++) g[v] = cmulc(g[v], __ldg(tab + fk[v]));
              cluster_fft_inv<C>(f, g, cl);
              const double2* c = a.coef + (long long)(i - 1) * 3 * a.nCoef;
              const double2 c0 = c[0], c1 = c[1], c2 = c[2];
#pragma unroll
              for (int v = 0; v < C; v++)
                g[v] = pdc_reverse_point(a, d, N, i, tn[v], c0, c1, c2, prev[tn[v]], g[v], true);
            } else {
              cluster_idle(cl, 2);
            }
          }
        } else {
          cluster_idle(cl, 2 * K);
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

void add_kernels_adjoint_cluster(std::vector<KernelEntry>& t) {
  // key + 300: one propagation per cluster of four CTAs
  t.push_back({kKindAdjoint, kChi2PDC + 300, 4, (const void*)k_adjoint_pdc_cluster<4>});
  // key + 200: pipelined on clusters of eight CTAs (two groups of four)
  t.push_back({kKindAdjoint, kChi2PDC + 200, 4, (const void*)k_adjoint_pdc_cluster_pipe<4>});
}

}  // namespace nlm
