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

void add_kernels_adjoint_cluster(std::vector<KernelEntry>& t) {
  // key + 300: one propagation per cluster of four CTAs
  t.push_back({kKindAdjoint, kChi2PDC + 300, 4, (const void*)k_adjoint_pdc_cluster<4>});
}

}  // namespace nlm
