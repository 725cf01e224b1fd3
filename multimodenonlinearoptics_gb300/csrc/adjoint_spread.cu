// adjoint_spread.cu -- the Chi2PDC reverse sweep (adjoint.cu) with each propagation on a cluster of four
// CTAs holding one point per thread (nlm_spread.cuh): the reverse of the forwards that run on the
// spread kernels (few rows on grids of 128 to 1024 points), whose checkpoints it reads.  Same steps as
// adjoint_cluster.cu: per segment between checkpoints the states are recomputed into per-cluster scratch
// (K > 1), then the reverse steps run: the dispersion pair as spread transforms, the transposed RK4 step
// point-wise in the time-domain ownership (the marching form with every state stored: P^T per point,
// the stage-factor gradients in a parallel launch afterwards).  The state and gradient of a point are
// read and written by the thread that owns the point in the time domain.
#include <vector>

#include "nlm_adjoint_pdc.cuh"
#include "nlm_spread.cuh"

namespace nlm {

// a.plan.N = M (N / 4 threads per CTA); a.tw: the N-point table.  d.seg: [cluster][K][N] when d.K > 1.
__global__ void __launch_bounds__(kMaxThreads) k_adjoint_pdc_spread(const PropArgs a, const AdjArgs d) {
  extern __shared__ double2 smem[];
  cg::cluster_group cl = cg::this_cluster();
  SpreadFFT f;
  const int rank = (int)cl.block_rank();
  const int M = a.plan.N;
  spread_init(f, smem, a.tw, M, rank);
  const int N = M * kSpreadC;
  const int tn = rank + kSpreadC * f.j, fk = f.j + M * rank;
  const int K = d.K;
  const long long clusterId = blockIdx.x / kSpreadC, nClusters = gridDim.x / kSpreadC;
  double2* seg = K > 1 ? d.seg + clusterId * (long long)K * N : nullptr;
  for (long long local = clusterId; local < a.nInst; local += nClusters) {
    const long long inst = a.instBase + local;
    const double2* ck = d.ckpt + inst * (long long)d.nCk * N;
    double2 g = cscale(d.gout[inst * (long long)N + fk], (double)N);
    int segEnd = a.nZ - 1;
    while (segEnd >= 1) {
      const int jseg = (segEnd - 1) / K, s0 = jseg * K;
      const double2* states = ck + (long long)s0 * N;   // K = 1: checkpoint i-1 is the state s_{i-1}
      if (K > 1) {
        // states s_{s0} .. s_{segEnd-1} into seg[0 ..]
        double2 x = ck[(long long)jseg * N + tn];
        seg[tn] = x;
        for (int i = s0 + 1; i < segEnd; i++) {
          x = pdc_step_point(a, N, i, tn, x);
          x = spread_inv(f, cmul(spread_fwd(f, x, cl), __ldg(a.dstep + fk)), cl);
          seg[(long long)(i - s0) * N + tn] = x;
        }
        states = seg;
      }
      for (int i = segEnd; i > s0; i--) {
        if (i < a.nZ - 1) g = spread_fwd(f, g, cl);
        const double2* tab = (i == a.nZ - 1) ? a.dlast : a.dstep;
        g = spread_inv(f, cmulc(g, __ldg(tab + fk)), cl);
        if (d.gp) {   // marching form: P^T per point, the stage-factor gradients afterwards in parallel
          g = pdc_march_point(a, d, N, i, tn, inst, g, true);
          continue;
        }
        const double2* c = a.coef + (long long)(i - 1) * 3 * a.nCoef;
        const double2* prev = states + (long long)(i - 1 - s0) * N;
        g = pdc_reverse_point(a, d, N, i, tn, c[0], c[1], c[2], prev[tn], g, true);
      }
      segEnd = s0;
    }
    // gradient of the input spectrum: s_0 = IFFT(half X_in)
    g = spread_fwd(f, g, cl);
    d.gin[inst * (long long)N + fk] = cmulc(g, __ldg(a.half + fk));
  }
}

// Pipelined form for checkpoint intervals K > 1 on clusters of eight CTAs (two groups of four, as in
// k_adjoint_pdc_cluster_pipe): ranks 4..7 recompute the states of segment j-1 from its checkpoint into
// one half of STG while ranks 0..3 reverse segment j from the other half.  Every spread transform ends
// with one barrier of the whole cluster, so per segment iteration both groups run exactly K step slots
// of 2 transforms (a recomputed step: the forward and inverse transform of the dispersion step; a
// reverse step: the same pair, with a bare barrier in place of the forward transform for the last step,
// whose gradient starts in the frequency domain) and then one barrier; a slot without a step passes 2
// bare barriers.  The final forward transform of the input gradient is matched by one bare barrier in
// the recomputing group.  d.seg: [cluster][2][K][N].
__global__ void __launch_bounds__(kMaxThreads) k_adjoint_pdc_spread_pipe(const PropArgs a, const AdjArgs d) {
  extern __shared__ double2 smem[];
  cg::cluster_group cl = cg::this_cluster();
  const int crank = (int)cl.block_rank();
  const int role = crank / kSpreadC;   // 0: reverse sweep, 1: recomputation
  SpreadFFT f;
  const int M = a.plan.N;
  spread_init(f, smem, a.tw, M, crank - role * kSpreadC);
  f.base = role * kSpreadC;
  const int N = M * kSpreadC;
  const int tn = f.rank + kSpreadC * f.j, fk = f.j + M * f.rank;
  const int K = d.K;
  const long long clusterId = blockIdx.x / (2 * kSpreadC), nClusters = gridDim.x / (2 * kSpreadC);
  const long long bufStride = (long long)K * N;
  double2* STG = d.seg + clusterId * 2 * bufStride;
  const int nSeg = (a.nZ - 2) / K + 1;
  for (long long local = clusterId; local < a.nInst; local += nClusters) {
    const long long inst = a.instBase + local;
    const double2* ck = d.ckpt + inst * (long long)d.nCk * N;
    double2 g = czero();
    if (role == 0) g = cscale(d.gout[inst * (long long)N + fk], (double)N);
    for (int it = 0; it <= nSeg; it++) {
      if (role == 1) {
        if (it < nSeg) {
          const int jseg = nSeg - 1 - it, s0 = jseg * K, segEnd = min(s0 + K, a.nZ - 1);
          double2* stg = STG + (long long)(it & 1) * bufStride;
          double2 x = ck[(long long)jseg * N + tn];
          stg[tn] = x;
          for (int q = 1; q <= K; q++) {
            const int i = s0 + q;
            if (i < segEnd) {
              x = pdc_step_point(a, N, i, tn, x);
              x = spread_inv(f, cmul(spread_fwd(f, x, cl), __ldg(a.dstep + fk)), cl);
              stg[(long long)q * N + tn] = x;
            } else {
              spread_idle(cl, 2);
            }
          }
        } else {
          spread_idle(cl, 2 * K);
        }
      } else {
        if (it >= 1) {
          const int jseg = nSeg - it, s0 = jseg * K, segEnd = min(s0 + K, a.nZ - 1);
          const double2* stg = STG + (long long)((it - 1) & 1) * bufStride;
          for (int q = 0; q < K; q++) {
            const int i = segEnd - q;
            if (i > s0) {
              const double2* prev = stg + (long long)(i - 1 - s0) * N;
              if (i < a.nZ - 1) g = spread_fwd(f, g, cl);
              else cl.sync();
              const double2* tab = (i == a.nZ - 1) ? a.dlast : a.dstep;
              g = spread_inv(f, cmulc(g, __ldg(tab + fk)), cl);
              const double2* c = a.coef + (long long)(i - 1) * 3 * a.nCoef;
              g = pdc_reverse_point(a, d, N, i, tn, c[0], c[1], c[2], prev[tn], g, true);
            } else {
              spread_idle(cl, 2);
            }
          }
        } else {
          spread_idle(cl, 2 * K);
        }
      }
      cl.sync();
    }
    if (role == 0) {
      g = spread_fwd(f, g, cl);
      d.gin[inst * (long long)N + fk] = cmulc(g, __ldg(a.half + fk));
    } else {
      cl.sync();
    }
  }
}

void add_kernels_adjoint_spread(std::vector<KernelEntry>& t) {
  // key + 300: one propagation per cluster of four CTAs; key + 200: pipelined on eight; R = 1 point
  // per thread
  t.push_back({kKindAdjoint, kChi2PDC + 300, 1, (const void*)k_adjoint_pdc_spread});
  t.push_back({kKindAdjoint, kChi2PDC + 200, 1, (const void*)k_adjoint_pdc_spread_pipe});
}

}  // namespace nlm
