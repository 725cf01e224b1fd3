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
  const int tn = rank + kSpreadC * f.t, fk = f.j + M * rank;
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
  const int tn = f.rank + kSpreadC * f.t, fk = f.j + M * f.rank;
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

// Stage-factor gradient groups beside the pipelined sweep, on clusters of 4 (2 + G) CTAs, for
// checkpoint intervals K > 1 with the RK4 propagator matrices built.  In k_adjoint_pdc_spread_pipe the
// reverse group also runs the transposed stages of every step (about 90 FP64 operations per point),
// so the recomputing group, whose step is 4 FMAs, waits at every shared barrier.  Here:
//   ranks 4..7 (group 1) recompute the states of segment j-1 into STG, as there;
//   ranks 0..3 (group 0) reverse segment j: the dispersion pair, then P^T per point (4 FMAs), storing
//     the gradient after each step's RK4 in GP;
//   ranks 8.. (groups 2 .. 1 + G) compute the stage-factor gradients of segment j+1, reversed in the
//     previous iteration, from its states (STG) and stored gradients (GP).  Group 2 + s takes the steps
//     q = s mod G of the segment (q = 0 .. K-1): the loads and forward stages of step q in slot q, its
//     transposed stages and stores in slot q + 1 (or after the last slot), both before the slot's
//     first barrier.  That interval holds two local transforms in groups 0 and 1 (the inverse of the
//     previous slot, the forward of this one); the one between the slot's two barriers holds only the
//     cluster exchange.
// Per slot a point costs about 76 FP64 instructions in groups 0 and 1 and 90 / G in each stage group;
// the FP64 issue rate of an SM is fixed per scheduler, so G = 2 (sixteen CTAs) keeps the stage groups
// off the critical path and G = 1 (twelve) is the form for GPUs without 16-CTA clusters.  STG holds
// three segments (written by group 1 at iteration it, read by group 0 at it+1 and by the stage groups
// at it+2) and GP two.  After the last iteration all groups share the stage-factor gradients of
// segment 0, by steps.  Barriers per row: (nSeg + 1) (2K + 1) in the iterations, then one (the input
// gradient's transform in group 0) and one after the shared work, in every group.
// d.seg: [cluster][3 + 2][K][N].
template <int G>
__global__ void __launch_bounds__(kMaxThreads) k_adjoint_pdc_spread_stage(const PropArgs a, const AdjArgs d) {
  constexpr int kGroups = 2 + G;
  extern __shared__ double2 smem[];
  cg::cluster_group cl = cg::this_cluster();
  const int crank = (int)cl.block_rank();
  const int role = crank / kSpreadC;   // 0: reverse sweep, 1: recomputation, 2..: stage-factor gradients
  const int lr = crank - role * kSpreadC;
  const int M = a.plan.N;
  const int N = M * kSpreadC;
  SpreadFFT f;
  if (role < 2) {
    spread_init(f, smem, a.tw, M, lr);
    f.base = role * kSpreadC;
  }
  const int tn = lr + kSpreadC * spread_time_index((int)threadIdx.x, M), fk = (int)threadIdx.x + M * lr;
  const int pc = lr * M + (int)threadIdx.x;   // the point of this thread's stage-factor gradients
  const int K = d.K;
  const long long clusterId = blockIdx.x / (kGroups * kSpreadC), nClusters = gridDim.x / (kGroups * kSpreadC);
  const long long bufStride = (long long)K * N;
  double2* STG = d.seg + clusterId * 5 * bufStride;
  double2* GP = STG + 3 * bufStride;
  const int nSeg = (a.nZ - 2) / K + 1;
  // a stage group's step in flight: its forward stages, state and gradient (step 0: none)
  PdcStages st{};
  double2 sx = czero(), sg = czero();
  int si = 0;
  auto stageLoad = [&](const double2* stg, const double2* gps, int i, int s0) {
    sx = stg[(long long)(i - 1 - s0) * N + pc];
    sg = gps[(long long)(i - 1 - s0) * N + pc];
    const double2* c = a.coef + (long long)(i - 1) * 3 * a.nCoef;
    st = pdc_stages(a, N, i, pc, c[0], c[1], c[2], sx);
    si = i;
  };
  auto stageFinish = [&]() {
    if (si == 0) return;
    double2 ga0, ga1, ga2;
    pdc_stages_reverse(st, sx, sg, ga0, ga1, ga2);
    pdc_store_ga(d, N, si, pc, ga0, ga1, ga2);
    si = 0;
  };
  for (long long local = clusterId; local < a.nInst; local += nClusters) {
    const long long inst = a.instBase + local;
    const double2* ck = d.ckpt + inst * (long long)d.nCk * N;
    double2 g = czero();
    if (role == 0) g = cscale(d.gout[inst * (long long)N + fk], (double)N);
    for (int it = 0; it <= nSeg; it++) {
      if (role == 1) {
        if (it < nSeg) {
          const int jseg = nSeg - 1 - it, s0 = jseg * K, segEnd = min(s0 + K, a.nZ - 1);
          double2* stg = STG + (long long)(it % 3) * bufStride;
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
      } else if (role == 0) {
        if (it >= 1) {
          const int jseg = nSeg - it, s0 = jseg * K, segEnd = min(s0 + K, a.nZ - 1);
          double2* gps = GP + (long long)(it & 1) * bufStride;
          for (int q = 0; q < K; q++) {
            const int i = segEnd - q;
            if (i > s0) {
              if (i < a.nZ - 1) g = spread_fwd(f, g, cl);
              else cl.sync();
              const double2* tab = (i == a.nZ - 1) ? a.dlast : a.dstep;
              g = spread_inv(f, cmulc(g, __ldg(tab + fk)), cl);
              gps[(long long)(i - 1 - s0) * N + tn] = g;
              g = pdc_transpose_point(a, N, i, tn, g);
            } else {
              spread_idle(cl, 2);
            }
          }
        } else {
          spread_idle(cl, 2 * K);
        }
      } else {
        if (it >= 2) {
          const int sub = role - 2;
          const int jseg = nSeg - it + 1, s0 = jseg * K, segEnd = min(s0 + K, a.nZ - 1);
          const double2* stg = STG + (long long)((it - 2) % 3) * bufStride;
          const double2* gps = GP + (long long)((it - 1) & 1) * bufStride;
          for (int q = 0; q < K; q++) {
            stageFinish();   // the step loaded in an earlier slot
            const int i = s0 + 1 + q;
            if (q % G == sub && i <= segEnd) stageLoad(stg, gps, i, s0);
            spread_idle(cl, 2);
          }
          stageFinish();
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
    // segment 0 (reversed in the last iteration): its steps shared by all groups
    {
      const int segEnd = min(K, a.nZ - 1);
      const double2* stg = STG + (long long)((nSeg - 1) % 3) * bufStride;
      const double2* gps = GP + (long long)(nSeg & 1) * bufStride;
      for (int i = 1 + role; i <= segEnd; i += kGroups) {
        stageLoad(stg, gps, i, 0);
        stageFinish();
      }
    }
    cl.sync();
  }
}

void add_kernels_adjoint_spread(std::vector<KernelEntry>& t) {
  // key + 300: one propagation per cluster of four CTAs; key + 200: pipelined on eight; R = 1 point
  // per thread
  t.push_back({kKindAdjoint, kChi2PDC + 300, 1, (const void*)k_adjoint_pdc_spread});
  t.push_back({kKindAdjoint, kChi2PDC + 200, 1, (const void*)k_adjoint_pdc_spread_pipe});
  // key + 500 / + 600: stage-factor gradients in one / two groups of their own, on twelve / sixteen
  // CTAs (checkpoints with the propagator matrices)
  t.push_back({kKindAdjoint, kChi2PDC + 500, 1, (const void*)k_adjoint_pdc_spread_stage<1>});
  t.push_back({kKindAdjoint, kChi2PDC + 600, 1, (const void*)k_adjoint_pdc_spread_stage<2>});
}

}  // namespace nlm
