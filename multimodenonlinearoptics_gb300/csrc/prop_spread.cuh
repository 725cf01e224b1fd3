// prop_spread.cuh -- the one-point-per-thread cluster kernels (nlm_spread.cuh), templated on the
// cluster size C (4 or 8): single propagations and small batches, and the Chi3 pump march.
//
// k_pump_chi3_spread has the arithmetic of k_pump_chi3 / k_pump_chi3_cluster (solvers/Chi3.cpp:41-70);
// k_propagate_spread<S, C> that of k_propagate_cluster<S> (src/_NonlinearMedium.hpp:160-239): the same
// tables, the same order of operations per point, only the ownership of the points differs.
#pragma once
#include "nlm_spread.cuh"

namespace nlm {

// tw: the N-point table; M = N / C threads per CTA.
template <int C>
__global__ void __launch_bounds__(kMaxThreads) k_pump_chi3_spread(double2* __restrict__ pf, double2* __restrict__ pt,
                                                                  const double2* __restrict__ env,
                                                                  const double2* __restrict__ halfP,
                                                                  const double2* __restrict__ dstepP,
                                                                  const double2* __restrict__ backP,
                                                                  const double2* __restrict__ rel, int nRows, int M,
                                                                  const double2* __restrict__ tw) {
  extern __shared__ double2 smem[];
  cg::cluster_group cl = cg::this_cluster();
  SpreadFFT f;
  const int rank = (int)cl.block_rank();
  spread_init<C>(f, smem, tw, M, rank);
  const int N = M * C;
  const int tn = rank + C * f.t;          // time-domain point of this thread
  const int fk = f.j + M * rank;          // frequency bin of this thread
  const double invN = 1.0 / N;
  const double2 hp = halfP[fk], dp = dstepP[fk];
  double2 x = spread_fwd<C>(f, env[tn], cl);
  x = cmul(x, hp);
  x = cscale(spread_inv_store<C>(f, x, cl, [&](double2 v) { pf[fk] = v; }), invN);
  pt[tn] = x;
  for (int i = 1; i < nRows; i++) {
    const double2 r = rel[i - 1];
    const double a2 = cabs2(x);
    x = cmul(x, spm_factor(r.x * a2, r.y * a2));
    x = cmul(spread_fwd<C>(f, x, cl), dp);
    x = cscale(spread_inv_store<C>(f, x, cl, [&](double2 v) { pf[(long long)i * N + fk] = v; }), invN);
    pt[(long long)i * N + tn] = x;
  }
  // last row: undo half of the last pump dispersion step (each thread rereads its own bin)
  const long long last = (long long)(nRows - 1) * N;
  x = cmul(pf[last + fk], backP[fk]);
  pt[last + tn] = cscale(spread_inv_store<C>(f, x, cl, [&](double2 v) { pf[last + fk] = v; }), invN);
}

// All MD modes: time -> frequency domain; K = MD together, K = 1 one after another.
template <int C, int K, int MD>
__device__ __forceinline__ void spread_fwd_all(SpreadFFT& f, double2 (&x)[MD], cg::cluster_group& cl) {
  if constexpr (K > 1) {
    spread_fwd_k<C, MD>(f, x, cl);
  } else {
#pragma unroll
    for (int m = 0; m < MD; m++) x[m] = spread_fwd<C>(f, x[m], cl);
  }
}

// All MD modes: frequency -> time domain, store(m, v) given each mode's spectrum after its exchange.
template <int C, int K, int MD, class Store>
__device__ __forceinline__ void spread_inv_all(SpreadFFT& f, double2 (&x)[MD], cg::cluster_group& cl, Store store) {
  if constexpr (K > 1) {
    spread_inv_store_k<C, MD>(f, x, cl, store);
  } else {
#pragma unroll
    for (int m = 0; m < MD; m++) {
      const int mm = m;
      x[m] = spread_inv_store<C>(f, x[m], cl, [&](double2 v) { store(mm, v); });
    }
  }
}

// One propagation per cluster (clusters take instances in turn); a.plan.N = M, a.tw the N-point table.
// Point-wise work: the pump-driven solvers' RK4 matrices (a.prop) or the solver's DiffEq.  K = 1: the
// modes' transforms one after another; K = the solver's mode count: all modes in each transform
// together (spread_fwd_k, spread_inv_store_k: one barrier per stage and one cluster barrier per
// exchange for all of them), with K times the exchange and receive buffers.  Either way every mode
// goes through the same operations, so the results are identical.
template <class S, int C, int K = 1>
__global__ void __launch_bounds__(kMaxThreads) k_propagate_spread(const PropArgs a) {
  constexpr int MD = S::kM, P = S::kP > 0 ? S::kP : 1;
  static_assert(K == 1 || K == MD, "modes one at a time or all together");
  extern __shared__ double2 smem[];
  cg::cluster_group cl = cg::this_cluster();
  SpreadFFT f;
  const int rank = (int)cl.block_rank();
  const int M = a.plan.N;
  spread_init<C, K>(f, smem, a.tw, M, rank);
  const int N = M * C;
  const int tn = rank + C * f.t;
  const int fk = f.j + M * rank;
  const long long clusterId = blockIdx.x / C, nClusters = gridDim.x / C;
  const long long ms = (long long)a.nZ * N;
  for (long long local = clusterId; local < a.nInst; local += nClusters) {
    const long long inst = a.instBase + local;
    double2 x[MD];
    const double2* row = a.in + inst * a.inStride;
#pragma unroll
    for (int m = 0; m < MD; m++) {
      int seg = -1;
      if (m == a.inputMode) seg = 0;
      else if (a.inputMode < 1 && m < a.inChannels) seg = m;
      x[m] = seg >= 0 ? row[(long long)seg * N + (a.inTime ? tn : fk)] : czero();
    }
    if (a.inTime) spread_fwd_all<C, K, MD>(f, x, cl);
#pragma unroll
    for (int m = 0; m < MD; m++) x[m] = cmul(x[m], __ldg(a.half + (long long)m * N + fk));
    spread_inv_all<C, K, MD>(f, x, cl, [&](int m, double2 v) {
      if (a.gridF) a.gridF[m * ms + fk] = cscale(v, (double)N);
    });
    if (a.gridT) {
#pragma unroll
      for (int m = 0; m < MD; m++) a.gridT[m * ms + tn] = x[m];
    }
    // checkpoints for a reverse sweep: the time-domain state before steps 1, K + 1, 2 K + 1, ...
    double2* ckRow = a.ckpt ? a.ckpt + inst * a.ckN * MD * (long long)N : nullptr;
    if (ckRow && a.nZ > 1) {
#pragma unroll
      for (int m = 0; m < MD; m++) ckRow[(long long)m * N + tn] = x[m];
    }
    for (int i = 1; i < a.nZ; i++) {
      if (a.prop) {
        // the RK4 step as its per-point real (2M)x(2M) matrix, stored as pairs (row r, columns 2c and
        // 2c+1) at [step][r * M + c][N]
        constexpr int D = 2 * MD;
        const double2* mat = reinterpret_cast<const double2*>(a.prop) + (long long)(i - 1) * (D * D / 2) * N;
        double in[D], outv[D];
#pragma unroll
        for (int m = 0; m < MD; m++) {
          in[2 * m] = x[m].x;
          in[2 * m + 1] = x[m].y;
        }
#pragma unroll
        for (int r = 0; r < D; r++) {
          double acc = 0.0;
#pragma unroll
          for (int cc = 0; cc < D / 2; cc++) {
            const double2 e = __ldg(mat + (long long)(r * (D / 2) + cc) * N + tn);
            acc = fma(e.x, in[2 * cc], acc);
            acc = fma(e.y, in[2 * cc + 1], acc);
          }
          outv[r] = acc;
        }
#pragma unroll
        for (int m = 0; m < MD; m++) x[m] = make_double2(outv[2 * m], outv[2 * m + 1]);
      } else {
        const double2* c = a.coef + (long long)(i - 1) * 3 * a.nCoef;
        double2 p[3][P];
#pragma unroll
        for (int q = 0; q < P; q++) {
          if (S::kP > 0) {
            const double2* pr = a.pump + q * a.pumpStride + (long long)(2 * i - 2) * N + tn;
            p[0][q] = __ldg(pr);
            p[1][q] = __ldg(pr + N);
            p[2][q] = __ldg(pr + 2 * N);
          } else {
            p[0][q] = p[1][q] = p[2][q] = czero();
          }
        }
        rk4_point<S>(x, p, c);
      }
      const bool last = i == a.nZ - 1;
      const double2* table = last ? a.dlast : a.dstep;
      const bool wantTime = !last || a.inTime || a.gridT != nullptr;
      spread_fwd_all<C, K, MD>(f, x, cl);
#pragma unroll
      for (int m = 0; m < MD; m++) x[m] = cmul(x[m], __ldg(table + (long long)m * N + fk));
      auto storeF = [&](int m, double2 v) {
        if (a.gridF) a.gridF[m * ms + (long long)i * N + fk] = cscale(v, (double)N);
      };
      if (wantTime) {
        spread_inv_all<C, K, MD>(f, x, cl, storeF);
        if (a.gridT) {
#pragma unroll
          for (int m = 0; m < MD; m++) a.gridT[m * ms + (long long)i * N + tn] = x[m];
        }
      } else {
#pragma unroll
        for (int m = 0; m < MD; m++) storeF(m, x[m]);
      }
      if (ckRow && !last && i % a.ckK == 0) {
#pragma unroll
        for (int m = 0; m < MD; m++) ckRow[((long long)(i / a.ckK) * MD + m) * N + tn] = x[m];
      }
    }
    if (a.nZ == 1) {
      spread_fwd_all<C, K, MD>(f, x, cl);
#pragma unroll
      for (int m = 0; m < MD; m++) {
        x[m] = cmul(x[m], __ldg(a.back + (long long)m * N + fk));
        if (a.gridF) a.gridF[m * ms + fk] = cscale(x[m], (double)N);
      }
      if (a.inTime || a.gridT) {
        spread_inv_all<C, K, MD>(f, x, cl, [&](int, double2) {});
        if (a.gridT) {
#pragma unroll
          for (int m = 0; m < MD; m++) a.gridT[m * ms + tn] = x[m];
        }
      }
    }
    // the last row is in the time domain when the input was, else in the frequency domain
    if (a.out) {
      double2* o = a.out + inst * a.outStride;
      const double sc = a.inTime ? 1.0 : (double)N;
      for (int om = 0; om < a.nOut; om++) {
#pragma unroll
        for (int m = 0; m < MD; m++)
          if (m == a.outModes[om]) o[(long long)om * N + (a.inTime ? tn : fk)] = cscale(x[m], sc);
      }
    }
  }
}

}  // namespace nlm
