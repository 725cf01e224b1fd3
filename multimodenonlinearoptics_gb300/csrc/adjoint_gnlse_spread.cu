// adjoint_gnlse_spread.cu -- the Chi3GNLSE reverse sweep over stored stage values (k_adjoint_gnlse_stored
// in adjoint_gnlse_cluster.cu, solvers/Chi3GNLSE.cpp:39-92 run backwards) with one point per thread on
// clusters of C CTAs (the transforms of nlm_spread.cuh), for the forwards that ran on the same form
// (prop_gnlse_spread.cu).  The stage values are time-domain rows: Yi[s][N] = y_s, Yi[4 + s][N] = u2_s.
// The gradient stays in the frequency domain between steps (the reverse step of adjoint_gnlse.cu).
#include <vector>

#include "nlm_spread.cuh"

namespace nlm {

// a.plan.N = M (N / C threads per CTA); a.tw: the N-point table.  Sixteen CTAs: grids up to 4096 points.
template <int C>
__global__ void __launch_bounds__(C == 16 ? 256 : kMaxThreads) k_adjoint_gnlse_stored_spread(const PropArgs a,
                                                                                             const AdjArgs d) {
  extern __shared__ double2 smem[];
  cg::cluster_group cl = cg::this_cluster();
  SpreadFFT f;
  const int rank = (int)cl.block_rank();
  const int M = a.plan.N;
  spread_init<C>(f, smem, a.tw, M, rank);
  const int N = M * C;
  const int tn = rank + C * f.t, fk = f.j + M * rank;
  const double2 ram = __ldg(a.raman + fk), stp = __ldg(a.steep + fk);
  const double2 dst = __ldg(a.dstep + fk), dla = __ldg(a.dlast + fk);
  const long long clusterId = blockIdx.x / C, nClusters = gridDim.x / C;
  for (long long local = clusterId; local < a.nInst; local += nClusters) {
    const long long inst = a.instBase + local;
    const double2* stg = a.stages + inst * (long long)(a.nZ - 1) * 8 * N;
    // g: the gradient with respect to the spectrum after step i (this thread's bin), the transpose of
    // the forward's frequency-domain RK4 sum.  With h = N conj(D) g (D the dispersion factors, which
    // carry the 1/N of a transform pair), stage s's spectrum gets w_s h plus the transform of the
    // gradient its time-domain value takes through the next stage's input, and the spectrum before
    // the step h plus the transform of the stage inputs' gradient gx: 16 transforms per step.
    double2 g = cscale(d.gout[inst * (long long)N + fk], (double)N);
    for (int i = a.nZ - 1; i >= 1; i--) {
      const double2* Yi = stg + (long long)(i - 1) * 8 * N;
      const double2 h = cscale(cmulc(g, i == a.nZ - 1 ? dla : dst), (double)N);
      const double* rel = a.relInt + (long long)(i - 1) * 3;
      double2 gx = czero(), gke = czero();
      for (int s = 3; s >= 0; s--) {
        const double w = (s == 1 || s == 2) ? 2.0 / 6.0 : 1.0 / 6.0;
        const double fac = s == 0 ? 0.0 : (s == 3 ? 1.0 : 0.5);
        const double ri = __ldg(rel + (s == 0 ? 0 : (s == 3 ? 2 : 1)));
        const double2 y = Yi[(long long)s * N + tn], u2 = Yi[(long long)(4 + s) * N + tn];
        // g_k_s (spectrum); the fourth stage's has no later stage's part
        double2 u = s < 3 ? caxpy(spread_fwd<C>(f, gke, cl), w, h) : cscale(h, w);
        u = spread_inv<C>(f, cmulc(u, stp), cl);                        // g_u3
        double2 gy = cmulc(u, u2);                                    // conj(u2) g_u3
        u = cmulc(u, y);                                              // g_u2 = conj(y) g_u3
        u = spread_inv<C>(f, cmulc(spread_fwd<C>(f, u, cl), ram), cl);   // g_u1 (real part)
        gy = caxpy(gy, 2.0 * ri * u.x, y);
        gx = cadd(gx, gy);
        gke = cscale(gy, fac);
      }
      g = cadd(spread_fwd<C>(f, gx, cl), h);
    }
    // g: the gradient of the input spectrum, times half a dispersion step
    d.gin[inst * (long long)N + fk] = cmulc(g, __ldg(a.half + fk));
  }
}

void add_kernels_adjoint_gnlse_spread(std::vector<KernelEntry>& t) {
  // key + 500 (R = 1, one point per thread): four, eight and sixteen CTAs by the registered C
  t.push_back({kKindAdjoint, kChi3GNLSE + 500, 4, (const void*)k_adjoint_gnlse_stored_spread<4>});
  t.push_back({kKindAdjoint, kChi3GNLSE + 500, 8, (const void*)k_adjoint_gnlse_stored_spread<8>});
  t.push_back({kKindAdjoint, kChi3GNLSE + 500, 16, (const void*)k_adjoint_gnlse_stored_spread<16>});
}

}  // namespace nlm
