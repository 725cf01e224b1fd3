// prop_gnlse_spread.cu -- one Chi3GNLSE propagation on a cluster of C CTAs with one point per thread
// (the transforms of nlm_spread.cuh; the step of prop_cluster_gnlse.cu, solvers/Chi3GNLSE.cpp:39-92).
//
// A z step is 16 transforms inside the four RK4 stages,
//     k = IFFT[(g0 + g1 w) FFT[ y * IFFT[R~ FFT[rel |y|^2]] ]],
// plus the dispersion pair; with the RK4 sum in the frequency domain, 16 in all.  With four points per thread on four CTAs (prop_cluster_gnlse.cu) a
// single 4096-point propagation takes about 260 us per step; here it holds N / C points per CTA, one
// per thread: sixteen CTAs of 256 threads at 4096 points (the full-grid form), eight of 256 at 2048.
// The per-point tables (Raman response, self-steepening factors, dispersion) stay in registers.
#include <vector>

#include "nlm_spread.cuh"

namespace nlm {

// a.plan.N = M (N / C threads per CTA); a.tw: the N-point table.  Sixteen CTAs take grids up to 4096
// points (at most 256 threads per CTA, a bound that leaves the 16-point combine its registers).
template <int C>
__global__ void __launch_bounds__(C == 16 ? 256 : kMaxThreads) k_propagate_gnlse_spread(const PropArgs a) {
  extern __shared__ double2 smem[];
  cg::cluster_group cl = cg::this_cluster();
  SpreadFFT f;
  const int rank = (int)cl.block_rank();
  const int M = a.plan.N;
  spread_init<C>(f, smem, a.tw, M, rank);
  const int N = M * C;
  const int tn = rank + C * f.t;   // time-domain point of this thread
  const int fk = f.j + M * rank;   // frequency bin of this thread
  const double2 ram = __ldg(a.raman + fk), stp = __ldg(a.steep + fk);
  const double2 dst = __ldg(a.dstep + fk), dla = __ldg(a.dlast + fk);
  const long long clusterId = blockIdx.x / C, nClusters = gridDim.x / C;
  for (long long local = clusterId; local < a.nInst; local += nClusters) {
    const long long inst = a.instBase + local;
    const double2* row = a.in + inst * a.inStride;
    const bool has = a.inputMode == 0 || (a.inputMode < 1 && a.inChannels > 0);
    double2 x = has ? row[a.inTime ? tn : fk] : czero();
    if (a.inTime) x = spread_fwd<C>(f, x, cl);
    x = cmul(x, __ldg(a.half + fk));
    double2 xf = x;   // the state's spectrum (whose unscaled inverse transform is x)
    x = spread_inv_store<C>(f, x, cl, [&](double2 v) {
      if (a.gridF) a.gridF[fk] = cscale(v, (double)N);
    });
    if (a.gridT) a.gridT[tn] = x;
    // checkpoints for the reverse sweep: the time-domain state before steps 1, K + 1, 2 K + 1, ...
    double2* ckRow = a.ckpt ? a.ckpt + inst * a.ckN * (long long)N : nullptr;
    if (ckRow && a.nZ > 1) ckRow[tn] = x;
    for (int i = 1; i < a.nZ; i++) {
      const double* rel = a.relInt + (long long)(i - 1) * 3;
      double2* stg = a.stages ? a.stages + ((inst * (a.nZ - 1) + i - 1) * 8LL) * N : nullptr;
      // the RK4 sum in the frequency domain (k_propagate_gnlse_pair): each stage's k is formed as a
      // spectrum and transformed back only as the next stage's input; the step's end is
      // FFT[x + sum / 6] = N (xf + sum / 6), with no transform.  16 transforms per step.
      double2 k = czero(), acc = czero();
      for (int s = 0; s < 4; s++) {
        const double fac = s == 0 ? 0.0 : (s == 3 ? 1.0 : 0.5);
        const double wgt = (s == 1 || s == 2) ? 2.0 : 1.0;
        const double ri = __ldg(rel + (s == 0 ? 0 : (s == 3 ? 2 : 1)));
        const double2 y = caxpy(x, fac, k);
        double2 u = make_double2(ri * cabs2(y), 0.0);
        if (stg) stg[(long long)s * N + tn] = y;
        // Raman convolution R~ * (rel |y|^2)
        u = spread_fwd<C>(f, u, cl);
        u = spread_inv<C>(f, cmul(u, ram), cl);
        if (stg) stg[(long long)(4 + s) * N + tn] = u;
        // times the field, then the self-steepening operator (g0 + g1 w)
        u = cmul(spread_fwd<C>(f, cmul(u, y), cl), stp);
        acc = s == 0 ? u : caxpy(acc, wgt, u);
        if (s < 3) k = spread_inv<C>(f, u, cl);
      }
      const bool last = i == a.nZ - 1;
      x = cmul(cscale(caxpy(xf, 1.0 / 6.0, acc), (double)N), last ? dla : dst);
      if (!last) xf = x;
      auto storeF = [&](double2 v) {
        if (a.gridF) a.gridF[(long long)i * N + fk] = cscale(v, (double)N);
      };
      if (!last || a.inTime || a.gridT) {
        x = spread_inv_store<C>(f, x, cl, storeF);
        if (a.gridT) a.gridT[(long long)i * N + tn] = x;
        if (ckRow && !last && i % a.ckK == 0) ckRow[(long long)(i / a.ckK) * N + tn] = x;
      } else {
        storeF(x);
      }
    }
    if (a.nZ == 1) {
      x = cmul(spread_fwd<C>(f, x, cl), __ldg(a.back + fk));
      if (a.gridF) a.gridF[fk] = cscale(x, (double)N);
      if (a.inTime || a.gridT) {
        x = spread_inv<C>(f, x, cl);
        if (a.gridT) a.gridT[tn] = x;
      }
    }
    // the last row is in the time domain when the input was, else in the frequency domain
    if (a.out && a.nOut > 0 && a.outModes[0] == 0) {
      double2* o = a.out + inst * a.outStride;
      o[a.inTime ? tn : fk] = cscale(x, a.inTime ? 1.0 : (double)N);
    }
  }
}

// kind kKindCluster, R = 1 (one point per thread): key Chi3GNLSE (four CTAs), + kSpreadWideKey (eight),
// + kSpreadW16Key (sixteen)
void add_kernels_gnlse_spread(std::vector<KernelEntry>& t) {
  t.push_back({kKindCluster, kChi3GNLSE, 1, (const void*)k_propagate_gnlse_spread<4>});
  t.push_back({kKindCluster, kChi3GNLSE + kSpreadWideKey, 1, (const void*)k_propagate_gnlse_spread<8>});
  t.push_back({kKindCluster, kChi3GNLSE + kSpreadW16Key, 1, (const void*)k_propagate_gnlse_spread<16>});
}

}  // namespace nlm
