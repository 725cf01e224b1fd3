// prop_cluster_gnlse.cu -- one Chi3GNLSE propagation spread over a cluster of C CTAs
// (solvers/Chi3GNLSE.cpp:39-92, transforms as in nlm_cluster.cuh).
//
// A z step of the generalised NLSE is 16 transforms inside the four RK4 stages,
//     k = IFFT[(g0 + g1 w) FFT[ y * IFFT[R~ FFT[rel |y|^2]] ]],
// plus the dispersion pair; on one SM a single propagation at N=4096 runs about 0.9 ms per step.  The
// stages' spectra are summed in the frequency domain, which drops the fourth stage's inverse transform
// and the forward transform of the dispersion step: 16 transforms per step.  Here
// every transform is the cluster's four-step FFT, and the state, the stage input and the RK4 sum stay
// in registers (C points per thread), in the time-domain ownership of the cluster kernels.
#include <vector>

#include "nlm_cluster.cuh"

namespace nlm {

template <int C>
__global__ void __launch_bounds__(kMaxThreads) k_propagate_gnlse_cluster(const PropArgs a) {
  constexpr int R = C;
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
  auto tn = [&](int v) { return rank + C * (j + v * T); };
  auto fk = [&](int v) { return j + rank * T + M * v; };
  for (long long local = clusterId; local < a.nInst; local += nClusters) {
    const long long inst = a.instBase + local;
    const double2* row = a.in + inst * a.inStride;
    const bool has = a.inputMode == 0 || (a.inputMode < 1 && a.inChannels > 0);
    double2 x[R];
#pragma unroll
    for (int v = 0; v < R; v++) x[v] = has ? row[a.inTime ? tn(v) : fk(v)] : czero();
    if (a.inTime) cluster_fft_fwd<C>(f, x, cl);
#pragma unroll
    for (int v = 0; v < R; v++) x[v] = cmul(x[v], __ldg(a.half + fk(v)));
    if (a.gridF) {
#pragma unroll
      for (int v = 0; v < R; v++) a.gridF[fk(v)] = cscale(x[v], (double)N);
    }
    double2 xf[R];   // the state's spectrum (whose unscaled inverse transform is x)
#pragma unroll
    for (int v = 0; v < R; v++) xf[v] = x[v];
    cluster_fft_inv<C>(f, x, cl);
    if (a.gridT) {
#pragma unroll
      for (int v = 0; v < R; v++) a.gridT[tn(v)] = x[v];
    }
    // checkpoints for the reverse sweep: the time-domain state before steps 1, K + 1, 2 K + 1, ...
    double2* ckRow = a.ckpt ? a.ckpt + inst * a.ckN * (long long)N : nullptr;
    if (ckRow && a.nZ > 1) {
#pragma unroll
      for (int v = 0; v < R; v++) ckRow[tn(v)] = x[v];
    }
    for (int i = 1; i < a.nZ; i++) {
      const double* rel = a.relInt + (long long)(i - 1) * 3;
      double2* stg = a.stages ? a.stages + ((inst * (a.nZ - 1) + i - 1) * 8LL) * N : nullptr;
      // the RK4 sum in the frequency domain (k_propagate_gnlse_pair): each stage's k is formed as a
      // spectrum and transformed back only as the next stage's input; the step's end is
      // FFT[x + sum / 6] = N (xf + sum / 6), with no transform.  16 transforms per step.
      double2 k[R], acc[R];
#pragma unroll
      for (int v = 0; v < R; v++) k[v] = czero();
      for (int s = 0; s < 4; s++) {
        const double fac = s == 0 ? 0.0 : (s == 3 ? 1.0 : 0.5);
        const double wgt = (s == 1 || s == 2) ? 2.0 : 1.0;
        const double ri = __ldg(rel + (s == 0 ? 0 : (s == 3 ? 2 : 1)));
        double2 y[R], u[R];
#pragma unroll
        for (int v = 0; v < R; v++) {
          y[v] = caxpy(x[v], fac, k[v]);
          u[v] = make_double2(ri * cabs2(y[v]), 0.0);
          if (stg) stg[(long long)s * N + tn(v)] = y[v];
        }
        // Raman convolution R~ * (rel |y|^2)
        cluster_fft_fwd<C>(f, u, cl);
#pragma unroll
        for (int v = 0; v < R; v++) u[v] = cmul(u[v], __ldg(a.raman + fk(v)));
        cluster_fft_inv<C>(f, u, cl);
        if (stg) {
#pragma unroll
          for (int v = 0; v < R; v++) stg[(long long)(4 + s) * N + tn(v)] = u[v];
        }
        // times the field, then the self-steepening operator (g0 + g1 w)
#pragma unroll
        for (int v = 0; v < R; v++) u[v] = cmul(u[v], y[v]);
        cluster_fft_fwd<C>(f, u, cl);
#pragma unroll
        for (int v = 0; v < R; v++) {
          u[v] = cmul(u[v], __ldg(a.steep + fk(v)));
          acc[v] = s == 0 ? u[v] : caxpy(acc[v], wgt, u[v]);
        }
        if (s < 3) {
          cluster_fft_inv<C>(f, u, cl);
#pragma unroll
          for (int v = 0; v < R; v++) k[v] = u[v];
        }
      }
      const bool last = i == a.nZ - 1;
      const double2* table = last ? a.dlast : a.dstep;
#pragma unroll
      for (int v = 0; v < R; v++) {
        x[v] = cmul(cscale(caxpy(xf[v], 1.0 / 6.0, acc[v]), (double)N), __ldg(table + fk(v)));
        if (!last) xf[v] = x[v];
      }
      if (a.gridF) {
#pragma unroll
        for (int v = 0; v < R; v++) a.gridF[(long long)i * N + fk(v)] = cscale(x[v], (double)N);
      }
      if (!last || a.inTime || a.gridT) {
        cluster_fft_inv<C>(f, x, cl);
        if (a.gridT) {
#pragma unroll
          for (int v = 0; v < R; v++) a.gridT[(long long)i * N + tn(v)] = x[v];
        }
        if (ckRow && !last && i % a.ckK == 0) {
#pragma unroll
          for (int v = 0; v < R; v++) ckRow[(long long)(i / a.ckK) * N + tn(v)] = x[v];
        }
      }
    }
    if (a.nZ == 1) {
      cluster_fft_fwd<C>(f, x, cl);
#pragma unroll
      for (int v = 0; v < R; v++) x[v] = cmul(x[v], __ldg(a.back + fk(v)));
      if (a.gridF) {
#pragma unroll
        for (int v = 0; v < R; v++) a.gridF[fk(v)] = cscale(x[v], (double)N);
      }
      if (a.inTime || a.gridT) {
        cluster_fft_inv<C>(f, x, cl);
        if (a.gridT) {
#pragma unroll
          for (int v = 0; v < R; v++) a.gridT[tn(v)] = x[v];
        }
      }
    }
    // the last row is in the time domain when the input was, else in the frequency domain
    if (a.out && a.nOut > 0 && a.outModes[0] == 0) {
      double2* o = a.out + inst * a.outStride;
      const double sc = a.inTime ? 1.0 : (double)N;
#pragma unroll
      for (int v = 0; v < R; v++) o[a.inTime ? tn(v) : fk(v)] = cscale(x[v], sc);
    }
  }
}

void add_kernels_cluster_gnlse(std::vector<KernelEntry>& t) {
  t.push_back({kKindCluster, kChi3GNLSE, 4, (const void*)k_propagate_gnlse_cluster<4>});
}

}  // namespace nlm
