// prop_cluster_pump.cu -- the Chi3 pump march (solvers/Chi3.cpp:41-70) spread over a cluster of
// four CTAs (four SMs), with the four-step transforms of nlm_cluster.cuh.
//
// Same arithmetic as k_pump_chi3: row 0 = IFFT(half * FFT(envelope)) / N; every further row applies
// the self-phase factor exp(rel |A|^2) in the time domain, the dispersion step in the frequency
// domain (stored as the frequency row), and the inverse transform / N (the time row); the last
// frequency row then undoes half of the last dispersion step.  The tables are not divided by N here.
#include "nlm_cluster.cuh"
#include "nlm_launch.h"

namespace nlm {

// plan: the local M-point plan (M = N / 4, four points per thread); tw: the N-point table.
__global__ void __launch_bounds__(kMaxThreads) k_pump_chi3_cluster(double2* __restrict__ pf, double2* __restrict__ pt,
                                                                   const double2* __restrict__ env,
                                                                   const double2* __restrict__ halfP,
                                                                   const double2* __restrict__ dstepP,
                                                                   const double2* __restrict__ backP,
                                                                   const double2* __restrict__ rel, int nRows,
                                                                   const FFTPlanH plan, const double2* __restrict__ tw) {
  constexpr int C = 4, R = C;
  extern __shared__ double2 smem[];
  cg::cluster_group cl = cg::this_cluster();
  ClusterFFT<C> f;
  f.plan = &plan;
  const int M = plan.N, T = plan.T;
  const int N = M * C;
  f.rank = (int)cl.block_rank();
  f.j = threadIdx.x;
  f.phase = 0;
  double2* twM = smem;
  double2* twC = smem + M;
  f.buf = smem + 2 * M;
  f.recv = smem + 3 * M;
  for (int k = threadIdx.x; k < M; k += blockDim.x) {
    twM[k] = tw[(long long)k * C];
    twC[k] = tw[(long long)f.rank * k];
  }
  __syncthreads();
  f.twM = twM;
  f.twC = twC;
  const int j = f.j, rank = f.rank;
  auto tn = [&](int v) { return rank + C * (j + v * T); };
  auto fk = [&](int v) { return j + rank * T + M * v; };
  const double invN = 1.0 / N;
  double2 x[R];
#pragma unroll
  for (int v = 0; v < R; v++) x[v] = env[tn(v)];
  cluster_fft_fwd<C>(f, x, cl);
#pragma unroll
  for (int v = 0; v < R; v++) {
    x[v] = cmul(x[v], halfP[fk(v)]);
    pf[fk(v)] = x[v];
  }
  cluster_fft_inv<C>(f, x, cl);
#pragma unroll
  for (int v = 0; v < R; v++) {
    x[v] = cscale(x[v], invN);
    pt[tn(v)] = x[v];
  }
  for (int i = 1; i < nRows; i++) {
    const double2 r = rel[i - 1];
#pragma unroll
    for (int v = 0; v < R; v++) {
      const double a2 = cabs2(x[v]);
      x[v] = cmul(x[v], spm_factor(r.x * a2, r.y * a2));
    }
    cluster_fft_fwd<C>(f, x, cl);
#pragma unroll
    for (int v = 0; v < R; v++) {
      x[v] = cmul(x[v], dstepP[fk(v)]);
      pf[(long long)i * N + fk(v)] = x[v];
    }
    cluster_fft_inv<C>(f, x, cl);
#pragma unroll
    for (int v = 0; v < R; v++) {
      x[v] = cscale(x[v], invN);
      pt[(long long)i * N + tn(v)] = x[v];
    }
  }
  // last row: undo half of the last pump dispersion step (each thread rereads its own bins)
  const long long last = (long long)(nRows - 1) * N;
#pragma unroll
  for (int v = 0; v < R; v++) {
    x[v] = cmul(pf[last + fk(v)], backP[fk(v)]);
    pf[last + fk(v)] = x[v];
  }
  cluster_fft_inv<C>(f, x, cl);
#pragma unroll
  for (int v = 0; v < R; v++) pt[last + tn(v)] = cscale(x[v], invN);
}

cudaError_t launch_pump_chi3_cluster(double2* pumpFreq, double2* pumpTime, const double2* env, const double2* halfP,
                                     const double2* dstepP, const double2* backP, const double2* rel, int nRows,
                                     const FFTPlanH& localPlan, const double2* tw, cudaStream_t s) {
  constexpr int C = 4;
  const int M = localPlan.N;
  // M-point twiddles x2, exchange buffer, 2 x C x T receive; each CTA alone on its SM
  size_t smem = 0;
  cudaError_t e = exclusive_smem((const void*)k_pump_chi3_cluster, (size_t)5 * M * sizeof(double2), &smem);
  if (e != cudaSuccess) return e;
  if (smem == 0) return cudaErrorInvalidValue;
  FFTPlanH plan = localPlan;
  void* args[] = {(void*)&pumpFreq, (void*)&pumpTime, (void*)&env, (void*)&halfP, (void*)&dstepP, (void*)&backP,
                  (void*)&rel, (void*)&nRows, (void*)&plan, (void*)&tw};
  return launch_clustered((const void*)k_pump_chi3_cluster, C, localPlan.T, smem, s, C, args);
}

}  // namespace nlm
