// adjoint.cu -- reverse sweep of the split-step propagation for Chi2PDC (solvers/Chi2PDC.cpp:27-44).
//
// The reference has no gradient.  This is the exact discrete adjoint of what the forward kernels
// compute: for an output functional L of the last-row spectrum X, with g = dL/dRe + i dL/dIm, the
// sweep runs the z steps backwards,
//     g <- conj(table_i) * FFT(g),  g <- IFFT(g),  g <- RK4_i^T(g; s_{i-1})
// where RK4_i^T is the transposed RK4 step at each point, evaluated with the forward state s_{i-1}.
// s_{i-1} comes from checkpoints stored by the forward kernel every K steps; inside a segment the
// states are recomputed from its checkpoint (K = 1 stores every state and recomputes nothing), with
// the per-point RK4 propagator matrices when the engine provides them (PropArgs::prop).
// Per step the sweep also accumulates the gradients of the RK4 stage factors a_s = c_s P_s
// (c_s: poling sign x nonlinear step x phase mismatch of stage s, P_s: pump row 2i-2, 2i-1, 2i),
// from which the pump-spectrum and poling-profile gradients are reduced afterwards.
#include <vector>

#include <cooperative_groups.h>

#include "nlm_adjoint_pdc.cuh"

namespace cg = cooperative_groups;

namespace nlm {

// States s_{s0} .. s_{segEnd-1} of one segment, recomputed from its checkpoint into seg[0 ..].
template <int R>
__device__ __forceinline__ void pdc_recompute_segment(const PropArgs& a, const double2* ck, int jseg, int s0,
                                                      int segEnd, double2* seg, double2* buf, const double2* tw,
                                                      int j) {
  const FFTPlanH& plan = a.plan;
  const int N = plan.N, T = plan.T;
  double2 x[R];
#pragma unroll
  for (int v = 0; v < R; v++) {
    x[v] = ck[(long long)jseg * N + j + v * T];
    seg[j + v * T] = x[v];
  }
  for (int i = s0 + 1; i < segEnd; i++) {
#pragma unroll
    for (int v = 0; v < R; v++) x[v] = pdc_step_point(a, N, i, j + v * T, x[v]);
    fft_regs<R, false>(x, buf, tw, plan, j);
#pragma unroll
    for (int v = 0; v < R; v++) x[v] = cmul(x[v], __ldg(a.dstep + j + v * T));
    fft_regs<R, true>(x, buf, tw, plan, j);
#pragma unroll
    for (int v = 0; v < R; v++) seg[(long long)(i - s0) * N + j + v * T] = x[v];
  }
}

// Reverse steps i = segEnd .. s0+1; states[(i-1-s0) N ..] holds s_{i-1} (unused in the marching form).
template <int R>
__device__ __forceinline__ void pdc_reverse_segment(const PropArgs& a, const AdjArgs& d, const double2* states,
                                                    int s0, int segEnd, double2 (&gv)[R], bool active, double2* buf,
                                                    const double2* tw, int j, long long inst) {
  const FFTPlanH& plan = a.plan;
  const int N = plan.N, T = plan.T;
  for (int i = segEnd; i > s0; i--) {
    const double2* prev = states + (long long)(i - 1 - s0) * N;
    if (i < a.nZ - 1) fft_regs<R, false>(gv, buf, tw, plan, j);
    const double2* tab = (i == a.nZ - 1) ? a.dlast : a.dstep;
#pragma unroll
    for (int v = 0; v < R; v++) gv[v] = cmulc(gv[v], __ldg(tab + j + v * T));
    fft_regs<R, true>(gv, buf, tw, plan, j);
    if (d.gp) {
#pragma unroll
      for (int v = 0; v < R; v++) gv[v] = pdc_march_point(a, d, N, i, j + v * T, inst, gv[v], active);
      continue;
    }
    const double2* c = a.coef + (long long)(i - 1) * 3 * a.nCoef;
    const double2 c0 = c[0], c1 = c[1], c2 = c[2];
#pragma unroll
    for (int v = 0; v < R; v++) {
      const int t = j + v * T;
      gv[v] = pdc_reverse_point(a, d, N, i, t, c0, c1, c2, prev[t], gv[v], active);
    }
  }
}

template <int R>
__device__ __forceinline__ void pdc_load_gout(const PropArgs& a, const AdjArgs& d, long long inst, bool active,
                                              double2 (&gv)[R], int j) {
  const int N = a.plan.N, T = a.plan.T;
  const double2* go = d.gout + (active ? inst : 0) * (long long)N;
#pragma unroll
  for (int v = 0; v < R; v++) gv[v] = active ? cscale(go[j + v * T], (double)N) : czero();
}

// gradient of the input spectrum: s_0 = IFFT(half X_in)
template <int R>
__device__ __forceinline__ void pdc_store_gin(const PropArgs& a, const AdjArgs& d, long long inst, bool active,
                                              double2 (&gv)[R], double2* buf, const double2* tw, int j) {
  const int N = a.plan.N, T = a.plan.T;
  fft_regs<R, false>(gv, buf, tw, a.plan, j);
  if (active) {
#pragma unroll
    for (int v = 0; v < R; v++) d.gin[inst * (long long)N + j + v * T] = cmulc(gv[v], __ldg(a.half + j + v * T));
  }
}

template <int R>
__global__ void __launch_bounds__(kMaxThreads) k_adjoint_pdc(const PropArgs a, const AdjArgs d) {
  extern __shared__ double2 smem[];
  __shared__ long long s_group;
  const FFTPlanH& plan = a.plan;
  const int N = plan.N, T = plan.T;
  const int g = threadIdx.x / T, j = threadIdx.x - g * T;
  double2* bufs;
  const double2* tw = stage_twiddles<R>(a.tw, smem, N, &bufs);
  double2* buf = bufs + (long long)g * N;
  double2* segp = d.seg ? d.seg + ((long long)blockIdx.x * a.ipc + g) * (long long)d.K * N : nullptr;
  const long long nGroups = (a.nInst + a.ipc - 1) / a.ipc;
  for (long long cg = blockIdx.x; cg < nGroups; cg = next_group(a, cg, &s_group)) {
    const long long local = cg * a.ipc + g;
    const bool active = local < a.nInst;
    const long long inst = a.instBase + local;
    const double2* ck = d.ckpt + (active ? inst : 0) * (long long)d.nCk * N;
    double2 gv[R];
    pdc_load_gout<R>(a, d, inst, active, gv, j);
    int segEnd = a.nZ - 1;
    while (segEnd >= 1) {
      const int jseg = (segEnd - 1) / d.K;
      const int s0 = jseg * d.K;
      if (d.K > 1) pdc_recompute_segment<R>(a, ck, jseg, s0, segEnd, segp, buf, tw, j);
      pdc_reverse_segment<R>(a, d, d.K > 1 ? segp : ck + (long long)s0 * N, s0, segEnd, gv, active, buf, tw, j, inst);
      segEnd = s0;
    }
    pdc_store_gin<R>(a, d, inst, active, gv, buf, tw, j);
    __syncthreads();
  }
}

// Pipelined reverse sweep for checkpoint intervals K > 1, launched as clusters of two CTAs, one
// propagation per cluster at a time (ipc = 1).  CTA 1 of the cluster recomputes segment j-1 from
// its checkpoint while CTA 0 runs the reverse steps of segment j, so the recomputation that
// checkpointing adds runs on a second SM instead of lengthening the sweep.  The two alternate
// between two state buffers per cluster (d.seg: [cluster][2][K][N]); a cluster barrier (hardware,
// release/acquire at cluster scope) separates the iterations.  Both CTAs execute the same number of
// barriers: nSeg + 1 per propagation.
template <int R>
__global__ void __launch_bounds__(kMaxThreads) k_adjoint_pdc_pipe(const PropArgs a, const AdjArgs d) {
  extern __shared__ double2 smem[];
  cg::cluster_group cluster = cg::this_cluster();
  const FFTPlanH& plan = a.plan;
  const int N = plan.N;
  const int j = threadIdx.x;
  const int role = (int)cluster.block_rank();
  const long long clusterId = blockIdx.x / 2, nClusters = gridDim.x / 2;
  double2* buf;
  const double2* tw = stage_twiddles<R>(a.tw, smem, N, &buf);
  double2* states = d.seg + clusterId * 2LL * d.K * N;
  const int nSeg = (a.nZ - 2) / d.K + 1;
  for (long long local = clusterId; local < a.nInst; local += nClusters) {
    const long long inst = a.instBase + local;
    const double2* ck = d.ckpt + inst * (long long)d.nCk * N;
    double2 gv[R];
    if (role == 0) pdc_load_gout<R>(a, d, inst, true, gv, j);
    for (int it = 0; it <= nSeg; it++) {
      if (role == 1 && it < nSeg) {
        const int jseg = nSeg - 1 - it, s0 = jseg * d.K, segEnd = min(s0 + d.K, a.nZ - 1);
        pdc_recompute_segment<R>(a, ck, jseg, s0, segEnd, states + (long long)(it & 1) * d.K * N, buf, tw, j);
      }
      if (role == 0 && it >= 1) {
        const int jseg = nSeg - it, s0 = jseg * d.K, segEnd = min(s0 + d.K, a.nZ - 1);
        pdc_reverse_segment<R>(a, d, states + (long long)((it - 1) & 1) * d.K * N, s0, segEnd, gv, true, buf, tw, j,
                               inst);
      }
      cluster.sync();
    }
    if (role == 0) pdc_store_gin<R>(a, d, inst, true, gv, buf, tw, j);
    __syncthreads();
  }
}

// The stage-factor gradients of the marching form: for every step i and point t, the stage chain at
// the state before the step (checkpoint interval 1: d.ckpt row i-1) and the gradient after it (d.gp),
// summed over the rows.  Parallel over all steps and points, after the sequential march.
__global__ void k_adj_stage_grads(const PropArgs a, const AdjArgs d, int N, long long rows) {
  const long long total = (long long)(a.nZ - 1) * N;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(idx / N) + 1, t = (int)(idx - (long long)(i - 1) * N);
    const double2* c = a.coef + (long long)(i - 1) * 3 * a.nCoef;
    const double2 c0 = c[0], c1 = c[1], c2 = c[2];
    double2 s0 = czero(), s1 = czero(), s2 = czero();
    for (long long r = 0; r < rows; r++) {
      const double2 x = d.ckpt[(r * d.nCk + (i - 1)) * (long long)N + t];
      const double2 gp = d.gp[(r * (a.nZ - 1) + (i - 1)) * (long long)N + t];
      double2 g0, g1, g2;
      pdc_stage_chain(a, N, i, t, c0, c1, c2, x, gp, g0, g1, g2);
      s0 = cadd(s0, g0);
      s1 = cadd(s1, g1);
      s2 = cadd(s2, g2);
    }
    double2* gacc = d.ga + (long long)(i - 1) * 3 * N;
    gacc[t] = s0;
    gacc[N + t] = s1;
    gacc[2 * N + t] = s2;
  }
}

static int sm_count_adj();

cudaError_t launch_adj_stage_grads(const PropArgs& a, const AdjArgs& d, int N, long long rows, cudaStream_t s) {
  const long long total = (long long)(a.nZ - 1) * N;
  if (total <= 0) return cudaSuccess;
  long long grid = (total + 255) / 256;
  if (grid > 8LL * sm_count_adj()) grid = 8LL * sm_count_adj();
  k_adj_stage_grads<<<(unsigned)grid, 256, 0, s>>>(a, d, N, rows);
  return cudaGetLastError();
}

// Pump-row gradients: gP[r] = sum over the stages reading pump row r of conj(c_s) ga_s, times the
// intensity profile of the row (src/_NonlinearMedium.cpp:235-248).
__global__ void k_adj_pump_rows(const double2* __restrict__ ga, const double2* __restrict__ coef,
                                const double* __restrict__ prof, int nZ, int N, double2* __restrict__ gP) {
  const int nRows = 2 * nZ - 1;
  const long long total = (long long)nRows * N;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(idx / N), t = (int)(idx - (long long)r * N);
    double2 acc = czero();
    if (r & 1) {
      const int i = (r + 1) / 2;  // stage 1 (and 2) of step i reads row 2i-1
      acc = cmul(cconj(coef[(long long)(i - 1) * 3 + 1]), ga[((long long)(i - 1) * 3 + 1) * N + t]);
    } else {
      const int m = r / 2;
      if (m >= 1)  // last stage of step m reads row 2m
        acc = cmul(cconj(coef[(long long)(m - 1) * 3 + 2]), ga[((long long)(m - 1) * 3 + 2) * N + t]);
      if (m + 1 <= nZ - 1)  // first stage of step m+1 reads row 2m
        acc = cadd(acc, cmul(cconj(coef[(long long)m * 3]), ga[((long long)m * 3) * N + t]));
    }
    if (prof) acc = cscale(acc, prof[r]);
    gP[idx] = acc;
  }
}

// gF0[t] = (1/N) sum_r exp(-i r dzp D[t]) FFT(gP)[r][t]: the pump rows are IFFT(F0 exp(i r dzp D)).
// Grid: x over the bins, y over chunks of kPumpChunk rows.  Each chunk starts from an exact
// sincos and advances the phase by multiplying with exp(i dzp D) (error ~kPumpChunk ulp), and adds
// its partial sum into gF0 (zeroed by the launcher).
constexpr int kPumpChunk = 32;

__global__ void k_adj_pump_reduce(const double2* __restrict__ fgP, const double* __restrict__ disp, double dzp,
                                  int nRowsP, int N, double2* __restrict__ gF0) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= N) return;
  const int r0 = blockIdx.y * kPumpChunk;
  const int r1 = min(nRowsP, r0 + kPumpChunk);
  double sn, cs, sn1, cs1;
  sincos(((double)r0 * dzp) * disp[t], &sn, &cs);
  sincos(dzp * disp[t], &sn1, &cs1);
  double2 w = make_double2(cs, sn);
  const double2 step = make_double2(cs1, sn1);
  double2 acc = czero();
  for (int r = r0; r < r1; r++) {
    acc = cadd(acc, cmulc(fgP[(long long)r * N + t], w));
    w = cmul(w, step);
  }
  acc = cscale(acc, 1.0 / N);
  atomicAdd(&gF0[t].x, acc.x);
  atomicAdd(&gF0[t].y, acc.y);
}

// gc[i][s] = sum_t conj(P_row(i,s)[t]) ga[i][s][t]: gradient of the stage coefficient c_s of step i+1.
__global__ void k_adj_coef_reduce(const double2* __restrict__ ga, const double2* __restrict__ pump, int nZ, int N,
                                  double2* __restrict__ gc) {
  __shared__ double2 part[256];
  const int pair = blockIdx.x;          // (i-1)*3 + s
  const int i = pair / 3 + 1, s = pair % 3;
  const int row = 2 * i - 2 + s;
  double2 acc = czero();
  for (int t = threadIdx.x; t < N; t += blockDim.x)
    acc = cadd(acc, cmulc(ga[(long long)pair * N + t], pump[(long long)row * N + t]));
  part[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) part[threadIdx.x] = cadd(part[threadIdx.x], part[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) gc[pair] = part[0];
}

static int sm_count_adj() {
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 1;
}

cudaError_t launch_adj_pump_rows(const double2* ga, const double2* coef, const double* prof, int nZ, int N,
                                 double2* gP, cudaStream_t s) {
  const long long total = (long long)(2 * nZ - 1) * N;
  int grid = (int)((total + 255) / 256);
  if (grid > 32 * sm_count_adj()) grid = 32 * sm_count_adj();
  k_adj_pump_rows<<<grid > 0 ? grid : 1, 256, 0, s>>>(ga, coef, prof, nZ, N, gP);
  return cudaGetLastError();
}

cudaError_t launch_adj_pump_reduce(const double2* fgP, const double* disp, double dzp, int nRowsP, int N,
                                   double2* gF0, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(gF0, 0, (size_t)N * sizeof(double2), s);
  if (e != cudaSuccess) return e;
  const dim3 grid((unsigned)((N + 127) / 128), (unsigned)((nRowsP + kPumpChunk - 1) / kPumpChunk));
  k_adj_pump_reduce<<<grid, 128, 0, s>>>(fgP, disp, dzp, nRowsP, N, gF0);
  return cudaGetLastError();
}

cudaError_t launch_adj_coef_reduce(const double2* ga, const double2* pump, int nZ, int N, double2* gc,
                                   cudaStream_t s) {
  if (nZ < 2) return cudaSuccess;
  k_adj_coef_reduce<<<3 * (nZ - 1), 256, 0, s>>>(ga, pump, nZ, N, gc);
  return cudaGetLastError();
}

// key = solver id + 100: the pipelined two-CTA-cluster variant (checkpoint interval > 1)
void add_kernels_adjoint(std::vector<KernelEntry>& t) {
  t.push_back({kKindAdjoint, kChi2PDC + 100, 4, (const void*)k_adjoint_pdc_pipe<4>});
  t.push_back({kKindAdjoint, kChi2PDC + 100, 8, (const void*)k_adjoint_pdc_pipe<8>});
  t.push_back({kKindAdjoint, kChi2PDC + 100, 16, (const void*)k_adjoint_pdc_pipe<16>});
  t.push_back({kKindAdjoint, kChi2PDC, 4, (const void*)k_adjoint_pdc<4>});
  t.push_back({kKindAdjoint, kChi2PDC, 8, (const void*)k_adjoint_pdc<8>});
  t.push_back({kKindAdjoint, kChi2PDC, 16, (const void*)k_adjoint_pdc<16>});
}

}  // namespace nlm
