// prop_ff.cu -- single-mode linear split-step propagation in double-float arithmetic on the FP32 pipes.
//
// Same algorithm, data flow and index maps as k_propagate_linear<1, R> (nlm_propagate.cuh): per step
// the exact RK4 propagator of the undepleted-pump equation (a 2x2 real matrix per point) followed by
// the dispersion half step (forward FFT, table, inverse FFT).  Every value is a float-float pair
// (nlm_ff.cuh, ~48-bit significand), so the work runs on the FP32 units (61x the FP64 rate on this
// part) instead of the FP64 units; the tables are float-float copies of the FP64 tables.  Inputs and
// outputs stay FP64 (double2) in HBM.
#include <vector>

#include "nlm_ff.cuh"
#include "nlm_propagate.cuh"

namespace nlm {

// SMALL: radix of the one non-radix-8 pass of the plan (1 = none).  The z march is written as a
// loop over stages s = 0..last, each [inverse FFT][RK4 propagator][forward FFT][table], so that the
// kernel holds one forward and one inverse transform (the code of a float-float transform is large
// enough for instruction fetch to matter):
//   s = 0:          [forward FFT if the input is in the time domain] x exp(+i dz/2 D)/N
//   s = 1..nZ-1:    inverse FFT, propagator of step s, forward FFT, dispStep/N (dispStep exp(-i dz/2 D)/N last)
//   nZ = 1:         s = 1 is inverse FFT, forward FFT, exp(-i dz/2 D)/N (no propagator)
//   time-domain output: one more inverse FFT.
template <int R, int SMALL>
__device__ __forceinline__ void linear_ff_body(const PropArgs& a, const FFTables& f) {
  extern __shared__ float4 fsm[];
  __shared__ long long s_group;
  const FFTPlanH& plan = a.plan;
  const int N = plan.N, T = plan.T;
  const int g = threadIdx.x / T, j = threadIdx.x - g * T;
  const float4* tw;
  float4* bufs;
  if constexpr (R != 16) {   // twiddles staged in shared memory in front of the exchange buffers
    for (int k = threadIdx.x; k < N; k += blockDim.x) fsm[k] = f.tw[k];
    __syncthreads();
    tw = fsm;
    bufs = fsm + N;
  } else {
    tw = f.tw;
    bufs = fsm;
  }
  float4* buf = bufs + (long long)g * N;
  const long long nGroups = (a.nInst + a.ipc - 1) / a.ipc;
  const int last = a.nZ > 1 ? a.nZ - 1 : 1;
  for (long long cg = blockIdx.x; cg < nGroups; cg = next_group(a, cg, &s_group)) {
    const long long local = cg * a.ipc + g;
    const bool active = local < a.nInst;
    const long long inst = a.instBase + local;
    ffc x[R];
    if (a.inKind == 0) {
      // impulses: instance = ((im * N) + bin) * 2 + which; value 1 (which 0) or i (which 1)
      const long long pair = inst >> 1;
      const int bin = (int)(pair % N);
      const int im = (int)(pair / N);
      const int mode = active ? a.impModes[im < kMaxModes ? im : 0] : -1;
      const ffc val = (inst & 1) ? ffc{ff{0.f, 0.f}, ff{1.f, 0.f}} : ffc{ff{1.f, 0.f}, ff{0.f, 0.f}};
#pragma unroll
      for (int v = 0; v < R; v++) x[v] = (mode == 0 && j + v * T == bin) ? val : ffc_zero();
    } else {
      const double2* row = a.in + (active ? inst : 0) * a.inStride;
      const bool has = a.inputMode == 0 || (a.inputMode < 1 && a.inChannels > 0);
#pragma unroll
      for (int v = 0; v < R; v++) x[v] = (active && has) ? ffc_from(row[j + v * T]) : ffc_zero();
    }
    for (int s = 0;; s++) {
      if (s > 0) ffft_regs<R, SMALL, true>(x, buf, tw, plan, j);
      if (s > last) break;
      if (s > 0 && a.nZ > 1) {
        const float4* mat = f.prop + (long long)(s - 1) * 2 * N;
#pragma unroll
        for (int v = 0; v < R; v++) {
          const int t = j + v * T;
          const float4 e0 = __ldg(mat + t), e1 = __ldg(mat + N + t);
          const ff re = ff_dot2(ff{e0.x, e0.y}, x[v].re, ff{e0.z, e0.w}, x[v].im);
          const ff im = ff_dot2(ff{e1.x, e1.y}, x[v].re, ff{e1.z, e1.w}, x[v].im);
          x[v] = ffc{re, im};
        }
      }
      if (s > 0 || a.inTime) ffft_regs<R, SMALL, false>(x, buf, tw, plan, j);
      const float4* tab = s == 0 ? f.half : (a.nZ == 1 ? f.back : (s == last ? f.dlast : f.dstep));
#pragma unroll
      for (int v = 0; v < R; v++) x[v] = fmul(x[v], ffc_ldg(tab + j + v * T));
      if (s == last && !a.inTime) break;
    }
    if (active && a.out != nullptr) {
      const double scale = a.inTime ? 1.0 : (double)N;
      double2* o = a.out + inst * a.outStride;
      for (int om = 0; om < a.nOut; om++) {
        if (a.outModes[om] != 0) continue;
#pragma unroll
        for (int v = 0; v < R; v++) o[(long long)om * N + j + v * T] = cscale(ffc_to(x[v]), scale);
      }
    }
    __syncthreads();
  }
}

template <int R, int SMALL>
__global__ void __launch_bounds__(kMaxThreads) k_propagate_linear_ff(const PropArgs a, const FFTables f) {
  linear_ff_body<R, SMALL>(a, f);
}

// 128-thread CTAs with at least MINB resident per SM (fewer registers, more warps); an autotuner
// candidate where a CTA has 128 threads.
template <int R, int SMALL, int MINB>
__global__ void __launch_bounds__(128, MINB) k_propagate_linear_ff_occ(const PropArgs a, const FFTables f) {
  linear_ff_body<R, SMALL>(a, f);
}

constexpr int kMaxSplitSegs = 8;
struct SplitBatch {
  SplitSeg seg[kMaxSplitSegs];
  int n;
};

__global__ void k_split_ff(const SplitBatch b) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (int s = 0; s < b.n; s++) {
    const SplitSeg g = b.seg[s];
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < g.n; k += stride) {
      const double2 v = g.src[k];
      const float rh = __double2float_rn(v.x), ih = __double2float_rn(v.y);
      g.dst[k] = make_float4(rh, __double2float_rn(v.x - (double)rh), ih, __double2float_rn(v.y - (double)ih));
    }
  }
}

cudaError_t launch_split_ff(const SplitSeg* segs, int nSegs, cudaStream_t s) {
  long long longest = 0;
  for (int k0 = 0; k0 < nSegs; k0 += kMaxSplitSegs) {
    SplitBatch b{};
    b.n = nSegs - k0 < kMaxSplitSegs ? nSegs - k0 : kMaxSplitSegs;
    longest = 0;
    for (int k = 0; k < b.n; k++) {
      b.seg[k] = segs[k0 + k];
      if (b.seg[k].n > longest) longest = b.seg[k].n;
    }
    if (longest == 0) continue;
    long long blocks = (longest + 255) / 256;
    if (blocks > 152LL * 8) blocks = 152LL * 8;
    k_split_ff<<<(unsigned)blocks, 256, 0, s>>>(b);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// key = M + 10 * SMALL (single mode; SMALL the radix of the plan's short pass)
void add_kernels_ff(std::vector<KernelEntry>& t) {
  t.push_back({kKindLinearFF, 1 + 10 * 1, 8, (const void*)k_propagate_linear_ff<8, 1>});
  t.push_back({kKindLinearFF, 1 + 10 * 2, 8, (const void*)k_propagate_linear_ff<8, 2>});
  t.push_back({kKindLinearFF, 1 + 10 * 4, 8, (const void*)k_propagate_linear_ff<8, 4>});
  // autotuner candidates: 128-thread CTAs with 5 or 6 resident per SM (96 / 80 registers)
  t.push_back({kKindLinearFF, 1 + 10 * 1, 8, (const void*)k_propagate_linear_ff_occ<8, 1, 5>});
  t.push_back({kKindLinearFF, 1 + 10 * 2, 8, (const void*)k_propagate_linear_ff_occ<8, 2, 5>});
  t.push_back({kKindLinearFF, 1 + 10 * 4, 8, (const void*)k_propagate_linear_ff_occ<8, 4, 5>});
  t.push_back({kKindLinearFF, 1 + 10 * 1, 8, (const void*)k_propagate_linear_ff_occ<8, 1, 6>});
  t.push_back({kKindLinearFF, 1 + 10 * 2, 8, (const void*)k_propagate_linear_ff_occ<8, 2, 6>});
  t.push_back({kKindLinearFF, 1 + 10 * 4, 8, (const void*)k_propagate_linear_ff_occ<8, 4, 6>});
}

}  // namespace nlm
