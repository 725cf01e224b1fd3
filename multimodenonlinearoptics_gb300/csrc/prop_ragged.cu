// prop_ragged.cu -- one persistent launch over a ragged set of media (different grids, step counts,
// dispersion, poling and pumps), one seeded signal each.
//
// Every medium is an item described by its own PropArgs (tables, pump grid, per-step coefficients,
// input and output rows).  The host orders the items by cost (largest first); CTAs claim them from a
// work counter.  A CTA is sized for the largest grid of the set; for a smaller grid the threads past
// N/R take part in the barriers only.  The RK4 step is the solver's DiffEq evaluated per point
// (src/_NonlinearMedium.hpp:204-218 with solvers/*.cpp DiffEq), the dispersion half of the step is the
// register/shared-memory Stockham transform pair.  For pump-driven (linear) solvers the engine passes
// each medium's precomputed per-point RK4 matrices (PropArgs::prop, built in parallel over all steps
// and points before the launch), so the sequential march does a small matrix-vector product per point
// instead of the four stage evaluations.
#include <vector>

#include "nlm_propagate.cuh"

namespace nlm {

template <class S, int R>
__global__ void __launch_bounds__(kMaxThreads) k_propagate_ragged(const PropArgs* __restrict__ items, int nItems,
                                                                  unsigned long long* __restrict__ work) {
  constexpr int M = S::kM, P = S::kP > 0 ? S::kP : 1;
  extern __shared__ double2 buf[];
  __shared__ PropArgs sa;
  __shared__ int s_item;
  const int j = threadIdx.x;
  int item = blockIdx.x;
  while (item < nItems) {
    __syncthreads();  // the previous item's readers of sa are done
    {
      const unsigned* src = reinterpret_cast<const unsigned*>(items + item);
      unsigned* dst = reinterpret_cast<unsigned*>(&sa);
      for (int w = threadIdx.x; w < (int)(sizeof(PropArgs) / sizeof(unsigned)); w += blockDim.x) dst[w] = src[w];
    }
    __syncthreads();
    const PropArgs& a = sa;
    const FFTPlanH& plan = a.plan;
    const int N = plan.N, T = plan.T;
    const bool act = j < T;
    double2 x[M][R];
    // input row: one N-block into inputMode, or several into the first modes (src/_NonlinearMedium.hpp:164-192)
#pragma unroll
    for (int m = 0; m < M; m++) {
      int seg = -1;
      if (m == a.inputMode) seg = 0;
      else if (a.inputMode < 1 && m < a.inChannels) seg = m;
#pragma unroll
      for (int v = 0; v < R; v++) {
        x[m][v] = czero();
        if (act && seg >= 0) x[m][v] = a.in[(long long)seg * N + j + v * T];
      }
    }
#pragma unroll
    for (int m = 0; m < M; m++) {
      if (a.inTime) fft_regs<R, false, true>(x[m], buf, a.tw, plan, j, act);
      if (act) {
#pragma unroll
        for (int v = 0; v < R; v++) x[m][v] = cmul(x[m][v], __ldg(a.half + (long long)m * N + j + v * T));
      }
      fft_regs<R, true, true>(x[m], buf, a.tw, plan, j, act);
    }
    for (int i = 1; i < a.nZ; i++) {
      const double2* c = a.coef + (long long)(i - 1) * 3 * a.nCoef;
      if (act && a.prop) {
        // pump-driven solvers: the RK4 step as its per-point real (2M)x(2M) matrix, stored as pairs
        // (row r, columns 2c and 2c+1) at [step][r * M + c][N]
        constexpr int D = 2 * M;
        const double2* mat = reinterpret_cast<const double2*>(a.prop) + (long long)(i - 1) * (D * D / 2) * N;
#pragma unroll
        for (int v = 0; v < R; v++) {
          const int t = j + v * T;
          double in[D], outv[D];
#pragma unroll
          for (int m = 0; m < M; m++) {
            in[2 * m] = x[m][v].x;
            in[2 * m + 1] = x[m][v].y;
          }
#pragma unroll
          for (int r = 0; r < D; r++) {
            double acc = 0.0;
#pragma unroll
            for (int cc = 0; cc < D / 2; cc++) {
              const double2 e = __ldg(mat + (long long)(r * (D / 2) + cc) * N + t);
              acc = fma(e.x, in[2 * cc], acc);
              acc = fma(e.y, in[2 * cc + 1], acc);
            }
            outv[r] = acc;
          }
#pragma unroll
          for (int m = 0; m < M; m++) x[m][v] = make_double2(outv[2 * m], outv[2 * m + 1]);
        }
      } else if (act) {
#pragma unroll
        for (int v = 0; v < R; v++) {
          const int t = j + v * T;
          double2 p[3][P];
#pragma unroll
          for (int q = 0; q < P; q++) {
            if (S::kP > 0) {
              const double2* pr = a.pump + q * a.pumpStride + (long long)(2 * i - 2) * N + t;
              p[0][q] = __ldg(pr);
              p[1][q] = __ldg(pr + N);
              p[2][q] = __ldg(pr + 2 * N);
            } else {
              p[0][q] = p[1][q] = p[2][q] = czero();
            }
          }
          double2 xm[M];
#pragma unroll
          for (int m = 0; m < M; m++) xm[m] = x[m][v];
          rk4_point<S>(xm, p, c);
#pragma unroll
          for (int m = 0; m < M; m++) x[m][v] = xm[m];
        }
      }
      const bool last = i == a.nZ - 1;
      const double2* table = last ? a.dlast : a.dstep;
#pragma unroll
      for (int m = 0; m < M; m++) {
        fft_regs<R, false, true>(x[m], buf, a.tw, plan, j, act);
        if (act) {
#pragma unroll
          for (int v = 0; v < R; v++) x[m][v] = cmul(x[m][v], __ldg(table + (long long)m * N + j + v * T));
        }
        if (!last || a.inTime) fft_regs<R, true, true>(x[m], buf, a.tw, plan, j, act);
      }
    }
    if (a.nZ == 1) {
#pragma unroll
      for (int m = 0; m < M; m++) {
        fft_regs<R, false, true>(x[m], buf, a.tw, plan, j, act);
        if (act) {
#pragma unroll
          for (int v = 0; v < R; v++) x[m][v] = cmul(x[m][v], __ldg(a.back + (long long)m * N + j + v * T));
        }
        if (a.inTime) fft_regs<R, true, true>(x[m], buf, a.tw, plan, j, act);
      }
    }
    if (act) {
      const double sc = a.inTime ? 1.0 : (double)N;
      for (int om = 0; om < a.nOut; om++) {
#pragma unroll
        for (int m = 0; m < M; m++) {
          if (m != a.outModes[om]) continue;
#pragma unroll
          for (int v = 0; v < R; v++) a.out[(long long)om * N + j + v * T] = cscale(x[m][v], sc);
        }
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) s_item = (int)atomicAdd(work, 1ULL) + (int)gridDim.x;
    __syncthreads();
    item = s_item;
  }
}

void add_kernels_ragged(std::vector<KernelEntry>& t) {
  t.push_back({kKindRagged, kChi3, 8, (const void*)k_propagate_ragged<FChi3, 8>});
  t.push_back({kKindRagged, kChi2PDC, 8, (const void*)k_propagate_ragged<FChi2PDC, 8>});
  t.push_back({kKindRagged, kChi2SFG, 8, (const void*)k_propagate_ragged<FChi2SFG, 8>});
  // four points per thread: N/4 threads per medium (all four schedulers of an SM from N = 512)
  t.push_back({kKindRagged, kChi3, 4, (const void*)k_propagate_ragged<FChi3, 4>});
  t.push_back({kKindRagged, kChi2PDC, 4, (const void*)k_propagate_ragged<FChi2PDC, 4>});
  t.push_back({kKindRagged, kChi2SFG, 4, (const void*)k_propagate_ragged<FChi2SFG, 4>});
}

}  // namespace nlm
