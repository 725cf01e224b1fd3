// nlm_spread.cuh -- one propagation on a cluster of four CTAs with ONE point per thread.
//
// The FP64 units of an SM belong to its four schedulers: each issues at most 0.5 DFMA lanes per
// clock, and only for its own warps.  The four-points-per-thread cluster transforms (nlm_cluster.cuh)
// give a grid of N points N/16 threads per CTA: below N = 2048 that is fewer than four warps per SM,
// so some schedulers idle.  Here every CTA holds M = N/4 points, one per thread: N = 512 gives four
// warps on each of the four SMs, four times the FP64 issue of one SM.  The transforms:
//   time domain:       CTA c, thread j  <->  point n = c + 4 j
//   frequency domain:  CTA c, thread j  <->  bin   k = j + M c
// forward:  M-point DFT over j of the CTA's strided points (radix-2 Stockham through shared memory,
//           one output per thread and stage: out = e + W o as two FMAs per component), twiddle
//           exp(-2 pi i c j / N), then the 4-point DFT over the CTAs: every thread pushes its value to
//           all four CTAs through distributed shared memory, one cluster barrier, and each thread
//           combines the four values of its own column for its CTA's output row;
// inverse:  the 4-point inverse DFT over the CTAs first, the conjugate twiddle, then the local inverse
//           DFT (unscaled; 1/N is in the tables).
// Shared memory: M twiddles, two M-point exchange buffers (alternating, one barrier per stage: a thread
// writes a buffer only after the barrier that every reader of that buffer's previous contents has
// passed), and two halves of 4 x M cluster receive buffers (alternating per transform: a CTA writes a
// half only after the cluster barrier that its readers passed after their last read of it).
#pragma once
#include <cooperative_groups.h>

#include "nlm_propagate.cuh"

namespace cg = cooperative_groups;

namespace nlm {

constexpr int kSpreadC = 4;
static_assert(kSpreadSmemPerPoint == 1 + 2 + 2 * kSpreadC, "twiddles, exchange buffers, receive halves");

struct SpreadFFT {
  const double2* twM;   // [M] exp(-2 pi i m / M), shared memory
  double2 twC;          // exp(-2 pi i c j / N) of this thread (rank c, thread j)
  double2* buf;         // [2][M] exchange buffers of the local transform
  double2* recv;        // [2][4][M] cluster receive buffers
  int M, rank, j;
  int sel, phase;       // next exchange buffer / receive half
  int base;             // cluster rank of the group's first CTA (clusters holding two groups of four)
};

// Sets up the spread transform of this CTA: the M-point twiddles (every C-th entry of the N-point
// table `tw`) and this thread's cluster twiddle.  Ends with a CTA barrier.
__device__ __forceinline__ void spread_init(SpreadFFT& f, double2* smem, const double2* __restrict__ tw, int M,
                                            int rank) {
  f.M = M;
  f.rank = rank;
  f.j = threadIdx.x;
  f.sel = 0;
  f.phase = 0;
  f.base = 0;
  double2* twM = smem;
  f.buf = smem + M;
  f.recv = smem + 3 * M;
  for (int k = threadIdx.x; k < M; k += blockDim.x) twM[k] = tw[(long long)k * kSpreadC];
  f.twM = twM;
  f.twC = tw[(long long)rank * f.j];
  __syncthreads();
}

// M-point DFT over the CTA's threads: thread t holds element t on entry and bin t on return.
// Stage L -> 2L: y'[k' + 2L p] = y[k + L p] + W_2L^k' y[k + L p + M/2], k = k' mod L.
template <bool INV>
__device__ __forceinline__ double2 spread_local(SpreadFFT& f, double2 x) {
  const int M = f.M, t = f.j, half = M >> 1;
  // first stage: W_2^k' = +-1
  {
    double2* b = f.buf + f.sel * M;
    b[t] = x;
    __syncthreads();
    const int p = t >> 1;
    const double2 e = b[p], o = b[p + half];
    const double s = (t & 1) ? -1.0 : 1.0;
    x = make_double2(fma(s, o.x, e.x), fma(s, o.y, e.y));
    f.sel ^= 1;
  }
  for (int L = 2, shift = 1; L < M; L <<= 1, shift++) {
    double2* b = f.buf + f.sel * M;
    b[t] = x;
    __syncthreads();
    const int kp = t & (2 * L - 1);
    const int k = kp & (L - 1);
    const int src = k + L * (t >> (shift + 1));
    const double2 e = b[src], o = b[src + half];
    const double2 w = f.twM[kp * (half >> shift)];   // W_2L^k' = W_M^(k' M / 2L)
    const double wy = INV ? -w.y : w.y;
    x.x = fma(-wy, o.y, fma(w.x, o.x, e.x));
    x.y = fma(wy, o.x, fma(w.x, o.y, e.y));
    f.sel ^= 1;
  }
  return x;
}

// 4-point DFT over the cluster's CTAs: thread j of every CTA pushes y to column j of row `rank` in all
// four CTAs; after the barrier thread j of CTA r returns sum_c W_4^(+-r c) recv[c][j].
template <bool INV>
__device__ __forceinline__ double2 spread_exchange(SpreadFFT& f, double2 y, cg::cluster_group& cl) {
  const int M = f.M;
  double2* half = f.recv + (long long)f.phase * kSpreadC * M;
#pragma unroll
  for (int v = 0; v < kSpreadC; v++) *cl.map_shared_rank(half + f.rank * M + f.j, f.base + v) = y;
  cl.sync();
  const double2 r0 = half[f.j], r1 = half[M + f.j], r2 = half[2 * M + f.j], r3 = half[3 * M + f.j];
  f.phase ^= 1;
  // a = r0 + (-1)^r r2, b = r1 + (-1)^r r3, out = a + W_4^(+-r) b with W_4 = -i (forward)
  const int r = f.rank;
  const double sg = (r & 1) ? -1.0 : 1.0;
  const double2 a = make_double2(fma(sg, r2.x, r0.x), fma(sg, r2.y, r0.y));
  const double2 b = make_double2(fma(sg, r3.x, r1.x), fma(sg, r3.y, r1.y));
  // W_4^(r) for r = 0..3: 1, -i, -1, i (forward); conjugates for the inverse
  const int q = INV ? (4 - r) & 3 : r;
  switch (q) {
    case 0: return make_double2(a.x + b.x, a.y + b.y);
    case 1: return make_double2(a.x + b.y, a.y - b.x);    // a - i b
    case 2: return make_double2(a.x - b.x, a.y - b.y);
    default: return make_double2(a.x - b.y, a.y + b.x);   // a + i b
  }
}

// n bare cluster barriers: the transform slots of a group that has no transform to do while the other
// group of the same cluster does (every exchange ends with a barrier of the whole cluster)
__device__ __forceinline__ void spread_idle(cg::cluster_group& cl, int n) {
  for (int q = 0; q < n; q++) cl.sync();
}

// time-domain ownership -> frequency-domain ownership
__device__ __forceinline__ double2 spread_fwd(SpreadFFT& f, double2 x, cg::cluster_group& cl) {
  x = spread_local<false>(f, x);
  return spread_exchange<false>(f, cmul(x, f.twC), cl);
}

// frequency-domain ownership -> time-domain ownership (unscaled)
__device__ __forceinline__ double2 spread_inv(SpreadFFT& f, double2 x, cg::cluster_group& cl) {
  x = cmulc(spread_exchange<true>(f, x, cl), f.twC);
  return spread_local<true>(f, x);
}

}  // namespace nlm
