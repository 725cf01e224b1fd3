// nlm_spread.cuh -- one propagation on a cluster of four (or eight) CTAs with ONE point per thread.
//
// The FP64 units of an SM belong to its four schedulers: each issues at most 0.5 DFMA lanes per
// clock, and only for its own warps.  The four-points-per-thread cluster transforms (nlm_cluster.cuh)
// give a grid of N points N/16 threads per CTA: below N = 2048 that is fewer than four warps per SM,
// so some schedulers idle.  Here every CTA holds M = N/4 points, one per thread: N = 512 gives four
// warps on each of the four SMs, four times the FP64 issue of one SM.  With C = 8 CTAs (M = N/8) the
// same form doubles the SMs of a 2048- or 4096-point propagation, and C = 16 (a non-portable cluster
// size) doubles them again for the longest marches of a ragged batch.  The transforms:
//   time domain:       CTA c, thread j  <->  point n = c + C j
//   frequency domain:  CTA c, thread j  <->  bin   k = j + M c
// forward:  M-point DFT over j of the CTA's strided points (radix-2 Stockham through shared memory,
//           one output per thread and stage: out = e + W o as two FMAs per component), twiddle
//           exp(-2 pi i c j / N), then the C-point DFT over the CTAs: every thread pushes its value to
//           all C CTAs through distributed shared memory, one cluster barrier, and each thread
//           combines the C values of its own column for its CTA's output row;
// inverse:  the C-point inverse DFT over the CTAs first, the conjugate twiddle, then the local inverse
//           DFT (unscaled; 1/N is in the tables).
// Shared memory: M twiddles, two M-point exchange buffers (alternating, one barrier per stage: a thread
// writes a buffer only after the barrier that every reader of that buffer's previous contents has
// passed), and two halves of C x M cluster receive buffers (alternating per transform: a CTA writes a
// half only after the cluster barrier that its readers passed after their last read of it).
#pragma once
#include <cooperative_groups.h>

#include "nlm_propagate.cuh"

namespace cg = cooperative_groups;

namespace nlm {

constexpr int kSpreadC = 4;
static_assert(kSpreadSmemPerPoint == spread_smem_per_point(kSpreadC), "twiddles, exchange buffers, receive halves");

struct SpreadFFT {
  const double2* twM;   // [M] exp(-2 pi i m / M), shared memory
  double2 twC;          // exp(-2 pi i c j / N) of this thread (rank c, thread j)
  double2* buf;         // [2][M] exchange buffers of the local transform
  double2* recv;        // [2][C][M] cluster receive buffers
  int M, rank, j;
  int sel, phase;       // next exchange buffer / receive half
  int base;             // cluster rank of the group's first CTA (clusters holding two groups of four)
};

// Sets up the spread transform of this CTA: the M-point twiddles (every C-th entry of the N-point
// table `tw`) and this thread's cluster twiddle.  Ends with a CTA barrier.  K: fields transformed
// together (spread_fwd_k, spread_inv_store_k), which sizes the exchange and receive buffers.
template <int C = kSpreadC, int K = 1>
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
  f.recv = smem + (1 + 2 * K) * M;
  for (int k = threadIdx.x; k < M; k += blockDim.x) twM[k] = tw[(long long)k * C];
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

// C-point DFT of the values r[c] of this thread's column: sum_c W_C^(+-rank c) r[c].
template <bool INV, int C>
__device__ __forceinline__ double2 spread_combine(const SpreadFFT& f, const double2 (&r)[C]) {
  const int rk = f.rank;
  const double sg = (rk & 1) ? -1.0 : 1.0;   // W_C^(r C/2) = (-1)^r
  // W_4^(+-r) b for the four quarter turns: 1, -i, -1, i (forward); conjugates for the inverse
  const int q = INV ? (4 - (rk & 3)) & 3 : (rk & 3);
  auto quarter = [q](double2 b) {
    switch (q) {
      case 0: return b;
      case 1: return make_double2(b.y, -b.x);    // -i b
      case 2: return make_double2(-b.x, -b.y);
      default: return make_double2(-b.y, b.x);   // i b
    }
  };
  if constexpr (C == 4) {
    // a = r0 + (-1)^r r2, b = r1 + (-1)^r r3, out = a + W_4^(+-r) b
    const double2 a = make_double2(fma(sg, r[2].x, r[0].x), fma(sg, r[2].y, r[0].y));
    const double2 b = quarter(make_double2(fma(sg, r[3].x, r[1].x), fma(sg, r[3].y, r[1].y)));
    return make_double2(a.x + b.x, a.y + b.y);
  } else if constexpr (C == 8) {
    // u_c = r_c + (-1)^r r_(c+4); v0 = u0 + W_4^r u2, v1 = u1 + W_4^r u3; out = v0 + W_8^r v1
    double2 u[4];
#pragma unroll
    for (int c = 0; c < 4; c++) u[c] = make_double2(fma(sg, r[c + 4].x, r[c].x), fma(sg, r[c + 4].y, r[c].y));
    const double2 q2 = quarter(u[2]), q3 = quarter(u[3]);
    const double2 v0 = make_double2(u[0].x + q2.x, u[0].y + q2.y);
    const double2 v1 = make_double2(u[1].x + q3.x, u[1].y + q3.y);
    const double2 w = f.twM[rk * (f.M / 8)];    // W_8^r = W_M^(r M / 8)
    const double wy = INV ? -w.y : w.y;
    return make_double2(fma(-wy, v1.y, fma(w.x, v1.x, v0.x)), fma(wy, v1.x, fma(w.x, v1.y, v0.y)));
  } else {
    // sixteen CTAs: u_c = r_c + (-1)^r r_(c+8) (c < 8); w_c = u_c + W_4^r u_(c+4) (c < 4);
    // y_c = w_c + W_8^r w_(c+2) (c < 2); out = y_0 + W_16^r y_1
    static_assert(C == 16, "four, eight or sixteen CTAs");
    double2 u[8], w[4];
#pragma unroll
    for (int c = 0; c < 8; c++) u[c] = make_double2(fma(sg, r[c + 8].x, r[c].x), fma(sg, r[c + 8].y, r[c].y));
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const double2 q4 = quarter(u[c + 4]);
      w[c] = make_double2(u[c].x + q4.x, u[c].y + q4.y);
    }
    const double2 w8 = f.twM[(rk & 7) * (f.M / 8)];   // W_8^r
    const double w8y = INV ? -w8.y : w8.y;
    double2 y[2];
#pragma unroll
    for (int c = 0; c < 2; c++)
      y[c] = make_double2(fma(-w8y, w[c + 2].y, fma(w8.x, w[c + 2].x, w[c].x)),
                          fma(w8y, w[c + 2].x, fma(w8.x, w[c + 2].y, w[c].y)));
    const double2 w16 = f.twM[rk * (f.M / 16)];       // W_16^r = W_M^(r M / 16)
    const double w16y = INV ? -w16.y : w16.y;
    return make_double2(fma(-w16y, y[1].y, fma(w16.x, y[1].x, y[0].x)),
                        fma(w16y, y[1].x, fma(w16.x, y[1].y, y[0].y)));
  }
}

// C-point DFT over the cluster's CTAs: thread j of every CTA pushes y to column j of row `rank` in all
// C CTAs; after the barrier thread j of CTA r returns sum_c W_C^(+-r c) recv[c][j].
template <bool INV, int C = kSpreadC>
__device__ __forceinline__ double2 spread_exchange(SpreadFFT& f, double2 y, cg::cluster_group& cl) {
  static_assert(C == 4 || C == 8 || C == 16, "four, eight or sixteen CTAs");
  const int M = f.M;
  double2* half = f.recv + (long long)f.phase * C * M;
#pragma unroll
  for (int v = 0; v < C; v++) *cl.map_shared_rank(half + f.rank * M + f.j, f.base + v) = y;
  cl.sync();
  double2 r[C];
#pragma unroll
  for (int c = 0; c < C; c++) r[c] = half[c * M + f.j];
  f.phase ^= 1;
  return spread_combine<INV, C>(f, r);
}

// ---- K fields at once (the modes of a multi-mode solver): the same transforms with one barrier per
// stage and one cluster barrier per exchange for all K, and K independent chains in flight per thread.
// Buffers: [2][K][M] exchange, [2][C][K][M] receive.
template <bool INV, int K>
__device__ __forceinline__ void spread_local_k(SpreadFFT& f, double2 (&x)[K]) {
  const int M = f.M, t = f.j, half = M >> 1;
  {
    double2* b = f.buf + f.sel * K * M;
#pragma unroll
    for (int m = 0; m < K; m++) b[m * M + t] = x[m];
    __syncthreads();
    const int p = t >> 1;
    const double s = (t & 1) ? -1.0 : 1.0;
#pragma unroll
    for (int m = 0; m < K; m++) {
      const double2 e = b[m * M + p], o = b[m * M + p + half];
      x[m] = make_double2(fma(s, o.x, e.x), fma(s, o.y, e.y));
    }
    f.sel ^= 1;
  }
  for (int L = 2, shift = 1; L < M; L <<= 1, shift++) {
    double2* b = f.buf + f.sel * K * M;
#pragma unroll
    for (int m = 0; m < K; m++) b[m * M + t] = x[m];
    __syncthreads();
    const int kp = t & (2 * L - 1);
    const int k = kp & (L - 1);
    const int src = k + L * (t >> (shift + 1));
    const double2 w = f.twM[kp * (half >> shift)];
    const double wy = INV ? -w.y : w.y;
#pragma unroll
    for (int m = 0; m < K; m++) {
      const double2 e = b[m * M + src], o = b[m * M + src + half];
      x[m].x = fma(-wy, o.y, fma(w.x, o.x, e.x));
      x[m].y = fma(wy, o.x, fma(w.x, o.y, e.y));
    }
    f.sel ^= 1;
  }
}

template <bool INV, int C, int K>
__device__ __forceinline__ void spread_exchange_k(SpreadFFT& f, double2 (&y)[K], cg::cluster_group& cl) {
  static_assert(C == 4 || C == 8 || C == 16, "four, eight or sixteen CTAs");
  const int M = f.M;
  double2* half = f.recv + (long long)f.phase * C * K * M;
#pragma unroll
  for (int v = 0; v < C; v++) {
    double2* dst = cl.map_shared_rank(half + (long long)f.rank * K * M + f.j, f.base + v);
#pragma unroll
    for (int m = 0; m < K; m++) dst[m * M] = y[m];
  }
  cl.sync();
#pragma unroll
  for (int m = 0; m < K; m++) {
    double2 r[C];
#pragma unroll
    for (int c = 0; c < C; c++) r[c] = half[((long long)c * K + m) * M + f.j];
    y[m] = spread_combine<INV, C>(f, r);
  }
  f.phase ^= 1;
}

// time-domain ownership -> frequency-domain ownership, K fields
template <int C, int K>
__device__ __forceinline__ void spread_fwd_k(SpreadFFT& f, double2 (&x)[K], cg::cluster_group& cl) {
  spread_local_k<false, K>(f, x);
#pragma unroll
  for (int m = 0; m < K; m++) x[m] = cmul(x[m], f.twC);
  spread_exchange_k<false, C, K>(f, x, cl);
}

// frequency-domain ownership -> time-domain ownership (unscaled), K fields; store(m, v) receives each
// field's frequency-domain value right after the exchange's cluster barrier (see spread_inv_store)
template <int C, int K, class Store>
__device__ __forceinline__ void spread_inv_store_k(SpreadFFT& f, double2 (&x)[K], cg::cluster_group& cl, Store store) {
  double2 y[K];
#pragma unroll
  for (int m = 0; m < K; m++) y[m] = x[m];
  spread_exchange_k<true, C, K>(f, y, cl);
#pragma unroll
  for (int m = 0; m < K; m++) store(m, x[m]);
#pragma unroll
  for (int m = 0; m < K; m++) x[m] = cmulc(y[m], f.twC);
  spread_local_k<true, K>(f, x);
}

// n bare cluster barriers: the transform slots of a group that has no transform to do while the other
// group of the same cluster does (every exchange ends with a barrier of the whole cluster)
__device__ __forceinline__ void spread_idle(cg::cluster_group& cl, int n) {
  for (int q = 0; q < n; q++) cl.sync();
}

// time-domain ownership -> frequency-domain ownership
template <int C = kSpreadC>
__device__ __forceinline__ double2 spread_fwd(SpreadFFT& f, double2 x, cg::cluster_group& cl) {
  x = spread_local<false>(f, x);
  return spread_exchange<false, C>(f, cmul(x, f.twC), cl);
}

// frequency-domain ownership -> time-domain ownership (unscaled)
template <int C = kSpreadC>
__device__ __forceinline__ double2 spread_inv(SpreadFFT& f, double2 x, cg::cluster_group& cl) {
  x = cmulc(spread_exchange<true, C>(f, x, cl), f.twC);
  return spread_local<true>(f, x);
}

// spread_inv, with `store(x)` (the global store of the frequency-domain value) issued right after the
// exchange's cluster barrier instead of before it: the barrier's release fence then does not wait for
// the store, which drains during the local transform.
template <int C = kSpreadC, class Store>
__device__ __forceinline__ double2 spread_inv_store(SpreadFFT& f, double2 x, cg::cluster_group& cl, Store store) {
  const double2 y = spread_exchange<true, C>(f, x, cl);
  store(x);
  return spread_local<true>(f, cmulc(y, f.twC));
}

}  // namespace nlm
