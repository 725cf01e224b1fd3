// nlm_spread.cuh -- one propagation on a cluster of four (or eight) CTAs with ONE point per thread.
//
// The FP64 units of an SM belong to its four schedulers: each issues at most 0.5 DFMA lanes per
// clock, and only for its own warps.  The four-points-per-thread cluster transforms (nlm_cluster.cuh)
// give a grid of N points N/16 threads per CTA: below N = 2048 that is fewer than four warps per SM,
// so some schedulers idle.  Here every CTA holds M = N/4 points, one per thread: N = 512 gives four
// warps on each of the four SMs, four times the FP64 issue of one SM.  With C = 8 CTAs (M = N/8) the
// same form doubles the SMs of a 2048- or 4096-point propagation, and C = 16 (a non-portable cluster
// size) doubles them again for the longest marches of a ragged batch.  The transforms:
//   time domain:       CTA c, thread j  <->  point n = c + C t(j),  t(j) = g + G l
//   frequency domain:  CTA c, thread j  <->  bin   k = j + M c
// with l = j mod 32 (lane), g = j / 32 (warp) and G = M / 32 warps: the time ownership strides the
// CTA's points over the lanes so that each warp's 32 points are one decimated sub-sequence.
// forward:  the M-point DFT over the CTA's strided points as 32 x G: a 32-point DFT inside each warp
//           (lanes exchange through shuffles: no shared memory, no barrier), the twiddle W_M^(g l),
//           then a G-point DFT across the warps (radix-2 Stockham through shared memory, one barrier
//           per stage: log2 G of them); then the twiddle exp(-2 pi i c j / N) and the C-point DFT
//           over the CTAs: every thread pushes its value to all C CTAs through distributed shared
//           memory, one cluster barrier, and each thread combines the C values of its own column for
//           its CTA's output row;
// inverse:  the C-point inverse DFT over the CTAs first, the conjugate twiddle, then the local inverse
//           (the G-point DFT across warps, the conjugate W_M^(g l), the 32-point DFT in the warps;
//           unscaled, 1/N is in the tables).
// A transform of M = 128 points thus has two CTA barriers where a Stockham pass per radix-2 stage had
// seven.  Each output costs 4 FP64 instructions per radix-2 stage in both parts (the warp stage writes
// a +- W b for both lanes of a pair as A + (+-W) B, the sign and operand order chosen per lane).
// Shared memory: M twiddles, two M-point exchange buffers (alternating, one barrier per stage: a thread
// writes a buffer only after the barrier that every reader of that buffer's previous contents has
// passed), and two halves of C x M cluster receive buffers (alternating per transform: a CTA writes a
// half only after the cluster barrier that its readers passed after their last read of it).
// M is a power of two of at least 32.
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
  int l, g, t;          // lane, warp and local time index g + (M / 32) l of this thread
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
  f.l = f.j & 31;
  f.g = f.j >> 5;
  f.t = f.g + (M >> 5) * f.l;
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

// Local time index of thread j of a CTA of M threads (the time ownership above).
__device__ __forceinline__ int spread_time_index(int j, int M) { return (j >> 5) + (M >> 5) * (j & 31); }

__device__ __forceinline__ double2 spread_shfl(double2 v, int src) {
  return make_double2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}
__device__ __forceinline__ double2 spread_shfl_xor(double2 v, int s) {
  return make_double2(__shfl_xor_sync(0xffffffffu, v.x, s), __shfl_xor_sync(0xffffffffu, v.y, s));
}
// v or -v through the sign bit (integer operations, no FP64 instruction)
__device__ __forceinline__ double spread_neg_if(double v, bool neg) {
  return __hiloint2double(__double2hiint(v) ^ (neg ? (int)0x80000000 : 0), __double2loint(v));
}

// 32-point DFT over the lanes of a warp: lane l holds element l on entry and bin l on return.  Each
// lane first takes the element of its bit-reversed lane; then five radix-2 decimation-in-time stages
// (s = 1 .. 16) pair lane l with l ^ s: the lower lane computes a + W b, the upper a - W b, both as
// A + (+-W) B with W = W_2s^(l mod s) (conjugated for the inverse) from the M-point table.
// Stage s = 1 (W = 1): own + partner below, partner - own above.  Stage s = 2 (W = 1 or W_4 = -i, +i
// for the inverse): the product W B is a swap of B's components with a sign, so both stages cost 2
// FP64 instructions per output.
template <bool INV>
__device__ __forceinline__ double2 spread_warp_stage(double2 x, const double2* __restrict__ twM, int M, int l, int s) {
  const double2 p = spread_shfl_xor(x, s);
  const bool up = (l & s) != 0;
  if (s == 1) {
    const double sg = up ? -1.0 : 1.0;
    return make_double2(fma(sg, x.x, p.x), fma(sg, x.y, p.y));
  }
  const double2 a = up ? p : x, b = up ? x : p;
  if (s == 2) {
    // W B with W = (-i)^(l & 1) (forward) or i^(l & 1) (inverse), then +- by the lane's position
    const bool rot = (l & 1) != 0;
    const double bx = rot ? spread_neg_if(b.y, INV) : b.x, by = rot ? spread_neg_if(b.x, !INV) : b.y;
    const double sg = up ? -1.0 : 1.0;
    return make_double2(fma(sg, bx, a.x), fma(sg, by, a.y));
  }
  const double2 w = twM[(l & (s - 1)) * (M / (2 * s))];
  const double wx = spread_neg_if(w.x, up), wy = spread_neg_if(w.y, up != INV);
  return make_double2(fma(-wy, b.y, fma(wx, b.x, a.x)), fma(wy, b.x, fma(wx, b.y, a.y)));
}

template <bool INV>
__device__ __forceinline__ double2 spread_warp_dft(const SpreadFFT& f, double2 x) {
  const int l = f.l, M = f.M;
  x = spread_shfl(x, (int)(__brev((unsigned)l) >> 27));
#pragma unroll
  for (int s = 1; s < 32; s <<= 1) x = spread_warp_stage<INV>(x, f.twM, M, l, s);
  return x;
}

// One output e + W_2L^kp o of a Stockham stage across the warps; W_2 = -1 and W_4 = -i (i for the
// inverse) as component swaps and signs (2 FP64 instructions), 4 otherwise.
template <bool INV>
__device__ __forceinline__ double2 spread_cross_stage(double2 e, double2 o, const double2* __restrict__ twM, int M, int kp,
                                                      int L) {
  if (L <= 2) {
    // W = (-i)^q, q = kp (L = 2) or 2 kp (L = 1): 1, -i, -1, i (conjugates for the inverse)
    const int q = (L == 1 ? 2 * kp : kp) & 3;
    const bool swap = (q & 1) != 0;
    const double ox = swap ? o.y : o.x, oy = swap ? o.x : o.y;
    // the real and imaginary signs of W o: q = 0 (+,+), 1 (+,-), 2 (-,-), 3 (-,+); inverse: 1 and 3 swap
    const int qq = INV ? (4 - q) & 3 : q;
    const double sx = (qq == 2 || qq == 3) ? -1.0 : 1.0, sy = (qq == 1 || qq == 2) ? -1.0 : 1.0;
    return make_double2(fma(sx, ox, e.x), fma(sy, oy, e.y));
  }
  const double2 w = twM[kp * (M / (2 * L))];
  const double wy = INV ? -w.y : w.y;
  return make_double2(fma(-wy, o.y, fma(w.x, o.x, e.x)), fma(wy, o.x, fma(w.x, o.y, e.y)));
}

// G-point DFT across the warps (G = M / 32) for every lane: thread (g, l) holds element g of its lane's
// sequence on entry and bin g on return.  Radix-2 Stockham stages L -> 2L through shared memory:
// y'[k' + 2L p] = y[k + L p] + W_2L^k' y[k + L p + G/2], k = k' mod L, element e of lane l at e 32 + l.
template <bool INV>
__device__ __forceinline__ double2 spread_cross_warp(SpreadFFT& f, double2 x) {
  const int M = f.M, G = M >> 5, g = f.g, l = f.l, half = G >> 1;
  for (int L = 1, shift = 0; L < G; L <<= 1, shift++) {
    double2* b = f.buf + f.sel * M;
    b[f.j] = x;
    __syncthreads();
    const int kp = g & (2 * L - 1);
    const int src = (kp & (L - 1)) + L * (g >> (shift + 1));
    const double2 e = b[src * 32 + l], o = b[(src + half) * 32 + l];
    x = spread_cross_stage<INV>(e, o, f.twM, M, kp, L);
    f.sel ^= 1;
  }
  return x;
}

// M-point DFT over the CTA's threads: thread j holds element t(j) on entry and bin j on return
// (forward); the inverse maps bins back to elements (unscaled).
template <bool INV>
__device__ __forceinline__ double2 spread_local(SpreadFFT& f, double2 x) {
  const double2 w = f.twM[f.g * f.l];   // W_M^(g l); 1 in warp 0 (a warp-uniform branch skips it)
  if (!INV) {
    x = spread_warp_dft<false>(f, x);
    if (f.g > 0) x = cmul(x, w);
    return spread_cross_warp<false>(f, x);
  }
  x = spread_cross_warp<true>(f, x);
  if (f.g > 0) x = cmulc(x, w);
  return spread_warp_dft<true>(f, x);
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
__device__ __forceinline__ void spread_warp_dft_k(const SpreadFFT& f, double2 (&x)[K]) {
  const int l = f.l, M = f.M;
  const int src = (int)(__brev((unsigned)l) >> 27);
#pragma unroll
  for (int m = 0; m < K; m++) x[m] = spread_shfl(x[m], src);
#pragma unroll
  for (int s = 1; s < 32; s <<= 1)
#pragma unroll
    for (int m = 0; m < K; m++) x[m] = spread_warp_stage<INV>(x[m], f.twM, M, l, s);
}

template <bool INV, int K>
__device__ __forceinline__ void spread_cross_warp_k(SpreadFFT& f, double2 (&x)[K]) {
  const int M = f.M, G = M >> 5, g = f.g, l = f.l, half = G >> 1;
  for (int L = 1, shift = 0; L < G; L <<= 1, shift++) {
    double2* b = f.buf + f.sel * K * M;
#pragma unroll
    for (int m = 0; m < K; m++) b[m * M + f.j] = x[m];
    __syncthreads();
    const int kp = g & (2 * L - 1);
    const int src = (kp & (L - 1)) + L * (g >> (shift + 1));
#pragma unroll
    for (int m = 0; m < K; m++)
      x[m] = spread_cross_stage<INV>(b[m * M + src * 32 + l], b[m * M + (src + half) * 32 + l], f.twM, M, kp, L);
    f.sel ^= 1;
  }
}

template <bool INV, int K>
__device__ __forceinline__ void spread_local_k(SpreadFFT& f, double2 (&x)[K]) {
  const double2 w = f.twM[f.g * f.l];
  if (!INV) {
    spread_warp_dft_k<false, K>(f, x);
    if (f.g > 0)
#pragma unroll
      for (int m = 0; m < K; m++) x[m] = cmul(x[m], w);
    spread_cross_warp_k<false, K>(f, x);
    return;
  }
  spread_cross_warp_k<true, K>(f, x);
  if (f.g > 0)
#pragma unroll
    for (int m = 0; m < K; m++) x[m] = cmulc(x[m], w);
  spread_warp_dft_k<true, K>(f, x);
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
