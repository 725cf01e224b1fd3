// nlm_device.cuh -- FP64 complex arithmetic and the register-resident Stockham FFT.
//
// Layout contract used by every propagation kernel: an N-point field is held by T = N/R
// threads, thread j owning the R points j + v*T (v = 0..R-1) in registers.  A Stockham
// decimation-in-time pass of radix r reads X[j' + q*N/r] and writes
// Y[(j'-k)*r + k + s*L] (k = j' mod L), so its first pass reads exactly the register
// ownership above and its last pass writes it back: only the middle passes exchange
// data through one N-point shared-memory buffer.  Point-wise work (the RK4 step, the
// dispersion multiply) therefore never touches shared memory.
//
// The forward transform is unscaled and the inverse uses the conjugate twiddles without
// the 1/N factor; callers fold 1/N into their point-wise tables.  This is the convention
// of the reference's FFT adapter (src/CustomEigenFFT.h:91-101) once the scale is folded.
#pragma once
#include <cuda_runtime.h>
#include "nlm_kernels.h"

namespace nlm {

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
// a * b
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
__device__ __forceinline__ double2 cmulc(double2 a, double2 b) {
  return make_double2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
// a + s*b (s real)
__device__ __forceinline__ double2 caxpy(double2 a, double s, double2 b) {
  return make_double2(fma(s, b.x, a.x), fma(s, b.y, a.y));
}
__device__ __forceinline__ double cabs2(double2 a) { return a.x * a.x + a.y * a.y; }
__device__ __forceinline__ double2 csq(double2 a) { return make_double2(a.x * a.x - a.y * a.y, 2.0 * a.x * a.y); }
__device__ __forceinline__ double2 czero() { return make_double2(0.0, 0.0); }

// ------------------------------------------------------------------------------------------
// Small DFTs, in place on x[u + q*B] (q = 0..r-1), natural-order output.
// Forward kernel e^{-2 pi i qs/r}; INV selects e^{+2 pi i qs/r}.
// ------------------------------------------------------------------------------------------
template <bool INV>
__device__ __forceinline__ void dft2(double2& a0, double2& a1) {
  const double2 t = a0;
  a0 = cadd(t, a1);
  a1 = csub(t, a1);
}

template <bool INV>
__device__ __forceinline__ void dft4(double2& a0, double2& a1, double2& a2, double2& a3) {
  const double2 t0 = cadd(a0, a2), t1 = csub(a0, a2), t2 = cadd(a1, a3), t3 = csub(a1, a3);
  a0 = cadd(t0, t2);
  a2 = csub(t0, t2);
  if (!INV) {  // y1 = t1 - i t3, y3 = t1 + i t3
    a1 = make_double2(t1.x + t3.y, t1.y - t3.x);
    a3 = make_double2(t1.x - t3.y, t1.y + t3.x);
  } else {     // y1 = t1 + i t3, y3 = t1 - i t3
    a1 = make_double2(t1.x - t3.y, t1.y + t3.x);
    a3 = make_double2(t1.x + t3.y, t1.y - t3.x);
  }
}

template <bool INV>
__device__ __forceinline__ void dft8(double2& x0, double2& x1, double2& x2, double2& x3, double2& x4,
                                     double2& x5, double2& x6, double2& x7) {
  constexpr double s = 0.70710678118654752440084436210484903928483593768847;  // 1/sqrt(2)
  double2 e0 = x0, e1 = x2, e2 = x4, e3 = x6;
  double2 o0 = x1, o1 = x3, o2 = x5, o3 = x7;
  dft4<INV>(e0, e1, e2, e3);
  dft4<INV>(o0, o1, o2, o3);
  x0 = cadd(e0, o0);
  x4 = csub(e0, o0);
  // w^2 o2: forward -i o2, inverse +i o2
  const double2 w2 = INV ? make_double2(-o2.y, o2.x) : make_double2(o2.y, -o2.x);
  x2 = cadd(e2, w2);
  x6 = csub(e2, w2);
  // w^1 o1: forward (1-i)/sqrt2, inverse (1+i)/sqrt2
  const double u1 = INV ? (o1.x - o1.y) : (o1.x + o1.y);
  const double v1 = INV ? (o1.x + o1.y) : (o1.y - o1.x);
  x1 = make_double2(fma(u1, s, e1.x), fma(v1, s, e1.y));
  x5 = make_double2(fma(-u1, s, e1.x), fma(-v1, s, e1.y));
  // w^3 o3: forward (-1-i)/sqrt2, inverse (-1+i)/sqrt2
  const double u3 = INV ? -(o3.x + o3.y) : (o3.y - o3.x);
  const double v3 = INV ? (o3.x - o3.y) : -(o3.x + o3.y);
  x3 = make_double2(fma(u3, s, e3.x), fma(v3, s, e3.y));
  x7 = make_double2(fma(-u3, s, e3.x), fma(-v3, s, e3.y));
}

template <int r, bool INV, int R>
__device__ __forceinline__ void dft_r(double2 (&x)[R], int u, int B) {
  if constexpr (r == 2) {
    dft2<INV>(x[u], x[u + B]);
  } else if constexpr (r == 4) {
    dft4<INV>(x[u], x[u + B], x[u + 2 * B], x[u + 3 * B]);
  } else {
    dft8<INV>(x[u], x[u + B], x[u + 2 * B], x[u + 3 * B], x[u + 4 * B], x[u + 5 * B], x[u + 6 * B],
              x[u + 7 * B]);
  }
}

// Plan of a power-of-two transform: N = prod(radix[p]); T = N / R threads per field.
// (FFTPlanH in nlm_kernels.h is the same layout, filled on the host.)

// One Stockham pass.  Every shared-memory store is preceded by a barrier (all earlier
// loads of the buffer are complete) and every load is preceded by one (all stores are
// visible).  Barriers are CTA-wide and all branches here are uniform across the CTA.
template <int R, int r, bool INV, bool GUARD = false>
__device__ __forceinline__ void stockham_pass(double2 (&x)[R], double2* __restrict__ buf,
                                              const double2* __restrict__ tw, int N, int T, int j,
                                              int L, bool from_smem, bool to_smem, bool act = true) {
  // GUARD: threads with act == false (j >= T in a CTA sized for a larger grid) take part in the
  // barriers only and touch no memory.
  constexpr int B = R / r;
  if (from_smem) {
    __syncthreads();
    if (!GUARD || act) {
#pragma unroll
      for (int v = 0; v < R; v++) x[v] = buf[j + v * T];
    } else {
#pragma unroll
      for (int v = 0; v < R; v++) x[v] = czero();
    }
  }
  if (L > 1) {
    const int stride = N / (L * r);
#pragma unroll
    for (int u = 0; u < B; u++) {
      const int k = (j + u * T) & (L - 1);
#pragma unroll
      for (int q = 1; q < r; q++) {
        double2 w = czero();
        if (!GUARD || act) w = tw[k * q * stride];   // shared or global table (the caller's choice)
        x[u + q * B] = INV ? cmulc(x[u + q * B], w) : cmul(x[u + q * B], w);
      }
    }
  }
#pragma unroll
  for (int u = 0; u < B; u++) dft_r<r, INV>(x, u, B);
  if (to_smem) {
    __syncthreads();
    if (!GUARD || act) {
#pragma unroll
      for (int u = 0; u < B; u++) {
        const int jp = j + u * T;
        const int k = jp & (L - 1);
        const int base = (jp - k) * r + k;
#pragma unroll
        for (int s2 = 0; s2 < r; s2++) buf[base + s2 * L] = x[u + s2 * B];
      }
    }
  }
}

// Full transform of the R register points of thread j (ownership j + v*T in and out).
template <int R, bool INV, bool GUARD = false>
__device__ __forceinline__ void fft_regs(double2 (&x)[R], double2* __restrict__ buf,
                                         const double2* __restrict__ tw, const FFTPlanH& plan, int j,
                                         bool act = true) {
  int L = 1;
  for (int p = 0; p < plan.nPass; p++) {
    const bool from = p > 0, to = p < plan.nPass - 1;
    const int r = plan.radix[p];
    if constexpr (R >= 8) {
      if (r == 8) {
        stockham_pass<R, 8, INV, GUARD>(x, buf, tw, plan.N, plan.T, j, L, from, to, act);
        L *= 8;
        continue;
      }
    }
    if (r == 4) {
      stockham_pass<R, 4, INV, GUARD>(x, buf, tw, plan.N, plan.T, j, L, from, to, act);
      L *= 4;
    } else {
      stockham_pass<R, 2, INV, GUARD>(x, buf, tw, plan.N, plan.T, j, L, from, to, act);
      L *= 2;
    }
  }
}

// ------------------------------------------------------------------------------------------
// General transform (plan.gen == 1): any N, thread j owning the points j + v*T that are below N,
// T = ceil(N/R).  The owned points go to the shared-memory buffer, every pass reads its inputs from
// there and writes its outputs back, and the result comes back to the same ownership (points past N
// read as zero).  Pass of radix r with L = product of the earlier radices and stride = N/(L r),
// butterfly b < N/r, k = b mod L:
//     y_s = sum_q x[b + q N/r] w_N^{q (k stride + s N/r)},   written to [(b - k) r + k + s L]
// (the Stockham pass of the power-of-two kernels above, with any radix).  Radices 2, 4 and 8 run as
// butterflies (each thread holds the outputs of at most ceil(R/r) of them until the barrier); every
// other radix computes each output as its r-term sum, so a thread holds R outputs (one per owned
// index, read as the pair (b, s)).  This path serves the grids that are not powers of two; its
// barriers are CTA-wide in uniform control flow like those of stockham_pass.
// ------------------------------------------------------------------------------------------
template <int R, int r, bool INV>
__device__ __forceinline__ void gen_pass_pow2(double2* __restrict__ buf, const double2* __restrict__ tw, int N, int T,
                                              int j, int L) {
  constexpr int U = (R + r - 1) / r;   // butterflies per thread: N/r / ceil(N/R) <= R/r
  const int nb = N / r, stride = N / (L * r);
  double2 y[U][r];
#pragma unroll
  for (int u = 0; u < U; u++) {
    const int b = j + u * T;
    if (b < nb) {
      const int k = b % L;
      double2 a[r];
#pragma unroll
      for (int q = 0; q < r; q++) {
        a[q] = buf[b + q * nb];
        if (q > 0 && L > 1) {
          const double2 w = tw[k * q * stride];
          a[q] = INV ? cmulc(a[q], w) : cmul(a[q], w);
        }
      }
      if constexpr (r == 2) dft2<INV>(a[0], a[1]);
      else if constexpr (r == 4) dft4<INV>(a[0], a[1], a[2], a[3]);
      else dft8<INV>(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7]);
#pragma unroll
      for (int s = 0; s < r; s++) y[u][s] = a[s];
    }
  }
  __syncthreads();
#pragma unroll
  for (int u = 0; u < U; u++) {
    const int b = j + u * T;
    if (b < nb) {
      const int k = b % L;
      const int base = (b - k) * r + k;
#pragma unroll
      for (int s = 0; s < r; s++) buf[base + s * L] = y[u][s];
    }
  }
}

template <int R, bool INV>
__device__ __forceinline__ void gen_pass_any(double2* __restrict__ buf, const double2* __restrict__ tw, int N, int T,
                                             int j, int L, int r) {
  const int nb = N / r, stride = N / (L * r);
  double2 y[R];
#pragma unroll
  for (int v = 0; v < R; v++) {
    const int o = j + v * T;
    y[v] = czero();
    if (o < N) {
      const int b = o % nb, s = o / nb, k = b % L;
      const int step = (k * stride + s * nb) % N;
      int e = 0;
      double2 acc = czero();
      for (int q = 0; q < r; q++) {
        const double2 w = tw[e];
        const double2 xq = buf[b + q * nb];
        acc = INV ? cadd(acc, cmulc(xq, w)) : cadd(acc, cmul(xq, w));
        e += step;
        if (e >= N) e -= N;
      }
      y[v] = acc;
    }
  }
  __syncthreads();
#pragma unroll
  for (int v = 0; v < R; v++) {
    const int o = j + v * T;
    if (o < N) {
      const int b = o % nb, s = o / nb, k = b % L;
      buf[(b - k) * r + k + s * L] = y[v];
    }
  }
}

// The passes of the general plan, on the buffer alone: one out-of-line copy per (R, direction), so that
// a kernel with many transforms carries a call at each of them rather than the passes inlined.  The
// plan comes by value (its radices); every pass starts with a barrier and ends with its writes.
template <int R, bool INV>
__device__ __noinline__ void fft_general_passes(double2* __restrict__ buf, const double2* __restrict__ tw,
                                                const FFTPlanH plan, int j) {
  const int N = plan.N, T = plan.T;
  int L = 1;
  for (int p = 0; p < plan.nPass; p++) {
    const int r = plan.radix[p];
    __syncthreads();   // the previous pass's outputs (or the caller's scatter) are visible
    if (r == 8) gen_pass_pow2<R, 8, INV>(buf, tw, N, T, j, L);
    else if (r == 4) gen_pass_pow2<R, 4, INV>(buf, tw, N, T, j, L);
    else if (r == 2) gen_pass_pow2<R, 2, INV>(buf, tw, N, T, j, L);
    else gen_pass_any<R, INV>(buf, tw, N, T, j, L, r);
    L *= r;
  }
}

template <int R, bool INV>
__device__ __forceinline__ void fft_general(double2 (&x)[R], double2* __restrict__ buf, const double2* __restrict__ tw,
                                            const FFTPlanH& plan, int j) {
  const int N = plan.N, T = plan.T;
  __syncthreads();   // earlier readers of the buffer are done
#pragma unroll
  for (int v = 0; v < R; v++) {
    const int t = j + v * T;
    if (t < N) buf[t] = x[v];
  }
  fft_general_passes<R, INV>(buf, tw, plan, j);
  __syncthreads();
#pragma unroll
  for (int v = 0; v < R; v++) {
    const int t = j + v * T;
    x[v] = t < N ? buf[t] : czero();
  }
}

// The transform of the kernels that take both plans: GEN instantiations serve plan.gen == 1.
template <int R, bool INV, bool GEN>
__device__ __forceinline__ void fft_any(double2 (&x)[R], double2* __restrict__ buf, const double2* __restrict__ tw,
                                        const FFTPlanH& plan, int j) {
  if constexpr (GEN) fft_general<R, INV>(x, buf, tw, plan, j);
  else fft_regs<R, INV>(x, buf, tw, plan, j);
}

// exp(re + i im), the self-phase factor of one pump row.  im is the nonlinear phase of half a z step,
// small in practice: for |im| <= 1/4 sine and cosine come from their Taylor series (terms to x^13 and
// x^14; the first omitted term is below 1e-21 of the result), otherwise from sincos.  re is zero
// for a real nonlinear length, and exp(0) = 1 exactly.
__device__ __forceinline__ double2 spm_factor(double re, double im) {
  double sn, cs;
  if (fabs(im) <= 0.25) {
    const double x2 = im * im;
    sn = 1.0 / 6227020800.0;                      // 1/13!
    sn = fma(sn, -x2, 1.0 / 39916800.0);          // 1/11!
    sn = fma(sn, -x2, 1.0 / 362880.0);            // 1/9!
    sn = fma(sn, -x2, 1.0 / 5040.0);              // 1/7!
    sn = fma(sn, -x2, 1.0 / 120.0);               // 1/5!
    sn = fma(sn, -x2, 1.0 / 6.0);                 // 1/3!
    sn = fma(sn, -x2, 1.0);
    sn *= im;
    cs = 1.0 / 87178291200.0;                     // 1/14!
    cs = fma(cs, -x2, 1.0 / 479001600.0);         // 1/12!
    cs = fma(cs, -x2, 1.0 / 3628800.0);           // 1/10!
    cs = fma(cs, -x2, 1.0 / 40320.0);             // 1/8!
    cs = fma(cs, -x2, 1.0 / 720.0);               // 1/6!
    cs = fma(cs, -x2, 1.0 / 24.0);                // 1/4!
    cs = fma(cs, -x2, 0.5);                       // 1/2!
    cs = fma(cs, -x2, 1.0);
  } else {
    sincos(im, &sn, &cs);
  }
  const double e = re == 0.0 ? 1.0 : exp(re);
  return make_double2(e * cs, e * sn);
}

}  // namespace nlm
