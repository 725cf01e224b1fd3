// nlm_ff.cuh -- double-float ("float-float") complex arithmetic and its Stockham FFT.
//
// GB300 executes FP32 FMAs at 61x the FP64 rate (73 vs 1.2 TFLOP/s measured on this part).  A value
// held as an unevaluated sum hi + lo of two floats carries 48 significant bits; sums and products
// are formed with the error-free transformations TwoSum (Knuth) and TwoProduct by FMA
// (Dekker/Kahan), then renormalised (the "double-double" algorithms of Dekker 1971, Hida, Li and
// Bailey 2001, here in single precision).  Each operation has a relative error of a few 2^-48 with
// respect to the magnitudes of its operands, i.e. ~1e-14: far inside the 1e-9 tolerance of the
// propagation after thousands of steps.  The range is FP32's (1e-38 .. 3e38).
//
// Memory layout of a complex value: float4 {re.hi, re.lo, im.hi, im.lo} (16 bytes, like double2).
#pragma once
#include <cuda_runtime.h>

#include "nlm_kernels.h"

namespace nlm {

struct ff {
  float hi, lo;
};
struct ffc {
  ff re, im;
};

__device__ __forceinline__ ff ff_make(float hi, float lo) { return ff{hi, lo}; }

// All float operations below use the _rn intrinsics, which the compiler never contracts into FMAs:
// the error-free transformations depend on each rounding happening exactly as written.

// hi + lo with |lo| <= ulp(hi)/2 from s = fl(a + b) and a small error term e (Fast2Sum)
__device__ __forceinline__ ff ff_renorm(float s, float e) {
  const float hi = __fadd_rn(s, e);
  return ff{hi, __fsub_rn(e, __fsub_rn(hi, s))};
}

// a + b: error-free sum of the high parts (TwoSum), low parts and the rounding error added into
// the low part, without renormalisation.  The result's low part may reach a few ulp of its high
// part after chained additions; every multiplication below renormalises, and the FFT passes
// renormalise their outputs, so chains stay a few additions long.  Errors stay ~2^-47 of the
// operands' magnitudes (what the FFT's norm-wise error bound needs).
__device__ __forceinline__ ff ff_add(ff a, ff b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bb = __fsub_rn(s, a.hi);
  float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  return ff{s, e};
}
__device__ __forceinline__ ff ff_norm(ff a) { return ff_renorm(a.hi, a.lo); }
__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.hi, -a.lo}; }
__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }

// a * b (TwoProduct by FMA)
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return ff_renorm(p, e);
}

// a * b + c * d with one renormalisation
__device__ __forceinline__ ff ff_dot2(ff a, ff b, ff c, ff d) {
  const float p1 = __fmul_rn(a.hi, b.hi), p2 = __fmul_rn(c.hi, d.hi);
  const float e1 = __fmaf_rn(a.hi, b.hi, -p1), e2 = __fmaf_rn(c.hi, d.hi, -p2);
  const float s = __fadd_rn(p1, p2);
  const float bb = __fsub_rn(s, p1);
  float e = __fadd_rn(__fsub_rn(p1, __fsub_rn(s, bb)), __fsub_rn(p2, bb));
  e = __fadd_rn(e, __fadd_rn(e1, e2));
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  e = __fmaf_rn(c.hi, d.lo, e);
  e = __fmaf_rn(c.lo, d.hi, e);
  return ff_renorm(s, e);
}

// e + s * u
__device__ __forceinline__ ff ff_axpy(ff e0, ff s0, ff u) {
  const float p = __fmul_rn(s0.hi, u.hi);
  const float ep = __fmaf_rn(s0.hi, u.hi, -p);
  const float s = __fadd_rn(p, e0.hi);
  const float bb = __fsub_rn(s, p);
  float e = __fadd_rn(__fsub_rn(p, __fsub_rn(s, bb)), __fsub_rn(e0.hi, bb));
  e = __fadd_rn(e, __fadd_rn(ep, e0.lo));
  e = __fmaf_rn(s0.hi, u.lo, e);
  e = __fmaf_rn(s0.lo, u.hi, e);
  return ff_renorm(s, e);
}

__device__ __forceinline__ ffc ffc_load(const float4* p) {
  const float4 v = *p;
  return ffc{ff{v.x, v.y}, ff{v.z, v.w}};
}
__device__ __forceinline__ ffc ffc_ldg(const float4* p) {
  const float4 v = __ldg(p);
  return ffc{ff{v.x, v.y}, ff{v.z, v.w}};
}
__device__ __forceinline__ void ffc_store(float4* p, ffc a) { *p = make_float4(a.re.hi, a.re.lo, a.im.hi, a.im.lo); }
__device__ __forceinline__ ffc ffc_zero() { return ffc{ff{0.f, 0.f}, ff{0.f, 0.f}}; }
__device__ __forceinline__ ffc ffc_from(double2 v) {
  const float rh = (float)v.x, ih = (float)v.y;
  return ffc{ff{rh, (float)(v.x - (double)rh)}, ff{ih, (float)(v.y - (double)ih)}};
}
__device__ __forceinline__ double2 ffc_to(ffc a) {
  return make_double2((double)a.re.hi + (double)a.re.lo, (double)a.im.hi + (double)a.im.lo);
}

__device__ __forceinline__ ffc fnorm(ffc a) { return ffc{ff_norm(a.re), ff_norm(a.im)}; }
__device__ __forceinline__ ffc fadd(ffc a, ffc b) { return ffc{ff_add(a.re, b.re), ff_add(a.im, b.im)}; }
__device__ __forceinline__ ffc fsub(ffc a, ffc b) { return ffc{ff_sub(a.re, b.re), ff_sub(a.im, b.im)}; }
// a * b
__device__ __forceinline__ ffc fmul(ffc a, ffc b) {
  return ffc{ff_dot2(a.re, b.re, ff_neg(a.im), b.im), ff_dot2(a.re, b.im, a.im, b.re)};
}
// a * conj(b)
__device__ __forceinline__ ffc fmulc(ffc a, ffc b) {
  return ffc{ff_dot2(a.re, b.re, a.im, b.im), ff_dot2(a.im, b.re, ff_neg(a.re), b.im)};
}

// ---------------------------------------------------------------------------------------------
// small DFTs (same structure and sign conventions as the FP64 ones in nlm_device.cuh)
// ---------------------------------------------------------------------------------------------
template <bool INV>
__device__ __forceinline__ void fdft2(ffc& a0, ffc& a1) {
  const ffc t = a0;
  a0 = fadd(t, a1);
  a1 = fsub(t, a1);
}

template <bool INV>
__device__ __forceinline__ void fdft4(ffc& a0, ffc& a1, ffc& a2, ffc& a3) {
  const ffc t0 = fadd(a0, a2), t1 = fsub(a0, a2), t2 = fadd(a1, a3), t3 = fsub(a1, a3);
  a0 = fadd(t0, t2);
  a2 = fsub(t0, t2);
  if (!INV) {  // y1 = t1 - i t3, y3 = t1 + i t3
    a1 = ffc{ff_add(t1.re, t3.im), ff_sub(t1.im, t3.re)};
    a3 = ffc{ff_sub(t1.re, t3.im), ff_add(t1.im, t3.re)};
  } else {
    a1 = ffc{ff_sub(t1.re, t3.im), ff_add(t1.im, t3.re)};
    a3 = ffc{ff_add(t1.re, t3.im), ff_sub(t1.im, t3.re)};
  }
}

template <bool INV>
__device__ __forceinline__ void fdft8(ffc& x0, ffc& x1, ffc& x2, ffc& x3, ffc& x4, ffc& x5, ffc& x6, ffc& x7) {
  // 1/sqrt(2) = hi + lo
  const ff s = ff{0.70710676908493041992f, 1.2101617485882343e-08f};
  ffc e0 = x0, e1 = x2, e2 = x4, e3 = x6;
  ffc o0 = x1, o1 = x3, o2 = x5, o3 = x7;
  fdft4<INV>(e0, e1, e2, e3);
  fdft4<INV>(o0, o1, o2, o3);
  x0 = fadd(e0, o0);
  x4 = fsub(e0, o0);
  const ffc w2 = INV ? ffc{ff_neg(o2.im), o2.re} : ffc{o2.im, ff_neg(o2.re)};
  x2 = fadd(e2, w2);
  x6 = fsub(e2, w2);
  const ff u1 = INV ? ff_sub(o1.re, o1.im) : ff_add(o1.re, o1.im);
  const ff v1 = INV ? ff_add(o1.re, o1.im) : ff_sub(o1.im, o1.re);
  x1 = ffc{ff_axpy(e1.re, s, u1), ff_axpy(e1.im, s, v1)};
  x5 = ffc{ff_axpy(e1.re, s, ff_neg(u1)), ff_axpy(e1.im, s, ff_neg(v1))};
  const ff u3 = INV ? ff_neg(ff_add(o3.re, o3.im)) : ff_sub(o3.im, o3.re);
  const ff v3 = INV ? ff_sub(o3.re, o3.im) : ff_neg(ff_add(o3.re, o3.im));
  x3 = ffc{ff_axpy(e3.re, s, u3), ff_axpy(e3.im, s, v3)};
  x7 = ffc{ff_axpy(e3.re, s, ff_neg(u3)), ff_axpy(e3.im, s, ff_neg(v3))};
}

template <int r, bool INV, int R>
__device__ __forceinline__ void fdft_r(ffc (&x)[R], int u, int B) {
  if constexpr (r == 2) {
    fdft2<INV>(x[u], x[u + B]);
  } else if constexpr (r == 4) {
    fdft4<INV>(x[u], x[u + B], x[u + 2 * B], x[u + 3 * B]);
  } else {
    fdft8<INV>(x[u], x[u + B], x[u + 2 * B], x[u + 3 * B], x[u + 4 * B], x[u + 5 * B], x[u + 6 * B], x[u + 7 * B]);
  }
}

// Stockham pass on float-float values: same index map and barrier protocol as nlm_device.cuh.
template <int R, int r, bool INV>
__device__ __forceinline__ void fstockham_pass(ffc (&x)[R], float4* __restrict__ buf, const float4* __restrict__ tw,
                                               int N, int T, int j, int L, bool from_smem, bool to_smem) {
  constexpr int B = R / r;
  if (from_smem) {
    __syncthreads();
#pragma unroll
    for (int v = 0; v < R; v++) x[v] = ffc_load(buf + j + v * T);
  }
  if (L > 1) {
    const int stride = N / (L * r);
#pragma unroll
    for (int u = 0; u < B; u++) {
      const int k = (j + u * T) & (L - 1);
#pragma unroll
      for (int q = 1; q < r; q++) {
        const ffc w = ffc_load(tw + k * q * stride);
        x[u + q * B] = INV ? fmulc(x[u + q * B], w) : fmul(x[u + q * B], w);
      }
    }
  }
#pragma unroll
  for (int u = 0; u < B; u++) fdft_r<r, INV>(x, u, B);
#pragma unroll
  for (int v = 0; v < R; v++) x[v] = fnorm(x[v]);
  if (to_smem) {
    __syncthreads();
#pragma unroll
    for (int u = 0; u < B; u++) {
      const int jp = j + u * T;
      const int k = jp & (L - 1);
      const int base = (jp - k) * r + k;
#pragma unroll
      for (int s2 = 0; s2 < r; s2++) ffc_store(buf + base + s2 * L, x[u + s2 * B]);
    }
  }
}

// Transform with the plan of make_plan: radix-8 passes with one pass of radix SMALL (2 or 4; 1 =
// none) in position 1 (position 0 when it is the only pass).  SMALL is a template parameter so that
// each call site holds two pass bodies only.
template <int R, int SMALL, bool INV>
__device__ __forceinline__ void ffft_regs(ffc (&x)[R], float4* __restrict__ buf, const float4* __restrict__ tw,
                                          const FFTPlanH& plan, int j) {
  int L = 1;
  const int smallAt = plan.nPass > 1 ? 1 : 0;
  for (int p = 0; p < plan.nPass; p++) {
    const bool from = p > 0, to = p < plan.nPass - 1;
    if constexpr (SMALL > 1) {
      if (p == smallAt) {
        fstockham_pass<R, SMALL, INV>(x, buf, tw, plan.N, plan.T, j, L, from, to);
        L *= SMALL;
        continue;
      }
    }
    fstockham_pass<R, 8, INV>(x, buf, tw, plan.N, plan.T, j, L, from, to);
    L *= 8;
  }
}

}  // namespace nlm
