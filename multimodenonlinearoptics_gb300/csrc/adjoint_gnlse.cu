// adjoint_gnlse.cu -- reverse sweep of the Chi3GNLSE split-step propagation (solvers/Chi3GNLSE.cpp:39-92).
//
// Each RK4 stage of the generalised NLSE is
//     u1 = r |y|^2,  u2 = F^H(R' F u1),  k = F^H(St' F(u2 y)),   y_s = x + fac_s k_{s-1}
// (R' = Raman response / N, St' = (g0 + g1 w) / N, F unscaled).  Its adjoint with g = dL/dRe + i dL/dIm:
//     g_u3 = F^H(conj(St') F g_k),  g_y += conj(u2) g_u3,  g_u2 = conj(y) g_u3,
//     g_u1 = Re F^H(conj(R') F g_u2),  g_y += 2 r g_u1 y,  g_x += g_y,  g_k_{s-1} += fac_s g_y.
// For every step the stage inputs y_s and convolutions u2_s are recomputed from the state before the
// step (14 transforms: the last stage's self-steepening pair is not needed), then the 16 transforms
// of the reverse step run (gnlse_reverse_step: the gradient stays in the frequency domain).  States come from checkpoints every K steps;
// segments between checkpoints are recomputed.
// With K > 1 the segment's recomputation stores the stage values of its steps, which its reverse
// steps then read.  Scratch per propagation slot: Y[4][N], U2[4][N], GX[N], GXP[N], and for K > 1 the
// state being recomputed and STG[K][8][N].
#include <vector>

#include <cooperative_groups.h>

#include "nlm_propagate.cuh"

namespace cg = cooperative_groups;

namespace nlm {

// Forward stages of step i from the state in `xs` (global, this thread's points): stores y_s and
// u2_s, and (when acc != nullptr) the stage sum k0 + 2 k1 + 2 k2 + k3 into acc.  Without acc the
// last stage's self-steepening pair is skipped (14 transforms instead of 16).
template <int R>
__device__ __forceinline__ void gnlse_stages(const PropArgs& a, int i, int j, double2* buf, const double2* tw,
                                             const double2* xs, double2* Y, double2* U2, double2* acc) {
  const FFTPlanH& plan = a.plan;
  const int N = plan.N, T = plan.T;
  const double* rel = a.relInt + (long long)(i - 1) * 3;
  double2 k[R];
#pragma unroll
  for (int v = 0; v < R; v++) k[v] = czero();
  for (int s = 0; s < 4; s++) {
    const double fac = s == 0 ? 0.0 : (s == 3 ? 1.0 : 0.5);
    const double wgt = (s == 1 || s == 2) ? 2.0 : 1.0;
    const double ri = __ldg(rel + (s == 0 ? 0 : (s == 3 ? 2 : 1)));
    double2 y[R], u[R];
#pragma unroll
    for (int v = 0; v < R; v++) {
      y[v] = caxpy(xs[j + v * T], fac, k[v]);
      Y[(long long)s * N + j + v * T] = y[v];
      u[v] = make_double2(ri * cabs2(y[v]), 0.0);
    }
    fft_regs<R, false>(u, buf, tw, plan, j);
#pragma unroll
    for (int v = 0; v < R; v++) u[v] = cmul(u[v], __ldg(a.raman + j + v * T));
    fft_regs<R, true>(u, buf, tw, plan, j);
#pragma unroll
    for (int v = 0; v < R; v++) {
      U2[(long long)s * N + j + v * T] = u[v];
      u[v] = cmul(u[v], y[v]);
    }
    if (!acc && s == 3) break;   // the last stage's k only enters the next state: not needed here
    fft_regs<R, false>(u, buf, tw, plan, j);
#pragma unroll
    for (int v = 0; v < R; v++) u[v] = cmul(u[v], __ldg(a.steep + j + v * T));
    fft_regs<R, true>(u, buf, tw, plan, j);
#pragma unroll
    for (int v = 0; v < R; v++) {
      k[v] = u[v];
      if (acc) {
        const int t = j + v * T;
        acc[t] = s == 0 ? u[v] : caxpy(acc[t], wgt, u[v]);
      }
    }
  }
}

// One reverse step i: gv (this thread's points of the gradient with respect to the spectrum after the
// step) becomes the gradient with respect to the spectrum before it.  Y/U2: the stage inputs y_s and
// convolutions u2_s of step i; GX/GXP: per-propagation global scratch of N points each.  The transpose
// of the forward's frequency-domain RK4 sum: with H = N conj(D) g (D the step's dispersion factors,
// which carry the 1/N of a transform pair), stage s's spectrum gets w_s H plus the transform of the
// gradient its time-domain value takes through the next stage's input, and the spectrum before the
// step H plus the transform of the stage inputs' gradient.  16 transforms per step where the
// time-domain form takes 18; in exact arithmetic the same gradient.
template <int R>
__device__ __forceinline__ void gnlse_reverse_step(const PropArgs& a, int i, int j, double2* buf, const double2* tw,
                                                   const double2* Y, const double2* U2, double2* GX, double2* GXP,
                                                   double2 (&gv)[R]) {
  const FFTPlanH& plan = a.plan;
  const int N = plan.N, T = plan.T;
  const double2* tab = (i == a.nZ - 1) ? a.dlast : a.dstep;
#pragma unroll
  for (int v = 0; v < R; v++) {
    GXP[j + v * T] = cscale(cmulc(gv[v], __ldg(tab + j + v * T)), (double)N);   // H
    GX[j + v * T] = czero();
  }
  const double* rel = a.relInt + (long long)(i - 1) * 3;
  double2 gke[R];
#pragma unroll
  for (int v = 0; v < R; v++) gke[v] = czero();
  for (int s = 3; s >= 0; s--) {
    const double w = (s == 1 || s == 2) ? 2.0 / 6.0 : 1.0 / 6.0;
    const double fac = s == 0 ? 0.0 : (s == 3 ? 1.0 : 0.5);
    const double ri = __ldg(rel + (s == 0 ? 0 : (s == 3 ? 2 : 1)));
    double2 u[R];
    if (s < 3) {
#pragma unroll
      for (int v = 0; v < R; v++) u[v] = gke[v];
      fft_regs<R, false>(u, buf, tw, plan, j);
#pragma unroll
      for (int v = 0; v < R; v++) u[v] = caxpy(u[v], w, GXP[j + v * T]);   // g_k_s (spectrum)
    } else {
#pragma unroll
      for (int v = 0; v < R; v++) u[v] = cscale(GXP[j + v * T], w);
    }
#pragma unroll
    for (int v = 0; v < R; v++) u[v] = cmulc(u[v], __ldg(a.steep + j + v * T));
    fft_regs<R, true>(u, buf, tw, plan, j);                                   // g_u3
    double2 gy[R];
#pragma unroll
    for (int v = 0; v < R; v++) {
      const int t = j + v * T;
      const double2 y = Y[(long long)s * N + t], u2 = U2[(long long)s * N + t];
      gy[v] = cmulc(u[v], u2);     // conj(u2) g_u3
      u[v] = cmulc(u[v], y);       // g_u2 = conj(y) g_u3
    }
    fft_regs<R, false>(u, buf, tw, plan, j);
#pragma unroll
    for (int v = 0; v < R; v++) u[v] = cmulc(u[v], __ldg(a.raman + j + v * T));
    fft_regs<R, true>(u, buf, tw, plan, j);                                   // g_u1 (real part)
#pragma unroll
    for (int v = 0; v < R; v++) {
      const int t = j + v * T;
      const double2 y = Y[(long long)s * N + t];
      gy[v] = caxpy(gy[v], 2.0 * ri * u[v].x, y);
      GX[t] = cadd(GX[t], gy[v]);
      gke[v] = cscale(gy[v], fac);
    }
  }
#pragma unroll
  for (int v = 0; v < R; v++) gv[v] = GX[j + v * T];
  fft_regs<R, false>(gv, buf, tw, plan, j);
#pragma unroll
  for (int v = 0; v < R; v++) gv[v] = cadd(gv[v], GXP[j + v * T]);
}

template <int R>
__global__ void __launch_bounds__(kMaxThreads) k_adjoint_gnlse(const PropArgs a, const AdjArgs d) {
  extern __shared__ double2 smem[];
  __shared__ long long s_group;
  const FFTPlanH& plan = a.plan;
  const int N = plan.N, T = plan.T;
  const int g = threadIdx.x / T, j = threadIdx.x - g * T;
  double2* bufs;
  const double2* tw = stage_twiddles<R>(a.tw, smem, N, &bufs);
  double2* buf = bufs + (long long)g * N;
  double2* slot = d.seg + ((long long)blockIdx.x * a.ipc + g) * (long long)(10 + (d.K > 1 ? 1 + 8 * d.K : 0)) * N;
  double2* Y = slot;
  double2* U2 = slot + 4LL * N;
  double2* GX = slot + 8LL * N;
  double2* GXP = slot + 9LL * N;
  double2* XS = slot + 10LL * N;    // K > 1: the state being recomputed
  double2* STG = slot + 11LL * N;   // K > 1: y_s, u2_s of the segment's step q at STG + q 8 N
  const long long nGroups = (a.nInst + a.ipc - 1) / a.ipc;
  for (long long cg = blockIdx.x; cg < nGroups; cg = next_group(a, cg, &s_group)) {
    const long long local = cg * a.ipc + g;
    const bool active = local < a.nInst;
    const long long inst = a.instBase + local;
    const double2* ck = d.ckpt + (active ? inst : 0) * (long long)d.nCk * N;
    double2 gv[R];
    {
      const double2* go = d.gout + (active ? inst : 0) * (long long)N;
#pragma unroll
      for (int v = 0; v < R; v++) gv[v] = active ? cscale(go[j + v * T], (double)N) : czero();
    }
    int segEnd = a.nZ - 1;
    while (segEnd >= 1) {
      const int jseg = (segEnd - 1) / d.K;
      const int s0 = jseg * d.K;
      if (d.K > 1) {
        // recompute the segment's steps from its checkpoint, storing each step's stage values, then
        // reverse them from the store (no second recomputation of the stages)
#pragma unroll
        for (int v = 0; v < R; v++) XS[j + v * T] = ck[(long long)jseg * N + j + v * T];
        for (int i = s0 + 1; i <= segEnd; i++) {
          double2* Yq = STG + (long long)(i - 1 - s0) * 8 * N;
          const bool more = i < segEnd;
          gnlse_stages<R>(a, i, j, buf, tw, XS, Yq, Yq + 4LL * N, more ? GX : nullptr);   // GX: stage sum
          if (more) {
            double2 x[R];
#pragma unroll
            for (int v = 0; v < R; v++) x[v] = caxpy(XS[j + v * T], 1.0 / 6.0, GX[j + v * T]);
            fft_regs<R, false>(x, buf, tw, plan, j);
#pragma unroll
            for (int v = 0; v < R; v++) x[v] = cmul(x[v], __ldg(a.dstep + j + v * T));
            fft_regs<R, true>(x, buf, tw, plan, j);
#pragma unroll
            for (int v = 0; v < R; v++) XS[j + v * T] = x[v];
          }
        }
        for (int i = segEnd; i > s0; i--) {
          const double2* Yq = STG + (long long)(i - 1 - s0) * 8 * N;
          gnlse_reverse_step<R>(a, i, j, buf, tw, Yq, Yq + 4LL * N, GX, GXP, gv);
        }
      } else {
        for (int i = segEnd; i > s0; i--) {
          gnlse_stages<R>(a, i, j, buf, tw, ck + (long long)(i - 1) * N, Y, U2, nullptr);
          gnlse_reverse_step<R>(a, i, j, buf, tw, Y, U2, GX, GXP, gv);
        }
      }
      segEnd = s0;
    }
    // gv: the gradient of the input spectrum; times half a dispersion step
    if (active) {
#pragma unroll
      for (int v = 0; v < R; v++)
        d.gin[inst * (long long)N + j + v * T] = cmulc(gv[v], __ldg(a.half + j + v * T));
    }
    __syncthreads();
  }
}

// Pipelined reverse sweep, launched as clusters of two CTAs, one propagation per cluster at a time.
// CTA 1 marches segment j-1 forward from its checkpoint and stores the stage inputs y_s and the
// convolutions u2_s of every step; CTA 0 runs the reverse steps of segment j from the stored stages.
// Both do about one forward step of work per step (18 transforms), so the stage recomputation that
// the one-CTA sweep adds to every reverse step runs on a second SM.  Scratch per cluster:
// STG[2][K][8][N] (double-buffered stages), XS[N], ACC[N] (CTA 1), GX[N], GXP[N] (CTA 0).  A cluster
// barrier separates the iterations; both CTAs execute nSeg + 1 barriers per propagation.
template <int R>
__global__ void __launch_bounds__(kMaxThreads) k_adjoint_gnlse_pipe(const PropArgs a, const AdjArgs d) {
  extern __shared__ double2 smem[];
  cg::cluster_group cluster = cg::this_cluster();
  const FFTPlanH& plan = a.plan;
  const int N = plan.N, T = plan.T;
  const int j = threadIdx.x;
  const int role = (int)cluster.block_rank();
  const long long clusterId = blockIdx.x / 2, nClusters = gridDim.x / 2;
  double2* buf;
  const double2* tw = stage_twiddles<R>(a.tw, smem, N, &buf);
  const long long stepStride = 8LL * N, bufStride = (long long)d.K * stepStride;
  double2* STG = d.seg + clusterId * (2 * bufStride + 4LL * N);
  double2* XS = STG + 2 * bufStride;
  double2* ACC = XS + N;
  double2* GX = ACC + N;
  double2* GXP = GX + N;
  const int nSeg = (a.nZ - 2) / d.K + 1;
  for (long long local = clusterId; local < a.nInst; local += nClusters) {
    const long long inst = a.instBase + local;
    const double2* ck = d.ckpt + inst * (long long)d.nCk * N;
    double2 gv[R];
    if (role == 0) {
      const double2* go = d.gout + inst * (long long)N;
#pragma unroll
      for (int v = 0; v < R; v++) gv[v] = cscale(go[j + v * T], (double)N);
    }
    for (int it = 0; it <= nSeg; it++) {
      if (role == 1 && it < nSeg) {
        const int jseg = nSeg - 1 - it, s0 = jseg * d.K, segEnd = min(s0 + d.K, a.nZ - 1);
        double2* stg = STG + (long long)(it & 1) * bufStride;
#pragma unroll
        for (int v = 0; v < R; v++) XS[j + v * T] = ck[(long long)jseg * N + j + v * T];
        for (int i = s0 + 1; i <= segEnd; i++) {
          double2* Yi = stg + (long long)(i - 1 - s0) * stepStride;
          const bool more = i < segEnd;   // the state after step i starts the next step of the segment
          gnlse_stages<R>(a, i, j, buf, tw, XS, Yi, Yi + 4LL * N, more ? ACC : nullptr);
          if (more) {
            double2 x[R];
#pragma unroll
            for (int v = 0; v < R; v++) x[v] = caxpy(XS[j + v * T], 1.0 / 6.0, ACC[j + v * T]);
            fft_regs<R, false>(x, buf, tw, plan, j);
#pragma unroll
            for (int v = 0; v < R; v++) x[v] = cmul(x[v], __ldg(a.dstep + j + v * T));
            fft_regs<R, true>(x, buf, tw, plan, j);
#pragma unroll
            for (int v = 0; v < R; v++) XS[j + v * T] = x[v];
          }
        }
      }
      if (role == 0 && it >= 1) {
        const int jseg = nSeg - it, s0 = jseg * d.K, segEnd = min(s0 + d.K, a.nZ - 1);
        const double2* stg = STG + (long long)((it - 1) & 1) * bufStride;
        for (int i = segEnd; i > s0; i--) {
          const double2* Yi = stg + (long long)(i - 1 - s0) * stepStride;
          gnlse_reverse_step<R>(a, i, j, buf, tw, Yi, Yi + 4LL * N, GX, GXP, gv);
        }
      }
      cluster.sync();
    }
    if (role == 0) {
#pragma unroll
      for (int v = 0; v < R; v++) d.gin[inst * (long long)N + j + v * T] = cmulc(gv[v], __ldg(a.half + j + v * T));
    }
    __syncthreads();
  }
}

// ---- two rows per thread group ---------------------------------------------------------------
// The Raman operator L(z) = IFFT[H FFT[z]] with H = R~ or conj(R~) (the transform of a real response,
// Hermitian) maps real fields to real fields.  The forward's Raman input rel |y|^2 is real, and the
// reverse step only uses Re L(g_u2) = L(Re g_u2): so two rows' Raman transforms run as one complex
// pair, L(a + i b) = L(a) + i L(b).  Per row and step: 10 transforms to recompute the stages (4
// shared Raman pairs, 3 self-steepening pairs) and 12 to reverse the step in the frequency domain
// (7 for the self-steepening adjoints, 4 shared Raman pairs, one for the state), against 14 + 18.
// With checkpoint intervals K > 1 the segment's forward recomputation (14 per row and step) stores
// the stage values of its K steps and the reverse steps read them: 14 + 12 instead of 14 + 10 + 12.  Per-row scratch (each
// thread touches only its own points): Y[4], U2[4] (real, stored as complex), K, GX, GXP, G, GY, GKE,
// ZR (real, stored as complex), ACC: 16 N; for K > 1 also the state being recomputed and the stage
// store STG[K][8]: (1 + 8 K) N.
namespace {

constexpr int kPairRowSlot = 16;   // per-row scratch values in units of N

struct PairRow {
  double2 *Y, *U2, *K, *GX, *GXP, *G, *GY, *GKE, *ZR, *ACC, *SEG;
};

__device__ __forceinline__ PairRow pair_row(double2* base, int N, int K) {
  PairRow r;
  r.Y = base;
  r.U2 = base + 4LL * N;
  r.K = base + 8LL * N;
  r.GX = base + 9LL * N;
  r.GXP = base + 10LL * N;
  r.G = base + 11LL * N;
  r.GY = base + 12LL * N;
  r.GKE = base + 13LL * N;
  r.ZR = base + 14LL * N;
  r.ACC = base + 15LL * N;
  // checkpoint intervals K > 1: the state being recomputed, then the stage values of the K steps of
  // the segment (y_s and u2_s of step q at SEG + N + q 8 N)
  r.SEG = K > 1 ? base + (long long)kPairRowSlot * N : nullptr;
  return r;
}

// Stages of step i for both rows from their states xs[0], xs[1]: stores y_s and the real u2_s; with
// acc, also k_3 and the stage sums into ACC (a forward step), else the last self-steepening pair is
// skipped.
template <int R>
__device__ __forceinline__ void pair_stages(const PropArgs& a, int i, int j, double2* buf, const double2* tw,
                                            const double2* xs0, const double2* xs1, PairRow (&row)[2], bool acc) {
  const FFTPlanH& plan = a.plan;
  const int N = plan.N, T = plan.T;
  const double* rel = a.relInt + (long long)(i - 1) * 3;
  for (int s = 0; s < 4; s++) {
    const double fac = s == 0 ? 0.0 : (s == 3 ? 1.0 : 0.5);
    const double wgt = (s == 1 || s == 2) ? 2.0 : 1.0;
    const double ri = __ldg(rel + (s == 0 ? 0 : (s == 3 ? 2 : 1)));
    double2 u[R];
#pragma unroll
    for (int v = 0; v < R; v++) {
      const int t = j + v * T;
      const double2 y0 = s == 0 ? xs0[t] : caxpy(xs0[t], fac, row[0].K[t]);
      const double2 y1 = s == 0 ? xs1[t] : caxpy(xs1[t], fac, row[1].K[t]);
      row[0].Y[(long long)s * N + t] = y0;
      row[1].Y[(long long)s * N + t] = y1;
      u[v] = make_double2(ri * cabs2(y0), ri * cabs2(y1));
    }
    fft_regs<R, false>(u, buf, tw, plan, j);
#pragma unroll
    for (int v = 0; v < R; v++) u[v] = cmul(u[v], __ldg(a.raman + j + v * T));
    fft_regs<R, true>(u, buf, tw, plan, j);
#pragma unroll
    for (int v = 0; v < R; v++) {
      row[0].U2[(long long)s * N + j + v * T] = make_double2(u[v].x, 0.0);
      row[1].U2[(long long)s * N + j + v * T] = make_double2(u[v].y, 0.0);
    }
    if (!acc && s == 3) break;
#pragma unroll 1
    for (int r = 0; r < 2; r++) {
      double2 w[R];
#pragma unroll
      for (int v = 0; v < R; v++) {
        const int t = j + v * T;
        const double c = row[r].U2[(long long)s * N + t].x;
        const double2 y = row[r].Y[(long long)s * N + t];
        w[v] = make_double2(c * y.x, c * y.y);
      }
      fft_regs<R, false>(w, buf, tw, plan, j);
#pragma unroll
      for (int v = 0; v < R; v++) w[v] = cmul(w[v], __ldg(a.steep + j + v * T));
      fft_regs<R, true>(w, buf, tw, plan, j);
#pragma unroll
      for (int v = 0; v < R; v++) {
        const int t = j + v * T;
        row[r].K[t] = w[v];
        if (acc) row[r].ACC[t] = s == 0 ? w[v] : caxpy(row[r].ACC[t], wgt, w[v]);
      }
    }
  }
}

// One reverse step i for both rows.  G holds the gradient with respect to the spectrum after the step
// (the transform of the time-domain gradient; for the last step the output spectrum's gradient) and
// becomes the one before it.  The step in the frequency domain: with H = N conj(D) G (D the step's
// dispersion factors, which carry the 1/N of a transform pair), the gradient of stage s's spectrum k_s
// is w_s H plus, for s < 3, the transform of the gradient its time-domain value gets through the next
// stage's input; the self-steepening and Raman adjoints follow in time; and the spectrum before the
// step gets H plus the transform of the time-domain gradient the stage inputs give the state.  Per
// row 12 transforms (the fourth stage needs only the inverse, and no pair brackets the dispersion
// step), where the time-domain form takes 14; in exact arithmetic the same gradient.
template <int R>
__device__ __forceinline__ void pair_reverse_step(const PropArgs& a, int i, int j, double2* buf, const double2* tw,
                                                  PairRow (&row)[2]) {
  const FFTPlanH& plan = a.plan;
  const int N = plan.N, T = plan.T;
  const double2* tab = (i == a.nZ - 1) ? a.dlast : a.dstep;
  // H (frequency domain) in GXP; the stage inputs' gradient sum (time domain) in GX
#pragma unroll 1
  for (int r = 0; r < 2; r++) {
#pragma unroll
    for (int v = 0; v < R; v++) {
      const int t = j + v * T;
      row[r].GXP[t] = cscale(cmulc(row[r].G[t], __ldg(tab + t)), (double)N);
      row[r].GX[t] = czero();
      row[r].GKE[t] = czero();
    }
  }
  const double* rel = a.relInt + (long long)(i - 1) * 3;
  for (int s = 3; s >= 0; s--) {
    const double w = (s == 1 || s == 2) ? 2.0 / 6.0 : 1.0 / 6.0;
    const double fac = s == 0 ? 0.0 : (s == 3 ? 1.0 : 0.5);
    const double ri = __ldg(rel + (s == 0 ? 0 : (s == 3 ? 2 : 1)));
#pragma unroll 1
    for (int r = 0; r < 2; r++) {
      double2 u[R];
      if (s < 3) {
#pragma unroll
        for (int v = 0; v < R; v++) u[v] = row[r].GKE[j + v * T];
        fft_regs<R, false>(u, buf, tw, plan, j);
#pragma unroll
        for (int v = 0; v < R; v++) u[v] = caxpy(u[v], w, row[r].GXP[j + v * T]);   // g_k_s (spectrum)
      } else {
#pragma unroll
        for (int v = 0; v < R; v++) u[v] = cscale(row[r].GXP[j + v * T], w);
      }
#pragma unroll
      for (int v = 0; v < R; v++) u[v] = cmulc(u[v], __ldg(a.steep + j + v * T));
      fft_regs<R, true>(u, buf, tw, plan, j);                                         // g_u3
#pragma unroll
      for (int v = 0; v < R; v++) {
        const int t = j + v * T;
        const double2 y = row[r].Y[(long long)s * N + t];
        const double u2 = row[r].U2[(long long)s * N + t].x;
        row[r].GY[t] = make_double2(u[v].x * u2, u[v].y * u2);   // conj(u2) g_u3, u2 real
        row[r].ZR[t] = make_double2(y.x * u[v].x + y.y * u[v].y, 0.0);   // Re(conj(y) g_u3)
      }
    }
    // both rows' Raman adjoints: Re L(conj(y) g_u3) = L(Re(conj(y) g_u3))
    double2 p[R];
#pragma unroll
    for (int v = 0; v < R; v++) p[v] = make_double2(row[0].ZR[j + v * T].x, row[1].ZR[j + v * T].x);
    fft_regs<R, false>(p, buf, tw, plan, j);
#pragma unroll
    for (int v = 0; v < R; v++) p[v] = cmulc(p[v], __ldg(a.raman + j + v * T));
    fft_regs<R, true>(p, buf, tw, plan, j);                                           // g_u1 of both rows
#pragma unroll 1
    for (int r = 0; r < 2; r++) {
#pragma unroll
      for (int v = 0; v < R; v++) {
        const int t = j + v * T;
        const double g1 = r == 0 ? p[v].x : p[v].y;
        const double2 y = row[r].Y[(long long)s * N + t];
        const double2 gy = caxpy(row[r].GY[t], 2.0 * ri * g1, y);
        row[r].GX[t] = cadd(row[r].GX[t], gy);
        row[r].GKE[t] = cscale(gy, fac);
      }
    }
  }
  // the spectrum before the step: H + FFT[the stage inputs' gradient]
#pragma unroll 1
  for (int r = 0; r < 2; r++) {
    double2 gv[R];
#pragma unroll
    for (int v = 0; v < R; v++) gv[v] = row[r].GX[j + v * T];
    fft_regs<R, false>(gv, buf, tw, plan, j);
#pragma unroll
    for (int v = 0; v < R; v++) row[r].G[j + v * T] = cadd(gv[v], row[r].GXP[j + v * T]);
  }
}

}  // namespace

// a.nInst rows, two per thread group (a second row past the end propagates zeros and is not stored).
template <int R>
__global__ void __launch_bounds__(kMaxThreads) k_adjoint_gnlse_pair(const PropArgs a, const AdjArgs d) {
  extern __shared__ double2 smem[];
  __shared__ long long s_group;
  const FFTPlanH& plan = a.plan;
  const int N = plan.N, T = plan.T;
  const int g = threadIdx.x / T, j = threadIdx.x - g * T;
  double2* bufs;
  const double2* tw = stage_twiddles<R>(a.tw, smem, N, &bufs);
  double2* buf = bufs + (long long)g * N;
  const int K = d.K;
  const long long perRow = (long long)(kPairRowSlot + (K > 1 ? 1 + 8 * K : 0)) * N;
  double2* slot = d.seg + ((long long)blockIdx.x * a.ipc + g) * 2 * perRow;
  PairRow row[2] = {pair_row(slot, N, K), pair_row(slot + perRow, N, K)};
  const long long nPairs = (a.nInst + 1) / 2;
  const long long nGroups = (nPairs + a.ipc - 1) / a.ipc;
  for (long long cg = blockIdx.x; cg < nGroups; cg = next_group(a, cg, &s_group)) {
    const long long pair = cg * a.ipc + g;
    const bool act[2] = {pair < nPairs && 2 * pair < a.nInst, pair < nPairs && 2 * pair + 1 < a.nInst};
    const long long inst0 = a.instBase + 2 * pair;
    const double2* ck[2] = {d.ckpt + (act[0] ? inst0 : 0) * (long long)d.nCk * N,
                            d.ckpt + (act[1] ? inst0 + 1 : 0) * (long long)d.nCk * N};
#pragma unroll 1
    for (int r = 0; r < 2; r++) {
      const double2* go = d.gout + (act[r] ? inst0 + r : 0) * (long long)N;
#pragma unroll
      for (int v = 0; v < R; v++) row[r].G[j + v * T] = act[r] ? cscale(go[j + v * T], (double)N) : czero();
    }
    int segEnd = a.nZ - 1;
    while (segEnd >= 1) {
      const int jseg = (segEnd - 1) / K;
      const int s0 = jseg * K;
      if (K > 1) {
        // recompute the segment's steps from its checkpoint, storing each step's stage values: step
        // s0 + 1 + q at STG q (the state being advanced in SEG)
#pragma unroll 1
        for (int r = 0; r < 2; r++) {
#pragma unroll
          for (int v = 0; v < R; v++) row[r].SEG[j + v * T] = ck[r][(long long)jseg * N + j + v * T];
        }
        double2* const y0[2] = {row[0].Y, row[1].Y};
        double2* const u0[2] = {row[0].U2, row[1].U2};
        for (int i = s0 + 1; i <= segEnd; i++) {
          const long long q = i - 1 - s0;
          const bool more = i < segEnd;
#pragma unroll 1
          for (int r = 0; r < 2; r++) {
            row[r].Y = row[r].SEG + N + q * 8 * N;
            row[r].U2 = row[r].Y + 4LL * N;
          }
          pair_stages<R>(a, i, j, buf, tw, row[0].SEG, row[1].SEG, row, more);
          if (more) {
#pragma unroll 1
            for (int r = 0; r < 2; r++) {
              double2 x[R];
#pragma unroll
              for (int v = 0; v < R; v++) x[v] = caxpy(row[r].SEG[j + v * T], 1.0 / 6.0, row[r].ACC[j + v * T]);
              fft_regs<R, false>(x, buf, tw, plan, j);
#pragma unroll
              for (int v = 0; v < R; v++) x[v] = cmul(x[v], __ldg(a.dstep + j + v * T));
              fft_regs<R, true>(x, buf, tw, plan, j);
#pragma unroll
              for (int v = 0; v < R; v++) row[r].SEG[j + v * T] = x[v];
            }
          }
        }
        // reverse the segment from the stored stage values
        for (int i = segEnd; i > s0; i--) {
          const long long q = i - 1 - s0;
#pragma unroll 1
          for (int r = 0; r < 2; r++) {
            row[r].Y = row[r].SEG + N + q * 8 * N;
            row[r].U2 = row[r].Y + 4LL * N;
          }
          pair_reverse_step<R>(a, i, j, buf, tw, row);
        }
#pragma unroll 1
        for (int r = 0; r < 2; r++) {
          row[r].Y = y0[r];
          row[r].U2 = u0[r];
        }
      } else {
        for (int i = segEnd; i > s0; i--) {
          pair_stages<R>(a, i, j, buf, tw, ck[0] + (long long)(i - 1) * N, ck[1] + (long long)(i - 1) * N, row, false);
          pair_reverse_step<R>(a, i, j, buf, tw, row);
        }
      }
      segEnd = s0;
    }
    // G: the gradient of the input spectrum times half a dispersion step (its transform)
#pragma unroll 1
    for (int r = 0; r < 2; r++) {
      if (act[r]) {
#pragma unroll
        for (int v = 0; v < R; v++)
          d.gin[(inst0 + r) * (long long)N + j + v * T] = cmulc(row[r].G[j + v * T], __ldg(a.half + j + v * T));
      }
    }
    __syncthreads();
  }
}

void add_kernels_adjoint_gnlse(std::vector<KernelEntry>& t) {
  t.push_back({kKindAdjoint, kChi3GNLSE, 8, (const void*)k_adjoint_gnlse<8>});
  // key + 100: the pipelined two-CTA-cluster variant
  t.push_back({kKindAdjoint, kChi3GNLSE + 100, 8, (const void*)k_adjoint_gnlse_pipe<8>});
  // key + 400: two rows per thread group, shared Raman transforms
  t.push_back({kKindAdjoint, kChi3GNLSE + 400, 8, (const void*)k_adjoint_gnlse_pair<8>});
}

}  // namespace nlm
