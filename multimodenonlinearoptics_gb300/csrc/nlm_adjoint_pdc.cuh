// nlm_adjoint_pdc.cuh -- the point-wise parts of the Chi2PDC reverse sweep (solvers/Chi2PDC.cpp:27-44
// run backwards), shared by the one-CTA kernels (adjoint.cu) and the cluster kernel
// (adjoint_cluster.cu).  N is passed explicitly: the cluster kernels' plan is the local one.
#pragma once
#include "nlm_propagate.cuh"

namespace nlm {

__device__ __forceinline__ void atomic_add2(double2* p, double2 v) {
  atomicAdd(&p->x, v.x);
  atomicAdd(&p->y, v.y);
}

// The RK4 step i at time point t: the per-point real 2x2 propagator matrix (pairs (M00, M01),
// (M10, M11)) when the engine built it, else the four stage evaluations.
__device__ __forceinline__ double2 pdc_step_point(const PropArgs& a, int N, int i, int t, double2 x) {
  if (a.prop) {
    const double2* mat = reinterpret_cast<const double2*>(a.prop) + (long long)(i - 1) * 2 * N;
    const double2 e0 = __ldg(mat + t), e1 = __ldg(mat + N + t);
    return make_double2(fma(e0.y, x.y, e0.x * x.x), fma(e1.y, x.y, e1.x * x.x));
  }
  const double2* c = a.coef + (long long)(i - 1) * 3 * a.nCoef;
  const double2* pr = a.pump + (long long)(2 * i - 2) * N + t;
  double2 p[3][1] = {{__ldg(pr)}, {__ldg(pr + N)}, {__ldg(pr + 2 * N)}};
  double2 xm[1] = {x};
  rk4_point<FChi2PDC>(xm, p, c);
  return xm[0];
}

// The forward stages of RK4 step i at time point t (solvers/Chi2PDC.cpp:40-43), which its transpose
// reads: the stage factors a_s = c_s P_s (c0..c2: the step's coefficients) and the stage inputs.
struct PdcStages {
  double2 a0, a1, a2, y1, y2, y3;
};

__device__ __forceinline__ PdcStages pdc_stages(const PropArgs& a, int N, int i, int t, double2 c0, double2 c1,
                                                double2 c2, double2 x) {
  const double2* pr = a.pump + (long long)(2 * i - 2) * N + t;
  PdcStages s;
  s.a0 = cmul(c0, __ldg(pr));
  s.a1 = cmul(c1, __ldg(pr + N));
  s.a2 = cmul(c2, __ldg(pr + 2 * N));
  const double2 k1 = cmulc(s.a0, x);
  s.y1 = caxpy(x, 0.5, k1);
  const double2 k2 = cmulc(s.a1, s.y1);
  s.y2 = caxpy(x, 0.5, k2);
  const double2 k3 = cmulc(s.a1, s.y2);
  s.y3 = cadd(x, k3);
  return s;
}

// The transposed stages: gp is the gradient after the step, x the state before it.  Returns the
// gradient before the step and the gradients of the stage factors in ga0..ga2.
__device__ __forceinline__ double2 pdc_stages_reverse(const PdcStages& s, double2 x, double2 gp, double2& ga0,
                                                      double2& ga1, double2& ga2) {
  // x' = x + (k1 + 2 k2 + 2 k3 + k4) / 6 with k = a conj(y)
  double2 gx = gp;
  double2 gk1 = cscale(gp, 1.0 / 6.0);
  double2 gk2 = cscale(gp, 1.0 / 3.0);
  double2 gk3 = gk2;
  const double2 gk4 = gk1;
  ga2 = cmul(s.y3, gk4);
  const double2 gy3 = cmulc(s.a2, gk4);
  gx = cadd(gx, gy3);
  gk3 = cadd(gk3, gy3);
  ga1 = cmul(s.y2, gk3);
  const double2 gy2 = cmulc(s.a1, gk3);
  gx = cadd(gx, gy2);
  gk2 = caxpy(gk2, 0.5, gy2);
  ga1 = cadd(ga1, cmul(s.y1, gk2));
  const double2 gy1 = cmulc(s.a1, gk2);
  gx = cadd(gx, gy1);
  gk1 = caxpy(gk1, 0.5, gy1);
  ga0 = cmul(x, gk1);
  gx = cadd(gx, cmulc(s.a0, gk1));
  return gx;
}

// Transposed RK4 step i at time point t: both halves above.
__device__ __forceinline__ double2 pdc_stage_chain(const PropArgs& a, int N, int i, int t, double2 c0, double2 c1,
                                                   double2 c2, double2 x, double2 gp, double2& ga0, double2& ga1,
                                                   double2& ga2) {
  return pdc_stages_reverse(pdc_stages(a, N, i, t, c0, c1, c2, x), x, gp, ga0, ga1, ga2);
}

// The stage-factor gradients of step i at point t into d.ga (plain stores for a single instance,
// atomics otherwise).
__device__ __forceinline__ void pdc_store_ga(const AdjArgs& d, int N, int i, int t, double2 ga0, double2 ga1,
                                             double2 ga2) {
  double2* gacc = d.ga + (long long)(i - 1) * 3 * N;
  if (d.single) {   // the only instance: each element is written once
    gacc[t] = ga0;
    gacc[N + t] = ga1;
    gacc[2 * N + t] = ga2;
  } else {
    atomic_add2(gacc + t, ga0);
    atomic_add2(gacc + N + t, ga1);
    atomic_add2(gacc + 2 * N + t, ga2);
  }
}

// P^T gp at point t for step i, with P the step's real 2x2 RK4 matrix at the point (pairs (M00, M01),
// (M10, M11)): 4 FMAs.
__device__ __forceinline__ double2 pdc_transpose_point(const PropArgs& a, int N, int i, int t, double2 gp) {
  const double2* mat = reinterpret_cast<const double2*>(a.prop) + (long long)(i - 1) * 2 * N;
  const double2 e0 = __ldg(mat + t), e1 = __ldg(mat + N + t);
  return make_double2(fma(e1.x, gp.y, e0.x * gp.x), fma(e1.y, gp.y, e0.y * gp.x));
}

// pdc_stage_chain, with the stage-factor gradients added to d.ga.
__device__ __forceinline__ double2 pdc_reverse_point(const PropArgs& a, const AdjArgs& d, int N, int i, int t,
                                                     double2 c0, double2 c1, double2 c2, double2 x, double2 gp,
                                                     bool active) {
  double2 ga0, ga1, ga2;
  const double2 gx = pdc_stage_chain(a, N, i, t, c0, c1, c2, x, gp, ga0, ga1, ga2);
  if (active) pdc_store_ga(d, N, i, t, ga0, ga1, ga2);
  return gx;
}

// The reverse step's point-wise part in the marching form (d.gp set, propagator matrices in a.prop):
// the gradient after the step is stored for the stage-factor gradients, computed afterwards in
// parallel over all steps (k_adj_stage_grads), and the gradient before the step is P^T gp.
__device__ __forceinline__ double2 pdc_march_point(const PropArgs& a, const AdjArgs& d, int N, int i, int t,
                                                   long long inst, double2 gp, bool active) {
  if (active) d.gp[(inst * (a.nZ - 1) + (i - 1)) * (long long)N + t] = gp;
  return pdc_transpose_point(a, N, i, t, gp);
}

}  // namespace nlm
