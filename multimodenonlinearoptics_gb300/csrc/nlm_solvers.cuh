// nlm_solvers.cuh -- point-wise right-hand sides (the reference's DiffEq) as device functors.
//
// Each functor evaluates one RK4 stage at one grid point:
//     k = f(y, p, c)
// y: the signal modes at the point (already offset by the previous stage, y = x + h*k),
// p: the pump modes at the stage's z (pump rows 2i-2, 2i-1, 2i of the reference),
// c: the stage's complex coefficients.  The coefficients (poling sign, nonlinear step,
// phase mismatch, intensity profile, in the reference's own order of operations) are
// scalars per z step and are computed once on the host in double precision, the way the
// reference computes them inside each DiffEq.  The functor keeps the reference's
// association of the remaining point-wise products.
#pragma once
#include "nlm_device.cuh"

namespace nlm {

enum SolverId : int {
  kChi3 = 0, kChi2PDC, kChi2SFG, kChi2AFC, kChi2SFGPDC, kChi2SFGII, kChi2PDCII, kChi2SFGOPA, kChi2SFGXPM,
  kChi2SHG, kChi2SHGOPA, kChi2DSFG, kChi2SHGXPM, kChi2ASHG, kChi3GNLSE, kNumSolvers
};

// solvers/Chi3.cpp:73-85: k = g (2|P|^2 y + P^2 conj(y)); c = {nlStep}
struct FChi3 {
  static constexpr int kM = 1, kP = 1, kC = 1;
  __device__ static void f(const double2* y, const double2* p, const double2* c, double2* k) {
    const double2 t = caxpy(cmul(csq(p[0]), cconj(y[0])), 2.0 * cabs2(p[0]), y[0]);
    k[0] = cmul(c[0], t);
  }
};

// solvers/Chi2PDC.cpp:27-44: k = (pol g M) P conj(y); c = {pol*g*M}
struct FChi2PDC {
  static constexpr int kM = 1, kP = 1, kC = 1;
  __device__ static void f(const double2* y, const double2* p, const double2* c, double2* k) {
    k[0] = cmulc(cmul(c[0], p[0]), y[0]);
  }
};

// solvers/Chi2SFG.cpp:28-56: kS = (pol g0 M) P yO, kO = (pol g1 /M) conj(P) yS
struct FChi2SFG {
  static constexpr int kM = 2, kP = 1, kC = 2;
  __device__ static void f(const double2* y, const double2* p, const double2* c, double2* k) {
    k[0] = cmul(cmul(c[0], p[0]), y[1]);
    k[1] = cmul(cmul(c[1], cconj(p[0])), y[0]);
  }
};

// solvers/Chi2AFC.cpp:26-51: as Chi2SFG without poling, chirped mismatch
using FChi2AFC = FChi2SFG;

// solvers/Chi2SFGPDC.cpp:28-59: kS = (pol g0 M) P yO, kO = (pol g1) ((1/M) conj(P) yS + Mo P conj(yO))
struct FChi2SFGPDC {
  static constexpr int kM = 2, kP = 1, kC = 4;
  __device__ static void f(const double2* y, const double2* p, const double2* c, double2* k) {
    k[0] = cmul(cmul(c[0], p[0]), y[1]);
    const double2 a = cmul(cmul(c[2], cconj(p[0])), y[0]);
    const double2 b = cmulc(cmul(c[3], p[0]), y[1]);
    k[1] = cmul(c[1], cadd(a, b));
  }
};

// solvers/Chi2SFGII.cpp:34-90; modes {Sz, Sy, Oz, Oy}; c = {pol, g0 Mcz, g1 Msz, pol g0 Mcy, g0/Mcy, g1/Msz, pol g0/Mcz}
struct FChi2SFGII {
  static constexpr int kM = 4, kP = 1, kC = 7;
  __device__ static void f(const double2* y, const double2* p, const double2* c, double2* k) {
    const double pol = c[0].x;
    const double2 pp = cscale(p[0], pol);
    const double2 pc = cscale(cconj(p[0]), pol);
    k[0] = cmul(pp, cadd(cmul(c[1], y[3]), cmul(c[2], y[2])));
    k[1] = cmul(cmul(c[3], p[0]), y[2]);
    k[2] = cmul(pc, cadd(cmul(c[4], y[1]), cmul(c[5], y[0])));
    k[3] = cmul(cmul(c[6], cconj(p[0])), y[0]);
  }
};

// solvers/Chi2PDCII.cpp:29-55: kS = (pol g0 M) P conj(yO), kO = (pol g1 M) P conj(yS)
struct FChi2PDCII {
  static constexpr int kM = 2, kP = 1, kC = 2;
  __device__ static void f(const double2* y, const double2* p, const double2* c, double2* k) {
    k[0] = cmulc(cmul(c[0], p[0]), y[1]);
    k[1] = cmulc(cmul(c[1], p[0]), y[0]);
  }
};

// solvers/Chi2SFGOPA.cpp:31-77; modes {H, F}, pumps {P0, P1}
// c = {pol g0 Msfg, pol g2 Mdopa, pol g1 /Msfg, pol g3 Mdopa}
struct FChi2SFGOPA {
  static constexpr int kM = 2, kP = 2, kC = 4;
  __device__ static void f(const double2* y, const double2* p, const double2* c, double2* k) {
    k[0] = cadd(cmul(cmul(c[0], p[0]), y[1]), cmulc(cmul(c[1], p[1]), y[1]));
    k[1] = cadd(cmul(cmul(c[2], cconj(p[0])), y[0]), cmulc(cmul(c[3], p[1]), y[0]));
  }
};

// solvers/Chi2SFGXPM.cpp:29-58: kS = ((pol g0 M) P + g2 |P|^2) yO, kO = ((pol g1 /M) conj(P) + g3 |P|^2) yS
struct FChi2SFGXPM {
  static constexpr int kM = 2, kP = 1, kC = 4;
  __device__ static void f(const double2* y, const double2* p, const double2* c, double2* k) {
    const double a2 = cabs2(p[0]);
    k[0] = cmul(cadd(cmul(c[0], p[0]), cscale(c[2], a2)), y[1]);
    k[1] = cmul(cadd(cmul(c[1], cconj(p[0])), cscale(c[3], a2)), y[0]);
  }
};

// solvers/Chi2SHG.cpp:25-60 (fully nonlinear); modes {P, SH}
// c = {rel g0 M, rel g1 /M * .5}
struct FChi2SHG {
  static constexpr int kM = 2, kP = 0, kC = 2;
  __device__ static void f(const double2* y, const double2*, const double2* c, double2* k) {
    k[0] = cmul(cmul(c[0], cconj(y[0])), y[1]);
    k[1] = cmul(c[1], csq(y[0]));
  }
};

// solvers/Chi2ASHG.cpp:24-56 (fully nonlinear, chirped mismatch): same point-wise form as Chi2SHG
using FChi2ASHG = FChi2SHG;

// solvers/Chi2SHGOPA.cpp:32-84 (fully nonlinear); modes {P, SH, A1, A2}
// c = {rel g0 Mshg, rel g1, Mopa, (1/Mshg) .5, rel g2 /Mopa, rel g3 /Mopa}
struct FChi2SHGOPA {
  static constexpr int kM = 4, kP = 0, kC = 6;
  __device__ static void f(const double2* y, const double2*, const double2* c, double2* k) {
    k[0] = cmul(cmul(c[0], cconj(y[0])), y[1]);
    k[1] = cmul(c[1], cadd(cmul(cmul(c[2], y[3]), y[2]), cmul(c[3], csq(y[0]))));
    k[2] = cmulc(cmul(c[4], y[1]), y[3]);
    k[3] = cmulc(cmul(c[5], y[1]), y[2]);
  }
};

// solvers/Chi2DSFG.cpp:27-67 (fully nonlinear); modes {P, S, D}
// c = {rel g0 M, rel g1 /M, rel g2 M}
struct FChi2DSFG {
  static constexpr int kM = 3, kP = 0, kC = 3;
  __device__ static void f(const double2* y, const double2*, const double2* c, double2* k) {
    k[0] = cmulc(cmul(c[0], y[1]), y[2]);
    k[1] = cmul(cmul(c[1], y[0]), y[2]);
    k[2] = cmulc(cmul(c[2], y[1]), y[0]);
  }
};

// solvers/Chi2SHGXPM.cpp:25-65 (fully nonlinear); modes {P, SH}
// c = {rel g0 M, rel g1 /M * .5, relAmp^2 g2}
struct FChi2SHGXPM {
  static constexpr int kM = 2, kP = 0, kC = 3;
  __device__ static void f(const double2* y, const double2*, const double2* c, double2* k) {
    const double ap = cabs2(y[0]), ah = cabs2(y[1]);
    k[0] = cadd(cmul(cmul(c[0], cconj(y[0])), y[1]), cmul(cscale(c[2], ap + 2.0 * ah), y[0]));
    k[1] = cadd(cmul(c[1], csq(y[0])), cmul(cscale(cscale(c[2], 2.0), ah + 2.0 * ap), y[1]));
  }
};

// Number of coefficients per stage and modes/pumps per solver, host-visible.
struct SolverShape {
  int modes, pumps, coefs;
  bool linear;
};

}  // namespace nlm
