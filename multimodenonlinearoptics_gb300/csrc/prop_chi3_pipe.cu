// prop_chi3_pipe.cu -- the Chi3 pump march and one signal propagation in one cluster of eight CTAs.
//
// Ranks 0..3 march the pump with the arithmetic of k_pump_chi3_spread (solvers/Chi3.cpp:41-70); ranks
// 4..7 propagate the signal with that of k_propagate_spread<FChi3, 4> (src/_NonlinearMedium.hpp:160-239,
// the solver's DiffEq at every step), one phase behind the pump.  The signal's step i reads pump rows
// 2i-2, 2i-1 and 2i of the time-domain grid at its own points; the pump writes row 2p at the end of
// phase p, and the first cluster barrier of the next phase orders that write before the signal's read
// (barrier.cluster arrive has release and wait acquire semantics at cluster scope).  Each march alone
// is a chain of latency-bound transforms on four SMs; side by side the signal's march costs about
// nothing beyond the pump's.
//
// Every spread transform ends with one barrier of the whole cluster, so both groups pass the same
// sequence of barrier slots (4 nZ + 2, after one barrier that all eight CTAs pass first):
//   start        2 slots   pump: row 0 (forward, inverse)   signal: input (forward or bare), inverse
//   phase p      4 slots   pump: rows 2p-1 and 2p           signal: 2 bare, step p-1 (2 slots)
//                (p = 1 .. nZ-1; in phase 1 the signal passes 4 bare barriers)
// An interval between two barriers lasts as long as the slower group.  The pump's intervals alternate
// long (a local inverse transform, the store, the phase factor, a local forward transform) and short
// (the exchange's combination and the dispersion factor); the signal's step has the same shape (its
// long part: the pump loads, the DiffEq and the local forward transform; then the short part; its
// local inverse transform falls in the pump's next long interval), placed so that long meets long.
//   end          4 slots   pump: the last row's half-step   signal: 2 bare, step nZ-1 (forward, then
//                          undo (inverse), 3 bare                   inverse or bare)
// The pump group runs the operations of k_pump_chi3_spread in the same order; the two kernels' grids
// agree to rounding (the compiler may pair multiply-adds differently in each).
#include "nlm_launch.h"
#include "prop_spread.cuh"

namespace nlm {

__global__ void __launch_bounds__(kMaxThreads) k_chi3_pump_signal_spread(const PropArgs a, const PumpMarchArgs p) {
  extern __shared__ double2 smem[];
  cg::cluster_group cl = cg::this_cluster();
  const int crank = (int)cl.block_rank();
  const int role = crank / kSpreadC;   // 0: pump march, 1: signal
  SpreadFFT f;
  const int M = a.plan.N;
  spread_init(f, smem, a.tw, M, crank - role * kSpreadC);
  f.base = role * kSpreadC;
  const int N = M * kSpreadC;
  const int tn = f.rank + kSpreadC * f.t, fk = f.j + M * f.rank;
  const int nZ = a.nZ;
  cl.sync();   // every CTA of the cluster has started before the first exchange writes to its memory
  if (role == 0) {
    const double invN = 1.0 / N;
    const double2 hp = p.halfP[fk], dp = p.dstepP[fk];
    double2 x = spread_fwd(f, p.env[tn], cl);
    x = cmul(x, hp);
    x = cscale(spread_inv_store(f, x, cl, [&](double2 v) { p.pf[fk] = v; }), invN);
    p.pt[tn] = x;
    for (int i = 1; i < p.nRows; i++) {
      const double2 r = p.rel[i - 1];
      const double a2 = cabs2(x);
      x = cmul(x, spm_factor(r.x * a2, r.y * a2));
      x = cmul(spread_fwd(f, x, cl), dp);
      x = cscale(spread_inv_store(f, x, cl, [&](double2 v) { p.pf[(long long)i * N + fk] = v; }), invN);
      p.pt[(long long)i * N + tn] = x;
    }
    // last row: undo half of the last pump dispersion step (each thread rereads its own bin)
    const long long last = (long long)(p.nRows - 1) * N;
    x = cmul(p.pf[last + fk], p.backP[fk]);
    p.pt[last + tn] = cscale(spread_inv_store(f, x, cl, [&](double2 v) { p.pf[last + fk] = v; }), invN);
    spread_idle(cl, 3);
    return;
  }
  const long long inst = a.instBase;
  double2 x = a.in[inst * a.inStride + (a.inTime ? tn : fk)];
  if (a.inTime) x = spread_fwd(f, x, cl);
  else cl.sync();
  x = cmul(x, __ldg(a.half + fk));
  x = spread_inv_store(f, x, cl, [&](double2 v) {
    if (a.gridF) a.gridF[fk] = cscale(v, (double)N);
  });
  if (a.gridT) a.gridT[tn] = x;
  // step i: the DiffEq with pump rows 2i-2 .. 2i (plain loads: the pump group writes them during this
  // launch), then the dispersion step; two barrier slots
  auto step = [&](int i) {
    const double2* c = a.coef + (long long)(i - 1) * 3 * a.nCoef;
    const double2* pr = a.pump + (long long)(2 * i - 2) * N + tn;
    double2 pp[3][1] = {{pr[0]}, {pr[N]}, {pr[2 * N]}};
    double2 xm[1] = {x};
    rk4_point<FChi3>(xm, pp, c);
    const bool last = i == nZ - 1;
    const double2* table = last ? a.dlast : a.dstep;
    const bool wantTime = !last || a.inTime || a.gridT != nullptr;
    x = cmul(spread_fwd(f, xm[0], cl), __ldg(table + fk));
    auto storeF = [&](double2 v) {
      if (a.gridF) a.gridF[(long long)i * N + fk] = cscale(v, (double)N);
    };
    if (wantTime) {
      x = spread_inv_store(f, x, cl, storeF);
      if (a.gridT) a.gridT[(long long)i * N + tn] = x;
    } else {
      storeF(x);
      cl.sync();
    }
  };
  spread_idle(cl, 4);   // phase 1: the pump computes rows 1 and 2
  for (int ph = 2; ph < nZ; ph++) {
    // after the first barrier rows up to 2 ph - 2 are in place; after the second the step's long part
    // (loads, DiffEq, local forward transform) runs beside the pump's (local transforms, phase factor)
    spread_idle(cl, 2);
    step(ph - 1);
  }
  spread_idle(cl, 2);   // the pump's last row, then the barrier after its store
  step(nZ - 1);
}

cudaError_t launch_chi3_pump_signal_spread(const PropArgs& a, const PumpMarchArgs& p, cudaStream_t s, int* regs) {
  const int M = a.plan.N, N = M * kSpreadC;
  if (M < 32 || M > kMaxThreads || (M & (M - 1)) != 0 || a.nZ < 2 || p.nRows != 2 * a.nZ - 1 || a.nInst != 1 ||
      a.inStride < N)
    return cudaErrorInvalidValue;
  const void* fn = (const void*)k_chi3_pump_signal_spread;
  size_t smem = 0;
  cudaFuncAttributes fa;
  cudaError_t e = exclusive_smem(fn, (size_t)spread_smem_per_point(kSpreadC) * M * sizeof(double2), &smem, &fa);
  if (e != cudaSuccess) return e;
  if (smem == 0) return cudaErrorInvalidValue;
  if (regs) *regs = fa.numRegs;
  PropArgs ac = a;
  PumpMarchArgs pc = p;
  void* args[] = {(void*)&ac, (void*)&pc};
  return launch_clustered(fn, 2 * kSpreadC, M, smem, s, 2 * kSpreadC, args);
}

}  // namespace nlm
