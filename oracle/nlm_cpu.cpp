// nlm_cpu.cpp -- C++ restatement of the reference's optimised split-step loop, for the CPU baseline.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the product links or loads this file: `bench.py` times it
// as the CPU baseline (the reference's own C++ engine needs the Eigen 3 headers, absent on both
// machines, so it cannot be built), and `tests/test_cpu_port.py` checks it against the numpy oracle.
//
// What it restates (paths relative to the reference project root):
//  * the optimised split-step loop of src/_NonlinearMedium.hpp:160-239 (the `optimized` branch that
//    keeps one row): half dispersion in, (nZSteps-1) x [RK4 of the DiffEq -> FFT -> x dispStep ->
//    inverse FFT], half dispersion out;
//  * solvers/Chi2PDC.cpp:27-47 (DiffEq) and src/_NonlinearMedium.cpp:225-250 (the linear pump grid);
//  * solvers/Chi3GNLSE.cpp:39-92 (DiffEq with the Raman convolution and self-steepening);
//  * src/_NonlinearMedium.cpp:263-375 (computeGreensFunction: 2N impulse propagations over
//    std::threads in contiguous ranges, C/S from the pairs, transpose and block fftshift) and
//    :378-444 (batchSignalSimulation).
// The DFT is this file's own: an out-of-place radix-4 Stockham (one radix-2 pass when log2 N is
// odd) on split real/imaginary arrays, forward unscaled and inverse scaled by 1/N as in
// src/CustomEigenFFT.h:91-101.  Power-of-two grids only.
//
// Built by oracle/build_oracle.py (g++ -O3, portable flags) into oracle/_build/libnlm_cpu.so.
#include <cmath>
#include <complex>
#include <cstring>
#include <thread>
#include <vector>

namespace {

using cd = std::complex<double>;

// ---------------------------------------------------------------------------------------------
// Stockham FFT on split arrays.  Pass (L, r): reads x[j + q N/r] (j = b L + k, k < L), multiplies by
// exp(-2 pi i k q / (L r)), applies the r-point DFT and writes y[(b r + s) L + k].
// ---------------------------------------------------------------------------------------------
struct Plan {
  int n = 0;
  std::vector<int> radix;                      // radix of each pass, in order
  std::vector<std::vector<double>> wr, wi;     // per pass: [(q-1) L + k], q = 1..r-1
};

Plan make_plan(int n) {
  Plan p;
  p.n = n;
  int logn = 0;
  while ((1 << logn) < n) logn++;
  if (logn % 2) p.radix.push_back(2);
  for (int t = 0; t < logn / 2; t++) p.radix.push_back(4);
  int L = 1;
  for (int r : p.radix) {
    std::vector<double> a((size_t)(r - 1) * L), b((size_t)(r - 1) * L);
    for (int q = 1; q < r; q++)
      for (int k = 0; k < L; k++) {
        const double th = -2.0 * M_PI * (double)k * q / ((double)L * r);
        a[(size_t)(q - 1) * L + k] = std::cos(th);
        b[(size_t)(q - 1) * L + k] = std::sin(th);
      }
    p.wr.push_back(std::move(a));
    p.wi.push_back(std::move(b));
    L *= r;
  }
  return p;
}

template <bool INV>
void pass2(const double* xr, const double* xi, double* yr, double* yi, int n, int L, const double* wr,
           const double* wi) {
  const int h = n / 2, nb = n / (2 * L);
  for (int b = 0; b < nb; b++) {
    const double *x0r = xr + b * L, *x0i = xi + b * L, *x1r = x0r + h, *x1i = x0i + h;
    double *y0r = yr + 2 * b * L, *y0i = yi + 2 * b * L, *y1r = y0r + L, *y1i = y0i + L;
    for (int k = 0; k < L; k++) {
      const double c = wr[k], s = INV ? -wi[k] : wi[k];
      const double ar = x1r[k] * c - x1i[k] * s, ai = x1r[k] * s + x1i[k] * c;
      y0r[k] = x0r[k] + ar;
      y0i[k] = x0i[k] + ai;
      y1r[k] = x0r[k] - ar;
      y1i[k] = x0i[k] - ai;
    }
  }
}

template <bool INV>
inline void bfly4(double a0r, double a0i, double a1r, double a1i, double a2r, double a2i, double a3r, double a3i,
                  double* y0r, double* y0i, double* y1r, double* y1i, double* y2r, double* y2i, double* y3r,
                  double* y3i) {
  const double t0r = a0r + a2r, t0i = a0i + a2i, t1r = a0r - a2r, t1i = a0i - a2i;
  const double t2r = a1r + a3r, t2i = a1i + a3i, t3r = a1r - a3r, t3i = a1i - a3i;
  *y0r = t0r + t2r;
  *y0i = t0i + t2i;
  *y2r = t0r - t2r;
  *y2i = t0i - t2i;
  if (!INV) {   // y1 = t1 - i t3, y3 = t1 + i t3
    *y1r = t1r + t3i;
    *y1i = t1i - t3r;
    *y3r = t1r - t3i;
    *y3i = t1i + t3r;
  } else {      // y1 = t1 + i t3, y3 = t1 - i t3
    *y1r = t1r - t3i;
    *y1i = t1i + t3r;
    *y3r = t1r + t3i;
    *y3i = t1i - t3r;
  }
}

template <bool INV>
void pass4(const double* xr, const double* xi, double* yr, double* yi, int n, int L, const double* wr,
           const double* wi) {
  const int m = n / 4, nb = n / (4 * L);
  if (L == 1) {
    for (int b = 0; b < nb; b++) {
      double o[8];
      bfly4<INV>(xr[b], xi[b], xr[b + m], xi[b + m], xr[b + 2 * m], xi[b + 2 * m], xr[b + 3 * m], xi[b + 3 * m],
                 &o[0], &o[1], &o[2], &o[3], &o[4], &o[5], &o[6], &o[7]);
      for (int s = 0; s < 4; s++) {
        yr[4 * b + s] = o[2 * s];
        yi[4 * b + s] = o[2 * s + 1];
      }
    }
    return;
  }
  const double *w1r = wr, *w1i = wi, *w2r = wr + L, *w2i = wi + L, *w3r = wr + 2 * L, *w3i = wi + 2 * L;
  for (int b = 0; b < nb; b++) {
    const double* x0r = xr + b * L;
    const double* x0i = xi + b * L;
    double* y0r = yr + 4 * b * L;
    double* y0i = yi + 4 * b * L;
    for (int k = 0; k < L; k++) {
      const double s1 = INV ? -w1i[k] : w1i[k], s2 = INV ? -w2i[k] : w2i[k], s3 = INV ? -w3i[k] : w3i[k];
      const double b1r = x0r[k + m], b1i = x0i[k + m], b2r = x0r[k + 2 * m], b2i = x0i[k + 2 * m];
      const double b3r = x0r[k + 3 * m], b3i = x0i[k + 3 * m];
      const double a1r = b1r * w1r[k] - b1i * s1, a1i = b1r * s1 + b1i * w1r[k];
      const double a2r = b2r * w2r[k] - b2i * s2, a2i = b2r * s2 + b2i * w2r[k];
      const double a3r = b3r * w3r[k] - b3i * s3, a3i = b3r * s3 + b3i * w3r[k];
      bfly4<INV>(x0r[k], x0i[k], a1r, a1i, a2r, a2i, a3r, a3i, &y0r[k], &y0i[k], &y0r[k + L], &y0i[k + L],
                 &y0r[k + 2 * L], &y0i[k + 2 * L], &y0r[k + 3 * L], &y0i[k + 3 * L]);
    }
  }
}

// In place on (re, im) with the work arrays (tr, ti); unscaled.
template <bool INV>
void fft(const Plan& p, double* re, double* im, double* tr, double* ti) {
  double *sr = re, *si = im, *dr = tr, *di = ti;
  int L = 1;
  for (size_t t = 0; t < p.radix.size(); t++) {
    if (p.radix[t] == 4) pass4<INV>(sr, si, dr, di, p.n, L, p.wr[t].data(), p.wi[t].data());
    else pass2<INV>(sr, si, dr, di, p.n, L, p.wr[t].data(), p.wi[t].data());
    L *= p.radix[t];
    std::swap(sr, dr);
    std::swap(si, di);
  }
  if (sr != re) {
    std::memcpy(re, sr, sizeof(double) * p.n);
    std::memcpy(im, si, sizeof(double) * p.n);
  }
}

// Split copies of a complex table.
struct Split {
  std::vector<double> r, i;
  Split() = default;
  Split(const double* c, int n, double scale = 1.0) : r(n), i(n) {
    for (int k = 0; k < n; k++) {
      r[k] = c[2 * k] * scale;
      i[k] = c[2 * k + 1] * scale;
    }
  }
};

// Per-thread state of one propagation.
struct Work {
  std::vector<double> xr, xi, tr, ti, ar, ai, yr, yi, dr, di, ur, ui, vr, vi;
  explicit Work(int n)
      : xr(n), xi(n), tr(n), ti(n), ar(n), ai(n), yr(n), yi(n), dr(n), di(n), ur(n), ui(n), vr(n), vi(n) {}
};

// x <- x * t (complex tables, split)
inline void mul_table(double* xr, double* xi, const Split& t, int n) {
  for (int k = 0; k < n; k++) {
    const double r = xr[k] * t.r[k] - xi[k] * t.i[k], i = xr[k] * t.i[k] + xi[k] * t.r[k];
    xr[k] = r;
    xi[k] = i;
  }
}

// The dispersion half of a step (src/_NonlinearMedium.hpp:214-216): F = FFT(x) dispStep; x = IFFT(F).
// dstep carries dispStep / N (the inverse's scale folded in); on the last step the caller uses
// dstep * exp(-i dz/2 D) / N and keeps F (times N) as the output spectrum.
struct Medium {
  int n = 0, nz = 0;
  Plan plan;
  Split half;        // exp(+i dz/2 D) / N  (input: IFFT of the half-stepped spectrum)
  Split dstep;       // dispStep / N
  Split dlast;       // dispStep exp(-i dz/2 D) / N
};

// ---------------------------------------------------------------------------------------------
// Chi2PDC: k = polDir nlStep e^{i dB z} P conj(A)  (solvers/Chi2PDC.cpp:27-47)
// ---------------------------------------------------------------------------------------------
struct PDC {
  Medium md;
  std::vector<double> pr, pi;   // pump time grid, nZStepsP x N, split
  std::vector<cd> c;            // (nZ-1) x 3 stage factors polDir nlStep e^{i dB z}
};

// One propagation; spectrum (frequency domain, as in the Green's function) in xin (complex, n),
// output spectrum of the last row in outr/outi.
void pdc_propagate(const PDC& P, Work& w, const double* inr, const double* ini, double* outr, double* outi) {
  const int n = P.md.n;
  double *xr = w.xr.data(), *xi = w.xi.data();
  for (int k = 0; k < n; k++) {
    xr[k] = inr[k];
    xi[k] = ini[k];
  }
  mul_table(xr, xi, P.md.half, n);
  fft<true>(P.md.plan, xr, xi, w.tr.data(), w.ti.data());
  for (int i = 1; i < P.md.nz; i++) {
    const cd c0 = P.c[(size_t)(i - 1) * 3], c1 = P.c[(size_t)(i - 1) * 3 + 1], c2 = P.c[(size_t)(i - 1) * 3 + 2];
    const double* p0r = P.pr.data() + (size_t)(2 * i - 2) * n;
    const double* p0i = P.pi.data() + (size_t)(2 * i - 2) * n;
    const double *p1r = p0r + n, *p1i = p0i + n, *p2r = p1r + n, *p2i = p1i + n;
    const double c0r = c0.real(), c0i = c0.imag(), c1r = c1.real(), c1i = c1.imag(), c2r = c2.real(),
                 c2i = c2.imag();
    for (int k = 0; k < n; k++) {
      // a_s = c_s P_s; k = a_s conj(y)
      const double a0r = c0r * p0r[k] - c0i * p0i[k], a0i = c0r * p0i[k] + c0i * p0r[k];
      const double a1r = c1r * p1r[k] - c1i * p1i[k], a1i = c1r * p1i[k] + c1i * p1r[k];
      const double a2r = c2r * p2r[k] - c2i * p2i[k], a2i = c2r * p2i[k] + c2i * p2r[k];
      const double x_r = xr[k], x_i = xi[k];
      const double k1r = a0r * x_r + a0i * x_i, k1i = a0i * x_r - a0r * x_i;
      double yr = x_r + 0.5 * k1r, yi = x_i + 0.5 * k1i;
      const double k2r = a1r * yr + a1i * yi, k2i = a1i * yr - a1r * yi;
      yr = x_r + 0.5 * k2r;
      yi = x_i + 0.5 * k2i;
      const double k3r = a1r * yr + a1i * yi, k3i = a1i * yr - a1r * yi;
      yr = x_r + k3r;
      yi = x_i + k3i;
      const double k4r = a2r * yr + a2i * yi, k4i = a2i * yr - a2r * yi;
      xr[k] = x_r + (k1r + 2 * k2r + 2 * k3r + k4r) * (1.0 / 6.0);
      xi[k] = x_i + (k1i + 2 * k2i + 2 * k3i + k4i) * (1.0 / 6.0);
    }
    fft<false>(P.md.plan, xr, xi, w.tr.data(), w.ti.data());
    const bool last = i == P.md.nz - 1;
    mul_table(xr, xi, last ? P.md.dlast : P.md.dstep, n);
    if (!last) fft<true>(P.md.plan, xr, xi, w.tr.data(), w.ti.data());
  }
  for (int k = 0; k < n; k++) {   // the tables carry 1/N; the spectrum is N times that
    outr[k] = xr[k] * n;
    outi[k] = xi[k] * n;
  }
}

void build_medium(Medium& md, int n, int nz, double dz, const double* dispSign) {
  md.n = n;
  md.nz = nz;
  md.plan = make_plan(n);
  md.half.r.resize(n);
  md.half.i.resize(n);
  md.dstep = md.half;
  md.dlast = md.half;
  for (int k = 0; k < n; k++) {
    const cd h = std::exp(cd(0, 0.5 * dz * dispSign[k])) / (double)n;
    const cd b = std::exp(cd(0, -0.5 * dz * dispSign[k]));
    const cd d = std::exp(cd(0, dz * dispSign[k])) / (double)n;
    const cd l = d * b;
    md.half.r[k] = h.real();
    md.half.i[k] = h.imag();
    md.dstep.r[k] = d.real();
    md.dstep.i[k] = d.imag();
    md.dlast.r[k] = l.real();
    md.dlast.i[k] = l.imag();
  }
}

template <class F>
void parallel_ranges(long long total, int threads, F&& fn) {
  if (threads < 1) threads = 1;
  if (threads > total) threads = (int)(total > 0 ? total : 1);
  std::vector<std::thread> pool;
  // contiguous ranges, the split of src/_NonlinearMedium.cpp:350-353
  const long long per = total / threads, extra = total % threads;
  long long start = 0;
  for (int t = 0; t < threads; t++) {
    const long long cnt = per + (t < extra ? 1 : 0);
    pool.emplace_back([=, &fn] { fn(t, start, start + cnt); });
    start += cnt;
  }
  for (auto& th : pool) th.join();
}

// ---------------------------------------------------------------------------------------------
// Chi3GNLSE (solvers/Chi3GNLSE.cpp:39-92): per stage y = x + f d,
//   conv = IFFT(FFT(r |y|^2) R~),  k = IFFT(FFT(conv y) (nlStep0 + nlStep1 omega)).
// ---------------------------------------------------------------------------------------------
struct GNLSE {
  Medium md;
  Split raman;     // R~ / N
  Split steep;     // (nlStep0 + nlStep1 omega) / N
  std::vector<double> rel;   // (nZ-1) x 3 relative intensities
};

void gnlse_rhs(const GNLSE& G, Work& w, double r, const double* yr, const double* yi, double* kr, double* ki) {
  const int n = G.md.n;
  double *ur = w.ur.data(), *ui = w.ui.data(), *vr = w.vr.data(), *vi = w.vi.data();
  for (int k = 0; k < n; k++) {
    ur[k] = r * (yr[k] * yr[k] + yi[k] * yi[k]);
    ui[k] = 0.0;
  }
  fft<false>(G.md.plan, ur, ui, w.tr.data(), w.ti.data());
  mul_table(ur, ui, G.raman, n);
  fft<true>(G.md.plan, ur, ui, w.tr.data(), w.ti.data());
  for (int k = 0; k < n; k++) {
    vr[k] = ur[k] * yr[k] - ui[k] * yi[k];
    vi[k] = ur[k] * yi[k] + ui[k] * yr[k];
  }
  fft<false>(G.md.plan, vr, vi, w.tr.data(), w.ti.data());
  mul_table(vr, vi, G.steep, n);
  fft<true>(G.md.plan, vr, vi, w.tr.data(), w.ti.data());
  std::memcpy(kr, vr, sizeof(double) * n);
  std::memcpy(ki, vi, sizeof(double) * n);
}

// rec (optional): the spectrum after step i (the row i of the reference's full signalFreq grid) for
// every i < nZ-1 that is a multiple of `every`, at rec[(i / every - 1) * N] (complex, interleaved).
void gnlse_propagate(const GNLSE& G, Work& w, const double* inr, const double* ini, bool inTime, double* outr,
                     double* outi, double* rec = nullptr, int every = 0) {
  const int n = G.md.n;
  double *xr = w.xr.data(), *xi = w.xi.data();
  for (int k = 0; k < n; k++) {
    xr[k] = inr[k];
    xi[k] = ini[k];
  }
  if (inTime) fft<false>(G.md.plan, xr, xi, w.tr.data(), w.ti.data());
  mul_table(xr, xi, G.md.half, n);
  fft<true>(G.md.plan, xr, xi, w.tr.data(), w.ti.data());
  double *ar = w.ar.data(), *ai = w.ai.data(), *yr = w.yr.data(), *yi = w.yi.data(), *dr = w.dr.data(),
         *di = w.di.data();
  for (int i = 1; i < G.md.nz; i++) {
    const double* r = G.rel.data() + (size_t)(i - 1) * 3;
    const double rs[4] = {r[0], r[1], r[1], r[2]};
    const double fac[4] = {0.0, 0.5, 0.5, 1.0};
    const double wgt[4] = {1.0, 2.0, 2.0, 1.0};
    for (int k = 0; k < n; k++) ar[k] = ai[k] = 0.0;
    for (int st = 0; st < 4; st++) {
      if (st == 0) {
        std::memcpy(yr, xr, sizeof(double) * n);
        std::memcpy(yi, xi, sizeof(double) * n);
      } else {
        for (int k = 0; k < n; k++) {
          yr[k] = xr[k] + fac[st] * dr[k];
          yi[k] = xi[k] + fac[st] * di[k];
        }
      }
      gnlse_rhs(G, w, rs[st], yr, yi, dr, di);
      for (int k = 0; k < n; k++) {
        ar[k] += wgt[st] * dr[k];
        ai[k] += wgt[st] * di[k];
      }
    }
    for (int k = 0; k < n; k++) {
      xr[k] += ar[k] * (1.0 / 6.0);
      xi[k] += ai[k] * (1.0 / 6.0);
    }
    fft<false>(G.md.plan, xr, xi, w.tr.data(), w.ti.data());
    const bool last = i == G.md.nz - 1;
    mul_table(xr, xi, last ? G.md.dlast : G.md.dstep, n);
    if (rec && every > 0 && !last && i % every == 0) {
      double* row = rec + 2 * (size_t)(i / every - 1) * n;
      for (int k = 0; k < n; k++) {
        row[2 * k] = xr[k] * n;
        row[2 * k + 1] = xi[k] * n;
      }
    }
    if (!last || inTime) fft<true>(G.md.plan, xr, xi, w.tr.data(), w.ti.data());
  }
  const double scale = inTime ? 1.0 : (double)n;
  for (int k = 0; k < n; k++) {
    outr[k] = xr[k] * scale;
    outi[k] = xi[k] * scale;
  }
}

bool pow2(int n) { return n >= 4 && (n & (n - 1)) == 0; }

}  // namespace

extern "C" {

// computeGreensFunction of a Chi2PDC medium (inTimeDomain=false, runPump=true, normalize=false, one
// mode): the linear pump grid from the envelope (src/_NonlinearMedium.cpp:225-250, constant intensity
// profile when strength is NULL), then the 2N impulse propagations over `threads` std::threads, then C
// and S transposed and block-shifted (src/_NonlinearMedium.cpp:263-375).
//   envelope: N complex (interleaved); dispPump, dispSign: N; poling: nZ per-step orientations;
//   nlStepIm: nlStep = i nlStepIm; strength: nZStepsP row factors or NULL; C, S: N x N complex.
// Returns 0, or -1 for a grid that is not a power of two or fewer than two z steps.
int nlmcpu_chi2pdc_green(int n, int nz, int nzp, double dz, double dzp, const double* envelope, const double* dispPump,
                         const double* dispSign, const double* poling, double nlStepIm, double diffBeta0,
                         const double* strength, int threads, double* C, double* S) {
  if (!pow2(n) || nz < 2) return -1;
  PDC P;
  build_medium(P.md, n, nz, dz, dispSign);
  // pump grid: row 0 the envelope, row i = IFFT(FFT(env) exp(i (i dzp) D))
  P.pr.assign((size_t)nzp * n, 0.0);
  P.pi.assign((size_t)nzp * n, 0.0);
  {
    std::vector<double> fr(n), fi(n), tr(n), ti(n), rr(n), ri(n);
    for (int k = 0; k < n; k++) {
      fr[k] = envelope[2 * k];
      fi[k] = envelope[2 * k + 1];
      P.pr[k] = fr[k];
      P.pi[k] = fi[k];
    }
    fft<false>(P.md.plan, fr.data(), fi.data(), tr.data(), ti.data());
    for (int row = 1; row < nzp; row++) {
      for (int k = 0; k < n; k++) {
        const cd e = std::exp(cd(0, (row * dzp) * dispPump[k]));
        rr[k] = (fr[k] * e.real() - fi[k] * e.imag()) / n;
        ri[k] = (fr[k] * e.imag() + fi[k] * e.real()) / n;
      }
      fft<true>(P.md.plan, rr.data(), ri.data(), tr.data(), ti.data());
      std::memcpy(&P.pr[(size_t)row * n], rr.data(), sizeof(double) * n);
      std::memcpy(&P.pi[(size_t)row * n], ri.data(), sizeof(double) * n);
    }
    if (strength)
      for (int row = 0; row < nzp; row++)
        for (int k = 0; k < n; k++) {
          P.pr[(size_t)row * n + k] *= strength[row];
          P.pi[(size_t)row * n + k] *= strength[row];
        }
  }
  const cd nl(0.0, nlStepIm);
  P.c.resize((size_t)(nz > 1 ? nz - 1 : 0) * 3);
  for (int i = 1; i < nz; i++) {
    const double prev = poling[i - 1], cur = poling[i];
    P.c[(size_t)(i - 1) * 3 + 0] = prev * nl * std::exp(cd(0, diffBeta0 * ((i - 1) * dz)));
    P.c[(size_t)(i - 1) * 3 + 1] = 0.5 * (prev + cur) * nl * std::exp(cd(0, diffBeta0 * ((i - 0.5) * dz)));
    P.c[(size_t)(i - 1) * 3 + 2] = cur * nl * std::exp(cd(0, diffBeta0 * (i * dz)));
  }
  const int h = n / 2;
  std::memset(C, 0, sizeof(double) * 2 * (size_t)n * n);
  std::memset(S, 0, sizeof(double) * 2 * (size_t)n * n);
  // contiguous ranges of bins, both propagations of a bin in one thread (they fill the same column)
  parallel_ranges(n, threads, [&](int, long long begin, long long end) {
    Work w(n);
    std::vector<double> inr(n), ini(n), o1r(n), o1i(n), oir(n), oii(n);
    for (long long b = begin; b < end; b++) {
      const int bin = (int)b;
      std::fill(inr.begin(), inr.end(), 0.0);
      std::fill(ini.begin(), ini.end(), 0.0);
      inr[bin] = 1.0;
      pdc_propagate(P, w, inr.data(), ini.data(), o1r.data(), o1i.data());
      inr[bin] = 0.0;
      ini[bin] = 1.0;
      pdc_propagate(P, w, inr.data(), ini.data(), oir.data(), oii.data());
      // row `bin` of the pre-transpose matrices: C = 0.5 out(1) - 0.5 i out(i), S = 0.5 out(1) + 0.5 i out(i);
      // element (bin, o) lands at ((o + N/2) mod N, (bin + N/2) mod N) after the transpose and fftshift2
      const int col = (bin + h) % n;
      for (int o = 0; o < n; o++) {
        const size_t idx = 2 * ((size_t)((o + h) % n) * n + col);
        C[idx] = 0.5 * o1r[o] + 0.5 * oii[o];
        C[idx + 1] = 0.5 * o1i[o] - 0.5 * oir[o];
        S[idx] = 0.5 * o1r[o] - 0.5 * oii[o];
        S[idx + 1] = 0.5 * o1i[o] + 0.5 * oir[o];
      }
    }
  });
  return 0;
}

// Impulse propagations [start, start + count) of the Green's function above (instance = 2 bin + {0: 1,
// 1: i}), output spectra in out (count x N complex): the sampled form for timing a fixed amount of work.
int nlmcpu_chi2pdc_impulses(int n, int nz, int nzp, double dz, double dzp, const double* pumpTime,
                            const double* dispSign, const double* poling, double nlStepIm, double diffBeta0,
                            long long start, long long count, int threads, double* out) {
  if (!pow2(n) || nz < 2) return -1;
  PDC P;
  build_medium(P.md, n, nz, dz, dispSign);
  P.pr.resize((size_t)nzp * n);
  P.pi.resize((size_t)nzp * n);
  for (size_t k = 0; k < (size_t)nzp * n; k++) {
    P.pr[k] = pumpTime[2 * k];
    P.pi[k] = pumpTime[2 * k + 1];
  }
  const cd nl(0.0, nlStepIm);
  P.c.resize((size_t)(nz > 1 ? nz - 1 : 0) * 3);
  for (int i = 1; i < nz; i++) {
    const double prev = poling[i - 1], cur = poling[i];
    P.c[(size_t)(i - 1) * 3 + 0] = prev * nl * std::exp(cd(0, diffBeta0 * ((i - 1) * dz)));
    P.c[(size_t)(i - 1) * 3 + 1] = 0.5 * (prev + cur) * nl * std::exp(cd(0, diffBeta0 * ((i - 0.5) * dz)));
    P.c[(size_t)(i - 1) * 3 + 2] = cur * nl * std::exp(cd(0, diffBeta0 * (i * dz)));
  }
  parallel_ranges(count, threads, [&](int, long long begin, long long end) {
    Work w(n);
    std::vector<double> inr(n), ini(n), outr(n), outi(n);
    for (long long q = begin; q < end; q++) {
      const long long inst = start + q;
      const int bin = (int)((inst >> 1) % n);
      std::fill(inr.begin(), inr.end(), 0.0);
      std::fill(ini.begin(), ini.end(), 0.0);
      ((inst & 1) ? ini : inr)[bin] = 1.0;
      pdc_propagate(P, w, inr.data(), ini.data(), outr.data(), outi.data());
      for (int o = 0; o < n; o++) {
        out[2 * ((size_t)q * n + o)] = outr[o];
        out[2 * ((size_t)q * n + o) + 1] = outi[o];
      }
    }
  });
  return 0;
}

// batchSignalSimulation of a Chi3GNLSE medium (src/_NonlinearMedium.cpp:378-444 with
// solvers/Chi3GNLSE.cpp:39-92): rows x N complex inputs (time or frequency domain), the last row of
// each propagation in the same domain.  raman: N complex R~ = FFT(R(t)); steep: N complex
// nlStep0 + nlStep1 omega; rel: (nZ-1) x 3 relative intensities at i-1, i-1/2, i.
int nlmcpu_gnlse_batch(int n, int nz, double dz, const double* dispSign, const double* raman, const double* steep,
                       const double* rel, long long rows, const double* in, int inTime, int threads, double* out) {
  if (!pow2(n) || nz < 2) return -1;
  GNLSE G;
  build_medium(G.md, n, nz, dz, dispSign);
  G.raman = Split(raman, n, 1.0 / n);
  G.steep = Split(steep, n, 1.0 / n);
  G.rel.assign(rel, rel + (size_t)(nz > 1 ? nz - 1 : 0) * 3);
  parallel_ranges(rows, threads, [&](int, long long begin, long long end) {
    Work w(n);
    std::vector<double> inr(n), ini(n), outr(n), outi(n);
    for (long long row = begin; row < end; row++) {
      for (int k = 0; k < n; k++) {
        inr[k] = in[2 * ((size_t)row * n + k)];
        ini[k] = in[2 * ((size_t)row * n + k) + 1];
      }
      gnlse_propagate(G, w, inr.data(), ini.data(), inTime != 0, outr.data(), outi.data());
      for (int k = 0; k < n; k++) {
        out[2 * ((size_t)row * n + k)] = outr[k];
        out[2 * ((size_t)row * n + k) + 1] = outi[k];
      }
    }
  });
  return 0;
}

// One Chi3GNLSE propagation (as nlmcpu_gnlse_batch, one row) that also records the spectrum after
// every `every`-th step: rec holds floor((nZ-2) / every) rows of N complex values, the rows
// every, 2 every, ... of the reference's full signalFreq grid (src/_NonlinearMedium.hpp:195-233 with
// optimized = false).  out: the last row, in the input's domain.
int nlmcpu_gnlse_record(int n, int nz, double dz, const double* dispSign, const double* raman, const double* steep,
                        const double* rel, const double* in, int inTime, int every, double* rec, double* out) {
  if (!pow2(n) || nz < 2 || every < 1) return -1;
  GNLSE G;
  build_medium(G.md, n, nz, dz, dispSign);
  G.raman = Split(raman, n, 1.0 / n);
  G.steep = Split(steep, n, 1.0 / n);
  G.rel.assign(rel, rel + (size_t)(nz - 1) * 3);
  Work w(n);
  std::vector<double> inr(n), ini(n), outr(n), outi(n);
  for (int k = 0; k < n; k++) {
    inr[k] = in[2 * k];
    ini[k] = in[2 * k + 1];
  }
  gnlse_propagate(G, w, inr.data(), ini.data(), inTime != 0, outr.data(), outi.data(), rec, every);
  for (int k = 0; k < n; k++) {
    out[2 * k] = outr[k];
    out[2 * k + 1] = outi[k];
  }
  return 0;
}

}  // extern "C"
