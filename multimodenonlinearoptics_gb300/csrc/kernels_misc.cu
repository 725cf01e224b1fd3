// kernels_misc.cu -- pump generation, batched row transforms, the Green's-function
// epilogue, the Cascade composition GEMM, and the kernel registry.
#include <mutex>
#include <vector>

#include "nlm_device.cuh"
#include "nlm_kernels.h"
#include "nlm_solvers.cuh"

namespace nlm {

void add_kernels_linear(std::vector<KernelEntry>& t);
void add_kernels_direct_a(std::vector<KernelEntry>& t);
void add_kernels_direct_b(std::vector<KernelEntry>& t);
void add_kernels_gnlse(std::vector<KernelEntry>& t);
void add_kernels_adjoint(std::vector<KernelEntry>& t);
void add_kernels_ragged(std::vector<KernelEntry>& t);
void add_kernels_adjoint_gnlse(std::vector<KernelEntry>& t);
void add_kernels_ff(std::vector<KernelEntry>& t);
void add_kernels_direct_c(std::vector<KernelEntry>& t);
void add_kernels_cluster(std::vector<KernelEntry>& t);
void add_kernels_cluster_b(std::vector<KernelEntry>& t);
void add_kernels_spread(std::vector<KernelEntry>& t);
void add_kernels_spread_b(std::vector<KernelEntry>& t);
void add_kernels_adjoint_spread(std::vector<KernelEntry>& t);
void add_kernels_cluster_gnlse(std::vector<KernelEntry>& t);
void add_kernels_adjoint_gnlse_cluster(std::vector<KernelEntry>& t);
void add_kernels_adjoint_cluster(std::vector<KernelEntry>& t);
void add_kernels_gen_a(std::vector<KernelEntry>& t);
void add_kernels_gen_b(std::vector<KernelEntry>& t);
void add_kernels_gen_c(std::vector<KernelEntry>& t);
void add_kernels_gen_d(std::vector<KernelEntry>& t);
void add_kernels_gen_e(std::vector<KernelEntry>& t);
void add_kernels_spread_fused(std::vector<KernelEntry>& t);
void add_kernels_spread_w16(std::vector<KernelEntry>& t);
void add_kernels_gnlse_spread(std::vector<KernelEntry>& t);
void add_kernels_adjoint_gnlse_spread(std::vector<KernelEntry>& t);

const KernelEntry* kernel_table(int* count) {
  static std::vector<KernelEntry> table;
  static std::once_flag once;
  std::call_once(once, [] {
    add_kernels_linear(table);
    add_kernels_direct_a(table);
    add_kernels_direct_b(table);
    add_kernels_gnlse(table);
    add_kernels_adjoint(table);
    add_kernels_ragged(table);
    add_kernels_adjoint_gnlse(table);
    add_kernels_ff(table);
    add_kernels_direct_c(table);
    add_kernels_cluster(table);
    add_kernels_cluster_b(table);
    add_kernels_spread(table);
    add_kernels_spread_b(table);
    add_kernels_adjoint_spread(table);
    add_kernels_cluster_gnlse(table);
    add_kernels_adjoint_gnlse_cluster(table);
    add_kernels_adjoint_cluster(table);
    add_kernels_gen_a(table);
    add_kernels_gen_b(table);
    add_kernels_gen_c(table);
    add_kernels_gen_d(table);
    add_kernels_gen_e(table);
    add_kernels_spread_fused(table);
    add_kernels_spread_w16(table);
    add_kernels_gnlse_spread(table);
    add_kernels_adjoint_gnlse_spread(table);
  });
  *count = (int)table.size();
  return table.data();
}

// ------------------------------------------------------------------------------------------
// Batched transforms of contiguous rows: out = scale * FFT(in) [* post] (power-of-two N)
// ------------------------------------------------------------------------------------------
template <int R, bool INV, bool GEN = false>
__global__ void __launch_bounds__(512) k_fft_rows(const double2* __restrict__ in, double2* __restrict__ out,
                                                  long long rows, FFTPlanH plan, const double2* __restrict__ tw,
                                                  double scale, const double2* __restrict__ post, int rpc) {
  extern __shared__ double2 smem[];
  const int N = plan.N, T = plan.T;
  const int g = threadIdx.x / T, j = threadIdx.x - g * T;
  double2* buf = smem + (long long)g * N;
  for (long long base = (long long)blockIdx.x * rpc; base < rows; base += (long long)gridDim.x * rpc) {
    const long long row = base + g;
    const bool active = row < rows;
    double2 x[R];
#pragma unroll
    for (int v = 0; v < R; v++) x[v] = (active && (!GEN || j + v * T < N)) ? in[row * N + j + v * T] : czero();
    fft_any<R, INV, GEN>(x, buf, tw, plan, j);
    if (active) {
#pragma unroll
      for (int v = 0; v < R; v++) {
        if (GEN && j + v * T >= N) continue;
        double2 y = cscale(x[v], scale);
        if (post) y = cmul(y, post[j + v * T]);
        out[row * N + j + v * T] = y;
      }
    }
    __syncthreads();
  }
}

// Direct O(N^2) DFT of rows for grids that are not a power of two (or smaller than R).
template <bool INV>
__global__ void k_dft_rows(const double2* __restrict__ in, double2* __restrict__ out, long long rows, int N,
                           const double2* __restrict__ tw, double scale, const double2* __restrict__ post) {
  const long long total = rows * N;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long row = idx / N;
    const int k = (int)(idx - row * N);
    const double2* x = in + row * N;
    double2 acc = czero();
    long long m = 0;
    for (int t = 0; t < N; t++) {
      const double2 w = tw[m];
      acc = cadd(acc, INV ? cmulc(x[t], w) : cmul(x[t], w));
      m += k;
      if (m >= N) m -= N;
    }
    acc = cscale(acc, scale);
    if (post) acc = cmul(acc, post[k]);
    out[idx] = acc;   // in != out is required
  }
}

static int sm_count() {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  return sms;
}

static cudaError_t smem_optin(const void* fn) {
  static std::mutex mu;
  static std::vector<const void*> done;
  std::lock_guard<std::mutex> lock(mu);
  for (const void* f : done)
    if (f == fn) return cudaSuccess;
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, fn);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
  if (e == cudaSuccess) done.push_back(fn);
  return e;
}

template <int R, bool INV, bool GEN>
static cudaError_t fft_rows_R(const double2* in, double2* out, long long rows, const FFTPlanH& plan,
                              const double2* tw, double scale, const double2* post, cudaStream_t s) {
  const int T = plan.T;
  int rpc = T >= 128 ? 1 : 128 / T;
  if (rpc > rows) rpc = (int)rows;
  if (rpc < 1) rpc = 1;
  const size_t smem = (size_t)rpc * plan.N * sizeof(double2);
  const void* fn = (const void*)k_fft_rows<R, INV, GEN>;
  cudaError_t e = smem_optin(fn);
  if (e != cudaSuccess) return e;
  long long groups = (rows + rpc - 1) / rpc;
  int grid = (int)(groups < 8LL * sm_count() ? groups : 8LL * sm_count());
  if (grid < 1) grid = 1;
  k_fft_rows<R, INV, GEN><<<grid, T * rpc, smem, s>>>(in, out, rows, plan, tw, scale, post, rpc);
  return cudaGetLastError();
}

template <bool GEN>
static cudaError_t fft_rows_plan(const double2* in, double2* out, long long rows, const FFTPlanH& plan,
                                 const double2* tw, bool inverse, double scale, const double2* postMul,
                                 cudaStream_t s) {
  if (plan.R == 8) return inverse ? fft_rows_R<8, true, GEN>(in, out, rows, plan, tw, scale, postMul, s)
                                  : fft_rows_R<8, false, GEN>(in, out, rows, plan, tw, scale, postMul, s);
  if (plan.R == 16) return inverse ? fft_rows_R<16, true, GEN>(in, out, rows, plan, tw, scale, postMul, s)
                                   : fft_rows_R<16, false, GEN>(in, out, rows, plan, tw, scale, postMul, s);
  return cudaErrorInvalidValue;
}

cudaError_t launch_fft_rows(const double2* in, double2* out, long long rows, const FFTPlanH& plan,
                            const double2* tw, bool inverse, double scale, const double2* postMul,
                            cudaStream_t s) {
  if (rows <= 0) return cudaSuccess;
  const int N = plan.N;
  if (plan.T < 1 || plan.T > 512 || N > kMaxFFT) {
    // grids no transform plan takes: the direct O(N^2) DFT of each row
    if (in == out) return cudaErrorInvalidValue;
    const long long total = rows * N;
    int grid = (int)((total + 255) / 256);
    if (grid > 16 * sm_count()) grid = 16 * sm_count();
    if (inverse) k_dft_rows<true><<<grid, 256, 0, s>>>(in, out, rows, N, tw, scale, postMul);
    else k_dft_rows<false><<<grid, 256, 0, s>>>(in, out, rows, N, tw, scale, postMul);
    return cudaGetLastError();
  }
  return plan.gen ? fft_rows_plan<true>(in, out, rows, plan, tw, inverse, scale, postMul, s)
                  : fft_rows_plan<false>(in, out, rows, plan, tw, inverse, scale, postMul, s);
}

// ------------------------------------------------------------------------------------------
// Linear pump (src/_NonlinearMedium.cpp:230-233): row i = F[env] * exp(i * (i dzp) * D)
// ------------------------------------------------------------------------------------------
__global__ void k_pump_linear(const double2* __restrict__ f0, const double* __restrict__ disp, double dzp,
                              int nRows, int N, double2* __restrict__ pf) {
  const long long total = (long long)nRows * N;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(idx / N);
    const int t = (int)(idx - (long long)i * N);
    if (i == 0) {
      pf[idx] = f0[t];
      continue;
    }
    const double th = ((double)i * dzp) * disp[t];
    double sn, cs;
    sincos(th, &sn, &cs);
    pf[idx] = cmul(f0[t], make_double2(cs, sn));
  }
}

cudaError_t launch_pump_linear(const double2* freq0, const double* disp, double dzp, int nRows, int N,
                               double2* pumpFreq, cudaStream_t s) {
  const long long total = (long long)nRows * N;
  int grid = (int)((total + 255) / 256);
  if (grid > 32 * sm_count()) grid = 32 * sm_count();
  if (grid < 1) grid = 1;
  k_pump_linear<<<grid, 256, 0, s>>>(freq0, disp, dzp, nRows, N, pumpFreq);
  return cudaGetLastError();
}

__global__ void k_scale_rows(double2* a, const double* __restrict__ scale, int nRows, int N) {
  const long long total = (long long)nRows * N;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x)
    a[idx] = cscale(a[idx], scale[idx / N]);
}

cudaError_t launch_scale_rows(double2* a, const double* scale, int nRows, int N, cudaStream_t s) {
  const long long total = (long long)nRows * N;
  int grid = (int)((total + 255) / 256);
  if (grid > 32 * sm_count()) grid = 32 * sm_count();
  if (grid < 1) grid = 1;
  k_scale_rows<<<grid, 256, 0, s>>>(a, scale, nRows, N);
  return cudaGetLastError();
}

// ------------------------------------------------------------------------------------------
// Chi3 pump: sequential self-phase-modulation march on one CTA (solvers/Chi3.cpp:41-70)
// ------------------------------------------------------------------------------------------
// GEN: the general plan (padded ownership): points j + v*T at or past N are neither loaded nor stored.
template <int R, bool GEN = false>
__global__ void __launch_bounds__(512) k_pump_chi3(double2* __restrict__ pf, double2* __restrict__ pt,
                                                   const double2* __restrict__ env, const double2* __restrict__ halfP,
                                                   const double2* __restrict__ dstepP, const double2* __restrict__ backP,
                                                   const double2* __restrict__ rel, int nRows, FFTPlanH plan,
                                                   const double2* __restrict__ tw) {
  extern __shared__ double2 buf[];
  const int N = plan.N, T = plan.T, j = threadIdx.x;
  const double invN = 1.0 / N;
  auto own = [&](int v) { return !GEN || j + v * T < N; };
  double2 x[R];
#pragma unroll
  for (int v = 0; v < R; v++) x[v] = own(v) ? env[j + v * T] : czero();
  fft_any<R, false, GEN>(x, buf, tw, plan, j);
#pragma unroll
  for (int v = 0; v < R; v++) {
    if (!own(v)) continue;
    x[v] = cmul(x[v], halfP[j + v * T]);
    pf[j + v * T] = x[v];
  }
  fft_any<R, true, GEN>(x, buf, tw, plan, j);
#pragma unroll
  for (int v = 0; v < R; v++) {
    if (!own(v)) continue;
    x[v] = cscale(x[v], invN);
    pt[j + v * T] = x[v];
  }
  for (int i = 1; i < nRows; i++) {
    const double2 r = rel[i - 1];
#pragma unroll
    for (int v = 0; v < R; v++) {
      const double a2 = cabs2(x[v]);
      x[v] = cmul(x[v], spm_factor(r.x * a2, r.y * a2));
    }
    fft_any<R, false, GEN>(x, buf, tw, plan, j);
#pragma unroll
    for (int v = 0; v < R; v++) {
      if (!own(v)) continue;
      x[v] = cmul(x[v], dstepP[j + v * T]);
      pf[(long long)i * N + j + v * T] = x[v];
    }
    fft_any<R, true, GEN>(x, buf, tw, plan, j);
#pragma unroll
    for (int v = 0; v < R; v++) {
      if (!own(v)) continue;
      x[v] = cscale(x[v], invN);
      pt[(long long)i * N + j + v * T] = x[v];
    }
  }
  // last row: undo half of the last pump dispersion step
  __syncthreads();
  const long long last = (long long)(nRows - 1) * N;
#pragma unroll
  for (int v = 0; v < R; v++) {
    if (!own(v)) {
      x[v] = czero();
      continue;
    }
    x[v] = cmul(pf[last + j + v * T], backP[j + v * T]);
    pf[last + j + v * T] = x[v];
  }
  fft_any<R, true, GEN>(x, buf, tw, plan, j);
#pragma unroll
  for (int v = 0; v < R; v++)
    if (own(v)) pt[last + j + v * T] = cscale(x[v], invN);
}

template <int R, bool GEN>
static cudaError_t pump_chi3_R(double2* pumpFreq, double2* pumpTime, const double2* env, const double2* halfP,
                               const double2* dstepP, const double2* backP, const double2* rel, int nRows,
                               const FFTPlanH& plan, const double2* tw, cudaStream_t s) {
  const size_t smem = (size_t)plan.N * sizeof(double2);
  cudaError_t e = smem_optin((const void*)k_pump_chi3<R, GEN>);
  if (e != cudaSuccess) return e;
  k_pump_chi3<R, GEN><<<1, plan.T, smem, s>>>(pumpFreq, pumpTime, env, halfP, dstepP, backP, rel, nRows, plan, tw);
  return cudaGetLastError();
}

cudaError_t launch_pump_chi3(double2* pumpFreq, double2* pumpTime, const double2* env, const double2* halfP,
                             const double2* dstepP, const double2* backP, const double2* rel, int nRows,
                             const FFTPlanH& plan, const double2* tw, cudaStream_t s) {
  if (plan.T < 1 || plan.T > 512) return cudaErrorInvalidValue;
  switch (plan.R * 2 + (plan.gen ? 1 : 0)) {
    case 8: return pump_chi3_R<4, false>(pumpFreq, pumpTime, env, halfP, dstepP, backP, rel, nRows, plan, tw, s);
    case 16: return pump_chi3_R<8, false>(pumpFreq, pumpTime, env, halfP, dstepP, backP, rel, nRows, plan, tw, s);
    case 32: return pump_chi3_R<16, false>(pumpFreq, pumpTime, env, halfP, dstepP, backP, rel, nRows, plan, tw, s);
    case 9: return pump_chi3_R<4, true>(pumpFreq, pumpTime, env, halfP, dstepP, backP, rel, nRows, plan, tw, s);
    case 17: return pump_chi3_R<8, true>(pumpFreq, pumpTime, env, halfP, dstepP, backP, rel, nRows, plan, tw, s);
    case 33: return pump_chi3_R<16, true>(pumpFreq, pumpTime, env, halfP, dstepP, backP, rel, nRows, plan, tw, s);
    default: return cudaErrorInvalidValue;
  }
}

// ------------------------------------------------------------------------------------------
// Green's-function epilogue (src/_NonlinearMedium.cpp:329-345, 360-372): from the raw outputs
// of the impulse pair (1, i) of every input bin build C and S, transpose, block-fftshift and
// normalise.  flags per (om, im) block: bit 0 = shift, bit 1 = multiply by blockScale.
// ------------------------------------------------------------------------------------------
__global__ void k_green_epilogue(const double2* __restrict__ raw, long long rawStride, int N, int nIn, int nOut,
                                 const double2* __restrict__ blockScale, const uint8_t* __restrict__ flags,
                                 double2* __restrict__ C, double2* __restrict__ S) {
  __shared__ double2 t1[32][33];
  __shared__ double2 ti[32][33];
  const long long rows = (long long)nOut * N, cols = (long long)nIn * N;
  const long long r0 = (long long)blockIdx.y * 32, c0 = (long long)blockIdx.x * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int half = N / 2;
  // phase 1: gather along t (contiguous in the raw rows)
  for (int cc = ty; cc < 32; cc += 8) {
    const long long r = r0 + tx, c = c0 + cc;
    double2 v1 = czero(), vi = czero();
    if (r < rows && c < cols) {
      const int om = (int)(r / N), tp = (int)(r - (long long)om * N);
      const int im = (int)(c / N), bp = (int)(c - (long long)im * N);
      const uint8_t f = flags[om * nIn + im];
      const int t = (f & 1) ? (tp + half) % N : tp;
      const int b = (f & 1) ? (bp + half) % N : bp;
      const long long inst = ((long long)im * N + b) * 2;
      v1 = raw[inst * rawStride + (long long)om * N + t];
      vi = raw[(inst + 1) * rawStride + (long long)om * N + t];
    }
    t1[cc][tx] = v1;
    ti[cc][tx] = vi;
  }
  __syncthreads();
  // phase 2: write along c
  for (int rr = ty; rr < 32; rr += 8) {
    const long long r = r0 + rr, c = c0 + tx;
    if (r >= rows || c >= cols) continue;
    const double2 v1 = t1[tx][rr], vi = ti[tx][rr];
    // C = 0.5 out1 - 0.5i out_i ; S = 0.5 out1 + 0.5i out_i
    const double2 a = make_double2(0.5 * v1.x, 0.5 * v1.y);
    const double2 b = make_double2(-0.5 * vi.y, 0.5 * vi.x);
    double2 cv = csub(a, b), sv = cadd(a, b);
    const int om = (int)(r / N), im = (int)(c / N);
    const uint8_t f = flags[om * nIn + im];
    if (f & 2) {
      const double2 sc = blockScale[om * nIn + im];
      cv = cmul(cv, sc);
      sv = cmul(sv, sc);
    }
    C[r * cols + c] = cv;
    S[r * cols + c] = sv;
  }
}

cudaError_t launch_green_epilogue(const double2* raw, long long rawStride, int N, int nIn, int nOut,
                                  const double2* blockScale, const uint8_t* blockShift, double2* C,
                                  double2* S, cudaStream_t s) {
  const long long rows = (long long)nOut * N, cols = (long long)nIn * N;
  dim3 grid((unsigned)((cols + 31) / 32), (unsigned)((rows + 31) / 32));
  k_green_epilogue<<<grid, dim3(32, 8), 0, s>>>(raw, rawStride, N, nIn, nOut, blockScale, blockShift, C, S);
  return cudaGetLastError();
}

// ------------------------------------------------------------------------------------------
// setPump(other) (src/_NonlinearMedium.cpp:519-531): interpolated copy of another medium's
// signal spectrum with the frame-of-reference phase.
// ------------------------------------------------------------------------------------------
__global__ void k_pump_from(const double2* __restrict__ src, int otherRows, double ratio, double otherDz,
                            const double* __restrict__ dispP, const double* __restrict__ dispO, double dzp,
                            double b1delay, const double* __restrict__ omega, int nRowsP, int N, double z,
                            double otherZ, double2* __restrict__ pf) {
  const long long total = (long long)nRowsP * N;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(idx / N);
    const int t = (int)(idx - (long long)i * N);
    const double dl = b1delay * omega[t];
    double2 val;
    double th;
    if (i < nRowsP - 1) {
      const double jf = i * ratio;
      const int jj = (int)jf;
      const double frac = jf - jj;
      const double2 a = src[(long long)jj * N + t], b = src[(long long)(jj + 1) * N + t];
      val = make_double2((1 - frac) * a.x + frac * b.x, (1 - frac) * a.y + frac * b.y);
      th = (((double)i * dzp) * dispP[t] - ((jf + 0.5) * otherDz) * dispO[t]) + dl;
    } else {
      val = src[(long long)(otherRows - 1) * N + t];
      th = (z * dispP[t] - otherZ * dispO[t]) + dl;
    }
    double sn, cs;
    sincos(th, &sn, &cs);
    pf[idx] = cmul(val, make_double2(cs, sn));
  }
}

cudaError_t launch_pump_from(const double2* otherSignalFreq, int otherRows, double ratio, double otherDz,
                             const double* dispPump, const double* otherDispSign, double dzp, double b1delay,
                             const double* omega, int nRowsP, int N, double z, double otherZ, double2* pumpFreq,
                             cudaStream_t s) {
  const long long total = (long long)nRowsP * N;
  int grid = (int)((total + 255) / 256);
  if (grid > 32 * sm_count()) grid = 32 * sm_count();
  if (grid < 1) grid = 1;
  k_pump_from<<<grid, 256, 0, s>>>(otherSignalFreq, otherRows, ratio, otherDz, dispPump, otherDispSign, dzp, b1delay,
                                    omega, nRowsP, N, z, otherZ, pumpFreq);
  return cudaGetLastError();
}

// ------------------------------------------------------------------------------------------
// Cascade composition (src/Cascade.cpp:128-129):
//   Cout = Ci C + Si conj(S),  Sout = Ci S + Si conj(C)     (row-major, FP64 complex)
// ------------------------------------------------------------------------------------------
// 32 x 32 output tile per CTA of 16 x 16 threads, each thread a 2 x 2 register tile of both outputs
// (rows ty, ty + 16; columns tx, tx + 16): per k, 8 shared-memory loads feed 64 FMAs, and the 16
// accumulator chains of a thread are independent.
__global__ void __launch_bounds__(256) k_cgemm_compose(const double2* __restrict__ Ci, const double2* __restrict__ Si,
                                                       const double2* __restrict__ C, const double2* __restrict__ S,
                                                       int rows, int inner, int cols, double2* __restrict__ Co,
                                                       double2* __restrict__ So) {
  constexpr int TM = 32, TK = 16;
  __shared__ double2 aC[TM][TK + 1], aS[TM][TK + 1], bC[TK][TM + 1], bS[TK][TM + 1];
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * 16 + tx;
  const int r0 = blockIdx.y * TM, c0 = blockIdx.x * TM;
  double2 accC[2][2], accS[2][2];
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int b = 0; b < 2; b++) accC[a][b] = accS[a][b] = czero();
  for (int k0 = 0; k0 < inner; k0 += TK) {
    // A tiles: 32 rows x 16 k; B tiles: 16 k x 32 columns (two elements of each per thread)
#pragma unroll
    for (int e = 0; e < 2; e++) {
      const int q = tid + e * 256;
      const int ar = q / TK, ak = q - ar * TK;
      const int r = r0 + ar, ka = k0 + ak;
      const bool inA = r < rows && ka < inner;
      aC[ar][ak] = inA ? Ci[(long long)r * inner + ka] : czero();
      aS[ar][ak] = inA ? Si[(long long)r * inner + ka] : czero();
      const int bk = q / TM, bc = q - bk * TM;
      const int kb = k0 + bk, c = c0 + bc;
      const bool inB = kb < inner && c < cols;
      bC[bk][bc] = inB ? C[(long long)kb * cols + c] : czero();
      bS[bk][bc] = inB ? S[(long long)kb * cols + c] : czero();
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < TK; k++) {
      double2 ci[2], si[2], cc[2], ss[2];
#pragma unroll
      for (int a = 0; a < 2; a++) {
        ci[a] = aC[ty + 16 * a][k];
        si[a] = aS[ty + 16 * a][k];
        cc[a] = bC[k][tx + 16 * a];
        ss[a] = bS[k][tx + 16 * a];
      }
#pragma unroll
      for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 2; b++) {
          // Co += Ci C + Si conj(S), So += Ci S + Si conj(C)
          accC[a][b].x = fma(ci[a].x, cc[b].x, fma(-ci[a].y, cc[b].y, fma(si[a].x, ss[b].x, fma(si[a].y, ss[b].y, accC[a][b].x))));
          accC[a][b].y = fma(ci[a].x, cc[b].y, fma(ci[a].y, cc[b].x, fma(si[a].y, ss[b].x, fma(-si[a].x, ss[b].y, accC[a][b].y))));
          accS[a][b].x = fma(ci[a].x, ss[b].x, fma(-ci[a].y, ss[b].y, fma(si[a].x, cc[b].x, fma(si[a].y, cc[b].y, accS[a][b].x))));
          accS[a][b].y = fma(ci[a].x, ss[b].y, fma(ci[a].y, ss[b].x, fma(si[a].y, cc[b].x, fma(-si[a].x, cc[b].y, accS[a][b].y))));
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int b = 0; b < 2; b++) {
      const int r = r0 + ty + 16 * a, c = c0 + tx + 16 * b;
      if (r < rows && c < cols) {
        Co[(long long)r * cols + c] = accC[a][b];
        So[(long long)r * cols + c] = accS[a][b];
      }
    }
}

cudaError_t launch_cgemm_compose(const double2* Ci, const double2* Si, const double2* C, const double2* S, int rows,
                                 int inner, int cols, double2* Cout, double2* Sout, cudaStream_t s) {
  dim3 grid((cols + 31) / 32, (rows + 31) / 32);
  k_cgemm_compose<<<grid, dim3(16, 16), 0, s>>>(Ci, Si, C, S, rows, inner, cols, Cout, Sout);
  return cudaGetLastError();
}

// ------------------------------------------------------------------------------------------
// FP64 pipe peak: independent DFMA chains, used as the roofline denominator of the benchmark.
// ------------------------------------------------------------------------------------------
__global__ void k_fp64_peak(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int u = 0; u < 4; u++) {
      x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
      x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

cudaError_t launch_fp64_peak(double* out, int iters, int blocks, int threads, cudaStream_t s) {
  k_fp64_peak<<<blocks, threads, 0, s>>>(out, iters, 0.999999, 1e-7);
  return cudaGetLastError();
}

// FP64 tensor-core (DMMA) peak: independent m16n8k16 f64 MMAs per warp (4096 FMAs each).  Measures
// what a DFT-as-GEMM schedule could get from the tensor cores in FP64 on this device.
__global__ void k_fp64_mma_peak(double* out, int iters, double a0, double b0) {
  double a[8], b[4], c[4][4];
#pragma unroll
  for (int q = 0; q < 8; q++) a[q] = a0 + 1e-9 * (threadIdx.x + q);
#pragma unroll
  for (int q = 0; q < 4; q++) b[q] = b0 - 1e-9 * q;
#pragma unroll
  for (int u = 0; u < 4; u++)
#pragma unroll
    for (int q = 0; q < 4; q++) c[u][q] = 0.0;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int u = 0; u < 4; u++) {
      asm volatile(
          "mma.sync.aligned.m16n8k16.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5,%6,%7,%8,%9,%10,%11}, "
          "{%12,%13,%14,%15}, {%0,%1,%2,%3};"
          : "+d"(c[u][0]), "+d"(c[u][1]), "+d"(c[u][2]), "+d"(c[u][3])
          : "d"(a[0]), "d"(a[1]), "d"(a[2]), "d"(a[3]), "d"(a[4]), "d"(a[5]), "d"(a[6]), "d"(a[7]), "d"(b[0]),
            "d"(b[1]), "d"(b[2]), "d"(b[3]));
    }
  }
  double acc = 0.0;
#pragma unroll
  for (int u = 0; u < 4; u++)
#pragma unroll
    for (int q = 0; q < 4; q++) acc += c[u][q];
  out[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

cudaError_t launch_fp64_mma_peak(double* out, int iters, int blocks, int threads, cudaStream_t s) {
  k_fp64_mma_peak<<<blocks, threads, 0, s>>>(out, iters, 1e-3, 1e-3);
  return cudaGetLastError();
}

}  // namespace nlm
