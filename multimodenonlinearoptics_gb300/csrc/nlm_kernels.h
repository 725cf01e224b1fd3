// nlm_kernels.h -- launch interface between the host engine (engine.h) and the kernels.
// Plain C++ (no device code): included by both nvcc and g++ translation units.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace nlm {

constexpr int kMaxModes = 4;
constexpr int kMaxPumps = 2;
constexpr int kMaxCoefs = 8;
constexpr int kMaxFFT = 8192;   // largest grid of the fused kernels
constexpr int kTablePad = 16;   // zeroed values after every per-point device table (padded ownership reads)

// Plan of an N-point transform held by T threads of R points each.  gen == 0: N a power of two and
// T = N / R, radix-8/4/2 passes on the register ownership (nlm_device.cuh, fft_regs).  gen == 1: any N,
// T = ceil(N / R) (thread j owns the points j + v T that are below N), passes of any radix through
// shared memory (fft_general).
struct FFTPlanH {
  int N, T, nPass;
  int radix[16];
  int gen;
  int R;   // points per thread the plan was made for
};

// Arguments of every propagation kernel (batched impulses, dense rows, one full grid).
struct PropArgs {
  FFTPlanH plan;          // mirrors nlm::FFTPlan
  int R;                  // points per thread per mode
  int nModes;             // signal modes
  int nZ;                 // nZSteps
  long long nInst;        // independent propagations in this launch
  long long instBase;     // global index of the launch's first propagation
  int ipc;                // propagations per CTA
  unsigned long long* work;  // zeroed work counter for dynamic scheduling of the groups; null: static
  // input description
  int inKind;             // 0: impulses (Green's function), 1: dense rows
  int inTime;             // inputs and outputs in the time domain
  const double2* in;      // dense rows
  long long inStride;     // complex elements between rows
  int inChannels;         // number of N-blocks per row
  int inputMode;          // mode receiving a single N-block
  int impModes[kMaxModes];// impulses: input mode of impulse group im = inst / (2N)
  // output description (last row of the selected modes)
  int nOut;
  int outModes[kMaxModes];
  double2* out;
  long long outStride;
  // point-wise tables (device)
  const double2* tw;      // N twiddles exp(-2 pi i m / N)
  const double2* dstep;   // [mode][N] dispStep / N
  const double2* dlast;   // [mode][N] dispStep * exp(-i dz/2 D) / N
  const double2* half;    // [mode][N] exp(+i dz/2 D) / N
  const double2* back;    // [mode][N] exp(-i dz/2 D) / N
  const double* prop;     // linear propagator [(nZ-1)][(2M)^2][N]
  const double2* pump;    // pumpTime [pump][nZStepsP][N]
  long long pumpStride;   // nZStepsP * N
  int nPumps;
  const double2* coef;    // [(nZ-1)][3][nCoef]
  int nCoef;
  // full grids of a single propagation (runSignalSimulation); null otherwise
  double2* gridF;         // [mode][nZ][N]
  double2* gridT;
  // checkpoints of the forward states for the adjoint: state s_i (time domain, all modes) is stored
  // at ckpt[((inst * ckN) + i / ckK) * nModes + m][N] when i % ckK == 0 and i < nZ - 1
  double2* ckpt;
  int ckK, ckN;
  // Chi3GNLSE adjoint forward on clusters: the stage inputs y_s and convolutions u2_s of every step
  // (time domain) at stages[((inst * (nZ - 1) + i - 1) * 8 + {s, 4 + s})][N]; null otherwise
  double2* stages;
  // Chi3GNLSE tables
  const double2* raman;   // ramanResponse / N
  const double2* steep;   // (nlStep0 + nlStep1 * omega) / N
  const double* relInt;   // [(nZ-1)][3] relative intensity at i-1, i-1/2, i
};

// Arguments of the reverse (adjoint) sweep.
struct AdjArgs {
  const double2* gout;   // [nInst][N]: dL/dRe X + i dL/dIm X of the output spectrum
  const double2* ckpt;   // forward checkpoints (PropArgs::ckpt layout)
  int K, nCk;            // checkpoint interval and count
  double2* seg;          // scratch [slot][K][N] for the recomputed states of one segment (K > 1)
  double2* ga;           // [(nZ-1)][3][N] accumulated gradients of the stage factors a_s = c_s P_s
  double2* gin;          // [nInst][N]: gradient with respect to the input spectrum
  int single;            // 1: a single instance, whose stage-factor gradients are stored without atomics
  // marching form (checkpoint interval 1 with the propagator matrices): the gradient after every
  // step's RK4, [nInst][nZ-1][N], for k_adj_stage_grads; null otherwise
  double2* gp;
};

// Registry of the propagation kernels.  The host engine launches them generically with
// cudaLaunchKernel(fn, grid, block, {&PropArgs[, &scratch]}, smem, stream).
enum KernelKind : int {
  kKindDirect = 0,     // k_propagate_direct<Solver, R>      key = solver id
  kKindLinear = 1,     // k_propagate_linear<M, R>           key = number of modes M
  kKindGnlse = 2,      // k_propagate_gnlse<R>               key = solver id (Chi3GNLSE); extra arg: scratch
  kKindBuildProp = 3,  // k_build_propagator<Solver>         key = solver id, R = 0
  kKindAdjoint = 4,    // k_adjoint_pdc<R>                   key = solver id; args (PropArgs, AdjArgs)
  kKindRagged = 5,     // k_propagate_ragged<Solver, R>      key = solver id; args (items, nItems, work)
  kKindLinearFF = 6,   // k_propagate_linear_ff<R, SMALL>    key = M + 10 SMALL; args (PropArgs, FFTables)
  kKindCluster = 7,    // k_propagate_cluster<Solver, C>     key = solver id, R = C; cluster launch
  kKindSpreadFused = 8 // k_propagate_spread<Solver, C, M>   key as kKindCluster (R = 1): modes transformed together
};

// Float-float copies (float4 {re.hi, re.lo, im.hi, im.lo} per complex value) of the tables of a
// single-mode linear propagation, for the double-float kernel on the FP32 pipes.
struct FFTables {
  const float4* tw;      // N twiddles
  const float4* dstep;   // [N]
  const float4* dlast;
  const float4* half;
  const float4* back;
  const float4* prop;    // [(nZ-1)][2][N]: pairs (M00, M01) and (M10, M11)
};
struct KernelEntry {
  int kind;
  int key;
  int R;
  const void* fn;
};
// All registered kernels (filled on first call).
const KernelEntry* kernel_table(int* count);
cudaError_t launch_fft_rows(const double2* in, double2* out, long long rows, const FFTPlanH& plan,
                            const double2* tw, bool inverse, double scale, const double2* postMul,
                            cudaStream_t s);
cudaError_t launch_pump_linear(const double2* freq0, const double* disp, double dzp, int nRows, int N,
                               double2* pumpFreq, cudaStream_t s);
cudaError_t launch_scale_rows(double2* a, const double* scale, int nRows, int N, cudaStream_t s);
// stage-factor gradients of every step and point from the marching form's stored gradients (rows
// summed): d.ga = sum over rows of the stage chain at (state before the step, gradient after it)
cudaError_t launch_adj_stage_grads(const PropArgs& a, const AdjArgs& d, int N, long long rows, cudaStream_t s);
cudaError_t launch_pump_chi3(double2* pumpFreq, double2* pumpTime, const double2* env, const double2* halfP,
                             const double2* dstepP, const double2* backP, const double2* rel, int nRows,
                             const FFTPlanH& plan, const double2* tw, cudaStream_t s);
// the same march over a 4-CTA cluster; localPlan is the (N/4)-point plan with four points per thread
cudaError_t launch_pump_chi3_cluster(double2* pumpFreq, double2* pumpTime, const double2* env, const double2* halfP,
                                     const double2* dstepP, const double2* backP, const double2* rel, int nRows,
                                     const FFTPlanH& localPlan, const double2* tw, cudaStream_t s);
// Shared memory of a CTA of the one-point-per-thread cluster kernels (prop_spread.cu) of C CTAs, in
// double2 values per point of the CTA: M-point twiddles, two exchange buffers, two halves of C receive
// rows.
constexpr long long spread_smem_per_point(int C) { return 3 + 2LL * C; }
// The same for the kernels that transform their K modes together (kKindSpreadFused): twiddles, two
// K-field exchange buffers, two halves of C x K receive rows.
constexpr long long spread_smem_per_point_k(int C, int K) { return 1 + 2LL * K + 2LL * C * K; }
constexpr long long kSpreadSmemPerPoint = spread_smem_per_point(4);
// Registry key offset of the instantiations for the general plan (FFTPlanH::gen == 1): grids that are
// not powers of two (kKindDirect, kKindLinear, kKindGnlse).
constexpr int kGenKey = 2000;
// Registry key offset (kKindCluster) of the one-point-per-thread kernels on eight CTAs, and on sixteen.
constexpr int kSpreadWideKey = 800;
constexpr int kSpreadW16Key = 900;

// Chi3 pump march on a 4-CTA cluster with one point per thread (prop_spread.cu); N = 4 M, M a power of
// two from 32 to 1024.
cudaError_t launch_pump_chi3_spread(double2* pumpFreq, double2* pumpTime, const double2* env, const double2* halfP,
                                    const double2* dstepP, const double2* backP, const double2* rel, int nRows, int N,
                                    const double2* tw, cudaStream_t s);

// The Chi3 pump march's grids and per-point tables (k_pump_chi3_spread's arguments).
struct PumpMarchArgs {
  double2* pf;            // [nRows][N] frequency-domain grid
  double2* pt;            // [nRows][N] time-domain grid
  const double2* env;     // [N] time-domain envelope
  const double2* halfP;   // [N] half a dispersion step
  const double2* dstepP;  // [N] a dispersion step, 1/N folded in
  const double2* backP;   // [N] half a step back (the last row)
  const double2* rel;     // [nRows] nonlinear step factors
  int nRows;
};

// The Chi3 pump march and one signal propagation (a: the signal's launch, a.pump = p.pt, a.nInst = 1)
// pipelined on one cluster of eight CTAs (prop_chi3_pipe.cu); N = 4 M, M a power of two from 32 to
// 1024, p.nRows = 2 a.nZ - 1.  regs (optional): the kernel's registers per thread.
cudaError_t launch_chi3_pump_signal_spread(const PropArgs& a, const PumpMarchArgs& p, cudaStream_t s,
                                           int* regs = nullptr);
cudaError_t launch_green_epilogue(const double2* raw, long long rawStride, int N, int nIn, int nOut,
                                  const double2* blockScale, const uint8_t* blockShift, double2* C,
                                  double2* S, cudaStream_t s);
cudaError_t launch_pump_from(const double2* otherSignalFreq, int otherRows, double ratio, double otherDz,
                             const double* dispPump, const double* otherDispSign, double dzp, double beta1Delay,
                             const double* omega, int nRowsP, int N, double z, double otherZ, double2* pumpFreq,
                             cudaStream_t s);
cudaError_t launch_cgemm_compose(const double2* Ci, const double2* Si, const double2* C, const double2* S,
                                 int rows, int inner, int cols, double2* Cout, double2* Sout, cudaStream_t s);
// dst[k] = float-float split of src[k] for k < n (segments of several arrays in one launch)
struct SplitSeg {
  const double2* src;
  float4* dst;
  long long n;
};
cudaError_t launch_split_ff(const SplitSeg* segs, int nSegs, cudaStream_t s);
cudaError_t launch_fp64_peak(double* out, int iters, int blocks, int threads, cudaStream_t s);
cudaError_t launch_fp64_mma_peak(double* out, int iters, int blocks, int threads, cudaStream_t s);
// Green's-function consumers (greens_quadrature.cu): quadrature-basis Z and the a-basis block matrix
cudaError_t launch_quadrature_z(const double2* C, const double2* S, long long rows, long long cols, double* Z,
                                cudaStream_t s);
cudaError_t launch_abasis_z(const double2* C, const double2* S, long long rows, long long cols, double2* Za,
                            cudaStream_t s);
// Post-processing of the adjoint of Chi2PDC (adjoint.cu)
cudaError_t launch_adj_pump_rows(const double2* ga, const double2* coef, const double* prof, int nZ, int N,
                                 double2* gP, cudaStream_t s);
cudaError_t launch_adj_pump_reduce(const double2* fgP, const double* disp, double dzp, int nRowsP, int N,
                                   double2* gF0, cudaStream_t s);
cudaError_t launch_adj_coef_reduce(const double2* ga, const double2* pump, int nZ, int N, double2* gc,
                                   cudaStream_t s);

}  // namespace nlm
