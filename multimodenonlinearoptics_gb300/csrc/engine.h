// engine.h -- the host engine behind the C ABI (include/nlm_capi.h): the Medium class (one solver
// instance with its device state and the propagation, Green's-function, batch, adjoint and cluster
// paths) and its host helpers.  Shared by the C ABI (engine.cpp) and the ragged-batch scheduler
// (engine_ragged.cpp).
//
// The host side mirrors the reference's _NonlinearMedium / _FullyNonlinearMedium / Cascade
// classes: the scalar set-up (lengths, axes, dispersion, poling, pump envelopes, the per-step
// coefficients of every solver's DiffEq) is computed here in double precision with the same
// formulas and the same std::exp / std::sqrt as the reference, and every transform and every
// propagation runs on the GPU through the kernels of nlm_kernels.h.  There is no CPU path for
// any of them: without a usable device those calls return NLM_ERR_NO_DEVICE.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/nlm_capi.h"
#include "nlm_kernels.h"
#include "nlm_launch.h"

namespace nlm {

using cplx = std::complex<double>;
using uint = unsigned int;
inline const double kInf = std::numeric_limits<double>::infinity();
inline const cplx kI(0.0, 1.0);

// ----------------------------------------------------------------------------------------
// errors
// ----------------------------------------------------------------------------------------
struct IndexError : std::out_of_range {
  using std::out_of_range::out_of_range;
};
struct NoDevice : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct Unsupported : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct CudaFailure : std::runtime_error {
  using std::runtime_error::runtime_error;
};

inline thread_local std::string g_error;

void set_error_message(const std::string& msg);   // engine.cpp

inline void ck(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw CudaFailure(std::string(what) + ": " + cudaGetErrorString(e));
  }
}

template <class F>
inline nlm_status guarded(F&& f) {
  try {
    f();
    return NLM_OK;
  } catch (const std::invalid_argument& e) {
    g_error = e.what();
    return NLM_ERR_INVALID_ARGUMENT;
  } catch (const IndexError& e) {
    g_error = e.what();
    return NLM_ERR_INDEX;
  } catch (const std::out_of_range& e) {
    g_error = e.what();
    return NLM_ERR_INDEX;
  } catch (const NoDevice& e) {
    g_error = e.what();
    return NLM_ERR_NO_DEVICE;
  } catch (const Unsupported& e) {
    g_error = e.what();
    return NLM_ERR_UNSUPPORTED;
  } catch (const CudaFailure& e) {
    g_error = e.what();
    return NLM_ERR_CUDA;
  } catch (const std::length_error& e) {
    g_error = e.what();
    return NLM_ERR_INVALID_ARGUMENT;
  } catch (const std::runtime_error& e) {
    g_error = e.what();
    return NLM_ERR_RUNTIME;
  } catch (const std::exception& e) {
    g_error = e.what();
    return NLM_ERR_RUNTIME;
  }
}

// ----------------------------------------------------------------------------------------
// device helpers
// ----------------------------------------------------------------------------------------
inline int device_count() {
  static int count = -1;
  static std::once_flag once;
  std::call_once(once, [] {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
      cudaGetLastError();
      n = 0;
    }
    count = n;
  });
  return count;
}

inline void require_device() {
  if (device_count() <= 0) throw NoDevice("no CUDA device is available: this engine has no CPU fallback");
}

template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void alloc(size_t count) {
    if (count == n && p) return;
    release();
    if (count == 0) return;
    ck(cudaMalloc(&p, count * sizeof(T)), "cudaMalloc");
    n = count;
  }
  void reserve(size_t count) {
    if (count <= n && p) return;
    alloc(count);
  }
};

inline double2* d2(void* p) { return reinterpret_cast<double2*>(p); }

// Page-locked host staging: copies from and to it are asynchronous (a copy from pageable memory
// waits for earlier work before it starts, one to pageable memory blocks the caller until it ran).
template <class T>
struct PinnedBuf {
  T* p = nullptr;
  size_t n = 0;
  PinnedBuf() = default;
  PinnedBuf(const PinnedBuf&) = delete;
  PinnedBuf& operator=(const PinnedBuf&) = delete;
  ~PinnedBuf() {
    if (p) cudaFreeHost(p);
  }
  void reserve(size_t count) {
    if (count <= n && p) return;
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
    if (count == 0) return;
    ck(cudaHostAlloc(reinterpret_cast<void**>(&p), count * sizeof(T), cudaHostAllocDefault), "cudaHostAlloc");
    n = count;
  }
};

// Launch sequences captured into CUDA graphs and replayed.  The key holds the bytes of every
// host-side value the captured launches read (kernel arguments, grid shape, pointers), so a replay
// is exactly the launch sequence it stands for; any change of a key byte captures a new graph.
struct GraphKey {
  std::vector<unsigned char> bytes;
  template <class T>
  GraphKey& add(const T& v) {
    const unsigned char* p = reinterpret_cast<const unsigned char*>(&v);
    bytes.insert(bytes.end(), p, p + sizeof(T));
    return *this;
  }
};

// Key bytes of a PropArgs, field by field (the struct has padding, whose bytes are unspecified).
inline void add_prop_key(GraphKey& k, const PropArgs& a) {
  k.add(a.plan.N).add(a.plan.T).add(a.plan.nPass).add(a.plan.gen).add(a.plan.R);
  for (int i = 0; i < a.plan.nPass && i < 16; i++) k.add(a.plan.radix[i]);
  k.add(a.R).add(a.nModes).add(a.nZ).add(a.nInst).add(a.instBase).add(a.ipc).add(a.work);
  k.add(a.inKind).add(a.inTime).add(a.in).add(a.inStride).add(a.inChannels).add(a.inputMode);
  for (int i = 0; i < kMaxModes; i++) k.add(a.impModes[i]);
  k.add(a.nOut);
  for (int i = 0; i < kMaxModes; i++) k.add(a.outModes[i]);
  k.add(a.out).add(a.outStride).add(a.tw).add(a.dstep).add(a.dlast).add(a.half).add(a.back).add(a.prop);
  k.add(a.pump).add(a.pumpStride).add(a.nPumps).add(a.coef).add(a.nCoef).add(a.gridF).add(a.gridT);
  k.add(a.ckpt).add(a.ckK).add(a.ckN).add(a.stages).add(a.raman).add(a.steep).add(a.relInt);
}

struct GraphCache {
  struct Entry {
    std::vector<unsigned char> key;
    cudaGraphExec_t exec = nullptr;
    unsigned long long lastUse = 0;
  };
  static constexpr size_t kMaxEntries = 8;
  std::vector<Entry> entries;
  unsigned long long clock = 0;
  long captures = 0, replays = 0;

  GraphCache() = default;
  GraphCache(const GraphCache&) = delete;
  GraphCache& operator=(const GraphCache&) = delete;
  ~GraphCache() { clear(); }
  void clear() {
    for (auto& e : entries)
      if (e.exec) cudaGraphExecDestroy(e.exec);
    entries.clear();
  }

  // Enqueue `record` (launches on `stream` only: no allocation, synchronisation or pageable copy) as
  // a graph: replay of the graph captured for `key`, else capture, instantiate and launch.  Streams
  // that cannot be captured (the legacy default stream, or one already being captured by the
  // caller) get the launches directly.
  // Returns true when it replayed a captured graph (the host code of `record` did not run).
  bool run(const GraphKey& key, cudaStream_t stream, const std::function<void()>& record) {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    if (stream == nullptr || cudaStreamIsCapturing(stream, &st) != cudaSuccess || st != cudaStreamCaptureStatusNone) {
      record();
      return false;
    }
    clock++;
    for (auto& e : entries)
      if (e.key == key.bytes) {
        e.lastUse = clock;
        replays++;
        ck(cudaGraphLaunch(e.exec, stream), "graph launch");
        return true;
      }
    cudaGraph_t g = nullptr;
    ck(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "graph capture");
    try {
      record();
    } catch (...) {
      cudaStreamEndCapture(stream, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    ck(cudaStreamEndCapture(stream, &g), "graph capture");
    cudaGraphExec_t ex = nullptr;
    // node priorities: launches captured from prioritised streams keep their priority in the graph
    const cudaError_t e = cudaGraphInstantiate(&ex, g, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(g);
    ck(e, "graph instantiate");
    if (entries.size() >= kMaxEntries) {
      auto old = std::min_element(entries.begin(), entries.end(),
                                  [](const Entry& a, const Entry& b) { return a.lastUse < b.lastUse; });
      cudaGraphExecDestroy(old->exec);
      entries.erase(old);
    }
    entries.push_back(Entry{key.bytes, ex, clock});
    captures++;
    ck(cudaGraphLaunch(ex, stream), "graph launch");
    return false;
  }
};

// Twiddle table exp(-2 pi i m / N), one per grid size, per process.
struct TwiddleCache {
  std::mutex mu;
  std::map<int, std::shared_ptr<DevBuf<double2>>> tables;
  const double2* get(int N, cudaStream_t s) {
    std::lock_guard<std::mutex> lock(mu);
    auto it = tables.find(N);
    if (it != tables.end()) return it->second->p;
    std::vector<double2> h(N);
    for (int m = 0; m < N; m++) {
      // reduce to the first octant with exact symmetries, then evaluate in long double
      const long double ang = -2.0L * 3.141592653589793238462643383279502884L * (long double)m / (long double)N;
      h[m].x = (double)std::cos(ang);
      h[m].y = (double)std::sin(ang);
    }
    // exact values at the quarter points
    for (int q = 0; q < 4; q++) {
      if ((long long)N * q % 4 != 0) continue;
      const int m = N * q / 4;
      const double c[4] = {1, 0, -1, 0}, sn[4] = {0, -1, 0, 1};
      h[m].x = c[q];
      h[m].y = sn[q];
    }
    auto buf = std::make_shared<DevBuf<double2>>();
    buf->alloc(N);
    ck(cudaMemcpyAsync(buf->p, h.data(), N * sizeof(double2), cudaMemcpyHostToDevice, s), "twiddle upload");
    ck(cudaStreamSynchronize(s), "twiddle upload");
    tables[N] = buf;
    return buf->p;
  }
};
inline TwiddleCache g_twiddles;

inline bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

// The general plan (FFTPlanH::gen == 1) of an N-point transform with R points per thread: T = ceil(N/R)
// threads, passes of radix 8 (then one of 4 or 2) for the power-of-two factor and one per odd prime
// factor, in ascending order.  Any N >= 2 up to kMaxFFT.
inline FFTPlanH make_plan_gen(int N, int R) {
  FFTPlanH p{};
  p.N = N;
  p.R = R;
  p.gen = 1;
  p.T = (N + R - 1) / R;
  std::vector<int> rad;
  int n = N, twos = 0;
  while (n % 2 == 0) {
    n /= 2;
    twos++;
  }
  for (; twos >= 3; twos -= 3) rad.push_back(8);
  if (twos) rad.push_back(1 << twos);
  for (int q = 3; n > 1; q += 2)
    while (n % q == 0) {
      rad.push_back(q);
      n /= q;
    }
  if (rad.size() > 16) throw Unsupported("transform of " + std::to_string(N) + " points has too many factors");
  p.nPass = (int)rad.size();
  for (int i = 0; i < p.nPass; i++) p.radix[i] = rad[i];
  return p;
}

// Plan of an N-point transform with R points per thread: the register plan (gen == 0, radix-8 passes
// with one radix-2/4 pass, T = N/R) when N is a power of two of at least R points, the general plan
// otherwise.
inline FFTPlanH make_plan(int N, int R) {
  if (!is_pow2(N) || N < R) return make_plan_gen(N, R);
  FFTPlanH p{};
  p.N = N;
  p.R = R;
  p.T = N / R;
  int n = 0;
  while ((1 << n) < N) n++;
  const int rl = R >= 8 ? 3 : 2;
  int a = n / rl, rem = n % rl;
  std::vector<int> rad(a, 1 << rl);
  if (rem) rad.insert(rad.begin() + (a >= 1 ? 1 : 0), 1 << rem);
  p.nPass = (int)rad.size();
  for (int i = 0; i < p.nPass; i++) p.radix[i] = rad[i];
  return p;
}

// ----------------------------------------------------------------------------------------
// solver registry: constructor signatures and their mapping onto the base class
// (solvers/*.cpp constructors; py::init keyword lists)
// ----------------------------------------------------------------------------------------
enum Solver {
  kChi3 = 0, kChi2PDC, kChi2SFG, kChi2AFC, kChi2SFGPDC, kChi2SFGII, kChi2PDCII, kChi2SFGOPA, kChi2SFGXPM,
  kChi2SHG, kChi2SHGOPA, kChi2DSFG, kChi2SHGXPM, kChi2ASHG, kChi3GNLSE, kNumSolvers
};

struct SolverInfo {
  const char* name;
  // scalar arguments in positional order; "@customPump" / "@poling" mark array arguments
  const char* signature;
  int modes, pumps, coefs;
  bool fnl, linear;
};

inline const SolverInfo kSolvers[kNumSolvers] = {
    {"Chi3",
     "relativeLength,nlLength,beta2,@customPump,pulseType=0,beta3=0,rayleighLength=inf,tMax=10,tPrecision=512,"
     "zPrecision=100,intensityProfile=0,chirp=0",
     1, 1, 1, false, true},
    {"Chi2PDC",
     "relativeLength,nlLength,beta2,beta2s,@customPump,pulseType=0,beta1=0,beta1s=0,beta3=0,beta3s=0,diffBeta0=0,"
     "rayleighLength=inf,tMax=10,tPrecision=512,zPrecision=100,intensityProfile=0,chirp=0,delay=0,@poling",
     1, 1, 1, false, true},
    {"Chi2SFG",
     "relativeLength,nlLength,nlLengthOrig,beta2,beta2s,beta2o,@customPump,pulseType=0,beta1=0,beta1s=0,beta1o=0,"
     "beta3=0,beta3s=0,beta3o=0,diffBeta0=0,rayleighLength=inf,tMax=10,tPrecision=512,zPrecision=100,"
     "intensityProfile=0,chirp=0,delay=0,@poling",
     2, 1, 2, false, true},
    {"Chi2AFC",
     "relativeLength,nlLength,nlLengthOrig,beta2,beta2s,beta2o,@customPump,pulseType=0,beta1=0,beta1s=0,beta1o=0,"
     "beta3=0,beta3s=0,beta3o=0,diffBeta0Start=0,diffBeta0End=0,rayleighLength=inf,tMax=10,tPrecision=512,"
     "zPrecision=100,intensityProfile=0,chirp=0,delay=0",
     2, 1, 2, false, true},
    {"Chi2SFGPDC",
     "relativeLength,nlLength,nlLengthOrig,beta2,beta2s,beta2o,@customPump,pulseType=0,beta1=0,beta1s=0,beta1o=0,"
     "beta3=0,beta3s=0,beta3o=0,diffBeta0=0,diffBeta0o=0,rayleighLength=inf,tMax=10,tPrecision=512,zPrecision=100,"
     "intensityProfile=0,chirp=0,delay=0,@poling",
     2, 1, 4, false, true},
    {"Chi2SFGII",
     "relativeLength,nlLengthZY,nlLengthZZ,beta2,beta2sz,beta2sy,beta2oz,beta2oy,@customPump,pulseType=0,beta1=0,"
     "beta1sz=0,beta1sy=0,beta1oz=0,beta1oy=0,beta3=0,beta3sz=0,beta3sy=0,beta3oz=0,beta3oy=0,diffBeta0z=0,"
     "diffBeta0y=0,diffBeta0=0,rayleighLength=inf,tMax=10,tPrecision=512,zPrecision=100,intensityProfile=0,chirp=0,"
     "delay=0,@poling",
     4, 1, 7, false, true},
    {"Chi2PDCII",
     "relativeLength,nlLengthI,nlLengthII,beta2,beta2s,beta2o,@customPump,pulseType=0,beta1=0,beta1s=0,beta1o=0,"
     "beta3=0,beta3s=0,beta3o=0,diffBeta0=0,rayleighLength=inf,tMax=10,tPrecision=512,zPrecision=100,"
     "intensityProfile=0,chirp=0,delay=0,@poling",
     2, 1, 2, false, true},
    {"Chi2SFGOPA",
     "relativeLength,nlLengthSFGh,nlLengthSFGf,nlLengthDOPAh,nlLengthDOPAf,beta2F,beta2H,beta2h,beta2f,@customPump,"
     "pulseType=0,beta1F=0,beta1H=0,beta1h=0,beta1f=0,beta3F=0,beta3H=0,beta3h=0,beta3f=0,diffBeta0SFG=0,"
     "diffBeta0DOPA=0,rayleighLength=inf,tMax=10,tPrecision=512,zPrecision=100,intensityProfile=0,chirp=0,delay=0,"
     "@poling",
     2, 2, 4, false, true},
    {"Chi2SFGXPM",
     "relativeLength,nlLength,nlLengthOrig,nlLengthChi3,nlLengthChi3Orig,beta2,beta2s,beta2o,@customPump,pulseType=0,"
     "beta1=0,beta1s=0,beta1o=0,beta3=0,beta3s=0,beta3o=0,diffBeta0=0,rayleighLength=inf,tMax=10,tPrecision=512,"
     "zPrecision=100,intensityProfile=0,chirp=0,delay=0,@poling",
     2, 1, 4, false, true},
    {"Chi2SHG",
     "relativeLength,nlLengthH,nlLengthP,beta2h,beta2p,beta1h=0,beta1p=0,beta3h=0,beta3p=0,diffBeta0=0,"
     "rayleighLength=inf,tMax=10,tPrecision=512,zPrecision=100,intensityProfile=0,@poling",
     2, 0, 2, true, false},
    {"Chi2SHGOPA",
     "relativeLength,nlLengthP,nlLengthSH,nlLengthPA1,nlLengthPA2,beta2p,beta2sh,beta2pa1,beta2pa2,beta1p=0,"
     "beta1sh=0,beta1pa1=0,beta1pa2=0,beta3p=0,beta3sh=0,beta3pa1=0,beta3pa2=0,diffBeta0shg=0,diffBeta0opa=0,"
     "rayleighLength=inf,tMax=10,tPrecision=512,zPrecision=100,intensityProfile=0,@poling",
     4, 0, 6, true, false},
    {"Chi2DSFG",
     "relativeLength,nlLengthP,nlLengthS,nlLengthD,beta2p,beta2s,beta2d,beta1p=0,beta1s=0,beta1d=0,beta3p=0,"
     "beta3s=0,beta3d=0,diffBeta0=0,rayleighLength=inf,tMax=10,tPrecision=512,zPrecision=100,intensityProfile=0,"
     "@poling",
     3, 0, 3, true, false},
    {"Chi2SHGXPM",
     "relativeLength,nlLengthH,nlLengthP,nlLengthChi3,beta2h,beta2p,beta1h=0,beta1p=0,beta3h=0,beta3p=0,diffBeta0=0,"
     "rayleighLength=inf,tMax=10,tPrecision=512,zPrecision=100,intensityProfile=0,@poling",
     2, 0, 3, true, false},
    {"Chi2ASHG",
     "relativeLength,nlLengthH,nlLengthP,beta2h,beta2p,beta1h=0,beta1p=0,beta3h=0,beta3p=0,diffBeta0Start=0,"
     "diffBeta0End=0,rayleighLength=inf,tMax=10,tPrecision=512,zPrecision=100,intensityProfile=0",
     2, 0, 2, true, false},
    {"Chi3GNLSE",
     "relativeLength,nlLength,selfSteepLength,fr,fb,tau1,tau2,tau3,beta2,beta3=0,rayleighLength=inf,tMax=10,"
     "tPrecision=512,zPrecision=100,intensityProfile=0",
     1, 0, 0, true, false},
};

inline int solver_by_name(const char* name) {
  for (int i = 0; i < kNumSolvers; i++)
    if (std::strcmp(kSolvers[i].name, name) == 0) return i;
  return -1;
}

inline int scalar_arg_count(int solver) {
  int n = 0;
  const char* s = kSolvers[solver].signature;
  std::string tok;
  for (const char* c = s;; c++) {
    if (*c == ',' || *c == 0) {
      if (!tok.empty() && tok[0] != '@') n++;
      tok.clear();
      if (*c == 0) break;
    } else {
      tok += *c;
    }
  }
  return n;
}

// Arguments of the base-class constructor (src/_NonlinearMedium.hpp:59-67).
struct BaseParams {
  uint nSignal = 1, nPump = 1;
  bool poled = false, fnl = false;
  double relativeLength = 1;
  std::vector<double> nl, beta2, beta2s, beta1, beta1s, beta3, beta3s, diffBeta0;
  double rayleigh = kInf, tMax = 10;
  uint tPrecision = 512, zPrecision = 100;
  int profile = NLM_GAUSSIAN_BEAM;
  double chirp = 0, delay = 0;
  int pulseType = NLM_GAUSSIAN;
  // Chi3GNLSE
  double fr = 0, fb = 0, tau1 = 1, tau2 = 1, tau3 = 1;
};

inline uint as_uint(double v) {
  if (!(v >= 0) || v > 4294967295.0) throw std::invalid_argument("integer argument out of range");
  return (uint)v;
}

inline BaseParams map_ctor(int s, const double* a) {
  BaseParams b;
  const double halfPi = 0.5 * M_PI;
  auto tail = [&](int i, bool withChirp, bool withDelay) {
    // ..., rayleighLength, tMax, tPrecision, zPrecision, intensityProfile[, chirp[, delay]]
    b.rayleigh = a[i];
    b.tMax = a[i + 1];
    b.tPrecision = as_uint(a[i + 2]);
    b.zPrecision = as_uint(a[i + 3]);
    b.profile = (int)a[i + 4];
    if (withChirp) b.chirp = a[i + 5];
    if (withDelay) b.delay = a[i + 6];
  };
  switch (s) {
    case kChi3:  // solvers/Chi3.cpp:34-38
      b.nSignal = 1; b.nPump = 1; b.poled = false;
      b.relativeLength = a[0]; b.nl = {a[1]}; b.beta2 = {a[2]}; b.beta2s = {a[2]};
      b.pulseType = (int)a[3]; b.beta1 = {0}; b.beta1s = {0}; b.beta3 = {a[4]}; b.beta3s = {a[4]};
      b.rayleigh = a[5]; b.tMax = a[6]; b.tPrecision = as_uint(a[7]); b.zPrecision = as_uint(a[8]);
      b.profile = (int)a[9]; b.chirp = a[10]; b.delay = 0;
      break;
    case kChi2PDC:  // solvers/Chi2PDC.cpp:18-24
      b.nSignal = 1; b.nPump = 1; b.poled = true;
      b.relativeLength = a[0]; b.nl = {a[1]}; b.beta2 = {a[2]}; b.beta2s = {a[3]}; b.pulseType = (int)a[4];
      b.beta1 = {a[5]}; b.beta1s = {a[6]}; b.beta3 = {a[7]}; b.beta3s = {a[8]}; b.diffBeta0 = {a[9]};
      tail(10, true, true);
      break;
    case kChi2SFG:  // solvers/Chi2SFG.cpp:20-27
    case kChi2PDCII:  // solvers/Chi2PDCII.cpp:20-27
      b.nSignal = 2; b.nPump = 1; b.poled = true;
      b.relativeLength = a[0]; b.nl = {a[1], a[2]}; b.beta2 = {a[3]}; b.beta2s = {a[4], a[5]};
      b.pulseType = (int)a[6]; b.beta1 = {a[7]}; b.beta1s = {a[8], a[9]}; b.beta3 = {a[10]};
      b.beta3s = {a[11], a[12]}; b.diffBeta0 = {a[13]};
      tail(14, true, true);
      break;
    case kChi2AFC:  // solvers/Chi2AFC.cpp:17-23
      b.nSignal = 2; b.nPump = 1; b.poled = false;
      b.relativeLength = a[0]; b.nl = {halfPi * a[1], halfPi * a[2]}; b.beta2 = {a[3]}; b.beta2s = {a[4], a[5]};
      b.pulseType = (int)a[6]; b.beta1 = {a[7]}; b.beta1s = {a[8], a[9]}; b.beta3 = {a[10]};
      b.beta3s = {a[11], a[12]}; b.diffBeta0 = {a[13], a[14]};
      tail(15, true, true);
      break;
    case kChi2SFGPDC:  // solvers/Chi2SFGPDC.cpp:20-28
      b.nSignal = 2; b.nPump = 1; b.poled = true;
      b.relativeLength = a[0]; b.nl = {a[1], a[2]}; b.beta2 = {a[3]}; b.beta2s = {a[4], a[5]};
      b.pulseType = (int)a[6]; b.beta1 = {a[7]}; b.beta1s = {a[8], a[9]}; b.beta3 = {a[10]};
      b.beta3s = {a[11], a[12]}; b.diffBeta0 = {a[13], a[14]};
      tail(15, true, true);
      break;
    case kChi2SFGII:  // solvers/Chi2SFGII.cpp:23-34
      b.nSignal = 4; b.nPump = 1; b.poled = true;
      b.relativeLength = a[0]; b.nl = {a[1], a[2]}; b.beta2 = {a[3]}; b.beta2s = {a[4], a[5], a[6], a[7]};
      b.pulseType = (int)a[8]; b.beta1 = {a[9]}; b.beta1s = {a[10], a[11], a[12], a[13]}; b.beta3 = {a[14]};
      b.beta3s = {a[15], a[16], a[17], a[18]}; b.diffBeta0 = {a[19], a[20], a[21]};
      tail(22, true, true);
      break;
    case kChi2SFGOPA:  // solvers/Chi2SFGOPA.cpp:20-28
      b.nSignal = 2; b.nPump = 2; b.poled = true;
      b.relativeLength = a[0]; b.nl = {a[1], a[2], a[3], a[4]}; b.beta2 = {a[5], a[6]}; b.beta2s = {a[7], a[8]};
      b.pulseType = (int)a[9]; b.beta1 = {a[10], a[11]}; b.beta1s = {a[12], a[13]}; b.beta3 = {a[14], a[15]};
      b.beta3s = {a[16], a[17]}; b.diffBeta0 = {a[18], a[19]};
      tail(20, true, true);
      break;
    case kChi2SFGXPM:  // solvers/Chi2SFGXPM.cpp:20-27 (the XPM lengths are halved)
      b.nSignal = 2; b.nPump = 1; b.poled = true;
      b.relativeLength = a[0]; b.nl = {a[1], a[2], a[3] / 2, a[4] / 2}; b.beta2 = {a[5]}; b.beta2s = {a[6], a[7]};
      b.pulseType = (int)a[8]; b.beta1 = {a[9]}; b.beta1s = {a[10], a[11]}; b.beta3 = {a[12]};
      b.beta3s = {a[13], a[14]}; b.diffBeta0 = {a[15]};
      tail(16, true, true);
      break;
    case kChi2SHG:  // solvers/Chi2SHG.cpp:18-23: modes reordered to {P, SH}
      b.nSignal = 2; b.nPump = 0; b.poled = true; b.fnl = true;
      b.relativeLength = a[0]; b.nl = {a[2], a[1]}; b.beta2s = {a[4], a[3]}; b.beta1s = {a[6], a[5]};
      b.beta3s = {a[8], a[7]}; b.diffBeta0 = {a[9]};
      tail(10, false, false);
      break;
    case kChi2SHGOPA:  // solvers/Chi2SHGOPA.cpp:19-29
      b.nSignal = 4; b.nPump = 0; b.poled = true; b.fnl = true;
      b.relativeLength = a[0]; b.nl = {a[1], a[2], a[3], a[4]}; b.beta2s = {a[5], a[6], a[7], a[8]};
      b.beta1s = {a[9], a[10], a[11], a[12]}; b.beta3s = {a[13], a[14], a[15], a[16]}; b.diffBeta0 = {a[17], a[18]};
      tail(19, false, false);
      break;
    case kChi2DSFG:  // solvers/Chi2DSFG.cpp:16-22
      b.nSignal = 3; b.nPump = 0; b.poled = true; b.fnl = true;
      b.relativeLength = a[0]; b.nl = {a[1], a[2], a[3]}; b.beta2s = {a[4], a[5], a[6]};
      b.beta1s = {a[7], a[8], a[9]}; b.beta3s = {a[10], a[11], a[12]}; b.diffBeta0 = {a[13]};
      tail(14, false, false);
      break;
    case kChi2SHGXPM:  // solvers/Chi2SHGXPM.cpp:18-24: modes {P, SH}
      b.nSignal = 2; b.nPump = 0; b.poled = true; b.fnl = true;
      b.relativeLength = a[0]; b.nl = {a[2], a[1], a[3]}; b.beta2s = {a[5], a[4]}; b.beta1s = {a[7], a[6]};
      b.beta3s = {a[9], a[8]}; b.diffBeta0 = {a[10]};
      tail(11, false, false);
      break;
    case kChi2ASHG:  // solvers/Chi2ASHG.cpp:15-20
      b.nSignal = 2; b.nPump = 0; b.poled = false; b.fnl = true;
      b.relativeLength = a[0]; b.nl = {halfPi * a[2], halfPi * a[1]}; b.beta2s = {a[4], a[3]};
      b.beta1s = {a[6], a[5]}; b.beta3s = {a[8], a[7]}; b.diffBeta0 = {a[9], a[10]};
      tail(11, false, false);
      break;
    case kChi3GNLSE:  // solvers/Chi3GNLSE.cpp:20-24
      b.nSignal = 1; b.nPump = 0; b.poled = false; b.fnl = true;
      b.relativeLength = a[0]; b.nl = {a[1], a[2]}; b.fr = a[3]; b.fb = a[4]; b.tau1 = a[5]; b.tau2 = a[6];
      b.tau3 = a[7]; b.beta2s = {a[8]}; b.beta1s = {0}; b.beta3s = {a[9]};
      tail(10, false, false);
      break;
    default:
      throw std::invalid_argument("unknown solver");
  }
  return b;
}

// ----------------------------------------------------------------------------------------
// Medium
// ----------------------------------------------------------------------------------------
struct GridMirror {
  std::vector<double> host;   // interleaved complex
  long long version = -1;
};

struct Medium {
  int solver = -1;
  bool isCascade = false;
  uint nSignal = 0, nPump = 0;
  bool fnl = false, poled = false;
  double z = 0, dz = 0, dzp = 0, tMax = 0, rayleigh = kInf;
  uint nZ = 0, nZP = 0, N = 0;
  int profile = NLM_CONSTANT;
  std::vector<double> beta2, beta1, diffBeta0;
  std::vector<cplx> nlStep;
  std::vector<std::vector<cplx>> envelope;
  std::vector<double> poling, tau, omega;
  std::vector<std::vector<double>> dispPump, dispSign;
  std::vector<std::vector<cplx>> dstepPump, dstepSign;
  double fr = 0, fb = 0, tau1 = 1, tau2 = 1, tau3 = 1;
  std::vector<cplx> raman;   // Chi3GNLSE, filled at first device use

  // device state
  bool devReady = false;
  int devOrdinal = -1;   // the device holding this medium's tables (current device at set-up)
  cudaStream_t stream = nullptr;
  bool ownStream = false;
  const double2* tw = nullptr;
  DevBuf<double2> pumpFreq, pumpTime, sigFreq, sigTime;
  DevBuf<double2> dstep, dlast, half, back, coef, ramanD, steepD;
  DevBuf<double> relIntD, dispPumpD, dispSignD, omegaD;
  DevBuf<double> prop;
  long long propVersion = -1, propBuilds = 0;
  // arithmetic of the single-mode propagator path: 0 FP64, 1 double-float on the FP32 units
  int precision = 0;
  DevBuf<float4> twF, dstepF, dlastF, halfF, backF, propF;
  bool ffTables = false;
  long long propFFBuild = -1;
  DevBuf<double2> work, work2, raw, cs, io;
  DevBuf<double2> scratch;
  DevBuf<uint8_t> flagsD;
  DevBuf<unsigned long long> workCounter;
  // adjoint state: forward checkpoints of the last nlm_adjoint_forward
  DevBuf<double2> ckpt, adjSeg, adjGa, adjGP, adjFGP, adjGc, adjStages, adjGPS;
  bool adjStored = false;   // the last adjoint forward stored the Chi3GNLSE stage values of every step
  DevBuf<double> profD;
  long long adjRows = 0;
  int adjK = 0, adjNCk = 0;
  long long adjPumpVersion = -1;
  DevBuf<double2> scaleD;
  long long pumpVersion = 0, signalVersion = 0;
  // A Chi3 pump march that runPump prepared but did not launch (spread grids of up to 1024 points): the
  // next runSignal runs it beside the signal on one cluster of eight CTAs (prop_chi3_pipe.cu); any
  // other use of the pump grids runs it alone first (flushPump).
  struct DeferredPump {
    DevBuf<double2> env, half, dstep, back, rel;
    bool pending = false;
  } deferredPump;
  GridMirror mPumpF, mPumpT, mSigF, mSigT;
  std::vector<std::vector<double>> pumpMirrorF, pumpMirrorT, sigMirrorF, sigMirrorT;
  std::vector<long long> pumpMirrorVerF, pumpMirrorVerT, sigMirrorVerF, sigMirrorVerT;
  std::vector<double> axisBuf;
  long launches = 0;
  // kernel timing (measurement support)
  bool timeKernels = false;
  double kernelMs = 0;
  long kernelCount = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // schedule overrides
  int ctaPerSM = 0, usePropagator = -1, useGraph = 1;
  GraphCache graphs;

  // cascade
  std::vector<Medium*> media;
  std::vector<std::map<uint, uint>> connections;
  bool sharedPump = false;

  ~Medium() {
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (ownStream && stream) cudaStreamDestroy(stream);
  }

  // -- set-up, src/_NonlinearMedium.cpp:43-102 -------------------------------------------
  void setLengths(double relativeLength, const std::vector<double>& nl, uint zPrecision, double rayleighLength,
                  const std::vector<double>& b2, const std::vector<double>& b2s, const std::vector<double>& b1,
                  const std::vector<double>& b1s, const std::vector<double>& b3, const std::vector<double>& b3s) {
    bool negative = relativeLength <= 0 || rayleighLength <= 0;
    for (double l : nl) negative |= (l <= 0);
    if (negative) throw std::invalid_argument("Non-positive length scale");
    bool allNonUnit = true;
    for (const auto* g : {&b1, &b2, &b3, &b1s, &b2s, &b3s})
      for (double b : *g) allNonUnit &= (std::abs(b) != 1);
    for (double l : nl) allNonUnit &= (l != 1);
    allNonUnit &= (relativeLength != 1);
    allNonUnit &= (rayleighLength != 1);
    if (allNonUnit) throw std::invalid_argument("No unit length scale provided: please normalize variables");
    z = relativeLength;
    auto absComp = [](double a, double b) { return std::abs(a) < std::abs(b); };
    auto ext = [&](const std::vector<double>& v) { return v.empty() ? 0.0 : *std::max_element(v.begin(), v.end(), absComp); };
    const double minDispLength = 1 / std::abs(std::max({ext(b2), ext(b2s), ext(b1), ext(b1s), ext(b3), ext(b3s)}, absComp));
    const double minNl = nl.empty() ? 0 : *std::min_element(nl.begin(), nl.end());
    const double steps = zPrecision * z / std::min({1., minDispLength, rayleighLength, minNl});
    nZ = (std::isfinite(steps) && steps >= 0 && steps < 4294967296.0) ? (uint)steps : 0;
    nZP = 2 * nZ - 1;
    dz = z / (nZ - 1);
    dzp = z / (nZP - 1);
    nlStep.resize(nl.size());
    for (size_t p = 0; p < nl.size(); p++) nlStep[p] = 1.0 * kI / nl[p] * dz;
    rayleigh = rayleighLength;
  }

  // src/_NonlinearMedium.cpp:105-145
  void resetGrids(uint nFreqs, double tMaxIn) {
    if (nFreqs % 2 != 0 || nFreqs == 0) throw std::invalid_argument("Invalid number of Frequencies");
    if (nZ == 0) throw std::invalid_argument("Zero steps");
    if (tMaxIn <= 0) throw std::invalid_argument("Negative time span");
    N = nFreqs;
    tMax = tMaxIn;
    const int Nt = (int)N;
    std::vector<double> ramp(Nt);
    for (int k = 0; k < Nt; k++) ramp[k] = (double)(k - Nt / 2);
    tau.assign(Nt, 0);
    omega.assign(Nt, 0);
    const double st = 2 * tMax / Nt, sw = -M_PI / tMax;
    const int h = Nt / 2;
    for (int k = 0; k < Nt; k++) {  // fftshift of the linear ramps
      const int src = (k + h) % Nt;
      tau[k] = st * ramp[src];
      omega[k] = sw * ramp[src];
    }
  }

  // src/_NonlinearMedium.cpp:148-177
  void setDispersion(const std::vector<double>& b2, const std::vector<double>& b2s, const std::vector<double>& b1,
                     const std::vector<double>& b1s, const std::vector<double>& b3, const std::vector<double>& b3s,
                     const std::vector<double>& db0) {
    beta2 = b2;
    beta1 = b1;
    diffBeta0 = db0;
    dispPump.assign(nPump, std::vector<double>(N));
    for (uint m = 0; m < nPump; m++)
      for (uint k = 0; k < N; k++) dispPump[m][k] = omega[k] * (b1[m] + omega[k] * (0.5 * b2[m] + omega[k] * b3[m] / 6));
    dispSign.assign(nSignal, std::vector<double>(N));
    for (uint m = 0; m < nSignal; m++)
      for (uint k = 0; k < N; k++) dispSign[m][k] = omega[k] * (b1s[m] + omega[k] * (0.5 * b2s[m] + omega[k] * b3s[m] / 6));
    dstepPump.assign(nPump, std::vector<cplx>(N));
    for (uint m = 0; m < nPump; m++)
      for (uint k = 0; k < N; k++) dstepPump[m][k] = std::exp((1.0 * kI * dzp) * dispPump[m][k]);
    dstepSign.assign(nSignal, std::vector<cplx>(N));
    for (uint m = 0; m < nSignal; m++)
      for (uint k = 0; k < N; k++) dstepSign[m][k] = std::exp((1.0 * kI * dz) * dispSign[m][k]);
  }

  // src/_NonlinearMedium.cpp:470-503
  void setPoling(const std::vector<double>& pol) {
    if (pol.size() <= 1) {
      poling.assign(nZ, 1.0);
      return;
    }
    for (double p : pol)
      if (p <= 0) throw std::invalid_argument("Poling contains invalid domain length");
    std::vector<double> dom(pol.size());
    dom[0] = pol[0];
    for (size_t i = 1; i < pol.size(); i++) dom[i] = pol[i] + dom[i - 1];
    const double scale = nZ / dom.back();
    for (double& d : dom) d *= scale;
    poling.assign(nZ, 0.0);
    uint prevInd = 0;
    int direction = 1;
    for (size_t i = 0; i < dom.size(); i++) {
      const double currInd = dom[i];
      const uint currIndRound = (uint)currInd;
      if (currInd < prevInd) throw std::invalid_argument("Poling period too small for simulation resolution");
      for (uint k = prevInd; k < currIndRound && k < nZ; k++) poling[k] = direction;
      if (currIndRound < nZ) poling[currIndRound] = direction * (2 * std::abs(std::fmod(currInd, 1)) - 1);
      direction *= -1;
      prevInd = currIndRound + 1;
    }
  }

  // ---- device state -------------------------------------------------------------------
  void ensureDevice() {
    if (devReady) return;
    require_device();
    ck(cudaGetDevice(&devOrdinal), "device");
    if (!stream) {
      ck(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
      ownStream = true;
    }
    tw = g_twiddles.get((int)N, stream);
    const size_t n = N;
    if (nPump > 0 && nZP > 0) {
      pumpFreq.alloc((size_t)nPump * nZP * n + kTablePad);
      pumpTime.alloc((size_t)nPump * nZP * n + kTablePad);
      ck(cudaMemsetAsync(pumpFreq.p, 0, pumpFreq.n * sizeof(double2), stream), "memset");
      ck(cudaMemsetAsync(pumpTime.p, 0, pumpTime.n * sizeof(double2), stream), "memset");
    }
    sigFreq.alloc((size_t)nSignal * nZ * n);
    sigTime.alloc((size_t)nSignal * nZ * n);
    ck(cudaMemsetAsync(sigFreq.p, 0, sigFreq.n * sizeof(double2), stream), "memset");
    ck(cudaMemsetAsync(sigTime.p, 0, sigTime.n * sizeof(double2), stream), "memset");
    // point-wise factor tables with 1/N folded in (the inverse transforms are unscaled)
    std::vector<double2> hd(nSignal * n), hl(nSignal * n), hh(nSignal * n), hb(nSignal * n);
    const double invN = 1.0 / N;
    for (uint m = 0; m < nSignal; m++)
      for (uint k = 0; k < N; k++) {
        const cplx hf = std::exp((0.5 * kI * dz) * dispSign[m][k]);
        const cplx bk = std::exp((-0.5 * kI * dz) * dispSign[m][k]);
        const cplx d = dstepSign[m][k] * invN;
        const cplx dl = dstepSign[m][k] * bk * invN;
        const cplx h = hf * invN, b = bk * invN;
        hd[m * n + k] = make_double2(d.real(), d.imag());
        hl[m * n + k] = make_double2(dl.real(), dl.imag());
        hh[m * n + k] = make_double2(h.real(), h.imag());
        hb[m * n + k] = make_double2(b.real(), b.imag());
      }
    upload(dstep, hd);
    upload(dlast, hl);
    upload(half, hh);
    upload(back, hb);
    std::vector<double> hdp, hds;
    for (auto& v : dispPump) hdp.insert(hdp.end(), v.begin(), v.end());
    for (auto& v : dispSign) hds.insert(hds.end(), v.begin(), v.end());
    uploadD(dispPumpD, hdp);
    uploadD(dispSignD, hds);
    uploadD(omegaD, omega);
    buildCoefficients();
    if (solver == kChi3GNLSE) buildGnlse();
    ck(cudaStreamSynchronize(stream), "device set-up");
    devReady = true;
  }

  // Device tables carry kTablePad zeroed values after their data: a kernel on the general plan reads
  // the points of its padded ownership (j + v T up to R - 1 past N) without a bound check, and the
  // values it reads there only ever meet zeros.
  template <class V>
  void upload(DevBuf<double2>& d, const V& h) {
    if (h.empty()) {
      d.alloc(0);
      return;
    }
    d.alloc(h.size() + kTablePad);
    ck(cudaMemcpyAsync(d.p, h.data(), h.size() * sizeof(double2), cudaMemcpyHostToDevice, stream), "upload");
    ck(cudaMemsetAsync(d.p + h.size(), 0, kTablePad * sizeof(double2), stream), "upload");
  }
  void uploadD(DevBuf<double>& d, const std::vector<double>& h) {
    if (h.empty()) {
      d.alloc(0);
      return;
    }
    d.alloc(h.size() + kTablePad);
    ck(cudaMemcpyAsync(d.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, stream), "upload");
    ck(cudaMemsetAsync(d.p + h.size(), 0, kTablePad * sizeof(double), stream), "upload");
  }

  // relativeAmplitude / relativeIntensity, src/_FullyNonlinearMedium.hpp:40-63
  double relativeAmplitude(double i) const {
    switch (profile) {
      case NLM_GAUSSIAN_BEAM: return std::sqrt(1 / (1 + std::pow((i * dz - 0.5 * z) / rayleigh, 2)));
      case NLM_CONSTANT: return 1.;
      case NLM_GAUSSIAN_APODIZATION: return std::exp(-0.5 * std::pow((i * dz - 0.5 * z) / rayleigh, 2));
      default: return 0;
    }
  }
  double relativeIntensity(double i) const {
    switch (profile) {
      case NLM_GAUSSIAN_BEAM: return 1 / (1 + std::pow((i * dz - 0.5 * z) / rayleigh, 2));
      case NLM_CONSTANT: return 1.;
      case NLM_GAUSSIAN_APODIZATION: return std::exp(-std::pow((i * dz - 0.5 * z) / rayleigh, 2));
      default: return 0;
    }
  }

  // Per-step coefficients of each solver's DiffEq, evaluated with the reference's expressions.
  void stepCoefficients(uint i, int sub, cplx* c) const {
    const double prevPol = poling.empty() ? 1.0 : poling[i - 1];
    const double currPol = poling.empty() ? 1.0 : poling[i];
    const double intmPol = 0.5 * (prevPol + currPol);
    const double pol = sub == 0 ? prevPol : (sub == 1 ? intmPol : currPol);
    auto zpos = [&](void) -> double {
      return sub == 0 ? (double)(i - 1) * dz : (sub == 1 ? (i - .5) * dz : (double)i * dz);
    };
    auto mism = [&](double db) { return std::exp(1.0 * kI * db * zpos()); };
    auto chirped = [&](void) {
      const double arg = 0.5 * (diffBeta0[1] - diffBeta0[0]) / z;
      const double s = sub == 0 ? (double)(i - 1) : (sub == 1 ? i - .5 : (double)i);
      return std::exp(0.5 * kI * ((diffBeta0[0] + s * dz * arg) * s * dz));
    };
    const double relAmp = relativeAmplitude(sub == 0 ? (double)(i - 1) : (sub == 1 ? i - .5 : (double)i));
    switch (solver) {
      case kChi3:  // solvers/Chi3.cpp:81-84
        c[0] = nlStep[0];
        break;
      case kChi2PDC: {  // solvers/Chi2PDC.cpp:36-43
        c[0] = pol * nlStep[0] * mism(diffBeta0[0]);
        break;
      }
      case kChi2SFG: {  // solvers/Chi2SFG.cpp:37-52
        const cplx m = mism(diffBeta0[0]);
        c[0] = pol * nlStep[0] * m;
        c[1] = pol * nlStep[1] * (1. / m);
        break;
      }
      case kChi2AFC: {  // solvers/Chi2AFC.cpp:35-50
        const cplx m = chirped();
        c[0] = nlStep[0] * m;
        c[1] = nlStep[1] * (1. / m);
        break;
      }
      case kChi2SFGPDC: {  // solvers/Chi2SFGPDC.cpp:37-58
        const cplx m = mism(diffBeta0[0]);
        c[0] = pol * nlStep[0] * m;
        c[1] = pol * nlStep[1];
        c[2] = 1. / m;
        c[3] = mism(diffBeta0[1]);
        break;
      }
      case kChi2SFGII: {  // solvers/Chi2SFGII.cpp:43-89; the last stage keeps prevPolDir (:86-89)
        const double p = sub == 2 ? prevPol : pol;
        const cplx mcz = mism(diffBeta0[0]), mcy = mism(diffBeta0[1]), msz = mism(diffBeta0[2]);
        c[0] = cplx(p, 0);
        c[1] = nlStep[0] * mcz;
        c[2] = nlStep[1] * msz;
        c[3] = p * nlStep[0] * mcy;
        c[4] = nlStep[0] * (1. / mcy);
        c[5] = nlStep[1] * (1. / msz);
        c[6] = p * nlStep[0] * (1. / mcz);
        break;
      }
      case kChi2PDCII: {  // solvers/Chi2PDCII.cpp:38-54
        const cplx m = mism(diffBeta0[0]);
        c[0] = pol * nlStep[0] * m;
        c[1] = pol * nlStep[1] * m;
        break;
      }
      case kChi2SFGOPA: {  // solvers/Chi2SFGOPA.cpp:44-76
        const cplx ms = mism(diffBeta0[0]), md = mism(diffBeta0[1]);
        c[0] = pol * nlStep[0] * ms;
        c[1] = pol * nlStep[2] * md;
        c[2] = pol * nlStep[1] * (1. / ms);
        c[3] = pol * nlStep[3] * md;
        break;
      }
      case kChi2SFGXPM: {  // solvers/Chi2SFGXPM.cpp:38-57
        const cplx m = mism(diffBeta0[0]);
        c[0] = pol * nlStep[0] * m;
        c[1] = pol * nlStep[1] * (1. / m);
        c[2] = nlStep[2];
        c[3] = nlStep[3];
        break;
      }
      case kChi2SHG: {  // solvers/Chi2SHG.cpp:32-59
        const double rel = pol * relAmp;
        const cplx m = mism(diffBeta0[0]);
        c[0] = rel * nlStep[0] * m;
        c[1] = rel * nlStep[1] * (1. / m) * .5;
        break;
      }
      case kChi2SHGOPA: {  // solvers/Chi2SHGOPA.cpp:39-83
        const double rel = pol * relAmp;
        const cplx ms = mism(diffBeta0[0]), mo = mism(diffBeta0[1]);
        c[0] = rel * nlStep[0] * ms;
        c[1] = rel * nlStep[1];
        c[2] = mo;
        c[3] = (1. / ms) * .5;
        c[4] = rel * nlStep[2] * (1. / mo);
        c[5] = rel * nlStep[3] * (1. / mo);
        break;
      }
      case kChi2DSFG: {  // solvers/Chi2DSFG.cpp:31-64
        const double rel = pol * relAmp;
        const cplx m = mism(diffBeta0[0]);
        c[0] = rel * nlStep[0] * m;
        c[1] = rel * nlStep[1] * (1. / m);
        c[2] = rel * nlStep[2] * m;
        break;
      }
      case kChi2SHGXPM: {  // solvers/Chi2SHGXPM.cpp:29-41
        const double rel = pol * relAmp;
        const cplx m = mism(diffBeta0[0]);
        c[0] = rel * nlStep[0] * m;
        c[1] = rel * nlStep[1] * (1. / m) * .5;
        c[2] = std::pow(relAmp, 2) * nlStep[2];
        break;
      }
      case kChi2ASHG: {  // solvers/Chi2ASHG.cpp:28-55
        const cplx m = chirped();
        c[0] = relAmp * nlStep[0] * m;
        c[1] = relAmp * nlStep[1] * (1. / m) * .5;
        break;
      }
      default:
        break;
    }
  }

  void buildCoefficients() {
    const int nc = kSolvers[solver].coefs;
    if (nc == 0 || nZ < 2) return;
    std::vector<double2> h((size_t)(nZ - 1) * 3 * nc);
    std::vector<cplx> c(nc);
    for (uint i = 1; i < nZ; i++)
      for (int sub = 0; sub < 3; sub++) {
        stepCoefficients(i, sub, c.data());
        for (int k = 0; k < nc; k++)
          h[((size_t)(i - 1) * 3 + sub) * nc + k] = make_double2(c[k].real(), c[k].imag());
      }
    upload(coef, h);
  }

  // Raman response and self-steepening operator, solvers/Chi3GNLSE.cpp:20-36, :287
  void buildGnlse() {
    const double coeff1 = fr * (1. - fb) * (tau1 / (tau2 * tau2) + 1. / tau1);
    const double coeff2 = fr * fb / (tau3 * tau3);
    std::vector<double2> rt(N, make_double2(0, 0));
    for (uint k = 0; k < N / 2; k++) {
      const double t = tau[k];
      rt[k].x = coeff1 * std::exp(-t / tau2) * std::sin(t / tau1) + coeff2 * std::exp(-t / tau3) * (2 * tau3 - t);
    }
    rt[0].x += 1. - fr;
    DevBuf<double2> tmp;
    upload(tmp, rt);
    work.reserve(N);
    FFTPlanH plan = fftPlanRows();
    ck(launch_fft_rows(tmp.p, work.p, 1, plan, tw, false, 1.0, nullptr, stream), "raman fft");
    launches++;
    std::vector<double2> hr(N);
    ck(cudaMemcpyAsync(hr.data(), work.p, N * sizeof(double2), cudaMemcpyDeviceToHost, stream), "raman");
    ck(cudaStreamSynchronize(stream), "raman");
    raman.resize(N);
    std::vector<double2> rs(N), st(N);
    const double invN = 1.0 / N;
    for (uint k = 0; k < N; k++) {
      raman[k] = cplx(hr[k].x, hr[k].y);
      rs[k] = make_double2(hr[k].x * invN, hr[k].y * invN);
      const cplx s = (nlStep[0] + nlStep[1] * omega[k]) * invN;
      st[k] = make_double2(s.real(), s.imag());
    }
    upload(ramanD, rs);
    upload(steepD, st);
    std::vector<double> rel((size_t)(nZ > 1 ? nZ - 1 : 0) * 3);
    for (uint i = 1; i < nZ; i++) {
      rel[(i - 1) * 3 + 0] = relativeIntensity((double)(i - 1));
      rel[(i - 1) * 3 + 1] = relativeIntensity(i - .5);
      rel[(i - 1) * 3 + 2] = relativeIntensity((double)i);
    }
    uploadD(relIntD, rel);
  }

  // Plan of the batched row transforms (pump grids, chirp and delay, Raman response): the register
  // plan on power-of-two grids, the general plan on the others.
  FFTPlanH fftPlanRows() const {
    if (N <= (uint)kMaxFFT) return make_plan((int)N, N <= 4096 ? 8 : 16);
    FFTPlanH p{};
    p.N = (int)N;
    p.T = 0;   // no plan: the direct DFT
    return p;
  }

  // ---- pumps -----------------------------------------------------------------------------
  // src/_NonlinearMedium.cpp:198-203
  void chirpDelay(uint idx, double chirp, double delay) {
    if (chirp == 0 && delay == 0) return;
    ensureDevice();
    std::vector<double2> e(N), ph(N);
    for (uint k = 0; k < N; k++) {
      e[k] = make_double2(envelope[idx][k].real(), envelope[idx][k].imag());
      const cplx p = std::exp(1.0 * kI * (beta1[idx] * delay + 0.5 * beta2[idx] * chirp * omega[k]) * omega[k]);
      ph[k] = make_double2(p.real(), p.imag());
    }
    DevBuf<double2> de, dph, spec;
    upload(de, e);
    upload(dph, ph);
    spec.alloc(N);
    FFTPlanH plan = fftPlanRows();
    ck(launch_fft_rows(de.p, spec.p, 1, plan, tw, false, 1.0, dph.p, stream), "chirp fft");
    ck(launch_fft_rows(spec.p, de.p, 1, plan, tw, true, 1.0 / N, nullptr, stream), "chirp ifft");
    launches += 2;
    ck(cudaMemcpyAsync(e.data(), de.p, N * sizeof(double2), cudaMemcpyDeviceToHost, stream), "chirp");
    ck(cudaStreamSynchronize(stream), "chirp");
    for (uint k = 0; k < N; k++) envelope[idx][k] = cplx(e[k].x, e[k].y);
  }

  void setPumpType(int pulseType, double chirp, double delay, uint idx) {
    if (fnl || isCascade) throw std::runtime_error("Object does not have this method.");
    setPumpTypeImpl(pulseType, chirp, delay, idx);
  }
  // src/_NonlinearMedium.cpp:180-204
  void setPumpTypeImpl(int pulseType, double chirp, double delay, uint idx) {
    if (idx >= nPump) throw std::invalid_argument("Invalid pump index");
    std::vector<cplx>& env = envelope[idx];
    env.assign(N, 0);
    switch (pulseType) {
      default:
      case NLM_GAUSSIAN:
        for (uint k = 0; k < N; k++) env[k] = std::exp(-0.5 * (tau[k] * tau[k]));
        break;
      case NLM_SECH:
        for (uint k = 0; k < N; k++) env[k] = 1 / std::cosh(tau[k]);
        break;
      case NLM_SINC:
        for (uint k = 0; k < N; k++) env[k] = std::sin(tau[k]) / tau[k];
        env[0] = 1;
    }
    chirpDelay(idx, chirp, delay);
  }
  void setPumpCustom(const double* p, size_t n, double chirp, double delay, uint idx) {
    if (fnl || isCascade) throw std::runtime_error("Object does not have this method.");
    setPumpCustomImpl(p, n, chirp, delay, idx);
  }
  // src/_NonlinearMedium.cpp:207-222
  void setPumpCustomImpl(const double* p, size_t n, double chirp, double delay, uint idx) {
    if (n != N) throw std::invalid_argument("Custom pump array length does not match number of frequency/time bins");
    if (idx >= nPump) throw std::invalid_argument("Invalid pump index");
    envelope[idx].resize(N);
    for (uint k = 0; k < N; k++) envelope[idx][k] = cplx(p[2 * k], p[2 * k + 1]);
    chirpDelay(idx, chirp, delay);
  }

  void relativeStrength(std::vector<double>& s) const {
    s.assign(nZP, 1.0);
    const double lo = -0.5 * z, hi = 0.5 * z;
    const double step = nZP > 1 ? (hi - lo) / (nZP - 1) : 0;
    for (uint i = 0; i < nZP; i++) {
      const double zz = (i + 1 == nZP) ? hi : lo + i * step;
      const double x = zz / rayleigh;
      s[i] = profile == NLM_GAUSSIAN_APODIZATION ? std::exp(-0.5 * (x * x)) : 1 / std::sqrt(1 + x * x);
    }
  }

  void runPump() {
    if (fnl || isCascade) throw std::runtime_error("Object does not have this method.");
    ensureDevice();
    if (solver == kChi3) {
      runPumpChi3();
    } else {
      // src/_NonlinearMedium.cpp:225-250
      FFTPlanH plan = fftPlanRows();
      DevBuf<double2> env;
      for (uint m = 0; m < nPump; m++) {
        std::vector<double2> e(N);
        for (uint k = 0; k < N; k++) e[k] = make_double2(envelope[m][k].real(), envelope[m][k].imag());
        upload(env, e);
        double2* pf = pumpFreq.p + (size_t)m * nZP * N;
        double2* pt = pumpTime.p + (size_t)m * nZP * N;
        ck(launch_fft_rows(env.p, pf, 1, plan, tw, false, 1.0, nullptr, stream), "pump fft");
        ck(launch_pump_linear(pf, dispPumpD.p + (size_t)m * N, dzp, (int)nZP, (int)N, pf, stream), "pump phase");
        if (nZP > 1) ck(launch_fft_rows(pf + N, pt + N, nZP - 1, plan, tw, true, 1.0 / N, nullptr, stream), "pump ifft");
        ck(cudaMemcpyAsync(pt, env.p, N * sizeof(double2), cudaMemcpyDeviceToDevice, stream), "pump row 0");
        launches += 3;
        if (profile != NLM_CONSTANT) {
          std::vector<double> s;
          relativeStrength(s);
          DevBuf<double> sd;
          uploadD(sd, s);
          ck(launch_scale_rows(pf, sd.p, (int)nZP, (int)N, stream), "pump profile");
          ck(launch_scale_rows(pt, sd.p, (int)nZP, (int)N, stream), "pump profile");
          launches += 2;
          ck(cudaStreamSynchronize(stream), "pump");
        }
        ck(cudaStreamSynchronize(stream), "pump");
      }
    }
    pumpVersion++;
  }

  // solvers/Chi3.cpp:41-70
  void runPumpChi3() {
    if (N < 2 || N > (uint)kMaxFFT)
      throw Unsupported("the Chi3 pump march takes grids of 2 to " + std::to_string(kMaxFFT) + " points");
    // one CTA marches the pump: N/4 threads up to N=512 so that all four schedulers of the SM issue;
    // the general plan (ceil(N/R) threads) on grids that are not powers of two
    FFTPlanH plan = make_plan((int)N, N <= 512 ? 4 : (N <= 4096 ? 8 : 16));
    std::vector<double2> e(N), hP(N), dP(N), bP(N);
    for (uint k = 0; k < N; k++) {
      e[k] = make_double2(envelope[0][k].real(), envelope[0][k].imag());
      const cplx h = std::exp((0.5 * kI * dzp) * dispPump[0][k]);
      const cplx b = std::exp((-0.5 * kI * dzp) * dispPump[0][k]);
      hP[k] = make_double2(h.real(), h.imag());
      dP[k] = make_double2(dstepPump[0][k].real(), dstepPump[0][k].imag());
      bP[k] = make_double2(b.real(), b.imag());
    }
    std::vector<double2> rel(nZP);
    const cplx scale = dzp / dz * nlStep[0];
    const double lo = -0.5 * z, hi = 0.5 * z, step = nZP > 1 ? (hi - lo) / (nZP - 1) : 0;
    for (uint i = 0; i < nZP; i++) {
      const double zz = (i + 1 == nZP) ? hi : lo + i * step;
      const double x = zz / rayleigh;
      cplx r;
      switch (profile) {
        default:
        case NLM_CONSTANT: r = scale; break;
        case NLM_GAUSSIAN_BEAM: r = scale / (1 + x * x); break;
        case NLM_GAUSSIAN_APODIZATION: r = scale * std::exp(-(x * x)); break;
      }
      rel[i] = make_double2(r.real(), r.imag());
    }
    if (pipePumpGrid()) {
      DeferredPump& q = deferredPump;
      upload(q.env, e);
      upload(q.half, hP);
      upload(q.dstep, dP);
      upload(q.back, bP);
      upload(q.rel, rel);
      ck(cudaStreamSynchronize(stream), "chi3 pump tables");
      q.pending = true;
      return;
    }
    DevBuf<double2> de, dh, dd, db, dr;
    upload(de, e);
    upload(dh, hP);
    upload(dd, dP);
    upload(db, bP);
    upload(dr, rel);
    if (spreadGrid() || wideGrid()) {
      // the march on four (up to 1024 points) or eight SMs with one point per thread (prop_spread.cu)
      ck(launch_pump_chi3_spread(pumpFreq.p, pumpTime.p, de.p, dh.p, dd.p, db.p, dr.p, (int)nZP, (int)N, tw, stream),
         "chi3 pump (spread)");
    } else if (useCluster && is_pow2((int)N) && N >= 1024) {
      // 1024..8192 points: the march on four SMs (prop_cluster_pump.cu), four points per thread
      const FFTPlanH local = make_plan((int)N / kClusterSize, kClusterSize);
      ck(launch_pump_chi3_cluster(pumpFreq.p, pumpTime.p, de.p, dh.p, dd.p, db.p, dr.p, (int)nZP, local, tw, stream),
         "chi3 pump (cluster)");
    } else {
      ck(launch_pump_chi3(pumpFreq.p, pumpTime.p, de.p, dh.p, dd.p, db.p, dr.p, (int)nZP, plan, tw, stream),
         "chi3 pump");
    }
    launches++;
    ck(cudaStreamSynchronize(stream), "chi3 pump");
  }

  // The Chi3 pump march runs beside the next signal propagation: cluster mode 1, 128..1024 points (the
  // four-CTA spread form), one pump row per half step.
  bool pipePumpGrid() const {
    return solver == kChi3 && useCluster == 1 && spreadGrid() && nZ >= 2 && nZP == 2 * nZ - 1 && nSignal == 1;
  }

  PumpMarchArgs deferredPumpArgs() const {
    const DeferredPump& q = deferredPump;
    return PumpMarchArgs{pumpFreq.p, pumpTime.p, q.env.p, q.half.p, q.dstep.p, q.back.p, q.rel.p, (int)nZP};
  }

  // Runs a deferred pump march alone (four CTAs, k_pump_chi3_spread) and waits for it.  The march stays
  // deferred if its launch fails, so the next reader tries again rather than reading stale grids.
  void flushPump() {
    if (!deferredPump.pending) return;
    const PumpMarchArgs p = deferredPumpArgs();
    ck(launch_pump_chi3_spread(p.pf, p.pt, p.env, p.halfP, p.dstepP, p.backP, p.rel, p.nRows, (int)N, tw, stream),
       "chi3 pump (spread)");
    deferredPump.pending = false;
    launches++;
    ck(cudaStreamSynchronize(stream), "chi3 pump");
  }

  // src/_NonlinearMedium.cpp:506-534
  void setPumpFrom(Medium& other, uint modeIndex, double delay, uint idx) {
    if (fnl || isCascade) throw std::runtime_error("Object does not have this method.");
    flushPump();
    if (other.isCascade) throw std::invalid_argument("Medium does not have same time and frequency axes as this one");
    if (other.N != N || other.tMax != tMax)
      throw std::invalid_argument("Medium does not have same time and frequency axes as this one");
    if (modeIndex >= nSignal) throw std::invalid_argument("Mode index larger than number of modes in medium");
    if (idx >= nPump) throw std::invalid_argument("Invalid pump index");
    if (other.nZ < nZ) throw std::invalid_argument("Medium does not have sufficient resolution to be used with this one");
    if (modeIndex >= other.nSignal) throw std::invalid_argument("Mode index larger than number of modes in medium");
    ensureDevice();
    other.ensureDevice();
    ck(cudaStreamSynchronize(other.stream), "other medium");
    const double ratio = static_cast<double>(other.nZ - 1) / (nZP - 1);
    double2* pf = pumpFreq.p + (size_t)idx * nZP * N;
    double2* pt = pumpTime.p + (size_t)idx * nZP * N;
    ck(launch_pump_from(other.sigFreq.p + (size_t)modeIndex * other.nZ * N, (int)other.nZ, ratio, other.dz,
                        dispPumpD.p + (size_t)idx * N, other.dispSignD.p + (size_t)modeIndex * N, dzp,
                        beta1[idx] * delay, omegaD.p, (int)nZP, (int)N, z, other.z, pf, stream),
       "pump from");
    FFTPlanH plan = fftPlanRows();
    // rows 0..nZStepsP-2; the reference then re-transforms row nZSteps-1 (unchanged) and leaves the
    // last time-domain row as it was (src/_NonlinearMedium.cpp:533)
    if (nZP > 1) ck(launch_fft_rows(pf, pt, nZP - 1, plan, tw, true, 1.0 / N, nullptr, stream), "pump from ifft");
    launches += 2;
    ck(cudaStreamSynchronize(stream), "pump from");
    pumpVersion++;
  }

  // ---- propagation --------------------------------------------------------------------------
  int chooseR() const {
    const int M = (int)nSignal;
    if (solver == kChi3GNLSE) return 8;
    if (M >= 3) return 4;
    if (M == 1 && N > 4096) return 16;
    return 8;
  }

  static const KernelEntry* findKernelFn(const void* fn) {
    int count = 0;
    const KernelEntry* t = kernel_table(&count);
    for (int i = 0; i < count; i++)
      if (t[i].fn == fn) return &t[i];
    return nullptr;
  }

  const KernelEntry* findKernel(int kind, int key, int R) const {
    int count = 0;
    const KernelEntry* t = kernel_table(&count);
    for (int i = 0; i < count; i++)
      if (t[i].kind == kind && t[i].key == key && (R == 0 || t[i].R == R)) return &t[i];
    return nullptr;
  }

  bool linearSolver() const { return kSolvers[solver].linear; }

  static int smCount() {
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
  }

  // A grid that a cluster propagation can take (1024 to 8192 points); whether a launch runs on
  // clusters is decided in propagate(), which checks the one-CTA kernels' limits otherwise.
  bool clusterGrid() const {
    return useCluster && is_pow2((int)N) && N >= 1024 && N <= (uint)kMaxFFT &&
           findKernel(kKindCluster, solver, kClusterSize) != nullptr;
  }

  // Grids some propagation kernel takes: cluster grids, register-plan grids, and every other grid of
  // 2..kMaxFFT points on the general plan (propagate() picks the kernel).
  void checkGrid(int R) const {
    if (clusterGrid() || registerGrid(R)) return;
    if (N < 2 || N > (uint)kMaxFFT)
      throw Unsupported("grid of " + std::to_string(N) + " points: the fused split-step kernels take 2 to " +
                        std::to_string(kMaxFFT) + " points");
  }

  void checkGridStrict(int R) const {
    if (!is_pow2((int)N) || (int)N < R || N > (uint)kMaxFFT || N / R > 512)
      throw Unsupported("grid of " + std::to_string(N) + " points is not supported by the fused split-step kernels "
                        "(power of two, R=" + std::to_string(R) + " to 8192 points)");
  }

  // The register plan's one-CTA kernels take power-of-two grids of at least R points with N/R <= 512
  // threads; every other grid up to kMaxFFT points runs on the general plan (FFTPlanH::gen).
  bool registerGrid(int R) const { return is_pow2((int)N) && (int)N >= R && N <= (uint)kMaxFFT && N / R <= 512; }

  // The general-plan kernel of `kind` for `key` (registered at key + kGenKey) with the fewest points
  // per thread, from R up, whose CTA holds a propagation (ceil(N/R) <= 512 threads); sets *Rout.
  const KernelEntry* genKernel(int kind, int key, int R, int* Rout) const {
    if (N > (uint)kMaxFFT || N < 2)
      throw Unsupported("grid of " + std::to_string(N) + " points: the fused split-step kernels take 2 to " +
                        std::to_string(kMaxFFT) + " points");
    for (int r : {4, 8, 16}) {
      if (r < R || ((int)N + r - 1) / r > 512) continue;
      if (const KernelEntry* k = findKernel(kind, key + kGenKey, r)) {
        *Rout = r;
        return k;
      }
    }
    return nullptr;
  }

  struct Schedule {
    int grid, block, ipc;
    size_t smem;
    int maxActive, ctas;   // occupancy limit and chosen resident CTAs per SM
  };

  // Launch shape of a persistent propagation kernel: ipc propagations per CTA (N/R threads each; by
  // default enough for 128 threads, times ipcMul), `cta` resident CTAs per SM (0: the member
  // override or the occupancy maximum), grid = SMs x CTAs per SM, capped by the number of groups.
  Schedule schedule(const KernelEntry* k, long long nInst, int R, int cta = 0, int ipcMul = 1) {
    const int T = ((int)N + R - 1) / R;   // N / R on the register plan, ceil(N / R) on the general one
    int ipc = (T >= 128 ? 1 : 128 / T) * ipcMul;
    if (ipc > nInst) ipc = (int)std::max<long long>(1, nInst);
    const int block = T * ipc;
    // exchange buffers of the ipc propagations, plus the staged twiddle table when R != 16
    const size_t smem = (size_t)(ipc + (k->R != 16 ? 1 : 0)) * N * sizeof(double2);
    int dev = 0, sms = 1, optin = 0;
    ck(cudaGetDevice(&dev), "device");
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa;
    ck(cudaFuncGetAttributes(&fa, k->fn), "kernel attributes");
    const int dynMax = optin - (int)fa.sharedSizeBytes;   // static shared memory counts against the opt-in limit
    if ((int)smem > dynMax) throw Unsupported("grid too large for shared memory");
    ck(cudaFuncSetAttribute(k->fn, cudaFuncAttributeMaxDynamicSharedMemorySize, dynMax), "smem attribute");
    if (block > fa.maxThreadsPerBlock)
      throw Unsupported("propagation kernel cannot launch " + std::to_string(block) + " threads (registers)");
    int maxActive = 0;
    ck(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&maxActive, k->fn, block, smem), "occupancy");
    if (maxActive < 1) throw Unsupported("propagation kernel does not fit on an SM");
    const long long groups = (nInst + ipc - 1) / ipc;
    // The kernels claim groups from a work counter, so every SM keeps working until the queue is
    // empty whatever the number of resident CTAs: take the most resident warps (the FP64 pipe is
    // shared by all of them and needs several warps per scheduler to stay busy).
    int best = maxActive;
    if (cta > 0) best = std::min(cta, maxActive);
    else if (ctaPerSM > 0) best = std::min(ctaPerSM, maxActive);
    long long grid = std::min<long long>(groups, (long long)sms * best);
    Schedule s{(int)std::max<long long>(1, grid), block, ipc, smem, maxActive, best};
    return s;
  }

  // ---- autotuner -----------------------------------------------------------------------------
  // For a batched launch it times every registered kernel variant of the path (points per thread R),
  // ipc multiplier {1, 2} and resident CTAs per SM on the real arguments with the z march cut to a
  // few steps, and keeps the fastest per (kernel kind, key, grid, propagation count) for the process.
  struct TuneChoice {
    int R = 0, cta = 0, ipcMul = 1;
    float ms = 0;
    const void* fn = nullptr;   // the kernel variant (several may share kind, key and R)
  };
  static std::mutex& tuneMutex() {
    static std::mutex mu;
    return mu;
  }
  static std::map<std::vector<unsigned char>, TuneChoice>& tuneTable() {
    static std::map<std::vector<unsigned char>, TuneChoice> t;
    return t;
  }
  static bool autotuneEnabled() {
    const char* e = std::getenv("NLM_AUTOTUNE");
    return !(e && e[0] == '0');
  }
  DevBuf<unsigned long long> tuneCounter;
  Schedule lastSchedule{};
  int lastR = 0, lastTuned = 0, lastRegs = 0;
  long tuneTrials = 0;

  bool tuneWanted(const PropArgs& a, long long nInst) const {
    if (ctaPerSM != 0 || !autotuneEnabled()) return false;
    if (a.gridF || a.gridT || a.ckpt) return false;
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    if (stream == nullptr || cudaStreamIsCapturing(stream, &st) != cudaSuccess || st != cudaStreamCaptureStatusNone)
      return false;
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return nInst >= 2LL * sms;
  }

  void launchKernel(const KernelEntry* k, const Schedule& s, const PropArgs& a, const FFTables* ffT) {
    if (ffT) {
      void* args[] = {(void*)&a, (void*)ffT};
      ck(cudaLaunchKernel(k->fn, dim3(s.grid), dim3(s.block), args, s.smem, stream), "propagate");
    } else {
      void* args[] = {(void*)&a};
      ck(cudaLaunchKernel(k->fn, dim3(s.grid), dim3(s.block), args, s.smem, stream), "propagate");
    }
  }

  TuneChoice autotune(int kind, int key, const PropArgs& a0, long long nInst, const FFTables* ffT) {
    GraphKey tk;
    tk.add(kind).add(key).add(N).add(nInst).add(nSignal).add(a0.inKind).add(a0.inTime).add(a0.nOut);
    {
      std::lock_guard<std::mutex> g(tuneMutex());
      auto it = tuneTable().find(tk.bytes);
      if (it != tuneTable().end()) return it->second;
    }
    int count = 0;
    const KernelEntry* t = kernel_table(&count);
    TuneChoice best;
    best.ms = 1e30f;
    tuneCounter.reserve(1);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ck(cudaEventCreate(&e0), "event");
    ck(cudaEventCreate(&e1), "event");
    try {
      for (int i = 0; i < count; i++) {
        const KernelEntry* kc = &t[i];
        if (kc->kind != kind || kc->key != key) continue;
        const int R = kc->R;
        if (!is_pow2((int)N) || (int)N < R || N / R > 512 || N > (uint)kMaxFFT) continue;
        // the four-points-per-thread variant of the single-mode propagator serves latency-bound launches
        // (fewer propagations than SMs), which are not tuned; for two modes it is a candidate (the
        // eight-point variant spills)
        if (kind == kKindLinear && key == 1 && R == 4) continue;
        for (int ipcMul = 1; ipcMul <= 2; ipcMul++) {
          Schedule base;
          try {
            base = schedule(kc, nInst, R, 0, ipcMul);
          } catch (const Unsupported&) {
            continue;
          }
          for (int c = 1; c <= base.maxActive; c++) {
            const Schedule sc = schedule(kc, nInst, R, c, ipcMul);
            PropArgs ta = a0;
            ta.plan = make_plan((int)N, R);
            ta.R = R;
            ta.nZ = std::min<int>(a0.nZ, 17);
            ta.nInst = nInst;
            ta.ipc = sc.ipc;
            const bool counter = (long long)sc.grid < (nInst + sc.ipc - 1) / sc.ipc;
            ta.work = counter ? tuneCounter.p : nullptr;
            float ms = 0;
            for (int rep = 0; rep < 2; rep++) {
              if (counter) ck(cudaMemsetAsync(tuneCounter.p, 0, sizeof(unsigned long long), stream), "tune counter");
              ck(cudaEventRecord(e0, stream), "event");
              launchKernel(kc, sc, ta, ffT);
              ck(cudaEventRecord(e1, stream), "event");
              ck(cudaEventSynchronize(e1), "tune");
              ck(cudaEventElapsedTime(&ms, e0, e1), "event");
            }
            launches += 2;
            tuneTrials++;
            if (ms < best.ms) best = TuneChoice{R, c, ipcMul, ms, kc->fn};
          }
        }
      }
    } catch (...) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (best.R == 0) return best;
    std::lock_guard<std::mutex> g(tuneMutex());
    tuneTable()[tk.bytes] = best;
    return best;
  }

  // The launch description every kernel starts from; a deferred pump march runs first, since the
  // launch may read the pump grids.
  PropArgs baseArgs(int R) {
    flushPump();
    return plainArgs(R);
  }

  PropArgs plainArgs(int R) const {
    PropArgs a{};
    a.plan = make_plan((int)N, R);
    a.R = R;
    a.nModes = (int)nSignal;
    a.nZ = (int)nZ;
    a.tw = tw;
    a.dstep = dstep.p;
    a.dlast = dlast.p;
    a.half = half.p;
    a.back = back.p;
    a.pump = pumpTime.p;
    a.pumpStride = (long long)nZP * N;
    a.nPumps = (int)nPump;
    a.coef = coef.p;
    a.nCoef = kSolvers[solver].coefs;
    a.raman = ramanD.p;
    a.steep = steepD.p;
    a.relInt = relIntD.p;
    return a;
  }

  // The propagator's device buffer at its size, allocated ahead of a graph capture (which may not
  // allocate); buildPropagator then finds it in place.
  void reservePropagator() {
    const int M = (int)nSignal, E = 4 * M * M;
    const size_t count = (size_t)(nZ > 1 ? nZ - 1 : 0) * E * N;
    if (count) prop.alloc(count + 2 * kTablePad);
  }

  // on: the stream of the build (default: the medium's own)
  void buildPropagator(int R, cudaStream_t on = nullptr) {
    if (propVersion == pumpVersion && prop.p) return;
    const int M = (int)nSignal, E = 4 * M * M;
    const size_t count = (size_t)(nZ > 1 ? nZ - 1 : 0) * E * N;
    if (count == 0) return;
    prop.alloc(count + 2 * kTablePad);   // doubles; the padding is zeroed like that of the tables
    ck(cudaMemsetAsync(prop.p + count, 0, 2 * kTablePad * sizeof(double), on ? on : stream), "propagator");
    const KernelEntry* k = findKernel(kKindBuildProp, solver, 0);
    if (!k) throw Unsupported("no propagator kernel for this solver");
    PropArgs a = baseArgs(R);
    a.prop = prop.p;
    const long long total = (long long)(nZ - 1) * N;
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long grid = (total + 127) / 128;
    grid = std::min<long long>(grid, (long long)sms * 16);
    void* args[] = {(void*)&a};
    ck(cudaLaunchKernel(k->fn, dim3((unsigned)grid), dim3(128), args, 0, on ? on : stream), "propagator build");
    launches++;
    propVersion = pumpVersion;
    propBuilds++;
  }

  // ---- cluster-distributed propagation (prop_cluster.cu) -------------------------------------
  static constexpr int kClusterSize = 4;   // CTAs per propagation; also the points per thread
  // 1: clusters, with one point per thread on the grids of spreadGrid(); 2: four points per thread
  // only; 0: one CTA per propagation
  int useCluster = 1;
  static constexpr uint kSpreadMinN = 128, kSpreadMaxN = 1024, kWideMaxN = 4096;

  // A grid whose single propagations run on a 4-CTA cluster with one point per thread (prop_spread.cu):
  // M = N/4 threads per CTA gives one to eight warps per SM, where the four-points-per-thread cluster
  // form would give at most two (or, below 1024 points, is not built) and one CTA has one SM's FP64.
  // cluster mode 3 is mode 1 without the widest forms (sixteen CTAs on 2048 and 4096 points, eight on
  // 1024): four CTAs up to 1024 points and eight above, as a reference for them
  bool spreadGrid() const {
    return (useCluster == 1 || useCluster == 3) && is_pow2((int)N) && N >= kSpreadMinN && N <= kSpreadMaxN;
  }
  // 2048- and 4096-point grids: one point per thread on eight CTAs (prop_spread_b.cu), twice the SMs of
  // the four-points-per-thread cluster, for the launches that no reverse sweep pairs with (full grids,
  // the media of ragged batches marked by raggedWide) and the Chi3 pump march.
  bool wideGrid() const {
    return (useCluster == 1 || useCluster == 3) && is_pow2((int)N) && N > kSpreadMaxN && N <= kWideMaxN;
  }
  bool wideLaunch(const PropArgs& a) const {
    return wideGrid() && !a.ckpt && !a.stages && (a.gridF || a.gridT || raggedWide || raggedW16);
  }
  // Grids that take eight CTAs with one point per thread: 2048 and 4096 points, and in cluster mode 1
  // also 1024 points (128 per CTA) for full grids and the ragged media a plan gives that form
  bool w8Grid() const {
    return wideGrid() || (useCluster == 1 && N == kSpreadMaxN);
  }
  bool w8Launch(const PropArgs& a) const {
    if (!w8Grid() || a.ckpt || a.stages) return false;
    if (N > kSpreadMaxN) return wideLaunch(a);
    return raggedWide || a.gridF || a.gridT;
  }
  bool raggedWide = false;   // set by nlm_ragged_batch around the propagation of a medium given 8 CTAs
  bool raggedW16 = false;    // ... given 16 CTAs

  // The sixteen-CTA kernel of this medium (prop_spread_w16.cu; cluster mode 1): single-mode solvers,
  // and multi-mode solvers in the mode-fused form where its buffers fit in shared memory; nullptr
  // otherwise.
  const KernelEntry* w16Kernel() const {
    if (useCluster != 1 || !wideGrid()) return nullptr;
    const KernelEntry* k = nSignal < 2 ? findKernel(kKindCluster, solver + kSpreadW16Key, 1)
                                       : findKernel(kKindSpreadFused, solver + kSpreadW16Key, 1);
    if (!k || (nSignal >= 2 && !fusedFits(k, 16))) return nullptr;
    return w16Clusters(k) > 0 ? k : nullptr;
  }
  int w16Clusters(const KernelEntry* k) const { return spreadClusters(k, 16); }
  // C-CTA clusters of the one-point-per-thread kernel k for this grid, each CTA alone on its SM, that
  // the device holds at once (0 where none fits, e.g. sixteen CTAs on a partition without a GPC of
  // sixteen SMs).  A cluster sits in one GPC, so this can be well below SMs / C.  Queried once per
  // kernel, grid and C with the occupancy API.
  int spreadClusters(const KernelEntry* k, int C) const {
    static std::mutex mu;
    static std::map<std::tuple<const void*, uint, int>, int> known;
    std::lock_guard<std::mutex> lock(mu);
    const auto key = std::make_tuple(k->fn, N, C);
    auto it = known.find(key);
    if (it != known.end()) return it->second;
    const int M = (int)N / C;
    const long long perPoint = k->kind == kKindSpreadFused ? spread_smem_per_point_k(C, (int)nSignal)
                                                           : spread_smem_per_point(C);
    size_t smem = 0;
    int n = 0;
    if (exclusive_smem(k->fn, (size_t)perPoint * M * sizeof(double2), &smem) == cudaSuccess && smem &&
        (C <= 8 || cudaFuncSetAttribute(k->fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess)) {
      cudaLaunchAttribute attr;
      cudaLaunchConfig_t cfg = cluster_config(C, M, smem, nullptr, C, &attr);
      if (cudaOccupancyMaxActiveClusters(&n, k->fn, &cfg) != cudaSuccess) n = 0;
    }
    cudaGetLastError();
    known[key] = n;
    return n;
  }

  // Chi3GNLSE launches of few rows in cluster mode 1: the CTAs per row of the one-point-per-thread form
  // (prop_gnlse_spread.cu) whose clusters hold every row at once, the most first (16, 8, 4) with at
  // least 128 threads per CTA (at most 256 on sixteen CTAs, 512 otherwise); 0 when none applies (then
  // four points per thread on four CTAs).  The stored-stage reverse sweep takes the same form.
  int gnlseSpreadC(long long rows) const {
    if (solver != kChi3GNLSE || useCluster != 1 || !is_pow2((int)N)) return 0;
    for (int C : {16, 8, 4}) {
      const int M = (int)N / C;
      if (M < 128 || M > (C == 16 ? 256 : 512) || rows * C > smCount()) continue;
      const KernelEntry* k = C == 16 ? findKernel(kKindCluster, solver + kSpreadW16Key, 1)
                                     : findKernel(kKindCluster, C == 8 ? solver + kSpreadWideKey : solver, 1);
      if (!k || !findKernel(kKindAdjoint, solver + 500, C)) continue;
      if (spreadClusters(k, C) < rows) continue;
      return C;
    }
    return 0;
  }

  const KernelEntry* clusterKernel(const PropArgs& a, long long nInst, bool plainOne) const {
    // checkpointed forwards (the adjoint's, Chi2PDC and Chi3GNLSE) run on clusters too: their reverse
    // sweeps have cluster forms that read the same checkpoints
    if (!useCluster || plainOne || a.inKind != 1) return nullptr;
    if (!is_pow2((int)N) || N > (uint)kMaxFFT) return nullptr;
    if (const int Cs = gnlseSpreadC(nInst))
      return Cs == 16 ? findKernel(kKindCluster, solver + kSpreadW16Key, 1)
                      : findKernel(kKindCluster, Cs == 8 ? solver + kSpreadWideKey : solver, 1);
    // full grids and the ragged media given sixteen SMs: the sixteen-CTA form (mode 1); a ragged medium
    // given eight SMs keeps eight
    if (wideLaunch(a) && !raggedWide && nInst * 16 <= smCount())
      if (const KernelEntry* k16 = w16Kernel()) return k16;
    if (w8Launch(a) && nInst * 8 <= smCount())
      if (const KernelEntry* kw = findKernel(kKindCluster, solver + kSpreadWideKey, 1)) return fusedSpread(kw, 8);
    if (nInst * kClusterSize > smCount()) return nullptr;
    // the spread grids: one point per thread (the Chi2PDC reverse sweep has the same form,
    // adjoint_spread.cu; Chi3GNLSE, whose forward stores stage values, has no spread kernel)
    if (spreadGrid() && !a.stages)
      if (const KernelEntry* ks = findKernel(kKindCluster, solver, 1)) return fusedSpread(ks, kClusterSize);
    if (N < 1024) return nullptr;
    return findKernel(kKindCluster, solver, kClusterSize);
  }

  // The kernel of a multi-mode solver that transforms its modes together (kKindSpreadFused), in place of
  // the one-point-per-thread cluster kernel k of C CTAs, when its buffers fit in shared memory.
  const KernelEntry* fusedSpread(const KernelEntry* k, int C) const {
    if (nSignal < 2) return k;
    const KernelEntry* kf = findKernel(kKindSpreadFused, k->key, 1);
    return kf && fusedFits(kf, C) ? kf : k;
  }
  // whether the mode-fused kernel kf of C CTAs fits its buffers in one CTA's shared memory
  bool fusedFits(const KernelEntry* kf, int C) const {
    int dev = 0, optin = 0;
    cudaFuncAttributes fa;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
        cudaFuncGetAttributes(&fa, kf->fn) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    const long long need = spread_smem_per_point_k(C, (int)nSignal) * (long long)(N / C) * (long long)sizeof(double2);
    return need + (long long)fa.sharedSizeBytes <= optin;
  }

  void launchCluster(const KernelEntry* k, PropArgs a, long long nInst) {
    const bool spread = k->R == 1;   // one point per thread (prop_spread.cu, prop_spread_b.cu, prop_spread_w16.cu)
    const int C = k->key >= kSpreadW16Key ? 16 : k->key >= kSpreadWideKey ? 8 : kClusterSize;
    if (C > 8) ck(cudaFuncSetAttribute(k->fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1), "cluster size");
    const int M = (int)N / C;
    a.plan = make_plan(M, spread ? 1 : C);
    a.R = spread ? 1 : C;
    a.nInst = nInst;
    a.ipc = 1;
    a.work = nullptr;
    const int T = spread ? M : a.plan.T;
    // four points per thread: M-point twiddles x2, exchange buffer, 2 x C x T receive; one point per
    // thread: spread_smem_per_point(C) values per point.  Each CTA alone on its SM, e.g. beside the
    // CTAs of a ragged launch
    size_t smem = 0;
    cudaFuncAttributes fa;
    const long long perPoint = k->kind == kKindSpreadFused ? spread_smem_per_point_k(C, (int)nSignal)
                               : (spread ? spread_smem_per_point(C) : 5LL);
    const size_t need = (size_t)perPoint * M * sizeof(double2);
    ck(exclusive_smem(k->fn, need, &smem, &fa), "smem attribute");
    if (smem == 0) throw Unsupported("grid too large for the cluster kernel");
    const long long clusters = std::min<long long>(nInst, smCount() / C);
    lastSchedule = Schedule{(int)(C * clusters), T, 1, smem, 1, 1};
    lastR = a.R;
    lastTuned = 0;
    lastRegs = fa.numRegs;
    auto record = [&] {
      void* args[] = {(void*)&a};
      ck(launch_clustered(k->fn, (int)(C * clusters), T, smem, stream, C, args), "propagate (cluster)");
    };
    if (timeKernels) {
      if (!ev0) ck(cudaEventCreate(&ev0), "event");
      if (!ev1) ck(cudaEventCreate(&ev1), "event");
      ck(cudaEventRecord(ev0, stream), "event");
    }
    if (useGraph) {
      GraphKey key;
      add_prop_key(key, a);
      key.add(k->fn).add(clusters).add(smem);
      graphs.run(key, stream, record);
    } else {
      record();
    }
    launches++;
    if (timeKernels) {
      ck(cudaEventRecord(ev1, stream), "event");
      ck(cudaEventSynchronize(ev1), "event");
      float ms = 0;
      ck(cudaEventElapsedTime(&ms, ev0, ev1), "event");
      kernelMs += ms;
      kernelCount++;
    }
  }

  // Double-float path: the FP64 tables and propagator are split into float-float copies once
  // (and again after every rebuild of the propagator).
  bool wantFF(int R, const PropArgs& a) const {
    return precision == 1 && nSignal == 1 && R == 8 && !a.gridF && !a.gridT && !a.ckpt;
  }

  // radix of the plan's one non-radix-8 pass (1 when all passes are radix 8)
  static int shortRadix(const FFTPlanH& p) {
    for (int i = 0; i < p.nPass; i++)
      if (p.radix[i] != 8) return p.radix[i];
    return 1;
  }

  FFTables prepareFF() {
    std::vector<SplitSeg> segs;
    if (!ffTables) {
      for (auto* b : {&twF, &dstepF, &dlastF, &halfF, &backF}) b->alloc(N);
      segs.push_back({tw, twF.p, (long long)N});
      segs.push_back({dstep.p, dstepF.p, (long long)N});
      segs.push_back({dlast.p, dlastF.p, (long long)N});
      segs.push_back({half.p, halfF.p, (long long)N});
      segs.push_back({back.p, backF.p, (long long)N});
      ffTables = true;
    }
    if (propFFBuild != propBuilds) {
      const size_t count = (size_t)(nZ > 1 ? nZ - 1 : 0) * 2 * N;
      propF.alloc(count);
      if (count) segs.push_back({d2(prop.p), propF.p, (long long)count});
      propFFBuild = propBuilds;
    }
    if (!segs.empty()) {
      ck(launch_split_ff(segs.data(), (int)segs.size(), stream), "float-float tables");
      launches++;
    }
    return FFTables{twF.p, dstepF.p, dlastF.p, halfF.p, backF.p, propF.p};
  }

  double propagatorBytes() const { return (double)(nZ > 1 ? nZ - 1 : 0) * 4.0 * nSignal * nSignal * N * 8.0; }

  // Ragged batches run each medium once per call, and fill the GPU: a medium's RK4 matrices (2M stage
  // evaluations per point and step, built beside the propagations) pay off only when they are used
  // again.  Use them while fresh, build them when the medium runs again with the same pump, and
  // propagate with the DiffEq otherwise.
  bool raggedPropagator() {
    if (!linearSolver() || usePropagator == 0 || nZ <= 1 || propagatorBytes() > 16e9) return false;
    if (usePropagator == 1 || (propVersion == pumpVersion && prop.p)) return true;
    const bool again = raggedPumpVersion == pumpVersion;
    raggedPumpVersion = pumpVersion;
    return again;
  }
  long long raggedPumpVersion = -1;

  // The RK4 propagator matrices replace the four stage evaluations of every step and point by one
  // (2M x 2M) matrix product.  Their build evaluates the 2M unit vectors' RK4 steps for all steps and
  // points in one parallel launch: 2M propagations' worth of point-wise work, which a batch of 4M or
  // more propagations amortises, and which costs little wall time beside a latency-bound launch of
  // fewer propagations than SMs (the build runs on the idle SMs).
  bool wantPropagator(long long nInst) const {
    if (!linearSolver()) return false;
    if (usePropagator == 0) return false;
    if (propagatorBytes() > 16e9) return false;
    if (usePropagator == 1) return true;
    return nInst >= 4LL * nSignal || nInst < smCount();
  }

  // Launch one propagation kernel over `nInst` instances (inputs/outputs prepared in `a`).
  // `tail` (optional): launches that follow the propagation in the same graph (e.g. the Green's
  // function epilogue); `tailKey` holds the host values they read.
  void propagate(PropArgs a, long long nInst, bool allowPropagator, bool plainOne = false,
                 const std::function<void()>& tail = {}, const GraphKey* tailKey = nullptr) {
    const int R = chooseR();
    a.nInst = nInst;
    const KernelEntry* k = nullptr;
    bool gnlse = solver == kChi3GNLSE, ff = false;
    FFTables ffT{};
    // A few propagations on a large grid: each one spread over a cluster of kClusterSize CTAs (also on
    // grids that the one-CTA kernels do not take, e.g. Chi3GNLSE at N=8192)
    if (const KernelEntry* kc = clusterKernel(a, nInst, plainOne)) {
      if (allowPropagator && wantPropagator(nInst)) {
        buildPropagator(R);
        a.prop = prop.p;
      }
      launchCluster(kc, a, nInst);
      if (tail) tail();
      return;
    }
    if (a.stages) throw std::logic_error("stage values are stored by the cluster kernels only");
    // grids the register plan does not take: the general-plan kernels (any N up to kMaxFFT)
    const bool gen = !registerGrid(R);
    bool paired = false;
    if (gen) {
      if (a.ckpt) throw Unsupported("the adjoint's forward takes power-of-two grids (register plan) only");
      int Rg = R;
      if (!gnlse && allowPropagator && wantPropagator(nInst)) {
        k = genKernel(kKindLinear, (int)nSignal, R, &Rg);
        if (k) {
          buildPropagator(R);
          a.prop = prop.p;
        }
      }
      if (!k) k = genKernel(gnlse ? kKindGnlse : kKindDirect, solver, R, &Rg);
      if (!k)
        throw Unsupported("no fused kernel for a grid of " + std::to_string(N) + " points for this solver (" +
                          std::to_string(nSignal) + " modes)");
      a.plan = make_plan_gen((int)N, Rg);
      a.R = Rg;
    } else if (gnlse) {
      checkGridStrict(R);
      k = findKernel(kKindGnlse, solver, R);
      // more rows than SMs (one row per thread group would take a second wave): two rows per thread
      // group, sharing their Raman transforms (k_propagate_gnlse_pair: 14 transforms per row and step
      // instead of 18, so a pair takes 1.56 rows' time)
      if (!plainOne && nInst > smCount() && !a.gridF && !a.gridT) {
        if (const KernelEntry* kp = findKernel(kKindGnlse, solver + 400, R)) {
          k = kp;
          paired = true;
        }
      }
    } else if (allowPropagator && wantPropagator(nInst)) {
      checkGridStrict(R);
      buildPropagator(R);
      a.prop = prop.p;
      if (wantFF(R, a)) {
        ff = true;
        ffT = prepareFF();
        k = findKernel(kKindLinearFF, 1 + 10 * shortRadix(a.plan), R);
      } else {
        // the adjoint's checkpointed forwards: the checkpoint-writing instantiations (key + 100)
        const int lkey = (int)nSignal + (a.ckpt ? 100 : 0);
        k = findKernel(kKindLinear, lkey, R);
        // latency-bound launches: four points per thread, as for the direct kernels below
        if (nInst < smCount() && (int)N / R < 128 && (int)N / 4 <= 512) {
          if (const KernelEntry* k4 = findKernel(kKindLinear, lkey, 4)) {
            k = k4;
            a.plan = make_plan((int)N, 4);
            a.R = 4;
          }
        }
      }
    } else {
      checkGridStrict(R);
      k = findKernel(kKindDirect, solver, R);
      // Launches with fewer propagations than SMs are latency-bound: one SM's FP64 units run each
      // propagation, and N/R threads below 128 leave some of its four schedulers idle.  Use the
      // four-points-per-thread variant when there is one.
      if (nInst < smCount() && (int)N / R < 128 && (int)N / 4 <= 512) {
        if (const KernelEntry* k4 = findKernel(kKindDirect, solver, 4)) {
          k = k4;
          a.plan = make_plan((int)N, 4);
          a.R = 4;
        }
      }
    }
    if (!k) throw Unsupported("no fused kernel for this solver and grid");
    Schedule s{};
    lastTuned = 0;
    if (!plainOne && !gnlse && !gen && tuneWanted(a, nInst)) {
      const TuneChoice c = autotune(k->kind, k->key, a, nInst, ff ? &ffT : nullptr);
      if (c.R != 0) {
        k = findKernelFn(c.fn);
        a.plan = make_plan((int)N, c.R);
        a.R = c.R;
        s = schedule(k, nInst, c.R, c.cta, c.ipcMul);
        lastTuned = 1;
      }
    }
    long long units = paired ? (nInst + 1) / 2 : nInst;   // thread groups' work items
    if (!lastTuned) s = schedule(k, units, a.R, ctaPerSM < 0 ? 0 : ctaPerSM);
    // Paired rows run in waves of one pair per resident thread group.  When the last wave would leave
    // groups idle, the pairs fill whole waves and the rows left over run one per thread group in one
    // more wave of the single-row kernel (a pair takes about 1.56 rows' time): 1024 rows of 4096
    // points on 152 SMs take 3 pair waves and one single wave (5.7 row times) instead of 4 pair waves
    // (6.2).
    const KernelEntry* kTail = nullptr;
    Schedule sTail{};
    PropArgs aTail{};
    if (paired && !lastTuned && !plainOne) {
      const long long wave = (long long)smCount() * s.ctas * s.ipc;
      const long long fullPairs = units / wave * wave;
      const long long rest = nInst - 2 * fullPairs;
      if (fullPairs > 0 && rest > 0 && units % wave != 0) {
        if (const KernelEntry* k1 = findKernel(kKindGnlse, solver, a.R)) {
          const Schedule s1 = schedule(k1, rest, a.R, ctaPerSM < 0 ? 0 : ctaPerSM);
          if ((long long)s1.grid * s1.ipc >= rest) {   // the rest in one wave
            kTail = k1;
            sTail = s1;
            aTail = a;
            aTail.instBase = a.instBase + 2 * fullPairs;
            aTail.nInst = rest;
            aTail.ipc = s1.ipc;
            aTail.work = nullptr;
            a.nInst = 2 * fullPairs;
            units = fullPairs;
            s = schedule(k, units, a.R, ctaPerSM < 0 ? 0 : ctaPerSM);
          }
        }
      }
    }
    if (plainOne) s.grid = 1;
    lastSchedule = s;
    lastR = a.R;
    {
      cudaFuncAttributes fa;
      lastRegs = cudaFuncGetAttributes(&fa, k->fn) == cudaSuccess ? fa.numRegs : 0;
    }
    a.ipc = s.ipc;
    a.work = nullptr;
    const bool counter = !plainOne && (long long)s.grid < (units + s.ipc - 1) / s.ipc;
    if (counter) {
      workCounter.reserve(1);
      a.work = workCounter.p;
    }
    double2* sp = nullptr;
    if (gnlse) {
      // per thread group: 3 (9 when paired) parts of T R values (N on the register plan)
      const size_t slots = std::max((size_t)s.grid * s.ipc * (paired ? 9 : 3), (size_t)sTail.grid * sTail.ipc * 3);
      scratch.reserve(slots * ((size_t)a.plan.T * a.R));
      sp = scratch.p;
    }
    // with kernel timing on, the tail runs after the timed region, outside the graph
    const bool tailInside = tail && !timeKernels;
    auto record = [&] {
      if (counter) ck(cudaMemsetAsync(workCounter.p, 0, sizeof(unsigned long long), stream), "work counter");
      if (gnlse) {
        void* args[] = {(void*)&a, (void*)&sp};
        ck(cudaLaunchKernel(k->fn, dim3(s.grid), dim3(s.block), args, s.smem, stream), "propagate");
        if (kTail) {
          void* targs[] = {(void*)&aTail, (void*)&sp};
          ck(cudaLaunchKernel(kTail->fn, dim3(sTail.grid), dim3(sTail.block), targs, sTail.smem, stream),
             "propagate (single rows)");
        }
      } else if (ff) {
        void* args[] = {(void*)&a, (void*)&ffT};
        ck(cudaLaunchKernel(k->fn, dim3(s.grid), dim3(s.block), args, s.smem, stream), "propagate");
      } else {
        void* args[] = {(void*)&a};
        ck(cudaLaunchKernel(k->fn, dim3(s.grid), dim3(s.block), args, s.smem, stream), "propagate");
      }
      if (tailInside) tail();
    };
    if (timeKernels) {
      if (!ev0) ck(cudaEventCreate(&ev0), "event");
      if (!ev1) ck(cudaEventCreate(&ev1), "event");
      ck(cudaEventRecord(ev0, stream), "event");
    }
    if (useGraph && !plainOne) {
      GraphKey key;
      add_prop_key(key, a);
      key.add(s.grid).add(s.block).add(s.smem).add(k->fn).add(sp).add(ff);
      key.add(kTail ? kTail->fn : nullptr).add(sTail.grid).add(sTail.block).add(sTail.smem);
      if (kTail) add_prop_key(key, aTail);
      key.add(ffT.tw).add(ffT.dstep).add(ffT.dlast).add(ffT.half).add(ffT.back).add(ffT.prop);
      key.add(tailInside);
      if (tailInside && tailKey) key.bytes.insert(key.bytes.end(), tailKey->bytes.begin(), tailKey->bytes.end());
      graphs.run(key, stream, record);
    } else {
      record();
    }
    launches += kTail ? 2 : 1;
    if (timeKernels) {
      ck(cudaEventRecord(ev1, stream), "event");
      ck(cudaEventSynchronize(ev1), "event");
      float ms = 0;
      ck(cudaEventElapsedTime(&ms, ev0, ev1), "event");
      kernelMs += ms;
      kernelCount++;
    }
    if (tail && !tailInside) tail();
  }

  // ---- adjoint (no counterpart in the reference) -------------------------------------------------
  // Continuous poling d(z) on the nZSteps grid in place of the domain pattern (the reference's
  // protected _poling array).
  void setPolingProfile(const double* d, size_t n) {
    if (isCascade || fnl || !poled) throw std::invalid_argument("medium has no poling");
    if (n != nZ) throw std::invalid_argument("poling profile must have nZSteps values");
    poling.assign(d, d + n);
    if (devReady) {
      buildCoefficients();
      ck(cudaStreamSynchronize(stream), "coefficients");
    }
    propVersion = -1;
  }

  void adjointForward(const double2* in, size_t rows, double2* out, int interval) {
    if (solver != kChi2PDC && solver != kChi3GNLSE)
      throw Unsupported("the adjoint is implemented for Chi2PDC and Chi3GNLSE");
    if (rows == 0) throw std::invalid_argument("Too many threads requested!");
    if (nZ < 2) throw std::invalid_argument("the adjoint needs at least two z steps");
    if (!is_pow2((int)N)) throw Unsupported("the adjoint takes power-of-two grids");
    ensureDevice();
    const int R = chooseR();
    checkGrid(R);
    const size_t steps = nZ - 1;
    adjStored = false;
    if (interval <= 0 && storeStages(rows)) {
      // Chi3GNLSE with few rows on a cluster grid: the forward on 4-CTA clusters stores the stage values
      // of every step, and the reverse sweep reads them (nothing recomputed)
      adjStages.reserve((size_t)rows * steps * 8 * N);
      PropArgs a = baseArgs(R);
      a.inKind = 1;
      a.inTime = 0;
      a.in = in;
      a.inStride = (long long)N;
      a.inChannels = 1;
      a.inputMode = 0;
      a.nOut = 1;
      a.outModes[0] = 0;
      a.out = out;
      a.outStride = (long long)N;
      a.stages = adjStages.p;
      propagate(a, (long long)rows, false);
      ck(cudaStreamSynchronize(stream), "adjoint forward");
      adjStored = true;
      adjRows = (long long)rows;
      adjK = 0;
      adjNCk = 0;
      adjPumpVersion = pumpVersion;
      return;
    }
    int K = interval;
    if (K <= 0) {
      // every state while the states fit in 40 % of the free device memory (at most 96 GB: 1024 rows of
      // 4096 points over 999 steps take 67 GB), else every ceil(sqrt(steps)) steps
      const double bytes = (double)rows * steps * N * sizeof(double2);
      size_t freeB = 0, totalB = 0;
      if (cudaMemGetInfo(&freeB, &totalB) != cudaSuccess) {
        cudaGetLastError();
        freeB = 0;
      }
      K = bytes <= std::max(1e9, std::min(0.4 * (double)freeB, 96e9)) ? 1 : (int)std::ceil(std::sqrt((double)steps));
    }
    const int nCk = (int)((steps + K - 1) / K);
    ckpt.reserve((size_t)rows * nCk * N);
    PropArgs a = baseArgs(R);
    a.inKind = 1;
    a.inTime = 0;
    a.in = in;
    a.inStride = (long long)N;
    a.inChannels = 1;
    a.inputMode = 0;
    a.nOut = 1;
    a.outModes[0] = 0;
    a.out = out;
    a.outStride = (long long)N;
    a.ckpt = ckpt.p;
    a.ckK = K;
    a.ckN = nCk;
    propagate(a, (long long)rows, true);
    ck(cudaStreamSynchronize(stream), "adjoint forward");
    adjRows = (long long)rows;
    adjK = K;
    adjNCk = nCk;
    adjPumpVersion = pumpVersion;
  }

  // Stage values of every Chi3GNLSE step fit (at most a quarter of the free device memory and 64 GB),
  // and the forward of `rows` propagations runs on 4-CTA clusters (Medium::clusterKernel).
  bool storeStages(size_t rows) const {
    if (solver != kChi3GNLSE || !useCluster || !is_pow2((int)N) || N < 1024 || N > (uint)kMaxFFT) return false;
    if ((long long)rows * kClusterSize > smCount()) return false;
    if (!findKernel(kKindCluster, solver, kClusterSize) || !findKernel(kKindAdjoint, solver + 300, kClusterSize))
      return false;
    size_t freeB = 0, totalB = 0;
    if (cudaMemGetInfo(&freeB, &totalB) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    const double bytes = (double)rows * (nZ - 1) * 8.0 * N * sizeof(double2);
    return bytes <= std::min(0.25 * (double)freeB, 64e9);
  }

  // Reverse sweep over the stored stage values: one propagation per 4-CTA cluster.
  void adjointStored(const double2* gout, double2* gin) {
    // the form of the forward that stored the stages: one point per thread on Cs CTAs, or four points
    // per thread on four
    const int Cs = gnlseSpreadC(adjRows);
    if (Cs) {
      const KernelEntry* k = findKernel(kKindAdjoint, solver + 500, Cs);
      if (!k) throw Unsupported("no stored-stage adjoint kernel");
      const int M = (int)N / Cs;
      size_t smem = 0;
      cudaFuncAttributes fa;
      ck(exclusive_smem(k->fn, (size_t)spread_smem_per_point(Cs) * M * sizeof(double2), &smem, &fa), "smem attribute");
      if (smem == 0) throw Unsupported("grid too large for the cluster adjoint");
      if (Cs > 8) ck(cudaFuncSetAttribute(k->fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1), "cluster size");
      PropArgs a = baseArgs(kClusterSize);
      a.plan = make_plan(M, 1);
      a.R = 1;
      a.nInst = adjRows;
      a.ipc = 1;
      a.work = nullptr;
      a.stages = adjStages.p;
      AdjArgs d{};
      d.gout = gout;
      d.gin = gin;
      const long long clusters = std::min<long long>(adjRows, smCount() / Cs);
      void* args[] = {(void*)&a, (void*)&d};
      lastSchedule = Schedule{(int)(Cs * clusters), M, 1, smem, 1, 1};
      lastR = 1;
      lastTuned = 0;
      lastRegs = fa.numRegs;
      ck(launch_clustered(k->fn, (int)(Cs * clusters), M, smem, stream, Cs, args), "adjoint (stored stages)");
      launches++;
      ck(cudaStreamSynchronize(stream), "adjoint");
      return;
    }
    constexpr int C = kClusterSize;
    const KernelEntry* k = findKernel(kKindAdjoint, solver + 300, C);
    if (!k) throw Unsupported("no stored-stage adjoint kernel");
    const int M = (int)N / C;
    size_t smem = 0;
    cudaFuncAttributes fa;
    ck(exclusive_smem(k->fn, (size_t)5 * M * sizeof(double2), &smem, &fa), "smem attribute");
    if (smem == 0) throw Unsupported("grid too large for the cluster adjoint");
    PropArgs a = baseArgs(C);
    a.plan = make_plan(M, C);
    a.R = C;
    a.nInst = adjRows;
    a.ipc = 1;
    a.work = nullptr;
    a.stages = adjStages.p;
    AdjArgs d{};
    d.gout = gout;
    d.gin = gin;
    const long long clusters = std::min<long long>(adjRows, smCount() / C);
    void* args[] = {(void*)&a, (void*)&d};
    lastSchedule = Schedule{(int)(C * clusters), a.plan.T, 1, smem, 1, 1};
    lastR = C;
    lastTuned = 0;
    lastRegs = fa.numRegs;
    ck(launch_clustered(k->fn, (int)(C * clusters), a.plan.T, smem, stream, C, args), "adjoint (stored stages)");
    launches++;
    ck(cudaStreamSynchronize(stream), "adjoint");
  }

  // Chi3GNLSE on grids of 1024 to 8192 points with few rows: the pipelined sweep on clusters of eight
  // CTAs (adjoint_gnlse_cluster.cu), one cluster per row; false when it does not apply (more rows than
  // such clusters fit on the device at once, or a grid outside its range).
  bool adjointCluster(const double2* gout, double2* gin) {
    constexpr int C = kClusterSize;
    if (solver != kChi3GNLSE || !useCluster || !is_pow2((int)N) || N < 1024 || N > (uint)kMaxFFT) return false;
    const KernelEntry* k = findKernel(kKindAdjoint, solver + 200, C);
    if (!k) return false;
    const int M = (int)N / C;
    size_t smem = 0;
    cudaFuncAttributes fa;
    ck(exclusive_smem(k->fn, (size_t)5 * M * sizeof(double2), &smem, &fa), "smem attribute");
    if (smem == 0) return false;
    PropArgs a = baseArgs(C);
    a.plan = make_plan(M, C);
    a.R = C;
    a.nInst = adjRows;
    a.ipc = 1;
    a.work = nullptr;
    const int fit = maxActiveClusters(k->fn, 2 * C, a.plan.T, smem);
    // up to three waves of clusters (the two-CTA pipelined sweep is about 3.5 times slower per row)
    if (fit < 1 || adjRows > 3LL * fit) return false;
    const long long waves = (adjRows + fit - 1) / fit;
    const long long clusters = (adjRows + waves - 1) / waves;
    adjSeg.reserve((size_t)clusters * 2 * (size_t)adjK * 8 * N);   // per cluster: STG[2][K][8][N]
    AdjArgs d{};
    d.gout = gout;
    d.ckpt = ckpt.p;
    d.K = adjK;
    d.nCk = adjNCk;
    d.seg = adjSeg.p;
    d.ga = adjGa.p;
    d.gin = gin;
    d.single = adjRows == 1 ? 1 : 0;
    void* args[] = {(void*)&a, (void*)&d};
    lastSchedule = Schedule{(int)(2 * C * clusters), a.plan.T, 1, smem, 1, 1};
    lastR = C;
    lastTuned = 0;
    lastRegs = fa.numRegs;
    ck(launch_clustered(k->fn, (int)(2 * C * clusters), a.plan.T, smem, stream, 2 * C, args),
       "adjoint (cluster of eight)");
    launches++;
    ck(cudaStreamSynchronize(stream), "adjoint");
    return true;
  }

  // The marching form of the Chi2PDC reverse sweep (AdjArgs::gp): every state stored (interval 1) and
  // the RK4 propagator matrices available, the stored gradients (rows x (nZSteps-1) x N) within 8 GB.
  // The sequential sweep then applies P^T per point (4 FMAs) and the stage-factor gradients follow in
  // one parallel launch over all steps and points.
  bool marchForm() const {
    return solver == kChi2PDC && adjK == 1 && linearSolver() && usePropagator != 0 && propagatorBytes() <= 16e9 &&
           (double)adjRows * (nZ - 1) * N * sizeof(double2) <= 8e9;
  }

  // Chi2PDC with few rows on a cluster grid (the forward ran on 4-CTA clusters): the reverse sweep
  // over 4-CTA clusters too, with one point per thread on the spread grids (adjoint_spread.cu) and four
  // above (adjoint_cluster.cu); false when it does not apply.
  bool adjointClusterPdc(const double2* gout, double2* gin) {
    constexpr int C = kClusterSize;
    if (solver != kChi2PDC || !useCluster || !is_pow2((int)N) || N > (uint)kMaxFFT) return false;
    const bool spread = spreadGrid();
    if (!spread && N < 1024) return false;
    if (adjRows * C > smCount()) return false;
    const int Rk = spread ? 1 : C;   // points per thread
    const KernelEntry* k = findKernel(kKindAdjoint, solver + 300, Rk);
    if (!k) return false;
    const int M = (int)N / C;
    const size_t need = (size_t)(spread ? kSpreadSmemPerPoint : 5LL) * M * sizeof(double2);
    size_t smem = 0;
    cudaFuncAttributes fa;
    ck(exclusive_smem(k->fn, need, &smem, &fa), "smem attribute");
    if (smem == 0) return false;
    PropArgs a = baseArgs(C);
    a.plan = make_plan(M, Rk);
    a.R = Rk;
    const int T = spread ? M : a.plan.T;   // threads per CTA
    a.nInst = adjRows;
    a.ipc = 1;
    a.work = nullptr;
    // segments are recomputed with the RK4 propagator matrices when they fit; with every state stored,
    // the matrices give the marching form
    const bool march = marchForm();
    if ((adjK > 1 || march) && linearSolver() && usePropagator != 0 && propagatorBytes() <= 16e9) {
      buildPropagator(C);
      a.prop = prop.p;
    }
    // K > 1: the pipelined form on clusters of eight CTAs (segment recomputation beside the reverse
    // steps), in at most three waves of clusters
    int group = C;
    long long clusters = adjRows;
    // with the propagator matrices: the stage-factor gradients in a group of their own beside the
    // recomputation and the reverse steps, on twelve CTAs (a non-portable cluster size).  Measured on
    // the N=512, nZSteps=2000 problem with 45-step segments, two such groups on sixteen CTAs are no
    // faster (grad/fwd 2.10 both, 2.56 on eight).  NLM_ADJOINT_CTAS = 16 / 8 selects those forms.
    // At 2048 points the same kernels hold one point per thread with 512 threads per CTA (the forward's
    // checkpoints are time-domain rows, whatever form wrote them).
    bool staged = false;
    const char* ctasEnv = std::getenv("NLM_ADJOINT_CTAS");
    const int ctasWant = ctasEnv ? std::atoi(ctasEnv) : 12;
    const bool pointGrid = spread || (useCluster == 1 && N == 2 * kSpreadMaxN);
    int T1 = T, R1 = Rk;
    for (int G = 1; G <= 2 && adjK > 1 && pointGrid && a.prop && !staged; G++) {
      const int size = (2 + G) * C;
      if (size != ctasWant) continue;
      const KernelEntry* k3 = findKernel(kKindAdjoint, solver + 400 + 100 * G, 1);
      if (!k3) continue;
      size_t smem3 = 0;
      cudaFuncAttributes fa3;
      ck(exclusive_smem(k3->fn, (size_t)kSpreadSmemPerPoint * M * sizeof(double2), &smem3, &fa3), "smem attribute");
      int fit = 0;
      if (smem3 && cudaFuncSetAttribute(k3->fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess)
        fit = maxActiveClusters(k3->fn, size, M, smem3);
      else
        cudaGetLastError();
      if (fit >= 1 && adjRows <= 3LL * fit) {
        const long long waves = (adjRows + fit - 1) / fit;
        clusters = (adjRows + waves - 1) / waves;
        group = size;
        k = k3;
        smem = smem3;
        fa = fa3;
        staged = true;
        T1 = M;
        R1 = 1;
        a.plan = make_plan(M, 1);
        a.R = 1;
      }
    }
    if (adjK > 1 && !staged) {
      if (const KernelEntry* kp = findKernel(kKindAdjoint, solver + 200, Rk)) {
        size_t smemP = 0;
        cudaFuncAttributes faP;
        ck(exclusive_smem(kp->fn, need, &smemP, &faP), "smem attribute");
        const int fit = smemP ? maxActiveClusters(kp->fn, 2 * C, T, smemP) : 0;
        if (fit >= 1 && adjRows <= 3LL * fit) {
          const long long waves = (adjRows + fit - 1) / fit;
          clusters = (adjRows + waves - 1) / waves;
          group = 2 * C;
          k = kp;
          smem = smemP;
          fa = faP;
        }
      }
    }
    // [cluster][1 or 2][K][N]; with stage groups: [cluster][3 + 2][K][N]
    if (adjK > 1) adjSeg.reserve((size_t)clusters * (staged ? 5 : group / C) * adjK * N);
    AdjArgs d{};
    d.gout = gout;
    d.ckpt = ckpt.p;
    d.K = adjK;
    d.nCk = adjNCk;
    d.seg = adjK > 1 ? adjSeg.p : nullptr;
    d.ga = adjGa.p;
    d.gin = gin;
    d.single = adjRows == 1 ? 1 : 0;
    if (march) {
      adjGPS.reserve((size_t)adjRows * (nZ - 1) * N);
      d.gp = adjGPS.p;
    }
    void* args[] = {(void*)&a, (void*)&d};
    lastSchedule = Schedule{(int)(group * clusters), T1, 1, smem, 1, 1};
    lastR = R1;
    lastTuned = 0;
    lastRegs = fa.numRegs;
    ck(launch_clustered(k->fn, (int)(group * clusters), T1, smem, stream, group, args), "adjoint (cluster)");
    launches++;
    if (march) {
      ck(launch_adj_stage_grads(a, d, (int)N, adjRows, stream), "stage gradients");
      launches++;
    }
    return true;
  }

  // Clusters of clusterSize CTAs of `fn` that fit on the device at once (0 when the query fails).
  int maxActiveClusters(const void* fn, int clusterSize, int block, size_t smem) {
    cudaLaunchAttribute attr;
    cudaLaunchConfig_t cfg = cluster_config(clusterSize, block, smem, stream, clusterSize, &attr);
    int fit = 0;
    if (cudaOccupancyMaxActiveClusters(&fit, fn, &cfg) != cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    return fit;
  }

  // The one-CTA and two-CTA-cluster reverse sweeps (the stage-factor gradients go to adjGa).
  void adjointLaunch(const double2* gout, double2* gin) {
    const bool gn = solver == kChi3GNLSE;
    int R = chooseR();
    const KernelEntry* k = findKernel(kKindAdjoint, solver, R);
    // few rows: four points per thread, as for the forward (Medium::propagate)
    if (adjRows < (long long)smCount() && (int)N / R < 128 && (int)N / 4 <= 512) {
      if (const KernelEntry* k4 = findKernel(kKindAdjoint, solver, 4)) {
        k = k4;
        R = 4;
      }
    }
    if (!k) throw Unsupported("no adjoint kernel for this grid");
    // Few rows with checkpoint segments: the pipelined variant, one two-CTA cluster per propagation
    // (one CTA recomputes the next segment while the other reverses the current one).
    // (Chi3GNLSE: one CTA marches each segment forward storing the stage values of every step, the
    // other reverses the previous segment from them.)
    const KernelEntry* kp = ((gn || adjK > 1) && adjRows <= (long long)smCount() / 2)
                                ? findKernel(kKindAdjoint, solver + 100, R) : nullptr;
    if (kp) k = kp;
    // Chi3GNLSE with more rows than SMs (where the forward pairs rows as well): two rows per thread
    // group, sharing their Raman transforms (k_adjoint_gnlse_pair)
    const KernelEntry* kq =
        (gn && !kp && adjRows > smCount()) ? findKernel(kKindAdjoint, solver + 400, R) : nullptr;
    if (kq) k = kq;
    Schedule s = schedule(k, kq ? (adjRows + 1) / 2 : adjRows, R);
    // as for the paired forward (Medium::propagate): whole waves of pairs, the rows left over in one
    // wave of the single-row reverse sweep
    const KernelEntry* kTail = nullptr;
    Schedule sTail{};
    long long headRows = adjRows;
    if (kq) {
      const long long pairs = (adjRows + 1) / 2, wave = (long long)smCount() * s.ctas * s.ipc;
      const long long fullPairs = pairs / wave * wave, rest = adjRows - 2 * fullPairs;
      if (fullPairs > 0 && rest > 0 && pairs % wave != 0) {
        if (const KernelEntry* k1 = findKernel(kKindAdjoint, solver, R)) {
          const Schedule s1 = schedule(k1, rest, R);
          if ((long long)s1.grid * s1.ipc >= rest) {
            kTail = k1;
            sTail = s1;
            headRows = 2 * fullPairs;
            s = schedule(k, fullPairs, R);
          }
        }
      }
    }
    if (kp) {
      s.ipc = 1;
      s.block = (int)N / R;
      s.smem = (size_t)(1 + (R != 16 ? 1 : 0)) * N * sizeof(double2);
      s.grid = 2 * (int)adjRows;
    }
    if (kp && gn) {
      adjSeg.reserve((size_t)adjRows * (2 * (size_t)adjK * 8 + 4) * N);   // per cluster: STG[2][K][8][N], 4 N
    } else {
      size_t perSlot = gn ? (size_t)(10 + (adjK > 1 ? 1 + 8 * adjK : 0)) * N : (size_t)adjK * N;
      const size_t singleSlot = perSlot;
      if (kq) perSlot = 2 * (size_t)(16 + (adjK > 1 ? 1 + 8 * adjK : 0)) * N;   // two rows of the pair kernel's scratch
      if (gn || adjK > 1)
        adjSeg.reserve(std::max((size_t)s.grid * s.ipc * perSlot, (size_t)sTail.grid * sTail.ipc * singleSlot));
    }
    PropArgs a = baseArgs(R);
    a.nInst = headRows;
    a.ipc = s.ipc;
    a.work = nullptr;
    // segments between checkpoints are recomputed with the RK4 propagator matrices (built in parallel
    // over all steps and points) instead of the four stage evaluations per step; with every state
    // stored, the matrices give the marching form
    const bool march = marchForm();
    if (!gn && (adjK > 1 || march) && linearSolver() && usePropagator != 0 && propagatorBytes() <= 16e9) {
      buildPropagator(R);
      a.prop = prop.p;
    }
    AdjArgs d{};
    if (march) {
      adjGPS.reserve((size_t)adjRows * (nZ - 1) * N);
      d.gp = adjGPS.p;
    }
    d.gout = gout;
    d.ckpt = ckpt.p;
    d.K = adjK;
    d.nCk = adjNCk;
    d.seg = (gn || adjK > 1) ? adjSeg.p : nullptr;
    d.ga = adjGa.p;
    d.gin = gin;
    d.single = adjRows == 1 ? 1 : 0;
    void* args[] = {(void*)&a, (void*)&d};
    if (kp) {
      ck(launch_clustered(k->fn, s.grid, s.block, s.smem, stream, 2, args), "adjoint (cluster)");
    } else {
      ck(cudaLaunchKernel(k->fn, dim3(s.grid), dim3(s.block), args, s.smem, stream), "adjoint");
    }
    launches++;
    if (kTail) {
      PropArgs at = a;
      at.instBase = headRows;
      at.nInst = adjRows - headRows;
      at.ipc = sTail.ipc;
      void* targs[] = {(void*)&at, (void*)&d};
      ck(cudaLaunchKernel(kTail->fn, dim3(sTail.grid), dim3(sTail.block), targs, sTail.smem, stream),
         "adjoint (single rows)");
      launches++;
    }
    if (march) {
      ck(launch_adj_stage_grads(a, d, (int)N, adjRows, stream), "stage gradients");
      launches++;
    }
  }

  void adjointBackward(const double2* gout, double2* gin, double2* gpump, double* gpol) {
    if (adjRows == 0 || adjPumpVersion != pumpVersion)
      throw std::runtime_error("no adjoint forward pass to differentiate: run nlm_adjoint_forward first");
    const bool gn = solver == kChi3GNLSE;
    if (gn && (gpump || gpol)) throw std::invalid_argument("Chi3GNLSE has no pump or poling to differentiate");
    // Chi3GNLSE on cluster grids: over the stored stage values, or pipelined on clusters of eight CTAs
    if (gn && adjStored) {
      adjointStored(gout, gin);
      return;
    }
    if (gn && adjointCluster(gout, gin)) return;
    const size_t steps = nZ - 1;
    adjGa.reserve(steps * 3 * N);
    ck(cudaMemsetAsync(adjGa.p, 0, steps * 3 * N * sizeof(double2), stream), "memset");
    if (gn || !adjointClusterPdc(gout, gin)) adjointLaunch(gout, gin);
    if (gpump) {
      const size_t rowsP = nZP;
      adjGP.reserve(rowsP * N);
      adjFGP.reserve(rowsP * N);
      const double* prof = nullptr;
      if (profile != NLM_CONSTANT) {
        std::vector<double> sv;
        relativeStrength(sv);
        uploadD(profD, sv);
        prof = profD.p;
      }
      ck(launch_adj_pump_rows(adjGa.p, coef.p, prof, (int)nZ, (int)N, adjGP.p, stream), "pump rows");
      ck(launch_fft_rows(adjGP.p, adjFGP.p, (long long)rowsP, fftPlanRows(), tw, false, 1.0, nullptr, stream), "fft");
      ck(launch_adj_pump_reduce(adjFGP.p, dispPumpD.p, dzp, (int)rowsP, (int)N, gpump, stream), "pump reduce");
      launches += 3;
    }
    if (gpol) {
      adjGc.reserve(steps * 3);
      ck(launch_adj_coef_reduce(adjGa.p, pumpTime.p, (int)nZ, (int)N, adjGc.p, stream), "coef reduce");
      launches++;
      std::vector<double2> gc(steps * 3);
      ck(cudaMemcpyAsync(gc.data(), adjGc.p, gc.size() * sizeof(double2), cudaMemcpyDeviceToHost, stream), "gc");
      ck(cudaStreamSynchronize(stream), "adjoint");
      // c_s = pol_s q_s with q_s = nlStep * mismatch(z_s): dL/dpol_s = Re(g_c conj(q_s)),
      // pol_0 = d[i-1], pol_1 = (d[i-1] + d[i]) / 2, pol_2 = d[i]  (solvers/Chi2PDC.cpp:32-34)
      for (uint i = 0; i < nZ; i++) gpol[i] = 0;
      for (uint i = 1; i < nZ; i++) {
        double gs[3];
        for (int sub = 0; sub < 3; sub++) {
          const double zz = sub == 0 ? (double)(i - 1) * dz : (sub == 1 ? (i - .5) * dz : (double)i * dz);
          const cplx q = nlStep[0] * std::exp(1.0 * kI * diffBeta0[0] * zz);
          const double2 g = gc[(size_t)(i - 1) * 3 + sub];
          gs[sub] = (cplx(g.x, g.y) * std::conj(q)).real();
        }
        gpol[i - 1] += gs[0] + 0.5 * gs[1];
        gpol[i] += 0.5 * gs[1] + gs[2];
      }
    }
    ck(cudaStreamSynchronize(stream), "adjoint");
  }

  // ---- public operations ---------------------------------------------------------------------
  void runSignal(const double* in, size_t n, int inTime, uint inputMode) {
    if (isCascade) throw std::runtime_error("cascade");
    if (n % N != 0 || n / N == 0 || n / N > nSignal)
      throw std::invalid_argument("inputProf array size does not match number of frequency/time bins");
    if (inputMode >= nSignal) throw std::invalid_argument("inputModes does not match any mode in the system");
    ensureDevice();
    const int R = chooseR();
    checkGrid(R);
    io.reserve(n);
    ck(cudaMemcpyAsync(io.p, in, n * sizeof(double2), cudaMemcpyHostToDevice, stream), "input upload");
    const bool pipe = deferredPump.pending && pipePumpGrid() && n == N;
    PropArgs a = pipe ? plainArgs(R) : baseArgs(R);
    a.inKind = 1;
    a.inTime = inTime ? 1 : 0;
    a.in = io.p;
    a.inStride = (long long)n;
    a.inChannels = (int)(n / N);
    a.inputMode = (a.inChannels > 1 || nSignal <= 1) ? 0 : (int)inputMode;
    a.gridF = sigFreq.p;
    a.gridT = sigTime.p;
    if (pipe) launchPumpSignal(a);
    else propagate(a, 1, true);
    ck(cudaStreamSynchronize(stream), "signal simulation");
    signalVersion++;
  }

  // The deferred Chi3 pump march and this signal propagation on one cluster of eight CTAs: the pump on
  // four, the signal on the other four one pump step pair behind (the solver's DiffEq at every step, no
  // RK4 matrices), M = N / 4 threads per CTA.
  void launchPumpSignal(PropArgs a) {
    const int M = (int)N / 4;
    a.plan = make_plan(M, 1);
    a.R = 1;
    a.nInst = 1;
    a.ipc = 1;
    a.work = nullptr;
    a.prop = nullptr;
    const PumpMarchArgs p = deferredPumpArgs();
    lastSchedule = Schedule{8, M, 1, (size_t)spread_smem_per_point(4) * M * sizeof(double2), 1, 1};
    lastR = 1;
    lastTuned = 0;
    if (timeKernels) {
      if (!ev0) ck(cudaEventCreate(&ev0), "event");
      if (!ev1) ck(cudaEventCreate(&ev1), "event");
      ck(cudaEventRecord(ev0, stream), "event");
    }
    ck(launch_chi3_pump_signal_spread(a, p, stream, &lastRegs), "chi3 pump + signal (cluster of eight)");
    deferredPump.pending = false;   // only once launched: a failed launch leaves the march deferred
    launches++;
    if (timeKernels) {
      ck(cudaEventRecord(ev1, stream), "event");
      ck(cudaEventSynchronize(ev1), "event");
      float ms = 0;
      ck(cudaEventElapsedTime(&ms, ev0, ev1), "event");
      kernelMs += ms;
      kernelCount++;
    }
  }

  // mode selection of computeGreensFunction, src/_NonlinearMedium.cpp:266-302
  void greenModes(unsigned nThreads, const uint8_t* useIn, size_t nIn, const uint8_t* useOut, size_t nOut,
                  std::vector<int>& inputs, std::vector<int>& outputs) const {
    if (nIn > nSignal) throw std::invalid_argument("List of requested inputs indices longer than number of modes!");
    if (nOut > nSignal) throw std::invalid_argument("List of requested output indices longer than number of modes!");
    auto count = [&](const uint8_t* v, size_t n) {
      uint c = 0;
      for (size_t i = 0; i < n; i++) c += (v[i] < nSignal);
      return c;
    };
    if (nIn > 0 && count(useIn, nIn) == 0) throw std::invalid_argument("Requested no valid inputs!");
    if (nOut > 0 && count(useOut, nOut) == 0) throw std::invalid_argument("Requested no valid outputs!");
    inputs.clear();
    outputs.clear();
    for (uint m = 0; m < nSignal; m++) {
      if (nIn == 0 || (m < nIn && useIn[m])) inputs.push_back((int)m);
      if (nOut == 0 || (m < nOut && useOut[m])) outputs.push_back((int)m);
    }
    // the reference indexes past its selection here (undefined); a 0/1 mask is used instead
    if (inputs.empty()) throw std::invalid_argument("Requested no valid inputs!");
    if (outputs.empty()) throw std::invalid_argument("Requested no valid outputs!");
    if (nThreads > N * inputs.size()) throw std::invalid_argument("Too many threads requested!");
    if (nThreads == 0) throw std::invalid_argument("Too many threads requested!");
  }

  void green(int inTime, int runPumpFlag, unsigned nThreads, int normalize, const uint8_t* useIn, size_t nUseIn,
             const uint8_t* useOut, size_t nUseOut, double2* Cdst, double2* Sdst, bool deviceDst,
             long long maxInstances = -1) {
    if (fnl || isCascade) throw std::runtime_error("Object does not have this method.");
    std::vector<int> inputs, outputs;
    greenModes(nThreads, useIn, nUseIn, useOut, nUseOut, inputs, outputs);
    if (runPumpFlag) runPump();
    ensureDevice();
    const int R = chooseR();
    checkGrid(R);
    const int nIn = (int)inputs.size(), nOut = (int)outputs.size();
    const long long nInst = 2LL * nIn * N;
    const long long outStride = (long long)nOut * N;
    raw.reserve((size_t)nInst * outStride);
    PropArgs a = baseArgs(R);
    a.inKind = 0;
    a.inTime = inTime ? 1 : 0;
    for (int i = 0; i < nIn; i++) a.impModes[i] = inputs[i];
    a.nOut = nOut;
    for (int i = 0; i < nOut; i++) a.outModes[i] = outputs[i];
    a.out = raw.p;
    a.outStride = outStride;
    // epilogue flags per (om, im) block, src/_NonlinearMedium.cpp:360-372
    std::vector<uint8_t> flags((size_t)nOut * nIn, 0);
    std::vector<double2> scales((size_t)nOut * nIn, make_double2(1, 0));
    for (int im = 0; im < std::min(nOut, nIn); im++)
      for (int om = 0; om < nOut; om++) {
        uint8_t f = 1;
        if (normalize && im != om) {
          f |= 2;
          const cplx s = std::sqrt(nlStep[im] / nlStep[om]);
          scales[(size_t)om * nIn + im] = make_double2(s.real(), s.imag());
        }
        flags[(size_t)om * nIn + im] = f;
      }
    flagsD.reserve(flags.size());
    ck(cudaMemcpyAsync(flagsD.p, flags.data(), flags.size(), cudaMemcpyHostToDevice, stream), "flags");
    upload(scaleD, scales);
    const size_t mat = (size_t)nOut * N * nIn * N;
    double2 *C = nullptr, *S = nullptr;
    if (deviceDst) {
      C = Cdst;
      S = Sdst;
    } else {
      cs.reserve(2 * mat);
      C = cs.p;
      S = cs.p + mat;
    }
    // the epilogue reads the flags and scales through device pointers: they are uploaded above, on
    // the same stream and before the graph runs, so a replay reads this call's values
    auto epilogue = [&] {
      ck(launch_green_epilogue(raw.p, outStride, (int)N, nIn, nOut, scaleD.p, flagsD.p, C, S, stream), "epilogue");
    };
    if (maxInstances >= 0) {
      // one propagation per launch (timing helper)
      ck(cudaMemsetAsync(raw.p, 0, (size_t)nInst * outStride * sizeof(double2), stream), "memset");
      const long long todo = std::min(nInst, maxInstances == 0 ? nInst : maxInstances);
      for (long long i = 0; i < todo; i++) {
        PropArgs b = a;
        b.instBase = i;
        propagate(b, 1, false, true);
      }
      epilogue();
    } else {
      GraphKey ek;
      ek.add(raw.p).add(outStride).add(N).add(nIn).add(nOut).add(scaleD.p).add(flagsD.p).add(C).add(S);
      propagate(a, nInst, true, false, epilogue, &ek);
    }
    launches++;
    if (!deviceDst) {
      ck(cudaMemcpyAsync(Cdst, C, mat * sizeof(double2), cudaMemcpyDeviceToHost, stream), "C download");
      ck(cudaMemcpyAsync(Sdst, S, mat * sizeof(double2), cudaMemcpyDeviceToHost, stream), "S download");
    }
    ck(cudaStreamSynchronize(stream), "green");
  }

  // Raw outputs of impulse propagations [first, first + count) of the Green's function over all modes
  // (instance 2 (im N + bin) + {0: impulse 1, 1: impulse i}); the row block of one rank when the
  // 2 N nIn propagations are split over several GPUs.
  // rawOut: host memory, or (device = true) device memory written by the kernel directly.
  void greenRows(int inTime, int runPumpFlag, long long first, long long count, double2* rawOut, bool device = false) {
    if (fnl || isCascade) throw std::runtime_error("Object does not have this method.");
    const long long total = 2LL * nSignal * N;
    if (first < 0 || count < 0 || first + count > total) throw std::invalid_argument("impulse range out of bounds");
    if (runPumpFlag) runPump();
    ensureDevice();
    const int R = chooseR();
    checkGrid(R);
    const long long outStride = (long long)nSignal * N;
    if (!device) raw.reserve((size_t)std::max<long long>(count, 1) * outStride);
    double2* dst = device ? rawOut : raw.p;
    PropArgs a = baseArgs(R);
    a.inKind = 0;
    a.inTime = inTime ? 1 : 0;
    for (uint m = 0; m < nSignal; m++) a.impModes[m] = (int)m;
    a.nOut = (int)nSignal;
    for (uint m = 0; m < nSignal; m++) a.outModes[m] = (int)m;
    a.out = dst - first * outStride;   // the kernel indexes outputs by the global instance
    a.outStride = outStride;
    a.instBase = first;
    if (count > 0) propagate(a, count, true);
    if (count > 0 && !device)
      ck(cudaMemcpyAsync(rawOut, raw.p, (size_t)count * outStride * sizeof(double2), cudaMemcpyDeviceToHost, stream),
         "rows download");
    ck(cudaStreamSynchronize(stream), "green rows");
  }

  // C and S from the raw rows of all 2 N nSignal impulse propagations (the epilogue of green()).
  // rawIn, Cdst, Sdst: host memory, or (device = true) device memory read and written directly.
  void greenFinish(const double2* rawIn, int normalize, double2* Cdst, double2* Sdst, bool device = false) {
    if (fnl || isCascade) throw std::runtime_error("Object does not have this method.");
    ensureDevice();
    const int nIn = (int)nSignal, nOut = (int)nSignal;
    const long long nInst = 2LL * nIn * N, outStride = (long long)nOut * N;
    const double2* src = rawIn;
    if (!device) {
      raw.reserve((size_t)nInst * outStride);
      ck(cudaMemcpyAsync(raw.p, rawIn, (size_t)nInst * outStride * sizeof(double2), cudaMemcpyHostToDevice, stream),
         "rows upload");
      src = raw.p;
    }
    std::vector<uint8_t> flags((size_t)nOut * nIn, 1);
    std::vector<double2> scales((size_t)nOut * nIn, make_double2(1, 0));
    for (int im = 0; im < nIn; im++)
      for (int om = 0; om < nOut; om++)
        if (normalize && im != om) {
          flags[(size_t)om * nIn + im] |= 2;
          const cplx sc = std::sqrt(nlStep[im] / nlStep[om]);
          scales[(size_t)om * nIn + im] = make_double2(sc.real(), sc.imag());
        }
    flagsD.reserve(flags.size());
    ck(cudaMemcpyAsync(flagsD.p, flags.data(), flags.size(), cudaMemcpyHostToDevice, stream), "flags");
    upload(scaleD, scales);
    const size_t mat = (size_t)nOut * N * nIn * N;
    if (!device) cs.reserve(2 * mat);
    double2* Cd = device ? Cdst : cs.p;
    double2* Sd = device ? Sdst : cs.p + mat;
    ck(launch_green_epilogue(src, outStride, (int)N, nIn, nOut, scaleD.p, flagsD.p, Cd, Sd, stream), "epilogue");
    launches++;
    if (!device) {
      ck(cudaMemcpyAsync(Cdst, cs.p, mat * sizeof(double2), cudaMemcpyDeviceToHost, stream), "C download");
      ck(cudaMemcpyAsync(Sdst, cs.p + mat, mat * sizeof(double2), cudaMemcpyDeviceToHost, stream), "S download");
    }
    ck(cudaStreamSynchronize(stream), "green finish");
  }

  void greenDims(unsigned nThreads, const uint8_t* useIn, size_t nUseIn, const uint8_t* useOut, size_t nUseOut,
                 size_t* rows, size_t* cols) const {
    if (fnl || isCascade) throw std::runtime_error("Object does not have this method.");
    std::vector<int> inputs, outputs;
    greenModes(nThreads, useIn, nUseIn, useOut, nUseOut, inputs, outputs);
    *rows = outputs.size() * N;
    *cols = inputs.size() * N;
  }

  // src/_NonlinearMedium.cpp:380-406
  void batchModes(size_t rows, size_t cols, unsigned nThreads, uint inputMode, const uint8_t* useOut, size_t nUseOut,
                  std::vector<int>& outputs) const {
    if (cols % N != 0 || cols / N == 0 || cols / N > nSignal) throw std::invalid_argument("Signals not of correct length!");
    if (nThreads > rows || nThreads == 0) throw std::invalid_argument("Too many threads requested!");
    if (inputMode >= nSignal) throw std::invalid_argument("inputModes does not match any mode in the system");
    outputs.clear();
    if (nUseOut > 0) {
      uint c = 0;
      for (size_t i = 0; i < nUseOut; i++) c += (useOut[i] != 0);
      if (c == 0) throw std::invalid_argument("Requested no outputs!");
    }
    for (uint m = 0; m < nSignal; m++)
      if (nUseOut == 0 || (m < nUseOut && useOut[m])) outputs.push_back((int)m);
    if (outputs.empty()) throw std::invalid_argument("Requested no outputs!");
  }

  void batch(const double2* in, size_t rows, size_t cols, int inTime, int runPumpFlag, unsigned nThreads,
             uint inputMode, const uint8_t* useOut, size_t nUseOut, double2* out, bool device) {
    if (isCascade) throw std::runtime_error("cascade");
    std::vector<int> outputs;
    batchModes(rows, cols, nThreads, inputMode, useOut, nUseOut, outputs);
    if (runPumpFlag && !fnl) runPump();
    ensureDevice();
    const int R = chooseR();
    checkGrid(R);
    const int nOut = (int)outputs.size();
    const double2* din = in;
    double2* dout = out;
    if (!device) {
      io.reserve(rows * cols);
      ck(cudaMemcpyAsync(io.p, in, rows * cols * sizeof(double2), cudaMemcpyHostToDevice, stream), "batch upload");
      din = io.p;
      work2.reserve(rows * nOut * N);
      dout = work2.p;
    }
    PropArgs a = baseArgs(R);
    a.inKind = 1;
    a.inTime = inTime ? 1 : 0;
    a.in = din;
    a.inStride = (long long)cols;
    a.inChannels = (int)(cols / N);
    a.inputMode = (a.inChannels > 1 || nSignal <= 1) ? 0 : (int)inputMode;
    a.nOut = nOut;
    for (int i = 0; i < nOut; i++) a.outModes[i] = outputs[i];
    a.out = dout;
    a.outStride = (long long)nOut * N;
    propagate(a, (long long)rows, true);
    if (!device)
      ck(cudaMemcpyAsync(out, dout, rows * nOut * N * sizeof(double2), cudaMemcpyDeviceToHost, stream), "batch download");
    ck(cudaStreamSynchronize(stream), "batch");
  }

  // ---- getters ------------------------------------------------------------------------------
  const std::vector<double>& mirror(int which, uint idx, size_t* rows) {
    std::vector<std::vector<double>>* store;
    std::vector<long long>* vers;
    DevBuf<double2>* dev;
    uint count, nrows;
    long long ver;
    switch (which) {
      case 0: store = &pumpMirrorF; vers = &pumpMirrorVerF; dev = &pumpFreq; count = nPump; nrows = nZP; ver = pumpVersion; break;
      case 1: store = &pumpMirrorT; vers = &pumpMirrorVerT; dev = &pumpTime; count = nPump; nrows = nZP; ver = pumpVersion; break;
      case 2: store = &sigMirrorF; vers = &sigMirrorVerF; dev = &sigFreq; count = nSignal; nrows = nZ; ver = signalVersion; break;
      case 3: store = &sigMirrorT; vers = &sigMirrorVerT; dev = &sigTime; count = nSignal; nrows = nZ; ver = signalVersion; break;
      default: throw IndexError("vector::_M_range_check");
    }
    if (isCascade || idx >= count) throw IndexError("vector::_M_range_check: index out of range");
    if (which <= 1) flushPump();
    store->resize(count);
    vers->resize(count, -2);
    std::vector<double>& h = (*store)[idx];
    const size_t len = (size_t)nrows * N * 2;
    if (h.size() != len) {
      h.assign(len, 0.0);
      (*vers)[idx] = -2;
    }
    if ((*vers)[idx] != ver) {
      if (devReady && dev->p && len > 0) {
        ck(cudaMemcpyAsync(h.data(), dev->p + (size_t)idx * nrows * N, len * sizeof(double), cudaMemcpyDeviceToHost,
                           stream),
           "grid download");
        ck(cudaStreamSynchronize(stream), "grid download");
      }
      (*vers)[idx] = ver;
    }
    *rows = nrows;
    return h;
  }
};

// Launch description of a Chi3GNLSE batch whose scratch memory the caller provides (engine.cpp).
nlm_status prepare_gnlse_noalloc(nlm_medium* h, const void* in, size_t rows, int inTime, void* out,
                                 size_t scratchElems, PropArgs* args, int* grid, int* block, size_t* smem,
                                 const void** fn, cudaStream_t* stream);

}  // namespace nlm

struct nlm_medium {
  nlm::Medium* impl;
};

inline nlm::Medium* M(nlm_medium* h) {
  if (!h || !h->impl) throw std::invalid_argument("null medium handle");
  return h->impl;
}
inline const nlm::Medium* CM(const nlm_medium* h) {
  if (!h || !h->impl) throw std::invalid_argument("null medium handle");
  return h->impl;
}
