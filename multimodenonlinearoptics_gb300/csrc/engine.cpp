// engine.cpp -- the C ABI of the engine (include/nlm_capi.h) over the Medium class (engine.h):
// handles, errors, construction, pumps, signals, Green's functions, batches, cascades, grids,
// adjoints, engine controls and measurement entry points.  The ragged batch is engine_ragged.cpp.
#include "engine.h"

namespace nlm {

void set_error_message(const std::string& msg) { g_error = msg; }

// ----------------------------------------------------------------------------------------
// construction (src/_NonlinearMedium.cpp:8-40; src/_FullyNonlinearMedium.hpp:32-38)
// ----------------------------------------------------------------------------------------
static Medium* create_medium(int s, const double* args, const double* pump, size_t nPumpVals, const double* pol,
                             size_t nPol) {
  BaseParams b = map_ctor(s, args);
  std::unique_ptr<Medium> m(new Medium());
  m->solver = s;
  m->nSignal = b.nSignal;
  m->nPump = b.nPump;
  m->fnl = b.fnl;
  m->poled = b.poled;
  m->fr = b.fr;
  m->fb = b.fb;
  m->tau1 = b.tau1;
  m->tau2 = b.tau2;
  m->tau3 = b.tau3;
  double rayleigh = b.rayleigh;
  if (b.profile == NLM_CONSTANT) rayleigh = kInf;
  m->setLengths(b.relativeLength, b.nl, b.zPrecision, rayleigh, b.beta2, b.beta2s, b.beta1, b.beta1s, b.beta3, b.beta3s);
  m->resetGrids(b.tPrecision, b.tMax);
  m->setDispersion(b.beta2, b.beta2s, b.beta1, b.beta1s, b.beta3, b.beta3s, b.diffBeta0);
  if (b.poled) {
    std::vector<double> p(pol, pol + nPol);
    m->setPoling(p);
  }
  m->profile = m->rayleigh != kInf ? b.profile : NLM_CONSTANT;
  if (m->nPump > 0) {
    m->envelope.assign(m->nPump, std::vector<cplx>(m->N, 0.0));
    if (nPumpVals != 0)
      m->setPumpCustomImpl(pump, nPumpVals, b.chirp, b.delay, 0);
    else
      m->setPumpTypeImpl(b.pulseType, b.chirp, b.delay, 0);
    for (uint k = 1; k < m->nPump; k++) m->envelope[k].assign(m->N, 0.0);
  }
  if (m->fnl) {
    m->dzp = 0;
    m->nZP = 0;
  }
  return m.release();
}

}  // namespace nlm

// ==========================================================================================
// C ABI
// ==========================================================================================
using nlm::guarded;
using nlm::Medium;

// An output pointer of the C ABI, checked before it is written.
template <class T>
static T* out_ptr(T* p) {
  if (!p) throw std::invalid_argument("null output pointer");
  return p;
}


nlm_status nlm::prepare_gnlse_noalloc(nlm_medium* h, const void* in, size_t rows, int inTime, void* out,
                                      size_t scratchElems, PropArgs* args, int* grid, int* block, size_t* smem,
                                      const void** fn, cudaStream_t* stream) {
  return guarded([&] {
    Medium* m = M(h);
    if (m->solver != kChi3GNLSE)
      throw std::invalid_argument("the allocation-free batch entry point propagates Chi3GNLSE media only");
    if (!m->devReady || (m->relIntD.p == nullptr && m->nZ > 1))
      throw std::runtime_error("medium has no device tables yet: run one GPU call of it (e.g. batchSignalSimulation) "
                               "before the allocation-free entry point");
    if (!in || !out) throw std::invalid_argument("null input or output pointer");
    if (rows == 0) throw std::invalid_argument("Too many threads requested!");
    int dev = -1;
    ck(cudaGetDevice(&dev), "device");
    if (dev != m->devOrdinal)
      throw std::invalid_argument("the medium's tables live on device " + std::to_string(m->devOrdinal) +
                                  " but device " + std::to_string(dev) + " is current");
    const int R = m->chooseR();
    // only the one-CTA kernel takes its scratch from the caller: grids it cannot hold (more than
    // 512 threads of R points, or a grid the fused kernels do not take) are rejected here
    m->checkGridStrict(R);
    // the form whose RK4 sum stays in time: two scratch parts per propagation
    const KernelEntry* k = m->findKernel(kKindGnlse, m->solver + 700, R);
    if (!k) throw Unsupported("no one-CTA Chi3GNLSE kernel for a grid of " + std::to_string(m->N) + " points");
    Medium::Schedule s = m->schedule(k, (long long)rows, R);
    // the array bounds how many CTAs run at once (2 N values per resident propagation); more rows
    // than the resident propagations only means more rounds of the persistent grid
    const size_t perSlot = 2 * (size_t)m->N;
    const size_t slots = scratchElems / perSlot;
    if (slots < (size_t)s.ipc)
      throw std::invalid_argument("grid of " + std::to_string(m->N) + " points needs " +
                                  std::to_string(perSlot * s.ipc * sizeof(double2)) +
                                  " bytes of scratch per CTA; the allocation-free entry point holds " +
                                  std::to_string(scratchElems * sizeof(double2)) + " bytes");
    s.grid = (int)std::min<size_t>((size_t)s.grid, slots / (size_t)s.ipc);
    PropArgs a = m->baseArgs(R);
    a.inKind = 1;
    a.inTime = inTime ? 1 : 0;
    a.in = reinterpret_cast<const double2*>(in);
    a.inStride = (long long)m->N;
    a.inChannels = 1;
    a.inputMode = 0;
    a.nOut = 1;
    a.outModes[0] = 0;
    a.out = reinterpret_cast<double2*>(out);
    a.outStride = (long long)m->N;
    a.nInst = (long long)rows;
    a.ipc = s.ipc;
    a.work = nullptr;   // static round robin: no counter to allocate
    *out_ptr(args) = a;
    *out_ptr(grid) = s.grid;
    *out_ptr(block) = s.block;
    *out_ptr(smem) = s.smem;
    *out_ptr(fn) = k->fn;
    *out_ptr(stream) = m->stream;
  });
}

extern "C" {

const char* nlm_last_error(void) { return nlm::g_error.c_str(); }

const char* nlm_version(void) { return "nonlinearmedium-gb300 0.1"; }

int nlm_solver_count(void) { return nlm::kNumSolvers; }

const char* nlm_solver_name(int index) {
  if (index < 0 || index >= nlm::kNumSolvers) return nullptr;
  return nlm::kSolvers[index].name;
}

const char* nlm_solver_signature(const char* solver) {
  const int s = solver ? nlm::solver_by_name(solver) : -1;
  return s < 0 ? nullptr : nlm::kSolvers[s].signature;
}

nlm_status nlm_create(const char* solver, const double* args, size_t nargs, const double* custom_pump,
                      size_t n_custom_pump, const double* poling, size_t n_poling, nlm_medium** out) {
  return guarded([&] {
    if (!out) throw std::invalid_argument("null output handle");
    const int s = solver ? nlm::solver_by_name(solver) : -1;
    if (s < 0) throw std::invalid_argument(std::string("unknown solver ") + (solver ? solver : "(null)"));
    if ((int)nargs != nlm::scalar_arg_count(s)) throw std::invalid_argument("wrong number of constructor arguments");
    Medium* m = nlm::create_medium(s, args, custom_pump, n_custom_pump, poling, n_poling);
    *out = new nlm_medium{m};
  });
}

nlm_status nlm_destroy(nlm_medium* medium) {
  return guarded([&] {
    if (!medium) return;
    delete medium->impl;
    delete medium;
  });
}

nlm_status nlm_info(const nlm_medium* h, int* nSig, int* nPump, int* nFreqs, int* nZ, int* nZP, int* fnl, int* casc) {
  return guarded([&] {
    const Medium* m = CM(h);
    if (nSig) *nSig = (int)m->nSignal;
    if (nPump) *nPump = (int)m->nPump;
    if (nFreqs) *nFreqs = (int)m->N;
    if (nZ) *nZ = (int)m->nZ;
    if (nZP) *nZP = (int)m->nZP;
    if (fnl) *fnl = m->fnl ? 1 : 0;
    if (casc) *casc = m->isCascade ? 1 : 0;
  });
}

nlm_status nlm_lengths(const nlm_medium* h, double* z, double* dz, double* dzp, double* tMax) {
  return guarded([&] {
    const Medium* m = CM(h);
    if (z) *z = m->z;
    if (dz) *dz = m->dz;
    if (dzp) *dzp = m->dzp;
    if (tMax) *tMax = m->tMax;
  });
}

nlm_status nlm_set_pump_type(nlm_medium* h, int pulse_type, double chirp, double delay, unsigned pump_index) {
  return guarded([&] {
    Medium* m = M(h);
    if (m->isCascade) {  // src/Cascade.cpp:55-72
      if (m->sharedPump) m->media[0]->setPumpType(pulse_type, chirp, delay, pump_index);
      else for (Medium* x : m->media) x->setPumpType(pulse_type, chirp, delay, pump_index);
      return;
    }
    m->setPumpType(pulse_type, chirp, delay, pump_index);
  });
}

nlm_status nlm_set_pump_custom(nlm_medium* h, const double* custom_pump, size_t n, double chirp, double delay,
                               unsigned pump_index) {
  return guarded([&] {
    Medium* m = M(h);
    if (m->isCascade) {
      if (m->sharedPump) m->media[0]->setPumpCustom(custom_pump, n, chirp, delay, pump_index);
      else for (Medium* x : m->media) x->setPumpCustom(custom_pump, n, chirp, delay, pump_index);
      return;
    }
    m->setPumpCustom(custom_pump, n, chirp, delay, pump_index);
  });
}

nlm_status nlm_set_pump_from(nlm_medium* h, const nlm_medium* other, unsigned mode_index, double delay,
                             unsigned pump_index) {
  return guarded([&] {
    Medium* m = M(h);
    if (m->isCascade) throw std::runtime_error("Object does not have this method.");
    m->setPumpFrom(*const_cast<Medium*>(CM(other)), mode_index, delay, pump_index);
  });
}

static void cascade_run_pump(Medium* c) {
  // src/Cascade.cpp:75-88
  if (!c->sharedPump) {
    for (Medium* x : c->media) x->runPump();
  } else {
    c->media[0]->runPump();
    for (size_t i = 1; i < c->media.size(); i++) {
      Medium* prev = c->media[i - 1];
      Medium* cur = c->media[i];
      size_t rows = 0;
      const std::vector<double>& pt = prev->mirror(1, 0, &rows);
      if (cur->envelope.empty()) throw std::runtime_error("Object does not have this method.");
      if (cur->N != prev->N) throw std::invalid_argument("Medium does not have same time and frequency axes as the first");
      const size_t last = (rows - 1) * prev->N * 2;
      for (nlm::uint k = 0; k < cur->N; k++) cur->envelope[0][k] = nlm::cplx(pt[last + 2 * k], pt[last + 2 * k + 1]);
      cur->runPump();
    }
  }
}

nlm_status nlm_run_pump(nlm_medium* h) {
  return guarded([&] {
    Medium* m = M(h);
    m->launches = 0;
    if (m->isCascade) {
      cascade_run_pump(m);
      return;
    }
    m->runPump();
  });
}

nlm_status nlm_run_signal(nlm_medium* h, const double* input_prof, size_t n, int in_time_domain, unsigned input_mode) {
  return guarded([&] {
    Medium* m = M(h);
    m->launches = 0;
    if (m->isCascade) {  // src/Cascade.cpp:91-107
      m->media[0]->runSignal(input_prof, n, in_time_domain, input_mode);
      for (size_t i = 1; i < m->media.size(); i++) {
        const auto& conn = m->connections[i - 1];
        nlm::uint maxIn = 0;
        for (auto& kv : conn) maxIn = std::max(maxIn, kv.first);
        Medium* prev = m->media[i - 1];
        std::vector<double> nxt((size_t)m->N * (maxIn + 1) * 2, 0.0);
        for (auto& kv : conn) {
          size_t rows = 0;
          const std::vector<double>& sf = prev->mirror(2, kv.second, &rows);
          const size_t last = (rows - 1) * prev->N * 2;
          std::copy(sf.begin() + last, sf.begin() + last + 2 * m->N, nxt.begin() + (size_t)kv.first * m->N * 2);
        }
        m->media[i]->runSignal(nxt.data(), nxt.size() / 2, 0, 0);
      }
      return;
    }
    m->runSignal(input_prof, n, in_time_domain, input_mode);
  });
}

nlm_status nlm_green_dims(nlm_medium* h, unsigned n_threads, const uint8_t* use_input, size_t n_use_input,
                          const uint8_t* use_output, size_t n_use_output, size_t* rows, size_t* cols) {
  return guarded([&] {
    Medium* m = M(h);
    if (m->isCascade) {
      // composition of the media's matrices, src/Cascade.cpp:110-135
      size_t r = 0, c = 0;
      const size_t last = m->media.size() - 1;
      m->media[0]->greenDims(n_threads, use_input, n_use_input, last == 0 ? use_output : nullptr,
                             last == 0 ? n_use_output : 0, &r, &c);
      size_t cols0 = c;
      for (size_t i = 1; i < m->media.size(); i++) {
        size_t ri = 0, ci = 0;
        m->media[i]->greenDims(n_threads, nullptr, 0, i == last ? use_output : nullptr, i == last ? n_use_output : 0, &ri, &ci);
        if (ci != r) throw std::invalid_argument("Cascade Green's function dimensions do not chain");
        r = ri;
      }
      *out_ptr(rows) = r;
      *out_ptr(cols) = cols0;
      return;
    }
    m->greenDims(n_threads, use_input, n_use_input, use_output, n_use_output, out_ptr(rows), out_ptr(cols));
  });
}

static void cascade_green(Medium* c, int inTime, int runPump, unsigned nThreads, int normalize, const uint8_t* useIn,
                          size_t nIn, const uint8_t* useOut, size_t nOut, double2* Cdst, double2* Sdst, bool dev) {
  if (runPump) cascade_run_pump(c);
  const size_t last = c->media.size() - 1;
  Medium* m0 = c->media[0];
  size_t r = 0, cc = 0;
  m0->greenDims(nThreads, useIn, nIn, last == 0 ? useOut : nullptr, last == 0 ? nOut : 0, &r, &cc);
  nlm::DevBuf<double2> C, S, Ci, Si, Ct, St;
  C.alloc(r * cc);
  S.alloc(r * cc);
  m0->green(inTime, 0, nThreads, normalize, useIn, nIn, last == 0 ? useOut : nullptr, last == 0 ? nOut : 0, C.p, S.p, true);
  for (size_t i = 1; i < c->media.size(); i++) {
    Medium* mi = c->media[i];
    size_t ri = 0, ci = 0;
    mi->greenDims(nThreads, nullptr, 0, i == last ? useOut : nullptr, i == last ? nOut : 0, &ri, &ci);
    if (ci != r) throw std::invalid_argument("Cascade Green's function dimensions do not chain");
    Ci.alloc(ri * ci);
    Si.alloc(ri * ci);
    mi->green(inTime, 0, nThreads, normalize, nullptr, 0, i == last ? useOut : nullptr, i == last ? nOut : 0, Ci.p, Si.p, true);
    Ct.alloc(ri * cc);
    St.alloc(ri * cc);
    nlm::ck(nlm::launch_cgemm_compose(Ci.p, Si.p, C.p, S.p, (int)ri, (int)ci, (int)cc, Ct.p, St.p, mi->stream), "compose");
    nlm::ck(cudaStreamSynchronize(mi->stream), "compose");
    std::swap(C.p, Ct.p);
    std::swap(C.n, Ct.n);
    std::swap(S.p, St.p);
    std::swap(S.n, St.n);
    r = ri;
  }
  const size_t bytes = r * cc * sizeof(double2);
  nlm::ck(cudaMemcpy(Cdst, C.p, bytes, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost), "C");
  nlm::ck(cudaMemcpy(Sdst, S.p, bytes, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost), "S");
}

nlm_status nlm_green(nlm_medium* h, int in_time_domain, int run_pump, unsigned n_threads, int normalize,
                     const uint8_t* use_input, size_t n_use_input, const uint8_t* use_output, size_t n_use_output,
                     double* green_c, double* green_s) {
  return guarded([&] {
    Medium* m = M(h);
    m->launches = 0;
    if (m->isCascade) {
      cascade_green(m, in_time_domain, run_pump, n_threads, normalize, use_input, n_use_input, use_output, n_use_output,
                    reinterpret_cast<double2*>(green_c), reinterpret_cast<double2*>(green_s), false);
      return;
    }
    m->green(in_time_domain, run_pump, n_threads, normalize, use_input, n_use_input, use_output, n_use_output,
             reinterpret_cast<double2*>(green_c), reinterpret_cast<double2*>(green_s), false);
  });
}

nlm_status nlm_green_device(nlm_medium* h, int in_time_domain, int run_pump, unsigned n_threads, int normalize,
                            const uint8_t* use_input, size_t n_use_input, const uint8_t* use_output, size_t n_use_output,
                            void* green_c_dev, void* green_s_dev) {
  return guarded([&] {
    Medium* m = M(h);
    m->launches = 0;
    if (m->isCascade) {
      cascade_green(m, in_time_domain, run_pump, n_threads, normalize, use_input, n_use_input, use_output, n_use_output,
                    nlm::d2(green_c_dev), nlm::d2(green_s_dev), true);
      return;
    }
    m->green(in_time_domain, run_pump, n_threads, normalize, use_input, n_use_input, use_output, n_use_output,
             nlm::d2(green_c_dev), nlm::d2(green_s_dev), true);
  });
}

nlm_status nlm_green_plain(nlm_medium* h, int in_time_domain, int run_pump, size_t max_instances, double* green_c,
                           double* green_s) {
  return guarded([&] {
    Medium* m = M(h);
    m->launches = 0;
    m->green(in_time_domain, run_pump, 1, 0, nullptr, 0, nullptr, 0, reinterpret_cast<double2*>(green_c),
             reinterpret_cast<double2*>(green_s), false, (long long)max_instances);
  });
}

nlm_status nlm_batch_dims(nlm_medium* h, size_t rows, size_t cols, unsigned n_threads, unsigned input_mode,
                          const uint8_t* use_output, size_t n_use_output, size_t* out_cols) {
  return guarded([&] {
    Medium* m = M(h);
    if (m->isCascade) {
      // outputs of the last medium (src/Cascade.cpp:160-162)
      Medium* last = m->media.back();
      std::vector<int> outs;
      m->media[0]->batchModes(rows, cols, n_threads, input_mode, nullptr, 0, outs);
      last->batchModes(rows, last->N, n_threads, 0, use_output, n_use_output, outs);
      *out_ptr(out_cols) = outs.size() * last->N;
      return;
    }
    std::vector<int> outs;
    m->batchModes(rows, cols, n_threads, input_mode, use_output, n_use_output, outs);
    *out_ptr(out_cols) = outs.size() * m->N;
  });
}

static void cascade_batch(Medium* c, const double2* in, size_t rows, size_t cols, int inTime, int runPump,
                          unsigned nThreads, unsigned inputMode, const uint8_t* useOut, size_t nUseOut, double2* out,
                          bool device) {
  if (runPump) cascade_run_pump(c);
  const size_t last = c->media.size() - 1;
  Medium* m0 = c->media[0];
  std::vector<int> outs;
  m0->batchModes(rows, cols, nThreads, inputMode, last == 0 ? useOut : nullptr, last == 0 ? nUseOut : 0, outs);
  size_t curCols = outs.size() * m0->N;
  nlm::DevBuf<double2> a, b;
  a.alloc(rows * curCols);
  nlm::DevBuf<double2> inD;
  const double2* src = in;
  if (!device) {
    inD.alloc(rows * cols);
    nlm::ck(cudaMemcpy(inD.p, in, rows * cols * sizeof(double2), cudaMemcpyHostToDevice), "upload");
    src = inD.p;
  }
  m0->batch(src, rows, cols, inTime, 0, nThreads, inputMode, last == 0 ? useOut : nullptr, last == 0 ? nUseOut : 0,
            a.p, true);
  for (size_t i = 1; i < c->media.size(); i++) {
    Medium* mi = c->media[i];
    std::vector<int> o;
    mi->batchModes(rows, curCols, nThreads, 0, i == last ? useOut : nullptr, i == last ? nUseOut : 0, o);
    const size_t nc = o.size() * mi->N;
    b.alloc(rows * nc);
    mi->batch(a.p, rows, curCols, inTime, 0, nThreads, 0, i == last ? useOut : nullptr, i == last ? nUseOut : 0, b.p, true);
    std::swap(a.p, b.p);
    std::swap(a.n, b.n);
    curCols = nc;
  }
  nlm::ck(cudaMemcpy(out, a.p, rows * curCols * sizeof(double2), device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost),
          "download");
}

nlm_status nlm_batch(nlm_medium* h, const double* inputs, size_t rows, size_t cols, int in_time_domain, int run_pump,
                     unsigned n_threads, unsigned input_mode, const uint8_t* use_output, size_t n_use_output, double* out) {
  return guarded([&] {
    Medium* m = M(h);
    m->launches = 0;
    if (m->isCascade) {
      cascade_batch(m, reinterpret_cast<const double2*>(inputs), rows, cols, in_time_domain, run_pump, n_threads,
                    input_mode, use_output, n_use_output, reinterpret_cast<double2*>(out), false);
      return;
    }
    m->batch(reinterpret_cast<const double2*>(inputs), rows, cols, in_time_domain, run_pump, n_threads, input_mode,
             use_output, n_use_output, reinterpret_cast<double2*>(out), false);
  });
}

nlm_status nlm_batch_device(nlm_medium* h, const void* inputs_dev, size_t rows, size_t cols, int in_time_domain,
                            int run_pump, unsigned n_threads, unsigned input_mode, const uint8_t* use_output,
                            size_t n_use_output, void* out_dev) {
  return guarded([&] {
    Medium* m = M(h);
    m->launches = 0;
    if (m->isCascade) {
      cascade_batch(m, reinterpret_cast<const double2*>(inputs_dev), rows, cols, in_time_domain, run_pump, n_threads,
                    input_mode, use_output, n_use_output, nlm::d2(out_dev), true);
      return;
    }
    m->batch(reinterpret_cast<const double2*>(inputs_dev), rows, cols, in_time_domain, run_pump, n_threads, input_mode,
             use_output, n_use_output, nlm::d2(out_dev), true);
  });
}


nlm_status nlm_get_grid(nlm_medium* h, int which, unsigned index, const double** data, size_t* rows, size_t* cols) {
  return guarded([&] {
    Medium* m = M(h);
    if (which == 4) throw nlm::IndexError("vector::_M_range_check: field index out of range");  // no solver has fields
    size_t r = 0;
    out_ptr(data), out_ptr(rows), out_ptr(cols);
    const std::vector<double>& v = m->mirror(which, index, &r);
    *data = v.data();
    *rows = r;
    *cols = m->N;
  });
}

nlm_status nlm_get_axis(nlm_medium* h, int which, unsigned index, const double** data, size_t* n) {
  return guarded([&] {
    Medium* m = M(h);
    out_ptr(data), out_ptr(n);
    if (m->isCascade) m = m->media.at(0);
    switch (which) {
      case 0: *data = m->tau.data(); *n = m->tau.size(); break;
      case 1: *data = m->omega.data(); *n = m->omega.size(); break;
      case 2:
        if (M(h)->isCascade) { *data = nullptr; *n = 0; break; }
        *data = m->poling.data(); *n = m->poling.size(); break;
      case 3: {
        if (m->solver != nlm::kChi3GNLSE) throw std::invalid_argument("not a Chi3GNLSE medium");
        m->ensureDevice();
        m->axisBuf.resize(2 * m->N);
        for (nlm::uint k = 0; k < m->N; k++) {
          m->axisBuf[2 * k] = m->raman[k].real();
          m->axisBuf[2 * k + 1] = m->raman[k].imag();
        }
        *data = m->axisBuf.data();
        *n = m->N;
        break;
      }
      case 4: {
        if (index >= m->envelope.size()) throw nlm::IndexError("pump index out of range");
        *data = reinterpret_cast<const double*>(m->envelope[index].data());
        *n = m->envelope[index].size();
        break;
      }
      default: throw std::invalid_argument("unknown axis");
    }
  });
}

nlm_status nlm_cascade_create(nlm_medium* const* media, size_t n_media, const unsigned* connections,
                              const size_t* conn_counts, size_t n_junctions, int share_pump, nlm_medium** out) {
  return guarded([&] {
    // src/Cascade.cpp:3-36
    if (n_media == 0) throw std::invalid_argument("Cascade must contain at least one medium");
    std::unique_ptr<Medium> c(new Medium());
    c->isCascade = true;
    Medium* first = M(media[0]);
    c->N = first->N;
    c->tMax = first->tMax;
    c->solver = -1;
    for (size_t i = 0; i < n_media; i++) {
      Medium* m = M(media[i]);
      if (m->isCascade) throw std::invalid_argument("nested cascades are not supported");
      if (m->N != c->N || m->tMax != c->tMax)
        throw std::invalid_argument("Medium does not have same time and frequency axes as the first");
      c->media.push_back(m);
    }
    if (n_junctions != n_media - 1) throw std::invalid_argument("Must have one connection per pair of adjacent media");
    size_t off = 0;
    for (size_t i = 0; i + 1 < n_media; i++) {
      const size_t cnt = conn_counts ? conn_counts[i] : 0;
      if (cnt == 0) throw std::invalid_argument("Connections missing between media!");
      std::map<nlm::uint, nlm::uint> conn;
      for (size_t k = 0; k < cnt; k++) {
        const unsigned first_ = connections[2 * (off + k)], second = connections[2 * (off + k) + 1];
        if (second >= c->media[i]->nSignal || first_ >= c->media[i + 1]->nSignal)
          throw std::invalid_argument("Invalid connections, out of range");
        conn[first_] = second;
      }
      off += cnt;
      c->connections.push_back(conn);
    }
    c->sharedPump = share_pump != 0;
    *out = new nlm_medium{c.release()};
  });
}

nlm_status nlm_cascade_add(nlm_medium* cascade, nlm_medium* medium, const unsigned* connection, size_t n_pairs) {
  return guarded([&] {
    // src/Cascade.cpp:39-52
    Medium* c = M(cascade);
    Medium* m = M(medium);
    if (!c->isCascade) throw std::invalid_argument("not a cascade");
    if (m->N != c->N || m->tMax != c->tMax)
      throw std::invalid_argument("Medium does not have same time and frequency axes as the first");
    if (n_pairs == 0) throw std::invalid_argument("No connection!");
    std::map<nlm::uint, nlm::uint> conn;
    for (size_t k = 0; k < n_pairs; k++) {
      const unsigned first_ = connection[2 * k], second = connection[2 * k + 1];
      if (second >= c->media.back()->nSignal || first_ >= m->nSignal)
        throw std::invalid_argument("Invalid connections, out of range");
      conn[first_] = second;
    }
    c->media.push_back(m);
    c->connections.push_back(conn);
  });
}

nlm_status nlm_cascade_media(const nlm_medium* cascade, size_t* n_media) {
  return guarded([&] {
    const Medium* c = CM(cascade);
    *out_ptr(n_media) = c->isCascade ? c->media.size() : 0;
  });
}

nlm_status nlm_green_rows(nlm_medium* h, int in_time_domain, int run_pump, size_t first, size_t count, double* raw_out) {
  return guarded([&] {
    Medium* m = M(h);
    m->launches = 0;
    m->greenRows(in_time_domain, run_pump, (long long)first, (long long)count, reinterpret_cast<double2*>(raw_out));
  });
}

nlm_status nlm_green_finish(nlm_medium* h, const double* raw, int normalize, double* green_c, double* green_s) {
  return guarded([&] {
    Medium* m = M(h);
    m->launches = 0;
    m->greenFinish(reinterpret_cast<const double2*>(raw), normalize, reinterpret_cast<double2*>(green_c),
                   reinterpret_cast<double2*>(green_s));
  });
}

nlm_status nlm_green_rows_device(nlm_medium* h, int in_time_domain, int run_pump, size_t first, size_t count,
                                 void* raw_out_dev) {
  return guarded([&] {
    Medium* m = M(h);
    m->launches = 0;
    if (count > 0 && !raw_out_dev) throw std::invalid_argument("null device pointer");
    m->greenRows(in_time_domain, run_pump, (long long)first, (long long)count, nlm::d2(raw_out_dev), true);
  });
}

nlm_status nlm_green_finish_device(nlm_medium* h, const void* raw_dev, int normalize, void* green_c_dev,
                                   void* green_s_dev) {
  return guarded([&] {
    Medium* m = M(h);
    m->launches = 0;
    if (!raw_dev || !green_c_dev || !green_s_dev) throw std::invalid_argument("null device pointer");
    m->greenFinish(reinterpret_cast<const double2*>(raw_dev), normalize, nlm::d2(green_c_dev), nlm::d2(green_s_dev),
                   true);
  });
}

nlm_status nlm_set_poling_profile(nlm_medium* h, const double* profile, size_t n) {
  return guarded([&] { M(h)->setPolingProfile(profile, n); });
}

nlm_status nlm_adjoint_forward(nlm_medium* h, const void* inputs_dev, size_t rows, void* out_dev,
                               int checkpoint_interval, int* used_interval) {
  return guarded([&] {
    Medium* m = M(h);
    m->launches = 0;
    m->adjointForward(reinterpret_cast<const double2*>(inputs_dev), rows, nlm::d2(out_dev), checkpoint_interval);
    if (used_interval) *used_interval = m->adjK;
  });
}

nlm_status nlm_adjoint_backward(nlm_medium* h, const void* grad_out_dev, void* grad_in_dev, void* grad_pump_dev,
                                double* grad_poling) {
  return guarded([&] {
    Medium* m = M(h);
    m->launches = 0;
    m->adjointBackward(reinterpret_cast<const double2*>(grad_out_dev), nlm::d2(grad_in_dev), nlm::d2(grad_pump_dev),
                       grad_poling);
  });
}

nlm_status nlm_set_stream(nlm_medium* h, void* cuda_stream) {
  return guarded([&] {
    Medium* m = M(h);
    if (m->ownStream && m->stream) cudaStreamDestroy(m->stream);
    m->ownStream = false;
    m->stream = reinterpret_cast<cudaStream_t>(cuda_stream);
    if (!m->stream) {
      nlm::require_device();
      nlm::ck(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking), "stream");
      m->ownStream = true;
    }
  });
}

nlm_status nlm_synchronize(nlm_medium* h) {
  return guarded([&] {
    Medium* m = M(h);
    if (m->stream) nlm::ck(cudaStreamSynchronize(m->stream), "synchronize");
  });
}

int nlm_device_available(void) { return nlm::device_count() > 0 ? 1 : 0; }

nlm_status nlm_set_schedule(nlm_medium* h, int cta_per_sm, int use_propagator, int use_graph) {
  return guarded([&] {
    Medium* m = M(h);
    m->ctaPerSM = cta_per_sm;
    m->usePropagator = use_propagator;
    m->useGraph = use_graph;
  });
}

nlm_status nlm_set_cluster(nlm_medium* h, int enable) {
  return guarded([&] {
    Medium* m = M(h);
    if (enable < 0 || enable > 3) throw std::invalid_argument("cluster mode must be 0, 1, 2 or 3");
    m->useCluster = enable;
    for (Medium* c : m->media) c->useCluster = m->useCluster;
  });
}

nlm_status nlm_set_precision(nlm_medium* h, int precision) {
  return guarded([&] {
    if (precision != 0 && precision != 1) throw std::invalid_argument("precision must be 0 (FP64) or 1 (double-float)");
    Medium* m = M(h);
    m->precision = precision;
    for (Medium* c : m->media) c->precision = precision;
  });
}

nlm_status nlm_last_schedule(const nlm_medium* h, int* values) {
  return guarded([&] {
    const Medium* m = CM(h);
    values[0] = m->lastR;
    values[1] = m->lastSchedule.ipc;
    values[2] = m->lastSchedule.grid;
    values[3] = m->lastSchedule.block;
    values[4] = m->lastSchedule.ctas;
    values[5] = m->lastTuned;
    values[6] = (int)m->tuneTrials;
    values[7] = m->lastRegs;
  });
}

nlm_status nlm_graph_stats(const nlm_medium* h, long* captures, long* replays) {
  return guarded([&] {
    const Medium* m = CM(h);
    long c = m->graphs.captures, r = m->graphs.replays;
    for (const Medium* x : m->media) {
      c += x->graphs.captures;
      r += x->graphs.replays;
    }
    if (captures) *captures = c;
    if (replays) *replays = r;
  });
}

nlm_status nlm_last_launch_count(const nlm_medium* h, long* launches) {
  return guarded([&] { *launches = CM(h)->launches; });
}

nlm_status nlm_kernel_timing(nlm_medium* h, int enable, double* total_ms, long* count) {
  return guarded([&] {
    Medium* m = M(h);
    if (total_ms) *total_ms = m->kernelMs;
    if (count) *count = m->kernelCount;
    if (enable == 1) {
      m->kernelMs = 0;
      m->kernelCount = 0;
    }
    m->timeKernels = enable != 0;
  });
}

namespace {
// Two CUDA events, destroyed however the scope is left.
struct EventPair {
  cudaEvent_t a = nullptr, b = nullptr;
  EventPair() {
    nlm::ck(cudaEventCreate(&a), "event");
    if (cudaEventCreate(&b) != cudaSuccess) {
      cudaEventDestroy(a);
      throw std::runtime_error("event: cudaEventCreate failed");
    }
  }
  ~EventPair() {
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }
  EventPair(const EventPair&) = delete;
  EventPair& operator=(const EventPair&) = delete;
};

// Best of three timed launches (after one warm-up) of a peak kernel on blocksPerSM CTAs of `threads`
// threads per SM; flopsPerThreadIter flops per thread and iteration.
double time_peak(const std::function<cudaError_t(double*, int, int, int)>& launch, int iters, double flopsPerThreadIter,
                 int blocksPerSM = 4, int threads = 256) {
  int dev = 0, sms = 1;
  nlm::ck(cudaGetDevice(&dev), "device");
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * blocksPerSM;
  nlm::DevBuf<double> out;
  out.alloc((size_t)blocks * threads);
  EventPair ev;
  double best = 0;
  for (int rep = 0; rep < 4; rep++) {
    nlm::ck(cudaEventRecord(ev.a, 0), "event");
    nlm::ck(launch(out.p, iters, blocks, threads), "peak kernel");
    nlm::ck(cudaEventRecord(ev.b, 0), "event");
    nlm::ck(cudaEventSynchronize(ev.b), "event");
    float ms = 0;
    nlm::ck(cudaEventElapsedTime(&ms, ev.a, ev.b), "event");
    const double flops = flopsPerThreadIter * iters * (double)blocks * threads;
    if (rep > 0) best = std::max(best, flops / (ms * 1e-3) / 1e12);
  }
  return best;
}

}  // namespace

nlm_status nlm_fp64_peak(double* tflops) {
  return guarded([&] {
    nlm::require_device();
    // 32 FMAs (64 flops) per thread and iteration
    *out_ptr(tflops) = time_peak([](double* o, int it, int bl, int th) { return nlm::launch_fp64_peak(o, it, bl, th, 0); },
                                 2000, 64.0);
  });
}

nlm_status nlm_quadrature_greens(const void* green_c_dev, const void* green_s_dev, size_t rows, size_t cols,
                                 void* z_dev, void* cuda_stream) {
  return guarded([&] {
    nlm::require_device();
    if (!green_c_dev || !green_s_dev || !z_dev) throw std::invalid_argument("null device pointer");
    nlm::ck(nlm::launch_quadrature_z(reinterpret_cast<const double2*>(green_c_dev),
                                     reinterpret_cast<const double2*>(green_s_dev), (long long)rows, (long long)cols,
                                     static_cast<double*>(z_dev), static_cast<cudaStream_t>(cuda_stream)),
            "quadrature Z");
  });
}

nlm_status nlm_abasis_greens(const void* green_c_dev, const void* green_s_dev, size_t rows, size_t cols, void* z_dev,
                             void* cuda_stream) {
  return guarded([&] {
    nlm::require_device();
    if (!green_c_dev || !green_s_dev || !z_dev) throw std::invalid_argument("null device pointer");
    nlm::ck(nlm::launch_abasis_z(reinterpret_cast<const double2*>(green_c_dev),
                                 reinterpret_cast<const double2*>(green_s_dev), (long long)rows, (long long)cols,
                                 nlm::d2(z_dev), static_cast<cudaStream_t>(cuda_stream)),
            "a-basis Z");
  });
}

nlm_status nlm_cascade_compose(const void* c2_dev, const void* s2_dev, const void* c1_dev, const void* s1_dev,
                               size_t rows, size_t inner, size_t cols, void* c_out_dev, void* s_out_dev,
                               void* cuda_stream) {
  return guarded([&] {
    nlm::require_device();
    if (!c2_dev || !s2_dev || !c1_dev || !s1_dev || !c_out_dev || !s_out_dev)
      throw std::invalid_argument("null device pointer");
    if (rows == 0 || inner == 0 || cols == 0) throw std::invalid_argument("empty matrices");
    if (rows > (size_t)INT32_MAX || inner > (size_t)INT32_MAX || cols > (size_t)INT32_MAX)
      throw std::invalid_argument("matrix dimension too large");
    nlm::ck(nlm::launch_cgemm_compose(reinterpret_cast<const double2*>(c2_dev), reinterpret_cast<const double2*>(s2_dev),
                                      reinterpret_cast<const double2*>(c1_dev), reinterpret_cast<const double2*>(s1_dev),
                                      (int)rows, (int)inner, (int)cols, nlm::d2(c_out_dev), nlm::d2(s_out_dev),
                                      static_cast<cudaStream_t>(cuda_stream)),
            "compose");
  });
}

nlm_status nlm_fp64_warps_rate(int warps_per_sm, double* tflops) {
  return guarded([&] {
    nlm::require_device();
    if (warps_per_sm < 1 || warps_per_sm > 32) throw std::invalid_argument("warps_per_sm must be 1..32");
    // one CTA of warps_per_sm warps on every SM, 32 FMAs per thread and iteration
    *out_ptr(tflops) = time_peak([](double* o, int it, int bl, int th) { return nlm::launch_fp64_peak(o, it, bl, th, 0); },
                                 2000, 64.0, 1, 32 * warps_per_sm);
  });
}

nlm_status nlm_fp64_mma_peak(double* tflops) {
  return guarded([&] {
    nlm::require_device();
    // 4 m16n8k16 MMAs per warp and iteration: 4 x 2 x 16 x 8 x 16 flops over 32 threads
    *out_ptr(tflops) = time_peak(
        [](double* o, int it, int bl, int th) { return nlm::launch_fp64_mma_peak(o, it, bl, th, 0); }, 200,
        4.0 * 2 * 16 * 8 * 16 / 32);
  });
}

}  // extern "C"
