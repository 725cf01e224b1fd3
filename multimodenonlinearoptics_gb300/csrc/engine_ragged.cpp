// engine_ragged.cpp -- nlm_ragged_batch: one call over a ragged set of media (different grids and step
// counts), scheduled for its makespan over the SMs and captured into a CUDA graph.
//
// Every medium is a sequential z march; it can run in one of four forms:
//   one  -- one CTA (one SM) in a ragged launch, whose CTAs claim media largest first;
//   c4   -- a 4-CTA cluster on four SMs (one point per thread up to 1024 points, four from 2048);
//   w8   -- an 8-CTA cluster on eight SMs, one point per thread (1024 to 4096 points);
//   w16  -- a 16-CTA cluster (a non-portable size) on sixteen SMs, one point per thread.
// The larger forms finish a medium sooner but spend more SM time on it.  The planner picks a target
// makespan T (the smallest feasible one, scanned upward): every medium takes the form of least SM
// time that finishes within T; cluster-form media are packed first-fit, largest first, into slots (a
// stream running its media one after another on 4, 8 or 16 SMs); the one-SM media of each solver and
// grid share a ragged launch.  T is feasible when the slots fit in the SMs clusters can hold at once
// and the slots and the ragged launches together in the device's SMs.  The call is then enqueued on
// those streams (inputs in one copy, outputs in one copy) and captured into a CUDA graph, replayed by
// later calls with the same plan.
#include <cstdlib>
#include <map>

#include "engine.h"

using nlm::guarded;
using nlm::Medium;

namespace {

using namespace nlm;

enum Form { kOne = 0, kC4 = 1, kW8 = 2, kW16 = 3, kForms = 4 };
constexpr int kFormSMs[kForms] = {1, 4, 8, 16};

// Per-step time (microseconds) of a two-mode pump-driven medium (Chi2SFG) in each form on a GB300,
// measured with one propagation of 1199 steps per form: [RK4 propagator used][form][log2 N - 7] for
// N = 128 .. 2048 (eight CTAs from 1024 points, sixteen at 2048).  Zero: the form does not exist for that grid.  Larger grids scale as N log2 N from
// the table's end, smaller ones take the 128-point time (latency-bound); other solvers scale with
// their mode count.
constexpr double kStepUs[2][kForms][5] = {
    {{26.4, 27.9, 34.8, 67.9, 137.8}, {9.8, 10.5, 12.0, 21.0, 41.8}, {0, 0, 0, 14.3, 25.5}, {0, 0, 0, 0, 20.6}},
    {{18.4, 19.9, 27.8, 51.8, 99.5}, {7.7, 8.5, 10.0, 16.9, 33.7}, {0, 0, 0, 12.5, 21.5}, {0, 0, 0, 0, 19.3}}};

double step_us(int form, uint N, uint modes, bool prop) {
  int lg = 0;
  while ((1u << lg) < N) lg++;
  const int i = std::min(std::max(lg - 7, 0), 4);
  double t = kStepUs[prop ? 1 : 0][form][i];
  if (t == 0) return -1;
  if (lg > 11) t *= (double)N * lg / (2048.0 * 11);
  return t * std::max(1u, modes) / 2.0;
}

struct Job {
  size_t k;                  // index in the call's media
  int cls;                   // ragged launch class: media of one solver and one grid share a launch
  double t[kForms];          // estimated march time per form (us); < 0: form not available
  double best() const {
    double b = -1;
    for (double x : t)
      if (x >= 0 && (b < 0 || x < b)) b = x;
    return b;
  }
};

struct Plan {
  std::vector<int> form;                    // per job
  std::vector<std::vector<size_t>> slots;   // cluster slots: job indices in launch order
  std::vector<int> slotForm;
  int poolSMs = 0;                          // CTAs of the ragged launches
  std::map<int, int> classCTAs;             // per ragged launch class: its fewest CTAs (multiple of 4)
  double makespan = 0;
};

// Largest-first list schedule of `times` (descending) on m one-SM CTAs: its makespan.  The ragged
// launch's CTAs claim media in that order from a counter, which is this schedule.
double lpt_makespan(const std::vector<double>& times, int m) {
  std::vector<double> load((size_t)m, 0.0);
  for (double t : times) *std::min_element(load.begin(), load.end()) += t;
  return *std::max_element(load.begin(), load.end());
}

// Plan for target makespan T (us); false when the slots need more than `sms` SMs (the cluster budget)
// or the slots and the ragged launches more than poolSms.  maxW16: the sixteen-CTA slots that can run
// at once (one per GPC that holds sixteen SMs); gran: the ragged CTAs come in groups of gran.
bool plan_for(const std::vector<Job>& jobs, double T, int sms, int maxW16, int poolSms, int gran, Plan* out) {
  Plan p;
  p.form.assign(jobs.size(), -1);
  std::vector<double> slotLoad;
  // largest first (by the time of the fastest form)
  std::vector<size_t> order(jobs.size());
  for (size_t i = 0; i < order.size(); i++) order[i] = i;
  std::sort(order.begin(), order.end(), [&](size_t a, size_t b) { return jobs[a].best() > jobs[b].best(); });
  int used = 0, w16 = 0;
  for (size_t i : order) {
    const Job& j = jobs[i];
    // the forms that finish within T, least SM time first; a slot form takes the first slot of its
    // form with room, or a new slot (sixteen-CTA slots up to maxW16)
    int forms[kForms], nf = 0;
    for (int c = 0; c < kForms; c++)
      if (j.t[c] >= 0 && j.t[c] <= T) forms[nf++] = c;
    std::sort(forms, forms + nf, [&](int a, int b) { return j.t[a] * kFormSMs[a] < j.t[b] * kFormSMs[b]; });
    bool placed = false;
    for (int q = 0; q < nf && !placed; q++) {
      const int f = forms[q];
      if (f == kOne) {
        p.form[i] = f;
        placed = true;
        break;
      }
      size_t s = 0;
      for (; s < slotLoad.size(); s++)
        if (p.slotForm[s] == f && slotLoad[s] + j.t[f] <= T) break;
      if (s == slotLoad.size()) {
        if (f == kW16 && w16 >= maxW16) continue;
        slotLoad.push_back(0);
        p.slotForm.push_back(f);
        p.slots.emplace_back();
        used += kFormSMs[f];
        if (f == kW16) w16++;
      }
      slotLoad[s] += j.t[f];
      p.slots[s].push_back(i);
      p.form[i] = f;
      placed = true;
    }
    if (!placed) return false;
  }
  if (used > sms) return false;
  // per ragged launch class (the CTAs of a launch are sized for its grid), the fewest one-SM CTAs
  // whose largest-first schedule fits within T, in groups of gran
  std::map<int, std::vector<double>> byClass;
  for (size_t i : order)
    if (p.form[i] == kOne) byClass[jobs[i].cls].push_back(jobs[i].t[kOne]);
  int m = 0;
  for (auto& kv : byClass) {
    std::vector<double>& pool = kv.second;
    std::sort(pool.begin(), pool.end(), std::greater<double>());
    double sum = 0;
    for (double t : pool) sum += t;
    int mc = std::max(1, (int)std::ceil(sum / T));
    while (mc < (int)pool.size() && lpt_makespan(pool, mc) > T) mc++;
    if (lpt_makespan(pool, mc) > T) return false;
    mc = (mc + gran - 1) / gran * gran;
    p.classCTAs[kv.first] = mc;
    m += mc;
  }
  if (used + m > poolSms) return false;
  p.poolSMs = m;
  p.makespan = T;
  *out = p;
  return true;
}

// The plan of a set.  The makespan lies between the longest medium in its fastest form and every
// medium on one SM one after another.  Feasibility need not be monotonic in T (a medium at the edge of
// T moves between forms), so the targets are scanned upward in steps of 0.25 % and the first feasible
// one is taken.  When none fits the SMs at once (more cluster-only media than they hold), every medium
// takes its fastest form, each cluster medium a slot of its own, and the slots queue for SMs: false.
bool plan_set(const std::vector<Job>& jobs, int budget, int maxW16, int poolBudget, int gran, Plan* out) {
  double lo = 0, hi = 0;
  for (const Job& j : jobs) {
    lo = std::max(lo, j.best());
    hi += j.t[kOne] >= 0 ? j.t[kOne] : j.best();
  }
  for (double T = lo; lo > 0 && T <= hi * 1.0001; T *= 1.0025)
    if (plan_for(jobs, T, budget, maxW16, poolBudget, gran, out)) return true;
  if (plan_for(jobs, hi, budget, maxW16, poolBudget, gran, out)) return true;
  Plan plan;
  plan.form.assign(jobs.size(), kOne);
  for (size_t i = 0; i < jobs.size(); i++) {
    int f = kOne;
    for (int c = 0; c < kForms; c++)
      if (jobs[i].t[c] >= 0 && (jobs[i].t[f] < 0 || jobs[i].t[c] < jobs[i].t[f])) f = c;
    plan.form[i] = f;
    if (f != kOne) {
      plan.slots.push_back({i});
      plan.slotForm.push_back(f);
    } else {
      plan.classCTAs[jobs[i].cls] += 1;
    }
  }
  plan.poolSMs = 0;
  for (auto& kv : plan.classCTAs) plan.poolSMs += (kv.second = (kv.second + 3) / 4 * 4);
  *out = plan;
  return false;
}

// SMs that clusters of four CTAs, each CTA alone on its SM, can hold at once: every cluster sits in
// one GPC, so the SMs of a GPC beyond a multiple of four stay out of reach (on a GB300 with 19 SMs per
// GPC, 128 of the 152).  Measured once per process with the occupancy API on `fn`.
// NLM_RAGGED_CLUSTER_SMS overrides the measured figure.
int cluster_capacity_sms(const void* fn, int sms) {
  static int cached = 0;
  if (cached) return cached;
  if (const char* env = std::getenv("NLM_RAGGED_CLUSTER_SMS")) {
    const int v = std::atoi(env);
    if (v >= 4) return cached = std::min(v, sms);
  }
  size_t smem = 0;
  int cap = sms - 4;
  if (exclusive_smem(fn, 1024 * sizeof(double2), &smem) == cudaSuccess && smem) {
    cudaLaunchAttribute attr;
    cudaLaunchConfig_t cfg = cluster_config(4 * sms, 128, smem, nullptr, 4, &attr);
    int n = 0;
    const cudaError_t e = cudaOccupancyMaxActiveClusters(&n, fn, &cfg);
    if (e == cudaSuccess && n > 0) cap = std::min(cap, 4 * n);
    else cudaGetLastError();
  }
  cached = cap;
  return cached;
}
int g_capacityUsed = 0;
std::map<std::vector<double>, Plan> g_planCache;   // recent sets' plans (under the ragged workspace's mutex)

// Sixteen-SM slots that can run at once: the 16-CTA clusters of medium m's kernel (prop_spread_w16.cu)
// that fit on the device, one per GPC of sixteen SMs or more.  NLM_RAGGED_W16_SLOTS overrides the
// figure (0 turns the form off).
int w16_capacity(Medium* m) {
  if (const char* env = std::getenv("NLM_RAGGED_W16_SLOTS")) return std::max(0, std::atoi(env));
  const KernelEntry* k = m->w16Kernel();
  return k ? m->w16Clusters(k) : 0;
}

}  // namespace

extern "C" {

// Workspace of the ragged call (process-wide; calls are serialised by the mutex).
struct RaggedWorkspace {
  std::mutex mu;
  nlm::DevBuf<double2> in, out;                 // every fused medium's input and output, one block each
  nlm::DevBuf<nlm::PropArgs> items;             // the ragged launches' media
  nlm::PinnedBuf<double2> hin, hout;            // host staging of the inputs and outputs
  nlm::PinnedBuf<nlm::PropArgs> hitems;
  nlm::DevBuf<unsigned long long> counters;     // one work counter per ragged launch
  // The cluster slots' streams have the device's highest priority and the ragged launches' the lowest:
  // CTAs of the slots (and of each slot's next medium) are placed first wherever both wait for SMs, so
  // the one-SM CTAs never hold the GPC room a slot's cluster needs.
  cudaStream_t origin = nullptr;
  std::vector<cudaStream_t> slotStreams, poolStreams;
  std::vector<cudaEvent_t> events;
  cudaEvent_t t0 = nullptr, t1 = nullptr;        // timing events around the call on the origin stream
  nlm::GraphCache graphs;
  std::vector<unsigned char> lastKey;           // the previous call's plan
  // [0]: origin; then one per slot and one per ragged launch
  std::vector<cudaStream_t> callStreams(size_t nSlots, size_t nPool) {
    int least = 0, greatest = 0;
    ck(cudaDeviceGetStreamPriorityRange(&least, &greatest), "stream priorities");
    if (!origin) ck(cudaStreamCreateWithFlags(&origin, cudaStreamNonBlocking), "ragged stream");
    auto grow = [](std::vector<cudaStream_t>& v, size_t n, int prio) {
      while (v.size() < n) {
        cudaStream_t st = nullptr;
        ck(cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, prio), "ragged stream");
        v.push_back(st);
      }
    };
    grow(slotStreams, nSlots, greatest);
    grow(poolStreams, nPool, least);
    while (events.size() < 1 + nSlots + nPool) {
      cudaEvent_t e = nullptr;
      ck(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "ragged event");
      events.push_back(e);
    }
    std::vector<cudaStream_t> out{origin};
    out.insert(out.end(), slotStreams.begin(), slotStreams.begin() + (long)nSlots);
    out.insert(out.end(), poolStreams.begin(), poolStreams.begin() + (long)nPool);
    return out;
  }
};
static RaggedWorkspace g_ragged;

// What the last call planned and ran (nlm_ragged_last_plan).
struct RaggedStats {
  double makespan;
  int slotsC4, slotsW8, slotsW16, raggedCTAs;
  long captures, replays;
  int budget, w16Capacity;
  double gpuMs;   // device time of the call on its origin stream (CUDA events around the launch)
};
static RaggedStats g_lastRagged{0, 0, 0, 0, 0, 0, 0, 0, 0, 0};

nlm_status nlm_ragged_batch(nlm_medium* const* media, size_t n_media, const double* const* inputs, int in_time_domain,
                            double* const* outputs) {
  return guarded([&] {
    if (n_media == 0) return;
    std::vector<Medium*> ms(n_media);
    for (size_t k = 0; k < n_media; k++) {
      ms[k] = M(media[k]);
      if (ms[k]->isCascade) throw std::invalid_argument("ragged batches take single media");
      ms[k]->launches = 0;
    }
    // media without a ragged kernel (or with a grid it cannot take) run one batch call each
    std::vector<size_t> fused;
    for (size_t k = 0; k < n_media; k++) {
      Medium* m = ms[k];
      const KernelEntry* ke = m->findKernel(kKindRagged, m->solver, 8);
      const bool ok = ke && is_pow2((int)m->N) && m->N >= 8 && m->N / 8 <= 512;
      if (ok) {
        fused.push_back(k);
      } else {
        m->batch(reinterpret_cast<const double2*>(inputs[k]), 1, m->N, in_time_domain, 0, 1, 0, nullptr, 0,
                 reinterpret_cast<double2*>(outputs[k]), false);
      }
    }
    if (fused.empty()) return;
    std::lock_guard<std::mutex> lock(g_ragged.mu);
    for (size_t k : fused) {
      ms[k]->ensureDevice();
      ms[k]->flushPump();   // before any capture: the launches below read the pump grids
    }
    const int sms = Medium::smCount();

    // ---- plan: a form per medium (the RK4 propagator decision first: it changes the step cost) ----
    std::vector<bool> withProp(n_media, false), needBuild(n_media, false);
    for (size_t k : fused) {
      Medium* m = ms[k];
      withProp[k] = m->raggedPropagator();
      needBuild[k] = withProp[k] && !(m->propVersion == m->pumpVersion && m->prop.p);
    }
    std::vector<Job> jobs;
    for (size_t k : fused) {
      Medium* m = ms[k];
      int lg = 0;
      while ((1u << lg) < m->N) lg++;
      Job j{k, m->solver * 64 + lg, {-1, -1, -1, -1}};
      const double steps = (double)(m->nZ > 1 ? m->nZ - 1 : 1);
      j.t[kOne] = step_us(kOne, m->N, m->nSignal, withProp[k]) * steps;
      // four CTAs: one point per thread on the spread grids, four points per thread from 1024 points
      const bool c4 = (m->spreadGrid() && m->findKernel(kKindCluster, m->solver, 1)) || m->clusterGrid();
      if (c4) j.t[kC4] = step_us(kC4, m->N, m->nSignal, withProp[k]) * steps;
      if (m->w8Grid() && m->findKernel(kKindCluster, m->solver + kSpreadWideKey, 1))
        j.t[kW8] = step_us(kW8, m->N, m->nSignal, withProp[k]) * steps;
      if (m->w16Kernel()) j.t[kW16] = step_us(kW16, m->N, m->nSignal, withProp[k]) * steps;
      jobs.push_back(j);
    }
    int maxW16 = 0;
    for (const Job& j : jobs)
      if (j.t[kW16] >= 0) {
        maxW16 = w16_capacity(ms[j.k]);
        break;
      }
    // the makespan lies between the longest medium in its fastest form and every medium on one SM one
    // after another; the slots may use the SMs that clusters of four can hold at once
    const int budget = std::max(4, cluster_capacity_sms(ms[fused[0]]->findKernel(kKindRagged, ms[fused[0]]->solver, 8)->fn,
                                                        sms));
    g_capacityUsed = budget;
    // The ragged launches run without clusters, so their CTAs take any SM the slots leave, the SMs of
    // a GPC beyond its clusters' groups included: the slots must fit in the cluster budget, the slots
    // and the ragged CTAs together in all the device's SMs.  NLM_RAGGED_POOL_CLUSTERS=1 launches them
    // in clusters of four within the budget instead.  The plans of recent sets are kept: a repeated
    // call (the same estimates, budget and slot capacity) reuses its plan without the scan.
    const bool clusteredPool = std::getenv("NLM_RAGGED_POOL_CLUSTERS") != nullptr;
    const int gran = clusteredPool ? 4 : 1, poolBudget = clusteredPool ? budget : sms;
    std::vector<double> planKey{(double)budget, (double)maxW16, (double)clusteredPool};
    for (const Job& j : jobs) {
      planKey.push_back((double)j.cls);
      planKey.insert(planKey.end(), j.t, j.t + kForms);
    }
    Plan plan;
    auto cached = g_planCache.find(planKey);
    if (cached != g_planCache.end()) {
      plan = cached->second;
    } else if (plan_set(jobs, budget, maxW16, poolBudget, gran, &plan)) {
      if (g_planCache.size() >= 16) g_planCache.erase(g_planCache.begin());
      g_planCache[planKey] = plan;
    }

    // The plan's one-SM CTAs are the fewest that fit its target; the SMs the slots leave free all go to
    // the ragged launches (one CTA per medium at most), a margin against the estimates.
    int leftover = 0;
    {
      int slotSMs = 0;
      for (int f : plan.slotForm) slotSMs += kFormSMs[f];
      leftover = std::max(0, (poolBudget - slotSMs - plan.poolSMs) / gran * gran);
    }

    // ---- buffers, staging and the ragged launches' items (nothing is allocated inside the graph) ----
    std::vector<size_t> inOff(n_media, 0), outOff(n_media, 0);
    size_t inAll = 0, outAll = 0;
    for (size_t k : fused) {
      inOff[k] = inAll;
      outOff[k] = outAll;
      inAll += ms[k]->N;
      outAll += (size_t)ms[k]->nSignal * ms[k]->N;
    }
    g_ragged.in.reserve(inAll);
    g_ragged.out.reserve(outAll);
    g_ragged.hin.reserve(inAll);
    g_ragged.hout.reserve(outAll);
    for (size_t k : fused) std::memcpy(g_ragged.hin.p + inOff[k], inputs[k], ms[k]->N * sizeof(double2));
    for (size_t k : fused)
      if (withProp[k]) ms[k]->reservePropagator();
    auto rowArgs = [&](Medium* m, size_t k, int R) {
      PropArgs a = m->baseArgs(R);
      a.inKind = 1;
      a.inTime = in_time_domain ? 1 : 0;
      a.in = g_ragged.in.p + inOff[k];
      a.inStride = (long long)m->N;
      a.inChannels = 1;
      a.inputMode = 0;
      a.nOut = (int)m->nSignal;
      for (int mm = 0; mm < (int)m->nSignal; mm++) a.outModes[mm] = mm;
      a.out = g_ragged.out.p + outOff[k];
      a.outStride = (long long)m->nSignal * m->N;
      return a;
    };
    // one ragged launch per class (solver and grid) among the one-SM media, largest first, each with the
    // plan's CTAs for it and a share of the SMs left over (in proportion to its work)
    std::map<int, std::vector<size_t>> byClass;   // job indices
    double poolWork = 0;
    for (size_t i = 0; i < jobs.size(); i++)
      if (plan.form[i] == kOne) {
        byClass[jobs[i].cls].push_back(i);
        poolWork += jobs[i].t[kOne];
      }
    struct RaggedLaunch {
      const KernelEntry* ke;
      int grid, block, first, count;
      size_t smem;
    };
    std::vector<RaggedLaunch> raggedLaunches;
    std::vector<PropArgs> items;
    std::vector<size_t> itemJob;   // job index of every item
    for (auto& kv : byClass) {
      std::vector<size_t>& js = kv.second;
      const int solver = ms[jobs[js[0]].k]->solver;
      std::sort(js.begin(), js.end(), [&](size_t a, size_t b) { return jobs[a].t[kOne] > jobs[b].t[kOne]; });
      size_t maxN = 0;
      double work = 0;
      for (size_t i : js) {
        maxN = std::max<size_t>(maxN, ms[jobs[i].k]->N);
        work += jobs[i].t[kOne];
      }
      Medium* lead = ms[jobs[js[0]].k];
      // N/4 threads per medium when the largest grid allows it (four warps from N = 512), else N/8
      const KernelEntry* k4 = maxN / 4 <= 512 ? lead->findKernel(kKindRagged, solver, 4) : nullptr;
      const KernelEntry* ke = k4 ? k4 : lead->findKernel(kKindRagged, solver, 8);
      const int Rg = ke->R;
      RaggedLaunch rl{ke, 0, (int)((maxN / Rg + 31) / 32 * 32), (int)items.size(), (int)js.size(), 0};
      for (size_t i : js) {
        Medium* m = ms[jobs[i].k];
        PropArgs a = rowArgs(m, jobs[i].k, Rg);
        a.nInst = 1;
        a.ipc = 1;
        a.prop = withProp[jobs[i].k] ? m->prop.p : nullptr;
        items.push_back(a);
        itemJob.push_back(i);
      }
      // One CTA per SM: every medium is a sequential march bound by its SM's FP64 units.  Asking for
      // more than half of the SM's shared memory keeps other CTAs off its SM.
      cudaFuncAttributes fa;
      ck(exclusive_smem(ke->fn, maxN * sizeof(double2), &rl.smem, &fa), "smem attribute");
      if (rl.smem == 0) throw Unsupported("ragged kernel does not fit on an SM");
      if (rl.block > fa.maxThreadsPerBlock) throw Unsupported("ragged kernel cannot launch that many threads");
      // a share of the SMs the plan leaves free, in proportion to the launch's work
      const int extra = (int)((double)leftover * (poolWork > 0 ? work / poolWork : 1.0)) / gran * gran;
      const int most = ((int)js.size() + gran - 1) / gran * gran;
      rl.grid = std::min(most, std::max(gran, plan.classCTAs[kv.first] + extra));
      raggedLaunches.push_back(rl);
    }
    g_ragged.items.reserve(std::max<size_t>(items.size(), 1));
    g_ragged.hitems.reserve(std::max<size_t>(items.size(), 1));
    if (!items.empty()) std::memcpy(g_ragged.hitems.p, items.data(), items.size() * sizeof(PropArgs));
    g_ragged.counters.reserve(std::max<size_t>(raggedLaunches.size(), 1));
    const std::vector<cudaStream_t> streams = g_ragged.callStreams(plan.slots.size(), raggedLaunches.size());
    cudaStream_t origin = streams[0];

    // ---- the call: one input copy, the slots and ragged launches on their streams, one output copy --
    auto record = [&] {
      ck(cudaMemcpyAsync(g_ragged.in.p, g_ragged.hin.p, inAll * sizeof(double2), cudaMemcpyHostToDevice, origin),
         "ragged inputs");
      if (!items.empty())
        ck(cudaMemcpyAsync(g_ragged.items.p, g_ragged.hitems.p, items.size() * sizeof(PropArgs),
                           cudaMemcpyHostToDevice, origin),
           "ragged items");
      if (!raggedLaunches.empty())
        ck(cudaMemsetAsync(g_ragged.counters.p, 0, raggedLaunches.size() * sizeof(unsigned long long), origin),
           "ragged counters");
      ck(cudaEventRecord(g_ragged.events[0], origin), "ragged fork");
      size_t si = 1;
      for (size_t s = 0; s < plan.slots.size(); s++, si++) {
        cudaStream_t st = streams[si];
        ck(cudaStreamWaitEvent(st, g_ragged.events[0], 0), "ragged fork");
        for (size_t i : plan.slots[s]) {
          const size_t k = jobs[i].k;
          Medium* m = ms[k];
          const cudaStream_t own = m->stream;
          m->stream = st;
          m->raggedWide = plan.slotForm[s] == kW8;
          m->raggedW16 = plan.slotForm[s] == kW16;
          try {
            m->propagate(rowArgs(m, k, m->chooseR()), 1, withProp[k]);
          } catch (...) {
            m->stream = own;
            m->raggedWide = m->raggedW16 = false;
            throw;
          }
          m->stream = own;
          m->raggedWide = m->raggedW16 = false;
        }
      }
      for (size_t r = 0; r < raggedLaunches.size(); r++, si++) {
        const RaggedLaunch& rl = raggedLaunches[r];
        cudaStream_t st = streams[si];
        ck(cudaStreamWaitEvent(st, g_ragged.events[0], 0), "ragged fork");
        // the one-SM media's RK4 matrices, each built in parallel over all steps and points just before
        for (int q = rl.first; q < rl.first + rl.count; q++) {
          const size_t k = jobs[itemJob[q]].k;
          if (needBuild[k]) ms[k]->buildPropagator(8, st);
        }
        PropArgs* itemsD = g_ragged.items.p + rl.first;
        unsigned long long* ctr = g_ragged.counters.p + r;
        int nIt = rl.count;
        void* args[] = {(void*)&itemsD, (void*)&nIt, (void*)&ctr};
        ck(launch_clustered(rl.ke->fn, rl.grid, rl.block, rl.smem, st, gran, args), "ragged launch");
      }
      for (size_t j = 1; j < si; j++) {
        ck(cudaEventRecord(g_ragged.events[j], streams[j]), "ragged join");
        ck(cudaStreamWaitEvent(origin, g_ragged.events[j], 0), "ragged join");
      }
      ck(cudaMemcpyAsync(g_ragged.hout.p, g_ragged.out.p, outAll * sizeof(double2), cudaMemcpyDeviceToHost, origin),
         "ragged outputs");
    };

    // ---- one CUDA graph per plan: every host value the launches read goes into its key ----
    bool useGraph = true;
    GraphKey key;
    key.add(in_time_domain).add(inAll).add(outAll).add(g_ragged.in.p).add(g_ragged.out.p).add(g_ragged.hin.p);
    key.add(g_ragged.hout.p).add(g_ragged.items.p).add(g_ragged.hitems.p).add(g_ragged.counters.p);
    for (size_t k : fused) {
      Medium* m = ms[k];
      useGraph = useGraph && m->useGraph && !m->timeKernels;
      key.add(m).add((bool)withProp[k]).add((bool)needBuild[k]).add(m->prop.p).add(m->useCluster).add(m->ctaPerSM);
      key.add(m->usePropagator).add(m->precision);
      add_prop_key(key, rowArgs(m, k, m->chooseR()));
    }
    for (size_t s = 0; s < plan.slots.size(); s++) {
      key.add(plan.slotForm[s]).add(plan.slots[s].size());
      for (size_t i : plan.slots[s]) key.add(jobs[i].k);
    }
    for (const RaggedLaunch& rl : raggedLaunches) key.add(rl.ke->fn).add(rl.grid).add(rl.block).add(rl.smem);
    for (const PropArgs& a : items) add_prop_key(key, a);
    // a plan is captured the second time it comes (a one-off plan runs directly), then replayed
    bool replayed = false;
    if (!g_ragged.t0) ck(cudaEventCreate(&g_ragged.t0), "ragged timing");
    if (!g_ragged.t1) ck(cudaEventCreate(&g_ragged.t1), "ragged timing");
    ck(cudaEventRecord(g_ragged.t0, origin), "ragged timing");
    if (useGraph && key.bytes == g_ragged.lastKey) {
      replayed = g_ragged.graphs.run(key, origin, record);
    } else {
      record();
    }
    ck(cudaEventRecord(g_ragged.t1, origin), "ragged timing");
    g_ragged.lastKey = key.bytes;
    ck(cudaStreamSynchronize(origin), "ragged batch");
    float gpuMs = 0;
    ck(cudaEventElapsedTime(&gpuMs, g_ragged.t0, g_ragged.t1), "ragged timing");
    // host-side state of what ran: the matrices built; one launch per propagation, build and ragged
    // launch (credited to the launch's largest medium)
    for (size_t k : fused) {
      Medium* m = ms[k];
      m->launches = 0;
      if (needBuild[k]) {
        m->propVersion = m->pumpVersion;
        if (replayed) m->propBuilds++;
        m->launches++;
      }
    }
    for (size_t i = 0; i < jobs.size(); i++)
      if (plan.form[i] != kOne) ms[jobs[i].k]->launches++;
    for (const RaggedLaunch& rl : raggedLaunches) ms[jobs[itemJob[rl.first]].k]->launches++;
    g_lastRagged = RaggedStats{plan.makespan, 0, 0, 0, 0, g_ragged.graphs.captures, g_ragged.graphs.replays,
                               budget, maxW16, (double)gpuMs};
    for (int f : plan.slotForm)
      (f == kW16 ? g_lastRagged.slotsW16 : f == kW8 ? g_lastRagged.slotsW8 : g_lastRagged.slotsC4)++;
    for (const RaggedLaunch& rl : raggedLaunches) g_lastRagged.raggedCTAs += rl.grid;
    for (size_t k : fused)
      std::memcpy(outputs[k], g_ragged.hout.p + outOff[k], (size_t)ms[k]->nSignal * ms[k]->N * sizeof(double2));
  });
}

nlm_status nlm_ragged_plan(size_t n_media, const unsigned* n_freqs, const unsigned* n_modes,
                           const unsigned* n_z_steps, const int* propagator, const int* launch_class,
                           const unsigned* forms, int cluster_sms, int w16_slots, int pool_sms, int pool_granularity,
                           double* makespan_us, int* form, int* slot, int* ragged_ctas, double* times_us) {
  return guarded([&] {
    if (n_media == 0 || !n_freqs || !n_modes || !n_z_steps || !propagator || !launch_class || !forms)
      throw std::invalid_argument("ragged plan: no media");
    if (cluster_sms < 0 || w16_slots < 0 || pool_sms < 1 || pool_granularity < 1)
      throw std::invalid_argument("ragged plan: invalid SM budgets");
    std::vector<Job> jobs;
    for (size_t k = 0; k < n_media; k++) {
      if (n_freqs[k] < 2) throw std::invalid_argument("ragged plan: a grid needs at least 2 points");
      Job j{k, launch_class[k], {-1, -1, -1, -1}};
      const double steps = (double)(n_z_steps[k] > 1 ? n_z_steps[k] - 1 : 1);
      for (int c = 0; c < kForms; c++) {
        if (!((forms[k] >> c) & 1u)) continue;
        const double t = step_us(c, n_freqs[k], n_modes[k], propagator[k] != 0);
        if (t >= 0) j.t[c] = t * steps;
      }
      if (j.best() < 0) throw std::invalid_argument("ragged plan: a medium has no form for its grid");
      if (times_us)
        for (int c = 0; c < kForms; c++) times_us[k * kForms + c] = j.t[c];
      jobs.push_back(j);
    }
    Plan plan;
    const bool fits = plan_set(jobs, cluster_sms, w16_slots, pool_sms, pool_granularity, &plan);
    if (makespan_us) *makespan_us = fits ? plan.makespan : -1.0;
    if (ragged_ctas) *ragged_ctas = plan.poolSMs;
    for (size_t k = 0; k < n_media; k++) {
      if (form) form[k] = plan.form[k];
      if (slot) slot[k] = -1;
    }
    if (slot)
      for (size_t q = 0; q < plan.slots.size(); q++)
        for (size_t i : plan.slots[q]) slot[i] = (int)q;
  });
}

nlm_status nlm_ragged_last_plan(double* makespan_estimate_us, int* slots_c4, int* slots_w8, int* slots_w16,
                                int* ragged_ctas, long* graph_captures, long* graph_replays, int* sm_budget,
                                int* w16_capacity, double* gpu_ms) {
  return guarded([&] {
    std::lock_guard<std::mutex> lock(g_ragged.mu);
    if (sm_budget) *sm_budget = g_lastRagged.budget;
    if (w16_capacity) *w16_capacity = g_lastRagged.w16Capacity;
    if (gpu_ms) *gpu_ms = g_lastRagged.gpuMs;
    if (makespan_estimate_us) *makespan_estimate_us = g_lastRagged.makespan;
    if (slots_c4) *slots_c4 = g_lastRagged.slotsC4;
    if (slots_w8) *slots_w8 = g_lastRagged.slotsW8;
    if (slots_w16) *slots_w16 = g_lastRagged.slotsW16;
    if (ragged_ctas) *ragged_ctas = g_lastRagged.raggedCTAs;
    if (graph_captures) *graph_captures = g_lastRagged.captures;
    if (graph_replays) *graph_replays = g_lastRagged.replays;
  });
}

}  // extern "C"
