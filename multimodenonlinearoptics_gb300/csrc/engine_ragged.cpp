// engine_ragged.cpp -- nlm_ragged_batch: one persistent launch over a ragged set of media (different
// grids and step counts), with the costliest large-grid media as cluster propagations beside it.
#include "engine.h"

using nlm::guarded;
using nlm::Medium;

extern "C" {

// Workspace of the ragged launch (process-wide; the launch is serialised by the mutex).
struct RaggedWorkspace {
  std::mutex mu;
  nlm::DevBuf<double2> in, out;
  nlm::DevBuf<double2> cin, cout;   // inputs and outputs of the media run as cluster propagations
  nlm::DevBuf<nlm::PropArgs> items;
  nlm::PinnedBuf<double2> hin, hout;   // host staging of every medium's input and output
  nlm::PinnedBuf<nlm::PropArgs> hitems;
  nlm::DevBuf<unsigned long long> counter;
};
static RaggedWorkspace g_ragged;

nlm_status nlm_ragged_batch(nlm_medium* const* media, size_t n_media, const double* const* inputs, int in_time_domain,
                            double* const* outputs) {
  return guarded([&] {
    using namespace nlm;
    if (n_media == 0) return;
    std::vector<Medium*> ms(n_media);
    for (size_t k = 0; k < n_media; k++) {
      ms[k] = M(media[k]);
      if (ms[k]->isCascade) throw std::invalid_argument("ragged batches take single media");
      ms[k]->launches = 0;
    }
    // media without a ragged kernel (or with a grid it cannot take) run one launch each
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
    std::vector<cudaStream_t> clusterSync;   // streams holding the read-back of cluster propagations
    struct PendingCopy {
      double2* dst;
      const double2* src;
      size_t bytes;
      cudaStream_t st;
    };
    std::vector<PendingCopy> pendingD2H;
    auto flushD2H = [&] {
      for (const PendingCopy& c : pendingD2H)
        ck(cudaMemcpyAsync(c.dst, c.src, c.bytes, cudaMemcpyDeviceToHost, c.st), "ragged output");
      pendingD2H.clear();
    };
    {
      // room for every medium, so cluster propagations of different solver groups never share it
      size_t inAll = 0, outAll = 0;
      for (size_t k : fused) {
        inAll += ms[k]->N;
        outAll += (size_t)ms[k]->nSignal * ms[k]->N;
      }
      g_ragged.cin.reserve(inAll);
      g_ragged.cout.reserve(outAll);
      g_ragged.hin.reserve(inAll);
      g_ragged.hout.reserve(outAll);
    }
    // every input is staged in page-locked memory first, so no copy below waits on earlier work
    std::vector<size_t> hinOff(n_media, 0), houtOff(n_media, 0);
    {
      size_t io = 0, oo = 0;
      for (size_t k : fused) {
        hinOff[k] = io;
        houtOff[k] = oo;
        std::memcpy(g_ragged.hin.p + io, inputs[k], ms[k]->N * sizeof(double2));
        io += ms[k]->N;
        oo += (size_t)ms[k]->nSignal * ms[k]->N;
      }
    }
    size_t cio = 0, coo = 0;
    // one launch per solver present in the set
    std::map<int, std::vector<size_t>> bySolver;
    for (size_t k : fused) bySolver[ms[k]->solver].push_back(k);
    for (auto& kv : bySolver) {
      std::vector<size_t>& ks = kv.second;
      for (size_t k : ks) ms[k]->ensureDevice();
      // largest first (cost ~ nZSteps * modes * N log N)
      std::sort(ks.begin(), ks.end(), [&](size_t x, size_t y) {
        auto cost = [&](Medium* m) { return (double)m->nZ * m->nSignal * m->N * std::log2((double)m->N); };
        return cost(ms[x]) > cost(ms[y]);
      });
      // The costliest media on grids of 1024+ points run as cluster-distributed propagations (4 SMs
      // each, on their own streams, concurrently with the ragged launch of the others) while the
      // clusters leave the ragged launch about one SM per two remaining media: it claims its media
      // largest first from a work counter, so the smallest ones queue behind the others.
      std::vector<size_t> clustered;
      std::vector<bool> wide(n_media, false);
      {
        const int sms = Medium::smCount();
        std::vector<size_t> others;
        for (size_t k : ks) {
          Medium* m = ms[k];
          const bool eligible = m->useCluster && is_pow2((int)m->N) && m->N >= 1024 && m->N <= (uint)kMaxFFT &&
                                m->findKernel(kKindCluster, m->solver, Medium::kClusterSize) != nullptr;
          const size_t rest = ks.size() - clustered.size() - 1;   // the ragged launch's media if this one joins
          if (eligible && (clustered.size() + 1) * Medium::kClusterSize + (rest + 1) / 2 <= (size_t)sms)
            clustered.push_back(k);
          else
            others.push_back(k);   // still largest first
        }
        ks.swap(others);
        // the costliest of them on 2048- and 4096-point grids take eight CTAs (one point per thread,
        // twice the SMs) while the SMs allow, largest first
        size_t used = clustered.size() * Medium::kClusterSize + (ks.size() + 1) / 2;
        for (size_t k : clustered) {
          Medium* m = ms[k];
          if (m->wideGrid() && m->findKernel(kKindCluster, m->solver + kSpreadWideKey, 1) &&
              used + (8 - Medium::kClusterSize) <= (size_t)sms) {
            wide[k] = true;
            used += 8 - Medium::kClusterSize;
          }
        }
      }
      if (!clustered.empty()) {
        // Each cluster propagation runs on its medium's own stream: input copy (page-locked source),
        // propagation, and -- after the ragged launch of the other media is queued, below -- the
        // read-back.  No stream waits on another: CUDA maps the streams onto a few hardware queues,
        // and a cross-stream wait at the head of one would hold back whatever shares its queue.
        size_t io = cio, oo = coo;
        for (size_t k : clustered) {
          Medium* m = ms[k];
          ck(cudaMemcpyAsync(g_ragged.cin.p + io, g_ragged.hin.p + hinOff[k], m->N * sizeof(double2),
                             cudaMemcpyHostToDevice, m->stream),
             "ragged input");
          PropArgs a = m->baseArgs(m->chooseR());
          a.inKind = 1;
          a.inTime = in_time_domain ? 1 : 0;
          a.in = g_ragged.cin.p + io;
          a.inStride = (long long)m->N;
          a.inChannels = 1;
          a.inputMode = 0;
          a.nOut = (int)m->nSignal;
          for (int mm = 0; mm < (int)m->nSignal; mm++) a.outModes[mm] = mm;
          a.out = g_ragged.cout.p + oo;
          a.outStride = (long long)m->nSignal * m->N;
          m->raggedWide = wide[k];
          try {
            m->propagate(a, 1, m->raggedPropagator());
          } catch (...) {
            m->raggedWide = false;
            throw;
          }
          m->raggedWide = false;
          pendingD2H.push_back({g_ragged.hout.p + houtOff[k], g_ragged.cout.p + oo,
                                (size_t)m->nSignal * m->N * sizeof(double2), m->stream});
          clusterSync.push_back(m->stream);
          io += m->N;
          oo += (size_t)m->nSignal * m->N;
        }
        cio = io;
        coo = oo;
      }
      if (ks.empty()) {
        flushD2H();
        continue;
      }
      size_t inTot = 0, outTot = 0, maxN = 0;
      for (size_t k : ks) {
        inTot += ms[k]->N;
        outTot += (size_t)ms[k]->nSignal * ms[k]->N;
        maxN = std::max<size_t>(maxN, ms[k]->N);
      }
      Medium* lead = ms[ks[0]];
      cudaStream_t st = lead->stream;
      // pump-driven solvers: each medium's per-point RK4 matrices when Medium::raggedPropagator wants
      // them, built on the launch's stream just before it (each build is parallel over all steps and
      // points of its medium); the media run as cluster propagations build theirs on their own streams
      std::vector<bool> withProp(n_media, false);
      for (size_t k : ks) {
        Medium* m = ms[k];
        if (m->raggedPropagator()) {
          m->buildPropagator(8, st);
          withProp[k] = true;
        }
      }
      // N/4 threads per medium when the largest grid allows it (four warps from N = 512), else N/8
      const KernelEntry* k4 = maxN / 4 <= 512 ? lead->findKernel(kKindRagged, kv.first, 4) : nullptr;
      const KernelEntry* ke = k4 ? k4 : lead->findKernel(kKindRagged, kv.first, 8);
      const int Rg = ke->R;
      g_ragged.in.reserve(inTot);
      g_ragged.out.reserve(outTot);
      g_ragged.items.reserve(ks.size());
      g_ragged.counter.reserve(1);
      std::vector<PropArgs> items(ks.size());
      std::vector<size_t> outOff(ks.size());
      size_t io = 0, oo = 0;
      for (size_t q = 0; q < ks.size(); q++) {
        Medium* m = ms[ks[q]];
        ck(cudaMemcpyAsync(g_ragged.in.p + io, g_ragged.hin.p + hinOff[ks[q]], m->N * sizeof(double2),
                           cudaMemcpyHostToDevice, st),
           "ragged input");
        PropArgs a = m->baseArgs(Rg);
        a.nInst = 1;
        a.ipc = 1;
        a.inKind = 1;
        a.inTime = in_time_domain ? 1 : 0;
        a.in = g_ragged.in.p + io;
        a.inStride = (long long)m->N;
        a.inChannels = 1;
        a.inputMode = 0;
        a.nOut = (int)m->nSignal;
        for (int mm = 0; mm < (int)m->nSignal; mm++) a.outModes[mm] = mm;
        a.out = g_ragged.out.p + oo;
        a.outStride = (long long)m->nSignal * m->N;
        a.prop = withProp[ks[q]] ? m->prop.p : nullptr;
        items[q] = a;
        outOff[q] = oo;
        io += m->N;
        oo += (size_t)m->nSignal * m->N;
      }
      g_ragged.hitems.reserve(items.size());
      std::memcpy(g_ragged.hitems.p, items.data(), items.size() * sizeof(PropArgs));
      ck(cudaMemcpyAsync(g_ragged.items.p, g_ragged.hitems.p, items.size() * sizeof(PropArgs), cudaMemcpyHostToDevice,
                         st),
         "ragged items");
      ck(cudaMemsetAsync(g_ragged.counter.p, 0, sizeof(unsigned long long), st), "ragged counter");
      int block = (int)((maxN / Rg + 31) / 32 * 32);
      int dev = 0, sms = 1;
      ck(cudaGetDevice(&dev), "device");
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      // One CTA per SM: every medium is a sequential march bound by its SM's FP64 units, so a second
      // resident CTA (of this launch or of a cluster propagation running beside it) would only halve
      // both.  Asking for more than half of the SM's shared memory keeps the others off.
      size_t smem = 0;
      cudaFuncAttributes fa;
      ck(exclusive_smem(ke->fn, maxN * sizeof(double2), &smem, &fa), "smem attribute");
      if (smem == 0) throw Unsupported("ragged kernel does not fit on an SM");
      if (block > fa.maxThreadsPerBlock) throw Unsupported("ragged kernel cannot launch that many threads");
      int active = 0;
      ck(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&active, ke->fn, block, smem), "occupancy");
      if (active < 1) throw Unsupported("ragged kernel does not fit on an SM");
      const int nItems = (int)ks.size();
      // launched as clusters of four CTAs (each CTA still runs its own media): the hardware places a
      // cluster on four SMs of one GPC, so the ragged CTAs take whole groups of four SMs and do not
      // break up the groups that the cluster propagations launched beside them need
      const int grid = (std::min(nItems, sms * active) + Medium::kClusterSize - 1) / Medium::kClusterSize *
                       Medium::kClusterSize;
      PropArgs* itemsD = g_ragged.items.p;
      unsigned long long* ctr = g_ragged.counter.p;
      int nIt = nItems;
      void* args[] = {(void*)&itemsD, (void*)&nIt, (void*)&ctr};
      if (lead->timeKernels) {
        if (!lead->ev0) ck(cudaEventCreate(&lead->ev0), "event");
        if (!lead->ev1) ck(cudaEventCreate(&lead->ev1), "event");
        ck(cudaEventRecord(lead->ev0, st), "event");
      }
      ck(launch_clustered(ke->fn, grid, block, smem, st, Medium::kClusterSize, args), "ragged launch");
      lead->launches++;
      if (lead->timeKernels) {
        ck(cudaEventRecord(lead->ev1, st), "event");
        ck(cudaEventSynchronize(lead->ev1), "event");
        float ms_ = 0;
        ck(cudaEventElapsedTime(&ms_, lead->ev0, lead->ev1), "event");
        lead->kernelMs += ms_;
        lead->kernelCount++;
      }
      flushD2H();   // the cluster propagations' outputs (the ragged launch is queued by now)
      for (size_t q = 0; q < ks.size(); q++) {
        Medium* m = ms[ks[q]];
        ck(cudaMemcpyAsync(g_ragged.hout.p + houtOff[ks[q]], g_ragged.out.p + outOff[q],
                           (size_t)m->nSignal * m->N * sizeof(double2), cudaMemcpyDeviceToHost, st),
           "ragged output");
      }
      ck(cudaStreamSynchronize(st), "ragged batch");
    }
    for (cudaStream_t st : clusterSync) ck(cudaStreamSynchronize(st), "ragged batch (clusters)");
    for (size_t k : fused)
      std::memcpy(outputs[k], g_ragged.hout.p + houtOff[k], (size_t)ms[k]->nSignal * ms[k]->N * sizeof(double2));
  });
}

}  // extern "C"
