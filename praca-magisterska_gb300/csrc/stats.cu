// stats.cu -- see stats.h.
#include "stats.h"

#include <atomic>
#include <mutex>
#include <vector>

#include "../../include/wmom.h"

namespace wmom {
namespace stats {
namespace {

struct Rec {
  int c;
  cudaEvent_t e0, e1;
  double work;
};

std::atomic<bool> g_timing{false};
std::atomic<long long> g_launches[kNumCls];
std::mutex g_mu;
std::vector<Rec> g_recs;
std::vector<cudaEvent_t> g_pool;
double g_ms[kNumCls];
double g_work[kNumCls];
long long g_timed[kNumCls];

cudaEvent_t get_event() {
  if (!g_pool.empty()) {
    cudaEvent_t e = g_pool.back();
    g_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// Moves finished records into the totals (caller holds g_mu).
void drain(bool wait) {
  std::vector<Rec> keep;
  for (Rec& r : g_recs) {
    if (wait) cudaEventSynchronize(r.e1);
    if (cudaEventQuery(r.e1) == cudaSuccess) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, r.e0, r.e1);
      g_ms[r.c] += ms;
      g_work[r.c] += r.work;
      g_timed[r.c] += 1;
      g_pool.push_back(r.e0);
      g_pool.push_back(r.e1);
    } else {
      keep.push_back(r);
    }
  }
  g_recs.swap(keep);
}

}  // namespace

bool timing_enabled() { return g_timing.load(std::memory_order_relaxed); }

void count(Cls c, int launches) { g_launches[c].fetch_add(launches, std::memory_order_relaxed); }

Scope::Scope(Cls c, cudaStream_t s, double work, int launches) : c_(c), s_(s), work_(work) {
  count(c, launches);
  if (timing_enabled()) {
    std::lock_guard<std::mutex> lk(g_mu);
    e0_ = get_event();
    cudaEventRecord(e0_, s_);
  }
}

Scope::~Scope() {
  if (!e0_) return;
  std::lock_guard<std::mutex> lk(g_mu);
  cudaEvent_t e1 = get_event();
  cudaEventRecord(e1, s_);
  g_recs.push_back(Rec{c_, e0_, e1, work_});
  if (g_recs.size() > 4096) drain(false);
}

}  // namespace stats
}  // namespace wmom

using namespace wmom::stats;

extern "C" {

void wmom_stats_enable(int on) { g_timing.store(on != 0); }

void wmom_stats_reset(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  drain(true);
  for (int i = 0; i < kNumCls; ++i) {
    g_launches[i].store(0);
    g_ms[i] = 0.0;
    g_work[i] = 0.0;
    g_timed[i] = 0;
  }
}

int wmom_stats_read(double* ms, long long* launches, long long* timed, double* work, int n) {
  std::lock_guard<std::mutex> lk(g_mu);
  drain(true);
  const int m = n < kNumCls ? n : kNumCls;
  for (int i = 0; i < m; ++i) {
    if (ms) ms[i] = g_ms[i];
    if (launches) launches[i] = g_launches[i].load();
    if (timed) timed[i] = g_timed[i];
    if (work) work[i] = g_work[i];
  }
  return kNumCls;
}

}  // extern "C"
