// Launch counter and opt-in CUDA-event timing of kernel classes.
//
// Timing is per launch, on the stream the kernel is launched on, so a caller
// can time the dominant kernel inside a larger timed region (the bench's
// roofline figure) without a profiler.
#include "common.cuh"

#include <atomic>
#include <mutex>
#include <vector>

namespace mpdok {

static std::atomic<long long> g_launches{0};

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

struct ProfRec {
  cudaEvent_t a = nullptr, b = nullptr;
  int cls = 0;
  double work = 0.0;
  double bytes = 0.0;       // algorithmic bytes, where the class records flops in `work`
  bool closed = false;
  bool predicated = false;  // the launch read a device skip flag
};

static std::mutex g_pmu;
static bool g_prof_on = false;
static std::vector<ProfRec> g_recs;
static std::vector<cudaEvent_t> g_pool;
// Pinned copy of each predicated launch's skip flag, written on the stream
// right after the launch: a predicated-off launch returns at once, so counting
// its algorithmic work would overstate the achieved rate.
constexpr size_t PROF_MAX = 1u << 20;
static int* g_skiplog = nullptr;

static cudaEvent_t get_event() {
  if (!g_pool.empty()) {
    cudaEvent_t e = g_pool.back();
    g_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
  return e;
}

int prof_start(int cls, cudaStream_t s) {
  if (!g_prof_on) return -1;
  std::lock_guard<std::mutex> lk(g_pmu);
  if (g_recs.size() >= PROF_MAX) return -1;
  ProfRec r;
  r.cls = cls;
  r.a = get_event();
  r.b = get_event();
  if (!r.a || !r.b) return -1;
  cudaEventRecord(r.a, s);
  g_recs.push_back(r);
  return (int)g_recs.size() - 1;
}

void prof_stop_bytes(int slot, double bytes) {
  if (slot < 0) return;
  std::lock_guard<std::mutex> lk(g_pmu);
  if ((size_t)slot < g_recs.size()) g_recs[slot].bytes = bytes;
}

void prof_stop(int slot, cudaStream_t s, double work, const int* skip) {
  if (slot < 0) return;
  std::lock_guard<std::mutex> lk(g_pmu);
  if ((size_t)slot >= g_recs.size()) return;
  cudaEventRecord(g_recs[slot].b, s);
  g_recs[slot].work = work;
  g_recs[slot].closed = true;
  if (skip != nullptr) {
    if (!g_skiplog && cudaHostAlloc((void**)&g_skiplog, PROF_MAX * sizeof(int), cudaHostAllocDefault) != cudaSuccess) {
      g_skiplog = nullptr;
      return;
    }
    g_skiplog[slot] = 0;
    if (cudaMemcpyAsync(&g_skiplog[slot], skip, sizeof(int), cudaMemcpyDeviceToHost, s) == cudaSuccess)
      g_recs[slot].predicated = true;
  }
}

}  // namespace mpdok

using namespace mpdok;

extern "C" long long mpdok_launch_count(void) { return launch_count(); }

extern "C" int mpdok_profile_enable(int on) {
  std::lock_guard<std::mutex> lk(g_pmu);
  for (auto& r : g_recs) {
    if (r.a) g_pool.push_back(r.a);
    if (r.b) g_pool.push_back(r.b);
  }
  g_recs.clear();
  g_prof_on = on != 0;
  return MPDOK_OK;
}

// Totals over the launches of one class that did their work; launches that a
// device skip flag turned off are counted by mpdok_profile_skipped.
extern "C" int mpdok_profile_query(int cls, double* total_ms, long long* launches, double* work) {
  std::lock_guard<std::mutex> lk(g_pmu);
  double t = 0.0, w = 0.0;
  long long n = 0;
  for (size_t i = 0; i < g_recs.size(); ++i) {
    const ProfRec& r = g_recs[i];
    if (r.cls != cls || !r.closed) continue;
    float ms = 0.f;
    cudaError_t e = cudaEventElapsedTime(&ms, r.a, r.b);  // also orders the skip-flag copy before the read
    if (e != cudaSuccess) return cuda_status(e, "mpdok_profile_query");
    if (r.predicated && g_skiplog[i] != 0) continue;
    t += ms;
    w += r.work;
    ++n;
  }
  if (total_ms) *total_ms = t;
  if (launches) *launches = n;
  if (work) *work = w;
  return MPDOK_OK;
}

// Algorithmic bytes of one class (recorded where `work` counts flops).
extern "C" double mpdok_profile_bytes(int cls) {
  std::lock_guard<std::mutex> lk(g_pmu);
  double b = 0.0;
  for (size_t i = 0; i < g_recs.size(); ++i) {
    const ProfRec& r = g_recs[i];
    if (r.cls != cls || !r.closed) continue;
    if (r.predicated && g_skiplog[i] != 0) continue;
    b += r.bytes;
  }
  return b;
}

extern "C" long long mpdok_profile_skipped(int cls) {
  std::lock_guard<std::mutex> lk(g_pmu);
  long long n = 0;
  for (size_t i = 0; i < g_recs.size(); ++i) {
    const ProfRec& r = g_recs[i];
    if (r.cls != cls || !r.closed || !r.predicated) continue;
    if (cudaEventSynchronize(r.b) != cudaSuccess) return -1;
    if (g_skiplog[i] != 0) ++n;
  }
  return n;
}

// Timeline of the closed records in launch order: out[4 i .. 4 i + 3] =
// (class, start ms, end ms, work), the times relative to the first record's
// start.  Writes at most max_records records and returns how many there are.
extern "C" long long mpdok_profile_timeline(double* out, long long max_records) {
  std::lock_guard<std::mutex> lk(g_pmu);
  long long n = 0;
  cudaEvent_t t0 = nullptr;
  for (size_t i = 0; i < g_recs.size(); ++i) {
    const ProfRec& r = g_recs[i];
    if (!r.closed) continue;
    if (!t0) t0 = r.a;
    if (out && n < max_records) {
      float a = 0.f, b = 0.f;
      cudaError_t e = cudaEventElapsedTime(&a, t0, r.a);
      if (e == cudaSuccess) e = cudaEventElapsedTime(&b, t0, r.b);
      if (e != cudaSuccess) return cuda_status(e, "mpdok_profile_timeline");
      out[4 * n] = (double)r.cls;
      out[4 * n + 1] = (double)a;
      out[4 * n + 2] = (double)b;
      out[4 * n + 3] = r.work;
    }
    ++n;
  }
  return n;
}
