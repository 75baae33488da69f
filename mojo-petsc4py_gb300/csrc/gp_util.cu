// Library-wide utilities: error text, device properties, standalone scratch.
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <string>
#include <unordered_map>

#include "gp_internal.h"

namespace gp {

static thread_local std::string g_err;

void set_error(const std::string& msg) { g_err = msg; }
const char* last_error() { return g_err.c_str(); }

static int g_arith = -1;

int arith_mode() {
  if (g_arith < 0) {
    const char* e = std::getenv("GPETSC_ARITHMETIC");
    const std::string v = e ? e : "";
    g_arith = v == "exact" ? kExact : v == "ordered" ? kOrdered : kFma;
  }
  return g_arith;
}

void set_arith_mode(int mode) { g_arith = mode == kOrdered ? kOrdered : mode ? kFma : kExact; }

unsigned long long next_uid() {
  static std::atomic<unsigned long long> next{1};
  return next.fetch_add(1, std::memory_order_relaxed);
}

int num_sms() {
  static int cached[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 132;
  if (!cached[dev]) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0)
      v = 132;
    cached[dev] = v;
  }
  return cached[dev];
}

// Reduction grid: enough resident blocks to stream at full bandwidth, never
// more than the partials buffer holds, never more blocks than needed.  The
// value depends only on n and the device, so a reduction is reproducible.
int red_grid(int64_t n) {
  int64_t want = (n + kRedBlock - 1) / kRedBlock;
  int64_t cap = (int64_t)num_sms() * 4;
  if (cap > kMaxRedGrid) cap = kMaxRedGrid;
  if (want > cap) want = cap;
  if (want < 1) want = 1;
  return (int)want;
}

// One scratch per (host thread, device): standalone Vec/Mat reductions run on
// the caller's stream and read their result back synchronously.
int scratch_get(Scratch** out, int64_t need_grid) {
  static thread_local std::unordered_map<int, Scratch> pool;
  int dev = 0;
  GP_CUDA(cudaGetDevice(&dev));
  Scratch& sc = pool[dev];
  int stride = (int)std::max<int64_t>(kMaxRedGrid, need_grid);
  if (sc.device != dev || sc.stride < stride) {
    if (sc.slot.partials) cudaFree(sc.slot.partials);
    if (sc.slot.ticket) cudaFree(sc.slot.ticket);
    if (!sc.d_out) {
      GP_CUDA(cudaMalloc(&sc.d_out, 8 * sizeof(double)));
      GP_CUDA(cudaMallocHost(&sc.h_out, 8 * sizeof(double)));
      GP_CUDA(cudaMalloc(&sc.d_idx, 4 * sizeof(long long)));
      GP_CUDA(cudaMallocHost(&sc.h_idx, 4 * sizeof(long long)));
    }
    GP_CUDA(cudaMalloc(&sc.slot.partials, (size_t)stride * 4 * sizeof(double)));
    GP_CUDA(cudaMalloc(&sc.slot.ticket, sizeof(unsigned)));
    GP_CUDA(cudaMemset(sc.slot.ticket, 0, sizeof(unsigned)));
    sc.slot.stride = stride;
    sc.stride = stride;
    sc.device = dev;
  }
  *out = &sc;
  return GP_OK;
}

namespace {
struct SetupClock {
  bool on = std::getenv("GPETSC_SETUP_TIMING") != nullptr;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now(), last = t0;
  std::string log;
};
SetupClock& setup_clock() {
  static thread_local SetupClock c;
  return c;
}
}  // namespace

void setup_mark(const char* phase) {
  SetupClock& c = setup_clock();
  if (!c.on) return;
  const auto t = std::chrono::steady_clock::now();
  char buf[96];
  std::snprintf(buf, sizeof buf, " %s %.1f", phase,
                std::chrono::duration<double, std::milli>(t - c.last).count());
  c.log += buf;
  c.last = t;
}

void setup_report(const char* what) {
  SetupClock& c = setup_clock();
  if (!c.on) return;
  const auto t = std::chrono::steady_clock::now();
  std::fprintf(stderr, "gpetsc setup %s (ms):%s; total %.1f\n", what, c.log.c_str(),
               std::chrono::duration<double, std::milli>(t - c.t0).count());
  c.log.clear();
  c.t0 = c.last = t;
}

}  // namespace gp
