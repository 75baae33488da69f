// Device memory, page-locked host memory and copies for host programs with
// no CUDA binding of their own: the Python package's Vec and Mat classes keep
// their device copies in these blocks, so the drop-in needs nothing but this
// library.  Contracts are in include/gpetsc.h.
//
// Device blocks come from one stream-ordered pool per device, created by the
// library and kept for the life of the process (release threshold unlimited):
// freeing a vector and creating another of the same size reuses the block
// without a device synchronisation, as a caching allocator does.  Page-locked
// host blocks are recycled by size class (64 KiB granules) up to 4 GiB of
// cached blocks, since cudaMallocHost / cudaFreeHost synchronise the device.
#include <cstdint>
#include <map>
#include <mutex>
#include <unordered_map>

#include "../../include/gpetsc.h"
#include "gp_internal.h"

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_pool_mu;
cudaMemPool_t g_pool[kMaxDevices] = {};

int device_pool(cudaMemPool_t* out) {
  int dev = 0;
  GP_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    gp::set_error("gp_device_alloc: device ordinal out of range");
    return gp::GP_ERR_CUDA;
  }
  std::lock_guard<std::mutex> lk(g_pool_mu);
  if (!g_pool[dev]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool = nullptr;
    GP_CUDA(cudaMemPoolCreate(&pool, &props));
    uint64_t keep = UINT64_MAX;
    GP_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    g_pool[dev] = pool;
  }
  *out = g_pool[dev];
  return gp::GP_OK;
}

constexpr size_t kHostGranule = size_t(64) << 10;
constexpr size_t kHostCacheCap = size_t(4) << 30;
std::mutex g_host_mu;
std::unordered_map<void*, size_t> g_host_live;  // block -> capacity in bytes
std::multimap<size_t, void*> g_host_idle;       // capacity -> cached block
size_t g_host_idle_bytes = 0;

cudaStream_t S(void* s) { return reinterpret_cast<cudaStream_t>(s); }

int bad(const char* msg) {
  gp::set_error(msg);
  return GP_ERR_ARG;
}

}  // namespace

extern "C" {

int gp_device_alloc(void** ptr, int64_t bytes, void* stream) {
  if (!ptr || bytes < 0) return bad("gp_device_alloc: null result pointer or negative size");
  *ptr = nullptr;
  if (!bytes) return GP_OK;
  cudaMemPool_t pool = nullptr;
  if (int st = device_pool(&pool)) return st;
  GP_CUDA(cudaMallocFromPoolAsync(ptr, (size_t)bytes, pool, S(stream)));
  return GP_OK;
}

int gp_device_free(void* ptr, void* stream) {
  if (!ptr) return GP_OK;
  GP_CUDA(cudaFreeAsync(ptr, S(stream)));
  return GP_OK;
}

int gp_host_alloc(void** ptr, int64_t bytes) {
  if (!ptr || bytes < 0) return bad("gp_host_alloc: null result pointer or negative size");
  *ptr = nullptr;
  if (!bytes) return GP_OK;
  const size_t cap = ((size_t)bytes + kHostGranule - 1) / kHostGranule * kHostGranule;
  {
    std::lock_guard<std::mutex> lk(g_host_mu);
    auto it = g_host_idle.find(cap);
    if (it != g_host_idle.end()) {
      *ptr = it->second;
      g_host_idle.erase(it);
      g_host_idle_bytes -= cap;
      g_host_live[*ptr] = cap;
      return GP_OK;
    }
  }
  void* p = nullptr;
  GP_CUDA(cudaMallocHost(&p, cap));
  std::lock_guard<std::mutex> lk(g_host_mu);
  g_host_live[p] = cap;
  *ptr = p;
  return GP_OK;
}

int gp_host_free(void* ptr) {
  if (!ptr) return GP_OK;
  size_t cap = 0;
  {
    std::lock_guard<std::mutex> lk(g_host_mu);
    auto it = g_host_live.find(ptr);
    if (it == g_host_live.end()) return bad("gp_host_free: not a block from gp_host_alloc");
    cap = it->second;
    g_host_live.erase(it);
    if (g_host_idle_bytes + cap <= kHostCacheCap) {
      g_host_idle.emplace(cap, ptr);
      g_host_idle_bytes += cap;
      return GP_OK;
    }
  }
  GP_CUDA(cudaFreeHost(ptr));
  return GP_OK;
}

int gp_copy(void* dst, const void* src, int64_t bytes, int sync, void* stream) {
  if (bytes < 0 || (bytes && (!dst || !src))) return bad("gp_copy: null pointer or negative size");
  if (bytes) GP_CUDA(cudaMemcpyAsync(dst, src, (size_t)bytes, cudaMemcpyDefault, S(stream)));
  if (sync) GP_CUDA(cudaStreamSynchronize(S(stream)));
  return GP_OK;
}

int gp_stream_synchronize(void* stream) {
  GP_CUDA(cudaStreamSynchronize(S(stream)));
  return GP_OK;
}

}  // extern "C"
