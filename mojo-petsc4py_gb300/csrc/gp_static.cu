// gp_vec_reduce_static: the vector reductions of gp_vec_reduce for callers
// that cannot let the library allocate device memory.
//
// The reduction's scratch -- one partial sum per CTA and value, plus the
// last-CTA ticket -- lives in a fixed file-scope __device__ area instead of
// the lazily cudaMalloc'd per-device scratch the other entry points share.
// Its address is looked up once per device with cudaGetSymbolAddress.  The
// result goes to a caller-owned device buffer and the call does not
// synchronise, so nothing is allocated, freed or copied to the host.
//
// Limits and rules (stated in include/gpetsc.h as well):
//  * n <= kStaticMaxN (2^31 - 1, the element range of the library's vectors);
//    larger n is rejected with GP_ERR_ARG;
//  * at most kStaticRedBlocks CTAs (partials: 2 x 1024 doubles = 16 KB);
//  * the ticket must be zero when a call starts: static storage starts at zero
//    and the last CTA of every call resets it;
//  * one scratch area per device: calls that overlap on a device (different
//    streams or host threads without ordering between them) race;
//  * the first call on a device performs the symbol lookup and must not be
//    made inside a stream capture.
#include <mutex>

#include <exception>
#include <string>

#include "../../include/gpetsc.h"
#include "gp_internal.h"

namespace gp {

constexpr int kStaticRedBlocks = 1024;
constexpr int64_t kStaticMaxN = 2147483647;
constexpr int kStaticMaxDevices = 64;

static __device__ __align__(256) double g_static_partials[2 * kStaticRedBlocks];
static __device__ __align__(256) unsigned g_static_ticket;

struct StaticScratch {
  double* partials = nullptr;
  unsigned* ticket = nullptr;
};

static std::mutex g_static_mu;
static StaticScratch g_static[kStaticMaxDevices];

static int static_scratch(StaticScratch* out) {
  int dev = 0;
  GP_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kStaticMaxDevices) {
    set_error("gp_vec_reduce_static: device ordinal out of range");
    return GP_ERR_ARG;
  }
  std::lock_guard<std::mutex> lock(g_static_mu);
  StaticScratch& sc = g_static[dev];
  if (!sc.partials) {
    void* p = nullptr;
    void* t = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_static_partials);
    if (e == cudaSuccess) e = cudaGetSymbolAddress(&t, g_static_ticket);
    if (e != cudaSuccess) {
      cudaGetLastError();
      set_error(std::string("gp_vec_reduce_static: cudaGetSymbolAddress: ") +
                cudaGetErrorString(e));
      return GP_ERR_CUDA;
    }
    sc.partials = static_cast<double*>(p);
    sc.ticket = static_cast<unsigned*>(t);
  }
  *out = sc;
  return GP_OK;
}

static int vec_reduce_static(int op, int64_t n, const double* x, const double* y,
                             double* out, cudaStream_t stream) {
  {
    if (op < RED_DOT || op > RED_NORMINF) {
      set_error("gp_vec_reduce_static: op must be 0..5");
      return GP_ERR_ARG;
    }
    if (n < 0 || n > kStaticMaxN) {
      set_error("gp_vec_reduce_static: n must be in [0, 2^31 - 1]");
      return GP_ERR_ARG;
    }
    if (!out || (n > 0 && !x) || (n > 0 && (op == RED_DOT || op == RED_DOTNORM2) && !y)) {
      set_error("gp_vec_reduce_static: null pointer");
      return GP_ERR_ARG;
    }
    StaticScratch sc;
    int st = static_scratch(&sc);
    if (st != GP_OK) return st;
    RedSlot slot{};
    slot.partials = sc.partials;
    slot.ticket = sc.ticket;
    slot.stride = kStaticRedBlocks;
    return vec_reduce_into(stream, op, n, x, y, slot, kStaticRedBlocks, out);
  }
}

}  // namespace gp

extern "C" int gp_vec_reduce_static(int op, int64_t n, const double* x, const double* y,
                                    double* out, void* stream) {
  try {
    return gp::vec_reduce_static(op, n, x, y, out, static_cast<cudaStream_t>(stream));
  } catch (const std::exception& e) {
    gp::set_error(std::string("gp_vec_reduce_static: ") + e.what());
    return GP_ERR_INTERNAL;
  }
}
