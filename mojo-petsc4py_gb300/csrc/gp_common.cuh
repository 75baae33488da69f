// Shared device/host infrastructure for the GB300 Krylov library.
//
// Conventions used across every translation unit:
//   * Row/column indices are int32 on the device; values are float64 (the
//     mixed-precision form adds float32 copies).  Sizes cross the C ABI as
//     int64 and are checked to fit int32.
//   * Every floating-point step that mirrors a reference loop is written with
//     explicit round-to-nearest intrinsics (__dmul_rn, __dadd_rn, ...), so no
//     multiply-add is contracted into an FMA and each element is computed by
//     the same sequence of rounded operations as the sequential CPU code.
//   * Reductions are deterministic: a fixed grid, a fixed per-thread stride,
//     a fixed shuffle/shared-memory tree, and a last-block-done final pass
//     over the per-block partials in index order.
//   * Every spin-wait carries an iteration budget; when it runs out the
//     kernel records an error code in device memory and moves on.
#pragma once

#include <cstdlib>
#include <string>

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <string>

namespace gp {

// ------------------------------------------------------------------ errors
enum Status : int {
  GP_OK = 0,
  GP_ERR_ARG = 1,        // bad argument (size, null, type)
  GP_ERR_CUDA = 2,       // a CUDA runtime call failed
  GP_ERR_TIMEOUT = 3,    // a device spin-wait ran out of budget
  GP_ERR_NOT_SETUP = 4,  // object used before set-up
  GP_ERR_UNSUPPORTED = 5,
  GP_ERR_NUMERIC = 6,    // zero pivot etc. reported by a set-up kernel
  GP_ERR_INTERNAL = 7,
};

void set_error(const std::string& msg);
const char* last_error();

#define GP_CUDA(call)                                                           \
  do {                                                                          \
    cudaError_t e_ = (call);                                                    \
    if (e_ != cudaSuccess) {                                                    \
      ::gp::set_error(std::string(#call) + ": " + cudaGetErrorString(e_) +      \
                      " (" __FILE__ ":" + std::to_string(__LINE__) + ")");      \
      return ::gp::GP_ERR_CUDA;                                                 \
    }                                                                           \
  } while (0)

#define GP_CHECK_LAUNCH()                                                       \
  do {                                                                          \
    cudaError_t e_ = cudaGetLastError();                                        \
    if (e_ != cudaSuccess) {                                                    \
      ::gp::set_error(std::string("kernel launch: ") + cudaGetErrorString(e_) + \
                      " (" __FILE__ ":" + std::to_string(__LINE__) + ")");      \
      return ::gp::GP_ERR_CUDA;                                                 \
    }                                                                           \
  } while (0)

#define GP_TRY(expr)                       \
  do {                                     \
    int s_ = (expr);                       \
    if (s_ != ::gp::GP_OK) return s_;      \
  } while (0)

// ------------------------------------------------------------------ device
constexpr int kBlock = 256;        // default block for streaming kernels
constexpr int kRedBlock = 256;     // block for reductions
constexpr int kMaxRedGrid = 2048;  // partials buffer size per reduction slot

int num_sms();  // cached SM count of the current device
// A process-wide unique, increasing id (never 0): cached graphs key on the ids
// of the objects they were captured from, never on host addresses, which the
// allocator hands out again after a free.
unsigned long long next_uid();

// Arithmetic of the bandwidth-bound kernels (SpMV, Vec maps, reductions,
// solver updates).  kExact: every `a*x + y` is a rounded multiply then a
// rounded add, the operation sequence of the sequential CPU loops, so SpMV
// and the maps are bit-identical to them.  kFma: `a*x + y` is one fused
// multiply-add; GB300 issues FP64 at 1/64 of FP32, and the unfused form makes
// SpMV FP64-issue-bound below the HBM roofline, while the fused form halves
// the FP64 instructions.  kOrdered: kExact, and every reduction of the
// Krylov drivers and the Vec API summed in the reference's own blocked order
// (gp_ordred.cuh) instead of a parallel tree -- slow, and bit-identical to
// the reference's sequential solves.  Default kFma; GPETSC_ARITHMETIC=exact
// or =ordered selects another at load, gp_set_arithmetic() at run time.
enum Arith : int { kExact = 0, kFma = 1, kOrdered = 2 };
int arith_mode();
void set_arith_mode(int mode);
int red_grid(int64_t n);  // deterministic reduction grid for length n

// Device error word written by kernels (spin timeouts, numeric failures).
struct DevErr {
  int code;
  int where;
};

// Bit pattern a "not yet computed" entry holds in the value-as-flag arrays of
// the sync-free triangular sweeps: a signalling NaN with a fixed payload.
// Arithmetic never produces a signalling NaN (results are quiet), so a stored
// result can never equal it.
constexpr unsigned long long kPending = 0x7FF4DEAD0BADF00DULL;

// Programmatic dependent launch.  A kernel launched with the programmatic
// stream-serialization attribute may be scheduled while its predecessor in
// the stream drains; pdl_wait() blocks (in hardware, no polling) until that
// predecessor has completed and its writes are visible, so it must come
// before the first access to anything the predecessor writes, and before the
// kernel can exit (a successor's wait covers only this grid).  pdl_trigger()
// lets this grid's own successor be scheduled once every CTA has issued it.
// Both are no-ops for a kernel launched without the attribute.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Launch with programmatic dependent launch allowed (the kernel calls
// pdl_wait() before touching its predecessor's output).  GPETSC_PDL=0 turns
// the attribute off: ordinary stream order, same kernels.
inline bool pdl_enabled() {
  static bool v = [] {
    const char* e = std::getenv("GPETSC_PDL");
    return !(e && std::string(e) == "0");
  }();
  return v;
}

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), int grid, int block, cudaStream_t s,
                              Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = pdl_enabled() ? 1 : 0;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

__device__ __forceinline__ double ld_relaxed(const double* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return __longlong_as_double((long long)v);
}

__device__ __forceinline__ unsigned long long ld_relaxed_bits(const double* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_relaxed(double* p, double v) {
  asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(__double_as_longlong(v))
               : "memory");
}

__device__ __forceinline__ int ld_acquire_i32(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release_i32(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// exact-rounded arithmetic helpers (no contraction)
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double div_(double a, double b) { return __ddiv_rn(a, b); }

// a * x + y in the selected arithmetic (see Arith)
template <bool FMA>
__device__ __forceinline__ double madd(double a, double x, double y) {
  if constexpr (FMA)
    return __fma_rn(a, x, y);
  else
    return __dadd_rn(__dmul_rn(a, x), y);
}

// Grid-stride element loop in passes of U elements per thread: load(u, i)
// stages a pass's loads in registers, then emit(u, i) computes and stores, so
// U independent loads of every operand are in flight before the first store
// (operands that may alias -- W and Z in CG -- are still read before the same
// element is written).  Each thread visits tid, tid + stride, ... in
// ascending order, exactly as the plain grid-stride loop does, so reductions
// fold in the same order.
constexpr int kVecBatch = 4;
template <int U, typename L, typename E>
__device__ __forceinline__ void grid_batched(int n, L&& load, E&& emit) {
  // 32-bit unsigned indices: i0 < n < 2^31 and U * stride < 2^31
  const unsigned st = gridDim.x * blockDim.x, un = (unsigned)n;
  for (unsigned i0 = blockIdx.x * blockDim.x + threadIdx.x; i0 < un; i0 += U * st) {
#pragma unroll
    for (int u = 0; u < U; u++) {
      const unsigned i = i0 + u * st;
      if (i < un) load(u, i);
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const unsigned i = i0 + u * st;
      if (i < un) emit(u, i);
    }
  }
}

// Ticket increment with acquire-release semantics at GPU scope: releases
// this thread's earlier writes (and, cumulatively, the CTA's writes ordered
// before it by a barrier) and acquires the writes released by earlier
// increments.  Replaces a full fence (costly across the two dies) plus a
// relaxed atomic.
__device__ __forceinline__ unsigned atomic_add_acq_rel(unsigned* p, unsigned v) {
  unsigned old;
  asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], %2;"
               : "=r"(old)
               : "l"(p), "r"(v)
               : "memory");
  return old;
}

// ------------------------------------------------------------------ reduction
// Deterministic block reduction of NR doubles (result valid in thread 0);
// blockDim.x a power of two in [32, kRedBlock].  FP64 issue is the scarce
// resource on this part (2 FP64 lanes per clock per SM), so the tree keeps
// whole warps busy at every level: the halves fold in shared memory
// (128 + 64 + 32 lanes for 256 values) and one warp finishes with five
// shuffles -- 12 FP64 warp instructions per value instead of 45 for a
// per-warp shuffle tree.
template <int NR>
__device__ __forceinline__ void block_sum(double (&v)[NR]) {
  __shared__ double sh[NR][kRedBlock];
  const int t = threadIdx.x;
#pragma unroll
  for (int r = 0; r < NR; r++) sh[r][t] = v[r];
  __syncthreads();
  for (int h = blockDim.x >> 1; h >= 32; h >>= 1) {
    if (t < h) {
#pragma unroll
      for (int r = 0; r < NR; r++) sh[r][t] = add(sh[r][t], sh[r][t + h]);
    }
    __syncthreads();
  }
  if (t < 32) {
#pragma unroll
    for (int r = 0; r < NR; r++) {
      double x = sh[r][t];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x = add(x, __shfl_down_sync(0xffffffffu, x, o));
      v[r] = x;
    }
  }
  __syncthreads();
}

// Scratch for one deterministic multi-block reduction: per-block partials and
// the last-block-done ticket.
struct RedSlot {
  double* partials;    // [stride * NRmax]
  unsigned* ticket;    // one counter, returns to zero after every use
  int stride;          // >= gridDim.x of every kernel that uses the slot
};

// Every block writes its NR partial sums; the last block to arrive sums the
// partials in index order and returns true in all of its threads with the
// totals in `out` (valid in thread 0).  The ticket is reset for the next use.
template <int NR>
__device__ __forceinline__ bool grid_finish(double (&v)[NR], RedSlot slot, double (&out)[NR]) {
  __shared__ bool last;
  block_sum<NR>(v);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int r = 0; r < NR; r++) slot.partials[r * slot.stride + blockIdx.x] = v[r];
    last = atomic_add_acq_rel(slot.ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return false;
  // partials are read through L2 (ld.global.cg), several in flight per
  // thread; each thread still folds b = tid, tid + blockDim, ... in order
  double acc[NR];
#pragma unroll
  for (int r = 0; r < NR; r++) acc[r] = 0.0;
  constexpr int U = 8;
  const int nb = gridDim.x, bs = blockDim.x;
  for (int b0 = threadIdx.x; b0 < nb; b0 += U * bs) {
#pragma unroll
    for (int r = 0; r < NR; r++) {
      double t[U];
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int b = b0 + u * bs;
        t[u] = b < nb ? __ldcg(&slot.partials[r * slot.stride + b]) : 0.0;
      }
#pragma unroll
      for (int u = 0; u < U; u++)
        if (b0 + u * bs < nb) acc[r] = add(acc[r], t[u]);
    }
  }
  block_sum<NR>(acc);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int r = 0; r < NR; r++) out[r] = acc[r];
    *slot.ticket = 0u;
  }
  return true;
}

// A vector operand that is either a fixed device pointer or a device-resident
// pointer slot read at kernel start (solver loops keep "basis vector `it`" in
// such a slot, so one captured kernel serves every step).
struct DRef {
  double* p;
  double* const* ind;
  static DRef of(double* q) { return DRef{q, nullptr}; }
  static DRef of(const double* q) { return DRef{const_cast<double*>(q), nullptr}; }
  static DRef at(double* const* q) { return DRef{nullptr, q}; }
  __device__ __forceinline__ double* get() const {
    return ind ? *(double* const volatile*)ind : p;
  }
};

// Gate: kernels of a captured solver loop run only while the solver's state
// word equals the value they were captured for.
__device__ __forceinline__ bool gated_off(const int* gate, int want) {
  return gate != nullptr && *(volatile const int*)gate != want;
}

}  // namespace gp
