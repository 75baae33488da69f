// Internal host API shared by the translation units of libgpetsc.so.  Not part
// of the public C ABI (that is include/gpetsc.h).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <exception>
#include <mutex>
#include <thread>
#include <vector>

#include "gp_common.cuh"

namespace gp {

// Phase times of a preconditioner set-up: setup_mark(name) records the time
// since the previous mark; setup_report() prints the phases to stderr and
// starts over.  Both do nothing unless GPETSC_SETUP_TIMING is set.
void setup_mark(const char* phase);
void setup_report(const char* what);

// Host-side parallel loop of the set-up phases: f(lo, hi) over contiguous
// ranges covering [0, n), on up to 16 host threads (the caller's included),
// one range for n below `grain`.  An exception thrown by a worker is rethrown
// on the caller after every thread has joined, where the C ABI's guard turns
// it into an error status.
template <class F>
void host_parallel_for(int64_t n, F f, int64_t grain = 1 << 15) {
  const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
  const int nt = (int)std::max<int64_t>(1, std::min<int64_t>({(int64_t)hw, 16, n / grain}));
  if (nt <= 1) {
    if (n > 0) f((int64_t)0, n);
    return;
  }
  std::exception_ptr failure;
  std::mutex mu;
  auto run = [&](int k) {
    try {
      f(n * k / nt, n * (k + 1) / nt);
    } catch (...) {
      std::lock_guard<std::mutex> g(mu);
      if (!failure) failure = std::current_exception();
    }
  };
  std::vector<std::thread> pool;
  int started = 1;
  try {
    pool.reserve(nt - 1);
    for (int k = 1; k < nt; k++, started++) pool.emplace_back(run, k);
  } catch (...) {
    // a thread that could not start: its range and the later ones run here
  }
  for (int k = started; k < nt; k++) run(k);
  run(0);
  for (auto& th : pool) th.join();
  if (failure) std::rethrow_exception(failure);
}

// Reduction scratch owned by the library for one stream user (standalone Vec
// and Mat calls).  Solvers carry their own.
struct Scratch {
  RedSlot slot{};
  double* d_out = nullptr;   // device result words
  double* h_out = nullptr;   // pinned host mirror
  long long* d_idx = nullptr;
  long long* h_idx = nullptr;
  int device = -1;
  int stride = 0;
};
int scratch_get(Scratch** out, int64_t n_needed_grid);

// ------------------------------------------------------------- Vec kernels
enum MapOp : int {
  OP_COPY, OP_SET, OP_SCALE, OP_SHIFT, OP_AXPY, OP_AYPX, OP_AXPBY, OP_AXPBYPCZ,
  OP_WAXPY, OP_PMULT, OP_PDIV, OP_PMIN, OP_PMAX, OP_PMAXABS, OP_RECIP, OP_EXP,
  OP_LOG, OP_SQRTABS, OP_ABS, OP_CHOP, OP_SWAP, OP_ZERO, OP_SCALESET, OP_DIVS
};
// Elementwise op over n entries.  Scalars alpha/beta/gamma are host values.
// Operand roles follow the reference kernels: see gp_vec.cu for each op.
int vec_map(cudaStream_t s, int op, int64_t n, double* y, const double* x,
            const double* w, double alpha, double beta, double gamma);
int vec_maxpy(cudaStream_t s, int64_t n, double* y, int nv, const double* alpha_host,
              const double* const* xs_host);

enum RedOp : int { RED_DOT, RED_NORM2SQ, RED_ASUM, RED_SUM, RED_DOTNORM2, RED_NORMINF };
// Reductions return their result(s) to host memory (synchronous).
int vec_reduce(cudaStream_t s, int op, int64_t n, const double* x, const double* y,
               double* out_host);
int vec_reduce_into(cudaStream_t s, int op, int64_t n, const double* x, const double* y,
                    RedSlot slot, int max_grid, double* out_dev);
int vec_minmax(cudaStream_t s, int64_t n, const double* x, int is_max, long long* idx,
               double* val);
int vec_max_pointwise_divide(cudaStream_t s, int64_t n, const double* x, const double* y,
                             double* out_host);

// Device-scalar forms used inside solvers (gate-aware, result stays on device).
struct DevReduceArgs {
  const int* gate;
  int want;
  RedSlot slot;
};

// ------------------------------------------------------------- CSR matrix
// Row-stream form, FMA arithmetic: rows longer than kSpmvLongRow slots are
// summed by segments of kSpmvLongSeg slots, one CTA a segment, instead of by
// one thread (rows ascending; row i's segments are seg[i] .. seg[i + 1] - 1;
// part holds the segment sums and ticket counts a row's finished segments).
// When the other rows meet the row-per-thread bound (short_rows), one launch
// runs the segments and those rows side by side (k_spmv_split); otherwise the
// row stream takes them and skips the long ones.
struct SpmvLongRows {
  int nlong = 0, nseg = 0;
  bool short_rows = false;    // the other rows fit the row-per-thread form
  int* rows = nullptr;
  int* seg = nullptr;
  int* seg_long = nullptr;    // [nseg] index into rows
  double* part = nullptr;     // [nseg]
  unsigned* ticket = nullptr;  // [nlong]
};
// Lists the long rows of a row pointer (host copy) on the device; nothing
// when none or GPETSC_SPMV_SPLIT_LONG=0.
int long_rows_build(SpmvLongRows& L, int n, const int* h_rowptr, cudaStream_t s);
void long_rows_free(SpmvLongRows& L);

struct Csr {
  int n = 0;        // rows
  int ncols = 0;
  int64_t nnz = 0;
  int* rowptr = nullptr;     // device, n+1
  int* colind = nullptr;     // device, nnz
  double* val = nullptr;     // device, nnz
  float* val32 = nullptr;    // device, nnz (mixed-precision copy, lazily made)
  bool val32_stale = false;  // values changed since val32 was converted
  int* diagpos = nullptr;    // device, n: slot of a_ii or -1
  bool stream_rows = false;  // SpMV form: false row per thread, true row stream
  int l2_evict_first = 1;    // row form: matrix loads marked L2 evict-first
  // row form: each slot's column as an offset from its row (col - row), when
  // every offset fits 16 bits; the row kernels then read 2 bytes an entry
  // instead of 4 (null: they read colind)
  short* coff16 = nullptr;
  SpmvLongRows lr;             // row stream: long rows of A
  SpmvLongRows t_lr;           // and of A^T (built with its pattern)
  // transpose (built on demand): rows of A^T in ascending original row order
  int* t_rowptr = nullptr;
  int* t_colind = nullptr;
  int* t_src = nullptr;      // slot in A of each A^T entry
  double* t_val = nullptr;   // A^T's values in its row order (lazily gathered)
  bool t_val_stale = true;   // values changed since t_val was gathered
  bool t_stream_rows = false;  // SpMV form of A^T (as stream_rows)
  // host pattern copy for set-up analysis
  std::vector<int> h_rowptr, h_colind;
  bool owns = true;
  int device = -1;
  unsigned long long uid = 0;   // next_uid() at creation
  unsigned long long vver = 0;  // bumped whenever the values change
};

int csr_create(Csr** out, int64_t nrows, int64_t ncols, int64_t nnz, const int64_t* h_rowptr,
               const int64_t* h_colind, const double* h_val, cudaStream_t s);
int csr_create_i32(Csr** out, int64_t nrows, int64_t ncols, int64_t nnz,
                   const int32_t* h_rowptr, const int32_t* h_colind, const double* h_val,
                   cudaStream_t s);
int csr_set_values(Csr* A, const double* val, int on_device, cudaStream_t s);
int csr_destroy(Csr* A);
int csr_create_transpose(Csr* A, Csr** out, cudaStream_t s);
int csr_transpose_values(Csr* A, Csr* T, cudaStream_t s);
int csr_outer_on_pattern(const Csr* A, const double* u, const double* v, double alpha,
                         double* out, cudaStream_t s);
int csr_build_transpose(Csr* A, cudaStream_t s);
int csr_make_val32(Csr* A, cudaStream_t s);

// y = A x (fp64); optional fused dot p.y into a device scalar with finisher
int spmv(cudaStream_t s, const Csr* A, DRef x, DRef y, const int* gate = nullptr, int want = 0);
int spmv_add(cudaStream_t s, const Csr* A, const double* x, const double* v, double* y);
int spmv_t(cudaStream_t s, Csr* A, const double* x, double* y);
// A^T's pattern and values brought up to date (host work and a gather; call
// before capturing a loop that multiplies by A^T), then the multiply alone.
int spmv_t_prepare(cudaStream_t s, Csr* A);
int spmv_t(cudaStream_t s, const Csr* A, DRef x, DRef y, const int* gate, int want);
int mat_diagonal(cudaStream_t s, const Csr* A, double* d);
int spmv_grid(const Csr* A);

}  // namespace gp
