// SeqAIJ (CSR) matrix on the device: creation from host arrays, SpMV,
// SpMV-add, SpMV-transpose and the diagonal.
//
//   MatMult_SeqAIJ           src/ported.mojo:380-391  -> k_spmv
//   MatMultAdd_SeqAIJ        src/ported.mojo:394-405  -> k_spmv (init = v_i)
//   MatMultTranspose_SeqAIJ  src/ported.mojo:408-431  -> k_spmv over A^T (spmv_t)
//   MatGetDiagonal_SeqAIJ    src/ported.mojo:434-447  -> k_diag
//
// The transpose is stored as a pattern (row pointers, the original row of each
// entry, and the slot in A it came from), built once on the host from the
// pattern with a stable counting sort.  Column c of A is then summed in
// ascending original-row order, which is the order the reference's scatter
// loop adds into y[c]: the gather is bit-identical to the scatter.  The values
// of A^T are gathered through the source slots into a copy once per change of
// A's values, so the multiply streams them like any CSR matrix.
#include <algorithm>
#include <climits>
#include <cstdlib>
#include <string>
#include <vector>

#include "gp_internal.h"
#include "gp_spmv.cuh"

namespace gp {

// L2 policy of the row-per-thread SpMV's matrix loads.  Marking the matrix
// evict-first pays when the vectors a Krylov iteration cycles through (five
// of n doubles) fit in L2 and the matrix does not: the vectors stay resident
// while the matrix streams (7-point 128^3 CG + Jacobi: 49.8 ms marked, 53.1
// unmarked, on GB300).  When everything fits, the mark would only evict the
// matrix first; when the vectors alone exceed L2, their normal-priority lines
// fill it and leave the marked stream the spare ways, so the lines the L1
// re-requests come back from DRAM (7-point 160^3 SpMV: 4.4 TB/s marked, 5.4
// unmarked).  GPETSC_SPMV_EVICT_FIRST=0/1 overrides the choice.
static int spmv_evict_first(int n, int64_t nnz) {
  const char* e = std::getenv("GPETSC_SPMV_EVICT_FIRST");
  if (e && *e) return std::atoi(e) != 0;
  int dev = 0, l2 = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev) != cudaSuccess || l2 <= 0) {
    cudaGetLastError();
    return 1;
  }
  const double vecs = 40.0 * n;
  const double mat = 12.0 * (double)nnz + 4.0 * ((double)n + 1);
  return mat + vecs > l2 && vecs <= l2;
}

template <typename T>
static int dev_upload(T** d, const T* h, size_t count, cudaStream_t s) {
  GP_CUDA(cudaMalloc(d, std::max<size_t>(count, 1) * sizeof(T)));
  if (count) GP_CUDA(cudaMemcpyAsync(*d, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
  return GP_OK;
}

static bool spmv_split_long_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("GPETSC_SPMV_SPLIT_LONG");
    return !(e && std::string(e) == "0");
  }();
  return on;
}

int long_rows_build(SpmvLongRows& L, int n, const int* h_rowptr, cudaStream_t s) {
  long_rows_free(L);
  if (!spmv_split_long_enabled()) return GP_OK;
  std::vector<int> rows, seg(1, 0), seg_long;
  int64_t short_max = 0, short_nnz = 0;
  for (int i = 0; i < n; i++) {
    const int len = h_rowptr[i + 1] - h_rowptr[i];
    if (len > kSpmvLongRow) {
      const int ns = (len + kSpmvLongSeg - 1) / kSpmvLongSeg;
      for (int q = 0; q < ns; q++) seg_long.push_back((int)rows.size());
      rows.push_back(i);
      seg.push_back(seg.back() + ns);
    } else {
      short_max = std::max<int64_t>(short_max, len);
      short_nnz += len;
    }
  }
  if (rows.empty()) return GP_OK;
  L.nlong = (int)rows.size();
  // with the long rows split off, the rest goes one row a thread when it
  // meets the row form's own bound (as csr_finish chooses the form)
  const int nshort = n - L.nlong;
  const double avg = nshort ? (double)short_nnz / nshort : 0.0;
  L.short_rows = short_max <= kSpmvMaxRowLen && (double)short_max <= 8.0 * avg + 8.0;
  L.nseg = seg.back();
  GP_TRY(dev_upload(&L.rows, rows.data(), rows.size(), s));
  GP_TRY(dev_upload(&L.seg, seg.data(), seg.size(), s));
  GP_TRY(dev_upload(&L.seg_long, seg_long.data(), seg_long.size(), s));
  GP_CUDA(cudaMalloc(&L.part, (size_t)L.nseg * sizeof(double)));
  GP_CUDA(cudaMalloc(&L.ticket, (size_t)L.nlong * sizeof(unsigned)));
  GP_CUDA(cudaMemsetAsync(L.ticket, 0, (size_t)L.nlong * sizeof(unsigned), s));
  GP_CUDA(cudaStreamSynchronize(s));  // the host lists go out of scope
  return GP_OK;
}

void long_rows_free(SpmvLongRows& L) {
  cudaFree(L.rows);
  cudaFree(L.seg);
  cudaFree(L.seg_long);
  cudaFree(L.part);
  cudaFree(L.ticket);
  L = SpmvLongRows();
}

static bool spmv_coff16_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("GPETSC_SPMV_COFF16");
    return !(e && std::string(e) == "0");
  }();
  return on;
}

static int csr_finish(Csr* A, const double* h_val, cudaStream_t s) {
  const int n = A->n;
  std::vector<int> diag(std::max(n, 1), -1);
  for (int i = 0; i < n; i++)
    for (int j = A->h_rowptr[i]; j < A->h_rowptr[i + 1]; j++)
      if (A->h_colind[j] == i) {
        diag[i] = j;
        break;
      }
  // rows of bounded length go one per thread; a matrix with long rows (or a
  // few rows far longer than the rest) uses the row-stream form
  int64_t maxlen = 0;
  for (int i = 0; i < n; i++)
    maxlen = std::max<int64_t>(maxlen, A->h_rowptr[i + 1] - A->h_rowptr[i]);
  const double avg = n ? (double)A->nnz / n : 0.0;
  A->stream_rows = maxlen > kSpmvMaxRowLen || (double)maxlen > 8.0 * avg + 8.0;
  A->l2_evict_first = spmv_evict_first(n, A->nnz);
  // 16-bit column offsets for the row form when every |col - row| fits
  // (banded and stencil operators); GPETSC_SPMV_COFF16=0 keeps 32-bit columns
  std::vector<short> coff;
  if (!A->stream_rows && A->nnz > 0 && spmv_coff16_enabled()) {
    bool fits = true;
    for (int i = 0; i < n && fits; i++)
      for (int j = A->h_rowptr[i]; j < A->h_rowptr[i + 1]; j++) {
        const int d = A->h_colind[j] - i;
        if (d < -32768 || d > 32767) {
          fits = false;
          break;
        }
      }
    if (fits) {
      coff.resize(A->nnz);
      for (int i = 0; i < n; i++)
        for (int j = A->h_rowptr[i]; j < A->h_rowptr[i + 1]; j++)
          coff[j] = (short)(A->h_colind[j] - i);
    }
  }
  GP_TRY(dev_upload(&A->rowptr, A->h_rowptr.data(), (size_t)n + 1, s));
  GP_TRY(dev_upload(&A->colind, A->h_colind.data(), (size_t)A->nnz, s));
  if (!coff.empty()) GP_TRY(dev_upload(&A->coff16, coff.data(), coff.size(), s));
  // row stream: rows longer than kSpmvLongRow slots are summed by segments in
  // the FMA arithmetic
  if (A->stream_rows) GP_TRY(long_rows_build(A->lr, n, A->h_rowptr.data(), s));
  GP_TRY(dev_upload(&A->val, h_val, (size_t)A->nnz, s));
  GP_TRY(dev_upload(&A->diagpos, diag.data(), (size_t)n, s));
  // the host staging vectors must stay alive until the copies land
  GP_CUDA(cudaStreamSynchronize(s));
  return GP_OK;
}

static int check_sizes(int64_t nrows, int64_t ncols, int64_t nnz) {
  if (nrows < 0 || ncols < 0 || nnz < 0 || nrows > INT32_MAX - 1 || ncols > INT32_MAX - 1 ||
      nnz > INT32_MAX - 1) {
    set_error("matrix sizes must be non-negative and fit 32-bit indices");
    return GP_ERR_ARG;
  }
  return GP_OK;
}

static int validate_pattern(const Csr* A) {
  if (A->h_rowptr[0] != 0 || A->h_rowptr[A->n] != A->nnz) {
    set_error("indptr must start at 0 and end at nnz");
    return GP_ERR_ARG;
  }
  for (int i = 0; i < A->n; i++) {
    if (A->h_rowptr[i + 1] < A->h_rowptr[i]) {
      set_error("indptr must be non-decreasing");
      return GP_ERR_ARG;
    }
    for (int j = A->h_rowptr[i]; j < A->h_rowptr[i + 1]; j++) {
      int c = A->h_colind[j];
      if (c < 0 || c >= A->ncols) {
        set_error("column index out of range in row " + std::to_string(i));
        return GP_ERR_ARG;
      }
    }
  }
  return GP_OK;
}

int csr_create(Csr** out, int64_t nrows, int64_t ncols, int64_t nnz, const int64_t* h_rowptr,
               const int64_t* h_colind, const double* h_val, cudaStream_t s) {
  GP_TRY(check_sizes(nrows, ncols, nnz));
  Csr* A = new Csr();
  A->n = (int)nrows;
  A->ncols = (int)ncols;
  A->nnz = nnz;
  A->h_rowptr.resize(nrows + 1);
  A->h_colind.resize(nnz);
  for (int64_t i = 0; i <= nrows; i++) A->h_rowptr[i] = (int)h_rowptr[i];
  for (int64_t j = 0; j < nnz; j++) A->h_colind[j] = (int)h_colind[j];
  int st = validate_pattern(A);
  if (st == GP_OK) st = csr_finish(A, h_val, s);
  if (st != GP_OK) {
    csr_destroy(A);
    return st;
  }
  GP_CUDA(cudaGetDevice(&A->device));
  A->uid = next_uid();
  *out = A;
  return GP_OK;
}

int csr_create_i32(Csr** out, int64_t nrows, int64_t ncols, int64_t nnz,
                   const int32_t* h_rowptr, const int32_t* h_colind, const double* h_val,
                   cudaStream_t s) {
  GP_TRY(check_sizes(nrows, ncols, nnz));
  Csr* A = new Csr();
  A->n = (int)nrows;
  A->ncols = (int)ncols;
  A->nnz = nnz;
  A->h_rowptr.assign(h_rowptr, h_rowptr + nrows + 1);
  A->h_colind.assign(h_colind, h_colind + nnz);
  int st = validate_pattern(A);
  if (st == GP_OK) st = csr_finish(A, h_val, s);
  if (st != GP_OK) {
    csr_destroy(A);
    return st;
  }
  GP_CUDA(cudaGetDevice(&A->device));
  A->uid = next_uid();
  *out = A;
  return GP_OK;
}

int csr_set_values(Csr* A, const double* val, int on_device, cudaStream_t s) {
  if (A->nnz == 0) return GP_OK;
  // the library's own values array (written in place through
  // gp_mat_values_ptr) needs no copy, only the caches below marked
  if (val != A->val)
    GP_CUDA(cudaMemcpyAsync(A->val, val, (size_t)A->nnz * sizeof(double),
                            on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
  A->val32_stale = true;  // converted again, in place, by the next csr_make_val32
  A->t_val_stale = true;  // gathered again by the next transpose multiply
  A->vver += 1;
  return GP_OK;
}

int csr_destroy(Csr* A) {
  if (!A) return GP_OK;
  cudaFree(A->rowptr);
  cudaFree(A->colind);
  cudaFree(A->coff16);
  long_rows_free(A->lr);
  long_rows_free(A->t_lr);
  cudaFree(A->val);
  cudaFree(A->val32);
  cudaFree(A->diagpos);
  cudaFree(A->t_rowptr);
  cudaFree(A->t_colind);
  cudaFree(A->t_src);
  cudaFree(A->t_val);
  delete A;
  return GP_OK;
}

// csr_build_transpose (the pattern of A^T) is in gp_assemble.cu.

// At.val[k] = A.val[t_src[k]]: the values of A^T in its row order.
__global__ void k_gather_values(int64_t nnz, const int* __restrict__ src,
                                const double* __restrict__ a, double* __restrict__ out) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnz;
       k += (int64_t)gridDim.x * blockDim.x)
    out[k] = a[src[k]];
}

// MatTranspose (python/mojopetsc4py/PETSc/Mat.py:555-563, 683-746): a new CSR
// holding A^T, built from the cached transpose pattern; values gathered on the
// device.  The pattern has no duplicates (A's has none), so no summing.
int csr_create_transpose(Csr* A, Csr** out, cudaStream_t s) {
  GP_TRY(csr_build_transpose(A, s));
  const int m = A->ncols;
  std::vector<int> trp(m + 1), tcol(std::max<int64_t>(A->nnz, 1));
  GP_CUDA(cudaMemcpy(trp.data(), A->t_rowptr, (m + 1) * sizeof(int), cudaMemcpyDeviceToHost));
  if (A->nnz)
    GP_CUDA(cudaMemcpy(tcol.data(), A->t_colind, A->nnz * sizeof(int), cudaMemcpyDeviceToHost));
  std::vector<double> zeros(std::max<int64_t>(A->nnz, 1), 0.0);
  Csr* T = nullptr;
  GP_TRY(csr_create_i32(&T, m, A->n, A->nnz, trp.data(), tcol.data(), zeros.data(), s));
  int st = csr_transpose_values(A, T, s);
  if (st != GP_OK) {
    csr_destroy(T);
    return st;
  }
  *out = T;
  return GP_OK;
}

// Refresh T = A^T's values after A's changed (same pattern).
int csr_transpose_values(Csr* A, Csr* T, cudaStream_t s) {
  GP_TRY(csr_build_transpose(A, s));
  if (T->n != A->ncols || T->ncols != A->n || T->nnz != A->nnz) {
    set_error("transpose: the target does not have the transposed shape");
    return GP_ERR_ARG;
  }
  if (A->nnz) {
    const int g = (int)std::min<int64_t>((A->nnz + 255) / 256, (int64_t)num_sms() * 8);
    k_gather_values<<<g, 256, 0, s>>>(A->nnz, A->t_src, A->val, T->val);
    GP_CHECK_LAUNCH();
  }
  T->val32_stale = true;
  T->t_val_stale = true;
  T->vver += 1;
  return GP_OK;
}

// out[k] = alpha * u[row(k)] * v[col(k)] over A's nonzeros: the gradient of a
// loss through A x = b with respect to the stored values (u = -lambda, v = x).
__global__ void k_outer_on_pattern(int n, const int* __restrict__ rowptr,
                                   const int* __restrict__ colind, const double* __restrict__ u,
                                   const double* __restrict__ v, double alpha,
                                   double* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double ui = mul(alpha, u[i]);
    for (int k = rowptr[i]; k < rowptr[i + 1]; k++) out[k] = mul(ui, v[colind[k]]);
  }
}

int csr_outer_on_pattern(const Csr* A, const double* u, const double* v, double alpha,
                         double* out, cudaStream_t s) {
  if (A->n == 0) return GP_OK;
  const int g = std::max(1, std::min((A->n + 255) / 256, num_sms() * 8));
  k_outer_on_pattern<<<g, 256, 0, s>>>(A->n, A->rowptr, A->colind, u, v, alpha, out);
  GP_CHECK_LAUNCH();
  return GP_OK;
}

__global__ void k_to_f32(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    b[i] = __double2float_rn(a[i]);
}

// FP32 copy of the values, kept at one address (captured solve graphs of the
// mixed form read it there) and converted again after every value change.
int csr_make_val32(Csr* A, cudaStream_t s) {
  if (A->val32 && !A->val32_stale) return GP_OK;
  if (!A->val32) GP_CUDA(cudaMalloc(&A->val32, std::max<int64_t>(A->nnz, 1) * sizeof(float)));
  A->val32_stale = false;
  if (A->nnz) {
    k_to_f32<<<num_sms() * 8, 256, 0, s>>>(A->nnz, A->val, A->val32);
    GP_CHECK_LAUNCH();
  }
  return GP_OK;
}

// ------------------------------------------------------------------ kernels

// y = A x, or y = v + A x when v is given (MatMultAdd starts each row's sum
// from v_i).  Optional gate for use inside captured solver loops.
template <bool FMA, bool STREAM, typename CT = int>
__global__ void __launch_bounds__(kSpmvRows) k_spmv(int n, const int* __restrict__ rowptr,
                                                    const CT* __restrict__ colind,
                                                    const double* __restrict__ val, DRef xr,
                                                    const double* __restrict__ v, DRef yr,
                                                    const int* gate, int want, int evict_first,
                                                    int long_min = INT_MAX) {
  if (gated_off(gate, want)) return;
  const double* __restrict__ x = xr.get();
  double* __restrict__ y = yr.get();
  const int r0 = blockIdx.x * kSpmvRows;
  const int row = r0 + threadIdx.x;
  double init = (v != nullptr && row < n) ? v[row] : 0.0;
  if constexpr (!STREAM) {
    if (row < n)
      y[row] = spmv_row<FMA>(row, rowptr, colind, val, x, init, spmv_policy(evict_first));
    return;
  }
  else {
  double s;
  bool skipped = false;
  if constexpr (FMA) {
    __shared__ SpmvSmemF<double, double, double> sm;
    s = spmv_block_rows_fma<double, double, double>(sm, n, r0, rowptr, colind, val, x, init,
                                                    long_min, &skipped);
  } else {
    __shared__ SpmvSmem<double, double, double> sm;
    s = spmv_block_rows<double, double, double>(sm, n, r0, rowptr, colind, val, x, init);
  }
  if (row < n && !skipped) y[row] = s;
  }
}

// The long rows of the FMA row stream, by segments: CTA s sums segment s of
// its row (kSpmvLongSeg slots: thread-strided FMAs, then a fixed tree), and
// the CTA that finishes a row's last segment adds the row's segment sums in
// segment order to its start value (v_i for MatMultAdd, else 0) and stores it.
// The sum's order is fixed, so results repeat run to run; it differs from one
// FMA chain by rounding only.  Called by every thread of the CTA.
__device__ __forceinline__ void spmv_long_segment(int s, const int* __restrict__ rowptr,
                                                  const int* __restrict__ colind,
                                                  const double* __restrict__ val,
                                                  const double* __restrict__ x,
                                                  const double* __restrict__ v,
                                                  double* __restrict__ y, const SpmvLongRows& L) {
  const int* __restrict__ long_rows = L.rows;
  const int* __restrict__ long_seg = L.seg;
  const int* __restrict__ seg_long = L.seg_long;
  double* seg_part = L.part;
  unsigned* ticket = L.ticket;
  __shared__ double red[kSpmvRows / 32];
  __shared__ bool last;
  const int li = seg_long[s];
  const int row = long_rows[li];
  const int b = rowptr[row] + (s - long_seg[li]) * kSpmvLongSeg;
  const int e = min(b + kSpmvLongSeg, rowptr[row + 1]);
  // a thread's slots j = b + tid + u * kSpmvRows: all loads first (the
  // gathers in flight together), then the FMAs in j order
  static_assert(kSpmvLongSeg % kSpmvRows == 0, "whole slots a thread");
  constexpr int kPer = kSpmvLongSeg / kSpmvRows;
  double vv[kPer], xv[kPer];
  int cc[kPer];
#pragma unroll
  for (int u = 0; u < kPer; u++) {
    const int j = b + threadIdx.x + u * kSpmvRows;
    if (j < e) {
      vv[u] = val[j];
      cc[u] = colind[j];
    }
  }
#pragma unroll
  for (int u = 0; u < kPer; u++)
    if (b + threadIdx.x + u * kSpmvRows < e) xv[u] = x[cc[u]];
  double acc = 0.0;
#pragma unroll
  for (int u = 0; u < kPer; u++)
    if (b + threadIdx.x + u * kSpmvRows < e) acc = __fma_rn(vv[u], xv[u], acc);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc = __dadd_rn(acc, __shfl_down_sync(0xffffffffu, acc, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = red[0];
    for (int w = 1; w < kSpmvRows / 32; w++) t = __dadd_rn(t, red[w]);
    seg_part[s] = t;
    __threadfence();
    const unsigned nseg = (unsigned)(long_seg[li + 1] - long_seg[li]);
    last = atomicAdd(&ticket[li], 1u) == nseg - 1;
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  double sum = v ? v[row] : 0.0;
  for (int q = long_seg[li]; q < long_seg[li + 1]; q++)
    sum = __dadd_rn(sum, *(volatile double*)&seg_part[q]);
  y[row] = sum;
  ticket[li] = 0u;
}

__global__ void __launch_bounds__(kSpmvRows) k_spmv_long(
    const int* __restrict__ rowptr, const int* __restrict__ colind, const double* __restrict__ val,
    DRef xr, const double* __restrict__ v, DRef yr, SpmvLongRows L, const int* gate, int want) {
  if (gated_off(gate, want)) return;
  spmv_long_segment(blockIdx.x, rowptr, colind, val, xr.get(), v, yr.get(), L);
}

// FMA arithmetic, long rows split off and the other rows short: one launch,
// the long rows' segments in CTAs [0, nseg) and the other rows one a thread
// (the row form's FMA chain, the same per row as the row stream's) in the
// CTAs after them, so the two run side by side.
__global__ void __launch_bounds__(kSpmvRows) k_spmv_split(
    int n, const int* __restrict__ rowptr, const int* __restrict__ colind,
    const double* __restrict__ val, DRef xr, const double* __restrict__ v, DRef yr,
    SpmvLongRows L, const int* gate, int want, int evict_first) {
  if (gated_off(gate, want)) return;
  const double* __restrict__ x = xr.get();
  double* __restrict__ y = yr.get();
  if ((int)blockIdx.x < L.nseg) {
    spmv_long_segment(blockIdx.x, rowptr, colind, val, x, v, y, L);
    return;
  }
  const int row = ((int)blockIdx.x - L.nseg) * kSpmvRows + (int)threadIdx.x;
  if (row >= n || rowptr[row + 1] - rowptr[row] > kSpmvLongRow) return;
  y[row] = spmv_row<true>(row, rowptr, colind, val, x, v ? v[row] : 0.0,
                          spmv_policy(evict_first));
}

static void launch_spmv(cudaStream_t s, const Csr* A, DRef x, const double* v, DRef y,
                        const int* gate, int want) {
  const bool f = arith_mode() == kFma;
  if (A->coff16) {  // row form with 16-bit column offsets
    auto k = f ? k_spmv<true, false, short> : k_spmv<false, false, short>;
    k<<<spmv_grid(A), kSpmvRows, 0, s>>>(A->n, A->rowptr, A->coff16, A->val, x, v, y, gate,
                                         want, A->l2_evict_first, INT_MAX);
    return;
  }
  auto k = A->stream_rows ? (f ? k_spmv<true, true> : k_spmv<false, true>)
                          : (f ? k_spmv<true, false> : k_spmv<false, false>);
  const bool split = f && A->lr.nlong > 0;
  if (split && A->lr.short_rows) {
    k_spmv_split<<<A->lr.nseg + spmv_grid(A), kSpmvRows, 0, s>>>(
        A->n, A->rowptr, A->colind, A->val, x, v, y, A->lr, gate, want, A->l2_evict_first);
    return;
  }
  k<<<spmv_grid(A), kSpmvRows, 0, s>>>(A->n, A->rowptr, A->colind, A->val, x, v, y, gate, want,
                                       A->l2_evict_first, split ? kSpmvLongRow : INT_MAX);
  if (split)
    k_spmv_long<<<A->lr.nseg, kSpmvRows, 0, s>>>(A->rowptr, A->colind, A->val, x, v, y, A->lr,
                                                gate, want);
}

__global__ void k_diag(int n, const int* __restrict__ diagpos, const double* __restrict__ val,
                       double* __restrict__ d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int p = diagpos[i];
  d[i] = p >= 0 ? val[p] : 0.0;
}

int spmv_grid(const Csr* A) { return (A->n + kSpmvRows - 1) / kSpmvRows; }

int spmv(cudaStream_t s, const Csr* A, DRef x, DRef y, const int* gate, int want) {
  if (A->n == 0) return GP_OK;
  launch_spmv(s, A, x, nullptr, y, gate, want);
  GP_CHECK_LAUNCH();
  return GP_OK;
}

int spmv_add(cudaStream_t s, const Csr* A, const double* x, const double* v, double* y) {
  if (A->n == 0) return GP_OK;
  launch_spmv(s, A, DRef::of(x), v, DRef::of(y), nullptr, 0);
  GP_CHECK_LAUNCH();
  return GP_OK;
}

// y = A^T x: the row kernels over A^T's pattern and a copy of its values
// (gathered once per value change through the source slots).  Each row of
// A^T folds its entries in ascending row order of A, the order in which
// MatMultTranspose_SeqAIJ (src/ported.mojo:408-431) accumulates y_c.
int spmv_t_prepare(cudaStream_t s, Csr* A) {
  GP_TRY(csr_build_transpose(A, s));
  if (A->ncols == 0) return GP_OK;
  if (!A->t_val) {
    GP_CUDA(cudaMalloc(&A->t_val, std::max<int64_t>(A->nnz, 1) * sizeof(double)));
    A->t_val_stale = true;
  }
  if (A->t_val_stale && A->nnz) {
    const int g = (int)std::min<int64_t>((A->nnz + kBlock - 1) / kBlock, 8LL * num_sms());
    k_gather_values<<<g, kBlock, 0, s>>>(A->nnz, A->t_src, A->val, A->t_val);
    GP_CHECK_LAUNCH();
  }
  A->t_val_stale = false;
  return GP_OK;
}

int spmv_t(cudaStream_t s, const Csr* A, DRef x, DRef y, const int* gate, int want) {
  if (A->ncols == 0) return GP_OK;
  const bool f = arith_mode() == kFma;
  auto k = A->t_stream_rows ? (f ? k_spmv<true, true> : k_spmv<false, true>)
                            : (f ? k_spmv<true, false> : k_spmv<false, false>);
  const bool split = f && A->t_lr.nlong > 0;
  if (split && A->t_lr.short_rows) {
    k_spmv_split<<<A->t_lr.nseg + (A->ncols + kSpmvRows - 1) / kSpmvRows, kSpmvRows, 0, s>>>(
        A->ncols, A->t_rowptr, A->t_colind, A->t_val, x, nullptr, y, A->t_lr, gate, want,
        A->l2_evict_first);
    GP_CHECK_LAUNCH();
    return GP_OK;
  }
  k<<<(A->ncols + kSpmvRows - 1) / kSpmvRows, kSpmvRows, 0, s>>>(
      A->ncols, A->t_rowptr, A->t_colind, A->t_val, x, nullptr, y, gate, want,
      A->l2_evict_first, split ? kSpmvLongRow : INT_MAX);
  if (split)
    k_spmv_long<<<A->t_lr.nseg, kSpmvRows, 0, s>>>(A->t_rowptr, A->t_colind, A->t_val, x,
                                                  nullptr, y, A->t_lr, gate, want);
  GP_CHECK_LAUNCH();
  return GP_OK;
}

int spmv_t(cudaStream_t s, Csr* A, const double* x, double* y) {
  GP_TRY(spmv_t_prepare(s, A));
  return spmv_t(s, A, DRef::of(x), DRef::of(y), nullptr, 0);
}

int mat_diagonal(cudaStream_t s, const Csr* A, double* d) {
  if (A->n == 0) return GP_OK;
  k_diag<<<(A->n + kBlock - 1) / kBlock, kBlock, 0, s>>>(A->n, A->diagpos, A->val, d);
  GP_CHECK_LAUNCH();
  return GP_OK;
}

}  // namespace gp
