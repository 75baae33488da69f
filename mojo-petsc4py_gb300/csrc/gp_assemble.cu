// Matrix assembly on the device: the pending entries of MatSetValues folded
// into CSR, CSR from a dense array, and the transpose pattern of a CSR matrix.
//
// The reference assembles in Python (python/mojopetsc4py/PETSc/Mat.py:383-413:
// a dict of rows of {col: value}, sorted and coalesced on demand; 682-746:
// the transpose by a counting sort, from_dense by a scan of the array).  Here
// each is a sort plus a few passes on the GPU.  The sorts are CUB's
// DeviceRadixSort (the header library shipped with the CUDA toolkit): an LSD
// radix sort, stable, so entries with equal keys keep their call order.
//
// Entry semantics follow Mat._setValue (Mat.py:434-439): for one (row, col),
// the entries in call order fold from 0.0 -- an INSERT sets the value, an ADD
// adds to it (value = value + v, rounded) -- so the result is bit-identical
// to the reference's dict.
#include <algorithm>
#include <string>
#include <vector>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "../../include/gpetsc.h"
#include "gp_internal.h"
#include "gp_handles.h"
#include "gp_spmv.cuh"

namespace gp {

namespace {

constexpr int kAsmBlock = 256;

int asm_grid(int64_t n) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + kAsmBlock - 1) / kAsmBlock,
                                                     (int64_t)num_sms() * 16));
}

int bits_for(unsigned long long maxkey) {
  int b = 1;
  while (b < 64 && (maxkey >> b)) b++;
  return b;
}

// A device buffer freed on scope exit (set-up paths; allocation failures are
// reported by the caller's GP_CUDA checks on the pointer).
template <typename T>
struct DBuf {
  T* p = nullptr;
  ~DBuf() {
    if (p) cudaFree(p);
  }
  cudaError_t alloc(size_t n) { return cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)); }
};

__global__ void k_coo_keys(int64_t ne, int64_t nrows, int64_t ncols,
                           const int64_t* __restrict__ rows, const int64_t* __restrict__ cols,
                           unsigned long long* __restrict__ keys, int* __restrict__ idx,
                           int* __restrict__ bad) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < ne;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = rows[e], c = cols[e];
    if (r < 0 || r >= nrows || c < 0 || c >= ncols) {
      atomicExch(bad, 1);
      keys[e] = 0ull;
    } else {
      keys[e] = (unsigned long long)r * (unsigned long long)ncols + (unsigned long long)c;
    }
    idx[e] = (int)e;
  }
}

// head[k] = 1 where sorted entry k starts a new (row, col)
__global__ void k_heads(int64_t ne, const unsigned long long* __restrict__ keys,
                        int* __restrict__ head) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < ne;
       k += (int64_t)gridDim.x * blockDim.x)
    head[k] = (k == 0 || keys[k] != keys[k - 1]) ? 1 : 0;
}

// One thread per distinct (row, col): fold its entries in call order.
__global__ void k_fold(int64_t ne, int64_t ncols, const unsigned long long* __restrict__ keys,
                       const int* __restrict__ idx, const int* __restrict__ head,
                       const int* __restrict__ slot, const double* __restrict__ vals,
                       const unsigned char* __restrict__ add, int* __restrict__ row_of,
                       int* __restrict__ colind, double* __restrict__ out) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < ne;
       k += (int64_t)gridDim.x * blockDim.x) {
    if (!head[k]) continue;
    const unsigned long long key = keys[k];
    double acc = 0.0;
    for (int64_t q = k; q < ne && keys[q] == key; q++) {
      const int e = idx[q];
      acc = add[e] ? __dadd_rn(acc, vals[e]) : vals[e];
    }
    const int s = slot[k];
    row_of[s] = (int)(key / (unsigned long long)ncols);
    colind[s] = (int)(key % (unsigned long long)ncols);
    out[s] = acc;
  }
}

// rowptr from the sorted row of each slot: rowptr[r] = first slot of a row >= r.
__global__ void k_rowptr(int64_t nnz, int nrows, const int* __restrict__ row_of,
                         int* __restrict__ rowptr) {
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s <= nnz;
       s += (int64_t)gridDim.x * blockDim.x) {
    const int lo = s == 0 ? 0 : row_of[s - 1] + 1;
    const int hi = s == nnz ? nrows : row_of[s];
    for (int r = lo; r <= hi; r++) rowptr[r] = (int)s;
  }
}

__global__ void k_iota(int64_t n, int* __restrict__ v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    v[i] = (int)i;
}

__global__ void k_row_of_slots(int n, const int* __restrict__ rowptr, int* __restrict__ row_of) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
    for (int j = rowptr[r]; j < rowptr[r + 1]; j++) row_of[j] = r;
}

__global__ void k_gather_i(int64_t n, const int* __restrict__ src, const int* __restrict__ a,
                           int* __restrict__ out) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x)
    out[k] = a[src[k]];
}

// Dense rows: nonzero counts (one warp a row), then the entries in order.
__global__ void k_dense_counts(int nrows, int ncols, const double* __restrict__ a,
                               int* __restrict__ cnt) {
  const int lane = threadIdx.x & 31;
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int r = w; r < nrows; r += nw) {
    int c = 0;
    for (int j = lane; j < ncols; j += 32) c += a[(size_t)r * ncols + j] != 0.0;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if (lane == 0) cnt[r] = c;
  }
}

__global__ void k_dense_fill(int nrows, int ncols, const double* __restrict__ a,
                             const int* __restrict__ rowptr, int* __restrict__ colind,
                             double* __restrict__ val) {
  const int lane = threadIdx.x & 31;
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int r = w; r < nrows; r += nw) {
    int base = rowptr[r];
    for (int j0 = 0; j0 < ncols; j0 += 32) {
      const int j = j0 + lane;
      const double v = j < ncols ? a[(size_t)r * ncols + j] : 0.0;
      const bool nz = j < ncols && v != 0.0;
      const unsigned m = __ballot_sync(0xffffffffu, nz);
      if (nz) {
        const int k = base + __popc(m & ((1u << lane) - 1u));
        colind[k] = j;
        val[k] = v;
      }
      base += __popc(m);
    }
  }
}

__global__ void k_widen(int64_t n, const int* __restrict__ a, int64_t* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = a[i];
}

// Copy the device CSR (int32 indices) to caller-owned host arrays (int64).
int csr_to_host(int nrows, int64_t nnz, const int* d_rowptr, const int* d_colind,
                const double* d_val, int64_t* indptr, int64_t* indices, double* values,
                cudaStream_t s) {
  DBuf<int64_t> w;
  GP_CUDA(w.alloc((size_t)std::max<int64_t>(nrows + 1, nnz)));
  k_widen<<<asm_grid(nrows + 1), kAsmBlock, 0, s>>>(nrows + 1, d_rowptr, w.p);
  GP_CUDA(cudaMemcpyAsync(indptr, w.p, (size_t)(nrows + 1) * sizeof(int64_t),
                          cudaMemcpyDeviceToHost, s));
  GP_CUDA(cudaStreamSynchronize(s));
  if (nnz) {
    k_widen<<<asm_grid(nnz), kAsmBlock, 0, s>>>(nnz, d_colind, w.p);
    GP_CUDA(cudaMemcpyAsync(indices, w.p, (size_t)nnz * sizeof(int64_t), cudaMemcpyDeviceToHost,
                            s));
    GP_CUDA(cudaMemcpyAsync(values, d_val, (size_t)nnz * sizeof(double), cudaMemcpyDeviceToHost,
                            s));
  }
  GP_CUDA(cudaStreamSynchronize(s));
  return GP_OK;
}

}  // namespace

int coo_assemble(int64_t nrows, int64_t ncols, int64_t ne, const int64_t* rows,
                 const int64_t* cols, const double* vals, const unsigned char* add,
                 int64_t* indptr, int64_t* indices, double* values, int64_t* nnz_out,
                 cudaStream_t s) {
  if (nrows < 0 || ncols < 0 || ne < 0 || nrows > INT32_MAX - 1 || ncols > INT32_MAX - 1 ||
      ne > INT32_MAX - 1) {
    set_error("gp_coo_assemble: sizes must be non-negative and fit 32-bit indices");
    return GP_ERR_ARG;
  }
  *nnz_out = 0;
  if (ne == 0) {
    for (int64_t r = 0; r <= nrows; r++) indptr[r] = 0;
    return GP_OK;
  }
  const size_t n = (size_t)ne;
  DBuf<int64_t> drows, dcols;
  DBuf<double> dvals, dout;
  DBuf<unsigned char> dadd;
  DBuf<unsigned long long> k0, k1;
  DBuf<int> i0, i1, head, slot, row_of, colind, rowptr, bad;
  GP_CUDA(drows.alloc(n));
  GP_CUDA(dcols.alloc(n));
  GP_CUDA(dvals.alloc(n));
  GP_CUDA(dadd.alloc(n));
  GP_CUDA(k0.alloc(n));
  GP_CUDA(k1.alloc(n));
  GP_CUDA(i0.alloc(n));
  GP_CUDA(i1.alloc(n));
  GP_CUDA(head.alloc(n));
  GP_CUDA(slot.alloc(n));
  GP_CUDA(bad.alloc(1));
  GP_CUDA(cudaMemcpyAsync(drows.p, rows, n * sizeof(int64_t), cudaMemcpyHostToDevice, s));
  GP_CUDA(cudaMemcpyAsync(dcols.p, cols, n * sizeof(int64_t), cudaMemcpyHostToDevice, s));
  GP_CUDA(cudaMemcpyAsync(dvals.p, vals, n * sizeof(double), cudaMemcpyHostToDevice, s));
  GP_CUDA(cudaMemcpyAsync(dadd.p, add, n, cudaMemcpyHostToDevice, s));
  GP_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), s));
  const int g = asm_grid(ne);
  k_coo_keys<<<g, kAsmBlock, 0, s>>>(ne, nrows, ncols, drows.p, dcols.p, k0.p, i0.p, bad.p);
  int hbad = 0;
  GP_CUDA(cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  GP_CUDA(cudaStreamSynchronize(s));
  if (hbad) {
    set_error("gp_coo_assemble: an entry's row or column is out of range");
    return GP_ERR_ARG;
  }
  const unsigned long long maxkey =
      (unsigned long long)std::max<int64_t>(nrows, 1) * (unsigned long long)std::max<int64_t>(ncols, 1);
  const int nbits = bits_for(maxkey);
  size_t tmp_bytes = 0;
  GP_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, k0.p, k1.p, i0.p, i1.p, ne, 0,
                                          nbits, s));
  DBuf<unsigned char> tmp;
  GP_CUDA(tmp.alloc(tmp_bytes));
  GP_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, tmp_bytes, k0.p, k1.p, i0.p, i1.p, ne, 0,
                                          nbits, s));
  k_heads<<<g, kAsmBlock, 0, s>>>(ne, k1.p, head.p);
  size_t scan_bytes = 0;
  GP_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, head.p, slot.p, ne, s));
  DBuf<unsigned char> tmp2;
  GP_CUDA(tmp2.alloc(scan_bytes));
  GP_CUDA(cub::DeviceScan::ExclusiveSum(tmp2.p, scan_bytes, head.p, slot.p, ne, s));
  int last_slot = 0, last_head = 0;
  GP_CUDA(cudaMemcpyAsync(&last_slot, slot.p + (ne - 1), sizeof(int), cudaMemcpyDeviceToHost, s));
  GP_CUDA(cudaMemcpyAsync(&last_head, head.p + (ne - 1), sizeof(int), cudaMemcpyDeviceToHost, s));
  GP_CUDA(cudaStreamSynchronize(s));
  const int64_t nnz = (int64_t)last_slot + last_head;
  GP_CUDA(row_of.alloc((size_t)nnz));
  GP_CUDA(colind.alloc((size_t)nnz));
  GP_CUDA(dout.alloc((size_t)nnz));
  GP_CUDA(rowptr.alloc((size_t)nrows + 1));
  k_fold<<<g, kAsmBlock, 0, s>>>(ne, ncols, k1.p, i1.p, head.p, slot.p, dvals.p, dadd.p,
                                 row_of.p, colind.p, dout.p);
  k_rowptr<<<asm_grid(nnz + 1), kAsmBlock, 0, s>>>(nnz, (int)nrows, row_of.p, rowptr.p);
  GP_CHECK_LAUNCH();
  GP_TRY(csr_to_host((int)nrows, nnz, rowptr.p, colind.p, dout.p, indptr, indices, values, s));
  *nnz_out = nnz;
  return GP_OK;
}

int dense_to_csr(int64_t nrows, int64_t ncols, const double* dense, int64_t capacity,
                 int64_t* indptr, int64_t* indices, double* values, int64_t* nnz_out,
                 cudaStream_t s) {
  if (nrows < 0 || ncols < 0 || nrows > INT32_MAX - 1 || ncols > INT32_MAX - 1) {
    set_error("gp_dense_to_csr: sizes must be non-negative and fit 32-bit indices");
    return GP_ERR_ARG;
  }
  *nnz_out = 0;
  const size_t total = (size_t)nrows * (size_t)ncols;
  if (nrows == 0) {
    indptr[0] = 0;
    return GP_OK;
  }
  DBuf<double> a, val;
  DBuf<int> cnt, rowptr, colind;
  GP_CUDA(a.alloc(total));
  GP_CUDA(cnt.alloc((size_t)nrows + 1));
  GP_CUDA(rowptr.alloc((size_t)nrows + 1));
  if (total)
    GP_CUDA(cudaMemcpyAsync(a.p, dense, total * sizeof(double), cudaMemcpyHostToDevice, s));
  GP_CUDA(cudaMemsetAsync(cnt.p, 0, ((size_t)nrows + 1) * sizeof(int), s));
  const int gw = (int)std::max<int64_t>(1, std::min<int64_t>((nrows * 32 + kAsmBlock - 1) / kAsmBlock,
                                                             (int64_t)num_sms() * 16));
  if (ncols) k_dense_counts<<<gw, kAsmBlock, 0, s>>>((int)nrows, (int)ncols, a.p, cnt.p);
  size_t scan_bytes = 0;
  GP_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, cnt.p, rowptr.p, nrows + 1, s));
  DBuf<unsigned char> tmp;
  GP_CUDA(tmp.alloc(scan_bytes));
  GP_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, scan_bytes, cnt.p, rowptr.p, nrows + 1, s));
  int hnnz = 0;
  GP_CUDA(cudaMemcpyAsync(&hnnz, rowptr.p + nrows, sizeof(int), cudaMemcpyDeviceToHost, s));
  GP_CUDA(cudaStreamSynchronize(s));
  *nnz_out = hnnz;
  if (hnnz > capacity) {
    set_error("gp_dense_to_csr: more nonzeros than the output capacity (see *nnz)");
    return GP_ERR_ARG;
  }
  GP_CUDA(colind.alloc((size_t)hnnz));
  GP_CUDA(val.alloc((size_t)hnnz));
  if (ncols)
    k_dense_fill<<<gw, kAsmBlock, 0, s>>>((int)nrows, (int)ncols, a.p, rowptr.p, colind.p, val.p);
  GP_CHECK_LAUNCH();
  return csr_to_host((int)nrows, hnnz, rowptr.p, colind.p, val.p, indptr, indices, values, s);
}

// A^T's pattern on the device: a stable sort of the column indices carrying
// the slot numbers (t_src), so each column's entries keep ascending rows.
int csr_build_transpose(Csr* A, cudaStream_t s) {
  if (A->t_rowptr) return GP_OK;
  const int n = A->n, m = A->ncols;
  const int64_t nnz = A->nnz;
  const size_t nz = (size_t)std::max<int64_t>(nnz, 1);
  GP_CUDA(cudaMalloc(&A->t_rowptr, ((size_t)m + 1) * sizeof(int)));
  GP_CUDA(cudaMalloc(&A->t_colind, nz * sizeof(int)));
  GP_CUDA(cudaMalloc(&A->t_src, nz * sizeof(int)));
  DBuf<int> keys, iota, row_of;
  GP_CUDA(keys.alloc(nz));
  GP_CUDA(iota.alloc(nz));
  GP_CUDA(row_of.alloc(nz));
  if (nnz) {
    const int g = asm_grid(nnz);
    k_iota<<<g, kAsmBlock, 0, s>>>(nnz, iota.p);
    const int nbits = bits_for((unsigned long long)std::max(m, 1));
    size_t tmp_bytes = 0;
    GP_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, A->colind, keys.p, iota.p,
                                            A->t_src, (int)nnz, 0, nbits, s));
    DBuf<unsigned char> tmp;
    GP_CUDA(tmp.alloc(tmp_bytes));
    GP_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, tmp_bytes, A->colind, keys.p, iota.p,
                                            A->t_src, (int)nnz, 0, nbits, s));
    k_row_of_slots<<<asm_grid(n), kAsmBlock, 0, s>>>(n, A->rowptr, row_of.p);
    k_gather_i<<<g, kAsmBlock, 0, s>>>(nnz, A->t_src, row_of.p, A->t_colind);
    k_rowptr<<<asm_grid(nnz + 1), kAsmBlock, 0, s>>>(nnz, m, keys.p, A->t_rowptr);
  } else {
    GP_CUDA(cudaMemsetAsync(A->t_rowptr, 0, ((size_t)m + 1) * sizeof(int), s));
  }
  GP_CHECK_LAUNCH();
  // the SpMV form of A^T, from its row lengths (the column counts of A)
  std::vector<int> trp((size_t)m + 1);
  GP_CUDA(cudaMemcpyAsync(trp.data(), A->t_rowptr, ((size_t)m + 1) * sizeof(int),
                          cudaMemcpyDeviceToHost, s));
  GP_CUDA(cudaStreamSynchronize(s));
  int64_t maxlen = 0;
  for (int c = 0; c < m; c++) maxlen = std::max<int64_t>(maxlen, trp[c + 1] - trp[c]);
  const double avg = m ? (double)nnz / m : 0.0;
  A->t_stream_rows = maxlen > kSpmvMaxRowLen || (double)maxlen > 8.0 * avg + 8.0;
  if (A->t_stream_rows) GP_TRY(long_rows_build(A->t_lr, m, trp.data(), s));
  return GP_OK;
}

int csr_get(const Csr* A, int64_t* indptr, int64_t* indices, double* values, cudaStream_t s) {
  return csr_to_host(A->n, A->nnz, A->rowptr, A->colind, A->val, indptr, indices, values, s);
}

}  // namespace gp

extern "C" {

int gp_coo_assemble(int64_t nrows, int64_t ncols, int64_t nentries, const int64_t* rows,
                    const int64_t* cols, const double* values, const uint8_t* add,
                    int64_t* indptr, int64_t* indices, double* out_values, int64_t* nnz,
                    void* stream) {
  if (!nnz || !indptr || (nentries > 0 && (!rows || !cols || !values || !add || !indices ||
                                           !out_values))) {
    gp::set_error("gp_coo_assemble: null argument");
    return GP_ERR_ARG;
  }
  try {
    return gp::coo_assemble(nrows, ncols, nentries, rows, cols, values, add, indptr, indices,
                            out_values, nnz, reinterpret_cast<cudaStream_t>(stream));
  } catch (const std::exception& e) {
    gp::set_error(std::string("internal error: ") + e.what());
    return GP_ERR_INTERNAL;
  }
}

int gp_dense_to_csr(int64_t nrows, int64_t ncols, const double* dense, int64_t capacity,
                    int64_t* indptr, int64_t* indices, double* values, int64_t* nnz,
                    void* stream) {
  if (!nnz || !indptr || (nrows > 0 && ncols > 0 && !dense) ||
      (capacity > 0 && (!indices || !values)) || capacity < 0) {
    gp::set_error("gp_dense_to_csr: null argument or negative capacity");
    return GP_ERR_ARG;
  }
  try {
    return gp::dense_to_csr(nrows, ncols, dense, capacity, indptr, indices, values, nnz,
                            reinterpret_cast<cudaStream_t>(stream));
  } catch (const std::exception& e) {
    gp::set_error(std::string("internal error: ") + e.what());
    return GP_ERR_INTERNAL;
  }
}

int gp_mat_get_csr(gp_mat A, int64_t* indptr, int64_t* indices, double* values, void* stream) {
  if (!A || !indptr || (A->A->nnz && (!indices || !values))) {
    gp::set_error("gp_mat_get_csr: null argument");
    return GP_ERR_ARG;
  }
  try {
    return gp::csr_get(A->A, indptr, indices, values, reinterpret_cast<cudaStream_t>(stream));
  } catch (const std::exception& e) {
    gp::set_error(std::string("internal error: ") + e.what());
    return GP_ERR_INTERNAL;
  }
}

}  // extern "C"
