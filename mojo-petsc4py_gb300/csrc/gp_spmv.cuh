// CSR SpMV building blocks shared by the standalone multiply and the fused
// solver kernels.  Two forms, chosen per matrix (Csr::stream_rows), with
// bitwise-identical results: both fold each row from `init` in ascending slot
// order, one rounded product (or one FMA) per slot, as MatMult_SeqAIJ does
// (src/ported.mojo:380-391).
//
// Row per thread (spmv_row): rows of bounded length (stencils, FEM, graphs).
// Each thread loads its row's slots four at a time, then gathers x.  A warp's
// loads of a slot range are strided by the row length, but the 32 rows of a
// warp cover one contiguous span of the arrays, so L1 serves the re-touched
// lines and DRAM sees each byte once.  Matrix values and indices are read
// once per product; where the solver's vectors fit in the 129 MB L2 and the
// matrix does not, they are loaded with an L2 evict-first policy so the
// vectors stay resident while the matrix streams through (Csr::l2_evict_first).
//
// Row stream (spmv_block_rows*): rows of any length.  One CTA owns kSpmvRows
// consecutive rows.  The CTA walks the contiguous slot
// range of its rows in chunks: every thread loads values and column indices
// with unit stride (coalesced), forms value * x[col] into shared memory, and
// then each thread adds the products of its own row in ascending slot order.
// Each row is therefore summed exactly as MatMult_SeqAIJ sums it
// (src/ported.mojo:380-391): start at `init`, add one rounded product per slot
// in order -- bit-identical to the sequential loop -- while the memory traffic
// is fully coalesced apart from the x gather.
#pragma once

#include <climits>

#include "gp_common.cuh"

namespace gp {

constexpr int kSpmvRows = 256;    // rows per CTA == threads per CTA
constexpr int kSpmvChunk = 2048;  // products staged per pass
constexpr int kSpmvMaxRowLen = 64;  // longest row the row-per-thread form takes
constexpr int kSpmvLongRow = 2048;  // FMA row stream: longer rows go by segments
constexpr int kSpmvLongSeg = 2048;  // slots of one segment (one CTA)

// L2 evict-first loads for data read once per product.
__device__ __forceinline__ uint64_t l2_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t l2_evict_normal() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_normal.b64 %0, 1.0;" : "=l"(p));
  return p;
}
// The matrix stream's policy (Csr::l2_evict_first): evict-first keeps the
// vectors resident, normal lets the stream use L2 like any other data.
__device__ __forceinline__ uint64_t spmv_policy(int evict_first) {
  return evict_first ? l2_evict_first() : l2_evict_normal();
}
__device__ __forceinline__ double ld_stream(const double* a, uint64_t pol) {
  double v;
  asm volatile("ld.global.nc.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(a), "l"(pol));
  return v;
}
__device__ __forceinline__ float ld_stream(const float* a, uint64_t pol) {
  float v;
  asm volatile("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(a), "l"(pol));
  return v;
}
__device__ __forceinline__ int ld_stream(const int* a, uint64_t pol) {
  int v;
  asm volatile("ld.global.nc.L2::cache_hint.b32 %0, [%1], %2;" : "=r"(v) : "l"(a), "l"(pol));
  return v;
}
__device__ __forceinline__ short ld_stream(const short* a, uint64_t pol) {
  unsigned short v;
  asm volatile("ld.global.nc.L2::cache_hint.b16 %0, [%1], %2;" : "=h"(v) : "l"(a), "l"(pol));
  return (short)v;
}

// A slot's column in the row form: a 32-bit column index, or a 16-bit offset
// from the row (Csr::coff16).
__device__ __forceinline__ int spmv_col(const int* c, int j, int row, uint64_t pol) {
  (void)row;
  return ld_stream(c + j, pol);
}
__device__ __forceinline__ int spmv_col(const short* c, int j, int row, uint64_t pol) {
  return row + (int)ld_stream(c + j, pol);
}

// Row `row`'s sum, starting from `init` (caller checks row < n).  CT: int
// (column indices) or short (offsets from the row).  BOUND: each 4-slot
// batch issues only as many FMAs as the widest row of the warp still needs (a
// warp maximum a batch), so rows of 7 do not issue an eighth, predicated-off
// FP64 instruction; measured faster in the standalone multiply and slower in
// the fused CG pass, which keeps the plain form.
template <bool FMA, typename VT, typename XT, typename CT, bool BOUND = true>
__device__ __forceinline__ double spmv_row(int row, const int* __restrict__ rowptr,
                                           const CT* __restrict__ colind,
                                           const VT* __restrict__ val, const XT* __restrict__ x,
                                           double init, uint64_t pol) {
  const int b = rowptr[row], e = rowptr[row + 1];
  double acc = init;
  // four slots per batch: 32 registers, full occupancy (a GB300 scan of
  // 2/4/7/8-slot batches on the 7-point stencil put 4 first)
  for (int j0 = b; j0 < e; j0 += 4) {
    int cc[4];
    double vv[4];
#pragma unroll
    for (int u = 0; u < 4; u++)
      if (j0 + u < e) {
        cc[u] = spmv_col(colind, j0 + u, row, pol);
        vv[u] = (double)ld_stream(val + j0 + u, pol);
      }
    // the batch's widest row in the warp bounds the FMAs issued (uniform)
    const int wb = BOUND ? __reduce_max_sync(__activemask(), e - j0) : 4;
#pragma unroll
    for (int u = 0; u < 4; u++)
      if (u < wb && j0 + u < e) acc = madd<FMA>(vv[u], (double)x[cc[u]], acc);
  }
  return acc;
}

// A row's bounds and first batch of slots, loaded ahead of the x gather
// (spmv_row_preload), and the row's sum from there (spmv_row_from): the same
// loads and the same fold as spmv_row.
struct SpmvPre {
  int row, j, e;
  int cc[4];
  double vv[4];
};

template <typename VT, typename CT>
__device__ __forceinline__ void spmv_row_preload(int row, const int* __restrict__ rowptr,
                                                 const CT* __restrict__ colind,
                                                 const VT* __restrict__ val, uint64_t pol,
                                                 SpmvPre& pre) {
  pre.row = row;
  pre.j = rowptr[row];
  pre.e = rowptr[row + 1];
#pragma unroll
  for (int u = 0; u < 4; u++)
    if (pre.j + u < pre.e) {
      pre.cc[u] = spmv_col(colind, pre.j + u, row, pol);
      pre.vv[u] = (double)ld_stream(val + pre.j + u, pol);
    }
}

template <bool FMA, typename VT, typename XT, typename CT, bool BOUND = true>
__device__ __forceinline__ double spmv_row_from(const SpmvPre& pre,
                                                const CT* __restrict__ colind,
                                                const VT* __restrict__ val,
                                                const XT* __restrict__ x, double init,
                                                uint64_t pol) {
  double acc = init;
  const int b = pre.j, e = pre.e, row = pre.row;
  {
    const int wb = BOUND ? __reduce_max_sync(__activemask(), e - b) : 4;
#pragma unroll
    for (int u = 0; u < 4; u++)
      if (u < wb && b + u < e) acc = madd<FMA>(pre.vv[u], (double)x[pre.cc[u]], acc);
  }
  for (int j0 = b + 4; j0 < e; j0 += 4) {
    int cc[4];
    double vv[4];
#pragma unroll
    for (int u = 0; u < 4; u++)
      if (j0 + u < e) {
        cc[u] = spmv_col(colind, j0 + u, row, pol);
        vv[u] = (double)ld_stream(val + j0 + u, pol);
      }
    // the batch's widest row in the warp bounds the FMAs issued (uniform)
    const int wb = BOUND ? __reduce_max_sync(__activemask(), e - j0) : 4;
#pragma unroll
    for (int u = 0; u < 4; u++)
      if (u < wb && j0 + u < e) acc = madd<FMA>(vv[u], (double)x[cc[u]], acc);
  }
  return acc;
}

template <typename VT, typename XT, typename AT>
struct SpmvSmem {
  AT prod[kSpmvChunk];
  int rp[kSpmvRows + 1];
};

// Returns the row sum for row r0 + threadIdx.x (undefined for threads past
// the last row).  `init` is the starting value of that row's sum.  All threads
// of the CTA must call it.
template <typename VT, typename XT, typename AT>
__device__ __forceinline__ AT spmv_block_rows(SpmvSmem<VT, XT, AT>& sm, int n, int r0,
                                              const int* __restrict__ rowptr,
                                              const int* __restrict__ colind,
                                              const VT* __restrict__ val,
                                              const XT* __restrict__ x, AT init) {
  const int tid = threadIdx.x;
  const int nr = min(kSpmvRows, n - r0);
  for (int t = tid; t <= nr; t += blockDim.x) sm.rp[t] = rowptr[r0 + t];
  __syncthreads();
  const int base = sm.rp[0];
  const int end = sm.rp[nr];
  int my_b = 0, my_e = 0;
  if (tid < nr) {
    my_b = sm.rp[tid];
    my_e = sm.rp[tid + 1];
  }
  AT sum = init;
  for (int c0 = base; c0 < end; c0 += kSpmvChunk) {
    const int cn = min(kSpmvChunk, end - c0);
#pragma unroll 4
    for (int k = tid; k < cn; k += kSpmvRows) {
      const int slot = c0 + k;
      if constexpr (sizeof(AT) == 8) {
        sm.prod[k] = __dmul_rn((double)val[slot], (double)x[colind[slot]]);
      } else {
        sm.prod[k] = __fmul_rn((float)val[slot], (float)x[colind[slot]]);
      }
    }
    __syncthreads();
    const int lo = max(my_b, c0), hi = min(my_e, c0 + cn);
    for (int j = lo; j < hi; j++) {
      if constexpr (sizeof(AT) == 8)
        sum = __dadd_rn(sum, sm.prod[j - c0]);
      else
        sum = __fadd_rn(sum, sm.prod[j - c0]);
    }
    __syncthreads();
  }
  return sum;
}

// Fused-multiply-add form: the CTA stages each chunk's values and gathered x
// entries in shared memory (coalesced loads), then each thread folds its row
// with one FMA per slot in ascending slot order.  Half the FP64 instructions
// of the exact form, which matters on a part that issues FP64 at 1/64 of
// FP32.
constexpr int kSpmvChunkF = 1536;

template <typename VT, typename XT, typename AT>
struct SpmvSmemF {
  AT v[kSpmvChunkF];
  AT xv[kSpmvChunkF];
  int rp[kSpmvRows + 1];
  int nlong;                  // rows of this CTA longer than `long_min`
  int lb[kSpmvRows], le[kSpmvRows];  // their slot ranges, in row order
  int wcount[kSpmvRows / 32];
};

// Rows longer than `long_min` slots are left to the segmented kernel
// (k_spmv_long): their slots are not staged and their thread does not fold;
// *skipped tells the caller not to store the row.  long_min = INT_MAX keeps
// every row here.
template <typename VT, typename XT, typename AT>
__device__ __forceinline__ AT spmv_block_rows_fma(SpmvSmemF<VT, XT, AT>& sm, int n, int r0,
                                                  const int* __restrict__ rowptr,
                                                  const int* __restrict__ colind,
                                                  const VT* __restrict__ val,
                                                  const XT* __restrict__ x, AT init,
                                                  int long_min = INT_MAX,
                                                  bool* skipped = nullptr) {
  const int tid = threadIdx.x;
  const int nr = min(kSpmvRows, n - r0);
  for (int t = tid; t <= nr; t += blockDim.x) sm.rp[t] = rowptr[r0 + t];
  __syncthreads();
  const int base = sm.rp[0];
  const int end = sm.rp[nr];
  int my_b = 0, my_e = 0;
  if (tid < nr) {
    my_b = sm.rp[tid];
    my_e = sm.rp[tid + 1];
  }
  const bool mine_long = tid < nr && my_e - my_b > long_min;
  if (skipped) *skipped = mine_long;
  // the long rows' slot ranges, in row order (a ballot per warp, then the
  // warps' counts added up)
  int nlong = 0;
  if (long_min != INT_MAX) {
    const unsigned bal = __ballot_sync(0xffffffffu, mine_long);
    if ((tid & 31) == 0) sm.wcount[tid >> 5] = __popc(bal);
    __syncthreads();
    int before = __popc(bal & ((1u << (tid & 31)) - 1u));
    for (int w = 0; w < (tid >> 5); w++) before += sm.wcount[w];
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) nlong += sm.wcount[w];
    if (mine_long) {
      sm.lb[before] = my_b;
      sm.le[before] = my_e;
    }
    __syncthreads();
  }
  AT sum = init;
  // stage and fold the slot range between long rows, interval by interval
  int seg_lo = base;
  for (int li = 0; li <= nlong; li++) {
    const int seg_hi = li < nlong ? sm.lb[li] : end;
    for (int c0 = seg_lo; c0 < seg_hi; c0 += kSpmvChunkF) {
      const int cn = min(kSpmvChunkF, seg_hi - c0);
#pragma unroll 6
      for (int k = tid; k < cn; k += kSpmvRows) {
        const int slot = c0 + k;
        sm.v[k] = (AT)val[slot];
        sm.xv[k] = (AT)x[colind[slot]];
      }
      __syncthreads();
      if (!mine_long) {
        const int lo = max(my_b, c0), hi = min(my_e, c0 + cn);
        for (int j = lo; j < hi; j++) {
          if constexpr (sizeof(AT) == 8)
            sum = __fma_rn(sm.v[j - c0], sm.xv[j - c0], sum);
          else
            sum = __fmaf_rn(sm.v[j - c0], sm.xv[j - c0], sum);
        }
      }
      __syncthreads();
    }
    if (li < nlong) seg_lo = sm.le[li];
  }
  return sum;
}

}  // namespace gp
