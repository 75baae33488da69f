// CSR SpMV building block shared by the standalone multiply and the fused
// solver kernels.
//
// One CTA owns kSpmvRows consecutive rows.  The CTA walks the contiguous slot
// range of its rows in chunks: every thread loads values and column indices
// with unit stride (coalesced), forms value * x[col] into shared memory, and
// then each thread adds the products of its own row in ascending slot order.
// Each row is therefore summed exactly as MatMult_SeqAIJ sums it
// (src/ported.mojo:380-391): start at `init`, add one rounded product per slot
// in order -- bit-identical to the sequential loop -- while the memory traffic
// is fully coalesced apart from the x gather.
#pragma once

#include "gp_common.cuh"

namespace gp {

constexpr int kSpmvRows = 256;    // rows per CTA == threads per CTA
constexpr int kSpmvChunk = 2048;  // products staged per pass

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
};

template <typename VT, typename XT, typename AT>
__device__ __forceinline__ AT spmv_block_rows_fma(SpmvSmemF<VT, XT, AT>& sm, int n, int r0,
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
  for (int c0 = base; c0 < end; c0 += kSpmvChunkF) {
    const int cn = min(kSpmvChunkF, end - c0);
#pragma unroll 6
    for (int k = tid; k < cn; k += kSpmvRows) {
      const int slot = c0 + k;
      sm.v[k] = (AT)val[slot];
      sm.xv[k] = (AT)x[colind[slot]];
    }
    __syncthreads();
    const int lo = max(my_b, c0), hi = min(my_e, c0 + cn);
    for (int j = lo; j < hi; j++) {
      if constexpr (sizeof(AT) == 8)
        sum = __fma_rn(sm.v[j - c0], sm.xv[j - c0], sum);
      else
        sum = __fmaf_rn(sm.v[j - c0], sm.xv[j - c0], sum);
    }
    __syncthreads();
  }
  return sum;
}

}  // namespace gp
