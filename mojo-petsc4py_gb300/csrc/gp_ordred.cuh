// Reductions in the reference's own summation order (the "ordered"
// arithmetic).
//
// src/simdvec.mojo:332-473 sums a vector with four SIMD accumulators of
// SW = 4 lanes over blocks of BLK = 16 elements: lane l of accumulator k
// (chain c = 4k + l) folds elements 16t + c, t = 0, 1, ... in order.  The
// accumulators are then combined per lane as ((a0 + a1) + a2) + a3, the
// remaining elements are folded 4 at a time into those lanes, a scalar tail
// goes into a separate sum s, and the result is s + reduce_add(acc).
// _mdot_basis (src/ksp.mojo:956-1062) keeps the block chains but has no
// 4-wide step: its tail is scalar and the result is reduce_add(acc) + t.
// reduce_add's lane order is not fixed by the source; like the oracle this
// uses (acc0 + acc2) + (acc1 + acc3).
//
// Every chain is a sequential sum, which no parallel schedule can reproduce
// to the bit, so each chain runs in order on one warp (one CTA per chain;
// the warp loads 32 consecutive terms of its chain, the serial folds take
// them by shuffle) and the last CTA finishes the combination on one thread.
// A chain of n/16 dependent FP64 adds makes this slow (about 4 ms for
// n = 2^21): it exists so that whole solves can be compared with the
// reference's arithmetic to the bit, not for speed.
#pragma once

#include "gp_common.cuh"

namespace gp {

constexpr int kOrdSW = 4;
constexpr int kOrdBLK = 16;
constexpr int kOrdChains = 16;  // 4 accumulators x SW lanes

enum OrdOp : int { ORD_DOT, ORD_NRM, ORD_DOTNRM, ORD_ASUM, ORD_SUM };

template <int OP>
__device__ __forceinline__ double ord_term(double x, double y) {
  if constexpr (OP == ORD_DOT || OP == ORD_DOTNRM) return mul(x, y);
  if constexpr (OP == ORD_NRM) return mul(x, x);
  if constexpr (OP == ORD_ASUM) return fabs(x);
  return x;  // ORD_SUM
}

__device__ __forceinline__ double ord_lane_reduce(const double (&a)[kOrdSW]) {
  return add(add(a[0], a[2]), add(a[1], a[3]));
}

// Serial fold of chain c of (x, y): elements 16 t + c for t < nb, in order.
// One warp; every lane ends with the chain's sum.  NR = 2 also folds x.x
// (VecDotNorm2).  The next 32 terms are loaded before the current 32 fold.
template <int OP, int NR>
__device__ __forceinline__ void ord_chain(const double* __restrict__ x,
                                          const double* __restrict__ y, int64_t nb, int c,
                                          double (&acc)[NR]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int r = 0; r < NR; r++) acc[r] = 0.0;
  double xv = 0.0, yv = 0.0;
  if (lane < nb) {
    xv = x[(int64_t)lane * kOrdBLK + c];
    yv = (OP == ORD_DOT || OP == ORD_DOTNRM) ? y[(int64_t)lane * kOrdBLK + c] : 0.0;
  }
  for (int64_t t0 = 0; t0 < nb; t0 += 32) {
    double p0 = ord_term<OP>(xv, yv);
    double p1 = NR == 2 ? mul(xv, xv) : 0.0;
    const int64_t tn = t0 + 32 + lane;
    if (tn < nb) {
      xv = x[tn * kOrdBLK + c];
      yv = (OP == ORD_DOT || OP == ORD_DOTNRM) ? y[tn * kOrdBLK + c] : 0.0;
    }
    const int cnt = (int)min((int64_t)32, nb - t0);
    for (int j = 0; j < cnt; j++) {
      acc[0] = add(acc[0], __shfl_sync(0xffffffffu, p0, j));
      if (NR == 2) acc[NR - 1] = add(acc[NR - 1], __shfl_sync(0xffffffffu, p1, j));
    }
  }
}

// One reduction of length n in the reference's order.  Launch with
// kOrdChains CTAs of 32 threads; slot.stride >= kOrdChains.  Writes the sum
// to *out_raw, sqrt(|sum|) to *out_sqrt and, for ORD_DOTNRM, x.x to
// *out_raw2 (each pointer may be null).
template <int OP>
__global__ void __launch_bounds__(32) k_ord_red(const int* gate, int want, int64_t n, DRef xr,
                                                DRef yr, RedSlot slot, double* out_raw,
                                                double* out_sqrt, double* out_raw2) {
  if (gated_off(gate, want)) return;
  constexpr int NR = OP == ORD_DOTNRM ? 2 : 1;
  const double* __restrict__ x = xr.get();
  const double* __restrict__ y = (OP == ORD_DOT || OP == ORD_DOTNRM) ? yr.get() : x;
  const int64_t nb = n / kOrdBLK;
  const int c = blockIdx.x;
  double a[NR];
  ord_chain<OP, NR>(x, y, nb, c, a);
  __shared__ bool last;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int r = 0; r < NR; r++) slot.partials[(size_t)r * slot.stride + c] = a[r];
    last = atomic_add_acq_rel(slot.ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  double res[NR];
#pragma unroll
  for (int r = 0; r < NR; r++) {
    double acc[kOrdSW];
    for (int l = 0; l < kOrdSW; l++) {
      const double* p = slot.partials + (size_t)r * slot.stride;
      acc[l] = add(add(add(__ldcg(p + l), __ldcg(p + kOrdSW + l)), __ldcg(p + 2 * kOrdSW + l)),
                   __ldcg(p + 3 * kOrdSW + l));
    }
    int64_t i = nb * kOrdBLK;
    for (; i + kOrdSW <= n; i += kOrdSW)
      for (int l = 0; l < kOrdSW; l++)
        acc[l] = add(acc[l], r == 1 ? mul(x[i + l], x[i + l]) : ord_term<OP>(x[i + l], y[i + l]));
    double s = 0.0;
    for (; i < n; i++) s = add(s, r == 1 ? mul(x[i], x[i]) : ord_term<OP>(x[i], y[i]));
    res[r] = add(s, ord_lane_reduce(acc));
  }
  if (out_raw) *out_raw = res[0];
  if (out_sqrt) *out_sqrt = __dsqrt_rn(fabs(res[0]));
  if (NR == 2 && out_raw2) *out_raw2 = res[NR - 1];
  *slot.ticket = 0u;
}

// VecMDot of x against *count contiguous basis vectors (ld = n) in
// _mdot_basis's order.  Launch with kOrdChains * kmax CTAs of 32 threads,
// kmax >= *count; CTA b folds chain b % 16 of basis vector b / 16.  Partials
// go to slot.partials[j * slot.stride + c].
static __global__ void __launch_bounds__(32)
    k_ord_mdot(const int* gate, int want, int64_t n, DRef xr, const double* __restrict__ basis,
               const int* count, RedSlot slot, double* __restrict__ out) {
  if (gated_off(gate, want)) return;
  const double* __restrict__ x = xr.get();
  const int k = *count;
  const int j = blockIdx.x / kOrdChains, c = blockIdx.x % kOrdChains;
  const int64_t nb = n / kOrdBLK;
  __shared__ bool last;
  if (j < k) {
    double a[1];
    ord_chain<ORD_DOT, 1>(x, basis + (size_t)j * n, nb, c, a);
    if (threadIdx.x == 0) slot.partials[(size_t)j * slot.stride + c] = a[0];
  }
  if (threadIdx.x == 0) last = atomic_add_acq_rel(slot.ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  for (int jj = threadIdx.x; jj < k; jj += 32) {
    const double* p = slot.partials + (size_t)jj * slot.stride;
    const double* u = basis + (size_t)jj * n;
    double acc[kOrdSW];
    for (int l = 0; l < kOrdSW; l++)
      acc[l] = add(add(add(__ldcg(p + l), __ldcg(p + kOrdSW + l)), __ldcg(p + 2 * kOrdSW + l)),
                   __ldcg(p + 3 * kOrdSW + l));
    double t = 0.0;
    for (int64_t i = nb * kOrdBLK; i < n; i++) t = add(t, mul(x[i], u[i]));
    out[jj] = add(ord_lane_reduce(acc), t);
  }
  __syncwarp();
  if (threadIdx.x == 0) *slot.ticket = 0u;
}

}  // namespace gp
