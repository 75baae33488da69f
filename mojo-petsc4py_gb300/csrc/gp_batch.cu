// Batched CG: many independent SPD systems, each with R right-hand sides,
// solved together in one captured solve graph.
//
// The batch is one block-diagonal CSR matrix (system s owns rows
// [sys_row[s], sys_row[s+1]) and only couples to them) and R-column
// multi-vectors stored row-major (element (row, r) at row * R + r), so one
// sparse pass serves all R columns and the column loads of a row are one
// contiguous 8R-byte run.  Every (system, column) pair runs its own CG
// recurrence -- the PETSc CG of KSPSolve_CG (src/ksp.mojo:271-389), default
// preconditioned norm, Jacobi, IC(0) or no preconditioner -- with its own scalars,
// stopping test and iteration count.  A pair that stops is frozen; a system
// whose R pairs all stopped drops out of every later pass.
//
// Rows are cut into tiles that never cross a system.  A kernel walks tiles
// with a resident grid; per tile it folds the pair dot products in a fixed
// order and stores a partial; the last tile of a system to finish (a ticket
// per system) sums that system's partials in tile order and runs the scalar
// tail of every pair of the system.  No grid-wide barrier, deterministic
// results.
//
// Precision: T = double (plain) or float (the FP32 inner solve of the
// refinement form, whose per-thread and per-tile dot accumulation is FP32 as
// well; the cross-tile sums, the norms and all scalars are FP64).
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gpetsc.h"
#include "gp_common.cuh"
#include "gp_internal.h"
#include "gp_pc.h"

namespace gp {

// stop reasons (KSPConvergedReason values)
constexpr int BR_RTOL = 2, BR_ATOL = 3, BR_ITS = -3, BR_NAN = -4, BR_INDEF_PC = -8,
              BR_INDEF_MAT = -10;

struct BatchDev {
  int nsys, ntiles, n, R;
  const int* rowptr;
  const int* colind;
  const double* val;
  const float* val32;
  const double* dinv;      // Jacobi 1/a_ii (or nullptr: no preconditioner)
  const float* dinv32;
  const int* tile_sys;
  const int* tile_row0;
  const int* tile_nrows;
  const int* sys_tile0;
  const int* sys_ntiles;
  unsigned* sys_ticket;    // one per system, back to zero after every use
  int* sys_active;         // 1 while any pair of the system runs
  int* sys_pairs_left;
  int* active_systems;     // count
  double* partials;        // [ntiles * R * 2]
  // per pair (s * R + r)
  double *a, *beta, *betaold, *bcoef, *dpi, *dpiold, *dp, *rnorm0, *ttol;
  int *it, *its, *reason, *active;
  double rtol, atol, divtol;
  int max_it;
};

template <typename T>
__device__ __forceinline__ T fmadd(T a, T b, T c) {
  if constexpr (sizeof(T) == 8)
    return __fma_rn(a, b, c);
  else
    return __fmaf_rn(a, b, c);
}

__device__ __forceinline__ int dsgn(double x) { return (x > 0.0) - (x < 0.0); }

// ---------------------------------------------------------------- pair tails
__device__ void pair_stop(BatchDev& b, int s, int q, int reason) {
  b.reason[q] = reason;
  b.active[q] = 0;
  if (atomicSub(&b.sys_pairs_left[s], 1) == 1) {
    b.sys_active[s] = 0;
    atomicSub(b.active_systems, 1);
  }
}

// KSPConvergedDefault for pair q at iteration count its with norm dp.
__device__ int pair_conv(BatchDev& b, int q, int its, double dp) {
  if (its == 0) {
    b.rnorm0[q] = dp;
    b.ttol[q] = fmax(b.rtol * dp, b.atol);
  }
  if (!(dp == dp) || isinf(dp)) return BR_NAN;
  if (dp <= b.ttol[q]) return dp < b.atol ? BR_ATOL : BR_RTOL;
  if (its > 0 && dp >= b.divtol * b.rnorm0[q]) return BR_NAN;
  return 0;
}

// after ||z|| and z.r: record, test, form the top of the next iteration
__device__ void pair_after_update(BatchDev& b, int s, int q, double zz, double zr,
                                  bool first) {
  if (!b.active[q]) return;
  const double dp = sqrt(zz);
  b.dp[q] = dp;
  int its = first ? 0 : b.it[q] + 1;
  b.its[q] = its;
  int reason = pair_conv(b, q, its, dp);
  if (reason) {
    pair_stop(b, s, q, reason);
    return;
  }
  if (!first) {
    b.it[q] += 1;
    if (b.it[q] >= b.max_it) {
      pair_stop(b, s, q, BR_ITS);
      return;
    }
  } else {
    b.it[q] = 0;
    b.dpi[q] = 0.0;
    b.betaold[q] = 1.0;
  }
  const double beta = zr;
  b.beta[q] = beta;
  const int i = b.it[q];
  if (beta == 0.0) {
    pair_stop(b, s, q, BR_ATOL);
    return;
  }
  if (i > 0 && beta * b.betaold[q] < 0.0) {
    pair_stop(b, s, q, BR_INDEF_PC);
    return;
  }
  b.bcoef[q] = i == 0 ? 0.0 : beta / b.betaold[q];
  b.dpiold[q] = b.dpi[q];
}

__device__ void pair_after_spmm(BatchDev& b, int s, int q, double dpi) {
  if (!b.active[q]) return;
  const int i = b.it[q];
  b.dpi[q] = dpi;
  b.betaold[q] = b.beta[q];
  if (dpi == 0.0 || (i > 0 && dsgn(dpi) * dsgn(b.dpiold[q]) < 0)) {
    pair_stop(b, s, q, BR_INDEF_MAT);
    return;
  }
  b.a[q] = b.beta[q] / dpi;
}

// ------------------------------------------------------------- tile plumbing
// Per-column tile sums of NV values per thread (threads t with t % L == g own
// columns g*VR .. g*VR+VR-1), written to partials[(tile * R + col) * 2 + k].
template <typename T, int R, int VR, int NV>
__device__ __forceinline__ void tile_partials(const BatchDev& b, int tile, T (&acc)[NV][VR],
                                              T* sh) {
  constexpr int L = R / VR;
  const int t = threadIdx.x, slots = blockDim.x / L;
#pragma unroll
  for (int k = 0; k < NV; k++)
#pragma unroll
    for (int v = 0; v < VR; v++) sh[(k * VR + v) * blockDim.x + t] = acc[k][v];
  __syncthreads();
  for (int h = slots >> 1; h >= 1; h >>= 1) {
    if (t / L < h) {
#pragma unroll
      for (int k = 0; k < NV; k++)
#pragma unroll
        for (int v = 0; v < VR; v++) {
          T* p = &sh[(k * VR + v) * blockDim.x];
          p[t] = p[t] + p[t + h * L];
        }
    }
    __syncthreads();
  }
  // thread 0 stores them all, so the release of its ticket increment
  // (system_last) covers every partial of the tile
  if (t == 0) {
    for (int gg = 0; gg < L; gg++)
#pragma unroll
      for (int k = 0; k < NV; k++)
#pragma unroll
        for (int v = 0; v < VR; v++)
          b.partials[((size_t)tile * R + gg * VR + v) * 2 + k] =
              (double)sh[(k * VR + v) * blockDim.x + gg];
  }
  __syncthreads();
}

// True in every thread of the CTA that finished system s's last tile.
__device__ __forceinline__ bool system_last(BatchDev& b, int s) {
  __shared__ bool last;
  if (threadIdx.x == 0) last = atomic_add_acq_rel(&b.sys_ticket[s], 1u) == b.sys_ntiles[s] - 1;
  __syncthreads();
  return last;
}

// Sum system s's partials for every (column, value) pair: warp w folds sums
// j = w, w + nwarps, ... (j = column * NV + value); its lanes take tiles
// lane, lane + 32, ... in order and a shuffle tree combines them -- a fixed
// order, many loads in flight.  All threads call it; the totals are in the
// returned shared array (index j) afterwards.
__device__ __forceinline__ const double* system_sums(const BatchDev& b, int s, int R, int NV) {
  __shared__ double tot[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int t0 = b.sys_tile0[s], nt = b.sys_ntiles[s];
  for (int j = w; j < R * NV; j += nw) {
    const int col = j / NV, k = j % NV;
    double acc = 0.0;
    for (int tt = lane; tt < nt; tt += 32)
      acc += __ldcg(&b.partials[((size_t)(t0 + tt) * R + col) * 2 + k]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) tot[j] = acc;
  }
  __syncthreads();
  return tot;
}

// ------------------------------------------------------------------ kernels
#define TILE_LOOP(tile)                                                       \
  for (int tile = blockIdx.x; tile < b.ntiles; tile += gridDim.x)

// p = z (first) or z + bcoef p, active pairs only
template <typename T, int R>
__global__ void k_bp(BatchDev b, T* __restrict__ p, const T* __restrict__ z) {
  TILE_LOOP(tile) {
    const int s = b.tile_sys[tile];
    if (!b.sys_active[s]) continue;
    // blockDim is a multiple of R: a thread keeps one column for the tile
    const int q = s * R + threadIdx.x % R;
    if (!b.active[q]) continue;
    const double bc = b.bcoef[q];
    const T tb = (T)bc;
    const int r0 = b.tile_row0[tile], ne = b.tile_nrows[tile] * R;
    T* pp = p + (size_t)r0 * R;
    const T* zz = z + (size_t)r0 * R;
    if (bc == 0.0) {
      for (int e = threadIdx.x; e < ne; e += blockDim.x) pp[e] = zz[e];
    } else {
      for (int e = threadIdx.x; e < ne; e += blockDim.x) pp[e] = fmadd<T>(tb, pp[e], zz[e]);
    }
  }
}

// w = A p and the pair dots p.w; the system's last tile forms alpha
template <typename T, int R, int VR>
__global__ void k_bspmm(BatchDev b, const T* __restrict__ val, const T* __restrict__ p,
                        T* __restrict__ w) {
  constexpr int L = R / VR;
  extern __shared__ unsigned char smem_raw[];
  T* sh = reinterpret_cast<T*>(smem_raw);
  const int t = threadIdx.x, g = t % L, slots = blockDim.x / L;
  TILE_LOOP(tile) {
    const int s = b.tile_sys[tile];
    if (!b.sys_active[s]) continue;
    const int r0 = b.tile_row0[tile], nr = b.tile_nrows[tile];
    T dot[1][VR];
#pragma unroll
    for (int v = 0; v < VR; v++) dot[0][v] = (T)0;
    for (int rr = t / L; rr < nr; rr += slots) {
      const int row = r0 + rr;
      const int j0 = b.rowptr[row], j1 = b.rowptr[row + 1];
      T acc[VR];
#pragma unroll
      for (int v = 0; v < VR; v++) acc[v] = (T)0;
      // four slots per batch: their values, columns and gathers are all in
      // flight before the first multiply-add (the chain column -> gather is
      // otherwise paid once per nonzero)
      constexpr int S = 4;  // slots per batch (2 measured slower for 4-wide FP32 rows)
      for (int j = j0; j < j1; j += S) {
        T a[S], xv[S][VR];
        int c[S];
#pragma unroll
        for (int u = 0; u < S; u++)
          if (j + u < j1) {
            a[u] = val[j + u];
            c[u] = b.colind[j + u];
          }
#pragma unroll
        for (int u = 0; u < S; u++)
          if (j + u < j1) {
#pragma unroll
            for (int v = 0; v < VR; v++) xv[u][v] = p[(size_t)c[u] * R + g * VR + v];
          }
#pragma unroll
        for (int u = 0; u < S; u++)
          if (j + u < j1) {
#pragma unroll
            for (int v = 0; v < VR; v++) acc[v] = fmadd<T>(a[u], xv[u][v], acc[v]);
          }
      }
      const size_t o = (size_t)row * R + g * VR;
#pragma unroll
      for (int v = 0; v < VR; v++) {
        w[o + v] = acc[v];
        dot[0][v] = fmadd<T>(p[o + v], acc[v], dot[0][v]);
      }
    }
    tile_partials<T, R, VR, 1>(b, tile, dot, sh);
    if (system_last(b, s)) {
      const double* tot = system_sums(b, s, R, 1);
      if (t < R) pair_after_spmm(b, s, s * R + t, tot[t]);
      __syncthreads();
      if (t == 0) b.sys_ticket[s] = 0u;
    }
  }
}

// x += a p; r -= a w; z = D r (or r); pair ||z||^2, z.r; last tile: the tail
template <typename T, int R, int VR, bool FIRST>
__global__ void k_bupdate(BatchDev b, const T* __restrict__ dinv, T* __restrict__ x,
                          T* __restrict__ r, const T* __restrict__ p, const T* w, T* z) {
  constexpr int L = R / VR;
  extern __shared__ unsigned char smem_raw[];
  T* sh = reinterpret_cast<T*>(smem_raw);
  const int t = threadIdx.x, g = t % L, slots = blockDim.x / L;
  TILE_LOOP(tile) {
    const int s = b.tile_sys[tile];
    if (!b.sys_active[s]) continue;
    const int r0 = b.tile_row0[tile], nr = b.tile_nrows[tile];
    T acc[2][VR];
#pragma unroll
    for (int v = 0; v < VR; v++) acc[0][v] = acc[1][v] = (T)0;
    T al[VR];
    bool on[VR];
#pragma unroll
    for (int v = 0; v < VR; v++) {
      const int q = s * R + g * VR + v;
      on[v] = b.active[q] != 0;
      al[v] = FIRST ? (T)0 : (T)b.a[q];
    }
    for (int rr = t / L; rr < nr; rr += slots) {
      const int row = r0 + rr;
      const T d = dinv ? dinv[row] : (T)1;
      const size_t o = (size_t)row * R + g * VR;
#pragma unroll
      for (int v = 0; v < VR; v++) {
        if (!on[v]) continue;
        T ri = r[o + v];
        if (!FIRST) {
          x[o + v] = fmadd<T>(al[v], p[o + v], x[o + v]);
          ri = fmadd<T>(-al[v], w[o + v], ri);
          r[o + v] = ri;
        }
        const T zi = dinv ? ri * d : ri;
        z[o + v] = zi;
        acc[0][v] = fmadd<T>(zi, zi, acc[0][v]);
        acc[1][v] = fmadd<T>(zi, ri, acc[1][v]);
      }
    }
    tile_partials<T, R, VR, 2>(b, tile, acc, sh);
    if (system_last(b, s)) {
      const double* tot = system_sums(b, s, R, 2);
      if (t < R) pair_after_update(b, s, s * R + t, tot[2 * t], tot[2 * t + 1], FIRST);
      __syncthreads();
      if (t == 0) b.sys_ticket[s] = 0u;
    }
  }
}

// x += a p; r -= a w, active pairs only (the preconditioner and the pair
// dots follow: IC(0))
template <int R>
__global__ void k_bupdate_xr(BatchDev b, double* __restrict__ x, double* __restrict__ r,
                             const double* __restrict__ p, const double* __restrict__ w) {
  TILE_LOOP(tile) {
    const int s = b.tile_sys[tile];
    if (!b.sys_active[s]) continue;
    const int q = s * R + threadIdx.x % R;  // blockDim is a multiple of R
    if (!b.active[q]) continue;
    const double al = b.a[q];
    const int r0 = b.tile_row0[tile], ne = b.tile_nrows[tile] * R;
    const size_t o0 = (size_t)r0 * R;
    for (int e = threadIdx.x; e < ne; e += blockDim.x) {
      x[o0 + e] = fmadd<double>(al, p[o0 + e], x[o0 + e]);
      r[o0 + e] = fmadd<double>(-al, w[o0 + e], r[o0 + e]);
    }
  }
}

// pair ||z||^2 and z.r after a separate preconditioner apply; the system's
// last tile runs the pairs' tails
template <int R, bool FIRST>
__global__ void k_bdots(BatchDev b, const double* __restrict__ r, const double* __restrict__ z) {
  extern __shared__ unsigned char smem_raw[];
  double* sh = reinterpret_cast<double*>(smem_raw);
  const int t = threadIdx.x, slots = blockDim.x / R;
  TILE_LOOP(tile) {
    const int s = b.tile_sys[tile];
    if (!b.sys_active[s]) continue;
    const int r0 = b.tile_row0[tile], nr = b.tile_nrows[tile];
    double acc[2][1] = {{0.0}, {0.0}};
    const bool on = b.active[s * R + t % R] != 0;
    for (int rr = t / R; rr < nr && on; rr += slots) {
      const size_t o = (size_t)(r0 + rr) * R + t % R;
      const double zi = z[o];
      acc[0][0] = fmadd<double>(zi, zi, acc[0][0]);
      acc[1][0] = fmadd<double>(zi, r[o], acc[1][0]);
    }
    tile_partials<double, R, 1, 2>(b, tile, acc, sh);
    if (system_last(b, s)) {
      const double* tot = system_sums(b, s, R, 2);
      if (t < R) pair_after_update(b, s, s * R + t, tot[2 * t], tot[2 * t + 1], FIRST);
      __syncthreads();
      if (t == 0) b.sys_ticket[s] = 0u;
    }
  }
}

__global__ void k_bctrl(cudaGraphConditionalHandle h, int* active_systems, int* trips,
                        int cap) {
  *trips += 1;
  cudaGraphSetConditional(h, (*active_systems > 0 && *trips < cap) ? 1u : 0u);
}

// host-driven loop: the trip count without the graph conditional
__global__ void k_btrip(int* trips) { *trips += 1; }

// residual of the FP64 system for the refinement form: r = b - A x (FP64),
// per pair ||r||^2; the last tile stores rn = ||r|| and freezes pairs whose
// true relative residual is at most rtol (rn <= rtol * ||b||)
template <int R, int VR>
__global__ void k_bresid(BatchDev b, const double* __restrict__ bb, const double* __restrict__ x,
                         double* __restrict__ r, const double* __restrict__ bnorm,
                         double* __restrict__ rn, int freeze) {
  constexpr int L = R / VR;
  extern __shared__ unsigned char smem_raw[];
  double* sh = reinterpret_cast<double*>(smem_raw);
  const int t = threadIdx.x, g = t % L, slots = blockDim.x / L;
  TILE_LOOP(tile) {
    const int s = b.tile_sys[tile];
    if (freeze && !b.sys_active[s]) continue;
    const int r0 = b.tile_row0[tile], nr = b.tile_nrows[tile];
    double acc[1][VR];
#pragma unroll
    for (int v = 0; v < VR; v++) acc[0][v] = 0.0;
    for (int rr = t / L; rr < nr; rr += slots) {
      const int row = r0 + rr;
      const int j0 = b.rowptr[row], j1 = b.rowptr[row + 1];
      double ax[VR];
#pragma unroll
      for (int v = 0; v < VR; v++) ax[v] = 0.0;
      for (int j = j0; j < j1; j += 4) {
        double a[4], xv[4][VR];
        int c[4];
#pragma unroll
        for (int u = 0; u < 4; u++)
          if (j + u < j1) {
            a[u] = b.val[j + u];
            c[u] = b.colind[j + u];
          }
#pragma unroll
        for (int u = 0; u < 4; u++)
          if (j + u < j1) {
#pragma unroll
            for (int v = 0; v < VR; v++) xv[u][v] = x[(size_t)c[u] * R + g * VR + v];
          }
#pragma unroll
        for (int u = 0; u < 4; u++)
          if (j + u < j1) {
#pragma unroll
            for (int v = 0; v < VR; v++) ax[v] = fma(a[u], xv[u][v], ax[v]);
          }
      }
      const size_t o = (size_t)row * R + g * VR;
#pragma unroll
      for (int v = 0; v < VR; v++) {
        const double ri = bb[o + v] - ax[v];
        r[o + v] = ri;
        acc[0][v] = fma(ri, ri, acc[0][v]);
      }
    }
    tile_partials<double, R, VR, 1>(b, tile, acc, sh);
    if (system_last(b, s)) {
      const double* tot = system_sums(b, s, R, 1);
      if (t < R) {
        const int q = s * R + t;
        const double nrm = sqrt(tot[t]);
        rn[q] = nrm;
        if (freeze && b.active[q] && !(nrm > b.rtol * bnorm[q])) pair_stop(b, s, q, BR_RTOL);
      }
      __syncthreads();
      if (t == 0) b.sys_ticket[s] = 0u;
    }
  }
}

// ||b|| per pair (once, for the refinement form's stopping test)
template <int R>
__global__ void k_bnorm(BatchDev b, const double* __restrict__ bb, double* __restrict__ out) {
  extern __shared__ unsigned char smem_raw[];
  double* sh = reinterpret_cast<double*>(smem_raw);
  const int t = threadIdx.x, slots = blockDim.x / R;
  TILE_LOOP(tile) {
    const int s = b.tile_sys[tile];
    const int r0 = b.tile_row0[tile], nr = b.tile_nrows[tile];
    double acc[1][1] = {{0.0}};
    for (int rr = t / R; rr < nr; rr += slots) {
      const double v = bb[(size_t)(r0 + rr) * R + t % R];
      acc[0][0] = fma(v, v, acc[0][0]);
    }
    tile_partials<double, R, 1, 1>(b, tile, acc, sh);
    if (system_last(b, s)) {
      const double* tot = system_sums(b, s, R, 1);
      if (t < R) out[s * R + t] = sqrt(tot[t]);
      __syncthreads();
      if (t == 0) b.sys_ticket[s] = 0u;
    }
  }
}

// inner right-hand side r32 = r / rn (0 for frozen pairs), x32 = 0
template <int R>
__global__ void k_bscale_in(BatchDev b, const double* __restrict__ r,
                            const double* __restrict__ rn, float* __restrict__ r32,
                            float* __restrict__ x32) {
  TILE_LOOP(tile) {
    const int s = b.tile_sys[tile];
    const int r0 = b.tile_row0[tile], ne = b.tile_nrows[tile] * R;
    for (int e = threadIdx.x; e < ne; e += blockDim.x) {
      const int q = s * R + e % R;
      const size_t i = (size_t)r0 * R + e;
      r32[i] = b.active[q] ? __double2float_rn(r[i] / rn[q]) : 0.0f;
      x32[i] = 0.0f;
    }
  }
}

// x += rn * x32 for the pairs that were refined in this pass
template <int R>
__global__ void k_bacc(BatchDev b, const int* __restrict__ refined, const double* __restrict__ rn,
                       const float* __restrict__ x32, double* __restrict__ x) {
  TILE_LOOP(tile) {
    const int s = b.tile_sys[tile];
    const int r0 = b.tile_row0[tile], ne = b.tile_nrows[tile] * R;
    for (int e = threadIdx.x; e < ne; e += blockDim.x) {
      const int q = s * R + e % R;
      if (!refined[q]) continue;
      const size_t i = (size_t)r0 * R + e;
      x[i] = fma(rn[q], (double)x32[i], x[i]);
    }
  }
}

// pair and system state from a pair mask (all pairs when mask is null)
__global__ void k_bstate(BatchDev b, const int* __restrict__ mask) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < b.nsys; s += gridDim.x * blockDim.x) {
    int left = 0;
    for (int c = 0; c < b.R; c++) {
      const int q = s * b.R + c;
      const int on = mask ? mask[q] : 1;
      b.active[q] = on;
      if (mask == nullptr) {
        b.reason[q] = 0;
        b.its[q] = 0;
      }
      left += on;
    }
    b.sys_pairs_left[s] = left;
    b.sys_active[s] = left > 0;
    if (left) atomicAdd(b.active_systems, 1);
  }
}

__global__ void k_bsum_its(int npairs, const int* __restrict__ its, int* __restrict__ total) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < npairs; q += gridDim.x * blockDim.x)
    total[q] += its[q];
}

__global__ void k_bjacobi(int n, const int* __restrict__ diagpos, const double* __restrict__ val,
                          double* __restrict__ dinv, float* __restrict__ dinv32) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int p = diagpos[i];
    const double d = p >= 0 ? val[p] : 0.0;
    const double v = d != 0.0 ? 1.0 / d : 1.0;  // an exact zero keeps 1 (PCSetUp_Jacobi)
    dinv[i] = v;
    dinv32[i] = __double2float_rn(v);
  }
}

// ================================================================== host side
struct Tuning {
  int block = 256, vr = 1, tile_rows = 128;
  double spmm_us = 0.0;
};

struct Batch {
  int nsys = 0, n = 0, R = 0, ntiles = 0, device = -1;
  int64_t nnz = 0;
  // rows of each system renumbered by reverse Cuthill-McKee so that a row's
  // neighbours -- whose right-hand-side blocks the sparse pass gathers -- sit
  // close to it: perm[new] = old (global rows); right-hand sides come in and
  // solutions go out through it, in the caller's numbering
  int* perm = nullptr;
  double *bp = nullptr, *xp = nullptr;  // permuted B and X
  std::vector<int> sys_row;           // host, nsys + 1
  std::vector<int> h_rowptr, h_colind;
  // device matrix and preconditioner
  int *rowptr = nullptr, *colind = nullptr, *diagpos = nullptr;
  double* val = nullptr;
  float* val32 = nullptr;
  double* dinv = nullptr;
  float* dinv32 = nullptr;
  // tiles
  int *tile_sys = nullptr, *tile_row0 = nullptr, *tile_nrows = nullptr;
  int *sys_tile0 = nullptr, *sys_ntiles = nullptr;
  // state
  unsigned* sys_ticket = nullptr;
  int *sys_active = nullptr, *sys_pairs_left = nullptr, *counters = nullptr;  // [active, trips]
  double* partials = nullptr;
  double* pair_d = nullptr;   // 9 arrays of npairs
  int* pair_i = nullptr;      // 4 arrays of npairs + refined + its_total
  // work vectors (n * R)
  double *r = nullptr, *p = nullptr, *z = nullptr;
  float *x32 = nullptr, *r32 = nullptr, *p32 = nullptr, *z32 = nullptr;
  double *bnorm = nullptr, *rn = nullptr;
  // IC(0) of the block-diagonal matrix (set up on its first use) and its
  // sweeps' scratch (n * R each)
  Csr* icc_A = nullptr;
  Pc* icc = nullptr;
  double *icc_vf = nullptr, *icc_vb = nullptr, *icc_ys = nullptr;
  Tuning tune, tune32;          // FP64 and FP32 sparse-pass choices
  const Tuning* cur = &tune;    // the one the current solve launches with
  bool tuned = false;
  cudaStream_t cap_stream = nullptr;
  // captured solves: [0] FP64 CG between (cap_b, cap_x), [1] FP32 inner CG
  cudaGraphExec_t exec[2] = {nullptr, nullptr};
  cudaGraph_t graph[2] = {nullptr, nullptr};
  const double* cap_b[2] = {nullptr, nullptr};
  double* cap_x[2] = {nullptr, nullptr};
  double cap_key[2][10] = {};
};

static BatchDev dev_view(const Batch& B, double rtol, double atol, double divtol, int max_it,
                         int pc) {
  BatchDev d{};
  d.nsys = B.nsys;
  d.ntiles = B.ntiles;
  d.n = B.n;
  d.R = B.R;
  d.rowptr = B.rowptr;
  d.colind = B.colind;
  d.val = B.val;
  d.val32 = B.val32;
  d.dinv = pc == 2 ? B.dinv : nullptr;
  d.dinv32 = pc == 2 ? B.dinv32 : nullptr;
  d.tile_sys = B.tile_sys;
  d.tile_row0 = B.tile_row0;
  d.tile_nrows = B.tile_nrows;
  d.sys_tile0 = B.sys_tile0;
  d.sys_ntiles = B.sys_ntiles;
  d.sys_ticket = B.sys_ticket;
  d.sys_active = B.sys_active;
  d.sys_pairs_left = B.sys_pairs_left;
  d.active_systems = B.counters;
  d.partials = B.partials;
  const size_t np = (size_t)B.nsys * B.R;
  double* pd = B.pair_d;
  d.a = pd;
  d.beta = pd + np;
  d.betaold = pd + 2 * np;
  d.bcoef = pd + 3 * np;
  d.dpi = pd + 4 * np;
  d.dpiold = pd + 5 * np;
  d.dp = pd + 6 * np;
  d.rnorm0 = pd + 7 * np;
  d.ttol = pd + 8 * np;
  int* pi = B.pair_i;
  d.it = pi;
  d.its = pi + np;
  d.reason = pi + 2 * np;
  d.active = pi + 3 * np;
  d.rtol = rtol;
  d.atol = atol;
  d.divtol = divtol;
  d.max_it = max_it;
  return d;
}
static int* refined_of(const Batch& B) { return B.pair_i + 4 * (size_t)B.nsys * B.R; }
static int* its_total_of(const Batch& B) { return B.pair_i + 5 * (size_t)B.nsys * B.R; }

// ---------------------------------------------------------- launch dispatch
// R in {1, 2, 4, 8, 16}; VR in {1, 2, 4} dividing R.
template <typename F>
static int with_shape(int R, int vr, F&& f) {
#define SHAPE(RR, VV)                                                         \
  if (R == RR && vr == VV) {                                                  \
    f(std::integral_constant<int, RR>{}, std::integral_constant<int, VV>{}); \
    return GP_OK;                                                             \
  }
  SHAPE(1, 1) SHAPE(2, 1) SHAPE(2, 2) SHAPE(4, 1) SHAPE(4, 2) SHAPE(4, 4) SHAPE(8, 1)
  SHAPE(8, 2) SHAPE(8, 4) SHAPE(16, 1) SHAPE(16, 2) SHAPE(16, 4)
#undef SHAPE
  set_error("batched CG: unsupported right-hand-side count or vector width");
  return GP_ERR_ARG;
}

static int resident(const void* k, int block, size_t smem) {
  int per = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, block, smem) != cudaSuccess ||
      per < 1) {
    cudaGetLastError();
    per = 1;
  }
  return per * num_sms();
}

struct Launch {
  int grid, block;
  size_t smem;
};

template <typename T, int R, int VR, int NV>
static Launch shape_of(const Batch& B, const void* k) {
  Launch l;
  l.block = B.cur->block;
  l.smem = (size_t)NV * VR * l.block * sizeof(T);
  l.grid = std::max(1, std::min(B.ntiles, resident(k, l.block, l.smem)));
  return l;
}

template <typename T, int R, int VR>
static void launch_spmm(const Batch& B, const BatchDev& d, const T* val, const T* p, T* w,
                        cudaStream_t s) {
  auto k = k_bspmm<T, R, VR>;
  Launch l = shape_of<T, R, VR, 1>(B, (const void*)k);
  k<<<l.grid, l.block, l.smem, s>>>(d, val, p, w);
}

template <typename T, int R, int VR, bool FIRST>
static void launch_update(const Batch& B, const BatchDev& d, const T* dinv, T* x, T* r,
                          const T* p, const T* w, T* z, cudaStream_t s) {
  auto k = k_bupdate<T, R, VR, FIRST>;
  Launch l = shape_of<T, R, VR, 2>(B, (const void*)k);
  k<<<l.grid, l.block, l.smem, s>>>(d, dinv, x, r, p, w, z);
}

template <typename T, int R>
static void launch_p(const Batch& B, const BatchDev& d, T* p, const T* z, cudaStream_t s) {
  auto k = k_bp<T, R>;
  const int g = std::max(1, std::min(B.ntiles, resident((const void*)k, B.cur->block, 0)));
  k<<<g, B.cur->block, 0, s>>>(d, p, z);
}

template <int R>
static void launch_update_xr(const Batch& B, const BatchDev& d, double* x, double* r,
                             const double* p, const double* w, cudaStream_t s) {
  auto k = k_bupdate_xr<R>;
  const int g = std::max(1, std::min(B.ntiles, resident((const void*)k, B.cur->block, 0)));
  k<<<g, B.cur->block, 0, s>>>(d, x, r, p, w);
}

template <int R, bool FIRST>
static void launch_dots(const Batch& B, const BatchDev& d, const double* r, const double* z,
                        cudaStream_t s) {
  auto k = k_bdots<R, FIRST>;
  Launch l = shape_of<double, R, 1, 2>(B, (const void*)k);
  k<<<l.grid, l.block, l.smem, s>>>(d, r, z);
}

// IC(0) of the block-diagonal batch matrix in its (renumbered) rows: the
// library's PC set-up on the whole matrix -- no entry couples two systems,
// so this is each system's IC(0) -- built once, on the first IC solve.
static int batch_icc_setup(Batch& B, cudaStream_t s) {
  if (B.icc) return GP_OK;
  std::vector<double> hv((size_t)std::max<int64_t>(B.nnz, 1));
  if (B.nnz)
    GP_CUDA(cudaMemcpy(hv.data(), B.val, (size_t)B.nnz * sizeof(double),
                       cudaMemcpyDeviceToHost));
  GP_TRY(csr_create_i32(&B.icc_A, B.n, B.n, B.nnz, B.h_rowptr.data(), B.h_colind.data(),
                        hv.data(), s));
  GP_TRY(pc_create(&B.icc));
  B.icc->opt.type = PC_ICC;
  GP_TRY(pc_setup(B.icc, B.icc_A, s));
  const size_t nv = std::max<size_t>((size_t)B.n * B.R, 1);
  GP_CUDA(cudaMalloc(&B.icc_vf, nv * sizeof(double)));
  GP_CUDA(cudaMalloc(&B.icc_vb, nv * sizeof(double)));
  GP_CUDA(cudaMalloc(&B.icc_ys, nv * sizeof(double)));
  return GP_OK;
}

template <int R, int VR>
static void launch_resid(const Batch& B, const BatchDev& d, const double* b, const double* x,
                         int freeze, cudaStream_t s) {
  auto k = k_bresid<R, VR>;
  Launch l = shape_of<double, R, VR, 1>(B, (const void*)k);
  k<<<l.grid, l.block, l.smem, s>>>(d, b, x, B.r, B.bnorm, B.rn, freeze);
}

static void launch_state(const Batch& B, const BatchDev& d, const int* mask, cudaStream_t s) {
  cudaMemsetAsync(B.counters, 0, sizeof(int), s);
  k_bstate<<<std::max(1, std::min((B.nsys + 255) / 256, num_sms() * 4)), 256, 0, s>>>(d, mask);
}

// ---------------------------------------------------------------- tiles
static void free_tiles(Batch& B) {
  void* ptrs[] = {B.tile_sys, B.tile_row0, B.tile_nrows, B.sys_tile0, B.sys_ntiles,
                  B.partials};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  B.tile_sys = B.tile_row0 = B.tile_nrows = B.sys_tile0 = B.sys_ntiles = nullptr;
  B.partials = nullptr;
}

template <typename V>
static int upload_vec(V** d, const std::vector<V>& h, cudaStream_t s) {
  GP_CUDA(cudaMalloc(d, std::max<size_t>(h.size(), 1) * sizeof(V)));
  if (!h.empty())
    GP_CUDA(cudaMemcpyAsync(*d, h.data(), h.size() * sizeof(V), cudaMemcpyHostToDevice, s));
  return GP_OK;
}

static int build_tiles(Batch& B, int tile_rows, cudaStream_t s) {
  free_tiles(B);
  std::vector<int> ts, tr0, tnr, st0(B.nsys), snt(B.nsys);
  for (int sy = 0; sy < B.nsys; sy++) {
    st0[sy] = (int)ts.size();
    for (int r0 = B.sys_row[sy]; r0 < B.sys_row[sy + 1]; r0 += tile_rows) {
      ts.push_back(sy);
      tr0.push_back(r0);
      tnr.push_back(std::min(tile_rows, B.sys_row[sy + 1] - r0));
    }
    if ((int)ts.size() == st0[sy]) {  // an empty system still owns one (empty) tile
      ts.push_back(sy);
      tr0.push_back(B.sys_row[sy]);
      tnr.push_back(0);
    }
    snt[sy] = (int)ts.size() - st0[sy];
  }
  B.ntiles = (int)ts.size();
  GP_TRY(upload_vec(&B.tile_sys, ts, s));
  GP_TRY(upload_vec(&B.tile_row0, tr0, s));
  GP_TRY(upload_vec(&B.tile_nrows, tnr, s));
  GP_TRY(upload_vec(&B.sys_tile0, st0, s));
  GP_TRY(upload_vec(&B.sys_ntiles, snt, s));
  GP_CUDA(cudaMalloc(&B.partials, (size_t)B.ntiles * B.R * 2 * sizeof(double)));
  GP_CUDA(cudaStreamSynchronize(s));
  B.tune.tile_rows = tile_rows;
  return GP_OK;
}

static void drop_graphs(Batch& B) {
  for (int i = 0; i < 2; i++) {
    if (B.exec[i]) cudaGraphExecDestroy(B.exec[i]);
    if (B.graph[i]) cudaGraphDestroy(B.graph[i]);
    B.exec[i] = nullptr;
    B.graph[i] = nullptr;
  }
  B.cap_b[0] = B.cap_b[1] = nullptr;
  B.cap_x[0] = B.cap_x[1] = nullptr;
}

void batch_destroy(Batch* B) {
  if (!B) return;
  drop_graphs(*B);
  free_tiles(*B);
  void* ptrs[] = {B->rowptr, B->colind, B->diagpos, B->val, B->val32, B->dinv, B->dinv32,
                  B->sys_ticket, B->sys_active, B->sys_pairs_left, B->counters, B->pair_d,
                  B->pair_i, B->r, B->p, B->z, B->x32, B->r32, B->p32, B->z32, B->bnorm,
                  B->rn, B->perm, B->bp, B->xp, B->icc_vf, B->icc_vb, B->icc_ys};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (B->icc) pc_destroy(B->icc);
  if (B->icc_A) csr_destroy(B->icc_A);
  if (B->cap_stream) cudaStreamDestroy(B->cap_stream);
  delete B;
}

// out row k = in row perm[k] (gather) or out row perm[k] = in row k (scatter),
// R columns a row
__global__ void k_brows_permute(int n, int R, const int* __restrict__ perm, int scatter,
                                const double* __restrict__ in, double* __restrict__ out) {
  const int64_t total = (int64_t)n * R;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(q / R), c = (int)(q % R);
    const int64_t o = (int64_t)perm[k] * R + c;
    if (scatter)
      out[o] = in[q];
    else
      out[q] = in[o];
  }
}

__global__ void k_bto_f32(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    b[i] = __double2float_rn(a[i]);
}

int batch_create(Batch** out, int64_t nsys, const int64_t* sys_rows, const int64_t* indptr,
                 const int64_t* indices, const double* values, int nrhs, cudaStream_t s) {
  if (nsys < 1 || !sys_rows || !indptr) {
    set_error("batched CG: need at least one system and its row offsets");
    return GP_ERR_ARG;
  }
  if (nrhs != 1 && nrhs != 2 && nrhs != 4 && nrhs != 8 && nrhs != 16) {
    set_error("batched CG: right-hand sides per system must be 1, 2, 4, 8 or 16");
    return GP_ERR_ARG;
  }
  const int64_t n = sys_rows[nsys], nnz = indptr[n];
  if (sys_rows[0] != 0 || n < 0 || n >= INT32_MAX || nnz < 0 || nnz >= INT32_MAX ||
      (int64_t)n * nrhs >= ((int64_t)1 << 40)) {
    set_error("batched CG: sizes out of range");
    return GP_ERR_ARG;
  }
  Batch* B = new Batch();
  B->nsys = (int)nsys;
  B->n = (int)n;
  B->R = nrhs;
  B->nnz = nnz;
  B->sys_row.resize(nsys + 1);
  for (int64_t i = 0; i <= nsys; i++) {
    if (i && sys_rows[i] < sys_rows[i - 1]) {
      delete B;
      set_error("batched CG: system row offsets must not decrease");
      return GP_ERR_ARG;
    }
    B->sys_row[i] = (int)sys_rows[i];
  }
  // block-diagonal check and diagonal positions
  std::vector<int> diag(std::max<int64_t>(n, 1), -1);
  B->h_rowptr.resize(n + 1);
  B->h_colind.resize(std::max<int64_t>(nnz, 1));
  int st = GP_OK;
  for (int sy = 0; sy < B->nsys && st == GP_OK; sy++)
    for (int i = B->sys_row[sy]; i < B->sys_row[sy + 1] && st == GP_OK; i++) {
      if (indptr[i + 1] < indptr[i]) st = GP_ERR_ARG;
      for (int64_t j = indptr[i]; j < indptr[i + 1] && st == GP_OK; j++) {
        const int64_t c = indices[j];
        if (c < B->sys_row[sy] || c >= B->sys_row[sy + 1]) st = GP_ERR_ARG;
        if (c == i) diag[i] = (int)j;
        B->h_colind[j] = (int)c;
      }
    }
  if (st != GP_OK) {
    delete B;
    set_error("batched CG: every row must couple only to columns of its own system");
    return GP_ERR_ARG;
  }
  for (int64_t i = 0; i <= n; i++) B->h_rowptr[i] = (int)indptr[i];
  // renumber each system's rows by RCM (GPETSC_BATCH_RCM=0 keeps the caller's
  // numbering); values are permuted on the host before the upload
  std::vector<double> pval;
  std::vector<int> perm;
  {
    const char* e = std::getenv("GPETSC_BATCH_RCM");
    if (!(e && std::string(e) == "0") && nnz > 0) {
      perm.resize(n);
      std::vector<int> inv(n), nrp(n + 1, 0), nci(nnz), lrp, lci, lperm;
      std::vector<int64_t> nslot(nnz);
      for (int sy = 0; sy < B->nsys; sy++) {
        const int r0 = B->sys_row[sy], m = B->sys_row[sy + 1] - r0;
        lrp.assign(m + 1, 0);
        lci.clear();
        for (int i = 0; i < m; i++) {
          for (int j = B->h_rowptr[r0 + i]; j < B->h_rowptr[r0 + i + 1]; j++)
            lci.push_back(B->h_colind[j] - r0);
          lrp[i + 1] = (int)lci.size();
        }
        rcm_order(lrp, lci, m, lperm);
        for (int k = 0; k < m; k++) {
          perm[r0 + k] = r0 + lperm[k];
          inv[r0 + lperm[k]] = r0 + k;
        }
      }
      std::vector<std::pair<int, int64_t>> row;
      for (int64_t k = 0; k < n; k++) {
        const int old = perm[k];
        row.clear();
        for (int j = B->h_rowptr[old]; j < B->h_rowptr[old + 1]; j++)
          row.push_back({inv[B->h_colind[j]], j});
        std::sort(row.begin(), row.end());
        nrp[k + 1] = nrp[k] + (int)row.size();
        for (size_t q = 0; q < row.size(); q++) {
          nci[nrp[k] + q] = row[q].first;
          nslot[nrp[k] + q] = row[q].second;
        }
      }
      B->h_rowptr = nrp;
      for (int64_t j = 0; j < nnz; j++) B->h_colind[j] = nci[j];
      std::fill(diag.begin(), diag.end(), -1);
      for (int64_t k = 0; k < n; k++)
        for (int j = nrp[k]; j < nrp[k + 1]; j++)
          if (nci[j] == k) diag[k] = j;
      if (values) {
        pval.resize(nnz);
        for (int64_t j = 0; j < nnz; j++) pval[j] = values[nslot[j]];
      }
    }
  }
  GP_CUDA(cudaGetDevice(&B->device));
  const size_t np = (size_t)nsys * nrhs, nv = (size_t)std::max<int64_t>(n, 1) * nrhs;
  auto fail = [&](int code) {
    batch_destroy(B);
    return code;
  };
#define BT(x)                       \
  do {                              \
    int _s = (x);                   \
    if (_s != GP_OK) return fail(_s); \
  } while (0)
  BT(upload_vec(&B->rowptr, B->h_rowptr, s));
  BT(upload_vec(&B->colind, B->h_colind, s));
  BT(upload_vec(&B->diagpos, diag, s));
  if (cudaMalloc(&B->val, std::max<int64_t>(nnz, 1) * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&B->val32, std::max<int64_t>(nnz, 1) * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&B->dinv, std::max<int64_t>(n, 1) * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&B->dinv32, std::max<int64_t>(n, 1) * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&B->sys_ticket, nsys * sizeof(unsigned)) != cudaSuccess ||
      cudaMalloc(&B->sys_active, nsys * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&B->sys_pairs_left, nsys * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&B->counters, 4 * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&B->pair_d, 9 * np * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&B->pair_i, 6 * np * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&B->r, nv * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&B->p, nv * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&B->z, nv * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&B->x32, nv * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&B->r32, nv * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&B->p32, nv * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&B->z32, nv * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&B->bnorm, np * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&B->rn, np * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    set_error("batched CG: out of device memory");
    return fail(GP_ERR_CUDA);
  }
  if (nnz && values)
    if (cudaMemcpyAsync(B->val, pval.empty() ? values : pval.data(), nnz * sizeof(double),
                        cudaMemcpyHostToDevice, s) != cudaSuccess)
      return fail(GP_ERR_CUDA);
  if (!perm.empty()) {
    BT(upload_vec(&B->perm, perm, s));
    if (cudaMalloc(&B->bp, nv * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&B->xp, nv * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      set_error("batched CG: out of device memory");
      return fail(GP_ERR_CUDA);
    }
  }
  if (cudaMemsetAsync(B->sys_ticket, 0, nsys * sizeof(unsigned), s) != cudaSuccess ||
      cudaMemsetAsync(B->pair_i, 0, 6 * np * sizeof(int), s) != cudaSuccess ||
      cudaMemsetAsync(B->pair_d, 0, 9 * np * sizeof(double), s) != cudaSuccess)
    return fail(GP_ERR_CUDA);
  if (nnz) k_bto_f32<<<num_sms() * 8, 256, 0, s>>>(nnz, B->val, B->val32);
  if (n)
    k_bjacobi<<<std::max(1, std::min((int)((n + 255) / 256), num_sms() * 8)), 256, 0, s>>>(
        (int)n, B->diagpos, B->val, B->dinv, B->dinv32);
  if (cudaGetLastError() != cudaSuccess) return fail(GP_ERR_CUDA);
  BT(build_tiles(*B, B->tune.tile_rows, s));
  if (cudaStreamSynchronize(s) != cudaSuccess) return fail(GP_ERR_CUDA);  // host copies done
#undef BT
  *out = B;
  return GP_OK;
}

// ------------------------------------------------------------ options, tuning
struct BatchOptions {
  int pc = 2;           // 0 none, 2 jacobi
  int precision = 0;    // 0 FP64 CG, 1 FP32 inner CG + FP64 refinement
  int max_it = 10000;   // FP64: CG iterations; refinement: inner iterations per pass
  int max_outer = 20;   // refinement passes
  double rtol = 1e-8, atol = 1e-50, divtol = 1e4;
  double inner_rtol = 1e-4;
};

// Time the sparse pass for every (CTA size, columns per thread, tile rows)
// and keep the fastest: tile rows from the FP64 pass, then the FP64 and the
// FP32 pass each get their own CTA size and width.  State is reset before
// each timing (all systems active).
template <typename T>
static int time_spmm(Batch* B, Tuning* t, int bl, int vr, cudaEvent_t e0, cudaEvent_t e1,
                     cudaStream_t s, float* best_ms) {
  t->block = bl;
  t->vr = vr;
  B->cur = t;
  BatchDev d = dev_view(*B, 1e-8, 1e-50, 1e4, 1, 0);
  *best_ms = 1e30f;
  const T* val = sizeof(T) == 8 ? (const T*)B->val : (const T*)B->val32;
  T* pv = sizeof(T) == 8 ? (T*)B->p : (T*)B->p32;
  T* zv = sizeof(T) == 8 ? (T*)B->z : (T*)B->z32;
  if (sizeof(T) == 4) GP_CUDA(cudaMemsetAsync(B->p32, 0, (size_t)B->n * B->R * sizeof(float), s));
  int st = with_shape(B->R, vr, [&](auto RR, auto VV) {
    for (int rep = 0; rep < 6; rep++) {
      launch_state(*B, d, nullptr, s);
      cudaEventRecord(e0, s);
      launch_spmm<T, decltype(RR)::value, decltype(VV)::value>(*B, d, val, pv, zv, s);
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep >= 2) *best_ms = std::min(*best_ms, ms);
    }
  });
  GP_TRY(st);
  GP_CUDA(cudaGetLastError());
  return GP_OK;
}

int batch_autotune(Batch* B, cudaStream_t s) {
  drop_graphs(*B);
  const int blocks[] = {128, 256, 512};
  const int widths[] = {1, 2, 4};
  const int tiles[] = {128, 512};
  auto ok = [&](int bl, int vr) { return vr <= B->R && B->R % vr == 0 && bl / (B->R / vr) >= 1; };
  cudaEvent_t e0, e1;
  GP_CUDA(cudaEventCreate(&e0));
  GP_CUDA(cudaEventCreate(&e1));
  Tuning best, t;
  best.spmm_us = 1e30;
  for (int tr : tiles) {
    GP_TRY(build_tiles(*B, tr, s));
    for (int bl : blocks)
      for (int vr : widths) {
        if (!ok(bl, vr)) continue;
        float ms;
        GP_TRY(time_spmm<double>(B, &t, bl, vr, e0, e1, s, &ms));
        if (ms * 1e3 < best.spmm_us) {
          best.block = bl;
          best.vr = vr;
          best.tile_rows = tr;
          best.spmm_us = ms * 1e3;
        }
      }
  }
  GP_TRY(build_tiles(*B, best.tile_rows, s));
  Tuning best32 = best;
  best32.spmm_us = 1e30;
  for (int bl : blocks)
    for (int vr : widths) {
      if (!ok(bl, vr)) continue;
      float ms;
      GP_TRY(time_spmm<float>(B, &t, bl, vr, e0, e1, s, &ms));
      if (ms * 1e3 < best32.spmm_us) {
        best32.block = bl;
        best32.vr = vr;
        best32.spmm_us = ms * 1e3;
      }
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  B->tune = best;
  B->tune32 = best32;
  B->cur = &B->tune;
  B->tuned = true;
  return GP_OK;
}

// ------------------------------------------------------------ graph capture
// Capture `prologue`, a WHILE loop over `body` (ending with k_bctrl), then
// `epilogue` into one executable graph.
template <typename P, typename Bd, typename E>
static int capture_loop(Batch& B, cudaStream_t s2, int cap, P&& prologue, Bd&& body,
                        E&& epilogue, cudaGraph_t* g_out, cudaGraphExec_t* x_out) {
  cudaStream_t s = B.cap_stream;
  GP_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
  prologue(s);
  cudaGraph_t graph = nullptr, body_g = nullptr;
  cudaGraphConditionalHandle h = 0;
  cudaStreamCaptureStatus cs;
  const cudaGraphNode_t* deps = nullptr;
  size_t ndeps = 0;
  cudaError_t e = cudaStreamGetCaptureInfo(s, &cs, nullptr, &graph, &deps, nullptr, &ndeps);
  if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault);
  cudaGraphNode_t wnode = nullptr;
  if (e == cudaSuccess) {
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    e = cudaGraphAddNode(&wnode, graph, deps, nullptr, ndeps, &cp);
    if (e == cudaSuccess) body_g = cp.conditional.phGraph_out[0];
  }
  if (e == cudaSuccess)
    e = cudaStreamUpdateCaptureDependencies(s, &wnode, nullptr, 1, cudaStreamSetCaptureDependencies);
  if (e == cudaSuccess)
    e = cudaStreamBeginCaptureToGraph(s2, body_g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
  if (e == cudaSuccess) {
    body(s2);
    k_bctrl<<<1, 1, 0, s2>>>(h, B.counters, B.counters + 1, cap);
    cudaGraph_t bout = nullptr;
    e = cudaStreamEndCapture(s2, &bout);
  }
  if (e == cudaSuccess) epilogue(s);
  cudaGraph_t out = nullptr;
  cudaError_t ec = cudaStreamEndCapture(s, &out);
  if (e == cudaSuccess) e = ec;
  if (e != cudaSuccess) {
    if (out) cudaGraphDestroy(out);
    cudaGetLastError();
    set_error(std::string("batched CG graph capture: ") + cudaGetErrorString(e));
    return GP_ERR_CUDA;
  }
  *g_out = out;
  GP_CUDA(cudaGraphInstantiate(x_out, out, 0));
  return GP_OK;
}

// GPETSC_KSP_GRAPH=0: the same prologue / body / epilogue launched from the
// host, the loop polled every 8 trips (the form ncu profiles kernel by kernel).
static bool batch_eager() {
  static bool v = [] {
    const char* e = std::getenv("GPETSC_KSP_GRAPH");
    return e && std::string(e) == "0";
  }();
  return v;
}

template <typename P, typename Bd, typename E>
static int run_eager_loop(Batch& B, cudaStream_t s, int cap, P&& prologue, Bd&& body,
                          E&& epilogue) {
  prologue(s);
  for (int trip = 1;; trip++) {
    body(s);
    k_btrip<<<1, 1, 0, s>>>(B.counters + 1);
    if (trip % 8 == 0 || trip >= cap) {
      int c[2] = {0, 0};
      GP_CUDA(cudaMemcpyAsync(c, B.counters, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
      GP_CUDA(cudaStreamSynchronize(s));
      if (c[0] == 0 || c[1] >= cap) break;
    }
  }
  epilogue(s);
  GP_CUDA(cudaGetLastError());
  return GP_OK;
}

// Run the loop: re-use the captured graph in `slot` when its key matches,
// else capture it (or, in the host-driven mode, launch everything directly).
template <typename P, typename Bd, typename E>
static int run_loop(Batch& B, int slot, cudaStream_t s2, const double* b, double* x,
                    const double (&key)[10], int cap, P&& prologue, Bd&& body, E&& epilogue) {
  cudaStream_t s = B.cap_stream;
  if (batch_eager()) return run_eager_loop(B, s, cap, prologue, body, epilogue);
  const bool same = B.exec[slot] && B.cap_b[slot] == b && B.cap_x[slot] == x &&
                    std::equal(key, key + 10, B.cap_key[slot]);
  if (!same) {
    if (B.exec[slot]) cudaGraphExecDestroy(B.exec[slot]);
    if (B.graph[slot]) cudaGraphDestroy(B.graph[slot]);
    B.exec[slot] = nullptr;
    B.graph[slot] = nullptr;
    GP_TRY(capture_loop(B, s2, cap, prologue, body, epilogue, &B.graph[slot], &B.exec[slot]));
    B.cap_b[slot] = b;
    B.cap_x[slot] = x;
    std::copy(key, key + 10, B.cap_key[slot]);
  }
  GP_CUDA(cudaGraphLaunch(B.exec[slot], s));
  return GP_OK;
}

struct BatchResult {
  std::vector<int> its, reason;
  std::vector<double> relres;
  int outer = 0;
};

template <int R, int VR>
static int solve_shape(Batch& B, const BatchOptions& o, const double* b, double* x,
                       cudaStream_t caller, BatchResult& res) {
  static thread_local cudaStream_t s2 = nullptr;
  if (!B.cap_stream) GP_CUDA(cudaStreamCreateWithFlags(&B.cap_stream, cudaStreamNonBlocking));
  if (!s2) GP_CUDA(cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking));
  cudaStream_t s = B.cap_stream;
  cudaEvent_t ev;
  GP_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  GP_CUDA(cudaEventRecord(ev, caller));
  GP_CUDA(cudaStreamWaitEvent(s, ev, 0));
  const size_t nv = (size_t)B.n * R, np = (size_t)B.nsys * R;
  const BatchDev d64 = dev_view(B, o.rtol, o.atol, o.divtol, o.max_it, o.pc);
  const double* dinv = o.pc == 2 ? B.dinv : nullptr;
  const float* dinv32 = o.pc == 2 ? B.dinv32 : nullptr;
  // every value a captured kernel received by value
  const double key[10] = {(double)o.pc,      (double)o.max_it,     o.rtol,
                          o.atol,            o.divtol,             o.inner_rtol,
                          (double)B.cur->block, (double)B.cur->vr, (double)B.tune.tile_rows,
                          (double)B.ntiles};
  int* refined = refined_of(B);
  int* its_total = its_total_of(B);
  auto norms = [&](cudaStream_t st) {
    auto k = k_bnorm<R>;
    Launch l = shape_of<double, R, 1, 1>(B, (const void*)k);
    k<<<l.grid, l.block, l.smem, st>>>(d64, b, B.bnorm);
  };
  if (o.precision == 0 && o.pc == 6) {
    // IC(0): the update leaves z alone; z = M^-1 r, then the pair dots
    auto icc = [&](cudaStream_t st) {
      return pc_apply_icc_cols(B.icc, R, B.r, B.z, B.icc_vf, B.icc_vb, B.icc_ys, st);
    };
    int pst = GP_OK;
    GP_TRY(run_loop(
          B, 0, s2, b, x, key, o.max_it + 8,
          [&](cudaStream_t st) {
            cudaMemsetAsync(B.counters, 0, 2 * sizeof(int), st);
            cudaMemsetAsync(x, 0, nv * sizeof(double), st);
            cudaMemcpyAsync(B.r, b, nv * sizeof(double), cudaMemcpyDeviceToDevice, st);
            norms(st);
            launch_state(B, d64, nullptr, st);
            if (pst == GP_OK) pst = icc(st);
            launch_dots<R, true>(B, d64, B.r, B.z, st);
          },
          [&](cudaStream_t st) {
            launch_p<double, R>(B, d64, B.p, B.z, st);
            launch_spmm<double, R, VR>(B, d64, B.val, B.p, B.z, st);  // W shares Z's storage
            launch_update_xr<R>(B, d64, x, B.r, B.p, B.z, st);
            if (pst == GP_OK) pst = icc(st);
            launch_dots<R, false>(B, d64, B.r, B.z, st);
          },
          [&](cudaStream_t st) { launch_resid<R, VR>(B, d64, b, x, 0, st); }));
    GP_TRY(pst);
    GP_TRY(pc_check(B.icc, s));
  } else if (o.precision == 0) {
    GP_TRY(run_loop(
          B, 0, s2, b, x, key, o.max_it + 8,
          [&](cudaStream_t st) {
            cudaMemsetAsync(B.counters, 0, 2 * sizeof(int), st);
            cudaMemsetAsync(x, 0, nv * sizeof(double), st);
            cudaMemcpyAsync(B.r, b, nv * sizeof(double), cudaMemcpyDeviceToDevice, st);
            norms(st);
            launch_state(B, d64, nullptr, st);
            launch_update<double, R, 1, true>(B, d64, dinv, x, B.r, B.p, B.z, B.z, st);
          },
          [&](cudaStream_t st) {
            launch_p<double, R>(B, d64, B.p, B.z, st);
            launch_spmm<double, R, VR>(B, d64, B.val, B.p, B.z, st);  // W shares Z's storage
            launch_update<double, R, 1, false>(B, d64, dinv, x, B.r, B.p, B.z, B.z, st);
          },
          [&](cudaStream_t st) { launch_resid<R, VR>(B, d64, b, x, 0, st); }));
  } else {
    // FP32 inner CG on A d = r / ||r||, x += ||r|| d, until ||b - A x|| <= rtol ||b||
    const BatchDev d32 = dev_view(B, o.inner_rtol, 1e-30, 1e30, o.max_it, o.pc);
    auto pass = [&]() {
      return run_loop(
          B, 1, s2, b, x, key, o.max_it + 8,
          [&](cudaStream_t st) {
            cudaMemsetAsync(B.counters, 0, 2 * sizeof(int), st);
            launch_state(B, d32, refined, st);
            auto ks = k_bscale_in<R>;
            const int g = std::max(1, std::min(B.ntiles, resident((const void*)ks, B.cur->block, 0)));
            ks<<<g, B.cur->block, 0, st>>>(d32, B.r, B.rn, B.r32, B.x32);
            launch_update<float, R, 1, true>(B, d32, dinv32, B.x32, B.r32, B.p32, B.z32, B.z32,
                                              st);
          },
          [&](cudaStream_t st) {
            launch_p<float, R>(B, d32, B.p32, B.z32, st);
            launch_spmm<float, R, VR>(B, d32, B.val32, B.p32, B.z32, st);
            launch_update<float, R, 1, false>(B, d32, dinv32, B.x32, B.r32, B.p32, B.z32,
                                               B.z32, st);
          },
          [&](cudaStream_t st) {
            k_bsum_its<<<std::max(1, (int)std::min<size_t>((np + 255) / 256, 1024)), 256, 0, st>>>(
                (int)np, d32.its, its_total);
            launch_state(B, d64, refined, st);
            auto ka = k_bacc<R>;
            const int g = std::max(1, std::min(B.ntiles, resident((const void*)ka, B.cur->block, 0)));
            ka<<<g, B.cur->block, 0, st>>>(d64, refined, B.rn, B.x32, x);
            launch_resid<R, VR>(B, d64, b, x, 1, st);
            cudaMemcpyAsync(refined, d64.active, np * sizeof(int), cudaMemcpyDeviceToDevice, st);
          });
    };
    // first pass: r = b, rn = ||b||, pairs with b = 0 frozen
    GP_CUDA(cudaMemsetAsync(x, 0, nv * sizeof(double), s));
    GP_CUDA(cudaMemsetAsync(its_total, 0, np * sizeof(int), s));
    norms(s);
    launch_state(B, d64, nullptr, s);
    launch_resid<R, VR>(B, d64, b, x, 1, s);
    GP_CUDA(cudaMemcpyAsync(refined, d64.active, np * sizeof(int), cudaMemcpyDeviceToDevice, s));
    GP_CUDA(cudaGetLastError());
    for (res.outer = 0; res.outer < o.max_outer; res.outer++) {
      int left = 0;
      GP_CUDA(cudaMemcpyAsync(&left, B.counters, sizeof(int), cudaMemcpyDeviceToHost, s));
      GP_CUDA(cudaStreamSynchronize(s));
      if (left == 0) break;
      GP_TRY(pass());
    }
    launch_resid<R, VR>(B, d64, b, x, 0, s);
  }
  GP_CUDA(cudaGetLastError());
  // results
  std::vector<double> rn(np), bn(np);
  res.its.assign(np, 0);
  res.reason.assign(np, 0);
  res.relres.assign(np, 0.0);
  GP_CUDA(cudaMemcpyAsync(rn.data(), B.rn, np * sizeof(double), cudaMemcpyDeviceToHost, s));
  GP_CUDA(cudaMemcpyAsync(bn.data(), B.bnorm, np * sizeof(double), cudaMemcpyDeviceToHost, s));
  GP_CUDA(cudaMemcpyAsync(res.its.data(), o.precision ? its_total : d64.its, np * sizeof(int),
                          cudaMemcpyDeviceToHost, s));
  GP_CUDA(cudaMemcpyAsync(res.reason.data(), d64.reason, np * sizeof(int),
                          cudaMemcpyDeviceToHost, s));
  GP_CUDA(cudaStreamSynchronize(s));
  GP_CUDA(cudaEventRecord(ev, s));
  GP_CUDA(cudaStreamWaitEvent(caller, ev, 0));
  cudaEventDestroy(ev);
  for (size_t q = 0; q < np; q++) {
    res.relres[q] = bn[q] > 0.0 ? rn[q] / bn[q] : rn[q];
    if (o.precision) res.reason[q] = res.relres[q] <= o.rtol ? BR_RTOL : BR_ITS;
  }
  return GP_OK;
}

int batch_solve(Batch* B, const BatchOptions& o, const double* b, double* x, cudaStream_t s,
                BatchResult& res) {
  if (o.pc != 0 && o.pc != 2 && o.pc != 6) {
    set_error("batched CG: preconditioner must be none (0), jacobi (2) or icc (6)");
    return GP_ERR_UNSUPPORTED;
  }
  if (o.pc == 6 && o.precision != 0) {
    set_error("batched CG: icc(0) runs in the FP64 form (precision 0)");
    return GP_ERR_UNSUPPORTED;
  }
  if (o.pc == 6) GP_TRY(batch_icc_setup(*B, s));
  if (o.max_it < 1 || o.max_outer < 1 || !(o.rtol >= 0.0)) {
    set_error("batched CG: bad tolerances");
    return GP_ERR_ARG;
  }
  int st = GP_OK;
  B->cur = o.precision ? &B->tune32 : &B->tune;
  const double* bs = b;
  double* xs = x;
  const int g = std::max(1, std::min((int)(((int64_t)B->n * B->R + 255) / 256), num_sms() * 8));
  if (B->perm && B->n) {  // into the renumbered rows
    k_brows_permute<<<g, 256, 0, s>>>(B->n, B->R, B->perm, 0, b, B->bp);
    k_brows_permute<<<g, 256, 0, s>>>(B->n, B->R, B->perm, 0, x, B->xp);
    GP_CHECK_LAUNCH();
    bs = B->bp;
    xs = B->xp;
  }
  int r = with_shape(B->R, B->cur->vr, [&](auto RR, auto VV) {
    st = solve_shape<decltype(RR)::value, decltype(VV)::value>(*B, o, bs, xs, s, res);
  });
  GP_TRY(r);
  if (st == GP_OK && B->perm && B->n) {  // back to the caller's numbering
    k_brows_permute<<<g, 256, 0, s>>>(B->n, B->R, B->perm, 1, B->xp, x);
    GP_CHECK_LAUNCH();
  }
  return st;
}

}  // namespace gp

// ------------------------------------------------------------------- C ABI
struct gp_batch_s {
  gp::Batch* B;
};

extern "C" {

void gp_batch_options_default(gp_batch_options* o) {
  gp::BatchOptions d;
  std::memset(o, 0, sizeof(*o));
  o->pc_type = d.pc;
  o->precision = d.precision;
  o->max_it = d.max_it;
  o->max_outer = d.max_outer;
  o->rtol = d.rtol;
  o->atol = d.atol;
  o->divtol = d.divtol;
  o->inner_rtol = d.inner_rtol;
}

int gp_batch_create(gp_batch* out, int64_t nsys, const int64_t* sys_rows, const int64_t* indptr,
                    const int64_t* indices, const double* values, int32_t nrhs, void* stream) {
  if (!out) {
    gp::set_error("gp_batch_create: null argument");
    return GP_ERR_ARG;
  }
  try {
    gp::Batch* B = nullptr;
    int st = gp::batch_create(&B, nsys, sys_rows, indptr, indices, values, nrhs,
                              static_cast<cudaStream_t>(stream));
    if (st) return st;
    *out = new gp_batch_s{B};
    return GP_OK;
  } catch (const std::exception& e) {
    gp::set_error(std::string("gp_batch_create: ") + e.what());
    return GP_ERR_INTERNAL;
  }
}

int gp_batch_destroy(gp_batch b) {
  if (!b) return GP_OK;
  gp::batch_destroy(b->B);
  delete b;
  return GP_OK;
}

int gp_batch_autotune(gp_batch b, void* stream) {
  if (!b) {
    gp::set_error("gp_batch_autotune: null argument");
    return GP_ERR_ARG;
  }
  try {
    return gp::batch_autotune(b->B, static_cast<cudaStream_t>(stream));
  } catch (const std::exception& e) {
    gp::set_error(std::string("gp_batch_autotune: ") + e.what());
    return GP_ERR_INTERNAL;
  }
}

int gp_batch_tuning(gp_batch b, int32_t precision, int32_t* block, int32_t* vector_width,
                    int32_t* tile_rows, double* spmm_us) {
  if (!b) {
    gp::set_error("gp_batch_tuning: null argument");
    return GP_ERR_ARG;
  }
  const gp::Tuning& t = precision ? b->B->tune32 : b->B->tune;
  if (block) *block = t.block;
  if (vector_width) *vector_width = t.vr;
  if (tile_rows) *tile_rows = t.tile_rows;
  if (spmm_us) *spmm_us = t.spmm_us;
  return GP_OK;
}

int gp_batch_solve_cg(gp_batch b, const gp_batch_options* o, const double* B, double* X,
                      int64_t* its, int32_t* reason, double* relres, int32_t* passes,
                      void* stream) {
  if (!b || !o || (b->B->n && (!B || !X))) {
    gp::set_error("gp_batch_solve_cg: null argument");
    return GP_ERR_ARG;
  }
  if (B == X) {
    gp::set_error("gp_batch_solve_cg: X may not alias B");
    return GP_ERR_ARG;
  }
  try {
    gp::BatchOptions bo;
    bo.pc = o->pc_type;
    bo.precision = o->precision;
    bo.max_it = o->max_it;
    bo.max_outer = o->max_outer;
    bo.rtol = o->rtol;
    bo.atol = o->atol;
    bo.divtol = o->divtol;
    bo.inner_rtol = o->inner_rtol;
    gp::BatchResult res;
    int st = gp::batch_solve(b->B, bo, B, X, static_cast<cudaStream_t>(stream), res);
    if (st) return st;
    for (size_t q = 0; q < res.its.size(); q++) {
      if (its) its[q] = res.its[q];
      if (reason) reason[q] = res.reason[q];
      if (relres) relres[q] = res.relres[q];
    }
    if (passes) *passes = res.outer;
    return GP_OK;
  } catch (const std::exception& e) {
    gp::set_error(std::string("gp_batch_solve_cg: ") + e.what());
    return GP_ERR_INTERNAL;
  }
}

}  // extern "C"
