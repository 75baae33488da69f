// Device-resident Krylov drivers.
//
//   KSPConvergedDefault          src/ksp.mojo:96-152   -> conv_default()
//   KSP_PCApply / BAorAB / ...   src/ksp.mojo:155-265  -> pc_apply / apply_ba()
//   KSPSolve_CG                  src/ksp.mojo:271-389  -> solve_cg()
//   KSPSolve_BCGS                src/ksp.mojo:395-505  -> solve_bcgs()
//   KSPSolve_GMRES (+CGS, UpdateHessenberg, BuildSoln)  src/ksp.mojo:533-769
//   KSPSolve_FGMRES              src/ksp.mojo:775-903
//
// Every scalar of the iteration (alpha, beta, the residual norm, the
// Hessenberg matrix and its Givens rotations, the converged reason) lives in
// device memory.  The vector work of one iteration is captured once into the
// body of a CUDA-graph WHILE node; small single-thread "control" kernels carry
// the reference's scalar logic and branch structure and set the gate words
// that switch the following vector kernels on or off.  The whole solve is one
// graph launch with no host round trip; the control kernel at the end of the
// body sets the loop condition from the device state, with a hard cap on the
// number of trips so the loop always ends.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "gp_ksp.h"
#include "gp_ordred.cuh"
#include "gp_spmv.cuh"

namespace gp {

enum Reason : int {
  R_RTOL = 2, R_ATOL = 3, R_ITS = 4, R_HAPPY = 7, R_NULL = -2, R_DIVITS = -3, R_DTOL = -4,
  R_BREAKDOWN = -5, R_INDEF_PC = -8, R_NANORINF = -9, R_INDEF_MAT = -10
};
enum Norm : int { N_NONE = 1, N_PRECOND = 2, N_UNPRECOND = 3, N_NATURAL = 4 };
enum Phase : int { PH_DONE = 0, PH_RESTART = 1, PH_STEP = 2, PH_BUILD = 3 };

// KSPConvergedDefault, src/ksp.mojo:96-152.
__device__ int conv_default(KspState* st, int n, double rnorm) {
  if (st->convmaxits && n >= st->max_it) return R_ITS;
  if (st->normtype == N_NONE) return 0;
  if (!n && !st->seeded) {
    double rnorm0 = rnorm;
    if (st->seed_rhs) {
      double snorm = st->rhs_norm;
      if (!snorm) snorm = rnorm;
      rnorm0 = snorm;
    }
    st->rnorm0 = rnorm0;
    const double ttol = mul(st->rtol, rnorm0);
    st->ttol = ttol > st->atol ? ttol : st->atol;
    st->seeded = 1;
  }
  if (n <= st->chknorm) return 0;
  if (rnorm != rnorm || fabs(rnorm) == INFINITY) return R_NANORINF;
  if (n < st->min_it) return 0;
  if (rnorm <= st->ttol) {
    if (rnorm < st->atol) return R_ATOL;
    return R_RTOL;
  }
  if (rnorm >= mul(st->divtol, st->rnorm0)) return R_DTOL;
  return 0;
}

// Launch a kernel templated on the arithmetic (see Arith in gp_common.cuh).
#define FL(K, G, B, S, ...)                                   \
  do {                                                        \
    if (arith_mode() == kFma)                                 \
      K<true><<<(G), (B), 0, (S)>>>(__VA_ARGS__);             \
    else                                                      \
      K<false><<<(G), (B), 0, (S)>>>(__VA_ARGS__);            \
  } while (0)

// ------------------------------------------------------------ vector kernels
static int vgrid(int n) { return std::max(1, std::min((n + 255) / 256, num_sms() * 8)); }

#define GRID_LOOP(i, n)                                                          \
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += gridDim.x * blockDim.x)

// y_i = f(a_i, b_i, c_i) over NIN inputs, in batched passes (grid_batched):
// all loads of a pass before its stores; an input may be the output itself.
template <int NIN, typename F>
__device__ __forceinline__ void ew(int n, double* y, F f, const double* a,
                                   const double* b = nullptr, const double* c = nullptr) {
  constexpr int U = kVecBatch;
  double av[U], bv[U] = {}, cv[U] = {};
  grid_batched<U>(
      n,
      [&](int u, unsigned i) {
        av[u] = a[i];
        if constexpr (NIN > 1) bv[u] = b[i];
        if constexpr (NIN > 2) cv[u] = c[i];
      },
      [&](int u, unsigned i) {
        y[i] = f(av[u], bv[u], cv[u]);
      });
}

constexpr int kBodyUnroll = 1;    // default loop-body copies per graph trip
constexpr int kBodyUnrollCg = 8;  // the same for the fused CG body
constexpr int kEagerPoll = 8;   // host-driven loop: trips between state polls

__global__ void k_copy_d(const int* gate, int want, int n, DRef xr, DRef yr) {
  if (gated_off(gate, want)) return;
  ew<1>(n, yr.get(), [](double a, double, double) { return a; }, xr.get());
}

__global__ void k_zero_d(const int* gate, int want, int n, DRef yr) {
  if (gated_off(gate, want)) return;
  double* y = yr.get();
  GRID_LOOP(i, n) y[i] = 0.0;
}

// y = y + (sgn * a) x      (VecAXPY with a device scalar)
template <bool FMA>
__global__ void k_axpy_d(const int* gate, int want, int n, DRef yr, const double* a, double sgn,
                         DRef xr) {
  if (gated_off(gate, want)) return;
  double* y = yr.get();
  const double al = mul(sgn, *a);
  ew<2>(n, y, [=](double xv, double yv, double) { return madd<FMA>(al, xv, yv); }, xr.get(), y);
}

// y = x + alpha y (VecAYPX, general branch) with a host scalar
template <bool FMA>
__global__ void k_aypx_h(const int* gate, int want, int n, DRef yr, double alpha, DRef xr) {
  if (gated_off(gate, want)) return;
  double* y = yr.get();
  ew<2>(n, y, [=](double yv, double xv, double) { return madd<FMA>(alpha, yv, xv); }, y,
        xr.get());
}

// VecAYPX(y, *a, x) with the reference's branch structure decided on the
// device: a == 0 copies, a == 1 adds, otherwise x + a y.
template <bool FMA>
__global__ void k_aypx_d(const int* gate, int want, int n, DRef yr, const double* a, DRef xr) {
  if (gated_off(gate, want)) return;
  double* y = yr.get();
  const double* x = xr.get();
  const double al = *a;
  if (al == 0.0)
    ew<1>(n, y, [](double xv, double, double) { return xv; }, x);
  else if (al == 1.0)
    ew<2>(n, y, [=](double xv, double yv, double) { return madd<FMA>(al, xv, yv); }, x, y);
  else
    ew<2>(n, y, [=](double yv, double xv, double) { return madd<FMA>(al, yv, xv); }, y, x);
}

// z = a x + b y + c z      (VecAXPBYPCZ with device scalars)
template <bool FMA>
__global__ void k_axpbypcz_d(const int* gate, int want, int n, DRef zr, const double* a,
                             const double* b, const double* c, DRef xr, DRef yr) {
  if (gated_off(gate, want)) return;
  double* z = zr.get();
  const double al = *a, be = *b, ga = *c;
  ew<3>(
      n, z,
      [=](double zv, double yv, double xv) {
        return madd<FMA>(ga, zv, madd<FMA>(be, yv, mul(al, xv)));
      },
      z, yr.get(), xr.get());
}

// w = (sgn * a) x + y      (VecWAXPY)
template <bool FMA>
__global__ void k_waxpy_d(const int* gate, int want, int n, DRef wr, const double* a, double sgn,
                          DRef xr, DRef yr) {
  if (gated_off(gate, want)) return;
  const double al = mul(sgn, *a);
  ew<2>(n, wr.get(), [=](double xv, double yv, double) { return madd<FMA>(al, xv, yv); },
        xr.get(), yr.get());
}

// x = x * (*a)   (VecScale)  or  x = x / (*a) when *a > 0 (VecNormalize)
template <bool DIVIDE>
__global__ void k_scale_d(const int* gate, int want, int n, DRef xr, const double* a) {
  if (gated_off(gate, want)) return;
  double* x = xr.get();
  const double al = *a;
  if (DIVIDE) {
    if (!(al > 0.0)) return;
    ew<1>(n, x, [=](double xv, double, double) { return div_(xv, al); }, x);
  } else {
    ew<1>(n, x, [=](double xv, double, double) { return mul(xv, al); }, x);
  }
}

// CG update: x = x + a p; r = r + (-a) w
template <bool FMA>
__global__ void k_cg_xr(const int* gate, int want, int n, double* __restrict__ x,
                        double* __restrict__ r, const double* __restrict__ p,
                        const double* __restrict__ w, const double* a) {
  if (gated_off(gate, want)) return;
  const double al = *a, nal = -al;
  constexpr int U = kVecBatch;
  double pv[U], xv[U], wv[U], rv[U];
  grid_batched<U>(
      n,
      [&](int u, unsigned i) {
        pv[u] = p[i];
        xv[u] = x[i];
        wv[u] = w[i];
        rv[u] = r[i];
      },
      [&](int u, unsigned i) {
        x[i] = madd<FMA>(al, pv[u], xv[u]);
        r[i] = madd<FMA>(nal, wv[u], rv[u]);
      });
}

// ------------------------------------------------------------ reductions
enum DRed : int { D_DOT, D_NRM, D_DOTNRM };

// Deterministic reduction into device scalars: out_raw receives the sum,
// out_sqrt receives sqrt(|sum|) (the 2-norm, or sqrt|beta| for the natural
// norm).  D_DOTNRM writes (x.y, x.x) to out_raw[0], out_raw2.
template <int OP, bool FMA>
__global__ void __launch_bounds__(kRedBlock) k_dred(const int* gate, int want, int n, DRef xr,
                                                    DRef yr, RedSlot slot, double* out_raw,
                                                    double* out_sqrt, double* out_raw2) {
  if (gated_off(gate, want)) return;
  constexpr int NR = OP == D_DOTNRM ? 2 : 1;
  const double* __restrict__ x = xr.get();
  const double* __restrict__ y = OP == D_NRM ? x : yr.get();
  double v[NR];
#pragma unroll
  for (int r = 0; r < NR; r++) v[r] = 0.0;
  constexpr int U = kVecBatch;
  double xv[U], yv[U];
  grid_batched<U>(
      n,
      [&](int u, unsigned i) {
        xv[u] = x[i];
        yv[u] = OP == D_NRM ? xv[u] : y[i];
      },
      [&](int u, unsigned) {
        v[0] = madd<FMA>(xv[u], yv[u], v[0]);
        if (OP == D_DOTNRM) v[NR - 1] = madd<FMA>(xv[u], xv[u], v[NR - 1]);
      });
  double tot[NR];
  if (grid_finish<NR>(v, slot, tot) && threadIdx.x == 0) {
    if (out_raw) *out_raw = tot[0];
    if (out_sqrt) *out_sqrt = __dsqrt_rn(fabs(tot[0]));
    if (OP == D_DOTNRM && out_raw2) *out_raw2 = tot[NR - 1];
  }
}

// One batch of the multi-dot: v[q] += sum_i x_i basis_q,i for q < JN, over
// the grid-stride elements of this thread.
template <bool FMA, int JN>
__device__ __forceinline__ void mdot_batch(int n, const double* __restrict__ x,
                                           const double* __restrict__ basis, double (&v)[8]) {
  GRID_LOOP(i, n) {
    const double a = x[i];
#pragma unroll
    for (int q = 0; q < JN; q++) v[q] = madd<FMA>(a, basis[(size_t)q * n + i], v[q]);
  }
}

// VecMDot of x against `*count` contiguous basis vectors (ld = n): one pass
// over x and the basis, per-block partial sums for every vector, last block
// folds the partials.  Used by classical Gram-Schmidt.
constexpr int kMaxBasis = 64;
template <bool FMA>
__global__ void __launch_bounds__(kRedBlock) k_mdot(const int* gate, int want, int n, DRef xr,
                                                    const double* __restrict__ basis,
                                                    const int* count, RedSlot slot,
                                                    double* __restrict__ out) {
  if (gated_off(gate, want)) return;
  const double* __restrict__ x = xr.get();
  const int k = *count;
  __shared__ double sh[kRedBlock / 32][kMaxBasis];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int j0 = 0; j0 < k; j0 += 8) {
    double v[8];
#pragma unroll
    for (int q = 0; q < 8; q++) v[q] = 0.0;
    const int jn = min(8, k - j0);
    // the batch's width is the same in every thread: a body unrolled for
    // exactly jn dots, so a partial batch issues no predicated-off FMAs
    // (each would hold the FP64 unit for a full warp instruction)
    switch (jn) {
      case 1: mdot_batch<FMA, 1>(n, x, basis + (size_t)j0 * n, v); break;
      case 2: mdot_batch<FMA, 2>(n, x, basis + (size_t)j0 * n, v); break;
      case 3: mdot_batch<FMA, 3>(n, x, basis + (size_t)j0 * n, v); break;
      case 4: mdot_batch<FMA, 4>(n, x, basis + (size_t)j0 * n, v); break;
      case 5: mdot_batch<FMA, 5>(n, x, basis + (size_t)j0 * n, v); break;
      case 6: mdot_batch<FMA, 6>(n, x, basis + (size_t)j0 * n, v); break;
      case 7: mdot_batch<FMA, 7>(n, x, basis + (size_t)j0 * n, v); break;
      default: mdot_batch<FMA, 8>(n, x, basis + (size_t)j0 * n, v); break;
    }
    // warp sums of the 8 values by halving exchanges: at offset 16 a lane
    // keeps the half of the values its lane bit selects and adds its
    // partner's copy of that half (4 adds), then 2 at offset 8, 1 at offset
    // 4, and a plain pair of steps at 2 and 1 -- 9 FP64 adds a lane instead
    // of 8 shuffle trees of 5; lane 4 q' ends with value q' = the bits
    // (lane >> 2) read high to low.
    {
      const bool h4 = lane & 16, h3 = lane & 8, h2 = lane & 4;
      double u4[4], u2[2];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const double keep = h4 ? v[q + 4] : v[q], send = h4 ? v[q] : v[q + 4];
        u4[q] = add(keep, __shfl_xor_sync(0xffffffffu, send, 16));
      }
#pragma unroll
      for (int q = 0; q < 2; q++) {
        const double keep = h3 ? u4[q + 2] : u4[q], send = h3 ? u4[q] : u4[q + 2];
        u2[q] = add(keep, __shfl_xor_sync(0xffffffffu, send, 8));
      }
      double t;
      {
        const double keep = h2 ? u2[1] : u2[0], send = h2 ? u2[0] : u2[1];
        t = add(keep, __shfl_xor_sync(0xffffffffu, send, 4));
      }
      t = add(t, __shfl_xor_sync(0xffffffffu, t, 2));
      t = add(t, __shfl_xor_sync(0xffffffffu, t, 1));
      const int q = (h4 ? 4 : 0) + (h3 ? 2 : 0) + (h2 ? 1 : 0);
      if ((lane & 3) == 0 && q < jn) sh[wid][j0 + q] = t;
    }
  }
  __syncthreads();
  if (threadIdx.x < k) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t = add(t, sh[w][threadIdx.x]);
    slot.partials[(size_t)threadIdx.x * slot.stride + blockIdx.x] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) last = atomic_add_acq_rel(slot.ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  // warp w folds dots w, w + nwarps, ...: lanes take blocks lane, lane + 32,
  // ... in order (many loads in flight), then a shuffle tree -- a fixed order
  // without a serial chain over every block
  {
    const int nw = blockDim.x >> 5;
    for (int j = wid; j < k; j += nw) {
      double t = 0.0;
      for (int b = lane; b < (int)gridDim.x; b += 32)
        t = add(t, __ldcg(&slot.partials[(size_t)j * slot.stride + b]));
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) t = add(t, __shfl_down_sync(0xffffffffu, t, o));
      if (lane == 0) out[j] = t;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) *slot.ticket = 0u;
}

// y = (from_zero ? 0 : y) + sum_{j < *count} coef_j basis_j, ascending j per
// element (simdvec.maxpy, VecMAXPBY with beta = 0).
template <bool FMA>
__global__ void k_maxpy_dyn(const int* gate, int want, int n, DRef yr,
                            const double* __restrict__ basis, const double* __restrict__ coef,
                            const int* count, int from_zero) {
  if (gated_off(gate, want)) return;
  double* __restrict__ y = yr.get();
  const int k = *count;
  GRID_LOOP(i, n) {
    double v = from_zero ? 0.0 : y[i];
    for (int j = 0; j < k; j++) v = madd<FMA>(coef[j], basis[(size_t)j * n + i], v);
    y[i] = v;
  }
}

// ------------------------------------------------------------ loop control
constexpr int G_ON = 5;  // g[G_ON] == 1 while the driver runs

__device__ __forceinline__ void finish(KspState* st, double rnorm, int its, int reason) {
  st->rnorm = rnorm;
  st->its = its;
  st->reason = reason;
}

// Record the result and switch every gate of the loop body off.
__device__ __forceinline__ void stop(KspState* st, double rnorm, int its, int reason) {
  finish(st, rnorm, its, reason);
  st->active = 0;
  st->phase = PH_DONE;
#pragma unroll
  for (int k = 0; k < 16; k++) st->g[k] = 0;
}

// End of the loop body: keep looping while the driver is active and under the
// trip cap (every driver needs at most one trip per iteration, plus restarts).
__device__ __forceinline__ bool loop_trip(KspState* st) {
  st->trips += 1;
  const bool run = st->active == 1;
  const int cap = st->max_it * 2 + 64;
  if (run && st->trips >= cap) stop(st, st->rnorm, st->its, st->reason ? st->reason : R_DIVITS);
  return run && st->trips < cap;
}

__global__ void k_loop_ctrl(cudaGraphConditionalHandle h, KspState* st) {
  pdl_wait();
  cudaGraphSetConditional(h, loop_trip(st) ? 1u : 0u);
}

// host-driven loop: the same bookkeeping without the graph conditional
__global__ void k_loop_trip(KspState* st) { loop_trip(st); }

// ================================================================== CG
// gates: g[0] PC + ||z|| after the update, g[3] ||r||, g[4] natural norm,
//        g[1] PC after the test, g[2] recompute beta, g[5] on
__global__ void k_cg_init(KspState* st, double* hist) {
  const double dp = st->dp;
  hist[0] = dp;
  const int reason = conv_default(st, 0, dp);
  st->i = 0;
  st->dpi = 0.0;
  st->betaold = 1.0;
  if (reason) {
    stop(st, dp, 0, reason);
    return;
  }
  st->active = 1;
  const int nt = st->normtype;
  st->g[G_ON] = 1;
  st->g[1] = (nt != N_PRECOND && nt != N_NATURAL) ? 1 : 0;
  st->g[2] = (nt != N_NATURAL) ? 1 : 0;
  st->g[0] = st->g[3] = st->g[4] = 0;
}

// top of iteration i: breakdown tests, the beta/betaold ratio, dpiold
__global__ void k_cg_a(KspState* st) {
  if (st->active != 1) return;
  const int i = st->i;
  st->its = i + 1;
  const double beta = st->beta;
  if (beta == 0.0) {
    stop(st, st->dp, i + 1, R_ATOL);
    return;
  }
  if (i > 0 && mul(beta, st->betaold) < 0.0) {
    stop(st, st->dp, i + 1, R_INDEF_PC);
    return;
  }
  st->bcoef = i == 0 ? 0.0 : div_(beta, st->betaold);
  st->dpiold = st->dpi;
}

__device__ __forceinline__ int sgn(double x) { return x < 0.0 ? -1 : (x == 0.0 ? 0 : 1); }

// after dpi = p.Ap: indefinite-matrix test and a = beta / dpi
__global__ void k_cg_b(KspState* st) {
  if (st->active != 1) return;
  const int i = st->i;
  const double dpi = st->dpi;
  st->betaold = st->beta;
  if (dpi == 0.0 || (i > 0 && sgn(dpi) * sgn(st->dpiold) < 0)) {
    stop(st, st->dp, i + 1, R_INDEF_MAT);
    return;
  }
  st->a = div_(st->beta, dpi);
  const int nt = st->normtype;
  const bool now = st->chknorm < i + 2;
  st->g[0] = (nt == N_PRECOND && now) ? 1 : 0;
  st->g[3] = (nt == N_UNPRECOND && now) ? 1 : 0;
  st->g[4] = (nt == N_NATURAL) ? 1 : 0;
  if (!(st->g[0] || st->g[3] || st->g[4])) st->dp = 0.0;
}

// residual norm recorded, convergence test, gates for the tail of the body
__global__ void k_cg_c(KspState* st, double* hist) {
  if (st->active != 1) return;
  const int i = st->i, its = i + 1;
  const double dp = st->dp;
  hist[its] = dp;
  const int reason = conv_default(st, its, dp);
  if (reason) {
    stop(st, dp, its, reason);
    return;
  }
  const int nt = st->normtype;
  st->g[1] = ((nt != N_PRECOND && nt != N_NATURAL) || st->chknorm >= i + 2) ? 1 : 0;
  st->g[2] = (nt != N_NATURAL || st->chknorm >= i + 2) ? 1 : 0;
}

__global__ void k_cg_d(KspState* st) {
  if (st->active != 1) return;
  st->i += 1;
  if (st->i >= st->max_it) stop(st, st->dp, st->its, R_DIVITS);
}

// ================================================================== CG, fused
// The same recurrence as KSPSolve_CG with the preconditioned norm (the
// default), in three vector kernels per iteration instead of eight:
//   k_cgf_p       p = z + beta/betaold p (VecAYPX's branches; a copy at i = 0)
//   k_cgf_spmv    w = A p and dpi = p.w in one pass; the last CTA runs the
//                 indefinite-matrix test and forms a = beta / dpi
//   k_cgf_update  x += a p, r -= a w, then (Jacobi fused in) z = D r and
//                 ||z||^2, z.r in the same pass; the last CTA records the
//                 residual, runs KSPConvergedDefault, forms beta and the top
//                 of the next iteration.
// Every vector element is computed with the same operations as in the
// unfused kernels; the dot products are summed in a different fixed order.
// W shares Z's storage as in the reference (each w_i is read before z_i is
// written, by the same thread).

// Residual bookkeeping after ||z|| and z.r are known (first: the prologue).
__device__ void cg_tail(KspState* st, double* hist, double dp, double zr, bool first) {
  st->dp = dp;
  int its;
  if (first) {
    hist[0] = dp;
    const int reason = conv_default(st, 0, dp);
    if (reason) {
      stop(st, dp, 0, reason);
      return;
    }
    st->i = 0;
    st->dpi = 0.0;
    st->betaold = 1.0;
  } else {
    its = st->i + 1;
    hist[its] = dp;
    const int reason = conv_default(st, its, dp);
    if (reason) {
      stop(st, dp, its, reason);
      return;
    }
  }
  st->beta = zr;
  if (!first) {
    st->i += 1;
    if (st->i >= st->max_it) {
      stop(st, dp, st->i, R_DIVITS);
      return;
    }
  }
  // top of iteration i
  const int i = st->i;
  st->its = i + 1;
  const double beta = st->beta;
  if (beta == 0.0) {
    stop(st, dp, i + 1, R_ATOL);
    return;
  }
  if (i > 0 && mul(beta, st->betaold) < 0.0) {
    stop(st, dp, i + 1, R_INDEF_PC);
    return;
  }
  st->bcoef = i == 0 ? 0.0 : div_(beta, st->betaold);
  st->dpiold = st->dpi;
  st->active = 1;
  st->g[G_ON] = 1;
}

// Launched with programmatic dependent launch: p is not written by the
// predecessor (the update), so the first batch of p is loaded before the wait
// and its latency overlaps the predecessor's reduction tail.
template <bool FMA>
__global__ void k_cgf_p(KspState* st, int n, double* __restrict__ p,
                        const double* __restrict__ z) {
  pdl_trigger();
  constexpr int U = kVecBatch;
  const unsigned stride = gridDim.x * blockDim.x, un = (unsigned)n;
  const unsigned i0 = blockIdx.x * blockDim.x + threadIdx.x;
  double zv[U], pv[U];
#pragma unroll
  for (int u = 0; u < U; u++) {
    const unsigned i = i0 + u * stride;
    if (i < un) pv[u] = p[i];
  }
  pdl_wait();
  if (st->active != 1) return;
  const double bc = st->bcoef;
  // VecAYPX's branches (src/ported.mojo:285-294): a copy at i = 0.  Decided
  // once per thread: an FP64 compare per element costs FP64 issue slots.
  const int br = bc == 0.0 ? 0 : bc == 1.0 ? 1 : 2;
  for (unsigned j0 = i0; j0 < un; j0 += U * stride) {
#pragma unroll
    for (int u = 0; u < U; u++) {
      const unsigned i = j0 + u * stride;
      if (i < un) {
        if (j0 != i0) pv[u] = p[i];
        zv[u] = z[i];
      }
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const unsigned i = j0 + u * stride;
      if (i >= un) continue;
      if (br == 0)
        p[i] = zv[u];
      else if (br == 1)
        p[i] = madd<FMA>(bc, zv[u], pv[u]);
      else
        p[i] = madd<FMA>(bc, pv[u], zv[u]);
    }
  }
}

template <bool FMA, bool STREAM, typename CT = int>
__global__ void __launch_bounds__(kSpmvRows) k_cgf_spmv(KspState* st, int n,
                                                        const int* __restrict__ rowptr,
                                                        const CT* __restrict__ colind,
                                                        const double* __restrict__ val,
                                                        const double* __restrict__ p,
                                                        double* __restrict__ w, RedSlot slot,
                                                        int evict_first) {
  double v[1] = {0.0};
  if constexpr (!STREAM) {
    const uint64_t pol = spmv_policy(evict_first);
    // the matrix is constant: the first tile's row bounds and first slots
    // are loaded before the wait for p, overlapping the predecessor's tail
    const int row0 = blockIdx.x * kSpmvRows + threadIdx.x;
    SpmvPre pre;
    if (row0 < n) spmv_row_preload(row0, rowptr, colind, val, pol, pre);
    pdl_wait();
    pdl_trigger();
    if (st->active != 1) return;
    // a resident grid walks the row tiles, so each CTA pays the reduction
    // tail once rather than once per 256 rows
    for (int r0 = blockIdx.x * kSpmvRows; r0 < n; r0 += gridDim.x * kSpmvRows) {
      const int row = r0 + threadIdx.x;
      if (row < n) {
        const double s = row == row0
                             ? spmv_row_from<FMA, double, double, CT, false>(pre, colind,
                                                                            val, p, 0.0, pol)
                             : spmv_row<FMA, double, double, CT, false>(row, rowptr, colind,
                                                                        val, p, 0.0, pol);
        w[row] = s;
        v[0] = madd<FMA>(p[row], s, v[0]);
      }
    }
  } else {
    pdl_wait();
    pdl_trigger();
    if (st->active != 1) return;
    const int r0 = blockIdx.x * kSpmvRows;
    const int row = r0 + threadIdx.x;
    double s;
    if constexpr (FMA) {
      __shared__ SpmvSmemF<double, double, double> sm;
      s = spmv_block_rows_fma<double, double, double>(sm, n, r0, rowptr, colind, val, p, 0.0);
    } else {
      __shared__ SpmvSmem<double, double, double> sm;
      s = spmv_block_rows<double, double, double>(sm, n, r0, rowptr, colind, val, p, 0.0);
    }
    if (row < n) {
      w[row] = s;
      v[0] = madd<FMA>(p[row], s, 0.0);
    }
  }
  double tot[1];
  if (grid_finish<1>(v, slot, tot) && threadIdx.x == 0) {
    const double dpi = tot[0];
    st->dpi = dpi;
    const int i = st->i;
    st->betaold = st->beta;
    if (dpi == 0.0 || (i > 0 && sgn(dpi) * sgn(st->dpiold) < 0)) {
      stop(st, st->dp, i + 1, R_INDEF_MAT);
      return;
    }
    st->a = div_(st->beta, dpi);
  }
}

// Loop control folded into the last kernel of a body: `loop` 0 none, 1 the
// trip bookkeeping of the host-driven loop, 2 bookkeeping and the graph's
// loop condition.  Called by one thread per launch.
__device__ __forceinline__ void body_loop_ctrl(int loop, cudaGraphConditionalHandle h,
                                               KspState* st) {
  if (!loop) return;
  const bool run = loop_trip(st);
  if (loop == 2) cudaGraphSetConditional(h, run ? 1u : 0u);
}

// x += a p; r -= a w; (JACOBI) z = D r with ||z||^2 and z.r; else the PC
// follows and k_cgf_red reduces.  With `loop` set (Jacobi only) the kernel
// also ends the loop trip: the thread that finishes the reduction, or block 0
// when the body is switched off.
template <bool FMA, bool JACOBI>
__global__ void __launch_bounds__(kRedBlock, 4) k_cgf_update(
    KspState* st, double* hist, int n, double* __restrict__ x, double* __restrict__ r,
    const double* __restrict__ p, const double* w, double* z, const double* __restrict__ d,
    RedSlot slot, int loop, cudaGraphConditionalHandle h) {
  // x, r, p and d are not written by the predecessor (the SpMV writes only
  // w): the first batch of them is loaded before the wait
  constexpr int U = kVecBatch;
  const unsigned stride = gridDim.x * blockDim.x, un = (unsigned)n;
  const unsigned i0 = blockIdx.x * blockDim.x + threadIdx.x;
  double pv[U], xv[U], wv[U], rv[U], dv[U];
#pragma unroll
  for (int u = 0; u < U; u++) {
    const unsigned i = i0 + u * stride;
    if (i < un) {
      pv[u] = p[i];
      xv[u] = x[i];
      rv[u] = r[i];
      if constexpr (JACOBI) dv[u] = d[i];
    }
  }
  pdl_wait();
  pdl_trigger();
  if (st->active != 1) {
    if (blockIdx.x == 0 && threadIdx.x == 0) body_loop_ctrl(loop, h, st);
    return;
  }
  const double al = st->a, nal = -al;
  double v[2] = {0.0, 0.0};
  for (unsigned j0 = i0; j0 < un; j0 += U * stride) {
#pragma unroll
    for (int u = 0; u < U; u++) {
      const unsigned i = j0 + u * stride;
      if (i < un) {
        if (j0 != i0) {
          pv[u] = p[i];
          xv[u] = x[i];
          rv[u] = r[i];
          if constexpr (JACOBI) dv[u] = d[i];
        }
        wv[u] = w[i];
      }
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const unsigned i = j0 + u * stride;
      if (i >= un) continue;
      x[i] = madd<FMA>(al, pv[u], xv[u]);
      const double ri = madd<FMA>(nal, wv[u], rv[u]);
      r[i] = ri;
      if constexpr (JACOBI) {
        const double zi = mul(ri, dv[u]);
        z[i] = zi;
        v[0] = madd<FMA>(zi, zi, v[0]);
        v[1] = madd<FMA>(zi, ri, v[1]);
      }
    }
  }
  if constexpr (JACOBI) {
    double tot[2];
    if (grid_finish<2>(v, slot, tot) && threadIdx.x == 0) {
      cg_tail(st, hist, __dsqrt_rn(tot[0]), tot[1], false);
      body_loop_ctrl(loop, h, st);
    }
  }
}

// ||z||^2 and z.r after a separate preconditioner apply (first: prologue).
template <bool FMA>
__global__ void __launch_bounds__(kRedBlock) k_cgf_red(KspState* st, double* hist, int n,
                                                       const double* __restrict__ z,
                                                       const double* __restrict__ r,
                                                       RedSlot slot, int first) {
  if (!first && st->active != 1) return;
  double v[2] = {0.0, 0.0};
  constexpr int U = kVecBatch;
  double zv[U], rv[U];
  grid_batched<U>(
      n, [&](int u, unsigned i) { zv[u] = z[i]; rv[u] = r[i]; },
      [&](int u, unsigned) {
        v[0] = madd<FMA>(zv[u], zv[u], v[0]);
        v[1] = madd<FMA>(zv[u], rv[u], v[1]);
      });
  double tot[2];
  if (grid_finish<2>(v, slot, tot) && threadIdx.x == 0)
    cg_tail(st, hist, __dsqrt_rn(tot[0]), tot[1], first != 0);
}

// ================================================================== BCGS
// gates: g[5] on, g[6] "d2 == 0" branch, g[7] regular update, g[0] ||r||
__global__ void k_bcgs_init(KspState* st, double* hist) {
  const double dp = st->dp;
  hist[0] = dp;
  const int reason = conv_default(st, 0, dp);
  st->i = 0;
  st->its = 0;
  st->rhoold = st->alpha = st->omegaold = st->omega = st->rho = 1.0;
  st->c_one = 1.0;
  if (reason) {
    stop(st, dp, 0, reason);
    return;
  }
  st->active = 1;
  st->g[G_ON] = 1;
}

__global__ void k_bcgs_a(KspState* st) {
  if (st->active != 1) return;
  st->bbeta = mul(div_(st->rho, st->rhoold), div_(st->alpha, st->omegaold));
  st->c_omb = mul(-st->omegaold, st->bbeta);
}

__global__ void k_bcgs_b(KspState* st) {
  if (st->active != 1) return;
  if (st->d1 == 0.0) {
    stop(st, st->dp, st->its, R_BREAKDOWN);
    return;
  }
  st->alpha = div_(st->rho, st->d1);
}

__global__ void k_bcgs_c(KspState* st) {
  if (st->active != 1) return;
  if (st->d2 == 0.0) {
    st->g[6] = 1;
    st->g[7] = 0;
    st->g[0] = 0;
    return;
  }
  st->g[6] = 0;
  st->g[7] = 1;
  st->omega = div_(st->d1, st->d2);
  st->g[0] = (st->normtype != N_NONE && st->chknorm < st->i + 2) ? 1 : 0;
}

// d2 == 0: S.S decides between a breakdown and convergence
__global__ void k_bcgs_c2(KspState* st) {
  if (st->active != 1 || !st->g[6]) return;
  if (st->d1 != 0.0) stop(st, st->dp, st->its, R_BREAKDOWN);
}

__global__ void k_bcgs_c3(KspState* st) {
  if (st->active != 1 || !st->g[6]) return;
  stop(st, 0.0, st->its + 1, R_RTOL);
}

__global__ void k_bcgs_d(KspState* st, double* hist) {
  if (st->active != 1) return;
  st->rhoold = st->rho;
  st->omegaold = st->omega;
  st->its += 1;
  const int its = st->its;
  hist[its] = st->dp;
  const int reason = conv_default(st, its, st->dp);
  if (reason) {
    stop(st, st->dp, its, reason);
    return;
  }
  if (st->rho == 0.0) {
    stop(st, st->dp, its, R_BREAKDOWN);
    return;
  }
  st->i += 1;
  if (st->i >= st->max_it) stop(st, st->dp, its, R_DIVITS);
}

// ================================================================== GMRES
// hs block (src/ksp.mojo:32-39, 919-935), HH(a,b) = hh[b (m+2) + a]
struct Hs {
  double *hh, *hes, *cc, *ss, *rs;
  __device__ Hs(double* hs, int m) {
    hh = hs;
    hes = hh + (m + 2) * (m + 1);
    cc = hes + (m + 1) * (m + 1);
    ss = cc + (m + 1);
    rs = ss + (m + 1);
  }
};

// gates: g[0] restart phase, g[1] Arnoldi step, g[2] build, g[3] residual from
// A x, g[4] residual = b, g[5] on, g[6] solution update in build, g[7] CGS
// refinement, g[8] FGMRES build update, g[9] FGMRES residual, g[10] FGMRES
// scale v_{it+1}, g[11] FGMRES scale v_0, g[12] FGMRES zero TEMP.  Every gate
// is set or cleared by a control kernel that precedes its kernels in the body.
__device__ void gm_set_phase(KspState* st, int ph) {
  st->phase = ph;
  st->g[0] = ph == PH_RESTART;
  st->g[1] = ph == PH_STEP;
  st->g[2] = ph == PH_BUILD;
}

// KSPGMRESUpdateHessenberg, src/ksp.mojo:589-629
__device__ int gm_update_hessenberg(Hs& H, int it, int m, int hapend, double* res) {
  double* hh = H.hh;
  for (int j = 1; j <= it; j++) {
    const int idx = it * (m + 2) + (j - 1);
    const double tt = hh[idx];
    const double h1 = hh[idx + 1];
    hh[idx] = add(mul(H.cc[j - 1], tt), mul(H.ss[j - 1], h1));
    hh[idx + 1] = sub(mul(H.cc[j - 1], h1), mul(H.ss[j - 1], tt));
  }
  if (!hapend) {
    const int base = it * (m + 2) + it;
    const double a = hh[base], b = hh[base + 1];
    const double tt = __dsqrt_rn(add(mul(a, a), mul(b, b)));
    if (tt == 0.0) {
      *res = 0.0;
      return R_NULL;
    }
    H.cc[it] = div_(a, tt);
    H.ss[it] = div_(b, tt);
    H.rs[it + 1] = mul(-H.ss[it], H.rs[it]);
    H.rs[it] = mul(H.cc[it], H.rs[it]);
    hh[base] = add(mul(H.cc[it], a), mul(H.ss[it], b));
    *res = fabs(H.rs[it + 1]);
    return 0;
  }
  *res = 0.0;
  return 0;
}

__global__ void k_gm_init(KspState* st) {
  st->its = 0;
  st->itcount = 0;
  st->reason = 0;
  st->res = 0.0;
  st->prev_rnorm = -1.0;
  st->c_one = 1.0;
  st->active = 1;
#pragma unroll
  for (int k = 0; k < 16; k++) st->g[k] = 0;
  st->g[G_ON] = 1;
}

__global__ void k_gm_restart_prep(KspState* st) {
  // residual source for this cycle (KSPInitialResidual's guess_zero branch)
  if (!st->g[0]) return;
  st->g[3] = st->guess_zero ? 0 : 1;
  st->g[4] = st->guess_zero ? 1 : 0;
}

__global__ void k_gm_restart_ctrl(KspState* st, double* hs, double* hist, double* vv, int n) {
  if (!st->g[0]) return;
  Hs H(hs, st->m);
  const double res = st->res;
  if (st->prev_rnorm > 0.0 && fabs(sub(res, st->prev_rnorm)) > mul(st->breakdowntol, st->cfg8)) {
    stop(st, res, st->its, R_BREAKDOWN);
    return;
  }
  H.rs[0] = res;
  st->cfg8 = res;
  hist[st->its] = res;
  st->reason = !res ? R_ATOL : conv_default(st, st->its, res);
  st->it = 0;
  st->hapend = 0;
  st->g[3] = st->g[4] = 0;
  if (st->reason == 0 && st->it < st->m && st->its < st->max_it) {
    st->vv_it = vv;
    st->vv_it1 = vv + n;
    gm_set_phase(st, PH_STEP);
  } else {
    gm_set_phase(st, PH_BUILD);
  }
}

// classical Gram-Schmidt bookkeeping around the MDot / MAXPY pair
// (src/ksp.mojo:533-586).  pass 0: zero the column and set the count.
__global__ void k_gm_cgs0(KspState* st, double* hs) {
  if (!st->g[1]) return;
  Hs H(hs, st->m);
  const int it = st->it, m = st->m;
  for (int j = 0; j <= it; j++) {
    H.hh[it * (m + 2) + j] = 0.0;
    H.hes[it * (m + 1) + j] = 0.0;
  }
  st->kcount = it + 1;
  st->g[7] = st->cgstype == 2 ? 1 : 0;
}

// negate the projections and fold them into the Hessenberg column
__global__ void k_gm_cgs1(KspState* st, double* hs, double* lhh, int gate_idx) {
  if (!st->g[gate_idx]) return;
  Hs H(hs, st->m);
  const int it = st->it, m = st->m;
  double hnrm = 0.0;
  for (int j = 0; j <= it; j++) {
    lhh[j] = -lhh[j];
    H.hh[it * (m + 2) + j] = sub(H.hh[it * (m + 2) + j], lhh[j]);
    H.hes[it * (m + 1) + j] = sub(H.hes[it * (m + 1) + j], lhh[j]);
    hnrm = add(hnrm, mul(lhh[j], lhh[j]));
  }
  if (gate_idx == 1) st->red[1] = __dsqrt_rn(hnrm);
}

// REFINE_IFNEEDED: refine when ||v_{it+1}|| < ||h||
__global__ void k_gm_cgs_ifneeded(KspState* st) {
  if (!st->g[1]) return;
  if (st->red[0] < st->red[1]) st->g[7] = 1;
}

__global__ void k_gm_step_ctrl(KspState* st, double* hs, double* hist, double* vv, int n) {
  if (!st->g[1]) return;
  Hs H(hs, st->m);
  const int m = st->m;
  int it = st->it;
  const double tt = st->tt;
  H.hh[it * (m + 2) + it + 1] = tt;
  H.hes[it * (m + 1) + it + 1] = tt;
  double hapbnd = fabs(div_(tt, H.rs[it]));
  hapbnd = hapbnd > st->haptol ? st->haptol : hapbnd;
  const int hapend = tt < hapbnd ? 1 : 0;
  st->hapend = hapend;
  double res;
  int reason = gm_update_hessenberg(H, it, m, hapend, &res);
  st->res = res;
  it += 1;
  st->it = it;
  st->its += 1;
  hist[st->its] = res;
  if (!reason) {
    reason = conv_default(st, st->its, res);
    if (hapend) {
      if (st->normtype == N_NONE)
        reason = R_HAPPY;
      else if (reason == 0)
        reason = R_BREAKDOWN;
    }
  }
  st->reason = reason;
  st->g[7] = 0;
  if (reason == 0 && it < m && st->its < st->max_it) {
    st->vv_it = vv + (size_t)it * n;
    st->vv_it1 = vv + (size_t)(it + 1) * n;
  } else {
    gm_set_phase(st, PH_BUILD);
  }
}

// KSPGMRESBuildSoln's back substitution (src/ksp.mojo:632-664); the vector
// part follows as gated kernels.
__global__ void k_gm_backsub(KspState* st, double* hs) {
  if (!st->g[2]) return;
  Hs H(hs, st->m);
  const int m = st->m, it = st->it - 1;
  st->itb = it;
  st->g[6] = 0;
  int breason = 0;
  if (it >= 0) {
    double* hh = H.hh;
    double* rs = H.rs;
    if (hh[it * (m + 2) + it] != 0.0) {
      rs[it] = div_(rs[it], hh[it * (m + 2) + it]);
      for (int ii = 1; ii <= it && !breason; ii++) {
        const int k = it - ii;
        double tt = rs[k];
        for (int j = k + 1; j <= it; j++) tt = sub(tt, mul(hh[j * (m + 2) + k], rs[j]));
        if (hh[k * (m + 2) + k] == 0.0) {
          breason = R_BREAKDOWN;
          break;
        }
        rs[k] = div_(tt, hh[k * (m + 2) + k]);
      }
    } else {
      breason = R_BREAKDOWN;
    }
    if (!breason) {
      st->g[6] = 1;
      st->kcount = it + 1;
    }
  }
  st->red[2] = breason;
}

__global__ void k_gm_build_ctrl(KspState* st) {
  if (!st->g[2]) return;
  st->g[6] = 0;
  st->itcount += st->it;
  const int breason = (int)st->red[2];
  if (st->reason == 0 && breason != 0) st->reason = breason;
  if (st->itcount >= st->max_it) {
    stop(st, st->res, st->its, st->reason ? st->reason : R_DIVITS);
    return;
  }
  if (st->reason != 0) {
    stop(st, st->res, st->its, st->reason);
    return;
  }
  st->prev_rnorm = st->res;
  st->guess_zero = 0;
  gm_set_phase(st, PH_RESTART);
}

// ================================================================== FGMRES
__global__ void k_fg_start_ctrl(KspState* st, double* hs, double* hist, double* vv,
                                double* prevec, int n) {
  if (!st->g[0]) return;
  Hs H(hs, st->m);
  const double res = st->res;
  st->it = 0;
  st->hapend = 0;
  H.rs[0] = res;
  hist[st->its] = res;
  st->reason = conv_default(st, st->its, res);
  st->g[9] = 0;
  st->g[11] = 0;
  if (st->reason == 0) {
    st->inv = div_(1.0, res);
    st->g[11] = 1;  // scale v_0 by 1/res
    st->vv_scale = vv;
  }
  if (st->reason == 0 && st->it < st->m && st->its < st->max_it) {
    st->vv_it = vv;
    st->vv_it1 = vv + n;
    st->pv_it = prevec;
    gm_set_phase(st, PH_STEP);
  } else {
    gm_set_phase(st, PH_BUILD);
  }
}

__global__ void k_fg_step_ctrl(KspState* st, double* hs, double* hist, double* vv,
                               double* prevec, int n) {
  st->g[10] = 0;
  st->g[11] = 0;
  st->g[12] = 0;
  if (!st->g[1]) return;
  Hs H(hs, st->m);
  const int m = st->m;
  int it = st->it;
  const double tt = st->tt;
  H.hh[it * (m + 2) + it + 1] = tt;
  H.hes[it * (m + 1) + it + 1] = tt;
  double hapbnd = fabs(div_(tt, H.rs[it]));
  hapbnd = hapbnd > st->haptol ? st->haptol : hapbnd;
  int hapend = 0;
  if (tt > hapbnd) {
    st->inv = div_(1.0, tt);
    st->vv_scale = st->vv_it1;
    st->g[10] = 1;  // v_{it+1} *= 1/tt
  } else {
    st->g[12] = 1;  // TEMP = 0
    hapend = 1;
  }
  st->hapend = hapend;
  double res;
  int reason = gm_update_hessenberg(H, it, m, hapend, &res);
  st->res = res;
  st->g[7] = 0;
  if (reason) {
    st->reason = reason;
    gm_set_phase(st, PH_BUILD);
    return;
  }
  it += 1;
  st->it = it;
  st->its += 1;
  hist[st->its] = res;
  reason = conv_default(st, st->its, res);
  if (hapend && reason == 0) reason = R_BREAKDOWN;
  st->reason = reason;
  if (reason == 0 && it < m && st->its < st->max_it) {
    st->vv_it = vv + (size_t)it * n;
    st->vv_it1 = vv + (size_t)(it + 1) * n;
    st->pv_it = prevec + (size_t)it * n;
  } else {
    gm_set_phase(st, PH_BUILD);
  }
}

// KSPFGMRESBuildSoln's back substitution (src/ksp.mojo:880-903)
__global__ void k_fg_backsub(KspState* st, double* hs) {
  if (!st->g[2]) return;
  Hs H(hs, st->m);
  const int m = st->m, it = st->it - 1;
  st->g[8] = 0;
  if (it < 0) return;
  double* hh = H.hh;
  double* rs = H.rs;
  if (hh[it * (m + 2) + it] != 0.0)
    rs[it] = div_(rs[it], hh[it * (m + 2) + it]);
  else
    rs[it] = 0.0;
  for (int ii = 1; ii <= it; ii++) {
    const int k = it - ii;
    double tt = rs[k];
    for (int j = k + 1; j <= it; j++) tt = sub(tt, mul(hh[j * (m + 2) + k], rs[j]));
    rs[k] = div_(tt, hh[k * (m + 2) + k]);
  }
  st->kcount = it + 1;
  st->g[8] = 1;
}

__global__ void k_fg_build_ctrl(KspState* st) {
  if (!st->g[2]) return;
  st->g[8] = 0;
  st->g[11] = 0;
  if (st->its >= st->max_it) {
    stop(st, st->res, st->its, st->reason ? st->reason : R_DIVITS);
    return;
  }
  if (st->reason != 0) {
    stop(st, st->res, st->its, st->reason);
    return;
  }
  st->g[9] = 1;  // residual, then a new cycle
  gm_set_phase(st, PH_RESTART);
}

// ================================================================== host side

int ksp_create(Ksp** out) {
  *out = new Ksp();
  return GP_OK;
}

static void drop_graph(Ksp* k) {
  if (k->exec) cudaGraphExecDestroy(k->exec);
  if (k->graph) cudaGraphDestroy(k->graph);
  k->exec = nullptr;
  k->graph = nullptr;
  k->cap_A = k->cap_pc = nullptr;
}

int ksp_destroy(Ksp* k) {
  if (!k) return GP_OK;
  drop_graph(k);
  void* ptrs[] = {k->work, k->vv, k->prevec, k->hs, k->lhh, k->hist, k->st, k->slot.partials,
                  k->slot.ticket};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (k->h_st) cudaFreeHost(k->h_st);
  if (k->stream) cudaStreamDestroy(k->stream);
  if (k->stream2) cudaStreamDestroy(k->stream2);
  delete k;
  return GP_OK;
}

static int grow(double** p, size_t* have, size_t need) {
  if (*have >= need && *p) return GP_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  GP_CUDA(cudaMalloc(p, std::max<size_t>(need, 1) * sizeof(double)));
  *have = need;
  return 1000;  // signals "reallocated" to the caller
}

// Allocate (or keep) the workspace for this solve.  Returns whether any buffer
// moved, which invalidates a captured graph.
static int ensure(Ksp* k, int n, bool* moved) {
  const KspOptions& o = k->opt;
  const int m = o.restart;
  *moved = false;
  if (!k->stream) GP_CUDA(cudaStreamCreateWithFlags(&k->stream, cudaStreamNonBlocking));
  if (!k->st) {
    GP_CUDA(cudaMalloc(&k->st, sizeof(KspState)));
    GP_CUDA(cudaMallocHost(&k->h_st, sizeof(KspState)));
    GP_CUDA(cudaMalloc(&k->slot.partials, (size_t)kMaxBasis * kMaxRedGrid * sizeof(double)));
    GP_CUDA(cudaMalloc(&k->slot.ticket, sizeof(unsigned)));
    GP_CUDA(cudaMemset(k->slot.ticket, 0, sizeof(unsigned)));
    k->slot.stride = kMaxRedGrid;
    *moved = true;
  }
  const bool gm = o.type == KSP_GMRES || o.type == KSP_FGMRES;
  int r;
  r = grow(&k->work, &k->work_n, (size_t)(gm ? 2 : 7) * n);
  if (r != GP_OK && r != 1000) return r;
  *moved |= r == 1000;
  if (gm) {
    r = grow(&k->vv, &k->vv_n, (size_t)(m + 1) * n);
    if (r != GP_OK && r != 1000) return r;
    *moved |= r == 1000;
    const size_t hs = (size_t)(m + 2) * (m + 1) + (size_t)(m + 1) * (m + 1) + 2 * (m + 1) +
                      2 * (m + 2);
    r = grow(&k->hs, &k->hs_n, hs);
    if (r != GP_OK && r != 1000) return r;
    *moved |= r == 1000;
    size_t lhn = k->lhh ? (size_t)kMaxBasis : 0;
    r = grow(&k->lhh, &lhn, kMaxBasis);
    if (r != GP_OK && r != 1000) return r;
    *moved |= r == 1000;
    if (o.type == KSP_FGMRES) {
      r = grow(&k->prevec, &k->pv_n, (size_t)(m + 2) * n);
      if (r != GP_OK && r != 1000) return r;
      *moved |= r == 1000;
    }
  }
  size_t hc = (size_t)k->hist_cap;
  r = grow(&k->hist, &hc, (size_t)o.max_it + 2);
  if (r != GP_OK && r != 1000) return r;
  *moved |= r == 1000;
  k->hist_cap = (int)hc;
  return GP_OK;
}

namespace {

// launch helpers bound to one solve
struct Run {
  Ksp* k;
  Csr* A;
  Pc* pc;
  int n;
  cudaStream_t s;
  // loop control taken over by the body's last kernel (see body_ends_trip):
  // 0 none, 1 host-driven trip bookkeeping, 2 also the graph condition
  int loop = 0;
  cudaGraphConditionalHandle cond = 0;
  const int* G(int idx) const { return &k->st->g[idx]; }
  double* S(double KspState::*f) const { return &(k->st->*f); }
  int grid() const { return vgrid(n); }

  int copy(const int* g, DRef x, DRef y) const {
    k_copy_d<<<grid(), 256, 0, s>>>(g, 1, n, x, y);
    GP_CHECK_LAUNCH();
    return GP_OK;
  }
  int zero(const int* g, DRef y) const {
    k_zero_d<<<grid(), 256, 0, s>>>(g, 1, n, y);
    GP_CHECK_LAUNCH();
    return GP_OK;
  }
  template <int OP>
  int red(const int* g, DRef x, DRef y, double* raw, double* sq, double* raw2 = nullptr) const {
    if (arith_mode() == kOrdered) {
      constexpr int OOP = OP == D_DOT ? ORD_DOT : OP == D_NRM ? ORD_NRM : ORD_DOTNRM;
      k_ord_red<OOP><<<kOrdChains, 32, 0, s>>>(g, 1, n, x, y, k->slot, raw, sq, raw2);
    } else if (arith_mode() == kFma)
      k_dred<OP, true><<<red_grid(n), kRedBlock, 0, s>>>(g, 1, n, x, y, k->slot, raw, sq, raw2);
    else
      k_dred<OP, false><<<red_grid(n), kRedBlock, 0, s>>>(g, 1, n, x, y, k->slot, raw, sq, raw2);
    GP_CHECK_LAUNCH();
    return GP_OK;
  }
  // KSPSolveTranspose: A^T and M^-T in place of A and M^-1
  int matmult(const int* g, DRef x, DRef y) const {
    return k->transpose ? spmv_t(s, A, x, y, g, 1) : spmv(s, A, x, y, g, 1);
  }
  int pcapply(const int* g, DRef x, DRef y) const {
    return k->transpose ? pc_apply_transpose(pc, x, y, s, g, 1) : pc_apply(pc, x, y, s, g, 1);
  }
  int pcsym(const int* g, DRef x, DRef y) const {
    if (k->transpose && pc->opt.type != PC_JACOBI) return pc_apply_transpose(pc, x, y, s, g, 1);
    return pc_apply_symmetric(pc, x, y, s, g, 1);
  }
  // KSP_PCApplyBAorAB, src/ksp.mojo:246-265
  int apply_ba(const int* g, int side, DRef x, DRef y, DRef w) const {
    if (side == 1) {
      GP_TRY(pcapply(g, x, w));
      return matmult(g, w, y);
    }
    if (side == 0) {
      GP_TRY(matmult(g, x, w));
      return pcapply(g, w, y);
    }
    GP_TRY(pcsym(g, x, w));
    GP_TRY(matmult(g, w, y));
    GP_TRY(copy(g, y, w));
    return pcsym(g, w, y);
  }
  // KSPInitialResidual, src/ksp.mojo:221-243
  int initial_residual(int side, int guess_zero, DRef x, DRef vt1, DRef vt2, DRef vres,
                       DRef b) const {
    if (!guess_zero) {
      GP_TRY(matmult(nullptr, x, vt1));
      GP_TRY(copy(nullptr, b, vt2));
      FL(k_axpy_d, grid(), 256, s, nullptr, 1, n, vt2, S(&KspState::c_one), -1.0, vt1);
      GP_CHECK_LAUNCH();
    } else {
      GP_TRY(copy(nullptr, b, vt2));
    }
    if (side == 2) return pcsym(nullptr, vt2, vres);
    if (side == 0) return pcapply(nullptr, vt2, vres);
    return copy(nullptr, vt2, vres);
  }
};

}  // namespace

// ------------------------------------------------------------------ CG
static int cg_prologue(const Run& r, const double* b, double* x) {
  Ksp* k = r.k;
  const KspOptions& o = k->opt;
  const int n = r.n;
  DRef R = DRef::of(k->work), Z = DRef::of(k->work + n);
  if (!o.guess_zero) {
    GP_TRY(r.matmult(nullptr, DRef::of(x), R));
    FL(k_aypx_h, r.grid(), 256, r.s, nullptr, 1, n, R, -1.0, DRef::of(b));
    GP_CHECK_LAUNCH();
  } else {
    GP_TRY(r.copy(nullptr, DRef::of(b), R));
  }
  double* dp = r.S(&KspState::dp);
  double* beta = r.S(&KspState::beta);
  if (o.normtype == N_PRECOND) {
    GP_TRY(r.pcapply(nullptr, R, Z));
    GP_TRY(r.red<D_NRM>(nullptr, Z, Z, nullptr, dp));
  } else if (o.normtype == N_UNPRECOND) {
    GP_TRY(r.red<D_NRM>(nullptr, R, R, nullptr, dp));
  } else if (o.normtype == N_NATURAL) {
    GP_TRY(r.pcapply(nullptr, R, Z));
    GP_TRY(r.red<D_DOT>(nullptr, Z, R, beta, dp));
  }
  k_cg_init<<<1, 1, 0, r.s>>>(k->st, k->hist);
  GP_CHECK_LAUNCH();
  GP_TRY(r.pcapply(r.G(1), R, Z));
  GP_TRY(r.red<D_DOT>(r.G(2), Z, R, beta, nullptr));
  return GP_OK;
}

static int cg_body(const Run& r, double* x) {
  Ksp* k = r.k;
  const int n = r.n;
  double* R = k->work;
  double* Z = k->work + n;
  double* P = k->work + 2 * n;
  double* W = Z;  // the reference's W = Z aliasing
  KspState* st = k->st;
  const int* on = r.G(G_ON);
  k_cg_a<<<1, 1, 0, r.s>>>(st);
  FL(k_aypx_d, r.grid(), 256, r.s, on, 1, n, DRef::of(P), r.S(&KspState::bcoef), DRef::of(Z));
  GP_CHECK_LAUNCH();
  GP_TRY(r.matmult(on, DRef::of(P), DRef::of(W)));
  GP_TRY(r.red<D_DOT>(on, DRef::of(P), DRef::of(W), r.S(&KspState::dpi), nullptr));
  k_cg_b<<<1, 1, 0, r.s>>>(st);
  FL(k_cg_xr, r.grid(), 256, r.s, on, 1, n, x, R, P, W, r.S(&KspState::a));
  GP_CHECK_LAUNCH();
  const int nt = k->opt.normtype;
  double* dp = r.S(&KspState::dp);
  double* beta = r.S(&KspState::beta);
  if (nt == N_PRECOND) {
    GP_TRY(r.pcapply(r.G(0), DRef::of(R), DRef::of(Z)));
    GP_TRY(r.red<D_NRM>(r.G(0), DRef::of(Z), DRef::of(Z), nullptr, dp));
  } else if (nt == N_UNPRECOND) {
    GP_TRY(r.red<D_NRM>(r.G(3), DRef::of(R), DRef::of(R), nullptr, dp));
  } else if (nt == N_NATURAL) {
    GP_TRY(r.pcapply(r.G(4), DRef::of(R), DRef::of(Z)));
    GP_TRY(r.red<D_DOT>(r.G(4), DRef::of(Z), DRef::of(R), beta, dp));
  }
  k_cg_c<<<1, 1, 0, r.s>>>(st, k->hist);
  GP_TRY(r.pcapply(r.G(1), DRef::of(R), DRef::of(Z)));
  GP_TRY(r.red<D_DOT>(r.G(2), DRef::of(Z), DRef::of(R), beta, nullptr));
  k_cg_d<<<1, 1, 0, r.s>>>(st);
  GP_CHECK_LAUNCH();
  return GP_OK;
}

// ------------------------------------------------------------------ CG, fused
// CTAs of `kernel` that fit on the device at once (one full wave).
static int resident_grid(const void* kernel, int block) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0) != cudaSuccess ||
      per_sm < 1) {
    cudaGetLastError();
    per_sm = 1;
  }
  return std::max(1, std::min(per_sm * num_sms(), kMaxRedGrid));
}

static bool cg_fused_ok(const Run& r) {
  const KspOptions& o = r.k->opt;
  // the fused kernels sum their dots inside the vector passes (tree order)
  // and multiply by A itself
  // (a matrix whose long rows are summed by segments multiplies through
  // spmv(), which runs the segment kernel: the general loop)
  return arith_mode() != kOrdered && !r.k->transpose && o.normtype == N_PRECOND &&
         o.chknorm <= 1 && r.A->lr.nlong == 0 &&
         (int64_t)spmv_grid(r.A) <= (int64_t)kMaxBasis * kMaxRedGrid;
}

static int cg_prologue_fused(const Run& r, const double* b, double* x) {
  Ksp* k = r.k;
  const int n = r.n;
  DRef R = DRef::of(k->work), Z = DRef::of(k->work + n);
  if (!k->opt.guess_zero) {
    GP_TRY(r.matmult(nullptr, DRef::of(x), R));
    FL(k_aypx_h, r.grid(), 256, r.s, nullptr, 1, n, R, -1.0, DRef::of(b));
  } else {
    GP_TRY(r.copy(nullptr, DRef::of(b), R));
  }
  GP_TRY(r.pcapply(nullptr, R, Z));
  FL(k_cgf_red, red_grid(n), kRedBlock, r.s, k->st, k->hist, n, k->work + n, k->work, k->slot,
     1);
  GP_CHECK_LAUNCH();
  return GP_OK;
}

static int cg_body_fused(const Run& r, double* x) {
  Ksp* k = r.k;
  const int n = r.n;
  double* R = k->work;
  double* Z = k->work + n;
  double* P = k->work + 2 * n;
  double* W = Z;  // the reference's W = Z aliasing
  const Csr* A = r.A;
  GP_CUDA(launch_pdl(arith_mode() == kFma ? k_cgf_p<true> : k_cgf_p<false>, r.grid(), 256, r.s,
                     k->st, n, P, (const double*)Z));
  {
    const bool f = arith_mode() == kFma;
    if (A->coff16) {  // row form with 16-bit column offsets
      auto ks = f ? k_cgf_spmv<true, false, short> : k_cgf_spmv<false, false, short>;
      const int grid = std::min(spmv_grid(A), resident_grid((const void*)ks, kSpmvRows));
      GP_CUDA(launch_pdl(ks, grid, kSpmvRows, r.s, k->st, n, (const int*)A->rowptr,
                         (const short*)A->coff16, (const double*)A->val, (const double*)P, W,
                         k->slot, A->l2_evict_first));
    } else {
      auto ks = A->stream_rows ? (f ? k_cgf_spmv<true, true> : k_cgf_spmv<false, true>)
                               : (f ? k_cgf_spmv<true, false> : k_cgf_spmv<false, false>);
      int grid = spmv_grid(A);
      if (!A->stream_rows) grid = std::min(grid, resident_grid((const void*)ks, kSpmvRows));
      GP_CUDA(launch_pdl(ks, grid, kSpmvRows, r.s, k->st, n, (const int*)A->rowptr,
                         (const int*)A->colind, (const double*)A->val, (const double*)P, W,
                         k->slot, A->l2_evict_first));
    }
  }
  const bool jac = r.pc->opt.type == PC_JACOBI;
  const bool f = arith_mode() == kFma;
  const int g = red_grid(n);
  if (jac) {
    GP_CUDA(launch_pdl(f ? k_cgf_update<true, true> : k_cgf_update<false, true>, g, kRedBlock,
                       r.s, k->st, k->hist, n, x, R, (const double*)P, (const double*)W, Z,
                       (const double*)r.pc->diag, k->slot, r.loop, r.cond));
  } else {
    if (f)
      k_cgf_update<true, false><<<g, kRedBlock, 0, r.s>>>(k->st, k->hist, n, x, R, P, W, Z,
                                                          nullptr, k->slot, 0, 0);
    else
      k_cgf_update<false, false><<<g, kRedBlock, 0, r.s>>>(k->st, k->hist, n, x, R, P, W, Z,
                                                           nullptr, k->slot, 0, 0);
    GP_TRY(r.pcapply(r.G(G_ON), DRef::of(R), DRef::of(Z)));
    FL(k_cgf_red, g, kRedBlock, r.s, k->st, k->hist, n, Z, R, k->slot, 0);
  }
  GP_CHECK_LAUNCH();
  return GP_OK;
}

// ------------------------------------------------------------------ BCGS
static int bcgs_prologue(const Run& r, const double* b, double* x) {
  Ksp* k = r.k;
  const KspOptions& o = k->opt;
  const int n = r.n;
  double* w = k->work;
  DRef R = DRef::of(w), RP = DRef::of(w + n), V = DRef::of(w + 2 * n), T = DRef::of(w + 3 * n);
  DRef P = DRef::of(w + 5 * n), GUESS = DRef::of(w + 6 * n);
  GP_TRY(r.initial_residual(o.pc_side, o.guess_zero, DRef::of(x), V, T, R, DRef::of(b)));
  if (o.pc_side == 1 && !o.guess_zero) {
    GP_TRY(r.copy(nullptr, DRef::of(x), GUESS));
    GP_TRY(r.zero(nullptr, DRef::of(x)));
  }
  if (o.normtype != N_NONE)
    GP_TRY(r.red<D_NRM>(nullptr, R, R, nullptr, r.S(&KspState::dp)));
  k_bcgs_init<<<1, 1, 0, r.s>>>(k->st, k->hist);
  GP_CHECK_LAUNCH();
  const int* on = r.G(G_ON);
  GP_TRY(r.copy(on, R, RP));
  GP_TRY(r.zero(on, P));
  GP_TRY(r.zero(on, V));
  return GP_OK;
}

static int bcgs_body(const Run& r, double* x) {
  Ksp* k = r.k;
  const int n = r.n, side = k->opt.pc_side;
  double* w = k->work;
  DRef R = DRef::of(w), RP = DRef::of(w + n), V = DRef::of(w + 2 * n), T = DRef::of(w + 3 * n);
  DRef S = DRef::of(w + 4 * n), P = DRef::of(w + 5 * n), X = DRef::of(x);
  KspState* st = k->st;
  const int* on = r.G(G_ON);
  GP_TRY(r.red<D_DOT>(on, R, RP, r.S(&KspState::rho), nullptr));
  k_bcgs_a<<<1, 1, 0, r.s>>>(st);
  FL(k_axpbypcz_d, r.grid(), 256, r.s, on, 1, n, P, r.S(&KspState::c_one),
                                           r.S(&KspState::c_omb), r.S(&KspState::bbeta), R, V);
  GP_CHECK_LAUNCH();
  GP_TRY(r.apply_ba(on, side, P, V, T));
  GP_TRY(r.red<D_DOT>(on, V, RP, r.S(&KspState::d1), nullptr));
  k_bcgs_b<<<1, 1, 0, r.s>>>(st);
  FL(k_waxpy_d, r.grid(), 256, r.s, on, 1, n, S, r.S(&KspState::alpha), -1.0, V, R);
  GP_CHECK_LAUNCH();
  GP_TRY(r.apply_ba(on, side, S, T, R));
  // VecDotNorm2(S, T): (S.T, T.T) -- computed as (T.S, T.T), the same sums
  GP_TRY(r.red<D_DOTNRM>(on, T, S, r.S(&KspState::d1), nullptr, r.S(&KspState::d2)));
  k_bcgs_c<<<1, 1, 0, r.s>>>(st);
  GP_TRY(r.red<D_DOT>(r.G(6), S, S, r.S(&KspState::d1), nullptr));
  k_bcgs_c2<<<1, 1, 0, r.s>>>(st);
  FL(k_axpy_d, r.grid(), 256, r.s, r.G(6), 1, n, X, r.S(&KspState::alpha), 1.0, P);
  k_bcgs_c3<<<1, 1, 0, r.s>>>(st);
  FL(k_axpbypcz_d, r.grid(), 256, r.s, r.G(7), 1, n, X, r.S(&KspState::alpha),
                                           r.S(&KspState::omega), r.S(&KspState::c_one), P, S);
  FL(k_waxpy_d, r.grid(), 256, r.s, r.G(7), 1, n, R, r.S(&KspState::omega), -1.0, T, S);
  GP_CHECK_LAUNCH();
  GP_TRY(r.red<D_NRM>(r.G(0), R, R, nullptr, r.S(&KspState::dp)));
  k_bcgs_d<<<1, 1, 0, r.s>>>(st, k->hist);
  GP_CHECK_LAUNCH();
  return GP_OK;
}

static int bcgs_epilogue(const Run& r, double* x) {
  Ksp* k = r.k;
  const KspOptions& o = k->opt;
  const int n = r.n;
  double* w = k->work;
  DRef T = DRef::of(w + 3 * n), GUESS = DRef::of(w + 6 * n), X = DRef::of(x);
  // KSPUnwindPreconditioner (src/ksp.mojo:211-218)
  if (o.pc_side == 1) {
    GP_TRY(r.pcapply(nullptr, X, T));
    GP_TRY(r.copy(nullptr, T, X));
  }
  if (o.pc_side == 1 && !o.guess_zero) {
    FL(k_axpy_d, r.grid(), 256, r.s, nullptr, 1, n, X, r.S(&KspState::c_one), 1.0, GUESS);
    GP_CHECK_LAUNCH();
  }
  return GP_OK;
}

// ------------------------------------------------------------------ GMRES
// classical Gram-Schmidt on v_{it+1} against v_0..v_it, with the optional
// refinement pass (src/ksp.mojo:533-586)
static int cgs_pass(const Run& r, int gate_idx) {
  Ksp* k = r.k;
  const int* g = r.G(gate_idx);
  DRef v1 = DRef::at(&k->st->vv_it1);
  if (arith_mode() == kOrdered) {
    const int kmax = std::min(k->opt.restart + 1, kMaxBasis);
    k_ord_mdot<<<kOrdChains * kmax, 32, 0, r.s>>>(g, 1, r.n, v1, k->vv, &k->st->kcount,
                                                   k->slot, k->lhh);
  } else {
    FL(k_mdot, red_grid(r.n), kRedBlock, r.s, g, 1, r.n, v1, k->vv, &k->st->kcount, k->slot,
                                                k->lhh);
  }
  k_gm_cgs1<<<1, 1, 0, r.s>>>(k->st, k->hs, k->lhh, gate_idx);
  FL(k_maxpy_dyn, r.grid(), 256, r.s, g, 1, r.n, v1, k->vv, k->lhh, &k->st->kcount, 0);
  GP_CHECK_LAUNCH();
  return GP_OK;
}

static int cgs(const Run& r) {
  Ksp* k = r.k;
  k_gm_cgs0<<<1, 1, 0, r.s>>>(k->st, k->hs);
  GP_TRY(cgs_pass(r, 1));
  if (k->opt.cgstype == 1) {
    GP_TRY(r.red<D_NRM>(r.G(1), DRef::at(&k->st->vv_it1), DRef::at(&k->st->vv_it1), nullptr,
                        &k->st->red[0]));
    k_gm_cgs_ifneeded<<<1, 1, 0, r.s>>>(k->st);
  }
  if (k->opt.cgstype != 0) GP_TRY(cgs_pass(r, 7));
  return GP_OK;
}

// modified Gram-Schmidt (KSPGMRESModifiedGramSchmidtOrthogonalization,
// src/ksp.mojo:511-530): for k = 0..it, d = v_{it+1} . v_k, HH(k, it) =
// HES(k, it) = d, v_{it+1} -= d v_k.  The captured body holds `restart`
// (dot, store, axpy) triples; triple k runs while k <= it.
static_assert(kMaxBasis <= 64, "mgs_on holds one gate per basis vector");
__global__ void k_gm_mgs_prep(KspState* st) {
  const int on = st->g[1];
  for (int k = 0; k < kMaxBasis; k++) st->mgs_on[k] = on && k <= st->it ? 1 : 0;
}

__global__ void k_gm_mgs_store(KspState* st, double* hs, int k) {
  if (!st->mgs_on[k]) return;
  Hs H(hs, st->m);
  const int it = st->it, m = st->m;
  H.hh[it * (m + 2) + k] = st->mgs_d;
  H.hes[it * (m + 1) + k] = st->mgs_d;
}

static int mgs(const Run& r) {
  Ksp* k = r.k;
  KspState* st = k->st;
  DRef v1 = DRef::at(&st->vv_it1);
  k_gm_mgs_prep<<<1, 1, 0, r.s>>>(st);
  for (int kk = 0; kk < k->opt.restart; kk++) {
    const int* gate = &st->mgs_on[kk];
    DRef vk = DRef::of(k->vv + (size_t)kk * r.n);
    GP_TRY(r.red<D_DOT>(gate, v1, vk, &st->mgs_d, nullptr));
    k_gm_mgs_store<<<1, 1, 0, r.s>>>(st, k->hs, kk);
    FL(k_axpy_d, r.grid(), 256, r.s, gate, 1, r.n, v1, &st->mgs_d, -1.0, vk);
  }
  GP_CHECK_LAUNCH();
  return GP_OK;
}

// the first cycle starts with a restart (no solution to build yet)
__global__ void k_first_restart(KspState* st) { gm_set_phase(st, PH_RESTART); }

static int gmres_prologue(const Run& r) {
  k_gm_init<<<1, 1, 0, r.s>>>(r.k->st);
  k_first_restart<<<1, 1, 0, r.s>>>(r.k->st);
  GP_CHECK_LAUNCH();
  return GP_OK;
}

static int gmres_body(const Run& r, const double* b, double* x) {
  Ksp* k = r.k;
  const int n = r.n, side = k->opt.pc_side;
  KspState* st = k->st;
  DRef TEMP = DRef::of(k->work), TMATOP = DRef::of(k->work + n), VV0 = DRef::of(k->vv);
  DRef X = DRef::of(x), B = DRef::of(b);
  // ---- build the solution at the end of a cycle (KSPGMRESBuildSoln)
  k_gm_backsub<<<1, 1, 0, r.s>>>(st, k->hs);
  const int m = k->opt.restart;
  double* rs = k->hs + (size_t)(m + 2) * (m + 1) + (size_t)(m + 1) * (m + 1) + 2 * (m + 1);
  FL(k_maxpy_dyn, r.grid(), 256, r.s, r.G(6), 1, n, TEMP, k->vv, rs, &st->kcount, 1);
  GP_CHECK_LAUNCH();
  if (side == 1) {  // KSPUnwindPreconditioner for right preconditioning
    GP_TRY(r.pcapply(r.G(6), TEMP, TMATOP));
    GP_TRY(r.copy(r.G(6), TMATOP, TEMP));
  }
  FL(k_axpy_d, r.grid(), 256, r.s, r.G(6), 1, n, X, r.S(&KspState::c_one), 1.0, TEMP);
  k_gm_build_ctrl<<<1, 1, 0, r.s>>>(st);
  // ---- restart: r0 = M^-1 (b - A x) (or b), normalised
  k_gm_restart_prep<<<1, 1, 0, r.s>>>(st);
  GP_TRY(r.matmult(r.G(3), X, TEMP));
  GP_TRY(r.copy(r.G(3), B, TMATOP));
  FL(k_axpy_d, r.grid(), 256, r.s, r.G(3), 1, n, TMATOP, r.S(&KspState::c_one), -1.0, TEMP);
  GP_CHECK_LAUNCH();
  GP_TRY(r.copy(r.G(4), B, TMATOP));
  if (side == 2)
    GP_TRY(r.pcsym(r.G(0), TMATOP, VV0));
  else if (side == 0)
    GP_TRY(r.pcapply(r.G(0), TMATOP, VV0));
  else
    GP_TRY(r.copy(r.G(0), TMATOP, VV0));
  GP_TRY(r.red<D_NRM>(r.G(0), VV0, VV0, nullptr, r.S(&KspState::res)));
  k_scale_d<true><<<r.grid(), 256, 0, r.s>>>(r.G(0), 1, n, VV0, r.S(&KspState::res));
  k_gm_restart_ctrl<<<1, 1, 0, r.s>>>(st, k->hs, k->hist, k->vv, n);
  GP_CHECK_LAUNCH();
  // ---- one Arnoldi step
  DRef vit = DRef::at(&st->vv_it), vit1 = DRef::at(&st->vv_it1);
  GP_TRY(r.apply_ba(r.G(1), side, vit, vit1, TMATOP));
  GP_TRY(k->opt.orthog ? mgs(r) : cgs(r));
  GP_TRY(r.red<D_NRM>(r.G(1), vit1, vit1, nullptr, r.S(&KspState::tt)));
  k_scale_d<true><<<r.grid(), 256, 0, r.s>>>(r.G(1), 1, n, vit1, r.S(&KspState::tt));
  k_gm_step_ctrl<<<1, 1, 0, r.s>>>(st, k->hs, k->hist, k->vv, n);
  GP_CHECK_LAUNCH();
  return GP_OK;
}

// ------------------------------------------------------------------ FGMRES
static int fgmres_prologue(const Run& r, const double* b, double* x) {
  Ksp* k = r.k;
  const int n = r.n;
  k_gm_init<<<1, 1, 0, r.s>>>(k->st);
  GP_CHECK_LAUNCH();
  DRef TEMP = DRef::of(k->work), VV0 = DRef::of(k->vv);
  if (!k->opt.guess_zero) {  // KSPFGMRESResidual, src/ksp.mojo:871-877
    GP_TRY(r.matmult(nullptr, DRef::of(x), TEMP));
    FL(k_waxpy_d, r.grid(), 256, r.s, nullptr, 1, n, VV0, r.S(&KspState::c_one), -1.0, TEMP,
                                         DRef::of(b));
    GP_CHECK_LAUNCH();
  } else {
    GP_TRY(r.copy(nullptr, DRef::of(b), VV0));
  }
  k_first_restart<<<1, 1, 0, r.s>>>(k->st);
  GP_CHECK_LAUNCH();
  return GP_OK;
}


static int fgmres_body(const Run& r, const double* b, double* x) {
  Ksp* k = r.k;
  const int n = r.n, m = k->opt.restart;
  KspState* st = k->st;
  DRef TEMP = DRef::of(k->work), VV0 = DRef::of(k->vv), X = DRef::of(x), B = DRef::of(b);
  double* rs = k->hs + (size_t)(m + 2) * (m + 1) + (size_t)(m + 1) * (m + 1) + 2 * (m + 1);
  // ---- build (KSPFGMRESBuildSoln) and the next residual
  k_fg_backsub<<<1, 1, 0, r.s>>>(st, k->hs);
  FL(k_maxpy_dyn, r.grid(), 256, r.s, r.G(8), 1, n, TEMP, k->prevec, rs, &st->kcount, 1);
  FL(k_axpy_d, r.grid(), 256, r.s, r.G(8), 1, n, X, r.S(&KspState::c_one), 1.0, TEMP);
  k_fg_build_ctrl<<<1, 1, 0, r.s>>>(st);
  GP_CHECK_LAUNCH();
  GP_TRY(r.matmult(r.G(9), X, TEMP));
  FL(k_waxpy_d, r.grid(), 256, r.s, r.G(9), 1, n, VV0, r.S(&KspState::c_one), -1.0, TEMP, B);
  // ---- cycle start: ||r||, convergence test, v_0 = r / ||r|| (by reciprocal)
  GP_TRY(r.red<D_NRM>(r.G(0), VV0, VV0, nullptr, r.S(&KspState::res)));
  k_fg_start_ctrl<<<1, 1, 0, r.s>>>(st, k->hs, k->hist, k->vv, k->prevec, n);
  k_scale_d<false><<<r.grid(), 256, 0, r.s>>>(r.G(11), 1, n, VV0, r.S(&KspState::inv));
  GP_CHECK_LAUNCH();
  // ---- one flexible Arnoldi step
  DRef vit = DRef::at(&st->vv_it), vit1 = DRef::at(&st->vv_it1), pit = DRef::at(&st->pv_it);
  GP_TRY(r.pcapply(r.G(1), vit, pit));
  GP_TRY(r.matmult(r.G(1), pit, vit1));
  GP_TRY(k->opt.orthog ? mgs(r) : cgs(r));
  GP_TRY(r.red<D_NRM>(r.G(1), vit1, vit1, nullptr, r.S(&KspState::tt)));
  k_fg_step_ctrl<<<1, 1, 0, r.s>>>(st, k->hs, k->hist, k->vv, k->prevec, n);
  k_scale_d<false><<<r.grid(), 256, 0, r.s>>>(r.G(10), 1, n, DRef::at(&st->vv_scale),
                                              r.S(&KspState::inv));
  GP_TRY(r.zero(r.G(12), TEMP));
  GP_CHECK_LAUNCH();
  return GP_OK;
}

// ------------------------------------------------------------------ solve

// The whole solve as one graph: prologue kernels, a WHILE node whose body is
// one iteration, the epilogue, and the read-back of the state block.
static int count_kernels(cudaGraph_t g, int64_t* out) {
  size_t cnt = 0;
  GP_CUDA(cudaGraphGetNodes(g, nullptr, &cnt));
  std::vector<cudaGraphNode_t> nodes(cnt);
  if (cnt) GP_CUDA(cudaGraphGetNodes(g, nodes.data(), &cnt));
  int64_t k = 0;
  for (auto nd : nodes) {
    cudaGraphNodeType t;
    GP_CUDA(cudaGraphNodeGetType(nd, &t));
    if (t == cudaGraphNodeTypeKernel) k++;
  }
  *out = k;
  return GP_OK;
}

static int run_prologue(const Run& r, const double* b, double* x) {
  switch (r.k->opt.type) {
    case KSP_CG: return cg_fused_ok(r) ? cg_prologue_fused(r, b, x) : cg_prologue(r, b, x);
    case KSP_BCGS: return bcgs_prologue(r, b, x);
    case KSP_GMRES: return gmres_prologue(r);
    case KSP_FGMRES: return fgmres_prologue(r, b, x);
  }
  return GP_OK;
}

// Whether the body's last kernel ends the loop trip itself (the fused CG with
// Jacobi: its update kernel), so no separate loop-control kernel follows.
static bool body_ends_trip(const Run& r) {
  return r.k->opt.type == KSP_CG && cg_fused_ok(r) && r.pc->opt.type == PC_JACOBI;
}

static int run_body(const Run& r, const double* b, double* x) {
  switch (r.k->opt.type) {
    case KSP_CG: return cg_fused_ok(r) ? cg_body_fused(r, x) : cg_body(r, x);
    case KSP_BCGS: return bcgs_body(r, x);
    case KSP_GMRES: return gmres_body(r, b, x);
    case KSP_FGMRES: return fgmres_body(r, b, x);
  }
  return GP_OK;
}

// Loop-body copies per conditional trip (GPETSC_KSP_UNROLL, 1..16; by default
// kBodyUnrollCg for the three-kernel fused CG body, whose trips are short
// enough that the conditional node's re-launch shows, else kBodyUnroll).
static int body_unroll(const Run& r) {
  static int env = [] {
    const char* e = std::getenv("GPETSC_KSP_UNROLL");
    return e ? std::max(1, std::min(16, std::atoi(e))) : 0;
  }();
  if (env) return env;
  return body_ends_trip(r) ? kBodyUnrollCg : kBodyUnroll;
}

// GPETSC_KSP_GRAPH=0: drive the loop from the host (same kernels, launched on
// the stream, convergence polled every kEagerPoll trips) instead of one graph.
static bool eager_mode() {
  static bool v = [] {
    const char* e = std::getenv("GPETSC_KSP_GRAPH");
    return e && std::string(e) == "0";
  }();
  return v;
}

static int run_eager(const Run& r, const double* b, double* x) {
  Ksp* k = r.k;
  GP_TRY(run_prologue(r, b, x));
  const bool own = body_ends_trip(r);
  Run rl = r;
  rl.loop = own ? 1 : 0;
  for (int64_t trip = 1;; trip++) {
    GP_TRY(run_body(rl, b, x));
    if (!own) k_loop_trip<<<1, 1, 0, r.s>>>(k->st);
    GP_CHECK_LAUNCH();
    if (trip % kEagerPoll == 0) {
      int active = 0;
      GP_CUDA(cudaMemcpyAsync(&active, &k->st->active, sizeof(int), cudaMemcpyDeviceToHost, r.s));
      GP_CUDA(cudaStreamSynchronize(r.s));
      if (active != 1) break;
    }
  }
  if (k->opt.type == KSP_BCGS) GP_TRY(bcgs_epilogue(r, x));
  GP_CUDA(cudaMemcpyAsync(k->h_st, k->st, sizeof(KspState), cudaMemcpyDeviceToHost, r.s));
  k->top_kernels = -1;
  k->body_kernels = -1;
  return GP_OK;
}

static int capture(const Run& r, const double* b, double* x) {
  Ksp* k = r.k;
  drop_graph(k);
  if (!k->stream2) GP_CUDA(cudaStreamCreateWithFlags(&k->stream2, cudaStreamNonBlocking));
  GP_CUDA(cudaStreamBeginCapture(r.s, cudaStreamCaptureModeRelaxed));
  int st = run_prologue(r, b, x);
  cudaGraph_t graph = nullptr;
  cudaGraph_t body = nullptr;
  cudaGraphConditionalHandle h = 0;
  if (st == GP_OK) {
    cudaStreamCaptureStatus cs;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    cudaError_t e = cudaStreamGetCaptureInfo(r.s, &cs, nullptr, &graph, &deps, nullptr, &ndeps);
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault);
    cudaGraphNode_t wnode = nullptr;
    if (e == cudaSuccess) {
      cudaGraphNodeParams cp = {};
      cp.type = cudaGraphNodeTypeConditional;
      cp.conditional.handle = h;
      cp.conditional.type = cudaGraphCondTypeWhile;
      cp.conditional.size = 1;
      e = cudaGraphAddNode(&wnode, graph, deps, nullptr, ndeps, &cp);
      if (e == cudaSuccess) body = cp.conditional.phGraph_out[0];
    }
    if (e == cudaSuccess)
      e = cudaStreamUpdateCaptureDependencies(r.s, &wnode, nullptr, 1,
                                              cudaStreamSetCaptureDependencies);
    if (e == cudaSuccess)
      e = cudaStreamBeginCaptureToGraph(k->stream2, body, nullptr, nullptr, 0,
                                        cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) {
      set_error(std::string("building the solver graph: ") + cudaGetErrorString(e));
      st = GP_ERR_CUDA;
    } else {
      Run rb = r;
      rb.s = k->stream2;
      const bool own = body_ends_trip(r);
      // several gated copies of the body per conditional trip amortise the
      // conditional node's re-launch; copies after convergence are no-ops
      const int unroll = body_unroll(r);
      for (int u = 0; u < unroll && st == GP_OK; u++) {
        const bool last = u + 1 == unroll;
        rb.loop = own && last ? 2 : 0;
        rb.cond = h;
        st = run_body(rb, b, x);
      }
      if (st == GP_OK && !own) {
        cudaError_t el = launch_pdl(k_loop_ctrl, 1, 1, k->stream2, h, k->st);
        if (el != cudaSuccess) {
          set_error(std::string("loop control launch: ") + cudaGetErrorString(el));
          st = GP_ERR_CUDA;
        }
      }
      cudaGraph_t bout = nullptr;
      cudaError_t eb = cudaStreamEndCapture(k->stream2, &bout);
      if (st == GP_OK && eb != cudaSuccess) {
        set_error(std::string("body capture: ") + cudaGetErrorString(eb));
        st = GP_ERR_CUDA;
      }
    }
    if (st == GP_OK && k->opt.type == KSP_BCGS) st = bcgs_epilogue(r, x);
    if (st == GP_OK) {
      cudaError_t em = cudaMemcpyAsync(k->h_st, k->st, sizeof(KspState), cudaMemcpyDeviceToHost, r.s);
      if (em != cudaSuccess) {
        set_error(std::string("state read-back capture: ") + cudaGetErrorString(em));
        st = GP_ERR_CUDA;
      }
    }
  }
  cudaGraph_t out = nullptr;
  cudaError_t ec = cudaStreamEndCapture(r.s, &out);
  if (st != GP_OK) {
    if (out) cudaGraphDestroy(out);
    return st;
  }
  if (ec != cudaSuccess) {
    set_error(std::string("cudaStreamEndCapture: ") + cudaGetErrorString(ec));
    return GP_ERR_CUDA;
  }
  k->graph = out;
  GP_CUDA(cudaGraphInstantiate(&k->exec, k->graph, 0));
  int64_t top = 0, inner = 0;
  GP_TRY(count_kernels(k->graph, &top));
  GP_TRY(count_kernels(body, &inner));
  k->top_kernels = top;
  k->body_kernels = inner;
  return GP_OK;
}

int ksp_solve(Ksp* k, Csr* A, Pc* pc, const double* b, double* x, KspResult* res,
              double* hist_out, int64_t hist_len, cudaStream_t caller) {
  KspOptions& o = k->opt;
  if (A->n != A->ncols) {
    set_error("the solver matrix must be square");
    return GP_ERR_ARG;
  }
  if (!pc->ready || pc->n != A->n) {
    set_error("the preconditioner is not set up for an operator of this size");
    return GP_ERR_NOT_SETUP;
  }
  if (o.type != KSP_CG && o.type != KSP_BCGS && o.type != KSP_GMRES && o.type != KSP_FGMRES) {
    set_error("unsupported KSP type");
    return GP_ERR_UNSUPPORTED;
  }
  const bool gm = o.type == KSP_GMRES || o.type == KSP_FGMRES;
  if (gm && (o.restart < 1 || o.restart + 1 > kMaxBasis)) {
    set_error("GMRES restart must be between 1 and " + std::to_string(kMaxBasis - 1));
    return GP_ERR_UNSUPPORTED;
  }
  if (o.max_it < 0) o.max_it = 0;
  const int n = A->n;
  k->n = n;
  bool moved = false;
  GP_TRY(ensure(k, n, &moved));
  cudaStream_t s = k->stream;
  cudaEvent_t ev;
  GP_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  GP_CUDA(cudaEventRecord(ev, caller));
  GP_CUDA(cudaStreamWaitEvent(s, ev, 0));
  // configuration into the device state
  KspState& h = *k->h_st;
  std::memset(&h, 0, sizeof(KspState));
  h.rtol = o.rtol;
  h.atol = o.atol;
  h.divtol = o.divtol;
  h.haptol = o.haptol;
  h.breakdowntol = o.breakdowntol;
  h.rhs_norm = o.rhs_norm;
  h.normtype = o.normtype;
  h.pc_side = o.pc_side;
  h.guess_zero = o.guess_zero;
  h.min_it = o.min_it;
  h.chknorm = o.chknorm;
  h.convmaxits = o.convmaxits;
  h.max_it = o.max_it;
  h.m = o.restart;
  h.seed_rhs = o.seed_rhs;
  h.cgstype = o.cgstype;
  h.c_one = 1.0;
  h.prev_rnorm = -1.0;
  GP_CUDA(cudaMemcpyAsync(k->st, &h, sizeof(KspState), cudaMemcpyHostToDevice, s));
  GP_CUDA(cudaMemsetAsync(k->hist, 0, (size_t)k->hist_cap * sizeof(double), s));
  // a zero initial guess means x = 0 on entry (KSP.solve zeroes x first,
  // python/mojopetsc4py/PETSc/KSP.py:367-449): done here for every caller
  if (o.guess_zero && n) GP_CUDA(cudaMemsetAsync(x, 0, (size_t)n * sizeof(double), s));
  if (k->transpose) {
    // host work and value gathers of the transposed solve, outside capture
    GP_TRY(spmv_t_prepare(s, A));
    GP_TRY(pc_transpose_prepare(pc, s));
  }
  GP_TRY(pc_values_sync(pc, s));
  Run r{k, A, pc, n, s};
  // the solve graph depends on the buffers and on every option that shapes
  // it; the operator and the PC set-up by their unique ids (an address can
  // come back from the allocator for a new object)
  const int key[13] = {o.type,      o.normtype,    o.pc_side,    o.restart,
                       o.cgstype,   n,             pc->opt.type, pc->opt.sor_flag,
                       o.guess_zero, 0,            arith_mode(), o.orthog,
                       k->transpose};
  if (k->launch_form == 1 || (k->launch_form < 0 && eager_mode())) {
    GP_TRY(run_eager(r, b, x));
  } else {
  const bool same = !moved && k->exec && k->cap_A == A && k->cap_pc == pc &&
                    k->cap_A_uid == A->uid && k->cap_pc_gen == pc->generation &&
                    std::equal(key, key + 13, k->cap_key) && k->cap_b == b && k->cap_x == x;
  if (!same) {
    GP_TRY(capture(r, b, x));
    k->cap_A = A;
    k->cap_pc = pc;
    k->cap_A_uid = A->uid;
    k->cap_pc_gen = pc->generation;
    k->cap_b = b;
    k->cap_x = x;
    std::copy(key, key + 13, k->cap_key);
  }
  GP_CUDA(cudaGraphLaunch(k->exec, s));
  }
  GP_CUDA(cudaEventRecord(ev, s));
  GP_CUDA(cudaStreamWaitEvent(caller, ev, 0));
  GP_CUDA(cudaStreamSynchronize(s));
  cudaEventDestroy(ev);
  GP_TRY(pc_check(pc, s));
  res->its = h.its;
  res->reason = h.reason;
  res->rnorm = h.rnorm;
  k->last_trips = h.trips;
  if (hist_out && hist_len > 0) {
    const int64_t cnt = std::min<int64_t>(hist_len, std::min<int64_t>(h.its + 1, k->hist_cap));
    GP_CUDA(cudaMemcpy(hist_out, k->hist, (size_t)cnt * sizeof(double), cudaMemcpyDeviceToHost));
    for (int64_t i = cnt; i < hist_len; i++) hist_out[i] = 0.0;
  }
  return GP_OK;
}

}  // namespace gp
