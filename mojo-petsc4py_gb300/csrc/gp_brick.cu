// Brick form of the triangular sweeps (ILU, IC and SOR applies,
// src/ported.mojo:633-748, 864-952) for sweeps whose dependencies are the
// unit steps of a Cartesian grid in natural order -- the 5- and 7-point
// stencils, upwind convection-diffusion, any operator with that pattern.
//
// On such a grid (nx, ny, nz) a forward sweep's row r = i + nx (j + ny k)
// depends on r - 1 (i - 1), r - nx (j - 1) and r - nx ny (k - 1), each present
// exactly when that coordinate is >= 1; a backward sweep on r + 1, r + nx,
// r + nx ny (mirrored coordinates make both "coordinate minus one").  The
// dependency chain is nx + ny + nz - 2 levels long whatever the schedule, so
// what decides the speed is the cost of a level.  On GB300 a hand-off between
// two SMs through L2 takes ~0.45 us (store, poll and return) while a
// dependent FP64 operation takes 64 cycles, so a level whose inputs are on
// the SM costs a fraction of one that waits on another SM:
//
//   * a brick is BJ consecutive lines along i of one plane k (all of i).
//     One CTA takes a brick and each compute thread walks one line, line t
//     reaching row i at step s = i + t: the i - 1 value is the thread's own
//     previous one, the j - 1 value the previous step's value of thread t - 1
//     (shared memory, double buffered by step parity, one barrier of the
//     compute warps a step);
//   * rows are stored by position, step-major within a brick: position
//     base + s BJ + t (positions with no row are holes), so a warp's loads of
//     coefficients and diagonals and its stores of values are contiguous;
//   * the k - 1 values (the same step and line of the brick one plane below)
//     and the j - 1 values of line 0 (the brick below in j) come from other
//     CTAs.  Fetch warps poll them in global memory (the value-as-flag array;
//     a signalling NaN marks "not yet") -- a warp 32 lines at a time, one
//     coalesced load a step, several steps in flight -- and drop each step's
//     values into a shared-memory ring slot once all of them are in.  A
//     compute thread takes its value from the slot (normally already there)
//     and frees it; a fetch warp fills a slot only once it is free, so it runs
//     at most a ring's length ahead.  The compute warps never wait on a global
//     poll, and a brick that runs a hand-off behind its neighbour pays only
//     the on-SM chain per step;
//   * each row's coefficients, right-hand side and diagonal are loaded
//     kBrickAhead steps before use into a register ring indexed by the step
//     (uniform across the CTA, so the ring stays in registers);
//   * bricks are handed out by a ticket in wavefront order (J + K); a brick
//     depends only on the bricks at J - 1 and K - 1, which CTAs that are
//     already running hold, so the sweep cannot deadlock whatever the number
//     of resident CTAs.  Within a CTA the fetch warps wait only on other
//     bricks and on slots the compute threads free in step order, and every
//     wait has an iteration budget.
//
// Every row is the reference's fold of its terms in ascending-column order,
// with the same operations as k_ell_sweep: results are bit-identical to the
// reference's sequential sweeps and to the other forms.
#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "gp_pc.h"

namespace gp {

constexpr int kBrickMaxLines = 128;                  // compute threads (lines) per CTA
constexpr int kBrickMaxFace = kBrickMaxLines + 1;    // ring columns: BJ k-face lines, the j face
constexpr int kBrickKWarps = kBrickMaxLines / 32;    // fetch warps of the k face
constexpr int kBrickThreads = kBrickMaxLines + 32 * (kBrickKWarps + 1);
constexpr int kBrickAhead = 4;       // steps between a row's loads and its use
constexpr int kBrickIdxAhead = 8;    // steps between a row's input index load and its use
constexpr int kBrickRing = 9;        // register ring slots (kBrickIdxAhead + 1)
constexpr int kBrickSlots = 16;      // shared-memory ring slots per column (power of 2)
constexpr int kBrickPoll = 4;        // steps a fetch warp keeps in flight
constexpr int kBrickSpin = 1 << 22;  // polls before a wait gives up

struct BrickArgs {
  int nrows, npos;         // rows of the sweep; positions (holes included)
  int nx, ny, nz, BJ, nbJ, nbricks;
  int in_ident, out_ident;  // in_idx / out_idx are the row itself
  const int* border;       // [2 * nbricks]: (J, K) in hand-out order
  const int* bbase;        // [nbJ * nz]: first position of brick (J, K) at J + nbJ K
  const double* coef;      // [3][npos] by direction i, j, k; 0 where the row has no such term
  const int* in_idx;       // [npos]
  const int* out_idx;      // [npos]
  const double* dval;      // [npos]
  double* val;             // this sweep's value-as-flag array (by position)
  const double* fval;      // the forward sweep's values (backward sweeps)
  double* aux;             // by position
  const double* auxin;
  const double* idiag;     // by row (SOR)
  double om1;
  int use_t, write_out;
  int fetch_sleep_ns;      // back-off of a fetch warp that saw nothing new
  unsigned* tickets;
  DevErr* err;
};

// A row's fold is three terms in a fixed direction order -- (k, j, i) or
// (i, j, k), the reference's ascending-column slot order -- for every row: a
// term the row does not have (at the grid boundary) has coefficient 0 and
// value `absent`, and c * absent = -0 for ILU / SOR (sum - c v) and IC
// (sum + c v) alike, which leaves every sum, -0 included, unchanged: the same
// bits as skipping the term.
template <int MODE>
__device__ __forceinline__ double brick_absent() {
  return (MODE == ELL_ICC_F || MODE == ELL_ICC_B) ? -0.0 : 0.0;
}

template <int MODE, bool FMA>
__device__ __forceinline__ double brick_term(double sum, double c, double v) {
  if constexpr (MODE == ELL_ICC_F || MODE == ELL_ICC_B)
    return FMA ? __fma_rn(c, v, sum) : add(sum, mul(c, v));
  else
    return FMA ? __fma_rn(-c, v, sum) : sub(sum, mul(c, v));
}

template <int MODE>
__host__ __device__ constexpr bool brick_bwd() {
  return MODE == ELL_ILU_B || MODE == ELL_ICC_B || MODE == ELL_SOR_B;
}

// What a row needs, loaded kBrickAhead steps before it is computed.
struct BrickRow {
  double ci, cj, ck;          // coefficients by direction
  double sum0;                // the row's starting value
  double dv;                  // diagonal factor (ILU_B, ICC_F, SOR)
  double yf;                  // SOR_B: the forward value
  int out;                    // output index (ILU_B, ICC_B, SOR)
};

__device__ __forceinline__ bool brick_failed(DevErr* err) {
  return *reinterpret_cast<volatile int*>(&err->code) != 0;
}

// Take a value from its shared-memory ring slot and free the slot.
__device__ __forceinline__ double brick_take(double* slot, DevErr* err) {
  volatile unsigned long long* q = reinterpret_cast<volatile unsigned long long*>(slot);
  unsigned long long b = *q;
  for (int spins = 0; b == kPending; spins++) {
    // give up at the budget, or early once another wait has given up
    if (spins >= kBrickSpin || ((spins & 4095) == 4095 && brick_failed(err))) {
      if (atomicCAS(&err->code, 0, GP_ERR_TIMEOUT) == 0) err->where = 41;
      b = 0x7FF8000000000000ULL;
      break;
    }
    b = *q;
  }
  *q = kPending;
  return __longlong_as_double((long long)b);
}

// Bulk prefetch of [p, p + bytes) into L2 (the 16-byte aligned interior of
// the range; a hint that occupies no registers).
__device__ __forceinline__ void l2_prefetch(const void* p, size_t bytes) {
  const uintptr_t a = ((uintptr_t)p + 15) & ~(uintptr_t)15;
  const uintptr_t e = ((uintptr_t)p + bytes) & ~(uintptr_t)15;
  if (e > a)
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a), "r"((unsigned)(e - a))
                 : "memory");
}

__device__ __forceinline__ void compute_barrier(int nc) {
  asm volatile("bar.sync 1, %0;" ::"r"(nc) : "memory");
}

// One fetch warp: each active lane has a ring column `col` and values for
// steps [qlo, qhi) at val[src + q * stride].  The warp walks the steps in
// order and hands a step's values to the ring once every lane that has one
// sees it, each into its slot once the slot is free; kBrickPoll steps are
// polled together.
__device__ void brick_fetch(const BrickArgs& a, double* ring, bool act, int col, int qlo,
                            int qhi, long long src, int stride) {
  const unsigned full = 0xffffffffu;
  volatile unsigned long long* cv = reinterpret_cast<volatile unsigned long long*>(ring) + col;
  const int wq0 = __reduce_min_sync(full, act ? qlo : INT_MAX);
  const int wq1 = __reduce_max_sync(full, act ? qhi : INT_MIN);
  int q0 = wq0, spins = 0, held = 0;
  while (q0 < wq1) {
    bool ok[kBrickPoll];
    unsigned long long bits[kBrickPoll];
    bool run = true;
#pragma unroll
    for (int d = 0; d < kBrickPoll; d++) {
      const int q = q0 + d;
      const bool need = act && q >= qlo && q < qhi;
      const bool fr = !need || cv[(size_t)(q & (kBrickSlots - 1)) * kBrickMaxFace] == kPending;
      run = run && q < wq1 && __all_sync(full, fr);
      ok[d] = run;
      bits[d] = run && need ? ld_relaxed_bits(&a.val[src + (long long)q * stride]) : 0ull;
    }
    int got = 0;
    run = true;
#pragma unroll
    for (int d = 0; d < kBrickPoll; d++) {
      const int q = q0 + d;
      const bool need = act && q >= qlo && q < qhi;
      run = run && ok[d] && __all_sync(full, !need || bits[d] != kPending);
      if (run) {
        if (need) cv[(size_t)(q & (kBrickSlots - 1)) * kBrickMaxFace] = bits[d];
        got++;
      }
    }
    if (got) {
      q0 += got;
      spins = held = 0;
      continue;
    }
    // nothing handed on: the ring is full (the compute threads are a ring
    // behind) or a value is not in yet
    const bool failed = ((spins + held) & 1023) == 1023 && brick_failed(a.err);
    if (!ok[0]) {
      if (++held > kBrickSpin || failed) {
        if (atomicCAS(&a.err->code, 0, GP_ERR_TIMEOUT) == 0) a.err->where = 42;
        return;
      }
    } else if (++spins > kBrickSpin || failed) {
      // a value never arrived: record it and hand on quiet NaNs for the step
      if (atomicCAS(&a.err->code, 0, GP_ERR_TIMEOUT) == 0) a.err->where = 43;
      const bool need = act && q0 >= qlo && q0 < qhi;
      if (need) cv[(size_t)(q0 & (kBrickSlots - 1)) * kBrickMaxFace] = 0x7FF8000000000000ULL;
      q0++;
      spins = 0;
      continue;
    }
    if (a.fetch_sleep_ns > 0) __nanosleep(a.fetch_sleep_ns);
  }
}

// ORD 0 folds k, j, i; ORD 1 folds i, j, k.  Launched with nc + nf threads:
// nc = BJ rounded up to warps compute, nf = 32 (ceil(BJ / 32) + 1) fetch.
template <int MODE, bool FMA, int ORD>
__global__ void __launch_bounds__(kBrickThreads, 1) k_brick_sweep(const int* gate, int want,
                                                                  BrickArgs a, DRef inr,
                                                                  DRef outr) {
  if (gated_off(gate, want)) return;
  constexpr bool BWD = brick_bwd<MODE>();
  const double* __restrict__ in = inr.get();
  double* __restrict__ out = outr.get();
  __shared__ double sh[2][kBrickMaxLines];
  // value rings: [slot][column]; columns 0..BJ-1 the k face (line t of the
  // brick one plane below), column BJ the j face (the last line of the brick
  // below in j)
  __shared__ double ring[kBrickSlots * kBrickMaxFace];
  __shared__ int s_brick;
  const int t = threadIdx.x;
  const int BJ = a.BJ;
  const int nc = (BJ + 31) / 32 * 32;
  const int nx = a.nx, ny = a.ny, npos = a.npos;
  const double absent = brick_absent<MODE>();
  const double pend = __longlong_as_double((long long)kPending);
  for (int q = t; q < kBrickSlots * kBrickMaxFace; q += blockDim.x) ring[q] = pend;
  for (;;) {
    if (t == 0) s_brick = (int)atomicAdd(&a.tickets[0], 1u);
    __syncthreads();
    const int b = s_brick;
    __syncthreads();  // every thread has read s_brick before it changes
    if (b >= a.nbricks) break;
    const int J = a.border[2 * b], K = a.border[2 * b + 1];
    const int bj = min(BJ, ny - J * BJ);
    const int base = a.bbase[J + a.nbJ * K];
    const int nsteps = nx + bj - 1;
    if (t >= nc) {
      // ---- fetch warps: the k face (lines 32 w .. 32 w + 31), then the j face
      const int w = (t - nc) >> 5, lane = (t - nc) & 31;
      if (w < (BJ + 31) / 32) {
        if (K > 0) {
          const int lt = 32 * w + lane;
          brick_fetch(a, ring, lt < bj, lt, lt, lt + nx,
                      (long long)a.bbase[J + a.nbJ * (K - 1)] + lt, BJ);
        }
      } else if (J > 0) {
        // line 0 at step q = i takes row i of line BJ - 1 of brick (J - 1, K),
        // which that brick reached at its step i + BJ - 1
        brick_fetch(a, ring, lane == 0, BJ, 0, nx,
                    (long long)a.bbase[J - 1 + a.nbJ * K] + (long long)(BJ - 1) * BJ + BJ - 1,
                    BJ);
      }
    } else {
      // ---- compute: one line a thread
      const bool line = t < bj;
      const long long f_lo = (long long)nx * (J * BJ + (long long)ny * K);  // brick's first row
      if (t == 0) {
        // the brick's positions, and (forward sweeps) its rows of the input
        const size_t pb = (size_t)nsteps * BJ * 8;
        for (int d = 0; d < 3; d++) l2_prefetch(a.coef + (size_t)d * npos + base, pb);
        if constexpr (MODE == ELL_ILU_B || MODE == ELL_ICC_F) l2_prefetch(a.dval + base, pb);
        if (!a.in_ident) l2_prefetch(a.in_idx + base, pb / 2);
        if (!a.out_ident) l2_prefetch(a.out_idx + base, pb / 2);
        const long long r_lo = BWD ? a.nrows - f_lo - (long long)nx * bj : f_lo;
        if constexpr (MODE == ELL_ILU_F || MODE == ELL_ICC_F || MODE == ELL_SOR_F ||
                      MODE == ELL_SOR_B)
          l2_prefetch(in + r_lo, (size_t)nx * bj * 8);
        if constexpr (MODE == ELL_SOR_F || MODE == ELL_SOR_B)
          l2_prefetch(a.idiag + r_lo, (size_t)nx * bj * 8);
      }
      // Every load of the ring is unconditional: a row outside the line's
      // range (before its first step, after its last, or a line past the
      // brick's edge) loads the nearest row of the brick instead, so no load
      // result feeds a select and each stays in flight until its step.  The
      // input index (a gather through in_idx) is loaded kBrickIdxAhead steps
      // ahead, the row data kBrickAhead steps ahead.
      const int tl = min(t, bj - 1);
      const long long fl = (long long)nx * (J * BJ + tl + (long long)ny * K);
      auto clamp_li = [&](int s) { return min(max(s - tl, 0), nx - 1); };
      auto row_at = [&](int li) {
        return BWD ? (int)(a.nrows - 1 - (fl + li)) : (int)(fl + li);
      };
      int ixr[kBrickRing];
      auto load_idx = [&](int s, int& ix) {
        if (!a.in_ident) ix = a.in_idx[base + (clamp_li(s) + tl) * BJ + tl];
      };
      auto load = [&](int s, int ix, BrickRow& w) {
        const int li = clamp_li(s);
        const int p = base + (li + tl) * BJ + tl;
        const int r = row_at(li);
        w.ci = a.coef[p];
        w.cj = a.coef[(size_t)npos + p];
        w.ck = a.coef[2 * (size_t)npos + p];
        const int ii = a.in_ident ? r : ix;
        if constexpr (MODE == ELL_ILU_F || MODE == ELL_ICC_F) w.sum0 = in[ii];
        if constexpr (MODE == ELL_ILU_B) w.sum0 = a.fval[ii];
        if constexpr (MODE == ELL_ICC_B) w.sum0 = a.auxin[ii];
        if constexpr (MODE == ELL_SOR_F) w.sum0 = in[r];
        if constexpr (MODE == ELL_SOR_B) {
          if (a.use_t) {
            w.sum0 = a.auxin[ii];
            w.yf = a.fval[ii];
          } else {
            w.sum0 = in[r];
            w.yf = 0.0;
          }
        }
        if constexpr (MODE == ELL_ILU_B || MODE == ELL_ICC_F) w.dv = a.dval[p];
        if constexpr (MODE == ELL_SOR_F || MODE == ELL_SOR_B) w.dv = a.idiag[r];
        if constexpr (MODE == ELL_ILU_B || MODE == ELL_ICC_B)
          w.out = a.out_ident ? r : a.out_idx[p];
        if constexpr (MODE == ELL_SOR_F || MODE == ELL_SOR_B) w.out = r;
      };
      BrickRow rr[kBrickRing];
#pragma unroll
      for (int q = 0; q < kBrickIdxAhead; q++) load_idx(q, ixr[q]);
#pragma unroll
      for (int q = 0; q < kBrickAhead; q++) load(q, ixr[q], rr[q]);
      double prev = absent;  // the line's previous value (none before its first row)
      double* const col_k = ring + t;
      double* const col_j = ring + BJ;
      for (int L0 = 0; L0 < nsteps; L0 += kBrickRing) {
#pragma unroll
        for (int q = 0; q < kBrickRing; q++) {
          const int L = L0 + q;
          if (L + kBrickIdxAhead < nsteps)
            load_idx(L + kBrickIdxAhead, ixr[(q + kBrickIdxAhead) % kBrickRing]);
          if (L + kBrickAhead < nsteps)
            load(L + kBrickAhead, ixr[(q + kBrickAhead) % kBrickRing],
                 rr[(q + kBrickAhead) % kBrickRing]);
          const BrickRow& w = rr[q];
          const int par = L & 1;
          const int li = L - t;
          const size_t so = (size_t)(L & (kBrickSlots - 1)) * kBrickMaxFace;
          if (line && li >= 0 && li < nx) {
            double sum = w.sum0;
            if constexpr (ORD == 0) {
              const double vk = K > 0 ? brick_take(col_k + so, a.err) : absent;
              sum = brick_term<MODE, FMA>(sum, w.ck, vk);
              const double vj =
                  t > 0 ? sh[par ^ 1][t - 1] : J > 0 ? brick_take(col_j + so, a.err) : absent;
              sum = brick_term<MODE, FMA>(sum, w.cj, vj);
              sum = brick_term<MODE, FMA>(sum, w.ci, prev);
            } else {
              sum = brick_term<MODE, FMA>(sum, w.ci, prev);
              const double vj =
                  t > 0 ? sh[par ^ 1][t - 1] : J > 0 ? brick_take(col_j + so, a.err) : absent;
              sum = brick_term<MODE, FMA>(sum, w.cj, vj);
              const double vk = K > 0 ? brick_take(col_k + so, a.err) : absent;
              sum = brick_term<MODE, FMA>(sum, w.ck, vk);
            }
            // the value other bricks wait on goes out first
            double y;
            if constexpr (MODE == ELL_ILU_B || MODE == ELL_SOR_F)
              y = mul(sum, w.dv);
            else if constexpr (MODE == ELL_SOR_B)
              y = a.use_t ? add(mul(a.om1, w.yf), mul(sum, w.dv)) : mul(sum, w.dv);
            else
              y = sum;
            const int p = base + L * BJ + t;
            st_relaxed(&a.val[p], y);
            sh[par][t] = y;
            prev = y;
            if constexpr (MODE == ELL_ILU_B || MODE == ELL_ICC_B) {
              out[w.out] = y;
            } else if constexpr (MODE == ELL_ICC_F) {
              a.aux[p] = mul(sum, w.dv);
            } else if constexpr (MODE == ELL_SOR_F) {
              a.aux[p] = sum;
              if (a.write_out) out[w.out] = y;
            } else if constexpr (MODE == ELL_SOR_B) {
              out[w.out] = y;
            }
          }
          compute_barrier(nc);
        }
      }
    }
    __syncthreads();
  }
  if (t == 0 && atomic_add_acq_rel(&a.tickets[1], 1u) == gridDim.x - 1) {
    a.tickets[0] = 0u;
    a.tickets[1] = 0u;
  }
}

// ------------------------------------------------------------------ host
template <typename T>
static int bup(T** d, const std::vector<T>& h) {
  GP_CUDA(cudaMalloc(d, std::max<size_t>(h.size(), 1) * sizeof(T)));
  if (!h.empty()) GP_CUDA(cudaMemcpy(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
  return GP_OK;
}

// Settings of later set-ups (gp_set_sweep_bricks; GPETSC_SWEEP_BRICKS,
// GPETSC_BRICK_LINES, GPETSC_BRICK_CTAS_PER_SM and GPETSC_BRICK_FETCH_SLEEP_NS
// set the defaults).
struct BrickTuning {
  int mode = 0;        // 0 never, 1 where the model says it is faster, 2 wherever it applies
  int BJ = 0;          // lines of a brick; 0: chosen by the model
  int ctas_per_sm = 1;
  int max_ctas = 0;    // cap on the persistent grid (0: none)
  int fetch_sleep_ns = 0;
};
static BrickTuning& brick_tuning() {
  static BrickTuning t = [] {
    BrickTuning v;
    if (const char* e = std::getenv("GPETSC_SWEEP_BRICKS"))
      v.mode = std::max(0, std::min(2, std::atoi(e)));
    if (const char* e = std::getenv("GPETSC_BRICK_LINES"))
      v.BJ = std::max(0, std::min(kBrickMaxLines, std::atoi(e)));
    if (const char* e = std::getenv("GPETSC_BRICK_CTAS_PER_SM"))
      v.ctas_per_sm = std::max(1, std::min(4, std::atoi(e)));
    if (const char* e = std::getenv("GPETSC_BRICK_FETCH_SLEEP_NS"))
      v.fetch_sleep_ns = std::max(0, std::min(1000, std::atoi(e)));
    return v;
  }();
  return t;
}

void set_sweep_bricks(int mode, int lines, int max_ctas) {
  brick_tuning().mode = mode;
  brick_tuning().BJ = lines;
  brick_tuning().max_ctas = max_ctas;
}

// Grid detection: every row r (in sweep coordinates f = r forward, n-1-r
// backward; i = f % nx, j = f / nx % ny, k = f / (nx ny)) depends on exactly
// its grid neighbours r -/+ 1 (when i >= 1), nx (j >= 1) and nx ny (k >= 1),
// listed in one direction order for every row -- k, j, i (ord 0) or i, j, k
// (ord 1) -- so that each row's fold is the three-term fold with absent
// terms at the grid boundary.  On success slot[d][r] is the coefficient slot
// of row r's term in direction d (-1 where it has none).
static bool brick_detect(int n, bool forward, const std::vector<int>& dptr,
                         const std::vector<int>& dcol, const std::vector<int>& dsl,
                         int* nx_out, int* ny_out, int* nz_out, int* ord_out,
                         std::vector<int>& slot) {
  std::vector<long long> offs;
  for (int r = 0; r < n; r++) {
    if (dptr[r + 1] - dptr[r] > 3) return false;
    for (int q = dptr[r]; q < dptr[r + 1]; q++) {
      const long long o = forward ? (long long)r - dcol[q] : (long long)dcol[q] - r;
      if (o <= 0) return false;
      if (std::find(offs.begin(), offs.end(), o) == offs.end()) {
        offs.push_back(o);
        if (offs.size() > 3) return false;
      }
    }
  }
  std::sort(offs.begin(), offs.end());
  if (offs.empty() || offs[0] != 1) return false;
  const long long nx = offs.size() >= 2 ? offs[1] : n;
  const long long nxny = offs.size() >= 3 ? offs[2] : n;
  if (nx <= 1 || nxny % nx || n % nxny) return false;
  const long long ny = nxny / nx;
  int ord = -1;
  slot.assign((size_t)3 * n, -1);
  for (int r = 0; r < n; r++) {
    const long long f = forward ? r : (long long)n - 1 - r;
    const long long i = f % nx, j = (f / nx) % ny, k = f / nxny;
    const int want = (i >= 1 ? 1 : 0) | (j >= 1 ? 2 : 0) | (k >= 1 ? 4 : 0);
    int seen = 0, last = -1, up_all = -1;
    for (int q = dptr[r]; q < dptr[r + 1]; q++) {
      const long long o = forward ? (long long)r - dcol[q] : (long long)dcol[q] - r;
      const int d = o == 1 ? 0 : o == nx ? 1 : o == nxny ? 2 : -1;
      if (d < 0 || !(want >> d & 1) || (seen >> d & 1)) return false;
      if (last >= 0) {
        const int up = d > last ? 1 : 0;  // ord 1 ascends i, j, k; ord 0 descends
        if (up_all >= 0 && up != up_all) return false;
        up_all = up;
      }
      seen |= 1 << d;
      last = d;
      slot[(size_t)d * n + r] = dsl[q];
    }
    if (seen != want) return false;  // the full stencil, nothing missing
    if (up_all >= 0) {
      if (ord >= 0 && ord != up_all) return false;
      ord = up_all;
    }
  }
  *nx_out = (int)nx;
  *ny_out = (int)ny;
  *nz_out = (int)(n / nxny);
  *ord_out = ord < 0 ? 0 : ord;
  return true;
}

// Modelled duration of one brick sweep (us), from GB300 measurements: a
// step is the on-SM chain (three dependent FP64 operations of 64 cycles,
// shared memory, the compute barrier) or the SM's FP64 rate (~4 warp
// instructions a row, one a sub-partition every 64 cycles), whichever is
// longer; each brick boundary on the critical path costs a hand-off through
// L2 and the fetch ring, plus, along j, the BJ - 1 steps line BJ - 1 runs
// behind line 0.
static double brick_model_us(int nx, int ny, int nz, int BJ) {
  const double lat_step_us = 0.15, handoff_us = 0.8;
  const int nbJ = (ny + BJ - 1) / BJ;
  const int warps = (BJ + 31) / 32;
  const double step_us = std::max(lat_step_us, (warps + 3) / 4 * 4.0 * 64.0 / 2.07e3);
  return (nbJ - 1) * ((BJ - 1) * step_us + handoff_us) + (nz - 1) * handoff_us +
         (nx + BJ - 1) * step_us;
}

int brick_build(EllSweep& e, int mode, int n, bool forward, const std::vector<int>& dptr,
                const std::vector<int>& dcol, const std::vector<int>& dsl,
                const std::vector<int>& in_row, const std::vector<int>& out_row,
                const std::vector<int>& dslot_row, double other_us, bool* built,
                std::vector<int>* pos_of_row) {
  (void)mode;
  *built = false;
  const BrickTuning& tu = brick_tuning();
  if (tu.mode == 0 || n == 0) return GP_OK;
  int nx, ny, nz, ord;
  std::vector<int> slot;
  if (!brick_detect(n, forward, dptr, dcol, dsl, &nx, &ny, &nz, &ord, slot)) return GP_OK;
  // lines of a brick: at most kBrickMaxLines and the grid's ny, and at most
  // nx (a brick's steps, nx + BJ - 1, bound the holes of its layout)
  const int cap = std::min({kBrickMaxLines, ny, std::max(nx, 1)});
  int BJ = std::min(tu.BJ, cap);
  double best = 0.0;
  if (BJ <= 0) {
    std::vector<int> cand = {1, 2, 4, 8, 16, 32, 64, 128, ny};
    for (int c : cand) {
      if (c < 1 || c > cap) continue;
      const double est = brick_model_us(nx, ny, nz, c);
      if (!BJ || est < best) {
        BJ = c;
        best = est;
      }
    }
    if (!BJ) return GP_OK;
  } else {
    best = brick_model_us(nx, ny, nz, BJ);
  }
  if (tu.mode == 1 && !(best < other_us)) return GP_OK;
  const int nbJ = (ny + BJ - 1) / BJ;
  const long long nbricks = (long long)nbJ * nz;
  if (nbricks > INT_MAX / 2) return GP_OK;
  // hand-out order: wavefronts J + K, then K; positions are assigned in the
  // same order, BJ per step of each brick
  std::vector<int> border, bbase((size_t)nbricks, 0);
  border.reserve(2 * (size_t)nbricks);
  long long P = 0;
  for (long long w = 0; w <= nbJ + nz - 2; w++)
    for (long long K = std::max(0LL, w - (nbJ - 1)); K <= std::min<long long>(w, nz - 1); K++) {
      const int J = (int)(w - K);
      border.push_back(J);
      border.push_back((int)K);
      bbase[(size_t)J + (size_t)nbJ * K] = (int)P;
      const int bj = std::min(BJ, ny - J * BJ);
      P += (long long)(nx + bj - 1) * BJ;
      if (P > INT_MAX - 1) return GP_OK;  // positions are int32
    }
  // per-position data: coefficient slots by direction ([d][P]; -1 no term,
  // refreshed to 0), input / output / diagonal slots; holes have no terms
  const int W = 3;
  std::vector<int> cnt((size_t)P, 0), cs((size_t)3 * P, -1), in((size_t)P, 0), out((size_t)P, 0),
      ds((size_t)P, 0), pos(n);
  bool in_ident = true, out_ident = true;
  const long long nxny = (long long)nx * ny;
  for (int r = 0; r < n; r++) {
    const long long f = forward ? r : (long long)n - 1 - r;
    const int i = (int)(f % nx), j = (int)((f / nx) % ny), k = (int)(f / nxny);
    const int J = j / BJ, t = j % BJ;
    const long long p = (long long)bbase[(size_t)J + (size_t)nbJ * k] + (long long)(i + t) * BJ + t;
    pos[r] = (int)p;
    cnt[p] = W;
    for (int d = 0; d < 3; d++) cs[(size_t)d * P + p] = slot[(size_t)d * n + r];
    in[p] = in_row.empty() ? r : in_row[r];
    out[p] = out_row.empty() ? r : out_row[r];
    in_ident = in_ident && in[p] == r;
    out_ident = out_ident && out[p] == r;
    if (!dslot_row.empty()) ds[p] = dslot_row[r];
  }
  ell_free(e);
  e.n = (int)P;
  e.nrows = n;
  e.W = W;
  GP_TRY(bup(&e.cnt, cnt));
  GP_TRY(bup(&e.cslot, cs));
  if (!in_ident) GP_TRY(bup(&e.in_idx, in));
  if (!out_ident) GP_TRY(bup(&e.out_idx, out));
  if (!dslot_row.empty()) GP_TRY(bup(&e.dslot, ds));
  GP_TRY(bup(&e.border, border));
  GP_TRY(bup(&e.bbase, bbase));
  GP_CUDA(cudaMalloc(&e.coef, (size_t)W * P * sizeof(double)));
  GP_CUDA(cudaMalloc(&e.dval, std::max<long long>(P, 1) * sizeof(double)));
  e.brick = true;
  e.gx = nx;
  e.gy = ny;
  e.gz = nz;
  e.BJ = BJ;
  e.BK = 1;
  e.nbJ = nbJ;
  e.bord = ord;
  e.nbricks = (int)nbricks;
  e.in_ident = in_ident;
  e.out_ident = out_ident;
  e.est_us = best;
  e.bgrid = (int)std::max<long long>(1, std::min<long long>(nbricks, (long long)num_sms() * tu.ctas_per_sm));
  if (tu.max_ctas > 0) e.bgrid = std::min(e.bgrid, tu.max_ctas);
  e.ok = true;
  if (pos_of_row) *pos_of_row = pos;
  if (std::getenv("GPETSC_SWEEP_VERBOSE"))
    std::fprintf(stderr,
                 "gpetsc sweep: n=%d bricks grid %dx%dx%d lines %d bricks=%lld positions=%lld "
                 "grid=%d est=%.0fus (other form %.0fus)\n",
                 n, nx, ny, nz, BJ, nbricks, P, e.bgrid, best, other_us);
  *built = true;
  return GP_OK;
}

template <int MODE, bool FMA>
static void brick_launch_a(const EllSweep& e, const int* gate, int want, const BrickArgs& a,
                           DRef in, DRef out, cudaStream_t s) {
  // compute threads (a line each), then the fetch warps: the k face 32
  // lines a warp, and one for the j face
  const int threads = (e.BJ + 31) / 32 * 32 + 32 * ((e.BJ + 31) / 32 + 1);
  if (e.bord == 0)
    k_brick_sweep<MODE, FMA, 0><<<e.bgrid, threads, 0, s>>>(gate, want, a, in, out);
  else
    k_brick_sweep<MODE, FMA, 1><<<e.bgrid, threads, 0, s>>>(gate, want, a, in, out);
}

template <int MODE>
static void brick_launch(const EllSweep& e, const int* gate, int want, const BrickArgs& a,
                         DRef in, DRef out, cudaStream_t s) {
  if (arith_mode() == kFma)
    brick_launch_a<MODE, true>(e, gate, want, a, in, out, s);
  else
    brick_launch_a<MODE, false>(e, gate, want, a, in, out, s);
}

int brick_sweep(int mode, const EllSweep& e, const int* gate, int want, DRef in, DRef out,
                double* val, const double* fval, double* aux, const double* auxin,
                const double* idiag, double omega, int use_t, int write_out, unsigned* tickets,
                DevErr* err, cudaStream_t s) {
  if (e.n == 0) return GP_OK;
  BrickArgs a;
  a.nrows = e.nrows;
  a.npos = e.n;
  a.nx = e.gx;
  a.ny = e.gy;
  a.nz = e.gz;
  a.BJ = e.BJ;
  a.nbJ = e.nbJ;
  a.nbricks = e.nbricks;
  a.in_ident = e.in_ident ? 1 : 0;
  a.out_ident = e.out_ident ? 1 : 0;
  a.border = e.border;
  a.bbase = e.bbase;
  a.coef = e.coef;
  a.in_idx = e.in_idx;
  a.out_idx = e.out_idx;
  a.dval = e.dval;
  a.val = val;
  a.fval = fval;
  a.aux = aux;
  a.auxin = auxin;
  a.idiag = idiag;
  a.om1 = 1.0 - omega;
  a.use_t = use_t;
  a.write_out = write_out;
  a.fetch_sleep_ns = brick_tuning().fetch_sleep_ns;
  a.tickets = tickets;
  a.err = err;
  switch (mode) {
    case ELL_ILU_F: brick_launch<ELL_ILU_F>(e, gate, want, a, in, out, s); break;
    case ELL_ILU_B: brick_launch<ELL_ILU_B>(e, gate, want, a, in, out, s); break;
    case ELL_ICC_F: brick_launch<ELL_ICC_F>(e, gate, want, a, in, out, s); break;
    case ELL_ICC_B: brick_launch<ELL_ICC_B>(e, gate, want, a, in, out, s); break;
    case ELL_SOR_F: brick_launch<ELL_SOR_F>(e, gate, want, a, in, out, s); break;
    case ELL_SOR_B: brick_launch<ELL_SOR_B>(e, gate, want, a, in, out, s); break;
  }
  GP_CHECK_LAUNCH();
  return GP_OK;
}

}  // namespace gp
