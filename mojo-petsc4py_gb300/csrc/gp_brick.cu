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
// what decides the speed is the cost of a level.  In the level-ordered form a
// level is an L2 round trip; here most hand-offs stay on the SM:
//
//   * the grid's lines along i are grouped into bricks of BJ x BK lines (all
//     of i); one CTA takes a brick and each thread walks one line, so the
//     i - 1 value is in a register and the j - 1 and k - 1 values are the
//     previous level's values of the neighbouring threads in shared memory
//     (double buffered by level parity, one barrier per level);
//   * only rows on a brick's low j or k face read a value of another brick,
//     through the value-as-flag array in global memory (a signalling NaN
//     marks "not yet"); those loads, like every load of a row's coefficients,
//     right-hand side and diagonal, are issued kBrickAhead levels before the
//     row is computed, into a register ring indexed by the level (uniform
//     across the CTA, so the ring stays in registers), and no load depends on
//     another load's value;
//   * bricks are handed out by a ticket in wavefront order (J + K); a brick
//     depends only on the bricks at J - 1 and K - 1, which CTAs that are
//     already running hold, so the sweep cannot deadlock whatever the number
//     of resident CTAs.
//
// Every row is the reference's fold of its terms in ascending-column order,
// with the same operations as k_ell_sweep: results are bit-identical to the
// reference's sequential sweeps and to the other two forms.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "gp_pc.h"

namespace gp {

constexpr int kBrickMaxLines = 256;  // threads (lines) per CTA
constexpr int kBrickAhead = 3;       // levels between a row's loads and its use
constexpr int kBrickRing = 4;        // ring slots (kBrickAhead + 1)
constexpr int kBrickSpin = 1 << 22;  // polls before a wait gives up

struct BrickArgs {
  int n, nx, ny, nz;
  int BJ, BK, nbricks;
  int in_ident;            // in_idx is the identity
  const int* border;       // [2 * nbricks]: (J, K) in hand-out order
  const double* coef;      // [3][n] by direction i, j, k; 0 where the row has no such term
  const int* in_idx;
  const int* out_idx;      // ILU_B / ICC_B output index
  const double* dval;
  double* val;             // this sweep's value-as-flag array (by row)
  const double* fval;      // the forward sweep's values (backward sweeps)
  double* aux;
  const double* auxin;
  const double* idiag;
  double om1;
  int use_t, write_out;
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

// What a row needs, loaded kBrickAhead levels before it is computed.
struct BrickRow {
  double ci, cj, ck;          // coefficients by direction
  double sum0;                // the row's starting value
  double dv;                  // diagonal factor (ILU_B, ICC_F, SOR)
  double yf;                  // SOR_B: the forward value
  int out;                    // output index (ILU_B, ICC_B)
  unsigned long long ej, ek;  // neighbour-brick values (bits) for j and k
};

__device__ __forceinline__ double brick_value(unsigned long long bits, const double* p,
                                              DevErr* err) {
  for (int spins = 0; bits == kPending; spins++) {
    if (spins >= kBrickSpin) {
      if (atomicCAS(&err->code, 0, GP_ERR_TIMEOUT) == 0) err->where = 40;
      return __longlong_as_double(0x7FF8000000000000LL);
    }
    bits = ld_relaxed_bits(p);
  }
  return __longlong_as_double((long long)bits);
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

// ORD 0 folds k, j, i; ORD 1 folds i, j, k.
template <int MODE, bool FMA, int ORD>
__global__ void __launch_bounds__(kBrickMaxLines) k_brick_sweep(const int* gate, int want,
                                                                BrickArgs a, DRef inr,
                                                                DRef outr) {
  if (gated_off(gate, want)) return;
  constexpr bool BWD = brick_bwd<MODE>();
  const double* __restrict__ in = inr.get();
  double* __restrict__ out = outr.get();
  __shared__ double sh[2][kBrickMaxLines];
  __shared__ int s_brick;
  const int t = threadIdx.x;
  const int lj = t % a.BJ, lk = t / a.BJ;
  const int nx = a.nx, ny = a.ny, nz = a.nz, n = a.n;
  const int offj = nx, offk = nx * ny;
  const double absent = brick_absent<MODE>();
  const unsigned long long absent_bits = (unsigned long long)__double_as_longlong(absent);
  for (;;) {
    if (t == 0) s_brick = (int)atomicAdd(&a.tickets[0], 1u);
    __syncthreads();
    const int b = s_brick;
    __syncthreads();  // every thread has read s_brick before it changes
    if (b >= a.nbricks) break;
    const int J = a.border[2 * b], K = a.border[2 * b + 1];
    const int gj = J * a.BJ + lj, gk = K * a.BK + lk;
    const bool line = lk < a.BK && gj < ny && gk < nz;
    const int bj = min(a.BJ, ny - J * a.BJ), bk = min(a.BK, nz - K * a.BK);
    const int nlev = nx + bj + bk - 2;
    const int skew = lj + lk;
    // the line's rows: r0 + step * li, li = 0 .. nx - 1
    const int f0 = nx * (gj + ny * gk);
    const int r0 = BWD ? n - 1 - f0 : f0;
    constexpr int step = BWD ? -1 : 1;
    // neighbour-brick faces (j and k only: a brick holds whole lines)
    const bool fj = line && lj == 0 && gj > 0, fk = line && lk == 0 && gk > 0;
    if (line) {
      const int lo = BWD ? r0 - (nx - 1) : r0;
      for (int d = 0; d < 3; d++) l2_prefetch(a.coef + (size_t)d * n + lo, (size_t)nx * 8);
      if constexpr (MODE == ELL_ILU_F || MODE == ELL_ICC_F || MODE == ELL_SOR_F ||
                    MODE == ELL_SOR_B)
        l2_prefetch(in + lo, (size_t)nx * 8);
      if constexpr (MODE == ELL_ILU_B) l2_prefetch(a.fval + lo, (size_t)nx * 8);
      if constexpr (MODE == ELL_ICC_B) l2_prefetch(a.auxin + lo, (size_t)nx * 8);
      if constexpr (MODE == ELL_ILU_B || MODE == ELL_ICC_F)
        l2_prefetch(a.dval + lo, (size_t)nx * 8);
      if constexpr (MODE == ELL_SOR_F || MODE == ELL_SOR_B)
        l2_prefetch(a.idiag + lo, (size_t)nx * 8);
    }
    auto load = [&](int li, BrickRow& w) {
      if (!line || li < 0 || li >= nx) return;
      const int r = r0 + step * li;
      w.ci = a.coef[r];
      w.cj = a.coef[(size_t)n + r];
      w.ck = a.coef[2 * (size_t)n + r];
      const int ii = a.in_ident ? r : a.in_idx[r];
      if constexpr (MODE == ELL_ILU_F || MODE == ELL_ICC_F) w.sum0 = in[ii];
      if constexpr (MODE == ELL_ILU_B) w.sum0 = a.fval[ii];
      if constexpr (MODE == ELL_ICC_B) w.sum0 = a.auxin[ii];
      if constexpr (MODE == ELL_SOR_F) w.sum0 = in[r];
      if constexpr (MODE == ELL_SOR_B) {
        w.sum0 = a.use_t ? a.auxin[ii] : in[r];
        w.yf = a.use_t ? a.fval[ii] : 0.0;
      }
      if constexpr (MODE == ELL_ILU_B || MODE == ELL_ICC_F) w.dv = a.dval[r];
      if constexpr (MODE == ELL_SOR_F || MODE == ELL_SOR_B) w.dv = a.idiag[r];
      if constexpr (MODE == ELL_ILU_B || MODE == ELL_ICC_B) w.out = a.out_idx[r];
      w.ej = fj ? ld_relaxed_bits(&a.val[BWD ? r + offj : r - offj]) : absent_bits;
      w.ek = fk ? ld_relaxed_bits(&a.val[BWD ? r + offk : r - offk]) : absent_bits;
    };
    BrickRow ring[kBrickRing];
#pragma unroll
    for (int q = 0; q < kBrickAhead; q++) load(q - skew, ring[q]);
    double prev = absent;  // the line's previous value (none before its first row)
    for (int L0 = 0; L0 < nlev; L0 += kBrickRing) {
#pragma unroll
      for (int q = 0; q < kBrickRing; q++) {
        const int L = L0 + q;
        if (L + kBrickAhead < nlev)
          load(L + kBrickAhead - skew, ring[(q + kBrickAhead) % kBrickRing]);
        const BrickRow& w = ring[q];
        const int par = L & 1;
        const int li = L - skew;
        if (line && li >= 0 && li < nx) {
          const int r = r0 + step * li;
          const double vj = lj > 0 ? sh[par ^ 1][t - 1]
                                   : brick_value(w.ej, &a.val[BWD ? r + offj : r - offj], a.err);
          const double vk = lk > 0 ? sh[par ^ 1][t - a.BJ]
                                   : brick_value(w.ek, &a.val[BWD ? r + offk : r - offk], a.err);
          double sum = w.sum0;
          if constexpr (ORD == 0) {
            sum = brick_term<MODE, FMA>(sum, w.ck, vk);
            sum = brick_term<MODE, FMA>(sum, w.cj, vj);
            sum = brick_term<MODE, FMA>(sum, w.ci, prev);
          } else {
            sum = brick_term<MODE, FMA>(sum, w.ci, prev);
            sum = brick_term<MODE, FMA>(sum, w.cj, vj);
            sum = brick_term<MODE, FMA>(sum, w.ck, vk);
          }
          double y;
          if constexpr (MODE == ELL_ILU_F) {
            y = sum;
          } else if constexpr (MODE == ELL_ILU_B) {
            y = mul(sum, w.dv);
            out[w.out] = y;
          } else if constexpr (MODE == ELL_ICC_F) {
            a.aux[r] = mul(sum, w.dv);
            y = sum;
          } else if constexpr (MODE == ELL_ICC_B) {
            y = sum;
            out[w.out] = y;
          } else if constexpr (MODE == ELL_SOR_F) {
            a.aux[r] = sum;
            y = mul(sum, w.dv);
            if (a.write_out) out[r] = y;
          } else {
            y = a.use_t ? add(mul(a.om1, w.yf), mul(sum, w.dv)) : mul(sum, w.dv);
            out[r] = y;
          }
          st_relaxed(&a.val[r], y);
          sh[par][t] = y;
          prev = y;
        }
        __syncthreads();
      }
    }
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
// GPETSC_BRICK_DIMS=JxK and GPETSC_BRICK_CTAS_PER_SM set the defaults).
struct BrickTuning {
  int mode = 0;        // 0 never, 1 where the model says it is faster, 2 wherever it applies
  int BJ = 0, BK = 0;  // 0: chosen by the model
  int ctas_per_sm = 2;
  int max_ctas = 0;    // cap on the persistent grid (0: none)
};
static BrickTuning& brick_tuning() {
  static BrickTuning t = [] {
    BrickTuning v;
    if (const char* e = std::getenv("GPETSC_SWEEP_BRICKS"))
      v.mode = std::max(0, std::min(2, std::atoi(e)));
    if (const char* e = std::getenv("GPETSC_BRICK_DIMS")) std::sscanf(e, "%dx%d", &v.BJ, &v.BK);
    if (const char* e = std::getenv("GPETSC_BRICK_CTAS_PER_SM"))
      v.ctas_per_sm = std::max(1, std::min(16, std::atoi(e)));
    return v;
  }();
  return t;
}

void set_sweep_bricks(int mode, int bj, int bk, int max_ctas) {
  brick_tuning().mode = mode;
  brick_tuning().BJ = bj;
  brick_tuning().BK = bk;
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

// Modelled duration of one brick sweep (us): the critical path in levels --
// each brick runs its neighbour's face width plus a hand-off behind it --
// times the cost of a level, which grows once a CTA's lines outrun the SM's
// FP64 rate.
static double brick_model_us(int nx, int ny, int nz, int BJ, int BK) {
  const double lat_level_us = 0.14, handoff_levels = 6.0;
  const int nbJ = (ny + BJ - 1) / BJ, nbK = (nz + BK - 1) / BK;
  const double crit = (nbJ - 1) * (BJ + handoff_levels) + (nbK - 1) * (BK + handoff_levels) +
                      (nx + BJ + BK - 2);
  // FP64: ~4 dependent operations a row; one warp instruction per 19 cycles a SM
  const double lines = (double)BJ * BK;
  const double thr_level_us = lines * 4.0 / 32.0 * 19.0 / 2.07e3;
  return crit * std::max(lat_level_us, thr_level_us);
}

int brick_build(EllSweep& e, int mode, int n, bool forward, const std::vector<int>& dptr,
                const std::vector<int>& dcol, const std::vector<int>& dsl,
                const std::vector<int>& in_row, const std::vector<int>& out_row,
                const std::vector<int>& dslot_row, double other_us, bool* built) {
  *built = false;
  const BrickTuning& tu = brick_tuning();
  if (tu.mode == 0 || n == 0) return GP_OK;
  int nx, ny, nz, ord;
  std::vector<int> slot;
  if (!brick_detect(n, forward, dptr, dcol, dsl, &nx, &ny, &nz, &ord, slot)) return GP_OK;
  // brick shape: BJ x BK lines, at most kBrickMaxLines
  int BJ = tu.BJ, BK = tu.BK;
  double best = 0.0;
  if (BJ <= 0 || BK <= 0 || BJ * BK > kBrickMaxLines) {
    BJ = BK = 0;
    const int cand[] = {1, 2, 4, 8, 16, 32, 64, 128, 256};
    for (int bj : cand)
      for (int bk : cand) {
        if (bj * bk > kBrickMaxLines || bj * bk < 8) continue;
        if (bj > 2 * ny && bj > 1) continue;
        if (bk > 2 * nz && bk > 1) continue;
        const double est = brick_model_us(nx, ny, nz, bj, bk);
        if (!BJ || est < best) {
          BJ = bj;
          BK = bk;
          best = est;
        }
      }
    if (!BJ) return GP_OK;
  } else {
    best = brick_model_us(nx, ny, nz, BJ, BK);
  }
  if (tu.mode == 1 && !(best < other_us)) return GP_OK;
  const int nbJ = (ny + BJ - 1) / BJ, nbK = (nz + BK - 1) / BK;
  // hand-out order: wavefronts J + K, then K
  std::vector<int> border;
  border.reserve(2 * (size_t)nbJ * nbK);
  for (int w = 0; w <= nbJ + nbK - 2; w++)
    for (int K = 0; K < nbK; K++) {
      const int J = w - K;
      if (J < 0 || J >= nbJ) continue;
      border.push_back(J);
      border.push_back(K);
    }
  // per-row data in natural row order: coefficient slots by direction in the
  // layout the ELL refresh gathers ([d][n]; -1, no term, refreshes to 0),
  // input / output / diagonal slots
  const int W = 3;
  std::vector<int> cnt(n, W), in(n, 0), out(n, -1), ds(n, 0);
  bool in_ident = true;
  for (int r = 0; r < n; r++) {
    in[r] = in_row.empty() ? r : in_row[r];
    in_ident = in_ident && in[r] == r;
    if (!out_row.empty()) out[r] = out_row[r];
    if (!dslot_row.empty()) ds[r] = dslot_row[r];
  }
  ell_free(e);
  e.n = n;
  e.W = W;
  GP_TRY(bup(&e.cnt, cnt));
  GP_TRY(bup(&e.cslot, slot));
  GP_TRY(bup(&e.in_idx, in));
  GP_TRY(bup(&e.out_idx, out));
  if (!dslot_row.empty()) GP_TRY(bup(&e.dslot, ds));
  GP_TRY(bup(&e.border, border));
  GP_CUDA(cudaMalloc(&e.coef, (size_t)W * n * sizeof(double)));
  GP_CUDA(cudaMalloc(&e.dval, std::max(n, 1) * sizeof(double)));
  e.brick = true;
  e.gx = nx;
  e.gy = ny;
  e.gz = nz;
  e.BJ = BJ;
  e.BK = BK;
  e.bord = ord;
  e.nbricks = nbJ * nbK;
  e.in_ident = in_ident;
  e.est_us = best;
  e.bgrid = std::max(1, std::min(e.nbricks, num_sms() * tu.ctas_per_sm));
  if (tu.max_ctas > 0) e.bgrid = std::min(e.bgrid, tu.max_ctas);
  e.ok = true;
  if (std::getenv("GPETSC_SWEEP_VERBOSE"))
    std::fprintf(stderr,
                 "gpetsc sweep: n=%d bricks grid %dx%dx%d lines %dx%d bricks=%d grid=%d "
                 "est=%.0fus (other form %.0fus)\n",
                 n, nx, ny, nz, BJ, BK, e.nbricks, e.bgrid, best, other_us);
  *built = true;
  return GP_OK;
}

template <int MODE, bool FMA>
static void brick_launch_a(const EllSweep& e, const int* gate, int want, const BrickArgs& a,
                           DRef in, DRef out, cudaStream_t s) {
  const int threads = ((e.BJ * e.BK + 31) / 32) * 32;
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
  a.n = e.n;
  a.nx = e.gx;
  a.ny = e.gy;
  a.nz = e.gz;
  a.BJ = e.BJ;
  a.BK = e.BK;
  a.nbricks = e.nbricks;
  a.in_ident = e.in_ident ? 1 : 0;
  a.border = e.border;
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
