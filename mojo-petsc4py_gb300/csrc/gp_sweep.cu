// Level-ordered ELL sweeps: the fast form of the sync-free triangular sweeps
// of the ILU, IC and SOR applies (src/ported.mojo:633-748, 864-952).
//
// Each sweep is laid out on the host once, in processing order: position p
// holds row order[p]; its dependencies (at most W) are stored column-major as
// (position of the dependency, coefficient), so consecutive positions -- one
// warp -- load their coefficients and dependency positions with unit stride.
// A thread first loads everything that does not depend on other rows
// (coefficients, dependency positions, its right-hand-side entry, its
// diagonal), and only then waits on the values it needs; the wait-to-store
// chain between two levels is one L2 round trip.  Values live in
// value-as-flag arrays indexed by position.  Each row's sum is taken in the
// reference's slot order with rounded multiplies and adds, so the result is
// bit-identical to the sequential loop.
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <exception>
#include <functional>
#include <limits>
#include <map>
#include <mutex>
#include <queue>
#include <string>
#include <thread>
#include <vector>

#include "gp_pc.h"

namespace gp {

constexpr int kEllBlock = 256;
constexpr int kEllSpin = 1 << 22;
constexpr int kTileSmemMax = 227 * 1024;  // dynamic shared memory limit of one CTA
constexpr int kTileBulkPiece = 16384;     // bytes per bulk copy instruction
constexpr int kTileHeader = 8;  // ints: levels, rows, Lp, Cp, external entries, Ep, Cp8, 0

__device__ __forceinline__ double ell_wait(const double* p, DevErr* err, int where,
                                           int budget = kEllSpin, int sleep_after = 64,
                                           int sleep_ns = 20) {
  unsigned long long b = ld_relaxed_bits(p);
  if (b != kPending) return __longlong_as_double((long long)b);
  for (int spins = 0; spins < budget; spins++) {
    if (spins >= sleep_after && sleep_ns > 0) __nanosleep(sleep_ns);
    b = ld_relaxed_bits(p);
    if (b != kPending) return __longlong_as_double((long long)b);
  }
  if (atomicCAS(&err->code, 0, GP_ERR_TIMEOUT) == 0) err->where = where;
  return __longlong_as_double(0x7FF8000000000000LL);
}


// One dependency term of a sweep row: sum - c*v (ILU, SOR) or sum + c*v (IC),
// rounded after the product and after the sum (the reference's arithmetic),
// or fused into one rounding in the FMA arithmetic.
template <int MODE, bool FMA>
__device__ __forceinline__ double sweep_term(double sum, double c, double v) {
  if constexpr (MODE == ELL_ICC_F || MODE == ELL_ICC_B)
    return FMA ? __fma_rn(c, v, sum) : add(sum, mul(c, v));
  else
    return FMA ? __fma_rn(-c, v, sum) : sub(sum, mul(c, v));
}

struct EllArgs {
  int n;
  const int* cnt;
  const int* dep;
  const double* coef;
  const int* in_idx;   // per position: input index (b / x row, or forward position)
  const int* out_idx;  // per position: output index, or -1
  const double* dval;  // per position: diagonal factor (ILU_B, ICC_F)
  const int* rowof;    // per position: row (SOR: idiag index)
  double* val;         // this sweep's value-as-flag array
  const double* fval;  // the forward sweep's values (backward sweeps)
  double* aux;         // ICC_F: scaled values ys; SOR_F: checkpoint t
  const double* auxin; // ICC_B: ys; SOR_B: t
  const double* idiag; // SOR
  double om1;          // SOR: 1 - omega
  int use_t;           // SOR_B
  int write_out;       // SOR_F: also write y (no backward half follows)
  unsigned* tickets;
  DevErr* err;
  int sleep_after, sleep_ns;  // polling back-off of the waits
};

// Launch shape and polling back-off of the sweeps (GPETSC_SWEEP_CTAS_PER_SM,
// GPETSC_SWEEP_SLEEP_AFTER, GPETSC_SWEEP_SLEEP_NS override the defaults).
struct SweepTuning {
  // best of a scan (1-4 CTAs a SM x 0-300 ns back-off) of the level-ordered
  // IC(0)/ILU(0)/SOR sweeps on 128^3 with the per-lane polling kernel
  int ctas_per_sm = 1, sleep_after = 8, sleep_ns = 0;
  int block = kEllBlock;  // GPETSC_SWEEP_BLOCK: threads of a level-ordered sweep CTA (32-256)
  int tiles = 1;                // GPETSC_SWEEP_TILES=0: always the level-ordered ELL form
  int tile_smem = kTileSmemMax;  // GPETSC_TILE_SMEM: shared memory cap of one chunk
  int tile_rows = 0;            // GPETSC_TILE_ROWS: force this chunk size (0: chosen)
};
static SweepTuning& sweep_tuning_mut() {
  static SweepTuning t = [] {
    SweepTuning v;
    auto env = [](const char* k, int d) {
      const char* e = std::getenv(k);
      return e ? std::atoi(e) : d;
    };
    v.ctas_per_sm = std::max(1, std::min(8, env("GPETSC_SWEEP_CTAS_PER_SM", v.ctas_per_sm)));
    v.sleep_after = std::max(0, env("GPETSC_SWEEP_SLEEP_AFTER", v.sleep_after));
    v.sleep_ns = std::max(0, std::min(1000, env("GPETSC_SWEEP_SLEEP_NS", v.sleep_ns)));
    v.block = std::max(1, std::min(kEllBlock / 32, env("GPETSC_SWEEP_BLOCK", v.block) / 32)) * 32;
    v.tiles = env("GPETSC_SWEEP_TILES", v.tiles) != 0;
    v.tile_smem = std::max(16 * 1024, std::min(kTileSmemMax, env("GPETSC_TILE_SMEM", v.tile_smem)));
    v.tile_rows = std::max(0, std::min(8192, env("GPETSC_TILE_ROWS", v.tile_rows)));
    return v;
  }();
  return t;
}
static const SweepTuning& sweep_tuning() { return sweep_tuning_mut(); }

void set_sweep_form(int tiles, int tile_rows) {
  sweep_tuning_mut().tiles = tiles != 0;
  sweep_tuning_mut().tile_rows = std::max(0, std::min(8192, tile_rows));
}

template <int MODE, int WMAX, bool FMA>
__global__ void __launch_bounds__(kEllBlock) k_ell_sweep(const int* gate, int want, EllArgs a,
                                                         DRef inr, DRef outr) {
  if (gated_off(gate, want)) return;
  const double* __restrict__ in = inr.get();
  double* __restrict__ out = outr.get();
  const int n = a.n;
  const int lane = threadIdx.x & 31;
  for (;;) {
    unsigned base = 0;
    if (lane == 0) base = atomicAdd(&a.tickets[0], 32u);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= (unsigned)n) break;
    const int p = (int)base + lane;
    // ---- everything that does not wait
    int c = 0;
    int dp[WMAX];
    double cf[WMAX];
    double sum = 0.0, dv = 0.0, yf = 0.0;
    if (p < n) {
      c = a.cnt[p];
#pragma unroll
      for (int e = 0; e < WMAX; e++) {
        if (e < c) {
          dp[e] = a.dep[(size_t)e * n + p];
          cf[e] = a.coef[(size_t)e * n + p];
        }
      }
      if constexpr (MODE == ELL_ILU_F) {
        // from an earlier sweep's values when given (the transposed apply)
        sum = (a.fval ? a.fval : in)[a.in_idx[p]];
      } else if constexpr (MODE == ELL_ICC_F) {
        sum = in[a.in_idx[p]];
        dv = a.dval[p];
      } else if constexpr (MODE == ELL_ILU_B) {
        sum = (a.fval ? a.fval : in)[a.in_idx[p]];
        dv = a.dval[p];
      } else if constexpr (MODE == ELL_ICC_B) {
        sum = a.auxin[a.in_idx[p]];
      } else if constexpr (MODE == ELL_SOR_F) {
        sum = in[a.rowof[p]];
        dv = a.idiag[a.rowof[p]];
      } else {  // ELL_SOR_B
        const int fp = a.in_idx[p];
        sum = a.use_t ? a.auxin[fp] : in[a.rowof[p]];
        yf = a.use_t ? a.fval[fp] : 0.0;
        dv = a.idiag[a.rowof[p]];
      }
    }
    // ---- the dependency chain, in the reference's slot order.  Every
    // dependency is loaded up front (independent loads).  Then the warp
    // polls in lock step, but each lane folds its dependencies in order as
    // they arrive and stores its result in the same step as its last one:
    // no lane waits for the slowest of its warp before publishing.
    unsigned long long bits[WMAX];
#pragma unroll
    for (int e = 0; e < WMAX; e++)
      if (e < c) bits[e] = ld_relaxed_bits(&a.val[dp[e]]);
    // FP64 instructions are issued only behind warp votes: on this GPU a warp
    // FP64 instruction holds its sub-partition's FP64 unit for the same time
    // whether or not any lane is active, so a poll that re-issued predicated-
    // off folds would delay the folds of the warps that are on the critical
    // path.  The published value goes out before any other store.
    int ecur = 0;
    bool fin = p >= n;
    for (int spins = 0;; spins++) {
#pragma unroll
      for (int e = 0; e < WMAX; e++) {
        const bool go = !fin && e < c && e == ecur && bits[e] != kPending;
        if (__any_sync(0xffffffffu, go)) {
          if (go) {
            sum = sweep_term<MODE, FMA>(sum, cf[e], __longlong_as_double((long long)bits[e]));
            ecur++;
          }
        }
      }
      const bool done = !fin && ecur >= c;
      if (__any_sync(0xffffffffu, done) && done) {
        if constexpr (MODE == ELL_ILU_F) {
          st_relaxed(&a.val[p], sum);
          if (a.out_idx) out[a.out_idx[p]] = sum;
        } else if constexpr (MODE == ELL_ILU_B) {
          const double y = mul(sum, dv);
          st_relaxed(&a.val[p], y);
          if (a.out_idx) out[a.out_idx[p]] = y;
        } else if constexpr (MODE == ELL_ICC_F) {
          st_relaxed(&a.val[p], sum);
          a.aux[p] = mul(sum, dv);
        } else if constexpr (MODE == ELL_ICC_B) {
          st_relaxed(&a.val[p], sum);
          out[a.out_idx[p]] = sum;
        } else if constexpr (MODE == ELL_SOR_F) {
          const double y = mul(sum, dv);
          st_relaxed(&a.val[p], y);
          a.aux[p] = sum;
          if (a.out_idx) out[a.rowof[p]] = y;
        } else {
          const double y = a.use_t ? add(mul(a.om1, yf), mul(sum, dv)) : mul(sum, dv);
          st_relaxed(&a.val[p], y);
          out[a.rowof[p]] = y;
        }
        fin = true;
      }
      if (__all_sync(0xffffffffu, fin)) break;
      if (!fin) {
        if (spins >= kEllSpin) {
          // a dependency never arrived: record it and fold quiet NaNs
          if (atomicCAS(&a.err->code, 0, GP_ERR_TIMEOUT) == 0) a.err->where = 20 + MODE;
#pragma unroll
          for (int e = 0; e < WMAX; e++)
            if (e < c && bits[e] == kPending) bits[e] = 0x7FF8000000000000ULL;
        } else {
          if (spins >= a.sleep_after && a.sleep_ns > 0) __nanosleep(a.sleep_ns);
#pragma unroll
          for (int e = 0; e < WMAX; e++)
            if (e < c && e >= ecur && bits[e] == kPending) bits[e] = ld_relaxed_bits(&a.val[dp[e]]);
        }
      }
    }
  }
  if (lane == 0) {
    const unsigned total = gridDim.x * (blockDim.x / 32);
    if (atomic_add_acq_rel(&a.tickets[1], 1u) == total - 1) {
      a.tickets[0] = 0u;
      a.tickets[1] = 0u;
    }
  }
}

// ------------------------------------------------------------ tiled sweeps
//
// A chunk is a run of consecutive rows of the sweep's natural sequence
// (ascending rows forward, descending backward).  Inside a chunk its rows are
// sorted by their dependency level counted over the chunk's own rows.  One
// CTA of two warps takes a chunk: the compute warp walks it level by level,
// reading dependencies inside the chunk from shared memory (one __syncwarp
// between levels), while the fetch warp polls the chunk's dependencies in
// earlier chunks (the global value-as-flag array) in level order, several in
// flight per lane, and drops each into a shared-memory value-as-flag slot.
// The compute warp therefore pays an L2 round trip only where a value from
// another chunk arrives just in time, not on every level.  On a grid
// numbered in natural order most dependencies are neighbours inside the same
// chunk; the chunk size is chosen on the host by simulating the schedule
// (tile_choose), so chunk boundaries fall where the dependency chains break.
// Each chunk's level offsets, dependency counts, encoded dependencies,
// output indices and external positions form one contiguous blob staged
// with cp.async.bulk on an mbarrier; coefficients, diagonals and right-hand
// sides are gathered from global memory meanwhile.  Chunks are handed out by
// a ticket in order and a chunk waits only on earlier chunks, which running
// CTAs already hold, so the sweep cannot deadlock on CTAs that are not yet
// resident.  Per row the arithmetic and the dependency order are those of
// k_ell_sweep, so the results are bit-identical.

constexpr int kTileThreads = 128;  // warp 0 computes, warps 1-3 fetch; all gather
constexpr int kTileNoDep = -32768;  // int16 dependency code of an absent slot

// Per-row shared-memory columns a mode needs beyond coefficients, values and
// sums: a diagonal factor, and for the SOR backward half the forward value.
__host__ __device__ constexpr bool tile_has_dv(int mode) {
  return mode == ELL_ILU_B || mode == ELL_ICC_F || mode == ELL_SOR_F || mode == ELL_SOR_B;
}
__host__ __device__ constexpr int tile_extra_cols(int mode) {
  return (tile_has_dv(mode) ? 1 : 0) + (mode == ELL_SOR_B ? 1 : 0);
}

struct TileArgs {
  int nchunks, W, C, max_blob;
  const unsigned char* blob;
  const long long* blob_off;
  const int* cstart;
  const double* coefsrc;
};

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

// Bounded wait for the mbarrier phase `parity` to complete.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity, int budget) {
  const unsigned a = smem_u32(bar);
  for (int i = 0; i < budget; i++) {
    unsigned done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// global -> shared bulk copy (16-byte aligned addresses, size a multiple of 16)
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes,
                                         unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void st_shared_volatile(double* p, double v) {
  *reinterpret_cast<volatile double*>(p) = v;
}

// Wait for a shared-memory value-as-flag slot written by the fetch warp.  The
// fetch warp's own waits are bounded and write a NaN when they give up, so
// this budget only guards against a slot that is never written.
__device__ __forceinline__ double smem_wait(const double* p, DevErr* err, int where) {
  volatile const unsigned long long* q = reinterpret_cast<volatile const unsigned long long*>(p);
  unsigned long long b = *q;
  for (int i = 0; b == kPending && i < (1 << 26); i++) {
    if (i >= 64) __nanosleep(32);
    b = *q;
  }
  if (b == kPending) {
    if (atomicCAS(&err->code, 0, GP_ERR_TIMEOUT) == 0) err->where = where;
    return __longlong_as_double(0x7FF8000000000000LL);
  }
  return __longlong_as_double((long long)b);
}

template <int MODE, int WMAX, bool FMA>
__global__ void __launch_bounds__(kTileThreads, 1) k_tile_sweep(const int* gate, int want,
                                                                EllArgs a, TileArgs t, DRef inr,
                                                                DRef outr) {
  if (gated_off(gate, want)) return;
  extern __shared__ __align__(16) unsigned char sm[];
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(sm);
  unsigned* s_chunk = reinterpret_cast<unsigned*>(sm + 8);
  int* blob = reinterpret_cast<int*>(sm + 16);
  const int W = t.W, C = t.C;
  double* s_cf = reinterpret_cast<double*>(sm + 16 + t.max_blob);  // [W][C]
  double* s_val = s_cf + (size_t)(W > 0 ? W : 1) * C;
  double* s_sum = s_val + C;
  double* s_dv = s_sum + C;                            // modes with a diagonal
  double* s_yf = s_dv + (tile_has_dv(MODE) ? C : 0);   // SOR backward only
  double* s_ext = s_yf + (MODE == ELL_SOR_B ? C : 0);  // external values, value-as-flag
  const double* __restrict__ in = inr.get();
  double* __restrict__ out = outr.get();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) mbar_init(bar, 1);
  __syncthreads();
  unsigned parity = 0;
  for (;;) {
    if (tid == 0) *s_chunk = atomicAdd(&a.tickets[0], 1u);
    __syncthreads();
    const unsigned c = *s_chunk;
    if (c >= (unsigned)t.nchunks) break;
    const int cs = t.cstart[c];
    // ---- stage the chunk's blob (one elected thread issues the bulk copies)
    if (tid == 0) {
      const long long b0 = t.blob_off[c];
      const unsigned bytes = (unsigned)(t.blob_off[c + 1] - b0);
      // earlier generic reads of the blob area come before the async writes
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_expect_tx(bar, bytes);
      for (unsigned off = 0; off < bytes; off += kTileBulkPiece)
        bulk_g2s(sm + 16 + off, t.blob + b0 + off, min((unsigned)kTileBulkPiece, bytes - off),
                 bar);
    }
    const bool staged = mbar_wait(bar, parity, kEllSpin);
    if (!staged) {
      if (lane == 0 && atomicCAS(&a.err->code, 0, GP_ERR_TIMEOUT) == 0) a.err->where = 40 + MODE;
      // let the copies in flight land before leaving; a bulk copy that has
      // not landed after this second bounded wait is not recovered from: the
      // CTA leaves with the timeout recorded and the host reports the sweep
      // as failed (GP_ERR_TIMEOUT)
      mbar_wait(bar, parity, kEllSpin);
    }
    parity ^= 1u;
    if (__syncthreads_or(!staged)) break;
    const int nl = blob[0], Cc = blob[1], Lp = blob[2], Cp = blob[3], Ne = blob[4];
    const int Ep = blob[5], Cp8 = blob[6];
    const int* lo = blob + kTileHeader;
    const int* oidx = lo + Lp;
    const int* iidx = oidx + Cp;
    const int* gidx = iidx + Cp;
    const int* csl = gidx + Cp;
    const int* epos = csl + (size_t)W * Cp;
    const short* dep = reinterpret_cast<const short*>(epos + Ep);  // [W][Cp8]
    // ---- gathers that do not wait: coefficients, initial sums, diagonals
#pragma unroll 4
    for (int r = tid; r < Cc; r += kTileThreads) {
#pragma unroll
      for (int e = 0; e < WMAX; e++) {
        if (e < W) {
          const int slot = csl[(size_t)e * Cp + r];
          if (slot >= 0) s_cf[(size_t)e * C + r] = t.coefsrc[slot];
        }
      }
      if constexpr (MODE == ELL_ILU_F) {
        // from an earlier sweep's values when given (the transposed apply)
        s_sum[r] = (a.fval ? a.fval : in)[iidx[r]];
      } else if constexpr (MODE == ELL_ICC_F) {
        s_sum[r] = in[iidx[r]];
        s_dv[r] = t.coefsrc[gidx[r]];
      } else if constexpr (MODE == ELL_ILU_B) {
        s_sum[r] = (a.fval ? a.fval : in)[iidx[r]];
        s_dv[r] = t.coefsrc[gidx[r]];
      } else if constexpr (MODE == ELL_ICC_B) {
        s_sum[r] = a.auxin[iidx[r]];
      } else if constexpr (MODE == ELL_SOR_F) {
        s_sum[r] = in[gidx[r]];
        s_dv[r] = a.idiag[gidx[r]];
      } else {  // ELL_SOR_B
        const int fp = iidx[r];
        s_sum[r] = a.use_t ? a.auxin[fp] : in[gidx[r]];
        s_yf[r] = a.use_t ? a.fval[fp] : 0.0;
        s_dv[r] = a.idiag[gidx[r]];
      }
    }
    const double pend = __longlong_as_double((long long)kPending);
    for (int k = tid; k < Ne; k += kTileThreads) s_ext[k] = pend;
    __syncthreads();
    if (warp > 0) {
      // ---- fetch: external dependencies in level order.  Each lane follows
      // two strided streams of the list and stores each value the moment it
      // sees it, so no value waits for another lane's.
      const int f = tid - 32, nf = kTileThreads - 32;
      int k1 = f, k2 = f + nf;
      int sp1 = 0, sp2 = 0;
      for (;;) {
        const bool a1 = k1 < Ne, a2 = k2 < Ne;
        if (!__any_sync(0xffffffffu, a1 || a2)) break;
        const unsigned long long b1 = a1 ? ld_relaxed_bits(&a.val[epos[k1]]) : 0ull;
        const unsigned long long b2 = a2 ? ld_relaxed_bits(&a.val[epos[k2]]) : 0ull;
        bool idle = true;
        if (a1) {
          if (b1 != kPending || ++sp1 > kEllSpin) {
            if (b1 == kPending && atomicCAS(&a.err->code, 0, GP_ERR_TIMEOUT) == 0)
              a.err->where = 30 + MODE;
            st_shared_volatile(&s_ext[k1], b1 != kPending ? __longlong_as_double((long long)b1)
                                                          : __longlong_as_double(0x7FF8000000000000LL));
            k1 += 2 * nf;
            sp1 = 0;
            idle = false;
          }
        }
        if (a2) {
          if (b2 != kPending || ++sp2 > kEllSpin) {
            if (b2 == kPending && atomicCAS(&a.err->code, 0, GP_ERR_TIMEOUT) == 0)
              a.err->where = 30 + MODE;
            st_shared_volatile(&s_ext[k2], b2 != kPending ? __longlong_as_double((long long)b2)
                                                          : __longlong_as_double(0x7FF8000000000000LL));
            k2 += 2 * nf;
            sp2 = 0;
            idle = false;
          }
        }
        if (idle && a.sleep_ns > 0 && (sp1 >= a.sleep_after || sp2 >= a.sleep_after))
          __nanosleep(a.sleep_ns);
      }
    } else {
      // ---- compute: the chunk's levels; the next level's bounds are read
      // one level ahead, and each row loads all its operands before the sum
      int b0 = lo[0], b1 = nl > 0 ? lo[1] : 0;
      for (int l = 0; l < nl; l++) {
        const int b2 = l + 2 <= nl ? lo[l + 2] : 0;
        for (int r = b0 + lane; r < b1; r += 32) {
          int dd[WMAX];
          double cf[WMAX], v[WMAX];
#pragma unroll
          for (int e = 0; e < WMAX; e++) dd[e] = e < W ? dep[(size_t)e * Cp8 + r] : kTileNoDep;
#pragma unroll
          for (int e = 0; e < WMAX; e++) {
            if (dd[e] != kTileNoDep) {
              cf[e] = s_cf[(size_t)e * C + r];
              v[e] = dd[e] >= 0
                         ? s_val[dd[e]]
                         : *reinterpret_cast<volatile const double*>(&s_ext[-dd[e] - 1]);
            }
          }
          double sum = s_sum[r];
#pragma unroll
          for (int e = 0; e < WMAX; e++) {
            if (dd[e] != kTileNoDep) {
              if (dd[e] < 0 && __double_as_longlong(v[e]) == (long long)kPending)
                v[e] = smem_wait(&s_ext[-dd[e] - 1], a.err, 50 + MODE);
              sum = sweep_term<MODE, FMA>(sum, cf[e], v[e]);
            }
          }
          const int p = cs + r;
          // the value the next levels wait on is published first
          double res;
          if constexpr (MODE == ELL_ILU_B || MODE == ELL_SOR_F)
            res = mul(sum, s_dv[r]);
          else if constexpr (MODE == ELL_SOR_B)
            res = a.use_t ? add(mul(a.om1, s_yf[r]), mul(sum, s_dv[r])) : mul(sum, s_dv[r]);
          else
            res = sum;
          s_val[r] = res;
          st_relaxed(&a.val[p], res);
          if constexpr (MODE == ELL_ILU_F || MODE == ELL_ILU_B) {
            if (a.write_out) out[oidx[r]] = res;
          } else if constexpr (MODE == ELL_ICC_F) {
            a.aux[p] = mul(sum, s_dv[r]);
          } else if constexpr (MODE == ELL_ICC_B) {
            out[oidx[r]] = res;
          } else if constexpr (MODE == ELL_SOR_F) {
            a.aux[p] = sum;
            if (a.write_out) out[oidx[r]] = res;
          } else {
            out[oidx[r]] = res;
          }
        }
        __syncwarp();
        b0 = b1;
        b1 = b2;
      }
    }
    __syncthreads();
  }
  if (tid == 0) {
    if (atomic_add_acq_rel(&a.tickets[1], 1u) == gridDim.x - 1) {
      a.tickets[0] = 0u;
      a.tickets[1] = 0u;
    }
  }
}

// The sweeps' wait, on its own: one thread waits for `flag` with the given
// budget.  With a flag that nothing sets, the wait runs out, records
// GP_ERR_TIMEOUT in `err` and returns -- the failure path every sweep takes
// when a dependency never arrives, exercised without faulting anything.
__global__ void k_wait_probe(const double* flag, int budget, DevErr* err, double* out) {
  out[0] = ell_wait(flag, err, 99, budget);
}

// coefficient (and diagonal) refresh from the factor or matrix values
__global__ void k_ell_refresh(int n, int W, const int* __restrict__ cnt,
                              const int* __restrict__ cslot, const double* __restrict__ src,
                              double* __restrict__ coef, const int* __restrict__ dslot,
                              double* __restrict__ dval) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    const int c = cnt[p];
    for (int e = 0; e < c; e++) {
      const int cs = cslot[(size_t)e * n + p];
      coef[(size_t)e * n + p] = cs >= 0 ? src[cs] : 0.0;  // < 0: no term (brick form)
    }
    if (dslot) dval[p] = src[dslot[p]];
  }
}

// ------------------------------------------------------------------ host
template <typename T>
static int up(T** d, const std::vector<T>& h) {
  GP_CUDA(cudaMalloc(d, std::max<size_t>(h.size(), 1) * sizeof(T)));
  if (!h.empty()) GP_CUDA(cudaMemcpy(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
  return GP_OK;
}

void ell_free(EllSweep& e) {
  void* ptrs[] = {e.cnt,  e.dep,   e.cslot, e.coef,     e.in_idx, e.out_idx, e.dslot,
                  e.dval, e.rowof, e.blob,  e.blob_off, e.cstart, e.border, e.bbase};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  e = EllSweep();
}

// Chunked processing order of one sweep.  The sweep's natural sequence is
// ascending rows (forward: every dependency precedes its row) or descending
// rows (backward).  Chunk c holds sequence entries [c*C, (c+1)*C); inside it,
// rows are sorted (stably) by their level over dependencies inside the chunk.
struct TilePlan {
  int C = 0;
  std::vector<int> order;    // position -> row
  std::vector<int> cstart;   // [nchunks + 1]
  std::vector<int> lvl_ptr;  // [nchunks + 1] into lvl_off
  std::vector<int> lvl_off;  // per chunk: level offsets relative to its start (levels + 1)
  int max_ext = 0, max_levels = 0;
  size_t smem = 0;
  double est_us = 0.0;
};

static int round4(int v) { return (v + 3) & ~3; }

static void tile_order(int n, const std::vector<int>& dptr, const std::vector<int>& dcol,
                       bool forward, int C, TilePlan& tp) {
  const int nch = (n + C - 1) / C;
  tp.C = C;
  tp.order.assign(n, 0);
  tp.cstart.assign(nch + 1, 0);
  tp.lvl_ptr.assign(nch + 1, 0);
  tp.lvl_off.clear();
  tp.max_ext = tp.max_levels = 0;
  std::vector<int> lev(C), cnt;
  auto row_of = [&](int q) { return forward ? q : n - 1 - q; };
  for (int c = 0; c < nch; c++) {
    const int q0 = c * C, q1 = std::min(n, q0 + C);
    int maxl = 0, next = 0;
    for (int q = q0; q < q1; q++) {
      const int i = row_of(q);
      int l = 0;
      for (int e = dptr[i]; e < dptr[i + 1]; e++) {
        const int qj = forward ? dcol[e] : n - 1 - dcol[e];
        if (qj >= q0)
          l = std::max(l, lev[qj - q0] + 1);
        else
          next++;
      }
      lev[q - q0] = l;
      maxl = std::max(maxl, l);
    }
    tp.max_ext = std::max(tp.max_ext, next);
    tp.max_levels = std::max(tp.max_levels, maxl + 1);
    cnt.assign(maxl + 2, 0);
    for (int q = q0; q < q1; q++) cnt[lev[q - q0] + 1]++;
    for (int l = 0; l <= maxl; l++) cnt[l + 1] += cnt[l];
    tp.lvl_ptr[c] = (int)tp.lvl_off.size();
    for (int l = 0; l <= maxl + 1; l++) tp.lvl_off.push_back(cnt[l]);
    for (int q = q0; q < q1; q++) tp.order[q0 + cnt[lev[q - q0]]++] = row_of(q);
    tp.cstart[c] = q0;
  }
  tp.cstart[nch] = n;
  tp.lvl_ptr[nch] = (int)tp.lvl_off.size();
}

static int round8(int v) { return (v + 7) & ~7; }

// Bytes of one chunk's blob: header, level offsets, then int32 columns
// (output index, input index, diagonal or row index, W coefficient slots),
// the external positions, and the W int16 dependency columns.
static int tile_blob_bytes(int levels, int rows, int ext, int W) {
  return 4 * (kTileHeader + round4(levels + 1) + round4(rows) * (3 + W) + round4(ext)) +
         2 * W * round8(rows);
}

static size_t tile_smem_bytes(int mode, int C, int max_levels, int max_ext, int W) {
  const int C4 = round4(C);
  return 16 + (size_t)tile_blob_bytes(max_levels, C, max_ext, W) +
         8 * ((size_t)(std::max(W, 1) + 2 + tile_extra_cols(mode)) * C4 + (size_t)max_ext);
}

// Schedule model of the two sweep forms, in microseconds, fitted to GB300
// measurements of ILU(0)/IC(0)/SOR sweeps on 2-D and 3-D grids (128^3,
// 96^3, 256^2; within ~12%): one level of a chunk on the compute warp (its
// FP64 chain is ~64 cycles an operation), the hand-off of a value between
// CTAs through L2, the staging of a chunk, and one dependency level of the
// level-ordered ELL form.  Tiles are used when the simulated schedule is
// below 0.8 of the level-ordered estimate.
struct TileModel {
  double level = 0.4, handoff = 0.8, stage = 20.0, ell_level = 1.25;
};

// Simulated duration of a tiled sweep: chunks are taken in order by the
// first of `resident` CTAs to become free; a level of a chunk ends one level
// time after the later of the previous level and the arrival of its rows'
// values from earlier chunks.
// The simulation stops as soon as the schedule passes `limit` (the caller
// only needs to know that this chunk size loses) and returns the time so far.
static double tile_estimate(int n, const std::vector<int>& dptr, const std::vector<int>& dcol,
                            bool forward, const TilePlan& tp, int resident,
                            std::vector<double>& trow, double limit) {
  const TileModel m;
  const int nch = (int)tp.cstart.size() - 1;
  trow.assign(n, 0.0);
  std::priority_queue<double, std::vector<double>, std::greater<double>> freeq;
  for (int r = 0; r < std::max(1, std::min(resident, nch)); r++) freeq.push(0.0);
  double end = 0.0;
  for (int c = 0; c < nch; c++) {
    double t = freeq.top() + m.stage;
    freeq.pop();
    const int p0 = tp.cstart[c];
    const int* lo = tp.lvl_off.data() + tp.lvl_ptr[c];
    const int nl = tp.lvl_ptr[c + 1] - tp.lvl_ptr[c] - 1;
    for (int l = 0; l < nl; l++) {
      double ready = t;
      for (int r = lo[l]; r < lo[l + 1]; r++) {
        const int i = tp.order[p0 + r];
        for (int e = dptr[i]; e < dptr[i + 1]; e++) {
          const int qj = forward ? dcol[e] : n - 1 - dcol[e];
          if (qj < p0) ready = std::max(ready, trow[dcol[e]] + m.handoff);
        }
      }
      t = ready + m.level * ((lo[l + 1] - lo[l] + 31) / 32);
      for (int r = lo[l]; r < lo[l + 1]; r++) trow[tp.order[p0 + r]] = t;
    }
    freeq.push(t);
    end = std::max(end, t);
    if (end > limit) break;
  }
  return end;
}

static int tile_blocks_per_sm(size_t smem) {
  const size_t per_sm = 228 * 1024;  // shared memory of one SM, 1 KB reserved per CTA
  return (int)std::min<size_t>(2048 / kTileThreads, per_sm / (smem + 1024));
}

// Pick the chunk size whose simulated schedule is shortest, or none when the
// level-ordered form is expected to be faster.  Candidates: powers of two and
// multiples of the most frequent dependency distances (a grid's line and
// plane lengths), within the shared-memory budget.
static bool tile_choose(int mode, int n, int W, const std::vector<int>& dptr,
                        const std::vector<int>& dcol, bool forward, int nlevels,
                        const SweepTuning& tu, TilePlan& best, int* considered) {
  std::vector<int> cands;
  if (tu.tile_rows) {
    cands.push_back(tu.tile_rows);
  } else {
    for (int c = 64; c <= 8192; c *= 2) cands.push_back(c);
    std::map<int, long long> hist;
    const int scan = std::min(n, 1 << 18);
    for (int i = 0; i < scan; i++)
      for (int e = dptr[i]; e < dptr[i + 1]; e++) {
        const int d = std::abs(i - dcol[e]);
        if (d >= 8) hist[d]++;
      }
    std::vector<std::pair<long long, int>> top;
    for (auto& kv : hist) top.push_back({kv.second, kv.first});
    std::sort(top.rbegin(), top.rend());
    for (size_t k = 0; k < top.size() && k < 2; k++)
      for (int mlt : {1, 2, 3, 4, 6, 8, 12, 16})
        if ((long long)top[k].second * mlt <= 8192) cands.push_back(top[k].second * mlt);
    std::sort(cands.begin(), cands.end());
    cands.erase(std::unique(cands.begin(), cands.end()), cands.end());
  }
  const TileModel m;
  const double ell_us = m.ell_level * std::max(nlevels, 1);
  // a chunk size is only taken below 0.8 of the level-ordered estimate, so a
  // simulation past that bound can stop (a forced size is simulated in full)
  const double limit = tu.tile_rows ? std::numeric_limits<double>::infinity() : 0.8 * ell_us;
  const int sms = num_sms();
  cands.erase(std::remove_if(cands.begin(), cands.end(), [&](int C) { return C < 8 || C > n * 2; }),
              cands.end());
  // candidates are independent: simulate them on host threads, then pick the
  // shortest in candidate order (the same choice as one after another)
  const int nc = (int)cands.size();
  std::vector<TilePlan> plans(nc);
  std::vector<char> ok(nc, 0);
  auto eval = [&](int c) {
    TilePlan& tp = plans[c];
    tile_order(n, dptr, dcol, forward, std::min(cands[c], n), tp);
    tp.smem = tile_smem_bytes(mode, tp.C, tp.max_levels, tp.max_ext, W);
    if (tp.smem > (size_t)tu.tile_smem) return;
    const int bps = tile_blocks_per_sm(tp.smem);
    if (bps < 1) return;
    std::vector<double> trow;
    tp.est_us = tile_estimate(n, dptr, dcol, forward, tp, bps * sms, trow, limit);
    ok[c] = 1;
  };
  const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
  const int nthreads = std::min({nc, hw, 16, n >= (1 << 16) ? nc : 1});
  if (nthreads <= 1) {
    for (int c = 0; c < nc; c++) eval(c);
  } else {
    // an exception (bad_alloc) inside a worker would end the process; it is
    // caught there and rethrown on this thread, where the C ABI's guard turns
    // it into an error status
    std::atomic<int> next{0};
    std::exception_ptr failure;
    std::mutex failure_mu;
    std::vector<std::thread> pool;
    for (int t = 0; t < nthreads; t++)
      pool.emplace_back([&]() {
        try {
          for (int c; (c = next.fetch_add(1)) < nc;) eval(c);
        } catch (...) {
          std::lock_guard<std::mutex> lock(failure_mu);
          if (!failure) failure = std::current_exception();
          next.store(nc);
        }
      });
    for (auto& th : pool) th.join();
    if (failure) std::rethrow_exception(failure);
  }
  bool found = false;
  *considered = 0;
  for (int c = 0; c < nc; c++) {
    if (!ok[c]) continue;
    (*considered)++;
    if (!found || plans[c].est_us < best.est_us) {
      best = std::move(plans[c]);
      found = true;
    }
  }
  return found && (tu.tile_rows || best.est_us < limit);
}

// The per-chunk blobs of a tiled sweep (layout read by k_tile_sweep).
// Dependencies inside the chunk are encoded as the local index of the row,
// those in earlier chunks as -(k + 1), k the slot of the chunk's external list.
static int tile_upload(EllSweep& e, int mode, const TilePlan& tp, int W,
                       const std::vector<int>& cnt, const std::vector<int>& dep,
                       const std::vector<int>& cs, const std::vector<int>& in,
                       const std::vector<int>& out, const std::vector<int>& ds,
                       bool has_ds, const std::vector<int>& rowof) {
  const int n = e.n;
  const int nch = (int)tp.cstart.size() - 1;
  std::vector<long long> off(nch + 1, 0);
  std::vector<int> next(nch, 0);
  int maxC = 0, max_blob = 0, max_ext = 0;
  for (int c = 0; c < nch; c++) {
    const int p0 = tp.cstart[c], Cc = tp.cstart[c + 1] - p0;
    const int nl = tp.lvl_ptr[c + 1] - tp.lvl_ptr[c] - 1;
    for (int r = 0; r < Cc; r++)
      for (int q = 0; q < cnt[p0 + r]; q++) next[c] += dep[(size_t)q * n + p0 + r] < p0;
    const int bytes = tile_blob_bytes(nl, Cc, next[c], W);
    off[c + 1] = off[c] + bytes;
    maxC = std::max(maxC, Cc);
    max_blob = std::max(max_blob, bytes);
    max_ext = std::max(max_ext, next[c]);
  }
  std::vector<int> blob((size_t)(off[nch] / 4), 0);
  for (int c = 0; c < nch; c++) {
    int* b = blob.data() + off[c] / 4;
    const int p0 = tp.cstart[c], Cc = tp.cstart[c + 1] - p0;
    const int nl = tp.lvl_ptr[c + 1] - tp.lvl_ptr[c] - 1;
    const int Lp = round4(nl + 1), Cp = round4(Cc), Ne = next[c], Ep = round4(Ne);
    const int Cp8 = round8(Cc);
    b[0] = nl;
    b[1] = Cc;
    b[2] = Lp;
    b[3] = Cp;
    b[4] = Ne;
    b[5] = Ep;
    b[6] = Cp8;
    int* lo = b + kTileHeader;
    for (int l = 0; l <= nl; l++) lo[l] = tp.lvl_off[tp.lvl_ptr[c] + l];
    int* oidx = lo + Lp;
    int* iidx = oidx + Cp;
    int* gidx = iidx + Cp;
    int* csl = gidx + Cp;
    int* epos = csl + (size_t)W * Cp;
    int16_t* depc = reinterpret_cast<int16_t*>(epos + Ep);
    for (size_t q = 0; q < (size_t)W * Cp8; q++) depc[q] = (int16_t)kTileNoDep;
    for (size_t q = 0; q < (size_t)W * Cp; q++) csl[q] = -1;
    int k = 0;
    for (int r = 0; r < Cc; r++) {
      const int p = p0 + r;
      iidx[r] = in[p];
      gidx[r] = has_ds ? ds[p] : rowof[p];
      for (int q = 0; q < cnt[p]; q++) {
        csl[(size_t)q * Cp + r] = cs[(size_t)q * n + p];
        const int dp = dep[(size_t)q * n + p];
        if (dp >= p0) {
          depc[(size_t)q * Cp8 + r] = (int16_t)(dp - p0);
        } else {
          epos[k] = dp;
          depc[(size_t)q * Cp8 + r] = (int16_t)(-(k + 1));
          k++;
        }
      }
      oidx[r] = out[p] >= 0 ? out[p] : rowof[p];
    }
  }
  e.nchunks = nch;
  e.C = round4(maxC);
  e.max_blob = max_blob;
  e.smem = 16 + (size_t)max_blob +
           8 * ((size_t)(std::max(W, 1) + 2 + tile_extra_cols(mode)) * e.C + (size_t)max_ext);
  if (e.smem > (size_t)kTileSmemMax || maxC > 32767 || max_ext > 32767) return GP_ERR_UNSUPPORTED;
  GP_TRY(up(&e.blob, std::vector<unsigned char>((unsigned char*)blob.data(),
                                                (unsigned char*)(blob.data() + blob.size()))));
  GP_TRY(up(&e.blob_off, off));
  GP_TRY(up(&e.cstart, tp.cstart));
  return GP_OK;
}

static void tile_kernel_attrs(int W, const EllSweep& e, int* blocks_per_sm);

// Number of dependency levels of a sweep (the level-ordered form's depth).
static int sweep_levels(int n, const std::vector<int>& dptr, const std::vector<int>& dcol,
                        bool forward) {
  std::vector<int> lev(n, 0);
  int maxl = 0;
  for (int s = 0; s < n; s++) {
    const int i = forward ? s : n - 1 - s;
    int l = 0;
    for (int e = dptr[i]; e < dptr[i + 1]; e++) l = std::max(l, lev[dcol[e]] + 1);
    lev[i] = l;
    maxl = std::max(maxl, l);
  }
  return n ? maxl + 1 : 0;
}

// Lay out one sweep.  dptr/dcol/dsl: each row's dependencies (rows) and their
// coefficient slots, in the reference's order.  The positions follow the
// chunked order of the tiled form when its simulated schedule beats the
// level-ordered form, else `order` (dependency levels).
static int ell_build_impl(EllSweep& e, int mode, int n, bool forward,
                          const std::vector<int>& order_in,
                          const std::vector<int>& dptr, const std::vector<int>& dcol,
                          const std::vector<int>& dsl, const std::vector<int>& in_row,
                          const std::vector<int>& out_row, const std::vector<int>& dslot_row,
                          std::vector<int>* pos_of_row, bool allow_tiles,
                          bool allow_bricks = true, int nlevels = 0) {
  ell_free(e);
  int W = 0;
  for (int i = 0; i < n; i++) W = std::max(W, dptr[i + 1] - dptr[i]);
  e.n = n;
  e.W = W;
  if (W > kEllMaxW) return GP_OK;  // the CSR sweep kernels handle wide rows
  const SweepTuning& tu = sweep_tuning();
  TilePlan tp;
  bool tiled = false;
  int considered = 0, nlev = nlevels;  // the caller's level count, when it has one
  if (tu.tiles && allow_tiles && n > 0) {
    if (!nlev) nlev = sweep_levels(n, dptr, dcol, forward);
    tiled = tile_choose(mode, n, W, dptr, dcol, forward, nlev, tu, tp, &considered);
    setup_mark("chunk-model");
  }
  if (allow_tiles && allow_bricks && n > 0) {
    // the brick form, where the sweep is a grid in natural order and the
    // model puts it below the better of the other two forms
    if (!nlev) nlev = sweep_levels(n, dptr, dcol, forward);
    double other = TileModel().ell_level * nlev;
    if (tiled) other = std::min(other, tp.est_us);
    bool built = false;
    GP_TRY(brick_build(e, mode, n, forward, dptr, dcol, dsl, in_row, out_row, dslot_row, other,
                       &built, pos_of_row));
    setup_mark("brick-check");
    if (built) return GP_OK;
  }
  const std::vector<int>& order = tiled ? tp.order : order_in;
  std::vector<int> pos(n);
  for (int p = 0; p < n; p++) pos[order[p]] = p;
  const int Wc = std::max(W, 1);
  std::vector<int> cnt(n), dep((size_t)Wc * n, 0), cs((size_t)Wc * n, 0), rowof(n);
  std::vector<int> in(n, 0), out(n, -1), ds(n, 0);
  // positions are independent: host threads fill ranges of them
  host_parallel_for(n, [&](int64_t p0, int64_t p1) {
    for (int p = (int)p0; p < (int)p1; p++) {
      const int i = order[p];
      rowof[p] = i;
      cnt[p] = dptr[i + 1] - dptr[i];
      for (int q = 0; q < cnt[p]; q++) {
        dep[(size_t)q * n + p] = pos[dcol[dptr[i] + q]];
        cs[(size_t)q * n + p] = dsl[dptr[i] + q];
      }
      if (!in_row.empty()) in[p] = in_row[i];
      if (!out_row.empty()) out[p] = out_row[i];
      if (!dslot_row.empty()) ds[p] = dslot_row[i];
    }
  });
  setup_mark("layout");
  if (tiled) {
    int st = tile_upload(e, mode, tp, W, cnt, dep, cs, in, out, ds, !dslot_row.empty(), rowof);
    int bps = 0;
    if (st == GP_OK) tile_kernel_attrs(W, e, &bps);
    if (st == GP_OK && bps > 0) {
      e.grid = std::min(e.nchunks, bps * num_sms());
      e.tiled = true;
      e.est_us = tp.est_us;
      e.rows_per_chunk = tp.C;
      if (std::getenv("GPETSC_SWEEP_VERBOSE"))
        std::fprintf(stderr,
                     "gpetsc sweep: n=%d W=%d levels=%d tiled rows/chunk=%d chunks=%d "
                     "smem=%zu ctas/sm=%d grid=%d est=%.0fus (level order %.0fus, %d sizes)\n",
                     n, W, nlev, tp.C, e.nchunks, e.smem, bps, e.grid, tp.est_us,
                     TileModel().ell_level * nlev, considered);
      if (pos_of_row) *pos_of_row = pos;
      e.ok = true;
      return GP_OK;
    }
    if (st != GP_OK && st != GP_ERR_UNSUPPORTED) return st;
    // the tiled form does not fit: fall back to the level order
    ell_free(e);
    return ell_build_impl(e, mode, n, forward, order_in, dptr, dcol, dsl, in_row, out_row,
                          dslot_row, pos_of_row, false);
  }
  if (std::getenv("GPETSC_SWEEP_VERBOSE") && tu.tiles && allow_tiles && n > 0)
    std::fprintf(stderr, "gpetsc sweep: n=%d W=%d levels=%d level order (%d chunk sizes tried)\n",
                 n, W, nlev, considered);
  GP_TRY(up(&e.cnt, cnt));
  GP_TRY(up(&e.dep, dep));
  GP_TRY(up(&e.cslot, cs));
  GP_TRY(up(&e.rowof, rowof));
  GP_TRY(up(&e.in_idx, in));
  GP_TRY(up(&e.out_idx, out));
  if (!dslot_row.empty()) GP_TRY(up(&e.dslot, ds));
  GP_CUDA(cudaMalloc(&e.coef, (size_t)Wc * n * sizeof(double)));
  GP_CUDA(cudaMalloc(&e.dval, std::max(n, 1) * sizeof(double)));
  if (pos_of_row) *pos_of_row = pos;
  e.ok = true;
  return GP_OK;
}

int ell_build(EllSweep& e, int mode, int n, bool forward, const std::vector<int>& order,
              const std::vector<int>& dptr, const std::vector<int>& dcol,
              const std::vector<int>& dsl, const std::vector<int>& in_row,
              const std::vector<int>& out_row, const std::vector<int>& dslot_row,
              std::vector<int>* pos_of_row, int nlevels) {
  return ell_build_impl(e, mode, n, forward, order, dptr, dcol, dsl, in_row, out_row,
                        dslot_row, pos_of_row, true, true, nlevels);
}

int ell_build_chunked(EllSweep& e, int mode, int n, bool forward, const std::vector<int>& order,
                      const std::vector<int>& dptr, const std::vector<int>& dcol,
                      const std::vector<int>& dsl, const std::vector<int>& in_row,
                      const std::vector<int>& out_row, const std::vector<int>& dslot_row,
                      std::vector<int>* pos_of_row) {
  return ell_build_impl(e, mode, n, forward, order, dptr, dcol, dsl, in_row, out_row,
                        dslot_row, pos_of_row, true, false);
}

int ell_build_levels(EllSweep& e, int mode, int n, bool forward, const std::vector<int>& order,
                     const std::vector<int>& dptr, const std::vector<int>& dcol,
                     const std::vector<int>& dsl, const std::vector<int>& in_row,
                     const std::vector<int>& out_row, const std::vector<int>& dslot_row,
                     std::vector<int>* pos_of_row) {
  return ell_build_impl(e, mode, n, forward, order, dptr, dcol, dsl, in_row, out_row,
                        dslot_row, pos_of_row, false);
}

// Run the wait once on a pending flag (set = 0) or a ready one (set = 1) and
// report the status the host reads after a sweep.
int sweep_wait_probe(int budget, int set, cudaStream_t s) {
  double* buf = nullptr;
  DevErr* err = nullptr;
  GP_CUDA(cudaMalloc(&buf, 2 * sizeof(double)));
  cudaError_t e = cudaMalloc(&err, sizeof(DevErr));
  if (e != cudaSuccess) {
    cudaFree(buf);
    return GP_ERR_CUDA;
  }
  const unsigned long long pending = kPending;
  const double ready = 1.5;
  int st = GP_OK;
  if (cudaMemcpyAsync(buf, set ? (const void*)&ready : (const void*)&pending, sizeof(double),
                      cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemsetAsync(err, 0, sizeof(DevErr), s) != cudaSuccess) {
    st = GP_ERR_CUDA;
  } else {
    k_wait_probe<<<1, 1, 0, s>>>(buf, budget, err, buf + 1);
    DevErr h{};
    double got = 0.0;
    if (cudaMemcpyAsync(&h, err, sizeof(DevErr), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(&got, buf + 1, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
      st = GP_ERR_CUDA;
    } else if (h.code) {
      set_error("device wait ran out of its budget (site " + std::to_string(h.where) + ")");
      st = h.code;
    } else if (got != ready) {
      set_error("device wait returned a wrong value");
      st = GP_ERR_INTERNAL;
    }
  }
  cudaFree(buf);
  cudaFree(err);
  return st;
}

int ell_refresh(EllSweep& e, const double* src, cudaStream_t s) {
  if (!e.ok || e.tiled || e.n == 0) return GP_OK;  // the tiled form gathers at each sweep
  k_ell_refresh<<<std::max(1, std::min((e.n + 255) / 256, num_sms() * 8)), 256, 0, s>>>(
      e.n, e.W, e.cnt, e.cslot, src, e.coef, e.dslot, e.dval);
  GP_CHECK_LAUNCH();
  return GP_OK;
}

template <int WMAX, bool FMA>
static void tile_set_attrs() {
  auto set = [](const void* f) {
    cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, kTileSmemMax);
  };
  set((const void*)k_tile_sweep<ELL_ILU_F, WMAX, FMA>);
  set((const void*)k_tile_sweep<ELL_ILU_B, WMAX, FMA>);
  set((const void*)k_tile_sweep<ELL_ICC_F, WMAX, FMA>);
  set((const void*)k_tile_sweep<ELL_ICC_B, WMAX, FMA>);
  set((const void*)k_tile_sweep<ELL_SOR_F, WMAX, FMA>);
  set((const void*)k_tile_sweep<ELL_SOR_B, WMAX, FMA>);
}

template <int WMAX>
static void tile_attrs_w(const EllSweep& e, int* bps) {
  static unsigned long long done = 0;  // one bit per device
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 64 && !(done >> dev & 1ull)) {
    tile_set_attrs<WMAX, false>();
    tile_set_attrs<WMAX, true>();
    done |= 1ull << dev;
  }
  *bps = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, k_tile_sweep<ELL_SOR_B, WMAX, false>,
                                                    kTileThreads, e.smem) != cudaSuccess)
    *bps = 0;
  cudaGetLastError();
}

static void tile_kernel_attrs(int W, const EllSweep& e, int* bps) {
  if (W <= 4)
    tile_attrs_w<4>(e, bps);
  else if (W <= 8)
    tile_attrs_w<8>(e, bps);
  else
    tile_attrs_w<kEllMaxW>(e, bps);
}

template <int MODE, bool FMA>
static void launch_tile_a(const EllSweep& e, const int* gate, int want, EllArgs a, TileArgs t,
                          DRef in, DRef out, cudaStream_t s) {
  const int g = std::max(1, e.grid);
  if (e.W <= 4)
    k_tile_sweep<MODE, 4, FMA><<<g, kTileThreads, e.smem, s>>>(gate, want, a, t, in, out);
  else if (e.W <= 8)
    k_tile_sweep<MODE, 8, FMA><<<g, kTileThreads, e.smem, s>>>(gate, want, a, t, in, out);
  else
    k_tile_sweep<MODE, kEllMaxW, FMA><<<g, kTileThreads, e.smem, s>>>(gate, want, a, t, in, out);
}

template <int MODE>
static void launch_tile(const EllSweep& e, const int* gate, int want, EllArgs a, TileArgs t,
                        DRef in, DRef out, cudaStream_t s) {
  if (arith_mode() == kFma)
    launch_tile_a<MODE, true>(e, gate, want, a, t, in, out, s);
  else
    launch_tile_a<MODE, false>(e, gate, want, a, t, in, out, s);
}

template <int MODE, bool FMA>
static void launch_mode_a(const EllSweep& e, const int* gate, int want, EllArgs a, DRef in,
                          DRef out, cudaStream_t s) {
  const int g = num_sms() * sweep_tuning().ctas_per_sm;
  const int b = sweep_tuning().block;
  if (e.W <= 4)
    k_ell_sweep<MODE, 4, FMA><<<g, b, 0, s>>>(gate, want, a, in, out);
  else if (e.W <= 8)
    k_ell_sweep<MODE, 8, FMA><<<g, b, 0, s>>>(gate, want, a, in, out);
  else
    k_ell_sweep<MODE, kEllMaxW, FMA><<<g, b, 0, s>>>(gate, want, a, in, out);
}

template <int MODE>
static void launch_mode(const EllSweep& e, const int* gate, int want, EllArgs a, DRef in,
                        DRef out, cudaStream_t s) {
  if (arith_mode() == kFma)
    launch_mode_a<MODE, true>(e, gate, want, a, in, out, s);
  else
    launch_mode_a<MODE, false>(e, gate, want, a, in, out, s);
}

int ell_sweep(int mode, const EllSweep& e, const int* gate, int want, DRef in, DRef out,
              double* val, const double* fval, double* aux, const double* auxin,
              const double* idiag, double omega, int use_t, int write_out, unsigned* tickets,
              DevErr* err, const double* coefsrc, cudaStream_t s) {
  if (e.n == 0) return GP_OK;
  if (e.brick)
    return brick_sweep(mode, e, gate, want, in, out, val, fval, aux, auxin, idiag, omega, use_t,
                       write_out, tickets, err, s);
  EllArgs a;
  a.n = e.n;
  a.cnt = e.cnt;
  a.dep = e.dep;
  a.coef = e.coef;
  a.in_idx = e.in_idx;
  a.out_idx = write_out ? e.out_idx : nullptr;
  a.dval = e.dval;
  a.rowof = e.rowof;
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
  a.sleep_after = sweep_tuning().sleep_after;
  a.sleep_ns = sweep_tuning().sleep_ns;
  if (e.tiled) {
    TileArgs t;
    t.nchunks = e.nchunks;
    t.W = e.W;
    t.C = e.C;
    t.max_blob = e.max_blob;
    t.blob = e.blob;
    t.blob_off = e.blob_off;
    t.cstart = e.cstart;
    t.coefsrc = coefsrc;
    switch (mode) {
      case ELL_ILU_F: launch_tile<ELL_ILU_F>(e, gate, want, a, t, in, out, s); break;
      case ELL_ILU_B: launch_tile<ELL_ILU_B>(e, gate, want, a, t, in, out, s); break;
      case ELL_ICC_F: launch_tile<ELL_ICC_F>(e, gate, want, a, t, in, out, s); break;
      case ELL_ICC_B: launch_tile<ELL_ICC_B>(e, gate, want, a, t, in, out, s); break;
      case ELL_SOR_F: launch_tile<ELL_SOR_F>(e, gate, want, a, t, in, out, s); break;
      case ELL_SOR_B: launch_tile<ELL_SOR_B>(e, gate, want, a, t, in, out, s); break;
    }
    GP_CHECK_LAUNCH();
    return GP_OK;
  }
  switch (mode) {
    case ELL_ILU_F: launch_mode<ELL_ILU_F>(e, gate, want, a, in, out, s); break;
    case ELL_ILU_B: launch_mode<ELL_ILU_B>(e, gate, want, a, in, out, s); break;
    case ELL_ICC_F: launch_mode<ELL_ICC_F>(e, gate, want, a, in, out, s); break;
    case ELL_ICC_B: launch_mode<ELL_ICC_B>(e, gate, want, a, in, out, s); break;
    case ELL_SOR_F: launch_mode<ELL_SOR_F>(e, gate, want, a, in, out, s); break;
    case ELL_SOR_B: launch_mode<ELL_SOR_B>(e, gate, want, a, in, out, s); break;
  }
  GP_CHECK_LAUNCH();
  return GP_OK;
}

}  // namespace gp
