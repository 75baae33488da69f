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
#include <cstdlib>
#include <string>
#include <vector>

#include "gp_pc.h"

namespace gp {

constexpr int kEllBlock = 256;
constexpr int kEllSpin = 1 << 22;
constexpr int kTileSmemMax = 227 * 1024;  // dynamic shared memory limit of one CTA
constexpr int kTileBulkPiece = 16384;     // bytes per bulk copy instruction
constexpr int kTileHeader = 4;            // ints: levels, rows, padded levels+1, padded rows

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
  int ctas_per_sm = 2, sleep_after = 8, sleep_ns = 20;  // best of a scan on ICC(0), 128^3
  int tiles = 0;                // GPETSC_SWEEP_TILES=1: chunked form where it applies
  int tile_smem = 110 * 1024;   // GPETSC_TILE_SMEM: shared memory budget of one chunk
  int tile_rows = 0;            // GPETSC_TILE_ROWS: rows per chunk (0: from the budget)
};
static const SweepTuning& sweep_tuning() {
  static SweepTuning t = [] {
    SweepTuning v;
    auto env = [](const char* k, int d) {
      const char* e = std::getenv(k);
      return e ? std::atoi(e) : d;
    };
    v.ctas_per_sm = std::max(1, std::min(8, env("GPETSC_SWEEP_CTAS_PER_SM", v.ctas_per_sm)));
    v.sleep_after = std::max(0, env("GPETSC_SWEEP_SLEEP_AFTER", v.sleep_after));
    v.sleep_ns = std::max(0, std::min(1000, env("GPETSC_SWEEP_SLEEP_NS", v.sleep_ns)));
    v.tiles = env("GPETSC_SWEEP_TILES", v.tiles) != 0;
    v.tile_smem = std::max(16 * 1024, std::min(kTileSmemMax, env("GPETSC_TILE_SMEM", v.tile_smem)));
    v.tile_rows = std::max(0, std::min(8192, env("GPETSC_TILE_ROWS", v.tile_rows)));
    return v;
  }();
  return t;
}

template <int MODE, int WMAX>
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
    if (p < n) {
      // ---- everything that does not wait
      const int c = a.cnt[p];
      int dp[WMAX];
      double cf[WMAX];
#pragma unroll
      for (int e = 0; e < WMAX; e++) {
        if (e < c) {
          dp[e] = a.dep[(size_t)e * n + p];
          cf[e] = a.coef[(size_t)e * n + p];
        }
      }
      double sum;
      double dv = 0.0, yf = 0.0;
      if constexpr (MODE == ELL_ILU_F || MODE == ELL_ICC_F) {
        sum = in[a.in_idx[p]];
        if (MODE == ELL_ICC_F) dv = a.dval[p];
      } else if constexpr (MODE == ELL_ILU_B) {
        sum = a.fval[a.in_idx[p]];
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
      // ---- the dependency chain, in the reference's slot order.  Every
      // dependency is loaded once up front (independent loads, one L2 round
      // trip for all of them); only those still pending are polled.
      unsigned long long bits[WMAX];
#pragma unroll
      for (int e = 0; e < WMAX; e++)
        if (e < c) bits[e] = ld_relaxed_bits(&a.val[dp[e]]);
#pragma unroll
      for (int e = 0; e < WMAX; e++) {
        if (e < c) {
          const double v =
              bits[e] != kPending
                  ? __longlong_as_double((long long)bits[e])
                  : ell_wait(&a.val[dp[e]], a.err, 20 + MODE, kEllSpin, a.sleep_after,
                             a.sleep_ns);
          if constexpr (MODE == ELL_ICC_F || MODE == ELL_ICC_B)
            sum = add(sum, mul(cf[e], v));
          else
            sum = sub(sum, mul(cf[e], v));
        }
      }
      // ---- results
      if constexpr (MODE == ELL_ILU_F) {
        st_relaxed(&a.val[p], sum);
      } else if constexpr (MODE == ELL_ILU_B) {
        const double y = mul(sum, dv);
        out[a.out_idx[p]] = y;
        st_relaxed(&a.val[p], y);
      } else if constexpr (MODE == ELL_ICC_F) {
        a.aux[p] = mul(sum, dv);
        st_relaxed(&a.val[p], sum);
      } else if constexpr (MODE == ELL_ICC_B) {
        out[a.out_idx[p]] = sum;
        st_relaxed(&a.val[p], sum);
      } else if constexpr (MODE == ELL_SOR_F) {
        a.aux[p] = sum;
        const double y = mul(sum, dv);
        if (a.out_idx) out[a.rowof[p]] = y;
        st_relaxed(&a.val[p], y);
      } else {
        const double y = a.use_t ? add(mul(a.om1, yf), mul(sum, dv)) : mul(sum, dv);
        out[a.rowof[p]] = y;
        st_relaxed(&a.val[p], y);
      }
    }
    __syncwarp();
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
// sorted by their dependency level counted over the chunk's own rows, so one
// warp can walk the chunk level by level: dependencies inside the chunk are
// read from shared memory (one __syncwarp between levels), dependencies in
// earlier chunks are polled in the global value-as-flag array.  On a grid
// numbered in natural order most dependencies are neighbours inside the same
// chunk, so the global round trip is paid once per chunk boundary instead of
// once per level.  Each chunk's metadata (level offsets, dependency counts,
// positions, coefficient slots, input/output indices) is one contiguous blob
// staged with cp.async.bulk on an mbarrier; coefficients, diagonals and
// right-hand sides are then gathered by the warp.  Chunks are handed out by a
// ticket in order, and a chunk waits only on earlier chunks, which running
// CTAs already hold, so the sweep cannot deadlock on CTAs that are not yet
// resident.  Per row the arithmetic and the dependency order are those of
// k_ell_sweep, so the results are bit-identical.

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

template <int MODE, int WMAX>
__global__ void __launch_bounds__(32) k_tile_sweep(const int* gate, int want, EllArgs a,
                                                   TileArgs t, DRef inr, DRef outr) {
  if (gated_off(gate, want)) return;
  extern __shared__ __align__(16) unsigned char sm[];
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(sm);
  int* blob = reinterpret_cast<int*>(sm + 16);
  const int W = t.W, C = t.C;
  double* s_cf = reinterpret_cast<double*>(sm + 16 + t.max_blob);  // [W][C]
  double* s_val = s_cf + (size_t)(W > 0 ? W : 1) * C;
  double* s_sum = s_val + C;
  double* s_dv = s_sum + C;
  double* s_yf = s_dv + C;
  const double* __restrict__ in = inr.get();
  double* __restrict__ out = outr.get();
  const int lane = threadIdx.x;
  if (lane == 0) mbar_init(bar, 1);
  __syncwarp();
  unsigned parity = 0;
  for (;;) {
    unsigned c = 0;
    if (lane == 0) c = atomicAdd(&a.tickets[0], 1u);
    c = __shfl_sync(0xffffffffu, c, 0);
    if (c >= (unsigned)t.nchunks) break;
    const int cs = t.cstart[c];
    // ---- stage the chunk's blob (one elected lane issues the bulk copies)
    if (lane == 0) {
      const long long b0 = t.blob_off[c];
      const unsigned bytes = (unsigned)(t.blob_off[c + 1] - b0);
      // earlier generic reads of the blob area come before the async writes
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_expect_tx(bar, bytes);
      for (unsigned off = 0; off < bytes; off += kTileBulkPiece)
        bulk_g2s(sm + 16 + off, t.blob + b0 + off, min((unsigned)kTileBulkPiece, bytes - off),
                 bar);
    }
    if (!mbar_wait(bar, parity, kEllSpin)) {
      if (lane == 0 && atomicCAS(&a.err->code, 0, GP_ERR_TIMEOUT) == 0) a.err->where = 30 + MODE;
      // let the copies in flight land before the CTA leaves
      mbar_wait(bar, parity, kEllSpin);
      break;
    }
    parity ^= 1u;
    const int nl = blob[0], Cc = blob[1], Lp = blob[2], Cp = blob[3];
    const int* lo = blob + kTileHeader;
    const int* cnt = lo + Lp;
    const int* dep = cnt + Cp;
    const int* csl = dep + (size_t)W * Cp;
    const int* iidx = csl + (size_t)W * Cp;
    const int* oidx = iidx + Cp;
    const int* rowof = oidx + Cp;
    const int* dsl = rowof + Cp;
    // ---- gathers that do not wait: coefficients, initial sums, diagonals
#pragma unroll 4
    for (int r = lane; r < Cc; r += 32) {
      const int cn = cnt[r];
#pragma unroll
      for (int e = 0; e < WMAX; e++)
        if (e < cn) s_cf[(size_t)e * C + r] = t.coefsrc[csl[(size_t)e * Cp + r]];
      if constexpr (MODE == ELL_ILU_F) {
        s_sum[r] = in[iidx[r]];
      } else if constexpr (MODE == ELL_ICC_F) {
        s_sum[r] = in[iidx[r]];
        s_dv[r] = t.coefsrc[dsl[r]];
      } else if constexpr (MODE == ELL_ILU_B) {
        s_sum[r] = a.fval[iidx[r]];
        s_dv[r] = t.coefsrc[dsl[r]];
      } else if constexpr (MODE == ELL_ICC_B) {
        s_sum[r] = a.auxin[iidx[r]];
      } else if constexpr (MODE == ELL_SOR_F) {
        s_sum[r] = in[rowof[r]];
        s_dv[r] = a.idiag[rowof[r]];
      } else {  // ELL_SOR_B
        const int fp = iidx[r];
        s_sum[r] = a.use_t ? a.auxin[fp] : in[rowof[r]];
        s_yf[r] = a.use_t ? a.fval[fp] : 0.0;
        s_dv[r] = a.idiag[rowof[r]];
      }
    }
    __syncwarp();
    // ---- the chunk's levels
    for (int l = 0; l < nl; l++) {
      const int r1 = lo[l + 1];
      for (int r = lo[l] + lane; r < r1; r += 32) {
        const int p = cs + r;
        const int cn = cnt[r];
        int dp[WMAX];
        unsigned long long bits[WMAX];
#pragma unroll
        for (int e = 0; e < WMAX; e++) {
          if (e < cn) {
            dp[e] = dep[(size_t)e * Cp + r];
            bits[e] = dp[e] < cs ? ld_relaxed_bits(&a.val[dp[e]]) : 0ull;
          }
        }
        double sum = s_sum[r];
#pragma unroll
        for (int e = 0; e < WMAX; e++) {
          if (e < cn) {
            double v;
            if (dp[e] >= cs)
              v = s_val[dp[e] - cs];
            else if (bits[e] != kPending)
              v = __longlong_as_double((long long)bits[e]);
            else
              v = ell_wait(&a.val[dp[e]], a.err, 30 + MODE, kEllSpin, a.sleep_after, a.sleep_ns);
            if constexpr (MODE == ELL_ICC_F || MODE == ELL_ICC_B)
              sum = add(sum, mul(s_cf[(size_t)e * C + r], v));
            else
              sum = sub(sum, mul(s_cf[(size_t)e * C + r], v));
          }
        }
        double res;
        if constexpr (MODE == ELL_ILU_F) {
          res = sum;
        } else if constexpr (MODE == ELL_ILU_B) {
          res = mul(sum, s_dv[r]);
          out[oidx[r]] = res;
        } else if constexpr (MODE == ELL_ICC_F) {
          a.aux[p] = mul(sum, s_dv[r]);
          res = sum;
        } else if constexpr (MODE == ELL_ICC_B) {
          res = sum;
          out[oidx[r]] = res;
        } else if constexpr (MODE == ELL_SOR_F) {
          a.aux[p] = sum;
          res = mul(sum, s_dv[r]);
          if (a.write_out) out[rowof[r]] = res;
        } else {
          res = a.use_t ? add(mul(a.om1, s_yf[r]), mul(sum, s_dv[r])) : mul(sum, s_dv[r]);
          out[rowof[r]] = res;
        }
        s_val[r] = res;
        st_relaxed(&a.val[p], res);
      }
      __syncwarp();
    }
  }
  if (lane == 0) {
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
    for (int e = 0; e < c; e++) coef[(size_t)e * n + p] = src[cslot[(size_t)e * n + p]];
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
  void* ptrs[] = {e.cnt,  e.dep,    e.cslot, e.coef,     e.in_idx, e.out_idx,
                  e.dslot, e.dval,  e.rowof, e.blob,     e.blob_off, e.cstart};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  e = EllSweep();
}

// Chunked processing order of one sweep.  The sweep's natural sequence is
// ascending rows (forward: every dependency precedes its row) or descending
// rows (backward).  Chunk c holds sequence entries [c*C, (c+1)*C); inside it,
// rows are sorted (stably) by their level over dependencies inside the chunk.
struct TilePlan {
  std::vector<int> order;    // position -> row
  std::vector<int> cstart;   // [nchunks + 1]
  std::vector<int> lvl_ptr;  // [nchunks + 1] into lvl_off
  std::vector<int> lvl_off;  // per chunk: level offsets relative to its start (levels + 1)
  long long internal = 0, total = 0;
};

static void tile_order(int n, const std::vector<int>& dptr, const std::vector<int>& dcol,
                       bool forward, int C, TilePlan& tp) {
  const int nch = (n + C - 1) / C;
  tp.order.assign(n, 0);
  tp.cstart.assign(nch + 1, 0);
  tp.lvl_ptr.assign(nch + 1, 0);
  tp.lvl_off.clear();
  tp.internal = tp.total = 0;
  std::vector<int> lev(C), cnt;
  auto row_of = [&](int q) { return forward ? q : n - 1 - q; };
  for (int c = 0; c < nch; c++) {
    const int q0 = c * C, q1 = std::min(n, q0 + C);
    int maxl = 0;
    for (int q = q0; q < q1; q++) {
      const int i = row_of(q);
      int l = 0;
      for (int e = dptr[i]; e < dptr[i + 1]; e++) {
        const int qj = forward ? dcol[e] : n - 1 - dcol[e];
        tp.total++;
        if (qj >= q0) {
          tp.internal++;
          l = std::max(l, lev[qj - q0] + 1);
        }
      }
      lev[q - q0] = l;
      maxl = std::max(maxl, l);
    }
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

static int round4(int v) { return (v + 3) & ~3; }

// The per-chunk blobs of a tiled sweep (layout read by k_tile_sweep):
// header {levels, rows, Lp, Cp}, level offsets [Lp], then [Cp] columns:
// count, dependency positions x W, coefficient slots x W, input index,
// output index, row, diagonal slot.
static int tile_upload(EllSweep& e, const TilePlan& tp, int W, const std::vector<int>& cnt,
                       const std::vector<int>& dep, const std::vector<int>& cs,
                       const std::vector<int>& in, const std::vector<int>& out,
                       const std::vector<int>& ds, const std::vector<int>& rowof) {
  const int n = e.n;
  const int nch = (int)tp.cstart.size() - 1;
  std::vector<long long> off(nch + 1, 0);
  int maxC = 0, max_blob = 0;
  for (int c = 0; c < nch; c++) {
    const int Cc = tp.cstart[c + 1] - tp.cstart[c];
    const int nl = tp.lvl_ptr[c + 1] - tp.lvl_ptr[c] - 1;
    const int ints = kTileHeader + round4(nl + 1) + round4(Cc) * (5 + 2 * W);
    off[c + 1] = off[c] + (long long)ints * 4;
    maxC = std::max(maxC, Cc);
    max_blob = std::max(max_blob, ints * 4);
  }
  std::vector<int> blob((size_t)(off[nch] / 4), 0);
  for (int c = 0; c < nch; c++) {
    int* b = blob.data() + off[c] / 4;
    const int p0 = tp.cstart[c], Cc = tp.cstart[c + 1] - p0;
    const int nl = tp.lvl_ptr[c + 1] - tp.lvl_ptr[c] - 1;
    const int Lp = round4(nl + 1), Cp = round4(Cc);
    b[0] = nl;
    b[1] = Cc;
    b[2] = Lp;
    b[3] = Cp;
    int* lo = b + kTileHeader;
    for (int l = 0; l <= nl; l++) lo[l] = tp.lvl_off[tp.lvl_ptr[c] + l];
    int* col = lo + Lp;
    for (int r = 0; r < Cc; r++) {
      const int p = p0 + r;
      col[r] = cnt[p];
      for (int q = 0; q < cnt[p]; q++) {
        col[(size_t)(1 + q) * Cp + r] = dep[(size_t)q * n + p];
        col[(size_t)(1 + W + q) * Cp + r] = cs[(size_t)q * n + p];
      }
      col[(size_t)(1 + 2 * W) * Cp + r] = in[p];
      col[(size_t)(2 + 2 * W) * Cp + r] = out[p];
      col[(size_t)(3 + 2 * W) * Cp + r] = rowof[p];
      col[(size_t)(4 + 2 * W) * Cp + r] = ds[p];
    }
  }
  e.nchunks = nch;
  e.C = round4(maxC);
  e.max_blob = max_blob;
  e.smem = 16 + (size_t)max_blob + (size_t)(std::max(W, 1) + 4) * e.C * sizeof(double);
  if (e.smem > (size_t)kTileSmemMax) return GP_ERR_UNSUPPORTED;
  GP_TRY(up(&e.blob, std::vector<unsigned char>((unsigned char*)blob.data(),
                                                (unsigned char*)(blob.data() + blob.size()))));
  GP_TRY(up(&e.blob_off, off));
  GP_TRY(up(&e.cstart, tp.cstart));
  return GP_OK;
}

// Shared memory per chunk row of a tiled sweep with W dependencies a row.
static int tile_row_bytes(int W) { return 4 * (5 + 2 * W) + 8 * (std::max(W, 1) + 4) + 4; }

static void tile_kernel_attrs(int W, const EllSweep& e, int* blocks_per_sm);

// Lay out one sweep.  dptr/dcol/dsl: each row's dependencies (rows) and their
// coefficient slots, in the reference's order.  The positions follow the
// chunked order of the tiled form when most dependencies fall inside their
// chunk, else `order` (dependency levels).
static int ell_build_impl(EllSweep& e, int n, bool forward, const std::vector<int>& order_in,
                          const std::vector<int>& dptr, const std::vector<int>& dcol,
                          const std::vector<int>& dsl, const std::vector<int>& in_row,
                          const std::vector<int>& out_row, const std::vector<int>& dslot_row,
                          std::vector<int>* pos_of_row, bool allow_tiles) {
  ell_free(e);
  int W = 0;
  for (int i = 0; i < n; i++) W = std::max(W, dptr[i + 1] - dptr[i]);
  e.n = n;
  e.W = W;
  if (W > kEllMaxW) return GP_OK;  // the CSR sweep kernels handle wide rows
  const SweepTuning& tu = sweep_tuning();
  TilePlan tp;
  bool tiled = false;
  if (tu.tiles && allow_tiles && n > 0) {
    int C = tu.tile_rows ? tu.tile_rows : (tu.tile_smem / tile_row_bytes(W)) / 32 * 32;
    C = std::max(32, std::min(C, 8192));
    tile_order(n, dptr, dcol, forward, C, tp);
    tiled = tp.total == 0 || 2 * tp.internal >= tp.total;
    e.internal_pct = tp.total ? (int)(100 * tp.internal / tp.total) : 100;
  }
  const std::vector<int>& order = tiled ? tp.order : order_in;
  std::vector<int> pos(n);
  for (int p = 0; p < n; p++) pos[order[p]] = p;
  const int Wc = std::max(W, 1);
  std::vector<int> cnt(n), dep((size_t)Wc * n, 0), cs((size_t)Wc * n, 0), rowof(n);
  std::vector<int> in(n, 0), out(n, -1), ds(n, 0);
  for (int p = 0; p < n; p++) {
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
  if (tiled) {
    int st = tile_upload(e, tp, W, cnt, dep, cs, in, out, ds, rowof);
    if (st == GP_OK) {
      int bps = 0;
      tile_kernel_attrs(W, e, &bps);
      if (bps > 0) {
        e.grid = std::min(e.nchunks, bps * num_sms());
        e.tiled = true;
        if (pos_of_row) *pos_of_row = pos;
        e.ok = true;
        return GP_OK;
      }
    } else if (st != GP_ERR_UNSUPPORTED) {
      return st;
    }
    // the tiled form does not fit: fall back to the level order
    for (void* q : {(void*)e.blob, (void*)e.blob_off, (void*)e.cstart})
      if (q) cudaFree(q);
    e.blob = nullptr;
    e.blob_off = nullptr;
    e.cstart = nullptr;
    return ell_build_impl(e, n, forward, order_in, dptr, dcol, dsl, in_row, out_row,
                          dslot_row, pos_of_row, false);
  }
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

int ell_build(EllSweep& e, int n, bool forward, const std::vector<int>& order,
              const std::vector<int>& dptr, const std::vector<int>& dcol,
              const std::vector<int>& dsl, const std::vector<int>& in_row,
              const std::vector<int>& out_row, const std::vector<int>& dslot_row,
              std::vector<int>* pos_of_row) {
  return ell_build_impl(e, n, forward, order, dptr, dcol, dsl, in_row, out_row, dslot_row,
                        pos_of_row, true);
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

template <int WMAX>
static void tile_attrs_w(const EllSweep& e, int* bps) {
  static unsigned long long done = 0;  // one bit per device
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 64 && !(done >> dev & 1ull)) {
    auto set = [](const void* f) {
      cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, kTileSmemMax);
    };
    set((const void*)k_tile_sweep<ELL_ILU_F, WMAX>);
    set((const void*)k_tile_sweep<ELL_ILU_B, WMAX>);
    set((const void*)k_tile_sweep<ELL_ICC_F, WMAX>);
    set((const void*)k_tile_sweep<ELL_ICC_B, WMAX>);
    set((const void*)k_tile_sweep<ELL_SOR_F, WMAX>);
    set((const void*)k_tile_sweep<ELL_SOR_B, WMAX>);
    done |= 1ull << dev;
  }
  *bps = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, k_tile_sweep<ELL_SOR_B, WMAX>, 32,
                                                    e.smem) != cudaSuccess)
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

template <int MODE>
static void launch_tile(const EllSweep& e, const int* gate, int want, EllArgs a, TileArgs t,
                        DRef in, DRef out, cudaStream_t s) {
  const int g = std::max(1, e.grid);
  if (e.W <= 4)
    k_tile_sweep<MODE, 4><<<g, 32, e.smem, s>>>(gate, want, a, t, in, out);
  else if (e.W <= 8)
    k_tile_sweep<MODE, 8><<<g, 32, e.smem, s>>>(gate, want, a, t, in, out);
  else
    k_tile_sweep<MODE, kEllMaxW><<<g, 32, e.smem, s>>>(gate, want, a, t, in, out);
}

template <int MODE>
static void launch_mode(const EllSweep& e, const int* gate, int want, EllArgs a, DRef in,
                        DRef out, cudaStream_t s) {
  const int g = num_sms() * sweep_tuning().ctas_per_sm;
  if (e.W <= 4)
    k_ell_sweep<MODE, 4><<<g, kEllBlock, 0, s>>>(gate, want, a, in, out);
  else if (e.W <= 8)
    k_ell_sweep<MODE, 8><<<g, kEllBlock, 0, s>>>(gate, want, a, in, out);
  else
    k_ell_sweep<MODE, kEllMaxW><<<g, kEllBlock, 0, s>>>(gate, want, a, in, out);
}

int ell_sweep(int mode, const EllSweep& e, const int* gate, int want, DRef in, DRef out,
              double* val, const double* fval, double* aux, const double* auxin,
              const double* idiag, double omega, int use_t, int write_out, unsigned* tickets,
              DevErr* err, const double* coefsrc, cudaStream_t s) {
  if (e.n == 0) return GP_OK;
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
