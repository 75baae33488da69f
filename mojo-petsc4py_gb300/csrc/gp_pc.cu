// Preconditioner set-up and apply kernels.
//
//   PCSetUp_Jacobi / _Symmetric, PCApply_Jacobi  src/ported.mojo:505-567
//   MatInvertDiagonalForSOR_SeqAIJ, PCApply_SOR   src/ported.mojo:610-748
//   ILUApplyFactor_SeqAIJ                         src/ported.mojo:864-899
//   ICCApplyFactor_SeqAIJ                         src/ported.mojo:902-952
//   MatILUFactorNumeric_SeqAIJ                    src/ported.mojo:957-1037
//   MatICCFactorNumeric_SeqAIJ                    src/ported.mojo:1040-1124
//
// Triangular sweeps and numeric factorisations are sequential recurrences.
// They run as sync-free sweeps: warps take 32 rows at a time, in dependency
// level order, from a global ticket; a row reads each value it depends on
// from a value-as-flag array, spinning (with an iteration budget) until the
// producing row has stored it.  Every row computes its value with the same
// rounded operations in the same order as the sequential loop, so the applies
// and factors are bit-identical to the CPU recurrences.  Rows only wait on
// rows with smaller tickets, which are already held by running warps, so the
// sweep always makes progress.
#include <algorithm>
#include <vector>

#include "gp_pc.h"

namespace gp {

constexpr int kSweepBlock = 256;
constexpr int kSpinLimit = 1 << 22;   // polls per wait before giving up (~0.5 s)

__device__ __forceinline__ void raise_err(DevErr* err, int code, int where) {
  if (atomicCAS(&err->code, 0, code) == 0) err->where = where;
}

// Wait until *p holds a computed value (not the pending pattern).
__device__ __forceinline__ double wait_value(const double* p, DevErr* err, int where) {
  unsigned long long b = ld_relaxed_bits(p);
  if (b != kPending) return __longlong_as_double((long long)b);
  for (int spins = 0; spins < kSpinLimit; spins++) {
    __nanosleep(32);
    b = ld_relaxed_bits(p);
    if (b != kPending) return __longlong_as_double((long long)b);
  }
  raise_err(err, GP_ERR_TIMEOUT, where);
  return __longlong_as_double(0x7FF8000000000000LL);  // quiet NaN: dependents proceed
}

__device__ __forceinline__ bool wait_done(const int* p, int epoch, DevErr* err, int where) {
  if (ld_acquire_i32(p) == epoch) return true;
  for (int spins = 0; spins < kSpinLimit; spins++) {
    __nanosleep(32);
    if (ld_acquire_i32(p) == epoch) return true;
  }
  raise_err(err, GP_ERR_TIMEOUT, where);
  return false;
}

// Dynamic row hand-out: each warp takes 32 consecutive positions of `order`.
// The last warp to leave resets the ticket pair, so the next launch starts at
// zero without a separate reset.
template <class RowFn>
__device__ __forceinline__ void sweep_rows(int n, const int* __restrict__ order,
                                           unsigned* tickets, RowFn&& fn) {
  const int lane = threadIdx.x & 31;
  for (;;) {
    unsigned base = 0;
    if (lane == 0) base = atomicAdd(&tickets[0], 32u);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= (unsigned)n) break;
    const unsigned k = base + lane;
    if (k < (unsigned)n) fn(order[k]);
    __syncwarp();
  }
  if (lane == 0) {
    const unsigned total = gridDim.x * (blockDim.x / 32);
    // the last warp out resets the pair for the next launch
    if (atomic_add_acq_rel(&tickets[1], 1u) == total - 1) {
      tickets[0] = 0u;
      tickets[1] = 0u;
    }
  }
}

static int sweep_grid() { return num_sms() * 4; }
static int grid_for(int n) { return std::max(1, std::min((n + 255) / 256, num_sms() * 8)); }

// ------------------------------------------------------------------ Jacobi
__global__ void k_jacobi_fill(int n, int jtype, int sym, int use_abs, int fix_diag, double scale,
                              const int* __restrict__ rowptr, const double* __restrict__ val,
                              const int* __restrict__ diagpos, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double d = 0.0;
  if (jtype == 0) {
    d = diagpos[i] >= 0 ? val[diagpos[i]] : 0.0;
  } else {
    for (int j = rowptr[i]; j < rowptr[i + 1]; j++) {
      const double v = val[j];
      if (jtype == 1) {
        const double a = fabs(v);
        d = a > d ? a : d;
      } else if (jtype == 2) {
        d = add(d, fabs(v));
      } else {
        d = add(d, v);
      }
    }
  }
  if (sym) {  // PCSetUp_Jacobi_Symmetric: 1/sqrt|d|, zero -> 1
    out[i] = d < 0.0 ? div_(1.0, __dsqrt_rn(fabs(-d)))
                     : (d > 0.0 ? div_(1.0, __dsqrt_rn(fabs(d))) : 1.0);
    return;
  }
  if (jtype == 2) {  // rowl1: sign follows the true diagonal, optional blend
    const double td = diagpos[i] >= 0 ? val[diagpos[i]] : 0.0;
    if (td < 0.0) d = -d;
    if (scale != 1.0) d = add(mul(scale, sub(d, td)), td);
  }
  d = (d == 0.0) ? 0.0 : div_(1.0, d);
  if (use_abs) d = fabs(d);
  if (fix_diag && d == 0.0) d = 1.0;
  out[i] = d;
}

__global__ void k_pmult(const int* gate, int want, int n, DRef xr, const double* __restrict__ d,
                        DRef yr) {
  if (gated_off(gate, want)) return;
  const double* __restrict__ x = xr.get();
  double* __restrict__ y = yr.get();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    y[i] = mul(x[i], d[i]);
}

__global__ void k_copy_g(const int* gate, int want, int n, DRef xr, DRef yr) {
  if (gated_off(gate, want)) return;
  const double* __restrict__ x = xr.get();
  double* __restrict__ y = yr.get();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    y[i] = x[i];
}

// ------------------------------------------------------------------ SOR
__global__ void k_clear_word(const int* gate, int want, int* w) {
  if (gated_off(gate, want)) return;
  *w = 0;
}

static bool stream_capturing(cudaStream_t s) {
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &st) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return st != cudaStreamCaptureStatusNone;
}

// With `stale` given, runs only while *stale is nonzero (A's values changed
// since the last run): the result depends on the values alone.
__global__ void k_sor_diag(int n, double omega, double fshift, const int* __restrict__ diagpos,
                           const double* __restrict__ val, double* __restrict__ idiag,
                           double* __restrict__ mdiag, const int* gate = nullptr, int want = 0,
                           const int* stale = nullptr) {
  if (gated_off(gate, want)) return;
  if (stale && *stale == 0) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double a = val[diagpos[i]];
  mdiag[i] = a;
  idiag[i] = (omega == 1.0 && fshift <= 0.0) ? div_(1.0, a) : div_(omega, add(fshift, a));
}

// SOR's ELL coefficients follow A's current values (gathered by an apply
// while *stale is nonzero)
__global__ void k_ell_refresh_g(const int* gate, int want, int n, const int* __restrict__ cnt,
                                const int* __restrict__ cslot, const double* __restrict__ src,
                                double* __restrict__ coef, const int* stale) {
  if (gated_off(gate, want)) return;
  if (*stale == 0) return;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    const int c = cnt[p];
    for (int e = 0; e < c; e++) {
      const int cs = cslot[(size_t)e * n + p];
      coef[(size_t)e * n + p] = cs >= 0 ? src[cs] : 0.0;  // < 0: no term (brick form)
    }
  }
}

__global__ void k_fill_pending(const int* gate, int want, int n, double* __restrict__ a,
                               double* __restrict__ b) {
  if (gated_off(gate, want)) return;
  const double p = __longlong_as_double((long long)kPending);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    a[i] = p;
    if (b) b[i] = p;
  }
}

// Forward Gauss-Seidel half with zero initial guess: t_i = x_i - sum_{j<i}
// a_ij y_j, y_i = t_i * idiag_i.  (MatSOR_SeqAIJ's zero-guess prologue.)
__global__ void __launch_bounds__(kSweepBlock) k_sor_fwd(
    const int* gate, int want, int n, const int* __restrict__ order, unsigned* tickets,
    const int* __restrict__ rowptr, const int* __restrict__ colind, const double* __restrict__ val,
    const int* __restrict__ diagpos, const double* __restrict__ idiag, DRef xr,
    double* __restrict__ t, double* yf, DRef youtr, DevErr* err) {
  if (gated_off(gate, want)) return;
  const double* __restrict__ x = xr.get();
  double* __restrict__ yout = youtr.get();
  sweep_rows(n, order, tickets, [&](int i) {
    double sum = x[i];
    const int jend = diagpos[i];
    for (int j = rowptr[i]; j < jend; j++)
      sum = sub(sum, mul(val[j], wait_value(&yf[colind[j]], err, 1)));
    t[i] = sum;
    const double y = mul(sum, idiag[i]);
    if (yout) yout[i] = y;
    st_relaxed(&yf[i], y);
  });
}

// Backward half.  use_t: relax from the forward value, (1 - omega) y_i +
// (t_i - sum_{j>i} a_ij y_j) idiag_i; otherwise plain back substitution from x.
__global__ void __launch_bounds__(kSweepBlock) k_sor_bwd(
    const int* gate, int want, int n, const int* __restrict__ order, unsigned* tickets,
    const int* __restrict__ rowptr, const int* __restrict__ colind, const double* __restrict__ val,
    const int* __restrict__ diagpos, const double* __restrict__ idiag, DRef xr,
    const double* __restrict__ t, const double* __restrict__ yf, double* yb, DRef youtr,
    double omega, int use_t, DevErr* err) {
  if (gated_off(gate, want)) return;
  const double* __restrict__ x = xr.get();
  double* __restrict__ yout = youtr.get();
  const double om1 = sub(1.0, omega);
  sweep_rows(n, order, tickets, [&](int i) {
    double sum = use_t ? t[i] : x[i];
    const int jend = rowptr[i + 1];
    for (int j = diagpos[i] + 1; j < jend; j++)
      sum = sub(sum, mul(val[j], wait_value(&yb[colind[j]], err, 2)));
    const double y = use_t ? add(mul(om1, yf[i]), mul(sum, idiag[i])) : mul(sum, idiag[i]);
    yout[i] = y;
    st_relaxed(&yb[i], y);
  });
}

// ------------------------------------------------------------------ ILU solve
// Forward: yf_i = b_{r_i} - sum_{L(i)} ba_j yf_{bj_j}  (L rows, unit diagonal)
__global__ void __launch_bounds__(kSweepBlock) k_ilu_fwd(
    const int* gate, int want, int n, const int* __restrict__ order, unsigned* tickets,
    const int* __restrict__ bi, const int* __restrict__ bj, const double* __restrict__ ba,
    const int* __restrict__ perm_r, DRef br, double* yf, DevErr* err) {
  if (gated_off(gate, want)) return;
  const double* __restrict__ b = br.get();
  sweep_rows(n, order, tickets, [&](int i) {
    double sum = b[perm_r[i]];
    const int jend = bi[i + 1];
    for (int j = bi[i]; j < jend; j++) sum = sub(sum, mul(ba[j], wait_value(&yf[bj[j]], err, 3)));
    st_relaxed(&yf[i], sum);
  });
}

// Backward: yb_i = (yf_i - sum_{U(i)} ba_j yb_{bj_j}) * ba_{diag}; x_{c_i} = yb_i
__global__ void __launch_bounds__(kSweepBlock) k_ilu_bwd(
    const int* gate, int want, int n, const int* __restrict__ order, unsigned* tickets,
    const int* __restrict__ bj, const double* __restrict__ ba, const int* __restrict__ bdiag,
    const int* __restrict__ perm_c, const double* __restrict__ yf, double* yb, DRef xr,
    DevErr* err) {
  if (gated_off(gate, want)) return;
  double* __restrict__ x = xr.get();
  sweep_rows(n, order, tickets, [&](int i) {
    const int v = bdiag[i + 1] + 1;
    const int nz = bdiag[i] - bdiag[i + 1] - 1;
    double sum = yf[i];
    for (int j = 0; j < nz; j++)
      sum = sub(sum, mul(ba[v + j], wait_value(&yb[bj[v + j]], err, 4)));
    sum = mul(sum, ba[v + nz]);
    x[perm_c[i]] = sum;
    st_relaxed(&yb[i], sum);
  });
}

// ------------------------------------------------------------------ IC solve
// Forward (U^T D y = b in gather form): w_k = b_{c_k} + sum_{i<k, U(i,k)}
// ua(i,k) w_i in ascending i -- the order the reference's scatter adds them --
// and ys_k = w_k * ua_{diag(k)}.
__global__ void __launch_bounds__(kSweepBlock) k_icc_fwd(
    const int* gate, int want, int n, const int* __restrict__ order, unsigned* tickets,
    const int* __restrict__ tptr, const int* __restrict__ trow, const int* __restrict__ tslot,
    const double* __restrict__ ua, const int* __restrict__ bdiag,
    const int* __restrict__ perm_c, DRef br, double* yf, double* __restrict__ ys,
    DevErr* err) {
  if (gated_off(gate, want)) return;
  const double* __restrict__ b = br.get();
  sweep_rows(n, order, tickets, [&](int k) {
    double w = b[perm_c[k]];
    const int eend = tptr[k + 1];
    for (int e = tptr[k]; e < eend; e++)
      w = add(w, mul(ua[tslot[e]], wait_value(&yf[trow[e]], err, 5)));
    ys[k] = mul(w, ua[bdiag[k]]);
    st_relaxed(&yf[k], w);
  });
}

// Backward: z_i = ys_i + sum_{j in U(i) strict} ua_j z_{uj_j}; x_{c_i} = z_i
__global__ void __launch_bounds__(kSweepBlock) k_icc_bwd(
    const int* gate, int want, int n, const int* __restrict__ order, unsigned* tickets,
    const int* __restrict__ bi, const int* __restrict__ bj, const double* __restrict__ ua,
    const int* __restrict__ bdiag, const int* __restrict__ perm_c,
    const double* __restrict__ ys, double* yb, DRef xr, DevErr* err) {
  if (gated_off(gate, want)) return;
  double* __restrict__ x = xr.get();
  sweep_rows(n, order, tickets, [&](int i) {
    double z = ys[i];
    const int jend = bdiag[i];
    for (int j = bi[i]; j < jend; j++) z = add(z, mul(ua[j], wait_value(&yb[bj[j]], err, 6)));
    x[perm_c[i]] = z;
    st_relaxed(&yb[i], z);
  });
}

// ------------------------------------------------------------------ IC solve, R columns
// The same two sweeps on R right-hand sides stored row-major (element (row,
// c) at row * R + c): each row is handed to R lanes of a warp, one column a
// lane, each waiting on its own column's values.  Every column is folded with
// exactly the operations of k_icc_fwd / k_icc_bwd.
template <class RowFn>
__device__ __forceinline__ void sweep_rows_cols(int R, int n, const int* __restrict__ order,
                                                unsigned* tickets, RowFn&& fn) {
  const int lane = threadIdx.x & 31, per = 32 / R;
  for (;;) {
    unsigned base = 0;
    if (lane == 0) base = atomicAdd(&tickets[0], (unsigned)per);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= (unsigned)n) break;
    const unsigned k = base + lane / R;
    if (lane < per * R && k < (unsigned)n) fn(order[k], lane % R);
    __syncwarp();
  }
  if (lane == 0) {
    const unsigned total = gridDim.x * (blockDim.x / 32);
    if (atomic_add_acq_rel(&tickets[1], 1u) == total - 1) {
      tickets[0] = 0u;
      tickets[1] = 0u;
    }
  }
}

__global__ void __launch_bounds__(kSweepBlock) k_icc_fwd_cols(
    int R, int n, const int* __restrict__ order, unsigned* tickets, const int* __restrict__ tptr,
    const int* __restrict__ trow, const int* __restrict__ tslot, const double* __restrict__ ua,
    const int* __restrict__ bdiag, const int* __restrict__ perm_c, const double* __restrict__ b,
    double* yf, double* __restrict__ ys, DevErr* err) {
  sweep_rows_cols(R, n, order, tickets, [&](int k, int c) {
    double w = b[(size_t)perm_c[k] * R + c];
    const int eend = tptr[k + 1];
    for (int e = tptr[k]; e < eend; e++)
      w = add(w, mul(ua[tslot[e]], wait_value(&yf[(size_t)trow[e] * R + c], err, 15)));
    ys[(size_t)k * R + c] = mul(w, ua[bdiag[k]]);
    st_relaxed(&yf[(size_t)k * R + c], w);
  });
}

__global__ void __launch_bounds__(kSweepBlock) k_icc_bwd_cols(
    int R, int n, const int* __restrict__ order, unsigned* tickets, const int* __restrict__ bi,
    const int* __restrict__ bj, const double* __restrict__ ua, const int* __restrict__ bdiag,
    const int* __restrict__ perm_c, const double* __restrict__ ys, double* yb,
    double* __restrict__ x, DevErr* err) {
  sweep_rows_cols(R, n, order, tickets, [&](int i, int c) {
    double z = ys[(size_t)i * R + c];
    const int jend = bdiag[i];
    for (int j = bi[i]; j < jend; j++)
      z = add(z, mul(ua[j], wait_value(&yb[(size_t)bj[j] * R + c], err, 16)));
    x[(size_t)perm_c[i] * R + c] = z;
    st_relaxed(&yb[(size_t)i * R + c], z);
  });
}

int pc_apply_icc_cols(Pc* pc, int R, const double* x, double* y, double* vf, double* vb,
                      double* ys, cudaStream_t s) {
  if (!pc->ready || pc->opt.type != PC_ICC) {
    set_error("pc_apply_icc_cols: an IC preconditioner that has been set up is needed");
    return GP_ERR_NOT_SETUP;
  }
  if (R < 1 || R > 32 || (32 % R)) {
    set_error("pc_apply_icc_cols: R must divide 32");
    return GP_ERR_ARG;
  }
  const int n = pc->n;
  if (n == 0) return GP_OK;
  if ((int64_t)n * R > INT32_MAX) {
    set_error("pc_apply_icc_cols: n * R must fit in 32 bits");
    return GP_ERR_ARG;
  }
  k_fill_pending<<<grid_for(n * R), 256, 0, s>>>(nullptr, 0, n * R, vf, vb);
  const int sg = sweep_grid();
  k_icc_fwd_cols<<<sg, kSweepBlock, 0, s>>>(R, n, pc->fwd.order, pc->tickets, pc->tptr,
                                            pc->trow, pc->tslot, pc->ba, pc->bdiag, pc->perm_c,
                                            x, vf, ys, pc->err);
  k_icc_bwd_cols<<<sg, kSweepBlock, 0, s>>>(R, n, pc->bwd.order, pc->tickets + 2, pc->bi,
                                            pc->bj, pc->ba, pc->bdiag, pc->perm_c, ys, vb, y,
                                            pc->err);
  GP_CHECK_LAUNCH();
  return GP_OK;
}

// ------------------------------------------------------------------ ILU numeric
// Row i of the factor is accumulated in its own slots of `ba` (the reference's
// dense `rtmp` restricted to the row's pattern; positions outside the pattern
// are never stored or read back there either).

// upd_ptr/upd_dst/upd_src: for each L slot k of row i, the updates its pivot
// row makes to row i -- (row i's slot, pivot row's U slot) pairs in the
// pivot row's U order -- found once on the host (the pattern is fixed), so
// the numeric phase does no pattern searches.
__global__ void __launch_bounds__(kSweepBlock) k_ilu_numeric(
    int n, const int* __restrict__ order, unsigned* tickets, const int* __restrict__ arow,
    const double* __restrict__ aval, const int* __restrict__ amap, const int* __restrict__ perm_r,
    const int* __restrict__ bi, const int* __restrict__ bj, const int* __restrict__ bdiag,
    const int* __restrict__ upd_ptr, const int* __restrict__ upd_dst,
    const int* __restrict__ upd_src, double* ba, int* done, int epoch, DevErr* err) {
  sweep_rows(n, order, tickets, [&](int i) {
    // zero the row's slots, then load A's row r_i
    for (int j = bi[i]; j < bi[i + 1]; j++) ba[j] = 0.0;
    for (int j = bdiag[i + 1] + 1; j <= bdiag[i]; j++) ba[j] = 0.0;
    const int ri = perm_r[i];
    for (int j = arow[ri]; j < arow[ri + 1]; j++) {
      const int s = amap[j];
      if (s >= 0) ba[s] = aval[j];
    }
    // eliminate with each L entry in ascending column order; once the pivot
    // row is done its pivot and the U values this row needs are loaded
    // together (one L2 round trip), then applied in order
    constexpr int kU = 8;
    for (int k = bi[i]; k < bi[i + 1]; k++) {
      const double pc = ba[k];
      if (pc != 0.0) {
        const int row = bj[k];
        const int u0 = upd_ptr[k], u1 = upd_ptr[k + 1];
        int dst[kU], src[kU];
#pragma unroll
        for (int q = 0; q < kU; q++)
          if (u0 + q < u1) {
            dst[q] = upd_dst[u0 + q];
            src[q] = upd_src[u0 + q];
          }
        const int pslot = bdiag[row];
        wait_done(&done[row], epoch, err, 7);
        const double pv = __ldcg(&ba[pslot]);
        double sv[kU];
#pragma unroll
        for (int q = 0; q < kU; q++)
          if (u0 + q < u1) sv[q] = __ldcg(&ba[src[q]]);
        const double m = mul(pc, pv);
        ba[k] = m;
#pragma unroll
        for (int q = 0; q < kU; q++)
          if (u0 + q < u1) ba[dst[q]] = sub(ba[dst[q]], mul(m, sv[q]));
        for (int u = u0 + kU; u < u1; u++) {  // rows with more fill
          const int d = upd_dst[u];
          ba[d] = sub(ba[d], mul(m, __ldcg(&ba[upd_src[u]])));
        }
      }
    }
    ba[bdiag[i]] = div_(1.0, ba[bdiag[i]]);
    st_release_i32(&done[i], epoch);
  });
}

// ------------------------------------------------------------------ IC numeric
// Up-looking row k: dk and the strict row accumulate A's values, then each
// contributor row i (U(i,k) != 0) in the order the reference's il/c2r chains
// visit them (recorded on the host): uikdi = -U(i,k)/d_i, dk += uikdi U(i,k),
// row k += uikdi U(i, k+1:).  Unscaled rows live in `orig`; the scaled
// off-diagonal U(i,k) = uikdi is written into `ba` by row k, the only writer.
__device__ __forceinline__ int icc_find(int col, int k, const int* __restrict__ bi,
                                        const int* __restrict__ bj, const int* __restrict__ bdiag) {
  int lo = bi[k], hi = bdiag[k];
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    int c = bj[mid];
    if (c == col) return mid;
    if (c < col) lo = mid + 1; else hi = mid;
  }
  return -1;
}

__global__ void __launch_bounds__(kSweepBlock) k_icc_numeric(
    int n, const int* __restrict__ order, unsigned* tickets, const int* __restrict__ arow,
    const double* __restrict__ aval, const int* __restrict__ amap, const int* __restrict__ perm_r,
    const int* __restrict__ bi, const int* __restrict__ bj, const int* __restrict__ bdiag,
    const int* __restrict__ cptr, const int* __restrict__ crow, const int* __restrict__ cslot,
    double* ba, double* orig, int* done, int epoch, DevErr* err) {
  sweep_rows(n, order, tickets, [&](int k) {
    for (int j = bi[k]; j <= bdiag[k]; j++) orig[j] = 0.0;
    const int rk = perm_r[k];
    for (int j = arow[rk]; j < arow[rk + 1]; j++) {
      const int s = amap[j];
      if (s >= 0) orig[s] = aval[j];
    }
    double dk = orig[bdiag[k]];
    for (int e = cptr[k]; e < cptr[k + 1]; e++) {
      const int i = crow[e], ili = cslot[e];
      wait_done(&done[i], epoch, err, 8);
      const double uik = __ldcg(&orig[ili]);
      const double uikdi = mul(-uik, __ldcg(&ba[bdiag[i]]));
      dk = add(dk, mul(uikdi, uik));
      ba[ili] = uikdi;
      const int jmax = bdiag[i];
      for (int j = ili + 1; j < jmax; j++) {
        const int s = icc_find(bj[j], k, bi, bj, bdiag);
        if (s >= 0) orig[s] = add(orig[s], mul(uikdi, __ldcg(&orig[j])));
      }
    }
    for (int j = bi[k]; j < bdiag[k]; j++) ba[j] = orig[j];
    ba[bdiag[k]] = div_(1.0, dk);
    st_release_i32(&done[k], epoch);
  });
}

// ================================================================== host side

template <typename T>
static int upload(T** d, const std::vector<T>& h, cudaStream_t s) {
  GP_CUDA(cudaMalloc(d, std::max<size_t>(h.size(), 1) * sizeof(T)));
  if (!h.empty())
    GP_CUDA(cudaMemcpyAsync(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s));
  return GP_OK;
}

static int dalloc(double** p, int64_t n) {
  GP_CUDA(cudaMalloc(p, std::max<int64_t>(n, 1) * sizeof(double)));
  return GP_OK;
}

static void free_all(Pc* pc) {
  void* ptrs[] = {pc->diag, pc->diagsqrt, pc->idiag, pc->mdiag, pc->bi, pc->bj, pc->bdiag,
                  pc->perm_r, pc->perm_c, pc->perm_ic, pc->ba, pc->ba_orig, pc->done, pc->cptr, pc->crow,
                  pc->cslot, pc->tptr, pc->trow, pc->tslot, pc->amap, pc->fwd.order,
                  pc->bwd.order, pc->num.order, pc->yf, pc->yb, pc->ys, pc->t, pc->tickets,
                  pc->err, pc->upd_ptr, pc->upd_dst, pc->upd_src, pc->sor_stale};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  ell_free(pc->ef);
  ell_free(pc->eb);
  ell_free(pc->etf);
  ell_free(pc->etb);
  PcOptions keep = pc->opt;
  *pc = Pc();
  pc->opt = keep;
}

int pc_create(Pc** out) {
  *out = new Pc();
  return GP_OK;
}

int pc_destroy(Pc* pc) {
  if (!pc) return GP_OK;
  free_all(pc);
  delete pc;
  return GP_OK;
}

static int plan(SweepPlan& p, int n, const std::vector<int>& dptr, const std::vector<int>& dcol,
                bool forward, cudaStream_t s, std::vector<int>* order_out = nullptr) {
  std::vector<int> order;
  level_order(n, dptr, dcol, forward, order, &p.nlevels);
  if (order_out) *order_out = order;
  GP_TRY(upload(&p.order, order, s));
  return GP_OK;
}

int pc_check(Pc* pc, cudaStream_t s) {
  // none and Jacobi have no bounded waits that could set the flag: their
  // standalone apply stays asynchronous
  if (!pc->err || pc->opt.type == PC_NONE || pc->opt.type == PC_JACOBI) return GP_OK;
  DevErr h{};
  GP_CUDA(cudaMemcpyAsync(&h, pc->err, sizeof(DevErr), cudaMemcpyDeviceToHost, s));
  GP_CUDA(cudaStreamSynchronize(s));
  if (h.code == 0) return GP_OK;
  GP_CUDA(cudaMemsetAsync(pc->err, 0, sizeof(DevErr), s));
  GP_CUDA(cudaStreamSynchronize(s));
  set_error("preconditioner sweep wait ran out of budget (site " + std::to_string(h.where) +
            ")");
  return h.code;
}

static int check_sorted_with_diag(const Csr* A, const char* who) {
  for (int i = 0; i < A->n; i++) {
    bool diag = false;
    for (int j = A->h_rowptr[i]; j < A->h_rowptr[i + 1]; j++) {
      if (j > A->h_rowptr[i] && A->h_colind[j] <= A->h_colind[j - 1]) {
        set_error(std::string(who) + ": columns must be strictly ascending in each row");
        return GP_ERR_ARG;
      }
      if (A->h_colind[j] == i) diag = true;
    }
    if (!diag) {
      set_error(std::string(who) + ": row " + std::to_string(i) + " has no diagonal entry");
      return GP_ERR_ARG;
    }
  }
  return GP_OK;
}

static int setup_sor(Pc* pc, cudaStream_t s) {
  const Csr* A = pc->A;
  const int n = A->n;
  GP_TRY(check_sorted_with_diag(A, "SOR"));
  GP_TRY(dalloc(&pc->idiag, n));
  GP_TRY(dalloc(&pc->mdiag, n));
  // the strict triangles' columns and slots: counts per row, prefix sums,
  // then each row fills its own range (host threads)
  std::vector<int> lp(n + 1, 0), lc, ls, up(n + 1, 0), uc, us;
  const int* rp = A->h_rowptr.data();
  const int* ci = A->h_colind.data();
  host_parallel_for(n, [&](int64_t i0, int64_t i1) {
    for (int i = (int)i0; i < (int)i1; i++) {
      int nl = 0, nu = 0;
      for (int j = rp[i]; j < rp[i + 1]; j++) {
        nl += ci[j] < i;
        nu += ci[j] > i;
      }
      lp[i + 1] = nl;
      up[i + 1] = nu;
    }
  });
  for (int i = 0; i < n; i++) {
    lp[i + 1] += lp[i];
    up[i + 1] += up[i];
  }
  lc.resize(lp[n]);
  ls.resize(lp[n]);
  uc.resize(up[n]);
  us.resize(up[n]);
  host_parallel_for(n, [&](int64_t i0, int64_t i1) {
    for (int i = (int)i0; i < (int)i1; i++) {
      int ql = lp[i], qu = up[i];
      for (int j = rp[i]; j < rp[i + 1]; j++) {
        const int c = ci[j];
        if (c < i) {
          lc[ql] = c;
          ls[ql++] = j;
        }
        if (c > i) {
          uc[qu] = c;
          us[qu++] = j;
        }
      }
    }
  });
  std::vector<int> of, ob, fpos, none;
  setup_mark("triangles");
  GP_TRY(plan(pc->fwd, n, lp, lc, true, s, &of));
  GP_TRY(plan(pc->bwd, n, up, uc, false, s, &ob));
  setup_mark("levels");
  GP_TRY(ell_build(pc->ef, ELL_SOR_F, n, true, of, lp, lc, ls, none, none, none, &fpos,
                   pc->fwd.nlevels));
  setup_mark("fwd-layout");
  GP_TRY(ell_build(pc->eb, ELL_SOR_B, n, false, ob, up, uc, us, fpos, none, none, nullptr,
                   pc->bwd.nlevels));
  setup_mark("bwd-layout");
  pc->vlen = std::max({n, pc->ef.n, pc->eb.n});
  GP_TRY(dalloc(&pc->t, pc->vlen));
  GP_TRY(dalloc(&pc->yf, pc->vlen));
  GP_TRY(dalloc(&pc->yb, pc->vlen));
  GP_CUDA(cudaMalloc(&pc->sor_stale, sizeof(int)));
  GP_CUDA(cudaMemsetAsync(pc->sor_stale, 1, sizeof(int), s));  // nonzero: recompute
  pc->sor_vver = A->vver;
  if (n) {
    k_sor_diag<<<(n + 255) / 256, 256, 0, s>>>(n, pc->opt.omega, pc->opt.fshift, A->diagpos,
                                                A->val, pc->idiag, pc->mdiag);
    GP_CHECK_LAUNCH();
  }
  return GP_OK;
}

static int perms(Pc* pc, std::vector<int>& r, std::vector<int>& ic) {
  const Csr* A = pc->A;
  const int n = A->n;
  if (pc->opt.ordering == 1)
    GP_TRY(rcm_order(A->h_rowptr, A->h_colind, n, r));
  else if (pc->opt.ordering == 2)
    GP_TRY(color_order(A->h_rowptr, A->h_colind, n, r, nullptr));
  else {
    r.resize(n);
    for (int i = 0; i < n; i++) r[i] = i;
  }
  ic.assign(n, 0);
  for (int i = 0; i < n; i++) ic[r[i]] = i;
  return GP_OK;
}

// Sweep plans and device arrays of an ILU factor whose pattern is in pc->pat
// (the reference layout).  Used after the symbolic phase and when a factor is
// imported as it is.
static int ilu_prepare(Pc* pc, const std::vector<int>& perm_c, cudaStream_t s) {
  const int n = pc->n;
  FactorPattern& P = pc->pat;
  std::vector<int> lp(n + 1), lc(P.bj.begin(), P.bj.begin() + P.bi[n]), ls(P.bi[n]);
  for (int i = 0; i <= n; i++) lp[i] = P.bi[i];
  for (int j = 0; j < P.bi[n]; j++) ls[j] = j;
  // U rows (strict part, stored reversed between bdiag[i + 1] and bdiag[i])
  std::vector<int> up(n + 1, 0), uc, us, dsl(n);
  for (int i = 0; i < n; i++) up[i + 1] = up[i] + (P.bdiag[i] - P.bdiag[i + 1] - 1);
  uc.resize(up[n]);
  us.resize(up[n]);
  host_parallel_for(n, [&](int64_t i0, int64_t i1) {
    for (int i = (int)i0; i < (int)i1; i++) {
      int q = up[i];
      for (int j = P.bdiag[i + 1] + 1; j < P.bdiag[i]; j++, q++) {
        uc[q] = P.bj[j];
        us[q] = j;
      }
      dsl[i] = P.bdiag[i];
    }
  });
  std::vector<int> of, ob, fpos, none;
  setup_mark("triangles");
  GP_TRY(plan(pc->fwd, n, lp, lc, true, s, &of));
  GP_TRY(plan(pc->bwd, n, up, uc, false, s, &ob));
  setup_mark("levels");
  GP_TRY(ell_build(pc->ef, ELL_ILU_F, n, true, of, lp, lc, ls, P.r, none, none, &fpos,
                   pc->fwd.nlevels));
  setup_mark("fwd-layout");
  GP_TRY(ell_build(pc->eb, ELL_ILU_B, n, false, ob, up, uc, us, fpos, perm_c, dsl, nullptr,
                   pc->bwd.nlevels));
  setup_mark("bwd-layout");
  // the numeric phase's update lists (the searches of the elimination, once);
  // kept to the end of the function: the copies below are asynchronous
  std::vector<int> uptr(P.bi[n] + 1, 0), udst, usrc;
  {
    auto find = [&](int col, int i) {
      int lo, hi;
      if (col < i) {
        lo = P.bi[i];
        hi = P.bi[i + 1];
      } else if (col == i) {
        return P.bdiag[i];
      } else {
        lo = P.bdiag[i + 1] + 1;
        hi = P.bdiag[i];
      }
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const int c = P.bj[mid];
        if (c == col) return mid;
        if (c < col)
          lo = mid + 1;
        else
          hi = mid;
      }
      return -1;
    };
    // count the updates of each L slot, then fill them: both passes over
    // rows on host threads (a row's L slots are its own), the same lists in
    // the same order as one pass
    auto each = [&](int i, int k, auto&& hit) {
      const int row = P.bj[k];
      const int pj = P.bdiag[row + 1] + 1;
      const int nz = P.bdiag[row] - P.bdiag[row + 1] - 1;
      for (int j = 0; j < nz; j++) {
        const int d = find(P.bj[pj + j], i);
        if (d >= 0) hit(d, pj + j);
      }
    };
    host_parallel_for(n, [&](int64_t i0, int64_t i1) {
      for (int i = (int)i0; i < (int)i1; i++)
        for (int k = P.bi[i]; k < P.bi[i + 1]; k++) {
          int c = 0;
          each(i, k, [&](int, int) { c++; });
          uptr[k + 1] = c;
        }
    });
    int64_t tot = 0;
    for (int k = 0; k < P.bi[n]; k++) {
      tot += uptr[k + 1];
      if (tot > INT32_MAX - 1) {
        set_error("ILU: the factor's update lists are too large for 32-bit indices");
        return GP_ERR_ARG;
      }
      uptr[k + 1] = (int)tot;
    }
    udst.resize(tot);
    usrc.resize(tot);
    host_parallel_for(n, [&](int64_t i0, int64_t i1) {
      for (int i = (int)i0; i < (int)i1; i++)
        for (int k = P.bi[i]; k < P.bi[i + 1]; k++) {
          int q = uptr[k];
          each(i, k, [&](int d, int src) {
            udst[q] = d;
            usrc[q] = src;
            q++;
          });
        }
    });
    setup_mark("update-lists");
    GP_TRY(upload(&pc->upd_ptr, uptr, s));
    GP_TRY(upload(&pc->upd_dst, udst, s));
    GP_TRY(upload(&pc->upd_src, usrc, s));
  }
  GP_TRY(upload(&pc->bi, P.bi, s));
  GP_TRY(upload(&pc->bj, P.bj, s));
  GP_TRY(upload(&pc->bdiag, P.bdiag, s));
  GP_TRY(upload(&pc->perm_r, P.r, s));
  GP_TRY(upload(&pc->perm_c, perm_c, s));
  GP_TRY(upload(&pc->perm_ic, P.ic, s));
  GP_TRY(dalloc(&pc->ba, std::max(P.nnz, 1)));
  GP_CUDA(cudaMalloc(&pc->done, std::max(n, 1) * sizeof(int)));
  GP_CUDA(cudaMemsetAsync(pc->done, 0, std::max(n, 1) * sizeof(int), s));
  pc->vlen = std::max({n, pc->ef.n, pc->eb.n});
  GP_TRY(dalloc(&pc->yf, pc->vlen));
  GP_TRY(dalloc(&pc->yb, pc->vlen));
  GP_CUDA(cudaStreamSynchronize(s));  // host vectors above go out of scope
  return GP_OK;
}

// A slot -> factor slot, for the numeric factorisation from A's values.
static int ilu_amap(Pc* pc, const Csr* A, cudaStream_t s) {
  const int n = A->n;
  const FactorPattern& P = pc->pat;
  std::vector<int> amap(std::max<int64_t>(A->nnz, 1), -1);
  // rows are independent: each writes the slots of its own entries
  host_parallel_for(n, [&](int64_t i0, int64_t i1) {
    for (int i = (int)i0; i < (int)i1; i++) {
      const int ri = P.r[i];
      for (int j = A->h_rowptr[ri]; j < A->h_rowptr[ri + 1]; j++) {
        const int c = P.ic[A->h_colind[j]];
        int lo, hi;
        if (c < i) {
          lo = P.bi[i];
          hi = P.bi[i + 1];
        } else if (c == i) {
          amap[j] = P.bdiag[i];
          continue;
        } else {
          lo = P.bdiag[i + 1] + 1;
          hi = P.bdiag[i];
        }
        auto it = std::lower_bound(P.bj.begin() + lo, P.bj.begin() + hi, c);
        if (it != P.bj.begin() + hi && *it == c) amap[j] = (int)(it - P.bj.begin());
      }
    }
  });
  if (pc->amap) cudaFree(pc->amap);
  pc->amap = nullptr;
  GP_TRY(upload(&pc->amap, amap, s));
  GP_CUDA(cudaStreamSynchronize(s));
  return GP_OK;
}

static int setup_ilu(Pc* pc, cudaStream_t s) {
  const Csr* A = pc->A;
  std::vector<int> r, ic;
  GP_TRY(perms(pc, r, ic));
  setup_mark("ordering");
  GP_TRY(ilu_symbolic(A, pc->opt.levels, r, ic, pc->pat));
  setup_mark("symbolic");
  // the factor lives in the permuted ordering; the solution is mapped back
  // with the row ordering itself (python/mojopetsc4py/PETSc/PC.py:434-437)
  GP_TRY(ilu_prepare(pc, r, s));
  return ilu_amap(pc, A, s);
}

// Plans and device arrays of an IC factor in pc->pat: the transposed strict
// pattern (forward sweep), the contributor lists in the order the
// reference's il/c2r chains visit them (numeric factorisation), the strict
// rows (backward sweep).
static int icc_prepare(Pc* pc, const std::vector<int>& perm_c, cudaStream_t s) {
  const int n = pc->n;
  FactorPattern& P = pc->pat;
  // each row's contributors are visited while that row is processed, so
  // they go straight into the flat lists in row order
  std::vector<int> c2r(n, n), il(n, 0), cptr(n + 1, 0), crow, cslot;
  crow.reserve(std::max(P.nnz - n, 0));
  cslot.reserve(std::max(P.nnz - n, 0));
  for (int k = 0; k < n; k++) {  // src/ported.mojo:1040-1124 on the pattern alone
    int i = c2r[k];
    while (i < k) {
      const int nexti = c2r[i];
      const int ili = il[i];
      crow.push_back(i);
      cslot.push_back(ili);
      const int jmin = ili + 1, jmax = P.bi[i + 1];
      if (jmin < jmax) {
        il[i] = jmin;
        const int cj = P.bj[jmin];
        c2r[i] = c2r[cj];
        c2r[cj] = i;
      }
      i = nexti;
    }
    const int jmin = P.bi[k], jmax = P.bi[k + 1] - 1;
    if (jmin < jmax) {
      il[k] = jmin;
      const int cj = P.bj[jmin];
      c2r[k] = c2r[cj];
      c2r[cj] = k;
    }
    cptr[k + 1] = (int)crow.size();
  }
  std::vector<int> tptr(n + 1, 0), trow(std::max(P.nnz - n, 1)), tslot(std::max(P.nnz - n, 1));
  for (int i = 0; i < n; i++)
    for (int j = P.bi[i]; j < P.bdiag[i]; j++) tptr[P.bj[j] + 1]++;
  for (int k = 0; k < n; k++) tptr[k + 1] += tptr[k];
  {
    std::vector<int> fill(tptr.begin(), tptr.end() - 1);
    for (int i = 0; i < n; i++)
      for (int j = P.bi[i]; j < P.bdiag[i]; j++) {
        const int k = P.bj[j];
        trow[fill[k]] = i;
        tslot[fill[k]] = j;
        fill[k]++;
      }
  }
  std::vector<int> up(n + 1, 0), uc;
  for (int i = 0; i < n; i++) {
    for (int j = P.bi[i]; j < P.bdiag[i]; j++) uc.push_back(P.bj[j]);
    up[i + 1] = (int)uc.size();
  }
  std::vector<int> trow_deps(trow.begin(), trow.begin() + tptr[n]);
  std::vector<int> tsl(tslot.begin(), tslot.begin() + tptr[n]), us, dsl(n);
  for (int i = 0; i < n; i++) {
    for (int j = P.bi[i]; j < P.bdiag[i]; j++) us.push_back(j);
    dsl[i] = P.bdiag[i];
  }
  std::vector<int> of, ob, fpos, none;
  setup_mark("chains-transpose");
  GP_TRY(plan(pc->num, n, cptr, crow, true, s));
  GP_TRY(plan(pc->fwd, n, tptr, trow_deps, true, s, &of));
  GP_TRY(plan(pc->bwd, n, up, uc, false, s, &ob));
  setup_mark("levels");
  GP_TRY(ell_build(pc->ef, ELL_ICC_F, n, true, of, tptr, trow_deps, tsl, perm_c, none, dsl, &fpos,
                   pc->fwd.nlevels));
  setup_mark("fwd-layout");
  GP_TRY(ell_build(pc->eb, ELL_ICC_B, n, false, ob, up, uc, us, fpos, perm_c, none, nullptr,
                   pc->bwd.nlevels));
  setup_mark("bwd-layout");
  GP_TRY(upload(&pc->bi, P.bi, s));
  GP_TRY(upload(&pc->bj, P.bj, s));
  GP_TRY(upload(&pc->bdiag, P.bdiag, s));
  GP_TRY(upload(&pc->perm_r, P.r, s));
  GP_TRY(upload(&pc->perm_c, perm_c, s));
  GP_TRY(upload(&pc->perm_ic, P.ic, s));
  GP_TRY(upload(&pc->cptr, cptr, s));
  GP_TRY(upload(&pc->crow, crow, s));
  GP_TRY(upload(&pc->cslot, cslot, s));
  GP_TRY(upload(&pc->tptr, tptr, s));
  GP_TRY(upload(&pc->trow, trow, s));
  GP_TRY(upload(&pc->tslot, tslot, s));
  GP_TRY(dalloc(&pc->ba, std::max(P.nnz, 1)));
  GP_TRY(dalloc(&pc->ba_orig, std::max(P.nnz, 1)));
  GP_CUDA(cudaMalloc(&pc->done, std::max(n, 1) * sizeof(int)));
  GP_CUDA(cudaMemsetAsync(pc->done, 0, std::max(n, 1) * sizeof(int), s));
  pc->vlen = std::max({n, pc->ef.n, pc->eb.n});
  GP_TRY(dalloc(&pc->yf, pc->vlen));
  GP_TRY(dalloc(&pc->yb, pc->vlen));
  GP_TRY(dalloc(&pc->ys, pc->vlen));
  GP_CUDA(cudaStreamSynchronize(s));
  return GP_OK;
}

static int icc_amap(Pc* pc, const Csr* A, cudaStream_t s) {
  const int n = A->n;
  const FactorPattern& P = pc->pat;
  std::vector<int> amap(std::max<int64_t>(A->nnz, 1), -1);
  host_parallel_for(n, [&](int64_t k0, int64_t k1) {
    for (int k = (int)k0; k < (int)k1; k++) {
      const int rk = P.r[k];
      for (int j = A->h_rowptr[rk]; j < A->h_rowptr[rk + 1]; j++) {
        const int c = P.ic[A->h_colind[j]];
        if (c < k) continue;
        if (c == k) {
          amap[j] = P.bdiag[k];
          continue;
        }
        auto it = std::lower_bound(P.bj.begin() + P.bi[k], P.bj.begin() + P.bdiag[k], c);
        if (it != P.bj.begin() + P.bdiag[k] && *it == c) amap[j] = (int)(it - P.bj.begin());
      }
    }
  });
  if (pc->amap) cudaFree(pc->amap);
  pc->amap = nullptr;
  GP_TRY(upload(&pc->amap, amap, s));
  GP_CUDA(cudaStreamSynchronize(s));
  return GP_OK;
}

static int setup_icc(Pc* pc, cudaStream_t s) {
  const Csr* A = pc->A;
  std::vector<int> r, ic;
  GP_TRY(perms(pc, r, ic));
  setup_mark("ordering");
  GP_TRY(icc_symbolic(A, pc->opt.levels, r, ic, pc->pat));
  setup_mark("symbolic");
  GP_TRY(icc_prepare(pc, r, s));
  return icc_amap(pc, A, s);
}

// Numeric factorisation on the device for the current values of A.
int pc_factor_numeric(Pc* pc, cudaStream_t s) {
  const Csr* A = pc->A;
  const int n = A->n;
  if (n == 0) return GP_OK;
  pc->epoch = pc->epoch == INT32_MAX ? 1 : pc->epoch + 1;
  if (pc->opt.type == PC_ILU) {
    k_ilu_numeric<<<sweep_grid(), kSweepBlock, 0, s>>>(
        n, pc->fwd.order, pc->tickets, A->rowptr, A->val, pc->amap, pc->perm_r, pc->bi, pc->bj,
        pc->bdiag, pc->upd_ptr, pc->upd_dst, pc->upd_src, pc->ba, pc->done, pc->epoch, pc->err);
  } else {
    k_icc_numeric<<<sweep_grid(), kSweepBlock, 0, s>>>(
        n, pc->num.order, pc->tickets, A->rowptr, A->val, pc->amap, pc->perm_r, pc->bi, pc->bj,
        pc->bdiag, pc->cptr, pc->crow, pc->cslot, pc->ba, pc->ba_orig, pc->done, pc->epoch,
        pc->err);
  }
  GP_CHECK_LAUNCH();
  GP_TRY(ell_refresh(pc->ef, pc->ba, s));
  GP_TRY(ell_refresh(pc->eb, pc->ba, s));
  if (pc->trans_ready) {
    GP_TRY(ell_refresh(pc->etf, pc->ba, s));
    GP_TRY(ell_refresh(pc->etb, pc->ba, s));
  }
  return pc_check(pc, s);
}

int pc_update_values(Pc* pc, cudaStream_t s) {
  if (!pc->ready || !pc->A) {
    set_error("PC values updated before set-up");
    return GP_ERR_NOT_SETUP;
  }
  const Csr* A = pc->A;
  const int n = A->n;
  switch (pc->opt.type) {
    case PC_JACOBI:
      if (n) {
        const PcOptions& o = pc->opt;
        k_jacobi_fill<<<(n + 255) / 256, 256, 0, s>>>(n, o.jacobi_type, 0, o.use_abs,
                                                      o.fix_diag, o.rowl1_scale, A->rowptr,
                                                      A->val, A->diagpos, pc->diag);
        k_jacobi_fill<<<(n + 255) / 256, 256, 0, s>>>(n, o.jacobi_type, 1, 0, 0, 1.0,
                                                      A->rowptr, A->val, A->diagpos,
                                                      pc->diagsqrt);
        GP_CHECK_LAUNCH();
      }
      return GP_OK;
    case PC_ILU:
    case PC_ICC: return pc_factor_numeric(pc, s);
    case PC_SOR:
      // recomputed from the values by the next apply
      GP_CUDA(cudaMemsetAsync(pc->sor_stale, 1, sizeof(int), s));
      pc->sor_vver = A->vver;
      return GP_OK;
    default: return GP_OK;  // none
  }
}

int pc_values_sync(Pc* pc, cudaStream_t s) {
  if (pc->opt.type != PC_SOR || !pc->ready || !pc->A || !pc->sor_stale) return GP_OK;
  if (pc->A->vver != pc->sor_vver) {
    GP_CUDA(cudaMemsetAsync(pc->sor_stale, 1, sizeof(int), s));
    pc->sor_vver = pc->A->vver;
  }
  return GP_OK;
}

int pc_setup(Pc* pc, Csr* A, cudaStream_t s) {
  setup_report("(before)");
  free_all(pc);
  pc->generation = next_uid();
  pc->A = A;
  pc->n = A->n;
  GP_CUDA(cudaGetDevice(&pc->device));
  if (A->n != A->ncols) {
    set_error("the preconditioner matrix must be square");
    return GP_ERR_ARG;
  }
  const int n = A->n;
  GP_CUDA(cudaMalloc(&pc->err, sizeof(DevErr)));
  GP_CUDA(cudaMemsetAsync(pc->err, 0, sizeof(DevErr), s));
  GP_CUDA(cudaMalloc(&pc->tickets, 4 * sizeof(unsigned)));
  GP_CUDA(cudaMemsetAsync(pc->tickets, 0, 4 * sizeof(unsigned), s));
  switch (pc->opt.type) {
    case PC_NONE: break;
    case PC_JACOBI:
      GP_TRY(dalloc(&pc->diag, n));
      GP_TRY(dalloc(&pc->diagsqrt, n));
      if (n) {
        const PcOptions& o = pc->opt;
        k_jacobi_fill<<<(n + 255) / 256, 256, 0, s>>>(n, o.jacobi_type, 0, o.use_abs,
                                                      o.fix_diag, o.rowl1_scale, A->rowptr,
                                                      A->val, A->diagpos, pc->diag);
        k_jacobi_fill<<<(n + 255) / 256, 256, 0, s>>>(n, o.jacobi_type, 1, 0, 0, 1.0,
                                                      A->rowptr, A->val, A->diagpos,
                                                      pc->diagsqrt);
        GP_CHECK_LAUNCH();
      }
      break;
    case PC_SOR:
      GP_TRY(setup_sor(pc, s));
      GP_CUDA(cudaStreamSynchronize(s));
      setup_mark("rest");
      setup_report("sor");
      break;
    case PC_ILU:
      GP_TRY(setup_ilu(pc, s));
      setup_mark("amap");
      GP_TRY(pc_factor_numeric(pc, s));
      setup_mark("numeric");
      setup_report("ilu");
      break;
    case PC_ICC:
      GP_TRY(setup_icc(pc, s));
      setup_mark("amap");
      GP_TRY(pc_factor_numeric(pc, s));
      setup_mark("numeric");
      setup_report("icc");
      break;
    default: set_error("unsupported PC type"); return GP_ERR_UNSUPPORTED;
  }
  pc->ready = true;
  return GP_OK;
}


int pc_apply(Pc* pc, DRef x, DRef y, cudaStream_t s, const int* gate, int want) {
  if (!pc->ready) {
    set_error("PC used before set-up");
    return GP_ERR_NOT_SETUP;
  }
  const int n = pc->n;
  if (n == 0) return GP_OK;
  const int g = grid_for(n), sg = sweep_grid();
  unsigned* tk0 = pc->tickets;
  unsigned* tk1 = pc->tickets + 2;
  switch (pc->opt.type) {
    case PC_NONE:
      k_copy_g<<<g, 256, 0, s>>>(gate, want, n, x, y);
      break;
    case PC_JACOBI:
      k_pmult<<<g, 256, 0, s>>>(gate, want, n, x, pc->diag, y);
      break;
    case PC_SOR: {
      const Csr* A = pc->A;
      const int flag = pc->opt.sor_flag;
      const bool fw = flag & kSorForward, bw = flag & kSorBackward;
      // The reference runs MatInvertDiagonalForSOR_SeqAIJ on every apply, from
      // the current values (src/ported.mojo:610-633).  The inverted diagonal
      // and the sweeps' coefficients are functions of the values alone, so
      // they are recomputed only while the device word sor_stale is set: by
      // set-up, and before a launch when A's values changed since
      // (pc_values_sync; a captured solve calls it before every launch).
      if (!stream_capturing(s)) GP_TRY(pc_values_sync(pc, s));
      k_sor_diag<<<(n + 255) / 256, 256, 0, s>>>(n, pc->opt.omega, pc->opt.fshift, A->diagpos,
                                                  A->val, pc->idiag, pc->mdiag, gate, want,
                                                  pc->sor_stale);
      k_fill_pending<<<grid_for(pc->vlen), 256, 0, s>>>(gate, want, pc->vlen, pc->yf, pc->yb);
      if (pc->ef.ok && pc->eb.ok) {
        if (!pc->ef.tiled)
          k_ell_refresh_g<<<g, 256, 0, s>>>(gate, want, pc->ef.n, pc->ef.cnt, pc->ef.cslot,
                                            A->val, pc->ef.coef, pc->sor_stale);
        if (!pc->eb.tiled)
          k_ell_refresh_g<<<g, 256, 0, s>>>(gate, want, pc->eb.n, pc->eb.cnt, pc->eb.cslot,
                                            A->val, pc->eb.coef, pc->sor_stale);
        k_clear_word<<<1, 1, 0, s>>>(gate, want, pc->sor_stale);
        if (fw)
          GP_TRY(ell_sweep(ELL_SOR_F, pc->ef, gate, want, x, y, pc->yf, nullptr, pc->t, nullptr,
                           pc->idiag, pc->opt.omega, 0, bw ? 0 : 1, tk0, pc->err, A->val, s));
        if (bw)
          GP_TRY(ell_sweep(ELL_SOR_B, pc->eb, gate, want, x, y, pc->yb, pc->yf, nullptr, pc->t,
                           pc->idiag, pc->opt.omega, fw ? 1 : 0, 1, tk1, pc->err, A->val, s));
        break;
      }
      k_clear_word<<<1, 1, 0, s>>>(gate, want, pc->sor_stale);
      if (fw)
        k_sor_fwd<<<sg, kSweepBlock, 0, s>>>(gate, want, n, pc->fwd.order, tk0, A->rowptr,
                                             A->colind, A->val, A->diagpos, pc->idiag, x, pc->t,
                                             pc->yf, bw ? DRef::of((double*)nullptr) : y, pc->err);
      if (bw)
        k_sor_bwd<<<sg, kSweepBlock, 0, s>>>(gate, want, n, pc->bwd.order, tk1, A->rowptr,
                                             A->colind, A->val, A->diagpos, pc->idiag, x, pc->t,
                                             pc->yf, pc->yb, y, pc->opt.omega, fw ? 1 : 0,
                                             pc->err);
      break;
    }
    case PC_ILU:
      k_fill_pending<<<grid_for(pc->vlen), 256, 0, s>>>(gate, want, pc->vlen, pc->yf, pc->yb);
      if (pc->ef.ok && pc->eb.ok) {
        GP_TRY(ell_sweep(ELL_ILU_F, pc->ef, gate, want, x, y, pc->yf, nullptr, nullptr, nullptr,
                         nullptr, 0.0, 0, 0, tk0, pc->err, pc->ba, s));
        GP_TRY(ell_sweep(ELL_ILU_B, pc->eb, gate, want, x, y, pc->yb, pc->yf, nullptr, nullptr,
                         nullptr, 0.0, 0, 1, tk1, pc->err, pc->ba, s));
        break;
      }
      k_ilu_fwd<<<sg, kSweepBlock, 0, s>>>(gate, want, n, pc->fwd.order, tk0, pc->bi, pc->bj,
                                           pc->ba, pc->perm_r, x, pc->yf, pc->err);
      k_ilu_bwd<<<sg, kSweepBlock, 0, s>>>(gate, want, n, pc->bwd.order, tk1, pc->bj, pc->ba,
                                           pc->bdiag, pc->perm_c, pc->yf, pc->yb, y, pc->err);
      break;
    case PC_ICC:
      k_fill_pending<<<grid_for(pc->vlen), 256, 0, s>>>(gate, want, pc->vlen, pc->yf, pc->yb);
      if (pc->ef.ok && pc->eb.ok) {
        GP_TRY(ell_sweep(ELL_ICC_F, pc->ef, gate, want, x, y, pc->yf, nullptr, pc->ys, nullptr,
                         nullptr, 0.0, 0, 0, tk0, pc->err, pc->ba, s));
        GP_TRY(ell_sweep(ELL_ICC_B, pc->eb, gate, want, x, y, pc->yb, nullptr, nullptr, pc->ys,
                         nullptr, 0.0, 0, 1, tk1, pc->err, pc->ba, s));
        break;
      }
      k_icc_fwd<<<sg, kSweepBlock, 0, s>>>(gate, want, n, pc->fwd.order, tk0, pc->tptr,
                                           pc->trow, pc->tslot, pc->ba, pc->bdiag, pc->perm_c, x,
                                           pc->yf, pc->ys, pc->err);
      k_icc_bwd<<<sg, kSweepBlock, 0, s>>>(gate, want, n, pc->bwd.order, tk1, pc->bi, pc->bj,
                                           pc->ba, pc->bdiag, pc->perm_c, pc->ys, pc->yb, y,
                                           pc->err);
      break;
    default: set_error("unsupported PC type"); return GP_ERR_UNSUPPORTED;
  }
  GP_CHECK_LAUNCH();
  return GP_OK;
}

// The transposed ILU apply.  The forward apply is y = S_c U^-1 L^-1 G_r x
// (G_r gathers x[r[i]], S_c scatters y[c[i]]), so
//   M^-T x = G_r^T L^-T U^-T S_c^T x:
// gather t_i = x[c[i]]; solve U^T z = t (a forward sweep: row i of U^T holds
// U(k, i) for the rows k < i whose U part has column i, and U's diagonal is
// stored inverted); solve L^T w = z (a backward sweep over L(k, i), k > i,
// unit diagonal); scatter y[r[i]] = w_i.  Both sweeps are laid out once, in
// the level-ordered form, and gather their coefficients from the factor.
// There is no counterpart in the reference, whose applyTranspose is apply
// (python/mojopetsc4py/PETSc/PC.py:635-642).
int pc_transpose_prepare(Pc* pc, cudaStream_t s) {
  if (!pc->ready) {
    set_error("PC used before set-up");
    return GP_ERR_NOT_SETUP;
  }
  if (pc->opt.type == PC_SOR) {
    set_error("transposed apply: SOR on a nonsymmetric operator is not supported");
    return GP_ERR_UNSUPPORTED;
  }
  if (pc->opt.type != PC_ILU || pc->trans_ready || pc->n == 0) return GP_OK;
  const int n = pc->n;
  const FactorPattern& P = pc->pat;
  // U^T: per column i, the rows k < i holding it in their U part, ascending k
  std::vector<int> up(n + 1, 0), uc, us, dsl(n);
  {
    std::vector<std::vector<std::pair<int, int>>> cols(n);
    for (int k = 0; k < n; k++)
      for (int j = P.bdiag[k + 1] + 1; j < P.bdiag[k]; j++) cols[P.bj[j]].emplace_back(k, j);
    for (int i = 0; i < n; i++) {
      std::sort(cols[i].begin(), cols[i].end());
      for (auto& e : cols[i]) {
        uc.push_back(e.first);
        us.push_back(e.second);
      }
      up[i + 1] = (int)uc.size();
      dsl[i] = P.bdiag[i];
    }
  }
  // L^T: per column i, the rows k > i holding it in their L part, ascending k
  std::vector<int> lp(n + 1, 0), lc, ls;
  {
    std::vector<std::vector<std::pair<int, int>>> cols(n);
    for (int k = 0; k < n; k++)
      for (int j = P.bi[k]; j < P.bi[k + 1]; j++) cols[P.bj[j]].emplace_back(k, j);
    for (int i = 0; i < n; i++) {
      std::sort(cols[i].begin(), cols[i].end());
      for (auto& e : cols[i]) {
        lc.push_back(e.first);
        ls.push_back(e.second);
      }
      lp[i + 1] = (int)lc.size();
    }
  }
  std::vector<int> perm_c(n), of, ob, fpos, none;
  GP_CUDA(cudaMemcpy(perm_c.data(), pc->perm_c, n * sizeof(int), cudaMemcpyDeviceToHost));
  int nlev = 0;
  level_order(n, up, uc, true, of, &nlev);
  level_order(n, lp, lc, false, ob, &nlev);
  GP_TRY(ell_build_chunked(pc->etf, ELL_ILU_B, n, true, of, up, uc, us, perm_c, none, dsl, &fpos));
  GP_TRY(ell_build_chunked(pc->etb, ELL_ILU_F, n, false, ob, lp, lc, ls, fpos, P.r, none, nullptr));
  if (!pc->etf.ok || !pc->etb.ok) {
    ell_free(pc->etf);
    ell_free(pc->etb);
    set_error("transposed apply: a row of U^T or L^T has more than 16 entries");
    return GP_ERR_UNSUPPORTED;
  }
  GP_TRY(ell_refresh(pc->etf, pc->ba, s));
  GP_TRY(ell_refresh(pc->etb, pc->ba, s));
  pc->trans_ready = true;
  return GP_OK;
}

int pc_apply_transpose(Pc* pc, DRef x, DRef y, cudaStream_t s, const int* gate, int want) {
  if (!pc->ready) {
    set_error("PC used before set-up");
    return GP_ERR_NOT_SETUP;
  }
  if (pc->opt.type != PC_ILU) {
    if (pc->opt.type == PC_SOR) {
      set_error("transposed apply: SOR on a nonsymmetric operator is not supported");
      return GP_ERR_UNSUPPORTED;
    }
    return pc_apply(pc, x, y, s, gate, want);  // symmetric: none, Jacobi, IC
  }
  const int n = pc->n;
  if (n == 0) return GP_OK;
  if (!pc->trans_ready) {
    set_error("transposed apply used before pc_transpose_prepare");
    return GP_ERR_NOT_SETUP;
  }
  k_fill_pending<<<grid_for(n), 256, 0, s>>>(gate, want, n, pc->yf, pc->yb);
  // U^T z = x[c]: input gathered from x by the sweep's in_idx, no output
  GP_TRY(ell_sweep(ELL_ILU_B, pc->etf, gate, want, x, y, pc->yf, nullptr, nullptr, nullptr,
                   nullptr, 0.0, 0, 0, pc->tickets, pc->err, pc->ba, s));
  // L^T w = z: input from the first sweep's values, output scattered to y[r]
  GP_TRY(ell_sweep(ELL_ILU_F, pc->etb, gate, want, x, y, pc->yb, pc->yf, nullptr, nullptr,
                   nullptr, 0.0, 0, 1, pc->tickets + 2, pc->err, pc->ba, s));
  GP_CHECK_LAUNCH();
  return GP_OK;
}

int pc_apply_symmetric(Pc* pc, DRef x, DRef y, cudaStream_t s, const int* gate, int want) {
  if (pc->opt.type == PC_JACOBI) {
    const int n = pc->n;
    if (n == 0) return GP_OK;
    k_pmult<<<grid_for(n), 256, 0, s>>>(gate, want, n, x, pc->diagsqrt, y);
    GP_CHECK_LAUNCH();
    return GP_OK;
  }
  return pc_apply(pc, x, y, s, gate, want);
}

// A factor handed over in the reference's layout (the mp_* ABI): the pattern
// and optionally its values, with the plans for the device sweeps.  When A is
// given, the A-slot map for a numeric factorisation is built too.
int pc_import_factor(Pc* pc, int type, const FactorPattern& pat, const std::vector<int>& perm_c,
                     const double* ba_host, Csr* A, cudaStream_t s) {
  free_all(pc);
  pc->generation = next_uid();
  pc->opt.type = type;
  pc->n = (int)pat.bi.size() - 1;
  pc->A = A;
  pc->pat = pat;
  GP_CUDA(cudaGetDevice(&pc->device));
  GP_CUDA(cudaMalloc(&pc->err, sizeof(DevErr)));
  GP_CUDA(cudaMemsetAsync(pc->err, 0, sizeof(DevErr), s));
  GP_CUDA(cudaMalloc(&pc->tickets, 4 * sizeof(unsigned)));
  GP_CUDA(cudaMemsetAsync(pc->tickets, 0, 4 * sizeof(unsigned), s));
  if (type == PC_ILU) {
    GP_TRY(ilu_prepare(pc, perm_c, s));
    if (A) GP_TRY(ilu_amap(pc, A, s));
  } else if (type == PC_ICC) {
    GP_TRY(icc_prepare(pc, perm_c, s));
    if (A) GP_TRY(icc_amap(pc, A, s));
  } else {
    set_error("pc_import_factor: ILU or IC only");
    return GP_ERR_ARG;
  }
  if (ba_host && pat.nnz) {
    GP_CUDA(cudaMemcpyAsync(pc->ba, ba_host, (size_t)pat.nnz * sizeof(double),
                            cudaMemcpyHostToDevice, s));
    GP_TRY(ell_refresh(pc->ef, pc->ba, s));
    GP_TRY(ell_refresh(pc->eb, pc->ba, s));
  }
  GP_CUDA(cudaStreamSynchronize(s));
  pc->ready = true;
  return GP_OK;
}

// Jacobi with its diagonals given (the reference's pci block carries them).
int pc_import_jacobi(Pc* pc, int n, const double* diag, const double* diagsqrt, cudaStream_t s) {
  free_all(pc);
  pc->generation = next_uid();
  pc->opt.type = PC_JACOBI;
  pc->n = n;
  GP_CUDA(cudaGetDevice(&pc->device));
  GP_CUDA(cudaMalloc(&pc->err, sizeof(DevErr)));
  GP_CUDA(cudaMemsetAsync(pc->err, 0, sizeof(DevErr), s));
  GP_CUDA(cudaMalloc(&pc->tickets, 4 * sizeof(unsigned)));
  GP_CUDA(cudaMemsetAsync(pc->tickets, 0, 4 * sizeof(unsigned), s));
  GP_TRY(dalloc(&pc->diag, n));
  GP_TRY(dalloc(&pc->diagsqrt, n));
  if (n) {
    GP_CUDA(cudaMemcpyAsync(pc->diag, diag, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, s));
    if (diagsqrt)
      GP_CUDA(cudaMemcpyAsync(pc->diagsqrt, diagsqrt, (size_t)n * sizeof(double),
                              cudaMemcpyHostToDevice, s));
  }
  GP_CUDA(cudaStreamSynchronize(s));
  pc->ready = true;
  return GP_OK;
}

// Jacobi set-up kernels into caller device buffers (the mp_* set-up entries).
int jacobi_fill(const Csr* A, int jtype, int sym, int use_abs, int fix_diag, double scale,
                double* out, cudaStream_t s) {
  const int n = A->n;
  if (!n) return GP_OK;
  k_jacobi_fill<<<(n + 255) / 256, 256, 0, s>>>(n, jtype, sym, use_abs, fix_diag, scale,
                                                A->rowptr, A->val, A->diagpos, out);
  GP_CHECK_LAUNCH();
  return GP_OK;
}

// SOR diagonals for the current values (MatInvertDiagonalForSOR_SeqAIJ).
int sor_diagonals(Pc* pc, cudaStream_t s) {
  const int n = pc->n;
  if (!n) return GP_OK;
  k_sor_diag<<<(n + 255) / 256, 256, 0, s>>>(n, pc->opt.omega, pc->opt.fshift, pc->A->diagpos,
                                              pc->A->val, pc->idiag, pc->mdiag);
  GP_CHECK_LAUNCH();
  return GP_OK;
}

}  // namespace gp
