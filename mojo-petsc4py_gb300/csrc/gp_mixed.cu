// Mixed precision: FP32 inner FGMRES(m) with the ILU(0) factors in FP32, inside
// FP64 iterative refinement.
//
//   repeat:  r = b - A x (FP64 SpMV),  stop when ||r|| <= rtol ||b||
//            solve A d = r / ||r|| with one FGMRES(m) cycle in FP32
//            x += ||r|| d (FP64)
//
// FP64 is kept for the outer residual, the convergence norms and GMRES's
// Hessenberg / Givens least-squares (host side, per cycle); everything else --
// matrix values, Krylov and preconditioned vectors, dot-product accumulation
// inside a CTA -- is FP32 (cross-CTA sums in FP64).
//
// The preconditioner is the ILU(0) factor of the plain path (same symbolic and
// numeric phase, values rounded to FP32).  Its triangular solves are applied
// with `tri_sweeps` Jacobi iterations per triangle (y <- Pb - L_strict y;
// x <- D^-1 (y - U_strict x)) instead of level-scheduled substitution: each
// iteration is one fully parallel, bandwidth-bound pass, where the exact
// substitution is a chain of dependency levels (hundreds on a 3-D grid) whose
// cost is latency.  FGMRES tolerates the inexact, fixed-count application
// (its basis stores the preconditioned vectors), and the FP64 refinement
// makes the result independent of it.  tri_sweeps = 0 applies the factors
// exactly with the level-scheduled FP64 sweeps instead.
#include <algorithm>
#include <cstddef>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <map>
#include <vector>

#include "../../include/gpetsc.h"
#include "gp_ksp.h"
#include "gp_handles.h"
#include "gp_spmv.cuh"

namespace gp {

constexpr int kMixBlock = 256;
constexpr int kMixMaxM = 64;

// ------------------------------------------------------------------ kernels
// CTAs of the multi-dot kernels: four per SM (more loads in flight; the last
// CTA's fold stays short)
static int mdot_grid(int64_t n) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)num_sms() * 4));
}

static int mix_grid(int64_t n) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + kMixBlock - 1) / kMixBlock,
                                                     (int64_t)num_sms() * 8));
}

// y = A x in FP32 (row per thread, matrix streamed with L2 evict-first).  CT:
// int (column indices) or short (16-bit offsets from the row, Csr::coff16).
template <typename CT>
__global__ void __launch_bounds__(kMixBlock) k_spmv32(int n, const int* __restrict__ rp,
                                                      const CT* __restrict__ ci,
                                                      const float* __restrict__ val,
                                                      const float* __restrict__ x,
                                                      float* __restrict__ y) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= n) return;
  const uint64_t pol = l2_evict_first();
  const int b = rp[row], e = rp[row + 1];
  float acc = 0.f;
  for (int j0 = b; j0 < e; j0 += 8) {
    int cc[8];
    float vv[8];
#pragma unroll
    for (int u = 0; u < 8; u++)
      if (j0 + u < e) {
        cc[u] = spmv_col(ci, j0 + u, row, pol);
        vv[u] = ld_stream(val + j0 + u, pol);
      }
#pragma unroll
    for (int u = 0; u < 8; u++)
      if (j0 + u < e) acc = __fmaf_rn(vv[u], x[cc[u]], acc);
  }
  y[row] = acc;
}

// One Jacobi pass of a triangular solve with a strict triangle T (CSR):
//   out_i = s_i (rhs_i - sum_j T_ij in_j),  s = dinv (or 1 when dinv is null)
__global__ void __launch_bounds__(kMixBlock) k_tri_pass(int n, const int* __restrict__ rp,
                                                        const int* __restrict__ ci,
                                                        const float* __restrict__ val,
                                                        const float* __restrict__ dinv,
                                                        const float* __restrict__ rhs,
                                                        const float* __restrict__ in,
                                                        float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float acc = rhs[i];
  for (int j = rp[i]; j < rp[i + 1]; j++) acc = __fmaf_rn(-val[j], in[ci[j]], acc);
  out[i] = dinv ? acc * dinv[i] : acc;
}

__global__ void k_gather32(int n, const int* __restrict__ idx, const float* __restrict__ in,
                           float* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = in[idx[i]];
}

__global__ void k_scatter32(int n, const int* __restrict__ idx, const float* __restrict__ in,
                            float* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[idx[i]] = in[i];
}

__global__ void k_mul32(int n, const float* __restrict__ a, const float* __restrict__ b,
                        float* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = a[i] * b[i];
}

// values of a factor triangle, FP64 factor slots -> FP32 CSR
// ELL coefficients from the factor values (slot -1: absent, zero)
__global__ void k_ell32_refresh(int64_t m, const int* __restrict__ slot,
                                const double* __restrict__ src, float* __restrict__ dst) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < m;
       k += (int64_t)gridDim.x * blockDim.x)
    dst[k] = slot[k] >= 0 ? __double2float_rn(src[slot[k]]) : 0.f;
}

__global__ void k_slot_gather(int64_t m, const int* __restrict__ slot,
                              const double* __restrict__ ba, float* __restrict__ out) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < m;
       k += (int64_t)gridDim.x * blockDim.x)
    out[k] = __double2float_rn(ba[slot[k]]);
}

// out[j] = sum over the grid's per-CTA partials of value j (j < kk), in the
// last CTA: warp w folds values w, w + nwarps, ...; its lanes take CTAs
// lane, lane + 32, ... (many loads in flight) and a shuffle tree combines them.
__device__ __forceinline__ void fold_partials(const double* partials, int kk, double* out) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int j = wid; j < kk; j += nw) {
    double t = 0.0;
    for (int bb = lane; bb < (int)gridDim.x; bb += 32)
      t += __ldcg(&partials[(size_t)j * gridDim.x + bb]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (lane == 0) out[j] = t;
  }
}

// Dots of w against basis rows 0..k-1 (rows of V, leading dimension n), or
// ||w||^2 when V is null: FP32 per thread and per CTA, per-CTA partials in
// FP64; the last CTA folds them (FP64) into out[0..k-1].
__global__ void __launch_bounds__(kMixBlock) k_mdot32(int n, const float* __restrict__ V,
                                                      int k, const float* __restrict__ w,
                                                      double* __restrict__ partials,
                                                      unsigned* ticket, double* out) {
  __shared__ float sh[kMixBlock / 32][kMixMaxM + 1];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int kk = V ? k : 1;
  for (int j0 = 0; j0 < kk; j0 += 8) {
    float acc[8];
#pragma unroll
    for (int q = 0; q < 8; q++) acc[q] = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
      const float wi = w[i];
#pragma unroll
      for (int q = 0; q < 8; q++)
        if (j0 + q < kk) acc[q] = __fmaf_rn(V ? V[(size_t)(j0 + q) * n + i] : wi, wi, acc[q]);
    }
#pragma unroll
    for (int q = 0; q < 8; q++) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc[q] += __shfl_down_sync(0xffffffffu, acc[q], o);
      if (lane == 0 && j0 + q < kk) sh[wid][j0 + q] = acc[q];
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int j = 0; j < kk; j++) {
      float t = 0.f;
      for (int ww = 0; ww < (int)(blockDim.x >> 5); ww++) t += sh[ww][j];
      partials[(size_t)j * gridDim.x + blockIdx.x] = (double)t;
    }
    last = atomic_add_acq_rel(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  fold_partials(partials, kk, out);
  __syncthreads();
  if (threadIdx.x == 0) *ticket = 0u;
}

// w -= sum_{j<k} h_j V_j   (h in FP64 on the device, applied in FP32)
__global__ void k_maxpy32(int n, const float* __restrict__ V, int k, const double* __restrict__ h,
                          float* __restrict__ w) {
  __shared__ float hs[kMixMaxM + 1];
  for (int j = threadIdx.x; j < k; j += blockDim.x) hs[j] = (float)h[j];
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float v = w[i];
    for (int j = 0; j < k; j++) v = __fmaf_rn(-hs[j], V[(size_t)j * n + i], v);
    w[i] = v;
  }
}

// out = sum_{j<k} c_j Z_j   (c in FP64 on the device)
__global__ void k_lincomb32(int n, const float* __restrict__ Z, int k, const double* __restrict__ c,
                            float* __restrict__ out) {
  __shared__ float cs[kMixMaxM + 1];
  for (int j = threadIdx.x; j < k; j += blockDim.x) cs[j] = (float)c[j];
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float v = 0.f;
    for (int j = 0; j < k; j++) v = __fmaf_rn(cs[j], Z[(size_t)j * n + i], v);
    out[i] = v;
  }
}

__global__ void k_scale32(int n, const float* in, float s, float* out) {  // in may be out
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = in[i] * s;
}

// r = b - y (FP64) and r32 = r * inv (FP32)
__global__ void k_resid_parts(int n, const double* __restrict__ b, const double* __restrict__ y,
                              double* __restrict__ r) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    r[i] = b[i] - y[i];
}

__global__ void k_to32_scaled(int n, const double* __restrict__ r, double inv,
                              float* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = __double2float_rn(r[i] * inv);
}

// x += a d  (FP64 accumulate of the FP32 correction)
__global__ void k_axpy64_32(int n, double a, const float* __restrict__ d, double* __restrict__ x) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    x[i] = fma(a, (double)d[i], x[i]);
}

// ------------------------------------------------ block triangle passes
//
// The inner preconditioner's triangles, applied by runs ("blocks") of
// consecutive factor rows: within a block every row is solved exactly, in the
// block's own dependency-level order with the values in shared memory; the
// couplings to rows of other blocks are taken from the previous pass (none on
// the first pass, which makes it block-Jacobi).  Blocks are independent, so a
// pass is one launch with no waits, and on a grid numbered in natural order
// most couplings lie inside a block: the pass is far closer to the exact
// triangular solve than a point-Jacobi pass, at about the same cost.  FP32,
// like the rest of the inner cycle.
constexpr int kBtBlock = 256;

struct BtArgs {
  int n, W;
  const int* cstart;   // [blocks + 1] first position of each block
  const int* lvl_ptr;  // [blocks + 1] into lvl_off
  const int* lvl_off;  // per block: level offsets, local positions
  const int* row;      // [n] factor row at each position (output index)
  const int* ridx;     // [n] right-hand-side index of each position
  const int* cnt;      // [n] dependencies of the row
  const int* code;     // [W * n] local position (>= 0) or -(column + 1)
  const float* cf;     // [W * n] coefficients
  const float* dinv;   // [n] inverted diagonal (upper triangle), or null
};

// Staging runs in two phases so that every load of a phase is independent of
// the others (many in flight): first the block's columns (coalesced), then the
// gathers of right-hand sides and of the previous pass's values.
template <bool UPPER, int WMAX>
__global__ void __launch_bounds__(kBtBlock) k_mx_btri(const int* gate, BtArgs t,
                                                      const float* __restrict__ rhs,
                                                      const float* __restrict__ prev,
                                                      float* __restrict__ out,
                                                      const int* __restrict__ out_perm) {
  if (gated_off(gate, 1)) return;
  extern __shared__ __align__(16) unsigned char sm[];
  const int c = blockIdx.x;
  const int p0 = t.cstart[c], Cc = t.cstart[c + 1] - p0;
  const int lb = t.lvl_ptr[c], nl = t.lvl_ptr[c + 1] - lb - 1;
  const int n = t.n, W = t.W;
  float* s_sum = reinterpret_cast<float*>(sm);
  float* s_val = s_sum + Cc;                 // Cc + 1: slot Cc holds 0 (absent terms)
  float* s_dv = s_val + Cc + 1;
  int* s_row = reinterpret_cast<int*>(s_dv + Cc);
  int* s_cnt = s_row + Cc;
  int* s_lo = s_cnt + Cc;                    // nl + 1
  int* s_dep = s_lo + nl + 1;                // [W][Cc]
  float* s_cf = reinterpret_cast<float*>(s_dep + (size_t)W * Cc);  // [W][Cc]
  for (int l = threadIdx.x; l <= nl; l += blockDim.x) s_lo[l] = t.lvl_off[lb + l];
  // phase 1: the block's columns
#pragma unroll 4
  for (int r = threadIdx.x; r < Cc; r += blockDim.x) {
    const int p = p0 + r;
    const int row = t.row[p];
    s_row[r] = out_perm ? out_perm[row] : row;  // where the row's value goes
    s_cnt[r] = t.cnt[p];
    if (UPPER) s_dv[r] = t.dinv[p];
    const int cn = t.cnt[p];
#pragma unroll
    for (int e = 0; e < WMAX; e++) {
      if (e < W) {
        // every row gets W terms: absent and external ones read the zero slot
        const int cd = e < cn ? t.code[(size_t)e * n + p] : -1;
        s_dep[(size_t)e * Cc + r] = cd >= 0 ? cd : Cc;
        s_cf[(size_t)e * Cc + r] = cd >= 0 ? t.cf[(size_t)e * n + p] : 0.f;
      }
    }
  }
  if (threadIdx.x == 0) s_val[Cc] = 0.f;
  // phase 2: right-hand sides and couplings from the previous pass
#pragma unroll 4
  for (int r = threadIdx.x; r < Cc; r += blockDim.x) {
    const int p = p0 + r;
    const int cn = t.cnt[p];
    float sum = rhs[t.ridx[p]];
    if (prev) {
      float pv[WMAX];
#pragma unroll
      for (int e = 0; e < WMAX; e++) {
        const int cd = (e < cn) ? t.code[(size_t)e * n + p] : 0;
        pv[e] = cd < 0 ? prev[-cd - 1] : 0.f;
      }
#pragma unroll
      for (int e = 0; e < WMAX; e++) {
        const int cd = (e < cn) ? t.code[(size_t)e * n + p] : 0;
        if (cd < 0) sum = __fmaf_rn(-t.cf[(size_t)e * n + p], pv[e], sum);
      }
    }
    s_sum[r] = sum;
  }
  __syncthreads();
  if (threadIdx.x >= 32) return;
  const int lane = threadIdx.x;
  for (int l = 0; l < nl; l++) {
    const int r1 = s_lo[l + 1];
    for (int r = s_lo[l] + lane; r < r1; r += 32) {
      float v = s_sum[r];
      // branch-free: W terms a row (a divergent branch per term costs more
      // than the padded multiply-adds)
#pragma unroll
      for (int e = 0; e < WMAX; e++)
        if (e < W) v = __fmaf_rn(-s_cf[(size_t)e * Cc + r], s_val[s_dep[(size_t)e * Cc + r]], v);
      if (UPPER) v *= s_dv[r];
      s_val[r] = v;
      out[s_row[r]] = v;
    }
    __syncwarp();
  }
}

template <bool UPPER>
static void launch_btri(const BtArgs& t, int nblocks, size_t smem, const int* gate,
                        const float* rhs, const float* prev, float* out, const int* out_perm,
                        cudaStream_t s) {
  if (t.W <= 4)
    k_mx_btri<UPPER, 4><<<nblocks, kBtBlock, smem, s>>>(gate, t, rhs, prev, out, out_perm);
  else if (t.W <= 8)
    k_mx_btri<UPPER, 8><<<nblocks, kBtBlock, smem, s>>>(gate, t, rhs, prev, out, out_perm);
  else
    k_mx_btri<UPPER, 32><<<nblocks, kBtBlock, smem, s>>>(gate, t, rhs, prev, out, out_perm);
}

template <bool UPPER>
static cudaError_t btri_attr(int smem) {
  cudaError_t e = cudaFuncSetAttribute(k_mx_btri<UPPER, 4>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_mx_btri<UPPER, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_mx_btri<UPPER, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem);
  return e;
}

// coefficient refresh of a block layout from the factor values (FP64 -> FP32)
__global__ void k_bt_refresh(int n, int W, const int* __restrict__ cnt,
                             const int* __restrict__ slot, const double* __restrict__ src,
                             float* __restrict__ cf, const int* __restrict__ dslot,
                             float* __restrict__ dinv) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    const int c = cnt[p];
    for (int e = 0; e < c; e++) cf[(size_t)e * n + p] = __double2float_rn(src[slot[(size_t)e * n + p]]);
    if (dslot) dinv[p] = __double2float_rn(src[dslot[p]]);
  }
}

// ---------------------------------------------------------------- host side
struct MixedOptions {
  int restart = 30;
  int max_outer = 200;      // FGMRES cycles (one per refinement pass)
  int tri_sweeps = 4;       // passes per triangle; 0 = exact FP64 sweeps
  int tri_block = 0;        // block passes with this many rows (-1: chosen), 0: point Jacobi
  double rtol = 1e-10;      // on the true FP64 residual, relative to ||b||
  double inner_rtol = 1e-4; // per cycle, relative to the cycle's start
};

struct MixedResult {
  int passes = 0, inner_its = 0, converged = 0;
  double relres = 0.0;
};

// Device block layout of one factor triangle for k_mx_btri (see there).
struct BlockTri {
  int nblocks = 0, W = 0, rows = 0;
  size_t smem = 0;
  int *cstart = nullptr, *lvl_ptr = nullptr, *lvl_off = nullptr, *row = nullptr;
  int *cnt = nullptr, *code = nullptr, *slot = nullptr, *dslot = nullptr, *ridx = nullptr;
  float *cf = nullptr, *dinv = nullptr;
};

static void bt_free(BlockTri& b) {
  void* ptrs[] = {b.cstart, b.lvl_ptr, b.lvl_off, b.row, b.cnt, b.code, b.slot, b.dslot, b.cf,
                  b.dinv, b.ridx};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  b = BlockTri();
}

struct Mixed {
  int n = 0, m = 0, device = -1;
  BlockTri bl, bu;       // block layouts of L and U (tri_block != 0)
  int bt_rows = 0;       // their block length (0: not built)
  unsigned long long bt_generation = 0;
  int bt_epoch = -1;
  bool ident_r = false, ident_c = false;  // factor row / solution permutations are identities
  const Csr* A = nullptr;
  const Pc* pc = nullptr;
  unsigned long long pc_generation = 0;
  int pc_epoch = -1;
  // FP32 factor triangles (CSR) and permutations
  int *lrp = nullptr, *lci = nullptr, *lslot = nullptr;
  int *urp = nullptr, *uci = nullptr, *uslot = nullptr, *dslot = nullptr;
  float *lval = nullptr, *uval = nullptr, *udinv = nullptr;
  int64_t lnnz = 0, unnz = 0;
  // column-major ELL copies of the triangles (W slots a row; 0 when wider than 8)
  int lW = 0, uW = 0;
  int *lell_ci = nullptr, *lell_slot = nullptr, *uell_ci = nullptr, *uell_slot = nullptr;
  float *lell_val = nullptr, *uell_val = nullptr;
  // work
  float *V = nullptr, *Z = nullptr, *w = nullptr, *t0 = nullptr, *t1 = nullptr, *t2 = nullptr;
  float *t3 = nullptr, *t4 = nullptr;
  double *r = nullptr, *y = nullptr, *d64 = nullptr, *h_dev = nullptr, *partials = nullptr;
  double* x64tmp = nullptr;
  unsigned* ticket = nullptr;
  double* h_pinned = nullptr;
  // the captured refinement pass
  struct MixDev* st = nullptr;       // device state
  struct MixDev* h_st = nullptr;     // pinned host copy of its head
  double* part64 = nullptr;
  unsigned* ticket64 = nullptr;
  cudaStream_t cap_stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  const void* cap_key[6] = {};
  int cap_ikey[5] = {};
  unsigned long long cap_A_uid = 0, cap_pc_gen = 0;
};

static void mixed_free(Mixed* M) {
  bt_free(M->bl);
  bt_free(M->bu);
  void* ptrs[] = {M->lrp, M->lci, M->lslot, M->urp, M->uci, M->uslot, M->dslot, M->lval,
                  M->uval, M->udinv, M->lell_ci, M->lell_slot, M->uell_ci, M->uell_slot,
                  M->lell_val, M->uell_val, M->V, M->Z, M->w, M->t0, M->t1, M->t2, M->t3, M->t4,
                  M->r, M->y,
                  M->d64, M->h_dev, M->partials, M->x64tmp, M->ticket};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (M->h_pinned) cudaFreeHost(M->h_pinned);
  if (M->st) cudaFree(M->st);
  if (M->h_st) cudaFreeHost(M->h_st);
  if (M->part64) cudaFree(M->part64);
  if (M->ticket64) cudaFree(M->ticket64);
  if (M->exec) cudaGraphExecDestroy(M->exec);
  if (M->graph) cudaGraphDestroy(M->graph);
  if (M->cap_stream) cudaStreamDestroy(M->cap_stream);
  *M = Mixed();
}

template <typename V>
static int up_mixed(V** d, const std::vector<V>& h) {
  GP_CUDA(cudaMalloc(d, std::max<size_t>(h.size(), 1) * sizeof(V)));
  if (!h.empty()) GP_CUDA(cudaMemcpy(*d, h.data(), h.size() * sizeof(V), cudaMemcpyHostToDevice));
  return GP_OK;
}

// (Re)build the FP32 factor triangles from the PC's factor.
static int mixed_factors(Mixed* M, cudaStream_t s) {
  const Pc* pc = M->pc;
  const FactorPattern& P = pc->pat;
  const int n = M->n;
  if (M->pc_generation != pc->generation) {
    for (void** p : {(void**)&M->lrp, (void**)&M->lci, (void**)&M->lslot, (void**)&M->urp,
                     (void**)&M->uci, (void**)&M->uslot, (void**)&M->dslot, (void**)&M->lval,
                     (void**)&M->uval, (void**)&M->udinv, (void**)&M->lell_ci,
                     (void**)&M->lell_slot, (void**)&M->uell_ci, (void**)&M->uell_slot,
                     (void**)&M->lell_val, (void**)&M->uell_val})
      if (*p) {
        cudaFree(*p);
        *p = nullptr;
      }
    std::vector<int> lrp(n + 1, 0), lci, lsl, urp(n + 1, 0), uci, usl, dsl(n);
    for (int i = 0; i < n; i++) {
      for (int j = P.bi[i]; j < P.bi[i + 1]; j++) {
        lci.push_back(P.bj[j]);
        lsl.push_back(j);
      }
      lrp[i + 1] = (int)lci.size();
      for (int j = P.bdiag[i + 1] + 1; j < P.bdiag[i]; j++) {
        uci.push_back(P.bj[j]);
        usl.push_back(j);
      }
      urp[i + 1] = (int)uci.size();
      dsl[i] = P.bdiag[i];
    }
    M->lnnz = (int64_t)lci.size();
    M->unnz = (int64_t)uci.size();
    GP_TRY(up_mixed(&M->lrp, lrp));
    GP_TRY(up_mixed(&M->lci, lci));
    GP_TRY(up_mixed(&M->lslot, lsl));
    GP_TRY(up_mixed(&M->urp, urp));
    GP_TRY(up_mixed(&M->uci, uci));
    GP_TRY(up_mixed(&M->uslot, usl));
    GP_TRY(up_mixed(&M->dslot, dsl));
    GP_CUDA(cudaMalloc(&M->lval, std::max<int64_t>(M->lnnz, 1) * sizeof(float)));
    GP_CUDA(cudaMalloc(&M->uval, std::max<int64_t>(M->unnz, 1) * sizeof(float)));
    GP_CUDA(cudaMalloc(&M->udinv, std::max(n, 1) * sizeof(float)));
    // ELL copies
    auto ell = [&](const std::vector<int>& rp, const std::vector<int>& ci,
                   const std::vector<int>& sl, int& W, int** eci, int** esl,
                   float** eval) -> int {
      W = 0;
      for (int i = 0; i < n; i++) W = std::max(W, rp[i + 1] - rp[i]);
      if (W > 8 || W == 0) {
        W = 0;
        return GP_OK;
      }
      std::vector<int> c((size_t)W * n), t((size_t)W * n, -1);
      for (int i = 0; i < n; i++)
        for (int e = 0; e < W; e++) {
          const int j = rp[i] + e;
          c[(size_t)e * n + i] = j < rp[i + 1] ? ci[j] : i;
          if (j < rp[i + 1]) t[(size_t)e * n + i] = sl[j];
        }
      GP_TRY(up_mixed(eci, c));
      GP_TRY(up_mixed(esl, t));
      GP_CUDA(cudaMalloc(eval, (size_t)W * n * sizeof(float)));
      return GP_OK;
    };
    GP_TRY(ell(lrp, lci, lsl, M->lW, &M->lell_ci, &M->lell_slot, &M->lell_val));
    GP_TRY(ell(urp, uci, usl, M->uW, &M->uell_ci, &M->uell_slot, &M->uell_val));
    // identity permutations (natural ordering) are skipped by the passes
    std::vector<int> pr(n), pcv(n);
    if (n) {
      GP_CUDA(cudaMemcpy(pr.data(), pc->perm_r, n * sizeof(int), cudaMemcpyDeviceToHost));
      GP_CUDA(cudaMemcpy(pcv.data(), pc->perm_c, n * sizeof(int), cudaMemcpyDeviceToHost));
    }
    M->ident_r = M->ident_c = true;
    for (int i = 0; i < n; i++) {
      M->ident_r = M->ident_r && pr[i] == i;
      M->ident_c = M->ident_c && pcv[i] == i;
    }
    M->pc_generation = pc->generation;
    M->pc_epoch = -1;
  }
  if (M->pc_epoch != pc->epoch) {
    const int g = num_sms() * 8;
    if (M->lnnz) k_slot_gather<<<g, 256, 0, s>>>(M->lnnz, M->lslot, pc->ba, M->lval);
    if (M->unnz) k_slot_gather<<<g, 256, 0, s>>>(M->unnz, M->uslot, pc->ba, M->uval);
    k_slot_gather<<<g, 256, 0, s>>>(n, M->dslot, pc->ba, M->udinv);
    if (M->lW)
      k_ell32_refresh<<<g, 256, 0, s>>>((int64_t)M->lW * n, M->lell_slot, pc->ba, M->lell_val);
    if (M->uW)
      k_ell32_refresh<<<g, 256, 0, s>>>((int64_t)M->uW * n, M->uell_slot, pc->ba, M->uell_val);
    GP_CHECK_LAUNCH();
    M->pc_epoch = pc->epoch;
  }
  return GP_OK;
}

// Block layout of one triangle.  rp/ci/sl: each factor row's dependencies and
// their slots in the factor values; forward: dependencies precede the row
// (L), else they follow it (U, blocks taken from the last row down).
static int bt_build(BlockTri& b, int n, bool forward, const std::vector<int>& rp,
                    const std::vector<int>& ci, const std::vector<int>& sl,
                    const std::vector<int>* dsl, const std::vector<int>* rhs_perm, int rows) {
  bt_free(b);
  int W = 0;
  for (int i = 0; i < n; i++) W = std::max(W, rp[i + 1] - rp[i]);
  const int nb = (n + rows - 1) / rows;
  std::vector<int> cstart(nb + 1), lvl_ptr(nb + 1), lvl_off, order(n), lpos(n);
  std::vector<int> lev(rows), cntl;
  int maxl = 0;
  auto row_of = [&](int q) { return forward ? q : n - 1 - q; };
  for (int c = 0; c < nb; c++) {
    const int q0 = c * rows, q1 = std::min(n, q0 + rows);
    int ml = 0;
    for (int q = q0; q < q1; q++) {
      const int i = row_of(q);
      int l = 0;
      for (int e = rp[i]; e < rp[i + 1]; e++) {
        const int qj = forward ? ci[e] : n - 1 - ci[e];
        if (qj >= q0) l = std::max(l, lev[qj - q0] + 1);
      }
      lev[q - q0] = l;
      ml = std::max(ml, l);
    }
    maxl = std::max(maxl, ml + 1);
    cntl.assign(ml + 2, 0);
    for (int q = q0; q < q1; q++) cntl[lev[q - q0] + 1]++;
    for (int l = 0; l <= ml; l++) cntl[l + 1] += cntl[l];
    lvl_ptr[c] = (int)lvl_off.size();
    for (int l = 0; l <= ml + 1; l++) lvl_off.push_back(cntl[l]);
    for (int q = q0; q < q1; q++) {
      const int r = cntl[lev[q - q0]]++;
      order[q0 + r] = row_of(q);
      lpos[row_of(q)] = r;
    }
    cstart[c] = q0;
  }
  cstart[nb] = n;
  lvl_ptr[nb] = (int)lvl_off.size();
  const int Wc = std::max(W, 1);
  std::vector<int> cnt(n), code((size_t)Wc * n, 0), slot((size_t)Wc * n, 0), ds;
  for (int c = 0; c < nb; c++) {
    const int q0 = c * rows, q1 = std::min(n, q0 + rows);
    for (int p = q0; p < q1; p++) {
      const int i = order[p];
      cnt[p] = rp[i + 1] - rp[i];
      for (int e = 0; e < cnt[p]; e++) {
        const int j = ci[rp[i] + e];
        const int qj = forward ? j : n - 1 - j;
        code[(size_t)e * n + p] = qj >= q0 ? lpos[j] : -(j + 1);
        slot[(size_t)e * n + p] = sl[rp[i] + e];
      }
    }
  }
  if (dsl) {
    ds.resize(n);
    for (int p = 0; p < n; p++) ds[p] = (*dsl)[order[p]];
  }
  std::vector<int> ridx(n);
  for (int p = 0; p < n; p++) ridx[p] = rhs_perm ? (*rhs_perm)[order[p]] : order[p];
  b.nblocks = nb;
  b.W = Wc;
  b.rows = rows;
  b.smem = 4 * ((size_t)5 * rows + 1 + (size_t)maxl + 1 + (size_t)2 * Wc * rows);
  GP_TRY(up_mixed(&b.ridx, ridx));
  GP_TRY(up_mixed(&b.cstart, cstart));
  GP_TRY(up_mixed(&b.lvl_ptr, lvl_ptr));
  GP_TRY(up_mixed(&b.lvl_off, lvl_off));
  GP_TRY(up_mixed(&b.row, order));
  GP_TRY(up_mixed(&b.cnt, cnt));
  GP_TRY(up_mixed(&b.code, code));
  GP_TRY(up_mixed(&b.slot, slot));
  GP_CUDA(cudaMalloc(&b.cf, (size_t)Wc * std::max(n, 1) * sizeof(float)));
  if (dsl) {
    GP_TRY(up_mixed(&b.dslot, ds));
    GP_CUDA(cudaMalloc(&b.dinv, std::max(n, 1) * sizeof(float)));
  }
  return GP_OK;
}

// Block length for the block passes: a multiple of the most frequent
// dependency distance of L (a grid's line length) near 1536 rows, within the
// shared-memory limit; `want` > 0 forces it.
static int bt_rows_for(const FactorPattern& P, int n, int want) {
  if (want > 0) return std::min(want, std::max(n, 1));
  std::map<int, long long> hist;
  const int scan = std::min(n, 1 << 18);
  for (int i = 0; i < scan; i++)
    for (int j = P.bi[i]; j < P.bi[i + 1]; j++) {
      const int d = i - P.bj[j];
      if (d >= 8) hist[d]++;
    }
  int d = 0;
  long long best = 0;
  for (auto& kv : hist)
    if (kv.second > best) {
      best = kv.second;
      d = kv.first;
    }
  int rows = d > 0 ? d * std::max(1, (int)std::lround(1536.0 / d)) : 1536;
  return std::max(1, std::min(rows, std::min(n, 4096)));
}

// (Re)build the block layouts when the factor pattern or block length
// changed; refresh their coefficients when the factor values changed.
static int mixed_blocks(Mixed* M, int want, cudaStream_t s) {
  const Pc* pc = M->pc;
  const FactorPattern& P = pc->pat;
  const int n = M->n;
  const int rows = bt_rows_for(P, n, want);
  if (M->bt_rows != rows || M->bt_generation != pc->generation || !M->bl.cstart) {
    std::vector<int> lrp(n + 1, 0), lci, lsl, urp(n + 1, 0), uci, usl, dsl(n);
    for (int i = 0; i < n; i++) {
      for (int j = P.bi[i]; j < P.bi[i + 1]; j++) {
        lci.push_back(P.bj[j]);
        lsl.push_back(j);
      }
      lrp[i + 1] = (int)lci.size();
      for (int j = P.bdiag[i + 1] + 1; j < P.bdiag[i]; j++) {
        uci.push_back(P.bj[j]);
        usl.push_back(j);
      }
      urp[i + 1] = (int)uci.size();
      dsl[i] = P.bdiag[i];
    }
    GP_TRY(bt_build(M->bl, n, true, lrp, lci, lsl, nullptr, &P.r, rows));
    GP_TRY(bt_build(M->bu, n, false, urp, uci, usl, &dsl, nullptr, rows));
    const size_t mx = std::max(M->bl.smem, M->bu.smem);
    if (mx > 227 * 1024) {
      set_error("mixed solve: the block length does not fit in shared memory");
      return GP_ERR_ARG;
    }
    GP_CUDA(btri_attr<false>((int)mx));
    GP_CUDA(btri_attr<true>((int)mx));
    M->bt_rows = rows;
    M->bt_generation = pc->generation;
    M->bt_epoch = -1;
  }
  if (M->bt_epoch != pc->epoch) {
    const int g = num_sms() * 8;
    k_bt_refresh<<<g, 256, 0, s>>>(n, M->bl.W, M->bl.cnt, M->bl.slot, pc->ba, M->bl.cf, nullptr,
                                   nullptr);
    k_bt_refresh<<<g, 256, 0, s>>>(n, M->bu.W, M->bu.cnt, M->bu.slot, pc->ba, M->bu.cf,
                                   M->bu.dslot, M->bu.dinv);
    GP_CHECK_LAUNCH();
    M->bt_epoch = pc->epoch;
  }
  return GP_OK;
}

static BtArgs bt_args(const BlockTri& b, int n) {
  BtArgs t;
  t.n = n;
  t.W = b.W;
  t.cstart = b.cstart;
  t.lvl_ptr = b.lvl_ptr;
  t.lvl_off = b.lvl_off;
  t.row = b.row;
  t.ridx = b.ridx;
  t.cnt = b.cnt;
  t.code = b.code;
  t.cf = b.cf;
  t.dinv = b.dinv;
  return t;
}

static int mixed_buffers(Mixed* M, int n, int m) {
  if (M->n == n && M->m == m && M->V) return GP_OK;
  for (void** p : {(void**)&M->V, (void**)&M->Z, (void**)&M->w, (void**)&M->t0, (void**)&M->t1,
                   (void**)&M->t2, (void**)&M->t3, (void**)&M->t4, (void**)&M->r, (void**)&M->y,
                   (void**)&M->h_dev, (void**)&M->partials, (void**)&M->ticket})
    if (*p) {
      cudaFree(*p);
      *p = nullptr;
    }
  if (M->h_pinned) cudaFreeHost(M->h_pinned);
  M->h_pinned = nullptr;
  const size_t nn = std::max(n, 1);
  GP_CUDA(cudaMalloc(&M->V, (size_t)(m + 1) * nn * sizeof(float)));
  GP_CUDA(cudaMalloc(&M->Z, (size_t)m * nn * sizeof(float)));
  for (float** p : {&M->w, &M->t0, &M->t1, &M->t2, &M->t3, &M->t4})
    GP_CUDA(cudaMalloc(p, nn * sizeof(float)));
  GP_CUDA(cudaMalloc(&M->r, nn * sizeof(double)));
  GP_CUDA(cudaMalloc(&M->y, nn * sizeof(double)));
  GP_CUDA(cudaMalloc(&M->h_dev, (m + 2) * sizeof(double)));
  GP_CUDA(cudaMalloc(&M->partials, (size_t)(m + 2) * mix_grid(n) * sizeof(double)));
  GP_CUDA(cudaMalloc(&M->ticket, sizeof(unsigned)));
  GP_CUDA(cudaMemset(M->ticket, 0, sizeof(unsigned)));
  GP_CUDA(cudaMallocHost(&M->h_pinned, (m + 2) * sizeof(double)));
  M->n = n;
  M->m = m;
  return GP_OK;
}

// k dots of w against V's first k rows (or ||w||^2 with V null) into host h
static int mdot_host(Mixed* M, const float* V, int k, const float* w, double* h, cudaStream_t s) {
  const int n = M->n, g = mix_grid(n);
  k_mdot32<<<mdot_grid(n), kMixBlock, 0, s>>>(n, V, k, w, M->partials, M->ticket, M->h_dev);
  GP_CHECK_LAUNCH();
  const int kk = V ? k : 1;
  GP_CUDA(cudaMemcpyAsync(M->h_pinned, M->h_dev, kk * sizeof(double), cudaMemcpyDeviceToHost, s));
  GP_CUDA(cudaStreamSynchronize(s));
  std::memcpy(h, M->h_pinned, kk * sizeof(double));
  return GP_OK;
}

// z = M^-1 v with the FP32 factors (tri_sweeps Jacobi passes per triangle), or
// with the exact FP64 sweeps of the plain path when tri_sweeps == 0.
static int mixed_pc(Mixed* M, int tri_sweeps, const float* v, float* z, cudaStream_t s) {
  const int n = M->n;
  const int g = mix_grid(n), gr = (n + kMixBlock - 1) / kMixBlock;
  if (tri_sweeps <= 0) {
    // exact: through the FP64 level-scheduled sweeps
    GP_CUDA(cudaMemsetAsync(M->y, 0, n * sizeof(double), s));
    k_axpy64_32<<<g, kMixBlock, 0, s>>>(n, 1.0, v, M->y);
    GP_TRY(pc_apply(const_cast<Pc*>(M->pc), DRef::of(M->y), DRef::of(M->r), s));
    k_to32_scaled<<<g, kMixBlock, 0, s>>>(n, M->r, 1.0, z);
    GP_CHECK_LAUNCH();
    return GP_OK;
  }
  const Pc* pc = M->pc;
  float* bp = M->t0;
  k_gather32<<<g, kMixBlock, 0, s>>>(n, pc->perm_r, v, bp);
  // forward, unit lower: y <- bp - L y, from y = bp
  float* ya = M->t1;
  float* yb = M->t2;
  const float* yin = bp;
  for (int k = 0; k < tri_sweeps; k++) {
    k_tri_pass<<<gr, kMixBlock, 0, s>>>(n, M->lrp, M->lci, M->lval, nullptr, bp, yin, ya);
    yin = ya;
    std::swap(ya, yb);
  }
  // backward: x <- D^-1 (y - U x), from x = D^-1 y
  float* xa = M->t3;
  float* xb = M->t4;
  k_mul32<<<g, kMixBlock, 0, s>>>(n, M->udinv, yin, xa);
  const float* xin = xa;
  std::swap(xa, xb);
  for (int k = 0; k < tri_sweeps; k++) {
    k_tri_pass<<<gr, kMixBlock, 0, s>>>(n, M->urp, M->uci, M->uval, M->udinv, yin, xin, xa);
    xin = xa;
    std::swap(xa, xb);
  }
  k_scatter32<<<g, kMixBlock, 0, s>>>(n, pc->perm_c, xin, z);
  GP_CHECK_LAUNCH();
  return GP_OK;
}

int mixed_solve_graph(Mixed* M, Csr* A, Pc* pc, const double* b, double* x,
                      const MixedOptions& o, MixedResult& res, cudaStream_t caller);

// GPETSC_KSP_GRAPH=0: the host-driven form (one sync per reduction)
static bool mixed_host_mode() {
  static bool v = [] {
    const char* e = std::getenv("GPETSC_KSP_GRAPH");
    return e && std::string(e) == "0";
  }();
  return v;
}

int mixed_solve(Mixed* M, Csr* A, Pc* pc, const double* b, double* x, const MixedOptions& o,
                MixedResult& res, cudaStream_t s) {
  if (pc->opt.type != PC_ILU || !pc->ready || pc->n != A->n) {
    set_error("mixed solve: needs an ILU preconditioner set up on the operator");
    return GP_ERR_NOT_SETUP;
  }
  if (o.restart < 1 || o.restart > kMixMaxM || o.max_outer < 1 || o.tri_sweeps < 0) {
    set_error("mixed solve: restart must be 1..64, max_outer >= 1, tri_sweeps >= 0");
    return GP_ERR_ARG;
  }
  const int n = A->n, m = o.restart;
  M->A = A;
  M->pc = pc;
  res = MixedResult();
  if (n == 0) {
    res.converged = 1;
    return GP_OK;
  }
  GP_TRY(mixed_buffers(M, n, m));
  if (!mixed_host_mode()) return mixed_solve_graph(M, A, pc, b, x, o, res, s);
  GP_TRY(csr_make_val32(A, s));
  GP_TRY(mixed_factors(M, s));
  const int g = mix_grid(n), gr = (n + kMixBlock - 1) / kMixBlock;
  double bb = 0.0;
  GP_TRY(vec_reduce(s, RED_NORM2SQ, n, b, nullptr, &bb));
  const double bnorm = std::sqrt(bb);
  GP_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), s));
  std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), gv(m + 1), h(m + 1), yv(m);
  for (int pass = 0;; pass++) {
    // FP64 residual
    GP_TRY(spmv(s, A, DRef::of(x), DRef::of(M->y)));
    k_resid_parts<<<g, kMixBlock, 0, s>>>(n, b, M->y, M->r);
    double rr = 0.0;
    GP_TRY(vec_reduce(s, RED_NORM2SQ, n, M->r, nullptr, &rr));
    const double rn = std::sqrt(rr);
    res.relres = bnorm > 0.0 ? rn / bnorm : rn;
    if (!(rn > o.rtol * bnorm)) {
      res.converged = 1;
      break;
    }
    if (pass >= o.max_outer || !std::isfinite(rn)) break;
    res.passes = pass + 1;
    // one FP32 FGMRES(m) cycle on A d = r / ||r||
    k_to32_scaled<<<g, kMixBlock, 0, s>>>(n, M->r, 1.0 / rn, M->V);
    double beta2 = 0.0;
    GP_TRY(mdot_host(M, nullptr, 1, M->V, &beta2, s));
    const double beta = std::sqrt(beta2);
    if (!(beta > 0.0)) break;
    k_scale32<<<g, kMixBlock, 0, s>>>(n, M->V, (float)(1.0 / beta), M->V);
    std::fill(gv.begin(), gv.end(), 0.0);
    gv[0] = beta;
    int kdim = 0;
    for (int j = 0; j < m; j++) {
      float* vj = M->V + (size_t)j * n;
      float* zj = M->Z + (size_t)j * n;
      GP_TRY(mixed_pc(M, o.tri_sweeps, vj, zj, s));
      if (A->coff16)
        k_spmv32<short><<<gr, kMixBlock, 0, s>>>(n, A->rowptr, A->coff16, A->val32, zj, M->w);
      else
        k_spmv32<int><<<gr, kMixBlock, 0, s>>>(n, A->rowptr, A->colind, A->val32, zj, M->w);
      // classical Gram-Schmidt against v_0..v_j
      GP_TRY(mdot_host(M, M->V, j + 1, M->w, h.data(), s));
      k_maxpy32<<<g, kMixBlock, 0, s>>>(n, M->V, j + 1, M->h_dev, M->w);
      double hn2 = 0.0;
      GP_TRY(mdot_host(M, nullptr, 1, M->w, &hn2, s));
      const double hn = std::sqrt(hn2);
      res.inner_its += 1;
      // Hessenberg column j, previous rotations, new rotation (FP64, host)
      for (int i = 0; i <= j; i++) H[(size_t)i * m + j] = h[i];
      for (int i = 0; i < j; i++) {
        const double a = H[(size_t)i * m + j], c = H[(size_t)(i + 1) * m + j];
        H[(size_t)i * m + j] = cs[i] * a + sn[i] * c;
        H[(size_t)(i + 1) * m + j] = -sn[i] * a + cs[i] * c;
      }
      const double hjj = H[(size_t)j * m + j];
      const double den = std::hypot(hjj, hn);
      cs[j] = den > 0.0 ? hjj / den : 1.0;
      sn[j] = den > 0.0 ? hn / den : 0.0;
      H[(size_t)j * m + j] = den;
      gv[j + 1] = -sn[j] * gv[j];
      gv[j] = cs[j] * gv[j];
      kdim = j + 1;
      if (!(hn > 0.0) || std::fabs(gv[j + 1]) <= o.inner_rtol * beta) break;
      if (j + 1 < m)
        k_scale32<<<g, kMixBlock, 0, s>>>(n, M->w, (float)(1.0 / hn), M->V + (size_t)(j + 1) * n);
    }
    // y = H^-1 g (upper triangular), d = Z y, x += ||r|| d
    for (int i = kdim - 1; i >= 0; i--) {
      double t = gv[i];
      for (int k = i + 1; k < kdim; k++) t -= H[(size_t)i * m + k] * yv[k];
      yv[i] = H[(size_t)i * m + i] != 0.0 ? t / H[(size_t)i * m + i] : 0.0;
    }
    std::memcpy(M->h_pinned, yv.data(), kdim * sizeof(double));
    GP_CUDA(cudaMemcpyAsync(M->h_dev, M->h_pinned, kdim * sizeof(double), cudaMemcpyHostToDevice,
                            s));
    k_lincomb32<<<g, kMixBlock, 0, s>>>(n, M->Z, kdim, M->h_dev, M->w);
    k_axpy64_32<<<g, kMixBlock, 0, s>>>(n, rn, M->w, x);
    GP_CHECK_LAUNCH();
  }
  GP_CUDA(cudaStreamSynchronize(s));
  return GP_OK;
}

// ---------------------------------------------------- captured refinement pass
// One refinement pass as one CUDA graph: FP64 residual and its norm, then an
// FP32 FGMRES(m) cycle with every scalar on the device (Hessenberg column,
// Givens rotations, least-squares in FP64 by one thread), each step gated on
// `active` so the steps after the cycle converged are no-ops, then the
// correction.  The host launches passes and reads one status word per pass.
struct MixDev {
  int pass_on, active, kdim, its, passes, pad_;
  double rn, rtol_bnorm, beta2, beta, tol, inner_rtol, hn2;
  // reciprocals computed once by the one thread that has the norm (a divide
  // in every thread of a streaming kernel costs more than the stream)
  double inv_rn;
  float inv_beta, inv_hn;
  double H[(kMixMaxM + 1) * kMixMaxM];
  double cs[kMixMaxM], sn[kMixMaxM], g[kMixMaxM + 1], y[kMixMaxM];
};

__global__ void __launch_bounds__(kRedBlock) k_mx_resid(int n, const double* __restrict__ b,
                                                        const double* __restrict__ y,
                                                        double* __restrict__ r, RedSlot slot,
                                                        MixDev* st) {
  double v[1] = {0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double ri = b[i] - y[i];
    r[i] = ri;
    v[0] = fma(ri, ri, v[0]);
  }
  double tot[1];
  if (grid_finish<1>(v, slot, tot) && threadIdx.x == 0) {
    const double rn = sqrt(tot[0]);
    st->rn = rn;
    st->inv_rn = rn > 0.0 ? 1.0 / rn : 0.0;
    const int on = (rn > st->rtol_bnorm) && isfinite(rn);
    st->pass_on = on;
    st->active = on;
    st->kdim = 0;
    if (on) st->passes += 1;
  }
}

__global__ void k_mx_v0(int n, const double* __restrict__ r, const MixDev* st,
                        float* __restrict__ v0) {
  if (!st->pass_on) return;
  const double inv = st->inv_rn;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    v0[i] = __double2float_rn(r[i] * inv);
}

__global__ void k_mx_beta(MixDev* st, int m) {
  if (!st->pass_on) return;
  const double beta = sqrt(st->beta2);
  st->beta = beta;
  st->inv_beta = beta > 0.0 ? (float)(1.0 / beta) : 0.f;
  for (int i = 0; i <= m; i++) st->g[i] = 0.0;
  st->g[0] = beta;
  st->tol = st->inner_rtol * beta;
  if (!(beta > 0.0)) st->active = 0;
}

// out = in / beta (which = 0) or in / sqrt(hn2) (which = 1), while active
__global__ void k_mx_scale(int n, const float* in, float* out, const MixDev* st, int which) {
  pdl_wait();
  pdl_trigger();
  if (!st->active) return;
  const float s = which == 0 ? st->inv_beta : st->inv_hn;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = in[i] * s;
}

// One Jacobi pass of a factor triangle, gated; rhs and in may be read through
// a permutation, `in` scaled by in_scale, the output scattered through a
// permutation (first / last passes of the permuted factor solve).
__global__ void __launch_bounds__(kMixBlock) k_mx_tri(
    const int* gate, int n, const int* __restrict__ rp, const int* __restrict__ ci,
    const float* __restrict__ val, const float* __restrict__ dinv, const float* __restrict__ rhs,
    const int* __restrict__ rhs_perm, const float* __restrict__ in, const int* __restrict__ in_perm,
    const float* __restrict__ in_scale, float* __restrict__ out, const int* __restrict__ out_perm) {
  pdl_wait();
  pdl_trigger();
  if (gated_off(gate, 1)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float acc = rhs[rhs_perm ? rhs_perm[i] : i];
  for (int j = rp[i]; j < rp[i + 1]; j++) {
    const int c = ci[j];
    float xin = in[in_perm ? in_perm[c] : c];
    if (in_scale) xin *= in_scale[c];
    acc = __fmaf_rn(-val[j], xin, acc);
  }
  const float o = dinv ? acc * dinv[i] : acc;
  out[out_perm ? out_perm[i] : i] = o;
}

// The same pass over a column-major ELL copy of the triangle ([e * n + i],
// W slots a row, absent ones with a zero coefficient): no row-pointer loads,
// every column and coefficient load coalesced and issued before the gathers.
// Each thread takes kTriRows rows a grid-width apart (coalesced) and issues
// all their column/coefficient loads, then all their gathers, before any
// arithmetic: two memory round trips for the whole pass instead of two per
// row-wave.  Eight rows measured best on GB300 (4: 10% slower; 16: register
// pressure, 20% slower).
constexpr int kTriRows = 8;

template <int W>
__global__ void __launch_bounds__(kMixBlock) k_mx_tri_ell(
    const int* gate, int n, const int* __restrict__ ci, const float* __restrict__ val,
    const float* __restrict__ dinv, const float* __restrict__ rhs,
    const int* __restrict__ rhs_perm, const float* __restrict__ in,
    const int* __restrict__ in_perm, const float* __restrict__ in_scale, float* __restrict__ out,
    const int* __restrict__ out_perm) {
  const int stride = gridDim.x * blockDim.x;
  const int i0 = blockIdx.x * blockDim.x + threadIdx.x;
  int c[kTriRows][W];
  float a[kTriRows][W], acc[kTriRows];
  // The triangle is constant during a solve, so its loads go out before the
  // wait on the previous kernel and overlap its drain.  The gate read before
  // the wait only decides whether to load early (steps gated off after
  // convergence skip the loads); it is read again after the wait, and a step
  // found on then after all takes its rows one at a time.
  const bool early = !gated_off(gate, 1);
  if (early) {
#pragma unroll
    for (int q = 0; q < kTriRows; q++) {
      const int i = i0 + q * stride;
      if (i < n) {
#pragma unroll
        for (int e = 0; e < W; e++) {
          c[q][e] = ci[(size_t)e * n + i];
          a[q][e] = val[(size_t)e * n + i];
        }
      }
    }
  }
  pdl_wait();
  pdl_trigger();
  if (gated_off(gate, 1)) return;
  if (!early) {
    for (int q = 0; q < kTriRows; q++) {
      const int i = i0 + q * stride;
      if (i >= n) break;
      float r = rhs[rhs_perm ? rhs_perm[i] : i];
      for (int e = 0; e < W; e++) {
        const int cc = ci[(size_t)e * n + i];
        float xin = in[in_perm ? in_perm[cc] : cc];
        if (in_scale) xin *= in_scale[cc];
        r = __fmaf_rn(-val[(size_t)e * n + i], xin, r);
      }
      const float o = dinv ? r * dinv[i] : r;
      out[out_perm ? out_perm[i] : i] = o;
    }
    return;
  }
#pragma unroll
  for (int q = 0; q < kTriRows; q++) {
    const int i = i0 + q * stride;
    if (i < n) acc[q] = rhs[rhs_perm ? rhs_perm[i] : i];
  }
#pragma unroll
  for (int q = 0; q < kTriRows; q++) {
    const int i = i0 + q * stride;
    if (i < n) {
      float x[W];
#pragma unroll
      for (int e = 0; e < W; e++) {
        float xin = in[in_perm ? in_perm[c[q][e]] : c[q][e]];
        if (in_scale) xin *= in_scale[c[q][e]];
        x[e] = xin;
      }
#pragma unroll
      for (int e = 0; e < W; e++) acc[q] = __fmaf_rn(-a[q][e], x[e], acc[q]);
    }
  }
#pragma unroll
  for (int q = 0; q < kTriRows; q++) {
    const int i = i0 + q * stride;
    if (i < n) {
      const float o = dinv ? acc[q] * dinv[i] : acc[q];
      out[out_perm ? out_perm[i] : i] = o;
    }
  }
}

template <typename CT>
__global__ void __launch_bounds__(kMixBlock) k_mx_spmv32(const int* gate, int n,
                                                         const int* __restrict__ rp,
                                                         const CT* __restrict__ ci,
                                                         const float* __restrict__ val,
                                                         const float* __restrict__ x,
                                                         float* __restrict__ y) {
  pdl_wait();
  pdl_trigger();
  if (gated_off(gate, 1)) return;
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= n) return;
  const uint64_t pol = l2_evict_first();
  float acc = 0.f;
  for (int j = rp[row]; j < rp[row + 1]; j++)
    acc = __fmaf_rn(ld_stream(val + j, pol), x[spmv_col(ci, j, row, pol)], acc);
  y[row] = acc;
}

// w -= V h and ||w||^2 in one pass (the orthogonalised vector's norm is
// folded while it is written): FP32 per thread and per CTA, per-CTA partials
// in FP64, the last CTA folds them into *out.  Gated on `*gate == 1`.
__global__ void __launch_bounds__(kMixBlock) k_mx_maxpy_norm(const int* gate, int n,
                                                             const float* __restrict__ V, int k,
                                                             const double* __restrict__ h,
                                                             float* __restrict__ w,
                                                             double* __restrict__ partials,
                                                             unsigned* ticket, double* out) {
  pdl_wait();
  pdl_trigger();
  if (gated_off(gate, 1)) return;
  __shared__ float hs[kMixMaxM + 1];
  __shared__ float sh[kMixBlock / 32];
  __shared__ bool last;
  for (int j = threadIdx.x; j < k; j += blockDim.x) hs[j] = (float)h[j];
  __syncthreads();
  float acc = 0.f;
  // two rows a thread per step, eight basis loads of each in flight before
  // their (ordered) multiply-adds
  const int stride = gridDim.x * blockDim.x;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + stride < n; i += 2 * stride) {
    float v0 = w[i], v1 = w[i + stride];
    int j = 0;
    for (; j + 8 <= k; j += 8) {
      float t0[8], t1[8];
#pragma unroll
      for (int q = 0; q < 8; q++) {
        t0[q] = V[(size_t)(j + q) * n + i];
        t1[q] = V[(size_t)(j + q) * n + i + stride];
      }
#pragma unroll
      for (int q = 0; q < 8; q++) {
        v0 = __fmaf_rn(-hs[j + q], t0[q], v0);
        v1 = __fmaf_rn(-hs[j + q], t1[q], v1);
      }
    }
    for (; j < k; j++) {
      v0 = __fmaf_rn(-hs[j], V[(size_t)j * n + i], v0);
      v1 = __fmaf_rn(-hs[j], V[(size_t)j * n + i + stride], v1);
    }
    w[i] = v0;
    w[i + stride] = v1;
    acc = __fmaf_rn(v0, v0, acc);
    acc = __fmaf_rn(v1, v1, acc);
  }
  for (; i < n; i += stride) {
    float v = w[i];
    for (int j = 0; j < k; j++) v = __fmaf_rn(-hs[j], V[(size_t)j * n + i], v);
    w[i] = v;
    acc = __fmaf_rn(v, v, acc);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) sh[wid] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int ww = 0; ww < (int)(blockDim.x >> 5); ww++) t += sh[ww];
    partials[blockIdx.x] = (double)t;
    last = atomic_add_acq_rel(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  fold_partials(partials, 1, out);
  __syncthreads();
  if (threadIdx.x == 0) *ticket = 0u;
}

// Hessenberg column j, rotations and the residual estimate (one thread, FP64)
// One warp: the lanes stage the new column and the earlier rotations in
// shared memory (independent loads), then lane 0 runs the rotations out of
// shared memory -- the chain is the FP64 arithmetic, not a memory round trip
// per rotation.
__global__ void k_mx_givens(MixDev* st, const double* __restrict__ h, int j, int m) {
  pdl_wait();
  pdl_trigger();
  if (!st->active) return;
  __shared__ double col[kMixMaxM + 1], cs[kMixMaxM], sn[kMixMaxM];
  for (int i = threadIdx.x; i <= j; i += blockDim.x) {
    col[i] = h[i];
    if (i < j) {
      cs[i] = st->cs[i];
      sn[i] = st->sn[i];
    }
  }
  __syncwarp();
  if (threadIdx.x != 0) return;
  double* H = st->H;
  const double hn = sqrt(st->hn2);
  st->inv_hn = hn > 0.0 ? (float)(1.0 / hn) : 0.f;
  for (int i = 0; i < j; i++) {
    const double a = col[i], c = col[i + 1];
    col[i] = cs[i] * a + sn[i] * c;
    col[i + 1] = -sn[i] * a + cs[i] * c;
  }
  const double hjj = col[j];
  // one square root and one reciprocal (FP64 divide, square root and hypot
  // are long dependent sequences on this part; the operands are far from
  // overflow: a normalised basis keeps them O(||A||))
  const double den = sqrt(hjj * hjj + hn * hn);
  const double rden = den > 0.0 ? 1.0 / den : 0.0;
  const double cj = den > 0.0 ? hjj * rden : 1.0;
  const double sj = den > 0.0 ? hn * rden : 0.0;
  col[j] = den;
  for (int i = 0; i <= j; i++) H[i * m + j] = col[i];
  st->cs[j] = cj;
  st->sn[j] = sj;
  const double gj = st->g[j];
  st->g[j + 1] = -sj * gj;
  st->g[j] = cj * gj;
  st->kdim = j + 1;
  st->its += 1;
  if (!(hn > 0.0) || fabs(-sj * gj) <= st->tol || j + 1 == m) st->active = 0;
}

// Back-substitution of the least-squares system: the warp stages the upper
// triangle of H and g in shared memory, lane 0 solves out of it.
__global__ void k_mx_backsub(MixDev* st, int m) {
  if (!st->pass_on) return;
  __shared__ double Hs[kMixMaxM * kMixMaxM], gs[kMixMaxM], ys[kMixMaxM];
  const int k = st->kdim;
  for (int q = threadIdx.x; q < k * k; q += blockDim.x) {
    const int i = q / k, c = q % k;
    if (c >= i) Hs[i * k + c] = st->H[i * m + c];
  }
  for (int i = threadIdx.x; i < k; i += blockDim.x) gs[i] = st->g[i];
  __syncwarp();
  if (threadIdx.x == 0) {
    for (int i = k - 1; i >= 0; i--) {
      double t = gs[i];
      for (int c = i + 1; c < k; c++) t -= Hs[i * k + c] * ys[c];
      ys[i] = Hs[i * k + i] != 0.0 ? t / Hs[i * k + i] : 0.0;
    }
  }
  __syncwarp();
  for (int i = threadIdx.x; i < k; i += blockDim.x) st->y[i] = ys[i];
}

// x += rn * sum_{j < kdim} y_j Z_j
__global__ void k_mx_correct(int n, const float* __restrict__ Z, const MixDev* st,
                             double* __restrict__ x) {
  if (!st->pass_on) return;
  __shared__ float ys[kMixMaxM];
  const int k = st->kdim;
  for (int j = threadIdx.x; j < k; j += blockDim.x) ys[j] = (float)st->y[j];
  __syncthreads();
  const double rn = st->rn;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float d = 0.f;
    int j = 0;
    for (; j + 8 <= k; j += 8) {  // eight loads in flight before their ordered sums
      float t[8];
#pragma unroll
      for (int q = 0; q < 8; q++) t[q] = Z[(size_t)(j + q) * n + i];
#pragma unroll
      for (int q = 0; q < 8; q++) d = __fmaf_rn(ys[j + q], t[q], d);
    }
    for (; j < k; j++) d = __fmaf_rn(ys[j], Z[(size_t)j * n + i], d);
    x[i] = fma(rn, (double)d, x[i]);
  }
}

// the mdot of the host-driven form, gated on `*gate == 1`
__global__ void __launch_bounds__(kMixBlock) k_mx_mdot(const int* gate, int n,
                                                       const float* __restrict__ V, int k,
                                                       const float* __restrict__ w,
                                                       double* __restrict__ partials,
                                                       unsigned* ticket, double* out) {
  pdl_wait();
  pdl_trigger();
  if (gated_off(gate, 1)) return;
  __shared__ float sh[kMixBlock / 32][kMixMaxM + 1];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int kk = V ? k : 1;
  for (int j0 = 0; j0 < kk; j0 += 8) {
    float acc[8];
#pragma unroll
    for (int q = 0; q < 8; q++) acc[q] = 0.f;
    // two rows a thread per step, all their loads issued before the
    // multiply-adds (accumulation order per thread unchanged: row by row)
    const int stride = gridDim.x * blockDim.x;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + stride < n; i += 2 * stride) {
      const float w0 = w[i], w1 = w[i + stride];
      float v0[8], v1[8];
#pragma unroll
      for (int q = 0; q < 8; q++)
        if (j0 + q < kk) {
          v0[q] = V ? V[(size_t)(j0 + q) * n + i] : w0;
          v1[q] = V ? V[(size_t)(j0 + q) * n + i + stride] : w1;
        }
#pragma unroll
      for (int q = 0; q < 8; q++)
        if (j0 + q < kk) {
          acc[q] = __fmaf_rn(v0[q], w0, acc[q]);
          acc[q] = __fmaf_rn(v1[q], w1, acc[q]);
        }
    }
    for (; i < n; i += stride) {
      const float wi = w[i];
#pragma unroll
      for (int q = 0; q < 8; q++)
        if (j0 + q < kk) acc[q] = __fmaf_rn(V ? V[(size_t)(j0 + q) * n + i] : wi, wi, acc[q]);
    }
#pragma unroll
    for (int q = 0; q < 8; q++) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc[q] += __shfl_down_sync(0xffffffffu, acc[q], o);
      if (lane == 0 && j0 + q < kk) sh[wid][j0 + q] = acc[q];
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int j = 0; j < kk; j++) {
      float t = 0.f;
      for (int ww = 0; ww < (int)(blockDim.x >> 5); ww++) t += sh[ww][j];
      partials[(size_t)j * gridDim.x + blockIdx.x] = (double)t;
    }
    last = atomic_add_acq_rel(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  fold_partials(partials, kk, out);
  __syncthreads();
  if (threadIdx.x == 0) *ticket = 0u;
}

__global__ void k_mx_cast64(const int* gate, int n, const float* __restrict__ a,
                            double* __restrict__ b) {
  if (gated_off(gate, 1)) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    b[i] = (double)a[i];
}

__global__ void k_mx_cast32(const int* gate, int n, const double* __restrict__ a,
                            float* __restrict__ b) {
  if (gated_off(gate, 1)) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    b[i] = __double2float_rn(a[i]);
}

// One triangle pass: the ELL form when the triangle has at most 8 slots a row.
static void tri_pass(int W, const int* eci, const float* eval, const int* rp, const int* ci,
                     const float* val, const int* gate, int n, const float* dinv,
                     const float* rhs, const int* rhs_perm, const float* in, const int* in_perm,
                     const float* in_scale, float* out, const int* out_perm, cudaStream_t s) {
  const int gr = (n + kMixBlock * kTriRows - 1) / (kMixBlock * kTriRows);
#define GP_TRI_ELL(WW)                                                                     \
  case WW:                                                                                 \
    (void)launch_pdl(k_mx_tri_ell<WW>, gr, kMixBlock, s, gate, n, eci, eval, dinv, rhs,   \
                     rhs_perm, in, in_perm, in_scale, out, out_perm);                      \
    return;
  switch (W) {
    GP_TRI_ELL(1)
    GP_TRI_ELL(2)
    GP_TRI_ELL(3)
    GP_TRI_ELL(4)
    GP_TRI_ELL(5)
    GP_TRI_ELL(6)
    GP_TRI_ELL(7)
    GP_TRI_ELL(8)
    default:
      break;
  }
#undef GP_TRI_ELL
  (void)launch_pdl(k_mx_tri, (n + kMixBlock - 1) / kMixBlock, kMixBlock, s, gate, n, rp, ci, val,
                   dinv, rhs, rhs_perm, in, in_perm, in_scale, out, out_perm);
}

// Record one refinement pass into the current capture on stream s.
static int record_pass(Mixed* M, const Csr* A, const Pc* pc, const double* b, double* x,
                       int tri_sweeps, int tri_block, cudaStream_t s) {
  const int n = M->n, m = M->m, g = mix_grid(n), gr = (n + kMixBlock - 1) / kMixBlock;
  MixDev* st = M->st;
  const int* on = &st->pass_on;
  const int* act = &st->active;
  RedSlot slot{};
  slot.partials = M->part64;
  slot.ticket = M->ticket64;
  slot.stride = kMaxRedGrid;
  GP_TRY(spmv(s, A, DRef::of(x), DRef::of(M->y)));
  k_mx_resid<<<red_grid(n), kRedBlock, 0, s>>>(n, b, M->y, M->r, slot, st);
  k_mx_v0<<<g, kMixBlock, 0, s>>>(n, M->r, st, M->V);
  k_mx_mdot<<<mdot_grid(n), kMixBlock, 0, s>>>(on, n, nullptr, 1, M->V, M->partials, M->ticket,
                                     &st->beta2);
  k_mx_beta<<<1, 1, 0, s>>>(st, m);
  k_mx_scale<<<g, kMixBlock, 0, s>>>(n, M->V, M->V, st, 0);
  for (int j = 0; j < m; j++) {
    float* vj = M->V + (size_t)j * n;
    float* zj = M->Z + (size_t)j * n;
    const int* perm_r = M->ident_r ? nullptr : pc->perm_r;
    const int* perm_c = M->ident_c ? nullptr : pc->perm_c;
    if (tri_sweeps > 0 && tri_block != 0) {
      // block passes: exact inside each run of rows, couplings from the last pass
      const BtArgs tl = bt_args(M->bl, n), tu = bt_args(M->bu, n);
      float* ya = M->t1;
      float* yb = M->t2;
      const float* yprev = nullptr;
      for (int k = 0; k < tri_sweeps; k++) {
        launch_btri<false>(tl, M->bl.nblocks, M->bl.smem, act, vj, yprev, ya, nullptr, s);
        yprev = ya;
        std::swap(ya, yb);
      }
      const float* yfin = yprev;
      float* xa = M->t3;
      float* xb = M->t4;
      const float* xprev = nullptr;
      for (int k = 0; k < tri_sweeps; k++) {
        const bool lastp = k + 1 == tri_sweeps;
        launch_btri<true>(tu, M->bu.nblocks, M->bu.smem, act, yfin, xprev, lastp ? zj : xa,
                          lastp ? perm_c : nullptr, s);
        xprev = xa;
        std::swap(xa, xb);
      }
    } else if (tri_sweeps > 0) {
      // L: y <- Pv - L y from y = Pv;  U: x <- D^-1 (y - U x) from x = D^-1 y
      float* ya = M->t1;
      float* yb = M->t2;
      const float* yin = vj;
      const int* yperm = perm_r;
      for (int k = 0; k < tri_sweeps; k++) {
        tri_pass(M->lW, M->lell_ci, M->lell_val, M->lrp, M->lci, M->lval, act, n, nullptr, vj,
                 perm_r, yin, yperm, nullptr, ya, nullptr, s);
        yin = ya;
        yperm = nullptr;
        std::swap(ya, yb);
      }
      float* xa = M->t3;
      float* xb = M->t4;
      const float* xin = yin;
      const float* xscale = M->udinv;
      for (int k = 0; k < tri_sweeps; k++) {
        const bool lastp = k + 1 == tri_sweeps;
        tri_pass(M->uW, M->uell_ci, M->uell_val, M->urp, M->uci, M->uval, act, n, M->udinv, yin,
                 nullptr, xin, nullptr, xscale, lastp ? zj : xa, lastp ? perm_c : nullptr, s);
        xin = xa;
        xscale = nullptr;
        std::swap(xa, xb);
      }
    } else {
      // exact: the FP64 level-scheduled sweeps of the plain path, gated
      k_mx_cast64<<<g, kMixBlock, 0, s>>>(act, n, vj, M->y);
      GP_TRY(pc_apply(const_cast<Pc*>(pc), DRef::of(M->y), DRef::of(M->r), s, act, 1));
      k_mx_cast32<<<g, kMixBlock, 0, s>>>(act, n, M->r, zj);
    }
    // the step's kernels start while their predecessor drains (each waits
    // in pdl_wait() before reading it)
    if (A->coff16)
      GP_CUDA(launch_pdl(k_mx_spmv32<short>, gr, kMixBlock, s, act, n, A->rowptr,
                         (const short*)A->coff16, A->val32, zj, M->w));
    else
      GP_CUDA(launch_pdl(k_mx_spmv32<int>, gr, kMixBlock, s, act, n, A->rowptr,
                         (const int*)A->colind, A->val32, zj, M->w));
    GP_CUDA(launch_pdl(k_mx_mdot, mdot_grid(n), kMixBlock, s, act, n, M->V, j + 1, M->w,
                       M->partials, M->ticket, M->h_dev));
    GP_CUDA(launch_pdl(k_mx_maxpy_norm, g, kMixBlock, s, act, n, M->V, j + 1, M->h_dev, M->w,
                       M->partials, M->ticket, &st->hn2));
    GP_CUDA(launch_pdl(k_mx_givens, 1, 32, s, st, M->h_dev, j, m));
    if (j + 1 < m)
      GP_CUDA(launch_pdl(k_mx_scale, g, kMixBlock, s, n, M->w, M->V + (size_t)(j + 1) * n, st, 1));
  }
  k_mx_backsub<<<1, 32, 0, s>>>(st, m);
  k_mx_correct<<<g, kMixBlock, 0, s>>>(n, M->Z, st, x);
  GP_CUDA(cudaMemcpyAsync(M->h_st, st, offsetof(MixDev, H), cudaMemcpyDeviceToHost, s));
  GP_CHECK_LAUNCH();
  return GP_OK;
}

int mixed_solve_graph(Mixed* M, Csr* A, Pc* pc, const double* b, double* x,
                      const MixedOptions& o, MixedResult& res, cudaStream_t caller) {
  const int n = A->n, m = o.restart;
  if (!M->st) {
    GP_CUDA(cudaMalloc(&M->st, sizeof(MixDev)));
    GP_CUDA(cudaMallocHost(&M->h_st, sizeof(MixDev)));
    GP_CUDA(cudaMalloc(&M->part64, kMaxRedGrid * sizeof(double)));
    GP_CUDA(cudaMalloc(&M->ticket64, sizeof(unsigned)));
    GP_CUDA(cudaMemset(M->ticket64, 0, sizeof(unsigned)));
    GP_CUDA(cudaStreamCreateWithFlags(&M->cap_stream, cudaStreamNonBlocking));
  }
  cudaStream_t s = M->cap_stream;
  cudaEvent_t ev;
  GP_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  GP_CUDA(cudaEventRecord(ev, caller));
  GP_CUDA(cudaStreamWaitEvent(s, ev, 0));
  GP_TRY(csr_make_val32(A, s));
  GP_TRY(mixed_factors(M, s));
  if (o.tri_sweeps > 0 && o.tri_block != 0) GP_TRY(mixed_blocks(M, o.tri_block, s));
  double bb = 0.0;
  GP_TRY(vec_reduce(s, RED_NORM2SQ, n, b, nullptr, &bb));
  const double bnorm = std::sqrt(bb);
  // device state for this solve
  MixDev h{};
  h.rtol_bnorm = o.rtol * bnorm;
  h.inner_rtol = o.inner_rtol;
  std::memcpy(M->h_st, &h, offsetof(MixDev, H));
  GP_CUDA(cudaMemcpyAsync(M->st, M->h_st, offsetof(MixDev, H), cudaMemcpyHostToDevice, s));
  GP_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), s));
  const void* key[6] = {A, pc, b, x, pc->ba, A->val32};
  const int bt = (o.tri_sweeps > 0 && o.tri_block != 0) ? M->bt_rows : 0;
  const int ikey[5] = {n, m, o.tri_sweeps, 0, bt};
  // the operator and the PC set-up by their unique ids as well as their
  // addresses (an address can come back from the allocator)
  const bool same = M->exec && std::equal(key, key + 6, M->cap_key) &&
                    std::equal(ikey, ikey + 5, M->cap_ikey) && M->cap_A_uid == A->uid &&
                    M->cap_pc_gen == pc->generation;
  if (!same) {
    if (M->exec) cudaGraphExecDestroy(M->exec);
    if (M->graph) cudaGraphDestroy(M->graph);
    M->exec = nullptr;
    M->graph = nullptr;
    GP_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
    int st = record_pass(M, A, pc, b, x, o.tri_sweeps, bt, s);
    cudaGraph_t gph = nullptr;
    cudaError_t ec = cudaStreamEndCapture(s, &gph);
    if (st != GP_OK) {
      if (gph) cudaGraphDestroy(gph);
      return st;
    }
    if (ec != cudaSuccess) {
      set_error(std::string("mixed solve capture: ") + cudaGetErrorString(ec));
      return GP_ERR_CUDA;
    }
    M->graph = gph;
    GP_CUDA(cudaGraphInstantiate(&M->exec, gph, 0));
    std::copy(key, key + 6, M->cap_key);
    std::copy(ikey, ikey + 5, M->cap_ikey);
    M->cap_A_uid = A->uid;
    M->cap_pc_gen = pc->generation;
  }
  res = MixedResult();
  for (int pass = 0; pass <= o.max_outer; pass++) {
    GP_CUDA(cudaGraphLaunch(M->exec, s));
    GP_CUDA(cudaStreamSynchronize(s));
    const MixDev& hs = *M->h_st;
    res.relres = bnorm > 0.0 ? hs.rn / bnorm : hs.rn;
    res.inner_its = hs.its;
    res.passes = hs.passes;
    if (!hs.pass_on) {
      res.converged = hs.rn <= o.rtol * bnorm;
      break;
    }
  }
  if (!res.converged) {  // the last pass corrected x after its residual: measure again
    GP_TRY(spmv(s, A, DRef::of(x), DRef::of(M->y)));
    k_resid_parts<<<mix_grid(n), kMixBlock, 0, s>>>(n, b, M->y, M->r);
    double rr = 0.0;
    GP_TRY(vec_reduce(s, RED_NORM2SQ, n, M->r, nullptr, &rr));
    res.relres = bnorm > 0.0 ? std::sqrt(rr) / bnorm : std::sqrt(rr);
    res.converged = res.relres <= o.rtol;
  }
  GP_CUDA(cudaEventRecord(ev, s));
  GP_CUDA(cudaStreamWaitEvent(caller, ev, 0));
  cudaEventDestroy(ev);
  return GP_OK;
}

Mixed* mixed_create() { return new Mixed(); }
void mixed_destroy(Mixed* M) {
  if (!M) return;
  mixed_free(M);
  delete M;
}

}  // namespace gp

// ------------------------------------------------------------------- C ABI
struct gp_mixed_s {
  gp::Mixed* M;
};

extern "C" {

void gp_mixed_options_default(gp_mixed_options* o) {
  gp::MixedOptions d;
  std::memset(o, 0, sizeof(*o));
  o->restart = d.restart;
  o->max_outer = d.max_outer;
  o->tri_sweeps = d.tri_sweeps;
  o->tri_block = d.tri_block;
  o->rtol = d.rtol;
  o->inner_rtol = d.inner_rtol;
}

int gp_mixed_create(gp_mixed* out) {
  if (!out) {
    gp::set_error("gp_mixed_create: null argument");
    return GP_ERR_ARG;
  }
  *out = new gp_mixed_s{gp::mixed_create()};
  return GP_OK;
}

int gp_mixed_destroy(gp_mixed m) {
  if (!m) return GP_OK;
  gp::mixed_destroy(m->M);
  delete m;
  return GP_OK;
}

int gp_mixed_solve(gp_mixed m, gp_mat A, gp_pc pc, const gp_mixed_options* o, const double* b,
                   double* x, gp_mixed_result* result, void* stream) {
  if (!m || !A || !pc || !o || (A->A->n && (!b || !x))) {
    gp::set_error("gp_mixed_solve: null argument");
    return GP_ERR_ARG;
  }
  if (b == x) {
    gp::set_error("gp_mixed_solve: x may not alias b");
    return GP_ERR_ARG;
  }
  try {
    gp::MixedOptions mo;
    mo.restart = o->restart;
    mo.max_outer = o->max_outer;
    mo.tri_sweeps = o->tri_sweeps;
    mo.tri_block = o->tri_block;
    mo.rtol = o->rtol;
    mo.inner_rtol = o->inner_rtol;
    gp::MixedResult r;
    int st = gp::mixed_solve(m->M, A->A, pc->pc, b, x, mo, r, static_cast<cudaStream_t>(stream));
    if (st) return st;
    if (result) {
      result->passes = r.passes;
      result->inner_its = r.inner_its;
      result->converged = r.converged;
      result->relres = r.relres;
    }
    return GP_OK;
  } catch (const std::exception& e) {
    gp::set_error(std::string("gp_mixed_solve: ") + e.what());
    return GP_ERR_INTERNAL;
  }
}

}  // extern "C"
