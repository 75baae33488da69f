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
  unsigned* tickets;
  DevErr* err;
  int sleep_after, sleep_ns;  // polling back-off of the waits
};

// Launch shape and polling back-off of the sweeps (GPETSC_SWEEP_CTAS_PER_SM,
// GPETSC_SWEEP_SLEEP_AFTER, GPETSC_SWEEP_SLEEP_NS override the defaults).
struct SweepTuning {
  int ctas_per_sm = 2, sleep_after = 8, sleep_ns = 20;  // best of a scan on ICC(0), 128^3
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
      // ---- the dependency chain, in the reference's slot order
#pragma unroll
      for (int e = 0; e < WMAX; e++) {
        if (e < c) {
          const double v =
              ell_wait(&a.val[dp[e]], a.err, 20 + MODE, kEllSpin, a.sleep_after, a.sleep_ns);
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
  void* ptrs[] = {e.cnt, e.dep, e.cslot, e.coef, e.in_idx, e.out_idx, e.dslot, e.dval, e.rowof};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  e = EllSweep();
}

// Lay out one sweep.  dptr/dcol/dsl: each row's dependencies (rows) and their
// coefficient slots, in the reference's order; order: processing order.
int ell_build(EllSweep& e, int n, const std::vector<int>& order, const std::vector<int>& dptr,
              const std::vector<int>& dcol, const std::vector<int>& dsl,
              const std::vector<int>& in_row, const std::vector<int>& out_row,
              const std::vector<int>& dslot_row, std::vector<int>* pos_of_row) {
  ell_free(e);
  int W = 0;
  for (int i = 0; i < n; i++) W = std::max(W, dptr[i + 1] - dptr[i]);
  e.n = n;
  e.W = W;
  if (W > kEllMaxW) return GP_OK;  // the CSR sweep kernels handle wide rows
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
  if (!e.ok || e.n == 0) return GP_OK;
  k_ell_refresh<<<std::max(1, std::min((e.n + 255) / 256, num_sms() * 8)), 256, 0, s>>>(
      e.n, e.W, e.cnt, e.cslot, src, e.coef, e.dslot, e.dval);
  GP_CHECK_LAUNCH();
  return GP_OK;
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
              DevErr* err, cudaStream_t s) {
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
  a.tickets = tickets;
  a.err = err;
  a.sleep_after = sweep_tuning().sleep_after;
  a.sleep_ns = sweep_tuning().sleep_ns;
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
