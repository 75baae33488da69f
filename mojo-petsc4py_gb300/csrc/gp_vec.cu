// Vec kernels: elementwise maps, MAXPY and deterministic reductions.
//
// Maps follow the reference's per-element expressions and branch structure
// (src/ported.mojo:75-341 over src/simdvec.mojo:40-319): every element is one
// rounded operation sequence identical to the CPU loop, so maps are bit-exact.
// Reductions (src/simdvec.mojo:332-500) sum in a fixed GPU order instead of
// the CPU's 16-lane blocked order; they are reproducible run to run and agree
// with the CPU sums to rounding.
#include <algorithm>

#include "gp_internal.h"
#include "gp_ordred.cuh"

namespace gp {

// ------------------------------------------------------------------ maps

// Which operands an op reads (y is always written).
template <int OP>
struct MapReads {
  static constexpr bool y = OP == OP_SCALE || OP == OP_DIVS || OP == OP_SHIFT || OP == OP_AXPY ||
                            OP == OP_AYPX || OP == OP_AXPBY || OP == OP_AXPBYPCZ ||
                            OP == OP_RECIP || OP == OP_EXP || OP == OP_LOG ||
                            OP == OP_SQRTABS || OP == OP_ABS;
  static constexpr bool x = OP == OP_COPY || OP == OP_SCALESET || OP == OP_AXPY ||
                            OP == OP_AYPX || OP == OP_AXPBY || OP == OP_AXPBYPCZ ||
                            OP == OP_WAXPY || OP == OP_PMULT || OP == OP_PDIV ||
                            OP == OP_PMIN || OP == OP_PMAX || OP == OP_PMAXABS;
  static constexpr bool w = OP == OP_AXPBYPCZ || OP == OP_WAXPY || OP == OP_PMULT ||
                            OP == OP_PDIV || OP == OP_PMIN || OP == OP_PMAX || OP == OP_PMAXABS;
};

// One element of an op from its loaded operands.
template <int OP, bool FMA>
__device__ __forceinline__ double map_value(double yv, double xv, double wv, double alpha,
                                            double beta, double gamma) {
  if constexpr (OP == OP_COPY) {
    return xv;
  } else if constexpr (OP == OP_SET) {
    return alpha;
  } else if constexpr (OP == OP_ZERO) {
    return 0.0;
  } else if constexpr (OP == OP_SCALE) {
    return mul(yv, alpha);
  } else if constexpr (OP == OP_SCALESET) {  // x alpha into y
    return mul(xv, alpha);
  } else if constexpr (OP == OP_DIVS) {  // y / alpha (VecNormalize)
    return div_(yv, alpha);
  } else if constexpr (OP == OP_SHIFT) {
    return add(yv, alpha);
  } else if constexpr (OP == OP_AXPY) {  // y + alpha x
    return madd<FMA>(alpha, xv, yv);
  } else if constexpr (OP == OP_AYPX) {  // x + alpha y
    return madd<FMA>(alpha, yv, xv);
  } else if constexpr (OP == OP_AXPBY) {  // alpha x + beta y
    return madd<FMA>(alpha, xv, mul(beta, yv));
  } else if constexpr (OP == OP_AXPBYPCZ) {  // alpha x + beta w + gamma y
    return madd<FMA>(gamma, yv, madd<FMA>(beta, wv, mul(alpha, xv)));
  } else if constexpr (OP == OP_WAXPY) {  // alpha x + w
    return madd<FMA>(alpha, xv, wv);
  } else if constexpr (OP == OP_PMULT) {
    return mul(xv, wv);
  } else if constexpr (OP == OP_PDIV) {
    return div_(xv, wv);
  } else if constexpr (OP == OP_PMIN) {
    return (wv < xv) ? wv : xv;
  } else if constexpr (OP == OP_PMAX) {
    return (wv > xv) ? wv : xv;
  } else if constexpr (OP == OP_PMAXABS) {
    const double a = fabs(xv), b = fabs(wv);
    return (b > a) ? b : a;
  } else if constexpr (OP == OP_RECIP) {
    return (yv == 0.0) ? 0.0 : div_(1.0, yv);
  } else if constexpr (OP == OP_EXP) {
    return exp(yv);
  } else if constexpr (OP == OP_LOG) {
    return log(yv);
  } else if constexpr (OP == OP_SQRTABS) {
    return __dsqrt_rn(fabs(yv));
  } else {
    static_assert(OP == OP_ABS, "map op");
    return fabs(yv);
  }
}

// Elements a thread takes per trip (kMapU, or 1 where noted); all their
// loads are issued before the arithmetic.  With one element a trip a thread
// has one load per operand in flight and then waits on its FP64 operation
// (which holds the sub-partition's FP64 pipe ~64 cycles on GB300): scale,
// axpby, axpbypcz, maxpy and the two-operand reductions ran 4-8% faster with
// four, while axpy, aypx and the one-operand reductions ran 3-5% slower
// (2^24-2^26 doubles), so those keep one.
constexpr int kMapU = 4;

template <int OP>
__host__ __device__ constexpr int map_unroll() {
  return (OP == OP_AXPY || OP == OP_AYPX) ? 1 : kMapU;
}

// Warp-contiguous trips: the grid's warps take chunks of 32 U consecutive
// elements round robin (lane l of a warp owns elements c + 32 u + l of its
// chunk c), so each trip of a warp touches one contiguous span of 256 U
// bytes per operand; the ragged end (fewer than 32 U elements) goes one
// element a thread.  `body(idx[U])` handles one trip, `tail(i)` one element.
template <int U, typename Body, typename Tail>
__device__ __forceinline__ void warp_chunks(int64_t n, Body body, Tail tail) {
  constexpr int64_t C = 32 * U;
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t full = n / C;
  for (int64_t c = gw; c < full; c += nw) {
    int64_t idx[U];
#pragma unroll
    for (int u = 0; u < U; u++) idx[u] = c * C + 32 * u + lane;
    body(idx);
  }
  for (int64_t i = full * C + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    tail(i);
}

template <int OP, bool FMA>
__global__ void __launch_bounds__(kBlock) k_map(int64_t n, double* __restrict__ y,
                                                const double* __restrict__ x,
                                                const double* __restrict__ w, double alpha,
                                                double beta, double gamma) {
  using R = MapReads<OP>;
  if constexpr (OP == OP_CHOP) {  // writes only the entries it zeroes
    const int64_t T = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += T)
      if (fabs(y[i]) < alpha) y[i] = 0.0;
    return;
  } else {
    constexpr int U = map_unroll<OP>();
    warp_chunks<U>(
        n,
        [&](const int64_t* idx) {
          double yv[U], xv[U], wv[U];
#pragma unroll
          for (int u = 0; u < U; u++) {
            yv[u] = R::y ? y[idx[u]] : 0.0;
            xv[u] = R::x ? x[idx[u]] : 0.0;
            wv[u] = R::w ? w[idx[u]] : 0.0;
          }
#pragma unroll
          for (int u = 0; u < U; u++)
            y[idx[u]] = map_value<OP, FMA>(yv[u], xv[u], wv[u], alpha, beta, gamma);
        },
        [&](int64_t j) {
          y[j] = map_value<OP, FMA>(R::y ? y[j] : 0.0, R::x ? x[j] : 0.0, R::w ? w[j] : 0.0,
                                    alpha, beta, gamma);
        });
  }
}

__global__ void __launch_bounds__(kBlock) k_swap(int64_t n, double* a, double* b) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    double t = a[i];
    a[i] = b[i];
    b[i] = t;
  }
}

static int map_grid(int64_t n, int unroll = kMapU) {
  int64_t g = (n + (int64_t)kBlock * unroll - 1) / ((int64_t)kBlock * unroll);
  int64_t cap = (int64_t)num_sms() * 16;
  return (int)std::max<int64_t>(1, std::min(g, cap));
}

template <int OP>
static int launch_map(cudaStream_t s, int64_t n, double* y, const double* x, const double* w,
                      double a, double b, double c) {
  if (n <= 0) return GP_OK;
  if (arith_mode() == kFma)
    k_map<OP, true><<<map_grid(n, map_unroll<OP>()), kBlock, 0, s>>>(n, y, x, w, a, b, c);
  else
    k_map<OP, false><<<map_grid(n, map_unroll<OP>()), kBlock, 0, s>>>(n, y, x, w, a, b, c);
  GP_CHECK_LAUNCH();
  return GP_OK;
}

// Host dispatch keeps the reference's scalar branch structure:
//   VecSet alpha == 0 zeroes (ported.mojo:259-263); VecAYPX alpha == 0 copies
//   and alpha == 1 is an AXPY (:285-294); VecAXPBY beta == 0 is a scale-and-set
//   and alpha == 0 a VecScale (:297-308).
int vec_map(cudaStream_t s, int op, int64_t n, double* y, const double* x, const double* w,
            double alpha, double beta, double gamma) {
  switch (op) {
    case OP_COPY:
      if (x == y || n <= 0) return GP_OK;
      GP_CUDA(cudaMemcpyAsync(y, x, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, s));
      return GP_OK;
    case OP_ZERO:
      return launch_map<OP_ZERO>(s, n, y, x, w, 0, 0, 0);
    case OP_SET:
      if (alpha == 0.0) return launch_map<OP_ZERO>(s, n, y, x, w, 0, 0, 0);
      return launch_map<OP_SET>(s, n, y, x, w, alpha, 0, 0);
    case OP_SCALESET: return launch_map<OP_SCALESET>(s, n, y, x, w, alpha, 0, 0);
    case OP_DIVS: return launch_map<OP_DIVS>(s, n, y, x, w, alpha, 0, 0);
    case OP_SCALE: return launch_map<OP_SCALE>(s, n, y, x, w, alpha, 0, 0);
    case OP_SHIFT: return launch_map<OP_SHIFT>(s, n, y, x, w, alpha, 0, 0);
    case OP_AXPY: return launch_map<OP_AXPY>(s, n, y, x, w, alpha, 0, 0);
    case OP_AYPX:
      if (alpha == 0.0) return vec_map(s, OP_COPY, n, y, x, w, 0, 0, 0);
      if (alpha == 1.0) return launch_map<OP_AXPY>(s, n, y, x, w, alpha, 0, 0);
      return launch_map<OP_AYPX>(s, n, y, x, w, alpha, 0, 0);
    case OP_AXPBY:
      if (beta == 0.0) return launch_map<OP_SCALESET>(s, n, y, x, w, alpha, 0, 0);
      if (alpha == 0.0) return launch_map<OP_SCALE>(s, n, y, x, w, beta, 0, 0);
      return launch_map<OP_AXPBY>(s, n, y, x, w, alpha, beta, 0);
    case OP_AXPBYPCZ: return launch_map<OP_AXPBYPCZ>(s, n, y, x, w, alpha, beta, gamma);
    case OP_WAXPY: return launch_map<OP_WAXPY>(s, n, y, x, w, alpha, 0, 0);
    case OP_PMULT: return launch_map<OP_PMULT>(s, n, y, x, w, 0, 0, 0);
    case OP_PDIV: return launch_map<OP_PDIV>(s, n, y, x, w, 0, 0, 0);
    case OP_PMIN: return launch_map<OP_PMIN>(s, n, y, x, w, 0, 0, 0);
    case OP_PMAX: return launch_map<OP_PMAX>(s, n, y, x, w, 0, 0, 0);
    case OP_PMAXABS: return launch_map<OP_PMAXABS>(s, n, y, x, w, 0, 0, 0);
    case OP_RECIP: return launch_map<OP_RECIP>(s, n, y, x, w, 0, 0, 0);
    case OP_EXP: return launch_map<OP_EXP>(s, n, y, x, w, 0, 0, 0);
    case OP_LOG: return launch_map<OP_LOG>(s, n, y, x, w, 0, 0, 0);
    case OP_SQRTABS: return launch_map<OP_SQRTABS>(s, n, y, x, w, 0, 0, 0);
    case OP_ABS: return launch_map<OP_ABS>(s, n, y, x, w, 0, 0, 0);
    case OP_CHOP: return launch_map<OP_CHOP>(s, n, y, x, w, alpha, 0, 0);
    case OP_SWAP:
      if (n <= 0) return GP_OK;
      k_swap<<<map_grid(n, 1), kBlock, 0, s>>>(n, y, const_cast<double*>(x));
      GP_CHECK_LAUNCH();
      return GP_OK;
  }
  set_error("vec_map: unknown op");
  return GP_ERR_ARG;
}

// ------------------------------------------------------------------ MAXPY
// y += sum_k alpha_k x_k, with the k-sum done per element in ascending k
// (simdvec.mojo:503-518 runs k outermost; each element sees the same sequence
// of rounded updates, so one pass over all k vectors is bit-identical).
constexpr int kMaxpyChunk = 32;
struct MaxpyArgs {
  const double* x[kMaxpyChunk];
  double a[kMaxpyChunk];
  int nv;
};

template <bool FMA>
__global__ void __launch_bounds__(kBlock) k_maxpy(int64_t n, double* __restrict__ y, MaxpyArgs args) {
  // kMapU elements a trip: their k-th loads go out together and their
  // update chains interleave
  warp_chunks<kMapU>(
      n,
      [&](const int64_t* idx) {
        double v[kMapU];
#pragma unroll
        for (int u = 0; u < kMapU; u++) v[u] = y[idx[u]];
        for (int k = 0; k < args.nv; k++) {
          const double* __restrict__ xk = args.x[k];
          double t[kMapU];
#pragma unroll
          for (int u = 0; u < kMapU; u++) t[u] = xk[idx[u]];
#pragma unroll
          for (int u = 0; u < kMapU; u++) v[u] = madd<FMA>(args.a[k], t[u], v[u]);
        }
#pragma unroll
        for (int u = 0; u < kMapU; u++) y[idx[u]] = v[u];
      },
      [&](int64_t j) {
        double v = y[j];
        for (int k = 0; k < args.nv; k++) v = madd<FMA>(args.a[k], args.x[k][j], v);
        y[j] = v;
      });
}

int vec_maxpy(cudaStream_t s, int64_t n, double* y, int nv, const double* alpha,
              const double* const* xs) {
  if (n <= 0) return GP_OK;
  for (int k0 = 0; k0 < nv; k0 += kMaxpyChunk) {
    MaxpyArgs args;
    args.nv = std::min(kMaxpyChunk, nv - k0);
    for (int k = 0; k < args.nv; k++) {
      args.x[k] = xs[k0 + k];
      args.a[k] = alpha[k0 + k];
    }
    if (arith_mode() == kFma)
      k_maxpy<true><<<map_grid(n), kBlock, 0, s>>>(n, y, args);
    else
      k_maxpy<false><<<map_grid(n), kBlock, 0, s>>>(n, y, args);
    GP_CHECK_LAUNCH();
  }
  return GP_OK;
}

// ------------------------------------------------------------------ reductions
template <int OP, bool FMA>
__global__ void __launch_bounds__(kRedBlock) k_reduce(int64_t n, const double* __restrict__ x,
                                                      const double* __restrict__ y, RedSlot slot,
                                                      double* out) {
  constexpr int NR = (OP == RED_DOTNORM2) ? 2 : 1;
  double v[NR];
#pragma unroll
  for (int r = 0; r < NR; r++) v[r] = 0.0;
  constexpr bool RY = OP == RED_DOT || OP == RED_DOTNORM2;
  auto fold = [&](double a, double b) {
    if constexpr (OP == RED_DOT) {
      v[0] = madd<FMA>(a, b, v[0]);
    } else if constexpr (OP == RED_NORM2SQ) {
      v[0] = madd<FMA>(a, a, v[0]);
    } else if constexpr (OP == RED_ASUM) {
      v[0] = add(v[0], fabs(a));
    } else if constexpr (OP == RED_SUM) {
      v[0] = add(v[0], a);
    } else if constexpr (OP == RED_DOTNORM2) {
      v[0] = madd<FMA>(a, b, v[0]);
      v[1] = madd<FMA>(a, a, v[1]);
    }
  };
  // each thread folds its elements in a fixed order (warp-contiguous trips,
  // then the ragged end); the loads of a trip go out before its folds
  constexpr int U = RY ? kMapU : 1;
  warp_chunks<U>(
      n,
      [&](const int64_t* idx) {
        double a[U], b[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
          a[u] = x[idx[u]];
          b[u] = RY ? y[idx[u]] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < U; u++) fold(a[u], b[u]);
      },
      [&](int64_t j) { fold(x[j], RY ? y[j] : 0.0); });
  double tot[NR];
  if (grid_finish<NR>(v, slot, tot) && threadIdx.x == 0) {
#pragma unroll
    for (int r = 0; r < NR; r++) out[r] = tot[r];
  }
}

// max |x_i| with the first NaN adopted (simdvec.mojo:476-488), or, for the
// pointwise-divide form, max |x_i / y_i| with x_i where y_i == 0 (:491-500).
// Per-block results go to partials; the last block combines them.
template <bool DIVIDE>
__global__ void __launch_bounds__(kRedBlock) k_maxabs(int64_t n, const double* __restrict__ x,
                                                      const double* __restrict__ y, RedSlot slot,
                                                      double* out) {
  __shared__ double sh[kRedBlock];
  __shared__ bool last;
  double m = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    double t;
    if constexpr (DIVIDE) {
      double yi = y[i];
      t = fabs(yi == 0.0 ? x[i] : div_(x[i], yi));
      if (t > m) m = t;  // NaN never adopted in this form
    } else {
      t = fabs(x[i]);
      if (t > m || t != t) m = (m != m) ? m : t;  // NaN is sticky
    }
  }
  auto comb = [](double a, double b) {
    if (DIVIDE) return b > a ? b : a;
    if (a != a) return a;
    if (b != b) return b;
    return b > a ? b : a;
  };
  sh[threadIdx.x] = m;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] = comb(sh[threadIdx.x], sh[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    slot.partials[blockIdx.x] = sh[0];
    last = atomic_add_acq_rel(slot.ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  if (threadIdx.x == 0) {
    double r = 0.0;
    for (int b = 0; b < (int)gridDim.x; b++) r = comb(r, __ldcg(&slot.partials[b]));
    out[0] = r;
    *slot.ticket = 0u;
  }
}

// the ordered (reference-order) kernel for each reduction op
constexpr int ORD_OF_RED_DOT = ORD_DOT, ORD_OF_RED_NORM2SQ = ORD_NRM, ORD_OF_RED_ASUM = ORD_ASUM,
              ORD_OF_RED_SUM = ORD_SUM, ORD_OF_RED_DOTNORM2 = ORD_DOTNRM;

int vec_reduce(cudaStream_t s, int op, int64_t n, const double* x, const double* y,
               double* out_host) {
  Scratch* sc;
  GP_TRY(scratch_get(&sc, 0));
  int nr = (op == RED_DOTNORM2) ? 2 : 1;
  if (n <= 0) {
    for (int r = 0; r < nr; r++) out_host[r] = 0.0;
    return GP_OK;
  }
  int g = red_grid(n);
  const bool f = arith_mode() == kFma;
  const bool ordered = arith_mode() == kOrdered;
#define RED_LAUNCH(OPC)                                                              \
  if (ordered)                                                                       \
    k_ord_red<ORD_OF_##OPC><<<kOrdChains, 32, 0, s>>>(nullptr, 1, n, DRef::of(x),    \
                                                    DRef::of(y), sc->slot, sc->d_out, \
                                                    nullptr, sc->d_out + 1);          \
  else if (f)                                                                        \
    k_reduce<OPC, true><<<g, kRedBlock, 0, s>>>(n, x, y, sc->slot, sc->d_out);        \
  else                                                                               \
    k_reduce<OPC, false><<<g, kRedBlock, 0, s>>>(n, x, y, sc->slot, sc->d_out);
  switch (op) {
    case RED_DOT: RED_LAUNCH(RED_DOT); break;
    case RED_NORM2SQ: RED_LAUNCH(RED_NORM2SQ); break;
    case RED_ASUM: RED_LAUNCH(RED_ASUM); break;
    case RED_SUM: RED_LAUNCH(RED_SUM); break;
    case RED_DOTNORM2: RED_LAUNCH(RED_DOTNORM2); break;
    case RED_NORMINF:
      k_maxabs<false><<<g, kRedBlock, 0, s>>>(n, x, y, sc->slot, sc->d_out);
      break;
    default: set_error("vec_reduce: unknown op"); return GP_ERR_ARG;
  }
#undef RED_LAUNCH
  GP_CHECK_LAUNCH();
  GP_CUDA(cudaMemcpyAsync(sc->h_out, sc->d_out, nr * sizeof(double), cudaMemcpyDeviceToHost, s));
  GP_CUDA(cudaStreamSynchronize(s));
  for (int r = 0; r < nr; r++) out_host[r] = sc->h_out[r];
  return GP_OK;
}

// The reduction kernels of vec_reduce with caller-supplied scratch and a
// device result (nothing allocated, nothing synchronised); grid capped at
// max_grid partial slots per value.
int vec_reduce_into(cudaStream_t s, int op, int64_t n, const double* x, const double* y,
                    RedSlot slot, int max_grid, double* out_dev) {
  const int nr = op == RED_DOTNORM2 ? 2 : 1;
  if (n <= 0) {
    GP_CUDA(cudaMemsetAsync(out_dev, 0, nr * sizeof(double), s));
    return GP_OK;
  }
  const int g = std::min(red_grid(n), max_grid);
  const bool f = arith_mode() == kFma;
#define RED_LAUNCH(OPC)                                                     \
  if (f)                                                                    \
    k_reduce<OPC, true><<<g, kRedBlock, 0, s>>>(n, x, y, slot, out_dev);    \
  else                                                                      \
    k_reduce<OPC, false><<<g, kRedBlock, 0, s>>>(n, x, y, slot, out_dev);
  switch (op) {
    case RED_DOT: RED_LAUNCH(RED_DOT); break;
    case RED_NORM2SQ: RED_LAUNCH(RED_NORM2SQ); break;
    case RED_ASUM: RED_LAUNCH(RED_ASUM); break;
    case RED_SUM: RED_LAUNCH(RED_SUM); break;
    case RED_DOTNORM2: RED_LAUNCH(RED_DOTNORM2); break;
    case RED_NORMINF: k_maxabs<false><<<g, kRedBlock, 0, s>>>(n, x, y, slot, out_dev); break;
    default: set_error("vec_reduce: unknown op"); return GP_ERR_ARG;
  }
#undef RED_LAUNCH
  GP_CHECK_LAUNCH();
  return GP_OK;
}

int vec_max_pointwise_divide(cudaStream_t s, int64_t n, const double* x, const double* y,
                             double* out_host) {
  Scratch* sc;
  GP_TRY(scratch_get(&sc, 0));
  if (n <= 0) {
    *out_host = 0.0;
    return GP_OK;
  }
  k_maxabs<true><<<red_grid(n), kRedBlock, 0, s>>>(n, x, y, sc->slot, sc->d_out);
  GP_CHECK_LAUNCH();
  GP_CUDA(cudaMemcpyAsync(sc->h_out, sc->d_out, sizeof(double), cudaMemcpyDeviceToHost, s));
  GP_CUDA(cudaStreamSynchronize(s));
  *out_host = sc->h_out[0];
  return GP_OK;
}

// VecMax/VecMin (ported.mojo:165-196): the first index attaining the extreme,
// strict comparison, so NaN entries never win; when x[0] itself is NaN the
// scan never moves off it and the result is (NaN, 0).
template <bool MAX>
__global__ void __launch_bounds__(kRedBlock) k_minmax(int64_t n, const double* __restrict__ x,
                                                      RedSlot slot, double* out,
                                                      long long* oidx) {
  __shared__ double sv[kRedBlock];
  __shared__ long long si[kRedBlock];
  __shared__ bool last;
  double bv = 0.0;
  long long bi = -1;
  auto better = [](double av, long long ai, double bv_, long long bi_) {
    // is (av, ai) better than (bv_, bi_)?
    if (ai < 0) return false;
    if (bi_ < 0) return true;
    if (MAX ? (av > bv_) : (av < bv_)) return true;
    if (av == bv_ && ai < bi_) return true;
    return false;
  };
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    double v = x[i];
    if (v != v) continue;
    if (better(v, i, bv, bi)) {
      bv = v;
      bi = i;
    }
  }
  sv[threadIdx.x] = bv;
  si[threadIdx.x] = bi;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o && better(sv[threadIdx.x + o], si[threadIdx.x + o], sv[threadIdx.x],
                                  si[threadIdx.x])) {
      sv[threadIdx.x] = sv[threadIdx.x + o];
      si[threadIdx.x] = si[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    slot.partials[blockIdx.x] = sv[0];
    slot.partials[slot.stride + blockIdx.x] = __longlong_as_double(si[0]);
    last = atomic_add_acq_rel(slot.ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  if (threadIdx.x == 0) {
    double rv = 0.0;
    long long ri = -1;
    for (int b = 0; b < (int)gridDim.x; b++) {
      double v = __ldcg(&slot.partials[b]);
      long long ii = __double_as_longlong(__ldcg(&slot.partials[slot.stride + b]));
      if (better(v, ii, rv, ri)) {
        rv = v;
        ri = ii;
      }
    }
    double x0 = x[0];
    if (x0 != x0) {
      rv = x0;
      ri = 0;
    }
    out[0] = rv;
    oidx[0] = ri;
    *slot.ticket = 0u;
  }
}

int vec_minmax(cudaStream_t s, int64_t n, const double* x, int is_max, long long* idx,
               double* val) {
  if (n <= 0) {
    *idx = -1;
    *val = is_max ? -1.7976931348623157e308 : 1.7976931348623157e308;
    return GP_OK;
  }
  Scratch* sc;
  GP_TRY(scratch_get(&sc, 0));
  int g = red_grid(n);
  if (is_max)
    k_minmax<true><<<g, kRedBlock, 0, s>>>(n, x, sc->slot, sc->d_out, sc->d_idx);
  else
    k_minmax<false><<<g, kRedBlock, 0, s>>>(n, x, sc->slot, sc->d_out, sc->d_idx);
  GP_CHECK_LAUNCH();
  GP_CUDA(cudaMemcpyAsync(sc->h_out, sc->d_out, sizeof(double), cudaMemcpyDeviceToHost, s));
  GP_CUDA(cudaMemcpyAsync(sc->h_idx, sc->d_idx, sizeof(long long), cudaMemcpyDeviceToHost, s));
  GP_CUDA(cudaStreamSynchronize(s));
  *val = sc->h_out[0];
  *idx = sc->h_idx[0];
  return GP_OK;
}

}  // namespace gp
