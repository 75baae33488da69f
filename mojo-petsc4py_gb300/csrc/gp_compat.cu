// The reference's host C ABI (src/capi.mojo:32-424) on the GPU.
//
// Each mp_* entry keeps the reference's name, argument order and meaning:
// host pointers, int64 indices, double scalars, caller-owned buffers.  It
// copies its inputs to device buffers kept per host thread, runs the device
// kernels of this library, and copies the outputs back before returning.
// The symbolic set-up entries (diagonal markers, ILU/IC patterns, the
// contiguous passes, RCM) are integer host analysis, as in the reference.
// Errors cannot be returned through the reference's void signatures; the
// status of the last call is available from mp_last_status() and the message
// from gp_last_error().
#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/gpetsc.h"
#include "gp_ksp.h"

namespace {

using gp::Csr;
using gp::DRef;
using gp::Pc;

thread_local int g_status = 0;

// grow-only device buffers, one set per host thread
struct Pool {
  std::vector<void*> buf;
  std::vector<size_t> cap;
  void* get(int slot, size_t bytes) {
    if ((int)buf.size() <= slot) {
      buf.resize(slot + 1, nullptr);
      cap.resize(slot + 1, 0);
    }
    if (cap[slot] < bytes || !buf[slot]) {
      if (buf[slot]) cudaFree(buf[slot]);
      buf[slot] = nullptr;
      size_t want = std::max<size_t>(bytes, 256);
      if (cudaMalloc(&buf[slot], want) != cudaSuccess) {
        cap[slot] = 0;
        buf[slot] = nullptr;
        return nullptr;
      }
      cap[slot] = want;
    }
    return buf[slot];
  }
};
thread_local Pool g_pool;

double* dbuf(int slot, int64_t n) {
  return static_cast<double*>(g_pool.get(slot, (size_t)std::max<int64_t>(n, 1) * 8));
}

// device copy of a host vector in pool slot `slot`
double* up(int slot, const double* h, int64_t n) {
  double* d = dbuf(slot, n);
  if (d && n > 0) cudaMemcpy(d, h, (size_t)n * 8, cudaMemcpyHostToDevice);
  return d;
}

void down(double* h, const double* d, int64_t n) {
  if (n > 0) cudaMemcpy(h, d, (size_t)n * 8, cudaMemcpyDeviceToHost);
}

int finish_status(int st) {
  if (st == GP_OK) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      gp::set_error(std::string("CUDA: ") + cudaGetErrorString(e));
      st = GP_ERR_CUDA;
    }
  }
  g_status = st;
  return st;
}

// a temporary device CSR from the reference's host arrays
struct TmpCsr {
  Csr* A = nullptr;
  ~TmpCsr() { gp::csr_destroy(A); }
  int make(const int64_t* irow, const int64_t* icol, const double* data, int64_t nrow,
           int64_t ncols) {
    const int64_t nnz = nrow > 0 ? irow[nrow] - irow[0] : 0;
    if (nrow > 0 && irow[0] != 0) {
      gp::set_error("row starts must begin at 0");
      return GP_ERR_ARG;
    }
    if (ncols < 0) {  // MatMult takes its width from the column indices
      ncols = nrow;
      for (int64_t j = 0; j < nnz; j++) ncols = std::max<int64_t>(ncols, icol[j] + 1);
    }
    static const int64_t zero = 0;
    return gp::csr_create(&A, nrow, ncols, nnz, nrow > 0 ? irow : &zero, icol, data, nullptr);
  }
};

int vmap(int op, double* w, const double* x, const double* y, int64_t n, double a = 0,
         double b = 0, double c = 0, bool w_in = false) {
  if (n <= 0) return GP_OK;
  double* dx = x ? up(0, x, n) : nullptr;
  double* dy = y ? up(1, y, n) : nullptr;
  double* dw = w_in ? up(2, w, n) : dbuf(2, n);
  if ((x && !dx) || (y && !dy) || !dw) {
    gp::set_error("device allocation failed");
    return GP_ERR_CUDA;
  }
  int st = gp::vec_map(nullptr, op, n, dw, dx, dy, a, b, c);
  if (st) return st;
  down(w, dw, n);
  return GP_OK;
}

// in-place map on one vector
int vself(int op, double* x, int64_t n, double a = 0) {
  return vmap(op, x, nullptr, nullptr, n, a, 0, 0, true);
}

double vreduce(int op, const double* x, const double* y, int64_t n, double* second = nullptr) {
  double out[2] = {0, 0};
  if (n > 0) {
    double* dx = up(0, x, n);
    double* dy = y ? up(1, y, n) : nullptr;
    g_status = gp::vec_reduce(nullptr, op, n, dx, dy, out);
  }
  if (second) *second = out[1];
  return out[0];
}

std::vector<int> to_i32(const int64_t* p, int64_t n) {
  std::vector<int> v((size_t)std::max<int64_t>(n, 0));
  for (int64_t i = 0; i < n; i++) v[i] = (int)p[i];
  return v;
}

// Pattern of a reference-layout factor (ILU: bdiag of n+1; IC: bi = b->i of
// n+1 and bdiag of n+1 with the diagonal slot last in every row).
gp::FactorPattern pattern(const int64_t* bi, const int64_t* bj, const int64_t* bdiag,
                          const int64_t* r, int64_t n, bool ilu) {
  gp::FactorPattern P;
  P.bi = to_i32(bi, n + 1);
  P.bdiag = to_i32(bdiag, n + 1);
  const int64_t nslots = ilu ? (n ? bdiag[0] + 1 : 0) : (n ? bi[n] : 0);
  P.bj = to_i32(bj, std::max<int64_t>(nslots, 1));
  P.nnz = (int)nslots;
  P.r = to_i32(r, n);
  P.ic.assign(n, 0);
  for (int64_t i = 0; i < n; i++) P.ic[P.r[i]] = (int)i;
  return P;
}

}  // namespace

extern "C" {

int mp_last_status(void) { return g_status; }

// ------------------------------------------------------------ Mat
void mp_mat_mult(const double* x, double* y, const int64_t* irow, const int64_t* icol,
                 const double* data, int64_t nrow) {
  TmpCsr t;
  int st = t.make(irow, icol, data, nrow, -1);
  if (!st && nrow > 0) {
    double* dx = up(0, x, t.A->ncols);
    double* dy = dbuf(1, nrow);
    st = gp::spmv(nullptr, t.A, DRef::of(dx), DRef::of(dy));
    if (!st) down(y, dy, nrow);
  }
  finish_status(st);
}

void mp_mat_mult_add(const double* x, double* y, const int64_t* irow, const int64_t* icol,
                     const double* data, int64_t nrow) {
  TmpCsr t;
  int st = t.make(irow, icol, data, nrow, -1);
  if (!st && nrow > 0) {
    double* dx = up(0, x, t.A->ncols);
    double* dv = up(1, y, nrow);
    double* dy = dbuf(2, nrow);
    st = gp::spmv_add(nullptr, t.A, dx, dv, dy);
    if (!st) down(y, dy, nrow);
  }
  finish_status(st);
}

void mp_mat_mult_transpose(const double* x, double* y, const int64_t* irow, const int64_t* icol,
                           const double* data, int64_t nrow, int64_t ncols) {
  TmpCsr t;
  int st = t.make(irow, icol, data, nrow, ncols);
  if (!st && ncols > 0) {
    double* dx = up(0, x, std::max<int64_t>(nrow, 1));
    double* dy = dbuf(1, ncols);
    st = gp::spmv_t(nullptr, t.A, dx, dy);
    if (!st) down(y, dy, ncols);
  }
  finish_status(st);
}

void mp_mat_get_diagonal(double* diag, const int64_t* irow, const int64_t* icol,
                         const double* data, int64_t nrow) {
  TmpCsr t;
  int st = t.make(irow, icol, data, nrow, -1);
  if (!st && nrow > 0) {
    double* dd = dbuf(0, nrow);
    st = gp::mat_diagonal(nullptr, t.A, dd);
    if (!st) down(diag, dd, nrow);
  }
  finish_status(st);
}

void mp_mat_scale(double* data, int64_t nnz, double alpha) {
  finish_status(vself(gp::OP_SCALE, data, nnz, alpha));
}

void mp_mat_zero_entries(double* data, int64_t nnz) {
  finish_status(vmap(gp::OP_ZERO, data, nullptr, nullptr, nnz));
}

// ------------------------------------------------------------ Vec
void mp_vec_pointwise_mult(double* w, const double* x, const double* y, int64_t n) {
  finish_status(vmap(gp::OP_PMULT, w, x, y, n));
}
void mp_vec_pointwise_divide(double* w, const double* x, const double* y, int64_t n) {
  finish_status(vmap(gp::OP_PDIV, w, x, y, n));
}
void mp_vec_pointwise_min(double* w, const double* x, const double* y, int64_t n) {
  finish_status(vmap(gp::OP_PMIN, w, x, y, n));
}
void mp_vec_pointwise_max(double* w, const double* x, const double* y, int64_t n) {
  finish_status(vmap(gp::OP_PMAX, w, x, y, n));
}
void mp_vec_pointwise_max_abs(double* w, const double* x, const double* y, int64_t n) {
  finish_status(vmap(gp::OP_PMAXABS, w, x, y, n));
}

// VecNorm_Seq (src/ported.mojo:113-135)
void mp_vec_norm(const double* x, int64_t ntype, double* z, int64_t n) {
  double z0 = 0.0, z1 = 0.0;
  g_status = 0;
  if (n) {
    if (ntype == 1 || ntype == 2) {
      z0 = __builtin_sqrt(vreduce(gp::RED_NORM2SQ, x, nullptr, n));
    } else if (ntype == 4) {
      z0 = vreduce(gp::RED_ASUM, x, nullptr, n);
      z1 = __builtin_sqrt(vreduce(gp::RED_NORM2SQ, x, nullptr, n));
    } else if (ntype == 3) {
      z0 = vreduce(gp::RED_NORMINF, x, nullptr, n);
    } else if (ntype == 0) {
      z0 = vreduce(gp::RED_ASUM, x, nullptr, n);
    }
  }
  z[0] = z0;
  if (ntype == 4) z[1] = z1;
  finish_status(g_status);
}

void mp_vec_dot(const double* x, const double* y, double* val, int64_t n) {
  val[0] = vreduce(gp::RED_DOT, x, y, n);
  finish_status(g_status);
}
void mp_vec_tdot(const double* x, const double* y, double* val, int64_t n) {
  val[0] = vreduce(gp::RED_DOT, y, x, n);
  finish_status(g_status);
}
void mp_vec_dot_norm2(const double* x, const double* y, double* sval, double* rval, int64_t n) {
  double q = 0.0;
  sval[0] = vreduce(gp::RED_DOTNORM2, x, y, n, &q);
  rval[0] = q;
  finish_status(g_status);
}
void mp_vec_sum(const double* x, double* val, int64_t n) {
  val[0] = vreduce(gp::RED_SUM, x, nullptr, n);
  finish_status(g_status);
}
void mp_vec_mean(const double* x, double* val, int64_t n) {
  val[0] = vreduce(gp::RED_SUM, x, nullptr, n) / (double)n;
  finish_status(g_status);
}

static void minmax(const double* x, int64_t* idx, double* z, int64_t n, int is_max) {
  long long i = -1;
  double v = 0.0;
  int st = GP_OK;
  if (n > 0) {
    double* dx = up(0, x, n);
    st = gp::vec_minmax(nullptr, n, dx, is_max, &i, &v);
  } else {
    v = is_max ? -1.7976931348623157e308 : 1.7976931348623157e308;
  }
  idx[0] = i;
  z[0] = v;
  finish_status(st);
}
void mp_vec_max(const double* x, int64_t* idx, double* z, int64_t n) { minmax(x, idx, z, n, 1); }
void mp_vec_min(const double* x, int64_t* idx, double* z, int64_t n) { minmax(x, idx, z, n, 0); }

// VecNormalize_Seq: divide by the 2-norm when it is positive
void mp_vec_normalize(double* x, double* v, int64_t n) {
  double z = n ? __builtin_sqrt(vreduce(gp::RED_NORM2SQ, x, nullptr, n)) : 0.0;
  int st = g_status;
  if (!st && z > 0.0) st = vself(gp::OP_DIVS, x, n, z);
  v[0] = z;
  finish_status(st);
}

void mp_vec_reciprocal(double* x, int64_t n) { finish_status(vself(gp::OP_RECIP, x, n)); }
void mp_vec_exp(double* x, int64_t n) { finish_status(vself(gp::OP_EXP, x, n)); }
void mp_vec_log(double* x, int64_t n) { finish_status(vself(gp::OP_LOG, x, n)); }
void mp_vec_sqrtabs(double* x, int64_t n) { finish_status(vself(gp::OP_SQRTABS, x, n)); }
void mp_vec_chop(double* x, int64_t n, double tol) {
  finish_status(vself(gp::OP_CHOP, x, n, tol));
}
void mp_vec_abs(double* x, int64_t n) { finish_status(vself(gp::OP_ABS, x, n)); }
void mp_vec_conjugate(double* x, int64_t n) {
  (void)x;
  (void)n;
  finish_status(GP_OK);
}
void mp_vec_copy(const double* x, double* y, int64_t n) {
  finish_status(vmap(gp::OP_COPY, y, x, nullptr, n));
}
void mp_vec_swap(double* x, double* y, int64_t n) {
  int st = GP_OK;
  if (n > 0) {
    double* dx = up(0, x, n);
    double* dy = up(1, y, n);
    st = gp::vec_map(nullptr, gp::OP_SWAP, n, dx, dy, nullptr, 0, 0, 0);
    if (!st) {
      down(x, dx, n);
      down(y, dy, n);
    }
  }
  finish_status(st);
}
void mp_vec_set(double* x, double alpha, int64_t n) {
  finish_status(vmap(gp::OP_SET, x, nullptr, nullptr, n, alpha));
}
void mp_vec_zero_entries(double* x, int64_t n) {
  finish_status(vmap(gp::OP_ZERO, x, nullptr, nullptr, n));
}
void mp_vec_scale(double* x, double alpha, int64_t n) {
  finish_status(vself(gp::OP_SCALE, x, n, alpha));
}
void mp_vec_shift(double* x, double alpha, int64_t n) {
  finish_status(vself(gp::OP_SHIFT, x, n, alpha));
}
void mp_vec_axpy(double* y, double alpha, const double* x, int64_t n) {
  finish_status(vmap(gp::OP_AXPY, y, x, nullptr, n, alpha, 0, 0, true));
}
void mp_vec_aypx(double* y, double alpha, const double* x, int64_t n) {
  finish_status(vmap(gp::OP_AYPX, y, x, nullptr, n, alpha, 0, 0, true));
}
void mp_vec_axpby(double* y, double alpha, double beta, const double* x, int64_t n) {
  finish_status(vmap(gp::OP_AXPBY, y, x, nullptr, n, alpha, beta, 0, true));
}
void mp_vec_axpbypcz(double* z, double alpha, double beta, double gamma, const double* x,
                     const double* y, int64_t n) {
  finish_status(vmap(gp::OP_AXPBYPCZ, z, x, y, n, alpha, beta, gamma, true));
}
void mp_vec_waxpy(double* w, double alpha, const double* x, const double* y, int64_t n) {
  finish_status(vmap(gp::OP_WAXPY, w, x, y, n, alpha));
}
// VecMAXPY_Seq: x is an array of vector addresses
void mp_vec_maxpy(double* y, int64_t nv, const double* alpha, const int64_t* x, int64_t n) {
  int st = GP_OK;
  if (n > 0 && nv > 0) {
    double* dy = up(0, y, n);
    std::vector<const double*> xs(nv);
    for (int64_t k = 0; k < nv; k++)
      xs[k] = up(1 + (int)k, reinterpret_cast<const double*>((intptr_t)x[k]), n);
    st = gp::vec_maxpy(nullptr, n, dy, (int)nv, alpha, xs.data());
    if (!st) down(y, dy, n);
  }
  finish_status(st);
}
void mp_vec_max_pointwise_divide(const double* x, const double* y, double* rval, int64_t n) {
  double r = 0.0;
  int st = GP_OK;
  if (n > 0) st = gp::vec_max_pointwise_divide(nullptr, n, up(0, x, n), up(1, y, n), &r);
  rval[0] = r;
  finish_status(st);
}

// ------------------------------------------------------------ PC and factors

// MatGetDiagonalMarkers_SeqAIJ (src/ported.mojo:354-377): slot of a_ii, or
// the row end when absent; returns 1 when every row has its diagonal.
int64_t mp_mat_get_diagonal_markers(const int64_t* irow, const int64_t* icol, int64_t* diag,
                                    int64_t nrow) {
  int64_t dense = 1;
  for (int64_t i = 0; i < nrow; i++) {
    diag[i] = irow[i + 1];
    for (int64_t j = irow[i]; j < irow[i + 1]; j++)
      if (icol[j] == i) {
        diag[i] = j;
        break;
      }
    if (diag[i] == irow[i + 1]) dense = 0;
  }
  finish_status(GP_OK);
  return dense;
}

void mp_pc_jacobi_setup(double* diag, int64_t jtype, int64_t useabs, int64_t fixdiag,
                        double scale, const int64_t* irow, const int64_t* icol,
                        const double* data, int64_t nrow, double* didx) {
  TmpCsr t;
  int st = t.make(irow, icol, data, nrow, nrow);
  if (!st && nrow > 0) {
    double* dd = dbuf(0, nrow);
    st = gp::jacobi_fill(t.A, (int)jtype, 0, (int)useabs, (int)fixdiag, scale, dd, nullptr);
    if (!st) down(diag, dd, nrow);
    if (!st && jtype == 2) {  // the reference leaves the true diagonal in didx
      double* dg = dbuf(1, nrow);
      st = gp::mat_diagonal(nullptr, t.A, dg);
      if (!st) down(didx, dg, nrow);
    }
  }
  finish_status(st);
}

void mp_pc_jacobi_setup_symmetric(double* diagsqrt, int64_t jtype, const int64_t* irow,
                                  const int64_t* icol, const double* data, int64_t nrow) {
  TmpCsr t;
  int st = t.make(irow, icol, data, nrow, nrow);
  if (!st && nrow > 0) {
    double* dd = dbuf(0, nrow);
    st = gp::jacobi_fill(t.A, (int)jtype, 1, 0, 0, 1.0, dd, nullptr);
    if (!st) down(diagsqrt, dd, nrow);
  }
  finish_status(st);
}

void mp_pc_jacobi_apply(double* y, const double* x, const double* diag, int64_t n) {
  finish_status(vmap(gp::OP_PMULT, y, x, diag, n));
}

void mp_pc_sor_apply(const double* x, double* y, const int64_t* irow, const int64_t* icol,
                     const double* data, const int64_t* dmark, double* idiag, double* mdiag,
                     double* t, double omega, double fshift, int64_t flag, int64_t nrow) {
  (void)dmark;  // the device computes the same first-occurrence markers
  TmpCsr tc;
  int st = tc.make(irow, icol, data, nrow, nrow);
  Pc* pc = nullptr;
  gp::pc_create(&pc);
  if (!st && nrow > 0) {
    pc->opt.type = gp::PC_SOR;
    pc->opt.omega = omega;
    pc->opt.fshift = fshift;
    pc->opt.sor_flag = (int)flag;
    st = gp::pc_setup(pc, tc.A, nullptr);
    double* dx = st ? nullptr : up(0, x, nrow);
    double* dy = st ? nullptr : dbuf(1, nrow);
    if (!st) st = gp::pc_apply(pc, DRef::of(dx), DRef::of(dy), nullptr);
    if (!st) st = gp::pc_check(pc, nullptr);
    if (!st) {
      down(y, dy, nrow);
      down(idiag, pc->idiag, nrow);
      down(mdiag, pc->mdiag, nrow);
      if (flag & gp::kSorForward) down(t, pc->t, nrow);
    }
  }
  gp::pc_destroy(pc);
  finish_status(st);
}

static int factor_apply(int type, const double* b, double* x, const gp::FactorPattern& P,
                        const std::vector<int>& perm_c, const double* ba, int64_t n) {
  Pc* pc = nullptr;
  gp::pc_create(&pc);
  int st = gp::pc_import_factor(pc, type, P, perm_c, ba, nullptr, nullptr);
  if (!st) {
    double* db = up(0, b, n);
    double* dx = dbuf(1, n);
    st = gp::pc_apply(pc, DRef::of(db), DRef::of(dx), nullptr);
    if (!st) st = gp::pc_check(pc, nullptr);
    if (!st) down(x, dx, n);
  }
  gp::pc_destroy(pc);
  return st;
}

void mp_pc_ilu_apply(const double* b, double* x, double* tmp, const int64_t* bi,
                     const int64_t* bj, const double* ba, const int64_t* bdiag, const int64_t* r,
                     const int64_t* c, int64_t nrow) {
  (void)tmp;
  int st = GP_OK;
  if (nrow > 0) {
    gp::FactorPattern P = pattern(bi, bj, bdiag, r, nrow, true);
    st = factor_apply(gp::PC_ILU, b, x, P, to_i32(c, nrow), ba, nrow);
  }
  finish_status(st);
}

int64_t mp_pc_icc_apply(const double* b, double* x, const int64_t* ui, const int64_t* uj,
                        const double* ua, const int64_t* udiag, const int64_t* c,
                        double* scratch, int64_t nrow) {
  (void)scratch;
  int st = GP_OK;
  if (nrow > 0) {
    // the solve reads row i as ui[i] .. udiag[i]; b->i is ui
    gp::FactorPattern P = pattern(ui, uj, udiag, c, nrow, false);
    st = factor_apply(gp::PC_ICC, b, x, P, to_i32(c, nrow), ua, nrow);
  }
  finish_status(st);
  return 0;
}

int64_t mp_pc_ilu_numeric(double* ba, double* rtmp, const int64_t* irow, const int64_t* icol,
                          const double* data, const int64_t* bi, const int64_t* bj,
                          const int64_t* bdiag, const int64_t* r, const int64_t* ic, int64_t nrow) {
  (void)rtmp;
  (void)ic;
  if (nrow <= 0) {
    finish_status(GP_OK);
    return nrow ? 0 : bdiag[0] + 1;
  }
  TmpCsr t;
  int st = t.make(irow, icol, data, nrow, nrow);
  gp::FactorPattern P = pattern(bi, bj, bdiag, r, nrow, true);
  Pc* pc = nullptr;
  gp::pc_create(&pc);
  if (!st) st = gp::pc_import_factor(pc, gp::PC_ILU, P, P.r, nullptr, t.A, nullptr);
  if (!st) st = gp::pc_factor_numeric(pc, nullptr);
  if (!st) down(ba, pc->ba, P.nnz);
  gp::pc_destroy(pc);
  finish_status(st);
  return bdiag[0] + 1;
}

void mp_pc_icc_numeric(double* ua, double* rtmp, int64_t* il, int64_t* c2r, const int64_t* irow,
                       const int64_t* icol, const double* data, const int64_t* ui,
                       const int64_t* uj, const int64_t* udiag, const int64_t* r,
                       const int64_t* riip, int64_t nrow) {
  (void)rtmp;
  (void)il;
  (void)c2r;
  (void)riip;
  int st = GP_OK;
  if (nrow > 0) {
    TmpCsr t;
    st = t.make(irow, icol, data, nrow, nrow);
    gp::FactorPattern P = pattern(ui, uj, udiag, r, nrow, false);
    Pc* pc = nullptr;
    gp::pc_create(&pc);
    if (!st) st = gp::pc_import_factor(pc, gp::PC_ICC, P, P.r, nullptr, t.A, nullptr);
    if (!st) st = gp::pc_factor_numeric(pc, nullptr);
    if (!st) down(ua, pc->ba, P.nnz);
    gp::pc_destroy(pc);
  }
  finish_status(st);
}

// MatILUFactorSymbolic_SeqAIJ_ilu0 (src/factor.mojo:31-67): L rows copied in
// order, then U rows in reverse with the diagonal last.
int64_t mp_ilu_symbolic_ilu0(int64_t* bi, int64_t* bj, int64_t* bdiag, const int64_t* adiag,
                             const int64_t* irow, const int64_t* icol, int64_t nrow) {
  int64_t k = 0;
  bi[0] = 0;
  for (int64_t i = 0; i < nrow; i++) {
    const int64_t nz = adiag[i] - irow[i];
    bi[i + 1] = bi[i] + nz;
    for (int64_t j = 0; j < nz; j++) bj[k++] = icol[irow[i] + j];
  }
  bdiag[nrow] = bi[nrow] - 1;
  for (int64_t i = nrow - 1; i >= 0; i--) {
    const int64_t nz = irow[i + 1] - adiag[i] - 1;
    for (int64_t j = 0; j < nz; j++) bj[k++] = icol[adiag[i] + 1 + j];
    bj[k++] = i;
    bdiag[i] = bdiag[i + 1] + nz + 1;
  }
  finish_status(GP_OK);
  return k;
}

// Level-of-fill ILU pattern in the staging layout MatILUFactorSymbolic_SeqAIJ
// produces (src/factor.mojo:70-122): row i contiguous as its L columns, the
// diagonal, its U columns, with the levels in bjlvl and the L count in
// bdiag[i]; a negative return asks for a larger `cap`.
int64_t mp_ilu_symbolic(int64_t* bi, int64_t* bj, int64_t* bjlvl, int64_t* bdiag,
                        const int64_t* irow, const int64_t* icol, const int64_t* r,
                        const int64_t* ic, int64_t levels, int64_t cap, int64_t* scratch,
                        int64_t nrow) {
  (void)scratch;
  (void)ic;
  Csr A;
  A.n = A.ncols = (int)nrow;
  A.nnz = nrow ? irow[nrow] : 0;
  A.h_rowptr = to_i32(irow, nrow + 1);
  A.h_colind = to_i32(icol, A.nnz);
  std::vector<int> rr = to_i32(r, nrow), icv(nrow);
  for (int64_t i = 0; i < nrow; i++) icv[rr[i]] = (int)i;
  std::vector<std::vector<std::pair<int, int>>> rows;
  std::vector<int> nl;
  int st = gp::ilu_symbolic_rows(&A, (int)levels, rr, icv, rows, nl);
  A.h_rowptr.clear();
  if (st) {
    finish_status(st);
    return 0;
  }
  bi[0] = 0;
  bdiag[0] = 0;
  for (int64_t i = 0; i < nrow; i++) {
    const int64_t nzi = (int64_t)rows[i].size();
    if (bi[i] + nzi > cap) {
      finish_status(GP_OK);
      int64_t total = bi[i];
      for (int64_t q = i; q < nrow; q++) total += (int64_t)rows[q].size();
      return -total;
    }
    bi[i + 1] = bi[i] + nzi;
    bdiag[i] = nl[i];
    for (int64_t q = 0; q < nzi; q++) {
      bj[bi[i] + q] = rows[i][q].first;
      bjlvl[bi[i] + q] = rows[i][q].second;
    }
  }
  finish_status(GP_OK);
  return bi[nrow];
}

// PetscFreeSpaceContiguous_LU (src/factor.mojo:335-381): staged rows into the
// factor layout (L rows in order, U rows from the end, diagonal last).
void mp_ilu_contiguous_lu(const int64_t* bjsrc, int64_t* bi, int64_t* bdiag, int64_t* bj,
                          int64_t n) {
  std::vector<int64_t> start(n + 1), nl(n);
  for (int64_t i = 0; i <= n; i++) start[i] = bi[i];
  for (int64_t i = 0; i < n; i++) nl[i] = bdiag[i];
  const int64_t total = n ? start[n] : 0;
  int64_t ltot = 0;
  for (int64_t i = 0; i < n; i++) {
    bi[i] = ltot;
    for (int64_t q = 0; q < nl[i]; q++) bj[ltot + q] = bjsrc[start[i] + q];
    ltot += nl[i];
  }
  if (n) bi[n] = ltot;
  int64_t end = total;  // U rows of row 0 end the array
  for (int64_t i = 0; i < n; i++) {
    const int64_t nu = start[i + 1] - start[i] - nl[i] - 1;  // strict U count
    const int64_t base = end - nu - 1;
    for (int64_t q = 0; q < nu; q++) bj[base + q] = bjsrc[start[i] + nl[i] + 1 + q];
    bj[end - 1] = i;
    bdiag[i] = end - 1;
    end = base;
  }
  if (n) bdiag[n] = ltot - 1;
  finish_status(GP_OK);
}

// Level-of-fill IC pattern (src/factor.mojo:125-273): row k as its strict
// upper columns ascending, then the diagonal; udiag[k] is the diagonal slot.
int64_t mp_icc_symbolic(int64_t* ui, int64_t* uj, int64_t* ujlvl, int64_t* udiag,
                        const int64_t* irow, const int64_t* icol, const int64_t* r,
                        const int64_t* riip, int64_t levels, int64_t cap, int64_t* scratch,
                        int64_t nrow, int64_t scratchlen) {
  (void)scratch;
  (void)riip;
  const int64_t need_scratch = 6 * (nrow + 1) + 2 * cap;
  if (need_scratch > scratchlen) {
    finish_status(GP_OK);
    return -need_scratch;
  }
  Csr A;
  A.n = A.ncols = (int)nrow;
  A.nnz = nrow ? irow[nrow] : 0;
  A.h_rowptr = to_i32(irow, nrow + 1);
  A.h_colind = to_i32(icol, A.nnz);
  std::vector<int> rr = to_i32(r, nrow), icv(nrow);
  for (int64_t i = 0; i < nrow; i++) icv[rr[i]] = (int)i;
  std::vector<std::vector<std::pair<int, int>>> rows;
  int st = gp::icc_symbolic_rows(&A, (int)levels, rr, icv, rows);
  if (st) {
    finish_status(st);
    return 0;
  }
  int64_t total = 0;
  for (int64_t k = 0; k < nrow; k++) total += (int64_t)rows[k].size() + 1;
  if (total > cap) {
    finish_status(GP_OK);
    return -total;
  }
  int64_t pos = 0;
  ui[0] = 0;
  for (int64_t k = 0; k < nrow; k++) {
    for (auto& e : rows[k]) {
      uj[pos] = e.first;
      ujlvl[pos] = e.second;
      pos++;
    }
    uj[pos] = k;
    ujlvl[pos] = 0;
    udiag[k] = pos;
    pos++;
    ui[k + 1] = pos;
  }
  finish_status(GP_OK);
  return total;
}

// PetscFreeSpaceContiguous_Cholesky (src/factor.mojo:384-412)
void mp_icc_contiguous_cholesky(const int64_t* ujsrc, const int64_t* ui, const int64_t* udiag,
                                int64_t* bi, int64_t* bdiag, int64_t* bj, int64_t n) {
  for (int64_t row = 0; row < n; row++)
    for (int64_t j = ui[row]; j <= udiag[row]; j++) bj[j] = ujsrc[j];
  if (n) {
    bi[0] = 0;
    for (int64_t row = 0; row < n; row++) bi[row + 1] = udiag[row] + 1;
    bdiag[n] = bi[n];
  }
  finish_status(GP_OK);
}

void mp_ordering_rcm(int64_t* perm, int64_t* level, int64_t* visited, int64_t* queue,
                     const int64_t* irow, const int64_t* icol, int64_t nrow) {
  (void)queue;
  std::vector<int> rp = to_i32(irow, nrow + 1), ci = to_i32(icol, nrow ? irow[nrow] : 0), p;
  gp::rcm_order(rp, ci, (int)nrow, p);
  for (int64_t i = 0; i < nrow; i++) {
    perm[i] = p[i];
    level[i] = irow[i + 1] - irow[i];
    visited[i] = 1;
  }
  finish_status(GP_OK);
}

// ------------------------------------------------------------ KSP
// The pci/pcf blocks (src/ksp.mojo:25-30, filled by
// python/mojopetsc4py/PETSc/PC.py:495-547) name host buffers; the PC is
// rebuilt on the device from them for the duration of the call.
static int pc_from_block(Pc* pc, const int64_t* pci, const double* pcf, int64_t n, Csr* A,
                         TmpCsr& sor_mat) {
  const int64_t kind = pci[0];
  auto P = [&](int k) { return (const int64_t*)(intptr_t)pci[k]; };
  auto D = [&](int k) { return (const double*)(intptr_t)pci[k]; };
  if (kind == gp::PC_JACOBI) return gp::pc_import_jacobi(pc, (int)n, D(1), pci[2] ? D(2) : nullptr, nullptr);
  if (kind == gp::PC_SOR) {
    GP_TRY(sor_mat.make(P(1), P(2), D(3), n, n));
    pc->opt.type = gp::PC_SOR;
    pc->opt.omega = pcf[0];
    pc->opt.fshift = pcf[1];
    pc->opt.sor_flag = (int)pci[10];
    return gp::pc_setup(pc, sor_mat.A, nullptr);
  }
  if (kind == gp::PC_ILU) {
    gp::FactorPattern F = pattern(P(1), P(2), P(4), P(5), n, true);
    return gp::pc_import_factor(pc, gp::PC_ILU, F, to_i32(P(6), n), D(3), nullptr, nullptr);
  }
  if (kind == gp::PC_ICC) {
    gp::FactorPattern F = pattern(P(1), P(2), P(4), P(5), n, false);
    return gp::pc_import_factor(pc, gp::PC_ICC, F, F.r, D(3), nullptr, nullptr);
  }
  pc->opt.type = gp::PC_NONE;
  return gp::pc_setup(pc, A, nullptr);
}

static void ksp_compat(int type, int64_t n, const int64_t* irow, const int64_t* icol,
                       const double* data, const int64_t* pci, const double* pcf, double* cfg,
                       int64_t* cfgi, const double* b, double* x) {
  TmpCsr tA, tS;
  int st = tA.make(irow, icol, data, n, n);
  Pc* pc = nullptr;
  gp::Ksp* k = nullptr;
  gp::pc_create(&pc);
  gp::ksp_create(&k);
  if (!st) st = pc_from_block(pc, pci, pcf, n, tA.A, tS);
  if (!st) {
    gp::KspOptions& o = k->opt;
    o.type = type;
    o.rtol = cfg[0];
    o.atol = cfg[1];
    o.divtol = cfg[2];
    o.haptol = cfg[3];
    o.breakdowntol = cfg[4];
    o.normtype = (int)cfgi[0];
    o.pc_side = (int)cfgi[1];
    o.guess_zero = (int)cfgi[2];
    o.min_it = (int)cfgi[3];
    o.chknorm = (int)cfgi[4];
    o.convmaxits = (int)cfgi[5];
    o.max_it = (int)cfgi[6];
    o.restart = (int)cfgi[7];
    o.orthog = (int)cfgi[8];
    o.cgstype = (int)cfgi[9];
    o.seed_rhs = cfgi[12] ? 1 : 0;
    o.rhs_norm = cfg[12];
    double* db = up(0, b, n);
    double* dx = up(1, x, n);
    std::vector<double> hist((size_t)std::max(o.max_it, 0) + 2, 0.0);
    gp::KspResult res{};
    st = gp::ksp_solve(k, tA.A, pc, db, dx, &res, hist.data(), (int64_t)hist.size(), nullptr);
    if (!st) {
      down(x, dx, n);
      // outputs in the reference's cfg/cfgi slots (src/ksp.mojo:96-152, 1098-1101);
      // the history occupies cfg[9 + its] and shares slots 12 and 14
      cfg[5] = k->h_st->rnorm0;
      cfg[6] = k->h_st->ttol;
      cfg[14] = 1.0;
      if (type == gp::KSP_GMRES) cfg[8] = k->h_st->cfg8;
      for (int64_t i = 0; i <= res.its && i < (int64_t)hist.size(); i++) cfg[9 + i] = hist[i];
      cfg[7] = res.rnorm;
      cfgi[10] = res.its;
      cfgi[11] = res.reason;
    }
  }
  gp::ksp_destroy(k);
  gp::pc_destroy(pc);
  finish_status(st);
}

void mp_ksp_solve_cg(int64_t n, const int64_t* irow, const int64_t* icol, const double* data,
                     const int64_t* pci, const double* pcf, double* pstmp, double* work,
                     double* cfg, int64_t* cfgi, const double* b, double* x) {
  (void)pstmp;
  (void)work;
  ksp_compat(gp::KSP_CG, n, irow, icol, data, pci, pcf, cfg, cfgi, b, x);
}

void mp_ksp_solve_bcgs(int64_t n, const int64_t* irow, const int64_t* icol, const double* data,
                       const int64_t* pci, const double* pcf, double* pstmp, double* work,
                       double* cfg, int64_t* cfgi, const double* b, double* x) {
  (void)pstmp;
  (void)work;
  ksp_compat(gp::KSP_BCGS, n, irow, icol, data, pci, pcf, cfg, cfgi, b, x);
}

void mp_ksp_solve_gmres(int64_t n, const int64_t* irow, const int64_t* icol, const double* data,
                        const int64_t* pci, const double* pcf, double* pstmp, double* work,
                        double* vv, double* hs, double* cfg, int64_t* cfgi, const double* b,
                        double* x) {
  (void)pstmp;
  (void)work;
  (void)vv;
  (void)hs;
  ksp_compat(gp::KSP_GMRES, n, irow, icol, data, pci, pcf, cfg, cfgi, b, x);
}

void mp_ksp_solve_fgmres(int64_t n, const int64_t* irow, const int64_t* icol,
                         const double* data, const int64_t* pci, const double* pcf,
                         double* pstmp, double* work, double* vv, double* prevec, double* hs,
                         double* cfg, int64_t* cfgi, const double* b, double* x) {
  (void)pstmp;
  (void)work;
  (void)vv;
  (void)prevec;
  (void)hs;
  ksp_compat(gp::KSP_FGMRES, n, irow, icol, data, pci, pcf, cfg, cfgi, b, x);
}

}  // extern "C"
