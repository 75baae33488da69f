// extern "C" device layer (gp_*) of libgpetsc.so; declarations and the
// contract of each entry point are in include/gpetsc.h.
#include <cstring>
#include <exception>

#include "../../include/gpetsc.h"
#include "gp_ksp.h"

#include "gp_handles.h"



#define GUARD(expr)                                           \
  try {                                                       \
    return (expr);                                            \
  } catch (const std::exception& e) {                         \
    gp::set_error(std::string("internal error: ") + e.what()); \
    return gp::GP_ERR_INTERNAL;                               \
  } catch (...) {                                             \
    gp::set_error("internal error");                          \
    return gp::GP_ERR_INTERNAL;                               \
  }

static cudaStream_t S(void* s) { return reinterpret_cast<cudaStream_t>(s); }

static int bad(const char* msg) {
  gp::set_error(msg);
  return GP_ERR_ARG;
}

extern "C" {

int gp_version(void) { return 100; }
const char* gp_last_error(void) { return gp::last_error(); }

int gp_set_arithmetic(int mode) {
  if (mode != GP_ARITH_EXACT && mode != GP_ARITH_FMA && mode != GP_ARITH_ORDERED) {
    gp::set_error(
        "gp_set_arithmetic: mode must be GP_ARITH_EXACT (0), GP_ARITH_FMA (1) or "
        "GP_ARITH_ORDERED (2)");
    return GP_ERR_ARG;
  }
  gp::set_arith_mode(mode);
  return GP_OK;
}

int gp_get_arithmetic(void) { return gp::arith_mode(); }

int gp_device_count(int* count) {
  int c = 0;
  cudaError_t e = cudaGetDeviceCount(&c);
  if (e != cudaSuccess) {
    cudaGetLastError();
    c = 0;
  }
  *count = c;
  return GP_OK;
}

int gp_set_device(int device) {
  GP_CUDA(cudaSetDevice(device));
  return GP_OK;
}

// ------------------------------------------------------------ Mat
int gp_mat_create(gp_mat* out, int64_t nrows, int64_t ncols, int64_t nnz, const int64_t* indptr,
                  const int64_t* indices, const double* values) {
  if (!out || !indptr || (nnz && (!indices || !values))) return bad("gp_mat_create: null array");
  GUARD(([&]() {
    gp::Csr* A = nullptr;
    int st = gp::csr_create(&A, nrows, ncols, nnz, indptr, indices, values, nullptr);
    if (st) return st;
    *out = new gp_mat_s{A};
    return (int)GP_OK;
  })());
}

int gp_mat_create_i32(gp_mat* out, int64_t nrows, int64_t ncols, int64_t nnz,
                      const int32_t* indptr, const int32_t* indices, const double* values) {
  if (!out || !indptr || (nnz && (!indices || !values))) return bad("gp_mat_create: null array");
  GUARD(([&]() {
    gp::Csr* A = nullptr;
    int st = gp::csr_create_i32(&A, nrows, ncols, nnz, indptr, indices, values, nullptr);
    if (st) return st;
    *out = new gp_mat_s{A};
    return (int)GP_OK;
  })());
}

int gp_mat_destroy(gp_mat A) {
  if (!A) return GP_OK;
  gp::csr_destroy(A->A);
  delete A;
  return GP_OK;
}

int gp_mat_set_values(gp_mat A, const double* values, int on_device, void* stream) {
  if (!A || (!values && A->A->nnz)) return bad("gp_mat_set_values: null argument");
  return gp::csr_set_values(A->A, values, on_device, S(stream));
}

int gp_mat_values_ptr(gp_mat A, double** d_values) {
  if (!A || !d_values) return bad("gp_mat_values_ptr: null argument");
  *d_values = A->A->val;
  return GP_OK;
}

int gp_mat_info(gp_mat A, int64_t* nrows, int64_t* ncols, int64_t* nnz) {
  if (!A) return bad("gp_mat_info: null matrix");
  if (nrows) *nrows = A->A->n;
  if (ncols) *ncols = A->A->ncols;
  if (nnz) *nnz = A->A->nnz;
  return GP_OK;
}

int gp_mat_spmv_index_bytes(gp_mat A, int32_t* bytes) {
  if (!A || !bytes) return bad("gp_mat_spmv_index_bytes: null argument");
  *bytes = A->A->coff16 ? 2 : 4;
  return GP_OK;
}

int gp_mat_mult(gp_mat A, const double* x, double* y, void* stream) {
  if (!A || !x || !y) return bad("gp_mat_mult: null argument");
  if (x == y) return bad("gp_mat_mult: y may not alias x");
  GUARD(gp::spmv(S(stream), A->A, gp::DRef::of(x), gp::DRef::of(y)));
}

int gp_mat_mult_add(gp_mat A, const double* x, const double* v, double* y, void* stream) {
  if (!A || !x || !v || !y) return bad("gp_mat_mult_add: null argument");
  if (x == y) return bad("gp_mat_mult_add: y may not alias x");
  GUARD(gp::spmv_add(S(stream), A->A, x, v, y));
}

int gp_mat_mult_transpose(gp_mat A, const double* x, double* y, void* stream) {
  if (!A || !x || !y) return bad("gp_mat_mult_transpose: null argument");
  if (x == y) return bad("gp_mat_mult_transpose: y may not alias x");
  GUARD(gp::spmv_t(S(stream), A->A, x, y));
}

int gp_mat_transpose(gp_mat A, gp_mat* out, void* stream) {
  if (!A || !out) return bad("gp_mat_transpose: null argument");
  GUARD(([&]() {
    gp::Csr* T = nullptr;
    int st = gp::csr_create_transpose(A->A, &T, S(stream));
    if (st) return st;
    *out = new gp_mat_s{T};
    return (int)GP_OK;
  })());
}

int gp_mat_transpose_values(gp_mat A, gp_mat At, void* stream) {
  if (!A || !At) return bad("gp_mat_transpose_values: null argument");
  GUARD(gp::csr_transpose_values(A->A, At->A, S(stream)));
}

int gp_mat_outer_on_pattern(gp_mat A, const double* u, const double* v, double alpha,
                            double* out, void* stream) {
  if (!A || !out || (A->A->n && (!u || !v))) return bad("gp_mat_outer_on_pattern: null argument");
  GUARD(gp::csr_outer_on_pattern(A->A, u, v, alpha, out, S(stream)));
}

int gp_mat_get_diagonal(gp_mat A, double* d, void* stream) {
  if (!A || !d) return bad("gp_mat_get_diagonal: null argument");
  GUARD(gp::mat_diagonal(S(stream), A->A, d));
}

// ------------------------------------------------------------ Vec
int gp_vec_map(int op, int64_t n, double* y, const double* x, const double* w, double alpha,
               double beta, double gamma, void* stream) {
  if (n < 0) return bad("gp_vec_map: negative length");
  if (n > 0 && !y) return bad("gp_vec_map: null output");
  GUARD(gp::vec_map(S(stream), op, n, y, x, w, alpha, beta, gamma));
}

int gp_vec_maxpy(int64_t n, double* y, int64_t nv, const double* alpha, const double* const* xs,
                 void* stream) {
  if (n < 0 || nv < 0) return bad("gp_vec_maxpy: negative size");
  if (nv > INT32_MAX) return bad("gp_vec_maxpy: too many vectors");
  GUARD(gp::vec_maxpy(S(stream), n, y, (int)nv, alpha, xs));
}

int gp_vec_reduce(int op, int64_t n, const double* x, const double* y, double* out,
                  void* stream) {
  if (n < 0 || !out) return bad("gp_vec_reduce: bad argument");
  GUARD(gp::vec_reduce(S(stream), op, n, x, y, out));
}

int gp_vec_minmax(int64_t n, const double* x, int is_max, int64_t* idx, double* val,
                  void* stream) {
  if (n < 0 || !idx || !val) return bad("gp_vec_minmax: bad argument");
  GUARD(([&]() {
    long long i = -1;
    int st = gp::vec_minmax(S(stream), n, x, is_max, &i, val);
    *idx = i;
    return st;
  })());
}

int gp_vec_max_pointwise_divide(int64_t n, const double* x, const double* y, double* out,
                                void* stream) {
  if (n < 0 || !out) return bad("gp_vec_max_pointwise_divide: bad argument");
  GUARD(gp::vec_max_pointwise_divide(S(stream), n, x, y, out));
}

// ------------------------------------------------------------ PC
void gp_pc_options_default(gp_pc_options* o) {
  gp::PcOptions d;
  std::memset(o, 0, sizeof(*o));
  o->type = d.type;
  o->jacobi_type = d.jacobi_type;
  o->use_abs = d.use_abs;
  o->fix_diag = d.fix_diag;
  o->rowl1_scale = d.rowl1_scale;
  o->omega = d.omega;
  o->fshift = d.fshift;
  o->sor_flag = d.sor_flag;
  o->levels = d.levels;
  o->ordering = d.ordering;
}

int gp_pc_create(gp_pc* out) {
  if (!out) return bad("gp_pc_create: null argument");
  gp::Pc* p = nullptr;
  gp::pc_create(&p);
  *out = new gp_pc_s{p};
  return GP_OK;
}

int gp_pc_destroy(gp_pc pc) {
  if (!pc) return GP_OK;
  gp::pc_destroy(pc->pc);
  delete pc;
  return GP_OK;
}

int gp_pc_set_options(gp_pc pc, const gp_pc_options* o) {
  if (!pc || !o) return bad("gp_pc_set_options: null argument");
  if (o->type != 0 && o->type != 2 && o->type != 4 && o->type != 5 && o->type != 6)
    return bad("gp_pc_set_options: unknown PC type");
  if (o->levels < 0) return bad("gp_pc_set_options: negative levels");
  if (o->ordering < 0 || o->ordering > 2)
    return bad("gp_pc_set_options: ordering must be 0 (natural), 1 (rcm) or 2 (multicolour)");
  gp::PcOptions& d = pc->pc->opt;
  d.type = o->type;
  d.jacobi_type = o->jacobi_type;
  d.use_abs = o->use_abs;
  d.fix_diag = o->fix_diag;
  d.rowl1_scale = o->rowl1_scale;
  d.omega = o->omega;
  d.fshift = o->fshift;
  d.sor_flag = o->sor_flag;
  d.levels = o->levels;
  d.ordering = o->ordering;
  pc->pc->ready = false;
  return GP_OK;
}

int gp_pc_setup(gp_pc pc, gp_mat A, void* stream) {
  if (!pc || !A) return bad("gp_pc_setup: null argument");
  GUARD(gp::pc_setup(pc->pc, A->A, S(stream)));
}

int gp_wait_probe(int32_t spins, int32_t set, void* stream) {
  if (spins < 0) return bad("gp_wait_probe: spins must be >= 0");
  GUARD(gp::sweep_wait_probe(spins, set, S(stream)));
}

int gp_set_sweep_form(int32_t tiles, int32_t tile_rows) {
  if (tiles < 0 || tiles > 1 || tile_rows < 0 || tile_rows > 8192)
    return bad("gp_set_sweep_form: tiles must be 0 or 1 and tile_rows in [0, 8192]");
  gp::set_sweep_form(tiles, tile_rows);
  return GP_OK;
}

int gp_set_sweep_bricks(int32_t mode, int32_t lines_j, int32_t lines_k, int32_t max_ctas) {
  if (mode < 0 || mode > 2 || lines_j < 0 || lines_j > 128 || lines_k < 0 || lines_k > 1 ||
      max_ctas < 0)
    return bad("gp_set_sweep_bricks: mode must be 0, 1 or 2, 0 <= lines_j <= 128, lines_k 0 "
               "or 1 and max_ctas >= 0");
  gp::set_sweep_bricks(mode, lines_j, max_ctas);
  return GP_OK;
}

int gp_pc_sweep_bricks(gp_pc pc, int32_t which, int32_t* brick, int32_t* dims) {
  if (!pc || !brick || !dims || (which != 0 && which != 1))
    return bad("gp_pc_sweep_bricks: null argument or which not 0/1");
  const gp::EllSweep& e = which == 0 ? pc->pc->ef : pc->pc->eb;
  *brick = e.brick ? 1 : 0;
  const int32_t v[5] = {e.gx, e.gy, e.gz, e.BJ, e.BK};
  for (int k = 0; k < 5; k++) dims[k] = e.brick ? v[k] : 0;
  return GP_OK;
}

int gp_pc_sweep_form(gp_pc pc, int32_t which, int32_t* tiled, int32_t* rows_per_chunk,
                     int32_t* chunks) {
  if (!pc || !tiled || !rows_per_chunk || !chunks || which < 0 || which > 3)
    return bad("gp_pc_sweep_form: null argument or which not 0..3");
  const gp::Pc* p = pc->pc;
  const gp::EllSweep& e = which == 0 ? p->ef : which == 1 ? p->eb : which == 2 ? p->etf : p->etb;
  *tiled = e.tiled ? 1 : 0;
  *rows_per_chunk = e.tiled ? e.rows_per_chunk : 0;
  *chunks = e.tiled ? e.nchunks : 0;
  return GP_OK;
}

int gp_pc_update_values(gp_pc pc, void* stream) {
  if (!pc) return bad("gp_pc_update_values: null argument");
  GUARD(gp::pc_update_values(pc->pc, S(stream)));
}

int gp_pc_apply(gp_pc pc, const double* x, double* y, void* stream) {
  if (!pc || !x || !y) return bad("gp_pc_apply: null argument");
  if (x == y) return bad("gp_pc_apply: y may not alias x");
  GUARD(([&]() {
    int st = gp::pc_apply(pc->pc, gp::DRef::of(x), gp::DRef::of(y), S(stream));
    if (st) return st;
    return gp::pc_check(pc->pc, S(stream));
  })());
}

int gp_pc_apply_transpose(gp_pc pc, const double* x, double* y, void* stream) {
  if (!pc || !x || !y) return bad("gp_pc_apply_transpose: null argument");
  if (x == y) return bad("gp_pc_apply_transpose: y may not alias x");
  GUARD(([&]() {
    int st = gp::pc_transpose_prepare(pc->pc, S(stream));
    if (st) return st;
    st = gp::pc_apply_transpose(pc->pc, gp::DRef::of(x), gp::DRef::of(y), S(stream));
    if (st) return st;
    return gp::pc_check(pc->pc, S(stream));
  })());
}

int gp_pc_apply_symmetric(gp_pc pc, const double* x, double* y, void* stream) {
  if (!pc || !x || !y) return bad("gp_pc_apply_symmetric: null argument");
  if (x == y) return bad("gp_pc_apply_symmetric: y may not alias x");
  GUARD(([&]() {
    int st = gp::pc_apply_symmetric(pc->pc, gp::DRef::of(x), gp::DRef::of(y), S(stream));
    if (st) return st;
    return gp::pc_check(pc->pc, S(stream));
  })());
}

int gp_pc_factor_info(gp_pc pc, int64_t* n, int64_t* nslots) {
  if (!pc) return bad("gp_pc_factor_info: null argument");
  if (n) *n = pc->pc->n;
  if (nslots) *nslots = pc->pc->pat.nnz;
  return GP_OK;
}

int gp_pc_factor_get(gp_pc pc, int64_t* bi, int64_t* bj, double* ba, int64_t* bdiag,
                     int64_t* perm) {
  if (!pc) return bad("gp_pc_factor_get: null argument");
  gp::Pc* p = pc->pc;
  if (!p->ready || (p->opt.type != gp::PC_ILU && p->opt.type != gp::PC_ICC))
    return bad("gp_pc_factor_get: no factor");
  const gp::FactorPattern& P = p->pat;
  const int n = p->n;
  if (bi)
    for (int i = 0; i <= n; i++) bi[i] = P.bi[i];
  if (bj)
    for (int j = 0; j < P.nnz; j++) bj[j] = P.bj[j];
  if (bdiag)
    for (int i = 0; i <= n; i++) bdiag[i] = P.bdiag[i];
  if (perm)
    for (int i = 0; i < n; i++) perm[i] = P.r[i];
  if (ba) GP_CUDA(cudaMemcpy(ba, p->ba, (size_t)P.nnz * sizeof(double), cudaMemcpyDeviceToHost));
  return GP_OK;
}

// ------------------------------------------------------------ KSP
void gp_ksp_options_default(gp_ksp_options* o) {
  gp::KspOptions d;
  std::memset(o, 0, sizeof(*o));
  o->type = d.type;
  o->normtype = d.normtype;
  o->pc_side = d.pc_side;
  o->guess_zero = d.guess_zero;
  o->min_it = d.min_it;
  o->chknorm = d.chknorm;
  o->convmaxits = d.convmaxits;
  o->max_it = d.max_it;
  o->restart = d.restart;
  o->orthog = d.orthog;
  o->cgstype = d.cgstype;
  o->seed_rhs = d.seed_rhs;
  o->rtol = d.rtol;
  o->atol = d.atol;
  o->divtol = d.divtol;
  o->haptol = d.haptol;
  o->breakdowntol = d.breakdowntol;
  o->rhs_norm = d.rhs_norm;
}

int gp_ksp_create(gp_ksp* out) {
  if (!out) return bad("gp_ksp_create: null argument");
  gp::Ksp* k = nullptr;
  gp::ksp_create(&k);
  *out = new gp_ksp_s{k};
  return GP_OK;
}

int gp_ksp_destroy(gp_ksp ksp) {
  if (!ksp) return GP_OK;
  gp::ksp_destroy(ksp->k);
  delete ksp;
  return GP_OK;
}

int gp_ksp_set_options(gp_ksp ksp, const gp_ksp_options* o) {
  if (!ksp || !o) return bad("gp_ksp_set_options: null argument");
  if (o->normtype < 1 || o->normtype > 4) return bad("gp_ksp_set_options: normtype 1..4");
  if (o->pc_side < 0 || o->pc_side > 2) return bad("gp_ksp_set_options: pc_side 0..2");
  gp::KspOptions& d = ksp->k->opt;
  d.type = o->type;
  d.normtype = o->normtype;
  d.pc_side = o->pc_side;
  d.guess_zero = o->guess_zero;
  d.min_it = o->min_it;
  d.chknorm = o->chknorm;
  d.convmaxits = o->convmaxits;
  d.max_it = o->max_it;
  d.restart = o->restart;
  d.orthog = o->orthog;
  d.cgstype = o->cgstype;
  d.seed_rhs = o->seed_rhs;
  d.rtol = o->rtol;
  d.atol = o->atol;
  d.divtol = o->divtol;
  d.haptol = o->haptol;
  d.breakdowntol = o->breakdowntol;
  d.rhs_norm = o->rhs_norm;
  return GP_OK;
}

int gp_ksp_solve(gp_ksp ksp, gp_mat A, gp_pc pc, const double* b, double* x,
                 gp_ksp_result* result, double* hist, int64_t hist_len, void* stream) {
  if (!ksp || !A || !pc || !result) return bad("gp_ksp_solve: null argument");
  if (A->A->n > 0 && (!b || !x)) return bad("gp_ksp_solve: null vector");
  if (b == x && b) return bad("gp_ksp_solve: x may not alias b");
  GUARD(([&]() {
    gp::KspResult r{};
    int st = gp::ksp_solve(ksp->k, A->A, pc->pc, b, x, &r, hist, hist_len, S(stream));
    result->its = r.its;
    result->reason = r.reason;
    result->rnorm = r.rnorm;
    return st;
  })());
}

int gp_ksp_set_transpose(gp_ksp ksp, int transpose) {
  if (!ksp) return bad("gp_ksp_set_transpose: null solver");
  if (transpose != 0 && transpose != 1) return bad("gp_ksp_set_transpose: 0 or 1");
  ksp->k->transpose = transpose;
  return GP_OK;
}

int gp_ksp_set_launch_form(gp_ksp ksp, int form) {
  if (!ksp) return bad("gp_ksp_set_launch_form: null solver");
  if (form < -1 || form > 1) return bad("gp_ksp_set_launch_form: form must be -1, 0 or 1");
  ksp->k->launch_form = form;
  return GP_OK;
}

int gp_ksp_stats(gp_ksp ksp, int64_t* trips, int64_t* top_kernels, int64_t* body_kernels) {
  if (!ksp) return bad("gp_ksp_stats: null argument");
  if (trips) *trips = ksp->k->last_trips;
  if (top_kernels) *top_kernels = ksp->k->top_kernels;
  if (body_kernels) *body_kernels = ksp->k->body_kernels;
  return GP_OK;
}

}  // extern "C"
