// Preconditioner objects: device data, host set-up analysis and applies.
#pragma once

#include <vector>

#include "gp_internal.h"

namespace gp {

enum PcType : int { PC_NONE = 0, PC_JACOBI = 2, PC_SOR = 4, PC_ILU = 5, PC_ICC = 6 };

// MatSORType bits (petscmat.h), as the reference uses them.
constexpr int kSorForward = 1 | 4;    // SOR_FORWARD_SWEEP | SOR_LOCAL_FORWARD_SWEEP
constexpr int kSorBackward = 2 | 8;   // SOR_BACKWARD_SWEEP | SOR_LOCAL_BACKWARD_SWEEP

struct PcOptions {
  int type = PC_NONE;
  int jacobi_type = 0;   // 0 diagonal, 1 rowmax, 2 rowl1, 3 rowsum
  int use_abs = 0;
  int fix_diag = 1;
  double rowl1_scale = 1.0;
  double omega = 1.0;
  double fshift = 0.0;
  int sor_flag = 12 | 16;  // LOCAL_SYMMETRIC | ZERO_INITIAL_GUESS
  int levels = 0;
  int ordering = 0;      // 0 natural, 1 rcm, 2 multicolour
};

// Processing plan of one sync-free sweep: rows in dependency-level order and
// a ticket pair for the dynamic row hand-out.
struct SweepPlan {
  int* order = nullptr;      // device, n
  int nlevels = 0;
};

// A sweep laid out in processing order for the ELL sweep kernels
// (gp_sweep.cu); `ok` is false when some row has more than kEllMaxW
// dependencies, and the CSR sweep kernels are used instead.
constexpr int kEllMaxW = 16;
enum EllMode : int { ELL_ILU_F, ELL_ILU_B, ELL_ICC_F, ELL_ICC_B, ELL_SOR_F, ELL_SOR_B };
struct EllSweep {
  int n = 0, W = 0;
  bool ok = false;
  int* cnt = nullptr;
  int* dep = nullptr;
  int* cslot = nullptr;
  int* in_idx = nullptr;
  int* out_idx = nullptr;
  int* dslot = nullptr;
  int* rowof = nullptr;
  double* coef = nullptr;
  double* dval = nullptr;
  // Tiled form (gp_sweep.cu, k_tile_sweep): positions grouped in chunks of
  // consecutive rows of the sweep's natural sequence, each chunk sorted by
  // the dependency level among its own rows and processed by one warp that
  // stages the chunk's metadata in shared memory with one bulk copy.  When
  // `tiled` is set the ELL columns above are not allocated: every index the
  // tiled kernel reads is in the blob.
  bool tiled = false;
  int nchunks = 0, C = 0, max_blob = 0, grid = 0;
  size_t smem = 0;
  unsigned char* blob = nullptr;  // per chunk: header, level offsets, columns
  long long* blob_off = nullptr;  // [nchunks + 1] byte offsets into blob
  int* cstart = nullptr;          // [nchunks + 1] first position of each chunk
  double est_us = 0.0;            // simulated duration of one tiled sweep
  int rows_per_chunk = 0;         // chunk size of the tiled layout
  // Brick form (gp_brick.cu, k_brick_sweep): the sweep's dependencies are the
  // unit steps of a grid gx x gy x gz; CTAs take bricks of BJ grid lines of
  // one plane (BK = 1) and each thread walks one line.  `n` counts positions,
  // step-major within each brick with holes (nrows rows); the per-position
  // arrays are cslot / coef as [direction][n], in_idx, out_idx (absent when
  // the identity), dslot / dval, and values are indexed by position.
  bool brick = false;
  int gx = 0, gy = 0, gz = 0, BJ = 0, BK = 0, nbJ = 0, nbricks = 0, bgrid = 0, nrows = 0;
  int bord = 0;            // fold order of a row's terms: 0 k, j, i; 1 i, j, k
  bool in_ident = false, out_ident = false;
  int* border = nullptr;   // [2 * nbricks]: (J, K) of each brick in hand-out order
  int* bbase = nullptr;    // [nbJ * gz]: first position of brick (J, K) at J + nbJ K
};
void ell_free(EllSweep& e);
// Brick layout of a sweep when its dependencies have the grid structure and
// (unless forced) the model puts it below `other_us`; *built says whether.
// pos_of_row: each row's position in the brick layout.
int brick_build(EllSweep& e, int mode, int n, bool forward, const std::vector<int>& dptr,
                const std::vector<int>& dcol, const std::vector<int>& dsl,
                const std::vector<int>& in_row, const std::vector<int>& out_row,
                const std::vector<int>& dslot_row, double other_us, bool* built,
                std::vector<int>* pos_of_row);
int brick_sweep(int mode, const EllSweep& e, const int* gate, int want, DRef in, DRef out,
                double* val, const double* fval, double* aux, const double* auxin,
                const double* idiag, double omega, int use_t, int write_out, unsigned* tickets,
                DevErr* err, cudaStream_t s);
// Brick form of later set-ups: mode 0 never, 1 where modelled faster, 2
// wherever the structure allows; lines > 0 forces the lines of a brick;
// max_ctas > 0 caps the persistent grid.
void set_sweep_bricks(int mode, int lines, int max_ctas);
// Lay out one sweep.  forward: dependencies precede each row (ascending
// processing); otherwise they follow it.  `order` is the level order, used
// when the sweep is not tiled; nlevels its depth when known (0: counted here).
// mode: the EllMode of the kernel that will run the sweep.
int ell_build(EllSweep& e, int mode, int n, bool forward, const std::vector<int>& order,
              const std::vector<int>& dptr, const std::vector<int>& dcol,
              const std::vector<int>& dsl, const std::vector<int>& in_row,
              const std::vector<int>& out_row, const std::vector<int>& dslot_row,
              std::vector<int>* pos_of_row, int nlevels = 0);
int ell_refresh(EllSweep& e, const double* src, cudaStream_t s);
// ell_build choosing between the level-ordered and the chunked form only (no
// brick layout: its kernel reads the reference's inputs of each mode only).
int ell_build_chunked(EllSweep& e, int mode, int n, bool forward, const std::vector<int>& order,
                      const std::vector<int>& dptr, const std::vector<int>& dcol,
                      const std::vector<int>& dsl, const std::vector<int>& in_row,
                      const std::vector<int>& out_row, const std::vector<int>& dslot_row,
                      std::vector<int>* pos_of_row);
// ell_build in the level-ordered form only (no chunked or brick layout).
int ell_build_levels(EllSweep& e, int mode, int n, bool forward, const std::vector<int>& order,
                     const std::vector<int>& dptr, const std::vector<int>& dcol,
                     const std::vector<int>& dsl, const std::vector<int>& in_row,
                     const std::vector<int>& out_row, const std::vector<int>& dslot_row,
                     std::vector<int>* pos_of_row);
int sweep_wait_probe(int budget, int set, cudaStream_t s);
// Sweep form of later set-ups (gp_set_sweep_form).
void set_sweep_form(int tiles, int tile_rows);
// coefsrc: the array the sweep's coefficient slots index (the factor values
// for ILU/IC, the matrix values for SOR); the tiled form gathers from it.
int ell_sweep(int mode, const EllSweep& e, const int* gate, int want, DRef in, DRef out,
              double* val, const double* fval, double* aux, const double* auxin,
              const double* idiag, double omega, int use_t, int write_out, unsigned* tickets,
              DevErr* err, const double* coefsrc, cudaStream_t s);

// Host copy of a factor pattern in the reference's layout.
struct FactorPattern {
  // ILU: L rows bi[i]..bi[i+1], U rows (reversed) ending on the diagonal at
  // bdiag[i]; IC: row i = strict upper ascending then the diagonal slot
  // bdiag[i] = bi[i+1]-1.
  std::vector<int> bi, bj, bdiag;
  std::vector<int> r, ic;   // row ordering and its inverse
  int nnz = 0;              // number of factor slots
};

struct Pc {
  PcOptions opt;
  Csr* A = nullptr;  // operator the PC was set up from (not owned)
  int n = 0;
  // entries of the sweeps' value arrays yf, yb, ys, t: the rows, or more
  // where a sweep's layout has holes (the brick form)
  int vlen = 0;
  int device = -1;
  bool ready = false;
  int epoch = 0;
  // a fresh next_uid() at every set-up (device arrays reallocated): cached
  // solve graphs compare it, never the PC's address
  unsigned long long generation = 0;

  // Jacobi
  double* diag = nullptr;
  double* diagsqrt = nullptr;

  // SOR (uses A's arrays and diagpos)
  double* idiag = nullptr;
  double* mdiag = nullptr;
  // SOR: nonzero while the inverted diagonal and the sweeps' coefficients
  // must be recomputed from A's values (device word, read by the apply's
  // kernels); sor_vver is the A->vver they were last marked for
  int* sor_stale = nullptr;
  unsigned long long sor_vver = 0;

  // factor (ILU / IC), reference layout on the device
  FactorPattern pat;
  int* bi = nullptr;
  int* bj = nullptr;
  int* bdiag = nullptr;
  int* perm_r = nullptr;
  int* perm_c = nullptr;     // where row i of the factor's solution goes
  int* perm_ic = nullptr;
  double* ba = nullptr;      // factor values (what the solve reads)
  double* ba_orig = nullptr; // IC: unscaled strict rows
  int* done = nullptr;       // numeric row-done epochs
  // IC numeric: chain-ordered contributor lists (row k <- (i, slot))
  int* cptr = nullptr;
  int* crow = nullptr;
  int* cslot = nullptr;
  // IC forward sweep: transposed strict pattern, ascending source row
  int* tptr = nullptr;
  int* trow = nullptr;
  int* tslot = nullptr;
  int* amap = nullptr;       // A slot -> factor slot (or -1)
  // ILU numeric: per L slot, the (row slot, pivot U slot) updates it makes
  int* upd_ptr = nullptr;
  int* upd_dst = nullptr;
  int* upd_src = nullptr;

  SweepPlan fwd, bwd, num;
  EllSweep ef, eb;           // ELL forms of the forward and backward sweeps
  // ILU transposed apply (built on first use): sweeps over U^T (forward) and
  // L^T (backward) of the same factor
  EllSweep etf, etb;
  bool trans_ready = false;
  // sweep work: value-as-flag arrays and SOR checkpoint
  double* yf = nullptr;
  double* yb = nullptr;
  double* ys = nullptr;      // IC: scaled forward values
  double* t = nullptr;       // SOR checkpoint
  unsigned* tickets = nullptr;  // [4]: (ticket, exits) x 2
  DevErr* err = nullptr;
};

int pc_create(Pc** out);
int pc_destroy(Pc* pc);
int pc_setup(Pc* pc, Csr* A, cudaStream_t s);
// y = M^-1 x (x, y distinct device vectors).  Gate for captured loops.
int pc_apply(Pc* pc, DRef x, DRef y, cudaStream_t s, const int* gate = nullptr, int want = 0);
// y = M^-T x: the true transpose of the preconditioner (ILU: sweeps over U^T
// then L^T of the factor; none, Jacobi and IC are symmetric, so their apply;
// SOR: GP_ERR_UNSUPPORTED).  pc_transpose_prepare builds what it needs on the
// host (outside any stream capture).
int pc_transpose_prepare(Pc* pc, cudaStream_t s);
int pc_apply_transpose(Pc* pc, DRef x, DRef y, cudaStream_t s, const int* gate = nullptr,
                       int want = 0);
// IC(0)/IC(k) apply to R columns stored row-major (x, y: n * R; vf, vb, ys:
// n * R scratch), R dividing 32; no gate (not for captured solver loops of
// the single-vector drivers; the batched CG captures it).
int pc_apply_icc_cols(Pc* pc, int R, const double* x, double* y, double* vf, double* vb,
                      double* ys, cudaStream_t s);
// Jacobi symmetric half; other types fall back to pc_apply.
int pc_apply_symmetric(Pc* pc, DRef x, DRef y, cudaStream_t s, const int* gate = nullptr,
                       int want = 0);
// Read and clear the device error word (spin timeouts).  Synchronizes s.
int pc_check(Pc* pc, cudaStream_t s);

int pc_factor_numeric(Pc* pc, cudaStream_t s);
// Same operator pattern, new values: redo only the numeric phase (factor
// values, Jacobi diagonals) in the arrays of the last set-up.
int pc_update_values(Pc* pc, cudaStream_t s);
// Mark SOR's value-derived arrays for recomputation when the operator's values
// changed since they were last marked (outside stream capture; a captured
// solve graph calls it before every launch).
int pc_values_sync(Pc* pc, cudaStream_t s);
int pc_import_factor(Pc* pc, int type, const FactorPattern& pat, const std::vector<int>& perm_c,
                     const double* ba_host, Csr* A, cudaStream_t s);
int pc_import_jacobi(Pc* pc, int n, const double* diag, const double* diagsqrt, cudaStream_t s);
int jacobi_fill(const Csr* A, int jtype, int sym, int use_abs, int fix_diag, double scale,
                double* out, cudaStream_t s);
int sor_diagonals(Pc* pc, cudaStream_t s);

// host analysis (gp_pcsetup.cu)
int rcm_order(const std::vector<int>& rowptr, const std::vector<int>& colind, int n,
              std::vector<int>& perm);
int color_order(const std::vector<int>& rowptr, const std::vector<int>& colind, int n,
                std::vector<int>& perm, int* ncolors);
int ilu_symbolic_rows(const Csr* A, int levels, const std::vector<int>& r,
                      const std::vector<int>& ic,
                      std::vector<std::vector<std::pair<int, int>>>& rows, std::vector<int>& nL);
int icc_symbolic_rows(const Csr* A, int levels, const std::vector<int>& r,
                      const std::vector<int>& ic,
                      std::vector<std::vector<std::pair<int, int>>>& rows);
int ilu_symbolic(const Csr* A, int levels, const std::vector<int>& r,
                 const std::vector<int>& ic, FactorPattern& out);
int icc_symbolic(const Csr* A, int levels, const std::vector<int>& r,
                 const std::vector<int>& ic, FactorPattern& out);
// Levels of a DAG given as dependency lists; forward (deps < i) or backward.
void level_order(int n, const std::vector<int>& dptr, const std::vector<int>& dcol,
                 bool forward, std::vector<int>& order, int* nlevels);

}  // namespace gp
