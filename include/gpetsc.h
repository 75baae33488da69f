/*
 * gpetsc.h -- C ABI of libgpetsc.so, the GB300 (sm_103a) implementation of
 * lee101/mojo-petsc4py's sequential Krylov path.
 *
 * Two layers:
 *
 *  1. gp_*  Device layer.  Opaque handles for a CSR matrix, a preconditioner
 *     and a Krylov solver; vectors are device pointers (float64).  Every
 *     function returns 0 on success or a nonzero status (see GP_ERR_*), with
 *     the message available from gp_last_error().  Nothing throws across the
 *     ABI.  `stream` arguments are cudaStream_t values passed as void*; NULL
 *     is the legacy default stream.  Calls that return a host value (a
 *     reduction, a solve result) synchronize before returning.
 *
 *  2. mp_*  The reference's own host ABI (src/capi.mojo:32-424, declared for
 *     ctypes in python/mojopetsc4py/_lib.py:23-87): the same 59 names, the
 *     same argument order and meaning, host pointers for every buffer, int64
 *     for every index and size, double for every scalar.  Each call copies its
 *     inputs to the GPU, runs the CUDA kernels of layer 1 and copies the
 *     outputs back, so a caller of the reference's library can switch to this
 *     one without changing a call.  The reference passes addresses as int64;
 *     on LP64 targets a pointer argument has the same calling convention.
 *
 * Index arrays on the device are int32 (the reference stores int64; no value
 * depends on it): matrices must have fewer than 2^31 rows and nonzeros.
 */
#ifndef GPETSC_H
#define GPETSC_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------ status */
enum {
  GP_OK = 0,
  GP_ERR_ARG = 1,         /* bad argument: size, null pointer, alias, type */
  GP_ERR_CUDA = 2,        /* a CUDA runtime call failed */
  GP_ERR_TIMEOUT = 3,     /* a device wait ran out of its iteration budget */
  GP_ERR_NOT_SETUP = 4,   /* object used before set-up */
  GP_ERR_UNSUPPORTED = 5, /* option not available on the device path */
  GP_ERR_NUMERIC = 6,
  GP_ERR_INTERNAL = 7
};

/* Library version (major*10000 + minor*100 + patch). */
int gp_version(void);
/* Message of the last failed call on this host thread. */
const char *gp_last_error(void);
/* Floating-point form of every kernel launched after the call (the process
 * default comes from the environment: GPETSC_ARITHMETIC=exact or =ordered
 * selects that form, anything else FMA).
 *   GP_ARITH_EXACT    each product and sum rounded separately, in the
 *                     reference's order: SpMV, the Vec maps, the PC applies
 *                     and the factors are bit-identical to its sequential
 *                     loops (src/ported.mojo) on the same inputs; reductions
 *                     use a fixed parallel tree (equal to rounding).
 *   GP_ARITH_FMA      products folded into fused multiply-adds, same order:
 *                     half the FP64 instructions; results differ from the
 *                     exact form by rounding only.
 *   GP_ARITH_ORDERED  GP_ARITH_EXACT with every reduction (dot, norms,
 *                     dotNorm2, asum, sum, GMRES's multi-dot) summed in the
 *                     reference's blocked order (src/simdvec.mojo:332-473,
 *                     src/ksp.mojo:956-1062): whole solves bit-identical to
 *                     the reference's; each reduction is a sequential chain
 *                     of n/16 adds (milliseconds at n = 2^21), a checking
 *                     form, not a fast one.
 * No counterpart in the reference (its loops are compiled one way).  Solver
 * graphs captured in one form are re-captured when the form changes. */
enum { GP_ARITH_EXACT = 0, GP_ARITH_FMA = 1, GP_ARITH_ORDERED = 2 };
int gp_set_arithmetic(int mode);
int gp_get_arithmetic(void);
/* Number of visible CUDA devices (0 when none). */
int gp_device_count(int *count);
int gp_set_device(int device);

/* ------------------------------------------------------------ memory
 * Device and page-locked host memory and copies, so a host program needs no
 * CUDA binding besides this library (the Python package keeps every Vec and
 * Mat device copy in these blocks).  No counterpart in the reference, whose
 * vectors live in host numpy arrays (python/mojopetsc4py/PETSc/Vec.py:81-116).
 *
 * gp_device_alloc  `bytes` of device memory on the current device, from a
 *                  stream-ordered pool the library keeps for the process:
 *                  ordered on `stream` (NULL: the default stream); blocks
 *                  freed with gp_device_free are reused without a device
 *                  synchronisation.  bytes == 0 gives NULL.
 * gp_device_free   returns a block, ordered after the work queued on
 *                  `stream` (free on the stream that last used it).
 * gp_host_alloc    page-locked host memory (full-rate copies), recycled by
 *                  size within the process; gp_host_free returns it.
 * gp_copy          one cudaMemcpyAsync of `bytes` on `stream`, direction
 *                  from the pointers (unified addressing); with sync != 0 it
 *                  then waits for the stream.
 * gp_stream_synchronize  waits for the work queued on `stream`. */
int gp_device_alloc(void **ptr, int64_t bytes, void *stream);
int gp_device_free(void *ptr, void *stream);
int gp_host_alloc(void **ptr, int64_t bytes);
int gp_host_free(void *ptr);
int gp_copy(void *dst, const void *src, int64_t bytes, int sync, void *stream);
int gp_stream_synchronize(void *stream);

/* ------------------------------------------------------------ Mat */
typedef struct gp_mat_s *gp_mat;

/* CSR from host arrays in the reference's SeqAIJ layout (int64 indptr and
 * indices, ascending columns per row).  Replaces the Mat storage of
 * python/mojopetsc4py/PETSc/Mat.py:310-344 (setValuesCSR) on the device. */
int gp_mat_create(gp_mat *out, int64_t nrows, int64_t ncols, int64_t nnz,
                  const int64_t *indptr, const int64_t *indices, const double *values);
/* Same from int32 host arrays. */
int gp_mat_create_i32(gp_mat *out, int64_t nrows, int64_t ncols, int64_t nnz,
                      const int32_t *indptr, const int32_t *indices, const double *values);
int gp_mat_destroy(gp_mat A);
/* New values for the same pattern (host or device pointer). */
int gp_mat_set_values(gp_mat A, const double *values, int on_device, void *stream);
/* Device pointer of the values array (valid until gp_mat_destroy).  After
 * writing values through it, call gp_mat_set_values(A, that pointer, 1, s):
 * no copy is made, and the copies derived from the values (the FP32 copy of
 * the mixed form, A^T's values for gp_mat_mult_transpose) are refreshed on
 * their next use. */
int gp_mat_values_ptr(gp_mat A, double **d_values);
int gp_mat_info(gp_mat A, int64_t *nrows, int64_t *ncols, int64_t *nnz);
/* Bytes of column data the SpMV reads per stored entry: 2 where the matrix
 * takes the row-per-thread form and every |column - row| fits 16 bits (the
 * kernels then read row-relative 16-bit offsets, made at creation), else 4
 * (32-bit column indices).  Either way each row is summed in the same order
 * with the same operations.  No counterpart in the reference. */
int gp_mat_spmv_index_bytes(gp_mat A, int32_t *bytes);
/* y = A x.        Replaces MatMult_SeqAIJ (src/ported.mojo:380-391). */
int gp_mat_mult(gp_mat A, const double *x, double *y, void *stream);
/* y = A x + v.    Replaces MatMultAdd_SeqAIJ (src/ported.mojo:394-405). */
int gp_mat_mult_add(gp_mat A, const double *x, const double *v, double *y, void *stream);
/* y = A^T x.      Replaces MatMultTranspose_SeqAIJ (src/ported.mojo:408-431). */
int gp_mat_mult_transpose(gp_mat A, const double *x, double *y, void *stream);
/* MatTranspose (python/mojopetsc4py/PETSc/Mat.py:555-563, 683-746): a new
 * device matrix holding A^T (values gathered on the device through the cached
 * transpose pattern).  gp_mat_transpose_values refreshes At's values after A's
 * changed (MAT_REUSE_MATRIX). */
int gp_mat_transpose(gp_mat A, gp_mat *out, void *stream);
int gp_mat_transpose_values(gp_mat A, gp_mat At, void *stream);
/* out[k] = alpha * u[i] * v[j] for every stored nonzero k = (i, j) of A: the
 * gradient of a loss through A x = b with respect to A's stored values is
 * gp_mat_outer_on_pattern(A, lambda, x, -1, ...) with lambda = A^-T dL/dx.
 * No counterpart in the reference (its adjoint is not on the device). */
int gp_mat_outer_on_pattern(gp_mat A, const double *u, const double *v, double alpha,
                            double *out, void *stream);

/* d = diag(A).    Replaces MatGetDiagonal_SeqAIJ (src/ported.mojo:434-447). */
int gp_mat_get_diagonal(gp_mat A, double *d, void *stream);
/* The matrix's CSR copied to host arrays (int64 indptr[nrows+1], int64
 * indices[nnz], values[nnz]; nnz from gp_mat_info). */
int gp_mat_get_csr(gp_mat A, int64_t *indptr, int64_t *indices, double *values, void *stream);

/* ------------------------------------------------------------ assembly
 * Matrix assembly on the device; the reference assembles in Python
 * (python/mojopetsc4py/PETSc/Mat.py:383-413, 682-746).
 *
 * gp_coo_assemble  CSR (host arrays: int64 indptr[nrows+1]; indices and
 *                  out_values of capacity >= nentries) from entries given in
 *                  call order.  For each (row, col) the entries fold from
 *                  0.0: add[e] != 0 adds (value + v, rounded), add[e] == 0
 *                  sets -- MatSetValues with ADD_VALUES / INSERT_VALUES in
 *                  that order (Mat.py:434-439).  Columns ascend in each row;
 *                  *nnz receives the number of distinct entries.  GP_ERR_ARG
 *                  when an index is out of range.
 * gp_dense_to_csr  CSR of the entries v != 0.0 of a row-major dense host
 *                  array, row by row in column order (from_dense,
 *                  Mat.py:719-746); GP_ERR_ARG with *nnz set when more than
 *                  `capacity` entries are nonzero.
 * The sorts are stable radix sorts on the device. */
int gp_coo_assemble(int64_t nrows, int64_t ncols, int64_t nentries, const int64_t *rows,
                    const int64_t *cols, const double *values, const uint8_t *add,
                    int64_t *indptr, int64_t *indices, double *out_values, int64_t *nnz,
                    void *stream);
int gp_dense_to_csr(int64_t nrows, int64_t ncols, const double *dense, int64_t capacity,
                    int64_t *indptr, int64_t *indices, double *values, int64_t *nnz,
                    void *stream);

/* ------------------------------------------------------------ Vec */
/* Elementwise operations (src/ported.mojo:75-341, src/simdvec.mojo:40-319).
 * Operand roles per op (y is written):
 *   0 copy y=x, 1 set y=alpha, 2 scale y*=alpha, 3 shift y+=alpha,
 *   4 axpy y+=alpha x, 5 aypx y=x+alpha y, 6 axpby y=alpha x+beta y,
 *   7 axpbypcz y=alpha x+beta w+gamma y, 8 waxpy y=alpha x+w,
 *   9 pointwise mult y=x.*w, 10 divide y=x./w, 11 min, 12 max, 13 maxabs,
 *   14 reciprocal (y), 15 exp, 16 log, 17 sqrtabs, 18 abs, 19 chop(alpha),
 *   20 swap(y,x), 21 zero, 22 scale-set y=x*alpha, 23 divide y=y/alpha.
 * Scalar branches follow the reference (VecAYPX alpha 0/1, VecAXPBY beta 0 /
 * alpha 0, VecSet alpha 0). */
int gp_vec_map(int op, int64_t n, double *y, const double *x, const double *w,
               double alpha, double beta, double gamma, void *stream);
/* y += sum_k alpha[k] x[k]; alpha and the pointer array on the host. */
int gp_vec_maxpy(int64_t n, double *y, int64_t nv, const double *alpha,
                 const double *const *xs, void *stream);
/* Reductions into host memory: 0 dot(x,y), 1 sum x^2, 2 sum|x|, 3 sum x,
 * 4 (x.y, x.x), 5 max|x| (first NaN adopted).  Replaces the blocked
 * reductions of src/simdvec.mojo:332-488. */
int gp_vec_reduce(int op, int64_t n, const double *x, const double *y, double *out,
                  void *stream);
/* gp_vec_reduce without allocation, for callers that cannot let a library
 * allocate device memory (a host application with a fixed device-memory
 * budget or its own allocator, a loop that must not pay an allocation's
 * implicit synchronisation).  Same ops and the same kernels as
 * gp_vec_reduce; the result (2 doubles for op 4, else 1) goes to `out`, a
 * caller-owned DEVICE buffer, and the call does not synchronise.  Scratch is
 * a fixed 16 KB area of the library's static device memory (1024 per-CTA
 * partials per value and a ticket word, which starts at zero and which every
 * call leaves at zero).  n must not exceed 2^31 - 1 (GP_ERR_ARG otherwise).
 * There is one scratch area per device, so calls that overlap on a device
 * (different streams or threads with no ordering between them) race: order
 * them.  The first call on each device looks the area up
 * (cudaGetSymbolAddress) and must precede any stream capture.  No counterpart
 * in the reference (its reductions run on the host). */
int gp_vec_reduce_static(int op, int64_t n, const double *x, const double *y, double *out,
                         void *stream);
/* VecMin/VecMax (src/ported.mojo:165-196): value and first index. */
int gp_vec_minmax(int64_t n, const double *x, int is_max, int64_t *idx, double *val,
                  void *stream);
/* max |x_i / y_i| with x_i where y_i == 0 (src/simdvec.mojo:491-500). */
int gp_vec_max_pointwise_divide(int64_t n, const double *x, const double *y, double *out,
                                void *stream);

/* ------------------------------------------------------------ PC */
typedef struct gp_pc_s *gp_pc;

/* Preconditioner options; defaults are those of
 * python/mojopetsc4py/PETSc/PC.py:108-148. */
typedef struct {
  int32_t type;        /* 0 none, 2 jacobi, 4 sor, 5 ilu, 6 icc */
  int32_t jacobi_type; /* 0 diagonal, 1 rowmax, 2 rowl1, 3 rowsum */
  int32_t use_abs;
  int32_t fix_diag;
  double rowl1_scale;
  double omega;
  double fshift;
  int32_t sor_flag;    /* MatSORType bits, default 12|16 */
  int32_t levels;      /* factor levels of fill */
  int32_t ordering;    /* 0 natural, 1 rcm, 2 multicolour (greedy colouring; not
                          in the reference, which has natural and rcm) */
  int32_t reserved;
} gp_pc_options;

void gp_pc_options_default(gp_pc_options *o);
int gp_pc_create(gp_pc *out);
int gp_pc_destroy(gp_pc pc);
int gp_pc_set_options(gp_pc pc, const gp_pc_options *o);
/* Set-up for the operator A: Jacobi diagonals, SOR diagonal, or the ILU/IC
 * symbolic phase (host) followed by the numeric factorisation (device).
 * Replaces PC.setUp (python/mojopetsc4py/PETSc/PC.py:315-492). */
int gp_pc_setup(gp_pc pc, gp_mat A, void *stream);
/* y = M^-1 x.  Replaces KSP_PCApply (src/ksp.mojo:155-198). */
/* Failure detection: every device wait of the triangular sweeps and the
 * numeric factorisation has an iteration budget; when it runs out the kernel
 * records GP_ERR_TIMEOUT, returns, and the call that launched it reports
 * GP_ERR_TIMEOUT (the context stays usable).  gp_wait_probe runs that wait
 * once, on a flag that nothing sets (set = 0: returns GP_ERR_TIMEOUT after
 * `spins` polls) or on a ready one (set = 1: GP_OK).  No counterpart in the
 * reference (its sweeps are sequential host loops). */
int gp_wait_probe(int32_t spins, int32_t set, void *stream);
/* Form of the ILU/IC/SOR triangular sweeps laid out by later PC set-ups.
 *   tiles = 0       the level-ordered form: rows in dependency-level order,
 *                   32 rows a warp, each value passed through L2.
 *   tiles = 1       (default) the chunked form where a simulated schedule
 *                   of it beats the level-ordered form: runs of consecutive
 *                   rows, each chunk walked level by level by one warp with
 *                   in-chunk values in shared memory.
 *   tile_rows > 0   force the chunked form with this many rows a chunk (it
 *                   still falls back when the chunk does not fit in shared
 *                   memory); 0 lets the set-up choose.
 * Both forms give bit-identical results.  Default from GPETSC_SWEEP_TILES
 * and GPETSC_TILE_ROWS.  No counterpart in the reference (its sweeps are
 * sequential host loops). */
int gp_set_sweep_form(int32_t tiles, int32_t tile_rows);
/* Which form a set-up PC's sweeps got: for the forward (which = 0) and the
 * backward (which = 1) sweep, and the two sweeps of the transposed apply
 * (2: U^T, 3: L^T; reported once a transposed apply has prepared them),
 * tiled (0/1), rows per chunk and chunks (0 when not tiled).  No counterpart
 * in the reference. */
int gp_pc_sweep_form(gp_pc pc, int32_t which, int32_t *tiled, int32_t *rows_per_chunk,
                     int32_t *chunks);
/* Brick form of the sweeps of later set-ups, for sweeps whose dependencies are
 * the unit steps of a Cartesian grid in natural order (5-/7-point stencils and
 * operators with their pattern): CTAs take bricks of lines_j grid lines of one
 * plane and each thread walks one line, so most values pass through registers
 * and shared memory instead of L2; the values of neighbouring bricks are
 * fetched into a shared-memory ring by fetch warps.
 *   mode 0  never;  1 where its model beats the other forms;
 *   2  wherever the grid structure is found.
 *   lines_j in 1..128 forces the brick's lines; 0 lets the set-up choose.
 *   lines_k must be 0 or 1 (a brick lies in one plane).  max_ctas > 0 caps
 *   the persistent grid (each CTA then walks several bricks); 0 sizes it to
 *   the device.
 * Bit-identical to the other forms.  Defaults from GPETSC_SWEEP_BRICKS and
 * GPETSC_BRICK_LINES.  No counterpart in the reference. */
int gp_set_sweep_bricks(int32_t mode, int32_t lines_j, int32_t lines_k, int32_t max_ctas);
/* Whether a set-up PC's forward (which = 0) or backward (1) sweep got the
 * brick form, and dims[5] = grid nx, ny, nz and the brick's lines_j, lines_k
 * (zeros otherwise).  No counterpart in the reference. */
int gp_pc_sweep_bricks(gp_pc pc, int32_t which, int32_t *brick, int32_t *dims);
/* Same pattern, new operator values: redo only the numeric phase (ILU/IC factor
 * values on the device, Jacobi diagonals) in the arrays of the last set-up;
 * solver graphs captured with this PC stay valid. */
int gp_pc_update_values(gp_pc pc, void *stream);
int gp_pc_apply(gp_pc pc, const double *x, double *y, void *stream);
/* y = M^-T x, the true transpose of the preconditioner: for ILU the
 * triangular solves with U^T and then L^T of the same factor (sweeps laid out
 * on the first call, so make that call outside any stream capture); none,
 * Jacobi and IC are symmetric and apply M^-1; SOR returns GP_ERR_UNSUPPORTED.
 * No counterpart in the reference, whose applyTranspose is the plain apply
 * (python/mojopetsc4py/PETSc/PC.py:635-642); it is what PCApplyTranspose of
 * upstream PETSc computes. */
int gp_pc_apply_transpose(gp_pc pc, const double *x, double *y, void *stream);
/* Jacobi's symmetric half (src/ksp.mojo:201-208); other types apply M^-1. */
int gp_pc_apply_symmetric(gp_pc pc, const double *x, double *y, void *stream);
/* Factor sizes and host copies in the reference's layout (ILU: bi, bj, ba,
 * bdiag of n+1; IC: bi, bj, ba, bdiag of n+1).  Any output may be NULL. */
int gp_pc_factor_info(gp_pc pc, int64_t *n, int64_t *nslots);
int gp_pc_factor_get(gp_pc pc, int64_t *bi, int64_t *bj, double *ba, int64_t *bdiag,
                     int64_t *perm);

/* ------------------------------------------------------------ KSP */
typedef struct gp_ksp_s *gp_ksp;

/* Solver options; the fields of the reference's cfg/cfgi blocks
 * (src/ksp.mojo:13-23, python/mojopetsc4py/PETSc/KSP.py:457-494). */
typedef struct {
  int32_t type;        /* 2 cg, 6 bcgs, 12 gmres, 40 fgmres */
  int32_t normtype;    /* 1 none, 2 preconditioned, 3 unpreconditioned, 4 natural */
  int32_t pc_side;     /* 0 left, 1 right, 2 symmetric */
  int32_t guess_zero;
  int32_t min_it;
  int32_t chknorm;
  int32_t convmaxits;
  int32_t max_it;
  int32_t restart;
  int32_t orthog;      /* 0 classical Gram-Schmidt */
  int32_t cgstype;     /* 0 never, 1 if needed, 2 always */
  int32_t seed_rhs;    /* nonzero guess: rnorm0 from rhs_norm */
  double rtol, atol, divtol, haptol, breakdowntol, rhs_norm;
} gp_ksp_options;

typedef struct {
  int64_t its;
  int64_t reason;   /* KSPConvergedReason ordinal */
  double rnorm;
} gp_ksp_result;

void gp_ksp_options_default(gp_ksp_options *o);
int gp_ksp_create(gp_ksp *out);
int gp_ksp_destroy(gp_ksp ksp);
int gp_ksp_set_options(gp_ksp ksp, const gp_ksp_options *o);
/* Solve A x = b with preconditioner pc; b and x are device vectors (with the
 * default zero initial guess, x is zeroed first).  The residual history
 * (its+1 norms) goes to hist (host, may be NULL).
 * Replaces mp_ksp_solve_{cg,bcgs,gmres,fgmres} (src/capi.mojo:383-424)
 * behind KSP.solve (python/mojopetsc4py/PETSc/KSP.py:367-449). */
int gp_ksp_solve(gp_ksp ksp, gp_mat A, gp_pc pc, const double *b, double *x,
                 gp_ksp_result *result, double *hist, int64_t hist_len, void *stream);

/* transpose = 1: later solves solve A^T x = b with the same operator and
 * preconditioner -- every multiply by A becomes one by A^T (the cached
 * transposed pattern) and every preconditioner apply the true transposed one
 * (gp_pc_apply_transpose), as upstream PETSc's KSPSolveTranspose does; the
 * fused CG kernels are not used then.  0 (the default) solves A x = b.  No
 * counterpart in the reference. */
int gp_ksp_set_transpose(gp_ksp ksp, int transpose);
/* How later solves launch their kernels: 0 one captured CUDA graph per solve
 * (the loop is a conditional node), 1 the same kernels launched one by one
 * from a host loop that polls convergence every few iterations (each kernel
 * then appears on its own in a profiler's launch list), -1 (the default) the
 * process-wide choice of the environment (GPETSC_KSP_GRAPH=0 selects the
 * host loop).  Results are identical.  No counterpart in the reference. */
int gp_ksp_set_launch_form(gp_ksp ksp, int form);

/* Kernel-launch accounting of the last solve: loop trips, kernels outside the
 * loop (prologue, epilogue) and kernels per trip.  Kernels launched =
 * top_kernels + trips * body_kernels. */
int gp_ksp_stats(gp_ksp ksp, int64_t *trips, int64_t *top_kernels, int64_t *body_kernels);


/* ------------------------------------------------------------ mixed precision
 * A x = b to rtol on the true FP64 residual (||b - A x|| <= rtol ||b||) by
 * FP64 iterative refinement around an FP32 inner FGMRES(restart) cycle
 * preconditioned with the ILU(0) factor of `pc` (an ILU gp_pc set up on A)
 * in FP32.  tri_sweeps > 0 applies each triangle of the factor with that many
 * passes (inexact, tolerated by the flexible method): with tri_block = 0
 * point-Jacobi passes (bandwidth-bound); with tri_block != 0 block passes,
 * each solving runs of tri_block consecutive rows exactly (level by level in
 * shared memory, -1: length chosen from the matrix) with the couplings between
 * runs from the previous pass.  tri_sweeps = 0 applies the triangles exactly
 * with the level-scheduled FP64 sweeps.  Each pass runs
 * one inner cycle to inner_rtol; max_outer caps the passes.  x (device) is
 * overwritten (zero initial guess).  No counterpart in the reference. */
typedef struct gp_mixed_s *gp_mixed;
typedef struct {
  int32_t restart;
  int32_t max_outer;
  int32_t tri_sweeps;
  int32_t tri_block;
  double rtol;
  double inner_rtol;
} gp_mixed_options;
typedef struct {
  int32_t passes;      /* refinement passes (inner cycles) run */
  int32_t inner_its;   /* FGMRES steps in total */
  int32_t converged;   /* 1 when the true residual met rtol */
  int32_t reserved;
  double relres;       /* final ||b - A x|| / ||b|| (FP64) */
} gp_mixed_result;
void gp_mixed_options_default(gp_mixed_options *o);
int gp_mixed_create(gp_mixed *out);
int gp_mixed_destroy(gp_mixed m);
int gp_mixed_solve(gp_mixed m, gp_mat A, gp_pc pc, const gp_mixed_options *o, const double *b,
                   double *x, gp_mixed_result *result, void *stream);

/* ------------------------------------------------------------ batched CG
 * Many independent SPD systems with nrhs right-hand sides each, solved
 * together: one block-diagonal CSR (system s owns rows sys_rows[s] ..
 * sys_rows[s+1]-1 and may only couple to them; int64 host arrays as in
 * gp_mat_create) and row-major multi-vectors (entry (row, r) at
 * row * nrhs + r, device memory).  Every (system, column) pair runs its own
 * PETSc CG recurrence (src/ksp.mojo:271-389, preconditioned norm) with its own
 * stopping test; pairs that stop are frozen and finished systems drop out.
 * precision 0: FP64 CG.  precision 1: FP32 inner CG (FP32 values, vectors and
 * dot accumulation) to inner_rtol inside FP64 iterative refinement, stopping
 * when the true residual ||b - A x|| <= rtol ||b|| per pair (max_it then
 * caps the inner iterations of each pass, max_outer the passes).
 * nrhs must be 1, 2, 4, 8 or 16; pc_type 0 (none) or 2 (Jacobi).
 * gp_batch_autotune times the sparse pass for every (CTA size, columns per
 * thread, tile rows) and keeps the fastest, separately for the FP64 and the
 * FP32 pass; gp_batch_tuning reports the choice for a precision (0 / 1).
 * Outputs (host, nsys * nrhs entries, each may be NULL): iterations (total
 * inner iterations for precision 1), converged reason, and the final true
 * relative residual ||b - A x|| / ||b|| computed in FP64.
 * No counterpart in the reference (its solves are one system at a time). */
typedef struct gp_batch_s *gp_batch;
typedef struct {
  int32_t pc_type;     /* 0 none, 2 jacobi */
  int32_t precision;   /* 0 FP64, 1 FP32 inner + FP64 refinement */
  int32_t max_it;
  int32_t max_outer;
  double rtol, atol, divtol;
  double inner_rtol;
} gp_batch_options;
void gp_batch_options_default(gp_batch_options *o);
int gp_batch_create(gp_batch *out, int64_t nsys, const int64_t *sys_rows,
                    const int64_t *indptr, const int64_t *indices, const double *values,
                    int32_t nrhs, void *stream);
int gp_batch_destroy(gp_batch b);
int gp_batch_autotune(gp_batch b, void *stream);
int gp_batch_tuning(gp_batch b, int32_t precision, int32_t *block, int32_t *vector_width,
                    int32_t *tile_rows, double *spmm_us);
int gp_batch_solve_cg(gp_batch b, const gp_batch_options *o, const double *B, double *X,
                      int64_t *its, int32_t *reason, double *relres, int32_t *passes,
                      void *stream);

/* ------------------------------------------------------------ mp_* (reference host ABI) */
/* Mat (src/capi.mojo:32-65) */
void mp_mat_mult(const double *x, double *y, const int64_t *irow, const int64_t *icol,
                 const double *data, int64_t nrow);
void mp_mat_mult_add(const double *x, double *y, const int64_t *irow, const int64_t *icol,
                     const double *data, int64_t nrow);
void mp_mat_mult_transpose(const double *x, double *y, const int64_t *irow,
                           const int64_t *icol, const double *data, int64_t nrow,
                           int64_t ncols);
void mp_mat_get_diagonal(double *diag, const int64_t *irow, const int64_t *icol,
                         const double *data, int64_t nrow);
void mp_mat_scale(double *data, int64_t nnz, double alpha);
void mp_mat_zero_entries(double *data, int64_t nnz);
/* Vec (src/capi.mojo:69-238) */
void mp_vec_pointwise_mult(double *w, const double *x, const double *y, int64_t n);
void mp_vec_pointwise_divide(double *w, const double *x, const double *y, int64_t n);
void mp_vec_pointwise_min(double *w, const double *x, const double *y, int64_t n);
void mp_vec_pointwise_max(double *w, const double *x, const double *y, int64_t n);
void mp_vec_pointwise_max_abs(double *w, const double *x, const double *y, int64_t n);
void mp_vec_norm(const double *x, int64_t ntype, double *z, int64_t n);
void mp_vec_dot(const double *x, const double *y, double *val, int64_t n);
void mp_vec_tdot(const double *x, const double *y, double *val, int64_t n);
void mp_vec_dot_norm2(const double *x, const double *y, double *sval, double *rval, int64_t n);
void mp_vec_sum(const double *x, double *val, int64_t n);
void mp_vec_mean(const double *x, double *val, int64_t n);
void mp_vec_max(const double *x, int64_t *idx, double *z, int64_t n);
void mp_vec_min(const double *x, int64_t *idx, double *z, int64_t n);
void mp_vec_normalize(double *x, double *v, int64_t n);
void mp_vec_reciprocal(double *x, int64_t n);
void mp_vec_exp(double *x, int64_t n);
void mp_vec_log(double *x, int64_t n);
void mp_vec_sqrtabs(double *x, int64_t n);
void mp_vec_chop(double *x, int64_t n, double tol);
void mp_vec_abs(double *x, int64_t n);
void mp_vec_conjugate(double *x, int64_t n);
void mp_vec_copy(const double *x, double *y, int64_t n);
void mp_vec_swap(double *x, double *y, int64_t n);
void mp_vec_set(double *x, double alpha, int64_t n);
void mp_vec_zero_entries(double *x, int64_t n);
void mp_vec_scale(double *x, double alpha, int64_t n);
void mp_vec_shift(double *x, double alpha, int64_t n);
void mp_vec_axpy(double *y, double alpha, const double *x, int64_t n);
void mp_vec_aypx(double *y, double alpha, const double *x, int64_t n);
void mp_vec_axpby(double *y, double alpha, double beta, const double *x, int64_t n);
void mp_vec_axpbypcz(double *z, double alpha, double beta, double gamma, const double *x,
                     const double *y, int64_t n);
void mp_vec_waxpy(double *w, double alpha, const double *x, const double *y, int64_t n);
void mp_vec_maxpy(double *y, int64_t nv, const double *alpha, const int64_t *x, int64_t n);
void mp_vec_max_pointwise_divide(const double *x, const double *y, double *rval, int64_t n);
/* PC and factorisation (src/capi.mojo:242-379) */
int64_t mp_mat_get_diagonal_markers(const int64_t *irow, const int64_t *icol, int64_t *diag,
                                    int64_t nrow);
void mp_pc_jacobi_setup(double *diag, int64_t jtype, int64_t useabs, int64_t fixdiag,
                        double scale, const int64_t *irow, const int64_t *icol,
                        const double *data, int64_t nrow, double *didx);
void mp_pc_jacobi_setup_symmetric(double *diagsqrt, int64_t jtype, const int64_t *irow,
                                  const int64_t *icol, const double *data, int64_t nrow);
void mp_pc_jacobi_apply(double *y, const double *x, const double *diag, int64_t n);
void mp_pc_sor_apply(const double *x, double *y, const int64_t *irow, const int64_t *icol,
                     const double *data, const int64_t *dmark, double *idiag, double *mdiag,
                     double *t, double omega, double fshift, int64_t flag, int64_t nrow);
void mp_pc_ilu_apply(const double *b, double *x, double *tmp, const int64_t *bi,
                     const int64_t *bj, const double *ba, const int64_t *bdiag,
                     const int64_t *r, const int64_t *c, int64_t nrow);
int64_t mp_pc_icc_apply(const double *b, double *x, const int64_t *ui, const int64_t *uj,
                        const double *ua, const int64_t *udiag, const int64_t *c,
                        double *scratch, int64_t nrow);
int64_t mp_pc_ilu_numeric(double *ba, double *rtmp, const int64_t *irow, const int64_t *icol,
                          const double *data, const int64_t *bi, const int64_t *bj,
                          const int64_t *bdiag, const int64_t *r, const int64_t *ic,
                          int64_t nrow);
void mp_pc_icc_numeric(double *ua, double *rtmp, int64_t *il, int64_t *c2r,
                       const int64_t *irow, const int64_t *icol, const double *data,
                       const int64_t *ui, const int64_t *uj, const int64_t *udiag,
                       const int64_t *r, const int64_t *riip, int64_t nrow);
int64_t mp_ilu_symbolic_ilu0(int64_t *bi, int64_t *bj, int64_t *bdiag, const int64_t *adiag,
                             const int64_t *irow, const int64_t *icol, int64_t nrow);
int64_t mp_ilu_symbolic(int64_t *bi, int64_t *bj, int64_t *bjlvl, int64_t *bdiag,
                        const int64_t *irow, const int64_t *icol, const int64_t *r,
                        const int64_t *ic, int64_t levels, int64_t cap, int64_t *scratch,
                        int64_t nrow);
void mp_ilu_contiguous_lu(const int64_t *bjsrc, int64_t *bi, int64_t *bdiag, int64_t *bj,
                          int64_t n);
int64_t mp_icc_symbolic(int64_t *ui, int64_t *uj, int64_t *ujlvl, int64_t *udiag,
                        const int64_t *irow, const int64_t *icol, const int64_t *r,
                        const int64_t *riip, int64_t levels, int64_t cap, int64_t *scratch,
                        int64_t nrow, int64_t scratchlen);
void mp_icc_contiguous_cholesky(const int64_t *ujsrc, const int64_t *ui, const int64_t *udiag,
                                int64_t *bi, int64_t *bdiag, int64_t *bj, int64_t n);
void mp_ordering_rcm(int64_t *perm, int64_t *level, int64_t *visited, int64_t *queue,
                     const int64_t *irow, const int64_t *icol, int64_t nrow);
/* KSP (src/capi.mojo:383-424); cfg/cfgi/pci/pcf as in src/ksp.mojo:13-23 */
void mp_ksp_solve_cg(int64_t n, const int64_t *irow, const int64_t *icol, const double *data,
                     const int64_t *pci, const double *pcf, double *pstmp, double *work,
                     double *cfg, int64_t *cfgi, const double *b, double *x);
void mp_ksp_solve_bcgs(int64_t n, const int64_t *irow, const int64_t *icol, const double *data,
                       const int64_t *pci, const double *pcf, double *pstmp, double *work,
                       double *cfg, int64_t *cfgi, const double *b, double *x);
void mp_ksp_solve_gmres(int64_t n, const int64_t *irow, const int64_t *icol, const double *data,
                        const int64_t *pci, const double *pcf, double *pstmp, double *work,
                        double *vv, double *hs, double *cfg, int64_t *cfgi, const double *b,
                        double *x);
void mp_ksp_solve_fgmres(int64_t n, const int64_t *irow, const int64_t *icol,
                         const double *data, const int64_t *pci, const double *pcf,
                         double *pstmp, double *work, double *vv, double *prevec, double *hs,
                         double *cfg, int64_t *cfgi, const double *b, double *x);
/* Status of the last mp_* call on this thread (the reference's mp_* entries
 * return nothing; this reports a CUDA or argument failure instead of hiding
 * it). */
int mp_last_status(void);

#ifdef __cplusplus
}
#endif

#endif /* GPETSC_H */
