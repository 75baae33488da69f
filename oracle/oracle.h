/* CPU oracle for the sequential Krylov path: shared declarations.
 *
 * TEST INFRASTRUCTURE ONLY.  This directory is a plain-C restatement of the
 * reference's CPU algorithm (src/ksp.mojo, src/ported.mojo, src/simdvec.mojo,
 * src/simd.mojo and src/factor.mojo of lee101/mojo-petsc4py).  It exists to
 * check the CUDA product path and to time the reference's CPU path; the
 * product library never links, loads or calls it.
 *
 * It exports the reference's host C ABI (src/capi.mojo:32-424): every buffer
 * is a plain host pointer, every index array is int64, every scalar a double,
 * and the caller owns every buffer including scratch.
 *
 * Floating point follows the reference's operation order exactly.  The build
 * uses -ffp-contract=off so that `a += x * y` is a rounded multiply followed by
 * a rounded add, as the reference writes it.  The reductions keep the
 * reference's blocked order: four SIMD accumulators of SW = 4 lanes over
 * blocks of BLK = 16 (src/simd.mojo:18,32-33), then one-vector steps, then a
 * scalar tail.  The lane reduction of a 4-wide accumulator is not spelled out
 * in the reference's source; the oracle uses the halving tree
 * (l0 + l2) + (l1 + l3), which is how a power-of-two SIMD reduce folds.
 */
#ifndef GPETSC_ORACLE_H
#define GPETSC_ORACLE_H

#include <stdint.h>

typedef int64_t I;

#define O_SW 4
#define O_BLK 16

/* petscpc.h PCType ordinals, src/ported.mojo:479-483 */
#define O_PC_NONE 0
#define O_PC_JACOBI 2
#define O_PC_SOR 4
#define O_PC_ILU 5
#define O_PC_ICC 6

/* MatSORType bits, src/ported.mojo:491-496 */
#define O_SOR_FORWARD_SWEEP 1
#define O_SOR_BACKWARD_SWEEP 2
#define O_SOR_LOCAL_FORWARD_SWEEP 4
#define O_SOR_LOCAL_BACKWARD_SWEEP 8
#define O_SOR_ZERO_INITIAL_GUESS 16

/* simdvec restatements (src/simdvec.mojo) used across files */
double o_dot(const double *x, const double *y, I n);
void o_dot_norm2(const double *x, const double *y, I n, double *d, double *q);
double o_norm2sq(const double *x, I n);
double o_asum(const double *x, I n);
double o_total(const double *x, I n);
void o_mdot_basis(const double *x, const double *y, I nv, I n, double *res);
void o_maxpy(double *y, const double *alpha, I n, I nv, const double *base);
double o_vecnorm2(const double *x, I n);

/* ported.mojo Vec wrappers used by the drivers */
void o_copy(const double *x, double *y, I n);
void o_set(double *x, double alpha, I n);
void o_scale(double *x, double alpha, I n);
void o_axpy(double *y, double alpha, const double *x, I n);
void o_aypx(double *y, double alpha, const double *x, I n);
void o_axpbypcz(double *z, double alpha, double beta, double gamma,
                const double *x, const double *y, I n);
void o_waxpy(double *w, double alpha, const double *x, const double *y, I n);
void o_pointwise_mult(double *w, const double *x, const double *y, I n);

/* Mat kernels */
void o_matmult(const double *x, double *y, const I *irow, const I *icol,
               const double *data, I nrow);

/* PC applies */
void o_pc_sor_apply(const double *x, double *y, const I *arow, const I *acol,
                    const double *adata, const I *dmark, double *idiag,
                    double *mdiag, double *t, double omega, double fshift,
                    I its, I lits, I flag, I nrow);
void o_pc_ilu_apply(const double *b, double *x, double *tmp, const I *bi,
                    const I *bj, const double *ba, const I *bdiag, const I *r,
                    const I *c, I nrow);
I o_pc_icc_apply(const double *b, double *x, const I *ui, const I *uj,
                 const double *ua, const I *udiag, const I *c, double *scratch,
                 I nrow);

/* linked-list helpers of the symbolic phase, src/ported.mojo:759-861 */
I o_ll_insert_location(I assume_sorted, I k, I idx_start, I entry, I nlnk,
                       I *lnkdata, I *lnk);
I o_incomplete_ll_init(I nidx, const I *idx, I idx_start, const I *perm,
                       I *lnk, I *lnklvl, I *bt);
I o_incomplete_ll_add(I nidx, const I *idx, double level, const I *idxlvl,
                      I idx_start, I *lnk, I *lnklvl, I *bt, I prow_offset,
                      I assume_sorted);
void o_incomplete_ll_clean(I idx_start, I lnk_max, I nlnk, I *lnk, I *lnklvl,
                           I *indices, I *indiceslvl, I *bt);

#endif
