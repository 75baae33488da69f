/* Oracle: CSR (SeqAIJ) matrix kernels.  TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * Restates src/ported.mojo:354-476 (diagonal markers, MatMult, MatMultAdd,
 * MatMultTranspose, MatGetDiagonal, MatScale, MatZeroEntries) with the
 * reference's C ABI names (src/capi.mojo:32-65, :242-246).  Rows are summed
 * in ascending column-slot order starting from 0.0 (or from y for MatMultAdd).
 */
#include "oracle.h"

/* ported.mojo:354-377 MatGetDiagonalMarkers_SeqAIJ */
I mp_mat_get_diagonal_markers(const I *irow, const I *icol, I *diag, I n) {
    I dense = 1;
    for (I i = 0; i < n; i++) {
        I bl = irow[i], be = irow[i + 1];
        diag[i] = be;
        for (I j = bl; j < be; j++)
            if (icol[j] == i) {
                diag[i] = j;
                break;
            }
        if (diag[i] == be) dense = 0;
    }
    return dense;
}

/* ported.mojo:380-391 MatMult_SeqAIJ */
void o_matmult(const double *x, double *y, const I *irow, const I *icol,
               const double *data, I nrow) {
    for (I i = 0; i < nrow; i++) {
        double sum = 0.0;
        for (I j = irow[i]; j < irow[i + 1]; j++) sum += data[j] * x[icol[j]];
        y[i] = sum;
    }
}

void mp_mat_mult(const double *x, double *y, const I *irow, const I *icol,
                 const double *data, I nrow) {
    o_matmult(x, y, irow, icol, data, nrow);
}

/* ported.mojo:394-405 MatMultAdd_SeqAIJ: y = A x + y */
void mp_mat_mult_add(const double *x, double *y, const I *irow, const I *icol,
                     const double *data, I nrow) {
    for (I i = 0; i < nrow; i++) {
        double sum = y[i];
        for (I j = irow[i]; j < irow[i + 1]; j++) sum += data[j] * x[icol[j]];
        y[i] = sum;
    }
}

/* ported.mojo:408-431 MatMultTranspose_SeqAIJ: clear ncols entries, then
 * scatter row by row */
void mp_mat_mult_transpose(const double *x, double *y, const I *irow, const I *icol,
                           const double *data, I nrow, I ncols) {
    for (I j = 0; j < ncols; j++) y[j] = 0.0;
    for (I i = 0; i < nrow; i++) {
        double xi = x[i];
        for (I jb = irow[i]; jb < irow[i + 1]; jb++) {
            I c = icol[jb];
            y[c] = y[c] + data[jb] * xi;
        }
    }
}

/* ported.mojo:434-447 MatGetDiagonal_SeqAIJ: a missing diagonal stays 0 */
void mp_mat_get_diagonal(double *diag, const I *irow, const I *icol,
                         const double *data, I nrow) {
    for (I i = 0; i < nrow; i++) {
        double v = 0.0;
        for (I j = irow[i]; j < irow[i + 1]; j++)
            if (icol[j] == i) {
                v = data[j];
                break;
            }
        diag[i] = v;
    }
}

void mp_mat_scale(double *data, I nnz, double alpha) {
    for (I j = 0; j < nnz; j++) data[j] = data[j] * alpha;
}

void mp_mat_zero_entries(double *data, I nnz) {
    for (I j = 0; j < nnz; j++) data[j] = 0.0;
}
