/* Oracle: preconditioner set-up and applies.  TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * Restates src/ported.mojo:489-1124: Jacobi set-up (all four PCJACOBIType
 * fills, the rowl1 sign fix and scale, the zero-guarded reciprocal, useabs,
 * fixdiag) and apply; the symmetric Jacobi set-up; SOR (MatSOR_SeqAIJ with the
 * zero-initial-guess prologue and the its*lits sweep loop); the ILU and IC
 * triangular solves; the ILU and IC numeric factorisations (shift type none);
 * and the sorted linked-list helpers the symbolic phase uses.  Exported names
 * follow src/capi.mojo:242-322.
 */
#include <math.h>

#include "oracle.h"

void mp_mat_get_diagonal(double *diag, const I *irow, const I *icol,
                         const double *data, I nrow);

/* ported.mojo:570-607 row sums / abs sums / max abs */
static void row_fill(double *dst, I jtype, const I *arow, const I *acol,
                     const double *adata, I nrow) {
    if (jtype == 0) {
        mp_mat_get_diagonal(dst, arow, acol, adata, nrow);
        return;
    }
    for (I i = 0; i < nrow; i++) {
        double s = 0.0;
        for (I j = arow[i]; j < arow[i + 1]; j++) {
            double v = adata[j];
            if (jtype == 1) { /* ROWMAX */
                double a = fabs(v);
                s = a > s ? a : s;
            } else if (jtype == 2) { /* ROWL1 */
                s += fabs(v);
            } else { /* ROWSUM */
                s += v;
            }
        }
        dst[i] = s;
    }
}

/* ported.mojo:505-541 PCSetUp_Jacobi */
void mp_pc_jacobi_setup(double *diag, I jtype, I useabs, I fixdiag, double scale,
                        const I *arow, const I *acol, const double *adata, I nrow,
                        double *didx) {
    row_fill(diag, jtype, arow, acol, adata, nrow);
    if (jtype == 2) {
        mp_mat_get_diagonal(didx, arow, acol, adata, nrow);
        for (I i = 0; i < nrow; i++)
            if (didx[i] < 0.0) diag[i] = -diag[i];
        if (scale != 1.0)
            for (I i = 0; i < nrow; i++) diag[i] = scale * (diag[i] - didx[i]) + didx[i];
    }
    for (I i = 0; i < nrow; i++) diag[i] = (diag[i] == 0.0) ? 0.0 : 1.0 / diag[i];
    if (useabs)
        for (I i = 0; i < nrow; i++) diag[i] = fabs(diag[i]);
    if (fixdiag)
        for (I i = 0; i < nrow; i++)
            if (diag[i] == 0.0) diag[i] = 1.0;
}

/* ported.mojo:544-562 PCSetUp_Jacobi_Symmetric */
void mp_pc_jacobi_setup_symmetric(double *diagsqrt, I jtype, const I *arow,
                                  const I *acol, const double *adata, I nrow) {
    row_fill(diagsqrt, jtype, arow, acol, adata, nrow);
    for (I i = 0; i < nrow; i++) {
        double d = diagsqrt[i];
        if (d < 0.0)
            diagsqrt[i] = 1.0 / sqrt(fabs(-d));
        else if (d > 0.0)
            diagsqrt[i] = 1.0 / sqrt(fabs(d));
        else
            diagsqrt[i] = 1.0;
    }
}

/* ported.mojo:565-567 PCApply_Jacobi */
void mp_pc_jacobi_apply(double *y, const double *x, const double *diag, I n) {
    o_pointwise_mult(y, x, diag, n);
}

/* ported.mojo:610-630 MatInvertDiagonalForSOR_SeqAIJ */
static void sor_invert_diag(double *idiag, double *mdiag, const I *dmark,
                            const double *adata, double omega, double fshift, I nrow) {
    if (omega == 1.0 && fshift <= 0.0) {
        for (I i = 0; i < nrow; i++) {
            mdiag[i] = adata[dmark[i]];
            idiag[i] = 1.0 / adata[dmark[i]];
        }
    } else {
        for (I i = 0; i < nrow; i++) {
            mdiag[i] = adata[dmark[i]];
            idiag[i] = omega / (fshift + adata[dmark[i]]);
        }
    }
}

/* ported.mojo:633-748 PCApply_SOR: x is the right-hand side, y the result */
void o_pc_sor_apply(const double *x, double *y, const I *arow, const I *acol,
                    const double *adata, const I *dmark, double *idiag,
                    double *mdiag, double *t, double omega, double fshift,
                    I its, I lits, I flag, I nrow) {
    I it = its * lits;
    sor_invert_diag(idiag, mdiag, dmark, adata, omega, fshift, nrow);
    int use_t = 0;
    const I fw = O_SOR_FORWARD_SWEEP | O_SOR_LOCAL_FORWARD_SWEEP;
    const I bw = O_SOR_BACKWARD_SWEEP | O_SOR_LOCAL_BACKWARD_SWEEP;
    if (flag & fw) {
        for (I i = 0; i < nrow; i++) {
            double sum = x[i];
            for (I j = arow[i]; j < dmark[i]; j++) sum -= adata[j] * y[acol[j]];
            t[i] = sum;
            y[i] = sum * idiag[i];
        }
        use_t = 1;
    }
    if (flag & bw) {
        for (I i = nrow - 1; i >= 0; i--) {
            double sum = (use_t ? t : x)[i];
            for (I j = dmark[i] + 1; j < arow[i + 1]; j++) sum -= adata[j] * y[acol[j]];
            if (use_t)
                y[i] = (1.0 - omega) * y[i] + sum * idiag[i];
            else
                y[i] = sum * idiag[i];
        }
    }
    it -= 1;
    while (it > 0) {
        it -= 1;
        if (flag & fw) {
            for (I i = 0; i < nrow; i++) {
                double sum = x[i];
                for (I j = arow[i]; j < dmark[i]; j++) sum -= adata[j] * y[acol[j]];
                t[i] = sum;
                for (I j = dmark[i] + 1; j < arow[i + 1]; j++) sum -= adata[j] * y[acol[j]];
                y[i] = (1.0 - omega) * y[i] + sum * idiag[i];
            }
            use_t = 1;
        }
        if (flag & bw) {
            for (I i = nrow - 1; i >= 0; i--) {
                double sum = (use_t ? t : x)[i];
                if (use_t) {
                    for (I j = dmark[i] + 1; j < arow[i + 1]; j++) sum -= adata[j] * y[acol[j]];
                    y[i] = (1.0 - omega) * y[i] + sum * idiag[i];
                } else {
                    for (I j = arow[i]; j < arow[i + 1]; j++) sum -= adata[j] * y[acol[j]];
                    y[i] = (1.0 - omega) * y[i] + (sum + mdiag[i] * y[i]) * idiag[i];
                }
            }
        }
    }
}

/* capi.mojo:266-276: the exported SOR apply runs its = lits = 1 */
void mp_pc_sor_apply(const double *x, double *y, const I *irow, const I *icol,
                     const double *data, const I *dmark, double *idiag, double *mdiag,
                     double *t, double omega, double fshift, I flag, I nrow) {
    o_pc_sor_apply(x, y, irow, icol, data, dmark, idiag, mdiag, t, omega, fshift, 1, 1,
                   flag, nrow);
}

/* ported.mojo:864-899 ILUApplyFactor_SeqAIJ (MatSolve_SeqAIJ) */
void o_pc_ilu_apply(const double *b, double *x, double *tmp, const I *bi,
                    const I *bj, const double *ba, const I *bdiag, const I *r,
                    const I *c, I nrow) {
    if (!nrow) return;
    tmp[0] = b[r[0]];
    for (I i = 1; i < nrow; i++) {
        double sum = b[r[i]];
        for (I j = bi[i]; j < bi[i + 1]; j++) sum -= ba[j] * tmp[bj[j]];
        tmp[i] = sum;
    }
    for (I i = nrow - 1; i >= 0; i--) {
        I v = bdiag[i + 1] + 1;
        I nz = bdiag[i] - bdiag[i + 1] - 1;
        double sum = tmp[i];
        for (I j = 0; j < nz; j++) sum -= ba[v + j] * tmp[bj[v + j]];
        sum = sum * ba[v + nz];
        tmp[i] = sum;
        x[c[i]] = sum;
    }
}

void mp_pc_ilu_apply(const double *b, double *x, double *tmp, const I *bi, const I *bj,
                     const double *ba, const I *bdiag, const I *r, const I *c, I nrow) {
    o_pc_ilu_apply(b, x, tmp, bi, bj, ba, bdiag, r, c, nrow);
}

/* ported.mojo:902-952 ICCApplyFactor_SeqAIJ (MatSolve_SeqSBAIJ_1_inplace):
 * forward in scatter form, backward in gather form */
I o_pc_icc_apply(const double *b, double *x, const I *ui, const I *uj,
                 const double *ua, const I *udiag, const I *c, double *scratch,
                 I nrow) {
    if (!nrow) return 0;
    for (I i = 0; i < nrow; i++) scratch[i] = b[c[i]];
    for (I i = 0; i < nrow; i++) {
        double xi = scratch[i];
        for (I j = ui[i]; j < udiag[i]; j++) {
            I k = uj[j];
            scratch[k] = scratch[k] + ua[j] * xi;
        }
        scratch[i] = xi * ua[udiag[i]];
    }
    for (I i = nrow - 2; i >= 0; i--) {
        double xi = scratch[i];
        for (I j = ui[i]; j < udiag[i]; j++) xi += ua[j] * scratch[uj[j]];
        scratch[i] = xi;
        x[c[i]] = xi;
    }
    x[c[nrow - 1]] = scratch[nrow - 1];
    return 0;
}

I mp_pc_icc_apply(const double *b, double *x, const I *ui, const I *uj, const double *ua,
                  const I *udiag, const I *c, double *scratch, I nrow) {
    return o_pc_icc_apply(b, x, ui, uj, ua, udiag, c, scratch, nrow);
}

/* ported.mojo:957-1037 MatILUFactorNumeric_SeqAIJ, shift type none */
I mp_pc_ilu_numeric(double *ba, double *rtmp, const I *arow, const I *acol,
                    const double *adata, const I *bi, const I *bj, const I *bdiag,
                    const I *r, const I *ic, I nrow) {
    for (I i = 0; i < nrow; i++) {
        for (I jj = bi[i]; jj < bi[i + 1]; jj++) rtmp[bj[jj]] = 0.0;
        for (I jj = bdiag[i + 1] + 1, j = 0; j < bdiag[i] - bdiag[i + 1]; j++, jj++)
            rtmp[bj[jj]] = 0.0;
        I ri = r[i];
        for (I jj = arow[ri]; jj < arow[ri + 1]; jj++) rtmp[ic[acol[jj]]] = adata[jj];

        I jj = bi[i];
        I row = bj[jj];
        jj++;
        I nzl = bi[i + 1] - bi[i];
        for (I k = 0; k < nzl; k++) {
            double pc = rtmp[row];
            if (pc != 0.0) {
                double pv = ba[bdiag[row]];
                double multiplier = pc * pv;
                rtmp[row] = multiplier;
                I pj = bdiag[row + 1] + 1;
                I nz = bdiag[row] - bdiag[row + 1] - 1;
                for (I j = 0; j < nz; j++) {
                    I cc = bj[pj + j];
                    rtmp[cc] = rtmp[cc] - multiplier * ba[pj + j];
                }
            }
            row = bj[jj];
            jj++;
        }
        for (I q = bi[i]; q < bi[i + 1]; q++) ba[q] = rtmp[bj[q]];
        for (I q = bdiag[i + 1] + 1, j = 0; j < bdiag[i] - bdiag[i + 1] - 1; j++, q++)
            ba[q] = rtmp[bj[q]];
        ba[bdiag[i]] = 1.0 / rtmp[i];
    }
    return bdiag[0] + 1;
}

/* ported.mojo:1040-1124 MatICCFactorNumeric_SeqAIJ (MatCholeskyFactorNumeric
 * with shift type none): up-looking rows with the il / c2r row chains */
void mp_pc_icc_numeric(double *ba, double *rtmp, I *il, I *c2r, const I *arow,
                       const I *acol, const double *adata, const I *bi, const I *bj,
                       const I *bdiag, const I *r, const I *riip, I nrow) {
    for (I i = 0; i < nrow; i++) c2r[i] = nrow;
    if (nrow) il[0] = 0;
    for (I k = 0; k < nrow; k++) {
        for (I jj = bi[k]; jj < bi[k + 1]; jj++) rtmp[bj[jj]] = 0.0;
        I bval = bi[k];
        for (I j = arow[r[k]]; j < arow[r[k] + 1]; j++) {
            I col = riip[acol[j]];
            if (col >= k) {
                rtmp[col] = adata[j];
                ba[bval] = 0.0;
                bval++;
            }
        }
        double dk = rtmp[k];
        I i = c2r[k];
        while (i < k) {
            I nexti = c2r[i];
            I ili = il[i];
            double uikdi = -ba[ili] * ba[bdiag[i]];
            dk += uikdi * ba[ili];
            ba[ili] = uikdi;
            I jmin = ili + 1, jmax = bi[i + 1];
            if (jmin < jmax) {
                for (I j = jmin; j < jmax; j++) {
                    I cc = bj[j];
                    rtmp[cc] = rtmp[cc] + uikdi * ba[j];
                }
                il[i] = jmin;
                I cj = bj[jmin];
                c2r[i] = c2r[cj];
                c2r[cj] = i;
            }
            i = nexti;
        }
        I jmin = bi[k], jmax = bi[k + 1] - 1;
        if (jmin < jmax) {
            for (I j = jmin; j < jmax; j++) ba[j] = rtmp[bj[j]];
            il[k] = jmin;
            I cj = bj[jmin];
            c2r[k] = c2r[cj];
            c2r[cj] = k;
        }
        ba[bdiag[k]] = 1.0 / dk;
    }
}

/* ------------------------------------------------ ported.mojo:759-861 LL */

/* PetscLLInsertLocation_Private; returns the new nlnk, lnkdata by pointer */
I o_ll_insert_location(I assume_sorted, I k, I idx_start, I entry, I nlnk,
                       I *lnkdata, I *lnk) {
    I ld = *lnkdata;
    if (!assume_sorted && k != 0 && entry < ld) ld = idx_start;
    I location = ld;
    for (;;) {
        ld = lnk[location];
        if (entry > ld)
            location = ld;
        else
            break;
    }
    lnk[location] = entry;
    lnk[entry] = ld;
    *lnkdata = entry;
    return nlnk + 1;
}

static I bt_lookup_set(I *bt, I entry) {
    I old = bt[entry];
    bt[entry] = 1;
    return old;
}

/* PetscIncompleteLLInit: entries enter at level 0 */
I o_incomplete_ll_init(I nidx, const I *idx, I idx_start, const I *perm,
                       I *lnk, I *lnklvl, I *bt) {
    I nlnk = 0, lnkdata = idx_start;
    for (I k = 0; k < nidx; k++) {
        I entry = perm[idx[k]];
        if (bt_lookup_set(bt, entry) == 0) {
            nlnk = o_ll_insert_location(0, k, idx_start, entry, nlnk, &lnkdata, lnk);
            lnklvl[entry] = 0;
        }
    }
    return nlnk;
}

/* PetscIncompleteLLAdd_Private: levels capped at `level`, smaller kept */
I o_incomplete_ll_add(I nidx, const I *idx, double level, const I *idxlvl,
                      I idx_start, I *lnk, I *lnklvl, I *bt, I prow_offset,
                      I assume_sorted) {
    I nlnk = 0, lnkdata = idx_start;
    for (I k = 0; k < nidx; k++) {
        I incrlev = idxlvl[k] + prow_offset + 1;
        if ((double)incrlev <= level) {
            I entry = idx[k];
            if (bt_lookup_set(bt, entry) == 0) {
                nlnk = o_ll_insert_location(assume_sorted, k, idx_start, entry, nlnk,
                                            &lnkdata, lnk);
                lnklvl[entry] = incrlev;
            } else if (lnklvl[entry] > incrlev) {
                lnklvl[entry] = incrlev;
            }
        }
    }
    return nlnk;
}

/* PetscIncompleteLLClean: drain the list, reset it */
void o_incomplete_ll_clean(I idx_start, I lnk_max, I nlnk, I *lnk, I *lnklvl,
                           I *indices, I *indiceslvl, I *bt) {
    I idx = idx_start;
    for (I j = 0; j < nlnk; j++) {
        idx = lnk[idx];
        indices[j] = idx;
        indiceslvl[j] = lnklvl[idx];
        lnklvl[idx] = -1;
        bt[idx] = 0;
    }
    lnk[idx_start] = lnk_max;
}
