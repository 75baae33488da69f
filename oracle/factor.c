/* Oracle: incomplete-factor symbolic phase and ordering.
 * TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * Restates src/factor.mojo:31-412: ILU(0) pattern, level-of-fill ILU(k) and
 * IC(k) patterns with the caller-sized retry protocol (a negative return is
 * the capacity needed), reverse Cuthill-McKee by index, and the two
 * contiguous passes that rearrange the staged rows into the factor layouts.
 * Exported names follow src/capi.mojo:324-379.
 */
#include "oracle.h"

/* factor.mojo:31-67 MatILUFactorSymbolic_SeqAIJ_ilu0 */
I mp_ilu_symbolic_ilu0(I *bi, I *bj, I *bdiag, const I *adiag, const I *arow,
                       const I *acol, I nrow) {
    I k = 0;
    bi[0] = 0;
    for (I i = 0; i < nrow; i++) {
        I nz = adiag[i] - arow[i];
        bi[i + 1] = bi[i] + nz;
        for (I j = 0; j < nz; j++) bj[k++] = acol[arow[i] + j];
    }
    bdiag[nrow] = bi[nrow] - 1;
    for (I i = nrow - 1; i >= 0; i--) {
        I nz = arow[i + 1] - adiag[i] - 1;
        I src = adiag[i] + 1;
        for (I j = 0; j < nz; j++) bj[k++] = acol[src + j];
        bj[k++] = i;
        bdiag[i] = bdiag[i + 1] + nz + 1;
    }
    return k;
}

/* factor.mojo:70-122 MatILUFactorSymbolic_SeqAIJ (level of fill); `bj` is the
 * contiguous staging array */
I mp_ilu_symbolic(I *bi, I *bj, I *bjlvl, I *bdiag, const I *arow, const I *acol,
                  const I *r, const I *ic, I levels, I cap, I *scratch, I nrow) {
    I nlnk = nrow + 1;
    I *lnk = scratch, *lnklvl = scratch + nlnk, *bt = scratch + 2 * nlnk;
    lnk[nrow] = nrow;
    bi[0] = 0;
    bdiag[0] = 0;
    for (I i = 0; i < nrow; i++) {
        I ri = r[i];
        I nzi = 0;
        I nnz = arow[ri + 1] - arow[ri];
        const I *cols = acol + arow[ri];
        lnk[i] = -1;
        nzi += o_incomplete_ll_init(nnz, cols, nrow, ic, lnk, lnklvl, bt);
        I nzbd = 0;
        I prow = lnk[nrow];
        while (prow < i) {
            I nb = bdiag[prow];
            I *pcols = bj + bi[prow] + nb + 1;
            I *pcolslvl = bjlvl + bi[prow] + nb + 1;
            I lnz = bi[prow + 1] - bi[prow] - nb - 1;
            nzi += o_incomplete_ll_add(lnz, pcols, (double)levels, pcolslvl, nrow, lnk,
                                       lnklvl, bt, lnklvl[prow], 1);
            prow = lnk[prow];
            nzbd++;
        }
        bdiag[i] = nzbd;
        if (bi[i] + nzi > cap) return -(bi[i] + nzi);
        bi[i + 1] = bi[i] + nzi;
        o_incomplete_ll_clean(nrow, nrow, nzi, lnk, lnklvl, bj + bi[i], bjlvl + bi[i], bt);
    }
    return bi[nrow];
}

/* factor.mojo:125-273 MatICCFactorSymbolic_SeqAIJ (level of fill) */
I mp_icc_symbolic(I *ui, I *uj, I *ujlvl, I *udiag, const I *arow, const I *acol,
                  const I *rip, const I *riip, I levels, I cap, I *scratch, I nrow,
                  I scratchlen) {
    I nlnk = nrow + 1;
    if (6 * nlnk + 2 * cap > scratchlen) return -(6 * nlnk + 2 * cap);
    I *lnk = scratch, *lnklvl = scratch + nlnk, *bt = scratch + 2 * nlnk;
    I *jl = scratch + 3 * nlnk, *il = scratch + 4 * nlnk, *ajtmp = scratch + 5 * nlnk;
    I *ujtmp = scratch + 6 * nlnk, *ujtmp_lvl = scratch + 6 * nlnk + cap;
    for (I i = 0; i < nrow; i++) {
        jl[i] = nrow;
        il[i] = 0;
    }
    lnk[nrow] = nrow;
    ui[0] = 0;
    for (I k = 0; k < nrow; k++) {
        I nzk = 0;
        I rk = rip[k];
        I ncols = arow[rk + 1] - arow[rk];
        I ncols_upper = 0;
        for (I j = 0; j < ncols; j++) {
            I col = acol[arow[rk] + j];
            if (riip[col] > k) ajtmp[ncols_upper++] = col;
        }
        nzk += o_incomplete_ll_init(ncols_upper, ajtmp, nrow, riip, lnk, lnklvl, bt);
        if (bt[rk] == 0) {
            I ld = nrow;
            nzk = o_ll_insert_location(0, ncols_upper, nrow, rk, nzk, &ld, lnk);
            lnklvl[rk] = 0;
            bt[rk] = 1;
        }
        I uk = ui[k];
        I prow = jl[k];
        while (prow < k) {
            I nextprow = jl[prow];
            I jmin = il[prow] + 1;
            I jmax = ui[prow + 1];
            I ncols2 = jmax - jmin;
            I pbase = jmin - ui[prow];
            I *cols = ujtmp + pbase;
            I *colslvl = ujtmp_lvl + pbase;
            if (ncols2 > 0)
                nzk += o_incomplete_ll_add(ncols2, cols, (double)levels, colslvl, nrow, lnk,
                                           lnklvl, bt, colslvl[-1], 1);
            if (jmin < jmax) {
                il[prow] = jmin;
                I cj = cols[0];
                jl[prow] = jl[cj];
                jl[cj] = prow;
            }
            prow = nextprow;
        }
        if (uk + nzk > cap) return -(uk + nzk);
        o_incomplete_ll_clean(nrow, nrow, nzk, lnk, lnklvl, ujtmp, ujtmp_lvl, bt);
        if (nzk > 1) {
            I cj = ujtmp[1];
            jl[k] = jl[cj];
            jl[cj] = k;
            il[k] = uk + 1;
        }
        I diag_at = -1;
        for (I c = 0; c < nzk; c++)
            if (ujtmp[c] == rk) {
                diag_at = c;
                break;
            }
        I w = 0;
        for (I c = 0; c < nzk; c++)
            if (c != diag_at) {
                uj[uk + w] = ujtmp[c];
                ujlvl[uk + w] = ujtmp_lvl[c];
                w++;
            }
        for (I c = 1; c < w; c++) {
            I key = uj[uk + c];
            I kk = c - 1;
            while (kk >= 0 && uj[uk + kk] > key) {
                uj[uk + kk + 1] = uj[uk + kk];
                kk--;
            }
            uj[uk + kk + 1] = key;
        }
        uj[uk + nzk - 1] = rk;
        ujlvl[uk + nzk - 1] = ujtmp_lvl[diag_at];
        udiag[k] = uk + nzk - 1;
        ui[k + 1] = uk + nzk;
    }
    return ui[nrow];
}

/* factor.mojo:279-332 MatGetOrdering_RCM (neighbours by index) */
void mp_ordering_rcm(I *perm, I *level, I *visited, I *queue, const I *arow,
                     const I *acol, I nrow) {
    for (I i = 0; i < nrow; i++) {
        level[i] = arow[i + 1] - arow[i];
        visited[i] = 0;
    }
    I filled = 0;
    for (I start = 0; start < nrow; start++) {
        if (visited[start]) continue;
        visited[start] = 1;
        queue[0] = start;
        I head = 0, tail = 1;
        while (head < tail) {
            I node = queue[head++];
            for (I j = arow[node]; j < arow[node + 1]; j++) {
                I c = acol[j];
                if (!visited[c]) {
                    visited[c] = 1;
                    queue[tail++] = c;
                }
            }
        }
        for (I i = 0; i < tail / 2; i++) {
            I t = queue[i];
            queue[i] = queue[tail - 1 - i];
            queue[tail - 1 - i] = t;
        }
        for (I i = 0; i < tail; i++) perm[filled + i] = queue[i];
        filled += tail;
    }
}

/* factor.mojo:335-381 MatILUFreeSpaceContiguousLU */
void mp_ilu_contiguous_lu(const I *bjsrc, I *bi, I *bdiag, I *bj, I n) {
    I bi_temp = bi[n];
    I src = 0;
    I nnzl = bdiag[0];
    for (I row = 0; row < n; row++) {
        I nnz = bi[row + 1] - bi[row];
        if (row == 0)
            bi[row] = 0;
        else
            bi[row] = bi[row - 1] + nnzl;
        nnzl = bdiag[row];
        I dst = bi[row];
        for (I k = 0; k < nnzl; k++) bj[dst + k] = bjsrc[src + k];
        bdiag[row] = bi_temp - 1;
        bj[bi_temp - 1] = row;
        I nnzu = nnz - nnzl;
        bi_temp -= nnzu;
        nnzu -= 1;
        dst = bi_temp;
        for (I k = 0; k < nnzu; k++) bj[dst + k] = bjsrc[src + nnzl + 1 + k];
        src += nnz;
    }
    if (n) {
        bi[n] = bi[n - 1] + nnzl;
        bdiag[n] = bdiag[n - 1] - 1;
    }
}

/* factor.mojo:384-412 MatICCFreeSpaceContiguousCholesky */
void mp_icc_contiguous_cholesky(const I *ujsrc, const I *ui, const I *udiag, I *bi,
                                I *bdiag, I *bj, I n) {
    for (I row = 0; row < n; row++)
        for (I j = ui[row]; j < udiag[row] + 1; j++) bj[j] = ujsrc[j];
    if (n) {
        bi[0] = 0;
        for (I row = 0; row < n; row++) bi[row + 1] = udiag[row] + 1;
        bdiag[n] = bi[n];
    }
}
