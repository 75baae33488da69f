/* Oracle: the Krylov drivers.  TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * Restates src/ksp.mojo:96-1101: KSPConvergedDefault, the PC dispatch and
 * side compositions, KSPSolve_CG, KSPSolve_BCGS, KSPSolve_GMRES with MGS/CGS
 * and KSPGMRESUpdateHessenberg/BuildSoln, KSPSolve_FGMRES, and the flat
 * scalar-block layout.  Exported names follow src/capi.mojo:383-424.
 *
 *   cfg  (double) 0 rtol 1 atol 2 divtol 3 haptol 4 breakdowntol 5 rnorm0
 *                 6 ttol 7 rnorm(out) 8 gmres rnorm0 9.. residual history
 *                 12 RHS norm, 14 seeded flag (shared with history slots)
 *   cfgi (int64)  0 normtype 1 pc_side 2 guess_zero 3 min_it 4 chknorm
 *                 5 convmaxits 6 max_it 7 max_k 8 orthog 9 cgstype
 *                 10 its(out) 11 reason(out) 12 seed from RHS
 *   pci  (int64)  0 PC type, 1..9 aux0..aux8 (buffer addresses), 10 SOR flag
 *   pcf  (double) 0 omega 1 fshift
 *
 * One deliberate difference: PCApplySymmetric for Jacobi reads the
 * diagonal-square-root vector from pci[2], which is where the reference's own
 * PC packs it (python/mojopetsc4py/PETSc/PC.py:504-506); the reference driver
 * reads pci[5] there (src/ksp.mojo:205), which that PC leaves zero.
 */
#include <math.h>
#include <stdlib.h>

#include "oracle.h"

#define NORM_NONE 1
#define NORM_PRECONDITIONED 2
#define NORM_UNPRECONDITIONED 3
#define NORM_NATURAL 4
#define CGS_REFINE_IFNEEDED 1
#define CGS_REFINE_ALWAYS 2
#define ORTHOG_MGS 1
#define R_RTOL 2
#define R_ATOL 3
#define R_ITS 4
#define R_HAPPY 7
#define R_NULL (-2)
#define R_DIVITS (-3)
#define R_DTOL (-4)
#define R_BREAKDOWN (-5)
#define R_INDEF_PC (-8)
#define R_NANORINF (-9)
#define R_INDEF_MAT (-10)
#define PC_LEFT 0
#define PC_RIGHT 1
#define PC_SYMMETRIC 2

#define P(addr) ((double *)(intptr_t)(addr))
#define PI_(addr) ((const I *)(intptr_t)(addr))

typedef struct {
    I n;
    const I *arow, *acol;
    const double *adata;
    const I *pci;
    const double *pcf;
    double *pstmp;
} Ctx;

/* ksp.mojo:96-152 KSPConvergedDefault */
static I converged_default(I n, double rnorm, double *cfg, const I *cfgi) {
    I normtype = cfgi[0], min_it = cfgi[3], chknorm = cfgi[4];
    I convmaxits = cfgi[5], max_it = cfgi[6];
    if (convmaxits && n >= max_it) return R_ITS;
    if (normtype == NORM_NONE) return 0;
    double rtol = cfg[0], atol = cfg[1], divtol = cfg[2];
    if (!n && cfg[14] == 0.0) {
        double rnorm0 = rnorm;
        if (cfgi[12] != 0) {
            double snorm = cfg[12];
            if (!snorm) snorm = rnorm;
            rnorm0 = snorm;
        }
        cfg[5] = rnorm0;
        double ttol = rtol * rnorm0;
        cfg[6] = ttol > atol ? ttol : atol;
        cfg[14] = 1.0;
    }
    if (n <= chknorm) return 0;
    if (rnorm != rnorm || fabs(rnorm) == INFINITY) return R_NANORINF;
    if (n < min_it) return 0;
    double rnorm0 = cfg[5], ttol = cfg[6];
    if (rnorm <= ttol) {
        if (rnorm < atol) return R_ATOL;
        return R_RTOL;
    }
    if (rnorm >= divtol * rnorm0) return R_DTOL;
    return 0;
}

/* ksp.mojo:155-198 KSP_PCApply */
static void pc_apply(const Ctx *c, const double *x, double *y) {
    const I *pci = c->pci;
    I kind = pci[0];
    I n = c->n;
    if (kind == O_PC_JACOBI) {
        o_pointwise_mult(y, x, P(pci[1]), n);
    } else if (kind == O_PC_ILU) {
        o_pc_ilu_apply(x, y, c->pstmp, PI_(pci[1]), PI_(pci[2]), P(pci[3]), PI_(pci[4]),
                       PI_(pci[5]), PI_(pci[6]), n);
    } else if (kind == O_PC_ICC) {
        o_pc_icc_apply(x, y, PI_(pci[1]), PI_(pci[2]), P(pci[3]), PI_(pci[4]), PI_(pci[5]),
                       c->pstmp, n);
    } else if (kind == O_PC_SOR) {
        o_pc_sor_apply(x, y, PI_(pci[1]), PI_(pci[2]), P(pci[3]), PI_(pci[4]), P(pci[5]),
                       P(pci[6]), P(pci[7]), c->pcf[0], c->pcf[1], 1, 1, pci[10], n);
    } else {
        o_copy(x, y, n);
    }
}

/* ksp.mojo:201-208 PCApplySymmetric (Jacobi diagonal square root in pci[2]) */
static void pc_apply_symmetric(const Ctx *c, const double *x, double *y) {
    if (c->pci[0] == O_PC_JACOBI)
        o_pointwise_mult(y, x, P(c->pci[2]), c->n);
    else
        pc_apply(c, x, y);
}

/* ksp.mojo:211-218 KSPUnwindPreconditioner */
static void unwind(const Ctx *c, I pc_side, double *vsoln, double *vt1) {
    o_copy(vsoln, vt1, c->n);
    if (pc_side == PC_RIGHT) {
        pc_apply(c, vsoln, vt1);
        o_copy(vt1, vsoln, c->n);
    }
}

static void matmult(const Ctx *c, const double *x, double *y) {
    o_matmult(x, y, c->arow, c->acol, c->adata, c->n);
}

/* ksp.mojo:221-243 KSPInitialResidual */
static void initial_residual(const Ctx *c, I pc_side, I guess_zero, const double *vsoln,
                             double *vt1, double *vt2, double *vres, const double *vb) {
    I n = c->n;
    if (!guess_zero) {
        matmult(c, vsoln, vt1);
        o_copy(vb, vt2, n);
        o_axpy(vt2, -1.0, vt1, n);
    } else {
        o_copy(vb, vt2, n);
    }
    if (pc_side == PC_SYMMETRIC)
        pc_apply_symmetric(c, vt2, vres);
    else if (pc_side == PC_LEFT)
        pc_apply(c, vt2, vres);
    else
        o_copy(vt2, vres, n);
}

/* ksp.mojo:246-265 KSP_PCApplyBAorAB */
static void apply_ba(const Ctx *c, I pc_side, const double *x, double *y, double *w) {
    if (pc_side == PC_RIGHT) {
        pc_apply(c, x, w);
        matmult(c, w, y);
    } else if (pc_side == PC_LEFT) {
        matmult(c, x, w);
        pc_apply(c, w, y);
    } else {
        pc_apply_symmetric(c, x, w);
        matmult(c, w, y);
        o_copy(y, w, c->n);
        pc_apply_symmetric(c, w, y);
    }
}

static void finish(double *cfg, I *cfgi, double rnorm, I its, I reason) {
    cfg[7] = rnorm;
    cfgi[10] = its;
    cfgi[11] = reason;
}

static int sign_of(double x) { return x < 0.0 ? -1 : (x == 0.0 ? 0 : 1); }

/* ksp.mojo:271-389 KSPSolve_CG */
static void solve_cg(const Ctx *c, double *work, double *cfg, I *cfgi, const double *b,
                     double *x) {
    I n = c->n;
    I normtype = cfgi[0], guess_zero = cfgi[2], chknorm = cfgi[4], max_it = cfgi[6];
    double *R = work, *Z = work + n, *P = work + 2 * n, *W = Z;
    double a, beta = 0.0, betaold = 1.0, bcoef, dpi = 0.0, dpiold, dp = 0.0;
    I its = 0, reason = 0;
    (void)a;
    (void)bcoef;
    if (!guess_zero) {
        matmult(c, x, R);
        o_aypx(R, -1.0, b, n);
    } else {
        o_copy(b, R, n);
    }
    if (normtype == NORM_PRECONDITIONED) {
        pc_apply(c, R, Z);
        dp = o_vecnorm2(Z, n);
    } else if (normtype == NORM_UNPRECONDITIONED) {
        dp = o_vecnorm2(R, n);
    } else if (normtype == NORM_NATURAL) {
        pc_apply(c, R, Z);
        beta = o_dot(Z, R, n);
        dp = sqrt(fabs(beta));
    } else {
        dp = 0.0;
    }
    cfg[9] = dp;
    reason = converged_default(0, dp, cfg, cfgi);
    if (reason) {
        finish(cfg, cfgi, dp, its, reason);
        return;
    }
    if (normtype != NORM_PRECONDITIONED && normtype != NORM_NATURAL) pc_apply(c, R, Z);
    if (normtype != NORM_NATURAL) beta = o_dot(Z, R, n);
    I i = 0;
    for (;;) {
        its = i + 1;
        if (beta == 0.0) {
            reason = R_ATOL;
            break;
        } else if (i > 0 && beta * betaold < 0.0) {
            reason = R_INDEF_PC;
            break;
        }
        if (!i) {
            o_copy(Z, P, n);
            bcoef = 0.0;
        } else {
            bcoef = beta / betaold;
            o_aypx(P, bcoef, Z, n);
        }
        dpiold = dpi;
        matmult(c, P, W);
        dpi = o_dot(P, W, n);
        betaold = beta;
        if (dpi == 0.0 || (i > 0 && sign_of(dpi) * sign_of(dpiold) < 0)) {
            reason = R_INDEF_MAT;
            break;
        }
        a = beta / dpi;
        o_axpy(x, a, P, n);
        o_axpy(R, -a, W, n);
        if (normtype == NORM_PRECONDITIONED && chknorm < i + 2) {
            pc_apply(c, R, Z);
            dp = o_vecnorm2(Z, n);
        } else if (normtype == NORM_UNPRECONDITIONED && chknorm < i + 2) {
            dp = o_vecnorm2(R, n);
        } else if (normtype == NORM_NATURAL) {
            pc_apply(c, R, Z);
            beta = o_dot(Z, R, n);
            dp = sqrt(fabs(beta));
        } else {
            dp = 0.0;
        }
        cfg[9 + its] = dp;
        reason = converged_default(its, dp, cfg, cfgi);
        if (reason) break;
        if ((normtype != NORM_PRECONDITIONED && normtype != NORM_NATURAL) || chknorm >= i + 2)
            pc_apply(c, R, Z);
        if (normtype != NORM_NATURAL || chknorm >= i + 2) beta = o_dot(Z, R, n);
        i++;
        if (i >= max_it) break;
    }
    if (!reason) reason = R_DIVITS;
    finish(cfg, cfgi, dp, its, reason);
}

/* ksp.mojo:395-505 KSPSolve_BCGS */
static void solve_bcgs(const Ctx *c, double *work, double *cfg, I *cfgi, const double *b,
                       double *x) {
    I n = c->n;
    I normtype = cfgi[0], pc_side = cfgi[1], guess_zero = cfgi[2], chknorm = cfgi[4];
    I max_it = cfgi[6];
    double *R = work, *RP = work + n, *V = work + 2 * n, *T = work + 3 * n;
    double *S = work + 4 * n, *P = work + 5 * n, *GUESS = work + 6 * n;
    int has_guess = 0;
    initial_residual(c, pc_side, guess_zero, x, V, T, R, b);
    if (pc_side == PC_RIGHT && !guess_zero) {
        o_copy(x, GUESS, n);
        o_set(x, 0.0, n);
        has_guess = 1;
    }
    double dp = normtype != NORM_NONE ? o_vecnorm2(R, n) : 0.0;
    I its = 0;
    cfg[9] = dp;
    I reason = converged_default(0, dp, cfg, cfgi);
    if (reason) {
        if (has_guess) o_axpy(x, 1.0, GUESS, n);
        finish(cfg, cfgi, dp, its, reason);
        return;
    }
    o_copy(R, RP, n);
    double rhoold = 1.0, alpha = 1.0, omegaold = 1.0, omega, rho, d1, d2;
    o_set(P, 0.0, n);
    o_set(V, 0.0, n);
    I i = 0;
    for (;;) {
        rho = o_dot(R, RP, n);
        double beta = (rho / rhoold) * (alpha / omegaold);
        o_axpbypcz(P, 1.0, -omegaold * beta, beta, R, V, n);
        apply_ba(c, pc_side, P, V, T);
        d1 = o_dot(V, RP, n);
        if (d1 == 0.0) {
            reason = R_BREAKDOWN;
            break;
        }
        alpha = rho / d1;
        o_waxpy(S, -alpha, V, R, n);
        apply_ba(c, pc_side, S, T, R);
        d1 = o_dot(S, T, n);
        d2 = o_norm2sq(T, n);
        if (d2 == 0.0) {
            d1 = o_dot(S, S, n);
            if (d1 != 0.0) {
                reason = R_BREAKDOWN;
                break;
            }
            o_axpy(x, alpha, P, n);
            its++;
            dp = 0.0;
            reason = R_RTOL;
            break;
        }
        omega = d1 / d2;
        o_axpbypcz(x, alpha, omega, 1.0, P, S, n);
        o_waxpy(R, -omega, T, S, n);
        if (normtype != NORM_NONE && chknorm < i + 2) dp = o_vecnorm2(R, n);
        rhoold = rho;
        omegaold = omega;
        its++;
        cfg[9 + its] = dp;
        reason = converged_default(its, dp, cfg, cfgi);
        if (reason) break;
        if (rho == 0.0) {
            reason = R_BREAKDOWN;
            break;
        }
        i++;
        if (i >= max_it) break;
    }
    if (!reason) reason = R_DIVITS;
    unwind(c, pc_side, x, T);
    if (has_guess) o_axpy(x, 1.0, GUESS, n);
    finish(cfg, cfgi, dp, its, reason);
}

/* ------------------------------------------------------------- GMRES */

/* ksp.mojo:919-935 hs_off */
static double *hs_off(double *hs, I m, int which) {
    I hhn = (m + 2) * (m + 1), hesn = (m + 1) * (m + 1), ccn = m + 1, rsn = m + 2;
    switch (which) {
    case 0: return hs;
    case 1: return hs + hhn;
    case 2: return hs + hhn + hesn;
    case 3: return hs + hhn + hesn + ccn;
    case 4: return hs + hhn + hesn + 2 * ccn;
    default: return hs + hhn + hesn + 2 * ccn + rsn;
    }
}

/* ksp.mojo:511-530 MGS */
static void mgs(double *vv, double *hh, double *hes, I m, I it, I n) {
    for (I k = 0; k <= it; k++) {
        double d = o_dot(vv + (it + 1) * n, vv + k * n, n);
        hh[it * (m + 2) + k] = d;
        hes[it * (m + 1) + k] = d;
        o_axpy(vv + (it + 1) * n, -d, vv + k * n, n);
    }
}

static void cgs_pass(double *vv, double *hh, double *hes, double *lhh, I m, I it, I n) {
    o_mdot_basis(vv + (it + 1) * n, vv, it + 1, n, lhh);
    for (I j = 0; j <= it; j++) lhh[j] = -lhh[j];
    o_maxpy(vv + (it + 1) * n, lhh, n, it + 1, vv);
    for (I j = 0; j <= it; j++) {
        hh[it * (m + 2) + j] = hh[it * (m + 2) + j] - lhh[j];
        hes[it * (m + 1) + j] = hes[it * (m + 1) + j] - lhh[j];
    }
}

/* ksp.mojo:533-586 CGS with optional refinement */
static void cgs(double *vv, double *hh, double *hes, double *lhh, I m, I it, I n, I cgstype) {
    int refine = cgstype == CGS_REFINE_ALWAYS;
    for (I j = 0; j <= it; j++) {
        hh[it * (m + 2) + j] = 0.0;
        hes[it * (m + 1) + j] = 0.0;
    }
    cgs_pass(vv, hh, hes, lhh, m, it, n);
    if (cgstype == CGS_REFINE_IFNEEDED) {
        double hnrm = 0.0;
        for (I j = 0; j <= it; j++) hnrm += lhh[j] * lhh[j];
        hnrm = sqrt(hnrm);
        if (o_vecnorm2(vv + (it + 1) * n, n) < hnrm) refine = 1;
    }
    if (refine) cgs_pass(vv, hh, hes, lhh, m, it, n);
}

/* ksp.mojo:589-629 KSPGMRESUpdateHessenberg; returns the reason, *res out */
static I update_hessenberg(double *hh, double *cc, double *ss, double *rs, I it, I m,
                           int hapend, double *res) {
    for (I j = 1; j <= it; j++) {
        I idx = it * (m + 2) + (j - 1);
        double tt = hh[idx];
        hh[idx] = cc[j - 1] * tt + ss[j - 1] * hh[idx + 1];
        hh[idx + 1] = cc[j - 1] * hh[idx + 1] - ss[j - 1] * tt;
    }
    if (!hapend) {
        I base = it * (m + 2) + it;
        double a = hh[base], b = hh[base + 1];
        double tt = sqrt(a * a + b * b);
        if (tt == 0.0) {
            *res = 0.0;
            return R_NULL;
        }
        cc[it] = a / tt;
        ss[it] = b / tt;
        rs[it + 1] = -ss[it] * rs[it];
        rs[it] = cc[it] * rs[it];
        hh[base] = cc[it] * a + ss[it] * b;
        *res = fabs(rs[it + 1]);
        return 0;
    }
    *res = 0.0;
    return 0;
}

static void maxpy_n(double *y, const double *alpha, const double *base, I nvec, I n) {
    for (I i = 0; i < n; i++) y[i] = 0.0;
    o_maxpy(y, alpha, n, nvec, base);
}

/* ksp.mojo:632-664 KSPGMRESBuildSoln */
static I gmres_buildsoln(const Ctx *c, double *rs, double *hh, double *vv, double *temp,
                         double *wtmp, double *vdest, I m, I it, I pc_side) {
    I n = c->n;
    if (it < 0) return 0; /* vs == vdest in every call site */
    if (hh[it * (m + 2) + it] != 0.0)
        rs[it] = rs[it] / hh[it * (m + 2) + it];
    else
        return R_BREAKDOWN;
    for (I ii = 1; ii <= it; ii++) {
        I k = it - ii;
        double tt = rs[k];
        for (I j = k + 1; j <= it; j++) tt -= hh[j * (m + 2) + k] * rs[j];
        if (hh[k * (m + 2) + k] == 0.0) return R_BREAKDOWN;
        rs[k] = tt / hh[k * (m + 2) + k];
    }
    maxpy_n(temp, rs, vv, it + 1, n);
    unwind(c, pc_side, temp, wtmp);
    o_axpy(vdest, 1.0, temp, n);
    return 0;
}

static double normalize(double *x, I n) {
    double z = o_vecnorm2(x, n);
    if (z > 0.0)
        for (I i = 0; i < n; i++) x[i] = x[i] / z;
    return z;
}

/* ksp.mojo:667-769 KSPSolve_GMRES */
static void solve_gmres(const Ctx *c, double *work, double *vv, double *hs, double *cfg,
                        I *cfgi, const double *b, double *x) {
    I n = c->n;
    I normtype = cfgi[0], pc_side = cfgi[1], guess_zero = cfgi[2], max_it = cfgi[6];
    I m = cfgi[7], orthog = cfgi[8], cgstype = cfgi[9];
    double haptol = cfg[3], breakdowntol = cfg[4];
    double *HH = hs_off(hs, m, 0), *HES = hs_off(hs, m, 1), *CC = hs_off(hs, m, 2);
    double *SS = hs_off(hs, m, 3), *RS = hs_off(hs, m, 4), *ORTHOG = hs_off(hs, m, 5);
    double *TEMP = work, *TEMP_MATOP = work + n;
    I its = 0, itcount = 0, reason = 0;
    double res = 0.0, prev_rnorm = -1.0;
    while (reason == 0) {
        initial_residual(c, pc_side, guess_zero, x, TEMP, TEMP_MATOP, vv, b);
        I it = 0;
        res = normalize(vv, n);
        if (prev_rnorm > 0.0 && fabs(res - prev_rnorm) > breakdowntol * cfg[8]) {
            reason = R_BREAKDOWN;
            finish(cfg, cfgi, res, its, reason);
            return;
        }
        RS[0] = res;
        cfg[8] = res;
        cfg[9 + its] = res;
        if (!res)
            reason = R_ATOL;
        else
            reason = converged_default(its, res, cfg, cfgi);
        int hapend = 0;
        while (reason == 0 && it < m && its < max_it) {
            apply_ba(c, pc_side, vv + it * n, vv + (it + 1) * n, TEMP_MATOP);
            if (orthog == ORTHOG_MGS)
                mgs(vv, HH, HES, m, it, n);
            else
                cgs(vv, HH, HES, ORTHOG, m, it, n, cgstype);
            double tt = normalize(vv + (it + 1) * n, n);
            HH[it * (m + 2) + it + 1] = tt;
            HES[it * (m + 1) + it + 1] = tt;
            double hapbnd = fabs(tt / RS[it]);
            hapbnd = hapbnd > haptol ? haptol : hapbnd;
            hapend = tt < hapbnd;
            reason = update_hessenberg(HH, CC, SS, RS, it, m, hapend, &res);
            it++;
            its++;
            cfg[9 + its] = res;
            if (reason) break;
            reason = converged_default(its, res, cfg, cfgi);
            if (hapend) {
                if (normtype == NORM_NONE)
                    reason = R_HAPPY;
                else if (reason == 0) {
                    reason = R_BREAKDOWN;
                    break;
                }
            }
        }
        itcount += it;
        I breason = gmres_buildsoln(c, RS, HH, vv, TEMP, TEMP_MATOP, x, m, it - 1, pc_side);
        if (reason == 0 && breason != 0) reason = breason;
        if (itcount >= max_it) {
            if (reason == 0) reason = R_DIVITS;
            break;
        }
        prev_rnorm = res;
        guess_zero = 0;
    }
    finish(cfg, cfgi, res, its, reason);
}

/* ksp.mojo:871-877 KSPFGMRESResidual */
static void fgmres_residual(const Ctx *c, const double *x, double *temp, double *vv,
                            const double *b) {
    matmult(c, x, temp);
    o_waxpy(vv, -1.0, temp, b, c->n);
}

/* ksp.mojo:880-903 KSPFGMRESBuildSoln */
static void fgmres_buildsoln(double *rs, double *hh, double *prevec, double *temp, I m, I it,
                             I n, double *vdest) {
    if (it < 0) return;
    if (hh[it * (m + 2) + it] != 0.0)
        rs[it] = rs[it] / hh[it * (m + 2) + it];
    else
        rs[it] = 0.0;
    for (I ii = 1; ii <= it; ii++) {
        I k = it - ii;
        double tt = rs[k];
        for (I j = k + 1; j <= it; j++) tt -= hh[j * (m + 2) + k] * rs[j];
        rs[k] = tt / hh[k * (m + 2) + k];
    }
    maxpy_n(temp, rs, prevec, it + 1, n);
    o_axpy(vdest, 1.0, temp, n);
}

/* ksp.mojo:775-868 KSPSolve_FGMRES */
static void solve_fgmres(const Ctx *c, double *work, double *vv, double *prevec, double *hs,
                         double *cfg, I *cfgi, const double *b, double *x) {
    I n = c->n;
    I guess_zero = cfgi[2], max_it = cfgi[6], m = cfgi[7], orthog = cfgi[8];
    I cgstype = cfgi[9];
    double haptol = cfg[3];
    double *HH = hs_off(hs, m, 0), *HES = hs_off(hs, m, 1), *CC = hs_off(hs, m, 2);
    double *SS = hs_off(hs, m, 3), *RS = hs_off(hs, m, 4), *ORTHOG = hs_off(hs, m, 5);
    double *TEMP = work;
    I its = 0, reason = 0;
    double res_norm = 0.0;
    if (!guess_zero)
        fgmres_residual(c, x, TEMP, vv, b);
    else
        o_copy(b, vv, n);
    for (;;) {
        I loc_it = 0;
        res_norm = o_vecnorm2(vv, n);
        RS[0] = res_norm;
        cfg[9 + its] = res_norm;
        reason = converged_default(its, res_norm, cfg, cfgi);
        if (reason == 0) {
            o_scale(vv, 1.0 / res_norm, n);
            int hapend = 0;
            while (reason == 0 && loc_it < m && its < max_it) {
                pc_apply(c, vv + loc_it * n, prevec + loc_it * n);
                matmult(c, prevec + loc_it * n, vv + (loc_it + 1) * n);
                if (orthog == ORTHOG_MGS)
                    mgs(vv, HH, HES, m, loc_it, n);
                else
                    cgs(vv, HH, HES, ORTHOG, m, loc_it, n, cgstype);
                double tt = o_vecnorm2(vv + (loc_it + 1) * n, n);
                HH[loc_it * (m + 2) + loc_it + 1] = tt;
                HES[loc_it * (m + 1) + loc_it + 1] = tt;
                double hapbnd = fabs(tt / RS[loc_it]);
                hapbnd = hapbnd > haptol ? haptol : hapbnd;
                if (tt > hapbnd) {
                    o_scale(vv + (loc_it + 1) * n, 1.0 / tt, n);
                } else {
                    o_set(TEMP, 0.0, n);
                    hapend = 1;
                }
                reason = update_hessenberg(HH, CC, SS, RS, loc_it, m, hapend, &res_norm);
                if (reason) break;
                loc_it++;
                its++;
                cfg[9 + its] = res_norm;
                reason = converged_default(its, res_norm, cfg, cfgi);
                if (hapend && reason == 0) {
                    reason = R_BREAKDOWN;
                    break;
                }
            }
        }
        fgmres_buildsoln(RS, HH, prevec, TEMP, m, loc_it - 1, n, x);
        if (its >= max_it) {
            if (reason == 0) reason = R_DIVITS;
            break;
        }
        if (reason) break;
        fgmres_residual(c, x, TEMP, vv, b);
    }
    finish(cfg, cfgi, res_norm, its, reason);
}

/* ------------------------------------------------- exported KSP ABI */

static Ctx make_ctx(I n, const I *irow, const I *icol, const double *data, const I *pci,
                    const double *pcf, double *pstmp) {
    Ctx c = {n, irow, icol, data, pci, pcf, pstmp};
    return c;
}

void mp_ksp_solve_cg(I n, const I *irow, const I *icol, const double *data, const I *pci,
                     const double *pcf, double *pstmp, double *work, double *cfg, I *cfgi,
                     const double *b, double *x) {
    Ctx c = make_ctx(n, irow, icol, data, pci, pcf, pstmp);
    solve_cg(&c, work, cfg, cfgi, b, x);
}

void mp_ksp_solve_bcgs(I n, const I *irow, const I *icol, const double *data, const I *pci,
                       const double *pcf, double *pstmp, double *work, double *cfg, I *cfgi,
                       const double *b, double *x) {
    Ctx c = make_ctx(n, irow, icol, data, pci, pcf, pstmp);
    solve_bcgs(&c, work, cfg, cfgi, b, x);
}

void mp_ksp_solve_gmres(I n, const I *irow, const I *icol, const double *data, const I *pci,
                        const double *pcf, double *pstmp, double *work, double *vv,
                        double *hs, double *cfg, I *cfgi, const double *b, double *x) {
    Ctx c = make_ctx(n, irow, icol, data, pci, pcf, pstmp);
    solve_gmres(&c, work, vv, hs, cfg, cfgi, b, x);
}

void mp_ksp_solve_fgmres(I n, const I *irow, const I *icol, const double *data, const I *pci,
                         const double *pcf, double *pstmp, double *work, double *vv,
                         double *prevec, double *hs, double *cfg, I *cfgi, const double *b,
                         double *x) {
    Ctx c = make_ctx(n, irow, icol, data, pci, pcf, pstmp);
    solve_fgmres(&c, work, vv, prevec, hs, cfg, cfgi, b, x);
}
