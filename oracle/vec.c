/* Oracle: Vec maps and reductions.  TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * Restates src/simdvec.mojo (the contiguous maps :40-319, the blocked
 * reductions :332-473, the guarded scalar kernels :246-293 and :476-500,
 * maxpy :503-518) and the ported.mojo Vec wrappers with their branch
 * semantics (src/ported.mojo:75-341).  Exported names and argument order are
 * the reference's C ABI, src/capi.mojo:69-238.
 */
#include <math.h>
#include <string.h>

#include "oracle.h"

static double lane_reduce(const double a[O_SW]) {
    /* halving-tree fold of a 4-lane accumulator (see oracle.h) */
    return (a[0] + a[2]) + (a[1] + a[3]);
}

/* simdvec.mojo:332-353 dot: 4 accumulators x SW lanes over BLK blocks, then
 * SW-wide steps into the summed accumulator, then a scalar tail; the result is
 * `s + acc.reduce_add()`. */
double o_dot(const double *x, const double *y, I n) {
    double a[4][O_SW] = {{0}};
    I i = 0;
    for (; i + O_BLK <= n; i += O_BLK)
        for (int k = 0; k < 4; k++)
            for (int l = 0; l < O_SW; l++)
                a[k][l] += x[i + k * O_SW + l] * y[i + k * O_SW + l];
    double acc[O_SW];
    for (int l = 0; l < O_SW; l++) acc[l] = ((a[0][l] + a[1][l]) + a[2][l]) + a[3][l];
    for (; i + O_SW <= n; i += O_SW)
        for (int l = 0; l < O_SW; l++) acc[l] += x[i + l] * y[i + l];
    double s = 0.0;
    for (; i < n; i++) s += x[i] * y[i];
    return s + lane_reduce(acc);
}

/* simdvec.mojo:356-396 dot_norm2: (x.y, x.x) in one pass, same block order. */
void o_dot_norm2(const double *x, const double *y, I n, double *dout, double *qout) {
    double d[4][O_SW] = {{0}}, q[4][O_SW] = {{0}};
    I i = 0;
    for (; i + O_BLK <= n; i += O_BLK)
        for (int k = 0; k < 4; k++)
            for (int l = 0; l < O_SW; l++) {
                double v = x[i + k * O_SW + l];
                d[k][l] += v * y[i + k * O_SW + l];
                q[k][l] += v * v;
            }
    double dacc[O_SW], nacc[O_SW];
    for (int l = 0; l < O_SW; l++) {
        dacc[l] = ((d[0][l] + d[1][l]) + d[2][l]) + d[3][l];
        nacc[l] = ((q[0][l] + q[1][l]) + q[2][l]) + q[3][l];
    }
    for (; i + O_SW <= n; i += O_SW)
        for (int l = 0; l < O_SW; l++) {
            double v = x[i + l];
            dacc[l] += v * y[i + l];
            nacc[l] += v * v;
        }
    double ds = 0.0, qs = 0.0;
    for (; i < n; i++) {
        double v = x[i];
        ds += v * y[i];
        qs += v * v;
    }
    *dout = ds + lane_reduce(dacc);
    *qout = qs + lane_reduce(nacc);
}

/* simdvec.mojo:423-449 norm2 (the squared 2-norm). */
double o_norm2sq(const double *x, I n) {
    double a[4][O_SW] = {{0}};
    I i = 0;
    for (; i + O_BLK <= n; i += O_BLK)
        for (int k = 0; k < 4; k++)
            for (int l = 0; l < O_SW; l++) {
                double v = x[i + k * O_SW + l];
                a[k][l] += v * v;
            }
    double acc[O_SW];
    for (int l = 0; l < O_SW; l++) acc[l] = ((a[0][l] + a[1][l]) + a[2][l]) + a[3][l];
    for (; i + O_SW <= n; i += O_SW)
        for (int l = 0; l < O_SW; l++) acc[l] += x[i + l] * x[i + l];
    double s = 0.0;
    for (; i < n; i++) s += x[i] * x[i];
    return s + lane_reduce(acc);
}

/* simdvec.mojo:399-420 asum. */
double o_asum(const double *x, I n) {
    double a[4][O_SW] = {{0}};
    I i = 0;
    for (; i + O_BLK <= n; i += O_BLK)
        for (int k = 0; k < 4; k++)
            for (int l = 0; l < O_SW; l++) a[k][l] += fabs(x[i + k * O_SW + l]);
    double acc[O_SW];
    for (int l = 0; l < O_SW; l++) acc[l] = ((a[0][l] + a[1][l]) + a[2][l]) + a[3][l];
    for (; i + O_SW <= n; i += O_SW)
        for (int l = 0; l < O_SW; l++) acc[l] += fabs(x[i + l]);
    double s = 0.0;
    for (; i < n; i++) s += fabs(x[i]);
    return s + lane_reduce(acc);
}

/* simdvec.mojo:452-473 total. */
double o_total(const double *x, I n) {
    double a[4][O_SW] = {{0}};
    I i = 0;
    for (; i + O_BLK <= n; i += O_BLK)
        for (int k = 0; k < 4; k++)
            for (int l = 0; l < O_SW; l++) a[k][l] += x[i + k * O_SW + l];
    double acc[O_SW];
    for (int l = 0; l < O_SW; l++) acc[l] = ((a[0][l] + a[1][l]) + a[2][l]) + a[3][l];
    for (; i + O_SW <= n; i += O_SW)
        for (int l = 0; l < O_SW; l++) acc[l] += x[i + l];
    double s = 0.0;
    for (; i < n; i++) s += x[i];
    return s + lane_reduce(acc);
}

/* ksp.mojo:956-1062 _mdot_basis: x against nv contiguous vectors of y.  Each
 * row keeps the BLK-block accumulators and then a scalar tail; unlike `dot`
 * there is no SW-wide step between them, and the result is
 * `(a0 + a1 + a2 + a3).reduce_add() + t`. */
void o_mdot_basis(const double *x, const double *y, I nv, I n, double *res) {
    for (I j = 0; j < nv; j++) {
        const double *u = y + j * n;
        double a[4][O_SW] = {{0}};
        I i = 0;
        for (; i + O_BLK <= n; i += O_BLK)
            for (int k = 0; k < 4; k++)
                for (int l = 0; l < O_SW; l++)
                    a[k][l] += x[i + k * O_SW + l] * u[i + k * O_SW + l];
        double t = 0.0;
        for (; i < n; i++) t += x[i] * u[i];
        double acc[O_SW];
        for (int l = 0; l < O_SW; l++) acc[l] = ((a[0][l] + a[1][l]) + a[2][l]) + a[3][l];
        res[j] = lane_reduce(acc) + t;
    }
}

/* simdvec.mojo:503-518 maxpy: y += sum_k alpha[k] VV(k), vector by vector. */
void o_maxpy(double *y, const double *alpha, I n, I nv, const double *base) {
    for (I k = 0; k < nv; k++) {
        const double *xk = base + k * n;
        double a = alpha[k];
        for (I i = 0; i < n; i++) y[i] = y[i] + a * xk[i];
    }
}

/* ported.mojo:100-105 VecNorm2 */
double o_vecnorm2(const double *x, I n) {
    if (!n) return 0.0;
    return sqrt(o_norm2sq(x, n));
}

/* ---------------------------------------------------------------- maps */

void o_copy(const double *x, double *y, I n) {
    if (x != y) memmove(y, x, (size_t)n * sizeof(double));
}

void o_zero(double *x, I n) {
    for (I i = 0; i < n; i++) x[i] = 0.0;
}

/* ported.mojo:259-263 VecSet_Seq: alpha == 0 zeroes */
void o_set(double *x, double alpha, I n) {
    if (alpha == 0.0) {
        o_zero(x, n);
        return;
    }
    for (I i = 0; i < n; i++) x[i] = alpha;
}

/* simdvec.mojo:52-61 map1 (VecScale_Seq, ported.mojo:270-271) */
void o_scale(double *x, double alpha, I n) {
    for (I i = 0; i < n; i++) x[i] = x[i] * alpha;
}

/* simdvec.mojo:75-85 axpy (VecAXPY_Seq, ported.mojo:278-282) */
void o_axpy(double *y, double alpha, const double *x, I n) {
    for (I i = 0; i < n; i++) y[i] = y[i] + alpha * x[i];
}

/* ported.mojo:285-294 VecAYPX_Seq with its alpha = 0 / 1 branches */
void o_aypx(double *y, double alpha, const double *x, I n) {
    if (alpha == 0.0) {
        o_copy(x, y, n);
    } else if (alpha == 1.0) {
        o_axpy(y, alpha, x, n);
    } else {
        for (I i = 0; i < n; i++) y[i] = x[i] + alpha * y[i];
    }
}

/* ported.mojo:297-308 VecAXPBY_Seq: beta == 0 is a scale-and-set, alpha == 0
 * a VecScale */
static void o_axpby(double *y, double alpha, double beta, const double *x, I n) {
    if (beta == 0.0) {
        for (I i = 0; i < n; i++) y[i] = x[i] * alpha;
    } else if (alpha == 0.0) {
        o_scale(y, beta, n);
    } else {
        for (I i = 0; i < n; i++) y[i] = alpha * x[i] + beta * y[i];
    }
}

/* simdvec.mojo:114-132 axpbypcz */
void o_axpbypcz(double *z, double alpha, double beta, double gamma,
                const double *x, const double *y, I n) {
    for (I i = 0; i < n; i++) z[i] = alpha * x[i] + beta * y[i] + gamma * z[i];
}

/* simdvec.mojo:135-145 waxpy */
void o_waxpy(double *w, double alpha, const double *x, const double *y, I n) {
    for (I i = 0; i < n; i++) w[i] = alpha * x[i] + y[i];
}

void o_pointwise_mult(double *w, const double *x, const double *y, I n) {
    for (I i = 0; i < n; i++) w[i] = x[i] * y[i];
}

/* ------------------------------------------------------- exported Vec ABI */

void mp_vec_pointwise_mult(double *w, const double *x, const double *y, I n) {
    o_pointwise_mult(w, x, y, n);
}

void mp_vec_pointwise_divide(double *w, const double *x, const double *y, I n) {
    for (I i = 0; i < n; i++) w[i] = x[i] / y[i];
}

/* simdvec.mojo:170-202: Mojo's min/max on SIMD lanes select the smaller or
 * larger operand; restated as a comparison that keeps the first operand on
 * ties. */
void mp_vec_pointwise_min(double *w, const double *x, const double *y, I n) {
    for (I i = 0; i < n; i++) w[i] = (y[i] < x[i]) ? y[i] : x[i];
}

void mp_vec_pointwise_max(double *w, const double *x, const double *y, I n) {
    for (I i = 0; i < n; i++) w[i] = (y[i] > x[i]) ? y[i] : x[i];
}

void mp_vec_pointwise_max_abs(double *w, const double *x, const double *y, I n) {
    for (I i = 0; i < n; i++) {
        double a = fabs(x[i]), b = fabs(y[i]);
        w[i] = (b > a) ? b : a;
    }
}

/* ported.mojo:113-135 VecNorm_Seq: NORM_2 / FROBENIUS / 1_AND_2 / INFINITY /
 * NORM_1, the 2-norm landing in z[1] only for NORM_1_AND_2 */
void mp_vec_norm(const double *x, I ntype, double *z, I n) {
    double z0 = 0.0, z1 = 0.0;
    if (n) {
        if (ntype == 1 || ntype == 2 || ntype == 4) {
            if (ntype == 4) {
                z0 = o_asum(x, n);
                z1 = o_vecnorm2(x, n);
            } else {
                z0 = o_vecnorm2(x, n);
            }
        } else if (ntype == 3) {
            /* simdvec.mojo:476-488: first NaN adopted, scan ends */
            double m = 0.0;
            for (I i = 0; i < n; i++) {
                double t = fabs(x[i]);
                if (t > m || t != t) {
                    m = t;
                    if (t != t) break;
                }
            }
            z0 = m;
        } else if (ntype == 0) {
            z0 = o_asum(x, n);
        }
    }
    z[0] = z0;
    if (ntype == 4) z[1] = z1;
}

void mp_vec_dot(const double *x, const double *y, double *val, I n) {
    val[0] = o_dot(x, y, n);
}

/* ported.mojo:320-323 VecTDot_Seq: dot with the arguments swapped */
void mp_vec_tdot(const double *x, const double *y, double *val, I n) {
    val[0] = o_dot(y, x, n);
}

void mp_vec_dot_norm2(const double *x, const double *y, double *sval, double *rval, I n) {
    o_dot_norm2(x, y, n, sval, rval);
}

void mp_vec_sum(const double *x, double *val, I n) { val[0] = o_total(x, n); }

void mp_vec_mean(const double *x, double *val, I n) {
    val[0] = o_total(x, n) / (double)n;
}

/* ported.mojo:165-196 VecMinMax_Seq: the first index attaining the extreme
 * wins; an empty vector reports -1 and the sentinel */
static void o_minmax(const double *x, I *idx, double *z, double sentinel, int is_max, I n) {
    I j = -1;
    double mm = sentinel;
    if (n) {
        j = 0;
        mm = x[0];
        for (I i = 1; i < n; i++) {
            double t = x[i];
            if (is_max ? (t > mm) : (t < mm)) {
                j = i;
                mm = t;
            }
        }
    }
    z[0] = mm;
    idx[0] = j;
}

void mp_vec_max(const double *x, I *idx, double *z, I n) {
    o_minmax(x, idx, z, -1.7976931348623157e308, 1, n);
}

void mp_vec_min(const double *x, I *idx, double *z, I n) {
    o_minmax(x, idx, z, 1.7976931348623157e308, 0, n);
}

/* ported.mojo:209-214 VecNormalize_Seq: divide by the norm; zero left alone */
void mp_vec_normalize(double *x, double *v, I n) {
    double z = o_vecnorm2(x, n);
    if (z > 0.0)
        for (I i = 0; i < n; i++) x[i] = x[i] / z;
    v[0] = z;
}

/* simdvec.mojo:246-259: exact-zero guard only */
void mp_vec_reciprocal(double *x, I n) {
    for (I i = 0; i < n; i++) x[i] = (x[i] == 0.0) ? 0.0 : 1.0 / x[i];
}

/* simdvec.mojo:278-293 exp/log are libm calls per element; this oracle uses
 * the host libm, so they agree with the reference to libm accuracy only. */
void mp_vec_exp(double *x, I n) {
    for (I i = 0; i < n; i++) x[i] = exp(x[i]);
}

void mp_vec_log(double *x, I n) {
    for (I i = 0; i < n; i++) x[i] = log(x[i]);
}

void mp_vec_sqrtabs(double *x, I n) {
    for (I i = 0; i < n; i++) x[i] = sqrt(fabs(x[i]));
}

/* simdvec.mojo:262-275: strictly below tol is zeroed */
void mp_vec_chop(double *x, I n, double tol) {
    for (I i = 0; i < n; i++)
        if (fabs(x[i]) < tol) x[i] = 0.0;
}

void mp_vec_abs(double *x, I n) {
    for (I i = 0; i < n; i++) x[i] = fabs(x[i]);
}

void mp_vec_conjugate(double *x, I n) { (void)x; (void)n; }

void mp_vec_copy(const double *x, double *y, I n) { o_copy(x, y, n); }

void mp_vec_swap(double *x, double *y, I n) {
    for (I i = 0; i < n; i++) {
        double t = x[i];
        x[i] = y[i];
        y[i] = t;
    }
}

void mp_vec_set(double *x, double alpha, I n) { o_set(x, alpha, n); }

void mp_vec_zero_entries(double *x, I n) { o_zero(x, n); }

void mp_vec_scale(double *x, double alpha, I n) { o_scale(x, alpha, n); }

void mp_vec_shift(double *x, double alpha, I n) {
    for (I i = 0; i < n; i++) x[i] = x[i] + alpha;
}

void mp_vec_axpy(double *y, double alpha, const double *x, I n) { o_axpy(y, alpha, x, n); }

void mp_vec_aypx(double *y, double alpha, const double *x, I n) { o_aypx(y, alpha, x, n); }

void mp_vec_axpby(double *y, double alpha, double beta, const double *x, I n) {
    o_axpby(y, alpha, beta, x, n);
}

void mp_vec_axpbypcz(double *z, double alpha, double beta, double gamma,
                     const double *x, const double *y, I n) {
    o_axpbypcz(z, alpha, beta, gamma, x, y, n);
}

void mp_vec_waxpy(double *w, double alpha, const double *x, const double *y, I n) {
    o_waxpy(w, alpha, x, y, n);
}

/* ported.mojo:329-335 VecMAXPY_Seq: one axpy per vector address */
void mp_vec_maxpy(double *y, I nv, const double *alpha, const I *xaddr, I n) {
    for (I k = 0; k < nv; k++) o_axpy(y, alpha[k], (const double *)(intptr_t)xaddr[k], n);
}

/* simdvec.mojo:491-500: where y_i is exactly zero, x_i itself is used */
void mp_vec_max_pointwise_divide(const double *x, const double *y, double *rval, I n) {
    double m = 0.0;
    for (I i = 0; i < n; i++) {
        double v = fabs(y[i] == 0.0 ? x[i] : x[i] / y[i]);
        m = v > m ? v : m;
    }
    rval[0] = m;
}
