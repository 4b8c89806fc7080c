/*
 * swiftest_oracle.c -- CPU FP64 restatement of Swiftest's integrator hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker for swiftest_gb300's CUDA path).
 * Parity unpinned by the reference's own tests (it has no kernel-level golden
 * vectors and cannot be compiled here); pinned instead by the known-answer
 * tests under tests/.
 *
 * Every routine cites the reference routine it restates (paths are relative
 * to the Swiftest source tree).  Expressions keep the reference's operation
 * order; the file must be compiled with -ffp-contract=off so that no fused
 * multiply-add changes the rounding.
 */
#include "swiftest_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* src/globals/globals_module.f90:33-38,86-101,133-135 */
static const double TWOPI = 6.283185307179586476925286766559005768394;
static const double PIBY2 = 1.570796326794896619231321691639751442099;
static const double PI3BY2 = 4.712388980384689857693965074919254326296;
static const double THIRD = 0.333333333333333333333333333333333333333;
static const double SIXTH = 0.166666666666666666666666666666666666667;
#define ST_ACTIVE 0
#define ST_INACTIVE 1
#define ST_DISCARDED_DRIFTERR (-7)
#define ST_COLLIDED (-14)
/* sqrt(tiny(1.0_DP)) */
#define VSMALL 1.4916681462400413e-154

/* src/swiftest/swiftest_drift.f90:12-17 */
static const double E2MAX = 0.36;
static const double DM2MAX = 0.16;
static const double E2DM2MAX = 0.0016;
static const double DANBYB = 1.0e-13;
#define NLAG1 50
#define NLAG2 40

/* src/encounter/encounter_module.f90:21 */
static const double RSWEEP_FACTOR = 1.1;
/* src/symba/symba_module.f90:20-23 (RHSCALE is a run parameter here) */
#define NTENC 3
static const double RSHELL = 0.48075;

/* Square-and-multiply integer power, the expansion gfortran uses for
 * real**integer with a run-time exponent. */
static double powi(double x, int m) {
    unsigned n = m < 0 ? -(unsigned)m : (unsigned)m;
    double y = (n % 2) ? x : 1.0;
    while (n >>= 1) {
        x = x * x;
        if (n % 2) y = y * x;
    }
    return m < 0 ? 1.0 / y : y;
}

/* x**(-1.5) for the SyMBA shell kick (symba_kick.f90:204,307, where the reference
 * calls libm pow).  sqrt(x) and x*sqrt(x) are carried as double-double pairs with
 * Dekker's error-free transformations (residuals from fma), then one Newton step on
 * the reciprocal: within half an ulp of the exact value except in rare near-tie
 * cases, and the same bits on every IEEE machine with fma (the GPU side runs the
 * identical sequence), unlike libm pow whose last bit varies between libraries. */
static double pow_m1p5(double x) {
    if (!(x > 0.0) || isinf(x)) return pow(x, -1.5);
    double s = sqrt(x);
    double rs = fma(-s, s, x);
    double ds = rs / (2.0 * s);
    double p = x * s;
    double ep = fma(x, s, -p);
    double ql = ep + x * ds;
    double y0 = 1.0 / p;
    double err = fma(-y0, p, 1.0) - y0 * ql;
    return fma(y0, err, y0);
}

/* gfortran NORM2: scaled sum of squares (LAPACK dnrm2 style). */
static double norm2_3(const double *x) {
    double scale = 0.0, ssq = 1.0;
    for (int k = 0; k < 3; k++) {
        if (x[k] != 0.0) {
            double absx = fabs(x[k]);
            if (scale < absx) {
                double q = scale / absx;
                ssq = 1.0 + ssq * q * q;
                scale = absx;
            } else {
                double q = absx / scale;
                ssq = ssq + q * q;
            }
        }
    }
    return scale * sqrt(ssq);
}

/* =====================================================================
 * Kick: src/swiftest/swiftest_kick.f90
 * ===================================================================== */

/* swiftest_kick_getacch_int_one_pl, swiftest_kick.f90:418-446 */
static inline void kick_one_pl(double rji2, double xr, double yr, double zr, double Gmi, double Gmj, double *ahi,
                               double *ahj) {
    double irij3 = 1.0 / (rji2 * sqrt(rji2));
    double faci = Gmi * irij3;
    double facj = Gmj * irij3;
    ahi[0] = ahi[0] + facj * xr;
    ahi[1] = ahi[1] + facj * yr;
    ahi[2] = ahi[2] + facj * zr;
    ahj[0] = ahj[0] - faci * xr;
    ahj[1] = ahj[1] - faci * yr;
    ahj[2] = ahj[2] - faci * zr;
}

/* swiftest_kick_getacch_int_all_tri_rad_pl (:165-271) and _tri_norad_pl (:274-371).
 * The symmetric lmtiny branch's OpenMP reductions are evaluated in serial
 * (single-thread) order. */
void orc_kick_getacch_int_all_tri_pl(int32_t npl, int32_t nplm, const double *r, const double *Gmass,
                                     const double *radius, double *acc) {
    int32_t nplt = npl - nplm;
    int lmtiny = nplt > nplm;
    if (lmtiny) {
        double *ahi = calloc((size_t)3 * npl, sizeof(double));
        double *ahj = calloc((size_t)3 * npl, sizeof(double));
        for (int32_t i = 0; i < nplm; i++) {
            for (int32_t j = i + 1; j < npl; j++) {
                double rx = r[3 * j + 0] - r[3 * i + 0];
                double ry = r[3 * j + 1] - r[3 * i + 1];
                double rz = r[3 * j + 2] - r[3 * i + 2];
                double rji2 = rx * rx + ry * ry + rz * rz;
                if (radius) {
                    double rs = radius[i] + radius[j];
                    double rlim2 = rs * rs;
                    if (!(rji2 > rlim2)) continue;
                }
                kick_one_pl(rji2, rx, ry, rz, Gmass[i], Gmass[j], &ahi[3 * i], &ahj[3 * j]);
            }
        }
        for (int32_t i = 0; i < npl; i++)
            for (int d = 0; d < 3; d++) acc[3 * i + d] = acc[3 * i + d] + ahi[3 * i + d] + ahj[3 * i + d];
        free(ahi);
        free(ahj);
    } else {
        /* rows are independent: the reference's OpenMP row loop, each row summed in j order */
#pragma omp parallel for schedule(static)
        for (int32_t i = 0; i < nplm; i++) {
            for (int32_t j = 0; j < npl; j++) {
                if (j == i) continue;
                double rx = r[3 * j + 0] - r[3 * i + 0];
                double ry = r[3 * j + 1] - r[3 * i + 1];
                double rz = r[3 * j + 2] - r[3 * i + 2];
                double rji2 = rx * rx + ry * ry + rz * rz;
                if (radius) {
                    double rs = radius[i] + radius[j];
                    if (!(rji2 > rs * rs)) continue;
                }
                double fac = Gmass[j] / (rji2 * sqrt(rji2));
                acc[3 * i + 0] = acc[3 * i + 0] + fac * rx;
                acc[3 * i + 1] = acc[3 * i + 1] + fac * ry;
                acc[3 * i + 2] = acc[3 * i + 2] + fac * rz;
            }
        }
        for (int32_t i = nplm; i < npl; i++) {
            for (int32_t j = 0; j < nplm; j++) {
                double rx = r[3 * j + 0] - r[3 * i + 0];
                double ry = r[3 * j + 1] - r[3 * i + 1];
                double rz = r[3 * j + 2] - r[3 * i + 2];
                double rji2 = rx * rx + ry * ry + rz * rz;
                if (radius) {
                    double rs = radius[i] + radius[j];
                    if (!(rji2 > rs * rs)) continue;
                }
                double fac = Gmass[j] / (rji2 * sqrt(rji2));
                acc[3 * i + 0] = acc[3 * i + 0] + fac * rx;
                acc[3 * i + 1] = acc[3 * i + 1] + fac * ry;
                acc[3 * i + 2] = acc[3 * i + 2] + fac * rz;
            }
        }
    }
}

/* swiftest_kick_getacch_int_all_flat_rad_pl (:69-115) / _flat_norad_pl (:118-162), serial reduction order. */
void orc_kick_getacch_int_all_flat_pl(int32_t npl, int64_t nplpl, const int32_t *k_plpl, const double *r,
                                      const double *Gmass, const double *radius, double *acc) {
    double *ahi = calloc((size_t)3 * npl, sizeof(double));
    double *ahj = calloc((size_t)3 * npl, sizeof(double));
    for (int64_t k = 0; k < nplpl; k++) {
        int32_t i = k_plpl[2 * k + 0] - 1;
        int32_t j = k_plpl[2 * k + 1] - 1;
        double rx = r[3 * j + 0] - r[3 * i + 0];
        double ry = r[3 * j + 1] - r[3 * i + 1];
        double rz = r[3 * j + 2] - r[3 * i + 2];
        double rji2 = rx * rx + ry * ry + rz * rz;
        if (radius) {
            double rs = radius[i] + radius[j];
            if (!(rji2 > rs * rs)) continue;
        }
        kick_one_pl(rji2, rx, ry, rz, Gmass[i], Gmass[j], &ahi[3 * i], &ahj[3 * j]);
    }
    for (int32_t i = 0; i < npl; i++)
        for (int d = 0; d < 3; d++) acc[3 * i + d] = acc[3 * i + d] + ahi[3 * i + d] + ahj[3 * i + d];
    free(ahi);
    free(ahj);
}

/* swiftest_kick_getacch_int_all_tp (:374-415) + _one_tp (:449-470) */
void orc_kick_getacch_int_all_tp(int32_t ntp, int32_t npl, const double *rtp, const double *rpl,
                                 const double *GMpl, const int32_t *lmask, double *acc) {
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < ntp; i++) {
        if (!lmask[i]) continue;
        for (int32_t j = 0; j < npl; j++) {
            double rx = rtp[3 * i + 0] - rpl[3 * j + 0];
            double ry = rtp[3 * i + 1] - rpl[3 * j + 1];
            double rz = rtp[3 * i + 2] - rpl[3 * j + 2];
            double rji2 = rx * rx + ry * ry + rz * rz;
            double fac = GMpl[j] / (rji2 * sqrt(rji2));
            acc[3 * i + 0] = acc[3 * i + 0] - fac * rx;
            acc[3 * i + 1] = acc[3 * i + 1] - fac * ry;
            acc[3 * i + 2] = acc[3 * i + 2] - fac * rz;
        }
    }
}

/* swiftest_util_flatten_eucl_plpl (swiftest_util.f90:1090-1131) and the
 * SyMBA count nplplm = nplm*npl - nplm*(nplm+1)/2 (symba_util.f90:202).
 * Pairs (i<j) in row-major order; only rows i <= nplm are kept. */
int64_t orc_util_flatten_eucl_plpl(int32_t npl, int32_t nplm, int32_t *k_plpl) {
    int64_t n = (int64_t)nplm * npl - (int64_t)nplm * (nplm + 1) / 2;
    if (k_plpl) {
        int64_t k = 0;
        for (int32_t i = 1; i <= nplm; i++)
            for (int32_t j = i + 1; j <= npl; j++) {
                k_plpl[2 * k + 0] = i;
                k_plpl[2 * k + 1] = j;
                k++;
            }
    }
    return n;
}

/* =====================================================================
 * Drift: src/swiftest/swiftest_drift.f90
 * ===================================================================== */

static int64_t g_stumpff_count; /* instrumentation for the FP64 work estimate */

/* swiftest_orbel_scget, swiftest_orbel.f90:147-172 */
static void orbel_scget(double angle, double *sx, double *cx) {
    int32_t nper = (int32_t)(angle / TWOPI);
    double x = angle - nper * TWOPI;
    if (x < 0.0) x = x + TWOPI;
    *sx = sin(x);
    *cx = sqrt(1.0 - (*sx) * (*sx));
    if ((x > PIBY2) && (x < PI3BY2)) *cx = -*cx;
}

/* swiftest_drift_kepu_stumpff, :536-580 */
static void kepu_stumpff(double *xp, double *c0, double *c1, double *c2, double *c3) {
    double x = *xp;
    int n = 0;
    const double xm = 0.1;
    g_stumpff_count++;
    while (fabs(x) >= xm && n < 1100) { /* cap only binds for x = inf; finite x needs <= 520 */
        n = n + 1;
        x = x / 4.0;
    }
    *c2 = (1.0 - x * (1.0 - x * (1.0 - x * (1.0 - x * (1.0 - x * (1.0 - x / 182.0) / 132.0) / 90.0) / 56.0) / 30.0) /
                     12.0) /
          2.0;
    *c3 = (1.0 - x * (1.0 - x * (1.0 - x * (1.0 - x * (1.0 - x * (1.0 - x / 210.0) / 156.0) / 110.0) / 72.0) / 42.0) /
                     20.0) /
          6.0;
    *c1 = 1.0 - x * (*c3);
    *c0 = 1.0 - x * (*c2);
    if (n != 0) {
        for (int i = n; i >= 1; i--) {
            *c3 = (*c2 + (*c0) * (*c3)) / 4.0;
            *c2 = (*c1) * (*c1) / 2.0;
            *c1 = (*c0) * (*c1);
            *c0 = 2.0 * (*c0) * (*c0) - 1.0;
            x = x * 4.0;
        }
    }
    *xp = x;
}

/* swiftest_drift_kepmd, :234-276 */
static void drift_kepmd(double dm, double es, double ec, double *x, double *s, double *c) {
    const double a0 = 39916800.0, a1 = 6652800.0, a2 = 332640.0, a3 = 7920.0, a4 = 110.0;
    double fac1 = 1.0 / (1.0 - ec);
    double q = fac1 * dm;
    double fac2 = es * es * fac1 - ec / 3.0;
    double xx = q * (1.0 - 0.5 * fac1 * q * (es - q * fac2));
    double y = xx * xx;
    double ss = xx * (a0 - y * (a1 - y * (a2 - y * (a3 - y * (a4 - y))))) / a0;
    double cc = sqrt(1.0 - ss * ss);
    double f = xx - ec * ss + es * (1.0 - cc) - dm;
    double fp = 1.0 - ec * cc + es * ss;
    double fpp = ec * ss + es * cc;
    double fppp = ec * cc - es * ss;
    double dx = -(f / fp);
    dx = -(f / (fp + dx * fpp / 2.0));
    dx = -(f / (fp + dx * fpp / 2.0 + dx * dx * fppp * SIXTH));
    xx = xx + dx;
    y = xx * xx;
    ss = xx * (a0 - y * (a1 - y * (a2 - y * (a3 - y * (a4 - y))))) / a0;
    cc = sqrt(1.0 - ss * ss);
    *x = xx;
    *s = ss;
    *c = cc;
}

/* swiftest_drift_kepu_p3solve, :486-533 */
static void kepu_p3solve(double dt, double r0, double mu, double alpha, double u, double *s, int *iflag) {
    double denom = (mu - alpha * r0) * SIXTH;
    double a2 = 0.5 * u / denom;
    double a1 = r0 / denom;
    double a0 = -(dt / denom);
    double q = (a1 - a2 * a2 * THIRD) * THIRD;
    double r = (a1 * a2 - 3.0 * a0) * SIXTH - (a2 * a2 * a2) / 27.0;
    double sq2 = q * q * q + r * r;
    if (sq2 >= 0.0) {
        double sq = sqrt(sq2);
        double p1, p2;
        if ((r + sq) <= 0.0)
            p1 = -pow(-(r + sq), THIRD);
        else
            p1 = pow(r + sq, THIRD);
        if ((r - sq) <= 0.0)
            p2 = -pow(-(r - sq), THIRD);
        else
            p2 = pow(r - sq, THIRD);
        *iflag = 0;
        *s = p1 + p2 - a2 * THIRD;
    } else {
        *iflag = 1;
        *s = 0.0;
    }
}

/* swiftest_drift_kepu_guess, :337-378 */
static void kepu_guess(double dt, double r0, double mu, double alpha, double u, double *s) {
    const double thresh = 0.4, danbyk = 0.85;
    if (alpha > 0.0) {
        if (dt / r0 <= thresh) {
            *s = dt / r0 - (dt * dt * u) / (2.0 * r0 * r0 * r0);
        } else {
            double a = mu / alpha;
            double en = sqrt(mu / (a * a * a));
            double ec = 1.0 - r0 / a;
            double es = u / (en * a * a);
            double e = sqrt(ec * ec + es * es);
            double y = en * dt - es;
            double sy, cy;
            orbel_scget(y, &sy, &cy);
            double sigma = copysign(1.0, es * cy + ec * sy);
            double x = y + sigma * danbyk * e;
            *s = x / sqrt(alpha);
        }
    } else {
        int iflag;
        kepu_p3solve(dt, r0, mu, alpha, u, s, &iflag);
        if (iflag != 0) *s = dt / r0;
    }
}

/* swiftest_drift_kepu_fchk, :307-334 */
static void kepu_fchk(double dt, double r0, double mu, double alpha, double u, double s, double *f) {
    double x = (s * s) * alpha;
    double c0, c1, c2, c3;
    kepu_stumpff(&x, &c0, &c1, &c2, &c3);
    c1 = c1 * s;
    c2 = c2 * (s * s);
    c3 = c3 * (s * s * s);
    *f = r0 * c1 + u * c2 + mu * c3 - dt;
}

/* swiftest_drift_kepu_new, :435-483 */
static void kepu_new(double *s, double dt, double r0, double mu, double alpha, double u, double *fp, double *c1,
                     double *c2, double *c3, int *iflag) {
    for (int nc = 0; nc <= 6; nc++) {
        double x = *s * *s * alpha;
        double c0;
        kepu_stumpff(&x, &c0, c1, c2, c3);
        *c1 = *c1 * *s;
        *c2 = *c2 * *s * *s;
        *c3 = *c3 * *s * *s * *s;
        double f = r0 * *c1 + u * *c2 + mu * *c3 - dt;
        *fp = r0 * c0 + u * *c1 + mu * *c2;
        double fpp = (-(r0 * alpha) + mu) * *c1 + u * c0;
        double fppp = (-(r0 * alpha) + mu) * c0 - u * alpha * *c1;
        double ds = -(f / *fp);
        ds = -(f / (*fp + ds * fpp / 2.0));
        ds = -(f / (*fp + ds * fpp / 2.0 + ds * ds * fppp / 6.0));
        *s = *s + ds;
        double fdt = f / dt;
        if (fdt * fdt < DANBYB * DANBYB) {
            *iflag = 0;
            return;
        }
    }
    *iflag = 1;
}

/* swiftest_drift_kepu_lag, :381-432 */
static void kepu_lag(double *s, double dt, double r0, double mu, double alpha, double u, double *fp, double *c1,
                     double *c2, double *c3, int *iflag) {
    const int ln = 5;
    int ncmax = (alpha < 0.0) ? NLAG2 : NLAG1;
    for (int nc = 0; nc <= ncmax; nc++) {
        double x = *s * *s * alpha;
        double c0;
        kepu_stumpff(&x, &c0, c1, c2, c3);
        *c1 = *c1 * *s;
        *c2 = *c2 * *s * *s;
        *c3 = *c3 * *s * *s * *s;
        double f = r0 * *c1 + u * *c2 + mu * *c3 - dt;
        *fp = r0 * c0 + u * *c1 + mu * *c2;
        double fpp = (-(r0 * alpha) + mu) * *c1 + u * c0;
        double lnm1 = (double)ln - 1.0;
        double disc = fabs(lnm1 * lnm1 * *fp * *fp - lnm1 * (double)ln * f * fpp);
        double ds = -((double)ln * f / (*fp + copysign(1.0, *fp) * sqrt(disc)));
        *s = *s + ds;
        double fdt = f / dt;
        if (fdt * fdt < DANBYB * DANBYB) {
            *iflag = 0;
            return;
        }
    }
    *iflag = 2;
}

/* swiftest_drift_kepu, :279-304 */
static void drift_kepu(double dt, double r0, double mu, double alpha, double u, double *fp, double *c1, double *c2,
                       double *c3, int *iflag) {
    double s;
    kepu_guess(dt, r0, mu, alpha, u, &s);
    double st = s;
    kepu_new(&s, dt, r0, mu, alpha, u, fp, c1, c2, c3, iflag);
    if (*iflag != 0) {
        double fo, fn;
        kepu_fchk(dt, r0, mu, alpha, u, st, &fo);
        kepu_fchk(dt, r0, mu, alpha, u, s, &fn);
        if (fabs(fo) < fabs(fn)) s = st;
        kepu_lag(&s, dt, r0, mu, alpha, u, fp, c1, c2, c3, iflag);
    }
}

/* swiftest_drift_dan, :141-231 */
static void drift_dan(double mu, double *rx0, double *ry0, double *rz0, double *vx0, double *vy0, double *vz0,
                      double dt0, int *iflag) {
    double dt = dt0;
    *iflag = 0;
    double r0 = sqrt(*rx0 * *rx0 + *ry0 * *ry0 + *rz0 * *rz0);
    double v0s = *vx0 * *vx0 + *vy0 * *vy0 + *vz0 * *vz0;
    double u = *rx0 * *vx0 + *ry0 * *vy0 + *rz0 * *vz0;
    double alpha = 2.0 * mu / r0 - v0s;
    if (alpha > 0.0) {
        double a = mu / alpha;
        double asq = a * a;
        double en = sqrt(mu / (a * asq));
        double ec = 1.0 - r0 / a;
        double es = u / (en * asq);
        double esq = ec * ec + es * es;
        double dm = dt * en - (double)(int32_t)(dt * en / TWOPI) * TWOPI;
        dt = dm / en;
        if ((esq < E2MAX) && (dm * dm < DM2MAX) && (esq * (dm * dm) < E2DM2MAX)) {
            double xkep, s, c;
            drift_kepmd(dm, es, ec, &xkep, &s, &c);
            double fchk = (xkep - ec * s + es * (1.0 - c) - dm);
            if (fchk * fchk > DANBYB * DANBYB) {
                *iflag = 1;
                return;
            }
            double fp = 1.0 - ec * c + es * s;
            double f = a / r0 * (c - 1.0) + 1.0;
            double g = dt + (s - xkep) / en;
            double fdot = -(a / (r0 * fp) * en * s);
            double gdot = (c - 1.0) / fp + 1.0;
            double rx = *rx0 * f + *vx0 * g;
            double ry = *ry0 * f + *vy0 * g;
            double rz = *rz0 * f + *vz0 * g;
            double vx = *rx0 * fdot + *vx0 * gdot;
            double vy = *ry0 * fdot + *vy0 * gdot;
            double vz = *rz0 * fdot + *vz0 * gdot;
            *rx0 = rx;
            *ry0 = ry;
            *rz0 = rz;
            *vx0 = vx;
            *vy0 = vy;
            *vz0 = vz;
            *iflag = 0;
            return;
        }
    }
    double fp, c1, c2, c3;
    drift_kepu(dt, r0, mu, alpha, u, &fp, &c1, &c2, &c3, iflag);
    if (*iflag == 0) {
        double f = 1.0 - mu / r0 * c2;
        double g = dt - mu * c3;
        double fdot = -(mu / (fp * r0) * c1);
        double gdot = 1.0 - mu / fp * c2;
        double rx = *rx0 * f + *vx0 * g;
        double ry = *ry0 * f + *vy0 * g;
        double rz = *rz0 * f + *vz0 * g;
        double vx = *rx0 * fdot + *vx0 * gdot;
        double vy = *ry0 * fdot + *vy0 * gdot;
        double vz = *rz0 * fdot + *vz0 * gdot;
        *rx0 = rx;
        *ry0 = ry;
        *rz0 = rz;
        *vx0 = vx;
        *vy0 = vy;
        *vz0 = vz;
    }
}

/* swiftest_drift_one, :111-138 */
void orc_drift_one(double mu, double *rx, double *ry, double *rz, double *vx, double *vy, double *vz, double dt,
                   int32_t *iflag) {
    int fl;
    drift_dan(mu, rx, ry, rz, vx, vy, vz, dt, &fl);
    if (fl != 0) {
        double dttmp = 0.1 * dt;
        for (int i = 1; i <= 10; i++) {
            drift_dan(mu, rx, ry, rz, vx, vy, vz, dttmp, &fl);
            if (fl != 0) break;
        }
    }
    *iflag = fl;
}

/* swiftest_drift_all, :60-108 */
void orc_drift_all(const double *mu, double *x, double *v, int32_t n, int32_t lgr, double inv_c2, double dt,
                   const int32_t *lmask, int32_t *iflag) {
    if (n == 0) return;
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < n; i++) {
        if (!lmask[i]) continue;
        double dtp = dt;
        if (lgr) {
            double rmag = norm2_3(&x[3 * i]);
            double vmag2 = v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] + v[3 * i + 2] * v[3 * i + 2];
            double energy = 0.5 * vmag2 - mu[i] / rmag;
            dtp = dt * (1.0 + 3.0 * inv_c2 * energy);
        }
        orc_drift_one(mu[i], &x[3 * i], &x[3 * i + 1], &x[3 * i + 2], &v[3 * i], &v[3 * i + 1], &v[3 * i + 2], dtp,
                      &iflag[i]);
    }
}

int64_t orc_drift_all_count(const double *mu, double *x, double *v, int32_t n, double dt, const int32_t *lmask,
                            int32_t *iflag) {
    g_stumpff_count = 0;
    for (int32_t i = 0; i < n; i++) {
        if (!lmask[i]) continue;
        orc_drift_one(mu[i], &x[3 * i], &x[3 * i + 1], &x[3 * i + 2], &v[3 * i], &v[3 * i + 1], &v[3 * i + 2], dt,
                      &iflag[i]);
    }
    return g_stumpff_count;
}

/* =====================================================================
 * Orbital elements: src/swiftest/swiftest_orbel.f90
 * ===================================================================== */

#define ORB_TINY 4.0e-15 /* swiftest_orbel.f90:11 */
#define ORB_PI 3.141592653589793238462643383279502884197
enum { ORB_ELLIPSE = -1, ORB_PARABOLA = 0, ORB_HYPERBOLA = 1 };

/* swiftest_orbel_schget, :199-207 */
static void orbel_schget(double angle, double *shx, double *chx) {
    *shx = sinh(angle);
    *chx = sqrt(1.0 + (*shx) * (*shx));
}

/* swiftest_orbel_flon, :199-265 (line numbers of the function body in the module) */
static double orbel_flon(double e, double icapn) {
    const double a11 = 156.0, a9 = 17160.0, a7 = 1235520.0, a5 = 51891840.0, a3 = 1037836800.0;
    const double b11 = 11 * a11, b9 = 9 * a9, b7 = 7 * a7, b5 = 5 * a5, b3 = 3 * a3;
    int iflag = 0;
    double capn = icapn;
    if (icapn < 0.0) {
        iflag = 1;
        capn = -icapn;
    }
    double a1 = 6227020800.0 * (1.0 - 1.0 / e);
    double a0 = -(6227020800.0 * capn / e);
    double b1 = a1;
    double a = 6 * (e - 1.0) / e;
    double b = -(6 * capn / e);
    double sq = sqrt(0.25 * (b * b) + (a * a * a) / 27.0);
    double biga = pow(-(0.5 * b) + sq, 1.0 / 3.0);
    double bigb = -pow(0.5 * b + sq, 1.0 / 3.0);
    double x = biga + bigb;
    double flon = x;
    if (capn >= ORB_TINY) {
        for (int i = 1; i <= 10; i++) {
            double x2 = x * x;
            double f = a0 + x * (a1 + x2 * (a3 + x2 * (a5 + x2 * (a7 + x2 * (a9 + x2 * (a11 + x2))))));
            double fp = b1 + x2 * (b3 + x2 * (b5 + x2 * (b7 + x2 * (b9 + x2 * (b11 + 13 * x2)))));
            double dx = -f / fp;
            flon = x + dx;
            if (fabs(dx) <= ORB_TINY) break;
            x = flon;
        }
    }
    if (iflag == 1) flon = -flon;
    return flon;
}

/* swiftest_orbel_fget */
static double orbel_fget(double e, double capn) {
    double x;
    if (capn < 0.0)
        x = -log(-(2 * capn / e) + 1.8);
    else
        x = log(2 * capn / e + 1.8);
    double fget = x;
    for (int i = 1; i <= 10; i++) {
        double shx, chx;
        orbel_schget(x, &shx, &chx);
        double esh = e * shx, ech = e * chx;
        double f = esh - x - capn;
        double fp = ech - 1.0;
        double fpp = esh, fppp = ech;
        double dx = -f / fp;
        dx = -f / (fp + dx * fpp / 2.0);
        dx = -f / (fp + dx * fpp / 2.0 + (dx * dx) * fppp / 6.0);
        fget = x + dx;
        if (fabs(dx) <= ORB_TINY) return fget;
        x = fget;
    }
    return fget;
}

/* swiftest_orbel_zget */
static double orbel_zget(double iq) {
    double q = iq < 0.0 ? -iq : iq, z;
    if (q < 1.0e-3) {
        z = q * (1.0 - ((q * q) / 3.0) * (1.0 - q * q));
    } else {
        double x = 0.5 * (3 * q + sqrt(9 * (q * q) + 4.0));
        double tmp = pow(x, 1.0 / 3.0);
        z = tmp - 1.0 / tmp;
    }
    return iq < 0.0 ? -z : z;
}

/* swiftest_orbel_esolmd */
static double orbel_esolmd(double e, double m) {
    double sm, cm, sx, cx;
    orbel_scget(m, &sm, &cm);
    double x = m + e * sm * (1.0 + e * (cm + e * (1.0 - 1.5 * (sm * sm))));
    orbel_scget(x, &sx, &cx);
    double es = e * sx, ec = e * cx;
    double f = x - es - m, fp = 1.0 - ec, fpp = es, fppp = ec;
    double dx = -f / fp;
    dx = -f / (fp + dx * fpp / 2.0);
    dx = -f / (fp + dx * fpp / 2.0 + (dx * dx) * fppp / 6.0);
    return x + dx;
}

/* swiftest_orbel_ehie */
static double orbel_ehie(double e, double im) {
    int iflag = 0;
    int32_t nper = (int32_t)(im / TWOPI);
    double m = im - nper * TWOPI;
    if (m < 0.0) m = m + TWOPI;
    if (m > ORB_PI) {
        m = TWOPI - m;
        iflag = 1;
    }
    double x = pow(6 * m, 1.0 / 3.0) - m;
    for (int niter = 1; niter <= 3; niter++) {
        double sa, ca;
        orbel_scget(x + m, &sa, &ca);
        double esa = e * sa, eca = e * ca;
        double f = x - esa, fp = 1.0 - eca;
        double dx = -f / fp;
        dx = -f / (fp + 0.5 * dx * esa);
        dx = -f / (fp + 0.5 * dx * (esa + eca * dx / 3.0));
        x = x + dx;
    }
    double r = m + x;
    if (iflag == 1) r = TWOPI - r;
    return r;
}

/* swiftest_orbel_eget: two corrections; the first uses dx*2 where the second uses dx**2 */
static double orbel_eget(double e, double m) {
    double sm, cm, sx, cx;
    orbel_scget(m, &sm, &cm);
    double x = m + e * sm * (1.0 + e * (cm + e * (1.0 - 1.5 * sm * sm)));
    orbel_scget(x, &sx, &cx);
    double es = e * sx, ec = e * cx;
    double f = x - es - m, fp = 1.0 - ec, fpp = es, fppp = ec;
    double dx = -f / fp;
    dx = -f / (fp + dx * fpp / 2.0);
    dx = -f / (fp + dx * fpp / 2.0 + dx * 2 * fppp / 6.0);
    x = x + dx;
    orbel_scget(x, &sx, &cx);
    es = e * sx;
    ec = e * cx;
    f = x - es - m;
    fp = 1.0 - ec;
    fpp = es;
    fppp = ec;
    dx = -f / fp;
    dx = -f / (fp + dx * fpp / 2.0);
    dx = -f / (fp + dx * fpp / 2.0 + (dx * dx) * fppp / 6.0);
    return x + dx;
}

static double orbel_ehybrid(double e, double m) {
    if (e < 0.18) return orbel_esolmd(e, m);
    if (e <= 0.8) return orbel_eget(e, m);
    return orbel_ehie(e, m);
}

static double orbel_fhybrid(double e, double n) {
    double abn = n < 0.0 ? -n : n;
    if (abn < 0.636 * e - 0.6) return orbel_flon(e, n);
    return orbel_fget(e, n);
}

/* swiftest_orbel_el2xv, :45-144 */
static void orbel_el2xv(double mu, double a, double ie, double inc, double capom, double omega, double capm,
                        double *r, double *v) {
    int type;
    double e = ie;
    if (ie < 0.0) {
        e = 0.0;
        type = ORB_ELLIPSE;
    } else if (fabs(e - 1.0) < ORB_TINY) {
        type = ORB_PARABOLA;
    } else if (e > 1.0) {
        type = ORB_HYPERBOLA;
    } else {
        type = ORB_ELLIPSE;
    }
    double sip, cip, so, co, si, ci;
    orbel_scget(omega, &sip, &cip);
    orbel_scget(capom, &so, &co);
    orbel_scget(inc, &si, &ci);
    double d11 = cip * co - sip * so * ci, d12 = cip * so + sip * co * ci, d13 = sip * si;
    double d21 = -(sip * co) - cip * so * ci, d22 = -(sip * so) + cip * co * ci, d23 = cip * si;
    double xfac1 = 0.0, xfac2 = 0.0, vfac1 = 0.0, vfac2 = 0.0;
    if (type == ORB_ELLIPSE) {
        double cape = orbel_ehybrid(e, capm), scap, ccap;
        orbel_scget(cape, &scap, &ccap);
        double sqe = sqrt(1.0 - e * e), sqgma = sqrt(mu * a);
        xfac1 = a * (ccap - e);
        xfac2 = a * sqe * scap;
        double ri = 1.0 / (a * (1.0 - e * ccap));
        vfac1 = -ri * sqgma * scap;
        vfac2 = ri * sqgma * sqe * ccap;
    }
    if (type == ORB_HYPERBOLA) {
        double capf = orbel_fhybrid(e, capm), shcap, chcap;
        orbel_schget(capf, &shcap, &chcap);
        double sqe = sqrt(e * e - 1.0), sqgma = sqrt(mu * a);
        xfac1 = a * (e - chcap);
        xfac2 = a * sqe * shcap;
        double ri = 1.0 / (a * (e * chcap - 1.0));
        vfac1 = -ri * sqgma * shcap;
        vfac2 = ri * sqgma * sqe * chcap;
    }
    if (type == ORB_PARABOLA) {
        double zpara = orbel_zget(capm), sqgma = sqrt(2 * mu * a);
        xfac1 = a * (1.0 - zpara * zpara);
        xfac2 = 2 * a * zpara;
        double ri = 1.0 / (a * (1.0 + zpara * zpara));
        vfac1 = -ri * sqgma * zpara;
        vfac2 = ri * sqgma;
    }
    r[0] = d11 * xfac1 + d21 * xfac2;
    r[1] = d12 * xfac1 + d22 * xfac2;
    r[2] = d13 * xfac1 + d23 * xfac2;
    v[0] = d11 * vfac1 + d21 * vfac2;
    v[1] = d12 * vfac1 + d22 * vfac2;
    v[2] = d13 * vfac1 + d23 * vfac2;
}

/* swiftest_orbel_xv2el, :913-1072; out[11] = a, e, inc, capom, omega, capm, varpi, lam, f, cape, capf */
static void orbel_xv2el(double mu, const double *rv, const double *vv, double *out) {
    double rx = rv[0], ry = rv[1], rz = rv[2], vx = vv[0], vy = vv[1], vz = vv[2];
    double a = 0, e = 0, inc = 0, capom = 0, omega = 0, capm = 0, varpi = 0, lam = 0, f = 0, cape = 0, capf = 0;
    double hx = ry * vz - rz * vy, hy = rz * vx - rx * vz, hz = rx * vy - ry * vx;
    double h2 = hx * hx + hy * hy + hz * hz;
    double h = sqrt(h2);
    if (hz > h) {
        hz = h;
        hx = 0.0;
        hy = 0.0;
    }
    if (!(h2 <= 10 * 2.2250738585072014e-308)) {
        h = sqrt(h2);
        double r = sqrt(rx * rx + ry * ry + rz * rz);
        double v2 = vx * vx + vy * vy + vz * vz;
        double rdotv = rx * vx + ry * vy + rz * vz;
        double energy = 0.5 * v2 - mu / r;
        double fac = hz / h, u, w = 0.0;
        int type;
        if (fac < -1.0)
            inc = ORB_PI;
        else if (fac < 1.0)
            inc = acos(fac);
        fac = sqrt(hx * hx + hy * hy) / h;
        if (fac * fac < ORB_TINY) {
            u = atan2(ry, rx);
            if (hz < 0.0) u = -u;
        } else {
            capom = atan2(hx, -hy);
            u = atan2(rz / sin(inc), rx * cos(capom) + ry * sin(capom));
        }
        if (capom < 0.0) capom = capom + TWOPI;
        if (u < 0.0) u = u + TWOPI;
        if (fabs(energy * r / mu) < sqrt(ORB_TINY)) {
            type = ORB_PARABOLA;
        } else {
            a = -0.5 * mu / energy;
            if (a < 0.0) {
                fac = -h2 / (mu * a);
                type = fac > ORB_TINY ? ORB_HYPERBOLA : ORB_PARABOLA;
            } else {
                type = ORB_ELLIPSE;
            }
        }
        if (type == ORB_ELLIPSE) {
            fac = 1.0 - h2 / (mu * a);
            if (fac > ORB_TINY) {
                e = sqrt(fac);
                cape = 0.0;
                double face = (a - r) / (a * e);
                if (face < -1.0)
                    cape = ORB_PI;
                else if (face < 1.0)
                    cape = acos(face);
                if (rdotv < 0.0) cape = TWOPI - cape;
                fac = 1.0 - e * cos(cape);
                double cw = (cos(cape) - e) / fac;
                double sw = sqrt(1.0 - e * e) * sin(cape) / fac;
                w = atan2(sw, cw);
                if (w < 0.0) w = w + TWOPI;
            } else {
                cape = u;
                w = u;
            }
            capm = cape - e * sin(cape);
        } else if (type == ORB_PARABOLA) {
            a = 0.5 * h2 / mu;
            e = 1.0;
            w = 0.0;
            fac = 2 * a / r - 1.0;
            if (fac < -1.0)
                w = ORB_PI;
            else if (fac < 1.0)
                w = acos(fac);
            if (rdotv < 0.0) w = TWOPI - w;
            double tmpf = tan(0.5 * w);
            capm = tmpf * (1.0 + tmpf * tmpf / 3.0);
        } else {
            e = sqrt(1.0 + fac);
            double tmpf = fmax((a - r) / (a * e), 1.0);
            capf = log(tmpf + sqrt(tmpf * tmpf - 1.0));
            if (rdotv < 0.0) capf = -capf;
            fac = e * cosh(capf) - 1.0;
            double cw = (e - cosh(capf)) / fac;
            double sw = sqrt(e * e - 1.0) * sinh(capf) / fac;
            w = atan2(sw, cw);
            if (w < 0.0) w = w + TWOPI;
            capm = e * sinh(capf) - capf;
        }
        omega = u - w;
        if (omega < 0.0) omega = omega + TWOPI;
        varpi = fmod(omega + capom, TWOPI);
        lam = fmod(capm + varpi, TWOPI);
        if (e > ORB_TINY) {
            double cf = 1.0 / e * (a * (1.0 - e * e) / r - 1.0);
            double hr = h / r;
            double rdot = copysign(sqrt(fmax(v2 - hr * hr, 0.0)), rdotv);
            double sf = a * (1.0 - e * e) / (h * e) * rdot;
            f = atan2(sf, cf);
            if (f < 0.0) f = f + TWOPI;
        } else {
            f = u;
        }
    }
    double o[11] = {a, e, inc, capom, omega, capm, varpi, lam, f, cape, capf};
    memcpy(out, o, sizeof(o));
}

/* swiftest_orbel_el2xv_vec / swiftest_orbel_xv2el_vec, :14-42, 876-910: body i with mu[i];
 * el2xv reads el[k * n + i] (a, e, inc, capom, omega, capm), xv2el writes out[k * n + i] */
void orc_el2xv(int32_t n, const double *mu, const double *el, double *rh, double *vh) {
    for (int32_t i = 0; i < n; i++)
        orbel_el2xv(mu[i], el[i], el[n + i], el[2 * n + i], el[3 * n + i], el[4 * n + i], el[5 * n + i], &rh[3 * i],
                    &vh[3 * i]);
}
void orc_xv2el(int32_t n, const double *mu, const double *rh, const double *vh, double *out) {
    for (int32_t i = 0; i < n; i++) {
        double o[11];
        orbel_xv2el(mu[i], &rh[3 * i], &vh[3 * i], o);
        for (int k = 0; k < 11; k++) out[(size_t)k * n + i] = o[k];
    }
}

/* =====================================================================
 * Encounter checks: src/encounter/encounter_check.f90
 * ===================================================================== */

/* encounter_check_one, :573-621 */
void orc_encounter_check_one(double xr, double yr, double zr, double vxr, double vyr, double vzr, double renc,
                             double dt, int32_t *lencounter, int32_t *lvdotr) {
    double r2 = xr * xr + yr * yr + zr * zr;
    double r2crit = renc * renc;
    double vdotr, r2min;
    if (r2 > r2crit) {
        vdotr = vxr * xr + vyr * yr + vzr * zr;
        if (vdotr > 0.0) {
            r2min = r2;
        } else {
            double v2 = vxr * vxr + vyr * vyr + vzr * vzr;
            if (v2 <= VSMALL) {
                r2min = r2;
            } else {
                double tmin = -vdotr / v2;
                if (tmin < dt)
                    r2min = r2 - vdotr * vdotr / v2;
                else
                    r2min = r2 + 2.0 * vdotr * dt + v2 * (dt * dt);
            }
        }
    } else {
        vdotr = -1.0;
        r2min = r2;
    }
    *lvdotr = (vdotr < 0.0);
    *lencounter = (*lvdotr) && (r2min <= r2crit);
}

/* growable pair list */
typedef struct {
    int64_t n, cap;
    int32_t *i1, *i2, *lv;
} pairlist;

static void pl_push(pairlist *p, int32_t a, int32_t b, int32_t lv) {
    if (p->n == p->cap) {
        p->cap = p->cap ? 2 * p->cap : 256;
        p->i1 = realloc(p->i1, p->cap * sizeof(int32_t));
        p->i2 = realloc(p->i2, p->cap * sizeof(int32_t));
        p->lv = realloc(p->lv, p->cap * sizeof(int32_t));
    }
    p->i1[p->n] = a;
    p->i2[p->n] = b;
    p->lv[p->n] = lv;
    p->n++;
}
static void pl_free(pairlist *p) {
    free(p->i1);
    free(p->i2);
    free(p->lv);
    memset(p, 0, sizeof(*p));
}

static int pl_export(const pairlist *p, int64_t cap, int64_t *nenc, int32_t *index1, int32_t *index2,
                     int32_t *lvdotr) {
    *nenc = p->n;
    if (p->n > cap) return -3;
    for (int64_t k = 0; k < p->n; k++) {
        index1[k] = p->i1[k];
        index2[k] = p->i2[k];
        lvdotr[k] = p->lv[k];
    }
    return 0;
}

/* Triangular checks: encounter_check_all_triangular_plpl/_plplm/_pltp
 * (:436-475, :478-522, :525-570) with _triangular_one (:384-433).  Rows are
 * collapsed in row order (encounter_check_collapse_ragged_list, :624-673), so
 * the list is ordered by (index1, index2). */
static void tri_rect(int32_t n1, const double *r1, const double *v1, const double *renc1, int32_t n2,
                     const double *r2, const double *v2, const double *renc2, double dt, int upper, int32_t shift2,
                     pairlist *out) {
    /* rows are split into contiguous per-thread blocks (static schedule, like the
     * reference's OpenMP loop); concatenating the blocks in thread order keeps
     * the list in row order */
    int nthr = 1;
#ifdef _OPENMP
    nthr = omp_get_max_threads();
#endif
    pairlist *part = calloc((size_t)nthr, sizeof(pairlist));
#pragma omp parallel num_threads(nthr)
    {
        int t = 0;
#ifdef _OPENMP
        t = omp_get_thread_num();
#endif
#pragma omp for schedule(static)
        for (int32_t i = 0; i < n1; i++) {
            int32_t j0 = upper ? i + 1 : 0;
            for (int32_t j = j0; j < n2; j++) {
                double xr = r2[3 * j + 0] - r1[3 * i + 0];
                double yr = r2[3 * j + 1] - r1[3 * i + 1];
                double zr = r2[3 * j + 2] - r1[3 * i + 2];
                double vxr = v2[3 * j + 0] - v1[3 * i + 0];
                double vyr = v2[3 * j + 1] - v1[3 * i + 1];
                double vzr = v2[3 * j + 2] - v1[3 * i + 2];
                double renc12 = renc1[i] + (renc2 ? renc2[j] : 0.0);
                int32_t lenc, lv;
                orc_encounter_check_one(xr, yr, zr, vxr, vyr, vzr, renc12, dt, &lenc, &lv);
                if (lenc) pl_push(&part[t], i + 1, j + 1 + shift2, lv);
            }
        }
    }
    for (int t = 0; t < nthr; t++) {
        for (int64_t k = 0; k < part[t].n; k++) pl_push(out, part[t].i1[k], part[t].i2[k], part[t].lv[k]);
        pl_free(&part[t]);
    }
    free(part);
}

/* Sort of (index1,index2,lvdotr) triples by (index1, index2).  The pair keys
 * are unique, so any correct sort gives the reference's final order. */
static int cmp_pair(const void *a, const void *b) {
    const int32_t *x = a, *y = b;
    if (x[0] != y[0]) return x[0] < y[0] ? -1 : 1;
    if (x[1] != y[1]) return x[1] < y[1] ? -1 : 1;
    return 0;
}
static void sort_pairs_unique(pairlist *p) {
    int32_t *t = malloc((size_t)p->n * 3 * sizeof(int32_t));
    for (int64_t k = 0; k < p->n; k++) {
        t[3 * k] = p->i1[k];
        t[3 * k + 1] = p->i2[k];
        t[3 * k + 2] = p->lv[k];
    }
    qsort(t, p->n, 3 * sizeof(int32_t), cmp_pair);
    int64_t m = 0;
    for (int64_t k = 0; k < p->n; k++) {
        if (m > 0 && t[3 * k] == p->i1[m - 1] && t[3 * k + 1] == p->i2[m - 1]) continue;
        p->i1[m] = t[3 * k];
        p->i2[m] = t[3 * k + 1];
        p->lv[m] = t[3 * k + 2];
        m++;
    }
    p->n = m;
    free(t);
}

/* Extent sort: the reference's util_sort (base_module.f90:1361-1472) is a
 * quicksort seeded with the previous step's permutation, so ties between
 * equal extents are ordered by history.  Here ties are broken by extent
 * index; distinct extents get the same order under any correct sort. */
typedef struct {
    double key;
    int32_t idx;
} extent;
static int cmp_extent(const void *a, const void *b) {
    const extent *x = a, *y = b;
    if (x->key < y->key) return -1;
    if (x->key > y->key) return 1;
    return x->idx < y->idx ? -1 : (x->idx > y->idx);
}

/* Sort-and-sweep, 1-D radial AABB: encounter_check_all_sort_and_sweep_* (:143-326),
 * sort_aabb_1D (:763-792), sweep_aabb_single_list (:905-988), sweep_aabb_double_list
 * (:795-902), sweep_one (:329-381), remove_duplicates (:676-760).
 * n1 bodies of list 1 followed by n2 bodies of list 2 (n2 == 0: single list).
 * Returned pairs: (list-1 index, list-2 index) 1-based, ordered (index1, index2).
 * The reference's remove_duplicates does not carry lvdotr through its
 * within-group index2 sort (:736-737); here lvdotr stays with its pair. */
static void sort_and_sweep(int32_t n1, const double *r1, const double *v1, const double *renc1, int32_t n2,
                           const double *r2, const double *v2, const double *renc2, double dt, int single,
                           pairlist *out) {
    int32_t ntot = n1 + n2;
    extent *ext = malloc((size_t)2 * ntot * sizeof(extent));
    for (int32_t i = 0; i < ntot; i++) {
        const double *ri = i < n1 ? &r1[3 * i] : &r2[3 * (i - n1)];
        double rc = i < n1 ? renc1[i] : (renc2 ? renc2[i - n1] : 0.0);
        double rmag = norm2_3(ri);
        ext[i].key = rmag - RSWEEP_FACTOR * rc;
        ext[i].idx = i;
        ext[ntot + i].key = rmag + RSWEEP_FACTOR * rc;
        ext[ntot + i].idx = ntot + i;
    }
    qsort(ext, 2 * ntot, sizeof(extent), cmp_extent);
    int64_t *ibeg = malloc(sizeof(int64_t) * ntot), *iend = malloc(sizeof(int64_t) * ntot);
    for (int64_t k = 0; k < 2 * ntot; k++) {
        int32_t i = ext[k].idx;
        if (i < ntot)
            ibeg[i] = k + 1;
        else
            iend[i - ntot] = k + 1;
    }
    pairlist raw = {0};
    for (int32_t i = 0; i < ntot; i++) {
        if (!((ibeg[i] + 1) < (iend[i] - 1))) continue; /* loverlap quirk (:828,:951) */
        int ilist1 = i < n1;
        const double *ri = ilist1 ? &r1[3 * i] : &r2[3 * (i - n1)];
        const double *vi = ilist1 ? &v1[3 * i] : &v2[3 * (i - n1)];
        double renci = ilist1 ? renc1[i] : (renc2 ? renc2[i - n1] : 0.0);
        for (int64_t p = ibeg[i] + 1; p <= iend[i] - 1; p++) {
            int32_t b = ext[p - 1].idx;
            if (b >= ntot) b -= ntot;
            int blist1 = b < n1;
            if (!single && (blist1 == ilist1)) continue; /* double list: only the other list */
            const double *rb = blist1 ? &r1[3 * b] : &r2[3 * (b - n1)];
            const double *vb = blist1 ? &v1[3 * b] : &v2[3 * (b - n1)];
            double rencb = blist1 ? renc1[b] : (renc2 ? renc2[b - n1] : 0.0);
            double xr = rb[0] - ri[0], yr = rb[1] - ri[1], zr = rb[2] - ri[2];
            double vxr = vb[0] - vi[0], vyr = vb[1] - vi[1], vzr = vb[2] - vi[2];
            int32_t lenc, lv;
            orc_encounter_check_one(xr, yr, zr, vxr, vyr, vzr, renci + rencb, dt, &lenc, &lv);
            if (!lenc) continue;
            if (single) {
                int32_t a = i + 1, c = b + 1;
                if (a > c) {
                    int32_t t = a;
                    a = c;
                    c = t;
                }
                pl_push(&raw, a, c, lv);
            } else {
                if (ilist1)
                    pl_push(&raw, i + 1, b - n1 + 1, lv);
                else
                    pl_push(&raw, b + 1, i - n1 + 1, lv);
            }
        }
    }
    sort_pairs_unique(&raw);
    for (int64_t k = 0; k < raw.n; k++) pl_push(out, raw.i1[k], raw.i2[k], raw.lv[k]);
    pl_free(&raw);
    free(ext);
    free(ibeg);
    free(iend);
}

/* encounter_check_all_plpl, :14-39 */
int orc_encounter_check_all_plpl(int mode, int32_t npl, const double *r, const double *v, const double *renc,
                                 double dt, int64_t cap, int64_t *nenc, int32_t *index1, int32_t *index2,
                                 int32_t *lvdotr) {
    pairlist p = {0};
    if (npl > 0) {
        if (mode == ORC_ENC_SORTSWEEP)
            sort_and_sweep(npl, r, v, renc, 0, NULL, NULL, NULL, dt, 1, &p);
        else
            tri_rect(npl, r, v, renc, npl, r, v, renc, dt, 1, 0, &p);
    }
    int rc = pl_export(&p, cap, nenc, index1, index2, lvdotr);
    pl_free(&p);
    return rc;
}

/* encounter_check_all_plplm, :42-109: plm-plm list, then plm-plt list with
 * index2 shifted by nplm, concatenated and re-sorted by index1.  Both lists
 * are already ordered by (index1,index2), so the merged order is
 * (index1, index2). */
int orc_encounter_check_all_plplm(int mode, int32_t nplm, int32_t nplt, const double *rplm, const double *vplm,
                                  const double *rplt, const double *vplt, const double *rencm,
                                  const double *renct, double dt, int64_t cap, int64_t *nenc, int32_t *index1,
                                  int32_t *index2, int32_t *lvdotr) {
    pairlist p = {0};
    if (nplm > 0) {
        if (mode == ORC_ENC_SORTSWEEP)
            sort_and_sweep(nplm, rplm, vplm, rencm, 0, NULL, NULL, NULL, dt, 1, &p);
        else
            tri_rect(nplm, rplm, vplm, rencm, nplm, rplm, vplm, rencm, dt, 1, 0, &p);
    }
    if (nplm > 0 && nplt > 0) {
        pairlist q = {0};
        if (mode == ORC_ENC_SORTSWEEP)
            sort_and_sweep(nplm, rplm, vplm, rencm, nplt, rplt, vplt, renct, dt, 0, &q);
        else
            tri_rect(nplm, rplm, vplm, rencm, nplt, rplt, vplt, renct, dt, 0, 0, &q);
        for (int64_t k = 0; k < q.n; k++) pl_push(&p, q.i1[k], q.i2[k] + nplm, q.lv[k]);
        pl_free(&q);
        sort_pairs_unique(&p);
    }
    int rc = pl_export(&p, cap, nenc, index1, index2, lvdotr);
    pl_free(&p);
    return rc;
}

/* encounter_check_all_pltp, :112-140 (test particles have zero encounter radius) */
int orc_encounter_check_all_pltp(int mode, int32_t npl, int32_t ntp, const double *rpl, const double *vpl,
                                 const double *rtp, const double *vtp, const double *renc, double dt,
                                 int64_t cap, int64_t *nenc, int32_t *index1, int32_t *index2, int32_t *lvdotr) {
    pairlist p = {0};
    if (npl > 0 && ntp > 0) {
        if (mode == ORC_ENC_SORTSWEEP)
            sort_and_sweep(npl, rpl, vpl, renc, ntp, rtp, vtp, NULL, dt, 0, &p);
        else
            tri_rect(npl, rpl, vpl, renc, ntp, rtp, vtp, NULL, dt, 0, 0, &p);
    }
    int rc = pl_export(&p, cap, nenc, index1, index2, lvdotr);
    pl_free(&p);
    return rc;
}

/* =====================================================================
 * nbody system and step loops
 * ===================================================================== */

typedef struct {
    int64_t n, cap;
    int32_t *i1, *i2, *lvdotr, *status, *level;
} enclist;

static void enclist_reserve(enclist *e, int64_t n) {
    if (n <= e->cap) return;
    e->cap = n;
    e->i1 = realloc(e->i1, n * sizeof(int32_t));
    e->i2 = realloc(e->i2, n * sizeof(int32_t));
    e->lvdotr = realloc(e->lvdotr, n * sizeof(int32_t));
    e->status = realloc(e->status, n * sizeof(int32_t));
    e->level = realloc(e->level, n * sizeof(int32_t));
}
static void enclist_free(enclist *e) {
    free(e->i1);
    free(e->i2);
    free(e->lvdotr);
    free(e->status);
    free(e->level);
    memset(e, 0, sizeof(*e));
}

struct orc_system {
    int integrator;
    int32_t npl, ntp, nplm;
    double GMcb, Rcb;
    double cb_vb[3], cb_rb[3], ptbeg[3], ptend[3];
    /* massive bodies */
    double *rh, *vh, *vb, *ah, *rbeg, *rend, *Gmass, *radius, *rhill, *renc, *mu;
    double *xj, *vj, *eta, *muj, *ir3h, *ir3j;
    int32_t *status, *lmask, *levelg, *levelm, *lencounter, *nplenc, *ntpenc;
    int32_t *k_plpl;
    int64_t nplpl;
    /* test particles */
    double *trh, *tvh, *tvb, *tah, *tmu;
    int32_t *tstatus, *tlmask, *tlevelg, *tlevelm, *tnplenc;
    /* parameters */
    double dt, rhscale, gmtiny;
    int loop_mode, enc_plpl, enc_pltp, lclose;
    int lfirst_pl, lfirst_tp, lfirstkick;
    int irec;
    double t;
    /* collision bookkeeping (swiftest_module.f90:375-377, collision_generate.f90:219,
     * collision_resolve.f90:638), in G*m units */
    double E_collisions, L_escape[3];
    enclist plpl, pltp;
    int64_t stats[6];
    int64_t last_plpl_n, last_pltp_n;
    int32_t *last_plpl, *last_pltp;
};

orc_system *orc_system_create(int integrator, int32_t npl, int32_t ntp) {
    orc_system *s = calloc(1, sizeof(orc_system));
    s->integrator = integrator;
    s->npl = npl;
    s->ntp = ntp;
    size_t n3 = (size_t)3 * (npl > 0 ? npl : 1), n1 = (npl > 0 ? npl : 1);
    s->rh = calloc(n3, 8);
    s->vh = calloc(n3, 8);
    s->vb = calloc(n3, 8);
    s->ah = calloc(n3, 8);
    s->rbeg = calloc(n3, 8);
    s->rend = calloc(n3, 8);
    s->xj = calloc(n3, 8);
    s->vj = calloc(n3, 8);
    s->Gmass = calloc(n1, 8);
    s->radius = calloc(n1, 8);
    s->rhill = calloc(n1, 8);
    s->renc = calloc(n1, 8);
    s->mu = calloc(n1, 8);
    s->eta = calloc(n1, 8);
    s->muj = calloc(n1, 8);
    s->ir3h = calloc(n1, 8);
    s->ir3j = calloc(n1, 8);
    s->status = calloc(n1, 4);
    s->lmask = calloc(n1, 4);
    s->levelg = calloc(n1, 4);
    s->levelm = calloc(n1, 4);
    s->lencounter = calloc(n1, 4);
    s->nplenc = calloc(n1, 4);
    s->ntpenc = calloc(n1, 4);
    size_t t3 = (size_t)3 * (ntp > 0 ? ntp : 1), t1 = (ntp > 0 ? ntp : 1);
    s->trh = calloc(t3, 8);
    s->tvh = calloc(t3, 8);
    s->tvb = calloc(t3, 8);
    s->tah = calloc(t3, 8);
    s->tmu = calloc(t1, 8);
    s->tstatus = calloc(t1, 4);
    s->tlmask = calloc(t1, 4);
    s->tlevelg = calloc(t1, 4);
    s->tlevelm = calloc(t1, 4);
    s->tnplenc = calloc(t1, 4);
    s->rhscale = 6.5;
    s->lfirst_pl = s->lfirst_tp = s->lfirstkick = 1;
    s->nplm = npl;
    for (int32_t i = 0; i < npl; i++) s->lmask[i] = 1;
    for (int32_t i = 0; i < ntp; i++) s->tlmask[i] = 1;
    return s;
}

void orc_system_destroy(orc_system *s) {
    if (!s) return;
    double *d[] = {s->rh, s->vh, s->vb, s->ah, s->rbeg, s->rend, s->xj, s->vj, s->Gmass, s->radius, s->rhill,
                   s->renc, s->mu, s->eta, s->muj, s->ir3h, s->ir3j, s->trh, s->tvh, s->tvb, s->tah, s->tmu};
    for (size_t k = 0; k < sizeof(d) / sizeof(d[0]); k++) free(d[k]);
    int32_t *ii[] = {s->status, s->lmask, s->levelg, s->levelm, s->lencounter, s->nplenc, s->ntpenc, s->k_plpl,
                     s->tstatus, s->tlmask, s->tlevelg, s->tlevelm, s->tnplenc, s->last_plpl, s->last_pltp};
    for (size_t k = 0; k < sizeof(ii) / sizeof(ii[0]); k++) free(ii[k]);
    enclist_free(&s->plpl);
    enclist_free(&s->pltp);
    free(s);
}

void orc_system_set_cb(orc_system *s, double GMcb, double Rcb) {
    s->GMcb = GMcb;
    s->Rcb = Rcb;
}
void orc_system_set_pl(orc_system *s, const double *rh, const double *vh, const double *Gmass, const double *radius,
                       const double *rhill) {
    memcpy(s->rh, rh, sizeof(double) * 3 * s->npl);
    memcpy(s->vh, vh, sizeof(double) * 3 * s->npl);
    memcpy(s->Gmass, Gmass, sizeof(double) * s->npl);
    memcpy(s->radius, radius, sizeof(double) * s->npl);
    if (rhill) memcpy(s->rhill, rhill, sizeof(double) * s->npl);
}
void orc_system_set_tp(orc_system *s, const double *rh, const double *vh) {
    memcpy(s->trh, rh, sizeof(double) * 3 * s->ntp);
    memcpy(s->tvh, vh, sizeof(double) * 3 * s->ntp);
}
void orc_system_set_param(orc_system *s, double dt, int loop_mode, int enc_plpl, int enc_pltp, double rhscale,
                          int lclose, double gmtiny) {
    s->dt = dt;
    s->loop_mode = loop_mode;
    s->enc_plpl = enc_plpl;
    s->enc_pltp = enc_pltp;
    s->rhscale = rhscale;
    s->lclose = lclose;
    s->gmtiny = gmtiny;
}
int32_t orc_system_npl(const orc_system *s) { return s->npl; }

/* swiftest_util_coord_vh2vb_pl, swiftest_util.f90:424-456 */
static void vh2vb_pl(orc_system *s) {
    if (s->npl == 0) return;
    double Gmtot = s->GMcb;
    {
        double sum = 0.0;
        for (int32_t i = 0; i < s->npl; i++) sum = sum + s->Gmass[i];
        Gmtot = s->GMcb + sum;
    }
    double cbvb[3] = {0, 0, 0};
    for (int32_t i = 0; i < s->npl; i++)
        for (int d = 0; d < 3; d++) cbvb[d] = cbvb[d] - s->Gmass[i] * s->vh[3 * i + d];
    for (int d = 0; d < 3; d++) s->cb_vb[d] = cbvb[d] / Gmtot;
    for (int32_t i = 0; i < s->npl; i++)
        for (int d = 0; d < 3; d++) s->vb[3 * i + d] = s->vh[3 * i + d] + s->cb_vb[d];
}

/* swiftest_util_coord_vb2vh_pl, swiftest_util.f90:363-392 (reverse-order sum) */
static void vb2vh_pl(orc_system *s) {
    if (s->npl == 0) return;
    double cbvb[3] = {0, 0, 0};
    for (int32_t i = s->npl - 1; i >= 0; i--) {
        if (s->status[i] == ST_INACTIVE) continue;
        for (int d = 0; d < 3; d++) cbvb[d] = cbvb[d] - s->Gmass[i] * s->vb[3 * i + d] / s->GMcb;
    }
    for (int d = 0; d < 3; d++) s->cb_vb[d] = cbvb[d];
    for (int32_t i = 0; i < s->npl; i++)
        for (int d = 0; d < 3; d++) s->vh[3 * i + d] = s->vb[3 * i + d] - s->cb_vb[d];
}

/* swiftest_util_coord_vh2vb_tp / vb2vh_tp (:395-421, :459-485) */
static void vh2vb_tp(orc_system *s, const double *vbcb) {
    for (int32_t i = 0; i < s->ntp; i++)
        if (s->tlmask[i])
            for (int d = 0; d < 3; d++) s->tvb[3 * i + d] = s->tvh[3 * i + d] + vbcb[d];
}
static void vb2vh_tp(orc_system *s, const double *vbcb) {
    for (int32_t i = 0; i < s->ntp; i++)
        if (s->tlmask[i])
            for (int d = 0; d < 3; d++) s->tvh[3 * i + d] = s->tvb[3 * i + d] - vbcb[d];
}

/* swiftest_util_coord_rh2rb_pl, swiftest_util.f90:488-520 */
static void rh2rb_pl(orc_system *s, double *rb) {
    double Gmtot = s->GMcb;
    double xtmp[3] = {0, 0, 0};
    for (int32_t i = 0; i < s->npl; i++) {
        if (s->status[i] == ST_INACTIVE) continue;
        Gmtot = Gmtot + s->Gmass[i];
        for (int d = 0; d < 3; d++) xtmp[d] = xtmp[d] + s->Gmass[i] * s->rh[3 * i + d];
    }
    for (int d = 0; d < 3; d++) s->cb_rb[d] = -xtmp[d] / Gmtot;
    for (int32_t i = 0; i < s->npl; i++) {
        if (s->status[i] == ST_INACTIVE) continue;
        for (int d = 0; d < 3; d++) rb[3 * i + d] = s->rh[3 * i + d] + s->cb_rb[d];
    }
}

/* helio_drift_linear_pl (helio_drift.f90:129-163) */
static void lindrift_pl(orc_system *s, double dt, int lbeg) {
    if (s->npl == 0) return;
    double pt[3] = {0, 0, 0};
    for (int d = 0; d < 3; d++) {
        double sum = 0.0;
        for (int32_t i = 0; i < s->npl; i++)
            if (s->lmask[i]) sum = sum + s->Gmass[i] * s->vb[3 * i + d];
        pt[d] = sum;
    }
    for (int d = 0; d < 3; d++) pt[d] = pt[d] / s->GMcb;
    for (int32_t i = 0; i < s->npl; i++)
        if (s->lmask[i])
            for (int d = 0; d < 3; d++) s->rh[3 * i + d] = s->rh[3 * i + d] + pt[d] * dt;
    double *dst = lbeg ? s->ptbeg : s->ptend;
    for (int d = 0; d < 3; d++) dst[d] = pt[d];
}

/* helio_drift_linear_tp (helio_drift.f90:166-200) */
static void lindrift_tp(orc_system *s, double dt, int lbeg) {
    const double *pt = lbeg ? s->ptbeg : s->ptend;
    for (int32_t i = 0; i < s->ntp; i++)
        if (s->tlmask[i])
            for (int d = 0; d < 3; d++) s->trh[3 * i + d] = s->trh[3 * i + d] + pt[d] * dt;
}

/* pl-pl interaction accelerations: swiftest_kick_getacch_int_pl (swiftest_kick.f90:12-43) for
 * WHM/HELIO, symba_kick_getacch_int_pl (symba_kick.f90:14-33) for SyMBA. */
static void accel_int_pl(orc_system *s) {
    int symba = s->integrator == ORC_SYMBA;
    const double *rad = (symba || s->lclose) ? s->radius : NULL;
    int32_t nplm = symba ? s->nplm : s->npl;
    if (s->loop_mode == 1) {
        int64_t n = symba ? orc_util_flatten_eucl_plpl(s->npl, nplm, NULL) : s->nplpl;
        orc_kick_getacch_int_all_flat_pl(s->npl, n, s->k_plpl, s->rh, s->Gmass, rad, s->ah);
    } else {
        orc_kick_getacch_int_all_tri_pl(s->npl, nplm, s->rh, s->Gmass, rad, s->ah);
    }
}

/* symba_kick_getacch_pl (symba_kick.f90:36-76) or helio_kick_getacch_pl (helio_kick.f90:14-55) */
static void accel_pl_helio(orc_system *s) {
    accel_int_pl(s);
    if (s->integrator == ORC_SYMBA && s->plpl.n > 0) {
        double *ah_enc = calloc((size_t)3 * s->npl, 8);
        int32_t *k = malloc((size_t)2 * s->plpl.n * sizeof(int32_t));
        for (int64_t q = 0; q < s->plpl.n; q++) {
            k[2 * q] = s->plpl.i1[q];
            k[2 * q + 1] = s->plpl.i2[q];
        }
        orc_kick_getacch_int_all_flat_pl(s->npl, s->plpl.n, k, s->rh, s->Gmass, s->radius, ah_enc);
        for (int32_t i = 0; i < s->npl; i++)
            for (int d = 0; d < 3; d++) s->ah[3 * i + d] = s->ah[3 * i + d] - ah_enc[3 * i + d];
        free(ah_enc);
        free(k);
    }
}

/* helio_kick_vb_pl, helio_kick.f90:91-132 */
static void kick_vb_pl(orc_system *s, double dt, int lbeg) {
    if (s->npl == 0) return;
    memset(s->ah, 0, sizeof(double) * 3 * s->npl);
    accel_pl_helio(s);
    memcpy(lbeg ? s->rbeg : s->rend, s->rh, sizeof(double) * 3 * s->npl);
    for (int32_t i = 0; i < s->npl; i++)
        if (s->lmask[i])
            for (int d = 0; d < 3; d++) s->vb[3 * i + d] = s->vb[3 * i + d] + s->ah[3 * i + d] * dt;
}

/* helio_kick_vb_tp (helio_kick.f90:135-169) with symba_kick_getacch_tp (symba_kick.f90:79-123) */
static void kick_vb_tp(orc_system *s, double dt, int lbeg) {
    if (s->ntp == 0) return;
    memset(s->tah, 0, sizeof(double) * 3 * s->ntp);
    const double *rp = lbeg ? s->rbeg : s->rend;
    if (s->npl > 0) orc_kick_getacch_int_all_tp(s->ntp, s->npl, s->trh, rp, s->Gmass, s->tlmask, s->tah);
    if (s->integrator == ORC_SYMBA) {
        for (int64_t k = 0; k < s->pltp.n; k++) {
            int32_t i = s->pltp.i1[k] - 1, j = s->pltp.i2[k] - 1;
            if (!s->tlmask[j]) continue;
            double dx[3];
            for (int d = 0; d < 3; d++) dx[d] = s->trh[3 * j + d] - rp[3 * i + d];
            double rjj = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
            double fac = s->Gmass[i] / (rjj * sqrt(rjj));
            for (int d = 0; d < 3; d++) s->tah[3 * j + d] = s->tah[3 * j + d] + fac * dx[d];
        }
    }
    for (int32_t i = 0; i < s->ntp; i++)
        if (s->tlmask[i])
            for (int d = 0; d < 3; d++) s->tvb[3 * i + d] = s->tvb[3 * i + d] + s->tah[3 * i + d] * dt;
}

/* helio_drift_body (helio_drift.f90:14-54), masked by symba_drift_pl/_tp (symba_drift.f90:14-61) */
static void drift_pl(orc_system *s, double dt) {
    if (s->npl == 0) return;
    int32_t *iflag = calloc(s->npl, 4);
    int32_t *m = malloc(sizeof(int32_t) * s->npl);
    for (int32_t i = 0; i < s->npl; i++)
        m[i] = s->integrator == ORC_SYMBA ? (s->status[i] != ST_INACTIVE && s->levelg[i] == s->irec) : s->lmask[i];
    orc_drift_all(s->mu, s->rh, s->vb, s->npl, 0, 0.0, dt, m, iflag);
    for (int32_t i = 0; i < s->npl; i++) {
        if (iflag[i] != 0) s->status[i] = ST_DISCARDED_DRIFTERR;
        if (s->integrator == ORC_SYMBA) s->lmask[i] = s->status[i] != ST_INACTIVE;
    }
    free(iflag);
    free(m);
}
static void drift_tp(orc_system *s, double dt) {
    if (s->ntp == 0) return;
    int32_t *iflag = calloc(s->ntp, 4);
    int32_t *m = malloc(sizeof(int32_t) * s->ntp);
    for (int32_t i = 0; i < s->ntp; i++)
        m[i] = s->integrator == ORC_SYMBA ? (s->tstatus[i] != ST_INACTIVE && s->tlevelg[i] == s->irec) : s->tlmask[i];
    double *v = s->integrator == ORC_WHM ? s->tvh : s->tvb;
    orc_drift_all(s->tmu, s->trh, v, s->ntp, 0, 0.0, dt, m, iflag);
    for (int32_t i = 0; i < s->ntp; i++) {
        if (iflag[i] != 0) s->tstatus[i] = ST_DISCARDED_DRIFTERR;
        if (s->integrator == ORC_SYMBA) s->tlmask[i] = s->tstatus[i] != ST_INACTIVE;
    }
    free(iflag);
    free(m);
}

/* helio_step_pl / helio_step_tp (helio_step.f90:37-119) via whm_step_system (whm_step.f90:14-35) */
static void helio_step(orc_system *s, double dt) {
    double dth = 0.5 * dt;
    s->lfirst_tp = s->lfirst_pl;
    if (s->npl > 0) {
        if (s->lfirst_pl) {
            vh2vb_pl(s);
            s->lfirst_pl = 0;
        }
        lindrift_pl(s, dth, 1);
        kick_vb_pl(s, dth, 1);
        drift_pl(s, dt);
        kick_vb_pl(s, dth, 0);
        lindrift_pl(s, dth, 0);
        vb2vh_pl(s);
    }
    if (s->ntp > 0) {
        if (s->lfirst_tp) {
            double vbcb[3] = {-s->ptbeg[0], -s->ptbeg[1], -s->ptbeg[2]};
            vh2vb_tp(s, vbcb);
            s->lfirst_tp = 0;
        }
        lindrift_tp(s, dth, 1);
        kick_vb_tp(s, dth, 1);
        drift_tp(s, dt);
        kick_vb_tp(s, dth, 0);
        lindrift_tp(s, dth, 0);
        double vbcb[3] = {-s->ptend[0], -s->ptend[1], -s->ptend[2]};
        vb2vh_tp(s, vbcb);
    }
}

/* ---- WHM ---- */
/* whm_coord_h2j_pl (whm_coord.f90:14-51) */
static void whm_h2j(orc_system *s) {
    int32_t n = s->npl;
    for (int d = 0; d < 3; d++) {
        s->xj[d] = s->rh[d];
        s->vj[d] = s->vh[d];
    }
    double sumx[3] = {0, 0, 0}, sumv[3] = {0, 0, 0};
    for (int32_t i = 1; i < n; i++) {
        for (int d = 0; d < 3; d++) {
            sumx[d] = sumx[d] + s->Gmass[i - 1] * s->rh[3 * (i - 1) + d];
            sumv[d] = sumv[d] + s->Gmass[i - 1] * s->vh[3 * (i - 1) + d];
            double cap = sumx[d] / s->eta[i - 1];
            double capv = sumv[d] / s->eta[i - 1];
            s->xj[3 * i + d] = s->rh[3 * i + d] - cap;
            s->vj[3 * i + d] = s->vh[3 * i + d] - capv;
        }
    }
}
/* whm_coord_j2h_pl (:54-90) */
static void whm_j2h(orc_system *s) {
    int32_t n = s->npl;
    for (int d = 0; d < 3; d++) {
        s->rh[d] = s->xj[d];
        s->vh[d] = s->vj[d];
    }
    double sumx[3] = {0, 0, 0}, sumv[3] = {0, 0, 0};
    for (int32_t i = 1; i < n; i++) {
        for (int d = 0; d < 3; d++) {
            sumx[d] = sumx[d] + s->Gmass[i - 1] * s->xj[3 * (i - 1) + d] / s->eta[i - 1];
            sumv[d] = sumv[d] + s->Gmass[i - 1] * s->vj[3 * (i - 1) + d] / s->eta[i - 1];
            s->rh[3 * i + d] = s->xj[3 * i + d] + sumx[d];
            s->vh[3 * i + d] = s->vj[3 * i + d] + sumv[d];
        }
    }
}
/* whm_coord_vh2vj_pl (:93-124) */
static void whm_vh2vj(orc_system *s) {
    int32_t n = s->npl;
    for (int d = 0; d < 3; d++) s->vj[d] = s->vh[d];
    double sumv[3] = {0, 0, 0};
    for (int32_t i = 1; i < n; i++)
        for (int d = 0; d < 3; d++) {
            sumv[d] = sumv[d] + s->Gmass[i - 1] * s->vh[3 * (i - 1) + d];
            double capv = sumv[d] / s->eta[i - 1];
            s->vj[3 * i + d] = s->vh[3 * i + d] - capv;
        }
}
/* whm_kick_getacch_ah0 (whm_kick.f90:125-149) */
static void whm_ah0(const double *mu, const double *rhp, int32_t n, double *ah0) {
    ah0[0] = ah0[1] = ah0[2] = 0.0;
    for (int32_t i = 0; i < n; i++) {
        double r2 = rhp[3 * i] * rhp[3 * i] + rhp[3 * i + 1] * rhp[3 * i + 1] + rhp[3 * i + 2] * rhp[3 * i + 2];
        double ir3h = 1.0 / (r2 * sqrt(r2));
        double fac = mu[i] * ir3h;
        for (int d = 0; d < 3; d++) ah0[d] = ah0[d] - fac * rhp[3 * i + d];
    }
}
/* whm_kick_getacch_pl (whm_kick.f90:14-67), with set_ir3j (whm_util.f90:117-140), ah1 (:152-179), ah2 (:182-215) */
static void whm_accel_pl(orc_system *s) {
    int32_t n = s->npl;
    for (int32_t i = 0; i < n; i++) {
        double r2 = s->rh[3 * i] * s->rh[3 * i] + s->rh[3 * i + 1] * s->rh[3 * i + 1] + s->rh[3 * i + 2] * s->rh[3 * i + 2];
        double ir = 1.0 / sqrt(r2);
        s->ir3h[i] = ir / r2;
        r2 = s->xj[3 * i] * s->xj[3 * i] + s->xj[3 * i + 1] * s->xj[3 * i + 1] + s->xj[3 * i + 2] * s->xj[3 * i + 2];
        ir = 1.0 / sqrt(r2);
        s->ir3j[i] = ir / r2;
    }
    double ah0[3];
    whm_ah0(s->Gmass + 1, s->rh + 3, n - 1, ah0);
    for (int32_t i = 0; i < n; i++)
        for (int d = 0; d < 3; d++) s->ah[3 * i + d] = s->ah[3 * i + d] + ah0[d];
    for (int32_t i = 1; i < n; i++) {
        if (!s->lmask[i]) continue;
        for (int d = 0; d < 3; d++) {
            double ah1j = s->xj[3 * i + d] * s->ir3j[i];
            double ah1h = s->rh[3 * i + d] * s->ir3h[i];
            s->ah[3 * i + d] = s->ah[3 * i + d] + s->GMcb * (ah1j - ah1h);
        }
    }
    double ah2[3] = {0, 0, 0}, ah2o[3] = {0, 0, 0};
    double etaj = s->GMcb;
    for (int32_t i = 1; i < n; i++) {
        if (!s->lmask[i]) continue;
        etaj = etaj + s->Gmass[i - 1];
        double fac = s->Gmass[i] * s->GMcb * s->ir3j[i] / etaj;
        for (int d = 0; d < 3; d++) {
            ah2[d] = ah2o[d] + fac * s->xj[3 * i + d];
            s->ah[3 * i + d] = s->ah[3 * i + d] + ah2[d];
            ah2o[d] = ah2[d];
        }
    }
    accel_int_pl(s);
}
/* whm_kick_getacch_tp (whm_kick.f90:70-122) */
static void whm_accel_tp(orc_system *s, int lbeg) {
    if (s->ntp == 0 || s->npl == 0) return;
    const double *rp = lbeg ? s->rbeg : s->rend;
    double ah0[3];
    whm_ah0(s->Gmass, rp, s->npl, ah0);
    for (int32_t i = 0; i < s->ntp; i++)
        if (s->tlmask[i])
            for (int d = 0; d < 3; d++) s->tah[3 * i + d] = s->tah[3 * i + d] + ah0[d];
    orc_kick_getacch_int_all_tp(s->ntp, s->npl, s->trh, rp, s->Gmass, s->tlmask, s->tah);
}
/* whm_kick_vh_pl (whm_kick.f90:218-262) */
static void whm_kick_vh_pl(orc_system *s, double dt, int lbeg) {
    int32_t n = s->npl;
    if (n == 0) return;
    if (lbeg) {
        if (s->lfirst_pl) {
            whm_h2j(s);
            memset(s->ah, 0, sizeof(double) * 3 * n);
            whm_accel_pl(s);
            s->lfirst_pl = 0;
        }
        memcpy(s->rbeg, s->rh, sizeof(double) * 3 * n);
    } else {
        memset(s->ah, 0, sizeof(double) * 3 * n);
        whm_accel_pl(s);
        memcpy(s->rend, s->rh, sizeof(double) * 3 * n);
    }
    for (int32_t i = 0; i < n; i++)
        if (s->lmask[i])
            for (int d = 0; d < 3; d++) s->vh[3 * i + d] = s->vh[3 * i + d] + s->ah[3 * i + d] * dt;
}
/* whm_kick_vh_tp (whm_kick.f90:265-318) */
static void whm_kick_vh_tp(orc_system *s, double dt, int lbeg) {
    if (s->ntp == 0) return;
    if (s->lfirst_tp) {
        for (int32_t i = 0; i < s->ntp; i++)
            if (s->tlmask[i]) s->tah[3 * i] = s->tah[3 * i + 1] = s->tah[3 * i + 2] = 0.0;
        whm_accel_tp(s, 1);
        s->lfirst_tp = 0;
    }
    if (!lbeg) {
        for (int32_t i = 0; i < s->ntp; i++)
            if (s->tlmask[i]) s->tah[3 * i] = s->tah[3 * i + 1] = s->tah[3 * i + 2] = 0.0;
        whm_accel_tp(s, lbeg);
    }
    for (int32_t i = 0; i < s->ntp; i++)
        if (s->tlmask[i])
            for (int d = 0; d < 3; d++) s->tvh[3 * i + d] = s->tvh[3 * i + d] + s->tah[3 * i + d] * dt;
}
/* whm_step_system / _pl / _tp (whm_step.f90:14-104), whm_drift_pl (whm_drift.f90:14-58) */
static int whm_step(orc_system *s, double dt) {
    double dth = 0.5 * dt;
    s->lfirst_tp = s->lfirst_pl;
    if (s->npl > 0) {
        whm_kick_vh_pl(s, dth, 1);
        whm_vh2vj(s);
        int32_t *iflag = calloc(s->npl, 4);
        orc_drift_all(s->muj, s->xj, s->vj, s->npl, 0, 0.0, dt, s->lmask, iflag);
        int bad = 0;
        for (int32_t i = 0; i < s->npl; i++)
            if (iflag[i]) {
                s->status[i] = ST_DISCARDED_DRIFTERR;
                s->lmask[i] = 0;
                bad = 1;
            }
        free(iflag);
        if (bad) return -5; /* the reference aborts the run (base_util_exit) */
        whm_j2h(s);
        whm_kick_vh_pl(s, dth, 0);
    }
    if (s->ntp > 0) {
        whm_kick_vh_tp(s, dth, 1);
        drift_tp(s, dt);
        whm_kick_vh_tp(s, dth, 0);
    }
    return 0;
}

/* ---- SyMBA ---- */
/* symba_util_set_renc (symba_util.f90:245-267) */
static void symba_set_renc(orc_system *s, int scale) {
    double rshell_irec = 1.0;
    for (int i = 1; i <= scale; i++) rshell_irec = rshell_irec * RSHELL;
    for (int32_t i = 0; i < s->npl; i++) s->renc[i] = s->rhill[i] * s->rhscale * rshell_irec;
}

/* symba_step_reset_system (symba_step.f90:265-331) */
static void symba_reset(orc_system *s) {
    s->plpl.n = 0;
    s->pltp.n = 0;
    for (int32_t i = 0; i < s->npl; i++) {
        s->nplenc[i] = s->ntpenc[i] = 0;
        s->levelg[i] = s->levelm[i] = -1;
        s->lencounter[i] = 0;
        /* the reference sets lmask = .true. because merged bodies have left its arrays;
         * here they stay in place with status INACTIVE */
        s->lmask[i] = s->status[i] != ST_INACTIVE;
    }
    symba_set_renc(s, 0);
    for (int32_t i = 0; i < s->ntp; i++) {
        s->tnplenc[i] = 0;
        s->tlevelg[i] = s->tlevelm[i] = -1;
        s->tlmask[i] = s->tstatus[i] != ST_INACTIVE;
    }
    s->lfirst_tp = s->lfirstkick;
    s->lfirst_pl = s->lfirstkick;
}

/* symba_encounter_check_pl (symba_encounter_check.f90:14-87) */
static int symba_encounter_check_pl(orc_system *s, double dt, int irec) {
    if (s->npl == 0) return 0;
    symba_set_renc(s, irec);
    int64_t nenc = 0;
    int rc;
    for (;;) {
        int32_t nplt = s->npl - s->nplm;
        if (nplt == 0)
            rc = orc_encounter_check_all_plpl(s->enc_plpl, s->npl, s->rh, s->vb, s->renc, dt, s->plpl.cap, &nenc,
                                              s->plpl.i1, s->plpl.i2, s->plpl.lvdotr);
        else
            rc = orc_encounter_check_all_plplm(s->enc_plpl, s->nplm, nplt, s->rh, s->vb, s->rh + 3 * s->nplm,
                                               s->vb + 3 * s->nplm, s->renc, s->renc + s->nplm, dt, s->plpl.cap,
                                               &nenc, s->plpl.i1, s->plpl.i2, s->plpl.lvdotr);
        if (rc == 0) break;
        enclist_reserve(&s->plpl, nenc);
    }
    s->plpl.n = nenc;
    for (int64_t k = 0; k < nenc; k++) {
        int32_t i = s->plpl.i1[k] - 1, j = s->plpl.i2[k] - 1;
        s->plpl.status[k] = ST_ACTIVE;
        s->plpl.level[k] = irec;
        s->lencounter[i] = s->lencounter[j] = 1;
        s->levelg[i] = s->levelm[i] = irec;
        s->levelg[j] = s->levelm[j] = irec;
        s->nplenc[i]++;
        s->nplenc[j]++;
    }
    return nenc > 0;
}

/* symba_encounter_check_tp (symba_encounter_check.f90:238-296) */
static int symba_encounter_check_tp(orc_system *s, double dt, int irec) {
    if (s->ntp == 0) return 0;
    symba_set_renc(s, irec);
    int64_t nenc = 0;
    for (;;) {
        int rc = orc_encounter_check_all_pltp(s->enc_pltp, s->npl, s->ntp, s->rh, s->vb, s->trh, s->tvb, s->renc, dt,
                                              s->pltp.cap, &nenc, s->pltp.i1, s->pltp.i2, s->pltp.lvdotr);
        if (rc == 0) break;
        enclist_reserve(&s->pltp, nenc);
    }
    s->pltp.n = nenc;
    if (nenc > 0) {
        for (int32_t i = 0; i < s->npl; i++) s->lencounter[i] = 0;
        for (int64_t k = 0; k < nenc; k++) {
            int32_t i = s->pltp.i1[k] - 1, j = s->pltp.i2[k] - 1;
            s->pltp.status[k] = ST_ACTIVE;
            s->pltp.level[k] = irec;
            s->lencounter[i] = 1;
            s->levelg[i] = s->levelm[i] = irec;
            s->tlevelg[j] = s->tlevelm[j] = irec;
            s->ntpenc[i]++;
            s->tnplenc[j]++;
        }
    }
    return nenc > 0;
}

/* symba_encounter_check_list_plpl (symba_encounter_check.f90:90-160) */
static int symba_list_check_plpl(orc_system *s, double dt, int irec) {
    if (s->plpl.n == 0) return 0;
    int any_mask = 0;
    for (int64_t k = 0; k < s->plpl.n; k++)
        if (s->plpl.status[k] == ST_ACTIVE && s->plpl.level[k] == irec - 1) any_mask = 1;
    if (!any_mask) return 0;
    symba_set_renc(s, irec);
    int64_t n = s->plpl.n;
    int32_t *lenc = calloc(n, 4);
    for (int64_t k = 0; k < n; k++) {
        if (!(s->plpl.status[k] == ST_ACTIVE && s->plpl.level[k] == irec - 1)) continue;
        int32_t i = s->plpl.i1[k] - 1, j = s->plpl.i2[k] - 1;
        double xr[3], vr[3];
        for (int d = 0; d < 3; d++) {
            xr[d] = s->rh[3 * j + d] - s->rh[3 * i + d];
            vr[d] = s->vb[3 * j + d] - s->vb[3 * i + d];
        }
        double rcrit12 = s->renc[i] + s->renc[j];
        int32_t le, lv;
        orc_encounter_check_one(xr[0], xr[1], xr[2], vr[0], vr[1], vr[2], rcrit12, dt, &le, &lv);
        s->plpl.lvdotr[k] = lv;
        if (le) {
            double rs = s->radius[i] + s->radius[j];
            double rlim2 = rs * rs;
            double rji2 = xr[0] * xr[0] + xr[1] * xr[1] + xr[2] * xr[2];
            le = rji2 > rlim2;
        }
        lenc[k] = le;
    }
    int any = 0;
    for (int64_t k = 0; k < n; k++) {
        if (!lenc[k]) continue;
        any = 1;
        int32_t i = s->plpl.i1[k] - 1, j = s->plpl.i2[k] - 1;
        s->levelg[i] = irec;
        s->levelm[i] = irec > s->levelm[i] ? irec : s->levelm[i];
        s->levelg[j] = irec;
        s->levelm[j] = irec > s->levelm[j] ? irec : s->levelm[j];
        s->plpl.level[k] = irec;
    }
    free(lenc);
    return any;
}

/* symba_encounter_check_list_pltp (symba_encounter_check.f90:163-235) */
static int symba_list_check_pltp(orc_system *s, double dt, int irec) {
    if (s->pltp.n == 0) return 0;
    int any_mask = 0;
    for (int64_t k = 0; k < s->pltp.n; k++)
        if (s->pltp.status[k] == ST_ACTIVE && s->pltp.level[k] == irec - 1) any_mask = 1;
    if (!any_mask) return 0;
    symba_set_renc(s, irec);
    int64_t n = s->pltp.n;
    int32_t *lenc = calloc(n, 4);
    for (int64_t k = 0; k < n; k++) {
        if (!(s->pltp.status[k] == ST_ACTIVE && s->pltp.level[k] == irec - 1)) continue;
        int32_t i = s->pltp.i1[k] - 1, j = s->pltp.i2[k] - 1;
        double xr[3], vr[3];
        for (int d = 0; d < 3; d++) {
            xr[d] = s->trh[3 * j + d] - s->rh[3 * i + d];
            vr[d] = s->tvb[3 * j + d] - s->vb[3 * i + d];
        }
        int32_t le, lv;
        orc_encounter_check_one(xr[0], xr[1], xr[2], vr[0], vr[1], vr[2], s->renc[i], dt, &le, &lv);
        s->pltp.lvdotr[k] = lv;
        if (le) {
            double rlim2 = s->radius[i] * s->radius[i];
            double rji2 = xr[0] * xr[0] + xr[1] * xr[1] + xr[2] * xr[2];
            le = rji2 > rlim2;
        }
        lenc[k] = le;
    }
    int any = 0;
    for (int64_t k = 0; k < n; k++) {
        if (!lenc[k]) continue;
        any = 1;
        int32_t i = s->pltp.i1[k] - 1, j = s->pltp.i2[k] - 1;
        s->levelg[i] = irec;
        s->levelm[i] = irec > s->levelm[i] ? irec : s->levelm[i];
        s->tlevelg[j] = irec;
        s->tlevelm[j] = irec > s->tlevelm[j] ? irec : s->tlevelm[j];
        s->pltp.level[k] = irec;
    }
    free(lenc);
    return any;
}

/* symba_kick_list_plpl (symba_kick.f90:126-232) */
static void symba_kick_list_plpl(orc_system *s, double dt, int irec, int sgn) {
    int64_t nenc = s->plpl.n;
    if (nenc == 0 || s->npl == 0) return;
    for (int32_t i = 0; i < s->npl; i++) s->lmask[i] = s->status[i] != ST_INACTIVE;
    int irm1 = irec - 1;
    int irecl = sgn < 0 ? irec - 1 : irec;
    int32_t *good = calloc(nenc, 4);
    int64_t ngood = 0;
    for (int64_t k = 0; k < nenc; k++) {
        int32_t i = s->plpl.i1[k] - 1, j = s->plpl.i2[k] - 1;
        good[k] = (s->levelg[i] >= irm1) && (s->levelg[j] >= irm1);
        good[k] = (s->plpl.status[k] == ST_ACTIVE) && good[k];
        ngood += good[k];
    }
    if (ngood > 0) {
        for (int64_t k = 0; k < nenc; k++) {
            if (!good[k]) continue;
            int32_t i = s->plpl.i1[k] - 1, j = s->plpl.i2[k] - 1;
            for (int d = 0; d < 3; d++) s->ah[3 * i + d] = s->ah[3 * j + d] = 0.0;
        }
        double rs2 = s->rhscale * s->rhscale;
        double rshell_pow = powi(RSHELL, 2 * irecl);
        for (int64_t k = 0; k < nenc; k++) {
            if (!good[k]) continue;
            int32_t i = s->plpl.i1[k] - 1, j = s->plpl.i2[k] - 1;
            double rhs = s->rhill[i] + s->rhill[j];
            double ri = ((rhs * rhs) * rs2) * rshell_pow;
            double rim1 = ri * (RSHELL * RSHELL);
            double dx[3];
            for (int d = 0; d < 3; d++) dx[d] = s->rh[3 * j + d] - s->rh[3 * i + d];
            double r2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
            double fac;
            if (r2 < rim1) {
                good[k] = 0;
                continue;
            }
            if (r2 < ri) {
                double ris = sqrt(ri);
                double r = sqrt(r2);
                double rr = (ris - r) / (ris * (1.0 - RSHELL));
                fac = pow_m1p5(r2) * (1.0 - 3.0 * (rr * rr) + 2.0 * (rr * rr * rr));
            } else {
                double ir3 = 1.0 / (r2 * sqrt(r2));
                fac = ir3;
            }
            double faci = fac * s->Gmass[i];
            double facj = fac * s->Gmass[j];
            for (int d = 0; d < 3; d++) {
                s->ah[3 * i + d] = s->ah[3 * i + d] + facj * dx[d];
                s->ah[3 * j + d] = s->ah[3 * j + d] - faci * dx[d];
            }
        }
        for (int64_t k = 0; k < nenc; k++) {
            if (!good[k]) continue;
            int32_t i = s->plpl.i1[k] - 1, j = s->plpl.i2[k] - 1;
            for (int d = 0; d < 3; d++) {
                s->vb[3 * i + d] = s->vb[3 * i + d] + (double)sgn * dt * s->ah[3 * i + d];
                s->vb[3 * j + d] = s->vb[3 * j + d] + (double)sgn * dt * s->ah[3 * j + d];
            }
            for (int d = 0; d < 3; d++) s->ah[3 * i + d] = s->ah[3 * j + d] = 0.0;
        }
    }
    free(good);
}

/* symba_kick_list_pltp (symba_kick.f90:235-340) */
static void symba_kick_list_pltp(orc_system *s, double dt, int irec, int sgn) {
    int64_t nenc = s->pltp.n;
    if (nenc == 0 || s->npl == 0 || s->ntp == 0) return;
    for (int32_t i = 0; i < s->npl; i++) s->lmask[i] = s->status[i] != ST_INACTIVE;
    for (int32_t i = 0; i < s->ntp; i++) s->tlmask[i] = s->tstatus[i] != ST_INACTIVE;
    int irm1 = irec - 1;
    int irecl = sgn < 0 ? irec - 1 : irec;
    int32_t *good = calloc(nenc, 4);
    int64_t ngood = 0;
    for (int64_t k = 0; k < nenc; k++) {
        int32_t i = s->pltp.i1[k] - 1, j = s->pltp.i2[k] - 1;
        good[k] = (s->levelg[i] >= irm1) && (s->tlevelg[j] >= irm1);
        good[k] = (s->pltp.status[k] == ST_ACTIVE) && good[k];
        ngood += good[k];
    }
    if (ngood > 0) {
        for (int64_t k = 0; k < nenc; k++) {
            if (!good[k]) continue;
            int32_t j = s->pltp.i2[k] - 1;
            for (int d = 0; d < 3; d++) s->tah[3 * j + d] = 0.0;
        }
        double rs2 = s->rhscale * s->rhscale;
        double rshell_pow = powi(RSHELL, 2 * irecl);
        for (int64_t k = 0; k < nenc; k++) {
            if (!good[k]) continue;
            int32_t i = s->pltp.i1[k] - 1, j = s->pltp.i2[k] - 1;
            double ri = ((s->rhill[i] * s->rhill[i]) * rs2) * rshell_pow;
            double rim1 = ri * (RSHELL * RSHELL);
            double dx[3];
            for (int d = 0; d < 3; d++) dx[d] = s->trh[3 * j + d] - s->rh[3 * i + d];
            double r2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
            double fac;
            if (r2 < rim1) {
                good[k] = 0;
                continue;
            }
            if (r2 < ri) {
                double ris = sqrt(ri);
                double r = sqrt(r2);
                double rr = (ris - r) / (ris * (1.0 - RSHELL));
                fac = pow_m1p5(r2) * (1.0 - 3.0 * (rr * rr) + 2.0 * (rr * rr * rr));
            } else {
                double ir3 = 1.0 / (r2 * sqrt(r2));
                fac = ir3;
            }
            double faci = fac * s->Gmass[i];
            for (int d = 0; d < 3; d++) s->tah[3 * j + d] = s->tah[3 * j + d] - faci * dx[d];
        }
        for (int64_t k = 0; k < nenc; k++) {
            if (!good[k]) continue;
            int32_t j = s->pltp.i2[k] - 1;
            for (int d = 0; d < 3; d++) {
                s->tvb[3 * j + d] = s->tvb[3 * j + d] + (double)sgn * dt * s->tah[3 * j + d];
                s->tah[3 * j + d] = 0.0;
            }
        }
    }
    free(good);
}

/* symba_step_set_recur_levels_system (symba_step.f90:118-160) */
/* swiftest_orbel_xv2aeq (src/swiftest/swiftest_orbel.f90:700-764) */
static void xv2aeq(double mu, double rx, double ry, double rz, double vx, double vy, double vz, double *a,
                   double *e, double *q) {
    const double TINYV = 4.0e-15; /* swiftest_orbel.f90:11 */
    *a = 0.0;
    *e = 0.0;
    *q = 0.0;
    double r = sqrt(rx * rx + ry * ry + rz * rz);
    double v2 = vx * vx + vy * vy + vz * vz;
    double hx = ry * vz - rz * vy, hy = rz * vx - rx * vz, hz = rx * vy - ry * vx;
    double h2 = hx * hx + hy * hy + hz * hz;
    if (h2 < 2.2250738585072014e-308) return; /* tiny(1.0_DP) */
    double energy = 0.5 * v2 - mu / r;
    int type; /* -1 ellipse, 0 parabola, 1 hyperbola */
    double fac = 0.0;
    if (fabs(energy * r / mu) < sqrt(TINYV)) {
        type = 0;
    } else {
        *a = -0.5 * mu / energy;
        if (*a < 0.0) {
            fac = -h2 / (mu * *a);
            type = fac > TINYV ? 1 : 0;
        } else {
            type = -1;
        }
    }
    if (type == -1) {
        fac = 1.0 - h2 / (mu * *a);
        if (fac > TINYV) *e = sqrt(fac);
        *q = *a * (1.0 - *e);
    } else if (type == 0) {
        *a = 0.5 * h2 / mu;
        *e = 1.0;
        *q = *a;
    } else {
        *e = sqrt(1.0 + fac);
        *q = *a * (1.0 - *e);
    }
}

/* collision_check_one (src/collision/collision_check.f90:16-57) */
static int collision_check_one(double xr, double yr, double zr, double vxr, double vyr, double vzr, double Gmtot,
                               double rlim, double dt, int lvdotr) {
    double r2 = xr * xr + yr * yr + zr * zr;
    double rlim2 = rlim * rlim;
    if (r2 <= rlim2) return 1;
    double vdotr = xr * vxr + yr * vyr + zr * vzr;
    if (lvdotr && vdotr > 0.0) {
        double tcr2 = r2 / (vxr * vxr + vyr * vyr + vzr * vzr);
        double dt2 = dt * dt;
        if (tcr2 <= dt2) {
            double a, e, q;
            xv2aeq(Gmtot, xr, yr, zr, vxr, vyr, vzr, &a, &e, &q);
            return q < rlim;
        }
    }
    return 0;
}

/* collision_check_plpl (src/collision/collision_check.f90:60-160): ACTIVE pairs whose
 * index1 body sits at level >= irec; a colliding pair's status becomes COLLIDED and both of
 * its bodies are flagged (the reference sets their status to COLLIDED).  Returns whether
 * any pair collided. */
static int collision_check_plpl(orc_system *s, int irec, double dt, unsigned char *coll) {
    int any = 0;
    for (int64_t k = 0; k < s->plpl.n; k++) {
        if (s->plpl.status[k] != ST_ACTIVE) continue;
        int32_t i = s->plpl.i1[k] - 1, j = s->plpl.i2[k] - 1;
        if (s->levelg[i] < irec) continue;
        double x[3], v[3];
        for (int d = 0; d < 3; d++) {
            x[d] = s->rh[3 * i + d] - s->rh[3 * j + d];
            v[d] = s->vb[3 * i + d] - s->vb[3 * j + d];
        }
        if (collision_check_one(x[0], x[1], x[2], v[0], v[1], v[2], s->Gmass[i] + s->Gmass[j],
                                s->radius[i] + s->radius[j], dt, s->plpl.lvdotr[k] != 0)) {
            s->plpl.status[k] = ST_COLLIDED;
            if (coll) coll[i] = coll[j] = 1;
            any = 1;
        }
    }
    return any;
}

/* collision_check_pltp (src/collision/collision_check.f90:163-271): ACTIVE pairs whose tp
 * sits at level >= irec. */
static int collision_check_pltp(orc_system *s, int irec, double dt) {
    int any = 0;
    for (int64_t k = 0; k < s->pltp.n; k++) {
        if (s->pltp.status[k] != ST_ACTIVE) continue;
        int32_t i = s->pltp.i1[k] - 1, j = s->pltp.i2[k] - 1;
        if (s->tlevelg[j] < irec) continue;
        double x[3], v[3];
        for (int d = 0; d < 3; d++) {
            x[d] = s->rh[3 * i + d] - s->trh[3 * j + d];
            v[d] = s->vb[3 * i + d] - s->tvb[3 * j + d];
        }
        if (collision_check_one(x[0], x[1], x[2], v[0], v[1], v[2], s->Gmass[i], s->radius[i], dt,
                                s->pltp.lvdotr[k] != 0)) {
            s->pltp.status[k] = ST_COLLIDED;
            any = 1;
        }
    }
    return any;
}

/* ---- Resolution of the COLLIDED pairs by perfect merging.
 *
 * collision_resolve_plpl (src/collision/collision_resolve.f90:521-662) with the MERGE model
 * (collision_generate_merge, collision_generate.f90:158-260; collision_resolve_mergeaddsub,
 * collision_resolve.f90:326-518) and the parts of swiftest_util_rearray_pl
 * (swiftest_util.f90:1638-1808) that change the state, then collision_resolve_pltp
 * (:665-695).  Energy tracking is on, as in runs that report |dE/E|, and masses are G*m (the
 * reference's m = G*m/GU with GU = 1), so energies and angular momenta are G times the
 * reference's and every ratio is unchanged.  Per resolution:
 *   1. sync: the central body's barycentric velocity (vb2vh, reverse order) and position
 *      (rh2rb, which also gives every body's rb);
 *   2. E_before, L_before: the system's energy and angular momentum;
 *   3. each COLLIDED pair whose two bodies were both flagged by the check, in list order:
 *      the impactors' centre of mass (rb = rh + cb rb), the angular momentum of each
 *      impactor about it, L_escape += both (no rotation: the reference books the
 *      pre-collision orbital angular momentum as escaped), the merged body at the centre of
 *      mass with the summed G*m and the radius of the summed volume, its velocity torqued by
 *      the impactors' angular momentum (collision_util_velocity_torque), list entries of the
 *      removed body redirected to the merged one (a resulting self-pair becomes INACTIVE);
 *   4. the Hill radius of every body from its current orbit (set_rhill in rearray);
 *   5. the new system angular momentum: each merged body's velocity is torqued by
 *      -(L_after - L_before) * m / (sum of the merged masses), then E_collisions +=
 *      E_after - E_before (E_before stays the value of step 2 through a cascade, as in the
 *      reference);
 *   6. the cascade: the pl-pl list is checked again at the same level (newly collided pairs
 *      flag their bodies); repeat from 3 while any pair collides, at most 1000 times.
 * The merged body keeps the slot of the more massive impactor (the first on a tie); the
 * other stays in its slot with status INACTIVE, zero G*m, radius, Hill radius and
 * velocity, parked at a distant position of its own.  Not restated: the re-sort by mass
 * and the re-run of the encounter checks inside rearray (whose old and new lists are
 * matched entry by entry), and the kinship grouping of a body that collides with two
 * others in one check (the reference merges all three at once; here the first pair merges,
 * the other pair is set ACTIVE again and merges in the cascade if it still collides).
 * Returns -1 on a runaway cascade, else the number of merges plus discarded tp. */
static void park(double *r, double *v, int64_t k) {
    r[0] = 1.0e6 + (double)k;
    r[1] = r[2] = 0.0;
    v[0] = v[1] = v[2] = 0.0;
}

/* operator .unit. (src/operator/operator_unit.f90) */
static void unit3(const double *a, double *u) {
    double m = norm2_3(a);
    for (int d = 0; d < 3; d++) u[d] = m > 2.2250738585072014e-308 ? a[d] / m : 0.0;
}

/* operator .cross. (src/operator/operator_cross.f90) */
static void cross3(const double *a, const double *b, double *c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

/* collision_util_velocity_torque (src/collision/collision_util.f90:1001-1026) */
static void velocity_torque(const double *dL, double mass, const double *r, double *v) {
    double dLu[3], ru[3], q[3], c[3];
    unit3(dL, dLu);
    unit3(r, ru);
    double rmag = norm2_3(r), vmag = norm2_3(v);
    for (int d = 0; d < 3; d++) q[d] = dL[d] / (rmag * mass);
    double vapply_mag = norm2_3(q);
    if (vapply_mag / vmag > 2.220446049250313e-16) {
        cross3(dLu, ru, c);
        for (int d = 0; d < 3; d++) v[d] = v[d] + vapply_mag * c[d];
    }
}

/* swiftest_orbel_xv2el (src/swiftest/swiftest_orbel.f90:913-1072): the semimajor axis */
static double xv2el_a(double mu, const double *r, const double *v) {
    const double TINYV = 4.0e-15;
    double hx = r[1] * v[2] - r[2] * v[1], hy = r[2] * v[0] - r[0] * v[2], hz = r[0] * v[1] - r[1] * v[0];
    double h2 = hx * hx + hy * hy + hz * hz;
    if (h2 <= 10.0 * 2.2250738585072014e-308) return 0.0;
    double rr = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    double v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    double energy = 0.5 * v2 - mu / rr;
    if (fabs(energy * rr / mu) < sqrt(TINYV)) return 0.5 * h2 / mu; /* parabola */
    double a = -0.5 * mu / energy;
    if (a < 0.0 && !(-h2 / (mu * a) > TINYV)) return 0.5 * h2 / mu; /* parabola */
    return a;
}

/* swiftest_util_get_energy_and_momentum_system (swiftest_util.f90:1172-1291, triangular
 * potential :1350-1401) as the resolution calls it: body positions rb, velocities vb, the
 * central body's rb/vb as the resolution's sync left them, no spin terms. */
static void resolve_energy(const orc_system *s, const double *rb, const double *cbrb, const double *cbvb,
                           double *te, double *L) {
    int32_t n = s->npl;
    double mcb = s->GMcb;
    double kecb = mcb * (cbvb[0] * cbvb[0] + cbvb[1] * cbvb[1] + cbvb[2] * cbvb[2]);
    double Lcb[3] = {mcb * (cbrb[1] * cbvb[2] - cbrb[2] * cbvb[1]), mcb * (cbrb[2] * cbvb[0] - cbrb[0] * cbvb[2]),
                     mcb * (cbrb[0] * cbvb[1] - cbrb[1] * cbvb[0])};
    double kesum = 0.0, Lsum[3] = {0.0, 0.0, 0.0};
    for (int32_t i = 0; i < n; i++) {
        if (s->status[i] == ST_INACTIVE) continue;
        const double *r = &rb[3 * i], *v = &s->vb[3 * i];
        double m = s->Gmass[i];
        Lsum[0] = Lsum[0] + m * (r[1] * v[2] - r[2] * v[1]);
        Lsum[1] = Lsum[1] + m * (r[2] * v[0] - r[0] * v[2]);
        Lsum[2] = Lsum[2] + m * (r[0] * v[1] - r[1] * v[0]);
        kesum = kesum + m * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    }
    double pe = 0.0;
    for (int32_t i = 0; i < n; i++) {
        if (s->status[i] == ST_INACTIVE) continue;
        double row = 0.0;
        for (int32_t j = i + 1; j < n; j++) {
            if (s->status[j] == ST_INACTIVE) continue;
            double d[3] = {rb[3 * i] - rb[3 * j], rb[3 * i + 1] - rb[3 * j + 1], rb[3 * i + 2] - rb[3 * j + 2]};
            row = row + (-(s->Gmass[i] * s->Gmass[j]) / norm2_3(d));
        }
        pe = pe + row;
    }
    double pecb = 0.0, be = 0.0;
    for (int32_t i = 0; i < n; i++) {
        if (s->status[i] == ST_INACTIVE) continue;
        pecb = pecb + (-s->GMcb * s->Gmass[i] / norm2_3(&rb[3 * i]));
        be = be + (-3.0 * s->Gmass[i] * s->Gmass[i] / (5.0 * s->radius[i]));
    }
    pe = pe + pecb;
    double ke = 0.5 * (kecb + kesum);
    *te = ke + pe + be;
    for (int d = 0; d < 3; d++) L[d] = Lcb[d] + Lsum[d];
}

/* swiftest_util_coord_rh2rb_pl (swiftest_util.f90:488-521) into cbrb and rb */
static void resolve_rh2rb(const orc_system *s, double *cbrb, double *rb) {
    double Gmtot = s->GMcb, xtmp[3] = {0.0, 0.0, 0.0};
    for (int32_t i = 0; i < s->npl; i++) {
        if (s->status[i] == ST_INACTIVE) continue;
        Gmtot = Gmtot + s->Gmass[i];
        for (int d = 0; d < 3; d++) xtmp[d] = xtmp[d] + s->Gmass[i] * s->rh[3 * i + d];
    }
    for (int d = 0; d < 3; d++) cbrb[d] = -xtmp[d] / Gmtot;
    for (int32_t i = 0; i < s->npl; i++) {
        if (s->status[i] == ST_INACTIVE) continue;
        for (int d = 0; d < 3; d++) rb[3 * i + d] = s->rh[3 * i + d] + cbrb[d];
    }
}

static int64_t resolve_plpl(orc_system *s, int irec, double dtl) {
    int32_t n = s->npl;
    int any = 0;
    for (int64_t k = 0; k < s->plpl.n; k++) any |= s->plpl.status[k] == ST_COLLIDED;
    if (!any) return 0;
    unsigned char *coll = calloc((size_t)(n > 0 ? n : 1), 1);
    double *rb = calloc((size_t)3 * (n > 0 ? n : 1), 8);
    double *vh = calloc((size_t)3 * (n > 0 ? n : 1), 8);
    int32_t *newb = malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    for (int64_t k = 0; k < s->plpl.n; k++)
        if (s->plpl.status[k] == ST_COLLIDED) coll[s->plpl.i1[k] - 1] = coll[s->plpl.i2[k] - 1] = 1;
    /* 1. sync: vb2vh (swiftest_util.f90:363-395; vh is not refreshed afterwards, the merged
     * bodies get theirs from b2h) and rh2rb */
    double cbvb[3] = {0.0, 0.0, 0.0}, cbrb[3];
    for (int32_t b = n - 1; b >= 0; b--) {
        if (s->status[b] == ST_INACTIVE) continue;
        for (int d = 0; d < 3; d++) cbvb[d] = cbvb[d] - s->Gmass[b] * s->vb[3 * b + d] / s->GMcb;
    }
    for (int32_t b = 0; b < n; b++)
        for (int d = 0; d < 3; d++) vh[3 * b + d] = s->vb[3 * b + d] - cbvb[d];
    resolve_rh2rb(s, cbrb, rb);
    /* 2. */
    double E_before, L_before[3];
    resolve_energy(s, rb, cbrb, cbvb, &E_before, L_before);
    int64_t nres = 0;
    for (int loop = 1;; loop++) {
        /* 3. */
        int32_t nnew = 0;
        for (int64_t k = 0; k < s->plpl.n; k++) {
            if (s->plpl.status[k] != ST_COLLIDED) continue;
            int32_t i = s->plpl.i1[k] - 1, j = s->plpl.i2[k] - 1;
            if (!coll[i] || !coll[j]) {
                /* one impactor already merged in this pass: test the pair again */
                if (s->status[i] != ST_INACTIVE && s->status[j] != ST_INACTIVE && i != j)
                    s->plpl.status[k] = ST_ACTIVE;
                continue;
            }
            double m1 = s->Gmass[i], m2 = s->Gmass[j], mtot = m1 + m2;
            double rb1[3], rb2[3], rbcom[3], vbcom[3], rc1[3], rc2[3], vc1[3], vc2[3];
            const double *vb1 = &s->vb[3 * i], *vb2 = &s->vb[3 * j];
            for (int d = 0; d < 3; d++) {
                rb1[d] = s->rh[3 * i + d] + cbrb[d];
                rb2[d] = s->rh[3 * j + d] + cbrb[d];
            }
            for (int d = 0; d < 3; d++) {
                rbcom[d] = (m1 * rb1[d] + m2 * rb2[d]) / mtot;
                vbcom[d] = (m1 * vb1[d] + m2 * vb2[d]) / mtot;
            }
            for (int d = 0; d < 3; d++) {
                rc1[d] = rb1[d] - rbcom[d];
                rc2[d] = rb2[d] - rbcom[d];
                vc1[d] = vb1[d] - vbcom[d];
                vc2[d] = vb2[d] - vbcom[d];
            }
            double L1[3] = {m1 * (rc1[1] * vc1[2] - rc1[2] * vc1[1]), m1 * (rc1[2] * vc1[0] - rc1[0] * vc1[2]),
                            m1 * (rc1[0] * vc1[1] - rc1[1] * vc1[0])};
            double L2[3] = {m2 * (rc2[1] * vc2[2] - rc2[2] * vc2[1]), m2 * (rc2[2] * vc2[0] - rc2[0] * vc2[2]),
                            m2 * (rc2[0] * vc2[1] - rc2[1] * vc2[0])};
            double Lb[3];
            for (int d = 0; d < 3; d++) {
                Lb[d] = L1[d] + L2[d];
                s->L_escape[d] = s->L_escape[d] + L1[d] + L2[d];
            }
            double PI = 3.141592653589793238462643383279502884197;
            double Ri = s->radius[i], Rj = s->radius[j];
            double volume = 4.0 / 3.0 * PI * (Ri * Ri * Ri + Rj * Rj * Rj);
            double Rnew = pow(3.0 * volume / (4.0 * PI), THIRD);
            /* the merged body's velocity, torqued by the residual -(0 - Lb) */
            double vnew[3] = {vbcom[0], vbcom[1], vbcom[2]};
            double dL[3] = {-(0.0 - Lb[0]), -(0.0 - Lb[1]), -(0.0 - Lb[2])};
            velocity_torque(dL, mtot, rbcom, vnew);
            int32_t keep = m2 > m1 ? j : i, gone = keep == i ? j : i;
            for (int d = 0; d < 3; d++) {  /* collision_resolve_mergeaddsub: b2h of the new body */
                rb[3 * keep + d] = rbcom[d];
                s->rh[3 * keep + d] = rbcom[d] - cbrb[d];
                s->vb[3 * keep + d] = vnew[d];
                vh[3 * keep + d] = vnew[d] - cbvb[d];
            }
            s->Gmass[keep] = mtot;
            s->radius[keep] = Rnew;
            s->Gmass[gone] = 0.0;
            s->radius[gone] = 0.0;
            s->rhill[gone] = 0.0;
            s->status[gone] = ST_INACTIVE;
            s->lmask[gone] = 0;
            park(&s->rh[3 * gone], &s->vb[3 * gone], gone);
            coll[i] = coll[j] = 0;
            for (int64_t m = 0; m < s->plpl.n; m++) {
                if (s->plpl.i1[m] == gone + 1) s->plpl.i1[m] = keep + 1;
                if (s->plpl.i2[m] == gone + 1) s->plpl.i2[m] = keep + 1;
                if (s->plpl.i1[m] == s->plpl.i2[m]) s->plpl.status[m] = ST_INACTIVE;
            }
            for (int64_t m = 0; m < s->pltp.n; m++)
                if (s->pltp.i1[m] == gone + 1) s->pltp.i1[m] = keep + 1;
            newb[nnew++] = keep;
            nres++;
        }
        if (nnew == 0) break;
        double mnew = 0.0;
        for (int32_t q = 0; q < nnew; q++) mnew = mnew + s->Gmass[newb[q]];
        /* 4. */
        if (s->GMcb > 2.2250738585072014e-308) {
            for (int32_t b = 0; b < n; b++) {
                if (s->status[b] == ST_INACTIVE) continue;
                double a = xv2el_a(s->GMcb + s->Gmass[b], &s->rh[3 * b], &vh[3 * b]);
                double scale = pow(s->Gmass[b] / s->GMcb / 3.0, THIRD);
                s->rhill[b] = a > 0.0 ? a * scale : norm2_3(&s->rh[3 * b]) * scale;
            }
        }
        /* 5. */
        double E_after, L_after[3], dL[3];
        resolve_energy(s, rb, cbrb, cbvb, &E_after, L_after);
        for (int d = 0; d < 3; d++) dL[d] = L_after[d] - L_before[d];
        for (int32_t q = 0; q < nnew; q++) {
            int32_t b = newb[q];
            double t[3] = {-dL[0] * s->Gmass[b] / mnew, -dL[1] * s->Gmass[b] / mnew, -dL[2] * s->Gmass[b] / mnew};
            velocity_torque(t, s->Gmass[b], &rb[3 * b], &s->vb[3 * b]);
        }
        resolve_energy(s, rb, cbrb, cbvb, &E_after, L_after);
        s->E_collisions = s->E_collisions + (E_after - E_before);
        /* 6. */
        if (!collision_check_plpl(s, irec, dtl, coll)) break;
        if (loop == 1000) {
            nres = -1;
            break;
        }
        resolve_rh2rb(s, cbrb, rb);
    }
    free(coll);
    free(rb);
    free(vh);
    free(newb);
    return nres;
}

/* collision_resolve_pltp (collision_resolve.f90:665-695): the colliding tp is discarded */
static int64_t resolve_pltp(orc_system *s) {
    int64_t nres = 0;
    for (int64_t k = 0; k < s->pltp.n; k++) {
        if (s->pltp.status[k] != ST_COLLIDED) continue;
        int32_t j = s->pltp.i2[k] - 1;
        if (s->tstatus[j] == ST_INACTIVE) continue;
        s->tstatus[j] = ST_INACTIVE;
        s->tlmask[j] = 0;
        park(&s->trh[3 * j], &s->tvb[3 * j], (int64_t)s->npl + j);
        nres++;
    }
    return nres;
}

/* the collision step of symba_step_recur_system (symba_step.f90:242-249) */
static int symba_collisions(orc_system *s, int irec, double dtl) {
    int a = collision_check_plpl(s, irec, dtl, NULL);
    int b = collision_check_pltp(s, irec, dtl);
    if (a) {
        int64_t r = resolve_plpl(s, irec, dtl);
        if (r < 0) return -7;
        s->stats[4] += r;
    }
    if (b) s->stats[4] += resolve_pltp(s);
    return 0;
}

static void symba_set_recur_levels(orc_system *s, int ireci) {
    int irecp = ireci + 1;
    for (int32_t i = 0; i < s->npl; i++)
        if (s->levelg[i] == irecp) s->levelg[i] = ireci;
    for (int32_t i = 0; i < s->ntp; i++)
        if (s->tlevelg[i] == irecp) s->tlevelg[i] = ireci;
    for (int64_t k = 0; k < s->plpl.n; k++)
        if (s->plpl.level[k] == irecp) s->plpl.level[k] = ireci;
    for (int64_t k = 0; k < s->pltp.n; k++)
        if (s->pltp.level[k] == irecp) s->pltp.level[k] = ireci;
    s->irec = ireci;
}

/* symba_step_recur_system (symba_step.f90:163-262) */
static int symba_recur(orc_system *s, int ireci) {
    s->irec = ireci;
    double dtl = s->dt / (double)powi((double)NTENC, ireci);
    double dth = 0.5 * dtl;
    if (dtl / s->dt < 2.220446049250313e-16) return -6; /* local time step too small */
    int irecp = ireci + 1;
    if (irecp > s->stats[1]) s->stats[1] = irecp;
    int nloops = ireci == 0 ? 1 : NTENC;
    s->stats[5] += nloops;
    for (int j = 1; j <= nloops; j++) {
        int a = symba_list_check_plpl(s, dtl, irecp);
        int b = symba_list_check_pltp(s, dtl, irecp);
        int lencounter = a || b;
        symba_kick_list_plpl(s, dth, irecp, 1);
        symba_kick_list_pltp(s, dth, irecp, 1);
        if (ireci != 0) {
            symba_kick_list_plpl(s, dth, irecp, -1);
            symba_kick_list_pltp(s, dth, irecp, -1);
        }
        drift_pl(s, dtl);
        drift_tp(s, dtl);
        if (lencounter) {
            int rc = symba_recur(s, irecp);
            if (rc) return rc;
        }
        s->irec = ireci;
        symba_kick_list_plpl(s, dth, irecp, 1);
        symba_kick_list_pltp(s, dth, irecp, 1);
        if (ireci != 0) {
            symba_kick_list_plpl(s, dth, irecp, -1);
            symba_kick_list_pltp(s, dth, irecp, -1);
        }
        if (s->lclose) {
            int rc = symba_collisions(s, ireci, dtl);
            if (rc) return rc;
        }
        symba_set_recur_levels(s, ireci);
    }
    return 0;
}

/* symba_step_interp_system (symba_step.f90:55-115) */
static int symba_interp(orc_system *s, double dt) {
    double dth = 0.5 * dt;
    s->irec = -1;
    if (s->lfirst_pl) vh2vb_pl(s);
    lindrift_pl(s, dth, 1);
    kick_vb_pl(s, dth, 1);
    drift_pl(s, dt);
    if (s->ntp > 0) {
        if (s->lfirst_tp) {
            double vbcb[3] = {-s->ptbeg[0], -s->ptbeg[1], -s->ptbeg[2]};
            vh2vb_tp(s, vbcb);
        }
        lindrift_tp(s, dth, 1);
        kick_vb_tp(s, dth, 1);
        drift_tp(s, dt);
    }
    int rc = symba_recur(s, 0);
    if (rc) return rc;
    s->irec = -1;
    kick_vb_pl(s, dth, 0);
    lindrift_pl(s, dth, 0);
    vb2vh_pl(s);
    if (s->ntp > 0) {
        kick_vb_tp(s, dth, 0);
        lindrift_tp(s, dth, 0);
        double vbcb[3] = {-s->ptend[0], -s->ptend[1], -s->ptend[2]};
        vb2vh_tp(s, vbcb);
    }
    return 0;
}

/* symba_step_system (symba_step.f90:14-52).  Both encounter checks are
 * evaluated (the reference's `.or.` of two impure functions). */
static int symba_step(orc_system *s, double dt) {
    symba_reset(s);
    int a = symba_encounter_check_pl(s, dt, 0);
    int b = symba_encounter_check_tp(s, dt, 0);
    /* keep a copy of the level-0 lists for inspection */
    free(s->last_plpl);
    free(s->last_pltp);
    s->last_plpl_n = s->plpl.n;
    s->last_pltp_n = s->pltp.n;
    s->last_plpl = malloc(sizeof(int32_t) * 2 * (s->plpl.n + 1));
    s->last_pltp = malloc(sizeof(int32_t) * 2 * (s->pltp.n + 1));
    for (int64_t k = 0; k < s->plpl.n; k++) {
        s->last_plpl[2 * k] = s->plpl.i1[k];
        s->last_plpl[2 * k + 1] = s->plpl.i2[k];
    }
    for (int64_t k = 0; k < s->pltp.n; k++) {
        s->last_pltp[2 * k] = s->pltp.i1[k];
        s->last_pltp[2 * k + 1] = s->pltp.i2[k];
    }
    s->stats[2] += s->plpl.n;
    s->stats[3] += s->pltp.n;
    int rc = 0;
    if (a || b) {
        s->stats[0]++;
        rc = symba_interp(s, dt);
    } else {
        s->irec = -1;
        helio_step(s, dt);
    }
    s->lfirstkick = s->lfirst_pl;
    return rc;
}

int orc_system_initialize(orc_system *s) {
    for (int32_t i = 0; i < s->npl; i++) {
        s->status[i] = ST_ACTIVE;
        s->lmask[i] = 1;
        s->mu[i] = s->GMcb + s->Gmass[i];
    }
    for (int32_t i = 0; i < s->ntp; i++) {
        s->tstatus[i] = ST_ACTIVE;
        s->tlmask[i] = 1;
        s->tmu[i] = s->GMcb;
    }
    s->nplm = s->npl;
    if (s->gmtiny > 0.0) {
        int32_t m = 0;
        for (int32_t i = 0; i < s->npl; i++) m += !(s->Gmass[i] < s->gmtiny);
        s->nplm = m;
    }
    if (s->integrator == ORC_WHM) {
        /* whm_util_set_mu_eta_pl (whm_util.f90:175-198) */
        if (s->npl > 0) {
            s->eta[0] = s->GMcb + s->Gmass[0];
            s->muj[0] = s->eta[0];
            for (int32_t i = 1; i < s->npl; i++) {
                s->eta[i] = s->eta[i - 1] + s->Gmass[i];
                s->muj[i] = s->GMcb * s->eta[i] / s->eta[i - 1];
            }
        }
    } else {
        /* helio_util_setup_initialize_system (helio_util.f90:14-43): vh2vb, tp h2b */
        vh2vb_pl(s);
        for (int32_t i = 0; i < s->ntp; i++)
            for (int d = 0; d < 3; d++) s->tvb[3 * i + d] = s->tvh[3 * i + d] + s->cb_vb[d];
        for (int32_t i = 0; i < s->npl; i++) s->mu[i] = s->GMcb; /* helio_drift_body uses mu = GMcb */
    }
    /* flatten */
    free(s->k_plpl);
    s->k_plpl = NULL;
    s->nplpl = 0;
    if (s->loop_mode == 1 && s->npl > 1) {
        int32_t nplm = s->integrator == ORC_SYMBA ? s->nplm : s->npl;
        s->nplpl = orc_util_flatten_eucl_plpl(s->npl, s->npl, NULL);
        s->k_plpl = malloc(sizeof(int32_t) * 2 * s->nplpl);
        orc_util_flatten_eucl_plpl(s->npl, s->npl, s->k_plpl);
        (void)nplm;
    }
    s->lfirst_pl = s->lfirst_tp = s->lfirstkick = 1;
    s->irec = -1;
    return 0;
}

/* swiftest_discard_pl_close (src/swiftest/swiftest_discard.f90:293-336) */
static int discard_pl_close(const double *dx, const double *dv, double dt, double r2crit) {
    double r2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
    if (r2 <= r2crit) return 1;
    double vdotr = dx[0] * dv[0] + dx[1] * dv[1] + dx[2] * dv[2];
    if (vdotr > 0.0) return 0;
    double v2 = dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2];
    double tmin = -vdotr / v2;
    double r2min;
    if (tmin < dt)
        r2min = r2 - vdotr * vdotr / v2;
    else
        r2min = r2 + 2.0 * vdotr * dt + v2 * (dt * dt);
    r2min = r2min < r2 ? r2min : r2;
    return r2min <= r2crit;
}

/* swiftest_discard_pl_tp (src/swiftest/swiftest_discard.f90:244-290), the discard step of the
 * reference's main loop (swiftest_driver) after each step when param%lclose: an ACTIVE tp that comes within a pl's radius
 * leaves the system (the reference spills it out of its arrays; here it stays in its slot
 * with status INACTIVE, masked, parked with no velocity at 1e6 AU + (npl + its index)). */
static void discard_pl_tp(orc_system *s) {
    for (int32_t i = 0; i < s->ntp; i++) {
        if (s->tstatus[i] != ST_ACTIVE) continue;
        for (int32_t j = 0; j < s->npl; j++) {
            double dx[3], dv[3];
            for (int d = 0; d < 3; d++) {
                dx[d] = s->trh[3 * i + d] - s->rh[3 * j + d];
                dv[d] = s->tvh[3 * i + d] - s->vh[3 * j + d];
            }
            if (!discard_pl_close(dx, dv, s->dt, s->radius[j] * s->radius[j])) continue;
            s->tstatus[i] = ST_INACTIVE;
            s->tlmask[i] = 0;
            s->trh[3 * i] = 1.0e6 + (double)((int64_t)s->npl + i);
            s->trh[3 * i + 1] = s->trh[3 * i + 2] = 0.0;
            for (int d = 0; d < 3; d++) s->tvh[3 * i + d] = s->tvb[3 * i + d] = 0.0;
            s->stats[4]++;
            break;
        }
    }
}

int orc_system_step(orc_system *s, int32_t nsteps) {
    for (int32_t n = 0; n < nsteps; n++) {
        int rc = 0;
        if (s->integrator == ORC_WHM)
            rc = whm_step(s, s->dt);
        else if (s->integrator == ORC_HELIO) {
            helio_step(s, s->dt);
        } else
            rc = symba_step(s, s->dt);
        if (rc) return rc;
        if (s->lclose && s->npl > 0 && s->ntp > 0) discard_pl_tp(s);
        s->t += s->dt;
    }
    return 0;
}

void orc_system_get_pl(const orc_system *s, double *rh, double *vh, int32_t *status) {
    if (rh) memcpy(rh, s->rh, sizeof(double) * 3 * s->npl);
    if (vh) memcpy(vh, s->vh, sizeof(double) * 3 * s->npl);
    if (status) memcpy(status, s->status, sizeof(int32_t) * s->npl);
}
void orc_system_get_tp(const orc_system *s, double *rh, double *vh, int32_t *status) {
    if (rh) memcpy(rh, s->trh, sizeof(double) * 3 * s->ntp);
    if (vh) memcpy(vh, s->tvh, sizeof(double) * 3 * s->ntp);
    if (status) memcpy(status, s->tstatus, sizeof(int32_t) * s->ntp);
}
void orc_system_stats(const orc_system *s, int64_t *out) { memcpy(out, s->stats, sizeof(s->stats)); }
void orc_system_collision_terms(const orc_system *s, double *out) {
    out[0] = s->E_collisions;
    for (int d = 0; d < 3; d++) out[1 + d] = s->L_escape[d];
}
int64_t orc_system_plpl_list(const orc_system *s, int64_t cap, int32_t *i1, int32_t *i2) {
    for (int64_t k = 0; k < s->last_plpl_n && k < cap; k++) {
        i1[k] = s->last_plpl[2 * k];
        i2[k] = s->last_plpl[2 * k + 1];
    }
    return s->last_plpl_n;
}
int64_t orc_system_pltp_list(const orc_system *s, int64_t cap, int32_t *i1, int32_t *i2) {
    for (int64_t k = 0; k < s->last_pltp_n && k < cap; k++) {
        i1[k] = s->last_pltp[2 * k];
        i2[k] = s->last_pltp[2 * k + 1];
    }
    return s->last_pltp_n;
}

/* swiftest_util_get_energy_and_momentum_system (swiftest_util.f90:1172-1291) with the
 * triangular potential energy (:1350-1401).  Masses are taken as G*m (GU = 1), which
 * scales every energy term by the same factor and leaves relative errors unchanged. */
void orc_system_energy(orc_system *s, double *out) {
    int32_t n = s->npl;
    double *rb = calloc((size_t)3 * (n > 0 ? n : 1), 8);
    double *vb = calloc((size_t)3 * (n > 0 ? n : 1), 8);
    /* bring velocities to barycentric from heliocentric, positions via rh2rb */
    if (s->integrator == ORC_WHM) {
        /* WHM keeps heliocentric velocities; barycentric via vh2vb */
        double Gmtot = s->GMcb, cbvb[3] = {0, 0, 0};
        double sum = 0.0;
        for (int32_t i = 0; i < n; i++) sum = sum + s->Gmass[i];
        Gmtot = s->GMcb + sum;
        for (int32_t i = 0; i < n; i++)
            for (int d = 0; d < 3; d++) cbvb[d] = cbvb[d] - s->Gmass[i] * s->vh[3 * i + d];
        for (int d = 0; d < 3; d++) s->cb_vb[d] = cbvb[d] / Gmtot;
        for (int32_t i = 0; i < n; i++)
            for (int d = 0; d < 3; d++) vb[3 * i + d] = s->vh[3 * i + d] + s->cb_vb[d];
    } else {
        memcpy(vb, s->vb, sizeof(double) * 3 * n);
    }
    rh2rb_pl(s, rb);
    double GMtot = s->GMcb;
    {
        double sum = 0.0;
        for (int32_t i = 0; i < n; i++)
            if (s->status[i] != ST_INACTIVE) sum = sum + s->Gmass[i];
        GMtot = s->GMcb + sum;
    }
    double mcb = s->GMcb;
    double kecb = mcb * (s->cb_vb[0] * s->cb_vb[0] + s->cb_vb[1] * s->cb_vb[1] + s->cb_vb[2] * s->cb_vb[2]);
    double be_cb = -3.0 * s->GMcb * mcb / (5.0 * s->Rcb);
    double Lcb[3] = {mcb * (s->cb_rb[1] * s->cb_vb[2] - s->cb_rb[2] * s->cb_vb[1]),
                     mcb * (s->cb_rb[2] * s->cb_vb[0] - s->cb_rb[0] * s->cb_vb[2]),
                     mcb * (s->cb_rb[0] * s->cb_vb[1] - s->cb_rb[1] * s->cb_vb[0])};
    double kesum = 0.0, L[3] = {0, 0, 0};
    for (int32_t i = 0; i < n; i++) {
        if (s->status[i] == ST_INACTIVE) continue;
        const double *r = &rb[3 * i], *v = &vb[3 * i];
        double h0 = r[1] * v[2] - r[2] * v[1];
        double h1 = r[2] * v[0] - r[0] * v[2];
        double h2 = r[0] * v[1] - r[1] * v[0];
        double m = s->Gmass[i];
        L[0] = L[0] + m * h0;
        L[1] = L[1] + m * h1;
        L[2] = L[2] + m * h2;
        kesum = kesum + m * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    }
    double pe = 0.0;
    for (int32_t i = 0; i < n; i++) {
        if (s->status[i] == ST_INACTIVE) continue;
        double row = 0.0;
        for (int32_t j = i + 1; j < n; j++) {
            if (s->status[j] == ST_INACTIVE) continue;
            double d[3] = {rb[3 * i] - rb[3 * j], rb[3 * i + 1] - rb[3 * j + 1], rb[3 * i + 2] - rb[3 * j + 2]};
            row = row + (-(s->Gmass[i] * s->Gmass[j]) / norm2_3(d));
        }
        pe = pe + row;
    }
    double pecb = 0.0, pecb_h = 0.0;
    for (int32_t i = 0; i < n; i++)
        if (s->status[i] != ST_INACTIVE) {
            pecb = pecb + (-s->GMcb * s->Gmass[i] / norm2_3(&rb[3 * i]));
            pecb_h = pecb_h + (-s->GMcb * s->Gmass[i] / norm2_3(&s->rh[3 * i]));
        }
    const double pe_pairs = pe;
    pe = pe + pecb;
    double ke = 0.5 * (kecb + kesum);
    double be = 0.0;
    if (s->lclose)
        for (int32_t i = 0; i < n; i++)
            if (s->status[i] != ST_INACTIVE) be = be + (-3.0 * s->Gmass[i] * s->Gmass[i] / (5.0 * s->radius[i]));
    (void)be_cb;
    out[0] = ke + pe + be;
    out[1] = ke;
    out[2] = pe;
    out[3] = be;
    out[4] = Lcb[0] + L[0];
    out[5] = Lcb[1] + L[1];
    out[6] = Lcb[2] + L[2];
    out[7] = GMtot;
    /* same total with the central-body term taken at the heliocentric distance */
    out[8] = ke + (pe_pairs + pecb_h) + be;
    free(rb);
    free(vb);
}
