// drift_impl.cuh -- device functions of the Danby drift (shared by drift.cu and the
// SyMBA recursion kernel in system.cu).  See drift.cu for the reference citations.
#pragma once
#include <cuda_runtime.h>

#include "swg_internal.cuh"

namespace swg {

__device__ constexpr double E2MAX = 0.36;
__device__ constexpr double DM2MAX = 0.16;
__device__ constexpr double E2DM2MAX = 0.0016;
__device__ constexpr double DANBYB = 1.0e-13;
constexpr int NLAG1 = 50;
constexpr int NLAG2 = 40;

__device__ __forceinline__ void d_scget(double angle, double &sx, double &cx) {
    const int nper = (int)(angle / TWOPI);
    double x = angle - nper * TWOPI;
    if (x < 0.0) x = x + TWOPI;
    sx = sin(x);
    cx = sqrt(1.0 - sx * sx);
    if ((x > PIBY2) && (x < PI3BY2)) cx = -cx;
}

__device__ __forceinline__ void d_stumpff(double x, double &c0, double &c1, double &c2, double &c3) {
    int n = 0;
    while (fabs(x) >= 0.1 && n < 1100) {  // cap only binds for x = inf (finite x needs <= 520)
        n = n + 1;
        x = x / 4.0;
    }
    c2 = (1.0 - x * (1.0 - x * (1.0 - x * (1.0 - x * (1.0 - x * (1.0 - x / 182.0) / 132.0) / 90.0) / 56.0) / 30.0) /
                    12.0) /
         2.0;
    c3 = (1.0 - x * (1.0 - x * (1.0 - x * (1.0 - x * (1.0 - x * (1.0 - x / 210.0) / 156.0) / 110.0) / 72.0) / 42.0) /
                    20.0) /
         6.0;
    c1 = 1.0 - x * c3;
    c0 = 1.0 - x * c2;
    for (int i = n; i >= 1; i--) {
        c3 = (c2 + c0 * c3) / 4.0;
        c2 = c1 * c1 / 2.0;
        c1 = c0 * c1;
        c0 = 2.0 * c0 * c0 - 1.0;
    }
}

__device__ inline void d_kepmd(double dm, double es, double ec, double &x, double &s, double &c) {
    const double a0 = 39916800.0, a1 = 6652800.0, a2 = 332640.0, a3 = 7920.0, a4 = 110.0;
    const double fac1 = 1.0 / (1.0 - ec);
    const double q = fac1 * dm;
    const double fac2 = es * es * fac1 - ec / 3.0;
    double xx = q * (1.0 - 0.5 * fac1 * q * (es - q * fac2));
    double y = xx * xx;
    double ss = xx * (a0 - y * (a1 - y * (a2 - y * (a3 - y * (a4 - y))))) / a0;
    double cc = sqrt(1.0 - ss * ss);
    const double f = xx - ec * ss + es * (1.0 - cc) - dm;
    const double fp = 1.0 - ec * cc + es * ss;
    const double fpp = ec * ss + es * cc;
    const double fppp = ec * cc - es * ss;
    double dx = -(f / fp);
    dx = -(f / (fp + dx * fpp / 2.0));
    dx = -(f / (fp + dx * fpp / 2.0 + dx * dx * fppp * SIXTH));
    xx = xx + dx;
    y = xx * xx;
    ss = xx * (a0 - y * (a1 - y * (a2 - y * (a3 - y * (a4 - y))))) / a0;
    cc = sqrt(1.0 - ss * ss);
    x = xx;
    s = ss;
    c = cc;
}

__device__ inline void d_p3solve(double dt, double r0, double mu, double alpha, double u, double &s, int &iflag) {
    const double denom = (mu - alpha * r0) * SIXTH;
    const double a2 = 0.5 * u / denom;
    const double a1 = r0 / denom;
    const double a0 = -(dt / denom);
    const double q = (a1 - a2 * a2 * THIRD) * THIRD;
    const double r = (a1 * a2 - 3.0 * a0) * SIXTH - (a2 * a2 * a2) / 27.0;
    const double sq2 = q * q * q + r * r;
    if (sq2 >= 0.0) {
        const double sq = sqrt(sq2);
        double p1, p2;
        if ((r + sq) <= 0.0)
            p1 = -pow(-(r + sq), THIRD);
        else
            p1 = pow(r + sq, THIRD);
        if ((r - sq) <= 0.0)
            p2 = -pow(-(r - sq), THIRD);
        else
            p2 = pow(r - sq, THIRD);
        iflag = 0;
        s = p1 + p2 - a2 * THIRD;
    } else {
        iflag = 1;
        s = 0.0;
    }
}

__device__ inline void d_kepu_guess(double dt, double r0, double mu, double alpha, double u, double &s) {
    const double thresh = 0.4, danbyk = 0.85;
    if (alpha > 0.0) {
        if (dt / r0 <= thresh) {
            s = dt / r0 - (dt * dt * u) / (2.0 * r0 * r0 * r0);
        } else {
            const double a = mu / alpha;
            const double en = sqrt(mu / (a * a * a));
            const double ec = 1.0 - r0 / a;
            const double es = u / (en * a * a);
            const double e = sqrt(ec * ec + es * es);
            const double y = en * dt - es;
            double sy, cy;
            d_scget(y, sy, cy);
            const double sigma = copysign(1.0, es * cy + ec * sy);
            const double x = y + sigma * danbyk * e;
            s = x / sqrt(alpha);
        }
    } else {
        int iflag;
        d_p3solve(dt, r0, mu, alpha, u, s, iflag);
        if (iflag != 0) s = dt / r0;
    }
}

__device__ inline void d_kepu_fchk(double dt, double r0, double mu, double alpha, double u, double s, double &f) {
    const double x = (s * s) * alpha;
    double c0, c1, c2, c3;
    d_stumpff(x, c0, c1, c2, c3);
    c1 = c1 * s;
    c2 = c2 * (s * s);
    c3 = c3 * (s * s * s);
    f = r0 * c1 + u * c2 + mu * c3 - dt;
}

__device__ inline void d_kepu_new(double &s, double dt, double r0, double mu, double alpha, double u, double &fp,
                           double &c1, double &c2, double &c3, int &iflag) {
    for (int nc = 0; nc <= 6; nc++) {
        const double x = s * s * alpha;
        double c0;
        d_stumpff(x, c0, c1, c2, c3);
        c1 = c1 * s;
        c2 = c2 * s * s;
        c3 = c3 * s * s * s;
        const double f = r0 * c1 + u * c2 + mu * c3 - dt;
        fp = r0 * c0 + u * c1 + mu * c2;
        const double fpp = (-(r0 * alpha) + mu) * c1 + u * c0;
        const double fppp = (-(r0 * alpha) + mu) * c0 - u * alpha * c1;
        double ds = -(f / fp);
        ds = -(f / (fp + ds * fpp / 2.0));
        ds = -(f / (fp + ds * fpp / 2.0 + ds * ds * fppp / 6.0));
        s = s + ds;
        const double fdt = f / dt;
        if (fdt * fdt < DANBYB * DANBYB) {
            iflag = 0;
            return;
        }
    }
    iflag = 1;
}

__device__ inline void d_kepu_lag(double &s, double dt, double r0, double mu, double alpha, double u, double &fp,
                           double &c1, double &c2, double &c3, int &iflag) {
    const int ln = 5;
    const int ncmax = (alpha < 0.0) ? NLAG2 : NLAG1;
    for (int nc = 0; nc <= ncmax; nc++) {
        const double x = s * s * alpha;
        double c0;
        d_stumpff(x, c0, c1, c2, c3);
        c1 = c1 * s;
        c2 = c2 * s * s;
        c3 = c3 * s * s * s;
        const double f = r0 * c1 + u * c2 + mu * c3 - dt;
        fp = r0 * c0 + u * c1 + mu * c2;
        const double fpp = (-(r0 * alpha) + mu) * c1 + u * c0;
        const double lnm1 = (double)ln - 1.0;
        const double disc = fabs(lnm1 * lnm1 * fp * fp - lnm1 * (double)ln * f * fpp);
        const double ds = -((double)ln * f / (fp + copysign(1.0, fp) * sqrt(disc)));
        s = s + ds;
        const double fdt = f / dt;
        if (fdt * fdt < DANBYB * DANBYB) {
            iflag = 0;
            return;
        }
    }
    iflag = 2;
}

__device__ inline void d_kepu(double dt, double r0, double mu, double alpha, double u, double &fp, double &c1, double &c2,
                       double &c3, int &iflag) {
    double s;
    d_kepu_guess(dt, r0, mu, alpha, u, s);
    const double st = s;
    d_kepu_new(s, dt, r0, mu, alpha, u, fp, c1, c2, c3, iflag);
    if (iflag != 0) {
        double fo, fn;
        d_kepu_fchk(dt, r0, mu, alpha, u, st, fo);
        d_kepu_fchk(dt, r0, mu, alpha, u, s, fn);
        if (fabs(fo) < fabs(fn)) s = st;
        d_kepu_lag(s, dt, r0, mu, alpha, u, fp, c1, c2, c3, iflag);
    }
}

__device__ inline void d_drift_dan(double mu, double &rx0, double &ry0, double &rz0, double &vx0, double &vy0, double &vz0,
                            double dt0, int &iflag) {
    double dt = dt0;
    iflag = 0;
    const double r0 = sqrt(rx0 * rx0 + ry0 * ry0 + rz0 * rz0);
    const double v0s = vx0 * vx0 + vy0 * vy0 + vz0 * vz0;
    const double u = rx0 * vx0 + ry0 * vy0 + rz0 * vz0;
    const double alpha = 2.0 * mu / r0 - v0s;
    if (alpha > 0.0) {
        const double a = mu / alpha;
        const double asq = a * a;
        const double en = sqrt(mu / (a * asq));
        const double ec = 1.0 - r0 / a;
        const double es = u / (en * asq);
        const double esq = ec * ec + es * es;
        const double dm = dt * en - (double)(int)(dt * en / TWOPI) * TWOPI;
        dt = dm / en;
        if ((esq < E2MAX) && (dm * dm < DM2MAX) && (esq * (dm * dm) < E2DM2MAX)) {
            double xkep, s, c;
            d_kepmd(dm, es, ec, xkep, s, c);
            const double fchk = (xkep - ec * s + es * (1.0 - c) - dm);
            if (fchk * fchk > DANBYB * DANBYB) {
                iflag = 1;
                return;
            }
            const double fp = 1.0 - ec * c + es * s;
            const double f = a / r0 * (c - 1.0) + 1.0;
            const double g = dt + (s - xkep) / en;
            const double fdot = -(a / (r0 * fp) * en * s);
            const double gdot = (c - 1.0) / fp + 1.0;
            const double rx = rx0 * f + vx0 * g;
            const double ry = ry0 * f + vy0 * g;
            const double rz = rz0 * f + vz0 * g;
            const double vx = rx0 * fdot + vx0 * gdot;
            const double vy = ry0 * fdot + vy0 * gdot;
            const double vz = rz0 * fdot + vz0 * gdot;
            rx0 = rx;
            ry0 = ry;
            rz0 = rz;
            vx0 = vx;
            vy0 = vy;
            vz0 = vz;
            iflag = 0;
            return;
        }
    }
    double fp, c1, c2, c3;
    d_kepu(dt, r0, mu, alpha, u, fp, c1, c2, c3, iflag);
    if (iflag == 0) {
        const double f = 1.0 - mu / r0 * c2;
        const double g = dt - mu * c3;
        const double fdot = -(mu / (fp * r0) * c1);
        const double gdot = 1.0 - mu / fp * c2;
        const double rx = rx0 * f + vx0 * g;
        const double ry = ry0 * f + vy0 * g;
        const double rz = rz0 * f + vz0 * g;
        const double vx = rx0 * fdot + vx0 * gdot;
        const double vy = ry0 * fdot + vy0 * gdot;
        const double vz = rz0 * fdot + vz0 * gdot;
        rx0 = rx;
        ry0 = ry;
        rz0 = rz;
        vx0 = vx;
        vy0 = vy;
        vz0 = vz;
    }
}

__device__ inline int d_drift_one(double mu, double &rx, double &ry, double &rz, double &vx, double &vy, double &vz,
                           double dt) {
    int iflag;
    d_drift_dan(mu, rx, ry, rz, vx, vy, vz, dt, iflag);
    if (iflag != 0) {
        const double dttmp = 0.1 * dt;
        for (int i = 1; i <= 10; i++) {
            d_drift_dan(mu, rx, ry, rz, vx, vy, vz, dttmp, iflag);
            if (iflag != 0) break;
        }
    }
    return iflag;
}

// ------------------------------------------------------------------ fast FP64 form
// The same Danby drift for the mixed-precision path.  Where the reference divides by the
// same quantity several times (r0, mu, alpha, en, fp) the fast form takes one reciprocal (or
// reciprocal square root) and multiplies, contracts products into FMAs, and folds the
// constant divisors; on GB300 each FP64 divide or square root is a multi-instruction
// sequence on the narrow FP64 pipe.  The elliptic small-step branch solves Kepler's
// difference equation (d_kepmd_fast) in FP32 and polishes the root with one FP64 Newton
// step.  Results agree with the reference form to a few units in the last place; the
// universal-variable branch (large steps or eccentric orbits) is the reference form
// unchanged.
//
// Kepler's difference equation f(x) = x - ec sin x + es (1 - cos x) - dm = 0 (the
// reference's _kepmd, swiftest_drift.f90:234-276): the reference's series guess and its
// three corrections of increasing order run in FP32, which leaves x within a few FP32 ulps
// of the root (|dx| below ~3e-7 over the branch: |dm| < 0.4, e < 0.6, f' >= 1 - e); one
// Halley step in FP64, dx = -2 f f' / (2 f'^2 - f f''), then leaves an error of order dx^3,
// below FP64 resolution.  sin and cos are formed once in FP64 at the FP32 root (the
// reference's degree-11 sine polynomial, cos from sqrt(1 - sin^2)) and carried to the
// polished root by their Taylor expansion to second order in dx.
__device__ inline void d_kepmd_fast(double dm, double es, double ec, double &x, double &s, double &c) {
    const double a0 = 39916800.0, a1 = 6652800.0, a2 = 332640.0, a3 = 7920.0, a4 = 110.0;
    const double inv_a0 = 1.0 / 39916800.0;
    // FP32 root: sin x as its Taylor series to x^11 in nested form
    const float dmf = (float)dm, esf = (float)es, ecf = (float)ec;
    const float fac1 = 1.0f / (1.0f - ecf);
    const float q = fac1 * dmf;
    const float fac2 = fmaf(esf * esf, fac1, -ecf * (1.0f / 3.0f));
    float xf = q * (1.0f - 0.5f * fac1 * q * fmaf(-q, fac2, esf));
    {
        const float yf = xf * xf;
        const float sf = xf * fmaf(-yf * (1.0f / 6.0f),
                                   fmaf(-yf * (1.0f / 20.0f),
                                        fmaf(-yf * (1.0f / 42.0f),
                                             fmaf(-yf * (1.0f / 72.0f), fmaf(-yf, 1.0f / 110.0f, 1.0f), 1.0f), 1.0f),
                                        1.0f),
                                   1.0f);
        const float cf = sqrtf(fmaf(-sf, sf, 1.0f));
        const float f = fmaf(esf, 1.0f - cf, fmaf(-ecf, sf, xf)) - dmf;
        const float fp = fmaf(esf, sf, fmaf(-ecf, cf, 1.0f));
        const float fpp = fmaf(ecf, sf, esf * cf);
        const float fppp = fmaf(ecf, cf, -esf * sf);
        float dx = -(f / fp);
        dx = -(f / fmaf(dx * fpp, 0.5f, fp));
        dx = -(f / fmaf(dx * dx * fppp, 1.0f / 6.0f, fmaf(dx * fpp, 0.5f, fp)));
        xf += dx;
    }
    // FP64 Halley step at the FP32 root
    const double xx = (double)xf;
    const double y = xx * xx;
    const double ss = xx * fma(-y, fma(-y, fma(-y, fma(-y, a4 - y, a3), a2), a1), a0) * inv_a0;
    const double cc = sqrt(fma(-ss, ss, 1.0));
    const double f = fma(es, 1.0 - cc, fma(-ec, ss, xx)) - dm;
    const double fp = fma(es, ss, fma(-ec, cc, 1.0));
    const double fpp = fma(ec, ss, es * cc);
    const double dx = -(2.0 * f * fp) / fma(2.0 * fp, fp, -f * fpp);
    x = xx + dx;
    s = fma(dx, fma(-0.5 * ss, dx, cc), ss);  // sin(x + dx) = s + c dx - s dx^2 / 2
    c = fma(dx, fma(-0.5 * cc, dx, -ss), cc);  // cos(x + dx) = c - s dx - c dx^2 / 2
}

// inv_mu: 1/mu when the caller has it (the same value, formed once), else 0
__device__ inline void d_drift_dan_fast(double mu, double &rx0, double &ry0, double &rz0, double &vx0, double &vy0,
                                        double &vz0, double dt0, int &iflag, double inv_mu0 = 0.0) {
    iflag = 0;
    const double r2 = fma(rz0, rz0, fma(ry0, ry0, rx0 * rx0));
    const double inv_r0 = rsqrt(r2);
    const double v0s = fma(vz0, vz0, fma(vy0, vy0, vx0 * vx0));
    const double u = fma(rz0, vz0, fma(ry0, vy0, rx0 * vx0));
    const double alpha = fma(2.0 * mu, inv_r0, -v0s);
    if (alpha > 0.0) {
        const double inv_mu = inv_mu0 != 0.0 ? inv_mu0 : 1.0 / mu;
        const double rsa = rsqrt(alpha);
        const double a = mu * rsa * rsa;                 // mu / alpha
        const double ia = alpha * inv_mu;                // 1 / a
        const double en = alpha * (alpha * rsa) * inv_mu;  // sqrt(mu / a^3)
        const double inv_en = mu * (rsa * rsa * rsa);
        const double ec = fma(-(r2 * inv_r0), ia, 1.0);
        const double es = u * inv_en * ia * ia;
        const double esq = fma(ec, ec, es * es);
        const double den = dt0 * en;
        const double dm = fma(-(double)(int)(den * (1.0 / TWOPI)), TWOPI, den);
        if ((esq < E2MAX) && (dm * dm < DM2MAX) && (esq * (dm * dm) < E2DM2MAX)) {
            const double dt = dm * inv_en;
            double xkep, s, c;
            d_kepmd_fast(dm, es, ec, xkep, s, c);
            const double fchk = fma(es, 1.0 - c, fma(-ec, s, xkep)) - dm;
            if (fchk * fchk > DANBYB * DANBYB) {
                iflag = 1;
                return;
            }
            const double fp = fma(es, s, fma(-ec, c, 1.0));
            const double inv_fp = 1.0 / fp;
            const double ar = a * inv_r0;
            const double f = fma(ar, c - 1.0, 1.0);
            const double g = fma(s - xkep, inv_en, dt);
            const double fdot = -(ar * inv_fp * en * s);
            const double gdot = fma(c - 1.0, inv_fp, 1.0);
            const double rx = fma(rx0, f, vx0 * g), ry = fma(ry0, f, vy0 * g), rz = fma(rz0, f, vz0 * g);
            const double vx = fma(rx0, fdot, vx0 * gdot), vy = fma(ry0, fdot, vy0 * gdot),
                         vz = fma(rz0, fdot, vz0 * gdot);
            rx0 = rx;
            ry0 = ry;
            rz0 = rz;
            vx0 = vx;
            vy0 = vy;
            vz0 = vz;
            return;
        }
    }
    d_drift_dan(mu, rx0, ry0, rz0, vx0, vy0, vz0, dt0, iflag);  // universal variables: the reference form
}

__device__ inline int d_drift_one_fast(double mu, double &rx, double &ry, double &rz, double &vx, double &vy,
                                       double &vz, double dt, double inv_mu = 0.0) {
    int iflag;
    d_drift_dan_fast(mu, rx, ry, rz, vx, vy, vz, dt, iflag, inv_mu);
    if (iflag != 0) {
        const double dttmp = 0.1 * dt;
        for (int i = 1; i <= 10; i++) {
            d_drift_dan_fast(mu, rx, ry, rz, vx, vy, vz, dttmp, iflag, inv_mu);
            if (iflag != 0) break;
        }
    }
    return iflag;
}

}  // namespace swg
