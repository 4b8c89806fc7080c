// orbel.cu -- orbital elements <-> heliocentric Cartesian state, one thread per body.
//
// Restates swiftest_orbel_el2xv (src/swiftest/swiftest_orbel.f90:45-144) with its Kepler
// solvers (esolmd :241-280, ehie :283-343, eget :346-400, ehybrid :403-425, flon :199-265,
// fget :268-318, fhybrid :428-450, zget :321-357, scget :147-172, schget :199-207) and
// swiftest_orbel_xv2el (:913-1072), as the vectorised wrappers el2xv_vec (:14-42) and
// xv2el_vec (:876-910) call them: element i with mu(i) (the caller supplies mu = GMcb + Gm
// for massive bodies, GMcb for test particles, as set_mu does).  FP64 in the reference's
// operation order (this file is compiled with -fmad=false); the transcendental functions
// (sin, sinh, acos, atan2, log, pow ...) are CUDA's, which may differ from glibc's in the
// last bit.  Kept as in the reference: the first Halley correction of eget uses dx*2 where
// its second correction uses dx**2 (:377).
#include <cuda_runtime.h>

#include "swg_internal.cuh"

namespace swg {

namespace {

constexpr double TINYV = 4.0e-15;  // swiftest_orbel.f90:11
constexpr double PI = 3.141592653589793238462643383279502884197;
enum { ELLIPSE = -1, PARABOLA = 0, HYPERBOLA = 1 };

__device__ void o_scget(double angle, double &sx, double &cx) {
    const int nper = (int)(angle / TWOPI);
    double x = angle - nper * TWOPI;
    if (x < 0.0) x = x + TWOPI;
    sx = sin(x);
    cx = sqrt(1.0 - sx * sx);
    if ((x > PIBY2) && (x < PI3BY2)) cx = -cx;
}

__device__ void o_schget(double angle, double &shx, double &chx) {
    shx = sinh(angle);
    chx = sqrt(1.0 + shx * shx);
}

__device__ double o_flon(double e, double icapn) {
    const int IMAX = 10;
    const double a11 = 156.0, a9 = 17160.0, a7 = 1235520.0, a5 = 51891840.0, a3 = 1037836800.0;
    const double b11 = 11 * a11, b9 = 9 * a9, b7 = 7 * a7, b5 = 5 * a5, b3 = 3 * a3;
    int iflag = 0;
    double capn = icapn;
    if (icapn < 0.0) {
        iflag = 1;
        capn = -icapn;
    }
    const double a1 = 6227020800.0 * (1.0 - 1.0 / e);
    const double a0 = -6227020800.0 * capn / e;
    const double b1 = a1;
    const double a = 6 * (e - 1.0) / e;
    const double b = -6 * capn / e;
    const double sq = sqrt(0.25 * (b * b) + (a * a * a) / 27.0);
    const double biga = pow(-0.5 * b + sq, 1.0 / 3.0);
    const double bigb = -pow(+0.5 * b + sq, 1.0 / 3.0);
    double x = biga + bigb;
    double flon = x;
    if (capn >= TINYV) {
        for (int i = 1; i <= IMAX; i++) {
            const double x2 = x * x;
            const double f = a0 + x * (a1 + x2 * (a3 + x2 * (a5 + x2 * (a7 + x2 * (a9 + x2 * (a11 + x2))))));
            const double fp = b1 + x2 * (b3 + x2 * (b5 + x2 * (b7 + x2 * (b9 + x2 * (b11 + 13 * x2)))));
            const double dx = -f / fp;
            flon = x + dx;
            if (fabs(dx) <= TINYV) break;
            x = flon;
        }
    }
    if (iflag == 1) flon = -flon;
    return flon;
}

__device__ double o_fget(double e, double capn) {
    const int IMAX = 10;
    double x;
    if (capn < 0.0) {
        const double tmp = -2 * capn / e + 1.8;
        x = -log(tmp);
    } else {
        const double tmp = +2 * capn / e + 1.8;
        x = log(tmp);
    }
    double fget = x;
    for (int i = 1; i <= IMAX; i++) {
        double shx, chx;
        o_schget(x, shx, chx);
        const double esh = e * shx, ech = e * chx;
        const double f = esh - x - capn;
        const double fp = ech - 1.0;
        const double fpp = esh, fppp = ech;
        double dx = -f / fp;
        dx = -f / (fp + dx * fpp / 2.0);
        dx = -f / (fp + dx * fpp / 2.0 + (dx * dx) * fppp / 6.0);
        fget = x + dx;
        if (fabs(dx) <= TINYV) return fget;
        x = fget;
    }
    return fget;
}

__device__ double o_zget(double iq) {
    const double q = iq < 0.0 ? -iq : iq;
    double z;
    if (q < 1.0e-3) {
        z = q * (1.0 - ((q * q) / 3.0) * (1.0 - q * q));
    } else {
        const double x = 0.5 * (3 * q + sqrt(9 * (q * q) + 4.0));
        const double tmp = pow(x, 1.0 / 3.0);
        z = tmp - 1.0 / tmp;
    }
    return iq < 0.0 ? -z : z;
}

// The three-pass correction of esolmd / eget from x (reference_dx2: dx*2 in the third pass)
__device__ double o_esolve_pass(double e, double m, double x, bool reference_dx2) {
    double sx, cx;
    o_scget(x, sx, cx);
    const double es = e * sx, ec = e * cx;
    const double f = x - es - m;
    const double fp = 1.0 - ec;
    const double fpp = es, fppp = ec;
    double dx = -f / fp;
    dx = -f / (fp + dx * fpp / 2.0);
    const double d2 = reference_dx2 ? dx * 2 : dx * dx;
    dx = -f / (fp + dx * fpp / 2.0 + d2 * fppp / 6.0);
    return x + dx;
}

// series start of esolmd (1.5 sm**2) and eget (1.5 sm sm: another rounding)
__device__ double o_start(double e, double m, bool eget) {
    double sm, cm;
    o_scget(m, sm, cm);
    const double t = eget ? 1.5 * sm * sm : 1.5 * (sm * sm);
    return m + e * sm * (1.0 + e * (cm + e * (1.0 - t)));
}

__device__ double o_esolmd(double e, double m) { return o_esolve_pass(e, m, o_start(e, m, false), false); }

__device__ double o_eget(double e, double m) {
    const double x = o_esolve_pass(e, m, o_start(e, m, true), true);  // the reference's dx*2 (:377)
    return o_esolve_pass(e, m, x, false);
}

__device__ double o_ehie(double e, double im) {
    const int NMAX = 3;
    int iflag = 0;
    const int nper = (int)(im / TWOPI);
    double m = im - nper * TWOPI;
    if (m < 0.0) m = m + TWOPI;
    if (m > PI) {
        m = TWOPI - m;
        iflag = 1;
    }
    double x = pow(6 * m, 1.0 / 3.0) - m;
    for (int niter = 1; niter <= NMAX; niter++) {
        double sa, ca;
        o_scget(x + m, sa, ca);
        const double esa = e * sa, eca = e * ca;
        const double f = x - esa;
        const double fp = 1.0 - eca;
        double dx = -f / fp;
        dx = -f / (fp + 0.5 * dx * esa);
        dx = -f / (fp + 0.5 * dx * (esa + eca * dx / 3.0));
        x = x + dx;
    }
    double r = m + x;
    if (iflag == 1) r = TWOPI - r;
    return r;
}

__device__ double o_ehybrid(double e, double m) {
    if (e < 0.18) return o_esolmd(e, m);
    if (e <= 0.8) return o_eget(e, m);
    return o_ehie(e, m);
}

__device__ double o_fhybrid(double e, double n) {
    const double abn = n < 0.0 ? -n : n;
    if (abn < 0.636 * e - 0.6) return o_flon(e, n);
    return o_fget(e, n);
}

// swiftest_orbel_el2xv (:45-144)
__device__ void o_el2xv(double mu, double a, double ie, double inc, double capom, double omega, double capm,
                        double *r, double *v) {
    int type;
    double e = ie;
    if (ie < 0.0) {
        e = 0.0;
        type = ELLIPSE;
    } else {
        const double em1 = e - 1.0;
        if (fabs(em1) < TINYV)
            type = PARABOLA;
        else if (e > 1.0)
            type = HYPERBOLA;
        else
            type = ELLIPSE;
    }
    double sip, cip, so, co, si, ci;
    o_scget(omega, sip, cip);
    o_scget(capom, so, co);
    o_scget(inc, si, ci);
    const double d11 = cip * co - sip * so * ci, d12 = cip * so + sip * co * ci, d13 = sip * si;
    const double d21 = -sip * co - cip * so * ci, d22 = -sip * so + cip * co * ci, d23 = cip * si;
    double xfac1 = 0.0, xfac2 = 0.0, vfac1 = 0.0, vfac2 = 0.0;
    if (type == ELLIPSE) {
        const double cape = o_ehybrid(e, capm);
        double scap, ccap;
        o_scget(cape, scap, ccap);
        const double sqe = sqrt(1.0 - e * e);
        const double sqgma = sqrt(mu * a);
        xfac1 = a * (ccap - e);
        xfac2 = a * sqe * scap;
        const double ri = 1.0 / (a * (1.0 - e * ccap));
        vfac1 = -ri * sqgma * scap;
        vfac2 = ri * sqgma * sqe * ccap;
    }
    if (type == HYPERBOLA) {
        const double capf = o_fhybrid(e, capm);
        double shcap, chcap;
        o_schget(capf, shcap, chcap);
        const double sqe = sqrt(e * e - 1.0);
        const double sqgma = sqrt(mu * a);
        xfac1 = a * (e - chcap);
        xfac2 = a * sqe * shcap;
        const double ri = 1.0 / (a * (e * chcap - 1.0));
        vfac1 = -ri * sqgma * shcap;
        vfac2 = ri * sqgma * sqe * chcap;
    }
    if (type == PARABOLA) {
        const double zpara = o_zget(capm);
        const double sqgma = sqrt(2 * mu * a);
        xfac1 = a * (1.0 - zpara * zpara);
        xfac2 = 2 * a * zpara;
        const double ri = 1.0 / (a * (1.0 + zpara * zpara));
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

// Fortran SIGN(a, b) and MOD(a, p) for positive p
__device__ __forceinline__ double f_sign(double a, double b) { return copysign(fabs(a), b); }
__device__ __forceinline__ double f_mod(double a, double p) { return a - trunc(a / p) * p; }

// swiftest_orbel_xv2el (:913-1072); out: a, e, inc, capom, omega, capm, varpi, lam, f, cape, capf
__device__ void o_xv2el(double mu, const double *rv, const double *vv, double *out) {
    const double rx = rv[0], ry = rv[1], rz = rv[2], vx = vv[0], vy = vv[1], vz = vv[2];
    double a = 0.0, e = 0.0, inc = 0.0, capom = 0.0, omega = 0.0, capm = 0.0, varpi = 0.0, lam = 0.0, f = 0.0,
           cape = 0.0, capf = 0.0;
    double hx = ry * vz - rz * vy, hy = rz * vx - rx * vz, hz = rx * vy - ry * vx;
    const double h2 = hx * hx + hy * hy + hz * hz;
    double h = sqrt(h2);
    if (hz > h) {  // Hal's fix
        hz = h;
        hx = 0.0;
        hy = 0.0;
    }
    if (!(h2 <= 10 * 2.2250738585072014e-308)) {
        h = sqrt(h2);
        const double r = sqrt(rx * rx + ry * ry + rz * rz);
        const double v2 = vx * vx + vy * vy + vz * vz;
        const double rdotv = rx * vx + ry * vy + rz * vz;
        const double energy = 0.5 * v2 - mu / r;
        double fac = hz / h;
        if (fac < -1.0)
            inc = PI;
        else if (fac < 1.0)
            inc = acos(fac);
        fac = sqrt(hx * hx + hy * hy) / h;
        double u;
        if (fac * fac < TINYV) {
            u = atan2(ry, rx);
            if (hz < 0.0) u = -u;
        } else {
            capom = atan2(hx, -hy);
            u = atan2(rz / sin(inc), rx * cos(capom) + ry * sin(capom));
        }
        if (capom < 0.0) capom = capom + TWOPI;
        if (u < 0.0) u = u + TWOPI;
        int type;
        if (fabs(energy * r / mu) < sqrt(TINYV)) {
            type = PARABOLA;
        } else {
            a = -0.5 * mu / energy;
            if (a < 0.0) {
                fac = -h2 / (mu * a);
                type = fac > TINYV ? HYPERBOLA : PARABOLA;
            } else {
                type = ELLIPSE;
            }
        }
        double w = 0.0;
        if (type == ELLIPSE) {
            fac = 1.0 - h2 / (mu * a);
            if (fac > TINYV) {
                e = sqrt(fac);
                cape = 0.0;
                const double face = (a - r) / (a * e);
                if (face < -1.0)
                    cape = PI;
                else if (face < 1.0)
                    cape = acos(face);
                if (rdotv < 0.0) cape = TWOPI - cape;
                fac = 1.0 - e * cos(cape);
                const double cw = (cos(cape) - e) / fac;
                const double sw = sqrt(1.0 - e * e) * sin(cape) / fac;
                w = atan2(sw, cw);
                if (w < 0.0) w = w + TWOPI;
            } else {
                cape = u;
                w = u;
            }
            capm = cape - e * sin(cape);
        } else if (type == PARABOLA) {
            a = 0.5 * h2 / mu;
            e = 1.0;
            w = 0.0;
            fac = 2 * a / r - 1.0;
            if (fac < -1.0)
                w = PI;
            else if (fac < 1.0)
                w = acos(fac);
            if (rdotv < 0.0) w = TWOPI - w;
            const double tmpf = tan(0.5 * w);
            capm = tmpf * (1.0 + tmpf * tmpf / 3.0);
        } else {
            e = sqrt(1.0 + fac);
            const double tmpf = fmax((a - r) / (a * e), 1.0);
            capf = log(tmpf + sqrt(tmpf * tmpf - 1.0));
            if (rdotv < 0.0) capf = -capf;
            fac = e * cosh(capf) - 1.0;
            const double cw = (e - cosh(capf)) / fac;
            const double sw = sqrt(e * e - 1.0) * sinh(capf) / fac;
            w = atan2(sw, cw);
            if (w < 0.0) w = w + TWOPI;
            capm = e * sinh(capf) - capf;
        }
        omega = u - w;
        if (omega < 0.0) omega = omega + TWOPI;
        varpi = f_mod(omega + capom, TWOPI);
        lam = f_mod(capm + varpi, TWOPI);
        if (e > TINYV) {
            const double cf = 1.0 / e * (a * (1.0 - e * e) / r - 1.0);
            const double hr = h / r;
            const double rdot = f_sign(sqrt(fmax(v2 - hr * hr, 0.0)), rdotv);
            const double sf = a * (1.0 - e * e) / (h * e) * rdot;
            f = atan2(sf, cf);
            if (f < 0.0) f = f + TWOPI;
        } else {
            f = u;
        }
    }
    const double o[11] = {a, e, inc, capom, omega, capm, varpi, lam, f, cape, capf};
    for (int k = 0; k < 11; k++) out[k] = o[k];
}

__global__ void k_el2xv(int n, const double *__restrict__ mu, const double *__restrict__ a,
                        const double *__restrict__ e, const double *__restrict__ inc,
                        const double *__restrict__ capom, const double *__restrict__ omega,
                        const double *__restrict__ capm, double *__restrict__ rh, double *__restrict__ vh) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    o_el2xv(mu[i], a[i], e[i], inc[i], capom[i], omega[i], capm[i], rh + 3 * i, vh + 3 * i);
}

__global__ void k_xv2el(int n, const double *__restrict__ mu, const double *__restrict__ rh,
                        const double *__restrict__ vh, double *const *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double o[11];
    o_xv2el(mu[i], rh + 3 * i, vh + 3 * i, o);
    for (int k = 0; k < 11; k++)
        if (out[k]) out[k][i] = o[k];
}

}  // namespace

int orbel_el2xv_launch(swg_ctx *c, int32_t n, const double *mu, const double *a, const double *e,
                       const double *inc, const double *capom, const double *omega, const double *capm, double *rh,
                       double *vh) {
    if (n <= 0) return SWG_OK;
    k_el2xv<<<(n + 127) / 128, 128, 0, c->stream>>>(n, mu, a, e, inc, capom, omega, capm, rh, vh);
    c->launches++;
    return launch_status(c, "el2xv");
}

int orbel_xv2el_launch(swg_ctx *c, int32_t n, const double *mu, const double *rh, const double *vh,
                       double *const *out_dev) {
    if (n <= 0) return SWG_OK;
    k_xv2el<<<(n + 127) / 128, 128, 0, c->stream>>>(n, mu, rh, vh, out_dev);
    c->launches++;
    return launch_status(c, "xv2el");
}

}  // namespace swg
