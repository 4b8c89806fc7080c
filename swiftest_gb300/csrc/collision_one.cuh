// collision_one.cuh -- the pair test of the collision check and the potential term of the
// energy, shared by device kernels (symba_dev.cuh, collision.cu) and the host collision
// resolution (collision.cu), so both take the same operations (both are compiled without
// FMA contraction).
#pragma once
#include <cmath>

namespace swg {

// gfortran NORM2 of a 3-vector (the operators .mag. and .unit., and the potential's
// norm2(rb_i - rb_j)): scaled sum of squares
__host__ __device__ inline double hd_norm2_3(double x0, double x1, double x2) {
    double scale = 0.0, ssq = 1.0;
    const double v[3] = {x0, x1, x2};
    for (int k = 0; k < 3; k++) {
        if (v[k] != 0.0) {
            const double absx = fabs(v[k]);
            if (scale < absx) {
                const double q = scale / absx;
                ssq = 1.0 + ssq * q * q;
                scale = absx;
            } else {
                const double q = absx / scale;
                ssq = ssq + q * q;
            }
        }
    }
    return scale * sqrt(ssq);
}

// One term of the pairwise potential (swiftest_util.f90:1385): -(Gm_i Gm_j) / |rb_i - rb_j|
__host__ __device__ inline double hd_pot_term(const double *ri, const double *rj, double Gmi, double Gmj) {
    return -(Gmi * Gmj) / hd_norm2_3(ri[0] - rj[0], ri[1] - rj[1], ri[2] - rj[2]);
}

// swiftest_orbel_xv2aeq (src/swiftest/swiftest_orbel.f90:700-764): semimajor axis,
// eccentricity and pericentre distance of the relative two-body orbit.
__host__ __device__ inline void d_xv2aeq(double mu, double rx, double ry, double rz, double vx, double vy, double vz,
                                         double &a, double &e, double &q) {
    const double TINYV = 4.0e-15;  // swiftest_orbel.f90:11
    a = 0.0;
    e = 0.0;
    q = 0.0;
    const double r = sqrt(rx * rx + ry * ry + rz * rz);
    const double v2 = vx * vx + vy * vy + vz * vz;
    const double hx = ry * vz - rz * vy, hy = rz * vx - rx * vz, hz = rx * vy - ry * vx;
    const double h2 = hx * hx + hy * hy + hz * hz;
    if (h2 < 2.2250738585072014e-308) return;  // tiny(1.0_DP)
    const double energy = 0.5 * v2 - mu / r;
    int type;  // -1 ellipse, 0 parabola, 1 hyperbola
    double fac = 0.0;
    if (fabs(energy * r / mu) < sqrt(TINYV)) {
        type = 0;
    } else {
        a = -0.5 * mu / energy;
        if (a < 0.0) {
            fac = -h2 / (mu * a);
            type = fac > TINYV ? 1 : 0;
        } else {
            type = -1;
        }
    }
    if (type == -1) {
        fac = 1.0 - h2 / (mu * a);
        if (fac > TINYV) e = sqrt(fac);
        q = a * (1.0 - e);
    } else if (type == 0) {
        a = 0.5 * h2 / mu;
        e = 1.0;
        q = a;
    } else {
        e = sqrt(1.0 + fac);
        q = a * (1.0 - e);
    }
}

// collision_check_one (src/collision/collision_check.f90:16-57)
__host__ __device__ inline bool d_collision_one(double xr, double yr, double zr, double vxr, double vyr, double vzr,
                                                double Gmtot, double rlim, double dt, bool lvdotr) {
    const double r2 = xr * xr + yr * yr + zr * zr;
    const double rlim2 = rlim * rlim;
    if (r2 <= rlim2) return true;
    const double vdotr = xr * vxr + yr * vyr + zr * vzr;
    if (lvdotr && vdotr > 0.0) {
        const double tcr2 = r2 / (vxr * vxr + vyr * vyr + vzr * vzr);
        const double dt2 = dt * dt;
        if (tcr2 <= dt2) {
            double a, e, q;
            d_xv2aeq(Gmtot, xr, yr, zr, vxr, vyr, vzr, a, e, q);
            return q < rlim;
        }
    }
    return false;
}

}  // namespace swg
