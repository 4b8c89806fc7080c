// encounter_dev.cuh -- device pieces of the close-encounter test shared by the
// encounter kernels (encounter.cu, encounter_sorted.cu): encounter_check_one in FP64
// with the reference's expression order (src/encounter/encounter_check.f90:573-621), the
// float copy of a body used by the prefilter, and the conservative FP32 prefilter.
#pragma once
#include <cuda_runtime.h>

#include "swg_internal.cuh"

namespace swg {

// encounter_check_one (:573-621), FP64, reference expression order
__device__ __forceinline__ void d_encounter_one(double xr, double yr, double zr, double vxr, double vyr, double vzr,
                                                double renc, double dt, int &lenc, int &lvdotr) {
    const double r2 = xr * xr + yr * yr + zr * zr;
    const double r2crit = renc * renc;
    double vdotr, r2min;
    if (r2 > r2crit) {
        vdotr = vxr * xr + vyr * yr + vzr * zr;
        if (vdotr > 0.0) {
            r2min = r2;
        } else {
            const double v2 = vxr * vxr + vyr * vyr + vzr * vzr;
            if (v2 <= VSMALL) {
                r2min = r2;
            } else {
                const double tmin = -vdotr / v2;
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
    lvdotr = (vdotr < 0.0);
    lenc = lvdotr && (r2min <= r2crit);
}

// swiftest_discard_pl_close (src/swiftest/swiftest_discard.f90:293-336): does the relative
// linear motion (dx, dv) come within sqrt(r2crit) during the step dt?
__device__ __forceinline__ bool d_discard_close(double dx, double dy, double dz, double dvx, double dvy, double dvz,
                                                double dt, double r2crit) {
    const double r2 = dx * dx + dy * dy + dz * dz;
    if (r2 <= r2crit) return true;
    const double vdotr = dx * dvx + dy * dvy + dz * dvz;
    if (vdotr > 0.0) return false;
    const double v2 = dvx * dvx + dvy * dvy + dvz * dvz;
    const double tmin = -vdotr / v2;
    double r2min;
    if (tmin < dt)
        r2min = r2 - vdotr * vdotr / v2;
    else
        r2min = r2 + 2.0 * vdotr * dt + v2 * (dt * dt);
    r2min = r2min < r2 ? r2min : r2;
    return r2min <= r2crit;
}

struct BodyF {
    float4 a;  // x_hi, y_hi, z_hi, renc
    float4 b;  // x_lo, y_lo, z_lo, |r|
    float4 v;  // vx, vy, vz, |v|
};

__device__ __forceinline__ BodyF load_body(const double *r, const double *v, const double *renc, int i) {
    BodyF o;
    const double x = r[3 * i], y = r[3 * i + 1], z = r[3 * i + 2];
    const float xh = __double2float_rn(x), yh = __double2float_rn(y), zh = __double2float_rn(z);
    o.a = make_float4(xh, yh, zh, renc ? __double2float_rn(renc[i]) : 0.f);
    o.b = make_float4(__double2float_rn(x - (double)xh), __double2float_rn(y - (double)yh),
                      __double2float_rn(z - (double)zh), sqrtf(xh * xh + yh * yh + zh * zh));
    const float vx = __double2float_rn(v[3 * i]), vy = __double2float_rn(v[3 * i + 1]),
                vz = __double2float_rn(v[3 * i + 2]);
    o.v = make_float4(vx, vy, vz, sqrtf(vx * vx + vy * vy + vz * vz));
    return o;
}

// True when the pair certainly fails encounter_check_one.  The FP64 test accepts a
// pair only if its computed r2min <= R^2, and that computed value is at least
// D^2 - 6.7e-16 r^2 with D >= |x| - |v| |dt| (the closest approach of the linear
// motion over the step).  So |x| (1 - 2.6e-8) > R + |v| |dt| guarantees rejection.
// It is evaluated without square roots or divisions: |v| is bounded by the L1 norm
// of the float velocity difference, and the comparison is made on squares,
//     r^2 (1 - 4e-6) > (R (1 + 1e-5) + V |dt| + e_x)^2,
// where the relative margins cover float rounding of r^2, R and |x| (< 1e-6) and
// e_x, V's extra term cover the hi/lo position split and the float rounding of the
// velocities.  NaN or inf inputs make the comparison false: such pairs go to the FP64 test.
__device__ __forceinline__ bool prefilter_reject(const BodyF &p, const BodyF &q, float dtf) {
    const float dx = (p.a.x - q.a.x) + (p.b.x - q.b.x);
    const float dy = (p.a.y - q.a.y) + (p.b.y - q.b.y);
    const float dz = (p.a.z - q.a.z) + (p.b.z - q.b.z);
    const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
    const float vl1 = fabsf(p.v.x - q.v.x) + fabsf(p.v.y - q.v.y) + fabsf(p.v.z - q.v.z);
    const float vhi = fmaf(vl1, 1.0f + 2e-6f, 2e-7f * (p.v.w + q.v.w));
    const float reff = fmaf(p.a.w + q.a.w, 1.0f + 1e-5f, fmaf(vhi, dtf, 1e-13f * (p.b.w + q.b.w)));
    return r2 * (1.0f - 4e-6f) > reff * reff;
}

}  // namespace swg
