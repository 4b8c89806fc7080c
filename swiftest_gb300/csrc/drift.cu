// drift.cu -- Danby universal-variable Kepler drift for sm_103a.
//
// Restates swiftest_drift_all / _one / _dan / _kepmd / _kepu / _kepu_guess /
// _kepu_new / _kepu_lag / _kepu_fchk / _kepu_p3solve / _kepu_stumpff
// (src/swiftest/swiftest_drift.f90:60-580) and swiftest_orbel_scget
// (src/swiftest/swiftest_orbel.f90:147-172), one thread per body, FP64, in the
// reference's operation order (this file is compiled with -fmad=false so no
// expression is contracted into an FMA).  Each iterative loop keeps the
// reference's bounded iteration caps (Newton 7, Laguerre 50/40, 10 sub-steps),
// so every thread terminates; non-convergence is reported through iflag.
//
// Bound: the drift reads mu, r, v, mask (60 B) and writes r, v, iflag (52 B)
// per body, but costs hundreds of FP64 operations per body (divides, square
// roots, Stumpff series), so on GB300 it is limited by the FP64 pipe, not HBM.
#include <cuda_runtime.h>

#include "drift_impl.cuh"
#include "swg_internal.cuh"

namespace swg {

// gfortran NORM2 (scaled sum of squares)
__device__ __forceinline__ double d_norm2(double a, double b, double c) {
    double scale = 0.0, ssq = 1.0;
    const double v[3] = {a, b, c};
#pragma unroll
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

// swiftest_drift_all (:60-108); mu may be an array or a scalar (mu == nullptr)
__global__ void __launch_bounds__(128) k_drift_all(const double *__restrict__ mu, double mu_scalar, double *x,
                                                   double *v, int n, int lgr, double inv_c2, double dt,
                                                   const int32_t *__restrict__ lmask, int32_t *__restrict__ iflag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (!lmask[i]) return;
    double rx = x[3 * i], ry = x[3 * i + 1], rz = x[3 * i + 2];
    double vx = v[3 * i], vy = v[3 * i + 1], vz = v[3 * i + 2];
    const double m = mu ? mu[i] : mu_scalar;
    double dtp = dt;
    if (lgr) {
        const double rmag = d_norm2(rx, ry, rz);
        const double vmag2 = vx * vx + vy * vy + vz * vz;
        const double energy = 0.5 * vmag2 - m / rmag;
        dtp = dt * (1.0 + 3.0 * inv_c2 * energy);
    }
    const int fl = d_drift_one(m, rx, ry, rz, vx, vy, vz, dtp);
    x[3 * i] = rx;
    x[3 * i + 1] = ry;
    x[3 * i + 2] = rz;
    v[3 * i] = vx;
    v[3 * i + 1] = vy;
    v[3 * i + 2] = vz;
    iflag[i] = fl;
}

// helio_drift_body (helio_drift.f90:14-54) under symba_drift_pl/_tp's mask
// (symba_drift.f90:14-61): drift bodies with status /= INACTIVE and
// levelg == irec (levelg == nullptr: every body with status /= INACTIVE);
// failures set status = DISCARDED_DRIFTERR and are counted in *nfail.
// mu_sys/sys (optional): the body's own system's central-body mu (CSR-packed ensembles).
// FAST: the fast FP64 form of the solver (mixed-precision path, see drift_impl.cuh).
template <bool FAST>
__global__ void __launch_bounds__(128) k_drift_masked(double mu, double *x, double *v, int n,
                                                      const int32_t *__restrict__ levelg, int irec, double dt,
                                                      int32_t *__restrict__ status, int32_t *nfail,
                                                      const double *__restrict__ mu_sys,
                                                      const int32_t *__restrict__ sys) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (status[i] == ST_INACTIVE) return;
    if (levelg && levelg[i] != irec) return;
    double rx = x[3 * i], ry = x[3 * i + 1], rz = x[3 * i + 2];
    double vx = v[3 * i], vy = v[3 * i + 1], vz = v[3 * i + 2];
    const double m = mu_sys ? mu_sys[sys[i]] : mu;
    const int fl = FAST ? d_drift_one_fast(m, rx, ry, rz, vx, vy, vz, dt) : d_drift_one(m, rx, ry, rz, vx, vy, vz, dt);
    x[3 * i] = rx;
    x[3 * i + 1] = ry;
    x[3 * i + 2] = rz;
    v[3 * i] = vx;
    v[3 * i + 1] = vy;
    v[3 * i + 2] = vz;
    if (fl != 0) {
        status[i] = ST_DISCARDED_DRIFTERR;
        if (nfail) atomicAdd(nfail, 1);
    }
}

int drift_all(swg_ctx *c, const double *mu, double mu_scalar, double *x, double *v, int32_t n, int32_t lgr,
              double inv_c2, double dt, const int32_t *lmask, int32_t *iflag) {
    if (n <= 0) return SWG_OK;
    k_drift_all<<<(n + 127) / 128, 128, 0, c->stream>>>(mu, mu_scalar, x, v, n, lgr, inv_c2, dt, lmask, iflag);
    c->launches++;
    return launch_status(c, "drift_all");
}

int drift_masked(swg_ctx *c, double mu, double *x, double *v, int32_t n, const int32_t *levelg, int irec, double dt,
                 int32_t *status, int32_t *nfail, const double *mu_sys, const int32_t *sys, bool fast) {
    if (n <= 0) return SWG_OK;
    if (fast)
        k_drift_masked<true><<<(n + 127) / 128, 128, 0, c->stream>>>(mu, x, v, n, levelg, irec, dt, status, nfail,
                                                                     mu_sys, sys);
    else
        k_drift_masked<false><<<(n + 127) / 128, 128, 0, c->stream>>>(mu, x, v, n, levelg, irec, dt, status, nfail,
                                                                      mu_sys, sys);
    c->launches++;
    return launch_status(c, "drift_masked");
}

}  // namespace swg
