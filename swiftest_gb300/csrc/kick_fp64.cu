// kick_fp64.cu -- FP64 pair kick in the reference's exact operation order, spread over all SMs.
//
// Restates swiftest_kick_getacch_int_all_tri_* (src/swiftest/swiftest_kick.f90:165-371),
// the flat forms (:69-162) and swiftest_kick_getacch_int_all_tp (:374-415).
//
// Every per-body sum must add its terms one at a time in ascending partner order
// to reproduce the reference's rounding, which leaves no parallelism inside one
// body's sum.  The expensive part of a term (three differences, r^2, sqrt, an
// IEEE divide: ~32 FP64 instructions) has no such constraint, so a block of 256
// threads owns RT receivers and walks the partners in rounds of PT = 256/RT:
// all 256 threads compute one term each into shared memory, then RT threads
// fold their receiver's PT terms in order (3 dependent adds per term).  GB300's
// FP64 pipe (~1 TFLOP/s measured) is then fed from every SM instead of from the
// npl/128 blocks a thread-per-receiver kernel would launch.
//
// Modes (see kick.cu): KICK_DIRECT adds Gm_j/(r^2 sqrt r^2) * dx straight into
// acc; KICK_SPLIT keeps ahi (partners j > i) and ahj (j < i) separately with
// irij3 = 1/(r^2 sqrt r^2) and finishes acc = (acc + ahi) + ahj.
#include <cuda_runtime.h>

#include "swg_internal.cuh"

namespace swg {

constexpr int FT = 256;  // threads per block
constexpr int FP64_RT = 8;  // receivers per block (FT / FP64_RT partners per round)

// Receivers [i0, i0 + RT) of one system against all its partners, whole block.
template <bool RAD, int MODE, int RT>
__device__ __forceinline__ void fp64_plpl_group(int npl, int nplm, const double *__restrict__ r,
                                                const double *__restrict__ Gm, const double *__restrict__ R,
                                                double *__restrict__ acc, int acc_is_zero, int i0) {
    constexpr int PT = FT / RT;
    __shared__ double sx[PT], sy[PT], sz[PT], sg[PT], sr[PT];
    __shared__ double tx[RT][PT + 1], ty[RT][PT + 1], tz[RT][PT + 1];
    __shared__ unsigned char tf[RT][PT];
    const int t = threadIdx.x;
    const int rr = t / PT, pp = t % PT;
    const int i = i0 + rr;  // receiver of this thread's terms
    double xi = 0, yi = 0, zi = 0, Ri = 0;
    if (i < npl) {
        xi = r[3 * i + 0];
        yi = r[3 * i + 1];
        zi = r[3 * i + 2];
        if (RAD) Ri = R[i];
    }
    const int jend = (i < nplm) ? npl : nplm;  // partner range of receiver i
    // accumulators: thread t < RT owns receiver i0 + t
    const int ia = i0 + t;
    double ax = 0, ay = 0, az = 0, bx = 0, by = 0, bz = 0;
    if (MODE == KICK_DIRECT && t < RT && ia < npl && !acc_is_zero) {
        ax = acc[3 * ia + 0];
        ay = acc[3 * ia + 1];
        az = acc[3 * ia + 2];
    }
    const int blk_jend = (i0 < nplm) ? npl : nplm;
    for (int j0 = 0; j0 < blk_jend; j0 += PT) {
        if (t < PT && j0 + t < npl) {
            const int jl = j0 + t;
            sx[t] = r[3 * jl + 0];
            sy[t] = r[3 * jl + 1];
            sz[t] = r[3 * jl + 2];
            sg[t] = Gm[jl];
            if (RAD) sr[t] = R[jl];
        }
        __syncthreads();
        const int j = j0 + pp;
        unsigned char flag = 0;
        double fx = 0, fy = 0, fz = 0;
        if (i < npl && j < jend && j != i) {
            const double rx = sx[pp] - xi;
            const double ry = sy[pp] - yi;
            const double rz = sz[pp] - zi;
            const double rji2 = rx * rx + ry * ry + rz * rz;
            bool ok = true;
            if (RAD) {
                const double rs = Ri + sr[pp];
                ok = rji2 > rs * rs;
            }
            if (ok) {
                double fac;
                if (MODE == KICK_DIRECT) {
                    fac = sg[pp] / (rji2 * sqrt(rji2));
                    flag = 1;
                } else {
                    const double irij3 = 1.0 / (rji2 * sqrt(rji2));
                    fac = sg[pp] * irij3;
                    flag = j > i ? 1 : 2;
                }
                fx = fac * rx;
                fy = fac * ry;
                fz = fac * rz;
            }
        }
        tx[rr][pp] = fx;
        ty[rr][pp] = fy;
        tz[rr][pp] = fz;
        tf[rr][pp] = flag;
        __syncthreads();
        if (t < RT && ia < npl) {
#pragma unroll 4
            for (int p = 0; p < PT; p++) {
                const unsigned char f = tf[t][p];
                if (f == 1) {
                    ax = ax + tx[t][p];
                    ay = ay + ty[t][p];
                    az = az + tz[t][p];
                } else if (f == 2) {
                    bx = bx + tx[t][p];
                    by = by + ty[t][p];
                    bz = bz + tz[t][p];
                }
            }
        }
        // the next round's first barrier orders these reads before the next term writes
    }
    if (t < RT && ia < npl) {
        if (MODE == KICK_DIRECT) {
            acc[3 * ia + 0] = ax;
            acc[3 * ia + 1] = ay;
            acc[3 * ia + 2] = az;
        } else {
            const double a0 = acc_is_zero ? 0.0 : acc[3 * ia + 0];
            const double a1 = acc_is_zero ? 0.0 : acc[3 * ia + 1];
            const double a2 = acc_is_zero ? 0.0 : acc[3 * ia + 2];
            acc[3 * ia + 0] = a0 + ax + bx;
            acc[3 * ia + 1] = a1 + ay + by;
            acc[3 * ia + 2] = a2 + az + bz;
        }
    }
}

// pl -> tp (swiftest_kick.f90:374-415): acc -= Gm_j/(r^2 sqrt r^2) * (r_tp - r_j), masked
template <int RT>
__device__ __forceinline__ void fp64_tp_group(int ntp, int npl, const double *__restrict__ rtp,
                                              const double *__restrict__ rpl, const double *__restrict__ Gm,
                                              const int32_t *__restrict__ lmask, double *__restrict__ acc,
                                              int acc_is_zero, int i0) {
    constexpr int PT = FT / RT;
    __shared__ double sx[PT], sy[PT], sz[PT], sg[PT];
    __shared__ double tx[RT][PT + 1], ty[RT][PT + 1], tz[RT][PT + 1];
    const int t = threadIdx.x;
    const int rr = t / PT, pp = t % PT;
    const int i = i0 + rr;
    const bool iact = i < ntp && lmask[i] != 0;
    double xi = 0, yi = 0, zi = 0;
    if (iact) {
        xi = rtp[3 * i + 0];
        yi = rtp[3 * i + 1];
        zi = rtp[3 * i + 2];
    }
    const int ia = i0 + t;
    const bool aact = t < RT && ia < ntp && lmask[ia] != 0;
    double ax = 0, ay = 0, az = 0;
    if (aact && !acc_is_zero) {
        ax = acc[3 * ia + 0];
        ay = acc[3 * ia + 1];
        az = acc[3 * ia + 2];
    }
    for (int j0 = 0; j0 < npl; j0 += PT) {
        if (t < PT && j0 + t < npl) {
            const int jl = j0 + t;
            sx[t] = rpl[3 * jl + 0];
            sy[t] = rpl[3 * jl + 1];
            sz[t] = rpl[3 * jl + 2];
            sg[t] = Gm[jl];
        }
        __syncthreads();
        double fx = 0, fy = 0, fz = 0;
        if (iact && j0 + pp < npl) {
            const double rx = xi - sx[pp];
            const double ry = yi - sy[pp];
            const double rz = zi - sz[pp];
            const double rji2 = rx * rx + ry * ry + rz * rz;
            const double fac = sg[pp] / (rji2 * sqrt(rji2));
            fx = fac * rx;
            fy = fac * ry;
            fz = fac * rz;
        }
        tx[rr][pp] = fx;
        ty[rr][pp] = fy;
        tz[rr][pp] = fz;
        __syncthreads();
        if (aact) {
            const int np = min(PT, npl - j0);
#pragma unroll 4
            for (int p = 0; p < np; p++) {
                ax = ax - tx[t][p];
                ay = ay - ty[t][p];
                az = az - tz[t][p];
            }
        }
    }
    if (aact) {
        acc[3 * ia + 0] = ax;
        acc[3 * ia + 1] = ay;
        acc[3 * ia + 2] = az;
    } else if (t < RT && ia < ntp && acc_is_zero) {
        acc[3 * ia + 0] = 0.0;
        acc[3 * ia + 1] = 0.0;
        acc[3 * ia + 2] = 0.0;
    }
}

template <bool RAD, int MODE, int RT>
__global__ void __launch_bounds__(FT) k_kick_plpl_fp64(int npl, int nplm, const double *__restrict__ r,
                                                      const double *__restrict__ Gm, const double *__restrict__ R,
                                                      double *__restrict__ acc, int acc_is_zero) {
    fp64_plpl_group<RAD, MODE, RT>(npl, nplm, r, Gm, R, acc, acc_is_zero, blockIdx.x * RT);
}

template <int RT>
__global__ void __launch_bounds__(FT) k_kick_tp_fp64(int ntp, int npl, const double *__restrict__ rtp,
                                                    const double *__restrict__ rpl, const double *__restrict__ Gm,
                                                    const int32_t *__restrict__ lmask, double *__restrict__ acc,
                                                    int acc_is_zero) {
    fp64_tp_group<RT>(ntp, npl, rtp, rpl, Gm, lmask, acc, acc_is_zero, blockIdx.x * RT);
}

// Batched (ensemble) forms: block b takes item b = (system s, first receiver r0) of a
// table sorted by cost; system s's pl occupy [poff[s], poff[s] + npl[s]) and its tp
// [toff[s], toff[s] + ntp[s]).  nplm (optional): per system the count of fully
// interacting bodies (GMTINY, SyMBA), which selects the reference's loop shape as the single
// system does (KICK_SPLIT when the semi-interacting bodies outnumber the others); without
// it every system is fully interacting (KICK_DIRECT).  With sys_flag, the pl-pl form kicks
// only systems whose flag equals `phase`.
template <bool RAD, int RT>
__global__ void __launch_bounds__(FT) k_kick_plpl_fp64_batched(const int4 *__restrict__ items,
                                                              const int32_t *__restrict__ poff,
                                                              const int32_t *__restrict__ npl,
                                                              const double *__restrict__ r,
                                                              const double *__restrict__ Gm,
                                                              const double *__restrict__ R, double *__restrict__ acc,
                                                              int acc_is_zero, const int32_t *__restrict__ sys_flag,
                                                              int phase, const int32_t *__restrict__ nplm) {
    const int4 w = items[blockIdx.x];
    if (sys_flag && sys_flag[w.x] != phase) return;  // another launch's system
    const int o = poff[w.x], n = npl[w.x], m = nplm ? nplm[w.x] : n;
    if (n - m > m)  // block-uniform
        fp64_plpl_group<RAD, KICK_SPLIT, RT>(n, m, r + 3 * (size_t)o, Gm + o, RAD ? R + o : nullptr,
                                             acc + 3 * (size_t)o, acc_is_zero, w.y);
    else
        fp64_plpl_group<RAD, KICK_DIRECT, RT>(n, m, r + 3 * (size_t)o, Gm + o, RAD ? R + o : nullptr,
                                              acc + 3 * (size_t)o, acc_is_zero, w.y);
}

template <int RT>
__global__ void __launch_bounds__(FT) k_kick_tp_fp64_batched(const int4 *__restrict__ items,
                                                            const int32_t *__restrict__ toff,
                                                            const int32_t *__restrict__ ntp,
                                                            const int32_t *__restrict__ poff,
                                                            const int32_t *__restrict__ npl,
                                                            const double *__restrict__ rtp,
                                                            const double *__restrict__ rpl,
                                                            const double *__restrict__ Gm,
                                                            const int32_t *__restrict__ lmask,
                                                            double *__restrict__ acc, int acc_is_zero) {
    const int4 w = items[blockIdx.x];
    const int ot = toff[w.x], op = poff[w.x];
    fp64_tp_group<RT>(ntp[w.x], npl[w.x], rtp + 3 * (size_t)ot, rpl + 3 * (size_t)op, Gm + op, lmask + ot,
                      acc + 3 * (size_t)ot, acc_is_zero, w.y);
}

static inline int div_up_i(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

int kick_plpl_fp64(swg_ctx *c, int32_t npl, int32_t nplm, const double *r, const double *Gm, const double *R,
                   double *acc, int mode, int acc_is_zero) {
    if (npl <= 0) return SWG_OK;
    constexpr int RT = 8;
    const int grid = div_up_i(npl, RT);
    if (mode == KICK_DIRECT) {
        if (R)
            k_kick_plpl_fp64<true, KICK_DIRECT, RT><<<grid, FT, 0, c->stream>>>(npl, nplm, r, Gm, R, acc, acc_is_zero);
        else
            k_kick_plpl_fp64<false, KICK_DIRECT, RT><<<grid, FT, 0, c->stream>>>(npl, nplm, r, Gm, R, acc, acc_is_zero);
    } else {
        if (R)
            k_kick_plpl_fp64<true, KICK_SPLIT, RT><<<grid, FT, 0, c->stream>>>(npl, nplm, r, Gm, R, acc, acc_is_zero);
        else
            k_kick_plpl_fp64<false, KICK_SPLIT, RT><<<grid, FT, 0, c->stream>>>(npl, nplm, r, Gm, R, acc, acc_is_zero);
    }
    c->launches++;
    return launch_status(c, "kick_plpl_fp64");
}

int kick_tp_fp64(swg_ctx *c, int32_t ntp, int32_t npl, const double *rtp, const double *rpl, const double *Gm,
                 const int32_t *lmask, double *acc, int acc_is_zero) {
    if (ntp <= 0) return SWG_OK;
    constexpr int RT = 8;
    k_kick_tp_fp64<RT><<<div_up_i(ntp, RT), FT, 0, c->stream>>>(ntp, npl, rtp, rpl, Gm, lmask, acc, acc_is_zero);
    c->launches++;
    return launch_status(c, "kick_tp_fp64");
}

int kick_plpl_fp64_batched(swg_ctx *c, bool rad, int nitems, const int4 *items, const int32_t *poff,
                           const int32_t *npl, const double *r, const double *Gm, const double *R, double *acc,
                           int acc_is_zero, const int32_t *sys_flag, int phase, const int32_t *nplm) {
    if (nitems <= 0) return SWG_OK;
    if (rad)
        k_kick_plpl_fp64_batched<true, FP64_RT><<<nitems, FT, 0, c->stream>>>(items, poff, npl, r, Gm, R, acc,
                                                                              acc_is_zero, sys_flag, phase, nplm);
    else
        k_kick_plpl_fp64_batched<false, FP64_RT><<<nitems, FT, 0, c->stream>>>(items, poff, npl, r, Gm, nullptr, acc,
                                                                               acc_is_zero, sys_flag, phase, nplm);
    c->launches++;
    return launch_status(c, "kick_plpl_fp64_batched");
}

int kick_tp_fp64_batched(swg_ctx *c, int nitems, const int4 *items, const int32_t *toff, const int32_t *ntp,
                         const int32_t *poff, const int32_t *npl, const double *rtp, const double *rpl,
                         const double *Gm, const int32_t *lmask, double *acc, int acc_is_zero) {
    if (nitems <= 0) return SWG_OK;
    k_kick_tp_fp64_batched<FP64_RT><<<nitems, FT, 0, c->stream>>>(items, toff, ntp, poff, npl, rtp, rpl, Gm, lmask,
                                                                  acc, acc_is_zero);
    c->launches++;
    return launch_status(c, "kick_tp_fp64_batched");
}

}  // namespace swg
