// symba_dev.cuh -- device building blocks shared by the single-system step loops
// (system.cu) and the batched ensemble (ensemble.cu): ordered block sums, the
// encounter test and shell-kick helpers, the SyMBA recursion as a block-wide device
// function, and the energy / momentum diagnostic.
//
// Everything here works on global body indices into arrays that the caller
// passes, so one system (offset 0) and a CSR-packed ensemble (system s occupying
// a contiguous index range) use the same code.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "collision_one.cuh"
#include "drift_impl.cuh"
#include "swg_internal.cuh"

namespace swg {
namespace sdev {

// device-side central-body record (doubles): barycentric velocity and position of
// the central body, and the linear-drift momentum at the start and end of a step
enum { CB_VB = 0, CB_RB = 3, CB_PTBEG = 6, CB_PTEND = 9, CB_N = 12 };

// ---------------------------------------------------------------- small kernels
// Ordered sums of the reference's O(N) serial loops.  exact == 1: the terms are formed
// by the whole block into shared memory, chunk by chunk, and thread 0 adds them one at
// a time in the reference's index order, which reproduces its rounding.  exact == 0:
// thread t adds its own terms t, t + RB, t + 2 RB, ... in registers, then the block
// combines the partial sums as a tree (warp shuffles, then one warp over the warp
// sums): a fixed order, so results are deterministic, with no serial chain.  The block
// may have any multiple of 32 threads up to RB.
constexpr int RB = 1024;  // most threads of the reduction kernels

struct Sum3 {
    double x, y, z;
};

// Sum over i of sign*term(i) for i = 0..n-1 (reverse: n-1..0); term_fn(i, x, y, z)
// writes the components and returns the 0/1 mask.
// shared-memory workspace of ordered_sum3 (one per kernel)
struct SumScratch {
    double cx[RB], cy[RB], cz[RB];
    double rx[RB / 32], ry[RB / 32], rz[RB / 32];
    unsigned char cm[RB];
    Sum3 acc;
};

__device__ __forceinline__ void warp_sum3(double &x, double &y, double &z) {
    for (int off = 16; off > 0; off >>= 1) {
        x += __shfl_down_sync(0xffffffffu, x, off);
        y += __shfl_down_sync(0xffffffffu, y, off);
        z += __shfl_down_sync(0xffffffffu, z, off);
    }
}

template <class TermFn>
__device__ Sum3 ordered_sum3(int n, bool reverse, bool exact, TermFn term_fn, double sign, SumScratch &sh) {
    double *cx = sh.cx, *cy = sh.cy, *cz = sh.cz, *rx = sh.rx, *ry = sh.ry, *rz = sh.rz;
    unsigned char *cm = sh.cm;
    Sum3 &acc = sh.acc;
    __syncthreads();  // a previous sum's result may still be being read
    if (exact) {
        if (threadIdx.x == 0) acc = {0.0, 0.0, 0.0};
        __syncthreads();
        const int nb = blockDim.x;
        for (int c0 = 0; c0 < n; c0 += nb) {
            const int k = threadIdx.x;
            const int idx = reverse ? n - 1 - (c0 + k) : c0 + k;
            double tx = 0, ty = 0, tz = 0;
            unsigned char m = 0;
            if (c0 + k < n) m = term_fn(idx, tx, ty, tz);
            const int cnt = min(nb, n - c0);
            cx[k] = tx;
            cy[k] = ty;
            cz[k] = tz;
            cm[k] = m;
            __syncthreads();
            if (threadIdx.x == 0) {
                double ax = acc.x, ay = acc.y, az = acc.z;
                for (int q = 0; q < cnt; q++) {
                    if (!cm[q]) continue;
                    ax = ax + sign * cx[q];
                    ay = ay + sign * cy[q];
                    az = az + sign * cz[q];
                }
                acc = {ax, ay, az};
            }
            __syncthreads();
        }
        return acc;
    }
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
        double tx, ty, tz;
        if (term_fn(reverse ? n - 1 - q : q, tx, ty, tz)) {
            ax += tx;
            ay += ty;
            az += tz;
        }
    }
    warp_sum3(ax, ay, az);
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        rx[w] = ax;
        ry[w] = ay;
        rz[w] = az;
    }
    __syncthreads();
    if (w == 0) {
        const bool have = threadIdx.x < (blockDim.x >> 5);  // one warp sum per warp of the block
        double x = have ? rx[threadIdx.x] : 0.0, y = have ? ry[threadIdx.x] : 0.0, z = have ? rz[threadIdx.x] : 0.0;
        warp_sum3(x, y, z);
        if (threadIdx.x == 0) acc = {sign * x, sign * y, sign * z};
    }
    __syncthreads();
    return acc;
}
static_assert(RB / 32 == 32, "ordered_sum3 combines the warp sums in one warp");

// helio_drift_linear_pl (helio_drift.f90:129-163): pt = sum(Gm*vb, mask)/GMcb ; rh += pt*dt
static __device__ void blk_lindrift_pl(int npl, const double *__restrict__ Gm,
                                                    const double *__restrict__ vb, const int32_t *__restrict__ lmask,
                                                    double GMcb, double *rh, double dt, double *dcb, int slot,
                                int exact, SumScratch &sh) {
    auto term = [&](int i, double &x, double &y, double &z) -> unsigned char {
        x = Gm[i] * vb[3 * i + 0];
        y = Gm[i] * vb[3 * i + 1];
        z = Gm[i] * vb[3 * i + 2];
        return lmask[i] != 0;
    };
    const Sum3 s = ordered_sum3(npl, false, exact != 0, term, 1.0, sh);
    const double ptx = s.x / GMcb, pty = s.y / GMcb, ptz = s.z / GMcb;
    for (int i = threadIdx.x; i < npl; i += blockDim.x) {
        if (!lmask[i]) continue;
        if (exact) {
            rh[3 * i + 0] = rh[3 * i + 0] + ptx * dt;
            rh[3 * i + 1] = rh[3 * i + 1] + pty * dt;
            rh[3 * i + 2] = rh[3 * i + 2] + ptz * dt;
        } else {  // one rounding per coordinate (the FP64 pipe is narrow)
            rh[3 * i + 0] = fma(ptx, dt, rh[3 * i + 0]);
            rh[3 * i + 1] = fma(pty, dt, rh[3 * i + 1]);
            rh[3 * i + 2] = fma(ptz, dt, rh[3 * i + 2]);
        }
    }
    if (threadIdx.x == 0) {
        dcb[slot + 0] = ptx;
        dcb[slot + 1] = pty;
        dcb[slot + 2] = ptz;
    }
}

// swiftest_util_coord_vh2vb_pl (swiftest_util.f90:424-456)
static __device__ void blk_vh2vb_pl(int npl, const double *__restrict__ Gm,
                                                 const double *__restrict__ vh, double *vb, double GMcb, double *dcb,
                             int exact, SumScratch &sh) {
    auto gm = [&](int i, double &x, double &y, double &z) -> unsigned char {
        x = Gm[i];
        y = z = 0.0;
        return 1;
    };
    const Sum3 g = ordered_sum3(npl, false, exact != 0, gm, 1.0, sh);
    const double Gmtot = GMcb + g.x;
    auto term = [&](int i, double &x, double &y, double &z) -> unsigned char {
        x = Gm[i] * vh[3 * i + 0];
        y = Gm[i] * vh[3 * i + 1];
        z = Gm[i] * vh[3 * i + 2];
        return 1;
    };
    const Sum3 s = ordered_sum3(npl, false, exact != 0, term, -1.0, sh);
    const double cx = s.x / Gmtot, cy = s.y / Gmtot, cz = s.z / Gmtot;
    if (threadIdx.x == 0) {
        dcb[CB_VB + 0] = cx;
        dcb[CB_VB + 1] = cy;
        dcb[CB_VB + 2] = cz;
    }
    for (int i = threadIdx.x; i < npl; i += blockDim.x) {
        vb[3 * i + 0] = vh[3 * i + 0] + cx;
        vb[3 * i + 1] = vh[3 * i + 1] + cy;
        vb[3 * i + 2] = vh[3 * i + 2] + cz;
    }
}

// swiftest_util_coord_vb2vh_pl (swiftest_util.f90:363-392), reverse-order sum.  The
// reference divides every term by GMcb; the non-exact path multiplies by the reciprocal
// instead (an FP64 divide is ~20 instructions on the narrow FP64 pipe).
static __device__ void blk_vb2vh_pl(int npl, const double *__restrict__ Gm,
                                                 const double *__restrict__ vb, const int32_t *__restrict__ status,
                                                 double *vh, double GMcb, double *dcb, int exact, SumScratch &sh) {
    const double inv = 1.0 / GMcb;
    auto term = [&](int i, double &x, double &y, double &z) -> unsigned char {
        if (exact) {
            x = Gm[i] * vb[3 * i + 0] / GMcb;
            y = Gm[i] * vb[3 * i + 1] / GMcb;
            z = Gm[i] * vb[3 * i + 2] / GMcb;
        } else {
            const double g = Gm[i] * inv;
            x = g * vb[3 * i + 0];
            y = g * vb[3 * i + 1];
            z = g * vb[3 * i + 2];
        }
        return status[i] != ST_INACTIVE;
    };
    const Sum3 s = ordered_sum3(npl, true, exact != 0, term, -1.0, sh);
    if (threadIdx.x == 0) {
        dcb[CB_VB + 0] = s.x;
        dcb[CB_VB + 1] = s.y;
        dcb[CB_VB + 2] = s.z;
    }
    for (int i = threadIdx.x; i < npl; i += blockDim.x) {
        vh[3 * i + 0] = vb[3 * i + 0] - s.x;
        vh[3 * i + 1] = vb[3 * i + 1] - s.y;
        vh[3 * i + 2] = vb[3 * i + 2] - s.z;
    }
}

// level-0 bookkeeping of symba_encounter_check_pl / _tp (symba_encounter_check.f90:53-83, 267-290)
static __global__ void k_level0_mark(int64_t n, int32_t *l, int64_t cap, int tp, int32_t *levelg, int32_t *levelm,
                              int32_t *cnt1, int32_t *tlevelg, int32_t *tlevelm, int32_t *cnt2) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    int32_t *i1 = l, *i2 = l + cap, *st = l + 3 * cap, *lev = l + 4 * cap;
    const int i = i1[k] - 1, j = i2[k] - 1;
    st[k] = ST_ACTIVE;
    lev[k] = 0;
    levelg[i] = 0;
    levelm[i] = 0;
    if (!tp) {
        levelg[j] = 0;
        levelm[j] = 0;
        atomicAdd(&cnt1[i], 1);
        atomicAdd(&cnt1[j], 1);
    } else {
        tlevelg[j] = 0;
        tlevelm[j] = 0;
        atomicAdd(&cnt1[i], 1);
        atomicAdd(&cnt2[j], 1);
    }
}

// Sort a short raw pair list by (index1, index2), drop repeated pairs, and write it as a
// SyMBA encounter list with status ACTIVE, level 0 and the level-0 body marks of
// symba_encounter_check_pl / _tp (symba_encounter_check.f90:53-83, 267-290).  One block.
constexpr int FIN_N = 4096;
static __global__ void __launch_bounds__(1024) k_list_finalize(int n, const int32_t *__restrict__ ri1,
                                                        const int32_t *__restrict__ ri2,
                                                        const int32_t *__restrict__ rlv, int32_t *l, int64_t cap,
                                                        int tp, int32_t *levelg, int32_t *levelm, int32_t *cnt1,
                                                        int32_t *tlevelg, int32_t *tlevelm, int32_t *cnt2,
                                                        unsigned long long *nout) {
    __shared__ unsigned long long key[FIN_N];
    __shared__ int s_part[1024];
    int npad = 1;
    while (npad < n) npad <<= 1;
    for (int t = threadIdx.x; t < npad; t += blockDim.x)
        key[t] = t < n ? (((unsigned long long)(uint32_t)ri1[t] << 33) | ((unsigned long long)(uint32_t)ri2[t] << 1) |
                          (unsigned long long)(rlv[t] != 0))
                       : ~0ull;
    __syncthreads();
    for (int k = 2; k <= npad; k <<= 1)
        for (int jj = k >> 1; jj > 0; jj >>= 1) {
            for (int t = threadIdx.x; t < npad; t += blockDim.x) {
                const int p = t ^ jj;
                if (p > t) {
                    const bool up = (t & k) == 0;
                    const unsigned long long a = key[t], b = key[p];
                    if (up ? a > b : a < b) {
                        key[t] = b;
                        key[p] = a;
                    }
                }
            }
            __syncthreads();
        }
    // each thread owns 4 consecutive entries; keep the first of each (index1, index2)
    const int base = 4 * threadIdx.x;
    int keep[4], cntk = 0;
    for (int q = 0; q < 4; q++) {
        const int t = base + q;
        keep[q] = t < n && (t == 0 || (key[t] >> 1) != (key[t - 1] >> 1));
        cntk += keep[q];
    }
    s_part[threadIdx.x] = cntk;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        const int v = threadIdx.x >= (unsigned)off ? s_part[threadIdx.x - off] : 0;
        __syncthreads();
        s_part[threadIdx.x] += v;
        __syncthreads();
    }
    int o = s_part[threadIdx.x] - cntk;
    for (int q = 0; q < 4; q++) {
        if (!keep[q]) continue;
        const unsigned long long kk = key[base + q];
        const int i1 = (int)(kk >> 33), i2 = (int)((kk >> 1) & 0xffffffffull), lv = (int)(kk & 1ull);
        l[o] = i1;
        l[cap + o] = i2;
        l[2 * cap + o] = lv;
        l[3 * cap + o] = ST_ACTIVE;
        l[4 * cap + o] = 0;
        levelg[i1 - 1] = 0;
        levelm[i1 - 1] = 0;
        atomicAdd(&cnt1[i1 - 1], 1);
        if (!tp) {
            levelg[i2 - 1] = 0;
            levelm[i2 - 1] = 0;
            atomicAdd(&cnt1[i2 - 1], 1);
        } else {
            tlevelg[i2 - 1] = 0;
            tlevelm[i2 - 1] = 0;
            atomicAdd(&cnt2[i2 - 1], 1);
        }
        o++;
    }
    if (threadIdx.x == 1023) *nout = (unsigned long long)s_part[1023];
}

// symba_util_set_renc (symba_util.f90:245-267)
__device__ __forceinline__ double d_renc(double rhill, double rhscale, int scale) {
    double rshell_irec = 1.0;
    for (int k = 1; k <= scale; k++) rshell_irec = rshell_irec * RSHELL;
    return rhill * rhscale * rshell_irec;
}

// encounter_check_one (encounter_check.f90:573-621)
__device__ __forceinline__ void d_enc_one(double xr, double yr, double zr, double vxr, double vyr, double vzr,
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

// encounter_check_one for the recursion's list checks of the mixed path: the same test with
// FMA-contracted dot products and one reciprocal of v^2 for its two quotients (each FP64
// divide is a long sequence on GB300's narrow FP64 pipe, which sets the recursion's pace)
__device__ __forceinline__ void d_enc_one_fast(double xr, double yr, double zr, double vxr, double vyr, double vzr,
                                               double renc, double dt, int &lenc, int &lvdotr) {
    const double r2 = fma(zr, zr, fma(yr, yr, xr * xr));
    const double r2crit = renc * renc;
    double vdotr, r2min;
    if (r2 > r2crit) {
        vdotr = fma(vzr, zr, fma(vyr, yr, vxr * xr));
        if (vdotr > 0.0) {
            r2min = r2;
        } else {
            const double v2 = fma(vzr, vzr, fma(vyr, vyr, vxr * vxr));
            if (v2 <= VSMALL) {
                r2min = r2;
            } else {
                const double iv2 = 1.0 / v2;
                const double tmin = -vdotr * iv2;
                if (tmin < dt)
                    r2min = fma(-(vdotr * vdotr), iv2, r2);
                else
                    r2min = fma(v2, dt * dt, fma(2.0 * vdotr, dt, r2));
            }
        }
    } else {
        vdotr = -1.0;
        r2min = r2;
    }
    lvdotr = (vdotr < 0.0);
    lenc = lvdotr && (r2min <= r2crit);
}

// x**(-1.5) of the shell kick (symba_kick.f90:204,307): sqrt(x) and x*sqrt(x) as
// double-double pairs (Dekker's error-free transformations with fma residuals),
// then one Newton step on the reciprocal.  Within half an ulp except in rare
// near-tie cases, and the same bits as the host evaluation of the same sequence.
__device__ __forceinline__ double pow_m1p5(double x) {
    if (!(x > 0.0) || isinf(x)) return pow(x, -1.5);
    const double s = sqrt(x);
    const double rs = fma(-s, s, x);
    const double ds = rs / (2.0 * s);
    const double p = x * s;
    const double ep = fma(x, s, -p);
    const double ql = ep + x * ds;
    const double y0 = 1.0 / p;
    const double err = fma(-y0, p, 1.0) - y0 * ql;
    return fma(y0, err, y0);
}

// powi: square-and-multiply (gfortran's real**integer)
__device__ __forceinline__ double d_powi(double x, int m) {
    unsigned n = m < 0 ? -(unsigned)m : (unsigned)m;
    double y = (n % 2) ? x : 1.0;
    while (n >>= 1) {
        x = x * x;
        if (n % 2) y = y * x;
    }
    return m < 0 ? 1.0 / y : y;
}

// Encounter lists live in one int32 allocation per kind: [i1 | i2 | lvdotr | status | level],
// each `cap` long.
struct RecArgs {
    int npl, ntp;
    int64_t npp, ppcap, npt, ptcap;
    int32_t *pp, *pt;
    double *rh, *vb, *ah, *trh, *tvb, *tah;
    const double *Gm, *rhill, *radius;
    int32_t *status, *tstatus, *levelg, *levelm, *tlevelg, *tlevelm;
    double GMcb, rhscale, dt;
    uint8_t *lenc, *good, *good2;   // list-sized byte scratch
    double *terms;                  // 12 doubles per list entry
    int32_t *bpl, *btp;             // compact sets of bodies that appear in the lists
    int32_t *adj_end, *adj;         // per-body list entries (CSR: end offsets, entry indices)
    int32_t *mark_pl, *mark_tp;     // per-body marks, zero outside this kernel
    int32_t *out;                   // [0] status, [1] deepest level reached
    int lclose;                     // check for collisions at every level (param%lclose)
    int fast;                       // mixed path: fast FP64 forms of the drift and of r^-1.5
    int32_t *resume;                // REC_STATE ints: saved recursion stack of a paused step
    int32_t *pend;                  // set to 1 when the recursion pauses for a collision
    int64_t stage_bytes;            // dynamic shared memory of the launch (0: none)
};

// Saved stack of a recursion paused for a collision: [0] 1 when paused, [1] level,
// [2, 2 + MAXLEV) loop counters, [2 + MAXLEV, 2 + 2 MAXLEV) phases.
constexpr int MAXLEV = 48;
constexpr int REC_STATE = 2 + 2 * MAXLEV;

// Item index of this thread in the recursion kernel's block loops (blockDim a multiple
// of 128): items k, k+1, k+2, k+3 go to warps 0-3, one per SM sub-partition, then to the
// next lane, and items from 128 on to warps 4-7.  On GB300 a warp issues an FP64
// instruction at most every ~64 cycles, with one active lane or 32, and an SM at most
// one every ~19 cycles over all its warps (measured with FMA chains); the recursion's
// few pairs and bodies each run a long FP64 chain, so the fewest warps that still keep
// every sub-partition busy (four) run them fastest.  Spreading them over eight warps
// doubles the SM's FP64 issue load; packing them into one or two warps makes each warp
// carry the divergent paths (iteration counts, branch kinds) of many chains.
__device__ __forceinline__ int spread_tid() {
    const int w = threadIdx.x >> 5;
    return (w >> 2) * 128 + (threadIdx.x & 31) * 4 + (w & 3);
}

// symba_encounter_check_list_plpl / _pltp (symba_encounter_check.f90:90-235), whole block.
// rs_pow[k] = RSHELL^k formed as d_renc forms it (repeated products), k <= MAXLEV.
static __device__ void blk_list_check(const RecArgs &a, int irec, double dt, int *s_any, const double *rs_pow) {
    const int64_t npp = a.npp, npt = a.npt;
    for (int64_t k = spread_tid(); k < npp + npt; k += blockDim.x) {
        const bool isp = k < npp;
        const int64_t q = isp ? k : k - npp;
        int32_t *l = isp ? a.pp : a.pt;
        const int64_t cap = isp ? a.ppcap : a.ptcap;
        int32_t *i1 = l, *i2 = l + cap, *lv = l + 2 * cap, *st = l + 3 * cap, *lev = l + 4 * cap;
        uint8_t le_out = 0;
        if (st[q] == ST_ACTIVE && lev[q] == irec - 1) {
            const int i = i1[q] - 1, j = i2[q] - 1;
            double xr[3], vr[3];
            const double *rj = isp ? &a.rh[3 * j] : &a.trh[3 * j];
            const double *vj = isp ? &a.vb[3 * j] : &a.tvb[3 * j];
            for (int d = 0; d < 3; d++) {
                xr[d] = rj[d] - a.rh[3 * i + d];
                vr[d] = vj[d] - a.vb[3 * i + d];
            }
            const double renci = a.rhill[i] * a.rhscale * rs_pow[irec];  // d_renc(rhill_i, rhscale, irec)
            const double rcrit = isp ? renci + a.rhill[j] * a.rhscale * rs_pow[irec] : renci;
            int le, lvd;
            if (a.fast)
                d_enc_one_fast(xr[0], xr[1], xr[2], vr[0], vr[1], vr[2], rcrit, dt, le, lvd);
            else
                d_enc_one(xr[0], xr[1], xr[2], vr[0], vr[1], vr[2], rcrit, dt, le, lvd);
            lv[q] = lvd;
            if (le) {
                const double rs = isp ? a.radius[i] + a.radius[j] : a.radius[i];
                const double rlim2 = isp ? rs * rs : a.radius[i] * a.radius[i];
                const double rji2 = xr[0] * xr[0] + xr[1] * xr[1] + xr[2] * xr[2];
                le = rji2 > rlim2;
            }
            le_out = (uint8_t)le;
        }
        a.lenc[k] = le_out;
    }
    __syncthreads();
    for (int64_t k = spread_tid(); k < npp + npt; k += blockDim.x) {
        if (!a.lenc[k]) continue;
        *s_any = 1;
        const bool isp = k < npp;
        const int64_t q = isp ? k : k - npp;
        int32_t *l = isp ? a.pp : a.pt;
        const int64_t cap = isp ? a.ppcap : a.ptcap;
        const int i = l[q] - 1, j = l[cap + q] - 1;
        a.levelg[i] = irec;
        atomicMax(&a.levelm[i], irec);
        if (isp) {
            a.levelg[j] = irec;
            atomicMax(&a.levelm[j], irec);
        } else {
            a.tlevelg[j] = irec;
            atomicMax(&a.tlevelm[j], irec);
        }
        l[4 * cap + q] = irec;
    }
    __syncthreads();
}

// One kick phase of symba_step_recur_system (symba_step.f90:214-219 / 232-237): the +1
// kicks of both lists (symba_kick_list_plpl / _pltp, symba_kick.f90:126-340) and, below
// level 0 (both), the -1 kicks, whole block.  The per-pair factors (sqrt, divide, the
// shell polynomial) depend only on positions, so every pair is evaluated in parallel into
// `terms`, for both signs in one pass: the two signs differ only in the shell radius
// (irecl = irec for +1, irec - 1 for -1), so the displacement, r^2, r, r^-3 and (FP64
// path) r^-1.5 are formed once with the reference's operations and shared.  The
// additions are then made by one thread per body, which walks its own entries (the
// adjacency built at entry to the recursion, in increasing list order) and keeps the two
// signs' sums apart; the +1 velocity kick is applied before the -1 kick, so each body
// receives exactly the reference's additions in the reference's order, while GB300's
// narrow FP64 pipe sees one instruction stream for all bodies instead of one serial
// stream per pair.  A body that sits in several pairs gets its velocity kicked once per
// sign with its full acceleration, as in the reference (its later pairs add zero).
// good[k] (+1) and good2[k] (-1): 0 not kicked, 1 kicked, 2 zeroed then skipped
// (r^2 < rim1).  terms: 12 doubles per entry, the +1 pair terms then the -1 pair terms.
// The reference's lmask refresh at entry is kept by the step loop instead (lmask ==
// status /= INACTIVE wherever the recursion runs).
// pw[m] = d_powi(RSHELL, m), m <= 2 MAXLEV.
static __device__ void blk_kick_lists(const RecArgs &a, int nbpl, int nbtp, double dt, int irec, bool both,
                                      const double *pw) {
    const int64_t npp = a.npp, npt = a.npt;
    if (npp + npt == 0) return;
    const int irm1 = irec - 1;
    const double rs2 = a.rhscale * a.rhscale;
    const double shell_p = pw[2 * irec], shell_m = pw[2 * (irec - 1)];
    const int32_t *pi1 = a.pp, *pi2 = a.pp + a.ppcap, *pst = a.pp + 3 * a.ppcap;
    const int32_t *ti1 = a.pt, *ti2 = a.pt + a.ptcap, *tst = a.pt + 3 * a.ptcap;
    const bool do_pp = a.npl > 0, do_pt = a.npl > 0 && a.ntp > 0;
    // good flags and per-pair terms of both signs; three items per pair, one per vector
    // component c (each forms the pair's factors and writes only its component's terms)
    for (int64_t kc = spread_tid(); kc < 3 * (npp + npt); kc += blockDim.x) {
        const int64_t k = kc / 3;
        const int c = (int)(kc - 3 * k);
        const bool isp = k < npp;
        const int64_t q = isp ? k : k - npp;
        const int i = (isp ? pi1 : ti1)[q] - 1, j = (isp ? pi2 : ti2)[q] - 1;
        bool g;
        if (isp)
            g = do_pp && (pst[q] == ST_ACTIVE) && (a.levelg[i] >= irm1) && (a.levelg[j] >= irm1);
        else
            g = do_pt && (tst[q] == ST_ACTIVE) && (a.levelg[i] >= irm1) && (a.tlevelg[j] >= irm1);
        if (!g) {
            if (c == 0) {
                a.good[k] = 0;
                a.good2[k] = 0;
            }
            continue;
        }
        double base;
        if (isp) {
            const double rhs = a.rhill[i] + a.rhill[j];
            base = (rhs * rhs) * rs2;
        } else {
            base = (a.rhill[i] * a.rhill[i]) * rs2;
        }
        const double ri_p = base * shell_p, ri_m = base * shell_m;
        const double *rj = isp ? &a.rh[3 * j] : &a.trh[3 * j];
        double dx[3];
        for (int d = 0; d < 3; d++) dx[d] = rj[d] - a.rh[3 * i + d];
        const double r2 = a.fast ? fma(dx[2], dx[2], fma(dx[1], dx[1], dx[0] * dx[0]))
                                 : dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
        const bool kp = !(r2 < ri_p * (RSHELL * RSHELL));
        const bool km = both && !(r2 < ri_m * (RSHELL * RSHELL));
        if (c == 0) {
            a.good[k] = kp ? 1 : 2;
            a.good2[k] = both ? (km ? 1 : 2) : 0;
        }
        if (!kp && !km) continue;
        const bool shp = kp && r2 < ri_p, shm = km && r2 < ri_m;
        // FP64 path: IEEE square root and divide, and the correctly rounded r^-1.5 shared
        // with the oracle; mixed path: r and r^-3 from one reciprocal square root
        double r, ir3;
        if (a.fast) {
            const double y = rsqrt(r2);
            r = r2 * y;
            ir3 = (y * y) * y;
        } else {
            r = sqrt(r2);
            ir3 = 1.0 / (r2 * r);
        }
        double p = ir3;
        if (!a.fast && (shp || shm)) p = pow_m1p5(r2);
        auto shell = [&](double ri) {
            // rr = (sqrt(ri) - r) / (sqrt(ri) (1 - RSHELL)); mixed path as (1 - r / sqrt(ri)) / (1 - RSHELL)
            if (a.fast) {  // 1 - 3 rr^2 + 2 rr^3 as 1 + rr^2 (2 rr - 3)
                const double rr = fma(-r, rsqrt(ri), 1.0) * (1.0 / (1.0 - RSHELL));
                return p * fma(rr * rr, fma(2.0, rr, -3.0), 1.0);
            }
            const double rr = (sqrt(ri) - r) / (sqrt(ri) * (1.0 - RSHELL));
            return p * (1.0 - 3.0 * (rr * rr) + 2.0 * (rr * rr * rr));
        };
        double *t = &a.terms[12 * k];
        const double dc = c == 0 ? dx[0] : (c == 1 ? dx[1] : dx[2]);
        for (int sg = 0; sg < 2; sg++) {
            if (!(sg == 0 ? kp : km)) continue;
            const bool sh = sg == 0 ? shp : shm;
            const double fac = sh ? shell(sg == 0 ? ri_p : ri_m) : ir3;
            double *ts = t + 6 * sg;
            const double faci = fac * a.Gm[i];
            if (isp) {
                const double facj = fac * a.Gm[j];
                ts[c] = facj * dc;
                ts[3 + c] = faci * dc;
            } else {
                ts[c] = faci * dc;
            }
        }
    }
    __syncthreads();
    // ordered per-body accumulation and the velocity kicks, +1 then -1; three items per body,
    // one per vector component (each component's additions in list order, as one thread for
    // all three would make them)
    for (int bc = spread_tid(); bc < 3 * (nbpl + nbtp); bc += blockDim.x) {
        const int b = bc / 3, c = bc - 3 * b;
        const bool isp = b < nbpl;
        const int body = isp ? a.bpl[b] : a.btp[b - nbpl];
        bool zeroed[2] = {false, false}, kicked[2] = {false, false};
        double ac[2] = {0.0, 0.0};
        const int e0 = b == 0 ? 0 : a.adj_end[b - 1], e1 = a.adj_end[b];
        for (int e = e0; e < e1; e++) {
            const int k = a.adj[e];
            // pl-pl entry: + its first three terms as index1, - the last three as index2;
            // pl-tp entry (tp side): - its first three terms
            const int off = (isp && pi1[k] - 1 != body) ? 3 : 0;
            const bool sub = !isp || off == 3;
            for (int sg = 0; sg < 2; sg++) {
                const uint8_t g = sg == 0 ? a.good[k] : a.good2[k];
                if (g == 0) continue;
                zeroed[sg] = true;
                if (g != 1) continue;
                kicked[sg] = true;
                const double tc = a.terms[12 * k + 6 * sg + off + c];
                ac[sg] = sub ? ac[sg] - tc : ac[sg] + tc;
            }
        }
        double *v = isp ? &a.vb[3 * body + c] : &a.tvb[3 * body + c];
        double *acc = isp ? &a.ah[3 * body + c] : &a.tah[3 * body + c];
        for (int sg = 0; sg < 2; sg++) {
            if (!zeroed[sg]) continue;
            const double sdt = sg == 0 ? dt : -dt;
            if (kicked[sg]) *v = a.fast ? fma(sdt, ac[sg], *v) : *v + sdt * ac[sg];
            *acc = 0.0;
        }
    }
    __syncthreads();
}

// symba_drift_pl / _tp at level irec (symba_drift.f90:14-61) over the bodies that
// appear in the lists (every other body has levelg == -1 inside the recursion).
static __device__ void blk_drift(const RecArgs &a, int nbpl, int nbtp, int irec, double dt, double inv_gm) {
    for (int b = spread_tid(); b < nbpl + nbtp; b += blockDim.x) {
        const bool isp = b < nbpl;
        const int i = isp ? a.bpl[b] : a.btp[b - nbpl];
        const int32_t *lev = isp ? a.levelg : a.tlevelg;
        int32_t *st = isp ? a.status : a.tstatus;
        if (lev[i] != irec || st[i] == ST_INACTIVE) continue;
        double *x = isp ? &a.rh[3 * i] : &a.trh[3 * i];
        double *v = isp ? &a.vb[3 * i] : &a.tvb[3 * i];
        double rx = x[0], ry = x[1], rz = x[2], vx = v[0], vy = v[1], vz = v[2];
        const int fl = a.fast ? d_drift_one_fast(a.GMcb, rx, ry, rz, vx, vy, vz, dt, inv_gm)
                              : d_drift_one(a.GMcb, rx, ry, rz, vx, vy, vz, dt);
        x[0] = rx;
        x[1] = ry;
        x[2] = rz;
        v[0] = vx;
        v[1] = vy;
        v[2] = vz;
        if (fl != 0) st[i] = ST_DISCARDED_DRIFTERR;
    }
    __syncthreads();
}

// symba_step_set_recur_levels_system (symba_step.f90:118-160)
static __device__ void blk_set_recur_levels(const RecArgs &a, int nbpl, int nbtp, int ireci) {
    const int irecp = ireci + 1;
    for (int b = spread_tid(); b < nbpl + nbtp; b += blockDim.x) {
        int32_t *lev = b < nbpl ? &a.levelg[a.bpl[b]] : &a.tlevelg[a.btp[b - nbpl]];
        if (*lev == irecp) *lev = ireci;
    }
    for (int64_t k = threadIdx.x; k < a.npp + a.npt; k += blockDim.x) {
        int32_t *lev = k < a.npp ? &a.pp[4 * a.ppcap + k] : &a.pt[4 * a.ptcap + (k - a.npp)];
        if (*lev == irecp) *lev = ireci;
    }
    __syncthreads();
}

// collision_check_plpl / _pltp (src/collision/collision_check.f90:60-271) for the pairs of
// one system at recursion level irec: ACTIVE pairs whose pl (pl-pl: index1) or tp (pl-tp:
// index2) sits at level >= irec are tested; a colliding pair's status becomes COLLIDED
// and *s_coll is set.  The host resolves the collisions (merge, tp discard).
static __device__ void blk_collision_check(const RecArgs &a, int irec, double dt, int *s_coll) {
    for (int64_t k = spread_tid(); k < a.npp + a.npt; k += blockDim.x) {
        const bool isp = k < a.npp;
        const int64_t q = isp ? k : k - a.npp;
        int32_t *l = isp ? a.pp : a.pt;
        const int64_t cap = isp ? a.ppcap : a.ptcap;
        int32_t *st = l + 3 * cap;
        if (st[q] != ST_ACTIVE) continue;
        const int i = l[q] - 1, j = l[cap + q] - 1;
        if ((isp ? a.levelg[i] : a.tlevelg[j]) < irec) continue;
        const double *rj = isp ? &a.rh[3 * j] : &a.trh[3 * j];
        const double *vj = isp ? &a.vb[3 * j] : &a.tvb[3 * j];
        const double xr = a.rh[3 * i] - rj[0], yr = a.rh[3 * i + 1] - rj[1], zr = a.rh[3 * i + 2] - rj[2];
        const double vxr = a.vb[3 * i] - vj[0], vyr = a.vb[3 * i + 1] - vj[1], vzr = a.vb[3 * i + 2] - vj[2];
        const double Gmtot = isp ? a.Gm[i] + a.Gm[j] : a.Gm[i];
        const double rlim = isp ? a.radius[i] + a.radius[j] : a.radius[i];
        if (d_collision_one(xr, yr, zr, vxr, vyr, vzr, Gmtot, rlim, dt, l[2 * cap + q] != 0)) {
            st[q] = ST_COLLIDED;
            *s_coll = 1;
        }
    }
    __syncthreads();
}

// ---- per-system sums of the mixed path over chunks of every system
// A block-per-system sum leaves each system on one SM, and these sums are FP64 work on
// GB300's narrow FP64 pipe (an SM issues about one FP64 warp instruction per 19 cycles);
// the mixed path instead forms partial sums over chunks of bodies of every system (grid
// over all chunks: CHUNK bodies per chunk in ensembles, CHUNK_ONE for a single system), then
// each chunk adds its system's partials in chunk order and applies the result to its own
// bodies.  The order is fixed, so results are deterministic.
constexpr int CHUNK = 256, CHUNK_ONE = 128, CHUNK_T = 64;  // bodies per chunk, threads per chunk block
enum { SUM_VH2VB = 0, SUM_LIN = 1, SUM_VB2VH = 2 };

// chunk: (system, first body, bodies, unused); out: 4 doubles per chunk (sum of weights
// for SUM_VH2VB, then the three momentum components)
template <int MODE>
__global__ void __launch_bounds__(CHUNK_T) k_chunk_sums(int nchunks, const int4 *__restrict__ chunks,
                                                       const int32_t *__restrict__ lfirst,
                                                       const double *__restrict__ Gm, const double *__restrict__ v,
                                                       const int32_t *__restrict__ mask, double *__restrict__ out) {
    const int c = blockIdx.x;
    const int4 ch = chunks[c];
    if (MODE == SUM_VH2VB && lfirst && !lfirst[ch.x]) return;
    double w = 0.0, x = 0.0, y = 0.0, z = 0.0;
    for (int k = threadIdx.x; k < ch.z; k += CHUNK_T) {
        const int i = ch.y + k;
        bool on = true;
        if (MODE == SUM_LIN) on = mask[i] != 0;
        if (MODE == SUM_VB2VH) on = mask[i] != ST_INACTIVE;
        if (!on) continue;
        const double g = Gm[i];
        w += g;
        x = fma(g, v[3 * i + 0], x);
        y = fma(g, v[3 * i + 1], y);
        z = fma(g, v[3 * i + 2], z);
    }
    __shared__ double sh[CHUNK_T / 32][4];
    for (int off = 16; off > 0; off >>= 1) {
        if (MODE == SUM_VH2VB) w += __shfl_down_sync(0xffffffffu, w, off);
        x += __shfl_down_sync(0xffffffffu, x, off);
        y += __shfl_down_sync(0xffffffffu, y, off);
        z += __shfl_down_sync(0xffffffffu, z, off);
    }
    const int wp = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        sh[wp][0] = w;
        sh[wp][1] = x;
        sh[wp][2] = y;
        sh[wp][3] = z;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double t = 0.0;
        for (int q = 0; q < CHUNK_T / 32; q++) t += sh[q][threadIdx.x];
        out[4 * c + threadIdx.x] = t;
    }
}

// The system's chunk partials added in chunk order, then applied to this chunk's bodies:
// SUM_VH2VB: vb = vh + c, c = -sum(Gm vh) / (GMcb + sum Gm) (swiftest_util_coord_vh2vb_pl);
// SUM_LIN: pt = sum(Gm vb) / GMcb, rh += pt dt (helio_drift_linear_pl);
// SUM_VB2VH: c = -sum(Gm vb) / GMcb, vh = vb - c (swiftest_util_coord_vb2vh_pl).
// GMcb: per-system central-body masses, or nullptr for the single value GMcb0.
// The system's first chunk records the result in the central-body record.
template <int MODE>
__global__ void __launch_bounds__(CHUNK_T) k_chunk_apply(const int4 *__restrict__ chunks,
                                                        const int2 *__restrict__ sys_chunks,
                                                        const int32_t *__restrict__ lfirst,
                                                        const double *__restrict__ part,
                                                        const double *__restrict__ GMcb, double GMcb0,
                                                        const int32_t *__restrict__ lmask, const double *vin,
                                                        double *vout, double *rh, double dt, double *dcb, int slot) {
    const int c = blockIdx.x;
    const int4 ch = chunks[c];
    const int s = ch.x;
    if (MODE == SUM_VH2VB && lfirst && !lfirst[s]) return;
    __shared__ double tot[4];
    if (threadIdx.x < 4) {
        const int2 r = sys_chunks[s];
        double t = 0.0;
        for (int q = r.x; q < r.x + r.y; q++) t += part[4 * q + threadIdx.x];
        tot[threadIdx.x] = t;
    }
    __syncthreads();
    double cx, cy, cz;
    const double gmcb = GMcb ? GMcb[s] : GMcb0;
    if (MODE == SUM_VH2VB) {
        const double f = -1.0 / (gmcb + tot[0]);
        cx = tot[1] * f;
        cy = tot[2] * f;
        cz = tot[3] * f;
    } else {
        const double f = (MODE == SUM_LIN ? 1.0 : -1.0) / gmcb;
        cx = tot[1] * f;
        cy = tot[2] * f;
        cz = tot[3] * f;
    }
    if (ch.w == 0 && threadIdx.x == 0) {
        double *d = dcb + CB_N * s + (MODE == SUM_LIN ? slot : CB_VB);
        d[0] = cx;
        d[1] = cy;
        d[2] = cz;
    }
    for (int k = threadIdx.x; k < ch.z; k += CHUNK_T) {
        const int i = ch.y + k;
        if (MODE == SUM_VH2VB) {
            vout[3 * i + 0] = vin[3 * i + 0] + cx;
            vout[3 * i + 1] = vin[3 * i + 1] + cy;
            vout[3 * i + 2] = vin[3 * i + 2] + cz;
        } else if (MODE == SUM_LIN) {
            if (!lmask[i]) continue;
            rh[3 * i + 0] = fma(cx, dt, rh[3 * i + 0]);
            rh[3 * i + 1] = fma(cy, dt, rh[3 * i + 1]);
            rh[3 * i + 2] = fma(cz, dt, rh[3 * i + 2]);
        } else {
            vout[3 * i + 0] = vin[3 * i + 0] - cx;
            vout[3 * i + 1] = vin[3 * i + 1] - cy;
            vout[3 * i + 2] = vin[3 * i + 2] - cz;
        }
    }
}

constexpr int RECT = 256;  // threads of the recursion kernel

// In-place exclusive prefix sum of v[0, n) by the whole block (blockDim a multiple of 32,
// at most 1024 threads).
static __device__ void blk_exclusive_scan(int32_t *v, int n) {
    __shared__ int32_t s_w[32], s_carry;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int base = 0; base < n; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const int own = i < n ? v[i] : 0;
        int x = own;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_w[w] = x;
        __syncthreads();
        if (w == 0) {
            int t = lane < nw ? s_w[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= o) t += y;
            }
            if (lane < nw) s_w[lane] = t;
        }
        __syncthreads();
        const int carry = s_carry;
        if (i < n) v[i] = x - own + (w > 0 ? s_w[w - 1] : 0) + carry;
        __syncthreads();
        if (threadIdx.x == 0) s_carry = carry + s_w[nw - 1];
        __syncthreads();
    }
}

// Per-body adjacency of the encounter lists, built once per recursion launch: body slot b
// (bpl slots first, then btp) owns entries adj[adj_end[b-1], adj_end[b]) (from 0 for b = 0),
// the pl-pl entries naming a bpl body or the pl-tp entries naming a btp body, as combined
// list indices (pl-tp entry q is npp + q) in increasing order.  The kick's per-body walk
// then visits only the body's own entries, in the order the reference adds them.  On
// return mark_pl / mark_tp hold slot + 1 of each listed body (cleared at kernel exit).
static __device__ void blk_build_adjacency(const RecArgs &a, int nbpl, int nbtp) {
    const int nb = nbpl + nbtp;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
        if (b < nbpl) a.mark_pl[a.bpl[b]] = b + 1;
        else a.mark_tp[a.btp[b - nbpl]] = b + 1;
        a.adj_end[b] = 0;
    }
    __syncthreads();
    // entry counts per slot
    for (int64_t k = threadIdx.x; k < a.npp + a.npt; k += blockDim.x) {
        if (k < a.npp) {
            atomicAdd(&a.adj_end[a.mark_pl[a.pp[k] - 1] - 1], 1);
            atomicAdd(&a.adj_end[a.mark_pl[a.pp[a.ppcap + k] - 1] - 1], 1);
        } else {
            atomicAdd(&a.adj_end[a.mark_tp[a.pt[a.ptcap + (k - a.npp)] - 1] - 1], 1);
        }
    }
    __syncthreads();
    blk_exclusive_scan(a.adj_end, nb);
    // fill: each append advances the slot's start offset, which ends at the slot's end
    for (int64_t k = threadIdx.x; k < a.npp + a.npt; k += blockDim.x) {
        if (k < a.npp) {
            a.adj[atomicAdd(&a.adj_end[a.mark_pl[a.pp[k] - 1] - 1], 1)] = (int32_t)k;
            a.adj[atomicAdd(&a.adj_end[a.mark_pl[a.pp[a.ppcap + k] - 1] - 1], 1)] = (int32_t)k;
        } else {
            a.adj[atomicAdd(&a.adj_end[a.mark_tp[a.pt[a.ptcap + (k - a.npp)] - 1] - 1], 1)] = (int32_t)k;
        }
    }
    __syncthreads();
    // the atomics fill in any order: sort each slot's entries (few per body)
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
        const int e0 = b == 0 ? 0 : a.adj_end[b - 1], e1 = a.adj_end[b];
        for (int e = e0 + 1; e < e1; e++) {
            const int32_t v = a.adj[e];
            int f = e - 1;
            while (f >= e0 && a.adj[f] > v) {
                a.adj[f + 1] = a.adj[f];
                f--;
            }
            a.adj[f + 1] = v;
        }
    }
    __syncthreads();
}

// ---- the recursion's state staged in shared memory
// Every phase of a sub-step is a short FP64 chain preceded by dependent global loads (list
// entry -> body index -> position); on GB300 each L2 round trip costs hundreds of cycles on
// that chain.  When the lists fit, the listed bodies (by slot) and the list entries are
// copied into the block's dynamic shared memory once per launch, the phases below work
// there with the same arithmetic as the global-memory phases above, and the state is
// written back at the end (or at a pause for a collision).
struct RecStage {
    double *r, *v;                 // per slot: position, velocity (3 each)
    double *gm, *rhill, *rad;      // per slot: G*m, Hill radius, radius (0 for test particles)
    double *terms;                 // 12 per entry
    int32_t *lev, *st, *gidx;      // per slot: levelg / tlevelg, status / tstatus, global index
    int32_t *s1, *s2;              // per entry: slots of index1 and index2
    int32_t *est, *elev, *elv;     // per entry: status, level, lvdotr
    int32_t *adj_end, *adj;        // the adjacency of blk_build_adjacency
    uint8_t *lenc, *good, *good2;  // per entry
};
// Largest stage of a single-system launch, and of each block of an ensemble launch (every
// block gets the same size; systems whose lists do not fit use the global arrays).
constexpr size_t REC_STAGE_MAX = 160 * 1024, REC_STAGE_ENS = 64 * 1024;
// Bytes of the stage for npp pl-pl and npt pl-tp entries: at most two bodies per entry
// (a pl-tp entry names one pl and one tp), and 2 npp + npt adjacency entries.
__host__ __device__ inline size_t rec_stage_bytes(int64_t npp, int64_t npt) {
    const int64_t n = npp + npt, nb = 2 * n;
    return (size_t)(9 * nb + 12 * n) * 8 + (size_t)(4 * nb + 5 * n + 2 * npp + npt) * 4 + (size_t)(3 * n + 16);
}
static __device__ RecStage rec_stage_carve(void *base, int64_t npp, int64_t npt) {
    const int64_t n = npp + npt, nb = 2 * n;
    RecStage S;
    double *d = (double *)base;
    S.r = d;
    S.v = d + 3 * nb;
    S.gm = d + 6 * nb;
    S.rhill = d + 7 * nb;
    S.rad = d + 8 * nb;
    S.terms = d + 9 * nb;
    int32_t *i = (int32_t *)(S.terms + 12 * n);
    S.lev = i;
    S.st = i + nb;
    S.gidx = i + 2 * nb;
    S.adj_end = i + 3 * nb;
    S.s1 = i + 4 * nb;
    S.s2 = S.s1 + n;
    S.est = S.s2 + n;
    S.elev = S.est + n;
    S.elv = S.elev + n;
    S.adj = S.elv + n;
    uint8_t *b = (uint8_t *)(S.adj + 2 * npp + npt);
    S.lenc = b;
    S.good = b + n;
    S.good2 = b + 2 * n;
    return S;
}
// Copy the listed bodies and the list entries in (after blk_build_adjacency: mark_pl /
// mark_tp hold slot + 1), whole block.
static __device__ void stg_load(const RecArgs &a, const RecStage &S, int nbpl, int nbtp) {
    const int nb = nbpl + nbtp;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
        const bool isp = b < nbpl;
        const int g = isp ? a.bpl[b] : a.btp[b - nbpl];
        const double *x = isp ? &a.rh[3 * g] : &a.trh[3 * g];
        const double *w = isp ? &a.vb[3 * g] : &a.tvb[3 * g];
        for (int d = 0; d < 3; d++) {
            S.r[3 * b + d] = x[d];
            S.v[3 * b + d] = w[d];
        }
        S.gm[b] = isp ? a.Gm[g] : 0.0;
        S.rhill[b] = isp ? a.rhill[g] : 0.0;
        S.rad[b] = isp ? a.radius[g] : 0.0;
        S.lev[b] = isp ? a.levelg[g] : a.tlevelg[g];
        S.st[b] = isp ? a.status[g] : a.tstatus[g];
        S.gidx[b] = g;
        S.adj_end[b] = a.adj_end[b];
    }
    const int64_t n = a.npp + a.npt;
    for (int64_t k = threadIdx.x; k < n; k += blockDim.x) {
        const bool isp = k < a.npp;
        const int64_t q = isp ? k : k - a.npp;
        const int32_t *l = isp ? a.pp : a.pt;
        const int64_t cap = isp ? a.ppcap : a.ptcap;
        const int i = l[q] - 1, j = l[cap + q] - 1;
        S.s1[k] = a.mark_pl[i] - 1;
        S.s2[k] = isp ? a.mark_pl[j] - 1 : a.mark_tp[j] - 1;
        S.elv[k] = l[2 * cap + q];
        S.est[k] = l[3 * cap + q];
        S.elev[k] = l[4 * cap + q];
    }
    for (int64_t e = threadIdx.x; e < 2 * a.npp + a.npt; e += blockDim.x) S.adj[e] = a.adj[e];
    __syncthreads();
}
// Write the staged state back to the global arrays, whole block.
static __device__ void stg_store(const RecArgs &a, const RecStage &S, int nbpl, int nbtp) {
    __syncthreads();
    const int nb = nbpl + nbtp;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
        const bool isp = b < nbpl;
        const int g = S.gidx[b];
        double *x = isp ? &a.rh[3 * g] : &a.trh[3 * g];
        double *w = isp ? &a.vb[3 * g] : &a.tvb[3 * g];
        for (int d = 0; d < 3; d++) {
            x[d] = S.r[3 * b + d];
            w[d] = S.v[3 * b + d];
        }
        (isp ? a.levelg : a.tlevelg)[g] = S.lev[b];
        (isp ? a.status : a.tstatus)[g] = S.st[b];
    }
    const int64_t n = a.npp + a.npt;
    for (int64_t k = threadIdx.x; k < n; k += blockDim.x) {
        const bool isp = k < a.npp;
        const int64_t q = isp ? k : k - a.npp;
        int32_t *l = isp ? a.pp : a.pt;
        const int64_t cap = isp ? a.ppcap : a.ptcap;
        l[2 * cap + q] = S.elv[k];
        l[3 * cap + q] = S.est[k];
        l[4 * cap + q] = S.elev[k];
    }
    __syncthreads();
}
// blk_list_check on the stage
static __device__ void stg_list_check(const RecArgs &a, const RecStage &S, int irec, double dt, int *s_any,
                                      const double *rs_pow) {
    const int64_t npp = a.npp, n = a.npp + a.npt;
    for (int64_t k = spread_tid(); k < n; k += blockDim.x) {
        const bool isp = k < npp;
        uint8_t le_out = 0;
        if (S.est[k] == ST_ACTIVE && S.elev[k] == irec - 1) {
            const int b1 = S.s1[k], b2 = S.s2[k];
            double xr[3], vr[3];
            for (int d = 0; d < 3; d++) {
                xr[d] = S.r[3 * b2 + d] - S.r[3 * b1 + d];
                vr[d] = S.v[3 * b2 + d] - S.v[3 * b1 + d];
            }
            const double renci = S.rhill[b1] * a.rhscale * rs_pow[irec];  // d_renc(rhill_i, rhscale, irec)
            const double rcrit = isp ? renci + S.rhill[b2] * a.rhscale * rs_pow[irec] : renci;
            int le, lvd;
            if (a.fast)
                d_enc_one_fast(xr[0], xr[1], xr[2], vr[0], vr[1], vr[2], rcrit, dt, le, lvd);
            else
                d_enc_one(xr[0], xr[1], xr[2], vr[0], vr[1], vr[2], rcrit, dt, le, lvd);
            S.elv[k] = lvd;
            if (le) {
                const double rs = isp ? S.rad[b1] + S.rad[b2] : S.rad[b1];
                const double rlim2 = isp ? rs * rs : S.rad[b1] * S.rad[b1];
                const double rji2 = xr[0] * xr[0] + xr[1] * xr[1] + xr[2] * xr[2];
                le = rji2 > rlim2;
            }
            le_out = (uint8_t)le;
        }
        S.lenc[k] = le_out;
    }
    __syncthreads();
    for (int64_t k = spread_tid(); k < n; k += blockDim.x) {
        if (!S.lenc[k]) continue;
        *s_any = 1;
        const bool isp = k < npp;
        const int b1 = S.s1[k], b2 = S.s2[k];
        S.lev[b1] = irec;
        atomicMax(&a.levelm[S.gidx[b1]], irec);
        S.lev[b2] = irec;
        atomicMax(isp ? &a.levelm[S.gidx[b2]] : &a.tlevelm[S.gidx[b2]], irec);
        S.elev[k] = irec;
    }
    __syncthreads();
}
// blk_kick_lists on the stage (same pair terms, same per-body order)
static __device__ void stg_kick_lists(const RecArgs &a, const RecStage &S, int nbpl, int nbtp, double dt, int irec,
                                      bool both, const double *pw) {
    const int64_t npp = a.npp, n = a.npp + a.npt;
    if (n == 0) return;
    const int irm1 = irec - 1;
    const double rs2 = a.rhscale * a.rhscale;
    const double shell_p = pw[2 * irec], shell_m = pw[2 * (irec - 1)];
    const bool do_pp = a.npl > 0, do_pt = a.npl > 0 && a.ntp > 0;
    // three items per pair, one per vector component c: each forms the pair's factors (the
    // same instructions in every lane, which costs a warp no more FP64 issue than one lane)
    // and writes only its component's terms
    for (int64_t kc = spread_tid(); kc < 3 * n; kc += blockDim.x) {
        const int64_t k = kc / 3;
        const int c = (int)(kc - 3 * k);
        const bool isp = k < npp;
        const int b1 = S.s1[k], b2 = S.s2[k];
        const bool g = (isp ? do_pp : do_pt) && (S.est[k] == ST_ACTIVE) && (S.lev[b1] >= irm1) && (S.lev[b2] >= irm1);
        if (!g) {
            if (c == 0) {
                S.good[k] = 0;
                S.good2[k] = 0;
            }
            continue;
        }
        double base;
        if (isp) {
            const double rhs = S.rhill[b1] + S.rhill[b2];
            base = (rhs * rhs) * rs2;
        } else {
            base = (S.rhill[b1] * S.rhill[b1]) * rs2;
        }
        const double ri_p = base * shell_p, ri_m = base * shell_m;
        double dx[3];
        for (int d = 0; d < 3; d++) dx[d] = S.r[3 * b2 + d] - S.r[3 * b1 + d];
        const double r2 = a.fast ? fma(dx[2], dx[2], fma(dx[1], dx[1], dx[0] * dx[0]))
                                 : dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
        const bool kp = !(r2 < ri_p * (RSHELL * RSHELL));
        const bool km = both && !(r2 < ri_m * (RSHELL * RSHELL));
        if (c == 0) {
            S.good[k] = kp ? 1 : 2;
            S.good2[k] = both ? (km ? 1 : 2) : 0;
        }
        if (!kp && !km) continue;
        const bool shp = kp && r2 < ri_p, shm = km && r2 < ri_m;
        double r, ir3;
        if (a.fast) {
            const double y = rsqrt(r2);
            r = r2 * y;
            ir3 = (y * y) * y;
        } else {
            r = sqrt(r2);
            ir3 = 1.0 / (r2 * r);
        }
        double p = ir3;
        if (!a.fast && (shp || shm)) p = pow_m1p5(r2);
        auto shell = [&](double ri) {
            if (a.fast) {  // 1 - 3 rr^2 + 2 rr^3 as 1 + rr^2 (2 rr - 3)
                const double rr = fma(-r, rsqrt(ri), 1.0) * (1.0 / (1.0 - RSHELL));
                return p * fma(rr * rr, fma(2.0, rr, -3.0), 1.0);
            }
            const double rr = (sqrt(ri) - r) / (sqrt(ri) * (1.0 - RSHELL));
            return p * (1.0 - 3.0 * (rr * rr) + 2.0 * (rr * rr * rr));
        };
        double *t = &S.terms[12 * k];
        const double dc = c == 0 ? dx[0] : (c == 1 ? dx[1] : dx[2]);
        for (int sg = 0; sg < 2; sg++) {
            if (!(sg == 0 ? kp : km)) continue;
            const bool sh = sg == 0 ? shp : shm;
            const double fac = sh ? shell(sg == 0 ? ri_p : ri_m) : ir3;
            double *ts = t + 6 * sg;
            const double faci = fac * S.gm[b1];
            if (isp) {
                const double facj = fac * S.gm[b2];
                ts[c] = facj * dc;
                ts[3 + c] = faci * dc;
            } else {
                ts[c] = faci * dc;
            }
        }
    }
    __syncthreads();
    // three items per body, one per vector component c: each adds its component of the
    // body's terms in list order (the same additions as one thread for all three, so the
    // same bits) and applies its component's velocity kicks
    for (int bc = spread_tid(); bc < 3 * (nbpl + nbtp); bc += blockDim.x) {
        const int b = bc / 3, c = bc - 3 * b;
        const bool isp = b < nbpl;
        bool zeroed[2] = {false, false}, kicked[2] = {false, false};
        double ac[2] = {0.0, 0.0};
        const int e0 = b == 0 ? 0 : S.adj_end[b - 1], e1 = S.adj_end[b];
        for (int e = e0; e < e1; e++) {
            const int k = S.adj[e];
            const int off = (isp && S.s1[k] != b) ? 3 : 0;
            const bool sub = !isp || off == 3;
            for (int sg = 0; sg < 2; sg++) {
                const uint8_t g = sg == 0 ? S.good[k] : S.good2[k];
                if (g == 0) continue;
                zeroed[sg] = true;
                if (g != 1) continue;
                kicked[sg] = true;
                const double tc = S.terms[12 * k + 6 * sg + off + c];
                ac[sg] = sub ? ac[sg] - tc : ac[sg] + tc;
            }
        }
        double *v = &S.v[3 * b + c];
        double *acc = isp ? &a.ah[3 * S.gidx[b] + c] : &a.tah[3 * S.gidx[b] + c];
        for (int sg = 0; sg < 2; sg++) {
            if (!zeroed[sg]) continue;
            const double sdt = sg == 0 ? dt : -dt;
            if (kicked[sg]) *v = a.fast ? fma(sdt, ac[sg], *v) : *v + sdt * ac[sg];
            *acc = 0.0;
        }
    }
    __syncthreads();
}
// blk_drift on the stage
static __device__ void stg_drift(const RecArgs &a, const RecStage &S, int nbpl, int nbtp, int irec, double dt,
                                 double inv_gm) {
    for (int b = spread_tid(); b < nbpl + nbtp; b += blockDim.x) {
        if (S.lev[b] != irec || S.st[b] == ST_INACTIVE) continue;
        double *x = &S.r[3 * b], *v = &S.v[3 * b];
        double rx = x[0], ry = x[1], rz = x[2], vx = v[0], vy = v[1], vz = v[2];
        const int fl = a.fast ? d_drift_one_fast(a.GMcb, rx, ry, rz, vx, vy, vz, dt, inv_gm)
                              : d_drift_one(a.GMcb, rx, ry, rz, vx, vy, vz, dt);
        x[0] = rx;
        x[1] = ry;
        x[2] = rz;
        v[0] = vx;
        v[1] = vy;
        v[2] = vz;
        if (fl != 0) S.st[b] = ST_DISCARDED_DRIFTERR;
    }
    __syncthreads();
}
// blk_set_recur_levels on the stage
static __device__ void stg_set_recur_levels(const RecArgs &a, const RecStage &S, int nbpl, int nbtp, int ireci) {
    const int irecp = ireci + 1;
    for (int b = spread_tid(); b < nbpl + nbtp; b += blockDim.x)
        if (S.lev[b] == irecp) S.lev[b] = ireci;
    for (int64_t k = threadIdx.x; k < a.npp + a.npt; k += blockDim.x)
        if (S.elev[k] == irecp) S.elev[k] = ireci;
    __syncthreads();
}
// blk_collision_check on the stage
static __device__ void stg_collision_check(const RecArgs &a, const RecStage &S, int irec, double dt, int *s_coll) {
    for (int64_t k = spread_tid(); k < a.npp + a.npt; k += blockDim.x) {
        if (S.est[k] != ST_ACTIVE) continue;
        const bool isp = k < a.npp;
        const int b1 = S.s1[k], b2 = S.s2[k];
        if ((isp ? S.lev[b1] : S.lev[b2]) < irec) continue;
        const double *ri = &S.r[3 * b1], *rj = &S.r[3 * b2], *vi = &S.v[3 * b1], *vj = &S.v[3 * b2];
        const double xr = ri[0] - rj[0], yr = ri[1] - rj[1], zr = ri[2] - rj[2];
        const double vxr = vi[0] - vj[0], vyr = vi[1] - vj[1], vzr = vi[2] - vj[2];
        const double Gmtot = isp ? S.gm[b1] + S.gm[b2] : S.gm[b1];
        const double rlim = isp ? S.rad[b1] + S.rad[b2] : S.rad[b1];
        if (d_collision_one(xr, yr, zr, vxr, vyr, vzr, Gmtot, rlim, dt, S.elv[k] != 0)) {
            S.est[k] = ST_COLLIDED;
            *s_coll = 1;
        }
    }
    __syncthreads();
}

// symba_step_recur_system (symba_step.f90:163-262) for the whole recursion tree of one
// step, started at level 0, in a single block: the reference's recursive calls become
// an explicit stack of (loop counter, phase) per level, and every per-level operation
// is a block-wide device function separated by barriers.  a.out[0] receives
// SWG_ERR_RECURSION if the step falls below machine precision (the caller zeroes it),
// a.out[1] the deepest level (atomicMax) and a.out[2] the sub-steps run (atomicAdd), so
// several blocks (systems of an ensemble) may share one out array.  STAGED: the listed
// bodies and the list entries live in `stage` (dynamic shared memory) during the launch.
template <bool STAGED>
static __device__ void blk_symba_recursion_t(const RecArgs &a, void *stage) {
    __shared__ int s_nbpl, s_nbtp, s_any;
    __shared__ int s_j[MAXLEV], s_phase[MAXLEV];
    // shell-radius powers, formed once per launch with the per-call algorithms (same bits):
    // s_pw[m] = d_powi(RSHELL, m) (the kick's shell radii), s_rs[k] = RSHELL^k by repeated
    // products (d_renc, the list check's encounter radii)
    __shared__ double s_pw[2 * MAXLEV + 2], s_rs[MAXLEV + 1];
    // each level's step dt / 3^k and the underflow test of symba_step.f90:196-201, formed
    // once per launch as the loop would form them (the FP64 divides are long on GB300)
    __shared__ double s_dtl[MAXLEV];
    __shared__ unsigned char s_under[MAXLEV];
    for (int m = threadIdx.x; m < 2 * MAXLEV + 2; m += blockDim.x) s_pw[m] = d_powi(RSHELL, m);
    for (int k = threadIdx.x; k < MAXLEV; k += blockDim.x) {
        double p3 = 1.0;
        for (int q = 0; q < k; q++) p3 *= 3.0;
        const double d = a.dt / p3;
        s_dtl[k] = d;
        s_under[k] = d / a.dt < 2.220446049250313e-16;
    }
    if (threadIdx.x == 0) {
        double p = 1.0;
        s_rs[0] = p;
        for (int k = 1; k <= MAXLEV; k++) {
            p = p * RSHELL;
            s_rs[k] = p;
        }
    }
    if (threadIdx.x == 0) s_nbpl = s_nbtp = 0;
    __syncthreads();
    // compact sets of bodies named in the lists
    for (int64_t k = threadIdx.x; k < a.npp + a.npt; k += blockDim.x) {
        const bool isp = k < a.npp;
        const int64_t q = isp ? k : k - a.npp;
        const int32_t *l = isp ? a.pp : a.pt;
        const int64_t cap = isp ? a.ppcap : a.ptcap;
        const int i = l[q] - 1, j = l[cap + q] - 1;
        if (atomicExch(&a.mark_pl[i], 1) == 0) a.bpl[atomicAdd(&s_nbpl, 1)] = i;
        if (isp) {
            if (atomicExch(&a.mark_pl[j], 1) == 0) a.bpl[atomicAdd(&s_nbpl, 1)] = j;
        } else {
            if (atomicExch(&a.mark_tp[j], 1) == 0) a.btp[atomicAdd(&s_nbtp, 1)] = j;
        }
    }
    __syncthreads();
    const int nbpl = s_nbpl, nbtp = s_nbtp;
    blk_build_adjacency(a, nbpl, nbtp);
    RecStage S{};
    if constexpr (STAGED) {
        S = rec_stage_carve(stage, a.npp, a.npt);
        stg_load(a, S, nbpl, nbtp);
    }
    int ireci = 0;
    const bool resumed = a.resume && a.resume[0] == 1;
    if (resumed) {  // continue a step paused after a collision check
        ireci = a.resume[1];
        for (int k = threadIdx.x; k <= ireci; k += blockDim.x) {
            s_j[k] = a.resume[2 + k];
            s_phase[k] = a.resume[2 + MAXLEV + k];
        }
    } else if (threadIdx.x == 0) {
        s_j[0] = 1;
        s_phase[0] = 0;
    }
    __syncthreads();
    int deepest = 0, substeps = 0;
    bool paused = false;
    const double inv_gm = 1.0 / a.GMcb;  // the fast drift's 1/mu, formed once
    for (;;) {
        const double dtl = s_dtl[ireci];
        const double dth = 0.5 * dtl;
        const int irecp = ireci + 1;
        const int nloops = ireci == 0 ? 1 : NTENC;
        if (s_phase[ireci] == 2) goto after_collision;  // resumed: collisions of this loop resolved
        if (s_phase[ireci] == 0) {
            if (s_j[ireci] > nloops) {
                if (ireci == 0) break;
                __syncthreads();
                ireci--;
                if (threadIdx.x == 0) s_phase[ireci] = 1;
                __syncthreads();
                continue;
            }
            if (s_under[ireci]) {
                if (threadIdx.x == 0) a.out[0] = SWG_ERR_RECURSION;
                break;
            }
            if (irecp > deepest) deepest = irecp;
            substeps++;
            if (threadIdx.x == 0) s_any = 0;
            __syncthreads();
            if constexpr (STAGED) {
                stg_list_check(a, S, irecp, dtl, &s_any, s_rs);
                stg_kick_lists(a, S, nbpl, nbtp, dth, irecp, ireci != 0, s_pw);
                stg_drift(a, S, nbpl, nbtp, ireci, dtl, inv_gm);
            } else {
                blk_list_check(a, irecp, dtl, &s_any, s_rs);
                blk_kick_lists(a, nbpl, nbtp, dth, irecp, ireci != 0, s_pw);
                blk_drift(a, nbpl, nbtp, ireci, dtl, inv_gm);
            }
            const int any = s_any;
            __syncthreads();
            if (any) {
                if (ireci + 1 >= MAXLEV) {
                    if (threadIdx.x == 0) a.out[0] = SWG_ERR_RECURSION;
                    break;
                }
                ireci++;
                if (threadIdx.x == 0) {
                    s_j[ireci] = 1;
                    s_phase[ireci] = 0;
                }
                __syncthreads();
                continue;
            }
        }
        // after the deeper levels (or none) for loop j of level ireci
        if constexpr (STAGED)
            stg_kick_lists(a, S, nbpl, nbtp, dth, irecp, ireci != 0, s_pw);
        else
            blk_kick_lists(a, nbpl, nbtp, dth, irecp, ireci != 0, s_pw);
        if (a.lclose) {
            if (threadIdx.x == 0) s_any = 0;
            __syncthreads();
            if constexpr (STAGED)
                stg_collision_check(a, S, ireci, dtl, &s_any);
            else
                blk_collision_check(a, ireci, dtl, &s_any);
            if (s_any) {  // pause: the host resolves the collisions, then resumes here
                if (threadIdx.x == 0) {
                    s_phase[ireci] = 2;
                    a.resume[0] = 1;
                    a.resume[1] = ireci;
                    for (int k = 0; k <= ireci; k++) {
                        a.resume[2 + k] = s_j[k];
                        a.resume[2 + MAXLEV + k] = s_phase[k];
                    }
                    *a.pend = 1;
                }
                paused = true;
                break;
            }
        }
    after_collision:
        if constexpr (STAGED)
            stg_set_recur_levels(a, S, nbpl, nbtp, ireci);
        else
            blk_set_recur_levels(a, nbpl, nbtp, ireci);
        if (threadIdx.x == 0) {
            s_j[ireci]++;
            s_phase[ireci] = 0;
        }
        __syncthreads();
    }
    __syncthreads();
    if constexpr (STAGED) stg_store(a, S, nbpl, nbtp);
    if (!paused && resumed && threadIdx.x == 0) a.resume[0] = 0;
    for (int b = threadIdx.x; b < nbpl; b += blockDim.x) a.mark_pl[a.bpl[b]] = 0;
    for (int b = threadIdx.x; b < nbtp; b += blockDim.x) a.mark_tp[a.btp[b]] = 0;
    if (threadIdx.x == 0) {
        atomicMax(&a.out[1], deepest);
        atomicAdd(&a.out[2], substeps);
    }
}

// The recursion of one system: staged in the launch's dynamic shared memory when its lists
// fit there (a.stage_bytes: that memory's size, 0 for none), else on the global arrays.
// Both forms take the same arithmetic in the same order, so they give the same bits.
static __device__ void blk_symba_recursion(const RecArgs &a) {
    extern __shared__ __align__(16) unsigned char rec_dyn[];
    if (a.stage_bytes > 0 && rec_stage_bytes(a.npp, a.npt) <= (size_t)a.stage_bytes)
        blk_symba_recursion_t<true>(a, rec_dyn);
    else
        blk_symba_recursion_t<false>(a, nullptr);
}

// ---- energy / momentum (swiftest_util.f90:1172-1401), masses as G*m
__device__ __forceinline__ double d_norm2s(double a, double b, double c) {
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
// Row i of the pairwise potential sum: sum over j > i of -Gm_i Gm_j / |rb_i - rb_j|,
// active bodies only, in ascending j (swiftest_util.f90:1294-1401).
__device__ __forceinline__ double d_energy_row(int i, int n, const double *rb, const double *Gm,
                                               const int32_t *status) {
    double row = 0.0;
    if (status[i] != ST_INACTIVE) {
        for (int j = i + 1; j < n; j++) {
            if (status[j] == ST_INACTIVE) continue;
            row = row + (-(Gm[i] * Gm[j]) / d_norm2s(rb[3 * i] - rb[3 * j], rb[3 * i + 1] - rb[3 * j + 1],
                                                    rb[3 * i + 2] - rb[3 * j + 2]));
        }
    }
    return row;
}
// Totals of swiftest_util_get_energy_and_momentum_system for one system, whole block of
// RB threads: writes the barycentric positions rb (needed by the potential rows) and
// out[9] = te, ke, pe, be, Lx, Ly, Lz, GMtot, te_helio (the total with the central-body
// potential taken at the heliocentric distance).  rows[] from an earlier pass.
static __device__ void blk_energy_final(int n, int whm, const double *rh, const double *vh, const double *vbin,
                                 const double *Gm, const double *radius, const int32_t *status, double GMcb,
                                 int lclose, const double *rows, double *rb, double *out, SumScratch &sh) {
    double cbvb[3];
    if (whm) {
        auto gm = [&](int i, double &x, double &y, double &z) -> unsigned char {
            x = Gm[i];
            y = z = 0.0;
            return 1;
        };
        const double Gmtot = GMcb + ordered_sum3(n, false, false, gm, 1.0, sh).x;
        auto t = [&](int i, double &x, double &y, double &z) -> unsigned char {
            x = Gm[i] * vh[3 * i];
            y = Gm[i] * vh[3 * i + 1];
            z = Gm[i] * vh[3 * i + 2];
            return 1;
        };
        const Sum3 c3 = ordered_sum3(n, false, false, t, -1.0, sh);
        cbvb[0] = c3.x / Gmtot;
        cbvb[1] = c3.y / Gmtot;
        cbvb[2] = c3.z / Gmtot;
    } else {
        auto t = [&](int i, double &x, double &y, double &z) -> unsigned char {
            x = Gm[i] * vbin[3 * i] / GMcb;
            y = Gm[i] * vbin[3 * i + 1] / GMcb;
            z = Gm[i] * vbin[3 * i + 2] / GMcb;
            return status[i] != ST_INACTIVE;
        };
        const Sum3 c3 = ordered_sum3(n, true, false, t, -1.0, sh);
        cbvb[0] = c3.x;
        cbvb[1] = c3.y;
        cbvb[2] = c3.z;
    }
    auto gact = [&](int i, double &x, double &y, double &z) -> unsigned char {
        x = Gm[i];
        y = z = 0.0;
        return status[i] != ST_INACTIVE;
    };
    const double gsum = ordered_sum3(n, false, false, gact, 1.0, sh).x;
    const double Gmtot = GMcb + gsum;
    auto xt = [&](int i, double &x, double &y, double &z) -> unsigned char {
        x = Gm[i] * rh[3 * i];
        y = Gm[i] * rh[3 * i + 1];
        z = Gm[i] * rh[3 * i + 2];
        return status[i] != ST_INACTIVE;
    };
    const Sum3 x3 = ordered_sum3(n, false, false, xt, 1.0, sh);
    const double cbrb[3] = {-x3.x / Gmtot, -x3.y / Gmtot, -x3.z / Gmtot};
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        for (int d = 0; d < 3; d++) rb[3 * i + d] = rh[3 * i + d] + cbrb[d];
    __syncthreads();
    auto vel = [&](int i, int d) { return whm ? vh[3 * i + d] + cbvb[d] : vbin[3 * i + d]; };
    auto Lt = [&](int i, double &x, double &y, double &z) -> unsigned char {
        const double *r = &rb[3 * i];
        const double v0 = vel(i, 0), v1 = vel(i, 1), v2 = vel(i, 2);
        x = Gm[i] * (r[1] * v2 - r[2] * v1);
        y = Gm[i] * (r[2] * v0 - r[0] * v2);
        z = Gm[i] * (r[0] * v1 - r[1] * v0);
        return status[i] != ST_INACTIVE;
    };
    const Sum3 Lp = ordered_sum3(n, false, false, Lt, 1.0, sh);
    auto kt = [&](int i, double &x, double &y, double &z) -> unsigned char {
        const double v0 = vel(i, 0), v1 = vel(i, 1), v2 = vel(i, 2);
        x = Gm[i] * (v0 * v0 + v1 * v1 + v2 * v2);
        y = -GMcb * Gm[i] / d_norm2s(rb[3 * i], rb[3 * i + 1], rb[3 * i + 2]);
        z = -GMcb * Gm[i] / d_norm2s(rh[3 * i], rh[3 * i + 1], rh[3 * i + 2]);
        return status[i] != ST_INACTIVE;
    };
    const Sum3 kp = ordered_sum3(n, false, false, kt, 1.0, sh);
    auto bt = [&](int i, double &x, double &y, double &z) -> unsigned char {
        const bool act = status[i] != ST_INACTIVE;  // a removed body has no radius: no binding term
        x = lclose && act ? -3.0 * Gm[i] * Gm[i] / (5.0 * radius[i]) : 0.0;
        y = rows[i];
        z = 0.0;
        return act;
    };
    const Sum3 bp = ordered_sum3(n, false, false, bt, 1.0, sh);
    if (threadIdx.x == 0) {
        const double mcb = GMcb;
        const double kecb = mcb * (cbvb[0] * cbvb[0] + cbvb[1] * cbvb[1] + cbvb[2] * cbvb[2]);
        const double L[3] = {mcb * (cbrb[1] * cbvb[2] - cbrb[2] * cbvb[1]), mcb * (cbrb[2] * cbvb[0] - cbrb[0] * cbvb[2]),
                             mcb * (cbrb[0] * cbvb[1] - cbrb[1] * cbvb[0])};
        const double pe_pairs = bp.y;
        const double pe = pe_pairs + kp.y;
        const double be = bp.x;
        const double ke = 0.5 * (kecb + kp.x);
        out[0] = ke + pe + be;
        out[1] = ke;
        out[2] = pe;
        out[3] = be;
        out[4] = L[0] + Lp.x;
        out[5] = L[1] + Lp.y;
        out[6] = L[2] + Lp.z;
        out[7] = GMcb + gsum;
        out[8] = ke + (pe_pairs + kp.z) + be;
    }
}

// ---- WHM (Jacobi coordinates)
// The reference's Jacobi conversions and the ah0 / ah2 accelerations are running sums over
// the bodies in index order.  Here the whole block forms the terms (products and quotients)
// into shared memory, the running sums are taken (exact: one thread per component adds
// them in index order with the reference's operands, so FP64 results stay bit-identical;
// mixed path: a segmented warp scan per component), and the block uses them; bodies go
// through in chunks of WCH.
constexpr int WCH = 512;
struct WhmScratch {
    double t[6][WCH];      // terms, then (in place) inclusive running sums
    double run[6];         // running sums carried across chunks
    double e[WCH];         // ah2: etaj per body
    unsigned char m[WCH];  // ah2: the body's mask
};

// v[q] <- run + v[0] + ... + v[q] for q < cnt, and run <- the last value, by one whole warp
// (mixed path): lane l sums its segment of ceil(cnt / 32) terms, the warp scans the
// segment sums, and each lane re-adds its segment from its prefix.  ~2 cnt / 32 + 6 FP64
// issues on the warp instead of cnt serial additions (a warp issues an FP64 instruction
// at most every ~64 cycles on GB300); the rounding differs from the serial order.
static __device__ __forceinline__ void warp_seg_scan(double *v, int cnt, double &run) {
    const int lane = threadIdx.x & 31;
    const int seg = (cnt + 31) >> 5, q0 = min(cnt, lane * seg), q1 = min(cnt, q0 + seg);
    double own = 0.0;
    for (int q = q0; q < q1; q++) own += v[q];
    double incl = own;
    for (int o = 1; o < 32; o <<= 1) {
        const double y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    const double excl = __shfl_up_sync(0xffffffffu, incl, 1);
    const double base = run;
    double acc = lane == 0 ? base : base + excl;
    for (int q = q0; q < q1; q++) {
        acc += v[q];
        v[q] = acc;
    }
    const double total = __shfl_sync(0xffffffffu, incl, 31);
    __syncwarp();
    if (lane == 0) run = base + total;
}

// t[c][q] <- run[c] + t[c][0] + ... + t[c][q] for c < m.  exact: one thread per component
// adds in index order (the reference's operands and order); otherwise one warp per
// component runs warp_seg_scan (blockDim >= 32 m).
static __device__ __forceinline__ void whm_running(WhmScratch &sh, int m, int cnt, bool exact) {
    __syncthreads();
    if (exact) {
        if (threadIdx.x < m) {
            const int c = threadIdx.x;
            double s = sh.run[c];
            for (int q = 0; q < cnt; q++) {
                s = s + sh.t[c][q];
                sh.t[c][q] = s;
            }
            sh.run[c] = s;
        }
    } else if ((int)(threadIdx.x >> 5) < m) {
        const int c = threadIdx.x >> 5;
        warp_seg_scan(sh.t[c], cnt, sh.run[c]);
    }
    __syncthreads();
}

// whm_coord_h2j_pl (whm_coord.f90:14-51)
static __device__ void blk_whm_h2j(int n, const double *Gm, const double *eta, const double *rh, const double *vh,
                                   double *xj, double *vj, WhmScratch &sh, bool exact) {
    if (n <= 0) return;
    if (threadIdx.x < 3) {
        xj[threadIdx.x] = rh[threadIdx.x];
        vj[threadIdx.x] = vh[threadIdx.x];
    }
    if (threadIdx.x < 6) sh.run[threadIdx.x] = 0.0;
    for (int c0 = 1; c0 < n; c0 += WCH) {
        const int cnt = min(WCH, n - c0);
        __syncthreads();
        for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
            const int k = c0 + q - 1;
            for (int d = 0; d < 3; d++) {
                sh.t[d][q] = Gm[k] * rh[3 * k + d];
                sh.t[3 + d][q] = Gm[k] * vh[3 * k + d];
            }
        }
        whm_running(sh, 6, cnt, exact);
        for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
            const int i = c0 + q;
            for (int d = 0; d < 3; d++) {
                const double cap = sh.t[d][q] / eta[i - 1];
                const double capv = sh.t[3 + d][q] / eta[i - 1];
                xj[3 * i + d] = rh[3 * i + d] - cap;
                vj[3 * i + d] = vh[3 * i + d] - capv;
            }
        }
    }
}
// whm_coord_j2h_pl (:54-90)
static __device__ void blk_whm_j2h(int n, const double *Gm, const double *eta, const double *xj, const double *vj,
                                   double *rh, double *vh, WhmScratch &sh, bool exact) {
    if (n <= 0) return;
    if (threadIdx.x < 3) {
        rh[threadIdx.x] = xj[threadIdx.x];
        vh[threadIdx.x] = vj[threadIdx.x];
    }
    if (threadIdx.x < 6) sh.run[threadIdx.x] = 0.0;
    for (int c0 = 1; c0 < n; c0 += WCH) {
        const int cnt = min(WCH, n - c0);
        __syncthreads();
        for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
            const int k = c0 + q - 1;
            for (int d = 0; d < 3; d++) {
                sh.t[d][q] = Gm[k] * xj[3 * k + d] / eta[k];
                sh.t[3 + d][q] = Gm[k] * vj[3 * k + d] / eta[k];
            }
        }
        whm_running(sh, 6, cnt, exact);
        for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
            const int i = c0 + q;
            for (int d = 0; d < 3; d++) {
                rh[3 * i + d] = xj[3 * i + d] + sh.t[d][q];
                vh[3 * i + d] = vj[3 * i + d] + sh.t[3 + d][q];
            }
        }
    }
}
// whm_coord_vh2vj_pl (:93-124)
static __device__ void blk_whm_vh2vj(int n, const double *Gm, const double *eta, const double *vh, double *vj,
                                     WhmScratch &sh, bool exact) {
    if (n <= 0) return;
    if (threadIdx.x < 3) vj[threadIdx.x] = vh[threadIdx.x];
    if (threadIdx.x < 3) sh.run[threadIdx.x] = 0.0;
    for (int c0 = 1; c0 < n; c0 += WCH) {
        const int cnt = min(WCH, n - c0);
        __syncthreads();
        for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
            const int k = c0 + q - 1;
            for (int d = 0; d < 3; d++) sh.t[d][q] = Gm[k] * vh[3 * k + d];
        }
        whm_running(sh, 3, cnt, exact);
        for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
            const int i = c0 + q;
            for (int d = 0; d < 3; d++) {
                const double capv = sh.t[d][q] / eta[i - 1];
                vj[3 * i + d] = vh[3 * i + d] - capv;
            }
        }
    }
}
// whm_kick_getacch_ah0 (whm_kick.f90:125-149): ah0 = -sum mu_i rhp_i / |rhp_i|^3 in index
// order, into out[3] (shared or global), visible to the block on return
static __device__ void blk_whm_ah0(const double *mu, const double *rhp, int n, double *out, WhmScratch &sh,
                                   bool exact) {
    if (threadIdx.x < 3) sh.run[threadIdx.x] = 0.0;
    for (int c0 = 0; c0 < n; c0 += WCH) {
        const int cnt = min(WCH, n - c0);
        __syncthreads();
        for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
            const int i = c0 + q;
            const double r2 =
                rhp[3 * i] * rhp[3 * i] + rhp[3 * i + 1] * rhp[3 * i + 1] + rhp[3 * i + 2] * rhp[3 * i + 2];
            const double ir3h = 1.0 / (r2 * sqrt(r2));
            const double fac = mu[i] * ir3h;
            for (int d = 0; d < 3; d++) sh.t[d][q] = -(fac * rhp[3 * i + d]);  // a - b == a + (-b)
        }
        whm_running(sh, 3, cnt, exact);
    }
    __syncthreads();
    if (threadIdx.x < 3) out[threadIdx.x] = sh.run[threadIdx.x];
    __syncthreads();
}
// whm_kick_getacch_pl (whm_kick.f90:14-67) up to accel_int, with set_ir3j (whm_util.f90:117-140),
// ah1 (:152-179) and ah2 (:182-215), whole block
static __device__ void blk_whm_accel_pl(int n, const double *Gm, double GMcb, const double *rh, const double *xj,
                                        const int32_t *lmask, double *ir3h, double *ir3j, double *ah,
                                        WhmScratch &sh, bool exact) {
    __shared__ double s_ah0[3];
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double r2 = rh[3 * i] * rh[3 * i] + rh[3 * i + 1] * rh[3 * i + 1] + rh[3 * i + 2] * rh[3 * i + 2];
        double ir = 1.0 / sqrt(r2);
        ir3h[i] = ir / r2;
        r2 = xj[3 * i] * xj[3 * i] + xj[3 * i + 1] * xj[3 * i + 1] + xj[3 * i + 2] * xj[3 * i + 2];
        ir = 1.0 / sqrt(r2);
        ir3j[i] = ir / r2;
    }
    blk_whm_ah0(Gm + 1, rh + 3, n - 1, s_ah0, sh, exact);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        for (int d = 0; d < 3; d++) ah[3 * i + d] = ah[3 * i + d] + s_ah0[d];
        if (i >= 1 && lmask[i])
            for (int d = 0; d < 3; d++) {
                const double ah1j = xj[3 * i + d] * ir3j[i];
                const double ah1h = rh[3 * i + d] * ir3h[i];
                ah[3 * i + d] = ah[3 * i + d] + GMcb * (ah1j - ah1h);
            }
    }
    // ah2: etaj = GMcb + the masked Gm[i-1] in order; ah2_i = ah2_(previous masked) + fac_i xj_i
    if (threadIdx.x == 0) sh.run[3] = GMcb;
    if (threadIdx.x < 3) sh.run[threadIdx.x] = 0.0;
    for (int c0 = 1; c0 < n; c0 += WCH) {
        const int cnt = min(WCH, n - c0);
        __syncthreads();
        for (int q = threadIdx.x; q < cnt; q += blockDim.x) {  // stage the masks and Gm[i-1]
            sh.m[q] = lmask[c0 + q] != 0;
            sh.e[q] = Gm[c0 + q - 1];
        }
        __syncthreads();
        if (exact) {
            if (threadIdx.x == 0) {
                double etaj = sh.run[3];
                for (int q = 0; q < cnt; q++) {
                    if (!sh.m[q]) continue;
                    etaj = etaj + sh.e[q];
                    sh.e[q] = etaj;
                }
                sh.run[3] = etaj;
            }
        } else {  // unmasked bodies add zero; their running values are not used
            for (int q = threadIdx.x; q < cnt; q += blockDim.x)
                if (!sh.m[q]) sh.e[q] = 0.0;
            __syncthreads();
            if (threadIdx.x < 32) warp_seg_scan(sh.e, cnt, sh.run[3]);
        }
        __syncthreads();
        for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
            if (!sh.m[q]) {
                for (int d = 0; d < 3; d++) sh.t[d][q] = 0.0;
                continue;
            }
            const int i = c0 + q;
            const double fac = Gm[i] * GMcb * ir3j[i] / sh.e[q];
            for (int d = 0; d < 3; d++) sh.t[d][q] = fac * xj[3 * i + d];
        }
        __syncthreads();
        if (exact) {
            if (threadIdx.x < 3) {
                const int d = threadIdx.x;
                double a2 = sh.run[d];
                for (int q = 0; q < cnt; q++) {
                    if (!sh.m[q]) continue;
                    a2 = a2 + sh.t[d][q];
                    sh.t[d][q] = a2;
                }
                sh.run[d] = a2;
            }
        } else if (threadIdx.x < 96) {
            const int d = threadIdx.x >> 5;
            warp_seg_scan(sh.t[d], cnt, sh.run[d]);
        }
        __syncthreads();
        for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
            if (!sh.m[q]) continue;
            const int i = c0 + q;
            for (int d = 0; d < 3; d++) ah[3 * i + d] = ah[3 * i + d] + sh.t[d][q];
        }
    }
    __syncthreads();
}

// ---- flat per-body kernels of the step loops
// v += a*dt (masked) ; optionally rcopy = r (set_beg_end)
static __global__ void k_kick_update(int n, double *v, const double *__restrict__ a, const int32_t *__restrict__ lmask,
                              double dt, const double *__restrict__ r, double *rcopy) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (rcopy)
        for (int d = 0; d < 3; d++) rcopy[3 * i + d] = r[3 * i + d];
    if (!lmask[i]) return;
    for (int d = 0; d < 3; d++) v[3 * i + d] = v[3 * i + d] + a[3 * i + d] * dt;
}

// symba_step_reset_system (symba_step.f90:265-331) + set_renc(0).  The reference sets
// lmask = .true. because removed bodies have left the arrays; here they stay in place with
// status INACTIVE, so lmask is status /= INACTIVE.
static __global__ void k_symba_reset(int npl, int ntp, int32_t *levelg, int32_t *levelm, int32_t *nplenc, int32_t *ntpenc,
                              int32_t *lmask, int32_t *tlevelg, int32_t *tlevelm, int32_t *tnplenc,
                              int32_t *tlmask, const int32_t *__restrict__ status,
                              const int32_t *__restrict__ tstatus) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < npl) {
        levelg[i] = -1;
        levelm[i] = -1;
        nplenc[i] = 0;
        ntpenc[i] = 0;
        lmask[i] = status[i] != ST_INACTIVE;  // bodies removed by a collision stay masked
    }
    if (i < ntp) {
        tlevelg[i] = -1;
        tlevelm[i] = -1;
        tnplenc[i] = 0;
        tlmask[i] = tstatus[i] != ST_INACTIVE;
    }
}

// renc of every body at recursion level `scale`
static __global__ void k_set_renc(int npl, const double *rhill, double rhscale, int scale, double *renc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < npl) renc[i] = d_renc(rhill[i], rhscale, scale);
}

// Test particles flagged by the close-approach scan (swiftest_discard_pl_tp) leave the
// system: status INACTIVE, masked, parked with no velocity at 1e6 AU + (npl + local index)
// (the reference spills them out of its arrays).  tsys/toff/npls (optional) give each
// test particle's system in a CSR-packed ensemble; otherwise one system of npl bodies.
static __global__ void k_apply_discard(int64_t ntp, int32_t *flag, int32_t *tstatus, int32_t *tlmask, double *trh,
                                       double *tvh, double *tvb, int npl, const int32_t *__restrict__ tsys,
                                       const int32_t *__restrict__ toff, const int32_t *__restrict__ npls,
                                       unsigned long long *count) {
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= ntp || !flag[j]) return;
    flag[j] = 0;
    int64_t slot = npl + j;
    if (tsys) {
        const int s = tsys[j];
        slot = npls[s] + (j - toff[s]);
    }
    tstatus[j] = ST_INACTIVE;
    tlmask[j] = 0;
    trh[3 * j] = 1.0e6 + (double)slot;
    trh[3 * j + 1] = trh[3 * j + 2] = 0.0;
    for (int d = 0; d < 3; d++) tvh[3 * j + d] = tvb[3 * j + d] = 0.0;
    atomicAdd(count, 1ull);
}

}  // namespace sdev
}  // namespace swg
