// kick_mixed.cuh -- FP32 pair arithmetic of the mixed-precision kick, shared by the
// broadcast kernels (kick.cu) and the symmetric pair kernel (kick_sym.cu).
//
// Each FP64 coordinate is split into a float hi/lo pair; a displacement is formed as
// (xj_hi - xi_hi) + (xj_lo - xi_lo) in FP32, r^-3 comes from the hardware rsqrt estimate
// refined by one Newton step, and FP32 partial sums over short partner runs are folded
// into float-float (TwoSum) accumulators.
#pragma once
#include <cuda_runtime.h>

namespace swg {

constexpr int MT = 64;        // partners per FP32 partial (mixed)

// ------------------------------------------------------------------ mixed
struct FF {
    float hi, lo;
};
static __device__ __forceinline__ void ff_add(FF &a, float p) {
    // TwoSum (Knuth): exact error of hi + p, folded into lo.
    const float s = a.hi + p;
    const float bp = s - a.hi;
    const float err = (a.hi - (s - bp)) + (p - bp);
    a.hi = s;
    a.lo = a.lo + err;
}

static __device__ __forceinline__ void split_hi_lo(double x, float &hi, float &lo) {
    hi = __double2float_rn(x);
    lo = __double2float_rn(x - (double)hi);
}

// One receiving body of the mixed kick: its coordinates split into float hi/lo.
struct MixedRecv {
    float xh, yh, zh, xl, yl, zl, R;
};

template <bool RAD>
__device__ __forceinline__ MixedRecv mixed_recv(const double *__restrict__ r, const double *__restrict__ R, int i) {
    MixedRecv q;
    split_hi_lo(r[3 * i + 0], q.xh, q.xl);
    split_hi_lo(r[3 * i + 1], q.yh, q.yl);
    split_hi_lo(r[3 * i + 2], q.zh, q.zl);
    q.R = RAD ? __double2float_rn(R[i]) : 0.f;
    return q;
}

// Hardware reciprocal square root estimate (one MUFU instruction, subnormals flushed):
// r^2 of two distinct bodies is never subnormal, and a zero r^2 (a body paired with
// itself) gives +inf, which the pair rule replaces by a zero factor.
static __device__ __forceinline__ float rsqrt_approx(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// r^-3 in FP32: the hardware estimate y0 refined by one Newton step applied to the cube.
// With e = 1 - r2 y0^2 the Newton iterate is y1 = y0 (1 + e/2), and
// y1^3 = y0^3 (1 + 3e/2) + O(e^2) = y0^3 (2.5 - 1.5 r2 y0^2); e ~ 1e-7, so the dropped
// terms are ~1e-14 relative.
static __device__ __forceinline__ float rinv3(float r2) {
    const float y = rsqrt_approx(r2);
    const float t = y * y;
    return (t * y) * fmaf(-1.5f, r2 * t, 2.5f);
}

// ---- packed FP32 pairs (f32x2): one instruction applies the same operation to the two
// halves of a 64-bit register, with the scalar instruction's IEEE rounding.  On GB300 it
// occupies the FP32 pipe for two lane-slots but a single issue slot, so an issue-bound
// pair loop moves onto the FP32 pipe's own limit.
typedef unsigned long long f32x2;
static __device__ __forceinline__ f32x2 f2_pack(float lo, float hi) {
    f32x2 d;
    asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(lo), "f"(hi));
    return d;
}
static __device__ __forceinline__ void f2_unpack(f32x2 v, float &lo, float &hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
static __device__ __forceinline__ f32x2 f2_add(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
static __device__ __forceinline__ f32x2 f2_sub(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
static __device__ __forceinline__ f32x2 f2_mul(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
static __device__ __forceinline__ f32x2 f2_fma(f32x2 a, f32x2 b, f32x2 c) {
    f32x2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

// Partner tile layout of the pl-tp (TP) kick: partners 2p and 2p+1 side by side, so that
// one 64-bit word holds the same coordinate of both.  With sA, sB the tile's two 64-entry
// float4 arrays: sA[p] = (xh, yh) pairs, sA[MT/2 + p] = (zh, Gm) pairs, sB[p] = (xl, yl)
// pairs, sB[MT/2 + p] = (zl, R) pairs, each pair as (partner 2p, partner 2p+1).
static __device__ __forceinline__ void stage_pair(float4 *sA, float4 *sB, int p, const float4 &a0,
                                                  const float4 &b0, const float4 &a1, const float4 &b1) {
    sA[p] = make_float4(a0.x, a1.x, a0.y, a1.y);
    sA[MT / 2 + p] = make_float4(a0.z, a1.z, a0.w, a1.w);
    sB[p] = make_float4(b0.x, b1.x, b0.y, b1.y);
    sB[MT / 2 + p] = make_float4(b0.z, b1.z, b0.w, b1.w);
}

// The pl-tp tile on packed pairs: each instruction evaluates one receiver against the
// partner pair (2p, 2p+1), with the scalar loop's operations term by term; the even and
// odd partners accumulate in the two halves and are added at the end of the tile.
// Unused tile slots hold zero mass (their terms are zero).
template <int RPT>
__device__ __forceinline__ void mixed_tile_tp2(int nt, const MixedRecv (&q)[RPT], const float4 *sA, const float4 *sB,
                                               float (&px)[RPT], float (&py)[RPT], float (&pz)[RPT]) {
    const ulonglong2 *hA = reinterpret_cast<const ulonglong2 *>(sA);
    const ulonglong2 *hB = reinterpret_cast<const ulonglong2 *>(sB);
    f32x2 xh[RPT], yh[RPT], zh[RPT], xl[RPT], yl[RPT], zl[RPT], ax[RPT], ay[RPT], az[RPT];
#pragma unroll
    for (int k = 0; k < RPT; k++) {
        xh[k] = f2_pack(q[k].xh, q[k].xh);
        yh[k] = f2_pack(q[k].yh, q[k].yh);
        zh[k] = f2_pack(q[k].zh, q[k].zh);
        xl[k] = f2_pack(q[k].xl, q[k].xl);
        yl[k] = f2_pack(q[k].yl, q[k].yl);
        zl[k] = f2_pack(q[k].zl, q[k].zl);
        ax[k] = ay[k] = az[k] = 0ull;
    }
    const f32x2 c15 = f2_pack(-1.5f, -1.5f), c25 = f2_pack(2.5f, 2.5f);
    const int np = (nt + 1) >> 1;
#pragma unroll 4
    for (int jp = 0; jp < np; jp++) {
        const ulonglong2 h1 = hA[jp], h2 = hA[MT / 2 + jp], l1 = hB[jp], l2 = hB[MT / 2 + jp];
#pragma unroll
        for (int k = 0; k < RPT; k++) {
            const f32x2 dx = f2_add(f2_sub(h1.x, xh[k]), f2_sub(l1.x, xl[k]));
            const f32x2 dy = f2_add(f2_sub(h1.y, yh[k]), f2_sub(l1.y, yl[k]));
            const f32x2 dz = f2_add(f2_sub(h2.x, zh[k]), f2_sub(l2.x, zl[k]));
            const f32x2 r2 = f2_fma(dz, dz, f2_fma(dy, dy, f2_mul(dx, dx)));
            float r2a, r2b;
            f2_unpack(r2, r2a, r2b);
            const f32x2 y = f2_pack(rsqrt_approx(r2a), rsqrt_approx(r2b));
            const f32x2 t = f2_mul(y, y);
            const f32x2 ir3 = f2_mul(f2_mul(t, y), f2_fma(c15, f2_mul(r2, t), c25));
            const f32x2 fac = f2_mul(h2.y, ir3);
            ax[k] = f2_fma(fac, dx, ax[k]);
            ay[k] = f2_fma(fac, dy, ay[k]);
            az[k] = f2_fma(fac, dz, az[k]);
        }
    }
#pragma unroll
    for (int k = 0; k < RPT; k++) {
        float e, o;
        f2_unpack(ax[k], e, o);
        px[k] = e + o;
        f2_unpack(ay[k], e, o);
        py[k] = e + o;
        f2_unpack(az[k], e, o);
        pz[k] = e + o;
    }
}

// One 64-partner tile for this thread's RPT receivers: FP32 partials px/py/pz (from zero).
// GUARD applies the pl-pl pair rule to every pair (below).  Without it every pair is
// taken, and with RAD the smallest r^2 met is kept in mn so that the caller can tell
// whether the radius rule would have dropped a pair.
template <bool TP, bool RAD, bool GMT, bool GUARD, int RPT>
__device__ __forceinline__ void mixed_tile(int j0, int nt, const int (&self)[RPT], int nplm, const bool (&self_m)[RPT],
                                           const MixedRecv (&q)[RPT], const float4 *sA, const float4 *sB,
                                           float (&px)[RPT], float (&py)[RPT], float (&pz)[RPT], float (&mn)[RPT]) {
#pragma unroll
    for (int k = 0; k < RPT; k++) px[k] = py[k] = pz[k] = 0.f;
#pragma unroll 8
    for (int jj = 0; jj < nt; jj++) {
        const float4 a = sA[jj];
        const float4 b = sB[jj];
#pragma unroll
        for (int k = 0; k < RPT; k++) {
            const float dx = (a.x - q[k].xh) + (b.x - q[k].xl);
            const float dy = (a.y - q[k].yh) + (b.y - q[k].yl);
            const float dz = (a.z - q[k].zh) + (b.z - q[k].zl);
            const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
            float fac = a.w * rinv3(r2);
            if (!TP && GUARD) {
                const int j = j0 + jj;
                bool ok = true;
                if (GMT) ok = self_m[k] || j < nplm;
                if (RAD) {
                    const float rs = q[k].R + b.w;
                    ok = ok && (r2 > rs * rs);
                } else {
                    ok = ok && (j != self[k]);
                }
                fac = ok ? fac : 0.f;
            }
            if (!TP && !GUARD && RAD) mn[k] = fminf(mn[k], r2);
            px[k] = fmaf(fac, dx, px[k]);
            py[k] = fmaf(fac, dy, py[k]);
            pz[k] = fmaf(fac, dz, pz[k]);
        }
    }
}

}  // namespace swg
