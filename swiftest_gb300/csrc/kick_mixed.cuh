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
