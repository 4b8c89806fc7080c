// encounter_sorted.cu -- batched TRIANGULAR pl-pl check over radius-sorted tiles.
//
// The reference's triangular check (src/encounter/encounter_check.f90:436-475) tests every
// pair i < j with encounter_check_one (:573-621).  Here, per system, the bodies are ordered
// by heliocentric distance (one shared-memory sort per system) and cut into sub-tiles of
// 32; a warp of 32 receivers skips every partner sub-tile in which no pair with its
// receivers can pass the FP64 test, and every other pair goes through the same FP32
// prefilter and FP64 decision as the unsorted kernel, on
// the bodies' original indices and in the reference's orientation (i < j).  The list is
// sorted by (index1, index2) afterwards, so it is the triangular check's list exactly; the
// order only decides how much is skipped.
//
// The order only has to be roughly radial, so it is refreshed every few steps (bodies move
// ~1e-4 of the disk width per step); the bounds are recomputed from the current state at
// every check.
//
// Why a tile pair can be skipped.  encounter_check_one accepts (i, j) only if its computed
// r2min <= (renc_i + renc_j)^2, where r2min is the minimum over t in [0, dt] of
// |x_rel + v_rel t|^2 up to a rounding of 6.7e-16 r^2 (see prefilter_reject), i.e. only if
// D <= R (1 + 1e-15) + 2.6e-8 r with D = min_t |x_rel(t)|.  By the reverse triangle
// inequality D >= min_t | |x_j + v_j t| - |x_i + v_i t| |, and for |t| <= |dt|
//     |x|^2 - 2 |x.v| |dt|  <=  |x + v t|^2  <=  |x|^2 + 2 |x.v| |dt| + |v|^2 dt^2,
// so each body's distance from the central body stays in an interval [lo, hi] over the
// step.  If the intervals of two tiles are separated by a gap larger than the largest
// renc_i + renc_j (plus margins for float rounding of the bounds and the 2.6e-8 r term,
// r <= hi_i + hi_j), no pair across them is accepted.  NaN positions make every
// comparison false, so such tiles are never skipped.
#include <cuda_runtime.h>

#include <algorithm>

#include "encounter_dev.cuh"
#include "swg_internal.cuh"

namespace swg {

constexpr int SB = 64;                   // bodies per bound tile
constexpr int SQ = 128;                  // receivers per block (two bound tiles)
constexpr int SORT_MAX = 16384;          // largest system ordered in shared memory
static_assert(SQ == ENC_SORTED_TILE && SB == ENC_BOUND_TILE, "tile sizes of the sorted check");

// Per system (one block of RS_T threads): order the bodies by |r| (ties by index).
// perm[poff + p] is the global index of the body at sorted position p.  Systems above
// SORT_MAX keep their order.  The order only steers the culling (every pair the cull keeps
// is still decided in FP64), so a 24-bit key is enough: the FP32 |r| with its 7 lowest
// mantissa bits dropped (its bit pattern orders like the value for r >= 0; a NaN sorts
// last).  Stable LSD radix sort in shared memory, three passes of 8 bits: each warp takes
// a contiguous segment of the bodies 32 at a time, ranks equal digits among its lanes with
// __match_any_sync, and counts per (digit, warp); an exclusive scan over the counts in
// (digit, warp) order gives every warp's first slot per digit, so each pass keeps the
// previous order among equal digits and the result is ordered by (key, index).
constexpr int RS_T = 512;                 // threads of k_radial_sort
constexpr int RS_W = RS_T / 32;           // warps of k_radial_sort
constexpr int RS_HIST = 256 * RS_W;       // (digit, warp) counts
__global__ void __launch_bounds__(RS_T) k_radial_sort(const int32_t *__restrict__ poff, const int32_t *__restrict__ npl,
                                                      const double *__restrict__ r, int32_t *__restrict__ perm) {
    extern __shared__ unsigned char smem[];
    const int s = blockIdx.x;
    const int n = npl[s], o = poff[s];
    if (n > SORT_MAX) {
        for (int t = threadIdx.x; t < n; t += blockDim.x) perm[o + t] = o + t;
        return;
    }
    uint32_t *hist = (uint32_t *)smem;  // [digit][warp]
    uint32_t *key[2] = {hist + RS_HIST, hist + RS_HIST + n};
    uint16_t *idx[2] = {(uint16_t *)(hist + RS_HIST + 2 * n), (uint16_t *)(hist + RS_HIST + 2 * n) + n};
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        const double *x = &r[3 * (size_t)(o + t)];
        const float x0 = (float)x[0], x1 = (float)x[1], x2 = (float)x[2];
        float k = sqrtf(fmaf(x2, x2, fmaf(x1, x1, x0 * x0)));
        if (!(k >= 0.f)) k = __int_as_float(0x7f800000);
        key[0][t] = (uint32_t)__float_as_int(k) >> 7;
        idx[0][t] = (uint16_t)t;
    }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int seg = (n + RS_W - 1) / RS_W, b0 = min(n, w * seg), b1 = min(n, b0 + seg);
    const unsigned lt = (1u << lane) - 1u;
    int in = 0;
    for (int shift = 0; shift < 24; shift += 8, in ^= 1) {
        for (int t = threadIdx.x; t < RS_HIST; t += blockDim.x) hist[t] = 0;
        __syncthreads();  // keys of this pass written, counts cleared
        for (int b = b0; b < b1; b += 32) {  // counts of this warp's segment
            const int i = b + lane;
            const int d = i < b1 ? (int)((key[in][i] >> shift) & 255u) : 256;
            const unsigned peers = __match_any_sync(0xffffffffu, d);
            if (d < 256 && lane == __ffs(peers) - 1) hist[d * RS_W + w] += __popc(peers);
            __syncwarp();
        }
        __syncthreads();
        // exclusive scan of the counts in (digit, warp) order: each thread its RS_HIST / RS_T
        // consecutive entries, then the thread sums across the block
        constexpr int PER = RS_HIST / RS_T;
        uint32_t loc[PER], sum = 0;
#pragma unroll
        for (int q = 0; q < PER; q++) {
            loc[q] = hist[threadIdx.x * PER + q];
            sum += loc[q];
        }
        uint32_t inc = sum;  // inclusive scan of the thread sums: in the warp, then across warps
#pragma unroll
        for (int dd = 1; dd < 32; dd <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, inc, dd);
            if (lane >= dd) inc += y;
        }
        __shared__ uint32_t wsum[RS_W];
        if (lane == 31) wsum[w] = inc;
        __syncthreads();
        uint32_t wbase = 0;
        for (int q = 0; q < w; q++) wbase += wsum[q];
        uint32_t run = wbase + inc - sum;
#pragma unroll
        for (int q = 0; q < PER; q++) {
            hist[threadIdx.x * PER + q] = run;
            run += loc[q];
        }
        __syncthreads();  // first slots ready; wsum free for the next pass
        for (int b = b0; b < b1; b += 32) {  // scatter, in segment order
            const int i = b + lane;
            const bool ok = i < b1;
            const int d = ok ? (int)((key[in][i] >> shift) & 255u) : 256;
            const unsigned peers = __match_any_sync(0xffffffffu, d);
            uint32_t pos = 0;
            if (ok) pos = hist[d * RS_W + w] + __popc(peers & lt);
            __syncwarp();  // every lane has read its digit's slot before the leader moves it
            if (ok) {
                key[in ^ 1][pos] = key[in][i];
                idx[in ^ 1][pos] = idx[in][i];
                if (lane == __ffs(peers) - 1) hist[d * RS_W + w] += __popc(peers);
            }
            __syncwarp();
        }
        __syncthreads();  // the pass's output complete
    }
    for (int t = threadIdx.x; t < n; t += blockDim.x) perm[o + t] = o + (int32_t)idx[in][t];
}

// One block of SB threads per bound tile (sys, first sorted position): the prefilter's
// float copies in sorted order and the bounds (min lo, max hi, max renc), rounded outward,
// of each 32-body half u of the tile (bounds[2 t + u]; a half without bodies gets
// (+inf, -inf, 0), which is apart from everything).
__global__ void __launch_bounds__(SB) k_sorted_prep(const int2 *__restrict__ tiles, const int32_t *__restrict__ poff,
                                                    const int32_t *__restrict__ npl, const int32_t *__restrict__ perm,
                                                    const double *__restrict__ r, const double *__restrict__ v,
                                                    const double *__restrict__ renc, float adt, float4 *A, float4 *B,
                                                    float4 *V, float4 *bounds) {
    const int2 tl = tiles[blockIdx.x];
    const int p = poff[tl.x] + tl.y + threadIdx.x;
    const bool in = tl.y + (int)threadIdx.x < npl[tl.x];
    float lo = __int_as_float(0x7f800000), hi = -__int_as_float(0x7f800000), Rm = 0.f;
    if (in) {
        const int g = perm[p];
        const BodyF o = load_body(r, v, renc, g);
        A[p] = o.a;
        B[p] = o.b;
        V[p] = o.v;
        // The interval in FP32 from the float copies.  The hi parts and the rounded
        // velocity are within 6e-8 (relative) of the FP64 values, and the float sums
        // below add < 5e-7 relative to |x|^2, |v|^2 and, for x.v (which may cancel),
        // < 5e-7 |x| |v| absolute; the margins (1e-5 of each term, plus 1e-5 |x||v| on
        // x.v) bound the true interval from outside.
        const float x2 = fmaf(o.a.z, o.a.z, fmaf(o.a.y, o.a.y, o.a.x * o.a.x));
        const float v2 = fmaf(o.v.z, o.v.z, fmaf(o.v.y, o.v.y, o.v.x * o.v.x));
        const float xv = fabsf(fmaf(o.a.z, o.v.z, fmaf(o.a.y, o.v.y, o.a.x * o.v.x))) + 1e-5f * sqrtf(x2 * v2);
        const float T = adt;
        lo = sqrtf(fmaxf(x2 * (1.0f - 1e-5f) - 2.0f * xv * T * (1.0f + 1e-5f), 0.0f)) * (1.0f - 1e-5f);
        hi = sqrtf((x2 + 2.0f * xv * T + v2 * T * T) * (1.0f + 1e-5f)) * (1.0f + 1e-5f);
        Rm = o.a.w * (1.0f + 1e-5f);
    }
    for (int off = 16; off > 0; off >>= 1) {
        lo = fminf(lo, __shfl_down_sync(0xffffffffu, lo, off));
        hi = fmaxf(hi, __shfl_down_sync(0xffffffffu, hi, off));
        Rm = fmaxf(Rm, __shfl_down_sync(0xffffffffu, Rm, off));
    }
    if ((threadIdx.x & 31) == 0) bounds[(SB / 32) * blockIdx.x + (threadIdx.x >> 5)] = make_float4(lo, hi, Rm, 0.f);
}

// True when no pair across tiles P and Q can pass the FP64 test (see the file comment).
__device__ __forceinline__ bool tiles_apart(float4 P, float4 Q) {
    const float gap = fmaxf(__fsub_rd(P.x, Q.y), __fsub_rd(Q.x, P.y));
    const float reach = __fmaf_ru(__fadd_ru(P.z, Q.z), 1.0f + 1e-5f, 1e-6f * __fadd_ru(P.y, Q.y));
    return gap > reach;
}

// One warp's partners: each lane stages one partner (float copies and global index) in the
// warp's own shared slots.
struct WarpStage {
    float4 a[32], b[32], v[32];
    int32_t g[32];
};

// Item (system, first receiver in sorted order q0, receivers nr): receivers are sorted
// positions [q0, q0 + nr), partners sorted positions p < q.  Each warp works alone on its
// 32 receivers (no block barriers): its lanes test the bounds of 32 partner sub-tiles (32
// bodies each) at a time against the warp's own sub-tile bound, and for every sub-tile
// that is not apart the lanes stage its partners in the warp's shared slots and each lane
// runs its receiver against them.  nplm (optional, GMTINY): per system the count of fully
// interacting bodies; a pair of two bodies both at local index >= nplm[s] is not tested
// (the reference checks plm x pl only: encounter_check_all_plplm).
__global__ void __launch_bounds__(SQ) k_encounter_sorted(const int4 *__restrict__ items, const int32_t *__restrict__ poff,
                                                         const int32_t *__restrict__ tbase,
                                                         const int32_t *__restrict__ perm, const float4 *__restrict__ A,
                                                         const float4 *__restrict__ B, const float4 *__restrict__ V,
                                                         const float4 *__restrict__ sub, const double *__restrict__ r,
                                                         const double *__restrict__ v, const double *__restrict__ renc,
                                                         double dt, long long cap, int32_t *__restrict__ o1,
                                                         int32_t *__restrict__ o2, int32_t *__restrict__ olv,
                                                         unsigned long long *__restrict__ count,
                                                         const int32_t *__restrict__ nplm) {
    __shared__ WarpStage st_all[SQ / 32];
    const int4 w = items[blockIdx.x];
    const int s = w.x, q0 = w.y, nr = w.z;
    const int wq = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (32 * wq >= nr) return;  // no receivers in this warp
    WarpStage &st = st_all[wq];
    const int o = poff[s];
    const float4 *S = sub + (SB / 32) * (size_t)tbase[s];  // the system's sub-tile (half-tile) bounds
    const float4 QW = S[q0 / 32 + wq];
    const int q = q0 + threadIdx.x;  // sorted position within the system
    const int qb = min(q0 + nr, q0 + 32 * wq + 32);  // this warp's receivers end here
    const bool active = q < qb;
    BodyF me;
    int gq = 0;
    if (active) {
        me.a = A[o + q];
        me.b = B[o + q];
        me.v = V[o + q];
        gq = perm[o + q];
    }
    const float dtf = __double2float_ru(fabs(dt)) * (1.0f + 1e-6f);
    const int gm = nplm ? o + nplm[s] : INT32_MAX;  // first semi-interacting body (global index)
    const int pend = qb - 1;  // partners p < q <= qb - 1
    const int nsub = (pend + 31) / 32;
    for (int u0 = 0; u0 < nsub; u0 += 32) {
        const bool keep = u0 + lane < nsub && !tiles_apart(S[u0 + lane], QW);
        unsigned m = __ballot_sync(0xffffffffu, keep);
        while (m) {
            const int p0 = 32 * (u0 + __ffs(m) - 1);
            m &= m - 1;
            __syncwarp();  // the previous sub-tile is consumed
            if (p0 + lane < pend) {
                const int pp = o + p0 + lane;
                st.a[lane] = A[pp];
                st.b[lane] = B[pp];
                st.v[lane] = V[pp];
                st.g[lane] = perm[pp];
            }
            __syncwarp();
            if (!active) continue;
            const int nt = min(32, q - p0);  // partners p < q of this sub-tile
            for (int ii = 0; ii < nt; ii++) {
                BodyF other;
                other.a = st.a[ii];
                other.b = st.b[ii];
                other.v = st.v[ii];
                if (prefilter_reject(other, me, dtf)) continue;
                const int gp = st.g[ii];
                const int i = min(gp, gq), j = max(gp, gq);  // the reference's orientation, i < j
                if (i >= gm) continue;  // both semi-interacting
                const double xr = r[3 * (size_t)j + 0] - r[3 * (size_t)i + 0];
                const double yr = r[3 * (size_t)j + 1] - r[3 * (size_t)i + 1];
                const double zr = r[3 * (size_t)j + 2] - r[3 * (size_t)i + 2];
                const double vxr = v[3 * (size_t)j + 0] - v[3 * (size_t)i + 0];
                const double vyr = v[3 * (size_t)j + 1] - v[3 * (size_t)i + 1];
                const double vzr = v[3 * (size_t)j + 2] - v[3 * (size_t)i + 2];
                int lenc, lv;
                d_encounter_one(xr, yr, zr, vxr, vyr, vzr, renc[i] + renc[j], dt, lenc, lv);
                if (lenc) {
                    const unsigned long long kk = atomicAdd(count, 1ull);
                    if ((long long)kk < cap) {
                        o1[kk] = i + 1;
                        o2[kk] = j + 1;
                        olv[kk] = lv;
                    }
                }
            }
        }
    }
}

// pl-tp over radius-sorted tiles: the level-0 pl-tp check (encounter_check_all_pltp,
// TRIANGULAR, encounter_check.f90:525-570, tp renc = 0) or, DISCARD, the close-approach scan
// of swiftest_discard_pl_tp (swiftest_discard.f90:244-290: flag[tp] = 1 when an ACTIVE tp
// comes within a pl's radius, renc = radius).  Item (system, first tp in sorted order q0,
// tp count nr): the tp receivers against every pl tile of the system that is not apart
// from them (the bound argument of the file comment holds for both tests: same closest-
// approach expression), each warp of 32 tp skipping the 32-body pl sub-tiles that are apart
// from it, as in k_encounter_sorted.  Pairs are written with global 1-based indices (pl, tp).
// pchunk > 0: the item's fourth field c selects the pl sub-tiles [c pchunk, (c + 1) pchunk)
// (a single system splits its pl range over several items to fill the GPU); 0: all of them.
template <bool DISCARD>
__global__ void __launch_bounds__(SQ) k_pltp_sorted(const int4 *__restrict__ items, const int32_t *__restrict__ poff,
                                                    const int32_t *__restrict__ npl, const int32_t *__restrict__ ptbase,
                                                    const int32_t *__restrict__ pperm, const float4 *__restrict__ PA,
                                                    const float4 *__restrict__ PB, const float4 *__restrict__ PV,
                                                    const float4 *__restrict__ psub, const double *__restrict__ rp,
                                                    const double *__restrict__ vp, const double *__restrict__ rencp,
                                                    const int32_t *__restrict__ toff,
                                                    const int32_t *__restrict__ ttbase,
                                                    const int32_t *__restrict__ tperm, const float4 *__restrict__ TA,
                                                    const float4 *__restrict__ TB, const float4 *__restrict__ TV,
                                                    const float4 *__restrict__ tsub, const double *__restrict__ rt,
                                                    const double *__restrict__ vt,
                                                    const int32_t *__restrict__ tstatus, double dt, long long cap,
                                                    int32_t *__restrict__ o1, int32_t *__restrict__ o2,
                                                    int32_t *__restrict__ olv, unsigned long long *__restrict__ count,
                                                    int32_t *__restrict__ flag, int pchunk) {
    __shared__ WarpStage st_all[SQ / 32];
    const int4 w = items[blockIdx.x];
    const int s = w.x, q0 = w.y, nr = w.z;
    const int wq = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (32 * wq >= nr) return;  // no tp in this warp
    WarpStage &st = st_all[wq];
    const int po = poff[s], n1 = npl[s], to = toff[s];
    const float4 *SP = psub + (SB / 32) * (size_t)ptbase[s];
    const float4 QW = tsub[(SB / 32) * (size_t)ttbase[s] + q0 / 32 + wq];
    bool active = (int)threadIdx.x < nr;
    BodyF me;
    int gq = 0;
    if (active) {
        me.a = TA[to + q0 + threadIdx.x];
        me.b = TB[to + q0 + threadIdx.x];
        me.v = TV[to + q0 + threadIdx.x];
        gq = tperm[to + q0 + threadIdx.x];
        if (DISCARD) active = tstatus[gq] == ST_ACTIVE;
    }
    const float dtf = __double2float_ru(fabs(dt)) * (1.0f + 1e-6f);
    int ubeg = 0, uend = (n1 + 31) / 32;
    if (pchunk > 0) {
        ubeg = w.w * pchunk;
        uend = min(uend, ubeg + pchunk);
    }
    for (int u0 = ubeg; u0 < uend; u0 += 32) {
        const bool keep = u0 + lane < uend && !tiles_apart(SP[u0 + lane], QW);
        unsigned m = __ballot_sync(0xffffffffu, keep);
        while (m) {
            const int p0 = 32 * (u0 + __ffs(m) - 1);
            m &= m - 1;
            __syncwarp();  // the previous sub-tile is consumed
            if (p0 + lane < n1) {
                const int pp = po + p0 + lane;
                st.a[lane] = PA[pp];
                st.b[lane] = PB[pp];
                st.v[lane] = PV[pp];
                st.g[lane] = pperm[pp];
            }
            __syncwarp();
            if (!active) continue;
            const int nt = min(32, n1 - p0);
            for (int ii = 0; ii < nt; ii++) {
                BodyF other;
                other.a = st.a[ii];
                other.b = st.b[ii];
                other.v = st.v[ii];
                if (prefilter_reject(other, me, dtf)) continue;
                const int i = st.g[ii];  // pl (global index)
                const double xr = rt[3 * (size_t)gq + 0] - rp[3 * (size_t)i + 0];
                const double yr = rt[3 * (size_t)gq + 1] - rp[3 * (size_t)i + 1];
                const double zr = rt[3 * (size_t)gq + 2] - rp[3 * (size_t)i + 2];
                const double vxr = vt[3 * (size_t)gq + 0] - vp[3 * (size_t)i + 0];
                const double vyr = vt[3 * (size_t)gq + 1] - vp[3 * (size_t)i + 1];
                const double vzr = vt[3 * (size_t)gq + 2] - vp[3 * (size_t)i + 2];
                if (DISCARD) {
                    if (d_discard_close(xr, yr, zr, vxr, vyr, vzr, dt, rencp[i] * rencp[i])) flag[gq] = 1;
                    continue;
                }
                int lenc, lv;
                d_encounter_one(xr, yr, zr, vxr, vyr, vzr, rencp[i] + 0.0, dt, lenc, lv);
                if (lenc) {
                    const unsigned long long kk = atomicAdd(count, 1ull);
                    if ((long long)kk < cap) {
                        o1[kk] = i + 1;
                        o2[kk] = gq + 1;
                        olv[kk] = lv;
                    }
                }
            }
        }
    }
}

// k_radial_sort over nsys systems of up to nmax bodies; its dynamic shared memory holds the
// counts, two key and two index buffers.
static int radial_sort_launch(swg_ctx *c, int nsys, int nmax, const int32_t *poff, const int32_t *npl,
                              const double *r, int32_t *perm) {
    const size_t smem = 4 * (size_t)RS_HIST + 12 * (size_t)std::min(nmax, SORT_MAX);
    static size_t smem_set = 0;  // the kernel's shared-memory limit raised so far
    if (smem > 48 * 1024 && smem > smem_set) {
        SWG_TRY(cuda_status(c, cudaFuncSetAttribute(k_radial_sort, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                    (int)smem),
                            "radial sort smem"));
        smem_set = smem;
    }
    k_radial_sort<<<nsys, RS_T, smem, c->stream>>>(poff, npl, r, perm);
    c->launches++;
    return launch_status(c, "radial_sort");
}

int sorted_set_prep(swg_ctx *c, const SortedSet &x, int nsys, bool resort, double dt) {
    if (x.ntiles <= 0) return SWG_OK;
    if (resort) SWG_TRY(radial_sort_launch(c, nsys, x.nmax, x.off, x.n, x.r, x.perm));
    const float adt = (float)fabs(dt) * (1.0f + 1e-6f);
    k_sorted_prep<<<x.ntiles, SB, 0, c->stream>>>(x.tiles, x.off, x.n, x.perm, x.r, x.v, x.renc, adt, x.F, x.F + x.N,
                                                  x.F + 2 * x.N, x.bounds);
    c->launches++;
    return launch_status(c, "sorted_prep");
}

int pltp_sorted_batched(swg_ctx *c, bool discard, const SortedSet &pl, const SortedSet &tp, const int32_t *tstatus,
                        int nitems, const int4 *items, double dt, long long cap, int32_t *o1, int32_t *o2,
                        int32_t *olv, unsigned long long *count, int32_t *flag, int pchunk) {
    if (nitems <= 0 || pl.ntiles <= 0) return SWG_OK;
#define SWG_PLTP_ARGS                                                                                                 \
    items, pl.off, pl.n, pl.tbase, pl.perm, pl.F, pl.F + pl.N, pl.F + 2 * pl.N, pl.bounds, pl.r, pl.v,    \
        pl.renc, tp.off, tp.tbase, tp.perm, tp.F, tp.F + tp.N, tp.F + 2 * tp.N, tp.bounds, tp.r, tp.v,      \
        tstatus, dt, cap, o1, o2, olv, count, flag, pchunk
    if (discard)
        k_pltp_sorted<true><<<nitems, SQ, 0, c->stream>>>(SWG_PLTP_ARGS);
    else
        k_pltp_sorted<false><<<nitems, SQ, 0, c->stream>>>(SWG_PLTP_ARGS);
#undef SWG_PLTP_ARGS
    c->launches++;
    return launch_status(c, discard ? "discard_pltp_sorted" : "encounter_pltp_sorted");
}

int encounter_plpl_sorted_batched(swg_ctx *c, int nsys, int nmax, const int32_t *poff, const int32_t *npl,
                                  const double *r, const double *v, const double *renc, double dt, bool resort,
                                  int32_t *perm, float4 *F, int64_t NPL, int ntiles, const int2 *tiles,
                                  const int32_t *tbase, float4 *bounds, int nitems, const int4 *items, long long cap,
                                  int32_t *o1, int32_t *o2, int32_t *olv, unsigned long long *count,
                                  const int32_t *nplm) {
    if (nitems <= 0 || ntiles <= 0) return SWG_OK;
    if (resort) SWG_TRY(radial_sort_launch(c, nsys, nmax, poff, npl, r, perm));
    const float adt = (float)fabs(dt) * (1.0f + 1e-6f);  // |dt| rounded to float, then up
    k_sorted_prep<<<ntiles, SB, 0, c->stream>>>(tiles, poff, npl, perm, r, v, renc, adt, F, F + NPL, F + 2 * NPL,
                                                bounds);
    c->launches++;
    SWG_TRY(launch_status(c, "sorted_prep"));
    k_encounter_sorted<<<nitems, SQ, 0, c->stream>>>(items, poff, tbase, perm, F, F + NPL, F + 2 * NPL, bounds, r,
                                                     v, renc, dt, cap, o1, o2, olv, count, nplm);
    c->launches++;
    return launch_status(c, "encounter_sorted");
}

}  // namespace swg
