// kick_sym.cu -- symmetric mixed-precision pl-pl kick of CSR-packed systems.
//
// Same sums as swiftest_kick_getacch_int_all_tri_* (src/swiftest/swiftest_kick.f90:183-264):
// acc_i += Gm_j (r_j - r_i)/r^3 and acc_j -= Gm_i (r_j - r_i)/r^3 for every pair, with the
// pair rule (radius guard, or j != i without radii).  The reference's triangular loop
// evaluates each pair once and applies it to both bodies; this kernel does the same in
// the FP32 pair arithmetic of the mixed kick (kick_mixed.cuh), which halves the
// instructions per interaction against the broadcast kernels that evaluate each pair
// once per receiving body.
//
// Work: every system's bodies form tiles of KICK_SYM_TILE = 128 (four 32-body sub-tiles).
// An item is a strip of one row of the upper triangle of tile pairs: tile I against tiles
// J0 .. J0 + nJ - 1 of one system; a persistent grid of one-warp blocks pulls items from a
// work queue.  Lane t holds the four receivers 32k + t of tile I (k = 0..3) in registers.
// Tile J is staged in shared memory with each 32-partner sub-tile stored twice in a row,
// so that lane t reads partner (t + s) mod 32 at step s without wrapping.
//   * I < J, for each sub-tile u of J: at every step s each lane evaluates its receivers
//     against partner (t + s) mod 32, adds to its receiver partials, and subtracts from an
//     accumulator of that partner which the warp rotates one lane down after the step
//     (three shuffles): after 32 steps every partner accumulator holds the sum over the
//     128 receivers and is back on the lane of its partner.
//   * I == J: sub-tile u against receivers k < u as above (so each pair is evaluated once);
//     the partner accumulators of sub-tile u then belong to receiver u of the same lane.
//     Receiver u against its own sub-tile is evaluated one-sided with the pair rule
//     applied pair by pair (self pairs).
// Tiles and sub-tiles other than the diagonal ones hold no self pairs; with radii, pairs
// that the radius rule could drop are found per sub-tile (the smallest r^2 a receiver met
// against its radius plus the sub-tile's largest radius) and that sub-tile is recomputed
// with the rule applied pair by pair, so every kept pair gets the same operations.
// Receiver sums (32-partner FP32 partials folded into float-float) go to one receiver slot
// per item; partner sums of each off-diagonal tile pair (FP32 sums over 128 receivers) to
// the system's pair slot of (I, J).  A second kernel adds, for every body, its pair slots
// (tiles below its own) and then its receiver slots, in float-float, converted to FP64
// once.  No atomics touch the sums, so results are deterministic.
// Row groups (k_kick_mixed_sym_grp): a block of 2 or 4 warps takes as many consecutive
// rows against one strip, tile J by tile J, and adds its warps' partner sums of J in
// shared memory before writing them, so that one pair slot serves the whole group: fewer
// slot bytes to write and read back.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "kick_mixed.cuh"
#include "swg_internal.cuh"

namespace swg {

namespace {

constexpr int TS = KICK_SYM_TILE;  // bodies per tile by default (the single-system plan's tile)
constexpr int MAX_STRIP = 4;       // most tiles J per item (one row strip of the upper triangle)
constexpr float PAD_POS = 3.0e6f;  // position of the padding beyond a system's last body
constexpr unsigned FULL = 0xffffffffu;

// pair slot of tiles (I, J), I < J, among a system's nt tiles (row-major strict upper triangle)
__host__ __device__ __forceinline__ int pair_slot(int I, int J, int nt) {
    return I * (nt - 1) - I * (I - 1) / 2 + (J - I - 1);
}

// Shared layout of a staged 32-partner sub-tile: entry e (0 <= e < 48) holds partners
// a = e mod 32 and b = (e + 16) mod 32 side by side in four 16-byte words,
//   P[0][e] = (xh_a, xh_b, yh_a, yh_b)   P[1][e] = (zh_a, zh_b, Gm_a, Gm_b)
//   P[2][e] = (xl_a, xl_b, yl_a, yl_b)   P[3][e] = (zl_a, zl_b, R_a, R_b)
// so that each 64-bit half-word is the same quantity of the two partners, ready for the
// packed FP32 (f32x2) instructions.  Lane t reads entry t + s at step s (s < 16) without
// wrapping, i.e. partners t + s and t + s + 16 (mod 32): every partner once in 16 steps.
constexpr int PE = 48;  // entries per staged sub-tile
struct SubTile {
    ulonglong2 w[4][PE];
};

// Stage the sub-tile whose partner for this lane is (a, b) = (hi, Gm), (lo, R): lane t
// writes entry t and, for t < 16, entry t + 32 (the same two partners t, t + 16).
__device__ __forceinline__ void stage_subtile(SubTile &P, const float4 &a, const float4 &b, int lane) {
    const float4 xa = make_float4(__shfl_xor_sync(FULL, a.x, 16), __shfl_xor_sync(FULL, a.y, 16),
                                  __shfl_xor_sync(FULL, a.z, 16), __shfl_xor_sync(FULL, a.w, 16));
    const float4 xb = make_float4(__shfl_xor_sync(FULL, b.x, 16), __shfl_xor_sync(FULL, b.y, 16),
                                  __shfl_xor_sync(FULL, b.z, 16), __shfl_xor_sync(FULL, b.w, 16));
    // entry t = (partner t, partner (t + 16) mod 32), and (t + 16) mod 32 == t ^ 16
    const float4 lo_a = a, hi_a = xa, lo_b = b, hi_b = xb;
    const ulonglong2 w0 = make_ulonglong2(f2_pack(lo_a.x, hi_a.x), f2_pack(lo_a.y, hi_a.y));
    const ulonglong2 w1 = make_ulonglong2(f2_pack(lo_a.z, hi_a.z), f2_pack(lo_a.w, hi_a.w));
    const ulonglong2 w2 = make_ulonglong2(f2_pack(lo_b.x, hi_b.x), f2_pack(lo_b.y, hi_b.y));
    const ulonglong2 w3 = make_ulonglong2(f2_pack(lo_b.z, hi_b.z), f2_pack(lo_b.w, hi_b.w));
    P.w[0][lane] = w0;
    P.w[1][lane] = w1;
    P.w[2][lane] = w2;
    P.w[3][lane] = w3;
    if (lane < 16) {
        P.w[0][lane + 32] = w0;
        P.w[1][lane + 32] = w1;
        P.w[2][lane + 32] = w2;
        P.w[3][lane + 32] = w3;
    }
}

// A receiver of this lane in packed form: each coordinate (and the mass) in both halves.
struct Recv2 {
    f32x2 xh, yh, zh, xl, yl, zl, gm;
    float R;
};

// The pair rule on both halves: zero fi and fj of a pair within the radii (RAD) or, with
// jself >= 0, of the self pair (partner index jself within the sub-tile).
template <bool RAD>
__device__ __forceinline__ void rule2(f32x2 r2, f32x2 Rp, float Rk, int ja, int jb, int jself, f32x2 &fi, f32x2 &fj) {
    float r2a, r2b, fia, fib, fja, fjb;
    f2_unpack(r2, r2a, r2b);
    f2_unpack(fi, fia, fib);
    f2_unpack(fj, fja, fjb);
    bool oka, okb;
    if (RAD) {
        float Ra, Rb;
        f2_unpack(Rp, Ra, Rb);
        const float rsa = Rk + Ra, rsb = Rk + Rb;
        oka = r2a > rsa * rsa;
        okb = r2b > rsb * rsb;
    } else {
        oka = ja != jself;
        okb = jb != jself;
    }
    fi = f2_pack(oka ? fia : 0.f, okb ? fib : 0.f);
    fj = f2_pack(oka ? fja : 0.f, okb ? fjb : 0.f);
}

// 16 steps of one sub-tile for receivers k < NK of this lane (see the file comment): at
// step s the lane evaluates its receivers against its entry's two partners with the
// packed instructions, adds to packed receiver partials, and adds Gm_k r^-3 d to a packed
// accumulator of the two partners, which the warp rotates one lane down after the step.
// After 16 steps lane t holds partners (t + 16, t); the halves of each partner are joined
// across lanes t and t ^ 16.  Outputs: receiver partials px.. and minus the partner sums
// in qx.. (for this lane's partner t).  P points at the lane's first entry.
// GUARD: the pair rule pair by pair (RAD only); else, with RAD, mn keeps the smallest r^2.
// NR: receivers per lane (the tile's 32-body sub-tiles); K0: the first receiver taken
// (receivers K0 <= k < NK).
template <bool RAD, bool GUARD, int NK, int NR, int K0 = 0>
__device__ __forceinline__ void sym_subtile(const SubTile &S, int lane, const Recv2 (&q)[NR], int src, float (&px)[NR],
                                            float (&py)[NR], float (&pz)[NR], float &qx, float &qy, float &qz,
                                            float (&mn)[NR]) {
    f32x2 ax[NK], ay[NK], az[NK];
#pragma unroll
    for (int k = K0; k < NK; k++) {
        ax[k] = ay[k] = az[k] = 0ull;
        mn[k] = 3.0e38f;
    }
    f32x2 bx = 0ull, by = 0ull, bz = 0ull;
    const f32x2 c15 = f2_pack(-1.5f, -1.5f), c25 = f2_pack(2.5f, 2.5f);
    const ulonglong2 *W0 = S.w[0] + lane, *W1 = S.w[1] + lane, *W2 = S.w[2] + lane, *W3 = S.w[3] + lane;
#pragma unroll 4
    for (int s = 0; s < 16; s++) {
        const ulonglong2 h = W0[s], hz = W1[s], l = W2[s], lz = W3[s];
#pragma unroll
        for (int k = K0; k < NK; k++) {
            const f32x2 dx = f2_add(f2_sub(h.x, q[k].xh), f2_sub(l.x, q[k].xl));
            const f32x2 dy = f2_add(f2_sub(h.y, q[k].yh), f2_sub(l.y, q[k].yl));
            const f32x2 dz = f2_add(f2_sub(hz.x, q[k].zh), f2_sub(lz.x, q[k].zl));
            const f32x2 r2 = f2_fma(dz, dz, f2_fma(dy, dy, f2_mul(dx, dx)));
            float r2a, r2b;
            f2_unpack(r2, r2a, r2b);
            const f32x2 y = f2_pack(rsqrt_approx(r2a), rsqrt_approx(r2b));
            const f32x2 t = f2_mul(y, y);
            const f32x2 r3 = f2_mul(f2_mul(t, y), f2_fma(c15, f2_mul(r2, t), c25));
            f32x2 fi = f2_mul(hz.y, r3), fj = f2_mul(q[k].gm, r3);
            if (RAD && GUARD) rule2<true>(r2, lz.y, q[k].R, 0, 0, -1, fi, fj);
            if (RAD && !GUARD) mn[k] = fminf(mn[k], fminf(r2a, r2b));
            ax[k] = f2_fma(fi, dx, ax[k]);
            ay[k] = f2_fma(fi, dy, ay[k]);
            az[k] = f2_fma(fi, dz, az[k]);
            bx = f2_fma(fj, dx, bx);
            by = f2_fma(fj, dy, by);
            bz = f2_fma(fj, dz, bz);
        }
        bx = __shfl_sync(FULL, bx, src);
        by = __shfl_sync(FULL, by, src);
        bz = __shfl_sync(FULL, bz, src);
    }
#pragma unroll
    for (int k = K0; k < NK; k++) {
        float e, o;
        f2_unpack(ax[k], e, o);
        px[k] = e + o;
        f2_unpack(ay[k], e, o);
        py[k] = e + o;
        f2_unpack(az[k], e, o);
        pz[k] = e + o;
    }
    float lo, hi;
    f2_unpack(bx, lo, hi);
    qx = -(hi + __shfl_xor_sync(FULL, lo, 16));
    f2_unpack(by, lo, hi);
    qy = -(hi + __shfl_xor_sync(FULL, lo, 16));
    f2_unpack(bz, lo, hi);
    qz = -(hi + __shfl_xor_sync(FULL, lo, 16));
}

// sym_subtile without the rule, then (RAD) recomputed with it when some receiver
// K0 <= k < NK may meet a partner within the radii.
template <bool RAD, int NK, int NR, int K0 = 0>
__device__ __forceinline__ void sym_subtile_ruled(const SubTile &S, int lane, const Recv2 (&q)[NR],
                                                  const bool (&ok)[NR], int src, float (&px)[NR], float (&py)[NR],
                                                  float (&pz)[NR], float &qx, float &qy, float &qz) {
    float mn[NR];
    sym_subtile<RAD, false, NK, NR, K0>(S, lane, q, src, px, py, pz, qx, qy, qz, mn);
    if (RAD) {
        float Ra, Rb;
        f2_unpack(S.w[3][lane].y, Ra, Rb);  // the lane's entry: partners lane and lane ^ 16
        const float rt = __uint_as_float(__reduce_max_sync(FULL, __float_as_uint(fmaxf(Ra, Rb))));  // radii >= 0
        bool need = false;
#pragma unroll
        for (int k = K0; k < NK; k++) {
            const float rs = q[k].R + rt;
            need = need || (ok[k] && mn[k] <= rs * rs);
        }
        if (__any_sync(FULL, need))  // rare: a pair may lie within the radii
            sym_subtile<RAD, true, NK, NR, K0>(S, lane, q, src, px, py, pz, qx, qy, qz, mn);
    }
}

__device__ __forceinline__ void ff_add3(FF &x, FF &y, FF &z, float a, float b, float c) {
    ff_add(x, a);
    ff_add(y, b);
    ff_add(z, c);
}

// Receiver k of this lane (body 32 k + lane of the diagonal tile) against its own
// sub-tile, one-sided with the pair rule applied pair by pair (the self pair, and with RAD
// the radius rule): partners lane + s and lane + s + 16 at step s.
template <bool RAD>
__device__ __forceinline__ void own_subtile(const SubTile &S, int lane, const Recv2 &q, float &sx, float &sy,
                                            float &sz) {
    f32x2 ax = 0ull, ay = 0ull, az = 0ull;
    const f32x2 c15 = f2_pack(-1.5f, -1.5f), c25 = f2_pack(2.5f, 2.5f);
    const ulonglong2 *W0 = S.w[0] + lane, *W1 = S.w[1] + lane, *W2 = S.w[2] + lane, *W3 = S.w[3] + lane;
#pragma unroll 4
    for (int s = 0; s < 16; s++) {
        const ulonglong2 h = W0[s], hz = W1[s], l = W2[s], lz = W3[s];
        const f32x2 dx = f2_add(f2_sub(h.x, q.xh), f2_sub(l.x, q.xl));
        const f32x2 dy = f2_add(f2_sub(h.y, q.yh), f2_sub(l.y, q.yl));
        const f32x2 dz = f2_add(f2_sub(hz.x, q.zh), f2_sub(lz.x, q.zl));
        const f32x2 r2 = f2_fma(dz, dz, f2_fma(dy, dy, f2_mul(dx, dx)));
        float r2a, r2b;
        f2_unpack(r2, r2a, r2b);
        const f32x2 y = f2_pack(rsqrt_approx(r2a), rsqrt_approx(r2b));
        const f32x2 t = f2_mul(y, y);
        const f32x2 r3 = f2_mul(f2_mul(t, y), f2_fma(c15, f2_mul(r2, t), c25));
        f32x2 fi = f2_mul(hz.y, r3), fj = 0ull;
        rule2<RAD>(r2, lz.y, q.R, (lane + s) & 31, (lane + s + 16) & 31, lane, fi, fj);
        ax = f2_fma(fi, dx, ax);
        ay = f2_fma(fi, dy, ay);
        az = f2_fma(fi, dz, az);
    }
    float e, o;
    f2_unpack(ax, e, o);
    sx = e + o;
    f2_unpack(ay, e, o);
    sy = e + o;
    f2_unpack(az, e, o);
    sz = e + o;
}

// Sub-tile U of a diagonal tile (I == J): receivers k < U against it with the rotation,
// whose partner sums belong to receiver U of this lane, and receiver U against it
// one-sided with the pair rule.
template <bool RAD, int U, int NR>
__device__ __forceinline__ void diag_subtile(const SubTile (&sP)[NR], const Recv2 (&q)[NR], const bool (&ok)[NR],
                                             int lane, FF (&ax)[NR], FF (&ay)[NR], FF (&az)[NR]) {
    float qx = 0.f, qy = 0.f, qz = 0.f;
    if constexpr (U > 0) {
        float px[NR], py[NR], pz[NR];
        sym_subtile_ruled<RAD, U, NR>(sP[U], lane, q, ok, (lane + 1) & 31, px, py, pz, qx, qy, qz);
#pragma unroll
        for (int k = 0; k < U; k++) ff_add3(ax[k], ay[k], az[k], px[k], py[k], pz[k]);
    }
    float sx, sy, sz;
    own_subtile<RAD>(sP[U], lane, q[U], sx, sy, sz);
    ff_add3(ax[U], ay[U], az[U], sx, sy, sz);
    if (U > 0) ff_add3(ax[U], ay[U], az[U], qx, qy, qz);
}

// Item: (system, tile I, first tile J0 | tiles nJ << 24, receiver slot).  pA/pB: every
// body split into (x_hi, y_hi, z_hi, Gm), (x_lo, y_lo, z_lo, R).  A receiver slot is
// [x_hi, x_lo, y_hi, y_lo, z_hi, z_lo] x T floats, a pair slot [x, y, z] x T floats.
// W warps per block, each an independent worker with its own staged tile (the block size
// only changes how the warps are packed on the SMs; every item's arithmetic is the same).
// T bodies per tile: 128 (four receivers per lane) or 64 (two).
template <bool RAD, int W, int T>
__global__ void __launch_bounds__(32 * W) k_kick_mixed_sym(int nitems, const int4 *__restrict__ items,
                                                      const int32_t *__restrict__ poff,
                                                      const int32_t *__restrict__ npl,
                                                      const int32_t *__restrict__ sbase,
                                                      const float4 *__restrict__ pA, const float4 *__restrict__ pB,
                                                      float *__restrict__ rpart, float *__restrict__ ppart,
                                                      unsigned *__restrict__ head,
                                                      const int32_t *__restrict__ sys_flag, int phase,
                                                      const uint8_t *__restrict__ iflag, unsigned accept) {
    constexpr int SR = T / 32;  // receivers per lane = 32-body sub-tiles per tile
    static_assert(SR == 2 || SR == 4, "tiles of 64 or 128 bodies");
    __shared__ SubTile sPw[W][SR];
    SubTile(&sP)[SR] = sPw[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const float4 pad_a = make_float4(PAD_POS, PAD_POS, PAD_POS, 0.f), zero = make_float4(0.f, 0.f, 0.f, 0.f);
    for (;;) {
        unsigned it = 0;
        if (lane == 0) it = atomicAdd(head, 1u);
        it = __shfl_sync(FULL, it, 0);
        if (it >= (unsigned)nitems) break;
        const int4 w = items[it];
        const int s = w.x, I = w.y, J0 = w.z & 0xffffff, nJ = w.z >> 24;
        if (sys_flag && sys_flag[s] != phase) continue;  // warp-uniform
        if (iflag && !((accept >> iflag[it]) & 1u)) continue;
        const int p0 = poff[s], n = npl[s], nt = (n + T - 1) / T;
        Recv2 q[SR];
        bool ok[SR];
#pragma unroll
        for (int k = 0; k < SR; k++) {
            const int i = I * T + k * 32 + lane;
            ok[k] = i < n;
            const float4 a = ok[k] ? pA[p0 + i] : pad_a;
            const float4 b = ok[k] ? pB[p0 + i] : zero;
            q[k] = Recv2{f2_pack(a.x, a.x), f2_pack(a.y, a.y), f2_pack(a.z, a.z), f2_pack(b.x, b.x),
                         f2_pack(b.y, b.y), f2_pack(b.z, b.z), f2_pack(a.w, a.w), b.w};
        }
        FF ax[SR], ay[SR], az[SR];
#pragma unroll
        for (int k = 0; k < SR; k++) ax[k] = ay[k] = az[k] = FF{0.f, 0.f};
        for (int jj = 0; jj < nJ; jj++) {
            const int J = J0 + jj;
            __syncwarp();  // the previous tile's shared data is consumed
#pragma unroll
            for (int u = 0; u < SR; u++) {
                const int j = J * T + u * 32 + lane;
                const float4 a = j < n ? pA[p0 + j] : pad_a;
                const float4 b = j < n ? pB[p0 + j] : zero;
                stage_subtile(sP[u], a, b, lane);
            }
            __syncwarp();
            if (I == J) {
                diag_subtile<RAD, 0, SR>(sP, q, ok, lane, ax, ay, az);
                diag_subtile<RAD, 1, SR>(sP, q, ok, lane, ax, ay, az);
                if constexpr (SR > 2) {
                    diag_subtile<RAD, 2, SR>(sP, q, ok, lane, ax, ay, az);
                    diag_subtile<RAD, 3, SR>(sP, q, ok, lane, ax, ay, az);
                }
                continue;
            }
            float *o1 = ppart + (size_t)(sbase[2 * s + 1] + pair_slot(I, J, nt)) * 3 * T;
            for (int u = 0; u < SR; u++) {
                float px[SR], py[SR], pz[SR], qx, qy, qz;
                sym_subtile_ruled<RAD, SR, SR>(sP[u], lane, q, ok, (lane + 1) & 31, px, py, pz, qx, qy, qz);
#pragma unroll
                for (int k = 0; k < SR; k++) ff_add3(ax[k], ay[k], az[k], px[k], py[k], pz[k]);
                o1[0 * T + u * 32 + lane] = qx;
                o1[1 * T + u * 32 + lane] = qy;
                o1[2 * T + u * 32 + lane] = qz;
            }
        }
        float *o0 = rpart + (size_t)w.w * 6 * T;
#pragma unroll
        for (int k = 0; k < SR; k++) {
            const int il = k * 32 + lane;
            o0[0 * T + il] = ax[k].hi;
            o0[1 * T + il] = ax[k].lo;
            o0[2 * T + il] = ay[k].hi;
            o0[3 * T + il] = ay[k].lo;
            o0[4 * T + il] = az[k].hi;
            o0[5 * T + il] = az[k].lo;
        }
    }
}

// Row groups of G tiles (128 bodies): an item is G consecutive receiver tiles
// I0 .. I0 + G - 1 (warp w of the block holds tile I0 + w) against a strip of tiles
// J0 .. J0 + nJ - 1 (J0 >= I0), processed one tile J at a time by the whole block: J is
// staged once in shared memory (each warp stages G-th of its sub-tiles), every warp
// evaluates its tile against it (I < J with the rotation, I == J as a diagonal tile,
// I > J not at all), and the warps' partner sums of J are added in warp order into the
// pair slot (g, J) of the row group g = I0 / G, J > I0.  A row group thus writes one pair
// slot per tile J where rows of one tile write G, so G times fewer pair slots go to memory
// and come back in the per-body sums.  Each warp's receiver sums of the strip go to
// receiver slot w.w + w.  Every body's terms are the same as with one-row items, grouped
// into different partial sums (the results agree within the mixed-kick tolerance); each
// launch gives the same bits.
// With G = 2 the first two tiles of a group's first strip (the diagonal block: tiles I0 and
// I0 + 1 on themselves and against each other) are one round in which both warps work:
// warp 0 takes diagonal tile I0 and tile I0 against sub-tiles 0-1 of tile I0 + 1, warp 1
// diagonal tile I0 + 1 and its sub-tiles 2-3 as receivers against tile I0 (staged apart),
// whose partner sums warp 0 adds to its receiver sums; in step, one warp would wait for the
// other on each of these two tiles.
template <bool RAD, int G>
__global__ void __launch_bounds__(32 * G) k_kick_mixed_sym_grp(int nitems, const int4 *__restrict__ items,
                                                          const int32_t *__restrict__ poff,
                                                          const int32_t *__restrict__ npl,
                                                          const int32_t *__restrict__ sbase,
                                                          const float4 *__restrict__ pA,
                                                          const float4 *__restrict__ pB, float *__restrict__ rpart,
                                                          float *__restrict__ ppart, unsigned *__restrict__ head,
                                                          const int32_t *__restrict__ sys_flag, int phase,
                                                          const uint8_t *__restrict__ iflag, unsigned accept) {
    constexpr int T = KICK_SYM_TILE, SR = T / 32;
    static_assert(G == 2 || G == 4, "row groups of 2 or 4 tiles");
    __shared__ SubTile sP[SR];
    __shared__ float sq[G][3 * T];  // partner sums of the staged tile J, one row per warp
    __shared__ unsigned s_it[2];    // the item of each pull (two buffers: one barrier per pull)
    __shared__ SubTile sP0[G == 2 ? SR : 1];  // G = 2: tile I0 in the diagonal round
    __shared__ float sq0[G == 2 ? 3 * T : 1];  // G = 2: partner sums for tile I0 from warp 1
    const int wq = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const float4 pad_a = make_float4(PAD_POS, PAD_POS, PAD_POS, 0.f), zero = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int buf = 0;; buf ^= 1) {
        if (threadIdx.x == 0) s_it[buf] = atomicAdd(head, 1u);
        __syncthreads();
        const unsigned it = s_it[buf];
        if (it >= (unsigned)nitems) break;  // block-uniform, as are the two skips below
        const int4 w = items[it];
        const int s = w.x, I0 = w.y, J0 = w.z & 0xffffff, nJ = w.z >> 24;
        if (sys_flag && sys_flag[s] != phase) continue;
        if (iflag && !((accept >> iflag[it]) & 1u)) continue;
        const int p0 = poff[s], n = npl[s], nt = (n + T - 1) / T, I = I0 + wq, g = I0 / G;
        // pair slot (g, J) = pbase + J: the groups before g hold nt - g'G - 1 slots each
        const int pbase = sbase[2 * s + 1] + g * (nt - 1) - G * g * (g - 1) / 2 - I0 - 1;
        Recv2 q[SR];
        bool ok[SR];
#pragma unroll
        for (int k = 0; k < SR; k++) {
            const int i = I * T + k * 32 + lane;
            ok[k] = i < n;
            const float4 a = ok[k] ? pA[p0 + i] : pad_a;
            const float4 b = ok[k] ? pB[p0 + i] : zero;
            q[k] = Recv2{f2_pack(a.x, a.x), f2_pack(a.y, a.y), f2_pack(a.z, a.z), f2_pack(b.x, b.x),
                         f2_pack(b.y, b.y), f2_pack(b.z, b.z), f2_pack(a.w, a.w), b.w};
        }
        FF ax[SR], ay[SR], az[SR];
#pragma unroll
        for (int k = 0; k < SR; k++) ax[k] = ay[k] = az[k] = FF{0.f, 0.f};
        int jj0 = 0;
        if constexpr (G == 2) {
            if (J0 == I0 && nJ >= 2 && I0 + 1 < nt) {  // the diagonal round (block-uniform)
                SubTile(&own)[SR] = wq == 0 ? sP0 : sP;  // warp w stages its own tile I0 + w
#pragma unroll
                for (int u = 0; u < SR; u++) {
                    const int j = I * T + u * 32 + lane;
                    const float4 a = j < n ? pA[p0 + j] : pad_a;
                    const float4 b = j < n ? pB[p0 + j] : zero;
                    stage_subtile(own[u], a, b, lane);
                }
                __syncthreads();
                diag_subtile<RAD, 0, SR>(own, q, ok, lane, ax, ay, az);
                diag_subtile<RAD, 1, SR>(own, q, ok, lane, ax, ay, az);
                diag_subtile<RAD, 2, SR>(own, q, ok, lane, ax, ay, az);
                diag_subtile<RAD, 3, SR>(own, q, ok, lane, ax, ay, az);
                if (wq == 0) {
                    for (int u = 0; u < SR; u++) {
                        float qx = 0.f, qy = 0.f, qz = 0.f;
                        if (u < 2) {
                            float px[SR], py[SR], pz[SR];
                            sym_subtile_ruled<RAD, SR, SR>(sP[u], lane, q, ok, (lane + 1) & 31, px, py, pz, qx, qy,
                                                           qz);
#pragma unroll
                            for (int k = 0; k < SR; k++) ff_add3(ax[k], ay[k], az[k], px[k], py[k], pz[k]);
                        }
                        sq[0][0 * T + u * 32 + lane] = qx;
                        sq[0][1 * T + u * 32 + lane] = qy;
                        sq[0][2 * T + u * 32 + lane] = qz;
                    }
                } else {
                    for (int u = 0; u < SR; u++) {
                        float px[SR], py[SR], pz[SR], qx, qy, qz;
                        sym_subtile_ruled<RAD, SR, SR, 2>(sP0[u], lane, q, ok, (lane + 1) & 31, px, py, pz, qx, qy,
                                                          qz);
#pragma unroll
                        for (int k = 2; k < SR; k++) ff_add3(ax[k], ay[k], az[k], px[k], py[k], pz[k]);
                        sq0[0 * T + u * 32 + lane] = qx;
                        sq0[1 * T + u * 32 + lane] = qy;
                        sq0[2 * T + u * 32 + lane] = qz;
                    }
                }
                __syncthreads();
                float *o = ppart + (size_t)(pbase + I0 + 1) * 3 * T;  // pair slot (g, I0 + 1): warp 0's sums
                for (int e = threadIdx.x; e < 3 * T; e += 32 * G) o[e] = sq[0][e];
                if (wq == 0) {
#pragma unroll
                    for (int u = 0; u < SR; u++)
                        ff_add3(ax[u], ay[u], az[u], sq0[u * 32 + lane], sq0[T + u * 32 + lane],
                                sq0[2 * T + u * 32 + lane]);
                }
                jj0 = 2;
            }
        }
        for (int jj = jj0; jj < nJ; jj++) {
            const int J = J0 + jj;
            for (int u = wq; u < SR; u += G) {
                const int j = J * T + u * 32 + lane;
                const float4 a = j < n ? pA[p0 + j] : pad_a;
                const float4 b = j < n ? pB[p0 + j] : zero;
                stage_subtile(sP[u], a, b, lane);
            }
            __syncthreads();  // J staged; the previous tile's partner sums are consumed
            if (I == J) {
                diag_subtile<RAD, 0, SR>(sP, q, ok, lane, ax, ay, az);
                diag_subtile<RAD, 1, SR>(sP, q, ok, lane, ax, ay, az);
                diag_subtile<RAD, 2, SR>(sP, q, ok, lane, ax, ay, az);
                diag_subtile<RAD, 3, SR>(sP, q, ok, lane, ax, ay, az);
            } else if (I < J) {
                for (int u = 0; u < SR; u++) {
                    float px[SR], py[SR], pz[SR], qx, qy, qz;
                    sym_subtile_ruled<RAD, SR, SR>(sP[u], lane, q, ok, (lane + 1) & 31, px, py, pz, qx, qy, qz);
#pragma unroll
                    for (int k = 0; k < SR; k++) ff_add3(ax[k], ay[k], az[k], px[k], py[k], pz[k]);
                    sq[wq][0 * T + u * 32 + lane] = qx;
                    sq[wq][1 * T + u * 32 + lane] = qy;
                    sq[wq][2 * T + u * 32 + lane] = qz;
                }
            }
            __syncthreads();  // partner sums of J complete; the staged tile is free
            if (J > I0) {
                const int nw = min(G, J - I0);  // warps whose tile lies below J
                float *o = ppart + (size_t)(pbase + J) * 3 * T;
                for (int e = threadIdx.x; e < 3 * T; e += 32 * G) {
                    float v = sq[0][e];
                    for (int m = 1; m < nw; m++) v += sq[m][e];
                    o[e] = v;
                }
            }
        }
        if (I < nt) {
            float *o0 = rpart + (size_t)(w.w + wq) * 6 * T;
#pragma unroll
            for (int k = 0; k < SR; k++) {
                const int il = k * 32 + lane;
                o0[0 * T + il] = ax[k].hi;
                o0[1 * T + il] = ax[k].lo;
                o0[2 * T + il] = ay[k].hi;
                o0[3 * T + il] = ay[k].lo;
                o0[4 * T + il] = az[k].hi;
                o0[5 * T + il] = az[k].lo;
            }
        }
    }
}

// One warp per item: 0 for a system without encounters, else 2 when one of the item's
// receiver tiles (grp of them from tile I) or one of the strip's tiles J holds a body
// marked in enc, else 1 (see kick_sym_item_flags).
__global__ void k_kick_sym_item_flags(int nitems, const int4 *__restrict__ items, const int32_t *__restrict__ poff,
                                      const int32_t *__restrict__ npl, const int32_t *__restrict__ sys_enc,
                                      const uint8_t *__restrict__ enc, uint8_t *__restrict__ iflag, int ts, int grp) {
    const int it = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (it >= nitems) return;  // whole warps leave together
    const int4 w = items[it];
    const int s = w.x, I = w.y, J0 = w.z & 0xffffff, nJ = w.z >> 24;
    if (!sys_enc[s]) {
        if (lane == 0) iflag[it] = 0;
        return;
    }
    const int p0 = poff[s], n = npl[s];
    bool dirty = false;
    for (int t = -grp; t < nJ; t++) {
        const int T = t < 0 ? I + grp + t : J0 + t;
        for (int k = lane; k < ts; k += 32) {
            const int i = T * ts + k;
            if (i < n && enc[p0 + i]) dirty = true;
        }
    }
    dirty = __any_sync(FULL, dirty);
    if (lane == 0) iflag[it] = dirty ? 2 : 1;
}

// Per body: acc (+)= its slots in a fixed order (pair slots of the row groups below its
// tile, in group order, then the receiver slots of its own tile's items).  The slots'
// values are added in float-float (hi parts by TwoSum, lo parts plainly) and converted to
// FP64 once: FP64 arithmetic per slot would run on the narrow FP64 pipe and bound this
// kernel.  grp: tiles per row group (1: one-row items, whose pair slot (g, K) is
// pair_slot(g, K, nt)); a group g holds nt - g grp - 1 pair slots and one item per strip
// of its tiles J >= g grp, each item grp receiver slots.
__global__ void k_kick_sym_reduce(int64_t n, const int32_t *__restrict__ psys, const int32_t *__restrict__ poff,
                                  const int32_t *__restrict__ npl, const int32_t *__restrict__ sbase,
                                  const float *__restrict__ rpart, const float *__restrict__ ppart,
                                  double *__restrict__ acc, int acc_is_zero, const int32_t *__restrict__ sys_flag,
                                  int phase, int strip, int ts, int grp) {
    const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b >= n) return;
    const int s = psys ? psys[b] : 0;
    if (sys_flag && sys_flag[s] != phase) return;
    const int i = (int)(b - poff[s]);
    const int nt = (npl[s] + ts - 1) / ts, K = i / ts, l = i % ts, gK = K / grp;
    FF fx{0.f, 0.f}, fy{0.f, 0.f}, fz{0.f, 0.f};
    float lx = 0.f, ly = 0.f, lz = 0.f;
    int pslot = sbase[2 * s + 1];  // first pair slot of group g
    int row = 0;                   // items of the groups before gK
    for (int g = 0; g <= gK; g++) {
        const int I0 = g * grp;
        if (I0 < K) {
            const float *o = ppart + (size_t)(pslot + K - I0 - 1) * 3 * ts;
            ff_add3(fx, fy, fz, o[l], o[ts + l], o[2 * ts + l]);
        }
        if (g < gK) {
            pslot += nt - I0 - 1;
            row += (nt - I0 + strip - 1) / strip;
        }
    }
    for (int m = 0; m < (nt - gK * grp + strip - 1) / strip; m++) {
        const float *o = rpart + ((size_t)(sbase[2 * s] + (row + m) * grp + K - gK * grp)) * 6 * ts;
        ff_add3(fx, fy, fz, o[l], o[2 * ts + l], o[4 * ts + l]);
        lx += o[ts + l];
        ly += o[3 * ts + l];
        lz += o[5 * ts + l];
    }
    const double sx = (double)fx.hi + ((double)fx.lo + (double)lx);
    const double sy = (double)fy.hi + ((double)fy.lo + (double)ly);
    const double sz = (double)fz.hi + ((double)fz.lo + (double)lz);
    double *a = acc + 3 * b;
    a[0] = (acc_is_zero ? 0.0 : a[0]) + sx;
    a[1] = (acc_is_zero ? 0.0 : a[1]) + sy;
    a[2] = (acc_is_zero ? 0.0 : a[2]) + sz;
}

}  // namespace

int kick_sym_item_flags(swg_ctx *c, int nitems, const int4 *items, const int32_t *poff, const int32_t *npl,
                        const int32_t *sys_enc, const uint8_t *enc, uint8_t *iflag, int tile, int group) {
    if (nitems <= 0) return SWG_OK;
    const int64_t threads = (int64_t)nitems * 32;
    k_kick_sym_item_flags<<<(int)((threads + 255) / 256), 256, 0, c->stream>>>(nitems, items, poff, npl, sys_enc,
                                                                              enc, iflag, tile, group);
    c->launches++;
    return launch_status(c, "kick_sym_item_flags");
}

int kick_sym_strip(int32_t nsys, const int32_t *npl, int num_sms, int tile) {
    int64_t pairs = 0;
    for (int s = 0; s < nsys; s++) {
        const int64_t nt = (npl[s] + tile - 1) / tile;
        pairs += nt * (nt + 1) / 2;
    }
    // strips of MAX_STRIP measured fastest whenever they leave a few items per SM; shorter
    // strips only when the work would not spread over the SMs otherwise
    return pairs >= 4 * MAX_STRIP * (int64_t)(num_sms > 0 ? num_sms : 152) ? MAX_STRIP : 1;
}

bool kick_sym_single_ok(int32_t npl, int num_sms) {
    const int64_t nt = (npl + TS - 1) / TS;
    return nt * (nt + 1) / 2 >= 32 * (int64_t)(num_sms > 0 ? num_sms : 152);
}

int64_t kick_sym_items(int32_t nsys, const int32_t *npl, int strip, std::vector<int4> &items,
                       std::vector<int32_t> &sbase, int64_t *npair_slots, int tile, int group) {
    items.clear();
    sbase.assign(2 * (size_t)nsys, 0);
    std::vector<int64_t> cost;
    int64_t nrs = 0, nps = 0;
    for (int s = 0; s < nsys; s++) {
        const int nt = (npl[s] + tile - 1) / tile;
        sbase[2 * s] = (int32_t)nrs;
        sbase[2 * s + 1] = (int32_t)nps;
        auto rows = [&](int T) { return (int64_t)std::min(tile, npl[s] - T * tile); };
        for (int I0 = 0; I0 < nt; I0 += group) {
            for (int J0 = I0; J0 < nt; J0 += strip) {
                const int nJ = std::min(strip, nt - J0);
                items.push_back(make_int4(s, I0, J0 | (nJ << 24), (int)nrs));
                nrs += group;
                // a row group's warps go through the strip's tiles J together: each J costs
                // the largest of its rows' shares
                int64_t c = 0;
                for (int J = J0; J < J0 + nJ; J++) {
                    int64_t m = 0;
                    for (int I = I0; I < std::min(I0 + group, nt) && I <= J; I++) m = std::max(m, rows(I));
                    c += m * rows(J);
                }
                cost.push_back(c);
            }
            nps += nt - I0 - 1;
        }
    }
    std::vector<size_t> ord(items.size());
    for (size_t k = 0; k < ord.size(); k++) ord[k] = k;
    std::stable_sort(ord.begin(), ord.end(), [&](size_t a, size_t b) { return cost[a] > cost[b]; });
    std::vector<int4> sorted(items.size());
    for (size_t k = 0; k < ord.size(); k++) sorted[k] = items[ord[k]];
    items.swap(sorted);
    *npair_slots = nps;
    return nrs;
}

template <bool RAD, int W, int T>
int sym_launch(swg_ctx *c, int nitems, const int4 *items, const int32_t *poff, const int32_t *npl,
               const int32_t *sbase, const float4 *pA, const float4 *pB, float *rpart, float *ppart, unsigned *head,
               const int32_t *sys_flag, int phase, const uint8_t *iflag, unsigned accept) {
    static int o = 0;  // resident blocks per SM, queried once per variant
    if (o == 0) {
        int nb = 0;
        SWG_TRY(cuda_status(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_kick_mixed_sym<RAD, W, T>, 32 * W, 0),
                            "occupancy"));
        o = nb > 0 ? nb : 1;
    }
    const int grid = std::min((nitems + W - 1) / W, o * (c->num_sms > 0 ? c->num_sms : 152));
    k_kick_mixed_sym<RAD, W, T><<<grid, 32 * W, 0, c->stream>>>(nitems, items, poff, npl, sbase, pA, pB, rpart, ppart,
                                                              head, sys_flag, phase, iflag, accept);
    return SWG_OK;
}

template <bool RAD, int G>
int sym_grp_launch(swg_ctx *c, int nitems, const int4 *items, const int32_t *poff, const int32_t *npl,
                   const int32_t *sbase, const float4 *pA, const float4 *pB, float *rpart, float *ppart, unsigned *head,
                   const int32_t *sys_flag, int phase, const uint8_t *iflag, unsigned accept) {
    static int o = 0;  // resident blocks per SM, queried once per variant
    if (o == 0) {
        int nb = 0;
        SWG_TRY(cuda_status(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_kick_mixed_sym_grp<RAD, G>, 32 * G, 0),
                            "occupancy"));
        o = nb > 0 ? nb : 1;
    }
    const int grid = std::min(nitems, o * (c->num_sms > 0 ? c->num_sms : 152));
    k_kick_mixed_sym_grp<RAD, G><<<grid, 32 * G, 0, c->stream>>>(nitems, items, poff, npl, sbase, pA, pB, rpart, ppart,
                                                               head, sys_flag, phase, iflag, accept);
    return SWG_OK;
}

int kick_mixed_sym_batched(swg_ctx *c, bool rad, int nitems, const int4 *items, const int32_t *poff,
                           const int32_t *npl, const int32_t *sbase, const float4 *pA, const float4 *pB, float *rpart,
                           float *ppart, unsigned *head, const int32_t *sys_flag, int phase, const uint8_t *iflag,
                           unsigned accept, int warps, int tile, int group) {
    if (nitems <= 0) return SWG_OK;
    if ((warps != 1 && warps != 2 && warps != 4) || (tile != 64 && tile != 128) ||
        (group != 1 && group != 2 && group != 4) || (group > 1 && tile != KICK_SYM_TILE))
        return SWG_ERR_ARG;
    SWG_TRY(cuda_status(c, cudaMemsetAsync(head, 0, sizeof(unsigned), c->stream), "memset"));
#define SWG_SYM_ARGS c, nitems, items, poff, npl, sbase, pA, pB, rpart, ppart, head, sys_flag, phase, iflag, accept
    // 64-body tiles run with one warp per block (the block size is tuned on 128-body tiles);
    // row groups take one warp per tile of the group
    int rc;
    if (group == 2)
        rc = rad ? sym_grp_launch<true, 2>(SWG_SYM_ARGS) : sym_grp_launch<false, 2>(SWG_SYM_ARGS);
    else if (group == 4)
        rc = rad ? sym_grp_launch<true, 4>(SWG_SYM_ARGS) : sym_grp_launch<false, 4>(SWG_SYM_ARGS);
    else if (tile == 64)
        rc = rad ? sym_launch<true, 1, 64>(SWG_SYM_ARGS) : sym_launch<false, 1, 64>(SWG_SYM_ARGS);
    else if (rad)
        rc = warps == 1 ? sym_launch<true, 1, 128>(SWG_SYM_ARGS)
                        : (warps == 2 ? sym_launch<true, 2, 128>(SWG_SYM_ARGS) : sym_launch<true, 4, 128>(SWG_SYM_ARGS));
    else
        rc = warps == 1 ? sym_launch<false, 1, 128>(SWG_SYM_ARGS)
                        : (warps == 2 ? sym_launch<false, 2, 128>(SWG_SYM_ARGS) : sym_launch<false, 4, 128>(SWG_SYM_ARGS));
#undef SWG_SYM_ARGS
    SWG_TRY(rc);
    c->launches++;
    return launch_status(c, "kick_mixed_sym");
}

int kick_mixed_sym_reduce(swg_ctx *c, int strip, int64_t n, const int32_t *psys, const int32_t *poff,
                          const int32_t *npl, const int32_t *sbase, const float *rpart, const float *ppart,
                          double *acc, int acc_is_zero, const int32_t *sys_flag, int phase, int tile, int group) {
    if (n <= 0) return SWG_OK;
    k_kick_sym_reduce<<<(int)((n + 255) / 256), 256, 0, c->stream>>>(n, psys, poff, npl, sbase, rpart, ppart, acc,
                                                                      acc_is_zero, sys_flag, phase, strip, tile, group);
    c->launches++;
    return launch_status(c, "kick_sym_reduce");
}

// ---- one system (the C ABI kicks and the single-system step loops)
// Plan of the last system size seen by the context: items, [poff = 0, npl, slot bases],
// slots, split partners and a queue head.
struct SymSingle {
    int32_t npl = -1;
    int nitems = 0, strip = 1;
    int4 *items = nullptr;
    int32_t *meta = nullptr;
    float *part = nullptr, *ppart = nullptr;
    float4 *pA = nullptr, *pB = nullptr;
    unsigned *head = nullptr;
    void release() {
        void *ptrs[] = {items, meta, part, pA, pB, head};
        for (void *p : ptrs)
            if (p) cudaFree(p);
        *this = SymSingle();
    }
};

void kick_sym_single_free(swg_ctx *c) {
    if (!c->sym_single) return;
    SymSingle *p = (SymSingle *)c->sym_single;
    p->release();
    delete p;
    c->sym_single = nullptr;
}

template <typename T>
static int sym_alloc(swg_ctx *c, T **p, size_t n) {
    const cudaError_t e = cudaMalloc((void **)p, (n ? n : 1) * sizeof(T));
    if (e != cudaSuccess) {
        c->err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
        return SWG_ERR_NOMEM;
    }
    return SWG_OK;
}

int kick_mixed_sym_single(swg_ctx *c, int32_t npl, const double *r, const double *Gm, const double *R, double *acc,
                          int acc_is_zero) {
    if (npl <= 0) return SWG_OK;
    if (!c->sym_single) c->sym_single = new SymSingle();
    SymSingle &p = *(SymSingle *)c->sym_single;
    if (p.npl != npl) {
        SWG_TRY(cuda_status(c, cudaStreamSynchronize(c->stream), "sync"));
        p.release();
        std::vector<int4> items;
        std::vector<int32_t> base;
        int64_t npair = 0;
        p.strip = kick_sym_strip(1, &npl, c->num_sms, TS);
        const int64_t nrecv = kick_sym_items(1, &npl, p.strip, items, base, &npair, TS);
        const int32_t meta[4] = {0, npl, base[0], base[1]};
        SWG_TRY(sym_alloc(c, &p.items, items.size()));
        SWG_TRY(sym_alloc(c, &p.meta, 4));
        SWG_TRY(sym_alloc(c, &p.part, (size_t)(6 * nrecv + 3 * npair) * TS));
        SWG_TRY(sym_alloc(c, &p.pA, (size_t)npl));
        SWG_TRY(sym_alloc(c, &p.pB, (size_t)npl));
        SWG_TRY(sym_alloc(c, &p.head, 1));
        SWG_TRY(cuda_status(c, cudaMemcpy(p.items, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice),
                            "upload"));
        SWG_TRY(cuda_status(c, cudaMemcpy(p.meta, meta, sizeof(meta), cudaMemcpyHostToDevice), "upload"));
        p.ppart = p.part + (size_t)6 * nrecv * TS;
        p.nitems = (int)items.size();
        p.npl = npl;
    }
    SWG_TRY(kick_split_launch(c, npl, r, Gm, R, p.pA, p.pB));
    SWG_TRY(kick_mixed_sym_batched(c, R != nullptr, p.nitems, p.items, p.meta, p.meta + 1, p.meta + 2, p.pA, p.pB,
                                   p.part, p.ppart, p.head));
    return kick_mixed_sym_reduce(c, p.strip, npl, nullptr, p.meta, p.meta + 1, p.meta + 2, p.part, p.ppart, acc,
                                 acc_is_zero);
}

}  // namespace swg
