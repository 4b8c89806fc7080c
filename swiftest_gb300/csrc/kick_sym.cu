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
// Work: every system's bodies form tiles of KICK_SYM_TILE; an item is a pair of tiles (I, J),
// I <= J, of one system, pulled from a work queue by a persistent grid.
//   * I < J: the block's two warps hold 64 receivers of tile I each (two per lane); tile
//     J is staged in shared memory as four 32-partner sub-tiles, each stored twice in a
//     row so that lane t reads partner (t + s) mod 32 at step s without wrapping.  At
//     every step each lane evaluates its receivers against that partner, adds to its own
//     receiver partials, and subtracts from an accumulator of that partner which the warp
//     rotates one lane down after the step (three shuffles), so after 32 steps every
//     partner accumulator holds the sum over the warp's 64 receivers and is back on the
//     lane of its partner.  Tiles I < J hold no self pairs; with radii, pairs that the
//     radius rule could drop are found per sub-tile (the smallest r^2 a receiver met
//     against its radius plus the sub-tile's largest) and that sub-tile is recomputed with
//     the rule applied pair by pair, so every kept pair gets the same operations.
//   * I == J: each receiver sums over the whole tile with the pair rule applied pair by
//     pair (as the broadcast kernel does).
// Receiver-side sums (32-partner FP32 partials folded into float-float) and partner-side
// sums (64-receiver FP32 partials per warp, folded across the warps into float-float) go
// to per-item slots; a second kernel adds, for every body, its slots in a fixed order
// (tiles below its own as partner side, then its own and above as receiver side) in
// float-float, converted to FP64 once.
// No atomics touch the sums, so results are deterministic.
#include <cuda_runtime.h>

#include <algorithm>

#include "kick_mixed.cuh"
#include "swg_internal.cuh"

namespace swg {

namespace {

constexpr int SW = 2;                  // warps per block
constexpr int SR = 2;                  // receivers per lane
constexpr int TS = KICK_SYM_TILE;      // bodies per tile
constexpr int NSUB = TS / 32;          // 32-partner sub-tiles per tile
static_assert(TS == SW * 32 * SR && TS % 32 == 0, "tile of the symmetric kick");
constexpr float PAD_POS = 3.0e6f;      // position of the padding beyond a system's last body

// slot of tile pair (I, J), I <= J, among a system's nt tiles (row-major upper triangle)
__host__ __device__ __forceinline__ int tri_slot(int I, int J, int nt) { return I * nt - I * (I - 1) / 2 + (J - I); }

// 32 steps of one sub-tile for this lane's receivers (see the file comment).  A/B point
// at the lane's first partner of the doubled sub-tile; src is the lane above.
// GUARD: the radius rule pair by pair (RAD only); else, with RAD, mn keeps the smallest r^2.
template <bool RAD, bool GUARD>
__device__ __forceinline__ void sym_subtile(const float4 *A, const float4 *B, const MixedRecv (&q)[SR],
                                            const float (&gm)[SR], int src, float (&px)[SR], float (&py)[SR],
                                            float (&pz)[SR], float &qx, float &qy, float &qz, float (&mn)[SR]) {
#pragma unroll
    for (int k = 0; k < SR; k++) {
        px[k] = py[k] = pz[k] = 0.f;
        mn[k] = 3.0e38f;
    }
    qx = qy = qz = 0.f;
#pragma unroll 8
    for (int s = 0; s < 32; s++) {
        const float4 a = A[s];
        const float4 b = B[s];
#pragma unroll
        for (int k = 0; k < SR; k++) {
            const float dx = (a.x - q[k].xh) + (b.x - q[k].xl);
            const float dy = (a.y - q[k].yh) + (b.y - q[k].yl);
            const float dz = (a.z - q[k].zh) + (b.z - q[k].zl);
            const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
            const float r3 = rinv3(r2);
            float fi = a.w * r3, fj = gm[k] * r3;
            if (RAD && GUARD) {
                const float rs = q[k].R + b.w;
                if (!(r2 > rs * rs)) fi = fj = 0.f;
            }
            if (RAD && !GUARD) mn[k] = fminf(mn[k], r2);
            px[k] = fmaf(fi, dx, px[k]);
            py[k] = fmaf(fi, dy, py[k]);
            pz[k] = fmaf(fi, dz, pz[k]);
            qx = fmaf(-fj, dx, qx);
            qy = fmaf(-fj, dy, qy);
            qz = fmaf(-fj, dz, qz);
        }
        qx = __shfl_sync(0xffffffffu, qx, src);
        qy = __shfl_sync(0xffffffffu, qy, src);
        qz = __shfl_sync(0xffffffffu, qz, src);
    }
}

// Item: (system, tile I, tile J, slot).  pA/pB: every body split into (x_hi, y_hi, z_hi, Gm),
// (x_lo, y_lo, z_lo, R); part: per slot [side 0 receivers | side 1 partners] x
// [x_hi, x_lo, y_hi, y_lo, z_hi, z_lo] x TS floats.
template <bool RAD>
__global__ void __launch_bounds__(SW * 32) k_kick_mixed_sym(int nitems, const int4 *__restrict__ items,
                                                           const int32_t *__restrict__ poff,
                                                           const int32_t *__restrict__ npl,
                                                           const float4 *__restrict__ pA,
                                                           const float4 *__restrict__ pB, float *__restrict__ part,
                                                           unsigned *__restrict__ head,
                                                           const int32_t *__restrict__ sys_flag, int phase) {
    __shared__ float4 sA[NSUB * 64];  // sub-tile u at [64u, 64u + 64): its 32 partners twice
    __shared__ float4 sB[NSUB * 64];
    __shared__ float sQ[SW][3][TS];   // partner-side partials of each warp
    __shared__ int s_item;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const float4 pad_a = make_float4(PAD_POS, PAD_POS, PAD_POS, 0.f), zero = make_float4(0.f, 0.f, 0.f, 0.f);
    for (;;) {
        __syncthreads();  // every thread is done with the previous item's shared data
        if (threadIdx.x == 0) s_item = (int)atomicAdd(head, 1u);
        __syncthreads();
        const int it = s_item;
        if (it >= nitems) break;
        const int4 w = items[it];
        const int s = w.x, I = w.y, J = w.z;
        if (sys_flag && sys_flag[s] != phase) continue;  // block-uniform
        const int p0 = poff[s], n = npl[s];
        for (int t = threadIdx.x; t < TS; t += SW * 32) {
            const int j = J * TS + t;
            const float4 a = j < n ? pA[p0 + j] : pad_a;
            const float4 b = j < n ? pB[p0 + j] : zero;
            const int o = (t >> 5) * 64 + (t & 31);
            sA[o] = a;
            sA[o + 32] = a;
            sB[o] = b;
            sB[o + 32] = b;
        }
        MixedRecv q[SR];
        float gm[SR];
        bool ok[SR];
        int self[SR];
        bool self_m[SR];
#pragma unroll
        for (int k = 0; k < SR; k++) {
            const int i = I * TS + warp * 32 * SR + k * 32 + lane;
            ok[k] = i < n;
            self[k] = i;
            self_m[k] = true;
            const float4 a = ok[k] ? pA[p0 + i] : pad_a;
            const float4 b = ok[k] ? pB[p0 + i] : zero;
            q[k] = MixedRecv{a.x, a.y, a.z, b.x, b.y, b.z, b.w};
            gm[k] = a.w;
        }
        __syncthreads();
        FF ax[SR], ay[SR], az[SR];
#pragma unroll
        for (int k = 0; k < SR; k++) ax[k] = ay[k] = az[k] = FF{0.f, 0.f};
        float px[SR], py[SR], pz[SR], mn[SR];
        if (I == J) {
            for (int u = 0; u < NSUB; u++) {
                mixed_tile<false, RAD, false, true, SR>(J * TS + u * 32, 32, self, 0, self_m, q, sA + u * 64,
                                                        sB + u * 64, px, py, pz, mn);
#pragma unroll
                for (int k = 0; k < SR; k++) {
                    ff_add(ax[k], px[k]);
                    ff_add(ay[k], py[k]);
                    ff_add(az[k], pz[k]);
                }
            }
        } else {
            const int src = (lane + 1) & 31;
            for (int u = 0; u < NSUB; u++) {
                const float4 *A = sA + u * 64 + lane;
                const float4 *B = sB + u * 64 + lane;
                float qx, qy, qz;
                sym_subtile<RAD, false>(A, B, q, gm, src, px, py, pz, qx, qy, qz, mn);
                if (RAD) {
                    const float rt = __uint_as_float(__reduce_max_sync(0xffffffffu, __float_as_uint(B[0].w)));
                    bool need = false;
#pragma unroll
                    for (int k = 0; k < SR; k++) {
                        const float rs = q[k].R + rt;
                        need = need || (ok[k] && mn[k] <= rs * rs);
                    }
                    if (__any_sync(0xffffffffu, need))  // rare: a pair may lie within the radii
                        sym_subtile<RAD, true>(A, B, q, gm, src, px, py, pz, qx, qy, qz, mn);
                }
#pragma unroll
                for (int k = 0; k < SR; k++) {
                    ff_add(ax[k], px[k]);
                    ff_add(ay[k], py[k]);
                    ff_add(az[k], pz[k]);
                }
                sQ[warp][0][u * 32 + lane] = qx;
                sQ[warp][1][u * 32 + lane] = qy;
                sQ[warp][2][u * 32 + lane] = qz;
            }
        }
        float *o0 = part + (size_t)w.w * 12 * TS;
#pragma unroll
        for (int k = 0; k < SR; k++) {
            const int il = warp * 32 * SR + k * 32 + lane;
            o0[0 * TS + il] = ax[k].hi;
            o0[1 * TS + il] = ax[k].lo;
            o0[2 * TS + il] = ay[k].hi;
            o0[3 * TS + il] = ay[k].lo;
            o0[4 * TS + il] = az[k].hi;
            o0[5 * TS + il] = az[k].lo;
        }
        if (I != J) {
            __syncthreads();
            float *o1 = o0 + 6 * TS;
            for (int t = threadIdx.x; t < TS; t += SW * 32) {
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    FF f{0.f, 0.f};
#pragma unroll
                    for (int v = 0; v < SW; v++) ff_add(f, sQ[v][c][t]);
                    o1[(2 * c) * TS + t] = f.hi;
                    o1[(2 * c + 1) * TS + t] = f.lo;
                }
            }
        }
    }
}

// Per body: acc (+)= its slots in a fixed order.  The slots' float-float values are added
// in float-float (hi parts by TwoSum, lo parts plainly) and converted to FP64 once: FP64
// arithmetic per slot would run on the narrow FP64 pipe and bound this kernel.
__device__ __forceinline__ void ff_acc(FF &a, float &lo, const float *o, int l) {
    ff_add(a, o[l]);
    lo += o[KICK_SYM_TILE + l];
}

__global__ void k_kick_sym_reduce(int64_t n, const int32_t *__restrict__ psys, const int32_t *__restrict__ poff,
                                  const int32_t *__restrict__ npl, const int32_t *__restrict__ sbase,
                                  const float *__restrict__ part, double *__restrict__ acc, int acc_is_zero,
                                  const int32_t *__restrict__ sys_flag, int phase) {
    const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b >= n) return;
    const int s = psys[b];
    if (sys_flag && sys_flag[s] != phase) return;
    const int i = (int)(b - poff[s]);
    const int nt = (npl[s] + TS - 1) / TS, K = i / TS, l = i % TS;
    FF fx{0.f, 0.f}, fy{0.f, 0.f}, fz{0.f, 0.f};
    float lx = 0.f, ly = 0.f, lz = 0.f;
    for (int I = 0; I < K; I++) {
        const float *o = part + ((size_t)(sbase[s] + tri_slot(I, K, nt)) * 12 + 6) * TS;
        ff_acc(fx, lx, o, l);
        ff_acc(fy, ly, o + 2 * TS, l);
        ff_acc(fz, lz, o + 4 * TS, l);
    }
    for (int J = K; J < nt; J++) {
        const float *o = part + (size_t)(sbase[s] + tri_slot(K, J, nt)) * 12 * TS;
        ff_acc(fx, lx, o, l);
        ff_acc(fy, ly, o + 2 * TS, l);
        ff_acc(fz, lz, o + 4 * TS, l);
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

int64_t kick_sym_items(int32_t nsys, const int32_t *npl, std::vector<int4> &items, std::vector<int32_t> &sbase) {
    items.clear();
    sbase.assign(nsys, 0);
    std::vector<int64_t> cost;
    int64_t nslot = 0;
    for (int s = 0; s < nsys; s++) {
        const int nt = (npl[s] + TS - 1) / TS;
        sbase[s] = (int32_t)nslot;
        for (int I = 0; I < nt; I++)
            for (int J = I; J < nt; J++) {
                items.push_back(make_int4(s, I, J, (int)(nslot + tri_slot(I, J, nt))));
                cost.push_back((int64_t)std::min(TS, npl[s] - I * TS) * std::min(TS, npl[s] - J * TS));
            }
        nslot += (int64_t)nt * (nt + 1) / 2;
    }
    std::vector<size_t> ord(items.size());
    for (size_t k = 0; k < ord.size(); k++) ord[k] = k;
    std::stable_sort(ord.begin(), ord.end(), [&](size_t a, size_t b) { return cost[a] > cost[b]; });
    std::vector<int4> sorted(items.size());
    for (size_t k = 0; k < ord.size(); k++) sorted[k] = items[ord[k]];
    items.swap(sorted);
    return nslot;
}

int kick_mixed_sym_batched(swg_ctx *c, bool rad, int nitems, const int4 *items, const int32_t *poff,
                           const int32_t *npl, const float4 *pA, const float4 *pB, float *part, unsigned *head,
                           const int32_t *sys_flag, int phase) {
    if (nitems <= 0) return SWG_OK;
    SWG_TRY(cuda_status(c, cudaMemsetAsync(head, 0, sizeof(unsigned), c->stream), "memset"));
    static int occ[2] = {0, 0};  // resident blocks per SM, queried once per variant
    int &o = occ[rad ? 1 : 0];
    if (o == 0) {
        int nb = 0;
        SWG_TRY(cuda_status(c, rad ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_kick_mixed_sym<true>, SW * 32, 0)
                                   : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_kick_mixed_sym<false>, SW * 32, 0),
                            "occupancy"));
        o = nb > 0 ? nb : 1;
    }
    const int grid = std::min(nitems, o * (c->num_sms > 0 ? c->num_sms : 152));
    if (rad)
        k_kick_mixed_sym<true><<<grid, SW * 32, 0, c->stream>>>(nitems, items, poff, npl, pA, pB, part, head, sys_flag,
                                                               phase);
    else
        k_kick_mixed_sym<false><<<grid, SW * 32, 0, c->stream>>>(nitems, items, poff, npl, pA, pB, part, head, sys_flag,
                                                                phase);
    c->launches++;
    return launch_status(c, "kick_mixed_sym");
}

int kick_mixed_sym_reduce(swg_ctx *c, int64_t n, const int32_t *psys, const int32_t *poff, const int32_t *npl,
                          const int32_t *sbase, const float *part, double *acc, int acc_is_zero,
                          const int32_t *sys_flag, int phase) {
    if (n <= 0) return SWG_OK;
    k_kick_sym_reduce<<<(int)((n + 255) / 256), 256, 0, c->stream>>>(n, psys, poff, npl, sbase, part, acc, acc_is_zero,
                                                                      sys_flag, phase);
    c->launches++;
    return launch_status(c, "kick_sym_reduce");
}

}  // namespace swg
