// kick.cu -- pair-gravity kick kernels for sm_103a.
//
// Restates swiftest_kick_getacch_int_all_* (src/swiftest/swiftest_kick.f90:69-470).
//
// Layout: positions are the reference's (3,n) FP64 arrays.  Each thread owns one
// receiving body and walks the partners in ascending index order through
// shared-memory tiles, so every per-body sum has the same operands in the same
// order as the reference's serial loop:
//   * KICK_DIRECT  -- the triangular loop without GMTINY bodies
//                     (swiftest_kick.f90:221-264): acc_i += Gm_j/(r^2 sqrt r^2) * dx
//   * KICK_SPLIT   -- the symmetric loops (flat :69-162, triangular with GMTINY
//                     bodies :183-219): ahi_i = sum_{j>i} Gm_j irij3 dx,
//                     ahj_i = sum_{j<i} Gm_j irij3 dx, acc = (acc + ahi) + ahj.
// The FP64 path is therefore bit-identical to the reference loop evaluated
// serially with no FMA contraction (this file is compiled with -fmad=false).
//
// The mixed path (SWG_MIXED) splits each FP64 coordinate into a float hi/lo
// pair, forms displacements as (xj_hi - xi_hi) + (xj_lo - xi_lo) in FP32, takes
// r^-3 from the hardware rsqrt estimate refined by one Newton step, accumulates 64-partner FP32
// partials into float-float (TwoSum) accumulators, and adds the total to the
// FP64 acceleration.  Partner ranges are split over blocks to fill all SMs;
// the last block of each body tile folds the partials in a fixed order, so
// results are deterministic.
#include <cuda_runtime.h>

#include <algorithm>

#include "kick_mixed.cuh"
#include "swg_internal.cuh"

namespace swg {

constexpr int MBLOCK = 128;   // threads per block (mixed, one system)

// Sweep of partners [jbeg, jstop) (indices into the partner arrays) for this thread's RPT
// receivers, whole block: 64-partner FP32 partials folded into float-float (ax, ay, az).
// pA/pB hold the partners already split into (x_hi, y_hi, z_hi, Gm), (x_lo, y_lo, z_lo, R);
// without them each tile converts rpart/Gm/R itself.
// Pair rule (pl-pl; TP has none): the reference skips j == i and, with GMTINY bodies,
// pairs of two bodies both at index >= nplm (GMT); with RAD it also skips pairs closer
// than the sum of the radii, which covers j == i (r^2 == 0 exactly), so the index test
// is only made without RAD.  self[k] is receiver k's index in the partner arrays; every
// receiver of the block lies in [slo, shi).
// The rule is applied pair by pair only on tiles that can need it: tiles holding one of
// the block's own receivers (the self pairs) and, with GMT, every tile.  On the others
// the pairs are taken unguarded and, with RAD, a receiver whose closest partner in the
// tile lies within its radius plus the tile's largest radius recomputes that tile with
// the rule.  A pair the rule keeps gets the same operations either way, so the partials
// are the same bits as with the rule applied everywhere.
template <bool TP, bool RAD, bool GMT, int RPT>
__device__ __forceinline__ void mixed_sweep(int jbeg, int jstop, const int (&self)[RPT], int slo, int shi, int nplm,
                                            const bool (&self_m)[RPT], const MixedRecv (&q)[RPT],
                                            const double *__restrict__ rpart, const double *__restrict__ Gm,
                                            const double *__restrict__ R, const float4 *__restrict__ pA,
                                            const float4 *__restrict__ pB, float4 *sA, float4 *sB, FF (&ax)[RPT],
                                            FF (&ay)[RPT], FF (&az)[RPT]) {
    __shared__ unsigned sRmax[2];  // largest partner radius of the tile, per loading warp (float bits)
    for (int j0 = jbeg; j0 < jstop; j0 += MT) {
        float rmax = 0.f;
        // partner jl split into (x_hi, y_hi, z_hi, Gm) and (x_lo, y_lo, z_lo, R); zero past jstop
        auto load = [&](int jl, float4 &a, float4 &b) {
            a = make_float4(0.f, 0.f, 0.f, 0.f);
            b = make_float4(0.f, 0.f, 0.f, 0.f);
            if (jl < jstop && pA) {
                a = pA[jl];
                b = pB[jl];
            } else if (jl < jstop) {
                split_hi_lo(rpart[3 * jl + 0], a.x, b.x);
                split_hi_lo(rpart[3 * jl + 1], a.y, b.y);
                split_hi_lo(rpart[3 * jl + 2], a.z, b.z);
                a.w = __double2float_rn(Gm[jl]);
                b.w = RAD ? __double2float_rn(R[jl]) : 0.f;
            }
        };
        if (TP) {  // paired layout of mixed_tile_tp2
            for (int p = threadIdx.x; p < MT / 2; p += blockDim.x) {
                float4 a0, b0, a1, b1;
                load(j0 + 2 * p, a0, b0);
                load(j0 + 2 * p + 1, a1, b1);
                stage_pair(sA, sB, p, a0, b0, a1, b1);
            }
        } else {
            for (int t = threadIdx.x; t < MT; t += blockDim.x) {
                float4 a, b;
                load(j0 + t, a, b);
                sA[t] = a;
                sB[t] = b;
                rmax = fmaxf(rmax, b.w);
            }
        }
        if (!TP && RAD && threadIdx.x < MT) {  // whole warps: blockDim.x is a multiple of 32
            const unsigned m = __reduce_max_sync(0xffffffffu, __float_as_uint(rmax));  // radii are >= 0
            if ((threadIdx.x & 31) == 0) {
                sRmax[threadIdx.x >> 5] = m;
                if (blockDim.x == 32) sRmax[1] = 0u;
            }
        }
        __syncthreads();
        const int nt = min(MT, jstop - j0);
        float px[RPT], py[RPT], pz[RPT], mn[RPT];
        const bool guard = !TP && (GMT || (j0 < shi && j0 + nt > slo));  // block-uniform
        if (TP) {
            mixed_tile_tp2<RPT>(nt, q, sA, sB, px, py, pz);
        } else if (guard) {
            mixed_tile<TP, RAD, GMT, true, RPT>(j0, nt, self, nplm, self_m, q, sA, sB, px, py, pz, mn);
        } else {
#pragma unroll
            for (int k = 0; k < RPT; k++) mn[k] = 3.0e38f;
            mixed_tile<TP, RAD, GMT, false, RPT>(j0, nt, self, nplm, self_m, q, sA, sB, px, py, pz, mn);
            if (!TP && RAD) {
                const float rt = fmaxf(__uint_as_float(sRmax[0]), __uint_as_float(sRmax[1]));
#pragma unroll
                for (int k = 0; k < RPT; k++) {
                    const float rs = q[k].R + rt;
                    if (mn[k] <= rs * rs) {  // rare: a pair of this tile may lie within the radii
                        float gx[RPT], gy[RPT], gz[RPT], gm[RPT];
                        mixed_tile<TP, RAD, GMT, true, RPT>(j0, nt, self, nplm, self_m, q, sA, sB, gx, gy, gz, gm);
                        px[k] = gx[k];
                        py[k] = gy[k];
                        pz[k] = gz[k];
                    }
                }
            }
        }
#pragma unroll
        for (int k = 0; k < RPT; k++) {
            ff_add(ax[k], px[k]);
            ff_add(ay[k], py[k]);
            ff_add(az[k], pz[k]);
        }
        __syncthreads();
    }
}

// acc (+)= the float-float totals.  pl-pl: acc_i += sum Gm_j (r_j - r_i)/r^3; tp:
// acc_tp -= sum Gm_j (r_tp - r_j)/r^3, i.e. the same partner-minus-self sum added to acc.
__device__ __forceinline__ void mixed_store(double *a, const FF &ax, const FF &ay, const FF &az, int acc_is_zero) {
    const double sx = (double)ax.hi + (double)ax.lo, sy = (double)ay.hi + (double)ay.lo,
                 sz = (double)az.hi + (double)az.lo;
    a[0] = (acc_is_zero ? 0.0 : a[0]) + sx;
    a[1] = (acc_is_zero ? 0.0 : a[1]) + sy;
    a[2] = (acc_is_zero ? 0.0 : a[2]) + sz;
}

// Receivers i in [blockIdx.x*MBLOCK, ...), partners j in chunk blockIdx.y of
// length chunk.  TP: receivers are test particles (partners all pl, sign -),
// else pl-pl with the (i<nplm || j<nplm) interaction rule and optional radius guard.
template <bool TP, bool RAD, bool GMT>
__global__ void __launch_bounds__(MBLOCK) k_kick_mixed(int nrecv, int npart, int nplm, const double *__restrict__ rrecv,
                                                      const double *__restrict__ rpart,
                                                      const double *__restrict__ Gm, const double *__restrict__ R,
                                                      const int32_t *__restrict__ lmask, double *__restrict__ acc,
                                                      int acc_is_zero, int chunk, float *__restrict__ partial,
                                                      unsigned *__restrict__ counters,
                                                      const float4 *__restrict__ pA, const float4 *__restrict__ pB) {
    __shared__ float4 sA[MT];  // x_hi, y_hi, z_hi, Gm
    __shared__ float4 sB[MT];  // x_lo, y_lo, z_lo, R
    __shared__ bool s_last;
    const int i = blockIdx.x * MBLOCK + threadIdx.x;
    const bool inrange = i < nrecv;
    const bool active = inrange && (!TP || lmask[i] != 0);
    MixedRecv q[1] = {{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f}};
    if (inrange) q[0] = mixed_recv<RAD>(rrecv, R, i);
    FF axa[1] = {{0.f, 0.f}}, aya[1] = {{0.f, 0.f}}, aza[1] = {{0.f, 0.f}};
    const int jbeg = blockIdx.y * chunk;
    const int jstop = min(npart, jbeg + chunk);
    const int self[1] = {i};
    const bool self_m[1] = {i < nplm};
    const int slo = blockIdx.x * MBLOCK;
    mixed_sweep<TP, RAD, GMT, 1>(jbeg, jstop, self, slo, slo + MBLOCK, nplm, self_m, q, rpart, Gm, R, pA, pB, sA, sB,
                                 axa, aya, aza);
    const FF ax = axa[0], ay = aya[0], az = aza[0];
    const int nchunk = gridDim.y;
    if (nchunk == 1) {
        if (active)
            mixed_store(&acc[3 * i], ax, ay, az, acc_is_zero);
        else if (inrange && acc_is_zero)
            acc[3 * i + 0] = acc[3 * i + 1] = acc[3 * i + 2] = 0.0;
        return;
    }
    // Multi-chunk: publish partials, last block of this receiver tile folds them.
    if (inrange) {
        float *p = &partial[((size_t)blockIdx.y * nrecv + i) * 6];
        p[0] = ax.hi;
        p[1] = ax.lo;
        p[2] = ay.hi;
        p[3] = ay.lo;
        p[4] = az.hi;
        p[5] = az.lo;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned prev = atomicAdd(&counters[blockIdx.x], 1u);
        s_last = (prev == (unsigned)nchunk - 1);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    if (active) {
        // the chunks' float-float partials are folded in float-float (FP32 instructions)
        // and converted once: a fold in FP64 would put 12 FP64 instructions per chunk and
        // receiver on the narrow FP64 pipe of the one SM that runs the last block
        FF fx = {0.f, 0.f}, fy = {0.f, 0.f}, fz = {0.f, 0.f};
        for (int cidx = 0; cidx < nchunk; cidx++) {
            const volatile float *p = &partial[((size_t)cidx * nrecv + i) * 6];
            ff_add(fx, p[0]);
            ff_add(fx, p[1]);
            ff_add(fy, p[2]);
            ff_add(fy, p[3]);
            ff_add(fz, p[4]);
            ff_add(fz, p[5]);
        }
        const double sx = (double)fx.hi + (double)fx.lo, sy = (double)fy.hi + (double)fy.lo,
                     sz = (double)fz.hi + (double)fz.lo;
        double *a = &acc[3 * i];
        a[0] = (acc_is_zero ? 0.0 : a[0]) + sx;
        a[1] = (acc_is_zero ? 0.0 : a[1]) + sy;
        a[2] = (acc_is_zero ? 0.0 : a[2]) + sz;
    } else if (inrange && acc_is_zero) {
        acc[3 * i + 0] = acc[3 * i + 1] = acc[3 * i + 2] = 0.0;
    }
    if (threadIdx.x == 0) counters[blockIdx.x] = 0u;  // re-arm for the next launch
}

// Batched (ensemble) mixed kick: a persistent grid pulls receiver tiles of CSR-packed
// systems from a work queue (items sorted by cost, largest first, so the tail is made
// of small tiles).  With sys_flag, only systems whose flag equals `phase` are kicked (the
// ensemble kicks systems without encounters while the recursion of the others runs).
// Item: system s, receivers [r0, r0 + nr) of that system, nr <= T * RPT: T threads own
// RPT receivers each (r0 + t, r0 + t + T, ...), sharing each shared-memory partner read.
// Receivers sit at roff[s] + i in rrecv/acc/lmask, partners at poff[s] + j (j < npart[s])
// in the pre-split pA/pB.  pl-pl (!TP): rrecv is the pl array, roff == poff, and the
// receiver is skipped as its own partner through the radius rule (RAD) or the index test.
// Every (T, RPT) variant adds each receiver's terms in the same order (64-partner tiles in
// partner order), so the variants give identical bits; the autotuner picks among them.
// GMT (pl-pl with GMTINY): nplm[s] fully interacting bodies per system; a pair of two bodies
// both at index >= nplm[s] is skipped (the reference's nplm loop bounds).
template <bool TP, bool RAD, bool GMT, int T, int RPT>
__global__ void __launch_bounds__(T) k_kick_mixed_batched(int nitems, const int4 *__restrict__ items,
                                                         const int32_t *__restrict__ roff,
                                                         const int32_t *__restrict__ poff,
                                                         const int32_t *__restrict__ npart,
                                                         const double *__restrict__ rrecv,
                                                         const double *__restrict__ R,
                                                         const float4 *__restrict__ pA, const float4 *__restrict__ pB,
                                                         const int32_t *__restrict__ lmask, double *__restrict__ acc,
                                                         int acc_is_zero, unsigned *__restrict__ head,
                                                         const int32_t *__restrict__ sys_flag, int phase,
                                                         const int32_t *__restrict__ nplm) {
    __shared__ float4 sA[MT];
    __shared__ float4 sB[MT];
    __shared__ int s_item;
    for (;;) {
        __syncthreads();  // every thread has read the previous s_item
        if (threadIdx.x == 0) s_item = (int)atomicAdd(head, 1u);
        __syncthreads();
        const int it = s_item;
        if (it >= nitems) break;
        const int4 w = items[it];  // (system, r0, nr, unused)
        const int s = w.x;
        if (sys_flag && sys_flag[s] != phase) continue;  // another launch's system (block-uniform)
        MixedRecv q[RPT];
        FF ax[RPT], ay[RPT], az[RPT];
        int gi[RPT];
        bool inr[RPT], sm[RPT];
#pragma unroll
        for (int k = 0; k < RPT; k++) {
            const int l = threadIdx.x + k * T;
            inr[k] = l < w.z;
            gi[k] = roff[s] + w.y + l;
            sm[k] = true;
            q[k] = MixedRecv{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            if (inr[k]) q[k] = mixed_recv<RAD>(rrecv, R, gi[k]);
            ax[k] = ay[k] = az[k] = FF{0.f, 0.f};
        }
        const int p0 = poff[s];
        const int slo = roff[s] + w.y;  // receivers in partner indexing (pl-pl: roff == poff)
        const int nm = GMT ? p0 + nplm[s] : 0;  // first semi-interacting body, partner indexing
        if (GMT) {
#pragma unroll
            for (int k = 0; k < RPT; k++) sm[k] = gi[k] < nm;
        }
        mixed_sweep<TP, RAD, GMT, RPT>(p0, p0 + npart[s], gi, slo, slo + w.z, nm, sm, q, nullptr, nullptr, nullptr, pA,
                                       pB, sA, sB, ax, ay, az);
#pragma unroll
        for (int k = 0; k < RPT; k++) {
            if (!inr[k]) continue;
            if (!TP || lmask[gi[k]] != 0)
                mixed_store(&acc[3 * gi[k]], ax[k], ay[k], az[k], acc_is_zero);
            else if (acc_is_zero)
                acc[3 * gi[k] + 0] = acc[3 * gi[k] + 1] = acc[3 * gi[k] + 2] = 0.0;
        }
    }
}

// Partners split once per kick into float hi/lo pairs (the conversion runs on the
// FP64 pipe, which is narrow on GB300; doing it here instead of in every block
// keeps the pair kernel on the FP32 pipe).
// sysid/flag (optional): split only bodies whose system's flag equals phase.
// enc/enc_want (optional): split only bodies with enc[j] == enc_want.
__global__ void k_kick_split(int n, const double *__restrict__ r, const double *__restrict__ Gm,
                             const double *__restrict__ R, float4 *A, float4 *B, const int32_t *__restrict__ sysid,
                             const int32_t *__restrict__ flag, int phase, const uint8_t *__restrict__ enc,
                             int enc_want) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    if (sysid && flag[sysid[j]] != phase) return;
    if (enc && enc[j] != enc_want) return;
    float4 a, b;
    split_hi_lo(r[3 * j + 0], a.x, b.x);
    split_hi_lo(r[3 * j + 1], a.y, b.y);
    split_hi_lo(r[3 * j + 2], a.z, b.z);
    a.w = __double2float_rn(Gm[j]);
    b.w = R ? __double2float_rn(R[j]) : 0.f;
    A[j] = a;
    B[j] = b;
}

// ------------------------------------------------------------------ pair lists
// Serial pass over an explicit pair list, restating the flat loop
// (swiftest_kick.f90:69-115) in list order: ahi/ahj accumulate per body.
template <bool RAD>
__global__ void k_kick_pairs_serial(int64_t npairs, const int32_t *__restrict__ k, const int32_t *__restrict__ i1,
                                    const int32_t *__restrict__ i2, const double *__restrict__ r,
                                    const double *__restrict__ Gm, const double *__restrict__ R, double *ahi,
                                    double *ahj) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    for (int64_t q = 0; q < npairs; q++) {
        const int i = (k ? k[2 * q] : i1[q]) - 1;
        const int j = (k ? k[2 * q + 1] : i2[q]) - 1;
        const double rx = r[3 * j + 0] - r[3 * i + 0];
        const double ry = r[3 * j + 1] - r[3 * i + 1];
        const double rz = r[3 * j + 2] - r[3 * i + 2];
        const double rji2 = rx * rx + ry * ry + rz * rz;
        if (RAD) {
            const double rs = R[i] + R[j];
            if (!(rji2 > rs * rs)) continue;
        }
        const double irij3 = 1.0 / (rji2 * sqrt(rji2));
        const double faci = Gm[i] * irij3;
        const double facj = Gm[j] * irij3;
        ahi[3 * i + 0] = ahi[3 * i + 0] + facj * rx;
        ahi[3 * i + 1] = ahi[3 * i + 1] + facj * ry;
        ahi[3 * i + 2] = ahi[3 * i + 2] + facj * rz;
        ahj[3 * j + 0] = ahj[3 * j + 0] - faci * rx;
        ahj[3 * j + 1] = ahj[3 * j + 1] - faci * ry;
        ahj[3 * j + 2] = ahj[3 * j + 2] - faci * rz;
    }
}

// Short lists (npairs <= PAIRS_SMALL), one block, same bits as k_kick_pairs_serial: thread q
// evaluates pair q (the FP64 square root and divide of all pairs run at once), then the
// thread holding the first pair of a body adds that body's terms of every later pair in
// list order (ahi for index1, ahj for index2), as the serial loop does.
constexpr int PAIRS_SMALL = 256;
template <bool RAD>
__global__ void __launch_bounds__(PAIRS_SMALL) k_kick_pairs_small(int npairs, const int32_t *__restrict__ k,
                                                                  const int32_t *__restrict__ i1,
                                                                  const int32_t *__restrict__ i2,
                                                                  const double *__restrict__ r,
                                                                  const double *__restrict__ Gm,
                                                                  const double *__restrict__ R, double *ahi,
                                                                  double *ahj) {
    __shared__ double tI[PAIRS_SMALL][3], tJ[PAIRS_SMALL][3];
    __shared__ int sI[PAIRS_SMALL], sJ[PAIRS_SMALL];
    __shared__ unsigned char ok[PAIRS_SMALL];
    const int q = threadIdx.x;
    if (q < npairs) {
        const int i = (k ? k[2 * q] : i1[q]) - 1;
        const int j = (k ? k[2 * q + 1] : i2[q]) - 1;
        sI[q] = i;
        sJ[q] = j;
        const double rx = r[3 * j + 0] - r[3 * i + 0];
        const double ry = r[3 * j + 1] - r[3 * i + 1];
        const double rz = r[3 * j + 2] - r[3 * i + 2];
        const double rji2 = rx * rx + ry * ry + rz * rz;
        bool keep = true;
        if (RAD) {
            const double rs = R[i] + R[j];
            keep = rji2 > rs * rs;
        }
        ok[q] = keep;
        if (keep) {
            const double irij3 = 1.0 / (rji2 * sqrt(rji2));
            const double faci = Gm[i] * irij3;
            const double facj = Gm[j] * irij3;
            tI[q][0] = facj * rx;
            tI[q][1] = facj * ry;
            tI[q][2] = facj * rz;
            tJ[q][0] = faci * rx;
            tJ[q][1] = faci * ry;
            tJ[q][2] = faci * rz;
        }
    }
    __syncthreads();
    if (q >= npairs) return;
    for (int side = 0; side < 2; side++) {
        const int *s = side == 0 ? sI : sJ;
        const int b = s[q];
        bool first = true;
        for (int p = 0; p < q && first; p++) first = s[p] != b;
        if (!first) continue;
        double *a = (side == 0 ? ahi : ahj) + 3 * b;
        double x = a[0], y = a[1], z = a[2];
        for (int p = q; p < npairs; p++) {
            if (s[p] != b || !ok[p]) continue;
            if (side == 0) {
                x = x + tI[p][0];
                y = y + tI[p][1];
                z = z + tI[p][2];
            } else {
                x = x - tJ[p][0];
                y = y - tJ[p][1];
                z = z - tJ[p][2];
            }
        }
        a[0] = x;
        a[1] = y;
        a[2] = z;
    }
}

// Parallel variant for long lists: atomic accumulation (order not fixed).
template <bool RAD>
__global__ void k_kick_pairs_atomic(int64_t npairs, const int32_t *__restrict__ k, const int32_t *__restrict__ i1,
                                    const int32_t *__restrict__ i2, const double *__restrict__ r,
                                    const double *__restrict__ Gm, const double *__restrict__ R, double *ahi,
                                    double *ahj) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < npairs; q += (int64_t)gridDim.x * blockDim.x) {
        const int i = (k ? k[2 * q] : i1[q]) - 1;
        const int j = (k ? k[2 * q + 1] : i2[q]) - 1;
        const double rx = r[3 * j + 0] - r[3 * i + 0];
        const double ry = r[3 * j + 1] - r[3 * i + 1];
        const double rz = r[3 * j + 2] - r[3 * i + 2];
        const double rji2 = rx * rx + ry * ry + rz * rz;
        if (RAD) {
            const double rs = R[i] + R[j];
            if (!(rji2 > rs * rs)) continue;
        }
        const double irij3 = 1.0 / (rji2 * sqrt(rji2));
        const double faci = Gm[i] * irij3;
        const double facj = Gm[j] * irij3;
        atomicAdd(&ahi[3 * i + 0], facj * rx);
        atomicAdd(&ahi[3 * i + 1], facj * ry);
        atomicAdd(&ahi[3 * i + 2], facj * rz);
        atomicAdd(&ahj[3 * j + 0], -(faci * rx));
        atomicAdd(&ahj[3 * j + 1], -(faci * ry));
        atomicAdd(&ahj[3 * j + 2], -(faci * rz));
    }
}

// sign > 0: acc = (acc + ahi) + ahj     (flat kernel semantics)
// sign < 0: acc = acc - ((0 + ahi) + ahj) (symba_kick_getacch_pl, symba_kick.f90:61-70)
__global__ void k_apply_pairs(int npl, const double *__restrict__ ahi, const double *__restrict__ ahj, double *acc,
                              double sign) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * npl) return;
    if (sign > 0)
        acc[t] = acc[t] + ahi[t] + ahj[t];
    else
        acc[t] = acc[t] - (ahi[t] + ahj[t]);
}

// ------------------------------------------------------------------ launchers
static inline int div_up(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

// pl-pl variants of k_kick_mixed: radius guard or not, GMTINY rule or not
static void launch_mixed_plpl(dim3 grid, cudaStream_t st, int npl, int nplm, const double *r, const double *Gm,
                              const double *R, double *acc, int acc_is_zero, int chunk, float *partial,
                              unsigned *counters, const float4 *pA, const float4 *pB) {
    const bool gmt = nplm < npl;
    if (R && gmt)
        k_kick_mixed<false, true, true><<<grid, MBLOCK, 0, st>>>(npl, npl, nplm, r, r, Gm, R, nullptr, acc,
                                                                 acc_is_zero, chunk, partial, counters, pA, pB);
    else if (R)
        k_kick_mixed<false, true, false><<<grid, MBLOCK, 0, st>>>(npl, npl, nplm, r, r, Gm, R, nullptr, acc,
                                                                  acc_is_zero, chunk, partial, counters, pA, pB);
    else if (gmt)
        k_kick_mixed<false, false, true><<<grid, MBLOCK, 0, st>>>(npl, npl, nplm, r, r, Gm, nullptr, nullptr, acc,
                                                                  acc_is_zero, chunk, partial, counters, pA, pB);
    else
        k_kick_mixed<false, false, false><<<grid, MBLOCK, 0, st>>>(npl, npl, nplm, r, r, Gm, nullptr, nullptr, acc,
                                                                   acc_is_zero, chunk, partial, counters, pA, pB);
}

size_t kick_mixed_scratch_bytes(int nrecv, int npart, int nchunk) {
    return KICK_COUNTERS * sizeof(unsigned) + (size_t)nchunk * nrecv * 6 * sizeof(float) +
           (size_t)2 * sizeof(float4) * (size_t)npart + 512;
}

int ensure_kick_scratch(swg_ctx *c, DevBuf &buf, size_t bytes) {
    if (buf.ptr && buf.bytes >= bytes) return SWG_OK;
    void *old = buf.ptr;
    buf.ptr = nullptr;
    buf.bytes = 0;
    if (old) cudaFree(old);
    SWG_TRY(ensure(c, buf, bytes));
    return cuda_status(c, cudaMemsetAsync(buf.ptr, 0, KICK_COUNTERS * sizeof(unsigned), c->stream), "memset");
}

// Chooses the partner split so that the grid covers ~8 blocks (32 warps) per SM: the
// pair loop is latency-bound (rsqrt and dependent FMAs), so occupancy hides it.
int kick_mixed_nchunk(int num_sms, int nrecv, int npart) {
    const int bx = div_up(nrecv, MBLOCK);
    const int target = 8 * (num_sms > 0 ? num_sms : 152);
    int nchunk = div_up(target, bx);
    const int maxchunk = div_up(npart, MT);  // at least one tile per chunk
    if (nchunk > maxchunk) nchunk = maxchunk;
    if (nchunk < 1) nchunk = 1;
    return nchunk;
}

int kick_mixed_chunks(swg_ctx *c, int nrecv, int npart) { return kick_mixed_nchunk(c->num_sms, nrecv, npart); }

int kick_mixed_launch(swg_ctx *c, bool tp, int nrecv, int npart, int nplm, const double *rrecv, const double *rpart,
                      const double *Gm, const double *R, const int32_t *lmask, double *acc, int acc_is_zero,
                      int nchunk, void *scratch) {
    if (nrecv <= 0) return SWG_OK;
    const int bx = div_up(nrecv, MBLOCK);
    int chunk = div_up(npart, nchunk);
    chunk = div_up(chunk, MT) * MT;
    nchunk = npart > 0 ? div_up(npart, chunk) : 1;
    if (bx > (int)KICK_COUNTERS) return SWG_ERR_ARG;
    unsigned *counters = (unsigned *)scratch;
    float *partial = (float *)((char *)scratch + KICK_COUNTERS * sizeof(unsigned));
    const size_t poff = ((KICK_COUNTERS * sizeof(unsigned) + (size_t)nchunk * nrecv * 6 * sizeof(float)) + 255) & ~size_t(255);
    float4 *pA = (float4 *)((char *)scratch + poff), *pB = pA + npart;
    if (npart > 0) {
        k_kick_split<<<div_up(npart, 256), 256, 0, c->stream>>>(npart, rpart, Gm, tp ? nullptr : R, pA, pB, nullptr,
                                                                 nullptr, 0, nullptr, 0);
        c->launches++;
    }
    dim3 grid(bx, nchunk);
    if (tp)
        k_kick_mixed<true, false, false><<<grid, MBLOCK, 0, c->stream>>>(
            nrecv, npart, 0, rrecv, rpart, Gm, nullptr, lmask, acc, acc_is_zero, chunk, partial, counters, pA, pB);
    else
        launch_mixed_plpl(grid, c->stream, nrecv, nplm, rrecv, Gm, R, acc, acc_is_zero, chunk, partial, counters, pA,
                          pB);
    c->launches++;
    return launch_status(c, "kick_mixed");
}

// Grid of the mixed pl-pl kick of one system: bx receiver blocks by nchunk partner chunks
// of `chunk` partners, exactly as kick_mixed_launch derives it from kick_mixed_chunks.
// partials = float-float partial-sum entries (6 floats each) the launch writes, 0 when
// there is one chunk.
MixedPlplGrid kick_mixed_plpl_grid(int num_sms, int npl) {
    MixedPlplGrid g{0, 1, 0, 0};
    if (npl <= 0) return g;
    g.bx = div_up(npl, MBLOCK);
    const int nch = kick_mixed_nchunk(num_sms, npl, npl);
    g.chunk = div_up(div_up(npl, nch), MT) * MT;
    g.nchunk = div_up(npl, g.chunk);
    g.partials = g.nchunk > 1 ? (int64_t)g.nchunk * npl : 0;
    return g;
}

// Mixed pl-pl kick on a caller's stream with caller-provided scratch (block counters
// first, then partials); used by the entry point that allocates nothing
// (kick_noalloc.cu).  Same grid and kernel as kick_mixed_launch; the partners are split
// inside each tile instead of by k_kick_split, which gives the same floats, so the
// accelerations are the same bits.
cudaError_t kick_mixed_plpl_on_stream(cudaStream_t stream, const MixedPlplGrid &g, int npl, int nplm,
                                      const double *r, const double *Gm, const double *R, double *acc, void *scratch,
                                      size_t counter_bytes) {
    if (npl <= 0) return cudaSuccess;
    unsigned *counters = (unsigned *)scratch;
    float *partial = (float *)((char *)scratch + counter_bytes);
    dim3 grid(g.bx, g.nchunk);
    launch_mixed_plpl(grid, stream, npl, nplm, r, Gm, R, acc, 0, g.chunk, partial, counters, nullptr, nullptr);
    return cudaGetLastError();
}

// Split n partner bodies into float hi/lo tiles (A = x_hi, y_hi, z_hi, Gm; B = x_lo, y_lo, z_lo, R).
int kick_split_launch(swg_ctx *c, int64_t n, const double *r, const double *Gm, const double *R, float4 *A,
                      float4 *B, const int32_t *sysid, const int32_t *flag, int phase, const uint8_t *enc,
                      int enc_want) {
    if (n <= 0) return SWG_OK;
    k_kick_split<<<div_up(n, 256), 256, 0, c->stream>>>((int)n, r, Gm, R, A, B, sysid, flag, phase, enc, enc_want);
    c->launches++;
    return launch_status(c, "kick_split");
}

// Tile shapes of the batched mixed kick: (threads per block, receivers per thread).
struct KickShape {
    int threads, rpt;
};
static constexpr KickShape KICK_SHAPES[KICK_NVARIANT] = {{64, 2}, {128, 1}, {128, 2}, {32, 4}, {64, 4}};

int kick_variant_tile(int variant) { return KICK_SHAPES[variant].threads * KICK_SHAPES[variant].rpt; }

template <bool TP, bool RAD, bool GMT, int T, int RPT>
static int launch_batched(swg_ctx *c, int nitems, const int4 *items, const int32_t *roff, const int32_t *poff,
                          const int32_t *npart, const double *rrecv, const double *R, const float4 *pA,
                          const float4 *pB, const int32_t *lmask, double *acc, int acc_is_zero, unsigned *head,
                          const int32_t *sys_flag, int phase, const int32_t *nplm) {
    static int occ = 0;  // resident blocks per SM of this variant, queried once
    if (occ == 0) {
        int nb = 0;
        SWG_TRY(cuda_status(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                                   &nb, k_kick_mixed_batched<TP, RAD, GMT, T, RPT>, T, 0),
                            "occupancy"));
        occ = nb > 0 ? nb : 1;
    }
    const int grid = std::min(nitems, occ * (c->num_sms > 0 ? c->num_sms : 152));
    k_kick_mixed_batched<TP, RAD, GMT, T, RPT><<<grid, T, 0, c->stream>>>(nitems, items, roff, poff, npart, rrecv, R,
                                                                           pA, pB, lmask, acc, acc_is_zero, head,
                                                                           sys_flag, phase, nplm);
    c->launches++;
    return launch_status(c, "kick_mixed_batched");
}

template <bool TP, bool RAD, bool GMT>
static int launch_variant(swg_ctx *c, int variant, int nitems, const int4 *items, const int32_t *roff,
                          const int32_t *poff, const int32_t *npart, const double *rrecv, const double *R,
                          const float4 *pA, const float4 *pB, const int32_t *lmask, double *acc, int acc_is_zero,
                          unsigned *head, const int32_t *sys_flag, int phase, const int32_t *nplm) {
#define SWG_KV(T, P)                                                                                                  \
    return launch_batched<TP, RAD, GMT, T, P>(c, nitems, items, roff, poff, npart, rrecv, R, pA, pB, lmask, acc,      \
                                              acc_is_zero, head, sys_flag, phase, nplm)
    switch (variant) {
        case 0: SWG_KV(64, 2);
        case 1: SWG_KV(128, 1);
        case 2: SWG_KV(128, 2);
        case 3: SWG_KV(32, 4);
        default: SWG_KV(64, 4);
    }
#undef SWG_KV
}

// Persistent batched mixed kick over a work queue of receiver tiles (see
// k_kick_mixed_batched); pA/pB must hold the split partners and the items must be tiles of
// kick_variant_tile(variant) receivers.  The queue head is reset on the stream before the
// launch; the grid is one wave of resident blocks.
int kick_mixed_batched(swg_ctx *c, int variant, bool tp, bool rad, int nitems, const int4 *items,
                       const int32_t *roff, const int32_t *poff, const int32_t *npart, const double *rrecv,
                       const double *R, const float4 *pA, const float4 *pB, const int32_t *lmask, double *acc,
                       int acc_is_zero, unsigned *head, const int32_t *sys_flag, int phase, const int32_t *nplm) {
    if (nitems <= 0) return SWG_OK;
    if (variant < 0 || variant >= KICK_NVARIANT) return SWG_ERR_ARG;
    SWG_TRY(cuda_status(c, cudaMemsetAsync(head, 0, sizeof(unsigned), c->stream), "memset"));
    if (tp)
        return launch_variant<true, false, false>(c, variant, nitems, items, roff, poff, npart, rrecv, nullptr, pA, pB,
                                                  lmask, acc, acc_is_zero, head, sys_flag, phase, nullptr);
    if (rad && nplm)  // GMTINY (SyMBA, always with radii)
        return launch_variant<false, true, true>(c, variant, nitems, items, roff, poff, npart, rrecv, R, pA, pB,
                                                 nullptr, acc, acc_is_zero, head, sys_flag, phase, nplm);
    if (nplm) return SWG_ERR_ARG;
    if (rad)
        return launch_variant<false, true, false>(c, variant, nitems, items, roff, poff, npart, rrecv, R, pA, pB,
                                                  nullptr, acc, acc_is_zero, head, sys_flag, phase, nullptr);
    return launch_variant<false, false, false>(c, variant, nitems, items, roff, poff, npart, rrecv, nullptr, pA, pB,
                                               nullptr, acc, acc_is_zero, head, sys_flag, phase, nullptr);
}

int kick_pairs(swg_ctx *c, int32_t npl, int64_t npairs, const int32_t *k, const int32_t *i1, const int32_t *i2,
               const double *r, const double *Gm, const double *R, double *acc, double sign, double *ahi_ahj) {
    if (npairs <= 0 || npl <= 0) return SWG_OK;
    double *ahi = ahi_ahj, *ahj = ahi_ahj + 3 * (size_t)npl;
    SWG_TRY(cuda_status(c, cudaMemsetAsync(ahi_ahj, 0, sizeof(double) * 6 * (size_t)npl, c->stream), "memset"));
    if (npairs <= PAIRS_SMALL) {
        if (R)
            k_kick_pairs_small<true><<<1, PAIRS_SMALL, 0, c->stream>>>((int)npairs, k, i1, i2, r, Gm, R, ahi, ahj);
        else
            k_kick_pairs_small<false><<<1, PAIRS_SMALL, 0, c->stream>>>((int)npairs, k, i1, i2, r, Gm, R, ahi, ahj);
    } else if (npairs <= 65536) {
        if (R)
            k_kick_pairs_serial<true><<<1, 32, 0, c->stream>>>(npairs, k, i1, i2, r, Gm, R, ahi, ahj);
        else
            k_kick_pairs_serial<false><<<1, 32, 0, c->stream>>>(npairs, k, i1, i2, r, Gm, R, ahi, ahj);
    } else {
        const int grid = (int)std::min<int64_t>((npairs + 255) / 256, 4 * 152);
        if (R)
            k_kick_pairs_atomic<true><<<grid, 256, 0, c->stream>>>(npairs, k, i1, i2, r, Gm, R, ahi, ahj);
        else
            k_kick_pairs_atomic<false><<<grid, 256, 0, c->stream>>>(npairs, k, i1, i2, r, Gm, R, ahi, ahj);
    }
    c->launches++;
    SWG_TRY(launch_status(c, "kick_pairs"));
    k_apply_pairs<<<div_up(3 * (int64_t)npl, 256), 256, 0, c->stream>>>(npl, ahi, ahj, acc, sign);
    c->launches++;
    return launch_status(c, "apply_pairs");
}

}  // namespace swg
