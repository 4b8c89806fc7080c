// encounter.cu -- close-encounter checks for sm_103a.
//
// Restates encounter_check_all_plpl / _plplm / _pltp (src/encounter/encounter_check.f90:14-140)
// in both of the reference's modes:
//   * TRIANGULAR (:384-570): every pair is tested with encounter_check_one (:573-621).
//   * SORTSWEEP  (:143-326, :763-988): 1-D radial bounding boxes |r| +- 1.1 renc,
//     sorted by a stable radix sort on the extents (radix_sort.cu; ties by extent index);
//     each body whose box holds >= 2 foreign extents strictly inside (the reference's
//     loverlap test) tests the bodies whose extents lie inside.
//
// The encounter decision is made in FP64 with the reference's expression order
// (this file is compiled with -fmad=false), so lists are bit-identical to the
// reference loop.  In TRIANGULAR mode a conservative FP32 prefilter first
// rejects pairs whose closest approach over the step provably exceeds the
// encounter radius (min_t |x + v t| >= |x| - |v| |dt|; see prefilter_reject for
// the margins).  Only pairs the FP64 test could accept reach it, so the
// prefilter changes speed, never the list.
//
// Output: pairs are appended with an atomic counter (up to cap), then sorted by
// (index1, index2) with a bitonic sort (single CTA in shared memory when the
// padded length fits, else global compare-exchange passes); the lists are short.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "encounter_dev.cuh"
#include "swg_internal.cuh"

namespace swg {

constexpr int ET = 128;  // partner tile / block size

// Float copies of the bodies for the prefilter, written once per check.
__global__ void k_encounter_prep(int n, const double *__restrict__ r, const double *__restrict__ v,
                                 const double *__restrict__ renc, float4 *A, float4 *B, float4 *V) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const BodyF o = load_body(r, v, renc, i);
    A[i] = o.a;
    B[i] = o.b;
    V[i] = o.v;
}

constexpr int EP = 64;  // partners per shared-memory tile


// Receivers: list-2 bodies j in [j0, j0 + ET) (one thread each).  Partners: list-1 bodies
// i in [ibeg, iend) (i < j when `upper`, i.e. pl-pl).  A pair is written as
// (i + 1 + base1, j + 1 + base2); lists are sorted afterwards, so the tiling is invisible.
// DISCARD: the close-approach scan of swiftest_discard_pl_tp instead (list 1 = pl with
// renc1 = their radii, list 2 = the tp with status st2): the FP64 test is
// swiftest_discard_pl_close with r2crit = radius^2, and a hit sets o2[base2 + j] = 1.  The
// prefilter bound holds for it too (same closest-approach expression).
// Whole block; returns at once (block-uniformly) when the range is empty.
template <bool DISCARD>
__device__ __forceinline__ void enc_tri_tile(
    int n1, const float4 *__restrict__ A1, const float4 *__restrict__ B1, const float4 *__restrict__ V1,
    const double *__restrict__ r1, const double *__restrict__ v1, const double *__restrict__ renc1, int n2,
    const float4 *__restrict__ A2, const float4 *__restrict__ B2, const float4 *__restrict__ V2,
    const double *__restrict__ r2, const double *__restrict__ v2, const double *__restrict__ renc2, int upper, int j0,
    int ibeg, int iend, int base1, int base2, double dt, long long cap, int32_t *__restrict__ o1,
    int32_t *__restrict__ o2, int32_t *__restrict__ olv, unsigned long long *__restrict__ count,
    const int32_t *__restrict__ st2 = nullptr) {
    __shared__ float4 sa[EP], sb[EP], sv[EP];
    const int j = j0 + threadIdx.x;
    const bool active = j < n2 && (!DISCARD || st2[j] == ST_ACTIVE);
    iend = min(n1, iend);
    if (upper) iend = min(iend, j0 + ET);
    if (ibeg >= iend) return;  // whole block outside the upper triangle
    BodyF q;
    if (active) {
        q.a = A2[j];
        q.b = B2[j];
        q.v = V2[j];
    }
    const int own_end = upper ? min(iend, j) : iend;
    const float dtf = __double2float_ru(fabs(dt)) * (1.0f + 1e-6f);  // |dt| bounds either direction of time
    for (int i0 = ibeg; i0 < iend; i0 += EP) {
        if (threadIdx.x < EP && i0 + threadIdx.x < iend) {
            sa[threadIdx.x] = A1[i0 + threadIdx.x];
            sb[threadIdx.x] = B1[i0 + threadIdx.x];
            sv[threadIdx.x] = V1[i0 + threadIdx.x];
        }
        __syncthreads();
        if (active) {
            const int nt = min(EP, own_end - i0);
            for (int ii = 0; ii < nt; ii++) {
                BodyF p;
                p.a = sa[ii];
                p.b = sb[ii];
                p.v = sv[ii];
                if (prefilter_reject(p, q, dtf)) continue;
                const int i = i0 + ii;
                const double xr = r2[3 * j + 0] - r1[3 * i + 0];
                const double yr = r2[3 * j + 1] - r1[3 * i + 1];
                const double zr = r2[3 * j + 2] - r1[3 * i + 2];
                const double vxr = v2[3 * j + 0] - v1[3 * i + 0];
                const double vyr = v2[3 * j + 1] - v1[3 * i + 1];
                const double vzr = v2[3 * j + 2] - v1[3 * i + 2];
                if (DISCARD) {
                    if (d_discard_close(xr, yr, zr, vxr, vyr, vzr, dt, renc1[i] * renc1[i])) o2[base2 + j] = 1;
                    continue;
                }
                const double renc12 = renc1[i] + (renc2 ? renc2[j] : 0.0);
                int lenc, lv;
                d_encounter_one(xr, yr, zr, vxr, vyr, vzr, renc12, dt, lenc, lv);
                if (lenc) {
                    const unsigned long long k = atomicAdd(count, 1ull);
                    if ((long long)k < cap) {
                        o1[k] = i + 1 + base1;
                        o2[k] = j + 1 + base2;
                        olv[k] = lv;
                    }
                }
            }
        }
        __syncthreads();
    }
}

// One system: receivers tile blockIdx.x, partner chunk blockIdx.y.
template <bool DISCARD>
__global__ void __launch_bounds__(ET) k_encounter_tri(
    int n1, const float4 *__restrict__ A1, const float4 *__restrict__ B1, const float4 *__restrict__ V1,
    const double *__restrict__ r1, const double *__restrict__ v1, const double *__restrict__ renc1, int n2,
    const float4 *__restrict__ A2, const float4 *__restrict__ B2, const float4 *__restrict__ V2,
    const double *__restrict__ r2, const double *__restrict__ v2, const double *__restrict__ renc2, int upper,
    int shift2, double dt, int chunk, long long cap, int32_t *__restrict__ o1, int32_t *__restrict__ o2,
    int32_t *__restrict__ olv, unsigned long long *__restrict__ count, const int32_t *__restrict__ st2) {
    const int ibeg = blockIdx.y * chunk;
    enc_tri_tile<DISCARD>(n1, A1, B1, V1, r1, v1, renc1, n2, A2, B2, V2, r2, v2, renc2, upper, blockIdx.x * ET, ibeg,
                          ibeg + chunk, 0, shift2, dt, cap, o1, o2, olv, count, st2);
}

// Batched (ensemble) check: block b takes item b = (system s, first receiver j0) of a
// table sorted by cost.  List 1 is system s's pl ([off1[s], off1[s] + n1[s]) in the
// float/double arrays), list 2 its pl again (upper, pl-pl) or its tp (off2, n2).  Pairs
// are written with global 1-based indices, so the sorted list groups by system.
template <bool DISCARD>
__global__ void __launch_bounds__(ET) k_encounter_tri_batched(
    const int4 *__restrict__ items, const int32_t *__restrict__ off1, const int32_t *__restrict__ n1s,
    const float4 *__restrict__ A1, const float4 *__restrict__ B1, const float4 *__restrict__ V1,
    const double *__restrict__ r1, const double *__restrict__ v1, const double *__restrict__ renc1,
    const int32_t *__restrict__ off2, const int32_t *__restrict__ n2s, const float4 *__restrict__ A2,
    const float4 *__restrict__ B2, const float4 *__restrict__ V2, const double *__restrict__ r2,
    const double *__restrict__ v2, const double *__restrict__ renc2, int upper, double dt, long long cap,
    int32_t *__restrict__ o1, int32_t *__restrict__ o2, int32_t *__restrict__ olv,
    unsigned long long *__restrict__ count, const int32_t *__restrict__ st2) {
    const int4 w = items[blockIdx.x];
    const int s = w.x;
    const int a = off1[s], b = off2[s];
    enc_tri_tile<DISCARD>(n1s[s], A1 + a, B1 + a, V1 + a, r1 + 3 * (size_t)a, v1 + 3 * (size_t)a, renc1 + a,
                          n2s[s], A2 + b, B2 + b, V2 + b, r2 + 3 * (size_t)b, v2 + 3 * (size_t)b,
                          renc2 ? renc2 + b : nullptr, upper, w.y, 0, n1s[s], a, b, dt, cap, o1, o2, olv, count,
                          st2 ? st2 + b : nullptr);
}

// ------------------------------------------------------------------ sorting
// Generic (key, val) sort, ascending by (key, val).  Padding uses all-ones.
constexpr int SORT_SMEM_N = 4096;  // elements sorted in one CTA (48 KB)

__device__ __forceinline__ bool kv_greater(uint64_t ka, uint32_t va, uint64_t kb, uint32_t vb) {
    return ka > kb || (ka == kb && va > vb);
}

__global__ void k_bitonic_shared(uint64_t *keys, uint32_t *vals, int64_t n_pad, int kmax_global) {
    // Sorts each SORT_SMEM_N segment completely (kmax_global == 0) or finishes the
    // merge stages j < SORT_SMEM_N of a global stage k (kmax_global == k).
    __shared__ uint64_t sk[SORT_SMEM_N];
    __shared__ uint32_t sv[SORT_SMEM_N];
    const int64_t base = (int64_t)blockIdx.x * SORT_SMEM_N;
    const int len = (int)((n_pad - base) < (int64_t)SORT_SMEM_N ? (n_pad - base) : (int64_t)SORT_SMEM_N);
    for (int t = threadIdx.x; t < len; t += blockDim.x) {
        sk[t] = keys[base + t];
        sv[t] = vals[base + t];
    }
    __syncthreads();
    if (kmax_global == 0) {
        for (int k = 2; k <= len; k <<= 1) {
            for (int jj = k >> 1; jj > 0; jj >>= 1) {
                for (int t = threadIdx.x; t < len; t += blockDim.x) {
                    const int p = t ^ jj;
                    if (p > t) {
                        const int64_t gt = base + t;
                        const bool up = ((gt & k) == 0);
                        const bool sw = up ? kv_greater(sk[t], sv[t], sk[p], sv[p]) : kv_greater(sk[p], sv[p], sk[t], sv[t]);
                        if (sw) {
                            uint64_t tk = sk[t];
                            sk[t] = sk[p];
                            sk[p] = tk;
                            uint32_t tv = sv[t];
                            sv[t] = sv[p];
                            sv[p] = tv;
                        }
                    }
                }
                __syncthreads();
            }
        }
    } else {
        const int64_t k = kmax_global;
        for (int jj = SORT_SMEM_N >> 1; jj > 0; jj >>= 1) {
            for (int t = threadIdx.x; t < len; t += blockDim.x) {
                const int p = t ^ jj;
                if (p > t) {
                    const int64_t gt = base + t;
                    const bool up = ((gt & k) == 0);
                    const bool sw = up ? kv_greater(sk[t], sv[t], sk[p], sv[p]) : kv_greater(sk[p], sv[p], sk[t], sv[t]);
                    if (sw) {
                        uint64_t tk = sk[t];
                        sk[t] = sk[p];
                        sk[p] = tk;
                        uint32_t tv = sv[t];
                        sv[t] = sv[p];
                        sv[p] = tv;
                    }
                }
            }
            __syncthreads();
        }
    }
    for (int t = threadIdx.x; t < len; t += blockDim.x) {
        keys[base + t] = sk[t];
        vals[base + t] = sv[t];
    }
}

__global__ void k_bitonic_global(uint64_t *keys, uint32_t *vals, int64_t n_pad, int64_t k, int64_t jj) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= n_pad) return;
    const int64_t p = t ^ jj;
    if (p <= t) return;
    const bool up = ((t & k) == 0);
    const uint64_t kt = keys[t], kp = keys[p];
    const uint32_t vt = vals[t], vp = vals[p];
    const bool sw = up ? kv_greater(kt, vt, kp, vp) : kv_greater(kp, vp, kt, vt);
    if (sw) {
        keys[t] = kp;
        keys[p] = kt;
        vals[t] = vp;
        vals[p] = vt;
    }
}

__global__ void k_fill_pad(uint64_t *keys, uint32_t *vals, int64_t n, int64_t n_pad) {
    const int64_t t = n + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t < n_pad) {
        keys[t] = ~0ull;
        vals[t] = ~0u;
    }
}

int64_t sort_padded_len(int64_t n) {
    int64_t p = 1;
    while (p < n) p <<= 1;
    return p < 2 ? 2 : p;
}

// keys/vals must have room for sort_padded_len(n) elements.
int sort_kv(swg_ctx *c, int64_t n, uint64_t *keys, uint32_t *vals) {
    if (n <= 1) return SWG_OK;
    const int64_t n_pad = sort_padded_len(n);
    if (n_pad > n) {
        k_fill_pad<<<(int)((n_pad - n + 255) / 256), 256, 0, c->stream>>>(keys, vals, n, n_pad);
        c->launches++;
    }
    const int64_t nseg = (n_pad + SORT_SMEM_N - 1) / SORT_SMEM_N;
    k_bitonic_shared<<<(int)nseg, 512, 0, c->stream>>>(keys, vals, n_pad, 0);
    c->launches++;
    for (int64_t k = 2 * (int64_t)SORT_SMEM_N; k <= n_pad; k <<= 1) {
        for (int64_t jj = k >> 1; jj >= SORT_SMEM_N; jj >>= 1) {
            k_bitonic_global<<<(int)((n_pad + 255) / 256), 256, 0, c->stream>>>(keys, vals, n_pad, k, jj);
            c->launches++;
        }
        k_bitonic_shared<<<(int)nseg, 512, 0, c->stream>>>(keys, vals, n_pad, (int)k);
        c->launches++;
    }
    return launch_status(c, "sort_kv");
}

// pack (i1,i2,lv) into key=(i1<<32|i2), val=lv ; and back
__global__ void k_pack_pairs(int64_t n, const int32_t *i1, const int32_t *i2, const int32_t *lv, uint64_t *keys,
                             uint32_t *vals) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= n) return;
    keys[t] = ((uint64_t)(uint32_t)i1[t] << 32) | (uint64_t)(uint32_t)i2[t];
    vals[t] = (uint32_t)lv[t];
}
// unpack, dropping repeated (i1,i2) keys (they carry the same lvdotr); the
// surviving count goes to *nout.  Single pass with a block-wide prefix via atomics
// is not order-preserving, so compaction uses a flag + scan in one block.
__global__ void k_unpack_unique(int64_t n, const uint64_t *keys, const uint32_t *vals, int32_t *i1, int32_t *i2,
                                int32_t *lv, unsigned long long *nout) {
    // one block; sequential chunks with block scan
    __shared__ int64_t s_base;
    __shared__ int s_scan[1024];
    if (threadIdx.x == 0) s_base = 0;
    __syncthreads();
    for (int64_t c0 = 0; c0 < n; c0 += blockDim.x) {
        const int64_t t = c0 + threadIdx.x;
        int keep = 0;
        if (t < n) keep = (t == 0) || (keys[t] != keys[t - 1]);
        s_scan[threadIdx.x] = keep;
        __syncthreads();
        for (int off = 1; off < (int)blockDim.x; off <<= 1) {
            int add = (threadIdx.x >= (unsigned)off) ? s_scan[threadIdx.x - off] : 0;
            __syncthreads();
            s_scan[threadIdx.x] += add;
            __syncthreads();
        }
        if (keep) {
            const int64_t o = s_base + s_scan[threadIdx.x] - 1;
            i1[o] = (int32_t)(keys[t] >> 32);
            i2[o] = (int32_t)(keys[t] & 0xffffffffull);
            lv[o] = (int32_t)vals[t];
        }
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) s_base += s_scan[threadIdx.x];
        __syncthreads();
    }
    if (threadIdx.x == 0) *nout = (unsigned long long)s_base;
}

// scratch: 12 bytes per padded element
size_t sort_pairs_scratch_bytes(int64_t n) { return (size_t)sort_padded_len(n) * 12 + 256; }

int sort_pairs_unique(swg_ctx *c, int64_t n, int32_t *i1, int32_t *i2, int32_t *lv, void *scratch,
                      unsigned long long *d_nout) {
    if (n <= 0) return SWG_OK;
    const int64_t n_pad = sort_padded_len(n);
    uint64_t *keys = (uint64_t *)scratch;
    uint32_t *vals = (uint32_t *)(keys + n_pad);
    k_pack_pairs<<<(int)((n + 255) / 256), 256, 0, c->stream>>>(n, i1, i2, lv, keys, vals);
    c->launches++;
    SWG_TRY(sort_kv(c, n, keys, vals));
    k_unpack_unique<<<1, 1024, 0, c->stream>>>(n, keys, vals, i1, i2, lv, d_nout);
    c->launches++;
    return launch_status(c, "sort_pairs_unique");
}

// ------------------------------------------------------------------ sort & sweep
// orderable bit pattern of a double (ascending numeric order)
__device__ __forceinline__ uint64_t d2key(double x) {
    if (x == 0.0) x = 0.0;  // -0.0 compares equal to +0.0: one key for both
    uint64_t u = (uint64_t)__double_as_longlong(x);
    return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}

// gfortran NORM2 (scaled sum of squares), as used for |r| in the sweep extents
__device__ __forceinline__ double d_norm2e(double a, double b, double c) {
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

// extents: body b (0..ntot-1) -> keys[b] = rmin, keys[ntot+b] = rmax, vals = extent index
__global__ void k_sas_extents(int n1, const double *r1, const double *renc1, int n2, const double *r2,
                              const double *renc2, uint64_t *keys, uint32_t *vals) {
    const int ntot = n1 + n2;
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= ntot) return;
    const double *r = b < n1 ? &r1[3 * b] : &r2[3 * (b - n1)];
    const double rc = b < n1 ? renc1[b] : (renc2 ? renc2[b - n1] : 0.0);
    const double rmag = d_norm2e(r[0], r[1], r[2]);
    keys[b] = d2key(rmag - RSWEEP_FACTOR * rc);
    vals[b] = (uint32_t)b;
    keys[ntot + b] = d2key(rmag + RSWEEP_FACTOR * rc);
    vals[ntot + b] = (uint32_t)(ntot + b);
}

__global__ void k_sas_positions(int ntot, const uint32_t *vals, int32_t *ibeg, int32_t *iend) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= 2 * ntot) return;
    const uint32_t e = vals[k];
    if (e < (uint32_t)ntot)
        ibeg[e] = k + 1;
    else
        iend[e - ntot] = k + 1;
}

// sweep: body b with loverlap tests the bodies whose extents are strictly inside its box.
// FA/FB/FV: float copies of the ntot bodies (list 1 then list 2) for the conservative FP32
// prefilter, which drops only pairs the FP64 test is certain to reject (see
// prefilter_reject), so the list is the same.  One warp per body: its lanes take the
// entries of the body's box 32 at a time (a box holds up to hundreds of entries in a
// disk, and a thread per body left the scan latency-bound on its serial loads); the
// pairs' order in the output does not matter (the lists are sorted afterwards).
__global__ void k_sas_sweep(int n1, const double *r1, const double *v1, const double *renc1, int n2,
                            const double *r2, const double *v2, const double *renc2, int single, int shift2, double dt,
                            const uint32_t *vals, const int32_t *ibeg, const int32_t *iend, const float4 *FA,
                            const float4 *FB, const float4 *FV, long long cap, int32_t *o1, int32_t *o2, int32_t *olv,
                            unsigned long long *count) {
    const int ntot = n1 + n2;
    const int i = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);  // warp-uniform
    if (i >= ntot) return;
    if (!((ibeg[i] + 1) < (iend[i] - 1))) return;
    const bool il1 = i < n1;
    const double *ri = il1 ? &r1[3 * i] : &r2[3 * (i - n1)];
    const double *vi = il1 ? &v1[3 * i] : &v2[3 * (i - n1)];
    const double renci = il1 ? renc1[i] : (renc2 ? renc2[i - n1] : 0.0);
    const BodyF q = {FA[i], FB[i], FV[i]};
    const float dtf = __double2float_ru(fabs(dt)) * (1.0f + 1e-6f);  // |dt| bounds either direction of time
    const int pend = iend[i] - 1;
    for (int p = ibeg[i] + 1 + (int)(threadIdx.x & 31); p <= pend; p += 32) {
        int b = (int)vals[p - 1];
        if (b >= ntot) b -= ntot;
        const bool bl1 = b < n1;
        if (!single && bl1 == il1) continue;
        const BodyF f = {FA[b], FB[b], FV[b]};
        if (prefilter_reject(f, q, dtf)) continue;
        const double *rb = bl1 ? &r1[3 * b] : &r2[3 * (b - n1)];
        const double *vb = bl1 ? &v1[3 * b] : &v2[3 * (b - n1)];
        const double rencb = bl1 ? renc1[b] : (renc2 ? renc2[b - n1] : 0.0);
        int lenc, lv;
        d_encounter_one(rb[0] - ri[0], rb[1] - ri[1], rb[2] - ri[2], vb[0] - vi[0], vb[1] - vi[1], vb[2] - vi[2],
                        renci + rencb, dt, lenc, lv);
        if (!lenc) continue;
        int a, cidx;
        if (single) {
            a = min(i, b) + 1;
            cidx = max(i, b) + 1;
        } else if (il1) {
            a = i + 1;
            cidx = b - n1 + 1 + shift2;
        } else {
            a = b + 1;
            cidx = i - n1 + 1 + shift2;
        }
        const unsigned long long k = atomicAdd(count, 1ull);
        if ((long long)k < cap) {
            o1[k] = a;
            o2[k] = cidx;
            olv[k] = lv;
        }
    }
}

// keys | vals | ibeg | iend | radix-sort scratch, each 256-byte aligned
static size_t align256(size_t b) { return (b + 255) & ~size_t(255); }
size_t sas_scratch_bytes(int ntot) {
    const int64_t ne = 2 * (int64_t)ntot;
    return align256((size_t)ne * 8) + align256((size_t)ne * 4) + align256((size_t)ntot * 8) +
           align256((size_t)ntot * 3 * sizeof(float4)) + radix_sort_scratch_bytes(ne) + 256;
}

// Sort-and-sweep check of one list (single, pl-pl: list 1) or two lists (pl-tp), of one
// system or, with seg_of (the system of every extent, 2 (n1 + n2) entries), of every system
// of an ensemble at once: the extents sort into per-system runs and each body sweeps only its
// own run.  Pairs land unsorted in (o1, o2, olv) with the total in *count.  host_skip: the
// radix sort reads its digit counts back to skip constant digits (synchronizes the stream).
int sas_launch(swg_ctx *c, int n1, const double *r1, const double *v1, const double *renc1, int n2, const double *r2,
               const double *v2, const double *renc2, int single, int shift2, double dt, long long cap, int32_t *o1,
               int32_t *o2, int32_t *olv, unsigned long long *count, void *scratch, const int32_t *seg_of,
               int seg_bits, bool host_skip) {
    const int nb1 = n1, nb2 = single ? 0 : n2;
    const int ntot = nb1 + nb2;
    if (ntot <= 0) return SWG_OK;
    const int64_t ne = 2 * (int64_t)ntot;
    char *p = (char *)scratch;
    uint64_t *keys = (uint64_t *)p;
    uint32_t *vals = (uint32_t *)(p += align256((size_t)ne * 8));
    int32_t *ibeg = (int32_t *)(p += align256((size_t)ne * 4));
    int32_t *iend = ibeg + ntot;
    float4 *FA = (float4 *)(p += align256((size_t)ntot * 8)), *FB = FA + ntot, *FV = FB + ntot;
    void *rs = p + align256((size_t)ntot * 3 * sizeof(float4));
    k_sas_extents<<<(ntot + 127) / 128, 128, 0, c->stream>>>(nb1, r1, renc1, nb2, r2, renc2, keys, vals);
    c->launches++;
    if (nb1 > 0) {
        k_encounter_prep<<<(nb1 + 255) / 256, 256, 0, c->stream>>>(nb1, r1, v1, renc1, FA, FB, FV);
        c->launches++;
    }
    if (nb2 > 0) {
        k_encounter_prep<<<(nb2 + 255) / 256, 256, 0, c->stream>>>(nb2, r2, v2, renc2, FA + nb1, FB + nb1, FV + nb1);
        c->launches++;
    }
    // stable radix sort by extent; the extents enter in index order, so ties keep it
    SWG_TRY(radix_sort_kv(c, ne, keys, vals, rs, seg_of, seg_bits, host_skip));
    k_sas_positions<<<(int)((ne + 255) / 256), 256, 0, c->stream>>>(ntot, vals, ibeg, iend);
    c->launches++;
    k_sas_sweep<<<(unsigned)((32 * (int64_t)ntot + 127) / 128), 128, 0, c->stream>>>(
        nb1, r1, v1, renc1, nb2, r2, v2, renc2, single, shift2, dt, vals, ibeg, iend, FA, FB, FV, cap, o1, o2, olv,
        count);
    c->launches++;
    return launch_status(c, "encounter_sas");
}

// Runs one encounter check; pairs land unsorted in (o1,o2,olv) (first cap of
// them) and the total in *count (device).  Caller sorts/dedups afterwards.
int encounter_launch(swg_ctx *c, int mode, int n1, const double *r1, const double *v1, const double *renc1, int n2,
                     const double *r2, const double *v2, const double *renc2, int upper, int shift2, double dt,
                     long long cap, int32_t *o1, int32_t *o2, int32_t *olv, unsigned long long *count,
                     void *sas_scratch) {
    if (mode == SWG_ENC_SORTSWEEP)  // single list when upper (pl-pl), double list otherwise
        return sas_launch(c, n1, r1, v1, renc1, n2, r2, v2, renc2, upper ? 1 : 0, shift2, dt, cap, o1, o2, olv, count,
                          sas_scratch, nullptr, 0, true);
    if (n1 <= 0 || n2 <= 0) return SWG_OK;
    // float copies for the prefilter: list 1 then (unless it is the same list) list 2
    float4 *A1 = (float4 *)sas_scratch, *B1 = A1 + n1, *V1 = B1 + n1;
    float4 *A2 = A1, *B2 = B1, *V2 = V1;
    k_encounter_prep<<<(n1 + 255) / 256, 256, 0, c->stream>>>(n1, r1, v1, renc1, A1, B1, V1);
    c->launches++;
    const bool same = upper && r2 == r1;
    if (!same) {
        A2 = V1 + n1;
        B2 = A2 + n2;
        V2 = B2 + n2;
        k_encounter_prep<<<(n2 + 255) / 256, 256, 0, c->stream>>>(n2, r2, v2, renc2, A2, B2, V2);
        c->launches++;
    }
    const int bx = (n2 + ET - 1) / ET;
    const int target = 4 * (c->num_sms > 0 ? c->num_sms : 152);
    int nchunk = (target + bx - 1) / bx;
    const int maxchunk = (n1 + EP - 1) / EP;
    if (nchunk > maxchunk) nchunk = maxchunk;
    if (nchunk < 1) nchunk = 1;
    int chunk = (n1 + nchunk - 1) / nchunk;
    chunk = (chunk + EP - 1) / EP * EP;
    nchunk = (n1 + chunk - 1) / chunk;
    k_encounter_tri<false><<<dim3(bx, nchunk), ET, 0, c->stream>>>(n1, A1, B1, V1, r1, v1, renc1, n2, A2, B2, V2, r2,
                                                                   v2, renc2, upper, shift2, dt, chunk, cap, o1, o2, olv,
                                                                   count, nullptr);
    c->launches++;
    return launch_status(c, "encounter_tri");
}

// Float copies (A, B, V) of n bodies for the prefilter of the batched check.
int encounter_prep_launch(swg_ctx *c, int64_t n, const double *r, const double *v, const double *renc, float4 *A,
                          float4 *B, float4 *V) {
    if (n <= 0) return SWG_OK;
    k_encounter_prep<<<(int)((n + 255) / 256), 256, 0, c->stream>>>((int)n, r, v, renc, A, B, V);
    c->launches++;
    return launch_status(c, "encounter_prep");
}

// Batched TRIANGULAR check over an item table (see k_encounter_tri_batched); F1/F2 are
// the prepared float copies (3 arrays of float4 each, A|B|V) of list 1 and list 2.
int encounter_tri_batched(swg_ctx *c, int nitems, const int4 *items, const int32_t *off1, const int32_t *n1,
                          const float4 *F1, int64_t nf1, const double *r1, const double *v1, const double *renc1,
                          const int32_t *off2, const int32_t *n2, const float4 *F2, int64_t nf2, const double *r2,
                          const double *v2, const double *renc2, int upper, double dt, long long cap, int32_t *o1,
                          int32_t *o2, int32_t *olv, unsigned long long *count) {
    if (nitems <= 0) return SWG_OK;
    k_encounter_tri_batched<false><<<nitems, ET, 0, c->stream>>>(items, off1, n1, F1, F1 + nf1, F1 + 2 * nf1, r1, v1,
                                                                 renc1, off2, n2, F2, F2 + nf2, F2 + 2 * nf2, r2, v2,
                                                                 renc2, upper, dt, cap, o1, o2, olv, count, nullptr);
    c->launches++;
    return launch_status(c, "encounter_tri_batched");
}

// Close-approach discard scan (swiftest_discard_pl_tp, src/swiftest/swiftest_discard.f90:244-290)
// of the ACTIVE test particles of one system against its massive bodies: heliocentric
// positions and velocities, r2crit = radius^2; flag[j] = 1 for every tp that comes too
// close to some pl (flag zeroed by the caller).  F: scratch for the float copies,
// 3 * (npl + ntp) float4.
int discard_pl_tp_launch(swg_ctx *c, int32_t npl, const double *rpl, const double *vpl, const double *radius,
                         int32_t ntp, const double *rtp, const double *vtp, const int32_t *tstatus, double dt,
                         float4 *F, int32_t *flag) {
    if (npl <= 0 || ntp <= 0) return SWG_OK;
    float4 *A1 = F, *B1 = A1 + npl, *V1 = B1 + npl, *A2 = V1 + npl, *B2 = A2 + ntp, *V2 = B2 + ntp;
    k_encounter_prep<<<(npl + 255) / 256, 256, 0, c->stream>>>(npl, rpl, vpl, radius, A1, B1, V1);
    k_encounter_prep<<<(ntp + 255) / 256, 256, 0, c->stream>>>(ntp, rtp, vtp, nullptr, A2, B2, V2);
    c->launches += 2;
    const int bx = (ntp + ET - 1) / ET;
    const int target = 4 * (c->num_sms > 0 ? c->num_sms : 152);
    int nchunk = std::max(1, std::min((target + bx - 1) / bx, (npl + EP - 1) / EP));
    int chunk = (npl + nchunk - 1) / nchunk;
    chunk = (chunk + EP - 1) / EP * EP;
    nchunk = (npl + chunk - 1) / chunk;
    k_encounter_tri<true><<<dim3(bx, nchunk), ET, 0, c->stream>>>(npl, A1, B1, V1, rpl, vpl, radius, ntp, A2, B2, V2,
                                                                  rtp, vtp, nullptr, 0, 0, dt, chunk, 0, nullptr,
                                                                  flag, nullptr, nullptr, tstatus);
    c->launches++;
    return launch_status(c, "discard_pl_tp");
}

// The same scan for every system of an ensemble over its pl-tp item table; F1/F2: the
// float copies (A|B|V) of all pl (nf1 = NPL) and tp (nf2 = NTP), prepared here.
int discard_pl_tp_batched(swg_ctx *c, int nitems, const int4 *items, const int32_t *poff, const int32_t *npl,
                          int64_t NPL, const double *rpl, const double *vpl, const double *radius,
                          const int32_t *toff, const int32_t *ntp, int64_t NTP, const double *rtp, const double *vtp,
                          const int32_t *tstatus, double dt, float4 *F1, float4 *F2, int32_t *flag) {
    if (nitems <= 0) return SWG_OK;
    SWG_TRY(encounter_prep_launch(c, NPL, rpl, vpl, radius, F1, F1 + NPL, F1 + 2 * NPL));
    SWG_TRY(encounter_prep_launch(c, NTP, rtp, vtp, nullptr, F2, F2 + NTP, F2 + 2 * NTP));
    k_encounter_tri_batched<true><<<nitems, ET, 0, c->stream>>>(items, poff, npl, F1, F1 + NPL, F1 + 2 * NPL, rpl, vpl,
                                                                radius, toff, ntp, F2, F2 + NTP, F2 + 2 * NTP, rtp,
                                                                vtp, nullptr, 0, dt, 0, nullptr, flag, nullptr,
                                                                nullptr, tstatus);
    c->launches++;
    return launch_status(c, "discard_pl_tp_batched");
}

// scratch of one encounter_launch call (mode, list sizes)
size_t encounter_scratch_bytes(int mode, int n1, int n2) {
    if (mode == SWG_ENC_SORTSWEEP) return sas_scratch_bytes(n1 + n2);
    return (size_t)3 * sizeof(float4) * (size_t)(n1 + n2) + 256;
}

// shift index2 by `shift` for entries [from, to)
__global__ void k_shift_i2(long long from, long long to, int32_t *i2, int shift) {
    const long long t = from + blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < to) i2[t] += shift;
}

int shift_index2(swg_ctx *c, long long from, long long to, int32_t *i2, int shift) {
    if (to <= from || shift == 0) return SWG_OK;
    k_shift_i2<<<(int)((to - from + 255) / 256), 256, 0, c->stream>>>(from, to, i2, shift);
    c->launches++;
    return launch_status(c, "shift_i2");
}

}  // namespace swg

namespace swg {

int encounter_check_kind(swg_ctx *c, EncWork &w, int kind, int mode, int32_t n1, const double *r1,
                         const double *v1, const double *renc1, int32_t n2, const double *r2, const double *v2,
                         const double *renc2, double dt, int64_t *n_out, int32_t **o1, int32_t **o2,
                         int32_t **olv) {
    *n_out = 0;
    SWG_TRY(ensure(c, w.counters, 2 * sizeof(unsigned long long)));
    unsigned long long *d_count = (unsigned long long *)w.counters.ptr;
    if (w.rawcap < 1024) {
        w.rawcap = 1024;
        SWG_TRY(ensure(c, w.raw, (size_t)w.rawcap * 3 * sizeof(int32_t)));
    }
    const int ntot = (kind == 0 ? n1 : n1 + n2);
    SWG_TRY(ensure(c, w.sort, encounter_scratch_bytes(mode, n1, kind == 0 ? n1 : n2)));
    (void)ntot;
    unsigned long long h_count = 0;
    for (int attempt = 0; attempt < 8; attempt++) {
        int32_t *i1 = (int32_t *)w.raw.ptr, *i2 = i1 + w.rawcap, *lv = i2 + w.rawcap;
        SWG_TRY(cuda_status(c, cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), c->stream), "memset"));
        if (kind == 0) {
            SWG_TRY(encounter_launch(c, mode, n1, r1, v1, renc1, n1, r1, v1, renc1, 1, 0, dt, w.rawcap, i1, i2, lv,
                                     d_count, w.sort.ptr));
        } else if (kind == 1) {
            SWG_TRY(encounter_launch(c, mode, n1, r1, v1, renc1, n1, r1, v1, renc1, 1, 0, dt, w.rawcap, i1, i2, lv,
                                     d_count, w.sort.ptr));
            if (n2 > 0)
                SWG_TRY(encounter_launch(c, mode, n1, r1, v1, renc1, n2, r2, v2, renc2, 0, n1, dt, w.rawcap, i1, i2,
                                         lv, d_count, w.sort.ptr));
        } else {
            SWG_TRY(encounter_launch(c, mode, n1, r1, v1, renc1, n2, r2, v2, nullptr, 0, 0, dt, w.rawcap, i1, i2, lv,
                                     d_count, w.sort.ptr));
        }
        SWG_TRY(cuda_status(c, cudaMemcpyAsync(&h_count, d_count, sizeof(h_count), cudaMemcpyDeviceToHost, c->stream),
                            "count"));
        SWG_TRY(cuda_status(c, cudaStreamSynchronize(c->stream), "sync"));
        if ((int64_t)h_count <= w.rawcap) break;
        // grow the raw buffers and redo the check
        w.rawcap = (int64_t)h_count + h_count / 2 + 1024;
        DevBuf fresh;
        SWG_TRY(ensure(c, fresh, (size_t)w.rawcap * 3 * sizeof(int32_t)));
        cudaFree(w.raw.ptr);
        w.raw = fresh;
    }
    int32_t *i1 = (int32_t *)w.raw.ptr, *i2 = i1 + w.rawcap, *lv = i2 + w.rawcap;
    *o1 = i1;
    *o2 = i2;
    *olv = lv;
    if (h_count == 0) return SWG_OK;
    const bool need_unique = (mode == SWG_ENC_SORTSWEEP);
    (void)need_unique;
    // sort by (index1, index2) and drop repeats (sweep duplicates); the sort scratch
    // is separate from the sweep scratch only in size, the sweep is finished.
    const size_t need = sort_pairs_scratch_bytes((int64_t)h_count);
    if (mode == SWG_ENC_SORTSWEEP) {
        if (w.sort.bytes < need) SWG_TRY(ensure(c, w.sort, need));
    } else {
        SWG_TRY(ensure(c, w.sort, need));
    }
    SWG_TRY(sort_pairs_unique(c, (int64_t)h_count, i1, i2, lv, w.sort.ptr, d_count + 1));
    unsigned long long h_unique = 0;
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(&h_unique, d_count + 1, sizeof(h_unique), cudaMemcpyDeviceToHost, c->stream),
                        "count"));
    SWG_TRY(cuda_status(c, cudaStreamSynchronize(c->stream), "sync"));
    *n_out = (int64_t)h_unique;
    return SWG_OK;
}

}  // namespace swg
