// radix_sort.cu -- stable LSD radix sort of (64-bit key, 32-bit value) pairs for sm_103a.
//
// Sorts the bounding-box extents of the sort-and-sweep encounter check
// (encounter_check.f90:763-792 sorts them with a quicksort; here the order is the same
// because ties break by extent index, see below).  Keys are order-preserving bit patterns
// of doubles; values are extent indices, given in ascending order, so a stable sort by key
// orders the pairs by (key, value).  An optional segment id per value (the system of an
// extent in a batched ensemble) forms the most significant digits: one call sorts every
// system's extents into contiguous per-system runs.
//
// Passes: 8-bit digits, least significant first, each a reduce-then-scan over tiles of 256
// to 2048 elements (fewer per tile for small sorts): per-tile digit counts (k_rs_upsweep),
// an exclusive scan of each digit's row of tile counts with the row totals (k_rs_scan_rows,
// one block per digit), and a stable scatter (k_rs_scatter) that adds the digit's base from
// the totals and ranks the tile's
// elements column by column with warp match_any and per-warp prefix counts in shared
// memory.  One pass over the data first counts every digit of every pass
// (k_rs_hist_all); the host reads those counts and skips the passes whose digit is the
// same for all elements (for example the exponent bytes of positions within one or two
// octaves); a caller that must not synchronize runs every pass instead.  No kernel waits
// on another block: there is nothing to spin on.
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "swg_internal.cuh"

namespace swg {

namespace {

constexpr int RS_BINS = 256;
constexpr int RS_THREADS = 256;
constexpr int RS_COLS = 8;                       // most elements per thread per tile (tiles of up to 2048)
constexpr int RS_KEY_PASSES = 8;                 // 64-bit keys
constexpr int RS_MAX_SEG_PASSES = 4;             // 32-bit segment ids
constexpr int RS_MAX_PASSES = RS_KEY_PASSES + RS_MAX_SEG_PASSES;
constexpr unsigned FULL = 0xffffffffu;

// digit of pass p: key bytes first (p < 8), then segment-id bytes
__device__ __forceinline__ unsigned rs_digit(int p, uint64_t key, uint32_t val, const int32_t *__restrict__ seg_of) {
    if (p < RS_KEY_PASSES) return (unsigned)(key >> (8 * p)) & 0xffu;
    return ((unsigned)seg_of[val] >> (8 * (p - RS_KEY_PASSES))) & 0xffu;
}

// counts of every digit of every pass: hist[p * 256 + d]
__global__ void __launch_bounds__(RS_THREADS) k_rs_hist_all(int64_t n, const uint64_t *__restrict__ keys,
                                                            const uint32_t *__restrict__ vals,
                                                            const int32_t *__restrict__ seg_of, int npass,
                                                            unsigned *__restrict__ hist) {
    __shared__ unsigned sh[RS_MAX_PASSES * RS_BINS];
    for (int t = threadIdx.x; t < npass * RS_BINS; t += RS_THREADS) sh[t] = 0u;
    __syncthreads();
    for (int64_t e = blockIdx.x * (int64_t)RS_THREADS + threadIdx.x; e < n; e += (int64_t)gridDim.x * RS_THREADS) {
        const uint64_t k = keys[e];
        const uint32_t v = vals[e];
        for (int p = 0; p < npass; p++) atomicAdd(&sh[p * RS_BINS + rs_digit(p, k, v, seg_of)], 1u);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < npass * RS_BINS; t += RS_THREADS)
        if (sh[t]) atomicAdd(&hist[t], sh[t]);
}

// per-tile digit counts of pass p: cnt[d * ntiles + tile]
__global__ void __launch_bounds__(RS_THREADS) k_rs_upsweep(int64_t n, const uint64_t *__restrict__ keys,
                                                           const uint32_t *__restrict__ vals,
                                                           const int32_t *__restrict__ seg_of, int p, int cols,
                                                           unsigned *__restrict__ cnt) {
    __shared__ unsigned sh[RS_BINS];
    sh[threadIdx.x] = 0u;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * RS_THREADS * cols;
    for (int c = 0; c < cols; c++) {
        const int64_t e = base + c * RS_THREADS + threadIdx.x;
        if (e < n) atomicAdd(&sh[rs_digit(p, keys[e], vals[e], seg_of)], 1u);
    }
    __syncthreads();
    cnt[(int64_t)threadIdx.x * gridDim.x + blockIdx.x] = sh[threadIdx.x];
}

// Exclusive scan of each digit's row of tile counts in place (block d scans row d,
// cnt[d * ntiles + tile], coalesced), and the row totals tot[d].  The scatter adds the
// digits' exclusive prefix of tot (a 256-wide scan per block), so the offsets are the
// digit-major exclusive scan of all counts without a single-block pass over all of them.
__global__ void __launch_bounds__(1024) k_rs_scan_rows(int64_t ntiles, unsigned *__restrict__ cnt,
                                                       unsigned *__restrict__ tot) {
    __shared__ unsigned s_w[32], s_carry;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    unsigned *row = cnt + (int64_t)blockIdx.x * ntiles;
    if (t == 0) s_carry = 0u;
    __syncthreads();
    for (int64_t b0 = 0; b0 < ntiles; b0 += 1024) {
        const int64_t i = b0 + t;
        const unsigned own = i < ntiles ? row[i] : 0u;
        unsigned x = own;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(FULL, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_w[w] = x;
        __syncthreads();
        if (w == 0) {
            unsigned z = s_w[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned y = __shfl_up_sync(FULL, z, o);
                if (lane >= o) z += y;
            }
            s_w[lane] = z;
        }
        __syncthreads();
        const unsigned carry = s_carry;
        if (i < ntiles) row[i] = carry + x - own + (w > 0 ? s_w[w - 1] : 0u);
        __syncthreads();
        if (t == 0) s_carry = carry + s_w[31];
        __syncthreads();
    }
    if (t == 0) tot[blockIdx.x] = s_carry;
}

// stable scatter of pass p: element e of the tile goes to its digit's offset for this tile
// plus the number of same-digit elements before it in the tile.  The tile is read in
// columns (element c * 256 + t at column c), which is its element order.
__global__ void __launch_bounds__(RS_THREADS) k_rs_scatter(int64_t n, const uint64_t *__restrict__ kin,
                                                           const uint32_t *__restrict__ vin,
                                                           const int32_t *__restrict__ seg_of, int p, int cols,
                                                           const unsigned *__restrict__ off,
                                                           const unsigned *__restrict__ tot,
                                                           uint64_t *__restrict__ kout, uint32_t *__restrict__ vout) {
    constexpr int NW = RS_THREADS / 32;
    __shared__ unsigned s_base[RS_BINS];      // next free position of each digit for this tile
    __shared__ unsigned s_wc[NW][RS_BINS];    // per-warp counts, then per-warp offsets, of one column
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    {  // digit t's first position: the totals of the smaller digits (256-wide exclusive scan)
        const unsigned own = tot[t];
        unsigned x = own;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(FULL, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_wc[0][w] = x;
        __syncthreads();
        unsigned before = 0u;
        for (int q = 0; q < w; q++) before += s_wc[0][q];
        s_base[t] = before + x - own + off[(int64_t)t * gridDim.x + blockIdx.x];
        __syncthreads();  // s_wc is cleared next
    }
    const int64_t base = (int64_t)blockIdx.x * RS_THREADS * cols;
    for (int c = 0; c < cols; c++) {
#pragma unroll
        for (int q = 0; q < NW; q++) s_wc[q][t] = 0u;
        __syncthreads();
        const int64_t e = base + c * RS_THREADS + t;
        const bool in = e < n;
        uint64_t k = 0;
        uint32_t v = 0;
        unsigned d = RS_BINS;  // out of range: a digit of its own, never written
        if (in) {
            k = kin[e];
            v = vin[e];
            d = rs_digit(p, k, v, seg_of);
        }
        const unsigned peers = __match_any_sync(FULL, d);
        const unsigned lower = peers & ((1u << lane) - 1u);
        const int rank = __popc(lower);
        if (in && lower == 0u) s_wc[w][d] = __popc(peers);
        __syncthreads();
        {  // thread t owns digit t: per-warp offsets within the column, then the new base
            unsigned run = s_base[t];
#pragma unroll
            for (int q = 0; q < NW; q++) {
                const unsigned x = s_wc[q][t];
                s_wc[q][t] = run;
                run += x;
            }
            s_base[t] = run;
        }
        __syncthreads();
        if (in) {
            const unsigned dst = s_wc[w][d] + rank;
            kout[dst] = k;
            vout[dst] = v;
        }
        __syncthreads();
    }
}

// util_sort with an index (base_module.f90:1361-1472): keys of the values, indices 0..n-1
__global__ void k_sort_index_keys(int64_t n, const double *__restrict__ arr, uint64_t *__restrict__ keys,
                                  uint32_t *__restrict__ vals) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    double x = arr[k];
    if (x == 0.0) x = 0.0;  // -0.0 compares equal to +0.0: one key for both
    const uint64_t u = (uint64_t)__double_as_longlong(x);
    keys[k] = (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
    vals[k] = (uint32_t)k;
}
__global__ void k_sort_index_out(int64_t n, const uint32_t *__restrict__ vals, int32_t *__restrict__ ind) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k < n) ind[k] = (int32_t)vals[k] + 1;
}

}  // namespace

size_t util_sort_index_scratch_bytes(int64_t n) { return (size_t)n * 12 + 256 + radix_sort_scratch_bytes(n); }

// ind = the 1-based permutation that sorts arr ascending, ties by index (device arrays)
int util_sort_index(swg_ctx *c, int64_t n, const double *arr, int32_t *ind, void *scratch) {
    if (n <= 0) return SWG_OK;
    uint64_t *keys = (uint64_t *)scratch;
    uint32_t *vals = (uint32_t *)(keys + n);
    void *rs = (char *)scratch + (((size_t)n * 12 + 255) & ~size_t(255));
    const int grid = (int)((n + 255) / 256);
    k_sort_index_keys<<<grid, 256, 0, c->stream>>>(n, arr, keys, vals);
    c->launches++;
    SWG_TRY(launch_status(c, "sort_index_keys"));
    SWG_TRY(radix_sort_kv(c, n, keys, vals, rs, nullptr, 0, true));
    k_sort_index_out<<<grid, 256, 0, c->stream>>>(n, vals, ind);
    c->launches++;
    return launch_status(c, "sort_index_out");
}

// Elements per thread of a tile: fewer for small sorts, so that the tiles still spread
// over the SMs (two per SM where n allows), at most RS_COLS.
static int rs_cols(int64_t n, int num_sms) {
    const int64_t per = (int64_t)RS_THREADS * 2 * (num_sms > 0 ? num_sms : 152);
    const int64_t cols = n / per;
    return (int)(cols < 1 ? 1 : (cols > RS_COLS ? RS_COLS : cols));
}

size_t radix_sort_scratch_bytes(int64_t n) {
    const int64_t ntiles = (n + RS_THREADS - 1) / RS_THREADS;  // enough for any tile size
    return (size_t)n * 12 + (size_t)ntiles * RS_BINS * 4 + (RS_MAX_PASSES + 1) * RS_BINS * 4 + 1024;
}

int radix_sort_kv(swg_ctx *c, int64_t n, uint64_t *keys, uint32_t *vals, void *scratch, const int32_t *seg_of,
                  int seg_bits, bool host_skip) {
    if (n <= 1) return SWG_OK;
    if (n > 0xffffffffll || seg_bits < 0 || seg_bits > 8 * RS_MAX_SEG_PASSES || (seg_bits > 0 && !seg_of))
        return SWG_ERR_ARG;
    const int cols = rs_cols(n, c->num_sms);
    const int64_t tile = (int64_t)RS_THREADS * cols, ntiles = (n + tile - 1) / tile;
    const int nseg = seg_of ? (seg_bits + 7) / 8 : 0;
    const int npass = RS_KEY_PASSES + nseg;
    uint64_t *k2 = (uint64_t *)scratch;
    uint32_t *v2 = (uint32_t *)(k2 + n);
    unsigned *cnt = (unsigned *)(v2 + n);
    unsigned *hist = cnt + ntiles * RS_BINS;
    unsigned *tot = hist + RS_MAX_PASSES * RS_BINS;  // row totals of the current pass
    std::vector<unsigned> h;
    if (host_skip) {
        SWG_TRY(cuda_status(c, cudaMemsetAsync(hist, 0, sizeof(unsigned) * npass * RS_BINS, c->stream), "memset"));
        const int hblocks =
            (int)std::min<int64_t>((n + RS_THREADS - 1) / RS_THREADS, 2 * (int64_t)std::max(c->num_sms, 1));
        k_rs_hist_all<<<hblocks, RS_THREADS, 0, c->stream>>>(n, keys, vals, seg_of, npass, hist);
        c->launches++;
        SWG_TRY(launch_status(c, "radix_hist"));
        h.resize(npass * RS_BINS);
        SWG_TRY(cuda_status(c, cudaMemcpyAsync(h.data(), hist, sizeof(unsigned) * h.size(), cudaMemcpyDeviceToHost,
                                               c->stream),
                            "radix_hist"));
        SWG_TRY(cuda_status(c, cudaStreamSynchronize(c->stream), "radix_hist"));
    }
    uint64_t *kin = keys, *kout = k2;
    uint32_t *vin = vals, *vout = v2;
    for (int p = 0; p < npass; p++) {
        bool trivial = false;
        for (int d = 0; d < RS_BINS && host_skip; d++) trivial |= h[p * RS_BINS + d] == (unsigned)n;
        if (trivial) continue;  // every element has the same digit: the pass keeps the order
        k_rs_upsweep<<<(int)ntiles, RS_THREADS, 0, c->stream>>>(n, kin, vin, seg_of, p, cols, cnt);
        k_rs_scan_rows<<<RS_BINS, 1024, 0, c->stream>>>(ntiles, cnt, tot);
        k_rs_scatter<<<(int)ntiles, RS_THREADS, 0, c->stream>>>(n, kin, vin, seg_of, p, cols, cnt, tot, kout,
                                                                 vout);
        c->launches += 3;
        SWG_TRY(launch_status(c, "radix_pass"));
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
    if (kin != keys) {
        SWG_TRY(cuda_status(c, cudaMemcpyAsync(keys, kin, sizeof(uint64_t) * n, cudaMemcpyDeviceToDevice, c->stream),
                            "radix_copy"));
        SWG_TRY(cuda_status(c, cudaMemcpyAsync(vals, vin, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, c->stream),
                            "radix_copy"));
    }
    return SWG_OK;
}

}  // namespace swg
