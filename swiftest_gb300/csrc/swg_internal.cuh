// swg_internal.cuh -- shared declarations of the swiftest_gb300 CUDA library.
//
// All translation units are compiled with -fmad=false so that FP64 expressions
// keep the reference's rounding (no contraction into fused multiply-adds);
// kernels that want FMA (the mixed-precision kick) call fmaf() explicitly.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/swiftest_gb300.h"

namespace swg {

// Reference status codes, src/globals/globals_module.f90:86-101.
constexpr int ST_ACTIVE = 0;
constexpr int ST_INACTIVE = 1;
constexpr int ST_DISCARDED_DRIFTERR = -7;
constexpr int ST_COLLIDED = -14;

// Reference constants, src/globals/globals_module.f90:33-38.
constexpr double TWOPI = 6.283185307179586476925286766559005768394;
constexpr double PIBY2 = 1.570796326794896619231321691639751442099;
constexpr double PI3BY2 = 4.712388980384689857693965074919254326296;
constexpr double THIRD = 0.333333333333333333333333333333333333333;
constexpr double SIXTH = 0.166666666666666666666666666666666666667;
constexpr double VSMALL = 1.4916681462400413e-154;  // sqrt(tiny(1.0_DP))
constexpr double RSWEEP_FACTOR = 1.1;                // encounter_module.f90:21
constexpr double RSHELL = 0.48075;                   // symba_module.f90:23
constexpr int NTENC = 3;                             // symba_module.f90:21

// Grow-only device buffer.
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
};

// Encounter workspace: raw pair buffers, sort scratch and counters, grown on demand.
struct EncWork {
    DevBuf raw;      // i1, i2, lv raw (3 * rawcap int32)
    int64_t rawcap = 0;
    DevBuf sort;     // sort / sweep scratch
    DevBuf counters; // 2 x unsigned long long
};

// CUDA-event profile of a step loop by kernel class: begin() records the start event of
// a record on the stream and returns its index (-1 when off), end() its stop event;
// read() sums launches and milliseconds per class after a synchronization.
struct StepProfile {
    bool on = false;
    std::vector<cudaEvent_t> pool;  // events 2k, 2k+1 of record k
    std::vector<int> cls;           // class of record k
    size_t n = 0;
    int begin(cudaStream_t st, int c) {
        if (!on) return -1;
        const size_t k = n++;
        while (pool.size() < 2 * n) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return -1;
            pool.push_back(e);
        }
        if (cls.size() < n) cls.resize(n);
        cls[k] = c;
        cudaEventRecord(pool[2 * k], st);
        return (int)k;
    }
    void end(cudaStream_t st, int k) {
        if (k >= 0) cudaEventRecord(pool[2 * k + 1], st);
    }
    // out[2c] += launches, out[2c + 1] += ms for classes c < ncls; clears the records
    void read(double *out, int ncls) {
        for (int k = 0; k < 2 * ncls; k++) out[k] = 0.0;
        for (size_t k = 0; k < n; k++) {
            float ms = 0.f;
            if (cls[k] >= ncls || cudaEventElapsedTime(&ms, pool[2 * k], pool[2 * k + 1]) != cudaSuccess) continue;
            out[2 * cls[k]] += 1.0;
            out[2 * cls[k] + 1] += ms;
        }
        n = 0;
    }
    void release() {
        for (cudaEvent_t e : pool) cudaEventDestroy(e);
        pool.clear();
    }
};
// RAII record of one kernel class
struct ProfScope {
    StepProfile &p;
    cudaStream_t st;
    int k;
    ProfScope(StepProfile &p_, cudaStream_t st_, int c) : p(p_), st(st_), k(p_.begin(st_, c)) {}
    ~ProfScope() { p.end(st, k); }
};
// kernel classes of the step profiles
enum { PROF_KICK_PL = 0, PROF_KICK_TP = 1, PROF_DRIFT = 2, PROF_ENC0 = 3, PROF_RECUR = 4, PROF_NCLS = 5 };

}  // namespace swg

struct swg_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    int64_t launches = 0;
    int num_sms = 0;
    // scratch arena slots used by the flat C entry points (host-memory staging
    // and kernel scratch); each slot is grow-only.  Slot 10 holds the mixed kick's zeroed
    // block counters (ensure_kick_scratch) and must hold nothing else.
    swg::DevBuf slot[24];
    swg::EncWork enc;
    void *events[16] = {nullptr};  // measurement events (cudaEvent_t), created on first use
    std::vector<void *> systems;   // live swg_system objects, destroyed with the context
    std::vector<void *> ensembles; // live swg_ensemble objects, destroyed with the context
    void *sym_single = nullptr;    // cached plan of the one-system symmetric kick (kick_sym.cu)
};

namespace swg {

// Ensure buf holds at least `bytes` (grow-only); returns SWG_OK or SWG_ERR_NOMEM.
int ensure(swg_ctx *c, DevBuf &buf, size_t bytes);
// Records a CUDA error into the context; returns SWG_ERR_CUDA if e != success.
int cuda_status(swg_ctx *c, cudaError_t e, const char *what);
// Checks the last launch error.
int launch_status(swg_ctx *c, const char *what);
int ensure_slot(swg_ctx *c, int slot, size_t bytes, void **out);
// Mixed-kick scratch: a fixed block of zeroed "last block" counters followed by
// the partial sums; (re)allocation zeroes the counters.
constexpr size_t KICK_COUNTERS = 65536;
int ensure_kick_scratch(swg_ctx *c, DevBuf &buf, size_t bytes);

// ---------------------------------------------------------------- kernels API
// All pointers are device pointers; work is ordered on c->stream.

// kick.cu -- pair kick
enum KickMode { KICK_DIRECT = 0, KICK_SPLIT = 1 };
int kick_plpl_fp64(swg_ctx *c, int32_t npl, int32_t nplm, const double *r, const double *Gm, const double *R,
                   double *acc, int mode, int acc_is_zero);
int kick_tp_fp64(swg_ctx *c, int32_t ntp, int32_t npl, const double *rtp, const double *rpl, const double *Gm,
                 const int32_t *lmask, double *acc, int acc_is_zero);
size_t kick_mixed_scratch_bytes(int nrecv, int npart, int nchunk);
int kick_mixed_nchunk(int num_sms, int nrecv, int npart);
int kick_mixed_chunks(swg_ctx *c, int nrecv, int npart);
int kick_mixed_launch(swg_ctx *c, bool tp, int nrecv, int npart, int nplm, const double *rrecv, const double *rpart,
                      const double *Gm, const double *R, const int32_t *lmask, double *acc, int acc_is_zero,
                      int nchunk, void *scratch);
struct MixedPlplGrid {
    int bx, nchunk, chunk;
    int64_t partials;  // float-float partial entries written (6 floats each), 0 with one chunk
};
MixedPlplGrid kick_mixed_plpl_grid(int num_sms, int npl);
cudaError_t kick_mixed_plpl_on_stream(cudaStream_t stream, const MixedPlplGrid &g, int npl, int nplm,
                                      const double *r, const double *Gm, const double *R, double *acc, void *scratch,
                                      size_t counter_bytes);
// explicit 1-based pair list (k_plpl(2,n) or separate i1/i2); ahi_ahj: 6*npl doubles of scratch
// sign > 0: acc = (acc + ahi) + ahj ; sign < 0: acc = acc - (ahi + ahj)
int kick_pairs(swg_ctx *c, int32_t npl, int64_t npairs, const int32_t *k, const int32_t *i1, const int32_t *i2,
               const double *r, const double *Gm, const double *R, double *acc, double sign, double *ahi_ahj);

// Batched (ensemble) pair kernels.  Items are int4 (system, first receiver, receivers,
// unused) sorted by cost, largest first; per-system offsets and counts are device arrays.
// sys_flag/phase (optional, pl-pl): only systems s with sys_flag[s] == phase are processed.
// enc/enc_want (optional): split only the bodies j with enc[j] == enc_want.
int kick_split_launch(swg_ctx *c, int64_t n, const double *r, const double *Gm, const double *R, float4 *A,
                      float4 *B, const int32_t *sysid = nullptr, const int32_t *sys_flag = nullptr, int phase = 0,
                      const uint8_t *enc = nullptr, int enc_want = 0);
// variant: tile shape of the batched mixed kick (0 .. KICK_NVARIANT-1; identical results),
// whose items are tiles of kick_variant_tile(variant) receivers.
constexpr int KICK_NVARIANT = SWG_KICK_NVARIANT;
constexpr int KICK_SYMMETRIC = SWG_KICK_SYMMETRIC;  // the symmetric pl-pl kernel (kick_sym.cu)
int kick_variant_tile(int variant);
int kick_mixed_batched(swg_ctx *c, int variant, bool tp, bool rad, int nitems, const int4 *items,
                       const int32_t *roff, const int32_t *poff, const int32_t *npart, const double *rrecv,
                       const double *R, const float4 *pA, const float4 *pB, const int32_t *lmask, double *acc,
                       int acc_is_zero, unsigned *head, const int32_t *sys_flag = nullptr, int phase = 0,
                       const int32_t *nplm = nullptr);
int kick_plpl_fp64_batched(swg_ctx *c, bool rad, int nitems, const int4 *items, const int32_t *poff,
                           const int32_t *npl, const double *r, const double *Gm, const double *R, double *acc,
                           int acc_is_zero, const int32_t *sys_flag = nullptr, int phase = 0,
                           const int32_t *nplm = nullptr);
int kick_tp_fp64_batched(swg_ctx *c, int nitems, const int4 *items, const int32_t *toff, const int32_t *ntp,
                         const int32_t *poff, const int32_t *npl, const double *rtp, const double *rpl,
                         const double *Gm, const int32_t *lmask, double *acc, int acc_is_zero);
// orbel.cu -- orbital elements <-> Cartesian (swiftest_orbel_el2xv / _xv2el), device arrays;
// out_dev: a device array of 11 device pointers (a, e, inc, capom, omega, capm, varpi, lam, f,
// cape, capf), null entries skipped
int orbel_el2xv_launch(swg_ctx *c, int32_t n, const double *mu, const double *a, const double *e,
                       const double *inc, const double *capom, const double *omega, const double *capm, double *rh,
                       double *vh);
int orbel_xv2el_launch(swg_ctx *c, int32_t n, const double *mu, const double *rh, const double *vh,
                       double *const *out_dev);

// kick_sym.cu -- symmetric mixed pl-pl kick (each pair once, applied to both bodies) over
// tile pairs of `tile` bodies (KICK_SYM_TILE = 128 by default, or 64).  kick_sym_items builds
// the items (strips of tile pairs of a row group of `group` tiles, sorted by cost) and per
// system its first receiver slot and first pair slot (sbase[2s], sbase[2s+1]); returns the
// number of receiver slots, *npair_slots the number of pair slots.  A receiver slot holds
// 6 * tile floats, a pair slot 3 * tile; kick_mixed_sym_reduce writes acc (+)= the sums.  The
// same tile, strip and group must be passed to every call on one plan; groups of 2 or 4
// tiles take 128-body tiles.
constexpr int KICK_SYM_TILE = 128;
// strip: tiles J per item (4, or 1 when that would leave too few items to fill the GPU)
int kick_sym_strip(int32_t nsys, const int32_t *npl, int num_sms, int tile = KICK_SYM_TILE);
int64_t kick_sym_items(int32_t nsys, const int32_t *npl, int strip, std::vector<int4> &items,
                       std::vector<int32_t> &sbase, int64_t *npair_slots, int tile = KICK_SYM_TILE,
                       int group = 1);
// a single system has enough tile pairs to fill the GPU (else the broadcast kernel is faster)
bool kick_sym_single_ok(int32_t npl, int num_sms);
// iflag/accept (optional): only items it with bit iflag[it] of accept set are processed.
// warps: warps per block of one-row items (1, 2 or 4; the same bits for each; tiles of 64
// take one); with group 2 or 4 a block of `group` warps takes each row-group item.
int kick_mixed_sym_batched(swg_ctx *c, bool rad, int nitems, const int4 *items, const int32_t *poff,
                           const int32_t *npl, const int32_t *sbase, const float4 *pA, const float4 *pB, float *rpart,
                           float *ppart, unsigned *head, const int32_t *sys_flag = nullptr, int phase = 0,
                           const uint8_t *iflag = nullptr, unsigned accept = 0, int warps = 1,
                           int tile = KICK_SYM_TILE, int group = 1);
// iflag[it] of every item: 0 when its system has no encounter (sys_enc[s] == 0), else 2 when
// one of its tiles holds a body with enc[body] != 0, else 1.
int kick_sym_item_flags(swg_ctx *c, int nitems, const int4 *items, const int32_t *poff, const int32_t *npl,
                        const int32_t *sys_enc, const uint8_t *enc, uint8_t *iflag, int tile = KICK_SYM_TILE,
                        int group = 1);
// one system (psys == nullptr below): plan cached in the context for the last npl; acc (+)= the
// pair accelerations (radius rule with R, else j != i); no GMTINY bodies
int kick_mixed_sym_single(swg_ctx *c, int32_t npl, const double *r, const double *Gm, const double *R, double *acc,
                          int acc_is_zero);
void kick_sym_single_free(swg_ctx *c);
int kick_mixed_sym_reduce(swg_ctx *c, int strip, int64_t n, const int32_t *psys, const int32_t *poff,
                          const int32_t *npl, const int32_t *sbase, const float *rpart, const float *ppart,
                          double *acc, int acc_is_zero, const int32_t *sys_flag = nullptr, int phase = 0,
                          int tile = KICK_SYM_TILE, int group = 1);
// autotune.cu -- cache of tuned kernel shapes: key of (device, kind, size bucket); the cached
// variant or -1; store (kept for the process and appended to the cache file)
std::string tune_key(int device, const char *kind, int bucket);
int tune_lookup(const std::string &key);
void tune_store(const std::string &key, int variant);
// receivers per item of the batched kernels
constexpr int KICK_FP64_TILE = 8;
constexpr int ENC_TILE = 128;
constexpr int ENC_SORTED_TILE = 128;  // receivers per item of the radius-sorted pl-pl check
constexpr int ENC_BOUND_TILE = 64;    // bodies per bound tile of the radius-sorted check

// drift.cu -- Danby drift
int drift_all(swg_ctx *c, const double *mu, double mu_scalar, double *x, double *v, int32_t n, int32_t lgr,
              double inv_c2, double dt, const int32_t *lmask, int32_t *iflag);
// mu_sys/sys (optional): body i uses mu_sys[sys[i]] instead of mu (CSR-packed ensembles);
// fast: the fast FP64 form of the solver (mixed-precision path)
int drift_masked(swg_ctx *c, double mu, double *x, double *v, int32_t n, const int32_t *levelg, int irec, double dt,
                 int32_t *status, int32_t *nfail, const double *mu_sys = nullptr, const int32_t *sys = nullptr,
                 bool fast = false);

// encounter.cu -- encounter checks and sorting
int64_t sort_padded_len(int64_t n);
// Stable LSD radix sort of (key, val) by key (radix_sort.cu); with seg_of, the segment id
// seg_of[val] (seg_bits wide) is the most significant part of the key.  host_skip: read a
// digit histogram back to the host to skip constant digits (synchronizes the stream).
size_t radix_sort_scratch_bytes(int64_t n);
int radix_sort_kv(swg_ctx *c, int64_t n, uint64_t *keys, uint32_t *vals, void *scratch, const int32_t *seg_of,
                  int seg_bits, bool host_skip);
size_t util_sort_index_scratch_bytes(int64_t n);
int util_sort_index(swg_ctx *c, int64_t n, const double *arr, int32_t *ind, void *scratch);
// sort-and-sweep check (encounter.cu); scratch of sas_scratch_bytes(n1 + n2) (single: n1)
size_t sas_scratch_bytes(int ntot);
int sas_launch(swg_ctx *c, int n1, const double *r1, const double *v1, const double *renc1, int n2, const double *r2,
               const double *v2, const double *renc2, int single, int shift2, double dt, long long cap, int32_t *o1,
               int32_t *o2, int32_t *olv, unsigned long long *count, void *scratch, const int32_t *seg_of,
               int seg_bits, bool host_skip);
size_t sort_pairs_scratch_bytes(int64_t n);
int sort_pairs_unique(swg_ctx *c, int64_t n, int32_t *i1, int32_t *i2, int32_t *lv, void *scratch,
                      unsigned long long *d_nout);
size_t sas_scratch_bytes(int ntot);
// scratch one encounter_launch call needs (the `sas_scratch` argument, either mode)
size_t encounter_scratch_bytes(int mode, int n1, int n2);
int encounter_launch(swg_ctx *c, int mode, int n1, const double *r1, const double *v1, const double *renc1, int n2,
                     const double *r2, const double *v2, const double *renc2, int upper, int shift2, double dt,
                     long long cap, int32_t *o1, int32_t *o2, int32_t *olv, unsigned long long *count,
                     void *sas_scratch);

int encounter_prep_launch(swg_ctx *c, int64_t n, const double *r, const double *v, const double *renc, float4 *A,
                          float4 *B, float4 *V);
int encounter_tri_batched(swg_ctx *c, int nitems, const int4 *items, const int32_t *off1, const int32_t *n1,
                          const float4 *F1, int64_t nf1, const double *r1, const double *v1, const double *renc1,
                          const int32_t *off2, const int32_t *n2, const float4 *F2, int64_t nf2, const double *r2,
                          const double *v2, const double *renc2, int upper, double dt, long long cap, int32_t *o1,
                          int32_t *o2, int32_t *olv, unsigned long long *count);

// swiftest_discard_pl_tp close-approach scans (encounter.cu): flag[j] = 1 (flag zeroed by
// the caller) for each ACTIVE tp that comes within a pl's radius during the step.
int discard_pl_tp_launch(swg_ctx *c, int32_t npl, const double *rpl, const double *vpl, const double *radius,
                         int32_t ntp, const double *rtp, const double *vtp, const int32_t *tstatus, double dt,
                         float4 *F, int32_t *flag);
int discard_pl_tp_batched(swg_ctx *c, int nitems, const int4 *items, const int32_t *poff, const int32_t *npl,
                          int64_t NPL, const double *rpl, const double *vpl, const double *radius,
                          const int32_t *toff, const int32_t *ntp, int64_t NTP, const double *rtp, const double *vtp,
                          const int32_t *tstatus, double dt, float4 *F1, float4 *F2, int32_t *flag);

// Batched TRIANGULAR pl-pl check over radius-sorted tiles (encounter_sorted.cu): per
// system sort by |r| into perm, float copies F (3 * NPL float4, sorted order) and bound
// tiles (tiles[k] = (system, first sorted position), tbase[s] = system's first tile),
// then one block per item (system, first sorted receiver, receivers).  nmax: largest
// system.  Pairs are written with global 1-based indices, index1 < index2.
// resort: refresh the radial order (perm is kept between calls; any permutation gives the
// same list, the order only decides how many tile pairs are skipped).
int encounter_plpl_sorted_batched(swg_ctx *c, int nsys, int nmax, const int32_t *poff, const int32_t *npl,
                                  const double *r, const double *v, const double *renc, double dt, bool resort,
                                  int32_t *perm, float4 *F, int64_t NPL, int ntiles, const int2 *tiles,
                                  const int32_t *tbase, float4 *bounds, int nitems, const int4 *items, long long cap,
                                  int32_t *o1, int32_t *o2, int32_t *olv, unsigned long long *count,
                                  const int32_t *nplm = nullptr);

// One set of bodies (pl or tp) of CSR-packed systems ordered by |r| per system, for the
// radius-sorted checks: offsets and counts, positions, velocities, encounter radii (nullptr:
// zero), the order perm, float copies F (3 * N float4, sorted order), bound tiles
// (ENC_BOUND_TILE bodies: tiles[k] = (system, first sorted position), tbase[s] = the
// system's first tile) and the bounds of their 32-body halves (bounds[2 k + u], half u of
// tile k); nmax = the largest system.
struct SortedSet {
    const int32_t *off = nullptr, *n = nullptr;
    const double *r = nullptr, *v = nullptr, *renc = nullptr;
    int32_t *perm = nullptr;
    float4 *F = nullptr;
    int64_t N = 0;
    int ntiles = 0;
    const int2 *tiles = nullptr;
    const int32_t *tbase = nullptr;
    float4 *bounds = nullptr;
    int nmax = 0;
};
// resort: refresh the order; then the float copies and bounds from the current state
int sorted_set_prep(swg_ctx *c, const SortedSet &x, int nsys, bool resort, double dt);
// pl-tp over radius-sorted tiles (both sets prepared at the current state): the level-0
// pl-tp check (pairs (pl, tp), global 1-based, into o1/o2/olv/count) or, discard, the
// close-approach scan of swiftest_discard_pl_tp (flag[tp] = 1; tp renc = pl radius).
// Items: (system, first tp in sorted order, tp count <= ENC_SORTED_TILE, pl chunk); pchunk > 0:
// the item covers the pl sub-tiles (32 bodies) [chunk pchunk, (chunk + 1) pchunk), else all.
int pltp_sorted_batched(swg_ctx *c, bool discard, const SortedSet &pl, const SortedSet &tp, const int32_t *tstatus,
                        int nitems, const int4 *items, double dt, long long cap, int32_t *o1, int32_t *o2,
                        int32_t *olv, unsigned long long *count, int32_t *flag, int pchunk = 0);

// Full check of one kind (0 plpl, 1 plplm, 2 pltp): sorted unique pairs in the
// workspace's raw buffers; *n_out gets the count (host).  Synchronizes.
int encounter_check_kind(swg_ctx *c, EncWork &w, int kind, int mode, int32_t n1, const double *r1,
                         const double *v1, const double *renc1, int32_t n2, const double *r2, const double *v2,
                         const double *renc2, double dt, int64_t *n_out, int32_t **i1, int32_t **i2, int32_t **lv);

// collision.cu -- host-side resolution of detected collisions (perfect merging) for one
// system, on host copies of its arrays (local indices; lists hold 1-based local indices).
// Returns the number of collisions resolved.
struct CollisionSystem {
    int32_t npl = 0, ntp = 0;
    double GMcb = 0.0;
    double *rh = nullptr, *vb = nullptr, *Gm = nullptr, *R = nullptr, *rhill = nullptr;
    int32_t *status = nullptr, *lmask = nullptr;
    double *trh = nullptr, *tvb = nullptr;
    int32_t *tstatus = nullptr, *tlmask = nullptr;
    int64_t npp = 0, npt = 0;
    int32_t *pp_i1 = nullptr, *pp_i2 = nullptr, *pp_st = nullptr, *pp_lv = nullptr;
    int32_t *pt_i1 = nullptr, *pt_i2 = nullptr, *pt_st = nullptr;
    int32_t *levelg = nullptr;  // recursion levels of the massive bodies (for the cascade check)
    int irec = 0;               // recursion level at which the collisions were found
    double dt = 0.0;            // that level's step
    double E_collisions = 0.0;  // inout: collision_resolve.f90:638 (G*m units)
    double L_escape[3] = {0.0, 0.0, 0.0};  // inout: collision_generate.f90:219
    swg_ctx *dev = nullptr;     // context whose device forms the O(N^2) potential rows
};
// Step of recursion level irec, formed as the device recursion forms it: dt / 3^irec.
inline double level_dt(double dt, int irec) {
    double p3 = 1.0;
    for (int k = 0; k < irec; k++) p3 *= 3.0;
    return dt / p3;
}
// Resolves the COLLIDED pairs in place; returns the number of merges plus discarded test
// particles, -1 for a runaway collisional cascade, or -2 if the device work failed (the
// error is in c.dev->err).
int64_t resolve_collisions_host(CollisionSystem &c);

// Scalar-broadcast helpers
__host__ __device__ inline int64_t nplplm_count(int64_t npl, int64_t nplm) {
    return nplm * npl - nplm * (nplm + 1) / 2;
}

}  // namespace swg

#define SWG_TRY(expr)                 \
    do {                              \
        int _rc = (expr);             \
        if (_rc != SWG_OK) return _rc; \
    } while (0)
