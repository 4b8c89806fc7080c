// ensemble.cu -- batched ensembles of independent systems (HELIO and SyMBA).
//
// Many independent planetary systems of uneven size are packed CSR-style and step
// together: every kernel of a step covers all systems at once, so one launch
// sequence advances the whole ensemble.  The decomposition per kernel kind:
//   * per-body work (kick update, linear drift of tp, Danby drift, resets): flat
//     over all bodies, the body's system found through psys / tsys;
//   * the reference's O(N) ordered sums (vh2vb, vb2vh, linear drift momentum, the
//     energy totals) and the SyMBA recursion: one block per system;
//   * the pair kernels (kick, level-0 encounter check): a table of receiver tiles of
//     every system sorted by cost, largest first (kick.cu, kick_fp64.cu, encounter.cu),
//     the mixed kick as one persistent launch pulling tiles from a device queue;
//   * encounter-list kernels that the reference runs serially per system (pair
//     subtraction from the kick, the tp add-back): one thread per system.
// Each system takes exactly the steps of the single-system path (system.cu, which
// restates whm_step.f90 / helio_step.f90 / symba_step.f90), so in FP64 mode every
// system's trajectory is bit-identical to stepping it alone.
//
// HBM layout: system s owns massive bodies [poff[s], poff[s] + npl[s]) of the (3, NPL)
// FP64 arrays rh, vh, vb, ah, ... and test particles [toff[s], toff[s] + ntp[s]) of the
// (3, NTP) arrays; per-system scalars (GMcb, the central-body record dcb, first-step
// flags, encounter-list segments) are small device arrays indexed by s.  Encounter
// lists of all systems share one pool per kind with global 1-based body indices,
// sorted by (index1, index2), so system s's pairs form one contiguous segment.
// The systems share dt; GMTINY is not supported (every body fully interacting).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "drift_impl.cuh"
#include "swg_internal.cuh"
#include "symba_dev.cuh"

using namespace swg;
using namespace swg::sdev;

static_assert(KICK_FP64_TILE == 8 && ENC_TILE == 128, "tile sizes of the batched kernels");

// Arguments of the ensemble recursion kernel: the shared base plus per-system tables.
struct EnsRecArgs {
    RecArgs base;  // global arrays, list pools and scratch bases
    const int32_t *seg_pp, *seg_pt, *npl, *ntp;
    const double *GMcb;
    int32_t *resume, *pend;  // REC_STATE ints and one pause flag per system
};

struct swg_ensemble {
    swg_ctx *c = nullptr;
    int integrator = SWG_SYMBA;
    int32_t nsys = 0;
    int64_t NPL = 0, NTP = 0;
    std::vector<int32_t> h_npl, h_ntp, h_poff, h_toff;
    std::vector<double> h_GMcb, h_Rcb;
    double dt = 0, rhscale = 6.5, t = 0;
    int lclose = 0, precision = SWG_FP64, initialized = 0, cb_set = 0;
    // GMTINY (SyMBA): per system the count of fully interacting bodies (Gmass >= gmtiny,
    // bodies ordered by Gmass descending); tiny: some system has semi-interacting bodies
    double gmtiny = 0.0;
    int32_t *nplm = nullptr;
    bool tiny = false;
    // level-0 encounter checks (encounter_check_all_plpl / _pltp modes)
    int enc_plpl = SWG_ENC_TRIANGULAR, enc_pltp = SWG_ENC_TRIANGULAR;
    // sort-and-sweep: the system of every extent (pl-pl: 2 NPL; pl-tp: 2 (NPL + NTP)), built on first use
    int32_t *ext_pp = nullptr, *ext_pt = nullptr;
    DevBuf sas;  // extents, positions and the radix-sort scratch
    // per system (device)
    int32_t *npl = nullptr, *ntp = nullptr, *poff = nullptr, *toff = nullptr;
    double *GMcb = nullptr, *dcb = nullptr;  // dcb: CB_N doubles per system
    int32_t *lfirst = nullptr, *lany = nullptr, *seg_pp = nullptr, *seg_pt = nullptr, *enc_steps = nullptr;
    // massive bodies
    int32_t *psys = nullptr;
    double *rh = nullptr, *vh = nullptr, *vb = nullptr, *ah = nullptr, *rbeg = nullptr, *rend = nullptr;
    double *Gmass = nullptr, *radius = nullptr, *rhill = nullptr, *renc = nullptr;
    int32_t *status = nullptr, *lmask = nullptr, *levelg = nullptr, *levelm = nullptr, *nplenc = nullptr,
            *ntpenc = nullptr, *mark_pl = nullptr;
    // test particles
    int32_t *tsys = nullptr;
    double *trh = nullptr, *tvh = nullptr, *tvb = nullptr, *tah = nullptr;
    int32_t *tstatus = nullptr, *tlmask = nullptr, *tlevelg = nullptr, *tlevelm = nullptr, *tnplenc = nullptr,
            *mark_tp = nullptr;
    // float copies: split partners of the mixed kick (A|B), prefilter copies (A|B|V) of the
    // tp and the pl, both in radius order
    float4 *kA = nullptr, *kB = nullptr, *eT = nullptr, *eS = nullptr;
    // second split of the HELIO step's closing kick (kA2/kB2, used when kend is set), so the
    // tp kick at the step's start can still read kA/kB on the side stream
    float4 *kA2 = nullptr, *kB2 = nullptr;
    bool kend = false;
    // radius-sorted pl-pl check: order, bound tiles (system, first sorted position), the
    // systems' first tiles, bounds, receiver items
    int32_t *perm = nullptr, *tbase = nullptr;
    int2 *tiles = nullptr;
    float4 *bounds = nullptr;
    int4 *it_esp = nullptr;
    int ntiles = 0, n_esp = 0, nmax = 0;
    // radius-sorted pl-tp checks (level 0 and the discard scan): the tp order, tp bound tiles,
    // the systems' first tp tiles, bounds, tp receiver items; eT holds the tp float copies in
    // sorted order
    int32_t *tperm = nullptr, *ttbase = nullptr;
    int2 *ttiles = nullptr;
    float4 *tbounds = nullptr;
    int4 *it_tsp = nullptr;
    int nttiles = 0, n_tsp = 0, ntmax = 0;
    int64_t ndisc = 0;  // discard scans so far (HELIO/WHM refresh the orders every RESORT_EVERY)
    // level-0 checks: the state they read (the bodies' arrays, or the copy of them in snap,
    // which lets the checks run on the side stream while the first kick runs)
    const double *l0_r = nullptr, *l0_v = nullptr, *l0_tr = nullptr, *l0_tv = nullptr;
    double *snap = nullptr;  // SyMBA: rh | vb | trh | tvb at the start of the step
    // item tables of the batched pair kernels
    int4 *it_fpl = nullptr, *it_ftp = nullptr;
    int n_fpl = 0, n_ftp = 0;
    // mixed kick of kind k (0 pl-pl, 1 pl-tp): tile-shape variant (-1 until chosen by the
    // autotuner at the first such kick) and its items; force_variant >= 0 overrides the tuner
    int kv[2] = {-1, -1}, n_kit[2] = {0, 0};
    int4 *kit[2] = {nullptr, nullptr};
    int force_variant = -1;
    // symmetric pl-pl mixed kick (the default): tile-pair items, each system's first slot, slot sums
    int4 *it_sym = nullptr;
    int n_sym = 0, sym_strip = 1, sym_warps = 1, sym_tile = KICK_SYM_TILE, sym_group = 1;
    int force_strip = 0;  // > 0: strip length of the symmetric kick forced (0: tuned)
    int force_warps = 0;  // > 0: warps per block of the symmetric kick forced (0: tuned)
    int force_tile = 0;   // > 0: bodies per tile of the symmetric kick forced (0: tuned)
    int force_group = 0;  // > 0: tiles per row group of the symmetric kick forced (0: tuned)
    int32_t *sym_base = nullptr;
    float *sym_part = nullptr, *sym_ppart = nullptr;  // receiver slots, then pair slots (one allocation)
    unsigned *head = nullptr;
    // encounter lists: [i1 | i2 | lvdotr | status | level] * cap, global 1-based indices
    int32_t *pp_l = nullptr, *pt_l = nullptr;
    int64_t pp_n = 0, pt_n = 0, pp_cap = 0, pt_cap = 0;
    EncWork enc_pp, enc_pt;
    int32_t *rec_out = nullptr;  // [0] status, [1] deepest level, [2] sub-steps
    int32_t *rec_resume = nullptr, *rec_pend = nullptr;  // per system: paused recursion stack, pause flag
    int32_t *tflag = nullptr;                // tp flagged by the close-approach scan
    unsigned long long *ndiscard = nullptr;  // tp removed by the scan
    DevBuf rec_scratch, rows;
    DevBuf pair_terms;  // pl-pl pool: six pair terms and a kept flag per entry
    DevBuf close_part;  // mixed path: six per-chunk sums of the closing half-step (close_pl)
    // WHM: per-body eta / muj (whm_util_set_mu_eta_pl), Jacobi coordinates, ir3 terms, drift
    // flags, the per-system ah0 of the tp kick, first-step flag (host: all systems start together)
    double *eta = nullptr, *muj = nullptr, *xj = nullptr, *vj = nullptr, *ir3h = nullptr, *ir3j = nullptr,
           *whm_ah0 = nullptr;
    int32_t *iflag = nullptr, *whm_fail = nullptr;
    int whm_first = 1;
    // chunks of the mixed path's per-system sums: (system, first body, bodies, chunk index in
    // its system), each system's (first chunk, chunks), four partial sums per chunk
    int4 *chunks = nullptr;
    int2 *sys_chunks = nullptr;
    double *chunk_part = nullptr;
    int nchunks = 0;
    double *eout = nullptr;      // 9 per system
    int32_t *h_flags = nullptr;  // pinned: [2] recursion status; +8: two unsigned long long counts
    std::vector<int32_t> h_pend;  // per-system pause flags read after a recursion launch
    EnsRecArgs rec_args;          // arguments of the step's recursion launch (reused to resume)
    int64_t stats[6] = {0, 0, 0, 0, 0, 0};
    // per system: E_collisions, L_escape (x, y, z) booked by the collision resolution (G*m units)
    std::vector<double> coll_terms;
    double rec_dt = 0.0;  // step of the running recursion
    StepProfile prof;
    // side stream for the closing kick of systems without encounters (overlaps the recursion)
    cudaStream_t side = nullptr;
    // HELIO mixed step: the test particles in two groups of systems (tgroup 0/1; group 1's
    // bodies from tsplit on), each on its own stream (side, side2)
    cudaStream_t side2 = nullptr;
    cudaEvent_t ev_g0 = nullptr, ev_join2 = nullptr;
    int32_t *tgroup = nullptr;
    int64_t tsplit = 0;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_drift = nullptr, ev_split = nullptr;
    // SyMBA mixed closing kick: bodies in the encounter lists (enc_body) and per item of the
    // symmetric kick 0 / 1 / 2 = system without encounters / no listed body / a listed body
    uint8_t *enc_body = nullptr;
    DevBuf sym_iflag;
    bool drift_pending = false;   // the level-0 drift runs on the side stream (ev_drift)
    unsigned *head2 = nullptr;
    int64_t nchecks = 0;  // level-0 checks so far (the radial order is refreshed every RESORT_EVERY)
    // CUDA graph of one HELIO step (+ discard scan): captured after one eager step, replayed
    bool use_graph = true;
    int64_t eager_steps = 0, graph_launches = 0;
    cudaGraphExec_t graph = nullptr;
};

// level-0 checks between refreshes of the radial order of the pl-pl check
constexpr int RESORT_EVERY = 8;

namespace {

inline int grid_for(int64_t n, int bs) { return (int)std::max<int64_t>(1, (n + bs - 1) / bs); }

int L(swg_ctx *c, const char *what) {
    c->launches++;
    return launch_status(c, what);
}

template <typename T>
int dalloc(swg_ctx *c, T **p, size_t n) {
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
    if (e != cudaSuccess) {
        c->err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
        return SWG_ERR_NOMEM;
    }
    return cuda_status(c, cudaMemsetAsync(*p, 0, n * sizeof(T), c->stream), "memset");
}

template <typename T>
int upload(swg_ctx *c, T *dst, const std::vector<T> &src) {
    if (src.empty()) return SWG_OK;
    return cuda_status(c, cudaMemcpyAsync(dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice, c->stream),
                       "upload");
}

// ---------------------------------------------------------------- kernels
// threads per system of the per-system sums: a system has a few thousand bodies at most
// and several systems share an SM, so small blocks keep the reduction trees short
constexpr int ENS_SUM_T = 256;

// one block per system: swiftest_util_coord_vh2vb_pl (only systems whose first-step
// flag is set when lfirst != nullptr), helio_drift_linear_pl, swiftest_util_coord_vb2vh_pl
__global__ void __launch_bounds__(ENS_SUM_T) k_ens_vh2vb(const int32_t *__restrict__ poff, const int32_t *__restrict__ npl,
                                                  const int32_t *__restrict__ lfirst, const double *__restrict__ Gm,
                                                  const double *__restrict__ vh, double *vb,
                                                  const double *__restrict__ GMcb, double *dcb, int exact) {
    const int s = blockIdx.x;
    if (npl[s] == 0 || (lfirst && !lfirst[s])) return;
    __shared__ SumScratch sh;
    const size_t o = poff[s];
    blk_vh2vb_pl(npl[s], Gm + o, vh + 3 * o, vb + 3 * o, GMcb[s], dcb + CB_N * s, exact, sh);
}
__global__ void __launch_bounds__(ENS_SUM_T) k_ens_lindrift(const int32_t *__restrict__ poff, const int32_t *__restrict__ npl,
                                                     const double *__restrict__ Gm, const double *__restrict__ vb,
                                                     const int32_t *__restrict__ lmask, const double *__restrict__ GMcb,
                                                     double *rh, double dt, double *dcb, int slot, int exact) {
    const int s = blockIdx.x;
    if (npl[s] == 0) return;
    __shared__ SumScratch sh;
    const size_t o = poff[s];
    blk_lindrift_pl(npl[s], Gm + o, vb + 3 * o, lmask + o, GMcb[s], rh + 3 * o, dt, dcb + CB_N * s, slot, exact, sh);
}
__global__ void __launch_bounds__(ENS_SUM_T) k_ens_vb2vh(const int32_t *__restrict__ poff, const int32_t *__restrict__ npl,
                                                  const double *__restrict__ Gm, const double *__restrict__ vb,
                                                  const int32_t *__restrict__ status, double *vh,
                                                  const double *__restrict__ GMcb, double *dcb, int exact) {
    const int s = blockIdx.x;
    if (npl[s] == 0) return;
    __shared__ SumScratch sh;
    const size_t o = poff[s];
    blk_vb2vh_pl(npl[s], Gm + o, vb + 3 * o, status + o, vh + 3 * o, GMcb[s], dcb + CB_N * s, exact, sh);
}

// Test-particle coordinate updates with their own system's central-body record (modes
// as k_tp_misc of system.cu: 2 linear drift, 3 linear drift then vb2vh, 4 vh2vb then
// linear drift, 5 vb = vh + the central body's vb).  mode_first >= 0 replaces mode
// for systems still in their first step.
__global__ void k_ens_tp_misc(int64_t ntp, const int32_t *__restrict__ tsys, const int32_t *__restrict__ tlmask,
                              double *trh, double *tvh, double *tvb, const double *__restrict__ dcb, int slot,
                              double dt, int mode, int mode_first, const int32_t *__restrict__ lfirst) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= ntp || !tlmask[i]) return;
    const int s = tsys[i];
    const int m = (mode_first >= 0 && lfirst[s]) ? mode_first : mode;
    const double *cb = dcb + CB_N * s;
    for (int d = 0; d < 3; d++) {
        const double pt = cb[slot + d];
        const double vbcb = -pt;
        if (m == 4) tvb[3 * i + d] = tvh[3 * i + d] + vbcb;
        if (m == 2 || m == 3 || m == 4) trh[3 * i + d] = trh[3 * i + d] + pt * dt;
        if (m == 3) tvh[3 * i + d] = tvb[3 * i + d] - vbcb;
        if (m == 5) tvb[3 * i + d] = tvh[3 * i + d] + cb[slot + d];
    }
}

// Segment (first entry, count) of each system in an encounter-list pool sorted by index1
// (global 1-based pl index): binary searches for the system's pl range, so a system
// without pairs still gets the position where its pairs would start (the recursion
// places its scratch by these positions).
__device__ __forceinline__ int64_t lower_bound_i32(const int32_t *__restrict__ a, int64_t n, int32_t v) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (a[mid] < v)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}
__global__ void k_ens_segments(int nsys, int64_t n, const int32_t *__restrict__ i1, const int32_t *__restrict__ poff,
                               int32_t *seg) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsys) return;
    const int64_t b = lower_bound_i32(i1, n, poff[s] + 1), e = lower_bound_i32(i1, n, poff[s + 1] + 1);
    seg[2 * s] = (int32_t)b;
    seg[2 * s + 1] = (int32_t)(e - b);
}

// symba_kick_getacch_pl's subtraction of the encountering pairs (symba_kick.f90:61-70)
// through the flat pair loop (swiftest_kick.f90:69-115), one thread per system walking
// its list segment in order: ahi/ahj of the listed bodies, then acc -= ahi + ahj once
// per body (unlisted bodies would subtract zero).
// Terms of symba_kick_getacch_pl's pair subtraction for every entry of the pl-pl pool, one
// thread each: t = (Gm_j irij3 dx, Gm_i irij3 dx), ok = the pair passes the radius rule.
// The square root and divide of each pair run here in parallel; k_ens_kick_pairs adds the
// terms in list order.
__global__ void k_ens_pair_terms(int64_t n, const int32_t *__restrict__ l, int64_t cap, const double *__restrict__ r,
                                 const double *__restrict__ Gm, const double *__restrict__ R, double *t,
                                 uint8_t *ok) {
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= n) return;
    const int i = l[q] - 1, j = l[cap + q] - 1;
    const double rx = r[3 * j + 0] - r[3 * i + 0];
    const double ry = r[3 * j + 1] - r[3 * i + 1];
    const double rz = r[3 * j + 2] - r[3 * i + 2];
    const double rji2 = rx * rx + ry * ry + rz * rz;
    const double rs = R[i] + R[j];
    if (!(rji2 > rs * rs)) {
        ok[q] = 0;
        return;
    }
    const double irij3 = 1.0 / (rji2 * sqrt(rji2));
    const double faci = Gm[i] * irij3;
    const double facj = Gm[j] * irij3;
    double *o = t + 6 * q;
    o[0] = facj * rx;
    o[1] = facj * ry;
    o[2] = facj * rz;
    o[3] = faci * rx;
    o[4] = faci * ry;
    o[5] = faci * rz;
    ok[q] = 1;
}

// symba_kick_getacch_pl (symba_kick.f90:36-76) pair subtraction of every system: per body,
// the pair terms of the pairs naming it as index1 (ahi) and as index2 (ahj) added in list
// order (swiftest_kick_getacch_int_all_flat order), then acc -= ahi + ahj once per body.
// One warp per system: a body's sums are formed by the lane that holds its first occurrence
// in the order (pair 0 index1, pair 0 index2, pair 1 index1, ...).
__global__ void k_ens_kick_pairs_warp(int nsys, const int32_t *__restrict__ seg, const int32_t *__restrict__ l,
                                      int64_t cap, const double *__restrict__ t, const uint8_t *__restrict__ ok,
                                      double *acc) {
    const int s = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (s >= nsys || seg[2 * s + 1] == 0) return;
    const int n = seg[2 * s + 1];
    const int32_t *i1 = l + seg[2 * s], *i2 = i1 + cap;
    const double *ts = t + 6 * (int64_t)seg[2 * s];
    const uint8_t *oks = ok + seg[2 * s];
    for (int occ = lane; occ < 2 * n; occ += 32) {
        const int q = occ >> 1;
        const int b = ((occ & 1) ? i2[q] : i1[q]) - 1;
        bool first = true;
        for (int o = 0; o < occ && first; o++) first = (((o & 1) ? i2[o >> 1] : i1[o >> 1]) - 1) != b;
        if (!first) continue;
        double hx = 0.0, hy = 0.0, hz = 0.0, jx = 0.0, jy = 0.0, jz = 0.0;
        for (int p = 0; p < n; p++) {
            if (!oks[p]) continue;
            const double *o = ts + 6 * p;
            if (i1[p] - 1 == b) {
                hx = hx + o[0];
                hy = hy + o[1];
                hz = hz + o[2];
            }
            if (i2[p] - 1 == b) {
                jx = jx - o[3];
                jy = jy - o[4];
                jz = jz - o[5];
            }
        }
        acc[3 * b + 0] = acc[3 * b + 0] - (hx + jx);
        acc[3 * b + 1] = acc[3 * b + 1] - (hy + jy);
        acc[3 * b + 2] = acc[3 * b + 2] - (hz + jz);
    }
}

// symba_kick_getacch_tp add-back loop (symba_kick.f90:104-118) of every system
__global__ void k_ens_pltp_addback(int nsys, const int32_t *__restrict__ seg, const int32_t *__restrict__ l,
                                   int64_t cap, const int32_t *__restrict__ tlmask, const double *__restrict__ trh,
                                   const double *__restrict__ rp, const double *__restrict__ Gm, double *tah) {
    // one warp per system; each test particle's pairs are added, in list order, by the lane
    // that holds its first pair (particles in parallel, the reference's order per particle)
    const int s = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (s >= nsys || seg[2 * s + 1] == 0) return;
    const int n = seg[2 * s + 1];
    const int32_t *i1 = l + seg[2 * s], *i2 = i1 + cap;
    for (int k = lane; k < n; k += 32) {
        const int j = i2[k] - 1;
        if (!tlmask[j]) continue;
        bool first = true;
        for (int p = 0; p < k && first; p++) first = i2[p] - 1 != j;
        if (!first) continue;
        double x = tah[3 * j + 0], y = tah[3 * j + 1], z = tah[3 * j + 2];
        for (int p = k; p < n; p++) {
            if (i2[p] - 1 != j) continue;
            const int i = i1[p] - 1;
            const double dx = trh[3 * j + 0] - rp[3 * i + 0];
            const double dy = trh[3 * j + 1] - rp[3 * i + 1];
            const double dz = trh[3 * j + 2] - rp[3 * i + 2];
            const double rjj = dx * dx + dy * dy + dz * dz;
            const double fac = Gm[i] / (rjj * sqrt(rjj));
            x = x + fac * dx;
            y = y + fac * dy;
            z = z + fac * dz;
        }
        tah[3 * j + 0] = x;
        tah[3 * j + 1] = y;
        tah[3 * j + 2] = z;
    }
}

// End of step: a system that took the plain HELIO step clears its first-step flag
// (helio_step.f90), one that interpolated keeps it (symba_step_interp_system never
// clears lfirst); count the steps with encounters.  lany == nullptr: HELIO ensemble.
__global__ void k_ens_finish(int nsys, const int32_t *__restrict__ lany, int32_t *lfirst, int32_t *enc_steps) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsys) return;
    const int any = lany ? lany[s] : 0;
    if (!any) lfirst[s] = 0;
    enc_steps[s] += any;
}
__global__ void k_ens_lany(int nsys, const int32_t *__restrict__ seg_pp, const int32_t *__restrict__ seg_pt,
                           int32_t *lany) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < nsys) lany[s] = (seg_pp[2 * s + 1] + seg_pt[2 * s + 1]) > 0;
}

// enc[i] = 1 for a body in this step's encounter lists (levelg >= 0), else 0
__global__ void k_mark_enc(int64_t n, const int32_t *__restrict__ levelg, uint8_t *__restrict__ enc) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) enc[i] = levelg[i] >= 0 ? 1 : 0;
}

// The SyMBA recursion of every system with encounters this step, one block each
// (blk_symba_recursion on the system's list segments; body arrays are global).
__global__ void __launch_bounds__(RECT) k_ens_symba_recursion(EnsRecArgs e, int resume_only) {
    const int s = blockIdx.x;
    const int64_t k0 = e.seg_pp[2 * s], npp = e.seg_pp[2 * s + 1];
    const int64_t t0 = e.seg_pt[2 * s], npt = e.seg_pt[2 * s + 1];
    if (npp + npt == 0) return;
    if (resume_only && e.resume[(size_t)REC_STATE * s] == 0) return;  // finished before the pause
    RecArgs a = e.base;
    a.npl = e.npl[s];
    a.ntp = e.ntp[s];
    a.npp = npp;
    a.npt = npt;
    a.pp = e.base.pp + k0;
    a.pt = e.base.pt + t0;
    a.GMcb = e.GMcb[s];
    const int64_t q = k0 + t0;  // entries of the systems before s
    a.terms = e.base.terms + 12 * q;
    a.lenc = e.base.lenc + q;
    a.good = e.base.good + q;
    a.good2 = e.base.good2 + q;
    a.bpl = e.base.bpl + 2 * k0 + t0;
    a.btp = e.base.btp + t0;
    a.adj_end = e.base.adj_end + 2 * (k0 + t0);  // bpl and btp slots
    a.adj = e.base.adj + 2 * k0 + t0;
    a.resume = e.resume + (size_t)REC_STATE * s;
    a.pend = e.pend + s;
    blk_symba_recursion(a);
}

// ---- WHM (whm_step.f90, whm_kick.f90, whm_coord.f90) of every system: one block per system
// for the Jacobi running sums (FP64 path: one thread, in the reference's order)
enum { WHM_H2J = 0, WHM_J2H = 1, WHM_VH2VJ = 2 };
__global__ void k_ens_whm_coord(int mode, const int32_t *__restrict__ poff, const int32_t *__restrict__ npl,
                                const double *Gm, const double *eta, double *rh, double *vh, double *xj, double *vj,
                                int exact) {
    const int s = blockIdx.x;
    if (npl[s] == 0) return;
    __shared__ WhmScratch sh;
    const size_t o = poff[s];
    if (mode == WHM_H2J)
        blk_whm_h2j(npl[s], Gm + o, eta + o, rh + 3 * o, vh + 3 * o, xj + 3 * o, vj + 3 * o, sh, exact);
    else if (mode == WHM_J2H)
        blk_whm_j2h(npl[s], Gm + o, eta + o, xj + 3 * o, vj + 3 * o, rh + 3 * o, vh + 3 * o, sh, exact);
    else
        blk_whm_vh2vj(npl[s], Gm + o, eta + o, vh + 3 * o, vj + 3 * o, sh, exact);
}
__global__ void k_ens_whm_accel(const int32_t *__restrict__ poff, const int32_t *__restrict__ npl, const double *Gm,
                                const double *__restrict__ GMcb, const double *rh, const double *xj,
                                const int32_t *lmask, double *ir3h, double *ir3j, double *ah, int exact) {
    const int s = blockIdx.x;
    if (npl[s] == 0) return;
    __shared__ WhmScratch sh;
    const size_t o = poff[s];
    blk_whm_accel_pl(npl[s], Gm + o, GMcb[s], rh + 3 * o, xj + 3 * o, lmask + o, ir3h + o, ir3j + o, ah + 3 * o, sh,
                     exact);
}
// ah0 of whm_kick_getacch_tp (whm_kick.f90:70-122) per system at the pl positions rp
__global__ void k_ens_whm_ah0(const int32_t *__restrict__ poff, const int32_t *__restrict__ npl, const double *Gm,
                              const double *rp, double *ah0, int exact) {
    const int s = blockIdx.x;
    __shared__ WhmScratch sh;
    const size_t o = poff[s];
    blk_whm_ah0(Gm + o, rp + 3 * o, npl[s], ah0 + 3 * s, sh, exact);
}
// tah = ah0 of the test particle's system (masked), before the pair kick adds to it
__global__ void k_ens_whm_tp_ah0(int64_t ntp, const int32_t *__restrict__ tsys, const int32_t *__restrict__ tlmask,
                                 const double *__restrict__ ah0, double *tah) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= ntp || !tlmask[i]) return;
    const double *a = ah0 + 3 * tsys[i];
    for (int d = 0; d < 3; d++) tah[3 * i + d] = 0.0 + a[d];
}
// whm_drift_pl's failure handling (whm_drift.f90:14-58): status, mask and a run-wide flag
__global__ void k_ens_whm_drift_status(int64_t n, const int32_t *__restrict__ iflag, int32_t *status, int32_t *lmask,
                                       int32_t *fail) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n && iflag[i] != 0) {
        status[i] = ST_DISCARDED_DRIFTERR;
        lmask[i] = 0;
        atomicOr(fail, 1);
    }
}

// energy / momentum per system: totals (one block each) and potential rows (flat)
__global__ void __launch_bounds__(RB) k_ens_energy_final(const int32_t *__restrict__ poff,
                                                         const int32_t *__restrict__ npl, const double *rh,
                                                         const double *vh, const double *vb, const double *Gm,
                                                         const double *radius, const int32_t *status,
                                                         const double *__restrict__ GMcb, int lclose, int whm,
                                                         const double *rows, double *rb, double *out) {
    const int s = blockIdx.x;
    __shared__ SumScratch sh;
    const size_t o = poff[s];
    blk_energy_final(npl[s], whm, rh + 3 * o, vh + 3 * o, vb + 3 * o, Gm + o, radius + o, status + o, GMcb[s], lclose,
                     rows + o, rb + 3 * o, out + 9 * s, sh);
}
__global__ void k_ens_energy_rows(int64_t n, const int32_t *__restrict__ psys, const int32_t *__restrict__ poff,
                                  const int32_t *__restrict__ npl, const double *rb, const double *Gm,
                                  const int32_t *status, double *rows) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int s = psys[i];
    const size_t o = poff[s];
    rows[i] = d_energy_row((int)(i - o), npl[s], rb + 3 * o, Gm + o, status + o);
}

// ---------------------------------------------------------------- host side
bool exact(const swg_ensemble *e) { return e->precision == SWG_FP64; }

// Tiles of every system, sorted by cost (largest first; ties keep system order).
// recv(s) receivers per system in tiles of `tile`; cost(s, r0, nr) orders them.
template <class Recv, class Cost>
std::vector<int4> make_items(int nsys, int tile, Recv recv, Cost cost) {
    std::vector<int4> it;
    std::vector<double> w;
    for (int s = 0; s < nsys; s++) {
        const int n = recv(s);
        for (int r0 = 0; r0 < n; r0 += tile) {
            const int nr = std::min(tile, n - r0);
            it.push_back(make_int4(s, r0, nr, 0));
            w.push_back(cost(s, r0, nr));
        }
    }
    std::vector<size_t> ord(it.size());
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](size_t a, size_t b) { return w[a] > w[b]; });
    std::vector<int4> out(it.size());
    for (size_t k = 0; k < ord.size(); k++) out[k] = it[ord[k]];
    return out;
}

int put_items(swg_ensemble *e, int4 **dst, int *n, const std::vector<int4> &items) {
    if (*dst) cudaFree(*dst);
    *dst = nullptr;
    *n = (int)items.size();
    SWG_TRY(dalloc(e->c, dst, items.size()));
    return upload(e->c, *dst, items);
}

int build_items(swg_ensemble *e) {
    const int S = e->nsys;
    auto npl = [&](int s) { return e->h_npl[s]; };
    auto ntp = [&](int s) { return e->h_ntp[s]; };
    auto plcost = [&](int s, int, int nr) { return (double)nr * e->h_npl[s]; };
    SWG_TRY(put_items(e, &e->it_fpl, &e->n_fpl, make_items(S, KICK_FP64_TILE, npl, plcost)));
    SWG_TRY(put_items(e, &e->it_ftp, &e->n_ftp, make_items(S, KICK_FP64_TILE, ntp, plcost)));
    auto tp_with_pl = [&](int s) { return e->h_npl[s] > 0 ? e->h_ntp[s] : 0; };
    SWG_TRY(put_items(e, &e->it_tsp, &e->n_tsp, make_items(S, ENC_SORTED_TILE, tp_with_pl, plcost)));
    {  // tp bound tiles of the sorted pl-tp checks
        std::vector<int2> tt;
        std::vector<int32_t> tb(S + 1, 0);
        for (int s = 0; s < S; s++) {
            tb[s] = (int32_t)tt.size();
            for (int p0 = 0; p0 < e->h_ntp[s]; p0 += ENC_BOUND_TILE) tt.push_back(make_int2(s, p0));
            e->ntmax = std::max(e->ntmax, (int)e->h_ntp[s]);
        }
        tb[S] = (int32_t)tt.size();
        e->nttiles = (int)tt.size();
        SWG_TRY(dalloc(e->c, &e->ttiles, tt.size()));
        SWG_TRY(upload(e->c, e->ttiles, tt));
        SWG_TRY(dalloc(e->c, &e->ttbase, tb.size()));
        SWG_TRY(upload(e->c, e->ttbase, tb));
        SWG_TRY(dalloc(e->c, &e->tbounds, 2 * tt.size()));  // bounds of each tile's two 32-body halves
    }
    // radius-sorted pl-pl check: receiver tiles in system order (their cost depends on
    // the geometry), bound tiles of every system
    SWG_TRY(put_items(e, &e->it_esp, &e->n_esp, make_items(S, ENC_SORTED_TILE, npl, [](int, int, int) { return 0.0; })));
    std::vector<int2> tiles;
    std::vector<int32_t> tbase(S + 1, 0);
    for (int s = 0; s < S; s++) {
        tbase[s] = (int32_t)tiles.size();
        for (int p0 = 0; p0 < e->h_npl[s]; p0 += ENC_BOUND_TILE) tiles.push_back(make_int2(s, p0));
        e->nmax = std::max(e->nmax, (int)e->h_npl[s]);
    }
    tbase[S] = (int32_t)tiles.size();
    e->ntiles = (int)tiles.size();
    SWG_TRY(dalloc(e->c, &e->tiles, tiles.size()));
    SWG_TRY(upload(e->c, e->tiles, tiles));
    SWG_TRY(dalloc(e->c, &e->tbase, tbase.size()));
    SWG_TRY(upload(e->c, e->tbase, tbase));
    SWG_TRY(dalloc(e->c, &e->bounds, 2 * tiles.size()));  // bounds of each tile's two 32-body halves
    std::vector<int4> chunks;
    std::vector<int2> sys_chunks(S);
    for (int s = 0; s < S; s++) {
        sys_chunks[s] = make_int2((int)chunks.size(), 0);
        for (int b0 = 0, k = 0; b0 < e->h_npl[s]; b0 += CHUNK, k++)
            chunks.push_back(make_int4(s, e->h_poff[s] + b0, std::min(CHUNK, e->h_npl[s] - b0), k));
        sys_chunks[s].y = (int)chunks.size() - sys_chunks[s].x;
    }
    e->nchunks = (int)chunks.size();
    SWG_TRY(dalloc(e->c, &e->chunks, chunks.size()));
    SWG_TRY(upload(e->c, e->chunks, chunks));
    SWG_TRY(dalloc(e->c, &e->sys_chunks, sys_chunks.size()));
    SWG_TRY(upload(e->c, e->sys_chunks, sys_chunks));
    return dalloc(e->c, &e->chunk_part, 4 * chunks.size());
}

int ensure_pool(swg_ensemble *e, int32_t **l, int64_t *cap, int64_t need) {
    if (need <= *cap) return SWG_OK;
    const int64_t ncap = std::max<int64_t>(need + need / 2, 1024);
    int32_t *fresh = nullptr;
    SWG_TRY(dalloc(e->c, &fresh, (size_t)5 * ncap));
    if (*l) cudaFree(*l);
    *l = fresh;
    *cap = ncap;
    return SWG_OK;
}

// ------------------------------------------------ mixed kick: tile shape chosen by timing
// Receiver tiles of the mixed kick of kind k (0 pl-pl, 1 pl-tp) for tiles of `tile`.
std::vector<int4> kick_items(const swg_ensemble *e, int k, int tile) {
    auto recv = [&](int s) { return k == 0 ? e->h_npl[s] : e->h_ntp[s]; };
    auto cost = [&](int s, int, int nr) { return (double)nr * e->h_npl[s]; };
    return make_items(e->nsys, tile, recv, cost);
}

// Size bucket of the tuning key: floor(log2) of the mean receivers per system.
int size_bucket(const swg_ensemble *e, int k) {
    int b = 0;
    for (double m = (double)(k == 0 ? e->NPL : e->NTP) / std::max(1, e->nsys); m >= 2.0; m *= 0.5) b++;
    return b;
}

// One mixed kick of kind k with the given shape and items into acc (overwritten); the
// partners must be split into kA/kB.
int mixed_kick(swg_ensemble *e, int k, int variant, const int4 *items, int nitems, double *acc, bool rad,
               unsigned *head, const int32_t *flag, int phase, int acc_is_zero = 1) {
    const float4 *pa = e->kend ? e->kA2 : e->kA, *pb = e->kend ? e->kB2 : e->kB;
    if (k == 0)
        return kick_mixed_batched(e->c, variant, false, rad, nitems, items, e->poff, e->poff, e->npl, e->rh,
                                  rad ? e->radius : nullptr, pa, pb, nullptr, acc, acc_is_zero, head, flag, phase,
                                  e->tiny ? e->nplm : nullptr);
    return kick_mixed_batched(e->c, variant, true, false, nitems, items, e->toff, e->poff, e->npl, e->trh, nullptr,
                              pa, pb, e->tlmask, acc, acc_is_zero, head, flag, phase);
}

// Scratch of the timing runs, released on every exit path.
struct TuneScratch {
    double *acc = nullptr;
    int4 *items = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    ~TuneScratch() {
        if (acc) cudaFree(acc);
        if (items) cudaFree(items);
        for (cudaEvent_t x : ev)
            if (x) cudaEventDestroy(x);
    }
};

// Times every tile shape of the mixed kick of kind k on this ensemble's current data (one
// warm-up and three timed launches each, into scratch accelerations) and returns the
// fastest.  All shapes give identical results, so only the time differs.
int time_kick_variants(swg_ensemble *e, int k, bool rad, unsigned *head, const int32_t *flag, int phase, int *best) {
    swg_ctx *c = e->c;
    TuneScratch t;
    SWG_TRY(dalloc(c, &t.acc, 3 * (size_t)(k == 0 ? e->NPL : e->NTP)));
    for (cudaEvent_t &x : t.ev) SWG_TRY(cuda_status(c, cudaEventCreate(&x), "event"));
    float best_ms = 0.f;
    *best = 0;
    for (int v = 0; v < KICK_NVARIANT; v++) {
        const std::vector<int4> items = kick_items(e, k, kick_variant_tile(v));
        if (t.items) cudaFree(t.items);
        t.items = nullptr;
        SWG_TRY(dalloc(c, &t.items, items.size()));
        SWG_TRY(upload(c, t.items, items));
        const int n = (int)items.size();
        SWG_TRY(mixed_kick(e, k, v, t.items, n, t.acc, rad, head, flag, phase));
        SWG_TRY(cuda_status(c, cudaEventRecord(t.ev[0], c->stream), "event"));
        for (int rep = 0; rep < 3; rep++) SWG_TRY(mixed_kick(e, k, v, t.items, n, t.acc, rad, head, flag, phase));
        SWG_TRY(cuda_status(c, cudaEventRecord(t.ev[1], c->stream), "event"));
        SWG_TRY(cuda_status(c, cudaEventSynchronize(t.ev[1]), "event"));
        float ms = 0.f;
        SWG_TRY(cuda_status(c, cudaEventElapsedTime(&ms, t.ev[0], t.ev[1]), "event"));
        if (v == 0 || ms < best_ms) {
            best_ms = ms;
            *best = v;
        }
    }
    return SWG_OK;
}

// The symmetric pl-pl kick's plan for strips of `strip` tiles J against row groups of
// e->sym_group tiles of e->sym_tile bodies: items, per-system slot bases and the receiver
// and pair slots (replacing any previous plan).
int build_sym_plan(swg_ensemble *e, int strip) {
    swg_ctx *c = e->c;
    std::vector<int4> items;
    std::vector<int32_t> base;
    int64_t npair = 0;
    const int64_t nrecv =
        kick_sym_items(e->nsys, e->h_npl.data(), strip, items, base, &npair, e->sym_tile, e->sym_group);
    SWG_TRY(put_items(e, &e->it_sym, &e->n_sym, items));
    if (e->sym_base) cudaFree(e->sym_base);
    if (e->sym_part) cudaFree(e->sym_part);
    e->sym_base = nullptr;
    e->sym_part = nullptr;
    SWG_TRY(dalloc(c, &e->sym_base, base.size()));
    SWG_TRY(upload(c, e->sym_base, base));
    SWG_TRY(dalloc(c, &e->sym_part, (size_t)(6 * nrecv + 3 * npair) * e->sym_tile));
    e->sym_ppart = e->sym_part + (size_t)nrecv * 6 * e->sym_tile;
    e->sym_strip = strip;
    return SWG_OK;
}

// Strip lengths (tile pairs per work item) the autotuner tries for the symmetric kick.  The
// strip decides how each body's receiver sums are split into slots, so unlike the
// broadcast shapes the strips add the same terms in different groupings: results agree
// within the mixed-kick tolerance, and each strip is deterministic.
constexpr int SYM_STRIPS[] = {1, 2, 4, 8, 16};
constexpr int SYM_NSTRIP = 5;

// Warps per block the autotuner tries for the symmetric kick (each warp is an independent
// worker, so every count gives the same bits).
constexpr int SYM_WARPS[] = {1, 2, 4};
constexpr int SYM_NWARPS = 3;

// Row groups (tiles per item row, one warp each) and their strips the autotuner tries for
// the symmetric kick with 128-body tiles.  A row group writes 1/group of the pair slots of
// one-row items, which the per-body sums read back: on the C4 ensemble the slots fall from
// 124 MB to 89 MB with groups of 2 at strip 4, and the pair kernel's DRAM bytes from 2.85x
// to 1.61x the algorithmic bytes at the same kick time alone; in the SyMBA step, where the
// closing kick shares the SMs with the FP64 drift and the recursion, the group's warps
// wait for each other at every tile J and the step is 0.4-0.9% slower.  So a group is
// taken, like every other candidate, only when it is more than 3% faster.  Strips stop at
// 4: longer ones make the closing kick's items that touch a listed body (and so wait for
// the recursion) coarser (strip 8: 1.5% slower steps).
constexpr int SYM_GROUPS[] = {2, 4};
constexpr int SYM_NGROUP = 2;
constexpr int SYM_GROUP_STRIPS[] = {2, 4};
constexpr int SYM_NGROUP_STRIP = 2;

// Times the symmetric kick (pair kernel and per-body sums into scratch accelerations) on
// this ensemble's current data: first the two tile sizes (128 and 64 bodies, each at its
// default strip), then every candidate strip at the chosen tile with one warp per block,
// then (128-body tiles) every candidate block size at the chosen strip; each candidate one
// warm-up, then the shortest of five launches timed one by one.  The defaults (128 bodies,
// kick_sym_strip's strip, one warp) stay unless another candidate is faster by more than
// 3%, so that timing noise does not move the choice between near-equal candidates.  Last
// (128-body tiles) the row groups at their strips, by the same rule.  The partners must be
// split into kA/kB.
int time_sym_plan(swg_ensemble *e, bool rad, unsigned *head, int *best_tile, int *best_strip, int *best_warps,
                  int *best_group) {
    swg_ctx *c = e->c;
    TuneScratch t;
    SWG_TRY(dalloc(c, &t.acc, 3 * (size_t)e->NPL));
    for (cudaEvent_t &x : t.ev) SWG_TRY(cuda_status(c, cudaEventCreate(&x), "event"));
    const float4 *pa = e->kend ? e->kA2 : e->kA, *pb = e->kend ? e->kB2 : e->kB;
    auto timed = [&](int warps, float *out) -> int {
        auto once = [&]() -> int {
            SWG_TRY(kick_mixed_sym_batched(c, rad, e->n_sym, e->it_sym, e->poff, e->npl, e->sym_base, pa, pb,
                                           e->sym_part, e->sym_ppart, head, nullptr, 0, nullptr, 0, warps,
                                           e->sym_tile, e->sym_group));
            return kick_mixed_sym_reduce(c, e->sym_strip, e->NPL, e->psys, e->poff, e->npl, e->sym_base, e->sym_part,
                                         e->sym_ppart, t.acc, 1, nullptr, 0, e->sym_tile, e->sym_group);
        };
        SWG_TRY(once());
        *out = 3.0e38f;
        for (int rep = 0; rep < 5; rep++) {
            SWG_TRY(cuda_status(c, cudaEventRecord(t.ev[0], c->stream), "event"));
            SWG_TRY(once());
            SWG_TRY(cuda_status(c, cudaEventRecord(t.ev[1], c->stream), "event"));
            SWG_TRY(cuda_status(c, cudaEventSynchronize(t.ev[1]), "event"));
            float ms = 0.f;
            SWG_TRY(cuda_status(c, cudaEventElapsedTime(&ms, t.ev[0], t.ev[1]), "event"));
            *out = std::min(*out, ms);
        }
        return SWG_OK;
    };
    // tile size: 128 unless 64 is more than 3% faster, each at its default strip
    float ms_tile[2];
    e->sym_group = 1;
    for (int q = 0; q < 2; q++) {
        e->sym_tile = q == 0 ? KICK_SYM_TILE : 64;
        SWG_TRY(build_sym_plan(e, kick_sym_strip(e->nsys, e->h_npl.data(), c->num_sms, e->sym_tile)));
        SWG_TRY(timed(1, &ms_tile[q]));
    }
    e->sym_tile = ms_tile[1] < 0.97f * ms_tile[0] ? 64 : KICK_SYM_TILE;
    *best_tile = e->sym_tile;
    const int deflt = kick_sym_strip(e->nsys, e->h_npl.data(), c->num_sms, e->sym_tile);
    float ms_strip[SYM_NSTRIP], deflt_ms = 0.f;
    for (int q = 0; q < SYM_NSTRIP; q++) {
        SWG_TRY(build_sym_plan(e, SYM_STRIPS[q]));
        SWG_TRY(timed(1, &ms_strip[q]));
        if (SYM_STRIPS[q] == deflt) deflt_ms = ms_strip[q];
    }
    *best_strip = deflt;
    float best_ms = deflt_ms;
    for (int q = 0; q < SYM_NSTRIP; q++)
        if (ms_strip[q] < 0.97f * deflt_ms && ms_strip[q] < best_ms) {
            best_ms = ms_strip[q];
            *best_strip = SYM_STRIPS[q];
        }
    SWG_TRY(build_sym_plan(e, *best_strip));
    *best_warps = 1;
    const float one_ms = best_ms;
    for (int q = 1; q < SYM_NWARPS && e->sym_tile == KICK_SYM_TILE; q++) {
        float ms = 0.f;
        SWG_TRY(timed(SYM_WARPS[q], &ms));
        if (ms < 0.97f * one_ms && ms < best_ms) {
            best_ms = ms;
            *best_warps = SYM_WARPS[q];
        }
    }
    *best_group = 1;
    if (e->sym_tile == KICK_SYM_TILE) {
        float group_ms = 3.0e38f;
        int group = 1, group_strip = 0;
        for (int a = 0; a < SYM_NGROUP; a++)
            for (int b = 0; b < SYM_NGROUP_STRIP; b++) {
                e->sym_group = SYM_GROUPS[a];
                SWG_TRY(build_sym_plan(e, SYM_GROUP_STRIPS[b]));
                float ms = 0.f;
                SWG_TRY(timed(1, &ms));
                if (ms < group_ms) {
                    group_ms = ms;
                    group = SYM_GROUPS[a];
                    group_strip = SYM_GROUP_STRIPS[b];
                }
            }
        if (group_ms < 0.97f * best_ms) {
            *best_group = group;
            *best_strip = group_strip;
            *best_warps = group;
        }
        e->sym_group = 1;
    }
    return SWG_OK;
}

// Makes sure the mixed kick of kind k has a tile shape and items: the forced shape, else
// the cached choice for (GPU, kind, size bucket), else the fastest one timed here (and
// cached).  Runs eagerly at the first such kick; a CUDA graph capture never meets an
// unchosen kind (graphs are captured after an eager step, and every change of shape or
// kind drops the graph).
int ensure_kick_plan(swg_ensemble *e, int k, bool rad, unsigned *head, const int32_t *flag, int phase) {
    if (e->kv[k] >= 0) return SWG_OK;
    swg_ctx *c = e->c;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    SWG_TRY(cuda_status(c, cudaStreamIsCapturing(c->stream, &cap), "capture status"));
    if (cap != cudaStreamCaptureStatusNone) {
        c->err = "mixed kick shape not chosen before graph capture";
        return SWG_ERR_STATE;
    }
    int v = e->force_variant;
    if (v < 0 && k == 0 && !e->tiny) {  // pl-pl: the symmetric kernel (it has no GMTINY rule), its shape forced,
                                        // cached or timed here
        if (!e->it_sym) {
            int tile = e->force_tile, strip = e->force_strip, warps = e->force_warps, group = e->force_group;
            if (tile <= 0 || strip <= 0 || warps <= 0 || group <= 0) {
                const std::string key = tune_key(c->device, rad ? "kick_sym4_rad" : "kick_sym4", size_bucket(e, 0));
                // cached as log2(strip) + 8 log2(warps) + 64 (tile == 64) + 128 log2(group)
                const int l = tune_lookup(key);
                int tt = 0, ts = 0, tw = 0, tg = 0;
                if (l >= 0 && (l & 7) < SYM_NSTRIP && ((l >> 3) & 7) < SYM_NWARPS && (l >> 7) <= SYM_NGROUP) {
                    tt = ((l >> 6) & 1) ? 64 : KICK_SYM_TILE;
                    ts = 1 << (l & 7);
                    tw = 1 << ((l >> 3) & 7);
                    tg = 1 << (l >> 7);
                } else {
                    SWG_TRY(time_sym_plan(e, rad, head, &tt, &ts, &tw, &tg));
                    int ls = 0, lw = 0, lg = 0;
                    while ((1 << ls) < ts) ls++;
                    while ((1 << lw) < tw) lw++;
                    while ((1 << lg) < tg) lg++;
                    tune_store(key, ls + 8 * lw + (tt == 64 ? 64 : 0) + 128 * lg);
                }
                if (tile <= 0) tile = group > 1 ? KICK_SYM_TILE : tt;  // row groups take 128-body tiles
                if (strip <= 0) strip = ts;
                if (warps <= 0) warps = tw;
                if (group <= 0) group = tg;
            }
            // a forced one-row shape (warps per block or 64-body tiles) leaves row groups out
            if (tile != KICK_SYM_TILE || (e->force_warps > 0 && e->force_group <= 0)) group = 1;
            e->sym_tile = tile;
            e->sym_group = group;
            SWG_TRY(build_sym_plan(e, strip));
            e->sym_warps = group > 1 ? group : (tile == KICK_SYM_TILE ? warps : 1);
        }
        e->kv[0] = KICK_SYMMETRIC;
        return SWG_OK;
    }
    if (v < 0) {
        const std::string key =
            tune_key(c->device, k == 0 ? (rad ? "kick_pl_rad" : "kick_pl") : "kick_tp", size_bucket(e, k));
        v = tune_lookup(key);
        if (v < 0) {
            SWG_TRY(time_kick_variants(e, k, rad, head, flag, phase, &v));
            tune_store(key, v);
        }
    }
    SWG_TRY(put_items(e, &e->kit[k], &e->n_kit[k], kick_items(e, k, kick_variant_tile(v))));
    e->kv[k] = v;
    return SWG_OK;
}

// Forget the chosen shapes (and the graph holding their items).
void reset_kick_plans(swg_ensemble *e) {
    for (int k = 0; k < 2; k++) e->kv[k] = -1;
    if (e->graph) cudaGraphExecDestroy(e->graph);
    e->graph = nullptr;
    e->eager_steps = 0;
}

// pl-pl accelerations into ah (helio_kick_getacch_int_pl / symba_kick_getacch_int_pl) of all
// systems, or (flag != nullptr) of the systems whose flag equals phase, on c->stream.
int accel_int_pl(swg_ensemble *e, unsigned *head, const int32_t *flag = nullptr, int phase = 0, int acc_is_zero = 1) {
    swg_ctx *c = e->c;
    const bool rad = e->integrator == SWG_SYMBA || e->lclose;
    const double *R = rad ? e->radius : nullptr;
    if (e->precision == SWG_MIXED) {
        float4 *pa = e->kend ? e->kA2 : e->kA, *pb = e->kend ? e->kB2 : e->kB;
        SWG_TRY(kick_split_launch(c, e->NPL, e->rh, e->Gmass, R, pa, pb, flag ? e->psys : nullptr, flag, phase));
        SWG_TRY(ensure_kick_plan(e, 0, rad, head, flag, phase));
        if (e->kv[0] == KICK_SYMMETRIC) {  // never with semi-interacting bodies (ensure_kick_plan)
            SWG_TRY(kick_mixed_sym_batched(c, rad, e->n_sym, e->it_sym, e->poff, e->npl, e->sym_base, pa, pb,
                                           e->sym_part, e->sym_ppart, head, flag, phase, nullptr, 0, e->sym_warps,
                                           e->sym_tile, e->sym_group));
            return kick_mixed_sym_reduce(c, e->sym_strip, e->NPL, e->psys, e->poff, e->npl, e->sym_base, e->sym_part,
                                         e->sym_ppart, e->ah, acc_is_zero, flag, phase, e->sym_tile, e->sym_group);
        }
        return mixed_kick(e, 0, e->kv[0], e->kit[0], e->n_kit[0], e->ah, rad, head, flag, phase, acc_is_zero);
    }
    return kick_plpl_fp64_batched(c, rad, e->n_fpl, e->it_fpl, e->poff, e->npl, e->rh, e->Gmass, R, e->ah,
                                  acc_is_zero, flag, phase, e->tiny ? e->nplm : nullptr);
}

// Runs f with the context's stream temporarily replaced (single host thread).
template <class F>
int on_stream(swg_ctx *c, cudaStream_t st, F f) {
    const cudaStream_t saved = c->stream;
    c->stream = st;
    const int rc = f();
    c->stream = saved;
    return rc;
}

// helio_kick_vb_pl (helio_kick.f90:91-132) with symba_kick_getacch_pl (symba_kick.f90:36-76).
// have_acc: the accelerations are already in ah (see ens_step); update: apply vb += ah dt
// here (close_pl applies the closing kick inside its sums instead).
int kick_vb_pl(swg_ensemble *e, double dt, int lbeg, bool have_acc = false, bool update = true) {
    swg_ctx *c = e->c;
    if (e->NPL == 0) return SWG_OK;
    if (!have_acc) {
        ProfScope ps(e->prof, c->stream, PROF_KICK_PL);
        SWG_TRY(accel_int_pl(e, e->head));
    }
    if (e->integrator == SWG_SYMBA && e->pp_n > 0) {
        SWG_TRY(ensure(c, e->pair_terms, (size_t)e->pp_n * (6 * sizeof(double) + 1)));
        double *t = (double *)e->pair_terms.ptr;
        uint8_t *ok = (uint8_t *)(t + 6 * e->pp_n);
        k_ens_pair_terms<<<grid_for(e->pp_n, 128), 128, 0, c->stream>>>(e->pp_n, e->pp_l, e->pp_cap, e->rh, e->Gmass,
                                                                        e->radius, t, ok);
        SWG_TRY(L(c, "ens_pair_terms"));
        k_ens_kick_pairs_warp<<<grid_for(32 * (int64_t)e->nsys, 128), 128, 0, c->stream>>>(
            e->nsys, e->seg_pp, e->pp_l, e->pp_cap, t, ok, e->ah);
        SWG_TRY(L(c, "ens_kick_pairs"));
    }
    if (!update) return SWG_OK;
    k_kick_update<<<grid_for(e->NPL, 128), 128, 0, c->stream>>>((int)e->NPL, e->vb, e->ah, e->lmask, dt, e->rh,
                                                                 lbeg ? e->rbeg : e->rend);
    return L(c, "kick_update_pl");
}

// helio_kick_vb_tp (helio_kick.f90:135-169) with symba_kick_getacch_tp (symba_kick.f90:79-123).
// The mixed path reuses the partner split of the pl kick just before it: the pl
// positions it was taken from are exactly rbeg / rend.
// head: the work-queue counter (a stream of its own when the tp kick runs beside the pl work).
int kick_vb_tp(swg_ensemble *e, double dt, int lbeg, unsigned *head = nullptr) {
    swg_ctx *c = e->c;
    if (e->NTP == 0) return SWG_OK;
    const double *rp = lbeg ? e->rbeg : e->rend;
    if (!head) head = e->head;
    {
        ProfScope ps(e->prof, c->stream, PROF_KICK_TP);
        if (e->precision == SWG_MIXED) {
            SWG_TRY(ensure_kick_plan(e, 1, false, head, nullptr, 0));
            SWG_TRY(mixed_kick(e, 1, e->kv[1], e->kit[1], e->n_kit[1], e->tah, false, head, nullptr, 0));
        } else {
            SWG_TRY(kick_tp_fp64_batched(c, e->n_ftp, e->it_ftp, e->toff, e->ntp, e->poff, e->npl, e->trh, rp,
                                         e->Gmass, e->tlmask, e->tah, 1));
        }
    }
    if (e->integrator == SWG_SYMBA && e->pt_n > 0) {
        k_ens_pltp_addback<<<grid_for(32 * (int64_t)e->nsys, 128), 128, 0, c->stream>>>(
            e->nsys, e->seg_pt, e->pt_l, e->pt_cap, e->tlmask, e->trh, rp, e->Gmass, e->tah);
        SWG_TRY(L(c, "ens_pltp_addback"));
    }
    k_kick_update<<<grid_for(e->NTP, 128), 128, 0, c->stream>>>((int)e->NTP, e->tvb, e->tah, e->tlmask, dt, nullptr,
                                                                 nullptr);
    return L(c, "kick_update_tp");
}

// Mixed path: one per-system sum over chunks (partials, then apply).
template <int MODE>
int chunk_sum(swg_ensemble *e, const int32_t *lfirst, const double *vsum, const int32_t *mask, const double *vin,
              double *vout, double dt, int slot) {
    swg_ctx *c = e->c;
    if (e->nchunks == 0) return SWG_OK;
    k_chunk_sums<MODE><<<e->nchunks, CHUNK_T, 0, c->stream>>>(e->nchunks, e->chunks, lfirst, e->Gmass, vsum, mask,
                                                              e->chunk_part);
    SWG_TRY(L(c, "chunk_sums"));
    k_chunk_apply<MODE><<<e->nchunks, CHUNK_T, 0, c->stream>>>(e->chunks, e->sys_chunks, lfirst, e->chunk_part,
                                                               e->GMcb, 0.0, e->lmask, vin, vout, e->rh, dt, e->dcb,
                                                               slot);
    return L(c, "chunk_apply");
}

int lindrift_pl(swg_ensemble *e, double dt, int slot) {
    if (e->NPL == 0) return SWG_OK;
    if (!exact(e)) return chunk_sum<SUM_LIN>(e, nullptr, e->vb, e->lmask, nullptr, nullptr, dt, slot);
    k_ens_lindrift<<<e->nsys, ENS_SUM_T, 0, e->c->stream>>>(e->poff, e->npl, e->Gmass, e->vb, e->lmask, e->GMcb, e->rh, dt,
                                                     e->dcb, slot, exact(e));
    return L(e->c, "ens_lindrift");
}
int tp_misc(swg_ensemble *e, int slot, double dt, int mode, int mode_first) {
    if (e->NTP == 0) return SWG_OK;
    k_ens_tp_misc<<<grid_for(e->NTP, 256), 256, 0, e->c->stream>>>(e->NTP, e->tsys, e->tlmask, e->trh, e->tvh, e->tvb,
                                                                    e->dcb, slot, dt, mode, mode_first, e->lfirst);
    return L(e->c, "ens_tp_misc");
}
int vh2vb_pl(swg_ensemble *e, bool first_only) {
    if (e->NPL == 0) return SWG_OK;
    if (!exact(e))
        return chunk_sum<SUM_VH2VB>(e, first_only ? e->lfirst : nullptr, e->vh, nullptr, e->vh, e->vb, 0.0, 0);
    k_ens_vh2vb<<<e->nsys, ENS_SUM_T, 0, e->c->stream>>>(e->poff, e->npl, first_only ? e->lfirst : nullptr, e->Gmass, e->vh,
                                                  e->vb, e->GMcb, e->dcb, exact(e));
    return L(e->c, "ens_vh2vb");
}
int vb2vh_pl(swg_ensemble *e) {
    if (e->NPL == 0) return SWG_OK;
    if (!exact(e)) return chunk_sum<SUM_VB2VH>(e, nullptr, e->vb, e->status, e->vb, e->vh, 0.0, 0);
    k_ens_vb2vh<<<e->nsys, ENS_SUM_T, 0, e->c->stream>>>(e->poff, e->npl, e->Gmass, e->vb, e->status, e->vh, e->GMcb, e->dcb,
                                                  exact(e));
    return L(e->c, "ens_vb2vh");
}
// The mixed path's closing pl half-step in two passes over the chunks (close_pl): the
// closing velocity kick (k_kick_update's operation, with the copy of rh to rcopy for the
// test particles' closing kick) and, on the kicked velocities, both per-chunk sums of the
// step's end: sum(Gm vb) over lmask (helio_drift_linear_pl) and over status /= INACTIVE
// (swiftest_util_coord_vb2vh_pl), each formed exactly as k_chunk_sums forms it (the same
// thread per body, the same shuffles and warp order); then both results applied as
// k_chunk_apply applies them.  vb is not changed by the linear drift, so the vb2vh sum can
// be taken in the same pass: the same bits as the three separate steps.
__global__ void __launch_bounds__(CHUNK_T) k_chunk_close_sums(const int4 *__restrict__ chunks,
                                                             const double *__restrict__ Gm, double *v,
                                                             const double *__restrict__ a,
                                                             const int32_t *__restrict__ lmask,
                                                             const int32_t *__restrict__ status, double dt,
                                                             const double *__restrict__ r, double *rcopy,
                                                             double *__restrict__ out) {
    const int c = blockIdx.x;
    const int4 ch = chunks[c];
    double s[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int k = threadIdx.x; k < ch.z; k += CHUNK_T) {
        const int i = ch.y + k;
        if (rcopy)
            for (int d = 0; d < 3; d++) rcopy[3 * i + d] = r[3 * i + d];
        const bool lm = lmask[i] != 0;
        if (lm)
            for (int d = 0; d < 3; d++) v[3 * i + d] = v[3 * i + d] + a[3 * i + d] * dt;
        const double g = Gm[i];
        if (lm)
            for (int d = 0; d < 3; d++) s[d] = fma(g, v[3 * i + d], s[d]);
        if (status[i] != ST_INACTIVE)
            for (int d = 0; d < 3; d++) s[3 + d] = fma(g, v[3 * i + d], s[3 + d]);
    }
    __shared__ double sh[CHUNK_T / 32][6];
    for (int off = 16; off > 0; off >>= 1)
        for (int q = 0; q < 6; q++) s[q] += __shfl_down_sync(0xffffffffu, s[q], off);
    if ((threadIdx.x & 31) == 0)
        for (int q = 0; q < 6; q++) sh[threadIdx.x >> 5][q] = s[q];
    __syncthreads();
    if (threadIdx.x < 6) {
        double t = 0.0;
        for (int w = 0; w < CHUNK_T / 32; w++) t += sh[w][threadIdx.x];
        out[6 * c + threadIdx.x] = t;
    }
}
__global__ void __launch_bounds__(CHUNK_T) k_chunk_close_apply(const int4 *__restrict__ chunks,
                                                              const int2 *__restrict__ sys_chunks,
                                                              const double *__restrict__ part,
                                                              const double *__restrict__ GMcb,
                                                              const int32_t *__restrict__ lmask,
                                                              const double *__restrict__ vb, double *vh, double *rh,
                                                              double dt, double *dcb, int slot) {
    const int c = blockIdx.x;
    const int4 ch = chunks[c];
    const int s = ch.x;
    __shared__ double tot[6];
    if (threadIdx.x < 6) {
        const int2 rg = sys_chunks[s];
        double t = 0.0;
        for (int q = rg.x; q < rg.x + rg.y; q++) t += part[6 * q + threadIdx.x];
        tot[threadIdx.x] = t;
    }
    __syncthreads();
    const double fl = 1.0 / GMcb[s], fv = -1.0 / GMcb[s];
    const double px = tot[0] * fl, py = tot[1] * fl, pz = tot[2] * fl;
    const double cx = tot[3] * fv, cy = tot[4] * fv, cz = tot[5] * fv;
    if (ch.w == 0 && threadIdx.x == 0) {
        double *d = dcb + CB_N * s;
        d[slot + 0] = px;
        d[slot + 1] = py;
        d[slot + 2] = pz;
        d[CB_VB + 0] = cx;
        d[CB_VB + 1] = cy;
        d[CB_VB + 2] = cz;
    }
    for (int k = threadIdx.x; k < ch.z; k += CHUNK_T) {
        const int i = ch.y + k;
        if (lmask[i]) {
            rh[3 * i + 0] = fma(px, dt, rh[3 * i + 0]);
            rh[3 * i + 1] = fma(py, dt, rh[3 * i + 1]);
            rh[3 * i + 2] = fma(pz, dt, rh[3 * i + 2]);
        }
        vh[3 * i + 0] = vb[3 * i + 0] - cx;
        vh[3 * i + 1] = vb[3 * i + 1] - cy;
        vh[3 * i + 2] = vb[3 * i + 2] - cz;
    }
}

// The closing pl half of a step: kick_vb_pl (closing), lindrift_pl (CB_PTEND), vb2vh_pl.
// The mixed path runs the velocity update and both sums as k_chunk_close_sums /
// k_chunk_close_apply (same bits, two launches instead of five).
int close_pl(swg_ensemble *e, double dth, bool have_acc = false) {
    swg_ctx *c = e->c;
    if (exact(e) || e->NPL == 0 || e->nchunks == 0) {
        SWG_TRY(kick_vb_pl(e, dth, 0, have_acc));
        SWG_TRY(lindrift_pl(e, dth, CB_PTEND));
        return vb2vh_pl(e);
    }
    SWG_TRY(kick_vb_pl(e, dth, 0, have_acc, false));
    SWG_TRY(ensure(c, e->close_part, sizeof(double) * 6 * (size_t)e->nchunks));
    double *part = (double *)e->close_part.ptr;
    k_chunk_close_sums<<<e->nchunks, CHUNK_T, 0, c->stream>>>(e->chunks, e->Gmass, e->vb, e->ah, e->lmask, e->status,
                                                              dth, e->rh, e->NTP > 0 ? e->rend : nullptr, part);
    SWG_TRY(L(c, "chunk_close_sums"));
    k_chunk_close_apply<<<e->nchunks, CHUNK_T, 0, c->stream>>>(e->chunks, e->sys_chunks, part, e->GMcb, e->lmask,
                                                               e->vb, e->vh, e->rh, dth, e->dcb, CB_PTEND);
    return L(c, "chunk_close_apply");
}

// Danby drift of every body at level -1 (SyMBA: bodies outside encounters) with its
// own system's GMcb; HELIO drifts every active body.
int drift_bodies(swg_ensemble *e, double dt, bool pl = true, bool tp = true) {
    swg_ctx *c = e->c;
    ProfScope ps(e->prof, c->stream, PROF_DRIFT);
    const bool symba = e->integrator == SWG_SYMBA;
    if (pl && e->NPL > 0)
        SWG_TRY(drift_masked(c, 0.0, e->rh, e->vb, (int32_t)e->NPL, symba ? e->levelg : nullptr, -1, dt, e->status,
                             nullptr, e->GMcb, e->psys, !exact(e)));
    if (tp && e->NTP > 0)
        SWG_TRY(drift_masked(c, 0.0, e->trh, e->tvb, (int32_t)e->NTP, symba ? e->tlevelg : nullptr, -1, dt,
                             e->tstatus, nullptr, e->GMcb, e->tsys, !exact(e)));
    return SWG_OK;
}

// The pl and tp sets of the radius-sorted checks (renc: the pl encounter radii, or the
// radii for the discard scan); v: the velocities the check uses.
SortedSet pl_set(swg_ensemble *e, const double *r, const double *v, const double *renc) {
    SortedSet x;
    x.off = e->poff;
    x.n = e->npl;
    x.r = r;
    x.v = v;
    x.renc = renc;
    x.perm = e->perm;
    x.F = e->eS;
    x.N = e->NPL;
    x.ntiles = e->ntiles;
    x.tiles = e->tiles;
    x.tbase = e->tbase;
    x.bounds = e->bounds;
    x.nmax = e->nmax;
    return x;
}
SortedSet tp_set(swg_ensemble *e, const double *r, const double *v) {
    SortedSet x;
    x.off = e->toff;
    x.n = e->ntp;
    x.r = r;
    x.v = v;
    x.perm = e->tperm;
    x.F = e->eT;
    x.N = e->NTP;
    x.ntiles = e->nttiles;
    x.tiles = e->ttiles;
    x.tbase = e->ttbase;
    x.bounds = e->tbounds;
    x.nmax = e->ntmax;
    return x;
}

// System of every sort-and-sweep extent: the bodies of list 1 (n1, systems psys) then list
// 2 (n2, systems tsys), their lower extents first, then their upper ones (k_sas_extents).
__global__ void k_ext_systems(int64_t n1, const int32_t *__restrict__ psys, int64_t n2,
                              const int32_t *__restrict__ tsys, int32_t *ext) {
    const int64_t ntot = n1 + n2;
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= 2 * ntot) return;
    const int64_t b = k < ntot ? k : k - ntot;
    ext[k] = b < n1 ? psys[b] : tsys[b - n1];
}

int bits_for(int32_t n) {
    int b = 1;
    while (b < 31 && (int64_t(1) << b) < n) b++;
    return b;
}

// One level-0 check (kind 0 pl-pl, 1 pl-tp) of every system into the raw buffer, counted,
// the count copied to the host.  resort: refresh the radial orders (pl-pl check).
// SORTSWEEP: one sort of every system's extents (systems as the most significant digits),
// then each body sweeps its own system's run; the raw list may hold a pair twice.
int level0_check(swg_ensemble *e, int kind, double dt, bool resort) {
    swg_ctx *c = e->c;
    EncWork &x = kind == 0 ? e->enc_pp : e->enc_pt;
    unsigned long long *h = (unsigned long long *)(e->h_flags + 8);
    int32_t *i1 = (int32_t *)x.raw.ptr, *i2 = i1 + x.rawcap, *lv = i2 + x.rawcap;
    unsigned long long *cnt = (unsigned long long *)x.counters.ptr;
    SWG_TRY(cuda_status(c, cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), c->stream), "memset"));
    const int mode = kind == 0 ? e->enc_plpl : e->enc_pltp;
    if (mode == SWG_ENC_SORTSWEEP) {
        const int64_t n1 = e->NPL, n2 = kind == 0 ? 0 : e->NTP, ntot = n1 + n2;
        if (ntot > INT32_MAX / 2) return SWG_ERR_ARG;
        int32_t *&ext = kind == 0 ? e->ext_pp : e->ext_pt;
        if (!ext) {
            SWG_TRY(dalloc(c, &ext, 2 * (size_t)ntot));
            k_ext_systems<<<grid_for(2 * ntot, 256), 256, 0, c->stream>>>(n1, e->psys, n2, e->tsys, ext);
            SWG_TRY(L(c, "ext_systems"));
        }
        SWG_TRY(ensure(c, e->sas, sas_scratch_bytes((int)ntot)));
        SWG_TRY(sas_launch(c, (int)n1, e->l0_r, e->l0_v, e->renc, (int)n2, e->l0_tr, e->l0_tv, nullptr, kind == 0, 0,
                           dt, x.rawcap, i1, i2, lv, cnt, e->sas.ptr, ext, bits_for(e->nsys), false));
    } else if (kind == 1 && e->enc_plpl == SWG_ENC_SORTSWEEP) {  // pl set prepared by level0_launch
        SWG_TRY(pltp_sorted_batched(c, false, pl_set(e, e->l0_r, e->l0_v, e->renc), tp_set(e, e->l0_tr, e->l0_tv),
                                    nullptr, e->n_tsp, e->it_tsp, dt, x.rawcap, i1, i2, lv, cnt, nullptr));
    } else if (kind == 0)
        SWG_TRY(encounter_plpl_sorted_batched(c, e->nsys, e->nmax, e->poff, e->npl, e->l0_r, e->l0_v, e->renc, dt,
                                              resort, e->perm, e->eS, e->NPL, e->ntiles, e->tiles, e->tbase,
                                              e->bounds, e->n_esp, e->it_esp, x.rawcap, i1, i2, lv, cnt,
                                              e->tiny ? e->nplm : nullptr));
    else  // the pl set was prepared (renc, this state) by the pl-pl check just before
        SWG_TRY(pltp_sorted_batched(c, false, pl_set(e, e->l0_r, e->l0_v, e->renc), tp_set(e, e->l0_tr, e->l0_tv),
                                    nullptr, e->n_tsp, e->it_tsp, dt, x.rawcap, i1, i2, lv, cnt, nullptr));
    return cuda_status(c, cudaMemcpyAsync(&h[kind], cnt, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                          c->stream),
                       "count");
}

// Level-0 checks of every system (symba_encounter_check_pl / _tp,
// symba_encounter_check.f90:14-87, 238-296), TRIANGULAR, in two halves: level0_launch
// queues the checks on c->stream, reading the positions and velocities r, v (pl) and
// tr, tv (tp) -- the state at the start of the step, or a copy of it -- and the pair
// counts' copies to the host; level0_finish waits for the counts (one host
// synchronisation of c->stream), redoes a check whose raw buffer overflowed, and sorts the
// lists into the pools with the level marks and per-system segments.
int level0_launch(swg_ensemble *e, double dt, const double *r, const double *v, const double *tr, const double *tv) {
    swg_ctx *c = e->c;
    e->pp_n = e->pt_n = 0;
    e->l0_r = r;
    e->l0_v = v;
    e->l0_tr = tr;
    e->l0_tv = tv;
    k_set_renc<<<grid_for(e->NPL, 128), 128, 0, c->stream>>>((int)e->NPL, e->rhill, e->rhscale, 0, e->renc);
    SWG_TRY(L(c, "set_renc"));
    EncWork *w[2] = {&e->enc_pp, &e->enc_pt};
    for (int k = 0; k < 2; k++) {
        SWG_TRY(ensure(c, w[k]->counters, 2 * sizeof(unsigned long long)));
        if (w[k]->rawcap < 4096) {
            w[k]->rawcap = 4096;
            SWG_TRY(ensure(c, w[k]->raw, (size_t)w[k]->rawcap * 3 * sizeof(int32_t)));
        }
    }
    unsigned long long *h = (unsigned long long *)(e->h_flags + 8);
    const bool resort = e->nchecks++ % RESORT_EVERY == 0;
    h[0] = h[1] = 0;
    if (e->n_tsp > 0) SWG_TRY(sorted_set_prep(c, tp_set(e, tr, tv), e->nsys, resort, dt));
    // the pl-tp check and the discard scan use the pl radial order and tiles, which a
    // TRIANGULAR pl-pl check refreshes; after a sweep they are prepared here
    if (e->n_tsp > 0 && e->enc_plpl == SWG_ENC_SORTSWEEP)
        SWG_TRY(sorted_set_prep(c, pl_set(e, r, v, e->renc), e->nsys, resort, dt));
    SWG_TRY(level0_check(e, 0, dt, resort));
    if (e->n_tsp > 0) SWG_TRY(level0_check(e, 1, dt, resort));
    return SWG_OK;
}

int level0_finish(swg_ensemble *e, double dt) {
    swg_ctx *c = e->c;
    EncWork *w[2] = {&e->enc_pp, &e->enc_pt};
    unsigned long long *h = (unsigned long long *)(e->h_flags + 8);
    SWG_TRY(cuda_status(c, cudaStreamSynchronize(c->stream), "level0"));
    for (int k = 0; k < 2; k++) {  // capacity overflow: grow the raw buffers and redo that check
        if ((int64_t)h[k] <= w[k]->rawcap) continue;
        w[k]->rawcap = (int64_t)h[k] + (int64_t)h[k] / 2 + 4096;
        DevBuf fresh;
        SWG_TRY(ensure(c, fresh, (size_t)w[k]->rawcap * 3 * sizeof(int32_t)));
        cudaFree(w[k]->raw.ptr);
        w[k]->raw = fresh;
        SWG_TRY(level0_check(e, k, dt, false));  // the sets are still prepared from this state
        SWG_TRY(cuda_status(c, cudaStreamSynchronize(c->stream), "level0"));
    }
    SWG_TRY(cuda_status(c, cudaMemsetAsync(e->seg_pp, 0, sizeof(int32_t) * 2 * e->nsys, c->stream), "memset"));
    SWG_TRY(cuda_status(c, cudaMemsetAsync(e->seg_pt, 0, sizeof(int32_t) * 2 * e->nsys, c->stream), "memset"));
    for (int k = 0; k < 2; k++) {
        int64_t n = (int64_t)h[k];  // triangular lists hold no repeated pairs; a sweep's may
        if (n == 0) continue;
        const bool sweep = (k == 0 ? e->enc_plpl : e->enc_pltp) == SWG_ENC_SORTSWEEP;
        EncWork &x = *w[k];
        int32_t **list = k == 0 ? &e->pp_l : &e->pt_l;
        int64_t *cap = k == 0 ? &e->pp_cap : &e->pt_cap;
        SWG_TRY(ensure_pool(e, list, cap, n));
        int32_t *i1 = (int32_t *)x.raw.ptr, *i2 = i1 + x.rawcap, *lv = i2 + x.rawcap;
        unsigned long long *cnt = (unsigned long long *)x.counters.ptr;
        // the number of distinct pairs of a sweep's list, known once the list is sorted
        auto unique_count = [&]() -> int {
            SWG_TRY(cuda_status(c, cudaMemcpyAsync(&h[2 + k], cnt + 1, sizeof(unsigned long long),
                                                   cudaMemcpyDeviceToHost, c->stream),
                                "count"));
            SWG_TRY(cuda_status(c, cudaStreamSynchronize(c->stream), "count"));
            n = (int64_t)h[2 + k];
            return SWG_OK;
        };
        if (n <= 4096) {
            k_list_finalize<<<1, 1024, 0, c->stream>>>((int)n, i1, i2, lv, *list, *cap, k, e->levelg, e->levelm,
                                                       k == 0 ? e->nplenc : e->ntpenc, e->tlevelg, e->tlevelm,
                                                       e->tnplenc, cnt + 1);
            SWG_TRY(L(c, "list_finalize"));
            if (sweep) SWG_TRY(unique_count());
        } else {
            SWG_TRY(ensure(c, x.sort, sort_pairs_scratch_bytes(n)));
            SWG_TRY(sort_pairs_unique(c, n, i1, i2, lv, x.sort.ptr, cnt + 1));
            if (sweep) SWG_TRY(unique_count());
            for (int f = 0; f < 3; f++) {
                const int32_t *src = f == 0 ? i1 : (f == 1 ? i2 : lv);
                SWG_TRY(cuda_status(c, cudaMemcpyAsync(*list + f * *cap, src, sizeof(int32_t) * n,
                                                       cudaMemcpyDeviceToDevice, c->stream),
                                    "copy list"));
            }
            k_level0_mark<<<grid_for(n, 128), 128, 0, c->stream>>>(n, *list, *cap, k, e->levelg, e->levelm,
                                                                   k == 0 ? e->nplenc : e->ntpenc, e->tlevelg,
                                                                   e->tlevelm, e->tnplenc);
            SWG_TRY(L(c, "level0_mark"));
        }
        k_ens_segments<<<grid_for(e->nsys, 128), 128, 0, c->stream>>>(e->nsys, n, *list, e->poff,
                                                                       k == 0 ? e->seg_pp : e->seg_pt);
        SWG_TRY(L(c, "ens_segments"));
        (k == 0 ? e->pp_n : e->pt_n) = n;
    }
    k_ens_lany<<<grid_for(e->nsys, 128), 128, 0, c->stream>>>(e->nsys, e->seg_pp, e->seg_pt, e->lany);
    SWG_TRY(L(c, "ens_lany"));
    e->stats[2] += e->pp_n;
    e->stats[3] += e->pt_n;
    return SWG_OK;
}

// Collisions found by system s's paused recursion: host copies of the system's slices and
// list segments (indices made local), perfect merging, and the modified arrays written back.
int resolve_collisions(swg_ensemble *e, int s) {
    swg_ctx *c = e->c;
    const int32_t p0 = e->h_poff[s], npl = e->h_npl[s], t0 = e->h_toff[s], ntp = e->h_ntp[s];
    int32_t seg[4];
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(seg, e->seg_pp + 2 * s, 2 * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                           c->stream),
                        "collision"));
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(seg + 2, e->seg_pt + 2 * s, 2 * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                           c->stream),
                        "collision"));
    SWG_TRY(cuda_status(c, cudaStreamSynchronize(c->stream), "collision"));
    const int64_t npp = seg[1], npt = seg[3];
    const size_t n = std::max(npl, 1), m = std::max(ntp, 1);
    std::vector<double> rh(3 * n), vb(3 * n), Gm(n), R(n), rhill(n), trh(3 * m), tvb(3 * m);
    std::vector<int32_t> st(n), lm(n), lev(n), tst(m), tlm(m);
    std::vector<int32_t> pp(4 * std::max<int64_t>(npp, 1)), pt(3 * std::max<int64_t>(npt, 1));
    int32_t irec = 0;
    struct Copy {
        void *h;
        void *d;
        size_t bytes;
    };
    const size_t P = p0, T = t0;
    std::vector<Copy> xs = {{rh.data(), e->rh + 3 * P, 24 * (size_t)npl},    {vb.data(), e->vb + 3 * P, 24 * (size_t)npl},
                            {Gm.data(), e->Gmass + P, 8 * (size_t)npl},      {R.data(), e->radius + P, 8 * (size_t)npl},
                            {rhill.data(), e->rhill + P, 8 * (size_t)npl},   {st.data(), e->status + P, 4 * (size_t)npl},
                            {lm.data(), e->lmask + P, 4 * (size_t)npl},      {trh.data(), e->trh + 3 * T, 24 * (size_t)ntp},
                            {tvb.data(), e->tvb + 3 * T, 24 * (size_t)ntp},  {tst.data(), e->tstatus + T, 4 * (size_t)ntp},
                            {tlm.data(), e->tlmask + T, 4 * (size_t)ntp}};
    for (int f = 0; f < 3; f++) {  // i1, i2, status of each list segment
        const int field = f == 2 ? 3 : f;
        if (npp) xs.push_back({pp.data() + f * npp, e->pp_l + field * e->pp_cap + seg[0], 4 * (size_t)npp});
        if (npt) xs.push_back({pt.data() + f * npt, e->pt_l + field * e->pt_cap + seg[2], 4 * (size_t)npt});
    }
    // read only: the pl-pl lvdotr field and the levels (for the cascade check), the paused level
    std::vector<Copy> inputs = {{lev.data(), e->levelg + P, 4 * (size_t)npl},
                                {&irec, e->rec_resume + (size_t)REC_STATE * s + 1, 4}};
    if (npp) inputs.push_back({pp.data() + 3 * npp, e->pp_l + 2 * e->pp_cap + seg[0], 4 * (size_t)npp});
    for (auto *v : {&xs, &inputs})
        for (const Copy &x : *v)
            if (x.bytes)
                SWG_TRY(cuda_status(c, cudaMemcpyAsync(x.h, x.d, x.bytes, cudaMemcpyDeviceToHost, c->stream),
                                    "collision"));
    SWG_TRY(cuda_status(c, cudaStreamSynchronize(c->stream), "collision"));
    // global 1-based indices -> local
    for (int64_t k = 0; k < npp; k++) {
        pp[k] -= p0;
        pp[npp + k] -= p0;
    }
    for (int64_t k = 0; k < npt; k++) {
        pt[k] -= p0;
        pt[npt + k] -= t0;
    }
    CollisionSystem cs;
    cs.npl = npl;
    cs.ntp = ntp;
    cs.GMcb = e->h_GMcb[s];
    cs.rh = rh.data();
    cs.vb = vb.data();
    cs.Gm = Gm.data();
    cs.R = R.data();
    cs.rhill = rhill.data();
    cs.status = st.data();
    cs.lmask = lm.data();
    cs.trh = trh.data();
    cs.tvb = tvb.data();
    cs.tstatus = tst.data();
    cs.tlmask = tlm.data();
    cs.npp = npp;
    cs.npt = npt;
    cs.pp_i1 = pp.data();
    cs.pp_i2 = pp.data() + npp;
    cs.pp_st = pp.data() + 2 * npp;
    cs.pt_i1 = pt.data();
    cs.pt_i2 = pt.data() + npt;
    cs.pt_st = pt.data() + 2 * npt;
    cs.pp_lv = pp.data() + 3 * npp;
    cs.levelg = lev.data();
    cs.irec = irec;
    cs.dt = level_dt(e->rec_dt, irec);
    double *ct = &e->coll_terms[4 * (size_t)s];
    cs.E_collisions = ct[0];
    for (int d = 0; d < 3; d++) cs.L_escape[d] = ct[1 + d];
    cs.dev = c;
    const int64_t nres = resolve_collisions_host(cs);
    if (nres == -2) return SWG_ERR_CUDA;
    if (nres < 0) {
        c->err = "runaway collisional cascade (more than 1000 rounds of merges in one resolution)";
        return SWG_ERR_STATE;
    }
    e->stats[4] += nres;
    ct[0] = cs.E_collisions;
    for (int d = 0; d < 3; d++) ct[1 + d] = cs.L_escape[d];
    for (int64_t k = 0; k < npp; k++) {
        pp[k] += p0;
        pp[npp + k] += p0;
    }
    for (int64_t k = 0; k < npt; k++) {
        pt[k] += p0;
        pt[npt + k] += t0;
    }
    for (const Copy &x : xs)
        if (x.bytes)
            SWG_TRY(cuda_status(c, cudaMemcpyAsync(x.d, x.h, x.bytes, cudaMemcpyHostToDevice, c->stream), "collision"));
    return cuda_status(c, cudaStreamSynchronize(c->stream), "collision");
}

// Launch the SyMBA recursion of every system with encounters (one block each).  Paused
// systems are resumed by recursion_finish.
int recursion_launch(swg_ensemble *e, double dt) {
    swg_ctx *c = e->c;
    e->rec_dt = dt;
    const int64_t n = e->pp_n + e->pt_n;
    SWG_TRY(ensure(c, e->rec_scratch, sizeof(double) * (size_t)(12 * n + 8) + (size_t)(3 * n + 96) +
                                          sizeof(int32_t) * (size_t)(7 * n + 128)));
    EnsRecArgs x;
    RecArgs &a = x.base;
    a.npl = 0;
    a.ntp = 0;
    a.npp = a.npt = 0;
    a.ppcap = e->pp_cap;
    a.ptcap = e->pt_cap;
    a.pp = e->pp_l;
    a.pt = e->pt_l;
    a.rh = e->rh;
    a.vb = e->vb;
    a.ah = e->ah;
    a.trh = e->trh;
    a.tvb = e->tvb;
    a.tah = e->tah;
    a.Gm = e->Gmass;
    a.rhill = e->rhill;
    a.radius = e->radius;
    a.status = e->status;
    a.tstatus = e->tstatus;
    a.levelg = e->levelg;
    a.levelm = e->levelm;
    a.tlevelg = e->tlevelg;
    a.tlevelm = e->tlevelm;
    a.GMcb = 0.0;
    a.rhscale = e->rhscale;
    a.dt = dt;
    a.terms = (double *)e->rec_scratch.ptr;
    int32_t *ibuf = (int32_t *)(a.terms + 12 * n + 8);
    a.bpl = ibuf;               // 2 * npp + npt per system
    a.btp = ibuf + 2 * n + 32;  // npt per system
    a.adj_end = ibuf + 3 * n + 64;  // one per listed body: 2 * (npp + npt) per system
    a.adj = ibuf + 5 * n + 96;      // two per pl-pl entry, one per pl-tp entry
    uint8_t *bbuf = (uint8_t *)(ibuf + 7 * n + 128);
    a.lenc = bbuf;
    a.good = bbuf + n + 32;
    a.good2 = bbuf + 2 * n + 64;
    a.mark_pl = e->mark_pl;
    a.mark_tp = e->mark_tp;
    a.out = e->rec_out;
    a.lclose = e->lclose;
    a.fast = !exact(e);
    // every block gets room for the stage of all lists together, up to REC_STAGE_ENS; a
    // system whose own lists do not fit runs on the global arrays
    a.stage_bytes = (int64_t)std::min(rec_stage_bytes(e->pp_n, e->pt_n), REC_STAGE_ENS);
    static bool smem_set = false;  // the kernel's own shared arrays come on top of the stage
    if (a.stage_bytes > 0 && !smem_set) {
        SWG_TRY(cuda_status(c, cudaFuncSetAttribute(k_ens_symba_recursion, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                    (int)REC_STAGE_ENS),
                            "recursion smem"));
        smem_set = true;
    }
    x.seg_pp = e->seg_pp;
    x.seg_pt = e->seg_pt;
    x.npl = e->npl;
    x.ntp = e->ntp;
    x.GMcb = e->GMcb;
    x.resume = e->rec_resume;
    x.pend = e->rec_pend;
    e->rec_args = x;
    SWG_TRY(cuda_status(c, cudaMemsetAsync(e->rec_out, 0, sizeof(int32_t), c->stream), "memset"));
    if (e->lclose)
        SWG_TRY(cuda_status(c, cudaMemsetAsync(e->rec_pend, 0, sizeof(int32_t) * e->nsys, c->stream), "memset"));
    k_ens_symba_recursion<<<e->nsys, RECT, (size_t)a.stage_bytes, c->stream>>>(x, 0);
    return L(c, "ens_symba_recursion");
}

// With collision checks on (lclose), wait for the recursion, resolve the collisions of the
// systems whose recursion paused on the host and resume those systems, until none pauses.
int recursion_finish(swg_ensemble *e) {
    swg_ctx *c = e->c;
    if (e->lclose && e->drift_pending) {
        // collision resolution copies whole system slices: the level-0 drift on the side
        // stream must be done first
        SWG_TRY(cuda_status(c, cudaStreamWaitEvent(c->stream, e->ev_drift, 0), "drift"));
        e->drift_pending = false;
    }
    while (e->lclose) {
        SWG_TRY(cuda_status(c, cudaMemcpyAsync(e->h_pend.data(), e->rec_pend, sizeof(int32_t) * e->nsys,
                                               cudaMemcpyDeviceToHost, c->stream),
                            "pending"));
        SWG_TRY(cuda_status(c, cudaStreamSynchronize(c->stream), "recursion"));
        bool any = false;
        for (int s = 0; s < e->nsys; s++)
            if (e->h_pend[s]) {
                any = true;
                SWG_TRY(resolve_collisions(e, s));
            }
        if (!any) break;
        SWG_TRY(cuda_status(c, cudaMemsetAsync(e->rec_pend, 0, sizeof(int32_t) * e->nsys, c->stream), "memset"));
        k_ens_symba_recursion<<<e->nsys, RECT, (size_t)e->rec_args.base.stage_bytes, c->stream>>>(e->rec_args, 1);
        SWG_TRY(L(c, "ens_symba_recursion"));
    }
    return cuda_status(c, cudaMemcpyAsync(e->h_flags + 2, e->rec_out, sizeof(int32_t), cudaMemcpyDeviceToHost,
                                          c->stream),
                       "recursion status");
}



// The rest of a HELIO step (helio_step_system, helio_step.f90:14-119) after the opening
// pl sums, with the test particles on the side stream: their half-steps need the pl only
// through the start positions (rbeg and the first partner split) and, for the closing kick,
// the end positions (rend, the second split kA2/kB2) and the closing central-body drift
// slot, so the tp kick, drift and kick (FP32, FP64, FP32) run beside the pl drift, closing
// kick and sums.  Each body's arithmetic and order are those of the sequential step.
// Test particles [t0, t1) of one group: the half-step pieces of helio_step_tp on the
// context's current stream (tp_misc, the mixed pl-tp kick of the group's systems with its
// velocity update, and the Danby drift).
int tp_misc_range(swg_ensemble *e, int64_t t0, int64_t t1, int slot, double dt, int mode, int mode_first) {
    if (t1 <= t0) return SWG_OK;
    k_ens_tp_misc<<<grid_for(t1 - t0, 256), 256, 0, e->c->stream>>>(t1 - t0, e->tsys + t0, e->tlmask + t0,
                                                                     e->trh + 3 * t0, e->tvh + 3 * t0, e->tvb + 3 * t0,
                                                                     e->dcb, slot, dt, mode, mode_first, e->lfirst);
    return L(e->c, "ens_tp_misc");
}
int kick_tp_group(swg_ensemble *e, double dt, int group, int64_t t0, int64_t t1, unsigned *head) {
    swg_ctx *c = e->c;
    SWG_TRY(ensure_kick_plan(e, 1, false, head, nullptr, 0));
    SWG_TRY(mixed_kick(e, 1, e->kv[1], e->kit[1], e->n_kit[1], e->tah, false, head, e->tgroup, group));
    if (t1 <= t0) return SWG_OK;
    k_kick_update<<<grid_for(t1 - t0, 128), 128, 0, c->stream>>>((int)(t1 - t0), e->tvb + 3 * t0, e->tah + 3 * t0,
                                                                  e->tlmask + t0, dt, nullptr, nullptr);
    return L(c, "kick_update_tp");
}
int drift_tp_range(swg_ensemble *e, int64_t t0, int64_t t1, double dt) {
    if (t1 <= t0) return SWG_OK;
    return drift_masked(e->c, 0.0, e->trh + 3 * t0, e->tvb + 3 * t0, (int32_t)(t1 - t0), nullptr, -1, dt,
                        e->tstatus + t0, nullptr, e->GMcb, e->tsys + t0, !exact(e));
}

// Mixed path of helio_step_split with the test particles in two groups of systems: group
// 1's opening kick runs while group 0 drifts, and group 1 drifts while group 0 takes its
// closing kick, so the FP64 drift overlaps the FP32 kick.
int helio_step_groups(swg_ensemble *e, double dt) {
    swg_ctx *c = e->c;
    const double dth = 0.5 * dt;
    const int64_t T = e->tsplit, M = e->NTP;
    unsigned *h0 = e->head + 1, *h1 = e->head + 2;
    SWG_TRY(kick_vb_pl(e, dth, 1));
    // the pl-tp kick's tile shape is timed here, on this stream, before the side streams run
    // beside it (as in the sequential step, which tunes at the same point)
    SWG_TRY(ensure_kick_plan(e, 1, false, e->head, nullptr, 0));
    SWG_TRY(cuda_status(c, cudaEventRecord(e->ev_fork, c->stream), "fork"));
    SWG_TRY(cuda_status(c, cudaStreamWaitEvent(e->side, e->ev_fork, 0), "fork"));
    SWG_TRY(on_stream(c, e->side, [&] {
        SWG_TRY(tp_misc_range(e, 0, T, CB_PTBEG, dth, 2, 4));
        SWG_TRY(kick_tp_group(e, dth, 0, 0, T, h0));
        SWG_TRY(cuda_status(c, cudaEventRecord(e->ev_g0, c->stream), "group 0"));
        return drift_tp_range(e, 0, T, dt);
    }));
    SWG_TRY(cuda_status(c, cudaStreamWaitEvent(e->side2, e->ev_g0, 0), "group 0"));
    SWG_TRY(on_stream(c, e->side2, [&] {
        SWG_TRY(tp_misc_range(e, T, M, CB_PTBEG, dth, 2, 4));
        SWG_TRY(kick_tp_group(e, dth, 1, T, M, h1));
        return drift_tp_range(e, T, M, dt);
    }));
    SWG_TRY(drift_bodies(e, dt, true, false));
    e->kend = true;
    int rc = close_pl(e, dth);
    if (rc == SWG_OK) rc = cuda_status(c, cudaEventRecord(e->ev_drift, c->stream), "pl done");
    if (rc == SWG_OK) rc = cuda_status(c, cudaStreamWaitEvent(e->side, e->ev_drift, 0), "pl done");
    if (rc == SWG_OK) rc = cuda_status(c, cudaStreamWaitEvent(e->side2, e->ev_drift, 0), "pl done");
    if (rc == SWG_OK) rc = on_stream(c, e->side, [&] {
        SWG_TRY(kick_tp_group(e, dth, 0, 0, T, h0));
        SWG_TRY(tp_misc_range(e, 0, T, CB_PTEND, dth, 3, -1));
        return cuda_status(c, cudaEventRecord(e->ev_join, c->stream), "join");
    });
    if (rc == SWG_OK) rc = on_stream(c, e->side2, [&] {
        SWG_TRY(kick_tp_group(e, dth, 1, T, M, h1));
        SWG_TRY(tp_misc_range(e, T, M, CB_PTEND, dth, 3, -1));
        return cuda_status(c, cudaEventRecord(e->ev_join2, c->stream), "join");
    });
    e->kend = false;
    SWG_TRY(rc);
    SWG_TRY(cuda_status(c, cudaStreamWaitEvent(c->stream, e->ev_join, 0), "join"));
    SWG_TRY(cuda_status(c, cudaStreamWaitEvent(c->stream, e->ev_join2, 0), "join"));
    k_ens_finish<<<grid_for(e->nsys, 128), 128, 0, c->stream>>>(e->nsys, nullptr, e->lfirst, e->enc_steps);
    return L(c, "ens_finish");
}

int helio_step_split(swg_ensemble *e, double dt) {
    swg_ctx *c = e->c;
    const double dth = 0.5 * dt;
    unsigned *head_tp = e->head + 1;
    if (e->precision == SWG_MIXED && e->tgroup && e->tsplit > 0 && e->tsplit < e->NTP)
        return helio_step_groups(e, dt);
    SWG_TRY(kick_vb_pl(e, dth, 1));
    if (e->precision == SWG_MIXED) SWG_TRY(ensure_kick_plan(e, 1, false, e->head, nullptr, 0));  // see above
    SWG_TRY(cuda_status(c, cudaEventRecord(e->ev_fork, c->stream), "fork"));
    SWG_TRY(cuda_status(c, cudaStreamWaitEvent(e->side, e->ev_fork, 0), "fork"));
    SWG_TRY(on_stream(c, e->side, [&] {
        SWG_TRY(tp_misc(e, CB_PTBEG, dth, 2, 4));
        SWG_TRY(kick_vb_tp(e, dth, 1, head_tp));
        return drift_bodies(e, dt, false, true);
    }));
    SWG_TRY(drift_bodies(e, dt, true, false));
    e->kend = true;
    int rc = close_pl(e, dth);
    if (rc == SWG_OK) rc = cuda_status(c, cudaEventRecord(e->ev_drift, c->stream), "pl done");
    if (rc == SWG_OK) rc = cuda_status(c, cudaStreamWaitEvent(e->side, e->ev_drift, 0), "pl done");
    if (rc == SWG_OK) rc = on_stream(c, e->side, [&] {
        SWG_TRY(kick_vb_tp(e, dth, 0, head_tp));
        return tp_misc(e, CB_PTEND, dth, 3, -1);
    });
    e->kend = false;
    SWG_TRY(rc);
    SWG_TRY(cuda_status(c, cudaEventRecord(e->ev_join, e->side), "join"));
    SWG_TRY(cuda_status(c, cudaStreamWaitEvent(c->stream, e->ev_join, 0), "join"));
    k_ens_finish<<<grid_for(e->nsys, 128), 128, 0, c->stream>>>(e->nsys, nullptr, e->lfirst, e->enc_steps);
    return L(c, "ens_finish");
}

// One step of every system: symba_step_system (symba_step.f90:14-52) or
// helio_step_system (helio_step.f90:14-119).  A SyMBA system without encounters takes
// the HELIO step; the kernel sequence below is the same for both cases (empty lists
// make the pair subtraction, the add-back and the recursion no-ops, and every body sits
// at level -1), so all systems advance in one sequence.  Order as in
// symba_step_interp_system: pl and tp first halves, recursion, second halves.
int ens_step(swg_ensemble *e, double dt) {
    swg_ctx *c = e->c;
    const bool symba = e->integrator == SWG_SYMBA;
    const double dth = 0.5 * dt;
    bool have_acc = false;
    if (symba) {
        const int64_t nmax = std::max(e->NPL, e->NTP);
        k_symba_reset<<<grid_for(nmax, 256), 256, 0, c->stream>>>((int)e->NPL, (int)e->NTP, e->levelg, e->levelm,
                                                                   e->nplenc, e->ntpenc, e->lmask, e->tlevelg,
                                                                   e->tlevelm, e->tnplenc, e->tlmask, e->status,
                                                                   e->tstatus);
        SWG_TRY(L(c, "symba_reset"));
        if (!e->prof.on && e->NPL > 0) {
            // The level-0 checks read a copy of the start-of-step state on the side stream
            // while this stream runs the per-system sums and the first pair accelerations,
            // which do not depend on the lists; the lists are joined before the pair
            // subtraction.  Same arithmetic as the sequential order.
            const size_t n = e->NPL, m = e->NTP;
            double *sr = e->snap, *sv = sr + 3 * n, *st = sv + 3 * n, *stv = st + 3 * m;
            SWG_TRY(cuda_status(c, cudaMemcpyAsync(sr, e->rh, 24 * n, cudaMemcpyDeviceToDevice, c->stream), "snap"));
            SWG_TRY(cuda_status(c, cudaMemcpyAsync(sv, e->vb, 24 * n, cudaMemcpyDeviceToDevice, c->stream), "snap"));
            if (m) {
                SWG_TRY(cuda_status(c, cudaMemcpyAsync(st, e->trh, 24 * m, cudaMemcpyDeviceToDevice, c->stream),
                                    "snap"));
                SWG_TRY(cuda_status(c, cudaMemcpyAsync(stv, e->tvb, 24 * m, cudaMemcpyDeviceToDevice, c->stream),
                                    "snap"));
            }
            SWG_TRY(cuda_status(c, cudaEventRecord(e->ev_fork, c->stream), "fork"));
            SWG_TRY(cuda_status(c, cudaStreamWaitEvent(e->side, e->ev_fork, 0), "fork"));
            SWG_TRY(on_stream(c, e->side, [&] { return level0_launch(e, dt, sr, sv, st, stv); }));
            SWG_TRY(vh2vb_pl(e, true));
            SWG_TRY(lindrift_pl(e, dth, CB_PTBEG));
            SWG_TRY(accel_int_pl(e, e->head));
            SWG_TRY(on_stream(c, e->side, [&] { return level0_finish(e, dt); }));
            SWG_TRY(cuda_status(c, cudaEventRecord(e->ev_join, e->side), "join"));
            SWG_TRY(cuda_status(c, cudaStreamWaitEvent(c->stream, e->ev_join, 0), "join"));
            have_acc = true;
        } else {
            ProfScope ps(e->prof, c->stream, PROF_ENC0);
            SWG_TRY(level0_launch(e, dt, e->rh, e->vb, e->trh, e->tvb));
            SWG_TRY(level0_finish(e, dt));
        }
    }
    if (!have_acc) {
        SWG_TRY(vh2vb_pl(e, true));
        SWG_TRY(lindrift_pl(e, dth, CB_PTBEG));
    }
    if (!symba && !e->prof.on && e->NPL > 0 && e->NTP > 0) return helio_step_split(e, dt);
    SWG_TRY(kick_vb_pl(e, dth, 1, have_acc));
    SWG_TRY(tp_misc(e, CB_PTBEG, dth, 2, 4));
    SWG_TRY(kick_vb_tp(e, dth, 1));
    const bool rec = symba && e->pp_n + e->pt_n > 0;
    if (rec && !e->prof.on && e->NPL > 0) {
        // The level-0 drift moves only the bodies outside the lists (levelg == -1) and the
        // recursion only the bodies in them, and the closing accelerations of systems
        // without encounters do not depend on the recursion: the side stream drifts and
        // then computes those accelerations while the recursion runs (launched first, so
        // its blocks are resident); the recursing systems' accelerations follow both.
        // Each system's arithmetic is unchanged.
        swg_ctx *c = e->c;
        // Mixed symmetric kick: the closing kick's items that involve no listed body (the
        // bodies the recursion moves) do not wait for the recursion either; flag them now,
        // while the levels still say which bodies are listed.
        const bool by_item = e->precision == SWG_MIXED && e->kv[0] == KICK_SYMMETRIC && e->n_sym > 0 && e->enc_body;
        if (by_item) {
            k_mark_enc<<<grid_for(e->NPL, 256), 256, 0, c->stream>>>(e->NPL, e->levelg, e->enc_body);
            SWG_TRY(L(c, "mark_enc"));
            SWG_TRY(ensure(c, e->sym_iflag, (size_t)e->n_sym));
            SWG_TRY(kick_sym_item_flags(c, e->n_sym, e->it_sym, e->poff, e->npl, e->lany, e->enc_body,
                                        (uint8_t *)e->sym_iflag.ptr, e->sym_tile, e->sym_group));
        }
        SWG_TRY(cuda_status(c, cudaEventRecord(e->ev_fork, c->stream), "fork"));
        SWG_TRY(cuda_status(c, cudaStreamWaitEvent(e->side, e->ev_fork, 0), "fork"));
        SWG_TRY(recursion_launch(e, dt));
        SWG_TRY(on_stream(c, e->side, [&] { return drift_bodies(e, dt); }));
        SWG_TRY(cuda_status(c, cudaEventRecord(e->ev_drift, e->side), "drift"));
        e->drift_pending = true;
        const uint8_t *iflag = (const uint8_t *)e->sym_iflag.ptr;
        if (by_item) {
            // side: the unlisted bodies' partner split, then every item of the systems without
            // encounters and the unlisted items of the others, and the former's sums
            SWG_TRY(on_stream(c, e->side, [&] {
                SWG_TRY(kick_split_launch(c, e->NPL, e->rh, e->Gmass, e->radius, e->kA, e->kB, nullptr, nullptr, 0,
                                          e->enc_body, 0));
                SWG_TRY(cuda_status(c, cudaEventRecord(e->ev_split, c->stream), "split"));
                SWG_TRY(kick_mixed_sym_batched(c, true, e->n_sym, e->it_sym, e->poff, e->npl, e->sym_base, e->kA,
                                               e->kB, e->sym_part, e->sym_ppart, e->head2, nullptr, 0, iflag, 3u,
                                               e->sym_warps, e->sym_tile, e->sym_group));
                return kick_mixed_sym_reduce(c, e->sym_strip, e->NPL, e->psys, e->poff, e->npl, e->sym_base,
                                             e->sym_part, e->sym_ppart, e->ah, 1, e->lany, 0, e->sym_tile, e->sym_group);
            }));
        } else {
            SWG_TRY(on_stream(c, e->side, [&] { return accel_int_pl(e, e->head2, e->lany, 0); }));
        }
        SWG_TRY(cuda_status(c, cudaEventRecord(e->ev_join, e->side), "join"));
        SWG_TRY(recursion_finish(e));
        if (e->drift_pending) {
            SWG_TRY(cuda_status(c, cudaStreamWaitEvent(c->stream, e->ev_drift, 0), "drift"));
            e->drift_pending = false;
        }
        if (by_item) {
            // main: the listed bodies' split, the listed items, then every sum of the systems
            // with encounters once the side's items are in
            SWG_TRY(cuda_status(c, cudaStreamWaitEvent(c->stream, e->ev_split, 0), "split"));
            SWG_TRY(kick_split_launch(c, e->NPL, e->rh, e->Gmass, e->radius, e->kA, e->kB, nullptr, nullptr, 0,
                                      e->enc_body, 1));
            SWG_TRY(kick_mixed_sym_batched(c, true, e->n_sym, e->it_sym, e->poff, e->npl, e->sym_base, e->kA, e->kB,
                                           e->sym_part, e->sym_ppart, e->head, nullptr, 0, iflag, 4u, e->sym_warps,
                                           e->sym_tile, e->sym_group));
            SWG_TRY(cuda_status(c, cudaStreamWaitEvent(c->stream, e->ev_join, 0), "join"));
            SWG_TRY(kick_mixed_sym_reduce(c, e->sym_strip, e->NPL, e->psys, e->poff, e->npl, e->sym_base, e->sym_part,
                                          e->sym_ppart, e->ah, 1, e->lany, 1, e->sym_tile, e->sym_group));
        } else {
            SWG_TRY(accel_int_pl(e, e->head, e->lany, 1));
            SWG_TRY(cuda_status(c, cudaStreamWaitEvent(c->stream, e->ev_join, 0), "join"));
        }
        SWG_TRY(close_pl(e, dth, true));
    } else {
        SWG_TRY(drift_bodies(e, dt));
        if (rec) {
            ProfScope ps(e->prof, c->stream, PROF_RECUR);
            SWG_TRY(recursion_launch(e, dt));
            SWG_TRY(recursion_finish(e));
        }
        SWG_TRY(close_pl(e, dth));
    }
    SWG_TRY(kick_vb_tp(e, dth, 0));
    SWG_TRY(tp_misc(e, CB_PTEND, dth, 3, -1));
    k_ens_finish<<<grid_for(e->nsys, 128), 128, 0, c->stream>>>(e->nsys, symba ? e->lany : nullptr, e->lfirst,
                                                                 e->enc_steps);
    return L(c, "ens_finish");
}

// ---- WHM step of every system (whm_step_system, whm_step.f90:14-104).  The first-step flag
// is shared (all systems start together), so after the first step every step runs the same
// launch sequence and is replayed from a CUDA graph.
// whm_kick_vh_pl (whm_kick.f90:218-262): accelerations (whm_kick_getacch_pl: ah0, ah1, ah2,
// then the pair kick added on top) and vh += ah dt
int whm_accel_pl(swg_ensemble *e) {
    swg_ctx *c = e->c;
    SWG_TRY(cuda_status(c, cudaMemsetAsync(e->ah, 0, sizeof(double) * 3 * e->NPL, c->stream), "memset"));
    k_ens_whm_accel<<<e->nsys, 256, 0, c->stream>>>(e->poff, e->npl, e->Gmass, e->GMcb, e->rh, e->xj, e->lmask,
                                                    e->ir3h, e->ir3j, e->ah, exact(e));
    SWG_TRY(L(c, "ens_whm_accel"));
    ProfScope ps(e->prof, c->stream, PROF_KICK_PL);
    return accel_int_pl(e, e->head, nullptr, 0, 0);
}
int whm_coord(swg_ensemble *e, int mode) {
    k_ens_whm_coord<<<e->nsys, 256, 0, e->c->stream>>>(mode, e->poff, e->npl, e->Gmass, e->eta, e->rh, e->vh, e->xj,
                                                       e->vj, exact(e));
    return L(e->c, "ens_whm_coord");
}
int whm_kick_vh_pl(swg_ensemble *e, double dt, int lbeg) {
    swg_ctx *c = e->c;
    if (!lbeg || e->whm_first) {
        if (lbeg) SWG_TRY(whm_coord(e, WHM_H2J));
        SWG_TRY(whm_accel_pl(e));
    }
    k_kick_update<<<grid_for(e->NPL, 128), 128, 0, c->stream>>>((int)e->NPL, e->vh, e->ah, e->lmask, dt, e->rh,
                                                                 lbeg ? e->rbeg : e->rend);
    return L(c, "kick_update_whm");
}
// whm_kick_vh_tp (whm_kick.f90:265-318) with whm_kick_getacch_tp (:70-122): tah = ah0 of the
// system at rp, plus the pl-tp pair kick
int whm_accel_tp(swg_ensemble *e, int lbeg, unsigned *head = nullptr) {
    swg_ctx *c = e->c;
    const double *rp = lbeg ? e->rbeg : e->rend;
    if (!head) head = e->head;
    k_ens_whm_ah0<<<e->nsys, 256, 0, c->stream>>>(e->poff, e->npl, e->Gmass, rp, e->whm_ah0, exact(e));
    SWG_TRY(L(c, "ens_whm_ah0"));
    k_ens_whm_tp_ah0<<<grid_for(e->NTP, 256), 256, 0, c->stream>>>(e->NTP, e->tsys, e->tlmask, e->whm_ah0, e->tah);
    SWG_TRY(L(c, "ens_whm_tp_ah0"));
    ProfScope ps(e->prof, c->stream, PROF_KICK_TP);
    if (e->precision == SWG_MIXED) {
        // the partner split of the pl kick just before holds rp (rbeg or rend)
        SWG_TRY(ensure_kick_plan(e, 1, false, head, nullptr, 0));
        return mixed_kick(e, 1, e->kv[1], e->kit[1], e->n_kit[1], e->tah, false, head, nullptr, 0, 0);
    }
    return kick_tp_fp64_batched(c, e->n_ftp, e->it_ftp, e->toff, e->ntp, e->poff, e->npl, e->trh, rp, e->Gmass,
                                e->tlmask, e->tah, 0);
}
int whm_kick_vh_tp(swg_ensemble *e, double dt, int lbeg, bool first, unsigned *head = nullptr) {
    swg_ctx *c = e->c;
    if (first) SWG_TRY(whm_accel_tp(e, 1, head));
    if (!lbeg) SWG_TRY(whm_accel_tp(e, 0, head));
    k_kick_update<<<grid_for(e->NTP, 128), 128, 0, c->stream>>>((int)e->NTP, e->tvh, e->tah, e->tlmask, dt, nullptr,
                                                                 nullptr);
    return L(c, "kick_update_whm_tp");
}
int whm_ens_step(swg_ensemble *e, double dt) {
    swg_ctx *c = e->c;
    const double dth = 0.5 * dt;
    const bool first_tp = e->whm_first != 0;
    // After the first step the test particles' opening kick reuses the accelerations of the
    // previous closing kick and their drift needs nothing of the pl: both run on the side
    // stream beside the pl half-steps; the closing accelerations (at the pl end positions
    // and their partner split) wait for the pl.  Each body's arithmetic is unchanged.
    const bool split = !first_tp && !e->prof.on && e->NPL > 0 && e->NTP > 0;
    unsigned *head_tp = e->head + 1;
    if (split) {
        SWG_TRY(cuda_status(c, cudaEventRecord(e->ev_fork, c->stream), "fork"));
        SWG_TRY(cuda_status(c, cudaStreamWaitEvent(e->side, e->ev_fork, 0), "fork"));
        SWG_TRY(on_stream(c, e->side, [&] {
            SWG_TRY(whm_kick_vh_tp(e, dth, 1, false, head_tp));
            return drift_masked(c, 0.0, e->trh, e->tvh, (int32_t)e->NTP, nullptr, -1, dt, e->tstatus, nullptr,
                                e->GMcb, e->tsys, !exact(e));
        }));
    }
    if (e->NPL > 0) {
        SWG_TRY(whm_kick_vh_pl(e, dth, 1));
        e->whm_first = 0;
        SWG_TRY(whm_coord(e, WHM_VH2VJ));
        {
            ProfScope ps(e->prof, c->stream, PROF_DRIFT);
            SWG_TRY(drift_all(c, e->muj, 0.0, e->xj, e->vj, (int32_t)e->NPL, 0, 0.0, dt, e->lmask, e->iflag));
        }
        k_ens_whm_drift_status<<<grid_for(e->NPL, 256), 256, 0, c->stream>>>(e->NPL, e->iflag, e->status, e->lmask,
                                                                             e->whm_fail);
        SWG_TRY(L(c, "ens_whm_drift_status"));
        SWG_TRY(whm_coord(e, WHM_J2H));
        SWG_TRY(whm_kick_vh_pl(e, dth, 0));
    }
    if (split) {
        SWG_TRY(cuda_status(c, cudaEventRecord(e->ev_drift, c->stream), "pl done"));
        SWG_TRY(cuda_status(c, cudaStreamWaitEvent(e->side, e->ev_drift, 0), "pl done"));
        SWG_TRY(on_stream(c, e->side, [&] { return whm_kick_vh_tp(e, dth, 0, false, head_tp); }));
        SWG_TRY(cuda_status(c, cudaEventRecord(e->ev_join, e->side), "join"));
        return cuda_status(c, cudaStreamWaitEvent(c->stream, e->ev_join, 0), "join");
    }
    if (e->NTP > 0) {
        SWG_TRY(whm_kick_vh_tp(e, dth, 1, first_tp));
        {
            ProfScope ps(e->prof, c->stream, PROF_DRIFT);
            SWG_TRY(drift_masked(c, 0.0, e->trh, e->tvh, (int32_t)e->NTP, nullptr, -1, dt, e->tstatus, nullptr,
                                 e->GMcb, e->tsys, !exact(e)));
        }
        SWG_TRY(whm_kick_vh_tp(e, dth, 0, false));
    }
    return SWG_OK;
}

// swiftest_discard_pl_tp of every system (src/swiftest/swiftest_discard.f90:244-290), after
// each step when close encounters are checked, on the pl-tp items of the encounter check.
int discard_step(swg_ensemble *e) {
    if (!e->lclose || e->n_tsp == 0) return SWG_OK;
    swg_ctx *c = e->c;
    // SyMBA refreshes the orders in its level-0 checks; HELIO and WHM here
    const bool resort = e->integrator != SWG_SYMBA && e->ndisc++ % RESORT_EVERY == 0;
    const SortedSet pl = pl_set(e, e->rh, e->vh, e->radius), tp = tp_set(e, e->trh, e->tvh);
    SWG_TRY(sorted_set_prep(c, pl, e->nsys, resort, e->dt));
    SWG_TRY(sorted_set_prep(c, tp, e->nsys, resort, e->dt));
    SWG_TRY(pltp_sorted_batched(c, true, pl, tp, e->tstatus, e->n_tsp, e->it_tsp, e->dt, 0, nullptr, nullptr, nullptr,
                                nullptr, e->tflag));
    k_apply_discard<<<grid_for(e->NTP, 256), 256, 0, c->stream>>>(e->NTP, e->tflag, e->tstatus, e->tlmask, e->trh,
                                                                   e->tvh, e->tvb, 0, e->tsys, e->toff, e->npl,
                                                                   e->ndiscard);
    return L(c, "apply_discard");
}

}  // namespace

// ======================================================================== C ABI
extern "C" {

int swg_ensemble_destroy(swg_ensemble *e);

int swg_ensemble_create(swg_ctx *c, int integrator, int32_t nsys, const int32_t *npl, const int32_t *ntp,
                        swg_ensemble **out) {
    if (!c || !out || nsys <= 0 || !npl || (integrator != SWG_WHM && integrator != SWG_HELIO && integrator != SWG_SYMBA))
        return SWG_ERR_ARG;
    int64_t NPL = 0, NTP = 0;
    for (int s = 0; s < nsys; s++) {
        const int32_t m = ntp ? ntp[s] : 0;
        if (npl[s] < 0 || m < 0) return SWG_ERR_ARG;
        NPL += npl[s];
        NTP += m;
    }
    if (NPL >= (int64_t)1 << 31 || NTP >= (int64_t)1 << 31) return SWG_ERR_ARG;
    swg_ensemble *e = new swg_ensemble();
    e->c = c;
    c->ensembles.push_back(e);
    e->integrator = integrator;
    e->nsys = nsys;
    e->NPL = NPL;
    e->NTP = NTP;
    e->h_npl.assign(npl, npl + nsys);
    e->h_ntp.assign(nsys, 0);
    if (ntp) e->h_ntp.assign(ntp, ntp + nsys);
    e->h_poff.assign(nsys + 1, 0);
    e->h_toff.assign(nsys + 1, 0);
    for (int s = 0; s < nsys; s++) {
        e->h_poff[s + 1] = e->h_poff[s] + e->h_npl[s];
        e->h_toff[s + 1] = e->h_toff[s] + e->h_ntp[s];
    }
    std::vector<int32_t> psys(NPL), tsys(NTP);
    for (int s = 0; s < nsys; s++) {
        std::fill(psys.begin() + e->h_poff[s], psys.begin() + e->h_poff[s + 1], s);
        std::fill(tsys.begin() + e->h_toff[s], tsys.begin() + e->h_toff[s + 1], s);
    }
    const size_t n = std::max<int64_t>(NPL, 1), m = std::max<int64_t>(NTP, 1), S = nsys;
    int rc = SWG_OK;
    int32_t **ps[] = {&e->npl, &e->ntp, &e->poff, &e->toff, &e->lfirst, &e->lany, &e->enc_steps};
    for (auto p : ps)
        if (rc == SWG_OK) rc = dalloc(c, p, S + 1);
    if (rc == SWG_OK) rc = dalloc(c, &e->seg_pp, 2 * S);
    if (rc == SWG_OK) rc = dalloc(c, &e->seg_pt, 2 * S);
    if (rc == SWG_OK) rc = dalloc(c, &e->GMcb, S);
    if (rc == SWG_OK) rc = dalloc(c, &e->dcb, CB_N * S);
    if (rc == SWG_OK) rc = dalloc(c, &e->eout, 9 * S);
    double **pd[] = {&e->rh, &e->vh, &e->vb, &e->ah, &e->rbeg, &e->rend};
    for (auto p : pd)
        if (rc == SWG_OK) rc = dalloc(c, p, 3 * n);
    double **pn[] = {&e->Gmass, &e->radius, &e->rhill, &e->renc};
    for (auto p : pn)
        if (rc == SWG_OK) rc = dalloc(c, p, n);
    int32_t **pi[] = {&e->psys, &e->status, &e->lmask, &e->levelg, &e->levelm, &e->nplenc, &e->ntpenc, &e->mark_pl};
    for (auto p : pi)
        if (rc == SWG_OK) rc = dalloc(c, p, n);
    double **td[] = {&e->trh, &e->tvh, &e->tvb, &e->tah};
    for (auto p : td)
        if (rc == SWG_OK) rc = dalloc(c, p, 3 * m);
    int32_t **ti[] = {&e->tsys, &e->tstatus, &e->tlmask, &e->tlevelg, &e->tlevelm, &e->tnplenc, &e->mark_tp};
    for (auto p : ti)
        if (rc == SWG_OK) rc = dalloc(c, p, m);
    if (rc == SWG_OK) rc = dalloc(c, &e->kA, 4 * n);
    if (rc == SWG_OK) {
        e->kB = e->kA + n;
        e->kA2 = e->kA + 2 * n;
        e->kB2 = e->kA + 3 * n;
    }
    if (rc == SWG_OK) rc = dalloc(c, &e->tperm, m);
    if (rc == SWG_OK) rc = dalloc(c, &e->eT, 3 * m);
    if (rc == SWG_OK) rc = dalloc(c, &e->eS, 3 * n);
    if (rc == SWG_OK) rc = dalloc(c, &e->perm, n);
    if (rc == SWG_OK) rc = dalloc(c, &e->head, 4);
    if (rc == SWG_OK) rc = dalloc(c, &e->head2, 4);
    if (rc == SWG_OK) rc = cuda_status(c, cudaStreamCreateWithFlags(&e->side, cudaStreamNonBlocking), "side stream");
    if (rc == SWG_OK) rc = cuda_status(c, cudaEventCreateWithFlags(&e->ev_fork, cudaEventDisableTiming), "event");
    if (rc == SWG_OK) rc = cuda_status(c, cudaEventCreateWithFlags(&e->ev_join, cudaEventDisableTiming), "event");
    if (rc == SWG_OK) rc = cuda_status(c, cudaEventCreateWithFlags(&e->ev_drift, cudaEventDisableTiming), "event");
    if (rc == SWG_OK) rc = cuda_status(c, cudaEventCreateWithFlags(&e->ev_split, cudaEventDisableTiming), "event");
    if (rc == SWG_OK && integrator == SWG_SYMBA) rc = dalloc(c, &e->enc_body, n);
    if (rc == SWG_OK) rc = dalloc(c, &e->rec_out, 4);
    if (rc == SWG_OK) rc = dalloc(c, &e->rec_resume, (size_t)REC_STATE * S);
    if (rc == SWG_OK) rc = dalloc(c, &e->rec_pend, S);
    if (rc == SWG_OK) rc = dalloc(c, &e->tflag, m);
    if (rc == SWG_OK) rc = dalloc(c, &e->ndiscard, 1);
    e->h_pend.assign(S, 0);
    e->coll_terms.assign(4 * (size_t)S, 0.0);
    if (rc == SWG_OK && integrator == SWG_HELIO && m > 0 && S > 1) {
        // two groups of systems with about equal pl-tp kick work (N_tp N_pl), split at a system
        double total = 0.0, cum = 0.0;
        for (int s = 0; s < S; s++) total += (double)e->h_ntp[s] * e->h_npl[s];
        int split = S;
        for (int s = 0; s < S; s++) {
            cum += (double)e->h_ntp[s] * e->h_npl[s];
            if (cum >= 0.5 * total) {
                split = s + 1;
                break;
            }
        }
        std::vector<int32_t> g(S);
        for (int s = 0; s < S; s++) g[s] = s >= split ? 1 : 0;
        e->tsplit = split < S ? e->h_toff[split] : m;
        rc = dalloc(c, &e->tgroup, S);
        if (rc == SWG_OK) rc = upload(c, e->tgroup, g);
        if (rc == SWG_OK)
            rc = cuda_status(c, cudaStreamCreateWithFlags(&e->side2, cudaStreamNonBlocking), "side stream");
        if (rc == SWG_OK) rc = cuda_status(c, cudaEventCreateWithFlags(&e->ev_g0, cudaEventDisableTiming), "event");
        if (rc == SWG_OK) rc = cuda_status(c, cudaEventCreateWithFlags(&e->ev_join2, cudaEventDisableTiming), "event");
    }
    if (integrator == SWG_SYMBA && rc == SWG_OK) rc = dalloc(c, &e->snap, 6 * n + 6 * m);
    if (integrator == SWG_WHM) {
        double **wd[] = {&e->eta, &e->muj, &e->ir3h, &e->ir3j};
        for (auto p : wd)
            if (rc == SWG_OK) rc = dalloc(c, p, n);
        if (rc == SWG_OK) rc = dalloc(c, &e->xj, 3 * n);
        if (rc == SWG_OK) rc = dalloc(c, &e->vj, 3 * n);
        if (rc == SWG_OK) rc = dalloc(c, &e->whm_ah0, 3 * S);
        if (rc == SWG_OK) rc = dalloc(c, &e->iflag, n);
        if (rc == SWG_OK) rc = dalloc(c, &e->whm_fail, 1);
    }
    if (rc == SWG_OK) rc = ensure(c, e->rows, sizeof(double) * 4 * n);
    if (rc == SWG_OK) {
        cudaError_t err = cudaMallocHost((void **)&e->h_flags, 64);
        if (err != cudaSuccess) rc = cuda_status(c, err, "cudaMallocHost");
    }
    if (rc == SWG_OK) rc = upload(c, e->npl, e->h_npl);
    if (rc == SWG_OK) rc = upload(c, e->ntp, e->h_ntp);
    if (rc == SWG_OK) rc = upload(c, e->poff, e->h_poff);
    if (rc == SWG_OK) rc = upload(c, e->toff, e->h_toff);
    if (rc == SWG_OK) rc = upload(c, e->psys, psys);
    if (rc == SWG_OK) rc = upload(c, e->tsys, tsys);
    if (rc == SWG_OK) rc = build_items(e);
    if (rc == SWG_OK) rc = cuda_status(c, cudaStreamSynchronize(c->stream), "create");
    if (rc != SWG_OK) {
        swg_ensemble_destroy(e);
        return rc;
    }
    *out = e;
    return SWG_OK;
}

int swg_ensemble_destroy(swg_ensemble *e) {
    if (!e) return SWG_OK;
    swg_ctx *c = e->c;
    if (c) {
        cudaStreamSynchronize(c->stream);
        auto it = std::find(c->ensembles.begin(), c->ensembles.end(), (void *)e);
        if (it != c->ensembles.end()) c->ensembles.erase(it);
    }
    void *ptrs[] = {e->npl, e->ntp, e->poff, e->toff, e->GMcb, e->dcb, e->lfirst, e->lany, e->seg_pp, e->seg_pt,
                    e->enc_steps, e->psys, e->rh, e->vh, e->vb, e->ah, e->rbeg, e->rend, e->Gmass, e->radius,
                    e->rhill, e->renc, e->status, e->lmask, e->levelg, e->levelm, e->nplenc, e->ntpenc, e->mark_pl,
                    e->tsys, e->trh, e->tvh, e->tvb, e->tah, e->tstatus, e->tlmask,
                    e->tlevelg, e->tlevelm, e->tnplenc, e->mark_tp, e->kA, e->eT, e->eS, e->perm, e->tbase, e->tperm, e->ttbase, e->ttiles, e->tbounds, e->it_tsp,
                    e->tiles, e->bounds, e->it_esp, e->head2, e->kit[0], e->kit[1], e->it_sym, e->sym_base, e->sym_part,
                    e->it_fpl, e->it_ftp, e->head, e->pp_l, e->pt_l, e->enc_pp.raw.ptr,
                    e->enc_pp.sort.ptr, e->enc_pp.counters.ptr, e->enc_pt.raw.ptr, e->enc_pt.sort.ptr,
                    e->enc_pt.counters.ptr, e->ext_pp, e->ext_pt, e->sas.ptr, e->rec_out, e->rec_resume, e->rec_pend, e->tflag, e->ndiscard, e->rec_scratch.ptr, e->rows.ptr, e->pair_terms.ptr, e->close_part.ptr, e->nplm, e->chunks, e->sys_chunks, e->chunk_part, e->eta, e->muj, e->xj, e->vj, e->ir3h, e->ir3j, e->whm_ah0, e->iflag, e->whm_fail, e->snap, e->eout};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (e->h_flags) cudaFreeHost(e->h_flags);
    if (e->side) cudaStreamSynchronize(e->side);
    if (e->graph) cudaGraphExecDestroy(e->graph);
    if (e->ev_fork) cudaEventDestroy(e->ev_fork);
    if (e->ev_join) cudaEventDestroy(e->ev_join);
    if (e->ev_drift) cudaEventDestroy(e->ev_drift);
    if (e->ev_split) cudaEventDestroy(e->ev_split);
    if (e->enc_body) cudaFree(e->enc_body);
    if (e->sym_iflag.ptr) cudaFree(e->sym_iflag.ptr);
    if (e->side) cudaStreamDestroy(e->side);
    if (e->side2) cudaStreamDestroy(e->side2);
    if (e->ev_g0) cudaEventDestroy(e->ev_g0);
    if (e->ev_join2) cudaEventDestroy(e->ev_join2);
    if (e->tgroup) cudaFree(e->tgroup);
    e->prof.release();
    delete e;
    return SWG_OK;
}

int swg_ensemble_set_cb(swg_ensemble *e, const double *GMcb, const double *Rcb) {
    if (!e || !GMcb) return SWG_ERR_ARG;
    for (int s = 0; s < e->nsys; s++)
        if (!(GMcb[s] > 0.0)) return SWG_ERR_ARG;
    e->h_GMcb.assign(GMcb, GMcb + e->nsys);
    e->h_Rcb.assign(e->nsys, 0.0);
    if (Rcb) e->h_Rcb.assign(Rcb, Rcb + e->nsys);
    e->cb_set = 1;
    SWG_TRY(upload(e->c, e->GMcb, e->h_GMcb));
    return cuda_status(e->c, cudaStreamSynchronize(e->c->stream), "set_cb");
}

int swg_ensemble_set_pl(swg_ensemble *e, const double *rh, const double *vh, const double *Gmass,
                        const double *radius, const double *rhill) {
    if (!e) return SWG_ERR_ARG;
    swg_ctx *c = e->c;
    const size_t n = e->NPL;
    if (n == 0) return SWG_OK;
    if (!rh || !vh || !Gmass || !radius || !rhill) return SWG_ERR_ARG;
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(e->rh, rh, 24 * n, cudaMemcpyHostToDevice, c->stream), "set_pl"));
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(e->vh, vh, 24 * n, cudaMemcpyHostToDevice, c->stream), "set_pl"));
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(e->Gmass, Gmass, 8 * n, cudaMemcpyHostToDevice, c->stream), "set_pl"));
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(e->radius, radius, 8 * n, cudaMemcpyHostToDevice, c->stream), "set_pl"));
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(e->rhill, rhill, 8 * n, cudaMemcpyHostToDevice, c->stream), "set_pl"));
    e->initialized = 0;
    return cuda_status(c, cudaStreamSynchronize(c->stream), "set_pl");
}

int swg_ensemble_set_tp(swg_ensemble *e, const double *rh, const double *vh) {
    if (!e) return SWG_ERR_ARG;
    swg_ctx *c = e->c;
    const size_t n = e->NTP;
    if (n == 0) return SWG_OK;
    if (!rh || !vh) return SWG_ERR_ARG;
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(e->trh, rh, 24 * n, cudaMemcpyHostToDevice, c->stream), "set_tp"));
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(e->tvh, vh, 24 * n, cudaMemcpyHostToDevice, c->stream), "set_tp"));
    e->initialized = 0;
    return cuda_status(c, cudaStreamSynchronize(c->stream), "set_tp");
}

int swg_ensemble_set_gmtiny(swg_ensemble *e, double gmtiny) {
    if (!e || !(gmtiny >= 0.0)) return SWG_ERR_ARG;
    e->gmtiny = gmtiny;
    e->initialized = 0;
    return SWG_OK;
}

int swg_ensemble_set_param(swg_ensemble *e, double dt, double rhscale, int lclose, int precision) {
    if (!e || !(dt > 0.0) || !(rhscale > 0.0) || (precision != SWG_FP64 && precision != SWG_MIXED))
        return SWG_ERR_ARG;
    reset_kick_plans(e);  // a captured step holds the old parameters; the kick kind may change
    e->dt = dt;
    e->rhscale = rhscale;
    e->lclose = lclose != 0;
    e->precision = precision;
    return SWG_OK;
}

int swg_ensemble_set_encounter_modes(swg_ensemble *e, int enc_plpl, int enc_pltp) {
    auto ok = [](int m) { return m == SWG_ENC_TRIANGULAR || m == SWG_ENC_SORTSWEEP; };
    if (!e || !ok(enc_plpl) || !ok(enc_pltp)) return SWG_ERR_ARG;
    if (e->integrator != SWG_SYMBA) return SWG_ERR_STATE;  // only SyMBA checks encounters
    e->enc_plpl = enc_plpl;
    e->enc_pltp = enc_pltp;
    return SWG_OK;
}

// helio_util_setup_initialize_system (helio_util.f90:14-43) for every system; bodies
// arrive sorted as the reference's initialize leaves them (by mass, descending)
int swg_ensemble_initialize(swg_ensemble *e) {
    if (!e || !e->cb_set || !(e->dt > 0.0)) return SWG_ERR_STATE;
    swg_ctx *c = e->c;
    e->coll_terms.assign(4 * (size_t)e->nsys, 0.0);
    std::vector<int32_t> ones(std::max(e->NPL, e->NTP), 1), first(e->nsys, 1);
    SWG_TRY(cuda_status(c, cudaMemsetAsync(e->status, 0, 4 * std::max<int64_t>(e->NPL, 1), c->stream), "init"));
    SWG_TRY(cuda_status(c, cudaMemsetAsync(e->tstatus, 0, 4 * std::max<int64_t>(e->NTP, 1), c->stream), "init"));
    if (e->NPL > 0)
        SWG_TRY(cuda_status(c, cudaMemcpyAsync(e->lmask, ones.data(), 4 * e->NPL, cudaMemcpyHostToDevice, c->stream),
                            "init"));
    if (e->NTP > 0)
        SWG_TRY(cuda_status(c, cudaMemcpyAsync(e->tlmask, ones.data(), 4 * e->NTP, cudaMemcpyHostToDevice, c->stream),
                            "init"));
    SWG_TRY(cuda_status(c, cudaMemsetAsync(e->dcb, 0, sizeof(double) * CB_N * e->nsys, c->stream), "init"));
    SWG_TRY(cuda_status(c, cudaMemsetAsync(e->enc_steps, 0, sizeof(int32_t) * e->nsys, c->stream), "init"));
    SWG_TRY(cuda_status(c, cudaMemsetAsync(e->rec_out, 0, sizeof(int32_t) * 4, c->stream), "init"));
    SWG_TRY(upload(c, e->lfirst, first));
    if (e->integrator == SWG_WHM) {  // whm_util_set_mu_eta_pl (whm_util.f90:175-198) per system
        std::vector<double> Gm(e->NPL), eta(e->NPL), muj(e->NPL);
        if (e->NPL > 0) {
            SWG_TRY(cuda_status(c, cudaMemcpyAsync(Gm.data(), e->Gmass, 8 * e->NPL, cudaMemcpyDeviceToHost, c->stream),
                                "init"));
            SWG_TRY(cuda_status(c, cudaStreamSynchronize(c->stream), "init"));
        }
        for (int s = 0; s < e->nsys; s++) {
            const int32_t o = e->h_poff[s], n = e->h_npl[s];
            if (n == 0) continue;
            eta[o] = e->h_GMcb[s] + Gm[o];
            muj[o] = eta[o];
            for (int i = 1; i < n; i++) {
                eta[o + i] = eta[o + i - 1] + Gm[o + i];
                muj[o + i] = e->h_GMcb[s] * eta[o + i] / eta[o + i - 1];
            }
        }
        SWG_TRY(upload(c, e->eta, eta));
        SWG_TRY(upload(c, e->muj, muj));
        SWG_TRY(cuda_status(c, cudaMemsetAsync(e->whm_fail, 0, sizeof(int32_t), c->stream), "init"));
        SWG_TRY(cuda_status(c, cudaStreamSynchronize(c->stream), "init"));
        e->whm_first = 1;
        e->t = 0.0;
        e->nchecks = 0;
        e->eager_steps = 0;
        if (e->graph) cudaGraphExecDestroy(e->graph);
        e->graph = nullptr;
        std::memset(e->stats, 0, sizeof(e->stats));
        e->initialized = 1;
        return SWG_OK;
    }
    // GMTINY (symba_util_set_renc and the nplm loop bounds; fixed at initialisation as in the
    // single-system path): the bodies of each system with Gmass >= gmtiny, which lead its block
    e->tiny = false;
    if (e->integrator == SWG_SYMBA && e->gmtiny > 0.0 && e->NPL > 0) {
        std::vector<double> Gm(e->NPL);
        SWG_TRY(cuda_status(c, cudaMemcpyAsync(Gm.data(), e->Gmass, 8 * e->NPL, cudaMemcpyDeviceToHost, c->stream),
                            "init"));
        SWG_TRY(cuda_status(c, cudaStreamSynchronize(c->stream), "init"));
        std::vector<int32_t> m(e->nsys, 0);
        for (int s = 0; s < e->nsys; s++) {
            for (int i = 0; i < e->h_npl[s]; i++) m[s] += !(Gm[e->h_poff[s] + i] < e->gmtiny);
            e->tiny = e->tiny || m[s] < e->h_npl[s];
        }
        if (e->tiny && e->enc_plpl == SWG_ENC_SORTSWEEP) {
            c->err = "GMTINY ensembles take TRIANGULAR pl-pl level-0 checks";
            return SWG_ERR_ARG;
        }
        if (!e->nplm) SWG_TRY(dalloc(c, &e->nplm, (size_t)e->nsys));
        SWG_TRY(upload(c, e->nplm, m));
    }
    reset_kick_plans(e);  // the pl-pl kernel depends on GMTINY
    SWG_TRY(vh2vb_pl(e, false));
    SWG_TRY(tp_misc(e, CB_VB, 0.0, 5, -1));  // tp vb = vh + the central body's vb
    e->t = 0.0;
    e->nchecks = 0;
    e->eager_steps = 0;
    if (e->graph) cudaGraphExecDestroy(e->graph);
    e->graph = nullptr;
    std::memset(e->stats, 0, sizeof(e->stats));
    e->initialized = 1;
    return cuda_status(c, cudaStreamSynchronize(c->stream), "init");
}

int swg_ensemble_step(swg_ensemble *e, int32_t nsteps) {
    if (!e || !e->initialized) return SWG_ERR_STATE;
    swg_ctx *c = e->c;
    e->h_flags[2] = 0;
    // A HELIO step takes no host decision (first-step flags live on the device), so after
    // one eager step (which also makes every lazy allocation and query) the step and its
    // discard scan are captured once as a CUDA graph and replayed.  SyMBA steps read the
    // encounter-list sizes on the host and run eagerly.
    const bool graphable = e->integrator != SWG_SYMBA && e->use_graph && !e->prof.on;
    for (int32_t k = 0; k < nsteps; k++) {
        if (graphable && e->eager_steps > 0) {
            if (!e->graph) {
                cudaGraph_t g = nullptr;
                const int64_t l0 = c->launches;
                SWG_TRY(cuda_status(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "capture"));
                int rc = e->integrator == SWG_WHM ? whm_ens_step(e, e->dt) : ens_step(e, e->dt);
                if (rc == SWG_OK) rc = discard_step(e);
                const cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
                SWG_TRY(rc);
                SWG_TRY(cuda_status(c, ce, "capture"));
                e->graph_launches = c->launches - l0;
                c->launches = l0;
                const cudaError_t ie = cudaGraphInstantiate(&e->graph, g, 0);
                cudaGraphDestroy(g);
                SWG_TRY(cuda_status(c, ie, "graph instantiate"));
            }
            SWG_TRY(cuda_status(c, cudaGraphLaunch(e->graph, c->stream), "graph launch"));
            c->launches += e->graph_launches;
        } else {
            SWG_TRY(e->integrator == SWG_WHM ? whm_ens_step(e, e->dt) : ens_step(e, e->dt));
            SWG_TRY(discard_step(e));
            e->eager_steps++;
        }
        if (e->h_flags[2] != 0) {  // recursion status of an earlier step, seen at a sync point
            e->c->err = "SyMBA local time step too small";
            return e->h_flags[2];
        }
        e->t += e->dt;
    }
    if (e->integrator == SWG_WHM && e->NPL > 0)
        SWG_TRY(cuda_status(c, cudaMemcpyAsync(e->h_flags + 3, e->whm_fail, sizeof(int32_t), cudaMemcpyDeviceToHost,
                                               c->stream),
                            "flag"));
    SWG_TRY(cuda_status(e->c, cudaStreamSynchronize(e->c->stream), "step"));
    if (e->h_flags[2] != 0) {
        e->c->err = "SyMBA local time step too small";
        return e->h_flags[2];
    }
    if (e->integrator == SWG_WHM && e->NPL > 0 && e->h_flags[3] != 0) {
        e->c->err = "Danby drift failed for a massive body (WHM stops the run)";
        return SWG_ERR_DRIFT;
    }
    return SWG_OK;
}

int swg_ensemble_get_pl_masses(swg_ensemble *e, double *Gmass, double *radius, double *rhill) {
    if (!e) return SWG_ERR_ARG;
    swg_ctx *c = e->c;
    const size_t n = e->NPL;
    if (n == 0) return SWG_OK;
    const std::pair<double *, const double *> xs[] = {{Gmass, e->Gmass}, {radius, e->radius}, {rhill, e->rhill}};
    for (const auto &x : xs)
        if (x.first)
            SWG_TRY(cuda_status(c, cudaMemcpyAsync(x.first, x.second, 8 * n, cudaMemcpyDeviceToHost, c->stream),
                                "get_pl_masses"));
    return cuda_status(c, cudaStreamSynchronize(c->stream), "get_pl_masses");
}

int swg_ensemble_get_pl(swg_ensemble *e, double *rh, double *vh, int32_t *status) {
    if (!e) return SWG_ERR_ARG;
    swg_ctx *c = e->c;
    const size_t n = e->NPL;
    if (n == 0) return SWG_OK;
    if (rh) SWG_TRY(cuda_status(c, cudaMemcpyAsync(rh, e->rh, 24 * n, cudaMemcpyDeviceToHost, c->stream), "get_pl"));
    if (vh) SWG_TRY(cuda_status(c, cudaMemcpyAsync(vh, e->vh, 24 * n, cudaMemcpyDeviceToHost, c->stream), "get_pl"));
    if (status)
        SWG_TRY(cuda_status(c, cudaMemcpyAsync(status, e->status, 4 * n, cudaMemcpyDeviceToHost, c->stream), "get_pl"));
    return cuda_status(c, cudaStreamSynchronize(c->stream), "get_pl");
}

int swg_ensemble_get_tp(swg_ensemble *e, double *rh, double *vh, int32_t *status) {
    if (!e) return SWG_ERR_ARG;
    swg_ctx *c = e->c;
    const size_t n = e->NTP;
    if (n == 0) return SWG_OK;
    if (rh) SWG_TRY(cuda_status(c, cudaMemcpyAsync(rh, e->trh, 24 * n, cudaMemcpyDeviceToHost, c->stream), "get_tp"));
    if (vh) SWG_TRY(cuda_status(c, cudaMemcpyAsync(vh, e->tvh, 24 * n, cudaMemcpyDeviceToHost, c->stream), "get_tp"));
    if (status)
        SWG_TRY(cuda_status(c, cudaMemcpyAsync(status, e->tstatus, 4 * n, cudaMemcpyDeviceToHost, c->stream), "get_tp"));
    return cuda_status(c, cudaStreamSynchronize(c->stream), "get_tp");
}

int swg_ensemble_energy(swg_ensemble *e, double *out) {
    if (!e || !out) return SWG_ERR_ARG;
    swg_ctx *c = e->c;
    const int64_t n = std::max<int64_t>(e->NPL, 1);
    double *rows = (double *)e->rows.ptr, *rb = rows + n;
    // the totals kernel also writes rb, which the rows need: totals, rows, totals
    k_ens_energy_final<<<e->nsys, RB, 0, c->stream>>>(e->poff, e->npl, e->rh, e->vh, e->vb, e->Gmass, e->radius,
                                                      e->status, e->GMcb, e->lclose, e->integrator == SWG_WHM, rows, rb,
                                                      e->eout);
    SWG_TRY(L(c, "ens_energy_rb"));
    if (e->NPL > 0) {
        k_ens_energy_rows<<<grid_for(e->NPL, 128), 128, 0, c->stream>>>(e->NPL, e->psys, e->poff, e->npl, rb,
                                                                         e->Gmass, e->status, rows);
        SWG_TRY(L(c, "ens_energy_rows"));
    }
    k_ens_energy_final<<<e->nsys, RB, 0, c->stream>>>(e->poff, e->npl, e->rh, e->vh, e->vb, e->Gmass, e->radius,
                                                      e->status, e->GMcb, e->lclose, e->integrator == SWG_WHM, rows, rb,
                                                      e->eout);
    SWG_TRY(L(c, "ens_energy_final"));
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(out, e->eout, sizeof(double) * 9 * e->nsys, cudaMemcpyDeviceToHost,
                                           c->stream),
                        "energy"));
    return cuda_status(c, cudaStreamSynchronize(c->stream), "energy");
}

int swg_ensemble_collision_terms(swg_ensemble *e, double *out) {
    if (!e || !out) return SWG_ERR_ARG;
    for (size_t k = 0; k < e->coll_terms.size(); k++) out[k] = e->coll_terms[k];
    return SWG_OK;
}

int swg_ensemble_stats(swg_ensemble *e, int64_t *out) {
    if (!e || !out) return SWG_ERR_ARG;
    swg_ctx *c = e->c;
    std::vector<int32_t> steps(e->nsys);
    int32_t dev[4];
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(steps.data(), e->enc_steps, 4 * e->nsys, cudaMemcpyDeviceToHost, c->stream),
                        "stats"));
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(dev, e->rec_out, sizeof(dev), cudaMemcpyDeviceToHost, c->stream), "stats"));
    SWG_TRY(cuda_status(c, cudaStreamSynchronize(c->stream), "stats"));
    int64_t tot = 0;
    for (int32_t v : steps) tot += v;
    unsigned long long nd = 0;
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(&nd, e->ndiscard, sizeof(nd), cudaMemcpyDeviceToHost, c->stream), "stats"));
    SWG_TRY(cuda_status(c, cudaStreamSynchronize(c->stream), "stats"));
    e->stats[0] = tot;
    e->stats[1] = dev[1];
    e->stats[5] = dev[2];
    std::memcpy(out, e->stats, sizeof(e->stats));
    out[4] += (int64_t)nd;
    return SWG_OK;
}

// Level-0 encounter list of system `sys` from the last step, local 1-based indices.
int swg_ensemble_plpl_list(swg_ensemble *e, int32_t sys, int64_t cap, int64_t *n, int32_t *i1, int32_t *i2) {
    if (!e || !n || sys < 0 || sys >= e->nsys) return SWG_ERR_ARG;
    swg_ctx *c = e->c;
    int32_t seg[2] = {0, 0};
    *n = 0;
    if (e->pp_n > 0) {
        SWG_TRY(cuda_status(c, cudaMemcpyAsync(seg, e->seg_pp + 2 * sys, sizeof(seg), cudaMemcpyDeviceToHost, c->stream),
                            "list"));
        SWG_TRY(cuda_status(c, cudaStreamSynchronize(c->stream), "list"));
    }
    *n = seg[1];
    if (seg[1] > cap) return SWG_ERR_CAPACITY;
    if (seg[1] == 0) return SWG_OK;
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(i1, e->pp_l + seg[0], 4 * (size_t)seg[1], cudaMemcpyDeviceToHost, c->stream),
                        "list"));
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(i2, e->pp_l + e->pp_cap + seg[0], 4 * (size_t)seg[1],
                                           cudaMemcpyDeviceToHost, c->stream),
                        "list"));
    SWG_TRY(cuda_status(c, cudaStreamSynchronize(c->stream), "list"));
    const int32_t o = e->h_poff[sys];
    for (int32_t k = 0; k < seg[1]; k++) {
        i1[k] -= o;
        i2[k] -= o;
    }
    return SWG_OK;
}

int swg_ensemble_set_state(swg_ensemble *e, const double *rh, const double *vh, const double *trh, const double *tvh) {
    if (!e || !e->initialized) return SWG_ERR_STATE;
    swg_ctx *c = e->c;
    const size_t n = e->NPL, m = e->NTP;
    if (n && rh) SWG_TRY(cuda_status(c, cudaMemcpyAsync(e->rh, rh, 24 * n, cudaMemcpyHostToDevice, c->stream), "state"));
    if (n && vh) SWG_TRY(cuda_status(c, cudaMemcpyAsync(e->vh, vh, 24 * n, cudaMemcpyHostToDevice, c->stream), "state"));
    if (m && trh)
        SWG_TRY(cuda_status(c, cudaMemcpyAsync(e->trh, trh, 24 * m, cudaMemcpyHostToDevice, c->stream), "state"));
    if (m && tvh)
        SWG_TRY(cuda_status(c, cudaMemcpyAsync(e->tvh, tvh, 24 * m, cudaMemcpyHostToDevice, c->stream), "state"));
    return SWG_OK;
}

int swg_ensemble_reset_first_step(swg_ensemble *e) {
    if (!e || !e->initialized) return SWG_ERR_STATE;
    swg_ctx *c = e->c;
    SWG_TRY(upload(c, e->lfirst, std::vector<int32_t>(e->nsys, 1)));
    e->whm_first = 1;
    // the captured step graph holds the steps after the first (WHM's first step differs on the host)
    SWG_TRY(cuda_status(c, cudaStreamSynchronize(c->stream), "first step"));
    if (e->graph) cudaGraphExecDestroy(e->graph);
    e->graph = nullptr;
    e->eager_steps = 0;
    return SWG_OK;
}

int swg_ensemble_get_state_async(swg_ensemble *e, double *rh, double *vh, double *trh, double *tvh) {
    if (!e) return SWG_ERR_ARG;
    swg_ctx *c = e->c;
    const size_t n = e->NPL, m = e->NTP;
    if (n && rh) SWG_TRY(cuda_status(c, cudaMemcpyAsync(rh, e->rh, 24 * n, cudaMemcpyDeviceToHost, c->stream), "state"));
    if (n && vh) SWG_TRY(cuda_status(c, cudaMemcpyAsync(vh, e->vh, 24 * n, cudaMemcpyDeviceToHost, c->stream), "state"));
    if (m && trh)
        SWG_TRY(cuda_status(c, cudaMemcpyAsync(trh, e->trh, 24 * m, cudaMemcpyDeviceToHost, c->stream), "state"));
    if (m && tvh)
        SWG_TRY(cuda_status(c, cudaMemcpyAsync(tvh, e->tvh, 24 * m, cudaMemcpyDeviceToHost, c->stream), "state"));
    return SWG_OK;
}

int swg_ensemble_use_graphs(swg_ensemble *e, int enable) {
    if (!e) return SWG_ERR_ARG;
    e->use_graph = enable != 0;
    return SWG_OK;
}

int swg_ensemble_getacch_int_pl(swg_ensemble *e, double *acc) {
    if (!e || !acc) return SWG_ERR_ARG;
    if (e->NPL == 0) return SWG_OK;
    swg_ctx *c = e->c;
    SWG_TRY(accel_int_pl(e, e->head));
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(acc, e->ah, sizeof(double) * 3 * e->NPL, cudaMemcpyDeviceToHost, c->stream),
                        "getacch"));
    return cuda_status(c, cudaStreamSynchronize(c->stream), "getacch");
}

int swg_ensemble_set_kick_variant(swg_ensemble *e, int variant) {
    if (!e || variant < -1 || variant >= KICK_NVARIANT) return SWG_ERR_ARG;
    SWG_TRY(cuda_status(e->c, cudaStreamSynchronize(e->c->stream), "kick variant"));
    e->force_variant = variant;
    reset_kick_plans(e);
    return SWG_OK;
}

int swg_ensemble_kick_variant(swg_ensemble *e, int kind, int *variant) {
    if (!e || !variant || kind < 0 || kind > 5) return SWG_ERR_ARG;
    if (kind == 5)
        *variant = e->it_sym ? e->sym_group : -1;
    else if (kind == 2)
        *variant = e->it_sym ? e->sym_strip : -1;
    else if (kind == 3)
        *variant = e->it_sym ? e->sym_warps : -1;
    else if (kind == 4)
        *variant = e->it_sym ? e->sym_tile : -1;
    else
        *variant = e->kv[kind];
    return SWG_OK;
}

int swg_ensemble_set_kick_strip(swg_ensemble *e, int strip) {
    if (!e || !(strip == 0 || strip == 1 || strip == 2 || strip == 4 || strip == 8 || strip == 16))
        return SWG_ERR_ARG;
    SWG_TRY(cuda_status(e->c, cudaStreamSynchronize(e->c->stream), "kick strip"));
    e->force_strip = strip;
    if (e->it_sym) cudaFree(e->it_sym);
    e->it_sym = nullptr;
    e->n_sym = 0;
    reset_kick_plans(e);
    return SWG_OK;
}

int swg_ensemble_set_kick_warps(swg_ensemble *e, int warps) {
    if (!e || !(warps == 0 || warps == 1 || warps == 2 || warps == 4)) return SWG_ERR_ARG;
    SWG_TRY(cuda_status(e->c, cudaStreamSynchronize(e->c->stream), "kick warps"));
    e->force_warps = warps;
    if (e->it_sym) cudaFree(e->it_sym);
    e->it_sym = nullptr;
    e->n_sym = 0;
    reset_kick_plans(e);
    return SWG_OK;
}

int swg_ensemble_set_kick_tile(swg_ensemble *e, int tile) {
    if (!e || !(tile == 0 || tile == 64 || tile == 128)) return SWG_ERR_ARG;
    SWG_TRY(cuda_status(e->c, cudaStreamSynchronize(e->c->stream), "kick tile"));
    e->force_tile = tile;
    if (e->it_sym) cudaFree(e->it_sym);
    e->it_sym = nullptr;
    e->n_sym = 0;
    reset_kick_plans(e);
    return SWG_OK;
}

int swg_ensemble_set_kick_group(swg_ensemble *e, int group) {
    if (!e || !(group == 0 || group == 1 || group == 2 || group == 4)) return SWG_ERR_ARG;
    SWG_TRY(cuda_status(e->c, cudaStreamSynchronize(e->c->stream), "kick group"));
    e->force_group = group;
    if (e->it_sym) cudaFree(e->it_sym);
    e->it_sym = nullptr;
    e->n_sym = 0;
    reset_kick_plans(e);
    return SWG_OK;
}

int swg_ensemble_profile(swg_ensemble *e, int enable) {
    if (!e) return SWG_ERR_ARG;
    e->prof.on = enable != 0;
    e->prof.n = 0;
    return SWG_OK;
}

int swg_ensemble_profile_read(swg_ensemble *e, double *out) {
    if (!e || !out) return SWG_ERR_ARG;
    SWG_TRY(cuda_status(e->c, cudaStreamSynchronize(e->c->stream), "profile"));
    e->prof.read(out, PROF_NCLS);
    return SWG_OK;
}

}  // extern "C"
