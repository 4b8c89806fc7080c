// system.cu -- device-resident n-body system and the WHM / HELIO / SyMBA step loops.
//
// Host C++ here plays the role of the reference's type-bound procedures
// (whm_step.f90, helio_step.f90, symba_step.f90): it orders kernels on the
// context's stream and keeps every array in HBM between steps.  The host only
// waits where the reference makes a data-dependent decision: after the level-0
// encounter check (interp vs plain HELIO step) and, inside the SyMBA
// recursion, on the "any deeper encounter" flag of each sub-step.
//
// O(N) serial sums of the reference (the Sun's barycentric momentum in
// helio_drift_linear_pl, vh2vb / vb2vh, WHM Jacobi prefix sums) run in one
// thread in the reference's index order when the kick precision is FP64, so the
// FP64 path reproduces the serial reference loop bit for bit; in the mixed path
// they use a fixed-order block reduction.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "drift_impl.cuh"
#include "swg_internal.cuh"
#include "symba_dev.cuh"

using namespace swg;
using namespace swg::sdev;


// Radius-sorted pl and tp sets of one system, for its pl-tp level-0 check and close-approach
// discard scan (the ensemble's radius-sorted kernels run with one system): the radial orders,
// float copies and 32-body sub-tile bounds (encounter_sorted.cu), the 64-body bound tiles and
// the tp receiver items.  Built at the first use (npl and ntp are fixed for the system's life).
struct SortedOne {
    int32_t *meta = nullptr;  // [0] 0 (first body and first tile of each set), [1] npl, [2] ntp
    int32_t *pperm = nullptr, *tperm = nullptr;
    float4 *pF = nullptr, *tF = nullptr, *pbounds = nullptr, *tbounds = nullptr;
    int2 *ptiles = nullptr, *ttiles = nullptr;
    int4 *items = nullptr;
    int nitems = 0, nptiles = 0, nttiles = 0, pchunk = 0;  // pchunk: pl sub-tiles per item
    int64_t npl_prep = 0, ntp_prep = 0;  // preparations so far: the pl order is refreshed at every
                                         // 8th, the tp order at every 32nd (and at the first)
    void release() {
        void *ptrs[] = {meta, pperm, tperm, pF, tF, pbounds, tbounds, ptiles, ttiles, items};
        for (void *p : ptrs)
            if (p) cudaFree(p);
    }
};

struct swg_system {
    swg_ctx *c = nullptr;
    int integrator = SWG_HELIO;
    int32_t npl = 0, ntp = 0, nplm = 0;
    double GMcb = 0, Rcb = 0;
    double dt = 0, rhscale = 6.5, gmtiny = 0;
    int loop_mode = 0, enc_plpl = 0, enc_pltp = 0, lclose = 0, precision = SWG_FP64;
    int lfirst_pl = 1, lfirst_tp = 1, lfirstkick = 1, irec = -1, initialized = 0;
    double t = 0;
    // massive bodies
    double *rh = nullptr, *vh = nullptr, *vb = nullptr, *ah = nullptr, *rbeg = nullptr, *rend = nullptr;
    double *Gmass = nullptr, *radius = nullptr, *rhill = nullptr;
    double *xj = nullptr, *vj = nullptr, *eta = nullptr, *muj = nullptr, *ir3h = nullptr, *ir3j = nullptr;
    int32_t *status = nullptr, *lmask = nullptr, *levelg = nullptr, *levelm = nullptr, *nplenc = nullptr,
            *ntpenc = nullptr, *iflag = nullptr;
    // test particles
    double *trh = nullptr, *tvh = nullptr, *tvb = nullptr, *tah = nullptr;
    int32_t *tstatus = nullptr, *tlmask = nullptr, *tlevelg = nullptr, *tlevelm = nullptr, *tnplenc = nullptr,
            *tiflag = nullptr;
    double *dcb = nullptr;  // CB_N doubles
    // encounter lists (SyMBA): i1, i2, lvdotr, status, level
    int32_t *plpl_l = nullptr, *pltp_l = nullptr;  // 5 * cap int32 each
    int64_t plpl_n = 0, pltp_n = 0, plpl_cap = 0, pltp_cap = 0;
    EncWork enc, enc2;
    // scratch
    DevBuf kick_scratch, kick_scratch_tp, pair_scratch, flags, red;
    // SyMBA: the level-0 checks and the test particles' half-steps run on a second stream
    // beside the massive bodies' (events: 0 opening ready, 1 tp opening done, 2 closing
    // ready, 3 central-body drift ready, 4 tp closing done, 5 level-0 lists ready)
    cudaStream_t side = nullptr, side2 = nullptr;  // side2: the pl-tp check beside the pl-pl one on side
    cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    DevBuf snap;  // the start-of-step rh, vb, trh, tvb that the overlapped level-0 checks read
    int32_t *h_flags = nullptr;  // pinned: [0] lencounter, [1] nfail, [2] recursion status, [3] deepest level,
                                 // [4] collision pending
    int32_t *mark_pl = nullptr, *mark_tp = nullptr, *rec_out = nullptr, *rec_resume = nullptr;
    DevBuf rec_scratch;
    DevBuf discard_scratch;                 // float copies of the close-approach scan
    DevBuf chunk_buf;                       // mixed path: chunk table, system range, chunk partials
    int nchunks = 0;
    int32_t *tflag = nullptr;               // tp flagged by the scan
    unsigned long long *ndiscard = nullptr; // tp removed by the scan
    int64_t stats[6] = {0, 0, 0, 0, 0, 0};
    double E_collisions = 0.0, L_escape[3] = {0.0, 0.0, 0.0};  // collision bookkeeping (G*m units)
    double rec_dt = 0.0;                                        // step of the running recursion
    StepProfile prof;  // optional CUDA-event profile per kernel class (PROF_*)
    SortedOne *srt = nullptr;  // radius-sorted sets of the pl-tp check and discard scan
};

namespace {

inline int grid_for(int64_t n, int bs) { return (int)std::max<int64_t>(1, (n + bs - 1) / bs); }

template <typename T>
int dalloc(swg_ctx *c, T **p, size_t n) {
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
    if (e != cudaSuccess) {
        c->err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
        return SWG_ERR_NOMEM;
    }
    cudaMemsetAsync(*p, 0, n * sizeof(T), c->stream);
    return SWG_OK;
}


// One-block kernels over a single system's arrays (block-wide bodies in symba_dev.cuh).
__global__ void __launch_bounds__(RB) k_lindrift_pl(int npl, const double *__restrict__ Gm,
                                                    const double *__restrict__ vb, const int32_t *__restrict__ lmask,
                                                    double GMcb, double *rh, double dt, double *dcb, int slot,
                                                    int exact) {
    __shared__ SumScratch sh;
    blk_lindrift_pl(npl, Gm, vb, lmask, GMcb, rh, dt, dcb, slot, exact, sh);
}
__global__ void __launch_bounds__(RB) k_vh2vb_pl(int npl, const double *__restrict__ Gm,
                                                 const double *__restrict__ vh, double *vb, double GMcb, double *dcb,
                                                 int exact) {
    __shared__ SumScratch sh;
    blk_vh2vb_pl(npl, Gm, vh, vb, GMcb, dcb, exact, sh);
}
__global__ void __launch_bounds__(RB) k_vb2vh_pl(int npl, const double *__restrict__ Gm,
                                                 const double *__restrict__ vb, const int32_t *__restrict__ status,
                                                 double *vh, double GMcb, double *dcb, int exact) {
    __shared__ SumScratch sh;
    blk_vb2vh_pl(npl, Gm, vb, status, vh, GMcb, dcb, exact, sh);
}

// test particles: mode 0 vh2vb(vbcb=-pt) ; 1 vb2vh(vbcb=-pt) ; 2 lindrift rh += pt*dt ;
// 3 lindrift then vb2vh (end of step) ; 4 vh2vb then lindrift (start of step) ;
// 5 heliocentric to barycentric velocity with the central body's vb (initialisation)
__global__ void k_tp_misc(int ntp, const int32_t *__restrict__ tlmask, double *trh, double *tvh, double *tvb,
                          const double *__restrict__ dcb, int slot, double dt, int mode) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ntp || !tlmask[i]) return;
    for (int d = 0; d < 3; d++) {
        const double pt = dcb[slot + d];
        const double vbcb = -pt;
        if (mode == 0 || mode == 4) tvb[3 * i + d] = tvh[3 * i + d] + vbcb;
        if (mode == 2 || mode == 3 || mode == 4) trh[3 * i + d] = trh[3 * i + d] + pt * dt;
        if (mode == 1 || mode == 3) tvh[3 * i + d] = tvb[3 * i + d] - vbcb;
        if (mode == 5) tvb[3 * i + d] = tvh[3 * i + d] + dcb[slot + d];
    }
}


// symba_kick_getacch_tp add-back loop (symba_kick.f90:104-118), list order
__global__ void k_pltp_addback(int64_t n, const int32_t *__restrict__ i1, const int32_t *__restrict__ i2,
                               const int32_t *__restrict__ tlmask, const double *__restrict__ trh,
                               const double *__restrict__ rp, const double *__restrict__ Gm, double *tah) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    for (int64_t k = 0; k < n; k++) {
        const int i = i1[k] - 1, j = i2[k] - 1;
        if (!tlmask[j]) continue;
        const double dx = trh[3 * j + 0] - rp[3 * i + 0];
        const double dy = trh[3 * j + 1] - rp[3 * i + 1];
        const double dz = trh[3 * j + 2] - rp[3 * i + 2];
        const double rjj = dx * dx + dy * dy + dz * dz;
        const double fac = Gm[i] / (rjj * sqrt(rjj));
        tah[3 * j + 0] = tah[3 * j + 0] + fac * dx;
        tah[3 * j + 1] = tah[3 * j + 1] + fac * dy;
        tah[3 * j + 2] = tah[3 * j + 2] + fac * dz;
    }
}



// The same add-back for short lists (n <= ADDBACK_SMALL), one block, same bits: thread k
// evaluates pair k, then the thread holding a test particle's first pair adds that
// particle's terms in list order.
constexpr int ADDBACK_SMALL = 256;
__global__ void __launch_bounds__(ADDBACK_SMALL) k_pltp_addback_small(int n, const int32_t *__restrict__ i1,
                                                                     const int32_t *__restrict__ i2,
                                                                     const int32_t *__restrict__ tlmask,
                                                                     const double *__restrict__ trh,
                                                                     const double *__restrict__ rp,
                                                                     const double *__restrict__ Gm, double *tah) {
    __shared__ double t[ADDBACK_SMALL][3];
    __shared__ int sj[ADDBACK_SMALL];
    __shared__ unsigned char ok[ADDBACK_SMALL];
    const int k = threadIdx.x;
    if (k < n) {
        const int i = i1[k] - 1, j = i2[k] - 1;
        sj[k] = j;
        ok[k] = tlmask[j] != 0;
        if (ok[k]) {
            const double dx = trh[3 * j + 0] - rp[3 * i + 0];
            const double dy = trh[3 * j + 1] - rp[3 * i + 1];
            const double dz = trh[3 * j + 2] - rp[3 * i + 2];
            const double rjj = dx * dx + dy * dy + dz * dz;
            const double fac = Gm[i] / (rjj * sqrt(rjj));
            t[k][0] = fac * dx;
            t[k][1] = fac * dy;
            t[k][2] = fac * dz;
        }
    }
    __syncthreads();
    if (k >= n || !ok[k]) return;
    const int j = sj[k];
    for (int p = 0; p < k; p++)
        if (sj[p] == j) return;  // not the particle's first pair
    double x = tah[3 * j + 0], y = tah[3 * j + 1], z = tah[3 * j + 2];
    for (int p = k; p < n; p++) {
        if (sj[p] != j || !ok[p]) continue;
        x = x + t[p][0];
        y = y + t[p][1];
        z = z + t[p][2];
    }
    tah[3 * j + 0] = x;
    tah[3 * j + 1] = y;
    tah[3 * j + 2] = z;
}

// The whole SyMBA recursion of one step, one block (blk_symba_recursion).
__global__ void __launch_bounds__(RECT) k_symba_recursion(RecArgs a) {
    if (threadIdx.x == 0) a.out[0] = 0;
    blk_symba_recursion(a);
}

// energy diagnostic: potential rows (one thread per row) and the one-block totals
__global__ void k_energy_rows(int n, const double *rb, const double *Gm, const int32_t *status, double *rows) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) rows[i] = d_energy_row(i, n, rb, Gm, status);
}
__global__ void __launch_bounds__(RB) k_energy_final(int n, int whm, const double *rh, const double *vh,
                                                     const double *vbin, const double *Gm, const double *radius,
                                                     const int32_t *status, double GMcb, int lclose,
                                                     const double *rows, double *rb, double *out) {
    __shared__ SumScratch sh;
    blk_energy_final(n, whm, rh, vh, vbin, Gm, radius, status, GMcb, lclose, rows, rb, out, sh);
}

// ---- WHM coordinate kernels and accelerations (block device code in symba_dev.cuh)
__global__ void k_whm_h2j(int n, const double *Gm, const double *eta, const double *rh, const double *vh, double *xj,
                          double *vj, int exact) {
    __shared__ WhmScratch sh;
    blk_whm_h2j(n, Gm, eta, rh, vh, xj, vj, sh, exact);
}
__global__ void k_whm_j2h(int n, const double *Gm, const double *eta, const double *xj, const double *vj, double *rh,
                          double *vh, int exact) {
    __shared__ WhmScratch sh;
    blk_whm_j2h(n, Gm, eta, xj, vj, rh, vh, sh, exact);
}
__global__ void k_whm_vh2vj(int n, const double *Gm, const double *eta, const double *vh, double *vj, int exact) {
    __shared__ WhmScratch sh;
    blk_whm_vh2vj(n, Gm, eta, vh, vj, sh, exact);
}
__global__ void k_whm_accel_pl(int n, const double *Gm, double GMcb, const double *rh, const double *xj,
                               const int32_t *lmask, double *ir3h, double *ir3j, double *ah, int exact) {
    __shared__ WhmScratch sh;
    blk_whm_accel_pl(n, Gm, GMcb, rh, xj, lmask, ir3h, ir3j, ah, sh, exact);
}
// whm_kick_getacch_tp ah0 part (:70-122): tah += ah0(rp) for masked tp ; zero first when requested
__global__ void k_whm_tp_ah0(int ntp, int npl, const double *Gm, const double *rp, const int32_t *tlmask, double *tah,
                             int zero, int exact) {
    __shared__ WhmScratch sh;
    __shared__ double s_ah0[3];
    blk_whm_ah0(Gm, rp, npl, s_ah0, sh, exact);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ntp; i += gridDim.x * blockDim.x) {
        if (!tlmask[i]) continue;
        for (int d = 0; d < 3; d++) tah[3 * i + d] = (zero ? 0.0 : tah[3 * i + d]) + s_ah0[d];
    }
}
__global__ void k_any_nonzero(int n, const int32_t *v, int32_t *flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && v[i] != 0) atomicOr(flag, 1);
}
__global__ void k_whm_drift_status(int n, const int32_t *iflag, int32_t *status, int32_t *lmask) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && iflag[i] != 0) {
        status[i] = ST_DISCARDED_DRIFTERR;
        lmask[i] = 0;
    }
}


}  // namespace

// ======================================================================== host side
namespace {

int L(swg_ctx *c, const char *what) {
    c->launches++;
    return launch_status(c, what);
}

bool exact(const swg_system *s) { return s->precision == SWG_FP64; }

int pair_scratch(swg_system *s, double **p) {
    SWG_TRY(ensure(s->c, s->pair_scratch, sizeof(double) * 6 * (size_t)std::max(1, s->npl)));
    *p = (double *)s->pair_scratch.ptr;
    return SWG_OK;
}

// pl-pl interaction accelerations (swiftest_kick.f90:12-43 / symba_kick.f90:14-33), acc starts at zero
int accel_int_pl(swg_system *s, int acc_is_zero) {
    swg_ctx *c = s->c;
    const bool symba = s->integrator == SWG_SYMBA;
    const double *rad = (symba || s->lclose) ? s->radius : nullptr;
    const int32_t nplm = symba ? s->nplm : s->npl;
    if (s->precision == SWG_MIXED && nplm == s->npl && kick_sym_single_ok(s->npl, c->num_sms))
        return kick_mixed_sym_single(c, s->npl, s->rh, s->Gmass, rad, s->ah, acc_is_zero);
    if (s->precision == SWG_MIXED) {
        const int nch = kick_mixed_chunks(c, s->npl, s->npl);
        SWG_TRY(ensure_kick_scratch(c, s->kick_scratch, kick_mixed_scratch_bytes(s->npl, s->npl, nch)));
        return kick_mixed_launch(c, false, s->npl, s->npl, nplm, s->rh, s->rh, s->Gmass, rad, nullptr, s->ah,
                                 acc_is_zero, nch, s->kick_scratch.ptr);
    }
    // flat, or triangular with GMTINY bodies dominating -> symmetric (split) sums
    const int mode = (s->loop_mode == 1 || (s->npl - nplm) > nplm) ? KICK_SPLIT : KICK_DIRECT;
    return kick_plpl_fp64(c, s->npl, nplm, s->rh, s->Gmass, rad, s->ah, mode, acc_is_zero);
}

// helio_kick_vb_pl (helio_kick.f90:91-132) with symba_kick_getacch_pl (symba_kick.f90:36-76);
// copy_r: record the positions as the step's start (lbeg) or end positions for the test
// particles' kick (a caller that already copied them passes false)
// (have_acc: the pair accelerations are already in ah)
int kick_vb_pl(swg_system *s, double dt, int lbeg, bool copy_r = true, bool have_acc = false) {
    swg_ctx *c = s->c;
    if (s->npl == 0) return SWG_OK;
    if (!have_acc) {
        ProfScope ps(s->prof, s->c->stream, PROF_KICK_PL);
        SWG_TRY(accel_int_pl(s, 1));
    }
    if (s->integrator == SWG_SYMBA && s->plpl_n > 0) {
        double *scr;
        SWG_TRY(pair_scratch(s, &scr));
        SWG_TRY(kick_pairs(c, s->npl, s->plpl_n, nullptr, s->plpl_l, s->plpl_l + s->plpl_cap, s->rh, s->Gmass,
                           s->radius, s->ah, -1.0, scr));
    }
    k_kick_update<<<grid_for(s->npl, 128), 128, 0, c->stream>>>(s->npl, s->vb, s->ah, s->lmask, dt, s->rh,
                                                                 copy_r ? (lbeg ? s->rbeg : s->rend) : nullptr);
    return L(c, "kick_update_pl");
}

// helio_kick_vb_tp (helio_kick.f90:135-169) with symba_kick_getacch_tp (symba_kick.f90:79-123)
int kick_vb_tp(swg_system *s, double dt, int lbeg) {
    swg_ctx *c = s->c;
    if (s->ntp == 0) return SWG_OK;
    const double *rp = lbeg ? s->rbeg : s->rend;
    if (s->npl > 0) {
        ProfScope ps(s->prof, s->c->stream, PROF_KICK_TP);
        if (s->precision == SWG_MIXED) {
            const int nch = kick_mixed_chunks(c, s->ntp, s->npl);
            SWG_TRY(ensure_kick_scratch(c, s->kick_scratch_tp, kick_mixed_scratch_bytes(s->ntp, s->npl, nch)));
            SWG_TRY(kick_mixed_launch(c, true, s->ntp, s->npl, 0, s->trh, rp, s->Gmass, nullptr, s->tlmask, s->tah,
                                      1, nch, s->kick_scratch_tp.ptr));
        } else {
            SWG_TRY(kick_tp_fp64(c, s->ntp, s->npl, s->trh, rp, s->Gmass, s->tlmask, s->tah, 1));
        }
    } else {
        SWG_TRY(cuda_status(c, cudaMemsetAsync(s->tah, 0, sizeof(double) * 3 * s->ntp, c->stream), "memset"));
    }
    if (s->integrator == SWG_SYMBA && s->pltp_n > 0) {
        if (s->pltp_n <= ADDBACK_SMALL)
            k_pltp_addback_small<<<1, ADDBACK_SMALL, 0, c->stream>>>((int)s->pltp_n, s->pltp_l,
                                                                      s->pltp_l + s->pltp_cap, s->tlmask, s->trh, rp,
                                                                      s->Gmass, s->tah);
        else
            k_pltp_addback<<<1, 32, 0, c->stream>>>(s->pltp_n, s->pltp_l, s->pltp_l + s->pltp_cap, s->tlmask,
                                                    s->trh, rp, s->Gmass, s->tah);
        SWG_TRY(L(c, "pltp_addback"));
    }
    k_kick_update<<<grid_for(s->ntp, 128), 128, 0, c->stream>>>(s->ntp, s->tvb, s->tah, s->tlmask, dt, nullptr,
                                                                 nullptr);
    return L(c, "kick_update_tp");
}

// Mixed path: the per-system sum MODE over chunks of CHUNK_ONE bodies on many SMs
// (k_chunk_sums, then k_chunk_apply), instead of one block.
template <int MODE>
int chunk_sum(swg_system *s, const double *vsum, const int32_t *mask, const double *vin, double *vout, double dt,
              int slot) {
    swg_ctx *c = s->c;
    if (s->nchunks == 0) {
        std::vector<int4> tab;
        for (int b0 = 0, k = 0; b0 < s->npl; b0 += CHUNK_ONE, k++)
            tab.push_back(make_int4(0, b0, std::min(CHUNK_ONE, s->npl - b0), k));
        const size_t nt = tab.size();
        SWG_TRY(ensure(c, s->chunk_buf, sizeof(int4) * (nt + 1) + sizeof(double) * 4 * nt));
        const int2 range = make_int2(0, (int)nt);
        SWG_TRY(cuda_status(c, cudaMemcpyAsync(s->chunk_buf.ptr, tab.data(), sizeof(int4) * nt, cudaMemcpyHostToDevice,
                                               c->stream),
                            "chunks"));
        SWG_TRY(cuda_status(c, cudaMemcpyAsync((int4 *)s->chunk_buf.ptr + nt, &range, sizeof(int2),
                                               cudaMemcpyHostToDevice, c->stream),
                            "chunks"));
        SWG_TRY(cuda_status(c, cudaStreamSynchronize(c->stream), "chunks"));  // the host vectors go out of scope
        s->nchunks = (int)nt;
    }
    const int4 *tab = (const int4 *)s->chunk_buf.ptr;
    const int2 *range = (const int2 *)(tab + s->nchunks);
    double *part = (double *)(tab + s->nchunks + 1);
    k_chunk_sums<MODE><<<s->nchunks, CHUNK_T, 0, c->stream>>>(s->nchunks, tab, nullptr, s->Gmass, vsum, mask, part);
    SWG_TRY(L(c, "chunk_sums"));
    k_chunk_apply<MODE><<<s->nchunks, CHUNK_T, 0, c->stream>>>(tab, range, nullptr, part, nullptr, s->GMcb, s->lmask,
                                                               vin, vout, s->rh, dt, s->dcb, slot);
    return L(c, "chunk_apply");
}

int lindrift_pl(swg_system *s, double dt, int lbeg) {
    if (s->npl == 0) return SWG_OK;
    if (!exact(s)) return chunk_sum<SUM_LIN>(s, s->vb, s->lmask, nullptr, nullptr, dt, lbeg ? CB_PTBEG : CB_PTEND);
    k_lindrift_pl<<<1, RB, 0, s->c->stream>>>(s->npl, s->Gmass, s->vb, s->lmask, s->GMcb, s->rh, dt, s->dcb,
                                               lbeg ? CB_PTBEG : CB_PTEND, exact(s));
    return L(s->c, "lindrift_pl");
}
int tp_misc(swg_system *s, int slot, double dt, int mode) {
    if (s->ntp == 0) return SWG_OK;
    k_tp_misc<<<grid_for(s->ntp, 256), 256, 0, s->c->stream>>>(s->ntp, s->tlmask, s->trh, s->tvh, s->tvb, s->dcb,
                                                                slot, dt, mode);
    return L(s->c, "tp_misc");
}
int vh2vb_pl(swg_system *s) {
    if (s->npl == 0) return SWG_OK;
    if (!exact(s)) return chunk_sum<SUM_VH2VB>(s, s->vh, nullptr, s->vh, s->vb, 0.0, 0);
    k_vh2vb_pl<<<1, RB, 0, s->c->stream>>>(s->npl, s->Gmass, s->vh, s->vb, s->GMcb, s->dcb, exact(s));
    return L(s->c, "vh2vb_pl");
}
int vb2vh_pl(swg_system *s) {
    if (s->npl == 0) return SWG_OK;
    if (!exact(s)) return chunk_sum<SUM_VB2VH>(s, s->vb, s->status, s->vb, s->vh, 0.0, 0);
    k_vb2vh_pl<<<1, RB, 0, s->c->stream>>>(s->npl, s->Gmass, s->vb, s->status, s->vh, s->GMcb, s->dcb, exact(s));
    return L(s->c, "vb2vh_pl");
}
// drift with the SyMBA level mask (levelg == irec) or the plain status mask
int drift_pl(swg_system *s, double dt) {
    if (s->npl == 0) return SWG_OK;
    const int32_t *lev = s->integrator == SWG_SYMBA ? s->levelg : nullptr;
    ProfScope ps(s->prof, s->c->stream, PROF_DRIFT);
    return drift_masked(s->c, s->GMcb, s->rh, s->vb, s->npl, lev, s->irec, dt, s->status, nullptr, nullptr, nullptr,
                        !exact(s));
}
int drift_tp(swg_system *s, double dt) {
    if (s->ntp == 0) return SWG_OK;
    const int32_t *lev = s->integrator == SWG_SYMBA ? s->tlevelg : nullptr;
    double *v = s->integrator == SWG_WHM ? s->tvh : s->tvb;
    ProfScope ps(s->prof, s->c->stream, PROF_DRIFT);
    return drift_masked(s->c, s->GMcb, s->trh, v, s->ntp, lev, s->irec, dt, s->tstatus, nullptr, nullptr, nullptr,
                        !exact(s));
}

// helio_step_pl / _tp (helio_step.f90:37-119) via whm_step_system (whm_step.f90:14-35)
// opened: the opening sums and the pl-pl accelerations already ran (symba_step)
int helio_step(swg_system *s, double dt, bool opened = false) {
    const double dth = 0.5 * dt;
    s->lfirst_tp = s->lfirst_pl;
    if (s->npl > 0) {
        if (s->lfirst_pl) {
            if (!opened) SWG_TRY(vh2vb_pl(s));
            s->lfirst_pl = 0;
        }
        if (!opened) SWG_TRY(lindrift_pl(s, dth, 1));
        SWG_TRY(kick_vb_pl(s, dth, 1, true, opened));
        SWG_TRY(drift_pl(s, dt));
        SWG_TRY(kick_vb_pl(s, dth, 0));
        SWG_TRY(lindrift_pl(s, dth, 0));
        SWG_TRY(vb2vh_pl(s));
    }
    if (s->ntp > 0) {
        if (s->lfirst_tp) {
            SWG_TRY(tp_misc(s, CB_PTBEG, dth, 4));
            s->lfirst_tp = 0;
        } else {
            SWG_TRY(tp_misc(s, CB_PTBEG, dth, 2));
        }
        SWG_TRY(kick_vb_tp(s, dth, 1));
        SWG_TRY(drift_tp(s, dt));
        SWG_TRY(kick_vb_tp(s, dth, 0));
        SWG_TRY(tp_misc(s, CB_PTEND, dth, 3));
    }
    return SWG_OK;
}

// ---- WHM (whm_step.f90:14-104)
int whm_accel_pl(swg_system *s) {
    swg_ctx *c = s->c;
    SWG_TRY(cuda_status(c, cudaMemsetAsync(s->ah, 0, sizeof(double) * 3 * s->npl, c->stream), "memset"));
    k_whm_accel_pl<<<1, 256, 0, c->stream>>>(s->npl, s->Gmass, s->GMcb, s->rh, s->xj, s->lmask, s->ir3h, s->ir3j,
                                             s->ah, exact(s));
    SWG_TRY(L(c, "whm_accel_pl"));
    return accel_int_pl(s, 0);
}
int whm_kick_vh_pl(swg_system *s, double dt, int lbeg) {
    swg_ctx *c = s->c;
    if (lbeg) {
        if (s->lfirst_pl) {
            k_whm_h2j<<<1, 256, 0, c->stream>>>(s->npl, s->Gmass, s->eta, s->rh, s->vh, s->xj, s->vj, exact(s));
            SWG_TRY(L(c, "whm_h2j"));
            SWG_TRY(whm_accel_pl(s));
            s->lfirst_pl = 0;
        }
        k_kick_update<<<grid_for(s->npl, 128), 128, 0, c->stream>>>(s->npl, s->vh, s->ah, s->lmask, dt, s->rh,
                                                                     s->rbeg);
    } else {
        SWG_TRY(whm_accel_pl(s));
        k_kick_update<<<grid_for(s->npl, 128), 128, 0, c->stream>>>(s->npl, s->vh, s->ah, s->lmask, dt, s->rh,
                                                                     s->rend);
    }
    return L(c, "kick_update_whm");
}
int whm_accel_tp(swg_system *s, int lbeg, int zero) {
    swg_ctx *c = s->c;
    const double *rp = lbeg ? s->rbeg : s->rend;
    k_whm_tp_ah0<<<grid_for(s->ntp, 256), 256, 0, c->stream>>>(s->ntp, s->npl, s->Gmass, rp, s->tlmask, s->tah, zero,
                                                                     exact(s));
    SWG_TRY(L(c, "whm_tp_ah0"));
    if (s->precision == SWG_MIXED) {
        const int nch = kick_mixed_chunks(c, s->ntp, s->npl);
        SWG_TRY(ensure_kick_scratch(c, s->kick_scratch, kick_mixed_scratch_bytes(s->ntp, s->npl, nch)));
        return kick_mixed_launch(c, true, s->ntp, s->npl, 0, s->trh, rp, s->Gmass, nullptr, s->tlmask, s->tah, 0,
                                 nch, s->kick_scratch.ptr);
    }
    return kick_tp_fp64(c, s->ntp, s->npl, s->trh, rp, s->Gmass, s->tlmask, s->tah, 0);
}
int whm_kick_vh_tp(swg_system *s, double dt, int lbeg) {
    swg_ctx *c = s->c;
    if (s->lfirst_tp) {
        SWG_TRY(whm_accel_tp(s, 1, 1));
        s->lfirst_tp = 0;
    }
    if (!lbeg) SWG_TRY(whm_accel_tp(s, 0, 1));
    k_kick_update<<<grid_for(s->ntp, 128), 128, 0, c->stream>>>(s->ntp, s->tvh, s->tah, s->tlmask, dt, nullptr,
                                                                 nullptr);
    return L(c, "kick_update_whm_tp");
}
int whm_step(swg_system *s, double dt) {
    swg_ctx *c = s->c;
    const double dth = 0.5 * dt;
    s->lfirst_tp = s->lfirst_pl;
    if (s->npl > 0) {
        SWG_TRY(whm_kick_vh_pl(s, dth, 1));
        k_whm_vh2vj<<<1, 256, 0, c->stream>>>(s->npl, s->Gmass, s->eta, s->vh, s->vj, exact(s));
        SWG_TRY(L(c, "whm_vh2vj"));
        SWG_TRY(drift_all(c, s->muj, 0.0, s->xj, s->vj, s->npl, 0, 0.0, dt, s->lmask, s->iflag));
        int32_t *dflag = (int32_t *)s->flags.ptr;
        SWG_TRY(cuda_status(c, cudaMemsetAsync(dflag + 1, 0, sizeof(int32_t), c->stream), "memset"));
        k_any_nonzero<<<grid_for(s->npl, 256), 256, 0, c->stream>>>(s->npl, s->iflag, dflag + 1);
        SWG_TRY(L(c, "any_nonzero"));
        k_whm_drift_status<<<grid_for(s->npl, 256), 256, 0, c->stream>>>(s->npl, s->iflag, s->status, s->lmask);
        SWG_TRY(L(c, "whm_drift_status"));
        SWG_TRY(cuda_status(c, cudaMemcpyAsync(s->h_flags + 1, dflag + 1, sizeof(int32_t), cudaMemcpyDeviceToHost,
                                               c->stream),
                            "flag"));
        SWG_TRY(cuda_status(c, cudaStreamSynchronize(c->stream), "sync"));
        if (s->h_flags[1] != 0) {
            c->err = "Danby drift failed for a massive body (WHM stops the run)";
            return SWG_ERR_DRIFT;
        }
        k_whm_j2h<<<1, 256, 0, c->stream>>>(s->npl, s->Gmass, s->eta, s->xj, s->vj, s->rh, s->vh, exact(s));
        SWG_TRY(L(c, "whm_j2h"));
        SWG_TRY(whm_kick_vh_pl(s, dth, 0));
    }
    if (s->ntp > 0) {
        SWG_TRY(whm_kick_vh_tp(s, dth, 1));
        SWG_TRY(drift_tp(s, dt));
        SWG_TRY(whm_kick_vh_tp(s, dth, 0));
    }
    return SWG_OK;
}

// ---- SyMBA
// Runs f with the context's stream temporarily replaced (single host thread).
template <class F>
int on_stream(swg_ctx *c, cudaStream_t st, F f) {
    const cudaStream_t saved = c->stream;
    c->stream = st;
    const int rc = f();
    c->stream = saved;
    return rc;
}

int ensure_side(swg_system *s) {
    if (s->side) return SWG_OK;
    SWG_TRY(cuda_status(s->c, cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking), "side stream"));
    SWG_TRY(cuda_status(s->c, cudaStreamCreateWithFlags(&s->side2, cudaStreamNonBlocking), "side stream"));
    for (cudaEvent_t &e : s->ev) SWG_TRY(cuda_status(s->c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event"));
    return SWG_OK;
}
// stream b waits for the work queued so far on stream a (event e)
int join(swg_ctx *c, cudaStream_t a, cudaStream_t b, cudaEvent_t e) {
    SWG_TRY(cuda_status(c, cudaEventRecord(e, a), "event"));
    return cuda_status(c, cudaStreamWaitEvent(b, e, 0), "event");
}

int ensure_list(swg_system *s, int32_t **l, int64_t *cap, int64_t need) {
    if (need <= *cap) return SWG_OK;
    const int64_t ncap = std::max<int64_t>(need + need / 2, 256);
    int32_t *fresh = nullptr;
    SWG_TRY(dalloc(s->c, &fresh, (size_t)5 * ncap));
    if (*l) cudaFree(*l);
    *l = fresh;
    *cap = ncap;
    return SWG_OK;
}

// The radius-sorted sets of the system (SortedOne), built at the first call.
template <typename T>
int upload_vec(swg_ctx *c, T **dst, const std::vector<T> &v) {
    SWG_TRY(dalloc(c, dst, v.size()));
    if (v.empty()) return SWG_OK;
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(*dst, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, c->stream),
                        "upload"));
    return cuda_status(c, cudaStreamSynchronize(c->stream), "upload");
}
int build_sorted(swg_system *s, SortedOne *x) {
    swg_ctx *c = s->c;
    const std::vector<int32_t> meta = {0, s->npl, s->ntp};
    std::vector<int2> pt, tt;
    for (int p0 = 0; p0 < s->npl; p0 += ENC_BOUND_TILE) pt.push_back(make_int2(0, p0));
    for (int p0 = 0; p0 < s->ntp; p0 += ENC_BOUND_TILE) tt.push_back(make_int2(0, p0));
    // tp receivers of ENC_SORTED_TILE by chunks of the pl's 32-body sub-tiles: about 1024
    // blocks, so that one system fills the GPU
    const int nq = (s->ntp + ENC_SORTED_TILE - 1) / ENC_SORTED_TILE, nsub = (s->npl + 31) / 32;
    const int nch = std::max(1, std::min(nsub, 1024 / std::max(nq, 1)));
    x->pchunk = (nsub + nch - 1) / nch;
    std::vector<int4> items;
    for (int q0 = 0; q0 < s->ntp; q0 += ENC_SORTED_TILE)
        for (int u = 0, k = 0; u < nsub; u += x->pchunk, k++)
            items.push_back(make_int4(0, q0, std::min(ENC_SORTED_TILE, s->ntp - q0), k));
    x->nptiles = (int)pt.size();
    x->nttiles = (int)tt.size();
    x->nitems = (int)items.size();
    SWG_TRY(upload_vec(c, &x->meta, meta));
    SWG_TRY(upload_vec(c, &x->ptiles, pt));
    SWG_TRY(upload_vec(c, &x->ttiles, tt));
    SWG_TRY(upload_vec(c, &x->items, items));
    SWG_TRY(dalloc(c, &x->pperm, (size_t)s->npl));
    SWG_TRY(dalloc(c, &x->tperm, (size_t)s->ntp));
    SWG_TRY(dalloc(c, &x->pF, 3 * (size_t)s->npl));
    SWG_TRY(dalloc(c, &x->tF, 3 * (size_t)s->ntp));
    SWG_TRY(dalloc(c, &x->pbounds, 2 * pt.size()));  // bounds of each tile's two 32-body halves
    return dalloc(c, &x->tbounds, 2 * tt.size());
}
int ensure_sorted(swg_system *s) {
    if (s->srt) return SWG_OK;
    SortedOne *x = new SortedOne();
    const int rc = build_sorted(s, x);
    if (rc != SWG_OK) {  // nothing half-built is kept
        x->release();
        delete x;
        return rc;
    }
    s->srt = x;
    return SWG_OK;
}
SortedSet sorted_pl(swg_system *s, const double *r, const double *v, const double *renc) {
    SortedOne &x = *s->srt;
    SortedSet p;
    p.off = x.meta;
    p.n = x.meta + 1;
    p.r = r;
    p.v = v;
    p.renc = renc;
    p.perm = x.pperm;
    p.F = x.pF;
    p.N = s->npl;
    p.ntiles = x.nptiles;
    p.tiles = x.ptiles;
    p.tbase = x.meta;
    p.bounds = x.pbounds;
    p.nmax = s->npl;
    return p;
}
SortedSet sorted_tp(swg_system *s, const double *r, const double *v) {
    SortedOne &x = *s->srt;
    SortedSet t;
    t.off = x.meta;
    t.n = x.meta + 2;
    t.r = r;
    t.v = v;
    t.perm = x.tperm;
    t.F = x.tF;
    t.N = s->ntp;
    t.ntiles = x.nttiles;
    t.tiles = x.ttiles;
    t.tbase = x.meta;
    t.bounds = x.tbounds;
    t.nmax = s->ntp;
    return t;
}

// level-0 checks: symba_encounter_check_pl / _tp (symba_encounter_check.f90:14-87, 238-296)
// Level-0 checks of symba_encounter_check_pl / _tp (symba_encounter_check.f90:14-87,
// 238-296).  Both checks are launched before one host synchronization reads the two
// counts; short lists are sorted, de-duplicated and turned into SyMBA encounter
// lists (status, level, level-0 marks) by one single-block kernel each.
// r, v, tr, tv: the positions and velocities the checks read (the state at the start of the
// step, or a copy of it)
int symba_level0(swg_system *s, double dt, int *lany, const double *r, const double *v, const double *tr,
                 const double *tv) {
    swg_ctx *c = s->c;
    *lany = 0;
    s->plpl_n = s->pltp_n = 0;
    double *renc = (double *)s->red.ptr;
    k_set_renc<<<grid_for(s->npl, 128), 128, 0, c->stream>>>(s->npl, s->rhill, s->rhscale, 0, renc);
    SWG_TRY(L(c, "set_renc"));
    const int32_t nplt = s->npl - s->nplm;
    const bool do_pp = s->npl > 0, do_pt = s->ntp > 0 && s->npl > 0;
    EncWork *w[2] = {&s->enc, &s->enc2};
    for (int k = 0; k < 2; k++) {
        SWG_TRY(ensure(c, w[k]->counters, 2 * sizeof(unsigned long long)));
        if (w[k]->rawcap < 1024) {
            w[k]->rawcap = 1024;
            SWG_TRY(ensure(c, w[k]->raw, (size_t)w[k]->rawcap * 3 * sizeof(int32_t)));
        }
    }
    SWG_TRY(ensure(c, s->enc.sort, encounter_scratch_bytes(s->enc_plpl, s->npl, s->npl)));
    SWG_TRY(ensure(c, s->enc2.sort, encounter_scratch_bytes(s->enc_pltp, s->npl, s->ntp)));
    if (do_pt && s->enc_pltp == SWG_ENC_TRIANGULAR) SWG_TRY(ensure_sorted(s));
    unsigned long long *h = (unsigned long long *)(s->h_flags + 8);
    auto launch = [&](int kind) -> int {
        EncWork &e = *w[kind];
        int32_t *i1 = (int32_t *)e.raw.ptr, *i2 = i1 + e.rawcap, *lv = i2 + e.rawcap;
        unsigned long long *cnt = (unsigned long long *)e.counters.ptr;
        SWG_TRY(cuda_status(c, cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), c->stream), "memset"));
        if (kind == 0) {
            if (nplt == 0) {
                SWG_TRY(encounter_launch(c, s->enc_plpl, s->npl, r, v, renc, s->npl, r, v, renc, 1, 0,
                                         dt, e.rawcap, i1, i2, lv, cnt, e.sort.ptr));
            } else {
                SWG_TRY(encounter_launch(c, s->enc_plpl, s->nplm, r, v, renc, s->nplm, r, v, renc, 1,
                                         0, dt, e.rawcap, i1, i2, lv, cnt, e.sort.ptr));
                SWG_TRY(encounter_launch(c, s->enc_plpl, s->nplm, r, v, renc, nplt, r + 3 * s->nplm,
                                         v + 3 * s->nplm, renc + s->nplm, 0, s->nplm, dt, e.rawcap, i1, i2, lv,
                                         cnt, e.sort.ptr));
            }
        } else if (s->enc_pltp == SWG_ENC_TRIANGULAR) {
            // the triangular pl-tp check over radius-sorted tiles (the same list once sorted)
            const SortedSet pl = sorted_pl(s, r, v, renc), tp = sorted_tp(s, tr, tv);
            SWG_TRY(sorted_set_prep(c, pl, 1, s->srt->npl_prep++ % 8 == 0, dt));
            SWG_TRY(sorted_set_prep(c, tp, 1, s->srt->ntp_prep++ % 32 == 0, dt));
            SWG_TRY(pltp_sorted_batched(c, false, pl, tp, nullptr, s->srt->nitems, s->srt->items, dt, e.rawcap, i1, i2,
                                        lv, cnt, nullptr, s->srt->pchunk));
        } else {
            SWG_TRY(encounter_launch(c, s->enc_pltp, s->npl, r, v, renc, s->ntp, tr, tv, nullptr, 0, 0,
                                     dt, e.rawcap, i1, i2, lv, cnt, e.sort.ptr));
        }
        return cuda_status(c, cudaMemcpyAsync(&h[kind], cnt, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                              c->stream),
                           "count");
    };
    h[0] = h[1] = 0;
    if (do_pp && do_pt) {  // the two checks are independent: pl-tp on another stream
        SWG_TRY(ensure_side(s));
        const cudaStream_t other = c->stream == s->side ? s->side2 : s->side;
        SWG_TRY(join(c, c->stream, other, s->ev[0]));
        SWG_TRY(on_stream(c, other, [&] { return launch(1); }));
        SWG_TRY(launch(0));
        SWG_TRY(join(c, other, c->stream, s->ev[1]));
    } else {
        if (do_pp) SWG_TRY(launch(0));
        if (do_pt) SWG_TRY(launch(1));
    }
    SWG_TRY(cuda_status(c, cudaStreamSynchronize(c->stream), "level0"));
    for (int k = 0; k < 2; k++) {  // capacity overflow: grow the raw buffers and redo that check
        if ((int64_t)h[k] <= w[k]->rawcap) continue;
        w[k]->rawcap = (int64_t)h[k] + (int64_t)h[k] / 2 + 1024;
        DevBuf fresh;
        SWG_TRY(ensure(c, fresh, (size_t)w[k]->rawcap * 3 * sizeof(int32_t)));
        cudaFree(w[k]->raw.ptr);
        w[k]->raw = fresh;
        SWG_TRY(launch(k));
        SWG_TRY(cuda_status(c, cudaStreamSynchronize(c->stream), "level0"));
    }
    bool need_count_sync = false;
    for (int k = 0; k < 2; k++) {
        const int64_t n = (int64_t)h[k];
        if (n == 0) continue;
        EncWork &e = *w[k];
        int32_t **list = k == 0 ? &s->plpl_l : &s->pltp_l;
        int64_t *cap = k == 0 ? &s->plpl_cap : &s->pltp_cap;
        SWG_TRY(ensure_list(s, list, cap, n));
        int32_t *i1 = (int32_t *)e.raw.ptr, *i2 = i1 + e.rawcap, *lv = i2 + e.rawcap;
        unsigned long long *cnt = (unsigned long long *)e.counters.ptr;
        if (n <= FIN_N) {
            k_list_finalize<<<1, 1024, 0, c->stream>>>((int)n, i1, i2, lv, *list, *cap, k, s->levelg, s->levelm,
                                                       k == 0 ? s->nplenc : s->ntpenc, s->tlevelg, s->tlevelm,
                                                       s->tnplenc, cnt + 1);
            SWG_TRY(L(c, "list_finalize"));
        } else {
            SWG_TRY(ensure(c, e.sort, sort_pairs_scratch_bytes(n)));
            SWG_TRY(sort_pairs_unique(c, n, i1, i2, lv, e.sort.ptr, cnt + 1));
            SWG_TRY(cuda_status(c, cudaMemcpyAsync(&h[2 + k], cnt + 1, sizeof(unsigned long long),
                                                   cudaMemcpyDeviceToHost, c->stream),
                                "count"));
            SWG_TRY(cuda_status(c, cudaStreamSynchronize(c->stream), "level0"));
            const int64_t m = (int64_t)h[2 + k];
            for (int f = 0; f < 3; f++) {
                const int32_t *src = f == 0 ? i1 : (f == 1 ? i2 : lv);
                SWG_TRY(cuda_status(c, cudaMemcpyAsync(*list + f * *cap, src, sizeof(int32_t) * m,
                                                       cudaMemcpyDeviceToDevice, c->stream),
                                    "copy list"));
            }
            k_level0_mark<<<grid_for(m, 128), 128, 0, c->stream>>>(m, *list, *cap, k, s->levelg, s->levelm,
                                                                   k == 0 ? s->nplenc : s->ntpenc, s->tlevelg,
                                                                   s->tlevelm, s->tnplenc);
            SWG_TRY(L(c, "level0_mark"));
            (k == 0 ? s->plpl_n : s->pltp_n) = m;
            continue;
        }
        const int mode = k == 0 ? s->enc_plpl : s->enc_pltp;
        if (mode == SWG_ENC_SORTSWEEP) {
            // the sweep can report a pair twice; the exact count is known after de-duplication
            SWG_TRY(cuda_status(c, cudaMemcpyAsync(&h[2 + k], cnt + 1, sizeof(unsigned long long),
                                                   cudaMemcpyDeviceToHost, c->stream),
                                "count"));
            need_count_sync = true;
        } else {
            (k == 0 ? s->plpl_n : s->pltp_n) = n;  // triangular lists hold no repeats
        }
    }
    if (need_count_sync) {
        SWG_TRY(cuda_status(c, cudaStreamSynchronize(c->stream), "level0"));
        if (s->enc_plpl == SWG_ENC_SORTSWEEP && h[0] > 0 && h[0] <= FIN_N) s->plpl_n = (int64_t)h[2];
        if (s->enc_pltp == SWG_ENC_SORTSWEEP && h[1] > 0 && h[1] <= FIN_N) s->pltp_n = (int64_t)h[3];
    }
    s->stats[2] += s->plpl_n;
    s->stats[3] += s->pltp_n;
    *lany = (s->plpl_n + s->pltp_n) > 0;
    return SWG_OK;
}

// Collisions found by a paused recursion: host copies of the system, perfect merging
// (resolve_collisions_host), and the modified arrays written back.
int resolve_collisions(swg_system *s) {
    swg_ctx *c = s->c;
    const size_t n = std::max(s->npl, 1), m = std::max(s->ntp, 1);
    std::vector<double> rh(3 * n), vb(3 * n), Gm(n), R(n), rhill(n), trh(3 * m), tvb(3 * m);
    std::vector<int32_t> st(n), lm(n), lev(n), tst(m), tlm(m);
    const int64_t npp = s->plpl_n, npt = s->pltp_n;
    std::vector<int32_t> pp(4 * std::max<int64_t>(npp, 1)), pt(3 * std::max<int64_t>(npt, 1));
    int32_t irec = 0;
    struct Copy {
        void *h;
        void *d;
        size_t bytes;
    };
    std::vector<Copy> pl_arrays = {{rh.data(), s->rh, 24 * (size_t)s->npl},   {vb.data(), s->vb, 24 * (size_t)s->npl},
                                   {Gm.data(), s->Gmass, 8 * (size_t)s->npl}, {R.data(), s->radius, 8 * (size_t)s->npl},
                                   {rhill.data(), s->rhill, 8 * (size_t)s->npl},
                                   {st.data(), s->status, 4 * (size_t)s->npl}, {lm.data(), s->lmask, 4 * (size_t)s->npl},
                                   {trh.data(), s->trh, 24 * (size_t)s->ntp}, {tvb.data(), s->tvb, 24 * (size_t)s->ntp},
                                   {tst.data(), s->tstatus, 4 * (size_t)s->ntp},
                                   {tlm.data(), s->tlmask, 4 * (size_t)s->ntp}};
    std::vector<Copy> lists;
    for (int f = 0; f < 3; f++) {  // i1, i2, status of each list
        const int field = f == 2 ? 3 : f;
        if (npp) lists.push_back({pp.data() + f * npp, s->plpl_l + field * s->plpl_cap, 4 * (size_t)npp});
        if (npt) lists.push_back({pt.data() + f * npt, s->pltp_l + field * s->pltp_cap, 4 * (size_t)npt});
    }
    // read only: the pl-pl lvdotr field and the levels (for the cascade check), the paused level
    std::vector<Copy> inputs = {{lev.data(), s->levelg, 4 * (size_t)s->npl}, {&irec, s->rec_resume + 1, 4}};
    if (npp) inputs.push_back({pp.data() + 3 * npp, s->plpl_l + 2 * s->plpl_cap, 4 * (size_t)npp});
    for (auto *v : {&pl_arrays, &lists, &inputs})
        for (const Copy &x : *v)
            if (x.bytes)
                SWG_TRY(cuda_status(c, cudaMemcpyAsync(x.h, x.d, x.bytes, cudaMemcpyDeviceToHost, c->stream), "collision"));
    SWG_TRY(cuda_status(c, cudaStreamSynchronize(c->stream), "collision"));
    CollisionSystem cs;
    cs.npl = s->npl;
    cs.ntp = s->ntp;
    cs.GMcb = s->GMcb;
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
    cs.dt = level_dt(s->rec_dt, irec);
    cs.E_collisions = s->E_collisions;
    for (int d = 0; d < 3; d++) cs.L_escape[d] = s->L_escape[d];
    cs.dev = c;
    const int64_t nres = resolve_collisions_host(cs);
    if (nres == -2) return SWG_ERR_CUDA;
    if (nres < 0) {
        c->err = "runaway collisional cascade (more than 1000 rounds of merges in one resolution)";
        return SWG_ERR_STATE;
    }
    s->stats[4] += nres;
    s->E_collisions = cs.E_collisions;
    for (int d = 0; d < 3; d++) s->L_escape[d] = cs.L_escape[d];
    for (auto *v : {&pl_arrays, &lists})
        for (const Copy &x : *v)
            if (x.bytes)
                SWG_TRY(cuda_status(c, cudaMemcpyAsync(x.d, x.h, x.bytes, cudaMemcpyHostToDevice, c->stream), "collision"));
    return cuda_status(c, cudaStreamSynchronize(c->stream), "collision");
}

// Launch the whole SyMBA recursion of one step (symba_step_recur_system from level 0)
// as one single-block kernel; no host round trip until the next step's checks.
int symba_recursion(swg_system *s, double dt) {
    swg_ctx *c = s->c;
    s->rec_dt = dt;
    const int64_t n = s->plpl_n + s->pltp_n;
    SWG_TRY(ensure(c, s->rec_scratch, sizeof(double) * (size_t)(12 * n + 8) + (size_t)(3 * n + 96) +
                                          sizeof(int32_t) * (size_t)(7 * n + 128)));
    RecArgs a;
    a.npl = s->npl;
    a.ntp = s->ntp;
    a.npp = s->plpl_n;
    a.ppcap = s->plpl_cap;
    a.npt = s->pltp_n;
    a.ptcap = s->pltp_cap;
    a.pp = s->plpl_l;
    a.pt = s->pltp_l;
    a.rh = s->rh;
    a.vb = s->vb;
    a.ah = s->ah;
    a.trh = s->trh;
    a.tvb = s->tvb;
    a.tah = s->tah;
    a.Gm = s->Gmass;
    a.rhill = s->rhill;
    a.radius = s->radius;
    a.status = s->status;
    a.tstatus = s->tstatus;
    a.levelg = s->levelg;
    a.levelm = s->levelm;
    a.tlevelg = s->tlevelg;
    a.tlevelm = s->tlevelm;
    a.GMcb = s->GMcb;
    a.rhscale = s->rhscale;
    a.dt = dt;
    a.terms = (double *)s->rec_scratch.ptr;
    int32_t *ibuf = (int32_t *)(a.terms + 12 * n + 8);
    a.bpl = ibuf;                 // up to 2*npp + npt bodies
    a.btp = ibuf + 2 * n + 32;    // up to npt bodies
    a.adj_end = ibuf + 3 * n + 64;  // one per listed body (up to 2 * (npp + npt))
    a.adj = ibuf + 5 * n + 96;      // two per pl-pl entry, one per pl-tp entry
    uint8_t *bbuf = (uint8_t *)(ibuf + 7 * n + 128);
    a.lenc = bbuf;
    a.good = bbuf + n + 32;
    a.good2 = bbuf + 2 * n + 64;
    a.mark_pl = s->mark_pl;
    a.mark_tp = s->mark_tp;
    a.out = s->rec_out;
    a.lclose = s->lclose;
    a.fast = !exact(s);
    a.resume = s->rec_resume;
    a.pend = s->rec_out + 3;
    // lists that fit are staged in shared memory (a collision resolution can redirect list
    // entries but never adds any, so the size holds for the resumed launches)
    const size_t need = rec_stage_bytes(s->plpl_n, s->pltp_n);
    const size_t smem = need <= REC_STAGE_MAX ? need : 0;
    a.stage_bytes = (int64_t)smem;
    static bool smem_set = false;  // the kernel's own shared arrays come on top of the stage
    if (smem > 0 && !smem_set) {
        SWG_TRY(cuda_status(c, cudaFuncSetAttribute(k_symba_recursion, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                    (int)REC_STAGE_MAX),
                            "recursion smem"));
        smem_set = true;
    }
    ProfScope ps(s->prof, s->c->stream, PROF_RECUR);
    for (;;) {
        if (s->lclose)
            SWG_TRY(cuda_status(c, cudaMemsetAsync(a.pend, 0, sizeof(int32_t), c->stream), "memset"));
        k_symba_recursion<<<1, RECT, smem, c->stream>>>(a);
        SWG_TRY(L(c, "symba_recursion"));
        if (!s->lclose) break;
        // a collision pauses the recursion: resolve it on the host, then resume
        SWG_TRY(cuda_status(c, cudaMemcpyAsync(s->h_flags + 4, a.pend, sizeof(int32_t), cudaMemcpyDeviceToHost,
                                               c->stream),
                            "pending"));
        SWG_TRY(cuda_status(c, cudaStreamSynchronize(c->stream), "recursion"));
        if (s->h_flags[4] == 0) break;
        SWG_TRY(resolve_collisions(s));
    }
    // status word read back at the next host synchronization
    return cuda_status(c, cudaMemcpyAsync(s->h_flags + 2, s->rec_out, 2 * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                          c->stream),
                       "recursion status");
}

// symba_step_interp_system (symba_step.f90:55-115).  With test particles, their half-steps
// run on a second stream beside the massive bodies': they read the massive bodies only
// through the start and end positions (copied to rbeg / rend before the fork) and the
// central-body record, and the recursion (which moves the listed test particles) waits
// for their opening half.  Each kernel's arithmetic is unchanged, so the results are the
// serial order's bits.
// opened: the opening sums and the pl-pl accelerations already ran (symba_step).
int symba_interp(swg_system *s, double dt, bool opened = false) {
    swg_ctx *c = s->c;
    const double dth = 0.5 * dt;
    s->irec = -1;
    const bool fork = s->ntp > 0 && s->npl > 0;
    if (fork) SWG_TRY(ensure_side(s));
    if (!opened) {
        if (s->lfirst_pl) SWG_TRY(vh2vb_pl(s));
        SWG_TRY(lindrift_pl(s, dth, 1));
    }
    if (fork) {
        SWG_TRY(cuda_status(c, cudaMemcpyAsync(s->rbeg, s->rh, 24 * (size_t)s->npl, cudaMemcpyDeviceToDevice, c->stream),
                            "rbeg"));
        SWG_TRY(join(c, c->stream, s->side, s->ev[0]));
        SWG_TRY(on_stream(c, s->side, [&] {
            SWG_TRY(tp_misc(s, CB_PTBEG, dth, s->lfirst_tp ? 4 : 2));
            SWG_TRY(kick_vb_tp(s, dth, 1));
            return drift_tp(s, dt);
        }));
    }
    SWG_TRY(kick_vb_pl(s, dth, 1, !fork, opened));
    SWG_TRY(drift_pl(s, dt));
    if (fork) {
        SWG_TRY(join(c, s->side, c->stream, s->ev[1]));
    } else if (s->ntp > 0) {
        SWG_TRY(tp_misc(s, CB_PTBEG, dth, s->lfirst_tp ? 4 : 2));
        SWG_TRY(kick_vb_tp(s, dth, 1));
        SWG_TRY(drift_tp(s, dt));
    }
    SWG_TRY(symba_recursion(s, dt));
    s->irec = -1;
    if (fork) {
        SWG_TRY(cuda_status(c, cudaMemcpyAsync(s->rend, s->rh, 24 * (size_t)s->npl, cudaMemcpyDeviceToDevice, c->stream),
                            "rend"));
        SWG_TRY(join(c, c->stream, s->side, s->ev[2]));
        SWG_TRY(on_stream(c, s->side, [&] { return kick_vb_tp(s, dth, 0); }));
    }
    SWG_TRY(kick_vb_pl(s, dth, 0, !fork));
    SWG_TRY(lindrift_pl(s, dth, 0));
    if (fork) {  // the test particles' closing linear drift needs the central-body record
        SWG_TRY(join(c, c->stream, s->side, s->ev[3]));
        SWG_TRY(on_stream(c, s->side, [&] { return tp_misc(s, CB_PTEND, dth, 3); }));
    }
    SWG_TRY(vb2vh_pl(s));
    if (fork) {
        SWG_TRY(join(c, s->side, c->stream, s->ev[4]));
    } else if (s->ntp > 0) {
        SWG_TRY(kick_vb_tp(s, dth, 0));
        SWG_TRY(tp_misc(s, CB_PTEND, dth, 3));
    }
    return SWG_OK;
}

// swiftest_discard_pl_tp (src/swiftest/swiftest_discard.f90:244-290), run after each step
// when close encounters are checked (param%lclose), as the reference's main loop
// (swiftest_driver) does after every step.
// The scan runs over the radius-sorted sets (the same flags as the all-pairs scan: a pl and a
// tp whose radial intervals over the step are farther apart than the pl's radius are skipped).
int discard_step(swg_system *s) {
    if (!s->lclose || s->npl == 0 || s->ntp == 0) return SWG_OK;
    swg_ctx *c = s->c;
    SWG_TRY(ensure_sorted(s));
    const SortedSet pl = sorted_pl(s, s->rh, s->vh, s->radius), tp = sorted_tp(s, s->trh, s->tvh);
    SWG_TRY(sorted_set_prep(c, pl, 1, s->srt->npl_prep++ % 8 == 0, s->dt));
    SWG_TRY(sorted_set_prep(c, tp, 1, s->srt->ntp_prep++ % 32 == 0, s->dt));
    SWG_TRY(pltp_sorted_batched(c, true, pl, tp, s->tstatus, s->srt->nitems, s->srt->items, s->dt, 0, nullptr, nullptr,
                                nullptr, nullptr, s->tflag, s->srt->pchunk));
    k_apply_discard<<<grid_for(s->ntp, 256), 256, 0, c->stream>>>(s->ntp, s->tflag, s->tstatus, s->tlmask, s->trh,
                                                                  s->tvh, s->tvb, s->npl, nullptr, nullptr, nullptr,
                                                                  s->ndiscard);
    return L(c, "apply_discard");
}

// symba_step_system (symba_step.f90:14-52); both level-0 checks are evaluated
int symba_step(swg_system *s, double dt) {
    swg_ctx *c = s->c;
    const int nmax = std::max(s->npl, s->ntp);
    k_symba_reset<<<grid_for(nmax, 256), 256, 0, c->stream>>>(s->npl, s->ntp, s->levelg, s->levelm, s->nplenc,
                                                               s->ntpenc, s->lmask, s->tlevelg, s->tlevelm,
                                                               s->tnplenc, s->tlmask, s->status, s->tstatus);
    SWG_TRY(L(c, "symba_reset"));
    s->lfirst_tp = s->lfirstkick;
    s->lfirst_pl = s->lfirstkick;
    int lany = 0;
    if (s->prof.on || s->npl == 0) {
        {
            ProfScope ps(s->prof, s->c->stream, PROF_ENC0);
            SWG_TRY(symba_level0(s, dt, &lany, s->rh, s->vb, s->trh, s->tvb));
        }
        if (lany) {
            s->stats[0]++;
            SWG_TRY(symba_interp(s, dt));
        } else {
            s->irec = -1;
            SWG_TRY(helio_step(s, dt));
        }
        s->lfirstkick = s->lfirst_pl;
        return SWG_OK;
    }
    // The level-0 checks read a copy of the start-of-step state on the second stream while
    // this stream runs the opening per-system sums (vh2vb on the first step, the linear
    // drift) and the opening pair accelerations, which both the interpolated step and the
    // HELIO step take first and which do not need the lists; the lists are joined before
    // the encounter-pair subtraction.  Every kernel's arithmetic is unchanged.
    SWG_TRY(ensure_side(s));
    const size_t n = s->npl, m = s->ntp;
    SWG_TRY(ensure(c, s->snap, sizeof(double) * 6 * (n + m)));
    double *sr = (double *)s->snap.ptr, *sv = sr + 3 * n, *st = sv + 3 * n, *stv = st + 3 * m;
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(sr, s->rh, 24 * n, cudaMemcpyDeviceToDevice, c->stream), "snap"));
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(sv, s->vb, 24 * n, cudaMemcpyDeviceToDevice, c->stream), "snap"));
    if (m) {
        SWG_TRY(cuda_status(c, cudaMemcpyAsync(st, s->trh, 24 * m, cudaMemcpyDeviceToDevice, c->stream), "snap"));
        SWG_TRY(cuda_status(c, cudaMemcpyAsync(stv, s->tvb, 24 * m, cudaMemcpyDeviceToDevice, c->stream), "snap"));
    }
    SWG_TRY(join(c, c->stream, s->side, s->ev[5]));
    const double dth = 0.5 * dt;
    if (s->lfirst_pl) SWG_TRY(vh2vb_pl(s));
    SWG_TRY(lindrift_pl(s, dth, 1));
    SWG_TRY(accel_int_pl(s, 1));
    // the checks (their host synchronisation waits for the second stream only)
    SWG_TRY(on_stream(c, s->side, [&] { return symba_level0(s, dt, &lany, sr, sv, st, stv); }));
    SWG_TRY(join(c, s->side, c->stream, s->ev[5]));
    if (lany) {
        s->stats[0]++;
        SWG_TRY(symba_interp(s, dt, true));
    } else {
        s->irec = -1;
        SWG_TRY(helio_step(s, dt, true));
    }
    s->lfirstkick = s->lfirst_pl;
    return SWG_OK;
}

}  // namespace

// ======================================================================== C ABI
extern "C" {

int swg_system_create(swg_ctx *c, int integrator, int32_t npl, int32_t ntp, swg_system **out) {
    if (!c || !out || npl < 0 || ntp < 0 || integrator < SWG_WHM || integrator > SWG_SYMBA) return SWG_ERR_ARG;
    swg_system *s = new swg_system();
    s->c = c;
    c->systems.push_back(s);
    s->integrator = integrator;
    s->npl = npl;
    s->ntp = ntp;
    s->nplm = npl;
    const size_t n = std::max(npl, 1), m = std::max(ntp, 1);
    int rc = SWG_OK;
    double **pd[] = {&s->rh, &s->vh, &s->vb, &s->ah, &s->rbeg, &s->rend, &s->xj, &s->vj};
    for (auto p : pd)
        if (rc == SWG_OK) rc = dalloc(c, p, 3 * n);
    double **pn[] = {&s->Gmass, &s->radius, &s->rhill, &s->eta, &s->muj, &s->ir3h, &s->ir3j};
    for (auto p : pn)
        if (rc == SWG_OK) rc = dalloc(c, p, n);
    int32_t **pi[] = {&s->status, &s->lmask, &s->levelg, &s->levelm, &s->nplenc, &s->ntpenc, &s->iflag};
    for (auto p : pi)
        if (rc == SWG_OK) rc = dalloc(c, p, n);
    double **td[] = {&s->trh, &s->tvh, &s->tvb, &s->tah};
    for (auto p : td)
        if (rc == SWG_OK) rc = dalloc(c, p, 3 * m);
    int32_t **ti[] = {&s->tstatus, &s->tlmask, &s->tlevelg, &s->tlevelm, &s->tnplenc, &s->tiflag};
    for (auto p : ti)
        if (rc == SWG_OK) rc = dalloc(c, p, m);
    if (rc == SWG_OK) rc = dalloc(c, &s->dcb, CB_N);
    if (rc == SWG_OK) rc = dalloc(c, &s->mark_pl, n);
    if (rc == SWG_OK) rc = dalloc(c, &s->mark_tp, m);
    if (rc == SWG_OK) rc = dalloc(c, &s->rec_out, 4);
    if (rc == SWG_OK) rc = dalloc(c, &s->rec_resume, REC_STATE);
    if (rc == SWG_OK) rc = dalloc(c, &s->tflag, m);
    if (rc == SWG_OK) rc = dalloc(c, &s->ndiscard, 1);
    if (rc == SWG_OK) rc = ensure(c, s->flags, 64);
    if (rc == SWG_OK) rc = ensure(c, s->red, sizeof(double) * (4 * n + 64));
    if (rc == SWG_OK) {
        cudaError_t e = cudaMallocHost((void **)&s->h_flags, 64);
        if (e != cudaSuccess) rc = cuda_status(c, e, "cudaMallocHost");
    }
    if (rc != SWG_OK) {
        swg_system_destroy(s);
        return rc;
    }
    *out = s;
    return cuda_status(c, cudaStreamSynchronize(c->stream), "create");
}

int swg_system_destroy(swg_system *s) {
    if (!s) return SWG_OK;
    swg_ctx *c = s->c;
    if (c) {
        cudaStreamSynchronize(c->stream);
        auto it = std::find(c->systems.begin(), c->systems.end(), (void *)s);
        if (it != c->systems.end()) c->systems.erase(it);
    }
    void *ptrs[] = {s->rh, s->vh, s->vb, s->ah, s->rbeg, s->rend, s->xj, s->vj, s->Gmass, s->radius, s->rhill,
                    s->eta, s->muj, s->ir3h, s->ir3j, s->status, s->lmask, s->levelg, s->levelm, s->nplenc,
                    s->ntpenc, s->iflag, s->trh, s->tvh, s->tvb, s->tah, s->tstatus, s->tlmask, s->tlevelg,
                    s->tlevelm, s->tnplenc, s->tiflag, s->dcb, s->plpl_l, s->pltp_l, s->enc.raw.ptr,
                    s->enc.sort.ptr, s->enc.counters.ptr, s->enc2.raw.ptr, s->enc2.sort.ptr, s->enc2.counters.ptr, s->kick_scratch.ptr, s->pair_scratch.ptr, s->flags.ptr,
                    s->red.ptr, s->mark_pl, s->mark_tp, s->rec_out, s->rec_resume, s->rec_scratch.ptr,
                    s->discard_scratch.ptr, s->tflag, s->ndiscard, s->chunk_buf.ptr, s->kick_scratch_tp.ptr,
                    s->snap.ptr};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (s->h_flags) cudaFreeHost(s->h_flags);
    for (cudaEvent_t e : s->ev)
        if (e) cudaEventDestroy(e);
    if (s->side) cudaStreamDestroy(s->side);
    if (s->side2) cudaStreamDestroy(s->side2);
    s->prof.release();
    if (s->srt) {
        s->srt->release();
        delete s->srt;
    }
    delete s;
    return SWG_OK;
}

int swg_system_set_cb(swg_system *s, double GMcb, double Rcb) {
    if (!s || !(GMcb > 0.0)) return SWG_ERR_ARG;
    s->GMcb = GMcb;
    s->Rcb = Rcb;
    return SWG_OK;
}

int swg_system_set_pl(swg_system *s, const double *rh, const double *vh, const double *Gmass, const double *radius,
                      const double *rhill) {
    if (!s) return SWG_ERR_ARG;
    swg_ctx *c = s->c;
    const size_t n = s->npl;
    if (n == 0) return SWG_OK;
    if (!rh || !vh || !Gmass || !radius || !rhill) return SWG_ERR_ARG;
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(s->rh, rh, 24 * n, cudaMemcpyHostToDevice, c->stream), "set_pl"));
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(s->vh, vh, 24 * n, cudaMemcpyHostToDevice, c->stream), "set_pl"));
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(s->Gmass, Gmass, 8 * n, cudaMemcpyHostToDevice, c->stream), "set_pl"));
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(s->radius, radius, 8 * n, cudaMemcpyHostToDevice, c->stream), "set_pl"));
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(s->rhill, rhill, 8 * n, cudaMemcpyHostToDevice, c->stream), "set_pl"));
    s->initialized = 0;
    return cuda_status(c, cudaStreamSynchronize(c->stream), "set_pl");
}

int swg_system_set_tp(swg_system *s, const double *rh, const double *vh) {
    if (!s) return SWG_ERR_ARG;
    swg_ctx *c = s->c;
    const size_t n = s->ntp;
    if (n == 0) return SWG_OK;
    if (!rh || !vh) return SWG_ERR_ARG;
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(s->trh, rh, 24 * n, cudaMemcpyHostToDevice, c->stream), "set_tp"));
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(s->tvh, vh, 24 * n, cudaMemcpyHostToDevice, c->stream), "set_tp"));
    s->initialized = 0;
    return cuda_status(c, cudaStreamSynchronize(c->stream), "set_tp");
}

int swg_system_set_param(swg_system *s, double dt, int loop_mode, int enc_plpl, int enc_pltp, double rhscale,
                         int lclose, double gmtiny, int precision) {
    if (!s || !(dt > 0.0) || (loop_mode != 0 && loop_mode != 1) || (precision != SWG_FP64 && precision != SWG_MIXED))
        return SWG_ERR_ARG;
    if ((enc_plpl != SWG_ENC_TRIANGULAR && enc_plpl != SWG_ENC_SORTSWEEP) ||
        (enc_pltp != SWG_ENC_TRIANGULAR && enc_pltp != SWG_ENC_SORTSWEEP) || !(rhscale > 0.0))
        return SWG_ERR_ARG;
    s->dt = dt;
    s->loop_mode = loop_mode;
    s->enc_plpl = enc_plpl;
    s->enc_pltp = enc_pltp;
    s->rhscale = rhscale;
    s->lclose = lclose;
    s->gmtiny = gmtiny;
    s->precision = precision;
    return SWG_OK;
}

// Initialisation as helio_util_setup_initialize_system (helio_util.f90:14-43) /
// whm_util_set_mu_eta_pl (whm_util.f90:175-198); bodies arrive pre-sorted.
int swg_system_initialize(swg_system *s) {
    if (!s || !(s->GMcb > 0.0) || !(s->dt > 0.0)) return SWG_ERR_STATE;
    swg_ctx *c = s->c;
    s->E_collisions = 0.0;
    s->L_escape[0] = s->L_escape[1] = s->L_escape[2] = 0.0;
    const int n = s->npl;
    std::vector<int32_t> ones(std::max(n, s->ntp), 1), zeros(std::max(n, s->ntp), 0);
    if (n > 0) {
        SWG_TRY(cuda_status(c, cudaMemcpyAsync(s->status, zeros.data(), 4 * n, cudaMemcpyHostToDevice, c->stream), "init"));
        SWG_TRY(cuda_status(c, cudaMemcpyAsync(s->lmask, ones.data(), 4 * n, cudaMemcpyHostToDevice, c->stream), "init"));
    }
    if (s->ntp > 0) {
        SWG_TRY(cuda_status(c, cudaMemcpyAsync(s->tstatus, zeros.data(), 4 * s->ntp, cudaMemcpyHostToDevice, c->stream), "init"));
        SWG_TRY(cuda_status(c, cudaMemcpyAsync(s->tlmask, ones.data(), 4 * s->ntp, cudaMemcpyHostToDevice, c->stream), "init"));
    }
    std::vector<double> Gm(n);
    if (n > 0)
        SWG_TRY(cuda_status(c, cudaMemcpyAsync(Gm.data(), s->Gmass, 8 * n, cudaMemcpyDeviceToHost, c->stream), "init"));
    SWG_TRY(cuda_status(c, cudaStreamSynchronize(c->stream), "init"));
    s->nplm = n;
    if (s->gmtiny > 0.0) {
        int m = 0;
        for (int i = 0; i < n; i++) m += !(Gm[i] < s->gmtiny);
        s->nplm = m;
    }
    if (s->integrator == SWG_WHM) {
        std::vector<double> eta(n), muj(n);
        if (n > 0) {
            eta[0] = s->GMcb + Gm[0];
            muj[0] = eta[0];
            for (int i = 1; i < n; i++) {
                eta[i] = eta[i - 1] + Gm[i];
                muj[i] = s->GMcb * eta[i] / eta[i - 1];
            }
            SWG_TRY(cuda_status(c, cudaMemcpyAsync(s->eta, eta.data(), 8 * n, cudaMemcpyHostToDevice, c->stream), "init"));
            SWG_TRY(cuda_status(c, cudaMemcpyAsync(s->muj, muj.data(), 8 * n, cudaMemcpyHostToDevice, c->stream), "init"));
        }
    } else {
        SWG_TRY(vh2vb_pl(s));
        if (s->ntp > 0) {
            // tp h2b: vb = vh + cb%vb
            SWG_TRY(tp_misc(s, CB_VB, 0.0, 5));
        }
    }
    s->lfirst_pl = s->lfirst_tp = s->lfirstkick = 1;
    s->irec = -1;
    s->t = 0.0;
    s->initialized = 1;
    return cuda_status(c, cudaStreamSynchronize(c->stream), "init");
}

int swg_system_step(swg_system *s, int32_t nsteps) {
    if (!s || !s->initialized) return SWG_ERR_STATE;
    s->h_flags[2] = 0;
    for (int32_t k = 0; k < nsteps; k++) {
        int rc;
        if (s->integrator == SWG_WHM)
            rc = whm_step(s, s->dt);
        else if (s->integrator == SWG_HELIO)
            rc = helio_step(s, s->dt);
        else
            rc = symba_step(s, s->dt);
        if (rc != SWG_OK) return rc;
        SWG_TRY(discard_step(s));
        if (s->h_flags[2] != 0) {  // recursion status of an earlier step, seen at a sync point
            s->c->err = "SyMBA local time step too small";
            return s->h_flags[2];
        }
        s->t += s->dt;
    }
    if (s->integrator == SWG_SYMBA) {
        SWG_TRY(cuda_status(s->c, cudaStreamSynchronize(s->c->stream), "step"));
        if (s->h_flags[2] != 0) {
            s->c->err = "SyMBA local time step too small";
            return s->h_flags[2];
        }
    }
    return SWG_OK;
}

int swg_system_get_pl_masses(swg_system *s, double *Gmass, double *radius, double *rhill) {
    if (!s) return SWG_ERR_ARG;
    swg_ctx *c = s->c;
    const size_t n = s->npl;
    if (n == 0) return SWG_OK;
    const std::pair<double *, const double *> xs[] = {{Gmass, s->Gmass}, {radius, s->radius}, {rhill, s->rhill}};
    for (const auto &x : xs)
        if (x.first)
            SWG_TRY(cuda_status(c, cudaMemcpyAsync(x.first, x.second, 8 * n, cudaMemcpyDeviceToHost, c->stream),
                                "get_pl_masses"));
    return cuda_status(c, cudaStreamSynchronize(c->stream), "get_pl_masses");
}

int swg_system_get_pl(swg_system *s, double *rh, double *vh, int32_t *status) {
    if (!s) return SWG_ERR_ARG;
    swg_ctx *c = s->c;
    const size_t n = s->npl;
    if (n == 0) return SWG_OK;
    if (rh) SWG_TRY(cuda_status(c, cudaMemcpyAsync(rh, s->rh, 24 * n, cudaMemcpyDeviceToHost, c->stream), "get_pl"));
    if (vh) SWG_TRY(cuda_status(c, cudaMemcpyAsync(vh, s->vh, 24 * n, cudaMemcpyDeviceToHost, c->stream), "get_pl"));
    if (status)
        SWG_TRY(cuda_status(c, cudaMemcpyAsync(status, s->status, 4 * n, cudaMemcpyDeviceToHost, c->stream), "get_pl"));
    return cuda_status(c, cudaStreamSynchronize(c->stream), "get_pl");
}

int swg_system_get_tp(swg_system *s, double *rh, double *vh, int32_t *status) {
    if (!s) return SWG_ERR_ARG;
    swg_ctx *c = s->c;
    const size_t n = s->ntp;
    if (n == 0) return SWG_OK;
    if (rh) SWG_TRY(cuda_status(c, cudaMemcpyAsync(rh, s->trh, 24 * n, cudaMemcpyDeviceToHost, c->stream), "get_tp"));
    if (vh) SWG_TRY(cuda_status(c, cudaMemcpyAsync(vh, s->tvh, 24 * n, cudaMemcpyDeviceToHost, c->stream), "get_tp"));
    if (status)
        SWG_TRY(cuda_status(c, cudaMemcpyAsync(status, s->tstatus, 4 * n, cudaMemcpyDeviceToHost, c->stream), "get_tp"));
    return cuda_status(c, cudaStreamSynchronize(c->stream), "get_tp");
}

int swg_system_energy(swg_system *s, double *out) {
    if (!s || !out) return SWG_ERR_ARG;
    swg_ctx *c = s->c;
    const int n = s->npl;
    double *rows = (double *)s->red.ptr;
    double *rb = rows + std::max(n, 1);
    double *dout = rb + 3 * std::max(n, 1);
    // barycentric positions first (energy rows need rb): the final kernel computes rb,
    // so run it twice: once for rb, then rows, then again for the totals.
    k_energy_final<<<1, RB, 0, c->stream>>>(n, s->integrator == SWG_WHM, s->rh, s->vh, s->vb, s->Gmass, s->radius,
                                            s->status, s->GMcb, s->lclose, rows, rb, dout);
    SWG_TRY(L(c, "energy_rb"));
    k_energy_rows<<<grid_for(n, 128), 128, 0, c->stream>>>(n, rb, s->Gmass, s->status, rows);
    SWG_TRY(L(c, "energy_rows"));
    k_energy_final<<<1, RB, 0, c->stream>>>(n, s->integrator == SWG_WHM, s->rh, s->vh, s->vb, s->Gmass, s->radius,
                                            s->status, s->GMcb, s->lclose, rows, rb, dout);
    SWG_TRY(L(c, "energy_final"));
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(out, dout, 9 * 8, cudaMemcpyDeviceToHost, c->stream), "energy"));
    return cuda_status(c, cudaStreamSynchronize(c->stream), "energy");
}

int swg_system_collision_terms(swg_system *s, double *out) {
    if (!s || !out) return SWG_ERR_ARG;
    out[0] = s->E_collisions;
    for (int d = 0; d < 3; d++) out[1 + d] = s->L_escape[d];
    return SWG_OK;
}

int swg_system_stats(swg_system *s, int64_t *out) {
    if (!s || !out) return SWG_ERR_ARG;
    if (s->integrator == SWG_SYMBA) {
        int32_t dev[4];
        SWG_TRY(cuda_status(s->c, cudaMemcpyAsync(dev, s->rec_out, sizeof(dev), cudaMemcpyDeviceToHost, s->c->stream),
                            "stats"));
        SWG_TRY(cuda_status(s->c, cudaStreamSynchronize(s->c->stream), "stats"));
        s->stats[1] = dev[1];
        s->stats[5] = dev[2];
    }
    unsigned long long nd = 0;
    SWG_TRY(cuda_status(s->c, cudaMemcpyAsync(&nd, s->ndiscard, sizeof(nd), cudaMemcpyDeviceToHost, s->c->stream),
                        "stats"));
    SWG_TRY(cuda_status(s->c, cudaStreamSynchronize(s->c->stream), "stats"));
    std::memcpy(out, s->stats, sizeof(s->stats));
    out[4] += (int64_t)nd;
    return SWG_OK;
}

static int copy_list(swg_system *s, int32_t *l, int64_t lcap, int64_t n, int64_t cap, int64_t *nout, int32_t *i1,
                     int32_t *i2) {
    *nout = n;
    if (n > cap) return SWG_ERR_CAPACITY;
    if (n == 0) return SWG_OK;
    swg_ctx *c = s->c;
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(i1, l, 4 * n, cudaMemcpyDeviceToHost, c->stream), "list"));
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(i2, l + lcap, 4 * n, cudaMemcpyDeviceToHost, c->stream), "list"));
    return cuda_status(c, cudaStreamSynchronize(c->stream), "list");
}
int swg_system_plpl_list(swg_system *s, int64_t cap, int64_t *n, int32_t *i1, int32_t *i2) {
    if (!s || !n) return SWG_ERR_ARG;
    return copy_list(s, s->plpl_l, s->plpl_cap, s->plpl_n, cap, n, i1, i2);
}
int swg_system_pltp_list(swg_system *s, int64_t cap, int64_t *n, int32_t *i1, int32_t *i2) {
    if (!s || !n) return SWG_ERR_ARG;
    return copy_list(s, s->pltp_l, s->pltp_cap, s->pltp_n, cap, n, i1, i2);
}

int swg_system_set_state(swg_system *s, const double *rh, const double *vh, const double *trh, const double *tvh) {
    if (!s || !s->initialized) return SWG_ERR_STATE;
    swg_ctx *c = s->c;
    const size_t n = s->npl, m = s->ntp;
    if (n && rh) SWG_TRY(cuda_status(c, cudaMemcpyAsync(s->rh, rh, 24 * n, cudaMemcpyHostToDevice, c->stream), "state"));
    if (n && vh) SWG_TRY(cuda_status(c, cudaMemcpyAsync(s->vh, vh, 24 * n, cudaMemcpyHostToDevice, c->stream), "state"));
    if (m && trh) SWG_TRY(cuda_status(c, cudaMemcpyAsync(s->trh, trh, 24 * m, cudaMemcpyHostToDevice, c->stream), "state"));
    if (m && tvh) SWG_TRY(cuda_status(c, cudaMemcpyAsync(s->tvh, tvh, 24 * m, cudaMemcpyHostToDevice, c->stream), "state"));
    return SWG_OK;
}

int swg_system_reset_first_step(swg_system *s) {
    if (!s || !s->initialized) return SWG_ERR_STATE;
    swg_ctx *c = s->c;
    SWG_TRY(cuda_status(c, cudaStreamSynchronize(c->stream), "first step"));
    s->lfirst_pl = s->lfirst_tp = s->lfirstkick = 1;
    return SWG_OK;
}

int swg_system_get_state_async(swg_system *s, double *rh, double *vh, double *trh, double *tvh) {
    if (!s) return SWG_ERR_ARG;
    swg_ctx *c = s->c;
    const size_t n = s->npl, m = s->ntp;
    if (n && rh) SWG_TRY(cuda_status(c, cudaMemcpyAsync(rh, s->rh, 24 * n, cudaMemcpyDeviceToHost, c->stream), "state"));
    if (n && vh) SWG_TRY(cuda_status(c, cudaMemcpyAsync(vh, s->vh, 24 * n, cudaMemcpyDeviceToHost, c->stream), "state"));
    if (m && trh) SWG_TRY(cuda_status(c, cudaMemcpyAsync(trh, s->trh, 24 * m, cudaMemcpyDeviceToHost, c->stream), "state"));
    if (m && tvh) SWG_TRY(cuda_status(c, cudaMemcpyAsync(tvh, s->tvh, 24 * m, cudaMemcpyDeviceToHost, c->stream), "state"));
    return SWG_OK;
}

int swg_system_profile(swg_system *s, int enable) {
    if (!s) return SWG_ERR_ARG;
    s->prof.on = enable != 0;
    s->prof.n = 0;
    return SWG_OK;
}

int swg_system_profile_read(swg_system *s, double *out) {
    if (!s || !out) return SWG_ERR_ARG;
    SWG_TRY(cuda_status(s->c, cudaStreamSynchronize(s->c->stream), "profile"));
    s->prof.read(out, PROF_NCLS);
    return SWG_OK;
}

}  // extern "C"
