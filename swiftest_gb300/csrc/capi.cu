// capi.cu -- context management and the kernel-level C ABI entry points.
//
// Each entry point mirrors one Fortran procedure of the reference (cited in
// include/swiftest_gb300.h).  With SWG_MEM_HOST the arrays are staged through
// the context's grow-only device slots; with SWG_MEM_DEVICE the caller's
// device pointers are used directly.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "kick_mixed.cuh"
#include "swg_internal.cuh"

namespace swg {

int cuda_status(swg_ctx *c, cudaError_t e, const char *what) {
    if (e == cudaSuccess) return SWG_OK;
    if (c) c->err = std::string(what) + ": " + cudaGetErrorString(e);
    return SWG_ERR_CUDA;
}

int launch_status(swg_ctx *c, const char *what) { return cuda_status(c, cudaGetLastError(), what); }

int ensure(swg_ctx *c, DevBuf &buf, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (buf.ptr && buf.bytes >= bytes) return SWG_OK;
    if (buf.ptr) {
        cudaFree(buf.ptr);
        buf.ptr = nullptr;
        buf.bytes = 0;
    }
    cudaError_t e = cudaMalloc(&buf.ptr, bytes);
    if (e != cudaSuccess) {
        buf.ptr = nullptr;
        if (c) c->err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
        return SWG_ERR_NOMEM;
    }
    buf.bytes = bytes;
    return SWG_OK;
}

int ensure_slot(swg_ctx *c, int slot, size_t bytes, void **out) {
    SWG_TRY(ensure(c, c->slot[slot], bytes));
    *out = c->slot[slot].ptr;
    return SWG_OK;
}

}  // namespace swg

using namespace swg;

namespace {

// Stage an input array: host -> slot, or pass the device pointer through.
template <typename T>
int stage_in(swg_ctx *c, int mem, int slot, const T *p, size_t n, T **d) {
    if (!p) {
        *d = nullptr;
        return SWG_OK;
    }
    if (mem == SWG_MEM_DEVICE) {
        *d = const_cast<T *>(p);
        return SWG_OK;
    }
    void *q;
    SWG_TRY(ensure_slot(c, slot, sizeof(T) * (n ? n : 1), &q));
    if (n) SWG_TRY(cuda_status(c, cudaMemcpyAsync(q, p, sizeof(T) * n, cudaMemcpyHostToDevice, c->stream), "H2D"));
    *d = (T *)q;
    return SWG_OK;
}
template <typename T>
int stage_out(swg_ctx *c, int mem, T *p, const T *d, size_t n) {
    if (mem == SWG_MEM_DEVICE || !p || n == 0) return SWG_OK;
    return cuda_status(c, cudaMemcpyAsync(p, d, sizeof(T) * n, cudaMemcpyDeviceToHost, c->stream), "D2H");
}
int finish(swg_ctx *c, int mem) {
    if (mem == SWG_MEM_DEVICE) return launch_status(c, "launch");
    return cuda_status(c, cudaStreamSynchronize(c->stream), "sync");
}
bool bad_mem(int mem) { return mem != SWG_MEM_HOST && mem != SWG_MEM_DEVICE; }
bool bad_prec(int p) { return p != SWG_FP64 && p != SWG_MIXED; }

}  // namespace

extern "C" {

int swg_create(swg_ctx **ctx, int device) {
    if (!ctx) return SWG_ERR_ARG;
    *ctx = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) return SWG_ERR_CUDA;
    if (device < 0 || device >= ndev) return SWG_ERR_ARG;
    e = cudaSetDevice(device);
    if (e != cudaSuccess) return SWG_ERR_CUDA;
    swg_ctx *c = new swg_ctx();
    c->device = device;
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        return SWG_ERR_CUDA;
    }
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
    *ctx = c;
    return SWG_OK;
}

int swg_destroy(swg_ctx *c) {
    if (!c) return SWG_OK;
    // systems still alive belong to this context: release them first
    while (!c->systems.empty()) swg_system_destroy((swg_system *)c->systems.back());
    while (!c->ensembles.empty()) swg_ensemble_destroy((swg_ensemble *)c->ensembles.back());
    cudaStreamSynchronize(c->stream);
    kick_sym_single_free(c);
    for (auto &b : c->slot)
        if (b.ptr) cudaFree(b.ptr);
    DevBuf *eb[] = {&c->enc.raw, &c->enc.sort, &c->enc.counters};
    for (DevBuf *b : eb)
        if (b->ptr) cudaFree(b->ptr);
    for (void *e : c->events)
        if (e) cudaEventDestroy((cudaEvent_t)e);
    cudaStreamDestroy(c->stream);
    delete c;
    return SWG_OK;
}

int swg_synchronize(swg_ctx *c) {
    if (!c) return SWG_ERR_ARG;
    return cuda_status(c, cudaStreamSynchronize(c->stream), "sync");
}

const char *swg_last_error(const swg_ctx *c) { return c ? c->err.c_str() : "no context"; }

int64_t swg_launch_count(const swg_ctx *c) { return c ? c->launches : 0; }

int swg_kick_getacch_int_all_tri_pl(swg_ctx *c, int32_t npl, int32_t nplm, const double *r, const double *Gmass,
                                    const double *radius, double *acc, int precision, int mem) {
    if (!c || npl < 0 || nplm < 0 || nplm > npl || bad_mem(mem) || bad_prec(precision)) return SWG_ERR_ARG;
    if (npl == 0) return SWG_OK;
    if (!r || !Gmass || !acc) return SWG_ERR_ARG;
    double *dr, *dg, *dR, *da;
    SWG_TRY(stage_in(c, mem, 0, r, 3 * (size_t)npl, &dr));
    SWG_TRY(stage_in(c, mem, 1, Gmass, (size_t)npl, &dg));
    SWG_TRY(stage_in(c, mem, 2, radius, (size_t)npl, &dR));
    SWG_TRY(stage_in(c, mem, 3, (const double *)acc, 3 * (size_t)npl, &da));
    if (precision == SWG_MIXED && nplm == npl && kick_sym_single_ok(npl, c->num_sms)) {
        SWG_TRY(kick_mixed_sym_single(c, npl, dr, dg, dR, da, 0));
    } else if (precision == SWG_MIXED) {
        const int nch = kick_mixed_chunks(c, npl, npl);
        SWG_TRY(ensure_kick_scratch(c, c->slot[10], kick_mixed_scratch_bytes(npl, npl, nch)));
        SWG_TRY(kick_mixed_launch(c, false, npl, npl, nplm, dr, dr, dg, dR, nullptr, da, 0, nch, c->slot[10].ptr));
    } else {
        const int mode = (npl - nplm) > nplm ? KICK_SPLIT : KICK_DIRECT;
        SWG_TRY(kick_plpl_fp64(c, npl, nplm, dr, dg, dR, da, mode, 0));
    }
    SWG_TRY(stage_out(c, mem, acc, da, 3 * (size_t)npl));
    return finish(c, mem);
}

int swg_kick_getacch_int_all_flat_pl(swg_ctx *c, int32_t npl, int32_t nplm, int64_t nplpl, const int32_t *k_plpl,
                                     const double *r, const double *Gmass, const double *radius, double *acc,
                                     int precision, int mem) {
    if (!c || npl < 0 || nplm < 0 || nplm > npl || nplpl < 0 || bad_mem(mem) || bad_prec(precision))
        return SWG_ERR_ARG;
    if (npl == 0) return SWG_OK;
    if (!r || !Gmass || !acc) return SWG_ERR_ARG;
    double *dr, *dg, *dR, *da;
    SWG_TRY(stage_in(c, mem, 0, r, 3 * (size_t)npl, &dr));
    SWG_TRY(stage_in(c, mem, 1, Gmass, (size_t)npl, &dg));
    SWG_TRY(stage_in(c, mem, 2, radius, (size_t)npl, &dR));
    SWG_TRY(stage_in(c, mem, 3, (const double *)acc, 3 * (size_t)npl, &da));
    if (!k_plpl) {
        if (nplpl != nplplm_count(npl, nplm)) {
            c->err = "nplpl does not match the canonical pair count for (npl, nplm)";
            return SWG_ERR_ARG;
        }
        if (precision == SWG_MIXED && nplm == npl && kick_sym_single_ok(npl, c->num_sms)) {
            SWG_TRY(kick_mixed_sym_single(c, npl, dr, dg, dR, da, 0));
        } else if (precision == SWG_MIXED) {
            const int nch = kick_mixed_chunks(c, npl, npl);
            SWG_TRY(ensure_kick_scratch(c, c->slot[10], kick_mixed_scratch_bytes(npl, npl, nch)));
            SWG_TRY(kick_mixed_launch(c, false, npl, npl, nplm, dr, dr, dg, dR, nullptr, da, 0, nch, c->slot[10].ptr));
        } else {
            SWG_TRY(kick_plpl_fp64(c, npl, nplm, dr, dg, dR, da, KICK_SPLIT, 0));
        }
    } else {
        int32_t *dk;
        SWG_TRY(stage_in(c, mem, 4, k_plpl, 2 * (size_t)nplpl, &dk));
        void *scr;
        SWG_TRY(ensure_slot(c, 11, sizeof(double) * 6 * (size_t)npl, &scr));
        SWG_TRY(kick_pairs(c, npl, nplpl, dk, nullptr, nullptr, dr, dg, dR, da, 1.0, (double *)scr));
    }
    SWG_TRY(stage_out(c, mem, acc, da, 3 * (size_t)npl));
    return finish(c, mem);
}

int swg_kick_getacch_int_all_tp(swg_ctx *c, int32_t ntp, int32_t npl, const double *rtp, const double *rpl,
                                const double *GMpl, const int32_t *lmask, double *acc, int precision, int mem) {
    if (!c || ntp < 0 || npl < 0 || bad_mem(mem) || bad_prec(precision)) return SWG_ERR_ARG;
    if (ntp == 0 || npl == 0) return SWG_OK;
    if (!rtp || !rpl || !GMpl || !lmask || !acc) return SWG_ERR_ARG;
    double *drt, *drp, *dg, *da;
    int32_t *dm;
    SWG_TRY(stage_in(c, mem, 0, rtp, 3 * (size_t)ntp, &drt));
    SWG_TRY(stage_in(c, mem, 1, rpl, 3 * (size_t)npl, &drp));
    SWG_TRY(stage_in(c, mem, 2, GMpl, (size_t)npl, &dg));
    SWG_TRY(stage_in(c, mem, 4, lmask, (size_t)ntp, &dm));
    SWG_TRY(stage_in(c, mem, 3, (const double *)acc, 3 * (size_t)ntp, &da));
    if (precision == SWG_MIXED) {
        const int nch = kick_mixed_chunks(c, ntp, npl);
        SWG_TRY(ensure_kick_scratch(c, c->slot[10], kick_mixed_scratch_bytes(ntp, npl, nch)));
        SWG_TRY(kick_mixed_launch(c, true, ntp, npl, 0, drt, drp, dg, nullptr, dm, da, 0, nch, c->slot[10].ptr));
    } else {
        SWG_TRY(kick_tp_fp64(c, ntp, npl, drt, drp, dg, dm, da, 0));
    }
    SWG_TRY(stage_out(c, mem, acc, da, 3 * (size_t)ntp));
    return finish(c, mem);
}

int swg_orbel_el2xv(swg_ctx *c, int32_t n, const double *mu, const double *a, const double *e, const double *inc,
                    const double *capom, const double *omega, const double *capm, double *rh, double *vh, int mem) {
    if (!c || n < 0 || bad_mem(mem)) return SWG_ERR_ARG;
    if (n == 0) return SWG_OK;
    if (!mu || !a || !e || !inc || !capom || !omega || !capm || !rh || !vh) return SWG_ERR_ARG;
    const double *in[7] = {mu, a, e, inc, capom, omega, capm};
    double *d[7], *dr = rh, *dv = vh;
    for (int k = 0; k < 7; k++) SWG_TRY(stage_in(c, mem, k, in[k], (size_t)n, &d[k]));
    if (mem == SWG_MEM_HOST) {  // outputs only: device room, no copy in
        void *q;
        SWG_TRY(ensure_slot(c, 7, 24 * (size_t)n, &q));
        dr = (double *)q;
        SWG_TRY(ensure_slot(c, 8, 24 * (size_t)n, &q));
        dv = (double *)q;
    }
    SWG_TRY(orbel_el2xv_launch(c, n, d[0], d[1], d[2], d[3], d[4], d[5], d[6], dr, dv));
    SWG_TRY(stage_out(c, mem, rh, dr, 3 * (size_t)n));
    SWG_TRY(stage_out(c, mem, vh, dv, 3 * (size_t)n));
    return finish(c, mem);
}

int swg_orbel_xv2el(swg_ctx *c, int32_t n, const double *mu, const double *rh, const double *vh, double *a,
                    double *e, double *inc, double *capom, double *omega, double *capm, double *varpi, double *lam,
                    double *f, double *cape, double *capf, int mem) {
    if (!c || n < 0 || bad_mem(mem)) return SWG_ERR_ARG;
    if (n == 0) return SWG_OK;
    if (!mu || !rh || !vh) return SWG_ERR_ARG;
    double *dmu, *dr, *dv;
    SWG_TRY(stage_in(c, mem, 0, mu, (size_t)n, &dmu));
    SWG_TRY(stage_in(c, mem, 1, rh, 3 * (size_t)n, &dr));
    SWG_TRY(stage_in(c, mem, 2, vh, 3 * (size_t)n, &dv));
    double *out[11] = {a, e, inc, capom, omega, capm, varpi, lam, f, cape, capf};
    double *dout[11];
    void *q;  // one scratch slot: the 11 output pointers (device array), then host-mode outputs
    SWG_TRY(ensure_slot(c, 22, sizeof(dout) + (mem == SWG_MEM_HOST ? 11 * 8 * (size_t)n : 0), &q));
    double *room = (double *)((char *)q + sizeof(dout));
    for (int k = 0; k < 11; k++) dout[k] = out[k] && mem == SWG_MEM_HOST ? room + (size_t)k * n : out[k];
    void *tab = q;
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(tab, dout, sizeof(dout), cudaMemcpyHostToDevice, c->stream), "H2D"));
    SWG_TRY(orbel_xv2el_launch(c, n, dmu, dr, dv, (double *const *)tab));
    for (int k = 0; k < 11; k++) SWG_TRY(stage_out(c, mem, out[k], dout[k], (size_t)n));
    return cuda_status(c, cudaStreamSynchronize(c->stream), "sync");  // the pointer table is a stack array
}

int swg_drift_all(swg_ctx *c, const double *mu, double *x, double *v, int32_t n, int32_t lgr, double inv_c2,
                  double dt, const int32_t *lmask, int32_t *iflag, int mem) {
    if (!c || n < 0 || bad_mem(mem)) return SWG_ERR_ARG;
    if (n == 0) return SWG_OK;
    if (!mu || !x || !v || !lmask || !iflag) return SWG_ERR_ARG;
    double *dmu, *dx, *dv;
    int32_t *dm, *df;
    SWG_TRY(stage_in(c, mem, 0, mu, (size_t)n, &dmu));
    SWG_TRY(stage_in(c, mem, 1, (const double *)x, 3 * (size_t)n, &dx));
    SWG_TRY(stage_in(c, mem, 2, (const double *)v, 3 * (size_t)n, &dv));
    SWG_TRY(stage_in(c, mem, 4, lmask, (size_t)n, &dm));
    SWG_TRY(stage_in(c, mem, 5, (const int32_t *)iflag, (size_t)n, &df));
    SWG_TRY(drift_all(c, dmu, 0.0, dx, dv, n, lgr, inv_c2, dt, dm, df));
    SWG_TRY(stage_out(c, mem, x, dx, 3 * (size_t)n));
    SWG_TRY(stage_out(c, mem, v, dv, 3 * (size_t)n));
    SWG_TRY(stage_out(c, mem, iflag, df, (size_t)n));
    return finish(c, mem);
}

int swg_util_sort_index(swg_ctx *c, int64_t n, const double *arr, int32_t *ind, int mem) {
    if (!c || n < 0 || n > INT32_MAX || bad_mem(mem)) return SWG_ERR_ARG;
    if (n == 0) return SWG_OK;
    if (!arr || !ind) return SWG_ERR_ARG;
    double *da;
    int32_t *di;
    void *scr;
    SWG_TRY(stage_in(c, mem, 0, arr, (size_t)n, &da));
    if (mem == SWG_MEM_DEVICE) {
        di = ind;
    } else {
        void *p;
        SWG_TRY(ensure_slot(c, 1, sizeof(int32_t) * (size_t)n, &p));
        di = (int32_t *)p;
    }
    SWG_TRY(ensure_slot(c, 2, util_sort_index_scratch_bytes(n), &scr));
    SWG_TRY(util_sort_index(c, n, da, di, scr));
    SWG_TRY(stage_out(c, mem, ind, (const int32_t *)di, (size_t)n));
    return finish(c, mem);
}

}  // extern "C"

namespace {
int enc_common(swg_ctx *c, int kind, int mode, int32_t n1, const double *r1, const double *v1, const double *renc1,
               int32_t n2, const double *r2, const double *v2, const double *renc2, double dt, int64_t cap,
               int64_t *nenc, int32_t *index1, int32_t *index2, int32_t *lvdotr, int mem) {
    if (!c || !nenc || n1 < 0 || n2 < 0 || cap < 0 || bad_mem(mem)) return SWG_ERR_ARG;
    if (mode != SWG_ENC_TRIANGULAR && mode != SWG_ENC_SORTSWEEP) return SWG_ERR_ARG;
    *nenc = 0;
    if (n1 == 0 || (kind != 0 && n2 == 0 && kind == 2)) return SWG_OK;
    double *d1r, *d1v, *d1c, *d2r = nullptr, *d2v = nullptr, *d2c = nullptr;
    SWG_TRY(stage_in(c, mem, 0, r1, 3 * (size_t)n1, &d1r));
    SWG_TRY(stage_in(c, mem, 1, v1, 3 * (size_t)n1, &d1v));
    SWG_TRY(stage_in(c, mem, 2, renc1, (size_t)n1, &d1c));
    if (kind != 0 && n2 > 0) {
        SWG_TRY(stage_in(c, mem, 3, r2, 3 * (size_t)n2, &d2r));
        SWG_TRY(stage_in(c, mem, 4, v2, 3 * (size_t)n2, &d2v));
        SWG_TRY(stage_in(c, mem, 5, renc2, (size_t)n2, &d2c));
    }
    int64_t n = 0;
    int32_t *i1, *i2, *lv;
    SWG_TRY(encounter_check_kind(c, c->enc, kind, mode, n1, d1r, d1v, d1c, n2, d2r, d2v, d2c, dt, &n, &i1, &i2, &lv));
    *nenc = n;
    if (n > cap) return SWG_ERR_CAPACITY;
    if (n == 0) return SWG_OK;
    if (!index1 || !index2 || !lvdotr) return SWG_ERR_ARG;
    const cudaMemcpyKind kd = mem == SWG_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(index1, i1, 4 * n, kd, c->stream), "enc out"));
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(index2, i2, 4 * n, kd, c->stream), "enc out"));
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(lvdotr, lv, 4 * n, kd, c->stream), "enc out"));
    return cuda_status(c, cudaStreamSynchronize(c->stream), "enc sync");
}
}  // namespace

extern "C" {

int swg_encounter_check_all_plpl(swg_ctx *c, int mode, int32_t npl, const double *r, const double *v,
                                 const double *renc, double dt, int64_t cap, int64_t *nenc, int32_t *index1,
                                 int32_t *index2, int32_t *lvdotr, int mem) {
    return enc_common(c, 0, mode, npl, r, v, renc, 0, nullptr, nullptr, nullptr, dt, cap, nenc, index1, index2,
                      lvdotr, mem);
}

int swg_encounter_check_all_plplm(swg_ctx *c, int mode, int32_t nplm, int32_t nplt, const double *rplm,
                                  const double *vplm, const double *rplt, const double *vplt, const double *rencm,
                                  const double *renct, double dt, int64_t cap, int64_t *nenc, int32_t *index1,
                                  int32_t *index2, int32_t *lvdotr, int mem) {
    return enc_common(c, 1, mode, nplm, rplm, vplm, rencm, nplt, rplt, vplt, renct, dt, cap, nenc, index1, index2,
                      lvdotr, mem);
}

int swg_encounter_check_all_pltp(swg_ctx *c, int mode, int32_t npl, int32_t ntp, const double *rpl,
                                 const double *vpl, const double *rtp, const double *vtp, const double *renc,
                                 double dt, int64_t cap, int64_t *nenc, int32_t *index1, int32_t *index2,
                                 int32_t *lvdotr, int mem) {
    return enc_common(c, 2, mode, npl, rpl, vpl, renc, ntp, rtp, vtp, nullptr, dt, cap, nenc, index1, index2,
                      lvdotr, mem);
}

}  // extern "C"

// ---------------------------------------------------------------- measurement helpers
namespace {
__global__ void k_probe_ffma(float *out, int iters, float seed) {
    float a0 = seed + threadIdx.x, a1 = a0 + 1.f, a2 = a0 + 2.f, a3 = a0 + 3.f, a4 = a0 + 4.f, a5 = a0 + 5.f,
          a6 = a0 + 6.f, a7 = a0 + 7.f;
    const float m = 0.9999999f, b = 1e-7f;
    for (int k = 0; k < iters; k++) {
        a0 = fmaf(a0, m, b);
        a1 = fmaf(a1, m, b);
        a2 = fmaf(a2, m, b);
        a3 = fmaf(a3, m, b);
        a4 = fmaf(a4, m, b);
        a5 = fmaf(a5, m, b);
        a6 = fmaf(a6, m, b);
        a7 = fmaf(a7, m, b);
    }
    const float s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == 12345.678f) out[0] = s;  // keeps the chain live
}
// The same chains in packed FP32 pairs (fma.rn.f32x2: two FMAs per lane and instruction).
__global__ void k_probe_ffma2(float *out, int iters, float seed) {
    f32x2 a[8];
#pragma unroll
    for (int k = 0; k < 8; k++) a[k] = f2_pack(seed + threadIdx.x + k, seed + threadIdx.x + k + 0.5f);
    const f32x2 m = f2_pack(0.9999999f, 0.9999999f), b = f2_pack(1e-7f, 1e-7f);
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int k = 0; k < 8; k++) a[k] = f2_fma(a[k], m, b);
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        float lo, hi;
        f2_unpack(a[k], lo, hi);
        s += lo + hi;
    }
    if (s == 12345.678f) out[0] = s;  // keeps the chains live
}
__global__ void k_probe_dfma(double *out, int iters, double seed) {
    double a0 = seed + threadIdx.x, a1 = a0 + 1.0, a2 = a0 + 2.0, a3 = a0 + 3.0;
    const double m = 0.9999999, b = 1e-7;
    for (int k = 0; k < iters; k++) {
        a0 = fma(a0, m, b);
        a1 = fma(a1, m, b);
        a2 = fma(a2, m, b);
        a3 = fma(a3, m, b);
    }
    const double s = a0 + a1 + a2 + a3;
    if (s == 12345.678) out[0] = s;
}
}  // namespace

extern "C" {

int swg_flush_l2(swg_ctx *c, int64_t bytes) {
    if (!c || bytes <= 0) return SWG_ERR_ARG;
    void *p;
    SWG_TRY(ensure_slot(c, 20, (size_t)bytes, &p));
    return cuda_status(c, cudaMemsetAsync(p, (int)(c->launches & 0xff), (size_t)bytes, c->stream), "flush");
}

int swg_event_record(swg_ctx *c, int slot) {
    if (!c || slot < 0 || slot >= 16) return SWG_ERR_ARG;
    if (!c->events[slot]) SWG_TRY(cuda_status(c, cudaEventCreate((cudaEvent_t *)&c->events[slot]), "event"));
    return cuda_status(c, cudaEventRecord((cudaEvent_t)c->events[slot], c->stream), "event");
}

int swg_event_elapsed(swg_ctx *c, int a, int b, double *ms) {
    if (!c || !ms || a < 0 || b < 0 || a >= 16 || b >= 16 || !c->events[a] || !c->events[b]) return SWG_ERR_ARG;
    SWG_TRY(cuda_status(c, cudaEventSynchronize((cudaEvent_t)c->events[b]), "event"));
    float f = 0.f;
    SWG_TRY(cuda_status(c, cudaEventElapsedTime(&f, (cudaEvent_t)c->events[a], (cudaEvent_t)c->events[b]), "event"));
    *ms = f;
    return SWG_OK;
}

int swg_probe_peak(swg_ctx *c, int kind, double *tflops) {
    if (!c || !tflops || kind < 0 || kind > 2) return SWG_ERR_ARG;
    void *p;
    SWG_TRY(ensure_slot(c, 21, 64, &p));
    const int blocks = (c->num_sms > 0 ? c->num_sms : 152) * 8, threads = 256;
    const int iters = kind == 1 ? 1 << 11 : 1 << 16;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double best = 0.0;
    for (int rep = 0; rep < 4; rep++) {
        cudaEventRecord(e0, c->stream);
        if (kind == 0)
            k_probe_ffma<<<blocks, threads, 0, c->stream>>>((float *)p, iters, 1.0f);
        else if (kind == 2)
            k_probe_ffma2<<<blocks, threads, 0, c->stream>>>((float *)p, iters, 1.0f);
        else
            k_probe_dfma<<<blocks, threads, 0, c->stream>>>((double *)p, iters, 1.0);
        cudaEventRecord(e1, c->stream);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        const double flops = 2.0 * iters * (kind == 0 ? 8 : kind == 2 ? 16 : 4) * (double)blocks * threads;
        if (rep > 0 && ms > 0.f) best = std::max(best, flops / (ms * 1e-3) / 1e12);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c->launches += 4;
    *tflops = best;
    return launch_status(c, "probe");
}

}  // extern "C"
