// kick_noalloc.cu -- the mixed-precision pl-pl kick for callers that cannot allocate
// device memory.
//
// Who needs it: a host integrator that runs inside an application which owns every
// device allocation (a memory pool, a fixed arena sized at start-up) must not call
// cudaMalloc/cudaFree mid-run: the pool has taken the memory, so a new allocation can
// fail or fragment it, and both calls can synchronize the whole device, stalling the
// work the application keeps in flight on its other streams.  The regular entry points
// grow scratch buffers on demand, so they cannot serve such a caller.  This variant
// keeps its scratch (the per-block completion counters and the float-float partial
// sums of the mixed kick) in a fixed, file-scope device array instead.
//
// Limits and sharing:
//  * the array is NOALLOC_SCRATCH_BYTES (16 MiB) and every GPU that loads the library
//    holds one copy until the process exits;
//  * npl is limited to SWG_NOALLOC_MAX_NPL; larger inputs, and a launch layout whose
//    partial sums would not fit the array (a GPU with far more SMs than GB300's 152),
//    are rejected with SWG_ERR_ARG before anything is launched;
//  * all calls on a device share the one array and it keeps the last call's contents:
//    the counters that must start at zero are cleared (cudaMemsetAsync) at the start
//    of every call, and two calls that overlap on the GPU (different streams, no
//    ordering between them) race on the array and give wrong results;
//  * the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) and the SM count with that device current; make that first
//    call before any stream capture begins.  A first call made while its stream is
//    capturing returns SWG_ERR_STATE without touching the capture.
//
// The grid (receiver blocks by partner chunks) is the one the regular mixed entry
// point takes, so wherever swg_kick_getacch_int_all_tri_pl (SWG_MIXED) runs the
// broadcast kernel (nplm < npl, or npl too small for its symmetric kernel to fill the
// GPU) the two give the same bits.
#include <cuda_runtime.h>

#include <mutex>

#include "swg_internal.cuh"

namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = size_t(16) << 20;
constexpr size_t NOALLOC_COUNTER_BYTES = size_t(64) << 10;  // 16384 block counters
constexpr int MAX_DEVICES = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

struct DeviceSetup {
    void *ptr = nullptr;
    int num_sms = 0;
    bool ready = false;
};
DeviceSetup g_setup[MAX_DEVICES];
std::mutex g_setup_mutex;

// Host code cannot use the name g_noalloc_scratch as a device address: resolve it once
// per device, with that device current.
// The lookup is refused while `st` is capturing: in the global capture mode it would
// invalidate the caller's capture.
int setup_current_device(cudaStream_t st, DeviceSetup **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return SWG_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    DeviceSetup &d = g_setup[dev];
    if (!d.ready) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) return SWG_ERR_CUDA;
        if (cs != cudaStreamCaptureStatusNone) return SWG_ERR_STATE;
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return SWG_ERR_CUDA;
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return SWG_ERR_CUDA;
        d.ptr = p;
        d.num_sms = sms;
        d.ready = true;
    }
    *out = &d;
    return SWG_OK;
}

}  // namespace

extern "C" int swg_kick_getacch_int_all_tri_pl_noalloc(int32_t npl, int32_t nplm, const double *r,
                                                       const double *Gmass, const double *radius, double *acc,
                                                       void *stream) {
    if (npl < 0 || nplm < 0 || nplm > npl) return SWG_ERR_ARG;
    if (npl > SWG_NOALLOC_MAX_NPL) return SWG_ERR_ARG;
    if (npl == 0) return SWG_OK;
    if (!r || !Gmass || !acc) return SWG_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    DeviceSetup *d = nullptr;
    int rc = setup_current_device(st, &d);
    if (rc != SWG_OK) return rc;
    const swg::MixedPlplGrid g = swg::kick_mixed_plpl_grid(d->num_sms, npl);
    if ((size_t)g.bx * sizeof(unsigned) > NOALLOC_COUNTER_BYTES ||
        (size_t)g.partials * 6 * sizeof(float) > NOALLOC_SCRATCH_BYTES - NOALLOC_COUNTER_BYTES)
        return SWG_ERR_ARG;
    if (cudaMemsetAsync(d->ptr, 0, NOALLOC_COUNTER_BYTES, st) != cudaSuccess) return SWG_ERR_CUDA;
    const cudaError_t e =
        swg::kick_mixed_plpl_on_stream(st, g, npl, nplm, r, Gmass, radius, acc, d->ptr, NOALLOC_COUNTER_BYTES);
    return e == cudaSuccess ? SWG_OK : SWG_ERR_CUDA;
}
