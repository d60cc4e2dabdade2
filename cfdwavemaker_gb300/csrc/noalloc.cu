// Allocation-free variant of the irregular-sea point evaluation.
//
// cfdwm_irregular_fields_noalloc computes the same fields as
// cfdwm_irregular_fields (Irregular::eta/u/v/w/dp without ramp or seabed
// clamp), but never allocates device memory: its workspace -- the phasors,
// ramps and first-order sums of the batch -- lives in one file-scope device
// array of fixed size that every GPU loading the library holds until the
// process exits.  It is meant for host codes that cannot let a library
// allocate while they run, for example CFD solvers that reserve all device
// memory for their own pool at start-up or run under a fixed device-memory
// budget.
//
// Host code must not use the array's name as a device address (in host code
// it names a host-side stand-in): the device address is looked up with
// cudaGetSymbolAddress, once per device, with that device current.  Under
// lazy module loading (the CUDA default) that lookup is also what loads this
// file's module and commits the array's 32 MiB, so wave_Initialize does it
// for the device it initialises on an irregular sea (noalloc_prepare), while
// the caller may still allocate; calls only reuse the address.  Calls must
// be made with that device current and on its memory.
#include "cfdwm.h"
#include "../../include/cfdwavemaker_gb300.h"

#include <cuda_runtime.h>
#include <cstdio>
#include <mutex>
#include <string>

namespace cfdwm {

const DevSea *api_loaded_sea(int *wavetype);
int api_model_device();
void api_set_error(const char *msg);
void *api_user_stream();

namespace {

constexpr size_t NOALLOC_BYTES = size_t(32) << 20;   // 32 MiB per device
constexpr int MAX_DEVICES = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

std::mutex g_setup_mtx;
void *g_scratch_ptr[MAX_DEVICES] = {nullptr};

// Device address of the scratch array on the current device (looked up once
// per device; wave_Initialize does it for the model's device).
int scratch_address(void **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) {
        cudaGetLastError();
        api_set_error("no usable CUDA device for the scratch set-up");
        return E_CUDA;
    }
    std::lock_guard<std::mutex> lk(g_setup_mtx);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            cudaGetLastError();
            api_set_error((std::string("cudaGetSymbolAddress failed: ") + cudaGetErrorString(e)).c_str());
            return E_CUDA;
        }
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return OK;
}

// device memory of device `dev` (or managed memory)
bool on_device(const void *p, int dev) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (at.type == cudaMemoryTypeManaged) return true;
    return at.type == cudaMemoryTypeDevice && at.device == dev;
}

}  // namespace

// Set-up at initialisation of an irregular sea on the current device.  A
// failure here is not an initialisation error: the entry point reports it.
int noalloc_prepare() {
    void *p = nullptr;
    return scratch_address(&p);
}

}  // namespace cfdwm

using namespace cfdwm;

extern "C" int cfdwm_irregular_fields_noalloc(const double *x, const double *y, const double *z,
                                              const double *t, long n, int mask, double *out) {
    int wt = 0;
    const DevSea *sea = api_loaded_sea(&wt);
    if (!sea) {
        api_set_error("no wave model loaded");
        return E_NOT_INITIALIZED;
    }
    if (wt != WT_IRREGULAR && wt != WT_IRR_SGRID) {
        api_set_error("cfdwm_irregular_fields_noalloc serves irregular seas only");
        return E_UNSUPPORTED;
    }
    if (n < 0) return E_BAD_ARGUMENT;
    if (n == 0) return OK;
    if ((mask & 30) && sea->order == 2 && !sea->d_tab_point) {
        api_set_error("the point-API pair table is not built for this model (wave type 5); "
                      "call cfdwm_irregular_fields once first");
        return E_UNSUPPORTED;
    }
    // the sea's tables live on the device current at wave_Initialize: the
    // call and its arrays must be on that device too
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        api_set_error("no usable CUDA device");
        return E_CUDA;
    }
    if (dev != api_model_device()) {
        char msg[160];
        std::snprintf(msg, sizeof msg,
                      "cfdwm_irregular_fields_noalloc: current device %d, but the model was initialised on "
                      "device %d", dev, api_model_device());
        api_set_error(msg);
        return E_BAD_ARGUMENT;
    }
    const void *ptrs[5] = {x, y, z, t, out};
    for (const void *p : ptrs)
        if (!p || !on_device(p, dev)) {
            api_set_error("cfdwm_irregular_fields_noalloc needs x, y, z, t and out in the memory of the "
                          "device the model was initialised on");
            return E_BAD_ARGUMENT;
        }
    size_t need = irregular_eval_scratch_bytes(*sea, n);
    if (need > NOALLOC_BYTES) {
        char msg[256];
        std::snprintf(msg, sizeof msg,
                      "batch of %ld points needs %zu bytes of workspace; the allocation-free entry "
                      "point has %zu (split the batch)", n, need, NOALLOC_BYTES);
        api_set_error(msg);
        return E_TOO_LARGE;
    }
    void *base = nullptr;
    int rc = scratch_address(&base);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)api_user_stream();
    // outputs not requested stay zero, as in cfdwm_irregular_fields
    if (cudaMemsetAsync(out, 0, sizeof(double) * 5 * (size_t)n, s) != cudaSuccess) {
        api_set_error("cudaMemsetAsync failed");
        return E_CUDA;
    }
    Workspace ws;
    ws.base = base;
    ws.bytes = NOALLOC_BYTES;
    rc = irregular_eval(*sea, n, x, y, z, t, mask, out, ws, s);
    if (rc) return rc;
    if (cudaStreamSynchronize(s) != cudaSuccess) {
        api_set_error("kernel execution failed");
        return E_CUDA;
    }
    return OK;
}
