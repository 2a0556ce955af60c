// sph_ctx_download_noalloc: a field download that allocates no device memory.
//
// sph_ctx_download converts a field to FP64 in original particle order in a
// device buffer it cudaMallocs for the call and cudaFrees afterwards.  Some
// callers cannot do that: a frame-export hook inside a long-running serving
// process whose device memory is fully reserved for resident scenes (a new
// allocation can fail or fragment the reserve), and real-time drivers for
// which cudaFree is off limits because it waits for the whole device,
// stalling every other stream in flight.  This variant stages through one
// file-scope __device__ array instead, so it needs no allocation at all.
//
// The array holds kNoAllocMaxValues doubles (4 MiB).  Every GPU that loads the
// library keeps it for the life of the process, and every call shares it.
// In host code its name is only a host-side stand-in, never a device address:
// its device address is looked up with cudaGetSymbolAddress once per device
// (with that device current), on the first call made on that device, and
// that pointer is what the kernel receives.  The address is kept for the
// life of the process: a cudaDeviceReset on a device ends every context
// there, and a process that resets a device must not call this entry point
// on that device again.
#include <cuda_runtime.h>

#include <mutex>

#include "sph_device.cuh"
#include "sph_scene_base.h"

namespace sph {

constexpr size_t kNoAllocMaxValues = 524288;  // 4 MiB of doubles

static __device__ __align__(256) double g_noalloc_stage[kNoAllocMaxValues];

namespace {

std::mutex g_stage_mutex;
constexpr int kMaxDevices = 64;
double* g_stage_ptr[kMaxDevices] = {};

// Device address of the staging array on `device` (which must be current).
cudaError_t stage_address(int device, double** out)
{
    std::lock_guard<std::mutex> lock(g_stage_mutex);
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    if (!g_stage_ptr[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_stage);
        if (e != cudaSuccess) return e;
        g_stage_ptr[device] = static_cast<double*>(p);
    }
    *out = g_stage_ptr[device];
    return cudaSuccess;
}

template <typename R>
__device__ __forceinline__ void abs_pos_of(const P4<R>& p, uint32_t c, const FieldView& v, double* a)
{
    if constexpr (sizeof(R) == 4) {
        a[0] = (double)(cell_x(c) + v.ox) * v.h + (double)p.x;
        a[1] = (double)(cell_y(c) + v.oy) * v.h + (double)p.y;
        a[2] = (double)(cell_z(c) + v.oz) * v.h + (double)p.z;
    } else {
        a[0] = p.x; a[1] = p.y; a[2] = p.z;
    }
}

// Sorted-order field -> original order in FP64, written to `stage` (the
// staging array's device address).  Every one of the field's values is
// written, so nothing in the array needs clearing between calls.
template <typename R>
__global__ void k_download_staged(FieldView v, double* __restrict__ stage)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.n) return;
    const uint32_t o = v.id[i];
    if (v.kind == 2) {
        stage[o] = (double)static_cast<const R*>(v.s)[i];
        return;
    }
    const P4<R> p = static_cast<const P4<R>*>(v.v4)[i];
    if (v.kind == 1) {
        double a[3];
        abs_pos_of(p, v.cell[i], v, a);
        stage[3 * o] = a[0]; stage[3 * o + 1] = a[1]; stage[3 * o + 2] = a[2];
    } else {
        stage[3 * o] = (double)p.x; stage[3 * o + 1] = (double)p.y; stage[3 * o + 2] = (double)p.z;
    }
}

}  // namespace

int download_noalloc(SceneBase* scene, int field, double* out, std::string* err)
{
    FieldView v;
    int rc = scene->field_view(field, &v);
    if (rc != SPH_OK) { *err = scene->err; return rc; }
    if (v.count > kNoAllocMaxValues) {
        *err = "field has " + std::to_string(v.count) + " values; sph_ctx_download_noalloc stages at most " +
               std::to_string(kNoAllocMaxValues) + " (use sph_ctx_download)";
        return SPH_ERR_CAPACITY;
    }
    if (v.count == 0) return SPH_OK;
    int prev = 0;
    cudaError_t e = cudaGetDevice(&prev);
    if (e == cudaSuccess && prev != v.device) e = cudaSetDevice(v.device);
    double* stage = nullptr;
    if (e == cudaSuccess) e = stage_address(v.device, &stage);
    if (e == cudaSuccess) {
        const unsigned blocks = (v.n + 255) / 256;
        if (v.fp64) k_download_staged<double><<<blocks, 256, 0, v.stream>>>(v, stage);
        else k_download_staged<float><<<blocks, 256, 0, v.stream>>>(v, stage);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, stage, v.count * sizeof(double), cudaMemcpyDeviceToHost, v.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(v.stream);
    if (prev != v.device) cudaSetDevice(prev);
    if (e != cudaSuccess) {
        *err = std::string("sph_ctx_download_noalloc: ") + cudaGetErrorString(e);
        return SPH_ERR_CUDA;
    }
    return SPH_OK;
}

}  // namespace sph
