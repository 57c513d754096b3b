// Allocation-free variant of the per-warp flow update (rfk_warp_update).
//
// Some callers cannot allocate device memory when they run this step: a
// real-time pipeline that forbids cudaMalloc after start-up (an allocation
// can synchronise the device and stall every stream), or a host framework
// whose own allocator owns the device memory budget and does not hand out
// scratch buffers.  rfk_warp_update needs two scratch planes for the
// intermediate u + median(duhat); this variant keeps them in a file-scope
// device array instead, so the caller passes only inputs and outputs.
//
// Limits and sharing:
//  * the array holds two planes of RF_NOALLOC_MAX_PLANE floats (16 MiB per
//    device, held by every GPU that loads this library until the process
//    exits); calls with h * s above RF_NOALLOC_MAX_PLANE are rejected;
//  * every call on a device uses the same array, so calls whose kernels
//    overlap on the GPU (different streams, or different host threads)
//    race on it and corrupt each other's results; order them on one stream;
//  * nothing in the array needs to start at zero: the first kernel writes
//    every pixel of the image that the second one reads, and whatever an
//    earlier call left there is overwritten before use;
//  * host code cannot use the array's name as a device address, so the first
//    call on each device looks the address up (cudaGetSymbolAddress) with that
//    device current and caches it; make that first call before any stream
//    capture on the device.  The cached address lives as long as the
//    process's context on that device: after cudaDeviceReset it is stale,
//    so the entry point must not be used on that device again.
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "../../include/reconflow_gb300.h"
#include "rf_kernels.cuh"

namespace {

constexpr size_t kMaxPlane = RF_NOALLOC_MAX_PLANE;
constexpr int kMaxDevices = 64;

// plane 0: u + median(duhat), plane 1: v + median(dvhat)
static __device__ __align__(256) float g_warp_update_scratch[2 * kMaxPlane];

float* g_scratch_addr[kMaxDevices];
std::mutex g_scratch_mu;

rf_status noalloc_fail(rf_status st, const std::string& msg) {
    return static_cast<rf_status>(rf::set_last_error(st, msg.c_str()));
}

}  // namespace

extern "C" rf_status rfk_warp_update_noalloc(const float* duhat, const float* dvhat,
                                              const float* u, const float* v, int w, int h, int s,
                                              float* out_u, float* out_v, void* stream) {
    if (!duhat || !dvhat || !u || !v || !out_u || !out_v || w <= 0 || h <= 0 || s < w)
        return noalloc_fail(RF_ERR_INVALID_ARG, "rfk_warp_update_noalloc: bad argument");
    const size_t need = (size_t)h * (size_t)s;
    if (need > kMaxPlane)
        return noalloc_fail(RF_ERR_INVALID_ARG,
                            "rfk_warp_update_noalloc: height * stride = " + std::to_string(need) +
                                " exceeds the static scratch plane of " +
                                std::to_string(kMaxPlane) + " floats (1920x1088 is the largest "
                                "full-HD frame that fits); use rfk_warp_update with caller scratch");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return noalloc_fail(RF_ERR_CUDA, std::string("rfk_warp_update_noalloc: cudaGetDevice: ") +
                                             cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices)
        return noalloc_fail(RF_ERR_UNSUPPORTED, "rfk_warp_update_noalloc: device index too large");
    float* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_scratch_mu);
        if (!g_scratch_addr[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_warp_update_scratch);
            if (e != cudaSuccess || !p)
                return noalloc_fail(RF_ERR_CUDA,
                                    std::string("rfk_warp_update_noalloc: cudaGetSymbolAddress: ") +
                                        cudaGetErrorString(e));
            g_scratch_addr[dev] = static_cast<float*>(p);
        }
        base = g_scratch_addr[dev];
    }
    rf::LevelDims d{w, h, s};
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (rf::launch_median_add(duhat, dvhat, u, v, base, base + kMaxPlane, d, st) != 0 ||
        rf::launch_median5(base, base + kMaxPlane, out_u, out_v, d, st) != 0)
        return noalloc_fail(RF_ERR_CUDA, std::string("rfk_warp_update_noalloc: launch: ") +
                                             cudaGetErrorString(rf::last_launch_error()));
    return RF_OK;
}
