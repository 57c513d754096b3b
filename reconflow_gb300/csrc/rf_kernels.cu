// CUDA kernels of the Reconflow flow + depth path for sm_103a.
//
// Layout: float32 planes, row-major, `s` elements per row, every buffer sized
// for level 0 plus one zero guard row; level l uses the first h_l rows with
// stride s_l (the reference's flat reuse, Reconflow.cu:42-61).
//
// One ReconFlow inner iteration (Reconflow.cu:284-406, eight launches in the
// reference) runs as two kernels:
//   recon_a: data step (solveReconDataL1.cu:4-102), projection blend
//            (solveUVProj.cu:4-22) with uc recomputed from the current 3D
//            state (solveUcSk.cu:3-35), and the per-pixel 3x3 triangulation
//            (solve3dMinimalArea.cu:3-193);
//   recon_b: dual TV step (solveSmoothDualTVGlobal.cu:4-65), 3x3 median of
//            the 3D points (medianFilter.cu:166-243), outlier clean-up
//            (solve3dMinimalArea.cu:248-297) and the multiplier update
//            (solveUcSk.cu:80-97).
// All pixel-local state (duhat, p, uproj, sk) is updated in place: each is
// read at a neighbour only by the other kernel of the pair.
#include <atomic>
#include <cooperative_groups.h>
#include <cstdint>
#include <cstdlib>

#include "../../include/reconflow_gb300.h"
#include "rf_alloc.h"
#include "rf_kernels.cuh"
#include "rf_ops.cuh"

namespace {

// allocation gate (rf_alloc.h): the allocation numbered g_fail_at since the
// last rf_test_fail_alloc call fails; 0 = none
std::atomic<long long> g_alloc_count{0};
std::atomic<long long> g_fail_at{-1};

long long fail_at() {
    long long v = g_fail_at.load();
    if (v < 0) {
        const char* e = std::getenv("RF_FAIL_ALLOC");
        long long k = e ? std::atoll(e) : 0;
        long long expect = -1;
        g_fail_at.compare_exchange_strong(expect, k < 0 ? 0 : k);
        v = g_fail_at.load();
    }
    return v;
}

bool injected_failure() {
    const long long k = fail_at();
    return k > 0 && g_alloc_count.fetch_add(1) + 1 == k;
}

}  // namespace

namespace rf {

cudaError_t dev_malloc(void** p, size_t bytes) {
    if (injected_failure()) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMalloc(p, bytes);
}

cudaError_t host_malloc(void** p, size_t bytes) {
    if (injected_failure()) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMallocHost(p, bytes);
}

namespace {

constexpr int BX = 32;
constexpr int BY = 8;

inline dim3 grid_for(int w, int h) { return dim3((w + BX - 1) / BX, (h + BY - 1) / BY); }

// the error the last failed launch helper consumed (cudaGetLastError clears
// it), for the caller's message
thread_local cudaError_t t_launch_error = cudaSuccess;

inline int check_launch() {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) t_launch_error = e;
    return e == cudaSuccess ? 0 : 1;
}

// ---------------------------------------------------------------------------
// Input conversion (rgbToGray.cu:3-77)
// ---------------------------------------------------------------------------
__global__ void k_convert(const void* __restrict__ in, int type, int w, int h, int in_pitch,
                          float* __restrict__ out, int s) {
    int ix = blockIdx.x * blockDim.x + threadIdx.x;
    int iy = blockIdx.y * blockDim.y + threadIdx.y;
    if (ix >= w || iy >= h) return;
    size_t i = (size_t)ix + (size_t)iy * in_pitch;
    float g;
    if (type == 1) {
        const uint8_t* p = static_cast<const uint8_t*>(in) + 3 * i;
        g = ((float)p[0] + (float)p[1] + (float)p[2]) / 3.0f;
        g = g / 256.0f;
    } else if (type == 2) {
        g = (float)static_cast<const uint8_t*>(in)[i] / 256.0f;
    } else if (type == 3) {
        g = (float)static_cast<const uint16_t*>(in)[i] / 65536.0f;
    } else {
        g = static_cast<const float*>(in)[i];
    }
    out[ix + iy * s] = g;
}

// ---------------------------------------------------------------------------
// Pyramid (downscale.cu:6-48, upscale.cu:14-27)
// ---------------------------------------------------------------------------
__global__ void k_downscale2(const float* __restrict__ a, const float* __restrict__ b, LevelDims f,
                             LevelDims c, float* __restrict__ oa, float* __restrict__ ob) {
    int ix = blockIdx.x * blockDim.x + threadIdx.x;
    int iy = blockIdx.y * blockDim.y + threadIdx.y;
    if (ix >= c.w || iy >= c.h) return;
    oa[ix + iy * c.s] = 0.25f * downscale_px(a, f, c.w, c.h, ix, iy);
    ob[ix + iy * c.s] = 0.25f * downscale_px(b, f, c.w, c.h, ix, iy);
}

__global__ void k_downscale(const float* __restrict__ src, LevelDims f, LevelDims c, float scale,
                            int scaled, float* __restrict__ out) {
    int ix = blockIdx.x * blockDim.x + threadIdx.x;
    int iy = blockIdx.y * blockDim.y + threadIdx.y;
    if (ix >= c.w || iy >= c.h) return;
    float sum = downscale_px(src, f, c.w, c.h, ix, iy);
    out[ix + iy * c.s] = scaled ? scale * 0.25f * sum : 0.25f * sum;
}

struct UpscaleArgs {
    const float* src[12];
    float* dst[12];
    float scale[12];
    int n;
};

__global__ void k_upscale_fields(UpscaleArgs a, LevelDims c, LevelDims f) {
    int ix = blockIdx.x * blockDim.x + threadIdx.x;
    int iy = blockIdx.y * blockDim.y + threadIdx.y;
    if (ix >= f.w || iy >= f.h) return;
    float x = ((float)ix + 0.5f) / (float)f.w;
    float y = ((float)iy + 0.5f) / (float)f.h;
    Taps tx = taps_of(x, c.w);
    Taps ty = taps_of(y, c.h);
    int pos = ix + iy * f.s;
#pragma unroll 1
    for (int i = 0; i < a.n; i++) a.dst[i][pos] = bilerp(a.src[i], c.s, tx, ty) * a.scale[i];
}

// ---------------------------------------------------------------------------
// Warp and derivatives (warpImage.cu:15-29, computeDerivatives.cu:8-57)
// ---------------------------------------------------------------------------
__global__ void k_warp(const float* __restrict__ I1, const float* __restrict__ u,
                       const float* __restrict__ v, LevelDims d, float* __restrict__ out) {
    int ix = blockIdx.x * blockDim.x + threadIdx.x;
    int iy = blockIdx.y * blockDim.y + threadIdx.y;
    if (ix >= d.w || iy >= d.h) return;
    warp_px(I1, u, v, d, out, ix, iy);
}

__global__ void k_derivatives(const float* __restrict__ I0, const float* __restrict__ I1,
                              LevelDims d, float* __restrict__ Ix, float* __restrict__ Iy,
                              float* __restrict__ Iz) {
    int ix = blockIdx.x * blockDim.x + threadIdx.x;
    int iy = blockIdx.y * blockDim.y + threadIdx.y;
    if (ix >= d.w || iy >= d.h) return;
    derivatives_px(I0, I1, d, Ix, Iy, Iz, ix, iy);
}

// the two fused (warp_deriv_tile): one BX x BY tile per block
__global__ void __launch_bounds__(BX* BY) k_warp_deriv(const float* __restrict__ I0,
                                                       const float* __restrict__ I1,
                                                       const float* __restrict__ u,
                                                       const float* __restrict__ v, LevelDims d,
                                                       float* __restrict__ Ix,
                                                       float* __restrict__ Iy,
                                                       float* __restrict__ Iz) {
    __shared__ float sm[2 * (BX + 4) * (BY + 4)];
    warp_deriv_tile(I0, I1, u, v, d, blockIdx.x * BX, blockIdx.y * BY, BX, BY, sm, Ix, Iy, Iz);
}

// ---------------------------------------------------------------------------
// ReconFlow inner iteration, part A: data step, projection blend, Solve3d
// ---------------------------------------------------------------------------
#ifndef RF_MINB_A
#define RF_MINB_A 1
#endif
#ifndef RF_MINB_B
#define RF_MINB_B 4  // 64 registers: 4 blocks per SM (fewer registers spill; measured slower)
#endif
// Programmatic dependent launch: a kernel launched with the programmatic
// stream-serialization attribute may start while its predecessor drains;
// griddepcontrol.wait blocks until the predecessor has completed and its
// writes are visible, and launch_dependents lets the successor be scheduled.
// Both are no-ops for a normal launch.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_release() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <int PRIOR>
__global__ void __launch_bounds__(BX* BY, RF_MINB_A) k_recon_a(ReconFields f, const LevelConsts* __restrict__ lcp,
                                                    Weights wt, LevelDims d, int first,
                                                    int uc_from_buffer) {
    pdl_wait();
    pdl_release();
    int ix = blockIdx.x * blockDim.x + threadIdx.x;
    int iy = blockIdx.y * blockDim.y + threadIdx.y;
    if (ix >= d.w || iy >= d.h) return;
    recon_a_px<PRIOR>(f, *lcp, wt, d, ix, iy, first, uc_from_buffer);
}

__global__ void __launch_bounds__(BX* BY, RF_MINB_B) k_recon_b(ReconFields f, Weights wt, LevelDims d,
                                                    int first) {
    pdl_wait();
    pdl_release();
    int ix = blockIdx.x * blockDim.x + threadIdx.x;
    int iy = blockIdx.y * blockDim.y + threadIdx.y;
    if (ix >= d.w || iy >= d.h) return;
    recon_b_px(f, wt, d, ix, iy, first);
}

// ---------------------------------------------------------------------------
// Every inner iteration of one warp of a small level in one launch: a
// thread-block cluster of kClusterCtas CTAs covers the level (grid-stride
// over its pixels) and runs part A, a cluster barrier, part B, a cluster
// barrier, n_iters times.  The barrier (barrier.cluster arrive.release /
// wait.acquire) stands where the launch boundary was: part A reads p, X and
// sk that part B wrote at other pixels, B reads duhat and X1 that A wrote,
// and within a part no thread reads what another writes, so the per-pixel
// code and every value are those of the two-launch loop.  The state stays
// in global memory (a level this small lives in L2).  Every thread runs
// every loop iteration and reaches every barrier (no early exit).
// ---------------------------------------------------------------------------
constexpr int kClusterCtas = 16;
constexpr int kClusterThreads = 512;

template <int PRIOR>
__global__ void __launch_bounds__(kClusterThreads, 1)
    k_recon_cluster(ReconFields f, const LevelConsts* __restrict__ lcp, Weights wt, LevelDims d,
                    int n_iters, int uc_from_buffer) {
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    const int nthr = gridDim.x * blockDim.x;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int npx = d.w * d.h;
    for (int it = 0; it < n_iters; it++) {
        const int first = it == 0 ? 1 : 0;
        const int ucb = it == 0 ? uc_from_buffer : 0;
        for (int i = tid; i < npx; i += nthr)
            recon_a_px<PRIOR>(f, *lcp, wt, d, i % d.w, i / d.w, first, ucb);
        cluster.sync();
        for (int i = tid; i < npx; i += nthr) recon_b_px(f, wt, d, i % d.w, i / d.w, first);
        cluster.sync();
    }
}

// ---------------------------------------------------------------------------
// Plain TV-L1 (solveDataL1.cu:4-91 + solveSmoothDualTVGlobal.cu:4-65)
// ---------------------------------------------------------------------------
__global__ void k_plain_data(float* __restrict__ duhat0, float* __restrict__ dvhat0,
                             const float* __restrict__ pu1, const float* __restrict__ pu2,
                             const float* __restrict__ pv1, const float* __restrict__ pv2,
                             const float* __restrict__ Ix, const float* __restrict__ Iy,
                             const float* __restrict__ Iz, Weights wt, LevelDims d, int first) {
    int ix = blockIdx.x * blockDim.x + threadIdx.x;
    int iy = blockIdx.y * blockDim.y + threadIdx.y;
    if (ix >= d.w || iy >= d.h) return;
    plain_data_px(duhat0, dvhat0, pu1, pu2, pv1, pv2, Ix, Iy, Iz, wt, d, first, ix, iy);
}

__global__ void k_plain_tv(const float* __restrict__ duhat, const float* __restrict__ dvhat,
                           float* __restrict__ pu1, float* __restrict__ pu2,
                           float* __restrict__ pv1, float* __restrict__ pv2, Weights wt,
                           LevelDims d, int first) {
    int ix = blockIdx.x * blockDim.x + threadIdx.x;
    int iy = blockIdx.y * blockDim.y + threadIdx.y;
    if (ix >= d.w || iy >= d.h) return;
    plain_tv_px(duhat, dvhat, pu1, pu2, pv1, pv2, wt, d, first, ix, iy);
}

// ---------------------------------------------------------------------------
// 5x5 medians (medianFilter.cu:3-75): taps clamp along one axis, 0 at corners
// ---------------------------------------------------------------------------
// u + median5(duhat): MedianFilter then Add (Reconflow.cu:410-416)
// Both 5x5 median kernels take two rows per thread (pixels (ix, iy) and
// (ix, iy + 1), iy even): the windows share 20 taps (median5_pair2).
__global__ void k_median_add(const float* __restrict__ duhat, const float* __restrict__ dvhat,
                             const float* u, const float* v, float* ou, float* ov, LevelDims d) {
    int ix = blockIdx.x * blockDim.x + threadIdx.x;
    int iy = 2 * (blockIdx.y * blockDim.y + threadIdx.y);
    if (ix >= d.w || iy >= d.h) return;
    float mu[2], mv[2];
    median5_pair2(duhat, dvhat, ix, iy, d, mu, mv);
    const int pos = ix + iy * d.s;
    const bool has1 = iy + 1 < d.h;
    const float a0 = u[pos] + mu[0], b0 = v[pos] + mv[0];
    float a1 = 0.0f, b1 = 0.0f;
    if (has1) {
        a1 = u[pos + d.s] + mu[1];
        b1 = v[pos + d.s] + mv[1];
    }
    ou[pos] = a0;
    ov[pos] = b0;
    if (has1) {
        ou[pos + d.s] = a1;
        ov[pos + d.s] = b1;
    }
}

__global__ void k_median5(const float* __restrict__ u, const float* __restrict__ v,
                          float* __restrict__ ou, float* __restrict__ ov, LevelDims d) {
    int ix = blockIdx.x * blockDim.x + threadIdx.x;
    int iy = 2 * (blockIdx.y * blockDim.y + threadIdx.y);
    if (ix >= d.w || iy >= d.h) return;
    float mu[2], mv[2];
    median5_pair2(u, v, ix, iy, d, mu, mv);
    ou[ix + iy * d.s] = mu[0];
    ov[ix + iy * d.s] = mv[0];
    if (iy + 1 < d.h) {
        ou[ix + (iy + 1) * d.s] = mu[1];
        ov[ix + (iy + 1) * d.s] = mv[1];
    }
}

__global__ void k_median3d(const float* __restrict__ X, const float* __restrict__ Y,
                           const float* __restrict__ Z, float* __restrict__ X1,
                           float* __restrict__ Y1, float* __restrict__ Z1, LevelDims d) {
    int ix = blockIdx.x * blockDim.x + threadIdx.x;
    int iy = blockIdx.y * blockDim.y + threadIdx.y;
    if (ix >= d.w || iy >= d.h) return;
    float mX[9], mY[9], mZ[9];
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
        for (int i = 0; i < 3; i++) {
            int at = median3_tap(ix + i - 1, iy + j - 1, d.w, d.h, d.s);
            int k = j * 3 + i;
            mX[k] = at >= 0 ? X[at] : 0.0f;
            mY[k] = at >= 0 ? Y[at] : 0.0f;
            mZ[k] = at >= 0 ? Z[at] : 0.0f;
        }
    int pos = ix + iy * d.s;
    X1[pos] = median9_exchange(mX);
    Y1[pos] = median9_exchange(mY);
    Z1[pos] = median9_exchange(mZ);
}

__global__ void k_solve_uc(const float* __restrict__ X, const float* __restrict__ Y,
                           const float* __restrict__ Z, const LevelConsts* __restrict__ lc,
                           LevelDims d, float* __restrict__ uc, float* __restrict__ vc) {
    int ix = blockIdx.x * blockDim.x + threadIdx.x;
    int iy = blockIdx.y * blockDim.y + threadIdx.y;
    if (ix >= d.w || iy >= d.h) return;
    int pos = ix + iy * d.s;
    float a, b;
    project_uc(*lc, X[pos], Y[pos], Z[pos], ix, iy, a, b);
    uc[pos] = a;
    vc[pos] = b;
}

__global__ void k_inv_depth(const float* __restrict__ Z, LevelDims d, float* __restrict__ out) {
    int ix = blockIdx.x * blockDim.x + threadIdx.x;
    int iy = blockIdx.y * blockDim.y + threadIdx.y;
    if (ix >= d.w || iy >= d.h) return;
    int pos = ix + iy * d.s;
    out[pos] = 1.0f / Z[pos];
}

// RemoveEdgeArtifacts3DKernel (solve3dMinimalArea.cu:320-378)
__global__ void k_remove_edge(const float* __restrict__ X0, const float* __restrict__ Y0,
                              const float* __restrict__ Z0, int range, float maxArea, LevelDims d,
                              float* __restrict__ X1, float* __restrict__ Y1,
                              float* __restrict__ Z1) {
    int ix = blockIdx.x * blockDim.x + threadIdx.x;
    int iy = blockIdx.y * blockDim.y + threadIdx.y;
    if (ix >= d.w || iy >= d.h) return;
    const int s = d.s, pos = ix + iy * s;
    float Xx, Yx, Zx, Xy, Yy, Zy;
    if (ix + range > d.w) {
        int a = ix - range + iy * s;
        Xx = -X0[a] + X0[pos]; Yx = -Y0[a] + Y0[pos]; Zx = -Z0[a] + Z0[pos];
    } else {
        int a = ix + range + iy * s;
        Xx = X0[a] - X0[pos]; Yx = Y0[a] - Y0[pos]; Zx = Z0[a] - Z0[pos];
    }
    if (iy + range > d.h) {
        int a = ix + (iy - range) * s;
        Xy = -X0[a] + X0[pos]; Yy = -Y0[a] + Y0[pos]; Zy = -Z0[a] + Z0[pos];
    } else {
        int a = ix + (iy + range) * s;
        Xy = X0[a] - X0[pos]; Yy = Y0[a] - Y0[pos]; Zy = Z0[a] - Z0[pos];
    }
    float area = sqrtf((Yx * Zy - Zx * Yy) * (Yx * Zy - Zx * Yy) +
                       (Zx * Xy - Xx * Zy) * (Zx * Xy - Xx * Zy) +
                       (Xx * Yy - Yx * Xy) * (Xx * Yy - Yx * Xy));
    if (area > maxArea) {
        X1[pos] = 0.0f; Y1[pos] = 0.0f; Z1[pos] = 0.0f;
    } else {
        X1[pos] = X0[pos]; Y1[pos] = Y0[pos]; Z1[pos] = Z0[pos];
    }
}

// Middlebury colour wheel (flowToHSV.cu:194-302); entry 55 (reached when the
// angle term rounds to exactly one) wraps to entry 0.
__constant__ float c_wheel[3][55] = {
    {255, 255, 255, 255, 255, 255, 255, 255, 255, 255, 255, 255, 255, 255, 255, 255, 213, 170, 128,
     85,  43,  0,   0,   0,   0,   0,   0,   0,   0,   0,   0,   0,   0,   0,   0,   0,   0,   19,
     39,  58,  78,  98,  117, 137, 156, 176, 196, 215, 235, 255, 255, 255, 255, 255, 255},
    {0,   17,  34,  51,  68,  85,  102, 119, 136, 153, 170, 187, 204, 221, 238, 255, 255, 255, 255,
     255, 255, 255, 255, 255, 255, 255, 232, 209, 186, 163, 140, 116, 93,  70,  47,  24,  0,   0,
     0,   0,   0,   0,   0,   0,   0,   0,   0,   0,   0,   0,   0,   0,   0,   0,   0},
    {0,   0,   0,   0,   0,   0,   0,   0,   0,   0,   0,   0,   0,   0,   0,   0,   0,   0,   0,
     0,   0,   0,   63,  127, 191, 255, 255, 255, 255, 255, 255, 255, 255, 255, 255, 255, 255, 255,
     255, 255, 255, 255, 255, 255, 255, 255, 255, 255, 255, 255, 213, 170, 128, 85,  43}};

__global__ void k_flow_color(const float* __restrict__ u, const float* __restrict__ v,
                             LevelDims d, float flow_scale, float* __restrict__ rgb) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    int r = blockIdx.y * blockDim.y + threadIdx.y;
    if (c >= d.w || r >= d.h) return;
    int pos = c + d.s * r;
    // the flow vector in units of flow_scale, its length and its angle
    // mapped onto the wheel's 55 hues (the hue position wraps from the last
    // entry back to the first)
    float fx = u[pos] / flow_scale;
    float fy = v[pos] / flow_scale;
    const int n_hues = 55;
    float len = sqrtf(fx * fx + fy * fy);
    float ang = atan2f(-fy, -fx) / 3.14159f;
    float hue = (ang + 1) / 2 * ((float)n_hues - 1) + 1;
    int lo = (int)floorf(hue);
    int hi = lo + 1;
    if (hi == n_hues + 1) hi = 1;
    float t = hue - (float)lo;
    lo %= n_hues;
    hi %= n_hues;
    float col[3];
#pragma unroll
    for (int ch = 0; ch < 3; ch++) {
        float mix = (1 - t) * (c_wheel[ch][lo] / 255.0f) + t * (c_wheel[ch][hi] / 255.0f);
        // inside the unit circle, desaturate towards white; outside, darken
        if (len <= 1) mix = 1 - len * (1 - mix);
        else mix = mix * 0.75f;
        col[ch] = mix;
    }
    // float3 (x, y, z) = (B, G, R) as the reference stores it
    rgb[3 * pos + 0] = col[2];
    rgb[3 * pos + 1] = col[1];
    rgb[3 * pos + 2] = col[0];
}

}  // namespace

// Energy of a solution on level 0 (no reference counterpart; see
// rf_energy): per-block double partial sums, then one block adds the
// partials in a fixed order, so the result is deterministic.
constexpr int kEnergyThreads = 256;

// One pixel's energy: per-pixel terms in FP32 (GB300's FP64 division and
// square root would bound the kernel).
__device__ __forceinline__ float energy_px(const EnergyArgs& a, LevelDims d, int ix, int iy) {
    const int s = d.s, pos = ix + iy * s;
    float x = ((float)ix + a.u[pos] + 0.5f) / (float)d.w;
    float y = ((float)iy + a.v[pos] + 0.5f) / (float)d.h;
    float i1w = tex2d(a.I1, d.w, d.h, s, x, y);
    const float u0 = a.u[pos], v0 = a.v[pos];
    const float data = a.lambda * fabsf(i1w - a.I0[pos]);
    const float ux = ix + 1 < d.w ? a.u[pos + 1] - u0 : 0.0f;
    const float uy = iy + 1 < d.h ? a.u[pos + s] - u0 : 0.0f;
    const float vx = ix + 1 < d.w ? a.v[pos + 1] - v0 : 0.0f;
    const float vy = iy + 1 < d.h ? a.v[pos + s] - v0 : 0.0f;
    const float tv = sqrtf(ux * ux + uy * uy) + sqrtf(vx * vx + vy * vy);
    float proj = 0.0f;
    if (a.recon) {
        const float Xp = a.X[pos], Yp = a.Y[pos], Zp = a.Z[pos];
        const float X2 = a.R1f[0] * Xp + a.R1f[1] * Yp + a.R1f[2] * Zp + a.t1f[0];
        const float Y2 = a.R1f[3] * Xp + a.R1f[4] * Yp + a.R1f[5] * Zp + a.t1f[1];
        const float Z2 = a.R1f[6] * Xp + a.R1f[7] * Yp + a.R1f[8] * Zp + a.t1f[2];
        const float uc = a.fxf * X2 / Z2 + a.cxf - (float)ix;
        const float vc = a.fxf * Y2 / Z2 + a.cyf - (float)iy;
        const float du = u0 - uc, dv = v0 - vc;
        float r2 = du * du + dv * dv;
        if (!(r2 < 1.0f)) r2 = 1.0f;  // truncated at 1 px^2 (NaN included)
        proj = 0.5f * a.alpha_proj * r2;
    }
    float px_e = data + tv + proj;
    // a pixel whose flow is not finite (a NaN or infinite gradient) counts
    // each term at its cap: a unit brightness residual, unit gradients of u
    // and v, the truncated reprojection residual
    if (!isfinite(px_e)) px_e = a.lambda + 2.0f + (a.recon ? 0.5f * a.alpha_proj : 0.0f);
    return px_e;
}

// Block `blk` of `nblk` of one energy evaluation: its grid-stride share of
// the pixels (pixel i = iy * w + ix, then i + step, ...).  Each thread sums
// its own pixels in FP32 in that order (at most a few dozen: GB300's FP64
// pipe, not memory, bounded a per-pixel double sum), then the warp and the
// block add the thread sums in double, in a fixed order, into partial[blk].
__device__ __forceinline__ void energy_block(const EnergyArgs& a, LevelDims d, int blk, int nblk,
                                             double* partial) {
    __shared__ double red[kEnergyThreads / 32];
    float et = 0.0f;
    const int npx = d.w * d.h;
    const int step = nblk * kEnergyThreads;
    int i = blk * kEnergyThreads + (int)threadIdx.x;
    // (ix, iy) of pixel i, advanced by `step` without a division per pixel
    int iy = i / d.w, ix = i - iy * d.w;
    const int sy = step / d.w, sx = step - sy * d.w;
    // two pixels per pass, so that their loads overlap; added in order
    while (i + step < npx) {
        int ix1 = ix + sx, iy1 = iy + sy;
        if (ix1 >= d.w) {
            ix1 -= d.w;
            iy1++;
        }
        const float e0 = energy_px(a, d, ix, iy);
        const float e1 = energy_px(a, d, ix1, iy1);
        et += e0;
        et += e1;
        i += 2 * step;
        ix = ix1 + sx;
        iy = iy1 + sy;
        if (ix >= d.w) {
            ix -= d.w;
            iy++;
        }
    }
    if (i < npx) et += energy_px(a, d, ix, iy);
    double e = (double)et;
    for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = e;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < kEnergyThreads / 32; k++) t += red[k];
        partial[blk] = t;
    }
}

__global__ void __launch_bounds__(kEnergyThreads) k_energy_partial(EnergyArgs a, LevelDims d,
                                                                   double* partial) {
    energy_block(a, d, blockIdx.x, gridDim.x, partial);
}

// One warp: lane l adds partials l, l + 32, ... in order, then a fixed
// shuffle tree adds the 32 lane sums, so the result is deterministic.
__device__ __forceinline__ void energy_final(const double* partial, int n, double* out) {
    const int lane = threadIdx.x;
    double t = 0.0;
    for (int k = lane; k < n; k += 32) t += partial[k];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (lane == 0) *out = t;
}

__global__ void k_energy_final(const double* partial, int n, double* out) {
    energy_final(partial, n, out);
}

// Many evaluations in one launch: block b belongs to the job whose block
// range holds it and does that job's block b - first_block, so every job's
// partials and sum are the ones its own two launches would make.
__global__ void __launch_bounds__(kEnergyThreads) k_energy_partial_jobs(const EnergyJob* jobs,
                                                                        int n) {
    const int b = blockIdx.x;
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].first_block <= b)
            lo = mid;
        else
            hi = mid - 1;
    }
    const EnergyJob& j = jobs[lo];
    energy_block(j.a, j.d, b - j.first_block, j.nblocks, j.partial);
}

// The same blocks on a 2D grid: blockIdx.y = the job, blockIdx.x = its
// block (blocks past the job's count return), no search.
__global__ void __launch_bounds__(kEnergyThreads) k_energy_partial_grid(const EnergyJob* jobs) {
    const EnergyJob& j = jobs[blockIdx.y];
    if ((int)blockIdx.x >= j.nblocks) return;
    energy_block(j.a, j.d, (int)blockIdx.x, j.nblocks, j.partial);
}

__global__ void k_energy_final_jobs(const EnergyJob* jobs) {
    const EnergyJob& j = jobs[blockIdx.x];
    energy_final(j.partial, j.nblocks, j.out);
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
int launch_status() { return check_launch(); }

cudaError_t last_launch_error() {
    const cudaError_t e = t_launch_error;
    t_launch_error = cudaSuccess;
    return e;
}

int launch_convert(const void* in, int type, int w, int h, int in_pitch, float* out, int s,
                   cudaStream_t st) {
    k_convert<<<grid_for(w, h), dim3(BX, BY), 0, st>>>(in, type, w, h, in_pitch, out, s);
    return check_launch();
}

int launch_downscale2(const float* a, const float* b, LevelDims fine, LevelDims coarse, float* oa,
                      float* ob, cudaStream_t st) {
    k_downscale2<<<grid_for(coarse.w, coarse.h), dim3(BX, BY), 0, st>>>(a, b, fine, coarse, oa, ob);
    return check_launch();
}

int launch_downscale(const float* src, LevelDims fine, LevelDims coarse, float scale, bool scaled,
                     float* out, cudaStream_t st) {
    k_downscale<<<grid_for(coarse.w, coarse.h), dim3(BX, BY), 0, st>>>(src, fine, coarse, scale,
                                                                      scaled ? 1 : 0, out);
    return check_launch();
}

int launch_warp(const float* I1, const float* u, const float* v, LevelDims d, float* out,
                cudaStream_t st) {
    k_warp<<<grid_for(d.w, d.h), dim3(BX, BY), 0, st>>>(I1, u, v, d, out);
    return check_launch();
}

int launch_warp_deriv(const float* I0, const float* I1, const float* u, const float* v,
                      LevelDims d, float* Ix, float* Iy, float* Iz, cudaStream_t st) {
    k_warp_deriv<<<grid_for(d.w, d.h), dim3(BX, BY), 0, st>>>(I0, I1, u, v, d, Ix, Iy, Iz);
    return check_launch();
}

int launch_derivatives(const float* I0, const float* I1w, LevelDims d, float* Ix, float* Iy,
                       float* Iz, cudaStream_t st) {
    k_derivatives<<<grid_for(d.w, d.h), dim3(BX, BY), 0, st>>>(I0, I1w, d, Ix, Iy, Iz);
    return check_launch();
}

bool use_pdl() {
    static int v = -1;
    if (v < 0) {
        // opt-in (RF_PDL=1): measured no gain inside the captured graph on GB300
        const char* e = std::getenv("RF_PDL");
        v = (e && e[0] == '1') ? 1 : 0;
    }
    return v == 1;
}

// Launch with the programmatic stream-serialization attribute (see pdl_wait).
template <typename... KArgs, typename... Args>
int launch_pdl(void (*kern)(KArgs...), dim3 g, dim3 b, cudaStream_t st, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = g;
    cfg.blockDim = b;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = use_pdl() ? 1 : 0;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, kern, args...);
    if (e != cudaSuccess) t_launch_error = e;
    return e == cudaSuccess ? 0 : 1;
}

int launch_recon_a(const ReconFields& f, const LevelConsts* lc, const Weights& wt, LevelDims d,
                   bool first, bool uc_from_buffer, int prior, cudaStream_t st, dim3 b) {
    dim3 g((d.w + b.x - 1) / b.x, (d.h + b.y - 1) / b.y);
    int fi = first ? 1 : 0, ub = uc_from_buffer ? 1 : 0;
    if (prior == 1) return launch_pdl(k_recon_a<1>, g, b, st, f, lc, wt, d, fi, ub);
    if (prior == 2) return launch_pdl(k_recon_a<2>, g, b, st, f, lc, wt, d, fi, ub);
    return launch_pdl(k_recon_a<0>, g, b, st, f, lc, wt, d, fi, ub);
}

int launch_recon_b(const ReconFields& f, const Weights& wt, LevelDims d, bool first,
                   cudaStream_t st, dim3 b) {
    dim3 g((d.w + b.x - 1) / b.x, (d.h + b.y - 1) / b.y);
    return launch_pdl(k_recon_b, g, b, st, f, wt, d, first ? 1 : 0);
}

#ifdef RF_BOUNDS_CHECK
__global__ void k_oob_selftest(ReconFields f) { RF_AT(f, duhat, f.extent) += 0.0f; }
#endif

unsigned long long kernels_oob_take(long long* first) {
#ifdef RF_BOUNDS_CHECK
    return rf_oob_take(first);
#else
    (void)first;
    return 0;
#endif
}

int launch_oob_selftest() {
#ifdef RF_BOUNDS_CHECK
    ReconFields f{};
    f.extent = 1;  // f.duhat is never dereferenced: index 1 is redirected to the sink
    k_oob_selftest<<<1, 1>>>(f);
    return check_launch();
#else
    return 1;
#endif
}

int launch_recon_cluster(const ReconFields& f, const LevelConsts* lc, const Weights& wt,
                         LevelDims d, int n_iters, bool uc_from_buffer, int prior,
                         cudaStream_t st) {
    void (*kern)(ReconFields, const LevelConsts*, Weights, LevelDims, int, int) =
        prior == 1 ? k_recon_cluster<1> : (prior == 2 ? k_recon_cluster<2> : k_recon_cluster<0>);
    static bool attr_set[3] = {false, false, false};
    const int k = prior < 0 || prior > 2 ? 0 : prior;
    if (!attr_set[k]) {
        // 16 CTAs is above the portable cluster size of 8
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) {
            t_launch_error = e;
            return 1;
        }
        attr_set[k] = true;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(kClusterCtas);
    cfg.blockDim = dim3(kClusterThreads);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kClusterCtas;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e =
        cudaLaunchKernelEx(&cfg, kern, f, lc, wt, d, n_iters, uc_from_buffer ? 1 : 0);
    if (e != cudaSuccess) t_launch_error = e;
    return e == cudaSuccess ? 0 : 1;
}

bool cluster_supported() {
    static int v = -1;
    if (v < 0) {
        // a 16-CTA cluster of the kernel must fit on the device
        cudaFuncSetAttribute(k_recon_cluster<0>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(kClusterCtas);
        cfg.blockDim = dim3(kClusterThreads);
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = kClusterCtas;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int n = 0;
        const cudaError_t e = cudaOccupancyMaxActiveClusters(&n, k_recon_cluster<0>, &cfg);
        v = (e == cudaSuccess && n >= 1) ? 1 : 0;
        cudaGetLastError();
    }
    return v == 1;
}

int launch_plain_data(float* duhat, float* dvhat, const float* pu1, const float* pu2,
                      const float* pv1, const float* pv2, const float* Ix, const float* Iy,
                      const float* Iz, const Weights& wt, LevelDims d, bool first,
                      cudaStream_t st) {
    k_plain_data<<<grid_for(d.w, d.h), dim3(BX, BY), 0, st>>>(duhat, dvhat, pu1, pu2, pv1, pv2,
                                                             Ix, Iy, Iz, wt, d, first);
    return check_launch();
}

int launch_plain_tv(const float* duhat, const float* dvhat, float* pu1, float* pu2, float* pv1,
                    float* pv2, const Weights& wt, LevelDims d, bool first, cudaStream_t st) {
    k_plain_tv<<<grid_for(d.w, d.h), dim3(BX, BY), 0, st>>>(duhat, dvhat, pu1, pu2, pv1, pv2, wt,
                                                           d, first);
    return check_launch();
}

int launch_median_add(const float* duhat, const float* dvhat, const float* u, const float* v,
                      float* ou, float* ov, LevelDims d, cudaStream_t st) {
    k_median_add<<<grid_for(d.w, (d.h + 1) / 2), dim3(BX, BY), 0, st>>>(duhat, dvhat, u, v, ou,
                                                                       ov, d);
    return check_launch();
}

int launch_median5(const float* u, const float* v, float* ou, float* ov, LevelDims d,
                   cudaStream_t st) {
    k_median5<<<grid_for(d.w, (d.h + 1) / 2), dim3(BX, BY), 0, st>>>(u, v, ou, ov, d);
    return check_launch();
}

int launch_median3d(const float* X, const float* Y, const float* Z, float* X1, float* Y1,
                    float* Z1, LevelDims d, cudaStream_t st) {
    k_median3d<<<grid_for(d.w, d.h), dim3(BX, BY), 0, st>>>(X, Y, Z, X1, Y1, Z1, d);
    return check_launch();
}

int launch_solve_uc(const float* X, const float* Y, const float* Z, const LevelConsts* lc,
                    LevelDims d, float* uc, float* vc, cudaStream_t st) {
    k_solve_uc<<<grid_for(d.w, d.h), dim3(BX, BY), 0, st>>>(X, Y, Z, lc, d, uc, vc);
    return check_launch();
}

int launch_upscale_fields(int n, const float* const* src, float* const* dst, const float* scales,
                          LevelDims coarse, LevelDims fine, cudaStream_t st) {
    if (n < 1 || n > 12) return 1;
    UpscaleArgs a;
    a.n = n;
    for (int i = 0; i < n; i++) {
        a.src[i] = src[i];
        a.dst[i] = dst[i];
        a.scale[i] = scales[i];
    }
    k_upscale_fields<<<grid_for(fine.w, fine.h), dim3(BX, BY), 0, st>>>(a, coarse, fine);
    return check_launch();
}

int launch_upscale(const float* src, LevelDims coarse, LevelDims fine, float scale, float* out,
                   cudaStream_t st) {
    float* dst[1] = {out};
    const float* s[1] = {src};
    return launch_upscale_fields(1, s, dst, &scale, coarse, fine, st);
}

int launch_inv_depth(const float* Z, LevelDims d, float* out, cudaStream_t st) {
    k_inv_depth<<<grid_for(d.w, d.h), dim3(BX, BY), 0, st>>>(Z, d, out);
    return check_launch();
}

int launch_remove_edge(const float* X, const float* Y, const float* Z, int range, float max_area,
                       LevelDims d, float* X1, float* Y1, float* Z1, cudaStream_t st) {
    k_remove_edge<<<grid_for(d.w, d.h), dim3(BX, BY), 0, st>>>(X, Y, Z, range, max_area, d, X1,
                                                              Y1, Z1);
    return check_launch();
}

int launch_flow_color(const float* u, const float* v, LevelDims d, float flow_scale, float* rgb,
                      cudaStream_t st) {
    k_flow_color<<<grid_for(d.w, d.h), dim3(BX, BY), 0, st>>>(u, v, d, flow_scale, rgb);
    return check_launch();
}

}  // namespace rf

namespace rf {
EnergyArgs energy_args(const float* I0, const float* I1, const float* u, const float* v,
                       const float* X, const float* Y, const float* Z, float lambda,
                       float alpha_proj, const double* R1, const double* t1, const double* K1,
                       int recon) {
    EnergyArgs a;
    a.I0 = I0; a.I1 = I1; a.u = u; a.v = v; a.X = X; a.Y = Y; a.Z = Z;
    for (int i = 0; i < 9; i++) a.R1f[i] = (float)(R1 ? R1[i] : (i % 4 == 0 ? 1.0 : 0.0));
    for (int i = 0; i < 3; i++) a.t1f[i] = (float)(t1 ? t1[i] : 0.0);
    a.fxf = (float)(K1 ? K1[0] : 1.0);
    a.cxf = (float)(K1 ? K1[2] : 0.0);
    a.cyf = (float)(K1 ? K1[5] : 0.0);
    a.lambda = lambda;
    a.alpha_proj = alpha_proj;
    a.recon = recon;
    return a;
}

int launch_energy(const float* I0, const float* I1, const float* u, const float* v,
                  const float* X, const float* Y, const float* Z, LevelDims d, float lambda,
                  float alpha_proj, const double* R1, const double* t1, const double* K1,
                  int recon, double* partial, int nblocks, double* out, cudaStream_t st) {
    const EnergyArgs a = energy_args(I0, I1, u, v, X, Y, Z, lambda, alpha_proj, R1, t1, K1, recon);
    k_energy_partial<<<nblocks, kEnergyThreads, 0, st>>>(a, d, partial);
    k_energy_final<<<1, 32, 0, st>>>(partial, nblocks, out);
    return check_launch();
}

// at least 8 pixels per thread (fewer thread sums to add in double), at
// most kEnergyMaxBlocks blocks
int energy_blocks(LevelDims d) {
    const long long per_block = 8LL * kEnergyThreads;
    const long long nb = ((long long)d.w * d.h + per_block - 1) / per_block;
    return nb < kEnergyMaxBlocks ? (int)nb : kEnergyMaxBlocks;
}

int launch_energy_jobs(const EnergyJob* jobs, int n, int total_blocks, int max_blocks,
                       cudaStream_t st) {
    if (n <= 0 || total_blocks <= 0) return 0;
    if (n <= 65535 && max_blocks > 0)
        k_energy_partial_grid<<<dim3(max_blocks, n), kEnergyThreads, 0, st>>>(jobs);
    else
        k_energy_partial_jobs<<<total_blocks, kEnergyThreads, 0, st>>>(jobs, n);
    k_energy_final_jobs<<<n, 32, 0, st>>>(jobs);
    return check_launch();
}
}  // namespace rf

extern "C" void rf_test_fail_alloc(long long k) {
    g_fail_at.store(k < 0 ? 0 : k);
    g_alloc_count.store(0);
}
