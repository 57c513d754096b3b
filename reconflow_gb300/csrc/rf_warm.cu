// Learned warm start, the stencil parts around the network: the network's
// input features from a frame pair and its pose, and the solver's warm-start
// state (flow and 3D points at a pyramid level) from the network's inverse
// depth.  No counterpart in the reference, which always starts the solve
// from zero flow at its coarsest level (Reconflow.cu:209-220).
//
// Geometry (the solver's convention, solveUcSk.cu:21-33): a camera-0 pixel
// x~ = (x, y, 1) at inverse depth rho is the point X = K^-1 x~ / rho; camera
// 1 sees X1 = R X + t, so its image is pi(K (R K^-1 x~ + rho t)) =
// (a + rho b) / (a_z + rho b_z) with a = K R K^-1 x~ and b = K t.
//
// Features (16 channels, NHWC, one sample per pixel of the coarse grid):
//   0   I0 - 0.5 at the coarse grid (box average of factor x factor pixels)
//   1   I1 - 0.5
//   2.. 13   |I1(x'(rho_k)) - I0(x)| * 10 for rho_k = k * 0.05, k = 0..11
//            (a plane sweep over inverse depth 0 .. 0.55 1/m; I1 bilinear,
//            clamped to the edge)
//   14, 15   d x'/d rho at rho = 0.25, in coarse pixels per 10 1/m: the
//            epipolar direction and how far a unit of inverse depth moves
//            the match
// Every launch handles up to kWsChunk pairs (per-pair pointers and cameras
// travel as kernel parameters), so a batch needs no device-side tables.
#include <cmath>
#include <cstring>
#include <string>

#include <cuda_runtime.h>

#include "../../include/reconflow_gb300.h"
#include "rf_kernels.cuh"
#include "rf_nvtx.h"

namespace rf_warm_impl {

constexpr int kWsChunk = 32;
constexpr int kHyp = 12;
constexpr float kRhoStep = 0.05f;

struct WsCam {
    float fx, fy, cx, cy;
    float R[9];
    float t[3];
};

struct FeatArgs {
    const float* I0[kWsChunk];
    const float* I1[kWsChunk];
    WsCam cam[kWsChunk];
};

struct StateArgs {
    float* u[kWsChunk];
    float* v[kWsChunk];
    float* X[kWsChunk];
    float* Y[kWsChunk];
    float* Z[kWsChunk];
    WsCam cam[kWsChunk];
};

// pass 1: box average of factor x factor level-0 pixels into channels 0, 1
__global__ void k_ws_coarse(FeatArgs a, int s0, int factor, int wn, int hn, int first_pair,
                            float* __restrict__ out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int p = blockIdx.z;
    if (x >= wn || y >= hn) return;
    const float* I0 = a.I0[p];
    const float* I1 = a.I1[p];
    float s0v = 0.0f, s1v = 0.0f;
    for (int j = 0; j < factor; j++) {
        const int row = (y * factor + j) * s0 + x * factor;
        for (int i = 0; i < factor; i++) {
            s0v += I0[row + i];
            s1v += I1[row + i];
        }
    }
    const float inv = 1.0f / (float)(factor * factor);
    float* o = out + (((size_t)(first_pair + p) * hn + y) * wn + x) * 16;
    o[0] = s0v * inv - 0.5f;
    o[1] = s1v * inv - 0.5f;
}

__device__ __forceinline__ float sample_ch1(const float* __restrict__ img, int wn, int hn, float x,
                                            float y) {
    x = fminf(fmaxf(x, 0.0f), (float)(wn - 1));
    y = fminf(fmaxf(y, 0.0f), (float)(hn - 1));
    const int x0 = min((int)x, wn - 2 < 0 ? 0 : wn - 2);
    const int y0 = min((int)y, hn - 2 < 0 ? 0 : hn - 2);
    const int x1 = min(x0 + 1, wn - 1), y1 = min(y0 + 1, hn - 1);
    const float ax = x - (float)x0, ay = y - (float)y0;
    const float v00 = img[((size_t)y0 * wn + x0) * 16 + 1];
    const float v01 = img[((size_t)y0 * wn + x1) * 16 + 1];
    const float v10 = img[((size_t)y1 * wn + x0) * 16 + 1];
    const float v11 = img[((size_t)y1 * wn + x1) * 16 + 1];
    return (1.0f - ay) * ((1.0f - ax) * v00 + ax * v01) + ay * ((1.0f - ax) * v10 + ax * v11);
}

// pass 2: plane-sweep costs and the epipolar derivative
__global__ void k_ws_sweep(FeatArgs a, int wn, int hn, int first_pair, float* __restrict__ out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int p = blockIdx.z;
    if (x >= wn || y >= hn) return;
    const WsCam& c = a.cam[p];
    const float* img = out + (size_t)(first_pair + p) * hn * wn * 16;
    float* o = out + (((size_t)(first_pair + p) * hn + y) * wn + x) * 16;
    const float i0 = o[0];
    const float xn = ((float)x - c.cx) / c.fx, yn = ((float)y - c.cy) / c.fy;
    const float r0 = c.R[0] * xn + c.R[1] * yn + c.R[2];
    const float r1 = c.R[3] * xn + c.R[4] * yn + c.R[5];
    const float r2 = c.R[6] * xn + c.R[7] * yn + c.R[8];
    const float ax = c.fx * r0 + c.cx * r2, ay = c.fy * r1 + c.cy * r2, az = r2;
    const float bx = c.fx * c.t[0] + c.cx * c.t[2], by = c.fy * c.t[1] + c.cy * c.t[2], bz = c.t[2];
#pragma unroll
    for (int k = 0; k < kHyp; k++) {
        const float rho = kRhoStep * (float)k;
        const float den = az + rho * bz;
        float cost = 1.0f;  // behind the camera: maximal cost
        if (den > 1e-6f) {
            const float x2 = (ax + rho * bx) / den, y2 = (ay + rho * by) / den;
            cost = fabsf(sample_ch1(img, wn, hn, x2, y2) - i0) * 10.0f;
        }
        o[2 + k] = cost;
    }
    const float rm = 0.25f, den = az + rm * bz;
    float dx = 0.0f, dy = 0.0f;
    if (fabsf(den) > 1e-6f) {
        dx = (bx * den - (ax + rm * bx) * bz) / (den * den);
        dy = (by * den - (ay + rm * by) * bz) / (den * den);
    }
    o[14] = dx * 0.1f;
    o[15] = dy * 0.1f;
}

// warm-start state at a pyramid level from the network's inverse depth
// (channel 2 of an NHWC map of C channels): bilinear upsampling
// (half-pixel centres, clamped), inverse depth clamped to [0.02, 2] 1/m,
// X = Z K^-1 x~, and the flow of that point as the solver's SolveUc forms it
// (focal fx for both components, solveUcSk.cu:31-33).
__global__ void k_ws_state(StateArgs a, const float* __restrict__ net, int C, int wn, int hn,
                           int w, int h, int s, float up, int first_pair) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int p = blockIdx.z;
    if (x >= w || y >= h) return;
    const WsCam& c = a.cam[p];
    const float* m = net + (size_t)(first_pair + p) * hn * wn * C;
    float sx = fminf(fmaxf(((float)x + 0.5f) / up - 0.5f, 0.0f), (float)(wn - 1));
    float sy = fminf(fmaxf(((float)y + 0.5f) / up - 0.5f, 0.0f), (float)(hn - 1));
    const int x0 = min((int)sx, wn - 1), y0 = min((int)sy, hn - 1);
    const int x1 = min(x0 + 1, wn - 1), y1 = min(y0 + 1, hn - 1);
    const float fx = sx - (float)x0, fy = sy - (float)y0;
    const float r00 = m[((size_t)y0 * wn + x0) * C + 2], r01 = m[((size_t)y0 * wn + x1) * C + 2];
    const float r10 = m[((size_t)y1 * wn + x0) * C + 2], r11 = m[((size_t)y1 * wn + x1) * C + 2];
    float rho = (1.0f - fy) * ((1.0f - fx) * r00 + fx * r01) + fy * ((1.0f - fx) * r10 + fx * r11);
    rho = isfinite(rho) ? fminf(fmaxf(rho, 0.02f), 2.0f) : 0.2f;
    const float Z = 1.0f / rho;
    const float X = Z * ((float)x - c.cx) / c.fx;
    const float Y = Z * ((float)y - c.cy) / c.fy;
    const float X2 = c.R[0] * X + c.R[1] * Y + c.R[2] * Z + c.t[0];
    const float Y2 = c.R[3] * X + c.R[4] * Y + c.R[5] * Z + c.t[1];
    const float Z2 = c.R[6] * X + c.R[7] * Y + c.R[8] * Z + c.t[2];
    const int pos = x + y * s;
    a.u[p][pos] = c.fx * X2 / Z2 + c.cx - (float)x;
    a.v[p][pos] = c.fx * Y2 / Z2 + c.cy - (float)y;
    a.X[p][pos] = X;
    a.Y[p][pos] = Y;
    a.Z[p][pos] = Z;
}

// Temporal warm start for frame sequences: frame k's coarse inverse-depth
// grid from frame k-1's solved depth.  Every pixel of frame k-1 with a finite
// positive depth is lifted to 3D in camera k-1 (X = z K^-1 x~), moved by the
// relative pose (camera k-1 -> camera k, the previous pair's R, t) and
// projected into frame k; a point that lands at a depth of 0.5 .. 50 m adds
// its inverse depth to the cell of the factor-times-coarser grid it lands
// in, and a cell takes the mean of its points (the box mean the network's
// training targets use; a nearest-point z-buffer would let the few badly
// conditioned depths of a solve win whole cells).  The sums are fixed point
// (2^-16 1/m; a cell holds up to 2^15 points) in unsigned integers, so they
// do not depend on the order of
// the atomic adds and the grid is reproducible bit for bit.  Cells no point
// reaches take the median of the filled cells.  Every floating-point
// operation is an explicitly rounded intrinsic in a fixed order;
// oracle/temporal_oracle.py's float32 restatement gives the same bits.
constexpr float kPropScale = 65536.0f;  // 2^16 per 1/m

struct PropArgs {
    const float* Z[kWsChunk];
    WsCam cam[kWsChunk];  // level-0 intrinsics, relative pose
};

__global__ void k_ws_prop_clear(unsigned* __restrict__ acc, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) acc[i] = 0u;
}

// acc: per pair, `cells` sums then `cells` counts
__global__ void k_ws_prop_scatter(PropArgs a, int w, int h, int s, int factor, int wn, int hn,
                                  int first_pair, unsigned* __restrict__ acc) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int p = blockIdx.z;
    if (x >= w || y >= h) return;
    const float z = a.Z[p][x + y * s];
    if (!(isfinite(z) && z > 0.0f)) return;
    const WsCam& c = a.cam[p];
    const float X = __fdiv_rn(__fmul_rn(__fsub_rn((float)x, c.cx), z), c.fx);
    const float Y = __fdiv_rn(__fmul_rn(__fsub_rn((float)y, c.cy), z), c.fy);
    const float Q0 = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(c.R[0], X), __fmul_rn(c.R[1], Y)),
                                         __fmul_rn(c.R[2], z)), c.t[0]);
    const float Q1 = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(c.R[3], X), __fmul_rn(c.R[4], Y)),
                                         __fmul_rn(c.R[5], z)), c.t[1]);
    const float Q2 = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(c.R[6], X), __fmul_rn(c.R[7], Y)),
                                         __fmul_rn(c.R[8], z)), c.t[2]);
    if (!(Q2 >= 0.5f && Q2 <= 50.0f)) return;
    const float u = __fadd_rn(__fdiv_rn(__fmul_rn(c.fx, Q0), Q2), c.cx);
    const float v = __fadd_rn(__fdiv_rn(__fmul_rn(c.fy, Q1), Q2), c.cy);
    const float fu = floorf(__fdiv_rn(u, (float)factor));
    const float fv = floorf(__fdiv_rn(v, (float)factor));
    if (!(fu >= 0.0f && fu < (float)wn && fv >= 0.0f && fv < (float)hn)) return;
    const unsigned q = __float2uint_rn(__fmul_rn(__fdiv_rn(1.0f, Q2), kPropScale));
    const size_t cells = (size_t)wn * hn;
    const size_t cell = (size_t)fv * wn + (size_t)fu;
    unsigned* pa = acc + (size_t)(first_pair + p) * 2 * cells;
    atomicAdd(pa + cell, q);
    atomicAdd(pa + cells + cell, 1u);
}

// one block per pair: every filled cell's mean into channel `ch` of the
// grid; the median of those means (the mean of the two middle ones for an
// even count), found by a radix select on their bit patterns, into every
// empty cell; no filled cell: every cell 0
__global__ void __launch_bounds__(1024) k_ws_prop_fill(int cells, int C, int ch,
                                                       const unsigned* __restrict__ acc,
                                                       float* __restrict__ grid) {
    const unsigned* sum = acc + (size_t)blockIdx.x * 2 * cells;
    const unsigned* cnt = sum + cells;
    float* g = grid + (size_t)blockIdx.x * cells * C + ch;
    unsigned* gb = reinterpret_cast<unsigned*>(g);
    __shared__ unsigned hist[256];
    __shared__ unsigned s_prefix, s_rank, s_n;
    __shared__ float s_med[2];
    if (threadIdx.x == 0) s_n = 0u;
    __syncthreads();
    unsigned nf = 0;
    for (int i = threadIdx.x; i < cells; i += blockDim.x) {
        float m = 0.0f;
        if (cnt[i] != 0u) {
            m = (float)((double)sum[i] / (double)cnt[i] / (double)kPropScale);
            nf++;
        }
        g[(size_t)i * C] = m;
    }
    atomicAdd(&s_n, nf);
    __syncthreads();
    const unsigned n = s_n;
    if (n == 0u) return;
    for (int r = 0; r < 2; r++) {
        const unsigned want = r == 0 ? (n - 1u) / 2u : n / 2u;
        if (threadIdx.x == 0) {
            s_prefix = 0u;
            s_rank = want;
        }
        __syncthreads();
        for (int shift = 24; shift >= 0; shift -= 8) {
            for (int b = threadIdx.x; b < 256; b += blockDim.x) hist[b] = 0u;
            __syncthreads();
            const unsigned prefix = s_prefix;
            const unsigned hi_mask = shift == 24 ? 0u : (0xFFFFFFFFu << (shift + 8));
            for (int i = threadIdx.x; i < cells; i += blockDim.x) {
                const unsigned b = gb[(size_t)i * C];
                if (cnt[i] != 0u && (b & hi_mask) == prefix)
                    atomicAdd(&hist[(b >> shift) & 255u], 1u);
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                unsigned rank = s_rank, k = 0;
                while (hist[k] <= rank) {
                    rank -= hist[k];
                    k++;
                }
                s_rank = rank;
                s_prefix = prefix | (k << shift);
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) s_med[r] = __uint_as_float(s_prefix);
        __syncthreads();
    }
    const float med = (n & 1u) ? s_med[0] : __fmul_rn(__fadd_rn(s_med[0], s_med[1]), 0.5f);
    for (int i = threadIdx.x; i < cells; i += blockDim.x)
        if (cnt[i] == 0u) g[(size_t)i * C] = med;
}

WsCam make_cam(const double* K, const double* R, const double* t, double kscale) {
    WsCam c;
    c.fx = (float)(K[0] * kscale);
    c.fy = (float)(K[4] * kscale);
    c.cx = (float)(K[2] * kscale);
    c.cy = (float)(K[5] * kscale);
    for (int i = 0; i < 9; i++) c.R[i] = (float)R[i];
    for (int i = 0; i < 3; i++) c.t[i] = (float)t[i];
    return c;
}

rf_status wfail(rf_status st, const std::string& msg) {
    return static_cast<rf_status>(rf::set_last_error(st, msg.c_str()));
}

}  // namespace rf_warm_impl

using namespace rf_warm_impl;

extern "C" {

rf_status rf_ws_features(int n, const float* const* I0, const float* const* I1, int w0, int h0,
                         int s0, int factor, const double* K, const double* R, const double* t,
                         float* out, void* stream) {
    rf::NvtxRange range("rf_ws_features");
    if (n < 1 || !I0 || !I1 || !K || !R || !t || !out)
        return wfail(RF_ERR_INVALID_ARG, "rf_ws_features: null argument");
    if (factor < 1 || w0 < factor || h0 < factor || s0 < w0)
        return wfail(RF_ERR_INVALID_ARG, "rf_ws_features: bad size or factor");
    const int wn = w0 / factor, hn = h0 / factor;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    for (int p0 = 0; p0 < n; p0 += kWsChunk) {
        const int m = n - p0 < kWsChunk ? n - p0 : kWsChunk;
        FeatArgs a;
        std::memset(&a, 0, sizeof a);
        for (int i = 0; i < m; i++) {
            if (!I0[p0 + i] || !I1[p0 + i])
                return wfail(RF_ERR_INVALID_ARG, "rf_ws_features: null image pointer");
            a.I0[i] = I0[p0 + i];
            a.I1[i] = I1[p0 + i];
            a.cam[i] = make_cam(K + 9 * (p0 + i), R + 9 * (p0 + i), t + 3 * (p0 + i),
                                1.0 / (double)factor);
        }
        dim3 blk(32, 8), grd((wn + 31) / 32, (hn + 7) / 8, m);
        k_ws_coarse<<<grd, blk, 0, st>>>(a, s0, factor, wn, hn, p0, out);
        k_ws_sweep<<<grd, blk, 0, st>>>(a, wn, hn, p0, out);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return wfail(RF_ERR_CUDA, std::string("rf_ws_features: ") + cudaGetErrorString(e));
    }
    return RF_OK;
}

rf_status rf_ws_propagate(int n, const float* const* Z, int w, int h, int s, const double* K,
                          const double* R, const double* t, int factor, int wn, int hn,
                          int channels, int channel, float* grid, unsigned int* scratch,
                          void* stream) {
    rf::NvtxRange range("rf_ws_propagate");
    if (n < 1 || !Z || !K || !R || !t || !grid || !scratch)
        return wfail(RF_ERR_INVALID_ARG, "rf_ws_propagate: null argument");
    if (w < 1 || h < 1 || s < w || factor < 1 || factor > 32 || wn < 1 || hn < 1 ||
        channels < 1 || channel < 0 || channel >= channels)
        return wfail(RF_ERR_INVALID_ARG, "rf_ws_propagate: bad size or factor (1 .. 32)");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int cells = wn * hn;
    const int total = 2 * cells * n;
    k_ws_prop_clear<<<(total + 255) / 256, 256, 0, st>>>(scratch, total);
    for (int p0 = 0; p0 < n; p0 += kWsChunk) {
        const int m = n - p0 < kWsChunk ? n - p0 : kWsChunk;
        PropArgs a;
        std::memset(&a, 0, sizeof a);
        for (int i = 0; i < m; i++) {
            if (!Z[p0 + i]) return wfail(RF_ERR_INVALID_ARG, "rf_ws_propagate: null depth plane");
            a.Z[i] = Z[p0 + i];
            a.cam[i] = make_cam(K + 9 * (p0 + i), R + 9 * (p0 + i), t + 3 * (p0 + i), 1.0);
        }
        dim3 blk(32, 8), grd((w + 31) / 32, (h + 7) / 8, m);
        k_ws_prop_scatter<<<grd, blk, 0, st>>>(a, w, h, s, factor, wn, hn, p0, scratch);
    }
    k_ws_prop_fill<<<n, 1024, 0, st>>>(cells, channels, channel, scratch, grid);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return wfail(RF_ERR_CUDA, std::string("rf_ws_propagate: ") + cudaGetErrorString(e));
    return RF_OK;
}

rf_status rf_ws_state(int n, const float* net, int channels, int wn, int hn, int w, int h, int s,
                      float up, const double* K_level, const double* R, const double* t,
                      float* const* u, float* const* v, float* const* X, float* const* Y,
                      float* const* Z, void* stream) {
    rf::NvtxRange range("rf_ws_state");
    if (n < 1 || !net || !K_level || !R || !t || !u || !v || !X || !Y || !Z)
        return wfail(RF_ERR_INVALID_ARG, "rf_ws_state: null argument");
    if (channels < 3 || wn < 1 || hn < 1 || w < 1 || h < 1 || s < w || !(up > 0.0f))
        return wfail(RF_ERR_INVALID_ARG, "rf_ws_state: bad size");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    for (int p0 = 0; p0 < n; p0 += kWsChunk) {
        const int m = n - p0 < kWsChunk ? n - p0 : kWsChunk;
        StateArgs a;
        std::memset(&a, 0, sizeof a);
        for (int i = 0; i < m; i++) {
            const int q = p0 + i;
            if (!u[q] || !v[q] || !X[q] || !Y[q] || !Z[q])
                return wfail(RF_ERR_INVALID_ARG, "rf_ws_state: null plane pointer");
            a.u[i] = u[q]; a.v[i] = v[q]; a.X[i] = X[q]; a.Y[i] = Y[q]; a.Z[i] = Z[q];
            a.cam[i] = make_cam(K_level + 9 * q, R + 9 * q, t + 3 * q, 1.0);
        }
        dim3 blk(32, 8), grd((w + 31) / 32, (h + 7) / 8, m);
        k_ws_state<<<grd, blk, 0, st>>>(a, net, channels, wn, hn, w, h, s, up, p0);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return wfail(RF_ERR_CUDA, std::string("rf_ws_state: ") + cudaGetErrorString(e));
    }
    return RF_OK;
}

}  // extern "C"
