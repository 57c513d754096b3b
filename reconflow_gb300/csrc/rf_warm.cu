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

rf_status rf_ws_state(int n, const float* net, int channels, int wn, int hn, int w, int h, int s,
                      float up, const double* K_level, const double* R, const double* t,
                      float* const* u, float* const* v, float* const* X, float* const* Y,
                      float* const* Z, void* stream) {
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
