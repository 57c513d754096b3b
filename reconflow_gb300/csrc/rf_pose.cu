// Pose front end on the GPU: the CameraPose path (reconflow/CameraPose.cpp:
// 47-118) rebuilt without OpenCV.  The reference runs OpenCV's closed
// SURF_CUDA, a brute-force k = 2 matcher with a 0.6 ratio test, then
// findEssentialMat (LMEDS) and recoverPose.  Here SURF follows its
// publication (H. Bay, A. Ess, T. Tuytelaars, L. Van Gool, "Speeded-up robust
// features (SURF)", CVIU 110(3), 2008) with these definitions, which the CPU
// oracle restates and the tests compare bit for bit:
//
// * integral image S of the 8-bit frame, (w + 1) x (h + 1) uint32, exact;
// * octave o, layer k: box-filter size L = 3 (2^(o+1) (k + 1) + 1) (9, 15,
//   21, 27; 15, 27, 39, 51; ...), responses on the grid of step 2^o, lobe
//   l = L / 3: Dxx = three l-wide boxes of height 2l - 1 (+1, -2, +1), Dyy
//   its transpose, Dxy = four l x l boxes around a one-pixel cross (+, -, -,
//   +); det = dxx dyy - 0.81 dxy^2 with each term divided by L^2; a response
//   is defined where the whole filter lies inside the frame;
// * keypoints: responses above the threshold and strictly above their 26
//   neighbours in (x, y, layer), layers 1..n_layers, refined by one Newton
//   step on the quadratic fit (rejected unless every offset is within 0.5);
//   scale s = 1.2 L / 9 at the interpolated L; the strongest max_keypoints
//   are kept (ties by octave, layer, cell);
// * orientation: Haar responses of size 4s (clamped boxes) at the 109 grid
//   points within radius 6s, weighted by a Gaussian of sigma 2.5s; 72
//   windows of pi/3 starting every 5 degrees; the angle of the largest
//   window sum;
// * descriptor: a 20s x 20s window turned to the orientation, 20 x 20 samples
//   one s apart, Haar responses of size 2s rotated into the window frame,
//   Gaussian weight sigma 3.3s, sums (dx, dy, |dx|, |dy|) over 4 x 4
//   sub-regions, unit length;
// * angles, sines and cosines from this file's own polynomial forms (below),
//   so host and device agree exactly;
// * matching: squared Euclidean distances summed in descriptor order, the two
//   nearest under (distance, index), ratio sqrt(d1) < 0.6 sqrt(d2).
//
// Built with -fmad=false: every value is a deterministic function of the
// frames.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/reconflow_gb300.h"
#include "rf_alloc.h"
#include "rf_nvtx.h"
#include "rf_epipolar.h"
#include "rf_kernels.cuh"

namespace rf_pose_impl {

constexpr int kMaxOctaves = 8;
constexpr int kMaxLayers = 8;  // response layers per octave (n_octave_layers + 2)
constexpr int kDesc = 64;
constexpr int kOriSamples = 109;
constexpr int kOriWindows = 72;
constexpr int kDescSamples = 400;

constexpr float kPi = 3.14159265358979323846f;
constexpr float kTwoPi = 6.28318530717958647692f;
constexpr float kHalfPi = 1.57079632679489661923f;
constexpr float kTwoOverPi = 0.63661977236758134308f;
constexpr float kOriStep = 0.08726646259971647884f;  // 5 degrees
constexpr float kOriWin = 1.04719755119659774615f;   // 60 degrees

__host__ __device__ inline int filter_size(int o, int k) { return 3 * ((2 << o) * (k + 1) + 1); }

// atan on [0, 1]: above tan(pi/12) shift by pi/6 with
// atan z = pi/6 + atan((sqrt3 z - 1) / (z + sqrt3)), then the odd Taylor
// series to z^11 on |z| <= tan(pi/12) (truncation below 3e-9).
__device__ __forceinline__ float atan_unit(float z) {
    float off = 0.0f;
    if (z > 0.267949192f) {
        z = (z * 1.73205081f - 1.0f) / (z + 1.73205081f);
        off = 0.523598776f;
    }
    const float z2 = z * z;
    float p = -0.0909090909f;
    p = p * z2 + 0.111111111f;
    p = p * z2 - 0.142857143f;
    p = p * z2 + 0.2f;
    p = p * z2 - 0.333333333f;
    p = p * z2 + 1.0f;
    return off + z * p;
}

// angle of (x, y) in [0, 2 pi); 0 for the zero vector
__device__ __forceinline__ float atan2_pos(float y, float x) {
    if (x == 0.0f && y == 0.0f) return 0.0f;
    const float ax = fabsf(x), ay = fabsf(y);
    float a = ay <= ax ? atan_unit(ay / ax) : kHalfPi - atan_unit(ax / ay);
    if (x < 0.0f) a = kPi - a;
    if (y < 0.0f) a = kTwoPi - a;
    if (a >= kTwoPi) a = 0.0f;
    return a;
}

// sine and cosine: reduction to the nearest multiple of pi/2, Taylor series
// to r^9 / r^8 on |r| <= pi/4 (truncation below 2e-9)
__device__ __forceinline__ void sincos_own(float a, float& s, float& c) {
    const float q = floorf(a * kTwoOverPi + 0.5f);
    const float r = a - q * kHalfPi;
    const int k = ((int)q) & 3;
    const float r2 = r * r;
    float ps = 2.75573192e-6f;
    ps = ps * r2 - 1.98412698e-4f;
    ps = ps * r2 + 8.33333333e-3f;
    ps = ps * r2 - 0.166666667f;
    ps = ps * r2 + 1.0f;
    const float sr = r * ps;
    float pc = 2.48015873e-5f;
    pc = pc * r2 - 1.38888889e-3f;
    pc = pc * r2 + 4.16666667e-2f;
    pc = pc * r2 - 0.5f;
    const float cr = pc * r2 + 1.0f;
    switch (k) {
        case 0: s = sr; c = cr; break;
        case 1: s = cr; c = -sr; break;
        case 2: s = -sr; c = -cr; break;
        default: s = -cr; c = sr; break;
    }
}

// sum of the frame over [x0, x1) x [y0, y1), inside the frame
__device__ __forceinline__ int box_sum(const uint32_t* __restrict__ S, int W1, int x0, int y0,
                                       int x1, int y1) {
    return (int)(S[y1 * W1 + x1] - S[y0 * W1 + x1] - S[y1 * W1 + x0] + S[y0 * W1 + x0]);
}

// the same box clipped to the frame (0 when nothing is left)
__device__ __forceinline__ int box_clip(const uint32_t* __restrict__ S, int w, int h, int x0,
                                        int y0, int x1, int y1) {
    x0 = min(max(x0, 0), w);
    x1 = min(max(x1, 0), w);
    y0 = min(max(y0, 0), h);
    y1 = min(max(y1, 0), h);
    if (x1 <= x0 || y1 <= y0) return 0;
    return box_sum(S, w + 1, x0, y0, x1, y1);
}

// Haar wavelet responses of size 2 half at (px, py)
__device__ __forceinline__ void haar(const uint32_t* __restrict__ S, int w, int h, int px, int py,
                                     int half, float& dx, float& dy) {
    dx = (float)(box_clip(S, w, h, px, py - half, px + half, py + half) -
                 box_clip(S, w, h, px - half, py - half, px, py + half));
    dy = (float)(box_clip(S, w, h, px - half, py, px + half, py + half) -
                 box_clip(S, w, h, px - half, py - half, px + half, py));
}

struct DevKp {
    float x, y, scale, response, angle;
    int octave, layer, cell;
};

struct Tables {
    float ori_w[kOriSamples];
    int ori_i[kOriSamples], ori_j[kOriSamples];
    float desc_w[kDescSamples];
};

// ---- kernels ---------------------------------------------------------------

__global__ void k_to_u8(const float* __restrict__ in, int w, int h, int pitch, uint8_t* out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    const float v = in[(size_t)y * pitch + x] * 255.0f + 0.5f;
    int u = v >= 0.0f ? (int)floorf(v < 255.0f ? v : 255.0f) : 0;
    out[(size_t)y * w + x] = (uint8_t)u;
}

// row pass: S[y + 1][x + 1] = sum of row y up to x (one warp per row)
__global__ void k_integral_rows(const uint8_t* __restrict__ img, int w, int h, uint32_t* S) {
    const int row = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (row >= h) return;
    const int W1 = w + 1;
    uint32_t carry = 0;
    if (lane == 0) S[(size_t)(row + 1) * W1] = 0;
    for (int x0 = 0; x0 < w; x0 += 32) {
        const int x = x0 + lane;
        uint32_t v = x < w ? img[(size_t)row * w + x] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += t;
        }
        if (x < w) S[(size_t)(row + 1) * W1 + x + 1] = carry + v;
        carry += __shfl_sync(0xffffffffu, v, 31);
    }
}

// column pass in three steps over row segments of kSeg rows: running sums
// inside each segment (and the segment's total), the totals' running sums,
// then each segment's offset added (uint32 sums, exact modulo 2^32)
constexpr int kSeg = 32;

__global__ void k_integral_cols_seg(int w, int h, uint32_t* S, uint32_t* tot) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, g = blockIdx.y, W1 = w + 1;
    if (x >= W1) return;
    if (g == 0) S[x] = 0;
    const int y0 = 1 + g * kSeg, y1 = min(h, y0 + kSeg - 1);
    uint32_t acc = 0;
    for (int y = y0; y <= y1; y++) {
        acc += S[(size_t)y * W1 + x];
        S[(size_t)y * W1 + x] = acc;
    }
    tot[(size_t)g * W1 + x] = acc;
}

__global__ void k_integral_cols_add(int w, int h, uint32_t* S, const uint32_t* tot) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, g = blockIdx.y, W1 = w + 1;
    if (x >= W1 || g == 0) return;
    uint32_t off = 0;
    for (int q = 0; q < g; q++) off += tot[(size_t)q * W1 + x];
    const int y0 = 1 + g * kSeg, y1 = min(h, y0 + kSeg - 1);
    for (int y = y0; y <= y1; y++) S[(size_t)y * W1 + x] += off;
}

__global__ void k_hessian(const uint32_t* __restrict__ S, int w, int h, int octave, float* resp) {
    const int cols = w >> octave, rows = h >> octave;
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= cols || j >= rows) return;
    const int x = i << octave, y = j << octave;
    const int L = filter_size(octave, k), l = L / 3, r = (L - 1) / 2, c = (l - 1) / 2;
    float det = 0.0f;
    if (x >= r && x < w - r && y >= r && y < h - r) {
        const int W1 = w + 1;
        const int dxx = box_sum(S, W1, x - c - l, y - l + 1, x - c, y + l) +
                        box_sum(S, W1, x + c + 1, y - l + 1, x + c + 1 + l, y + l) -
                        2 * box_sum(S, W1, x - c, y - l + 1, x + c + 1, y + l);
        const int dyy = box_sum(S, W1, x - l + 1, y - c - l, x + l, y - c) +
                        box_sum(S, W1, x - l + 1, y + c + 1, x + l, y + c + 1 + l) -
                        2 * box_sum(S, W1, x - l + 1, y - c, x + l, y + c + 1);
        const int dxy = box_sum(S, W1, x - l, y - l, x, y) +
                        box_sum(S, W1, x + 1, y + 1, x + 1 + l, y + 1 + l) -
                        box_sum(S, W1, x + 1, y - l, x + 1 + l, y) -
                        box_sum(S, W1, x - l, y + 1, x, y + 1 + l);
        const float inv = 1.0f / (float)(L * L);
        const float fxx = (float)dxx * inv, fyy = (float)dyy * inv, fxy = (float)dxy * inv;
        det = fxx * fyy - 0.81f * fxy * fxy;
    }
    resp[((size_t)k * rows + j) * cols + i] = det;
}

__global__ void k_extrema(const float* __restrict__ resp, int w, int h, int octave, float thr,
                          DevKp* out, int* count, int cap) {
    const int cols = w >> octave, rows = h >> octave;
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z + 1;
    if (i >= cols || j >= rows) return;
    const int step = 1 << octave, x = i << octave, y = j << octave;
    const int rb = (filter_size(octave, k + 1) - 1) / 2;
    if (x - step < rb || x + step >= w - rb || y - step < rb || y + step >= h - rb) return;
    auto R = [&](int kk, int jj, int ii) { return resp[((size_t)kk * rows + jj) * cols + ii]; };
    const float v = R(k, j, i);
    if (!(v > thr)) return;
    for (int dk = -1; dk <= 1; dk++)
        for (int dj = -1; dj <= 1; dj++)
            for (int di = -1; di <= 1; di++) {
                if (dk == 0 && dj == 0 && di == 0) continue;
                if (!(v > R(k + dk, j + dj, i + di))) return;
            }
    const float dx = (R(k, j, i + 1) - R(k, j, i - 1)) * 0.5f;
    const float dy = (R(k, j + 1, i) - R(k, j - 1, i)) * 0.5f;
    const float ds = (R(k + 1, j, i) - R(k - 1, j, i)) * 0.5f;
    const float a11 = (R(k, j, i + 1) + R(k, j, i - 1)) - 2.0f * v;
    const float a22 = (R(k, j + 1, i) + R(k, j - 1, i)) - 2.0f * v;
    const float a33 = (R(k + 1, j, i) + R(k - 1, j, i)) - 2.0f * v;
    const float a12 = (((R(k, j + 1, i + 1) - R(k, j + 1, i - 1)) - R(k, j - 1, i + 1)) +
                       R(k, j - 1, i - 1)) * 0.25f;
    const float a13 = (((R(k + 1, j, i + 1) - R(k + 1, j, i - 1)) - R(k - 1, j, i + 1)) +
                       R(k - 1, j, i - 1)) * 0.25f;
    const float a23 = (((R(k + 1, j + 1, i) - R(k + 1, j - 1, i)) - R(k - 1, j + 1, i)) +
                       R(k - 1, j - 1, i)) * 0.25f;
    const float b1 = -dx, b2 = -dy, b3 = -ds;
    const float det = a11 * (a22 * a33 - a23 * a23) - a12 * (a12 * a33 - a23 * a13) +
                      a13 * (a12 * a23 - a22 * a13);
    if (!(det != 0.0f)) return;
    const float nx = b1 * (a22 * a33 - a23 * a23) - a12 * (b2 * a33 - a23 * b3) +
                     a13 * (b2 * a23 - a22 * b3);
    const float ny = a11 * (b2 * a33 - a23 * b3) - b1 * (a12 * a33 - a23 * a13) +
                     a13 * (a12 * b3 - b2 * a13);
    const float ns = a11 * (a22 * b3 - b2 * a23) - a12 * (a12 * b3 - b2 * a13) +
                     b1 * (a12 * a23 - a22 * a13);
    const float ox = nx / det, oy = ny / det, os = ns / det;
    if (!(fabsf(ox) <= 0.5f && fabsf(oy) <= 0.5f && fabsf(os) <= 0.5f)) return;
    const int L0 = filter_size(octave, k), dL = filter_size(octave, k + 1) - L0;
    const float Lf = (float)L0 + os * (float)dL;
    DevKp p;
    p.x = ((float)i + ox) * (float)step;
    p.y = ((float)j + oy) * (float)step;
    p.scale = 1.2f * Lf / 9.0f;
    p.response = v;
    p.angle = 0.0f;
    p.octave = octave;
    p.layer = k;
    p.cell = j * cols + i;
    const int at = atomicAdd(count, 1);
    if (at < cap) out[at] = p;
}

// one warp per keypoint
__global__ void __launch_bounds__(128) k_orientation(const uint32_t* __restrict__ S, int w, int h,
                                                     DevKp* kp, int n, const Tables* __restrict__ T) {
    __shared__ float sdx[4][kOriSamples], sdy[4][kOriSamples], sang[4][kOriSamples];
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int idx = blockIdx.x * 4 + wl;
    if (idx >= n) return;
    const DevKp p = kp[idx];
    const float s = p.scale;
    const int half = max(1, (int)floorf(2.0f * s + 0.5f));  // Haar size 4s
    for (int q = lane; q < kOriSamples; q += 32) {
        const int px = (int)floorf(p.x + (float)T->ori_i[q] * s + 0.5f);
        const int py = (int)floorf(p.y + (float)T->ori_j[q] * s + 0.5f);
        float dx, dy;
        haar(S, w, h, px, py, half, dx, dy);
        const float g = T->ori_w[q];
        const float fx = g * dx, fy = g * dy;
        sdx[wl][q] = fx;
        sdy[wl][q] = fy;
        sang[wl][q] = atan2_pos(fy, fx);
    }
    __syncwarp();
    float best = -1.0f, bx = 0.0f, by = 0.0f;
    int bwin = INT_MAX;
    for (int win = lane; win < kOriWindows; win += 32) {
        const float a0 = (float)win * kOriStep;
        float sx = 0.0f, sy = 0.0f;
        for (int q = 0; q < kOriSamples; q++) {
            float d = sang[wl][q] - a0;
            if (d < 0.0f) d = d + kTwoPi;
            if (d < kOriWin) {
                sx = sx + sdx[wl][q];
                sy = sy + sdy[wl][q];
            }
        }
        const float mag = sx * sx + sy * sy;
        if (mag > best) {
            best = mag;
            bwin = win;
            bx = sx;
            by = sy;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const float om = __shfl_down_sync(0xffffffffu, best, o);
        const int ow = __shfl_down_sync(0xffffffffu, bwin, o);
        const float ox = __shfl_down_sync(0xffffffffu, bx, o);
        const float oy = __shfl_down_sync(0xffffffffu, by, o);
        if (om > best || (om == best && ow < bwin)) {
            best = om;
            bwin = ow;
            bx = ox;
            by = oy;
        }
    }
    if (lane == 0) kp[idx].angle = best > 0.0f ? atan2_pos(by, bx) : 0.0f;
}

// one warp per keypoint; lanes 0..15 own the 4 x 4 sub-regions
__global__ void __launch_bounds__(128) k_descriptor(const uint32_t* __restrict__ S, int w, int h,
                                                    const DevKp* __restrict__ kp, int n,
                                                    const Tables* __restrict__ T, float* desc) {
    __shared__ float vals[4][kDesc];
    __shared__ float nrm[4];
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int idx = blockIdx.x * 4 + wl;
    if (idx >= n) return;
    const DevKp p = kp[idx];
    const float s = p.scale;
    float sn, c;
    sincos_own(p.angle, sn, c);
    const int half = max(1, (int)floorf(s + 0.5f));  // Haar size 2s
    if (lane < 16) {
        const int sv = lane >> 2, su = lane & 3;
        float sdx = 0.0f, sdy = 0.0f, sax = 0.0f, say = 0.0f;
        for (int v = 0; v < 5; v++)
            for (int u = 0; u < 5; u++) {
                const int U = su * 5 + u, V = sv * 5 + v;
                const float ou = (float)U - 9.5f, ov = (float)V - 9.5f;
                const float rxp = c * ou - sn * ov, ryp = sn * ou + c * ov;
                const int px = (int)floorf(p.x + s * rxp + 0.5f);
                const int py = (int)floorf(p.y + s * ryp + 0.5f);
                float dx, dy;
                haar(S, w, h, px, py, half, dx, dy);
                const float g = T->desc_w[V * 20 + U];
                const float rx = g * (c * dx + sn * dy), ry = g * (c * dy - sn * dx);
                sdx = sdx + rx;
                sdy = sdy + ry;
                sax = sax + fabsf(rx);
                say = say + fabsf(ry);
            }
        vals[wl][lane * 4 + 0] = sdx;
        vals[wl][lane * 4 + 1] = sdy;
        vals[wl][lane * 4 + 2] = sax;
        vals[wl][lane * 4 + 3] = say;
    }
    __syncwarp();
    if (lane == 0) {
        float n2 = 0.0f;
        for (int q = 0; q < kDesc; q++) n2 = n2 + vals[wl][q] * vals[wl][q];
        nrm[wl] = sqrtf(n2);
    }
    __syncwarp();
    const float nv = nrm[wl];
    for (int q = lane; q < kDesc; q += 32)
        desc[(size_t)idx * kDesc + q] = nv > 0.0f ? vals[wl][q] / nv : 0.0f;
}

// D (n x 64) -> DT (64 x ld)
__global__ void k_transpose_desc(const float* __restrict__ D, int n, int ld, float* DT) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int q = 0; q < kDesc; q++) DT[(size_t)q * ld + i] = D[(size_t)i * kDesc + q];
}

struct Best2 {
    float d1, d2;
    int i1, i2;
};

__device__ __forceinline__ bool before(float da, int ia, float db, int ib) {
    return da < db || (da == db && ia < ib);
}

__device__ __forceinline__ void insert(Best2& b, float d, int i) {
    if (before(d, i, b.d1, b.i1)) {
        b.d2 = b.d1;
        b.i2 = b.i1;
        b.d1 = d;
        b.i1 = i;
    } else if (before(d, i, b.d2, b.i2)) {
        b.d2 = d;
        b.i2 = i;
    }
}

// one 128-thread block per query of frame 0: the two nearest of frame 1
__global__ void __launch_bounds__(128) k_match(const float* __restrict__ D0, int n0,
                                               const float* __restrict__ D1T, int n1, int ld,
                                               int* best, float* d1, float* d2) {
    __shared__ float q[kDesc];
    __shared__ Best2 part[4];
    const int qi = blockIdx.x;
    if (threadIdx.x < kDesc) q[threadIdx.x] = D0[(size_t)qi * kDesc + threadIdx.x];
    __syncthreads();
    Best2 b{INFINITY, INFINITY, INT_MAX, INT_MAX};
    for (int t = threadIdx.x; t < n1; t += blockDim.x) {
        float d = 0.0f;
        for (int k = 0; k < kDesc; k++) {
            const float e = q[k] - D1T[(size_t)k * ld + t];
            d = d + e * e;
        }
        insert(b, d, t);
    }
    for (int o = 16; o > 0; o >>= 1) {
        Best2 ob;
        ob.d1 = __shfl_down_sync(0xffffffffu, b.d1, o);
        ob.d2 = __shfl_down_sync(0xffffffffu, b.d2, o);
        ob.i1 = __shfl_down_sync(0xffffffffu, b.i1, o);
        ob.i2 = __shfl_down_sync(0xffffffffu, b.i2, o);
        insert(b, ob.d1, ob.i1);
        insert(b, ob.d2, ob.i2);
    }
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = b;
    __syncthreads();
    if (threadIdx.x == 0) {
        Best2 r = part[0];
        for (int k = 1; k < 4; k++) {
            insert(r, part[k].d1, part[k].i1);
            insert(r, part[k].d2, part[k].i2);
        }
        best[qi] = r.i1;
        d1[qi] = r.d1;
        d2[qi] = r.d2;
    }
}

// LMedS scoring: one block per hypothesis; the squared Sampson distances of
// all n matches (npow2 >= n slots, the rest +inf) are sorted in shared memory
// (bitonic network) and the (n / 2)-th is the hypothesis' median -- the same
// order statistic the host's nth_element gives.  The distances are >= 0 or
// +inf, so their bit patterns sort as unsigned integers: the network runs on
// the integer pipes, not the FP64 units.
constexpr int kMaxGpuMatches = 16384;

__global__ void __launch_bounds__(256) k_lmeds_median(const double* __restrict__ hyp,
                                                      const double* __restrict__ x0,
                                                      const double* __restrict__ x1, int n,
                                                      int npow2, double* med) {
    extern __shared__ unsigned long long e[];
    __shared__ double E[9];
    if (threadIdx.x < 9) E[threadIdx.x] = hyp[(size_t)blockIdx.x * 9 + threadIdx.x];
    __syncthreads();
    for (int i = threadIdx.x; i < npow2; i += blockDim.x)
        e[i] = (unsigned long long)__double_as_longlong(
            i < n ? rf_epi::sampson2(E, x0 + 2 * i, x1 + 2 * i) : INFINITY);
    __syncthreads();
    for (int k = 2; k <= npow2; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < npow2; i += blockDim.x) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const bool up = (i & k) == 0;
                    const unsigned long long a = e[i], b = e[ixj];
                    if ((a > b) == up) {
                        e[i] = b;
                        e[ixj] = a;
                    }
                }
            }
            __syncthreads();
        }
    if (threadIdx.x == 0) med[blockIdx.x] = __longlong_as_double((long long)e[n / 2]);
}

}  // namespace rf_pose_impl

using namespace rf_pose_impl;

struct rf_pose {
    rf_pose_params p{};
    int w = 0, h = 0, max_kp = 0, cand_cap = 0;
    cudaStream_t own = nullptr, stream = nullptr;
    uint8_t* d_img[2] = {nullptr, nullptr};
    float* d_f32 = nullptr;            // float frame staging
    uint32_t* d_int[2] = {nullptr, nullptr};
    float* d_resp[2][kMaxOctaves] = {};
    DevKp* d_cand[2] = {nullptr, nullptr};
    int* d_count = nullptr;            // [2]
    DevKp* d_kp[2] = {nullptr, nullptr};
    float* d_desc[2] = {nullptr, nullptr};
    float* d_descT = nullptr;
    int* d_best = nullptr;
    float* d_d1 = nullptr;
    float* d_d2 = nullptr;
    Tables* d_tab = nullptr;
    uint32_t* d_seg = nullptr;         // column-pass segment totals
    double* d_x = nullptr;             // LMedS scoring: matches (2 x 2n doubles)
    double* d_hyp = nullptr;           // hypotheses (9 doubles each)
    double* d_med = nullptr;           // their medians
    size_t x_cap = 0, hyp_cap = 0;
    uint64_t launches = 0;
    int lmeds_h = 0, lmeds_n = 0;  // hypotheses and matches of the last GPU scoring
    // last solve
    std::vector<DevKp> kp[2];
    std::vector<int> m0, m1;
    std::vector<float> mdist;
    std::vector<uint8_t> minl;
    int n_inliers = 0;
    bool solved = false;
};

namespace rf_pose_impl {

rf_status pfail(rf_status st, const std::string& msg) {
    return static_cast<rf_status>(rf::set_last_error(st, msg.c_str()));
}

#define PC(call)                                                                       \
    do {                                                                               \
        cudaError_t e__ = (call);                                                      \
        if (e__ != cudaSuccess)                                                        \
            return pfail(e__ == cudaErrorMemoryAllocation ? RF_ERR_OOM : RF_ERR_CUDA,         \
                        std::string(#call ": ") + cudaGetErrorString(e__));            \
    } while (0)
#define PL()                                                                           \
    do {                                                                               \
        cudaError_t e__ = cudaGetLastError();                                          \
        if (e__ != cudaSuccess)                                                        \
            return pfail(RF_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e__)); \
        h->launches++;                                                                 \
    } while (0)

// Gaussian weight tables and the orientation sample grid (host double, then
// float)
Tables make_tables() {
    Tables t{};
    int n = 0;
    for (int j = -6; j <= 6; j++)
        for (int i = -6; i <= 6; i++)
            if (i * i + j * j < 36) {
                t.ori_i[n] = i;
                t.ori_j[n] = j;
                t.ori_w[n] = (float)std::exp(-(double)(i * i + j * j) / (2.0 * 2.5 * 2.5));
                n++;
            }
    for (int V = 0; V < 20; V++)
        for (int U = 0; U < 20; U++) {
            const double ou = U - 9.5, ov = V - 9.5;
            t.desc_w[V * 20 + U] = (float)std::exp(-(ou * ou + ov * ov) / (2.0 * 3.3 * 3.3));
        }
    return t;
}

bool kp_order(const DevKp& a, const DevKp& b) {
    if (a.response != b.response) return a.response > b.response;
    if (a.octave != b.octave) return a.octave < b.octave;
    if (a.layer != b.layer) return a.layer < b.layer;
    return a.cell < b.cell;
}

rf_status launch_integral(rf_pose* h, int f) {
    const int w = h->w, hh = h->h;
    dim3 blk(128);
    k_integral_rows<<<(hh + 3) / 4, blk, 0, h->stream>>>(h->d_img[f], w, hh, h->d_int[f]);
    PL();
    const dim3 grd((w + 1 + 127) / 128, (hh + kSeg - 1) / kSeg);
    k_integral_cols_seg<<<grd, blk, 0, h->stream>>>(w, hh, h->d_int[f], h->d_seg);
    PL();
    k_integral_cols_add<<<grd, blk, 0, h->stream>>>(w, hh, h->d_int[f], h->d_seg);
    PL();
    return RF_OK;
}

// responses (stage 1) and keypoint candidates (stage 2) of every octave
rf_status launch_octaves(rf_pose* h, int f, bool responses, bool extrema) {
    const int w = h->w, hh = h->h;
    const int layers = h->p.n_octave_layers + 2;
    for (int o = 0; o < h->p.n_octaves; o++) {
        const int cols = w >> o, rows = hh >> o;
        if (cols < 1 || rows < 1) break;
        dim3 blk(32, 8), grd((cols + 31) / 32, (rows + 7) / 8, layers);
        if (responses) {
            k_hessian<<<grd, blk, 0, h->stream>>>(h->d_int[f], w, hh, o, h->d_resp[f][o]);
            PL();
        }
        if (extrema) {
            dim3 grd2((cols + 31) / 32, (rows + 7) / 8, h->p.n_octave_layers);
            k_extrema<<<grd2, blk, 0, h->stream>>>(h->d_resp[f][o], w, hh, o,
                                                   (float)h->p.hessian_threshold, h->d_cand[f],
                                                   h->d_count + f, h->cand_cap);
            PL();
        }
    }
    return RF_OK;
}

rf_status launch_describe(rf_pose* h, int f, bool orient, bool describe) {
    const int n = (int)h->kp[f].size();
    if (orient) {
        k_orientation<<<(n + 3) / 4, 128, 0, h->stream>>>(h->d_int[f], h->w, h->h, h->d_kp[f], n,
                                                          h->d_tab);
        PL();
    }
    if (describe) {
        k_descriptor<<<(n + 3) / 4, 128, 0, h->stream>>>(h->d_int[f], h->w, h->h, h->d_kp[f], n,
                                                         h->d_tab, h->d_desc[f]);
        PL();
    }
    return RF_OK;
}

rf_status launch_match(rf_pose* h) {
    const int n0 = (int)h->kp[0].size(), n1 = (int)h->kp[1].size();
    k_transpose_desc<<<(n1 + 127) / 128, 128, 0, h->stream>>>(h->d_desc[1], n1, h->max_kp,
                                                              h->d_descT);
    PL();
    k_match<<<n0, 128, 0, h->stream>>>(h->d_desc[0], n0, h->d_descT, n1, h->max_kp, h->d_best,
                                       h->d_d1, h->d_d2);
    PL();
    return RF_OK;
}

rf_status detect(rf_pose* h, int f) {
    rf_status rs = launch_integral(h, f);
    if (rs != RF_OK) return rs;
    return launch_octaves(h, f, true, true);
}

rf_status solve(rf_pose* h, const double* K, double* R, double* t) {
    h->solved = false;
    PC(cudaMemsetAsync(h->d_count, 0, 2 * sizeof(int), h->stream));
    for (int f = 0; f < 2; f++) {
        rf_status rs = detect(h, f);
        if (rs != RF_OK) return rs;
    }
    int cnt[2];
    PC(cudaMemcpyAsync(cnt, h->d_count, 2 * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    PC(cudaStreamSynchronize(h->stream));
    for (int f = 0; f < 2; f++) {
        if (cnt[f] > h->cand_cap)
            return pfail(RF_ERR_STATE, "rf_pose_solve: more keypoint candidates than the buffer "
                                       "holds; raise hessian_threshold");
        std::vector<DevKp>& v = h->kp[f];
        v.resize(cnt[f]);
        if (cnt[f] > 0)
            PC(cudaMemcpy(v.data(), h->d_cand[f], sizeof(DevKp) * cnt[f], cudaMemcpyDeviceToHost));
        std::sort(v.begin(), v.end(), kp_order);
        if ((int)v.size() > h->max_kp) v.resize(h->max_kp);
        if (v.empty()) return pfail(RF_ERR_STATE, "rf_pose_solve: no keypoints found");
        PC(cudaMemcpyAsync(h->d_kp[f], v.data(), sizeof(DevKp) * v.size(), cudaMemcpyHostToDevice,
                           h->stream));
        rf_status rs = launch_describe(h, f, true, true);
        if (rs != RF_OK) return rs;
    }
    const int n0 = (int)h->kp[0].size(), n1 = (int)h->kp[1].size();
    {
        rf_status rs = launch_match(h);
        if (rs != RF_OK) return rs;
    }
    std::vector<int> best(n0);
    std::vector<float> d1(n0), d2(n0);
    for (int f = 0; f < 2; f++)
        PC(cudaMemcpyAsync(h->kp[f].data(), h->d_kp[f], sizeof(DevKp) * h->kp[f].size(),
                           cudaMemcpyDeviceToHost, h->stream));
    PC(cudaMemcpyAsync(best.data(), h->d_best, sizeof(int) * n0, cudaMemcpyDeviceToHost, h->stream));
    PC(cudaMemcpyAsync(d1.data(), h->d_d1, sizeof(float) * n0, cudaMemcpyDeviceToHost, h->stream));
    PC(cudaMemcpyAsync(d2.data(), h->d_d2, sizeof(float) * n0, cudaMemcpyDeviceToHost, h->stream));
    PC(cudaStreamSynchronize(h->stream));
    // ratio test (CameraPose.cpp:69-78)
    h->m0.clear();
    h->m1.clear();
    h->mdist.clear();
    for (int q = 0; q < n0; q++) {
        if (n1 < 2) break;
        const float a = std::sqrt(d1[q]), b = std::sqrt(d2[q]);
        if ((double)a < h->p.ratio * (double)b) {
            h->m0.push_back(q);
            h->m1.push_back(best[q]);
            h->mdist.push_back(a);
        }
    }
    const int nm = (int)h->m0.size();
    h->minl.assign(nm, 0);
    h->n_inliers = 0;
    if (nm < 5) return pfail(RF_ERR_STATE, "rf_pose_solve: fewer than 5 matches");
    // normalized coordinates x = K^-1 [u v 1]
    const double fx = K[0], sk = K[1], cx = K[2], fy = K[4], cy = K[5];
    std::vector<double> x0(2 * nm), x1(2 * nm);
    for (int m = 0; m < nm; m++) {
        const DevKp& a = h->kp[0][h->m0[m]];
        const DevKp& b = h->kp[1][h->m1[m]];
        x0[2 * m + 1] = ((double)a.y - cy) / fy;
        x0[2 * m] = ((double)a.x - cx - sk * x0[2 * m + 1]) / fx;
        x1[2 * m + 1] = ((double)b.y - cy) / fy;
        x1[2 * m] = ((double)b.x - cx - sk * x1[2 * m + 1]) / fx;
    }
    // LMedS (CameraPose.cpp:80): hypotheses on host threads, medians on the GPU
    const std::vector<double> hyp =
        rf_epi::lmeds_hypotheses(x0.data(), x1.data(), nm, h->p.confidence, h->p.seed);
    const int H = (int)(hyp.size() / 9);
    std::vector<double> med;
    if (H > 0 && nm <= kMaxGpuMatches) {
        if ((size_t)nm > h->x_cap) {
            cudaFree(h->d_x);
            h->d_x = nullptr;
            h->x_cap = 0;
            PC(rf::dev_malloc((void**)&h->d_x, sizeof(double) * 4 * nm));
            h->x_cap = nm;
        }
        if ((size_t)H > h->hyp_cap) {
            cudaFree(h->d_hyp);
            cudaFree(h->d_med);
            h->d_hyp = nullptr;
            h->d_med = nullptr;
            h->hyp_cap = 0;
            PC(rf::dev_malloc((void**)&h->d_hyp, sizeof(double) * 9 * H));
            PC(rf::dev_malloc((void**)&h->d_med, sizeof(double) * H));
            h->hyp_cap = H;
        }
        PC(cudaMemcpyAsync(h->d_x, x0.data(), sizeof(double) * 2 * nm, cudaMemcpyHostToDevice,
                           h->stream));
        PC(cudaMemcpyAsync(h->d_x + 2 * nm, x1.data(), sizeof(double) * 2 * nm,
                           cudaMemcpyHostToDevice, h->stream));
        PC(cudaMemcpyAsync(h->d_hyp, hyp.data(), sizeof(double) * 9 * H, cudaMemcpyHostToDevice,
                           h->stream));
        int npow2 = 1;
        while (npow2 < nm) npow2 <<= 1;
        const size_t smem = sizeof(double) * npow2;
        k_lmeds_median<<<H, 256, smem, h->stream>>>(h->d_hyp, h->d_x, h->d_x + 2 * nm, nm, npow2,
                                                     h->d_med);
        PL();
        h->lmeds_h = H;
        h->lmeds_n = nm;
        med.resize(H);
        PC(cudaMemcpyAsync(med.data(), h->d_med, sizeof(double) * H, cudaMemcpyDeviceToHost,
                           h->stream));
        PC(cudaStreamSynchronize(h->stream));
    } else {
        med = rf_epi::lmeds_medians(hyp, x0.data(), x1.data(), nm);
    }
    double E[9];
    if (!rf_epi::lmeds_select(hyp, med, x0.data(), x1.data(), nm, E, h->minl.data()))
        return pfail(RF_ERR_STATE, "rf_pose_solve: no essential matrix");
    rf_epi::recover_pose(E, x0.data(), x1.data(), nm, h->minl.data(), R, t);
    if (h->p.refine) rf_epi::refine_pose(x0.data(), x1.data(), nm, h->minl.data(), R, t);
    for (uint8_t v : h->minl) h->n_inliers += v;
    h->solved = true;
    return RF_OK;
}

}  // namespace rf_pose_impl

extern "C" {

rf_status rf_pose_params_default(rf_pose_params* p) {
    if (!p) return pfail(RF_ERR_INVALID_ARG, "rf_pose_params_default: null");
    p->hessian_threshold = 2000.0;
    p->n_octaves = 4;
    p->n_octave_layers = 2;
    p->max_keypoints = 0;
    p->ratio = 0.6;
    p->confidence = 0.999;
    p->seed = 0x5eedULL;
    p->refine = 0;
    return RF_OK;
}

rf_status rf_pose_create(const rf_pose_params* p, int width, int height, rf_pose** out) {
    if (!p || !out || width < 16 || height < 16 || (long long)width * height > (1LL << 26))
        return pfail(RF_ERR_INVALID_ARG, "rf_pose_create: bad argument");
    if (p->n_octaves < 1 || p->n_octaves > kMaxOctaves || p->n_octave_layers < 1 ||
        p->n_octave_layers + 2 > kMaxLayers || !(p->ratio > 0.0) ||
        !(p->confidence > 0.0 && p->confidence < 1.0) || p->max_keypoints < 0)
        return pfail(RF_ERR_INVALID_ARG, "rf_pose_create: parameters out of range");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1)
        return pfail(RF_ERR_NO_DEVICE, "rf_pose_create: no CUDA device");
    rf_pose* h = new rf_pose();
    h->p = *p;
    h->w = width;
    h->h = height;
    h->max_kp = p->max_keypoints > 0 ? p->max_keypoints : std::max(16, width * height / 100);
    h->cand_cap = std::max(4 * h->max_kp, 65536);
    const size_t npx = (size_t)width * height, nint = (size_t)(width + 1) * (height + 1);
    cudaError_t e = cudaStreamCreateWithFlags(&h->own, cudaStreamNonBlocking);
    for (int f = 0; f < 2 && e == cudaSuccess; f++) {
        e = rf::dev_malloc((void**)&h->d_img[f], npx);
        if (e == cudaSuccess) e = rf::dev_malloc((void**)&h->d_int[f], nint * sizeof(uint32_t));
        for (int o = 0; o < p->n_octaves && e == cudaSuccess; o++) {
            const size_t cells = (size_t)(width >> o) * (height >> o);
            if (cells == 0) break;
            e = rf::dev_malloc((void**)&h->d_resp[f][o], cells * (p->n_octave_layers + 2) * sizeof(float));
        }
        if (e == cudaSuccess) e = rf::dev_malloc((void**)&h->d_cand[f], sizeof(DevKp) * h->cand_cap);
        if (e == cudaSuccess) e = rf::dev_malloc((void**)&h->d_kp[f], sizeof(DevKp) * h->max_kp);
        if (e == cudaSuccess) e = rf::dev_malloc((void**)&h->d_desc[f], sizeof(float) * kDesc * h->max_kp);
    }
    if (e == cudaSuccess) e = rf::dev_malloc((void**)&h->d_f32, npx * sizeof(float));
    if (e == cudaSuccess) e = rf::dev_malloc((void**)&h->d_count, 2 * sizeof(int));
    if (e == cudaSuccess) e = rf::dev_malloc((void**)&h->d_descT, sizeof(float) * kDesc * h->max_kp);
    if (e == cudaSuccess) e = rf::dev_malloc((void**)&h->d_best, sizeof(int) * h->max_kp);
    if (e == cudaSuccess) e = rf::dev_malloc((void**)&h->d_d1, sizeof(float) * h->max_kp);
    if (e == cudaSuccess) e = rf::dev_malloc((void**)&h->d_d2, sizeof(float) * h->max_kp);
    if (e == cudaSuccess) e = rf::dev_malloc((void**)&h->d_tab, sizeof(Tables));
    if (e == cudaSuccess)
        e = rf::dev_malloc((void**)&h->d_seg, sizeof(uint32_t) * (width + 1) * ((height + kSeg - 1) / kSeg));
    // the scoring kernel's largest shared-memory need, set once (the same
    // value from every handle)
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_lmeds_median, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(sizeof(double) * kMaxGpuMatches));
    if (e == cudaSuccess) {
        const Tables t = make_tables();
        e = cudaMemcpy(h->d_tab, &t, sizeof(Tables), cudaMemcpyHostToDevice);
    }
    // the table copy ran on the legacy default stream: finish it before the
    // handle's non-blocking stream reads the tables
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        rf_pose_destroy(h);
        return pfail(RF_ERR_OOM, std::string("rf_pose_create: ") + cudaGetErrorString(e));
    }
    h->stream = h->own;
    *out = h;
    return RF_OK;
}

rf_status rf_pose_destroy(rf_pose* h) {
    if (!h) return RF_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    for (int f = 0; f < 2; f++) {
        cudaFree(h->d_img[f]);
        cudaFree(h->d_int[f]);
        for (int o = 0; o < kMaxOctaves; o++) cudaFree(h->d_resp[f][o]);
        cudaFree(h->d_cand[f]);
        cudaFree(h->d_kp[f]);
        cudaFree(h->d_desc[f]);
    }
    cudaFree(h->d_f32);
    cudaFree(h->d_count);
    cudaFree(h->d_descT);
    cudaFree(h->d_best);
    cudaFree(h->d_d1);
    cudaFree(h->d_d2);
    cudaFree(h->d_tab);
    cudaFree(h->d_seg);
    cudaFree(h->d_x);
    cudaFree(h->d_hyp);
    cudaFree(h->d_med);
    if (h->own) cudaStreamDestroy(h->own);
    delete h;
    return RF_OK;
}

rf_status rf_pose_set_stream(rf_pose* h, void* stream) {
    if (!h) return pfail(RF_ERR_INVALID_ARG, "rf_pose_set_stream: null handle");
    PC(cudaStreamSynchronize(h->stream));
    h->stream = stream ? (cudaStream_t)stream : h->own;
    return RF_OK;
}

rf_status rf_pose_solve_u8(rf_pose* h, const uint8_t* im0, const uint8_t* im1, int pitch,
                           const double K[9], double R[9], double t[3]) {
    rf::NvtxRange range("rf_pose_solve");
    if (!h || !im0 || !im1 || !K || !R || !t || pitch < h->w)
        return pfail(RF_ERR_INVALID_ARG, "rf_pose_solve_u8: bad argument");
    const uint8_t* src[2] = {im0, im1};
    for (int f = 0; f < 2; f++)
        PC(cudaMemcpy2DAsync(h->d_img[f], h->w, src[f], pitch, h->w, h->h, cudaMemcpyDefault,
                             h->stream));
    return solve(h, K, R, t);
}

rf_status rf_pose_solve_f32(rf_pose* h, const float* im0, const float* im1, int pitch,
                            const double K[9], double R[9], double t[3]) {
    rf::NvtxRange range("rf_pose_solve");
    if (!h || !im0 || !im1 || !K || !R || !t || pitch < h->w)
        return pfail(RF_ERR_INVALID_ARG, "rf_pose_solve_f32: bad argument");
    const float* src[2] = {im0, im1};
    for (int f = 0; f < 2; f++) {
        PC(cudaMemcpy2DAsync(h->d_f32, h->w * sizeof(float), src[f], pitch * sizeof(float),
                             h->w * sizeof(float), h->h, cudaMemcpyDefault, h->stream));
        dim3 blk(32, 8), grd((h->w + 31) / 32, (h->h + 7) / 8);
        k_to_u8<<<grd, blk, 0, h->stream>>>(h->d_f32, h->w, h->h, h->w, h->d_img[f]);
        PL();
    }
    return solve(h, K, R, t);
}

rf_status rf_pose_counts(const rf_pose* h, int* n_kp0, int* n_kp1, int* n_matches,
                         int* n_inliers) {
    if (!h) return pfail(RF_ERR_INVALID_ARG, "rf_pose_counts: null handle");
    if (n_kp0) *n_kp0 = (int)h->kp[0].size();
    if (n_kp1) *n_kp1 = (int)h->kp[1].size();
    if (n_matches) *n_matches = (int)h->m0.size();
    if (n_inliers) *n_inliers = h->n_inliers;
    return RF_OK;
}

rf_status rf_pose_keypoints(const rf_pose* h, int frame, rf_keypoint* kp, float* desc, int cap) {
    if (!h || frame < 0 || frame > 1 || cap < 0)
        return pfail(RF_ERR_INVALID_ARG, "rf_pose_keypoints: bad argument");
    const int n = std::min(cap, (int)h->kp[frame].size());
    for (int i = 0; kp && i < n; i++) {
        const DevKp& d = h->kp[frame][i];
        kp[i] = rf_keypoint{d.x, d.y, d.scale, d.angle, d.response, d.octave};
    }
    if (desc && n > 0)
        PC(cudaMemcpy(desc, h->d_desc[frame], sizeof(float) * kDesc * n, cudaMemcpyDeviceToHost));
    return RF_OK;
}

rf_status rf_pose_matches(const rf_pose* h, int* idx0, int* idx1, float* dist, uint8_t* inlier,
                          int cap) {
    if (!h || cap < 0) return pfail(RF_ERR_INVALID_ARG, "rf_pose_matches: bad argument");
    const int n = std::min(cap, (int)h->m0.size());
    for (int i = 0; i < n; i++) {
        if (idx0) idx0[i] = h->m0[i];
        if (idx1) idx1[i] = h->m1[i];
        if (dist) dist[i] = h->mdist[i];
        if (inlier) inlier[i] = i < (int)h->minl.size() ? h->minl[i] : 0;
    }
    return RF_OK;
}

uint64_t rf_pose_kernel_launches(const rf_pose* h) { return h ? h->launches : 0; }

rf_status rf_pose_profile(rf_pose* h, const float* im0, const float* im1, int pitch,
                          const double K[9], int n_iters, float* ms) {
    if (!h || !ms || n_iters < 1) return pfail(RF_ERR_INVALID_ARG, "rf_pose_profile: bad argument");
    double R[9], t[3];
    rf_status rs = rf_pose_solve_f32(h, im0, im1, pitch, K, R, t);
    if (rs != RF_OK) return rs;
    cudaEvent_t e0, e1;
    PC(cudaEventCreate(&e0));
    PC(cudaEventCreate(&e1));
    for (int stage = 0; stage < 7; stage++) {
        PC(cudaStreamSynchronize(h->stream));
        PC(cudaEventRecord(e0, h->stream));
        for (int it = 0; it < n_iters; it++) {
            switch (stage) {
                case 0: rs = launch_integral(h, 0); break;
                case 1: rs = launch_octaves(h, 0, true, false); break;
                case 2: rs = launch_octaves(h, 0, false, true); break;
                case 3: rs = launch_describe(h, 0, true, false); break;
                case 4: rs = launch_describe(h, 0, false, true); break;
                case 5: rs = launch_match(h); break;
                default:
                    if (h->lmeds_h > 0) {
                        int npow2 = 1;
                        while (npow2 < h->lmeds_n) npow2 <<= 1;
                        k_lmeds_median<<<h->lmeds_h, 256, sizeof(double) * npow2, h->stream>>>(
                            h->d_hyp, h->d_x, h->d_x + 2 * h->lmeds_n, h->lmeds_n, npow2,
                            h->d_med);
                        PL();
                    }
                    break;
            }
            if (rs != RF_OK) return rs;
        }
        PC(cudaEventRecord(e1, h->stream));
        PC(cudaEventSynchronize(e1));
        float t_ms = 0.0f;
        PC(cudaEventElapsedTime(&t_ms, e0, e1));
        ms[stage] = t_ms / n_iters;
    }
    ms[7] = (float)h->kp[0].size();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return RF_OK;
}

rf_status rf_pose_responses(const rf_pose* h, int frame, int octave, float* out, size_t cap) {
    if (!h || !out || frame < 0 || frame > 1 || octave < 0 || octave >= h->p.n_octaves)
        return pfail(RF_ERR_INVALID_ARG, "rf_pose_responses: bad argument");
    const size_t n = (size_t)(h->w >> octave) * (h->h >> octave) * (h->p.n_octave_layers + 2);
    if (cap < n || !h->d_resp[frame][octave])
        return pfail(RF_ERR_INVALID_ARG, "rf_pose_responses: buffer too small");
    PC(cudaStreamSynchronize(h->stream));
    PC(cudaMemcpy(out, h->d_resp[frame][octave], n * sizeof(float), cudaMemcpyDeviceToHost));
    return RF_OK;
}

}  // extern "C"
