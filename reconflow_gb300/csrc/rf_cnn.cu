// Learned warm start: a small convolutional encoder-decoder that maps a
// coarse image pair (+ pixel coordinates and camera pose) to flow and inverse
// depth at two scales, trained on the GPU with hand-written forward and
// backward kernels.  No counterpart in the reference.
//
// Network (NHWC, 3x3 convolutions, padding 1):
//   in  (16 ch: the features of rf_ws_features: coarse frames, plane-sweep
//        costs, epipolar derivative)
//   c1  16 -> 32, ReLU                      (input resolution, "1/8")
//   c2  32 -> 96, stride 2, ReLU            (half resolution, "1/16")
//   c3  96 -> 96, ReLU
//   h16 96 -> 8 (u, v, inverse depth, 5 unused), linear   -> output at 1/16
//   cat [nearest-upsampled c3 (96), c1 (32)] = 128 channels
//   c4  128 -> 64, ReLU
//   h8  64 -> 8, linear                                    -> output at 1/8
// Weights and activations are BF16, accumulation FP32; the master weights
// and Adam moments are FP32.
//
// Every convolution (forward, gradient of its input, gradient of its
// weights) is one implicit GEMM on the Blackwell tensor cores (rf_tc.cuh:
// tcgen05.mma, BF16 operands gathered into shared memory, FP32 accumulator
// in tensor memory).  The weight gradient splits the pixel (reduction)
// dimension into chunks whose partial sums are added in a fixed order, so
// training is deterministic.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/reconflow_gb300.h"
#include "rf_alloc.h"
#include "rf_nvtx.h"
#include "rf_kernels.cuh"
#include "rf_tc.cuh"

namespace rf_cnn_impl {

typedef __nv_bfloat16 bf16;

__device__ __forceinline__ uint32_t pack2(bf16 lo, bf16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

struct Shape {
    int B, H, W, C;  // NHWC
};

// ---- tcgen05 GEMM operands: 8 consecutive K elements of one row ----------
__device__ __forceinline__ uint4 pack8(const bf16 (&v)[8]) {
    return make_uint4(pack2(v[0], v[1]), pack2(v[2], v[3]), pack2(v[4], v[5]), pack2(v[6], v[7]));
}

// forward A: im2col row of output pixel m, k = (ky*3 + kx)*Cin + ci (Cin % 8 == 0)
struct TcConvIn {
    static constexpr bool kAsync = true;
    const bf16* x;
    int B, H, W, C, Ho, Wo, stride;
    __device__ const void* base() const { return x; }
    __device__ const void* src(int m, int k) const {
        int ci = k % C, t = k / C, kx = t % 3, ky = t / 3;
        int xo = m % Wo, r = m / Wo, yo = r % Ho, b = r / Ho;
        int y = yo * stride + ky - 1, xx = xo * stride + kx - 1;
        if (y < 0 || y >= H || xx < 0 || xx >= W) return nullptr;
        return x + (((size_t)b * H + y) * W + xx) * C + ci;
    }
};

// K-major matrix rows: w[n][k], K % 8 == 0
struct TcRows {
    static constexpr bool kAsync = true;
    const bf16* w;
    int K;
    __device__ const void* base() const { return w; }
    __device__ const void* src(int n, int k) const { return w + (size_t)n * K + k; }
};

// input-gradient A: input pixel m, k = (ky*3 + kx)*Cout + co -> dy at the
// output pixel that tap (ky, kx) of m feeds (Cout % 8 == 0)
struct TcDataGradA {
    static constexpr bool kAsync = true;
    const bf16* dy;
    int H, W, Ho, Wo, Cout, stride;
    __device__ const void* base() const { return dy; }
    __device__ const void* src(int m, int k) const {
        int co = k % Cout, t = k / Cout, kx = t % 3, ky = t / 3;
        int xx = m % W, r = m / W, y = r % H, b = r / H;
        int ty = y + 1 - ky, tx = xx + 1 - kx;
        if (ty < 0 || tx < 0 || ty % stride || tx % stride) return nullptr;
        int yo = ty / stride, xo = tx / stride;
        if (yo >= Ho || xo >= Wo) return nullptr;
        return dy + (((size_t)b * Ho + yo) * Wo + xo) * Cout + co;
    }
};

// weight-gradient A: row m = (ky*3 + kx)*Cin + ci of im2col^T, k = output pixel
struct TcWGradA {
    static constexpr bool kAsync = false;
    const bf16* x;
    int H, W, C, Ho, Wo, stride;
    __device__ uint4 operator()(int m, int k, int k_end) const {
        int ci = m % C, t = m / C, kx = t % 3, ky = t / 3;
        bf16 v[8];
#pragma unroll
        for (int e = 0; e < 8; e++) {
            int p = k + e;
            v[e] = __float2bfloat16(0.f);
            if (p < k_end) {
                int xo = p % Wo, r = p / Wo, yo = r % Ho, b = r / Ho;
                int y = yo * stride + ky - 1, xx = xo * stride + kx - 1;
                if (y >= 0 && y < H && xx >= 0 && xx < W)
                    v[e] = x[(((size_t)b * H + y) * W + xx) * C + ci];
            }
        }
        return pack8(v);
    }
};

// weight-gradient B: row n = co, k = output pixel -> dy[pixel][co]
struct TcWGradB {
    static constexpr bool kAsync = false;
    const bf16* dy;
    int Cout;
    __device__ uint4 operator()(int n, int k, int k_end) const {
        bf16 v[8];
#pragma unroll
        for (int e = 0; e < 8; e++)
            v[e] = k + e < k_end ? dy[(size_t)(k + e) * Cout + n] : __float2bfloat16(0.f);
        return pack8(v);
    }
};

// weight-gradient partial of split z: part[z][co = n][row m]
struct TcStoreWGrad {
    float* part;
    int M, N;
    __device__ void operator()(int z, int m, int n, float v) const {
        part[((size_t)z * N + n) * M + m] = v;
    }
};

// [co][tap][ci] -> [ci][tap][co] (the input gradient's K-major B operand)
__global__ void k_transpose_w(const bf16* w, int cin, int cout, bf16* wt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int n = cout * 9 * cin;
    if (i >= n) return;
    int ci = i % cin, t = (i / cin) % 9, co = i / (9 * cin);
    wt[((size_t)ci * 9 + t) * cout + co] = w[i];
}

// forward epilogue: + bias, optional ReLU; BF16 activation and/or FP32 copy
struct ConvOut {
    const float* bias;
    bf16* y;
    float* yf;
    int M, Cout, relu;
    __device__ void operator()(int, int m, int n, float v) const {
        if (m >= M || n >= Cout) return;
        v += bias[n];
        if (relu) v = fmaxf(v, 0.f);
        if (y) y[(size_t)m * Cout + n] = __float2bfloat16(v);
        if (yf) yf[(size_t)m * Cout + n] = v;
    }
};

struct StoreF32 {
    float* out;
    int M, N;
    __device__ void operator()(int, int m, int n, float v) const {
        if (m < M && n < N) out[(size_t)m * N + n] = v;
    }
};

__global__ void k_reduce_partials(const float* part, int chunks, int n, float* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float s = 0.f;
    for (int c = 0; c < chunks; c++) s += part[(size_t)c * n + i];
    out[i] = s;
}

// bias gradient, stage 1: block b sums dy over its pixel range
// [b * span, (b + 1) * span) for every channel; thread t takes channel t % C
// and every R-th pixel from t / C (R = 256 / C), then the R partial sums of a
// channel are added in a fixed order.  Stage 2 (k_reduce_partials) adds the
// block partials in block order, so the result is deterministic.
constexpr int kBiasThreads = 256;

__global__ void __launch_bounds__(kBiasThreads) k_bias_partial(const float* dy, int P, int C,
                                                               int span, float* part) {
    __shared__ float red[kBiasThreads];
    const int t = threadIdx.x, R = kBiasThreads / C;
    const int c = t % C, r = t / C;
    const int p0 = blockIdx.x * span, p1 = min(P, p0 + span);
    float acc = 0.f;
    if (r < R)
        for (int p = p0 + r; p < p1; p += R) acc += dy[(size_t)p * C + c];
    red[t] = acc;
    __syncthreads();
    if (t < C) {
        float s = 0.f;
        for (int k = 0; k < R; k++) s += red[t + k * C];
        part[(size_t)blockIdx.x * C + t] = s;
    }
}

__global__ void k_f32_to_bf16(const float* a, bf16* b, size_t n) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = __float2bfloat16(a[i]);
}

// dy = g * [activation > 0] (ReLU backward), in place on g, and a BF16 copy
__global__ void k_relu_grad(float* g, const bf16* act, bf16* gb, size_t n) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float v = __bfloat162float(act[i]) > 0.f ? g[i] : 0.f;
    g[i] = v;
    gb[i] = __float2bfloat16(v);
}

// cat = [nearest 2x upsample of a (Ha x Wa x Ca), b (H x W x Cb)]
__global__ void k_concat_up(const bf16* a, int Ha, int Wa, int Ca, const bf16* b, int Cb,
                            int Bn, int H, int W, bf16* cat) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t n = (size_t)Bn * H * W * (Ca + Cb);
    if (i >= n) return;
    int C = Ca + Cb;
    int c = i % C;
    size_t p = i / C;
    int x = p % W, r = p / W, y = r % H, bb = r / H;
    if (c < Ca)
        cat[i] = a[(((size_t)bb * Ha + y / 2) * Wa + x / 2) * Ca + c];
    else
        cat[i] = b[p * Cb + (c - Ca)];
}

// split the concat gradient: d_a (half resolution) += sum of its 2x2
// children; d_b (+)= the rest.  accumulate != 0 adds to the existing values.
__global__ void k_concat_up_grad(const float* dcat, int Ha, int Wa, int Ca, int Cb, int Bn,
                                 int H, int W, float* da, float* db, int accumulate_b) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t na = (size_t)Bn * Ha * Wa * Ca;
    size_t nb = (size_t)Bn * H * W * Cb;
    int C = Ca + Cb;
    if (i < na) {
        int c = i % Ca;
        size_t p = i / Ca;
        int x = p % Wa, r = p / Wa, y = r % Ha, bb = r / Ha;
        float s = 0.f;
        for (int dy = 0; dy < 2; dy++)
            for (int dx = 0; dx < 2; dx++) {
                int yy = 2 * y + dy, xx = 2 * x + dx;
                if (yy < H && xx < W) s += dcat[(((size_t)bb * H + yy) * W + xx) * C + c];
            }
        da[i] += s;
    }
    if (i < nb) {
        int c = i % Cb;
        size_t p = i / Cb;
        float v = dcat[p * C + Ca + c];
        db[i] = accumulate_b ? db[i] + v : v;
    }
}

// L1 loss on channels 0..2 with per-channel weights, masked; writes dL/dpred
// (already divided by the number of valid pixels) and accumulates the loss.
__global__ void k_l1_loss(const float* pred, const float* tgt, const float* mask, int P, int C,
                          float w0, float w1, float w2, float inv_count, float* grad,
                          double* loss) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    double l = 0.0;
    if (p < P) {
        float m = mask[p];
        for (int c = 0; c < C; c++) {
            float g = 0.f;
            if (c < 3 && m > 0.f) {
                float wc = c == 0 ? w0 : (c == 1 ? w1 : w2);
                float d = pred[(size_t)p * C + c] - tgt[(size_t)p * C + c];
                l += (double)(wc * fabsf(d)) * inv_count;
                g = (d > 0.f ? wc : (d < 0.f ? -wc : 0.f)) * inv_count;
            }
            grad[(size_t)p * C + c] = g;
        }
    }
    for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, l);
}

__global__ void k_adam(float* w, const float* g, float* m, float* v, size_t n, float lr, float b1,
                       float b2, float eps, float c1, float c2) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float gi = g[i];
    float mi = b1 * m[i] + (1.f - b1) * gi;
    float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    float mh = mi / c1, vh = vi / c2;
    w[i] -= lr * mh / (sqrtf(vh) + eps);
}

__global__ void k_add(float* a, const float* b, size_t n) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] += b[i];
}

inline unsigned blocks_for(size_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

// ---- inference path on padded activations (rf_tc::k_tc_conv3) -------------
// A padded buffer holds [B][H + 2][W + 2][C] BF16 with a zero one-pixel
// border; interior pixel (b, y, x) is at position (b (H + 2) + y + 1)(W + 2)
// + x + 1.  Borders are zeroed once at creation and never written.
__device__ __forceinline__ size_t pad_pos(int b, int y, int x, int H, int W) {
    return ((size_t)b * (H + 2) + y + 1) * (W + 2) + x + 1;
}

// FP32 input [B][H][W][16] -> padded BF16 interior, 8 channels per thread
__global__ void k_pad_input(const float* in, int B, int H, int W, bf16* xp) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t n = (size_t)B * H * W * 2;
    if (i >= n) return;
    const int g = (int)(i % 2);
    const size_t p = i / 2;
    const int x = (int)(p % W), r = (int)(p / W), y = r % H, b = r / H;
    const float* s = in + p * 16 + g * 8;
    bf16 v[8];
#pragma unroll
    for (int e = 0; e < 8; e++) v[e] = __float2bfloat16(s[e]);
    *(uint4*)(xp + pad_pos(b, y, x, H, W) * 16 + g * 8) = pack8(v);
}

// padded cat = [nearest 2x upsample of a (Ha x Wa x Ca), b (H x W x Cb)],
// 8 channels per thread (Ca, Cb multiples of 8)
__global__ void k_concat_up_pad(const bf16* a, int Ha, int Wa, int Ca, const bf16* bsrc, int Cb,
                                int Bn, int H, int W, bf16* cat) {
    const int C = Ca + Cb, G = C / 8;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t n = (size_t)Bn * H * W * G;
    if (i >= n) return;
    const int c = (int)(i % G) * 8;
    const size_t p = i / G;
    const int x = (int)(p % W), r = (int)(p / W), y = r % H, bb = r / H;
    uint4 v = c < Ca ? *(const uint4*)(a + pad_pos(bb, y / 2, x / 2, Ha, Wa) * Ca + c)
                     : *(const uint4*)(bsrc + pad_pos(bb, y, x, H, W) * Cb + (c - Ca));
    *(uint4*)(cat + pad_pos(bb, y, x, H, W) * C + c) = v;
}

// weights [co][tap][ci] -> the direct kernel's [stage][tap][NT / 8][2][8][8]
// (co = 8 group + row, ci = 16 stage + 8 half + e; rows co >= cout are zero)
__global__ void k_conv_wc(const bf16* w, int cin, int cout, int NT, bf16* wc) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int ng = NT / 8;
    size_t n = (size_t)(cin / 16) * 9 * NT * 16;
    if (i >= n) return;
    const int e = (int)(i % 8), r = (int)(i / 8 % 8), kh = (int)(i / 64 % 2);
    const int gi = (int)(i / 128 % ng), t = (int)(i / (128 * (size_t)ng) % 9);
    const int j = (int)(i / (128 * (size_t)ng * 9));
    const int co = gi * 8 + r, ci = 16 * j + 8 * kh + e;
    wc[i] = co < cout ? w[((size_t)co * 9 + t) * cin + ci] : __float2bfloat16(0.f);
}

// epilogue of the direct kernel: + bias, optional ReLU; BF16 into the padded
// output (same geometry as the input) and / or FP32 into an unpadded
// [B][H][W][cout_f] buffer
struct ConvOutPadded {
    const float* bias;
    int nbias;
    bf16* y;  // padded [pos][cout] or null
    int cout;
    float* yf;  // unpadded FP32 or null
    int cout_f;
    int relu, H, W, npos;
    __device__ int pos(int q) const {
        if (q >= npos) return -1;
        const int Wp = W + 2, Hp = H + 2;
        const int x = q % Wp, r = q / Wp, yy = r % Hp, b = r / Hp;
        if (x < 1 || x > W || yy < 1 || yy > H) return -1;
        return (b * H + yy - 1) * W + (x - 1);
    }
    __device__ void store(int q, int p, int c, const float (&v)[8]) const {
        float o[8];
#pragma unroll
        for (int e = 0; e < 8; e++) {
            float t = v[e] + (c + e < nbias ? bias[c + e] : 0.f);
            o[e] = relu ? fmaxf(t, 0.f) : t;
        }
        if (y && c < cout) {
            bf16 h[8];
#pragma unroll
            for (int e = 0; e < 8; e++) h[e] = __float2bfloat16(o[e]);
            *(uint4*)(y + (size_t)q * cout + c) = pack8(h);
        }
        if (yf)
#pragma unroll
            for (int e = 0; e < 8; e++)
                if (c + e < cout_f) yf[(size_t)p * cout_f + c + e] = o[e];
    }
};

// the stride-2 layer keeps the im2col GEMM: its input and output padded
struct TcConvInPadded {
    static constexpr bool kAsync = true;
    const bf16* x;
    int H, W, C, Ho, Wo, stride;
    __device__ const void* base() const { return x; }
    __device__ const void* src(int m, int k) const {
        int ci = k % C, t = k / C, kx = t % 3, ky = t / 3;
        int xo = m % Wo, r = m / Wo, yo = r % Ho, b = r / Ho;
        // padded coordinates: the border supplies the zeros of the padding
        int y = yo * stride + ky, xx = xo * stride + kx;
        return x + (((size_t)b * (H + 2) + y) * (W + 2) + xx) * C + ci;
    }
};

struct ConvOutToPadded {
    const float* bias;
    bf16* y;
    int M, Cout, relu, Ho, Wo;
    __device__ void operator()(int, int m, int n, float v) const {
        if (m >= M || n >= Cout) return;
        v += bias[n];
        if (relu) v = fmaxf(v, 0.f);
        int xo = m % Wo, r = m / Wo, yo = r % Ho, b = r / Ho;
        y[pad_pos(b, yo, xo, Ho, Wo) * Cout + n] = __float2bfloat16(v);
    }
};

struct Layer {
    int cin, cout, stride, relu;
    size_t woff, boff;  // offsets into the parameter vector
};

}  // namespace rf_cnn_impl

using namespace rf_cnn_impl;

struct rf_cnn {
    int max_batch = 0, H = 0, W = 0;  // input resolution
    std::vector<Layer> layers;        // c1, c2, c3, h16, c4, h8
    size_t n_params = 0;
    float *w = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;  // FP32 master, grad, Adam
    bf16* wb = nullptr;               // BF16 copy used by the kernels
    bf16* wt = nullptr;               // BF16 weights per layer as [ci][tap][co]
    int* d_status = nullptr;          // set by a tensor-core launch whose wait gave up
    int test_first_wait_polls = -1;   // rf_cnn_set_test_wait_limit (-1: the normal limit)
    int step = 0;
    // activations (BF16) and gradients (FP32 / BF16)
    bf16 *x = nullptr, *a1 = nullptr, *a2 = nullptr, *a3 = nullptr, *cat = nullptr, *a4 = nullptr;
    float *o16 = nullptr, *o8 = nullptr;
    float *g_o16 = nullptr, *g_o8 = nullptr, *g_a4 = nullptr, *g_cat = nullptr, *g_a3 = nullptr,
          *g_a2 = nullptr, *g_a1 = nullptr;
    bf16* gb = nullptr;   // BF16 staging of the gradient being propagated
    float* part = nullptr;
    size_t part_floats = 0;
    double* d_loss = nullptr;
    cudaStream_t stream = nullptr;
    uint64_t launches = 0;
    // inference on padded activations (rf_cnn_forward; training keeps the GEMMs)
    bool direct = false;
    bf16 *xp = nullptr, *a1p = nullptr, *a2p = nullptr, *a3p = nullptr, *catp = nullptr,
         *a4p = nullptr;
    int pad_h = -1, pad_w = -1;  // the frame size whose borders the padded buffers hold zero
    size_t pad_elems[6] = {};    // BF16 elements allocated per padded buffer
    bf16* wc[6] = {};  // per layer, the direct kernel's weight layout (null: c2)
    int nt[6] = {};    // per layer, the direct kernel's N tile
    CUtensorMap map_x{}, map_a2{}, map_a3{}, map_cat{}, map_a4{};
};

namespace rf_cnn_impl {

rf_status cfail(rf_status st, const std::string& msg) {
    return static_cast<rf_status>(rf::set_last_error(st, msg.c_str()));
}

#define CN(call)                                                                      \
    do {                                                                              \
        cudaError_t e__ = (call);                                                     \
        if (e__ != cudaSuccess)                                                       \
            return cfail(e__ == cudaErrorMemoryAllocation ? RF_ERR_OOM : RF_ERR_CUDA,         \
                        std::string(#call ": ") + cudaGetErrorString(e__));            \
    } while (0)

int Ho_of(int H, int s) { return s == 1 ? H : (H + 1) / 2; }

template <int NT, class LA, class LB, class EP>
rf_status tc_launch(rf_cnn* c, int M, int N, int K, int splits, LA la, LB lb, EP ep) {
    using S = rf_tc::TcSmem<NT, rf_tc::stages_for<LA, LB>()>;
    static bool attr_set = false;
    if (!attr_set) {
        CN(cudaFuncSetAttribute(rf_tc::k_tc_gemm<NT, LA, LB, EP>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, S::kBytes));
        attr_set = true;
    }
    int kspan = ((K + splits - 1) / splits + rf_tc::kTK - 1) / rf_tc::kTK * rf_tc::kTK;
    splits = (K + kspan - 1) / kspan;
    dim3 grid((M + rf_tc::kTM - 1) / rf_tc::kTM, (N + NT - 1) / NT, splits);
    rf_tc::k_tc_gemm<NT, LA, LB, EP><<<grid, rf_tc::kThreads, S::kBytes, c->stream>>>(
        M, N, K, kspan, la, lb, ep, c->d_status, c->test_first_wait_polls);
    c->launches++;
    CN(cudaGetLastError());
    return RF_OK;
}

// D[M x N] = A[M x K] B[N x K]^T on the tensor cores; returns the number of
// K splits actually used through *used (if not null)
template <class LA, class LB, class EP>
rf_status tc_gemm(rf_cnn* c, int M, int N, int K, int splits, LA la, LB lb, EP ep,
                  int* used = nullptr) {
    if (used) {
        int kspan = ((K + splits - 1) / splits + rf_tc::kTK - 1) / rf_tc::kTK * rf_tc::kTK;
        *used = (K + kspan - 1) / kspan;
    }
    if (N <= 16) return tc_launch<16>(c, M, N, K, splits, la, lb, ep);
    if (N <= 32) return tc_launch<32>(c, M, N, K, splits, la, lb, ep);
    if (N <= 64) return tc_launch<64>(c, M, N, K, splits, la, lb, ep);
    if (N <= 96) return tc_launch<96>(c, M, N, K, splits, la, lb, ep);
    return tc_launch<128>(c, M, N, K, splits, la, lb, ep);
}

// forward conv of layer L: x (B x H x W x cin) -> y (BF16) and/or yf (FP32)
rf_status conv_fwd(rf_cnn* c, const Layer& L, const bf16* x, int B, int H, int W, bf16* y,
                   float* yf) {
    int Ho = Ho_of(H, L.stride), Wo = Ho_of(W, L.stride);
    int M = B * Ho * Wo, K = 9 * L.cin;
    TcConvIn la{x, B, H, W, L.cin, Ho, Wo, L.stride};
    TcRows lb{c->wb + L.woff, K};
    ConvOut ep{c->w + L.boff, y, yf, M, L.cout, L.relu};
    return tc_gemm(c, M, L.cout, K, 1, la, lb, ep);
}

// backward of layer L given dy (FP32, already through the ReLU mask) and its
// BF16 copy: weight and bias gradients, and the input gradient if dx != null
rf_status conv_bwd(rf_cnn* c, const Layer& L, const bf16* x, int B, int H, int W,
                   const float* dy, const bf16* dyb, float* dx) {
    int Ho = Ho_of(H, L.stride), Wo = Ho_of(W, L.stride);
    int P = B * Ho * Wo, Mw = 9 * L.cin;
    // weight gradient: [tap*cin + ci] x [co] over the pixels, split over K
    int splits = std::max(1, std::min(128, P / 4096));
    int used = 1;
    size_t need = (size_t)splits * L.cout * Mw;
    if (need > c->part_floats) return cfail(RF_ERR_STATE, "cnn: partial buffer too small");
    rf_status rs = tc_gemm(c, Mw, L.cout, P, splits, TcWGradA{x, H, W, L.cin, Ho, Wo, L.stride},
                           TcWGradB{dyb, L.cout}, TcStoreWGrad{c->part, Mw, L.cout}, &used);
    if (rs != RF_OK) return rs;
    k_reduce_partials<<<blocks_for((size_t)L.cout * Mw), 256, 0, c->stream>>>(
        c->part, used, L.cout * Mw, c->g + L.woff);
    // bias: the weight-gradient partials are consumed above, so their buffer is free
    const int span = 2048, nblk = (P + span - 1) / span;
    if ((size_t)nblk * L.cout > c->part_floats || L.cout > kBiasThreads)
        return cfail(RF_ERR_STATE, "cnn: partial buffer too small for the bias gradient");
    k_bias_partial<<<nblk, kBiasThreads, 0, c->stream>>>(dy, P, L.cout, span, c->part);
    k_reduce_partials<<<blocks_for(L.cout, 64), 64, 0, c->stream>>>(c->part, nblk, L.cout,
                                                                   c->g + L.boff);
    c->launches += 3;
    if (dx) {
        int M = B * H * W, K = 9 * L.cout;
        rs = tc_gemm(c, M, L.cin, K, 1, TcDataGradA{dyb, H, W, Ho, Wo, L.cout, L.stride},
                     TcRows{c->wt + L.woff, K}, StoreF32{dx, M, L.cin});
        if (rs != RF_OK) return rs;
    }
    CN(cudaGetLastError());
    return RF_OK;
}

rf_status sync_bf16_weights(rf_cnn* c) {
    k_f32_to_bf16<<<blocks_for(c->n_params), 256, 0, c->stream>>>(c->w, c->wb, c->n_params);
    c->launches++;
    for (size_t li = 0; li < c->layers.size(); li++) {
        const Layer& L = c->layers[li];
        k_transpose_w<<<blocks_for((size_t)L.cout * 9 * L.cin), 256, 0, c->stream>>>(
            c->wb + L.woff, L.cin, L.cout, c->wt + L.woff);
        c->launches++;
        if (c->wc[li]) {
            const size_t n = (size_t)(L.cin / 16) * 9 * c->nt[li] * 16;
            k_conv_wc<<<blocks_for(n), 256, 0, c->stream>>>(c->wb + L.woff, L.cin, L.cout,
                                                           c->nt[li], c->wc[li]);
            c->launches++;
        }
    }
    CN(cudaGetLastError());
    return RF_OK;
}

// one stride-1 layer on the direct kernel: `map` covers its padded input
template <int NT>
rf_status conv3_direct(rf_cnn* c, int li, const CUtensorMap& map, int B, int H, int W,
                       bf16* y, float* yf) {
    const Layer& L = c->layers[li];
    using S = rf_tc::ConvSmem<NT>;
    rf_tc::ConvGeom g;
    g.Wp = W + 2;
    g.npos = B * (H + 2) * (W + 2);
    g.nbox = (rf_tc::kTM + 2 * (W + 3) + rf_tc::kConvBox - 1) / rf_tc::kConvBox;
    g.stages = L.cin / 16;
    const size_t smem = S::bytes(g.nbox);
    static bool attr_set = false;
    if (!attr_set) {
        CN(cudaFuncSetAttribute(rf_tc::k_tc_conv3<NT, ConvOutPadded>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
        attr_set = true;
    }
    if (smem > 227 * 1024) return cfail(RF_ERR_UNSUPPORTED, "cnn: row too long for the direct kernel");
    ConvOutPadded ep{c->w + L.boff, L.cout, y, L.cout, yf, L.cout, L.relu, H, W, g.npos};
    const unsigned grid = (unsigned)((g.npos + rf_tc::kTM - 1) / rf_tc::kTM);
    rf_tc::k_tc_conv3<NT, ConvOutPadded><<<grid, rf_tc::kThreads, smem, c->stream>>>(
        map, c->wc[li], g, ep, c->d_status, c->test_first_wait_polls);
    c->launches++;
    CN(cudaGetLastError());
    return RF_OK;
}

// inference: padded activations (laid out for this call's frame size, up to
// the allocated one), the stride-1 layers on the direct kernel, the stride-2
// layer on the im2col GEMM
rf_status forward_direct(rf_cnn* c, const float* input, int B, int H, int W) {
    const int H2 = Ho_of(H, 2), W2 = Ho_of(W, 2);
    const Layer &c1 = c->layers[0], &c2 = c->layers[1], &c3 = c->layers[2];
    if (H != c->pad_h || W != c->pad_w) {
        // a new frame size moves the borders: clear the buffers once (the
        // kernels never write a border position of the size they run at)
        bf16* bufs[6] = {c->xp, c->a1p, c->a2p, c->a3p, c->catp, c->a4p};
        for (int k = 0; k < 6; k++)
            CN(cudaMemsetAsync(bufs[k], 0, c->pad_elems[k] * 2, c->stream));
        c->pad_h = H;
        c->pad_w = W;
    }
    k_pad_input<<<blocks_for((size_t)B * H * W * 2), 256, 0, c->stream>>>(input, B, H, W, c->xp);
    c->launches++;
    rf_status rs = conv3_direct<32>(c, 0, c->map_x, B, H, W, c->a1p, nullptr);
    if (rs == RF_OK) {
        const int M = B * H2 * W2, K = 9 * c2.cin;
        rs = tc_gemm(c, M, c2.cout, K, 1,
                     TcConvInPadded{c->a1p, H, W, c2.cin, H2, W2, c2.stride},
                     TcRows{c->wb + c2.woff, K},
                     ConvOutToPadded{c->w + c2.boff, c->a2p, M, c2.cout, c2.relu, H2, W2});
    }
    if (rs == RF_OK) rs = conv3_direct<96>(c, 2, c->map_a2, B, H2, W2, c->a3p, nullptr);
    if (rs == RF_OK) rs = conv3_direct<16>(c, 3, c->map_a3, B, H2, W2, nullptr, c->o16);
    if (rs != RF_OK) return rs;
    k_concat_up_pad<<<blocks_for((size_t)B * H * W * ((c3.cout + c1.cout) / 8)), 256, 0,
                      c->stream>>>(c->a3p, H2, W2, c3.cout, c->a1p, c1.cout, B, H, W, c->catp);
    c->launches++;
    rs = conv3_direct<64>(c, 4, c->map_cat, B, H, W, c->a4p, nullptr);
    if (rs == RF_OK) rs = conv3_direct<16>(c, 5, c->map_a4, B, H, W, nullptr, c->o8);
    if (rs != RF_OK) return rs;
    CN(cudaGetLastError());
    return RF_OK;
}

rf_status forward(rf_cnn* c, const float* input, int B, int H, int W) {
    const Layer &c1 = c->layers[0], &c2 = c->layers[1], &c3 = c->layers[2], &h16 = c->layers[3],
                &c4 = c->layers[4], &h8 = c->layers[5];
    size_t nin = (size_t)B * H * W * 16;
    k_f32_to_bf16<<<blocks_for(nin), 256, 0, c->stream>>>(input, c->x, nin);
    c->launches++;
    int H2 = Ho_of(H, 2), W2 = Ho_of(W, 2);
    rf_status rs = conv_fwd(c, c1, c->x, B, H, W, c->a1, nullptr);
    if (rs == RF_OK) rs = conv_fwd(c, c2, c->a1, B, H, W, c->a2, nullptr);
    if (rs == RF_OK) rs = conv_fwd(c, c3, c->a2, B, H2, W2, c->a3, nullptr);
    if (rs == RF_OK) rs = conv_fwd(c, h16, c->a3, B, H2, W2, nullptr, c->o16);
    if (rs != RF_OK) return rs;
    size_t ncat = (size_t)B * H * W * (c3.cout + c1.cout);
    k_concat_up<<<blocks_for(ncat), 256, 0, c->stream>>>(c->a3, H2, W2, c3.cout, c->a1, c1.cout,
                                                         B, H, W, c->cat);
    c->launches++;
    rs = conv_fwd(c, c4, c->cat, B, H, W, c->a4, nullptr);
    if (rs == RF_OK) rs = conv_fwd(c, h8, c->a4, B, H, W, nullptr, c->o8);
    return rs;
}

rf_status backward(rf_cnn* c, int B, int H, int W) {
    const Layer &c1 = c->layers[0], &c2 = c->layers[1], &c3 = c->layers[2], &h16 = c->layers[3],
                &c4 = c->layers[4], &h8 = c->layers[5];
    int H2 = Ho_of(H, 2), W2 = Ho_of(W, 2);
    size_t n8 = (size_t)B * H * W * 8, n16 = (size_t)B * H2 * W2 * 8;
    // heads (linear)
    k_f32_to_bf16<<<blocks_for(n8), 256, 0, c->stream>>>(c->g_o8, c->gb, n8);
    rf_status rs = conv_bwd(c, h8, c->a4, B, H, W, c->g_o8, c->gb, c->g_a4);
    if (rs != RF_OK) return rs;
    size_t n4 = (size_t)B * H * W * c4.cout;
    k_relu_grad<<<blocks_for(n4), 256, 0, c->stream>>>(c->g_a4, c->a4, c->gb, n4);
    rs = conv_bwd(c, c4, c->cat, B, H, W, c->g_a4, c->gb, c->g_cat);
    if (rs != RF_OK) return rs;
    // split the concat gradient: g_a3 = up^T(g_cat[:96]), g_a1 = g_cat[96:]
    size_t n3 = (size_t)B * H2 * W2 * c3.cout;
    size_t n1 = (size_t)B * H * W * c1.cout;
    CN(cudaMemsetAsync(c->g_a3, 0, n3 * sizeof(float), c->stream));
    k_concat_up_grad<<<blocks_for(std::max(n3, n1)), 256, 0, c->stream>>>(
        c->g_cat, H2, W2, c3.cout, c1.cout, B, H, W, c->g_a3, c->g_a1, 0);
    // 1/16 head adds into g_a3
    k_f32_to_bf16<<<blocks_for(n16), 256, 0, c->stream>>>(c->g_o16, c->gb, n16);
    float* tmp = c->g_a2;  // scratch for the head's input gradient (same size as g_a3)
    rs = conv_bwd(c, h16, c->a3, B, H2, W2, c->g_o16, c->gb, tmp);
    if (rs != RF_OK) return rs;
    // g_a3 += tmp (reuse the ReLU kernel path: add then mask)
    k_add<<<blocks_for(n3), 256, 0, c->stream>>>(c->g_a3, tmp, n3);
    k_relu_grad<<<blocks_for(n3), 256, 0, c->stream>>>(c->g_a3, c->a3, c->gb, n3);
    rs = conv_bwd(c, c3, c->a2, B, H2, W2, c->g_a3, c->gb, c->g_a2);
    if (rs != RF_OK) return rs;
    size_t n2 = (size_t)B * H2 * W2 * c2.cout;
    k_relu_grad<<<blocks_for(n2), 256, 0, c->stream>>>(c->g_a2, c->a2, c->gb, n2);
    // c2's input gradient adds into g_a1 (which holds the skip part): use tmp2
    float* tmp2 = c->g_a4;  // free now, large enough (B*H*W*64 >= B*H*W*32)
    rs = conv_bwd(c, c2, c->a1, B, H, W, c->g_a2, c->gb, tmp2);
    if (rs != RF_OK) return rs;
    k_add<<<blocks_for(n1), 256, 0, c->stream>>>(c->g_a1, tmp2, n1);
    k_relu_grad<<<blocks_for(n1), 256, 0, c->stream>>>(c->g_a1, c->a1, c->gb, n1);
    rs = conv_bwd(c, c1, c->x, B, H, W, c->g_a1, c->gb, nullptr);
    c->launches += 9;
    if (rs != RF_OK) return rs;
    CN(cudaGetLastError());
    return RF_OK;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against libcuda): a 2D map over a padded buffer viewed as [positions][C]
// BF16, boxes of 8 channels x kConvBox positions, zero fill outside
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

bool encode_positions_map(CUtensorMap* m, const bf16* base, int C, size_t npos) {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !p)
            return false;
        fn = (EncodeTiledFn)p;
    }
    const cuuint64_t dims[2] = {(cuuint64_t)C, (cuuint64_t)npos};
    const cuuint64_t strides[1] = {(cuuint64_t)C * 2};
    const cuuint32_t box[2] = {8, (cuuint32_t)rf_tc::kConvBox};
    const cuuint32_t es[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void*)base, dims, strides, box, es,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// whether the direct kernel's shared memory fits rows of width W
bool direct_fits(int W) {
    const int nbox = (rf_tc::kTM + 2 * (W + 3) + rf_tc::kConvBox - 1) / rf_tc::kConvBox;
    const size_t lim = 227 * 1024;
    return rf_tc::ConvSmem<32>::bytes(nbox) <= lim && rf_tc::ConvSmem<64>::bytes(nbox) <= lim &&
           rf_tc::ConvSmem<96>::bytes(nbox) <= lim;
}

}  // namespace rf_cnn_impl

extern "C" {

rf_status rf_cnn_create(int max_batch, int height, int width, unsigned long long seed,
                        rf_cnn** out) {
    if (!out || max_batch < 1 || height < 2 || width < 2 || (long long)max_batch * height * width > (1LL << 26))
        return cfail(RF_ERR_INVALID_ARG, "rf_cnn_create: bad size");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1)
        return cfail(RF_ERR_NO_DEVICE, "rf_cnn_create: no CUDA device");
    rf_cnn* c = new rf_cnn();
    c->max_batch = max_batch;
    c->H = height;
    c->W = width;
    const int spec[6][4] = {{16, 32, 1, 1}, {32, 96, 2, 1}, {96, 96, 1, 1},
                            {96, 8, 1, 0},  {128, 64, 1, 1}, {64, 8, 1, 0}};
    size_t off = 0;
    for (auto& s : spec) {
        Layer L{s[0], s[1], s[2], s[3], 0, 0};
        L.woff = off;
        off += (size_t)L.cout * 9 * L.cin;
        L.boff = off;
        off += L.cout;
        c->layers.push_back(L);
    }
    c->n_params = off;
    // He-normal initialization from a seeded generator (Box-Muller on a
    // 64-bit LCG), biases zero
    std::vector<float> hw(off, 0.0f);
    uint64_t st = seed * 6364136223846793005ULL + 1442695040888963407ULL;
    auto uni = [&]() {
        st = st * 6364136223846793005ULL + 1442695040888963407ULL;
        return ((st >> 11) + 0.5) / 9007199254740992.0;
    };
    for (const Layer& L : c->layers) {
        double sd = std::sqrt(2.0 / (9.0 * L.cin)) * (L.relu ? 1.0 : 0.1);
        for (size_t i = 0; i < (size_t)L.cout * 9 * L.cin; i++) {
            double u1 = uni(), u2 = uni();
            hw[L.woff + i] = (float)(sd * std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2));
        }
    }
    const size_t B = max_batch, P = (size_t)height * width;
    const size_t P2 = (size_t)((height + 1) / 2) * ((width + 1) / 2);
    cudaError_t e = cudaSuccess;
    auto alloc = [&](auto** p, size_t bytes) {
        if (e == cudaSuccess) e = rf::dev_malloc((void**)p, bytes);
    };
    alloc(&c->w, off * 4); alloc(&c->g, off * 4); alloc(&c->m, off * 4); alloc(&c->v, off * 4);
    alloc(&c->wb, off * 2);
    alloc(&c->wt, off * 2);
    alloc(&c->d_status, sizeof(int));
    alloc(&c->x, B * P * 16 * 2); alloc(&c->a1, B * P * 32 * 2); alloc(&c->a2, B * P2 * 96 * 2);
    alloc(&c->a3, B * P2 * 96 * 2); alloc(&c->cat, B * P * 128 * 2); alloc(&c->a4, B * P * 64 * 2);
    alloc(&c->o16, B * P2 * 8 * 4); alloc(&c->o8, B * P * 8 * 4);
    alloc(&c->g_o16, B * P2 * 8 * 4); alloc(&c->g_o8, B * P * 8 * 4);
    alloc(&c->g_a4, B * P * 64 * 4); alloc(&c->g_cat, B * P * 128 * 4);
    alloc(&c->g_a3, B * P2 * 96 * 4); alloc(&c->g_a2, B * P2 * 96 * 4);
    alloc(&c->g_a1, B * P * 32 * 4); alloc(&c->gb, B * P * 128 * 2);
    c->part_floats = (size_t)256 * 96 * 9 * 96;  // chunks x largest cout x 9 cin
    alloc(&c->part, c->part_floats * 4);
    alloc(&c->d_loss, sizeof(double));
    // inference on padded activations: on unless RF_CNN_DIRECT=0 (or rows too long)
    const char* de = std::getenv("RF_CNN_DIRECT");
    c->direct = !(de && de[0] == '0') && direct_fits(width);
    const size_t PP = (size_t)(height + 2) * (width + 2);
    const size_t PP2 = (size_t)((height + 1) / 2 + 2) * ((width + 1) / 2 + 2);
    if (c->direct) {
        alloc(&c->xp, B * PP * 16 * 2); alloc(&c->a1p, B * PP * 32 * 2);
        alloc(&c->a2p, B * PP2 * 96 * 2); alloc(&c->a3p, B * PP2 * 96 * 2);
        alloc(&c->catp, B * PP * 128 * 2); alloc(&c->a4p, B * PP * 64 * 2);
        const int nts[6] = {32, 0, 96, 16, 64, 16};  // c2 (stride 2) keeps the GEMM
        for (int li = 0; li < 6; li++)
            if (nts[li]) {
                c->nt[li] = nts[li];
                alloc(&c->wc[li], (size_t)(c->layers[li].cin / 16) * 9 * nts[li] * 16 * 2);
            }
        // cleared before the first call (forward_direct, per frame size)
        const size_t elems[6] = {B * PP * 16, B * PP * 32, B * PP2 * 96,
                                 B * PP2 * 96, B * PP * 128, B * PP * 64};
        for (int k = 0; k < 6; k++) c->pad_elems[k] = elems[k];
        if (e == cudaSuccess &&
            !(encode_positions_map(&c->map_x, c->xp, 16, B * PP) &&
              encode_positions_map(&c->map_a2, c->a2p, 96, B * PP2) &&
              encode_positions_map(&c->map_a3, c->a3p, 96, B * PP2) &&
              encode_positions_map(&c->map_cat, c->catp, 128, B * PP) &&
              encode_positions_map(&c->map_a4, c->a4p, 64, B * PP))) {
            rf_cnn_destroy(c);
            return cfail(RF_ERR_CUDA, "rf_cnn_create: tensor map encoding failed");
        }
    }
    if (e == cudaSuccess) e = cudaMemcpy(c->w, hw.data(), off * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(c->m, 0, off * 4);
    if (e == cudaSuccess) e = cudaMemset(c->v, 0, off * 4);
    if (e == cudaSuccess) e = cudaMemset(c->g, 0, off * 4);
    if (e != cudaSuccess) {
        rf_cnn_destroy(c);
        return cfail(RF_ERR_OOM, std::string("rf_cnn_create: ") + cudaGetErrorString(e));
    }
    if (cudaMemset(c->d_status, 0, sizeof(int)) != cudaSuccess) {
        rf_cnn_destroy(c);
        return cfail(RF_ERR_CUDA, "rf_cnn_create: status init");
    }
    rf_status rs = sync_bf16_weights(c);
    // the initialisation above ran on the legacy default stream; a stream
    // set later (rf_cnn_set_stream) may be non-blocking: finish it now
    if (rs == RF_OK && cudaDeviceSynchronize() != cudaSuccess)
        rs = cfail(RF_ERR_CUDA, "rf_cnn_create: initialisation");
    if (rs != RF_OK) {
        rf_cnn_destroy(c);
        return rs;
    }
    *out = c;
    return RF_OK;
}

rf_status rf_cnn_destroy(rf_cnn* c) {
    if (!c) return RF_OK;
    cudaDeviceSynchronize();
    for (void* p : {(void*)c->wt, (void*)c->d_status}) if (p) cudaFree(p);
    for (void* p : {(void*)c->w, (void*)c->g, (void*)c->m, (void*)c->v, (void*)c->wb, (void*)c->x,
                    (void*)c->a1, (void*)c->a2, (void*)c->a3, (void*)c->cat, (void*)c->a4,
                    (void*)c->o16, (void*)c->o8, (void*)c->g_o16, (void*)c->g_o8, (void*)c->g_a4,
                    (void*)c->g_cat, (void*)c->g_a3, (void*)c->g_a2, (void*)c->g_a1, (void*)c->gb,
                    (void*)c->part, (void*)c->d_loss, (void*)c->xp, (void*)c->a1p,
                    (void*)c->a2p, (void*)c->a3p, (void*)c->catp, (void*)c->a4p})
        if (p) cudaFree(p);
    for (bf16* p : c->wc)
        if (p) cudaFree(p);
    delete c;
    return RF_OK;
}

int rf_cnn_num_params(const rf_cnn* c) { return c ? (int)c->n_params : -1; }

rf_status rf_cnn_set_stream(rf_cnn* c, void* stream) {
    if (!c) return cfail(RF_ERR_INVALID_ARG, "rf_cnn_set_stream: null");
    c->stream = static_cast<cudaStream_t>(stream);
    return RF_OK;
}

rf_status rf_cnn_get_params(rf_cnn* c, float* host) {
    if (!c || !host) return cfail(RF_ERR_INVALID_ARG, "rf_cnn_get_params: null");
    CN(cudaStreamSynchronize(c->stream));
    CN(cudaMemcpy(host, c->w, c->n_params * 4, cudaMemcpyDeviceToHost));
    return RF_OK;
}

rf_status rf_cnn_set_params(rf_cnn* c, const float* host) {
    if (!c || !host) return cfail(RF_ERR_INVALID_ARG, "rf_cnn_set_params: null");
    // on the network's stream, ahead of the conversion kernels that read it
    CN(cudaMemcpyAsync(c->w, host, c->n_params * 4, cudaMemcpyHostToDevice, c->stream));
    return sync_bf16_weights(c);
}

rf_status rf_cnn_get_grads(rf_cnn* c, float* host) {
    if (!c || !host) return cfail(RF_ERR_INVALID_ARG, "rf_cnn_get_grads: null");
    CN(cudaStreamSynchronize(c->stream));
    CN(cudaMemcpy(host, c->g, c->n_params * 4, cudaMemcpyDeviceToHost));
    return RF_OK;
}

static rf_status check_batch(rf_cnn* c, int B, int H, int W) {
    if (B < 1 || B > c->max_batch || H > c->H || W > c->W || H < 2 || W < 2)
        return cfail(RF_ERR_INVALID_ARG, "rf_cnn: batch or size beyond the allocation");
    return RF_OK;
}

rf_status rf_cnn_forward(rf_cnn* c, const float* input, int B, int H, int W, float* out16,
                         float* out8) {
    rf::NvtxRange range("rf_cnn_forward");
    if (!c || !input) return cfail(RF_ERR_INVALID_ARG, "rf_cnn_forward: null");
    rf_status rs = check_batch(c, B, H, W);
    if (rs == RF_OK)
        rs = c->direct ? forward_direct(c, input, B, H, W) : forward(c, input, B, H, W);
    if (rs != RF_OK) return rs;
    int H2 = (H + 1) / 2, W2 = (W + 1) / 2;
    if (out16)
        CN(cudaMemcpyAsync(out16, c->o16, (size_t)B * H2 * W2 * 8 * 4, cudaMemcpyDeviceToDevice,
                           c->stream));
    if (out8)
        CN(cudaMemcpyAsync(out8, c->o8, (size_t)B * H * W * 8 * 4, cudaMemcpyDeviceToDevice,
                           c->stream));
    return RF_OK;
}

rf_status rf_cnn_backward(rf_cnn* c, const float* input, const float* tgt16, const float* mask16,
                          const float* tgt8, const float* mask8, int B, int H, int W,
                          const float* weights, double* loss) {
    rf::NvtxRange range("rf_cnn_backward");
    if (!c || !input || !tgt16 || !mask16 || !tgt8 || !mask8 || !weights)
        return cfail(RF_ERR_INVALID_ARG, "rf_cnn_backward: null");
    rf_status rs = check_batch(c, B, H, W);
    if (rs == RF_OK) rs = forward(c, input, B, H, W);
    if (rs != RF_OK) return rs;
    int H2 = (H + 1) / 2, W2 = (W + 1) / 2;
    int P8 = B * H * W, P16 = B * H2 * W2;
    CN(cudaMemsetAsync(c->d_loss, 0, sizeof(double), c->stream));
    k_l1_loss<<<blocks_for(P16), 256, 0, c->stream>>>(c->o16, tgt16, mask16, P16, 8, weights[0],
                                                      weights[1], weights[2], 1.0f / P16,
                                                      c->g_o16, c->d_loss);
    k_l1_loss<<<blocks_for(P8), 256, 0, c->stream>>>(c->o8, tgt8, mask8, P8, 8, weights[0],
                                                     weights[1], weights[2], 1.0f / P8, c->g_o8,
                                                     c->d_loss);
    c->launches += 2;
    rs = backward(c, B, H, W);
    if (rs != RF_OK) return rs;
    if (loss) {
        CN(cudaMemcpyAsync(loss, c->d_loss, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        CN(cudaStreamSynchronize(c->stream));
    }
    return RF_OK;
}

rf_status rf_cnn_adam_step(rf_cnn* c, float lr, float beta1, float beta2, float eps) {
    rf::NvtxRange range("rf_cnn_adam_step");
    if (!c) return cfail(RF_ERR_INVALID_ARG, "rf_cnn_adam_step: null");
    c->step++;
    float c1 = 1.0f - std::pow(beta1, (float)c->step);
    float c2 = 1.0f - std::pow(beta2, (float)c->step);
    k_adam<<<blocks_for(c->n_params), 256, 0, c->stream>>>(c->w, c->g, c->m, c->v, c->n_params, lr,
                                                           beta1, beta2, eps, c1, c2);
    c->launches++;
    CN(cudaGetLastError());
    return sync_bf16_weights(c);
}

uint64_t rf_cnn_kernel_launches(const rf_cnn* c) { return c ? c->launches : 0; }

rf_status rf_cnn_status(rf_cnn* c, int* gave_up) {
    if (!c || !gave_up) return cfail(RF_ERR_INVALID_ARG, "rf_cnn_status: null");
    int v = 0;
    CN(cudaMemcpyAsync(&v, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CN(cudaStreamSynchronize(c->stream));
    if (v) CN(cudaMemsetAsync(c->d_status, 0, sizeof(int), c->stream));
    *gave_up = v;
    return RF_OK;
}

rf_status rf_cnn_set_test_wait_limit(rf_cnn* c, int polls) {
    if (!c) return cfail(RF_ERR_INVALID_ARG, "rf_cnn_set_test_wait_limit: null");
    c->test_first_wait_polls = polls < 0 ? -1 : polls;
    return RF_OK;
}

}  // extern "C"
