// Host side of the C ABI (include/reconflow_gb300.h): buffer management,
// the coarse-to-fine schedule of ReconFlow::solveReconFlow
// (Reconflow.cu:147-466) and CudaFlow::_solveOpticalFlow (Cudaflow.cu:403-621),
// and CUDA-graph capture of the whole schedule.
//
// The schedule is recorded once per handle into a CUDA graph and replayed by
// every solve; the per-solve camera constants live in a small device block
// that the kernels read, so one graph serves every pose.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/reconflow_gb300.h"
#include "rf_alloc.h"
#include "rf_nvtx.h"
#include "rf_kernels.cuh"

using namespace rf;

namespace rf {
int set_last_error(int st, const char* msg);
}

namespace {

thread_local std::string g_err;

rf_status fail(rf_status st, const std::string& msg) {
    g_err = msg;
    return st;
}

}  // namespace

int rf::set_last_error(int st, const char* msg) {
    g_err = msg;
    return st;
}

namespace {

rf_status cuda_fail(cudaError_t e, const char* what) {
    g_err = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? RF_ERR_OOM : RF_ERR_CUDA;
}

#define RF_CUDA(call)                                   \
    do {                                                \
        cudaError_t e__ = (call);                       \
        if (e__ != cudaSuccess) return cuda_fail(e__, #call); \
    } while (0)

int align_up(int n, int m) {
    int mod = n % m;
    return mod ? n + m - mod : n;
}

}  // namespace

struct rf_handle {
    rf_params p{};
    int L = 0;
    std::vector<int> W, H, S;
    int stride = 0, height = 0;
    size_t plane = 0;  // floats per plane: stride * (height + 1)

    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    float* pool = nullptr;
    size_t pool_floats = 0;
    size_t pool_used = 0;

    std::vector<float*> I0, I1;
    float *i1w = nullptr, *Ix = nullptr, *Iy = nullptr, *Iz = nullptr;
    float *duhat = nullptr, *dvhat = nullptr;
    float *pu1 = nullptr, *pu2 = nullptr, *pv1 = nullptr, *pv2 = nullptr;
    float *X = nullptr, *Y = nullptr, *Z = nullptr, *X1 = nullptr, *Y1 = nullptr, *Z1 = nullptr;
    float *ufn = nullptr, *vfn = nullptr, *mask = nullptr;
    float *ufn_l = nullptr, *vfn_l = nullptr, *mask_l = nullptr;
    float* scratch = nullptr;      // inverse depth / colour output
    std::vector<float*> spare;     // ping-pong planes for fields that change buffers
    void* staging[2] = {nullptr, nullptr};
    size_t staging_bytes = 0;

    LevelConsts* d_consts = nullptr;
    LevelConsts* h_consts = nullptr;  // pinned

    double K0[9], K1[9];
    bool cams_set = false, images_set = false, prior_set = false;

    cudaGraphExec_t graph = nullptr;
    int graph_kind = -1;  // 0 = recon, 1 = plain
    uint64_t graph_nodes = 0;
    uint64_t launches = 0;
    uint64_t enqueue_launches = 0;

    // result planes after the last solve, and where the carried state ended up
    float *res_u = nullptr, *res_v = nullptr;
    float *st_uproj = nullptr, *st_vproj = nullptr, *st_sku = nullptr, *st_skv = nullptr;
    float *st_uc = nullptr, *st_vc = nullptr;
    // warm start (rf_solve_warm): staging planes and the schedule's start
    float* warm[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    int warm_level = -1, warm_warps = 0, warm_iters = 0;
    long long graph_key[4] = {-1, -1, -1, -1};  // warm level, warps, iterations; cluster threshold
    // tile shape of the inner-iteration kernels at each level (rf_set_tiles)
    std::vector<int> tile_w, tile_h;
    // energy reduction buffers and the pose of the last solve
    double* d_energy = nullptr;  // [0] = result, [1..1024] = block partials
    double last_R1[9], last_t1[3];
    bool solved = false;

    float* alloc_plane() {
        if (pool_used + plane > pool_floats) return nullptr;
        float* p = pool + pool_used;
        pool_used += (plane + 63) / 64 * 64;
        return p;
    }
};

namespace {

bool valid_method(int m) {
    return m == RF_METHOD_TVL1 || m == RF_METHODR_TVL1_MS || m == RF_METHODR_TVL1_MS_FN ||
           m == RF_METHODR_TVL1_MS_FNSPARSE;
}

int prior_kind(int m) {
    return m == RF_METHODR_TVL1_MS_FN ? 1 : (m == RF_METHODR_TVL1_MS_FNSPARSE ? 2 : 0);
}

size_t input_elem_bytes(int t) {
    switch (t) {
        case RF_INPUT_RGB8: return 3;
        case RF_INPUT_U8: return 1;
        case RF_INPUT_U16: return 2;
        default: return 4;
    }
}

Weights make_weights(const rf_params& p);

}  // namespace

Weights rf::solver_weights(const rf_params* p) { return make_weights(*p); }

namespace {

Weights make_weights(const rf_params& p) {
    Weights w{};
    w.lambda = p.lambda;
    w.alpha_tv = p.alpha_tv;
    w.alpha_proj = p.alpha_proj;
    w.alpha_fn = p.alpha_fn;
    w.A = p.alpha_tv + p.alpha_proj;
    w.lambdaf = p.lambdaf;
    w.lambdams = p.lambdams;
    w.proj_den = p.lambdaf + p.alpha_proj;
    w.theta = p.theta;
    if (p.method == RF_METHOD_TVL1) {
        w.fac = p.tau / p.theta;
    } else {
        float thetaTv = 1.0f / p.alpha_tv;  // Reconflow.cu:32
        w.fac = p.tau / thetaTv;
    }
    return w;
}

void level_consts(const rf_handle* h, const double* R0, const double* t0, const double* R1,
                  const double* t1, LevelConsts* out) {
    rf::camera_level_consts(h->K0, h->K1, h->L, h->p.scale, h->p.fix_quirks, R0, t0, R1, t1, out);
}

}  // namespace

// Reconflow.cu:98-110 (K pyramid) and :225-226 (P = K [R | t]), in double.
void rf::camera_level_consts(const double* K0in, const double* K1in, int L, float scale,
                             int fix_quirks, const double* R0, const double* t0, const double* R1,
                             const double* t1, LevelConsts* out) {
    double K0[9], K1[9];
    std::memcpy(K0, K0in, sizeof K0);
    std::memcpy(K1, K1in, sizeof K1);
    const bool fix_k = (fix_quirks & RF_FIX_K_PYRAMID) != 0;
    for (int l = 0; l < L; l++) {
        if (l > 0) {
            double a[9] = {0}, b[9] = {0};
            const double f = scale;
            a[0] = K0[0] / f; a[2] = K0[2] / f; a[4] = K0[4] / f; a[5] = K0[5] / f;
            b[0] = K1[0] / f; b[2] = K1[2] / f; b[4] = K1[4] / f; b[5] = K1[5] / f;
            if (fix_k) a[8] = b[8] = 1.0;
            std::memcpy(K0, a, sizeof a);
            std::memcpy(K1, b, sizeof b);
        }
        double Rt0[12], Rt1[12];
        for (int r = 0; r < 3; r++) {
            for (int c = 0; c < 3; c++) {
                Rt0[r * 4 + c] = R0[r * 3 + c];
                Rt1[r * 4 + c] = R1[r * 3 + c];
            }
            Rt0[r * 4 + 3] = t0[r];
            Rt1[r * 4 + 3] = t1[r];
        }
        LevelConsts& c = out[l];
        for (int r = 0; r < 3; r++)
            for (int k4 = 0; k4 < 4; k4++) {
                double a = 0, b = 0;
                for (int k = 0; k < 3; k++) {
                    a += K0[r * 3 + k] * Rt0[k * 4 + k4];
                    b += K1[r * 3 + k] * Rt1[k * 4 + k4];
                }
                c.P[r * 4 + k4] = (float)a;
                c.Q[r * 4 + k4] = (float)b;
            }
        for (int i = 0; i < 9; i++) c.R1[i] = (float)R1[i];
        for (int i = 0; i < 3; i++) c.t1[i] = (float)t1[i];
        c.focal = (float)K1[0];
        c.cx = (float)K1[2];
        c.cy = (float)K1[5];
        c.pad = 0.0f;
    }
}

namespace {

// Levels of at most this many pixels run a warp's inner iterations as one
// thread-block-cluster launch (launch_recon_cluster); RF_CLUSTER_PX sets it.
// Off by default: on GB300 the graph of two launches per iteration was
// faster at every level size tried (the 16 SMs of one cluster issue too
// slowly for a level of thousands of pixels, and a cluster barrier costs
// more than a launch boundary inside a graph for the smallest levels).
std::atomic<long long> g_cluster_px{-1};

long long cluster_max_px() {
    long long v = g_cluster_px.load();
    if (v < 0) {
        const char* e = std::getenv("RF_CLUSTER_PX");
        v = e ? std::atoll(e) : 0;
        if (v < 0) v = 0;
        long long expect = -1;
        g_cluster_px.compare_exchange_strong(expect, v);
        v = g_cluster_px.load();
    }
    return v;
}

bool use_cluster_at(const rf_handle*, LevelDims d) {
    const long long m = cluster_max_px();
    return m > 0 && (long long)d.w * d.h <= m && cluster_supported();
}

#define RF_LAUNCH(expr)                                                               \
    do {                                                                              \
        if ((expr) != 0)                                                              \
            return cuda_fail(rf::last_launch_error(), "kernel launch " #expr);        \
        h->enqueue_launches++;                                                        \
    } while (0)

// Shared front of both schedules: input conversion and the image pyramid
// (Reconflow.cu:162-206, Cudaflow.cu:405-464).
rf_status enqueue_pyramid(rf_handle* h) {
    cudaStream_t st = h->stream;
    const rf_params& p = h->p;
    if (p.input_type != RF_INPUT_F32) {
        RF_LAUNCH(launch_convert(h->staging[0], p.input_type, p.width, p.height, h->stride,
                                 h->I0[0], h->stride, st));
        RF_LAUNCH(launch_convert(h->staging[1], p.input_type, p.width, p.height, h->stride,
                                 h->I1[0], h->stride, st));
    }
    for (int l = 1; l < h->L; l++) {
        LevelDims f{h->W[l - 1], h->H[l - 1], h->S[l - 1]}, c{h->W[l], h->H[l], h->S[l]};
        RF_LAUNCH(launch_downscale2(h->I0[l - 1], h->I1[l - 1], f, c, h->I0[l], h->I1[l], st));
    }
    return RF_OK;
}

// ReconFlow::solveReconFlow (Reconflow.cu:147-466) for methods 14 / 17 / 20.
// Copy the warm-start planes (level `lvl`) into the solver's role buffers.
rf_status copy_warm(rf_handle* h, int lvl, float* const* dst, int n) {
    const size_t sp = h->S[lvl] * sizeof(float);
    for (int k = 0; k < n; k++)
        RF_CUDA(cudaMemcpy2DAsync(dst[k], sp, h->warm[k < 2 ? k : k], sp,
                                  h->W[lvl] * sizeof(float), h->H[lvl], cudaMemcpyDeviceToDevice,
                                  h->stream));
    return RF_OK;
}

rf_status enqueue_recon(rf_handle* h, float** res_u, float** res_v, bool warm = false) {
    cudaStream_t st = h->stream;
    const rf_params& p = h->p;
    const int top = warm ? h->warm_level : h->L - 1;
    const int n_warps = warm ? h->warm_warps : p.n_warp_iters;
    const int n_iters = warm ? h->warm_iters : p.n_solver_iters;
    const Weights wt = make_weights(p);
    const int prior = prior_kind(p.method);
    const size_t plane_bytes = h->plane * sizeof(float);

    // field roles (pointer swaps replace the reference's Swap calls)
    float *u = h->spare[0], *v = h->spare[1], *uc = h->spare[2], *vc = h->spare[3];
    float *uproj = h->spare[4], *vproj = h->spare[5], *sku = h->spare[6], *skv = h->spare[7];
    float *tu = h->spare[8], *tv = h->spare[9];
    std::vector<float*> free_planes(h->spare.begin() + 10, h->spare.end());

    rf_status rs = enqueue_pyramid(h);
    if (rs != RF_OK) return rs;
    // Reconflow.cu:209-220
    for (float* b : {u, v, uproj, vproj, uc, vc, sku, skv, h->X, h->Y, h->Z})
        RF_CUDA(cudaMemsetAsync(b, 0, plane_bytes, st));
    bool uc_in_buffer = true;
    if (warm) {
        // u, v and the points from the staging planes; uproj = u; uc from the points
        float* dst[5] = {u, v, h->X, h->Y, h->Z};
        rf_status ws = copy_warm(h, top, dst, 5);
        if (ws != RF_OK) return ws;
        float* dp[2] = {uproj, vproj};
        ws = copy_warm(h, top, dp, 2);
        if (ws != RF_OK) return ws;
        uc_in_buffer = false;
    }

    for (int level = top; level >= 0; level--) {
        NvtxRange level_range("level %d", level);
        LevelDims d{h->W[level], h->H[level], h->S[level]};
        const LevelConsts* lc = h->d_consts + level;
        ReconFields f{};
        f.extent = (long long)h->plane;
        if (prior) {
            // Reconflow.cu:232-241: prior resampled from level 0 at every level
            LevelDims d0{h->W[0], h->H[0], h->S[0]};
            float sc = (float)h->W[level] / (float)h->W[0];
            RF_LAUNCH(launch_downscale(h->ufn, d0, d, sc, true, h->ufn_l, st));
            RF_LAUNCH(launch_downscale(h->vfn, d0, d, sc, true, h->vfn_l, st));
            RF_LAUNCH(launch_downscale(h->mask, d0, d, 1.0f, false, h->mask_l, st));
        }
        for (int warp = 0; warp < n_warps; warp++) {
            NvtxRange warp_range("level %d warp %d", level, warp);
            RF_LAUNCH(launch_warp_deriv(h->I0[level], h->I1[level], u, v, d, h->Ix, h->Iy,
                                        h->Iz, st));
            f.u = u; f.v = v;
            f.duhat = h->duhat; f.dvhat = h->dvhat;
            f.pu1 = h->pu1; f.pu2 = h->pu2; f.pv1 = h->pv1; f.pv2 = h->pv2;
            f.uproj = uproj; f.vproj = vproj; f.sku = sku; f.skv = skv;
            f.Ix = h->Ix; f.Iy = h->Iy; f.Iz = h->Iz;
            f.X = h->X; f.Y = h->Y; f.Z = h->Z; f.X1 = h->X1; f.Y1 = h->Y1; f.Z1 = h->Z1;
            f.uc = uc; f.vc = vc;
            f.ufn = h->ufn_l; f.vfn = h->vfn_l; f.mask = h->mask_l;
            if (n_iters > 0 && use_cluster_at(h, d)) {
                // a small level: all of the warp's iterations in one cluster launch
                RF_LAUNCH(launch_recon_cluster(f, lc, wt, d, n_iters, uc_in_buffer, prior, st));
                uc_in_buffer = false;
            }
            for (int iter = 0; iter < n_iters && !use_cluster_at(h, d); iter++) {
                const dim3 tile(h->tile_w[level], h->tile_h[level]);
                RF_LAUNCH(launch_recon_a(f, lc, wt, d, iter == 0, uc_in_buffer, prior, st, tile));
                RF_LAUNCH(launch_recon_b(f, wt, d, iter == 0, st, tile));
                uc_in_buffer = false;
            }
            if (n_iters == 0) {
                // the reference's memsets leave duhat = 0 when no iteration runs
                RF_CUDA(cudaMemsetAsync(h->duhat, 0, plane_bytes, st));
                RF_CUDA(cudaMemsetAsync(h->dvhat, 0, plane_bytes, st));
            }
            // Reconflow.cu:410-420: median of duhat, u += it, median of u
            RF_LAUNCH(launch_median_add(h->duhat, h->dvhat, u, v, tu, tv, d, st));
            RF_LAUNCH(launch_median5(tu, tv, u, v, d, st));
        }
        if (level > 0) {
            LevelDims fd{h->W[level - 1], h->H[level - 1], h->S[level - 1]};
            if (!uc_in_buffer) RF_LAUNCH(launch_solve_uc(h->X, h->Y, h->Z, lc, d, uc, vc, st));
            // Reconflow.cu:424-458: u, v, uc, vc, uproj, vproj, sku, skv scaled by fScale
            float* src[8] = {u, v, uc, vc, uproj, vproj, sku, skv};
            float* dst[8];
            float sc[8];
            for (int i = 0; i < 8; i++) {
                dst[i] = free_planes[i];
                sc[i] = p.scale;
            }
            RF_LAUNCH(launch_upscale_fields(8, src, dst, sc, d, fd, st));
            for (int i = 0; i < 8; i++) free_planes[i] = src[i];
            u = dst[0]; v = dst[1]; uc = dst[2]; vc = dst[3];
            uproj = dst[4]; vproj = dst[5]; sku = dst[6]; skv = dst[7];
            uc_in_buffer = true;
            if (p.fix_quirks & RF_FIX_XYZ_UPSCALE) {
                const float* xs[3] = {h->X, h->Y, h->Z};
                float* xd[3] = {h->X1, h->Y1, h->Z1};
                float one[3] = {1.0f, 1.0f, 1.0f};
                RF_LAUNCH(launch_upscale_fields(3, xs, xd, one, d, fd, st));
                float* xt[3] = {h->X, h->Y, h->Z};
                for (int c = 0; c < 3; c++)
                    RF_CUDA(cudaMemcpy2DAsync(xt[c], fd.s * sizeof(float), xd[c],
                                              fd.s * sizeof(float), fd.w * sizeof(float), fd.h,
                                              cudaMemcpyDeviceToDevice, st));
            }
        }
    }
    *res_u = u;
    *res_v = v;
    h->st_uproj = uproj; h->st_vproj = vproj; h->st_sku = sku; h->st_skv = skv;
    h->st_uc = uc; h->st_vc = vc;
    return RF_OK;
}


// CudaFlow::_solveOpticalFlow (Cudaflow.cu:403-621), METHOD_TVL1.
rf_status enqueue_plain(rf_handle* h, float** res_u, float** res_v, bool warm = false) {
    cudaStream_t st = h->stream;
    const rf_params& p = h->p;
    const Weights wt = make_weights(p);
    const size_t plane_bytes = h->plane * sizeof(float);
    const int top = warm ? h->warm_level : h->L - 1;
    const int n_warps = warm ? h->warm_warps : p.n_warp_iters;
    const int n_iters = warm ? h->warm_iters : p.n_solver_iters;
    float *u = h->spare[0], *v = h->spare[1];
    float *us = h->spare[2], *vs = h->spare[3];
    rf_status rs = enqueue_pyramid(h);
    if (rs != RF_OK) return rs;
    RF_CUDA(cudaMemsetAsync(u, 0, plane_bytes, st));
    RF_CUDA(cudaMemsetAsync(v, 0, plane_bytes, st));
    if (warm) {
        float* dst[2] = {u, v};
        rf_status ws = copy_warm(h, top, dst, 2);
        if (ws != RF_OK) return ws;
    }
    for (int level = top; level >= 0; level--) {
        NvtxRange level_range("level %d", level);
        LevelDims d{h->W[level], h->H[level], h->S[level]};
        for (int warp = 0; warp < n_warps; warp++) {
            NvtxRange warp_range("level %d warp %d", level, warp);
            RF_LAUNCH(launch_warp_deriv(h->I0[level], h->I1[level], u, v, d, h->Ix, h->Iy,
                                        h->Iz, st));
            for (int iter = 0; iter < n_iters; iter++) {
                RF_LAUNCH(launch_plain_data(h->duhat, h->dvhat, h->pu1, h->pu2, h->pv1, h->pv2,
                                            h->Ix, h->Iy, h->Iz, wt, d, iter == 0, st));
                RF_LAUNCH(launch_plain_tv(h->duhat, h->dvhat, h->pu1, h->pu2, h->pv1, h->pv2, wt,
                                          d, iter == 0, st));
            }
            if (n_iters == 0) {
                RF_CUDA(cudaMemsetAsync(h->duhat, 0, plane_bytes, st));
                RF_CUDA(cudaMemsetAsync(h->dvhat, 0, plane_bytes, st));
            }
            // Cudaflow.cu:580-587: median of duhat, u += it (no median of u)
            RF_LAUNCH(launch_median_add(h->duhat, h->dvhat, u, v, u, v, d, st));
        }
        if (level > 0) {
            LevelDims fd{h->W[level - 1], h->H[level - 1], h->S[level - 1]};
            const float* src[2] = {u, v};
            float* dst[2] = {us, vs};
            float sc[2] = {p.scale, p.scale};
            RF_LAUNCH(launch_upscale_fields(2, src, dst, sc, d, fd, st));
            std::swap(u, us);
            std::swap(v, vs);
        }
    }
    *res_u = u;
    *res_v = v;
    return RF_OK;
}

bool use_graphs() {
    const char* e = std::getenv("RF_USE_GRAPHS");
    return !(e && e[0] == '0');
}

// Record the schedule into a graph on first use, then replay it.
rf_status run_schedule(rf_handle* h, int kind) {
    NvtxRange range(kind == 1 || kind == 3 ? "rf_solve_flow" : "rf_solve");
    auto enqueue = [&](float** ru, float** rv) {
        if (kind == 1) return enqueue_plain(h, ru, rv);
        if (kind == 2) return enqueue_recon(h, ru, rv, true);
        if (kind == 3) return enqueue_plain(h, ru, rv, true);
        return enqueue_recon(h, ru, rv);
    };
    // a captured schedule is reused while nothing it was captured with has
    // changed (rf_set_cluster_pixels changes which levels take the cluster
    // launch)
    const long long key[4] = {kind >= 2 ? h->warm_level : -1, kind >= 2 ? h->warm_warps : -1,
                              kind >= 2 ? h->warm_iters : -1, cluster_max_px()};
    if (h->graph && (key[0] != h->graph_key[0] || key[1] != h->graph_key[1] ||
                     key[2] != h->graph_key[2] || key[3] != h->graph_key[3])) {
        cudaGraphExecDestroy(h->graph);
        h->graph = nullptr;
    }
    std::memcpy(h->graph_key, key, sizeof key);
    if (!use_graphs()) {
        h->enqueue_launches = 0;
        rf_status rs = enqueue(&h->res_u, &h->res_v);
        h->launches += h->enqueue_launches;
        return rs;
    }
    if (h->graph && h->graph_kind != kind) {
        cudaGraphExecDestroy(h->graph);
        h->graph = nullptr;
    }
    if (!h->graph) {
        cudaGraph_t g = nullptr;
        RF_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        h->enqueue_launches = 0;
        rf_status rs = enqueue(&h->res_u, &h->res_v);
        cudaError_t ce = cudaStreamEndCapture(h->stream, &g);
        if (rs != RF_OK) {
            if (g) cudaGraphDestroy(g);
            return rs;
        }
        if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
        cudaError_t ie = cudaGraphInstantiate(&h->graph, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) {
            h->graph = nullptr;
            return cuda_fail(ie, "cudaGraphInstantiate");
        }
        h->graph_kind = kind;
        h->graph_nodes = h->enqueue_launches;
    }
    RF_CUDA(cudaGraphLaunch(h->graph, h->stream));
    h->launches += h->graph_nodes;
    return RF_OK;
}

}  // namespace

extern "C" {

rf_status rf_params_default(rf_params* p, int method) {
    if (!p) return fail(RF_ERR_INVALID_ARG, "rf_params_default: null params");
    std::memset(p, 0, sizeof *p);
    p->channels = 1;
    p->input_type = RF_INPUT_F32;
    p->scale = 2.0f;
    p->method = method;
    p->stride_alignment = 32;
    p->block_width = 32;
    p->block_height = 12;
    if (method == RF_METHOD_TVL1) {
        // Cudaflow.cu:16-18
        p->lambda = 100.0f; p->lambdagrad = 400.0f; p->theta = 0.33f; p->tau = 0.25f;
        p->n_warp_iters = 1; p->n_solver_iters = 100;
    } else {
        // Reconflow.cu:15-18
        p->lambda = 100.0f; p->lambdagrad = 400.0f; p->lambdaf = 100.0f; p->lambdams = 100.0f;
        p->alpha_tv = 3.0f; p->alpha_proj = 1.0f; p->alpha_fn = 0.5f; p->tau = 0.25f;
        p->theta = 1.0f / 3.0f; p->n_warp_iters = 1; p->n_solver_iters = 100;
    }
    return RF_OK;
}

rf_status rf_create(const rf_params* p, rf_handle** out) {
    if (!p || !out) return fail(RF_ERR_INVALID_ARG, "rf_create: null argument");
    *out = nullptr;
    if (!valid_method(p->method))
        return fail(RF_ERR_UNSUPPORTED, "rf_create: method " + std::to_string(p->method) +
                                            " is not implemented (0, 14, 17, 20 are)");
    if (p->input_type < 0 || p->input_type > 3)
        return fail(RF_ERR_UNSUPPORTED, "rf_create: unknown input type");
    if (p->width < 1 || p->height < 1 || p->n_levels < 1 || p->n_levels > 16)
        return fail(RF_ERR_INVALID_ARG, "rf_create: width/height/n_levels out of range");
    if (!(p->scale > 1.0f) || p->stride_alignment < 1 || p->n_warp_iters < 0 ||
        p->n_solver_iters < 0)
        return fail(RF_ERR_INVALID_ARG, "rf_create: scale/stride_alignment/iteration counts");
    if ((long long)p->width * p->height > (1LL << 28))
        return fail(RF_ERR_INVALID_ARG, "rf_create: image too large");
    if (p->method == RF_METHOD_TVL1 ? !(p->theta != 0.0f) : !(p->alpha_tv != 0.0f))
        return fail(RF_ERR_INVALID_ARG, "rf_create: theta / alpha_tv must be non-zero");
    rf_handle* h = new rf_handle();
    h->p = *p;
    h->L = p->n_levels;
    h->W.resize(h->L); h->H.resize(h->L); h->S.resize(h->L);
    h->tile_w.assign(h->L, 32);
    h->tile_h.assign(h->L, 8);
    // Cudaflow.cu:146-171
    int nh = p->height, nw = p->width, ns = align_up(p->width, p->stride_alignment);
    for (int l = 0; l < h->L; l++) {
        h->W[l] = nw; h->H[l] = nh; h->S[l] = ns;
        nh = (int)((float)nh / p->scale);
        nw = (int)((float)nw / p->scale);
        ns = align_up(nw, p->stride_alignment);
    }
    for (int l = 0; l < h->L; l++)
        if (h->W[l] < 1 || h->H[l] < 1) {
            delete h;
            return fail(RF_ERR_INVALID_ARG, "rf_create: too many levels for the image size");
        }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        delete h;
        return fail(RF_ERR_NO_DEVICE, "rf_create: no CUDA device");
    }
    h->stride = h->S[0];
    h->height = h->H[0];
    h->plane = (size_t)h->stride * (h->height + 1);

    const bool recon = p->method != RF_METHOD_TVL1;
    const int prior = prior_kind(p->method);
    int n_planes = 2 * h->L + 4 /*i1w, Ix, Iy, Iz*/ + 6 /*duhat, p*/ + 1 /*scratch*/ +
                   5 /*warm-start staging*/;
    int n_spare = recon ? 31 : 4;
    if (recon) n_planes += 6; /* X, X1 */
    if (prior) n_planes += 6;
    n_planes += n_spare;
    const size_t plane_alloc = (h->plane + 63) / 64 * 64;
    h->pool_floats = plane_alloc * (size_t)n_planes + plane_alloc * 3 /* colour output */;
    cudaError_t e = rf::dev_malloc((void**)&h->pool, h->pool_floats * sizeof(float));
    if (e != cudaSuccess) {
        delete h;
        return fail(RF_ERR_OOM, std::string("rf_create: device allocation: ") + cudaGetErrorString(e));
    }
    for (int l = 0; l < h->L; l++) {
        h->I0.push_back(h->alloc_plane());
        h->I1.push_back(h->alloc_plane());
    }
    h->i1w = h->alloc_plane(); h->Ix = h->alloc_plane(); h->Iy = h->alloc_plane(); h->Iz = h->alloc_plane();
    h->duhat = h->alloc_plane(); h->dvhat = h->alloc_plane();
    h->pu1 = h->alloc_plane(); h->pu2 = h->alloc_plane(); h->pv1 = h->alloc_plane(); h->pv2 = h->alloc_plane();
    if (recon) {
        h->X = h->alloc_plane(); h->Y = h->alloc_plane(); h->Z = h->alloc_plane();
        h->X1 = h->alloc_plane(); h->Y1 = h->alloc_plane(); h->Z1 = h->alloc_plane();
    }
    if (prior) {
        h->ufn = h->alloc_plane(); h->vfn = h->alloc_plane(); h->mask = h->alloc_plane();
        h->ufn_l = h->alloc_plane(); h->vfn_l = h->alloc_plane(); h->mask_l = h->alloc_plane();
    }
    for (int i = 0; i < n_spare; i++) h->spare.push_back(h->alloc_plane());
    h->scratch = h->alloc_plane();
    for (int i = 0; i < 5; i++) h->warm[i] = h->alloc_plane();
    // zero everything once: guard rows and never-written padding read as 0
    e = cudaMemset(h->pool, 0, h->pool_floats * sizeof(float));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = rf::dev_malloc((void**)&h->d_consts, sizeof(LevelConsts) * h->L);
    if (e == cudaSuccess) e = rf::dev_malloc((void**)&h->d_energy, 1025 * sizeof(double));
    if (e == cudaSuccess) e = rf::host_malloc((void**)&h->h_consts, sizeof(LevelConsts) * h->L);
    if (e == cudaSuccess && p->input_type != RF_INPUT_F32) {
        h->staging_bytes = (size_t)h->stride * h->height * input_elem_bytes(p->input_type);
        e = rf::dev_malloc((void**)&h->staging[0], h->staging_bytes);
        if (e == cudaSuccess) e = rf::dev_malloc((void**)&h->staging[1], h->staging_bytes);
    }
    if (e != cudaSuccess) {
        rf_destroy(h);
        return fail(RF_ERR_OOM, std::string("rf_create: ") + cudaGetErrorString(e));
    }
    h->stream = h->own_stream;
    if (prior) {
        // the mask defaults to ones (Cudaflow.cu:327-331)
        std::vector<float> ones((size_t)h->stride * h->height, 1.0f);
        e = cudaMemcpy(h->mask, ones.data(), ones.size() * sizeof(float), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            rf_destroy(h);
            return cuda_fail(e, "rf_create: mask init");
        }
    }
    // the clearing memset and copies above ran on the legacy default stream,
    // which the handle's non-blocking stream does not wait for: finish them
    // before any solve can read the pool
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        rf_destroy(h);
        return cuda_fail(e, "rf_create: initialisation");
    }
    *out = h;
    return RF_OK;
}

rf_status rf_destroy(rf_handle* h) {
    if (!h) return RF_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->graph) cudaGraphExecDestroy(h->graph);
    if (h->pool) cudaFree(h->pool);
    if (h->d_consts) cudaFree(h->d_consts);
    if (h->d_energy) cudaFree(h->d_energy);
    if (h->h_consts) cudaFreeHost(h->h_consts);
    for (void* s : h->staging)
        if (s) cudaFree(s);
    if (h->own_stream) cudaStreamDestroy(h->own_stream);
    delete h;
    return RF_OK;
}

int rf_stride(const rf_handle* h) { return h ? h->stride : -1; }

rf_status rf_pyramid_dims(const rf_handle* h, int* W, int* H, int* S) {
    if (!h || !W || !H || !S) return fail(RF_ERR_INVALID_ARG, "rf_pyramid_dims: null argument");
    for (int l = 0; l < h->L; l++) {
        W[l] = h->W[l];
        H[l] = h->H[l];
        S[l] = h->S[l];
    }
    return RF_OK;
}

rf_status rf_set_cameras(rf_handle* h, const double K0[9], const double K1[9]) {
    if (!h || !K0 || !K1) return fail(RF_ERR_INVALID_ARG, "rf_set_cameras: null argument");
    std::memcpy(h->K0, K0, sizeof h->K0);
    std::memcpy(h->K1, K1, sizeof h->K1);
    h->cams_set = true;
    return RF_OK;
}

static rf_status upload(rf_handle* h, const void* i0, const void* i1, int pitch, bool device) {
    if (!h || !i0 || !i1) return fail(RF_ERR_INVALID_ARG, "rf_upload_images: null argument");
    const rf_params& p = h->p;
    if (pitch < p.width) return fail(RF_ERR_INVALID_ARG, "rf_upload_images: pitch < width");
    const size_t eb = input_elem_bytes(p.input_type);
    const cudaMemcpyKind kind = device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    for (int k = 0; k < 2; k++) {
        const void* src = k == 0 ? i0 : i1;
        void* dst = p.input_type == RF_INPUT_F32 ? (void*)(k == 0 ? h->I0[0] : h->I1[0])
                                                 : h->staging[k];
        RF_CUDA(cudaMemcpy2DAsync(dst, h->stride * eb, src, (size_t)pitch * eb, p.width * eb,
                                  p.height, kind, h->stream));
    }
    h->images_set = true;
    return RF_OK;
}

rf_status rf_upload_images(rf_handle* h, const void* i0, const void* i1, int pitch) {
    return upload(h, i0, i1, pitch, false);
}

rf_status rf_upload_images_device(rf_handle* h, const void* i0, const void* i1, int pitch) {
    return upload(h, i0, i1, pitch, true);
}

rf_status rf_set_prior_flow(rf_handle* h, const float* u, const float* v, const float* mask,
                            int pitch) {
    if (!h || !u || !v) return fail(RF_ERR_INVALID_ARG, "rf_set_prior_flow: null argument");
    if (!prior_kind(h->p.method))
        return fail(RF_ERR_STATE, "rf_set_prior_flow: method has no prior-flow term");
    if (pitch < h->p.width) return fail(RF_ERR_INVALID_ARG, "rf_set_prior_flow: pitch < width");
    // the reference copies whole stride x height planes (Cudaflow.cu:338-343);
    // columns past `width` are zero here
    const size_t sp = h->stride * sizeof(float);
    for (int k = 0; k < 3; k++) {
        float* dst = k == 0 ? h->ufn : (k == 1 ? h->vfn : h->mask);
        const float* src = k == 0 ? u : (k == 1 ? v : mask);
        if (!src) {
            // on the handle's stream, ordered before the next solve (a
            // pageable source is staged before the call returns)
            std::vector<float> ones((size_t)h->stride * h->height, 1.0f);
            RF_CUDA(cudaMemcpyAsync(dst, ones.data(), ones.size() * sizeof(float),
                                    cudaMemcpyHostToDevice, h->stream));
            continue;
        }
        RF_CUDA(cudaMemcpy2DAsync(dst, sp, src, (size_t)pitch * sizeof(float),
                                  h->p.width * sizeof(float), h->p.height, cudaMemcpyHostToDevice,
                                  h->stream));
    }
    h->prior_set = true;
    return RF_OK;
}

rf_status rf_solve(rf_handle* h, const double R0[9], const double t0[3], const double R1[9],
                   const double t1[3]) {
    if (!h || !R1 || !t1) return fail(RF_ERR_INVALID_ARG, "rf_solve: null argument");
    if (h->p.method == RF_METHOD_TVL1)
        return fail(RF_ERR_STATE, "rf_solve: handle was created for plain TV-L1 (use rf_solve_flow)");
    if (!h->cams_set) return fail(RF_ERR_STATE, "rf_solve: rf_set_cameras not called");
    if (!h->images_set) return fail(RF_ERR_STATE, "rf_solve: no images uploaded");
    const double I[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    const double z[3] = {0, 0, 0};
    if (!R0) R0 = I;
    if (!t0) t0 = z;
    // the pinned block may still feed the previous solve's copy
    RF_CUDA(cudaStreamSynchronize(h->stream));
    level_consts(h, R0, t0, R1, t1, h->h_consts);
    std::memcpy(h->last_R1, R1, sizeof h->last_R1);
    std::memcpy(h->last_t1, t1, sizeof h->last_t1);
    RF_CUDA(cudaMemcpyAsync(h->d_consts, h->h_consts, sizeof(LevelConsts) * h->L,
                            cudaMemcpyHostToDevice, h->stream));
    rf_status rs = run_schedule(h, 0);
    h->solved = rs == RF_OK;
    return rs;
}

static rf_status stage_warm(rf_handle* h, int level, const float* const* src, int n, int pitch,
                            int on_device, int warps, int iters) {
    if (level < 0 || level >= h->L) return fail(RF_ERR_INVALID_ARG, "warm start: level out of range");
    if (pitch < h->W[level]) return fail(RF_ERR_INVALID_ARG, "warm start: pitch < level width");
    for (int k = 0; k < n; k++)
        if (!src[k]) return fail(RF_ERR_INVALID_ARG, "warm start: null input plane");
    const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    for (int k = 0; k < n; k++)
        RF_CUDA(cudaMemcpy2DAsync(h->warm[k], h->S[level] * sizeof(float), src[k],
                                  (size_t)pitch * sizeof(float), h->W[level] * sizeof(float),
                                  h->H[level], kind, h->stream));
    h->warm_level = level;
    h->warm_warps = warps < 0 ? h->p.n_warp_iters : warps;
    h->warm_iters = iters < 0 ? h->p.n_solver_iters : iters;
    return RF_OK;
}

rf_status rf_solve_warm(rf_handle* h, const double R0[9], const double t0[3], const double R1[9],
                        const double t1[3], int level, const float* u, const float* v,
                        const float* X, const float* Y, const float* Z, int pitch, int on_device,
                        int warps, int iters) {
    if (!h || !R1 || !t1) return fail(RF_ERR_INVALID_ARG, "rf_solve_warm: null argument");
    if (h->p.method != RF_METHODR_TVL1_MS)
        return fail(RF_ERR_UNSUPPORTED, "rf_solve_warm: warm start runs method 14");
    if (!h->cams_set || !h->images_set)
        return fail(RF_ERR_STATE, "rf_solve_warm: cameras or images missing");
    RF_CUDA(cudaStreamSynchronize(h->stream));
    const float* src[5] = {u, v, X, Y, Z};
    rf_status rs = stage_warm(h, level, src, 5, pitch, on_device, warps, iters);
    if (rs != RF_OK) return rs;
    const double I[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    const double z[3] = {0, 0, 0};
    level_consts(h, R0 ? R0 : I, t0 ? t0 : z, R1, t1, h->h_consts);
    std::memcpy(h->last_R1, R1, sizeof h->last_R1);
    std::memcpy(h->last_t1, t1, sizeof h->last_t1);
    RF_CUDA(cudaMemcpyAsync(h->d_consts, h->h_consts, sizeof(LevelConsts) * h->L,
                            cudaMemcpyHostToDevice, h->stream));
    rs = run_schedule(h, 2);
    h->solved = rs == RF_OK;
    return rs;
}

rf_status rf_solve_flow_warm(rf_handle* h, int level, const float* u, const float* v, int pitch,
                             int on_device, int warps, int iters) {
    if (!h) return fail(RF_ERR_INVALID_ARG, "rf_solve_flow_warm: null handle");
    if (h->p.method != RF_METHOD_TVL1)
        return fail(RF_ERR_STATE, "rf_solve_flow_warm: handle was created for a ReconFlow method");
    if (!h->images_set) return fail(RF_ERR_STATE, "rf_solve_flow_warm: no images uploaded");
    RF_CUDA(cudaStreamSynchronize(h->stream));
    const float* src[2] = {u, v};
    rf_status rs = stage_warm(h, level, src, 2, pitch, on_device, warps, iters);
    if (rs != RF_OK) return rs;
    rs = run_schedule(h, 3);
    h->solved = rs == RF_OK;
    return rs;
}

rf_status rf_energy(rf_handle* h, double* energy) {
    if (!h || !energy) return fail(RF_ERR_INVALID_ARG, "rf_energy: null argument");
    if (!h->solved) return fail(RF_ERR_STATE, "rf_energy: no solve has run");
    const bool recon = h->p.method != RF_METHOD_TVL1;
    LevelDims d{h->W[0], h->H[0], h->S[0]};
    const int nb = energy_blocks(d);
    if (launch_energy(h->I0[0], h->I1[0], h->res_u, h->res_v, recon ? h->X : nullptr,
                      recon ? h->Y : nullptr, recon ? h->Z : nullptr, d, h->p.lambda,
                      h->p.alpha_proj, recon ? h->last_R1 : nullptr, recon ? h->last_t1 : nullptr,
                      recon ? h->K1 : nullptr, recon ? 1 : 0, h->d_energy + 1, nb, h->d_energy,
                      h->stream) != 0)
        return cuda_fail(rf::last_launch_error(), "rf_energy: launch");
    h->launches += 2;
    RF_CUDA(cudaMemcpyAsync(energy, h->d_energy, sizeof(double), cudaMemcpyDeviceToHost,
                            h->stream));
    RF_CUDA(cudaStreamSynchronize(h->stream));
    return RF_OK;
}

rf_status rf_solve_flow(rf_handle* h) {
    if (!h) return fail(RF_ERR_INVALID_ARG, "rf_solve_flow: null handle");
    if (h->p.method != RF_METHOD_TVL1)
        return fail(RF_ERR_STATE, "rf_solve_flow: handle was created for a ReconFlow method");
    if (!h->images_set) return fail(RF_ERR_STATE, "rf_solve_flow: no images uploaded");
    rf_status rs = run_schedule(h, 1);
    h->solved = rs == RF_OK;
    return rs;
}


static rf_status download(rf_handle* h, const float* src, float* dst, int pitch) {
    RF_CUDA(cudaMemcpy2DAsync(dst, (size_t)pitch * sizeof(float), src, h->stride * sizeof(float),
                              h->p.width * sizeof(float), h->p.height, cudaMemcpyDeviceToHost,
                              h->stream));
    return RF_OK;
}

rf_status rf_download_flow(rf_handle* h, float* u, float* v, int pitch) {
    if (!h || !u || !v) return fail(RF_ERR_INVALID_ARG, "rf_download_flow: null argument");
    if (!h->solved) return fail(RF_ERR_STATE, "rf_download_flow: no solve has run");
    if (pitch < h->p.width) return fail(RF_ERR_INVALID_ARG, "rf_download_flow: pitch < width");
    rf_status rs = download(h, h->res_u, u, pitch);
    if (rs == RF_OK) rs = download(h, h->res_v, v, pitch);
    if (rs == RF_OK) RF_CUDA(cudaStreamSynchronize(h->stream));
    return rs;
}

rf_status rf_download_points(rf_handle* h, float* X, float* Y, float* Z, int pitch) {
    if (!h || !X || !Y || !Z) return fail(RF_ERR_INVALID_ARG, "rf_download_points: null argument");
    if (h->p.method == RF_METHOD_TVL1)
        return fail(RF_ERR_STATE, "rf_download_points: plain TV-L1 has no 3D output");
    if (!h->solved) return fail(RF_ERR_STATE, "rf_download_points: no solve has run");
    if (pitch < h->p.width) return fail(RF_ERR_INVALID_ARG, "rf_download_points: pitch < width");
    rf_status rs = download(h, h->X, X, pitch);
    if (rs == RF_OK) rs = download(h, h->Y, Y, pitch);
    if (rs == RF_OK) rs = download(h, h->Z, Z, pitch);
    if (rs == RF_OK) RF_CUDA(cudaStreamSynchronize(h->stream));
    return rs;
}

rf_status rf_download_inv_depth(rf_handle* h, float* inv, int pitch) {
    if (!h || !inv) return fail(RF_ERR_INVALID_ARG, "rf_download_inv_depth: null argument");
    if (h->p.method == RF_METHOD_TVL1)
        return fail(RF_ERR_STATE, "rf_download_inv_depth: plain TV-L1 has no depth");
    if (!h->solved) return fail(RF_ERR_STATE, "rf_download_inv_depth: no solve has run");
    if (pitch < h->p.width) return fail(RF_ERR_INVALID_ARG, "rf_download_inv_depth: pitch < width");
    LevelDims d{h->W[0], h->H[0], h->S[0]};
    if (launch_inv_depth(h->Z, d, h->scratch, h->stream) != 0)
        return cuda_fail(rf::last_launch_error(), "rf_download_inv_depth: launch");
    h->launches++;
    rf_status rs = download(h, h->scratch, inv, pitch);
    if (rs == RF_OK) RF_CUDA(cudaStreamSynchronize(h->stream));
    return rs;
}

rf_status rf_download_flow_color(rf_handle* h, float flow_scale, float* rgb, int pitch) {
    if (!h || !rgb) return fail(RF_ERR_INVALID_ARG, "rf_download_flow_color: null argument");
    if (!h->solved) return fail(RF_ERR_STATE, "rf_download_flow_color: no solve has run");
    if (pitch < h->p.width) return fail(RF_ERR_INVALID_ARG, "rf_download_flow_color: pitch < width");
    float* out = h->pool + (h->pool_floats - ((h->plane + 63) / 64 * 64) * 3);
    LevelDims d{h->W[0], h->H[0], h->S[0]};
    if (launch_flow_color(h->res_u, h->res_v, d, flow_scale, out, h->stream) != 0)
        return cuda_fail(rf::last_launch_error(), "rf_download_flow_color: launch");
    h->launches++;
    RF_CUDA(cudaMemcpy2DAsync(rgb, (size_t)pitch * 3 * sizeof(float), out,
                              (size_t)h->stride * 3 * sizeof(float), h->p.width * 3 * sizeof(float),
                              h->p.height, cudaMemcpyDeviceToHost, h->stream));
    RF_CUDA(cudaStreamSynchronize(h->stream));
    return RF_OK;
}

rf_status rf_remove_edge_artifacts(rf_handle* h, int surface_width, float max_area) {
    if (!h) return fail(RF_ERR_INVALID_ARG, "rf_remove_edge_artifacts: null handle");
    if (h->p.method == RF_METHOD_TVL1 || !h->solved)
        return fail(RF_ERR_STATE, "rf_remove_edge_artifacts: needs a ReconFlow solve");
    // ix - range stays >= 0 wherever ix + range > width only if 2*range <= width
    if (surface_width < 0 || 2 * surface_width > h->p.width || 2 * surface_width > h->p.height)
        return fail(RF_ERR_INVALID_ARG, "rf_remove_edge_artifacts: surface_width out of range");
    LevelDims d{h->W[0], h->H[0], h->S[0]};
    if (launch_remove_edge(h->X, h->Y, h->Z, surface_width, max_area, d, h->X1, h->Y1, h->Z1,
                           h->stream) != 0)
        return cuda_fail(rf::last_launch_error(), "rf_remove_edge_artifacts: launch");
    h->launches++;
    // the reference swaps X <-> Xs; copy back so X keeps its buffer
    const size_t bytes = (size_t)h->stride * h->height * sizeof(float);
    RF_CUDA(cudaMemcpyAsync(h->X, h->X1, bytes, cudaMemcpyDeviceToDevice, h->stream));
    RF_CUDA(cudaMemcpyAsync(h->Y, h->Y1, bytes, cudaMemcpyDeviceToDevice, h->stream));
    RF_CUDA(cudaMemcpyAsync(h->Z, h->Z1, bytes, cudaMemcpyDeviceToDevice, h->stream));
    return RF_OK;
}

rf_status rf_device_results(rf_handle* h, const float** u, const float** v, const float** X,
                            const float** Y, const float** Z) {
    if (!h) return fail(RF_ERR_INVALID_ARG, "rf_device_results: null handle");
    if (!h->solved) return fail(RF_ERR_STATE, "rf_device_results: no solve has run");
    if (u) *u = h->res_u;
    if (v) *v = h->res_v;
    if (X) *X = h->X;
    if (Y) *Y = h->Y;
    if (Z) *Z = h->Z;
    return RF_OK;
}

rf_status rf_debug_bounds(unsigned long long* count, long long* first) {
#ifdef RF_BOUNDS_CHECK
    if (!count) return fail(RF_ERR_INVALID_ARG, "rf_debug_bounds: null count");
    long long f1 = -1, f2 = -1;
    const unsigned long long c1 = rf::kernels_oob_take(&f1);
    const unsigned long long c2 = rf::batch_oob_take(&f2);
    *count = c1 + c2;
    if (first) *first = c1 ? f1 : (c2 ? f2 : -1);
    return RF_OK;
#else
    (void)count;
    (void)first;
    return fail(RF_ERR_UNSUPPORTED, "rf_debug_bounds: library built without RF_BOUNDS_CHECK");
#endif
}

rf_status rf_debug_bounds_selftest() {
    if (rf::launch_oob_selftest() != 0)
        return fail(RF_ERR_UNSUPPORTED, "rf_debug_bounds_selftest: needs an RF_BOUNDS_CHECK build");
    return RF_OK;
}

rf_status rf_set_cluster_pixels(long long max_px) {
    g_cluster_px.store(max_px < 0 ? 16384 : max_px);
    return RF_OK;
}

rf_status rf_set_tiles(rf_handle* h, const int* tile_w, const int* tile_h) {
    if (!h || !tile_w || !tile_h) return fail(RF_ERR_INVALID_ARG, "rf_set_tiles: null argument");
    for (int l = 0; l < h->L; l++) {
        const int w = tile_w[l], t = tile_h[l];
        if (w < 1 || t < 1 || w * t > 256 || (w * t) % 32 != 0)
            return fail(RF_ERR_INVALID_ARG,
                        "rf_set_tiles: a tile needs 32..256 threads, a multiple of 32");
    }
    RF_CUDA(cudaStreamSynchronize(h->stream));
    h->tile_w.assign(tile_w, tile_w + h->L);
    h->tile_h.assign(tile_h, tile_h + h->L);
    if (h->graph) {  // the captured schedule has the old launch shapes
        cudaGraphExecDestroy(h->graph);
        h->graph = nullptr;
        h->graph_kind = -1;
    }
    return RF_OK;
}

rf_status rf_set_stream(rf_handle* h, void* stream) {
    if (!h) return fail(RF_ERR_INVALID_ARG, "rf_set_stream: null handle");
    RF_CUDA(cudaStreamSynchronize(h->stream));
    h->stream = stream ? static_cast<cudaStream_t>(stream) : h->own_stream;
    return RF_OK;
}

rf_status rf_synchronize(rf_handle* h) {
    if (!h) return fail(RF_ERR_INVALID_ARG, "rf_synchronize: null handle");
    RF_CUDA(cudaStreamSynchronize(h->stream));
    return RF_OK;
}

rf_status rf_host_alloc(size_t bytes, void** ptr) {
    if (!ptr) return fail(RF_ERR_INVALID_ARG, "rf_host_alloc: null argument");
    cudaError_t e = rf::host_malloc(ptr, bytes);
    if (e != cudaSuccess) return fail(RF_ERR_OOM, std::string("rf_host_alloc: ") + cudaGetErrorString(e));
    return RF_OK;
}

rf_status rf_host_free(void* ptr) {
    if (ptr) RF_CUDA(cudaFreeHost(ptr));
    return RF_OK;
}

rf_status rf_profile_iterations(rf_handle* h, int level, int n_iters, float* ms) {
    if (!h || !ms || n_iters < 1 || level < 0 || level >= h->L)
        return fail(RF_ERR_INVALID_ARG, "rf_profile_iterations: bad argument");
    if (!h->solved) return fail(RF_ERR_STATE, "rf_profile_iterations: needs a prior solve");
    cudaStream_t st = h->stream;
    const Weights wt = make_weights(h->p);
    LevelDims d{h->W[level], h->H[level], h->S[level]};
    const bool recon = h->p.method != RF_METHOD_TVL1;
    ReconFields f{};
    f.extent = (long long)h->plane;
    if (recon) {
        f.u = h->res_u; f.v = h->res_v;
        f.duhat = h->duhat; f.dvhat = h->dvhat;
        f.pu1 = h->pu1; f.pu2 = h->pu2; f.pv1 = h->pv1; f.pv2 = h->pv2;
        f.uproj = h->st_uproj; f.vproj = h->st_vproj; f.sku = h->st_sku; f.skv = h->st_skv;
        f.Ix = h->Ix; f.Iy = h->Iy; f.Iz = h->Iz;
        f.X = h->X; f.Y = h->Y; f.Z = h->Z; f.X1 = h->X1; f.Y1 = h->Y1; f.Z1 = h->Z1;
        f.uc = h->st_uc; f.vc = h->st_vc;
        f.ufn = h->ufn_l; f.vfn = h->vfn_l; f.mask = h->mask_l;
    }
    const int prior = prior_kind(h->p.method);
    // Each kernel alone: n_iters launches back to back captured in one CUDA
    // graph (the form the solve uses), the graph launch timed with events;
    // ms = graph time / n_iters.  The first replay warms the graph up.
    for (int k = 0; k < 2; k++) {
        cudaGraph_t g = nullptr;
        cudaGraphExec_t ge = nullptr;
        RF_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        int bad = 0;
        for (int i = 0; i < n_iters && !bad; i++) {
            if (recon)
                bad = k == 0 ? launch_recon_a(f, h->d_consts + level, wt, d, false, false, prior, st,
                                              dim3(h->tile_w[level], h->tile_h[level]))
                             : launch_recon_b(f, wt, d, false, st,
                                              dim3(h->tile_w[level], h->tile_h[level]));
            else
                bad = k == 0 ? launch_plain_data(h->duhat, h->dvhat, h->pu1, h->pu2, h->pv1,
                                                 h->pv2, h->Ix, h->Iy, h->Iz, wt, d, false, st)
                             : launch_plain_tv(h->duhat, h->dvhat, h->pu1, h->pu2, h->pv1,
                                               h->pv2, wt, d, false, st);
        }
        cudaError_t ce = cudaStreamEndCapture(st, &g);
        if (bad || ce != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return cuda_fail(bad ? rf::last_launch_error() : ce,
                             "rf_profile_iterations: capture");
        }
        ce = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) return cuda_fail(ce, "rf_profile_iterations: instantiate");
        cudaEvent_t e0, e1;
        RF_CUDA(cudaEventCreate(&e0));
        RF_CUDA(cudaEventCreate(&e1));
        RF_CUDA(cudaGraphLaunch(ge, st));
        RF_CUDA(cudaEventRecord(e0, st));
        RF_CUDA(cudaGraphLaunch(ge, st));
        RF_CUDA(cudaEventRecord(e1, st));
        RF_CUDA(cudaEventSynchronize(e1));
        float t = 0;
        cudaEventElapsedTime(&t, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaGraphExecDestroy(ge);
        ms[k] = t / (float)n_iters;
        h->launches += 2 * (uint64_t)n_iters;
    }
    h->solved = false;
    return RF_OK;
}

uint64_t rf_kernel_launches(const rf_handle* h) { return h ? h->launches : 0; }

const char* rf_last_error_string(void) { return g_err.c_str(); }

const char* rf_version(void) { return "reconflow_gb300 0.1 (sm_103a)"; }

// ---------------------------------------------------------------------------
// Kernel-level entry points
// ---------------------------------------------------------------------------
#define RFK_CHECK(cond, name) \
    if (!(cond)) return fail(RF_ERR_INVALID_ARG, name ": bad argument")
#define RFK_RET(expr, name) \
    return (expr) == 0 ? RF_OK : cuda_fail(rf::last_launch_error(), name)

rf_status rfk_downscale(const float* src, int w, int h, int s, int nw, int nh, int ns, float scale,
                        int scaled, float* out, void* stream) {
    RFK_CHECK(src && out && w > 0 && h > 0 && s >= w && nw > 0 && nh > 0 && ns >= nw, "rfk_downscale");
    RFK_RET(launch_downscale(src, LevelDims{w, h, s}, LevelDims{nw, nh, ns}, scale, scaled != 0, out,
                             (cudaStream_t)stream),
            "rfk_downscale");
}

rf_status rfk_upscale(const float* src, int w, int h, int s, int nw, int nh, int ns, float scale,
                      float* out, void* stream) {
    RFK_CHECK(src && out && w > 0 && h > 0 && s >= w && nw > 0 && nh > 0 && ns >= nw, "rfk_upscale");
    RFK_RET(launch_upscale(src, LevelDims{w, h, s}, LevelDims{nw, nh, ns}, scale, out,
                           (cudaStream_t)stream),
            "rfk_upscale");
}

rf_status rfk_warp(const float* src, int w, int h, int s, const float* u, const float* v,
                   float* out, void* stream) {
    RFK_CHECK(src && u && v && out && w > 0 && h > 0 && s >= w, "rfk_warp");
    RFK_RET(launch_warp(src, u, v, LevelDims{w, h, s}, out, (cudaStream_t)stream), "rfk_warp");
}

rf_status rfk_warp_derivatives(const float* I0, const float* I1, const float* u, const float* v,
                               int w, int h, int s, float* Ix, float* Iy, float* Iz,
                               void* stream) {
    RFK_CHECK(I0 && I1 && u && v && Ix && Iy && Iz && w > 0 && h > 0 && s >= w,
              "rfk_warp_derivatives");
    RFK_RET(launch_warp_deriv(I0, I1, u, v, LevelDims{w, h, s}, Ix, Iy, Iz,
                              (cudaStream_t)stream),
            "rfk_warp_derivatives");
}

rf_status rfk_derivatives(const float* I0, const float* I1w, int w, int h, int s, float* Ix,
                          float* Iy, float* Iz, void* stream) {
    RFK_CHECK(I0 && I1w && Ix && Iy && Iz && w > 0 && h > 0 && s >= w, "rfk_derivatives");
    RFK_RET(launch_derivatives(I0, I1w, LevelDims{w, h, s}, Ix, Iy, Iz, (cudaStream_t)stream),
            "rfk_derivatives");
}

rf_status rfk_median5(const float* u, const float* v, int w, int h, int s, float* ou, float* ov,
                      void* stream) {
    RFK_CHECK(u && v && ou && ov && w > 0 && h > 0 && s >= w, "rfk_median5");
    RFK_RET(launch_median5(u, v, ou, ov, LevelDims{w, h, s}, (cudaStream_t)stream), "rfk_median5");
}

rf_status rfk_median3d(const float* X, const float* Y, const float* Z, int w, int h, int s,
                       float* X1, float* Y1, float* Z1, void* stream) {
    RFK_CHECK(X && Y && Z && X1 && Y1 && Z1 && w > 0 && h > 0 && s >= w, "rfk_median3d");
    RFK_RET(launch_median3d(X, Y, Z, X1, Y1, Z1, LevelDims{w, h, s}, (cudaStream_t)stream),
            "rfk_median3d");
}

rf_status rfk_warp_update(const float* duhat, const float* dvhat, const float* u, const float* v,
                          int w, int h, int s, float* tmp_u, float* tmp_v, float* out_u,
                          float* out_v, void* stream) {
    RFK_CHECK(duhat && dvhat && u && v && tmp_u && tmp_v && out_u && out_v && w > 0 && h > 0 &&
                  s >= w,
              "rfk_warp_update");
    LevelDims d{w, h, s};
    if (launch_median_add(duhat, dvhat, u, v, tmp_u, tmp_v, d, (cudaStream_t)stream) != 0)
        return cuda_fail(rf::last_launch_error(), "rfk_warp_update");
    RFK_RET(launch_median5(tmp_u, tmp_v, out_u, out_v, d, (cudaStream_t)stream), "rfk_warp_update");
}

rf_status rfk_rgb_to_gray(const uint8_t* rgb, int w, int h, int s, float* out, void* stream) {
    RFK_CHECK(rgb && out && w > 0 && h > 0 && s >= w, "rfk_rgb_to_gray");
    RFK_RET(launch_convert(rgb, RF_INPUT_RGB8, w, h, s, out, s, (cudaStream_t)stream),
            "rfk_rgb_to_gray");
}

rf_status rfk_remove_edge_artifacts(const float* X, const float* Y, const float* Z, int range,
                                    float max_area, int w, int h, int s, float* X1, float* Y1,
                                    float* Z1, void* stream) {
    RFK_CHECK(X && Y && Z && X1 && Y1 && Z1 && w > 0 && h > 0 && s >= w && range >= 0 &&
                  2 * range <= w && 2 * range <= h,
              "rfk_remove_edge_artifacts");
    RFK_RET(launch_remove_edge(X, Y, Z, range, max_area, LevelDims{w, h, s}, X1, Y1, Z1,
                               (cudaStream_t)stream),
            "rfk_remove_edge_artifacts");
}

rf_status rfk_flow_to_color(const float* u, const float* v, int w, int h, int s, float flow_scale,
                            float* rgb, void* stream) {
    RFK_CHECK(u && v && rgb && w > 0 && h > 0 && s >= w, "rfk_flow_to_color");
    RFK_RET(launch_flow_color(u, v, LevelDims{w, h, s}, flow_scale, rgb, (cudaStream_t)stream),
            "rfk_flow_to_color");
}

}  // extern "C"
