// Batched solver: many independent frame pairs, of different sizes, solved
// together.  Every step of the coarse-to-fine schedule (Reconflow.cu:147-466
// for ReconFlow, Cudaflow.cu:403-621 for plain TV-L1) is ONE launch covering
// that step for every pair, so small pyramid levels fill the GPU and the
// per-launch cost is paid once per step instead of once per pair.  The whole
// batch schedule is captured into one CUDA graph.
//
// Layout: plane-major.  Plane k (one role: u, duhat, X, ...) is one array
// holding every pair's level-0-sized region (its stride x (height + 1)
// floats, aligned to 64 floats) at the pair's offset off_i, the same offset
// in every plane; all pairs use the same plane index for the same role.  A
// pixel of pair i is therefore element off_i + x + y * stride of each of its
// planes, and the hot operations carry plain plane base pointers, so their
// per-field address arithmetic is the single-pair kernels'.  Blocks map to
// (pair, tile) through a per-level tile table.
//
// Per-pixel arithmetic is the shared code of the single-pair kernels
// (rf_ops.cuh), so a pair solved in a batch is bit-identical to the same pair
// solved alone.
#include <algorithm>
#include <climits>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/reconflow_gb300.h"
#include "rf_alloc.h"
#include "rf_nvtx.h"
#include "rf_kernels.cuh"
#include "rf_ops.cuh"

using namespace rf;

namespace rf_batch_impl {

// default tile of a level: 32 x 8 pixels = 256 threads (rf_batch_set_tiles
// chooses another shape per level; every tile has at most kMaxTile threads)
constexpr int BX = 32;
constexpr int BY = 8;
constexpr int kMaxTile = 256;
constexpr int kMaxLevels = 16;

struct BatchPair {
    LevelDims dims[kMaxLevels];
    int off;  // the pair's region: floats into every plane
};

// One block of a level: the tile whose first pixel is (x0, y0) in pair
// `pair`, whose region starts `off` floats into every plane.
struct __align__(16) TileEntry {
    int pair, x0, y0, off;
};

struct BatchCtx {
    const BatchPair* pairs;
    const TileEntry* tiles;     // this launch's level: one entry per block
    const LevelConsts* consts;  // [pair][level]
    float* pool;
    size_t total;               // floats per plane
    int n;
    int L;
    int prefetch;               // L2 prefetch distance in blocks (0 = none)
};

// plane k of the tile's pair
__device__ __forceinline__ float* plane_ptr(const BatchCtx& c, const TileEntry& t, int k) {
    return c.pool + (size_t)k * c.total + t.off;
}

__device__ __forceinline__ void prefetch_l2(const void* p) {
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// Operations with a `prefetch` member (the inner-iteration steps) first ask
// L2 for their fields at the same pixel of the tile `ctx.prefetch` blocks
// ahead -- the tile the next wave of blocks will run -- so its DRAM reads
// overlap this wave's work.
template <class Op, class = void>
struct HasPrefetch {
    static constexpr bool value = false;
};
template <class Op>
struct HasPrefetch<Op, decltype(void(&Op::prefetch))> {
    static constexpr bool value = true;
};

template <class Op>
__device__ __forceinline__ void prefetch_ahead(const BatchCtx& ctx, const TileEntry* tiles,
                                               int next, int count, int level, const Op& op) {
    if constexpr (HasPrefetch<Op>::value) {
        if (ctx.prefetch > 0 && next < count) {
            const TileEntry tn = tiles[next];
            const LevelDims dn = ctx.pairs[tn.pair].dims[level];
            const int ix = tn.x0 + (int)threadIdx.x, iy = tn.y0 + (int)threadIdx.y;
            if (ix < dn.w && iy < dn.h) op.prefetch(tn.off + ix + iy * dn.s);
        }
    }
}

// One block = one tile of one pair at `level` (the level's tile shape is
// the block shape; the tile table gives the pair and the tile's origin).
template <class Op>
__global__ void __launch_bounds__(kMaxTile) k_batch(BatchCtx ctx, int level, Op op) {
    prefetch_ahead(ctx, ctx.tiles, (int)blockIdx.x + ctx.prefetch, (int)gridDim.x, level, op);
    const TileEntry t = ctx.tiles[blockIdx.x];
    const LevelDims d = ctx.pairs[t.pair].dims[level];
    const int ix = t.x0 + (int)threadIdx.x, iy = t.y0 + (int)threadIdx.y;
    if (ix >= d.w || iy >= d.h) return;
    op(ctx, t, level, d, ix, iy);
}

// Two rows per thread: the block is the tile's width by half its height;
// thread (x, y) takes tile rows 2y and 2y + 1 (Op::two), so operations whose
// neighbouring rows share work (the 5x5 medians) do it once.
template <class Op>
__global__ void __launch_bounds__(kMaxTile) k_batch_rows2(BatchCtx ctx, int level, Op op) {
    const TileEntry t = ctx.tiles[blockIdx.x];
    const LevelDims d = ctx.pairs[t.pair].dims[level];
    const int ix = t.x0 + (int)threadIdx.x, iy = t.y0 + 2 * (int)threadIdx.y;
    if (ix >= d.w || iy >= d.h) return;
    op.two(t, d, ix, iy);
}

// Level-0 row copies (the staging gathers): one warp per row of a pair's
// level 0, block (pair, chunk of 8 rows, striding by the grid's chunks);
// Op::row(e0, w, lane) moves the row's w elements starting at element e0
// of every plane.
constexpr int kRowWarps = 8;
template <class Op>
__global__ void __launch_bounds__(32 * kRowWarps) k_batch_rows_l0(const BatchPair* pairs, Op op) {
    const BatchPair& p = pairs[blockIdx.x];
    const LevelDims d = p.dims[0];
    for (int row = (int)blockIdx.y * kRowWarps + ((int)threadIdx.x >> 5); row < d.h;
         row += (int)gridDim.y * kRowWarps)
        op.row((size_t)p.off + (size_t)row * d.s, d.w, (int)threadIdx.x & 31);
}

// Two operations in one launch on disjoint tile ranges of the level's table
// (x: [x0, x0 + nx), y: [y0, y0 + ny)), their blocks interleaved (x, y, x,
// y, ..., then the rest of the longer range) so that every SM holds blocks
// of both: the instruction-bound data step of one pair group runs beside
// the memory-bound dual step of the other.
template <class OpX, class OpY>
__global__ void __launch_bounds__(kMaxTile) k_batch_pair(BatchCtx ctx, int level, OpX opx, int x0,
                                                         int nx, OpY opy, int y0, int ny) {
    const int b = blockIdx.x, m = nx < ny ? nx : ny;
    bool is_x;
    int k;
    if (b < 2 * m) {
        is_x = (b & 1) == 0;
        k = b >> 1;
    } else {
        is_x = nx > ny;
        k = b - m;
    }
    if (is_x)
        prefetch_ahead(ctx, ctx.tiles + x0, k + ctx.prefetch / 2, nx, level, opx);
    else
        prefetch_ahead(ctx, ctx.tiles + y0, k + ctx.prefetch / 2, ny, level, opy);
    const TileEntry t = ctx.tiles[is_x ? x0 + k : y0 + k];
    const LevelDims d = ctx.pairs[t.pair].dims[level];
    const int ix = t.x0 + (int)threadIdx.x, iy = t.y0 + (int)threadIdx.y;
    if (ix >= d.w || iy >= d.h) return;
    if (is_x)
        opx(ctx, t, level, d, ix, iy);
    else
        opy(ctx, t, level, d, ix, iy);
}

// ---- per-step operations (plane indices resolved per pair) ----------------
struct OpDownscale2 {
    int a, b, oa, ob;  // fine planes (level-1) -> coarse planes (level)
    __device__ void operator()(const BatchCtx& ctx, const TileEntry& t, int level, LevelDims c,
                               int ix, int iy) const {
        LevelDims f = ctx.pairs[t.pair].dims[level - 1];
        plane_ptr(ctx, t, oa)[ix + iy * c.s] = 0.25f * downscale_px(plane_ptr(ctx, t, a), f, c.w, c.h, ix, iy);
        plane_ptr(ctx, t, ob)[ix + iy * c.s] = 0.25f * downscale_px(plane_ptr(ctx, t, b), f, c.w, c.h, ix, iy);
    }
};

struct OpWarp {
    int I1, u, v, out;
    __device__ void operator()(const BatchCtx& ctx, const TileEntry& t, int, LevelDims d, int ix,
                               int iy) const {
        warp_px(plane_ptr(ctx, t, I1), plane_ptr(ctx, t, u), plane_ptr(ctx, t, v), d, plane_ptr(ctx, t, out), ix, iy);
    }
};

struct OpDeriv {
    int I0, I1w, Ix, Iy, Iz;
    __device__ void operator()(const BatchCtx& ctx, const TileEntry& t, int, LevelDims d, int ix,
                               int iy) const {
        derivatives_px(plane_ptr(ctx, t, I0), plane_ptr(ctx, t, I1w), d, plane_ptr(ctx, t, Ix), plane_ptr(ctx, t, Iy),
                       plane_ptr(ctx, t, Iz), ix, iy);
    }
};

struct ReconIdx {
    int u, v, duhat, dvhat, pu1, pu2, pv1, pv2, uproj, vproj, sku, skv, Ix, Iy, Iz, X, Y, Z, X1,
        Y1, Z1, uc, vc;
};

// The inner-iteration operations carry the planes' base pointers
// (ReconFields, resolved on the host from plane indices); a pixel's element
// is the tile's pair offset plus its position in the level.
struct OpReconA {
    ReconFields f;
    Weights wt;
    int first, ucb;
    __device__ void operator()(const BatchCtx& ctx, const TileEntry& t, int level, LevelDims d,
                               int ix, int iy) const {
        recon_a_px<0>(f, ctx.consts[t.pair * ctx.L + level], wt, d, ix, iy, first, ucb, t.off);
    }
    // (no prefetch: the data step is bound by instruction issue; prefetching
    // all 18 of its fields took the 64-pair level-0 launch from 1410.6 to
    // 1537.9 us, five of them (X, Y, Z, u, v) from 1399.7 to 1487.3 us)
};

struct OpReconB {
    ReconFields f;
    Weights wt;
    int first;
    __device__ void operator()(const BatchCtx&, const TileEntry& t, int, LevelDims d, int ix,
                               int iy) const {
        recon_b_px(f, wt, d, ix, iy, first, t.off);
    }
    // the fields recon_b_px reads at a pixel (element e of every plane); the
    // dual / median step waits on memory, so reading the next wave's pixels
    // into L2 early pays
    __device__ void prefetch(int e) const {
        const float* p[] = {f.duhat, f.dvhat, f.pu1, f.pu2, f.pv1, f.pv2, f.X1, f.Y1, f.Z1,
                            f.sku, f.skv, f.u, f.v, f.uproj, f.vproj};
#pragma unroll
        for (const float* q : p) prefetch_l2(q + e);
    }
};

struct OpPlainData {
    int duhat, dvhat, pu1, pu2, pv1, pv2, Ix, Iy, Iz;
    Weights wt;
    int first;
    __device__ void operator()(const BatchCtx& ctx, const TileEntry& t, int, LevelDims d, int ix,
                               int iy) const {
        plain_data_px(plane_ptr(ctx, t, duhat), plane_ptr(ctx, t, dvhat), plane_ptr(ctx, t, pu1),
                      plane_ptr(ctx, t, pu2), plane_ptr(ctx, t, pv1), plane_ptr(ctx, t, pv2), plane_ptr(ctx, t, Ix),
                      plane_ptr(ctx, t, Iy), plane_ptr(ctx, t, Iz), wt, d, first, ix, iy);
    }
};

struct OpPlainTV {
    int duhat, dvhat, pu1, pu2, pv1, pv2;
    Weights wt;
    int first;
    __device__ void operator()(const BatchCtx& ctx, const TileEntry& t, int, LevelDims d, int ix,
                               int iy) const {
        plain_tv_px(plane_ptr(ctx, t, duhat), plane_ptr(ctx, t, dvhat), plane_ptr(ctx, t, pu1),
                    plane_ptr(ctx, t, pu2), plane_ptr(ctx, t, pv1), plane_ptr(ctx, t, pv2), wt, d, first, ix,
                    iy);
    }
};

// u + median5(duhat) (Reconflow.cu:410-416); out may be u itself
struct OpMedianAdd {
    const float* duhat;  // plane base pointers
    const float* dvhat;
    const float* u;
    const float* v;
    float* ou;
    float* ov;
    __device__ void operator()(const BatchCtx&, const TileEntry& t, int, LevelDims d, int ix,
                               int iy) const {
        float mu, mv;
        median5_pair(duhat, dvhat, ix, iy, d, mu, mv, t.off);
        int pos = t.off + ix + iy * d.s;
        float a = u[pos] + mu;
        float b = v[pos] + mv;
        ou[pos] = a;
        ov[pos] = b;
    }
    // pixels (ix, iy) and (ix, iy + 1) (the second when inside the level)
    __device__ void two(const TileEntry& t, LevelDims d, int ix, int iy) const {
        float mu[2], mv[2];
        median5_pair2(duhat, dvhat, ix, iy, d, mu, mv, t.off);
        const int pos = t.off + ix + iy * d.s;
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
};

struct OpMedian5 {
    const float* u;  // plane base pointers
    const float* v;
    float* ou;
    float* ov;
    __device__ void operator()(const BatchCtx&, const TileEntry& t, int, LevelDims d, int ix,
                               int iy) const {
        float mu, mv;
        median5_pair(u, v, ix, iy, d, mu, mv, t.off);
        ou[t.off + ix + iy * d.s] = mu;
        ov[t.off + ix + iy * d.s] = mv;
    }
    __device__ void two(const TileEntry& t, LevelDims d, int ix, int iy) const {
        float mu[2], mv[2];
        median5_pair2(u, v, ix, iy, d, mu, mv, t.off);
        const int pos = t.off + ix + iy * d.s;
        ou[pos] = mu[0];
        ov[pos] = mv[0];
        if (iy + 1 < d.h) {
            ou[pos + d.s] = mu[1];
            ov[pos + d.s] = mv[1];
        }
    }
};

struct OpSolveUc {
    int X, Y, Z, uc, vc;
    __device__ void operator()(const BatchCtx& ctx, const TileEntry& t, int level, LevelDims d,
                               int ix, int iy) const {
        int pos = ix + iy * d.s;
        float a, b;
        project_uc(ctx.consts[t.pair * ctx.L + level], plane_ptr(ctx, t, X)[pos], plane_ptr(ctx, t, Y)[pos],
                   plane_ptr(ctx, t, Z)[pos], ix, iy, a, b);
        plane_ptr(ctx, t, uc)[pos] = a;
        plane_ptr(ctx, t, vc)[pos] = b;
    }
};

// upscale.cu:14-27 for up to 8 fields: runs on the tiles of the fine level
// `level`; the coarse level is level + 1.
struct OpUpscale {
    int n;
    int src[8], dst[8];
    float scale;
    __device__ void operator()(const BatchCtx& ctx, const TileEntry& t, int level, LevelDims f,
                               int ix, int iy) const {
        LevelDims c = ctx.pairs[t.pair].dims[level + 1];
        float x = ((float)ix + 0.5f) / (float)f.w;
        float y = ((float)iy + 0.5f) / (float)f.h;
        Taps tx = taps_of(x, c.w);
        Taps ty = taps_of(y, c.h);
        int pos = ix + iy * f.s;
        // fixed trip count: the field indices stay in the parameter bank
#pragma unroll
        for (int i = 0; i < 8; i++)
            if (i < n)
                plane_ptr(ctx, t, dst[i])[pos] = bilerp(plane_ptr(ctx, t, src[i]), c.s, tx, ty) * scale;
    }
};

// staged frames -> the pairs' level-0 image planes (rf_batch_take_upload):
// the same pixels the per-pair copies of rf_batch_upload_images write, in
// one launch over every pair's rows (staging and pool share the layout)
struct OpStageIn {
    const float* s0;
    const float* s1;
    float* d0;
    float* d1;
    // k_batch_rows_l0: lane `lane` takes columns lane, lane + 32, ...; four
    // columns' loads go out before their stores
    __device__ void row(size_t e0, int w, int lane) const {
        int c = lane;
        for (; c + 96 < w; c += 128) {
            float a[4], b[4];
#pragma unroll
            for (int k = 0; k < 4; k++) {
                a[k] = s0[e0 + c + 32 * k];
                b[k] = s1[e0 + c + 32 * k];
            }
#pragma unroll
            for (int k = 0; k < 4; k++) {
                d0[e0 + c + 32 * k] = a[k];
                d1[e0 + c + 32 * k] = b[k];
            }
        }
        for (; c < w; c += 32) {
            const float a = s0[e0 + c], b = s1[e0 + c];
            d0[e0 + c] = a;
            d1[e0 + c] = b;
        }
    }
};

// the pairs' results -> the download staging planes (u, v, 1/Z, X, Y, Z
// at k * total; bit k of `mask` selects output k), one launch over every
// pair's rows
struct OpStageOut {
    const float* u;
    const float* v;
    const float* X;
    const float* Y;
    const float* Z;
    float* out;
    size_t total;
    int mask;
    // element e of every requested output
    __device__ __forceinline__ void at(size_t e) const {
        if (mask & 1) out[e] = u[e];
        if (mask & 2) out[total + e] = v[e];
        if (mask & 60) {
            const float z = Z[e];
            if (mask & 4) out[2 * total + e] = 1.0f / z;
            if (mask & 8) out[3 * total + e] = X[e];
            if (mask & 16) out[4 * total + e] = Y[e];
            if (mask & 32) out[5 * total + e] = z;
        }
    }
    // k_batch_rows_l0: as OpStageIn::row, the requested fields of four
    // columns loaded before their stores
    __device__ void row(size_t e0, int w, int lane) const {
        int c = lane;
        for (; c + 96 < w; c += 128) {
            float fu[4], fv[4], fx[4], fy[4], fz[4];
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const size_t e = e0 + c + 32 * k;
                fu[k] = (mask & 1) ? u[e] : 0.0f;
                fv[k] = (mask & 2) ? v[e] : 0.0f;
                fz[k] = (mask & 60) ? Z[e] : 0.0f;
                fx[k] = (mask & 8) ? X[e] : 0.0f;
                fy[k] = (mask & 16) ? Y[e] : 0.0f;
            }
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const size_t e = e0 + c + 32 * k;
                if (mask & 1) out[e] = fu[k];
                if (mask & 2) out[total + e] = fv[k];
                if (mask & 4) out[2 * total + e] = 1.0f / fz[k];
                if (mask & 8) out[3 * total + e] = fx[k];
                if (mask & 16) out[4 * total + e] = fy[k];
                if (mask & 32) out[5 * total + e] = fz[k];
            }
        }
        for (; c < w; c += 32) at(e0 + c);
    }
};

struct OpInvDepth {
    int Z, out;
    __device__ void operator()(const BatchCtx& ctx, const TileEntry& t, int, LevelDims d, int ix,
                               int iy) const {
        int pos = ix + iy * d.s;
        plane_ptr(ctx, t, out)[pos] = 1.0f / plane_ptr(ctx, t, Z)[pos];
    }
};

// warm start (rf_batch_solve_warm): the caller's planes at the start level
// become u, v (and uproj, vproj) and the 3D state, as rf_solve_warm stages them
struct OpWarmInit {
    int wu, wv, wX, wY, wZ, u, v, uproj, vproj, X, Y, Z;
    __device__ void operator()(const BatchCtx& ctx, const TileEntry& t, int, LevelDims d, int ix,
                               int iy) const {
        int pos = ix + iy * d.s;
        float a = plane_ptr(ctx, t, wu)[pos], c = plane_ptr(ctx, t, wv)[pos];
        plane_ptr(ctx, t, u)[pos] = a;
        plane_ptr(ctx, t, v)[pos] = c;
        plane_ptr(ctx, t, uproj)[pos] = a;
        plane_ptr(ctx, t, vproj)[pos] = c;
        plane_ptr(ctx, t, X)[pos] = plane_ptr(ctx, t, wX)[pos];
        plane_ptr(ctx, t, Y)[pos] = plane_ptr(ctx, t, wY)[pos];
        plane_ptr(ctx, t, Z)[pos] = plane_ptr(ctx, t, wZ)[pos];
    }
};

thread_local std::string g_batch_err;

rf_status bfail(rf_status st, const std::string& msg) {
    return static_cast<rf_status>(rf::set_last_error(st, msg.c_str()));
}

int align_up_i(int n, int m) {
    int mod = n % m;
    return mod ? n + m - mod : n;
}

}  // namespace rf_batch_impl

using namespace rf_batch_impl;

struct rf_batch {
    rf_params p{};
    int n = 0, L = 0;
    std::vector<std::vector<LevelDims>> dims;  // [pair][level]
    std::vector<size_t> plane, base_off;  // per pair: region size and offset in a plane
    size_t total = 0;                     // floats per plane (every pair's region)
    float* pool = nullptr;                // n_planes x total floats
    BatchPair* d_pairs = nullptr;
    TileEntry* d_tiles = nullptr;         // every level's tile table, level after level
    size_t tiles_cap = 0;                 // entries allocated at d_tiles
    std::vector<size_t> tile_start;       // first entry of each level
    std::vector<int> prefix;  // [level][n + 1] tile prefix sums
    std::vector<int> tile_w, tile_h;  // tile shape of each level
    LevelConsts* d_consts = nullptr;
    LevelConsts* h_consts = nullptr;
    std::vector<double> K0, K1;  // [pair][9]
    std::vector<char> cams;
    std::vector<char> imgs;
    cudaStream_t own = nullptr, stream = nullptr;
    cudaGraphExec_t graph = nullptr;
    int graph_kind = -1;
    // kind 2 (warm start): start level and warps / iterations per level
    int warm_level = -1;
    std::vector<int> warm_warps, warm_iters;
    std::vector<int> graph_sched;  // the warm schedule the graph was captured with
    std::vector<double> last_R1, last_t1;  // pose of the last solve, [pair][9], [pair][3]
    double* d_energy = nullptr;            // [pair][kEnergyMaxBlocks] partials, then [pair] sums
    EnergyJob* d_ejobs = nullptr;          // [pair]
    EnergyJob* h_ejobs = nullptr;          // pinned staging of d_ejobs
    cudaEvent_t ejobs_copied = nullptr;    // the last copy out of h_ejobs has run
    uint64_t launches = 0, graph_nodes = 0, enq = 0;
    int res_u = -1, res_v = -1;
    // pipelined inner iterations (pairs [0, split) and [split, n) half an
    // iteration apart); 0 = every inner half-iteration over all pairs at once
    int split = 0;
    int prefetch = 0;  // L2 prefetch distance of the inner-iteration launches, in blocks
    bool solved = false;
    int n_planes = 0;
    // pipelined transfers (rf_batch_stage_upload / rf_batch_stage_download):
    // device staging planes laid out like the pool's, one copy stream per
    // direction and the events that order them against the solve stream,
    // made on first use
    float* stage_in = nullptr;   // 2 planes: frame 0, frame 1
    float* stage_out = nullptr;  // 6 planes: u, v, inverse depth, X, Y, Z
    cudaStream_t copy_in = nullptr, copy_out = nullptr;
    cudaEvent_t in_staged = nullptr, in_free = nullptr, out_ready = nullptr, out_done = nullptr;
    bool up_staged = false;
    // plane indices
    int pI0(int l) const { return l; }
    int pI1(int l) const { return L + l; }
    int base_idx() const { return 2 * L; }
    int warm_idx(int k) const;  // warm-start input plane k (u, v, X, Y, Z)
};

namespace rf_batch_impl {

enum {
    P_I1W = 0, P_IX, P_IY, P_IZ, P_DUHAT, P_DVHAT, P_PU1, P_PU2, P_PV1, P_PV2, P_X, P_Y, P_Z, P_X1,
    P_Y1, P_Z1, P_SCRATCH, P_SPARE0
};
constexpr int kSpares = 18;
constexpr int kWarmPlanes = 5;

}  // namespace rf_batch_impl

int rf_batch::warm_idx(int k) const { return base_idx() + rf_batch_impl::P_SPARE0 + rf_batch_impl::kSpares + k; }

namespace rf_batch_impl {

// Per-level prefix sums of tile counts and the tile tables for the current
// tile shapes (row-major tiles of each pair, pairs in order), copied to the
// device; the caller makes sure no launch is in flight.
cudaError_t fill_tiles(rf_batch* b) {
    b->prefix.assign((size_t)b->L * (b->n + 1), 0);
    b->tile_start.assign(b->L, 0);
    std::vector<TileEntry> tab;
    for (int l = 0; l < b->L; l++) {
        b->tile_start[l] = tab.size();
        const int tw = b->tile_w[l], th = b->tile_h[l];
        for (int i = 0; i < b->n; i++) {
            const LevelDims& d = b->dims[i][l];
            const int nx = (d.w + tw - 1) / tw, ny = (d.h + th - 1) / th;
            for (int y = 0; y < ny; y++)
                for (int x = 0; x < nx; x++)
                    tab.push_back(TileEntry{i, x * tw, y * th, (int)b->base_off[i]});
            b->prefix[l * (b->n + 1) + i + 1] = b->prefix[l * (b->n + 1) + i] + nx * ny;
        }
    }
    if (tab.size() > b->tiles_cap) {
        if (b->d_tiles) cudaFree(b->d_tiles);
        b->d_tiles = nullptr;
        b->tiles_cap = 0;
        cudaError_t e = rf::dev_malloc((void**)&b->d_tiles, sizeof(TileEntry) * tab.size());
        if (e != cudaSuccess) return e;
        b->tiles_cap = tab.size();
    }
    // on the batch's stream (the legacy stream would not order it with the
    // non-blocking solve stream); the pageable source is staged on return
    return cudaMemcpyAsync(b->d_tiles, tab.data(), sizeof(TileEntry) * tab.size(),
                           cudaMemcpyHostToDevice, b->stream);
}

BatchCtx ctx_of(rf_batch* b, int level) {
    BatchCtx c;
    c.pairs = b->d_pairs;
    c.tiles = b->d_tiles + b->tile_start[level];
    c.consts = b->d_consts;
    c.pool = b->pool;
    c.total = b->total;
    c.n = b->n;
    c.L = b->L;
    c.prefetch = b->prefetch;
    return c;
}

// base pointer of plane k (every pair's region of it)
float* plane_base(rf_batch* b, int k) { return b->pool + (size_t)k * b->total; }

ReconFields fields_of(rf_batch* b, const ReconIdx& r) {
    ReconFields f{};
    f.extent = (long long)b->total;
    f.u = plane_base(b, r.u); f.v = plane_base(b, r.v);
    f.duhat = plane_base(b, r.duhat); f.dvhat = plane_base(b, r.dvhat);
    f.pu1 = plane_base(b, r.pu1); f.pu2 = plane_base(b, r.pu2);
    f.pv1 = plane_base(b, r.pv1); f.pv2 = plane_base(b, r.pv2);
    f.uproj = plane_base(b, r.uproj); f.vproj = plane_base(b, r.vproj);
    f.sku = plane_base(b, r.sku); f.skv = plane_base(b, r.skv);
    f.Ix = plane_base(b, r.Ix); f.Iy = plane_base(b, r.Iy); f.Iz = plane_base(b, r.Iz);
    f.X = plane_base(b, r.X); f.Y = plane_base(b, r.Y); f.Z = plane_base(b, r.Z);
    f.X1 = plane_base(b, r.X1); f.Y1 = plane_base(b, r.Y1); f.Z1 = plane_base(b, r.Z1);
    f.uc = plane_base(b, r.uc); f.vc = plane_base(b, r.vc);
    return f;
}

template <class Op>
int launch_op(rf_batch* b, int level, const Op& op) {
    int tiles = b->prefix[level * (b->n + 1) + b->n];
    if (tiles <= 0) return 0;
    const dim3 block(b->tile_w[level], b->tile_h[level]);
    k_batch<Op><<<tiles, block, 0, b->stream>>>(ctx_of(b, level), level, op);
    b->enq++;
    return rf::launch_status();
}

// a level-0 row operation (Op::row) over every pair's rows in one launch
template <class Op>
int launch_rows_l0(rf_batch* b, const Op& op) {
    int max_h = 0;
    for (int i = 0; i < b->n; i++) max_h = b->dims[i][0].h > max_h ? b->dims[i][0].h : max_h;
    int chunks = (max_h + kRowWarps - 1) / kRowWarps;
    if (chunks <= 0) return 0;
    if (chunks > 65535) chunks = 65535;  // the grid's y limit; blocks stride over the rest
    k_batch_rows_l0<Op><<<dim3(b->n, chunks), 32 * kRowWarps, 0, b->stream>>>(b->d_pairs, op);
    b->enq++;
    return rf::launch_status();
}

// an operation with a two-row form (Op::two) over the level's tiles, two
// rows per thread where the tile height is even (the one-row kernel if not)
template <class Op>
int launch_op_rows2(rf_batch* b, int level, const Op& op) {
    const int th = b->tile_h[level];
    if (th % 2 != 0) return launch_op(b, level, op);
    int tiles = b->prefix[level * (b->n + 1) + b->n];
    if (tiles <= 0) return 0;
    k_batch_rows2<Op><<<tiles, dim3(b->tile_w[level], th / 2), 0, b->stream>>>(ctx_of(b, level),
                                                                              level, op);
    b->enq++;
    return rf::launch_status();
}

// Tile range of pair group g at `level`: group 0 = pairs [0, split), group
// 1 = pairs [split, n).
void group_tiles(const rf_batch* b, int level, int g, int& begin, int& count) {
    const int* pre = &b->prefix[(size_t)level * (b->n + 1)];
    const int lo = g == 0 ? 0 : b->split, hi = g == 0 ? b->split : b->n;
    begin = pre[lo];
    count = pre[hi] - pre[lo];
}

// `op` over the tiles of pair group g only
template <class Op>
int launch_group(rf_batch* b, int level, int g, const Op& op) {
    int begin, count;
    group_tiles(b, level, g, begin, count);
    if (count <= 0) return 0;
    BatchCtx c = ctx_of(b, level);
    c.tiles += begin;
    const dim3 block(b->tile_w[level], b->tile_h[level]);
    k_batch<Op><<<count, block, 0, b->stream>>>(c, level, op);
    b->enq++;
    return rf::launch_status();
}

// `x` over pair group gx and `y` over the other group, in one launch
template <class OpX, class OpY>
int launch_pair(rf_batch* b, int level, int gx, const OpX& x, const OpY& y) {
    int xb, nx, yb, ny;
    group_tiles(b, level, gx, xb, nx);
    group_tiles(b, level, 1 - gx, yb, ny);
    if (nx + ny <= 0) return 0;
    const dim3 block(b->tile_w[level], b->tile_h[level]);
    k_batch_pair<OpX, OpY><<<nx + ny, block, 0, b->stream>>>(ctx_of(b, level), level, x, xb, nx,
                                                             y, yb, ny);
    b->enq++;
    return rf::launch_status();
}

#define BL(expr)                                                                       \
    do {                                                                               \
        if ((expr) != 0)                                                               \
            return bfail(RF_ERR_CUDA, std::string("batch launch: ") +                 \
                                          cudaGetErrorString(rf::last_launch_error())); \
    } while (0)
#define BC(call)                                                                       \
    do {                                                                               \
        cudaError_t e__ = (call);                                                      \
        if (e__ != cudaSuccess)                                                        \
            return bfail(e__ == cudaErrorMemoryAllocation ? RF_ERR_OOM : RF_ERR_CUDA,         \
                        std::string(#call ": ") + cudaGetErrorString(e__));            \
    } while (0)

// zero `count` planes starting at index k for every pair
rf_status memset_planes(rf_batch* b, std::initializer_list<int> ks) {
    for (int k : ks)
        BC(cudaMemsetAsync(plane_base(b, k), 0, b->total * sizeof(float), b->stream));
    return RF_OK;
}

rf_status enqueue_batch(rf_batch* b, int kind) {
    const rf_params& p = b->p;
    const Weights wt = solver_weights(&p);
    const int B0 = b->base_idx();
    auto P = [&](int k) { return B0 + k; };
    auto PB = [&](int k) { return plane_base(b, k); };
    // pyramid
    for (int l = 1; l < b->L; l++)
        BL(launch_op(b, l, OpDownscale2{b->pI0(l - 1), b->pI1(l - 1), b->pI0(l), b->pI1(l)}));
    int sp[kSpares];
    for (int i = 0; i < kSpares; i++) sp[i] = P(P_SPARE0 + i);
    int u = sp[0], v = sp[1], uc = sp[2], vc = sp[3], uproj = sp[4], vproj = sp[5], sku = sp[6],
        skv = sp[7], tu = sp[8], tv = sp[9];
    std::vector<int> freep(sp + 10, sp + kSpares);
    const bool recon = kind == 0 || kind == 2;
    const bool warm = kind == 2;
    const int top = warm ? b->warm_level : b->L - 1;
    if (recon) {
        rf_status rs = memset_planes(b, {u, v, uproj, vproj, uc, vc, sku, skv, P(P_X), P(P_Y), P(P_Z)});
        if (rs != RF_OK) return rs;
    } else {
        rf_status rs = memset_planes(b, {u, v});
        if (rs != RF_OK) return rs;
    }
    bool ucb = true;
    if (warm) {
        BL(launch_op(b, top, OpWarmInit{b->warm_idx(0), b->warm_idx(1), b->warm_idx(2),
                                        b->warm_idx(3), b->warm_idx(4), u, v, uproj, vproj,
                                        P(P_X), P(P_Y), P(P_Z)}));
        ucb = false;  // uc from the warm 3D state in the first iteration
    }
    for (int level = top; level >= 0; level--) {
        NvtxRange level_range("batch level %d", level);
        const int n_warps = warm ? b->warm_warps[level] : p.n_warp_iters;
        const int n_iters = warm ? b->warm_iters[level] : p.n_solver_iters;
        for (int warp = 0; warp < n_warps; warp++) {
            NvtxRange warp_range("batch level %d warp %d", level, warp);
            // WarpImage and ComputeDerivatives as two launches: the fused
            // shared-memory form recomputes its halo's warped values, which at
            // the tuned level-0 tile (32 x 2) costs more than the warped
            // image's round trip (0.312 vs 0.196 ms for 8 720p pairs)
            BL(launch_op(b, level, OpWarp{b->pI1(level), u, v, P(P_I1W)}));
            BL(launch_op(b, level, OpDeriv{b->pI0(level), P(P_I1W), P(P_IX), P(P_IY), P(P_IZ)}));
            const ReconFields r = fields_of(
                b, ReconIdx{u, v, P(P_DUHAT), P(P_DVHAT), P(P_PU1), P(P_PU2), P(P_PV1), P(P_PV2),
                            uproj, vproj, sku, skv, P(P_IX), P(P_IY), P(P_IZ), P(P_X), P(P_Y),
                            P(P_Z), P(P_X1), P(P_Y1), P(P_Z1), uc, vc});
            if (recon && b->split > 0 && n_iters > 0) {
                // the two pair groups one half-iteration apart: each launch
                // runs one group's data step (A) beside the other's dual step
                // (B); every pair still sees A, B, A, B, ... in order
                const int u0 = ucb ? 1 : 0;
                BL(launch_group(b, level, 0, OpReconA{r, wt, 1, u0}));
                for (int iter = 0; iter < n_iters; iter++) {
                    const int first = iter == 0;
                    BL(launch_pair(b, level, 0, OpReconB{r, wt, first},
                                   OpReconA{r, wt, first, first ? u0 : 0}));
                    if (iter + 1 < n_iters)
                        BL(launch_pair(b, level, 0, OpReconA{r, wt, 0, 0}, OpReconB{r, wt, first}));
                    else
                        BL(launch_group(b, level, 1, OpReconB{r, wt, first}));
                }
                ucb = false;
            }
            for (int iter = 0; iter < n_iters && !(recon && b->split > 0); iter++) {
                const int first = iter == 0;
                if (recon) {
                    BL(launch_op(b, level, OpReconA{r, wt, first, ucb ? 1 : 0}));
                    BL(launch_op(b, level, OpReconB{r, wt, first}));
                    ucb = false;
                } else {
                    BL(launch_op(b, level, OpPlainData{P(P_DUHAT), P(P_DVHAT), P(P_PU1), P(P_PU2),
                                                       P(P_PV1), P(P_PV2), P(P_IX), P(P_IY),
                                                       P(P_IZ), wt, first}));
                    BL(launch_op(b, level, OpPlainTV{P(P_DUHAT), P(P_DVHAT), P(P_PU1), P(P_PU2),
                                                     P(P_PV1), P(P_PV2), wt, first}));
                }
            }
            if (n_iters == 0) {
                rf_status rs = memset_planes(b, {P(P_DUHAT), P(P_DVHAT)});
                if (rs != RF_OK) return rs;
            }
            if (recon) {
                BL(launch_op_rows2(b, level, OpMedianAdd{PB(P(P_DUHAT)), PB(P(P_DVHAT)), PB(u), PB(v),
                                                   PB(tu), PB(tv)}));
                BL(launch_op_rows2(b, level, OpMedian5{PB(tu), PB(tv), PB(u), PB(v)}));
            } else {
                BL(launch_op_rows2(b, level, OpMedianAdd{PB(P(P_DUHAT)), PB(P(P_DVHAT)), PB(u), PB(v),
                                                   PB(u), PB(v)}));
            }
        }
        if (level > 0) {
            OpUpscale up{};
            if (recon) {
                if (!ucb) BL(launch_op(b, level, OpSolveUc{P(P_X), P(P_Y), P(P_Z), uc, vc}));
                int src[8] = {u, v, uc, vc, uproj, vproj, sku, skv};
                up.n = 8;
                for (int i = 0; i < 8; i++) {
                    up.src[i] = src[i];
                    up.dst[i] = freep[i];
                }
                up.scale = p.scale;
                BL(launch_op(b, level - 1, up));
                for (int i = 0; i < 8; i++) freep[i] = src[i];
                u = up.dst[0]; v = up.dst[1]; uc = up.dst[2]; vc = up.dst[3];
                uproj = up.dst[4]; vproj = up.dst[5]; sku = up.dst[6]; skv = up.dst[7];
                ucb = true;
            } else {
                up.n = 2;
                up.src[0] = u; up.src[1] = v;
                up.dst[0] = freep[0]; up.dst[1] = freep[1];
                up.scale = p.scale;
                BL(launch_op(b, level - 1, up));
                freep[0] = u; freep[1] = v;
                u = up.dst[0]; v = up.dst[1];
            }
        }
    }
    b->res_u = u;
    b->res_v = v;
    return RF_OK;
}

rf_status run_batch(rf_batch* b, int kind) {
    NvtxRange range(kind == 2 ? "rf_batch_solve_warm" : "rf_batch_solve");
    std::vector<int> sched;
    if (kind == 2) {
        sched.push_back(b->warm_level);
        sched.insert(sched.end(), b->warm_warps.begin(), b->warm_warps.end());
        sched.insert(sched.end(), b->warm_iters.begin(), b->warm_iters.end());
    }
    if (b->graph && (b->graph_kind != kind || b->graph_sched != sched)) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    if (!b->graph) {
        cudaGraph_t g = nullptr;
        BC(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        b->enq = 0;
        rf_status rs = enqueue_batch(b, kind);
        cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
        if (rs != RF_OK) {
            if (g) cudaGraphDestroy(g);
            return rs;
        }
        if (ce != cudaSuccess) return bfail(RF_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(ce));
        cudaError_t ie = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) {
            b->graph = nullptr;
            return bfail(RF_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(ie));
        }
        b->graph_kind = kind;
        b->graph_sched = sched;
        b->graph_nodes = b->enq;
    }
    BC(cudaGraphLaunch(b->graph, b->stream));
    b->launches += b->graph_nodes;
    return RF_OK;
}

float* pair_plane(rf_batch* b, int i, int k) { return plane_base(b, k) + b->base_off[i]; }


}  // namespace rf_batch_impl

namespace rf {
unsigned long long batch_oob_take(long long* first) {
#ifdef RF_BOUNDS_CHECK
    return rf_oob_take(first);
#else
    (void)first;
    return 0;
#endif
}
}  // namespace rf

extern "C" {

rf_status rf_batch_create(const rf_params* p, int n_pairs, const int* widths, const int* heights,
                          rf_batch** out) {
    if (!p || !widths || !heights || !out || n_pairs < 1)
        return bfail(RF_ERR_INVALID_ARG, "rf_batch_create: bad argument");
    *out = nullptr;
    if (p->method != RF_METHODR_TVL1_MS && p->method != RF_METHOD_TVL1)
        return bfail(RF_ERR_UNSUPPORTED, "rf_batch_create: batches run methods 0 and 14");
    if (p->input_type != RF_INPUT_F32)
        return bfail(RF_ERR_UNSUPPORTED, "rf_batch_create: batches take float32 gray input");
    if (p->n_levels < 1 || p->n_levels > kMaxLevels || !(p->scale > 1.0f) ||
        p->stride_alignment < 1 || p->n_warp_iters < 0 || p->n_solver_iters < 0 ||
        (p->method == RF_METHOD_TVL1 ? !(p->theta != 0.0f) : !(p->alpha_tv != 0.0f)))
        return bfail(RF_ERR_INVALID_ARG, "rf_batch_create: parameters out of range");
    rf_batch* b = new rf_batch();
    b->p = *p;
    b->n = n_pairs;
    b->L = p->n_levels;
    b->dims.resize(n_pairs);
    size_t total = 0;
    b->n_planes = 2 * b->L + P_SPARE0 + kSpares + kWarmPlanes;
    for (int i = 0; i < n_pairs; i++) {
        int w = widths[i], h = heights[i];
        if (w < 1 || h < 1 || (long long)w * h > (1LL << 28)) {
            delete b;
            return bfail(RF_ERR_INVALID_ARG, "rf_batch_create: pair size out of range");
        }
        int nh = h, nw = w, ns = align_up_i(w, p->stride_alignment);
        for (int l = 0; l < b->L; l++) {
            if (nw < 1 || nh < 1) {
                delete b;
                return bfail(RF_ERR_INVALID_ARG, "rf_batch_create: too many levels for a pair");
            }
            b->dims[i].push_back(LevelDims{nw, nh, ns});
            nh = (int)((float)nh / p->scale);
            nw = (int)((float)nw / p->scale);
            ns = align_up_i(nw, p->stride_alignment);
        }
        size_t pl = ((size_t)b->dims[i][0].s * (h + 1) + 63) / 64 * 64;
        b->plane.push_back(pl);
        b->base_off.push_back(total);
        total += pl;
    }
    // a pixel's element in a plane (pair offset + position) is a 32-bit int
    if (total > (size_t)INT_MAX) {
        delete b;
        return bfail(RF_ERR_INVALID_ARG, "rf_batch_create: batch too large (over 2^31 - 1 "
                                         "floats per plane)");
    }
    b->total = total;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        delete b;
        return bfail(RF_ERR_NO_DEVICE, "rf_batch_create: no CUDA device");
    }
    const size_t pool_floats = total * (size_t)b->n_planes;
    cudaError_t e = rf::dev_malloc((void**)&b->pool, pool_floats * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(b->pool, 0, pool_floats * sizeof(float));
    std::vector<BatchPair> hp(n_pairs);
    for (int i = 0; i < n_pairs; i++) {
        for (int l = 0; l < b->L; l++) hp[i].dims[l] = b->dims[i][l];
        hp[i].off = (int)b->base_off[i];
    }
    b->tile_w.assign(b->L, BX);
    b->tile_h.assign(b->L, BY);
    {
        // pipelined pair groups: opt-in (RF_BATCH_PIPELINE=1); with the L2
        // prefetch below the plain order measured as fast
        const char* e = std::getenv("RF_BATCH_PIPELINE");
        const bool on = e && e[0] == '1';
        b->split = on && n_pairs >= 2 ? n_pairs / 2 : 0;
        // distance = the blocks resident at once (one wave of 16 blocks per
        // SM), RF_BATCH_PREFETCH times (default 1; 0 = off)
        const char* pf = std::getenv("RF_BATCH_PREFETCH");
        const double waves = pf ? std::atof(pf) : 1.0;
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        b->prefetch = waves > 0.0 ? (int)(waves * sms * 16) : 0;
    }
    if (e == cudaSuccess) e = fill_tiles(b);
    if (e == cudaSuccess) e = rf::dev_malloc((void**)&b->d_pairs, sizeof(BatchPair) * n_pairs);
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_pairs, hp.data(), sizeof(BatchPair) * n_pairs, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = rf::dev_malloc((void**)&b->d_consts, sizeof(LevelConsts) * n_pairs * b->L);
    if (e == cudaSuccess) e = rf::host_malloc((void**)&b->h_consts, sizeof(LevelConsts) * n_pairs * b->L);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        rf_batch_destroy(b);
        return bfail(RF_ERR_OOM, std::string("rf_batch_create: ") + cudaGetErrorString(e));
    }
    b->stream = b->own;
    // the pool's clearing memset and the table copies ran on the legacy
    // default stream (fill_tiles before the stream existed): finish them
    // before the non-blocking stream can read the pool
    if (cudaDeviceSynchronize() != cudaSuccess) {
        rf_batch_destroy(b);
        return bfail(RF_ERR_CUDA, "rf_batch_create: initialisation");
    }
    b->K0.assign((size_t)9 * n_pairs, 0.0);
    b->K1.assign((size_t)9 * n_pairs, 0.0);
    b->cams.assign(n_pairs, 0);
    b->imgs.assign(n_pairs, 0);
    *out = b;
    return RF_OK;
}

rf_status rf_batch_destroy(rf_batch* b) {
    if (!b) return RF_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (cudaStream_t st : {b->copy_in, b->copy_out})
        if (st) {
            cudaStreamSynchronize(st);
            cudaStreamDestroy(st);
        }
    for (cudaEvent_t ev : {b->in_staged, b->in_free, b->out_ready, b->out_done, b->ejobs_copied})
        if (ev) cudaEventDestroy(ev);
    if (b->stage_in) cudaFree(b->stage_in);
    if (b->stage_out) cudaFree(b->stage_out);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    if (b->pool) cudaFree(b->pool);
    if (b->d_pairs) cudaFree(b->d_pairs);
    if (b->d_tiles) cudaFree(b->d_tiles);
    if (b->d_consts) cudaFree(b->d_consts);
    if (b->d_energy) cudaFree(b->d_energy);
    if (b->d_ejobs) cudaFree(b->d_ejobs);
    if (b->h_ejobs) cudaFreeHost(b->h_ejobs);
    if (b->h_consts) cudaFreeHost(b->h_consts);
    if (b->own) cudaStreamDestroy(b->own);
    delete b;
    return RF_OK;
}

int rf_batch_stride(const rf_batch* b, int pair) {
    if (!b || pair < 0 || pair >= b->n) return -1;
    return b->dims[pair][0].s;
}

rf_status rf_batch_set_cameras(rf_batch* b, int pair, const double K0[9], const double K1[9]) {
    if (!b || !K0 || !K1 || pair < 0 || pair >= b->n)
        return bfail(RF_ERR_INVALID_ARG, "rf_batch_set_cameras: bad argument");
    std::memcpy(&b->K0[(size_t)9 * pair], K0, 9 * sizeof(double));
    std::memcpy(&b->K1[(size_t)9 * pair], K1, 9 * sizeof(double));
    b->cams[pair] = 1;
    return RF_OK;
}

static rf_status batch_upload(rf_batch* b, int pair, const void* i0, const void* i1, int pitch,
                              cudaMemcpyKind kind) {
    if (!b || !i0 || !i1 || pair < 0 || pair >= b->n)
        return bfail(RF_ERR_INVALID_ARG, "rf_batch_upload_images: bad argument");
    const LevelDims& d = b->dims[pair][0];
    if (pitch < d.w) return bfail(RF_ERR_INVALID_ARG, "rf_batch_upload_images: pitch < width");
    BC(cudaMemcpy2DAsync(pair_plane(b, pair, b->pI0(0)), d.s * sizeof(float), i0,
                         (size_t)pitch * sizeof(float), d.w * sizeof(float), d.h, kind, b->stream));
    BC(cudaMemcpy2DAsync(pair_plane(b, pair, b->pI1(0)), d.s * sizeof(float), i1,
                         (size_t)pitch * sizeof(float), d.w * sizeof(float), d.h, kind, b->stream));
    b->imgs[pair] = 1;
    return RF_OK;
}

rf_status rf_batch_upload_images(rf_batch* b, int pair, const float* i0, const float* i1,
                                 int pitch) {
    return batch_upload(b, pair, i0, i1, pitch, cudaMemcpyHostToDevice);
}

rf_status rf_batch_upload_images_device(rf_batch* b, int pair, const float* i0, const float* i1,
                                        int pitch) {
    return batch_upload(b, pair, i0, i1, pitch, cudaMemcpyDeviceToDevice);
}

static rf_status batch_poses(rf_batch* b, const char* who, const double* R0, const double* t0,
                             const double* R1, const double* t1) {
    if (!b || !R1 || !t1) return bfail(RF_ERR_INVALID_ARG, std::string(who) + ": null argument");
    if (b->p.method == RF_METHOD_TVL1)
        return bfail(RF_ERR_STATE, std::string(who) + ": batch was created for plain TV-L1");
    for (int i = 0; i < b->n; i++)
        if (!b->cams[i] || !b->imgs[i])
            return bfail(RF_ERR_STATE, std::string(who) + ": pair " + std::to_string(i) +
                                           " has no cameras or images");
    BC(cudaStreamSynchronize(b->stream));
    const double I[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1}, z[3] = {0, 0, 0};
    for (int i = 0; i < b->n; i++)
        camera_level_consts(&b->K0[(size_t)9 * i], &b->K1[(size_t)9 * i], b->L, b->p.scale,
                            b->p.fix_quirks, R0 ? R0 + 9 * i : I, t0 ? t0 + 3 * i : z, R1 + 9 * i,
                            t1 + 3 * i, b->h_consts + (size_t)i * b->L);
    BC(cudaMemcpyAsync(b->d_consts, b->h_consts, sizeof(LevelConsts) * b->n * b->L,
                       cudaMemcpyHostToDevice, b->stream));
    b->last_R1.assign(R1, R1 + 9 * b->n);
    b->last_t1.assign(t1, t1 + 3 * b->n);
    return RF_OK;
}

rf_status rf_batch_solve(rf_batch* b, const double* R0, const double* t0, const double* R1,
                         const double* t1) {
    rf_status rs = batch_poses(b, "rf_batch_solve", R0, t0, R1, t1);
    if (rs != RF_OK) return rs;
    rs = run_batch(b, 0);
    b->solved = rs == RF_OK;
    return rs;
}

rf_status rf_batch_warm_planes(rf_batch* b, int pair, float** u, float** v, float** X, float** Y,
                               float** Z) {
    if (!b || pair < 0 || pair >= b->n)
        return bfail(RF_ERR_INVALID_ARG, "rf_batch_warm_planes: bad argument");
    float** out[5] = {u, v, X, Y, Z};
    for (int k = 0; k < 5; k++)
        if (out[k]) *out[k] = pair_plane(b, pair, b->warm_idx(k));
    return RF_OK;
}

rf_status rf_batch_energies(rf_batch* b, double* out) {
    if (!b || !out) return bfail(RF_ERR_INVALID_ARG, "rf_batch_energies: null argument");
    const rf_status rs = rf_batch_energies_async(b, out);
    if (rs != RF_OK) return rs;
    BC(cudaStreamSynchronize(b->stream));
    return RF_OK;
}

rf_status rf_batch_energies_async(rf_batch* b, double* out) {
    if (!b || !out) return bfail(RF_ERR_INVALID_ARG, "rf_batch_energies: null argument");
    if (!b->solved || b->p.method == RF_METHOD_TVL1 || b->last_R1.size() != (size_t)9 * b->n)
        return bfail(RF_ERR_STATE, "rf_batch_energies: needs a ReconFlow solve");
    if (!b->d_energy) BC(rf::dev_malloc((void**)&b->d_energy, sizeof(double) * b->n * (kEnergyMaxBlocks + 1)));
    if (!b->d_ejobs) BC(rf::dev_malloc((void**)&b->d_ejobs, sizeof(EnergyJob) * b->n));
    if (!b->h_ejobs) BC(rf::host_malloc((void**)&b->h_ejobs, sizeof(EnergyJob) * b->n));
    if (!b->ejobs_copied) BC(cudaEventCreateWithFlags(&b->ejobs_copied, cudaEventDisableTiming));
    // the pinned job table is free to refill once the last call's copy of it
    // has run (usually long ago: no wait on the solve itself)
    BC(cudaEventSynchronize(b->ejobs_copied));
    const int B0 = b->base_idx();
    double* sums = b->d_energy + (size_t)b->n * kEnergyMaxBlocks;
    int blocks = 0, max_blocks = 0;
    // every pair's evaluation in one launch (blocks in pair order) and the
    // sums in a second; each pair's value is its single-pair evaluation's
    for (int i = 0; i < b->n; i++) {
        EnergyJob& j = b->h_ejobs[i];
        j.a = energy_args(pair_plane(b, i, b->pI0(0)), pair_plane(b, i, b->pI1(0)),
                          pair_plane(b, i, b->res_u), pair_plane(b, i, b->res_v),
                          pair_plane(b, i, B0 + P_X), pair_plane(b, i, B0 + P_Y),
                          pair_plane(b, i, B0 + P_Z), b->p.lambda, b->p.alpha_proj,
                          &b->last_R1[(size_t)9 * i], &b->last_t1[(size_t)3 * i],
                          &b->K1[(size_t)9 * i], 1);
        j.d = b->dims[i][0];
        j.nblocks = energy_blocks(j.d);
        j.first_block = blocks;
        j.partial = b->d_energy + (size_t)i * kEnergyMaxBlocks;
        j.out = sums + i;
        blocks += j.nblocks;
        if (j.nblocks > max_blocks) max_blocks = j.nblocks;
    }
    BC(cudaMemcpyAsync(b->d_ejobs, b->h_ejobs, sizeof(EnergyJob) * b->n, cudaMemcpyHostToDevice,
                       b->stream));
    BC(cudaEventRecord(b->ejobs_copied, b->stream));
    if (launch_energy_jobs(b->d_ejobs, b->n, blocks, max_blocks, b->stream) != 0)
        return bfail(RF_ERR_CUDA, "rf_batch_energies: launch");
    b->launches += 2;
    BC(cudaMemcpyAsync(out, sums, sizeof(double) * b->n, cudaMemcpyDeviceToHost, b->stream));
    return RF_OK;
}

rf_status rf_batch_set_tiles(rf_batch* b, const int* tile_w, const int* tile_h) {
    if (!b || !tile_w || !tile_h) return bfail(RF_ERR_INVALID_ARG, "rf_batch_set_tiles: null argument");
    for (int l = 0; l < b->L; l++) {
        const int w = tile_w[l], h = tile_h[l];
        if (w < 1 || h < 1 || w * h > kMaxTile || (w * h) % 32 != 0)
            return bfail(RF_ERR_INVALID_ARG, "rf_batch_set_tiles: a tile needs 32..256 threads, a "
                                             "multiple of 32");
    }
    BC(cudaStreamSynchronize(b->stream));
    b->tile_w.assign(tile_w, tile_w + b->L);
    b->tile_h.assign(tile_h, tile_h + b->L);
    BC(fill_tiles(b));
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
        b->graph_kind = -1;
    }
    return RF_OK;
}

rf_status rf_batch_profile_level(rf_batch* b, int level, int n_iters, float* ms) {
    if (!b || !ms || n_iters < 1 || level < 0 || level >= b->L)
        return bfail(RF_ERR_INVALID_ARG, "rf_batch_profile_level: bad argument");
    if (!b->solved || b->p.method == RF_METHOD_TVL1)
        return bfail(RF_ERR_STATE, "rf_batch_profile_level: needs a ReconFlow solve");
    const Weights wt = solver_weights(&b->p);
    const int B0 = b->base_idx();
    auto P = [&](int k) { return B0 + k; };
    const int u = b->res_u, v = b->res_v;
    // the role planes of the last solve's finest level (values only matter for timing)
    const ReconFields r = fields_of(
        b, ReconIdx{u, v, P(P_DUHAT), P(P_DVHAT), P(P_PU1), P(P_PU2), P(P_PV1), P(P_PV2),
                    P(P_SPARE0 + 4), P(P_SPARE0 + 5), P(P_SPARE0 + 6), P(P_SPARE0 + 7), P(P_IX),
                    P(P_IY), P(P_IZ), P(P_X), P(P_Y), P(P_Z), P(P_X1), P(P_Y1), P(P_Z1),
                    P(P_SPARE0 + 2), P(P_SPARE0 + 3)});
    for (int k = 0; k < 2; k++) {
        cudaGraph_t g = nullptr;
        cudaGraphExec_t ge = nullptr;
        BC(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        int bad = 0;
        for (int i = 0; i < n_iters && !bad; i++)
            bad = k == 0 ? launch_op(b, level, OpReconA{r, wt, 0, 0})
                         : launch_op(b, level, OpReconB{r, wt, 0});
        cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
        if (bad || ce != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return bfail(RF_ERR_CUDA, "rf_batch_profile_level: capture");
        }
        ce = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) return bfail(RF_ERR_CUDA, "rf_batch_profile_level: instantiate");
        cudaEvent_t e0, e1;
        BC(cudaEventCreate(&e0));
        BC(cudaEventCreate(&e1));
        BC(cudaGraphLaunch(ge, b->stream));
        BC(cudaEventRecord(e0, b->stream));
        BC(cudaGraphLaunch(ge, b->stream));
        BC(cudaEventRecord(e1, b->stream));
        BC(cudaEventSynchronize(e1));
        float t = 0;
        cudaEventElapsedTime(&t, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaGraphExecDestroy(ge);
        ms[k] = t / (float)n_iters;
        b->launches += 2 * (uint64_t)n_iters;
    }
    b->solved = false;
    return RF_OK;
}

rf_status rf_batch_image_planes(rf_batch* b, int pair, int level, const float** I0,
                                const float** I1) {
    if (!b || pair < 0 || pair >= b->n || level < 0 || level >= b->L)
        return bfail(RF_ERR_INVALID_ARG, "rf_batch_image_planes: bad argument");
    if (I0) *I0 = pair_plane(b, pair, b->pI0(level));
    if (I1) *I1 = pair_plane(b, pair, b->pI1(level));
    return RF_OK;
}

rf_status rf_batch_solve_warm_levels(rf_batch* b, const double* R0, const double* t0,
                                     const double* R1, const double* t1, int level,
                                     const int* warps, const int* iters) {
    if (!b || !warps || !iters) return bfail(RF_ERR_INVALID_ARG, "rf_batch_solve_warm: null argument");
    if (level < 0 || level >= b->L)
        return bfail(RF_ERR_INVALID_ARG, "rf_batch_solve_warm: level out of range");
    for (int l = 0; l <= level; l++)
        if (warps[l] < 0 || iters[l] < 0 || warps[l] > 1000 || iters[l] > 100000)
            return bfail(RF_ERR_INVALID_ARG, "rf_batch_solve_warm: schedule out of range");
    rf_status rs = batch_poses(b, "rf_batch_solve_warm", R0, t0, R1, t1);
    if (rs != RF_OK) return rs;
    b->warm_level = level;
    b->warm_warps.assign(warps, warps + level + 1);
    b->warm_iters.assign(iters, iters + level + 1);
    rs = run_batch(b, 2);
    b->solved = rs == RF_OK;
    return rs;
}

rf_status rf_batch_solve_warm(rf_batch* b, const double* R0, const double* t0, const double* R1,
                              const double* t1, int level, int warps, int iters) {
    if (!b) return bfail(RF_ERR_INVALID_ARG, "rf_batch_solve_warm: null batch");
    if (level < 0 || level >= b->L)
        return bfail(RF_ERR_INVALID_ARG, "rf_batch_solve_warm: level out of range");
    std::vector<int> w(level + 1, warps), it(level + 1, iters);
    return rf_batch_solve_warm_levels(b, R0, t0, R1, t1, level, w.data(), it.data());
}

rf_status rf_batch_solve_flow(rf_batch* b) {
    if (!b) return bfail(RF_ERR_INVALID_ARG, "rf_batch_solve_flow: null batch");
    if (b->p.method != RF_METHOD_TVL1)
        return bfail(RF_ERR_STATE, "rf_batch_solve_flow: batch was created for ReconFlow");
    for (int i = 0; i < b->n; i++)
        if (!b->imgs[i]) return bfail(RF_ERR_STATE, "rf_batch_solve_flow: missing images");
    rf_status rs = run_batch(b, 1);
    b->solved = rs == RF_OK;
    return rs;
}

static rf_status batch_down(rf_batch* b, int pair, int k, float* dst, int pitch) {
    const LevelDims& d = b->dims[pair][0];
    BC(cudaMemcpy2DAsync(dst, (size_t)pitch * sizeof(float), pair_plane(b, pair, k),
                         d.s * sizeof(float), d.w * sizeof(float), d.h, cudaMemcpyDeviceToHost,
                         b->stream));
    return RF_OK;
}

rf_status rf_batch_download_flow(rf_batch* b, int pair, float* u, float* v, int pitch) {
    if (!b || !u || !v || pair < 0 || pair >= b->n)
        return bfail(RF_ERR_INVALID_ARG, "rf_batch_download_flow: bad argument");
    if (!b->solved) return bfail(RF_ERR_STATE, "rf_batch_download_flow: no solve has run");
    if (pitch < b->dims[pair][0].w) return bfail(RF_ERR_INVALID_ARG, "pitch < width");
    rf_status rs = batch_down(b, pair, b->res_u, u, pitch);
    if (rs == RF_OK) rs = batch_down(b, pair, b->res_v, v, pitch);
    if (rs == RF_OK) BC(cudaStreamSynchronize(b->stream));
    return rs;
}

rf_status rf_batch_download_points(rf_batch* b, int pair, float* X, float* Y, float* Z,
                                   int pitch) {
    if (!b || !X || !Y || !Z || pair < 0 || pair >= b->n)
        return bfail(RF_ERR_INVALID_ARG, "rf_batch_download_points: bad argument");
    if (b->p.method == RF_METHOD_TVL1 || !b->solved)
        return bfail(RF_ERR_STATE, "rf_batch_download_points: needs a ReconFlow solve");
    if (pitch < b->dims[pair][0].w) return bfail(RF_ERR_INVALID_ARG, "pitch < width");
    const int B0 = b->base_idx();
    rf_status rs = batch_down(b, pair, B0 + P_X, X, pitch);
    if (rs == RF_OK) rs = batch_down(b, pair, B0 + P_Y, Y, pitch);
    if (rs == RF_OK) rs = batch_down(b, pair, B0 + P_Z, Z, pitch);
    if (rs == RF_OK) BC(cudaStreamSynchronize(b->stream));
    return rs;
}

rf_status rf_batch_download_inv_depth(rf_batch* b, int pair, float* inv, int pitch) {
    if (!b || !inv || pair < 0 || pair >= b->n)
        return bfail(RF_ERR_INVALID_ARG, "rf_batch_download_inv_depth: bad argument");
    if (b->p.method == RF_METHOD_TVL1 || !b->solved)
        return bfail(RF_ERR_STATE, "rf_batch_download_inv_depth: needs a ReconFlow solve");
    if (pitch < b->dims[pair][0].w) return bfail(RF_ERR_INVALID_ARG, "pitch < width");
    const int B0 = b->base_idx();
    BL(launch_op(b, 0, OpInvDepth{B0 + P_Z, B0 + P_SCRATCH}));
    b->launches++;
    rf_status rs = batch_down(b, pair, B0 + P_SCRATCH, inv, pitch);
    if (rs == RF_OK) BC(cudaStreamSynchronize(b->stream));
    return rs;
}

rf_status rf_batch_upload_all(rf_batch* b, const float* const* i0, const float* const* i1,
                              int pitch) {
    if (!b || !i0 || !i1) return bfail(RF_ERR_INVALID_ARG, "rf_batch_upload_all: null argument");
    for (int i = 0; i < b->n; i++) {
        if (!i0[i] || !i1[i]) return bfail(RF_ERR_INVALID_ARG, "rf_batch_upload_all: null image");
        rf_status rs = batch_upload(b, i, i0[i], i1[i], pitch, cudaMemcpyHostToDevice);
        if (rs != RF_OK) return rs;
    }
    return RF_OK;
}

rf_status rf_batch_download_all(rf_batch* b, float* const* u, float* const* v,
                                float* const* inv_depth, float* const* X, float* const* Y,
                                float* const* Z, int pitch) {
    if (!b) return bfail(RF_ERR_INVALID_ARG, "rf_batch_download_all: null batch");
    if (!b->solved) return bfail(RF_ERR_STATE, "rf_batch_download_all: no solve has run");
    const bool recon = b->p.method != RF_METHOD_TVL1;
    if (!recon && (inv_depth || X || Y || Z))
        return bfail(RF_ERR_STATE, "rf_batch_download_all: plain TV-L1 has no 3D output");
    for (int i = 0; i < b->n; i++)
        if (pitch < b->dims[i][0].w) return bfail(RF_ERR_INVALID_ARG, "pitch < width");
    const int B0 = b->base_idx();
    if (inv_depth) {
        BL(launch_op(b, 0, OpInvDepth{B0 + P_Z, B0 + P_SCRATCH}));
        b->launches++;
    }
    struct Out {
        float* const* dst;
        int plane;
    } outs[6] = {{u, b->res_u}, {v, b->res_v}, {inv_depth, B0 + P_SCRATCH},
                 {X, B0 + P_X}, {Y, B0 + P_Y}, {Z, B0 + P_Z}};
    for (const Out& o : outs) {
        if (!o.dst) continue;
        for (int i = 0; i < b->n; i++) {
            if (!o.dst[i]) continue;
            rf_status rs = batch_down(b, i, o.plane, o.dst[i], pitch);
            if (rs != RF_OK) return rs;
        }
    }
    BC(cudaStreamSynchronize(b->stream));
    return RF_OK;
}

// Copy streams, events and the staging planes of one direction, made on
// first use (a batch that never pipelines its transfers holds none of them).
static rf_status ensure_staging(rf_batch* b, bool out) {
    for (cudaStream_t* st : {&b->copy_in, &b->copy_out})
        if (!*st) BC(cudaStreamCreateWithFlags(st, cudaStreamNonBlocking));
    for (cudaEvent_t* ev : {&b->in_staged, &b->in_free, &b->out_ready, &b->out_done})
        if (!*ev) BC(cudaEventCreateWithFlags(ev, cudaEventDisableTiming));
    float** buf = out ? &b->stage_out : &b->stage_in;
    if (!*buf) BC(rf::dev_malloc((void**)buf, b->total * (out ? 6 : 2) * sizeof(float)));
    return RF_OK;
}

rf_status rf_batch_stage_upload(rf_batch* b, const float* const* i0, const float* const* i1,
                                int pitch) {
    if (!b || !i0 || !i1) return bfail(RF_ERR_INVALID_ARG, "rf_batch_stage_upload: null argument");
    if (b->up_staged)
        return bfail(RF_ERR_STATE, "rf_batch_stage_upload: the staged frames were not taken yet");
    for (int i = 0; i < b->n; i++) {
        if (!i0[i] || !i1[i]) return bfail(RF_ERR_INVALID_ARG, "rf_batch_stage_upload: null image");
        if (pitch < b->dims[i][0].w)
            return bfail(RF_ERR_INVALID_ARG, "rf_batch_stage_upload: pitch < width");
    }
    rf_status rs = ensure_staging(b, false);
    if (rs != RF_OK) return rs;
    // the staging planes are free once the last rf_batch_take_upload's
    // copies out of them have run on the solve stream
    BC(cudaStreamWaitEvent(b->copy_in, b->in_free, 0));
    for (int i = 0; i < b->n; i++) {
        const LevelDims& d = b->dims[i][0];
        for (int k = 0; k < 2; k++)
            BC(cudaMemcpy2DAsync(b->stage_in + k * b->total + b->base_off[i], d.s * sizeof(float),
                                 k ? i1[i] : i0[i], (size_t)pitch * sizeof(float),
                                 d.w * sizeof(float), d.h, cudaMemcpyHostToDevice, b->copy_in));
    }
    BC(cudaEventRecord(b->in_staged, b->copy_in));
    b->up_staged = true;
    return RF_OK;
}

rf_status rf_batch_take_upload(rf_batch* b) {
    if (!b) return bfail(RF_ERR_INVALID_ARG, "rf_batch_take_upload: null batch");
    if (!b->up_staged) return bfail(RF_ERR_STATE, "rf_batch_take_upload: no frames staged");
    BC(cudaStreamWaitEvent(b->stream, b->in_staged, 0));
    // one kernel for every pair, a warp per row (128 pitched device copies
    // cost ~2 ms of the solve stream for 64 720p pairs)
    BL(launch_rows_l0(b, OpStageIn{b->stage_in, b->stage_in + b->total,
                                   plane_base(b, b->pI0(0)), plane_base(b, b->pI1(0))}));
    b->launches++;
    for (int i = 0; i < b->n; i++) b->imgs[i] = 1;
    BC(cudaEventRecord(b->in_free, b->stream));
    b->up_staged = false;
    return RF_OK;
}

rf_status rf_batch_stage_download(rf_batch* b, float* const* u, float* const* v,
                                  float* const* inv_depth, float* const* X, float* const* Y,
                                  float* const* Z, int pitch) {
    if (!b) return bfail(RF_ERR_INVALID_ARG, "rf_batch_stage_download: null batch");
    if (!b->solved) return bfail(RF_ERR_STATE, "rf_batch_stage_download: no solve has run");
    const bool recon = b->p.method != RF_METHOD_TVL1;
    if (!recon && (inv_depth || X || Y || Z))
        return bfail(RF_ERR_STATE, "rf_batch_stage_download: plain TV-L1 has no 3D output");
    for (int i = 0; i < b->n; i++)
        if (pitch < b->dims[i][0].w)
            return bfail(RF_ERR_INVALID_ARG, "rf_batch_stage_download: pitch < width");
    rf_status rs = ensure_staging(b, true);
    if (rs != RF_OK) return rs;
    const int B0 = b->base_idx();
    // the staging planes are free once the last download out of them has run
    BC(cudaStreamWaitEvent(b->stream, b->out_done, 0));
    float* const* dst[6] = {u, v, inv_depth, X, Y, Z};
    int mask = 0;
    for (int k = 0; k < 6; k++)
        if (dst[k]) mask |= 1 << k;
    // one kernel gathers the requested results (and 1/Z) of every pair
    if (mask) {
        const float* none = nullptr;
        BL(launch_rows_l0(b, OpStageOut{plane_base(b, b->res_u), plane_base(b, b->res_v),
                                        recon ? plane_base(b, B0 + P_X) : none,
                                        recon ? plane_base(b, B0 + P_Y) : none,
                                        recon ? plane_base(b, B0 + P_Z) : none, b->stage_out,
                                        b->total, mask}));
        b->launches++;
    }
    BC(cudaEventRecord(b->out_ready, b->stream));
    BC(cudaStreamWaitEvent(b->copy_out, b->out_ready, 0));
    for (int k = 0; k < 6; k++) {
        if (!dst[k]) continue;
        for (int i = 0; i < b->n; i++) {
            if (!dst[k][i]) continue;
            const LevelDims& d = b->dims[i][0];
            BC(cudaMemcpy2DAsync(dst[k][i], (size_t)pitch * sizeof(float),
                                 b->stage_out + k * b->total + b->base_off[i], d.s * sizeof(float),
                                 d.w * sizeof(float), d.h, cudaMemcpyDeviceToHost, b->copy_out));
        }
    }
    BC(cudaEventRecord(b->out_done, b->copy_out));
    return RF_OK;
}

rf_status rf_batch_wait_download(rf_batch* b) {
    if (!b) return bfail(RF_ERR_INVALID_ARG, "rf_batch_wait_download: null batch");
    if (b->out_done) BC(cudaEventSynchronize(b->out_done));
    return RF_OK;
}

rf_status rf_batch_device_results(rf_batch* b, int pair, const float** u, const float** v,
                                  const float** X, const float** Y, const float** Z) {
    if (!b || pair < 0 || pair >= b->n)
        return bfail(RF_ERR_INVALID_ARG, "rf_batch_device_results: bad argument");
    if (!b->solved) return bfail(RF_ERR_STATE, "rf_batch_device_results: no solve has run");
    const int B0 = b->base_idx();
    if (u) *u = pair_plane(b, pair, b->res_u);
    if (v) *v = pair_plane(b, pair, b->res_v);
    if (X) *X = pair_plane(b, pair, B0 + P_X);
    if (Y) *Y = pair_plane(b, pair, B0 + P_Y);
    if (Z) *Z = pair_plane(b, pair, B0 + P_Z);
    return RF_OK;
}

rf_status rf_batch_import_results(rf_batch* b, int pair, const float* u, const float* v,
                                  const float* X, const float* Y, const float* Z, int pitch) {
    if (!b || pair < 0 || pair >= b->n || !u || !v)
        return bfail(RF_ERR_INVALID_ARG, "rf_batch_import_results: bad argument");
    if (!b->solved) return bfail(RF_ERR_STATE, "rf_batch_import_results: no solve has run");
    const LevelDims d = b->dims[pair][0];
    if (pitch < d.w) return bfail(RF_ERR_INVALID_ARG, "rf_batch_import_results: pitch < width");
    const bool recon = b->p.method != RF_METHOD_TVL1;
    if (recon && (!X || !Y || !Z))
        return bfail(RF_ERR_INVALID_ARG, "rf_batch_import_results: 3D planes missing");
    const int B0 = b->base_idx();
    const struct {
        const float* src;
        int plane;
    } in[5] = {{u, b->res_u}, {v, b->res_v}, {X, B0 + P_X}, {Y, B0 + P_Y}, {Z, B0 + P_Z}};
    for (int k = 0; k < (recon ? 5 : 2); k++)
        BC(cudaMemcpy2DAsync(pair_plane(b, pair, in[k].plane), d.s * sizeof(float), in[k].src,
                             (size_t)pitch * sizeof(float), d.w * sizeof(float), d.h,
                             cudaMemcpyDeviceToDevice, b->stream));
    return RF_OK;
}

rf_status rf_batch_set_stream(rf_batch* b, void* stream) {
    if (!b) return bfail(RF_ERR_INVALID_ARG, "rf_batch_set_stream: null batch");
    BC(cudaStreamSynchronize(b->stream));
    b->stream = stream ? static_cast<cudaStream_t>(stream) : b->own;
    return RF_OK;
}

rf_status rf_batch_get_stream(rf_batch* b, void** stream) {
    if (!b || !stream) return bfail(RF_ERR_INVALID_ARG, "rf_batch_get_stream: null argument");
    *stream = static_cast<void*>(b->stream);
    return RF_OK;
}

rf_status rf_batch_synchronize(rf_batch* b) {
    if (!b) return bfail(RF_ERR_INVALID_ARG, "rf_batch_synchronize: null batch");
    BC(cudaStreamSynchronize(b->stream));
    for (cudaStream_t st : {b->copy_in, b->copy_out})
        if (st) BC(cudaStreamSynchronize(st));
    return RF_OK;
}

uint64_t rf_batch_kernel_launches(const rf_batch* b) { return b ? b->launches : 0; }

}  // extern "C"
