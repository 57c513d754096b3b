// Launch interface of the solver kernels (rf_kernels.cu), used by the host
// orchestration (rf_solver.cu) and the kernel-level C entry points.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

#include "rf_math.cuh"

struct rf_params;

namespace rf {

struct LevelDims {
    int w, h, s;
};

// Scalar solver weights in the exact float forms the kernels use.
struct Weights {
    float lambda;
    float alpha_tv, alpha_proj, alpha_fn;
    float A;          // alpha_tv + alpha_proj (data-term denominator)
    float fac;        // tau / thetaTv (dual step), or tau / theta in plain mode
    float lambdaf, lambdams;
    float proj_den;   // lambdaf + alpha_proj
    float theta;      // plain TV-L1 theta
};

// Fields of one ReconFlow inner iteration.
struct ReconFields {
    const float* u;
    const float* v;
    float* duhat;     // in place: read at the pixel, written by the data step
    float* dvhat;
    float* pu1;       // dual field, in place
    float* pu2;
    float* pv1;
    float* pv2;
    float* uproj;     // in place
    float* vproj;
    float* sku;       // in place
    float* skv;
    const float* Ix;
    const float* Iy;
    const float* Iz;
    float* X;         // post-cleanup 3D state (flat level-0 buffer)
    float* Y;
    float* Z;
    float* X1;        // Solve3d output (before median / cleanup)
    float* Y1;
    float* Z1;
    const float* uc;  // buffer read only when uc_from_buffer
    const float* vc;
    const float* ufn; // prior flow at this level (methods 17 / 20)
    const float* vfn;
    const float* mask;
    long long extent; // floats every field pointer may be indexed with: [0, extent)
};

// A field element of the inner iteration, f.name[i].  Built with
// RF_BOUNDS_CHECK, every index is checked against [0, f.extent): an index
// outside is counted (with the first offender kept) and the access goes to
// a sink cell instead of memory, so a bad index is reported, never used.
// Read the counts with rf_debug_bounds.
#ifdef RF_BOUNDS_CHECK
static __device__ unsigned long long g_oob_count;
static __device__ long long g_oob_first;
static __device__ float g_oob_sink;

__device__ __forceinline__ float& rf_checked(float* p, long long i, long long n) {
    if (i < 0 || i >= n) {
        if (atomicAdd(&g_oob_count, 1ull) == 0ull) g_oob_first = i;
        return g_oob_sink;
    }
    return p[i];
}
__device__ __forceinline__ const float& rf_checked(const float* p, long long i, long long n) {
    if (i < 0 || i >= n) {
        if (atomicAdd(&g_oob_count, 1ull) == 0ull) g_oob_first = i;
        return g_oob_sink;
    }
    return p[i];
}
#define RF_AT(f, name, idx) rf_checked((f).name, (long long)(idx), (f).extent)

// this translation unit's counts (and reset them)
static inline unsigned long long rf_oob_take(long long* first) {
    unsigned long long c = 0;
    long long fi = -1;
    cudaDeviceSynchronize();
    cudaMemcpyFromSymbol(&c, g_oob_count, sizeof c);
    cudaMemcpyFromSymbol(&fi, g_oob_first, sizeof fi);
    const unsigned long long zero = 0;
    cudaMemcpyToSymbol(g_oob_count, &zero, sizeof zero);
    if (first && c) *first = fi;
    return c;
}
#else
#define RF_AT(f, name, idx) (f).name[idx]
#endif

// Per-level camera constants of one pair (K pyramid, P = K0 [R0|t0],
// Q = K1 [R1|t1], float copies), fix_quirks as rf_params.
void camera_level_consts(const double* K0, const double* K1, int L, float scale, int fix_quirks,
                         const double* R0, const double* t0, const double* R1, const double* t1,
                         LevelConsts* out);

// Kernel weights of a parameter block (the exact float forms the kernels use).
Weights solver_weights(const rf_params* p);

// Records `msg` as the calling thread's rf_last_error_string(); returns st.
int set_last_error(int st, const char* msg);

int launch_convert(const void* in, int type, int w, int h, int in_pitch, float* out, int s,
                   cudaStream_t st);
int launch_downscale2(const float* a, const float* b, LevelDims fine, LevelDims coarse,
                      float* oa, float* ob, cudaStream_t st);
int launch_downscale(const float* src, LevelDims fine, LevelDims coarse, float scale, bool scaled,
                     float* out, cudaStream_t st);
int launch_warp(const float* I1, const float* u, const float* v, LevelDims d, float* out,
                cudaStream_t st);
// Every inner iteration of a warp of a small level in one launch of a
// 16-CTA thread-block cluster (barriers between the half-steps); results
// equal n_iters x (launch_recon_a, launch_recon_b).
int launch_recon_cluster(const ReconFields& f, const LevelConsts* lc, const Weights& wt,
                         LevelDims d, int n_iters, bool uc_from_buffer, int prior,
                         cudaStream_t st);
// RF_BOUNDS_CHECK builds: the out-of-range field accesses counted by this
// file's kernels (and those of the batched kernels), cleared when read; 0 in
// other builds.  launch_oob_selftest makes one checked access one past a
// field's extent (redirected to the sink: nothing outside is touched).
unsigned long long kernels_oob_take(long long* first);
unsigned long long batch_oob_take(long long* first);
int launch_oob_selftest();
// whether a 16-CTA cluster of that kernel can run on the current device
bool cluster_supported();
// WarpImage + ComputeDerivatives in one launch; the warped image stays on chip
int launch_warp_deriv(const float* I0, const float* I1, const float* u, const float* v,
                      LevelDims d, float* Ix, float* Iy, float* Iz, cudaStream_t st);
int launch_derivatives(const float* I0, const float* I1w, LevelDims d, float* Ix, float* Iy,
                       float* Iz, cudaStream_t st);
// `block` = the level's tile (default 32 x 8; at most 256 threads)
int launch_recon_a(const ReconFields& f, const LevelConsts* lc, const Weights& wt, LevelDims d,
                   bool first, bool uc_from_buffer, int prior, cudaStream_t st,
                   dim3 block = dim3(32, 8));
int launch_recon_b(const ReconFields& f, const Weights& wt, LevelDims d, bool first,
                   cudaStream_t st, dim3 block = dim3(32, 8));
int launch_plain_data(float* duhat, float* dvhat, const float* pu1, const float* pu2,
                      const float* pv1, const float* pv2, const float* Ix, const float* Iy,
                      const float* Iz, const Weights& wt, LevelDims d, bool first,
                      cudaStream_t st);
int launch_plain_tv(const float* duhat, const float* dvhat, float* pu1, float* pu2, float* pv1,
                    float* pv2, const Weights& wt, LevelDims d, bool first, cudaStream_t st);
// out = u + median5(duhat) (out may alias u)
int launch_median_add(const float* duhat, const float* dvhat, const float* u, const float* v,
                      float* ou, float* ov, LevelDims d, cudaStream_t st);
// 0 if the last kernel launch on this thread succeeded, else 1; a failure's
// error is kept for last_launch_error (cudaGetLastError clears it).
int launch_status();
// The CUDA error of the last launch helper on this thread that returned
// nonzero (cudaSuccess if none since the previous call); reading it clears it.
cudaError_t last_launch_error();

int launch_median5(const float* u, const float* v, float* ou, float* ov, LevelDims d,
                   cudaStream_t st);
int launch_median3d(const float* X, const float* Y, const float* Z, float* X1, float* Y1,
                    float* Z1, LevelDims d, cudaStream_t st);
int launch_solve_uc(const float* X, const float* Y, const float* Z, const LevelConsts* lc,
                    LevelDims d, float* uc, float* vc, cudaStream_t st);
// Upscale n fields by one pyramid step; scales[i] multiplies field i.
int launch_upscale_fields(int n, const float* const* src, float* const* dst, const float* scales,
                          LevelDims coarse, LevelDims fine, cudaStream_t st);
int launch_upscale(const float* src, LevelDims coarse, LevelDims fine, float scale, float* out,
                   cudaStream_t st);
int launch_inv_depth(const float* Z, LevelDims d, float* out, cudaStream_t st);
// Arguments of one solution-energy evaluation (float copies of the pose
// and intrinsics, as the per-pixel terms use them).
struct EnergyArgs {
    const float *I0, *I1, *u, *v, *X, *Y, *Z;
    float R1f[9], t1f[3], fxf, cxf, cyf;
    float lambda, alpha_proj;
    int recon;
};
EnergyArgs energy_args(const float* I0, const float* I1, const float* u, const float* v,
                       const float* X, const float* Y, const float* Z, float lambda,
                       float alpha_proj, const double* R1, const double* t1, const double* K1,
                       int recon);

// One evaluation of a batched energy launch: its blocks are
// [first_block, first_block + nblocks) of the launch.
struct EnergyJob {
    EnergyArgs a;
    LevelDims d;
    int nblocks, first_block;
    double* partial;  // nblocks doubles
    double* out;
};

constexpr int kEnergyMaxBlocks = 1024;
// blocks of one evaluation of a level of these dimensions
int energy_blocks(LevelDims d);
// every job of the device array `jobs` (blocks in job order, total_blocks in
// all): the same partials and sums as launch_energy of each job alone
int launch_energy_jobs(const EnergyJob* jobs, int n, int total_blocks, int max_blocks,
                       cudaStream_t st);

// Solution energy on one level (data + TV + reprojection) into *out (device
// double); `partial` holds `nblocks` doubles.
int launch_energy(const float* I0, const float* I1, const float* u, const float* v,
                  const float* X, const float* Y, const float* Z, LevelDims d, float lambda,
                  float alpha_proj, const double* R1, const double* t1, const double* K1,
                  int recon, double* partial, int nblocks, double* out, cudaStream_t st);
int launch_remove_edge(const float* X, const float* Y, const float* Z, int range, float max_area,
                       LevelDims d, float* X1, float* Y1, float* Z1, cudaStream_t st);
int launch_flow_color(const float* u, const float* v, LevelDims d, float flow_scale, float* rgb,
                      cudaStream_t st);

}  // namespace rf
