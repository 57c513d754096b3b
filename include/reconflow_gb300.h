/*
 * reconflow_gb300 — C ABI of the GB300 (sm_103a) simultaneous optical-flow and
 * depth solver.
 *
 * This is the drop-in boundary for the reference's ReconFlow / CudaFlow class
 * surface (menandro/Reconflow, reconflow/Reconflow.h:9-160 and
 * reconflow/Cudaflow.h:17-362).  Every entry point is plain C: handles,
 * pointers, sizes and status codes; no CUDA, OpenCV or torch types appear in
 * the signatures.  Each declaration names the reference member it replaces.
 *
 * Layout: every image and field is a row-major float32 plane with `stride`
 * elements per row, stride = width aligned up to `stride_alignment` (32), as
 * the reference pads its cv::Mat buffers (test_reconflow/main.cpp:57-67).
 * Host buffers passed to the upload / download calls have a caller-chosen
 * row pitch in elements (pass rf_stride(h) to match the reference exactly).
 *
 * Errors: every call returns an rf_status; the message of the last failure on
 * the calling thread is available from rf_last_error_string().  The reference
 * returns 0 unconditionally and aborts inside checkCudaErrors instead.
 *
 * Threading: handles share no global state; one host thread per handle.  All
 * device work of a handle is ordered on the handle's CUDA stream.
 */
#ifndef RECONFLOW_GB300_H
#define RECONFLOW_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RF_API __attribute__((visibility("default")))

typedef enum rf_status {
    RF_OK = 0,
    RF_ERR_INVALID_ARG = 1,  /* bad size, null pointer, mismatched dims */
    RF_ERR_UNSUPPORTED = 2,  /* method / input type not implemented */
    RF_ERR_CUDA = 3,         /* a CUDA runtime call failed */
    RF_ERR_OOM = 4,          /* device or pinned allocation failed */
    RF_ERR_STATE = 5,        /* call out of order (e.g. solve before upload) */
    RF_ERR_NO_DEVICE = 6     /* no CUDA device visible */
} rf_status;

/* Method codes, numerically equal to the reference's constants
 * (Cudaflow.h:20-28, Reconflow.h:46-52). */
enum {
    RF_METHOD_TVL1 = 0,            /* CudaFlow::METHOD_TVL1, plain TV-L1 flow */
    RF_METHODR_TVL1_MS = 14,       /* ReconFlow::METHODR_TVL1_MS, flow + 3D */
    RF_METHODR_TVL1_MS_FN = 17,    /* + dense prior flow term */
    RF_METHODR_TVL1_MS_FNSPARSE = 20 /* + masked (sparse) prior flow term */
};

/* Input image types (the reference's cvType argument, Cudaflow.cu:288-311). */
enum {
    RF_INPUT_F32 = 0,   /* CV_32F gray, used as is (rgbToGray.cu:66-77) */
    RF_INPUT_RGB8 = 1,  /* CV_8UC3, gray = (r+g+b)/3/256 (rgbToGray.cu:3-19) */
    RF_INPUT_U8 = 2,    /* CV_8U, gray = v/256 (rgbToGray.cu:21-36) */
    RF_INPUT_U16 = 3    /* CV_16U, gray = v/65536 (rgbToGray.cu:38-52) */
};

/* Reference behaviours that can be switched off (bit flags of fix_quirks).
 * 0 reproduces the reference. */
enum {
    /* pK[l] (l >= 1) starts from zeros, so K[2][2] = 0 and the third rows of
     * P and Q vanish at coarse levels (Reconflow.cu:98-110).  Set to use 1. */
    RF_FIX_K_PYRAMID = 1,
    /* X, Y, Z are not resampled at a level change; the coarse flat arrays are
     * re-read with the finer stride (Reconflow.cu:424-458).  Set to resample
     * them bilinearly instead. */
    RF_FIX_XYZ_UPSCALE = 2
};

/* Solver parameters: the arguments of CudaFlow::initialize (Cudaflow.h:36-46)
 * and ReconFlow::initializeR (Reconflow.h:67-70) in one POD block. */
typedef struct rf_params {
    int width, height;        /* level-0 image size */
    int channels;             /* informational (reference `channels`) */
    int input_type;           /* RF_INPUT_* */
    int n_levels;             /* pyramid levels */
    float scale;              /* pyramid factor fScale (2.0) */
    int method;               /* RF_METHOD* */
    float lambda;             /* data weight */
    float lambdagrad;         /* accepted, unused by the implemented methods */
    float lambdaf;            /* 3D / epipolar coupling weight */
    float lambdams;           /* minimal-surface-area weight */
    float alpha_tv;           /* ReconFlow: thetaTv = 1/alpha_tv */
    float alpha_proj;         /* projection coupling */
    float alpha_fn;           /* prior-flow weight (methods 17, 20) */
    float tau;                /* dual step */
    float theta;              /* plain TV-L1 coupling (method 0) */
    int n_warp_iters;
    int n_solver_iters;
    int stride_alignment;     /* 32 in the reference */
    int block_width, block_height; /* reference ctor launch shape; accepted, unused */
    int fix_quirks;           /* RF_FIX_* bit flags, 0 = reference behaviour */
} rf_params;

typedef struct rf_handle rf_handle;

/* Defaults of ReconFlow::initializeR (Reconflow.cu:15-18) for
 * method != RF_METHOD_TVL1, of CudaFlow::initialize (Cudaflow.cu:16-18)
 * otherwise; width/height/n_levels are left 0 for the caller. */
RF_API rf_status rf_params_default(rf_params* p, int method);

/* ReconFlow::ReconFlow + initializeR / CudaFlow::initialize
 * (Reconflow.cu:9-63, Cudaflow.cu:99-269): validates the parameters and
 * allocates every device buffer once, at level-0 size. */
RF_API rf_status rf_create(const rf_params* p, rf_handle** out);

/* ~ReconFlow / ~CudaFlow (Reconflow.cu:479-509, Cudaflow.cu:873-978). */
RF_API rf_status rf_destroy(rf_handle* h);

/* CudaFlow::iAlignUp(width) (Cudaflow.cu:984-994): the row stride in elements. */
RF_API int rf_stride(const rf_handle* h);

/* Level sizes of the pyramid (Cudaflow.cu:146-171); arrays of n_levels ints. */
RF_API rf_status rf_pyramid_dims(const rf_handle* h, int* W, int* H, int* S);

/* ReconFlow::setCameraMatrices(K0, K1) (Reconflow.cu:78-116): 3x3 row-major
 * intrinsics of both cameras. */
RF_API rf_status rf_set_cameras(rf_handle* h, const double K0[9], const double K1[9]);

/* CudaFlow::copyImagesToDevice (Cudaflow.cu:288-311): host images of the
 * handle's input type, `pitch` elements per row (pixels for RGB8). */
RF_API rf_status rf_upload_images(rf_handle* h, const void* i0, const void* i1, int pitch);

/* Same from device memory (no host copy; e.g. frames already in HBM). */
RF_API rf_status rf_upload_images_device(rf_handle* h, const void* i0, const void* i1, int pitch);

/* CudaFlow::copySparseOpticalFlowToDevice(u, v[, mask]) /
 * copyInitialOpticalFlowToDevice (Cudaflow.cu:327-343): the prior flow of
 * methods 17 and 20; mask may be NULL (all ones). */
RF_API rf_status rf_set_prior_flow(rf_handle* h, const float* u, const float* v,
                                   const float* mask, int pitch);

/* ReconFlow::solveR(R0, t0, R1, t1, flowScale) -> solveReconFlow
 * (Reconflow.cu:134-466).  R row-major 3x3, t 3x1, camera j maps a world
 * point X to R_j X + t_j.  R0/t0 may be NULL (identity / zero, as
 * solveR(R1, t1) does at Reconflow.cu:138-144).  Asynchronous on the
 * handle's stream. */
RF_API rf_status rf_solve(rf_handle* h, const double R0[9], const double t0[3],
                          const double R1[9], const double t1[3]);

/* CudaFlow::solveOpticalFlow (Cudaflow.cu:394-621): plain TV-L1 flow. */
RF_API rf_status rf_solve_flow(rf_handle* h);

/* Warm-started solve (no reference counterpart): the schedule begins at
 * pyramid `level` from the given flow u, v and 3D points X, Y, Z on that
 * level (planes of the level's size, `pitch` elements per row, host memory,
 * or device memory when on_device != 0), with uproj = u, sk = 0 and the
 * projection of the given points; levels `level`..0 then run `warps` warps of
 * `iters` iterations (-1 = the handle's counts).  Method 14 only.  Used to
 * refine a coarse estimate, e.g. a learned prediction. */
RF_API rf_status rf_solve_warm(rf_handle* h, const double R0[9], const double t0[3],
                               const double R1[9], const double t1[3], int level, const float* u,
                               const float* v, const float* X, const float* Y, const float* Z,
                               int pitch, int on_device, int warps, int iters);

/* Plain TV-L1 counterpart of rf_solve_warm (flow only). */
RF_API rf_status rf_solve_flow_warm(rf_handle* h, int level, const float* u, const float* v,
                                    int pitch, int on_device, int warps, int iters);

/* Energy of the last solution (no reference counterpart), summed over the
 * level-0 pixels: lambda * |I1(x + u) - I0(x)| + |grad u| +
 * |grad v| (+ alpha_proj / 2 * min(|(u, v) - uc(X)|^2, 1) for ReconFlow, uc
 * the projection of the solved point as SolveUc computes it; the
 * reprojection residual is truncated at 1 px^2, so a few pixels whose point
 * projects near infinity cannot dominate the sum).  Per-pixel terms in FP32;
 * each GPU thread adds its own few dozen pixels in FP32, and the thread sums
 * are added in double in a fixed order.  Blocking. */
RF_API rf_status rf_energy(rf_handle* h, double* energy);

/* CudaFlow::copyOpticalFlowToHost(u, v) (Cudaflow.cu:320-325). Blocking. */
RF_API rf_status rf_download_flow(rf_handle* h, float* u, float* v, int pitch);

/* ReconFlow::copy3dToHost(X, Y, Z) (Reconflow.cu:65-70). Blocking. */
RF_API rf_status rf_download_points(rf_handle* h, float* X, float* Y, float* Z, int pitch);

/* Inverse depth 1/Z of camera 0 (no reference counterpart: derived from
 * d_Z, Reconflow.h:26).  Blocking. */
RF_API rf_status rf_download_inv_depth(rf_handle* h, float* inv_depth, int pitch);

/* CudaFlow::copyOpticalFlowToHost(u, v, uvrgb) colour part
 * (Cudaflow.cu:313-318) via FlowToHSV (flowToHSV.cu:194-311): float RGB
 * triples (B, G, R order as the reference's float3 x, y, z), 3*pitch floats
 * per row. */
RF_API rf_status rf_download_flow_color(rf_handle* h, float flow_scale, float* rgb, int pitch);

/* ReconFlow::removeEdgeArtifacts3D (Reconflow.cu:468-477). */
RF_API rf_status rf_remove_edge_artifacts(rf_handle* h, int surface_width, float max_area);

/* Device pointers of the results (level-0 planes, rf_stride() per row);
 * valid until the next solve or destroy.  Any pointer argument may be NULL. */
RF_API rf_status rf_device_results(rf_handle* h, const float** u, const float** v,
                                   const float** X, const float** Y, const float** Z);

/* Levels of at most max_px pixels run all inner iterations of a warp in
 * one launch of a 16-CTA thread-block cluster with cluster barriers between
 * the half-steps, instead of two launches per iteration (the same values:
 * the per-pixel code is shared).  Applies to every single-pair handle of the
 * process from its next solve; 0 = never; negative = the default (0, or
 * RF_CLUSTER_PX from the environment).  No reference
 * counterpart. */
RF_API rf_status rf_set_cluster_pixels(long long max_px);
/* Debug builds compiled with RF_BOUNDS_CHECK (reconflow_gb300/build.py
 * --bounds-check, a separate library): every field access of the inner
 * iteration is checked against its plane; an index outside is counted and
 * redirected to a sink cell instead of touching memory.  rf_debug_bounds
 * returns (and clears) the count and the first offending index;
 * rf_debug_bounds_selftest makes one such access on purpose.  Other builds:
 * RF_ERR_UNSUPPORTED.  No reference counterpart. */
RF_API rf_status rf_debug_bounds(unsigned long long* count, long long* first);
RF_API rf_status rf_debug_bounds_selftest(void);
/* Tile shape of the inner-iteration kernels at each pyramid level
 * (tile_w[l] x tile_h[l] pixels, one thread each; 32 .. 256 threads, a
 * multiple of 32; default 32 x 8), as reconflow_gb300/autotune.py picks
 * them.  No reference counterpart (the reference's BlockWidth / BlockHeight
 * constructor arguments, Reconflow.h:12, play this role for all kernels).
 * Results do not depend on it. */
RF_API rf_status rf_set_tiles(rf_handle* h, const int* tile_w, const int* tile_h);

/* Use a caller's CUDA stream (cudaStream_t passed as void*; NULL = the
 * handle's own stream). */
RF_API rf_status rf_set_stream(rf_handle* h, void* stream);
RF_API rf_status rf_synchronize(rf_handle* h);

/* Pinned host memory for fast uploads/downloads. */
RF_API rf_status rf_host_alloc(size_t bytes, void** ptr);
RF_API rf_status rf_host_free(void* ptr);

/* Timing hook (no reference counterpart): after a solve, time each of the
 * two inner-iteration kernels at pyramid level `level` on the handle's
 * stream: `n_iters` launches of one kernel back to back, captured in a CUDA
 * graph as the solve captures them, the graph replay timed with CUDA events;
 * returns the mean time per launch in milliseconds (ms[0] = data /
 * projection / triangulation kernel, ms[1] = dual / median / clean-up
 * kernel; plain TV-L1: data, dual).  Changes the solver state; results of
 * the last solve are no longer valid afterwards. */
RF_API rf_status rf_profile_iterations(rf_handle* h, int level, int n_iters, float* ms);

/* Kernel launches issued by this handle so far (count of this library's
 * kernels, graph nodes included). */
RF_API uint64_t rf_kernel_launches(const rf_handle* h);

/* Message of the last failing call on this thread ("" if none). */
RF_API const char* rf_last_error_string(void);

/* Library version string. */
RF_API const char* rf_version(void);

/* ------------------------------------------------------------------------
 * Batched solve (no reference counterpart; the reference solves one pair per
 * object).  Many independent frame pairs, each with its own size, cameras and
 * pose, share one parameter block (methods 0 and 14, float32 gray input) and
 * are solved together: every step of the schedule is one launch covering all
 * pairs, captured in one CUDA graph.  A pair's results are bit-identical to
 * solving it alone with rf_solve / rf_solve_flow.  The per-pair calls take
 * the single-pair entry points' arguments, and through them the reference's:
 * rf_batch_set_cameras ~ setCameraMatrices (Reconflow.cu:78-116),
 * rf_batch_upload_images ~ copyImagesToDevice (Cudaflow.cu:288-311),
 * rf_batch_solve ~ solveR (Reconflow.cu:134-466), rf_batch_solve_flow ~
 * solveOpticalFlow (Cudaflow.cu:394-621), rf_batch_download_flow ~
 * copyOpticalFlowToHost (Cudaflow.cu:320-325), rf_batch_download_points ~
 * copy3dToHost (Reconflow.cu:65-70).
 * ---------------------------------------------------------------------- */
typedef struct rf_batch rf_batch;

RF_API rf_status rf_batch_create(const rf_params* p, int n_pairs, const int* widths,
                                 const int* heights, rf_batch** out);
RF_API rf_status rf_batch_destroy(rf_batch* b);
/* stride (elements per row) of pair `pair`'s planes */
RF_API int rf_batch_stride(const rf_batch* b, int pair);
RF_API rf_status rf_batch_set_cameras(rf_batch* b, int pair, const double K0[9],
                                      const double K1[9]);
RF_API rf_status rf_batch_upload_images(rf_batch* b, int pair, const float* i0, const float* i1,
                                        int pitch);
RF_API rf_status rf_batch_upload_images_device(rf_batch* b, int pair, const float* i0,
                                               const float* i1, int pitch);
/* R0, t0 may be NULL (identity / zero for every pair); otherwise arrays of
 * n_pairs x 9 and n_pairs x 3 doubles, pair-major. */
RF_API rf_status rf_batch_solve(rf_batch* b, const double* R0, const double* t0, const double* R1,
                                const double* t1);
RF_API rf_status rf_batch_solve_flow(rf_batch* b);
/* Warm-started batch solve (no reference counterpart): every pair starts at
 * pyramid level `level` from the planes rf_batch_warm_planes returns (flow
 * u, v and 3D points X, Y, Z at that level, the level's stride per row,
 * written by the caller on the batch's stream beforehand), then runs
 * `warps` x `iters` at that level and every finer one, like rf_solve_warm
 * does for one pair.  Poses as in rf_batch_solve. */
RF_API rf_status rf_batch_solve_warm(rf_batch* b, const double* R0, const double* t0,
                                     const double* R1, const double* t1, int level, int warps,
                                     int iters);
/* Energy of every pair's last ReconFlow solution (as rf_energy defines it
 * for one pair); out: n_pairs doubles on the host.  Synchronizes. */
RF_API rf_status rf_batch_energies(rf_batch* b, double* out);
/* rf_batch_energies without the wait: the evaluation and the copy of the n
 * values into `out` are queued on the batch's stream and the call returns
 * (with `out` in pinned host memory, rf_host_alloc, it returns at once);
 * the values are valid once the stream has reached them (rf_batch_synchronize
 * or a wait on the stream).  Lets a serving loop queue the next batch's
 * solve before it reads this one's energies.  No reference counterpart. */
RF_API rf_status rf_batch_energies_async(rf_batch* b, double* out);
/* rf_batch_solve_warm with its own warps / iterations at each level:
 * warps[l], iters[l] for l = 0 .. level (level 0 = the finest). */
RF_API rf_status rf_batch_solve_warm_levels(rf_batch* b, const double* R0, const double* t0,
                                            const double* R1, const double* t1, int level,
                                            const int* warps, const int* iters);
/* Tile shape of each pyramid level (tile_w[l] x tile_h[l] pixels, one
 * thread each; 32 .. 256 threads, a multiple of 32; default 32 x 8), as
 * reconflow_gb300/autotune.py picks them.  Results do not depend on it. */
RF_API rf_status rf_batch_set_tiles(rf_batch* b, const int* tile_w, const int* tile_h);
/* Timing hook (no reference counterpart): after a ReconFlow solve, the mean
 * time in milliseconds of one launch of each inner-iteration kernel over
 * every pair at `level` with the current tiles (ms[0] data / projection /
 * triangulation, ms[1] dual / median / clean-up; n_iters launches back to
 * back in a CUDA graph, CUDA events).  Invalidates the last solve. */
RF_API rf_status rf_batch_profile_level(rf_batch* b, int level, int n_iters, float* ms);
/* Device pointers of pair `pair`'s image planes at pyramid `level` (level 0
 * = the uploaded frames; coarser levels are filled by the next solve). */
RF_API rf_status rf_batch_image_planes(rf_batch* b, int pair, int level, const float** I0,
                                       const float** I1);
/* Device pointers of pair `pair`'s warm-start input planes (level-0-sized
 * planes; any pointer argument may be NULL). */
RF_API rf_status rf_batch_warm_planes(rf_batch* b, int pair, float** u, float** v, float** X,
                                      float** Y, float** Z);
RF_API rf_status rf_batch_download_flow(rf_batch* b, int pair, float* u, float* v, int pitch);
RF_API rf_status rf_batch_download_points(rf_batch* b, int pair, float* X, float* Y, float* Z,
                                          int pitch);
RF_API rf_status rf_batch_download_inv_depth(rf_batch* b, int pair, float* inv_depth, int pitch);
/* Every pair's frames at once (host arrays of n_pairs host pointers, one
 * pitch); asynchronous on the batch's stream like rf_batch_upload_images. */
RF_API rf_status rf_batch_upload_all(rf_batch* b, const float* const* i0, const float* const* i1,
                                     int pitch);
/* Every pair's results at once: host arrays of n_pairs host pointers per
 * output (an array, or an entry, may be NULL to skip it), one pitch; the
 * copies are queued together and the call synchronizes once.  Blocking. */
RF_API rf_status rf_batch_download_all(rf_batch* b, float* const* u, float* const* v,
                                       float* const* inv_depth, float* const* X,
                                       float* const* Y, float* const* Z, int pitch);
/* Pipelined transfers for a serving loop: the frames of the next solve go
 * up, and the results of the last solve come down, while a solve runs.
 * Each direction has its own copy stream and a device staging area laid
 * out like the batch's planes (made on first use).
 *
 * rf_batch_stage_upload queues every pair's frames (host arrays as for
 * rf_batch_upload_all) into the staging area and returns at once; the host
 * frames must stay unchanged until the solve that uses them has finished.
 * rf_batch_take_upload makes the batch's stream wait for them and copies
 * them into the pairs' frame planes (device to device), after which the
 * next rf_batch_stage_upload may start.  RF_ERR_STATE if frames are staged
 * twice without a take, or taken without being staged.
 *
 * rf_batch_stage_download copies the last solve's results (arguments as
 * for rf_batch_download_all) into the staging area on the batch's stream,
 * then to the host arrays on the copy stream, and returns at once: the next
 * solve may be queued immediately.  rf_batch_wait_download blocks until
 * the last staged download has reached the host.  The results are the same
 * bytes rf_batch_download_all writes.
 *
 * The calls return at once only when the host arrays are pinned
 * (rf_host_alloc, or cudaHostRegister on the caller's memory): with pageable
 * arrays the CUDA runtime stages the copies through its own buffers, so the
 * upload blocks while it copies and the download blocks until the solve it
 * follows has finished, and nothing overlaps. */
RF_API rf_status rf_batch_stage_upload(rf_batch* b, const float* const* i0,
                                       const float* const* i1, int pitch);
RF_API rf_status rf_batch_take_upload(rf_batch* b);
RF_API rf_status rf_batch_stage_download(rf_batch* b, float* const* u, float* const* v,
                                         float* const* inv_depth, float* const* X,
                                         float* const* Y, float* const* Z, int pitch);
RF_API rf_status rf_batch_wait_download(rf_batch* b);
RF_API rf_status rf_batch_device_results(rf_batch* b, int pair, const float** u, const float** v,
                                         const float** X, const float** Y, const float** Z);
/* Replace one pair's solution (u, v and, for ReconFlow methods, X, Y, Z)
 * with device planes of `pitch` floats per row, on the batch's stream: a
 * pair solved again outside the batch (the learned path's plain fallback)
 * then is what downloads, energies and later warm starts read.  No
 * reference counterpart. */
RF_API rf_status rf_batch_import_results(rf_batch* b, int pair, const float* u, const float* v,
                                         const float* X, const float* Y, const float* Z,
                                         int pitch);
RF_API rf_status rf_batch_set_stream(rf_batch* b, void* stream);
/* The stream the batch's work is enqueued on (the one set by
 * rf_batch_set_stream, else the batch's own non-blocking stream): kernels
 * that feed the batch (warm-start features, network, state) go on it so
 * that they are ordered with the solve.  No reference counterpart. */
RF_API rf_status rf_batch_get_stream(rf_batch* b, void** stream);
RF_API rf_status rf_batch_synchronize(rf_batch* b);
RF_API uint64_t rf_batch_kernel_launches(const rf_batch* b);

/* ------------------------------------------------------------------------
 * Learned warm start network (no reference counterpart): a small BF16
 * convolutional encoder-decoder run and trained with this library's own
 * tensor-core kernels.  Tensors are float32 NHWC in device memory.  Input:
 * 16 channels at the network's input resolution H x W (I0, I1, x and y in
 * [-0.5, 0.5], rotation vector x 30, translation x 10, zeros).  Outputs: 8
 * channels (u, v, inverse depth, then unused) at (H+1)/2 x (W+1)/2 ("out16")
 * and at H x W ("out8").
 * ---------------------------------------------------------------------- */
typedef struct rf_cnn rf_cnn;

/* Allocates for up to max_batch samples of up to height x width pixels;
 * weights He-initialised from `seed`. */
RF_API rf_status rf_cnn_create(int max_batch, int height, int width, unsigned long long seed,
                               rf_cnn** out);
RF_API rf_status rf_cnn_destroy(rf_cnn* c);
RF_API int rf_cnn_num_params(const rf_cnn* c);
RF_API rf_status rf_cnn_set_stream(rf_cnn* c, void* stream);
/* FP32 master weights (host, rf_cnn_num_params floats) */
RF_API rf_status rf_cnn_get_params(rf_cnn* c, float* host);
RF_API rf_status rf_cnn_set_params(rf_cnn* c, const float* host);
/* gradient of the last rf_cnn_backward (host, rf_cnn_num_params floats) */
RF_API rf_status rf_cnn_get_grads(rf_cnn* c, float* host);
RF_API rf_status rf_cnn_forward(rf_cnn* c, const float* input, int batch, int height, int width,
                                float* out16, float* out8);
/* forward + masked L1 loss (channel weights w[0..2] for u, v, inverse depth,
 * each scale averaged over its pixels) + backward; *loss (host) may be NULL */
RF_API rf_status rf_cnn_backward(rf_cnn* c, const float* input, const float* tgt16,
                                 const float* mask16, const float* tgt8, const float* mask8,
                                 int batch, int height, int width, const float* w, double* loss);
RF_API rf_status rf_cnn_adam_step(rf_cnn* c, float lr, float beta1, float beta2, float eps);
RF_API uint64_t rf_cnn_kernel_launches(const rf_cnn* c);
/* Whether a tensor-core launch of this network gave up on a bounded
 * mbarrier wait since the last call (its outputs are then undefined): sets
 * *gave_up to 1 or 0 and clears the flag.  Synchronizes the network's
 * stream. */
RF_API rf_status rf_cnn_status(rf_cnn* c, int* gave_up);
/* Test hook for the bounded waits (no reference counterpart): polls >= 0
 * caps the first ring-slot wait of every tensor-core CTA at that many polls
 * (0: it gives up at once, while the MMAs it waited for still complete), so
 * a test can drive the give-up path without a wait that never ends; the
 * launches then report through rf_cnn_status and write no outputs.  polls < 0
 * restores the normal limit. */
RF_API rf_status rf_cnn_set_test_wait_limit(rf_cnn* c, int polls);

/* Warm-start network input (no reference counterpart): for n frame pairs
 * (device planes of w0 x h0 float32 pixels, s0 floats per row; host arrays
 * of n device pointers), the 16-channel NHWC features on the grid of
 * (w0/factor) x (h0/factor) pixels, pair-major in `out` (device):
 * channels 0, 1 = the factor x factor box averages of I0, I1 minus 0.5;
 * 2..13 = 10 |I1(x'(rho_k)) - I0(x)| for inverse depths rho_k = 0.05 k
 * (x'(rho) = the camera-1 image of the camera-0 pixel x at inverse depth
 * rho, X1 = R X + t, I1 bilinear and clamped); 14, 15 = d x'/d rho at
 * rho = 0.25 in coarse pixels per 10 1/m.  K (level-0 intrinsics), R, t:
 * n x 9, n x 9 and n x 3 doubles on the host.  Runs on `stream`. */
RF_API rf_status rf_ws_features(int n, const float* const* I0, const float* const* I1, int w0,
                                int h0, int s0, int factor, const double* K, const double* R,
                                const double* t, float* out, void* stream);
/* Temporal warm start for frame sequences (no reference counterpart): for n
 * pairs, frame k's inverse depth on the wn x hn grid of `factor` x `factor`
 * level-0 cells (factor 1 .. 32) from frame k-1's solved depth Z (host array
 * of n device planes, w x h pixels, s floats per row; non-finite or <= 0 =
 * unknown): each pixel lifted to 3D with K (n x 9 host doubles, level 0),
 * moved by R, t (n x 9, n x 3: camera k-1 -> camera k, the previous pair's
 * pose) and projected; the points landing at 0.5 .. 50 m give each cell the
 * mean of their inverse depths (fixed-point sums: reproducible bit for bit),
 * cells nothing reaches take the median of the filled cells (0 if none).
 * Written to channel `channel` of the pair-major NHWC map `grid` (device,
 * n x hn x wn x channels floats), which rf_ws_state reads as it reads the
 * network's output (channel 2).  `scratch`: device, 2 x n x wn x hn unsigned
 * ints (cleared here). */
RF_API rf_status rf_ws_propagate(int n, const float* const* Z, int w, int h, int s,
                                 const double* K, const double* R, const double* t, int factor,
                                 int wn, int hn, int channels, int channel, float* grid,
                                 unsigned int* scratch, void* stream);
/* Warm-start state from the network's inverse depth (channel 2 of an NHWC
 * map of `channels` channels on a wn x hn grid per pair, device): for each
 * pixel of a w x h pyramid level (s floats per row) the inverse depth
 * bilinearly upsampled by `up`, clamped to [0.02, 2], the 3D point
 * X = K_level^-1 x~ / rho and the flow to camera 1 as SolveUc forms it
 * (solveUcSk.cu:21-33).  K_level, R, t: n x 9, n x 9, n x 3 host doubles;
 * u, v, X, Y, Z: host arrays of n device plane pointers. */
RF_API rf_status rf_ws_state(int n, const float* net, int channels, int wn, int hn, int w, int h,
                             int s, float up, const double* K_level, const double* R,
                             const double* t, float* const* u, float* const* v, float* const* X,
                             float* const* Y, float* const* Z, void* stream);

/* ------------------------------------------------------------------------
 * Kernel-level entry points (device pointers, caller's stream).  Each runs
 * one reference kernel's computation on one pyramid level so it can be
 * checked against the oracle in isolation.  Arrays are stride-major planes
 * of (h + 1) * s floats: kernels that read the row below or the column right
 * of the image (as the reference does) touch row h and column w. 
 * ---------------------------------------------------------------------- */

/* DownscaleKernel / DownscaleScalingKernel (downscale.cu:6-48). */
RF_API rf_status rfk_downscale(const float* src, int w, int h, int s, int nw, int nh, int ns,
                               float scale, int scaled, float* out, void* stream);
/* UpscaleKernel (upscale.cu:14-27). */
RF_API rf_status rfk_upscale(const float* src, int w, int h, int s, int nw, int nh, int ns,
                             float scale, float* out, void* stream);
/* WarpingKernel (warpImage.cu:15-29). */
RF_API rf_status rfk_warp(const float* src, int w, int h, int s, const float* u, const float* v,
                          float* out, void* stream);
/* ComputeDerivativesKernel (computeDerivatives.cu:8-57). */
RF_API rf_status rfk_derivatives(const float* I0, const float* I1w, int w, int h, int s,
                                 float* Ix, float* Iy, float* Iz, void* stream);
/* WarpingKernel then ComputeDerivativesKernel (warpImage.cu:15-29,
 * computeDerivatives.cu:8-57) in one launch, as the solver runs them: the
 * warped I1 is formed in shared memory with a 2-pixel halo and never
 * written; Ix, Iy, Iz equal rfk_warp followed by rfk_derivatives bit for
 * bit. */
RF_API rf_status rfk_warp_derivatives(const float* I0, const float* I1, const float* u,
                                      const float* v, int w, int h, int s, float* Ix, float* Iy,
                                      float* Iz, void* stream);
/* MedianFilterKernel5 (medianFilter.cu:3-75). */
RF_API rf_status rfk_median5(const float* u, const float* v, int w, int h, int s, float* ou,
                             float* ov, void* stream);
/* MedianFilter3DKernel3 (medianFilter.cu:166-243). */
RF_API rf_status rfk_median3d(const float* X, const float* Y, const float* Z, int w, int h, int s,
                              float* X1, float* Y1, float* Z1, void* stream);
/* The per-warp flow update of ReconFlow (Reconflow.cu:410-420): median of
 * duhat (MedianFilterKernel5), u += it (AddKernel), median of u.  The
 * intermediate u + median(duhat) goes to the caller's scratch planes
 * (tmp_u, tmp_v, (h + 1) * s floats each); results to out_u, out_v. */
RF_API rf_status rfk_warp_update(const float* duhat, const float* dvhat, const float* u,
                                 const float* v, int w, int h, int s, float* tmp_u, float* tmp_v,
                                 float* out_u, float* out_v, void* stream);
/* Largest height * stride (floats per plane) that rfk_warp_update_noalloc
 * accepts: 1920x1088 fits. */
#define RF_NOALLOC_MAX_PLANE (1u << 21)

/* rfk_warp_update without caller scratch and without any allocation, for
 * callers that cannot allocate device memory where this step runs (a
 * real-time pipeline that forbids cudaMalloc after start-up, or a host
 * framework that owns the device memory budget).  No counterpart in the
 * reference.  The intermediate planes live in a static 16 MiB device array
 * that every call on a device shares: calls that overlap on the GPU race, so
 * order them on one stream.  height * stride above RF_NOALLOC_MAX_PLANE is
 * rejected with RF_ERR_INVALID_ARG.  The first call on each device looks up
 * the array's device address with that device current; make it before any
 * stream capture on that device.  The address is kept for the life of the
 * process: do not call it again on a device after cudaDeviceReset (the reset
 * drops the module that held the array, and the kept address goes stale). */
RF_API rf_status rfk_warp_update_noalloc(const float* duhat, const float* dvhat, const float* u,
                                         const float* v, int w, int h, int s, float* out_u,
                                         float* out_v, void* stream);
/* Fault injection for tests (no reference counterpart): from this call on,
 * the k-th device or pinned-host allocation the library makes fails as if
 * the device were out of memory (k = 0: none).  RF_FAIL_ALLOC=k in the
 * environment sets the same before the first allocation.  Every create
 * call then returns RF_ERR_OOM and releases what it had allocated. */
RF_API void rf_test_fail_alloc(long long k);
/* rgbaToGrayKernel (rgbToGray.cu:3-19). */
RF_API rf_status rfk_rgb_to_gray(const uint8_t* rgb, int w, int h, int s, float* out,
                                 void* stream);
/* RemoveEdgeArtifacts3DKernel (solve3dMinimalArea.cu:320-378). */
RF_API rf_status rfk_remove_edge_artifacts(const float* X, const float* Y, const float* Z,
                                           int range, float max_area, int w, int h, int s,
                                           float* X1, float* Y1, float* Z1, void* stream);
/* ComputeColorKernel (flowToHSV.cu:194-302). */
RF_API rf_status rfk_flow_to_color(const float* u, const float* v, int w, int h, int s,
                                   float flow_scale, float* rgb, void* stream);

/* ---------------------------------------------------------------------------
 * Pose front end: CameraPose (reconflow/CameraPose.h:11-64,
 * CameraPose.cpp:11-128).  The reference detects SURF keypoints on the GPU
 * (OpenCV's closed SURF_CUDA), matches them by brute force (k = 2, ratio
 * 0.6), and estimates E by LMedS and the pose by recoverPose.  Here: SURF as
 * published (H. Bay et al., CVIU 110(3), 2008) restated as CUDA kernels
 * (integral image, box-filter Hessian responses over octaves, 3x3x3 maxima
 * with quadratic refinement, dominant orientation, 64-value descriptor), a
 * brute-force matcher kernel, and the five-point LMedS and pose recovery on
 * the host.  Every GPU stage is exact FP32 and equals the CPU oracle bit
 * for bit.
 * ------------------------------------------------------------------------ */
typedef struct rf_pose rf_pose;

typedef struct rf_pose_params {
    double hessian_threshold;  /* minHessian (CameraPose.cpp:21-24: 2000) */
    int n_octaves;             /* 4 */
    int n_octave_layers;       /* 2 (4 response layers per octave) */
    int max_keypoints;         /* per frame, strongest kept; 0 = 1% of the pixels */
    double ratio;              /* match ratio test (CameraPose.cpp:71: 0.6) */
    double confidence;         /* LMedS confidence (CameraPose.cpp:80: 0.999) */
    unsigned long long seed;   /* LMedS sampling */
    int refine;                /* 1: refine (R, t) on the inliers by Levenberg-Marquardt
                                  on their Sampson distances; 0 (default) = the
                                  reference, which stops at the LMedS model */
} rf_pose_params;

/* One detected keypoint (the fields of cv::KeyPoint the path uses). */
typedef struct rf_keypoint {
    float x, y;      /* position in pixels */
    float scale;     /* s = 1.2 L / 9 for the (interpolated) filter size L */
    float angle;     /* dominant orientation, radians in [0, 2 pi) */
    float response;  /* determinant-of-Hessian response */
    int octave;
} rf_keypoint;

RF_API rf_status rf_pose_params_default(rf_pose_params* p);
/* CameraPose::initialize: buffers for frames of width x height. */
RF_API rf_status rf_pose_create(const rf_pose_params* p, int width, int height, rf_pose** out);
RF_API rf_status rf_pose_destroy(rf_pose* h);
RF_API rf_status rf_pose_set_stream(rf_pose* h, void* stream);
/* CameraPose::solvePose_8uc1 (CameraPose.cpp:47-118): 8-bit gray frames
 * (pitch in bytes; host or device memory), intrinsics K (row-major 3x3,
 * both frames).
 * Writes R (row-major) and unit t with x1 = R x0 + t.  RF_ERR_STATE when
 * a frame has no keypoints, fewer than 5 matches survive, or no model is
 * found (the reference's "return 1" cases). */
RF_API rf_status rf_pose_solve_u8(rf_pose* h, const uint8_t* im0, const uint8_t* im1, int pitch,
                                  const double K[9], double R[9], double t[3]);
/* The same for float gray frames in [0, 1] (pitch in floats; host or device memory),
 * converted to 8 bits on the GPU as round(255 v) clamped to [0, 255]. */
RF_API rf_status rf_pose_solve_f32(rf_pose* h, const float* im0, const float* im1, int pitch,
                                   const double K[9], double R[9], double t[3]);
/* Keypoints, matches and inliers of the last solve. */
RF_API rf_status rf_pose_counts(const rf_pose* h, int* n_kp0, int* n_kp1, int* n_matches,
                                int* n_inliers);
/* Keypoints (strongest first) and their 64-value descriptors of frame 0 or 1;
 * at most `cap` of each. */
RF_API rf_status rf_pose_keypoints(const rf_pose* h, int frame, rf_keypoint* kp, float* desc,
                                   int cap);
/* Matches that passed the ratio test: keypoint indices in frame 0 and 1,
 * Euclidean descriptor distance, and the LMedS inlier flag. */
RF_API rf_status rf_pose_matches(const rf_pose* h, int* idx0, int* idx1, float* dist,
                                 uint8_t* inlier, int cap);
/* Determinant-of-Hessian responses of one octave of frame 0 or 1 from the
 * last solve: layers x (height >> octave) x (width >> octave) floats. */
RF_API rf_status rf_pose_responses(const rf_pose* h, int frame, int octave, float* out,
                                   size_t cap);

/* Kernels this handle has launched. */
RF_API uint64_t rf_pose_kernel_launches(const rf_pose* h);
/* Solve once (as rf_pose_solve_f32), then time each GPU stage of frame 0,
 * its launches repeated n_iters times back to back on the handle's stream
 * (CUDA events): ms[0] integral image, [1] Hessian responses of every
 * octave, [2] keypoint selection, [3] orientation, [4] descriptors, [5]
 * matching, [6] LMedS scoring; ms[7] = keypoints of frame 0. */
RF_API rf_status rf_pose_profile(rf_pose* h, const float* im0, const float* im1, int pitch,
                                 const double K[9], int n_iters, float* ms);

/* Host-side relative pose, also usable alone.  Normalized image points
 * (K^-1 applied), [n][2] doubles.
 * rf_essential_5pt: the five-point solver (D. Nister, IEEE PAMI 26(6), 2004)
 *   on five matches; writes up to 10 essential matrices (row-major, unit
 *   Frobenius norm) with x1^T E x0 = 0 and returns their number.
 * rf_essential_lmeds: least median of squared Sampson distances over random
 *   five-point samples (findEssentialMat with LMEDS, CameraPose.cpp:80);
 *   writes E and the inlier mask (n bytes).
 * rf_recover_pose: the (R, t) of E with the most triangulated inliers in
 *   front of both cameras (recoverPose, CameraPose.cpp:100).
 * Both samples and medians are deterministic for a seed. */
RF_API int rf_essential_5pt(const double* x0, const double* x1, double* E);
RF_API rf_status rf_essential_lmeds(const double* x0, const double* x1, int n, double confidence,
                                    unsigned long long seed, double E[9], unsigned char* mask);
RF_API rf_status rf_recover_pose(const double E[9], const double* x0, const double* x1, int n,
                                 const unsigned char* mask, double R[9], double t[3],
                                 int* n_good);
/* No reference counterpart: Levenberg-Marquardt on the inliers' summed
 * squared Sampson distances over the five degrees of freedom of (R, t);
 * R, t are the start and the result. */
RF_API rf_status rf_refine_pose(const double* x0, const double* x1, int n,
                                const unsigned char* mask, double R[9], double t[3]);

#ifdef __cplusplus
}
#endif

#endif /* RECONFLOW_GB300_H */
