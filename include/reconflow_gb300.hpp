// C++ class surface over the C ABI: drop-in replacements for the reference's
// CudaFlow (reconflow/Cudaflow.h:17-362), ReconFlow
// (reconflow/Reconflow.h:9-160) and CameraPose (reconflow/CameraPose.h:11-64)
// with the same method names, argument meaning and call order
// (test_reconflow/main.cpp:24-106).
//
// Images and results are raw host pointers with a row pitch in elements
// instead of cv::Mat (define RECONFLOW_GB300_WITH_OPENCV before including
// this header to get the cv::Mat overloads, which read Mat::ptr() with
// Mat::step like the reference).  Methods return 0 like the reference; on
// failure they throw reconflow_gb300::Error (the reference aborts inside
// checkCudaErrors).
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>

#include "reconflow_gb300.h"

#ifdef RECONFLOW_GB300_WITH_OPENCV
#include <opencv2/core.hpp>
#endif

namespace reconflow_gb300 {

class Error : public std::runtime_error {
public:
    Error(rf_status s, const std::string& what) : std::runtime_error(what), status(s) {}
    rf_status status;
};

inline void check(rf_status s) {
    if (s != RF_OK) throw Error(s, rf_last_error_string());
}

class CudaFlow {
public:
    static const int METHOD_TVL1 = RF_METHOD_TVL1;

    CudaFlow() : CudaFlow(32, 12, 32) {}
    CudaFlow(int BlockWidth, int BlockHeight, int StrideAlignment)
        : BlockWidth(BlockWidth), BlockHeight(BlockHeight), StrideAlignment(StrideAlignment) {}
    virtual ~CudaFlow() { close(); }
    CudaFlow(const CudaFlow&) = delete;
    CudaFlow& operator=(const CudaFlow&) = delete;

    // Cudaflow.cu:99-269 (cvType given as RF_INPUT_*)
    int initialize(int width, int height, int channels, int inputType, int nLevels, float scale,
                   int method, float lambda = 100.0f, float lambdagrad = 400.0f,
                   float theta = 0.33f, float tau = 0.25f, int nWarpIters = 1,
                   int nSolverIters = 100) {
        rf_params p;
        check(rf_params_default(&p, method));
        p.width = width; p.height = height; p.channels = channels; p.input_type = inputType;
        p.n_levels = nLevels; p.scale = scale; p.lambda = lambda; p.lambdagrad = lambdagrad;
        p.theta = theta; p.tau = tau; p.n_warp_iters = nWarpIters; p.n_solver_iters = nSolverIters;
        return create(p);
    }

    int iAlignUp(int n) const {
        int m = StrideAlignment, mod = n % m;
        return mod ? n + m - mod : n;
    }

    // Cudaflow.cu:288-311: pitch in elements (pixels for RGB8)
    int copyImagesToDevice(const void* i0, const void* i1, int pitch) {
        check(rf_upload_images(h_, i0, i1, pitch));
        return 0;
    }
    // Cudaflow.cu:394-399
    int solveOpticalFlow(float flowScale = 5.0f) {
        flowScale_ = flowScale;
        check(rf_solve_flow(h_));
        return 0;
    }
    // Cudaflow.cu:320-325
    int copyOpticalFlowToHost(float* u, float* v, int pitch) {
        check(rf_download_flow(h_, u, v, pitch));
        return 0;
    }
    // Cudaflow.cu:313-318: colour image as 3 floats per pixel (B, G, R)
    int copyOpticalFlowToHost(float* u, float* v, float* uvrgb, int pitch) {
        check(rf_download_flow(h_, u, v, pitch));
        check(rf_download_flow_color(h_, flowScale_, uvrgb, pitch));
        return 0;
    }
    // Cudaflow.h:47: the colour wheel is a constant table of the colour
    // kernel here, so there is nothing to set up; kept for call sites
    int initializeColorWheel() { return 0; }
    // Cudaflow.h:52-53, the reference's older names of the image upload and
    // the flow + colour download
    int copyToDevice(const void* i0, const void* i1, int pitch) {
        return copyImagesToDevice(i0, i1, pitch);
    }
    int copyToHost(float* u, float* v, float* uvrgb, int pitch) {
        return copyOpticalFlowToHost(u, v, uvrgb, pitch);
    }
    int close() {
        if (h_) rf_destroy(h_);
        h_ = nullptr;
        return 0;
    }
    rf_handle* handle() const { return h_; }

#ifdef RECONFLOW_GB300_WITH_OPENCV
    int copyImagesToDevice(cv::Mat i0, cv::Mat i1) {
        return copyImagesToDevice(i0.ptr(), i1.ptr(), (int)(i0.step / i0.elemSize()));
    }
    int copyOpticalFlowToHost(cv::Mat& u, cv::Mat& v) {
        return copyOpticalFlowToHost(u.ptr<float>(), v.ptr<float>(), (int)(u.step / sizeof(float)));
    }
#endif

    int width = 0, height = 0, stride = 0, nLevels = 0;
    int BlockWidth, BlockHeight, StrideAlignment;

protected:
    int create(rf_params& p) {
        close();
        p.stride_alignment = StrideAlignment;
        p.block_width = BlockWidth;
        p.block_height = BlockHeight;
        check(rf_create(&p, &h_));
        width = p.width; height = p.height; nLevels = p.n_levels;
        stride = rf_stride(h_);
        return 0;
    }
    rf_handle* h_ = nullptr;
    float flowScale_ = 5.0f;
};

class ReconFlow : public CudaFlow {
public:
    static const int METHODR_TVL1_MS = RF_METHODR_TVL1_MS;
    static const int METHODR_TVL1_MS_FN = RF_METHODR_TVL1_MS_FN;
    static const int METHODR_TVL1_MS_FNSPARSE = RF_METHODR_TVL1_MS_FNSPARSE;

    ReconFlow() : CudaFlow() {}
    ReconFlow(int BlockWidth, int BlockHeight, int StrideAlignment)
        : CudaFlow(BlockWidth, BlockHeight, StrideAlignment) {}

    // Reconflow.cu:15-25.  The reference forces 8-bit RGB input; inputType
    // selects any of RF_INPUT_*.  fixQuirks = RF_FIX_* bits (0 = reference).
    int initializeR(int width, int height, int channels, int nLevels, float scale, int method,
                    float lambda = 100.0f, float lambdagrad = 400.0f, float lambdaf = 100.0f,
                    float lambdams = 100.0f, float alphaTv = 3.0f, float alphaProj = 1.0f,
                    float alphaFn = 0.5f, float tau = 0.25f, int nWarpIters = 1,
                    int nSolverIters = 100, int inputType = RF_INPUT_RGB8, int fixQuirks = 0) {
        rf_params p;
        check(rf_params_default(&p, method));
        p.width = width; p.height = height; p.channels = channels; p.input_type = inputType;
        p.n_levels = nLevels; p.scale = scale; p.lambda = lambda; p.lambdagrad = lambdagrad;
        p.lambdaf = lambdaf; p.lambdams = lambdams; p.alpha_tv = alphaTv;
        p.alpha_proj = alphaProj; p.alpha_fn = alphaFn; p.tau = tau; p.theta = 1.0f / alphaTv;
        p.n_warp_iters = nWarpIters; p.n_solver_iters = nSolverIters; p.fix_quirks = fixQuirks;
        return create(p);
    }
    // Reconflow.cu:78-116 (3x3 row-major doubles)
    int setCameraMatrices(const double* K0, const double* K1) {
        check(rf_set_cameras(h_, K0, K1));
        return 0;
    }
    // Cudaflow.cu:327-343
    int copySparseOpticalFlowToDevice(const float* u, const float* v, const float* mask,
                                      int pitch) {
        check(rf_set_prior_flow(h_, u, v, mask, pitch));
        return 0;
    }
    int copyInitialOpticalFlowToDevice(const float* u, const float* v, int pitch) {
        return copySparseOpticalFlowToDevice(u, v, nullptr, pitch);
    }
    // Reconflow.cu:130-144
    int solveR(const double* R1, const double* t1, float flowScale = 5.0f) {
        return solveR(nullptr, nullptr, R1, t1, flowScale);
    }
    int solveR(const double* R0, const double* t0, const double* R1, const double* t1,
               float flowScale) {
        flowScale_ = flowScale;
        check(rf_solve(h_, R0, t0, R1, t1));
        return 0;
    }
    // Reconflow.h:76-77: the solve solveR forwards to
    int solveReconFlow(const double* R1, const double* t1, float flowScale) {
        return solveR(R1, t1, flowScale);
    }
    int solveReconFlow(const double* R0, const double* t0, const double* R1, const double* t1,
                       float flowScale) {
        return solveR(R0, t0, R1, t1, flowScale);
    }
    // Reconflow.cu:65-70
    int copy3dToHost(float* X, float* Y, float* Z, int pitch) {
        check(rf_download_points(h_, X, Y, Z, pitch));
        return 0;
    }
    int copyInverseDepthToHost(float* inv, int pitch) {
        check(rf_download_inv_depth(h_, inv, pitch));
        return 0;
    }
    // Reconflow.cu:468-477
    int removeEdgeArtifacts3D(int surfaceWidth, float maxSurfaceArea) {
        check(rf_remove_edge_artifacts(h_, surfaceWidth, maxSurfaceArea));
        return 0;
    }

#ifdef RECONFLOW_GB300_WITH_OPENCV
    int setCameraMatrices(cv::Mat K0, cv::Mat K1) {
        return setCameraMatrices(K0.ptr<double>(), K1.ptr<double>());
    }
    int solveR(cv::Mat R1, cv::Mat t1, float flowScale) {
        return solveR(R1.ptr<double>(), t1.ptr<double>(), flowScale);
    }
    int solveR(cv::Mat R0, cv::Mat t0, cv::Mat R1, cv::Mat t1, float flowScale) {
        return solveR(R0.ptr<double>(), t0.ptr<double>(), R1.ptr<double>(), t1.ptr<double>(),
                      flowScale);
    }
    int solveReconFlow(cv::Mat R1, cv::Mat t1, float flowScale) {
        return solveR(R1, t1, flowScale);
    }
    int solveReconFlow(cv::Mat R0, cv::Mat t0, cv::Mat R1, cv::Mat t1, float flowScale) {
        return solveR(R0, t0, R1, t1, flowScale);
    }
    int copySparseOpticalFlowToDevice(cv::Mat u, cv::Mat v) {
        return copySparseOpticalFlowToDevice(u.ptr<float>(), v.ptr<float>(), nullptr,
                                             (int)(u.step / sizeof(float)));
    }
    int copySparseOpticalFlowToDevice(cv::Mat u, cv::Mat v, cv::Mat mask) {
        return copySparseOpticalFlowToDevice(u.ptr<float>(), v.ptr<float>(), mask.ptr<float>(),
                                             (int)(u.step / sizeof(float)));
    }
    int copy3dToHost(cv::Mat& X, cv::Mat& Y, cv::Mat& Z) {
        return copy3dToHost(X.ptr<float>(), Y.ptr<float>(), Z.ptr<float>(),
                            (int)(X.step / sizeof(float)));
    }
#endif
};

// Many frame pairs solved together (rf_batch_*; no reference counterpart):
// pairs may differ in size, cameras and pose and share the solver
// parameters; a pair's results are bit-identical to solving it alone.
class ReconFlowBatch {
public:
    // p: parameters as rf_params_default(RF_METHODR_TVL1_MS) plus the
    // caller's weights and schedule; widths / heights: n_pairs sizes
    ReconFlowBatch(const rf_params& p, int n_pairs, const int* widths, const int* heights) {
        check(rf_batch_create(&p, n_pairs, widths, heights, &b_));
    }
    ~ReconFlowBatch() { rf_batch_destroy(b_); }
    ReconFlowBatch(const ReconFlowBatch&) = delete;
    ReconFlowBatch& operator=(const ReconFlowBatch&) = delete;

    int stride(int pair) const { return rf_batch_stride(b_, pair); }
    int setCameraMatrices(int pair, const double* K0, const double* K1) {
        check(rf_batch_set_cameras(b_, pair, K0, K1));
        return 0;
    }
    int copyImagesToDevice(int pair, const float* i0, const float* i1, int pitch) {
        check(rf_batch_upload_images(b_, pair, i0, i1, pitch));
        return 0;
    }
    // R1s, t1s: n_pairs x 9 and n_pairs x 3 doubles (camera 0 = identity)
    int solveR(const double* R1s, const double* t1s) {
        check(rf_batch_solve(b_, nullptr, nullptr, R1s, t1s));
        return 0;
    }
    // warm start at `level` from the planes of warmPlanes (filled beforehand)
    int solveWarm(int level, const int* warps, const int* iters, const double* R1s,
                  const double* t1s) {
        check(rf_batch_solve_warm_levels(b_, nullptr, nullptr, R1s, t1s, level, warps, iters));
        return 0;
    }
    int warmPlanes(int pair, float** u, float** v, float** X, float** Y, float** Z) {
        check(rf_batch_warm_planes(b_, pair, u, v, X, Y, Z));
        return 0;
    }
    int setTiles(const int* tile_w, const int* tile_h) {
        check(rf_batch_set_tiles(b_, tile_w, tile_h));
        return 0;
    }
    int copyOpticalFlowToHost(int pair, float* u, float* v, int pitch) {
        check(rf_batch_download_flow(b_, pair, u, v, pitch));
        return 0;
    }
    int copy3dToHost(int pair, float* X, float* Y, float* Z, int pitch) {
        check(rf_batch_download_points(b_, pair, X, Y, Z, pitch));
        return 0;
    }
    int energies(double* out) {
        check(rf_batch_energies(b_, out));
        return 0;
    }
    // pipelined transfers (rf_batch_stage_upload and its companions): i0 /
    // i1 / outputs are arrays of n_pairs host pointers, one pitch
    int stageUpload(const float* const* i0, const float* const* i1, int pitch) {
        check(rf_batch_stage_upload(b_, i0, i1, pitch));
        return 0;
    }
    int takeUpload() {
        check(rf_batch_take_upload(b_));
        return 0;
    }
    int stageDownload(float* const* u, float* const* v, float* const* inv_depth,
                      float* const* X, float* const* Y, float* const* Z, int pitch) {
        check(rf_batch_stage_download(b_, u, v, inv_depth, X, Y, Z, pitch));
        return 0;
    }
    int waitDownload() {
        check(rf_batch_wait_download(b_));
        return 0;
    }
    rf_batch* handle() { return b_; }

private:
    rf_batch* b_ = nullptr;
};

// CameraPose (reconflow/CameraPose.h:11-64): relative pose of two 8-bit gray
// frames.  solvePose_8uc1 returns 0 and fills R (row-major 3x3) and t (unit,
// x1 = R x0 + t) like the reference, or 1 when no keypoints / too few
// matches / no model (the reference's "return 1" cases).
class CameraPose {
public:
    CameraPose() { check(rf_pose_params_default(&p_)); }
    ~CameraPose() { rf_pose_destroy(h_); }
    CameraPose(const CameraPose&) = delete;
    CameraPose& operator=(const CameraPose&) = delete;

    int initialize(const double* intrinsic, int minHessian = 2000) {
        for (int i = 0; i < 9; i++) K_[i] = intrinsic[i];
        p_.hessian_threshold = minHessian;
        release();
        return 0;
    }
    int initialize(double focal, double ppx, double ppy, int minHessian = 2000) {
        const double K[9] = {focal, 0.0, ppx, 0.0, focal, ppy, 0.0, 0.0, 1.0};
        return initialize(K, minHessian);
    }
    int initialize(double focalx, double focaly, double ppx, double ppy, int minHessian) {
        const double K[9] = {focalx, 0.0, ppx, 0.0, focaly, ppy, 0.0, 0.0, 1.0};
        return initialize(K, minHessian);
    }
    // frames of width x height, `pitch` bytes per row
    int solvePose_8uc1(const uint8_t* im1, const uint8_t* im2, int width, int height, int pitch,
                       double* R, double* t) {
        if (!h_ || width != w_ || height != hgt_) {
            release();
            check(rf_pose_create(&p_, width, height, &h_));
            w_ = width;
            hgt_ = height;
        }
        const rf_status s = rf_pose_solve_u8(h_, im1, im2, pitch, K_, R, t);
        if (s == RF_ERR_STATE) return 1;
        check(s);
        return 0;
    }
    rf_pose_params& params() { return p_; }
    rf_pose* handle() { return h_; }

private:
    void release() {
        if (h_) rf_pose_destroy(h_);
        h_ = nullptr;
    }
    rf_pose_params p_{};
    rf_pose* h_ = nullptr;
    double K_[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    int w_ = 0, hgt_ = 0;
};

}  // namespace reconflow_gb300
