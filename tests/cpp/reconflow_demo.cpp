// Drives the C++ class surface in the call order of the reference demo
// (test_reconflow/main.cpp:24-106): construct, initializeR, setCameraMatrices,
// copyImagesToDevice, solveR, copyOpticalFlowToHost, copy3dToHost; then the
// batch class on the same pair and CameraPose on flat frames.  The input
// is a synthetic textured pair shifted by one pixel.  Prints one line:
// "ok <median u> <median Z>" or "error <status> <message>".
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "reconflow_gb300.hpp"

int main() {
    using reconflow_gb300::ReconFlow;
    const int width = 160, height = 120, nLevels = 3;
    try {
        ReconFlow flow(32, 12, 32);
        flow.initializeR(width, height, 1, nLevels, 2.0f, ReconFlow::METHODR_TVL1_MS, 50.0f, 0.0f,
                         0.1f, 100.0f, 1.0f / 0.33f, 60.0f, 0.5f, 0.25f, 2, 20, RF_INPUT_F32,
                         RF_FIX_K_PYRAMID);
        const int stride = flow.iAlignUp(width);
        std::vector<float> i0(stride * height, 0.0f), i1(stride * height, 0.0f);
        for (int y = 0; y < height; y++)
            for (int x = 0; x < width; x++) {
                auto tex = [](double xx, double yy) {
                    return 0.5 + 0.2 * std::sin(0.31 * xx + 0.17 * yy) + 0.1 * std::cos(0.07 * xx - 0.23 * yy);
                };
                i0[x + y * stride] = (float)tex(x, y);
                i1[x + y * stride] = (float)tex(x - 1.0, y);
            }
        const double f = 125.0;
        const double K[9] = {f, 0, width / 2.0, 0, f, height / 2.0, 0, 0, 1};
        const double R[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        const double t[3] = {0.1, 0.001, 0.001};  // content moves +1 px: depth f*b/d = 12.5
        flow.setCameraMatrices(K, K);
        flow.copyImagesToDevice(i0.data(), i1.data(), stride);
        flow.solveR(R, t, 50.0f);
        std::vector<float> u(stride * height), v(stride * height);
        std::vector<float> X(stride * height), Y(stride * height), Z(stride * height);
        flow.copyOpticalFlowToHost(u.data(), v.data(), stride);
        flow.copy3dToHost(X.data(), Y.data(), Z.data(), stride);
        std::vector<float> uu, zz;
        for (int y = 8; y < height - 8; y++)
            for (int x = 8; x < width - 8; x++) {
                uu.push_back(u[x + y * stride]);
                zz.push_back(Z[x + y * stride]);
            }
        std::nth_element(uu.begin(), uu.begin() + uu.size() / 2, uu.end());
        std::nth_element(zz.begin(), zz.begin() + zz.size() / 2, zz.end());
        // the same pair twice through the batch class: bit-identical to the
        // single-pair solve
        rf_params p;
        rf_params_default(&p, RF_METHODR_TVL1_MS);
        p.width = width;
        p.height = height;
        p.input_type = RF_INPUT_F32;
        p.n_levels = nLevels;
        p.lambda = 50.0f;
        p.lambdaf = 0.1f;
        p.lambdams = 100.0f;
        p.alpha_tv = 1.0f / 0.33f;
        p.alpha_proj = 60.0f;
        p.tau = 0.25f;
        p.theta = 0.33f;
        p.n_warp_iters = 2;
        p.n_solver_iters = 20;
        p.fix_quirks = RF_FIX_K_PYRAMID;
        const int ws[2] = {width, width}, hs[2] = {height, height};
        reconflow_gb300::ReconFlowBatch batch(p, 2, ws, hs);
        double Rs[18], ts[6];
        for (int k = 0; k < 2; k++) {
            batch.setCameraMatrices(k, K, K);
            batch.copyImagesToDevice(k, i0.data(), i1.data(), stride);
            for (int i = 0; i < 9; i++) Rs[9 * k + i] = R[i];
            for (int i = 0; i < 3; i++) ts[3 * k + i] = t[i];
        }
        batch.solveR(Rs, ts);
        std::vector<float> bu(stride * height), bv(stride * height);
        int same = 1;
        for (int k = 0; k < 2; k++) {
            batch.copyOpticalFlowToHost(k, bu.data(), bv.data(), stride);
            for (int y = 0; y < height; y++)
                for (int x = 0; x < width; x++)
                    same &= bu[x + y * stride] == u[x + y * stride] ||
                            (std::isnan(bu[x + y * stride]) && std::isnan(u[x + y * stride]));
        }
        if (!same) {
            std::printf("error 0 batch differs from the single-pair solve\n");
            return 1;
        }
        // CameraPose: a flat frame pair has no keypoints -> 1, as the reference
        reconflow_gb300::CameraPose pose;
        pose.initialize(K, 2000);
        std::vector<uint8_t> flat(width * height, 128);
        double Rp[9], tp[3];
        if (pose.solvePose_8uc1(flat.data(), flat.data(), width, height, width, Rp, tp) != 1) {
            std::printf("error 0 CameraPose found a pose in flat frames\n");
            return 1;
        }
        std::printf("ok %.4f %.4f\n", uu[uu.size() / 2], zz[zz.size() / 2]);
    } catch (const reconflow_gb300::Error& e) {
        std::printf("error %d %s\n", (int)e.status, e.what());
        return e.status == RF_ERR_NO_DEVICE ? 3 : 1;
    }
    return 0;
}
