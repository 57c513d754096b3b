// Drives the C++ class surface in the call order of the reference demo
// (test_reconflow/main.cpp:24-106): construct, initializeR, setCameraMatrices,
// copyImagesToDevice, solveR, copyOpticalFlowToHost, copy3dToHost.  The input
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
        std::printf("ok %.4f %.4f\n", uu[uu.size() / 2], zz[zz.size() / 2]);
    } catch (const reconflow_gb300::Error& e) {
        std::printf("error %d %s\n", (int)e.status, e.what());
        return e.status == RF_ERR_NO_DEVICE ? 3 : 1;
    }
    return 0;
}
