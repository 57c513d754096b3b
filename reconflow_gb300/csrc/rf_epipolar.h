// Host-side relative pose (rf_epipolar.cpp) as used by the pose front end
// (rf_pose.cu), which scores the LMedS hypotheses on the GPU with the same
// squared Sampson distance.
#pragma once

#include <cmath>
#include <cstdint>
#include <vector>

#ifdef __CUDACC__
#define RF_HD __host__ __device__
#else
#define RF_HD
#endif

namespace rf_epi {

// Squared Sampson distance of a match (normalized points a in frame 0, b in
// frame 1) under E: (b^T E a)^2 / ((E a)_1^2 + (E a)_2^2 + (E^T b)_1^2 +
// (E^T b)_2^2).  The same operations on host and device.
RF_HD inline double sampson2(const double* E, const double* a, const double* b) {
    const double x0[3] = {a[0], a[1], 1.0}, x1[3] = {b[0], b[1], 1.0};
    double Ex0[3], Etx1[3];
    for (int i = 0; i < 3; i++) {
        Ex0[i] = E[i * 3 + 0] * x0[0] + E[i * 3 + 1] * x0[1] + E[i * 3 + 2] * x0[2];
        Etx1[i] = E[0 * 3 + i] * x1[0] + E[1 * 3 + i] * x1[1] + E[2 * 3 + i] * x1[2];
    }
    const double r = x1[0] * Ex0[0] + x1[1] * Ex0[1] + x1[2] * Ex0[2];
    const double d = Ex0[0] * Ex0[0] + Ex0[1] * Ex0[1] + Etx1[0] * Etx1[0] + Etx1[1] * Etx1[1];
    return d > 0.0 ? r * r / d : (r == 0.0 ? 0.0 : INFINITY);
}

// Every five-point hypothesis (9 doubles each) of the seeded LMedS samples,
// in sample order.
std::vector<double> lmeds_hypotheses(const double* x0, const double* x1, int n, double conf,
                                     uint64_t seed);
// Median squared Sampson distance of every hypothesis (host threads).
std::vector<double> lmeds_medians(const std::vector<double>& hyp, const double* x0,
                                  const double* x1, int n);
// The least-median hypothesis (first on ties) and its inlier mask.
bool lmeds_select(const std::vector<double>& hyp, const std::vector<double>& med, const double* x0,
                  const double* x1, int n, double* E, unsigned char* mask);
// (R, t) of E with the most inliers triangulated in front of both cameras.
int recover_pose(const double* E, const double* x0, const double* x1, int n,
                 const unsigned char* mask, double* R, double* t);

// Levenberg-Marquardt refinement of (R, t) on the inliers' Sampson distances.
void refine_pose(const double* x0, const double* x1, int n, const unsigned char* mask, double* R,
                 double* t);

}  // namespace rf_epi
