// Relative pose from point matches, host side of the pose front end
// (CameraPose::solvePose_8uc1, reconflow/CameraPose.cpp:79-104, which calls
// OpenCV's findEssentialMat(..., LMEDS, 0.999) and recoverPose).  OpenCV is
// not used here; the published methods are restated:
//
// * the five-point solver (rf_fivept.cuh);
// * least median of squares (P. J. Rousseeuw, "Least median of squares
//   regression", JASA 79, 1984) over random five-point samples with the
//   squared Sampson distance, the sample count for confidence `conf` at an
//   outlier ratio of 0.45, and the inlier threshold
//   (2.5 * 1.4826 * (1 + 5 / (n - 5)))^2 * median;
// * pose recovery: E = U diag(1, 1, 0) V^T, the four (R, t) candidates
//   U W V^T / U W^T V^T with t = +-u3, the least-squares depths of every
//   inlier in both cameras and the cheirality count (positive depth in both,
//   depth < 50).
//
// Everything is double precision and deterministic (seeded sampling).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <atomic>
#include <thread>
#include <vector>

#include "../../include/reconflow_gb300.h"
#include "rf_epipolar.h"
#include "rf_fivept.cuh"

namespace rf_epi {

// ---------------------------------------------------------------------------
// Small dense linear algebra
// ---------------------------------------------------------------------------

// Cyclic Jacobi eigen-decomposition of a symmetric n x n matrix (row-major,
// destroyed): eigenvalues into w, eigenvectors into the columns of V.
void jacobi_eigen(double* A, int n, double* w, double* V) {
    double total = 0.0;
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            V[i * n + j] = i == j ? 1.0 : 0.0;
            total += A[i * n + j] * A[i * n + j];
        }
    for (int sweep = 0; sweep < 60; sweep++) {
        double off = 0.0;
        for (int p = 0; p < n; p++)
            for (int q = p + 1; q < n; q++) off += A[p * n + q] * A[p * n + q];
        // converged: the off-diagonal part is below rounding of the whole
        if (!(off > 1e-34 * total)) break;
        for (int p = 0; p < n; p++)
            for (int q = p + 1; q < n; q++) {
                const double apq = A[p * n + q];
                if (std::fabs(apq) < 1e-300) continue;
                const double app = A[p * n + p], aqq = A[q * n + q];
                const double theta = (aqq - app) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) /
                                 (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; k++) {
                    const double akp = A[k * n + p], akq = A[k * n + q];
                    A[k * n + p] = c * akp - s * akq;
                    A[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; k++) {
                    const double apk = A[p * n + k], aqk = A[q * n + k];
                    A[p * n + k] = c * apk - s * aqk;
                    A[q * n + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; k++) {
                    const double vkp = V[k * n + p], vkq = V[k * n + q];
                    V[k * n + p] = c * vkp - s * vkq;
                    V[k * n + q] = s * vkp + c * vkq;
                }
            }
    }
    for (int i = 0; i < n; i++) w[i] = A[i * n + i];
}

// indices of w sorted ascending
void argsort(const double* w, int n, int* idx) {
    for (int i = 0; i < n; i++) idx[i] = i;
    std::sort(idx, idx + n, [&](int a, int b) { return w[a] < w[b] || (w[a] == w[b] && a < b); });
}

void mat3_mul(const double* A, const double* B, double* C) {
    double T[9];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            T[i * 3 + j] = A[i * 3 + 0] * B[0 * 3 + j] + A[i * 3 + 1] * B[1 * 3 + j] +
                           A[i * 3 + 2] * B[2 * 3 + j];
    std::memcpy(C, T, sizeof(T));
}

void mat3_transpose(const double* A, double* T) {
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) T[j * 3 + i] = A[i * 3 + j];
}

double det3(const double* A) {
    return A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
           A[2] * (A[3] * A[7] - A[4] * A[6]);
}

void cross3(const double* a, const double* b, double* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

// SVD of a 3x3 matrix: A = U diag(s) V^T, s descending, U and V orthogonal
// (from the eigen-decomposition of A^T A; u3 = u1 x u2 completes U).
void svd3(const double* A, double* U, double* s, double* V) {
    double AtA[9], At[9], w[3], Vu[9];
    mat3_transpose(A, At);
    mat3_mul(At, A, AtA);
    jacobi_eigen(AtA, 3, w, Vu);
    int idx[3];
    argsort(w, 3, idx);
    const int ord[3] = {idx[2], idx[1], idx[0]};
    for (int k = 0; k < 3; k++) {
        s[k] = std::sqrt(std::max(w[ord[k]], 0.0));
        for (int i = 0; i < 3; i++) V[i * 3 + k] = Vu[i * 3 + ord[k]];
    }
    double u[3][3];
    for (int k = 0; k < 2; k++) {
        double n = 0.0;
        for (int i = 0; i < 3; i++) {
            u[k][i] = A[i * 3 + 0] * V[0 * 3 + k] + A[i * 3 + 1] * V[1 * 3 + k] +
                      A[i * 3 + 2] * V[2 * 3 + k];
            n += u[k][i] * u[k][i];
        }
        n = std::sqrt(n);
        for (int i = 0; i < 3; i++) u[k][i] = n > 0 ? u[k][i] / n : (i == k ? 1.0 : 0.0);
    }
    if (!(s[1] > 0.0)) {  // rank < 2: any unit vector orthogonal to u1
        const double a[3] = {std::fabs(u[0][0]) < 0.9 ? 1.0 : 0.0, std::fabs(u[0][0]) < 0.9 ? 0.0 : 1.0, 0.0};
        cross3(u[0], a, u[1]);
        double n = std::sqrt(u[1][0] * u[1][0] + u[1][1] * u[1][1] + u[1][2] * u[1][2]);
        for (int i = 0; i < 3; i++) u[1][i] /= n;
    }
    cross3(u[0], u[1], u[2]);
    for (int i = 0; i < 3; i++)
        for (int k = 0; k < 3; k++) U[i * 3 + k] = u[k][i];
}

using rf_fivept::five_point;

uint64_t splitmix64(uint64_t& s) {
    uint64_t z = (s += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

// uniform integer in [0, n) without modulo bias
int uniform_below(uint64_t& s, int n) {
    const uint64_t lim = UINT64_MAX - UINT64_MAX % (uint64_t)n;
    uint64_t v;
    do {
        v = splitmix64(s);
    } while (v >= lim);
    return (int)(v % (uint64_t)n);
}

// Least-median-of-squares essential matrix over n >= 5 normalized matches.
// Returns false when no sample gave a model.
// calls of parallel_for running at once (from several handles' threads)
std::atomic<int> g_active{0};

// f(i) for i in [0, n) on host threads: the cores shared among the calls
// running at once, static contiguous ranges, so every i is computed exactly
// as on one thread.
template <class F>
void parallel_for(int n, F&& f) {
    const unsigned hw = std::thread::hardware_concurrency();
    const int active = ++g_active;
    const int threads = std::max(1, std::min({(int)(hw ? hw : 1) / active, 16, n / 8}));
    struct Leave {
        ~Leave() { --g_active; }
    } leave;
    if (threads <= 1) {
        for (int i = 0; i < n; i++) f(i);
        return;
    }
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; t++)
        pool.emplace_back([&, t] {
            const int lo = (int)((long long)n * t / threads), hi = (int)((long long)n * (t + 1) / threads);
            for (int i = lo; i < hi; i++) f(i);
        });
    for (auto& th : pool) th.join();
}

int lmeds_iterations(double conf) {
    const double ep = 0.45;
    const double denom = std::log(1.0 - std::pow(1.0 - ep, 5.0));
    const int iters = (int)std::lround(std::log(1.0 - conf) / denom);
    return std::max(1, std::min(iters, 1000));
}

// The seeded LMedS samples: lmeds_iterations(conf) sets of five distinct
// match indices, [sample][5].
static std::vector<int> lmeds_samples(int n, double conf, uint64_t seed) {
    const int iters = lmeds_iterations(conf);
    std::vector<int> samples((size_t)iters * 5);
    uint64_t st = seed;
    for (int it = 0; it < iters; it++) {
        int* s = &samples[(size_t)it * 5];
        for (int k = 0; k < 5; k++) {
            for (;;) {
                s[k] = uniform_below(st, n);
                bool dup = false;
                for (int q = 0; q < k; q++) dup |= s[q] == s[k];
                if (!dup) break;
            }
        }
    }
    return samples;
}

// Every five-point hypothesis of the seeded samples, in sample order.
std::vector<double> lmeds_hypotheses(const double* x0, const double* x1, int n, double conf,
                                     uint64_t seed) {
    const std::vector<int> samples = lmeds_samples(n, conf, seed);
    const int iters = (int)(samples.size() / 5);
    std::vector<double> sols((size_t)iters * 90);
    std::vector<int> counts(iters);
    parallel_for(iters, [&](int it) {
        const int* s = &samples[(size_t)it * 5];
        double a[10], b[10];
        for (int k = 0; k < 5; k++) {
            a[2 * k] = x0[2 * s[k]];
            a[2 * k + 1] = x0[2 * s[k] + 1];
            b[2 * k] = x1[2 * s[k]];
            b[2 * k + 1] = x1[2 * s[k] + 1];
        }
        counts[it] = five_point(a, b, &sols[(size_t)it * 90]);
    });
    // sample order: the first counts[s] matrices of each slot of 10
    std::vector<double> hyp;
    for (int it = 0; it < iters; it++)
        hyp.insert(hyp.end(), sols.begin() + (size_t)it * 90,
                   sols.begin() + (size_t)it * 90 + 9 * counts[it]);
    return hyp;
}

// Median squared Sampson distance of every hypothesis: the (n / 2)-th
// smallest of the n distances.
std::vector<double> lmeds_medians(const std::vector<double>& hyp, const double* x0,
                                  const double* x1, int n) {
    const int H = (int)(hyp.size() / 9);
    std::vector<double> med(H);
    parallel_for(H, [&](int h) {
        std::vector<double> tmp(n);
        for (int i = 0; i < n; i++) tmp[i] = sampson2(&hyp[(size_t)h * 9], x0 + 2 * i, x1 + 2 * i);
        std::nth_element(tmp.begin(), tmp.begin() + n / 2, tmp.end());
        med[h] = tmp[n / 2];
    });
    return med;
}

// The hypothesis with the least median (the first on ties) and its inlier
// mask; false when there is none.
bool lmeds_select(const std::vector<double>& hyp, const std::vector<double>& med, const double* x0,
                  const double* x1, int n, double* E, unsigned char* mask) {
    int best = -1;
    for (int h = 0; h < (int)med.size(); h++)
        if (best < 0 ? med[h] < INFINITY : med[h] < med[best]) best = h;
    if (best < 0) return false;
    std::memcpy(E, &hyp[(size_t)best * 9], 9 * sizeof(double));
    double sigma = 2.5 * 1.4826 * (1.0 + 5.0 / (n > 5 ? n - 5 : 1)) * std::sqrt(med[best]);
    sigma = std::max(sigma, 0.001);
    const double thr = sigma * sigma;
    for (int i = 0; i < n; i++) mask[i] = sampson2(E, x0 + 2 * i, x1 + 2 * i) <= thr ? 1 : 0;
    return true;
}

// Least-median-of-squares essential matrix over n >= 5 normalized matches.
bool lmeds(const double* x0, const double* x1, int n, double conf, uint64_t seed, double* E,
           unsigned char* mask) {
    const std::vector<double> hyp = lmeds_hypotheses(x0, x1, n, conf, seed);
    return lmeds_select(hyp, lmeds_medians(hyp, x0, x1, n), x0, x1, n, E, mask);
}

// Depths of one match with camera 0 = [I | 0], camera 1 = [R | t]: the
// least-squares (z0, z1) of z1 b = z0 R a + t for the rays a = (x0, 1),
// b = (x1, 1) (the two normal equations solved in closed form); -1 when the
// rays are parallel.
void triangulate(const double* R, const double* t, const double* a, const double* b, double& z0,
                 double& z1) {
    const double ra[3] = {R[0] * a[0] + R[1] * a[1] + R[2], R[3] * a[0] + R[4] * a[1] + R[5],
                          R[6] * a[0] + R[7] * a[1] + R[8]};
    const double bb[3] = {b[0], b[1], 1.0};
    // minimise |z0 ra - z1 bb + t|^2
    const double A11 = ra[0] * ra[0] + ra[1] * ra[1] + ra[2] * ra[2];
    const double A12 = -(ra[0] * bb[0] + ra[1] * bb[1] + ra[2] * bb[2]);
    const double A22 = bb[0] * bb[0] + bb[1] * bb[1] + bb[2] * bb[2];
    const double r1 = -(ra[0] * t[0] + ra[1] * t[1] + ra[2] * t[2]);
    const double r2 = bb[0] * t[0] + bb[1] * t[1] + bb[2] * t[2];
    const double det = A11 * A22 - A12 * A12;
    if (!(std::fabs(det) > 1e-18 * A11 * A22)) {
        z0 = z1 = -1.0;
        return;
    }
    z0 = (r1 * A22 - A12 * r2) / det;
    z1 = (A11 * r2 - A12 * r1) / det;
}

int recover_pose(const double* E, const double* x0, const double* x1, int n,
                 const unsigned char* mask, double* R, double* t) {
    double U[9], s[3], V[9];
    svd3(E, U, s, V);
    if (det3(U) < 0)
        for (double& u : U) u = -u;
    if (det3(V) < 0)
        for (double& v : V) v = -v;
    const double W[9] = {0, 1, 0, -1, 0, 0, 0, 0, 1};
    double Vt[9], Wt[9], R1[9], R2[9], tmp[9];
    mat3_transpose(V, Vt);
    mat3_transpose(W, Wt);
    mat3_mul(U, W, tmp);
    mat3_mul(tmp, Vt, R1);
    mat3_mul(U, Wt, tmp);
    mat3_mul(tmp, Vt, R2);
    double tt[3] = {U[2], U[5], U[8]};
    const double tn = std::sqrt(tt[0] * tt[0] + tt[1] * tt[1] + tt[2] * tt[2]);
    for (double& v : tt) v /= tn;
    const double* Rc[4] = {R1, R2, R1, R2};
    const double sg[4] = {1, 1, -1, -1};
    int good[4] = {0, 0, 0, 0};
    const double dist = 50.0;
    for (int c = 0; c < 4; c++) {
        const double tc[3] = {sg[c] * tt[0], sg[c] * tt[1], sg[c] * tt[2]};
        for (int i = 0; i < n; i++) {
            if (mask && !mask[i]) continue;
            double z0, z1;
            triangulate(Rc[c], tc, x0 + 2 * i, x1 + 2 * i, z0, z1);
            if (z0 > 0 && z1 > 0 && z0 < dist && z1 < dist) good[c]++;
        }
    }
    int best = 0;
    for (int c = 1; c < 4; c++)
        if (good[c] > good[best]) best = c;
    std::memcpy(R, Rc[best], 9 * sizeof(double));
    for (int i = 0; i < 3; i++) t[i] = sg[best] * tt[i];
    return good[best];
}

// Rotation exp([w]x) (Rodrigues' formula).
void rodrigues(const double* w, double* R) {
    const double th = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
    if (th < 1e-300) {
        for (int i = 0; i < 9; i++) R[i] = i % 4 == 0 ? 1.0 : 0.0;
        return;
    }
    const double k[3] = {w[0] / th, w[1] / th, w[2] / th};
    const double c = std::cos(th), s = std::sin(th), v = 1.0 - c;
    R[0] = c + k[0] * k[0] * v;
    R[1] = k[0] * k[1] * v - k[2] * s;
    R[2] = k[0] * k[2] * v + k[1] * s;
    R[3] = k[1] * k[0] * v + k[2] * s;
    R[4] = c + k[1] * k[1] * v;
    R[5] = k[1] * k[2] * v - k[0] * s;
    R[6] = k[2] * k[0] * v - k[1] * s;
    R[7] = k[2] * k[1] * v + k[0] * s;
    R[8] = c + k[2] * k[2] * v;
}

// (R, t) moved by p = (w, a, b): R' = exp([w]x) R, t' = unit(t + a b1 + b b2)
// with b1, b2 an orthonormal basis of the plane orthogonal to t.
void perturb(const double* R, const double* t, const double* b1, const double* b2,
             const double* p, double* Ro, double* to) {
    double dR[9];
    rodrigues(p, dR);
    mat3_mul(dR, R, Ro);
    double n = 0.0;
    for (int i = 0; i < 3; i++) {
        to[i] = t[i] + p[3] * b1[i] + p[4] * b2[i];
        n += to[i] * to[i];
    }
    n = std::sqrt(n);
    for (int i = 0; i < 3; i++) to[i] /= n;
}

double sampson_cost(const double* R, const double* t, const double* x0, const double* x1, int n,
                    const unsigned char* mask) {
    double E[9];
    const double S[9] = {0, -t[2], t[1], t[2], 0, -t[0], -t[1], t[0], 0};
    mat3_mul(S, R, E);
    double c = 0.0;
    for (int i = 0; i < n; i++)
        if (!mask || mask[i]) c += sampson2(E, x0 + 2 * i, x1 + 2 * i);
    return c;
}

// Levenberg-Marquardt on the summed squared Sampson distance of the inliers
// over the five degrees of freedom of (R, t) (rotation increment and a move
// of t on the unit sphere), with a forward-difference Jacobian of the
// signed Sampson residuals; stops when a step no longer lowers the cost.
void refine_pose(const double* x0, const double* x1, int n, const unsigned char* mask, double* R,
                 double* t) {
    std::vector<int> idx;
    for (int i = 0; i < n; i++)
        if (!mask || mask[i]) idx.push_back(i);
    const int m = (int)idx.size();
    if (m < 6) return;
    auto residuals = [&](const double* Rr, const double* tr, std::vector<double>& r) {
        double E[9];
        const double S[9] = {0, -tr[2], tr[1], tr[2], 0, -tr[0], -tr[1], tr[0], 0};
        mat3_mul(S, Rr, E);
        for (int k = 0; k < m; k++) {
            const double* a = x0 + 2 * idx[k];
            const double* b = x1 + 2 * idx[k];
            const double xa[3] = {a[0], a[1], 1.0}, xb[3] = {b[0], b[1], 1.0};
            double Ea[3], Etb[3];
            for (int i = 0; i < 3; i++) {
                Ea[i] = E[i * 3] * xa[0] + E[i * 3 + 1] * xa[1] + E[i * 3 + 2] * xa[2];
                Etb[i] = E[i] * xb[0] + E[3 + i] * xb[1] + E[6 + i] * xb[2];
            }
            const double e = xb[0] * Ea[0] + xb[1] * Ea[1] + xb[2] * Ea[2];
            const double d = Ea[0] * Ea[0] + Ea[1] * Ea[1] + Etb[0] * Etb[0] + Etb[1] * Etb[1];
            r[k] = d > 0.0 ? e / std::sqrt(d) : 0.0;
        }
    };
    std::vector<double> r(m), rp(m), J((size_t)m * 5);
    double lambda = 1e-3;
    for (int it = 0; it < 20; it++) {
        // basis orthogonal to t
        double b1[3], b2[3];
        const double ax[3] = {std::fabs(t[0]) < 0.9 ? 1.0 : 0.0, std::fabs(t[0]) < 0.9 ? 0.0 : 1.0, 0.0};
        cross3(t, ax, b1);
        double nb = std::sqrt(b1[0] * b1[0] + b1[1] * b1[1] + b1[2] * b1[2]);
        for (double& v : b1) v /= nb;
        cross3(t, b1, b2);
        residuals(R, t, r);
        double cost = 0.0;
        for (double v : r) cost += v * v;
        const double h = 1e-7;
        for (int q = 0; q < 5; q++) {
            double p[5] = {0, 0, 0, 0, 0};
            p[q] = h;
            double Rq[9], tq[3];
            perturb(R, t, b1, b2, p, Rq, tq);
            residuals(Rq, tq, rp);
            for (int k = 0; k < m; k++) J[(size_t)k * 5 + q] = (rp[k] - r[k]) / h;
        }
        double JtJ[25] = {}, Jtr[5] = {};
        for (int k = 0; k < m; k++)
            for (int a = 0; a < 5; a++) {
                Jtr[a] += J[(size_t)k * 5 + a] * r[k];
                for (int b = 0; b < 5; b++) JtJ[a * 5 + b] += J[(size_t)k * 5 + a] * J[(size_t)k * 5 + b];
            }
        bool improved = false;
        for (int tries = 0; tries < 8 && !improved; tries++) {
            double A[25], g[5];
            for (int a = 0; a < 25; a++) A[a] = JtJ[a];
            for (int a = 0; a < 5; a++) {
                A[a * 5 + a] *= 1.0 + lambda;
                g[a] = -Jtr[a];
            }
            // solve A p = g (Gaussian elimination, partial pivoting)
            for (int c = 0; c < 5; c++) {
                int pv = c;
                for (int rr = c + 1; rr < 5; rr++)
                    if (std::fabs(A[rr * 5 + c]) > std::fabs(A[pv * 5 + c])) pv = rr;
                if (!(std::fabs(A[pv * 5 + c]) > 0.0)) return;
                for (int k = 0; k < 5; k++) std::swap(A[c * 5 + k], A[pv * 5 + k]);
                std::swap(g[c], g[pv]);
                for (int rr = c + 1; rr < 5; rr++) {
                    const double f = A[rr * 5 + c] / A[c * 5 + c];
                    for (int k = c; k < 5; k++) A[rr * 5 + k] -= f * A[c * 5 + k];
                    g[rr] -= f * g[c];
                }
            }
            double p[5];
            for (int c = 4; c >= 0; c--) {
                double v = g[c];
                for (int k = c + 1; k < 5; k++) v -= A[c * 5 + k] * p[k];
                p[c] = v / A[c * 5 + c];
            }
            double Rn[9], tn[3];
            perturb(R, t, b1, b2, p, Rn, tn);
            const double cn = sampson_cost(Rn, tn, x0, x1, n, mask);
            if (cn < cost) {
                std::memcpy(R, Rn, sizeof(Rn));
                std::memcpy(t, tn, sizeof(tn));
                lambda = std::max(lambda * 0.1, 1e-12);
                improved = true;
                if (cost - cn <= 1e-12 * cost) return;
            } else {
                lambda *= 10.0;
            }
        }
        if (!improved) return;
    }
}

}  // namespace rf_epi

using namespace rf_epi;

extern "C" {

RF_API int rf_essential_5pt(const double* x0, const double* x1, double* E) {
    if (!x0 || !x1 || !E) return -1;
    return five_point(x0, x1, E);
}

RF_API rf_status rf_essential_lmeds(const double* x0, const double* x1, int n, double confidence,
                                    unsigned long long seed, double E[9], unsigned char* mask) {
    if (!x0 || !x1 || !E || !mask || n < 5 || !(confidence > 0.0 && confidence < 1.0))
        return RF_ERR_INVALID_ARG;
    return lmeds(x0, x1, n, confidence, seed, E, mask) ? RF_OK : RF_ERR_STATE;
}

RF_API rf_status rf_refine_pose(const double* x0, const double* x1, int n,
                                const unsigned char* mask, double R[9], double t[3]) {
    if (!x0 || !x1 || !R || !t || n < 1) return RF_ERR_INVALID_ARG;
    refine_pose(x0, x1, n, mask, R, t);
    return RF_OK;
}

RF_API rf_status rf_recover_pose(const double E[9], const double* x0, const double* x1, int n,
                                 const unsigned char* mask, double R[9], double t[3],
                                 int* n_good) {
    if (!E || !x0 || !x1 || !R || !t || n < 1) return RF_ERR_INVALID_ARG;
    const int g = recover_pose(E, x0, x1, n, mask, R, t);
    if (n_good) *n_good = g;
    return RF_OK;
}

}  // extern "C"
