// Per-pixel arithmetic of the Reconflow update equations, as __device__ code.
//
// Every expression keeps the reference kernels' operation order and is built
// with -fmad=false (IEEE division / square root, no contraction), so a result
// is a deterministic function of its inputs.  The texture fetches of the
// reference (normalized coordinates, mirror addressing, linear filtering;
// downscale.cu:50-67, upscale.cu:42-58, warpImage.cu:33-50,
// computeDerivatives.cu:60-84) are replaced by explicit exact bilinear
// interpolation with half-sample-symmetric tap indices.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include <utility>

namespace rf {

// Half-sample-symmetric extension of a tap index (period 2n): -1 -> 0,
// -2 -> 1, n -> n-1, n+1 -> n-2.
__device__ __forceinline__ int mirror_index(int i, int n) {
    if (i >= 0 && i < n) return i;
    int p = 2 * n;
    i %= p;
    if (i < 0) i += p;
    return i < n ? i : p - 1 - i;
}

// Mirror addressing of a normalized coordinate (period 2, reflected into
// [0, 1]); a non-finite coordinate reads at 0.
__device__ __forceinline__ float mirror_coord(float t) {
    if (t >= 0.0f && t <= 1.0f) return t;
    if (!isfinite(t)) return 0.0f;
    if (t < 0.0f) t = -t;
    t = fmodf(t, 2.0f);
    if (t > 1.0f) t = 2.0f - t;
    return t;
}

// Tap indices and weights of one linear fetch along an axis of n texels.
struct Taps {
    int i0, i1;
    float a;
};

__device__ __forceinline__ Taps taps_of(float tn, int n) {
    float tm = mirror_coord(tn);
    float tx = tm * (float)n - 0.5f;
    float f = floorf(tx);
    Taps t;
    int x0 = (int)f;
    t.a = tx - f;
    t.i0 = mirror_index(x0, n);
    t.i1 = mirror_index(x0 + 1, n);
    return t;
}

__device__ __forceinline__ float bilerp(const float* __restrict__ src, int s, const Taps& tx,
                                        const Taps& ty) {
    float r0 = (1.0f - tx.a) * src[tx.i0 + ty.i0 * s] + tx.a * src[tx.i1 + ty.i0 * s];
    float r1 = (1.0f - tx.a) * src[tx.i0 + ty.i1 * s] + tx.a * src[tx.i1 + ty.i1 * s];
    return (1.0f - ty.a) * r0 + ty.a * r1;
}

__device__ __forceinline__ float tex2d(const float* __restrict__ src, int W, int H, int S,
                                       float xn, float yn) {
    Taps tx = taps_of(xn, W);
    Taps ty = taps_of(yn, H);
    return bilerp(src, S, tx, ty);
}

__device__ __forceinline__ bool finite3(float a, float b, float c) {
    return isfinite(a) && isfinite(b) && isfinite(c);
}

// Divergence of the dual field with one-sided borders
// (solveReconDataL1.cu:66-97).  l = p1 at x-1, d = p2 at y-1.
__device__ __forceinline__ float divergence(float p1, float p1l, float p2, float p2d, int ix,
                                            int iy) {
    if (ix - 1 < 0) {
        if (iy - 1 < 0) return p1 + p2;
        return p1 + p2 - p2d;
    }
    if (iy - 1 < 0) return p1 - p1l + p2;
    return p1 - p1l + p2 - p2d;
}

// L1 threshold step of the ReconFlow data term (solveReconDataL1.cu:36-63).
// A = alphaTv + alphaProj (+ alphaFn); `upper` = lambda*g/A.
__device__ __forceinline__ void l1_threshold(float dusub, float dvsub, float dix, float diy,
                                             float dit, float lambda, float A, float& du,
                                             float& dv) {
    float rho = (dix * dusub + diy * dvsub + dit);
    float upper = lambda * (dix * dix + diy * diy) / A;
    float lower = -upper;  // == -lambda*g/A exactly (negation is exact)
    // The three branches differ only in the numerator factor, the divisor and
    // the sign of the step, so each component takes one division whichever
    // branch its pixel is in (a warp whose pixels diverge would otherwise run
    // the divisions of every branch); every value is formed exactly as the
    // branch formulas form it.
    const bool inside = (rho <= upper) && (rho >= lower);
    const float magi = dix * dix + diy * diy;
    const bool step = inside ? (magi != 0) : (rho < lower || rho > upper);  // NaN rho: no step
    const float fac = inside ? rho : lambda;
    const float den = inside ? magi : A;
    const float qu = fac * dix / (step ? den : 1.0f);
    const float qv = fac * diy / (step ? den : 1.0f);
    const bool plus = !inside && (rho < lower);
    du = !step ? dusub : (plus ? dusub + qu : dusub - qu);
    dv = !step ? dvsub : (plus ? dvsub + qv : dvsub - qv);
}

// Plain TV-L1 threshold step (solveDataL1.cu:27-51); lt = lambda*theta.
__device__ __forceinline__ void l1_threshold_plain(float duhat, float dvhat, float dix, float diy,
                                                   float dit, float lambda, float theta,
                                                   float& du, float& dv) {
    float rho = (dix * duhat + diy * dvhat + dit);
    float upper = lambda * theta * (dix * dix + diy * diy);
    float lower = -lambda * theta * (dix * dix + diy * diy);
    du = duhat;
    dv = dvhat;
    if ((rho <= upper) && (rho >= lower)) {
        float magi = dix * dix + diy * diy;
        if (magi != 0) {
            du = duhat - rho * dix / magi;
            dv = dvhat - rho * diy / magi;
        }
    } else if (rho < lower) {
        du = duhat + lambda * theta * dix;
        dv = dvhat + lambda * theta * diy;
    } else if (rho > upper) {
        du = duhat - lambda * theta * dix;
        dv = dvhat - lambda * theta * diy;
    }
}

// Semi-implicit dual step (solveSmoothDualTVGlobal.cu:46-60); fac = tau/theta.
__device__ __forceinline__ void dual_step(float dx, float dy, float fac, float& p1, float& p2) {
    float mag = sqrtf(dx * dx + dy * dy);
    float den = 1.0f + fac * mag;
    p1 = (p1 + fac * dx) / den;
    p2 = (p2 + fac * dy) / den;
}

// Per-level camera constants (float copies, as the reference passes them:
// solve3dMinimalArea.cu:204-228, solveUcSk.cu:42-56).  16-byte aligned (52
// floats = 13 x 16 bytes) so a thread reads them with 128-bit loads.
struct __align__(16) LevelConsts {
    float P[12];
    float Q[12];
    float R1[9];
    float t1[3];
    float focal, cx, cy;
    float pad;
};

// SolveUcKernel (solveUcSk.cu:21-33).
__device__ __forceinline__ void project_uc(const LevelConsts& c, float X, float Y, float Z, int ix,
                                           int iy, float& uc, float& vc) {
    float X2 = c.R1[0] * X + c.R1[1] * Y + c.R1[2] * Z + c.t1[0];
    float Y2 = c.R1[3] * X + c.R1[4] * Y + c.R1[5] * Z + c.t1[1];
    float Z2 = c.R1[6] * X + c.R1[7] * Y + c.R1[8] * Z + c.t1[2];
    float xproj = c.focal * X2 / Z2 + c.cx;
    float yproj = c.focal * Y2 / Z2 + c.cy;
    uc = xproj - (float)ix;
    vc = yproj - (float)iy;
}

// Solve3dMinimalAreaKernel body (solve3dMinimalArea.cu:23-184).  nb[] holds
// X0, Y0, Z0 at: 0 = pos, 1 = x+1 (flat pos+1), 2 = y+1 (flat pos+stride),
// 3 = x-1, 4 = y-1 (3, 4 unused at the left / top border).
__device__ __forceinline__ void solve3d_pixel(const LevelConsts& c, float uproj, float vproj,
                                              int ix, int iy, const float (&Xn)[5],
                                              const float (&Yn)[5], const float (&Zn)[5],
                                              float lambdaf, float lambdams, float& Xo, float& Yo,
                                              float& Zo) {
    const float* P = c.P;
    const float* Q = c.Q;
    float x1 = (float)ix;
    float y1 = (float)iy;
    float x2 = (float)ix + uproj;
    float y2 = (float)iy + vproj;

    float p1 = x1 * P[8] - P[0], p2 = x1 * P[9] - P[1], p3 = x1 * P[10] - P[2], p4 = x1 * P[11] - P[3];
    float q1 = y1 * P[8] - P[4], q2 = y1 * P[9] - P[5], q3 = y1 * P[10] - P[6], q4 = y1 * P[11] - P[7];
    float r1 = x2 * Q[8] - Q[0], r2 = x2 * Q[9] - Q[1], r3 = x2 * Q[10] - Q[2], r4 = x2 * Q[11] - Q[3];
    float s1 = y2 * Q[8] - Q[4], s2 = y2 * Q[9] - Q[5], s3 = y2 * Q[10] - Q[6], s4 = y2 * Q[11] - Q[7];

    float ax = lambdaf * (p1 * p1 + q1 * q1 + r1 * r1 + s1 * s1);
    float bx = lambdaf * (p1 * p2 + q1 * q2 + r1 * r2 + s1 * s2);
    float cx = lambdaf * (p1 * p3 + q1 * q3 + r1 * r3 + s1 * s3);
    float dx = lambdaf * (p1 * p4 + q1 * q4 + r1 * r4 + s1 * s4);
    float ay = lambdaf * (p2 * p1 + q2 * q1 + r2 * r1 + s2 * s1);
    float by = lambdaf * (p2 * p2 + q2 * q2 + r2 * r2 + s2 * s2);
    float cy = lambdaf * (p2 * p3 + q2 * q3 + r2 * r3 + s2 * s3);
    float dy = lambdaf * (p2 * p4 + q2 * q4 + r2 * r4 + s2 * s4);
    float az = lambdaf * (p3 * p1 + q3 * q1 + r3 * r1 + s3 * s1);
    float bz = lambdaf * (p3 * p2 + q3 * q2 + r3 * r2 + s3 * s2);
    float cz = lambdaf * (p3 * p3 + q3 * q3 + r3 * r3 + s3 * s3);
    float dz = lambdaf * (p3 * p4 + q3 * q4 + r3 * r4 + s3 * s4);

    float Xx = Xn[1] - Xn[0], Yx = Yn[1] - Yn[0], Zx = Zn[1] - Zn[0];
    float Xy = Xn[2] - Xn[0], Yy = Yn[2] - Yn[0], Zy = Zn[2] - Zn[0];

    float lambetams = lambdams / sqrtf((Yx * Zy - Zx * Yy) * (Yx * Zy - Zx * Yy) +
                                       (Zx * Xy - Xx * Zy) * (Zx * Xy - Xx * Zy) +
                                       (Xx * Yy - Yx * Xy) * (Xx * Yy - Yx * Xy) + 0.001f);

    float Xibar, Yibar, Zibar, Xjbar, Yjbar, Zjbar;
    if (ix - 1 < 0) {
        Xibar = Xn[1];
        Yibar = Yn[1];
        Zibar = Zn[1];
    } else {
        Xibar = 0.5f * Xn[3] + 0.5f * Xn[1];
        Yibar = 0.5f * Yn[3] + 0.5f * Yn[1];
        Zibar = 0.5f * Zn[3] + 0.5f * Zn[1];
    }
    if (iy - 1 < 0) {
        Xjbar = Xn[2];
        Yjbar = Yn[2];
        Zjbar = Zn[2];
    } else {
        Xjbar = 0.5f * Xn[4] + 0.5f * Xn[2];
        Yjbar = 0.5f * Yn[4] + 0.5f * Yn[2];
        Zjbar = 0.5f * Zn[4] + 0.5f * Zn[2];
    }

    float a11 = ax + lambetams * (Yx * Yx + Zx * Zx + Yy * Yy + Zy * Zy);
    float a12 = bx - lambetams * (Xx * Yx + Xy * Yy);
    float a13 = cx - lambetams * (Xx * Zx + Xy * Zy);
    float a21 = ay - lambetams * (Xx * Yx + Xy * Yy);
    float a22 = by + lambetams * (Xx * Xx + Zx * Zx + Xy * Xy + Zy * Zy);
    float a23 = cy - lambetams * (Yx * Zx + Yy * Zy);
    float a31 = az - lambetams * (Xx * Zx + Xy * Zy);
    float a32 = bz - lambetams * (Yx * Zx + Yy * Zy);
    float a33 = cz + lambetams * (Xx * Xx + Yx * Yx + Xy * Xy + Yy * Yy);

    float detA = a11 * (a22 * a33 - a23 * a32) - a12 * (a21 * a33 - a23 * a31) +
                 a13 * (a21 * a32 - a22 * a31);

    float E11 = a22 * a33 - a23 * a32;
    float E12 = a13 * a32 - a12 * a33;
    float E13 = a12 * a23 - a13 * a22;
    float E21 = a23 * a31 - a21 * a33;
    float E22 = a11 * a33 - a13 * a31;
    float E23 = a13 * a21 - a11 * a23;
    float E31 = a21 * a32 - a22 * a31;
    float E32 = a12 * a31 - a11 * a32;
    float E33 = a11 * a22 - a12 * a21;

    float b1 = lambetams * ((Zy * Zy + Yy * Yy) * Xibar + (Zx * Zx + Yx * Yx) * Xjbar -
                            (Xy * Yy) * Yibar - (Xx * Yx) * Yjbar - (Xy * Zy) * Zibar -
                            (Xx * Zx) * Zjbar) -
               dx;
    float b2 = lambetams * (-(Xy * Yy) * Xibar - (Xx * Yx) * Xjbar + (Xy * Xy + Zy * Zy) * Yibar +
                            (Xx * Xx + Zx * Zx) * Yjbar - (Yy * Zy) * Zibar - (Yx * Zx) * Zjbar) -
               dy;
    float b3 = lambetams * (-(Xy * Zy) * Xibar - (Xx * Zx) * Xjbar - (Yy * Zy) * Yibar -
                            (Yx * Zx) * Yjbar + (Xy * Xy + Yy * Yy) * Zibar +
                            (Xx * Xx + Yx * Yx) * Zjbar) -
               dz;

    float Xsub = (E11 * b1 + E12 * b2 + E13 * b3) / detA;
    float Ysub = (E21 * b1 + E22 * b2 + E23 * b3) / detA;
    float Zsub = (E31 * b1 + E32 * b2 + E33 * b3) / detA;

    if (finite3(Xsub, Ysub, Zsub)) {
        Xo = Xsub;
        Yo = Ysub;
        Zo = Zsub;
    } else {
        Xo = Xn[0];
        Yo = Yn[0];
        Zo = Zn[0];
    }
}

// Exchange-selection median of 9 (medianFilter.cu:216-242): 5 passes, the
// reference's compare order, so ties (+0/-0) resolve identically.
__device__ __forceinline__ float median9_exchange(float (&m)[9]) {
#pragma unroll
    for (int j = 0; j < 5; j++) {
#pragma unroll
        for (int i = j + 1; i < 9; i++) {
            if (m[j] > m[i]) {
                float t = m[j];
                m[j] = m[i];
                m[i] = t;
            }
        }
    }
    return m[4];
}

// Median of 9 finite values with the 19-comparator min/max network for the
// 3x3 median (A. Paeth, "Median finding on a 3x3 grid", Graphics Gems, 1990,
// in N. Devillard's ordering).  For finite inputs its value equals the
// exchange selection's; the two can differ only in the sign of a zero
// result, so a zero result is recomputed with the reference's exchange order.
// Inputs must not be NaN (the 3D state fed to it is finite by construction).
__device__ __forceinline__ float median9_finite(const float (&in)[9]) {
    float p0 = in[0], p1 = in[1], p2 = in[2], p3 = in[3], p4 = in[4], p5 = in[5], p6 = in[6],
          p7 = in[7], p8 = in[8];
#define RF_SORT2(a, b)            \
    {                             \
        float lo__ = fminf(a, b); \
        b = fmaxf(a, b);          \
        a = lo__;                 \
    }
    RF_SORT2(p1, p2); RF_SORT2(p4, p5); RF_SORT2(p7, p8);
    RF_SORT2(p0, p1); RF_SORT2(p3, p4); RF_SORT2(p6, p7);
    RF_SORT2(p1, p2); RF_SORT2(p4, p5); RF_SORT2(p7, p8);
    p3 = fmaxf(p0, p3);
    p5 = fminf(p5, p8);
    RF_SORT2(p4, p7);
    p6 = fmaxf(p3, p6);
    p4 = fmaxf(p1, p4);
    p2 = fminf(p2, p5);
    p4 = fminf(p4, p7);
    RF_SORT2(p4, p2);
    p4 = fmaxf(p6, p4);
    p4 = fminf(p4, p2);
#undef RF_SORT2
    if (p4 == 0.0f) {
        float m[9];
#pragma unroll
        for (int k = 0; k < 9; k++) m[k] = in[k];
        return median9_exchange(m);
    }
    return p4;
}

// Exchange-selection median of 25 (medianFilter.cu:55-74): 13 passes.
__device__ __forceinline__ float median25_exchange(float (&m)[25]) {
#pragma unroll
    for (int j = 0; j < 13; j++) {
#pragma unroll
        for (int i = j + 1; i < 25; i++) {
            if (m[j] > m[i]) {
                float t = m[j];
                m[j] = m[i];
                m[i] = t;
            }
        }
    }
    return m[12];
}

// Comparators of Batcher's odd-even merge sort of 32 keys (K. E. Batcher,
// "Sorting networks and their applications", AFIPS SJCC 1968), keeping only
// those whose both keys are among the first 25: a comparator against a key
// >= 25 would meet +inf padding and change nothing.  The 140 comparators
// sort 25 keys; the median needs the 113 of them that reach key 12, and the
// compiler drops the rest once the loop below is unrolled.
constexpr int sortnet25_count_or_pair(int want, int which) {
    int n = 0;
    for (int p = 1; p < 32; p <<= 1)
        for (int k = p; k >= 1; k >>= 1)
            for (int j = k % p; j + k < 32; j += 2 * k)
                for (int i = 0; i < k && i < 32 - j - k; i++)
                    if ((i + j) / (2 * p) == (i + j + k) / (2 * p) && i + j + k < 25) {
                        if (n == want) return which == 0 ? i + j : i + j + k;
                        n++;
                    }
    return n;  // want < 0: the comparator count
}
constexpr int kSortNet25 = sortnet25_count_or_pair(-1, 0);

template <int A, int B>
__device__ __forceinline__ void cmp_exchange(float (&s)[25]) {
    const float lo = fminf(s[A], s[B]);
    s[B] = fmaxf(s[A], s[B]);
    s[A] = lo;
}

template <int... C>
__device__ __forceinline__ void sortnet25(float (&s)[25], std::integer_sequence<int, C...>) {
    (cmp_exchange<sortnet25_count_or_pair(C, 0), sortnet25_count_or_pair(C, 1)>(s), ...);
}

// The same construction for any key count N <= 32 (comparators of the
// 32-key merge sort whose keys are both below N); used for the 20 shared
// and the 5 own taps of two vertically adjacent 5x5 windows.
template <int N>
constexpr int batcher_count_or_pair(int want, int which) {
    int n = 0;
    for (int p = 1; p < 32; p <<= 1)
        for (int k = p; k >= 1; k >>= 1)
            for (int j = k % p; j + k < 32; j += 2 * k)
                for (int i = 0; i < k && i < 32 - j - k; i++)
                    if ((i + j) / (2 * p) == (i + j + k) / (2 * p) && i + j + k < N) {
                        if (n == want) return which == 0 ? i + j : i + j + k;
                        n++;
                    }
    return n;
}

template <int N, int A, int B>
__device__ __forceinline__ void cmp_exchange_n(float (&s)[N]) {
    const float lo = fminf(s[A], s[B]);
    s[B] = fmaxf(s[A], s[B]);
    s[A] = lo;
}

template <int N, int... C>
__device__ __forceinline__ void batcher_sort_seq(float (&s)[N], std::integer_sequence<int, C...>) {
    (cmp_exchange_n<N, batcher_count_or_pair<N>(C, 0), batcher_count_or_pair<N>(C, 1)>(s), ...);
}

template <int N>
__device__ __forceinline__ void batcher_sort(float (&s)[N]) {
    batcher_sort_seq(s, std::make_integer_sequence<int, batcher_count_or_pair<N>(-1, 0)>{});
}

// Medians of two vertically adjacent 5x5 windows.  `w` holds six rows of
// five taps: pixel 0's window is rows 0-4, pixel 1's rows 1-5.  The 20 taps
// of rows 1-4 are sorted once (A) and each pixel's own row (B) on its own;
// the 13th smallest of the union of the sorted A and B is
// min over i = 0..5 of max(A[12 - i], B[i - 1]) (i taps taken from B;
// B[-1] = -inf), the selection of the k-th element of two sorted lists.
// Without NaN inputs every min / max returns one of its operands, so a
// non-zero result is bitwise the value the reference's exchange selection
// returns (equal non-zero floats have equal bits); returns false when an
// input is NaN, and the caller takes the exchange path (also for a zero
// result, whose sign the exchange order decides).
__device__ __forceinline__ bool median25_two(const float (&w)[30], float& m0, float& m1) {
    bool nan_in = false;
#pragma unroll
    for (int k = 0; k < 30; k++) nan_in |= isnan(w[k]);
    if (nan_in) return false;
    float A[20], B0[5], B1[5];
#pragma unroll
    for (int k = 0; k < 20; k++) A[k] = w[5 + k];
#pragma unroll
    for (int k = 0; k < 5; k++) {
        B0[k] = w[k];
        B1[k] = w[25 + k];
    }
    batcher_sort(A);
    batcher_sort(B0);
    batcher_sort(B1);
    m0 = A[12];
    m1 = A[12];
#pragma unroll
    for (int i = 1; i <= 5; i++) {
        m0 = fminf(m0, fmaxf(A[12 - i], B0[i - 1]));
        m1 = fminf(m1, fmaxf(A[12 - i], B1[i - 1]));
    }
    return true;
}

// Median of 25 with the min/max network above, sorting `s` in place.  For
// inputs without NaN the network's key 12 is the value the exchange
// selection (median25_exchange) returns, except possibly for the sign of a
// zero; returns false when that answer is not certain (a NaN input or a zero
// result), and the caller then takes the exchange path on the inputs.
__device__ __forceinline__ bool median25_net(float (&s)[25], float& out) {
    bool nan_in = false;
#pragma unroll
    for (int k = 0; k < 25; k++) nan_in |= isnan(s[k]);
    if (nan_in) return false;
    sortnet25(s, std::make_integer_sequence<int, kSortNet25>{});
    out = s[12];
    return out != 0.0f;
}

// The exchange selection's answer when median25_net gave none: a zero result
// whose inputs hold zeros of one sign only is that zero (the selection moves
// values, it never makes one); otherwise the exchange order decides.
__device__ __forceinline__ float median25_resolve(float (&m)[25]) {
    bool nan_in = false, pos0 = false, neg0 = false;
#pragma unroll
    for (int k = 0; k < 25; k++) {
        nan_in |= isnan(m[k]);
        const unsigned b = __float_as_uint(m[k]);
        pos0 |= b == 0u;
        neg0 |= b == 0x80000000u;
    }
    if (!nan_in && !(pos0 && neg0)) return neg0 ? -0.0f : 0.0f;
    return median25_exchange(m);
}

// CleanUp3DKernel body (solve3dMinimalArea.cu:259-295).
__device__ __forceinline__ void cleanup_pixel(float X, float Y, float Z, float Xm, float Ym,
                                              float Zm, float& Xo, float& Yo, float& Zo) {
    if (finite3(X, Y, Z) && finite3(Xm, Ym, Zm)) {
        Xo = fabsf(Xm - X) > 5.0f ? Xm : X;
        Yo = fabsf(Ym - Y) > 5.0f ? Ym : Y;
        Zo = fabsf(Zm - Z) > 5.0f ? Zm : Z;
    } else {
        Xo = 0.0f;
        Yo = 0.0f;
        Zo = 0.0f;
    }
}

}  // namespace rf
