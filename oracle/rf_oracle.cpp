// Oracle for the Reconflow flow+depth path: TEST INFRASTRUCTURE ONLY.
//
// A plain CPU restatement of the reference's update equations and schedule,
// templated on the arithmetic type: `double` is the FP64 oracle that parity is
// measured against, `float` is the reference-semantics FP32 path (IEEE
// division and square root, no contraction: build with -ffp-contract=off)
// that doubles as the timed CPU baseline.  Only tests/, the smoke check and
// the CPU-baseline leg of the benchmark may load this library; the product
// never does.
//
// Every function cites the reference file:line it restates (paths relative to
// the menandro/Reconflow project root).  Where the reference depends on GPU
// texture hardware or reads memory it never wrote, this file DEFINES the
// behaviour (documented at each site) and the CUDA kernels follow the same
// definition:
//   * texture fetches (normalized coords, mirror addressing, linear filter)
//     are exact bilinear interpolation with half-sample-symmetric tap indices;
//   * derivative taps land on texel centres and are plain gathers;
//   * reads of row `height` past the level-0 allocation return 0;
//   * a data-term pixel whose residual is NaN keeps the blended value.
// Parity status: the reference has no tests, no golden outputs and does not
// build here (OpenCV absent; legacy texture references were removed in
// CUDA 12), so this restatement is pinned only through the tests' analytic
// known answers and properties.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------------------
// Sizes and index helpers
// ---------------------------------------------------------------------------

// Cudaflow.cu:984-994 (iAlignUp)
inline int align_up(int n, int m) {
    int mod = n % m;
    return mod ? n + m - mod : n;
}

// Cudaflow.cu:146-171: level sizes; newH = (int)(h / fScale) in float.
void pyramid_dims(int w, int h, int levels, float scale, int align,
                  int* W, int* H, int* S) {
    int nh = h, nw = w, ns = align_up(w, align);
    for (int l = 0; l < levels; l++) {
        W[l] = nw; H[l] = nh; S[l] = ns;
        nh = (int)((float)nh / scale);
        nw = (int)((float)nw / scale);
        ns = align_up(nw, align);
    }
}

// Half-sample-symmetric extension of an integer tap index (period 2n):
// -1 -> 0, -2 -> 1, n -> n-1, n+1 -> n-2.  This is what mirror addressing
// gives for the taps of a linear texture fetch.
inline int mirror_index(int i, int n) {
    int p = 2 * n;
    i %= p;
    if (i < 0) i += p;
    return i < n ? i : p - 1 - i;
}

// cudaAddressModeMirror on a normalized coordinate: reflect into [0, 1]
// with period 2.  A non-finite coordinate is defined to read at 0.
template <typename T>
inline T mirror_coord(T t) {
    if (t >= T(0) && t <= T(1)) return t;
    if (!std::isfinite(t)) return T(0);
    if (t < T(0)) t = -t;
    t = std::fmod(t, T(2));
    if (t > T(1)) t = T(2) - t;
    return t;
}

// tex2D with normalized coordinates, mirror addressing and linear filtering
// (downscale.cu:50-67, upscale.cu:42-58, warpImage.cu:33-50 bind textures this
// way).  Exact weights replace the hardware's 8-bit filter fractions.
template <typename T>
T tex2d(const T* src, int W, int H, int S, T xn, T yn) {
    T xm = mirror_coord(xn);
    T ym = mirror_coord(yn);
    T tx = xm * (T)W - T(0.5);
    T ty = ym * (T)H - T(0.5);
    T fx = std::floor(tx);
    T fy = std::floor(ty);
    int x0 = (int)fx, y0 = (int)fy;
    T a = tx - fx;
    T b = ty - fy;
    int xa = mirror_index(x0, W), xb = mirror_index(x0 + 1, W);
    int ya = mirror_index(y0, H), yb = mirror_index(y0 + 1, H);
    T r0 = (T(1) - a) * src[xa + ya * S] + a * src[xb + ya * S];
    T r1 = (T(1) - a) * src[xa + yb * S] + a * src[xb + yb * S];
    return (T(1) - b) * r0 + b * r1;
}

template <typename T>
inline bool finite3(T a, T b, T c) {
    return std::isfinite(a) && std::isfinite(b) && std::isfinite(c);
}

// ---------------------------------------------------------------------------
// Per-kernel restatements (one loop nest per reference kernel)
// ---------------------------------------------------------------------------

// rgbToGray.cu:3-19 (rgbaToGrayKernel): ((r+g+b)/3)/256
template <typename T>
void k_rgb_to_gray(const uint8_t* rgb, int w, int h, int s, T* out) {
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            int i = x + y * s;
            T g = ((T)rgb[3 * i] + (T)rgb[3 * i + 1] + (T)rgb[3 * i + 2]) / T(3);
            out[i] = g / T(256);
        }
}

// rgbToGray.cu:21-36 (Cv8uToGray), :38-52 (Cv16uToGray), :66-77 (Cv32fToGray)
template <typename T>
void k_u8_to_gray(const uint8_t* in, int w, int h, int s, T* out) {
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) out[x + y * s] = (T)in[x + y * s] / T(256);
}
template <typename T>
void k_u16_to_gray(const uint16_t* in, int w, int h, int s, T* out) {
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) out[x + y * s] = (T)in[x + y * s] / T(65536);
}
template <typename T>
void k_f32_to_gray(const float* in, int w, int h, int s, T* out) {
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) out[x + y * s] = (T)in[x + y * s];
}

// downscale.cu:6-26 (DownscaleKernel) and :28-48 (DownscaleScalingKernel,
// scale != 1).  Four fetches at +-1/4 of a coarse texel around its centre.
template <typename T>
void k_downscale(const T* src, int w, int h, int s, int nw, int nh, int ns,
                 T scale, bool scaled, T* out) {
#pragma omp parallel for schedule(static)
    for (int iy = 0; iy < nh; iy++)
        for (int ix = 0; ix < nw; ix++) {
            T dx = T(1) / (T)nw;
            T dy = T(1) / (T)nh;
            T x = ((T)ix + T(0.5)) * dx;
            T y = ((T)iy + T(0.5)) * dy;
            T sum = tex2d(src, w, h, s, x - dx * T(0.25), y) +
                    tex2d(src, w, h, s, x + dx * T(0.25), y) +
                    tex2d(src, w, h, s, x, y - dy * T(0.25)) +
                    tex2d(src, w, h, s, x, y + dy * T(0.25));
            out[ix + iy * ns] = scaled ? scale * T(0.25) * sum : T(0.25) * sum;
        }
}

// upscale.cu:14-27 (UpscaleKernel): fetch the coarse field at the fine
// centres, times `scale`.
template <typename T>
void k_upscale(const T* src, int w, int h, int s, int nw, int nh, int ns, T scale, T* out) {
#pragma omp parallel for schedule(static)
    for (int iy = 0; iy < nh; iy++)
        for (int ix = 0; ix < nw; ix++) {
            T x = ((T)ix + T(0.5)) / (T)nw;
            T y = ((T)iy + T(0.5)) / (T)nh;
            out[ix + iy * ns] = tex2d(src, w, h, s, x, y) * scale;
        }
}

// warpImage.cu:15-29 (WarpingKernel): I1 fetched at (ix+u+0.5, iy+v+0.5)/size.
template <typename T>
void k_warp(const T* src, int w, int h, int s, const T* u, const T* v, T* out) {
#pragma omp parallel for schedule(static)
    for (int iy = 0; iy < h; iy++)
        for (int ix = 0; ix < w; ix++) {
            int pos = ix + iy * s;
            T x = ((T)ix + u[pos] + T(0.5)) / (T)w;
            T y = ((T)iy + v[pos] + T(0.5)) / (T)h;
            out[pos] = tex2d(src, w, h, s, x, y);
        }
}

// computeDerivatives.cu:8-57: 5-tap central differences [1,-8,0,8,-1]/12 of
// I0 and the warped I1, averaged; Iz = I1w - I0.  The taps sit on texel
// centres, so each fetch is a gather with mirrored indices.
template <typename T>
void k_derivatives(const T* I0, const T* I1, int w, int h, int s, T* Ix, T* Iy, T* Iz) {
#pragma omp parallel for schedule(static)
    for (int iy = 0; iy < h; iy++)
        for (int ix = 0; ix < w; ix++) {
            int pos = ix + iy * s;
            int xm2 = mirror_index(ix - 2, w) + iy * s, xm1 = mirror_index(ix - 1, w) + iy * s;
            int xp1 = mirror_index(ix + 1, w) + iy * s, xp2 = mirror_index(ix + 2, w) + iy * s;
            int ym2 = ix + mirror_index(iy - 2, h) * s, ym1 = ix + mirror_index(iy - 1, h) * s;
            int yp1 = ix + mirror_index(iy + 1, h) * s, yp2 = ix + mirror_index(iy + 2, h) * s;
            T t0, t1;
            t0 = I0[xm2];
            t0 -= I0[xm1] * T(8);
            t0 += I0[xp1] * T(8);
            t0 -= I0[xp2];
            t0 /= T(12);
            t1 = I1[xm2];
            t1 -= I1[xm1] * T(8);
            t1 += I1[xp1] * T(8);
            t1 -= I1[xp2];
            t1 /= T(12);
            Ix[pos] = (t0 + t1) * T(0.5);
            Iz[pos] = I1[pos] - I0[pos];
            t0 = I0[ym2];
            t0 -= I0[ym1] * T(8);
            t0 += I0[yp1] * T(8);
            t0 -= I0[yp2];
            t0 /= T(12);
            t1 = I1[ym2];
            t1 -= I1[ym1] * T(8);
            t1 += I1[yp1] * T(8);
            t1 -= I1[yp2];
            t1 /= T(12);
            Iy[pos] = (t0 + t1) * T(0.5);
        }
}

// Divergence of the dual field with the reference's one-sided borders
// (solveReconDataL1.cu:66-97, solveDataL1.cu:53-85).
template <typename T>
inline T divergence(const T* p1, const T* p2, int ix, int iy, int s) {
    int pos = ix + iy * s;
    if (ix - 1 < 0) {
        if (iy - 1 < 0) return p1[pos] + p2[pos];
        return p1[pos] + p2[pos] - p2[pos - s];
    }
    if (iy - 1 < 0) return p1[pos] - p1[pos - 1] + p2[pos];
    return p1[pos] - p1[pos - 1] + p2[pos] - p2[pos - s];
}

// solveReconDataL1.cu:4-102 (plain), :139-240 (dense prior, mask == null),
// :276-378 (sparse prior, per-pixel mask).  `prior` selects the variant.
template <typename T>
void k_recon_data_l1(const T* u0, const T* v0, const T* duhat0, const T* dvhat0,
                     const T* uproj0, const T* vproj0, const T* ufn0, const T* vfn0,
                     const T* fnmask, const T* sku0, const T* skv0,
                     const T* pu1, const T* pu2, const T* pv1, const T* pv2,
                     const T* Ix, const T* Iy, const T* It, int w, int h, int s,
                     T lambda, T alphaTv, T alphaProj, T alphaFnVal, int prior,
                     T* duhat1, T* dvhat1) {
#pragma omp parallel for schedule(static)
    for (int iy = 0; iy < h; iy++)
        for (int ix = 0; ix < w; ix++) {
            int pos = ix + iy * s;
            T dix = Ix[pos], diy = Iy[pos], dit = It[pos];
            T duhat = duhat0[pos], dvhat = dvhat0[pos];
            T uproj = uproj0[pos], vproj = vproj0[pos];
            T u = u0[pos], v = v0[pos];
            T sku = sku0[pos], skv = skv0[pos];
            T A, dusub, dvsub;
            if (prior == 0) {
                A = alphaTv + alphaProj;
                dusub = (alphaTv * duhat + alphaProj * (uproj - u - sku)) / (alphaTv + alphaProj);
                dvsub = (alphaTv * dvhat + alphaProj * (vproj - v - skv)) / (alphaTv + alphaProj);
            } else {
                T alphaFn = prior == 2 ? alphaFnVal * fnmask[pos] : alphaFnVal;
                T ufn = ufn0[pos], vfn = vfn0[pos];
                A = alphaTv + alphaProj + alphaFn;
                dusub = (alphaFn * (ufn - u) + alphaTv * duhat + alphaProj * (uproj - u - sku)) /
                        (alphaTv + alphaProj + alphaFn);
                dvsub = (alphaFn * (vfn - v) + alphaTv * dvhat + alphaProj * (vproj - v - skv)) /
                        (alphaTv + alphaProj + alphaFn);
            }
            T rho = (dix * dusub + diy * dvsub + dit);
            T upper = lambda * (dix * dix + diy * diy) / A;
            T lower = -lambda * (dix * dix + diy * diy) / A;
            T du = dusub, dv = dvsub;  // NaN residual: defined to keep the blend
            if ((rho <= upper) && (rho >= lower)) {
                T magi = dix * dix + diy * diy;
                if (magi != 0) {
                    du = dusub - rho * dix / magi;
                    dv = dvsub - rho * diy / magi;
                }
            } else if (rho < lower) {
                du = dusub + lambda * dix / A;
                dv = dvsub + lambda * diy / A;
            } else if (rho > upper) {
                du = dusub - lambda * dix / A;
                dv = dvsub - lambda * diy / A;
            }
            T divpu = divergence(pu1, pu2, ix, iy, s);
            T divpv = divergence(pv1, pv2, ix, iy, s);
            duhat1[pos] = du + divpu / A;
            dvhat1[pos] = dv + divpv / A;
        }
}

// solveDataL1.cu:4-91 (plain TV-L1 threshold step)
template <typename T>
void k_data_l1(const T* duhat0, const T* dvhat0, const T* pu1, const T* pu2,
               const T* pv1, const T* pv2, const T* Ix, const T* Iy, const T* It,
               int w, int h, int s, T lambda, T theta, T* duhat1, T* dvhat1) {
#pragma omp parallel for schedule(static)
    for (int iy = 0; iy < h; iy++)
        for (int ix = 0; ix < w; ix++) {
            int pos = ix + iy * s;
            T dix = Ix[pos], diy = Iy[pos], dit = It[pos];
            T duhat = duhat0[pos], dvhat = dvhat0[pos];
            T rho = (dix * duhat + diy * dvhat + dit);
            T upper = lambda * theta * (dix * dix + diy * diy);
            T lower = -lambda * theta * (dix * dix + diy * diy);
            T du = duhat, dv = dvhat;
            if ((rho <= upper) && (rho >= lower)) {
                T magi = dix * dix + diy * diy;
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
            T divpu = divergence(pu1, pu2, ix, iy, s);
            T divpv = divergence(pv1, pv2, ix, iy, s);
            duhat1[pos] = du + theta * divpu;
            dvhat1[pos] = dv + theta * divpv;
        }
}

// solveSmoothDualTVGlobal.cu:4-65: forward differences (0 at the far
// border), semi-implicit dual step.
template <typename T>
void k_dual_tv(const T* duhat, const T* dvhat, const T* pu1, const T* pu2,
               const T* pv1, const T* pv2, int w, int h, int s, T tau, T theta,
               T* pu1s, T* pu2s, T* pv1s, T* pv2s) {
#pragma omp parallel for schedule(static)
    for (int iy = 0; iy < h; iy++)
        for (int ix = 0; ix < w; ix++) {
            int pos = ix + iy * s;
            T dux, duy, dvx, dvy;
            if ((ix + 1) >= w) {
                dux = 0;
                dvx = 0;
            } else {
                dux = duhat[pos + 1] - duhat[pos];
                dvx = dvhat[pos + 1] - dvhat[pos];
            }
            if ((iy + 1) >= h) {
                duy = 0;
                dvy = 0;
            } else {
                duy = duhat[pos + s] - duhat[pos];
                dvy = dvhat[pos + s] - dvhat[pos];
            }
            T magdu = std::sqrt(dux * dux + duy * duy);
            T magdv = std::sqrt(dvx * dvx + dvy * dvy);
            T fac = tau / theta;
            pu1s[pos] = (pu1[pos] + fac * dux) / (T(1) + fac * magdu);
            pu2s[pos] = (pu2[pos] + fac * duy) / (T(1) + fac * magdu);
            pv1s[pos] = (pv1[pos] + fac * dvx) / (T(1) + fac * magdv);
            pv2s[pos] = (pv2[pos] + fac * dvy) / (T(1) + fac * magdv);
        }
}

// solveUVProj.cu:4-22
template <typename T>
void k_uv_proj(const T* u0, const T* v0, const T* du0, const T* dv0, const T* uc0,
               const T* vc0, const T* sku0, const T* skv0, int w, int h, int s,
               T lambdaf, T alphaProj, T* uproj1, T* vproj1) {
#pragma omp parallel for schedule(static)
    for (int iy = 0; iy < h; iy++)
        for (int ix = 0; ix < w; ix++) {
            int pos = ix + iy * s;
            uproj1[pos] = (lambdaf * uc0[pos] + alphaProj * (u0[pos] + du0[pos] + sku0[pos])) /
                          (lambdaf + alphaProj);
            vproj1[pos] = (lambdaf * vc0[pos] + alphaProj * (v0[pos] + dv0[pos] + skv0[pos])) /
                          (lambdaf + alphaProj);
        }
}

// solve3dMinimalArea.cu:3-193.  Per pixel: DLT rows of both cameras plus the
// minimal-surface-area smoothing, solved with the adjugate.  The conditions
// `ix + 1 > width` / `iy + 1 > height` never hold, so the forward
// difference always reads x+1 and y+1: at x = w-1 that is the padding cell
// (stride > w) or the next row's first pixel (stride == w); at y = h-1 it is
// row h, which past the level-0 allocation reads the guard row (0).
template <typename T>
void k_solve3d(const T* uproj0, const T* vproj0, const T* X0, const T* Y0, const T* Z0,
               const T* P, const T* Q, T lambdaf, T lambdams, int width, int height,
               int stride, T* X, T* Y, T* Z) {
    const T P11 = P[0], P12 = P[1], P13 = P[2], P14 = P[3];
    const T P21 = P[4], P22 = P[5], P23 = P[6], P24 = P[7];
    const T P31 = P[8], P32 = P[9], P33 = P[10], P34 = P[11];
    const T Q11 = Q[0], Q12 = Q[1], Q13 = Q[2], Q14 = Q[3];
    const T Q21 = Q[4], Q22 = Q[5], Q23 = Q[6], Q24 = Q[7];
    const T Q31 = Q[8], Q32 = Q[9], Q33 = Q[10], Q34 = Q[11];
#pragma omp parallel for schedule(static)
    for (int iy = 0; iy < height; iy++)
        for (int ix = 0; ix < width; ix++) {
            int pos = ix + iy * stride;
            T x1 = (T)ix;
            T y1 = (T)iy;
            T x2 = (T)ix + uproj0[pos];
            T y2 = (T)iy + vproj0[pos];

            T p1 = x1 * P31 - P11, p2 = x1 * P32 - P12, p3 = x1 * P33 - P13, p4 = x1 * P34 - P14;
            T q1 = y1 * P31 - P21, q2 = y1 * P32 - P22, q3 = y1 * P33 - P23, q4 = y1 * P34 - P24;
            T r1 = x2 * Q31 - Q11, r2 = x2 * Q32 - Q12, r3 = x2 * Q33 - Q13, r4 = x2 * Q34 - Q14;
            T s1 = y2 * Q31 - Q21, s2 = y2 * Q32 - Q22, s3 = y2 * Q33 - Q23, s4 = y2 * Q34 - Q24;

            T ax = lambdaf * (p1 * p1 + q1 * q1 + r1 * r1 + s1 * s1);
            T bx = lambdaf * (p1 * p2 + q1 * q2 + r1 * r2 + s1 * s2);
            T cx = lambdaf * (p1 * p3 + q1 * q3 + r1 * r3 + s1 * s3);
            T dx = lambdaf * (p1 * p4 + q1 * q4 + r1 * r4 + s1 * s4);
            T ay = lambdaf * (p2 * p1 + q2 * q1 + r2 * r1 + s2 * s1);
            T by = lambdaf * (p2 * p2 + q2 * q2 + r2 * r2 + s2 * s2);
            T cy = lambdaf * (p2 * p3 + q2 * q3 + r2 * r3 + s2 * s3);
            T dy = lambdaf * (p2 * p4 + q2 * q4 + r2 * r4 + s2 * s4);
            T az = lambdaf * (p3 * p1 + q3 * q1 + r3 * r1 + s3 * s1);
            T bz = lambdaf * (p3 * p2 + q3 * q2 + r3 * r2 + s3 * s2);
            T cz = lambdaf * (p3 * p3 + q3 * q3 + r3 * r3 + s3 * s3);
            T dz = lambdaf * (p3 * p4 + q3 * q4 + r3 * r4 + s3 * s4);

            // forward differences, always x+1 / y+1 (see above)
            int px = ix + 1 + iy * stride;
            int py = ix + (iy + 1) * stride;
            T Xx = X0[px] - X0[pos], Yx = Y0[px] - Y0[pos], Zx = Z0[px] - Z0[pos];
            T Xy = X0[py] - X0[pos], Yy = Y0[py] - Y0[pos], Zy = Z0[py] - Z0[pos];

            T lambetams = lambdams / std::sqrt((Yx * Zy - Zx * Yy) * (Yx * Zy - Zx * Yy) +
                                               (Zx * Xy - Xx * Zy) * (Zx * Xy - Xx * Zy) +
                                               (Xx * Yy - Yx * Xy) * (Xx * Yy - Yx * Xy) + T(0.001f));

            T Xibar, Yibar, Zibar, Xjbar, Yjbar, Zjbar;
            if (ix - 1 < 0) {
                Xibar = X0[px];
                Yibar = Y0[px];
                Zibar = Z0[px];
            } else {
                Xibar = T(0.5) * X0[pos - 1] + T(0.5) * X0[px];
                Yibar = T(0.5) * Y0[pos - 1] + T(0.5) * Y0[px];
                Zibar = T(0.5) * Z0[pos - 1] + T(0.5) * Z0[px];
            }
            if (iy - 1 < 0) {
                Xjbar = X0[py];
                Yjbar = Y0[py];
                Zjbar = Z0[py];
            } else {
                Xjbar = T(0.5) * X0[pos - stride] + T(0.5) * X0[py];
                Yjbar = T(0.5) * Y0[pos - stride] + T(0.5) * Y0[py];
                Zjbar = T(0.5) * Z0[pos - stride] + T(0.5) * Z0[py];
            }

            T a11 = ax + lambetams * (Yx * Yx + Zx * Zx + Yy * Yy + Zy * Zy);
            T a12 = bx - lambetams * (Xx * Yx + Xy * Yy);
            T a13 = cx - lambetams * (Xx * Zx + Xy * Zy);
            T a21 = ay - lambetams * (Xx * Yx + Xy * Yy);
            T a22 = by + lambetams * (Xx * Xx + Zx * Zx + Xy * Xy + Zy * Zy);
            T a23 = cy - lambetams * (Yx * Zx + Yy * Zy);
            T a31 = az - lambetams * (Xx * Zx + Xy * Zy);
            T a32 = bz - lambetams * (Yx * Zx + Yy * Zy);
            T a33 = cz + lambetams * (Xx * Xx + Yx * Yx + Xy * Xy + Yy * Yy);

            T detA = a11 * (a22 * a33 - a23 * a32) - a12 * (a21 * a33 - a23 * a31) +
                     a13 * (a21 * a32 - a22 * a31);

            T E11 = a22 * a33 - a23 * a32;
            T E12 = a13 * a32 - a12 * a33;
            T E13 = a12 * a23 - a13 * a22;
            T E21 = a23 * a31 - a21 * a33;
            T E22 = a11 * a33 - a13 * a31;
            T E23 = a13 * a21 - a11 * a23;
            T E31 = a21 * a32 - a22 * a31;
            T E32 = a12 * a31 - a11 * a32;
            T E33 = a11 * a22 - a12 * a21;

            T b1 = lambetams * ((Zy * Zy + Yy * Yy) * Xibar + (Zx * Zx + Yx * Yx) * Xjbar -
                                (Xy * Yy) * Yibar - (Xx * Yx) * Yjbar - (Xy * Zy) * Zibar -
                                (Xx * Zx) * Zjbar) -
                   dx;
            T b2 = lambetams * (-(Xy * Yy) * Xibar - (Xx * Yx) * Xjbar + (Xy * Xy + Zy * Zy) * Yibar +
                                (Xx * Xx + Zx * Zx) * Yjbar - (Yy * Zy) * Zibar - (Yx * Zx) * Zjbar) -
                   dy;
            T b3 = lambetams * (-(Xy * Zy) * Xibar - (Xx * Zx) * Xjbar - (Yy * Zy) * Yibar -
                                (Yx * Zx) * Yjbar + (Xy * Xy + Yy * Yy) * Zibar +
                                (Xx * Xx + Yx * Yx) * Zjbar) -
                   dz;

            T Xsub = (E11 * b1 + E12 * b2 + E13 * b3) / detA;
            T Ysub = (E21 * b1 + E22 * b2 + E23 * b3) / detA;
            T Zsub = (E31 * b1 + E32 * b2 + E33 * b3) / detA;

            if (finite3(Xsub, Ysub, Zsub)) {
                X[pos] = Xsub;
                Y[pos] = Ysub;
                Z[pos] = Zsub;
            } else {
                X[pos] = X0[pos];
                Y[pos] = Y0[pos];
                Z[pos] = Z0[pos];
            }
        }
}

// medianFilter.cu:166-243 (MedianFilter3DKernel3): per component 3x3 median
// by 5 passes of exchange selection.  Taps left/above the image clamp to the
// edge; taps right of or below it (col == w, row == h) and the corners stay 0.
template <typename T>
void k_median3d(const T* X, const T* Y, const T* Z, int w, int h, int s,
                T* X1, T* Y1, T* Z1) {
#pragma omp parallel for schedule(static)
    for (int iy = 0; iy < h; iy++)
        for (int ix = 0; ix < w; ix++) {
            T m[3][9];
            const T* src[3] = {X, Y, Z};
            for (int c = 0; c < 3; c++)
                for (int k = 0; k < 9; k++) m[c][k] = 0;
            for (int j = 0; j < 3; j++)
                for (int i = 0; i < 3; i++) {
                    int col = ix + i - 1, row = iy + j - 1, idx = j * 3 + i;
                    int at = -1;
                    if (col >= 0 && col < w && row >= 0 && row < h) at = col + s * row;
                    else if (col < 0 && row >= 0 && row < h) at = s * row;
                    else if (col > w && row >= 0 && row < h) at = w - 1 + s * row;
                    else if (col >= 0 && col < w && row < 0) at = col;
                    else if (col >= 0 && col < w && row > h) at = col + s * (h - 1);
                    if (at >= 0)
                        for (int c = 0; c < 3; c++) m[c][idx] = src[c][at];
                }
            for (int c = 0; c < 3; c++)
                for (int j = 0; j < 5; j++)
                    for (int i = j + 1; i < 9; i++)
                        if (m[c][j] > m[c][i]) std::swap(m[c][j], m[c][i]);
            int pos = ix + iy * s;
            X1[pos] = m[0][4];
            Y1[pos] = m[1][4];
            Z1[pos] = m[2][4];
        }
}

// medianFilter.cu:3-75 (MedianFilterKernel5): 5x5 median of u and v by 13
// passes of exchange selection.  Out-of-range taps clamp along one axis;
// taps out of range on both axes stay 0.
template <typename T>
void k_median5(const T* u, const T* v, int w, int h, int s, T* ou, T* ov) {
#pragma omp parallel for schedule(static)
    for (int iy = 0; iy < h; iy++)
        for (int ix = 0; ix < w; ix++) {
            T mu[25], mv[25];
            for (int k = 0; k < 25; k++) mu[k] = mv[k] = 0;
            for (int j = 0; j < 5; j++)
                for (int i = 0; i < 5; i++) {
                    int col = ix + i - 2, row = iy + j - 2;
                    int at = -1;
                    if (col >= 0 && col < w && row >= 0 && row < h) at = col + s * row;
                    else if (col < 0 && row >= 0 && row < h) at = s * row;
                    else if (col >= w && row >= 0 && row < h) at = w - 1 + s * row;
                    else if (col >= 0 && col < w && row < 0) at = col;
                    else if (col >= 0 && col < w && row >= h) at = col + s * (h - 1);
                    if (at >= 0) {
                        mu[j * 5 + i] = u[at];
                        mv[j * 5 + i] = v[at];
                    }
                }
            for (int j = 0; j < 13; j++)
                for (int i = j + 1; i < 25; i++) {
                    if (mu[j] > mu[i]) std::swap(mu[j], mu[i]);
                    if (mv[j] > mv[i]) std::swap(mv[j], mv[i]);
                }
            ou[ix + iy * s] = mu[12];
            ov[ix + iy * s] = mv[12];
        }
}

// solve3dMinimalArea.cu:248-297 (CleanUp3DKernel)
template <typename T>
void k_cleanup3d(const T* X0, const T* Y0, const T* Z0, const T* Xm, const T* Ym,
                 const T* Zm, int w, int h, int s, T* X1, T* Y1, T* Z1) {
#pragma omp parallel for schedule(static)
    for (int iy = 0; iy < h; iy++)
        for (int ix = 0; ix < w; ix++) {
            int pos = ix + iy * s;
            T Xmed = Xm[pos], Ymed = Ym[pos], Zmed = Zm[pos];
            T X = X0[pos], Y = Y0[pos], Z = Z0[pos];
            if (finite3(X, Y, Z) && finite3(Xmed, Ymed, Zmed)) {
                X1[pos] = std::fabs(Xmed - X) > T(5) ? Xmed : X;
                Y1[pos] = std::fabs(Ymed - Y) > T(5) ? Ymed : Y;
                Z1[pos] = std::fabs(Zmed - Z) > T(5) ? Zmed : Z;
            } else {
                X1[pos] = 0;
                Y1[pos] = 0;
                Z1[pos] = 0;
            }
        }
}

// solveUcSk.cu:3-35 (SolveUcKernel): project into camera 1 with R1, t1 and
// (fx, cx, cy) of K1 at this level.
template <typename T>
void k_solve_uc(const T* X0, const T* Y0, const T* Z0, const T* R, const T* t,
                T focal, T cx, T cy, int w, int h, int s, T* uc, T* vc) {
#pragma omp parallel for schedule(static)
    for (int iy = 0; iy < h; iy++)
        for (int ix = 0; ix < w; ix++) {
            int pos = ix + iy * s;
            T X = X0[pos], Y = Y0[pos], Z = Z0[pos];
            T X2 = R[0] * X + R[1] * Y + R[2] * Z + t[0];
            T Y2 = R[3] * X + R[4] * Y + R[5] * Z + t[1];
            T Z2 = R[6] * X + R[7] * Y + R[8] * Z + t[2];
            T xproj = focal * X2 / Z2 + cx;
            T yproj = focal * Y2 / Z2 + cy;
            uc[pos] = xproj - (T)ix;
            vc[pos] = yproj - (T)iy;
        }
}

// solveUcSk.cu:80-97 (UpdateSkKernel)
template <typename T>
void k_update_sk(const T* sku0, const T* skv0, const T* u0, const T* v0, const T* du0,
                 const T* dv0, const T* uproj0, const T* vproj0, int w, int h, int s,
                 T* sku1, T* skv1) {
#pragma omp parallel for schedule(static)
    for (int iy = 0; iy < h; iy++)
        for (int ix = 0; ix < w; ix++) {
            int pos = ix + iy * s;
            sku1[pos] = sku0[pos] + u0[pos] + du0[pos] - uproj0[pos];
            skv1[pos] = skv0[pos] + v0[pos] + dv0[pos] - vproj0[pos];
        }
}

// addKernel.cu:3-11, run over h*stride elements (padding included)
template <typename T>
void k_add(const T* a, const T* b, int count, T* out) {
    for (int i = 0; i < count; i++) out[i] = a[i] + b[i];
}

// solve3dMinimalArea.cu:320-378 (RemoveEdgeArtifacts3DKernel)
template <typename T>
void k_remove_edge_artifacts(const T* X0, const T* Y0, const T* Z0, int range, T maxArea,
                             int width, int height, int stride, T* X1, T* Y1, T* Z1) {
    for (int iy = 0; iy < height; iy++)
        for (int ix = 0; ix < width; ix++) {
            int pos = ix + iy * stride;
            int ax = (ix + range > width) ? ix - range + iy * stride : ix + range + iy * stride;
            int ay = (iy + range > height) ? ix + (iy - range) * stride : ix + (iy + range) * stride;
            T Xx, Yx, Zx, Xy, Yy, Zy;
            if (ix + range > width) {
                Xx = -X0[ax] + X0[pos]; Yx = -Y0[ax] + Y0[pos]; Zx = -Z0[ax] + Z0[pos];
            } else {
                Xx = X0[ax] - X0[pos]; Yx = Y0[ax] - Y0[pos]; Zx = Z0[ax] - Z0[pos];
            }
            if (iy + range > height) {
                Xy = -X0[ay] + X0[pos]; Yy = -Y0[ay] + Y0[pos]; Zy = -Z0[ay] + Z0[pos];
            } else {
                Xy = X0[ay] - X0[pos]; Yy = Y0[ay] - Y0[pos]; Zy = Z0[ay] - Z0[pos];
            }
            T area = std::sqrt((Yx * Zy - Zx * Yy) * (Yx * Zy - Zx * Yy) +
                               (Zx * Xy - Xx * Zy) * (Zx * Xy - Xx * Zy) +
                               (Xx * Yy - Yx * Xy) * (Xx * Yy - Yx * Xy));
            if (area > maxArea) {
                X1[pos] = 0; Y1[pos] = 0; Z1[pos] = 0;
            } else {
                X1[pos] = X0[pos]; Y1[pos] = Y0[pos]; Z1[pos] = Z0[pos];
            }
        }
}

}  // namespace

// ---------------------------------------------------------------------------
// Full schedules
// ---------------------------------------------------------------------------

extern "C" {

// Mirrors the C-ABI parameter block of the library (include/reconflow_gb300.h).
typedef struct rfo_params {
    int width, height;
    int input_type;  // 0 = f32 gray, 1 = rgb8, 2 = u8 gray, 3 = u16 gray
    int n_levels;
    float scale;
    int method;  // 0 = plain TV-L1, 14 = ReconFlow, 17 = + dense prior, 20 = + sparse prior
    float lambda, lambdaf, lambdams, alpha_tv, alpha_proj, alpha_fn, tau, theta;
    int n_warp_iters, n_solver_iters;
    int stride_alignment;
    int fix_quirks;  // 0 = reference behaviour; bit 0: K[2][2] = 1 at every level,
                     // bit 1: resample X, Y, Z to the finer level instead of re-reading
} rfo_params;

}  // extern "C"

namespace {

template <typename T>
struct Pool {
    std::vector<std::vector<T>> bufs;
    size_t n;
    explicit Pool(size_t n_) : n(n_) {}
    T* make() {
        bufs.emplace_back(n, T(0));
        return bufs.back().data();
    }
};

template <typename T>
void load_input(const rfo_params& p, const void* img, int s, T* out) {
    int w = p.width, h = p.height;
    switch (p.input_type) {
        case 1: k_rgb_to_gray(static_cast<const uint8_t*>(img), w, h, s, out); break;
        case 2: k_u8_to_gray(static_cast<const uint8_t*>(img), w, h, s, out); break;
        case 3: k_u16_to_gray(static_cast<const uint16_t*>(img), w, h, s, out); break;
        default: k_f32_to_gray(static_cast<const float*>(img), w, h, s, out); break;
    }
}

// Reconflow.cu:78-116: K pyramid; levels >= 1 start from zeros, so K[2][2]
// is 0 there (only fx, cx, fy, cy are carried down).
void k_pyramid(const double* K, int L, float fScale, std::vector<std::vector<double>>& pK,
               bool fix_k22 = false) {
    pK.assign(L, std::vector<double>(9, 0.0));
    for (int i = 0; i < 9; i++) pK[0][i] = K[i];
    for (int l = 1; l < L; l++) {
        if (fix_k22) pK[l][8] = 1.0;
        pK[l][0] = pK[l - 1][0] / fScale;
        pK[l][2] = pK[l - 1][2] / fScale;
        pK[l][4] = pK[l - 1][4] / fScale;
        pK[l][5] = pK[l - 1][5] / fScale;
    }
}

// Reconflow.cu:150-152,225-226: P = K * [R | t] in double.
void camera_matrix(const std::vector<double>& K, const double* R, const double* t, double* P) {
    double Rt[12];
    for (int r = 0; r < 3; r++) {
        for (int c = 0; c < 3; c++) Rt[r * 4 + c] = R[r * 3 + c];
        Rt[r * 4 + 3] = t[r];
    }
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 4; c++) {
            double acc = 0;
            for (int k = 0; k < 3; k++) acc += K[r * 3 + k] * Rt[k * 4 + c];
            P[r * 4 + c] = acc;
        }
}

// Reconflow.cu:147-466 (solveReconFlow, METHODR_TVL1_MS and the prior
// variants) and Cudaflow.cu:403-621 (_solveOpticalFlow, METHOD_TVL1).  All
// work buffers are flat level-0-sized arrays (plus one zero guard row) and
// are exchanged by pointer swaps exactly as the reference does, because the
// 3D buffers are re-read with the next level's stride without upscaling.
// Warm start (no reference counterpart): begin the schedule at `level`
// with flow u, v and 3D points X, Y, Z given on that level (planes with the
// level's stride); uproj = u, sk = 0, uc recomputed from the points; levels
// `level`..0 run `warps` warps of `iters` iterations each.
struct WarmStart {
    int level = -1;
    const float *u = nullptr, *v = nullptr, *X = nullptr, *Y = nullptr, *Z = nullptr;
    int warps = 0, iters = 0;
};

template <typename T>
int solve(const rfo_params& p, const void* i0, const void* i1, int in_stride,
          const double* K0, const double* K1, const double* R0, const double* t0,
          const double* R1, const double* t1, const float* ufn, const float* vfn,
          const float* fnmask, T* out_u, T* out_v, T* out_X, T* out_Y, T* out_Z,
          const WarmStart* warm = nullptr) {
    const int L = p.n_levels;
    std::vector<int> W(L), H(L), S(L);
    pyramid_dims(p.width, p.height, L, p.scale, p.stride_alignment, W.data(), H.data(), S.data());
    const int stride = S[0], height = H[0];
    const size_t n = (size_t)stride * (height + 1);  // + guard row
    const bool recon = p.method != 0;
    const int prior = p.method == 17 ? 1 : (p.method == 20 ? 2 : 0);

    Pool<T> pool(n);
    std::vector<T*> pI0(L), pI1(L);
    for (int l = 0; l < L; l++) {
        pI0[l] = pool.make();
        pI1[l] = pool.make();
    }
    T *d_i1warp = pool.make(), *d_Ix = pool.make(), *d_Iy = pool.make(), *d_Iz = pool.make();
    T *d_dumed = pool.make(), *d_dvmed = pool.make(), *d_dumeds = pool.make(), *d_dvmeds = pool.make();
    T *d_pu1 = pool.make(), *d_pu2 = pool.make(), *d_pv1 = pool.make(), *d_pv2 = pool.make();
    T *d_pu1s = pool.make(), *d_pu2s = pool.make(), *d_pv1s = pool.make(), *d_pv2s = pool.make();
    T *d_u = pool.make(), *d_v = pool.make(), *d_us = pool.make(), *d_vs = pool.make();
    T *d_uproj = pool.make(), *d_vproj = pool.make(), *d_uc = pool.make(), *d_vc = pool.make();
    T *d_sku = pool.make(), *d_skv = pool.make(), *d_skus = pool.make(), *d_skvs = pool.make();
    T *d_X = pool.make(), *d_Y = pool.make(), *d_Z = pool.make();
    T *d_Xs = pool.make(), *d_Ys = pool.make(), *d_Zs = pool.make();
    T *d_Xmed = pool.make(), *d_Ymed = pool.make(), *d_Zmed = pool.make();
    T *d_ufn = nullptr, *d_vfn = nullptr, *d_mask = nullptr;
    T *d_ufn_l = nullptr, *d_vfn_l = nullptr, *d_mask_l = nullptr;
    if (prior) {
        d_ufn = pool.make(); d_vfn = pool.make(); d_mask = pool.make();
        d_ufn_l = pool.make(); d_vfn_l = pool.make(); d_mask_l = pool.make();
        for (int y = 0; y < height; y++)
            for (int x = 0; x < stride; x++) {
                size_t i = x + (size_t)y * stride;
                d_ufn[i] = (T)ufn[i];
                d_vfn[i] = (T)vfn[i];
                d_mask[i] = fnmask ? (T)fnmask[i] : T(1);
            }
    }
    auto zero = [&](T* b) { std::fill(b, b + (size_t)stride * height, T(0)); };

    const T lambda = (T)p.lambda, lambdaf = (T)p.lambdaf, lambdams = (T)p.lambdams;
    const T alphaTv = (T)p.alpha_tv, alphaProj = (T)p.alpha_proj, alphaFn = (T)p.alpha_fn;
    const T tau = (T)p.tau;
    const bool is64 = std::is_same<T, double>::value;
    // Reconflow.cu:32: thetaTv = 1/alphaTv, formed in float by the reference
    // (kept exact by the FP64 oracle); plain TV-L1 uses theta directly.
    const T theta = recon ? (is64 ? T(1) / (T)p.alpha_tv : (T)(1.0f / p.alpha_tv)) : (T)p.theta;

    std::vector<std::vector<double>> pK0, pK1;
    if (recon) {
        k_pyramid(K0, L, p.scale, pK0, (p.fix_quirks & 1) != 0);
        k_pyramid(K1, L, p.scale, pK1, (p.fix_quirks & 1) != 0);
    }

    load_input<T>(p, i0, in_stride, pI0[0]);
    load_input<T>(p, i1, in_stride, pI1[0]);
    for (int l = 1; l < L; l++) {
        k_downscale(pI0[l - 1], W[l - 1], H[l - 1], S[l - 1], W[l], H[l], S[l], T(1), false, pI0[l]);
        k_downscale(pI1[l - 1], W[l - 1], H[l - 1], S[l - 1], W[l], H[l], S[l], T(1), false, pI1[l]);
    }
    zero(d_u); zero(d_v);
    if (recon) {
        zero(d_uproj); zero(d_vproj); zero(d_uc); zero(d_vc);
        zero(d_X); zero(d_Y); zero(d_Z); zero(d_sku); zero(d_skv);
    }
    // SolveUc takes float copies of R1, t1 (solveUcSk.cu:42-53); FP64 keeps doubles.
    T R1f[9], t1f[3];
    for (int i = 0; i < 9; i++) R1f[i] = is64 ? (T)R1[i] : (T)(float)R1[i];
    for (int i = 0; i < 3; i++) t1f[i] = is64 ? (T)t1[i] : (T)(float)t1[i];

    const bool is_warm = warm && warm->level >= 0;
    const int top = is_warm ? warm->level : L - 1;
    const int n_warps = is_warm ? warm->warps : p.n_warp_iters;
    const int n_iters = is_warm ? warm->iters : p.n_solver_iters;
    bool uc_from_points = false;
    if (is_warm) {
        const int w = W[top], h = H[top], s = S[top];
        for (int y = 0; y < h; y++)
            for (int x = 0; x < w; x++) {
                size_t i = x + (size_t)y * s;
                d_u[i] = (T)warm->u[i];
                d_v[i] = (T)warm->v[i];
                if (recon) {
                    d_uproj[i] = (T)warm->u[i];
                    d_vproj[i] = (T)warm->v[i];
                    d_X[i] = (T)warm->X[i];
                    d_Y[i] = (T)warm->Y[i];
                    d_Z[i] = (T)warm->Z[i];
                }
            }
        uc_from_points = recon;
    }

    for (int level = top; level >= 0; level--) {
        const int w = W[level], h = H[level], s = S[level];
        T P[12], Q[12];
        T focal = 0, cxl = 0, cyl = 0;
        if (recon) {
            double Pd[12], Qd[12];
            camera_matrix(pK0[level], R0, t0, Pd);
            camera_matrix(pK1[level], R1, t1, Qd);
            // Solve3dMinimalArea / SolveUc take float copies (solve3dMinimalArea.cu:204-228,
            // solveUcSk.cu:42-56); the FP64 oracle keeps the doubles.
            for (int i = 0; i < 12; i++) {
                P[i] = is64 ? (T)Pd[i] : (T)(float)Pd[i];
                Q[i] = is64 ? (T)Qd[i] : (T)(float)Qd[i];
            }
            const std::vector<double>& k1 = pK1[level];
            focal = is64 ? (T)k1[0] : (T)(float)k1[0];
            cxl = is64 ? (T)k1[2] : (T)(float)k1[2];
            cyl = is64 ? (T)k1[5] : (T)(float)k1[5];
        }
        if (prior) {
            // Reconflow.cu:232-241: the prior is resampled from level 0 each level.
            T sc = (T)((float)W[level] / (float)W[0]);
            k_downscale(d_ufn, W[0], H[0], S[0], w, h, s, sc, true, d_ufn_l);
            k_downscale(d_vfn, W[0], H[0], S[0], w, h, s, sc, true, d_vfn_l);
            k_downscale(d_mask, W[0], H[0], S[0], w, h, s, T(1), false, d_mask_l);
        }
        if (uc_from_points) {
            // warm start: uc of the supplied points at this level
            k_solve_uc(d_X, d_Y, d_Z, R1f, t1f, focal, cxl, cyl, w, h, s, d_uc, d_vc);
            uc_from_points = false;
        }
        for (int warp = 0; warp < n_warps; warp++) {
            zero(d_dumed); zero(d_dvmed); zero(d_dumeds); zero(d_dvmeds);
            zero(d_pu1); zero(d_pu2); zero(d_pv1); zero(d_pv2);
            k_warp(pI1[level], w, h, s, d_u, d_v, d_i1warp);
            k_derivatives(pI0[level], d_i1warp, w, h, s, d_Ix, d_Iy, d_Iz);
            for (int iter = 0; iter < n_iters; iter++) {
                if (recon) {
                    k_recon_data_l1(d_u, d_v, d_dumed, d_dvmed, d_uproj, d_vproj, d_ufn_l, d_vfn_l,
                                    d_mask_l, d_sku, d_skv, d_pu1, d_pu2, d_pv1, d_pv2, d_Ix, d_Iy,
                                    d_Iz, w, h, s, lambda, alphaTv, alphaProj, alphaFn, prior,
                                    d_dumeds, d_dvmeds);
                } else {
                    k_data_l1(d_dumed, d_dvmed, d_pu1, d_pu2, d_pv1, d_pv2, d_Ix, d_Iy, d_Iz, w, h,
                              s, lambda, theta, d_dumeds, d_dvmeds);
                }
                std::swap(d_dumed, d_dumeds);
                std::swap(d_dvmed, d_dvmeds);
                k_dual_tv(d_dumed, d_dvmed, d_pu1, d_pu2, d_pv1, d_pv2, w, h, s, tau,
                          theta, d_pu1s, d_pu2s, d_pv1s, d_pv2s);
                std::swap(d_pu1, d_pu1s); std::swap(d_pu2, d_pu2s);
                std::swap(d_pv1, d_pv1s); std::swap(d_pv2, d_pv2s);
                if (!recon) continue;
                k_uv_proj(d_u, d_v, d_dumed, d_dvmed, d_uc, d_vc, d_sku, d_skv, w, h, s, lambdaf,
                          alphaProj, d_uproj, d_vproj);
                k_solve3d(d_uproj, d_vproj, d_X, d_Y, d_Z, P, Q, lambdaf, lambdams, w, h, s,
                          d_Xs, d_Ys, d_Zs);
                std::swap(d_X, d_Xs); std::swap(d_Y, d_Ys); std::swap(d_Z, d_Zs);
                k_median3d(d_X, d_Y, d_Z, w, h, s, d_Xmed, d_Ymed, d_Zmed);
                k_cleanup3d(d_X, d_Y, d_Z, d_Xmed, d_Ymed, d_Zmed, w, h, s, d_Xs, d_Ys, d_Zs);
                std::swap(d_X, d_Xs); std::swap(d_Y, d_Ys); std::swap(d_Z, d_Zs);
                k_solve_uc(d_X, d_Y, d_Z, R1f, t1f, focal, cxl, cyl, w, h, s, d_uc, d_vc);
                k_update_sk(d_sku, d_skv, d_u, d_v, d_dumed, d_dvmed, d_uproj, d_vproj, w, h, s,
                            d_skus, d_skvs);
                std::swap(d_sku, d_skus); std::swap(d_skv, d_skvs);
            }
            k_median5(d_dumed, d_dvmed, w, h, s, d_dumeds, d_dvmeds);
            std::swap(d_dumed, d_dumeds); std::swap(d_dvmed, d_dvmeds);
            k_add(d_u, d_dumed, h * s, d_u);
            k_add(d_v, d_dvmed, h * s, d_v);
            if (recon) {
                k_median5(d_u, d_v, w, h, s, d_dumeds, d_dvmeds);
                std::swap(d_u, d_dumeds); std::swap(d_v, d_dvmeds);
            }
        }
        if (level > 0) {
            const int fw = W[level - 1], fh = H[level - 1], fs = S[level - 1];
            const T sc = (T)p.scale;
            k_upscale(d_u, w, h, s, fw, fh, fs, sc, d_us); std::swap(d_u, d_us);
            k_upscale(d_v, w, h, s, fw, fh, fs, sc, d_vs); std::swap(d_v, d_vs);
            if (recon) {
                k_upscale(d_uc, w, h, s, fw, fh, fs, sc, d_us); std::swap(d_uc, d_us);
                k_upscale(d_vc, w, h, s, fw, fh, fs, sc, d_vs); std::swap(d_vc, d_vs);
                k_upscale(d_uproj, w, h, s, fw, fh, fs, sc, d_us); std::swap(d_uproj, d_us);
                k_upscale(d_vproj, w, h, s, fw, fh, fs, sc, d_vs); std::swap(d_vproj, d_vs);
                k_upscale(d_sku, w, h, s, fw, fh, fs, sc, d_us); std::swap(d_sku, d_us);
                k_upscale(d_skv, w, h, s, fw, fh, fs, sc, d_vs); std::swap(d_skv, d_vs);
                if (p.fix_quirks & 2) {
                    k_upscale(d_X, w, h, s, fw, fh, fs, T(1), d_Xs);
                    k_upscale(d_Y, w, h, s, fw, fh, fs, T(1), d_Ys);
                    k_upscale(d_Z, w, h, s, fw, fh, fs, T(1), d_Zs);
                    // only the fine level's pixels are replaced
                    for (int y = 0; y < fh; y++) {
                        size_t o = (size_t)y * fs;
                        std::copy(d_Xs + o, d_Xs + o + fw, d_X + o);
                        std::copy(d_Ys + o, d_Ys + o + fw, d_Y + o);
                        std::copy(d_Zs + o, d_Zs + o + fw, d_Z + o);
                    }
                }
            }
        }
    }
    const size_t m = (size_t)stride * height;
    std::copy(d_u, d_u + m, out_u);
    std::copy(d_v, d_v + m, out_v);
    if (recon && out_X) {
        std::copy(d_X, d_X + m, out_X);
        std::copy(d_Y, d_Y + m, out_Y);
        std::copy(d_Z, d_Z + m, out_Z);
    }
    return 0;
}

// Energy of a solution (no reference counterpart; defines the fallback test
// of the warm-started solve), summed in double over the level-0 pixels:
//   lambda * |I1(x + u) - I0(x)|                      (brightness residual,
//                                                      I1 fetched as WarpingKernel)
// + |grad u| + |grad v|                               (forward differences,
//                                                      0 at the far border)
// + alpha_proj / 2 * min(|(u, v) - uc(X)|^2, 1)       (reprojection of the
//                                                      solved 3D point, truncated
//                                                      at 1 px^2; recon only)
// A pixel whose sum is not finite (non-finite flow) counts every term at its
// cap: lambda + 2 + alpha_proj / 2.
double energy(const float* I0, const float* I1, const float* u, const float* v, const float* X,
              const float* Y, const float* Z, int w, int h, int s, float lambda,
              float alpha_proj, const double* R1, const double* t1, const double* K1,
              int recon) {
    double e = 0.0;
    for (int iy = 0; iy < h; iy++)
        for (int ix = 0; ix < w; ix++) {
            int pos = ix + iy * s;
            float x = ((float)ix + u[pos] + 0.5f) / (float)w;
            float y = ((float)iy + v[pos] + 0.5f) / (float)h;
            float i1w = tex2d(I1, w, h, s, x, y);
            double data = (double)lambda * std::fabs((double)i1w - (double)I0[pos]);
            double ux = ix + 1 < w ? (double)u[pos + 1] - u[pos] : 0.0;
            double uy = iy + 1 < h ? (double)u[pos + s] - u[pos] : 0.0;
            double vx = ix + 1 < w ? (double)v[pos + 1] - v[pos] : 0.0;
            double vy = iy + 1 < h ? (double)v[pos + s] - v[pos] : 0.0;
            double tv = std::sqrt(ux * ux + uy * uy) + std::sqrt(vx * vx + vy * vy);
            double proj = 0.0;
            if (recon) {
                double Xp = X[pos], Yp = Y[pos], Zp = Z[pos];
                double X2 = R1[0] * Xp + R1[1] * Yp + R1[2] * Zp + t1[0];
                double Y2 = R1[3] * Xp + R1[4] * Yp + R1[5] * Zp + t1[1];
                double Z2 = R1[6] * Xp + R1[7] * Yp + R1[8] * Zp + t1[2];
                double uc = K1[0] * X2 / Z2 + K1[2] - ix;
                double vc = K1[0] * Y2 / Z2 + K1[5] - iy;  // fx for both, as SolveUc
                double du = u[pos] - uc, dv = v[pos] - vc;
                double r2 = du * du + dv * dv;
                if (!(r2 < 1.0)) r2 = 1.0;  // truncated at 1 px^2 (NaN included)
                proj = 0.5 * (double)alpha_proj * r2;
            }
            double px_e = data + tv + proj;
            // a non-finite pixel term counts each term at its cap
            if (!std::isfinite(px_e))
                px_e = (double)lambda + 2.0 + (recon ? 0.5 * (double)alpha_proj : 0.0);
            e += px_e;
        }
    return e;
}

}  // namespace

// ---------------------------------------------------------------------------
// C entry points (loaded with ctypes by the tests and the CPU baseline)
// ---------------------------------------------------------------------------
extern "C" {

int rfo_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void rfo_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

void rfo_pyramid_dims(int w, int h, int levels, float scale, int align, int* W, int* H, int* S) {
    pyramid_dims(w, h, levels, scale, align, W, H, S);
}

void rfo_k_pyramid(const double* K, int levels, float scale, double* out) {
    std::vector<std::vector<double>> pK;
    k_pyramid(K, levels, scale, pK);
    for (int l = 0; l < levels; l++)
        for (int i = 0; i < 9; i++) out[l * 9 + i] = pK[l][i];
}

void rfo_camera_matrix(const double* K, const double* R, const double* t, double* P) {
    std::vector<double> k(K, K + 9);
    camera_matrix(k, R, t, P);
}

#define RFO_KERNELS(T, SFX)                                                                        \
    void rfo_downscale_##SFX(const T* src, int w, int h, int s, int nw, int nh, int ns, T scale,  \
                             int scaled, T* out) {                                                 \
        k_downscale<T>(src, w, h, s, nw, nh, ns, scale, scaled != 0, out);                         \
    }                                                                                              \
    void rfo_upscale_##SFX(const T* src, int w, int h, int s, int nw, int nh, int ns, T scale,    \
                           T* out) {                                                               \
        k_upscale<T>(src, w, h, s, nw, nh, ns, scale, out);                                        \
    }                                                                                              \
    void rfo_warp_##SFX(const T* src, int w, int h, int s, const T* u, const T* v, T* out) {      \
        k_warp<T>(src, w, h, s, u, v, out);                                                        \
    }                                                                                              \
    void rfo_derivatives_##SFX(const T* I0, const T* I1, int w, int h, int s, T* Ix, T* Iy,       \
                               T* Iz) {                                                            \
        k_derivatives<T>(I0, I1, w, h, s, Ix, Iy, Iz);                                             \
    }                                                                                              \
    void rfo_median5_##SFX(const T* u, const T* v, int w, int h, int s, T* ou, T* ov) {           \
        k_median5<T>(u, v, w, h, s, ou, ov);                                                       \
    }                                                                                              \
    void rfo_median3d_##SFX(const T* X, const T* Y, const T* Z, int w, int h, int s, T* X1,       \
                            T* Y1, T* Z1) {                                                        \
        k_median3d<T>(X, Y, Z, w, h, s, X1, Y1, Z1);                                               \
    }                                                                                              \
    void rfo_recon_data_l1_##SFX(const T* u, const T* v, const T* duhat, const T* dvhat,          \
                                 const T* uproj, const T* vproj, const T* ufn, const T* vfn,      \
                                 const T* mask, const T* sku, const T* skv, const T* pu1,         \
                                 const T* pu2, const T* pv1, const T* pv2, const T* Ix,           \
                                 const T* Iy, const T* Iz, int w, int h, int s, T lambda,         \
                                 T alphaTv, T alphaProj, T alphaFn, int prior, T* duhat1,         \
                                 T* dvhat1) {                                                      \
        k_recon_data_l1<T>(u, v, duhat, dvhat, uproj, vproj, ufn, vfn, mask, sku, skv, pu1, pu2,  \
                           pv1, pv2, Ix, Iy, Iz, w, h, s, lambda, alphaTv, alphaProj, alphaFn,    \
                           prior, duhat1, dvhat1);                                                 \
    }                                                                                              \
    void rfo_data_l1_##SFX(const T* duhat, const T* dvhat, const T* pu1, const T* pu2,            \
                           const T* pv1, const T* pv2, const T* Ix, const T* Iy, const T* Iz,     \
                           int w, int h, int s, T lambda, T theta, T* duhat1, T* dvhat1) {        \
        k_data_l1<T>(duhat, dvhat, pu1, pu2, pv1, pv2, Ix, Iy, Iz, w, h, s, lambda, theta,        \
                     duhat1, dvhat1);                                                              \
    }                                                                                              \
    void rfo_dual_tv_##SFX(const T* duhat, const T* dvhat, const T* pu1, const T* pu2,            \
                           const T* pv1, const T* pv2, int w, int h, int s, T tau, T theta,       \
                           T* pu1s, T* pu2s, T* pv1s, T* pv2s) {                                  \
        k_dual_tv<T>(duhat, dvhat, pu1, pu2, pv1, pv2, w, h, s, tau, theta, pu1s, pu2s, pv1s,     \
                     pv2s);                                                                        \
    }                                                                                              \
    void rfo_uv_proj_##SFX(const T* u, const T* v, const T* du, const T* dv, const T* uc,         \
                           const T* vc, const T* sku, const T* skv, int w, int h, int s,          \
                           T lambdaf, T alphaProj, T* uproj, T* vproj) {                          \
        k_uv_proj<T>(u, v, du, dv, uc, vc, sku, skv, w, h, s, lambdaf, alphaProj, uproj, vproj);  \
    }                                                                                              \
    void rfo_solve3d_##SFX(const T* uproj, const T* vproj, const T* X0, const T* Y0,              \
                           const T* Z0, const T* P, const T* Q, T lambdaf, T lambdams, int w,     \
                           int h, int s, T* X, T* Y, T* Z) {                                      \
        k_solve3d<T>(uproj, vproj, X0, Y0, Z0, P, Q, lambdaf, lambdams, w, h, s, X, Y, Z);        \
    }                                                                                              \
    void rfo_cleanup3d_##SFX(const T* X0, const T* Y0, const T* Z0, const T* Xm, const T* Ym,     \
                             const T* Zm, int w, int h, int s, T* X1, T* Y1, T* Z1) {             \
        k_cleanup3d<T>(X0, Y0, Z0, Xm, Ym, Zm, w, h, s, X1, Y1, Z1);                               \
    }                                                                                              \
    void rfo_solve_uc_##SFX(const T* X, const T* Y, const T* Z, const T* R, const T* t, T f,      \
                            T cx, T cy, int w, int h, int s, T* uc, T* vc) {                      \
        k_solve_uc<T>(X, Y, Z, R, t, f, cx, cy, w, h, s, uc, vc);                                  \
    }                                                                                              \
    void rfo_update_sk_##SFX(const T* sku, const T* skv, const T* u, const T* v, const T* du,     \
                             const T* dv, const T* uproj, const T* vproj, int w, int h, int s,    \
                             T* sku1, T* skv1) {                                                   \
        k_update_sk<T>(sku, skv, u, v, du, dv, uproj, vproj, w, h, s, sku1, skv1);                 \
    }                                                                                              \
    void rfo_remove_edge_artifacts_##SFX(const T* X0, const T* Y0, const T* Z0, int range,        \
                                         T maxArea, int w, int h, int s, T* X1, T* Y1, T* Z1) {    \
        k_remove_edge_artifacts<T>(X0, Y0, Z0, range, maxArea, w, h, s, X1, Y1, Z1);               \
    }                                                                                              \
    int rfo_solve_##SFX(const rfo_params* p, const void* i0, const void* i1, int in_stride,       \
                        const double* K0, const double* K1, const double* R0, const double* t0,   \
                        const double* R1, const double* t1, const float* ufn, const float* vfn,   \
                        const float* mask, T* u, T* v, T* X, T* Y, T* Z) {                        \
        return solve<T>(*p, i0, i1, in_stride, K0, K1, R0, t0, R1, t1, ufn, vfn, mask, u, v, X,   \
                        Y, Z);                                                                     \
    }

RFO_KERNELS(float, f32)
RFO_KERNELS(double, f64)

int rfo_solve_warm_f32(const rfo_params* p, const float* i0, const float* i1, int in_stride,
                       const double* K0, const double* K1, const double* R0, const double* t0,
                       const double* R1, const double* t1, int level, const float* wu,
                       const float* wv, const float* wX, const float* wY, const float* wZ,
                       int warps, int iters, float* u, float* v, float* X, float* Y, float* Z) {
    WarmStart ws;
    ws.level = level; ws.u = wu; ws.v = wv; ws.X = wX; ws.Y = wY; ws.Z = wZ;
    ws.warps = warps; ws.iters = iters;
    return solve<float>(*p, i0, i1, in_stride, K0, K1, R0, t0, R1, t1, nullptr, nullptr, nullptr,
                        u, v, X, Y, Z, &ws);
}

// The same warm-started schedule in FP64 (the warm state is given in float,
// as the FP32 path receives it).
int rfo_solve_warm_f64(const rfo_params* p, const float* i0, const float* i1, int in_stride,
                       const double* K0, const double* K1, const double* R0, const double* t0,
                       const double* R1, const double* t1, int level, const float* wu,
                       const float* wv, const float* wX, const float* wY, const float* wZ,
                       int warps, int iters, double* u, double* v, double* X, double* Y,
                       double* Z) {
    WarmStart ws;
    ws.level = level; ws.u = wu; ws.v = wv; ws.X = wX; ws.Y = wY; ws.Z = wZ;
    ws.warps = warps; ws.iters = iters;
    return solve<double>(*p, i0, i1, in_stride, K0, K1, R0, t0, R1, t1, nullptr, nullptr,
                         nullptr, u, v, X, Y, Z, &ws);
}

double rfo_energy(const float* I0, const float* I1, const float* u, const float* v,
                  const float* X, const float* Y, const float* Z, int w, int h, int s,
                  float lambda, float alpha_proj, const double* R1, const double* t1,
                  const double* K1, int recon) {
    return energy(I0, I1, u, v, X, Y, Z, w, h, s, lambda, alpha_proj, R1, t1, K1, recon);
}

void rfo_rgb_to_gray_f32(const uint8_t* rgb, int w, int h, int s, float* out) {
    k_rgb_to_gray<float>(rgb, w, h, s, out);
}

}  // extern "C"
