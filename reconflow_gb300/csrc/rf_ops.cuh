// Per-pixel operations of the Reconflow kernels, shared by the single-pair
// kernels (rf_kernels.cu) and the batched kernels (rf_batch.cu).  Every
// function computes one pixel exactly as the reference kernel it cites.
#pragma once

#include "rf_kernels.cuh"

namespace rf {
namespace {

// downscale.cu:6-26: sum of the four fetches at +-1/4 coarse texel.
__device__ __forceinline__ float downscale_px(const float* __restrict__ src, LevelDims f, int nw,
                                              int nh, int ix, int iy) {
    float dx = 1.0f / (float)nw;
    float dy = 1.0f / (float)nh;
    float x = ((float)ix + 0.5f) * dx;
    float y = ((float)iy + 0.5f) * dy;
    return tex2d(src, f.w, f.h, f.s, x - dx * 0.25f, y) + tex2d(src, f.w, f.h, f.s, x + dx * 0.25f, y) +
           tex2d(src, f.w, f.h, f.s, x, y - dy * 0.25f) + tex2d(src, f.w, f.h, f.s, x, y + dy * 0.25f);
}


// computeDerivatives.cu:26-36: [1, -8, 0, 8, -1] / 12 in the reference's order.
__device__ __forceinline__ float deriv5(float m2, float m1, float p1, float p2) {
    float t = m2;
    t -= m1 * 8.0f;
    t += p1 * 8.0f;
    t -= p2;
    t /= 12.0f;
    return t;
}

// `base`: element of the level's pixel (0, 0) in every field (0 for a
// single pair; a pair's offset in the batched solver's planes).
template <int PRIOR>
__device__ __forceinline__ void recon_a_px(const ReconFields& f, const LevelConsts& c,
                                           const Weights& wt, LevelDims d, int ix, int iy,
                                           int first, int uc_from_buffer, int base = 0) {
    const int s = d.s;
    const int pos = base + ix + iy * s;

    // Every load of the pixel is issued before any arithmetic or store, so a
    // thread waits for memory once.  The kernel writes only duhat, uproj and
    // X1 at its own pixel, and reads none of those at another pixel, so the
    // order of loads and stores does not change any value.
    float u = RF_AT(f, u, pos), v = RF_AT(f, v, pos);
    float dix = RF_AT(f, Ix, pos), diy = RF_AT(f, Iy, pos), dit = RF_AT(f, Iz, pos);
    float uproj = RF_AT(f, uproj, pos), vproj = RF_AT(f, vproj, pos);
    float sku = RF_AT(f, sku, pos), skv = RF_AT(f, skv, pos);
    float duhat = 0.0f, dvhat = 0.0f;
    float pu1 = 0.0f, pu2 = 0.0f, pv1 = 0.0f, pv2 = 0.0f;
    float pu1l = 0.0f, pv1l = 0.0f, pu2d = 0.0f, pv2d = 0.0f;
    if (!first) {
        duhat = RF_AT(f, duhat, pos);
        dvhat = RF_AT(f, dvhat, pos);
        pu1 = RF_AT(f, pu1, pos);
        pu2 = RF_AT(f, pu2, pos);
        pv1 = RF_AT(f, pv1, pos);
        pv2 = RF_AT(f, pv2, pos);
        if (ix > 0) {
            pu1l = RF_AT(f, pu1, pos - 1);
            pv1l = RF_AT(f, pv1, pos - 1);
        }
        if (iy > 0) {
            pu2d = RF_AT(f, pu2, pos - s);
            pv2d = RF_AT(f, pv2, pos - s);
        }
    }
    // X0, Y0, Z0 at: 0 = pos, 1 = x+1 (flat pos+1), 2 = y+1 (flat pos+s),
    // 3 = x-1, 4 = y-1.  x+1 / y+1 are read at flat pos+1 / pos+s even on the
    // last column / row (solve3dMinimalArea.cu:65,76).
    float Xn[5], Yn[5], Zn[5];
    Xn[0] = RF_AT(f, X, pos);
    Yn[0] = RF_AT(f, Y, pos);
    Zn[0] = RF_AT(f, Z, pos);
    Xn[1] = RF_AT(f, X, pos + 1);
    Yn[1] = RF_AT(f, Y, pos + 1);
    Zn[1] = RF_AT(f, Z, pos + 1);
    Xn[2] = RF_AT(f, X, pos + s);
    Yn[2] = RF_AT(f, Y, pos + s);
    Zn[2] = RF_AT(f, Z, pos + s);
    Xn[3] = Yn[3] = Zn[3] = 0.0f;
    Xn[4] = Yn[4] = Zn[4] = 0.0f;
    if (ix > 0) {
        Xn[3] = RF_AT(f, X, pos - 1);
        Yn[3] = RF_AT(f, Y, pos - 1);
        Zn[3] = RF_AT(f, Z, pos - 1);
    }
    if (iy > 0) {
        Xn[4] = RF_AT(f, X, pos - s);
        Yn[4] = RF_AT(f, Y, pos - s);
        Zn[4] = RF_AT(f, Z, pos - s);
    }
    float ucb = 0.0f, vcb = 0.0f;
    if (uc_from_buffer) {
        ucb = RF_AT(f, uc, pos);
        vcb = RF_AT(f, vc, pos);
    }
    float ufn = 0.0f, vfn = 0.0f, mk = 1.0f;
    if (PRIOR != 0) {
        ufn = RF_AT(f, ufn, pos);
        vfn = RF_AT(f, vfn, pos);
        if (PRIOR == 2) mk = RF_AT(f, mask, pos);
    }

    // --- data step (solveReconDataL1.cu:24-100) ---
    float A, dusub, dvsub;
    if (PRIOR == 0) {
        A = wt.A;
        dusub = (wt.alpha_tv * duhat + wt.alpha_proj * (uproj - u - sku)) / A;
        dvsub = (wt.alpha_tv * dvhat + wt.alpha_proj * (vproj - v - skv)) / A;
    } else {
        float alphaFn = PRIOR == 2 ? wt.alpha_fn * mk : wt.alpha_fn;
        A = wt.alpha_tv + wt.alpha_proj + alphaFn;
        dusub = (alphaFn * (ufn - u) + wt.alpha_tv * duhat + wt.alpha_proj * (uproj - u - sku)) / A;
        dvsub = (alphaFn * (vfn - v) + wt.alpha_tv * dvhat + wt.alpha_proj * (vproj - v - skv)) / A;
    }
    float du, dv;
    l1_threshold(dusub, dvsub, dix, diy, dit, wt.lambda, A, du, dv);
    float divpu = divergence(pu1, pu1l, pu2, pu2d, ix, iy);
    float divpv = divergence(pv1, pv1l, pv2, pv2d, ix, iy);
    float duhat1 = du + divpu / A;
    float dvhat1 = dv + divpv / A;

    // --- projection blend (solveUVProj.cu:13-21), uc from the current 3D ---
    float uc, vc;
    if (uc_from_buffer) {
        uc = ucb;
        vc = vcb;
    } else {
        project_uc(c, Xn[0], Yn[0], Zn[0], ix, iy, uc, vc);
    }
    float uproj1 = (wt.lambdaf * uc + wt.alpha_proj * (u + duhat1 + sku)) / wt.proj_den;
    float vproj1 = (wt.lambdaf * vc + wt.alpha_proj * (v + dvhat1 + skv)) / wt.proj_den;

    // --- triangulation with minimal-area smoothing (solve3dMinimalArea.cu:23-184) ---
    float Xo, Yo, Zo;
    solve3d_pixel(c, uproj1, vproj1, ix, iy, Xn, Yn, Zn, wt.lambdaf, wt.lambdams, Xo, Yo, Zo);

    RF_AT(f, duhat, pos) = duhat1;
    RF_AT(f, dvhat, pos) = dvhat1;
    RF_AT(f, uproj, pos) = uproj1;
    RF_AT(f, vproj, pos) = vproj1;
    RF_AT(f, X1, pos) = Xo;
    RF_AT(f, Y1, pos) = Yo;
    RF_AT(f, Z1, pos) = Zo;
}

// 3x3 tap of the reference's 3D median with its border rules
// (medianFilter.cu:181-214): left / top clamp, right / bottom and corners 0.
__device__ __forceinline__ int median3_tap(int col, int row, int w, int h, int s) {
    if (col >= 0 && col < w && row >= 0 && row < h) return col + s * row;
    if (col < 0 && row >= 0 && row < h) return s * row;
    if (col >= 0 && col < w && row < 0) return col;
    return -1;
}

// ---------------------------------------------------------------------------
// ReconFlow inner iteration, part B: dual step, 3D median, clean-up, sk
// ---------------------------------------------------------------------------
// Part B's arithmetic and stores at element `pos` from its loaded inputs.
// xin / yin: the right / lower neighbour is inside the level.
__device__ __forceinline__ void recon_b_finish(const ReconFields& f, const Weights& wt, int pos,
                                               bool xin, bool yin, float duhat, float dvhat,
                                               float duhr, float dvhr, float duhd, float dvhd,
                                               float pu1, float pu2, float pv1, float pv2,
                                               float (&mX)[9], float (&mY)[9], float (&mZ)[9],
                                               float sku, float skv, float u, float v,
                                               float uproj, float vproj) {
    // --- dual TV step (solveSmoothDualTVGlobal.cu:26-64) ---
    float dux, duy, dvx, dvy;
    if (!xin) {
        dux = 0.0f;
        dvx = 0.0f;
    } else {
        dux = duhr - duhat;
        dvx = dvhr - dvhat;
    }
    if (!yin) {
        duy = 0.0f;
        dvy = 0.0f;
    } else {
        duy = duhd - duhat;
        dvy = dvhd - dvhat;
    }
    dual_step(dux, duy, wt.fac, pu1, pu2);
    dual_step(dvx, dvy, wt.fac, pv1, pv2);

    // --- 3x3 median of the triangulated points, then clean-up ---
    // (Solve3d outputs are finite: non-finite results fall back to the
    // previous, finite, state; so the min/max median network applies.)
    float X1 = mX[4], Y1 = mY[4], Z1 = mZ[4];
    float Xm = median9_finite(mX);
    float Ym = median9_finite(mY);
    float Zm = median9_finite(mZ);
    float Xo, Yo, Zo;
    cleanup_pixel(X1, Y1, Z1, Xm, Ym, Zm, Xo, Yo, Zo);

    RF_AT(f, pu1, pos) = pu1;
    RF_AT(f, pu2, pos) = pu2;
    RF_AT(f, pv1, pos) = pv1;
    RF_AT(f, pv2, pos) = pv2;
    RF_AT(f, X, pos) = Xo;
    RF_AT(f, Y, pos) = Yo;
    RF_AT(f, Z, pos) = Zo;
    // --- multiplier update (solveUcSk.cu:94-95) ---
    RF_AT(f, sku, pos) = sku + u + duhat - uproj;
    RF_AT(f, skv, pos) = skv + v + dvhat - vproj;
}

__device__ __forceinline__ void recon_b_px(const ReconFields& f, const Weights& wt, LevelDims d,
                                           int ix, int iy, int first, int base = 0) {
    const int s = d.s, w = d.w, h = d.h;
    const int pos = base + ix + iy * s;

    // All loads first (see recon_a_px): the kernel writes p, X and sk only at
    // its own pixel and reads p and sk only there, and reads no X.
    float duhat = RF_AT(f, duhat, pos), dvhat = RF_AT(f, dvhat, pos);
    float duhr = 0.0f, dvhr = 0.0f, duhd = 0.0f, dvhd = 0.0f;
    if ((ix + 1) < w) {
        duhr = RF_AT(f, duhat, pos + 1);
        dvhr = RF_AT(f, dvhat, pos + 1);
    }
    if ((iy + 1) < h) {
        duhd = RF_AT(f, duhat, pos + s);
        dvhd = RF_AT(f, dvhat, pos + s);
    }
    float pu1 = 0.0f, pu2 = 0.0f, pv1 = 0.0f, pv2 = 0.0f;
    if (!first) {
        pu1 = RF_AT(f, pu1, pos);
        pu2 = RF_AT(f, pu2, pos);
        pv1 = RF_AT(f, pv1, pos);
        pv2 = RF_AT(f, pv2, pos);
    }
    float mX[9], mY[9], mZ[9];
    if (ix > 0 && iy > 0 && ix + 1 < w && iy + 1 < h) {
#pragma unroll
        for (int j = 0; j < 3; j++) {
#pragma unroll
            for (int i = 0; i < 3; i++) {
                int at = pos + (j - 1) * s + (i - 1);
                mX[j * 3 + i] = RF_AT(f, X1, at);
                mY[j * 3 + i] = RF_AT(f, Y1, at);
                mZ[j * 3 + i] = RF_AT(f, Z1, at);
            }
        }
    } else {
        // 3x3 taps with the reference's border rules (medianFilter.cu:181-214)
#pragma unroll
        for (int j = 0; j < 3; j++) {
#pragma unroll
            for (int i = 0; i < 3; i++) {
                int at = median3_tap(ix + i - 1, iy + j - 1, w, h, s);
                int k = j * 3 + i;
                mX[k] = at >= 0 ? RF_AT(f, X1, base + at) : 0.0f;
                mY[k] = at >= 0 ? RF_AT(f, Y1, base + at) : 0.0f;
                mZ[k] = at >= 0 ? RF_AT(f, Z1, base + at) : 0.0f;
            }
        }
    }
    const float sku = RF_AT(f, sku, pos), skv = RF_AT(f, skv, pos);
    const float u = RF_AT(f, u, pos), v = RF_AT(f, v, pos);
    const float uproj = RF_AT(f, uproj, pos), vproj = RF_AT(f, vproj, pos);
    recon_b_finish(f, wt, pos, (ix + 1) < w, (iy + 1) < h, duhat, dvhat, duhr, dvhr, duhd, dvhd,
                   pu1, pu2, pv1, pv2, mX, mY, mZ, sku, skv, u, v, uproj, vproj);
}

__device__ __forceinline__ int median5_tap(int col, int row, int w, int h, int s) {
    bool cin = col >= 0 && col < w, rin = row >= 0 && row < h;
    if (cin && rin) return col + s * row;
    if (col < 0 && rin) return s * row;
    if (col >= w && rin) return w - 1 + s * row;
    if (cin && row < 0) return col;
    if (cin && row >= h) return col + s * (h - 1);
    return -1;
}

// The 5x5 window of a field around (ix, iy) with the reference's border
// rules (medianFilter.cu:26-53): taps off the image clamp to the nearest
// row / column; off both, 0.  `base` as recon_a_px.
__device__ __forceinline__ void load_window25(const float* __restrict__ a, int ix, int iy,
                                              LevelDims d, int base, bool interior,
                                              float (&m)[25]) {
    if (interior) {
        const float* p = a + base + ix + iy * d.s;
#pragma unroll
        for (int j = 0; j < 5; j++)
#pragma unroll
            for (int i = 0; i < 5; i++) m[j * 5 + i] = p[(i - 2) + (j - 2) * d.s];
    } else {
#pragma unroll
        for (int j = 0; j < 5; j++)
#pragma unroll
            for (int i = 0; i < 5; i++) {
                int at = median5_tap(ix + i - 2, iy + j - 2, d.w, d.h, d.s);
                m[j * 5 + i] = at >= 0 ? a[base + at] : 0.0f;
            }
    }
}

// Exchange-path median of a window, re-read from memory (kept out of line:
// it runs only for NaN inputs or a zero result).
__device__ __noinline__ float median25_slow(const float* __restrict__ a, int ix, int iy,
                                            LevelDims d, int base, bool interior) {
    float m[25];
    load_window25(a, ix, iy, d, base, interior, m);
    return median25_resolve(m);
}

// MedianFilterKernel5 (medianFilter.cu:3-76) of two fields at one pixel.
__device__ __forceinline__ void median5_pair(const float* __restrict__ a,
                                             const float* __restrict__ b, int ix, int iy,
                                             LevelDims d, float& ma, float& mb, int base = 0) {
    const bool interior = ix >= 2 && iy >= 2 && ix + 2 < d.w && iy + 2 < d.h;
    float mu[25], mv[25];
    load_window25(a, ix, iy, d, base, interior, mu);
    load_window25(b, ix, iy, d, base, interior, mv);
    if (!median25_net(mu, ma)) ma = median25_slow(a, ix, iy, d, base, interior);
    if (!median25_net(mv, mb)) mb = median25_slow(b, ix, iy, d, base, interior);
}

// Six rows of five taps around (ix, iy): rows iy-2 .. iy+3, the 5x5
// windows of (ix, iy) and (ix, iy+1) with the reference's border rules
// (median5_tap: the rule depends only on the tap's position, so a tap
// shared by both windows has one value).  `interior`: every tap inside.
__device__ __forceinline__ void load_window30(const float* __restrict__ a, int ix, int iy,
                                              LevelDims d, int base, bool interior,
                                              float (&m)[30]) {
    if (interior) {
        const float* p = a + base + ix + iy * d.s;
#pragma unroll
        for (int j = 0; j < 6; j++)
#pragma unroll
            for (int i = 0; i < 5; i++) m[j * 5 + i] = p[(i - 2) + (j - 2) * d.s];
    } else {
#pragma unroll
        for (int j = 0; j < 6; j++)
#pragma unroll
            for (int i = 0; i < 5; i++) {
                int at = median5_tap(ix + i - 2, iy + j - 2, d.w, d.h, d.s);
                m[j * 5 + i] = at >= 0 ? a[base + at] : 0.0f;
            }
    }
}

// The median of one pixel's window on its own (the network, then the
// exchange path for NaN or zero): the two-pixel form's answer when either
// window holds a NaN.  Out of line: it runs only for NaN inputs.
__device__ __noinline__ float median25_single(const float* __restrict__ a, int ix, int iy,
                                              LevelDims d, int base, bool interior) {
    float m[25];
    load_window25(a, ix, iy, d, base, interior, m);
    float r;
    if (!median25_net(m, r)) r = median25_slow(a, ix, iy, d, base, interior);
    return r;
}

// MedianFilterKernel5 (medianFilter.cu:3-76) of two fields at (ix, iy) and
// (ix, iy + 1) (the second only when iy + 1 < d.h; its outputs are then
// unused otherwise): 20 of each window's 25 taps are shared, sorted once
// (median25_two).  A NaN among the 30 taps sends both pixels to the
// one-window path (the NaN may lie in one window only); a zero result takes
// the exchange path of the pixel concerned, as median5_pair does.
__device__ __forceinline__ void median5_pair2(const float* __restrict__ a,
                                              const float* __restrict__ b, int ix, int iy,
                                              LevelDims d, float (&ma)[2], float (&mb)[2],
                                              int base = 0) {
    const bool in_x = ix >= 2 && ix + 2 < d.w;
    const bool interior = in_x && iy >= 2 && iy + 3 < d.h;
    const bool in0 = in_x && iy >= 2 && iy + 2 < d.h;
    const bool in1 = in_x && iy + 1 >= 2 && iy + 3 < d.h;
    const bool has1 = iy + 1 < d.h;
    float w[30];
    load_window30(a, ix, iy, d, base, interior, w);
    if (!median25_two(w, ma[0], ma[1])) {
        ma[0] = median25_single(a, ix, iy, d, base, in0);
        ma[1] = has1 ? median25_single(a, ix, iy + 1, d, base, in1) : 0.0f;
    } else {
        if (ma[0] == 0.0f) ma[0] = median25_slow(a, ix, iy, d, base, in0);
        if (has1 && ma[1] == 0.0f) ma[1] = median25_slow(a, ix, iy + 1, d, base, in1);
    }
    load_window30(b, ix, iy, d, base, interior, w);
    if (!median25_two(w, mb[0], mb[1])) {
        mb[0] = median25_single(b, ix, iy, d, base, in0);
        mb[1] = has1 ? median25_single(b, ix, iy + 1, d, base, in1) : 0.0f;
    } else {
        if (mb[0] == 0.0f) mb[0] = median25_slow(b, ix, iy, d, base, in0);
        if (has1 && mb[1] == 0.0f) mb[1] = median25_slow(b, ix, iy + 1, d, base, in1);
    }
}

// warpImage.cu:15-29
__device__ __forceinline__ void warp_px(const float* __restrict__ I1, const float* __restrict__ u,
                                        const float* __restrict__ v, LevelDims d,
                                        float* __restrict__ out, int ix, int iy) {
    int pos = ix + iy * d.s;
    float x = ((float)ix + u[pos] + 0.5f) / (float)d.w;
    float y = ((float)iy + v[pos] + 0.5f) / (float)d.h;
    out[pos] = tex2d(I1, d.w, d.h, d.s, x, y);
}

// WarpImage and ComputeDerivatives fused through shared memory, for one
// block-shaped tile (tw x th pixels at x0, y0; the block's threads).  The
// tile plus a 2-pixel halo of I0 and of the warped I1 are staged in `sm`
// ((tw + 4) x (th + 4) floats each); a halo cell outside the level holds the
// value at its mirrored pixel, which is what the derivative taps read
// (computeDerivatives.cu:26-56), and the warped value of every cell is
// warp_px's arithmetic at that pixel, so Ix, Iy, Iz are bit-identical to
// the two-kernel path while the warped image never leaves the chip.  Every
// thread of the block must call it (it synchronises the block).
__device__ __forceinline__ void warp_deriv_tile(const float* __restrict__ I0,
                                                const float* __restrict__ I1,
                                                const float* __restrict__ u,
                                                const float* __restrict__ v, LevelDims d, int x0,
                                                int y0, int tw, int th, float* sm,
                                                float* __restrict__ Ix, float* __restrict__ Iy,
                                                float* __restrict__ Iz) {
    const int sw = tw + 4, cells = sw * (th + 4);
    float* sI0 = sm;
    float* sW = sm + cells;
    const int tid = threadIdx.x + threadIdx.y * blockDim.x;
    const int nthr = blockDim.x * blockDim.y;
    for (int c = tid; c < cells; c += nthr) {
        const int mx = mirror_index(x0 + c % sw - 2, d.w);
        const int my = mirror_index(y0 + c / sw - 2, d.h);
        const int p = mx + my * d.s;
        const float x = ((float)mx + u[p] + 0.5f) / (float)d.w;
        const float y = ((float)my + v[p] + 0.5f) / (float)d.h;
        sI0[c] = I0[p];
        sW[c] = tex2d(I1, d.w, d.h, d.s, x, y);
    }
    __syncthreads();
    const int ix = x0 + (int)threadIdx.x, iy = y0 + (int)threadIdx.y;
    if (ix >= d.w || iy >= d.h) return;
    const int c = (threadIdx.x + 2) + (threadIdx.y + 2) * sw;
    const int pos = ix + iy * d.s;
    float t0 = deriv5(sI0[c - 2], sI0[c - 1], sI0[c + 1], sI0[c + 2]);
    float t1 = deriv5(sW[c - 2], sW[c - 1], sW[c + 1], sW[c + 2]);
    Ix[pos] = (t0 + t1) * 0.5f;
    Iz[pos] = sW[c] - sI0[c];
    t0 = deriv5(sI0[c - 2 * sw], sI0[c - sw], sI0[c + sw], sI0[c + 2 * sw]);
    t1 = deriv5(sW[c - 2 * sw], sW[c - sw], sW[c + sw], sW[c + 2 * sw]);
    Iy[pos] = (t0 + t1) * 0.5f;
}

// computeDerivatives.cu:8-57 (taps on texel centres: mirrored gathers)
__device__ __forceinline__ void derivatives_px(const float* __restrict__ I0,
                                               const float* __restrict__ I1, LevelDims d,
                                               float* __restrict__ Ix, float* __restrict__ Iy,
                                               float* __restrict__ Iz, int ix, int iy) {
    int row = iy * d.s;
    int pos = ix + row;
    int xm2 = mirror_index(ix - 2, d.w) + row, xm1 = mirror_index(ix - 1, d.w) + row;
    int xp1 = mirror_index(ix + 1, d.w) + row, xp2 = mirror_index(ix + 2, d.w) + row;
    int ym2 = ix + mirror_index(iy - 2, d.h) * d.s, ym1 = ix + mirror_index(iy - 1, d.h) * d.s;
    int yp1 = ix + mirror_index(iy + 1, d.h) * d.s, yp2 = ix + mirror_index(iy + 2, d.h) * d.s;
    float t0 = deriv5(I0[xm2], I0[xm1], I0[xp1], I0[xp2]);
    float t1 = deriv5(I1[xm2], I1[xm1], I1[xp1], I1[xp2]);
    Ix[pos] = (t0 + t1) * 0.5f;
    Iz[pos] = I1[pos] - I0[pos];
    t0 = deriv5(I0[ym2], I0[ym1], I0[yp1], I0[yp2]);
    t1 = deriv5(I1[ym2], I1[ym1], I1[yp1], I1[yp2]);
    Iy[pos] = (t0 + t1) * 0.5f;
}

// solveDataL1.cu:4-91 (duhat updated in place: read and written only at the pixel)
__device__ __forceinline__ void plain_data_px(float* duhat0, float* dvhat0,
                                              const float* __restrict__ pu1,
                                              const float* __restrict__ pu2,
                                              const float* __restrict__ pv1,
                                              const float* __restrict__ pv2,
                                              const float* __restrict__ Ix,
                                              const float* __restrict__ Iy,
                                              const float* __restrict__ Iz, const Weights& wt,
                                              LevelDims d, int first, int ix, int iy) {
    const int s = d.s;
    const int pos = ix + iy * s;
    float duhat = 0.0f, dvhat = 0.0f;
    float p1u = 0.0f, p2u = 0.0f, p1v = 0.0f, p2v = 0.0f, p1ul = 0.0f, p1vl = 0.0f, p2ud = 0.0f,
          p2vd = 0.0f;
    if (!first) {
        duhat = duhat0[pos];
        dvhat = dvhat0[pos];
        p1u = pu1[pos];
        p2u = pu2[pos];
        p1v = pv1[pos];
        p2v = pv2[pos];
        if (ix > 0) {
            p1ul = pu1[pos - 1];
            p1vl = pv1[pos - 1];
        }
        if (iy > 0) {
            p2ud = pu2[pos - s];
            p2vd = pv2[pos - s];
        }
    }
    float du, dv;
    l1_threshold_plain(duhat, dvhat, Ix[pos], Iy[pos], Iz[pos], wt.lambda, wt.theta, du, dv);
    float divpu = divergence(p1u, p1ul, p2u, p2ud, ix, iy);
    float divpv = divergence(p1v, p1vl, p2v, p2vd, ix, iy);
    duhat0[pos] = du + wt.theta * divpu;
    dvhat0[pos] = dv + wt.theta * divpv;
}

// solveSmoothDualTVGlobal.cu:4-65 (p updated in place: read and written only at the pixel)
__device__ __forceinline__ void plain_tv_px(const float* __restrict__ duhat,
                                            const float* __restrict__ dvhat, float* pu1,
                                            float* pu2, float* pv1, float* pv2,
                                            const Weights& wt, LevelDims d, int first, int ix,
                                            int iy) {
    const int s = d.s;
    const int pos = ix + iy * s;
    float du0 = duhat[pos], dv0 = dvhat[pos];
    float dux = 0.0f, duy = 0.0f, dvx = 0.0f, dvy = 0.0f;
    if (ix + 1 < d.w) {
        dux = duhat[pos + 1] - du0;
        dvx = dvhat[pos + 1] - dv0;
    }
    if (iy + 1 < d.h) {
        duy = duhat[pos + s] - du0;
        dvy = dvhat[pos + s] - dv0;
    }
    float a = 0.0f, b = 0.0f, c = 0.0f, e = 0.0f;
    if (!first) {
        a = pu1[pos];
        b = pu2[pos];
        c = pv1[pos];
        e = pv2[pos];
    }
    dual_step(dux, duy, wt.fac, a, b);
    dual_step(dvx, dvy, wt.fac, c, e);
    pu1[pos] = a;
    pu2[pos] = b;
    pv1[pos] = c;
    pv2[pos] = e;
}


}  // namespace
}  // namespace rf
