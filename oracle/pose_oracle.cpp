// Oracle (test infrastructure only): a CPU restatement of the pose front
// end's feature stages -- integral image, box-filter Hessian responses,
// keypoint selection and refinement, orientation, descriptor, brute-force
// matching -- with the definitions the GPU path uses (SURF as published:
// H. Bay, A. Ess, T. Tuytelaars, L. Van Gool, CVIU 110(3), 2008; the
// reference's own detector is OpenCV's closed SURF_CUDA, called from
// reconflow/CameraPose.cpp:53-54, and its matcher is the brute-force k = 2
// search with the 0.6 ratio test of CameraPose.cpp:56-78).  Compiled with
// -ffp-contract=off: FP32 operations in written order, so the results equal
// the GPU's bit for bit.  The reference itself cannot run here (OpenCV with
// CUDA is absent), so this restatement is pinned by property tests, not by
// the reference's outputs.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

const float kPi = 3.14159265358979323846f;
const float kTwoPi = 6.28318530717958647692f;
const float kHalfPi = 1.57079632679489661923f;
const float kTwoOverPi = 0.63661977236758134308f;
const float kOriStep = 0.08726646259971647884f;
const float kOriWin = 1.04719755119659774615f;

int filter_size(int o, int k) { return 3 * ((2 << o) * (k + 1) + 1); }

// atan on [0, 1] (pi/6 shift above tan 15 degrees, odd Taylor series to z^11)
float atan_unit(float z) {
    float off = 0.0f;
    if (z > 0.267949192f) {
        z = (z * 1.73205081f - 1.0f) / (z + 1.73205081f);
        off = 0.523598776f;
    }
    const float z2 = z * z;
    float p = -0.0909090909f;
    p = p * z2 + 0.111111111f;
    p = p * z2 - 0.142857143f;
    p = p * z2 + 0.2f;
    p = p * z2 - 0.333333333f;
    p = p * z2 + 1.0f;
    return off + z * p;
}

float atan2_pos(float y, float x) {
    if (x == 0.0f && y == 0.0f) return 0.0f;
    const float ax = std::fabs(x), ay = std::fabs(y);
    float a = ay <= ax ? atan_unit(ay / ax) : kHalfPi - atan_unit(ax / ay);
    if (x < 0.0f) a = kPi - a;
    if (y < 0.0f) a = kTwoPi - a;
    if (a >= kTwoPi) a = 0.0f;
    return a;
}

void sincos_own(float a, float& s, float& c) {
    const float q = std::floor(a * kTwoOverPi + 0.5f);
    const float r = a - q * kHalfPi;
    const int k = ((int)q) & 3;
    const float r2 = r * r;
    float ps = 2.75573192e-6f;
    ps = ps * r2 - 1.98412698e-4f;
    ps = ps * r2 + 8.33333333e-3f;
    ps = ps * r2 - 0.166666667f;
    ps = ps * r2 + 1.0f;
    const float sr = r * ps;
    float pc = 2.48015873e-5f;
    pc = pc * r2 - 1.38888889e-3f;
    pc = pc * r2 + 4.16666667e-2f;
    pc = pc * r2 - 0.5f;
    const float cr = pc * r2 + 1.0f;
    if (k == 0) { s = sr; c = cr; }
    else if (k == 1) { s = cr; c = -sr; }
    else if (k == 2) { s = -sr; c = -cr; }
    else { s = -cr; c = sr; }
}

struct Integral {
    int w, h;
    std::vector<uint32_t> S;  // (h + 1) x (w + 1)
    uint32_t at(int x, int y) const { return S[(size_t)y * (w + 1) + x]; }
    int box(int x0, int y0, int x1, int y1) const {
        return (int)(at(x1, y1) - at(x1, y0) - at(x0, y1) + at(x0, y0));
    }
    int clipped(int x0, int y0, int x1, int y1) const {
        x0 = std::min(std::max(x0, 0), w);
        x1 = std::min(std::max(x1, 0), w);
        y0 = std::min(std::max(y0, 0), h);
        y1 = std::min(std::max(y1, 0), h);
        if (x1 <= x0 || y1 <= y0) return 0;
        return box(x0, y0, x1, y1);
    }
    void haar(int px, int py, int half, float& dx, float& dy) const {
        dx = (float)(clipped(px, py - half, px + half, py + half) -
                     clipped(px - half, py - half, px, py + half));
        dy = (float)(clipped(px - half, py, px + half, py + half) -
                     clipped(px - half, py - half, px + half, py));
    }
};

Integral integral(const uint8_t* img, int w, int h) {
    Integral I{w, h, std::vector<uint32_t>((size_t)(w + 1) * (h + 1), 0u)};
    for (int y = 0; y < h; y++) {
        uint32_t row = 0;
        for (int x = 0; x < w; x++) {
            row += img[(size_t)y * w + x];
            I.S[(size_t)(y + 1) * (w + 1) + x + 1] = I.S[(size_t)y * (w + 1) + x + 1] + row;
        }
    }
    return I;
}

// determinant-of-Hessian response at pixel (x, y) for filter size L
float hessian(const Integral& I, int x, int y, int L) {
    const int l = L / 3, r = (L - 1) / 2, c = (l - 1) / 2;
    if (!(x >= r && x < I.w - r && y >= r && y < I.h - r)) return 0.0f;
    const int left = I.box(x - c - l, y - l + 1, x - c, y + l);
    const int right = I.box(x + c + 1, y - l + 1, x + c + 1 + l, y + l);
    const int mid = I.box(x - c, y - l + 1, x + c + 1, y + l);
    const int top = I.box(x - l + 1, y - c - l, x + l, y - c);
    const int bottom = I.box(x - l + 1, y + c + 1, x + l, y + c + 1 + l);
    const int centre = I.box(x - l + 1, y - c, x + l, y + c + 1);
    const int tl = I.box(x - l, y - l, x, y), br = I.box(x + 1, y + 1, x + 1 + l, y + 1 + l);
    const int tr = I.box(x + 1, y - l, x + 1 + l, y), bl = I.box(x - l, y + 1, x, y + 1 + l);
    const int dxx = left + right - 2 * mid;
    const int dyy = top + bottom - 2 * centre;
    const int dxy = tl + br - tr - bl;
    const float inv = 1.0f / (float)(L * L);
    const float fxx = (float)dxx * inv, fyy = (float)dyy * inv, fxy = (float)dxy * inv;
    const float a = fxx * fyy;
    const float b = 0.81f * fxy;
    return a - b * fxy;
}

struct Kp {
    float x, y, scale, response, angle;
    int octave, layer, cell;
};

bool kp_order(const Kp& a, const Kp& b) {
    if (a.response != b.response) return a.response > b.response;
    if (a.octave != b.octave) return a.octave < b.octave;
    if (a.layer != b.layer) return a.layer < b.layer;
    return a.cell < b.cell;
}

}  // namespace

extern "C" {

// integral image, (h + 1) x (w + 1)
void rfo_surf_integral(const uint8_t* img, int w, int h, uint32_t* out) {
    const Integral I = integral(img, w, h);
    std::memcpy(out, I.S.data(), I.S.size() * sizeof(uint32_t));
}

// responses of one octave: layers x (h >> o) x (w >> o)
void rfo_surf_responses(const uint8_t* img, int w, int h, int octave, int layers, float* out) {
    const Integral I = integral(img, w, h);
    const int cols = w >> octave, rows = h >> octave;
    for (int k = 0; k < layers; k++)
        for (int j = 0; j < rows; j++)
            for (int i = 0; i < cols; i++)
                out[((size_t)k * rows + j) * cols + i] =
                    hessian(I, i << octave, j << octave, filter_size(octave, k));
}

// Keypoints (x, y, scale, angle, response, octave as float) and descriptors
// of one frame; returns the keypoint count (at most max_kp), or -1 when the
// candidates exceed cand_cap.
int rfo_surf_detect(const uint8_t* img, int w, int h, double threshold, int n_octaves,
                    int n_layers, int max_kp, int cand_cap, float* kp_out, float* desc_out) {
    const Integral I = integral(img, w, h);
    const int layers = n_layers + 2;
    std::vector<Kp> cand;
    for (int o = 0; o < n_octaves; o++) {
        const int cols = w >> o, rows = h >> o, step = 1 << o;
        if (cols < 1 || rows < 1) break;
        std::vector<float> R((size_t)layers * rows * cols);
        for (int k = 0; k < layers; k++)
            for (int j = 0; j < rows; j++)
                for (int i = 0; i < cols; i++)
                    R[((size_t)k * rows + j) * cols + i] = hessian(I, i << o, j << o, filter_size(o, k));
        auto at = [&](int k, int j, int i) { return R[((size_t)k * rows + j) * cols + i]; };
        const float thr = (float)threshold;
        for (int k = 1; k <= n_layers; k++) {
            const int rb = (filter_size(o, k + 1) - 1) / 2;
            for (int j = 0; j < rows; j++)
                for (int i = 0; i < cols; i++) {
                    const int x = i << o, y = j << o;
                    if (x - step < rb || x + step >= w - rb || y - step < rb || y + step >= h - rb)
                        continue;
                    const float v = at(k, j, i);
                    if (!(v > thr)) continue;
                    bool peak = true;
                    for (int dk = -1; dk <= 1 && peak; dk++)
                        for (int dj = -1; dj <= 1 && peak; dj++)
                            for (int di = -1; di <= 1 && peak; di++)
                                if ((dk || dj || di) && !(v > at(k + dk, j + dj, i + di))) peak = false;
                    if (!peak) continue;
                    // one Newton step on the quadratic through the 3x3x3 neighbourhood
                    const float gx = (at(k, j, i + 1) - at(k, j, i - 1)) * 0.5f;
                    const float gy = (at(k, j + 1, i) - at(k, j - 1, i)) * 0.5f;
                    const float gs = (at(k + 1, j, i) - at(k - 1, j, i)) * 0.5f;
                    const float hxx = (at(k, j, i + 1) + at(k, j, i - 1)) - 2.0f * v;
                    const float hyy = (at(k, j + 1, i) + at(k, j - 1, i)) - 2.0f * v;
                    const float hss = (at(k + 1, j, i) + at(k - 1, j, i)) - 2.0f * v;
                    const float hxy = (((at(k, j + 1, i + 1) - at(k, j + 1, i - 1)) -
                                        at(k, j - 1, i + 1)) + at(k, j - 1, i - 1)) * 0.25f;
                    const float hxs = (((at(k + 1, j, i + 1) - at(k + 1, j, i - 1)) -
                                        at(k - 1, j, i + 1)) + at(k - 1, j, i - 1)) * 0.25f;
                    const float hys = (((at(k + 1, j + 1, i) - at(k + 1, j - 1, i)) -
                                        at(k - 1, j + 1, i)) + at(k - 1, j - 1, i)) * 0.25f;
                    // Cramer's rule on [hxx hxy hxs; hxy hyy hys; hxs hys hss] o = -g
                    const float b1 = -gx, b2 = -gy, b3 = -gs;
                    const float m1 = hyy * hss - hys * hys;
                    const float det = hxx * m1 - hxy * (hxy * hss - hys * hxs) +
                                      hxs * (hxy * hys - hyy * hxs);
                    if (!(det != 0.0f)) continue;
                    const float nx = b1 * m1 - hxy * (b2 * hss - hys * b3) + hxs * (b2 * hys - hyy * b3);
                    const float ny = hxx * (b2 * hss - hys * b3) - b1 * (hxy * hss - hys * hxs) +
                                     hxs * (hxy * b3 - b2 * hxs);
                    const float ns = hxx * (hyy * b3 - b2 * hys) - hxy * (hxy * b3 - b2 * hxs) +
                                     b1 * (hxy * hys - hyy * hxs);
                    const float ox = nx / det, oy = ny / det, os = ns / det;
                    if (!(std::fabs(ox) <= 0.5f && std::fabs(oy) <= 0.5f && std::fabs(os) <= 0.5f))
                        continue;
                    const int L0 = filter_size(o, k), dL = filter_size(o, k + 1) - L0;
                    const float Lf = (float)L0 + os * (float)dL;
                    Kp p;
                    p.x = ((float)i + ox) * (float)step;
                    p.y = ((float)j + oy) * (float)step;
                    p.scale = 1.2f * Lf / 9.0f;
                    p.response = v;
                    p.angle = 0.0f;
                    p.octave = o;
                    p.layer = k;
                    p.cell = j * cols + i;
                    cand.push_back(p);
                }
        }
    }
    if ((int)cand.size() > cand_cap) return -1;
    std::sort(cand.begin(), cand.end(), kp_order);
    if ((int)cand.size() > max_kp) cand.resize(max_kp);
    // sample grid and Gaussian weights (double, then float)
    std::vector<int> oi, oj;
    std::vector<float> ow;
    for (int j = -6; j <= 6; j++)
        for (int i = -6; i <= 6; i++)
            if (i * i + j * j < 36) {
                oi.push_back(i);
                oj.push_back(j);
                ow.push_back((float)std::exp(-(double)(i * i + j * j) / (2.0 * 2.5 * 2.5)));
            }
    float dw[400];
    for (int V = 0; V < 20; V++)
        for (int U = 0; U < 20; U++) {
            const double ou = U - 9.5, ov = V - 9.5;
            dw[V * 20 + U] = (float)std::exp(-(ou * ou + ov * ov) / (2.0 * 3.3 * 3.3));
        }
    const int n = (int)cand.size();
    const int ns = (int)oi.size();
    std::vector<float> sx(ns), sy(ns), sa(ns);
    for (int q = 0; q < n; q++) {
        Kp& p = cand[q];
        const float s = p.scale;
        // orientation
        const int half4 = std::max(1, (int)std::floor(2.0f * s + 0.5f));
        for (int t = 0; t < ns; t++) {
            const float fxp = (float)oi[t] * s, fyp = (float)oj[t] * s;
            const int px = (int)std::floor(p.x + fxp + 0.5f);
            const int py = (int)std::floor(p.y + fyp + 0.5f);
            float dx, dy;
            I.haar(px, py, half4, dx, dy);
            sx[t] = ow[t] * dx;
            sy[t] = ow[t] * dy;
            sa[t] = atan2_pos(sy[t], sx[t]);
        }
        float best = -1.0f, bx = 0.0f, by = 0.0f;
        for (int win = 0; win < 72; win++) {
            const float a0 = (float)win * kOriStep;
            float ax = 0.0f, ay = 0.0f;
            for (int t = 0; t < ns; t++) {
                float d = sa[t] - a0;
                if (d < 0.0f) d = d + kTwoPi;
                if (d < kOriWin) {
                    ax = ax + sx[t];
                    ay = ay + sy[t];
                }
            }
            const float mag = ax * ax + ay * ay;
            if (mag > best) {
                best = mag;
                bx = ax;
                by = ay;
            }
        }
        p.angle = best > 0.0f ? atan2_pos(by, bx) : 0.0f;
        // descriptor
        float sn, c;
        sincos_own(p.angle, sn, c);
        const int half2 = std::max(1, (int)std::floor(s + 0.5f));
        float d[64];
        for (int sv = 0; sv < 4; sv++)
            for (int su = 0; su < 4; su++) {
                float a = 0.0f, b = 0.0f, aa = 0.0f, ab = 0.0f;
                for (int v = 0; v < 5; v++)
                    for (int u = 0; u < 5; u++) {
                        const int U = su * 5 + u, V = sv * 5 + v;
                        const float ou = (float)U - 9.5f, ov = (float)V - 9.5f;
                        const float rxp = c * ou - sn * ov, ryp = sn * ou + c * ov;
                        const int px = (int)std::floor(p.x + s * rxp + 0.5f);
                        const int py = (int)std::floor(p.y + s * ryp + 0.5f);
                        float dx, dy;
                        I.haar(px, py, half2, dx, dy);
                        const float g = dw[V * 20 + U];
                        const float rx = g * (c * dx + sn * dy), ry = g * (c * dy - sn * dx);
                        a = a + rx;
                        b = b + ry;
                        aa = aa + std::fabs(rx);
                        ab = ab + std::fabs(ry);
                    }
                const int base = (sv * 4 + su) * 4;
                d[base] = a;
                d[base + 1] = b;
                d[base + 2] = aa;
                d[base + 3] = ab;
            }
        float n2 = 0.0f;
        for (int t = 0; t < 64; t++) n2 = n2 + d[t] * d[t];
        const float nv = std::sqrt(n2);
        for (int t = 0; t < 64; t++) desc_out[(size_t)q * 64 + t] = nv > 0.0f ? d[t] / nv : 0.0f;
        float* k = kp_out + (size_t)q * 6;
        k[0] = p.x;
        k[1] = p.y;
        k[2] = p.scale;
        k[3] = p.angle;
        k[4] = p.response;
        k[5] = (float)p.octave;
    }
    return n;
}

// the two nearest descriptors of frame 1 for every descriptor of frame 0:
// squared distances summed in descriptor order, ties to the lower index
void rfo_surf_match(const float* d0, int n0, const float* d1, int n1, int* best, float* b1,
                    float* b2) {
    for (int q = 0; q < n0; q++) {
        float e1 = INFINITY, e2 = INFINITY;
        int i1 = -1;
        for (int t = 0; t < n1; t++) {
            float d = 0.0f;
            for (int k = 0; k < 64; k++) {
                const float e = d0[(size_t)q * 64 + k] - d1[(size_t)t * 64 + k];
                d = d + e * e;
            }
            if (d < e1) {
                e2 = e1;
                e1 = d;
                i1 = t;
            } else if (d < e2) {
                e2 = d;
            }
        }
        best[q] = i1;
        b1[q] = e1;
        b2[q] = e2;
    }
}

}  // extern "C"
