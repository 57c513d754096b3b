// Five-point relative pose (D. Nister, "An efficient solution to the
// five-point relative pose problem", IEEE PAMI 26(6), 2004), written as host
// and device code (no contraction on either side, correctly rounded
// division and square root, exact frexp / ldexp, so both give the same
// doubles).  The LMedS runs it on host threads (~12 us a solve on one x86
// core): one GPU thread per sample took 3.6 ms for a pose's 134 solves (a
// long chain of dependent FP64 operations and ~6 KB of local arrays per
// thread).
//
// Steps: null space of the 5 x 9 epipolar system by Householder QR, E = x X
// + y Y + z Z + W; the ten cubic constraints det(E) = 0 and 2 E E^T E -
// tr(E E^T) E = 0 over the twenty monomials in Nister's order; Gauss-Jordan
// elimination of the first ten columns; the rows <k> = <e> - z<f>,
// <l> = <g> - z<h>, <m> = <i> - z<j> as a 3 x 3 matrix of polynomials in z;
// its degree-10 determinant; the real roots (bracketed between the real
// roots of the derivatives, refined by Newton steps safeguarded by bisection
// inside each bracket); x, y from the null vector of B(z).
#pragma once

#include <math.h>

#ifdef __CUDACC__
#define RF_HD __host__ __device__
#else
#define RF_HD
#endif

namespace rf_fivept {

// Polynomials in (x, y, z): linear [x, y, z, 1]; quadratic over x^2 y^2 z^2
// xy xz yz x y z 1; cubic over Nister's twenty monomials x^3 y^3 x^2y xy^2
// x^2z x^2 y^2z y^2 xyz xy | xz^2 xz x yz^2 yz y z^3 z^2 z 1.  The product
// tables give the monomial index of each product of two monomials.
struct Lin {
    double c[4];
};
struct Quad {
    double c[10];
};
struct Cub {
    double c[20];
};

RF_HD inline Quad mul(const Lin& a, const Lin& b) {
    const int ll[4][4] = {{0, 3, 4, 6}, {3, 1, 5, 7}, {4, 5, 2, 8}, {6, 7, 8, 9}};
    Quad r{};
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) r.c[ll[i][j]] += a.c[i] * b.c[j];
    return r;
}

RF_HD inline Cub mul(const Quad& a, const Lin& b) {
    const int ql[10][4] = {{0, 2, 4, 5},     {3, 1, 6, 7},     {10, 13, 16, 17}, {2, 3, 8, 9},
                           {4, 8, 10, 11},   {8, 6, 13, 14},   {5, 9, 11, 12},   {9, 7, 14, 15},
                           {11, 14, 17, 18}, {12, 15, 18, 19}};
    Cub r{};
    for (int i = 0; i < 10; i++)
        for (int j = 0; j < 4; j++) r.c[ql[i][j]] += a.c[i] * b.c[j];
    return r;
}

template <class P>
RF_HD inline P lin_comb(const P& a, double ka, const P& b, double kb) {
    P r;
    for (int i = 0; i < (int)(sizeof(a.c) / sizeof(double)); i++) r.c[i] = ka * a.c[i] + kb * b.c[i];
    return r;
}

// polynomials in z of degree <= 10, coefficient k of z^k
struct Poly1 {
    double c[11];
    int n;  // number of coefficients
};

RF_HD inline Poly1 poly3(double c0, double c1, double c2) {
    Poly1 r{};
    r.c[0] = c0;
    r.c[1] = c1;
    r.c[2] = c2;
    r.n = 3;
    return r;
}

RF_HD inline Poly1 poly4(double c0, double c1, double c2, double c3) {
    Poly1 r = poly3(c0, c1, c2);
    r.c[3] = c3;
    r.n = 4;
    return r;
}

RF_HD inline Poly1 pmul(const Poly1& a, const Poly1& b) {
    Poly1 r{};
    r.n = a.n + b.n - 1;
    for (int i = 0; i < a.n; i++)
        for (int j = 0; j < b.n; j++) r.c[i + j] += a.c[i] * b.c[j];
    return r;
}

RF_HD inline Poly1 padd(const Poly1& a, const Poly1& b, double kb) {
    Poly1 r{};
    r.n = a.n > b.n ? a.n : b.n;
    for (int i = 0; i < a.n; i++) r.c[i] += a.c[i];
    for (int i = 0; i < b.n; i++) r.c[i] += kb * b.c[i];
    return r;
}

// z times p
RF_HD inline Poly1 pshift(const Poly1& a) {
    Poly1 r{};
    r.n = a.n + 1;
    for (int i = 0; i < a.n; i++) r.c[i + 1] = a.c[i];
    return r;
}

RF_HD inline double peval(const Poly1& p, double z) {
    double r = 0.0;
    for (int i = p.n; i-- > 0;) r = r * z + p.c[i];
    return r;
}

// p(z), p'(z) and sum |c_k| |z|^k (the scale of p's rounding error at z)
// in one Horner pass.
RF_HD inline void peval_d(const Poly1& p, double z, double& f, double& df, double& mag) {
    const double az = fabs(z);
    f = p.c[p.n - 1];
    df = 0.0;
    mag = fabs(f);
    for (int i = p.n - 1; i-- > 0;) {
        df = df * z + f;
        f = f * z + p.c[i];
        mag = mag * az + fabs(p.c[i]);
    }
}

// Root of p in [lo, hi] where p changes sign (neg_lo: p(lo) < 0): Newton
// steps safeguarded by the bracket (each evaluation shrinks it); a step
// that would leave the bracket, or that is not at most half the previous
// step, is replaced by a bisection.  Ends when p(x) is within about two
// units in the last place of sum |c_k| |x|^k (the usual size of Horner's
// rounding error), or when a Newton step or the bracket is below `rel` of
// the root's magnitude (at least 1).
RF_HD inline double bracket_root(const Poly1& p, double lo, double hi, bool neg_lo, double rel) {
    double x = 0.5 * (lo + hi), last = hi - lo;
    for (int it = 0; it < 200; it++) {
        double f, df, mag;
        peval_d(p, x, f, df, mag);
        if (fabs(f) <= 2.5e-16 * mag) return x;
        if ((f < 0.0) == neg_lo)
            lo = x;
        else
            hi = x;
        const double ax = fabs(x);
        const double tol = rel * (ax > 1.0 ? ax : 1.0);
        const double xn = x - f / df;  // inf / NaN when df = 0: fails the tests below
        double step;
        if (xn > lo && xn < hi && 2.0 * fabs(xn - x) <= last) {
            step = fabs(xn - x);
            x = xn;
            if (step <= tol) return x;
        } else {
            x = 0.5 * (lo + hi);
            step = 0.5 * (hi - lo);
        }
        if (hi - lo <= tol) return x;
        last = step;
    }
    return x;
}

// A power of two above every root's magnitude (Fujiwara's bound
// 2 max_k |a_(n-k) / a_n|^(1/k) with each term rounded up to a power of
// two through its binary exponent, so no pow is needed).
RF_HD inline double root_bound(const Poly1& p) {
    const int deg = p.n - 1;
    int e = -1000;
    for (int k = 1; k <= deg; k++) {
        double r = fabs(p.c[deg - k] / p.c[deg]);
        if (k == deg) r *= 0.5;
        if (!(r > 0.0)) continue;
        int ex;
        frexp(r, &ex);  // r < 2^ex
        const int ek = ex >= 0 ? (ex + k - 1) / k : -((-ex) / k);  // ceil(ex / k)
        if (ek > e) e = ek;
    }
    return e == -1000 ? 1.0 : ldexp(2.0, e);
}

// Real roots of p (ascending) into out; returns their number.  The k-th
// derivatives are formed first; the roots of each bracket those of the one
// below it, from the linear derivative down to p itself (derivatives only
// to a loose tolerance: they only bracket).
RF_HD inline int real_roots(Poly1 p, double* out) {
    double mx = 0.0;
    for (int i = 0; i < p.n; i++) mx = fabs(p.c[i]) > mx ? fabs(p.c[i]) : mx;
    while (p.n > 1 && fabs(p.c[p.n - 1]) <= 1e-14 * mx) p.n--;
    const int deg = p.n - 1;
    if (deg < 1) return 0;
    Poly1 d[10];  // d[k]: the k-th derivative
    d[0] = p;
    for (int k = 1; k < deg; k++) {
        d[k] = Poly1{};
        d[k].n = d[k - 1].n - 1;
        for (int i = 1; i < d[k - 1].n; i++) d[k].c[i - 1] = i * d[k - 1].c[i];
    }
    double roots[10];
    int nr = 1;
    roots[0] = -d[deg - 1].c[0] / d[deg - 1].c[1];  // the linear one
    for (int k = deg - 2; k >= 0; k--) {
        const Poly1& q = d[k];
        const double bound = root_bound(q);
        double pts[12];
        int np = 0;
        pts[np++] = -bound;
        for (int i = 0; i < nr; i++)
            if (roots[i] > -bound && roots[i] < bound && roots[i] > pts[np - 1]) pts[np++] = roots[i];
        pts[np++] = bound;
        const double rel = k == 0 ? 1e-15 : 1e-9;
        // q at every bracket point; a point where q is within its rounding
        // error (a root of even multiplicity sits at a root of q') is a root
        double fv[12];
        bool zero[12];
        for (int i = 0; i < np; i++) {
            double df, mag;
            peval_d(q, pts[i], fv[i], df, mag);
            zero[i] = fabs(fv[i]) <= 2.5e-16 * mag;
        }
        // at most deg(q) <= 10 roots are kept, which bounds every array here
        const int cap = q.n - 1;
        int n = 0;
        double found[10];
        for (int i = 0; i < np && n < cap; i++) {
            if (zero[i]) {
                found[n++] = pts[i];
                continue;
            }
            if (i + 1 < np && !zero[i + 1] && (fv[i] < 0) != (fv[i + 1] < 0))
                found[n++] = bracket_root(q, pts[i], pts[i + 1], fv[i] < 0, rel);
        }
        nr = n;
        for (int i = 0; i < n; i++) roots[i] = found[i];
    }
    for (int i = 0; i < nr; i++) out[i] = roots[i];
    return nr;
}

RF_HD inline void cross3(const double* a, const double* b, double* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

// x0, x1: five normalized image points each ([5][2]); writes up to 10
// essential matrices (row-major, unit Frobenius norm) with x1^T E x0 = 0
// and returns their number.
RF_HD inline int five_point(const double* x0, const double* x1, double* Es) {
    // epipolar rows: x1^T E x0 = sum_ij E_ij x1_i x0_j, as the columns of Q^T
    double A[9][5];
    for (int k = 0; k < 5; k++) {
        const double a[3] = {x0[2 * k], x0[2 * k + 1], 1.0};
        const double b[3] = {x1[2 * k], x1[2 * k + 1], 1.0};
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) A[i * 3 + j][k] = b[i] * a[j];
    }
    // null space: Householder QR of Q^T (9 x 5), Q^T = H1 ... H5 [R; 0]; the
    // last four columns of H1 ... H5 are orthogonal to every row of Q
    double hv[5][9];
    for (int k = 0; k < 5; k++) {
        double nrm = 0.0;
        for (int i = k; i < 9; i++) nrm += A[i][k] * A[i][k];
        nrm = sqrt(nrm);
        const double alpha = A[k][k] > 0 ? -nrm : nrm;
        for (int i = 0; i < 9; i++) hv[k][i] = i < k ? 0.0 : A[i][k];
        hv[k][k] -= alpha;
        double vn = 0.0;
        for (int i = k; i < 9; i++) vn += hv[k][i] * hv[k][i];
        if (vn > 0.0)
            for (int j = k; j < 5; j++) {
                double d = 0.0;
                for (int i = k; i < 9; i++) d += hv[k][i] * A[i][j];
                const double f = 2.0 * d / vn;
                for (int i = k; i < 9; i++) A[i][j] -= f * hv[k][i];
            }
        const double sv = vn > 0.0 ? sqrt(vn) : 0.0;
        for (int i = k; i < 9; i++) hv[k][i] = vn > 0.0 ? hv[k][i] / sv : 0.0;
    }
    double basis[4][9];  // X, Y, Z, W = H1 ... H5 e_(6..9)
    for (int b = 0; b < 4; b++) {
        double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        v[5 + b] = 1.0;
        for (int k = 4; k >= 0; k--) {
            double d = 0.0;
            for (int i = k; i < 9; i++) d += hv[k][i] * v[i];
            for (int i = k; i < 9; i++) v[i] -= 2.0 * d * hv[k][i];
        }
        for (int i = 0; i < 9; i++) basis[b][i] = v[i];
    }
    // E_ij = x X_ij + y Y_ij + z Z_ij + W_ij as linear polynomials
    Lin E[9];
    for (int i = 0; i < 9; i++) {
        E[i].c[0] = basis[0][i];
        E[i].c[1] = basis[1][i];
        E[i].c[2] = basis[2][i];
        E[i].c[3] = basis[3][i];
    }
    // ten cubic constraints: det(E) and 2 E E^T E - tr(E E^T) E
    double M[10][20];
    {
        const Quad m0 = lin_comb(mul(E[4], E[8]), 1.0, mul(E[5], E[7]), -1.0);
        const Quad m1 = lin_comb(mul(E[3], E[8]), 1.0, mul(E[5], E[6]), -1.0);
        const Quad m2 = lin_comb(mul(E[3], E[7]), 1.0, mul(E[4], E[6]), -1.0);
        const Cub c =
            lin_comb(lin_comb(mul(m0, E[0]), 1.0, mul(m1, E[1]), -1.0), 1.0, mul(m2, E[2]), 1.0);
        for (int m = 0; m < 20; m++) M[0][m] = c.c[m];
    }
    Quad EEt[9];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            Quad q{};
            for (int k = 0; k < 3; k++) q = lin_comb(q, 1.0, mul(E[i * 3 + k], E[j * 3 + k]), 1.0);
            EEt[i * 3 + j] = q;
        }
    const Quad tr = lin_comb(lin_comb(EEt[0], 1.0, EEt[4], 1.0), 1.0, EEt[8], 1.0);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            Cub c{};
            for (int k = 0; k < 3; k++) c = lin_comb(c, 1.0, mul(EEt[i * 3 + k], E[k * 3 + j]), 1.0);
            const Cub r = lin_comb(c, 2.0, mul(tr, E[i * 3 + j]), -1.0);
            for (int m = 0; m < 20; m++) M[1 + i * 3 + j][m] = r.c[m];
        }
    // Gauss-Jordan on the first ten columns (partial pivoting)
    for (int c = 0; c < 10; c++) {
        int piv = c;
        for (int r = c + 1; r < 10; r++)
            if (fabs(M[r][c]) > fabs(M[piv][c])) piv = r;
        if (!(fabs(M[piv][c]) > 1e-300)) return 0;
        if (piv != c)
            for (int m = 0; m < 20; m++) {
                const double t = M[piv][m];
                M[piv][m] = M[c][m];
                M[c][m] = t;
            }
        const double inv = 1.0 / M[c][c];
        for (int m = 0; m < 20; m++) M[c][m] *= inv;
        for (int r = 0; r < 10; r++) {
            if (r == c || M[r][c] == 0.0) continue;
            const double f = M[r][c];
            for (int m = 0; m < 20; m++) M[r][m] -= f * M[c][m];
        }
    }
    // rows e..j (4..9) lead with x^2z, x^2, y^2z, y^2, xyz, xy; each remainder
    // is x (B10 z^2 + B11 z + B12) + y (B13 z^2 + B14 z + B15)
    //    + B16 z^3 + B17 z^2 + B18 z + B19
    Poly1 B[3][3];
    for (int q = 0; q < 3; q++) {
        const int a = 4 + 2 * q, b = a + 1;  // <k> = <e> - z<f>, <l> = <g> - z<h>, <m> = <i> - z<j>
        B[q][0] = padd(poly3(M[a][12], M[a][11], M[a][10]),
                       pshift(poly3(M[b][12], M[b][11], M[b][10])), -1.0);
        B[q][1] = padd(poly3(M[a][15], M[a][14], M[a][13]),
                       pshift(poly3(M[b][15], M[b][14], M[b][13])), -1.0);
        B[q][2] = padd(poly4(M[a][19], M[a][18], M[a][17], M[a][16]),
                       pshift(poly4(M[b][19], M[b][18], M[b][17], M[b][16])), -1.0);
    }
    const Poly1 c0 = padd(pmul(B[1][1], B[2][2]), pmul(B[1][2], B[2][1]), -1.0);
    const Poly1 c1 = padd(pmul(B[1][0], B[2][2]), pmul(B[1][2], B[2][0]), -1.0);
    const Poly1 c2 = padd(pmul(B[1][0], B[2][1]), pmul(B[1][1], B[2][0]), -1.0);
    const Poly1 det = padd(padd(pmul(B[0][0], c0), pmul(B[0][1], c1), -1.0), pmul(B[0][2], c2), 1.0);
    double zs[10];
    const int nz = real_roots(det, zs);
    int count = 0;
    for (int zi = 0; zi < nz; zi++) {
        const double z = zs[zi];
        double Bz[3][3];
        for (int q = 0; q < 3; q++)
            for (int c = 0; c < 3; c++) Bz[q][c] = peval(B[q][c], z);
        // null vector of B(z): the largest cross product of two of its rows
        double best[3] = {0, 0, 0}, bn = -1.0;
        const int rp[3][2] = {{0, 1}, {0, 2}, {1, 2}};
        for (int k = 0; k < 3; k++) {
            double c[3];
            cross3(Bz[rp[k][0]], Bz[rp[k][1]], c);
            const double nn = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
            if (nn > bn) {
                bn = nn;
                best[0] = c[0];
                best[1] = c[1];
                best[2] = c[2];
            }
        }
        if (!(fabs(best[2]) > 1e-300)) continue;
        const double x = best[0] / best[2], y = best[1] / best[2];
        double Em[9], nrm = 0.0;
        for (int i = 0; i < 9; i++) {
            Em[i] = x * basis[0][i] + y * basis[1][i] + z * basis[2][i] + basis[3][i];
            nrm += Em[i] * Em[i];
        }
        nrm = sqrt(nrm);
        if (!(nrm > 0.0) || !(nrm < INFINITY)) continue;
        for (int i = 0; i < 9; i++) Es[count * 9 + i] = Em[i] / nrm;
        if (++count == 10) break;
    }
    return count;
}

}  // namespace rf_fivept
