// Reads polynomials from stdin (a line "n c0 c1 ... c(n-1)", coefficient k
// of z^k) and prints the real roots rf_fivept::real_roots finds, one line
// per polynomial ("count r0 r1 ..."), for the root-finder test.
#include <cstdio>

#include "rf_fivept.cuh"

int main() {
    int n;
    while (std::scanf("%d", &n) == 1) {
        if (n < 1 || n > 11) return 2;
        rf_fivept::Poly1 p{};
        p.n = n;
        for (int i = 0; i < n; i++)
            if (std::scanf("%lf", &p.c[i]) != 1) return 2;
        double r[10];
        const int k = rf_fivept::real_roots(p, r);
        std::printf("%d", k);
        for (int i = 0; i < k; i++) std::printf(" %.17g", r[i]);
        std::printf("\n");
    }
    return 0;
}
