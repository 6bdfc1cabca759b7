// Reads matrices "n a00 a01 ..." (row-major) from stdin, one per line, and prints
// the eigenvalues then the eigenvector matrix (row-major) from symmetric_eigh.
#include <cstdio>
#include <vector>

#include "../../ciflow_gb300/csrc/small_eigh.h"

int main() {
    int n;
    while (std::scanf("%d", &n) == 1) {
        std::vector<double> a((size_t)n * n), w, z;
        for (auto &x : a)
            if (std::scanf("%lf", &x) != 1) return 1;
        cigpu::symmetric_eigh(n, a, w, z);
        for (double x : w) std::printf("%.17g ", x);
        std::printf("\n");
        for (double x : z) std::printf("%.17g ", x);
        std::printf("\n");
    }
    return 0;
}
