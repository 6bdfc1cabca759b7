// Prints d_binom(n, k) for 0 <= k <= n <= 130 and space_dim for a few spaces, one
// value per line, for tests/test_binom_cpu.py to compare with exact integers.
#include <cstdio>

#include "../../ciflow_gb300/csrc/build.cuh"

int main() {
    for (int n = 0; n <= 130; ++n)
        for (int k = 0; k <= n; ++k) std::printf("b %d %d %lld\n", n, k, (long long)cigpu::d_binom(n, k));
    const int cases[][4] = {{0, 12, 6, 6}, {1, 24, 12, 12}, {0, 63, 31, 31}, {0, 64, 32, 32},
                            {0, 128, 64, 64}, {1, 128, 64, 64}, {0, 10, 11, 2}, {0, 10, -1, 2}};
    for (auto &c : cases)
        std::printf("d %d %d %d %d %lld\n", c[0], c[1], c[2], c[3], (long long)cigpu::space_dim(c[0], c[1], c[2], c[3]));
    return 0;
}
