// Host test of the checked build's predicates and error-word records (checked.cuh):
// prints one line per case for tests/test_checked_cpu.py.
#include <cstdio>

#include "../../ciflow_gb300/csrc/checked.cuh"

int main() {
    using namespace cigpu;
    const unsigned long long idx[] = {0ull, 1ull, 123456789ull, (1ull << 56) - 1, (1ull << 56), ~0ull};
    for (unsigned code = 1; code <= 6; ++code)
        for (unsigned long long i : idx) {
            const uint64_t w = check_record(code, i);
            std::printf("rec %u %llu %u %llu\n", code, i, check_record_code(w), (unsigned long long)check_record_index(w));
        }
    const unsigned long long iv[][2] = {{0, 1}, {0, 0}, {5, 5}, {4, 5}, {~0ull, 5}, {4294967295ull, 4294967295ull}};
    for (auto &c : iv) std::printf("idx %llu %llu %d\n", c[0], c[1], (int)index_ok(c[0], c[1]));
    const long long rv[][3] = {{0, 0, 1}, {0, 5, 5}, {0, 6, 5}, {3, 2, 10}, {-1, 2, 10}, {7, 9, 2}, {7, 9, 1}};
    for (auto &c : rv) std::printf("row %lld %lld %lld %d\n", c[0], c[1], c[2], (int)row_ok(c[0], c[1], c[2]));
    return 0;
}
