// first_bad_position (cdlgb_internal.h), the host-side check of the count, extension and
// rescore calls, against the conditions it replaces, written per entry: a window
// pos..pos + lens[k] - 1 (1-based, 0 = no entry) must lie in 1..L; without lens a
// position must lie in 0..L.  Random cases with negative, zero, in-range and
// out-of-range entries; prints "ok" or the first mismatch and exits non-zero.
#include <cstdio>
#include <cstdint>
#include <random>
#include <vector>

#include "cdlgb_internal.h"

int main() {
    std::mt19937 g(12345);
    for (int trial = 0; trial < 5000; ++trial) {
        const int K = 1 + (int)(g() % 9), N = 1 + (int)(g() % 12), L = 1 + (int)(g() % 40);
        std::vector<int32_t> lens(K), pos((size_t)K * N);
        for (auto& l : lens) l = 1 + (int)(g() % 50);
        for (auto& p : pos) {
            const int r = (int)(g() % 10);
            p = r == 0 ? -(int)(g() % 3) : r < 4 ? 0 : (int)(g() % (unsigned)(L + 4));
        }
        for (int mode = 0; mode < 2; ++mode) {
            long long want = -1;
            for (size_t i = 0; i < pos.size() && want < 0; ++i) {
                const int p = pos[i], k = (int)(i % K);
                const bool bad = mode == 0 ? (p < 0 || (p > 0 && p - 1 + lens[k] > L)) : (p < 0 || p > L);
                if (bad) want = (long long)i;
            }
            const long long got = first_bad_position(pos.data(), mode == 0 ? lens.data() : nullptr, K,
                                                     (size_t)N, L);
            if (got != want) {
                std::printf("mismatch: trial %d mode %d: %lld, expected %lld\n", trial, mode, got, want);
                return 1;
            }
        }
    }
    std::printf("ok\n");
    return 0;
}
