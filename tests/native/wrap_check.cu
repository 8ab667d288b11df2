// Host check of the REPEAT texel-index wrap of the atlas lookups
// (wrap_repeat in vulkanexp_gb300/csrc/common.cuh): for every axis length n
// in 1..64 and every index in a wide window around [0, n), plus indices
// near the int range ends and large axes, the result equals the remainder
// form ((i % n) + n) % n (taken in 64 bits here) that the bilinear fetch
// used before.
#include <climits>
#include <cstdio>

#include "../../vulkanexp_gb300/csrc/common.cuh"

int main() {
    long long checked = 0;
    int failures = 0;
    auto one = [&](int i, int n) {
        const int want = (int)((((long long)i % n) + n) % n);
        const int got = ddgi::wrap_repeat(i, n);
        ++checked;
        if (got != want && failures++ < 10) std::printf("FAIL: i %d n %d got %d want %d\n", i, n, got, want);
    };
    for (int n = 1; n <= 64; ++n) {
        for (int i = -5 * n - 3; i <= 6 * n + 3; ++i) one(i, n);
        for (int k = 0; k < 4; ++k) {
            one(INT_MAX - k, n);
            one(INT_MIN + k, n);
        }
    }
    for (int n : {4096, 8192, 12288, 1 << 20, INT_MAX / 2, INT_MAX}) {
        for (long long i : {-(long long)n - 1, -(long long)n, -(long long)n + 1, -1LL, 0LL, 1LL, (long long)n - 1,
                            (long long)n, (long long)n + 1, 2LL * n - 1, 2LL * n, (long long)INT_MAX,
                            (long long)INT_MIN, (long long)INT_MIN + 1})
            if (i >= INT_MIN && i <= INT_MAX) one((int)i, n);
    }
    std::printf("%lld indices checked\n", checked);
    if (failures) return 1;
    std::printf("all ok\n");
    return 0;
}
