// Multi-iteration X-step kernels (xiter.cuh) for Lg = 32 x P with the even per-lane
// lengths P = 26, 28, 30 (Lg = 832: L = 200 at W = 4; 896: L = 200 at W = 12; 960).
#include "xiter.cuh"

namespace xiter {

const Variant* variants_5(int* n) {
    static const Variant v[] = {
        XITER_VARIANT(32, 26, 288, 1, 16),
        XITER_VARIANT(32, 28, 288, 1, 16),
        XITER_VARIANT(32, 30, 288, 1, 16),
    };
    *n = (int)(sizeof(v) / sizeof(v[0]));
    return v;
}

}  // namespace xiter
