// Multi-iteration X-step kernels (xiter.cuh) for Lg = 16 x P, P = 21, 25, and 32 x P, P = 21, 25, 27.
#include "xiter.cuh"

namespace xiter {

const Variant* variants_4(int* n) {
    static const Variant v[] = {
        XITER_VARIANT(16, 21, 160, 2, 16),
        XITER_VARIANT(16, 25, 160, 2, 16),
        XITER_VARIANT(32, 21, 288, 1, 16),
        XITER_VARIANT(32, 25, 288, 1, 16),
        XITER_VARIANT(32, 27, 288, 1, 16),
    };
    *n = (int)(sizeof(v) / sizeof(v[0]));
    return v;
}

}  // namespace xiter
