// Multi-iteration X-step kernels (xiter.cuh) for Lg = 32 x P, P = 17, 19, 23, 31.
#include "xiter.cuh"

namespace xiter {

const Variant* variants_3(int* n) {
    static const Variant v[] = {
        XITER_VARIANT(32, 17, 288, 1, 16),
        XITER_VARIANT(32, 19, 288, 1, 16),
        XITER_VARIANT(32, 23, 288, 1, 16),
        XITER_VARIANT(32, 31, 288, 1, 16),
    };
    *n = (int)(sizeof(v) / sizeof(v[0]));
    return v;
}

}  // namespace xiter
