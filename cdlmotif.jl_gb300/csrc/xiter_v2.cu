// Multi-iteration X-step kernels (xiter.cuh) for Lg = 16 x P, P = 31, 33, 27.
#include "xiter.cuh"

namespace xiter {

const Variant* variants_2(int* n) {
    static const Variant v[] = {
        XITER_VARIANT(16, 31, 160, 2, 16),
        XITER_VARIANT(16, 33, 160, 2, 16),
        XITER_VARIANT(16, 27, 160, 2, 16),
    };
    *n = (int)(sizeof(v) / sizeof(v[0]));
    return v;
}

}  // namespace xiter
