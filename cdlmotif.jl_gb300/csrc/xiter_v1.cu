// Multi-iteration X-step kernels (xiter.cuh) for the L = 200, W = 16 length
// (Lg = 32 x 29), at 16 and at 8 filters per CTA.
#include "xiter.cuh"

namespace xiter {

const Variant* variants_1(int* n) {
    static const Variant v[] = {
        XITER_VARIANT(32, 29, 288, 1, 16),
        XITER_VARIANT(32, 29, 160, 2, 8),
    };
    *n = (int)(sizeof(v) / sizeof(v[0]));
    return v;
}

}  // namespace xiter
