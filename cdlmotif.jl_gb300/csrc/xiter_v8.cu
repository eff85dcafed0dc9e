// Multi-iteration X-step kernels (xiter.cuh) for Lg = 16 x P, P = 18, 20, 22, 24
// (Lg = 288, 320, 352, 384).
#include "xiter.cuh"

namespace xiter {

const Variant* variants_8(int* n) {
    static const Variant v[] = {
        XITER_VARIANT(16, 18, 160, 2, 16),
        XITER_VARIANT(16, 20, 160, 2, 16),
        XITER_VARIANT(16, 22, 160, 2, 16),
        XITER_VARIANT(16, 24, 160, 2, 16),
    };
    *n = (int)(sizeof(v) / sizeof(v[0]));
    return v;
}

}  // namespace xiter
