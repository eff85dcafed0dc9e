// Multi-iteration X-step kernels (xiter.cuh) for Lg = 32 x P, P = 18, 20, 22, 24
// (Lg = 576, 640, 704, 768), and 16 x P, P = 23, 29 (Lg = 368, 464).
#include "xiter.cuh"

namespace xiter {

const Variant* variants_7(int* n) {
    static const Variant v[] = {
        XITER_VARIANT(32, 18, 288, 1, 16),
        XITER_VARIANT(32, 20, 288, 1, 16),
        XITER_VARIANT(32, 22, 288, 1, 16),
        XITER_VARIANT(32, 24, 288, 1, 16),
        XITER_VARIANT(16, 23, 160, 2, 16),
        XITER_VARIANT(16, 29, 160, 2, 16),
    };
    *n = (int)(sizeof(v) / sizeof(v[0]));
    return v;
}

}  // namespace xiter
