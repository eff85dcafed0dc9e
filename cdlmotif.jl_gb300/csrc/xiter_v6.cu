// Multi-iteration X-step kernels (xiter.cuh) for Lg = 16 x P with the even per-lane
// lengths P = 26, 28, 30 (Lg = 416, 448, 480).
#include "xiter.cuh"

namespace xiter {

const Variant* variants_6(int* n) {
    static const Variant v[] = {
        XITER_VARIANT(16, 26, 160, 2, 16),
        XITER_VARIANT(16, 28, 160, 2, 16),
        XITER_VARIANT(16, 30, 160, 2, 16),
    };
    *n = (int)(sizeof(v) / sizeof(v[0]));
    return v;
}

}  // namespace xiter
