// D-step streaming transforms and row transforms (dstream.cuh) for the even per-lane
// lengths: Lg = 32 x P and 16 x P, P = 26, 28, 30.
#include "dstream.cuh"

namespace dstream {

const Variant* variants_4(int* n) {
    static const Variant v[] = {
        DSTREAM_VARIANT(32, 26),
        DSTREAM_VARIANT(32, 28),
        DSTREAM_VARIANT(32, 30),
        DSTREAM_VARIANT(16, 26),
        DSTREAM_VARIANT(16, 28),
        DSTREAM_VARIANT(16, 30),
    };
    *n = (int)(sizeof(v) / sizeof(v[0]));
    return v;
}

}  // namespace dstream
