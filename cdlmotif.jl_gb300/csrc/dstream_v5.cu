// D-step streaming transforms and row transforms (dstream.cuh) for Lg = 32 x P,
// P = 18, 20, 22, 24, and 16 x P, P = 23, 29.
#include "dstream.cuh"

namespace dstream {

const Variant* variants_5(int* n) {
    static const Variant v[] = {
        DSTREAM_VARIANT(32, 18),
        DSTREAM_VARIANT(32, 20),
        DSTREAM_VARIANT(32, 22),
        DSTREAM_VARIANT(32, 24),
        DSTREAM_VARIANT(16, 23),
        DSTREAM_VARIANT(16, 29),
    };
    *n = (int)(sizeof(v) / sizeof(v[0]));
    return v;
}

}  // namespace dstream
