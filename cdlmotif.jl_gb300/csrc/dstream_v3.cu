// D-step streaming transforms and row transforms (dstream.cuh) for Lg = 16 x P, P = 21, 25, and 32 x P, P = 21, 25, 27.
#include "dstream.cuh"

namespace dstream {

const Variant* variants_3(int* n) {
    static const Variant v[] = {
        DSTREAM_VARIANT(16, 21),
        DSTREAM_VARIANT(16, 25),
        DSTREAM_VARIANT(32, 21),
        DSTREAM_VARIANT(32, 25),
        DSTREAM_VARIANT(32, 27),
    };
    *n = (int)(sizeof(v) / sizeof(v[0]));
    return v;
}

}  // namespace dstream
