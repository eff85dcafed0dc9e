// D-step streaming transforms and row transforms (dstream.cuh) for Lg = 32 x 29 and 16 x P, P = 31, 33, 27.
#include "dstream.cuh"

namespace dstream {

const Variant* variants_1(int* n) {
    static const Variant v[] = {
        DSTREAM_VARIANT(32, 29),
        DSTREAM_VARIANT(16, 31),
        DSTREAM_VARIANT(16, 33),
        DSTREAM_VARIANT(16, 27),
    };
    *n = (int)(sizeof(v) / sizeof(v[0]));
    return v;
}

}  // namespace dstream
