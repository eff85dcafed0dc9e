// D-step streaming transforms and row transforms (dstream.cuh) for Lg = 32 x P, P = 17, 19, 23, 31.
#include "dstream.cuh"

namespace dstream {

const Variant* variants_2(int* n) {
    static const Variant v[] = {
        DSTREAM_VARIANT(32, 17),
        DSTREAM_VARIANT(32, 19),
        DSTREAM_VARIANT(32, 23),
        DSTREAM_VARIANT(32, 31),
    };
    *n = (int)(sizeof(v) / sizeof(v[0]));
    return v;
}

}  // namespace dstream
