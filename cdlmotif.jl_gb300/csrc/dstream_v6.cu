// D-step streaming transforms and row transforms (dstream.cuh) for Lg = 16 x P,
// P = 18, 20, 22, 24.
#include "dstream.cuh"

namespace dstream {

const Variant* variants_6(int* n) {
    static const Variant v[] = {
        DSTREAM_VARIANT(16, 18),
        DSTREAM_VARIANT(16, 20),
        DSTREAM_VARIANT(16, 22),
        DSTREAM_VARIANT(16, 24),
    };
    *n = (int)(sizeof(v) / sizeof(v[0]));
    return v;
}

}  // namespace dstream
