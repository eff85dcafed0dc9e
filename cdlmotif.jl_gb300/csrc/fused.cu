// Fused X-step / D-step kernels with in-kernel FFTs (filled in below).
#include "cdlgb_internal.h"

int fused_supported(int Lg, int M) { (void)Lg; (void)M; return 0; }
int fused_setup(cdlgb_ctx* c) { (void)c; return CDLGB_OK; }
void fused_free(cdlgb_ctx* c) { (void)c; }
int fused_xstep(cdlgb_ctx* c, const float*, float*, int) {
    return cdlgb_seterr(c, CDLGB_ENOTSUP, "fused path not built");
}
int fused_dstep(cdlgb_ctx* c) { return cdlgb_seterr(c, CDLGB_ENOTSUP, "fused path not built"); }
size_t fused_scratch_bytes(int, int, int) { return 0; }
