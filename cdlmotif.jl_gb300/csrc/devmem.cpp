// Device memory of the contexts: stream-ordered allocations from a memory pool the
// library owns on each device, and the pinned host scalars from one shared slab.
//
// cudaMalloc, cudaFree and cudaMallocHost synchronise with the work of every stream on
// the device, so a context that is created, loaded or destroyed while another context
// trains stalls that training; the training server runs up to 64 contexts at once and
// creates and destroys one per dataset.  A context therefore allocates every buffer
// with cudaMallocFromPoolAsync on its own stream and frees it with cudaFreeAsync there,
// which orders the allocation with that stream's work only.  The pool reuses a block
// only once its free has completed on the device (no dependency between streams is ever
// added for reuse).  While no server holds the pool, what is freed goes back to the
// device at the next synchronisation, as after cudaFree; a server raises the pool's
// release threshold for its lifetime so that the blocks of finished datasets are
// reused by the next ones without being mapped again.
#include "cdlgb_internal.h"

#include <mutex>
#include <vector>

namespace {

constexpr int kMaxDev = 64;
std::mutex g_mu;
cudaMemPool_t g_pool[kMaxDev] = {};
int g_hold[kMaxDev] = {};

// 4096 slots of 8 doubles, allocated at the first request
constexpr int kSlots = 4096;
constexpr int kSlotDoubles = 8;
double* g_slab = nullptr;
std::vector<int> g_free;

cudaError_t pool_for(int dev, cudaMemPool_t* out) {
    if (dev < 0 || dev >= kMaxDev) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_pool[dev]) {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.handleTypes = cudaMemHandleTypeNone;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t p = nullptr;
        cudaError_t e = cudaMemPoolCreate(&p, &props);
        if (e != cudaSuccess) return e;
        int no = 0;
        e = cudaMemPoolSetAttribute(p, cudaMemPoolReuseAllowInternalDependencies, &no);
        if (e != cudaSuccess) {
            cudaMemPoolDestroy(p);
            return e;
        }
        g_pool[dev] = p;
    }
    *out = g_pool[dev];
    return cudaSuccess;
}

}  // namespace

cudaError_t dev_malloc(cdlgb_ctx* c, void** p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) return cudaSuccess;
    cudaMemPool_t pool = nullptr;
    cudaError_t e = pool_for(c->dev, &pool);
    if (e == cudaSuccess) e = cudaMallocFromPoolAsync(p, bytes, pool, c->stream);
    return e;
}

cudaError_t dev_copy_in(cdlgb_ctx* c, void** p, const void* host, size_t bytes) {
    cudaError_t e = dev_malloc(c, p, bytes);
    // a pageable source: the call returns once the bytes are staged
    if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(*p, host, bytes, cudaMemcpyHostToDevice, c->stream);
    return e;
}

int dev_alloc(cdlgb_ctx* c, void** p, size_t bytes) {
    CU_TRY(c, dev_malloc(c, p, bytes));
    return CDLGB_OK;
}

void dev_free(cdlgb_ctx* c, void* p) {
    if (p) cudaFreeAsync(p, c->stream);
}

size_t devmem_reusable(int dev) {
    cudaMemPool_t pool = nullptr;
    if (pool_for(dev, &pool) != cudaSuccess) return 0;
    uint64_t reserved = 0, used = 0;
    if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved) != cudaSuccess ||
        cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used) != cudaSuccess)
        return 0;
    return reserved > used ? (size_t)(reserved - used) : 0;
}

int devmem_hold(int dev, int delta) {
    cudaMemPool_t pool = nullptr;
    if (pool_for(dev, &pool) != cudaSuccess) return CDLGB_ECUDA;
    std::lock_guard<std::mutex> lk(g_mu);
    const int before = g_hold[dev];
    g_hold[dev] = before + delta < 0 ? 0 : before + delta;
    uint64_t thr = g_hold[dev] > 0 ? ~(uint64_t)0 : 0;
    if ((before > 0) == (g_hold[dev] > 0)) return CDLGB_OK;
    if (cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr) != cudaSuccess)
        return CDLGB_ECUDA;
    if (g_hold[dev] == 0) cudaMemPoolTrimTo(pool, 0);
    return CDLGB_OK;
}

double* host_scalars_get() {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_slab) {
        double* s = nullptr;
        if (cudaHostAlloc((void**)&s, (size_t)kSlots * kSlotDoubles * sizeof(double),
                          cudaHostAllocPortable) != cudaSuccess)
            return nullptr;
        g_slab = s;
        g_free.reserve(kSlots);
        for (int i = kSlots - 1; i >= 0; --i) g_free.push_back(i);
    }
    if (g_free.empty()) return nullptr;
    const int i = g_free.back();
    g_free.pop_back();
    return g_slab + (size_t)i * kSlotDoubles;
}

void host_scalars_put(double* p) {
    if (!p) return;
    std::lock_guard<std::mutex> lk(g_mu);
    if (g_slab && p >= g_slab && p < g_slab + (size_t)kSlots * kSlotDoubles)
        g_free.push_back((int)((p - g_slab) / kSlotDoubles));
}
