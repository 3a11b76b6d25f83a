// dev_noalloc.cu -- exact FP64 top-k with no device allocation.
//
// Some callers cannot call cudaMalloc: code that runs where the process's
// allocator is off limits (an allocator hook or memory pool that owns every
// device byte, a real-time path that must not block on the driver's
// allocation lock, or a host that has already handed all free HBM to another
// component).  For them this file gives one variant of the plain FP64 search
// whose per-call scratch -- the padded query rows, their norms and the
// scan's partial top-k lists -- lives in a file-scope __device__ array of
// fixed size instead of the store's cudaMalloc'd scratch.  The store itself
// (built by vector_db_* / svdb_insert_batch) and the caller's query and
// result buffers are the only other device memory it touches.
//
// The array is kNoAllocScratchBytes on every GPU that loads this library, and
// it stays allocated until the process exits.  Every call shares it, and it
// keeps the last call's contents; nothing in it needs to start at zero (every
// byte a call reads was written earlier in the same call).  Two calls whose
// work overlaps on the GPU -- on different streams, or from two stores --
// race on the array; callers must order them.
//
// Loading.  With CUDA's lazy module loading, the code module holding the
// array (and so the array itself) is loaded, and its memory allocated, by the
// first use of anything in this file.  The store's own device set-up (its
// first device allocation, Store::ensure) calls noalloc_setup(), so by the
// time a store can be searched the array exists and its device address is
// known: the entry point then only reads that address.  The kernels it
// launches live in other modules (the FP64 scan's); their code is loaded by
// their first launch in the process, which the regular search's first call
// also does.  So the first search of any kind on a device may still allocate
// for module code; every later no-allocation call allocates nothing.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstring>
#include <mutex>

#include "dev_search.cuh"

namespace svdb {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;  // 16 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
struct ScratchSlot {
    unsigned long long ctx_id;  // the context the address belongs to (0: none yet)
    void* addr;
};
ScratchSlot g_slot[kMaxDevices] = {};
PFN_cuCtxGetCurrent_v4000 g_ctx_current = nullptr;
PFN_cuCtxGetId_v12000 g_ctx_id = nullptr;

// Unique id of the calling thread's current context (never reused within the
// process), so an address cached for a context that was torn down and created
// again (cudaDeviceReset, a reset primary context) is looked up afresh.
int current_context_id(unsigned long long* id) {
    if (!g_ctx_current || !g_ctx_id) {
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaDriverEntryPointQueryResult q1, q2;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 4000, cudaEnableDefault, &q1) != cudaSuccess ||
            q1 != cudaDriverEntryPointSuccess || !f1 ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
            q2 != cudaDriverEntryPointSuccess || !f2) {
            cudaGetLastError();
            svdb_set_error("search_noalloc: cuCtxGetCurrent / cuCtxGetId are not available from the driver");
            return SVDB_ECUDA;
        }
        g_ctx_current = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(f1);
        g_ctx_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(f2);
    }
    CUcontext ctx = nullptr;
    if (g_ctx_current(&ctx) != CUDA_SUCCESS || !ctx || g_ctx_id(ctx, id) != CUDA_SUCCESS) {
        svdb_set_error("search_noalloc: no current CUDA context");
        return SVDB_ECUDA;
    }
    return SVDB_OK;
}

}  // namespace

// Host code cannot use g_noalloc_scratch directly: its name stands for a host
// shadow, not a device address.  Look the device address up once per device
// (and context), with that device current.  Called by the store's device
// set-up, and by the entry point (which finds the address already known
// unless the context changed since).
int noalloc_setup(void** out) {
    int dev = 0;
    SVDB_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        svdb_set_error("search_noalloc: device ordinal %d out of range", dev);
        return SVDB_EINVAL;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    unsigned long long id = 0;
    int rc = current_context_id(&id);
    if (rc) return rc;
    if (g_slot[dev].ctx_id != id || !g_slot[dev].addr) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            svdb_set_error("search_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            return SVDB_ECUDA;
        }
        g_slot[dev].addr = p;
        g_slot[dev].ctx_id = id;
    }
    if (out) *out = g_slot[dev].addr;
    return SVDB_OK;
}

namespace {

__global__ void k_noalloc_fill_empty(int64_t* ids, double* dists, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        ids[i] = -1;
        dists[i] = __longlong_as_double(0x7ff8000000000000ll);
    }
}

}  // namespace

size_t noalloc_scratch_limit() { return kNoAllocScratchBytes; }

}  // namespace svdb

using namespace svdb;

extern "C" int svdbd_search_noalloc(svdbd_store* hs, const double* d_queries, size_t nq, size_t k, int metric,
                                    int64_t* d_ids, double* d_dists) {
    Store* s = reinterpret_cast<Store*>(hs);
    if (k == 0 || k > 128 || metric < 0 || metric > 2 || (nq && (!d_queries || !d_ids || !d_dists))) {
        svdb_set_error("search_noalloc: bad argument (k=%zu metric=%d; k must be 1..128)", k, metric);
        return SVDB_EINVAL;
    }
    if (nq == 0) return SVDB_OK;
    // syncing the store could allocate: the caller syncs it beforehand
    if (!s->stream || s->stage_rows || s->derive_lo >= 0 || !s->dirty_list.empty() || s->map_dirty) {
        svdb_set_error("search_noalloc: the store has changes not yet on the device; call svdb_sync first");
        return SVDB_EINVAL;
    }
    // bound nq before any size arithmetic, so no product below can wrap
    if (s->ld == 0 || nq > kNoAllocScratchBytes / (s->ld * sizeof(double))) {
        svdb_set_error(
            "search_noalloc: %zu queries at dimension %zu do not fit the fixed %zu-byte scratch array (use fewer "
            "queries per call)",
            nq, s->dim, kNoAllocScratchBytes);
        return SVDB_EINVAL;
    }
    const size_t qbytes = round_up(nq * s->ld * sizeof(double), 256);
    const size_t sqbytes = round_up(nq * sizeof(double), 256);
    const size_t kbytes = s->nlive ? search_fp64_scratch(s, nq, k) : 0;
    const size_t need = qbytes + sqbytes + kbytes;
    if (need > kNoAllocScratchBytes) {
        svdb_set_error(
            "search_noalloc: %zu queries x top-%zu at dimension %zu need %zu bytes of scratch; the fixed array "
            "holds %zu (use fewer queries per call)",
            nq, k, s->dim, need, kNoAllocScratchBytes);
        return SVDB_EINVAL;
    }
    void* base = nullptr;
    int rc = noalloc_setup(&base);
    if (rc) return rc;
    unsigned char* b = reinterpret_cast<unsigned char*>(base);
    double* qbuf = reinterpret_cast<double*>(b);
    double* qsq = reinterpret_cast<double*>(b + qbytes);
    rc = prep_queries_fp64(s, d_queries, s->dim, nq, qbuf, qsq);
    if (rc) return rc;
    if (s->nlive == 0) {
        k_noalloc_fill_empty<<<(unsigned)((nq * k + 255) / 256), 256, 0, s->stream>>>(d_ids, d_dists, nq * k);
        SVDB_LAUNCH_CHECK();
        return SVDB_OK;
    }
    SearchArgs a;
    a.q = qbuf;
    a.qsq = qsq;
    a.nq = nq;
    a.k = k;
    a.metric = metric;
    a.ids = d_ids;
    a.dists = d_dists;
    a.err = nullptr;
    return search_fp64(s, a, b + qbytes + sqbytes, kbytes, nullptr, false);
}
