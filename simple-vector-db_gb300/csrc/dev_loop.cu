// dev_loop.cu -- the server's request path as a device-side loop.
//
// The reference answers each request on its own host thread: /compare reads
// two rows and runs a float-accumulating metric (src/compare_handler.c:86-
// 185), POST /nearest walks the insertion-order KD tree (:403), POST / PUT /
// DELETE /vector append, overwrite or delete a row with positional indices
// (src/post_handler.c:333, src/put_handler.c:155,247,
// src/delete_handler.c:84,96; src/vector_database.c:81-195).  Here one
// persistent kernel (one CTA of 256 threads) owns the store and serves these
// requests as they arrive:
//
//   - Requests sit in a ring in page-locked host memory mapped into the
//     device.  A host thread claims a ticket, writes its request (and its
//     vector) into slot ticket % ring and publishes it by writing the slot's
//     sequence number last; no CUDA call is made to submit.
//   - The loop polls the next slot with a system-scope acquire load.  When a
//     request is there it takes every request already published after it (up
//     to max_batch) as one batch and answers them in ticket order: a run of
//     reads (/compare, /nearest) is answered in parallel, one thread per
//     request, against the same store state; a mutation is applied by the
//     whole CTA (the row copied by all threads, the bookkeeping by one) before
//     the next request.  This is one serial order of the requests -- the
//     ticket order -- and every answer is the one the reference gives for
//     that order.
//   - Answers go back to mapped host memory; a counter of answered tickets is
//     written after them (system-scope fence first), and the host reads it
//     with an acquire load.
//   - Positions are the reference's (delete shifts later rows down): rows
//     live in slots that never move, a Fenwick tree over slot occupancy maps
//     a position to its slot in O(log capacity), and a delete is one
//     decrement.  The KD tree is the reference's: every insert and every
//     update adds a node (index = the position it was given), deletes leave
//     the nodes alone (src/vector_database.c:169-195).
//   - Admission by HBM: the capacity (rows and KD nodes) is allocated when the
//     loop is created; an insert beyond it is answered SVDB_ENOMEM.
//   - Every wait is bounded: polling for work gives up after idle_us with no
//     request and the kernel returns (state "left idle"); a host stop flag is
//     seen at every poll.  Before leaving idle the loop announces it and looks
//     once more, so a request published at that moment is either served or
//     seen by the host, which then launches the loop again.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "dev_common.cuh"
#include "dev_ref.cuh"

namespace svdb {
namespace {

constexpr int kLoopThreads = 256;
constexpr int kLoopMaxKd = 32;  // KD dimensions the loop's descent keeps in registers
// loop states (LoopCtl::state); 0 is "not started", set by the host only
constexpr uint32_t kStateRunning = 1, kStateLeftIdle = 2, kStateStopped = 3, kStateLeaving = 4;

// one request slot of the ring (host memory, mapped)
struct __align__(64) LoopSlot {
    uint64_t seq;       // ticket + 1 once the request is complete (written last)
    int32_t op, metric;
    uint64_t a, b;
    uint32_t has_uuid;  // INSERT / UPDATE: the request carries a uuid
    uint32_t pad0;
    uint64_t free_for;  // host only: the ticket that may use this slot next
    uint64_t pad1[2];
};
static_assert(sizeof(LoopSlot) == 64, "ring slot layout");

struct LoopResp {
    int32_t status;
    float value;
    uint64_t index;
};

// control block (host memory, mapped)
struct __align__(64) LoopCtl {
    uint64_t done;        // tickets answered (written after their answers)
    uint64_t head;        // first ticket not yet taken (kept across launches)
    uint64_t size;        // rows in the store after the last batch
    uint64_t batches;     // batches served
    uint64_t idle_exits;  // launches that ended with nothing to do
    uint32_t state;       // kState*
    uint32_t stop;        // the host asks the loop to leave
};

struct LoopDev {
    LoopSlot* ring;
    LoopResp* resp;
    const double* vecs;  // ring x dim doubles (mapped)
    const char* uuids;   // ring x 40 bytes (mapped)
    LoopCtl* ctl;
    uint64_t mask;       // ring - 1
    double* x;           // capacity x dim rows
    char* uu;            // capacity x 40 uuid bytes
    int32_t* fen;        // Fenwick over slots, fen[1..fn]
    int64_t fn;          // power of two >= capacity
    int64_t* cnt;        // {slots used, live rows, KD nodes, KD height}
    double* kpts;        // KD nodes: kd_dim coordinates each
    int64_t* kidx;       // stored index per node
    int2* kchild;        // children (-1: none)
    int2* kstack;        // per thread: kstack_h entries
    int64_t cap, kcap;
    int dim, kdim, kstack_h, max_batch;
    uint64_t idle_ns;
};

__device__ __forceinline__ uint64_t ld_acquire_sys(const uint64_t* p) {
    uint64_t v;
    asm volatile("ld.acquire.sys.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_sys(uint64_t* p, uint64_t v) {
    asm volatile("st.release.sys.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void st_release_sys32(uint32_t* p, uint32_t v) {
    asm volatile("st.release.sys.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint64_t gtime() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// position p (0-based) -> its slot: the (p+1)-th live slot
__device__ __forceinline__ int64_t fen_find(const int32_t* fen, int64_t fn, int64_t p) {
    int64_t pos = 0, rem = p + 1;
    for (int64_t step = fn; step > 0; step >>= 1)
        if (pos + step <= fn && fen[pos + step] < rem) {
            pos += step;
            rem -= fen[pos];
        }
    return pos;
}
__device__ __forceinline__ void fen_add(int32_t* fen, int64_t fn, int64_t slot, int32_t d) {
    for (int64_t i = slot + 1; i <= fn; i += i & -i) fen[i] += d;
}

// kdtree_insert (src/kdtree.c:15-62): a new node for `idx` with the first
// kdim coordinates of `row`; depth % kdim is the axis, "<" goes left
__device__ void kd_insert(const LoopDev& L, const double* row, int64_t idx) {
    const int64_t node = L.cnt[2];
    double* p = L.kpts + node * L.kdim;
    for (int i = 0; i < L.kdim; ++i) p[i] = row[i];
    L.kidx[node] = idx;
    L.kchild[node] = make_int2(-1, -1);
    int64_t depth = 1;
    if (node > 0) {
        int cur = 0;
        for (int d = 0; d < L.kcap; ++d) {  // at most one step per node: the walk always ends
            const int ax = d % L.kdim;
            int2 ch = L.kchild[cur];
            const bool left = row[ax] < L.kpts[(int64_t)cur * L.kdim + ax];
            const int nxt = left ? ch.x : ch.y;
            if (nxt < 0) {
                if (left)
                    ch.x = (int)node;
                else
                    ch.y = (int)node;
                L.kchild[cur] = ch;
                depth = d + 2;
                break;
            }
            cur = nxt;
        }
    }
    L.cnt[2] = node + 1;
    if (depth > L.cnt[3]) L.cnt[3] = depth;
}

__global__ void __launch_bounds__(kLoopThreads, 1) k_serve_loop(LoopDev L) {
    __shared__ uint64_t s_head;
    __shared__ int s_n, s_leave, s_run_end;
    __shared__ int32_t s_op[kLoopThreads];
    __shared__ int s_status;
    __shared__ int64_t s_slot, s_pos;
    const int t = threadIdx.x;
    if (t == 0) {
        s_head = *(volatile uint64_t*)&L.ctl->head;
        st_release_sys32(&L.ctl->state, kStateRunning);
    }
    __syncthreads();
    for (;;) {
        // ------------------------------------------------ wait for a request
        if (t == 0) {
            int leave = 0;
            const uint64_t h = s_head;
            const uint64_t t0 = gtime();
            for (;;) {
                // the stop flag first: a shutdown is honoured between batches even
                // while requests keep coming (they stay in the ring for a later start)
                if (*(volatile uint32_t*)&L.ctl->stop) {
                    leave = (int)kStateStopped;
                    break;
                }
                if (ld_acquire_sys(&L.ring[h & L.mask].seq) == h + 1) break;
                if (gtime() - t0 > L.idle_ns) {
                    // announce the exit, then look once more: a request published
                    // now is served here, or the host sees the state and relaunches
                    st_release_sys32(&L.ctl->state, kStateLeaving);
                    __threadfence_system();
                    if (ld_acquire_sys(&L.ring[h & L.mask].seq) == h + 1) {
                        st_release_sys32(&L.ctl->state, kStateRunning);
                        break;
                    }
                    leave = (int)kStateLeftIdle;
                    break;
                }
                __nanosleep(256);
            }
            int n = 0;
            if (!leave) {
                n = 1;
                while (n < L.max_batch && ld_acquire_sys(&L.ring[(h + n) & L.mask].seq) == h + n + 1) ++n;
            }
            s_n = n;
            s_leave = leave;
        }
        __syncthreads();
        if (s_leave) break;
        const uint64_t h = s_head;
        const int n = s_n;
        if (t < n) s_op[t] = __ldcv((const int*)&L.ring[(h + t) & L.mask].op);
        __syncthreads();
        // ------------------------------------------------ answer the batch in ticket order
        int i = 0;
        while (i < n) {
            const int op = s_op[i];
            if (op == SVDB_REQ_COMPARE || op == SVDB_REQ_KD_NEAREST || op < 0 || op > SVDB_REQ_KD_NEAREST ||
                op == SVDB_REQ_NEAREST) {
                // a run of reads (and requests this loop does not serve): in parallel
                if (t == 0) {
                    int j = i + 1;
                    while (j < n) {
                        const int o = s_op[j];
                        if (o == SVDB_REQ_INSERT || o == SVDB_REQ_UPDATE || o == SVDB_REQ_DELETE) break;
                        ++j;
                    }
                    s_run_end = j;
                }
                __syncthreads();
                const int j = s_run_end;
                for (int r = i + t; r < j; r += kLoopThreads) {
                    const uint64_t tk = h + r;
                    const LoopSlot* sl = &L.ring[tk & L.mask];
                    LoopResp out;
                    out.status = SVDB_OK;
                    out.value = __int_as_float(0x7fc00000);
                    out.index = 0;
                    const int o = s_op[r];
                    const int64_t size = L.cnt[1];
                    if (o == SVDB_REQ_COMPARE) {
                        const uint64_t a = __ldcv((const unsigned long long*)&sl->a);
                        const uint64_t b = __ldcv((const unsigned long long*)&sl->b);
                        const int m = __ldcv((const int*)&sl->metric);
                        if (a >= (uint64_t)size || b >= (uint64_t)size) {
                            out.status = SVDB_CMP_OUT_OF_BOUNDS;  // src/compare_handler.c:101
                        } else if (m < 0 || m > 2) {
                            out.status = SVDB_CMP_UNKNOWN_METHOD;  // :161
                        } else {
                            const int64_t sa = fen_find(L.fen, L.fn, (int64_t)a), sb = fen_find(L.fen, L.fn, (int64_t)b);
                            out.value = ref_metric(m, L.x + sa * L.dim, L.x + sb * L.dim, L.dim);
                        }
                    } else if (o == SVDB_REQ_KD_NEAREST) {
                        if (L.cnt[3] > L.kstack_h) {
                            out.status = SVDB_EINVAL;  // the tree is deeper than the descent's stack
                        } else {
                            double q[kLoopMaxKd];
                            const double* v = L.vecs + (tk & L.mask) * (uint64_t)L.dim;
                            for (int c = 0; c < L.kdim; ++c) q[c] = __ldcv(v + c);
                            const int64_t r64 = kd_descend(L.kpts, L.kidx, L.kchild, L.kdim, L.cnt[2], q,
                                                           L.kstack + (size_t)t * L.kstack_h);
                            out.index = (uint64_t)r64;  // -1: (size_t)-1, no neighbour
                        }
                    } else {
                        out.status = SVDB_EINVAL;  // not a request this loop serves
                    }
                    L.resp[tk & L.mask] = out;
                }
                i = j;
                __syncthreads();
                continue;
            }
            // a mutation: the whole CTA
            const uint64_t tk = h + i;
            const LoopSlot* sl = &L.ring[tk & L.mask];
            const double* v = L.vecs + (tk & L.mask) * (uint64_t)L.dim;
            if (t == 0) {
                int st = SVDB_OK;
                int64_t slot = -1, pos = -1;
                const int64_t size = L.cnt[1];
                if (op == SVDB_REQ_INSERT) {
                    if (L.cnt[0] >= L.cap || L.cnt[2] >= L.kcap) {
                        st = SVDB_ENOMEM;
                    } else {
                        slot = L.cnt[0];
                        pos = size;
                    }
                } else {
                    const uint64_t a = __ldcv((const unsigned long long*)&sl->a);
                    if (a >= (uint64_t)size) {
                        st = SVDB_CMP_OUT_OF_BOUNDS;  // src/put_handler.c:155, src/delete_handler.c:84
                    } else if (op == SVDB_REQ_UPDATE && L.cnt[2] >= L.kcap) {
                        st = SVDB_ENOMEM;
                    } else {
                        pos = (int64_t)a;
                        slot = fen_find(L.fen, L.fn, pos);
                    }
                }
                s_status = st;
                s_slot = slot;
                s_pos = pos;
            }
            __syncthreads();
            if (s_status == SVDB_OK && op != SVDB_REQ_DELETE) {  // the row (and uuid) into its slot
                double* dst = L.x + s_slot * L.dim;
                for (int c = t; c < L.dim; c += kLoopThreads) dst[c] = __ldcv(v + c);
                if (__ldcv((const unsigned int*)&sl->has_uuid) && t < 40)
                    L.uu[s_slot * 40 + t] = __ldcv((const signed char*)L.uuids + (tk & L.mask) * 40 + t);
            }
            __syncthreads();
            if (t == 0) {
                LoopResp out;
                out.status = s_status;
                out.value = __int_as_float(0x7fc00000);
                out.index = 0;
                if (s_status == SVDB_OK) {
                    if (op == SVDB_REQ_INSERT) {
                        fen_add(L.fen, L.fn, s_slot, 1);
                        L.cnt[0] = s_slot + 1;
                        L.cnt[1] = s_pos + 1;
                        kd_insert(L, L.x + s_slot * L.dim, s_pos);
                        out.index = (uint64_t)s_pos;
                    } else if (op == SVDB_REQ_UPDATE) {
                        kd_insert(L, L.x + s_slot * L.dim, s_pos);  // a second node (src/vector_database.c:176)
                    } else {
                        fen_add(L.fen, L.fn, s_slot, -1);
                        L.cnt[1] = L.cnt[1] - 1;
                    }
                }
                L.resp[tk & L.mask] = out;
            }
            __syncthreads();
            ++i;
        }
        // ------------------------------------------------ publish: answers, then the counter
        __threadfence_system();
        __syncthreads();
        if (t == 0) {
            s_head = h + (uint64_t)n;
            *(volatile uint64_t*)&L.ctl->size = (uint64_t)L.cnt[1];
            *(volatile uint64_t*)&L.ctl->head = h + (uint64_t)n;
            *(volatile uint64_t*)&L.ctl->batches = *(volatile uint64_t*)&L.ctl->batches + 1;
            __threadfence_system();
            st_release_sys(&L.ctl->done, h + (uint64_t)n);
        }
        __syncthreads();
    }
    if (t == 0) {
        *(volatile uint64_t*)&L.ctl->head = s_head;
        if (s_leave == (int)kStateLeftIdle)
            *(volatile uint64_t*)&L.ctl->idle_exits = *(volatile uint64_t*)&L.ctl->idle_exits + 1;
        __threadfence_system();
        st_release_sys32(&L.ctl->state, (uint32_t)s_leave);
    }
}

}  // namespace

struct Loop {
    LoopDev d;
    cudaStream_t stream = nullptr;
    LoopSlot* ring = nullptr;  // host views of the mapped blocks
    LoopResp* resp = nullptr;
    double* vecs = nullptr;
    char* uuids = nullptr;
    LoopCtl* ctl = nullptr;
    uint64_t ring_n = 0;
    std::atomic<uint64_t> next{0};
    std::mutex launch_mu;
    bool launched = false;
    std::vector<void*> dev_allocs;
    std::vector<void*> host_allocs;
};

static void loop_free(Loop* l) {
    if (!l) return;
    if (l->stream) cudaStreamSynchronize(l->stream);
    for (void* p : l->dev_allocs) cudaFree(p);
    for (void* p : l->host_allocs) cudaFreeHost(p);
    if (l->stream) cudaStreamDestroy(l->stream);
    delete l;
}

static int loop_launch(Loop* l) {
    k_serve_loop<<<1, kLoopThreads, 0, l->stream>>>(l->d);
    SVDB_LAUNCH_CHECK();
    l->launched = true;
    return SVDB_OK;
}

}  // namespace svdb

using svdb::Loop;

extern "C" {

svdbd_loop* svdbd_loop_create(const svdb_loop_config* cfg, const double* rows, size_t n, const char* uuids37,
                              const double* kpts, const int64_t* kidx, const int32_t* kleft, const int32_t* kright,
                              size_t knodes, int kheight) {
    using namespace svdb;
    Loop* l = new (std::nothrow) Loop();
    if (!l) {
        svdb_set_error("loop: out of host memory");
        return nullptr;
    }
    const size_t dim = cfg->dim, kd = cfg->kd_dim, cap = cfg->capacity, kcap = cfg->kd_capacity;
    size_t ring = 1;
    while (ring < cfg->ring) ring <<= 1;
    int64_t fn = 1;
    while ((size_t)fn < cap) fn <<= 1;
    const int kstack_h = 4096;
    auto fail = [&](const char* what, cudaError_t e) -> svdbd_loop* {
        cudaGetLastError();
        svdb_set_error("loop: %s: %s", what, cudaGetErrorString(e));
        loop_free(l);
        return nullptr;
    };
    cudaError_t e = cudaStreamCreateWithFlags(&l->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return fail("stream", e);
    // device: the store, reserved whole now (admission by free HBM)
    auto dalloc = [&](void** p, size_t bytes) {
        cudaError_t r = cudaMalloc(p, std::max<size_t>(bytes, 256));
        if (r == cudaSuccess) l->dev_allocs.push_back(*p);
        return r;
    };
    void *x = nullptr, *uu = nullptr, *fen = nullptr, *cnt = nullptr, *kp = nullptr, *ki = nullptr, *kc = nullptr,
         *ks = nullptr;
    if ((e = dalloc(&x, cap * dim * sizeof(double))) != cudaSuccess ||
        (e = dalloc(&uu, cap * 40)) != cudaSuccess || (e = dalloc(&fen, (size_t)(fn + 1) * sizeof(int32_t))) != cudaSuccess ||
        (e = dalloc(&cnt, 4 * sizeof(int64_t))) != cudaSuccess ||
        (e = dalloc(&kp, kcap * kd * sizeof(double))) != cudaSuccess ||
        (e = dalloc(&ki, kcap * sizeof(int64_t))) != cudaSuccess || (e = dalloc(&kc, kcap * sizeof(int2))) != cudaSuccess ||
        (e = dalloc(&ks, (size_t)kLoopThreads * kstack_h * sizeof(int2))) != cudaSuccess) {
        cudaGetLastError();
        svdb_set_error("loop: %zu rows of dimension %zu (and %zu KD nodes) do not fit in free device memory", cap, dim,
                       kcap);
        loop_free(l);
        return nullptr;
    }
    // host: the ring, answers, vectors, uuids and control block, mapped
    auto halloc = [&](void** p, size_t bytes) {
        cudaError_t r = cudaHostAlloc(p, bytes, cudaHostAllocMapped | cudaHostAllocPortable);
        if (r == cudaSuccess) {
            l->host_allocs.push_back(*p);
            std::memset(*p, 0, bytes);
        }
        return r;
    };
    void *hr = nullptr, *hs = nullptr, *hv = nullptr, *hu = nullptr, *hc = nullptr;
    if ((e = halloc(&hr, ring * sizeof(LoopSlot))) != cudaSuccess || (e = halloc(&hs, ring * sizeof(LoopResp))) != cudaSuccess ||
        (e = halloc(&hv, ring * dim * sizeof(double))) != cudaSuccess || (e = halloc(&hu, ring * 40)) != cudaSuccess ||
        (e = halloc(&hc, sizeof(LoopCtl))) != cudaSuccess)
        return fail("page-locked ring", e);
    l->ring = (LoopSlot*)hr;
    l->resp = (LoopResp*)hs;
    l->vecs = (double*)hv;
    l->uuids = (char*)hu;
    l->ctl = (LoopCtl*)hc;
    l->ring_n = ring;
    for (uint64_t i = 0; i < ring; ++i) l->ring[i].free_for = i;
    LoopDev& D = l->d;
    if ((e = cudaHostGetDevicePointer((void**)&D.ring, hr, 0)) != cudaSuccess ||
        (e = cudaHostGetDevicePointer((void**)&D.resp, hs, 0)) != cudaSuccess ||
        (e = cudaHostGetDevicePointer((void**)&D.vecs, hv, 0)) != cudaSuccess ||
        (e = cudaHostGetDevicePointer((void**)&D.uuids, hu, 0)) != cudaSuccess ||
        (e = cudaHostGetDevicePointer((void**)&D.ctl, hc, 0)) != cudaSuccess)
        return fail("mapping the ring", e);
    D.mask = ring - 1;
    D.x = (double*)x;
    D.uu = (char*)uu;
    D.fen = (int32_t*)fen;
    D.fn = fn;
    D.cnt = (int64_t*)cnt;
    D.kpts = (double*)kp;
    D.kidx = (int64_t*)ki;
    D.kchild = (int2*)kc;
    D.kstack = (int2*)ks;
    D.cap = (int64_t)cap;
    D.kcap = (int64_t)kcap;
    D.dim = (int)dim;
    D.kdim = (int)kd;
    D.kstack_h = kstack_h;
    D.max_batch = (int)std::min<uint32_t>(std::max<uint32_t>(cfg->max_batch, 1u), (uint32_t)kLoopThreads);
    D.idle_ns = (uint64_t)std::max<uint32_t>(cfg->idle_us, 1u) * 1000ull;
    // the initial rows: slots 0..n-1, all live; the KD tree built by the caller
    std::vector<int32_t> hf((size_t)fn + 1, 0);
    for (int64_t i = 1; i <= fn; ++i) {  // fen[i] = live slots in (i - lowbit(i), i]
        const int64_t lo = i - (i & -i);
        hf[i] = (int32_t)std::max<int64_t>(0, std::min<int64_t>((int64_t)n, i) - lo);
    }
    const int64_t hcnt[4] = {(int64_t)n, (int64_t)n, (int64_t)knodes, (int64_t)kheight};
    std::vector<int2> hch(knodes);
    for (size_t i = 0; i < knodes; ++i) hch[i] = make_int2(kleft[i], kright[i]);
    if (n) {
        if ((e = cudaMemcpyAsync(x, rows, n * dim * sizeof(double), cudaMemcpyHostToDevice, l->stream)) != cudaSuccess)
            return fail("upload", e);
    }
    std::vector<char> hu40(std::max<size_t>(n, 1) * 40, 0);
    if (uuids37)
        for (size_t i = 0; i < n; ++i) std::memcpy(hu40.data() + i * 40, uuids37 + i * 37, 37);
    if ((n && (e = cudaMemcpyAsync(uu, hu40.data(), n * 40, cudaMemcpyHostToDevice, l->stream)) != cudaSuccess) ||
        (e = cudaMemcpyAsync(fen, hf.data(), hf.size() * sizeof(int32_t), cudaMemcpyHostToDevice, l->stream)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync(cnt, hcnt, sizeof(hcnt), cudaMemcpyHostToDevice, l->stream)) != cudaSuccess ||
        (knodes && (e = cudaMemcpyAsync(kp, kpts, knodes * kd * sizeof(double), cudaMemcpyHostToDevice, l->stream)) !=
                       cudaSuccess) ||
        (knodes && (e = cudaMemcpyAsync(ki, kidx, knodes * sizeof(int64_t), cudaMemcpyHostToDevice, l->stream)) !=
                       cudaSuccess) ||
        (knodes && (e = cudaMemcpyAsync(kc, hch.data(), knodes * sizeof(int2), cudaMemcpyHostToDevice, l->stream)) !=
                       cudaSuccess))
        return fail("upload", e);
    if ((e = cudaStreamSynchronize(l->stream)) != cudaSuccess) return fail("upload", e);
    l->ctl->size = n;
    return reinterpret_cast<svdbd_loop*>(l);
}

// Launch the loop when it is not running (first start, or after it left idle
// or was stopped).  A launch only happens once the previous kernel has
// returned, so two loops never serve the same ring.
int svdbd_loop_start(svdbd_loop* hl) {
    Loop* l = reinterpret_cast<Loop*>(hl);
    std::lock_guard<std::mutex> lk(l->launch_mu);
    if (l->launched) {
        const cudaError_t q = cudaStreamQuery(l->stream);
        if (q == cudaErrorNotReady) return SVDB_OK;  // still running
        if (q != cudaSuccess) {
            cudaGetLastError();
            svdb_set_error("loop: %s", cudaGetErrorString(q));
            return SVDB_ECUDA;
        }
    }
    __atomic_store_n(&l->ctl->stop, 0u, __ATOMIC_RELEASE);
    return svdb::loop_launch(l);
}

int svdbd_loop_submit(svdbd_loop* hl, const svdb_request* req, size_t dim, uint64_t* ticket, uint32_t timeout_us) {
    using namespace svdb;
    Loop* l = reinterpret_cast<Loop*>(hl);
    const uint64_t tk = l->next.fetch_add(1, std::memory_order_relaxed);
    LoopSlot* sl = &l->ring[tk & (l->ring_n - 1)];
    // the slot is free once the answer of its previous ticket has been taken
    const auto t0 = std::chrono::steady_clock::now();
    while (__atomic_load_n(&sl->free_for, __ATOMIC_ACQUIRE) != tk) {
        if (std::chrono::steady_clock::now() - t0 > std::chrono::microseconds(timeout_us)) {
            svdb_set_error("loop: ring slot of ticket %llu still holds an answer nobody took",
                           (unsigned long long)tk);
            return SVDB_ETIMEOUT;  // the ticket stays claimed: callers must take every answer
        }
    }
    sl->op = req->op;
    sl->metric = req->metric;
    sl->a = req->a;
    sl->b = req->b;
    sl->has_uuid = 0;
    const uint64_t ix = tk & (l->ring_n - 1);
    if ((req->op == SVDB_REQ_INSERT || req->op == SVDB_REQ_UPDATE || req->op == SVDB_REQ_KD_NEAREST) && req->vec)
        std::memcpy(l->vecs + ix * dim, req->vec, dim * sizeof(double));
    if ((req->op == SVDB_REQ_INSERT || req->op == SVDB_REQ_UPDATE) && (req->uuid || req->op == SVDB_REQ_INSERT)) {
        char* u = l->uuids + ix * 40;
        std::memset(u, 0, 40);
        if (req->uuid) std::strncpy(u, req->uuid, 37);
        sl->has_uuid = 1;
    }
    __atomic_store_n(&sl->seq, tk + 1, __ATOMIC_RELEASE);
    *ticket = tk;
    return SVDB_OK;
}

int svdbd_loop_wait(svdbd_loop* hl, uint64_t ticket, svdb_response* out, uint32_t timeout_us) {
    using namespace svdb;
    Loop* l = reinterpret_cast<Loop*>(hl);
    const auto t0 = std::chrono::steady_clock::now();
    for (uint32_t it = 0;; ++it) {
        if (__atomic_load_n(&l->ctl->done, __ATOMIC_ACQUIRE) > ticket) {
            LoopSlot* sl = &l->ring[ticket & (l->ring_n - 1)];
            const LoopResp r = l->resp[ticket & (l->ring_n - 1)];
            out->status = r.status;
            out->value = r.value;
            out->index = r.index;
            __atomic_store_n(&sl->free_for, ticket + l->ring_n, __ATOMIC_RELEASE);
            return SVDB_OK;
        }
        if ((it & 255) == 255) {
            // the loop may have left (idle, stopped): start it again for this ticket
            const uint32_t st = __atomic_load_n(&l->ctl->state, __ATOMIC_ACQUIRE);
            if (st != kStateRunning) {
                int rc = svdbd_loop_start(hl);
                if (rc) return rc;
            }
            if (std::chrono::steady_clock::now() - t0 > std::chrono::microseconds(timeout_us)) {
                svdb_set_error("loop: ticket %llu not answered within %u us", (unsigned long long)ticket, timeout_us);
                return SVDB_ETIMEOUT;
            }
        }
    }
}

int svdbd_loop_stop(svdbd_loop* hl) {
    Loop* l = reinterpret_cast<Loop*>(hl);
    std::lock_guard<std::mutex> lk(l->launch_mu);
    __atomic_store_n(&l->ctl->stop, 1u, __ATOMIC_RELEASE);
    const cudaError_t e = cudaStreamSynchronize(l->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        svdb_set_error("loop: %s", cudaGetErrorString(e));
        return SVDB_ECUDA;
    }
    return SVDB_OK;
}

int svdbd_loop_info(svdbd_loop* hl, svdb_loop_info* out) {
    Loop* l = reinterpret_cast<Loop*>(hl);
    out->state = __atomic_load_n(&l->ctl->state, __ATOMIC_ACQUIRE);
    out->size = __atomic_load_n(&l->ctl->size, __ATOMIC_ACQUIRE);
    out->answered = __atomic_load_n(&l->ctl->done, __ATOMIC_ACQUIRE);
    out->batches = __atomic_load_n(&l->ctl->batches, __ATOMIC_ACQUIRE);
    out->idle_exits = __atomic_load_n(&l->ctl->idle_exits, __ATOMIC_ACQUIRE);
    return SVDB_OK;
}

// a row and its uuid by position, with the loop not running
int svdbd_loop_read(svdbd_loop* hl, size_t position, double* row, char* uuid37) {
    using namespace svdb;
    Loop* l = reinterpret_cast<Loop*>(hl);
    std::lock_guard<std::mutex> lk(l->launch_mu);
    if (l->launched && cudaStreamQuery(l->stream) == cudaErrorNotReady) {
        svdb_set_error("loop: rows are read while the loop is not running (svdb_loop_stop first)");
        return SVDB_EINVAL;
    }
    int64_t cnt[4];
    SVDB_CUDA(cudaMemcpy(cnt, l->d.cnt, sizeof(cnt), cudaMemcpyDeviceToHost));
    if ((int64_t)position >= cnt[1]) {
        svdb_set_error("loop: position %zu past the %lld rows", position, (long long)cnt[1]);
        return SVDB_EINVAL;
    }
    std::vector<int32_t> fen((size_t)l->d.fn + 1);
    SVDB_CUDA(cudaMemcpy(fen.data(), l->d.fen, fen.size() * sizeof(int32_t), cudaMemcpyDeviceToHost));
    int64_t pos = 0, rem = (int64_t)position + 1;
    for (int64_t step = l->d.fn; step > 0; step >>= 1)
        if (pos + step <= l->d.fn && fen[pos + step] < rem) {
            pos += step;
            rem -= fen[pos];
        }
    SVDB_CUDA(cudaMemcpy(row, l->d.x + pos * l->d.dim, l->d.dim * sizeof(double), cudaMemcpyDeviceToHost));
    if (uuid37) SVDB_CUDA(cudaMemcpy(uuid37, l->d.uu + pos * 40, 37, cudaMemcpyDeviceToHost));
    return SVDB_OK;
}

void svdbd_loop_destroy(svdbd_loop* hl) {
    Loop* l = reinterpret_cast<Loop*>(hl);
    if (!l) return;
    __atomic_store_n(&l->ctl->stop, 1u, __ATOMIC_RELEASE);
    svdb::loop_free(l);
}

}  // extern "C"
