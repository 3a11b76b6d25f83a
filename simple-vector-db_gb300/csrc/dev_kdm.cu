// dev_kdm.cu -- a median-split KD tree over the store's rows, built on the
// device, and its batched exact nearest-neighbour descent (opt-in /nearest).
//
// The reference's tree (src/kdtree.c) is an insertion-order tree with stale
// nodes after updates and deletes; README.md:3,34 describes a median tree.
// This builds that median tree from the store's current searchable rows, over
// the first kdim coordinates: an exact 1-NN over the prefix like the
// reference's (src/kdtree.c:131-162, same unfused FP64 distance), with ties
// to the lowest position instead of the first node visited, and no stale
// nodes -- so it is an opt-in mode, not the drop-in /nearest.
//
// Layout: the implicit in-place tree.  Points are ordered so that the
// subtree of the range [lo, hi) at depth t has its root at mid = lo + (hi -
// lo) / 2, split on axis t % kdim: points of [lo, mid) come before the root
// in (coordinate, position) order, points of (mid, hi) after it.  No child
// pointers: a descent carries (lo, hi, depth).
//
// Build (all on the device, O(kdim n log n)): rows are compacted in slot
// (= position) order; for every axis the points are sorted once by
// (coordinate, position) with a stable LSD radix sort (4-bit digits on the
// order-preserving 64-bit image of the double); then level by level the
// split axis's list gives each range's median directly (its middle
// element), and every other axis's list is stably partitioned around that
// median inside each range (one 64-bit scan of {left, median} flags per list
// and level), which keeps each list sorted within the new ranges.  After the
// last level all lists hold the tree order.
#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "dev_common.cuh"
#include "dev_store.cuh"

namespace svdb {

struct KdmTree {
    size_t kdim = 0, n = 0;
    uint64_t version = ~0ull;  // store version the tree was built from
    double* pts = nullptr;     // n x kdim, tree order
    int64_t* pos = nullptr;    // n positions, tree order
    int height = 0;
};

namespace {

constexpr int kScanTile = 2048;  // elements per block of the scans (1024 threads x 2)

// ---- generic exclusive scan (int32 or uint64) --------------------------------
template <class T>
__global__ void __launch_bounds__(1024) k_scan_tile(const T* __restrict__ in, T* __restrict__ out, int64_t n,
                                                    T* __restrict__ totals) {
    __shared__ T s[kScanTile];
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    for (int j = threadIdx.x; j < kScanTile; j += 1024) s[j] = base + j < n ? in[base + j] : T(0);
    __syncthreads();
    // Blelloch scan in shared memory
    for (int d = 1; d < kScanTile; d <<= 1) {
        const int i = (threadIdx.x + 1) * 2 * d - 1;
        if (i < kScanTile) s[i] += s[i - d];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        totals[blockIdx.x] = s[kScanTile - 1];
        s[kScanTile - 1] = T(0);
    }
    __syncthreads();
    for (int d = kScanTile / 2; d >= 1; d >>= 1) {
        const int i = (threadIdx.x + 1) * 2 * d - 1;
        if (i < kScanTile) {
            const T t = s[i - d];
            s[i - d] = s[i];
            s[i] += t;
        }
        __syncthreads();
    }
    for (int j = threadIdx.x; j < kScanTile; j += 1024)
        if (base + j < n) out[base + j] = s[j];
}

// exclusive scan of the per-tile totals by one block (tiles are few)
template <class T>
__global__ void __launch_bounds__(1024) k_scan_totals(T* __restrict__ totals, int64_t nt) {
    __shared__ T part[1024];
    const int64_t per = (nt + 1023) / 1024;
    const int64_t lo = threadIdx.x * per, hi = std::min<int64_t>(lo + per, nt);
    T sum = T(0);
    for (int64_t i = lo; i < hi; ++i) sum += totals[i];
    part[threadIdx.x] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        T run = T(0);
        for (int i = 0; i < 1024; ++i) {
            const T t = part[i];
            part[i] = run;
            run += t;
        }
    }
    __syncthreads();
    T run = part[threadIdx.x];
    for (int64_t i = lo; i < hi; ++i) {
        const T t = totals[i];
        totals[i] = run;
        run += t;
    }
}

template <class T>
__global__ void k_scan_add(T* __restrict__ out, int64_t n, const T* __restrict__ totals) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] += totals[i / kScanTile];
}

// out[i] = sum of in[0..i); totals: ceil(n / kScanTile) entries of scratch
template <class T>
int exclusive_scan(const T* in, T* out, int64_t n, T* totals, cudaStream_t st) {
    if (n <= 0) return SVDB_OK;
    const int64_t nt = (n + kScanTile - 1) / kScanTile;
    k_scan_tile<T><<<(unsigned)nt, 1024, 0, st>>>(in, out, n, totals);
    SVDB_LAUNCH_CHECK();
    k_scan_totals<T><<<1, 1024, 0, st>>>(totals, nt);
    SVDB_LAUNCH_CHECK();
    k_scan_add<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out, n, totals);
    SVDB_LAUNCH_CHECK();
    return SVDB_OK;
}

// ---- compaction of the searchable rows ---------------------------------------
__global__ void k_kdm_flags(const uint8_t* __restrict__ live, int64_t slots, int* __restrict__ f) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s < slots) f[s] = live[s] == 1 ? 1 : 0;
}

__global__ void k_kdm_compact(const uint8_t* __restrict__ live, const int* __restrict__ dst, int64_t slots,
                              const double* __restrict__ x64, size_t ld, const int64_t* __restrict__ logical,
                              int kdim, double* __restrict__ P, int64_t* __restrict__ pos) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= slots || live[s] != 1) return;
    const int64_t i = dst[s];
    for (int a = 0; a < kdim; ++a) P[i * kdim + a] = x64[s * (int64_t)ld + a];
    pos[i] = logical[s];
}

// order-preserving image of a double (negatives reversed, sign flipped)
__device__ __forceinline__ uint64_t ord64(double x) {
    const uint64_t u = (uint64_t)__double_as_longlong(x);
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

__global__ void k_kdm_keys(const double* __restrict__ P, int kdim, int a, int64_t n, uint64_t* __restrict__ key,
                           int* __restrict__ id) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) {
        key[i] = ord64(P[i * kdim + a]);
        id[i] = (int)i;
    }
}

// ---- stable LSD radix sort, 4-bit digits, 1024-element tiles ------------------
constexpr int kRsThreads = 1024;

__global__ void __launch_bounds__(kRsThreads) k_rs_count(const uint64_t* __restrict__ key, int64_t n, int shift,
                                                         int* __restrict__ counts, int ntiles) {
    __shared__ int h[16];
    if (threadIdx.x < 16) h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * kRsThreads + threadIdx.x;
    if (i < n) atomicAdd(&h[(key[i] >> shift) & 15u], 1);
    __syncthreads();
    if (threadIdx.x < 16) counts[(int64_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(kRsThreads) k_rs_scatter(const uint64_t* __restrict__ key, const int* __restrict__ id,
                                                           int64_t n, int shift, const int* __restrict__ offs,
                                                           int ntiles, uint64_t* __restrict__ key2,
                                                           int* __restrict__ id2) {
    __shared__ int wcnt[kRsThreads / 32][16];
    __shared__ int woff[kRsThreads / 32][16];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t i = (int64_t)blockIdx.x * kRsThreads + threadIdx.x;
    const bool act = i < n;
    const uint64_t k = act ? key[i] : 0;
    const int d = act ? (int)((k >> shift) & 15u) : 16;  // 16: not a digit (inactive lanes)
    for (int j = threadIdx.x; j < (kRsThreads / 32) * 16; j += kRsThreads) (&wcnt[0][0])[j] = 0;
    __syncthreads();
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int rank = __popc(peers & ((1u << lane) - 1u));
    if (act && rank == 0) wcnt[warp][d] = __popc(peers);
    __syncthreads();
    if (threadIdx.x < 16) {
        int run = 0;
        for (int w = 0; w < kRsThreads / 32; ++w) {
            woff[w][threadIdx.x] = run;
            run += wcnt[w][threadIdx.x];
        }
    }
    __syncthreads();
    if (act) {
        const int64_t dst = (int64_t)offs[(int64_t)d * ntiles + blockIdx.x] + woff[warp][d] + rank;
        key2[dst] = k;
        id2[dst] = id[i];
    }
}

// ---- level step of the build ---------------------------------------------------
// Range of position i at depth `lvl` (descending from the root); returns
// false when i is the median of a shallower range (already placed).
__device__ __forceinline__ bool range_of(int64_t i, int64_t n, int lvl, int64_t& lo, int64_t& hi) {
    lo = 0;
    hi = n;
    for (int t = 0; t < lvl; ++t) {
        const int64_t mid = lo + (hi - lo) / 2;
        if (i < mid)
            hi = mid;
        else if (i > mid)
            lo = mid + 1;
        else
            return false;
    }
    return true;
}

__device__ __forceinline__ bool key_before(const double* __restrict__ P, const int64_t* __restrict__ pos, int kdim,
                                           int a, int e, int m) {
    const uint64_t ke = ord64(P[(int64_t)e * kdim + a]), km = ord64(P[(int64_t)m * kdim + a]);
    return ke < km || (ke == km && pos[e] < pos[m]);
}

// flags of list b at depth lvl: bit 0 = left of its range's median, bit 32 = the median
__global__ void k_kdm_flag(const int* __restrict__ La, const int* __restrict__ Lb, int64_t n, int lvl,
                           const double* __restrict__ P, const int64_t* __restrict__ pos, int kdim, int a,
                           uint64_t* __restrict__ f) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    int64_t lo, hi;
    uint64_t v = 0;
    if (range_of(i, n, lvl, lo, hi)) {
        const int m = La[lo + (hi - lo) / 2];
        const int e = Lb[i];
        if (e == m)
            v = 1ull << 32;
        else if (key_before(P, pos, kdim, a, e, m))
            v = 1;
    }
    f[i] = v;
}

__global__ void k_kdm_part(const int* __restrict__ Lb, int64_t n, int lvl, const uint64_t* __restrict__ f,
                           const uint64_t* __restrict__ sc, int* __restrict__ out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    int64_t lo, hi;
    if (!range_of(i, n, lvl, lo, hi)) {
        out[i] = Lb[i];
        return;
    }
    const int64_t mid = lo + (hi - lo) / 2;
    const uint64_t before = sc[i] - sc[lo];
    const int64_t left = (int64_t)(before & 0xffffffffull), med = (int64_t)(before >> 32);
    int64_t dst;
    if (f[i] >> 32)
        dst = mid;
    else if (f[i] & 1ull)
        dst = lo + left;
    else
        dst = mid + 1 + ((i - lo) - left - med);
    out[dst] = Lb[i];
}

__global__ void k_kdm_emit(const int* __restrict__ T, int64_t n, const double* __restrict__ P,
                           const int64_t* __restrict__ pos, int kdim, double* __restrict__ tp,
                           int64_t* __restrict__ tpos) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int e = T[i];
    for (int a = 0; a < kdim; ++a) tp[i * kdim + a] = P[(int64_t)e * kdim + a];
    tpos[i] = pos[e];
}

// ---- batched descent -----------------------------------------------------------
constexpr int kKdmStack = 96;  // > 2 x the depth of any tree of < 2^40 points

__global__ void __launch_bounds__(128) k_kdm_nearest(const double* __restrict__ tp, const int64_t* __restrict__ tpos,
                                                     int64_t n, int kdim, const double* __restrict__ q, size_t qs,
                                                     int nq, int64_t* __restrict__ out) {
    const int qi = blockIdx.x * blockDim.x + threadIdx.x;
    if (qi >= nq) return;
    const double* qq = q + (size_t)qi * qs;
    struct Ent {
        int64_t lo, hi;
        double plane;
        int depth;
    };
    Ent st[kKdmStack];
    int sp = 0;
    double best = __longlong_as_double(0x7ff0000000000000ll);
    int64_t bpos = -1;
    if (n > 0) st[sp++] = Ent{0, n, 0.0, 0};
    while (sp > 0) {
        const Ent e = st[--sp];
        if (e.lo >= e.hi || e.plane > best) continue;  // pruned: every point there is farther
        const int64_t mid = e.lo + (e.hi - e.lo) / 2;
        const double* p = tp + mid * kdim;
        double d = 0.0;
        for (int i = 0; i < kdim; ++i) {
            const double t = __dsub_rn(p[i], qq[i]);
            d = __dadd_rn(d, __dmul_rn(t, t));
        }
        const int64_t pp = tpos[mid];
        if (d < best || (d == best && pp < bpos)) {
            best = d;
            bpos = pp;
        }
        const int ax = e.depth % kdim;
        const double t = __dsub_rn(qq[ax], p[ax]);
        const double plane = __dmul_rn(t, t);
        const Ent L{e.lo, mid, 0.0, e.depth + 1}, R{mid + 1, e.hi, 0.0, e.depth + 1};
        const bool left_near = qq[ax] < p[ax];
        Ent nearE = left_near ? L : R, farE = left_near ? R : L;
        farE.plane = plane;
        if (sp + 2 <= kKdmStack) {  // depth <= 2 log2(n) + 2 keeps this true
            st[sp++] = farE;
            st[sp++] = nearE;
        }
    }
    out[qi] = bpos;
}

}  // namespace

void Store::kdm_free() {
    if (!kdm) return;
    cudaFree(kdm->pts);
    cudaFree(kdm->pos);
    delete kdm;
    kdm = nullptr;
}

// (re)build the median tree over the searchable rows when the rows changed
static int kdm_build(Store* s, size_t kdim) {
    if (s->kdm && s->kdm->version == s->version && s->kdm->kdim == kdim) return SVDB_OK;
    if (!s->kdm) {
        s->kdm = new (std::nothrow) KdmTree();
        if (!s->kdm) {
            svdb_set_error("median KD tree: out of host memory");
            return SVDB_ENOMEM;
        }
    }
    KdmTree* t = s->kdm;
    cudaFree(t->pts);
    cudaFree(t->pos);
    t->pts = nullptr;
    t->pos = nullptr;
    t->n = 0;
    t->kdim = kdim;
    const int64_t slots = (int64_t)s->slots;
    // live == 1 rows, compacted in slot order
    const int64_t ntile_s = (slots + kScanTile - 1) / kScanTile + 1;
    std::vector<void*> bufs;
    auto alloc = [&](void** p, size_t bytes) {
        cudaError_t e = cudaMalloc(p, std::max<size_t>(bytes, 256));
        if (e != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        bufs.push_back(*p);
        return true;
    };
    auto release = [&]() {
        for (void* p : bufs) cudaFree(p);
        bufs.clear();
    };
    int* flags = nullptr;
    int* dst = nullptr;
    int* itot = nullptr;
    if (!alloc((void**)&flags, slots * sizeof(int)) || !alloc((void**)&dst, slots * sizeof(int)) ||
        !alloc((void**)&itot, ntile_s * sizeof(int))) {
        release();
        svdb_set_error("median KD tree: cannot allocate build buffers");
        return SVDB_ENOMEM;
    }
    int rc = SVDB_OK;
    int64_t n = 0;
    if (slots) {
        k_kdm_flags<<<(unsigned)((slots + 255) / 256), 256, 0, s->stream>>>(s->live, slots, flags);
        SVDB_LAUNCH_CHECK();
        rc = exclusive_scan<int>(flags, dst, slots, itot, s->stream);
        if (rc) {
            release();
            return rc;
        }
        int last_dst = 0, last_flag = 0;
        SVDB_CUDA(cudaMemcpyAsync(&last_dst, dst + slots - 1, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
        SVDB_CUDA(cudaMemcpyAsync(&last_flag, flags + slots - 1, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
        SVDB_CUDA(cudaStreamSynchronize(s->stream));
        n = (int64_t)last_dst + last_flag;
    }
    if (n == 0) {
        release();
        t->version = s->version;
        t->height = 0;
        return SVDB_OK;
    }
    double* P = nullptr;
    int64_t* pos = nullptr;
    uint64_t *key = nullptr, *key2 = nullptr, *f = nullptr, *sc = nullptr, *ltot = nullptr;
    int *id2 = nullptr, *cnt = nullptr, *ctot = nullptr, *tmp = nullptr;
    std::vector<int*> L(kdim, nullptr);
    const int ntiles = (int)((n + kRsThreads - 1) / kRsThreads);
    const int64_t ntile_n = (n + kScanTile - 1) / kScanTile + 1;
    const int64_t ntile_c = (16 * (int64_t)ntiles + kScanTile - 1) / kScanTile + 1;
    bool ok = alloc((void**)&P, n * kdim * sizeof(double)) && alloc((void**)&pos, n * sizeof(int64_t)) &&
              alloc((void**)&key, n * sizeof(uint64_t)) && alloc((void**)&key2, n * sizeof(uint64_t)) &&
              alloc((void**)&id2, n * sizeof(int)) && alloc((void**)&cnt, 16 * (size_t)ntiles * sizeof(int)) &&
              alloc((void**)&ctot, ntile_c * sizeof(int)) && alloc((void**)&f, n * sizeof(uint64_t)) &&
              alloc((void**)&sc, n * sizeof(uint64_t)) && alloc((void**)&ltot, ntile_n * sizeof(uint64_t)) &&
              alloc((void**)&tmp, n * sizeof(int));
    for (size_t a = 0; a < kdim && ok; ++a) ok = alloc((void**)&L[a], n * sizeof(int));
    if (!ok) {
        release();
        svdb_set_error("median KD tree: cannot allocate build buffers for %lld rows", (long long)n);
        return SVDB_ENOMEM;
    }
    const unsigned gs = (unsigned)((slots + 255) / 256), gn = (unsigned)((n + 255) / 256);
    k_kdm_compact<<<gs, 256, 0, s->stream>>>(s->live, dst, slots, s->x64, s->ld, s->logical, (int)kdim, P, pos);
    SVDB_LAUNCH_CHECK();
    // one stable sort per axis by (coordinate, position): ids start in position order
    for (size_t a = 0; a < kdim; ++a) {
        k_kdm_keys<<<gn, 256, 0, s->stream>>>(P, (int)kdim, (int)a, n, key, L[a]);
        SVDB_LAUNCH_CHECK();
        uint64_t* kin = key;
        uint64_t* kout = key2;
        int* iin = L[a];
        int* iout = id2;
        for (int shift = 0; shift < 64; shift += 4) {
            k_rs_count<<<(unsigned)ntiles, kRsThreads, 0, s->stream>>>(kin, n, shift, cnt, ntiles);
            SVDB_LAUNCH_CHECK();
            rc = exclusive_scan<int>(cnt, cnt, 16 * (int64_t)ntiles, ctot, s->stream);
            if (rc) break;
            k_rs_scatter<<<(unsigned)ntiles, kRsThreads, 0, s->stream>>>(kin, iin, n, shift, cnt, ntiles, kout, iout);
            SVDB_LAUNCH_CHECK();
            std::swap(kin, kout);
            std::swap(iin, iout);
        }
        if (rc) break;
        // 16 passes: the result is back in (key, L[a])
    }
    // levels: the split axis's list gives the medians; the others are partitioned
    int levels = 0;
    for (int64_t m = n; m > 0; m /= 2) ++levels;
    for (int lvl = 0; lvl < levels && !rc; ++lvl) {
        const int a = lvl % (int)kdim;
        for (size_t b = 0; b < kdim && !rc; ++b) {
            if ((int)b == a) continue;
            k_kdm_flag<<<gn, 256, 0, s->stream>>>(L[a], L[b], n, lvl, P, pos, (int)kdim, a, f);
            SVDB_LAUNCH_CHECK();
            rc = exclusive_scan<uint64_t>(f, sc, n, ltot, s->stream);
            if (rc) break;
            k_kdm_part<<<gn, 256, 0, s->stream>>>(L[b], n, lvl, f, sc, tmp);
            SVDB_LAUNCH_CHECK();
            std::swap(L[b], tmp);
        }
    }
    if (!rc) {
        cudaError_t e = cudaMalloc(&t->pts, n * kdim * sizeof(double));
        if (e == cudaSuccess) e = cudaMalloc(&t->pos, n * sizeof(int64_t));
        if (e != cudaSuccess) {
            cudaGetLastError();
            svdb_set_error("median KD tree: cannot allocate the tree");
            rc = SVDB_ENOMEM;
        } else {
            k_kdm_emit<<<gn, 256, 0, s->stream>>>(L[0], n, P, pos, (int)kdim, t->pts, t->pos);
            SVDB_LAUNCH_CHECK();
        }
    }
    // every list pointer (swapped or not) is in `bufs`
    SVDB_CUDA(cudaStreamSynchronize(s->stream));
    release();
    if (rc) return rc;
    t->n = (size_t)n;
    t->height = levels;
    t->version = s->version;
    return SVDB_OK;
}

int Store::kdm_nearest(size_t kdim, const double* q, size_t nq, size_t qstride, int64_t* out) {
    int rc = sync();
    if (rc) return rc;
    if (kdim == 0 || kdim > dim || qstride < kdim) {
        svdb_set_error("median KD tree: kd dimension %zu must be 1..%zu and <= the query stride", kdim, dim);
        return SVDB_EINVAL;
    }
    rc = kdm_build(this, kdim);
    if (rc) return rc;
    if (nq == 0) return SVDB_OK;
    const size_t qb = round_up(nq * qstride * sizeof(double), 256);
    rc = scratch_reserve(qb + nq * sizeof(int64_t));
    if (!rc) rc = pinned_reserve(std::max(nq * qstride * sizeof(double), nq * sizeof(int64_t)));
    if (rc) return rc;
    double* dq = (double*)scratch;
    int64_t* dout = (int64_t*)((uint8_t*)scratch + qb);
    std::memcpy(pin, q, nq * qstride * sizeof(double));
    SVDB_CUDA(cudaMemcpyAsync(dq, pin, nq * qstride * sizeof(double), cudaMemcpyHostToDevice, stream));
    k_kdm_nearest<<<(unsigned)((nq + 127) / 128), 128, 0, stream>>>(kdm->pts, kdm->pos, (int64_t)kdm->n, (int)kdim, dq,
                                                                    qstride, (int)nq, dout);
    SVDB_LAUNCH_CHECK();
    SVDB_CUDA(cudaMemcpyAsync(pin, dout, nq * sizeof(int64_t), cudaMemcpyDeviceToHost, stream));
    SVDB_CUDA(cudaStreamSynchronize(stream));
    std::memcpy(out, pin, nq * sizeof(int64_t));
    return SVDB_OK;
}

}  // namespace svdb

extern "C" int svdbd_kdm_nearest(svdbd_store* hs, size_t kdim, const double* q, size_t nq, size_t qstride,
                                 int64_t* out_pos) {
    return reinterpret_cast<svdb::Store*>(hs)->kdm_nearest(kdim, q, nq, qstride, out_pos);
}
