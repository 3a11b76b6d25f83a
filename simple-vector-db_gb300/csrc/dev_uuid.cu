// dev_uuid.cu -- uuid -> positional index on the device, and rows of the
// reference's file format unpacked straight into HBM.
//
// The reference finds a row by uuid with a linear scan of the host array,
// first match in positional order, compared with strncmp(.., 37)
// (src/vector_database.c:145-158).  Here every slot's uuid is kept on the
// device as a 40-byte record: the bytes up to the first NUL (at most 37),
// zero padded -- two uuids are equal under strncmp(.., 37) exactly when their
// records are equal.  Non-empty records are indexed by a hash table of
// distinct keys (open addressing, linear probing, load <= 1/2) whose entries
// head chains of nodes {slot, next}; a slot whose uuid is set again gets a
// new node under its new key and its old node goes stale (a lookup compares
// the slot's current record, so stale nodes never match).  A lookup walks its
// key's chain and takes the lowest slot that is not deleted: slots never move
// and positions are ranks of live slots, so the lowest slot is the first
// match in positional order, as the reference's scan finds it.  The empty
// uuid "" is not indexed (rows inserted without one would make one chain of
// them all); its lookups take the lowest live slot whose record is empty, by
// a scan of all slots.
//
// A chain holds every node ever made for its key, so a key shared by m rows
// costs a walk of m nodes; the table is rebuilt from the current records
// (one node per slot, stale nodes dropped) whenever the nodes would exceed
// half its size.
#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "dev_common.cuh"
#include "dev_store.cuh"

namespace svdb {

struct __align__(8) UuidStage {
    int64_t slot;
    uint64_t w[5];  // normalized record
};

struct UuidIndex {
    uint64_t* rec = nullptr;  // reccap x 5 words
    size_t reccap = 0;
    uint64_t* tkey = nullptr;  // H: hash of the entry's key, 0 = empty
    int32_t* thead = nullptr;  // H: first node of the entry's chain, -1 = none
    int32_t* nslot = nullptr;  // P = H / 2: slot of each node
    int32_t* nnext = nullptr;  // P: next node, -1 = end
    size_t H = 0, nodes = 0;
    UuidStage* dstage = nullptr;  // device copy of the staged records
    size_t dstage_cap = 0;
    std::vector<UuidStage> stage;       // staged records, at most one per slot
    std::vector<int64_t> stage_at;      // slot -> index in stage + 1 (0: none), grown on demand
};

namespace {

// normalized record of a uuid as the reference stores it (char[37]); words
// are little-endian byte groups
void normalize(const char* u, uint64_t w[5]) {
    uint8_t b[40] = {0};
    for (int i = 0; i < 37 && u[i]; ++i) b[i] = (uint8_t)u[i];
    std::memcpy(w, b, 40);
}

__device__ __forceinline__ uint64_t rec_hash(const uint64_t w[5]) {
    // 64-bit mix of the five words (xor-multiply-shift rounds); never 0
    uint64_t h = 0x9e3779b97f4a7c15ull;
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        h ^= w[i] + 0x632be59bd9b4e019ull + (h << 6) + (h >> 2);
        h *= 0xff51afd7ed558ccdull;
        h ^= h >> 33;
    }
    return h | 1ull;
}

__device__ __forceinline__ bool rec_empty(const uint64_t w[5]) { return (w[0] | w[1] | w[2] | w[3] | w[4]) == 0; }

__device__ __forceinline__ bool rec_eq(const uint64_t* __restrict__ a, const uint64_t w[5]) {
    return a[0] == w[0] && a[1] == w[1] && a[2] == w[2] && a[3] == w[3] && a[4] == w[4];
}

// claim (or find) the table entry of hash h and push `node` on its chain;
// returns false when the probe wrapped around the whole table (cannot
// happen at load <= 1/2; reported instead of looping)
__device__ __forceinline__ bool table_push(uint64_t* tkey, int32_t* thead, int32_t* nnext, size_t H, uint64_t h,
                                           int32_t node) {
    const size_t mask = H - 1;
    size_t p = (size_t)h & mask;
    for (size_t probe = 0; probe < H; ++probe, p = (p + 1) & mask) {
        const unsigned long long k = atomicCAS((unsigned long long*)&tkey[p], 0ull, (unsigned long long)h);
        if (k == 0ull || k == h) {
            nnext[node] = atomicExch(&thead[p], node);
            return true;
        }
    }
    return false;
}

__global__ void k_uuid_put(const UuidStage* __restrict__ st, int n, int32_t node_base, uint64_t* __restrict__ rec,
                           uint64_t* tkey, int32_t* thead, int32_t* __restrict__ nslot, int32_t* nnext, size_t H,
                           int* err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint64_t w[5];
#pragma unroll
    for (int j = 0; j < 5; ++j) w[j] = st[i].w[j];
    const int64_t slot = st[i].slot;
#pragma unroll
    for (int j = 0; j < 5; ++j) rec[slot * 5 + j] = w[j];
    if (rec_empty(w)) return;
    const int32_t node = node_base + i;
    nslot[node] = (int32_t)slot;
    if (!table_push(tkey, thead, nnext, H, rec_hash(w), node)) atomicExch(err, 2);
}

// one node per slot (node s = slot s) from the current records
__global__ void k_uuid_rebuild(const uint64_t* __restrict__ rec, int64_t nslots, uint64_t* tkey, int32_t* thead,
                               int32_t* __restrict__ nslot, int32_t* nnext, size_t H, int* err) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < nslots; s += (int64_t)gridDim.x * blockDim.x) {
        uint64_t w[5];
#pragma unroll
        for (int j = 0; j < 5; ++j) w[j] = rec[s * 5 + j];
        if (rec_empty(w)) continue;
        nslot[s] = (int32_t)s;
        if (!table_push(tkey, thead, nnext, H, rec_hash(w), (int32_t)s)) atomicExch(err, 2);
    }
}

__global__ void k_fill_i32(int32_t* p, size_t n, int32_t v) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) p[i] = v;
}

// lowest live slot whose uuid is empty (for lookups of "")
__global__ void k_uuid_first_empty(const uint64_t* __restrict__ rec, const uint8_t* __restrict__ live, int64_t nslots,
                                   int* out) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < nslots; s += (int64_t)gridDim.x * blockDim.x) {
        if (!live[s]) continue;
        const uint64_t* r = rec ? rec + s * 5 : nullptr;
        if (!r || (r[0] | r[1] | r[2] | r[3] | r[4]) == 0) {
            atomicMin(out, (int)s);
            return;  // later slots of this thread are larger
        }
    }
}

__global__ void k_uuid_find(const uint64_t* __restrict__ keys, int n, const uint64_t* __restrict__ rec,
                            const uint8_t* __restrict__ live, const int64_t* __restrict__ logical,
                            const uint64_t* __restrict__ tkey, const int32_t* __restrict__ thead,
                            const int32_t* __restrict__ nslot, const int32_t* __restrict__ nnext, size_t H,
                            size_t nodes, const int* __restrict__ first_empty, int64_t* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint64_t w[5];
#pragma unroll
    for (int j = 0; j < 5; ++j) w[j] = keys[(size_t)i * 5 + j];
    int64_t best = -1;
    if (rec_empty(w)) {
        const int s = *first_empty;
        best = s < 0x7f7f7f7f ? s : -1;
    } else if (H) {
        const uint64_t h = rec_hash(w);
        const size_t mask = H - 1;
        size_t p = (size_t)h & mask;
        for (size_t probe = 0; probe < H && tkey[p] != 0; ++probe, p = (p + 1) & mask) {
            if (tkey[p] != h) continue;
            size_t steps = 0;
            for (int32_t node = thead[p]; node >= 0 && steps <= nodes; node = nnext[node], ++steps) {
                const int32_t s = nslot[node];
                if ((best < 0 || s < best) && live[s] && rec_eq(rec + (size_t)s * 5, w)) best = s;
            }
            break;
        }
    }
    out[i] = best >= 0 ? logical[best] : -1;
}

// Rows of the reference's file format (uuid[37], size_t dim, double[dim],
// src/vector_database.c:212-223), `rowbytes` apart in `raw` (so doubles sit
// at odd byte offsets): doubles are assembled from bytes into the FP64
// master rows (zero padded to ld), uuid records into the stage.
__global__ void k_unpack_rows(const uint8_t* __restrict__ raw, int64_t n, size_t dim, size_t rowbytes,
                              double* __restrict__ x64, size_t ld, int64_t first, UuidStage* __restrict__ st) {
    const int64_t total = n * (int64_t)ld;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / (int64_t)ld, e = t - i * (int64_t)ld;
        double v = 0.0;
        if ((size_t)e < dim) {
            const uint8_t* p = raw + (size_t)i * rowbytes + 45 + 8 * (size_t)e;
            uint64_t u = 0;
#pragma unroll
            for (int b = 0; b < 8; ++b) u |= (uint64_t)p[b] << (8 * b);
            v = __longlong_as_double((long long)u);
        }
        x64[(first + i) * (int64_t)ld + e] = v;
    }
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint8_t* p = raw + (size_t)i * rowbytes;
        uint64_t w[5] = {0, 0, 0, 0, 0};
        for (int b = 0; b < 37 && p[b]; ++b) w[b >> 3] |= (uint64_t)p[b] << (8 * (b & 7));
        st[i].slot = first + i;
#pragma unroll
        for (int j = 0; j < 5; ++j) st[i].w[j] = w[j];
    }
}

// uuid records of slots [first, first + n) as char[37] (the file format's field)
__global__ void k_pack_uuids(const uint64_t* __restrict__ rec, int64_t first, int64_t n, uint8_t* __restrict__ out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int b = 0; b < 37; ++b) {
        const uint64_t wd = rec ? rec[(first + i) * 5 + (b >> 3)] : 0;
        out[i * 37 + b] = (uint8_t)(wd >> (8 * (b & 7)));
    }
}

template <class T>
int dev_grow(T** p, size_t old_n, size_t new_n, cudaStream_t st, bool zero_new) {
    T* q = nullptr;
    cudaError_t e = cudaMalloc(&q, new_n * sizeof(T));
    if (e != cudaSuccess) {
        cudaGetLastError();
        svdb_set_error("uuid index: cannot allocate %zu bytes: %s", new_n * sizeof(T), cudaGetErrorString(e));
        return SVDB_ENOMEM;
    }
    if (old_n && *p) SVDB_CUDA(cudaMemcpyAsync(q, *p, old_n * sizeof(T), cudaMemcpyDeviceToDevice, st));
    if (zero_new && new_n > old_n) SVDB_CUDA(cudaMemsetAsync(q + old_n, 0, (new_n - old_n) * sizeof(T), st));
    SVDB_CUDA(cudaStreamSynchronize(st));
    cudaFree(*p);
    *p = q;
    return SVDB_OK;
}

}  // namespace

// records for every slot the store can hold (new slots start empty)
static int uid_reserve_rec(Store* s, UuidIndex* u) {
    if (u->reccap >= s->cap) return SVDB_OK;
    int rc = dev_grow(&u->rec, u->reccap * 5, s->cap * 5, s->stream, true);
    if (rc) return rc;
    u->reccap = s->cap;
    return SVDB_OK;
}

static int uid_rebuild(Store* s, UuidIndex* u, size_t incoming) {
    size_t H = 1024;
    while (H < 4 * (s->slots + incoming)) H *= 2;
    cudaFree(u->tkey);
    cudaFree(u->thead);
    cudaFree(u->nslot);
    cudaFree(u->nnext);
    u->tkey = nullptr;
    u->thead = nullptr;
    u->nslot = nullptr;
    u->nnext = nullptr;
    u->H = 0;
    u->nodes = 0;
    cudaError_t e = cudaMalloc(&u->tkey, H * sizeof(uint64_t));
    if (e == cudaSuccess) e = cudaMalloc(&u->thead, H * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&u->nslot, H / 2 * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&u->nnext, H / 2 * sizeof(int32_t));
    if (e != cudaSuccess) {
        cudaGetLastError();
        svdb_set_error("uuid index: cannot allocate a table of %zu entries: %s", H, cudaGetErrorString(e));
        return SVDB_ENOMEM;
    }
    SVDB_CUDA(cudaMemsetAsync(u->tkey, 0, H * sizeof(uint64_t), s->stream));
    k_fill_i32<<<(unsigned)std::min<size_t>((H + 255) / 256, 4096), 256, 0, s->stream>>>(u->thead, H, -1);
    SVDB_LAUNCH_CHECK();
    u->H = H;
    if (s->slots) {
        k_uuid_rebuild<<<(unsigned)std::min<size_t>((s->slots + 255) / 256, 4096), 256, 0, s->stream>>>(
            u->rec, (int64_t)s->slots, u->tkey, u->thead, u->nslot, u->nnext, H, s->d_err);
        SVDB_LAUNCH_CHECK();
    }
    u->nodes = s->slots;
    return SVDB_OK;
}

// push n device-staged records (slots already on the device)
static int uid_put(Store* s, UuidIndex* u, const UuidStage* d_st, size_t n) {
    int rc = uid_reserve_rec(s, u);
    if (rc) return rc;
    if (!u->H || u->nodes + n > u->H / 2) {
        rc = uid_rebuild(s, u, n);
        if (rc) return rc;
    }
    k_uuid_put<<<(unsigned)((n + 255) / 256), 256, 0, s->stream>>>(d_st, (int)n, (int32_t)u->nodes, u->rec, u->tkey,
                                                                   u->thead, u->nslot, u->nnext, u->H, s->d_err);
    SVDB_LAUNCH_CHECK();
    u->nodes += n;
    return SVDB_OK;
}

int Store::uuid_set(int64_t slot, const char* uuid37) {
    if (!uid) {
        uid = new (std::nothrow) UuidIndex();
        if (!uid) {
            svdb_set_error("uuid index: out of host memory");
            return SVDB_ENOMEM;
        }
    }
    UuidStage r;
    r.slot = slot;
    normalize(uuid37, r.w);
    try {
        if ((size_t)slot >= uid->stage_at.size()) uid->stage_at.resize(std::max<size_t>(slot + 1, 2 * uid->stage_at.size()), 0);
        int64_t& at = uid->stage_at[slot];
        if (at) {
            uid->stage[at - 1] = r;  // the last value set for a slot wins
        } else {
            uid->stage.push_back(r);
            at = (int64_t)uid->stage.size();
        }
    } catch (...) {
        svdb_set_error("uuid index: out of host memory");
        return SVDB_ENOMEM;
    }
    return SVDB_OK;
}

// after the rows are flushed (every staged slot exists on the device)
int Store::uuid_flush() {
    if (!uid || uid->stage.empty()) return SVDB_OK;
    UuidIndex* u = uid;
    const size_t n = u->stage.size();
    if (u->dstage_cap < n) {
        cudaFree(u->dstage);
        u->dstage = nullptr;
        u->dstage_cap = 0;
        const size_t c = std::max<size_t>(n, 4096);
        if (cudaMalloc(&u->dstage, c * sizeof(UuidStage)) != cudaSuccess) {
            cudaGetLastError();
            svdb_set_error("uuid index: cannot allocate the staging buffer");
            return SVDB_ENOMEM;
        }
        u->dstage_cap = c;
    }
    SVDB_CUDA(cudaMemcpyAsync(u->dstage, u->stage.data(), n * sizeof(UuidStage), cudaMemcpyHostToDevice, stream));
    int rc = uid_put(this, u, u->dstage, n);
    if (rc) return rc;
    SVDB_CUDA(cudaStreamSynchronize(stream));  // the host stage is reused
    for (const UuidStage& r : u->stage) u->stage_at[r.slot] = 0;
    u->stage.clear();
    return SVDB_OK;
}

void Store::uuid_free() {
    if (!uid) return;
    cudaFree(uid->rec);
    cudaFree(uid->tkey);
    cudaFree(uid->thead);
    cudaFree(uid->nslot);
    cudaFree(uid->nnext);
    cudaFree(uid->dstage);
    delete uid;
    uid = nullptr;
}

int Store::uuid_find(const char* uuids37, size_t n, int64_t* out) {
    int rc = sync();
    if (rc) return rc;
    if (n == 0) return SVDB_OK;
    std::vector<uint64_t> keys(n * 5);
    bool any_empty = false;
    for (size_t i = 0; i < n; ++i) {
        normalize(uuids37 + i * 37, &keys[i * 5]);
        any_empty |= (keys[i * 5] | keys[i * 5 + 1] | keys[i * 5 + 2] | keys[i * 5 + 3] | keys[i * 5 + 4]) == 0;
    }
    const size_t kb = round_up(n * 40, 256), ob = round_up(n * 8, 256);
    rc = scratch_reserve(kb + ob + 256);
    if (!rc) rc = pinned_reserve(std::max(n * 40, n * 8));
    if (rc) return rc;
    uint8_t* base = (uint8_t*)scratch;
    uint64_t* dkeys = (uint64_t*)base;
    int64_t* dout = (int64_t*)(base + kb);
    int* dfirst = (int*)(base + kb + ob);
    std::memcpy(pin, keys.data(), n * 40);
    SVDB_CUDA(cudaMemcpyAsync(dkeys, pin, n * 40, cudaMemcpyHostToDevice, stream));
    SVDB_CUDA(cudaMemsetAsync(dfirst, 0x7f, sizeof(int), stream));
    if (any_empty && slots) {
        k_uuid_first_empty<<<(unsigned)std::min<size_t>((slots + 255) / 256, 2048), 256, 0, stream>>>(
            uid ? uid->rec : nullptr, live, (int64_t)slots, dfirst);
        SVDB_LAUNCH_CHECK();
    }
    const bool indexed = uid && uid->H;
    k_uuid_find<<<(unsigned)((n + 127) / 128), 128, 0, stream>>>(
        dkeys, (int)n, indexed ? uid->rec : nullptr, live, logical, indexed ? uid->tkey : nullptr,
        indexed ? uid->thead : nullptr, indexed ? uid->nslot : nullptr, indexed ? uid->nnext : nullptr,
        indexed ? uid->H : 0, indexed ? uid->nodes : 0, dfirst, dout);
    SVDB_LAUNCH_CHECK();
    SVDB_CUDA(cudaMemcpyAsync(pin, dout, n * 8, cudaMemcpyDeviceToHost, stream));
    SVDB_CUDA(cudaStreamSynchronize(stream));
    std::memcpy(out, pin, n * 8);
    return check_error();
}

// Append n rows given in the reference's file format (host bytes, rows
// `rowbytes` = 45 + 8 dim apart): the raw bytes are copied to the device as
// they are and unpacked there into the master rows and uuid records.
int Store::append_raw(const void* rows, size_t n, size_t rowbytes) {
    int rc = flush();
    if (rc) return rc;
    if (n == 0) return SVDB_OK;
    if (rowbytes != 45 + 8 * dim) {
        svdb_set_error("append_raw: row size %zu does not match dimension %zu", rowbytes, dim);
        return SVDB_EINVAL;
    }
    const size_t first = slots;
    rc = grow(first + n);
    if (rc) return rc;
    if (!uid) {
        uid = new (std::nothrow) UuidIndex();
        if (!uid) {
            svdb_set_error("uuid index: out of host memory");
            return SVDB_ENOMEM;
        }
    }
    rc = uuid_flush();  // earlier staged records first (their slots exist)
    if (rc) return rc;
    const size_t rawb = round_up(n * rowbytes, 256), stb = n * sizeof(UuidStage);
    rc = scratch_reserve(rawb + stb);
    if (!rc) rc = pinned_reserve(n * rowbytes);
    if (rc) return rc;
    uint8_t* draw = (uint8_t*)scratch;
    UuidStage* dst = (UuidStage*)(draw + rawb);
    SVDB_CUDA(cudaStreamSynchronize(stream));  // the pinned buffer is free
    std::memcpy(pin, rows, n * rowbytes);
    SVDB_CUDA(cudaMemcpyAsync(draw, pin, n * rowbytes, cudaMemcpyHostToDevice, stream));
    SVDB_CUDA(cudaMemsetAsync(live + first, 1, n, stream));
    const int64_t work = (int64_t)(n * ld);
    k_unpack_rows<<<(unsigned)std::min<int64_t>((work + 255) / 256, 8192), 256, 0, stream>>>(draw, (int64_t)n, dim, rowbytes,
                                                                                          x64, ld, (int64_t)first, dst);
    SVDB_LAUNCH_CHECK();
    slots += n;
    ++epoch;
    ++version;
    rc = uid_put(this, uid, dst, n);
    if (rc) return rc;
    SVDB_CUDA(cudaStreamSynchronize(stream));
    if (derive_lo < 0 || (int64_t)first < derive_lo) derive_lo = (int64_t)first;
    derive_hi = (int64_t)slots;
    map_dirty = true;
    return SVDB_OK;
}

// rows [first, first + n) back to the host: FP64 rows (n x dim), uuids
// (n x 37 bytes, as the file format stores them) and live flags
int Store::read_block(int64_t first, size_t n, double* rows, char* uuids, uint8_t* lv) {
    int rc = sync();
    if (rc) return rc;
    if (n == 0) return SVDB_OK;
    if (first < 0 || (size_t)first + n > slots) {
        svdb_set_error("read_block: slots [%lld, %lld) out of range", (long long)first, (long long)(first + n));
        return SVDB_EINVAL;
    }
    rc = scratch_reserve(round_up(n * 37, 256));
    if (!rc) rc = pinned_reserve(n * dim * sizeof(double) + n * 37 + n);
    if (rc) return rc;
    uint8_t* hp = (uint8_t*)pin;
    SVDB_CUDA(cudaMemcpy2DAsync(hp, dim * sizeof(double), x64 + first * ld, ld * sizeof(double), dim * sizeof(double), n,
                                cudaMemcpyDeviceToHost, stream));
    k_pack_uuids<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(uid ? uid->rec : nullptr, first, (int64_t)n,
                                                                   (uint8_t*)scratch);
    SVDB_LAUNCH_CHECK();
    SVDB_CUDA(cudaMemcpyAsync(hp + n * dim * sizeof(double), scratch, n * 37, cudaMemcpyDeviceToHost, stream));
    SVDB_CUDA(cudaMemcpyAsync(hp + n * dim * sizeof(double) + n * 37, live + first, n, cudaMemcpyDeviceToHost, stream));
    SVDB_CUDA(cudaStreamSynchronize(stream));
    if (rows) std::memcpy(rows, hp, n * dim * sizeof(double));
    if (uuids) std::memcpy(uuids, hp + n * dim * sizeof(double), n * 37);
    if (lv) std::memcpy(lv, hp + n * dim * sizeof(double) + n * 37, n);
    return SVDB_OK;
}

}  // namespace svdb

using svdb::Store;

extern "C" {

int svdbd_store_set_uuid(svdbd_store* hs, int64_t slot, const char* uuid37) {
    return reinterpret_cast<Store*>(hs)->uuid_set(slot, uuid37);
}

int svdbd_uuid_find(svdbd_store* hs, const char* uuids37, size_t n, int64_t* out_pos) {
    return reinterpret_cast<Store*>(hs)->uuid_find(uuids37, n, out_pos);
}

int svdbd_store_append_raw(svdbd_store* hs, const void* rows, size_t n, size_t rowbytes) {
    return reinterpret_cast<Store*>(hs)->append_raw(rows, n, rowbytes);
}

int svdbd_store_read_block(svdbd_store* hs, int64_t first, size_t n, double* rows, char* uuids37, uint8_t* live) {
    return reinterpret_cast<Store*>(hs)->read_block(first, n, rows, uuids37, live);
}

}  // extern "C"
