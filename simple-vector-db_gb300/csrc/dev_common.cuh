// dev_common.cuh -- helpers shared by the CUDA translation units.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "svdb_device.h"

#define SVDB_CUDA(call)                                                                         \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess) {                                                                \
            svdb_set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
            return e_ == cudaErrorMemoryAllocation ? SVDB_ENOMEM : SVDB_ECUDA;                  \
        }                                                                                       \
    } while (0)

#define SVDB_LAUNCH_CHECK()                                                                    \
    do {                                                                                       \
        cudaError_t e_ = cudaGetLastError();                                                   \
        if (e_ != cudaSuccess) {                                                               \
            svdb_set_error("%s:%d launch: %s", __FILE__, __LINE__, cudaGetErrorString(e_));   \
            return SVDB_ECUDA;                                                                 \
        }                                                                                      \
    } while (0)

namespace svdb {

constexpr int kRowAlign = 16;  // FP64 master row stride: multiple of 16 doubles (128 B)
constexpr int kBf16Align = 64; // BF16 shadow row stride: multiple of 64 (one 128-B swizzle row)

// The BF16 shadows are stored the way the tensor-core screen consumes them:
// tiles of 256 rows x 64 columns (32 KB), the tiles of one 256-row group
// consecutive in column order, each tile in the 128-byte-swizzled layout
// (16-byte chunk c of row r at chunk c ^ (r & 7) of the row's 128 bytes).  A
// screen stage is then one contiguous 32 KB bulk copy, and HBM is read in
// whole tiles rather than 128 bytes from each of 256 rows.  Index of element
// e of row `slot`; ldb is a multiple of 64.
__host__ __device__ inline size_t bf16_tile_index(int64_t slot, size_t e, size_t ldb) {
    const size_t t = (size_t)slot >> 8, r = (size_t)slot & 255u, kb = e >> 6, c = (e >> 3) & 7u, w = e & 7u;
    return (((t * (ldb >> 6) + kb) << 8) + r) * 64u + ((c ^ (r & 7u)) << 3) + w;
}

// The FP8 (E4M3) cosine shadow uses the same tiles in bytes: 256 rows x 128
// elements (one 128-byte swizzle row each), 16-element chunks swizzled; ldb8
// is a multiple of 128.  Byte index of element e of row `slot`.
__host__ __device__ inline size_t f8_tile_index(int64_t slot, size_t e, size_t ldb8) {
    const size_t t = (size_t)slot >> 8, r = (size_t)slot & 255u, kb = e >> 7, c = (e >> 4) & 7u, w = e & 15u;
    return (((t * (ldb8 >> 7) + kb) << 8) + r) * 128u + ((c ^ (r & 7u)) << 4) + w;
}

// Power-of-two scale of the FP8 unit-norm shadow: |x/|x|| <= 1 per element,
// so 256 x/|x| stays inside E4M3's 448 and the key's rescaling is exact.
constexpr double kF8RowScale = 256.0;

static inline size_t round_up(size_t a, size_t b) { return (a + b - 1) / b * b; }

// ---------------------------------------------------------------------------
// Canonical FP64 reductions.  A row is reduced by a group of 4 lanes; lane s
// of the group owns element pairs {8j+2s, 8j+2s+1} and accumulates them in
// increasing order with fused multiply-adds; the group then combines
// (p0+p2)+(p1+p3) with two xor-shuffles.  The oracle restates exactly this
// order, so results are bit-identical.  Rows are zero-padded to a multiple
// of 16 doubles, and fma(0,0,p) == p for the partials (never -0.0), so the
// padding does not change the result.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double group4_sum(double p) {
    p += __shfl_xor_sync(0xffffffffu, p, 2);
    p += __shfl_xor_sync(0xffffffffu, p, 1);
    return p;
}

// The largest f with mx 2^f <= 448 (E4M3's largest finite value), for a
// finite mx > 0, in closed form: mx = r 2^k with r in [0.5, 1) and
// 448 = 0.875 x 2^9, so f = 9 - k when r <= 0.875, else 8 - k.  Exact for
// subnormal mx too (f up to 1082: callers clamp it).
__device__ __forceinline__ int e4m3_fit_exp(double mx) {
    int k;
    const double r = frexp(mx, &k);
    return (r <= 0.875 ? 9 : 8) - k;
}

// ---------------------------------------------------------------------------
// mbarrier and bulk-copy wrappers (sm_100a family)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t gtimer() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// plain bulk copy global -> shared (16-byte aligned, size a multiple of 16)
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
// Bounded wait on phase `parity` of an mbarrier: false when limit_ns of the
// global timer passed first.
__device__ inline bool mbar_wait_for(uint64_t* bar, uint32_t parity, uint64_t limit_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = gtimer();
    for (uint32_t it = 1;; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 31) == 0 && gtimer() - t0 > limit_ns) return false;
    }
}

// ordering key of a metric value: ascending key = better; NaN last
__device__ __forceinline__ double rank_key(int metric, double v) {
    double k = metric == SVDB_EUCLIDEAN ? v : -v;
    return isnan(k) ? __longlong_as_double(0x7ff0000000000000ll) : k;
}

__device__ __forceinline__ bool key_less(double ka, int ia, double kb, int ib) {
    return ka < kb || (ka == kb && ia < ib);
}

// ---------------------------------------------------------------------------
// WarpList<KS>: a warp-wide sorted list of up to 32*KS (key, id, value)
// entries, best first; position p lives in slot p/32 of lane p%32.  All
// calls are warp-uniform.  Empty entries have key +inf and id INT32_MAX.
// ---------------------------------------------------------------------------
template <int KS>
struct WarpList {
    double key[KS];
    double val[KS];
    int id[KS];

    __device__ __forceinline__ void init() {
#pragma unroll
        for (int s = 0; s < KS; ++s) {
            key[s] = __longlong_as_double(0x7ff0000000000000ll);
            val[s] = __longlong_as_double(0x7ff8000000000000ll);
            id[s] = 0x7fffffff;
        }
    }
    // key/id of position p (p < 32*KS), broadcast to all lanes
    __device__ __forceinline__ void at(int p, double& k, int& i) const {
        const int s = p >> 5, l = p & 31;
        double kk = key[0];
        int ii = id[0];
#pragma unroll
        for (int t = 1; t < KS; ++t)
            if (t == s) {
                kk = key[t];
                ii = id[t];
            }
        k = __shfl_sync(0xffffffffu, kk, l);
        i = __shfl_sync(0xffffffffu, ii, l);
    }
    // insert one warp-uniform candidate if it beats position k-1
    __device__ __forceinline__ void insert(double ck, int ci, double cv, int k) {
        double wk;
        int wi;
        at(k - 1, wk, wi);
        if (!key_less(ck, ci, wk, wi)) return;
        const int lane = threadIdx.x & 31;
        int pos = 0;
#pragma unroll
        for (int s = 0; s < KS; ++s) pos += __popc(__ballot_sync(0xffffffffu, key_less(key[s], id[s], ck, ci)));
        double nk[KS], nv[KS];
        int ni[KS];
#pragma unroll
        for (int s = 0; s < KS; ++s) {
            double uk = __shfl_up_sync(0xffffffffu, key[s], 1);
            double uv = __shfl_up_sync(0xffffffffu, val[s], 1);
            int ui = __shfl_up_sync(0xffffffffu, id[s], 1);
            if (s > 0) {
                double pk = __shfl_sync(0xffffffffu, key[s - 1], 31);
                double pv = __shfl_sync(0xffffffffu, val[s - 1], 31);
                int pi = __shfl_sync(0xffffffffu, id[s - 1], 31);
                if (lane == 0) {
                    uk = pk;
                    uv = pv;
                    ui = pi;
                }
            }
            const int p = s * 32 + lane;
            nk[s] = p > pos ? uk : (p == pos ? ck : key[s]);
            nv[s] = p > pos ? uv : (p == pos ? cv : val[s]);
            ni[s] = p > pos ? ui : (p == pos ? ci : id[s]);
        }
#pragma unroll
        for (int s = 0; s < KS; ++s) {
            key[s] = nk[s];
            val[s] = nv[s];
            id[s] = ni[s];
        }
    }
    // threshold key/id at position k-1
    __device__ __forceinline__ void worst(int k, double& wk, int& wi) const { at(k - 1, wk, wi); }
};

}  // namespace svdb
