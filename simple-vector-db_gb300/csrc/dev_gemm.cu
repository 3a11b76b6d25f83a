// dev_gemm.cu -- BF16 tensor-core screen + certified FP64 re-rank (exact top-k).
//
// Stage 1, k_screen_bf16 (the dominant kernel): S = bf16(Q) . bf16(X)^T with
// FP32 accumulation on the 5th-generation tensor cores.  One CTA owns one
// tile of 128 queries (the MMA's M, one TMEM lane per query) and sweeps a
// contiguous range of 256-row store tiles (the MMA's N):
//   warp 0      TMA producer: 128B-swizzled K-major tiles of the BF16 query
//               block and BF16 store shadow, 4-stage mbarrier ring;
//   warp 1      TMEM allocator + MMA issuer: tcgen05.mma kind::f16, M=128,
//               N=256, K=16, into two 256-column FP32 accumulators in TMEM
//               (double buffered, so the epilogue of one row tile overlaps
//               the MMAs of the next);
//   warps 2-9   epilogue: tcgen05.ld of the accumulator (thread = query),
//               screen key + certified error bound per (query, row), the
//               per-query threshold from k shared bins of lower bounds, and
//               emission of every row whose upper bound reaches it.
// The distance matrix never reaches HBM: only candidates are written.
// CTAs are grouped so that all query tiles of a group read the same store
// tile at the same time (one HBM read, the rest L2 hits).
//
// Certification.  For query q and row x with BF16 copies bq, bx:
//   |q.x - fl32(bq.bx)| <= |q|.|x - bx| + |q - bq|.|bx| + c_acc.|bq|.|bx|
// (Cauchy-Schwarz on the quantisation residuals; c_acc bounds the FP32
// accumulation of K products).  The screen key is the metric's ranking
// quantity (cosine: q.x/|x|; dot: q.x; Euclidean: q.x - |x|^2/2, larger is
// better) and E its bound, both in FP32 with directed rounding.  Any row
// whose upper bound key+E is below the k-th largest lower bound key-E over
// the store is strictly worse than k rows, so the candidates that survive
// that test contain the exact FP64 top-k.  E also carries a margin for the
// FP64 rounding of the reported values, so "strictly worse" holds for the
// reported numbers and ties among survivors are resolved by the re-rank.
//
// Stage 2, k_select: per query, exact k-th largest lower bound over the
// candidates (radix select), survivors = upper bound >= it.
// Stage 3, k_rerank: survivors scored in FP64 against the master copy in the
// canonical summation order (bit-identical to the FP64 scan), exact top-k by
// (value, lowest index); the screen bound is re-checked against the exact
// value for every survivor.
// Queries the screen cannot certify (candidate overflow, non-finite or zero
// query, fewer than k finite results, a bound check that failed) are
// answered by the exact FP64 scan instead ("widened").
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstring>
#include <type_traits>
#include <vector>

#include "dev_search.cuh"

#include <cuda_fp8.h>

namespace svdb {

namespace scr {
constexpr int kBM = 128;  // queries per tile (TMEM lanes)
constexpr int kBN = 256;  // store rows per tile (accumulator columns)
constexpr int kBK = 64;   // K per stage: one 128-byte swizzle row of BF16
constexpr int kStages = 4;
// Small batches: a query tile of at most 32 (64) queries stages only those
// rows, and the ring is 6 (5) deep instead of 4.
constexpr int stages_for_rows(int qr) { return qr <= 32 ? 6 : (qr <= 64 ? 5 : kStages); }
constexpr int kEpiWarps = 8;  // two per TMEM lane quadrant, each owning half of the columns
constexpr int kChunk = 16;    // accumulator columns per tcgen05.ld in the epilogue
constexpr int kThreads = 32 * (2 + kEpiWarps);
constexpr uint32_t kTmemCols = 2 * kBN;
constexpr uint32_t kStageA = kBM * kBK * 2;  // 16 KB
constexpr uint32_t kStageB = kBN * kBK * 2;  // 32 KB
constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s: far beyond any legitimate wait
constexpr int kCapMin = 8192, kCapMax = 65536;   // candidates kept per query (adaptive)
constexpr int kSubMin = 4096;                     // slots per sub-list when the budget allows
constexpr int kMaxSub = 1024;                     // sub-lists per query: 2 per segment of its query tile
constexpr int kWarmUnits = kBN / 2 / kChunk;       // chunks one epilogue thread publishes in a warm-up
constexpr int kSurvCap = 8192;                    // survivors re-ranked per query
constexpr size_t kCandBudget = size_t(16) << 30;  // bytes of candidate lists per search (HBM is plentiful)
constexpr float kC2 = 1.9073486328125e-06f;       // 2^-19: FP32 rounding of key and m, per unit of m
// flags
// per query: certified, or why the exact scan answers it (a candidate
// sub-list overflowed, an invalid query, fewer than k finite results, a bound
// that failed against the exact value, more survivors than the select keeps,
// more rows than the FP64 re-rank holds)
constexpr uint8_t kOk = 0, kOverflow = 1, kInvalidQuery = 2, kTooFew = 3, kBoundFail = 4, kSurvOverflow = 5,
                  kRerankOverflow = 6, kRerankLarge = 7;  // (7: between the re-rank's two passes only)
// per search: {candidates, survivors, re-ranked, widened, bound failures,
// widened by candidate overflow, by survivor overflow, by re-rank overflow}
constexpr int kStats = 8;

// Shared memory of one CTA.  PAIR (a CTA pair on two SMs, cta_group::2):
// each CTA holds its own 128 queries and half of the 256-row store tile, so
// a stage is 32 KB instead of 48 KB and the ring is 6 deep.  DUO (two CTAs
// on each SM): a 2-deep ring, so that two CTAs' shared memory fits one SM.
// QR < 128 (a batch of at most QR queries): a stage holds those query rows
// only (4 or 8 KB) and the ring is deeper, so more of the store is in
// flight.  The M = 128 MMA still reads 128 rows from the stage's address:
// rows past QR are whatever follows in shared memory (the next stages), and
// only the accumulator lanes of absent queries, which the epilogue ignores,
// depend on them.
template <bool PAIR, bool DUO = false, int QR = kBM>
struct SmemT {
    static constexpr int ST = PAIR ? 6 : (DUO ? 2 : stages_for_rows(QR));
    static constexpr uint32_t SA = (uint32_t)QR * kBK * 2;
    static constexpr uint32_t SB = PAIR ? kStageB / 2 : kStageB;
    // 1024-byte aligned stage buffers first (SW128 atoms need 1024 B alignment)
    uint8_t a[ST][SA];
    uint8_t b[ST][SB];
    float4 rp[2][kBN];  // screen parameters of the store tile in the accumulator of the same index
    uint64_t rp_full[2];
    uint64_t rp_empty[2];
    uint64_t full[ST];
    uint64_t empty[ST];
    uint64_t accfull[2];
    uint64_t accempty[2];
    uint64_t done;
    uint32_t tmem_base;
    int abort;
};
using Smem = SmemT<false>;
static_assert(Smem::SA == kStageA, "the default stage holds a full 128-query tile");
static_assert(sizeof(SmemT<false, false, 32>) + 1024 <= 232448 && sizeof(SmemT<false, false, 64>) + 1024 <= 232448,
              "the small-batch rings fit the opt-in shared memory");
static_assert(32 * kBK * 2 % 1024 == 0, "SW128 stages start on 1024-byte boundaries");
// DUO: accumulators per CTA (TMEM columns / 256); one, so two CTAs share an SM's 512 columns
template <bool DUO>
constexpr uint32_t tmem_cols() {
    return DUO ? (uint32_t)kBN : kTmemCols;
}
}  // namespace scr

// ---------------------------------------------------------------------------
// PTX wrappers (sm_100a family: tcgen05, TMA, mbarrier)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// Bounded wait: false when the limit ran out or another role raised `abort`.
__device__ __noinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort, uint64_t limit_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = gtimer();
    for (uint32_t it = 1;; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 31) == 0) {
            if (*abort) return false;
            if (gtimer() - t0 > limit_ns) {
                *abort = 1;
                return false;
            }
        }
    }
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
            smem_u32(dst)),
        "l"(map), "r"(smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
}
__device__ __forceinline__ void tma_prefetch_desc(const CUtensorMap* map) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(map) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// D[tmem] (+)= A[smem] . B[smem]^T, both K-major BF16, FP32 accumulate
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// D[tmem] (+)= A[smem] . B[smem]^T, both K-major E4M3 (32 per K step), FP32 accumulate
__device__ __forceinline__ void mma_f8(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                       uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// arrive on `bar` once every tcgen05 op issued so far by this thread has completed
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// ---- CTA pairs (cta_group::2): two CTAs of a cluster on two SMs share one
// MMA of M = 256 (128 queries each) over the whole 256-row store tile, each
// holding half of that tile; one thread of the even CTA issues the MMAs.
__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
// the shared::cluster address of this CTA's shared variable at `a` in CTA `rank`
__device__ __forceinline__ uint32_t cluster_addr(uint32_t a, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
    return r;
}
__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
    asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// arrive on an mbarrier given by its shared::cluster address (this CTA's or the peer's)
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t cbar) {
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(cbar) : "memory");
}
// tiled TMA load into this CTA's shared memory, completing on an mbarrier of
// either CTA of the pair (cbar: shared::cluster address)
__device__ __forceinline__ void tma_load_2d_pair(void* dst, const CUtensorMap* map, uint32_t cbar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, "
        "%4}], [%2];" ::"r"(smem_u32(dst)),
        "l"(map), "r"(cbar), "r"(x), "r"(y)
        : "memory");
}
__device__ __forceinline__ void tmem_alloc_pair(uint32_t* dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc_pair(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void mma_bf16_pair(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                              uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void mma_f8_pair(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                            uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::2.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// arrive on `bar` in both CTAs of the pair once the MMAs issued so far have completed
__device__ __forceinline__ void mma_commit_pair(uint64_t* bar) {
    asm volatile(
        "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(
            smem_u32(bar)),
        "h"((uint16_t)3)
        : "memory");
}
// ... on `bar` of the issuing CTA only
__device__ __forceinline__ void mma_commit_pair_local(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 32 lanes x 32 consecutive FP32 columns: thread t gets columns of its lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
}
// 32 lanes x 16 consecutive FP32 columns
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
// The wait, tied to the registers of the load it completes: the compiler sees
// it redefine them, so no use of them moves above it.
template <int N>
__device__ __forceinline__ void tmem_ld_wait(uint32_t (&r)[N]) {
    tmem_ld_wait();
#pragma unroll
    for (int i = 0; i < N; ++i) asm volatile("" : "+r"(r[i]));
}

// UMMA shared-memory descriptor: K-major, 128-byte swizzle, rows 128 B apart,
// 8-row swizzle atoms 1024 B apart (SBO); LBO unused for this layout.
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(1024u >> 4) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version (sm_100 family)
    d |= (uint64_t)2 << 61;  // SWIZZLE_128B
    return d;
}

// instruction descriptor, kind::f16: BF16 x BF16 -> FP32, both K-major
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
    return (1u << 4)                     // D format: F32
           | (1u << 7)                   // A format: BF16
           | (1u << 10)                  // B format: BF16
           | ((uint32_t)(n >> 3) << 17)  // N / 8
           | ((uint32_t)(m >> 4) << 24); // M / 16
}
// instruction descriptor, kind::f8f6f4: E4M3 x E4M3 -> FP32, both K-major
__host__ __device__ constexpr uint32_t idesc_e4m3(int m, int n) {
    return (1u << 4)                     // D format: F32
           | (0u << 7)                   // A format: E4M3
           | (0u << 10)                  // B format: E4M3
           | ((uint32_t)(n >> 3) << 17)  // N / 8
           | ((uint32_t)(m >> 4) << 24); // M / 16
}

// ---------------------------------------------------------------------------
// shared arithmetic of the certified screen
// ---------------------------------------------------------------------------
// ordered-int image of a float: a < b  <=>  f2ord(a) < f2ord(b) (as signed int)
__device__ __forceinline__ int f2ord(float f) {
    const int b = __float_as_int(f);
    return b >= 0 ? b : b ^ 0x7fffffff;
}
__device__ __forceinline__ float ord2f(int o) { return __int_as_float(o >= 0 ? o : o ^ 0x7fffffff); }

// Error bound of a screen key (FP32, rounded up): E = qn.a + eqq.b + 2^-19.m + eq0
// with row p = {mult, a, b, m} and query {qn, eqq, eq0}.  The FP32 rounding of
// the key itself (<= 2^-22 (|g|.mult + m), |g| <= (1 + c_acc)|bq||bx|) is
// folded into eqq (a multiple of |bq|) and the m term, so E does not depend
// on the key and the epilogue computes it with three FMAs.
__device__ __forceinline__ float screen_bound(float4 p, float qn, float eqq, float eq0) {
    return __fmaf_ru(qn, p.y, __fmaf_ru(eqq, p.z, __fmaf_ru(scr::kC2, p.w, eq0)));
}

// Work of one CTA: up to kMaxSeg segments, each a range of store tiles
// [lo, hi) against one query tile; `sub` numbers the segment among those of
// its query tile (it selects the candidate sub-lists the segment writes).
constexpr int kMaxCtas = 320;  // (two CTAs per SM in the DUO form)
static_assert(2 * kMaxCtas <= scr::kMaxSub, "a query tile split over every CTA has 2 sub-lists per CTA");
constexpr int kMaxSeg = 4;
// grp: the search the segment belongs to (a fused launch screens several at
// once; 0 otherwise); gq: the query tile's index among all the launch's query
// tiles (its segment count is nsq[gq]); qt: the query tile within its search
struct ScreenSeg {
    int32_t lo, hi;
    uint16_t qt, sub, grp, gq;
};
struct ScreenSched {
    ScreenSeg seg[kMaxCtas][kMaxSeg];
    uint8_t nseg[kMaxCtas];
    uint16_t nsq[kMaxCtas];  // segments of query tile gq (the `sub` values 0..nsq-1)
    uint16_t nst[kMaxCtas];  // of those, the ones that start with their CTA (the first nst subs)
    int direct;  // 1: no table; CTA i takes query tile i against every store tile
    int ntr;
};

// `u`: the schedule unit, a CTA (or a CTA pair: both CTAs share the unit's segments)
__device__ __forceinline__ ScreenSeg sched_seg(const ScreenSched& S, int u, int sg) {
    if (S.direct) return ScreenSeg{0, S.ntr, (uint16_t)u, 0, 0, (uint16_t)u};
    return S.seg[u][sg];
}

// everything the screen needs about one search
struct GroupParams {
    const uint8_t* xblk;  // the shadow being screened, in swizzled 256-row x 128-byte tiles (BF16 or E4M3)
    const float* qscale;  // FP8: per query, the exact power of two from accumulator units to key units
    const float4* rpar;  // per row {mult, a, b, m}; NaN rows are never candidates
    const float4* spar;  // per row {mult, b, m, 2^-19 m}: the screen's one-FMA form of the bound
    const int* alpha;    // max over rows of a/b (float bits): |q| a <= |q| alpha b
    const uint32_t* vbits;  // cosine: 1 bit per row (searchable with |x| > 0), whole 256-row tiles
    const int* nmax;        // cosine: {max |x/|x| - bxn|, max |bxn|} over the store (float bits)
    const float4* qpar;  // per query {qn, eqq, eq0, valid}
    int* tau;            // per query: shared lower bound of the k-th best key (ordered int)
    int* bins;           // k bins per query, bin-major (bin t of query q at t * nq + q, so a warp's 32
                         // queries read or raise one bin with one coalesced access): best chunk maximum
                         // of the chunks whose index % k is the bin
    int* cnt;            // per (query, sub-list): candidates emitted, -1 when they overflowed its room
    int* coff;           // per (query, sub-list): where its room starts in the query's list
    int2* cand;          // per query (stride cap): {row slot, key bits} in the sub-lists' rooms (epilogue)
    int* err;            // set to 1 when a wait timed out
    float* dump;         // DUMP (diagnostics) only: raw accumulators, nq x dump_ld
    size_t dump_ld;
    int nq, k, cap;
    int nsub;            // width of cnt / coff: 2 x the most segments of any query tile
                         // (sub-list = (segment, column half): one emitting thread each)
    int ntr;             // store tiles the query tiles' segments cover
    int kblocks;  // ldb / 64
};

// one launch over a single search
struct ScreenParams {
    GroupParams g;
    ScreenSched sched;
};

// A fused launch over several searches (of several stores, dimensions, query
// batches and k): their query tensor maps and
// parameters travel in the launch's own parameter space, and the schedule's
// units are CTAs of any of the searches.
constexpr int kMaxGroups = 16;     // searches in one fused launch
constexpr int kMaxUnitsM = 320;    // CTAs of a fused launch
constexpr int kMaxQTilesM = 640;   // query tiles over all its searches
struct ScreenSchedMulti {
    ScreenSeg seg[kMaxUnitsM][kMaxSeg];
    uint8_t nseg[kMaxUnitsM];
    uint16_t nsq[kMaxQTilesM];
    uint16_t nst[kMaxQTilesM];
    int direct;  // always 0 (every unit has its table row)
    int ntr;
};
struct ScreenParamsMulti {
    CUtensorMap map[kMaxGroups];  // query tensor map of each search (64-byte aligned)
    GroupParams grp[kMaxGroups];
    ScreenSchedMulti sched;
};

// a launch's parameters are limited to 32,764 bytes
static_assert(sizeof(ScreenParamsMulti) + 2 * sizeof(CUtensorMap) <= 32764, "fused launch parameters too large");
static_assert(sizeof(ScreenParams) + 2 * sizeof(CUtensorMap) <= 32764, "screen launch parameters too large");

__device__ __forceinline__ ScreenSeg sched_seg(const ScreenSchedMulti& S, int u, int sg) { return S.seg[u][sg]; }
__device__ __forceinline__ const GroupParams& seg_params(const ScreenParams& P, const ScreenSeg&) { return P.g; }
__device__ __forceinline__ const GroupParams& seg_params(const ScreenParamsMulti& P, const ScreenSeg& sg) {
    return P.grp[sg.grp];
}
__device__ __forceinline__ const CUtensorMap* seg_qmap(const ScreenParams&, const ScreenSeg&, const CUtensorMap* tmq) {
    return tmq;
}
__device__ __forceinline__ const CUtensorMap* seg_qmap(const ScreenParamsMulti& P, const ScreenSeg& sg,
                                                       const CUtensorMap*) {
    return &P.map[sg.grp];
}
template <bool MULTI>
using ScreenParamsT = std::conditional_t<MULTI, ScreenParamsMulti, ScreenParams>;

// NORM (cosine): the B operand is the unit-norm shadow, so the key is the
// accumulator itself and the bound is one constant per query,
//   E = |q| max|x/|x| - bxn| + eqq max|bxn| + eq0;
// the epilogue is a max, a compare and a mask per element, and a validity
// bit per row keeps dead, zero and padding rows out of the lower bounds.
// F8: E4M3 operands, kind::f8f6f4 with 128 elements per stage.  Cosine: the
// accumulator is in units of 2^e times the key (query scale x 256), so
// thresholds are scaled into accumulator units once per tile and emitted
// keys back once per candidate, both exactly (powers of two).  Dot /
// Euclidean: the rows carry their own power of two 2^f_i, so each
// accumulator is scaled into key units (x 2^-e, exact) before the row's
// multiplier 2^-f_i and offset apply, as in the BF16 form.
// DUMP (diagnostics, never used by a search): the epilogue writes every raw
// FP32 accumulator value to P.dump instead of screening, so a test can compare
// the tensor core's accumulation with an exact sum of the same operands.
// PAIR: a cluster of two CTAs (ranks 0, 1) on two SMs works as one unit on
// query tiles of 256 (rank r: queries 128 r .. 128 r + 127).  Each CTA loads
// its own queries and half of the 256-row store tile (rows 128 r ..; through
// the tensor map tmx over the shadow's tiles); the even CTA's MMA thread
// issues cta_group::2 MMAs of M = 256, N = 256 that read both CTAs' halves
// and write each CTA's 128 x 256 accumulator into that CTA's TMEM.  Stage
// completions land on the even CTA's full barriers (it expects both CTAs'
// bytes), MMA completions on both CTAs' empty / accumulator barriers, and
// both CTAs' epilogue warps free an accumulator on the even CTA's barrier.
// Per SM a K step moves 8 KB of operands instead of 12 KB.
// MULTI: a fused launch over several searches (of several stores, dimensions
// and query batches): each segment carries its search (seg.grp), whose
// parameters, shadow, K depth and query tensor map the three roles pick up at
// the segment's start.
// DUO: two CTAs per SM, each with one accumulator (the other CTA's MMAs run
// while this one's epilogue drains it) and a 2-deep ring; twice the epilogue
// warps per SM, for stores whose tiles are a few k blocks deep.
template <bool NORM, bool F8 = false, bool DUMP = false, bool PAIR = false, bool MULTI = false, bool DUO = false,
          int QR = scr::kBM>
__global__ void __launch_bounds__(scr::kThreads, DUO ? 2 : 1)
    k_screen_bf16(const __grid_constant__ CUtensorMap tmq, const __grid_constant__ CUtensorMap tmx,
                  const __grid_constant__ ScreenParamsT<MULTI> P) {
    static_assert(!(MULTI && (PAIR || DUMP)), "a fused launch is single-CTA and screens");
    static_assert(!(DUO && (PAIR || DUMP || MULTI)), "the two-CTA form is a plain screen");
    static_assert(QR == scr::kBM || !(PAIR || DUMP || MULTI || DUO), "the small-batch forms are plain screens");
    using namespace scr;
    using SM = SmemT<PAIR, DUO, QR>;
    constexpr uint32_t TC = tmem_cols<DUO>();
    constexpr int ST = SM::ST;
    // cosine FP8 works in accumulator units (thresholds scaled in, keys out);
    // dot / Euclidean FP8 scales each accumulator into key units at once
    constexpr bool ACCU = F8 && NORM;
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    SM& S = *reinterpret_cast<SM*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t rank = PAIR ? cluster_rank() : 0u;
    const bool leader = rank == 0;
    const int unit = PAIR ? (int)(blockIdx.x >> 1) : (int)blockIdx.x;
    const int nseg = P.sched.direct ? 1 : P.sched.nseg[unit];
    volatile int* abort = &S.abort;

    if (threadIdx.x == 0) {
        for (int i = 0; i < ST; ++i) {
            mbar_init(&S.full[i], 1);
            mbar_init(&S.empty[i], 1);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(&S.accfull[i], 1);
            mbar_init(&S.accempty[i], PAIR ? 2 * kEpiWarps : kEpiWarps);
        }
        mbar_init(&S.done, 1);
        for (int i = 0; i < 2; ++i) {
            mbar_init(&S.rp_full[i], 1);
            mbar_init(&S.rp_empty[i], kEpiWarps);
        }
        S.abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 0 && lane == 0) {
        tma_prefetch_desc(&tmq);
        if (PAIR) tma_prefetch_desc(&tmx);
    }
    // the peer's barriers exist before anything is signalled across the pair
    if constexpr (PAIR) cluster_sync_all();
    if (warp == 1) {
        if constexpr (PAIR)
            tmem_alloc_pair(&S.tmem_base, kTmemCols);  // one warp of each CTA, collectively
        else
            tmem_alloc(&S.tmem_base, TC);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = S.tmem_base;

    if (warp == 0) {
        // ------------------------------------------------------------ producer
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            uint32_t issued = 0;  // loads issued (for draining on abort)
            uint32_t rp_issued = 0;
            bool ok = true;
            uint32_t jt = 0;  // tiles so far (all segments)
            for (int sg = 0; sg < nseg && ok; ++sg) {
            const ScreenSeg seg = sched_seg(P.sched, unit, sg);
            const int qt = seg.qt;
            const GroupParams& GP = seg_params(P, seg);
            const CUtensorMap* tm = seg_qmap(P, seg, &tmq);
            if (MULTI) tma_prefetch_desc(tm);
            const int KB = GP.kblocks;
            for (int r = seg.lo; r < seg.hi && ok; ++r, ++jt) {
                if (!NORM) {  // the tile's screen parameters into the 2-slot ring (freed by the epilogue)
                    const uint32_t slot = jt & 1u;
                    if (!mbar_wait(&S.rp_empty[slot], ((jt >> 1) & 1u) ^ 1u, abort, kWaitLimitNs)) {
                        ok = false;
                        break;
                    }
                    mbar_expect_tx(&S.rp_full[slot], kBN * sizeof(float4));
                    bulk_load(S.rp[slot], GP.spar + (size_t)r * kBN, kBN * sizeof(float4), &S.rp_full[slot]);
                    ++rp_issued;
                }
                for (int kb = 0; kb < KB; ++kb) {
                    if (!mbar_wait(&S.empty[stage], phase ^ 1, abort, kWaitLimitNs)) {
                        ok = false;
                        break;
                    }
                    if constexpr (PAIR) {
                        // both CTAs' halves complete on the even CTA's barrier, which expects them all
                        if (leader) mbar_expect_tx(&S.full[stage], 2 * (SM::SA + SM::SB));
                        const uint32_t fb = cluster_addr(smem_u32(&S.full[stage]), 0);
                        tma_load_2d_pair(S.a[stage], &tmq, fb, kb * (F8 ? 2 * kBK : kBK),
                                         qt * 2 * kBM + (int)rank * kBM);
                        tma_load_2d_pair(S.b[stage], &tmx, fb, 0, (r * KB + kb) * kBN + (int)rank * (kBN / 2));
                    } else {
                        mbar_expect_tx(&S.full[stage], SM::SA + kStageB);  // (QR < 128: a query map of QR-row boxes)
                        tma_load_2d(S.a[stage], tm, &S.full[stage], kb * (F8 ? 2 * kBK : kBK), qt * kBM);
                        // the store tile: one contiguous 32 KB block, already swizzled
                        bulk_load(S.b[stage], GP.xblk + ((size_t)r * KB + kb) * kStageB, kStageB, &S.full[stage]);
                    }
                    ++issued;
                    if (++stage == ST) {
                        stage = 0;
                        phase ^= 1;
                    }
                }
            }
            }
            // every issued load must have landed before the CTA may exit:
            // wait (bounded) for the completion of the last ST loads (a pair's
            // loads all complete on the even CTA's barriers, so it waits for both)
            const uint32_t last = issued < (uint32_t)ST ? issued : (uint32_t)ST;
            volatile int no_abort = 0;
            for (uint32_t i = 0; i < last && (!PAIR || leader); ++i) {
                const uint32_t n = issued - 1 - i;  // load number n went to stage n % S, phase (n / S) & 1
                mbar_wait(&S.full[n % ST], (n / ST) & 1u, &no_abort, kWaitLimitNs / 4);
            }
            const uint32_t rlast = rp_issued < 2u ? rp_issued : 2u;
            for (uint32_t i = 0; i < rlast; ++i) {
                const uint32_t n = rp_issued - 1 - i;
                mbar_wait(&S.rp_full[n & 1u], (n >> 1) & 1u, &no_abort, kWaitLimitNs / 4);
            }
        }
    } else if (warp == 1) {
        // ------------------------------------------------------------ MMA issuer
        if (lane == 0 && (!PAIR || leader)) {
            constexpr int M = PAIR ? 2 * kBM : kBM;
            constexpr uint32_t idesc = F8 ? idesc_e4m3(M, kBN) : idesc_bf16(M, kBN);
            int stage = 0;
            uint32_t phase = 0;
            bool ok = true;
            int j = 0;
            for (int sg = 0; sg < nseg && ok; ++sg) {
            const ScreenSeg sgm = sched_seg(P.sched, unit, sg);
            const int KB = seg_params(P, sgm).kblocks;
            for (int r = sgm.lo, rh = sgm.hi; r < rh && ok; ++r, ++j) {
                const int b = DUO ? 0 : (j & 1);  // accumulator
                const uint32_t use = DUO ? (uint32_t)j : (uint32_t)j >> 1;
                if (!mbar_wait(&S.accempty[b], (use & 1u) ^ 1u, abort, kWaitLimitNs)) break;
                tc_fence_after();
                const uint32_t d = tmem + (uint32_t)(b * kBN);
                for (int kb = 0; kb < KB; ++kb) {
                    if (!mbar_wait(&S.full[stage], phase, abort, kWaitLimitNs)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint64_t ad = sdesc_sw128(smem_u32(S.a[stage]));
                    const uint64_t bd = sdesc_sw128(smem_u32(S.b[stage]));
#pragma unroll
                    for (int kk = 0; kk < kBK / 16; ++kk) {  // +32 bytes per K step (16 BF16 or 32 E4M3)
                        if constexpr (PAIR && F8)
                            mma_f8_pair(d, ad + 2u * kk, bd + 2u * kk, idesc, (kb | kk) != 0);
                        else if constexpr (PAIR)
                            mma_bf16_pair(d, ad + 2u * kk, bd + 2u * kk, idesc, (kb | kk) != 0);
                        else if constexpr (F8)
                            mma_f8(d, ad + 2u * kk, bd + 2u * kk, idesc, (kb | kk) != 0);
                        else
                            mma_bf16(d, ad + 2u * kk, bd + 2u * kk, idesc, (kb | kk) != 0);
                    }
                    if constexpr (PAIR)
                        mma_commit_pair(&S.empty[stage]);  // frees the stage in both CTAs
                    else
                        mma_commit(&S.empty[stage]);
                    if (++stage == ST) {
                        stage = 0;
                        phase ^= 1;
                    }
                }
                if (ok) {
                    if constexpr (PAIR)
                        mma_commit_pair(&S.accfull[b]);
                    else
                        mma_commit(&S.accfull[b]);
                }
            }
            }
            // all MMAs issued by this thread complete before TMEM is released
            if constexpr (PAIR)
                mma_commit_pair_local(&S.done);
            else
                mma_commit(&S.done);
            volatile int no_abort = 0;
            mbar_wait(&S.done, 0, &no_abort, kWaitLimitNs / 4);
        }
    } else {
        // ------------------------------------------------------------ epilogue
        // warp w >= 2: lane quadrant w % 4 (the TMEM lanes it may read), column
        // half (w - 2) / 4; thread = one query of the tile, 128 rows per tile
        const int quad = warp & 3;
        const int half = (warp - 2) >> 2;
        const int qi = quad * 32 + lane;
        const int col0 = half * (kBN / 2);
        int j = 0;  // tiles so far (all segments): accumulator buffer and phase
        bool alive = true;
        // the even CTA's accumulator-free barrier, which both CTAs' epilogues arrive on
        const uint32_t accempty_c0 = PAIR ? cluster_addr(smem_u32(&S.accempty[0]), 0) : 0u;
        for (int sg = 0; sg < nseg && alive; ++sg) {
        // every segment starts afresh: its query tile, threshold, warm-up
        const ScreenSeg seg = sched_seg(P.sched, unit, sg);
        const GroupParams& GP = seg_params(P, seg);
        const int q = PAIR ? seg.qt * 2 * kBM + (int)rank * kBM + qi : seg.qt * kBM + qi;
        float eq = 0.f, eq0 = 0.f;  // screen bound: E = eq . b + 2^-19 m + eq0 (NORM: eq0 = E)
        bool valid = false;
        // F8: key = accumulator x cs, cs a power of two (so both directions are exact)
        float cs = 1.f, ics = 1.f;
        if (F8 && q < GP.nq) {
            cs = GP.qscale[q];
            ics = __frcp_rn(cs);
        }
        if (q < GP.nq) {
            const float4 qp = GP.qpar[q];
            if (NORM) {
                eq0 = __fmaf_ru(qp.x, __int_as_float(__ldg(GP.nmax)),
                                __fmaf_ru(qp.y, __int_as_float(__ldg(GP.nmax + 1)), qp.z));
            } else {
                eq = __fmaf_ru(qp.x, __int_as_float(__ldg(GP.alpha)), qp.y);
                eq0 = qp.z;
            }
            valid = qp.w != 0.f;
        }
        const int nsq = P.sched.direct ? 1 : (int)P.sched.nsq[seg.gq];
        // The query tile's segments that start with their CTAs (nst, subs
        // 0..nst-1) warm up: enough tiles that their warm-up chunks together
        // reach all k bins.  A segment that starts later (a tail a CTA takes
        // after its first segment) finds the bins filled and does not.  Every
        // segment's units cycle through all k bins from its own offset.
        const int nst = P.sched.direct ? 1 : (int)P.sched.nst[seg.gq];
        const bool starter = sg == 0;
        const int nwarm = starter ? max(1, (GP.k + 2 * kWarmUnits * nst - 1) / (2 * kWarmUnits * nst)) : 0;
        const int boff = (int)(((int64_t)seg.sub * GP.k) / (starter ? nst : nsq));
        float tau_c = -INFINITY;  // the query's threshold: shared bins and tau (seed)
        // this thread's own sub-list of the query's candidates: emission needs no
        // atomic, the count stays in a register and is stored once at the end
        const int sub = 2 * seg.sub + half;
        // This sub-list's room in the query's list: half of the list is shared
        // evenly among the query tile's 2 x nsq sub-lists, the other half in
        // proportion to their segments' rows.  A query tile's segments cover
        // its store tiles in `sub` order ([lo, hi) following one another), so
        // the rooms follow one another too.
        const int64_t ntr_all = max(GP.ntr, 1), half_cap = GP.cap / 2;
        const int64_t even = half_cap / (2 * nsq);
        const int64_t pa = half_cap * seg.lo / ntr_all, pb = half_cap * seg.hi / ntr_all, pm = pa + (pb - pa) / 2;
        const int r0 = (int)(even * (2 * seg.sub + half) + (half ? pm : pa));
        const int subcap = (int)(even + (half ? pb - pm : pm - pa));
        int2* cq = GP.cand + (size_t)(q < GP.nq ? q : 0) * GP.cap + r0;
        int nemit = 0;
        for (int r = seg.lo, js = 0; r < seg.hi; ++r, ++j, ++js) {
            const int b = DUO ? 0 : (j & 1);  // accumulator
            const uint32_t use = DUO ? (uint32_t)j : (uint32_t)j >> 1;
            const int rb = j & 1;  // slot of the row-parameter ring (two deep whatever the accumulators)
            const uint32_t ruse = (uint32_t)j >> 1;
            const float4* rps = S.rp[rb] + col0;  // this warp's 128 rows, staged by the producer
            // cosine: validity words of this warp's 128 rows (lane c holds the word
            // of chunk c), loaded before the wait so their latency is hidden
            uint32_t vbl = 0;
            if (NORM && !DUMP && lane < kBN / 2 / 32) vbl = __ldg(GP.vbits + ((r * kBN + col0) >> 5) + lane);
            // Threshold refresh from the shared bins and tau (the 7 tiles after
            // the warm-up, then every 8th): read BEFORE the accumulator wait, so
            // the loads' latency overlaps it instead of stalling the epilogue.
            // Bins and tau only grow (atomicMax of valid lower bounds), so a value
            // read earlier is an older, smaller -- still valid -- threshold.
            // (Warm-up tiles read them after their own contributions, below.)
            const bool refresh = !DUMP && valid && js >= nwarm && (js < nwarm + 7 || (js & 7) == 0);
            int bmin_pre = 0x7fffffff, tau_pre = 0;
            if (refresh) {
                const int* bq = GP.bins + q;
                const size_t bs = (size_t)GP.nq;
                tau_pre = __ldcg(GP.tau + q);
                for (int t0 = 0; t0 < GP.k; t0 += 16) {  // 16 independent loads per round trip
                    int v16[16];
#pragma unroll
                    for (int u = 0; u < 16; ++u) v16[u] = t0 + u < GP.k ? __ldcg(bq + (size_t)(t0 + u) * bs) : 0x7fffffff;
#pragma unroll
                    for (int u = 0; u < 16; ++u) bmin_pre = min(bmin_pre, v16[u]);
                }
            }
            // tcgen05.ld is warp-collective (.sync.aligned): every branch that
            // leads to one must be taken by the whole warp, including this wait
            bool got = mbar_wait(&S.accfull[b], use & 1u, abort, kWaitLimitNs);
            if (!NORM) got = got && mbar_wait(&S.rp_full[rb], ruse & 1u, abort, kWaitLimitNs);
            if (!__all_sync(0xffffffffu, got)) {
                alive = false;
                break;
            }
            tc_fence_after();
            const uint32_t tbase = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(b * kBN + col0);
            const int row0 = r * kBN + col0;
            if constexpr (DUMP) {
#pragma unroll 1
                for (int c = 0; c < kBN / 2 / 32; ++c) {
                    uint32_t v[32];
                    __syncwarp();  // converged warp for the collective load
                    tmem_ld32(tbase + (uint32_t)(c * 32), v);
                    tmem_ld_wait(v);
                    if (q < GP.nq) {
                        float* o = GP.dump + (size_t)q * GP.dump_ld + row0 + c * 32;
#pragma unroll
                        for (int i = 0; i < 32; ++i) o[i] = __uint_as_float(v[i]);
                    }
                }
                tc_fence_before();
                __syncwarp();
                if (lane == 0) {
                    if constexpr (PAIR)
                        mbar_arrive_cluster(accempty_c0 + (uint32_t)(b * sizeof(uint64_t)));
                    else
                        mbar_arrive(&S.accempty[b]);
                    if (!NORM) mbar_arrive(&S.rp_empty[rb]);
                }
                continue;
            }
            if (js < nwarm) {  // warp-uniform: lanes of invalid queries load and discard
                // Warm-up on the segment's first tiles, before they emit: publish
                // the maxima of their 16-row chunks to the bins (one bin per
                // chunk, consecutive from the segment's offset), then read the
                // bins back.  The emitting pass below skips its bin update for
                // these tiles, so no row is counted twice.
#pragma unroll 1
                for (int c = 0; c < kBN / 2 / kChunk; ++c) {
                    uint32_t v[kChunk];
                    __syncwarp();  // converged warp for the collective load
                    tmem_ld16(tbase + (uint32_t)(c * kChunk), v);
                    tmem_ld_wait(v);
                    const float4* rc = rps + c * kChunk;
                    float maxl = -INFINITY;
                    if (NORM) {
                        const int rw = row0 + c * kChunk;
                        const uint32_t vb = __ldg(GP.vbits + (rw >> 5)) >> (rw & 31);
#pragma unroll
                        for (int i = 0; i < kChunk; ++i) {
                            // masked rows are NaN: every comparison with them is false
                            const float l = ((vb >> i) & 1u) ? __fsub_rd(F8 ? __uint_as_float(v[i]) * cs : __uint_as_float(v[i]), eq0) : __int_as_float(0x7fc00000);
                            maxl = fmaxf(maxl, l);
                        }
                    } else {
#pragma unroll
                        for (int i = 0; i < kChunk; ++i) {
                            const float4 p = rc[i];
                            const float key = __fmaf_rn(F8 ? __uint_as_float(v[i]) * cs : __uint_as_float(v[i]), p.x, -p.z);
                            const float l = __fsub_rd(__fsub_rd(key, __fmaf_ru(eq, p.y, p.w)), eq0);
                            maxl = fmaxf(maxl, l);
                        }
                    }
                    if (valid && maxl > -INFINITY)
                        atomicMax(&GP.bins[(size_t)((boff + (js * 2 + half) * kWarmUnits + c) % GP.k) * GP.nq + q],
                                  f2ord(maxl));
                }
            }
            // The k bins hold lower bounds of k distinct rows (chunks of different
            // bins are different rows), so their minimum is a valid threshold; it
            // reflects what every CTA has seen of this query, not only this one.
            if (refresh) {
                tau_c = fmaxf(tau_c, fmaxf(ord2f(tau_pre), ord2f(bmin_pre)));
            } else if (valid && js < nwarm) {  // after the warm-up's own contributions
                const int* bq = GP.bins + q;
                int bmin = 0x7fffffff;
                for (int t = 0; t < GP.k; ++t) bmin = min(bmin, __ldcg(bq + (size_t)t * GP.nq));
                tau_c = fmaxf(tau_c, fmaxf(ord2f(__ldcg(GP.tau + q)), ord2f(bmin)));
            }
            const float thr = valid ? tau_c : INFINITY;  // invalid queries never emit
            // the query's eq0 is folded into the threshold and the maxima
            // in accumulator units (cosine F8: exact rescale by a power of two)
            const float thr2 = ACCU ? __fsub_rd(thr, eq0) * ics : __fsub_rd(thr, eq0);
            constexpr int C = NORM ? 32 : 16;  // accumulator columns per collective load
            constexpr int NC = kBN / 2 / C;    // chunks of this warp's 128 columns
            float tmax = -INFINITY;            // best lower bound (less eq0) of this warp's 128 rows
            auto ld_chunk = [&](int c, uint32_t (&v)[C]) {
                __syncwarp();  // converged warp for the collective load
                if constexpr (C == 32)
                    tmem_ld32(tbase + (uint32_t)(c * C), v);
                else
                    tmem_ld16(tbase + (uint32_t)(c * C), v);
            };
            auto screen_chunk = [&](int c, uint32_t (&v)[C]) {
                const int rw = row0 + c * C;
                const float4* rc = rps + c * C;
                // per 8-column group: best upper bound (less eq0); emission is
                // handled group by group, only where some lane reaches the threshold
                constexpr int G = C / 8;
                float gm[G];
                if (NORM) {
                    // keys are the accumulator values; rows that are not searchable
                    // become NaN (every comparison with NaN is false)
                    const uint32_t vb = __shfl_sync(0xffffffffu, vbl, c);
                    if (vb != 0xFFFFFFFFu) {  // warp-uniform
#pragma unroll
                        for (int i = 0; i < C; ++i)
                            if (!((vb >> i) & 1u)) v[i] = 0x7fc00000u;
                    }
#pragma unroll
                    for (int g = 0; g < G; ++g) {
                        float m = __uint_as_float(v[8 * g]);
#pragma unroll
                        for (int i = 1; i < 8; ++i) m = fmaxf(m, __uint_as_float(v[8 * g + i]));
                        gm[g] = m;
                        tmax = fmaxf(tmax, m);
                    }
                } else {
#pragma unroll
                    for (int g = 0; g < G; ++g) {
                        float m = -INFINITY;
#pragma unroll
                        for (int i = 0; i < 8; ++i) {
                            const float4 p = rc[8 * g + i];
                            const float acc = __uint_as_float(v[8 * g + i]);
                            const float key = __fmaf_rn(F8 ? acc * cs : acc, p.x, -p.z);
                            const float e = __fmaf_ru(eq, p.y, p.w);
                            tmax = fmaxf(tmax, __fsub_rd(key, e));
                            m = fmaxf(m, __fadd_ru(key, e));
                            v[8 * g + i] = __float_as_uint(key);
                        }
                        gm[g] = m;
                    }
                }
                float mu = gm[0];
#pragma unroll
                for (int g = 1; g < G; ++g) mu = fmaxf(mu, gm[g]);
                const bool want = mu >= thr2 && q < GP.nq;
                if (__any_sync(0xffffffffu, want)) {
#pragma unroll
                    for (int g = 0; g < G; ++g) {
                        const bool wg = want && gm[g] >= thr2;
                        if (!__any_sync(0xffffffffu, wg)) continue;  // warp-uniform
                        uint32_t mask = 0;
#pragma unroll
                        for (int i = 0; i < 8; ++i) {
                            const float u = NORM ? __uint_as_float(v[8 * g + i])
                                                 : __fadd_ru(__uint_as_float(v[8 * g + i]),
                                                             __fmaf_ru(eq, rc[8 * g + i].y, rc[8 * g + i].w));
                            mask |= (wg && u >= thr2 ? 1u : 0u) << i;
                        }
                        // each lane stores its own columns, lowest first (the warp
                        // loops as often as its busiest lane has columns); column i
                        // of the group is picked by three selects on i's bits
                        int slot = nemit;
                        nemit += __popc(mask);
                        while (__any_sync(0xffffffffu, mask != 0u)) {
                            if (mask) {
                                const int i = __ffs(mask) - 1;
                                mask &= mask - 1u;
                                const uint32_t a0 = (i & 1) ? v[8 * g + 1] : v[8 * g + 0];
                                const uint32_t a1 = (i & 1) ? v[8 * g + 3] : v[8 * g + 2];
                                const uint32_t a2 = (i & 1) ? v[8 * g + 5] : v[8 * g + 4];
                                const uint32_t a3 = (i & 1) ? v[8 * g + 7] : v[8 * g + 6];
                                const uint32_t b0 = (i & 2) ? a1 : a0;
                                const uint32_t b1 = (i & 2) ? a3 : a2;
                                const uint32_t val = (i & 4) ? b1 : b0;
                                if (slot < subcap)
                                    cq[slot] = make_int2(rw + 8 * g + i,
                                                         ACCU ? __float_as_int(__uint_as_float(val) * cs) : (int)val);
                                ++slot;
                            }
                        }
                    }
                }
            };
#pragma unroll 1
            for (int c = 0; c < NC; ++c) {
                uint32_t v[C];
                ld_chunk(c, v);
                tmem_ld_wait(v);
                screen_chunk(c, v);
            }
            // The tile half's best lower bound goes to one bin (its unit's: the
            // segment's sequence continues after its warm-up chunks).  Any
            // assignment is valid as long as every row unit goes to one bin: the
            // warm-up tiles' rows are already in the bins as chunks and are not
            // published a second time (a row in two bins would make their
            // minimum exceed the k-th best lower bound).
            const float maxl = __fsub_rd(ACCU ? tmax * cs : tmax, eq0);
            if (valid && js >= nwarm && maxl > thr) {
                const int unit = boff + 2 * kWarmUnits * nwarm + (js - nwarm) * 2 + half;
                atomicMax(&GP.bins[(size_t)(unit % GP.k) * GP.nq + q], f2ord(maxl));
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) {
                if constexpr (PAIR)
                    mbar_arrive_cluster(accempty_c0 + (uint32_t)(b * sizeof(uint64_t)));
                else
                    mbar_arrive(&S.accempty[b]);
                if (!NORM) mbar_arrive(&S.rp_empty[rb]);
            }
        }
        if (!DUMP && q < GP.nq) {
            GP.cnt[(size_t)q * GP.nsub + sub] = nemit <= subcap ? nemit : -1;
            GP.coff[(size_t)q * GP.nsub + sub] = r0;
        }
        }
    }

    __syncthreads();
    if (threadIdx.x == 0 && S.abort)  // every search this CTA served
        for (int sg = 0; sg < nseg; ++sg) atomicExch(seg_params(P, sched_seg(P.sched, unit, sg)).err, 1);
    // neither CTA of a pair leaves (or frees TMEM) while the other may still
    // signal its barriers or the MMAs may still read its shared memory
    if constexpr (PAIR) cluster_sync_all();
    if (warp == 1) {
        tc_fence_after();
        if constexpr (PAIR)
            tmem_dealloc_pair(tmem, kTmemCols);
        else
            tmem_dealloc(tmem, TC);
    }
}

// ---------------------------------------------------------------------------
// per-search preparation
// ---------------------------------------------------------------------------
// BF16 copies of the (already padded FP64) queries + per-query bound terms.
// One warp per query: the FP64 pipe is narrow, and with fewer lanes a small
// batch waits on each lane's long chain of dependent FP64 operations.  The
// sums of squares (of the query, of its BF16 copy and of the difference) feed
// only the bounds, whose 1 + 2^-30 factor covers their FP64 rounding in any
// order; the canonical |q|^2 of the reported values is not read here.
constexpr int kPrepLanes = 32;
__global__ void k_prep_bf16(const double* __restrict__ qbuf, int nq, size_t ld,
                            size_t ldb, int metric, __nv_bfloat16* __restrict__ qb, float* __restrict__ q32,
                            float4* __restrict__ qpar) {
    const int lane = threadIdx.x & 31, s = lane;
    const int qi = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const bool active = qi < nq;  // warp-uniform
    double res = 0.0, bsq = 0.0, sqw = 0.0;  // sqw: |q|^2 in this warp's order (bounds only)
    bool finite = true;
    if (active) {
        const double* src = qbuf + (size_t)qi * ld;
        __nv_bfloat16* dst = qb + (size_t)qi * ldb;
        float* dst32 = q32 + (size_t)qi * ld;
        for (size_t j = 2 * s; j < ld; j += 2 * kPrepLanes) {
            const double a = src[j], c = src[j + 1];
            const __nv_bfloat16 ha = __double2bfloat16(a), hc = __double2bfloat16(c);
            const double fa = (double)__bfloat162float(ha), fc = (double)__bfloat162float(hc);
            finite = finite && isfinite(fa) && isfinite(fc);
            bsq = fma(fa, fa, bsq);
            bsq = fma(fc, fc, bsq);
            sqw = fma(a, a, sqw);
            sqw = fma(c, c, sqw);
            res = fma(a - fa, a - fa, res);
            res = fma(c - fc, c - fc, res);
            dst[j] = ha;
            dst[j + 1] = hc;
            *reinterpret_cast<float2*>(dst32 + j) = make_float2(__double2float_rn(a), __double2float_rn(c));
        }
        for (size_t j = ld + 2 * s; j < ldb; j += 2 * kPrepLanes) {
            dst[j] = __float2bfloat16(0.0f);
            dst[j + 1] = __float2bfloat16(0.0f);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        res += __shfl_xor_sync(0xffffffffu, res, o);
        bsq += __shfl_xor_sync(0xffffffffu, bsq, o);
        sqw += __shfl_xor_sync(0xffffffffu, sqw, o);
    }
    const unsigned all_finite = __all_sync(0xffffffffu, finite);  // the warp is the query
    if (active && s == 0) {
        // an upper bound of |q|^2 (the canonical |q|^2 of the reported values
        // may still be in flight on another stream)
        const double up = 1.0 + 9.313225746154785e-10;  // 1 + 2^-30: FP64 rounding of the sums
        const double sq = sqw * up;
        const double qn = sqrt(sq) * up;
        const double eq = sqrt(res) * up;
        const double bqn = sqrt(bsq) * up;
        // FP32 accumulation of K = ldb products in K/16 tensor-core steps
        const double cacc = (double)(ldb / 16 + 1) * 20.0 * 1.1920928955078125e-07;
        // quantisation + accumulation, FP64 rounding of the reported value (2^-38 qn),
        // and the FP32 rounding of the key (2^-20 (1 + c_acc) 1.02 |bq|, see screen_bound)
        const double eqq = (eq + cacc * bqn) * (1.0 + 9.5367431640625e-07) + 3.637978807091713e-12 * qn +
                           9.5367431640625e-07 * (1.0 + cacc) * 1.02 * bqn;
        // FP64 rounding of the reported value (2^-40 of its scale) + an absolute floor for FP32 underflow
        const double eq0 = 9.094947017729282e-13 * (metric == SVDB_EUCLIDEAN ? sq : qn) + 1e-30;
        // |q| < 1e15 keeps every BF16 product and FP32 sum far from overflow (rows are held to the same)
        const bool ok = all_finite && isfinite(sq) && sq < 1e30 && (metric != SVDB_COSINE || sq > 0.0);
        float4 p;
        p.x = __double2float_ru(qn);
        p.y = __double2float_ru(eqq);
        p.z = __double2float_ru(eq0);
        p.w = ok && isfinite(p.x) && isfinite(p.y) ? 1.0f : 0.0f;
        qpar[qi] = p;
    }
}

// The FP8 form of k_prep_bf16: the query scaled by a power of two 2^e (the
// largest with max |q_i| 2^e <= 448, E4M3's largest finite value), its E4M3
// copy (nq x ldb8 bytes, zero padded), the FP32 copy for the refinement, the
// bound terms and qscale: cosine 2^-(e+8), key = accumulator x qscale exactly
// (the unit-norm shadow carries 256 x/|x|); dot / Euclidean 2^-e, key =
// accumulator x qscale x 2^-f_i - m_i with the row's own power of two (the
// plain E4M3 shadow carries x 2^f_i).  The tensor core's
// accumulation of E4M3 products is modelled pessimistically, as if each K=32
// step kept only 13 bits: c_acc = (ldb8/32 + 1) x 40 x 2^-13 of |bq| |bx|
// (for D = 768 about 0.12; the E4M3 rounding itself is ~0.04 per vector).
__global__ void k_prep_f8(const double* __restrict__ qbuf, int nq, size_t ld,
                          size_t ldb8, int metric, uint8_t* __restrict__ q8, float* __restrict__ q32,
                          float4* __restrict__ qpar, float* __restrict__ qscale) {
    const int lane = threadIdx.x & 31, s = lane;  // one warp per query, as k_prep_bf16
    const int qi = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const bool active = qi < nq;  // warp-uniform
    const double* src = qbuf + (size_t)(active ? qi : 0) * ld;
    double m = 0.0;
    bool finite = true;
    if (active)
        for (size_t j = s; j < ld; j += kPrepLanes) {
            const double a = src[j];
            finite = finite && isfinite(a);
            m = fmax(m, fabs(a));
        }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    int e = 0;
    if (m > 0.0 && isfinite(m)) {
        e = max(-126, min(126, e4m3_fit_exp(m)));  // |e| >= 100 marks the query invalid below
    }
    const double sc = ldexp(1.0, e);
    double res = 0.0, bsq = 0.0, sqw = 0.0;  // sqw: |q|^2 in this warp's order (bounds only)
    if (active) {
        uint8_t* dst = q8 + (size_t)qi * ldb8;
        float* dst32 = q32 + (size_t)qi * ld;
        for (size_t j = 2 * s; j < ld; j += 2 * kPrepLanes) {
            const double a = src[j], c = src[j + 1];
            const __nv_fp8_storage_t ea = __nv_cvt_double_to_fp8(a * sc, __NV_SATFINITE, __NV_E4M3);
            const __nv_fp8_storage_t ec = __nv_cvt_double_to_fp8(c * sc, __NV_SATFINITE, __NV_E4M3);
            const double fa = (double)__half2float(__half(__nv_cvt_fp8_to_halfraw(ea, __NV_E4M3))) / sc;
            const double fc = (double)__half2float(__half(__nv_cvt_fp8_to_halfraw(ec, __NV_E4M3))) / sc;
            bsq = fma(fa, fa, bsq);
            bsq = fma(fc, fc, bsq);
            sqw = fma(a, a, sqw);
            sqw = fma(c, c, sqw);
            res = fma(a - fa, a - fa, res);
            res = fma(c - fc, c - fc, res);
            dst[j] = ea;
            dst[j + 1] = ec;
            *reinterpret_cast<float2*>(dst32 + j) = make_float2(__double2float_rn(a), __double2float_rn(c));
        }
        for (size_t j = ld + 2 * s; j < ldb8; j += 2 * kPrepLanes) {
            dst[j] = 0;
            dst[j + 1] = 0;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        res += __shfl_xor_sync(0xffffffffu, res, o);
        bsq += __shfl_xor_sync(0xffffffffu, bsq, o);
        sqw += __shfl_xor_sync(0xffffffffu, sqw, o);
    }
    const unsigned all_finite = __all_sync(0xffffffffu, finite);
    if (active && s == 0) {
        const double up = 1.0 + 9.313225746154785e-10;
        const double sq = sqw * up;  // an upper bound of |q|^2, as in k_prep_bf16
        const double qn = sqrt(sq) * up;
        const double eq = sqrt(res) * up;
        const double bqn = sqrt(bsq) * up;
        const double cacc = (double)(ldb8 / 32 + 1) * 40.0 * 1.220703125e-04;
        const double eqq = (eq + cacc * bqn) * (1.0 + 9.5367431640625e-07) + 3.637978807091713e-12 * qn +
                           9.5367431640625e-07 * (1.0 + cacc) * 1.02 * bqn;
        const double eq0 = 9.094947017729282e-13 * (metric == SVDB_EUCLIDEAN ? sq : qn) + 1e-30;
        // the key's rescale 2^-(e+8) (cosine: the rows carry 256 x/|x|) or 2^-e
        // (dot / Euclidean: the rows' own scale is applied per row) stays a
        // normal FP32 power of two
        const bool ok = all_finite && isfinite(sq) && sq < 1e30 && (metric != SVDB_COSINE || sq > 0.0) && e > -100 &&
                        e < 100;
        float4 p;
        p.x = __double2float_ru(qn);
        p.y = __double2float_ru(eqq);
        p.z = __double2float_ru(eq0);
        p.w = ok && isfinite(p.x) && isfinite(p.y) ? 1.0f : 0.0f;
        qpar[qi] = p;
        qscale[qi] = (float)ldexp(1.0, -(e + (metric == SVDB_COSINE ? 8 : 0)));
    }
}

// Per-row screen parameters for one metric; rows >= nslots (tile padding),
// dead slots and placeholder rows get NaN (never candidates).  rowp8 (dot /
// Euclidean on the E4M3 shadow): the rows' own power-of-two multiplier and
// the E4M3 residual and norm replace the BF16 ones.
//   rpar = {mult, a, b, m}: the tight bound E = |q| a + eqq b + 2^-19 m + eq0
//   spar = {mult, b, m, 2^-19 m}: the screen's one-FMA form, with a <= alpha b
//   vbits: 1 bit per row whose parameters are finite (the cosine screen's mask)
// alpha = max over rows of a / b (float bits, one atomic per block).  A row with
// b = 0 has a = 0; rows where that fails are unscreenable and never reach here.
// Cosine runs on the unit-norm shadow: key = q . x/|x|, a = |x/|x| - bxn|,
// b = |bxn| (zero rows: NaN, their cosine is NaN and ranks last).
__global__ void __launch_bounds__(256) k_row_params(const float4* __restrict__ rowp, const double* __restrict__ sq64,
                                                    const uint8_t* __restrict__ live, int64_t nslots, int64_t npad,
                                                    int metric, const float2* __restrict__ rowpn,
                                                    const float4* __restrict__ rowp8, float4* __restrict__ rpar,
                                                    float4* __restrict__ spar, int* __restrict__ alpha,
                                                    uint32_t* __restrict__ vbits) {
    __shared__ int wmax[8];
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const float nan = __int_as_float(0x7fc00000);
    float4 out = make_float4(nan, nan, nan, nan);
    if (i < nslots && live[i] == 1) {
        const float4 rp = rowp[i];  // {|x| up, |bx| up, |x - bx| up, |x|^2/2}
        const double sq = sq64[i];
        if (metric == SVDB_COSINE) {
            if (sq > 0.0) {
                const float2 pn = rowpn[i];
                out = make_float4(1.0f, pn.y, pn.x, 0.0f);
            }
        } else if (rowp8) {  // the E4M3 shadow x 2^f: mult = 2^-f, a and b of its residual and norm
            const float4 p8 = rowp8[i];
            out = make_float4(p8.z, p8.y, p8.x, metric == SVDB_DOT ? 0.0f : __double2float_rn(0.5 * sq));
        } else if (metric == SVDB_DOT) {
            out = make_float4(1.0f, rp.z, rp.y, 0.0f);
        } else {
            out = make_float4(1.0f, rp.z, rp.y, __double2float_rn(0.5 * sq));
        }
    }
    float ratio = 0.f;
    if (i < npad) {
        rpar[i] = out;
        spar[i] = make_float4(out.x, out.z, out.w, out.w * scr::kC2);
        if (out.z > 0.f) ratio = __fdiv_ru(out.y, out.z);
    }
    const unsigned vb = __ballot_sync(0xffffffffu, !isnan(out.x));
    if ((threadIdx.x & 31) == 0 && i < npad) vbits[i >> 5] = vb;  // npad is a multiple of 256
    int r = __reduce_max_sync(0xffffffffu, __float_as_int(ratio));  // ratio >= 0: int order = float order
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = r;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) r = max(r, wmax[w]);
        r = max(r, wmax[0]);
        if (r > 0) atomicMax(alpha, r);
    }
}

// seed (optional): a valid lower bound of each query's k-th best key, the
// running threshold's starting value
__global__ void k_init_search(int* tau, int* bins, int* cnt, int nsub, uint8_t* flags, int nq, int k, int* alpha,
                              int* redo_n, unsigned long long* stats, const float* seed = nullptr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nq) {
        tau[i] = f2ord(seed ? seed[i] : -INFINITY);
        for (int t = 0; t < k; ++t) bins[(size_t)t * nq + i] = f2ord(-INFINITY);  // bin-major
        for (int t = 0; t < nsub; ++t) cnt[(size_t)i * nsub + t] = 0;
        flags[i] = scr::kOk;
    }
    if (i == 0) {
        *alpha = 0;
        *redo_n = 0;
    }
    if (i < scr::kStats) stats[i] = 0;
}

// ---------------------------------------------------------------------------
// stage 2: k-th largest lower bound over the candidates; survivors = upper
// bound >= it, copied to the per-query survivor list
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t f2u_ord(float f) {
    const uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

// k-th largest of m ordered values get(i) (every thread of the block calls
// it): four 8-bit radix passes with a shared histogram.  Each thread keeps
// U loads in flight; warp 0 finds each pass's digit with a scan over the
// lanes (lane l holds the counts of digits 255 - 8l .. 248 - 8l, largest
// first), so no thread walks the 256 bins alone.
template <int U = 4, class Get>
__device__ uint32_t block_kth_largest(Get get, int m, int k, int* hist, uint32_t* sh) {
    if (threadIdx.x == 0) {
        sh[0] = 0;  // prefix
        sh[1] = 0;  // mask
        sh[2] = (uint32_t)k;
    }
    __syncthreads();
    const int nt = blockDim.x;
    for (int shift = 24; shift >= 0; shift -= 8) {
        for (int i = threadIdx.x; i < 256; i += nt) hist[i] = 0;
        __syncthreads();
        const uint32_t pre = sh[0], msk = sh[1];
        int i = threadIdx.x;
        for (; i + (U - 1) * nt < m; i += U * nt) {
            uint32_t v[U];
#pragma unroll
            for (int u = 0; u < U; ++u) v[u] = get(i + u * nt);
#pragma unroll
            for (int u = 0; u < U; ++u)
                if ((v[u] & msk) == pre) atomicAdd(&hist[(v[u] >> shift) & 255u], 1);
        }
        for (; i < m; i += nt) {
            const uint32_t v = get(i);
            if ((v & msk) == pre) atomicAdd(&hist[(v >> shift) & 255u], 1);
        }
        __syncthreads();
        if (threadIdx.x < 32) {
            const int lane = threadIdx.x;
            const int need = (int)sh[2];
            int c[8], sum = 0;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                c[j] = hist[255 - 8 * lane - j];
                sum += c[j];
            }
            int incl = sum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            const int total = __shfl_sync(0xffffffffu, incl, 31);
            const int excl = incl - sum;
            // the lane whose digits take the running count from below `need` to it
            const unsigned hit = __ballot_sync(0xffffffffu, excl < need && incl >= need);
            if (lane == (hit ? __ffs(hit) - 1 : 0)) {
                int cum = total, dsel = 0;  // fewer than `need` values: digit 0, as a full walk ends
                if (hit) {
                    cum = excl;
                    for (int j = 0; j < 8; ++j) {
                        dsel = 255 - 8 * lane - j;
                        if (cum + c[j] >= need) break;
                        cum += c[j];
                    }
                }
                sh[2] = (uint32_t)(need - cum);
                sh[0] = pre | ((uint32_t)dsel << shift);
                sh[1] = msk | (255u << shift);
            }
        }
        __syncthreads();
    }
    return sh[0];
}

// ---------------------------------------------------------------------------
// stage 1 for one or two cosine queries: CUDA cores stream the unit-norm
// BF16 shadow (a 128-query tensor tile would be 1/128 used).  Measured on
// 1M x 768: one query 0.47 ms per search, two 0.486 ms, against 0.58 ms
// through the tensor-core screen; at four queries the FMAs made it slower
// (screen stage 0.53 ms against ~0.42 ms), so batches of three or more take
// the tensor cores.
// ---------------------------------------------------------------------------
// The key is the same BF16 dot product bq . bxn as the tensor-core screen's,
// summed in FP32 by FMAs: the products of BF16 values are exact, and each
// lane adds KB x 8 of them before a 3-step shuffle tree, so its rounding is
// below (8 KB + 3) 2^-24 |bq| |bxn| -- far inside the tensor-core
// accumulation term of the screen bound (cacc |bq| |bxn|, cacc = 20 (ldb/16
// + 1) 2^-23), so that bound, and everything after the screen, hold as they
// are.  Three kernels: keys and per-tile maxima; per query the k-th largest
// tile maximum (tiles are disjoint, so k tile maxima are keys of k distinct
// rows: a valid lower bound of the k-th best key); then every row whose upper
// bound reaches the k-th lower bound is a candidate.
constexpr int kStreamQ = 2;               // queries per streamed search, at most
constexpr int kStreamWarps = 8;           // warps per store tile (rows 32w .. 32w+31)
constexpr int kStreamQBytes = 32 * 1024;  // query values (FP32) in shared memory

size_t stream_smem(size_t nq, size_t ldb) { return nq * ldb * sizeof(float); }

// One block per 256-row store tile, reading the tile's 32 KB blocks (256
// rows x one 128-byte k block, as stored for the tensor-core screen) whole
// and in order: warp w takes rows 32w .. 32w+31, four at a time (8 lanes per
// row, one 16-byte chunk each), 16 loads in flight per lane.  Plain vector
// loads from many resident blocks stream HBM faster here than a bulk-copy
// ring: on 1M x 768 the screen stage takes 0.345 ms, against 0.371 ms with
// one CTA per SM keeping six 32 KB bulk copies in flight.  Keys go
// to keys[q][slot]; each warp's maximum over its 32 rows of a tile to
// wmax[q][tile * 8 + warp] (disjoint rows: k of them bound the k-th best key).
template <int QN>
__global__ void __launch_bounds__(32 * kStreamWarps)
    k_stream_keys(const uint8_t* __restrict__ xbn, int KB, const __nv_bfloat16* __restrict__ qb, size_t ldb, int nq,
                  const uint32_t* __restrict__ vbits, size_t npad, int ntr, float* __restrict__ keys,
                  float* __restrict__ wmax) {
    extern __shared__ float s_q[];  // nq x K query values (BF16 -> FP32 is exact)
    const int K = KB * 64;
    for (int i = threadIdx.x; i < nq * K; i += blockDim.x) {
        const int qi = i / K;
        s_q[i] = __bfloat162float(qb[(size_t)qi * ldb + (i - qi * K)]);
    }
    __syncthreads();
    const int t = blockIdx.x, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g8 = lane & 7, rsub = lane >> 3;
    // the 128-byte swizzle: granule g8 of a row r holds chunk g8 ^ (r & 7); the
    // rows of step s are 32 warp + 4 s + rsub, so r & 7 = rsub (even s) or rsub + 4
    const int ce = g8 ^ rsub, co = g8 ^ (rsub + 4);
    const uint8_t* src = xbn + ((size_t)t * KB * 256 + warp * 32 + rsub) * 128 + g8 * 16;
    float acc[8][QN];
#pragma unroll
    for (int s = 0; s < 8; ++s)
#pragma unroll
        for (int qi = 0; qi < QN; ++qi) acc[s][qi] = 0.f;
    auto fold = [&](const uint4 (&v)[8], int kb) {
#pragma unroll
        for (int qi = 0; qi < QN; ++qi) {
            if (qi < nq) {
                const float* qq = s_q + (size_t)qi * K + kb * 64;
                const float4 e0 = *reinterpret_cast<const float4*>(qq + ce * 8);
                const float4 e1 = *reinterpret_cast<const float4*>(qq + ce * 8 + 4);
                const float4 o0 = *reinterpret_cast<const float4*>(qq + co * 8);
                const float4 o1 = *reinterpret_cast<const float4*>(qq + co * 8 + 4);
#pragma unroll
                for (int s = 0; s < 8; ++s) {
                    const float4 a = (s & 1) ? o0 : e0, b = (s & 1) ? o1 : e1;
                    float r = acc[s][qi];
                    r = __fmaf_rn(__uint_as_float(v[s].x << 16), a.x, r);
                    r = __fmaf_rn(__uint_as_float(v[s].x & 0xffff0000u), a.y, r);
                    r = __fmaf_rn(__uint_as_float(v[s].y << 16), a.z, r);
                    r = __fmaf_rn(__uint_as_float(v[s].y & 0xffff0000u), a.w, r);
                    r = __fmaf_rn(__uint_as_float(v[s].z << 16), b.x, r);
                    r = __fmaf_rn(__uint_as_float(v[s].z & 0xffff0000u), b.y, r);
                    r = __fmaf_rn(__uint_as_float(v[s].w << 16), b.z, r);
                    r = __fmaf_rn(__uint_as_float(v[s].w & 0xffff0000u), b.w, r);
                    acc[s][qi] = r;
                }
            }
        }
    };
    int kb = 0;
    for (; kb + 1 < KB; kb += 2) {  // two k blocks (16 loads) in flight
        uint4 v0[8], v1[8];
#pragma unroll
        for (int s = 0; s < 8; ++s) {
            v0[s] = __ldcs(reinterpret_cast<const uint4*>(src + (size_t)kb * 32768 + s * 512));
            v1[s] = __ldcs(reinterpret_cast<const uint4*>(src + (size_t)(kb + 1) * 32768 + s * 512));
        }
        fold(v0, kb);
        fold(v1, kb + 1);
    }
    if (kb < KB) {
        uint4 v0[8];
#pragma unroll
        for (int s = 0; s < 8; ++s) v0[s] = __ldcs(reinterpret_cast<const uint4*>(src + (size_t)kb * 32768 + s * 512));
        fold(v0, kb);
    }
    const uint32_t vw = __ldg(vbits + (((size_t)t * 256 + warp * 32) >> 5));  // this warp's 32 rows
    float m[QN];
#pragma unroll
    for (int qi = 0; qi < QN; ++qi) m[qi] = -INFINITY;
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        const int rw = s * 4 + rsub;  // row within the warp's 32
        const bool valid = (vw >> rw) & 1u;
        const size_t slot = (size_t)t * 256 + warp * 32 + rw;
#pragma unroll
        for (int qi = 0; qi < QN; ++qi) {
            float a = acc[s][qi];
            a = __fadd_rn(a, __shfl_xor_sync(0xffffffffu, a, 1));
            a = __fadd_rn(a, __shfl_xor_sync(0xffffffffu, a, 2));
            a = __fadd_rn(a, __shfl_xor_sync(0xffffffffu, a, 4));
            if (qi < nq) {
                if (g8 == 0) keys[(size_t)qi * npad + slot] = valid ? a : __int_as_float(0x7fc00000);
                if (valid) m[qi] = fmaxf(m[qi], a);
            }
        }
    }
#pragma unroll
    for (int qi = 0; qi < QN; ++qi) {
        float x = m[qi];
        for (int o = 16; o > 0; o >>= 1) x = fmaxf(x, __shfl_xor_sync(0xffffffffu, x, o));
        if (lane == 0 && qi < nq) wmax[(size_t)qi * ntr * kStreamWarps + (size_t)t * kStreamWarps + warp] = x;
    }
}

// per query: the candidate cut = (k-th largest warp maximum - E) - E, E the
// query's bound over every row (the screen's cosine eq0), rounded down
__global__ void __launch_bounds__(1024) k_stream_cut(const float* __restrict__ tmax, int ntr, int k,
                                                    const float4* __restrict__ qpar, const int* __restrict__ nmax,
                                                    float* __restrict__ cut) {
    __shared__ int hist[256];
    __shared__ uint32_t sh[3];
    const int q = blockIdx.x;
    const float* t = tmax + (size_t)q * ntr;
    const uint32_t u = ntr >= k ? block_kth_largest([&](int i) { return f2u_ord(t[i]); }, ntr, k, hist, sh)
                                : f2u_ord(-INFINITY);
    if (threadIdx.x == 0) {
        const float4 qp = qpar[q];
        const float kth = __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
        const float e = __fmaf_ru(qp.x, __int_as_float(__ldg(nmax)), __fmaf_ru(qp.y, __int_as_float(__ldg(nmax + 1)), qp.z));
        cut[q] = qp.w != 0.f ? __fsub_rd(__fsub_rd(kth, e), e) : INFINITY;  // invalid queries: no candidates
    }
}

// every row whose key reaches the cut, into the query's single candidate list
__global__ void __launch_bounds__(256) k_stream_emit(const float* __restrict__ keys, size_t npad, int nq,
                                                     const float* __restrict__ cut, int cap, int* __restrict__ cnt,
                                                     int2* __restrict__ cand) {
    const size_t row = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    for (int qi = 0; qi < nq; ++qi) {
        const float key = row < npad ? keys[(size_t)qi * npad + row] : __int_as_float(0x7fc00000);
        const bool want = key >= __ldg(cut + qi);  // NaN rows never
        const uint32_t m = __ballot_sync(0xffffffffu, want);
        if (!m) continue;
        int base = 0;
        if (lane == 0) base = atomicAdd(cnt + qi, __popc(m));
        base = __shfl_sync(0xffffffffu, base, 0);
        const int slot = base + __popc(m & ((1u << lane) - 1u));
        if (want && slot < cap) cand[(size_t)qi * cap + slot] = make_int2((int)row, __float_as_int(key));
    }
}

// Pass 1: a radix select over the candidates' lower bounds gives the exact
// k-th largest.  Pass 2: survivors.
//
// The query's candidates sit in nsub sub-lists (one per emitting thread of the
// screen, each at its own offset in the query's list); candidate i of the
// concatenation is found by a binary search over the exclusive prefix of the
// sub-list counts (shared memory).
// coff null: one list (the streamed screen's), room cap.
__global__ void __launch_bounds__(1024) k_select(const int2* __restrict__ cand, const int* __restrict__ cnt,
                                                 const int* __restrict__ coff, int cap, int nsub,
                                                 const float4* __restrict__ rpar,
                                                 const float4* __restrict__ qpar, int k, int2* __restrict__ surv,
                                                 int* __restrict__ nsurv, int* __restrict__ sig,
                                                 uint8_t* __restrict__ flags, float* __restrict__ kth_out = nullptr) {
    __shared__ int hist[256];
    __shared__ uint32_t s_sh[3];
    __shared__ int s_out, s_sig, s_over;
    __shared__ int s_pre[scr::kMaxSub + 1];
    __shared__ int s_off[scr::kMaxSub];
    const int q = blockIdx.x;
    const float4 qp = qpar[q];
    if (threadIdx.x < 32) {  // warp 0: prefix of the sub-list counts
        const int lane = threadIdx.x;
        int run = 0;
        bool over = false;
        for (int s0 = 0; s0 < nsub; s0 += 32) {
            const int s = s0 + lane;
            int c = s < nsub ? cnt[(size_t)q * nsub + s] : 0;
            over = over || (coff ? c < 0 : c > cap);
            if (c < 0) c = 0;
            if (s < nsub) s_off[s] = coff ? coff[(size_t)q * nsub + s] : 0;
            int incl = c;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            if (s < nsub) s_pre[s] = run + incl - c;
            run += __shfl_sync(0xffffffffu, incl, 31);
        }
        over = __any_sync(0xffffffffu, over);
        if (lane == 0) {
            s_pre[nsub] = run;
            s_over = over ? 1 : 0;
        }
    }
    __syncthreads();
    const int n = s_pre[nsub];
    if (qp.w == 0.f || s_over) {
        if (kth_out) {  // seed mode: no usable lower bound
            if (threadIdx.x == 0) kth_out[q] = -INFINITY;
            return;
        }
        if (threadIdx.x == 0) {
            flags[q] = qp.w == 0.f ? scr::kInvalidQuery : scr::kOverflow;
            nsurv[q] = 0;
            sig[q] = 0x7fffffff;
        }
        return;
    }
    const int2* cbase = cand + (size_t)q * cap;
    auto at = [&](int i) {  // the largest sub-list s with prefix <= i holds candidate i
        int lo = 0, hi = nsub - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (s_pre[mid] <= i)
                lo = mid;
            else
                hi = mid - 1;
        }
        return cbase[(size_t)s_off[lo] + (i - s_pre[lo])];
    };
    const int bd = blockDim.x;
    auto lower = [&](int i) {
        const int2 c = at(i);
        return f2u_ord(__fsub_rd(__int_as_float(c.y), screen_bound(__ldg(rpar + c.x), qp.x, qp.y, qp.z)));
    };
    if (threadIdx.x == 0) {
        s_out = 0;
        s_sig = 0x7fffffff;
    }
    uint32_t thr_ord = 0;  // fewer than k candidates: every one survives
    __syncthreads();
    if (n >= k) thr_ord = block_kth_largest<2>(lower, n, k, hist, s_sh);  // a binary search per value: two in flight
    if (kth_out) {  // seed mode: the exact k-th largest lower bound over these candidates, nothing else
        if (threadIdx.x == 0) {
            const uint32_t u = thr_ord;
            kth_out[q] = n >= k ? __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u) : -INFINITY;
        }
        return;
    }
    int2* sq = surv + (size_t)q * scr::kSurvCap;
    for (int i = threadIdx.x; i < n; i += bd) {
        const int2 c = at(i);
        const float U = __fadd_ru(__int_as_float(c.y), screen_bound(__ldg(rpar + c.x), qp.x, qp.y, qp.z));
        if (!isnan(U) && f2u_ord(U) >= thr_ord) {  // rows with NaN parameters never survive
            const int o = atomicAdd(&s_out, 1);
            if (o < scr::kSurvCap) sq[o] = c;
            atomicMin(&s_sig, c.x);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        sig[q] = s_sig;
        nsurv[q] = s_out;
        if (s_out > scr::kSurvCap) flags[q] = scr::kSurvOverflow;
    }
}

// Order of the refinement blocks: queries sorted by their survivor signature
// (smallest surviving row), so queries that share their survivors -- near-tie
// clusters -- are refined by blocks that run at the same time and hit each
// other's rows in L2.  One block, bitonic sort of (signature, query) in shared
// memory; n is a power of two >= nq (pad keys sort last).
__global__ void __launch_bounds__(1024) k_sort_queries(const int* __restrict__ sig, int nq, int n,
                                                        int* __restrict__ perm) {
    extern __shared__ unsigned long long keys[];
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        keys[i] = i < nq ? ((unsigned long long)(uint32_t)sig[i] << 32) | (uint32_t)i : ~0ull;
    __syncthreads();
    for (int size = 2; size <= n; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                const int j = i ^ stride;
                if (j > i) {
                    const bool up = (i & size) == 0;
                    const unsigned long long a = keys[i], b = keys[j];
                    if ((a > b) == up) {
                        keys[i] = b;
                        keys[j] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
    for (int i = threadIdx.x; i < nq; i += blockDim.x) perm[i] = (int)(keys[i] & 0xffffffffu);
}

// ---------------------------------------------------------------------------
// stage 2b: FP32 refinement.  For each survivor, S = sum (q32 - x32)^2 in
// FP32 from the FP32 shadows; the key follows from the exact FP64 norms,
//   cosine: (|q|^2 + |x|^2 - S) / (2|x|), dot: (|q|^2 + |x|^2 - S) / 2,
//   Euclidean: (|q|^2 - S) / 2,
// with a certified bound on |S - |q - x|^2|:
//   eta = 2^-23 (|q| + |x|) bounds the FP32 rounding of q, x and q - x,
//   |S_exact - |q - x|^2| <= eta (2 |t| + eta), |S - S_exact| <= gamma S,
// gamma = (chain length + 7) 2^-24 for the FP32 accumulation (16 lanes per
// row, 4 chains per lane, then 3 + 4 additions).  Working from
// differences keeps the error proportional to |q - x| (small for the near
// rows that survive the screen) instead of |q| |x|.  Survivors whose upper
// bound is below the k-th largest refined lower bound are dropped.
// ---------------------------------------------------------------------------
constexpr int kRefThreads = 256;

// k-th largest refined lower bound over a query's n survivors, then the rows
// whose refined upper bound reaches it, written over `luq` as {row, screen
// key} once every bound has been read (the re-rank reads them from there)
__device__ void refine_keep(int q, int n, int k, float2* luq, const int2* sq, int* nref, int* hist, uint32_t* s_sh,
                            int* s_out) {
    if (threadIdx.x == 0) *s_out = 0;
    const uint32_t thr_ord =
        n >= k ? block_kth_largest([&](int i) { return f2u_ord(__ldcg(&luq[i].x)); }, n, k, hist, s_sh) : 0u;
    constexpr int kPer = scr::kSurvCap / kRefThreads;
    uint32_t keepbits = 0;
#pragma unroll
    for (int m = 0; m < kPer; ++m) {
        const int i = threadIdx.x + m * kRefThreads;
        if (i < n && f2u_ord(__ldcg(&luq[i].y)) >= thr_ord) keepbits |= 1u << m;
    }
    __syncthreads();
    int o = keepbits ? atomicAdd(s_out, __popc(keepbits)) : 0;
    int2* out = reinterpret_cast<int2*>(luq);
    for (int m = 0; m < kPer; ++m)
        if ((keepbits >> m) & 1u) out[o++] = sq[threadIdx.x + m * kRefThreads];
    __syncthreads();
    if (threadIdx.x == 0) nref[q] = *s_out;
}

// Refined {L, U} of one survivor from p = S (see above): the key's interval.
// xb = sqf[row]: |x|^2 in [xb.x, xb.y], 1/(2|x|) in [xb.z, xb.w].
__device__ __forceinline__ float2 refine_interval(float p, float gamma, float qq_lo, float qq_hi, float qn_up,
                                                  float4 xb, float xn_up, int metric) {
    const float sup = __fmul_ru(p, 1.0f + gamma);
    const float eta = __fmul_ru(1.1921875e-07f, __fadd_ru(qn_up, xn_up));  // 2^-23 (1 + 2^-13)
    float ed2 = __fmaf_ru(gamma, sup, __fmul_ru(eta, __fadd_ru(__fmul_ru(2.0f, __fsqrt_ru(sup)), eta)));
    ed2 = __fmaf_ru(9.094947e-13f, __fadd_ru(qq_hi, xb.y), __fmul_ru(ed2, 1.000001f));  // + 2^-40 scale
    const float s_hi = __fadd_ru(p, ed2), s_lo = __fsub_rd(p, ed2);  // |q - x|^2 in [s_lo, s_hi]
    float L, U;
    if (metric == SVDB_EUCLIDEAN) {  // key = (|q|^2 - d^2) / 2
        L = __fmul_rd(__fsub_rd(qq_lo, s_hi), 0.5f);
        U = __fmul_ru(__fsub_ru(qq_hi, s_lo), 0.5f);
    } else {  // dot = (|q|^2 + |x|^2 - d^2) / 2
        const float a_lo = __fsub_rd(__fadd_rd(qq_lo, xb.x), s_hi);
        const float a_hi = __fsub_ru(__fadd_ru(qq_hi, xb.y), s_lo);
        if (metric == SVDB_DOT) {
            L = __fmul_rd(a_lo, 0.5f);
            U = __fmul_ru(a_hi, 0.5f);
        } else {  // cosine key = dot / |x|, 1/(2|x|) in [xb.z, xb.w]
            L = a_lo >= 0.f ? __fmul_rd(a_lo, xb.z) : __fmul_rd(a_lo, xb.w);
            U = a_hi >= 0.f ? __fmul_ru(a_hi, xb.w) : __fmul_ru(a_hi, xb.z);
            if (isnan(L)) L = -INFINITY;
            if (isnan(U)) U = INFINITY;
        }
    }
    return make_float2(L, U);
}

// Scores the survivors of query q in FP32 (one half warp per row, the
// query's FP32 copy `qs` in shared memory) and writes each survivor's refined
// {L, U} to luq.  Rows base = (split * warps + warp) * 2 + half, stepping by
// splits * warps * 2.
__device__ __forceinline__ void refine_rows(const float* __restrict__ x32, size_t ld, const float* qs,
                                            const float4* __restrict__ sqf, const float4* __restrict__ rowp,
                                            const int2* sq, int n, float2* luq, float gamma, float qq_lo,
                                            float qq_hi, float qn_up, int metric, int split, int splits) {
    constexpr int kWarps = kRefThreads / 32;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // half a warp per row: lane h of the half reads float4 h, h+16, ...
    // Software-pipelined: the next row's index and norm intervals are fetched
    // while this row's 3 KB are read and reduced, so a row costs one memory
    // round trip instead of three dependent ones.
    const int hw = lane >> 4, h = lane & 15;
    const int stride = splits * kWarps * 2;
    int base = (split * kWarps + warp) * 2;
    int row_n = base + hw < n ? sq[base + hw].x : 0;
    float4 xb_n = make_float4(0.f, 0.f, 0.f, 0.f);
    float xn_n = 0.f;
    if (base + hw < n && h == 0) {
        xb_n = sqf[row_n];
        xn_n = rowp[row_n].x;
    }
    for (; base < n; base += stride) {
        const int i = base + hw;
        const bool act = i < n;
        const int row = row_n;
        const float4 xb = xb_n;
        const float xn_up = xn_n;
        const int in = i + stride;
        row_n = in < n ? sq[in].x : 0;
        float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
        if (act) {
            const float4* x = reinterpret_cast<const float4*>(x32 + (size_t)row * ld);
            const float4* qv = reinterpret_cast<const float4*>(qs);
#pragma unroll 12
            for (size_t j = h; j < ld / 4; j += 16) {
                const float4 xv = __ldg(x + j);
                const float4 qq4 = qv[j];
                const float t0 = qq4.x - xv.x, t1 = qq4.y - xv.y, t2 = qq4.z - xv.z, t3 = qq4.w - xv.w;
                a0 = fmaf(t0, t0, a0);
                a1 = fmaf(t1, t1, a1);
                a2 = fmaf(t2, t2, a2);
                a3 = fmaf(t3, t3, a3);
            }
        }
        float p = (a0 + a1) + (a2 + a3);
        p += __shfl_xor_sync(0xffffffffu, p, 8);
        p += __shfl_xor_sync(0xffffffffu, p, 4);
        p += __shfl_xor_sync(0xffffffffu, p, 2);
        p += __shfl_xor_sync(0xffffffffu, p, 1);
        if (in < n && h == 0) {
            xb_n = sqf[row_n];
            xn_n = rowp[row_n].x;
        }
        if (act && h == 0) luq[i] = refine_interval(p, gamma, qq_lo, qq_hi, qn_up, xb, xn_up, metric);
    }
}

// The per-row key and bound are interval arithmetic in FP32 with directed
// rounding (GB300's FP64 pipe is narrow; one FP64 instruction per row per warp
// would dominate): |q|^2 and |x|^2 enter as [rd, ru] pairs, d^2 as [S - E, S + E].
// Each survivor's refined {L, U} goes to `lu` (the candidate list's storage,
// dead after the select), so no per-thread state limits the occupancy.
__global__ void __launch_bounds__(kRefThreads, 3) k_refine(const float* __restrict__ x32, size_t ld,
                                                           const float* __restrict__ q32,
                                                           const double* __restrict__ qsq,
                                                           const float4* __restrict__ sqf,
                                                           const float4* __restrict__ rowp,
                                                           const float4* __restrict__ qpar, int2* __restrict__ surv,
                                                           const int* __restrict__ nsurv, int* __restrict__ nref,
                                                           float2* __restrict__ lu, size_t lu_stride, int k, int metric,
                                                           const int* __restrict__ perm, uint8_t* __restrict__ flags) {
    extern __shared__ __align__(16) uint8_t sm[];
    float* qs = reinterpret_cast<float*>(sm);  // the query in FP32 (ld floats)
    __shared__ int hist[256];
    __shared__ uint32_t s_sh[3];
    __shared__ int s_out;
    const int q = perm ? perm[blockIdx.x] : blockIdx.x;
    const int split = blockIdx.y, splits = gridDim.y;  // splits > 1: k_refine_keep finishes
    if (flags[q] != scr::kOk) {
        if (threadIdx.x == 0 && split == 0) nref[q] = 0;
        return;
    }
    for (size_t i = threadIdx.x; i < ld; i += blockDim.x) qs[i] = q32[(size_t)q * ld + i];
    const int n = nsurv[q];
    int2* sq = surv + (size_t)q * scr::kSurvCap;
    __syncthreads();
    float2* luq = lu + (size_t)q * lu_stride;
    const double qq = qsq[q];
    // each lane: ld/64 steps into each of 4 accumulators, then 2 + 4 additions
    const float gamma = (float)(ld / 64 + 8) * 5.9604644775390625e-08f * 1.0001f;
    refine_rows(x32, ld, qs, sqf, rowp, sq, n, luq, gamma, __double2float_rd(qq), __double2float_ru(qq), qpar[q].x,
                metric, split, splits);
    if (splits == 1) {
        __syncthreads();
        refine_keep(q, n, k, luq, sq, nref, hist, s_sh, &s_out);
    }
}

// second half of a split refinement: one block per query
__global__ void __launch_bounds__(kRefThreads) k_refine_keep(const int2* __restrict__ surv,
                                                             const int* __restrict__ nsurv, int* __restrict__ nref,
                                                             float2* __restrict__ lu, size_t lu_stride, int k,
                                                             const uint8_t* __restrict__ flags) {
    __shared__ int hist[256];
    __shared__ uint32_t s_sh[3];
    __shared__ int s_out;
    const int q = blockIdx.x;
    if (flags[q] != scr::kOk) {
        if (threadIdx.x == 0) nref[q] = 0;
        return;
    }
    refine_keep(q, nsurv[q], k, lu + (size_t)q * lu_stride, surv + (size_t)q * scr::kSurvCap, nref, hist, s_sh,
                &s_out);
}

// ---------------------------------------------------------------------------
// stage 3: FP64 re-rank of what the refinement keeps
// ---------------------------------------------------------------------------
// One block per query scores the rows left (4 lanes per row, canonical
// order) and ranks them by counting, on order-preserving 64-bit integer
// images of the ranking key (the FP64 pipe is narrow; -0.0 is folded into
// +0.0 and NaN ranks as +inf, exactly as double comparisons order them), ties
// to the lowest row.  Two passes: up to kSmallRerank rows (the common case,
// small shared memory, many blocks per SM), then up to kLargeRerank rows for
// the queries the first pass handed on; queries with more rows are answered
// by the exact scan.
constexpr int kSmallRerank = 512, kLargeRerank = 2048;

__device__ __forceinline__ long long rank_ord(int metric, double v) {
    double kk = metric == SVDB_EUCLIDEAN ? v : -v;
    if (isnan(kk)) kk = __longlong_as_double(0x7ff0000000000000ll);
    if (kk == 0.0) kk = 0.0;
    const long long b = __double_as_longlong(kk);
    return b >= 0 ? b : b ^ 0x7fffffffffffffffll;
}

template <bool EUC, int CAP>
__global__ void __launch_bounds__(256) k_rerank_small(const double* __restrict__ x64, size_t ld,
                                                      const double* __restrict__ qbuf, const double* __restrict__ qsq,
                                                      const double* __restrict__ sq64, const int2* __restrict__ surv,
                                                      size_t surv_stride, const int* __restrict__ nsurv, int k,
                                                      int metric, int d, const float4* __restrict__ rpar,
                                                      const float4* __restrict__ qpar,
                                                      const int64_t* __restrict__ logical, int64_t* __restrict__ ids,
                                                      double* __restrict__ dists, double* __restrict__ err,
                                                      uint8_t* __restrict__ flags) {
    extern __shared__ __align__(16) uint8_t sm[];
    double* qs = reinterpret_cast<double*>(sm);
    long long* skey = reinterpret_cast<long long*>(qs + ld);
    double* sval = reinterpret_cast<double*>(skey + CAP);
    int* srow = reinterpret_cast<int*>(sval + CAP);
    int* spos = srow + CAP;  // candidate index at each output position
    __shared__ int s_bad;
    const int q = blockIdx.x;
    // the first pass takes certified queries, the second the ones it handed on
    if (flags[q] != (CAP == kSmallRerank ? scr::kOk : scr::kRerankLarge)) return;
    const int n = nsurv[q];
    if (n > CAP) {
        if (threadIdx.x == 0)  // the second pass, or else the exact scan, answers it
            flags[q] = CAP == kSmallRerank ? scr::kRerankLarge : scr::kRerankOverflow;
        return;
    }
    const int lane = threadIdx.x & 31, g = threadIdx.x >> 2, s = lane & 3;
    for (size_t i = threadIdx.x; i < ld; i += blockDim.x) qs[i] = qbuf[(size_t)q * ld + i];
    if (threadIdx.x == 0) s_bad = 0;
    for (int i = threadIdx.x; i < k; i += blockDim.x) spos[i] = -1;
    __syncthreads();
    const int2* sq = surv + (size_t)q * surv_stride;
    const double qq = qsq[q];
    const double qn = sqrt(qq);
    const float4 qp = qpar[q];
    for (int base = 0; base < n; base += 64) {
        const int i = base + g;
        const bool act = i < n;
        const int2 c = act ? sq[i] : make_int2(0, 0);
        double p = 0.0;
        if (act) {
            const double* x = x64 + (size_t)c.x * ld;
            for (size_t j = 2 * s; j < ld; j += 8) {
                const double2 v = *reinterpret_cast<const double2*>(x + j);
                const double2 qv = *reinterpret_cast<const double2*>(qs + j);
                if (EUC) {
                    const double t0 = qv.x - v.x, t1 = qv.y - v.y;
                    p = fma(t0, t0, p);
                    p = fma(t1, t1, p);
                } else {
                    p = fma(qv.x, v.x, p);
                    p = fma(qv.y, v.y, p);
                }
            }
        }
        p = group4_sum(p);
        if (act && s == 0) {
            const double xs = sq64[c.x];
            double val, kex;
            if (EUC) {
                val = sqrt(p);
                kex = 0.5 * (qq - p);
            } else if (metric == SVDB_COSINE) {
                val = p / (qn * sqrt(xs));
                kex = p / sqrt(xs);
            } else {
                val = p;
                kex = p;
            }
            // the screen's bound must hold against the exact value
            const float key = __int_as_float(c.y);
            if (!(fabs(kex - (double)key) <= (double)screen_bound(rpar[c.x], qp.x, qp.y, qp.z))) s_bad = 1;
            skey[i] = rank_ord(metric, val);
            sval[i] = val;
            srow[i] = c.x;
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const long long ki = skey[i];
        const int ri = srow[i];
        int pos = 0;
        for (int j = 0; j < n; ++j) pos += (skey[j] < ki || (skey[j] == ki && srow[j] < ri)) ? 1 : 0;
        if (pos < k) spos[pos] = i;
    }
    __syncthreads();
    if (threadIdx.x == 0 && s_bad) flags[q] = scr::kBoundFail;
    if (s_bad) return;
    // exact only with k finite results: NaN-valued rows, which the screen never
    // emits, could otherwise belong in the list
    int fin = 1;
    for (int t = threadIdx.x; t < k; t += blockDim.x) {
        const int i = spos[t];
        if (i < 0 || isnan(sval[i])) fin = 0;
    }
    if (!__syncthreads_and(fin)) {
        if (threadIdx.x == 0) flags[q] = scr::kTooFew;
        return;
    }
    for (int t = threadIdx.x; t < k; t += blockDim.x) {
        const int i = spos[t];
        const size_t o = (size_t)q * k + t;
        ids[o] = logical[srow[i]];
        dists[o] = sval[i];
        if (err) err[o] = result_err_bound(metric, d, sval[i], qq, sq64[srow[i]]);
    }
}

// gather query rows (padded FP64) of the queries to re-answer; scatter back
// queries the screen could not certify, compacted on the device, with the
// batch's statistics (scr::kStats)
__global__ void k_collect_redo(const uint8_t* __restrict__ flags, const int* __restrict__ cnt, int nsub,
                               const int* __restrict__ nsurv, const int* __restrict__ nref, int nq,
                               int* __restrict__ list, int* __restrict__ count,
                               unsigned long long* __restrict__ stats) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long v[scr::kStats] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (q < nq) {
        const uint8_t f = flags[q];
        if (f != scr::kOk) list[atomicAdd(count, 1)] = q;
        for (int t = 0; t < nsub; ++t) v[0] += (unsigned)max(cnt[(size_t)q * nsub + t], 0);
        v[1] = (unsigned)nsurv[q];
        v[2] = (unsigned)nref[q];
        v[3] = f != scr::kOk;
        v[4] = f == scr::kBoundFail;
        v[5] = f == scr::kOverflow;
        v[6] = f == scr::kSurvOverflow;
        v[7] = f == scr::kRerankOverflow;
    }
#pragma unroll
    for (int t = 0; t < scr::kStats; ++t) {
        unsigned long long x = v[t];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) == 0 && x) atomicAdd(stats + t, x);
    }
}

// gather query rows (padded FP64) of the queries to re-answer; scatter back
// (the count lives on the device: with nothing to re-answer these exit at once)
__global__ void k_gather_queries(const double* __restrict__ qbuf, const double* __restrict__ qsq, size_t ld,
                                 const int* __restrict__ list, const int* __restrict__ n_dev,
                                 double* __restrict__ qout, double* __restrict__ qsq_out) {
    const int i = blockIdx.x;
    if (i >= *n_dev) return;
    const int q = list[i];
    for (size_t j = threadIdx.x; j < ld; j += blockDim.x) qout[(size_t)i * ld + j] = qbuf[(size_t)q * ld + j];
    if (threadIdx.x == 0) qsq_out[i] = qsq[q];
}

__global__ void k_scatter_results(const int64_t* __restrict__ ids_in, const double* __restrict__ d_in,
                                  const double* __restrict__ e_in, const int* __restrict__ list,
                                  const int* __restrict__ n_dev, int k, int64_t* __restrict__ ids,
                                  double* __restrict__ dists, double* __restrict__ err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *n_dev * k) return;
    const int qi = i / k, j = i % k;
    const size_t o = (size_t)list[qi] * k + j;
    ids[o] = ids_in[i];
    dists[o] = d_in[i];
    if (err) err[o] = e_in[i];
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct GemmPlanCache {
    PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    bool attr_set[4] = {};  // per screen variant: 2 x E4M3 + cosine
    bool sort_attr = false;
    bool rerank_attr = false;
    bool refine_attr = false;
    bool stream_attr = false;
    size_t screen_smem = 0;
    size_t screen_smem_pair = 0;
    bool attr_pair[4] = {};
    bool attr_duo[4] = {};
    bool attr_sq[2][4] = {};       // the small-batch forms: 32 and 64 query rows
    size_t screen_smem_sq[2] = {};
    size_t screen_smem_duo = 0;
};

static int gemm_cache(Store* s, GemmPlanCache** out) {
    if (!s->gemm) {
        GemmPlanCache* c = new (std::nothrow) GemmPlanCache();
        if (!c) {
            svdb_set_error("search_bf16: out of host memory");
            return SVDB_ENOMEM;
        }
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult qr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &qr) !=
                cudaSuccess ||
            qr != cudaDriverEntryPointSuccess || !fn) {
            cudaGetLastError();
            delete c;
            svdb_set_error("search_bf16: cuTensorMapEncodeTiled is not available from the driver");
            return SVDB_ECUDA;
        }
        c->encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
        c->screen_smem = sizeof(scr::Smem) + 1024;
        c->screen_smem_duo = sizeof(scr::SmemT<false, true>) + 1024;
        c->screen_smem_sq[0] = sizeof(scr::SmemT<false, false, 32>) + 1024;
        c->screen_smem_sq[1] = sizeof(scr::SmemT<false, false, 64>) + 1024;
        c->screen_smem_pair = sizeof(scr::SmemT<true>) + 1024;
        s->gemm = c;
    }
    *out = s->gemm;
    return SVDB_OK;
}

void Store::release_extra() {
    delete gemm;
    gemm = nullptr;
}

// 2-D BF16 tensor map over rows x ldb (row-major), box = 64 x box_rows, 128B swizzle
static int make_map(GemmPlanCache* c, CUtensorMap* m, const void* base, size_t rows, size_t ldb, int box_rows) {
    const cuuint64_t dims[2] = {(cuuint64_t)ldb, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)(ldb * 2)};
    const cuuint32_t box[2] = {(cuuint32_t)scr::kBK, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = c->encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        svdb_set_error("search_bf16: cuTensorMapEncodeTiled failed (%d)", (int)r);
        return SVDB_ECUDA;
    }
    return SVDB_OK;
}

// E4M3 queries: the tensor map of make_map over bytes (128-element boxes)
static int make_map8(GemmPlanCache* c, CUtensorMap* m, const void* base, size_t rows, size_t ldb8, int box_rows) {
    const cuuint64_t dims[2] = {(cuuint64_t)ldb8, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ldb8};
    const cuuint32_t box[2] = {(cuuint32_t)(2 * scr::kBK), (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = c->encode(m, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<void*>(base), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        svdb_set_error("search_fp8: cuTensorMapEncodeTiled failed (%d)", (int)r);
        return SVDB_ECUDA;
    }
    return SVDB_OK;
}

// The paired screen (cta_group::2) is opt-in: SVDB_SCREEN_PAIR=1 in the
// environment (read once per process) uses it for batches of more than one
// 128-query tile.  It cuts the L2 -> shared-memory operand traffic by a third
// and, with an epilogue that does nothing, runs 5 % faster than the
// single-CTA form (1M x 768, Q = 4096: 3.54 against 3.73 ms), but with the
// real epilogue both CTAs of a pair must drain an accumulator before the MMAs
// reuse it, and it measured no faster for BF16 cosine (4.03 against 4.06 ms)
// and slower for FP8 (3.55 against 3.22 ms) and Euclidean (4.71 against
// 4.60 ms).  Pairs that can run at once: every two SMs, as far as the
// cluster scheduler places them (asked once per process).
static bool pair_enabled() {
    static int on = -1;
    if (on < 0) {
        const char* e = getenv("SVDB_SCREEN_PAIR");
        on = (e && e[0] == '1') ? 1 : 0;
    }
    return on == 1;
}

static bool screen_pair(size_t nq) { return nq > (size_t)scr::kBM && pair_enabled(); }

static int pair_units() {
    static int n = 0;
    if (!n) {
        n = std::max(1, num_sms() / 2);
        auto kern = k_screen_bf16<true, false, false, true>;
        const int smem = (int)(sizeof(scr::SmemT<true>) + 1024);
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) == cudaSuccess) {
            cudaLaunchConfig_t cfg = {};
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = 2;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.gridDim = dim3((unsigned)(2 * n));
            cfg.blockDim = dim3(scr::kThreads);
            cfg.dynamicSmemBytes = (size_t)smem;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            int m = 0;
            if (cudaOccupancyMaxActiveClusters(&m, (void*)kern, &cfg) == cudaSuccess && m > 0) n = std::min(n, m);
        }
        cudaGetLastError();
    }
    return n;
}

// Stores whose tiles are at most this many k blocks deep (D <= 128) screen
// with two CTAs per SM: there the epilogue, not the MMAs, sets the pace.
constexpr int kDuoMaxKb = 2;
static bool screen_duo(const Store* s, bool pair) { return !pair && (int)(s->ldb / scr::kBK) <= kDuoMaxKb; }

static int screen_units(bool pair, bool duo = false) {
    return pair ? pair_units() : std::min((duo ? 2 : 1) * num_sms(), kMaxCtas);
}

// tensor map over a shadow's swizzled tiles as rows of 128 bytes (256 rows per
// tile and k block), copied as they are (the paired screen loads half a tile)
static int make_map_tiles(GemmPlanCache* c, CUtensorMap* m, const void* base, size_t rows) {
    const cuuint64_t dims[2] = {128, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {128};
    const cuuint32_t box[2] = {128, (cuuint32_t)(scr::kBN / 2)};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = c->encode(m, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<void*>(base), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        svdb_set_error("search_bf16: cuTensorMapEncodeTiled (store tiles) failed (%d)", (int)r);
        return SVDB_ECUDA;
    }
    return SVDB_OK;
}

// one screen launch: `units` CTAs, or `units` clusters of a CTA pair
template <class K>
static int launch_screen(K kern, bool pair, int units, size_t smem, cudaStream_t st, const CUtensorMap& tmq,
                         const CUtensorMap& tmx, const ScreenParams& P) {
    if (!pair) {
        kern<<<(unsigned)units, scr::kThreads, smem, st>>>(tmq, tmx, P);
        SVDB_LAUNCH_CHECK();
        return SVDB_OK;
    }
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = 2;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3((unsigned)(2 * units));
    cfg.blockDim = dim3(scr::kThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    SVDB_CUDA(cudaLaunchKernelEx(&cfg, kern, tmq, tmx, P));
    return SVDB_OK;
}

struct Bf16Layout {
    bool pair = false;  // the paired screen (query tiles of 256)
    bool duo = false;   // two CTAs per SM (shallow tiles)
    int qr = scr::kBM;  // query rows per stage: 32 / 64 for batches that small (deeper rings)
    size_t qb, qscale, qb16, qpar16, seed, q32, qpar, rpar, spar, vbits, tau, bins, cnt, coff, cand, surv, nsurv, nref, sig, perm, flags, alpha, redo, redo_n, stats, rq, rsq, rres, rscr, total;
    size_t tmax = 0, cut = 0;  // the streamed screen of a single query (its keys reuse spar: npad floats)
    int ntr, cap;
    int nctas, nsub;
    int nsub_seed_max;  // sub-lists per query cnt / coff hold (>= nsub and the seeding screen's)
    size_t npad;
    ScreenSched sched;
};

// The screen's work, query tiles x store tiles, over G units: one CTA per SM,
// or one CTA pair per two SMs (then a query tile is 256 queries).  With
// G = base * ntq + ea, query tiles [0, ea) get base + 1 CTAs that split the
// store tiles evenly, the others base CTAs of T = ceil(ntq * ntr / G) tiles
// each; what those leave at the end of the store (ntr - base * T tiles per
// query tile) is shared out among the first family's CTAs, whose own share is
// shorter.  Every CTA then has ~T tiles; CTAs that cover the same store rows
// do so at the same time (a row is read from HBM about once per family).
// Returns the number of CTAs; *maxsub = most segments of one query tile.
static int screen_schedule(int ntq, int ntr, ScreenSched& S, int* maxsub, int units) {
    std::memset(&S, 0, sizeof(S));
    S.ntr = ntr;
    const int G = std::min(units, kMaxCtas);
    if (ntq >= G) {
        S.direct = 1;
        *maxsub = 1;
        return ntq;
    }
    std::vector<int> ord(ntq, 0);
    bool fits = true;
    std::vector<int> starters(ntq, 0);
    auto add = [&](int c, int qt, int lo, int hi) {
        if (hi <= lo) return;
        if (S.nseg[c] >= kMaxSeg) {
            fits = false;
            return;
        }
        if (S.nseg[c] == 0) ++starters[qt];
        S.seg[c][S.nseg[c]++] = ScreenSeg{lo, hi, (uint16_t)qt, (uint16_t)ord[qt]++, 0, (uint16_t)qt};
    };
    const int base = G / ntq, ea = G % ntq;
    const int T = (int)(((int64_t)ntq * ntr + G - 1) / G);
    int c = 0;
    for (int qt = 0; qt < ea; ++qt)
        for (int jj = 0; jj <= base; ++jj, ++c)
            add(c, qt, (int)((int64_t)jj * ntr / (base + 1)), (int)((int64_t)(jj + 1) * ntr / (base + 1)));
    const int helpers = c;
    for (int qt = ea; qt < ntq; ++qt)
        for (int jj = 0; jj < base; ++jj, ++c)
            add(c, qt, (int)std::min<int64_t>((int64_t)jj * T, ntr), (int)std::min<int64_t>((int64_t)(jj + 1) * T, ntr));
    const int64_t Rq = std::max<int64_t>(0, (int64_t)ntr - (int64_t)base * T);
    const int64_t R = (int64_t)(ntq - ea) * Rq;
    for (int h = 0; h < helpers && R > 0; ++h) {
        int64_t s0 = h * R / helpers;
        const int64_t e0 = (h + 1) * R / helpers;
        while (s0 < e0) {
            const int64_t qb = s0 / Rq, qe = std::min(e0, (qb + 1) * Rq);
            add(h, ea + (int)qb, (int)((int64_t)base * T + s0 - qb * Rq), (int)((int64_t)base * T + qe - qb * Rq));
            s0 = qe;
        }
    }
    if (fits && 2 * *std::max_element(ord.begin(), ord.end()) > scr::kMaxSub) fits = false;
    if (!fits) {  // plain row groups: query tile x row range, one segment each
        std::memset(&S, 0, sizeof(S));
        S.ntr = ntr;
        std::fill(ord.begin(), ord.end(), 0);
        c = 0;
        for (int g = 0; g < base; ++g)
            for (int qt = 0; qt < ntq; ++qt, ++c)
                S.seg[c][S.nseg[c]++] = ScreenSeg{(int)((int64_t)g * ntr / base), (int)((int64_t)(g + 1) * ntr / base),
                                                  (uint16_t)qt, (uint16_t)ord[qt]++, 0, (uint16_t)qt};
    }
    if (!fits) starters = ord;  // (row groups: one segment per CTA)
    for (int qt = 0; qt < ntq; ++qt) {
        S.nsq[qt] = (uint16_t)std::max(1, ord[qt]);
        S.nst[qt] = (uint16_t)std::max(1, starters[qt]);
    }
    *maxsub = std::max(1, *std::max_element(ord.begin(), ord.end()));
    return c;
}

constexpr size_t k_max_bf16 = 128;  // largest k the screen certifies

// maxsub_ext > 0: the search is screened by a fused launch whose schedule
// gives each of its query tiles at most maxsub_ext segments (single-CTA form)
static Bf16Layout bf16_layout(const Store* s, size_t nq, int maxsub_ext = 0) {
    Bf16Layout L;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off += round_up(bytes, 1024);
        return o;
    };
    L.ntr = (int)((std::max<size_t>(s->slots, 1) + scr::kBN - 1) / scr::kBN);
    L.npad = (size_t)L.ntr * scr::kBN;
    L.qb = take(std::max(nq * s->ldb * 2, nq * s->ldb8));  // BF16 queries, or the E4M3 ones
    L.qscale = take(nq * sizeof(float));
    // FP8 threshold seeding (BF16 screen of a sample of the rows)
    L.qb16 = take(nq * s->ldb * 2);
    L.qpar16 = take(nq * sizeof(float4));
    L.seed = take(nq * sizeof(float));
    L.q32 = take(nq * s->ld * sizeof(float));
    L.qpar = take(nq * sizeof(float4));
    L.rpar = take(L.npad * sizeof(float4));
    L.spar = take(L.npad * sizeof(float4));
    L.vbits = take(L.npad / 8);
    L.tau = take(nq * sizeof(int));
    L.bins = take(nq * k_max_bf16 * sizeof(int));
    if (nq <= (size_t)kStreamQ && maxsub_ext <= 0) {
        L.tmax = take(nq * (size_t)L.ntr * kStreamWarps * sizeof(float));
        L.cut = take(nq * sizeof(float));
    }
    int maxsub = 1;
    if (maxsub_ext > 0) {
        std::memset(&L.sched, 0, sizeof(L.sched));
        L.pair = false;
        L.nctas = 0;
        maxsub = maxsub_ext;
    } else {
        L.pair = screen_pair(nq);
        L.duo = screen_duo(s, L.pair);
        // measured on 1M x 768: screen 0.38-0.40 -> 0.32-0.34 ms at 3-32 queries (32 rows,
        // 6 stages), ~0.37 -> 0.355 ms at 48 (64 rows, 5 stages); at 64 queries the
        // 5-deep ring was no faster (0.382 against 0.377 ms)
        if (!L.pair && !L.duo) L.qr = nq <= 32 ? 32 : (nq <= 48 ? 64 : scr::kBM);
        const size_t tq = L.pair ? 2 * scr::kBM : scr::kBM;
        L.nctas = screen_schedule((int)((nq + tq - 1) / tq), L.ntr, L.sched, &maxsub, screen_units(L.pair, L.duo));
    }
    L.nsub = 2 * maxsub;
    // the threshold seeding's screen (a 1/16 sample of the store) has its own
    // schedule, whose query tiles may have more segments: cnt / coff hold
    // either search's sub-lists
    int nsub_cnt = L.nsub;
    if (L.ntr >= 32 && nq >= 32) {
        ScreenSched* ss = new (std::nothrow) ScreenSched();
        const size_t tq = L.pair ? 2 * scr::kBM : scr::kBM;
        int maxsub_s = scr::kMaxSub / 2;  // (the largest any schedule uses, if the sizing cannot be done here)
        if (ss) {
            screen_schedule((int)((nq + tq - 1) / tq), L.ntr / 16, *ss, &maxsub_s, screen_units(L.pair, L.duo));
            delete ss;
        }
        nsub_cnt = std::max(nsub_cnt, 2 * maxsub_s);
    }
    L.nsub_seed_max = nsub_cnt;
    L.cnt = take(nq * (size_t)nsub_cnt * sizeof(int));
    L.coff = take(nq * (size_t)nsub_cnt * sizeof(int));
    // candidate lists: as long as the budget allows (small batches emit more
    // per query before the running thresholds settle), split into one
    // sub-list per emitting thread; at least the survivor cap in all, since
    // the refinement reuses the storage
    size_t cap = std::max<size_t>(scr::kCapMax, (size_t)L.nsub * scr::kSubMin);
    while (cap > (size_t)scr::kCapMin && nq * cap * sizeof(int2) > scr::kCandBudget) cap >>= 1;
    L.cap = (int)cap;  // >= kCapMin = kSurvCap
    L.cand = take(nq * (size_t)L.cap * sizeof(int2));
    L.surv = take(nq * (size_t)scr::kSurvCap * sizeof(int2));
    L.nsurv = take(nq * sizeof(int));
    L.nref = take(nq * sizeof(int));
    L.sig = take(nq * sizeof(int));
    L.perm = take(nq * sizeof(int));
    L.flags = take(nq);
    L.alpha = take(sizeof(int));
    // the exact-scan fallback, sized for the whole batch (its count is on the device)
    L.redo = take(nq * sizeof(int));
    L.redo_n = take(sizeof(int));
    L.stats = take(scr::kStats * sizeof(unsigned long long));
    L.rq = take(nq * s->ld * sizeof(double));
    L.rsq = take(nq * sizeof(double));
    L.rres = take(nq * (size_t)k_max_bf16 * (sizeof(int64_t) + 2 * sizeof(double)));
    L.rscr = take(search_fp64_scratch(s, nq, k_max_bf16));
    L.total = off;
    return L;
}

size_t search_bf16_scratch(const Store* s, size_t nq, size_t /*k: the layout holds k up to k_max_bf16*/) {
    return bf16_layout(s, nq).total;
}

bool bf16_supported(const Store* s, size_t k) { return k <= k_max_bf16 && s->n_unscreen == 0 && s->nlive > 0; }

// One BF16 / FP8 search between its phases: begin (queries, row terms, the
// screen's parameters), the screen (a launch of its own, or its share of a
// fused launch), end (select, refinement, re-rank, exact redo of what the
// screen could not certify).  Every phase runs on the store's stream except a
// fused screen.
struct Bf16Run {
    Store* s = nullptr;
    SearchArgs a;
    GemmPlanCache* gc = nullptr;
    Bf16Layout L;
    uint8_t* base = nullptr;
    bool f8 = false, norm = false, stream = false;
    int nsub_use = 0;
    ScreenParams P;
    CUtensorMap tmq;
    uint32_t kernels = 0;
    template <class T>
    T* at(size_t off) const {
        return reinterpret_cast<T*>(base + off);
    }
};

template <bool PR>
static auto screen_kernel_of(bool e4m3, bool norm) {
    return e4m3 ? (norm ? k_screen_bf16<true, true, false, PR> : k_screen_bf16<false, true, false, PR>)
                : (norm ? k_screen_bf16<true, false, false, PR> : k_screen_bf16<false, false, false, PR>);
}

template <int QR>
static auto small_batch_kernel_of(bool e4m3, bool norm) {
    return e4m3 ? (norm ? k_screen_bf16<true, true, false, false, false, false, QR>
                        : k_screen_bf16<false, true, false, false, false, false, QR>)
                : (norm ? k_screen_bf16<true, false, false, false, false, false, QR>
                        : k_screen_bf16<false, false, false, false, false, false, QR>);
}

// one screen over nunits units (CTAs or pairs) with the query tensor map tmq_;
// the paired form also gets the tensor map of the shadow's tiles
static int run_screen(Bf16Run& R, bool e4m3, bool pair, int nunits, const CUtensorMap& tmq_, const ScreenParams& P_) {
    GemmPlanCache* gc = R.gc;
    Store* s = R.s;
    const int v = 2 * (e4m3 ? 1 : 0) + (R.norm ? 1 : 0);
    if (!pair && R.L.duo) {
        auto kern = e4m3 ? (R.norm ? k_screen_bf16<true, true, false, false, false, true>
                                   : k_screen_bf16<false, true, false, false, false, true>)
                         : (R.norm ? k_screen_bf16<true, false, false, false, false, true>
                                   : k_screen_bf16<false, false, false, false, false, true>);
        if (!gc->attr_duo[v]) {
            SVDB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gc->screen_smem_duo));
            gc->attr_duo[v] = true;
        }
        kern<<<(unsigned)nunits, scr::kThreads, gc->screen_smem_duo, s->stream>>>(tmq_, tmq_, P_);
        SVDB_LAUNCH_CHECK();
        return SVDB_OK;
    }
    if (!pair && R.L.qr < scr::kBM) {  // a small batch: the deeper ring (tmq_ has boxes of qr rows)
        const int f = R.L.qr == 32 ? 0 : 1;
        auto kern = f == 0 ? small_batch_kernel_of<32>(e4m3, R.norm) : small_batch_kernel_of<64>(e4m3, R.norm);
        if (!gc->attr_sq[f][v]) {
            SVDB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gc->screen_smem_sq[f]));
            gc->attr_sq[f][v] = true;
        }
        return launch_screen(kern, false, nunits, gc->screen_smem_sq[f], s->stream, tmq_, tmq_, P_);
    }
    if (!pair) {
        auto kern = screen_kernel_of<false>(e4m3, R.norm);
        if (!gc->attr_set[v]) {
            SVDB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gc->screen_smem));
            gc->attr_set[v] = true;
        }
        return launch_screen(kern, false, nunits, gc->screen_smem, s->stream, tmq_, tmq_, P_);
    }
    auto kern = screen_kernel_of<true>(e4m3, R.norm);
    if (!gc->attr_pair[v]) {
        SVDB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gc->screen_smem_pair));
        gc->attr_pair[v] = true;
    }
    CUtensorMap tmx;
    const size_t kbl = e4m3 ? s->ldb8 / (2 * scr::kBK) : s->ldb / scr::kBK;
    const int rc = make_map_tiles(gc, &tmx, P_.g.xblk, (size_t)R.L.ntr * kbl * scr::kBN);
    if (rc) return rc;
    return launch_screen(kern, true, nunits, gc->screen_smem_pair, s->stream, tmq_, tmx, P_);
}

// one_list: the streamed screen's single list (no sub-list offsets)
static int launch_select(Bf16Run& R, int nsub_, bool one_list, const float4* qp_, float* kth) {
    Store* s = R.s;
    if (nsub_ > scr::kMaxSub) {  // (k_select's prefix of the sub-list counts is in shared memory)
        svdb_set_error("search_bf16: %d candidate sub-lists per query, more than %d", nsub_, scr::kMaxSub);
        return SVDB_EINVAL;
    }
    const Bf16Layout& L = R.L;
    const int nq = (int)R.a.nq, k = (int)R.a.k;
    // small batches carry many candidates per query: wider blocks
    const int sel_threads = nq >= 256 ? 256 : 1024;
    int2* cand = R.at<int2>(L.cand);
    int* cnt = R.at<int>(L.cnt);
    const float4* rpar = R.at<float4>(L.rpar);
    int2* surv = R.at<int2>(L.surv);
    int* nsurv = R.at<int>(L.nsurv);
    int* sig = R.at<int>(L.sig);
    uint8_t* flags = R.at<uint8_t>(L.flags);
    k_select<<<(unsigned)nq, sel_threads, 0, s->stream>>>(cand, cnt, one_list ? nullptr : R.at<int>(L.coff), L.cap,
                                                          nsub_, rpar, qp_, k, surv, nsurv, sig, flags, kth);
    SVDB_LAUNCH_CHECK();
    return SVDB_OK;
}

// queries, row terms and the screen's parameters (R.P, R.tmq); maxsub_ext > 0:
// a fused screen (BF16 only) will take the place of bf16_screen
static int bf16_begin(Bf16Run& R, Store* s, const SearchArgs& a, void* scratch, size_t scratch_bytes, bool f8,
                      int maxsub_ext) {
    int rc = gemm_cache(s, &R.gc);
    if (rc) return rc;
    R.s = s;
    R.a = a;
    R.f8 = f8;
    R.L = bf16_layout(s, a.nq, maxsub_ext);
    const Bf16Layout& L = R.L;
    if (L.total > scratch_bytes) {
        svdb_set_error("search_bf16: scratch too small");
        return SVDB_EINVAL;
    }
    R.base = reinterpret_cast<uint8_t*>(scratch);
    GemmPlanCache* gc = R.gc;
    __nv_bfloat16* qb = R.at<__nv_bfloat16>(L.qb);
    float* q32 = R.at<float>(L.q32);
    float4* qpar = R.at<float4>(L.qpar);
    float4* rpar = R.at<float4>(L.rpar);
    float4* spar = R.at<float4>(L.spar);
    int* alpha = R.at<int>(L.alpha);
    uint32_t* vbits = R.at<uint32_t>(L.vbits);
    int* tau = R.at<int>(L.tau);
    int* bins = R.at<int>(L.bins);
    int* cnt = R.at<int>(L.cnt);
    int2* cand = R.at<int2>(L.cand);
    uint8_t* flags = R.at<uint8_t>(L.flags);
    int* redo_n = R.at<int>(L.redo_n);
    unsigned long long* dstats = R.at<unsigned long long>(L.stats);
    float* qscale = R.at<float>(L.qscale);
    const int nq = (int)a.nq, k = (int)a.k;
    // f8: cosine screens the E4M3 unit-norm shadow, dot / Euclidean the E4M3
    // shadow with per-row power-of-two scales
    R.norm = a.metric == SVDB_COSINE;  // cosine screens the unit-norm shadow
    const bool norm = R.norm;

    // Seeding (the FP8 screen by default; BF16 when asked): start the running
    // thresholds from the exact k-th largest BF16 lower bound over a sample of
    // the store (its first 1/16 of the rows, which are in no particular
    // order).  The E4M3 bound is ~16x the BF16 one, so an FP8 screen whose
    // thresholds start from random rows emits every row within that bound of
    // them until it meets rows of the query's cluster; a sample holding
    // enough of them puts the threshold at the cluster's level from the first
    // tile.  A BF16 screen of rows without clusters and a large k otherwise
    // emits many times k rows before its shared thresholds settle.  A lower
    // bound over a subset of the rows is a lower bound over all of them, so
    // the seed is a valid starting threshold.
    float* seed = nullptr;
    const bool want_seed = a.seed > 0 || (a.seed < 0 && f8);
    if (want_seed && L.ntr >= 32 && nq >= 32) {  // (a lone query's tile is split over every SM: its bins fill at once)
        __nv_bfloat16* qb16 = R.at<__nv_bfloat16>(L.qb16);
        float4* qpar16 = R.at<float4>(L.qpar16);
        seed = R.at<float>(L.seed);
        const int tq = L.pair ? 2 * scr::kBM : scr::kBM;
        const int ntq = (nq + tq - 1) / tq;
        const int ntr_seed = L.ntr / 16;
        const int64_t npad_seed = (int64_t)ntr_seed * scr::kBN;
        ScreenParams PS;
        int maxsub_s = 1;
        const int nctas_s = screen_schedule(ntq, ntr_seed, PS.sched, &maxsub_s, screen_units(L.pair, L.duo));
        const int nsub_s = 2 * maxsub_s;
        if (nsub_s > L.nsub_seed_max) {  // (the layout sized cnt / coff for this schedule)
            svdb_set_error("search_bf16: the seeding schedule does not fit its layout");
            return SVDB_EINVAL;
        }
        k_prep_bf16<<<(unsigned)((a.nq * kPrepLanes + 255) / 256), 256, 0, s->stream>>>(a.q, nq, s->ld, s->ldb, a.metric,
                                                                              qb16, q32, qpar16);
        SVDB_LAUNCH_CHECK();
        k_init_search<<<(unsigned)((a.nq + 255) / 256), 256, 0, s->stream>>>(tau, bins, cnt, nsub_s, flags, nq, k, alpha,
                                                                             redo_n, dstats);
        SVDB_LAUNCH_CHECK();
        k_row_params<<<(unsigned)((npad_seed + 255) / 256), 256, 0, s->stream>>>(
            s->rowp, s->sq64, s->live, std::min<int64_t>((int64_t)s->slots, npad_seed), npad_seed, a.metric, s->rowpn,
            nullptr, rpar, spar, alpha, vbits);
        SVDB_LAUNCH_CHECK();
        CUtensorMap tmq16;
        rc = make_map(gc, &tmq16, qb16, a.nq, s->ldb, L.qr);
        if (rc) return rc;
        PS.g.xblk = reinterpret_cast<const uint8_t*>(norm ? (const void*)s->xbn : (const void*)s->xb);
        PS.g.qscale = qscale;
        PS.g.rpar = rpar;
        PS.g.spar = spar;
        PS.g.alpha = alpha;
        PS.g.vbits = vbits;
        PS.g.nmax = s->d_count + 1;
        PS.g.qpar = qpar16;
        PS.g.tau = tau;
        PS.g.bins = bins;
        PS.g.cnt = cnt;
        PS.g.coff = R.at<int>(L.coff);
        PS.g.ntr = ntr_seed;
        PS.g.cand = cand;
        PS.g.err = s->d_err;
        PS.g.dump = nullptr;
        PS.g.dump_ld = 0;
        PS.g.nq = nq;
        PS.g.k = k;
        PS.g.cap = L.cap;
        PS.g.nsub = nsub_s;
        PS.g.kblocks = (int)(s->ldb / scr::kBK);
            rc = run_screen(R, false, L.pair, nctas_s, tmq16, PS);
        if (rc) return rc;
        rc = launch_select(R, nsub_s, false, qpar16, seed);
        if (rc) return rc;
        R.kernels += 5;
    }

    if (f8)
        k_prep_f8<<<(unsigned)((a.nq * kPrepLanes + 255) / 256), 256, 0, s->stream>>>(
            a.q, nq, s->ld, s->ldb8, a.metric, reinterpret_cast<uint8_t*>(qb), q32, qpar, qscale);
    else
        k_prep_bf16<<<(unsigned)((a.nq * kPrepLanes + 255) / 256), 256, 0, s->stream>>>(a.q, nq, s->ld, s->ldb,
                                                                              a.metric, qb, q32, qpar);
    SVDB_LAUNCH_CHECK();
    // one or two cosine queries: the streamed screen, one candidate list per query
    R.stream = maxsub_ext <= 0 && norm && !f8 && nq <= kStreamQ &&
               (size_t)nq * s->ldb * sizeof(float) <= (size_t)kStreamQBytes;
    R.nsub_use = R.stream ? 1 : L.nsub;
    k_init_search<<<(unsigned)((a.nq + 255) / 256), 256, 0, s->stream>>>(tau, bins, cnt, R.nsub_use, flags, nq, k,
                                                                         alpha, redo_n, dstats, seed);
    SVDB_LAUNCH_CHECK();
    k_row_params<<<(unsigned)((L.npad + 255) / 256), 256, 0, s->stream>>>(
        s->rowp, s->sq64, s->live, (int64_t)s->slots, (int64_t)L.npad, a.metric, f8 ? s->rowpn8 : s->rowpn,
        f8 && !norm ? s->rowp8 : nullptr, rpar, spar, alpha, vbits);
    SVDB_LAUNCH_CHECK();
    R.kernels += 3;
    if (R.stream) return SVDB_OK;

    rc = f8 ? make_map8(gc, &R.tmq, qb, a.nq, s->ldb8, L.qr) : make_map(gc, &R.tmq, qb, a.nq, s->ldb, L.qr);
    if (rc) return rc;
    GroupParams& g = R.P.g;
    g.xblk = reinterpret_cast<const uint8_t*>(f8 ? (norm ? (const void*)s->xbn8 : (const void*)s->xb8)
                                              : norm ? (const void*)s->xbn : (const void*)s->xb);
    g.qscale = qscale;
    g.rpar = rpar;
    g.spar = spar;
    g.alpha = alpha;
    g.vbits = vbits;
    g.nmax = s->d_count + (f8 ? 3 : 1);
    g.qpar = qpar;
    g.tau = tau;
    g.bins = bins;
    g.cnt = cnt;
    g.coff = R.at<int>(L.coff);
    g.ntr = L.ntr;
    g.cand = cand;
    g.err = s->d_err;  // persistent: read at the next synchronous point
    g.dump = nullptr;
    g.dump_ld = 0;
    g.nq = nq;
    g.k = k;
    g.cap = L.cap;
    g.nsub = L.nsub;
    g.kblocks = f8 ? (int)(s->ldb8 / (2 * scr::kBK)) : (int)(s->ldb / scr::kBK);
    R.P.sched = L.sched;
    return SVDB_OK;
}

// the search's own screen: streamed (a single cosine query) or tensor-core
static int bf16_screen(Bf16Run& R) {
    Store* s = R.s;
    const Bf16Layout& L = R.L;
    if (!R.stream) {
        const int rc = run_screen(R, R.f8, L.pair, L.nctas, R.tmq, R.P);
        if (rc) return rc;
        ++R.kernels;
        return SVDB_OK;
    }
    const int nq = (int)R.a.nq, k = (int)R.a.k;
    float* keys = R.at<float>(L.spar);  // nq x npad floats: the cosine screen does not use spar
    float* tmax = R.at<float>(L.tmax);
    float* cut = R.at<float>(L.cut);
    const int KB = (int)(s->ldb / scr::kBK);
    const size_t smem = stream_smem((size_t)nq, s->ldb);
    if (!R.gc->stream_attr) {
        SVDB_CUDA(cudaFuncSetAttribute(k_stream_keys<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, kStreamQBytes));
        SVDB_CUDA(cudaFuncSetAttribute(k_stream_keys<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, kStreamQBytes));
        R.gc->stream_attr = true;
    }
    static_assert(kStreamQ == 2, "one instantiation per query count");
    (nq == 1 ? k_stream_keys<1> : k_stream_keys<2>)<<<(unsigned)L.ntr, 32 * kStreamWarps, smem, s->stream>>>(
        reinterpret_cast<const uint8_t*>(s->xbn), KB, R.at<__nv_bfloat16>(L.qb), s->ldb, nq, R.at<uint32_t>(L.vbits),
        L.npad, L.ntr, keys, tmax);
    SVDB_LAUNCH_CHECK();
    k_stream_cut<<<(unsigned)nq, 1024, 0, s->stream>>>(tmax, L.ntr * kStreamWarps, k, R.at<float4>(L.qpar),
                                                        s->d_count + 1, cut);
    SVDB_LAUNCH_CHECK();
    k_stream_emit<<<(unsigned)(L.npad / 256), 256, 0, s->stream>>>(keys, L.npad, nq, cut, L.cap, R.at<int>(L.cnt),
                                                                   R.at<int2>(L.cand));
    SVDB_LAUNCH_CHECK();
    R.kernels += 3;
    return SVDB_OK;
}

// select, refinement, re-rank and the exact redo, on the store's stream
static int bf16_end(Bf16Run& R, svdb_search_stats* st) {
    Store* s = R.s;
    const SearchArgs& a = R.a;
    const Bf16Layout& L = R.L;
    GemmPlanCache* gc = R.gc;
    const int nq = (int)a.nq, k = (int)a.k;
    float4* qpar = R.at<float4>(L.qpar);
    float4* rpar = R.at<float4>(L.rpar);
    int* cnt = R.at<int>(L.cnt);
    int2* cand = R.at<int2>(L.cand);
    int2* surv = R.at<int2>(L.surv);
    int* nsurv = R.at<int>(L.nsurv);
    int* nref = R.at<int>(L.nref);
    int* sig = R.at<int>(L.sig);
    int* perm = R.at<int>(L.perm);
    uint8_t* flags = R.at<uint8_t>(L.flags);
    int* redo = R.at<int>(L.redo);
    int* redo_n = R.at<int>(L.redo_n);
    unsigned long long* dstats = R.at<unsigned long long>(L.stats);
    float* q32 = R.at<float>(L.q32);

    int rc = launch_select(R, R.nsub_use, R.stream, qpar, nullptr);
    if (rc) return rc;
    s->prof_mark(3);
    const size_t ref_smem = s->ld * sizeof(float);
    if (!gc->refine_attr) {
        SVDB_CUDA(cudaFuncSetAttribute(k_refine, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        gc->refine_attr = true;
    }
    // refinement order (batches of up to 16384 queries are sorted; larger ones keep index order)
    const int* order = nullptr;
    if (nq > 1 && nq <= 16384) {
        int n2 = 1;
        while (n2 < nq) n2 <<= 1;
        if (!gc->sort_attr) {
            SVDB_CUDA(cudaFuncSetAttribute(k_sort_queries, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           16384 * (int)sizeof(unsigned long long)));
            gc->sort_attr = true;
        }
        k_sort_queries<<<1, 1024, (size_t)n2 * sizeof(unsigned long long), s->stream>>>(sig, nq, n2, perm);
        SVDB_LAUNCH_CHECK();
        ++R.kernels;
        order = perm;
    }
    // the candidate list (cap >= 8192 entries per query) is dead after the select:
    // it holds the refined {L, U} of each survivor
    // small batches: several blocks per query score the survivors, then one keeps
    const int rsplits = std::max(1, std::min(32, 2 * num_sms() / std::max(nq, 1)));
    k_refine<<<dim3((unsigned)nq, (unsigned)rsplits), kRefThreads, ref_smem, s->stream>>>(
        s->x32, s->ld, q32, a.qsq, s->sqf, s->rowp, qpar, surv, nsurv, nref, reinterpret_cast<float2*>(cand),
        (size_t)L.cap, k, a.metric, order, flags);
    SVDB_LAUNCH_CHECK();
    if (rsplits > 1) {
        k_refine_keep<<<(unsigned)nq, kRefThreads, 0, s->stream>>>(surv, nsurv, nref, reinterpret_cast<float2*>(cand),
                                                                    (size_t)L.cap, k, flags);
        SVDB_LAUNCH_CHECK();
        ++R.kernels;
    }
    R.kernels += 2;
    s->prof_mark(4);

    {
        if (!gc->rerank_attr) {
            SVDB_CUDA(cudaFuncSetAttribute(k_rerank_small<true, kSmallRerank>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
            SVDB_CUDA(cudaFuncSetAttribute(k_rerank_small<false, kSmallRerank>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
            SVDB_CUDA(cudaFuncSetAttribute(k_rerank_small<true, kLargeRerank>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
            SVDB_CUDA(cudaFuncSetAttribute(k_rerank_small<false, kLargeRerank>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
            gc->rerank_attr = true;
        }
        const bool euc = a.metric == SVDB_EUCLIDEAN;
        const size_t sm_small = s->ld * sizeof(double) + (size_t)kSmallRerank * (8 + 8 + 4 + 4);
        const size_t sm_large = s->ld * sizeof(double) + (size_t)kLargeRerank * (8 + 8 + 4 + 4);
        auto rr_small = euc ? k_rerank_small<true, kSmallRerank> : k_rerank_small<false, kSmallRerank>;
        auto rr_large = euc ? k_rerank_small<true, kLargeRerank> : k_rerank_small<false, kLargeRerank>;
        rr_small<<<(unsigned)nq, 256, sm_small, s->stream>>>(s->x64, s->ld, a.q, a.qsq, s->sq64, cand, L.cap, nref, k,
                                                             a.metric, (int)s->dim, rpar, qpar, s->logical, a.ids,
                                                             a.dists, a.err, flags);
        SVDB_LAUNCH_CHECK();
        rr_large<<<(unsigned)nq, 256, sm_large, s->stream>>>(s->x64, s->ld, a.q, a.qsq, s->sq64, cand, L.cap, nref, k,
                                                             a.metric, (int)s->dim, rpar, qpar, s->logical, a.ids,
                                                             a.dists, a.err, flags);
        SVDB_LAUNCH_CHECK();
        R.kernels += 2;
    }

    // queries the screen could not certify: exact FP64 scan, entirely on the
    // device (no host round trip; with nothing to redo the kernels exit at once)
    k_collect_redo<<<(unsigned)((a.nq + 255) / 256), 256, 0, s->stream>>>(flags, cnt, R.nsub_use, nsurv, nref, nq, redo,
                                                                          redo_n, dstats);
    SVDB_LAUNCH_CHECK();
    {
        double* rq = R.at<double>(L.rq);
        double* rsq = R.at<double>(L.rsq);
        int64_t* rids = R.at<int64_t>(L.rres);
        double* rd = reinterpret_cast<double*>(rids + a.nq * a.k);
        double* re = rd + a.nq * a.k;
        k_gather_queries<<<(unsigned)nq, 256, 0, s->stream>>>(a.q, a.qsq, s->ld, redo, redo_n, rq, rsq);
        SVDB_LAUNCH_CHECK();
        SearchArgs b = a;
        b.q = rq;
        b.qsq = rsq;
        b.ids = rids;
        b.dists = rd;
        b.err = re;
        b.nq_dev = redo_n;
        uint32_t kk = 0;
        rc = search_fp64(s, b, R.base + L.rscr, search_fp64_scratch(s, a.nq, a.k), &kk, false);
        if (rc) return rc;
        k_scatter_results<<<(unsigned)((a.nq * a.k + 255) / 256), 256, 0, s->stream>>>(rids, rd, re, redo, redo_n,
                                                                                    (int)a.k, a.ids, a.dists, a.err);
        SVDB_LAUNCH_CHECK();
        R.kernels += kk + 3;
    }
    if (st) {  // statistics cost a host round trip: only when asked for
        unsigned long long h[5];
        SVDB_CUDA(cudaMemcpyAsync(h, dstats, sizeof(h), cudaMemcpyDeviceToHost, s->stream));
        SVDB_CUDA(cudaStreamSynchronize(s->stream));
        st->candidates += h[0];
        st->survivors += h[1];
        st->reranked += h[2];
        st->widened += (uint32_t)h[3];
        st->bound_failures += (uint32_t)h[4];
    }
    s->prof_mark(5);
    if (st) st->kernels += R.kernels;
    return SVDB_OK;
}

int search_bf16(Store* s, const SearchArgs& a, void* scratch, size_t scratch_bytes, svdb_search_stats* st, bool f8) {
    Bf16Run* R = new (std::nothrow) Bf16Run();  // (the schedule table makes it ~9 KB)
    if (!R) {
        svdb_set_error("search_bf16: out of host memory");
        return SVDB_ENOMEM;
    }
    int rc = bf16_begin(*R, s, a, scratch, scratch_bytes, f8, 0);
    if (!rc) rc = bf16_screen(*R);
    // the refinement and re-rank read the canonical |q|^2 (the screen did not)
    if (!rc && a.qsq_ready && cudaStreamWaitEvent(s->stream, a.qsq_ready, 0) != cudaSuccess) {
        svdb_set_error("search_bf16: cudaStreamWaitEvent: %s", cudaGetErrorString(cudaGetLastError()));
        rc = SVDB_ECUDA;
    }
    if (!rc) {
        s->prof_mark(2);
        rc = bf16_end(*R, st);
    }
    delete R;
    return rc;
}

// ---------------------------------------------------------------------------
// fused screens: several BF16 searches (up to 16) screened by one launch
// ---------------------------------------------------------------------------
// A search's screen is one pass of tensor-core tiles over its store; a batch
// spread over several stores (different dimensions, row counts and query
// counts) screened one launch per search leaves SMs idle at the tail of each
// launch and, for small searches, most of the launch.  A fused launch takes
// up to 16 searches together: every search gets a share of the
// launch's CTAs in proportion to its work (query tiles x store tiles x
// (k blocks + epilogue weight)), given out greedily to the search with the
// most work per CTA, and inside its share the single-search schedule
// (screen_schedule).  Each CTA's segments then carry their search, whose
// parameters and query tensor map travel in the launch's parameter space.
struct FusedPlan {
    struct Launch {
        std::vector<int> items;  // search of each group slot
        ScreenParamsMulti P;
        int nctas = 0;
    };
    std::vector<FusedItem> items;
    int metric = 0;
    std::vector<int> maxsub;     // per item
    std::vector<int> tbase;      // per item: its first query tile in its launch's schedule
    std::vector<size_t> qoff;    // per item: offset of the screen's scratch after the padded queries
    std::vector<size_t> bytes;   // per item
    std::vector<int> launch_of, slot_of;
    std::vector<Bf16Run*> runs;
    std::vector<Launch*> launches;
    ~FusedPlan() {
        for (Bf16Run* r : runs) delete r;
        for (Launch* l : launches) delete l;
    }
};

// CTAs of the fused launch for each job, then the jobs' segments; false when
// the launch's tables cannot hold the schedule
static bool fused_schedule(const std::vector<int>& ntq, const std::vector<int>& ntr, const std::vector<int>& kb,
                           int units, double epi_weight, ScreenSchedMulti& S, std::vector<int>& maxsub,
                           std::vector<int>& tbase, int* nctas) {
    const size_t n = ntq.size();
    std::memset(&S, 0, sizeof(S));
    if ((int)n > units) return false;
    std::vector<double> w(n);
    for (size_t i = 0; i < n; ++i) w[i] = (double)ntq[i] * ntr[i] * (kb[i] + epi_weight);
    std::vector<int> u(n, 1);
    for (int left = units - (int)n; left > 0; --left) {
        size_t best = 0;
        for (size_t i = 1; i < n; ++i)
            if (w[i] / u[i] > w[best] / u[best]) best = i;
        ++u[best];
    }
    int c = 0, gq = 0;
    maxsub.assign(n, 1);
    tbase.assign(n, 0);
    ScreenSched* one = new (std::nothrow) ScreenSched();
    if (!one) return false;
    bool ok = true;
    for (size_t i = 0; i < n && ok; ++i) {
        int ms = 1;
        const int cg = screen_schedule(ntq[i], ntr[i], *one, &ms, u[i]);
        if (c + cg > kMaxUnitsM || gq + ntq[i] > kMaxQTilesM) {
            ok = false;
            break;
        }
        for (int j = 0; j < cg; ++j) {
            const int ns = one->direct ? 1 : one->nseg[j];
            for (int sg = 0; sg < ns; ++sg) {
                ScreenSeg e = one->direct ? ScreenSeg{0, ntr[i], (uint16_t)j, 0, 0, (uint16_t)j} : one->seg[j][sg];
                e.grp = (uint16_t)i;
                e.gq = (uint16_t)(gq + e.qt);
                S.seg[c + j][sg] = e;
            }
            S.nseg[c + j] = (uint8_t)ns;
        }
        for (int q = 0; q < ntq[i]; ++q) {
            S.nsq[gq + q] = one->direct ? 1 : one->nsq[q];
            S.nst[gq + q] = one->direct ? 1 : one->nst[q];
        }
        maxsub[i] = ms;
        tbase[i] = gq;
        c += cg;
        gq += ntq[i];
    }
    delete one;
    S.direct = 0;
    *nctas = c;
    return ok;
}

int fused_create(const std::vector<FusedItem>& items, int metric, double epi_weight, FusedPlan** out,
                 std::vector<size_t>* bytes) {
    *out = nullptr;
    FusedPlan* p = new (std::nothrow) FusedPlan();
    if (!p) {
        svdb_set_error("fused screen: out of host memory");
        return SVDB_ENOMEM;
    }
    p->items = items;
    p->metric = metric;
    const size_t n = items.size();
    p->maxsub.assign(n, 1);
    p->tbase.assign(n, 0);
    p->launch_of.assign(n, -1);
    p->slot_of.assign(n, -1);
    // launches of at most kMaxGroups searches each (any k: the screen's
    // thresholds are each search's own bins)
    {
        FusedPlan::Launch* cur = nullptr;
        for (size_t i = 0; i < n; ++i) {
            if (!cur || cur->items.size() == (size_t)kMaxGroups) {
                cur = new (std::nothrow) FusedPlan::Launch();
                if (!cur) {
                    delete p;
                    svdb_set_error("fused screen: out of host memory");
                    return SVDB_ENOMEM;
                }
                p->launches.push_back(cur);
            }
            p->launch_of[i] = (int)p->launches.size() - 1;
            p->slot_of[i] = (int)cur->items.size();
            cur->items.push_back((int)i);
        }
    }
    const int units = num_sms();
    for (FusedPlan::Launch* l : p->launches) {
        std::vector<int> ntq, ntr, kb, ms, tb;
        for (int i : l->items) {
            const Store* s = items[i].s;
            ntq.push_back((int)((items[i].nq + scr::kBM - 1) / scr::kBM));
            ntr.push_back((int)((std::max<size_t>(s->slots, 1) + scr::kBN - 1) / scr::kBN));
            kb.push_back((int)(s->ldb / scr::kBK));
        }
        if (!fused_schedule(ntq, ntr, kb, units, epi_weight, l->P.sched, ms, tb, &l->nctas)) {
            delete p;
            svdb_set_error("fused screen: the searches do not fit one launch's schedule");
            return SVDB_EINVAL;
        }
        for (size_t j = 0; j < l->items.size(); ++j) {
            p->maxsub[l->items[j]] = ms[j];
            p->tbase[l->items[j]] = tb[j];
        }
    }
    bytes->assign(n, 0);
    p->qoff.assign(n, 0);
    for (size_t i = 0; i < n; ++i) {
        const Store* s = items[i].s;
        p->qoff[i] = round_up(items[i].nq * s->ld * sizeof(double), 1024) + round_up(items[i].nq * sizeof(double), 1024);
        (*bytes)[i] = p->qoff[i] + bf16_layout(s, items[i].nq, p->maxsub[i]).total;
        Bf16Run* r = new (std::nothrow) Bf16Run();
        if (!r) {
            delete p;
            svdb_set_error("fused screen: out of host memory");
            return SVDB_ENOMEM;
        }
        p->runs.push_back(r);
    }
    p->bytes = *bytes;
    *out = p;
    return SVDB_OK;
}

void fused_set_scratch(FusedPlan* p, size_t i, void* scratch) { p->items[i].scratch = scratch; }

size_t fused_launches(const FusedPlan* p) { return p->launches.size(); }
int fused_launch_of(const FusedPlan* p, size_t i) { return p->launch_of[i]; }

int fused_begin(FusedPlan* p, size_t i) {
    const FusedItem& it = p->items[i];
    Store* s = it.s;
    uint8_t* base = reinterpret_cast<uint8_t*>(it.scratch);
    double* qbuf = reinterpret_cast<double*>(base);
    double* qsq = reinterpret_cast<double*>(base + round_up(it.nq * s->ld * sizeof(double), 1024));
    int rc = prep_queries_fp64(s, it.q, s->dim, it.nq, qbuf, qsq);
    if (rc) return rc;
    SearchArgs a;
    a.q = qbuf;
    a.qsq = qsq;
    a.nq = it.nq;
    a.k = it.k;
    a.metric = p->metric;
    a.seed = it.seed;
    a.ids = it.ids;
    a.dists = it.dists;
    a.err = nullptr;
    Bf16Run& R = *p->runs[i];
    rc = bf16_begin(R, s, a, base + p->qoff[i], p->bytes[i] - p->qoff[i], false, p->maxsub[i]);
    if (rc) return rc;
    FusedPlan::Launch* l = p->launches[p->launch_of[i]];
    l->P.map[p->slot_of[i]] = R.tmq;
    l->P.grp[p->slot_of[i]] = R.P.g;

    return SVDB_OK;
}

int fused_screen(FusedPlan* p, size_t li, cudaStream_t st) {
    FusedPlan::Launch* l = p->launches[li];
    if (l->nctas == 0) return SVDB_OK;
    const bool norm = p->metric == SVDB_COSINE;
    auto kern = norm ? k_screen_bf16<true, false, false, false, true> : k_screen_bf16<false, false, false, false, true>;
    static bool attr[2] = {};
    const int v = norm ? 1 : 0;
    const size_t smem = sizeof(scr::Smem) + 1024;
    if (!attr[v]) {
        SVDB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr[v] = true;
    }
    const CUtensorMap& any = l->P.map[0];
    kern<<<(unsigned)l->nctas, scr::kThreads, smem, st>>>(any, any, l->P);
    SVDB_LAUNCH_CHECK();
    return SVDB_OK;
}

int fused_end(FusedPlan* p, size_t i) { return bf16_end(*p->runs[i], nullptr); }

int fused_stats(FusedPlan* p, size_t i, unsigned long long* out) {
    const Bf16Run& R = *p->runs[i];
    if (!R.base) {
        std::memset(out, 0, scr::kStats * sizeof(unsigned long long));
        return SVDB_OK;
    }
    SVDB_CUDA(cudaStreamSynchronize(R.s->stream));
    SVDB_CUDA(cudaMemcpy(out, R.at<unsigned long long>(R.L.stats), scr::kStats * sizeof(unsigned long long),
                         cudaMemcpyDeviceToHost));
    return SVDB_OK;
}

void fused_destroy(FusedPlan* p) { delete p; }

// ---------------------------------------------------------------------------
// self-test of the bounded waits (no fault, no hang)
// ---------------------------------------------------------------------------
// The screen's roles wait on mbarriers through mbar_wait: a wait that runs out
// raises the CTA's abort flag, every other role leaves its own wait when it
// sees the flag, the TMEM allocation is released and the kernel reports
// through the store's error word.  This kernel runs that same sequence on
// mbarriers that nothing ever arrives on: warp 0 waits with `limit_ns`, warp 1
// holds TMEM and waits with the full limit, so it can only leave through the
// abort flag.  `gave_up` gets bit w for each warp whose wait returned false.
__global__ void __launch_bounds__(64, 1) k_selftest_wait(uint64_t limit_ns, int* err, uint32_t* gave_up) {
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        abort_flag = 0;
    }
    if (warp == 1) tmem_alloc(&tmem_base, 32);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    volatile int* ab = &abort_flag;
    if (lane == 0) {
        const bool ok = mbar_wait(&bar[warp], 0, ab, warp == 0 ? limit_ns : scr::kWaitLimitNs);
        if (!ok) atomicOr(gave_up, 1u << warp);
    }
    __syncwarp();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (threadIdx.x == 0 && abort_flag) atomicExch(err, 1);
    if (warp == 1) tmem_dealloc(tmem_base, 32);
}

int selftest_wait(Store* s, uint32_t limit_us, uint32_t* gave_up) {
    int rc = s->ensure();
    if (!rc) rc = s->scratch_reserve(sizeof(uint32_t));
    if (rc) return rc;
    uint32_t* d_gave = reinterpret_cast<uint32_t*>(s->scratch);
    SVDB_CUDA(cudaMemsetAsync(d_gave, 0, sizeof(uint32_t), s->stream));
    const uint64_t lim = (uint64_t)std::min<uint32_t>(std::max<uint32_t>(limit_us, 1u), 1000000u) * 1000ull;
    k_selftest_wait<<<1, 64, 0, s->stream>>>(lim, s->d_err, d_gave);
    SVDB_LAUNCH_CHECK();
    uint32_t h = 0;
    SVDB_CUDA(cudaMemcpyAsync(&h, d_gave, sizeof(h), cudaMemcpyDeviceToHost, s->stream));
    SVDB_CUDA(cudaStreamSynchronize(s->stream));
    if (gave_up) *gave_up = h;
    return s->check_error();
}

// ---------------------------------------------------------------------------
// diagnostics: the screen's raw accumulators and the operands behind them
// ---------------------------------------------------------------------------
// Runs the screen kernel (DUMP form: same producer, same MMA issue sequence,
// same tiles and descriptors; the paired form for more than 128 queries) for
// up to 256 host queries against the store's
// first `rows` slots and returns every raw FP32 accumulator value, the query
// operand the MMAs read (BF16, or E4M3 scaled by the query's power of two) and
// the rows' shadow operand (un-swizzled), so the accumulation can be compared
// with an exact sum of the same products.  Not a search: nothing screened.
int debug_screen_acc(Store* s, const double* hq, size_t nq, int metric, bool f8, size_t rows, float* acc,
                     void* qops, void* rops, size_t* opbytes) {
    if (nq == 0 || nq > 2 * (size_t)scr::kBM || metric < 0 || metric > 2 || !hq || !acc) {
        svdb_set_error("debug_screen_acc: bad argument (1..256 queries)");
        return SVDB_EINVAL;
    }
    int rc = s->sync();
    if (rc) return rc;
    if (rows == 0 || rows > s->slots) {
        svdb_set_error("debug_screen_acc: rows must be 1..%zu", s->slots);
        return SVDB_EINVAL;
    }
    GemmPlanCache* gc = nullptr;
    rc = gemm_cache(s, &gc);
    if (rc) return rc;
    const bool norm = metric == SVDB_COSINE;
    const size_t ob = f8 ? s->ldb8 : s->ldb * 2;  // operand bytes per row
    if (opbytes) *opbytes = ob;
    const size_t ntiles = (rows + scr::kBN - 1) / scr::kBN, dld = ntiles * scr::kBN;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off += round_up(bytes, 1024);
        return o;
    };
    const size_t o_raw = take(nq * s->dim * sizeof(double)), o_qbuf = take(nq * s->ld * sizeof(double)),
                 o_qsq = take(nq * sizeof(double)), o_qb = take(nq * std::max(s->ldb * 2, s->ldb8)),
                 o_q32 = take(nq * s->ld * sizeof(float)), o_qpar = take(nq * sizeof(float4)),
                 o_qscale = take(nq * sizeof(float)), o_spar = take(dld * sizeof(float4)), o_alpha = take(sizeof(int)),
                 o_dump = take(nq * dld * sizeof(float));
    rc = s->scratch_reserve(off);
    if (rc) return rc;
    uint8_t* base = reinterpret_cast<uint8_t*>(s->scratch);
    double* qraw = reinterpret_cast<double*>(base + o_raw);
    double* qbuf = reinterpret_cast<double*>(base + o_qbuf);
    double* qsq = reinterpret_cast<double*>(base + o_qsq);
    void* qb = base + o_qb;
    float* q32 = reinterpret_cast<float*>(base + o_q32);
    float4* qpar = reinterpret_cast<float4*>(base + o_qpar);
    float* qscale = reinterpret_cast<float*>(base + o_qscale);
    float* dump = reinterpret_cast<float*>(base + o_dump);
    SVDB_CUDA(cudaMemcpyAsync(qraw, hq, nq * s->dim * sizeof(double), cudaMemcpyHostToDevice, s->stream));
    rc = prep_queries_fp64(s, qraw, s->dim, nq, qbuf, qsq);
    if (rc) return rc;
    if (f8)
        k_prep_f8<<<(unsigned)((nq * kPrepLanes + 255) / 256), 256, 0, s->stream>>>(
            qbuf, (int)nq, s->ld, s->ldb8, metric, reinterpret_cast<uint8_t*>(qb), q32, qpar, qscale);
    else
        k_prep_bf16<<<(unsigned)((nq * kPrepLanes + 255) / 256), 256, 0, s->stream>>>(
            qbuf, (int)nq, s->ld, s->ldb, metric, reinterpret_cast<__nv_bfloat16*>(qb), q32, qpar);
    SVDB_LAUNCH_CHECK();
    CUtensorMap tmq;
    rc = f8 ? make_map8(gc, &tmq, qb, nq, s->ldb8, scr::kBM) : make_map(gc, &tmq, qb, nq, s->ldb, scr::kBM);
    if (rc) return rc;
    ScreenParams P;
    std::memset(&P, 0, sizeof(P));
    P.g.xblk = reinterpret_cast<const uint8_t*>(f8 ? (norm ? (const void*)s->xbn8 : (const void*)s->xb8)
                                                 : norm ? (const void*)s->xbn : (const void*)s->xb);
    P.g.qscale = qscale;
    P.g.spar = reinterpret_cast<const float4*>(base + o_spar);
    P.g.alpha = reinterpret_cast<const int*>(base + o_alpha);
    P.g.nmax = s->d_count + (f8 ? 3 : 1);
    P.g.qpar = qpar;
    P.g.err = s->d_err;
    P.g.dump = dump;
    P.g.dump_ld = dld;
    P.g.nq = (int)nq;
    P.g.k = 1;
    P.g.kblocks = f8 ? (int)(s->ldb8 / (2 * scr::kBK)) : (int)(s->ldb / scr::kBK);
    P.sched.direct = 1;
    P.sched.ntr = (int)ntiles;
    P.g.ntr = (int)ntiles;
    // more than 128 queries: the paired form (one cluster of two CTAs, M = 256)
    const bool pair = nq > (size_t)scr::kBM;
    if (!pair) {
        auto kern = f8 ? (norm ? k_screen_bf16<true, true, true> : k_screen_bf16<false, true, true>)
                       : norm ? k_screen_bf16<true, false, true> : k_screen_bf16<false, false, true>;
        SVDB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gc->screen_smem));
        rc = launch_screen(kern, false, 1, gc->screen_smem, s->stream, tmq, tmq, P);
    } else {
        auto kern = f8 ? (norm ? k_screen_bf16<true, true, true, true> : k_screen_bf16<false, true, true, true>)
                       : norm ? k_screen_bf16<true, false, true, true> : k_screen_bf16<false, false, true, true>;
        SVDB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gc->screen_smem_pair));
        CUtensorMap tmx;
        const size_t kbl = f8 ? s->ldb8 / (2 * scr::kBK) : s->ldb / scr::kBK;
        const size_t ntr_all = (std::max<size_t>(s->slots, 1) + scr::kBN - 1) / scr::kBN;
        rc = make_map_tiles(gc, &tmx, P.g.xblk, ntr_all * kbl * scr::kBN);
        if (!rc) rc = launch_screen(kern, true, 1, gc->screen_smem_pair, s->stream, tmq, tmx, P);
    }
    if (rc) return rc;
    std::vector<float> hacc(nq * dld);
    SVDB_CUDA(cudaMemcpyAsync(hacc.data(), dump, hacc.size() * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    std::vector<uint8_t> hx;
    if (rops) {
        hx.resize(dld * ob);
        SVDB_CUDA(cudaMemcpyAsync(hx.data(), P.g.xblk, hx.size(), cudaMemcpyDeviceToHost, s->stream));
    }
    if (qops) SVDB_CUDA(cudaMemcpyAsync(qops, qb, nq * ob, cudaMemcpyDeviceToHost, s->stream));
    SVDB_CUDA(cudaStreamSynchronize(s->stream));
    rc = s->check_error();
    if (rc) return rc;
    for (size_t q = 0; q < nq; ++q) std::memcpy(acc + q * rows, hacc.data() + q * dld, rows * sizeof(float));
    if (rops) {
        uint8_t* out = reinterpret_cast<uint8_t*>(rops);
        for (size_t r = 0; r < rows; ++r) {
            if (f8)
                for (size_t e = 0; e < ob; ++e) out[r * ob + e] = hx[f8_tile_index((int64_t)r, e, s->ldb8)];
            else
                for (size_t e = 0; e < ob / 2; ++e)
                    std::memcpy(out + r * ob + 2 * e, hx.data() + 2 * bf16_tile_index((int64_t)r, e, s->ldb), 2);
        }
    }
    return SVDB_OK;
}

}  // namespace svdb

extern "C" int svdbd_selftest_wait(svdbd_store* hs, uint32_t limit_us, uint32_t* gave_up) {
    return svdb::selftest_wait(reinterpret_cast<svdb::Store*>(hs), limit_us, gave_up);
}

extern "C" int svdbd_debug_screen_acc(svdbd_store* hs, const double* q, size_t nq, int metric, int f8, size_t rows,
                                      float* acc, void* qops, void* rops, size_t* opbytes) {
    return svdb::debug_screen_acc(reinterpret_cast<svdb::Store*>(hs), q, nq, metric, f8 != 0, rows, acc, qops, rops,
                                  opbytes);
}
