// dev_search.cu -- exact FP64 top-k: streaming scan of the master copy with
// a fused warp-level top-k, a block merge and a per-query grid merge; plus
// the search entry point that dispatches FP64 / BF16 precision.
//
// Roofline: one query reads every live row once (N * D * 8 bytes) and does
// one FP64 FMA per element (two FP64 ops for Euclidean).  GB300's FP64 rate
// is low enough that a single-query scan is bounded by the FP64 pipe rather
// than by HBM; a batch of QB queries shares each loaded row (QB FMAs per
// 8 bytes) and is FP64-bound.
#include <algorithm>
#include <cstring>

#include "dev_search.cuh"

namespace svdb {

int num_sms() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
            cudaGetLastError();
            n = 148;
        }
    }
    return n;
}

__global__ void k_prep_queries(const double* __restrict__ q, size_t qs, int nq, int d, size_t ld,
                               double* __restrict__ qbuf, double* __restrict__ qsq) {
    const int lane = threadIdx.x & 31, s = lane & 3;
    const int qi = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 2);
    const bool active = qi < nq;
    double p = 0.0;
    if (active) {
        const double* src = q + (size_t)qi * qs;
        double* dst = qbuf + (size_t)qi * ld;
        for (size_t j = 2 * s; j < ld; j += 8) {
            const double a = j < (size_t)d ? src[j] : 0.0;
            const double b = j + 1 < (size_t)d ? src[j + 1] : 0.0;
            dst[j] = a;
            dst[j + 1] = b;
            p = fma(a, a, p);
            p = fma(b, b, p);
        }
    }
    p = group4_sum(p);
    if (active && s == 0) qsq[qi] = p;
}

// The canonical sums of squares alone, with exactly k_prep_queries'
// arithmetic (so the values are identical), and the padded copy alone, one
// thread per element.  A search whose screen needs no canonical |q|^2 runs the
// first beside its screen on the store's side stream.
__global__ void k_query_sq(const double* __restrict__ q, size_t qs, int nq, int d, size_t ld,
                           double* __restrict__ qsq) {
    const int lane = threadIdx.x & 31, s = lane & 3;
    const int qi = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 2);
    const bool active = qi < nq;
    double p = 0.0;
    if (active) {
        const double* src = q + (size_t)qi * qs;
        for (size_t j = 2 * s; j < ld; j += 8) {
            const double a = j < (size_t)d ? src[j] : 0.0;
            const double b = j + 1 < (size_t)d ? src[j + 1] : 0.0;
            p = fma(a, a, p);
            p = fma(b, b, p);
        }
    }
    p = group4_sum(p);
    if (active && s == 0) qsq[qi] = p;
}

__global__ void k_pad_queries(const double* __restrict__ q, size_t qs, int64_t n, int d, size_t ld,
                              double* __restrict__ qbuf) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;  // element of the nq x ld buffer
    if (i >= n) return;
    const int64_t qi = i / (int64_t)ld;
    const size_t j = (size_t)(i - qi * (int64_t)ld);
    qbuf[i] = j < (size_t)d ? q[(size_t)qi * qs + j] : 0.0;
}

int prep_queries_split(Store* s, const double* q_dev, size_t qs, size_t nq, double* qbuf, double* qsq,
                       cudaEvent_t* ready) {
    *ready = nullptr;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s->stream, &cs) != cudaSuccess) {
        cudaGetLastError();
        cs = cudaStreamCaptureStatusActive;
    }
    if (cs != cudaStreamCaptureStatusNone || s->side_ready() != SVDB_OK) return prep_queries_fp64(s, q_dev, qs, nq, qbuf, qsq);
    SVDB_CUDA(cudaEventRecord(s->ev_fork, s->stream));  // the queries are in place (their upload is on the stream)
    SVDB_CUDA(cudaStreamWaitEvent(s->side, s->ev_fork, 0));
    k_query_sq<<<(unsigned)((nq * 4 + 255) / 256), 256, 0, s->side>>>(q_dev, qs, (int)nq, (int)s->dim, s->ld, qsq);
    SVDB_LAUNCH_CHECK();
    SVDB_CUDA(cudaEventRecord(s->ev_side, s->side));
    const int64_t n = (int64_t)nq * (int64_t)s->ld;
    k_pad_queries<<<(unsigned)((n + 255) / 256), 256, 0, s->stream>>>(q_dev, qs, n, (int)s->dim, s->ld, qbuf);
    SVDB_LAUNCH_CHECK();
    *ready = s->ev_side;
    return SVDB_OK;
}

int prep_queries_fp64(Store* s, const double* q_dev, size_t qs, size_t nq, double* qbuf, double* qsq) {
    k_prep_queries<<<(unsigned)((nq * 4 + 255) / 256), 256, 0, s->stream>>>(q_dev, qs, (int)nq, (int)s->dim, s->ld,
                                                                         qbuf, qsq);
    SVDB_LAUNCH_CHECK();
    return SVDB_OK;
}

// ---------------------------------------------------------------------------
// scan: grid (slices, query blocks); block = 8 warps; warp = 8 row groups of
// 4 lanes; a row group reduces one row for QB queries in canonical order.
// ---------------------------------------------------------------------------
template <int QB, int KS, bool EUC>
__global__ void __launch_bounds__(256) k_scan_fp64(const double* __restrict__ x64, size_t ld,
                                                   const uint8_t* __restrict__ live,
                                                   const double* __restrict__ sq64, int64_t nslots,
                                                   int64_t rows_per_slice, const double* __restrict__ qbuf,
                                                   const double* __restrict__ qsq, int nq, int metric, int k,
                                                   Entry* __restrict__ part, int nslices,
                                                   const int* __restrict__ nq_dev, int* __restrict__ err_flag) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t qbar;
    if (nq_dev) nq = min(nq, *nq_dev);
    if ((int)blockIdx.y * QB >= nq) return;  // whole block beyond the answered queries
    double* qs = reinterpret_cast<double*>(smem_raw);
    const int qb0 = blockIdx.y * QB;
    const int slice = blockIdx.x;
    // The query tile: one bulk copy per query row (rows are ld doubles, a
    // multiple of 128 bytes, from a 16-byte aligned buffer) completing on
    // qbar; rows past the last query are zero-filled with plain stores.
    const int nrow = min(QB, nq - qb0);
    if (threadIdx.x == 0) {
        mbar_init(&qbar, 1);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(&qbar, (uint32_t)((size_t)nrow * ld * sizeof(double)));
        for (int qi = 0; qi < nrow; ++qi)
            bulk_load(qs + (size_t)qi * ld, qbuf + (size_t)(qb0 + qi) * ld, (uint32_t)(ld * sizeof(double)), &qbar);
    }
    for (size_t i = (size_t)nrow * ld + threadIdx.x; i < (size_t)QB * ld; i += blockDim.x) qs[i] = 0.0;
    __syncthreads();  // qbar initialised before anyone waits on it
    const bool got = mbar_wait_for(&qbar, 0, 2000000000ull);
    if (__syncthreads_or(!got)) {
        // the copy did not complete within 2 s: report it, give the copies in
        // flight one more bounded wait, and leave without results
        if (threadIdx.x == 0) {
            if (err_flag) atomicExch(err_flag, 1);
            mbar_wait_for(&qbar, 0, 2000000000ull);
        }
        __syncthreads();
        return;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, s = lane & 3;
    double qn[QB];
#pragma unroll
    for (int qi = 0; qi < QB; ++qi) qn[qi] = qb0 + qi < nq ? sqrt(qsq[qb0 + qi]) : 1.0;

    WarpList<KS> L[QB];
#pragma unroll
    for (int qi = 0; qi < QB; ++qi) L[qi].init();

    const int64_t r0 = (int64_t)slice * rows_per_slice;
    const int64_t r1 = min(nslots, r0 + rows_per_slice);
    for (int64_t base = r0 + warp * 8; base < r1; base += 64) {
        const int64_t row = base + g;
        const bool inrange = row < r1;
        const bool valid = inrange && live[row] == 1;
        double p[QB];
#pragma unroll
        for (int qi = 0; qi < QB; ++qi) p[qi] = 0.0;
        if (valid) {
            const double* x = x64 + row * ld;
            for (size_t j = 2 * s; j < ld; j += 8) {
                const double2 v = __ldcs(reinterpret_cast<const double2*>(x + j));
#pragma unroll
                for (int qi = 0; qi < QB; ++qi) {
                    const double2 qv = *reinterpret_cast<const double2*>(qs + qi * ld + j);
                    if (EUC) {
                        const double t0 = qv.x - v.x, t1 = qv.y - v.y;
                        p[qi] = fma(t0, t0, p[qi]);
                        p[qi] = fma(t1, t1, p[qi]);
                    } else {
                        p[qi] = fma(qv.x, v.x, p[qi]);
                        p[qi] = fma(qv.y, v.y, p[qi]);
                    }
                }
            }
        }
        const double xn = (valid && metric == SVDB_COSINE) ? sqrt(sq64[row]) : 1.0;
#pragma unroll
        for (int qi = 0; qi < QB; ++qi) {
            const double v = group4_sum(p[qi]);
            double val;
            if (EUC)
                val = sqrt(v);
            else if (metric == SVDB_COSINE)
                val = v / (qn[qi] * xn);
            else
                val = v;
            const double key = rank_key(metric, val);
            double wk;
            int wi;
            L[qi].worst(k, wk, wi);
            const bool cand = valid && s == 0 && (qb0 + qi < nq) && key_less(key, (int)row, wk, wi);
            unsigned m = __ballot_sync(0xffffffffu, cand);
            while (m) {
                const int src = __ffs(m) - 1;
                m &= m - 1;
                const double ck = __shfl_sync(0xffffffffu, key, src);
                const double cv = __shfl_sync(0xffffffffu, val, src);
                const int ci = __shfl_sync(0xffffffffu, (int)row, src);
                L[qi].insert(ck, ci, cv, k);
            }
        }
    }
    __syncthreads();  // query tile no longer needed: reuse shared memory for the block merge
    const int KP = 32 * KS;
    Entry* lists = reinterpret_cast<Entry*>(smem_raw);  // [warp][qi][KP]
#pragma unroll
    for (int qi = 0; qi < QB; ++qi)
#pragma unroll
        for (int t = 0; t < KS; ++t) {
            Entry e;
            e.val = L[qi].val[t];
            e.id = L[qi].id[t];
            e.pad = 0;
            lists[(warp * QB + qi) * KP + t * 32 + lane] = e;
        }
    __syncthreads();
    if (warp < QB && qb0 + warp < nq) {
        const int qi = warp;
        WarpList<KS> M;
        M.init();
        for (int w = 0; w < 8; ++w) {
            for (int c = 0; c < k; c += 32) {
                const int p = c + lane;
                Entry e = lists[(w * QB + qi) * KP + min(p, KP - 1)];
                const double key = rank_key(metric, e.val);
                double wk;
                int wi;
                M.worst(k, wk, wi);
                const bool cand = p < k && e.id != 0x7fffffff && key_less(key, e.id, wk, wi);
                unsigned m = __ballot_sync(0xffffffffu, cand);
                while (m) {
                    const int src = __ffs(m) - 1;
                    m &= m - 1;
                    M.insert(__shfl_sync(0xffffffffu, key, src), __shfl_sync(0xffffffffu, e.id, src),
                             __shfl_sync(0xffffffffu, e.val, src), k);
                }
            }
        }
        Entry* out = part + ((size_t)(qb0 + qi) * nslices + slice) * k;
#pragma unroll
        for (int t = 0; t < KS; ++t) {
            const int p = t * 32 + lane;
            if (p < k) {
                Entry e;
                e.val = M.val[t];
                e.id = M.id[t];
                e.pad = 0;
                out[p] = e;
            }
        }
    }
}

// one warp per query: merge nslices x k partial lists, write logical ids
template <int KS>
__global__ void k_merge_fp64(const Entry* __restrict__ part, int nslices, int nq, const int* __restrict__ nq_dev, int k,
                             int metric, int d,
                             const int64_t* __restrict__ logical, const double* __restrict__ qsq,
                             const double* __restrict__ sq64, int64_t* __restrict__ ids, double* __restrict__ dists,
                             double* __restrict__ err) {
    const int qi = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (nq_dev) nq = min(nq, *nq_dev);
    if (qi >= nq) return;
    WarpList<KS> M;
    M.init();
    const Entry* src = part + (size_t)qi * nslices * k;
    const int total = nslices * k;
    for (int c = 0; c < total; c += 32) {
        const int p = c + lane;
        Entry e;
        e.val = 0.0;
        e.id = 0x7fffffff;
        if (p < total) e = src[p];
        const double key = rank_key(metric, e.val);
        double wk;
        int wi;
        M.worst(k, wk, wi);
        const bool cand = p < total && e.id != 0x7fffffff && key_less(key, e.id, wk, wi);
        unsigned m = __ballot_sync(0xffffffffu, cand);
        while (m) {
            const int sl = __ffs(m) - 1;
            m &= m - 1;
            M.insert(__shfl_sync(0xffffffffu, key, sl), __shfl_sync(0xffffffffu, e.id, sl),
                     __shfl_sync(0xffffffffu, e.val, sl), k);
        }
    }
#pragma unroll
    for (int t = 0; t < KS; ++t) {
        const int p = t * 32 + lane;
        if (p < k) {
            const int slot = M.id[t];
            const bool ok = slot != 0x7fffffff;
            const size_t o = (size_t)qi * k + p;
            ids[o] = ok ? logical[slot] : -1;
            dists[o] = ok ? M.val[t] : __longlong_as_double(0x7ff8000000000000ll);
            if (err)
                err[o] = ok ? result_err_bound(metric, d, M.val[t], qsq[qi], sq64[slot])
                            : __longlong_as_double(0x7ff8000000000000ll);
        }
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct ScanPlan {
    int ks, qb, nqb, nslices;
    int64_t rows_per_slice;
    size_t smem;
};

// dynamic shared memory of a scan CTA at most: the opt-in limit (227 KB)
// less the static mbarrier of the query tile
constexpr size_t kScanSmemMax = 227 * 1024 - 64;

static ScanPlan plan_scan(const Store* s, size_t nq, size_t k) {
    ScanPlan p;
    p.ks = k <= 32 ? 1 : (k <= 64 ? 2 : 4);
    const int qbmax = p.ks == 1 ? 8 : (p.ks == 2 ? 4 : 2);
    p.qb = 1;
    while (p.qb < qbmax && (size_t)p.qb * 2 <= nq && (size_t)p.qb * 2 * s->ld * sizeof(double) <= kScanSmemMax) p.qb *= 2;
    p.nqb = (int)((nq + p.qb - 1) / p.qb);
    const int target = num_sms() * 4;
    int ns = std::max(1, (target + p.nqb - 1) / p.nqb);
    const int64_t slots = (int64_t)std::max<size_t>(s->slots, 1);
    p.rows_per_slice = (int64_t)round_up((size_t)((slots + ns - 1) / ns), 64);
    p.nslices = (int)((slots + p.rows_per_slice - 1) / p.rows_per_slice);
    const size_t qbytes = (size_t)p.qb * s->ld * sizeof(double);
    const size_t lbytes = (size_t)8 * p.qb * 32 * p.ks * sizeof(Entry);
    p.smem = std::max(qbytes, lbytes);
    return p;
}

size_t search_fp64_scratch(const Store* s, size_t nq, size_t k) {
    ScanPlan p = plan_scan(s, nq, k);
    return round_up((size_t)nq * p.nslices * k * sizeof(Entry), 256);
}

template <int QB, int KS, bool EUC>
static int launch_scan(Store* s, const ScanPlan& p, const SearchArgs& a, Entry* part) {
    auto kern = k_scan_fp64<QB, KS, EUC>;
    if (p.smem > kScanSmemMax) {  // one query row of more than ~29,000 doubles
        svdb_set_error("search_fp64: dimension %zu too large for the scan's query tile", s->dim);
        return SVDB_EINVAL;
    }
    if (p.smem > 48 * 1024 - 64)  // with the static mbarrier, beyond the default 48 KB
        SVDB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p.smem));
    if (reinterpret_cast<uintptr_t>(a.q) % 16 != 0) {  // the query tile is bulk-copied
        svdb_set_error("search_fp64: query buffer not 16-byte aligned");
        return SVDB_EINVAL;
    }
    dim3 grid((unsigned)p.nslices, (unsigned)p.nqb);
    kern<<<grid, 256, p.smem, s->stream>>>(s->x64, s->ld, s->live, s->sq64, (int64_t)s->slots, p.rows_per_slice, a.q,
                                          a.qsq, (int)a.nq, a.metric, (int)a.k, part, p.nslices, a.nq_dev, s->d_err);
    SVDB_LAUNCH_CHECK();
    return SVDB_OK;
}

template <int QB, int KS>
static int launch_scan_m(Store* s, const ScanPlan& p, const SearchArgs& a, Entry* part) {
    return a.metric == SVDB_EUCLIDEAN ? launch_scan<QB, KS, true>(s, p, a, part)
                                      : launch_scan<QB, KS, false>(s, p, a, part);
}

int search_fp64(Store* s, const SearchArgs& a, void* scratch, size_t scratch_bytes, uint32_t* kernels, bool marks) {
    ScanPlan p = plan_scan(s, a.nq, a.k);
    Entry* part = reinterpret_cast<Entry*>(scratch);
    if (search_fp64_scratch(s, a.nq, a.k) > scratch_bytes) {
        svdb_set_error("search_fp64: scratch too small");
        return SVDB_EINVAL;
    }
    int rc = SVDB_EINVAL;
    switch (p.ks * 100 + p.qb) {
        case 101: rc = launch_scan_m<1, 1>(s, p, a, part); break;
        case 102: rc = launch_scan_m<2, 1>(s, p, a, part); break;
        case 104: rc = launch_scan_m<4, 1>(s, p, a, part); break;
        case 108: rc = launch_scan_m<8, 1>(s, p, a, part); break;
        case 201: rc = launch_scan_m<1, 2>(s, p, a, part); break;
        case 202: rc = launch_scan_m<2, 2>(s, p, a, part); break;
        case 204: rc = launch_scan_m<4, 2>(s, p, a, part); break;
        case 401: rc = launch_scan_m<1, 4>(s, p, a, part); break;
        case 402: rc = launch_scan_m<2, 4>(s, p, a, part); break;
        default: svdb_set_error("search_fp64: no kernel for ks=%d qb=%d", p.ks, p.qb);
    }
    if (rc) return rc;
    if (marks) s->prof_mark(2);
    const unsigned blocks = (unsigned)((a.nq * 32 + 255) / 256);
    switch (p.ks) {
        case 1:
            k_merge_fp64<1><<<blocks, 256, 0, s->stream>>>(part, p.nslices, (int)a.nq, a.nq_dev, (int)a.k, a.metric, (int)s->dim,
                                                          s->logical, a.qsq, s->sq64, a.ids, a.dists, a.err);
            break;
        case 2:
            k_merge_fp64<2><<<blocks, 256, 0, s->stream>>>(part, p.nslices, (int)a.nq, a.nq_dev, (int)a.k, a.metric, (int)s->dim,
                                                          s->logical, a.qsq, s->sq64, a.ids, a.dists, a.err);
            break;
        default:
            k_merge_fp64<4><<<blocks, 256, 0, s->stream>>>(part, p.nslices, (int)a.nq, a.nq_dev, (int)a.k, a.metric, (int)s->dim,
                                                          s->logical, a.qsq, s->sq64, a.ids, a.dists, a.err);
    }
    SVDB_LAUNCH_CHECK();
    if (marks) s->prof_mark(3);
    if (kernels) *kernels += 2;
    return SVDB_OK;
}

__global__ void k_fill_empty(int64_t* ids, double* dists, double* err, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        ids[i] = -1;
        dists[i] = __longlong_as_double(0x7ff8000000000000ll);
        if (err) err[i] = __longlong_as_double(0x7ff8000000000000ll);
    }
}

}  // namespace svdb

using namespace svdb;

// Host memory the DMA engines can read directly (cudaHostAlloc'd or registered).
static bool host_pinned(const void* p) {
    if (!p) return false;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeHost;
}

extern "C" int svdbd_search(svdbd_store* hs, const double* q, size_t nq, size_t k, int metric, int precision,
                            int64_t* ids, double* dists, double* err, int on_device, svdb_search_stats* st) {
    return search_seeded(reinterpret_cast<Store*>(hs), q, nq, k, metric, precision, ids, dists, err, on_device, st,
                         -1);
}

// An SVDB_PREC_FP8 search runs the E4M3 screen where it was measured to pay
// (1M x 768 mixture, cosine): batches of at least 1,024 queries, whose BF16
// seed pass over 1/16 of the rows settles the E4M3 screen's looser
// thresholds, and k <= 32.  At k = 48 .. 100 the seed sample held fewer than
// k rows of a query's neighbourhood, the candidate lists overflowed and the
// queries fell back to the FP64 scan; at 64 queries and fewer the BF16
// screen (or the streamed one) was faster.  Elsewhere the BF16 screen runs:
// its results are identical.
static bool fp8_screen_pays(const Store* s, size_t nq, size_t k) {
    if (s->fp8_mode >= 0) return s->fp8_mode == 1;
    return nq >= 1024 && k <= 32;
}

int svdb::search_seeded(Store* s, const double* q, size_t nq, size_t k, int metric, int precision, int64_t* ids,
                        double* dists, double* err, int on_device, svdb_search_stats* st, int seed) {
    if (k == 0 || k > 128 || metric < 0 || metric > 2 ||
        (precision != SVDB_PREC_FP64 && precision != SVDB_PREC_BF16 && precision != SVDB_PREC_FP8)) {
        svdb_set_error("search: bad argument (k=%zu metric=%d precision=%d; k must be 1..128)", k, metric, precision);
        return SVDB_EINVAL;
    }
    if (st) std::memset(st, 0, sizeof(*st));
    if (nq == 0) return SVDB_OK;
    int rc = s->sync();
    if (rc) return rc;
    const size_t out_n = nq * k;
    // scratch: [padded queries | sums of squares | outputs (host mode) | kernel scratch]
    const size_t qbytes = round_up(nq * s->ld * sizeof(double), 256);
    const size_t sqbytes = round_up(nq * sizeof(double), 256);
    const size_t obytes = on_device ? 0 : round_up(out_n * (sizeof(int64_t) + 2 * sizeof(double)), 256);
    // the screen certifies k <= 128 on stores without unscreenable rows; the
    // rest is answered by the exact scan
    const bool use_bf16 = (precision == SVDB_PREC_BF16 || precision == SVDB_PREC_FP8) && bf16_supported(s, k);
    size_t kbytes = 0;
    if (s->nlive) kbytes = use_bf16 ? search_bf16_scratch(s, nq, k) : search_fp64_scratch(s, nq, k);
    const size_t qin = on_device ? 0 : round_up(nq * s->dim * sizeof(double), 256);
    rc = s->scratch_reserve(qbytes + sqbytes + obytes + kbytes + qin);
    if (rc) return rc;
    unsigned char* base = (unsigned char*)s->scratch;
    double* qbuf = (double*)base;
    double* qsq = (double*)(base + qbytes);
    unsigned char* outp = base + qbytes + sqbytes;
    unsigned char* kscr = outp + obytes;
    const double* qsrc = q;
    s->prof_begin();
    // host buffers: page-locked ones are read and written by DMA directly,
    // pageable ones go through the store's pinned staging buffer
    const bool pin_out = !on_device && host_pinned(ids) && host_pinned(dists) && (!err || host_pinned(err));
    if (!on_device) {
        double* qraw = (double*)(kscr + kbytes);
        if (host_pinned(q)) {
            SVDB_CUDA(cudaMemcpyAsync(qraw, q, nq * s->dim * sizeof(double), cudaMemcpyHostToDevice, s->stream));
        } else {
            rc = s->pinned_reserve(
                std::max(nq * s->dim * sizeof(double), out_n * (sizeof(int64_t) + 2 * sizeof(double))));
            if (rc) return rc;
            std::memcpy(s->pin, q, nq * s->dim * sizeof(double));
            SVDB_CUDA(cudaMemcpyAsync(qraw, s->pin, nq * s->dim * sizeof(double), cudaMemcpyHostToDevice, s->stream));
        }
        qsrc = qraw;
        if (!pin_out) {
            rc = s->pinned_reserve(
                std::max(nq * s->dim * sizeof(double), out_n * (sizeof(int64_t) + 2 * sizeof(double))));
            if (rc) return rc;
        }
    }
    SearchArgs a;
    a.q = qbuf;
    a.qsq = qsq;
    a.nq = nq;
    a.k = k;
    a.metric = metric;
    a.seed = seed >= 0 ? seed : s->seed_mode;
    if (on_device) {
        a.ids = ids;
        a.dists = dists;
        a.err = err;
    } else {
        a.ids = (int64_t*)outp;
        a.dists = (double*)(outp + out_n * sizeof(int64_t));
        a.err = (double*)(outp + out_n * (sizeof(int64_t) + sizeof(double)));
    }
    uint32_t kernels = 0;
    // the tensor-core screens need no canonical |q|^2: it is summed beside them
    cudaEvent_t qsq_ready = nullptr;
    if (s->nlive && use_bf16)
        rc = prep_queries_split(s, qsrc, s->dim, nq, qbuf, qsq, &qsq_ready);
    else
        rc = prep_queries_fp64(s, qsrc, s->dim, nq, qbuf, qsq);
    if (rc) return rc;
    kernels += qsq_ready ? 2 : 1;
    a.qsq_ready = qsq_ready;
    s->prof_mark(1);
    if (s->nlive == 0) {
        k_fill_empty<<<(unsigned)((out_n + 255) / 256), 256, 0, s->stream>>>(a.ids, a.dists, a.err, out_n);
        SVDB_LAUNCH_CHECK();
        ++kernels;
    } else if (!use_bf16) {
        rc = search_fp64(s, a, kscr, kbytes, &kernels);
        if (st) {
            if (precision != SVDB_PREC_FP64) st->widened += (uint32_t)nq;
            st->candidates += (uint64_t)nq * s->nlive;
            st->survivors += (uint64_t)nq * s->nlive;
            st->reranked += (uint64_t)nq * s->nlive;
        }
    } else {
        rc = search_bf16(s, a, kscr, kbytes, st, precision == SVDB_PREC_FP8 && fp8_screen_pays(s, nq, k));
        // joined whatever happened: nothing later on the stream may outrun the side stream's writes
        if (qsq_ready && cudaStreamWaitEvent(s->stream, qsq_ready, 0) != cudaSuccess) cudaGetLastError();
    }
    s->prof_mark(SVDB_NSTAGES);
    s->prof_end();
    if (rc) return rc;
    if (st) st->kernels += kernels;
    if (!on_device && pin_out && !st) {
        SVDB_CUDA(cudaMemcpyAsync(ids, a.ids, out_n * sizeof(int64_t), cudaMemcpyDeviceToHost, s->stream));
        SVDB_CUDA(cudaMemcpyAsync(dists, a.dists, out_n * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
        if (err) SVDB_CUDA(cudaMemcpyAsync(err, a.err, out_n * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
        SVDB_CUDA(cudaStreamSynchronize(s->stream));
        rc = s->check_error();
        if (rc) return rc;
    } else if (!on_device) {
        rc = s->pinned_reserve(std::max(nq * s->dim * sizeof(double), out_n * (sizeof(int64_t) + 2 * sizeof(double))));
        if (rc) return rc;
        unsigned char* hp = (unsigned char*)s->pin;
        SVDB_CUDA(cudaMemcpyAsync(hp, outp, out_n * (sizeof(int64_t) + 2 * sizeof(double)), cudaMemcpyDeviceToHost,
                                  s->stream));
        SVDB_CUDA(cudaStreamSynchronize(s->stream));
        rc = s->check_error();
        if (rc) return rc;
        std::memcpy(ids, hp, out_n * sizeof(int64_t));
        std::memcpy(dists, hp + out_n * sizeof(int64_t), out_n * sizeof(double));
        if (err) std::memcpy(err, hp + out_n * (sizeof(int64_t) + sizeof(double)), out_n * sizeof(double));
        if (st) {
            double m = 0.0;
            for (size_t i = 0; i < out_n; ++i) {
                const double e = ((double*)(hp + out_n * (sizeof(int64_t) + sizeof(double))))[i];
                if (e > m) m = e;
            }
            st->max_err_bound = m;
        }
    }
    return SVDB_OK;
}
