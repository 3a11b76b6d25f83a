// dev_store.cu -- device-resident vector store and the reference-exact
// /compare kernel.
//
// HBM layout of one store (capacity C slots, dimension D):
//   x64     C x ld   double   FP64 master, ld = D rounded up to 16 (128-B rows)
//   xb      C x ldb  bf16     BF16 shadow of x64, ldb = D rounded up to 64
//   x32     C x ld   float    FP32 shadow of x64 (refinement stage)
//   xbn     C x ldb  bf16     BF16 shadow of x64 / |x| (cosine screen)
//   rowpn   C        float2   {|bxn| up, |x/|x| - bxn| up}
//   xbn8    C x ldb8 e4m3     FP8 shadow of 256 x / |x| (FP8 cosine screen), ldb8 = D rounded up to 128
//   rowpn8  C        float2   {|bxn8|/256 up, |x/|x| - bxn8/256| up}
//   xb8     C x ldb8 e4m3     FP8 shadow of x 2^f per row (FP8 dot / Euclidean screen): 2^f the largest
//                              power of two with max_j |x_j| 2^f <= 448 (E4M3's largest finite value)
//   rowp8   C        float4   {|bx8| up, |x - bx8| up, 2^-f, 0}, bx8 = e4m3(x 2^f) 2^-f
//   sqf     C        float4   {|x|^2 down, |x|^2 up, 1/(2|x|) down, 1/(2|x|) up} in FP32
//   sq64    C        double   canonical sum of squares of the master row
//   rowp    C        float4   {|x| up, |bf16(x)| up, |x - bf16(x)| up, |x|^2/2}
//   live    C        uint8    1 = searchable row, 2 = row of another dimension
//                              (counted in positions, never searched), 0 = deleted
//   logical C        int64    slot -> positional index (rank among live slots)
#include <cstdarg>
#include <cstdio>
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "dev_common.cuh"
#include "dev_ref.cuh"
#include "dev_store.cuh"

#include <cuda_fp8.h>

namespace {
thread_local char g_err[512];
}

extern "C" void svdb_set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

extern "C" SVDB_API const char* svdb_last_error(void) { return g_err; }

namespace svdb {

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

// Derived per-row arrays for slots [lo, hi) or for an explicit slot list.
// One group of 4 lanes per row, canonical order for the sum of squares.
__global__ void k_derive_rows(const double* __restrict__ x64, size_t ld, __nv_bfloat16* __restrict__ xb,
                              size_t ldb, float* __restrict__ x32, __nv_bfloat16* __restrict__ xbn,
                              float2* __restrict__ rowpn, float4* __restrict__ sqf, double* __restrict__ sq64,
                              float4* __restrict__ rowp, uint8_t* __restrict__ xbn8, size_t ldb8,
                              float2* __restrict__ rowpn8, uint8_t* __restrict__ xb8, float4* __restrict__ rowp8,
                              const uint8_t* __restrict__ live, int64_t lo, int64_t hi,
                              const int64_t* __restrict__ list) {
    const int lane = threadIdx.x & 31, s = lane & 3;
    const int64_t gid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 2;
    const int64_t nrow = list ? hi : hi - lo;
    const bool active = gid < nrow;
    const int64_t slot = active ? (list ? list[gid] : lo + gid) : 0;
    const double* x = x64 + slot * ld;
    float* xf = x32 + slot * ld;
    double sq = 0.0, bh = 0.0, res = 0.0, mx = 0.0;
    if (active) {
        for (size_t j = 2 * s; j < ld; j += 8) {
            const double2 v = *reinterpret_cast<const double2*>(x + j);
            mx = fmax(mx, fmax(fabs(v.x), fabs(v.y)));
            sq = fma(v.x, v.x, sq);
            sq = fma(v.y, v.y, sq);
            const __nv_bfloat16 hx = __double2bfloat16(v.x), hy = __double2bfloat16(v.y);
            const double fx = (double)__bfloat162float(hx), fy = (double)__bfloat162float(hy);
            bh = fma(fx, fx, bh);
            bh = fma(fy, fy, bh);
            res = fma(v.x - fx, v.x - fx, res);
            res = fma(v.y - fy, v.y - fy, res);
            *reinterpret_cast<__nv_bfloat162*>(xb + bf16_tile_index(slot, j, ldb)) = __halves2bfloat162(hx, hy);
            *reinterpret_cast<float2*>(xf + j) = make_float2(__double2float_rn(v.x), __double2float_rn(v.y));
        }
        for (size_t j = ld + 2 * s; j < ldb; j += 8)  // zero the BF16 tail beyond ld
            *reinterpret_cast<__nv_bfloat162*>(xb + bf16_tile_index(slot, j, ldb)) = __floats2bfloat162_rn(0.f, 0.f);
    }
    sq = group4_sum(sq);
    bh = group4_sum(bh);
    res = group4_sum(res);
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, 2));
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, 1));
    // the row's E4M3 scale: the largest power of two 2^f with mx 2^f <= 448,
    // kept within 2^+-120 so 2^-f is a normal FP32 number (a row outside that
    // range only loses E4M3 precision, which its residual term accounts for)
    int f = 0;
    if (mx > 0.0 && isfinite(mx)) {
        f = max(-120, min(120, e4m3_fit_exp(mx)));
    }
    const double sc8 = ldexp(1.0, f);
    // second pass: the unit-norm row for the cosine screen, its BF16 and FP8
    // (E4M3 of 256 x/|x|) copies and their residuals, and the E4M3 copy of
    // x 2^f for the dot / Euclidean screen and its residual
    double nbh = 0.0, nres = 0.0, nbh8 = 0.0, nres8 = 0.0, pb8 = 0.0, pres8 = 0.0;
    if (active) {
        const double ixn = sq > 0.0 ? 1.0 / sqrt(sq) : 0.0;
        for (size_t j = 2 * s; j < ld; j += 8) {
            const double2 v = *reinterpret_cast<const double2*>(x + j);
            {
                const __nv_fp8_storage_t px = __nv_cvt_double_to_fp8(v.x * sc8, __NV_SATFINITE, __NV_E4M3);
                const __nv_fp8_storage_t py = __nv_cvt_double_to_fp8(v.y * sc8, __NV_SATFINITE, __NV_E4M3);
                const double gx = (double)__half2float(__half(__nv_cvt_fp8_to_halfraw(px, __NV_E4M3))) / sc8;
                const double gy = (double)__half2float(__half(__nv_cvt_fp8_to_halfraw(py, __NV_E4M3))) / sc8;
                pb8 = fma(gx, gx, pb8);
                pb8 = fma(gy, gy, pb8);
                pres8 = fma(v.x - gx, v.x - gx, pres8);
                pres8 = fma(v.y - gy, v.y - gy, pres8);
                *reinterpret_cast<uint16_t*>(xb8 + f8_tile_index(slot, j, ldb8)) = (uint16_t)(px | ((uint16_t)py << 8));
            }
            const double ux = v.x * ixn, uy = v.y * ixn;
            const __nv_bfloat16 hx = __double2bfloat16(ux), hy = __double2bfloat16(uy);
            const double fx = (double)__bfloat162float(hx), fy = (double)__bfloat162float(hy);
            nbh = fma(fx, fx, nbh);
            nbh = fma(fy, fy, nbh);
            nres = fma(ux - fx, ux - fx, nres);
            nres = fma(uy - fy, uy - fy, nres);
            *reinterpret_cast<__nv_bfloat162*>(xbn + bf16_tile_index(slot, j, ldb)) = __halves2bfloat162(hx, hy);
            const __nv_fp8_storage_t ex = __nv_cvt_double_to_fp8(kF8RowScale * ux, __NV_SATFINITE, __NV_E4M3);
            const __nv_fp8_storage_t ey = __nv_cvt_double_to_fp8(kF8RowScale * uy, __NV_SATFINITE, __NV_E4M3);
            const double gx = (double)__half2float(__half(__nv_cvt_fp8_to_halfraw(ex, __NV_E4M3))) / kF8RowScale;
            const double gy = (double)__half2float(__half(__nv_cvt_fp8_to_halfraw(ey, __NV_E4M3))) / kF8RowScale;
            nbh8 = fma(gx, gx, nbh8);
            nbh8 = fma(gy, gy, nbh8);
            nres8 = fma(ux - gx, ux - gx, nres8);
            nres8 = fma(uy - gy, uy - gy, nres8);
            *reinterpret_cast<uint16_t*>(xbn8 + f8_tile_index(slot, j, ldb8)) = (uint16_t)(ex | ((uint16_t)ey << 8));
        }
        for (size_t j = ld + 2 * s; j < ldb; j += 8)
            *reinterpret_cast<__nv_bfloat162*>(xbn + bf16_tile_index(slot, j, ldb)) = __floats2bfloat162_rn(0.f, 0.f);
        for (size_t j = ld + 2 * s; j < ldb8; j += 8) {
            *reinterpret_cast<uint16_t*>(xbn8 + f8_tile_index(slot, j, ldb8)) = 0;
            *reinterpret_cast<uint16_t*>(xb8 + f8_tile_index(slot, j, ldb8)) = 0;
        }
    }
    nbh = group4_sum(nbh);
    nres = group4_sum(nres);
    nbh8 = group4_sum(nbh8);
    nres8 = group4_sum(nres8);
    pb8 = group4_sum(pb8);
    pres8 = group4_sum(pres8);
    if (active && s == 0) {
        // x/|x| is itself rounded (relative 2^-52 per element): the 2^-30 margin covers it
        const double up = 1.0 + 9.313225746154785e-10;
        {
            // |x| to within 2^-50 relative either way (FP64 sum and square root)
            const double xn = sqrt(sq);
            const double lo = xn * (1.0 - 8.881784197001252e-16), hi = xn * (1.0 + 8.881784197001252e-16);
            sqf[slot] = make_float4(__double2float_rd(sq), __double2float_ru(sq), __double2float_rd(0.5 / hi),
                                    lo > 0.0 ? __double2float_ru(0.5 / lo) : __int_as_float(0x7f800000));
        }
        rowpn[slot] = make_float2(__double2float_ru(sqrt(nbh) * up), __double2float_ru(sqrt(nres) * up + 1e-300));
        rowpn8[slot] = make_float2(__double2float_ru(sqrt(nbh8) * up), __double2float_ru(sqrt(nres8) * up + 1e-300));
        rowp8[slot] = make_float4(__double2float_ru(sqrt(pb8) * up), __double2float_ru(sqrt(pres8) * up + 1e-300),
                                  (float)(1.0 / sc8), 0.0f);
        sq64[slot] = sq;
        float4 p;
        p.x = __double2float_ru(sqrt(sq));
        p.y = __double2float_ru(sqrt(bh));
        p.z = __double2float_ru(sqrt(res));
        p.w = __double2float_rn(0.5 * sq);
        // rows the screens cannot bound (overflow, non-finite, a nonzero row
        // whose BF16 copy or E4M3 copy of x 2^f is all zero -- the screens'
        // one-FMA bound needs |x - bx| <= alpha |bx|): mark them with an
        // infinite error term (the store then answers searches by the exact
        // scan); dead slots: |x| = -1
        if (!(sq < 1e30) || !isfinite(p.y) || (bh == 0.0 && res > 0.0) || (pb8 == 0.0 && pres8 > 0.0))
            p.z = __int_as_float(0x7f800000);
        if (live[slot] != 1) p.x = -1.0f;
        rowp[slot] = p;
    }
}

// Single-block exclusive scan of live flags -> slot->logical map, done in
// chunks of 1024*4 slots carrying the running count.
// slot -> logical rank (positional index) of every slot, -1 for deleted ones;
// nlive_out = number of occupied positions.  Three passes so the map scales
// with the store: per-chunk counts (one 1024-thread block per kMapChunk
// slots), an exclusive scan of the chunk counts, and a per-chunk block scan
// that writes the ranks.
constexpr int kMapChunk = 4096;

__global__ void __launch_bounds__(1024) k_map_count(const uint8_t* __restrict__ live, int64_t n,
                                                    int64_t* __restrict__ blk) {
    __shared__ int ws[32];
    const int64_t base = (int64_t)blockIdx.x * kMapChunk;
    int c = 0;
    for (int u = threadIdx.x; u < kMapChunk; u += 1024) c += (base + u < n && live[base + u] != 0) ? 1 : 0;
    c = __reduce_add_sync(0xffffffffu, c);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x < 32) {
        const int v = __reduce_add_sync(0xffffffffu, ws[threadIdx.x]);
        if (threadIdx.x == 0) blk[blockIdx.x] = v;
    }
}

// exclusive scan of nb chunk counts in place (one block), total to *nlive_out
__global__ void __launch_bounds__(1024) k_map_scan(int64_t* __restrict__ blk, int64_t nb,
                                                   int64_t* __restrict__ nlive_out) {
    __shared__ int64_t wt[32];
    __shared__ int64_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int64_t b0 = 0; b0 < nb; b0 += 1024) {
        const int64_t i = b0 + threadIdx.x;
        const int64_t v = i < nb ? blk[i] : 0;
        int64_t incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) wt[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            const int64_t w = wt[lane];
            int64_t wi = w;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int64_t t = __shfl_up_sync(0xffffffffu, wi, o);
                if (lane >= o) wi += t;
            }
            wt[lane] = wi - w;
        }
        __syncthreads();
        const int64_t c0 = carry;
        if (i < nb) blk[i] = c0 + wt[warp] + incl - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry = c0 + wt[warp] + incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) *nlive_out = carry;
}

__global__ void __launch_bounds__(1024) k_map_write(const uint8_t* __restrict__ live, int64_t n,
                                                    const int64_t* __restrict__ blk, int64_t* __restrict__ logical) {
    __shared__ int64_t wt[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t i0 = (int64_t)blockIdx.x * kMapChunk + threadIdx.x * 4;
    int c[4], tot = 0;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        c[u] = (i0 + u < n && live[i0 + u] != 0) ? 1 : 0;
        tot += c[u];
    }
    int incl = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) wt[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const int64_t w = wt[lane];
        int64_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += t;
        }
        wt[lane] = wi - w;
    }
    __syncthreads();
    int64_t run = blk[blockIdx.x] + wt[warp] + (incl - tot);
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        if (i0 + u < n) logical[i0 + u] = c[u] ? run : -1;
        run += c[u];
    }
}

// live rows whose BF16 screen terms are unbounded (marked +inf by k_derive_rows)
// ... and the store-wide maxima of the unit-norm shadow's residual and norm
// (count[1], count[2], float bits; non-negative floats order as ints)
__global__ void k_count_unscreenable(const float4* __restrict__ rowp, const float2* __restrict__ rowpn,
                                     const float2* __restrict__ rowpn8, const uint8_t* __restrict__ live, int64_t n,
                                     int* __restrict__ count) {
    int c = 0, ra = 0, rb = 0, ra8 = 0, rb8 = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (live[i] != 1) continue;
        c += !(rowp[i].z < 3.0e38f) ? 1 : 0;
        const float2 pn = rowpn[i], pn8 = rowpn8[i];
        ra = max(ra, __float_as_int(pn.y));
        rb = max(rb, __float_as_int(pn.x));
        ra8 = max(ra8, __float_as_int(pn8.y));
        rb8 = max(rb8, __float_as_int(pn8.x));
    }
    c = __reduce_add_sync(0xffffffffu, c);
    ra = __reduce_max_sync(0xffffffffu, ra);
    rb = __reduce_max_sync(0xffffffffu, rb);
    ra8 = __reduce_max_sync(0xffffffffu, ra8);
    rb8 = __reduce_max_sync(0xffffffffu, rb8);
    if ((threadIdx.x & 31) == 0) {
        if (c) atomicAdd(count, c);
        atomicMax(count + 1, ra);
        atomicMax(count + 2, rb);
        atomicMax(count + 3, ra8);
        atomicMax(count + 4, rb8);
    }
}

__global__ void k_set_live(uint8_t* live, const int64_t* slots, int n, uint8_t v) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) live[slots[i]] = v;
}

// metrics: per pair (the drop-in calls combined into one launch), or NULL for `metric`
__global__ void k_compare_slots(const double* __restrict__ x64, size_t ld, int d, int metric,
                                const int* __restrict__ metrics, const int64_t* __restrict__ s1,
                                const int64_t* __restrict__ s2, int n, float* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = ref_metric(metrics ? metrics[i] : metric, x64 + s1[i] * ld, x64 + s2[i] * ld, d);
}

// pairs of free-standing vectors packed into one buffer: pair i is
// {a offset, b offset, dimension, metric} (in doubles)
__global__ void k_compare_vecs(const double* __restrict__ buf, const int64_t* __restrict__ desc, int n,
                               float* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t* p = desc + 4 * (size_t)i;
    out[i] = ref_metric((int)p[3], buf + p[0], buf + p[1], (int)p[2]);
}

// ---------------------------------------------------------------------------
// stage timing
// ---------------------------------------------------------------------------
int Store::prof_enable(bool on) {
    int rc = ensure();
    if (rc) return rc;
    if (on && !prof_events) {
        for (int i = 0; i < kProfRing; ++i)
            for (int j = 0; j < kProfMarks; ++j) SVDB_CUDA(cudaEventCreate(&pev[i][j]));
        prof_events = true;
    }
    prof = on;
    return SVDB_OK;
}

void Store::prof_begin() {
    prof_cur = -1;
    if (!prof) return;
    if (prof_pending == kProfRing && prof_resolve_one() != SVDB_OK) return;
    prof_cur = (prof_head + prof_pending) % kProfRing;
    ++prof_pending;
    prof_mark(0);
}

// records `boundary` and every later one, so a stage a search skips reads 0
void Store::prof_mark(int boundary) {
    if (prof_cur < 0) return;
    for (int j = boundary; j < kProfMarks; ++j) cudaEventRecord(pev[prof_cur][j], stream);
}

int Store::prof_resolve_one() {
    if (!prof_pending) return SVDB_OK;
    cudaEvent_t* e = pev[prof_head];
    SVDB_CUDA(cudaEventSynchronize(e[kProfMarks - 1]));
    for (int j = 0; j < SVDB_NSTAGES; ++j) {
        float ms = 0.0f;
        SVDB_CUDA(cudaEventElapsedTime(&ms, e[j], e[j + 1]));
        prof_ms[j] += ms;
    }
    ++prof_calls;
    prof_head = (prof_head + 1) % kProfRing;
    --prof_pending;
    return SVDB_OK;
}

int Store::prof_read(double* ms, bool reset) {
    while (prof_pending) {
        int rc = prof_resolve_one();
        if (rc) return rc;
    }
    if (ms)
        for (int j = 0; j < SVDB_NSTAGES; ++j) ms[j] = prof_ms[j];
    const int64_t n = prof_calls;
    if (reset) {
        for (int j = 0; j < SVDB_NSTAGES; ++j) prof_ms[j] = 0.0;
        prof_calls = 0;
    }
    return (int)std::min<int64_t>(n, 0x7fffffff);
}

// ---------------------------------------------------------------------------
// store
// ---------------------------------------------------------------------------

int Store::ensure() {
    if (stream) return SVDB_OK;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        svdb_set_error("no usable CUDA device: %s", e != cudaSuccess ? cudaGetErrorString(e) : "none found");
        return SVDB_ENODEV;
    }
    cudaStream_t st = nullptr;
    SVDB_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    if (cudaMalloc(&d_nlive, sizeof(int64_t)) != cudaSuccess || cudaMalloc(&d_count, 8 * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&d_err, sizeof(int)) != cudaSuccess || cudaMemset(d_err, 0, sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        cudaStreamDestroy(st);
        svdb_set_error("device store: cannot allocate a counter");
        return SVDB_ENOMEM;
    }
    stream = st;
    // the no-allocation search's array: loaded now, with the store's own
    // allocations, so that search never loads it (a failure here is reported
    // by that search itself, which tries again)
    if (noalloc_setup(nullptr) != SVDB_OK) cudaGetLastError();
    return SVDB_OK;
}

int Store::grow(size_t need) {
    int erc = ensure();
    if (erc) return erc;
    if (need <= cap) return SVDB_OK;
    // the largest row count whose FP64 rows fit in the address space, halved
    // so the doubling below cannot wrap
    if (need > (SIZE_MAX / (ld * sizeof(double) + 64)) / 2) {
        svdb_set_error("device store: %zu rows of dim %zu exceed any device's memory", need, dim);
        return SVDB_ENOMEM;
    }
    size_t nc = cap ? cap : 1024;
    while (nc < need) nc *= 2;
    double* nx = nullptr;
    __nv_bfloat16* nb = nullptr;
    float* nf = nullptr;
    __nv_bfloat16* nbn = nullptr;
    float2* npn = nullptr;
    uint8_t* nb8 = nullptr;
    float2* npn8 = nullptr;
    uint8_t* nx8 = nullptr;
    float4* np8 = nullptr;
    float4* nsf = nullptr;
    double* nsq = nullptr;
    float4* np = nullptr;
    uint8_t* nl = nullptr;
    int64_t* nlog = nullptr;
    int64_t* nblk = nullptr;
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = cudaMalloc(&nx, nc * ld * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&nb, nc * ldb * sizeof(__nv_bfloat16));
    if (e == cudaSuccess) e = cudaMalloc(&nf, nc * ld * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&nbn, nc * ldb * sizeof(__nv_bfloat16));
    if (e == cudaSuccess) e = cudaMalloc(&npn, nc * sizeof(float2));
    if (e == cudaSuccess) e = cudaMalloc(&nb8, nc * ldb8);
    if (e == cudaSuccess) e = cudaMalloc(&npn8, nc * sizeof(float2));
    if (e == cudaSuccess) e = cudaMalloc(&nx8, nc * ldb8);
    if (e == cudaSuccess) e = cudaMalloc(&np8, nc * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc(&nsf, nc * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc(&nsq, nc * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&np, nc * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc(&nl, nc);
    if (e == cudaSuccess) e = cudaMalloc(&nlog, nc * sizeof(int64_t));
    if (e == cudaSuccess) e = cudaMalloc(&nblk, ((nc + kMapChunk - 1) / kMapChunk) * sizeof(int64_t));
    if (e != cudaSuccess) {
        cudaGetLastError();
        cudaFree(nx);
        cudaFree(nb);
        cudaFree(nf);
        cudaFree(nbn);
        cudaFree(npn);
        cudaFree(nb8);
        cudaFree(npn8);
        cudaFree(nx8);
        cudaFree(np8);
        cudaFree(nsf);
        cudaFree(nsq);
        cudaFree(np);
        cudaFree(nl);
        cudaFree(nlog);
        cudaFree(nblk);
        svdb_set_error("device store: cannot grow to %zu rows of dim %zu: %s", nc, dim, cudaGetErrorString(e));
        return SVDB_ENOMEM;
    }
    // BF16 shadows: whole 256-row tiles; rows never written stay zero
    SVDB_CUDA(cudaMemsetAsync(nb, 0, nc * ldb * sizeof(__nv_bfloat16), stream));
    SVDB_CUDA(cudaMemsetAsync(nbn, 0, nc * ldb * sizeof(__nv_bfloat16), stream));
    SVDB_CUDA(cudaMemsetAsync(nb8, 0, nc * ldb8, stream));
    SVDB_CUDA(cudaMemsetAsync(nx8, 0, nc * ldb8, stream));
    if (slots) {
        const size_t tile_rows = round_up(slots, 256);
        SVDB_CUDA(cudaMemcpyAsync(nx, x64, slots * ld * sizeof(double), cudaMemcpyDeviceToDevice, stream));
        SVDB_CUDA(cudaMemcpyAsync(nb, xb, tile_rows * ldb * sizeof(__nv_bfloat16), cudaMemcpyDeviceToDevice, stream));
        SVDB_CUDA(cudaMemcpyAsync(nf, x32, slots * ld * sizeof(float), cudaMemcpyDeviceToDevice, stream));
        SVDB_CUDA(cudaMemcpyAsync(nbn, xbn, tile_rows * ldb * sizeof(__nv_bfloat16), cudaMemcpyDeviceToDevice, stream));
        SVDB_CUDA(cudaMemcpyAsync(npn, rowpn, slots * sizeof(float2), cudaMemcpyDeviceToDevice, stream));
        SVDB_CUDA(cudaMemcpyAsync(nb8, xbn8, tile_rows * ldb8, cudaMemcpyDeviceToDevice, stream));
        SVDB_CUDA(cudaMemcpyAsync(npn8, rowpn8, slots * sizeof(float2), cudaMemcpyDeviceToDevice, stream));
        SVDB_CUDA(cudaMemcpyAsync(nx8, xb8, tile_rows * ldb8, cudaMemcpyDeviceToDevice, stream));
        SVDB_CUDA(cudaMemcpyAsync(np8, rowp8, slots * sizeof(float4), cudaMemcpyDeviceToDevice, stream));
        SVDB_CUDA(cudaMemcpyAsync(nsf, sqf, slots * sizeof(float4), cudaMemcpyDeviceToDevice, stream));
        SVDB_CUDA(cudaMemcpyAsync(nsq, sq64, slots * sizeof(double), cudaMemcpyDeviceToDevice, stream));
        SVDB_CUDA(cudaMemcpyAsync(np, rowp, slots * sizeof(float4), cudaMemcpyDeviceToDevice, stream));
        SVDB_CUDA(cudaMemcpyAsync(nl, live, slots, cudaMemcpyDeviceToDevice, stream));
        SVDB_CUDA(cudaMemcpyAsync(nlog, logical, slots * sizeof(int64_t), cudaMemcpyDeviceToDevice, stream));
        SVDB_CUDA(cudaStreamSynchronize(stream));
    }
    cudaFree(x64);
    cudaFree(xb);
    cudaFree(x32);
    cudaFree(xbn);
    cudaFree(rowpn);
    cudaFree(xbn8);
    cudaFree(rowpn8);
    cudaFree(xb8);
    cudaFree(rowp8);
    cudaFree(sqf);
    cudaFree(sq64);
    cudaFree(rowp);
    cudaFree(live);
    cudaFree(logical);
    cudaFree(mapblk);
    x64 = nx;
    xb = nb;
    x32 = nf;
    xbn = nbn;
    rowpn = npn;
    xbn8 = nb8;
    rowpn8 = npn8;
    xb8 = nx8;
    rowp8 = np8;
    sqf = nsf;
    sq64 = nsq;
    rowp = np;
    live = nl;
    logical = nlog;
    mapblk = nblk;
    cap = nc;
    ++epoch;
    return SVDB_OK;
}

int Store::scratch_reserve(size_t bytes) {
    int erc = ensure();
    if (erc) return erc;
    if (bytes <= scratch_bytes) return SVDB_OK;
    SVDB_CUDA(cudaStreamSynchronize(stream));
    if (side) SVDB_CUDA(cudaStreamSynchronize(side));  // (a search's |q|^2 may be written there)
    cudaFree(scratch);
    scratch = nullptr;
    scratch_bytes = 0;
    size_t nb = round_up(bytes + bytes / 4, 1 << 20);
    cudaError_t e = cudaMalloc(&scratch, nb);
    if (e != cudaSuccess) {
        cudaGetLastError();
        svdb_set_error("device scratch: cannot allocate %zu bytes: %s", nb, cudaGetErrorString(e));
        return SVDB_ENOMEM;
    }
    scratch_bytes = nb;
    ++epoch;
    return SVDB_OK;
}

// After the stream is idle: a device kernel's bounded wait that ran out shows
// here as SVDB_ETIMEOUT (once; the word is cleared).
int Store::side_ready() {
    if (side) return SVDB_OK;
    cudaStream_t st = nullptr;
    cudaEvent_t a = nullptr, b = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&a, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        if (st) cudaStreamDestroy(st);
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
        return SVDB_ECUDA;
    }
    side = st;
    ev_fork = a;
    ev_side = b;
    return SVDB_OK;
}

int Store::check_error() {
    if (!d_err) return SVDB_OK;
    int h = 0;
    SVDB_CUDA(cudaMemcpy(&h, d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (!h) return SVDB_OK;
    SVDB_CUDA(cudaMemset(d_err, 0, sizeof(int)));
    svdb_set_error("a search kernel's bounded wait ran out (its results are not valid)");
    return SVDB_ETIMEOUT;
}

int Store::scratch2_reserve(size_t bytes) {
    if (bytes <= scratch2_bytes) return SVDB_OK;
    SVDB_CUDA(cudaStreamSynchronize(stream));
    cudaFree(scratch2);
    scratch2 = nullptr;
    scratch2_bytes = 0;
    size_t nb = round_up(bytes + bytes / 4, 1 << 20);
    cudaError_t e = cudaMalloc(&scratch2, nb);
    if (e != cudaSuccess) {
        cudaGetLastError();
        svdb_set_error("device scratch: cannot allocate %zu bytes: %s", nb, cudaGetErrorString(e));
        return SVDB_ENOMEM;
    }
    scratch2_bytes = nb;
    ++epoch;
    return SVDB_OK;
}

int Store::pinned_reserve(size_t bytes) {
    int erc = ensure();
    if (erc) return erc;
    if (bytes <= pin_bytes) return SVDB_OK;
    SVDB_CUDA(cudaStreamSynchronize(stream));
    cudaFreeHost(pin);
    pin = nullptr;
    pin_bytes = 0;
    size_t nb = round_up(bytes + bytes / 4, 1 << 16);
    SVDB_CUDA(cudaMallocHost(&pin, nb));
    pin_bytes = nb;
    return SVDB_OK;
}

// Move staged appends to the device: one pitched copy of the staging block.
int Store::flush() {
    if (stage_rows == 0) return SVDB_OK;
    const size_t first = slots, n = stage_rows;
    int rc = grow(first + n);
    if (rc) return rc;
    SVDB_CUDA(cudaStreamSynchronize(stream));  // the pinned stage buffer is reused below
    rc = pinned_reserve(n * dim * sizeof(double));
    if (rc) return rc;
    std::memcpy(pin, stage.data(), n * dim * sizeof(double));
    SVDB_CUDA(cudaMemsetAsync(x64 + first * ld, 0, n * ld * sizeof(double), stream));
    SVDB_CUDA(cudaMemcpy2DAsync(x64 + first * ld, ld * sizeof(double), pin, dim * sizeof(double),
                                dim * sizeof(double), n, cudaMemcpyHostToDevice, stream));
    SVDB_CUDA(cudaMemcpyAsync(live + first, stage_live.data(), n, cudaMemcpyHostToDevice, stream));
    SVDB_CUDA(cudaStreamSynchronize(stream));  // stage_live is pageable and cleared below
    slots += n;
    ++epoch;
    ++version;
    stage.clear();
    stage_live.clear();
    stage_rows = 0;
    if (derive_lo < 0 || (int64_t)first < derive_lo) derive_lo = (int64_t)first;
    derive_hi = (int64_t)slots;
    map_dirty = true;
    return SVDB_OK;
}

int Store::sync() {
    int rc = ensure();
    if (rc) return rc;
    rc = flush();
    if (rc) return rc;
    rc = uuid_flush();
    if (rc) return rc;
    if (derive_lo >= 0 && derive_hi > derive_lo) {
        const int64_t n = derive_hi - derive_lo;
        const int threads = 256;
        const int64_t blocks = (n * 4 + threads - 1) / threads;
        k_derive_rows<<<(unsigned)blocks, threads, 0, stream>>>(x64, ld, xb, ldb, x32, xbn, rowpn, sqf, sq64, rowp, xbn8,
                                                              ldb8, rowpn8, xb8, rowp8, live, derive_lo,
                                                              derive_hi, nullptr);
        SVDB_LAUNCH_CHECK();
    }
    derive_lo = derive_hi = -1;
    if (!dirty_list.empty()) {
        const int64_t n = (int64_t)dirty_list.size();
        int64_t* d = nullptr;
        rc = scratch_reserve(n * sizeof(int64_t));
        if (rc) return rc;
        d = (int64_t*)scratch;
        SVDB_CUDA(cudaMemcpyAsync(d, dirty_list.data(), n * sizeof(int64_t), cudaMemcpyHostToDevice, stream));
        k_derive_rows<<<(unsigned)((n * 4 + 255) / 256), 256, 0, stream>>>(x64, ld, xb, ldb, x32, xbn, rowpn, sqf, sq64, rowp,
                                                                         xbn8, ldb8, rowpn8, xb8, rowp8, live, 0,
                                                                         n, d);
        SVDB_LAUNCH_CHECK();
        SVDB_CUDA(cudaStreamSynchronize(stream));
        dirty_list.clear();
    }
    if (map_dirty && slots) {
        const int64_t nb = ((int64_t)slots + kMapChunk - 1) / kMapChunk;
        k_map_count<<<(unsigned)nb, 1024, 0, stream>>>(live, (int64_t)slots, mapblk);
        SVDB_LAUNCH_CHECK();
        k_map_scan<<<1, 1024, 0, stream>>>(mapblk, nb, d_nlive);
        SVDB_LAUNCH_CHECK();
        k_map_write<<<(unsigned)nb, 1024, 0, stream>>>(live, (int64_t)slots, mapblk, logical);
        SVDB_LAUNCH_CHECK();
        SVDB_CUDA(cudaMemsetAsync(d_count, 0, 5 * sizeof(int), stream));
        k_count_unscreenable<<<(unsigned)std::min<size_t>((slots + 255) / 256, 1024), 256, 0, stream>>>(
            rowp, rowpn, rowpn8, live, (int64_t)slots, d_count);
        SVDB_LAUNCH_CHECK();
        int hc = 0;
        SVDB_CUDA(cudaMemcpyAsync(&h_nlive, d_nlive, sizeof(int64_t), cudaMemcpyDeviceToHost, stream));
        SVDB_CUDA(cudaMemcpyAsync(&hc, d_count, sizeof(int), cudaMemcpyDeviceToHost, stream));
        SVDB_CUDA(cudaStreamSynchronize(stream));
        nlive = (size_t)h_nlive;
        n_unscreen = hc;
        map_dirty = false;
        ++epoch;
    } else if (!slots) {
        nlive = 0;
        map_dirty = false;
    }
    return SVDB_OK;
}

}  // namespace svdb

using svdb::Store;

extern "C" {

svdbd_store* svdbd_store_create(size_t dim) {
    if (dim == 0) {
        svdb_set_error("device store: dimension 0");
        return nullptr;
    }
    Store* s = new (std::nothrow) Store();
    if (!s) return nullptr;
    s->dim = dim;
    s->ld = svdb::round_up(dim, svdb::kRowAlign);
    s->ldb = svdb::round_up(dim, svdb::kBf16Align);
    s->ldb8 = svdb::round_up(dim, 128);
    return reinterpret_cast<svdbd_store*>(s);
}

void svdbd_store_destroy(svdbd_store* hs) {
    Store* s = reinterpret_cast<Store*>(hs);
    if (!s) return;
    if (!s->stream) {  // never touched the GPU
        s->uuid_free();
        s->kdm_free();
        delete s;
        return;
    }
    cudaStreamSynchronize(s->stream);
    if (s->side) cudaStreamSynchronize(s->side);
    cudaFree(s->x64);
    cudaFree(s->xb);
    cudaFree(s->x32);
    cudaFree(s->xbn);
    cudaFree(s->rowpn);
    cudaFree(s->xbn8);
    cudaFree(s->rowpn8);
    cudaFree(s->xb8);
    cudaFree(s->rowp8);
    cudaFree(s->sqf);
    cudaFree(s->sq64);
    cudaFree(s->rowp);
    cudaFree(s->live);
    cudaFree(s->logical);
    cudaFree(s->mapblk);
    cudaFree(s->scratch);
    cudaFree(s->d_nlive);
    cudaFree(s->d_count);
    cudaFree(s->d_err);
    cudaFree(s->scratch2);
    cudaFreeHost(s->pin);
    if (s->prof_events)
        for (int i = 0; i < Store::kProfRing; ++i)
            for (int j = 0; j < Store::kProfMarks; ++j) cudaEventDestroy(s->pev[i][j]);
    s->release_extra();
    s->uuid_free();
    s->kdm_free();
    if (s->side) cudaStreamDestroy(s->side);
    if (s->ev_fork) cudaEventDestroy(s->ev_fork);
    if (s->ev_side) cudaEventDestroy(s->ev_side);
    cudaStreamDestroy(s->stream);
    delete s;
}

void* svdbd_store_stream(svdbd_store* hs) {
    Store* s = reinterpret_cast<Store*>(hs);
    return s->ensure() == SVDB_OK ? (void*)s->stream : nullptr;
}
size_t svdbd_store_dim(const svdbd_store* hs) { return reinterpret_cast<const Store*>(hs)->dim; }
size_t svdbd_store_slots(const svdbd_store* hs) {
    const Store* s = reinterpret_cast<const Store*>(hs);
    return s->slots + s->stage_rows;
}

int svdbd_store_reserve(svdbd_store* hs, size_t rows) {
    Store* s = reinterpret_cast<Store*>(hs);
    int rc = s->flush();
    return rc ? rc : s->grow(rows);
}

int svdbd_store_append(svdbd_store* hs, const double* const* rows, const uint8_t* live, size_t n) {
    Store* s = reinterpret_cast<Store*>(hs);
    const size_t d = s->dim;
    try {
        s->stage.resize((s->stage_rows + n) * d);
        s->stage_live.resize(s->stage_rows + n);
    } catch (...) {
        svdb_set_error("device store: host staging allocation failed");
        return SVDB_ENOMEM;
    }
    for (size_t i = 0; i < n; ++i) {
        double* dst = s->stage.data() + (s->stage_rows + i) * d;
        const uint8_t flag = (rows[i] && (!live || live[i] == 1)) ? 1 : 2;
        if (flag == 1)
            std::memcpy(dst, rows[i], d * sizeof(double));
        else
            std::memset(dst, 0, d * sizeof(double));
        s->stage_live[s->stage_rows + i] = flag;
    }
    s->stage_rows += n;
    if (s->stage_rows >= 65536) return s->flush();
    return SVDB_OK;
}

int svdbd_store_append_block(svdbd_store* hs, const double* rows, size_t n) {
    Store* s = reinterpret_cast<Store*>(hs);
    int rc = s->flush();
    if (rc) return rc;
    const size_t first = s->slots;
    rc = s->grow(first + n);
    if (rc) return rc;
    const size_t d = s->dim, chunk = 1 << 16;
    rc = s->pinned_reserve(std::min(n, chunk) * d * sizeof(double));
    if (rc) return rc;
    SVDB_CUDA(cudaMemsetAsync(s->x64 + first * s->ld, 0, n * s->ld * sizeof(double), s->stream));
    SVDB_CUDA(cudaMemsetAsync(s->live + first, 1, n, s->stream));
    for (size_t off = 0; off < n; off += chunk) {
        const size_t m = std::min(chunk, n - off);
        SVDB_CUDA(cudaStreamSynchronize(s->stream));
        std::memcpy(s->pin, rows + off * d, m * d * sizeof(double));
        SVDB_CUDA(cudaMemcpy2DAsync(s->x64 + (first + off) * s->ld, s->ld * sizeof(double), s->pin,
                                    d * sizeof(double), d * sizeof(double), m, cudaMemcpyHostToDevice, s->stream));
    }
    SVDB_CUDA(cudaStreamSynchronize(s->stream));
    s->slots += n;
    ++s->epoch;
    ++s->version;
    if (s->derive_lo < 0 || (int64_t)first < s->derive_lo) s->derive_lo = (int64_t)first;
    s->derive_hi = (int64_t)s->slots;
    s->map_dirty = true;
    return SVDB_OK;
}

int svdbd_store_overwrite(svdbd_store* hs, int64_t slot, const double* row, int live) {
    Store* s = reinterpret_cast<Store*>(hs);
    if (slot >= 0 && (size_t)slot >= s->slots && (size_t)slot < s->slots + s->stage_rows) {  // still staged
        const size_t st = (size_t)slot - s->slots;
        const bool ok = row && live == 1;
        if (ok)
            std::memcpy(s->stage.data() + st * s->dim, row, s->dim * sizeof(double));
        else
            std::memset(s->stage.data() + st * s->dim, 0, s->dim * sizeof(double));
        s->stage_live[st] = ok ? 1 : 2;
        ++s->version;
        return SVDB_OK;
    }
    int rc = s->flush();
    if (rc) return rc;
    if (slot < 0 || (size_t)slot >= s->slots) {
        svdb_set_error("overwrite: slot %lld out of range", (long long)slot);
        return SVDB_EINVAL;
    }
    const uint8_t lv = (row && live == 1) ? 1 : 2;
    SVDB_CUDA(cudaMemsetAsync(s->x64 + slot * s->ld, 0, s->ld * sizeof(double), s->stream));
    if (lv == 1)
        SVDB_CUDA(cudaMemcpyAsync(s->x64 + slot * s->ld, row, s->dim * sizeof(double), cudaMemcpyHostToDevice,
                                  s->stream));
    SVDB_CUDA(cudaMemcpyAsync(s->live + slot, &lv, 1, cudaMemcpyHostToDevice, s->stream));
    SVDB_CUDA(cudaStreamSynchronize(s->stream));
    s->dirty_list.push_back(slot);
    s->map_dirty = true;
    ++s->version;
    return SVDB_OK;
}

int svdbd_store_kill(svdbd_store* hs, int64_t slot) {
    Store* s = reinterpret_cast<Store*>(hs);
    if ((size_t)slot >= s->slots) {  // still staged: drop it from the stage
        const size_t st = (size_t)slot - s->slots;
        if (slot < 0 || st >= s->stage_rows) {
            svdb_set_error("kill: slot %lld out of range", (long long)slot);
            return SVDB_EINVAL;
        }
        s->stage_live[st] = 0;
        ++s->version;
        return SVDB_OK;
    }
    int rc = s->ensure();
    if (rc) return rc;
    const uint8_t zero = 0;
    SVDB_CUDA(cudaMemcpyAsync(s->live + slot, &zero, 1, cudaMemcpyHostToDevice, s->stream));
    SVDB_CUDA(cudaStreamSynchronize(s->stream));
    s->dirty_list.push_back(slot);  // its row error term becomes +inf (never screened)
    s->map_dirty = true;
    ++s->version;
    return SVDB_OK;
}

int svdbd_store_read_row(svdbd_store* hs, int64_t slot, double* out) {
    Store* s = reinterpret_cast<Store*>(hs);
    if (slot >= 0 && (size_t)slot >= s->slots && (size_t)slot < s->slots + s->stage_rows) {
        std::memcpy(out, s->stage.data() + ((size_t)slot - s->slots) * s->dim, s->dim * sizeof(double));
        return SVDB_OK;
    }
    if (slot < 0 || (size_t)slot >= s->slots) {
        svdb_set_error("read_row: slot %lld out of range", (long long)slot);
        return SVDB_EINVAL;
    }
    SVDB_CUDA(cudaMemcpyAsync(out, s->x64 + slot * s->ld, s->dim * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    SVDB_CUDA(cudaStreamSynchronize(s->stream));
    return SVDB_OK;
}

int svdbd_store_sync(svdbd_store* hs) { return reinterpret_cast<Store*>(hs)->sync(); }

int svdbd_store_set_seeding(svdbd_store* hs, int mode) {
    reinterpret_cast<Store*>(hs)->seed_mode = mode < 0 ? -1 : (mode ? 1 : 0);
    return SVDB_OK;
}
int svdbd_store_set_fp8(svdbd_store* hs, int mode) {
    reinterpret_cast<Store*>(hs)->fp8_mode = mode < 0 ? -1 : (mode ? 1 : 0);
    return SVDB_OK;
}
int svdbd_store_profile(svdbd_store* hs, int enable) { return reinterpret_cast<Store*>(hs)->prof_enable(enable != 0); }

int svdbd_store_profile_read(svdbd_store* hs, double* ms, int reset) {
    return reinterpret_cast<Store*>(hs)->prof_read(ms, reset != 0);
}

int svdbd_store_wait(svdbd_store* hs) {
    Store* s = reinterpret_cast<Store*>(hs);
    if (!s->stream) return SVDB_OK;
    SVDB_CUDA(cudaStreamSynchronize(s->stream));
    return s->check_error();
}

int svdbd_compare_slots(svdbd_store* hs, int metric, const int64_t* slot1, const int64_t* slot2, size_t n,
                        float* out) {
    Store* s = reinterpret_cast<Store*>(hs);
    if (n == 0) return SVDB_OK;
    int rc = s->sync();
    if (rc) return rc;
    const size_t bytes = n * (2 * sizeof(int64_t) + sizeof(float));
    rc = s->scratch_reserve(bytes);
    if (!rc) rc = s->pinned_reserve(bytes);
    if (rc) return rc;
    int64_t* d1 = (int64_t*)s->scratch;
    int64_t* d2 = d1 + n;
    float* dout = (float*)(d2 + n);
    std::memcpy(s->pin, slot1, n * sizeof(int64_t));
    std::memcpy((int64_t*)s->pin + n, slot2, n * sizeof(int64_t));
    SVDB_CUDA(cudaMemcpyAsync(d1, s->pin, 2 * n * sizeof(int64_t), cudaMemcpyHostToDevice, s->stream));
    svdb::k_compare_slots<<<(unsigned)((n + 127) / 128), 128, 0, s->stream>>>(s->x64, s->ld, (int)s->dim, metric,
                                                                             nullptr, d1, d2, (int)n, dout);
    SVDB_LAUNCH_CHECK();
    float* hout = (float*)((int64_t*)s->pin + 2 * n);
    SVDB_CUDA(cudaMemcpyAsync(hout, dout, n * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    SVDB_CUDA(cudaStreamSynchronize(s->stream));
    std::memcpy(out, hout, n * sizeof(float));
    return SVDB_OK;
}

// the same with a metric per pair (the drop-in metric calls, combined)
int svdbd_compare_slots_mixed(svdbd_store* hs, const int32_t* metric, const int64_t* slot1, const int64_t* slot2,
                              size_t n, float* out) {
    Store* s = reinterpret_cast<Store*>(hs);
    if (n == 0) return SVDB_OK;
    int rc = s->sync();
    if (rc) return rc;
    const size_t bytes = n * (2 * sizeof(int64_t) + sizeof(int32_t) + sizeof(float));
    rc = s->scratch_reserve(bytes);
    if (!rc) rc = s->pinned_reserve(bytes);
    if (rc) return rc;
    int64_t* d1 = (int64_t*)s->scratch;
    int64_t* d2 = d1 + n;
    int32_t* dm = (int32_t*)(d2 + n);
    float* dout = (float*)(dm + n);
    int64_t* h1 = (int64_t*)s->pin;
    std::memcpy(h1, slot1, n * sizeof(int64_t));
    std::memcpy(h1 + n, slot2, n * sizeof(int64_t));
    std::memcpy((int32_t*)(h1 + 2 * n), metric, n * sizeof(int32_t));
    SVDB_CUDA(cudaMemcpyAsync(d1, h1, n * (2 * sizeof(int64_t) + sizeof(int32_t)), cudaMemcpyHostToDevice,
                              s->stream));
    svdb::k_compare_slots<<<(unsigned)((n + 127) / 128), 128, 0, s->stream>>>(s->x64, s->ld, (int)s->dim, 0, dm, d1,
                                                                             d2, (int)n, dout);
    SVDB_LAUNCH_CHECK();
    float* hout = (float*)((int32_t*)(h1 + 2 * n) + n);
    SVDB_CUDA(cudaMemcpyAsync(hout, dout, n * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    SVDB_CUDA(cudaStreamSynchronize(s->stream));
    std::memcpy(out, hout, n * sizeof(float));
    return SVDB_OK;
}

// Free-standing host vectors (rows of no store, or of another dimension):
// packed into one page-locked block, one copy to the device, one launch.
// The buffers and stream are shared, guarded by a mutex.
namespace {
std::mutex g_vec_mu;
double* g_vec_buf = nullptr;  // device: vectors, then descriptors, then results
size_t g_vec_cap = 0;         // bytes
void* g_vec_pin = nullptr;
size_t g_vec_pin_cap = 0;
cudaStream_t g_vec_stream = nullptr;
}  // namespace

int svdbd_compare_vectors_batch(const int32_t* metric, const double* const* a, const double* const* b,
                                const size_t* d, size_t n, float* out) {
    if (n == 0) return SVDB_OK;
    std::lock_guard<std::mutex> lk(g_vec_mu);
    if (!g_vec_stream) SVDB_CUDA(cudaStreamCreateWithFlags(&g_vec_stream, cudaStreamNonBlocking));
    size_t nd = 0;
    for (size_t i = 0; i < n; ++i) nd += 2 * d[i];
    const size_t vbytes = svdb::round_up(nd * sizeof(double), 256), dbytes = svdb::round_up(n * 4 * sizeof(int64_t), 256);
    const size_t bytes = vbytes + dbytes + n * sizeof(float);
    if (bytes > g_vec_cap) {
        cudaFree(g_vec_buf);
        g_vec_buf = nullptr;
        g_vec_cap = 0;
        const size_t nc = svdb::round_up(bytes, 1 << 16);
        SVDB_CUDA(cudaMalloc(&g_vec_buf, nc));
        g_vec_cap = nc;
    }
    if (bytes > g_vec_pin_cap) {
        cudaFreeHost(g_vec_pin);
        g_vec_pin = nullptr;
        g_vec_pin_cap = 0;
        const size_t nc = svdb::round_up(bytes, 1 << 16);
        SVDB_CUDA(cudaMallocHost(&g_vec_pin, nc));
        g_vec_pin_cap = nc;
    }
    double* hv = (double*)g_vec_pin;
    int64_t* hd = (int64_t*)((char*)g_vec_pin + vbytes);
    size_t o = 0;
    for (size_t i = 0; i < n; ++i) {
        std::memcpy(hv + o, a[i], d[i] * sizeof(double));
        std::memcpy(hv + o + d[i], b[i], d[i] * sizeof(double));
        hd[4 * i] = (int64_t)o;
        hd[4 * i + 1] = (int64_t)(o + d[i]);
        hd[4 * i + 2] = (int64_t)d[i];
        hd[4 * i + 3] = metric[i];
        o += 2 * d[i];
    }
    SVDB_CUDA(cudaMemcpyAsync(g_vec_buf, g_vec_pin, vbytes + dbytes, cudaMemcpyHostToDevice, g_vec_stream));
    float* dout = (float*)((char*)g_vec_buf + vbytes + dbytes);
    svdb::k_compare_vecs<<<(unsigned)((n + 127) / 128), 128, 0, g_vec_stream>>>(
        g_vec_buf, (const int64_t*)((char*)g_vec_buf + vbytes), (int)n, dout);
    SVDB_LAUNCH_CHECK();
    float* hout = (float*)((char*)g_vec_pin + vbytes + dbytes);
    SVDB_CUDA(cudaMemcpyAsync(hout, dout, n * sizeof(float), cudaMemcpyDeviceToHost, g_vec_stream));
    SVDB_CUDA(cudaStreamSynchronize(g_vec_stream));
    std::memcpy(out, hout, n * sizeof(float));
    return SVDB_OK;
}

int svdbd_compare_vectors(int metric, const double* a, const double* b, size_t d, float* out) {
    const int32_t m = metric;
    return svdbd_compare_vectors_batch(&m, &a, &b, &d, 1, out);
}

}  // extern "C"
