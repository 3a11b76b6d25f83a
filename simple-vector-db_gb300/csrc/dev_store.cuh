// dev_store.cuh -- the device store object shared by the CUDA translation
// units (layout documented at the top of dev_store.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "svdb_device.h"

namespace svdb {

struct GemmPlanCache;  // dev_gemm.cu
struct UuidIndex;      // dev_uuid.cu
struct KdmTree;        // dev_kdm.cu

struct Store {
    size_t dim = 0, ld = 0, ldb = 0;
    size_t cap = 0;    // allocated slots
    size_t slots = 0;  // slots on the device
    size_t nlive = 0;  // live slots as of the last sync
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;      // work beside a search's screen (created on first use)
    cudaEvent_t ev_fork = nullptr, ev_side = nullptr;
    int side_ready();

    double* x64 = nullptr;
    __nv_bfloat16* xb = nullptr;
    float* x32 = nullptr;  // FP32 shadow (cap x ld), read by the refinement stage
    __nv_bfloat16* xbn = nullptr;  // BF16 shadow of x / |x| (cap x ldb): the cosine screen
    float2* rowpn = nullptr;       // {|bxn| up, |x/|x| - bxn| up} per row
    size_t ldb8 = 0;               // FP8 shadow row length (bytes), D rounded up to 128
    uint8_t* xbn8 = nullptr;       // E4M3 shadow of 256 x/|x| (cap x ldb8), FP8 cosine screen
    float2* rowpn8 = nullptr;      // {|bxn8|/256 up, |x/|x| - bxn8/256| up} per row
    uint8_t* xb8 = nullptr;        // E4M3 shadow of x 2^f_i (cap x ldb8), f_i per row: FP8 dot / Euclidean screen
    float4* rowp8 = nullptr;       // {|bx8| up, |x - bx8| up, 2^-f_i, 0} per row, bx8 = e4m3(x 2^f_i) 2^-f_i
    float4* sqf = nullptr;         // FP32 intervals for the refinement: {|x|^2 down, |x|^2 up,
                                   //  1/(2|x|) down, 1/(2|x|) up}
    int* d_nmax = nullptr;         // (unused; the maxima live in d_count[1..4])
    double* sq64 = nullptr;
    float4* rowp = nullptr;  // {|x| up (-1: dead slot), |bf16 x| up, |x - bf16 x| up (inf: unscreenable), |x|^2/2}
    uint8_t* live = nullptr;
    int64_t* logical = nullptr;
    int64_t* mapblk = nullptr;  // per-chunk offsets of the slot->logical map
    int64_t* d_nlive = nullptr;
    int64_t h_nlive = 0;

    // staged appends (host), flushed as one pitched copy
    std::vector<double> stage;
    std::vector<uint8_t> stage_live;
    size_t stage_rows = 0;

    // rows whose derived arrays must be rebuilt
    int64_t derive_lo = -1, derive_hi = -1;
    std::vector<int64_t> dirty_list;
    bool map_dirty = false;

    // live rows the BF16 screen cannot bound (|x| >= 1e15 or non-finite); as of the last sync
    int64_t n_unscreen = 0;
    int* d_count = nullptr;
    int* d_err = nullptr;  // set by a kernel whose bounded wait ran out; read and cleared at sync points
    int check_error();

    // per-call scratch (device) and staging (pinned host); scratch2 serves a
    // stage's fallback while scratch is still in use
    void* scratch = nullptr;
    size_t scratch_bytes = 0;
    void* scratch2 = nullptr;
    size_t scratch2_bytes = 0;
    void* pin = nullptr;
    size_t pin_bytes = 0;

    GemmPlanCache* gemm = nullptr;

    // Bumped whenever something a captured CUDA graph bakes in changes: an
    // array moves (growth, scratch reallocation), the slot count, the live
    // count or the unscreenable count changes.  A ragged plan compares it
    // with the value at capture time and captures again when it differs.
    uint64_t epoch = 0;
    // Bumped by every change of the rows' contents or liveness (derived
    // structures built from the rows, like the median KD tree, compare it).
    uint64_t version = 0;

    // stage timing (svdb_profile): a ring of per-search event sets, resolved
    // lazily so profiling adds no host synchronisation to a search
    static constexpr int kProfRing = 64;
    static constexpr int kProfMarks = SVDB_NSTAGES + 1;
    bool prof = false;
    int seed_mode = -1;  // tensor-core screens' threshold seeding: -1 the default rule, 0 off, 1 on
    int fp8_mode = -1;   // SVDB_PREC_FP8 searches: -1 the default rule, 0 BF16 screens, 1 E4M3 screens
    bool prof_events = false;
    cudaEvent_t pev[kProfRing][kProfMarks];
    int prof_head = 0, prof_pending = 0, prof_cur = -1;
    double prof_ms[SVDB_NSTAGES] = {};
    int64_t prof_calls = 0;
    int prof_enable(bool on);
    void prof_begin();
    void prof_mark(int boundary);
    void prof_end() { prof_cur = -1; }
    int prof_resolve_one();
    int prof_read(double* ms, bool reset);

    // uuid -> position index (dev_uuid.cu); created by the first uuid set
    UuidIndex* uid = nullptr;
    int uuid_set(int64_t slot, const char* uuid37);  // staged; applied at sync
    int uuid_flush();
    void uuid_free();
    int uuid_find(const char* uuids37, size_t n, int64_t* out_pos);
    int append_raw(const void* rows, size_t n, size_t rowbytes);
    int read_block(int64_t first, size_t n, double* rows, char* uuids37, uint8_t* live);

    // median-split KD tree over the searchable rows (dev_kdm.cu), rebuilt on demand
    KdmTree* kdm = nullptr;
    int kdm_nearest(size_t kdim, const double* q, size_t nq, size_t qstride, int64_t* out_pos);
    void kdm_free();

    int ensure();
    int grow(size_t need);
    int flush();
    int sync();
    int scratch_reserve(size_t bytes);
    int scratch2_reserve(size_t bytes);
    int pinned_reserve(size_t bytes);
    void release_extra();
};

// Device address of the no-allocation search's fixed scratch array for the
// current device and context (dev_noalloc.cu); the store's device set-up calls
// it so that the array's module is loaded with the store's own allocations.
int noalloc_setup(void** out);

}  // namespace svdb
