// dev_search.cuh -- pieces of the top-k search shared by the FP64 scan
// (dev_search.cu) and the BF16 screen + re-rank (dev_gemm.cu).
#pragma once

#include <vector>

#include "dev_common.cuh"
#include "dev_store.cuh"

namespace svdb {

// one (value, slot) result; 16 bytes
struct __align__(16) Entry {
    double val;
    int id;
    int pad;
};

// device buffers of one search call (all in the store's scratch)
struct SearchArgs {
    const double* q;     // nq x ld, zero-padded
    const double* qsq;   // nq canonical sums of squares
    size_t nq, k;
    int metric;
    int64_t* ids;        // nq x k (device)
    double* dists;       // nq x k (device)
    double* err;         // nq x k (device) or null
    const int* nq_dev = nullptr;  // if set: only the first *nq_dev queries are answered (device-side count)
    // tensor-core screens: start the running thresholds from the exact k-th
    // best lower bound over a sample of the rows (-1: for the FP8 screen only)
    int seed = -1;
    // set: qsq is written on another stream; wait on this event before reading it
    cudaEvent_t qsq_ready = nullptr;
};

// FP64 bound on |computed - exact| for one result (see dev_search.cu)
__device__ __forceinline__ double result_err_bound(int metric, int d, double val, double qsq, double xsq) {
    const double u = 1.1102230246251565e-16;  // 2^-53
    if (isnan(val)) return val;
    if (metric == SVDB_COSINE) return 2.0 * (d + 8) * u;
    if (metric == SVDB_EUCLIDEAN) return val * (d + 8) * u;
    return (d + 4) * u * sqrt(qsq) * sqrt(xsq) * (1.0 + 1e-15);
}

// queries (nq rows, stride qs) -> padded buffer (stride ld) + sums of squares
int prep_queries_fp64(Store* s, const double* q_dev, size_t qs, size_t nq, double* qbuf, double* qsq);
// the same, with the canonical sums of squares on the store's side stream
// (they are read only after the screen): *ready is the event that marks them
// written, or null when they were computed on the store's stream (a stream
// being captured into a graph keeps the one-stream form)
int prep_queries_split(Store* s, const double* q_dev, size_t qs, size_t nq, double* qbuf, double* qsq,
                       cudaEvent_t* ready);

// exact FP64 scan + merge over all live slots, writing SearchArgs outputs
// marks=false: called as the fallback of another stage (no profiling marks)
int search_fp64(Store* s, const SearchArgs& a, void* scratch, size_t scratch_bytes, uint32_t* kernels,
                bool marks = true);
size_t search_fp64_scratch(const Store* s, size_t nq, size_t k);

// BF16 screen + certified FP64 re-rank (dev_gemm.cu)
// f8: the cosine screen on the E4M3 shadow (other metrics keep BF16)
int search_bf16(Store* s, const SearchArgs& a, void* scratch, size_t scratch_bytes, svdb_search_stats* st,
                bool f8 = false);
size_t search_bf16_scratch(const Store* s, size_t nq, size_t k);
// the screen certifies k <= 128 on stores without unscreenable rows
bool bf16_supported(const Store* s, size_t k);

// Fused screens (dev_gemm.cu): several BF16 searches, on one or more stores
// and with any k, screened by one tensor-core launch (up to 16 searches per
// launch); each search's other phases run on its store's stream.
struct FusedItem {
    Store* s = nullptr;
    int seed = -1;              // SearchArgs::seed
    const double* q = nullptr;  // device queries, nq x s->dim
    size_t nq = 0, k = 0;       // 1 <= k <= 128; the store holds no unscreenable rows
    int64_t* ids = nullptr;     // device outputs, nq x k
    double* dists = nullptr;
    void* scratch = nullptr;    // device, the size fused_create gave (set with fused_set_scratch)
};
struct FusedPlan;
// the launches and their schedules, and each search's scratch size;
// epi_weight: the schedule's cost of a tile's epilogue, in k blocks
int fused_create(const std::vector<FusedItem>& items, int metric, double epi_weight, FusedPlan** out,
                 std::vector<size_t>* bytes);
void fused_set_scratch(FusedPlan* p, size_t i, void* scratch);
size_t fused_launches(const FusedPlan* p);
int fused_launch_of(const FusedPlan* p, size_t i);  // the launch that screens search i
int fused_begin(FusedPlan* p, size_t i);  // search i's queries and row terms, on its store's stream
int fused_screen(FusedPlan* p, size_t launch, cudaStream_t st);  // after every search's begin
int fused_end(FusedPlan* p, size_t i);    // search i's select ... redo, on its store's stream (after the screen)
// search i's statistics of its last run (8 counters, see scr::kStats); waits for its store's stream
int fused_stats(FusedPlan* p, size_t i, unsigned long long* out);
void fused_destroy(FusedPlan* p);

// svdbd_search with SearchArgs::seed chosen by the caller
int search_seeded(Store* s, const double* q, size_t nq, size_t k, int metric, int precision, int64_t* ids,
                  double* dists, double* err, int on_device, svdb_search_stats* st, int seed);

int num_sms();

}  // namespace svdb
