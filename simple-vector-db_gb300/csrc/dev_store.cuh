// dev_store.cuh -- the device store object shared by the CUDA translation
// units (layout documented at the top of dev_store.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

namespace svdb {

struct GemmPlanCache;  // dev_gemm.cu

struct Store {
    size_t dim = 0, ld = 0, ldb = 0;
    size_t cap = 0;    // allocated slots
    size_t slots = 0;  // slots on the device
    size_t nlive = 0;  // live slots as of the last sync
    cudaStream_t stream = nullptr;

    double* x64 = nullptr;
    __nv_bfloat16* xb = nullptr;
    double* sq64 = nullptr;
    float4* rowp = nullptr;  // {|x| up (-1: dead slot), |bf16 x| up, |x - bf16 x| up (inf: unscreenable), |x|^2/2}
    uint8_t* live = nullptr;
    int64_t* logical = nullptr;
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

    // per-call scratch (device) and staging (pinned host)
    void* scratch = nullptr;
    size_t scratch_bytes = 0;
    void* pin = nullptr;
    size_t pin_bytes = 0;

    GemmPlanCache* gemm = nullptr;

    int ensure();
    int grow(size_t need);
    int flush();
    int sync();
    int scratch_reserve(size_t bytes);
    int pinned_reserve(size_t bytes);
    void release_extra();
};

}  // namespace svdb
