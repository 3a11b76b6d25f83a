// dev_gemm.cu -- BF16 tensor-core screen + certified FP64 re-rank.
#include "dev_search.cuh"

namespace svdb {

struct GemmPlanCache {};

void Store::release_extra() {
    delete gemm;
    gemm = nullptr;
}

size_t search_bf16_scratch(const Store*, size_t, size_t) { return 256; }

int search_bf16(Store*, const SearchArgs&, void*, size_t, svdb_search_stats*) {
    svdb_set_error("search: BF16 precision is not available in this build");
    return SVDB_EINVAL;
}

}  // namespace svdb
