// dev_ragged.cu -- one ragged batch of top-k queries over several stores of
// different dimensions, replayed as one CUDA graph.
//
// A plan binds, per part, a store, its queries (device, nq x dim), a k per
// query (1..128) and the output buffers (device, nq x stride).  One run
// answers every part: the part's queries are searched on its store's stream
// (the same BF16 screen + certified re-rank or FP64 scan as a single search),
// and the results are scattered into the caller's layout, entries past a
// query's own k set to -1 / NaN.  The whole run is captured once into a CUDA
// graph and replayed with one launch; it is captured again when a store
// changes in a way the graph bakes in (the store's epoch).
//
// Choices that change the speed but not the results, timed by the autotuner
// on the plan's own inputs at creation:
//   grouping   0: one search per part, k = the part's largest k;
//              1: one search per k class (k <= 16, <= 32, <= 128), so
//                 small-k queries do not pay for the part's largest k (a
//                 screen's threshold is the minimum of k shared bins: fewer
//                 bins settle sooner);
//   concurrent 1: the parts of different stores run on their stores' streams
//                 at the same time (a screen fills the SMs another part's
//                 screen leaves idle at its tail); 0: one part after another;
//   fused      1: the BF16 searches' screens run as one tensor-core launch
//              (up to 16 searches) over all stores (work split in proportion
//              to each search's tiles, see dev_gemm.cu), their other phases
//              on the stores' streams; 0: every search launches its own
//              screen; with fused screens, also the schedule's epilogue weight;
//   seed       thresholds seeded from a 1/16 sample of each store, or not;
//   screen     (cosine with a tensor-core precision) per store, the BF16 or
//              the FP8 screen.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "dev_common.cuh"
#include "dev_search.cuh"
#include "dev_store.cuh"

namespace svdb {

// queries of one k class, gathered from the part's buffer (rows idx[i])
__global__ void k_ragged_gather(const double* __restrict__ src, size_t dim, const int* __restrict__ idx, int n,
                                double* __restrict__ dst) {
    const size_t total = (size_t)n * dim;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const size_t i = t / dim, e = t - i * dim;
        dst[t] = src[(size_t)idx[i] * dim + e];
    }
}

// results of one search (n x kg, best first) -> the caller's rows idx[i] (or
// i) of stride `stride`; entries at or past the query's own k are -1 / NaN
__global__ void k_ragged_scatter(const int64_t* __restrict__ gids, const double* __restrict__ gd, int kg,
                                 const int* __restrict__ idx, int n, const uint32_t* __restrict__ kq, size_t stride,
                                 int64_t* __restrict__ ids, double* __restrict__ dists) {
    const size_t total = (size_t)n * stride;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const size_t i = t / stride, j = t - i * stride;
        const size_t q = idx ? (size_t)idx[i] : i;
        const bool keep = j < (size_t)kq[q] && j < (size_t)kg;
        ids[q * stride + j] = keep ? gids[i * kg + j] : -1;
        dists[q * stride + j] = keep ? gd[i * kg + j] : __longlong_as_double(0x7ff8000000000000ll);
    }
}

namespace {

struct Part {
    Store* s = nullptr;
    size_t nq = 0, stride = 0;
    const double* q = nullptr;
    int64_t* ids = nullptr;
    double* dists = nullptr;
    std::vector<uint32_t> hk;
    uint32_t* d_k = nullptr;
};

// one search of a run: `n` queries of part `part` with k = kg
struct Group {
    int part = 0, n = 0, kg = 0;
    int fidx = -1;  // its index in the fused plan (-1: screened by a launch of its own)
    int* d_idx = nullptr;   // rows of the part (nullptr: all of them, in order)
    double* d_q = nullptr;  // gathered queries (nullptr: the part's own buffer)
    int64_t* d_ids = nullptr;
    double* d_dists = nullptr;
};

struct Plan {
    std::vector<Part> parts;
    std::vector<Store*> stores;  // distinct, in first-use order
    int metric = 0, precision = 0;
    std::vector<int> sprec;  // per store: the precision its searches run with (the autotuner may swap BF16 / FP8)
    bool graph_on = true;
    int grouping = 0, concurrent = 1;
    std::vector<Group> groups;
    cudaStream_t origin = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_done = nullptr, ev_t0 = nullptr, ev_t1 = nullptr;
    std::vector<cudaEvent_t> ev_store;  // per store: its part of a run is done / its earlier work is done
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<uint64_t> epochs;
    float tuned_ms[4] = {0, 0, 0, 0};
    float swap_ms[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    uint32_t captures = 0;
    // fused screens
    int fused = 0;
    double epi_weight = 2.0;
    FusedPlan* fp = nullptr;
    std::vector<void*> fscratch;
    std::vector<uint64_t> fepochs;  // store epochs the fused plan was made for
    std::vector<cudaEvent_t> ev_launch;  // per fused launch: its screen is done
    float fused_ms[2] = {0, 0};
    float weight_ms[3] = {0, 0, 0};
    int seed = -1;  // SearchArgs::seed of every search (the autotuner tries 1)
    float seed_ms = 0;
};

int k_class(uint32_t k) { return k <= 16 ? 0 : (k <= 32 ? 1 : 2); }

void free_fused(Plan* p) {
    if (p->fp) fused_destroy(p->fp);
    p->fp = nullptr;
    for (void* b : p->fscratch) cudaFree(b);
    p->fscratch.clear();
    p->fepochs.clear();
    for (Group& g : p->groups) g.fidx = -1;
}

void free_groups(Plan* p) {
    free_fused(p);
    for (Group& g : p->groups) {
        cudaFree(g.d_idx);
        cudaFree(g.d_q);
        cudaFree(g.d_ids);
        cudaFree(g.d_dists);
    }
    p->groups.clear();
}

void drop_graph(Plan* p) {
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    p->exec = nullptr;
    p->graph = nullptr;
}

// the searches of a run for the current grouping, with their device buffers
int make_groups(Plan* p) {
    free_groups(p);
    for (size_t pi = 0; pi < p->parts.size(); ++pi) {
        const Part& P = p->parts[pi];
        if (P.nq == 0) continue;
        std::vector<std::vector<int>> cls(p->grouping ? 3 : 1);
        for (size_t i = 0; i < P.nq; ++i) cls[p->grouping ? k_class(P.hk[i]) : 0].push_back((int)i);
        for (auto& rows : cls) {
            if (rows.empty()) continue;
            Group g;
            g.part = (int)pi;
            g.n = (int)rows.size();
            uint32_t kg = 0;
            for (int r : rows) kg = std::max(kg, P.hk[r]);
            g.kg = (int)kg;
            const bool all = rows.size() == P.nq;  // the whole part, in order: no gather
            cudaError_t e = cudaSuccess;
            if (!all) {
                e = cudaMalloc(&g.d_idx, rows.size() * sizeof(int));
                if (e == cudaSuccess) e = cudaMalloc(&g.d_q, rows.size() * P.s->dim * sizeof(double));
                if (e == cudaSuccess)
                    e = cudaMemcpy(g.d_idx, rows.data(), rows.size() * sizeof(int), cudaMemcpyHostToDevice);
            }
            if (e == cudaSuccess) e = cudaMalloc(&g.d_ids, rows.size() * kg * sizeof(int64_t));
            if (e == cudaSuccess) e = cudaMalloc(&g.d_dists, rows.size() * kg * sizeof(double));
            p->groups.push_back(g);
            if (e != cudaSuccess) {
                cudaGetLastError();
                svdb_set_error("ragged plan: cannot allocate group buffers: %s", cudaGetErrorString(e));
                return e == cudaErrorMemoryAllocation ? SVDB_ENOMEM : SVDB_ECUDA;
            }
        }
    }
    return SVDB_OK;
}

bool fused_current(const Plan* p) {
    if (!p->fp || p->fepochs.size() != p->stores.size()) return false;
    for (size_t i = 0; i < p->stores.size(); ++i)
        if (p->stores[i]->epoch != p->fepochs[i]) return false;
    return true;
}

// the fused plan over the searches that can take part (BF16 screen, a store
// the screen certifies), with its scratch; made again when a store changes
int build_fused(Plan* p) {
    free_fused(p);
    std::vector<FusedItem> items;
    std::vector<int> gi;
    for (size_t g = 0; g < p->groups.size(); ++g) {
        const Group& G = p->groups[g];
        const Part& P = p->parts[G.part];
        const size_t si = std::find(p->stores.begin(), p->stores.end(), P.s) - p->stores.begin();
        if (p->sprec[si] != SVDB_PREC_BF16 || !bf16_supported(P.s, (size_t)G.kg)) continue;
        FusedItem it;
        it.s = P.s;
        it.seed = p->seed;
        it.q = G.d_q ? G.d_q : P.q;
        it.nq = (size_t)G.n;
        it.k = (size_t)G.kg;
        it.ids = G.d_ids;
        it.dists = G.d_dists;
        items.push_back(it);
        gi.push_back((int)g);
    }
    if (items.empty()) return SVDB_OK;
    std::vector<size_t> bytes;
    int rc = fused_create(items, p->metric, p->epi_weight, &p->fp, &bytes);
    if (rc) return rc;
    for (size_t i = 0; i < items.size(); ++i) {
        void* b = nullptr;
        const cudaError_t e = cudaMalloc(&b, std::max<size_t>(bytes[i], 256));
        if (e != cudaSuccess) {
            cudaGetLastError();
            free_fused(p);
            svdb_set_error("ragged plan: cannot allocate fused screen scratch: %s", cudaGetErrorString(e));
            return e == cudaErrorMemoryAllocation ? SVDB_ENOMEM : SVDB_ECUDA;
        }
        p->fscratch.push_back(b);
        fused_set_scratch(p->fp, i, b);
        p->groups[gi[i]].fidx = (int)i;
    }
    while (p->ev_launch.size() < fused_launches(p->fp)) {  // (events outlive the fused plan: created once)
        cudaEvent_t ev = nullptr;
        const cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            cudaGetLastError();
            free_fused(p);
            svdb_set_error("ragged plan: cannot create events: %s", cudaGetErrorString(e));
            return SVDB_ECUDA;
        }
        p->ev_launch.push_back(ev);
    }
    for (Store* s : p->stores) p->fepochs.push_back(s->epoch);
    return SVDB_OK;
}

// the searches of one part's store (the plan's i-th), on that store's stream
int enqueue_store(Plan* p, size_t si) {
    Store* s = p->stores[si];
    for (const Group& g : p->groups) {
        const Part& P = p->parts[g.part];
        if (P.s != s || (p->fused && g.fidx >= 0)) continue;
        const double* q = P.q;
        if (g.d_idx) {
            const size_t total = (size_t)g.n * s->dim;
            k_ragged_gather<<<(unsigned)std::min<size_t>((total + 255) / 256, 4096), 256, 0, s->stream>>>(
                P.q, s->dim, g.d_idx, g.n, g.d_q);
            SVDB_LAUNCH_CHECK();
            q = g.d_q;
        }
        int rc = search_seeded(s, q, (size_t)g.n, (size_t)g.kg, p->metric, p->sprec[si], g.d_ids, g.d_dists,
                               nullptr, 1, nullptr, p->seed);
        if (rc) return rc;
        const size_t total = (size_t)g.n * P.stride;
        k_ragged_scatter<<<(unsigned)std::min<size_t>((total + 255) / 256, 4096), 256, 0, s->stream>>>(
            g.d_ids, g.d_dists, g.kg, g.d_idx, g.n, P.d_k, P.stride, P.ids, P.dists);
        SVDB_LAUNCH_CHECK();
    }
    return SVDB_OK;
}

// the fused searches' phases before (phase 0) or after (phase 1: those of
// fused launch `launch`) their screens, on store si's stream; phase 0 also
// runs the store's other searches
int enqueue_fused_store(Plan* p, size_t si, int phase, int launch = -1) {
    Store* s = p->stores[si];
    if (phase == 0) {
        int rc = enqueue_store(p, si);
        if (rc) return rc;
    }
    for (const Group& g : p->groups) {
        const Part& P = p->parts[g.part];
        if (P.s != s || g.fidx < 0) continue;
        if (phase == 1 && fused_launch_of(p->fp, (size_t)g.fidx) != launch) continue;
        if (phase == 0) {
            if (g.d_idx) {
                const size_t total = (size_t)g.n * s->dim;
                k_ragged_gather<<<(unsigned)std::min<size_t>((total + 255) / 256, 4096), 256, 0, s->stream>>>(
                    P.q, s->dim, g.d_idx, g.n, g.d_q);
                SVDB_LAUNCH_CHECK();
            }
            int rc = fused_begin(p->fp, (size_t)g.fidx);
            if (rc) return rc;
        } else {
            int rc = fused_end(p->fp, (size_t)g.fidx);
            if (rc) return rc;
            const size_t total = (size_t)g.n * P.stride;
            k_ragged_scatter<<<(unsigned)std::min<size_t>((total + 255) / 256, 4096), 256, 0, s->stream>>>(
                g.d_ids, g.d_dists, g.kg, g.d_idx, g.n, P.d_k, P.stride, P.ids, P.dists);
            SVDB_LAUNCH_CHECK();
        }
    }
    return SVDB_OK;
}

// a run with fused screens: every store's first phase at once, the fused
// launches on the origin stream, then every store's second phase
int enqueue_fused(Plan* p) {
    SVDB_CUDA(cudaEventRecord(p->ev_fork, p->origin));
    for (size_t i = 0; i < p->stores.size(); ++i) {
        Store* s = p->stores[i];
        SVDB_CUDA(cudaStreamWaitEvent(s->stream, p->ev_fork, 0));
        int rc = enqueue_fused_store(p, i, 0);
        if (rc) return rc;
        SVDB_CUDA(cudaEventRecord(p->ev_store[i], s->stream));
    }
    for (size_t i = 0; i < p->stores.size(); ++i) SVDB_CUDA(cudaStreamWaitEvent(p->origin, p->ev_store[i], 0));
    // launch l's searches finish on their stores' streams while launch l + 1 screens
    const size_t nl = fused_launches(p->fp);
    for (size_t l = 0; l < nl; ++l) {
        int rc = fused_screen(p->fp, l, p->origin);
        if (rc) return rc;
        SVDB_CUDA(cudaEventRecord(p->ev_launch[l], p->origin));
    }
    for (size_t i = 0; i < p->stores.size(); ++i) {
        Store* s = p->stores[i];
        for (size_t l = 0; l < nl; ++l) {
            SVDB_CUDA(cudaStreamWaitEvent(s->stream, p->ev_launch[l], 0));
            int rc = enqueue_fused_store(p, i, 1, (int)l);
            if (rc) return rc;
        }
        SVDB_CUDA(cudaEventRecord(p->ev_store[i], s->stream));
    }
    for (size_t i = 0; i < p->stores.size(); ++i) SVDB_CUDA(cudaStreamWaitEvent(p->origin, p->ev_store[i], 0));
    return SVDB_OK;
}

// one run, forked from and joined back to the origin stream (captured or not)
int enqueue(Plan* p) {
    if (p->fused) {
        if (!fused_current(p)) {
            int rc = build_fused(p);
            if (rc) return rc;
        }
        if (p->fp) return enqueue_fused(p);
    }
    SVDB_CUDA(cudaEventRecord(p->ev_fork, p->origin));
    cudaEvent_t prev = p->ev_fork;
    for (size_t i = 0; i < p->stores.size(); ++i) {
        Store* s = p->stores[i];
        SVDB_CUDA(cudaStreamWaitEvent(s->stream, p->concurrent ? p->ev_fork : prev, 0));
        int rc = enqueue_store(p, i);
        if (rc) return rc;
        SVDB_CUDA(cudaEventRecord(p->ev_store[i], s->stream));
        prev = p->ev_store[i];
    }
    for (size_t i = 0; i < p->stores.size(); ++i) SVDB_CUDA(cudaStreamWaitEvent(p->origin, p->ev_store[i], 0));
    return SVDB_OK;
}

bool epochs_current(const Plan* p) {
    if (p->epochs.size() != p->stores.size()) return false;
    for (size_t i = 0; i < p->stores.size(); ++i)
        if (p->stores[i]->epoch != p->epochs[i]) return false;
    return true;
}

int check_stores(Plan* p) {
    for (Store* s : p->stores) {
        int rc = s->check_error();
        if (rc) return rc;
    }
    return SVDB_OK;
}

// A direct run first (it sizes every store's scratch for this plan and makes
// the one-time kernel set-up), then the capture of a second run.
int capture(Plan* p) {
    drop_graph(p);
    int rc = enqueue(p);
    if (rc) return rc;
    SVDB_CUDA(cudaStreamSynchronize(p->origin));
    rc = check_stores(p);
    if (rc) return rc;
    p->epochs.clear();
    for (Store* s : p->stores) p->epochs.push_back(s->epoch);
    std::vector<char> prof(p->stores.size());
    for (size_t i = 0; i < p->stores.size(); ++i) {  // stage timing is not recorded inside a graph
        prof[i] = p->stores[i]->prof;
        p->stores[i]->prof = false;
    }
    SVDB_CUDA(cudaStreamBeginCapture(p->origin, cudaStreamCaptureModeThreadLocal));
    rc = enqueue(p);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(p->origin, &g);
    for (size_t i = 0; i < p->stores.size(); ++i) p->stores[i]->prof = prof[i] != 0;
    if (rc || e != cudaSuccess || !g) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        if (!rc) {
            svdb_set_error("ragged plan: graph capture failed: %s", cudaGetErrorString(e));
            rc = SVDB_ECUDA;
        }
        return rc;
    }
    p->graph = g;
    SVDB_CUDA(cudaGraphInstantiate(&p->exec, p->graph, 0));
    if (!epochs_current(p)) {  // nothing may move between the direct run and the capture
        drop_graph(p);
        svdb_set_error("ragged plan: a store changed during capture");
        return SVDB_ECUDA;
    }
    ++p->captures;
    return SVDB_OK;
}

int run(Plan* p) {
    for (Store* s : p->stores) {  // pending mutations are applied first (outside any capture)
        int rc = s->sync();
        if (rc) return rc;
    }
    if (!p->graph_on) return enqueue(p);
    if (!p->exec || !epochs_current(p)) {
        int rc = capture(p);
        if (rc) return rc;
    }
    // earlier work on the stores' streams comes first; later work on them
    // (mutations, searches) waits for this run
    for (size_t i = 0; i < p->stores.size(); ++i) {
        SVDB_CUDA(cudaEventRecord(p->ev_store[i], p->stores[i]->stream));
        SVDB_CUDA(cudaStreamWaitEvent(p->origin, p->ev_store[i], 0));
    }
    SVDB_CUDA(cudaGraphLaunch(p->exec, p->origin));
    SVDB_CUDA(cudaEventRecord(p->ev_done, p->origin));
    for (Store* s : p->stores) SVDB_CUDA(cudaStreamWaitEvent(s->stream, p->ev_done, 0));
    return SVDB_OK;
}

int configure(Plan* p, int grouping, int concurrent, int fused = 0) {
    drop_graph(p);
    const bool regroup = p->groups.empty() || grouping != p->grouping;
    p->grouping = grouping;
    p->concurrent = concurrent;
    p->fused = fused;
    if (!fused) free_fused(p);
    return regroup ? make_groups(p) : SVDB_OK;
}

// ms per run of the current configuration: one direct run (it sizes the
// stores' scratch; a configuration slower than `cutoff` ms stops there), then
// the capture, then the best of `reps` timed runs
int time_config(Plan* p, int reps, float cutoff, float* ms) {
    if (p->fused && !fused_current(p)) {  // its scratch is allocated outside the timed runs
        const int rb = build_fused(p);
        if (rb) return rb;
    }
    SVDB_CUDA(cudaEventRecord(p->ev_t0, p->origin));
    int rc = enqueue(p);
    if (rc) return rc;
    SVDB_CUDA(cudaEventRecord(p->ev_t1, p->origin));
    SVDB_CUDA(cudaEventSynchronize(p->ev_t1));
    float t = 0;
    SVDB_CUDA(cudaEventElapsedTime(&t, p->ev_t0, p->ev_t1));
    rc = check_stores(p);
    if (rc || t > cutoff) {
        *ms = t;
        return rc;
    }
    rc = run(p);
    if (rc) return rc;
    SVDB_CUDA(cudaStreamSynchronize(p->origin));
    float best = 1e30f;
    for (int r = 0; r < reps; ++r) {
        SVDB_CUDA(cudaEventRecord(p->ev_t0, p->origin));
        rc = run(p);
        if (rc) return rc;
        SVDB_CUDA(cudaEventRecord(p->ev_t1, p->origin));
        SVDB_CUDA(cudaEventSynchronize(p->ev_t1));
        SVDB_CUDA(cudaEventElapsedTime(&t, p->ev_t0, p->ev_t1));
        best = std::min(best, t);
    }
    *ms = best;
    return check_stores(p);
}

// First the layout: every (grouping, concurrency) pair with the plan's
// precision.  Then, for a cosine plan with a tensor-core precision, each
// store's screen in turn is swapped (BF16 <-> FP8: the same exact answers, at
// a speed that depends on the store's data and its queries) and the swap is
// kept when the run gets faster.  A trial already slower than 1.5x the best
// after its first run is not repeated (an FP8 screen over near-orthogonal
// rows passes most of them on to the refinement).
int autotune(Plan* p) {
    bool mixed = false;  // does any part hold queries of more than one k class?
    for (const Part& P : p->parts)
        for (size_t i = 1; i < P.nq && !mixed; ++i) mixed = k_class(P.hk[i]) != k_class(P.hk[0]);
    // (grouping, concurrent, fused); the fused screen runs every store's
    // other phases concurrently
    const int cfg[6][3] = {{0, 1, 0}, {1, 1, 0}, {0, 0, 0}, {1, 0, 0}, {0, 1, 1}, {1, 1, 1}};
    const bool tc = p->precision != SVDB_PREC_FP64;
    float ms[6] = {0, 0, 0, 0, 0, 0};
    int best = -1;
    for (int c = 0; c < 6; ++c) {
        if (cfg[c][0] && !mixed) continue;
        if (!cfg[c][1] && p->stores.size() < 2) continue;
        if (cfg[c][2] && !tc) continue;
        int rc = configure(p, cfg[c][0], cfg[c][1], cfg[c][2]);
        if (!rc) rc = time_config(p, 3, best < 0 ? 1e30f : 1.5f * ms[best], &ms[c]);
        if (rc) return rc;
        if (best < 0 || ms[c] < ms[best]) best = c;
    }
    for (int c = 0; c < 4; ++c) p->tuned_ms[c] = ms[c];
    p->fused_ms[0] = ms[4];
    p->fused_ms[1] = ms[5];
    int rc = configure(p, cfg[best][0], cfg[best][1], cfg[best][2]);
    if (rc) return rc;
    float best_ms = ms[best];
    if (p->fused) {  // the fused schedule's epilogue weight (work per tile beyond its k blocks)
        const double w[3] = {1.0, 4.0, 8.0};
        double keep = p->epi_weight;
        for (int i = 0; i < 3; ++i) {
            p->epi_weight = w[i];
            drop_graph(p);
            free_fused(p);
            rc = time_config(p, 3, 1.5f * best_ms, &p->weight_ms[i]);
            if (rc) return rc;
            if (p->weight_ms[i] < best_ms) {
                best_ms = p->weight_ms[i];
                keep = w[i];
            }
        }
        p->epi_weight = keep;
        drop_graph(p);
        free_fused(p);
    }
    if (tc) {  // thresholds seeded from a sample of each store (BF16 screens too)
        p->seed = 1;
        drop_graph(p);
        free_fused(p);
        rc = time_config(p, 3, 1.5f * best_ms, &p->seed_ms);
        if (rc) return rc;
        if (p->seed_ms < best_ms)
            best_ms = p->seed_ms;
        else
            p->seed = -1;
        drop_graph(p);
        free_fused(p);
    }
    if (p->metric != SVDB_COSINE || p->precision == SVDB_PREC_FP64) return p->fused ? build_fused(p) : SVDB_OK;
    for (size_t i = 0; i < p->stores.size() && i < 8; ++i) {
        const int keep = p->sprec[i];
        p->sprec[i] = keep == SVDB_PREC_BF16 ? SVDB_PREC_FP8 : SVDB_PREC_BF16;
        drop_graph(p);
        free_fused(p);
        rc = time_config(p, 3, 1.5f * best_ms, &p->swap_ms[i]);
        if (rc) return rc;
        if (p->swap_ms[i] < best_ms)
            best_ms = p->swap_ms[i];
        else
            p->sprec[i] = keep;
    }
    drop_graph(p);
    free_fused(p);
    return p->fused ? build_fused(p) : SVDB_OK;  // the kept choice, ready for the first run
}

void destroy(Plan* p) {
    if (p->origin) cudaStreamSynchronize(p->origin);
    drop_graph(p);
    free_groups(p);
    for (Part& P : p->parts) cudaFree(P.d_k);
    for (cudaEvent_t e : p->ev_store) cudaEventDestroy(e);
    for (cudaEvent_t e : p->ev_launch) cudaEventDestroy(e);
    for (cudaEvent_t e : {p->ev_fork, p->ev_done, p->ev_t0, p->ev_t1})
        if (e) cudaEventDestroy(e);
    if (p->origin) cudaStreamDestroy(p->origin);
    delete p;
}

}  // namespace
}  // namespace svdb

using svdb::Plan;
using svdb::Store;

extern "C" {

svdbd_ragged* svdbd_ragged_create(const svdbd_ragged_part* parts, size_t nparts, int metric, int precision,
                                  unsigned flags) {
    Plan* p = new (std::nothrow) Plan();
    if (!p) {
        svdb_set_error("ragged plan: out of host memory");
        return nullptr;
    }
    p->metric = metric;
    p->precision = precision;
    p->graph_on = !(flags & SVDB_RAGGED_NO_GRAPH);
    int rc = SVDB_OK;
    auto fail = [&](int code) {
        (void)code;
        svdb::destroy(p);
        return (svdbd_ragged*)nullptr;
    };
    for (size_t i = 0; i < nparts; ++i) {
        Store* s = reinterpret_cast<Store*>(parts[i].store);
        rc = s->ensure();
        if (rc) return fail(rc);
        svdb::Part P;
        P.s = s;
        P.nq = parts[i].nq;
        P.stride = parts[i].stride;
        P.q = parts[i].d_queries;
        P.ids = parts[i].d_ids;
        P.dists = parts[i].d_dists;
        P.hk.assign(parts[i].k, parts[i].k + parts[i].nq);
        if (P.nq) {
            cudaError_t e = cudaMalloc(&P.d_k, P.nq * sizeof(uint32_t));
            if (e == cudaSuccess) e = cudaMemcpy(P.d_k, P.hk.data(), P.nq * sizeof(uint32_t), cudaMemcpyHostToDevice);
            if (e != cudaSuccess) {
                cudaGetLastError();
                svdb_set_error("ragged plan: cannot allocate per-query k: %s", cudaGetErrorString(e));
                p->parts.push_back(P);
                return fail(SVDB_ENOMEM);
            }
        }
        p->parts.push_back(P);
        if (std::find(p->stores.begin(), p->stores.end(), s) == p->stores.end()) p->stores.push_back(s);
    }
    // stores with more work first: in the one-after-another order the longest
    // work starts first (rows x padded dimension x queries)
    {
        std::vector<std::pair<double, Store*>> w;
        for (Store* s : p->stores) {
            double q = 0;
            for (const svdb::Part& P : p->parts)
                if (P.s == s) q += (double)P.nq;
            w.push_back({-(double)s->slots * (double)s->ldb * q, s});
        }
        std::stable_sort(w.begin(), w.end(),
                         [](const std::pair<double, Store*>& a, const std::pair<double, Store*>& b) { return a.first < b.first; });
        for (size_t i = 0; i < w.size(); ++i) p->stores[i] = w[i].second;
    }
    cudaError_t e = cudaStreamCreateWithFlags(&p->origin, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->ev_done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreate(&p->ev_t0);
    if (e == cudaSuccess) e = cudaEventCreate(&p->ev_t1);
    for (size_t i = 0; i < p->stores.size() && e == cudaSuccess; ++i) {
        cudaEvent_t ev = nullptr;
        e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (e == cudaSuccess) p->ev_store.push_back(ev);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        svdb_set_error("ragged plan: cannot create streams/events: %s", cudaGetErrorString(e));
        return fail(SVDB_ECUDA);
    }
    for (Store* s : p->stores) {
        rc = s->sync();
        if (rc) return fail(rc);
    }
    p->sprec.assign(p->stores.size(), precision);
    if (flags & SVDB_RAGGED_SEED) p->seed = 1;
    rc = (flags & SVDB_RAGGED_AUTOTUNE)
             ? svdb::autotune(p)
             : svdb::configure(p, (flags & SVDB_RAGGED_BY_K_CLASS) ? 1 : 0, 1,
                               (flags & SVDB_RAGGED_FUSED) && precision != SVDB_PREC_FP64 ? 1 : 0);
    if (!rc && p->fused && !p->fp) rc = svdb::build_fused(p);  // ready for the first run (and reported)
    if (rc) return fail(rc);
    return reinterpret_cast<svdbd_ragged*>(p);
}

int svdbd_ragged_run(svdbd_ragged* hp) { return svdb::run(reinterpret_cast<Plan*>(hp)); }

int svdbd_ragged_wait(svdbd_ragged* hp) {
    Plan* p = reinterpret_cast<Plan*>(hp);
    SVDB_CUDA(cudaStreamSynchronize(p->origin));
    return svdb::check_stores(p);
}

void* svdbd_ragged_stream(svdbd_ragged* hp) { return reinterpret_cast<Plan*>(hp)->origin; }

int svdbd_ragged_info(svdbd_ragged* hp, svdb_ragged_info* out) {
    Plan* p = reinterpret_cast<Plan*>(hp);
    std::memset(out, 0, sizeof(*out));
    out->grouping = p->grouping;
    out->concurrent = p->concurrent;
    out->graph = p->graph_on ? 1 : 0;
    out->searches = (int32_t)p->groups.size();
    for (int i = 0; i < 4; ++i) out->tuned_ms[i] = p->tuned_ms[i];
    out->captures = p->captures;
    for (size_t i = 0; i < p->stores.size() && i < 32; ++i)
        if (p->sprec[i] == SVDB_PREC_FP8) out->fp8_stores |= 1u << i;
    for (int i = 0; i < 8; ++i) out->swap_ms[i] = p->swap_ms[i];
    out->fused = p->fused && p->fp ? 1 : 0;  // (a fused plan over no searches is no fused plan)
    out->fused_launches = p->fp ? (int32_t)svdb::fused_launches(p->fp) : 0;
    for (int i = 0; i < 2; ++i) out->fused_ms[i] = p->fused_ms[i];
    for (int i = 0; i < 3; ++i) out->weight_ms[i] = p->weight_ms[i];
    out->epi_weight = (float)p->epi_weight;
    out->seeded = p->seed > 0 ? 1 : 0;
    out->seed_ms = p->seed_ms;
    return SVDB_OK;
}

// per search of the last run: {part, k, queries, fused, candidates, survivors,
// re-ranked, widened, bound failures, widened by candidate / survivor /
// re-rank overflow}; the counters are those of fused searches (0 otherwise)
int svdbd_ragged_search_stats(svdbd_ragged* hp, uint64_t* out, size_t n) {
    Plan* p = reinterpret_cast<Plan*>(hp);
    SVDB_CUDA(cudaStreamSynchronize(p->origin));
    for (size_t i = 0; i < n && i < p->groups.size(); ++i) {
        const svdb::Group& g = p->groups[i];
        uint64_t* o = out + i * 12;
        std::memset(o, 0, 12 * sizeof(uint64_t));
        o[0] = (uint64_t)g.part;
        o[1] = (uint64_t)g.kg;
        o[2] = (uint64_t)g.n;
        if (p->fused && p->fp && g.fidx >= 0) {
            o[3] = 1;
            unsigned long long st[8];
            int rc = svdb::fused_stats(p->fp, (size_t)g.fidx, st);
            if (rc) return rc;
            for (int t = 0; t < 8; ++t) o[4 + t] = st[t];
        }
    }
    return SVDB_OK;
}

void svdbd_ragged_destroy(svdbd_ragged* hp) {
    if (hp) svdb::destroy(reinterpret_cast<Plan*>(hp));
}

}  // extern "C"
