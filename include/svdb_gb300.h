/*
 * svdb_gb300.h -- batch entry points of libsvdb_gb300.so (additive to the
 * drop-in vector_database.h / kdtree.h API).
 *
 * The reference answers one /compare pair or one /nearest query per HTTP
 * request.  These calls take whole batches so a server (or a batching
 * front end) can amortise one kernel launch over many requests.  Each
 * entry cites the reference code path whose semantics it keeps.
 *
 * Conventions: plain pointers and sizes, no CUDA or torch types.  Unless a
 * name ends in _device, every buffer is HOST memory and the call returns
 * when the results are in it.  Return value: SVDB_OK or a negative SVDB_E*
 * code; svdb_last_error() gives a message for the calling thread.
 */
#ifndef SVDB_GB300_H
#define SVDB_GB300_H

#include <stddef.h>
#include <stdint.h>

#include "vector_database.h"

#ifdef __cplusplus
extern "C" {
#endif

/* metrics: the three /compare/<metric> URLs (src/compare_handler.c:152-160) */
#define SVDB_COSINE 0
#define SVDB_EUCLIDEAN 1
#define SVDB_DOT 2

/* search precision */
#define SVDB_PREC_FP64 0 /* plain FP64 streaming scan of the master copy */
#define SVDB_PREC_BF16 1 /* BF16 tensor-core screen + certified FP64 re-rank */
#define SVDB_PREC_FP8 2  /* cosine: FP8-E4M3 tensor-core screen on the unit-norm shadow (256 x/|x|, an exact
                            power-of-two scale per query), its thresholds seeded (batches of 32+ queries) by
                            the BF16 screen of a 1/16 row sample, then the same certified refinement and
                            FP64 re-rank; dot / Euclidean searches run the BF16 screen */

/* return codes */
#define SVDB_OK 0
#define SVDB_EINVAL (-1)   /* bad argument (NULL pointer, k == 0, dimension mismatch) */
#define SVDB_ENOMEM (-2)   /* host/device allocation failed or admission refused */
#define SVDB_ECUDA (-3)    /* a CUDA call failed (message in svdb_last_error) */
#define SVDB_ETIMEOUT (-4) /* a kernel's bounded wait ran out; the context is still usable */
#define SVDB_ENODEV (-5)   /* no usable GPU */

/* per-pair status of svdb_compare_batch: the error branches of
 * compare_handler_callback (src/compare_handler.c:74-195), in its order */
#define SVDB_CMP_OK 0
#define SVDB_CMP_OUT_OF_BOUNDS 1  /* "Index out of bounds", 400 (:101-110) */
#define SVDB_CMP_NOT_FOUND 2      /* "Vector not found", 404 (:116-125) */
#define SVDB_CMP_DIFF_DIM 3       /* "Vectors have different dimensions", 400 (:127-136) */
#define SVDB_CMP_SIZE_MISMATCH 4  /* "Vector size mismatch", 400 (:139-147) */
#define SVDB_CMP_UNKNOWN_METHOD 5 /* "Unknown comparison method", 400 (:161-170) */

typedef struct svdb_search_stats {
    uint64_t candidates;     /* rows the BF16 screen emitted, over the batch (FP64 scan: rows scanned) */
    uint64_t survivors;      /* rows left after the exact k-th lower-bound filter of the screen */
    uint64_t reranked;       /* rows scored in FP64 against the master copy (after FP32 refinement) */
    uint32_t widened;        /* queries the screen could not certify, answered by the exact FP64 scan */
    uint32_t kernels;        /* kernel launches issued by the call */
    uint32_t bound_failures; /* queries whose screen bound did not hold against the exact value
                                (re-answered by the exact scan; nonzero means the bound model is wrong) */
    uint32_t reserved;
    double max_err_bound;    /* max over results of the bound on |reported - exact real value| */
} svdb_search_stats;

/*
 * GET /compare/<metric>?index1=&index2= for npairs pairs at once
 * (src/compare_handler.c:74-195).  out[i] is bit-identical to the reference's
 * float result; status[i] is SVDB_CMP_*.  expected_dim is the server's
 * db_vector_size (0 skips that check).  metric outside 0..2 gives
 * SVDB_CMP_UNKNOWN_METHOD for every pair.
 */
int svdb_compare_batch(VectorDatabase* db, int metric, const int64_t* index1, const int64_t* index2,
                       size_t npairs, size_t expected_dim, float* out, int32_t* status);

/*
 * POST /nearest for nq queries (src/compare_handler.c:403 -> kdtree_nearest,
 * src/kdtree.c:171-178): out_index[i] is the KD tree's stored index, or -1
 * for "No nearest neighbor found".  queries is nq x dim, row-major; only the
 * first kd-dimension coordinates are read.
 */
int svdb_nearest_batch(VectorDatabase* db, const double* queries, size_t nq, size_t dim,
                       int64_t* out_index);

/*
 * Request bodies of POST /nearest decoded on the device, in batches: the
 * JSON text of nearest_handler_callback (src/compare_handler.c:300-390) --
 * an array of exactly dim numbers -- to the doubles cJSON gives the
 * reference (each number the correctly rounded value of the decimal strtod
 * accepts).  Body i is text[offsets[i] .. offsets[i+1]) (a NUL byte ends it
 * early, as cJSON_Parse reads a C string); out[i*dim + j] is its j-th
 * number (NaN when status[i] != SVDB_DEC_OK).  Statuses follow the handler's
 * checks in its order.  The grammar is cJSON's (published 1.7 sources; the
 * reference does not pin a version): any byte <= 32 is whitespace, a UTF-8
 * byte-order mark is skipped, content after the value is ignored, nesting up
 * to 1000, and the children of a top-level object count like an array's.
 */
#define SVDB_DEC_OK 0
#define SVDB_DEC_INVALID_JSON 1   /* 400 {"error": "Invalid JSON"} (:300-313) */
#define SVDB_DEC_SIZE_MISMATCH 2  /* 400 {"error": "Vector size mismatch"} (:318-341) */
#define SVDB_DEC_INVALID_DATA 3   /* 400 {"error": "Invalid vector data"} (:366-384): a child is not a number */
int svdb_decode_vectors(const char* text, const uint64_t* offsets, size_t n, size_t dim, double* out,
                        int32_t* status);

/*
 * POST /nearest over a MEDIAN-split KD tree (opt-in; README.md:3,34 describes
 * one, src/kdtree.c builds an insertion-order tree instead).  The tree holds
 * the store's current rows of the store's dimension, split on the first
 * kd-dimension coordinates, and is built on the device whenever the rows
 * changed since the last call.  out_index[i] is the position of the row
 * nearest to query i over those coordinates (the same unfused FP64 distance
 * as src/kdtree.c:134-137), ties to the lowest position; -1 for an empty
 * store.  It differs from svdb_nearest_batch (the reference's /nearest) in
 * two ways: no stale nodes from updates and deletes (src/vector_database.c:
 * 169-195), and ties to the lowest position instead of the first node
 * visited.
 */
int svdb_nearest_batch_median(VectorDatabase* db, const double* queries, size_t nq, size_t dim,
                              int64_t* out_index);

/*
 * Exact top-k (no reference counterpart: /nearest is top-1 and documents an
 * unimplemented `number` parameter, README.md:287).  For each of nq queries
 * (nq x dim, row-major), ids[i*k + j] is the logical index of the j-th
 * result and dists[i*k + j] its FP64 value (cosine similarity, Euclidean
 * distance or dot product, the reference's formulas carried in double);
 * order is best first, ties to the lowest index; missing results are
 * id -1 / NaN.  Ids are exact for both precisions.  err (optional, nq*k)
 * receives a bound on |dists - exact real value|.
 */
int svdb_search_topk(VectorDatabase* db, const double* queries, size_t nq, size_t dim, size_t k,
                     int metric, int precision, int64_t* ids, double* dists, double* err,
                     svdb_search_stats* stats);

/* As svdb_search_topk with queries/ids/dists/err in DEVICE memory; the work
 * is queued on the database's stream (svdb_stream) and the call returns
 * without waiting for it.  stats may be NULL. */
int svdb_search_topk_device(VectorDatabase* db, const double* d_queries, size_t nq, size_t dim, size_t k,
                            int metric, int precision, int64_t* d_ids, double* d_dists, double* d_err,
                            svdb_search_stats* stats);

/*
 * Exact FP64 top-k that allocates no device memory; no counterpart in the
 * reference.  For callers that cannot call cudaMalloc -- an allocator hook or
 * memory pool that owns every device byte, a latency-critical path that must
 * not take the driver's allocation lock, a host that has handed all free HBM
 * to another component.  Same results as svdb_search_topk_device with
 * SVDB_PREC_FP64 (ids, values, ties to the lowest index); queries, ids and
 * dists are DEVICE buffers the caller owns, the work is queued on
 * svdb_stream(db) and the call returns without waiting.
 *
 * The per-call scratch (padded queries, norms, partial top-k lists) lives in
 * one fixed 16 MiB device array that every GPU loading this library holds
 * until the process exits.  A call needs about 8 D bytes per query plus 16
 * bytes per (query, result, row slice), at most 592 slices (64 queries of
 * D = 768, top-32: about 3 MB); one that needs more is rejected with
 * SVDB_EINVAL and a message saying how much it needed.  The store must have no pending
 * mutations (call svdb_sync before; syncing can allocate).  The array's
 * device address is looked up when a database first sets up its device
 * store (its first sync), with that device current, which also loads the
 * array; a call looks it up again only if the device's context was created
 * anew since (after cudaDeviceReset).  The scan kernels' code is loaded by
 * the first search of any kind in the process (CUDA's lazy module loading),
 * which may allocate for that code: make one search call, of any kind, before
 * the phase that must not allocate and before any stream capture; every later
 * call allocates nothing.  Every call shares the array: calls
 * whose work overlaps on the GPU (other streams, other databases) race, so
 * order them.
 */
int svdb_search_topk_fp64_noalloc(VectorDatabase* db, const double* d_queries, size_t nq, size_t dim, size_t k,
                                  int metric, int64_t* d_ids, double* d_dists);

/* ---- ragged batches over several collections -----------------------------
 *
 * No reference counterpart (the reference serves one collection, one query
 * per request).  A plan binds one uneven batch of top-k queries over several
 * stores, possibly of different dimensions, each query with its own k; one
 * svdb_ragged_run answers all of it with one CUDA graph launch.  Per part:
 * the store, nq queries (DEVICE, nq x dim, row-major), the k of each query
 * (HOST, nq values in 1..128, read at creation), and DEVICE outputs of nq x
 * stride (stride >= every k of the part): ids[i*stride + j] and
 * dists[i*stride + j] are exactly what svdb_search_topk_device gives for
 * query i with its own k, and -1 / NaN for j >= that k.
 *
 * The buffers are bound at creation: a run reads the queries' current
 * contents and overwrites the outputs (creation itself runs the plan, several
 * times with SVDB_RAGGED_AUTOTUNE).  Stores may change between runs (pending
 * mutations are applied at the start of a run, and a change the captured
 * graph depends on makes the run capture it again).  A run is queued on
 * svdb_ragged_stream and returns without waiting; later calls on the same
 * stores are ordered after it.  Destroy a plan before its stores.
 */
typedef struct svdb_ragged_part {
    VectorDatabase* db;
    size_t nq;
    size_t dim;               /* must equal the store's dimension */
    const double* d_queries;  /* device, nq x dim */
    const uint32_t* k;        /* host, nq entries */
    int64_t* d_ids;           /* device, nq x stride */
    double* d_dists;          /* device, nq x stride */
    size_t stride;
} svdb_ragged_part;

#define SVDB_RAGGED_AUTOTUNE 1u /* time the execution choices on these inputs, keep the fastest (cosine plans:
                                   also each store's BF16 versus FP8 screen; the results are the same) */
#define SVDB_RAGGED_NO_GRAPH 2u /* enqueue the kernels directly at each run (no graph) */
#define SVDB_RAGGED_FUSED 4u    /* without AUTOTUNE: screen the BF16 searches with one fused launch per k class */
#define SVDB_RAGGED_BY_K_CLASS 8u /* without AUTOTUNE: one search per k class (else one per part) */
#define SVDB_RAGGED_SEED 16u    /* start every tensor-core screen's thresholds from a 1/16 sample of the store */

typedef struct svdb_ragged_info {
    int32_t grouping;   /* 0: one search per part with its largest k; 1: one per k class (<=16, <=32, <=128) */
    int32_t concurrent; /* 1: different stores' searches run at the same time; 0: one after another */
    int32_t graph;      /* 1: runs replay a captured CUDA graph */
    int32_t searches;   /* searches per run */
    float tuned_ms[4];   /* autotuner's ms per run of (grouping, concurrent) = (0,1) (1,1) (0,0) (1,0); 0: not tried */
    uint32_t captures;   /* graph captures so far */
    uint32_t fp8_stores; /* bit i: the plan's i-th distinct store (first-use order) runs the FP8 screen */
    float swap_ms[8];    /* cosine plans with a tensor-core precision: autotuner's ms per run with store i's
                            screen swapped BF16 <-> FP8 (kept when faster); 0: not tried */
    int32_t fused;          /* 1: the BF16 searches' screens run as fused launches (one per k class) */
    int32_t fused_launches; /* fused screen launches per run */
    float fused_ms[2];      /* autotuner's ms per run with fused screens, grouping 0 / 1; 0: not tried */
    float weight_ms[3];     /* autotuner's ms per run with the fused schedule's epilogue weight 1 / 4 / 8 */
    float epi_weight;       /* the fused schedule's epilogue weight in use (k blocks per tile) */
    int32_t seeded;         /* 1: screens start from thresholds seeded by a sample of the store */
    float seed_ms;          /* autotuner's ms per run with seeded thresholds; 0: not tried */
} svdb_ragged_info;

typedef struct svdb_ragged svdb_ragged;
/* NULL on failure (message in svdb_last_error) */
svdb_ragged* svdb_ragged_create(const svdb_ragged_part* parts, size_t nparts, int metric, int precision,
                                unsigned flags);
int svdb_ragged_run(svdb_ragged* plan);
/* block until the plan's last run is done; SVDB_ETIMEOUT if a kernel's bounded wait ran out */
int svdb_ragged_wait(svdb_ragged* plan);
/* the CUDA stream (cudaStream_t) runs are queued on */
void* svdb_ragged_stream(svdb_ragged* plan);
int svdb_ragged_get_info(svdb_ragged* plan, svdb_ragged_info* info);
/* Per search of the plan's last run (info.searches of them), 12 values each:
 * part, k, queries, fused (1: screened by a fused launch), then for fused
 * searches candidates, survivors, re-ranked (over the search's queries),
 * queries answered by the exact scan, bound failures, and of those queries
 * how many overflowed the candidate lists, the survivor cap, the FP64
 * re-rank (0 for searches with a screen of their own).  Waits for the run. */
int svdb_ragged_get_search_stats(svdb_ragged* plan, uint64_t* out, size_t n);
void svdb_ragged_destroy(svdb_ragged* plan);

/* ---- serving: batches of mixed requests on a device-resident store -------
 *
 * A server store keeps its rows only in HBM (no host copies, no KD tree): the
 * request path of a server that batches requests as they arrive.  Positional
 * semantics are the reference's: rows are numbered 0..size-1 in insertion
 * order, an insert appends (src/vector_database.c:99-125), an update
 * overwrites in place (:160-175) and a delete shifts every later row down by
 * one (:185-195).  Deleted rows become tombstones in the device store and an
 * order-statistic tree maps positions to slots, so no mutation moves rows.
 *
 * svdb_server_execute runs one batch: every INSERT / UPDATE / DELETE in
 * request order first, then every NEAREST and COMPARE against the resulting
 * state -- one serial order of requests that were all waiting at the same
 * time.  NEARESTs with the same (metric, k) share one top-k search and
 * COMPAREs with the same metric one pair kernel.
 */
#define SVDB_REQ_NEAREST 0 /* exact top-k of vec (POST /nearest?number=k, README.md:287) */
#define SVDB_REQ_COMPARE 1 /* metric of rows a and b (GET /compare/..., src/compare_handler.c:86-170) */
#define SVDB_REQ_INSERT 2  /* append vec (POST /vector, src/post_handler.c:333) */
#define SVDB_REQ_UPDATE 3  /* overwrite row a with vec (PUT /vector, src/put_handler.c:155,247) */
#define SVDB_REQ_DELETE 4  /* delete row a (DELETE /vector, src/delete_handler.c:84,96) */
#define SVDB_REQ_KD_NEAREST 5 /* POST /nearest as the reference answers it: kdtree_nearest over the first
                                 kd_dim coordinates of vec (src/compare_handler.c:403); device loop only */

typedef struct svdb_request {
    int32_t op;        /* SVDB_REQ_* */
    int32_t metric;    /* NEAREST, COMPARE: SVDB_COSINE / SVDB_EUCLIDEAN / SVDB_DOT */
    uint32_t k;        /* NEAREST: 1..128 */
    uint32_t reserved; /* 0 */
    uint64_t a, b;     /* COMPARE: positions of the two rows; UPDATE, DELETE: a */
    const double* vec; /* NEAREST, INSERT, UPDATE: dim doubles in host memory */
    const char* uuid;  /* INSERT: the row's uuid (NULL: ""); UPDATE: its new uuid (NULL: unchanged);
                          a C string of which the first 37 bytes count, as char uuid[37] stores it */
} svdb_request;

typedef struct svdb_response {
    int32_t status; /* 0; SVDB_CMP_OUT_OF_BOUNDS (COMPARE, UPDATE, DELETE past the end);
                       SVDB_CMP_UNKNOWN_METHOD; SVDB_ENOMEM (INSERT refused: no HBM left);
                       SVDB_EINVAL (bad op, k or vec) */
    float value;    /* COMPARE: the reference's float metric */
    uint64_t index; /* INSERT: position of the new row */
} svdb_response;

typedef struct svdb_server svdb_server;

/* A server store of dimension dim with room for reserve_rows rows allocated
 * up front; NULL (message in svdb_last_error) when that does not fit in the
 * device's free memory. */
svdb_server* svdb_server_create(size_t dim, size_t reserve_rows);
void svdb_server_destroy(svdb_server* s);
size_t svdb_server_size(svdb_server* s);
/* bulk load: append n rows (n x dim, row-major); *first_index = position of the first */
int svdb_server_insert_block(svdb_server* s, const double* rows, size_t n, size_t* first_index);
/* bulk load with uuids: uuids is n x 37 bytes (char uuid[37] per row) or NULL */
int svdb_server_insert_rows(svdb_server* s, const double* rows, const char* uuids, size_t n, size_t* first_index);
/* GET /vector?index= (src/get_handler.c:88-101): copy row `index` to out[dim] */
int svdb_server_read(svdb_server* s, size_t index, double* out);
/* GET /vector?uuid= (src/get_handler.c:99-118, src/vector_database.c:145-158)
 * for n uuids (n x 37 bytes): out_index[i] = position of the first row whose
 * uuid equals uuid i under strncmp(.., 37), -1 if none.  Answered by the
 * device's uuid index. */
int svdb_server_find_uuid(svdb_server* s, const char* uuids, size_t n, int64_t* out_index);
/* vector_db_save's file format (src/vector_database.c:203-228): size_t n, then
 * per row uuid[37], size_t dim, double[dim], rows in positional order, read
 * back from HBM in blocks.  The reference counts rows it then skips (rows
 * without data); a server store has none, so n is always the rows written. */
int svdb_server_save(svdb_server* s, const char* filename);
/* A server store of dimension dim loaded from a file in that format
 * (vector_db_load, src/vector_database.c:237-292): the file's bytes are copied
 * to the device as they are, in blocks, and unpacked there into the FP64 rows
 * and the uuid index.  Every row must have dimension dim; a file that ends
 * early keeps the rows before the cut (message on stderr), as the drop-in
 * vector_db_load does.  reserve_rows: extra room beyond the file's rows.
 * NULL on failure (message in svdb_last_error). */
svdb_server* svdb_server_load(const char* filename, size_t dim, size_t reserve_rows);
/* One batch (see above).  NEAREST results of request i go to ids/dists +
 * i * stride (stride >= its k; -1 / NaN past the number of rows).  The
 * return value is SVDB_OK unless the batch as a whole failed (a CUDA error);
 * per-request outcomes are in resp[i].status.  stats (optional) adds up the
 * searches' statistics. */
int svdb_server_execute(svdb_server* s, const svdb_request* req, size_t n, svdb_response* resp, int precision,
                        int64_t* ids, double* dists, size_t stride, svdb_search_stats* stats);

/*
 * Health check of the kernels' failure path (no reference counterpart).  Runs
 * one CTA of the screen's bounded-wait sequence on mbarriers that nothing
 * arrives on: one role gives up after limit_us microseconds (1 .. 10^6), the
 * other role, holding tensor memory, leaves through the shared abort flag,
 * the tensor memory is released and the store's error word is raised.  A
 * working path returns SVDB_ETIMEOUT with *gave_up == 3 (both roles left
 * their waits) and leaves the GPU context and the store usable; any other
 * result means a search could not report a stalled pipeline.  Synchronous.
 */
int svdb_selftest_bounded_wait(VectorDatabase* db, uint32_t limit_us, uint32_t* gave_up);

/*
 * The request path as a device-side loop (no reference counterpart; it
 * replaces the reference's thread-per-connection handlers, src/main.c:381,
 * for /compare, POST /nearest and /vector).  One persistent kernel owns a
 * store and serves requests as they arrive: host threads put requests into a
 * ring in page-locked host memory mapped into the device (svdb_loop_submit
 * makes no CUDA call), the kernel polls it, takes every request already there
 * as one batch and answers it in ticket order -- a run of /compare and
 * /nearest requests in parallel, each insert / update / delete applied in
 * place before the next request -- with the reference's results and
 * positional semantics: SVDB_REQ_COMPARE (metric of positions a, b; the
 * reference's float), SVDB_REQ_KD_NEAREST (response.index = the stored index
 * kdtree_nearest returns over the insertion-order KD tree, (size_t)-1 when
 * empty; stale after deletes, as in the reference), SVDB_REQ_INSERT (index =
 * the new row's position; a KD node), SVDB_REQ_UPDATE (a second KD node),
 * SVDB_REQ_DELETE (later positions shift down; the KD tree is untouched).
 * Positions past the end get SVDB_CMP_OUT_OF_BOUNDS, an unknown metric
 * SVDB_CMP_UNKNOWN_METHOD, SVDB_REQ_NEAREST (top-k) SVDB_EINVAL (served by
 * svdb_server_execute).  Admission by HBM: capacity rows and kd_capacity KD
 * nodes are allocated at creation (NULL if they do not fit); an insert (or an
 * update's KD node) beyond them is answered SVDB_ENOMEM.  Every wait is
 * bounded: the kernel returns after idle_us with no request
 * (SVDB_LOOP_LEFT_IDLE) and sees svdb_loop_stop at every poll; svdb_loop_wait
 * starts it again when it is not running.  Every submitted ticket must be
 * waited for: its ring slot is reused only after its answer was taken.
 */
typedef struct svdb_loop svdb_loop;
typedef struct svdb_loop_config {
    size_t dim;          /* row dimension */
    size_t kd_dim;       /* the KD prefix (the server's kd_tree_dimension), 1..32, <= dim */
    size_t capacity;     /* rows the store may hold (>= the initial rows) */
    size_t kd_capacity;  /* KD nodes (inserts + updates add one each); 0: 2 x capacity */
    size_t ring;         /* requests in flight (rounded up to a power of two); 0: 4096 */
    uint32_t max_batch;  /* requests answered per pass, 1..256; 0: 256 */
    uint32_t idle_us;    /* the kernel returns after this long with nothing to do; 0: 1 s */
} svdb_loop_config;

#define SVDB_LOOP_NOT_STARTED 0
#define SVDB_LOOP_RUNNING 1
#define SVDB_LOOP_LEFT_IDLE 2
#define SVDB_LOOP_STOPPED 3
#define SVDB_LOOP_LEAVING 4
typedef struct svdb_loop_info {
    uint32_t state;       /* SVDB_LOOP_* */
    uint32_t reserved;
    uint64_t size;        /* rows after the last batch */
    uint64_t answered;    /* tickets answered */
    uint64_t batches;     /* batches served */
    uint64_t idle_exits;  /* launches that ended for want of requests */
} svdb_loop_info;

/* rows: n x dim initial rows (positions 0..n-1, KD tree built in that order);
 * uuids37: n x 37 bytes or NULL */
svdb_loop* svdb_loop_create(const svdb_loop_config* cfg, const double* rows, size_t n, const char* uuids37);
int svdb_loop_start(svdb_loop* l);
/* req->vec: dim doubles (INSERT, UPDATE, KD_NEAREST); req->uuid as for the server store */
int svdb_loop_submit(svdb_loop* l, const svdb_request* req, uint64_t* ticket);
/* spins until the ticket is answered (timeout_us: SVDB_ETIMEOUT) */
int svdb_loop_wait(svdb_loop* l, uint64_t ticket, svdb_response* resp, uint32_t timeout_us);
int svdb_loop_stop(svdb_loop* l);
int svdb_loop_get_info(svdb_loop* l, svdb_loop_info* out);
/* a row (dim doubles) and its uuid (37 bytes, may be NULL) by position; the loop must not be running */
int svdb_loop_read(svdb_loop* l, size_t position, double* row, char* uuid37);
void svdb_loop_destroy(svdb_loop* l);

/*
 * Response bodies printed on the GPU, as the reference's handlers print them
 * (replaces cJSON_PrintUnformatted of the objects built at
 * src/compare_handler.c:180-185 for GET /compare and :409-424 for POST
 * /nearest; cJSON is not vendored, its published number rule is restated:
 * "null" for NaN or an infinity, the decimal integer when the value equals
 * its int conversion, else printf's "%1.15g" when strtod of it is within
 * DBL_EPSILON (relative) of the value, else "%1.17g"; digits exact, ties to
 * even, as printf).  n texts are packed into out (cap bytes) with
 * offsets[0..n] (offsets[i+1] - offsets[i] bytes each, no NUL); out == NULL
 * only fills the offsets (the size to allocate).  SVDB_EINVAL when cap is too
 * small (offsets are still filled).  Synchronous.
 *
 * svdb_format_compare: metric (0..2) and float result per answer, status
 * SVDB_CMP_* (a nonzero status prints the handler's fixed error body,
 * src/compare_handler.c:103-163).
 * svdb_format_nearest: index[i] as kdtree_nearest returned it (-1 for
 * (size_t)-1): {"index":i,"vector":[...],"uuid":"..."} with the stored row,
 * {"error":"No nearest neighbor found"} for -1, {"error":"Nearest neighbor
 * not found"} for an index past the end (a KD node left by a delete).
 */
int svdb_format_compare(const int32_t* metric, const float* value, const int32_t* status, size_t n, char* out,
                        size_t cap, uint64_t* offsets);
int svdb_format_nearest(VectorDatabase* db, const int64_t* index, size_t n, char* out, size_t cap,
                        uint64_t* offsets);

/*
 * vector_db_save with options (replaces reference src/vector_database.c:203-223
 * when flags ask for a change).  The reference writes db->size as the row
 * count and then skips rows without data (dimension 0 or NULL data), so a
 * store holding such rows produces a file that promises more rows than it
 * holds; loading it reads past the last row.  vector_db_save keeps that
 * behaviour byte for byte.  SVDB_SAVE_EXACT_COUNT writes the number of rows
 * actually written instead (opt-in: the rows and their bytes are unchanged).
 * Returns SVDB_OK or SVDB_EINVAL (bad argument, file not writable).
 */
#define SVDB_SAVE_EXACT_COUNT 1u
int svdb_save(VectorDatabase* db, const char* filename, unsigned flags);

/*
 * Diagnostics of the screen's certification (no reference counterpart; not a
 * search).  The exact top-k rests on a bound of the tensor core's FP32
 * accumulation error, |acc - sum(bq_i bx_i)| <= c_acc |bq| |bx|, whose
 * internal order the hardware does not document.  This runs the screen
 * kernel itself, in a form whose epilogue stores instead of screens, for nq
 * (1..256; more than 128 run the paired two-SM form) host queries against
 * the store's first `rows` slots (synced
 * first) and returns every raw FP32 accumulator (acc: nq x rows), the query
 * operands the MMAs read (query_ops: nq x *op_bytes; may be NULL) and the
 * rows' shadow operands (row_ops: rows x *op_bytes, un-swizzled; may be
 * NULL).  precision SVDB_PREC_BF16: BF16 operands (cosine: the unit-norm
 * shadow; dot / Euclidean: the plain shadow); SVDB_PREC_FP8: E4M3 operands
 * (the query scaled by its power of two).  *op_bytes = 2 ldb (BF16) or ldb8
 * bytes.  Synchronous; uses the store's scratch.
 */
int svdb_debug_screen_accumulators(VectorDatabase* db, const double* queries, size_t nq, size_t dim, int metric,
                                   int precision, size_t rows, float* acc, void* query_ops, void* row_ops,
                                   size_t* op_bytes);

/*
 * Merge of per-shard top-k lists (host only, no GPU; no reference
 * counterpart).  A store split by row ranges over several GPUs or processes
 * answers a query with one exact top-k per shard; this combines nshards such
 * lists (ids already global, layout [shard][query][k]) into the exact global
 * top-k: order by value (Euclidean ascending, cosine / dot descending, NaN
 * last), ties to the lowest global id; missing entries are id -1 / NaN.
 */
int svdb_merge_topk(int metric, const int64_t* ids, const double* vals, size_t nshards, size_t nq, size_t k,
                    int64_t* out_ids, double* out_vals);

/* GET /vector?uuid= for n uuids (n x 37 bytes) on the drop-in store
 * (src/vector_database.c:145-158, src/get_handler.c:99-118): out_index[i] =
 * position of the first row whose uuid equals uuid i under strncmp(.., 37),
 * -1 if none.  vector_db_read_by_uuid is this with n = 1.  Answered by the
 * device's uuid index (a hash table of the stored uuids); no row is scanned. */
int svdb_find_uuid_batch(VectorDatabase* db, const char* uuids, size_t n, int64_t* out_index);

/* Bulk insert of n rows (n x dim, row-major, copied): the same result as n
 * vector_db_insert calls, including the KD nodes.  uuids: n*37 bytes or
 * NULL.  Returns the first new index in *first_index. */
int svdb_insert_batch(VectorDatabase* db, const double* rows, size_t n, size_t dim, const char* uuids,
                      size_t* first_index);

/* Reserve device capacity for `rows` rows of dimension `dim` (avoids
 * regrowth copies).  Refused with SVDB_ENOMEM when free HBM minus the
 * configured headroom is too small (admission by free memory). */
int svdb_reserve(VectorDatabase* db, size_t rows, size_t dim);

/* Push pending host-side mutations to the device and rebuild derived
 * arrays (norms, BF16 shadow, logical index map).  Searches do this
 * implicitly. */
int svdb_sync(VectorDatabase* db);

/* Stage timing.  With profiling on, every search records CUDA events on the
 * database's stream around its stages; svdb_profile_read adds up the device
 * time of each stage over the searches since the last reset (ms[i] for stage
 * i) and returns how many searches that covers, or a negative code. */
#define SVDB_STAGE_PREP 0   /* query upload + padding + norms */
#define SVDB_STAGE_SCREEN 1 /* FP64 streaming scan, or the BF16 tensor-core GEMM screen */
#define SVDB_STAGE_SELECT 2 /* top-k merge, or exact k-th lower-bound shortlist selection */
#define SVDB_STAGE_REFINE 3 /* FP32 refinement of the shortlist (BF16 precision only) */
#define SVDB_STAGE_RERANK 4 /* FP64 re-rank of what the refinement keeps (BF16 precision only) */
#define SVDB_NSTAGES 5
int svdb_profile(VectorDatabase* db, int enable);
int svdb_profile_read(VectorDatabase* db, double* ms, int reset);

/* Threshold seeding of the tensor-core screens (SVDB_PREC_BF16 / FP8): the
 * screen's running thresholds start from the exact k-th best lower bound
 * over a 1/16 sample of the rows (one extra screen of the sample and its
 * select).  Results are the same either way; the speed depends on the data:
 * rows without clusters searched for a large k emit many times k candidates
 * before unseeded thresholds settle.  mode -1: the default (FP8 screens
 * only), 0: never, 1: always (on stores of at least 32 tiles of 256 rows,
 * batches of at least 32 queries). */
int svdb_set_screen_seeding(VectorDatabase* db, int mode);

/* Which screen an SVDB_PREC_FP8 search runs (the results are the same: both
 * screens are certified and followed by the same exact refinement).  mode
 * -1: the default rule -- the E4M3 screen for batches of at least 1,024
 * queries with k <= 32, where it was measured to be the faster one (its
 * seed sample of 1/16 of the rows settles the looser E4M3 thresholds), the
 * BF16 screen otherwise; 0: always the BF16 screen; 1: always the E4M3
 * screen. */
int svdb_set_fp8_screen(VectorDatabase* db, int mode);

/* The CUDA stream (cudaStream_t) the database's kernels run on. */
void* svdb_stream(VectorDatabase* db);

/* Block until the database's queued device work is done. */
int svdb_wait(VectorDatabase* db);

/* Message for the last failing call on this thread ("" if none). */
const char* svdb_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* SVDB_GB300_H */
