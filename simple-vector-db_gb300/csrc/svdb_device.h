/*
 * svdb_device.h -- the thin C ABI between the C host layer (store, KD-tree
 * bookkeeping, request validation) and the CUDA layer (device-resident
 * store, kernels).  Private to libsvdb_gb300.so: plain pointers and sizes,
 * no CUDA types, every call returns SVDB_OK or a negative SVDB_E* code and
 * records a message with svdb_set_error().
 *
 * Row addressing: the device store keeps rows in PHYSICAL slots that never
 * move (append, overwrite in place, tombstone on delete).  The reference's
 * positional index (src/vector_database.c:185-195 shifts rows left on
 * delete) is the rank of a slot among live slots; the host keeps
 * logical->slot, the device derives slot->logical at sync time.
 */
#ifndef SVDB_DEVICE_H
#define SVDB_DEVICE_H

#include <stddef.h>
#include <stdint.h>

#include "../../include/svdb_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define SVDB_API __attribute__((visibility("default")))
#else
#define SVDB_API
#endif

typedef struct svdbd_store svdbd_store;
typedef struct svdbd_kd svdbd_kd;

/* thread-local error message */
void svdb_set_error(const char* fmt, ...);

/* ---- device store -------------------------------------------------------- */
svdbd_store* svdbd_store_create(size_t dim);
void svdbd_store_destroy(svdbd_store* s);
void* svdbd_store_stream(svdbd_store* s);
size_t svdbd_store_dim(const svdbd_store* s);
size_t svdbd_store_slots(const svdbd_store* s);
int svdbd_store_reserve(svdbd_store* s, size_t rows);
/* append n rows; rows[i] are host pointers to dim doubles.  live[i] (or 1
 * when live is NULL): 1 = searchable row, 2 = placeholder for a row of
 * another dimension (kept in the positional order, never searched; also
 * used when rows[i] is NULL).  overwrite takes the same flag; kill marks a
 * slot deleted (0). */
int svdbd_store_append(svdbd_store* s, const double* const* rows, const uint8_t* live, size_t n);
/* append n rows from one contiguous host block (n x dim) */
int svdbd_store_append_block(svdbd_store* s, const double* rows, size_t n);
int svdbd_store_overwrite(svdbd_store* s, int64_t slot, const double* row, int live);
int svdbd_store_kill(svdbd_store* s, int64_t slot);
/* copy one row (device or still staged) to host memory */
int svdbd_store_read_row(svdbd_store* s, int64_t slot, double* out);
/* flush staged mutations, rebuild derived arrays and the slot->logical map */
int svdbd_store_sync(svdbd_store* s);
int svdbd_store_wait(svdbd_store* s);
/* stage timing (svdb_profile / svdb_profile_read) */
int svdbd_store_profile(svdbd_store* s, int enable);
int svdbd_store_set_seeding(svdbd_store* s, int mode);
int svdbd_store_set_fp8(svdbd_store* s, int mode);
int svdbd_store_profile_read(svdbd_store* s, double* ms, int reset);

/* reference-exact /compare for n slot pairs (host arrays in/out) */
int svdbd_compare_slots(svdbd_store* s, int metric, const int64_t* slot1, const int64_t* slot2, size_t n,
                        float* out);
/* the same with a metric per pair (combined drop-in metric calls) */
int svdbd_compare_slots_mixed(svdbd_store* s, const int32_t* metric, const int64_t* slot1, const int64_t* slot2,
                              size_t n, float* out);
/* reference-exact metric of two host vectors (the drop-in cosine_similarity
 * etc. take Vectors that need not be stored rows); the batch form packs n
 * pairs of any dimensions into one copy and one launch */
int svdbd_compare_vectors(int metric, const double* a, const double* b, size_t d, float* out);
int svdbd_compare_vectors_batch(const int32_t* metric, const double* const* a, const double* const* b,
                                const size_t* d, size_t n, float* out);

/* exact top-k; q/ids/dists/err in host memory unless on_device */
int svdbd_search(svdbd_store* s, const double* q, size_t nq, size_t k, int metric, int precision,
                 int64_t* ids, double* dists, double* err, int on_device, svdb_search_stats* st);

/* exact FP64 top-k with every per-call scratch byte in a fixed device array
 * (dev_noalloc.cu); q/ids/dists in device memory; never allocates */
int svdbd_selftest_wait(svdbd_store* s, uint32_t limit_us, uint32_t* gave_up);
int svdbd_search_noalloc(svdbd_store* s, const double* d_queries, size_t nq, size_t k, int metric, int64_t* d_ids,
                         double* d_dists);

/* diagnostics: the screen's raw FP32 accumulators for nq <= 128 host queries
 * against the first `rows` slots, with the query and row operands the MMAs
 * read (opbytes per row; row operands un-swizzled); f8: the E4M3 cosine
 * operands (dev_gemm.cu) */
int svdbd_debug_screen_acc(svdbd_store* s, const double* q, size_t nq, int metric, int f8, size_t rows, float* acc,
                           void* qops, void* rops, size_t* opbytes);

/* uuid of a slot (char[37] as the reference stores it; staged, applied at
 * sync), batched lookup of positions by uuid (-1: none), rows of the
 * reference's file format appended straight into the device store, and a
 * block of slots read back (dev_uuid.cu) */
int svdbd_store_set_uuid(svdbd_store* s, int64_t slot, const char* uuid37);
int svdbd_uuid_find(svdbd_store* s, const char* uuids37, size_t n, int64_t* out_pos);
int svdbd_store_append_raw(svdbd_store* s, const void* rows, size_t n, size_t rowbytes);
int svdbd_store_read_block(svdbd_store* s, int64_t first, size_t n, double* rows, char* uuids37, uint8_t* live);

/* exact 1-NN over the first kdim coordinates by a median-split KD tree of the
 * store's searchable rows, built on the device when the rows changed
 * (dev_kdm.cu); q: nq host rows of qstride doubles; out: positions (-1: none) */
int svdbd_kdm_nearest(svdbd_store* s, size_t kdim, const double* q, size_t nq, size_t qstride, int64_t* out_pos);

/* POST /nearest bodies decoded on the device (dev_decode.cu): n bodies at
 * text[off[i] .. off[i+1]) -> n x dim doubles and a SVDB_DEC_* status each */
int svdbd_decode_bodies(const char* text, const uint64_t* off, size_t n, size_t dim, double* out, int32_t* status);

/* response bodies printed on the device as cJSON_PrintUnformatted writes them
 * (dev_decode.cu): n texts packed into out (cap bytes) at offsets[0..n];
 * out == NULL fills only the offsets.  /nearest: kind 1 a row (slot >= 0 in
 * the store, else host_rows[i]; dims[i] numbers), 0 no neighbour, -1 an index
 * that reads no row; hs NULL when the store has no device rows. */
int svdbd_format_compare(const int32_t* metric, const float* value, const int32_t* status, size_t n, char* out,
                         size_t cap, uint64_t* offsets);
int svdbd_format_nearest(svdbd_store* hs, size_t n, const int32_t* kind, const uint64_t* index, const int64_t* slot,
                         const uint32_t* dims, const double* const* host_rows, const char* uuids37, char* out,
                         size_t cap, uint64_t* offsets);

/* the device-side request loop (dev_loop.cu); the initial KD tree comes
 * built (flat arrays, knodes nodes, height = nodes on the longest path) */
typedef struct svdbd_loop svdbd_loop;
svdbd_loop* svdbd_loop_create(const svdb_loop_config* cfg, const double* rows, size_t n, const char* uuids37,
                              const double* kpts, const int64_t* kidx, const int32_t* kleft, const int32_t* kright,
                              size_t knodes, int kheight);
int svdbd_loop_start(svdbd_loop* l);
int svdbd_loop_submit(svdbd_loop* l, const svdb_request* req, size_t dim, uint64_t* ticket, uint32_t timeout_us);
int svdbd_loop_wait(svdbd_loop* l, uint64_t ticket, svdb_response* out, uint32_t timeout_us);
int svdbd_loop_stop(svdbd_loop* l);
int svdbd_loop_info(svdbd_loop* l, svdb_loop_info* out);
int svdbd_loop_read(svdbd_loop* l, size_t position, double* row, char* uuid37);
void svdbd_loop_destroy(svdbd_loop* l);

/* ragged batch over several stores, replayed as one CUDA graph (dev_ragged.cu) */
typedef struct svdbd_ragged svdbd_ragged;
typedef struct svdbd_ragged_part {
    svdbd_store* store;
    size_t nq, stride;
    const double* d_queries; /* nq x dim, device */
    const uint32_t* k;       /* host, nq entries (1..128) */
    int64_t* d_ids;          /* nq x stride, device */
    double* d_dists;
} svdbd_ragged_part;
svdbd_ragged* svdbd_ragged_create(const svdbd_ragged_part* parts, size_t nparts, int metric, int precision,
                                  unsigned flags);
int svdbd_ragged_run(svdbd_ragged* p);
int svdbd_ragged_wait(svdbd_ragged* p);
void* svdbd_ragged_stream(svdbd_ragged* p);
int svdbd_ragged_info(svdbd_ragged* p, svdb_ragged_info* out);
int svdbd_ragged_search_stats(svdbd_ragged* p, uint64_t* out, size_t n);
void svdbd_ragged_destroy(svdbd_ragged* p);

/* ---- KD tree mirror ------------------------------------------------------ */
svdbd_kd* svdbd_kd_create(size_t kdim);
void svdbd_kd_destroy(svdbd_kd* t);
/* mirror nodes [synced, n) and apply parent-link patches for nodes < synced */
int svdbd_kd_sync(svdbd_kd* t, const double* pts, const int64_t* index, const int32_t* left,
                  const int32_t* right, size_t n, size_t synced, const int32_t* patch_nodes, size_t npatch,
                  int height);
/* nq queries (host, row stride qstride doubles); out: stored index or -1 */
int svdbd_kd_nearest(svdbd_kd* t, const double* q, size_t nq, size_t qstride, int64_t* out);

#ifdef __cplusplus
}
#endif

#endif /* SVDB_DEVICE_H */
