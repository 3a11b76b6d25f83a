/*
 * vector_database.h -- drop-in store + /compare metric API of
 * simple-vector-db, served by libsvdb_gb300.so (one GB300, sm_103a).
 *
 * Types and prototypes keep the reference's layout and signatures so the
 * unmodified libmicrohttpd/cJSON handlers compile and link against this
 * library; each declaration cites the reference declaration it replaces.
 *
 * Behaviour kept from the reference:
 *   - rows are addressed by a positional index that shifts on delete;
 *   - insert/update take ownership of vec.data (a malloc'd host buffer);
 *   - update adds a second KD node for the row, delete leaves the KD tree
 *     untouched, load rebuilds the tree in row order;
 *   - the metrics return float, accumulate in float, and return -1.0f on a
 *     dimension mismatch.
 * What changes: every row is mirrored into a device-resident store (FP64
 * master + BF16 shadow + per-row norms) and every metric, /nearest and
 * top-k search runs as a CUDA kernel.  There is no CPU fallback: when the
 * GPU is unavailable, the calls fail the way the reference fails
 * ((size_t)-1, NULL, -1.0f) and svdb_last_error() says why.
 *
 * The VectorDatabase returned by vector_db_init/vector_db_load is the first
 * member of a larger private object; only pointers obtained from those two
 * calls may be passed to this API.
 */
#ifndef VECTOR_DATABASE_H
#define VECTOR_DATABASE_H

#include <pthread.h>
#include <stddef.h>

#include "kdtree.h"

#ifdef __cplusplus
extern "C" {
#endif

#define UUID_SIZE 37 /* 36 characters + NUL (reference include/vector_database.h:8) */

/* One stored row.  Same layout as reference include/vector_database.h:14-18. */
typedef struct Vector {
    char uuid[UUID_SIZE];
    size_t dimension;
    double* data;
} Vector;

/* The store.  Same layout as reference include/vector_database.h:24-30; the
 * handlers read size, vectors[i] and kdtree directly. */
typedef struct VectorDatabase {
    Vector* vectors;
    size_t size;
    size_t capacity;
    KDTree* kdtree;
    pthread_mutex_t mutex;
} VectorDatabase;

/* replaces vector_db_init, reference include/vector_database.h:39
 * (src/vector_database.c:17-54).  capacity 0 means 10; `dimension` is the
 * KD-tree prefix length. */
VectorDatabase* vector_db_init(size_t initial_capacity, size_t dimension);

/* replaces vector_db_free, reference include/vector_database.h:46 */
void vector_db_free(VectorDatabase* db);

/* replaces vector_db_insert, reference include/vector_database.h:55
 * (src/vector_database.c:81-119).  Returns the new index or (size_t)-1. */
size_t vector_db_insert(VectorDatabase* db, Vector vec);

/* replaces vector_db_read, reference include/vector_database.h:64 */
Vector* vector_db_read(VectorDatabase* db, size_t index);

/* replaces vector_db_read_by_uuid, reference include/vector_database.h:73 */
Vector* vector_db_read_by_uuid(VectorDatabase* db, const char* uuid);

/* replaces vector_db_update, reference include/vector_database.h:83
 * (src/vector_database.c:169-177); out-of-range indices are ignored. */
void vector_db_update(VectorDatabase* db, size_t index, Vector vec);

/* replaces vector_db_delete, reference include/vector_database.h:91
 * (src/vector_database.c:185-195); out-of-range indices are ignored. */
void vector_db_delete(VectorDatabase* db, size_t index);

/* replaces vector_db_save, reference include/vector_database.h:99
 * (file format of src/vector_database.c:203-228). */
void vector_db_save(VectorDatabase* db, const char* filename);

/* replaces vector_db_load, reference include/vector_database.h:108
 * (src/vector_database.c:237-292); `dimension` is the KD prefix length. */
VectorDatabase* vector_db_load(const char* filename, size_t dimension);

/* replaces cosine_similarity, reference include/vector_database.h:117
 * (src/vector_database.c:301-313), bit-identical results. */
float cosine_similarity(Vector vec1, Vector vec2);

/* replaces euclidean_distance, reference include/vector_database.h:126
 * (src/vector_database.c:322-333), bit-identical results. */
float euclidean_distance(Vector vec1, Vector vec2);

/* replaces dot_product, reference include/vector_database.h:135
 * (src/vector_database.c:342-352), bit-identical results. */
float dot_product(Vector vec1, Vector vec2);

#ifdef __cplusplus
}
#endif

#endif /* VECTOR_DATABASE_H */
