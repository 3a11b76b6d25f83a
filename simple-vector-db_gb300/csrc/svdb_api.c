/*
 * svdb_api.c -- the drop-in /compare metrics (reference
 * include/vector_database.h:117-135) and the batch entry points of
 * svdb_gb300.h.  Request validation mirrors compare_handler_callback
 * (src/compare_handler.c:74-195); the arithmetic runs on the GPU.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "svdb_internal.h"

int svdb_kd_nearest_batch(KDTree* tree, const double* q, size_t nq, size_t stride, int64_t* out);

/* One drop-in metric call (cosine_similarity & co.), combined with the
 * calls of other threads into one launch (svdb_combine.c). */
typedef struct {
    svdb_call h;
    int metric;
    const double* a;
    const double* b;
    size_t d;
    float out;
    int rc;
    char err[160];
} metric_call;

static svdb_combiner g_metric_comb = SVDB_COMBINER_INIT;
#define ANSWERED ((svdb_db*)(uintptr_t)1) /* a call of the batch already answered */

/* Answers a batch of metric calls: pairs of rows of one store (found by their
 * host buffers) are compared where they are in HBM, one launch per store;
 * every other pair is copied to the device, all of them in one block. */
static void run_metric_batch(void* ctx, svdb_call** calls, size_t n) {
    (void)ctx;
    metric_call** c = (metric_call**)calls;
    svdb_db** st = (svdb_db**)calloc(n, sizeof(svdb_db*));
    int64_t* s1 = (int64_t*)malloc(n * 2 * sizeof(int64_t));
    int32_t* mt = (int32_t*)malloc(n * sizeof(int32_t));
    size_t* pos = (size_t*)malloc(n * sizeof(size_t));
    float* res = (float*)malloc(n * sizeof(float));
    const double** va = (const double**)malloc(n * 2 * sizeof(double*));
    size_t* vd = (size_t*)malloc(n * sizeof(size_t));
    if (!st || !s1 || !mt || !pos || !res || !va || !vd) {
        for (size_t i = 0; i < n; ++i) {
            c[i]->rc = SVDB_ENOMEM;
            snprintf(c[i]->err, sizeof(c[i]->err), "metric: out of host memory");
        }
        goto done;
    }
    int64_t* s2 = s1 + n;
    for (size_t i = 0; i < n; ++i) {
        svdb_db *da = NULL, *db = NULL;
        int64_t sa = -1, sb = -1;
        if (c[i]->d && svdb_rows_find(c[i]->a, &da, &sa) && svdb_rows_find(c[i]->b, &db, &sb) && da == db &&
            da->dim == c[i]->d) {
            st[i] = da;
            s1[i] = sa;
            s2[i] = sb;
        }
    }
    /* stored pairs, store by store (a store whose lock is held elsewhere has
     * its pairs copied instead, so no caller can wait on itself); answered
     * calls are marked ANSWERED */
    for (size_t i = 0; i < n; ++i) {
        svdb_db* d = st[i];
        if (!d || d == ANSWERED) continue;
        int64_t* t1 = (int64_t*)malloc(n * 2 * sizeof(int64_t));
        if (!t1 || pthread_mutex_trylock(&d->pub.mutex) != 0) {
            free(t1);
            for (size_t j = i; j < n; ++j)
                if (st[j] == d) st[j] = NULL;
            continue;
        }
        size_t m = 0;
        for (size_t j = i; j < n; ++j)
            if (st[j] == d) {
                t1[m] = s1[j];
                t1[n + m] = s2[j];
                mt[m] = c[j]->metric;
                pos[m++] = j;
            }
        const int rc = d->dev ? svdbd_compare_slots_mixed(d->dev, mt, t1, t1 + n, m, res) : SVDB_ENODEV;
        pthread_mutex_unlock(&d->pub.mutex);
        for (size_t j = 0; j < m; ++j) {
            metric_call* r = c[pos[j]];
            r->rc = rc;
            r->out = rc ? NAN : res[j];
            if (rc) snprintf(r->err, sizeof(r->err), "%s", svdb_last_error());
            st[pos[j]] = ANSWERED;
        }
        free(t1);
    }
    /* everything else: the vectors themselves, in one copy */
    {
        size_t m = 0;
        for (size_t i = 0; i < n; ++i)
            if (st[i] != ANSWERED) {
                va[m] = c[i]->a;
                va[n + m] = c[i]->b;
                vd[m] = c[i]->d;
                mt[m] = c[i]->metric;
                pos[m++] = i;
            }
        if (m) {
            const int rc = svdbd_compare_vectors_batch(mt, va, va + n, vd, m, res);
            for (size_t j = 0; j < m; ++j) {
                metric_call* r = c[pos[j]];
                r->rc = rc;
                r->out = rc ? NAN : res[j];
                if (rc) snprintf(r->err, sizeof(r->err), "%s", svdb_last_error());
            }
        }
    }
done:
    free(st);
    free(s1);
    free(mt);
    free(pos);
    free(res);
    free(va);
    free(vd);
}

static float metric_vectors(int metric, Vector a, Vector b) {
    if (a.dimension != b.dimension) {
        fprintf(stderr, "Vectors have different dimensions\n"); /* src/vector_database.c:302-305 */
        return -1.0f;
    }
    metric_call call;
    memset(&call, 0, sizeof(call));
    call.metric = metric;
    call.a = a.data;
    call.b = b.data;
    call.d = a.dimension;
    svdb_combine(&g_metric_comb, &call.h, run_metric_batch, NULL);
    if (call.rc != SVDB_OK) {
        svdb_set_error("%s", call.err);
        fprintf(stderr, "metric: %s\n", call.err);
        return NAN;
    }
    return call.out;
}

SVDB_API float cosine_similarity(Vector vec1, Vector vec2) { return metric_vectors(SVDB_COSINE, vec1, vec2); }
SVDB_API float euclidean_distance(Vector vec1, Vector vec2) { return metric_vectors(SVDB_EUCLIDEAN, vec1, vec2); }
SVDB_API float dot_product(Vector vec1, Vector vec2) { return metric_vectors(SVDB_DOT, vec1, vec2); }

SVDB_API int svdb_compare_batch(VectorDatabase* db, int metric, const int64_t* index1, const int64_t* index2,
                                size_t npairs, size_t expected_dim, float* out, int32_t* status) {
    if (!db || (npairs && (!index1 || !index2 || !out || !status))) {
        svdb_set_error("svdb_compare_batch: NULL argument");
        return SVDB_EINVAL;
    }
    svdb_db* d = svdb_of(db);
    int rc = SVDB_OK;
    int64_t* s1 = (int64_t*)malloc((npairs ? npairs : 1) * 2 * sizeof(int64_t));
    size_t* pos = (size_t*)malloc((npairs ? npairs : 1) * sizeof(size_t));
    float* res = (float*)malloc((npairs ? npairs : 1) * sizeof(float));
    if (!s1 || !pos || !res) {
        free(s1);
        free(pos);
        free(res);
        svdb_set_error("svdb_compare_batch: out of host memory");
        return SVDB_ENOMEM;
    }
    int64_t* s2 = s1 + npairs;
    size_t ndev = 0;
    pthread_mutex_lock(&db->mutex);
    for (size_t i = 0; i < npairs; ++i) {
        out[i] = NAN;
        const int64_t a = index1[i], b = index2[i];
        if (a < 0 || b < 0 || (size_t)a >= db->size || (size_t)b >= db->size) {
            status[i] = SVDB_CMP_OUT_OF_BOUNDS;
            continue;
        }
        const Vector* va = &db->vectors[a];
        const Vector* vb = &db->vectors[b];
        if (va->dimension != vb->dimension) {
            status[i] = SVDB_CMP_DIFF_DIM;
            continue;
        }
        if (expected_dim && (va->dimension != expected_dim || vb->dimension != expected_dim)) {
            status[i] = SVDB_CMP_SIZE_MISMATCH;
            continue;
        }
        if (metric < 0 || metric > 2) {
            status[i] = SVDB_CMP_UNKNOWN_METHOD;
            continue;
        }
        status[i] = SVDB_CMP_OK;
        if (d->dev && va->dimension == d->dim) { /* both rows are in the device store */
            s1[ndev] = d->slot_of[a];
            s2[ndev] = d->slot_of[b];
            pos[ndev++] = i;
        } else { /* rows of another dimension: the free-standing vector kernel */
            int r = svdbd_compare_vectors(metric, va->data, vb->data, va->dimension, &out[i]);
            if (r && !rc) rc = r;
        }
    }
    if (!rc && ndev) {
        memmove(s1 + ndev, s2, ndev * sizeof(int64_t));
        rc = svdbd_compare_slots(d->dev, metric, s1, s1 + ndev, ndev, res);
        if (!rc)
            for (size_t j = 0; j < ndev; ++j) out[pos[j]] = res[j];
    }
    pthread_mutex_unlock(&db->mutex);
    free(s1);
    free(pos);
    free(res);
    return rc;
}

SVDB_API int svdb_nearest_batch(VectorDatabase* db, const double* queries, size_t nq, size_t dim,
                                int64_t* out_index) {
    if (!db || (nq && (!queries || !out_index))) {
        svdb_set_error("svdb_nearest_batch: NULL argument");
        return SVDB_EINVAL;
    }
    if (nq && dim < db->kdtree->dimension) {
        svdb_set_error("svdb_nearest_batch: query dimension %zu < KD dimension %zu", dim, db->kdtree->dimension);
        return SVDB_EINVAL;
    }
    /* src/compare_handler.c:403 calls kdtree_nearest without the store lock */
    return svdb_kd_nearest_batch(db->kdtree, queries, nq, dim, out_index);
}

SVDB_API int svdb_nearest_batch_median(VectorDatabase* db, const double* queries, size_t nq, size_t dim,
                                       int64_t* out_index) {
    if (!db || (nq && (!queries || !out_index))) {
        svdb_set_error("svdb_nearest_batch_median: NULL argument");
        return SVDB_EINVAL;
    }
    const size_t kdim = db->kdtree->dimension;
    if (nq && dim < kdim) {
        svdb_set_error("svdb_nearest_batch_median: query dimension %zu < KD dimension %zu", dim, kdim);
        return SVDB_EINVAL;
    }
    svdb_db* d = svdb_of(db);
    pthread_mutex_lock(&db->mutex);
    int rc = SVDB_OK;
    if (!d->dev) { /* no row of nonzero dimension: an empty tree */
        for (size_t i = 0; i < nq; ++i) out_index[i] = -1;
    } else {
        rc = svdbd_kdm_nearest(d->dev, kdim, queries, nq, dim, out_index);
    }
    pthread_mutex_unlock(&db->mutex);
    return rc;
}

static int search_common(VectorDatabase* db, const double* q, size_t nq, size_t dim, size_t k, int metric,
                         int precision, int64_t* ids, double* dists, double* err, int on_device,
                         svdb_search_stats* stats) {
    if (!db || (nq && (!q || !ids || !dists))) {
        svdb_set_error("svdb_search_topk: NULL argument");
        return SVDB_EINVAL;
    }
    svdb_db* d = svdb_of(db);
    pthread_mutex_lock(&db->mutex);
    int rc;
    if (!d->dev) {
        svdb_set_error("svdb_search_topk: the store holds no rows");
        rc = SVDB_EINVAL;
    } else if (dim != d->dim) {
        svdb_set_error("svdb_search_topk: query dimension %zu != store dimension %zu", dim, d->dim);
        rc = SVDB_EINVAL;
    } else {
        rc = svdbd_search(d->dev, q, nq, k, metric, precision, ids, dists, err, on_device, stats);
    }
    pthread_mutex_unlock(&db->mutex);
    return rc;
}

SVDB_API int svdb_search_topk(VectorDatabase* db, const double* queries, size_t nq, size_t dim, size_t k, int metric,
                              int precision, int64_t* ids, double* dists, double* err, svdb_search_stats* stats) {
    return search_common(db, queries, nq, dim, k, metric, precision, ids, dists, err, 0, stats);
}

SVDB_API int svdb_search_topk_device(VectorDatabase* db, const double* d_queries, size_t nq, size_t dim, size_t k,
                                     int metric, int precision, int64_t* d_ids, double* d_dists, double* d_err,
                                     svdb_search_stats* stats) {
    return search_common(db, d_queries, nq, dim, k, metric, precision, d_ids, d_dists, d_err, 1, stats);
}

void svdb_kd_insert_prefix(KDTree* tree, const double* point, size_t avail, size_t index);

SVDB_API int svdb_insert_batch(VectorDatabase* db, const double* rows, size_t n, size_t dim, const char* uuids,
                               size_t* first_index) {
    if (!db || (n && !rows)) {
        svdb_set_error("svdb_insert_batch: NULL argument");
        return SVDB_EINVAL;
    }
    svdb_db* d = svdb_of(db);
    pthread_mutex_lock(&db->mutex);
    int rc = SVDB_OK;
    const size_t first = db->size;
    if (first_index) *first_index = first;
    if (db->size + n > db->capacity) {
        size_t need = db->size + n;
        VectorDatabase* p = db;
        /* same doubling as single inserts */
        size_t nc = p->capacity;
        while (nc < need) nc = nc > SIZE_MAX / 2 ? SIZE_MAX : nc * 2;
        Vector* nv = (Vector*)realloc(p->vectors, nc * sizeof(Vector));
        int64_t* ns = nv ? (int64_t*)realloc(d->slot_of, nc * sizeof(int64_t)) : NULL;
        if (nv) p->vectors = nv;
        if (ns) d->slot_of = ns;
        if (!nv || !ns) {
            pthread_mutex_unlock(&db->mutex);
            svdb_set_error("svdb_insert_batch: out of host memory");
            return SVDB_ENOMEM;
        }
        p->capacity = nc;
    }
    if (svdb_db_ensure_dev(d, dim) != SVDB_OK) {
        pthread_mutex_unlock(&db->mutex);
        return SVDB_ENOMEM;
    }
    /* host copies, owned by the store as if each came from vector_db_insert */
    for (size_t i = 0; i < n; ++i) {
        Vector v;
        memset(&v, 0, sizeof(v));
        if (uuids) {
            memcpy(v.uuid, uuids + i * UUID_SIZE, UUID_SIZE);
        }
        v.dimension = dim;
        v.data = (double*)malloc((dim ? dim : 1) * sizeof(double));
        if (!v.data) {
            rc = SVDB_ENOMEM;
            svdb_set_error("svdb_insert_batch: out of host memory at row %zu", i);
            n = i;
            break;
        }
        memcpy(v.data, rows + i * dim, dim * sizeof(double));
        db->vectors[db->size + i] = v;
    }
    if (d->dev && n) {
        const size_t slot0 = svdbd_store_slots(d->dev);
        int r = dim == d->dim ? svdbd_store_append_block(d->dev, rows, n) : SVDB_OK;
        if (dim != d->dim) {
            for (size_t i = 0; i < n && !r; ++i) {
                const double* none = NULL;
                uint8_t flag = 2;
                r = svdbd_store_append(d->dev, &none, &flag, 1);
            }
        }
        for (size_t i = 0; i < n && !r && uuids; ++i)
            if (uuids[i * UUID_SIZE]) r = svdbd_store_set_uuid(d->dev, (int64_t)(slot0 + i), uuids + i * UUID_SIZE);
        if (r) {
            for (size_t i = 0; i < n; ++i) free(db->vectors[db->size + i].data);
            pthread_mutex_unlock(&db->mutex);
            return r;
        }
        for (size_t i = 0; i < n; ++i) d->slot_of[db->size + i] = (int64_t)(slot0 + i);
        if (dim == d->dim)
            for (size_t i = 0; i < n; ++i) svdb_rows_put(db->vectors[db->size + i].data, d, (int64_t)(slot0 + i));
    } else {
        for (size_t i = 0; i < n; ++i) d->slot_of[db->size + i] = -1;
    }
    for (size_t i = 0; i < n; ++i)
        svdb_kd_insert_prefix(db->kdtree, db->vectors[db->size + i].data, dim, db->size + i);
    db->size += n;
    pthread_mutex_unlock(&db->mutex);
    return rc;
}

SVDB_API int svdb_reserve(VectorDatabase* db, size_t rows, size_t dim) {
    if (!db) return SVDB_EINVAL;
    svdb_db* d = svdb_of(db);
    pthread_mutex_lock(&db->mutex);
    int rc = svdb_db_ensure_dev(d, dim);
    if (!rc && d->dev) {
        if (d->dim != dim) {
            svdb_set_error("svdb_reserve: dimension %zu != store dimension %zu", dim, d->dim);
            rc = SVDB_EINVAL;
        } else {
            rc = svdbd_store_reserve(d->dev, rows);
        }
    }
    pthread_mutex_unlock(&db->mutex);
    return rc;
}

SVDB_API int svdb_sync(VectorDatabase* db) {
    if (!db) return SVDB_EINVAL;
    svdb_db* d = svdb_of(db);
    pthread_mutex_lock(&db->mutex);
    int rc = d->dev ? svdbd_store_sync(d->dev) : SVDB_OK;
    if (!rc) {
        svdb_kd* t = svdb_kd_of(db->kdtree);
        pthread_mutex_lock(&t->lock);
        if (t->n && t->pub.dimension) rc = svdb_kd_sync_locked(t);
        pthread_mutex_unlock(&t->lock);
    }
    pthread_mutex_unlock(&db->mutex);
    return rc;
}

SVDB_API void* svdb_stream(VectorDatabase* db) {
    if (!db) return NULL;
    svdb_db* d = svdb_of(db);
    return d->dev ? svdbd_store_stream(d->dev) : NULL;
}

SVDB_API int svdb_wait(VectorDatabase* db) {
    if (!db) return SVDB_EINVAL;
    svdb_db* d = svdb_of(db);
    return d->dev ? svdbd_store_wait(d->dev) : SVDB_OK;
}

SVDB_API int svdb_set_fp8_screen(VectorDatabase* db, int mode) {
    if (!db) return SVDB_EINVAL;
    svdb_db* d = svdb_of(db);
    pthread_mutex_lock(&db->mutex);
    int rc = d->dev ? svdbd_store_set_fp8(d->dev, mode) : SVDB_EINVAL;
    if (!d->dev) svdb_set_error("svdb_set_fp8_screen: the store holds no rows");
    pthread_mutex_unlock(&db->mutex);
    return rc;
}

SVDB_API int svdb_set_screen_seeding(VectorDatabase* db, int mode) {
    if (!db) return SVDB_EINVAL;
    svdb_db* d = svdb_of(db);
    pthread_mutex_lock(&db->mutex);
    int rc = d->dev ? svdbd_store_set_seeding(d->dev, mode) : SVDB_EINVAL;
    if (!d->dev) svdb_set_error("svdb_set_screen_seeding: the store holds no rows");
    pthread_mutex_unlock(&db->mutex);
    return rc;
}

SVDB_API int svdb_profile(VectorDatabase* db, int enable) {
    if (!db) return SVDB_EINVAL;
    svdb_db* d = svdb_of(db);
    pthread_mutex_lock(&db->mutex);
    int rc = d->dev ? svdbd_store_profile(d->dev, enable) : SVDB_EINVAL;
    if (!d->dev) svdb_set_error("svdb_profile: the store holds no rows");
    pthread_mutex_unlock(&db->mutex);
    return rc;
}

SVDB_API int svdb_profile_read(VectorDatabase* db, double* ms, int reset) {
    if (!db) return SVDB_EINVAL;
    svdb_db* d = svdb_of(db);
    pthread_mutex_lock(&db->mutex);
    int rc = d->dev ? svdbd_store_profile_read(d->dev, ms, reset) : 0;
    pthread_mutex_unlock(&db->mutex);
    return rc;
}

/* See include/svdb_gb300.h: the search for callers that cannot allocate. */
SVDB_API int svdb_search_topk_fp64_noalloc(VectorDatabase* db, const double* d_queries, size_t nq, size_t dim,
                                           size_t k, int metric, int64_t* d_ids, double* d_dists) {
    if (!db) {
        svdb_set_error("svdb_search_topk_fp64_noalloc: NULL database");
        return SVDB_EINVAL;
    }
    svdb_db* d = svdb_of(db);
    pthread_mutex_lock(&db->mutex);
    int rc;
    if (!d->dev) {
        svdb_set_error("svdb_search_topk_fp64_noalloc: the store holds no rows");
        rc = SVDB_EINVAL;
    } else if (dim != d->dim) {
        svdb_set_error("svdb_search_topk_fp64_noalloc: query dimension %zu != store dimension %zu", dim, d->dim);
        rc = SVDB_EINVAL;
    } else {
        rc = svdbd_search_noalloc(d->dev, d_queries, nq, k, metric, d_ids, d_dists);
    }
    pthread_mutex_unlock(&db->mutex);
    return rc;
}

/* ---- POST /nearest bodies decoded on the device --------------------------- */
SVDB_API int svdb_decode_vectors(const char* text, const uint64_t* offsets, size_t n, size_t dim, double* out,
                                 int32_t* status) {
    if (n && (!text || !offsets || !out || !status)) {
        svdb_set_error("svdb_decode_vectors: NULL argument");
        return SVDB_EINVAL;
    }
    for (size_t i = 0; i < n; ++i)
        if (offsets[i + 1] < offsets[i]) {
            svdb_set_error("svdb_decode_vectors: offsets must not decrease (body %zu)", i);
            return SVDB_EINVAL;
        }
    return svdbd_decode_bodies(text, offsets, n, dim, out, status);
}

/* ---- GET /vector?uuid= in batches ---------------------------------------- */
SVDB_API int svdb_find_uuid_batch(VectorDatabase* db, const char* uuids, size_t n, int64_t* out_index) {
    if (!db || (n && (!uuids || !out_index))) {
        svdb_set_error("svdb_find_uuid_batch: NULL argument");
        return SVDB_EINVAL;
    }
    svdb_db* d = svdb_of(db);
    pthread_mutex_lock(&db->mutex);
    int rc = SVDB_OK;
    if (d->dev) {
        rc = svdbd_uuid_find(d->dev, uuids, n, out_index);
    } else { /* no row of nonzero dimension yet: nothing on the device */
        for (size_t q = 0; q < n; ++q) {
            out_index[q] = -1;
            for (size_t i = 0; i < db->size; ++i)
                if (strncmp(db->vectors[i].uuid, uuids + q * UUID_SIZE, UUID_SIZE) == 0) {
                    out_index[q] = (int64_t)i;
                    break;
                }
        }
    }
    pthread_mutex_unlock(&db->mutex);
    return rc;
}

/* ---- ragged batches over several collections ---------------------------- */
struct svdb_ragged {
    svdbd_ragged* dev;
    VectorDatabase** dbs; /* distinct, in address order (the order their locks are taken) */
    size_t ndb;
};

static int db_addr_cmp(const void* a, const void* b) {
    const uintptr_t x = (uintptr_t) * (VectorDatabase* const*)a, y = (uintptr_t) * (VectorDatabase* const*)b;
    return x < y ? -1 : (x > y);
}

static void ragged_lock(svdb_ragged* r, int lock) {
    for (size_t i = 0; i < r->ndb; ++i) {
        if (lock)
            pthread_mutex_lock(&r->dbs[i]->mutex);
        else
            pthread_mutex_unlock(&r->dbs[r->ndb - 1 - i]->mutex);
    }
}

SVDB_API svdb_ragged* svdb_ragged_create(const svdb_ragged_part* parts, size_t nparts, int metric, int precision,
                                         unsigned flags) {
    if (!parts || nparts == 0 || metric < 0 || metric > 2 ||
        (precision != SVDB_PREC_FP64 && precision != SVDB_PREC_BF16 && precision != SVDB_PREC_FP8)) {
        svdb_set_error("svdb_ragged_create: bad argument (parts, metric or precision)");
        return NULL;
    }
    svdb_ragged* r = (svdb_ragged*)calloc(1, sizeof(svdb_ragged));
    svdbd_ragged_part* dp = (svdbd_ragged_part*)calloc(nparts, sizeof(svdbd_ragged_part));
    if (r) r->dbs = (VectorDatabase**)calloc(nparts, sizeof(VectorDatabase*));
    if (!r || !dp || !r->dbs) {
        svdb_set_error("svdb_ragged_create: out of host memory");
        if (r) free(r->dbs);
        free(r);
        free(dp);
        return NULL;
    }
    for (size_t i = 0; i < nparts; ++i) {
        const svdb_ragged_part* p = &parts[i];
        if (!p->db || (p->nq && (!p->d_queries || !p->k || !p->d_ids || !p->d_dists))) {
            svdb_set_error("svdb_ragged_create: part %zu: NULL argument", i);
            goto fail;
        }
        size_t j = 0;
        while (j < r->ndb && r->dbs[j] != p->db) ++j;
        if (j == r->ndb) r->dbs[r->ndb++] = p->db;
    }
    qsort(r->dbs, r->ndb, sizeof(VectorDatabase*), db_addr_cmp);
    ragged_lock(r, 1);
    for (size_t i = 0; i < nparts; ++i) {
        const svdb_ragged_part* p = &parts[i];
        svdb_db* d = svdb_of(p->db);
        if (!d->dev) {
            svdb_set_error("svdb_ragged_create: part %zu: the store holds no rows", i);
            break;
        }
        if (p->dim != d->dim) {
            svdb_set_error("svdb_ragged_create: part %zu: query dimension %zu != store dimension %zu", i, p->dim,
                           d->dim);
            break;
        }
        size_t bad = p->nq;
        for (size_t q = 0; q < p->nq && bad == p->nq; ++q)
            if (p->k[q] == 0 || p->k[q] > 128 || p->k[q] > p->stride) bad = q;
        if (bad != p->nq) {
            svdb_set_error("svdb_ragged_create: part %zu query %zu: k = %u (must be 1..128 and <= stride %zu)", i,
                           bad, p->k[bad], p->stride);
            break;
        }
        dp[i].store = d->dev;
        dp[i].nq = p->nq;
        dp[i].stride = p->stride;
        dp[i].d_queries = p->d_queries;
        dp[i].k = p->k;
        dp[i].d_ids = p->d_ids;
        dp[i].d_dists = p->d_dists;
    }
    if (!dp[nparts - 1].store && parts[nparts - 1].db) {
        /* a part failed validation above (message already set) */
    } else {
        size_t ok = 0;
        while (ok < nparts && dp[ok].store) ++ok;
        if (ok == nparts) r->dev = svdbd_ragged_create(dp, nparts, metric, precision, flags);
    }
    ragged_lock(r, 0);
    if (!r->dev) goto fail;
    free(dp);
    return r;
fail:
    free(dp);
    free(r->dbs);
    free(r);
    return NULL;
}

SVDB_API int svdb_ragged_run(svdb_ragged* r) {
    if (!r) {
        svdb_set_error("svdb_ragged_run: NULL plan");
        return SVDB_EINVAL;
    }
    ragged_lock(r, 1);
    int rc = svdbd_ragged_run(r->dev);
    ragged_lock(r, 0);
    return rc;
}

SVDB_API int svdb_ragged_wait(svdb_ragged* r) {
    if (!r) {
        svdb_set_error("svdb_ragged_wait: NULL plan");
        return SVDB_EINVAL;
    }
    ragged_lock(r, 1);
    int rc = svdbd_ragged_wait(r->dev);
    ragged_lock(r, 0);
    return rc;
}

SVDB_API void* svdb_ragged_stream(svdb_ragged* r) { return r ? svdbd_ragged_stream(r->dev) : NULL; }

SVDB_API int svdb_ragged_get_search_stats(svdb_ragged* r, uint64_t* out, size_t n) {
    if (!r || (n && !out)) {
        svdb_set_error("svdb_ragged_get_search_stats: NULL argument");
        return SVDB_EINVAL;
    }
    ragged_lock(r, 1);
    int rc = svdbd_ragged_search_stats(r->dev, out, n);
    ragged_lock(r, 0);
    return rc;
}

SVDB_API int svdb_ragged_get_info(svdb_ragged* r, svdb_ragged_info* info) {
    if (!r || !info) {
        svdb_set_error("svdb_ragged_get_info: NULL argument");
        return SVDB_EINVAL;
    }
    return svdbd_ragged_info(r->dev, info);
}

SVDB_API void svdb_ragged_destroy(svdb_ragged* r) {
    if (!r) return;
    ragged_lock(r, 1);
    svdbd_ragged_destroy(r->dev);
    ragged_lock(r, 0);
    free(r->dbs);
    free(r);
}

SVDB_API int svdb_selftest_bounded_wait(VectorDatabase* db, uint32_t limit_us, uint32_t* gave_up) {
    if (!db) {
        svdb_set_error("svdb_selftest_bounded_wait: NULL database");
        return SVDB_EINVAL;
    }
    svdb_db* d = svdb_of(db);
    pthread_mutex_lock(&db->mutex);
    int rc;
    if (!d->dev) {
        svdb_set_error("svdb_selftest_bounded_wait: the store holds no rows (no device store yet)");
        rc = SVDB_EINVAL;
    } else {
        rc = svdbd_selftest_wait(d->dev, limit_us, gave_up);
    }
    pthread_mutex_unlock(&db->mutex);
    return rc;
}

/* See include/svdb_gb300.h: the screen's raw accumulators (diagnostics). */
SVDB_API int svdb_debug_screen_accumulators(VectorDatabase* db, const double* queries, size_t nq, size_t dim,
                                            int metric, int precision, size_t rows, float* acc, void* query_ops,
                                            void* row_ops, size_t* op_bytes) {
    if (!db || (precision != SVDB_PREC_BF16 && precision != SVDB_PREC_FP8)) {
        svdb_set_error("svdb_debug_screen_accumulators: NULL database or precision not BF16/FP8");
        return SVDB_EINVAL;
    }
    svdb_db* d = svdb_of(db);
    pthread_mutex_lock(&db->mutex);
    int rc;
    if (!d->dev) {
        svdb_set_error("svdb_debug_screen_accumulators: the store holds no rows (no device store yet)");
        rc = SVDB_EINVAL;
    } else if (dim != d->dim) {
        svdb_set_error("svdb_debug_screen_accumulators: query dimension %zu != store dimension %zu", dim, d->dim);
        rc = SVDB_EINVAL;
    } else {
        rc = svdbd_debug_screen_acc(d->dev, queries, nq, metric, precision == SVDB_PREC_FP8, rows, acc, query_ops,
                                    row_ops, op_bytes);
    }
    pthread_mutex_unlock(&db->mutex);
    return rc;
}

/* ---- the request path as a device-side loop (dev_loop.cu) ----------------- */
struct svdb_loop {
    svdbd_loop* dev;
    size_t dim;
};

SVDB_API svdb_loop* svdb_loop_create(const svdb_loop_config* cfg, const double* rows, size_t n,
                                     const char* uuids37) {
    if (!cfg || cfg->dim == 0 || cfg->kd_dim == 0 || cfg->kd_dim > 32 || cfg->kd_dim > cfg->dim ||
        cfg->capacity < n || cfg->capacity >= (size_t)1 << 31 || (n && !rows)) {
        svdb_set_error("svdb_loop_create: bad configuration (dim >= kd_dim in 1..32, capacity >= rows, < 2^31)");
        return NULL;
    }
    svdb_loop_config c = *cfg;
    if (!c.kd_capacity) c.kd_capacity = 2 * c.capacity;
    if (!c.ring) c.ring = 4096;
    if (!c.max_batch || c.max_batch > 256) c.max_batch = 256;
    if (!c.idle_us) c.idle_us = 1000000;
    if (c.kd_capacity < n || c.kd_capacity >= (size_t)1 << 31) {
        svdb_set_error("svdb_loop_create: kd_capacity must hold the initial rows' nodes (< 2^31)");
        return NULL;
    }
    /* the initial KD tree, built in row order exactly as n inserts would build it */
    KDTree* t = kdtree_create(c.kd_dim);
    if (!t) {
        svdb_set_error("svdb_loop_create: out of host memory");
        return NULL;
    }
    for (size_t i = 0; i < n; ++i) svdb_kd_insert_prefix(t, rows + i * c.dim, c.dim, i);
    svdb_kd* k = svdb_kd_of(t);
    if (k->n != n) {
        kdtree_free(t);
        svdb_set_error("svdb_loop_create: out of host memory building the KD tree");
        return NULL;
    }
    svdb_loop* l = (svdb_loop*)calloc(1, sizeof(svdb_loop));
    if (l) {
        l->dim = c.dim;
        l->dev = svdbd_loop_create(&c, rows, n, uuids37, k->pts, k->index, k->left, k->right, k->n, k->height);
        if (!l->dev) {
            free(l);
            l = NULL;
        }
    } else {
        svdb_set_error("svdb_loop_create: out of host memory");
    }
    kdtree_free(t);
    return l;
}

SVDB_API int svdb_loop_start(svdb_loop* l) {
    if (!l) return SVDB_EINVAL;
    return svdbd_loop_start(l->dev);
}

SVDB_API int svdb_loop_submit(svdb_loop* l, const svdb_request* req, uint64_t* ticket) {
    if (!l || !req || !ticket) {
        svdb_set_error("svdb_loop_submit: NULL argument");
        return SVDB_EINVAL;
    }
    if ((req->op == SVDB_REQ_INSERT || req->op == SVDB_REQ_UPDATE || req->op == SVDB_REQ_KD_NEAREST) && !req->vec) {
        svdb_set_error("svdb_loop_submit: request %d needs a vector", req->op);
        return SVDB_EINVAL;
    }
    return svdbd_loop_submit(l->dev, req, l->dim, ticket, 10000000u);
}

SVDB_API int svdb_loop_wait(svdb_loop* l, uint64_t ticket, svdb_response* resp, uint32_t timeout_us) {
    if (!l || !resp) return SVDB_EINVAL;
    return svdbd_loop_wait(l->dev, ticket, resp, timeout_us);
}

SVDB_API int svdb_loop_stop(svdb_loop* l) { return l ? svdbd_loop_stop(l->dev) : SVDB_EINVAL; }

SVDB_API int svdb_loop_get_info(svdb_loop* l, svdb_loop_info* out) {
    return (l && out) ? svdbd_loop_info(l->dev, out) : SVDB_EINVAL;
}

SVDB_API int svdb_loop_read(svdb_loop* l, size_t position, double* row, char* uuid37) {
    return (l && row) ? svdbd_loop_read(l->dev, position, row, uuid37) : SVDB_EINVAL;
}

SVDB_API void svdb_loop_destroy(svdb_loop* l) {
    if (!l) return;
    svdbd_loop_destroy(l->dev);
    free(l);
}

/* See include/svdb_gb300.h: response bodies of GET /compare. */
SVDB_API int svdb_format_compare(const int32_t* metric, const float* value, const int32_t* status, size_t n,
                                 char* out, size_t cap, uint64_t* offsets) {
    if (!offsets || (n && (!metric || !value || !status))) {
        svdb_set_error("svdb_format_compare: NULL argument");
        return SVDB_EINVAL;
    }
    for (size_t i = 0; i < n; ++i)
        if (status[i] == SVDB_CMP_OK && (metric[i] < 0 || metric[i] > 2)) {
            svdb_set_error("svdb_format_compare: metric %d of answer %zu is not 0..2", metric[i], i);
            return SVDB_EINVAL;
        }
    return svdbd_format_compare(metric, value, status, n, out, cap, offsets);
}

/* See include/svdb_gb300.h: response bodies of POST /nearest. */
SVDB_API int svdb_format_nearest(VectorDatabase* db, const int64_t* index, size_t n, char* out, size_t cap,
                                 uint64_t* offsets) {
    if (!db || !offsets || (n && !index)) {
        svdb_set_error("svdb_format_nearest: NULL argument");
        return SVDB_EINVAL;
    }
    svdb_db* d = svdb_of(db);
    const size_t m = n ? n : 1;
    int32_t* kind = (int32_t*)malloc(m * sizeof(int32_t));
    uint64_t* idx = (uint64_t*)malloc(m * sizeof(uint64_t));
    int64_t* slot = (int64_t*)malloc(m * sizeof(int64_t));
    uint32_t* dims = (uint32_t*)malloc(m * sizeof(uint32_t));
    const double** rows = (const double**)malloc(m * sizeof(double*));
    char* uu = (char*)calloc(m, UUID_SIZE);
    int rc = SVDB_OK;
    if (!kind || !idx || !slot || !dims || !rows || !uu) {
        svdb_set_error("svdb_format_nearest: out of host memory");
        rc = SVDB_ENOMEM;
        goto out_free;
    }
    pthread_mutex_lock(&db->mutex);
    for (size_t i = 0; i < n; ++i) {
        idx[i] = (uint64_t)index[i];
        slot[i] = -1;
        dims[i] = 0;
        rows[i] = NULL;
        if (index[i] < 0) { /* kdtree_nearest gave (size_t)-1 (src/compare_handler.c:422) */
            kind[i] = 0;
        } else if ((size_t)index[i] >= db->size) { /* a stale KD node: vector_db_read is NULL (:419) */
            kind[i] = -1;
        } else {
            const Vector* v = &db->vectors[index[i]];
            kind[i] = 1;
            dims[i] = (uint32_t)v->dimension;
            rows[i] = v->data;
            memcpy(uu + i * UUID_SIZE, v->uuid, UUID_SIZE);
            if (d->dev && v->data && v->dimension == d->dim && d->slot_of[index[i]] >= 0)
                slot[i] = d->slot_of[index[i]];
        }
    }
    rc = svdbd_format_nearest(d->dev, n, kind, idx, slot, dims, rows, uu, out, cap, offsets);
    pthread_mutex_unlock(&db->mutex);
out_free:
    free(kind);
    free(idx);
    free(slot);
    free(dims);
    free(rows);
    free(uu);
    return rc;
}

/* ---- merge of per-shard top-k lists (host) ------------------------------ */
typedef struct {
    double key;
    int64_t id;
    double val;
} merge_ent;

static double merge_key(int metric, double v) {
    if (isnan(v)) return INFINITY;
    return metric == SVDB_EUCLIDEAN ? v : -v;
}

static int merge_less(const merge_ent* a, const merge_ent* b) {
    return a->key < b->key || (a->key == b->key && a->id < b->id);
}

SVDB_API int svdb_merge_topk(int metric, const int64_t* ids, const double* vals, size_t nshards, size_t nq, size_t k,
                             int64_t* out_ids, double* out_vals) {
    if (metric < 0 || metric > 2 || k == 0 || (nq && (!ids || !vals || !out_ids || !out_vals))) {
        svdb_set_error("svdb_merge_topk: bad argument");
        return SVDB_EINVAL;
    }
    merge_ent* best = (merge_ent*)malloc(k * sizeof(merge_ent));
    if (!best) {
        svdb_set_error("svdb_merge_topk: out of host memory");
        return SVDB_ENOMEM;
    }
    for (size_t q = 0; q < nq; ++q) {
        size_t cnt = 0;
        for (size_t sh = 0; sh < nshards; ++sh) {
            const size_t base = (sh * nq + q) * k;
            for (size_t j = 0; j < k; ++j) {
                if (ids[base + j] < 0) continue;
                merge_ent e = {merge_key(metric, vals[base + j]), ids[base + j], vals[base + j]};
                if (cnt == k && !merge_less(&e, &best[k - 1])) continue;
                size_t pos = cnt < k ? cnt++ : k - 1;
                while (pos > 0 && merge_less(&e, &best[pos - 1])) {
                    best[pos] = best[pos - 1];
                    --pos;
                }
                best[pos] = e;
            }
        }
        for (size_t j = 0; j < k; ++j) {
            out_ids[q * k + j] = j < cnt ? best[j].id : -1;
            out_vals[q * k + j] = j < cnt ? best[j].val : NAN;
        }
    }
    free(best);
    return SVDB_OK;
}
