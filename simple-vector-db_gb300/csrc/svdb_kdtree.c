/*
 * svdb_kdtree.c -- the drop-in kdtree_* API (reference include/kdtree.h).
 *
 * Insert keeps the reference's tree exactly (src/kdtree.c:47-62: split axis
 * depth % dimension, "<" goes left, else right) but stores nodes in flat
 * arrays instead of one malloc per node, with no console output.  The walk
 * to the insertion point is O(depth) host bookkeeping; the arrays are
 * mirrored to the GPU incrementally (new nodes + changed parent links), and
 * every nearest-neighbour search runs there (dev_kd.cu).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "svdb_internal.h"

SVDB_API KDTree* kdtree_create(size_t dimension) {
    svdb_kd* t = (svdb_kd*)calloc(1, sizeof(svdb_kd));
    if (!t) return NULL;
    t->pub.root = NULL;
    t->pub.dimension = dimension;
    pthread_mutex_init(&t->lock, NULL);
    pthread_mutex_init(&t->comb.mu, NULL);
    pthread_cond_init(&t->comb.cv, NULL);
    return &t->pub;
}

SVDB_API void kdtree_free(KDTree* tree) {
    svdb_kd* t = svdb_kd_of(tree);
    if (!t) return;
    if (t->dev) svdbd_kd_destroy(t->dev);
    free(t->pts);
    free(t->index);
    free(t->left);
    free(t->right);
    free(t->patch);
    free(t->comb.q);
    pthread_cond_destroy(&t->comb.cv);
    pthread_mutex_destroy(&t->comb.mu);
    pthread_mutex_destroy(&t->lock);
    free(t);
}

static int kd_grow(svdb_kd* t) {
    size_t nc = t->cap ? t->cap * 2 : 1024;
    size_t dim = t->pub.dimension ? t->pub.dimension : 1;
    double* p = (double*)realloc(t->pts, nc * dim * sizeof(double));
    if (!p) return -1;
    t->pts = p;
    int64_t* ix = (int64_t*)realloc(t->index, nc * sizeof(int64_t));
    if (!ix) return -1;
    t->index = ix;
    int32_t* l = (int32_t*)realloc(t->left, nc * sizeof(int32_t));
    if (!l) return -1;
    t->left = l;
    int32_t* r = (int32_t*)realloc(t->right, nc * sizeof(int32_t));
    if (!r) return -1;
    t->right = r;
    t->cap = nc;
    return 0;
}

static int kd_note_patch(svdb_kd* t, int32_t node) {
    if ((size_t)node >= t->synced) return 0; /* not mirrored yet: goes up with its own record */
    if (t->npatch == t->patch_cap) {
        size_t nc = t->patch_cap ? 2 * t->patch_cap : 256;
        int32_t* p = (int32_t*)realloc(t->patch, nc * sizeof(int32_t));
        if (!p) return -1;
        t->patch = p;
        t->patch_cap = nc;
    }
    t->patch[t->npatch++] = node;
    return 0;
}

/* Insert with an explicit prefix length `avail` of valid coordinates in
 * `point` (missing coordinates read as 0). */
static void kd_insert_locked(svdb_kd* t, const double* point, size_t avail, size_t index) {
    const size_t dim = t->pub.dimension;
    if (dim == 0) return; /* the reference divides by zero here (src/kdtree.c:53) */
    if (t->n >= 0x7fffffff) return;
    if (t->n == t->cap && kd_grow(t) != 0) {
        fprintf(stderr, "kdtree_insert: out of memory\n");
        return;
    }
    const int32_t id = (int32_t)t->n;
    double* p = t->pts + (size_t)id * dim;
    for (size_t i = 0; i < dim; ++i) p[i] = i < avail ? point[i] : 0.0;
    t->index[id] = (int64_t)index;
    t->left[id] = t->right[id] = -1;
    t->n++;
    int depth = 1;
    if (id > 0) {
        int32_t cur = 0;
        size_t d = 0;
        for (;;) {
            const size_t cd = d % dim;
            int32_t* slot = p[cd] < t->pts[(size_t)cur * dim + cd] ? &t->left[cur] : &t->right[cur];
            ++depth;
            if (*slot < 0) {
                *slot = id;
                kd_note_patch(t, cur);
                break;
            }
            cur = *slot;
            ++d;
        }
    }
    if (depth > t->height) t->height = depth;
}

SVDB_API void kdtree_insert(KDTree* tree, const double* point, size_t index) {
    svdb_kd* t = svdb_kd_of(tree);
    if (!t || !point) return;
    pthread_mutex_lock(&t->lock);
    kd_insert_locked(t, point, t->pub.dimension, index);
    pthread_mutex_unlock(&t->lock);
}

/* used by the store when a row is shorter than the KD prefix */
void svdb_kd_insert_prefix(KDTree* tree, const double* point, size_t avail, size_t index) {
    svdb_kd* t = svdb_kd_of(tree);
    if (!t) return;
    pthread_mutex_lock(&t->lock);
    kd_insert_locked(t, point, avail, index);
    pthread_mutex_unlock(&t->lock);
}

int svdb_kd_sync_locked(svdb_kd* t) {
    if (!t->dev) {
        t->dev = svdbd_kd_create(t->pub.dimension);
        if (!t->dev) return SVDB_ENODEV;
    }
    if (t->synced == t->n && t->npatch == 0) return SVDB_OK;
    int rc = svdbd_kd_sync(t->dev, t->pts, t->index, t->left, t->right, t->n, t->synced, t->patch, t->npatch,
                           t->height);
    if (rc) return rc;
    t->synced = t->n;
    t->npatch = 0;
    return SVDB_OK;
}

/* nq queries with row stride `stride`; out[i] = stored index or -1 */
int svdb_kd_nearest_batch(KDTree* tree, const double* q, size_t nq, size_t stride, int64_t* out) {
    svdb_kd* t = svdb_kd_of(tree);
    if (!t || (!q && nq)) return SVDB_EINVAL;
    pthread_mutex_lock(&t->lock);
    int rc = SVDB_OK;
    if (t->n == 0 || t->pub.dimension == 0) {
        for (size_t i = 0; i < nq; ++i) out[i] = -1; /* src/kdtree.c:172-174 */
    } else {
        rc = svdb_kd_sync_locked(t);
        if (!rc) rc = svdbd_kd_nearest(t->dev, q, nq, stride, out);
    }
    pthread_mutex_unlock(&t->lock);
    return rc;
}

/* One kdtree_nearest call, combined with other threads' calls on the same
 * tree into one descent launch (svdb_combine.c). */
typedef struct {
    svdb_call h;
    const double* q;
    int64_t out;
    int rc;
    char err[160];
} nearest_call;

static void run_nearest_batch(void* ctx, svdb_call** calls, size_t n) {
    svdb_kd* t = (svdb_kd*)ctx;
    nearest_call** c = (nearest_call**)calls;
    const size_t kd = t->pub.dimension;
    double* q = (double*)malloc((n * kd ? n * kd : 1) * sizeof(double));
    int64_t* out = (int64_t*)malloc(n * sizeof(int64_t));
    int rc = (q && out) ? SVDB_OK : SVDB_ENOMEM;
    if (!rc) {
        for (size_t i = 0; i < n; ++i) memcpy(q + i * kd, c[i]->q, kd * sizeof(double));
        rc = svdb_kd_nearest_batch(&t->pub, q, n, kd, out);
    }
    for (size_t i = 0; i < n; ++i) {
        c[i]->rc = rc;
        c[i]->out = rc ? -1 : out[i];
        if (rc) snprintf(c[i]->err, sizeof(c[i]->err), "%s", rc == SVDB_ENOMEM ? "out of host memory" : svdb_last_error());
    }
    free(q);
    free(out);
}

SVDB_API size_t kdtree_nearest(KDTree* tree, const double* point) {
    if (!tree || !point) return (size_t)-1;
    nearest_call call;
    memset(&call, 0, sizeof(call));
    call.q = point;
    svdb_combine(&svdb_kd_of(tree)->comb, &call.h, run_nearest_batch, svdb_kd_of(tree));
    if (call.rc) {
        svdb_set_error("%s", call.err);
        fprintf(stderr, "kdtree_nearest: %s\n", call.err);
        return (size_t)-1;
    }
    return call.out < 0 ? (size_t)-1 : (size_t)call.out;
}
