/*
 * svdb_combine.c -- the drop-in per-call path: which stored row a Vector's
 * data pointer is, and combining of concurrent calls into one launch.
 *
 * The reference's handlers call the metric functions and kdtree_nearest one
 * request at a time, from one thread per connection
 * (src/compare_handler.c:153-159,403, src/main.c:381):
 *   cosine_similarity(*vector_db_read(db, i1), *vector_db_read(db, i2))
 * The Vectors they pass are the store's own rows, whose host buffers the
 * store owns (src/vector_database.c:113,172,188).  Two things make such calls
 * cheap on the GPU:
 *
 *  - a registry from a row's host buffer to its device slot, kept by the
 *    store on every insert, update, delete and free, so a metric of two
 *    stored rows reads them where they already are in HBM instead of copying
 *    them to the device first;
 *  - a combiner: callers that arrive while a launch is in flight queue up;
 *    when it finishes, one of them takes every queued call and answers all of
 *    them with one launch (per store), so concurrent callers share the round
 *    trip instead of waiting on one another's.
 *
 * Results are the reference's bit for bit (the same kernels as
 * svdb_compare_batch / svdb_nearest_batch).  A row changed behind the store's
 * back (writing through a pointer vector_db_read returned) is not seen by the
 * device copy; the reference's handlers never do that.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "svdb_internal.h"

/* ---- row registry: host buffer -> (store, slot) --------------------------- */
typedef struct {
    const double* key; /* NULL: empty; REG_TOMB: deleted */
    svdb_db* db;
    int64_t slot;
} reg_ent;

#define REG_TOMB ((const double*)(uintptr_t)1)

static pthread_rwlock_t g_reg_lock = PTHREAD_RWLOCK_INITIALIZER;
static reg_ent* g_reg = NULL;
static size_t g_reg_cap = 0, g_reg_used = 0; /* used counts live entries and tombstones */

static size_t reg_hash(const double* p, size_t cap) {
    uint64_t x = (uint64_t)(uintptr_t)p >> 3;
    x *= 0x9E3779B97F4A7C15ull;
    return (size_t)(x >> 17) & (cap - 1);
}

static int reg_grow_locked(size_t need) {
    size_t nc = g_reg_cap ? g_reg_cap : 1024;
    while (nc < 2 * need) nc *= 2;
    reg_ent* n = (reg_ent*)calloc(nc, sizeof(reg_ent));
    if (!n) return -1;
    size_t used = 0;
    for (size_t i = 0; i < g_reg_cap; ++i) {
        const reg_ent e = g_reg[i];
        if (!e.key || e.key == REG_TOMB) continue;
        size_t h = reg_hash(e.key, nc);
        while (n[h].key) h = (h + 1) & (nc - 1);
        n[h] = e;
        ++used;
    }
    free(g_reg);
    g_reg = n;
    g_reg_cap = nc;
    g_reg_used = used;
    return 0;
}

void svdb_rows_put(const double* data, svdb_db* d, int64_t slot) {
    if (!data) return;
    pthread_rwlock_wrlock(&g_reg_lock);
    if ((g_reg_used + 1) * 2 > g_reg_cap && reg_grow_locked(g_reg_used + 1) != 0) {
        pthread_rwlock_unlock(&g_reg_lock); /* out of memory: the row is simply not found (copied per call) */
        return;
    }
    size_t h = reg_hash(data, g_reg_cap), tomb = (size_t)-1;
    while (g_reg[h].key) {
        if (g_reg[h].key == data) { /* a buffer reused by the allocator for another row */
            g_reg[h].db = d;
            g_reg[h].slot = slot;
            pthread_rwlock_unlock(&g_reg_lock);
            return;
        }
        if (g_reg[h].key == REG_TOMB && tomb == (size_t)-1) tomb = h;
        h = (h + 1) & (g_reg_cap - 1);
    }
    if (tomb != (size_t)-1) {
        h = tomb;
    } else {
        ++g_reg_used;
    }
    g_reg[h].key = data;
    g_reg[h].db = d;
    g_reg[h].slot = slot;
    pthread_rwlock_unlock(&g_reg_lock);
}

void svdb_rows_drop(const double* data) {
    if (!data) return;
    pthread_rwlock_wrlock(&g_reg_lock);
    if (g_reg_cap) {
        size_t h = reg_hash(data, g_reg_cap);
        while (g_reg[h].key) {
            if (g_reg[h].key == data) {
                g_reg[h].key = REG_TOMB;
                g_reg[h].db = NULL;
                break;
            }
            h = (h + 1) & (g_reg_cap - 1);
        }
    }
    pthread_rwlock_unlock(&g_reg_lock);
}

int svdb_rows_find(const double* data, svdb_db** d, int64_t* slot) {
    int found = 0;
    if (!data) return 0;
    pthread_rwlock_rdlock(&g_reg_lock);
    if (g_reg_cap) {
        size_t h = reg_hash(data, g_reg_cap);
        while (g_reg[h].key) {
            if (g_reg[h].key == data) {
                *d = g_reg[h].db;
                *slot = g_reg[h].slot;
                found = 1;
                break;
            }
            h = (h + 1) & (g_reg_cap - 1);
        }
    }
    pthread_rwlock_unlock(&g_reg_lock);
    return found;
}

/* ---- combining of concurrent calls ---------------------------------------- */
void svdb_combine(svdb_combiner* c, svdb_call* call, svdb_batch_fn fn, void* ctx) {
    pthread_mutex_lock(&c->mu);
    if (c->n == c->cap) {
        size_t nc = c->cap ? 2 * c->cap : 64;
        svdb_call** q = (svdb_call**)realloc(c->q, nc * sizeof(svdb_call*));
        if (!q) { /* no room to queue: answer this call alone */
            pthread_mutex_unlock(&c->mu);
            fn(ctx, &call, 1);
            return;
        }
        c->q = q;
        c->cap = nc;
    }
    c->q[c->n++] = call;
    while (!call->done) {
        if (!c->busy) {
            /* lead: take every queued call, answer them with one launch */
            c->busy = 1;
            size_t n = c->n;
            svdb_call** batch = (svdb_call**)malloc(n * sizeof(svdb_call*));
            if (!batch) { /* answer only this call */
                for (size_t i = 0; i < c->n; ++i)
                    if (c->q[i] == call) {
                        c->q[i] = c->q[--c->n];
                        break;
                    }
                pthread_mutex_unlock(&c->mu);
                fn(ctx, &call, 1);
                pthread_mutex_lock(&c->mu);
                call->done = 1;
            } else {
                memcpy(batch, c->q, n * sizeof(svdb_call*));
                c->n = 0;
                pthread_mutex_unlock(&c->mu);
                fn(ctx, batch, n);
                pthread_mutex_lock(&c->mu);
                for (size_t i = 0; i < n; ++i) batch[i]->done = 1;
                free(batch);
            }
            c->busy = 0;
            pthread_cond_broadcast(&c->cv);
        } else {
            pthread_cond_wait(&c->cv, &c->mu);
        }
    }
    pthread_mutex_unlock(&c->mu);
}
