/*
 * svdb_server.c -- the request path of a batching server over a
 * device-resident store.
 *
 * The drop-in store (svdb_store.c) keeps the reference's host array of
 * Vector structs, because handlers index db->vectors directly
 * (src/get_handler.c:113-114); its delete therefore shifts that array, an
 * O(N) move per request.  A server store keeps rows only in the device store,
 * where a delete is a tombstone, and finds the slot of a position with a
 * Fenwick (binary indexed) tree over slot occupancy: position p is the slot
 * holding the (p+1)-th occupied entry, found in O(log slots).  The device
 * derives the same positions (slot -> rank among occupied slots) for search
 * results, so both sides agree without moving a row.
 */
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "svdb_device.h"

struct svdb_server {
    svdbd_store* st;
    size_t dim;
    size_t nslots; /* slots handed out, device + staged */
    size_t nlive;  /* rows (positions 0..nlive-1) */
    int32_t* fen;  /* Fenwick tree over slots, 1-based, fcap + 1 entries */
    size_t fcap;   /* a power of two */
    pthread_mutex_t mu;
    /* per-batch host scratch */
    double* qbuf;
    size_t qcap;
    int64_t* ibuf;
    double* dbuf;
    size_t ocap;
    int64_t* pairs;
    size_t* pos;
    float* vals;
    size_t pcap;
};

/* ---- order statistics over slots --------------------------------------- */
static int fen_reserve(svdb_server* s, size_t need) {
    if (need <= s->fcap) return SVDB_OK;
    size_t nc = s->fcap ? s->fcap : 1024;
    while (nc < need) nc *= 2;
    int32_t* f = (int32_t*)realloc(s->fen, (nc + 1) * sizeof(int32_t));
    if (!f) {
        svdb_set_error("server: out of host memory for the position index");
        return SVDB_ENOMEM;
    }
    memset(f + s->fcap + 1, 0, (nc - s->fcap) * sizeof(int32_t));
    if (s->fcap == 0) f[0] = 0;
    /* entry j covers slots (j - lowbit(j), j]; for the new powers of two that
     * is every old slot, for every other new entry only new (empty) slots */
    for (size_t c = s->fcap ? s->fcap * 2 : nc + 1; c <= nc; c *= 2) f[c] = (int32_t)s->nlive;
    s->fen = f;
    s->fcap = nc;
    return SVDB_OK;
}

static void fen_add(svdb_server* s, size_t slot, int32_t v) {
    for (size_t j = slot + 1; j <= s->fcap; j += j & (~j + 1)) s->fen[j] += v;
}

/* slot of position p (p < nlive) */
static int64_t fen_slot(const svdb_server* s, size_t p) {
    size_t at = 0;
    int64_t rem = (int64_t)p + 1;
    for (size_t step = s->fcap; step; step >>= 1)
        if (at + step <= s->fcap && s->fen[at + step] < rem) {
            at += step;
            rem -= s->fen[at];
        }
    return (int64_t)at;
}

/* ---- lifetime ----------------------------------------------------------- */
SVDB_API svdb_server* svdb_server_create(size_t dim, size_t reserve_rows) {
    if (dim == 0) {
        svdb_set_error("svdb_server_create: dimension 0");
        return NULL;
    }
    svdb_server* s = (svdb_server*)calloc(1, sizeof(svdb_server));
    if (!s) {
        svdb_set_error("svdb_server_create: out of host memory");
        return NULL;
    }
    s->dim = dim;
    pthread_mutex_init(&s->mu, NULL);
    s->st = svdbd_store_create(dim);
    if (!s->st || fen_reserve(s, reserve_rows ? reserve_rows : 1) ||
        svdbd_store_reserve(s->st, reserve_rows ? reserve_rows : 1)) {
        svdb_server_destroy(s);
        return NULL;
    }
    return s;
}

SVDB_API void svdb_server_destroy(svdb_server* s) {
    if (!s) return;
    if (s->st) svdbd_store_destroy(s->st);
    free(s->fen);
    free(s->qbuf);
    free(s->ibuf);
    free(s->dbuf);
    free(s->pairs);
    free(s->pos);
    free(s->vals);
    pthread_mutex_destroy(&s->mu);
    free(s);
}

SVDB_API size_t svdb_server_size(svdb_server* s) {
    if (!s) return 0;
    pthread_mutex_lock(&s->mu);
    size_t n = s->nlive;
    pthread_mutex_unlock(&s->mu);
    return n;
}

SVDB_API int svdb_server_insert_block(svdb_server* s, const double* rows, size_t n, size_t* first_index) {
    return svdb_server_insert_rows(s, rows, NULL, n, first_index);
}

SVDB_API int svdb_server_insert_rows(svdb_server* s, const double* rows, const char* uuids, size_t n,
                                     size_t* first_index) {
    if (!s || (n && !rows)) {
        svdb_set_error("svdb_server_insert_rows: NULL argument");
        return SVDB_EINVAL;
    }
    pthread_mutex_lock(&s->mu);
    if (first_index) *first_index = s->nlive;
    int rc = fen_reserve(s, s->nslots + n);
    if (!rc && n) rc = svdbd_store_append_block(s->st, rows, n);
    for (size_t i = 0; i < n && !rc && uuids; ++i)
        if (uuids[i * 37]) rc = svdbd_store_set_uuid(s->st, (int64_t)(s->nslots + i), uuids + i * 37);
    if (!rc) {
        for (size_t i = 0; i < n; ++i) fen_add(s, s->nslots + i, 1);
        s->nslots += n;
        s->nlive += n;
    }
    pthread_mutex_unlock(&s->mu);
    return rc;
}

SVDB_API int svdb_server_read(svdb_server* s, size_t index, double* out) {
    if (!s || !out) {
        svdb_set_error("svdb_server_read: NULL argument");
        return SVDB_EINVAL;
    }
    pthread_mutex_lock(&s->mu);
    int rc;
    if (index >= s->nlive) {
        svdb_set_error("svdb_server_read: index %zu out of bounds (size %zu)", index, s->nlive);
        rc = SVDB_EINVAL;
    } else {
        rc = svdbd_store_read_row(s->st, fen_slot(s, index), out);
    }
    pthread_mutex_unlock(&s->mu);
    return rc;
}

/* ---- one batch ---------------------------------------------------------- */
static int grow_scratch(void** p, size_t* cap, size_t need, size_t elem) {
    (void)cap;
    void* q = realloc(*p, (need ? need : 1) * elem);
    if (!q) {
        svdb_set_error("server: out of host memory for batch scratch");
        return SVDB_ENOMEM;
    }
    *p = q;
    return SVDB_OK;
}

static int batch_scratch(svdb_server* s, size_t nq, size_t kmax, size_t npairs) {
    int rc = SVDB_OK;
    if (nq * s->dim > s->qcap) {
        rc = grow_scratch((void**)&s->qbuf, &s->qcap, nq * s->dim, sizeof(double));
        if (rc) return rc;
        s->qcap = nq * s->dim;
    }
    if (nq * kmax > s->ocap) {
        rc = grow_scratch((void**)&s->ibuf, &s->ocap, nq * kmax, sizeof(int64_t));
        if (!rc) rc = grow_scratch((void**)&s->dbuf, &s->ocap, nq * kmax, sizeof(double));
        if (rc) return rc;
        s->ocap = nq * kmax;
    }
    if (npairs > s->pcap) {
        rc = grow_scratch((void**)&s->pairs, &s->pcap, 2 * npairs, sizeof(int64_t));
        if (!rc) rc = grow_scratch((void**)&s->pos, &s->pcap, npairs, sizeof(size_t));
        if (!rc) rc = grow_scratch((void**)&s->vals, &s->pcap, npairs, sizeof(float));
        if (rc) return rc;
        s->pcap = npairs;
    }
    return SVDB_OK;
}

static void add_stats(svdb_search_stats* acc, const svdb_search_stats* st) {
    acc->candidates += st->candidates;
    acc->survivors += st->survivors;
    acc->reranked += st->reranked;
    acc->widened += st->widened;
    acc->kernels += st->kernels;
    acc->bound_failures += st->bound_failures;
    if (st->max_err_bound > acc->max_err_bound) acc->max_err_bound = st->max_err_bound;
}

SVDB_API int svdb_server_execute(svdb_server* s, const svdb_request* req, size_t n, svdb_response* resp,
                                 int precision, int64_t* ids, double* dists, size_t stride,
                                 svdb_search_stats* stats) {
    if (!s || (n && (!req || !resp))) {
        svdb_set_error("svdb_server_execute: NULL argument");
        return SVDB_EINVAL;
    }
    if (stats) memset(stats, 0, sizeof(*stats));
    pthread_mutex_lock(&s->mu);
    int rc = SVDB_OK;
    size_t n_ins = 0, n_near = 0, n_cmp = 0, kmax = 0;
    for (size_t i = 0; i < n; ++i) {
        resp[i].status = 0;
        resp[i].value = NAN;
        resp[i].index = 0;
        switch (req[i].op) {
            case SVDB_REQ_INSERT:
                n_ins++;
                break;
            case SVDB_REQ_NEAREST:
                if (req[i].k == 0 || req[i].k > 128 || req[i].k > stride || !req[i].vec || !ids || !dists ||
                    req[i].metric < 0 || req[i].metric > 2) {
                    resp[i].status = SVDB_EINVAL;
                } else {
                    n_near++;
                    if (req[i].k > kmax) kmax = req[i].k;
                }
                break;
            case SVDB_REQ_COMPARE:
                n_cmp++;
                break;
            case SVDB_REQ_UPDATE:
            case SVDB_REQ_DELETE:
                break;
            default:
                resp[i].status = SVDB_EINVAL;
        }
    }
    /* admission: the batch's inserts go in only if HBM holds all of them */
    int admit = 1;
    if (n_ins) {
        if (fen_reserve(s, s->nslots + n_ins) || svdbd_store_reserve(s->st, s->nslots + n_ins)) admit = 0;
    }
    /* mutations, in request order */
    for (size_t i = 0; i < n && !rc; ++i) {
        const svdb_request* r = &req[i];
        svdb_response* o = &resp[i];
        if (r->op == SVDB_REQ_INSERT) {
            if (!r->vec) {
                o->status = SVDB_EINVAL;
            } else if (!admit) {
                o->status = SVDB_ENOMEM;
            } else {
                rc = svdbd_store_append(s->st, &r->vec, NULL, 1);
                if (!rc && r->uuid && r->uuid[0]) rc = svdbd_store_set_uuid(s->st, (int64_t)s->nslots, r->uuid);
                if (!rc) {
                    fen_add(s, s->nslots++, 1);
                    o->index = s->nlive++;
                }
            }
        } else if (r->op == SVDB_REQ_UPDATE || r->op == SVDB_REQ_DELETE) {
            if (r->a >= s->nlive) {
                o->status = SVDB_CMP_OUT_OF_BOUNDS;
            } else if (r->op == SVDB_REQ_UPDATE && !r->vec) {
                o->status = SVDB_EINVAL;
            } else {
                const int64_t slot = fen_slot(s, (size_t)r->a);
                if (r->op == SVDB_REQ_UPDATE) {
                    rc = svdbd_store_overwrite(s->st, slot, r->vec, 1);
                    if (!rc && r->uuid) rc = svdbd_store_set_uuid(s->st, slot, r->uuid);
                } else {
                    rc = svdbd_store_kill(s->st, slot);
                    if (!rc) {
                        fen_add(s, (size_t)slot, -1);
                        s->nlive--;
                    }
                }
            }
        }
    }
    if (!rc && (n_near || n_cmp)) rc = svdbd_store_sync(s->st);
    if (!rc) rc = batch_scratch(s, n_near, kmax, n_cmp);
    /* NEAREST: one search per (metric, k) */
    uint8_t* done = NULL;
    if (!rc && n_near) {
        done = (uint8_t*)calloc(n, 1);
        if (!done) {
            svdb_set_error("server: out of host memory");
            rc = SVDB_ENOMEM;
        }
    }
    for (size_t i = 0; i < n && !rc && n_near; ++i) {
        if (req[i].op != SVDB_REQ_NEAREST || resp[i].status || done[i]) continue;
        const int metric = req[i].metric;
        const uint32_t k = req[i].k;
        size_t m = 0;
        for (size_t j = i; j < n; ++j)
            if (req[j].op == SVDB_REQ_NEAREST && !resp[j].status && !done[j] && req[j].metric == metric &&
                req[j].k == k) {
                memcpy(s->qbuf + m * s->dim, req[j].vec, s->dim * sizeof(double));
                m++;
            }
        svdb_search_stats st;
        rc = svdbd_search(s->st, s->qbuf, m, k, metric, precision, s->ibuf, s->dbuf, NULL, 0, stats ? &st : NULL);
        if (rc) break;
        if (stats) add_stats(stats, &st);
        size_t t = 0;
        for (size_t j = i; j < n; ++j)
            if (req[j].op == SVDB_REQ_NEAREST && !resp[j].status && !done[j] && req[j].metric == metric &&
                req[j].k == k) {
                memcpy(ids + j * stride, s->ibuf + t * k, k * sizeof(int64_t));
                memcpy(dists + j * stride, s->dbuf + t * k, k * sizeof(double));
                done[j] = 1;
                t++;
            }
    }
    free(done);
    /* COMPARE: one pair kernel per metric */
    for (int metric = 0; metric < 3 && !rc && n_cmp; ++metric) {
        size_t m = 0;
        for (size_t i = 0; i < n; ++i) {
            if (req[i].op != SVDB_REQ_COMPARE || req[i].metric != metric) continue;
            if (req[i].a >= s->nlive || req[i].b >= s->nlive) {
                resp[i].status = SVDB_CMP_OUT_OF_BOUNDS;
                continue;
            }
            s->pairs[m] = fen_slot(s, (size_t)req[i].a);
            s->pairs[n_cmp + m] = fen_slot(s, (size_t)req[i].b);
            s->pos[m++] = i;
        }
        if (!m) continue;
        rc = svdbd_compare_slots(s->st, metric, s->pairs, s->pairs + n_cmp, m, s->vals);
        for (size_t j = 0; j < m && !rc; ++j) resp[s->pos[j]].value = s->vals[j];
    }
    /* the handler checks the indices before the method (src/compare_handler.c:101,161) */
    for (size_t i = 0; i < n; ++i)
        if (req[i].op == SVDB_REQ_COMPARE && (req[i].metric < 0 || req[i].metric > 2))
            resp[i].status = (req[i].a >= s->nlive || req[i].b >= s->nlive) ? SVDB_CMP_OUT_OF_BOUNDS
                                                                             : SVDB_CMP_UNKNOWN_METHOD;
    pthread_mutex_unlock(&s->mu);
    return rc;
}

/* ---- uuid lookups and persistence --------------------------------------- */
SVDB_API int svdb_server_find_uuid(svdb_server* s, const char* uuids, size_t n, int64_t* out_index) {
    if (!s || (n && (!uuids || !out_index))) {
        svdb_set_error("svdb_server_find_uuid: NULL argument");
        return SVDB_EINVAL;
    }
    pthread_mutex_lock(&s->mu);
    int rc = svdbd_uuid_find(s->st, uuids, n, out_index);
    pthread_mutex_unlock(&s->mu);
    return rc;
}

/* rows read back from HBM in blocks of this many slots */
#define SERVER_IO_BLOCK 16384

SVDB_API int svdb_server_save(svdb_server* s, const char* filename) {
    if (!s || !filename) {
        svdb_set_error("svdb_server_save: NULL argument");
        return SVDB_EINVAL;
    }
    pthread_mutex_lock(&s->mu);
    int rc = SVDB_OK;
    const size_t blk = SERVER_IO_BLOCK;
    double* rows = (double*)malloc(blk * s->dim * sizeof(double));
    char* uu = (char*)malloc(blk * 37);
    uint8_t* lv = (uint8_t*)malloc(blk);
    FILE* f = fopen(filename, "wb");
    if (!rows || !uu || !lv || !f) {
        svdb_set_error(f ? "svdb_server_save: out of host memory" : "svdb_server_save: cannot open the file");
        rc = f ? SVDB_ENOMEM : SVDB_EINVAL;
    }
    if (!rc) {
        const size_t n = s->nlive, dim = s->dim;
        size_t written = 0;
        if (fwrite(&n, sizeof(size_t), 1, f) != 1) rc = SVDB_EINVAL;
        for (size_t first = 0; first < s->nslots && !rc; first += blk) {
            const size_t m = s->nslots - first < blk ? s->nslots - first : blk;
            rc = svdbd_store_read_block(s->st, (int64_t)first, m, rows, uu, lv);
            for (size_t i = 0; i < m && !rc; ++i) {
                if (!lv[i]) continue;
                if (fwrite(uu + i * 37, 1, 37, f) != 37 || fwrite(&dim, sizeof(size_t), 1, f) != 1 ||
                    fwrite(rows + i * dim, sizeof(double), dim, f) != dim)
                    rc = SVDB_EINVAL;
                written++;
            }
        }
        if (!rc && written != n) {
            svdb_set_error("svdb_server_save: %zu rows written, %zu expected", written, n);
            rc = SVDB_ECUDA;
        } else if (rc == SVDB_EINVAL) {
            svdb_set_error("svdb_server_save: write error");
        }
    }
    if (f && fclose(f) != 0 && !rc) {
        svdb_set_error("svdb_server_save: write error");
        rc = SVDB_EINVAL;
    }
    free(rows);
    free(uu);
    free(lv);
    pthread_mutex_unlock(&s->mu);
    return rc;
}

SVDB_API svdb_server* svdb_server_load(const char* filename, size_t dim, size_t reserve_rows) {
    if (!filename || dim == 0) {
        svdb_set_error("svdb_server_load: NULL file name or dimension 0");
        return NULL;
    }
    FILE* f = fopen(filename, "rb");
    if (!f) {
        svdb_set_error("svdb_server_load: cannot open the file");
        return NULL;
    }
    size_t n = 0;
    if (fread(&n, sizeof(size_t), 1, f) != 1) n = 0;
    const size_t rowbytes = 37 + sizeof(size_t) + dim * sizeof(double);
    long long avail = -1; /* rows the file can hold at most (a bad count cannot reserve absurd memory) */
    if (fseek(f, 0, SEEK_END) == 0) {
        const long end = ftell(f);
        if (end >= 8) avail = (long long)((size_t)(end - 8) / rowbytes);
        fseek(f, 8, SEEK_SET);
    }
    if (avail >= 0 && (size_t)avail < n) {
        fprintf(stderr, "svdb_server_load: the file counts %zu rows but holds %lld (truncated file)\n", n, avail);
        n = (size_t)avail;
    }
    svdb_server* s = svdb_server_create(dim, n + reserve_rows);
    if (!s) {
        fclose(f);
        return NULL;
    }
    /* blocks of about 64 MB of file bytes */
    size_t blk = ((size_t)64 << 20) / rowbytes;
    if (blk == 0) blk = 1;
    uint8_t* buf = (uint8_t*)malloc(blk * rowbytes);
    int rc = buf ? SVDB_OK : SVDB_ENOMEM;
    if (rc) svdb_set_error("svdb_server_load: out of host memory");
    size_t done = 0;
    while (!rc && done < n) {
        const size_t want = n - done < blk ? n - done : blk;
        const size_t got = fread(buf, rowbytes, want, f);
        size_t m = 0;
        for (; m < got; ++m) { /* every row must have the store's dimension */
            size_t d = 0;
            memcpy(&d, buf + m * rowbytes + 37, sizeof(size_t));
            if (d != dim) break;
        }
        if (m < got) {
            svdb_set_error("svdb_server_load: row %zu has dimension != %zu", done + m, dim);
            rc = SVDB_EINVAL;
        }
        if (m) {
            pthread_mutex_lock(&s->mu);
            int r = fen_reserve(s, s->nslots + m);
            if (!r) r = svdbd_store_append_raw(s->st, buf, m, rowbytes);
            if (!r) {
                for (size_t i = 0; i < m; ++i) fen_add(s, s->nslots + i, 1);
                s->nslots += m;
                s->nlive += m;
            }
            pthread_mutex_unlock(&s->mu);
            if (r && !rc) rc = r;
        }
        done += m;
        if (!rc && got < want) {
            fprintf(stderr, "svdb_server_load: truncated file at row %zu\n", done);
            break;
        }
    }
    free(buf);
    fclose(f);
    if (rc) {
        svdb_server_destroy(s);
        return NULL;
    }
    return s;
}
