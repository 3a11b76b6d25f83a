/*
 * svdb_oracle.c -- CPU oracle for the similarity path of simple-vector-db.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library links, loads or
 * calls this file; only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg do, and only as the checker.
 *
 * It restates, in plain C, the arithmetic of the reference's hot path:
 *
 *   orc_ref_cosine / orc_ref_euclidean / orc_ref_dot
 *       src/vector_database.c:301-313, :322-333, :342-352 -- FP64 inputs,
 *       FLOAT accumulators; every "acc += a*b" is a double product and a
 *       double add rounded back to float.  Must be compiled with
 *       -ffp-contract=off (the reference ships at -O0, where GCC never
 *       contracts; at -O2 on aarch64 it would fuse and change the bits).
 *
 *   orc_kd_*      src/kdtree.c:15-178 -- the insertion-order KD tree over the
 *       first `dim` coordinates: split axis depth % dim, "<" goes left
 *       (:53-59); exact 1-NN with strict "<" replacement (:139) and the
 *       plane prune (q[cd]-p[cd])^2 < best (:157); (size_t)-1 when empty
 *       (:171-174).
 *
 *   orc_store_*   src/vector_database.c:81-195 -- positional store:
 *       insert appends and adds a KD node with index = size (:113-115);
 *       update replaces the row and adds a SECOND KD node (:169-177);
 *       delete shifts later rows left and leaves the KD tree alone
 *       (:185-195); out-of-range update/delete are ignored.
 *
 *   orc_fp64_*    the same three metric formulas carried in double.  Two
 *       summation orders are provided: `seq` (i = 0..d-1, as the reference
 *       loops) and `canon`, the order the GPU kernels use (element i goes to
 *       partial sum (i/2)%4 with a fused multiply-add, result
 *       (p0+p2)+(p1+p3)); both are exact restatements of the formulas, and
 *       they agree to ~1e-16 relative.
 *
 *   orc_topk      FP64 brute force top-k (no reference symbol: /nearest is
 *       top-1 only); order = (key ascending, id ascending) where key is the
 *       distance for Euclidean and the negated value for cosine/dot, NaN
 *       ranked last.
 *
 *   orc_decode_body  src/compare_handler.c:300-390 -- the checks the /nearest
 *       handler makes on its body through cJSON (the third-party JSON
 *       library the reference links; version not pinned, restated from the
 *       published cJSON 1.7 sources): cJSON_Parse of the text (whitespace =
 *       bytes <= 32, a UTF-8 BOM skipped, content after the value ignored,
 *       nesting up to 1000, cJSON's string escapes, numbers = strtod on the
 *       run of [0-9+-eE.] characters, at most 63), then the child count
 *       against dim, then every child a number.  Numbers come from the C
 *       library's strtod itself, as in cJSON.
 *
 *   orc_format_*  src/compare_handler.c:180-185 and :409-424 -- the response
 *       bodies the handlers print with cJSON_PrintUnformatted.  cJSON's
 *       number rule (published 1.7 sources, restated): "null" for NaN or an
 *       infinity; the decimal integer when the value equals its int
 *       conversion (clamped to INT_MIN..INT_MAX); else the text of "%1.15g"
 *       if strtod of it is within DBL_EPSILON (relative to the larger
 *       magnitude) of the value, else "%1.17g".  Strings are quoted with
 *       '"' and '\' escaped, \b \f \n \r \t for those bytes and \u00xx
 *       for other bytes below 32.  The digits come from the C library's own
 *       printf and strtod, as in cJSON.
 *
 *   orc_find_uuid src/vector_database.c:145-158 -- the linear scan of
 *       vector_db_read_by_uuid: first row whose uuid[37] equals the key
 *       under strncmp(.., 37); n keys, each scanned independently, spread
 *       over `threads` threads.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_COSINE 0
#define ORC_EUCLIDEAN 1
#define ORC_DOT 2

/* ------------------------------------------------------------------------ */
/* Reference-exact metrics (float accumulators).                             */
/* ------------------------------------------------------------------------ */

float orc_ref_cosine(const double* a, const double* b, size_t d) {
    float dot = 0.0f, na = 0.0f, nb = 0.0f;
    for (size_t i = 0; i < d; ++i) {
        dot = (float)((double)dot + a[i] * b[i]);
        na = (float)((double)na + a[i] * a[i]);
        nb = (float)((double)nb + b[i] * b[i]);
    }
    return (float)((double)dot / (sqrt((double)na) * sqrt((double)nb)));
}

float orc_ref_euclidean(const double* a, const double* b, size_t d) {
    float sum = 0.0f;
    for (size_t i = 0; i < d; ++i) {
        float diff = (float)(a[i] - b[i]);
        sum = sum + diff * diff;
    }
    return (float)sqrt((double)sum);
}

float orc_ref_dot(const double* a, const double* b, size_t d) {
    float r = 0.0f;
    for (size_t i = 0; i < d; ++i) r = (float)((double)r + a[i] * b[i]);
    return r;
}

/* metric on two vectors of possibly different dimension: -1.0f on mismatch,
 * as every metric in src/vector_database.c:302-305 does. */
float orc_ref_metric(int metric, const double* a, size_t da, const double* b, size_t db) {
    if (da != db) return -1.0f;
    switch (metric) {
        case ORC_COSINE: return orc_ref_cosine(a, b, da);
        case ORC_EUCLIDEAN: return orc_ref_euclidean(a, b, da);
        default: return orc_ref_dot(a, b, da);
    }
}

/* ------------------------------------------------------------------------ */
/* FP64 metrics.                                                             */
/* ------------------------------------------------------------------------ */

static double canon_dot(const double* a, const double* b, size_t d) {
    double p[4] = {0.0, 0.0, 0.0, 0.0};
    for (size_t i = 0; i < d; ++i) {
        size_t s = (i >> 1) & 3u;
        p[s] = fma(a[i], b[i], p[s]);
    }
    return (p[0] + p[2]) + (p[1] + p[3]);
}

static double canon_sqdist(const double* a, const double* b, size_t d) {
    double p[4] = {0.0, 0.0, 0.0, 0.0};
    for (size_t i = 0; i < d; ++i) {
        size_t s = (i >> 1) & 3u;
        double t = a[i] - b[i];
        p[s] = fma(t, t, p[s]);
    }
    return (p[0] + p[2]) + (p[1] + p[3]);
}

double orc_canon_sumsq(const double* a, size_t d) { return canon_dot(a, a, d); }

/* FP64 metric value in the canonical order; qn/xn are sqrt(canon sumsq). */
static double canon_metric(int metric, const double* q, double qn, const double* x, double xn, size_t d) {
    switch (metric) {
        case ORC_COSINE: return canon_dot(q, x, d) / (qn * xn);
        case ORC_EUCLIDEAN: return sqrt(canon_sqdist(q, x, d));
        default: return canon_dot(q, x, d);
    }
}

double orc_fp64_canon(int metric, const double* a, const double* b, size_t d) {
    double an = sqrt(canon_dot(a, a, d)), bn = sqrt(canon_dot(b, b, d));
    return canon_metric(metric, a, an, b, bn, d);
}

double orc_fp64_seq(int metric, const double* a, const double* b, size_t d) {
    double dot = 0.0, na = 0.0, nb = 0.0, sq = 0.0;
    for (size_t i = 0; i < d; ++i) {
        dot += a[i] * b[i];
        na += a[i] * a[i];
        nb += b[i] * b[i];
        double t = a[i] - b[i];
        sq += t * t;
    }
    switch (metric) {
        case ORC_COSINE: return dot / (sqrt(na) * sqrt(nb));
        case ORC_EUCLIDEAN: return sqrt(sq);
        default: return dot;
    }
}

/* ------------------------------------------------------------------------ */
/* FP64 brute-force top-k.                                                   */
/* ------------------------------------------------------------------------ */

static double rank_key(int metric, double v) {
    if (isnan(v)) return INFINITY;
    return metric == ORC_EUCLIDEAN ? v : -v;
}

typedef struct {
    int metric, seq;
    const double* x;
    const double* xn;
    size_t n, d, k;
    const double* q;
    size_t nq;
    int64_t* ids;
    double* vals;
    size_t next;
    pthread_mutex_t lock;
} topk_job;

static void topk_one(topk_job* J, size_t qi, double* keys, int64_t* kid, double* kval) {
    const double* q = J->q + qi * J->d;
    double qn = sqrt(canon_dot(q, q, J->d));
    size_t cnt = 0;
    for (size_t r = 0; r < J->n; ++r) {
        const double* x = J->x + r * J->d;
        double v = J->seq ? orc_fp64_seq(J->metric, q, x, J->d)
                          : canon_metric(J->metric, q, qn, x, J->xn[r], J->d);
        double key = rank_key(J->metric, v);
        if (cnt == J->k && !(key < keys[cnt - 1])) continue; /* ids ascend: equal key loses */
        size_t pos = cnt < J->k ? cnt++ : J->k - 1;
        while (pos > 0 && key < keys[pos - 1]) {
            keys[pos] = keys[pos - 1];
            kid[pos] = kid[pos - 1];
            kval[pos] = kval[pos - 1];
            --pos;
        }
        keys[pos] = key;
        kid[pos] = (int64_t)r;
        kval[pos] = v;
    }
    for (size_t j = 0; j < J->k; ++j) {
        J->ids[qi * J->k + j] = j < cnt ? kid[j] : -1;
        J->vals[qi * J->k + j] = j < cnt ? kval[j] : NAN;
    }
}

static void* topk_worker(void* arg) {
    topk_job* J = (topk_job*)arg;
    double* keys = (double*)malloc(J->k * sizeof(double));
    int64_t* kid = (int64_t*)malloc(J->k * sizeof(int64_t));
    double* kval = (double*)malloc(J->k * sizeof(double));
    for (;;) {
        pthread_mutex_lock(&J->lock);
        size_t qi = J->next++;
        pthread_mutex_unlock(&J->lock);
        if (qi >= J->nq) break;
        topk_one(J, qi, keys, kid, kval);
    }
    free(keys);
    free(kid);
    free(kval);
    return NULL;
}

/* Exact FP64 top-k of every query against all n rows.  seq=0: canonical
 * summation order (bit-identical to the GPU kernels); seq=1: sequential. */
int orc_topk(int metric, int seq, const double* x, size_t n, size_t d, const double* q, size_t nq,
             size_t k, int64_t* ids, double* vals, int nthreads) {
    if (k == 0) return 0;
    double* xn = (double*)malloc((n ? n : 1) * sizeof(double));
    if (!xn) return -1;
    for (size_t r = 0; r < n; ++r) xn[r] = sqrt(canon_dot(x + r * d, x + r * d, d));
    topk_job J = {metric, seq, x, xn, n, d, k, q, nq, ids, vals, 0, PTHREAD_MUTEX_INITIALIZER};
    if (nthreads < 1) nthreads = 1;
    pthread_t* th = (pthread_t*)malloc((size_t)nthreads * sizeof(pthread_t));
    int started = 0;
    for (int t = 1; t < nthreads; ++t)
        if (pthread_create(&th[started], NULL, topk_worker, &J) == 0) ++started;
    topk_worker(&J);
    for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
    free(th);
    free(xn);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Insertion-order KD tree (flat arrays).                                    */
/* ------------------------------------------------------------------------ */

typedef struct {
    size_t dim, n, cap;
    double* pts;   /* n * dim prefix copies (src/kdtree.c:26-28) */
    size_t* index; /* stored index (src/kdtree.c:30) */
    int64_t* left;
    int64_t* right;
} orc_kd;

orc_kd* orc_kd_create(size_t dim) {
    orc_kd* t = (orc_kd*)calloc(1, sizeof(orc_kd));
    if (t) t->dim = dim;
    return t;
}

void orc_kd_free(orc_kd* t) {
    if (!t) return;
    free(t->pts);
    free(t->index);
    free(t->left);
    free(t->right);
    free(t);
}

int orc_kd_insert(orc_kd* t, const double* p, size_t index) {
    if (t->n == t->cap) {
        size_t nc = t->cap ? 2 * t->cap : 64;
        double* np = (double*)realloc(t->pts, nc * t->dim * sizeof(double));
        if (!np) return -1;
        t->pts = np;
        size_t* ni = (size_t*)realloc(t->index, nc * sizeof(size_t));
        if (!ni) return -1;
        t->index = ni;
        int64_t* nl = (int64_t*)realloc(t->left, nc * sizeof(int64_t));
        if (!nl) return -1;
        t->left = nl;
        int64_t* nr = (int64_t*)realloc(t->right, nc * sizeof(int64_t));
        if (!nr) return -1;
        t->right = nr;
        t->cap = nc;
    }
    int64_t id = (int64_t)t->n++;
    memcpy(t->pts + (size_t)id * t->dim, p, t->dim * sizeof(double));
    t->index[id] = index;
    t->left[id] = t->right[id] = -1;
    if (id == 0) return 0;
    int64_t cur = 0;
    size_t depth = 0;
    for (;;) {
        size_t cd = depth % t->dim;
        int64_t* slot = p[cd] < t->pts[(size_t)cur * t->dim + cd] ? &t->left[cur] : &t->right[cur];
        if (*slot < 0) {
            *slot = id;
            return 0;
        }
        cur = *slot;
        ++depth;
    }
}

static void kd_nearest_rec(const orc_kd* t, int64_t node, const double* q, size_t depth, int64_t* best,
                           double* best_d) {
    if (node < 0) return;
    const double* p = t->pts + (size_t)node * t->dim;
    double d = 0.0;
    for (size_t i = 0; i < t->dim; ++i) d += (p[i] - q[i]) * (p[i] - q[i]);
    if (d < *best_d) {
        *best_d = d;
        *best = node;
    }
    size_t cd = depth % t->dim;
    int64_t nxt, oth;
    if (q[cd] < p[cd]) {
        nxt = t->left[node];
        oth = t->right[node];
    } else {
        nxt = t->right[node];
        oth = t->left[node];
    }
    kd_nearest_rec(t, nxt, q, depth + 1, best, best_d);
    if ((q[cd] - p[cd]) * (q[cd] - p[cd]) < *best_d) kd_nearest_rec(t, oth, q, depth + 1, best, best_d);
}

size_t orc_kd_nearest(const orc_kd* t, const double* q) {
    if (!t || t->n == 0) return (size_t)-1;
    int64_t best = -1;
    double best_d = INFINITY;
    kd_nearest_rec(t, 0, q, 0, &best, &best_d);
    return best >= 0 ? t->index[best] : (size_t)-1;
}

size_t orc_kd_size(const orc_kd* t) { return t->n; }

/* ------------------------------------------------------------------------ */
/* Positional store with the reference's mutation semantics.                 */
/* ------------------------------------------------------------------------ */

typedef struct {
    size_t d, size, cap;
    double* rows; /* size * d, logical order */
    orc_kd* kd;
} orc_store;

orc_store* orc_store_create(size_t d, size_t kd_dim) {
    orc_store* s = (orc_store*)calloc(1, sizeof(orc_store));
    if (!s) return NULL;
    s->d = d;
    s->kd = orc_kd_create(kd_dim);
    return s;
}

void orc_store_free(orc_store* s) {
    if (!s) return;
    free(s->rows);
    orc_kd_free(s->kd);
    free(s);
}

size_t orc_store_insert(orc_store* s, const double* v) {
    if (s->size == s->cap) {
        size_t nc = s->cap ? 2 * s->cap : 16;
        double* nr = (double*)realloc(s->rows, nc * s->d * sizeof(double));
        if (!nr) return (size_t)-1;
        s->rows = nr;
        s->cap = nc;
    }
    memcpy(s->rows + s->size * s->d, v, s->d * sizeof(double));
    orc_kd_insert(s->kd, v, s->size);
    return s->size++;
}

void orc_store_update(orc_store* s, size_t index, const double* v) {
    if (index >= s->size) return;
    memcpy(s->rows + index * s->d, v, s->d * sizeof(double));
    orc_kd_insert(s->kd, v, index);
}

void orc_store_delete(orc_store* s, size_t index) {
    if (index >= s->size) return;
    memmove(s->rows + index * s->d, s->rows + (index + 1) * s->d, (s->size - index - 1) * s->d * sizeof(double));
    s->size--;
}

size_t orc_store_size(const orc_store* s) { return s->size; }
const double* orc_store_rows(const orc_store* s) { return s->rows; }

/* /nearest as src/compare_handler.c:403-419 resolves it: the KD index, or
 * (size_t)-1 for "No nearest neighbor found"; an index >= size is the
 * "Nearest neighbor not found" outcome (the row was deleted). */
size_t orc_store_nearest(const orc_store* s, const double* q) { return orc_kd_nearest(s->kd, q); }

/* ---- uuid lookup (src/vector_database.c:145-158) ------------------------ */
typedef struct {
    const char* table; /* n x 37 */
    size_t n;
    const char* keys; /* nk x 37 */
    size_t nk;
    int64_t* out;
    int threads, t;
} uuid_job;

static void* uuid_worker(void* arg) {
    uuid_job* J = (uuid_job*)arg;
    for (size_t q = (size_t)J->t; q < J->nk; q += (size_t)J->threads) {
        J->out[q] = -1;
        for (size_t i = 0; i < J->n; ++i)
            if (strncmp(J->table + i * 37, J->keys + q * 37, 37) == 0) {
                J->out[q] = (int64_t)i;
                break;
            }
    }
    return NULL;
}

int orc_find_uuid(const char* table, size_t n, const char* keys, size_t nk, int64_t* out, int threads) {
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    pthread_t th[256];
    uuid_job J[256];
    for (int t = 0; t < threads; ++t) {
        J[t] = (uuid_job){table, n, keys, nk, out, threads, t};
        if (pthread_create(&th[t], NULL, uuid_worker, &J[t]) != 0) return -1;
    }
    for (int t = 0; t < threads; ++t) pthread_join(th[t], NULL);
    return 0;
}

/* ---- /nearest body decode (cJSON_Parse + the handler's checks) ----------- */
#include <stdio.h>

typedef struct {
    const unsigned char* p;
    size_t n; /* bytes before the first NUL */
    size_t i;
    int depth;
} jcur;

static void jws(jcur* c) {
    while (c->i < c->n && c->p[c->i] <= 32) c->i++;
}

static int jhex(unsigned char ch) {
    if (ch >= '0' && ch <= '9') return ch - '0';
    if (ch >= 'A' && ch <= 'F') return ch - 'A' + 10;
    if (ch >= 'a' && ch <= 'f') return ch - 'a' + 10;
    return -1;
}

static unsigned jhex4(const unsigned char* s) {
    unsigned h = 0;
    for (int k = 0; k < 4; ++k) {
        int v = jhex(s[k]);
        if (v < 0) return 0;
        h = (h << 4) | (unsigned)v;
    }
    return h;
}

static int jstring(jcur* c) {
    if (c->i >= c->n || c->p[c->i] != '"') return 0;
    size_t e = c->i + 1;
    while (e < c->n && c->p[e] != '"') {
        if (c->p[e] == '\\') {
            if (e + 1 >= c->n) return 0;
            e++;
        }
        e++;
    }
    if (e >= c->n) return 0;
    for (size_t k = c->i + 1; k < e;) {
        if (c->p[k] != '\\') {
            k++;
            continue;
        }
        unsigned char x = c->p[k + 1];
        if (strchr("bfnrt\"\\/", x) && x) {
            k += 2;
        } else if (x == 'u') {
            if (e - k < 6) return 0;
            unsigned a = jhex4(c->p + k + 2);
            if (a >= 0xDC00 && a <= 0xDFFF) return 0;
            if (a >= 0xD800 && a <= 0xDBFF) {
                if (e - (k + 6) < 6 || c->p[k + 6] != '\\' || c->p[k + 7] != 'u') return 0;
                unsigned b = jhex4(c->p + k + 8);
                if (b < 0xDC00 || b > 0xDFFF) return 0;
                k += 12;
            } else {
                k += 6;
            }
        } else {
            return 0;
        }
    }
    c->i = e + 1;
    return 1;
}

/* one value; *is_num: it was a number, *num: its value */
static int jvalue(jcur* c, int* is_num, double* num, size_t* nchild, size_t dim, double* out, int* bad, int top);

static int jnumber(jcur* c, double* v) {
    char buf[64];
    size_t k = 0;
    while (k < 63 && c->i + k < c->n && strchr("0123456789+-eE.", c->p[c->i + k]) && c->p[c->i + k]) {
        buf[k] = (char)c->p[c->i + k];
        k++;
    }
    buf[k] = 0;
    char* end = NULL;
    *v = strtod(buf, &end);
    if (end == buf) return 0;
    c->i += (size_t)(end - buf);
    return 1;
}

static int jcontainer(jcur* c, int obj, size_t* nchild, size_t dim, double* out, int* bad, int top) {
    if (c->depth >= 1000) return 0;
    c->depth++;
    c->i++;
    jws(c);
    if (c->i < c->n && c->p[c->i] == (obj ? '}' : ']')) {
        c->i++;
        c->depth--;
        return 1;
    }
    for (;;) {
        jws(c);
        if (obj) {
            if (!jstring(c)) return 0;
            jws(c);
            if (c->i >= c->n || c->p[c->i] != ':') return 0;
            c->i++;
            jws(c);
        }
        int isn = 0;
        double v = 0;
        if (!jvalue(c, &isn, &v, NULL, 0, NULL, NULL, 0)) return 0;
        if (top) {
            if (*nchild < dim) {
                out[*nchild] = v;
                if (!isn) *bad = 1;
            }
            (*nchild)++;
        }
        jws(c);
        if (c->i < c->n && c->p[c->i] == ',') {
            c->i++;
            continue;
        }
        if (c->i < c->n && c->p[c->i] == (obj ? '}' : ']')) {
            c->i++;
            c->depth--;
            return 1;
        }
        return 0;
    }
}

static int jvalue(jcur* c, int* is_num, double* num, size_t* nchild, size_t dim, double* out, int* bad, int top) {
    *is_num = 0;
    if (c->i >= c->n) return 0;
    unsigned char ch = c->p[c->i];
    if (c->n - c->i >= 4 && memcmp(c->p + c->i, "null", 4) == 0) {
        c->i += 4;
        return 1;
    }
    if (c->n - c->i >= 5 && memcmp(c->p + c->i, "false", 5) == 0) {
        c->i += 5;
        return 1;
    }
    if (c->n - c->i >= 4 && memcmp(c->p + c->i, "true", 4) == 0) {
        c->i += 4;
        return 1;
    }
    if (ch == '"') return jstring(c);
    if (ch == '-' || (ch >= '0' && ch <= '9')) {
        *is_num = 1;
        return jnumber(c, num);
    }
    if (ch == '[' || ch == '{') return jcontainer(c, ch == '{', nchild, dim, out, bad, top);
    return 0;
}

/* status as the /nearest handler decides it: 0 ok, 1 "Invalid JSON",
 * 2 "Vector size mismatch", 3 "Invalid vector data"; out: dim values */
int orc_decode_body(const char* text, size_t len, size_t dim, double* out) {
    jcur c;
    c.p = (const unsigned char*)text;
    c.n = len;
    for (size_t k = 0; k < len; ++k)
        if (text[k] == 0) {
            c.n = k;
            break;
        }
    c.i = 0;
    c.depth = 0;
    if (c.n >= 4 && c.p[0] == 0xEF && c.p[1] == 0xBB && c.p[2] == 0xBF) c.i = 3;
    jws(&c);
    size_t nchild = 0;
    int bad = 0, isn = 0;
    double v = 0;
    if (!jvalue(&c, &isn, &v, &nchild, dim, out, &bad, 1)) return 1;
    if (nchild != dim) return 2;
    if (bad) return 3;
    return 0;
}

/* ---- response bodies as cJSON_PrintUnformatted writes them ---------------- */
#include <float.h>
#include <limits.h>

/* one number; returns its length (at most 25) */
int orc_format_number(double d, char* out) {
    if (isnan(d) || isinf(d)) return sprintf(out, "null");
    const int vi = d >= (double)INT_MAX ? INT_MAX : d <= (double)INT_MIN ? INT_MIN : (int)d;
    if (d == (double)vi) return sprintf(out, "%d", vi);
    int n = sprintf(out, "%1.15g", d);
    const double back = strtod(out, NULL);
    const double m = fabs(back) > fabs(d) ? fabs(back) : fabs(d);
    if (!(fabs(back - d) <= m * DBL_EPSILON)) n = sprintf(out, "%1.17g", d);
    return n;
}

static size_t put_string(const char* s, size_t maxlen, char* out) {
    size_t o = 0;
    out[o++] = '"';
    for (size_t i = 0; i < maxlen && s[i]; ++i) {
        const unsigned char c = (unsigned char)s[i];
        if (c == '"' || c == '\\') {
            out[o++] = '\\';
            out[o++] = (char)c;
        } else if (c < 32) {
            out[o++] = '\\';
            switch (c) {
                case '\b': out[o++] = 'b'; break;
                case '\f': out[o++] = 'f'; break;
                case '\n': out[o++] = 'n'; break;
                case '\r': out[o++] = 'r'; break;
                case '\t': out[o++] = 't'; break;
                default: o += (size_t)sprintf(out + o, "u%04x", c);
            }
        } else {
            out[o++] = (char)c;
        }
    }
    out[o++] = '"';
    return o;
}

/* GET /compare/<metric> answer {"<key>":<value>} (src/compare_handler.c:
 * 152-185; result is the float metric widened to double) */
size_t orc_format_compare(int metric, float value, char* out) {
    static const char* keys[3] = {"cosine_similarity", "euclidean_distance", "dot_product"};
    size_t o = (size_t)sprintf(out, "{\"%s\":", keys[metric]);
    o += (size_t)orc_format_number((double)value, out + o);
    out[o++] = '}';
    out[o] = 0;
    return o;
}

/* POST /nearest answer (src/compare_handler.c:409-424): found = 1 with the
 * row (dim doubles), its position and uuid (char[37]); found = 0: no
 * neighbour (kdtree_nearest returned (size_t)-1); found = -1: the index read
 * no row (a stale KD node past the end of the store) */
size_t orc_format_nearest(int found, uint64_t index, const double* row, size_t dim, const char* uuid37, char* out) {
    size_t o = 0;
    if (found == 0) return (size_t)sprintf(out, "{\"error\":\"No nearest neighbor found\"}");
    if (found < 0) return (size_t)sprintf(out, "{\"error\":\"Nearest neighbor not found\"}");
    o += (size_t)sprintf(out + o, "{\"index\":");
    o += (size_t)orc_format_number((double)index, out + o);
    o += (size_t)sprintf(out + o, ",\"vector\":[");
    for (size_t i = 0; i < dim; ++i) {
        if (i) out[o++] = ',';
        o += (size_t)orc_format_number(row[i], out + o);
    }
    o += (size_t)sprintf(out + o, "],\"uuid\":");
    o += put_string(uuid37, 37, out + o);
    out[o++] = '}';
    out[o] = 0;
    return o;
}
