/*
 * percall_driver.c -- timing harness for the drop-in per-call API, built as
 * its own small library (not part of libsvdb_gb300.so).
 *
 * The reference's server answers each request on its own thread
 * (MHD_USE_THREAD_PER_CONNECTION, src/main.c:381) with one call per request:
 * cosine_similarity / euclidean_distance / dot_product on two stored rows
 * (src/compare_handler.c:153-159) or kdtree_nearest (:403).  This harness
 * runs T threads that each make `calls` such calls one after another and
 * records every call's latency, so a caller-side implementation (this
 * library's drop-in functions, or a CPU restatement) can be timed the way
 * the server would use it, without any interpreter in the loop.
 *
 * The function under test is passed as a pointer with one of two calling
 * conventions:
 *   abi 0: float f(Vector a, Vector b)                          (the drop-in API)
 *   abi 1: float f(int metric, const double* a, size_t na,
 *                  const double* b, size_t nb)                   (a CPU restatement)
 * and for /nearest: size_t f(void* tree, const double* q).
 */
#define _GNU_SOURCE
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "../../include/vector_database.h"

#if defined(__GNUC__)
#define PC_API __attribute__((visibility("default")))
#else
#define PC_API
#endif

typedef float (*metric_abi0)(Vector, Vector);
typedef float (*metric_abi1)(int, const double*, size_t, const double*, size_t);
typedef size_t (*nearest_fn)(void*, const double*);

typedef struct {
    int kind; /* 0 metric, 1 nearest */
    void* fn;
    int abi, metric;
    const Vector* va;
    const Vector* vb;
    size_t npairs;
    void* tree;
    const double* q;
    size_t nq, dim;
    size_t calls;
    int t;
    double* lat_ns;
    float* out;
    int64_t* near_out;
    struct gate* start;
} job;

/* start gate: every thread begins at once; `cancel` sends them home */
struct gate {
    pthread_mutex_t mu;
    pthread_cond_t cv;
    int go, cancel;
};

static double now_ns(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec * 1e9 + (double)ts.tv_nsec;
}

static void* run(void* arg) {
    job* j = (job*)arg;
    pthread_mutex_lock(&j->start->mu);
    while (!j->start->go) pthread_cond_wait(&j->start->cv, &j->start->mu);
    const int cancel = j->start->cancel;
    pthread_mutex_unlock(&j->start->mu);
    if (cancel) return NULL;
    for (size_t c = 0; c < j->calls; ++c) {
        const size_t k = (size_t)j->t * j->calls + c;
        const double t0 = now_ns();
        if (j->kind == 0) {
            const size_t p = k % j->npairs;
            float r;
            if (j->abi == 0) {
                r = ((metric_abi0)j->fn)(j->va[p], j->vb[p]);
            } else {
                r = ((metric_abi1)j->fn)(j->metric, j->va[p].data, j->va[p].dimension, j->vb[p].data,
                                         j->vb[p].dimension);
            }
            if (j->out) j->out[k] = r;
        } else {
            const size_t p = k % j->nq;
            const size_t r = ((nearest_fn)j->fn)(j->tree, j->q + p * j->dim);
            if (j->near_out) j->near_out[k] = (int64_t)r;
        }
        j->lat_ns[k] = now_ns() - t0;
    }
    return NULL;
}

static int run_all(job* proto, int threads, double* wall_ns) {
    pthread_t* th = (pthread_t*)malloc((size_t)threads * sizeof(pthread_t));
    job* js = (job*)malloc((size_t)threads * sizeof(job));
    struct gate g;
    if (!th || !js) {
        free(th);
        free(js);
        return -1;
    }
    pthread_mutex_init(&g.mu, NULL);
    pthread_cond_init(&g.cv, NULL);
    g.go = 0;
    g.cancel = 0;
    int started = 0;
    for (int t = 0; t < threads; ++t) {
        js[t] = *proto;
        js[t].t = t;
        js[t].start = &g;
        if (pthread_create(&th[t], NULL, run, &js[t]) != 0) break;
        ++started;
    }
    pthread_mutex_lock(&g.mu);
    g.go = 1;
    g.cancel = started != threads;
    const double t0 = now_ns();
    pthread_cond_broadcast(&g.cv);
    pthread_mutex_unlock(&g.mu);
    for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
    *wall_ns = now_ns() - t0;
    pthread_cond_destroy(&g.cv);
    pthread_mutex_destroy(&g.mu);
    free(th);
    free(js);
    return started == threads ? 0 : -1;
}

/* T threads x calls metric calls on the pairs (va[i], vb[i]), i cycling;
 * lat_ns[T x calls]; out (optional) the results; *wall_ns the elapsed time. */
PC_API int svdb_percall_metric(void* fn, int abi, int metric, const Vector* va, const Vector* vb, size_t npairs,
                               int threads, size_t calls, double* lat_ns, float* out, double* wall_ns) {
    if (!fn || !va || !vb || !npairs || threads < 1 || !lat_ns || !wall_ns) return -1;
    job p;
    memset(&p, 0, sizeof(p));
    p.kind = 0;
    p.fn = fn;
    p.abi = abi;
    p.metric = metric;
    p.va = va;
    p.vb = vb;
    p.npairs = npairs;
    p.calls = calls;
    p.lat_ns = lat_ns;
    p.out = out;
    return run_all(&p, threads, wall_ns);
}

/* T threads x calls nearest calls on queries q (nq x dim), cycling. */
PC_API int svdb_percall_nearest(void* fn, void* tree, const double* q, size_t nq, size_t dim, int threads,
                                size_t calls, double* lat_ns, int64_t* out, double* wall_ns) {
    if (!fn || !q || !nq || threads < 1 || !lat_ns || !wall_ns) return -1;
    job p;
    memset(&p, 0, sizeof(p));
    p.kind = 1;
    p.fn = fn;
    p.tree = tree;
    p.q = q;
    p.nq = nq;
    p.dim = dim;
    p.calls = calls;
    p.lat_ns = lat_ns;
    p.near_out = out;
    return run_all(&p, threads, wall_ns);
}

/* ---- open-loop replay through a request loop (svdb_loop_submit / _wait) ---
 * One thread submits request i at t0 + arrival_s[i] (spinning on the clock),
 * another takes the answers in ticket order and stamps each one: lat_ns[i] =
 * completion - (t0 + arrival_s[i]), queueing included. */
typedef int (*loop_submit_fn)(void*, const void*, uint64_t*);
typedef int (*loop_wait_fn)(void*, uint64_t, void*, uint32_t);

typedef struct {
    void* submit;
    void* wait;
    void* loop;
    const char* reqs;
    size_t req_size;
    const double* arrival;
    size_t n;
    double* lat;
    char* resps;
    size_t resp_size;
    uint64_t* tickets;
    volatile size_t published;
    double t0;
    int rc;
} replay;

static void* replay_submit(void* arg) {
    replay* r = (replay*)arg;
    for (size_t i = 0; i < r->n; ++i) {
        const double due = r->t0 + r->arrival[i] * 1e9;
        while (now_ns() < due) {
        }
        uint64_t t = 0;
        if (((loop_submit_fn)r->submit)(r->loop, r->reqs + i * r->req_size, &t) != 0) {
            r->rc = -1;
            __atomic_store_n(&r->published, r->n + 1, __ATOMIC_RELEASE);
            return NULL;
        }
        r->tickets[i] = t;
        __atomic_store_n(&r->published, i + 1, __ATOMIC_RELEASE);
    }
    return NULL;
}

PC_API int svdb_percall_loop_replay(void* submit, void* wait, void* loop, const void* reqs, size_t req_size,
                                    const double* arrival_s, size_t n, double* lat_ns, void* resps, size_t resp_size,
                                    double* wall_ns) {
    if (!submit || !wait || !loop || !reqs || !arrival_s || !lat_ns || !resps || !wall_ns) return -1;
    replay r;
    memset(&r, 0, sizeof(r));
    r.submit = submit;
    r.wait = wait;
    r.loop = loop;
    r.reqs = (const char*)reqs;
    r.req_size = req_size;
    r.arrival = arrival_s;
    r.n = n;
    r.lat = lat_ns;
    r.resps = (char*)resps;
    r.resp_size = resp_size;
    r.tickets = (uint64_t*)malloc((n ? n : 1) * sizeof(uint64_t));
    if (!r.tickets) return -1;
    r.t0 = now_ns() + 2e6;  /* 2 ms to get going */
    pthread_t th;
    if (pthread_create(&th, NULL, replay_submit, &r) != 0) {
        free(r.tickets);
        return -1;
    }
    int rc = 0;
    for (size_t i = 0; i < n; ++i) {
        size_t p;
        while ((p = __atomic_load_n(&r.published, __ATOMIC_ACQUIRE)) <= i) {
        }
        if (p > n) {
            rc = -1;
            break;
        }
        if (((loop_wait_fn)wait)(loop, r.tickets[i], r.resps + i * resp_size, 30000000u) != 0) {
            rc = -1;
            break;
        }
        lat_ns[i] = now_ns() - (r.t0 + arrival_s[i] * 1e9);
    }
    pthread_join(th, NULL);
    *wall_ns = now_ns() - r.t0;
    free(r.tickets);
    return rc ? rc : r.rc;
}
