/*
 * svdb_internal.h -- private objects behind the drop-in VectorDatabase and
 * KDTree pointers (C host layer).
 */
#ifndef SVDB_INTERNAL_H
#define SVDB_INTERNAL_H

#include <pthread.h>
#include <stddef.h>
#include <stdint.h>

#include "svdb_device.h"

/* Combining of concurrent calls (svdb_combine.c): every call starts with an
 * svdb_call; a caller queues its call and either waits for a batch that
 * answers it or, when no batch is in flight, answers every queued call with
 * one run of `fn`. */
typedef struct svdb_call {
    int done;
} svdb_call;
typedef void (*svdb_batch_fn)(void* ctx, svdb_call** calls, size_t n);
typedef struct svdb_combiner {
    pthread_mutex_t mu;
    pthread_cond_t cv;
    int busy;
    svdb_call** q;
    size_t n, cap;
} svdb_combiner;
#define SVDB_COMBINER_INIT {PTHREAD_MUTEX_INITIALIZER, PTHREAD_COND_INITIALIZER, 0, NULL, 0, 0}
void svdb_combine(svdb_combiner* c, svdb_call* call, svdb_batch_fn fn, void* ctx);

/* KD tree: the reference's insertion-order tree in flat arrays.  `pub` must
 * stay the first member: KDTree* and svdb_kd* are the same address. */
typedef struct svdb_kd {
    KDTree pub;
    pthread_mutex_t lock;
    size_t n, cap;
    double* pts;      /* n x dim prefix copies */
    int64_t* index;   /* stored index per node */
    int32_t* left;    /* -1 = none */
    int32_t* right;
    int height;       /* nodes on the longest root path */
    size_t synced;    /* nodes [0, synced) are mirrored on the device */
    int32_t* patch;   /* mirrored nodes whose child links changed since the last sync */
    size_t npatch, patch_cap;
    svdbd_kd* dev;
    svdb_combiner comb; /* concurrent kdtree_nearest calls */
} svdb_kd;

/* Store: `pub` must stay the first member. */
typedef struct svdb_db {
    VectorDatabase pub;
    int64_t* slot_of; /* logical index -> device slot (capacity pub.capacity) */
    size_t dim;       /* device-store dimension, fixed by the first stored row */
    svdbd_store* dev;
} svdb_db;

static inline svdb_db* svdb_of(VectorDatabase* db) { return (svdb_db*)db; }
static inline svdb_kd* svdb_kd_of(KDTree* t) { return (svdb_kd*)t; }

/* Registry of the stores' searchable rows by their host buffer
 * (svdb_combine.c): put when a row gets a device slot, drop before its
 * buffer is freed; find answers which store and slot a Vector's data is. */
void svdb_rows_put(const double* data, svdb_db* d, int64_t slot);
void svdb_rows_drop(const double* data);
int svdb_rows_find(const double* data, svdb_db** d, int64_t* slot);

/* create the device store on the first row of nonzero dimension (db lock held) */
int svdb_db_ensure_dev(svdb_db* d, size_t dim);

/* ensure the device mirror holds every node inserted so far (lock held) */
int svdb_kd_sync_locked(svdb_kd* t);

#endif /* SVDB_INTERNAL_H */
