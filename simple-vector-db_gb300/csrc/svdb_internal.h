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

/* create the device store on the first row of nonzero dimension (db lock held) */
int svdb_db_ensure_dev(svdb_db* d, size_t dim);

/* ensure the device mirror holds every node inserted so far (lock held) */
int svdb_kd_sync_locked(svdb_kd* t);

#endif /* SVDB_INTERNAL_H */
