/*
 * svdb_store.c -- the drop-in vector_db_* API (reference
 * include/vector_database.h:39-108, src/vector_database.c:17-292).
 *
 * The host keeps the reference's VectorDatabase exactly (the handlers read
 * db->size, db->vectors[i] and db->kdtree directly) and mirrors every row
 * into the device store:
 *   insert  -> staged append to a new device slot (flushed in batches);
 *   update  -> in-place overwrite of the row's slot + a second KD node for
 *              the same index (src/vector_database.c:169-177);
 *   delete  -> the host array shifts left as in the reference
 *              (src/vector_database.c:185-195); the device slot is
 *              tombstoned, so later slots keep their place and the
 *              positional index becomes the rank among live slots.  The KD
 *              tree is left untouched, as in the reference.
 * All calls hold db->mutex, as the reference's do.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "svdb_internal.h"

void svdb_kd_insert_prefix(KDTree* tree, const double* point, size_t avail, size_t index);

SVDB_API VectorDatabase* vector_db_init(size_t initial_capacity, size_t dimension) {
    svdb_db* d = (svdb_db*)calloc(1, sizeof(svdb_db));
    if (!d) {
        fprintf(stderr, "Failed to allocate memory for database\n");
        return NULL;
    }
    VectorDatabase* db = &d->pub;
    db->size = 0;
    db->capacity = initial_capacity > 0 ? initial_capacity : 10;
    db->vectors = (Vector*)malloc(db->capacity * sizeof(Vector));
    d->slot_of = (int64_t*)malloc(db->capacity * sizeof(int64_t));
    if (!db->vectors || !d->slot_of) {
        fprintf(stderr, "Failed to allocate memory for vectors\n");
        free(db->vectors);
        free(d->slot_of);
        free(d);
        return NULL;
    }
    db->kdtree = kdtree_create(dimension);
    if (!db->kdtree) {
        fprintf(stderr, "Failed to create KDTree\n");
        free(db->vectors);
        free(d->slot_of);
        free(d);
        return NULL;
    }
    if (pthread_mutex_init(&db->mutex, NULL) != 0) {
        fprintf(stderr, "Failed to initialize mutex\n");
        kdtree_free(db->kdtree);
        free(db->vectors);
        free(d->slot_of);
        free(d);
        return NULL;
    }
    return db;
}

SVDB_API void vector_db_free(VectorDatabase* db) {
    if (!db) return;
    svdb_db* d = svdb_of(db);
    for (size_t i = 0; i < db->size; ++i) {
        svdb_rows_drop(db->vectors[i].data);
        free(db->vectors[i].data);
    }
    kdtree_free(db->kdtree);
    free(db->vectors);
    free(d->slot_of);
    if (d->dev) svdbd_store_destroy(d->dev);
    pthread_mutex_destroy(&db->mutex);
    free(d);
}

/* capacity doubling of the host arrays (src/vector_database.c:85-103) */
static int db_reserve_locked(svdb_db* d, size_t need) {
    VectorDatabase* db = &d->pub;
    if (need <= db->capacity) return 0;
    size_t nc = db->capacity;
    while (nc < need) {
        size_t next = nc > SIZE_MAX / 2 ? SIZE_MAX : nc * 2;
        if (next <= nc || next > SIZE_MAX / sizeof(Vector)) {
            fprintf(stderr, "Capacity overflow detected, unable to allocate more memory for vectors\n");
            return -1;
        }
        nc = next;
    }
    Vector* nv = (Vector*)realloc(db->vectors, nc * sizeof(Vector));
    if (!nv) {
        fprintf(stderr, "Failed to allocate more memory for vectors\n");
        return -1;
    }
    db->vectors = nv;
    int64_t* ns = (int64_t*)realloc(d->slot_of, nc * sizeof(int64_t));
    if (!ns) {
        fprintf(stderr, "Failed to allocate more memory for vectors\n");
        return -1;
    }
    d->slot_of = ns;
    db->capacity = nc;
    return 0;
}

/* The device store is created by the first row with a nonzero dimension,
 * which fixes the store's dimension.  Every row owns a slot: rows of another
 * dimension (and rows stored before the device store existed) hold
 * placeholder slots that keep positions right but are never searched. */
int svdb_db_ensure_dev(svdb_db* d, size_t dim) {
    if (d->dev || dim == 0) return SVDB_OK;
    d->dev = svdbd_store_create(dim);
    if (!d->dev) return SVDB_ENOMEM;
    d->dim = dim;
    for (size_t i = 0; i < d->pub.size; ++i) {
        const double* none = NULL;
        uint8_t flag = 2;
        d->slot_of[i] = (int64_t)svdbd_store_slots(d->dev);
        int rc = svdbd_store_append(d->dev, &none, &flag, 1);
        if (!rc && d->pub.vectors[i].uuid[0]) rc = svdbd_store_set_uuid(d->dev, d->slot_of[i], d->pub.vectors[i].uuid);
        if (rc) return rc;
    }
    return SVDB_OK;
}

static uint8_t row_flag(const svdb_db* d, const Vector* v) {
    return (v->data && v->dimension == d->dim) ? 1 : 2;
}

static size_t insert_locked(svdb_db* d, Vector vec) {
    VectorDatabase* db = &d->pub;
    if (db->size >= db->capacity && db_reserve_locked(d, db->size + 1) != 0) return (size_t)-1;
    if (!db->kdtree) {
        fprintf(stderr, "KDTree is NULL before inserting\n");
        return (size_t)-1;
    }
    if (svdb_db_ensure_dev(d, vec.dimension) != SVDB_OK) {
        fprintf(stderr, "vector_db_insert: %s\n", svdb_last_error());
        return (size_t)-1;
    }
    int64_t slot = -1;
    if (d->dev) {
        const double* row = vec.data;
        uint8_t live = row_flag(d, &vec);
        slot = (int64_t)svdbd_store_slots(d->dev);
        if (svdbd_store_append(d->dev, &row, &live, 1) != SVDB_OK ||
            (vec.uuid[0] && svdbd_store_set_uuid(d->dev, slot, vec.uuid) != SVDB_OK)) {
            fprintf(stderr, "vector_db_insert: %s\n", svdb_last_error());
            return (size_t)-1;
        }
    }
    db->vectors[db->size] = vec; /* uuid included, as src/vector_database.c:113 */
    d->slot_of[db->size] = slot;
    if (d->dev && row_flag(d, &vec) == 1) svdb_rows_put(vec.data, d, slot);
    svdb_kd_insert_prefix(db->kdtree, vec.data, vec.data ? vec.dimension : 0, db->size);
    return db->size++;
}

SVDB_API size_t vector_db_insert(VectorDatabase* db, Vector vec) {
    if (!db) return (size_t)-1;
    pthread_mutex_lock(&db->mutex);
    size_t r = insert_locked(svdb_of(db), vec);
    pthread_mutex_unlock(&db->mutex);
    return r;
}

SVDB_API Vector* vector_db_read(VectorDatabase* db, size_t index) {
    if (!db) return NULL;
    pthread_mutex_lock(&db->mutex);
    Vector* v = index < db->size ? &db->vectors[index] : NULL;
    pthread_mutex_unlock(&db->mutex);
    return v;
}

/* src/vector_database.c:145-158: the first row in positional order whose
 * uuid equals `uuid` under strncmp(.., 37).  The reference scans the array;
 * here the device's uuid index answers (dev_uuid.cu).  A store that has never
 * held a row of nonzero dimension has no device store -- nothing to index --
 * and its (dimensionless) rows are scanned. */
SVDB_API Vector* vector_db_read_by_uuid(VectorDatabase* db, const char* uuid) {
    if (!db || !uuid) return NULL;
    svdb_db* d = svdb_of(db);
    pthread_mutex_lock(&db->mutex);
    Vector* v = NULL;
    if (d->dev) {
        char key[UUID_SIZE];
        memset(key, 0, sizeof(key));
        for (size_t i = 0; i < UUID_SIZE && uuid[i]; ++i) key[i] = uuid[i];
        int64_t pos = -1;
        if (svdbd_uuid_find(d->dev, key, 1, &pos) != SVDB_OK)
            fprintf(stderr, "vector_db_read_by_uuid: %s\n", svdb_last_error());
        else if (pos >= 0 && (size_t)pos < db->size)
            v = &db->vectors[pos];
    } else {
        for (size_t i = 0; i < db->size; ++i)
            if (strncmp(db->vectors[i].uuid, uuid, UUID_SIZE) == 0) {
                v = &db->vectors[i];
                break;
            }
    }
    pthread_mutex_unlock(&db->mutex);
    return v;
}

SVDB_API void vector_db_update(VectorDatabase* db, size_t index, Vector vec) {
    if (!db) return;
    svdb_db* d = svdb_of(db);
    pthread_mutex_lock(&db->mutex);
    if (index < db->size) {
        if (svdb_db_ensure_dev(d, vec.dimension) != SVDB_OK)
            fprintf(stderr, "vector_db_update: %s\n", svdb_last_error());
        else if (d->dev &&
                 (svdbd_store_overwrite(d->dev, d->slot_of[index], vec.data, row_flag(d, &vec)) != SVDB_OK ||
                  svdbd_store_set_uuid(d->dev, d->slot_of[index], vec.uuid) != SVDB_OK))
            fprintf(stderr, "vector_db_update: %s\n", svdb_last_error());
        svdb_rows_drop(db->vectors[index].data);
        free(db->vectors[index].data);
        db->vectors[index] = vec;
        if (d->dev && row_flag(d, &vec) == 1) svdb_rows_put(vec.data, d, d->slot_of[index]);
        svdb_kd_insert_prefix(db->kdtree, vec.data, vec.data ? vec.dimension : 0, index);
    }
    pthread_mutex_unlock(&db->mutex);
}

SVDB_API void vector_db_delete(VectorDatabase* db, size_t index) {
    if (!db) return;
    svdb_db* d = svdb_of(db);
    pthread_mutex_lock(&db->mutex);
    if (index < db->size) {
        if (d->dev && d->slot_of[index] >= 0 && svdbd_store_kill(d->dev, d->slot_of[index]) != SVDB_OK)
            fprintf(stderr, "vector_db_delete: %s\n", svdb_last_error());
        svdb_rows_drop(db->vectors[index].data);
        free(db->vectors[index].data);
        memmove(db->vectors + index, db->vectors + index + 1, (db->size - index - 1) * sizeof(Vector));
        memmove(d->slot_of + index, d->slot_of + index + 1, (db->size - index - 1) * sizeof(int64_t));
        db->size--;
    }
    pthread_mutex_unlock(&db->mutex);
}

/* file format of src/vector_database.c:203-228: size_t n, then per row
 * uuid[37], size_t dim, double[dim]; rows with no data are skipped but still
 * counted in n, exactly as the reference writes them. */
/* The file format of src/vector_database.c:203-223: the row count, then per
 * row uuid[37], size_t dimension, double[dimension].  Rows without data are
 * skipped; the reference still writes db->size as the count (so such a file
 * promises more rows than it holds).  exact_count writes the number of rows
 * actually written instead (svdb_save with SVDB_SAVE_EXACT_COUNT). */
static int save_locked(VectorDatabase* db, const char* filename, int exact_count) {
    FILE* f = fopen(filename, "wb");
    if (!f) {
        perror("Failed to open file for writing");
        svdb_set_error("save: cannot open %s for writing", filename);
        return SVDB_EINVAL;
    }
    size_t n = db->size;
    if (exact_count) {
        n = 0;
        for (size_t i = 0; i < db->size; ++i) n += db->vectors[i].dimension != 0 && db->vectors[i].data != NULL;
    }
    int ok = fwrite(&n, sizeof(size_t), 1, f) == 1;
    for (size_t i = 0; i < db->size; ++i) {
        const Vector* v = &db->vectors[i];
        if (v->dimension == 0 || v->data == NULL) {
            fprintf(stderr, "Invalid vector at index %zu, skipping\n", i);
            continue;
        }
        ok = ok && fwrite(v->uuid, sizeof(char), UUID_SIZE, f) == UUID_SIZE;
        ok = ok && fwrite(&v->dimension, sizeof(size_t), 1, f) == 1;
        ok = ok && fwrite(v->data, sizeof(double), v->dimension, f) == v->dimension;
    }
    ok = (fclose(f) == 0) && ok;
    if (!ok) {
        svdb_set_error("save: write to %s failed", filename);
        return SVDB_EINVAL;
    }
    return SVDB_OK;
}

SVDB_API void vector_db_save(VectorDatabase* db, const char* filename) {
    if (!db || !filename) return;
    pthread_mutex_lock(&db->mutex);
    save_locked(db, filename, 0);
    pthread_mutex_unlock(&db->mutex);
}

SVDB_API int svdb_save(VectorDatabase* db, const char* filename, unsigned flags) {
    if (!db || !filename || (flags & ~(unsigned)SVDB_SAVE_EXACT_COUNT)) {
        svdb_set_error("svdb_save: NULL argument or unknown flag");
        return SVDB_EINVAL;
    }
    pthread_mutex_lock(&db->mutex);
    const int rc = save_locked(db, filename, (flags & SVDB_SAVE_EXACT_COUNT) != 0);
    pthread_mutex_unlock(&db->mutex);
    return rc;
}

SVDB_API VectorDatabase* vector_db_load(const char* filename, size_t dimension) {
    if (!filename) return NULL;
    FILE* f = fopen(filename, "rb");
    if (!f) {
        perror("Failed to open file for reading");
        return NULL;
    }
    size_t n = 0;
    if (fread(&n, sizeof(size_t), 1, f) != 1) n = 0;
    VectorDatabase* db = vector_db_init(n > 0 ? n : 10, dimension);
    if (!db) {
        fclose(f);
        return NULL;
    }
    svdb_db* d = svdb_of(db);
    for (size_t i = 0; i < n; ++i) {
        Vector v;
        memset(&v, 0, sizeof(v));
        size_t dim = 0;
        if (fread(v.uuid, sizeof(char), UUID_SIZE, f) != UUID_SIZE || fread(&dim, sizeof(size_t), 1, f) != 1) {
            fprintf(stderr, "vector_db_load: truncated file at row %zu\n", i);
            break;
        }
        v.dimension = dim;
        v.data = (double*)malloc((dim ? dim : 1) * sizeof(double));
        if (!v.data) {
            fprintf(stderr, "Failed to allocate memory for vector data\n");
            vector_db_free(db);
            fclose(f);
            return NULL;
        }
        if (fread(v.data, sizeof(double), dim, f) != dim) {
            fprintf(stderr, "vector_db_load: truncated file at row %zu\n", i);
            free(v.data);
            break;
        }
        if (insert_locked(d, v) == (size_t)-1) {
            free(v.data);
            vector_db_free(db);
            fclose(f);
            return NULL;
        }
    }
    fclose(f);
    return db;
}
