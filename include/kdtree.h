/*
 * kdtree.h -- drop-in KD-tree API of simple-vector-db, served by
 * libsvdb_gb300.so.
 *
 * The tree is the reference's: unbalanced, built in insertion order over the
 * first `dimension` coordinates of each point, split axis depth % dimension,
 * "<" goes left; kdtree_nearest is the exact 1-NN over that prefix with the
 * reference's tie rule (first node visited wins).  Nodes live in flat arrays
 * mirrored to the GPU, and kdtree_nearest runs as a CUDA kernel.
 *
 * KDTree keeps the reference layout so code that stores or NULL-checks
 * db->kdtree still compiles; its `root` field is always NULL here (the
 * nodes are not KDTreeNode objects).  Only pointers returned by
 * kdtree_create may be passed to this API.
 */
#ifndef KDTREE_H
#define KDTREE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same layout as reference include/kdtree.h:10-15 (kept for source
 * compatibility; this library does not allocate KDTreeNode objects). */
typedef struct KDTreeNode {
    double* point;
    size_t index;
    struct KDTreeNode* left;
    struct KDTreeNode* right;
} KDTreeNode;

/* Same layout as reference include/kdtree.h:21-24. */
typedef struct KDTree {
    KDTreeNode* root;
    size_t dimension;
} KDTree;

/* replaces kdtree_create, reference include/kdtree.h:32 (src/kdtree.c:70-78) */
KDTree* kdtree_create(size_t dimension);

/* replaces kdtree_insert, reference include/kdtree.h:41 (src/kdtree.c:87-91) */
void kdtree_insert(KDTree* tree, const double* point, size_t index);

/* replaces kdtree_free, reference include/kdtree.h:48 (src/kdtree.c:112-118) */
void kdtree_free(KDTree* tree);

/* replaces kdtree_nearest, reference include/kdtree.h:57
 * (src/kdtree.c:131-178).  Returns the stored index of the nearest node, or
 * (size_t)-1 when the tree is empty or the GPU call failed. */
size_t kdtree_nearest(KDTree* tree, const double* point);

#ifdef __cplusplus
}
#endif

#endif /* KDTREE_H */
