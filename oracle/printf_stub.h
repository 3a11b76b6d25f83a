/*
 * Test infrastructure only: force-included when the reference's own
 * src/vector_database.c and src/kdtree.c are compiled into oracle/_ref.
 *
 * The reference prints on every KD-tree level it walks (src/kdtree.c:16,48,89)
 * and on every insert (src/vector_database.c:84-89), so any timing of it
 * would measure stdout. stdio.h is included first so its prototypes are
 * untouched; every later printf(...) in the reference becomes a no-op.
 * fprintf/perror (error paths only) are left alone.
 */
#include <stdio.h>
#define printf(...) ((void)0)
