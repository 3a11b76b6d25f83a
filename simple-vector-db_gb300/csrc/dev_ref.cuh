// dev_ref.cuh -- the reference's own per-request arithmetic as device
// functions, shared by the batch kernels (dev_store.cu, dev_kd.cu) and the
// device-side request loop (dev_loop.cu).
#pragma once

#include <stdint.h>

#include "svdb_device.h"

namespace svdb {

// Reference-exact metrics: the float-accumulating loops of
// src/vector_database.c:301-352, IEEE intrinsics so nothing is contracted
// into an FMA.  One thread per pair: the order of the additions is the
// reference's, so the loop cannot be split.
__device__ __forceinline__ float ref_metric(int metric, const double* __restrict__ a, const double* __restrict__ b,
                                            int d) {
    if (metric == SVDB_EUCLIDEAN) {
        float sum = 0.0f;
        for (int i = 0; i < d; ++i) {
            const float diff = __double2float_rn(__dsub_rn(a[i], b[i]));
            sum = __fadd_rn(sum, __fmul_rn(diff, diff));
        }
        return __double2float_rn(__dsqrt_rn((double)sum));
    }
    float dot = 0.0f, na = 0.0f, nb = 0.0f;
    for (int i = 0; i < d; ++i) {
        const double ai = a[i], bi = b[i];
        dot = __double2float_rn(__dadd_rn((double)dot, __dmul_rn(ai, bi)));
        if (metric == SVDB_COSINE) {
            na = __double2float_rn(__dadd_rn((double)na, __dmul_rn(ai, ai)));
            nb = __double2float_rn(__dadd_rn((double)nb, __dmul_rn(bi, bi)));
        }
    }
    if (metric == SVDB_DOT) return dot;
    return __double2float_rn(__ddiv_rn((double)dot, __dmul_rn(__dsqrt_rn((double)na), __dsqrt_rn((double)nb))));
}

__device__ __forceinline__ double kd_sqdist(const double* __restrict__ p, const double* __restrict__ q, int kdim) {
    double d = 0.0;
    for (int i = 0; i < kdim; ++i) {
        const double t = __dsub_rn(p[i], q[i]);
        d = __dadd_rn(d, __dmul_rn(t, t));
    }
    return d;
}

// kdtree_nearest (src/kdtree.c:131-178) over the flat insertion-order tree:
// node i has pts[i*kdim ..], its stored index index[i] and children child[i]
// (-1: none), root 0.  The recursion becomes an explicit stack (`stack`,
// room for the tree's height) with the same visit order: the node, then the
// near subtree, then the far one if (q[cd]-p[cd])^2 < best; strict "<"
// replacement and unfused FP64 arithmetic, so ties go to the same (first
// visited) node.  Returns the stored index, or -1 for an empty tree.
__device__ __forceinline__ int64_t kd_descend(const double* __restrict__ pts, const int64_t* __restrict__ index,
                                              const int2* __restrict__ child, int kdim, int64_t n,
                                              const double* __restrict__ qq, int2* stack) {
    double best = __longlong_as_double(0x7ff0000000000000ll);
    int bestn = -1;
    int sp = 0;
    int cur = n > 0 ? 0 : -1;
    int depth = 0;
    for (;;) {
        while (cur >= 0) {
            const double* p = pts + (size_t)cur * kdim;
            const double d = kd_sqdist(p, qq, kdim);
            if (d < best) {
                best = d;
                bestn = cur;
            }
            const int cd = depth % kdim;
            const int2 ch = child[cur];
            stack[sp++] = make_int2(cur, depth);
            cur = qq[cd] < p[cd] ? ch.x : ch.y;
            ++depth;
        }
        bool more = false;
        while (sp > 0) {
            const int2 e = stack[--sp];
            const int cd = e.y % kdim;
            const double pc = pts[(size_t)e.x * kdim + cd], qc = qq[cd];
            const double t = __dsub_rn(qc, pc);
            if (__dmul_rn(t, t) < best) {
                const int2 ch = child[e.x];
                cur = qc < pc ? ch.y : ch.x;
                depth = e.y + 1;
                if (cur >= 0) {
                    more = true;
                    break;
                }
            }
        }
        if (!more) break;
    }
    return bestn >= 0 ? index[bestn] : -1;
}

}  // namespace svdb
