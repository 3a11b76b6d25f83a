// dev_kd.cu -- device mirror of the insertion-order KD tree and the batched
// exact nearest-neighbour descent.
//
// HBM layout (n nodes, prefix length kdim):
//   pts    n x kdim  double   prefix copy of each inserted point (src/kdtree.c:26-28)
//   index  n         int64    stored index (src/kdtree.c:30)
//   child  n         int2     {left, right}, -1 = none
//
// k_kd_nearest is one thread per query and restates kdtree_nearest_rec
// (src/kdtree.c:131-162) as an explicit-stack loop with the same visit order
// (node, near subtree, then far subtree if (q[cd]-p[cd])^2 < best), the same
// strict "<" replacement and the same unfused FP64 arithmetic, so the
// returned index is the reference's, ties included.
#include <algorithm>
#include <cstring>
#include <vector>

#include "dev_common.cuh"
#include "dev_ref.cuh"

namespace svdb {

struct Kd {
    size_t kdim = 0;
    cudaStream_t stream = nullptr;
    size_t cap = 0, n = 0;
    double* pts = nullptr;
    int64_t* index = nullptr;
    int2* child = nullptr;
    int height = 0;
    void* scratch = nullptr;
    size_t scratch_bytes = 0;
    void* pin = nullptr;
    size_t pin_bytes = 0;
};

__global__ void k_kd_patch(int2* child, const int4* patches, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const int4 p = patches[i];
        child[p.x] = make_int2(p.y, p.z);
    }
}

// MAXH > 0: stack in registers/local memory; MAXH == 0: stack in `gstack`
// (height entries per query).
template <int MAXH>
__global__ void __launch_bounds__(128) k_kd_nearest(const double* __restrict__ pts, const int64_t* __restrict__ index,
                                                    const int2* __restrict__ child, int kdim, int64_t n,
                                                    const double* __restrict__ q, size_t qs, int nq,
                                                    int64_t* __restrict__ out, int2* __restrict__ gstack,
                                                    int height) {
    const int qi = blockIdx.x * blockDim.x + threadIdx.x;
    if (qi >= nq) return;
    int2 lstack[MAXH > 0 ? MAXH : 1];
    int2* stack = MAXH > 0 ? lstack : gstack + (size_t)qi * height;
    out[qi] = kd_descend(pts, index, child, kdim, n, q + (size_t)qi * qs, stack);
}

static int kd_reserve_dev(Kd* t, size_t need) {
    if (need <= t->cap) return SVDB_OK;
    size_t nc = t->cap ? t->cap : 1024;
    while (nc < need) nc *= 2;
    double* np = nullptr;
    int64_t* ni = nullptr;
    int2* nc2 = nullptr;
    cudaError_t e = cudaMalloc(&np, nc * t->kdim * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&ni, nc * sizeof(int64_t));
    if (e == cudaSuccess) e = cudaMalloc(&nc2, nc * sizeof(int2));
    if (e != cudaSuccess) {
        cudaGetLastError();
        cudaFree(np);
        cudaFree(ni);
        cudaFree(nc2);
        svdb_set_error("kd mirror: cannot grow to %zu nodes", nc);
        return SVDB_ENOMEM;
    }
    if (t->n) {
        SVDB_CUDA(cudaMemcpyAsync(np, t->pts, t->n * t->kdim * sizeof(double), cudaMemcpyDeviceToDevice, t->stream));
        SVDB_CUDA(cudaMemcpyAsync(ni, t->index, t->n * sizeof(int64_t), cudaMemcpyDeviceToDevice, t->stream));
        SVDB_CUDA(cudaMemcpyAsync(nc2, t->child, t->n * sizeof(int2), cudaMemcpyDeviceToDevice, t->stream));
        SVDB_CUDA(cudaStreamSynchronize(t->stream));
    }
    cudaFree(t->pts);
    cudaFree(t->index);
    cudaFree(t->child);
    t->pts = np;
    t->index = ni;
    t->child = nc2;
    t->cap = nc;
    return SVDB_OK;
}

static int kd_scratch(Kd* t, size_t bytes) {
    if (bytes <= t->scratch_bytes) return SVDB_OK;
    SVDB_CUDA(cudaStreamSynchronize(t->stream));
    cudaFree(t->scratch);
    t->scratch = nullptr;
    t->scratch_bytes = 0;
    const size_t nb = round_up(bytes + bytes / 4, 1 << 16);
    SVDB_CUDA(cudaMalloc(&t->scratch, nb));
    t->scratch_bytes = nb;
    return SVDB_OK;
}

static int kd_pinned(Kd* t, size_t bytes) {
    if (bytes <= t->pin_bytes) return SVDB_OK;
    SVDB_CUDA(cudaStreamSynchronize(t->stream));
    cudaFreeHost(t->pin);
    t->pin = nullptr;
    t->pin_bytes = 0;
    const size_t nb = round_up(bytes + bytes / 4, 1 << 16);
    SVDB_CUDA(cudaMallocHost(&t->pin, nb));
    t->pin_bytes = nb;
    return SVDB_OK;
}

}  // namespace svdb

using svdb::Kd;

extern "C" {

svdbd_kd* svdbd_kd_create(size_t kdim) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        svdb_set_error("no CUDA device");
        return nullptr;
    }
    Kd* t = new (std::nothrow) Kd();
    if (!t) return nullptr;
    t->kdim = kdim;
    if (cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        svdb_set_error("kd mirror: stream creation failed");
        delete t;
        return nullptr;
    }
    return reinterpret_cast<svdbd_kd*>(t);
}

void svdbd_kd_destroy(svdbd_kd* ht) {
    Kd* t = reinterpret_cast<Kd*>(ht);
    if (!t) return;
    cudaStreamSynchronize(t->stream);
    cudaFree(t->pts);
    cudaFree(t->index);
    cudaFree(t->child);
    cudaFree(t->scratch);
    cudaFreeHost(t->pin);
    cudaStreamDestroy(t->stream);
    delete t;
}

int svdbd_kd_sync(svdbd_kd* ht, const double* pts, const int64_t* index, const int32_t* left, const int32_t* right,
                  size_t n, size_t synced, const int32_t* patch_nodes, size_t npatch, int height) {
    Kd* t = reinterpret_cast<Kd*>(ht);
    int rc = svdb::kd_reserve_dev(t, n);
    if (rc) return rc;
    const size_t nn = n - synced;
    const size_t bytes = nn * (t->kdim * sizeof(double) + sizeof(int64_t) + sizeof(int2)) + npatch * sizeof(int4);
    rc = svdb::kd_pinned(t, bytes + 64);
    if (!rc) rc = svdb::kd_scratch(t, npatch * sizeof(int4) + 64);
    if (rc) return rc;
    SVDB_CUDA(cudaStreamSynchronize(t->stream));
    unsigned char* hp = (unsigned char*)t->pin;
    if (nn) {
        std::memcpy(hp, pts + synced * t->kdim, nn * t->kdim * sizeof(double));
        SVDB_CUDA(cudaMemcpyAsync(t->pts + synced * t->kdim, hp, nn * t->kdim * sizeof(double), cudaMemcpyHostToDevice,
                                  t->stream));
        hp += nn * t->kdim * sizeof(double);
        std::memcpy(hp, index + synced, nn * sizeof(int64_t));
        SVDB_CUDA(cudaMemcpyAsync(t->index + synced, hp, nn * sizeof(int64_t), cudaMemcpyHostToDevice, t->stream));
        hp += nn * sizeof(int64_t);
        int2* hc = (int2*)hp;
        for (size_t i = 0; i < nn; ++i) hc[i] = make_int2(left[synced + i], right[synced + i]);
        SVDB_CUDA(cudaMemcpyAsync(t->child + synced, hc, nn * sizeof(int2), cudaMemcpyHostToDevice, t->stream));
        hp += nn * sizeof(int2);
    }
    if (npatch) {
        int4* hpt = (int4*)hp;
        for (size_t i = 0; i < npatch; ++i) {
            const int32_t p = patch_nodes[i];
            hpt[i] = make_int4(p, left[p], right[p], 0);
        }
        int4* dpt = (int4*)t->scratch;
        SVDB_CUDA(cudaMemcpyAsync(dpt, hpt, npatch * sizeof(int4), cudaMemcpyHostToDevice, t->stream));
        svdb::k_kd_patch<<<(unsigned)((npatch + 255) / 256), 256, 0, t->stream>>>(t->child, dpt, (int)npatch);
        SVDB_LAUNCH_CHECK();
    }
    SVDB_CUDA(cudaStreamSynchronize(t->stream));
    t->n = n;
    t->height = height;
    return SVDB_OK;
}

int svdbd_kd_nearest(svdbd_kd* ht, const double* q, size_t nq, size_t qstride, int64_t* out) {
    Kd* t = reinterpret_cast<Kd*>(ht);
    if (nq == 0) return SVDB_OK;
    const size_t kd = t->kdim;
    const int h = std::max(t->height, 1);
    const bool local = h <= 64;
    const size_t qbytes = svdb::round_up(nq * kd * sizeof(double), 256);
    const size_t obytes = svdb::round_up(nq * sizeof(int64_t), 256);
    const size_t sbytes = local ? 0 : nq * (size_t)h * sizeof(int2);
    int rc = svdb::kd_scratch(t, qbytes + obytes + sbytes);
    if (!rc) rc = svdb::kd_pinned(t, std::max(qbytes, obytes));
    if (rc) return rc;
    double* hq = (double*)t->pin;
    for (size_t i = 0; i < nq; ++i) std::memcpy(hq + i * kd, q + i * qstride, kd * sizeof(double));
    unsigned char* base = (unsigned char*)t->scratch;
    double* dq = (double*)base;
    int64_t* dout = (int64_t*)(base + qbytes);
    int2* gst = (int2*)(base + qbytes + obytes);
    SVDB_CUDA(cudaMemcpyAsync(dq, hq, nq * kd * sizeof(double), cudaMemcpyHostToDevice, t->stream));
    const unsigned blocks = (unsigned)((nq + 127) / 128);
    if (local)
        svdb::k_kd_nearest<64><<<blocks, 128, 0, t->stream>>>(t->pts, t->index, t->child, (int)kd, (int64_t)t->n, dq,
                                                              kd, (int)nq, dout, nullptr, h);
    else
        svdb::k_kd_nearest<0><<<blocks, 128, 0, t->stream>>>(t->pts, t->index, t->child, (int)kd, (int64_t)t->n, dq,
                                                             kd, (int)nq, dout, gst, h);
    SVDB_LAUNCH_CHECK();
    SVDB_CUDA(cudaMemcpyAsync(t->pin, dout, nq * sizeof(int64_t), cudaMemcpyDeviceToHost, t->stream));
    SVDB_CUDA(cudaStreamSynchronize(t->stream));
    std::memcpy(out, t->pin, nq * sizeof(int64_t));
    return SVDB_OK;
}

}  // extern "C"
