// compress.cu -- the per-cell coefficient classes of the operator, built on the device.
//
// Operator_SSE_Compressed::CompressOperator (FDTD/operator_sse_compressed.cpp:114-175) keeps one
// copy of every distinct coefficient tuple and an index per position; its std::map walks the
// mesh serially.  Here a cell's tuple is its 12 coefficients (vv, vi, ii, iv of the three
// components), compared bitwise like SSE_coeff::operator== (:193-203), and the classes are found
// by sort + unique on the GPU:
//   1. a 64-bit hash of every cell's tuple (k_tuple_hash);
//   2. a stable radix sort of (hash, cell) pairs, so equal tuples become neighbours with their
//      cells in increasing order;
//   3. a new class starts where the hash or the tuple differs from the previous sorted entry
//      (tuples are compared in full, so a hash collision costs at most a duplicate class, never a
//      wrong one), and an inclusive scan numbers the runs;
//   4. the runs are renumbered in order of their first cell, which is the order in which the
//      serial host walk meets them (classes numbered by first appearance, x, y, z loops);
//   5. the per-cell index [Nx][Ny][Pz] and the two float4 tables are written from each class's
//      first cell.
// The dense arrays arrive in N-I-J-K order from the caller and are copied to the device once.
#include <cuda_runtime.h>

#include <cub/cub.cuh>

#include "engine_impl.h"

using namespace oems;

namespace {

__device__ __forceinline__ void tuple_of(const float* __restrict__ vv, const float* __restrict__ vi,
                                         const float* __restrict__ ii, const float* __restrict__ iv, size_t cells,
                                         size_t c, unsigned w[12])
{
#pragma unroll
    for (int n = 0; n < 3; ++n) {
        w[n] = __float_as_uint(vv[n * cells + c]);
        w[3 + n] = __float_as_uint(vi[n * cells + c]);
        w[6 + n] = __float_as_uint(ii[n * cells + c]);
        w[9 + n] = __float_as_uint(iv[n * cells + c]);
    }
}

__global__ void k_tuple_hash(const float* vv, const float* vi, const float* ii, const float* iv, size_t cells,
                             unsigned long long* key, unsigned* cell)
{
    const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cells) return;
    unsigned w[12];
    tuple_of(vv, vi, ii, iv, cells, c, w);
    unsigned long long h = 1469598103934665603ULL;
#pragma unroll
    for (int i = 0; i < 12; ++i) {
        h ^= w[i];
        h *= 1099511628211ULL;
        h ^= h >> 31;
    }
    key[c] = h;
    cell[c] = (unsigned)c;
}

// head[i] = 1 where sorted entry i starts a run of equal tuples
__global__ void k_run_heads(const float* vv, const float* vi, const float* ii, const float* iv, size_t cells,
                            const unsigned long long* key, const unsigned* cell, unsigned* head)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cells) return;
    unsigned h = 1u;
    if (i > 0 && key[i] == key[i - 1]) {
        unsigned a[12], b[12];
        tuple_of(vv, vi, ii, iv, cells, cell[i], a);
        tuple_of(vv, vi, ii, iv, cells, cell[i - 1], b);
        h = 0u;
#pragma unroll
        for (int k = 0; k < 12; ++k) h |= a[k] != b[k];
    }
    head[i] = h;
}

// first cell of every run (runs numbered 1..U by the inclusive scan)
__global__ void k_run_first(const unsigned* head, const unsigned* run, const unsigned* cell, size_t cells,
                            unsigned* first, unsigned* ids)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cells || !head[i]) return;
    first[run[i] - 1] = cell[i];
    ids[run[i] - 1] = run[i] - 1;
}

// class of run r = its rank among the runs ordered by first cell
__global__ void k_rank(const unsigned* run_by_first, unsigned U, unsigned* cls_of_run)
{
    const unsigned k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < U) cls_of_run[run_by_first[k]] = k;
}

__global__ void k_scatter_index(const unsigned* run, const unsigned* cell, const unsigned* cls_of_run, size_t cells,
                                unsigned Nz, unsigned Pz, unsigned* index)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cells) return;
    const unsigned c = cell[i];
    const unsigned row = c / Nz, z = c - row * Nz;
    index[(size_t)row * Pz + z] = cls_of_run[run[i] - 1];
}

// tables of class k from the first cell of its run (first cells sorted by cell = class order)
__global__ void k_tables(const float* vv, const float* vi, const float* ii, const float* iv, size_t cells,
                         const unsigned* first_sorted, unsigned U, float4* tabV, float4* tabI)
{
    const unsigned k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= U) return;
    const size_t c = first_sorted[k];
    tabV[2 * k] = make_float4(vv[c], vv[cells + c], vv[2 * cells + c], vi[c]);
    tabV[2 * k + 1] = make_float4(vi[cells + c], vi[2 * cells + c], 0.f, 0.f);
    tabI[2 * k] = make_float4(ii[c], ii[cells + c], ii[2 * cells + c], iv[c]);
    tabI[2 * k + 1] = make_float4(iv[cells + c], iv[2 * cells + c], 0.f, 0.f);
}

// a CUDA failure: the error text on the engine, the OEMS code returned
int cfail(oems_cuda_engine* e, cudaError_t c, const char* what)
{
    cudaGetLastError();
    e->err = std::string("operator compression: ") + what + ": " + cudaGetErrorString(c);
    return c == cudaErrorMemoryAllocation ? OEMS_ERR_NOMEM : OEMS_ERR_CUDA;
}

// a device allocation owned by the engine (freed with it)
template <class T>
cudaError_t keep(oems_cuda_engine* e, T** out, size_t n)
{
    void* q = nullptr;
    cudaError_t c = cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T));
    if (c == cudaSuccess) e->allocs.push_back(q);
    *out = (T*)q;
    return c;
}

struct Scratch {
    std::vector<void*> p;
    ~Scratch()
    {
        for (void* q : p) cudaFree(q);
    }
    template <class T>
    cudaError_t get(T** out, size_t n)
    {
        void* q = nullptr;
        cudaError_t c = cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T));
        if (c == cudaSuccess) p.push_back(q);
        *out = (T*)q;
        return c;
    }
};

}  // namespace

// 0: classes built (e->didx, e->dtabV, e->dtabI set); 1: more than `cap` classes (the caller keeps
// the dense arrays); otherwise an OEMS error code.
int compress_dense_device(oems_cuda_engine* e, const float* vv, const float* vi, const float* ii, const float* iv,
                          unsigned cap)
{
    const size_t cells = (size_t)e->N[0] * e->N[1] * e->N[2];
    if (cells >= (1ull << 32)) return 1;
    cudaStream_t s = e->stream;
    Scratch t;
    float *dvv, *dvi, *dii, *div;
    unsigned long long *key, *key2;
    unsigned *cell, *cell2, *head, *run;
#define CKS(x)                                                   \
    do {                                                         \
        cudaError_t c_ = (x);                                    \
        if (c_ != cudaSuccess) return cfail(e, c_, #x);          \
    } while (0)
    CKS(t.get(&dvv, 3 * cells));
    CKS(t.get(&dvi, 3 * cells));
    CKS(t.get(&dii, 3 * cells));
    CKS(t.get(&div, 3 * cells));
    CKS(cudaMemcpyAsync(dvv, vv, 3 * cells * sizeof(float), cudaMemcpyHostToDevice, s));
    CKS(cudaMemcpyAsync(dvi, vi, 3 * cells * sizeof(float), cudaMemcpyHostToDevice, s));
    CKS(cudaMemcpyAsync(dii, ii, 3 * cells * sizeof(float), cudaMemcpyHostToDevice, s));
    CKS(cudaMemcpyAsync(div, iv, 3 * cells * sizeof(float), cudaMemcpyHostToDevice, s));
    CKS(t.get(&key, cells));
    CKS(t.get(&key2, cells));
    CKS(t.get(&cell, cells));
    CKS(t.get(&cell2, cells));
    CKS(t.get(&head, cells));
    CKS(t.get(&run, cells));
    const unsigned blocks = (unsigned)((cells + 255) / 256);
    k_tuple_hash<<<blocks, 256, 0, s>>>(dvv, dvi, dii, div, cells, key, cell);
    CKS(cudaGetLastError());
    size_t tb = 0, tb2 = 0;
    CKS(cub::DeviceRadixSort::SortPairs(nullptr, tb, key, key2, cell, cell2, (int64_t)cells, 0, 64, s));
    CKS(cub::DeviceScan::InclusiveSum(nullptr, tb2, head, run, (int64_t)cells, s));
    void* tmp = nullptr;
    CKS(t.get((char**)&tmp, std::max(tb, tb2)));
    CKS(cub::DeviceRadixSort::SortPairs(tmp, tb, key, key2, cell, cell2, (int64_t)cells, 0, 64, s));
    k_run_heads<<<blocks, 256, 0, s>>>(dvv, dvi, dii, div, cells, key2, cell2, head);
    CKS(cudaGetLastError());
    CKS(cub::DeviceScan::InclusiveSum(tmp, tb2, head, run, (int64_t)cells, s));
    unsigned U = 0;
    CKS(cudaMemcpyAsync(&U, run + (cells - 1), sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    CKS(cudaStreamSynchronize(s));
    if (U > cap) return 1;
    unsigned *first, *ids, *first2, *ids2, *cls_of_run;
    CKS(t.get(&first, U));
    CKS(t.get(&ids, U));
    CKS(t.get(&first2, U));
    CKS(t.get(&ids2, U));
    CKS(t.get(&cls_of_run, U));
    k_run_first<<<blocks, 256, 0, s>>>(head, run, cell2, cells, first, ids);
    CKS(cudaGetLastError());
    size_t tb3 = 0;
    CKS(cub::DeviceRadixSort::SortPairs(nullptr, tb3, first, first2, ids, ids2, (int)U, 0, 32, s));
    void* tmp3 = nullptr;
    CKS(t.get((char**)&tmp3, tb3));
    CKS(cub::DeviceRadixSort::SortPairs(tmp3, tb3, first, first2, ids, ids2, (int)U, 0, 32, s));
    const unsigned ublocks = (U + 255) / 256;
    k_rank<<<ublocks, 256, 0, s>>>(ids2, U, cls_of_run);
    const size_t nidx = (size_t)e->N[0] * e->N[1] * e->Pz;
    CKS(keep(e, &e->didx, nidx));
    CKS(cudaMemsetAsync(e->didx, 0, nidx * sizeof(unsigned), s));   // padding lanes: class 0
    CKS(keep(e, &e->dtabV, 2 * (size_t)U));
    CKS(keep(e, &e->dtabI, 2 * (size_t)U));
    k_scatter_index<<<blocks, 256, 0, s>>>(run, cell2, cls_of_run, cells, e->N[2], e->Pz, e->didx);
    k_tables<<<ublocks, 256, 0, s>>>(dvv, dvi, dii, div, cells, first2, U, e->dtabV, e->dtabI);
    CKS(cudaGetLastError());
    CKS(cudaStreamSynchronize(s));
#undef CKS
    e->compressed = true;
    e->nclasses = U;
    e->op_set = true;
    return OEMS_OK;
}
