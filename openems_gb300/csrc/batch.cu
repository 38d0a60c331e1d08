// batch.cu -- batched form: many independent simulations of uneven size and step count advance
// together in persistent, grid-synchronised launches captured in one CUDA graph.
//
// Each instance is an ordinary engine handle (oems_cuda_init done), so its device state,
// probes and results are the same objects the serial engine uses.  A persistent launch runs a
// chunk of timesteps for the instances that are active throughout that chunk; chunk boundaries
// are the instances' step targets, so no launch carries finished instances.  Per step:
//   phase V : every cell of every active instance (update_v_cell, UPML fused) + its soft
//             voltage sources (Engine_Ext_Excitation::Apply2Voltages fused on the owning thread)
//   barrier
//   phase I : update_i_cell + soft current sources
//   barrier
//   phase P : probes of each instance at numTS+1 (ProcessIntegral::Process), then ++numTS
//   barrier
// The grid barrier is a counter/generation pair in device memory; every wait is bounded and
// raises an error flag (the launch then ends) instead of spinning forever.  The launch is
// cooperative, so all blocks are co-resident.
//
// Work items: (instance, run of `depth` x-planes, chunk of blockDim cells of the y-z plane);
// the block size and the depth are chosen by timing candidates on the first steps of the run
// (the per-cell arithmetic does not depend on the decomposition, so tuning steps are real
// steps and results stay bit-exact).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "engine_impl.h"

using namespace oems;

namespace {

constexpr unsigned kMaxFusedSources = 64;
constexpr unsigned long long kSpinLimit = 1ull << 24;   // ~2 s of __nanosleep(100) polls

struct BatchInst {
    GridDev g;
    ExcDev ev, ei;
    const ProbeDev* probes;
    int nprobe;
    unsigned* numTS;
    int compressed, upml;
    unsigned xitV, xitI;       // x-runs per instance (ceil(Nx/depth), ceil((Nx-1)/depth))
    unsigned pchunk;           // plane chunks: ceil(Ny*Pz / blockDim)
    unsigned vbox[6], ibox[6]; // bounding boxes (x0,x1,y0,y1,z0,z1 inclusive) of the source cells
};

// the block's current instance descriptor, staged in shared memory (descriptor reads then cost
// a shared load instead of a global one per cell)
__device__ __forceinline__ void stage_inst(BatchInst* dst, const BatchInst* src)
{
    __syncthreads();
    const unsigned* s = reinterpret_cast<const unsigned*>(src);
    unsigned* d = reinterpret_cast<unsigned*>(dst);
    for (unsigned i = threadIdx.x; i < sizeof(BatchInst) / 4; i += blockDim.x) d[i] = __ldg(s + i);
    __syncthreads();
}

__device__ __forceinline__ bool in_box(const unsigned* b, unsigned x, unsigned y, unsigned z)
{
    return x >= b[0] && x <= b[1] && y >= b[2] && y <= b[3] && z >= b[4] && z <= b[5];
}

struct GridBar {
    unsigned count;
    unsigned gen;
    unsigned err;
};

struct BatchDev {
    const BatchInst* inst;     // active instances of this chunk
    const unsigned* prefV;     // item prefix sums, size n+1
    const unsigned* prefI;
    int n;
    unsigned steps;
    unsigned depth;
    GridBar* bar;
};

__device__ __forceinline__ bool grid_barrier(GridBar* b)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* vgen = &b->gen;
        const unsigned g = *vgen;
        __threadfence();
        if (atomicAdd(&b->count, 1u) == gridDim.x - 1) {
            atomicExch(&b->count, 0u);
            __threadfence();
            atomicAdd(&b->gen, 1u);
        } else {
            unsigned long long spins = 0;
            while (*vgen == g) {
                if (++spins > kSpinLimit) { atomicExch(&b->err, 1u); break; }
                __nanosleep(100);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return *(volatile unsigned*)&b->err == 0u;
}

__device__ __forceinline__ int find_inst(const unsigned* pref, int n, unsigned item)
{
    int lo = 0, hi = n - 1;   // largest k with pref[k] <= item
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (pref[mid] <= item) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// soft source add on the thread that owns the cell (same arithmetic as k_excitation)
__device__ __forceinline__ void fused_sources(float* F, const ExcDev& e, int ts, unsigned long long o,
                                              unsigned long long S)
{
    for (unsigned k = 0; k < e.count; ++k) {
        const unsigned long long off = e.off[k];
        if (off != o && off != o + S && off != o + 2 * S) continue;
        const int p = e.period ? (int)e.period : ts + 1;
        int exc_pos = ts - (int)e.delay[k];
        exc_pos *= (exc_pos > 0);
        exc_pos %= p;
        exc_pos *= (exc_pos < (int)e.length);
        F[off] = fadd(__ldcg(F + off), fmul(e.amp[k], e.sig[exc_pos]));
    }
}

__global__ void __launch_bounds__(512) k_batch(BatchDev b)
{
    __shared__ __align__(16) unsigned char s_raw[sizeof(BatchInst)];
    BatchInst& in = *reinterpret_cast<BatchInst*>(s_raw);
    const unsigned totV = b.prefV[b.n], totI = b.prefI[b.n];
    for (unsigned step = 0; step < b.steps; ++step) {
        // ---- phase V
        int cur = -1;
        for (unsigned item = blockIdx.x; item < totV; item += gridDim.x) {
            const int k = find_inst(b.prefV, b.n, item);
            if (k != cur) { stage_inst(&in, b.inst + k); cur = k; }
            const GridDev& g = in.g;
            const unsigned local = item - b.prefV[k];
            const unsigned xr = local / in.pchunk, pc = local - xr * in.pchunk;
            const unsigned t = pc * blockDim.x + threadIdx.x;
            const unsigned y = t / g.Pz, z = t - y * g.Pz;
            if (y < g.Ny && z < g.Nz) {
                const int ts = (int)__ldcg(in.numTS);
                const unsigned x0 = xr * b.depth, x1 = min(x0 + b.depth, g.Nx);
                for (unsigned x = x0; x < x1; ++x) {
                    if (in.compressed) {
                        if (in.upml) update_v_cell<true, true, true>(g, x, y, z); else update_v_cell<true, false, true>(g, x, y, z);
                    } else {
                        if (in.upml) update_v_cell<false, true, true>(g, x, y, z); else update_v_cell<false, false, true>(g, x, y, z);
                    }
                    if (in.ev.count && in_box(in.vbox, x, y, z))
                        fused_sources(g.V, in.ev, ts, ((unsigned long long)x * g.Ny + y) * g.Pz + z, g.S);
                }
            }
        }
        if (!grid_barrier(b.bar)) return;
        // ---- phase I
        cur = -1;
        for (unsigned item = blockIdx.x; item < totI; item += gridDim.x) {
            const int k = find_inst(b.prefI, b.n, item);
            if (k != cur) { stage_inst(&in, b.inst + k); cur = k; }
            const GridDev& g = in.g;
            const unsigned local = item - b.prefI[k];
            const unsigned xr = local / in.pchunk, pc = local - xr * in.pchunk;
            const unsigned t = pc * blockDim.x + threadIdx.x;
            const unsigned y = t / g.Pz, z = t - y * g.Pz;
            if (y + 1 < g.Ny && z + 1 < g.Nz) {
                const int ts = (int)__ldcg(in.numTS);
                const unsigned x0 = xr * b.depth, x1 = min(x0 + b.depth, g.Nx - 1);
                for (unsigned x = x0; x < x1; ++x) {
                    if (in.compressed) {
                        if (in.upml) update_i_cell<true, true, true>(g, x, y, z); else update_i_cell<true, false, true>(g, x, y, z);
                    } else {
                        if (in.upml) update_i_cell<false, true, true>(g, x, y, z); else update_i_cell<false, false, true>(g, x, y, z);
                    }
                    if (in.ei.count && in_box(in.ibox, x, y, z))
                        fused_sources(g.I, in.ei, ts, ((unsigned long long)x * g.Ny + y) * g.Pz + z, g.S);
                }
            }
        }
        if (!grid_barrier(b.bar)) return;
        // ---- phase P: probes at the completed step, then advance numTS
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        for (int k = blockIdx.x; k < b.n; k += gridDim.x) {
            stage_inst(&in, b.inst + k);
            const unsigned ts = __ldcg(in.numTS) + 1;
            for (int p = warp; p < in.nprobe; p += blockDim.x >> 5) probe_eval(in.g, in.probes[p], ts, lane);
            __syncthreads();
            if (threadIdx.x == 0) *in.numTS = ts;
        }
        if (!grid_barrier(b.bar)) return;
    }
}

// ---- per-phase launches: one block per work item; kernel boundaries order the phases, so
// the read-only path (__ldg) is valid and no grid barrier is needed.
__global__ void __launch_bounds__(512) k_bv(BatchDev b)
{
    __shared__ __align__(16) unsigned char s_raw[sizeof(BatchInst)];
    BatchInst& in = *reinterpret_cast<BatchInst*>(s_raw);
    const unsigned item = blockIdx.x;
    const int k = find_inst(b.prefV, b.n, item);
    stage_inst(&in, b.inst + k);
    const GridDev& g = in.g;
    const unsigned local = item - b.prefV[k];
    const unsigned xr = local / in.pchunk, pc = local - xr * in.pchunk;
    const unsigned t = pc * blockDim.x + threadIdx.x;
    const unsigned y = t / g.Pz, z = t - y * g.Pz;
    if (y >= g.Ny || z >= g.Nz) return;
    const int ts = (int)*in.numTS;
    const unsigned x0 = xr * b.depth, x1 = min(x0 + b.depth, g.Nx);
    for (unsigned x = x0; x < x1; ++x) {
        if (in.compressed) {
            if (in.upml) update_v_cell<true, true>(g, x, y, z); else update_v_cell<true, false>(g, x, y, z);
        } else {
            if (in.upml) update_v_cell<false, true>(g, x, y, z); else update_v_cell<false, false>(g, x, y, z);
        }
        if (in.ev.count && in_box(in.vbox, x, y, z))
            fused_sources(g.V, in.ev, ts, ((unsigned long long)x * g.Ny + y) * g.Pz + z, g.S);
    }
}

__global__ void __launch_bounds__(512) k_bi(BatchDev b)
{
    __shared__ __align__(16) unsigned char s_raw[sizeof(BatchInst)];
    BatchInst& in = *reinterpret_cast<BatchInst*>(s_raw);
    const unsigned item = blockIdx.x;
    const int k = find_inst(b.prefI, b.n, item);
    stage_inst(&in, b.inst + k);
    const GridDev& g = in.g;
    const unsigned local = item - b.prefI[k];
    const unsigned xr = local / in.pchunk, pc = local - xr * in.pchunk;
    const unsigned t = pc * blockDim.x + threadIdx.x;
    const unsigned y = t / g.Pz, z = t - y * g.Pz;
    if (y + 1 >= g.Ny || z + 1 >= g.Nz) return;
    const int ts = (int)*in.numTS;
    const unsigned x0 = xr * b.depth, x1 = min(x0 + b.depth, g.Nx - 1);
    for (unsigned x = x0; x < x1; ++x) {
        if (in.compressed) {
            if (in.upml) update_i_cell<true, true>(g, x, y, z); else update_i_cell<true, false>(g, x, y, z);
        } else {
            if (in.upml) update_i_cell<false, true>(g, x, y, z); else update_i_cell<false, false>(g, x, y, z);
        }
        if (in.ei.count && in_box(in.ibox, x, y, z))
            fused_sources(g.I, in.ei, ts, ((unsigned long long)x * g.Ny + y) * g.Pz + z, g.S);
    }
}

__global__ void __launch_bounds__(256) k_bp(BatchDev b)
{
    const int k = blockIdx.x;
    const BatchInst& in = b.inst[k];
    const unsigned ts = *in.numTS + 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int p = warp; p < in.nprobe; p += blockDim.x >> 5) probe_eval(in.g, in.probes[p], ts, lane);
    __syncthreads();
    if (threadIdx.x == 0) *in.numTS = ts;
}

}  // namespace

struct oems_cuda_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<oems_cuda_engine*> eng;
    GridBar* bar = nullptr;
    std::vector<void*> allocs;
    int mode = -1;                      // tuned mode (see kCands)
    size_t l2_budget = 0;               // bytes of instance state per group in mode 2
    unsigned block = 0, depth = 0;
    float tune_ms[16] = {0};
    unsigned ncand = 0;
    bool used_graph = false;
    int sms = 0;
};

namespace {

struct Cand {
    int mode;
    unsigned block, depth;
};
// mode 0: one persistent launch per chunk; 1: per-phase launches over every active instance;
// 2: per-phase launches over L2-sized groups of instances (each group runs the chunk's steps
// while its state stays in L2, then the next group); 3: concurrent graph branches, one per
// instance, each running that instance's own step kernels; 4: mode 3 over L2-sized groups
const Cand kCands[] = {{0, 128, 1}, {0, 256, 4}, {0, 512, 4},
                       {1, 128, 1}, {1, 256, 1}, {1, 256, 2}, {1, 512, 1},
                       {2, 128, 1}, {2, 256, 1}, {2, 256, 2}, {2, 512, 1}, {3, 256, 1}, {4, 256, 1}};
constexpr unsigned kNumCands = sizeof(kCands) / sizeof(kCands[0]);
constexpr unsigned kGraphSteps = 16;

int bfail(oems_cuda_batch* b, int code)
{
    (void)b;
    cudaGetLastError();
    return code;
}

BatchInst make_inst(const oems_cuda_engine* e, unsigned block, unsigned depth)
{
    BatchInst in{};
    in.g = e->grid;
    in.ev = e->excV;
    in.ei = e->excI;
    in.probes = e->stepend.probes;
    in.nprobe = e->stepend.nprobe;
    in.numTS = e->d_numTS;
    in.compressed = e->compressed ? 1 : 0;
    in.upml = e->upml.empty() ? 0 : 1;
    in.xitV = (e->N[0] + depth - 1) / depth;
    in.xitI = (e->N[0] - 1 + depth - 1) / depth;
    in.pchunk = (e->N[1] * e->Pz + block - 1) / block;
    // source bounding boxes from the linear offsets
    auto box = [&](const std::vector<unsigned long long>& offs, unsigned* bx) {
        bx[0] = bx[2] = bx[4] = 0xFFFFFFFFu;
        bx[1] = bx[3] = bx[5] = 0u;
        for (unsigned long long o : offs) {
            const unsigned long long c = o % e->S;
            const unsigned z = (unsigned)(c % e->Pz);
            const unsigned y = (unsigned)((c / e->Pz) % e->N[1]);
            const unsigned x = (unsigned)(c / ((unsigned long long)e->Pz * e->N[1]));
            bx[0] = std::min(bx[0], x); bx[1] = std::max(bx[1], x);
            bx[2] = std::min(bx[2], y); bx[3] = std::max(bx[3], y);
            bx[4] = std::min(bx[4], z); bx[5] = std::max(bx[5], z);
        }
    };
    box(e->exc_voff, in.vbox);
    box(e->exc_ioff, in.ibox);
    return in;
}

// device bytes an instance streams per step (fields, class index, UPML fluxes and class index)
size_t instance_bytes(const oems_cuda_engine* e)
{
    size_t b = e->S * (3 * 4 * 2 + 4);
    for (int r = 0; r < e->grid.nupml; ++r) {
        const UpmlDev& u = e->grid.upml[r];
        b += (size_t)u.n * (3 * 4 * 2 + (u.cls ? 2 : 3 * 4 * 6));
    }
    return b;
}

struct Chunk {
    BatchDev d;
    unsigned totV, totI;
};

// upload one chunk's descriptor (instances + prefix sums) into device memory owned by the batch
int upload_chunk(oems_cuda_batch* b, const std::vector<int>& active, unsigned block, unsigned depth, unsigned steps,
                 Chunk* out)
{
    std::vector<BatchInst> inst;
    std::vector<unsigned> pv(1, 0u), pi(1, 0u);
    for (int k : active) {
        inst.push_back(make_inst(b->eng[k], block, depth));
        pv.push_back(pv.back() + inst.back().xitV * inst.back().pchunk);
        pi.push_back(pi.back() + inst.back().xitI * inst.back().pchunk);
    }
    void *di = nullptr, *dv = nullptr, *dpi = nullptr;
    if (cudaMalloc(&di, inst.size() * sizeof(BatchInst)) != cudaSuccess) return bfail(b, OEMS_ERR_NOMEM);
    b->allocs.push_back(di);
    if (cudaMalloc(&dv, pv.size() * sizeof(unsigned)) != cudaSuccess) return bfail(b, OEMS_ERR_NOMEM);
    b->allocs.push_back(dv);
    if (cudaMalloc(&dpi, pi.size() * sizeof(unsigned)) != cudaSuccess) return bfail(b, OEMS_ERR_NOMEM);
    b->allocs.push_back(dpi);
    if (cudaMemcpy(di, inst.data(), inst.size() * sizeof(BatchInst), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dv, pv.data(), pv.size() * sizeof(unsigned), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dpi, pi.data(), pi.size() * sizeof(unsigned), cudaMemcpyHostToDevice) != cudaSuccess)
        return bfail(b, OEMS_ERR_CUDA);
    out->d.inst = static_cast<const BatchInst*>(di);
    out->d.prefV = static_cast<const unsigned*>(dv);
    out->d.prefI = static_cast<const unsigned*>(dpi);
    out->d.n = (int)active.size();
    out->d.steps = steps;
    out->d.depth = depth;
    out->d.bar = b->bar;
    out->totV = pv.back();
    out->totI = pi.back();
    return OEMS_OK;
}

// persistent mode: the whole chunk in one cooperative launch
int launch_persistent(oems_cuda_batch* b, const Chunk& c, unsigned block)
{
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch, (int)block, 0) != cudaSuccess || per_sm < 1)
        return bfail(b, OEMS_ERR_CUDA);
    const unsigned grid = (unsigned)(per_sm * b->sms);
    BatchDev arg = c.d;
    void* args[] = {&arg};
    cudaError_t e = cudaLaunchCooperativeKernel((const void*)k_batch, dim3(grid), dim3(block), args, 0, b->stream);
    if (e != cudaSuccess) return bfail(b, OEMS_ERR_CUDA);
    return OEMS_OK;
}

// per-phase mode: `steps` timesteps as 3 launches each
int launch_phases(oems_cuda_batch* b, const Chunk& c, unsigned block, unsigned steps)
{
    for (unsigned s = 0; s < steps; ++s) {
        k_bv<<<c.totV, block, 0, b->stream>>>(c.d);
        k_bi<<<c.totI, block, 0, b->stream>>>(c.d);
        k_bp<<<c.d.n, 256, 0, b->stream>>>(c.d);
    }
    if (cudaGetLastError() != cudaSuccess) return OEMS_ERR_CUDA;
    return OEMS_OK;
}

int capture_phases(oems_cuda_batch* b, const Chunk& c, unsigned block, unsigned steps, cudaGraphExec_t* exec)
{
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return bfail(b, OEMS_ERR_CUDA);
    int rc = launch_phases(b, c, block, steps);
    cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
    if (rc || e != cudaSuccess || !graph) { if (graph) cudaGraphDestroy(graph); return bfail(b, OEMS_ERR_CUDA); }
    e = cudaGraphInstantiate(exec, graph, 0);
    cudaGraphDestroy(graph);
    return e == cudaSuccess ? OEMS_OK : bfail(b, OEMS_ERR_CUDA);
}

// mode 3: one graph per chunk whose branches are the instances' own step sequences (each on
// its engine's stream, forked from and joined to the batch stream), so instances of different
// sizes run concurrently with their specialised kernels.
int capture_concurrent(oems_cuda_batch* b, const std::vector<int>& act, unsigned steps, cudaGraphExec_t* exec)
{
    cudaEvent_t fork;
    if (cudaEventCreateWithFlags(&fork, cudaEventDisableTiming) != cudaSuccess) return bfail(b, OEMS_ERR_CUDA);
    std::vector<cudaEvent_t> join(act.size(), nullptr);
    for (auto& j : join) cudaEventCreateWithFlags(&j, cudaEventDisableTiming);
    cudaGraph_t graph = nullptr;
    int rc = OEMS_OK;
    if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) rc = OEMS_ERR_CUDA;
    if (rc == OEMS_OK && cudaEventRecord(fork, b->stream) != cudaSuccess) rc = OEMS_ERR_CUDA;
    for (size_t i = 0; i < act.size() && rc == OEMS_OK; ++i) {
        oems_cuda_engine* e = b->eng[act[i]];
        if (cudaStreamWaitEvent(e->stream, fork, 0) != cudaSuccess) { rc = OEMS_ERR_CUDA; break; }
        for (unsigned s = 0; s < steps && rc == OEMS_OK; ++s)
            rc = enqueue_step(e, nullptr, nullptr, (s == 0 ? 1u : 0u) | (s + 1 == steps ? 2u : 0u));
        if (rc == OEMS_OK && (cudaEventRecord(join[i], e->stream) != cudaSuccess ||
                              cudaStreamWaitEvent(b->stream, join[i], 0) != cudaSuccess))
            rc = OEMS_ERR_CUDA;
    }
    cudaError_t c = cudaStreamEndCapture(b->stream, &graph);
    if (rc == OEMS_OK && (c != cudaSuccess || !graph)) rc = OEMS_ERR_CUDA;
    if (rc == OEMS_OK && cudaGraphInstantiate(exec, graph, 0) != cudaSuccess) rc = OEMS_ERR_CUDA;
    if (graph) cudaGraphDestroy(graph);
    cudaEventDestroy(fork);
    for (auto& j : join) cudaEventDestroy(j);
    if (rc) cudaGetLastError();
    return rc;
}

// ev (optional): two events recorded around the launches only, after every graph is built
int run_concurrent(oems_cuda_batch* b, const std::vector<int>& act, unsigned steps, cudaEvent_t* ev)
{
    const unsigned full = steps / kGraphSteps, tail = steps % kGraphSteps;
    cudaGraphExec_t g16 = nullptr, g1 = nullptr;
    int rc = OEMS_OK;
    if (full && (rc = capture_concurrent(b, act, kGraphSteps, &g16))) return rc;
    if (tail && (rc = capture_concurrent(b, act, 1, &g1))) { if (g16) cudaGraphExecDestroy(g16); return rc; }
    cudaError_t e = cudaSuccess;
    if (ev) cudaEventRecord(ev[0], b->stream);
    for (unsigned r = 0; r < full && e == cudaSuccess; ++r) e = cudaGraphLaunch(g16, b->stream);
    for (unsigned r = 0; r < tail && e == cudaSuccess; ++r) e = cudaGraphLaunch(g1, b->stream);
    if (ev) cudaEventRecord(ev[1], b->stream);
    // no wait here: an executable graph destroyed while in flight is freed when it completes, and
    // the next chunk's graphs are built while this one runs
    if (g16) cudaGraphExecDestroy(g16);
    if (g1) cudaGraphExecDestroy(g1);
    return e == cudaSuccess ? OEMS_OK : bfail(b, OEMS_ERR_CUDA);
}

// mode 4: the instances in groups whose state fits the L2; each group runs the chunk's steps as
// concurrent per-instance branches (mode 3) before the next group starts.  Every group's graphs
// are built first; ev (optional) brackets the launches alone.
int run_concurrent_groups(oems_cuda_batch* b, const std::vector<std::vector<int>>& groups, unsigned steps,
                          cudaEvent_t* ev)
{
    const unsigned full = steps / kGraphSteps, tail = steps % kGraphSteps;
    std::vector<std::pair<cudaGraphExec_t, cudaGraphExec_t>> gx;
    int rc = OEMS_OK;
    for (const auto& grp : groups) {
        cudaGraphExec_t g16 = nullptr, g1 = nullptr;
        if (full && (rc = capture_concurrent(b, grp, kGraphSteps, &g16))) break;
        if (tail && (rc = capture_concurrent(b, grp, 1, &g1))) {
            if (g16) cudaGraphExecDestroy(g16);
            break;
        }
        gx.push_back({g16, g1});
    }
    cudaError_t e = cudaSuccess;
    if (rc == OEMS_OK) {
        if (ev) cudaEventRecord(ev[0], b->stream);
        for (const auto& g : gx) {
            for (unsigned r = 0; r < full && e == cudaSuccess; ++r) e = cudaGraphLaunch(g.first, b->stream);
            for (unsigned r = 0; r < tail && e == cudaSuccess; ++r) e = cudaGraphLaunch(g.second, b->stream);
        }
        if (ev) cudaEventRecord(ev[1], b->stream);
    }
    for (const auto& g : gx) {                      // freed when their launches complete
        if (g.first) cudaGraphExecDestroy(g.first);
        if (g.second) cudaGraphExecDestroy(g.second);
    }
    if (rc) return rc;
    return e == cudaSuccess ? OEMS_OK : bfail(b, OEMS_ERR_CUDA);
}

}  // namespace

extern "C" {

int oems_cuda_batch_create(oems_cuda_engine* const* engines, unsigned int count, oems_cuda_batch** out)
{
    if (!engines || !count || !out) return OEMS_ERR_ARG;
    auto* b = new (std::nothrow) oems_cuda_batch();
    if (!b) return OEMS_ERR_NOMEM;
    *out = b;
    for (unsigned k = 0; k < count; ++k) {
        oems_cuda_engine* e = engines[k];
        if (!e || !e->inited) return OEMS_ERR_STATE;
        if (k == 0) b->device = e->device;
        if (e->device != b->device) return OEMS_ERR_ARG;
        // the fused batch step covers the excitation, UPML and probe paths
        if (!e->mur.empty() || !e->lor.empty() || !e->dumps.empty() || e->has_tfsf || e->rlc.count || e->cyl_closed)
            return OEMS_ERR_UNSUPPORTED;
        if (e->excV.count > kMaxFusedSources || e->excI.count > kMaxFusedSources) return OEMS_ERR_UNSUPPORTED;
        b->eng.push_back(e);
    }
    if (cudaSetDevice(b->device) != cudaSuccess) return bfail(b, OEMS_ERR_CUDA);
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, b->device);
    if (!coop) return OEMS_ERR_UNSUPPORTED;
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
    int l2 = 0;
    cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, b->device);
    b->l2_budget = (size_t)(0.6 * (l2 > 0 ? l2 : (64 << 20)));
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) return bfail(b, OEMS_ERR_CUDA);
    if (cudaMalloc(&b->bar, sizeof(GridBar)) != cudaSuccess) return bfail(b, OEMS_ERR_NOMEM);
    if (cudaMemset(b->bar, 0, sizeof(GridBar)) != cudaSuccess) return bfail(b, OEMS_ERR_CUDA);
    return OEMS_OK;
}

void oems_cuda_batch_destroy(oems_cuda_batch* b)
{
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (void* p : b->allocs) cudaFree(p);
    if (b->bar) cudaFree(b->bar);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

// block_size: 0 = autotune; depth: x-planes per work item; the mode is encoded in depth's high
// bit (depth | 0x80000000 selects per-phase launches) for callers that pin a configuration.
int oems_cuda_batch_run(oems_cuda_batch* b, const unsigned int* steps, unsigned int block_size, unsigned int depth)
{
    if (!b || !steps) return OEMS_ERR_ARG;
    if (cudaSetDevice(b->device) != cudaSuccess) return bfail(b, OEMS_ERR_CUDA);
    const int n = (int)b->eng.size();
    std::vector<unsigned> rem(n);
    for (int k = 0; k < n; ++k) {
        oems_cuda_engine* e = b->eng[k];
        if ((unsigned long long)e->host_numTS + steps[k] > e->max_ts) return OEMS_ERR_ARG;
        rem[k] = steps[k];
        // the engines' own streams must be idle before the batch stream touches their state
        if (cudaStreamSynchronize(e->stream) != cudaSuccess) return bfail(b, OEMS_ERR_CUDA);
    }
    if (block_size) {
        if (block_size % 32 || block_size > 512) return OEMS_ERR_ARG;
        b->block = block_size;
        b->mode = (depth & 0x10000000u) ? 4 : (depth & 0x20000000u) ? 3 : (depth & 0x40000000u) ? 2
                                                                                          : ((depth & 0x80000000u) ? 1 : 0);
        b->depth = (depth & 0x0FFFFFFFu) ? (depth & 0x0FFFFFFFu) : 1;
    }
    if (cudaMemsetAsync(b->bar, 0, sizeof(GridBar), b->stream) != cudaSuccess) return bfail(b, OEMS_ERR_CUDA);
    std::vector<unsigned> levels(rem.begin(), rem.end());
    std::sort(levels.begin(), levels.end());
    levels.erase(std::unique(levels.begin(), levels.end()), levels.end());
    auto active_at = [&](unsigned level) {
        std::vector<int> a;
        for (int k = 0; k < n; ++k)
            if (rem[k] >= level) a.push_back(k);
        return a;
    };
    // run `steps` timesteps of the instances in `act` with configuration (mode, block, depth).
    // Every chunk descriptor and graph is built first; ev (optional) brackets the launches alone,
    // so the tuner compares device time, not graph construction.
    bool captured = true;
    auto run_steps = [&](const std::vector<int>& act, unsigned stp, int mode, unsigned block, unsigned depth,
                         bool use_graph, cudaEvent_t* ev) -> int {
        if (mode == 3) return run_concurrent(b, act, stp, ev);
        std::vector<std::vector<int>> groups;
        if (mode == 2 || mode == 4) {
            // consecutive instances while their state fits the budget (mode 4: the whole L2,
            // mode 2: 60 % of it)
            const size_t budget = mode == 4 ? b->l2_budget / 6 * 10 : b->l2_budget;
            size_t acc = 0;
            for (int k : act) {
                const size_t bytes = instance_bytes(b->eng[k]);
                if (groups.empty() || acc + bytes > budget) { groups.emplace_back(); acc = 0; }
                groups.back().push_back(k);
                acc += bytes;
            }
            if (mode == 4) return run_concurrent_groups(b, groups, stp, ev);
        } else {
            groups.push_back(act);
        }
        struct Prep {
            Chunk c;
            cudaGraphExec_t g16, g1;
        };
        std::vector<Prep> prep;
        const unsigned full = stp / kGraphSteps, tail = stp % kGraphSteps;
        auto release = [&]() {
            for (auto& p : prep) {
                if (p.g16) cudaGraphExecDestroy(p.g16);
                if (p.g1) cudaGraphExecDestroy(p.g1);
            }
        };
        int rc = OEMS_OK;
        for (const auto& grp : groups) {
            prep.push_back(Prep{Chunk{}, nullptr, nullptr});
            Prep& p = prep.back();
            if ((rc = upload_chunk(b, grp, block, depth, stp, &p.c))) break;
            if (mode == 0 || !use_graph) continue;
            if (full && (rc = capture_phases(b, p.c, block, kGraphSteps, &p.g16))) break;
            if (tail && (rc = capture_phases(b, p.c, block, 1, &p.g1))) break;
        }
        if (rc) { release(); return rc; }
        if (ev) cudaEventRecord(ev[0], b->stream);
        cudaError_t e = cudaSuccess;
        for (auto& p : prep) {
            if (mode == 0) {
                if ((rc = launch_persistent(b, p.c, block))) break;
            } else if (!use_graph) {
                if ((rc = launch_phases(b, p.c, block, stp))) break;
            } else {
                for (unsigned r = 0; r < full && e == cudaSuccess; ++r) e = cudaGraphLaunch(p.g16, b->stream);
                for (unsigned r = 0; r < tail && e == cudaSuccess; ++r) e = cudaGraphLaunch(p.g1, b->stream);
                if (e != cudaSuccess) break;
            }
        }
        if (ev) cudaEventRecord(ev[1], b->stream);
        release();                                  // in-flight graphs are freed on completion
        if (rc) return rc;
        return e == cudaSuccess ? OEMS_OK : bfail(b, OEMS_ERR_CUDA);
    };
    unsigned done = 0;
    // ---- autotune on the first chunk (real steps; results do not depend on the configuration)
    if (b->mode < 0) {
        const unsigned first = levels.empty() ? 0 : levels[0];
        const unsigned per = 16;
        if (first >= per * (kNumCands + 1) + 1) {
            std::vector<int> act = active_at(1);
            cudaEvent_t e0, e1;
            cudaEventCreate(&e0);
            cudaEventCreate(&e1);
            float best = 1e30f;
            int rc = run_steps(act, per, kCands[0].mode, kCands[0].block, kCands[0].depth, true, nullptr);  // warm
            if (rc) return rc;
            done += per;
            cudaEvent_t ev[2] = {e0, e1};
            for (unsigned c = 0; c < kNumCands; ++c) {
                if ((rc = run_steps(act, per, kCands[c].mode, kCands[c].block, kCands[c].depth, true, ev))) return rc;
                if (cudaEventSynchronize(e1) != cudaSuccess) return bfail(b, OEMS_ERR_CUDA);
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                b->tune_ms[c] = ms;
                if (ms < best) {
                    best = ms;
                    b->mode = kCands[c].mode;
                    b->block = kCands[c].block;
                    b->depth = kCands[c].depth;
                }
                done += per;
            }
            b->ncand = kNumCands;
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
        } else {
            b->mode = 2;
            b->block = 256;
            b->depth = 1;
        }
    }
    // ---- remaining chunks
    if (b->mode == 0) {
        // every chunk is one persistent launch; all of them captured in one graph
        std::vector<Chunk> chunks;
        unsigned prev = done;
        for (unsigned level : levels) {
            if (level <= prev) continue;
            Chunk c{};
            int rc = upload_chunk(b, active_at(level), b->block, b->depth, level - prev, &c);
            if (rc) return rc;
            chunks.push_back(c);
            prev = level;
        }
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        captured = false;
        if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
            int rc = OEMS_OK;
            for (const auto& c : chunks)
                if ((rc = launch_persistent(b, c, b->block))) break;
            cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
            if (rc == OEMS_OK && e == cudaSuccess && graph && cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess)
                captured = true;
            if (graph) cudaGraphDestroy(graph);
            cudaGetLastError();
        }
        if (captured) {
            cudaError_t e = cudaGraphLaunch(exec, b->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
            cudaGraphExecDestroy(exec);
            if (e != cudaSuccess) return bfail(b, OEMS_ERR_CUDA);
        } else {
            for (const auto& c : chunks) {
                int rc = launch_persistent(b, c, b->block);
                if (rc) return rc;
            }
        }
    } else {
        unsigned prev = done;
        for (unsigned level : levels) {
            if (level <= prev) continue;
            int rc = run_steps(active_at(level), level - prev, b->mode, b->block, b->depth, true, nullptr);
            if (rc) return rc;
            prev = level;
        }
    }
    b->used_graph = captured;
    if (cudaStreamSynchronize(b->stream) != cudaSuccess) return bfail(b, OEMS_ERR_CUDA);
    GridBar hb{};
    if (cudaMemcpy(&hb, b->bar, sizeof(GridBar), cudaMemcpyDeviceToHost) != cudaSuccess) return bfail(b, OEMS_ERR_CUDA);
    if (hb.err) return OEMS_ERR_DEVICE;
    for (int k = 0; k < n; ++k) b->eng[k]->host_numTS += steps[k];
    return OEMS_OK;
}

int oems_cuda_batch_config(const oems_cuda_batch* b, unsigned int* block_size, unsigned int* depth, int* used_graph,
                           float* tune_ms, unsigned int* ncand)
{
    if (!b) return OEMS_ERR_ARG;
    if (block_size) *block_size = b->block;
    if (depth)
        *depth = b->depth | (b->mode == 1 ? 0x80000000u : 0u) | (b->mode == 2 ? 0xC0000000u : 0u) |
                 (b->mode == 3 ? 0x20000000u : 0u) | (b->mode == 4 ? 0x10000000u : 0u);
    if (used_graph) *used_graph = b->used_graph ? 1 : 0;
    if (tune_ms) for (unsigned c = 0; c < b->ncand; ++c) tune_ms[c] = b->tune_ms[c];
    if (ncand) *ncand = b->ncand;
    return OEMS_OK;
}

}  // extern "C"
