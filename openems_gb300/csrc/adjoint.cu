// adjoint.cu -- reverse-mode (adjoint) EC-FDTD: gradients of an objective built from probe
// samples with respect to the voltage coefficients (vv, vi) of the edges in a design box.
//
// One forward timestep (FDTD/engine.cpp:267-286 with the UPML hooks of
// FDTD/extensions/engine_ext_upml.cpp:52-229 and the additive excitation of
// FDTD/extensions/engine_ext_excitation.cpp:33-94) is affine in the state (V, I, UPML fluxes):
//     V' = vv*V + vi*K_V I   (UPML pre/post around it)      I' = ii*I + iv*K_I V'
// where K_V / K_I are the curl stencils of k_update_v / k_update_i.  Its transpose, applied to
// the adjoint state (lV, lI, UPML adjoint fluxes), runs in reverse order:
//   k_adj_iwi : lI += K_V^T w (finishes the previous reverse step), then I post^T, update^T
//               (u = iv * lambda kept for the V side), pre^T
//   k_adj_v   : lV += K_I^T u, then V post^T, update^T (w = vi * lambda kept, gradient sums
//               dJ/dvv += lambda V^n, dJ/dvi += lambda K_V I^n in the design box), pre^T
//   k_adj_inject : lambda += dJ/d(probe sample at numTS = n) on the probe edges
// The curl transposes are gathers (no atomics), derived from the forward stencils including the
// reference's "same cell" read at index 0 (a shift of 0 makes the two terms cancel).
//
// Memory is bounded by checkpoints: the forward run stores the full state every K steps; the
// reverse sweep restores one K-step segment at a time, recomputes it (field updates and
// excitation only), keeps the design box's V^n and K_V I^n per step, and then walks the segment
// backwards.  Gradient sums are accumulated in double.
#include <cuda_runtime.h>

#include <algorithm>
#include <new>
#include <vector>

#include "engine_impl.h"

using namespace oems;

namespace {

struct AdjDev {
    GridDev g;
    float* lV;            // [3][S] adjoint of V
    float* lI;            // [3][S] adjoint of I
    float* wv;            // [3][S] vi * lambda (V update^T), read by the next k_adj_iwi
    float* ui;            // [3][S] iv * lambda (I update^T), 0 where I is not updated
    float* lpsi[OEMS_MAX_UPML];
    float* lphi[OEMS_MAX_UPML];
    unsigned b0[3], bn[3];
    unsigned B;
    const float* fv;      // [3][B] V^n in the design box
    const float* fc;      // [3][B] K_V I^n in the design box
    double* gvv;          // [3][B]
    double* gvi;          // [3][B]
};

__device__ __forceinline__ void coef_v(const GridDev& g, unsigned long long o, int m, float& vv, float& vi)
{
    if (g.idx) {
        const unsigned c = __ldg(g.idx + o);
        const float* t = reinterpret_cast<const float*>(g.tabV + 2 * c);
        vv = __ldg(t + m);
        vi = __ldg(t + 3 + m);
    } else {
        vv = __ldg(g.vv + m * g.S + o);
        vi = __ldg(g.vi + m * g.S + o);
    }
}

__device__ __forceinline__ void coef_i(const GridDev& g, unsigned long long o, int m, float& ii, float& iv)
{
    if (g.idx) {
        const unsigned c = __ldg(g.idx + o);
        const float* t = reinterpret_cast<const float*>(g.tabI + 2 * c);
        ii = __ldg(t + m);
        iv = __ldg(t + 3 + m);
    } else {
        ii = __ldg(g.ii + m * g.S + o);
        iv = __ldg(g.iv + m * g.S + o);
    }
}

// lI += K_V^T w, then the transposed I sub-step.
__global__ void __launch_bounds__(256) k_adj_iwi(AdjDev a)
{
    const GridDev& g = a.g;
    const unsigned x = blockIdx.y;
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned y = t / g.Pz, z = t - y * g.Pz;
    if (y >= g.Ny || z >= g.Nz) return;
    const unsigned long long S = g.S;
    const unsigned long long o = ((unsigned long long)x * g.Ny + y) * g.Pz + z;
    const unsigned long long sx = (unsigned long long)g.Ny * g.Pz, sy = g.Pz;
    const float* w = a.wv;
    auto W = [&](int m, unsigned long long off, bool ok) -> float { return ok ? __ldg(w + m * S + off) : 0.f; };
    const bool hx = x + 1 < g.Nx, hy = y + 1 < g.Ny, hz = z + 1 < g.Nz;
    // d/dI of sum_o w(o) . K_V I (o): the forward's index-0 self reads cancel the direct term
    const float d[3] = {
        fadd(fsub(fsub(W(1, o, z > 0), W(1, o + 1, hz)), W(2, o, y > 0)), W(2, o + sy, hy)),
        fadd(fsub(fsub(W(2, o, x > 0), W(2, o + sx, hx)), W(0, o, z > 0)), W(0, o + 1, hz)),
        fadd(fsub(fsub(W(0, o, y > 0), W(0, o + sy, hy)), W(1, o, x > 0)), W(1, o + sx, hx))};
    if (!(hx && hy && hz)) {            // I is never updated here: identity
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            a.lI[m * S + o] = fadd(a.lI[m * S + o], d[m]);
            a.ui[m * S + o] = 0.f;
        }
        return;
    }
    unsigned loc = 0;
    const int r = upml_find(g, x, y, z, loc);
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        const unsigned long long q = m * S + o;
        float l = fadd(a.lI[q], d[m]);                   // lambda of I after the step
        float lpost = 0.f;
        if (r >= 0) {                                    // post^T: I = h + iifn*flux, flux = I
            const UpmlDev& u = g.upml[r];
            const unsigned k = m * u.n + loc;
            lpost = l;
            l = fadd(fmul(__ldg(u.iifn + k), l), a.lphi[r][k]);
        }
        float ii, iv;
        coef_i(g, o, m, ii, iv);
        a.ui[q] = fmul(iv, l);
        l = fmul(ii, l);
        if (r >= 0) {                                    // pre^T: f = ii*I - iifo*flux; I = flux; flux = f
            const UpmlDev& u = g.upml[r];
            const unsigned k = m * u.n + loc;
            a.lphi[r][k] = fsub(l, fmul(__ldg(u.iifo + k), lpost));
            l = fmul(__ldg(u.ii + k), lpost);
        }
        a.lI[q] = l;
    }
}

// lV += K_I^T u, then the transposed V sub-step with the design-box gradient sums.
__global__ void __launch_bounds__(256) k_adj_v(AdjDev a)
{
    const GridDev& g = a.g;
    const unsigned x = blockIdx.y;
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned y = t / g.Pz, z = t - y * g.Pz;
    if (y >= g.Ny || z >= g.Nz) return;
    const unsigned long long S = g.S;
    const unsigned long long o = ((unsigned long long)x * g.Ny + y) * g.Pz + z;
    const unsigned long long sx = (unsigned long long)g.Ny * g.Pz, sy = g.Pz;
    const float* u = a.ui;
    auto U = [&](int m, unsigned long long off, bool ok) -> float { return ok ? __ldg(u + m * S + off) : 0.f; };
    const float gs[3] = {
        fadd(fsub(fsub(U(1, o, true), U(1, o - 1, z > 0)), U(2, o, true)), U(2, o - sy, y > 0)),
        fsub(fadd(fsub(U(2, o, true), U(2, o - sx, x > 0)), U(0, o - 1, z > 0)), U(0, o, true)),
        fadd(fsub(fsub(U(0, o, true), U(0, o - sy, y > 0)), U(1, o, true)), U(1, o - sx, x > 0))};
    unsigned loc = 0;
    const int r = upml_find(g, x, y, z, loc);
    int kb = -1;
    {
        const unsigned bx = x - a.b0[0], by = y - a.b0[1], bz = z - a.b0[2];
        if (bx < a.bn[0] && by < a.bn[1] && bz < a.bn[2]) kb = (int)((bx * a.bn[1] + by) * a.bn[2] + bz);
    }
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        const unsigned long long q = m * S + o;
        float l = fadd(a.lV[q], gs[m]);                 // lambda of V after the step
        float lpost = 0.f;
        if (r >= 0) {
            const UpmlDev& up = g.upml[r];
            const unsigned k = m * up.n + loc;
            lpost = l;
            l = fadd(fmul(__ldg(up.vvfn + k), l), a.lpsi[r][k]);
        }
        float vv, vi;
        coef_v(g, o, m, vv, vi);
        a.wv[q] = fmul(vi, l);
        if (kb >= 0) {                                   // the design box lies outside every UPML region
            const unsigned kk = m * a.B + kb;
            a.gvv[kk] += (double)l * (double)__ldg(a.fv + kk);
            a.gvi[kk] += (double)l * (double)__ldg(a.fc + kk);
        }
        l = fmul(vv, l);
        if (r >= 0) {
            const UpmlDev& up = g.upml[r];
            const unsigned k = m * up.n + loc;
            a.lpsi[r][k] = fsub(l, fmul(__ldg(up.vvfo + k), lpost));
            l = fmul(__ldg(up.vv + k), lpost);
        }
        a.lV[q] = l;
    }
}

struct InjDev {
    int nprobe;
    const ProbeDev* probes;    // the engine's device probe array
    const int* ids;            // objective probes
    const double* src;         // [nprobe][stride]
    unsigned stride;
    unsigned n;
    float* lV;
    float* lI;
};

// dJ/d(sample) * weight * sign into the probe edges; one thread, since probes may share edges
__global__ void k_adj_inject(InjDev d)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    for (int k = 0; k < d.nprobe; ++k) {
        const ProbeDev& p = d.probes[d.ids[k]];
        const double s = d.src[(unsigned long long)k * d.stride + d.n];
        if (s == 0.0) continue;
        float* L = p.type == 0 ? d.lV : d.lI;
        for (unsigned j = 0; j < p.nterm; ++j)
            L[p.term[j]] = fadd(L[p.term[j]], (float)(s * p.weight * (double)p.sign[j]));
    }
}

// V^n and K_V I^n (the arithmetic of update_v_cell) in the design box
__global__ void k_adj_factors(AdjDev a, float* fv, float* fc)
{
    const unsigned kb = blockIdx.x * blockDim.x + threadIdx.x;
    if (kb >= a.B) return;
    const GridDev& g = a.g;
    const unsigned bz = kb % a.bn[2], by = (kb / a.bn[2]) % a.bn[1], bx = kb / (a.bn[2] * a.bn[1]);
    const unsigned x = a.b0[0] + bx, y = a.b0[1] + by, z = a.b0[2] + bz;
    const unsigned long long S = g.S;
    const unsigned long long o = ((unsigned long long)x * g.Ny + y) * g.Pz + z;
    const unsigned long long sx = x ? (unsigned long long)g.Ny * g.Pz : 0ull;
    const unsigned long long sy = y ? (unsigned long long)g.Pz : 0ull;
    const unsigned long long sz = z ? 1ull : 0ull;
    const float* I = g.I;
    const float i0 = I[o], i1 = I[S + o], i2 = I[2 * S + o];
    fc[kb] = fadd(fsub(fsub(i2, I[2 * S + o - sy]), i1), I[S + o - sz]);
    fc[a.B + kb] = fadd(fsub(fsub(i0, I[o - sz]), i2), I[2 * S + o - sx]);
    fc[2 * a.B + kb] = fadd(fsub(fsub(i1, I[S + o - sx]), i0), I[o - sy]);
    fv[kb] = g.V[o];
    fv[a.B + kb] = g.V[S + o];
    fv[2 * a.B + kb] = g.V[2 * S + o];
}

__global__ void k_inc(unsigned* c)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) *c += 1u;
}

}  // namespace

struct oems_adjoint_state {
    unsigned K = 256;
    unsigned steps = 0;
    std::vector<std::pair<void*, size_t>> regions;   // state: V, I, UPML fluxes
    std::vector<char*> ckpt;                          // one per segment start + the end state
    AdjDev dev{};
    float* seg_fv = nullptr;
    float* seg_fc = nullptr;
    unsigned* rec_numTS = nullptr;
    std::vector<void*> allocs;
    size_t state_bytes = 0;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    float fwd_ms = 0.f, bwd_ms = 0.f;
    unsigned launches_per_reverse_step = 0;
};

namespace {

int afail(oems_cuda_engine* e, int code, const char* msg)
{
    cudaGetLastError();
    e->err = msg;
    return code;
}

template <typename T>
int aalloc(oems_cuda_engine* e, oems_adjoint_state* s, T** p, size_t count)
{
    void* q = nullptr;
    const size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
    if (cudaMalloc(&q, bytes) != cudaSuccess) return afail(e, OEMS_ERR_NOMEM, "adjoint allocation");
    s->allocs.push_back(q);
    if (cudaMemsetAsync(q, 0, bytes, e->stream) != cudaSuccess) return afail(e, OEMS_ERR_CUDA, "adjoint memset");
    *p = static_cast<T*>(q);
    return OEMS_OK;
}

int copy_state(oems_cuda_engine* e, oems_adjoint_state* s, char* ck, bool save)
{
    size_t off = 0;
    for (const auto& r : s->regions) {
        const cudaError_t c = save ? cudaMemcpyAsync(ck + off, r.first, r.second, cudaMemcpyDeviceToDevice, e->stream)
                                   : cudaMemcpyAsync(r.first, ck + off, r.second, cudaMemcpyDeviceToDevice, e->stream);
        if (c != cudaSuccess) return afail(e, OEMS_ERR_CUDA, "checkpoint copy");
        off += r.second;
    }
    return OEMS_OK;
}

// one forward step without processing, the step counter being rec_numTS; returns the launches
unsigned recompute_step(oems_cuda_engine* e, oems_adjoint_state* s)
{
    const GridDev& g = e->grid;
    const unsigned plane = e->N[1] * e->Pz;
    const dim3 gv((plane + 255) / 256, e->N[0]), gi((plane + 255) / 256, e->N[0] - 1);
    const bool up = !e->upml.empty();
    cudaStream_t st = e->stream;
    unsigned L = 3;
    if (e->compressed) { if (up) k_update_v<true, true><<<gv, 256, 0, st>>>(g); else k_update_v<true, false><<<gv, 256, 0, st>>>(g); }
    else { if (up) k_update_v<false, true><<<gv, 256, 0, st>>>(g); else k_update_v<false, false><<<gv, 256, 0, st>>>(g); }
    if (e->excV.count) { k_excitation<<<(e->excV.count + 127) / 128, 128, 0, st>>>(e->dV, e->excV, s->rec_numTS); ++L; }
    if (e->compressed) { if (up) k_update_i<true, true><<<gi, 256, 0, st>>>(g); else k_update_i<true, false><<<gi, 256, 0, st>>>(g); }
    else { if (up) k_update_i<false, true><<<gi, 256, 0, st>>>(g); else k_update_i<false, false><<<gi, 256, 0, st>>>(g); }
    if (e->excI.count) { k_excitation<<<(e->excI.count + 127) / 128, 128, 0, st>>>(e->dI, e->excI, s->rec_numTS); ++L; }
    k_inc<<<1, 32, 0, st>>>(s->rec_numTS);
    return L;
}

}  // namespace

extern "C" {

int oems_cuda_adjoint_setup(oems_cuda_engine* e, unsigned int checkpoint_every, const unsigned int box_start[3],
                            const unsigned int box_stop[3])
{
    if (!e || !box_start || !box_stop || checkpoint_every == 0) return OEMS_ERR_ARG;
    if (!e->inited) return afail(e, OEMS_ERR_STATE, "engine not initialised");
    if (e->adj) return afail(e, OEMS_ERR_STATE, "adjoint already set up");
    if (!e->mur.empty() || !e->lor.empty())
        return afail(e, OEMS_ERR_UNSUPPORTED, "adjoint: Mur walls and dispersive materials are not supported");
    for (int a = 0; a < 3; ++a)
        if (box_start[a] >= box_stop[a] || box_stop[a] > e->N[a]) return afail(e, OEMS_ERR_ARG, "adjoint: design box outside the mesh");
    for (const auto& u : e->upml) {
        bool overlap = true;
        for (int a = 0; a < 3; ++a) overlap = overlap && box_start[a] < u.start[a] + u.nl[a] && u.start[a] < box_stop[a];
        if (overlap) return afail(e, OEMS_ERR_ARG, "adjoint: design box overlaps a UPML region");
    }
    if (cudaSetDevice(e->device) != cudaSuccess) return afail(e, OEMS_ERR_CUDA, "cudaSetDevice");
    auto* s = new (std::nothrow) oems_adjoint_state();
    if (!s) return OEMS_ERR_NOMEM;
    e->adj = s;
    s->K = checkpoint_every;
    s->regions.push_back({e->dV, 3 * e->S * sizeof(float)});
    s->regions.push_back({e->dI, 3 * e->S * sizeof(float)});
    for (int r = 0; r < e->grid.nupml; ++r) {
        s->regions.push_back({e->grid.upml[r].vflux, 3ull * e->grid.upml[r].n * sizeof(float)});
        s->regions.push_back({e->grid.upml[r].iflux, 3ull * e->grid.upml[r].n * sizeof(float)});
    }
    for (const auto& r : s->regions) s->state_bytes += r.second;
    AdjDev& d = s->dev;
    d.g = e->grid;
    int rc;
    if ((rc = aalloc(e, s, &d.lV, 3 * e->S))) return rc;
    if ((rc = aalloc(e, s, &d.lI, 3 * e->S))) return rc;
    if ((rc = aalloc(e, s, &d.wv, 3 * e->S))) return rc;
    if ((rc = aalloc(e, s, &d.ui, 3 * e->S))) return rc;
    for (int r = 0; r < e->grid.nupml; ++r) {
        if ((rc = aalloc(e, s, &d.lpsi[r], 3ull * e->grid.upml[r].n))) return rc;
        if ((rc = aalloc(e, s, &d.lphi[r], 3ull * e->grid.upml[r].n))) return rc;
    }
    d.B = 1;
    for (int a = 0; a < 3; ++a) {
        d.b0[a] = box_start[a];
        d.bn[a] = box_stop[a] - box_start[a];
        d.B *= d.bn[a];
    }
    if ((rc = aalloc(e, s, &d.gvv, 3ull * d.B))) return rc;
    if ((rc = aalloc(e, s, &d.gvi, 3ull * d.B))) return rc;
    if ((rc = aalloc(e, s, &s->seg_fv, 3ull * d.B * s->K))) return rc;
    if ((rc = aalloc(e, s, &s->seg_fc, 3ull * d.B * s->K))) return rc;
    if ((rc = aalloc(e, s, &s->rec_numTS, 1))) return rc;
    if (cudaEventCreate(&s->ev[0]) != cudaSuccess || cudaEventCreate(&s->ev[1]) != cudaSuccess)
        return afail(e, OEMS_ERR_CUDA, "adjoint events");
    if (cudaStreamSynchronize(e->stream) != cudaSuccess) return afail(e, OEMS_ERR_CUDA, "adjoint setup sync");
    return OEMS_OK;
}

int oems_cuda_adjoint_forward(oems_cuda_engine* e, unsigned int steps)
{
    if (!e || !e->adj) return OEMS_ERR_STATE;
    oems_adjoint_state* s = e->adj;
    if (e->host_numTS != 0) return afail(e, OEMS_ERR_STATE, "adjoint forward must start at numTS = 0");
    if (steps == 0 || steps > e->max_ts) return afail(e, OEMS_ERR_ARG, "adjoint forward: bad step count");
    for (char* c : s->ckpt) cudaFree(c);
    s->ckpt.clear();
    s->steps = 0;
    const unsigned nseg = (steps + s->K - 1) / s->K;
    for (unsigned k = 0; k <= nseg; ++k) {
        char* c = nullptr;
        if (cudaMalloc(&c, s->state_bytes) != cudaSuccess) return afail(e, OEMS_ERR_NOMEM, "checkpoint allocation");
        s->ckpt.push_back(c);
    }
    cudaEventRecord(s->ev[0], e->stream);
    for (unsigned k = 0; k < nseg; ++k) {
        int rc = copy_state(e, s, s->ckpt[k], true);
        if (rc) return rc;
        const unsigned n = std::min(s->K, steps - k * s->K);
        if ((rc = oems_cuda_iterate(e, n))) return rc;
    }
    int rc = copy_state(e, s, s->ckpt[nseg], true);
    if (rc) return rc;
    cudaEventRecord(s->ev[1], e->stream);
    if (cudaEventSynchronize(s->ev[1]) != cudaSuccess) return afail(e, OEMS_ERR_CUDA, "adjoint forward sync");
    cudaEventElapsedTime(&s->fwd_ms, s->ev[0], s->ev[1]);
    s->steps = steps;
    return OEMS_OK;
}

int oems_cuda_adjoint_backward(oems_cuda_engine* e, unsigned int nprobe, const int* probe_ids, const double* sources,
                               double* gvv, double* gvi)
{
    if (!e || !e->adj) return OEMS_ERR_STATE;
    oems_adjoint_state* s = e->adj;
    if (!s->steps) return afail(e, OEMS_ERR_STATE, "adjoint backward before forward");
    if (!gvv || !gvi || (nprobe && (!probe_ids || !sources))) return OEMS_ERR_ARG;
    for (unsigned k = 0; k < nprobe; ++k)
        if (probe_ids[k] < 0 || probe_ids[k] >= (int)e->probe_dev.size()) return afail(e, OEMS_ERR_ARG, "bad probe id");
    AdjDev& d = s->dev;
    cudaStream_t st = e->stream;
    const unsigned N = s->steps;
    const size_t nsrc = (size_t)nprobe * (N + 1);
    int* dids = nullptr;
    double* dsrc = nullptr;
    if (cudaMalloc(&dids, std::max(1u, nprobe) * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&dsrc, std::max<size_t>(1, nsrc) * sizeof(double)) != cudaSuccess) {
        cudaFree(dids);
        return afail(e, OEMS_ERR_NOMEM, "adjoint source allocation");
    }
    cudaEventRecord(s->ev[0], st);
    if (nprobe) {
        cudaMemcpyAsync(dids, probe_ids, nprobe * sizeof(int), cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(dsrc, sources, nsrc * sizeof(double), cudaMemcpyHostToDevice, st);
    }
    cudaMemsetAsync(d.lV, 0, 3 * e->S * sizeof(float), st);
    cudaMemsetAsync(d.lI, 0, 3 * e->S * sizeof(float), st);
    cudaMemsetAsync(d.wv, 0, 3 * e->S * sizeof(float), st);
    for (int r = 0; r < e->grid.nupml; ++r) {
        cudaMemsetAsync(d.lpsi[r], 0, 3ull * e->grid.upml[r].n * sizeof(float), st);
        cudaMemsetAsync(d.lphi[r], 0, 3ull * e->grid.upml[r].n * sizeof(float), st);
    }
    cudaMemsetAsync(d.gvv, 0, 3ull * d.B * sizeof(double), st);
    cudaMemsetAsync(d.gvi, 0, 3ull * d.B * sizeof(double), st);
    InjDev inj{};
    inj.nprobe = (int)nprobe;
    inj.probes = e->stepend.probes;
    inj.ids = dids;
    inj.src = dsrc;
    inj.stride = N + 1;
    inj.lV = d.lV;
    inj.lI = d.lI;
    inj.n = N;
    k_adj_inject<<<1, 32, 0, st>>>(inj);
    const unsigned plane = e->N[1] * e->Pz;
    const dim3 grid((plane + 255) / 256, e->N[0]);
    const unsigned nseg = (N + s->K - 1) / s->K;
    int rc = OEMS_OK;
    unsigned lps = 0;
    for (int seg = (int)nseg - 1; seg >= 0 && rc == OEMS_OK; --seg) {
        const unsigned a0 = seg * s->K, a1 = std::min(N, a0 + s->K);
        if ((rc = copy_state(e, s, s->ckpt[seg], false))) break;
        cudaMemcpyAsync(s->rec_numTS, &a0, sizeof(unsigned), cudaMemcpyHostToDevice, st);
        for (unsigned n = a0; n < a1; ++n) {
            const size_t off = (size_t)(n - a0) * 3 * d.B;
            k_adj_factors<<<(d.B + 255) / 256, 256, 0, st>>>(d, s->seg_fv + off, s->seg_fc + off);
            lps = 1 + recompute_step(e, s);
        }
        for (int n = (int)a1 - 1; n >= (int)a0; --n) {
            const size_t off = (size_t)(n - a0) * 3 * d.B;
            d.fv = s->seg_fv + off;
            d.fc = s->seg_fc + off;
            k_adj_iwi<<<grid, 256, 0, st>>>(d);
            k_adj_v<<<grid, 256, 0, st>>>(d);
            inj.n = (unsigned)n;
            k_adj_inject<<<1, 32, 0, st>>>(inj);
        }
        if (cudaGetLastError() != cudaSuccess) rc = afail(e, OEMS_ERR_CUDA, "adjoint launch");
    }
    s->launches_per_reverse_step = lps + 3;
    // leave the engine at its forward end state
    if (rc == OEMS_OK) rc = copy_state(e, s, s->ckpt[nseg], false);
    if (rc == OEMS_OK) {
        cudaMemcpyAsync(gvv, d.gvv, 3ull * d.B * sizeof(double), cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(gvi, d.gvi, 3ull * d.B * sizeof(double), cudaMemcpyDeviceToHost, st);
        cudaEventRecord(s->ev[1], st);
        if (cudaEventSynchronize(s->ev[1]) != cudaSuccess) rc = afail(e, OEMS_ERR_CUDA, "adjoint sync");
        else cudaEventElapsedTime(&s->bwd_ms, s->ev[0], s->ev[1]);
    } else {
        cudaStreamSynchronize(st);
    }
    cudaFree(dids);
    cudaFree(dsrc);
    return rc;
}

int oems_cuda_adjoint_timing(const oems_cuda_engine* e, float* forward_ms, float* backward_ms,
                             unsigned int* launches_per_reverse_step)
{
    if (!e || !e->adj) return OEMS_ERR_STATE;
    if (forward_ms) *forward_ms = e->adj->fwd_ms;
    if (backward_ms) *backward_ms = e->adj->bwd_ms;
    if (launches_per_reverse_step) *launches_per_reverse_step = e->adj->launches_per_reverse_step;
    return OEMS_OK;
}

}  // extern "C"

void oems_adjoint_free(oems_adjoint_state* s)
{
    if (!s) return;
    for (char* c : s->ckpt) cudaFree(c);
    for (void* p : s->allocs) cudaFree(p);
    for (cudaEvent_t ev : s->ev)
        if (ev) cudaEventDestroy(ev);
    delete s;
}
