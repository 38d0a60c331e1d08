// engine.cu -- host side of the GB300 EC-FDTD engine: the C ABI of include/oems_cuda.h.
//
// The engine owns device memory and one CUDA stream.  oems_cuda_init() uploads every table,
// builds the per-step kernel sequence and captures it into CUDA graphs (1 step and a batch of
// steps); oems_cuda_iterate() replays them.  The timestep counter numTS lives on the device
// and is advanced by the last kernel of each step, so graph replays need no host round trip.
//
// Per-step kernel order (the reference's phase order, FDTD/engine.cpp:267-286 and the
// extension priorities of FDTD/extensions/engine_extension.h:21-29):
//   [Lorentz pre-V] [Mur pre] update_v(+UPML pre/post) [Mur post] [Lorentz apply-V]
//   [Mur apply] [excitation V] [Lorentz pre-I] update_i(+UPML pre/post) [Lorentz apply-I]
//   [excitation I] step_end(probes, FD dumps, ++numTS)
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <unordered_map>
#include <vector>

#include "engine_impl.h"
#include "march.cuh"

#include <cudaTypedefs.h>

using namespace oems;

namespace {

int fail(oems_cuda_engine* e, int code, const std::string& msg)
{
    if (e) e->err = msg;
    return code;
}

int cuda_fail(oems_cuda_engine* e, cudaError_t c, const char* what)
{
    std::string m = std::string(what) + ": " + cudaGetErrorString(c);
    cudaGetLastError();
    return fail(e, c == cudaErrorMemoryAllocation ? OEMS_ERR_NOMEM : OEMS_ERR_CUDA, m);
}

#define CK(call)                                             \
    do {                                                     \
        cudaError_t _c = (call);                             \
        if (_c != cudaSuccess) return cuda_fail(e, _c, #call); \
    } while (0)

template <typename T>
int dalloc(oems_cuda_engine* e, T** p, size_t count, bool zero = true, bool is_state = false)
{
    size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
    void* q = nullptr;
    CK(cudaMalloc(&q, bytes));
    e->allocs.push_back(q);
    if (zero) CK(cudaMemsetAsync(q, 0, bytes, e->stream));
    if (is_state) e->state.push_back({q, bytes});
    *p = static_cast<T*>(q);
    return OEMS_OK;
}

template <typename T>
int dupload(oems_cuda_engine* e, T** p, const T* src, size_t count)
{
    int rc = dalloc(e, p, count, false);
    if (rc) return rc;
    if (count) CK(cudaMemcpyAsync(*p, src, count * sizeof(T), cudaMemcpyHostToDevice, e->stream));
    return OEMS_OK;
}

inline unsigned long long cell_off(const oems_cuda_engine* e, unsigned n, unsigned x, unsigned y, unsigned z)
{
    return (unsigned long long)n * e->S + ((unsigned long long)x * e->N[1] + y) * e->Pz + z;
}

// UPML coefficient classes of one region: the 18 values (vv, vvfo, vvfn, ii, iifo, iifn of the
// three components) of each cell, deduplicated; false when there are more than 65535 classes.
bool compress_upml(const UpmlHost& u, std::vector<unsigned short>& cls, std::vector<float4>& tab)
{
    const size_t n = (size_t)u.nl[0] * u.nl[1] * u.nl[2];
    struct Key18 { uint32_t w[18]; };
    std::vector<Key18> keys;
    cls.assign(n, 0);
    size_t hcap = 1u << 12;
    std::vector<int64_t> htab(hcap, -1);
    auto hash = [](const Key18& k) {
        uint64_t h = 1469598103934665603ULL;
        for (int i = 0; i < 18; ++i) { h ^= k.w[i]; h *= 1099511628211ULL; h ^= h >> 31; }
        return h;
    };
    Key18 k;
    for (size_t c = 0; c < n; ++c) {
        for (int t = 0; t < 6; ++t)
            for (int m = 0; m < 3; ++m) memcpy(&k.w[3 * t + m], &u.tab[t][m * n + c], 4);
        size_t slot = hash(k) & (hcap - 1);
        int64_t found = -1;
        while (htab[slot] >= 0) {
            if (memcmp(&keys[htab[slot]], &k, sizeof(Key18)) == 0) { found = htab[slot]; break; }
            slot = (slot + 1) & (hcap - 1);
        }
        if (found < 0) {
            if (keys.size() >= 65535) return false;
            found = (int64_t)keys.size();
            keys.push_back(k);
            htab[slot] = found;
            if (keys.size() * 2 > hcap) {
                hcap *= 4;
                htab.assign(hcap, -1);
                for (size_t j = 0; j < keys.size(); ++j) {
                    size_t s2 = hash(keys[j]) & (hcap - 1);
                    while (htab[s2] >= 0) s2 = (s2 + 1) & (hcap - 1);
                    htab[s2] = (int64_t)j;
                }
            }
        }
        cls[c] = (unsigned short)found;
    }
    // per class: (f0 f1 f2 fo0)(fo1 fo2 fn0 fn1)(fn2 0 0 0) for the voltage and the current triple
    tab.assign(keys.size() * 6, make_float4(0.f, 0.f, 0.f, 0.f));
    for (size_t j = 0; j < keys.size(); ++j)
        for (int half = 0; half < 2; ++half) {
            float v[12] = {0};
            memcpy(v, &keys[j].w[9 * half], 9 * sizeof(float));
            float4* t = &tab[6 * j + 3 * half];
            t[0] = make_float4(v[0], v[1], v[2], v[3]);
            t[1] = make_float4(v[4], v[5], v[6], v[7]);
            t[2] = make_float4(v[8], v[9], v[10], v[11]);
        }
    return true;
}

int upload_dense(oems_cuda_engine* e, const float* src, float** dst)
{
    const unsigned Nx = e->N[0], Ny = e->N[1], Nz = e->N[2];
    int rc = dalloc(e, dst, 3 * (size_t)e->S, true);
    if (rc) return rc;
    // 2-D copy: rows of Nz floats into rows of Pz floats
    CK(cudaMemcpy2DAsync(*dst, e->Pz * sizeof(float), src, Nz * sizeof(float), Nz * sizeof(float),
                         (size_t)3 * Nx * Ny, cudaMemcpyHostToDevice, e->stream));
    return OEMS_OK;
}

}  // namespace

// =============================================================================================
// C ABI
// =============================================================================================
extern "C" {

int oems_cuda_create(const unsigned int num_lines[3], double dt, int device, oems_cuda_engine** out)
{
    if (!num_lines || !out || !(dt > 0)) return OEMS_ERR_ARG;
    for (int n = 0; n < 3; ++n)
        if (num_lines[n] < 3 || num_lines[n] > 65535) return OEMS_ERR_ARG;
    auto* e = new (std::nothrow) oems_cuda_engine();
    if (!e) return OEMS_ERR_NOMEM;
    *out = e;
    e->device = device;
    memcpy(e->N, num_lines, sizeof(e->N));
    e->Pz = (num_lines[2] + 3u) & ~3u;
    e->S = (unsigned long long)num_lines[0] * num_lines[1] * e->Pz;
    e->dt = dt;
    CK(cudaSetDevice(device));
    CK(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
    int rc;
    if ((rc = dalloc(e, &e->dV, 3 * (size_t)e->S, true, true))) return rc;
    if ((rc = dalloc(e, &e->dI, 3 * (size_t)e->S, true, true))) return rc;
    if ((rc = dalloc(e, &e->d_numTS, 1, true, true))) return rc;
    if ((rc = dalloc(e, &e->d_zero, 1, true))) return rc;
    if ((rc = dalloc(e, &e->d_blocks_done, 1, true))) return rc;
    CK(cudaStreamSynchronize(e->stream));
    return OEMS_OK;
}

void oems_cuda_destroy(oems_cuda_engine* e)
{
    if (!e) return;
    cudaSetDevice(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    td_free(e);
    if (e->graph1) cudaGraphExecDestroy(e->graph1);
    if (e->graphK) cudaGraphExecDestroy(e->graphK);
    if (e->graphK_alt) cudaGraphExecDestroy(e->graphK_alt);
    oems_adjoint_free(e->adj);
    for (void* p : e->allocs) cudaFree(p);
    if (e->stream_r) {
        cudaStreamSynchronize(e->stream_r);
        cudaStreamDestroy(e->stream_r);
    }
    if (e->ev_fork) cudaEventDestroy(e->ev_fork);
    if (e->ev_join) cudaEventDestroy(e->ev_join);
    if (e->stream_se) {
        cudaStreamSynchronize(e->stream_se);
        cudaStreamDestroy(e->stream_se);
    }
    for (cudaEvent_t ev : {e->ev_se_fork, e->ev_se_a, e->ev_se_b})
        if (ev) cudaEventDestroy(ev);
    if (e->stream) cudaStreamDestroy(e->stream);
    if (e->pcache.pin) cudaFreeHost(e->pcache.pin);
    if (e->latest_host) cudaFreeHost(e->latest_host);
    delete e;
}

const char* oems_cuda_last_error(const oems_cuda_engine* e)
{
    return e ? e->err.c_str() : "null engine handle";
}

int oems_cuda_set_operator(oems_cuda_engine* e, const float* vv, const float* vi, const float* ii, const float* iv,
                           unsigned int max_classes)
{
    if (!e || !vv || !vi || !ii || !iv) return OEMS_ERR_ARG;
    if (e->inited || e->op_set) return fail(e, OEMS_ERR_STATE, "operator already set");
    CK(cudaSetDevice(e->device));
    // per-cell coefficient classes, found on the device (compress.cu); too many classes keep
    // the dense arrays
    const unsigned cap = max_classes ? max_classes : (1u << 22);
    int rc = compress_dense_device(e, vv, vi, ii, iv, cap);
    if (rc != 1) return rc;
    if ((rc = upload_dense(e, vv, &e->dvv))) return rc;
    if ((rc = upload_dense(e, vi, &e->dvi))) return rc;
    if ((rc = upload_dense(e, ii, &e->dii))) return rc;
    if ((rc = upload_dense(e, iv, &e->div))) return rc;
    CK(cudaStreamSynchronize(e->stream));
    e->compressed = false;
    e->nclasses = 0;
    e->op_set = true;
    return OEMS_OK;
}

int oems_cuda_set_operator_sse_compressed(oems_cuda_engine* e, unsigned int U, const float* f4_vv, const float* f4_vi,
                                          const float* f4_ii, const float* f4_iv, const unsigned int* op_index)
{
    if (!e || !f4_vv || !f4_vi || !f4_ii || !f4_iv || !op_index || U == 0) return OEMS_ERR_ARG;
    if (e->inited || e->op_set) return fail(e, OEMS_ERR_STATE, "operator already set");
    const unsigned Nx = e->N[0], Ny = e->N[1], Nz = e->N[2];
    const unsigned nv = (Nz + 3) / 4;
    const size_t cells = (size_t)Nx * Ny * Nz;
    // expand the lane-strided 4-lane tables to per-cell N-I-J-K arrays, then compress per cell
    std::vector<float> a[4];
    for (auto& v : a) v.resize(3 * cells);
    const float* src[4] = {f4_vv, f4_vi, f4_ii, f4_iv};
    for (unsigned x = 0; x < Nx; ++x)
        for (unsigned y = 0; y < Ny; ++y)
            for (unsigned z = 0; z < Nz; ++z) {
                const unsigned v = z % nv, l = z / nv;
                const unsigned c = op_index[((size_t)x * Ny + y) * nv + v];
                if (c >= U) return fail(e, OEMS_ERR_ARG, "op_index out of range");
                for (int t = 0; t < 4; ++t)
                    for (int n = 0; n < 3; ++n)
                        a[t][n * cells + ((size_t)x * Ny + y) * Nz + z] = src[t][((size_t)n * U + c) * 4 + l];
            }
    return oems_cuda_set_operator(e, a[0].data(), a[1].data(), a[2].data(), a[3].data(), 0);
}

int oems_cuda_operator_classes(const oems_cuda_engine* e, unsigned int* nc)
{
    if (!e || !nc) return OEMS_ERR_ARG;
    *nc = e->compressed ? e->nclasses : 0;
    return OEMS_OK;
}

int oems_cuda_set_excitation(oems_cuda_engine* e, unsigned int nV, const unsigned int* v_idx, const unsigned short* v_dir,
                             const float* v_amp, const unsigned int* v_delay, unsigned int nI,
                             const unsigned int* i_idx, const unsigned short* i_dir, const float* i_amp,
                             const unsigned int* i_delay, const float* sig_v, const float* sig_i,
                             unsigned int length, unsigned int period)
{
    if (!e) return OEMS_ERR_ARG;
    if (e->inited) return fail(e, OEMS_ERR_STATE, "engine already initialised");
    if ((nV || nI) && (length == 0 || !sig_v || !sig_i)) return fail(e, OEMS_ERR_ARG, "excitation signal missing");
    if ((nV && (!v_idx || !v_dir || !v_amp || !v_delay)) || (nI && (!i_idx || !i_dir || !i_amp || !i_delay)))
        return fail(e, OEMS_ERR_ARG, "excitation arrays missing");
    e->exc_voff.clear(); e->exc_ioff.clear();
    for (unsigned k = 0; k < nV; ++k) {
        const unsigned x = v_idx[k], y = v_idx[nV + k], z = v_idx[2 * nV + k];
        if (x >= e->N[0] || y >= e->N[1] || z >= e->N[2] || v_dir[k] > 2)
            return fail(e, OEMS_ERR_ARG, "voltage excitation index out of range");
        e->exc_voff.push_back(cell_off(e, v_dir[k], x, y, z));
    }
    for (unsigned k = 0; k < nI; ++k) {
        const unsigned x = i_idx[k], y = i_idx[nI + k], z = i_idx[2 * nI + k];
        if (x >= e->N[0] || y >= e->N[1] || z >= e->N[2] || i_dir[k] > 2)
            return fail(e, OEMS_ERR_ARG, "current excitation index out of range");
        e->exc_ioff.push_back(cell_off(e, i_dir[k], x, y, z));
    }
    e->exc_vamp.assign(v_amp, v_amp + nV);
    e->exc_iamp.assign(i_amp, i_amp + nI);
    e->exc_vdelay.assign(v_delay, v_delay + nV);
    e->exc_idelay.assign(i_delay, i_delay + nI);
    e->sig_v.assign(sig_v, sig_v + length);
    e->sig_i.assign(sig_i, sig_i + length);
    e->sig_len = length;
    e->period = period;
    e->has_exc = true;
    return OEMS_OK;
}

static int tfsf_terms(oems_cuda_engine* e, unsigned n, const unsigned* idx, const unsigned short* dir,
                      const unsigned* delay, const float* delta, const float* amp, unsigned max_delay, TfsfHost& t)
{
    if (n && (!idx || !dir || !delay || !delta || !amp)) return fail(e, OEMS_ERR_ARG, "TFSF arrays missing");
    t = TfsfHost{};
    for (unsigned k = 0; k < n; ++k) {
        const unsigned x = idx[k], y = idx[n + k], z = idx[2 * (size_t)n + k];
        if (x >= e->N[0] || y >= e->N[1] || z >= e->N[2] || dir[k] > 2)
            return fail(e, OEMS_ERR_ARG, "TFSF index out of range");
        // the reference's delay lookup table has max_delay + 1 entries and is read at delay + 1
        if (delay[k] >= max_delay) return fail(e, OEMS_ERR_ARG, "TFSF delay exceeds max_delay");
        t.off.push_back(cell_off(e, dir[k], x, y, z));
    }
    t.delay.assign(delay, delay + n);
    t.delta.assign(delta, delta + n);
    t.amp.assign(amp, amp + n);
    return OEMS_OK;
}

int oems_cuda_set_tfsf(oems_cuda_engine* e, unsigned int volt_count, const unsigned int* volt_index,
                       const unsigned short* volt_dir, const unsigned int* volt_delay, const float* volt_delta,
                       const float* volt_amp, unsigned int curr_count, const unsigned int* curr_index,
                       const unsigned short* curr_dir, const unsigned int* curr_delay, const float* curr_delta,
                       const float* curr_amp, const float* sig_volt, const float* sig_curr, unsigned int length,
                       unsigned int period, unsigned int max_delay)
{
    if (!e) return OEMS_ERR_ARG;
    if (e->inited) return fail(e, OEMS_ERR_STATE, "engine already initialised");
    if (length == 0 || !sig_volt || !sig_curr) return fail(e, OEMS_ERR_ARG, "TFSF signal missing");
    if (period > length) return fail(e, OEMS_ERR_ARG, "TFSF signal period longer than the signal");
    int rc;
    if ((rc = tfsf_terms(e, volt_count, volt_index, volt_dir, volt_delay, volt_delta, volt_amp, max_delay, e->tfsf_v)))
        return rc;
    if ((rc = tfsf_terms(e, curr_count, curr_index, curr_dir, curr_delay, curr_delta, curr_amp, max_delay, e->tfsf_i)))
        return rc;
    e->tfsf_sig_v.assign(sig_volt, sig_volt + length);
    e->tfsf_sig_i.assign(sig_curr, sig_curr + length);
    e->tfsf_len = length;
    e->tfsf_period = period;
    e->has_tfsf = volt_count || curr_count;
    return OEMS_OK;
}

int oems_cuda_set_cylinder(oems_cuda_engine* e, int closed_alpha, int r0_included, const float* vv_r0,
                           const float* vi_r0)
{
    if (!e) return OEMS_ERR_ARG;
    if (e->inited) return fail(e, OEMS_ERR_STATE, "engine already initialised");
    if (r0_included && (!closed_alpha || !vv_r0 || !vi_r0))
        return fail(e, OEMS_ERR_ARG, "rho = 0 needs a closed alpha mesh and its axis coefficients");
    if (e->N[1] < 3) return fail(e, OEMS_ERR_ARG, "a closed alpha mesh needs at least 3 alpha lines");
    e->cyl_closed = closed_alpha != 0;
    e->cyl_r0 = e->cyl_closed && r0_included != 0;
    e->cyl_vv_r0.assign(e->cyl_r0 ? vv_r0 : nullptr, e->cyl_r0 ? vv_r0 + e->N[2] : nullptr);
    e->cyl_vi_r0.assign(e->cyl_r0 ? vi_r0 : nullptr, e->cyl_r0 ? vi_r0 + e->N[2] : nullptr);
    return OEMS_OK;
}

int oems_cuda_set_lumped_rlc(oems_cuda_engine* e, unsigned int count, const unsigned int* pos, const int* dir,
                             const float* ilv, const float* i2v, const float* vv2, const float* vj1, const float* vj2,
                             const float* vvd, const float* ib0, const float* b1, const float* b2)
{
    if (!e) return OEMS_ERR_ARG;
    if (e->inited) return fail(e, OEMS_ERR_STATE, "engine already initialised");
    if (count && (!pos || !dir || !ilv || !i2v || !vv2 || !vj1 || !vj2 || !vvd || !ib0 || !b1 || !b2))
        return fail(e, OEMS_ERR_ARG, "lumped RLC arrays missing");
    RlcHost r;
    for (unsigned k = 0; k < count; ++k) {
        const unsigned x = pos[k], y = pos[count + k], z = pos[2 * (size_t)count + k];
        if (x >= e->N[0] || y >= e->N[1] || z >= e->N[2] || dir[k] < 0 || dir[k] > 2)
            return fail(e, OEMS_ERR_ARG, "lumped RLC position out of range");
        r.off.push_back(cell_off(e, (unsigned)dir[k], x, y, z));
    }
    std::vector<unsigned long long> sorted(r.off);
    std::sort(sorted.begin(), sorted.end());
    if (std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end())
        return fail(e, OEMS_ERR_ARG, "two lumped RLC elements on one edge");
    const float* src[9] = {ilv, i2v, vv2, vj1, vj2, vvd, ib0, b1, b2};
    for (int q = 0; q < 9; ++q) r.c.insert(r.c.end(), src[q], src[q] + count);
    e->rlc_host = std::move(r);
    return OEMS_OK;
}

int oems_cuda_add_upml(oems_cuda_engine* e, const unsigned int start[3], const unsigned int nl[3], const float* vv,
                       const float* vvfo, const float* vvfn, const float* ii, const float* iifo, const float* iifn)
{
    if (!e || !start || !nl || !vv || !vvfo || !vvfn || !ii || !iifo || !iifn) return OEMS_ERR_ARG;
    if (e->inited) return fail(e, OEMS_ERR_STATE, "engine already initialised");
    if (e->upml.size() >= OEMS_MAX_UPML) return fail(e, OEMS_ERR_UNSUPPORTED, "more than 6 UPML regions");
    for (int n = 0; n < 3; ++n)
        if (nl[n] == 0 || start[n] + nl[n] > e->N[n]) return fail(e, OEMS_ERR_ARG, "UPML region outside the mesh");
    for (const auto& u : e->upml) {
        bool overlap = true;
        for (int n = 0; n < 3; ++n)
            overlap &= start[n] < u.start[n] + u.nl[n] && u.start[n] < start[n] + nl[n];
        if (overlap) return fail(e, OEMS_ERR_ARG, "UPML regions overlap");
    }
    UpmlHost u;
    memcpy(u.start, start, 12);
    memcpy(u.nl, nl, 12);
    const size_t m = 3 * (size_t)nl[0] * nl[1] * nl[2];
    const float* src[6] = {vv, vvfo, vvfn, ii, iifo, iifn};
    for (int t = 0; t < 6; ++t) u.tab[t].assign(src[t], src[t] + m);
    e->upml.push_back(std::move(u));
    return OEMS_OK;
}

int oems_cuda_add_mur(oems_cuda_engine* e, int ny, unsigned int line, unsigned int shift, unsigned int start_ts,
                      const float* cP, const float* cPP)
{
    if (!e || !cP || !cPP || ny < 0 || ny > 2) return OEMS_ERR_ARG;
    if (e->inited) return fail(e, OEMS_ERR_STATE, "engine already initialised");
    if (e->mur.size() >= OEMS_MAX_MUR) return fail(e, OEMS_ERR_UNSUPPORTED, "more than 6 Mur walls");
    if (line >= e->N[ny] || shift >= e->N[ny]) return fail(e, OEMS_ERR_ARG, "Mur line outside the mesh");
    MurHost m;
    m.ny = ny; m.line = line; m.shift = shift; m.start_ts = start_ts;
    const size_t n = (size_t)e->N[(ny + 1) % 3] * e->N[(ny + 2) % 3];
    m.cP.assign(cP, cP + n);
    m.cPP.assign(cPP, cPP + n);
    e->mur.push_back(std::move(m));
    return OEMS_OK;
}

int oems_cuda_add_lorentz_order(oems_cuda_engine* e, unsigned int count, const unsigned int* pos, int von, int con,
                                int vlon, int clon, const float* vint, const float* vext, const float* vlor,
                                const float* iint, const float* iext, const float* ilor)
{
    if (!e || (count && !pos)) return OEMS_ERR_ARG;
    if (e->inited) return fail(e, OEMS_ERR_STATE, "engine already initialised");
    if ((von && (!vint || !vext)) || (con && (!iint || !iext)) || (von && vlon && !vlor) || (con && clon && !ilor))
        return fail(e, OEMS_ERR_ARG, "dispersive coefficient table missing");
    LorHost l;
    l.count = count;
    l.pos.assign(pos, pos + 3 * (size_t)count);
    for (unsigned i = 0; i < count; ++i)
        for (int a = 0; a < 3; ++a)
            if (pos[a * count + i] >= e->N[a]) return fail(e, OEMS_ERR_ARG, "dispersive position outside the mesh");
    l.von = von; l.con = con; l.vlon = vlon && von; l.clon = clon && con;
    const size_t m = 3 * (size_t)count;
    if (von) { l.vint.assign(vint, vint + m); l.vext.assign(vext, vext + m); }
    if (l.vlon) l.vlor.assign(vlor, vlor + m);
    if (con) { l.iint.assign(iint, iint + m); l.iext.assign(iext, iext + m); }
    if (l.clon) l.ilor.assign(ilor, ilor + m);
    e->lor.push_back(std::move(l));
    return OEMS_OK;
}

static int add_probe(oems_cuda_engine* e, int type, const unsigned* start, const unsigned* stop, int nd,
                     const int* si, const int* ei, double weight, unsigned interval, unsigned start_ts,
                     unsigned stop_ts, int* id)
{
    if (!e || !start || !stop || !id) return OEMS_ERR_ARG;
    if (e->inited) return fail(e, OEMS_ERR_STATE, "engine already initialised");
    for (int a = 0; a < 3; ++a)
        if (start[a] >= e->N[a] || stop[a] >= e->N[a]) return fail(e, OEMS_ERR_ARG, "probe outside the mesh");
    if (type == 0 && ((start[0] != stop[0]) + (start[1] != stop[1]) + (start[2] != stop[2])) != 1)
        return fail(e, OEMS_ERR_ARG, "only a 1D/line voltage integration is allowed");
    if (type == 1 && (nd < 0 || nd > 2)) return fail(e, OEMS_ERR_ARG, "invalid current probe normal direction");
    ProbeHost p;
    p.type = type;
    memcpy(p.start, start, 12);
    memcpy(p.stop, stop, 12);
    p.nd = nd;
    for (int a = 0; a < 3; ++a) { p.si[a] = si ? si[a] : 1; p.ei[a] = ei ? ei[a] : 1; }
    p.weight = weight;
    p.interval = interval ? interval : 1;
    p.start_ts = start_ts;
    p.stop_ts = stop_ts;
    *id = (int)e->probes.size();
    e->probes.push_back(std::move(p));
    return OEMS_OK;
}

int oems_cuda_add_field_probe(oems_cuda_engine* e, int field, const unsigned int pos[3], const double el[3],
                              double weight, unsigned int interval, unsigned int start_ts, unsigned int stop_ts,
                              int* id)
{
    if (!e || !el || (field != 0 && field != 1)) return OEMS_ERR_ARG;
    const int rc = add_probe(e, 2 + field, pos, pos, -1, nullptr, nullptr, weight, interval, start_ts, stop_ts, id);
    if (rc == OEMS_OK) memcpy(e->probes[*id].el, el, sizeof(double) * 3);
    return rc;
}

int oems_cuda_add_voltage_probe(oems_cuda_engine* e, const unsigned int start[3], const unsigned int stop[3],
                                double weight, unsigned int interval, unsigned int start_ts, unsigned int stop_ts,
                                int* id)
{
    return add_probe(e, 0, start, stop, -1, nullptr, nullptr, weight, interval, start_ts, stop_ts, id);
}

int oems_cuda_add_current_probe(oems_cuda_engine* e, const unsigned int start[3], const unsigned int stop[3],
                                int norm_dir, const int start_inside[3], const int stop_inside[3], double weight,
                                unsigned int interval, unsigned int start_ts, unsigned int stop_ts, int* id)
{
    return add_probe(e, 1, start, stop, norm_dir, start_inside, stop_inside, weight, interval, start_ts, stop_ts, id);
}

int oems_cuda_set_probe_dft(oems_cuda_engine* e, int id, unsigned int fd_interval, unsigned int nf,
                            const double* freqs)
{
    if (!e || id < 0 || id >= (int)e->probes.size() || (nf && !freqs)) return OEMS_ERR_ARG;
    if (e->inited) return fail(e, OEMS_ERR_STATE, "engine already initialised");
    e->probes[id].fd_interval = fd_interval;
    e->probes[id].freqs.assign(freqs, freqs + nf);
    return OEMS_OK;
}

int oems_cuda_set_dump_rho(oems_cuda_engine* e, int id, const double* rho)
{
    if (!e || !rho || id < 0 || id >= (int)e->dumps.size()) return OEMS_ERR_ARG;
    if (e->inited) return fail(e, OEMS_ERR_STATE, "engine already initialised");
    if (e->dumps[id].interp != 0) return fail(e, OEMS_ERR_ARG, "cylindrical dumps without interpolation only");
    e->dumps[id].rho.assign(rho, rho + e->N[0]);
    return OEMS_OK;
}

int oems_cuda_add_fd_dump(oems_cuda_engine* e, int field, int interp, const unsigned int start[3],
                          const unsigned int stop[3], unsigned int fd_interval, unsigned int nf, const double* freqs,
                          const double* el, const double* del, int* id)
{
    if (!e || !start || !stop || !el || !del || !id || (field != 0 && field != 1) || (nf && !freqs) ||
        interp < 0 || interp > 2)
        return OEMS_ERR_ARG;
    if (e->inited) return fail(e, OEMS_ERR_STATE, "engine already initialised");
    DumpHost d;
    d.field = field;
    d.interp = interp;
    for (int a = 0; a < 3; ++a) {
        if (start[a] > stop[a] || stop[a] >= e->N[a]) return fail(e, OEMS_ERR_ARG, "dump box outside the mesh");
        d.start[a] = start[a];
        d.stop[a] = stop[a];
    }
    d.fd_interval = fd_interval;
    d.freqs.assign(freqs, freqs + nf);
    const size_t tot = (size_t)e->N[0] + e->N[1] + e->N[2];
    d.el.assign(field == 0 ? el : del, (field == 0 ? el : del) + tot);
    *id = (int)e->dumps.size();
    e->dumps.push_back(std::move(d));
    return OEMS_OK;
}

int oems_cuda_add_td_dump(oems_cuda_engine* e, int field, int interp, const unsigned int start[3],
                          const unsigned int stop[3], unsigned int interval, unsigned int start_ts,
                          unsigned int stop_ts, const double* el, const double* del, const double* coords,
                          const char* file_prefix, int* id)
{
    if (!e || !start || !stop || !el || !del || !coords || !file_prefix || !id || (field != 0 && field != 1) ||
        interp < 0 || interp > 2 || interval == 0 || !file_prefix[0])
        return OEMS_ERR_ARG;
    if (e->inited) return fail(e, OEMS_ERR_STATE, "engine already initialised");
    DumpHost d;
    d.field = field;
    d.interp = interp;
    size_t nc = 0;
    for (int a = 0; a < 3; ++a) {
        if (start[a] > stop[a] || stop[a] >= e->N[a]) return fail(e, OEMS_ERR_ARG, "dump box outside the mesh");
        d.start[a] = start[a];
        d.stop[a] = stop[a];
        nc += stop[a] - start[a] + 1;
    }
    d.fd_interval = 0;
    d.td = true;
    d.td_interval = interval;
    d.td_start = start_ts;
    d.td_stop = stop_ts;
    d.prefix = file_prefix;
    d.coords.assign(coords, coords + nc);
    const size_t tot = (size_t)e->N[0] + e->N[1] + e->N[2];
    d.el.assign(field == 0 ? el : del, (field == 0 ? el : del) + tot);
    *id = (int)e->dumps.size();
    e->dumps.push_back(std::move(d));
    e->has_td = true;
    return OEMS_OK;
}

int oems_cuda_flush_dumps(oems_cuda_engine* e)
{
    if (!e) return OEMS_ERR_ARG;
    if (!e->inited || !e->td) return OEMS_OK;
    CK(cudaSetDevice(e->device));
    int rc = td_flush(e);
    if (rc) return rc;
    return td_wait(e);
}

// ---------------------------------------------------------------------------------------------
// init: upload, build device structs, capture graphs

}  // extern "C" (enqueue_step below is internal C++)

void make_split(const oems_cuda_engine* e, const unsigned R[3], SplitDev& sp)
{
    sp = SplitDev{};
    const GridDev& g = e->grid;
    sp.nreg = (unsigned)g.nupml;
    // region extents clipped to R
    unsigned cs[OEMS_MAX_UPML][3], ce[OEMS_MAX_UPML][3];
    unsigned long long in_r = 0;
    for (int r = 0; r < g.nupml; ++r) {
        unsigned long long v = 1;
        for (int a = 0; a < 3; ++a) {
            cs[r][a] = std::min(g.upml[r].start[a], R[a]);
            ce[r][a] = std::min(g.upml[r].start[a] + g.upml[r].nl[a], R[a]);
            v *= ce[r][a] - cs[r][a];
        }
        in_r += v;
    }
    const unsigned long long total = (unsigned long long)R[0] * R[1] * R[2];
    const unsigned long long rest = total - in_r;
    // bounding box of the cells outside every region: a plane is fully covered when the regions'
    // (disjoint) cross-sections add up to its area
    unsigned lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    bool any = rest > 0;
    for (int a = 0; a < 3 && any; ++a) {
        const int b = (a + 1) % 3, c = (a + 2) % 3;
        const unsigned long long area = (unsigned long long)R[b] * R[c];
        auto covered = [&](unsigned k) {
            unsigned long long s2 = 0;
            for (int r = 0; r < g.nupml; ++r)
                if (k >= cs[r][a] && k < ce[r][a]) s2 += (unsigned long long)(ce[r][b] - cs[r][b]) * (ce[r][c] - cs[r][c]);
            return s2 >= area;
        };
        unsigned k0 = 0;
        while (k0 < R[a] && covered(k0)) ++k0;
        unsigned k1 = R[a];
        while (k1 > k0 && covered(k1 - 1)) --k1;
        lo[a] = k0;
        hi[a] = k1;
    }
    const unsigned long long box = any ? (unsigned long long)(hi[0] - lo[0]) * (hi[1] - lo[1]) * (hi[2] - lo[2]) : 0;
    if (any && box == rest) {
        sp.full = 0;
        for (int a = 0; a < 3; ++a) { sp.lo[a] = lo[a]; sp.n[a] = hi[a] - lo[a]; }
    } else {
        sp.full = 1;
        for (int a = 0; a < 3; ++a) { sp.lo[a] = 0; sp.n[a] = R[a]; }
    }
    sp.main_cells = rest ? sp.n[0] * sp.n[1] * sp.n[2] : 0;
    sp.main_blocks = (sp.main_cells + 255) / 256;
    // four z cells per thread in the main box of the compressed forward kernels: the box's z range
    // on multiples of four, 32-bit offsets (the adjoint kernels keep one cell per thread)
    sp.v4 = (!sp.full && sp.main_cells && e->compressed && e->vec4 && 3ull * e->S < (1ull << 32)) ? 1 : 0;
    sp.z4 = sp.lo[2] & ~3u;
    sp.n4 = sp.v4 ? (((sp.lo[2] + sp.n[2] + 3u) & ~3u) - sp.z4) / 4u : 0u;
    sp.main_cells4 = sp.v4 ? sp.n[0] * sp.n[1] * sp.n4 : 0;
    sp.main_blocks4 = (sp.main_cells4 + 255) / 256;
    sp.first_block[0] = 0;
    for (int r = 0; r < g.nupml; ++r) sp.first_block[r + 1] = sp.first_block[r] + (g.upml[r].n + 255) / 256;
    // the regions four z cells per thread (k_update_reg4): each region on z rows of whole groups
    // of four, its coefficients in classes; OEMS_CUDA_REG4=0 keeps the one-cell region blocks
    const char* r4 = getenv("OEMS_CUDA_REG4");
    sp.reg4 = (sp.v4 && g.nupml > 0 && !(r4 && r4[0] == '0')) ? 1 : 0;
    sp.first4[0] = 0;
    sp.first4h[0] = 0;
    for (int r = 0; r < g.nupml; ++r) {
        const UpmlDev& u = g.upml[r];
        if (!u.cls) sp.reg4 = 0;
        const unsigned zs = u.start[2], ze = zs + u.nl[2];
        const unsigned groups = u.nl[0] * u.nl[1] * ((((ze + 3u) & ~3u) - (zs & ~3u)) / 4u);
        sp.first4[r + 1] = sp.first4[r] + (groups + 255) / 256;
        sp.first4h[r + 1] = sp.first4h[r] + (groups + 127) / 128;
    }
}

template <bool C, bool U, int M, typename IX = unsigned long long>
static void launch_v(const dim3& grid, cudaStream_t s, const GridDev& g, const MurDev& m, const unsigned* ts)
{
    k_update_v<C, U, M, IX><<<grid, 256, 0, s>>>(g, m, ts);
}

void launch_update(oems_cuda_engine* e, bool curr, cudaStream_t s, const char** name, const FacOut* fac)
{
    const GridDev& g = e->grid;
    const MurDev& m = e->murdev;
    // the lane-parallel Mur form has every wall active from step 0, so its hooks' activity test
    // reads a constant 0 instead of the step counter (which a concurrent step-end part may be
    // advancing)
    const unsigned* ts = m.lanes ? e->d_zero : e->d_numTS;
    // name != nullptr: report the kernel this configuration launches, launch nothing
    auto go = [&](const char* n) {
        if (name) *name = n;
        return name == nullptr;
    };
    // the voltage update carries the Mur pre/post hooks when there are walls
    const bool mur = !curr && !e->mur.empty() && !e->mur_separate;
    if (e->use_split) {
        const SplitDev& sp = curr ? e->splitI : e->splitV;
        if (sp.v4 && !mur) {
            // the region blocks, then the main box four cells per thread (the two write disjoint
            // cells; as separate launches each gets its own register budget)
            if (!go(sp.reg4 ? "k_update_reg4+k_update_box4" : "k_update_split+k_update_box4")) return;
            // the region kernel on the branch stream when there is one (joined below)
            cudaStream_t rs = e->stream_r ? e->stream_r : s;
            if (e->stream_r) {
                cudaEventRecord(e->ev_fork, s);
                cudaStreamWaitEvent(rs, e->ev_fork, 0);
            }
            if (sp.reg4) {
                const unsigned tb = e->reg_block, nb = tb == 128u ? sp.first4h[sp.nreg] : sp.first4[sp.nreg];
                if (curr) k_update_reg4<true><<<nb, tb, 0, rs>>>(g, sp);
                else k_update_reg4<false><<<nb, tb, 0, rs>>>(g, sp);
            } else if (const unsigned rb = sp.first_block[sp.nreg]) {
                if (curr) k_update_split<true, true><<<rb, 256, 0, rs>>>(g, sp, m, ts);
                else k_update_split<true, false><<<rb, 256, 0, rs>>>(g, sp, m, ts);
            }
            if (sp.main_blocks4) {
                const unsigned tb = e->box_block, nb = (sp.main_cells4 + tb - 1) / tb;
                if (curr) k_update_box4<true><<<nb, tb, 0, s>>>(g, sp);
                else if (fac) k_update_box4<false, true><<<nb, tb, 0, s>>>(g, sp, *fac);
                else k_update_box4<false><<<nb, tb, 0, s>>>(g, sp);
            }
            if (e->stream_r) {
                cudaEventRecord(e->ev_join, rs);
                cudaStreamWaitEvent(s, e->ev_join, 0);
            }
            return;
        }
        const unsigned blocks = sp.main_blocks + sp.first_block[sp.nreg];
        if (!go("k_update_split")) return;
        if (!blocks) return;
        if (e->compressed) {
            if (curr) k_update_split<true, true><<<blocks, 256, 0, s>>>(g, sp, m, ts);
            else if (mur) k_update_split<true, false, true><<<blocks, 256, 0, s>>>(g, sp, m, ts);
            else k_update_split<true, false><<<blocks, 256, 0, s>>>(g, sp, m, ts);
        } else {
            if (curr) k_update_split<false, true><<<blocks, 256, 0, s>>>(g, sp, m, ts);
            else if (mur) k_update_split<false, false, true><<<blocks, 256, 0, s>>>(g, sp, m, ts);
            else k_update_split<false, false><<<blocks, 256, 0, s>>>(g, sp, m, ts);
        }
        return;
    }
    const unsigned plane = e->N[1] * e->Pz;
    const bool up = !e->upml.empty();
    // 32-bit cell offsets when every component offset fits
    const bool o32 = 3ull * e->S < (1ull << 32);
    if (!curr) {
        const dim3 gv((plane + 255) / 256, e->N[0]);
        const int mode = !mur ? 0 : (m.lanes ? 2 : 1);
        if (up) {
            if (!go("k_update_v")) return;
            if (e->compressed) { if (mode) launch_v<true, true, 1>(gv, s, g, m, ts); else launch_v<true, true, 0>(gv, s, g, m, ts); }
            else { if (mode) launch_v<false, true, 1>(gv, s, g, m, ts); else launch_v<false, true, 0>(gv, s, g, m, ts); }
        } else if (e->compressed) {
            if (o32 && e->vec4 && (mode == 0 || (mode == 2 && e->mur_v4))) {
                const unsigned vb = e->v4_block;
                const dim3 gv4((plane / 4 + vb - 1) / vb, e->N[0]);
                if (mode == 2 && m.park) {
                    // every direct-column group streams; the z walls' hooks run around this launch
                    if (go("k_update_v4w<park>")) k_update_v4w<unsigned, true><<<gv4, vb, 0, s>>>(g, m, ts, gv4.x);
                } else if (mode == 2) {
                    // the interior blocks, then one thread per direct column's z-wall group
                    const unsigned walls = m.nz > 0 ? (e->N[1] * (unsigned)m.nz + vb - 1) / vb : 0;
                    const dim3 gw(gv4.x + walls, e->N[0]);
                    if (go("k_update_v4w")) k_update_v4w<unsigned><<<gw, vb, 0, s>>>(g, m, ts, gv4.x);
                }
                else if (go("k_update_v4")) k_update_v4<unsigned><<<gv4, vb, 0, s>>>(g);
            } else if (o32) {
                if (!go("k_update_v")) return;
                if (mode == 2) launch_v<true, false, 2, unsigned>(gv, s, g, m, ts);
                else if (mode == 1) launch_v<true, false, 1, unsigned>(gv, s, g, m, ts);
                else launch_v<true, false, 0, unsigned>(gv, s, g, m, ts);
            } else {
                if (!go("k_update_v")) return;
                if (mode == 2) launch_v<true, false, 2>(gv, s, g, m, ts);
                else if (mode == 1) launch_v<true, false, 1>(gv, s, g, m, ts);
                else launch_v<true, false, 0>(gv, s, g, m, ts);
            }
        } else {
            if (!go("k_update_v")) return;
            if (mode == 2) launch_v<false, false, 2>(gv, s, g, m, ts);
            else if (mode == 1) launch_v<false, false, 1>(gv, s, g, m, ts);
            else launch_v<false, false, 0>(gv, s, g, m, ts);
        }
    } else {
        const dim3 gi((plane + 255) / 256, e->N[0] - 1);
        if (up) {
            if (!go("k_update_i")) return;
            if (e->compressed) k_update_i<true, true><<<gi, 256, 0, s>>>(g); else k_update_i<false, true><<<gi, 256, 0, s>>>(g);
        } else if (e->compressed) {
            if (o32 && e->vec4) {
                const unsigned tb = e->i4_block;
                const dim3 gi4((plane / 4 + tb - 1) / tb, e->N[0] - 1);
                if (go("k_update_i4")) k_update_i4<unsigned><<<gi4, tb, 0, s>>>(g);
            } else {
                if (!go("k_update_i")) return;
                if (o32) k_update_i<true, false, unsigned><<<gi, 256, 0, s>>>(g);
                else k_update_i<true, false><<<gi, 256, 0, s>>>(g);
            }
        } else if (go("k_update_i")) k_update_i<false, false><<<gi, 256, 0, s>>>(g);
    }
}

int enqueue_fused_step(oems_cuda_engine* e, int parity, unsigned* nlaunch)
{
    const FusedDev& f = e->fused[parity];
    if (e->march_minb == 2)
        k_step_march<2><<<e->march_grid, e->march_threads, e->march_smem, e->stream>>>(e->march[parity],
                                                                                    e->march_map[parity]);
    else
        k_step_march<1><<<e->march_grid, e->march_threads, e->march_smem, e->stream>>>(e->march[parity],
                                                                                    e->march_map[parity]);
    // processing on the fields this step wrote
    GridDev g = e->grid;
    g.V = f.Vo;
    g.I = f.Io;
    k_step_end<<<e->stepend_blocks, 256, 0, e->stream>>>(g, e->stepend);
    if (nlaunch) *nlaunch = 2;
    cudaError_t c = cudaGetLastError();
    if (c != cudaSuccess) return cuda_fail(e, c, "one-kernel step launch");
    return OEMS_OK;
}

int enqueue_step(oems_cuda_engine* e, unsigned* nlaunch, StepProfiler* prof, unsigned seq)
{
    // seq bit 0: first step of the enqueued sequence, bit 1: last.  Inside a sequence the
    // dispersive apply of one step and the pre of the next run as one k_lorentz_carry launch at
    // the end of the half-step; a sequence starts with the plain pre and ends with the plain
    // apply, so between sequences the ADE state is the reference's.
    const bool carry_v = e->lor_carry_v && !(seq & 2), pre_v = !e->lor_carry_v || (seq & 1);
    const bool carry_i = e->lor_carry_i && !(seq & 2), pre_i = !e->lor_carry_i || (seq & 1);
    const GridDev& g = e->grid;
    const dim3 blk(256);
    unsigned L = 0;
    cudaStream_t s = e->stream;
    // optional per-launch events (profiling path only, never inside a captured graph)
    auto pre = [&](int k) {
        if (prof && prof->n < 64) { prof->cls[prof->n] = k; cudaEventRecord(prof->ev[2 * prof->n], s); }
    };
    auto post = [&]() {
        if (prof && prof->n < 64) { cudaEventRecord(prof->ev[2 * prof->n + 1], s); ++prof->n; }
    };
    // ---- voltages
    if (pre_v)
        for (const auto& l : e->lorV) { pre(OEMS_KC_LORENTZ); k_lorentz_pre<<<(l.count + 255) / 256, blk, 0, s>>>(e->dV, e->S, l); post(); ++L; }
    unsigned mur_pts = 0;
    for (const auto& m : e->mur) mur_pts = std::max<unsigned>(mur_pts, (unsigned)m.cP.size());
    const dim3 mur_grid((mur_pts + 255) / 256, (unsigned)e->mur.size());
    // the Mur pre/post hooks run inside the voltage update unless mur_separate
    const bool mur_sep = !e->mur.empty() && e->mur_separate;
    if (mur_sep) { pre(OEMS_KC_MUR); k_mur<<<mur_grid, blk, 0, s>>>(g, e->murdev, 0, e->d_numTS); post(); ++L; }
    // park mode: the direct columns' z-wall hooks around the voltage update (one thread per wall
    // and column)
    const bool park = e->murdev.park != 0;
    const unsigned park_blocks = park ? ((unsigned)e->murdev.nz * g.Nx * g.Ny + 255) / 256 : 0;
    if (park) { pre(OEMS_KC_MUR); k_mur_zsave<<<park_blocks, blk, 0, s>>>(g, e->murdev); post(); ++L; }
    pre(OEMS_KC_UPDATE_V);
    launch_update(e, false, s);
    post();
    ++L;
    // the split step end (inside sequences; a single step keeps the one launch): the previous
    // step's current-side part ran beside this voltage update; it bumps numTS, which the hooks
    // below read
    const bool se_split = e->se_split && !prof && seq != 3;
    if (se_split && e->se_pending) {
        cudaStreamWaitEvent(s, e->ev_se_b, 0);
        e->se_pending = false;
    }
    if (park) { pre(OEMS_KC_MUR); k_mur_zpost<<<park_blocks, blk, 0, s>>>(g, e->murdev); post(); ++L; }
    const unsigned cyl_v = g.Nx * g.Nz, cyl_i = (g.Nx - 1) * (g.Nz - 1);
    if (e->cyl.closed) {   // post-voltage hook, priority 1e5: before TFSF and Mur
        pre(OEMS_KC_MUR);
        k_cyl_post_v<<<(cyl_v + 255) / 256, blk, 0, s>>>(g, e->cyl);
        post(); ++L;
    }
    if (e->tfsfV.ntarget) {
        pre(OEMS_KC_EXCITE);
        k_tfsf<<<(e->tfsfV.ntarget + 255) / 256, blk, 0, s>>>(e->dV, e->tfsfV, e->d_numTS);
        post(); ++L;
    }
    if (mur_sep) { pre(OEMS_KC_MUR); k_mur<<<mur_grid, blk, 0, s>>>(g, e->murdev, 1, e->d_numTS); post(); ++L; }
    // apply hooks in priority order: lumped RLC, dispersive, Mur, excitation
    if (e->rlc.count) {
        pre(OEMS_KC_LORENTZ);
        k_lumped_rlc<<<(e->rlc.count + 127) / 128, 128, 0, s>>>(e->dV, e->rlc, e->d_numTS);
        post(); ++L;
    }
    const unsigned mur_blocks = e->mur.empty() ? 0u : e->murdev.afirst[e->murdev.nwall];
    if (e->vtail) {
        // Mur apply, dispersive carry (or the apply at a sequence's end) and excitation in one launch
        const LorDev& l = e->lorV[0];
        const unsigned lor0 = mur_blocks, exc0 = lor0 + (l.count + 255) / 256;
        const unsigned blocks = exc0 + (e->excV.count + 255) / 256;
        pre(OEMS_KC_LORENTZ);
        if (carry_v) k_vtail<true><<<blocks, blk, 0, s>>>(g, e->murdev, l, e->excV, e->d_numTS, lor0, exc0);
        else k_vtail<false><<<blocks, blk, 0, s>>>(g, e->murdev, l, e->excV, e->d_numTS, lor0, exc0);
        post(); ++L;
    } else {
        if (!carry_v)
            for (const auto& l : e->lorV) { pre(OEMS_KC_LORENTZ); k_lorentz_apply<<<(l.count + 255) / 256, blk, 0, s>>>(e->dV, e->S, l); post(); ++L; }
        if (mur_blocks) { pre(OEMS_KC_MUR); k_mur_apply<<<mur_blocks, blk, 0, s>>>(g, e->murdev, e->d_numTS); post(); ++L; }
        if (e->excV.count) { pre(OEMS_KC_EXCITE); k_excitation<<<(e->excV.count + 127) / 128, 128, 0, s>>>(e->dV, e->excV, e->d_numTS); post(); ++L; }
        if (carry_v)
            for (const auto& l : e->lorV) { pre(OEMS_KC_LORENTZ); k_lorentz_carry<<<(l.count + 255) / 256, blk, 0, s>>>(e->dV, e->S, l); post(); ++L; }
    }
    // ---- currents
    if (se_split) {
        // the voltage-side probes and dumps beside the current update (which does not write V)
        cudaEventRecord(e->ev_se_fork, s);
        cudaStreamWaitEvent(e->stream_se, e->ev_se_fork, 0);
        k_step_end<<<e->stepend_blocks, blk, 0, e->stream_se>>>(g, e->stepend, 0);
        cudaEventRecord(e->ev_se_a, e->stream_se);
        ++L;
    }
    if (pre_i)
        for (const auto& l : e->lorI) { pre(OEMS_KC_LORENTZ); k_lorentz_pre<<<(l.count + 255) / 256, blk, 0, s>>>(e->dI, e->S, l); post(); ++L; }
    pre(OEMS_KC_UPDATE_I);
    launch_update(e, true, s);
    post();
    ++L;
    if (e->cyl.closed) {
        pre(OEMS_KC_MUR);
        k_cyl_post_i<<<(cyl_i + 255) / 256, blk, 0, s>>>(g);
        post(); ++L;
    }
    if (e->tfsfI.ntarget) {
        pre(OEMS_KC_EXCITE);
        k_tfsf<<<(e->tfsfI.ntarget + 255) / 256, blk, 0, s>>>(e->dI, e->tfsfI, e->d_numTS);
        post(); ++L;
    }
    if (!carry_i)
        for (const auto& l : e->lorI) { pre(OEMS_KC_LORENTZ); k_lorentz_apply<<<(l.count + 255) / 256, blk, 0, s>>>(e->dI, e->S, l); post(); ++L; }
    if (e->excI.count) { pre(OEMS_KC_EXCITE); k_excitation<<<(e->excI.count + 127) / 128, 128, 0, s>>>(e->dI, e->excI, e->d_numTS); post(); ++L; }
    if (carry_i)
        for (const auto& l : e->lorI) { pre(OEMS_KC_LORENTZ); k_lorentz_carry<<<(l.count + 255) / 256, blk, 0, s>>>(e->dI, e->S, l); post(); ++L; }
    // ---- processing + numTS
    if (se_split) {
        // the voltage side is done before the next voltage update; the current side (and the
        // numTS bump) runs beside it, joined there (or here at a sequence's last step)
        cudaStreamWaitEvent(s, e->ev_se_a, 0);
        cudaEventRecord(e->ev_se_fork, s);
        cudaStreamWaitEvent(e->stream_se, e->ev_se_fork, 0);
        k_step_end<<<e->stepend_blocks, blk, 0, e->stream_se>>>(g, e->stepend, 1);
        cudaEventRecord(e->ev_se_b, e->stream_se);
        ++L;
        e->se_pending = true;
        if (seq & 2) {
            cudaStreamWaitEvent(s, e->ev_se_b, 0);
            e->se_pending = false;
        }
    } else {
        pre(OEMS_KC_STEP_END);
        k_step_end<<<e->stepend_blocks, blk, 0, s>>>(g, e->stepend); ++L;
        post();
    }
    if (nlaunch) *nlaunch = L;
    cudaError_t c = cudaGetLastError();
    if (c != cudaSuccess) return cuda_fail(e, c, "kernel launch");
    return OEMS_OK;
}

extern "C" {

// the buffers and tables of the fused step (second field/flux set, source cells, both parities)
static int setup_fused(oems_cuda_engine* e)
{
    int rc;
    if ((rc = dalloc(e, &e->dV2, 3 * e->S, true))) return rc;
    if ((rc = dalloc(e, &e->dI2, 3 * e->S, true))) return rc;
    FusedDev base{};
    base.excV = e->excV;
    base.excI = e->excI;
    base.numTS = e->d_numTS;
    auto cells = [&](const std::vector<unsigned long long>& off, const unsigned long long** dptr,
                     unsigned long long& lo, unsigned long long& hi) -> int {
        *dptr = nullptr;
        lo = 1;
        hi = 0;
        if (off.empty()) return OEMS_OK;
        std::vector<unsigned long long> c(off.size());
        for (size_t k = 0; k < off.size(); ++k) c[k] = off[k] % e->S;
        lo = *std::min_element(c.begin(), c.end());
        hi = *std::max_element(c.begin(), c.end());
        unsigned long long* d = nullptr;
        const int r2 = dupload(e, &d, c.data(), c.size());
        *dptr = d;
        return r2;
    };
    if ((rc = cells(e->exc_voff, &base.srcV_cell, base.srcV_lo, base.srcV_hi))) return rc;
    if ((rc = cells(e->exc_ioff, &base.srcI_cell, base.srcI_lo, base.srcI_hi))) return rc;
    FusedDev& f0 = e->fused[0];
    FusedDev& f1 = e->fused[1];
    f0 = base;
    f1 = base;
    f0.g = e->grid;                                  // A -> B
    f0.Vo = e->dV2;
    f0.Io = e->dI2;
    f1.g = e->grid;                                  // B -> A
    f1.g.V = e->dV2;
    f1.g.I = e->dI2;
    f1.Vo = e->dV;
    f1.Io = e->dI;
    return OEMS_OK;
}

// cuTensorMapEncodeTiled from the driver (the runtime exports no wrapper)
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// rows per tile and x-planes per block of the plane march; OEMS_CUDA_MARCH_TY / _XCHUNK override
static void march_shape(const oems_cuda_engine* e, unsigned& ty, unsigned& xchunk, unsigned& smem)
{
    const unsigned Pz = e->Pz, G = Pz / 4;
    auto bytes_of = [&](unsigned t) {
        const unsigned slot = ((3u * (t + 2) * Pz + 31u) & ~31u), vbuf = ((3u * (t + 1) * Pz + 31u) & ~31u);
        return 4u * (3u * slot + 2u * vbuf) + 8u * MARCH_SLOTS;
    };
    // the largest tile of at most 512 threads (one block per SM: the kernel holds about 108
    // registers a thread) within the 227 KB of shared memory a block may have
    ty = 1;
    for (unsigned t = 1; t < 64 && (t + 2) * G <= 512 && t < e->N[1]; ++t)
        if (bytes_of(t + 1) <= 227u * 1024u) ty = t + 1;
    const char* s = getenv("OEMS_CUDA_MARCH_TY");
    if (s && atoi(s) > 0) ty = (unsigned)atoi(s);
    while (ty > 1 && ((ty + 1) * G > 512 || bytes_of(ty) > 227u * 1024u)) --ty;
    const unsigned long long tiles = (e->N[1] + ty - 1) / ty;
    // 32 planes per block (the fastest chunk on 256^3 and 512x512x256 meshes; 16 and 64 were
    // slower), fewer on small meshes so that every one of the 152 SMs gets a block: 4..32
    xchunk = (unsigned)std::min<unsigned long long>(32, std::max<unsigned long long>(4, e->N[0] * tiles / 152));
    const char* xc = getenv("OEMS_CUDA_MARCH_XCHUNK");
    if (xc && atoi(xc) > 0) xchunk = (unsigned)atoi(xc);
    smem = bytes_of(ty);
}

// the plane march on top of the fused step's buffers (setup_fused must have run)
static int setup_march(oems_cuda_engine* e)
{
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) return fail(e, OEMS_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    unsigned ty, xchunk, smem;
    march_shape(e, ty, xchunk, smem);
    int rc;
    if ((rc = dalloc(e, &e->d_march_err, 1, true))) return rc;
    const unsigned Pz = e->Pz;
    for (int p = 0; p < 2; ++p) {
        MarchDev& m = e->march[p];
        m.f = e->fused[p];
        m.ty = ty;
        m.groups = Pz / 4;
        m.xchunk = xchunk;
        m.slot_floats = (3u * (ty + 2) * Pz + 31u) & ~31u;
        m.box_bytes = 12u * (ty + 2) * Pz;
        m.vbuf_floats = (3u * (ty + 1) * Pz + 31u) & ~31u;
        m.err = e->d_march_err;
        // I of the input set as [3][Nx][Ny][Pz]; one box = all z, ty + 2 rows, one plane, 3 components
        const cuuint64_t dims[4] = {Pz, e->N[1], e->N[0], 3};
        const cuuint64_t strides[3] = {(cuuint64_t)Pz * 4, (cuuint64_t)e->N[1] * Pz * 4, (cuuint64_t)e->S * 4};
        const cuuint32_t box[4] = {Pz, ty + 2, 1, 3};
        const cuuint32_t estr[4] = {1, 1, 1, 1};
        const CUresult r = enc(&e->march_map[p], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, (void*)m.f.g.I, dims, strides, box,
                               estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                               CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return fail(e, OEMS_ERR_CUDA, "cuTensorMapEncodeTiled failed for the plane march");
    }
    e->march_threads = (((ty + 1) * (Pz / 4)) + 31u) & ~31u;
    e->march_smem = smem;
    e->march_grid = dim3((e->N[1] + ty - 1) / ty, (e->N[0] + xchunk - 1) / xchunk);
    const char* mb = getenv("OEMS_CUDA_MARCH_MINB");
    e->march_minb = (mb && mb[0] == '2') ? 2 : 1;
    CK(cudaFuncSetAttribute(k_step_march<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CK(cudaFuncSetAttribute(k_step_march<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    return OEMS_OK;
}

static int capture(oems_cuda_engine* e, unsigned steps, cudaGraphExec_t* out, bool fused)
{
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
    int rc = OEMS_OK;
    for (unsigned s = 0; s < steps && rc == OEMS_OK; ++s) {
        const unsigned seq = (s == 0 ? 1u : 0u) | (s + 1 == steps ? 2u : 0u);
        // launches per step: a step inside the sequence where there is one
        const bool count = s == (steps > 2 ? 1u : 0u);
        rc = fused ? enqueue_fused_step(e, (int)(s & 1), s == 0 ? &e->fused_launches : nullptr)
                   : enqueue_step(e, count ? &e->launches : nullptr, nullptr, seq);
    }
    cudaError_t c = cudaStreamEndCapture(e->stream, &graph);
    if (rc) { if (graph) cudaGraphDestroy(graph); return rc; }
    if (c != cudaSuccess) return cuda_fail(e, c, "cudaStreamEndCapture");
    c = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    if (c != cudaSuccess) return cuda_fail(e, c, "cudaGraphInstantiate");
    return OEMS_OK;
}

int oems_cuda_init(oems_cuda_engine* e, unsigned int max_ts)
{
    if (!e) return OEMS_ERR_ARG;
    if (e->inited) return fail(e, OEMS_ERR_STATE, "engine already initialised");
    if (!e->op_set) return fail(e, OEMS_ERR_STATE, "operator not set");
    CK(cudaSetDevice(e->device));
    int rc;
    e->max_ts = max_ts;
    GridDev& g = e->grid;
    g.Nx = e->N[0]; g.Ny = e->N[1]; g.Nz = e->N[2]; g.Pz = e->Pz; g.S = e->S;
    g.V = e->dV; g.I = e->dI;
    g.idx = e->didx; g.tabV = e->dtabV; g.tabI = e->dtabI;
    g.vv = e->dvv; g.vi = e->dvi; g.ii = e->dii; g.iv = e->div;
    // the class index in 16 bits where every class fits: 2 bytes less per cell and half-step for
    // every update kernel (OEMS_CUDA_IDX16=0 keeps the 32-bit index)
    g.idx16 = nullptr;
    {
        const char* ix = getenv("OEMS_CUDA_IDX16");
        if (e->compressed && e->didx && e->nclasses <= 65536u && !(ix && ix[0] == '0')) {
            unsigned short* d16 = nullptr;
            if ((rc = dalloc(e, &d16, (size_t)e->S, false))) return rc;
            k_narrow_index<<<(unsigned)((e->S + 255) / 256), 256, 0, e->stream>>>(d16, e->didx, e->S);
            CK(cudaGetLastError());
            g.idx16 = d16;
        }
    }

    // float4 update kernels (OEMS_CUDA_SCALAR=1 keeps the one-cell-per-thread form)
    {
        const char* sc = getenv("OEMS_CUDA_SCALAR");
        e->vec4 = !(sc && sc[0] == '1');
        // threads per block of the float4 updates: 128 measured faster than 256 on 512x512x256
        // (the voltage update with the Mur walls 0.408 -> 0.394 ms, the current update 0.392 ->
        // 0.387 ms); OEMS_CUDA_I4_BLOCK / OEMS_CUDA_V4_BLOCK = 256 restores the larger blocks
        // (64 for the voltage update: 0.394 -> 0.392 ms more; the current update gains nothing
        // below 128)
        auto block_env = [](const char* name, unsigned dflt) -> unsigned {
            const char* v = getenv(name);
            const int b = v ? atoi(v) : 0;
            return (b == 64 || b == 128 || b == 256) ? (unsigned)b : dflt;
        };
        e->i4_block = block_env("OEMS_CUDA_I4_BLOCK", 128u);
        e->v4_block = block_env("OEMS_CUDA_V4_BLOCK", 64u);
        // and of the UPML main box (design mesh 92.2 -> 91.2 us per step, 512x512x256 with UPML
        // 1.075 -> 1.059 ms); OEMS_CUDA_BOX4_BLOCK=256 restores the larger blocks
        e->box_block = block_env("OEMS_CUDA_BOX4_BLOCK", 128u);
        // and of the UPML region kernel (patch 47.2 -> 45.8 us per step); OEMS_CUDA_REG4_BLOCK=256
        const char* rb = getenv("OEMS_CUDA_REG4_BLOCK");
        e->reg_block = (rb && atoi(rb) == 256) ? 256u : 128u;
        // the reverse sweep's main box and regions (1,384 -> 1,360 ms for the 8,000-step design
        // run; OEMS_CUDA_ADJ_BLOCK=256 restores the larger blocks)
        const char* ab = getenv("OEMS_CUDA_ADJ_BLOCK");
        e->adj_box_block = e->adj_reg_block = (ab && atoi(ab) == 256) ? 256u : 128u;
    }

    // UPML
    g.nupml = (int)e->upml.size();
    for (size_t r = 0; r < e->upml.size(); ++r) {
        const UpmlHost& u = e->upml[r];
        UpmlDev& d = g.upml[r];
        memcpy(d.start, u.start, 12);
        memcpy(d.nl, u.nl, 12);
        d.n = u.nl[0] * u.nl[1] * u.nl[2];
        std::vector<unsigned short> cls;
        std::vector<float4> ctab;
        d.cls = nullptr; d.ctab = nullptr;
        d.vv = d.vvfo = d.vvfn = d.ii = d.iifo = d.iifn = nullptr;
        if (compress_upml(u, cls, ctab)) {
            unsigned short* dc;
            float4* dt;
            if ((rc = dupload(e, &dc, cls.data(), cls.size()))) return rc;
            if ((rc = dupload(e, &dt, ctab.data(), ctab.size()))) return rc;
            d.cls = dc; d.ctab = dt;
        } else {
            float* t[6];
            for (int k = 0; k < 6; ++k)
                if ((rc = dupload(e, &t[k], u.tab[k].data(), u.tab[k].size()))) return rc;
            d.vv = t[0]; d.vvfo = t[1]; d.vvfn = t[2]; d.ii = t[3]; d.iifo = t[4]; d.iifn = t[5];
        }
        if ((rc = dalloc(e, &d.vflux, 3 * (size_t)d.n, true, true))) return rc;
        if ((rc = dalloc(e, &d.iflux, 3 * (size_t)d.n, true, true))) return rc;
    }

    e->use_split = g.nupml > 0;
    if (e->use_split) {
        const unsigned RV[3] = {e->N[0], e->N[1], e->N[2]};
        const unsigned RI[3] = {e->N[0] - 1, e->N[1] - 1, e->N[2] - 1};
        make_split(e, RV, e->splitV);
        make_split(e, RI, e->splitI);
        // the region kernel and the main box run as two branches (a fork/join in the graphs), so
        // the latency-bound region blocks overlap the streaming box; OEMS_CUDA_SPLIT_BRANCH=0
        // runs them one after the other on the engine stream
        const char* br = getenv("OEMS_CUDA_SPLIT_BRANCH");
        if (e->splitV.v4 && !(br && br[0] == '0')) {
            CK(cudaStreamCreateWithFlags(&e->stream_r, cudaStreamNonBlocking));
            CK(cudaEventCreateWithFlags(&e->ev_fork, cudaEventDisableTiming));
            CK(cudaEventCreateWithFlags(&e->ev_join, cudaEventDisableTiming));
        }
    }

    // excitation
    auto setup_exc = [&](ExcDev& x, const std::vector<unsigned long long>& off, const std::vector<float>& amp,
                         const std::vector<unsigned>& delay, const std::vector<float>& sig) -> int {
        x.count = (unsigned)off.size();
        x.length = e->sig_len;
        x.period = e->period;
        if (!x.count) return OEMS_OK;
        int r2;
        unsigned long long* o; float* a; unsigned* dl; float* sg;
        if ((r2 = dupload(e, &o, off.data(), off.size()))) return r2;
        if ((r2 = dupload(e, &a, amp.data(), amp.size()))) return r2;
        if ((r2 = dupload(e, &dl, delay.data(), delay.size()))) return r2;
        if ((r2 = dupload(e, &sg, sig.data(), sig.size()))) return r2;
        x.off = o; x.amp = a; x.delay = dl; x.sig = sg;
        return OEMS_OK;
    };
    if ((rc = setup_exc(e->excV, e->exc_voff, e->exc_vamp, e->exc_vdelay, e->sig_v))) return rc;
    if ((rc = setup_exc(e->excI, e->exc_ioff, e->exc_iamp, e->exc_idelay, e->sig_i))) return rc;

    // Mur
    e->murdev.nwall = (int)e->mur.size();
    for (size_t w = 0; w < e->mur.size(); ++w) {
        const MurHost& m = e->mur[w];
        MurWallDev& d = e->murdev.w[w];
        d.ny = m.ny; d.nyP = (m.ny + 1) % 3; d.nyPP = (m.ny + 2) % 3;
        d.line = m.line; d.shift = m.shift; d.start_ts = m.start_ts;
        d.n1 = e->N[d.nyP]; d.n2 = e->N[d.nyPP];
        float *cp, *cpp;
        if (d.nyP == 2) {
            // tables with z tangential go up z fastest ([n2][n1], mur_k)
            std::vector<float> tP(m.cP.size()), tPP(m.cPP.size());
            for (unsigned i = 0; i < d.n1; ++i)
                for (unsigned j = 0; j < d.n2; ++j) {
                    tP[(size_t)j * d.n1 + i] = m.cP[(size_t)i * d.n2 + j];
                    tPP[(size_t)j * d.n1 + i] = m.cPP[(size_t)i * d.n2 + j];
                }
            if ((rc = dupload(e, &cp, tP.data(), tP.size()))) return rc;
            if ((rc = dupload(e, &cpp, tPP.data(), tPP.size()))) return rc;
        } else {
            if ((rc = dupload(e, &cp, m.cP.data(), m.cP.size()))) return rc;
            if ((rc = dupload(e, &cpp, m.cPP.data(), m.cPP.size()))) return rc;
        }
        d.cP = cp; d.cPP = cpp;
        if ((rc = dalloc(e, &d.bP, m.cP.size(), true, true))) return rc;
        if ((rc = dalloc(e, &d.bPP, m.cP.size(), true, true))) return rc;
    }
    // per axis: the walls with that normal, and the window of coordinates that are no line or
    // shift of them (lines below the middle bound it from below, the others from above)
    {
        int j = 0;
        for (int a = 0; a < 3; ++a) {
            e->murdev.first[a] = j;
            unsigned lo = 0, hi = e->N[a] - 1;
            for (size_t w = 0; w < e->mur.size(); ++w) {
                if (e->mur[w].ny != a) continue;
                e->murdev.order[j++] = (int)w;
                for (unsigned c : {e->mur[w].line, e->mur[w].shift}) {
                    if (2 * c < e->N[a]) lo = std::max(lo, c + 1);
                    else if (c >= 1) hi = std::min(hi, c - 1);
                    else lo = e->N[a];
                }
            }
            if (lo <= hi && lo < e->N[a]) { e->murdev.lo[a] = lo; e->murdev.span[a] = hi - lo; }
            else { e->murdev.lo[a] = e->N[a]; e->murdev.span[a] = 0; }   // no window: every coordinate is checked
        }
        e->murdev.first[3] = j;
    }
    // the lane-parallel z-wall form needs at most two z walls with neighbouring line and shift
    // and four distinct z among them (nz = -1: every wall goes through mur_cell)
    {
        MurDev& md = e->murdev;
        md.nz = 0;
        std::vector<unsigned> zs;
        for (int q = md.first[2]; q < md.first[3]; ++q) {
            const MurWallDev& d = md.w[md.order[q]];
            const bool adjacent = d.line + 1 == d.shift || d.shift + 1 == d.line;
            if (md.nz >= 2 || !adjacent) { md.nz = -1; break; }
            md.z[md.nz++] = d;
            zs.push_back(d.line);
            zs.push_back(d.shift);
        }
        std::sort(zs.begin(), zs.end());
        if (md.nz >= 0 && std::adjacent_find(zs.begin(), zs.end()) != zs.end()) md.nz = -1;
        // OEMS_CUDA_MUR_SEPARATE=1: the pre/post hooks as separate launches (k_mur phases 0/1).
        // A TFSF plane wave needs them too: its post-voltage hook (priority 5e4) runs before the
        // Mur post hook (priority 0) and may change the values Mur reads at a shift line.  So do
        // lumped RLC loads: their apply reads the raw updated value of an edge that may be a
        // Mur line, which the form inside the voltage update does not keep.
        const char* ms = getenv("OEMS_CUDA_MUR_SEPARATE");
        // The cylinder's post-voltage hook (priority 1e5) rewrites the alpha seam and the axis
        // before the Mur post hook reads its lines, so it needs them too.
        e->mur_separate = (ms && ms[0] == '1') || e->has_tfsf || !e->rlc_host.off.empty() || e->cyl_closed;
        // the lane-parallel form: no UPML (plain update kernel), every wall active from step 0
        bool always = true;
        for (const auto& m : e->mur) always = always && m.start_ts == 0;
        md.lanes = (!e->mur.empty() && !e->mur_separate && md.nz >= 0 && g.nupml == 0 && always) ? 1 : 0;
        // the float4 form of the lane-parallel hooks (k_update_v4w): each z wall's line and shift
        // in one group of four z, no group with two walls; OEMS_CUDA_MUR_V4=0 keeps the one-cell form
        bool groups_ok = md.nz >= 0;
        for (int q = 0; q < md.nz && groups_ok; ++q) groups_ok = (md.z[q].line >> 2) == (md.z[q].shift >> 2);
        if (md.nz == 2) groups_ok = groups_ok && (md.z[0].line >> 2) != (md.z[1].line >> 2);
        const char* mv = getenv("OEMS_CUDA_MUR_V4");
        e->mur_v4 = md.lanes && groups_ok && !(mv && mv[0] == '0');
        // park mode of the float4 form (OEMS_CUDA_MUR_PARK=1): the direct columns' z-wall hooks as
        // k_mur_zsave before and k_mur_zpost after the update.  The update itself then streams
        // every group, but the two wall-plane kernels read one sector per z row at a row stride
        // and cost more than they save, so the default keeps the hooks inside the update.
        const char* mp = getenv("OEMS_CUDA_MUR_PARK");
        md.park = (e->mur_v4 && md.nz > 0 && mp && mp[0] == '1') ? 1 : 0;
        md.zsave = nullptr;
        if (md.park && (rc = dalloc(e, &md.zsave, 2 * (size_t)md.nz * e->N[0] * e->N[1], true))) return rc;
        // the flat apply: with the lane-parallel form a z wall's apply visits only the columns
        // that are not direct (the update stores the direct ones' final values)
        md.zedge = nullptr;
        md.nzedge = 0;
        if (md.lanes && md.first[3] > md.first[2]) {
            std::vector<unsigned> edge;
            for (unsigned x = 0; x < e->N[0]; ++x)
                for (unsigned y = 0; y < e->N[1]; ++y) {
                    const bool direct = (x - md.lo[0] <= md.span[0]) && (y - md.lo[1] <= md.span[1]);
                    if (!direct) edge.push_back(x * e->N[1] + y);
                }
            md.nzedge = (unsigned)edge.size();
            unsigned* de = nullptr;
            if (!edge.empty() && (rc = dupload(e, &de, edge.data(), edge.size()))) return rc;
            md.zedge = de;
        }
        md.afirst[0] = 0;
        for (int w = 0; w < md.nwall; ++w) {
            const MurWallDev& d = md.w[w];
            const unsigned pts = (md.lanes && d.ny == 2 && md.zedge) ? md.nzedge : d.n1 * d.n2;
            md.afirst[w + 1] = md.afirst[w] + (pts + 255) / 256;
        }
    }

    // cylinder extension
    if (e->cyl_closed) {
        e->cyl.closed = 1;
        e->cyl.r0 = e->cyl_r0;
        if (e->cyl_r0) {
            float *a, *b;
            if ((rc = dupload(e, &a, e->cyl_vv_r0.data(), e->cyl_vv_r0.size()))) return rc;
            if ((rc = dupload(e, &b, e->cyl_vi_r0.data(), e->cyl_vi_r0.size()))) return rc;
            e->cyl.vv_r0 = a;
            e->cyl.vi_r0 = b;
        }
    }

    // TFSF: group the terms by target cell (stable, so each cell keeps the reference's order)
    if (e->has_tfsf) {
        float *sv, *si;
        if ((rc = dupload(e, &sv, e->tfsf_sig_v.data(), e->tfsf_sig_v.size()))) return rc;
        if ((rc = dupload(e, &si, e->tfsf_sig_i.data(), e->tfsf_sig_i.size()))) return rc;
        for (int w = 0; w < 2; ++w) {
            const TfsfHost& t = w ? e->tfsf_i : e->tfsf_v;
            TfsfDev& d = w ? e->tfsfI : e->tfsfV;
            d = TfsfDev{};
            d.sig = w ? sv : si;   // the voltage hook adds the current signal and vice versa
            d.length = e->tfsf_len;
            d.period = e->tfsf_period;
            const size_t n = t.off.size();
            if (!n) continue;
            std::vector<unsigned> order(n);
            for (size_t k = 0; k < n; ++k) order[k] = (unsigned)k;
            std::stable_sort(order.begin(), order.end(), [&](unsigned a, unsigned b) { return t.off[a] < t.off[b]; });
            std::vector<unsigned long long> toff;
            std::vector<unsigned> first, dl;
            std::vector<float> dd, am;
            for (size_t q = 0; q < n; ++q) {
                const unsigned k = order[q];
                if (toff.empty() || toff.back() != t.off[k]) { toff.push_back(t.off[k]); first.push_back((unsigned)q); }
                dl.push_back(t.delay[k]);
                dd.push_back(t.delta[k]);
                am.push_back(t.amp[k]);
            }
            first.push_back((unsigned)n);
            unsigned long long* o;
            unsigned *f, *de;
            float *dt, *ap;
            if ((rc = dupload(e, &o, toff.data(), toff.size()))) return rc;
            if ((rc = dupload(e, &f, first.data(), first.size()))) return rc;
            if ((rc = dupload(e, &de, dl.data(), dl.size()))) return rc;
            if ((rc = dupload(e, &dt, dd.data(), dd.size()))) return rc;
            if ((rc = dupload(e, &ap, am.data(), am.size()))) return rc;
            d.ntarget = (unsigned)toff.size();
            d.off = o; d.first = f; d.delay = de; d.delta = dt; d.amp = ap;
        }
    }

    // lumped RLC loads
    if (!e->rlc_host.off.empty()) {
        RlcDev& r = e->rlc;
        r.count = (unsigned)e->rlc_host.off.size();
        unsigned long long* o;
        float* c;
        if ((rc = dupload(e, &o, e->rlc_host.off.data(), e->rlc_host.off.size()))) return rc;
        if ((rc = dupload(e, &c, e->rlc_host.c.data(), e->rlc_host.c.size()))) return rc;
        r.off = o;
        r.c = c;
        if ((rc = dalloc(e, &r.il, r.count, true, true))) return rc;
        if ((rc = dalloc(e, &r.vd, 3 * (size_t)r.count, true, true))) return rc;
        if ((rc = dalloc(e, &r.j, 3 * (size_t)r.count, true, true))) return rc;
    }

    // Lorentz / Drude orders
    // the cells (component 0 offsets) of the excitation edges, sorted
    auto exc_cells = [&](const std::vector<unsigned long long>& off) {
        std::vector<unsigned long long> c;
        for (auto o : off) c.push_back(o % e->S);
        std::sort(c.begin(), c.end());
        return c;
    };
    const std::vector<unsigned long long> exc_v = exc_cells(e->exc_voff), exc_i = exc_cells(e->exc_ioff);
    {
        const char* lc = getenv("OEMS_CUDA_LOR_CARRY");
        const bool on = !(lc && lc[0] == '0');
        // the carried apply moves past the Mur apply: only where the walls' components are in skip.
        // One order only: a position in two orders takes both applies before either pre.
        const bool one = e->lor.size() <= 1;
        e->lor_carry_v = on && one && (e->mur.empty() || e->murdev.lanes);
        e->lor_carry_i = on && one;
    }
    for (const auto& l : e->lor) {
        std::vector<unsigned long long> off(l.count);
        for (unsigned i = 0; i < l.count; ++i) off[i] = cell_off(e, 0, l.pos[i], l.pos[l.count + i], l.pos[2 * l.count + i]);
        // 32-bit offsets when every component's offset fits
        const bool o32 = 3ull * e->S < (1ull << 32);
        unsigned long long* doff = nullptr;
        unsigned* doff32 = nullptr;
        if (o32) {
            std::vector<unsigned> o(off.begin(), off.end());
            if ((rc = dupload(e, &doff32, o.data(), o.size()))) return rc;
        } else if ((rc = dupload(e, &doff, off.data(), off.size()))) return rc;
        // an excitation edge among the positions' components keeps the apply in its own place
        for (unsigned i = 0; i < l.count; ++i) {
            if (l.von && !exc_v.empty() && std::binary_search(exc_v.begin(), exc_v.end(), off[i])) e->lor_carry_v = false;
            if (l.con && !exc_i.empty() && std::binary_search(exc_i.begin(), exc_i.end(), off[i])) e->lor_carry_i = false;
        }
        const size_t m = 3 * (size_t)l.count;
        // coefficient classes: each position's nine coefficients (int, ext, lor per component)
        // as an index into a table of distinct tuples, bit-exact (keys are the float bits)
        auto classes = [&](const std::vector<float>& ci, const std::vector<float>& ce, const std::vector<float>& cl,
                           bool lor, LorDev& d) -> int {
            std::vector<unsigned short> cls(l.count);
            std::vector<float> tab;                                // 12 floats per class
            std::vector<int> slot(1u << 17, -1);                   // open addressing over class ids
            unsigned ncls = 0;
            uint32_t prev[9];
            int prev_c = -1;
            for (unsigned i = 0; i < l.count; ++i) {
                float t[9];
                for (unsigned n = 0; n < 3; ++n) {
                    t[n] = ci[n * l.count + i];
                    t[3 + n] = ce[n * l.count + i];
                    t[6 + n] = lor ? cl[n * l.count + i] : 0.f;
                }
                uint32_t w[9];
                memcpy(w, t, sizeof w);
                if (prev_c >= 0 && !memcmp(w, prev, sizeof w)) { cls[i] = (unsigned short)prev_c; continue; }
                uint64_t h = 1469598103934665603ull;
                for (int k = 0; k < 9; ++k) h = (h ^ w[k]) * 1099511628211ull;
                const size_t mask = slot.size() - 1;
                size_t q = (size_t)(h ^ (h >> 29)) & mask;
                int c = -1;
                while (slot[q] >= 0) {
                    if (!memcmp(&tab[12 * (size_t)slot[q]], t, sizeof t)) { c = slot[q]; break; }
                    q = (q + 1) & mask;
                }
                if (c < 0) {
                    if (ncls >= 65536 || 2 * (ncls + 1) > slot.size()) return OEMS_OK;   // too many: raw arrays
                    c = (int)ncls++;
                    slot[q] = c;
                    tab.insert(tab.end(), t, t + 9);
                    tab.insert(tab.end(), 3, 0.f);
                }
                cls[i] = (unsigned short)c;
                memcpy(prev, w, sizeof w);
                prev_c = c;
            }
            unsigned short* dc = nullptr;
            float* dt = nullptr;
            int r2;
            if ((r2 = dupload(e, &dc, cls.data(), cls.size()))) return r2;
            if ((r2 = dupload(e, &dt, tab.data(), tab.size()))) return r2;
            d.cls = dc;
            d.ctab = reinterpret_cast<const float4*>(dt);
            return OEMS_OK;
        };
        if (l.von) {
            LorDev d{};
            d.count = l.count; d.off = doff; d.off32 = doff32; d.lor = l.vlon;
            if (e->murdev.lanes) {
                // the voltage update writes final Mur values: the apply leaves every component an
                // (always active) wall owns alone, as the reference's later Mur apply overwrites it
                std::vector<unsigned char> sk(l.count, 0);
                bool any = false;
                for (unsigned i = 0; i < l.count; ++i) {
                    const unsigned p[3] = {l.pos[i], l.pos[l.count + i], l.pos[2 * l.count + i]};
                    for (const auto& w : e->mur)
                        if (p[w.ny] == w.line) sk[i] |= (unsigned char)(7u & ~(1u << w.ny));
                    any = any || sk[i];
                }
                unsigned char* dsk = nullptr;
                if (any && (rc = dupload(e, &dsk, sk.data(), sk.size()))) return rc;
                d.skip = dsk;
            }
            if ((rc = classes(l.vint, l.vext, l.vlor, l.vlon, d))) return rc;
            if (!d.cls) {
                float *ci, *ce, *cl = nullptr;
                if ((rc = dupload(e, &ci, l.vint.data(), m))) return rc;
                if ((rc = dupload(e, &ce, l.vext.data(), m))) return rc;
                if (l.vlon && (rc = dupload(e, &cl, l.vlor.data(), m))) return rc;
                d.c_int = ci; d.c_ext = ce; d.c_lor = cl;
            }
            if ((rc = dalloc(e, &d.ade, m, true, true))) return rc;
            if (l.vlon && (rc = dalloc(e, &d.lade, m, true, true))) return rc;
            e->lorV.push_back(d);
        }
        if (l.con) {
            LorDev d{};
            d.count = l.count; d.off = doff; d.off32 = doff32; d.lor = l.clon;
            if ((rc = classes(l.iint, l.iext, l.ilor, l.clon, d))) return rc;
            if (!d.cls) {
                float *ci, *ce, *cl = nullptr;
                if ((rc = dupload(e, &ci, l.iint.data(), m))) return rc;
                if ((rc = dupload(e, &ce, l.iext.data(), m))) return rc;
                if (l.clon && (rc = dupload(e, &cl, l.ilor.data(), m))) return rc;
                d.c_int = ci; d.c_ext = ce; d.c_lor = cl;
            }
            if ((rc = dalloc(e, &d.ade, m, true, true))) return rc;
            if (l.clon && (rc = dalloc(e, &d.lade, m, true, true))) return rc;
            e->lorI.push_back(d);
        }
    }

    // the voltage half-step's end as one launch (k_vtail): the Mur apply, the dispersive carry
    // (inside a sequence) or apply (its last step, a single step) and the excitation touch
    // disjoint values
    e->vtail = false;
    if (e->lor_carry_v && e->lorV.size() == 1 && !e->lorV[0].skip) {
        bool ok = true;
        const unsigned long long plane = (unsigned long long)e->N[1] * e->Pz;
        for (auto o : e->exc_voff) {
            const unsigned n = (unsigned)(o / e->S);
            const unsigned long long c = o % e->S;
            const unsigned p[3] = {(unsigned)(c / plane), (unsigned)((c / e->Pz) % e->N[1]), (unsigned)(c % e->Pz)};
            for (const auto& w : e->mur)
                if (p[w.ny] == w.line && (int)n != w.ny) ok = false;
        }
        const char* vt = getenv("OEMS_CUDA_VTAIL");
        e->vtail = ok && !(vt && vt[0] == '0');
    }

    // probes: term lists in the reference's summation order + phasor tables
    for (const auto& p : e->probes) {
        ProbeDev d{};
        d.type = p.type;
        std::vector<unsigned long long> term;
        std::vector<signed char> sign;
        auto add = [&](int comp, unsigned x, unsigned y, unsigned z, int sg) {
            term.push_back(cell_off(e, comp, x, y, z));
            sign.push_back((signed char)sg);
        };
        if (p.type >= 2) {  // ProcessFieldProbe: one term per component, divided by its edge length
            for (int n = 0; n < 3; ++n) {
                add(n, p.start[0], p.start[1], p.start[2], +1);
                d.el[n] = p.el[n];
            }
        } else if (p.type == 0) {  // Engine_Interface_FDTD::CalcVoltageIntegral
            for (int n = 0; n < 3; ++n) {
                if (p.start[n] < p.stop[n]) {
                    unsigned pos[3] = {p.start[0], p.start[1], p.start[2]};
                    for (; pos[n] < p.stop[n]; ++pos[n]) add(n, pos[0], pos[1], pos[2], +1);
                } else {
                    unsigned pos[3] = {p.stop[0], p.stop[1], p.stop[2]};
                    for (; pos[n] < p.start[n]; ++pos[n]) add(n, pos[0], pos[1], pos[2], -1);
                }
            }
        } else {  // ProcessCurrent::CalcIntegral
            const unsigned *s = p.start, *t = p.stop;
            const int *si = p.si, *ei = p.ei;
            switch (p.nd) {
            case 0:
                if (ei[0] && si[2]) for (unsigned i = s[1] + 1; i <= t[1]; ++i) add(1, t[0], i, s[2], +1);
                if (ei[0] && ei[1]) for (unsigned i = s[2] + 1; i <= t[2]; ++i) add(2, t[0], t[1], i, +1);
                if (si[0] && ei[2]) for (unsigned i = s[1] + 1; i <= t[1]; ++i) add(1, s[0], i, t[2], -1);
                if (si[0] && si[1]) for (unsigned i = s[2] + 1; i <= t[2]; ++i) add(2, s[0], s[1], i, -1);
                break;
            case 1:
                if (si[0] && si[1]) for (unsigned i = s[2] + 1; i <= t[2]; ++i) add(2, s[0], s[1], i, +1);
                if (ei[1] && ei[2]) for (unsigned i = s[0] + 1; i <= t[0]; ++i) add(0, i, t[1], t[2], +1);
                if (ei[0] && ei[1]) for (unsigned i = s[2] + 1; i <= t[2]; ++i) add(2, t[0], t[1], i, -1);
                if (si[1] && si[2]) for (unsigned i = s[0] + 1; i <= t[0]; ++i) add(0, i, s[1], s[2], -1);
                break;
            default:
                if (si[1] && si[2]) for (unsigned i = s[0] + 1; i <= t[0]; ++i) add(0, i, s[1], s[2], +1);
                if (ei[0] && si[2]) for (unsigned i = s[1] + 1; i <= t[1]; ++i) add(1, t[0], i, s[2], +1);
                if (ei[1] && ei[2]) for (unsigned i = s[0] + 1; i <= t[0]; ++i) add(0, i, t[1], t[2], -1);
                if (si[0] && ei[2]) for (unsigned i = s[1] + 1; i <= t[1]; ++i) add(1, s[0], i, t[2], -1);
                break;
            }
        }
        d.nterm = (unsigned)term.size();
        unsigned long long* dt_; signed char* ds;
        if ((rc = dupload(e, &dt_, term.data(), term.size()))) return rc;
        if ((rc = dupload(e, &ds, sign.data(), sign.size()))) return rc;
        d.term = dt_; d.sign = ds;
        d.weight = p.weight;
        d.interval = p.interval; d.start_ts = p.start_ts; d.stop_ts = p.stop_ts;
        d.nslots = max_ts / p.interval + 1;
        d.ncomp = p.type >= 2 ? 3u : 1u;
        {
            std::vector<double> nan((size_t)d.nslots * d.ncomp, std::nan(""));
            double* ser;
            if ((rc = dupload(e, &ser, nan.data(), nan.size()))) return rc;
            e->state.push_back({ser, nan.size() * sizeof(double)});
            d.series = ser;
        }
        d.fd_interval = p.fd_interval;
        d.nf = (unsigned)p.freqs.size();
        d.dt = e->dt;
        if (d.fd_interval && d.nf) {
            d.nsamp = max_ts / d.fd_interval + 1;
            std::vector<double2> ph((size_t)d.nsamp * d.nf);
            for (unsigned k = 0; k < d.nsamp; ++k) {
                const double ts = (double)k * d.fd_interval;
                const double time = (ts + (double)(p.type == 1 || p.type == 3) * 0.5) * e->dt;
                for (unsigned f = 0; f < d.nf; ++f) {
                    const std::complex<double> ex = std::exp(std::complex<double>(-0.0, ((-2.0 * kPI) * p.freqs[f]) * time));
                    ph[(size_t)k * d.nf + f] = make_double2(ex.real(), ex.imag());
                }
            }
            double2* dph;
            if ((rc = dupload(e, &dph, ph.data(), ph.size()))) return rc;
            d.phasor = dph;
            double* dd;
            if ((rc = dalloc(e, &dd, 2 * (size_t)d.nf * d.ncomp, true, true))) return rc;
            d.dft = dd;
        } else {
            d.fd_interval = 0;
            d.nf = 0;
        }
        e->probe_dev.push_back(d);
    }
    // mapped host memory for the probes' newest samples: [nprobe][3] values, then [nprobe] slots
    if (!e->probe_dev.empty()) {
        const size_t np = e->probe_dev.size();
        void* h = nullptr;
        CK(cudaHostAlloc(&h, np * (3 * sizeof(double) + sizeof(unsigned)), cudaHostAllocMapped));
        e->latest_host = static_cast<double*>(h);
        e->latest_slot_host = reinterpret_cast<unsigned*>(e->latest_host + 3 * np);
        for (size_t j = 0; j < np; ++j) e->latest_slot_host[j] = UINT_MAX;
        void* dv = nullptr;
        CK(cudaHostGetDevicePointer(&dv, h, 0));
        double* dl = static_cast<double*>(dv);
        for (size_t j = 0; j < np; ++j) {
            e->probe_dev[j].latest = dl + 3 * j;
            e->probe_dev[j].latest_slot = reinterpret_cast<unsigned*>(dl + 3 * np) + j;
        }
    }

    // FD dumps
    std::vector<unsigned> block0(1, 1u);
    for (const auto& p : e->dumps) {
        DumpDev d{};
        d.field = p.field;
        d.interp = p.interp;
        for (int a = 0; a < 3; ++a) { d.start[a] = p.start[a]; d.sz[a] = p.stop[a] - p.start[a] + 1; }
        d.npos = d.sz[0] * d.sz[1] * d.sz[2];
        d.fd_interval = p.fd_interval;
        d.nf = (unsigned)p.freqs.size();
        if (p.td) {
            // ring of device slots: up to two K-step graphs of samples within about 1 GB
            const size_t slot_bytes = 12ull * d.npos;
            const size_t fit = std::max<size_t>(1, (size_t(1) << 30) / slot_bytes);
            d.td = 1;
            d.td_interval = p.td_interval;
            d.td_start = p.td_start;
            d.td_stop = p.td_stop;
            d.nslot = (unsigned)std::min<size_t>(2ull * e->K, fit);
            // OEMS_CUDA_TD_SLOTS=n caps the ring (small rings exercise the flush and single-step paths)
            if (const char* ev = getenv("OEMS_CUDA_TD_SLOTS")) {
                const long v = strtol(ev, nullptr, 10);
                if (v >= 1 && (unsigned long)v < d.nslot) d.nslot = (unsigned)v;
            }
            float* ring;
            if ((rc = dalloc(e, &ring, (size_t)d.nslot * 3 * d.npos, true))) return rc;
            d.ring = ring;
            d.fd_interval = 0;
            d.nf = 0;
        } else if (d.fd_interval && d.nf) {
            d.nsamp = max_ts / d.fd_interval + 1;
            std::vector<float2> ph((size_t)d.nsamp * d.nf);
            for (unsigned k = 0; k < d.nsamp; ++k) {
                const double ts = (double)k * d.fd_interval;
                const double T = (ts + (double)(p.field == 1) * 0.5) * e->dt;
                for (unsigned f = 0; f < d.nf; ++f) {
                    // ProcessFieldsFD::Process: exp in complex<float>, *2, *dt*FD_Interval
                    std::complex<float> ex = std::exp(std::complex<float>(-0.0f, (float)(((-2.0 * kPI) * p.freqs[f]) * T)));
                    ex *= 2.0f;
                    ex *= (float)(e->dt * (double)d.fd_interval);
                    ph[(size_t)k * d.nf + f] = make_float2(ex.real(), ex.imag());
                }
            }
            float2* dph;
            if ((rc = dupload(e, &dph, ph.data(), ph.size()))) return rc;
            d.phasor = dph;
        } else {
            d.fd_interval = 0;
            d.nf = 0;
        }
        double* del;
        if ((rc = dupload(e, &del, p.el.data(), p.el.size()))) return rc;
        d.el = del;
        if (!p.rho.empty()) {
            double* dr;
            if ((rc = dupload(e, &dr, p.rho.data(), p.rho.size()))) return rc;
            d.rho = dr;
        }
        float2* acc;
        if ((rc = dalloc(e, &acc, std::max<size_t>(1, (size_t)d.nf * 3 * d.npos), true, true))) return rc;
        d.acc = acc;
        e->dump_dev.push_back(d);
        block0.push_back(block0.back() + (d.npos + 255) / 256);
    }
    StepEndDev& s = e->stepend;
    s.nprobe = (int)e->probe_dev.size();
    s.ndump = (int)e->dump_dev.size();
    ProbeDev* dp = nullptr;
    DumpDev* dd = nullptr;
    unsigned* db0 = nullptr;
    if ((rc = dupload(e, &dp, e->probe_dev.data(), e->probe_dev.size()))) return rc;
    if ((rc = dupload(e, &dd, e->dump_dev.data(), e->dump_dev.size()))) return rc;
    if ((rc = dupload(e, &db0, block0.data(), block0.size()))) return rc;
    s.probes = dp; s.dumps = dd; s.dump_block0 = db0;
    s.numTS = e->d_numTS;
    s.blocks_done = e->d_blocks_done;
    e->stepend_blocks = block0.back();
    // the step end in two parts beside the updates (OEMS_CUDA_SE_SPLIT=0: one launch at the end):
    // only where nothing in the voltage update reads numTS (no TFSF or lumped RLC, Mur only in
    // the lane-parallel form, which reads a constant) and the time-domain dump pipeline is off
    {
        const char* ss = getenv("OEMS_CUDA_SE_SPLIT");
        const bool mur_ok = e->mur.empty() || (e->murdev.lanes && !e->mur_separate);
        e->se_split = mur_ok && !e->has_tfsf && e->rlc_host.off.empty() && !e->has_td && !(ss && ss[0] == '0');
        if (e->se_split) {
            CK(cudaStreamCreateWithFlags(&e->stream_se, cudaStreamNonBlocking));
            CK(cudaEventCreateWithFlags(&e->ev_se_fork, cudaEventDisableTiming));
            CK(cudaEventCreateWithFlags(&e->ev_se_a, cudaEventDisableTiming));
            CK(cudaEventCreateWithFlags(&e->ev_se_b, cudaEventDisableTiming));
        }
    }

    // energy scratch
    e->energy_blocks = 1024;
    if ((rc = dalloc(e, &e->d_energy_partial, 2 * (size_t)e->energy_blocks, true))) return rc;

    CK(cudaStreamSynchronize(e->stream));

    // probes at numTS = 0 (all fields zero): a step_end launch with numTS = -1 records slot 0
    {
        unsigned minus1 = 0xFFFFFFFFu;
        CK(cudaMemcpyAsync(e->d_numTS, &minus1, 4, cudaMemcpyHostToDevice, e->stream));
        k_step_end<<<e->stepend_blocks, 256, 0, e->stream>>>(e->grid, e->stepend);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(e->stream));
    }
    // The TMA-staged plane march (one kernel per step) applies where the engine is compressed,
    // has no hook but the soft sources and its z lines fit one TMA box.  OEMS_CUDA_MARCH=1 always
    // uses it, =0 never; otherwise both K-step graphs are captured and the first long iterate
    // times one of each and keeps the faster (both give the same bits).
    bool tune = false;
    {
        const char* env = getenv("OEMS_CUDA_MARCH");
        const bool force = env && env[0] == '1', never = env && env[0] == '0';
        const bool fits = e->compressed && e->grid.nupml == 0 && e->mur.empty() && e->lor.empty() && !e->has_tfsf &&
                          !e->rlc.count && !e->cyl_closed && e->Pz <= 256 && e->K % 2 == 0 &&
                          e->excV.count <= (unsigned)FT_MAX_SRC && e->excI.count <= (unsigned)FT_MAX_SRC;
        if (fits && (force || (!never && !e->has_td))) {
            if ((rc = setup_fused(e))) return rc;
            if ((rc = setup_march(e))) return rc;
            e->use_fused = e->use_march = force;
            tune = !force;
        }
    }
    if ((rc = capture(e, 1, &e->graph1, false))) return rc;
    if (tune) {
        if ((rc = capture(e, e->K, &e->graphK_alt, true))) return rc;       // the march
        e->march_tune = true;
    }
    if ((rc = capture(e, e->K, &e->graphK, e->use_fused))) return rc;
    e->inited = true;
    // time-domain dumps: start the writer and hand it the numTS = 0 samples
    if (e->has_td) {
        if ((rc = td_start_pipeline(e))) return rc;
        if ((rc = td_flush(e))) return rc;
    }
    return OEMS_OK;
}

int oems_cuda_iterate(oems_cuda_engine* e, unsigned int n)
{
    if (!e) return OEMS_ERR_ARG;
    if (!e->inited) return fail(e, OEMS_ERR_STATE, "engine not initialised");
    if ((unsigned long long)e->host_numTS + n > e->max_ts)
        return fail(e, OEMS_ERR_ARG, "iterating beyond max_timesteps given to oems_cuda_init");
    CK(cudaSetDevice(e->device));
    if (e->has_td) return td_iterate(e, n);
    unsigned done = 0;
    if (e->march_tune && n >= 4 * e->K) {
        // one warm-up launch of each, then one timed launch of each (real steps, same results)
        cudaEvent_t ev[3];
        for (auto& x : ev) CK(cudaEventCreate(&x));
        CK(cudaGraphLaunch(e->graphK_alt, e->stream));
        CK(cudaGraphLaunch(e->graphK, e->stream));
        CK(cudaEventRecord(ev[0], e->stream));
        CK(cudaGraphLaunch(e->graphK_alt, e->stream));
        CK(cudaEventRecord(ev[1], e->stream));
        CK(cudaGraphLaunch(e->graphK, e->stream));
        CK(cudaEventRecord(ev[2], e->stream));
        CK(cudaEventSynchronize(ev[2]));
        cudaEventElapsedTime(&e->march_tune_ms[0], ev[0], ev[1]);
        cudaEventElapsedTime(&e->march_tune_ms[1], ev[1], ev[2]);
        for (auto& x : ev) cudaEventDestroy(x);
        if (e->march_tune_ms[0] < e->march_tune_ms[1]) {
            std::swap(e->graphK, e->graphK_alt);
            e->use_fused = e->use_march = true;
        }
        e->march_tune = false;
        done = 4 * e->K;
    }
    while (n - done >= e->K) { CK(cudaGraphLaunch(e->graphK, e->stream)); done += e->K; }
    while (done < n) { CK(cudaGraphLaunch(e->graph1, e->stream)); ++done; }
    e->host_numTS += n;
    return OEMS_OK;
}

int oems_cuda_sync(oems_cuda_engine* e)
{
    if (!e) return OEMS_ERR_ARG;
    CK(cudaStreamSynchronize(e->stream));
    if (e->d_march_err) {                          // a plane-march block gave up on a copy
        unsigned err = 0;
        CK(cudaMemcpy(&err, e->d_march_err, sizeof(err), cudaMemcpyDeviceToHost));
        if (err) return fail(e, OEMS_ERR_DEVICE, "plane march: a TMA copy did not complete in time");
    }
    return OEMS_OK;
}

unsigned int oems_cuda_num_timesteps(const oems_cuda_engine* e)
{
    return e ? e->host_numTS : 0;
}

int oems_cuda_timed_iterate(oems_cuda_engine* e, unsigned int n, float* ms)
{
    if (!e || !ms) return OEMS_ERR_ARG;
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    CK(cudaEventRecord(a, e->stream));
    int rc = oems_cuda_iterate(e, n);
    CK(cudaEventRecord(b, e->stream));
    CK(cudaEventSynchronize(b));
    CK(cudaEventElapsedTime(ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return rc;
}

int oems_cuda_profile_steps(oems_cuda_engine* e, unsigned int n, float* ms, unsigned int* launches)
{
    if (!e) return OEMS_ERR_ARG;
    if (!e->inited) return fail(e, OEMS_ERR_STATE, "engine not initialised");
    if (e->has_td) return fail(e, OEMS_ERR_UNSUPPORTED, "profiled steps bypass the time-domain dump pipeline");
    if ((unsigned long long)e->host_numTS + n > e->max_ts)
        return fail(e, OEMS_ERR_ARG, "iterating beyond max_timesteps given to oems_cuda_init");
    CK(cudaSetDevice(e->device));
    float acc[OEMS_KC_COUNT] = {0};
    unsigned cnt[OEMS_KC_COUNT] = {0};
    StepProfiler prof;
    for (int i = 0; i < 128; ++i) CK(cudaEventCreate(&prof.ev[i]));
    int rc = OEMS_OK;
    for (unsigned st = 0; st < n && rc == OEMS_OK; ++st) {
        prof.n = 0;
        rc = enqueue_step(e, nullptr, &prof, (st == 0 ? 1u : 0u) | (st + 1 == n ? 2u : 0u));
        if (rc) break;
        ++e->host_numTS;
        cudaError_t c = cudaEventSynchronize(prof.ev[2 * prof.n - 1]);
        if (c != cudaSuccess) { rc = cuda_fail(e, c, "profile sync"); break; }
        for (int k = 0; k < prof.n; ++k) {
            float t = 0.f;
            cudaEventElapsedTime(&t, prof.ev[2 * k], prof.ev[2 * k + 1]);
            acc[prof.cls[k]] += t;
            ++cnt[prof.cls[k]];
        }
    }
    for (int i = 0; i < 128; ++i) cudaEventDestroy(prof.ev[i]);
    if (ms) for (int k = 0; k < OEMS_KC_COUNT; ++k) ms[k] = acc[k];
    if (launches) for (int k = 0; k < OEMS_KC_COUNT; ++k) launches[k] = cnt[k];
    return rc;
}

int oems_cuda_update_kernels(oems_cuda_engine* e, char* volt, char* curr, size_t cap)
{
    if (!e || !volt || !curr || !cap) return OEMS_ERR_ARG;
    if (!e->inited) return fail(e, OEMS_ERR_STATE, "engine not initialised");
    const char *v = "", *i = "";
    if (e->use_march) v = i = "k_step_march";
    else {
        launch_update(e, false, e->stream, &v);
        launch_update(e, true, e->stream, &i);
    }
    snprintf(volt, cap, "%s", v);
    snprintf(curr, cap, "%s", i);
    return OEMS_OK;
}

int oems_cuda_launches_per_step(const oems_cuda_engine* e, unsigned int* l)
{
    if (!e || !l) return OEMS_ERR_ARG;
    *l = e->use_fused ? e->fused_launches : e->launches;
    return OEMS_OK;
}

// ---------------------------------------------------------------------------------------------
// field access

int oems_cuda_read_field(oems_cuda_engine* e, int which, float* out)
{
    if (!e || !out || (which != OEMS_VOLT && which != OEMS_CURR)) return OEMS_ERR_ARG;
    CK(cudaSetDevice(e->device));
    const float* src = which == OEMS_VOLT ? e->dV : e->dI;
    CK(cudaMemcpy2DAsync(out, e->N[2] * sizeof(float), src, e->Pz * sizeof(float), e->N[2] * sizeof(float),
                         (size_t)3 * e->N[0] * e->N[1], cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    return OEMS_OK;
}

int oems_cuda_write_field(oems_cuda_engine* e, int which, const float* in)
{
    if (!e || !in || (which != OEMS_VOLT && which != OEMS_CURR)) return OEMS_ERR_ARG;
    CK(cudaSetDevice(e->device));
    float* dst = which == OEMS_VOLT ? e->dV : e->dI;
    CK(cudaMemcpy2DAsync(dst, e->Pz * sizeof(float), in, e->N[2] * sizeof(float), e->N[2] * sizeof(float),
                         (size_t)3 * e->N[0] * e->N[1], cudaMemcpyHostToDevice, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    return OEMS_OK;
}

int oems_cuda_get_value(oems_cuda_engine* e, int which, unsigned n, unsigned x, unsigned y, unsigned z, float* v)
{
    if (!e || !v || n > 2 || x >= e->N[0] || y >= e->N[1] || z >= e->N[2]) return OEMS_ERR_ARG;
    const float* src = (which == OEMS_VOLT ? e->dV : e->dI) + cell_off(e, n, x, y, z);
    CK(cudaMemcpyAsync(v, src, 4, cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    return OEMS_OK;
}

int oems_cuda_set_value(oems_cuda_engine* e, int which, unsigned n, unsigned x, unsigned y, unsigned z, float v)
{
    if (!e || n > 2 || x >= e->N[0] || y >= e->N[1] || z >= e->N[2]) return OEMS_ERR_ARG;
    float* dst = (which == OEMS_VOLT ? e->dV : e->dI) + cell_off(e, n, x, y, z);
    CK(cudaMemcpyAsync(dst, &v, 4, cudaMemcpyHostToDevice, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    return OEMS_OK;
}

int oems_cuda_read_probe(oems_cuda_engine* e, int id, double* out, size_t cap, size_t* count)
{
    if (!e || !out || !count || id < 0 || id >= (int)e->probe_dev.size()) return OEMS_ERR_ARG;
    if (!e->inited) return fail(e, OEMS_ERR_STATE, "engine not initialised");
    const ProbeDev& d = e->probe_dev[id];
    const size_t n = std::min<size_t>(cap, (size_t)d.nslots * d.ncomp);
    CK(cudaMemcpyAsync(out, d.series, n * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    *count = n;
    return OEMS_OK;
}

int oems_cuda_read_probe_range(oems_cuda_engine* e, int id, size_t first, size_t count, double* out)
{
    if (!e || (!out && count) || id < 0 || id >= (int)e->probe_dev.size()) return OEMS_ERR_ARG;
    if (!e->inited) return fail(e, OEMS_ERR_STATE, "engine not initialised");
    const ProbeDev& d = e->probe_dev[id];
    if (first + count > d.nslots) return fail(e, OEMS_ERR_ARG, "probe slot range out of bounds");
    if (!count) return OEMS_OK;
    if (count == 1 && e->latest_host) {
        // the newest sample: after the synchronisation the step-end kernel's copy in mapped
        // memory is current
        CK(cudaStreamSynchronize(e->stream));
        if (e->latest_slot_host[id] == first) {
            memcpy(out, e->latest_host + 3 * (size_t)id, d.ncomp * sizeof(double));
            return OEMS_OK;
        }
    }
    if (count > 64) {
        CK(cudaMemcpyAsync(out, d.series + first * d.ncomp, count * d.ncomp * sizeof(double),
                           cudaMemcpyDeviceToHost, e->stream));
        CK(cudaStreamSynchronize(e->stream));
        return OEMS_OK;
    }
    // short ranges (a processing loop reading each probe's newest samples): the first read after
    // a step fetches the same slot range of every probe into pinned memory with one
    // synchronisation; the other probes' reads of that range are served from it until the engine
    // steps again or is restored
    ProbeCache& c = e->pcache;
    const bool hit = c.valid && c.ts == e->host_numTS && c.gen == e->series_gen && c.first == first &&
                     c.count == count && c.off[id] != SIZE_MAX;
    if (!hit) {
        c.valid = false;
        c.off.assign(e->probe_dev.size(), SIZE_MAX);
        size_t need = 0;
        for (size_t j = 0; j < e->probe_dev.size(); ++j)
            if (first + count <= e->probe_dev[j].nslots) { c.off[j] = need; need += count * e->probe_dev[j].ncomp; }
        if (need > c.cap) {
            if (c.pin) cudaFreeHost(c.pin);
            c.pin = nullptr;
            c.cap = 0;
            CK(cudaMallocHost(&c.pin, need * sizeof(double)));
            c.cap = need;
        }
        for (size_t j = 0; j < e->probe_dev.size(); ++j)
            if (c.off[j] != SIZE_MAX) {
                const ProbeDev& q = e->probe_dev[j];
                CK(cudaMemcpyAsync(c.pin + c.off[j], q.series + first * q.ncomp, count * q.ncomp * sizeof(double),
                                   cudaMemcpyDeviceToHost, e->stream));
            }
        CK(cudaStreamSynchronize(e->stream));
        c.valid = true;
        c.ts = e->host_numTS;
        c.gen = e->series_gen;
        c.first = first;
        c.count = count;
    }
    memcpy(out, c.pin + c.off[id], count * d.ncomp * sizeof(double));
    return OEMS_OK;
}

int oems_cuda_read_probe_dft(oems_cuda_engine* e, int id, double* out)
{
    if (!e || !out || id < 0 || id >= (int)e->probe_dev.size()) return OEMS_ERR_ARG;
    if (!e->inited) return fail(e, OEMS_ERR_STATE, "engine not initialised");
    const ProbeDev& d = e->probe_dev[id];
    if (d.nf) {
        CK(cudaMemcpyAsync(out, d.dft, 2 * d.nf * d.ncomp * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
        CK(cudaStreamSynchronize(e->stream));
    }
    return OEMS_OK;
}

int oems_cuda_read_fd_dump(oems_cuda_engine* e, int id, float* out, size_t cap)
{
    if (!e || !out || id < 0 || id >= (int)e->dump_dev.size()) return OEMS_ERR_ARG;
    if (!e->inited) return fail(e, OEMS_ERR_STATE, "engine not initialised");
    const DumpDev& d = e->dump_dev[id];
    if (d.td) return fail(e, OEMS_ERR_ARG, "dump is a time-domain dump (written to files)");
    const size_t n = (size_t)d.nf * 3 * d.npos * 2;
    if (cap < n) return fail(e, OEMS_ERR_ARG, "output buffer too small");
    if (n) {
        CK(cudaMemcpyAsync(out, d.acc, n * sizeof(float), cudaMemcpyDeviceToHost, e->stream));
        CK(cudaStreamSynchronize(e->stream));
    }
    return OEMS_OK;
}

int oems_cuda_energy(oems_cuda_engine* e, double* out)
{
    if (!e || !out) return OEMS_ERR_ARG;
    if (!e->inited) return fail(e, OEMS_ERR_STATE, "engine not initialised");
    k_energy<<<e->energy_blocks, 256, 0, e->stream>>>(e->grid, e->d_energy_partial);
    CK(cudaGetLastError());
    std::vector<double> part(2 * (size_t)e->energy_blocks);
    CK(cudaMemcpyAsync(part.data(), e->d_energy_partial, part.size() * sizeof(double), cudaMemcpyDeviceToHost,
                       e->stream));
    CK(cudaStreamSynchronize(e->stream));
    double E = 0, H = 0;
    for (unsigned b = 0; b < e->energy_blocks; ++b) { E += part[2 * b]; H += part[2 * b + 1]; }
    *out = 8.85418781762e-12 * E + 1.256637062e-6 * H;
    return OEMS_OK;
}

int oems_cuda_snapshot_size(const oems_cuda_engine* e, size_t* bytes)
{
    if (!e || !bytes) return OEMS_ERR_ARG;
    size_t b = 0;
    for (const auto& r : e->state) b += r.second;
    *bytes = b + sizeof(unsigned);
    return OEMS_OK;
}

int oems_cuda_snapshot(oems_cuda_engine* e, void* host, size_t bytes)
{
    size_t need = 0;
    if (!e || !host || oems_cuda_snapshot_size(e, &need) || bytes < need) return OEMS_ERR_ARG;
    if (!e->inited) return fail(e, OEMS_ERR_STATE, "engine not initialised");
    char* p = static_cast<char*>(host);
    for (const auto& r : e->state) {
        CK(cudaMemcpyAsync(p, r.first, r.second, cudaMemcpyDeviceToHost, e->stream));
        p += r.second;
    }
    CK(cudaStreamSynchronize(e->stream));
    memcpy(p, &e->host_numTS, sizeof(unsigned));
    return OEMS_OK;
}

int oems_cuda_restore(oems_cuda_engine* e, const void* host, size_t bytes)
{
    size_t need = 0;
    if (!e || !host || oems_cuda_snapshot_size(e, &need) || bytes < need) return OEMS_ERR_ARG;
    if (!e->inited) return fail(e, OEMS_ERR_STATE, "engine not initialised");
    const char* p = static_cast<const char*>(host);
    for (const auto& r : e->state) {
        CK(cudaMemcpyAsync(r.first, p, r.second, cudaMemcpyHostToDevice, e->stream));
        p += r.second;
    }
    CK(cudaStreamSynchronize(e->stream));
    memcpy(&e->host_numTS, p, sizeof(unsigned));
    ++e->series_gen;                 // the probe series changed under an unchanged step count
    if (e->latest_slot_host)
        for (size_t j = 0; j < e->probe_dev.size(); ++j) e->latest_slot_host[j] = UINT_MAX;
    return OEMS_OK;
}

}  // extern "C"
