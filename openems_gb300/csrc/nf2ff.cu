// nf2ff.cu -- NF2FF far-field transform (nf2ff/nf2ff_calc.cpp) on the FD field dumps that the
// engine accumulates on the device, Cartesian meshes, no mirror planes.
//
// The reference reads the dumps back from HDF5 files and sums, per (theta, phi) and thread, over
// every face sample.  Here the samples never leave the device:
//   k_nf2ff_pack   : per face sample, Js = n x H and Ms = -n x E (eq. 8.15a/b,
//                    nf2ff_calc.cpp:66-76), the sample area and its position relative to the
//                    centre, plus the sample's radiated-power term (:409-418), block-summed in double;
//   k_nf2ff_angles : one thread per angle, the face samples of one chunk staged in shared memory;
//                    N_theta, N_phi, L_theta, L_phi (:104-150) accumulated in float over the chunk;
//   k_nf2ff_reduce : the chunk sums added in double in a fixed order (deterministic).
// The far fields E_theta, E_phi, P_rad and the directivity (:489-528) are formed on the host.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "engine_impl.h"

using namespace oems;

namespace {

constexpr int NF_ANG = 128;      // angles per block (one per thread)
constexpr int NF_STAGE = 128;    // face samples staged per round

struct FaceDev {
    const float2* E;             // dump accumulators of the selected frequency: [3][npos]
    const float2* H;
    unsigned npos, first;        // samples of this face; index of its first packed sample
    unsigned sz[3];
    int ny;                      // normal axis
    float nd;                    // outward normal sign
    const float* pos[3];         // sample coordinates minus the centre, per axis
    const float* len[3];         // sample edge lengths along the tangential axes (unused on ny)
};

struct Packed {
    float4* geo;                 // (x, y, z, area)
    float2* jm;                  // [6][n]: Js x,y,z then Ms x,y,z
    unsigned n;
};

// Js, Ms, geometry and the power term of every sample of one face
__global__ void k_nf2ff_pack(FaceDev f, Packed p, double* power_part)
{
    __shared__ double red[256];
    const unsigned q = blockIdx.x * blockDim.x + threadIdx.x;
    double pw = 0.0;
    if (q < f.npos) {
        const unsigned c = q % f.sz[2], b = (q / f.sz[2]) % f.sz[1], a = q / (f.sz[2] * f.sz[1]);
        const unsigned idx[3] = {a, b, c};
        const int nP = (f.ny + 1) % 3, nPP = (f.ny + 2) % 3;
        const float area = f.len[nP][idx[nP]] * f.len[nPP][idx[nPP]];
        float2 E[3], H[3];
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            E[m] = f.E[(size_t)m * f.npos + q];
            H[m] = f.H[(size_t)m * f.npos + q];
        }
        const float nd[3] = {f.ny == 0 ? f.nd : 0.f, f.ny == 1 ? f.nd : 0.f, f.ny == 2 ? f.nd : 0.f};
        // Js = n x H, Ms = -n x E (the reference's component formulas)
        float2 J[3], M[3];
        J[0] = make_float2(nd[1] * H[2].x - nd[2] * H[1].x, nd[1] * H[2].y - nd[2] * H[1].y);
        J[1] = make_float2(nd[2] * H[0].x - nd[0] * H[2].x, nd[2] * H[0].y - nd[0] * H[2].y);
        J[2] = make_float2(nd[0] * H[1].x - nd[1] * H[0].x, nd[0] * H[1].y - nd[1] * H[0].y);
        M[0] = make_float2(nd[2] * E[1].x - nd[1] * E[2].x, nd[2] * E[1].y - nd[1] * E[2].y);
        M[1] = make_float2(nd[0] * E[2].x - nd[2] * E[0].x, nd[0] * E[2].y - nd[2] * E[0].y);
        M[2] = make_float2(nd[1] * E[0].x - nd[0] * E[1].x, nd[1] * E[0].y - nd[0] * E[1].y);
        const unsigned o = f.first + q;
        p.geo[o] = make_float4(f.pos[0][a], f.pos[1][b], f.pos[2][c], area);
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            p.jm[(size_t)m * p.n + o] = J[m];
            p.jm[(size_t)(3 + m) * p.n + o] = M[m];
        }
        // Re(E_P conj(H_PP) - E_PP conj(H_P)) in double
        const double re = ((double)E[nP].x * H[nPP].x + (double)E[nP].y * H[nPP].y) -
                          ((double)E[nPP].x * H[nP].x + (double)E[nPP].y * H[nP].y);
        pw = 0.5 * (double)area * re * (double)f.nd;
    }
    red[threadIdx.x] = pw;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) power_part[blockIdx.x] = red[0];
}

struct AngleDev {
    const float* theta;
    const float* phi;
    unsigned ntheta, nphi;
    float k;
    unsigned chunk;              // samples per chunk (blockIdx.y)
    float4* part;                // [nchunk][nangle][2]: (Nt, Np), (Lt, Lp) as (re, im, re, im)
};

// radiation vectors of one chunk of samples for NF_ANG angles
__global__ void __launch_bounds__(NF_ANG) k_nf2ff_angles(Packed p, AngleDev a)
{
    __shared__ float4 sg[NF_STAGE];
    __shared__ float2 sjm[6][NF_STAGE];
    const unsigned nang = a.ntheta * a.nphi;
    const unsigned ang = blockIdx.x * NF_ANG + threadIdx.x;
    const unsigned c0 = blockIdx.y * a.chunk, c1 = min(p.n, c0 + a.chunk);
    float sT = 0.f, cT = 0.f, sP = 0.f, cP = 0.f;
    if (ang < nang) {
        const float th = a.theta[ang / a.nphi], ph = a.phi[ang % a.nphi];
        sincosf(th, &sT, &cT);
        sincosf(ph, &sP, &cP);
    }
    const float cTcP = cT * cP, cTsP = cT * sP, cPsT = cP * sT, sTsP = sP * sT;
    float2 nt = make_float2(0.f, 0.f), np = nt, lt = nt, lp = nt;
    for (unsigned base = c0; base < c1; base += NF_STAGE) {
        const unsigned cnt = min((unsigned)NF_STAGE, c1 - base);
        __syncthreads();
        for (unsigned s = threadIdx.x; s < cnt; s += NF_ANG) {
            sg[s] = p.geo[base + s];
#pragma unroll
            for (int m = 0; m < 6; ++m) sjm[m][s] = p.jm[(size_t)m * p.n + base + s];
        }
        __syncthreads();
        if (ang < nang) {
            for (unsigned s = 0; s < cnt; ++s) {
                const float4 g = sg[s];
                const float r_cos_psi = g.x * cPsT + g.y * sTsP + g.z * cT;
                float si, co;
                sincosf(a.k * r_cos_psi, &si, &co);
                const float2 w = make_float2(g.w * co, g.w * si);          // area * exp(j k r.r_hat)
                const float2 J0 = sjm[0][s], J1 = sjm[1][s], J2 = sjm[2][s];
                const float2 M0 = sjm[3][s], M1 = sjm[4][s], M2 = sjm[5][s];
                const float2 jt = make_float2(J0.x * cTcP + J1.x * cTsP - J2.x * sT, J0.y * cTcP + J1.y * cTsP - J2.y * sT);
                const float2 jp = make_float2(J1.x * cP - J0.x * sP, J1.y * cP - J0.y * sP);
                const float2 mt = make_float2(M0.x * cTcP + M1.x * cTsP - M2.x * sT, M0.y * cTcP + M1.y * cTsP - M2.y * sT);
                const float2 mp = make_float2(M1.x * cP - M0.x * sP, M1.y * cP - M0.y * sP);
                nt.x += w.x * jt.x - w.y * jt.y; nt.y += w.x * jt.y + w.y * jt.x;
                np.x += w.x * jp.x - w.y * jp.y; np.y += w.x * jp.y + w.y * jp.x;
                lt.x += w.x * mt.x - w.y * mt.y; lt.y += w.x * mt.y + w.y * mt.x;
                lp.x += w.x * mp.x - w.y * mp.y; lp.y += w.x * mp.y + w.y * mp.x;
            }
        }
    }
    if (ang < nang) {
        float4* o = a.part + ((size_t)blockIdx.y * nang + ang) * 2;
        o[0] = make_float4(nt.x, nt.y, np.x, np.y);
        o[1] = make_float4(lt.x, lt.y, lp.x, lp.y);
    }
}

// out[ang][8] (double) = sum over the chunks, in chunk order
__global__ void k_nf2ff_reduce(const float4* __restrict__ part, unsigned nchunk, unsigned nang, double* out)
{
    const unsigned ang = blockIdx.x * blockDim.x + threadIdx.x;
    if (ang >= nang) return;
    double s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (unsigned c = 0; c < nchunk; ++c) {
        const float4 a = part[((size_t)c * nang + ang) * 2], b = part[((size_t)c * nang + ang) * 2 + 1];
        s[0] += a.x; s[1] += a.y; s[2] += a.z; s[3] += a.w;
        s[4] += b.x; s[5] += b.y; s[6] += b.z; s[7] += b.w;
    }
#pragma unroll
    for (int m = 0; m < 8; ++m) out[(size_t)ang * 8 + m] = s[m];
}

}  // namespace

extern "C" {

int oems_cuda_nf2ff(oems_cuda_engine* e, unsigned int nface, const int* e_dumps, const int* h_dumps,
                    const double* coords, unsigned int freq_index, double freq, unsigned int ntheta,
                    const double* theta, unsigned int nphi, const double* phi, const double center[3], double radius,
                    double eps_r, double mu_r, double* e_theta, double* e_phi, double* p_rad, double* rad_power,
                    double* max_dir)
{
    if (!e || !e_dumps || !h_dumps || !coords || !theta || !phi || !center || !e_theta || !e_phi || !p_rad ||
        nface == 0 || ntheta == 0 || nphi == 0 || !(radius > 0))
        return OEMS_ERR_ARG;
    if (!e->inited) { e->err = "engine not initialised"; return OEMS_ERR_STATE; }
    if (cudaSetDevice(e->device) != cudaSuccess) { cudaGetLastError(); e->err = "cudaSetDevice"; return OEMS_ERR_CUDA; }
    const float fc[3] = {(float)center[0], (float)center[1], (float)center[2]};
    // faces: validate and build their float tables (the reference keeps lines in float)
    std::vector<FaceDev> faces(nface);
    std::vector<std::vector<float>> tabs;                // per face: pos x,y,z then len x,y,z
    size_t off = 0;
    unsigned total = 0;
    for (unsigned f = 0; f < nface; ++f) {
        const int ie = e_dumps[f], ih = h_dumps[f];
        if (ie < 0 || ih < 0 || ie >= (int)e->dump_dev.size() || ih >= (int)e->dump_dev.size()) {
            e->err = "nf2ff: bad dump id"; return OEMS_ERR_ARG;
        }
        const DumpDev& de = e->dump_dev[ie];
        const DumpDev& dh = e->dump_dev[ih];
        if (de.field != 0 || dh.field != 1 || freq_index >= de.nf || freq_index >= dh.nf ||
            de.sz[0] != dh.sz[0] || de.sz[1] != dh.sz[1] || de.sz[2] != dh.sz[2]) {
            e->err = "nf2ff: each face needs an E and an H dump of the same box containing the frequency";
            return OEMS_ERR_ARG;
        }
        int ny = -1;
        for (int a = 0; a < 3; ++a)
            if (de.sz[a] == 1 && de.sz[(a + 1) % 3] > 2 && de.sz[(a + 2) % 3] > 2) ny = a;
        if (ny < 0) { e->err = "nf2ff: a face must be planar with more than two lines per tangential axis"; return OEMS_ERR_ARG; }
        FaceDev& fd = faces[f];
        fd.E = de.acc + (size_t)freq_index * 3 * de.npos;
        fd.H = dh.acc + (size_t)freq_index * 3 * dh.npos;
        fd.npos = de.npos;
        fd.first = total;
        total += de.npos;
        for (int a = 0; a < 3; ++a) fd.sz[a] = de.sz[a];
        fd.ny = ny;
        std::vector<float> t;
        std::vector<float> lines[3];
        for (int a = 0; a < 3; ++a) {
            for (unsigned i = 0; i < de.sz[a]; ++i) lines[a].push_back((float)coords[off + i]);
            off += de.sz[a];
        }
        fd.nd = lines[ny][0] >= fc[ny] ? 1.f : -1.f;    // nf2ff_calc.cpp:329-336
        for (int a = 0; a < 3; ++a)
            for (float l : lines[a]) t.push_back(l - fc[a]);
        for (int a = 0; a < 3; ++a) {                     // edge lengths, nf2ff_calc.cpp:338-353
            const std::vector<float>& L = lines[a];
            const size_t n = L.size();
            for (size_t i = 0; i < n; ++i) {
                float v = 0.f;
                if (n > 1) {
                    if (i == 0) v = 0.5f * std::fabs(L[1] - L[0]);
                    else if (i == n - 1) v = 0.5f * std::fabs(L[n - 1] - L[n - 2]);
                    else v = 0.5f * std::fabs(L[i + 1] - L[i - 1]);
                }
                t.push_back(v);
            }
        }
        tabs.push_back(std::move(t));
    }
    const unsigned nang = ntheta * nphi;
    std::vector<float> th(ntheta), ph(nphi);
    for (unsigned i = 0; i < ntheta; ++i) th[i] = (float)theta[i];
    for (unsigned i = 0; i < nphi; ++i) ph[i] = (float)phi[i];
    const float k = (float)(2.0 * kPI * (double)(float)freq / 299792458.0 * std::sqrt(eps_r * mu_r));
    // device work
    std::vector<void*> mem;
    auto dmalloc = [&](size_t bytes) -> void* {
        void* q = nullptr;
        if (cudaMalloc(&q, std::max<size_t>(bytes, 16)) != cudaSuccess) return nullptr;
        mem.push_back(q);
        return q;
    };
    auto release = [&]() { for (void* q : mem) cudaFree(q); mem.clear(); };
    cudaStream_t st = e->stream;
    Packed pk;
    pk.n = total;
    pk.geo = (float4*)dmalloc((size_t)total * sizeof(float4));
    pk.jm = (float2*)dmalloc((size_t)total * 6 * sizeof(float2));
    const unsigned angle_tiles = (nang + NF_ANG - 1) / NF_ANG;
    // enough chunks for about four blocks per SM of a 152-SM GPU
    unsigned nchunk = std::max(1u, std::min((608 + angle_tiles - 1) / angle_tiles, (total + 255) / 256));
    const unsigned chunk = (total + nchunk - 1) / nchunk;
    nchunk = (total + chunk - 1) / chunk;
    float4* part = (float4*)dmalloc((size_t)nchunk * nang * 2 * sizeof(float4));
    double* sums = (double*)dmalloc((size_t)nang * 8 * sizeof(double));
    float* dth = (float*)dmalloc(ntheta * sizeof(float));
    float* dph = (float*)dmalloc(nphi * sizeof(float));
    unsigned pblocks = 0;
    for (const FaceDev& fd : faces) pblocks += (fd.npos + 255) / 256;
    double* pwp = (double*)dmalloc((size_t)pblocks * sizeof(double));
    std::vector<float*> dtabs;
    for (const auto& t : tabs) dtabs.push_back((float*)dmalloc(t.size() * sizeof(float)));
    for (void* q : mem)
        if (!q) { release(); e->err = "nf2ff: device allocation failed"; return OEMS_ERR_NOMEM; }
    if (mem.size() != 7 + tabs.size()) { release(); e->err = "nf2ff: device allocation failed"; return OEMS_ERR_NOMEM; }
    cudaMemcpyAsync(dth, th.data(), ntheta * sizeof(float), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dph, ph.data(), nphi * sizeof(float), cudaMemcpyHostToDevice, st);
    unsigned pb = 0;
    for (unsigned f = 0; f < nface; ++f) {
        FaceDev& fd = faces[f];
        cudaMemcpyAsync(dtabs[f], tabs[f].data(), tabs[f].size() * sizeof(float), cudaMemcpyHostToDevice, st);
        const float* base = dtabs[f];
        fd.pos[0] = base;
        fd.pos[1] = fd.pos[0] + fd.sz[0];
        fd.pos[2] = fd.pos[1] + fd.sz[1];
        fd.len[0] = fd.pos[2] + fd.sz[2];
        fd.len[1] = fd.len[0] + fd.sz[0];
        fd.len[2] = fd.len[1] + fd.sz[1];
        const unsigned nb = (fd.npos + 255) / 256;
        k_nf2ff_pack<<<nb, 256, 0, st>>>(fd, pk, pwp + pb);
        pb += nb;
    }
    AngleDev ad{dth, dph, ntheta, nphi, k, chunk, part};
    k_nf2ff_angles<<<dim3(angle_tiles, nchunk), NF_ANG, 0, st>>>(pk, ad);
    k_nf2ff_reduce<<<(nang + 255) / 256, 256, 0, st>>>(part, nchunk, nang, sums);
    std::vector<double> hs((size_t)nang * 8), hp(pblocks);
    cudaMemcpyAsync(hs.data(), sums, hs.size() * sizeof(double), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(hp.data(), pwp, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, st);
    const cudaError_t c = cudaStreamSynchronize(st);
    release();
    if (c != cudaSuccess || cudaGetLastError() != cudaSuccess) { e->err = "nf2ff: kernel failure"; return OEMS_ERR_CUDA; }
    double prad = 0.0;
    for (double v : hp) prad += v;
    // far fields, nf2ff_calc.cpp:489-528
    const double z0 = 376.730313461 * std::sqrt(mu_r / eps_r);
    const double kr = (double)k * radius;
    const double fr = (double)k / (4.0 * kPI * radius);                 // factor = j fr e^{-j k r}
    const double fre = -fr * std::sin(-kr), fim = fr * std::cos(-kr);
    double pmax = 0.0;
    for (unsigned i = 0; i < nang; ++i) {
        const double* s = &hs[(size_t)i * 8];
        const double ntr = s[0], nti = s[1], npr = s[2], npi = s[3], ltr = s[4], lti = s[5], lpr = s[6], lpi = s[7];
        const double ar = lpr + z0 * ntr, ai = lpi + z0 * nti;          // E_theta = -factor (Lp + Z0 Nt)
        const double br = ltr - z0 * npr, bi = lti - z0 * npi;          // E_phi = factor (Lt - Z0 Np)
        const double etr = -(fre * ar - fim * ai), eti = -(fre * ai + fim * ar);
        const double epr = fre * br - fim * bi, epi = fre * bi + fim * br;
        e_theta[2 * i] = etr; e_theta[2 * i + 1] = eti;
        e_phi[2 * i] = epr; e_phi[2 * i + 1] = epi;
        p_rad[i] = (etr * etr + eti * eti + epr * epr + epi * epi) / (2.0 * z0);
        pmax = std::max(pmax, p_rad[i]);
    }
    if (rad_power) *rad_power = prad;
    if (max_dir) *max_dir = prad != 0.0 ? pmax * 4.0 * kPI * radius * radius / prad : 0.0;
    return OEMS_OK;
}

}  // extern "C"
