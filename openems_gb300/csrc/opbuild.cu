// opbuild.cu -- the operator's per-edge numerics on the device, for geometries given as a
// painted list of material boxes:
//   k_ec      : quarter-cell averaged material (Operator::AverageMatQuarterCell,
//               FDTD/operator.cpp:1447-1564) and the equivalent circuit C, G, L, R of every
//               edge (Operator::Calc_ECPos, :1189-1254);
//   k_var3    : the Rennings timestep criterion per node (Operator::CalcTimestep_Var3,
//               :1956-2030), reduced to its minimum;
//   k_coef    : vv, vi, ii, iv from C, G, L, R and dt (Operator::Calc_ECOperatorPos, :956-984).
// The arithmetic is the host restatement's (openems_gb300/operator.py) in double precision with
// every multiply, add and divide rounded separately (no contraction), so the results are
// bit-identical to it.  Boundary conditions, metal, lumped elements and the extensions stay with
// the host operator, which edits a handful of edges.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <new>
#include <string>
#include <vector>

#include "../../include/oems_cuda.h"

namespace {

constexpr double kEPS0 = 8.85418781762e-12;   // tools/constants.h:23
constexpr double kMUE0 = 1.256637062e-6;      // tools/constants.h:24

__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dd(double a, double b) { return __ddiv_rn(a, b); }

struct Mesh {
    unsigned N[3];
    const double* L[3];          // lines (drawing units)
    double unit;
    unsigned nrec;
    const double* lo;            // [nrec][3] paint records in painting order: the last containing wins
    const double* hi;
    const double* par;           // [nrec][4] eps_r, kappa, mu_r, sigma
    double bg[4];
    // record masks: bit r of mask[((ax * 3 + kind) * Nmax + i) * W + r / 64] is set when the
    // sample coordinate of kind `kind` at index i of axis ax lies in record r's [lo, hi] along ax
    // (the same double compares as a direct test); kinds: SAMPLE_HALF, SAMPLE_QUP, SAMPLE_QDN
    const unsigned long long* mask;
    unsigned W, Nmax;
};

enum { SAMPLE_HALF = 0, SAMPLE_QUP = 1, SAMPLE_QDN = 2 };

// GetRawDiscDelta (FDTD/operator.cpp:1256-1266) for index i (may be -1 or >= N-1)
__device__ __forceinline__ double raw_delta(const double* L, unsigned N, int i)
{
    if (i < 0) return ds(L[0], L[1]);
    if (i >= (int)N - 1) return ds(L[N - 2], L[N - 1]);
    return ds(L[i + 1], L[i]);
}
// GetDiscDelta(n, pos, false): main delta, the last repeating the previous
__device__ __forceinline__ double main_delta(const double* L, unsigned N, int i)
{
    return i < (int)N - 1 ? ds(L[i + 1], L[i]) : ds(L[N - 1], L[N - 2]);
}
// GetDiscLine(n, pos, true)
__device__ __forceinline__ double dual_line(const double* L, unsigned N, int i)
{
    return i < (int)N - 1 ? dm(0.5, da(L[i], L[i + 1])) : da(L[N - 1], dm(0.5, ds(L[N - 1], L[N - 2])));
}
// GetDiscDelta(n, pos, true)
__device__ __forceinline__ double dual_delta(const double* L, unsigned N, int i)
{
    return i == 0 ? ds(L[1], L[0]) : ds(dual_line(L, N, i), dual_line(L, N, i - 1));
}

// the sample coordinates of the quarter-cell averaging (FDTD/operator.cpp:1447-1564 as
// restated): half a cell up, a quarter up, a quarter down from line i
__device__ __forceinline__ double sample_coord(const double* L, unsigned N, int i, int kind)
{
    if (kind == SAMPLE_HALF) return da(L[i], dm(raw_delta(L, N, i), 0.5));
    if (kind == SAMPLE_QUP) return da(L[i], dm(raw_delta(L, N, i), 0.25));
    return ds(L[i], dm(raw_delta(L, N, i - 1), 0.25));
}

// one thread per (axis, kind, index, mask word)
__global__ void k_masks(Mesh m, unsigned long long* mask)
{
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned w = t % m.W, rest = t / m.W;
    const unsigned i = rest % m.Nmax, ak = rest / m.Nmax;
    if (ak >= 9) return;
    const int ax = (int)(ak / 3), kind = (int)(ak % 3);
    unsigned long long bits = 0ull;
    if (i < m.N[ax]) {
        const double c = sample_coord(m.L[ax], m.N[ax], (int)i, kind);
        for (unsigned b = 0; b < 64; ++b) {
            const unsigned r = w * 64 + b;
            if (r >= m.nrec) break;
            if (c >= m.lo[3 * r + ax] && c <= m.hi[3 * r + ax]) bits |= 1ull << b;
        }
    }
    mask[t] = bits;
}

// the material parameters at a sample point given by its per-axis (index, kind): the last paint
// record containing it, else the background
__device__ __forceinline__ const double* lookup(const Mesh& m, const unsigned idx[3], const int kind[3])
{
    const unsigned long long* p0 = m.mask + ((size_t)(0 * 3 + kind[0]) * m.Nmax + idx[0]) * m.W;
    const unsigned long long* p1 = m.mask + ((size_t)(1 * 3 + kind[1]) * m.Nmax + idx[1]) * m.W;
    const unsigned long long* p2 = m.mask + ((size_t)(2 * 3 + kind[2]) * m.Nmax + idx[2]) * m.W;
    for (int w = (int)m.W - 1; w >= 0; --w) {
        const unsigned long long b = __ldg(p0 + w) & __ldg(p1 + w) & __ldg(p2 + w);
        if (b) return m.par + 4 * (64 * w + 63 - __clzll((long long)b));
    }
    return m.bg;
}

struct ECOut {
    float* C;                    // [3][N] each, x,y,z order, z fastest
    float* G;
    float* L;
    float* R;
    int* bad;                    // set when an effective parameter is not finite
};

// one thread per node, direction n
__global__ void k_ec(Mesh m, int n, ECOut o)
{
    const unsigned long long cells = (unsigned long long)m.N[0] * m.N[1] * m.N[2];
    const unsigned long long t = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cells) return;
    const unsigned iz = (unsigned)(t % m.N[2]), iy = (unsigned)((t / m.N[2]) % m.N[1]), ix = (unsigned)(t / ((unsigned long long)m.N[2] * m.N[1]));
    const unsigned idx[3] = {ix, iy, iz};
    const int a = n, p = (n + 1) % 3, pp = (n + 2) % 3;
    const double* L = m.L[a];
    const double* Lp = m.L[p];
    const double* Lpp = m.L[pp];
    const unsigned N = m.N[a], Np = m.N[p], Npp = m.N[pp];
    const int i = (int)idx[a], j = (int)idx[p], k = (int)idx[pp];
    const double u = m.unit;
    auto wmain = [&](int ax, int q) -> double { return q >= 0 ? dm(main_delta(m.L[ax], m.N[ax], q), u) : 0.0; };
    // the four quarter-cell samples: half a cell up along n, a quarter up / down across
    // (sample_coord; the records containing each come from the per-axis masks)
    const double Wp = wmain(p, j), WpM = wmain(p, j - 1), Wpp = wmain(pp, k), WppM = wmain(pp, k - 1);
    const int kp[4] = {SAMPLE_QUP, SAMPLE_QDN, SAMPLE_QUP, SAMPLE_QDN};
    const int kpp[4] = {SAMPLE_QUP, SAMPLE_QUP, SAMPLE_QDN, SAMPLE_QDN};
    const double swa[4] = {Wp, WpM, Wp, WpM}, swb[4] = {Wpp, Wpp, WppM, WppM};
    double eps_acc = 0.0, kap_acc = 0.0, area = 0.0;
    for (int q = 0; q < 4; ++q) {
        int k3[3];
        k3[a] = SAMPLE_HALF;
        k3[p] = kp[q];
        k3[pp] = kpp[q];
        const double* par = lookup(m, idx, k3);
        const double A = dm(swa[q], swb[q]);
        if (q == 0) {
            eps_acc = dm(par[0], A);
            kap_acc = dm(par[1], A);
            area = A;
        } else {
            eps_acc = da(eps_acc, dm(par[0], A));
            kap_acc = da(kap_acc, dm(par[1], A));
            area = da(area, A);
        }
    }
    const double e0 = dm(eps_acc, dd(kEPS0, area));
    const double e1 = dd(kap_acc, area);
    // mu and sigma: two samples along n at the cell centres across
    const double Ddn = wmain(a, i - 1), Dup = wmain(a, i);
    int k3[3];
    k3[a] = SAMPLE_QDN;
    k3[p] = SAMPLE_HALF;
    k3[pp] = SAMPLE_HALF;
    const double* pdn = lookup(m, idx, k3);
    k3[a] = SAMPLE_QUP;
    const double* pup = lookup(m, idx, k3);
    double e2 = dd(Ddn, pdn[2]);
    double e3 = pdn[3] != 0.0 ? dd(Ddn, pdn[3]) : 0.0;
    double length = Ddn;
    e2 = da(e2, dd(Dup, pup[2]));
    e3 = pup[3] != 0.0 ? da(e3, dd(Dup, pup[3])) : 0.0;
    length = da(length, Dup);
    e2 = dd(dm(length, kMUE0), e2);
    e3 = e3 != 0.0 ? dd(length, e3) : e3;
    if (!isfinite(e0) || !isfinite(e1) || !isfinite(e2) || !isfinite(e3)) atomicExch(o.bad, 1);
    // Calc_ECPos
    const double Dn = dm(main_delta(L, N, i), u);
    const double area_e = dm(dm(dual_delta(Lp, Np, j), u), dm(dual_delta(Lpp, Npp, k), u));
    const double Dh = dm(dual_delta(L, N, i), u);
    const double area_h = dm(dm(main_delta(Lp, Np, j), u), dm(main_delta(Lpp, Npp, k), u));
    const unsigned long long out = (unsigned long long)n * cells + t;
    o.C[out] = (float)(Dn != 0.0 ? dd(dm(e0, area_e), Dn) : 0.0);
    o.G[out] = (float)(Dn != 0.0 ? dd(dm(e1, area_e), Dn) : 0.0);
    o.L[out] = (float)(Dh != 0.0 ? dd(dm(e2, area_h), Dh) : 0.0);
    o.R[out] = (float)(Dh != 0.0 ? dd(dm(e3, area_h), Dh) : 0.0);
}

// np.minimum: NaN if either operand is NaN
__device__ __forceinline__ double nmin(double a, double b) { return (isnan(a) || isnan(b)) ? nan("") : (a < b ? a : b); }

struct Var3In {
    unsigned N[3];
    const float* C;              // [3][N]
    const float* L;
    double* part;                // per block: the minimum of the finite positive node timesteps
};

// Rennings criterion per node and direction (the host restatement of CalcTimestep_Var3): shifts
// clamp at the mesh ends (AdrOp reflection), terms are added in the restatement's order
__global__ void k_var3(Var3In v)
{
    __shared__ double red[256];
    const unsigned long long cells = (unsigned long long)v.N[0] * v.N[1] * v.N[2];
    const unsigned long long t = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    double best = 1e200;
    if (t < cells) {
        const int pos[3] = {(int)(t / ((unsigned long long)v.N[2] * v.N[1])), (int)((t / v.N[2]) % v.N[1]), (int)(t % v.N[2])};
        auto at = [&](const float* F, int comp, int s0, int s1, int s2) -> double {
            int q[3] = {pos[0] + s0, pos[1] + s1, pos[2] + s2};
            for (int d = 0; d < 3; ++d) q[d] = min(max(q[d], 0), (int)v.N[d] - 1);
            return (double)F[(unsigned long long)comp * cells + ((unsigned long long)q[0] * v.N[1] + q[1]) * v.N[2] + q[2]];
        };
        for (int n = 0; n < 3; ++n) {
            const int a = n, p = (n + 1) % 3, pp = (n + 2) % 3;
            int ep[3] = {0, 0, 0}, epp[3] = {0, 0, 0}, ea[3] = {0, 0, 0};
            ep[p] = 1; epp[pp] = 1; ea[a] = 1;
            const double Lpp = at(v.L, pp, 0, 0, 0), Lp = at(v.L, p, 0, 0, 0);
            const double Cn = at(v.C, n, 0, 0, 0);
            const double Cn_p = at(v.C, n, ep[0], ep[1], ep[2]);
            const double Cn_pp = at(v.C, n, epp[0], epp[1], epp[2]);
            const double Cn_mp = at(v.C, n, -ep[0], -ep[1], -ep[2]);
            const double Cn_mpmpp = at(v.C, n, -ep[0] - epp[0], -ep[1] - epp[1], -ep[2] - epp[2]);
            const double Lpp_m = at(v.L, pp, -ep[0], -ep[1], -ep[2]);
            const double Lp_mm = at(v.L, p, -ep[0] - epp[0], -ep[1] - epp[1], -ep[2] - epp[2]);
            const double Lp_ppm = at(v.L, p, -epp[0], -epp[1], -epp[2]);
            double wqp = da(dd(1.0, dm(Lpp, Cn_p)), dd(1.0, dm(Lpp, Cn)));
            wqp = da(wqp, da(dd(1.0, dm(Lp, Cn_pp)), dd(1.0, dm(Lp, Cn))));
            wqp = da(wqp, da(dd(1.0, dm(Lpp_m, Cn)), dd(1.0, dm(Lpp_m, Cn_mp))));
            wqp = da(wqp, da(dd(1.0, dm(Lp_mm, Cn_mp)), dd(1.0, dm(Lp_mm, Cn_mpmpp))));
            auto wt = [&](double Cp, double Cpp) {
                const double w0 = dd(1.0, dm(Lpp, Cp)), w1 = dd(1.0, dm(Lpp_m, Cp));
                const double w2 = dd(1.0, dm(Lp, Cpp)), w3 = dd(1.0, dm(Lp_ppm, Cpp));
                return ds(da(da(da(w0, w1), w2), w3), dm(2.0, nmin(nmin(w0, w1), nmin(w2, w3))));
            };
            const double wt1 = wt(at(v.C, p, 0, 0, 0), at(v.C, pp, 0, 0, 0));
            const double wt2 = wt(at(v.C, p, ea[0], ea[1], ea[2]), at(v.C, pp, ea[0], ea[1], ea[2]));
            const double newT = dd(2.0, __dsqrt_rn(da(da(wqp, wt1), wt2)));
            if (isfinite(newT) && newT > 0.0 && newT < best) best = newT;
        }
    }
    red[threadIdx.x] = best;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) red[threadIdx.x] = fmin(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) v.part[blockIdx.x] = red[0];
}

// Calc_ECOperatorPos: vv, vi from C, G and ii, iv from L, R (0 where C or L is not positive)
__global__ void k_coef(unsigned long long n, const float* C, const float* G, const float* L, const float* R, double dT,
                       float* vv, float* vi, float* ii, float* iv)
{
    const unsigned long long t = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const double c = C[t], g = G[t], l = L[t], r = R[t];
    if (c > 0.0) {
        const double x = dd(dd(dm(dT, g), 2.0), c);
        vv[t] = (float)dd(ds(1.0, x), da(1.0, x));
        vi[t] = (float)dd(dd(dT, c), da(1.0, x));
    } else {
        vv[t] = 0.f;
        vi[t] = 0.f;
    }
    if (l > 0.0) {
        const double y = dd(dd(dm(dT, r), 2.0), l);
        ii[t] = (float)dd(ds(1.0, y), da(1.0, y));
        iv[t] = (float)dd(dd(dT, l), da(1.0, y));
    } else {
        ii[t] = 0.f;
        iv[t] = 0.f;
    }
}

}  // namespace

struct oems_cuda_opbuild {
    Mesh m{};
    std::vector<void*> mem;
    float* ec[4] = {nullptr, nullptr, nullptr, nullptr};
    int* bad = nullptr;
    bool ec_done = false;
    std::string err;
};

namespace {

int ob_fail(oems_cuda_opbuild* b, int code, const char* msg)
{
    cudaGetLastError();
    b->err = msg;
    return code;
}

template <typename T>
T* ob_alloc(oems_cuda_opbuild* b, size_t count)
{
    void* q = nullptr;
    if (cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T)) != cudaSuccess) return nullptr;
    b->mem.push_back(q);
    return static_cast<T*>(q);
}

}  // namespace

extern "C" {

int oems_cuda_opbuild_create(const unsigned int num_lines[3], const double* lines, double unit, unsigned int nrec,
                             const double* rec_lo, const double* rec_hi, const double* rec_par,
                             const double background[4], oems_cuda_opbuild** out)
{
    if (!num_lines || !lines || !background || !out || (nrec && (!rec_lo || !rec_hi || !rec_par)) || !(unit > 0))
        return OEMS_ERR_ARG;
    for (int a = 0; a < 3; ++a)
        if (num_lines[a] < 3) return OEMS_ERR_ARG;
    auto* b = new (std::nothrow) oems_cuda_opbuild();
    if (!b) return OEMS_ERR_NOMEM;
    *out = b;
    Mesh& m = b->m;
    m.unit = unit;
    m.nrec = nrec;
    for (int k = 0; k < 4; ++k) m.bg[k] = background[k];
    size_t off = 0;
    for (int a = 0; a < 3; ++a) {
        m.N[a] = num_lines[a];
        double* d = ob_alloc<double>(b, num_lines[a]);
        if (!d || cudaMemcpy(d, lines + off, num_lines[a] * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
            return ob_fail(b, OEMS_ERR_NOMEM, "opbuild: mesh upload");
        m.L[a] = d;
        off += num_lines[a];
    }
    double* lo = ob_alloc<double>(b, 3 * (size_t)nrec);
    double* hi = ob_alloc<double>(b, 3 * (size_t)nrec);
    double* par = ob_alloc<double>(b, 4 * (size_t)nrec);
    b->bad = ob_alloc<int>(b, 1);
    if (!lo || !hi || !par || !b->bad) return ob_fail(b, OEMS_ERR_NOMEM, "opbuild: allocation");
    if (nrec && (cudaMemcpy(lo, rec_lo, 3 * nrec * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
                 cudaMemcpy(hi, rec_hi, 3 * nrec * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
                 cudaMemcpy(par, rec_par, 4 * nrec * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess))
        return ob_fail(b, OEMS_ERR_CUDA, "opbuild: record upload");
    m.lo = lo;
    m.hi = hi;
    m.par = par;
    // the per-axis record masks of the sample coordinates
    m.W = std::max(1u, (nrec + 63) / 64);
    m.Nmax = std::max(num_lines[0], std::max(num_lines[1], num_lines[2]));
    const size_t nmask = 9ull * m.Nmax * m.W;
    unsigned long long* mk = ob_alloc<unsigned long long>(b, nmask);
    if (!mk) return ob_fail(b, OEMS_ERR_NOMEM, "opbuild: allocation");
    k_masks<<<(unsigned)((nmask + 255) / 256), 256>>>(m, mk);
    if (cudaGetLastError() != cudaSuccess) return ob_fail(b, OEMS_ERR_CUDA, "opbuild: mask kernel");
    m.mask = mk;
    return OEMS_OK;
}

int oems_cuda_opbuild_ec(oems_cuda_opbuild* b, float* C, float* G, float* L, float* R, double* dt_var3)
{
    if (!b) return OEMS_ERR_ARG;
    const Mesh& m = b->m;
    const unsigned long long cells = (unsigned long long)m.N[0] * m.N[1] * m.N[2];
    if (!b->ec_done) {
        for (int k = 0; k < 4; ++k)
            if (!(b->ec[k] = ob_alloc<float>(b, 3 * cells))) return ob_fail(b, OEMS_ERR_NOMEM, "opbuild: EC allocation");
        cudaMemset(b->bad, 0, sizeof(int));
        ECOut o{b->ec[0], b->ec[1], b->ec[2], b->ec[3], b->bad};
        const unsigned blocks = (unsigned)((cells + 255) / 256);
        for (int n = 0; n < 3; ++n) k_ec<<<blocks, 256>>>(m, n, o);
        int bad = 0;
        if (cudaMemcpy(&bad, b->bad, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
            return ob_fail(b, OEMS_ERR_CUDA, "opbuild: EC kernel");
        if (bad) return ob_fail(b, OEMS_ERR_ARG, "opbuild: an effective material parameter is not finite");
        b->ec_done = true;
    }
    float* dst[4] = {C, G, L, R};
    for (int k = 0; k < 4; ++k)
        if (dst[k] && cudaMemcpy(dst[k], b->ec[k], 3 * cells * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
            return ob_fail(b, OEMS_ERR_CUDA, "opbuild: EC download");
    if (dt_var3) {
        const unsigned blocks = (unsigned)((cells + 255) / 256);
        double* part = ob_alloc<double>(b, blocks);
        if (!part) return ob_fail(b, OEMS_ERR_NOMEM, "opbuild: allocation");
        Var3In v{{m.N[0], m.N[1], m.N[2]}, b->ec[0], b->ec[2], part};
        k_var3<<<blocks, 256>>>(v);
        std::vector<double> h(blocks);
        if (cudaMemcpy(h.data(), part, blocks * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
            return ob_fail(b, OEMS_ERR_CUDA, "opbuild: timestep kernel");
        double dT = 1e200;
        for (double x : h) dT = std::min(dT, x);
        *dt_var3 = dT;
    }
    return OEMS_OK;
}

int oems_cuda_opbuild_coefficients(oems_cuda_opbuild* b, double dt, float* vv, float* vi, float* ii, float* iv)
{
    if (!b || !vv || !vi || !ii || !iv || !(dt > 0)) return OEMS_ERR_ARG;
    if (!b->ec_done) return ob_fail(b, OEMS_ERR_STATE, "opbuild: EC not computed");
    const Mesh& m = b->m;
    const unsigned long long n = 3ull * m.N[0] * m.N[1] * m.N[2];
    float* d[4];
    for (int k = 0; k < 4; ++k)
        if (!(d[k] = ob_alloc<float>(b, n))) return ob_fail(b, OEMS_ERR_NOMEM, "opbuild: allocation");
    k_coef<<<(unsigned)((n + 255) / 256), 256>>>(n, b->ec[0], b->ec[1], b->ec[2], b->ec[3], dt, d[0], d[1], d[2], d[3]);
    float* dst[4] = {vv, vi, ii, iv};
    for (int k = 0; k < 4; ++k)
        if (cudaMemcpy(dst[k], d[k], n * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
            return ob_fail(b, OEMS_ERR_CUDA, "opbuild: coefficient download");
    for (int k = 3; k >= 0; --k) {                           // coefficient buffers are not kept
        cudaFree(d[k]);
        b->mem.pop_back();
    }
    return OEMS_OK;
}

const char* oems_cuda_opbuild_last_error(const oems_cuda_opbuild* b) { return b ? b->err.c_str() : "null handle"; }

void oems_cuda_opbuild_destroy(oems_cuda_opbuild* b)
{
    if (!b) return;
    for (void* q : b->mem) cudaFree(q);
    delete b;
}

}  // extern "C"
