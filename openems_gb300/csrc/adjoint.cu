// adjoint.cu -- reverse-mode (adjoint) EC-FDTD: gradients of an objective built from probe
// samples with respect to the voltage coefficients (vv, vi) of the edges in a design box.
//
// One forward timestep (FDTD/engine.cpp:267-286 with the UPML hooks of
// FDTD/extensions/engine_ext_upml.cpp:52-229 and the additive excitation of
// FDTD/extensions/engine_ext_excitation.cpp:33-94) is affine in the state:
//     V' = vv*V + vi*K_V I          I' = ii*I + iv*K_I V'
// with K_V / K_I the curl stencils of k_update_v / k_update_i (UPML cells add pre/post hooks).
// For the adjoint (lambda_V, lambda_I) of one step, with a = lambda_I' and b = lambda_V' + K_I^T(iv a):
//     lambda_I = ii*a + K_V^T(vi*b)      lambda_V = vv*b
// In the scaled variables U = iv*a and W = vi*b the reverse step is again a pair of
// forward-like updates with the transposed curls:
//     U <- ii*U + iv*(K_V^T W + s_I)     W <- vv*W + vi*(K_I^T U + s_V)
// where s_I, s_V are dJ/d(probe sample) on the probe edges (a sample at numTS = n+1 enters the
// reverse step of forward step n).  Inside UPML regions the unscaled adjoints of V, I and of the
// two fluxes are kept in region-local arrays and the transposed pre/post hooks are applied.
// Gradients (design box, outside every UPML region): dJ/dvv += b V^n, dJ/dvi += b K_V I^n, with
// b = W/vi, accumulated in double.
//
// The curl transposes are gathers (no atomics), derived from the forward stencils including the
// reference's "same cell" read at index 0 (a shift of 0 makes the two terms cancel).
//
// The factors V^n and K_V I^n of the design box come either from checkpoints plus
// recomputation (checkpoint_every = K > 0: the full state every K steps, each K-step segment
// recomputed once in the reverse sweep) or from a record of every step kept during the forward
// run (checkpoint_every = 0: 24 bytes per design edge triple and step, no recomputation).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <new>
#include <vector>

#include "engine_impl.h"

using namespace oems;

namespace {

struct InjList {
    unsigned count;
    unsigned long long lo, hi;        // range of the cell offsets (component removed)
    const unsigned long long* cell;   // [count] cell offset
    const int* comp;                  // [count] component
    const int* row;                   // [count] source row (objective probe)
    const double* coef;               // [count] weight * sign
    // the split main box's groups of four z (k_adj_box4) that hold a source cell: their offsets (z
    // a multiple of four).  The float4 box kernel skips them; blocks of their own update them.
    const unsigned long long* grp;
    unsigned ngrp;
};

// true when one of the list's cells lies in the group of four at offset o
__device__ __forceinline__ bool group_has_source(const InjList& L, unsigned long long o)
{
    for (unsigned k = 0; k < L.count; ++k) {
        const unsigned long long c = L.cell[k];
        if (c >= o && c < o + 4) return true;
    }
    return false;
}

struct AdjDev {
    GridDev g;
    float* U;             // [3][S] iv * lambda_I (0 where I is not updated)
    float* W;             // [3][S] vi * (lambda_V + K_I^T U)
    float* lV[OEMS_MAX_UPML];      // [3][n] lambda_V in UPML cells
    float* lI[OEMS_MAX_UPML];      // [3][n] lambda_I in UPML cells
    float* lpsi[OEMS_MAX_UPML];    // [3][n] adjoint of the voltage flux
    float* lphi[OEMS_MAX_UPML];    // [3][n] adjoint of the current flux
    unsigned b0[3], bn[3];
    unsigned B;
    const float* fv;      // [3][B] V^n in the design box
    const float* fc;      // [3][B] K_V I^n in the design box
    double* gvv;          // [3][B]
    double* gvi;          // [3][B]
    const double* src;    // [rows][stride]
    unsigned stride;
    unsigned n;           // forward step being reversed; sources of sample n+1 enter
    // graph replay of the reverse sweep: n from device counters instead, n = counter - noff
    // (nctr for the update kernels, gctr for the design-box sums; noff is the step's place in
    // the captured graph, and each counter is stepped down once per replay on its own stream),
    // the factors of step n in slot (n % fK) of fbase
    const unsigned* nctr;
    const unsigned* gctr;
    unsigned noff;
    const float* fbase;
    unsigned fK;
    InjList injV, injI;
};

__device__ __forceinline__ void coef_v(const GridDev& g, unsigned long long o, float vv[3], float vi[3])
{
    if (g.idx) {
        const unsigned c = op_cls(g, o);
        const float4 a = __ldg(g.tabV + 2 * c), b = __ldg(g.tabV + 2 * c + 1);
        vv[0] = a.x; vv[1] = a.y; vv[2] = a.z; vi[0] = a.w; vi[1] = b.x; vi[2] = b.y;
    } else {
#pragma unroll
        for (int m = 0; m < 3; ++m) { vv[m] = __ldg(g.vv + m * g.S + o); vi[m] = __ldg(g.vi + m * g.S + o); }
    }
}

__device__ __forceinline__ void coef_i(const GridDev& g, unsigned long long o, float ii[3], float iv[3])
{
    if (g.idx) {
        const unsigned c = op_cls(g, o);
        const float4 a = __ldg(g.tabI + 2 * c), b = __ldg(g.tabI + 2 * c + 1);
        ii[0] = a.x; ii[1] = a.y; ii[2] = a.z; iv[0] = a.w; iv[1] = b.x; iv[2] = b.y;
    } else {
#pragma unroll
        for (int m = 0; m < 3; ++m) { ii[m] = __ldg(g.ii + m * g.S + o); iv[m] = __ldg(g.iv + m * g.S + o); }
    }
}

// probe sources of sample n+1 at cell o (few entries; only threads inside the probes' range look)
__device__ __forceinline__ void add_sources(const AdjDev& a, const InjList& L, unsigned long long o, float s[3])
{
    if (L.count == 0 || o < L.lo || o > L.hi) return;
    for (unsigned k = 0; k < L.count; ++k)
        if (L.cell[k] == o) {
            const unsigned n = a.nctr ? *a.nctr - a.noff : a.n;
            const float v = (float)(a.src[(unsigned long long)L.row[k] * a.stride + n + 1] * L.coef[k]);
            const int m = L.comp[k];                       // constant indices keep s in registers
            if (m == 0) s[0] = fadd(s[0], v);
            else if (m == 1) s[1] = fadd(s[1], v);
            else s[2] = fadd(s[2], v);
        }
}

// U <- ii*U + iv*(K_V^T W + s_I) for one cell with x < Nx-1, y < Ny-1, z < Nz-1 (I is never
// updated elsewhere, so U stays 0 there).  UPML cells: transposed post/update/pre on the local
// adjoints.  rk/lk: the cell's region and local offset when known (rk = -2: look up).
__device__ __forceinline__ void adj_u_cell(const AdjDev& a, unsigned x, unsigned y, unsigned z, int rk, unsigned lk)
{
    const GridDev& g = a.g;
    const unsigned long long S = g.S;
    const unsigned long long o = ((unsigned long long)x * g.Ny + y) * g.Pz + z;
    const unsigned long long sx = (unsigned long long)g.Ny * g.Pz, sy = g.Pz;
    const float* __restrict__ W = a.W;
    // every independent load first: W at the cell and its +x/+y/+z neighbours, the coefficients,
    // the cell's own adjoint state
    const float w0 = __ldg(W + o), w1 = __ldg(W + S + o), w2 = __ldg(W + 2 * S + o);
    const float w1z = __ldg(W + S + o + 1), w2y = __ldg(W + 2 * S + o + sy), w2x = __ldg(W + 2 * S + o + sx);
    const float w0z = __ldg(W + o + 1), w0y = __ldg(W + o + sy), w1x = __ldg(W + S + o + sx);
    float ii[3], iv[3];
    coef_i(g, o, ii, iv);
    unsigned loc = lk;
    const int r = rk == -2 ? upml_find(g, x, y, z, loc) : rk;
    float st[3];
    if (r < 0) {
#pragma unroll
        for (int m = 0; m < 3; ++m) st[m] = a.U[m * S + o];
    } else {
#pragma unroll
        for (int m = 0; m < 3; ++m) st[m] = a.lI[r][m * g.upml[r].n + loc];
    }
    // d/dI of sum_o W(o) . K_V I (o); the forward's index-0 self reads cancel the direct term
    float d[3] = {
        fadd(fsub(fsub(z > 0 ? w1 : 0.f, w1z), y > 0 ? w2 : 0.f), w2y),
        fadd(fsub(fsub(x > 0 ? w2 : 0.f, w2x), z > 0 ? w0 : 0.f), w0z),
        fadd(fsub(fsub(y > 0 ? w0 : 0.f, w0y), x > 0 ? w1 : 0.f), w1x)};
    add_sources(a, a.injI, o, d);
    if (r < 0) {
#pragma unroll
        for (int m = 0; m < 3; ++m) a.U[m * S + o] = fadd(fmul(ii[m], st[m]), fmul(iv[m], d[m]));
        return;
    }
    float pc[9];
    upml_coef<true>(g.upml[r], loc, pc);
    const unsigned n = g.upml[r].n;
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        const unsigned k = m * n + loc;
        const float lam = fadd(st[m], d[m]);                    // adjoint of I after the step
        const float lin = fadd(fmul(pc[6 + m], lam), a.lphi[r][k]);   // post^T: I = h + iifn*flux
        a.U[m * S + o] = fmul(iv[m], lin);
        a.lphi[r][k] = fsub(fmul(ii[m], lin), fmul(pc[3 + m], lam));  // pre^T: f = ii*I - iifo*flux
        a.lI[r][k] = fmul(pc[m], lam);
    }
}

// W <- vv*W + vi*(K_I^T U + s_V) for one cell, with the design-box gradient sums
__device__ __forceinline__ void adj_w_cell(const AdjDev& a, unsigned x, unsigned y, unsigned z, int rk, unsigned lk)
{
    const GridDev& g = a.g;
    const unsigned long long S = g.S;
    const unsigned long long o = ((unsigned long long)x * g.Ny + y) * g.Pz + z;
    // -x/-y/-z neighbours; at index 0 the cell itself is read and the term dropped below
    const unsigned long long sx = x ? (unsigned long long)g.Ny * g.Pz : 0ull;
    const unsigned long long sy = y ? (unsigned long long)g.Pz : 0ull;
    const unsigned long long sz = z ? 1ull : 0ull;
    const float* __restrict__ U = a.U;
    const float u0 = __ldg(U + o), u1 = __ldg(U + S + o), u2 = __ldg(U + 2 * S + o);
    const float u1z = __ldg(U + S + o - sz), u2y = __ldg(U + 2 * S + o - sy), u2x = __ldg(U + 2 * S + o - sx);
    const float u0z = __ldg(U + o - sz), u0y = __ldg(U + o - sy), u1x = __ldg(U + S + o - sx);
    float vv[3], vi[3];
    coef_v(g, o, vv, vi);
    unsigned loc = lk;
    const int r = rk == -2 ? upml_find(g, x, y, z, loc) : rk;
    float st[3];
    if (r < 0) {
#pragma unroll
        for (int m = 0; m < 3; ++m) st[m] = a.W[m * S + o];
    } else {
#pragma unroll
        for (int m = 0; m < 3; ++m) st[m] = a.lV[r][m * g.upml[r].n + loc];
    }
    float gs[3] = {
        fadd(fsub(fsub(u1, z ? u1z : 0.f), u2), y ? u2y : 0.f),
        fsub(fadd(fsub(u2, x ? u2x : 0.f), z ? u0z : 0.f), u0),
        fadd(fsub(fsub(u0, y ? u0y : 0.f), u1), x ? u1x : 0.f)};
    add_sources(a, a.injV, o, gs);
    if (r < 0) {
        float wn[3];
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            wn[m] = fadd(fmul(vv[m], st[m]), fmul(vi[m], gs[m]));
            a.W[m * S + o] = wn[m];
        }
        const unsigned bx = x - a.b0[0], by = y - a.b0[1], bz = z - a.b0[2];
        if (bx < a.bn[0] && by < a.bn[1] && bz < a.bn[2]) {
            const unsigned kb = (bx * a.bn[1] + by) * a.bn[2] + bz;
            // per-step products in float (FP64 arithmetic is slow on this GPU), sums in double
#pragma unroll
            for (int m = 0; m < 3; ++m) {
                if (vi[m] == 0.f) continue;                     // PEC edge: no dependence
                const float b = fmul(wn[m], __frcp_rn(vi[m]));
                const unsigned kk = m * a.B + kb;
                a.gvv[kk] += (double)fmul(b, __ldg(a.fv + kk));
                a.gvi[kk] += (double)fmul(b, __ldg(a.fc + kk));
            }
        }
        return;
    }
    float pc[9];
    upml_coef<false>(g.upml[r], loc, pc);
    const unsigned n = g.upml[r].n;
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        const unsigned k = m * n + loc;
        const float b = fadd(st[m], gs[m]);                     // adjoint of V after the step
        const float lvn = fadd(fmul(pc[6 + m], b), a.lpsi[r][k]);      // post^T: V = h + vvfn*flux
        a.W[m * S + o] = fmul(vi[m], lvn);
        a.lpsi[r][k] = fsub(fmul(vv[m], lvn), fmul(pc[3 + m], b));     // pre^T: f = vv*V - vvfo*flux
        a.lV[r][k] = fmul(pc[m], b);
    }
}

// one thread per cell of an x-plane (blockIdx.y = x), for engines without UPML
__global__ void __launch_bounds__(256) k_adj_u(AdjDev a)
{
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned y = t / a.g.Pz, z = t - y * a.g.Pz;
    if (y + 1 >= a.g.Ny || z + 1 >= a.g.Nz) return;
    adj_u_cell(a, blockIdx.y, y, z, -2, 0);
}

__global__ void __launch_bounds__(256) k_adj_w(AdjDev a)
{
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned y = t / a.g.Pz, z = t - y * a.g.Pz;
    if (y >= a.g.Ny || z >= a.g.Nz) return;
    adj_w_cell(a, blockIdx.y, y, z, -2, 0);
}

// The UPML regions four z cells per thread (the forward's k_update_reg4 groups: aligned to four
// z in the mesh, lanes outside the region computed but not stored): adj_u_cell / adj_w_cell's
// region branch lane by lane, with 16-byte loads of the adjoint fields and, where the region's
// z rows are whole groups, of the region-local adjoint arrays.  U lanes at z = Nz-1 (and groups at
// x = Nx-1 or y = Ny-1) are not updated.
template <bool CURR>
__device__ __forceinline__ void adj_src_group(const AdjDev& a, const SplitDev& sp, unsigned j);

template <bool CURR>
__global__ void __launch_bounds__(256, 3) k_adj_reg4(const __grid_constant__ AdjDev a, const __grid_constant__ SplitDev sp)
{
    const GridDev& g = a.g;
    const unsigned b = blockIdx.x;
    const unsigned* fblk = blockDim.x == 128u ? sp.first4h : sp.first4;
    if (b >= fblk[sp.nreg]) {                       // the main box's source groups (k_adj_box4 skips them)
        const unsigned j = (b - fblk[sp.nreg]) * blockDim.x + threadIdx.x;
        if (j < (CURR ? a.injI.ngrp : a.injV.ngrp)) adj_src_group<CURR>(a, sp, j);
        return;
    }
    int r = 0;
    while (r + 1 < (int)sp.nreg && b >= fblk[r + 1]) ++r;
    const UpmlDev& u = g.upml[r];
    const unsigned j = (b - fblk[r]) * blockDim.x + threadIdx.x;
    if (j >= u.nl[0] * u.nl[1] * reg_groups_per_row(u)) return;
    const RegGroup q = reg_group(u, j);
    const unsigned x = q.x, y = q.y, z0 = q.z0;
    if (CURR && (x + 1 >= g.Nx || y + 1 >= g.Ny)) return;
    unsigned mask = q.mask;
    if (CURR)
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (z0 + k + 1 >= g.Nz) mask &= ~(1u << k);
    const unsigned S = (unsigned)g.S, n = u.n;
    const unsigned o = (x * g.Ny + y) * g.Pz + z0;
    const uint4 ci = op_cls4(g, o);
    unsigned ucl[4];
    ld_cls(u.cls + q.loc0, q.vec, mask, ucl);
    // the cell's adjoint state (lI / lV) and the flux adjoint (lphi / lpsi), region-local
    float* const ls = (CURR ? a.lI[r] : a.lV[r]) + q.loc0;
    float* const lf = (CURR ? a.lphi[r] : a.lpsi[r]) + q.loc0;
    float4 s0 = ld_lanes(ls, q.vec, mask), s1 = ld_lanes(ls + n, q.vec, mask), s2 = ld_lanes(ls + 2 * n, q.vec, mask);
    float4 f0 = ld_lanes(lf, q.vec, mask), f1 = ld_lanes(lf + n, q.vec, mask), f2 = ld_lanes(lf + 2 * n, q.vec, mask);
    float4 d0, d1, d2;                          // K^T of the other adjoint field, lane by lane
    if (CURR) {
        const float* __restrict__ W = a.W;
        const unsigned sx = g.Ny * g.Pz, sy = g.Pz;
        const float4 w0 = ldg4(W + o), w1 = ldg4(W + (S + o)), w2 = ldg4(W + (2 * S + o));
        const float w1z4 = __ldg(W + (S + o + 4)), w0z4 = __ldg(W + (o + 4));
        const float4 w2y = ldg4(W + (2 * S + o + sy)), w0y = ldg4(W + (o + sy));
        const float4 w2x = ldg4(W + (2 * S + o + sx)), w1x = ldg4(W + (S + o + sx));
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const unsigned z = z0 + k;
            const float a1z = k < 3 ? f4(w1, k + 1) : w1z4, a0z = k < 3 ? f4(w0, k + 1) : w0z4;
            set4(d0, k, fadd(fsub(fsub(z > 0 ? f4(w1, k) : 0.f, a1z), y > 0 ? f4(w2, k) : 0.f), f4(w2y, k)));
            set4(d1, k, fadd(fsub(fsub(x > 0 ? f4(w2, k) : 0.f, f4(w2x, k)), z > 0 ? f4(w0, k) : 0.f), a0z));
            set4(d2, k, fadd(fsub(fsub(y > 0 ? f4(w0, k) : 0.f, f4(w0y, k)), x > 0 ? f4(w1, k) : 0.f), f4(w1x, k)));
        }
    } else {
        const float* __restrict__ U = a.U;
        const unsigned sx = x ? g.Ny * g.Pz : 0u, sy = y ? g.Pz : 0u;
        const float4 u0 = ldg4(U + o), u1 = ldg4(U + (S + o)), u2 = ldg4(U + (2 * S + o));
        const float u1m = z0 ? __ldg(U + (S + o - 1)) : 0.f, u0m = z0 ? __ldg(U + (o - 1)) : 0.f;
        const float4 u2y = ldg4(U + (2 * S + o - sy)), u0y = ldg4(U + (o - sy));
        const float4 u2x = ldg4(U + (2 * S + o - sx)), u1x = ldg4(U + (S + o - sx));
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const unsigned z = z0 + k;
            const float b1z = k ? f4(u1, k - 1) : u1m, b0z = k ? f4(u0, k - 1) : u0m;
            set4(d0, k, fadd(fsub(fsub(f4(u1, k), z ? b1z : 0.f), f4(u2, k)), y ? f4(u2y, k) : 0.f));
            set4(d1, k, fsub(fadd(fsub(f4(u2, k), x ? f4(u2x, k) : 0.f), z ? b0z : 0.f), f4(u0, k)));
            set4(d2, k, fadd(fsub(fsub(f4(u0, k), y ? f4(u0y, k) : 0.f), f4(u1, k)), x ? f4(u1x, k) : 0.f));
        }
    }
    const InjList& L = CURR ? a.injI : a.injV;
    const bool src = L.count && (unsigned long long)o + 3 >= L.lo && (unsigned long long)o <= L.hi;
    const unsigned cls[4] = {ci.x, ci.y, ci.z, ci.w};
    const float4* tab = CURR ? g.tabI : g.tabV;
    float4 o0 = make_float4(0.f, 0.f, 0.f, 0.f), o1 = o0, o2 = o0;   // the new U / W
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (!(mask & (1u << k))) continue;
        float dd[3] = {f4(d0, k), f4(d1, k), f4(d2, k)};
        if (src) add_sources(a, L, (unsigned long long)o + k, dd);
        const float4 ca = __ldg(tab + 2 * cls[k]), cb = __ldg(tab + 2 * cls[k] + 1);
        const float4* t = u.ctab + 6u * ucl[k] + (CURR ? 3 : 0);
        const float4 pa = __ldg(t), pb = __ldg(t + 1), pd = __ldg(t + 2);
        const float pc[9] = {pa.x, pa.y, pa.z, pa.w, pb.x, pb.y, pb.z, pb.w, pd.x};
        const float cd[3] = {ca.x, ca.y, ca.z}, cs[3] = {ca.w, cb.x, cb.y};   // (ii, iv) or (vv, vi)
        const float st[3] = {f4(s0, k), f4(s1, k), f4(s2, k)};
        const float fl[3] = {f4(f0, k), f4(f1, k), f4(f2, k)};
        float on[3], fn[3], sn[3];
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            const float lam = fadd(st[m], dd[m]);               // adjoint of the field after the step
            const float lin = fadd(fmul(pc[6 + m], lam), fl[m]);   // post^T: F = h + fn*flux
            on[m] = fmul(cs[m], lin);
            fn[m] = fsub(fmul(cd[m], lin), fmul(pc[3 + m], lam));  // pre^T: f = c*F - fo*flux
            sn[m] = fmul(pc[m], lam);
        }
        set4(o0, k, on[0]); set4(o1, k, on[1]); set4(o2, k, on[2]);
        set4(f0, k, fn[0]); set4(f1, k, fn[1]); set4(f2, k, fn[2]);
        set4(s0, k, sn[0]); set4(s1, k, sn[1]); set4(s2, k, sn[2]);
    }
    float* __restrict__ F = CURR ? a.U : a.W;
    st4_masked(F + o, o0, mask);
    st4_masked(F + (S + o), o1, mask);
    st4_masked(F + (2 * S + o), o2, mask);
    st_lanes(lf, f0, q.vec, mask);
    st_lanes(lf + n, f1, q.vec, mask);
    st_lanes(lf + 2 * n, f2, q.vec, mask);
    st_lanes(ls, s0, q.vec, mask);
    st_lanes(ls + n, s1, q.vec, mask);
    st_lanes(ls + 2 * n, s2, q.vec, mask);
}

// the engine's UPML work split (k_update_split): the region blocks first, then the blocks of the
// cells outside every region (a launch of the first first_block[nreg] blocks covers the regions
// alone, followed by k_adj_box4_* over the main box)
template <bool CURR>
__global__ void __launch_bounds__(256, 6) k_adj_split(AdjDev a, SplitDev sp)
{
    const GridDev& g = a.g;
    unsigned b = blockIdx.x;
    const unsigned rblocks = sp.first_block[sp.nreg];
    if (b >= rblocks) {
        unsigned t = (b - rblocks) * 256u + threadIdx.x;
        if (t >= sp.main_cells) return;
        const unsigned z = sp.lo[2] + t % sp.n[2];
        t /= sp.n[2];
        const unsigned y = sp.lo[1] + t % sp.n[1];
        const unsigned x = sp.lo[0] + t / sp.n[1];
        int r = -1;
        unsigned loc = 0;
        if (sp.full) r = upml_find(g, x, y, z, loc);
        if (r >= 0) return;
        if (CURR) adj_u_cell(a, x, y, z, -1, 0);
        else adj_w_cell(a, x, y, z, -1, 0);
        return;
    }
    int r = 0;
    while (r + 1 < (int)sp.nreg && b >= sp.first_block[r + 1]) ++r;
    const UpmlDev& u = g.upml[r];
    const unsigned loc = (b - sp.first_block[r]) * 256u + threadIdx.x;
    if (loc >= u.n) return;
    const unsigned lz = loc % u.nl[2], rest = loc / u.nl[2];
    const unsigned x = u.start[0] + rest / u.nl[1], y = u.start[1] + rest % u.nl[1], z = u.start[2] + lz;
    if (CURR) {
        if (x + 1 >= g.Nx || y + 1 >= g.Ny || z + 1 >= g.Nz) return;
        adj_u_cell(a, x, y, z, r, loc);
    } else {
        adj_w_cell(a, x, y, z, r, loc);
    }
}

// The main box of the split (compressed operator, no UPML cell in it), four z cells per thread:
// adj_u_cell / adj_w_cell's arithmetic per lane, with the float4 loads of the forward's
// update_*4_cells.  Lane k is cell z0 + k; groups start on multiples of four, and lanes outside
// the box's z range are computed but not stored (their cells belong to the region blocks).
// one group of four of the U update in k_adj_box4<true>; SRC: it may hold source cells of injI
template <bool SRC>
__device__ __forceinline__ void adj_u4_group(const AdjDev& a, const SplitDev& sp, unsigned x, unsigned y, unsigned z0)
{
    unsigned mask = 0u;
#pragma unroll
    for (int k = 0; k < 4; ++k) mask |= (z0 + k >= sp.lo[2] && z0 + k < sp.lo[2] + sp.n[2]) ? (1u << k) : 0u;
    const GridDev& g = a.g;
    const unsigned S = (unsigned)g.S;
    const unsigned o = (x * g.Ny + y) * g.Pz + z0;
    const unsigned sx = g.Ny * g.Pz, sy = g.Pz;
    const float* __restrict__ W = a.W;
    const float4 w0 = ldg4(W + o), w1 = ldg4(W + (S + o)), w2 = ldg4(W + (2 * S + o));
    const float w1z4 = __ldg(W + (S + o + 4)), w0z4 = __ldg(W + (o + 4));
    const float4 w2y = ldg4(W + (2 * S + o + sy)), w0y = ldg4(W + (o + sy));
    const float4 w2x = ldg4(W + (2 * S + o + sx)), w1x = ldg4(W + (S + o + sx));
    const uint4 ci = op_cls4(g, o);
    float4 u0 = ld4(a.U + o), u1 = ld4(a.U + (S + o)), u2 = ld4(a.U + (2 * S + o));
    const unsigned cls[4] = {ci.x, ci.y, ci.z, ci.w};
    const bool src = SRC && a.injI.count && (unsigned long long)o + 3 >= a.injI.lo && (unsigned long long)o <= a.injI.hi;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const unsigned z = z0 + k;
        const float4 ca = __ldg(g.tabI + 2 * cls[k]), cb = __ldg(g.tabI + 2 * cls[k] + 1);
        const float a1z = k < 3 ? f4(w1, k + 1) : w1z4, a0z = k < 3 ? f4(w0, k + 1) : w0z4;
        float d[3] = {
            fadd(fsub(fsub(z > 0 ? f4(w1, k) : 0.f, a1z), y > 0 ? f4(w2, k) : 0.f), f4(w2y, k)),
            fadd(fsub(fsub(x > 0 ? f4(w2, k) : 0.f, f4(w2x, k)), z > 0 ? f4(w0, k) : 0.f), a0z),
            fadd(fsub(fsub(y > 0 ? f4(w0, k) : 0.f, f4(w0y, k)), x > 0 ? f4(w1, k) : 0.f), f4(w1x, k))};
        if (src) add_sources(a, a.injI, (unsigned long long)o + k, d);
        set4(u0, k, fadd(fmul(ca.x, f4(u0, k)), fmul(ca.w, d[0])));
        set4(u1, k, fadd(fmul(ca.y, f4(u1, k)), fmul(cb.x, d[1])));
        set4(u2, k, fadd(fmul(ca.z, f4(u2, k)), fmul(cb.y, d[2])));
    }
    st4_masked(a.U + o, u0, mask);
    st4_masked(a.U + (S + o), u1, mask);
    st4_masked(a.U + (2 * S + o), u2, mask);
}

// one group of four of the W update in k_adj_box4<false>; SRC: it may hold source cells of injV
template <bool SRC>
__device__ __forceinline__ void adj_w4_group(const AdjDev& a, const SplitDev& sp, unsigned x, unsigned y, unsigned z0)
{
    unsigned mask = 0u;
#pragma unroll
    for (int k = 0; k < 4; ++k) mask |= (z0 + k >= sp.lo[2] && z0 + k < sp.lo[2] + sp.n[2]) ? (1u << k) : 0u;
    const GridDev& g = a.g;
    const unsigned S = (unsigned)g.S;
    const unsigned o = (x * g.Ny + y) * g.Pz + z0;
    const unsigned sx = x ? g.Ny * g.Pz : 0u, sy = y ? g.Pz : 0u;
    const float* __restrict__ U = a.U;
    const float4 u0 = ldg4(U + o), u1 = ldg4(U + (S + o)), u2 = ldg4(U + (2 * S + o));
    const float u1m = z0 ? __ldg(U + (S + o - 1)) : 0.f, u0m = z0 ? __ldg(U + (o - 1)) : 0.f;
    const float4 u2y = ldg4(U + (2 * S + o - sy)), u0y = ldg4(U + (o - sy));
    const float4 u2x = ldg4(U + (2 * S + o - sx)), u1x = ldg4(U + (S + o - sx));
    const uint4 ci = op_cls4(g, o);
    float4 n0 = ld4(a.W + o), n1 = ld4(a.W + (S + o)), n2 = ld4(a.W + (2 * S + o));
    const unsigned cls[4] = {ci.x, ci.y, ci.z, ci.w};
    const bool src = SRC && a.injV.count && (unsigned long long)o + 3 >= a.injV.lo && (unsigned long long)o <= a.injV.hi;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const unsigned z = z0 + k;
        const float4 ca = __ldg(g.tabV + 2 * cls[k]), cb = __ldg(g.tabV + 2 * cls[k] + 1);
        // -z neighbours: lane k-1, for lane 0 the float before the vector (none at z = 0)
        const float b1z = k ? f4(u1, k - 1) : u1m, b0z = k ? f4(u0, k - 1) : u0m;
        float gs[3] = {
            fadd(fsub(fsub(f4(u1, k), z ? b1z : 0.f), f4(u2, k)), y ? f4(u2y, k) : 0.f),
            fsub(fadd(fsub(f4(u2, k), x ? f4(u2x, k) : 0.f), z ? b0z : 0.f), f4(u0, k)),
            fadd(fsub(fsub(f4(u0, k), y ? f4(u0y, k) : 0.f), f4(u1, k)), x ? f4(u1x, k) : 0.f)};
        if (src) add_sources(a, a.injV, (unsigned long long)o + k, gs);
        const float vv[3] = {ca.x, ca.y, ca.z}, vi[3] = {ca.w, cb.x, cb.y};
        const float wn[3] = {fadd(fmul(vv[0], f4(n0, k)), fmul(vi[0], gs[0])),
                             fadd(fmul(vv[1], f4(n1, k)), fmul(vi[1], gs[1])),
                             fadd(fmul(vv[2], f4(n2, k)), fmul(vi[2], gs[2]))};
        set4(n0, k, wn[0]);
        set4(n1, k, wn[1]);
        set4(n2, k, wn[2]);
    }
    st4_masked(a.W + o, n0, mask);
    st4_masked(a.W + (S + o), n1, mask);
    st4_masked(a.W + (2 * S + o), n2, mask);
}

// The design-box gradient sums of adj_w_cell for the cells k_adj_box4<false> updated (the box lies
// outside every UPML region, so all of it is in the split's main box): one thread per design
// cell, reading back the new W.  Apart from the streaming kernel it keeps that kernel free of the
// box's dependent loads and double-precision sums; the values, and their order per sum, are
// adj_w_cell's.
__global__ void __launch_bounds__(256) k_adj_grad(AdjDev a)
{
    const unsigned kb = blockIdx.x * blockDim.x + threadIdx.x;
    if (kb >= a.B) return;
    const GridDev& g = a.g;
    const unsigned bz = kb % a.bn[2], by = (kb / a.bn[2]) % a.bn[1], bx = kb / (a.bn[2] * a.bn[1]);
    const unsigned x = a.b0[0] + bx, y = a.b0[1] + by, z = a.b0[2] + bz;
    const unsigned long long o = ((unsigned long long)x * g.Ny + y) * g.Pz + z;
    const float* fv = a.fv;
    if (a.gctr) fv = a.fbase + (size_t)((*a.gctr - a.noff) % a.fK) * 6u * a.B;
    const float* fc = fv + 3u * a.B;
    float vv[3], vi[3];
    coef_v(g, o, vv, vi);
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        if (vi[m] == 0.f) continue;                             // PEC edge: no dependence
        const float b = fmul(a.W[m * g.S + o], __frcp_rn(vi[m]));
        const unsigned kk = m * a.B + kb;
        a.gvv[kk] += (double)fmul(b, __ldg(fv + kk));
        a.gvi[kk] += (double)fmul(b, __ldg(fc + kk));
    }
}

// The main box four cells per thread.  The groups that hold a probe source are left to blocks of
// their own (in the region launch, or k_adj_box4_src): without the source code the streaming
// threads fit 64 registers with no spills.
template <bool CURR>
__global__ void __launch_bounds__(256, 4) k_adj_box4(AdjDev a, SplitDev sp)
{
    unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= sp.main_cells4) return;
    const unsigned z0 = sp.z4 + ((t % sp.n4) << 2);
    t /= sp.n4;
    const unsigned y = sp.lo[1] + t % sp.n[1];
    const unsigned x = sp.lo[0] + t / sp.n[1];
    const InjList& L = CURR ? a.injI : a.injV;
    const unsigned long long o = ((unsigned long long)x * a.g.Ny + y) * a.g.Pz + z0;
    if (L.count && o + 3 >= L.lo && o <= L.hi && group_has_source(L, o)) return;
    if (CURR) adj_u4_group<false>(a, sp, x, y, z0);
    else adj_w4_group<false>(a, sp, x, y, z0);
}

// the main-box group j of the source-group list: its update with the sources
template <bool CURR>
__device__ __forceinline__ void adj_src_group(const AdjDev& a, const SplitDev& sp, unsigned j)
{
    const InjList& L = CURR ? a.injI : a.injV;
    const unsigned long long og = L.grp[j];
    const unsigned long long row = og / a.g.Pz;
    const unsigned z0 = (unsigned)(og - row * a.g.Pz), y = (unsigned)(row % a.g.Ny), x = (unsigned)(row / a.g.Ny);
    if (CURR) adj_u4_group<true>(a, sp, x, y, z0);
    else adj_w4_group<true>(a, sp, x, y, z0);
}

// the source groups alone (splits whose regions run one cell per thread)
template <bool CURR>
__global__ void __launch_bounds__(64) k_adj_box4_src(AdjDev a, SplitDev sp)
{
    const unsigned j = blockIdx.x * 64u + threadIdx.x;
    if (j < (CURR ? a.injI.ngrp : a.injV.ngrp)) adj_src_group<CURR>(a, sp, j);
}

// V^n and K_V I^n (the arithmetic of update_v_cell) in the design box, into slot
// (*counter % modulo) of `base` (each slot [2][3][B]: V, then K_V I)
__global__ void k_adj_factors(AdjDev a, float* base, const unsigned* counter, unsigned modulo)
{
    const unsigned kb = blockIdx.x * blockDim.x + threadIdx.x;
    if (kb >= a.B) return;
    const unsigned slot = *counter % modulo;
    float* fv = base + (size_t)slot * 6 * a.B;
    float* fc = fv + 3 * a.B;
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

__global__ void k_inc(unsigned* c, unsigned by = 1u)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) *c += by;
}

__global__ void k_dec(unsigned* c, unsigned by = 1u)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) *c -= by;
}

}  // namespace

// checkpoint mode: factor buffers of K slots each (24 B per design edge triple and step: 400 MB
// per buffer for 64x64x16 design cells at K = 256).  The forward run keeps the factors of its last
// FB-1 segments, which the reverse sweep then needs not recompute, and the recompute of the others
// runs up to FB-1 segments ahead of the sweep.
constexpr unsigned FB = 6;

struct oems_adjoint_state {
    unsigned K = 256;                                 // 0: record mode
    unsigned steps = 0;
    std::vector<std::pair<void*, size_t>> regions;   // state: V, I, UPML fluxes
    std::vector<char*> ckpt;                          // checkpoints: segment starts + the end state
    AdjDev dev{};
    float* fac = nullptr;                             // factor slots [K or steps][2][3][B]
    size_t fac_slots = 0;
    unsigned* rec_numTS = nullptr;
    std::vector<void*> allocs;
    size_t state_bytes = 0;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    // checkpoint mode: the reverse sweep of segment k runs on `rs` while the engine stream
    // recomputes the segments below it into the other factor buffers (FB x K slots)
    cudaStream_t rs = nullptr;
    cudaEvent_t ev_recomputed[FB] = {};
    cudaEvent_t ev_reversed[FB] = {};
    // UPML split with a float4 main box (k_adj_box4): the design-box sums (k_adj_grad) run on
    // `gs`, after ev_w (W of the step done), and the next W update waits for ev_grad
    bool box4 = false;
    cudaStream_t gs = nullptr;
    cudaEvent_t ev_w = nullptr, ev_grad = nullptr, ev_grad_c = nullptr;
    // the float4 region kernels on a branch of their own beside the main box
    cudaStream_t rr = nullptr;
    cudaEvent_t ev_rfork = nullptr, ev_rjoin = nullptr;
    // graph replay of the reverse sweep: the step counters of the update kernels and of the sums
    unsigned* rev_n = nullptr;
    unsigned* rev_ng = nullptr;
    // checkpoint mode: segments from this one on had their factors recorded by the forward run
    // (until a reverse sweep overwrites those slots)
    unsigned recorded_from = ~0u;
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

// device-to-device copy of `bytes` (a multiple of 4) as 16-byte vectors where both ends allow it;
// as a kernel it streams at HBM rate, where a device-to-device cudaMemcpyAsync took about 0.6 ms
// per 130 MB checkpoint
__global__ void k_copy(float* __restrict__ dst, const float* __restrict__ src, size_t n)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool vec = ((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) & 15u) == 0;
    if (vec) {
        const size_t n4 = n / 4;
        for (size_t k = i; k < n4; k += stride)
            reinterpret_cast<float4*>(dst)[k] = __ldg(reinterpret_cast<const float4*>(src) + k);
        for (size_t k = n4 * 4 + i; k < n; k += stride) dst[k] = src[k];
    } else {
        for (size_t k = i; k < n; k += stride) dst[k] = src[k];
    }
}

int copy_state(oems_cuda_engine* e, oems_adjoint_state* s, char* ck, bool save)
{
    size_t off = 0;
    for (const auto& r : s->regions) {
        float* dst = reinterpret_cast<float*>(save ? ck + off : static_cast<char*>(r.first));
        const float* src = reinterpret_cast<const float*>(save ? static_cast<const char*>(r.first) : ck + off);
        const size_t n = r.second / sizeof(float);
        const unsigned blocks = (unsigned)std::min<size_t>(152 * 8, (n / 4 + 255) / 256 + 1);
        k_copy<<<blocks, 256, 0, e->stream>>>(dst, src, n);
        if (cudaGetLastError() != cudaSuccess) return afail(e, OEMS_ERR_CUDA, "checkpoint copy");
        off += (r.second + 255) & ~(size_t)255;          // every region on a 256-byte boundary
    }
    return OEMS_OK;
}

// kernels of one recompute step (recompute_step)
unsigned recompute_launches(const oems_cuda_engine* e)
{
    const unsigned per_update = (e->use_split && e->splitV.v4) ? 2u : 1u;
    return 2 * per_update + 1 + (e->excV.count ? 1u : 0u) + (e->excI.count ? 1u : 0u);
}

// one forward step without processing, the step counter being rec_numTS; returns the launches.
// fac != nullptr: the voltage update writes the design-box factors of this step itself.
// toff: the step's place after the counter (inside a captured run of steps whose counter is
// stepped once at its end; inc = false leaves the counter to that)
unsigned recompute_step(oems_cuda_engine* e, oems_adjoint_state* s, const FacOut* fac = nullptr, unsigned toff = 0,
                        bool inc = true)
{
    cudaStream_t st = e->stream;
    // two update launches (the split's region kernel and main box count two each) and k_inc
    const unsigned per_update = (e->use_split && e->splitV.v4) ? 2u : 1u;
    unsigned L = 2 * per_update + (inc ? 1u : 0u);
    launch_update(e, false, st, nullptr, fac);
    if (e->excV.count) {
        k_excitation<<<(e->excV.count + 127) / 128, 128, 0, st>>>(e->dV, e->excV, s->rec_numTS, toff);
        ++L;
    }
    launch_update(e, true, st);
    if (e->excI.count) {
        k_excitation<<<(e->excI.count + 127) / 128, 128, 0, st>>>(e->dI, e->excI, s->rec_numTS, toff);
        ++L;
    }
    if (inc) k_inc<<<1, 32, 0, st>>>(s->rec_numTS);
    return L;
}

// forward run that records the factors of every step (record mode): graphs of 1 and 16 steps,
// each step preceded by the factor kernel writing slot numTS
// base/modulo: the factors of step numTS go to slot numTS % modulo of base (record mode: all of
// s->fac, one slot per step; checkpoint mode: the last segments, into their factor buffers)
int record_forward(oems_cuda_engine* e, oems_adjoint_state* s, unsigned steps, float* base = nullptr,
                   unsigned modulo = 0xFFFFFFFFu)
{
    if (!base) base = s->fac;
    const unsigned KG = 16;
    cudaGraphExec_t gx[2] = {nullptr, nullptr};
    const unsigned counts[2] = {1, KG};
    const unsigned fb = (s->dev.B + 255) / 256;
    for (int k = 0; k < 2; ++k) {
        cudaGraph_t graph = nullptr;
        if (cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
            return afail(e, OEMS_ERR_CUDA, "record capture");
        int rc = OEMS_OK;
        for (unsigned j = 0; j < counts[k] && rc == OEMS_OK; ++j) {
            k_adj_factors<<<fb, 256, 0, e->stream>>>(s->dev, base, e->d_numTS, modulo);
            unsigned L = 0;
            rc = enqueue_step(e, &L);
        }
        const cudaError_t c = cudaStreamEndCapture(e->stream, &graph);
        if (rc != OEMS_OK || c != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            for (auto& x : gx) if (x) cudaGraphExecDestroy(x);
            return rc != OEMS_OK ? rc : afail(e, OEMS_ERR_CUDA, "record capture");
        }
        const cudaError_t ci = cudaGraphInstantiate(&gx[k], graph, 0);
        cudaGraphDestroy(graph);
        if (ci != cudaSuccess) {
            for (auto& x : gx) if (x) cudaGraphExecDestroy(x);
            return afail(e, OEMS_ERR_CUDA, "record graph instantiate");
        }
    }
    int rc = OEMS_OK;
    unsigned done = 0;
    while (done < steps && rc == OEMS_OK) {
        const int k = steps - done >= KG ? 1 : 0;
        if (cudaGraphLaunch(gx[k], e->stream) != cudaSuccess) rc = afail(e, OEMS_ERR_CUDA, "record graph launch");
        done += counts[k];
    }
    e->host_numTS += done;
    for (auto& x : gx) cudaGraphExecDestroy(x);
    return rc;
}

// the engine's probe terms of the objective probes of one type, for the reverse kernels; the
// device arrays are appended to `tmp` (freed by the caller)
int build_injection(oems_cuda_engine* e, unsigned nprobe, const int* ids, int type, InjList& L,
                    std::vector<void*>& tmp)
{
    std::vector<unsigned long long> cell;
    std::vector<int> comp, row;
    std::vector<double> coef;
    for (unsigned k = 0; k < nprobe; ++k) {
        const ProbeDev& p = e->probe_dev[ids[k]];
        if (p.type != type || p.nterm == 0) continue;
        std::vector<unsigned long long> term(p.nterm);
        std::vector<signed char> sign(p.nterm);
        if (cudaMemcpy(term.data(), p.term, p.nterm * sizeof(unsigned long long), cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(sign.data(), p.sign, p.nterm, cudaMemcpyDeviceToHost) != cudaSuccess)
            return afail(e, OEMS_ERR_CUDA, "probe term copy");
        for (unsigned j = 0; j < p.nterm; ++j) {
            comp.push_back((int)(term[j] / e->S));
            cell.push_back(term[j] % e->S);
            row.push_back((int)k);
            coef.push_back(p.weight * (double)sign[j]);
        }
    }
    L = InjList{};
    L.count = (unsigned)cell.size();
    if (!L.count) return OEMS_OK;
    L.lo = *std::min_element(cell.begin(), cell.end());
    L.hi = *std::max_element(cell.begin(), cell.end());
    void* p[4] = {nullptr, nullptr, nullptr, nullptr};
    const size_t bytes[4] = {cell.size() * sizeof(unsigned long long), comp.size() * sizeof(int),
                             row.size() * sizeof(int), coef.size() * sizeof(double)};
    for (int k = 0; k < 4; ++k) {
        if (cudaMalloc(&p[k], bytes[k]) != cudaSuccess) return afail(e, OEMS_ERR_NOMEM, "adjoint source allocation");
        tmp.push_back(p[k]);
    }
    auto* dc = static_cast<unsigned long long*>(p[0]);
    auto* dm = static_cast<int*>(p[1]);
    auto* dr = static_cast<int*>(p[2]);
    auto* dw = static_cast<double*>(p[3]);
    cudaMemcpyAsync(dc, cell.data(), cell.size() * sizeof(unsigned long long), cudaMemcpyHostToDevice, e->stream);
    cudaMemcpyAsync(dm, comp.data(), comp.size() * sizeof(int), cudaMemcpyHostToDevice, e->stream);
    cudaMemcpyAsync(dr, row.data(), row.size() * sizeof(int), cudaMemcpyHostToDevice, e->stream);
    cudaMemcpyAsync(dw, coef.data(), coef.size() * sizeof(double), cudaMemcpyHostToDevice, e->stream);
    L.cell = dc; L.comp = dm; L.row = dr; L.coef = dw;
    // the main-box groups of four that hold a source cell (k_adj_box4 leaves them out)
    const SplitDev& sp = type == 0 ? e->splitV : e->splitI;
    std::vector<unsigned long long> grp;
    if (e->use_split && sp.v4) {
        for (const unsigned long long c : cell) {
            const unsigned long long r = c / e->Pz;
            const unsigned z = (unsigned)(c - r * e->Pz), y = (unsigned)(r % e->N[1]), x = (unsigned)(r / e->N[1]);
            const unsigned z0 = z & ~3u;
            if (x >= sp.lo[0] && x < sp.lo[0] + sp.n[0] && y >= sp.lo[1] && y < sp.lo[1] + sp.n[1] && z0 >= sp.z4 &&
                (z0 - sp.z4) / 4 < sp.n4)
                grp.push_back(r * e->Pz + z0);
        }
        std::sort(grp.begin(), grp.end());
        grp.erase(std::unique(grp.begin(), grp.end()), grp.end());
    }
    if (!grp.empty()) {
        void* q = nullptr;
        if (cudaMalloc(&q, grp.size() * sizeof(unsigned long long)) != cudaSuccess)
            return afail(e, OEMS_ERR_NOMEM, "adjoint source allocation");
        tmp.push_back(q);
        cudaMemcpyAsync(q, grp.data(), grp.size() * sizeof(unsigned long long), cudaMemcpyHostToDevice, e->stream);
        L.grp = static_cast<const unsigned long long*>(q);
        L.ngrp = (unsigned)grp.size();
    }
    return OEMS_OK;
}

}  // namespace

extern "C" {

int oems_cuda_adjoint_setup(oems_cuda_engine* e, unsigned int checkpoint_every, const unsigned int box_start[3],
                            const unsigned int box_stop[3])
{
    if (!e || !box_start || !box_stop) return OEMS_ERR_ARG;
    if (!e->inited) return afail(e, OEMS_ERR_STATE, "engine not initialised");
    if (e->adj) return afail(e, OEMS_ERR_STATE, "adjoint already set up");
    if (!e->mur.empty() || !e->lor.empty() || e->has_tfsf || e->rlc.count || e->has_td || e->cyl_closed)
        return afail(e, OEMS_ERR_UNSUPPORTED,
                     "adjoint: Mur walls, dispersive materials, TFSF, lumped RLC loads and cylinder meshes are not supported");
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
    for (const auto& r : s->regions) s->state_bytes += (r.second + 255) & ~(size_t)255;
    AdjDev& d = s->dev;
    d.g = e->grid;
    int rc;
    if ((rc = aalloc(e, s, &d.U, 3 * e->S))) return rc;
    if ((rc = aalloc(e, s, &d.W, 3 * e->S))) return rc;
    for (int r = 0; r < e->grid.nupml; ++r) {
        const size_t n3 = 3ull * e->grid.upml[r].n;
        if ((rc = aalloc(e, s, &d.lV[r], n3)) || (rc = aalloc(e, s, &d.lI[r], n3)) ||
            (rc = aalloc(e, s, &d.lpsi[r], n3)) || (rc = aalloc(e, s, &d.lphi[r], n3)))
            return rc;
    }
    d.B = 1;
    for (int a = 0; a < 3; ++a) {
        d.b0[a] = box_start[a];
        d.bn[a] = box_stop[a] - box_start[a];
        d.B *= d.bn[a];
    }
    if ((rc = aalloc(e, s, &d.gvv, 3ull * d.B))) return rc;
    if ((rc = aalloc(e, s, &d.gvi, 3ull * d.B))) return rc;
    if (s->K) {
        s->fac_slots = (size_t)FB * s->K;
        if ((rc = aalloc(e, s, &s->fac, s->fac_slots * 6ull * d.B))) return rc;
        if (cudaStreamCreateWithFlags(&s->rs, cudaStreamNonBlocking) != cudaSuccess)
            return afail(e, OEMS_ERR_CUDA, "adjoint stream");
        for (unsigned b = 0; b < FB; ++b)
            if (cudaEventCreateWithFlags(&s->ev_recomputed[b], cudaEventDisableTiming) != cudaSuccess ||
                cudaEventCreateWithFlags(&s->ev_reversed[b], cudaEventDisableTiming) != cudaSuccess)
                return afail(e, OEMS_ERR_CUDA, "adjoint events");
    }
    if ((rc = aalloc(e, s, &s->rec_numTS, 1))) return rc;
    if ((rc = aalloc(e, s, &s->rev_n, 2))) return rc;
    s->rev_ng = s->rev_n + 1;
    if (cudaEventCreate(&s->ev[0]) != cudaSuccess || cudaEventCreate(&s->ev[1]) != cudaSuccess)
        return afail(e, OEMS_ERR_CUDA, "adjoint events");
    s->box4 = e->use_split && e->compressed && e->splitI.v4 && e->splitV.v4;
    if (s->box4 && (cudaStreamCreateWithFlags(&s->gs, cudaStreamNonBlocking) != cudaSuccess ||
                    cudaEventCreateWithFlags(&s->ev_w, cudaEventDisableTiming) != cudaSuccess ||
                    cudaEventCreateWithFlags(&s->ev_grad, cudaEventDisableTiming) != cudaSuccess ||
                    cudaEventCreateWithFlags(&s->ev_grad_c, cudaEventDisableTiming) != cudaSuccess ||
                    cudaStreamCreateWithFlags(&s->rr, cudaStreamNonBlocking) != cudaSuccess ||
                    cudaEventCreateWithFlags(&s->ev_rfork, cudaEventDisableTiming) != cudaSuccess ||
                    cudaEventCreateWithFlags(&s->ev_rjoin, cudaEventDisableTiming) != cudaSuccess))
        return afail(e, OEMS_ERR_CUDA, "adjoint side streams");
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
    const unsigned nseg = s->K ? (steps + s->K - 1) / s->K : 0;
    for (unsigned k = 0; k <= nseg; ++k) {            // segment starts + the end state (record mode: end only)
        char* c = nullptr;
        if (cudaMalloc(&c, s->state_bytes) != cudaSuccess) return afail(e, OEMS_ERR_NOMEM, "checkpoint allocation");
        s->ckpt.push_back(c);
    }
    if (!s->K && s->fac_slots < steps) {               // record mode: one factor slot per step
        if (s->fac) {
            cudaFree(s->fac);
            s->allocs.erase(std::find(s->allocs.begin(), s->allocs.end(), (void*)s->fac));
            s->fac = nullptr;
        }
        int rc = aalloc(e, s, &s->fac, (size_t)steps * 6 * s->dev.B);
        if (rc) return rc;
        s->fac_slots = steps;
    }
    cudaEventRecord(s->ev[0], e->stream);
    int rc = OEMS_OK;
    if (s->K) {
        // the last FB-1 segments also record their factors, into their factor buffers, so the
        // reverse sweep starts on them without recomputing them
        const unsigned nrec = std::min(nseg, FB - 1);
        const size_t half = (size_t)s->K * 6 * s->dev.B;
        for (unsigned k = 0; k < nseg && rc == OEMS_OK; ++k) {
            if ((rc = copy_state(e, s, s->ckpt[k], true))) break;
            const unsigned len = std::min(s->K, steps - k * s->K);
            if (k + nrec >= nseg) rc = record_forward(e, s, len, s->fac + (k % FB) * half, s->K);
            else rc = oems_cuda_iterate(e, len);
        }
        s->recorded_from = nseg - nrec;
    } else {
        rc = record_forward(e, s, steps);
    }
    if (rc == OEMS_OK) rc = copy_state(e, s, s->ckpt[nseg], true);
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
    for (unsigned k = 0; k < nprobe; ++k) {
        if (probe_ids[k] < 0 || probe_ids[k] >= (int)e->probe_dev.size()) return afail(e, OEMS_ERR_ARG, "bad probe id");
        if (e->probe_dev[probe_ids[k]].type >= 2)
            return afail(e, OEMS_ERR_ARG, "field probes are not objectives (voltage/current probes only)");
    }
    AdjDev& d = s->dev;
    cudaStream_t st = e->stream;
    const unsigned N = s->steps;
    const size_t nsrc = (size_t)nprobe * (N + 1);
    std::vector<void*> tmp;
    auto release = [&]() {
        for (void* q : tmp) cudaFree(q);
        tmp.clear();
    };
    int rc;
    if ((rc = build_injection(e, nprobe, probe_ids, 0, d.injV, tmp)) ||
        (rc = build_injection(e, nprobe, probe_ids, 1, d.injI, tmp))) {
        cudaStreamSynchronize(st);
        release();
        return rc;
    }
    double* dsrc = nullptr;
    if (cudaMalloc(&dsrc, std::max<size_t>(1, nsrc) * sizeof(double)) != cudaSuccess) {
        cudaStreamSynchronize(st);
        release();
        return afail(e, OEMS_ERR_NOMEM, "adjoint source allocation");
    }
    tmp.push_back(dsrc);
    cudaEventRecord(s->ev[0], st);
    if (nsrc) cudaMemcpyAsync(dsrc, sources, nsrc * sizeof(double), cudaMemcpyHostToDevice, st);
    d.src = dsrc;
    d.stride = N + 1;
    cudaMemsetAsync(d.U, 0, 3 * e->S * sizeof(float), st);
    cudaMemsetAsync(d.W, 0, 3 * e->S * sizeof(float), st);
    for (int r = 0; r < e->grid.nupml; ++r) {
        const size_t b3 = 3ull * e->grid.upml[r].n * sizeof(float);
        cudaMemsetAsync(d.lV[r], 0, b3, st);
        cudaMemsetAsync(d.lI[r], 0, b3, st);
        cudaMemsetAsync(d.lpsi[r], 0, b3, st);
        cudaMemsetAsync(d.lphi[r], 0, b3, st);
    }
    cudaMemsetAsync(d.gvv, 0, 3ull * d.B * sizeof(double), st);
    cudaMemsetAsync(d.gvi, 0, 3ull * d.B * sizeof(double), st);
    const unsigned plane = e->N[1] * e->Pz;
    const dim3 gu((plane + 255) / 256, e->N[0] - 1), gw((plane + 255) / 256, e->N[0]);
    const unsigned fb = (d.B + 255) / 256;
    rc = OEMS_OK;
    // kernels per reverse step: the adjoint updates (+ the design-box sums and, in graph replay,
    // the two counter steps) and, in checkpoint mode, the recompute (+ the factor launch when the
    // voltage update does not record them)
    unsigned lps = (e->use_split && s->box4) ? 4u + (d.B ? 1u : 0u) : 2u;
    if (s->K) {
        const unsigned rec = recompute_launches(e);
        lps += rec + (s->box4 ? 0u : 1u);
        // (graph replay adds two counter launches per 16 steps)
    }
    const unsigned bu = e->splitI.main_blocks + e->splitI.first_block[e->splitI.nreg];
    const unsigned bw = e->splitV.main_blocks + e->splitV.first_block[e->splitV.nreg];
    // one reverse step of the float4 split on rst.  wait_grad: the W update waits for the previous
    // step's design-box sums (in a captured graph the first step's wait is the graph boundary);
    // ctr: the sums' counter to step down after them (graph replay)
    auto reverse_box4 = [&](const AdjDev& dd, cudaStream_t rst, bool wait_grad, unsigned* gctr, cudaEvent_t evg) {
        const SplitDev* sp[2] = {&e->splitI, &e->splitV};
        for (int h = 0; h < 2; ++h) {
            if (h == 1 && wait_grad) cudaStreamWaitEvent(rst, evg, 0);
            const unsigned ng = h == 0 ? dd.injI.ngrp : dd.injV.ngrp;
            if (sp[h]->reg4) {
                cudaEventRecord(s->ev_rfork, rst);
                cudaStreamWaitEvent(s->rr, s->ev_rfork, 0);
                const unsigned tb = e->adj_reg_block;
                const unsigned rblk = (tb == 128u ? sp[h]->first4h[sp[h]->nreg] : sp[h]->first4[sp[h]->nreg]) +
                                      (ng + tb - 1) / tb;
                if (h == 0) k_adj_reg4<true><<<rblk, tb, 0, s->rr>>>(dd, *sp[h]);
                else k_adj_reg4<false><<<rblk, tb, 0, s->rr>>>(dd, *sp[h]);
            } else {
                if (const unsigned rblk = sp[h]->first_block[sp[h]->nreg]) {
                    if (h == 0) k_adj_split<true><<<rblk, 256, 0, rst>>>(dd, *sp[h]);
                    else k_adj_split<false><<<rblk, 256, 0, rst>>>(dd, *sp[h]);
                }
                if (ng) {
                    if (h == 0) k_adj_box4_src<true><<<(ng + 63) / 64, 64, 0, rst>>>(dd, *sp[h]);
                    else k_adj_box4_src<false><<<(ng + 63) / 64, 64, 0, rst>>>(dd, *sp[h]);
                }
            }
            if (sp[h]->main_blocks4) {
                const unsigned tb = e->adj_box_block, nb = (sp[h]->main_cells4 + tb - 1) / tb;
                if (h == 0) k_adj_box4<true><<<nb, tb, 0, rst>>>(dd, *sp[h]);
                else k_adj_box4<false><<<nb, tb, 0, rst>>>(dd, *sp[h]);
            }
            if (sp[h]->reg4) {
                cudaEventRecord(s->ev_rjoin, s->rr);
                cudaStreamWaitEvent(rst, s->ev_rjoin, 0);
            }
        }
        if (dd.B) {
            cudaEventRecord(s->ev_w, rst);
            cudaStreamWaitEvent(s->gs, s->ev_w, 0);
            k_adj_grad<<<(dd.B + 255) / 256, 256, 0, s->gs>>>(dd);
            if (gctr) k_dec<<<1, 32, 0, s->gs>>>(gctr);
            cudaEventRecord(evg, s->gs);
        }
    };
    auto reverse = [&](unsigned n, const float* slot, cudaStream_t rst) {
        d.n = n;
        d.fv = slot;
        d.fc = slot + 3 * d.B;
        if (e->use_split && s->box4) {
            reverse_box4(d, rst, true, nullptr, s->ev_grad);
            return;
        }
        if (e->use_split) {
            if (bu) k_adj_split<true><<<bu, 256, 0, rst>>>(d, e->splitI);
            if (bw) k_adj_split<false><<<bw, 256, 0, rst>>>(d, e->splitV);
        } else {
            k_adj_u<<<gu, 256, 0, rst>>>(d);
            k_adj_w<<<gw, 256, 0, rst>>>(d);
        }
    };
    if (s->K) {
        // Two-stage pipeline over the segments, last to first. The engine stream restores
        // checkpoint k and recomputes segment k, recording its factors into buffer k % FB; the
        // reverse stream then sweeps segment k from those factors while the engine stream already
        // recomputes the segments below it, up to FB-1 ahead (a buffer is reused once the sweep
        // of its previous segment has released it). The two streams share nothing else: the
        // sweep reads the coefficients, the factors and its own adjoint arrays, the recompute the
        // engine state.  The last FB-1 segments were recorded by the forward run.
        const unsigned nseg = (N + s->K - 1) / s->K;
        const size_t half = (size_t)s->K * 6 * d.B;
        auto fac_out = [&](unsigned hb) {
            return FacOut{s->fac + hb * half, s->rec_numTS, s->K, {d.b0[0], d.b0[1], d.b0[2]},
                          {d.bn[0], d.bn[1], d.bn[2]}, d.B};
        };
        // With the float4 split the voltage update records the factors itself (the design box lies
        // in its main box), and the recompute of a whole segment replays a captured graph of 16
        // steps per factor half (the step counter and the slot come from device memory).
        constexpr unsigned RG = 16;
        cudaGraphExec_t rgraph[FB] = {};
        if (s->box4 && s->K % RG == 0) {
            for (unsigned hb = 0; hb < FB && rc == OEMS_OK; ++hb) {
                FacOut fo = fac_out(hb);
                cudaGraph_t graph = nullptr;
                if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
                    rc = afail(e, OEMS_ERR_CUDA, "recompute graph capture");
                    break;
                }
                // step j runs at counter + j; the counter steps once at the end
                for (unsigned j = 0; j < RG; ++j) {
                    fo.coff = j;
                    recompute_step(e, s, &fo, j, false);
                }
                k_inc<<<1, 32, 0, st>>>(s->rec_numTS, RG);
                if (cudaStreamEndCapture(st, &graph) != cudaSuccess ||
                    cudaGraphInstantiate(&rgraph[hb], graph, 0) != cudaSuccess)
                    rc = afail(e, OEMS_ERR_CUDA, "recompute graph");
                if (graph) cudaGraphDestroy(graph);
            }
        }
        // the reverse sweep of a whole segment likewise replays a graph of 16 reverse steps per
        // factor half, n coming from the device counters (set at the segment's start)
        cudaGraphExec_t vgraph[FB] = {};
        if (s->box4 && s->K % RG == 0 && rc == OEMS_OK) {
            for (unsigned hb = 0; hb < FB && rc == OEMS_OK; ++hb) {
                AdjDev dg = d;
                dg.nctr = s->rev_n;
                dg.gctr = d.B ? s->rev_ng : nullptr;
                dg.fbase = s->fac + hb * half;
                dg.fK = s->K;
                cudaGraph_t graph = nullptr;
                if (cudaStreamBeginCapture(s->rs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
                    rc = afail(e, OEMS_ERR_CUDA, "reverse graph capture");
                    break;
                }
                // (an event of its own: the direct steps never wait on one recorded in a capture);
                // step j reverses n = counter - j, and the counters step down by RG at the end
                for (unsigned j = 0; j < RG; ++j) {
                    dg.noff = j;
                    reverse_box4(dg, s->rs, j > 0, nullptr, s->ev_grad_c);
                }
                k_dec<<<1, 32, 0, s->rs>>>(s->rev_n, RG);
                if (d.B) {
                    k_dec<<<1, 32, 0, s->gs>>>(s->rev_ng, RG);                // after the last sums
                    cudaEventRecord(s->ev_grad_c, s->gs);
                    cudaStreamWaitEvent(s->rs, s->ev_grad_c, 0);            // the sums rejoin the graph
                }
                if (cudaStreamEndCapture(s->rs, &graph) != cudaSuccess ||
                    cudaGraphInstantiate(&vgraph[hb], graph, 0) != cudaSuccess)
                    rc = afail(e, OEMS_ERR_CUDA, "reverse graph");
                if (graph) cudaGraphDestroy(graph);
            }
        }
        auto recompute = [&](unsigned seg) -> int {
            if (seg >= s->recorded_from) {                  // recorded by the forward run
                cudaEventRecord(s->ev_recomputed[seg % FB], st);
                return OEMS_OK;
            }
            const unsigned a0 = seg * s->K, a1 = std::min(N, a0 + s->K);
            float* base = s->fac + (seg % FB) * half;
            int r2;
            if ((r2 = copy_state(e, s, s->ckpt[seg], false))) return r2;
            cudaMemcpyAsync(s->rec_numTS, &a0, sizeof(unsigned), cudaMemcpyHostToDevice, st);
            const FacOut fo = fac_out(seg % FB);
            unsigned n = a0;
            if (rgraph[seg % FB])
                for (; n + RG <= a1; n += RG)
                    if (cudaGraphLaunch(rgraph[seg % FB], st) != cudaSuccess)
                        return afail(e, OEMS_ERR_CUDA, "recompute graph launch");
            for (; n < a1; ++n) {
                if (s->box4) {
                    recompute_step(e, s, &fo);
                } else {
                    k_adj_factors<<<fb, 256, 0, st>>>(d, base, s->rec_numTS, s->K);
                    recompute_step(e, s);
                }
            }
            cudaEventRecord(s->ev_recomputed[seg % FB], st);
            return OEMS_OK;
        };
        // the first FB-1 segments of the sweep, then one more ahead per swept segment
        for (int seg = (int)nseg - 1; seg >= (int)nseg - (int)(FB - 1) && seg >= 0 && rc == OEMS_OK; --seg)
            rc = recompute((unsigned)seg);
        for (int seg = (int)nseg - 1; seg >= 0 && rc == OEMS_OK; --seg) {
            const unsigned a0 = seg * s->K, a1 = std::min(N, a0 + s->K);
            const int ahead = seg - (int)(FB - 1);
            if (ahead >= 0) {
                // segment `ahead` reuses the buffer of segment ahead+FB: wait for that sweep
                if (ahead + (int)FB < (int)nseg) cudaStreamWaitEvent(st, s->ev_reversed[(ahead + FB) % FB], 0);
                if ((rc = recompute((unsigned)ahead))) break;
            }
            cudaStreamWaitEvent(s->rs, s->ev_recomputed[seg % FB], 0);
            const float* base = s->fac + (seg % FB) * half;
            if (vgraph[seg % FB] && a1 - a0 == s->K) {
                // the previous direct step's sums first; then n = a1-1 down to a0 from the counters
                cudaStreamWaitEvent(s->rs, s->ev_grad, 0);
                const unsigned start[2] = {a1 - 1, a1 - 1};
                cudaMemcpyAsync(s->rev_n, start, sizeof(start), cudaMemcpyHostToDevice, s->rs);
                for (unsigned r = 0; r < s->K / RG; ++r)
                    if (cudaGraphLaunch(vgraph[seg % FB], s->rs) != cudaSuccess) {
                        rc = afail(e, OEMS_ERR_CUDA, "reverse graph launch");
                        break;
                    }
            } else {
                for (int n = (int)a1 - 1; n >= (int)a0; --n)
                    reverse((unsigned)n, base + (size_t)(n % s->K) * 6 * d.B, s->rs);
            }
            if (s->ev_grad) cudaStreamWaitEvent(s->rs, s->ev_grad, 0);   // the sums read this half too
            cudaEventRecord(s->ev_reversed[seg % FB], s->rs);
            if (cudaGetLastError() != cudaSuccess) rc = afail(e, OEMS_ERR_CUDA, "adjoint launch");
        }
        // the gradients, the timing event and the state restore follow the last sweep
        if (s->ev_grad) cudaStreamWaitEvent(s->rs, s->ev_grad, 0);
        cudaEventRecord(s->ev_reversed[0], s->rs);
        cudaStreamWaitEvent(st, s->ev_reversed[0], 0);
        for (auto& x : rgraph)
            if (x) cudaGraphExecDestroy(x);             // freed when their last launch completes
        for (auto& x : vgraph)
            if (x) cudaGraphExecDestroy(x);
    } else {
        for (int n = (int)N - 1; n >= 0; --n) reverse((unsigned)n, s->fac + (size_t)n * 6 * d.B, st);
        if (s->ev_grad) cudaStreamWaitEvent(st, s->ev_grad, 0);
        if (cudaGetLastError() != cudaSuccess) rc = afail(e, OEMS_ERR_CUDA, "adjoint launch");
    }
    s->launches_per_reverse_step = lps;
    // the recompute of earlier segments reused the recorded halves: a later sweep recomputes all
    if (s->K && s->recorded_from != ~0u && s->recorded_from > 0) s->recorded_from = ~0u;
    // leave the engine at its forward end state
    if (rc == OEMS_OK && s->K) rc = copy_state(e, s, s->ckpt.back(), false);
    if (rc == OEMS_OK) {
        cudaMemcpyAsync(gvv, d.gvv, 3ull * d.B * sizeof(double), cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(gvi, d.gvi, 3ull * d.B * sizeof(double), cudaMemcpyDeviceToHost, st);
        cudaEventRecord(s->ev[1], st);
        if (cudaEventSynchronize(s->ev[1]) != cudaSuccess) rc = afail(e, OEMS_ERR_CUDA, "adjoint sync");
        else cudaEventElapsedTime(&s->bwd_ms, s->ev[0], s->ev[1]);
    } else {
        cudaStreamSynchronize(st);
    }
    if (s->rs) cudaStreamSynchronize(s->rs);
    if (s->gs) cudaStreamSynchronize(s->gs);
    if (s->rr) cudaStreamSynchronize(s->rr);
    release();
    d.src = nullptr;
    d.injV = InjList{};
    d.injI = InjList{};
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
    for (unsigned b = 0; b < FB; ++b) {
        if (s->ev_recomputed[b]) cudaEventDestroy(s->ev_recomputed[b]);
        if (s->ev_reversed[b]) cudaEventDestroy(s->ev_reversed[b]);
    }
    if (s->rs) cudaStreamDestroy(s->rs);
    if (s->ev_w) cudaEventDestroy(s->ev_w);
    if (s->ev_grad) cudaEventDestroy(s->ev_grad);
    if (s->ev_grad_c) cudaEventDestroy(s->ev_grad_c);
    if (s->gs) cudaStreamDestroy(s->gs);
    if (s->ev_rfork) cudaEventDestroy(s->ev_rfork);
    if (s->ev_rjoin) cudaEventDestroy(s->ev_rjoin);
    if (s->rr) cudaStreamDestroy(s->rr);
    delete s;
}
