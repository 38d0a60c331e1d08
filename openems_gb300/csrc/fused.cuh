// fused.cuh -- one kernel per timestep: the voltage and current updates of
// Engine::UpdateVoltages / UpdateCurrents (FDTD/engine.cpp:110-222) with the UPML hooks
// (FDTD/extensions/engine_ext_upml.cpp:52-229) and the soft excitation
// (FDTD/extensions/engine_ext_excitation.cpp:33-94) in one sweep over the mesh.
//
// Each block owns a tile of FT_Z x FT_Y cells in the y-z plane and marches over a chunk of
// x-planes.  For plane x it stages I_old(x) (tile plus a one-cell -y/-z halo) in shared memory,
// computes V'(x) on the tile plus a one-cell +y/+z halo (the halo values are recomputed, not
// exchanged), and then computes I'(x-1) of its own tile from V'(x-1) and V'(x).  The step reads
// V and I once and writes them once (about 52 bytes per cell-step with the class index, against
// 80 for the two separate half-step kernels), so the fields ping-pong between two buffers: the
// step reads (V, I, voltage UPML flux) from one set and writes the other.  Current fluxes are
// only touched by their own cell and stay in place.  Arithmetic is identical to
// update_v_cell/update_i_cell plus k_excitation, so results are bit-identical.
//
// Used for engines without Mur walls and dispersive materials (their hooks read neighbouring
// lines between the two half-steps).
#pragma once

#include "kernels.cuh"

namespace oems {

constexpr int FT_Z = 32;      // tile extent along z (one warp per y-row)
constexpr int FT_Y = 8;       // tile extent along y
constexpr int FT_THREADS = FT_Z * FT_Y;        // one thread per tile cell
constexpr int FT_NHALO = FT_Z + 1 + FT_Y;       // V' halo cells: the +y row and the +z column
constexpr int FT_BLOCK = FT_THREADS + 64;       // plus two warps for the halo cells
constexpr int FT_MAX_SRC = 64;

struct FusedDev {
    GridDev g;                 // V, I, UPML voltage fluxes: the buffers read by this step
    float* Vo;                 // written by this step
    float* Io;
    float* vflux_o[OEMS_MAX_UPML];
    ExcDev excV, excI;
    const unsigned long long* srcV_cell;   // excitation cells (component removed), per source
    const unsigned long long* srcI_cell;
    unsigned long long srcV_lo, srcV_hi, srcI_lo, srcI_hi;
    const unsigned* numTS;
    unsigned xchunk;           // x-planes per block
};

// the excitation value of source k at step ts (k_excitation's arithmetic)
__device__ __forceinline__ float exc_value(const ExcDev& e, unsigned k, int ts)
{
    const int p = e.period ? (int)e.period : ts + 1;
    int exc_pos = ts - (int)e.delay[k];
    exc_pos *= (exc_pos > 0);
    exc_pos %= p;
    exc_pos *= (exc_pos < (int)e.length);
    return fmul(e.amp[k], e.sig[exc_pos]);
}

// add the sources at cell o (component m) to f[m], in source order
__device__ __forceinline__ void add_excitation(const ExcDev& e, const unsigned long long* cell, unsigned long long lo,
                                               unsigned long long hi, unsigned long long o, unsigned long long S,
                                               int ts, float f[3])
{
    if (e.count == 0 || o < lo || o > hi) return;
    for (unsigned k = 0; k < e.count; ++k)
        if (cell[k] == o) {
            // constant indices keep f in registers
            const int m = (int)(e.off[k] / S);
            const float v = exc_value(e, k, ts);
            if (m == 0) f[0] = fadd(f[0], v);
            else if (m == 1) f[1] = fadd(f[1], v);
            else f[2] = fadd(f[2], v);
        }
}

constexpr int FI_Y = FT_Y + 2, FI_Z = FT_Z + 2;   // staged I plane: tile + one cell on -y/-z and +y/+z
constexpr int FV_Y = FT_Y + 1, FV_Z = FT_Z + 1;   // V' plane: tile + one cell on +y/+z

__device__ __forceinline__ int fi_idx(int c, int yy, int zz) { return (c * FI_Y + yy) * FI_Z + zz; }
__device__ __forceinline__ int fv_idx(int c, int yy, int zz) { return (c * FV_Y + yy) * FV_Z + zz; }

// V'(x, y, z) from the staged planes Ic = I_old(x), Ip = I_old(x-1) (tile coordinates ty, tz of
// the V' region); update_v_cell's arithmetic, then the soft sources.  owner: the cell belongs to
// this block and plane, so its new value and UPML flux are written.
template <bool COMPRESSED>
__device__ __forceinline__ void fused_v_cell(const FusedDev& f, unsigned x, unsigned y, unsigned z, int ty, int tz,
                                             const float* Ic, const float* Ip, float* Vc, bool owner, int ts,
                                             const float vold[3], unsigned cls, int r, unsigned loc)
{
    const GridDev& g = f.g;
    const unsigned long long S = g.S;
    const unsigned long long o = ((unsigned long long)x * g.Ny + y) * g.Pz + z;
    const int yy = ty + 1, zz = tz + 1;
    const float i0 = Ic[fi_idx(0, yy, zz)], i1 = Ic[fi_idx(1, yy, zz)], i2 = Ic[fi_idx(2, yy, zz)];
    const float c0 = fadd(fsub(fsub(i2, Ic[fi_idx(2, yy - 1, zz)]), i1), Ic[fi_idx(1, yy, zz - 1)]);
    const float c1 = fadd(fsub(fsub(i0, Ic[fi_idx(0, yy, zz - 1)]), i2), Ip[fi_idx(2, yy, zz)]);
    const float c2 = fadd(fsub(fsub(i1, Ip[fi_idx(1, yy, zz)]), i0), Ic[fi_idx(0, yy - 1, zz)]);
    float vv0, vv1, vv2, vi0, vi1, vi2;
    if (COMPRESSED) {                                      // cls and vold were prefetched a plane ahead
        const float4 a = __ldg(g.tabV + 2 * cls), b = __ldg(g.tabV + 2 * cls + 1);
        vv0 = a.x; vv1 = a.y; vv2 = a.z; vi0 = a.w; vi1 = b.x; vi2 = b.y;
    } else {
        vv0 = __ldg(g.vv + o); vv1 = __ldg(g.vv + S + o); vv2 = __ldg(g.vv + 2 * S + o);
        vi0 = __ldg(g.vi + o); vi1 = __ldg(g.vi + S + o); vi2 = __ldg(g.vi + 2 * S + o);
    }
    const float v0 = vold[0], v1 = vold[1], v2 = vold[2];
    float out[3];
    if (r >= 0) {                                          // r, loc: the cell's UPML region (-1: none)
        const UpmlDev& u = g.upml[r];
        float pc[9];
        upml_coef<false>(u, loc, pc);
        const float vin[3] = {v0, v1, v2}, cc[3] = {c0, c1, c2};
        const float cvv[3] = {vv0, vv1, vv2}, cvi[3] = {vi0, vi1, vi2};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const unsigned q = k * u.n + loc;
            const float flux = __ldg(u.vflux + q);
            const float fpre = fsub(fmul(pc[k], vin[k]), fmul(pc[3 + k], flux));
            const float vn = fadd(fmul(flux, cvv[k]), fmul(cvi[k], cc[k]));
            if (owner) f.vflux_o[r][q] = vn;
            out[k] = fadd(fpre, fmul(pc[6 + k], vn));
        }
    } else {
        out[0] = fadd(fmul(v0, vv0), fmul(vi0, c0));
        out[1] = fadd(fmul(v1, vv1), fmul(vi1, c1));
        out[2] = fadd(fmul(v2, vv2), fmul(vi2, c2));
    }
    add_excitation(f.excV, f.srcV_cell, f.srcV_lo, f.srcV_hi, o, S, ts, out);
#pragma unroll
    for (int k = 0; k < 3; ++k) Vc[fv_idx(k, ty, tz)] = out[k];
    if (owner) {
        f.Vo[o] = out[0];
        f.Vo[S + o] = out[1];
        f.Vo[2 * S + o] = out[2];
    }
}

// I'(x, y, z) of an own cell from the staged V' planes Vp = V'(x) and Vc = V'(x+1) and the staged
// I_old(x) plane Ip; update_i_cell's arithmetic (UPML current flux in place), then the sources.
template <bool COMPRESSED>
__device__ __forceinline__ void fused_i_cell(const FusedDev& f, unsigned x, unsigned y, unsigned z, int ty, int tz,
                                             const float* Vp, const float* Vc, const float* Ip, int ts, unsigned cls,
                                             int r, unsigned loc)
{
    const GridDev& g = f.g;
    const unsigned long long S = g.S;
    const unsigned long long o = ((unsigned long long)x * g.Ny + y) * g.Pz + z;
    const float w0 = Vp[fv_idx(0, ty, tz)], w1 = Vp[fv_idx(1, ty, tz)], w2 = Vp[fv_idx(2, ty, tz)];
    const float c0 = fadd(fsub(fsub(w2, Vp[fv_idx(2, ty + 1, tz)]), w1), Vp[fv_idx(1, ty, tz + 1)]);
    const float c1 = fadd(fsub(fsub(w0, Vp[fv_idx(0, ty, tz + 1)]), w2), Vc[fv_idx(2, ty, tz)]);
    const float c2 = fadd(fsub(fsub(w1, Vc[fv_idx(1, ty, tz)]), w0), Vp[fv_idx(0, ty + 1, tz)]);
    float ii0, ii1, ii2, iv0, iv1, iv2;
    if (COMPRESSED) {
        const float4 a = __ldg(g.tabI + 2 * cls), b = __ldg(g.tabI + 2 * cls + 1);
        ii0 = a.x; ii1 = a.y; ii2 = a.z; iv0 = a.w; iv1 = b.x; iv2 = b.y;
    } else {
        ii0 = __ldg(g.ii + o); ii1 = __ldg(g.ii + S + o); ii2 = __ldg(g.ii + 2 * S + o);
        iv0 = __ldg(g.iv + o); iv1 = __ldg(g.iv + S + o); iv2 = __ldg(g.iv + 2 * S + o);
    }
    const int yy = ty + 1, zz = tz + 1;
    const float a0 = Ip[fi_idx(0, yy, zz)], a1 = Ip[fi_idx(1, yy, zz)], a2 = Ip[fi_idx(2, yy, zz)];
    float out[3];
    if (r >= 0) {
        const UpmlDev& u = g.upml[r];
        float pc[9];
        upml_coef<true>(u, loc, pc);
        const float iin[3] = {a0, a1, a2}, cc[3] = {c0, c1, c2};
        const float cii[3] = {ii0, ii1, ii2}, civ[3] = {iv0, iv1, iv2};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const unsigned q = k * u.n + loc;
            const float flux = u.iflux[q];
            const float fpre = fsub(fmul(pc[k], iin[k]), fmul(pc[3 + k], flux));
            const float in = fadd(fmul(flux, cii[k]), fmul(civ[k], cc[k]));
            u.iflux[q] = in;
            out[k] = fadd(fpre, fmul(pc[6 + k], in));
        }
    } else {
        out[0] = fadd(fmul(a0, ii0), fmul(iv0, c0));
        out[1] = fadd(fmul(a1, ii1), fmul(iv1, c1));
        out[2] = fadd(fmul(a2, ii2), fmul(iv2, c2));
    }
    add_excitation(f.excI, f.srcI_cell, f.srcI_lo, f.srcI_hi, o, S, ts, out);
    f.Io[o] = out[0];
    f.Io[S + o] = out[1];
    f.Io[2 * S + o] = out[2];
}

// 4-byte asynchronous global->shared copies (the staged I planes)
__device__ __forceinline__ void cp_async4(float* dst, const float* src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

// The march is software-pipelined: while plane x is computed, the copies of I_old(x+1) into a
// three-slot ring are in flight and V_old(x+1) and the class index of x+1 are being loaded into
// registers.  Plane p lives in ring slot (p + 1 - xa) % 3.
template <bool COMPRESSED>
__global__ void __launch_bounds__(FT_BLOCK) k_step_fused(FusedDev f)
{
    __shared__ float sI[3][3 * FI_Y * FI_Z];
    __shared__ float sV[2][3 * FV_Y * FV_Z];
    const GridDev& g = f.g;
    const int t = threadIdx.x;
    const bool tile = t < FT_THREADS;
    const int h = t - FT_THREADS;
    int cy, cz;                                            // this thread's cell in the V' region
    if (tile) { cy = t / FT_Z; cz = t % FT_Z; }
    else if (h <= FT_Z) { cy = FT_Y; cz = h; }
    else { cy = h - FT_Z - 1; cz = FT_Z; }
    const unsigned z0 = blockIdx.x * FT_Z, y0 = blockIdx.y * FT_Y;
    const unsigned xa = blockIdx.z * f.xchunk;
    if (xa >= g.Nx) return;
    const unsigned xb = min(g.Nx, xa + f.xchunk);          // own planes [xa, xb)
    const unsigned xend = min(xb + 1, g.Nx);               // V' planes [xa, xend)
    const unsigned y = y0 + cy, z = z0 + cz;
    const bool inV = (tile || h < FT_NHALO) && y < g.Ny && z < g.Nz;
    const bool inI = tile && y + 1 < g.Ny && z + 1 < g.Nz;
    const unsigned long long S = g.S, plane = (unsigned long long)g.Ny * g.Pz;
    const unsigned long long yz = (unsigned long long)y * g.Pz + z;
    const int ts = (int)*f.numTS;

    // I_old(px) over the tile and its one-cell rim into ring slot `slot`; rows/columns before
    // index 0 repeat index 0 (the reference's zero shift), those past the mesh are clamped (unused)
    // the staged elements of this thread (k = t + j * FT_BLOCK) and their plane-relative offsets,
    // computed once for the whole march
    constexpr int NSTAGE = 3 * FI_Y * FI_Z, NE = (NSTAGE + FT_BLOCK - 1) / FT_BLOCK;
    unsigned goff[NE];
#pragma unroll
    for (int j = 0; j < NE; ++j) {
        const int k = t + j * FT_BLOCK;
        goff[j] = 0;
        if (k < NSTAGE) {
            const int c = k / (FI_Y * FI_Z), rem = k - c * FI_Y * FI_Z, yy = rem / FI_Z, zz = rem - yy * FI_Z;
            const int yg = min(max((int)y0 + yy - 1, 0), (int)g.Ny - 1);
            const int zg = min(max((int)z0 + zz - 1, 0), (int)g.Nz - 1);
            goff[j] = (unsigned)(c * S + (unsigned long long)yg * g.Pz + zg);
        }
    }
    auto issue_I = [&](int slot, unsigned px) {
        const float* base = g.I + px * plane;
#pragma unroll
        for (int j = 0; j < NE; ++j)
            if (t + j * FT_BLOCK < NSTAGE) cp_async4(&sI[slot][t + j * FT_BLOCK], base + goff[j]);
    };
    auto prefetch = [&](unsigned px, float v[3], unsigned& c) {
        if (!inV) return;
        const unsigned long long o = px * plane + yz;
        v[0] = __ldg(g.V + o);
        v[1] = __ldg(g.V + S + o);
        v[2] = __ldg(g.V + 2 * S + o);
        if (COMPRESSED) c = __ldg(g.idx + o);
    };

    issue_I(0, xa > 0 ? xa - 1 : 0);                       // at x = 0 the -x neighbour is the plane itself
    issue_I(1, xa);
    cp_async_commit();
    float vc[3] = {0.f, 0.f, 0.f};
    unsigned cc = 0, cprev = 0;
    int rprev = -1;                                        // UPML region of the own cell at plane x-1
    unsigned lprev = 0;
    prefetch(xa, vc, cc);
    for (unsigned x = xa; x < xend; ++x) {
        const int sc = (int)((x + 1 - xa) % 3), sp = (int)((x - xa) % 3);
        const bool more = x + 1 < xend;
        if (more) issue_I((int)((x + 2 - xa) % 3), x + 1);
        cp_async_commit();
        cp_async_wait1();                                  // I_old(x) and I_old(x-1) have landed
        __syncthreads();
        float vn[3] = {0.f, 0.f, 0.f};
        unsigned cn = 0;
        if (more) prefetch(x + 1, vn, cn);
        float* Vc = sV[(x - xa) & 1];
        const float* Vp = sV[(x - xa + 1) & 1];
        unsigned loc = 0;
        const int r = (inV && g.nupml) ? upml_find(g, x, y, z, loc) : -1;
        if (inV) fused_v_cell<COMPRESSED>(f, x, y, z, cy, cz, sI[sc], sI[sp], Vc, tile && x < xb, ts, vc, cc, r, loc);
        __syncthreads();
        if (x > xa && tile && y < g.Ny && z < g.Nz) {
            if (inI) {
                fused_i_cell<COMPRESSED>(f, x - 1, y, z, cy, cz, Vp, Vc, sI[sp], ts, cprev, rprev, lprev);
            } else {                                       // I is never updated here: carry it over
                const unsigned long long o = (x - 1) * plane + yz;
#pragma unroll
                for (int k = 0; k < 3; ++k) f.Io[k * S + o] = sI[sp][fi_idx(k, cy + 1, cz + 1)];
            }
        }
        __syncthreads();
        cprev = cc;
        cc = cn;
        rprev = r;
        lprev = loc;
        vc[0] = vn[0]; vc[1] = vn[1]; vc[2] = vn[2];
    }
    if (xb == g.Nx && tile && y < g.Ny && z < g.Nz) {      // the last plane: I is never updated
        const float* Il = sI[(g.Nx - xa) % 3];
        const unsigned long long o = (unsigned long long)(g.Nx - 1) * plane + yz;
#pragma unroll
        for (int k = 0; k < 3; ++k) f.Io[k * S + o] = Il[fi_idx(k, cy + 1, cz + 1)];
    }
}

}  // namespace oems
