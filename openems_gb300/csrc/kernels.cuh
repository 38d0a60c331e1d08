// kernels.cuh -- device code of the GB300 EC-FDTD engine (sm_103a).
//
// Arithmetic rule: every float/double operation that the reference writes as a separate
// multiply and add/sub is issued with the _rn intrinsics (__fmul_rn, __fadd_rn, __fsub_rn,
// __dmul_rn, __dadd_rn) so the compiler cannot contract it into an FMA.  Together with the
// default -ftz=false this reproduces the reference's FP32 engine (FDTD/engine.cpp:110-222) bit
// for bit.  The kernels are memory-bound; the extra instruction cost is hidden.
//
// Field layout in HBM: float [3][Nx][Ny][Pz], Pz = Nz rounded up to a multiple of 4 so every
// z-row starts on a 16-byte boundary (padding lanes are never read as neighbours of real cells
// and stay zero).  Component stride S = Nx*Ny*Pz.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define OEMS_MAX_UPML 6
#define OEMS_MAX_MUR 6

namespace oems {

struct UpmlDev {
    unsigned start[3];
    unsigned nl[3];
    unsigned n;                 // nl[0]*nl[1]*nl[2]
    // coefficients, class-compressed (cls != nullptr) or dense
    const unsigned short* cls;  // [n] class of each cell
    const float4* ctab;         // [U][6]: (vv0 vv1 vv2 vvfo0)(vvfo1 vvfo2 vvfn0 vvfn1)(vvfn2 - - -), same for ii/iifo/iifn
    const float* vv;            // dense [3][n] each
    const float* vvfo;
    const float* vvfn;
    const float* ii;
    const float* iifo;
    const float* iifn;
    float* vflux;
    float* iflux;
};

struct GridDev {
    unsigned Nx, Ny, Nz, Pz;
    unsigned long long S;       // component stride
    float* V;
    float* I;
    // coefficients: compressed (idx != nullptr) or dense
    const unsigned* idx;        // [Nx][Ny][Pz]
    const unsigned short* idx16;  // the same in 16 bits when every class fits; read instead of idx
    const float4* tabV;         // [U][2]: (vv0,vv1,vv2,vi0) (vi1,vi2,-,-)
    const float4* tabI;         // [U][2]: (ii0,ii1,ii2,iv0) (iv1,iv2,-,-)
    const float* vv;            // dense [3][S]
    const float* vi;
    const float* ii;
    const float* iv;
    int nupml;
    UpmlDev upml[OEMS_MAX_UPML];
};

// the 16-bit copy of the class index (every class < 65,536)
static __global__ void k_narrow_index(unsigned short* __restrict__ dst, const unsigned* __restrict__ src,
                                      unsigned long long n)
{
    const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = (unsigned short)src[i];
}

// the operator class of cell o, and of the four cells o..o+3 (o a multiple of 4)
__device__ __forceinline__ unsigned op_cls(const GridDev& g, unsigned long long o)
{
    return g.idx16 ? (unsigned)__ldg(g.idx16 + o) : __ldg(g.idx + o);
}
__device__ __forceinline__ uint4 op_cls4(const GridDev& g, unsigned long long o)
{
    if (g.idx16) {
        const uint2 v = __ldg(reinterpret_cast<const uint2*>(g.idx16 + o));
        return make_uint4(v.x & 0xFFFFu, v.x >> 16, v.y & 0xFFFFu, v.y >> 16);
    }
    return __ldg(reinterpret_cast<const uint4*>(g.idx + o));
}

__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }

// UPML coefficients of one cell: c = {f0 f1 f2, fo0 fo1 fo2, fn0 fn1 fn2} with (f, fo, fn) =
// (vv, vvfo, vvfn) for CURR == false and (ii, iifo, iifn) for CURR == true
template <bool CURR>
__device__ __forceinline__ void upml_coef(const UpmlDev& u, unsigned loc, float c[9])
{
    if (u.cls) {
        const float4* t = u.ctab + 6u * __ldg(u.cls + loc) + (CURR ? 3 : 0);
        const float4 a = __ldg(t), b = __ldg(t + 1), d = __ldg(t + 2);
        c[0] = a.x; c[1] = a.y; c[2] = a.z; c[3] = a.w;
        c[4] = b.x; c[5] = b.y; c[6] = b.z; c[7] = b.w; c[8] = d.x;
    } else {
        const float* f = CURR ? u.ii : u.vv;
        const float* fo = CURR ? u.iifo : u.vvfo;
        const float* fn = CURR ? u.iifn : u.vvfn;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            c[k] = __ldg(f + k * u.n + loc);
            c[3 + k] = __ldg(fo + k * u.n + loc);
            c[6 + k] = __ldg(fn + k * u.n + loc);
        }
    }
}

// returns region index and local linear offset (without component) or -1
__device__ __forceinline__ int upml_find(const GridDev& g, unsigned x, unsigned y, unsigned z, unsigned& loc)
{
#pragma unroll
    for (int r = 0; r < OEMS_MAX_UPML; ++r) {
        if (r >= g.nupml) break;
        const UpmlDev& u = g.upml[r];
        unsigned lx = x - u.start[0], ly = y - u.start[1], lz = z - u.start[2];
        if (lx < u.nl[0] && ly < u.nl[1] && lz < u.nl[2]) {
            loc = (lx * u.nl[1] + ly) * u.nl[2] + lz;
            return r;
        }
    }
    return -1;
}

// Mur walls (FDTD/extensions/engine_ext_mur_abc.cpp:83-178): wall w updates the two tangential
// components on mesh line `line` of axis ny from the neighbouring line `shift`; the wall
// buffers bP/bPP and tables cP/cPP are indexed k = mur_k(pos[nyP], pos[nyPP]).
struct MurWallDev {
    int ny, nyP, nyPP;
    unsigned line, shift, start_ts, n1, n2;
    const float* cP;
    const float* cPP;
    float* bP;
    float* bPP;
};
struct MurDev {
    int nwall;
    MurWallDev w[OEMS_MAX_MUR];      // insertion order (the apply priority)
    // per axis a: coordinates in [lo[a], lo[a] + span[a]] are no line or shift of a wall with
    // normal a; the walls with normal a are w[order[first[a] .. first[a+1])]
    unsigned lo[3], span[3];
    int first[4];
    int order[OEMS_MAX_MUR];
    // z walls for the lane-parallel form (mur_z_*): nz <= 2 walls with |line - shift| = 1 whose
    // lines and shifts are four distinct z (the host checks this before choosing the form);
    // lanes = 1 while the voltage update runs that form (k_mur then skips the direct columns)
    int nz;
    MurWallDev z[2];
    int lanes;
    // park = 1: the voltage update runs the plain float4 form in the direct columns too, and the
    // z walls' hooks there are k_mur_zsave (before the update) and k_mur_zpost (after it); zsave
    // holds [nz][2][Nx*Ny]: the pre-update Mur value of tangential components 0 and 1
    int park;
    float* zsave;
    // the apply as one flat launch (k_mur_apply, k_vtail): wall wi's points are the blocks
    // [afirst[wi], afirst[wi + 1]); a z wall of the lane-parallel form covers only the columns
    // in zedge (k = x*Ny + y, the columns that are not direct)
    unsigned afirst[OEMS_MAX_MUR + 1];
    const unsigned* zedge;
    unsigned nzedge;
};

// Where the Mur pre and post voltage hooks (engine_ext_mur_abc.cpp:83-149) run: inside the
// voltage update, by the thread of each wall's shift cell,
//   bP = (V_old(shift) - cP * V_old(line)) + cP * V_new(shift),
// with V_new(shift) the cell's own new value before any later hook, exactly what the post hook
// reads.  The update of a line cell leaves the tangential components of every active wall
// unwritten: the wall's apply (k_mur) overwrites them after the dispersive apply hooks, so the
// raw value is never observed, and V_old(line) can still be read from memory by the shift cell
// while the launch runs.

// the index of a wall point in the wall's tables (cP, cPP, bP, bPP), iP / iPP its coordinates
// along nyP / nyPP: z fastest where z is tangential (the host stores those walls' tables
// transposed), so the threads that walk z touch consecutive entries
__device__ __forceinline__ unsigned mur_k(const MurWallDev& d, unsigned iP, unsigned iPP)
{
    return d.nyP == 2 ? iPP * d.n1 + iP : iP * d.n2 + iPP;
}

// true when a coordinate of the cell lies outside its axis window (a possible line or shift);
// NA = 2 checks x and y only
template <int NA = 3>
__device__ __forceinline__ bool mur_wall_cell(const MurDev& m, unsigned x, unsigned y, unsigned z)
{
    bool r = (x - m.lo[0] > m.span[0]) | (y - m.lo[1] > m.span[1]);
    if (NA == 3) r |= (z - m.lo[2] > m.span[2]);
    return r;
}

// The hooks of the walls with normal axis a < NA at one cell; returns the store mask of the
// cell's three components.  Divergent and serial (its loads follow the update's loads): meant
// for cells the caller has found outside the windows.
template <int NA = 3>
__device__ __forceinline__ unsigned mur_cell(const GridDev& g, const MurDev& m, unsigned ts, unsigned x, unsigned y,
                                             unsigned z, unsigned long long o, float vo0, float vo1, float vo2,
                                             float vn0, float vn1, float vn2)
{
    unsigned keep = 7u;
#pragma unroll
    for (int a = 0; a < NA; ++a) {
        const unsigned c = a == 0 ? x : (a == 1 ? y : z);
        if (c - m.lo[a] <= m.span[a]) continue;
        const int aP = (a + 1) % 3, aPP = (a + 2) % 3;
        const unsigned long long stride = a == 0 ? (unsigned long long)g.Ny * g.Pz : (a == 1 ? (unsigned long long)g.Pz : 1ull);
        const float oP = aP == 0 ? vo0 : (aP == 1 ? vo1 : vo2), oPP = aPP == 0 ? vo0 : (aPP == 1 ? vo1 : vo2);
        const float nP = aP == 0 ? vn0 : (aP == 1 ? vn1 : vn2), nPP = aPP == 0 ? vn0 : (aPP == 1 ? vn1 : vn2);
        const unsigned iP = aP == 0 ? x : (aP == 1 ? y : z), iPP = aPP == 0 ? x : (aPP == 1 ? y : z);
        for (int j = m.first[a]; j < m.first[a + 1]; ++j) {
            const MurWallDev& d = m.w[m.order[j]];
            if (ts < d.start_ts) continue;                  // Engine_Ext_Mur_ABC::IsActive
            if (c == d.line) keep &= ~((1u << aP) | (1u << aPP));
            if (c == d.shift) {
                const unsigned long long ol = o + (unsigned long long)((long long)d.line - (long long)d.shift) * stride;
                const unsigned k = mur_k(d, iP, iPP);
                const float lP = g.V[(unsigned long long)aP * g.S + ol];
                const float lPP = g.V[(unsigned long long)aPP * g.S + ol];
                const float cP = __ldg(d.cP + k), cPP = __ldg(d.cPP + k);
                d.bP[k] = fadd(fsub(oP, fmul(cP, lP)), fmul(cP, nP));
                d.bPP[k] = fadd(fsub(oPP, fmul(cPP, lPP)), fmul(cPP, nPP));
            }
        }
    }
    return keep;
}

// Shift-lane form for the z walls (mode 2 of update_v_cell; every wall active from step 0).
// Threads walk z, so a z wall's line and shift cells are neighbouring threads. The thread of the
// shift cell holds V_old(shift) and V_new(shift) in registers, reads V_old(line) from memory (the
// line cell never stores its tangential components, so memory keeps the old value while the
// launch runs; the line is the neighbouring float, in the sector the warp loads anyway) and forms
//   b = (V_old(shift) - cP * V_old(line)) + cP * V_new(shift).
// In a "direct" column -- no x/y wall line or shift there (inside both windows) -- it stores b as
// the line's final value, so the apply has nothing left to do; the dispersive apply hooks skip the
// Mur-owned components (the reference's apply overwrites them). In the other columns it writes
// the wall buffer and k_mur applies it with the edge priorities of the walls. No other thread
// reads the tangential components of a direct column's line cell in the voltage update: x/y wall
// hooks only read cells outside the windows. The tangential components of a z wall are 0 and 1;
// the table index is x*Ny + y.
__device__ __forceinline__ bool mur_z_direct(const MurDev& m, unsigned x, unsigned y)
{
    return (x - m.lo[0] <= m.span[0]) && (y - m.lo[1] <= m.span[1]);
}

// before the update's loads: start the shift thread's coefficient loads into L1 (a prefetch holds
// no register across the update)
__device__ __forceinline__ void mur_z_prefetch(const MurDev& m, unsigned x, unsigned y, unsigned z, unsigned Ny)
{
    const MurWallDev& A = m.z[0];
    const MurWallDev& B = m.z[1];
    const bool sa = m.nz > 0 && z == A.shift, sb = m.nz > 1 && z == B.shift;
    if (sa || sb) {
        const unsigned k = x * Ny + y;
        asm volatile("prefetch.global.L1 [%0];" ::"l"((sb ? B.cP : A.cP) + k));
        asm volatile("prefetch.global.L1 [%0];" ::"l"((sb ? B.cPP : A.cPP) + k));
    }
}

// store mask of a z-wall line cell: its tangential components 0 and 1 are the wall's
__device__ __forceinline__ unsigned mur_z_keep(const MurDev& m, unsigned z)
{
    const bool l = (m.nz > 0 && z == m.z[0].line) || (m.nz > 1 && z == m.z[1].line);
    return l ? 4u : 7u;
}

// the z-wall work of a shift cell (vo = V_old, vn = V_new of its components 0 and 1)
__device__ __forceinline__ void mur_z_shift(const GridDev& g, const MurDev& m, unsigned x, unsigned y, unsigned z,
                                            unsigned long long o, float vo0, float vo1, float vn0, float vn1)
{
    const MurWallDev& A = m.z[0];
    const MurWallDev& B = m.z[1];
    const bool sa = m.nz > 0 && z == A.shift, sb = m.nz > 1 && z == B.shift;
    if (!(sa || sb)) return;
    const MurWallDev& W = sb ? B : A;
    const unsigned long long ol = W.line > W.shift ? o + 1 : o - 1;
    const float l0 = g.V[ol], l1 = g.V[g.S + ol];
    const unsigned k = x * g.Ny + y;
    const float cP = __ldg(W.cP + k), cPP = __ldg(W.cPP + k);
    const float b0 = fadd(fsub(vo0, fmul(cP, l0)), fmul(cP, vn0));
    const float b1 = fadd(fsub(vo1, fmul(cPP, l1)), fmul(cPP, vn1));
    if (mur_z_direct(m, x, y)) {
        g.V[ol] = b0;
        g.V[g.S + ol] = b1;
    } else {
        W.bP[k] = b0;
        W.bPP[k] = b1;
    }
}

// ---------------------------------------------------------------------------------------------
// Engine::UpdateVoltages (FDTD/engine.cpp:110-168) fused with Engine_Ext_UPML pre/post voltage
// updates (FDTD/extensions/engine_ext_upml.cpp:52-137) for one cell (x, y, z < Nz).
// COHERENT: field loads bypass L1 (ld.global.cg). Needed inside persistent launches, where the
// other field was rewritten by other blocks earlier in the same launch; a single-phase launch
// can use the read-only path.
template <bool COHERENT>
__device__ __forceinline__ float ldf(const float* p)
{
    return COHERENT ? __ldcg(p) : __ldg(p);
}

// rk/lk: the cell's UPML region and local offset when the caller knows them (rk = -2: look up).
// MUR: the Mur pre/post hooks of the walls are done here (m, ts = the walls and the step
// number): 1 = every wall by mur_cell, 2 = the z walls by their shift cells (mur_z_*) and the x/y
// walls by mur_cell.
template <bool COMPRESSED, bool UPML, bool COHERENT = false, int MUR = 0, typename IX = unsigned long long>
__device__ __forceinline__ void update_v_cell(const GridDev& g, unsigned x, unsigned y, unsigned z, int rk = -2,
                                              unsigned lk = 0, const MurDev* m = nullptr, unsigned ts = 0)
{
    if (MUR == 2) mur_z_prefetch(*m, x, y, z, g.Ny);
    const IX S = (IX)g.S;
    const IX o = ((IX)x * g.Ny + y) * g.Pz + z;
    const IX sx = x ? (IX)g.Ny * g.Pz : (IX)0;
    const IX sy = y ? (IX)g.Pz : (IX)0;
    const IX sz = z ? (IX)1 : (IX)0;
    const float* __restrict__ I = g.I;
    float* __restrict__ V = g.V;

    const float i0 = ldf<COHERENT>(I + o), i1 = ldf<COHERENT>(I + (S + o)), i2 = ldf<COHERENT>(I + (2 * S + o));
    // curl terms in the reference's evaluation order ((a - b) - c) + d
    const float c0 = fadd(fsub(fsub(i2, ldf<COHERENT>(I + (2 * S + o - sy))), i1), ldf<COHERENT>(I + (S + o - sz)));
    const float c1 = fadd(fsub(fsub(i0, ldf<COHERENT>(I + (o - sz))), i2), ldf<COHERENT>(I + (2 * S + o - sx)));
    const float c2 = fadd(fsub(fsub(i1, ldf<COHERENT>(I + (S + o - sx))), i0), ldf<COHERENT>(I + (o - sy)));

    float vv0, vv1, vv2, vi0, vi1, vi2;
    if (COMPRESSED) {
        const unsigned c = op_cls(g, o);
        const float4 a = __ldg(g.tabV + 2 * c), b = __ldg(g.tabV + 2 * c + 1);
        vv0 = a.x; vv1 = a.y; vv2 = a.z; vi0 = a.w; vi1 = b.x; vi2 = b.y;
    } else {
        vv0 = __ldg(g.vv + o); vv1 = __ldg(g.vv + (S + o)); vv2 = __ldg(g.vv + (2 * S + o));
        vi0 = __ldg(g.vi + o); vi1 = __ldg(g.vi + (S + o)); vi2 = __ldg(g.vi + (2 * S + o));
    }
    float v0, v1, v2;
    if (COHERENT) { v0 = __ldcg(V + o); v1 = __ldcg(V + (S + o)); v2 = __ldcg(V + (2 * S + o)); }
    else { v0 = V[o]; v1 = V[S + o]; v2 = V[2 * S + o]; }

    int r = -1;
    unsigned loc = 0;
    if (UPML) {
        if (rk == -2) r = upml_find(g, x, y, z, loc);
        else { r = rk; loc = lk; }
    }
    float out[3];
    if (UPML && r >= 0) {
        const UpmlDev& u = g.upml[r];
        const unsigned n = u.n;
        float vin[3] = {v0, v1, v2};
        const float cc[3] = {c0, c1, c2};
        const float cvv[3] = {vv0, vv1, vv2};
        const float cvi[3] = {vi0, vi1, vi2};
        float pc[9];
        upml_coef<false>(u, loc, pc);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const unsigned q = k * n + loc;
            const float flux = u.vflux[q];
            // pre: f = vv*V - vvfo*flux; V = flux; flux = f
            const float f = fsub(fmul(pc[k], vin[k]), fmul(pc[3 + k], flux));
            float vn = flux;
            vn = fadd(fmul(vn, cvv[k]), fmul(cvi[k], cc[k]));
            // post: h = flux; flux = V; V = h + vvfn*flux
            u.vflux[q] = vn;
            out[k] = fadd(f, fmul(pc[6 + k], vn));
        }
    } else {
        out[0] = fadd(fmul(v0, vv0), fmul(vi0, c0));
        out[1] = fadd(fmul(v1, vv1), fmul(vi1, c1));
        out[2] = fadd(fmul(v2, vv2), fmul(vi2, c2));
    }
    unsigned keep = 7u;
    if (MUR == 1) keep = mur_cell<3>(g, *m, ts, x, y, z, o, v0, v1, v2, out[0], out[1], out[2]);
    if (MUR == 2) {
        // x/y walls: their hooks read this cell's raw new values
        if (mur_wall_cell<2>(*m, x, y, z)) keep = mur_cell<2>(g, *m, ts, x, y, z, o, v0, v1, v2, out[0], out[1], out[2]);
        keep &= mur_z_keep(*m, z);
        mur_z_shift(g, *m, x, y, z, o, v0, v1, out[0], out[1]);
    }
    if (keep & 1u) V[o] = out[0];
    if (keep & 2u) V[S + o] = out[1];
    if (keep & 4u) V[2 * S + o] = out[2];
}

// Engine::UpdateCurrents (FDTD/engine.cpp:170-222) fused with the UPML current hooks
// (FDTD/extensions/engine_ext_upml.cpp:144-229) for one cell x<Nx-1, y<Ny-1, z<Nz-1.
template <bool COMPRESSED, bool UPML, bool COHERENT = false, typename IX = unsigned long long>
__device__ __forceinline__ void update_i_cell(const GridDev& g, unsigned x, unsigned y, unsigned z, int rk = -2,
                                              unsigned lk = 0)
{
    const IX S = (IX)g.S;
    const IX o = ((IX)x * g.Ny + y) * g.Pz + z;
    const IX sx = (IX)g.Ny * g.Pz;
    const IX sy = g.Pz;
    const float* __restrict__ V = g.V;
    float* __restrict__ I = g.I;

    const float w0 = ldf<COHERENT>(V + o), w1 = ldf<COHERENT>(V + (S + o)), w2 = ldf<COHERENT>(V + (2 * S + o));
    const float c0 = fadd(fsub(fsub(w2, ldf<COHERENT>(V + (2 * S + o + sy))), w1), ldf<COHERENT>(V + (S + o + 1)));
    const float c1 = fadd(fsub(fsub(w0, ldf<COHERENT>(V + (o + 1))), w2), ldf<COHERENT>(V + (2 * S + o + sx)));
    const float c2 = fadd(fsub(fsub(w1, ldf<COHERENT>(V + (S + o + sx))), w0), ldf<COHERENT>(V + (o + sy)));

    float ii0, ii1, ii2, iv0, iv1, iv2;
    if (COMPRESSED) {
        const unsigned c = op_cls(g, o);
        const float4 a = __ldg(g.tabI + 2 * c), b = __ldg(g.tabI + 2 * c + 1);
        ii0 = a.x; ii1 = a.y; ii2 = a.z; iv0 = a.w; iv1 = b.x; iv2 = b.y;
    } else {
        ii0 = __ldg(g.ii + o); ii1 = __ldg(g.ii + (S + o)); ii2 = __ldg(g.ii + (2 * S + o));
        iv0 = __ldg(g.iv + o); iv1 = __ldg(g.iv + (S + o)); iv2 = __ldg(g.iv + (2 * S + o));
    }
    float a0, a1, a2;
    if (COHERENT) { a0 = __ldcg(I + o); a1 = __ldcg(I + (S + o)); a2 = __ldcg(I + (2 * S + o)); }
    else { a0 = I[o]; a1 = I[S + o]; a2 = I[2 * S + o]; }

    int r = -1;
    unsigned loc = 0;
    if (UPML) {
        if (rk == -2) r = upml_find(g, x, y, z, loc);
        else { r = rk; loc = lk; }
    }
    if (UPML && r >= 0) {
        const UpmlDev& u = g.upml[r];
        const unsigned n = u.n;
        float iin[3] = {a0, a1, a2};
        const float cc[3] = {c0, c1, c2};
        const float cii[3] = {ii0, ii1, ii2};
        const float civ[3] = {iv0, iv1, iv2};
        float pc[9];
        upml_coef<true>(u, loc, pc);
        float out[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const unsigned q = k * n + loc;
            const float flux = u.iflux[q];
            const float f = fsub(fmul(pc[k], iin[k]), fmul(pc[3 + k], flux));
            float in = flux;
            in = fadd(fmul(in, cii[k]), fmul(civ[k], cc[k]));
            u.iflux[q] = in;
            out[k] = fadd(f, fmul(pc[6 + k], in));
        }
        I[o] = out[0]; I[S + o] = out[1]; I[2 * S + o] = out[2];
        return;
    }
    I[o] = fadd(fmul(a0, ii0), fmul(iv0, c0));
    I[S + o] = fadd(fmul(a1, ii1), fmul(iv1, c1));
    I[2 * S + o] = fadd(fmul(a2, ii2), fmul(iv2, c2));
}

// One thread per cell of an x-plane (blockIdx.y = x), z fastest for coalescing.
// MUR (the update_v_cell modes): with the Mur pre/post hooks; numTS is the device step counter.
// IX: the type of the cell offsets (32-bit when 3 * S fits, one address instruction per access).
// Mode 2 decides per warp: a warp without a cell outside the wall windows runs the plain update
// (the kernel is issue-bound, so the hooks must cost those warps nothing); in a warp with one,
// only the wall cells' threads do extra work (x/y wall hooks, the z-wall shift thread).  Full
// occupancy needs 32 registers: 8 blocks of 256 threads per SM.
template <bool COMPRESSED, bool UPML, int MUR = 0, typename IX = unsigned long long>
__global__ void __launch_bounds__(256, (MUR == 2 ? 8 : 1)) k_update_v(GridDev g, MurDev m,
                                                                      const unsigned* __restrict__ numTS)
{
    const unsigned x = blockIdx.y;
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned y = t / g.Pz, z = t - y * g.Pz;
    const bool valid = y < g.Ny && z < g.Nz;
    static_assert(!(UPML && MUR == 2), "mode 2 is chosen for meshes without UPML only");
    if (MUR == 2) {
        const bool wall = __any_sync(0xffffffffu, valid && mur_wall_cell(m, x, y, z));
        if (!valid) return;
        if (wall) update_v_cell<COMPRESSED, UPML, false, 2, IX>(g, x, y, z, -2, 0, &m, __ldg(numTS));
        else update_v_cell<COMPRESSED, UPML, false, 0, IX>(g, x, y, z);
        return;
    }
    if (!valid) return;
    if (MUR == 1 && mur_wall_cell(m, x, y, z)) update_v_cell<COMPRESSED, UPML, false, 1, IX>(g, x, y, z, -2, 0, &m, __ldg(numTS));
    else update_v_cell<COMPRESSED, UPML, false, 0, IX>(g, x, y, z);
}

// Vectorised current update of the compressed operator without UPML: one thread per four
// consecutive z cells (a 16-byte aligned float4 of every component; Pz is a multiple of 4).
// The +z neighbours are the same float4 shifted by one lane plus the next float; lanes at or past
// z = Nz-1 keep their loaded value (the reference never updates that line, and the padding stays
// zero).  Per cell the arithmetic is update_i_cell's.
__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ float4 ldg4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }
__device__ __forceinline__ float f4(const float4& v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w)); }
__device__ __forceinline__ void set4(float4& v, int k, float a)
{
    if (k == 0) v.x = a; else if (k == 1) v.y = a; else if (k == 2) v.z = a; else v.w = a;
}

// store the lanes of `mask` (bit k = lane k) of a float4: one vector store when all four are set
__device__ __forceinline__ void st4_masked(float* p, const float4 v, unsigned mask)
{
    if (mask == 15u) {
        *reinterpret_cast<float4*>(p) = v;
        return;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (mask & (1u << k)) p[k] = f4(v, k);
}

// four current cells (x, y, z0..z0+3) of the compressed operator without UPML; only the lanes of
// `mask` are stored (the others belong to another kernel's cells)
template <typename IX = unsigned>
__device__ __forceinline__ void update_i4_cells(const GridDev& g, unsigned x, unsigned y, unsigned z0,
                                                unsigned mask = 15u)
{
    const IX S = (IX)g.S;
    const IX o = ((IX)x * g.Ny + y) * g.Pz + z0;
    const IX sx = (IX)g.Ny * g.Pz;
    const IX sy = g.Pz;
    const float* __restrict__ V = g.V;
    float* __restrict__ I = g.I;
    const float4 w0 = ldg4(V + o), w1 = ldg4(V + (S + o)), w2 = ldg4(V + (2 * S + o));
    const float4 w2y = ldg4(V + (2 * S + o + sy)), w0y = ldg4(V + (o + sy));
    const float4 w2x = ldg4(V + (2 * S + o + sx)), w1x = ldg4(V + (S + o + sx));
    const float w0z4 = __ldg(V + (o + 4)), w1z4 = __ldg(V + (S + o + 4));
    const uint4 ci = op_cls4(g, o);
    float4 a0 = ld4(I + o), a1 = ld4(I + (S + o)), a2 = ld4(I + (2 * S + o));
    const unsigned cls[4] = {ci.x, ci.y, ci.z, ci.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (z0 + k + 1 >= g.Nz) break;
        const float4 ca = __ldg(g.tabI + 2 * cls[k]), cb = __ldg(g.tabI + 2 * cls[k] + 1);
        const float v1z = k < 3 ? f4(w1, k + 1) : w1z4, v0z = k < 3 ? f4(w0, k + 1) : w0z4;
        const float c0 = fadd(fsub(fsub(f4(w2, k), f4(w2y, k)), f4(w1, k)), v1z);
        const float c1 = fadd(fsub(fsub(f4(w0, k), v0z), f4(w2, k)), f4(w2x, k));
        const float c2 = fadd(fsub(fsub(f4(w1, k), f4(w1x, k)), f4(w0, k)), f4(w0y, k));
        set4(a0, k, fadd(fmul(f4(a0, k), ca.x), fmul(ca.w, c0)));
        set4(a1, k, fadd(fmul(f4(a1, k), ca.y), fmul(cb.x, c1)));
        set4(a2, k, fadd(fmul(f4(a2, k), ca.z), fmul(cb.y, c2)));
    }
    st4_masked(I + o, a0, mask);
    st4_masked(I + (S + o), a1, mask);
    st4_masked(I + (2 * S + o), a2, mask);
}

template <typename IX = unsigned>
__global__ void __launch_bounds__(256) k_update_i4(GridDev g)
{
    const unsigned x = blockIdx.y;
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned pz4 = g.Pz >> 2;
    const unsigned y = t / pz4, z0 = (t - y * pz4) << 2;
    if (y + 1 >= g.Ny || z0 + 1 >= g.Nz) return;
    update_i4_cells<IX>(g, x, y, z0);
}

// Vectorised voltage update of the compressed operator without UPML and without Mur walls, four
// consecutive z cells per thread (see k_update_i4).  The -z neighbour of lane k is lane k-1, of
// lane 0 the float before the vector (the cell itself at z = 0, the reference's "same cell"
// read).  Lanes past z = Nz-1 are padding and keep their zero.  (With Mur walls the one-cell form
// carrying the hooks stays the faster choice on GB300: a float4 update with the z walls' hooks in
// the registers of the wall thread measured 94 us against 78 us without walls on 256x256x192,
// every warp holding one wall thread, and a register spill or an exposed coefficient load with it.)
// four voltage cells (x, y, z0..z0+3) of the compressed operator without UPML and Mur hooks;
// only the lanes of `mask` are stored
// Optional output of the voltage update for the reverse sweep's recomputation: V^n and K_V I^n of
// the cells of a design box, into slot (*counter % modulo) of `base` (each slot [2][3][B]: V, then
// K_V I; design cell kb = (bx * bn[1] + by) * bn[2] + bz), exactly the values the update uses.
struct FacOut {
    float* base;
    const unsigned* counter;
    unsigned modulo;
    unsigned b0[3], bn[3], B;
    unsigned coff;               // the slot is (*counter + coff) % modulo
};

template <typename IX = unsigned, bool FAC = false>
__device__ __forceinline__ void update_v4_cells(const GridDev& g, unsigned x, unsigned y, unsigned z0,
                                                unsigned mask = 15u, const FacOut* fo = nullptr)
{
    const IX S = (IX)g.S;
    const IX o = ((IX)x * g.Ny + y) * g.Pz + z0;
    const IX sx = x ? (IX)g.Ny * g.Pz : (IX)0;
    const IX sy = y ? (IX)g.Pz : (IX)0;
    const float* __restrict__ I = g.I;
    float* __restrict__ V = g.V;
    const float4 i0 = ldg4(I + o), i1 = ldg4(I + (S + o)), i2 = ldg4(I + (2 * S + o));
    const float4 i2y = ldg4(I + (2 * S + o - sy)), i0y = ldg4(I + (o - sy));
    const float4 i2x = ldg4(I + (2 * S + o - sx)), i1x = ldg4(I + (S + o - sx));
    // the float before the vector; at z = 0 the cell's own value
    const float i1m = z0 ? __ldg(I + (S + o - 1)) : i1.x, i0m = z0 ? __ldg(I + (o - 1)) : i0.x;
    const uint4 ci = op_cls4(g, o);
    float4 n0 = ld4(V + o), n1 = ld4(V + (S + o)), n2 = ld4(V + (2 * S + o));
    const unsigned cls[4] = {ci.x, ci.y, ci.z, ci.w};
    // FAC: this row's design cells (the box's rows are x, y inside it; lanes z inside it)
    const unsigned fbx = x - (FAC ? fo->b0[0] : 0u), fby = y - (FAC ? fo->b0[1] : 0u);
    const bool frow = FAC && fbx < fo->bn[0] && fby < fo->bn[1];
    float* fslot = nullptr;
    if (frow) fslot = fo->base + (size_t)((__ldg(fo->counter) + fo->coff) % fo->modulo) * 6u * fo->B;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (z0 + k >= g.Nz) break;
        const float4 ca = __ldg(g.tabV + 2 * cls[k]), cb = __ldg(g.tabV + 2 * cls[k] + 1);
        const float i1z = k ? f4(i1, k - 1) : i1m, i0z = k ? f4(i0, k - 1) : i0m;
        const float c0 = fadd(fsub(fsub(f4(i2, k), f4(i2y, k)), f4(i1, k)), i1z);
        const float c1 = fadd(fsub(fsub(f4(i0, k), i0z), f4(i2, k)), f4(i2x, k));
        const float c2 = fadd(fsub(fsub(f4(i1, k), f4(i1x, k)), f4(i0, k)), f4(i0y, k));
        if (frow) {
            const unsigned bz = z0 + k - fo->b0[2];
            if (bz < fo->bn[2] && (mask & (1u << k))) {
                const unsigned kb = (fbx * fo->bn[1] + fby) * fo->bn[2] + bz, B = fo->B;
                fslot[kb] = f4(n0, k);
                fslot[B + kb] = f4(n1, k);
                fslot[2 * B + kb] = f4(n2, k);
                fslot[3 * B + kb] = c0;
                fslot[4 * B + kb] = c1;
                fslot[5 * B + kb] = c2;
            }
        }
        set4(n0, k, fadd(fmul(f4(n0, k), ca.x), fmul(ca.w, c0)));
        set4(n1, k, fadd(fmul(f4(n1, k), ca.y), fmul(cb.x, c1)));
        set4(n2, k, fadd(fmul(f4(n2, k), ca.z), fmul(cb.y, c2)));
    }
    st4_masked(V + o, n0, mask);
    st4_masked(V + (S + o), n1, mask);
    st4_masked(V + (2 * S + o), n2, mask);
}

template <typename IX = unsigned>
__global__ void __launch_bounds__(256) k_update_v4(GridDev g)
{
    const unsigned x = blockIdx.y;
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned pz4 = g.Pz >> 2;
    const unsigned y = t / pz4, z0 = (t - y * pz4) << 2;
    if (y >= g.Ny || z0 >= g.Nz) return;
    update_v4_cells<IX>(g, x, y, z0);
}

// Four cells (x, y, z0..z0+3) of a column on an x/y wall line or shift: the float4 update, then
// per lane the hooks of mode 2 (mur_cell for the x/y walls, mur_z_keep / mur_z_shift for the z
// walls) on the lane's old and new values, and a store of the lanes and components the hooks
// leave to this update.  The lines' tangential components stay unwritten, so the shift lanes
// (of other threads, and of this one for a z wall) read their old values from memory.
template <typename IX = unsigned>
__device__ __forceinline__ void mur_wall_v4(const GridDev& g, const MurDev& m, unsigned ts, unsigned x, unsigned y,
                                            unsigned z0)
{
    const IX S = (IX)g.S;
    const IX o = ((IX)x * g.Ny + y) * g.Pz + z0;
    const IX sx = x ? (IX)g.Ny * g.Pz : (IX)0;
    const IX sy = y ? (IX)g.Pz : (IX)0;
    const float* __restrict__ I = g.I;
    float* __restrict__ V = g.V;
    const float4 i0 = ldg4(I + o), i1 = ldg4(I + (S + o)), i2 = ldg4(I + (2 * S + o));
    const float4 i2y = ldg4(I + (2 * S + o - sy)), i0y = ldg4(I + (o - sy));
    const float4 i2x = ldg4(I + (2 * S + o - sx)), i1x = ldg4(I + (S + o - sx));
    const float i1m = z0 ? __ldg(I + (S + o - 1)) : i1.x, i0m = z0 ? __ldg(I + (o - 1)) : i0.x;
    const uint4 ci = op_cls4(g, o);
    const float4 v0 = ld4(V + o), v1 = ld4(V + (S + o)), v2 = ld4(V + (2 * S + o));
    float4 n0 = v0, n1 = v1, n2 = v2;
    const unsigned cls[4] = {ci.x, ci.y, ci.z, ci.w};
    unsigned m0 = 15u, m1 = 15u, m2 = 15u;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (z0 + k >= g.Nz) break;
        const float4 ca = __ldg(g.tabV + 2 * cls[k]), cb = __ldg(g.tabV + 2 * cls[k] + 1);
        const float i1z = k ? f4(i1, k - 1) : i1m, i0z = k ? f4(i0, k - 1) : i0m;
        const float c0 = fadd(fsub(fsub(f4(i2, k), f4(i2y, k)), f4(i1, k)), i1z);
        const float c1 = fadd(fsub(fsub(f4(i0, k), i0z), f4(i2, k)), f4(i2x, k));
        const float c2 = fadd(fsub(fsub(f4(i1, k), f4(i1x, k)), f4(i0, k)), f4(i0y, k));
        set4(n0, k, fadd(fmul(f4(v0, k), ca.x), fmul(ca.w, c0)));
        set4(n1, k, fadd(fmul(f4(v1, k), ca.y), fmul(cb.x, c1)));
        set4(n2, k, fadd(fmul(f4(v2, k), ca.z), fmul(cb.y, c2)));
        const unsigned z = z0 + k;
        unsigned keep = mur_cell<2>(g, m, ts, x, y, z, (unsigned long long)o + k, f4(v0, k), f4(v1, k), f4(v2, k),
                                    f4(n0, k), f4(n1, k), f4(n2, k));
        keep &= mur_z_keep(m, z);
        mur_z_shift(g, m, x, y, z, (unsigned long long)o + k, f4(v0, k), f4(v1, k), f4(n0, k), f4(n1, k));
        if (!(keep & 1u)) m0 &= ~(1u << k);
        if (!(keep & 2u)) m1 &= ~(1u << k);
        if (!(keep & 4u)) m2 &= ~(1u << k);
    }
    st4_masked(V + o, n0, m0);                  // lanes past Nz-1 are padding: they keep their zero
    st4_masked(V + (S + o), n1, m1);
    st4_masked(V + (2 * S + o), n2, m2);
}

// the z wall whose line lies in the group of four z starting at z0, or -1
__device__ __forceinline__ int mur_z_group(const MurDev& m, unsigned z0)
{
    if (m.nz > 0 && (m.z[0].line >> 2) == (z0 >> 2)) return 0;
    if (m.nz > 1 && (m.z[1].line >> 2) == (z0 >> 2)) return 1;
    return -1;
}

// The group of four z holding z wall q's line and shift in a direct column (inside both x/y
// windows): the float4 update, with the wall's hooks on registers.  The thread has V_old(line),
// V_old(shift) and V_new(shift) and forms
//     b = (V_old(shift) - cP * V_old(line)) + cP * V_new(shift)
// as the line's final tangential values, in the same float4 store (no wall buffer).
template <typename IX = unsigned>
__device__ __forceinline__ void mur_zwall_v4(const GridDev& g, const MurDev& m, unsigned x, unsigned y, unsigned q)
{
    const MurWallDev& W = q ? m.z[1] : m.z[0];
    const unsigned z0 = W.line & ~3u;
    const int kl = (int)(W.line - z0), ks = (int)(W.shift - z0);
    const unsigned kc = x * g.Ny + y;
    const float cP = __ldg(W.cP + kc), cPP = __ldg(W.cPP + kc);
    const IX S = (IX)g.S;
    const IX o = ((IX)x * g.Ny + y) * g.Pz + z0;
    const IX sx = x ? (IX)g.Ny * g.Pz : (IX)0;
    const IX sy = y ? (IX)g.Pz : (IX)0;
    const float* __restrict__ I = g.I;
    float* __restrict__ V = g.V;
    const float4 i0 = ldg4(I + o), i1 = ldg4(I + (S + o)), i2 = ldg4(I + (2 * S + o));
    const float4 i2y = ldg4(I + (2 * S + o - sy)), i0y = ldg4(I + (o - sy));
    const float4 i2x = ldg4(I + (2 * S + o - sx)), i1x = ldg4(I + (S + o - sx));
    const float i1m = z0 ? __ldg(I + (S + o - 1)) : i1.x, i0m = z0 ? __ldg(I + (o - 1)) : i0.x;
    const uint4 ci = op_cls4(g, o);
    float4 n0 = ld4(V + o), n1 = ld4(V + (S + o)), n2 = ld4(V + (2 * S + o));
    // pre-voltage part, from the old values
    const float pre0 = fsub(f4(n0, ks), fmul(cP, f4(n0, kl)));
    const float pre1 = fsub(f4(n1, ks), fmul(cPP, f4(n1, kl)));
    const unsigned cls[4] = {ci.x, ci.y, ci.z, ci.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (z0 + k >= g.Nz) break;
        const float4 ca = __ldg(g.tabV + 2 * cls[k]), cb = __ldg(g.tabV + 2 * cls[k] + 1);
        const float i1z = k ? f4(i1, k - 1) : i1m, i0z = k ? f4(i0, k - 1) : i0m;
        const float c0 = fadd(fsub(fsub(f4(i2, k), f4(i2y, k)), f4(i1, k)), i1z);
        const float c1 = fadd(fsub(fsub(f4(i0, k), i0z), f4(i2, k)), f4(i2x, k));
        const float c2 = fadd(fsub(fsub(f4(i1, k), f4(i1x, k)), f4(i0, k)), f4(i0y, k));
        set4(n0, k, fadd(fmul(f4(n0, k), ca.x), fmul(ca.w, c0)));
        set4(n1, k, fadd(fmul(f4(n1, k), ca.y), fmul(cb.x, c1)));
        set4(n2, k, fadd(fmul(f4(n2, k), ca.z), fmul(cb.y, c2)));
    }
    // post-voltage part and the apply of a direct column
    set4(n0, kl, fadd(pre0, fmul(cP, f4(n0, ks))));
    set4(n1, kl, fadd(pre1, fmul(cPP, f4(n1, ks))));
    *reinterpret_cast<float4*>(V + o) = n0;     // lanes past Nz-1 are padding: they keep their zero
    *reinterpret_cast<float4*>(V + (S + o)) = n1;
    *reinterpret_cast<float4*>(V + (2 * S + o)) = n2;
}

// k_update_v4 with the Mur walls' pre/post voltage hooks (FDTD/extensions/engine_ext_mur_abc.cpp:
// 83-149) in the lane-parallel form (MurDev::lanes: every wall active from step 0).  The host
// chooses it when each z wall's line and shift lie in one group of four z and no group holds
// two walls.  The first `interior` blocks of a plane map its groups as k_update_v4 does:
// - a column on an x/y wall line or shift (outside the windows: whole rows and planes, so whole
//   warps) runs mur_wall_v4: the float4 update with mode 2's hooks lane by lane;
// - in every other (direct) column, a group holding a z wall's line is left to the wall blocks,
//   and the others run the plain float4 update, which then carries no hook code at all.
// The blocks after them take one direct column's z-wall group per thread (mur_zwall_v4).  The
// wall work thus sits in warps of its own, and the streaming warps keep k_update_v4's registers
// and loads in flight.
// PARK: the direct columns' z-wall groups are updated like every other group (their hooks are
// k_mur_zsave / k_mur_zpost around this launch), so the streaming blocks carry no wall test and
// there are no wall blocks.
template <typename IX = unsigned, bool PARK = false>
__global__ void __launch_bounds__(256, 4) k_update_v4w(GridDev g, MurDev m, const unsigned* __restrict__ numTS,
                                                       unsigned interior)
{
    const unsigned x = blockIdx.y;
    if (blockIdx.x < interior) {
        const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
        const unsigned pz4 = g.Pz >> 2;
        const unsigned y = t / pz4, z0 = (t - y * pz4) << 2;
        if (y >= g.Ny || z0 >= g.Nz) return;
        if (mur_wall_cell<2>(m, x, y, 0u)) {
            mur_wall_v4<IX>(g, m, __ldg(numTS), x, y, z0);
            return;
        }
        if (!PARK && mur_z_group(m, z0) >= 0) return;
        update_v4_cells<IX>(g, x, y, z0);
        return;
    }
    if (PARK) return;
    const unsigned t = (blockIdx.x - interior) * blockDim.x + threadIdx.x;
    const unsigned nz = (unsigned)m.nz;
    const unsigned y = t / nz, q = t - y * nz;
    if (y >= g.Ny || mur_wall_cell<2>(m, x, y, 0u)) return;
    mur_zwall_v4<IX>(g, m, x, y, q);
}

template <bool COMPRESSED, bool UPML, typename IX = unsigned long long>
__global__ void __launch_bounds__(256) k_update_i(GridDev g)
{
    const unsigned x = blockIdx.y;
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned y = t / g.Pz, z = t - y * g.Pz;
    if (y + 1 >= g.Ny || z + 1 >= g.Nz) return;
    update_i_cell<COMPRESSED, UPML, false, IX>(g, x, y, z);
}

// Work split for meshes with UPML regions: the first blocks map the cells of each region in
// region order, the following blocks the cells outside every region (a box when the regions are
// boundary slabs, else the whole range with UPML cells skipped).  Every warp then runs one code
// path, and region cells read their fluxes with region-local coalesced offsets.  The region blocks
// come first because they carry the longer dependent load chains (class index, then the class
// table, then the fluxes): started first, they overlap with the streaming main blocks instead of
// forming the launch's tail.  With v4 the host launches only the region blocks of this kernel and
// then walks the main box with k_update_box4, four z cells per thread (the float4 bodies of the
// plain kernels, in groups aligned to four z): the two need different register budgets.
struct SplitDev {
    unsigned lo[3], n[3];                      // main part: this box of cells
    unsigned main_cells, main_blocks;
    int full;                                  // 1: the box is the whole update range, skip UPML cells
    int v4;                                    // 1: main box four z cells per thread (k_update_box4)
    unsigned z4, n4;                           // first z of the groups of four, groups per row
    unsigned main_cells4, main_blocks4;        // groups of four and their blocks when v4
    unsigned nreg;
    unsigned first_block[OEMS_MAX_UPML + 1];   // region r: blocks [first_block[r], first_block[r+1])
    int reg4;                                  // 1: the regions four z cells per thread (k_update_reg4)
    unsigned first4[OEMS_MAX_UPML + 1];        // region r: its blocks of groups of four (256 threads)
    unsigned first4h[OEMS_MAX_UPML + 1];       // the same for blocks of 128 threads
};

// The compressed-operator form without Mur hooks fits 32 registers (a few bytes spill to L1), so
// 8 blocks of 256 threads share an SM; the latency-bound split launches gain from the extra warps.
template <bool COMPRESSED, bool CURR, bool MUR = false>
__global__ void __launch_bounds__(256, (COMPRESSED && !MUR) ? 8 : 1)
    k_update_split(GridDev g, SplitDev sp, MurDev m, const unsigned* __restrict__ numTS)
{
    unsigned b = blockIdx.x;
    const unsigned rblocks = sp.first_block[sp.nreg];
    if (b >= rblocks) {
        b -= rblocks;
        unsigned t = b * 256u + threadIdx.x;
        if (t >= sp.main_cells) return;
        const unsigned z = sp.lo[2] + t % sp.n[2];
        t /= sp.n[2];
        const unsigned y = sp.lo[1] + t % sp.n[1];
        const unsigned x = sp.lo[0] + t / sp.n[1];
        if (sp.full) {
            unsigned loc;
            if (upml_find(g, x, y, z, loc) >= 0) return;
        }
        if (CURR) update_i_cell<COMPRESSED, false>(g, x, y, z);
        else if (MUR && mur_wall_cell(m, x, y, z)) update_v_cell<COMPRESSED, false, false, 1>(g, x, y, z, -2, 0, &m, __ldg(numTS));
        else update_v_cell<COMPRESSED, false>(g, x, y, z);
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
        update_i_cell<COMPRESSED, true>(g, x, y, z, r, loc);
    } else {
        if (MUR && mur_wall_cell(m, x, y, z)) update_v_cell<COMPRESSED, true, false, 1>(g, x, y, z, r, loc, &m, __ldg(numTS));
        else update_v_cell<COMPRESSED, true>(g, x, y, z, r, loc);
    }
}

// The main box of a UPML split, four z cells per thread (compressed operator, no Mur hooks).
// Groups of four start on multiples of four (z4 = lo[2] rounded down); lanes outside the box's
// z range are computed but not stored (their cells belong to the region blocks).
// FAC (voltage update only): also the design-box factors of the reverse sweep's recomputation
template <bool CURR, bool FAC = false>
__global__ void __launch_bounds__(256, 4) k_update_box4(GridDev g, SplitDev sp, FacOut fo = FacOut{})
{
    unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= sp.main_cells4) return;
    const unsigned z = sp.z4 + ((t % sp.n4) << 2);
    t /= sp.n4;
    const unsigned y = sp.lo[1] + t % sp.n[1];
    const unsigned x = sp.lo[0] + t / sp.n[1];
    const unsigned zlo = sp.lo[2], zhi = sp.lo[2] + sp.n[2];
    unsigned mask = 0u;
#pragma unroll
    for (int k = 0; k < 4; ++k) mask |= (z + k >= zlo && z + k < zhi) ? (1u << k) : 0u;
    if (CURR) update_i4_cells<unsigned>(g, x, y, z, mask);
    else update_v4_cells<unsigned, FAC>(g, x, y, z, mask, &fo);
}

// Region-local arrays (fluxes, classes) in the float4 region kernels: a group's four lanes are
// four consecutive local offsets starting at p (lane 0).  When the region's z rows start and end
// on multiples of four (`vec`) they are one aligned vector; otherwise the lanes of `mask` are
// read and written one by one (p may then point before the row: masked lanes are not touched).
__device__ __forceinline__ float4 ld_lanes(const float* p, bool vec, unsigned mask)
{
    if (vec) return ld4(p);
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (mask & 1u) v.x = p[0];
    if (mask & 2u) v.y = p[1];
    if (mask & 4u) v.z = p[2];
    if (mask & 8u) v.w = p[3];
    return v;
}

__device__ __forceinline__ void st_lanes(float* p, const float4 v, bool vec, unsigned mask)
{
    if (vec && mask == 15u) {
        *reinterpret_cast<float4*>(p) = v;
        return;
    }
    if (mask & 1u) p[0] = v.x;
    if (mask & 2u) p[1] = v.y;
    if (mask & 4u) p[2] = v.z;
    if (mask & 8u) p[3] = v.w;
}

__device__ __forceinline__ void ld_cls(const unsigned short* p, bool vec, unsigned mask, unsigned c[4])
{
    if (vec) {
        const ushort4 u = __ldg(reinterpret_cast<const ushort4*>(p));
        c[0] = u.x; c[1] = u.y; c[2] = u.z; c[3] = u.w;
        return;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) c[k] = (mask & (1u << k)) ? __ldg(p + k) : 0u;
}

// A UPML region's groups of four z (aligned to multiples of four in the mesh, like the main box):
// groups per z row, and the group `j` of the region as (x, y, z0, local offset of lane 0, lane
// mask of the cells inside the region)
struct RegGroup {
    unsigned x, y, z0, mask;
    int loc0;
    bool vec;
};

__device__ __forceinline__ unsigned reg_groups_per_row(const UpmlDev& u)
{
    const unsigned zs = u.start[2], ze = zs + u.nl[2];
    return (((ze + 3u) & ~3u) - (zs & ~3u)) >> 2;
}

__device__ __forceinline__ RegGroup reg_group(const UpmlDev& u, unsigned j)
{
    const unsigned ngz = reg_groups_per_row(u);
    const unsigned row = j / ngz, gz = j - row * ngz;
    const unsigned zs = u.start[2], ze = zs + u.nl[2];
    RegGroup q;
    q.z0 = (zs & ~3u) + (gz << 2);
    q.x = u.start[0] + row / u.nl[1];
    q.y = u.start[1] + row % u.nl[1];
    q.mask = 0u;
#pragma unroll
    for (int k = 0; k < 4; ++k) q.mask |= (q.z0 + k >= zs && q.z0 + k < ze) ? (1u << k) : 0u;
    q.loc0 = (int)(row * u.nl[2]) + (int)q.z0 - (int)zs;
    q.vec = (zs % 4u == 0u) && (u.nl[2] % 4u == 0u);
    return q;
}

// The UPML regions four z cells per thread: update_v_cell / update_i_cell's UPML branch lane by
// lane.  Groups are aligned to multiples of four z in the mesh, so every field and class-index
// load is a 16-byte vector; lanes outside the region are computed on the side and not stored
// (they belong to another region or the main box), and the region-local fluxes and classes are
// vectors when the region's z rows are whole groups (ld_lanes).  Current lanes at z = Nz-1 (and
// groups at x = Nx-1 or y = Ny-1) are not updated, as in the one-cell form.
// Three blocks of 256 per SM (80 registers, a few bytes spilled) measured 2 % faster than two
// blocks at 98 registers on the 512x512x256 and 200x200x100 UPML meshes.
template <bool CURR>
__global__ void __launch_bounds__(256, 3) k_update_reg4(const __grid_constant__ GridDev g, const __grid_constant__ SplitDev sp)
{
    const unsigned b = blockIdx.x;
    const unsigned* fblk = blockDim.x == 128u ? sp.first4h : sp.first4;
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
    float* __restrict__ flux = CURR ? u.iflux : u.vflux;
    float* const f0p = flux + q.loc0;
    float4 fl0 = ld_lanes(f0p, q.vec, mask), fl1 = ld_lanes(f0p + n, q.vec, mask), fl2 = ld_lanes(f0p + 2 * n, q.vec, mask);
    float4 c0v, c1v, c2v;                       // curls, lane by lane
    float4 a0, a1, a2;                          // the field being updated
    float* __restrict__ F;
    if (CURR) {
        const float* __restrict__ V = g.V;
        F = g.I;
        const unsigned sx = g.Ny * g.Pz, sy = g.Pz;
        const float4 w0 = ldg4(V + o), w1 = ldg4(V + (S + o)), w2 = ldg4(V + (2 * S + o));
        const float4 w2y = ldg4(V + (2 * S + o + sy)), w0y = ldg4(V + (o + sy));
        const float4 w2x = ldg4(V + (2 * S + o + sx)), w1x = ldg4(V + (S + o + sx));
        const float w0z4 = z0 + 4 < g.Pz ? __ldg(V + (o + 4)) : 0.f, w1z4 = z0 + 4 < g.Pz ? __ldg(V + (S + o + 4)) : 0.f;
        a0 = ld4(F + o); a1 = ld4(F + (S + o)); a2 = ld4(F + (2 * S + o));
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float v1z = k < 3 ? f4(w1, k + 1) : w1z4, v0z = k < 3 ? f4(w0, k + 1) : w0z4;
            set4(c0v, k, fadd(fsub(fsub(f4(w2, k), f4(w2y, k)), f4(w1, k)), v1z));
            set4(c1v, k, fadd(fsub(fsub(f4(w0, k), v0z), f4(w2, k)), f4(w2x, k)));
            set4(c2v, k, fadd(fsub(fsub(f4(w1, k), f4(w1x, k)), f4(w0, k)), f4(w0y, k)));
        }
    } else {
        const float* __restrict__ I = g.I;
        F = g.V;
        const unsigned sx = x ? g.Ny * g.Pz : 0u, sy = y ? g.Pz : 0u;
        const float4 i0 = ldg4(I + o), i1 = ldg4(I + (S + o)), i2 = ldg4(I + (2 * S + o));
        const float4 i2y = ldg4(I + (2 * S + o - sy)), i0y = ldg4(I + (o - sy));
        const float4 i2x = ldg4(I + (2 * S + o - sx)), i1x = ldg4(I + (S + o - sx));
        const float i1m = z0 ? __ldg(I + (S + o - 1)) : i1.x, i0m = z0 ? __ldg(I + (o - 1)) : i0.x;
        a0 = ld4(F + o); a1 = ld4(F + (S + o)); a2 = ld4(F + (2 * S + o));
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float i1z = k ? f4(i1, k - 1) : i1m, i0z = k ? f4(i0, k - 1) : i0m;
            set4(c0v, k, fadd(fsub(fsub(f4(i2, k), f4(i2y, k)), f4(i1, k)), i1z));
            set4(c1v, k, fadd(fsub(fsub(f4(i0, k), i0z), f4(i2, k)), f4(i2x, k)));
            set4(c2v, k, fadd(fsub(fsub(f4(i1, k), f4(i1x, k)), f4(i0, k)), f4(i0y, k)));
        }
    }
    const unsigned cls[4] = {ci.x, ci.y, ci.z, ci.w};
    const float4* tab = CURR ? g.tabI : g.tabV;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (!(mask & (1u << k))) continue;
        const float4 ca = __ldg(tab + 2 * cls[k]), cb = __ldg(tab + 2 * cls[k] + 1);
        const float4* t = u.ctab + 6u * ucl[k] + (CURR ? 3 : 0);
        const float4 pa = __ldg(t), pb = __ldg(t + 1), pd = __ldg(t + 2);
        const float pc[9] = {pa.x, pa.y, pa.z, pa.w, pb.x, pb.y, pb.z, pb.w, pd.x};
        const float cvv[3] = {ca.x, ca.y, ca.z}, cvi[3] = {ca.w, cb.x, cb.y};
        const float fin[3] = {f4(a0, k), f4(a1, k), f4(a2, k)};
        const float cc[3] = {f4(c0v, k), f4(c1v, k), f4(c2v, k)};
        const float fx[3] = {f4(fl0, k), f4(fl1, k), f4(fl2, k)};
        float out[3], nf[3];
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            // pre: f = c*F - fo*flux; F = flux; flux = f.  update.  post: h = flux; flux = F; F = h + fn*flux
            const float f = fsub(fmul(pc[m], fin[m]), fmul(pc[3 + m], fx[m]));
            nf[m] = fadd(fmul(fx[m], cvv[m]), fmul(cvi[m], cc[m]));
            out[m] = fadd(f, fmul(pc[6 + m], nf[m]));
        }
        set4(a0, k, out[0]); set4(a1, k, out[1]); set4(a2, k, out[2]);
        set4(fl0, k, nf[0]); set4(fl1, k, nf[1]); set4(fl2, k, nf[2]);
    }
    st4_masked(F + o, a0, mask);
    st4_masked(F + (S + o), a1, mask);
    st4_masked(F + (2 * S + o), a2, mask);
    st_lanes(f0p, fl0, q.vec, mask);
    st_lanes(f0p + n, fl1, q.vec, mask);
    st_lanes(f0p + 2 * n, fl2, q.vec, mask);
}

// ---------------------------------------------------------------------------------------------
// Engine_Ext_Excitation::Apply2VoltagesImpl / Apply2CurrentImpl
// (FDTD/extensions/engine_ext_excitation.cpp:33-94).  One thread per source edge; the source
// edges are distinct so the adds do not race.  numTS is the device step counter.
struct ExcDev {
    unsigned count;
    const unsigned long long* off;   // linear field offset incl. component
    const float* amp;
    const unsigned* delay;
    const float* sig;
    unsigned length;
    unsigned period;                 // 0 = aperiodic
};

__device__ __forceinline__ void exc_point(float* __restrict__ F, const ExcDev& e, unsigned k, unsigned numTS)
{
    if (k >= e.count) return;
    const int ts = (int)numTS;
    const int p = e.period ? (int)e.period : ts + 1;
    int exc_pos = ts - (int)e.delay[k];
    exc_pos *= (exc_pos > 0);
    exc_pos %= p;
    exc_pos *= (exc_pos < (int)e.length);
    const unsigned long long o = e.off[k];
    F[o] = fadd(F[o], fmul(e.amp[k], e.sig[exc_pos]));
}

// toff: added to the step counter (steps of a captured run whose counter moves once at its end)
static __global__ void k_excitation(float* __restrict__ F, ExcDev e, const unsigned* __restrict__ numTS,
                                    unsigned toff = 0)
{
    exc_point(F, e, blockIdx.x * blockDim.x + threadIdx.x, *numTS + toff);
}

// ---------------------------------------------------------------------------------------------
// Engine_Ext_TFSF::DoPostVoltageUpdates / DoPostCurrentUpdates (engine_ext_tfsf.cpp:36-215): the
// incident plane wave added on the faces of the total-field box.  The host groups the reference's
// term list by target cell (terms of one cell keep their reference order; at most one term per
// face plane tangential to the component), so one thread owns one cell and no two threads touch
// the same value.  The arithmetic follows the reference's C++ promotion exactly:
//   V + (1.0 - dd)*amp*sig[a]   (double)   + dd*amp*sig[b]   (float product, added in double)
// and the sum is rounded to float once per term, as each SetVolt/SetCurr stores a float.
struct TfsfDev {
    unsigned ntarget;
    const unsigned long long* off;   // linear field offset (component included) of each target
    const unsigned* first;           // terms of target k: [first[k], first[k+1])
    const unsigned* delay;
    const float* delta;
    const float* amp;
    const float* sig;                // current signal in the voltage hook, voltage signal in the current hook
    unsigned length;
    unsigned period;                 // 0 = aperiodic
};

// m_DelayLookup[d] of the reference for the step numTS = ts
__device__ __forceinline__ unsigned tfsf_lookup(unsigned ts, unsigned d, unsigned length, unsigned period)
{
    unsigned v;
    if (ts < d) v = 0;
    else if (ts - d >= length && period == 0) v = 0;
    else v = ts - d;
    if (period > 0) v %= period;
    return v;
}

static __global__ void k_tfsf(float* __restrict__ F, TfsfDev t, const unsigned* __restrict__ numTS)
{
    const unsigned k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= t.ntarget) return;
    const unsigned ts = *numTS;
    const unsigned long long o = t.off[k];
    float v = F[o];
    const unsigned q1 = t.first[k + 1];
    for (unsigned q = t.first[k]; q < q1; ++q) {
        const unsigned d = t.delay[q];
        const float dd = t.delta[q], a = t.amp[q];
        const float s0 = t.sig[tfsf_lookup(ts, d, t.length, t.period)];
        const float s1 = t.sig[tfsf_lookup(ts, d + 1, t.length, t.period)];
        const double A = __dmul_rn(__dmul_rn(__dsub_rn(1.0, (double)dd), (double)a), (double)s0);
        const float B = __fmul_rn(__fmul_rn(dd, a), s1);
        v = __double2float_rn(__dadd_rn(__dadd_rn((double)v, A), (double)B));
    }
    F[o] = v;
}

// ---------------------------------------------------------------------------------------------
// Engine_Ext_LumpedRLC (FDTD/extensions/engine_ext_lumpedRLC.cpp:80-147): series RLC and parallel
// RLC loads as an auxiliary differential equation per lumped edge.  The reference's pre-voltage
// hook only advances the parallel inductor current from the previous step's node voltage, and
// nothing else touches that state between the two hooks, so one launch after the voltage update
// (in the apply slot) does both.  The reference rotates three buffers of node voltages Vd and
// auxiliary currents J by pointer once per step; here slot numTS % 3 is the current one ([0]),
// (numTS + 2) % 3 the previous ([1]) and (numTS + 1) % 3 the one before ([2]).  Float arithmetic
// in the reference's evaluation order.  The element edges are distinct (checked on the host).
struct RlcDev {
    unsigned count;
    const unsigned long long* off;   // field offset (component included)
    const float* c;                  // [9][count]: ilv, i2v, vv2, vj1, vj2, vvd, ib0, b1, b2
    float* il;                       // [count] parallel inductor current
    float* vd;                       // [3][count] node voltages
    float* j;                        // [3][count] auxiliary currents
};

// Engine_Ext_Cylinder (FDTD/extensions/engine_ext_cylinder.cpp:45-101) on a closed alpha mesh
// (y = alpha, line Ny-2 is line 0 once more); with rho = 0 on the mesh the axis z voltage is
// rebuilt from the alpha currents around it.
struct CylDev {
    int closed, r0;
    const float* vv_r0;   // [Nz]
    const float* vi_r0;   // [Nz]
};

// DoPostVoltageUpdates: one thread per (rho, z).  Thread (0, z) first sums the axis voltage in
// the reference's order and writes it to every alpha line (alpha voltages there are zero); every
// thread then copies the rho and z voltages of alpha line Ny-2 onto line 0.  A thread writes only
// its own (rho, z) lines, so the threads are independent.
static __global__ void __launch_bounds__(256) k_cyl_post_v(GridDev g, CylDev c)
{
    const unsigned long long t = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (unsigned long long)g.Nx * g.Nz) return;
    const unsigned r = (unsigned)(t / g.Nz), z = (unsigned)(t % g.Nz), last = g.Ny - 2;
    auto off = [&](unsigned n, unsigned x, unsigned a) {
        return (unsigned long long)n * g.S + ((unsigned long long)x * g.Ny + a) * g.Pz + z;
    };
    float* V = g.V;
    if (c.r0 && r == 0) {
        float volt = fmul(V[off(2, 0, 0)], c.vv_r0[z]);
        for (unsigned a = 0; a + 1 < g.Ny; ++a) volt = fadd(volt, fmul(c.vi_r0[z], g.I[off(1, 0, a)]));
        for (unsigned a = 0; a < g.Ny; ++a) {
            V[off(1, 0, a)] = 0.0f;
            V[off(2, 0, a)] = volt;
        }
    }
    V[off(0, r, 0)] = V[off(0, r, last)];
    V[off(2, r, 0)] = V[off(2, r, last)];
}

// DoPostCurrentUpdates: the rho and z currents of alpha line 0 onto line Ny-2, one thread per
// (rho, z) with rho < Nx-1 and z < Nz-1.
static __global__ void __launch_bounds__(256) k_cyl_post_i(GridDev g)
{
    const unsigned long long t = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned nz = g.Nz - 1;
    if (t >= (unsigned long long)(g.Nx - 1) * nz) return;
    const unsigned r = (unsigned)(t / nz), z = (unsigned)(t % nz), last = g.Ny - 2;
    auto off = [&](unsigned n, unsigned a) {
        return (unsigned long long)n * g.S + ((unsigned long long)r * g.Ny + a) * g.Pz + z;
    };
    g.I[off(0, last)] = g.I[off(0, 0)];
    g.I[off(2, last)] = g.I[off(2, 0)];
}

static __global__ void k_lumped_rlc(float* __restrict__ V, RlcDev r, const unsigned* __restrict__ numTS)
{
    const unsigned k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= r.count) return;
    const unsigned n = r.count;
    const unsigned t = *numTS;
    const unsigned s0 = t % 3u, s1 = (t + 2u) % 3u, s2 = (t + 1u) % 3u;
    const float ilv = r.c[k], i2v = r.c[n + k], vv2 = r.c[2 * n + k], vj1 = r.c[3 * n + k];
    const float vj2 = r.c[4 * n + k], vvd = r.c[5 * n + k], ib0 = r.c[6 * n + k], b1 = r.c[7 * n + k];
    const float b2 = r.c[8 * n + k];
    // DoPreVoltageUpdates: Il += i2v*ilv*Vd[n-1]
    const float il = fadd(r.il[k], fmul(fmul(i2v, ilv), r.vd[s1 * n + k]));
    r.il[k] = il;
    // Apply2Voltages
    const float vd2 = r.vd[s2 * n + k], j1 = r.j[s1 * n + k], j2 = r.j[s2 * n + k];
    const unsigned long long o = r.off[k];
    float vd0 = V[o];
    vd0 = fmul(vvd, fadd(fadd(fadd(fsub(vd0, il), fmul(vv2, vd2)), fmul(vj1, j1)), fmul(vj2, j2)));
    r.j[s0 * n + k] = fsub(fsub(fmul(ib0, fsub(vd0, vd2)), fmul(fmul(b1, ib0), j1)), fmul(fmul(b2, ib0), j2));
    r.vd[s0 * n + k] = vd0;
    V[o] = vd0;
}

// The z walls' hooks of the direct columns in park mode, around the voltage update: one thread per
// (wall, column), consecutive threads on consecutive y, so the coefficient tables and the saved
// values are read and written coalesced (the field values sit one per z row).  The reference's
// pre-voltage hook and post-voltage hook with the apply folded in
// (FDTD/extensions/engine_ext_mur_abc.cpp:83-178):
//   k_mur_zsave (before): pre = V_old(shift) - cP * V_old(line), per tangential component;
//   k_mur_zpost (after):  V(line) = pre + cP * V_new(shift).
// The same values and operation order as the shift-lane form inside the update (mur_z_shift).
__device__ __forceinline__ bool mur_zpark_item(const GridDev& g, const MurDev& m, unsigned t, unsigned& k,
                                               unsigned& q, unsigned long long& ol, unsigned long long& os)
{
    const unsigned nn = g.Nx * g.Ny;
    q = t / nn;
    if (q >= (unsigned)m.nz) return false;
    k = t - q * nn;
    const unsigned x = k / g.Ny, y = k - x * g.Ny;
    if (!mur_z_direct(m, x, y)) return false;              // x/y wall columns: the update's own hooks
    const MurWallDev& W = q ? m.z[1] : m.z[0];
    const unsigned long long row = (unsigned long long)k * g.Pz;
    ol = row + W.line;
    os = row + W.shift;
    return true;
}

static __global__ void k_mur_zsave(GridDev g, MurDev m)
{
    unsigned k, q;
    unsigned long long ol, os;
    if (!mur_zpark_item(g, m, blockIdx.x * blockDim.x + threadIdx.x, k, q, ol, os)) return;
    const MurWallDev& W = q ? m.z[1] : m.z[0];
    const unsigned nn = g.Nx * g.Ny;
    float* sv = m.zsave + (size_t)q * 2 * nn;
    sv[k] = fsub(g.V[os], fmul(__ldg(W.cP + k), g.V[ol]));
    sv[nn + k] = fsub(g.V[g.S + os], fmul(__ldg(W.cPP + k), g.V[g.S + ol]));
}

static __global__ void k_mur_zpost(GridDev g, MurDev m)
{
    unsigned k, q;
    unsigned long long ol, os;
    if (!mur_zpark_item(g, m, blockIdx.x * blockDim.x + threadIdx.x, k, q, ol, os)) return;
    const MurWallDev& W = q ? m.z[1] : m.z[0];
    const unsigned nn = g.Nx * g.Ny;
    const float* sv = m.zsave + (size_t)q * 2 * nn;
    g.V[ol] = fadd(sv[k], fmul(__ldg(W.cP + k), g.V[os]));
    g.V[g.S + ol] = fadd(sv[nn + k], fmul(__ldg(W.cPP + k), g.V[g.S + os]));
}

// ---------------------------------------------------------------------------------------------
// Engine_Ext_Mur_ABC (FDTD/extensions/engine_ext_mur_abc.cpp:83-178) as separate launches: k_mur
// phase 0 = pre (before the voltage update), 1 = post (after it), one launch for every wall
// (blockIdx.y = wall, threads over the wall plane [n1][n2]); k_mur_apply = the apply (after the
// dispersive apply hooks), one flat launch.  With the hooks inside the voltage update
// (mur_cell / mur_z_*) only the apply runs.
__device__ __forceinline__ unsigned long long mur_off(const GridDev& g, int comp, const unsigned p[3])
{
    return (unsigned long long)comp * g.S + ((unsigned long long)p[0] * g.Ny + p[1]) * g.Pz + p[2];
}

// the apply of wall wi at point t of its plane, or of its t-th listed column (zedge)
__device__ __forceinline__ void mur_apply_point(const GridDev& g, const MurDev& m, int wi, unsigned t, unsigned ts)
{
    const MurWallDev& w = m.w[wi];
    if (ts < w.start_ts) return;              // Engine_Ext_Mur_ABC::IsActive
    const bool listed = m.lanes && w.ny == 2 && m.zedge;
    unsigned i, j;
    if (listed) {
        if (t >= m.nzedge) return;
        const unsigned c = __ldg(m.zedge + t);
        i = c / w.n2;
        j = c - i * w.n2;
    } else {
        if (t >= w.n1 * w.n2) return;
        // consecutive threads walk the tangential axis that is contiguous in memory (z when it
        // is tangential, else y); the small per-wall tables are L2-resident either way
        if (w.nyP == 2) { i = t % w.n1; j = t / w.n1; }
        else { i = t / w.n2; j = t - i * w.n2; }
    }
    const unsigned k = mur_k(w, i, j);
    unsigned pos[3];
    pos[w.ny] = w.line;
    pos[w.nyP] = i;
    pos[w.nyPP] = j;
    // a direct column of the lane-parallel z-wall form holds its final value already
    if (!listed && m.lanes && w.ny == 2 && mur_z_direct(m, pos[0], pos[1])) return;
    // walls are applied in reverse insertion order, so on shared edges the wall with the
    // lowest index is the last writer; skip components a lower active wall also writes
    bool wP = true, wPP = true;
    for (int q = 0; q < wi; ++q) {
        const MurWallDev& o = m.w[q];
        if (ts < o.start_ts || pos[o.ny] != o.line) continue;
        if (w.nyP != o.ny) wP = false;
        if (w.nyPP != o.ny) wPP = false;
    }
    float* V = g.V;
    if (wP) V[mur_off(g, w.nyP, pos)] = w.bP[k];
    if (wPP) V[mur_off(g, w.nyPP, pos)] = w.bPP[k];
}

static __global__ void k_mur(GridDev g, MurDev m, int phase, const unsigned* __restrict__ numTS)
{
    const int wi = blockIdx.y;
    if (wi >= m.nwall) return;
    const MurWallDev& w = m.w[wi];
    const unsigned ts = *numTS;
    if (ts < w.start_ts) return;              // Engine_Ext_Mur_ABC::IsActive
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= w.n1 * w.n2) return;
    // consecutive threads walk the tangential axis that is contiguous in memory (z when it is
    // tangential, else y); the small per-wall tables are L2-resident either way
    unsigned i, j;
    if (w.nyP == 2) { i = t % w.n1; j = t / w.n1; }
    else { i = t / w.n2; j = t - i * w.n2; }
    const unsigned k = mur_k(w, i, j);
    unsigned pos[3], ps[3];
    pos[w.ny] = w.line; ps[w.ny] = w.shift;
    pos[w.nyP] = ps[w.nyP] = i;
    pos[w.nyPP] = ps[w.nyPP] = j;
    float* V = g.V;
    if (phase == 0) {
        w.bP[k] = fsub(V[mur_off(g, w.nyP, ps)], fmul(w.cP[k], V[mur_off(g, w.nyP, pos)]));
        w.bPP[k] = fsub(V[mur_off(g, w.nyPP, ps)], fmul(w.cPP[k], V[mur_off(g, w.nyPP, pos)]));
        return;
    }
    if (phase == 1) {
        w.bP[k] = fadd(w.bP[k], fmul(w.cP[k], V[mur_off(g, w.nyP, ps)]));
        w.bPP[k] = fadd(w.bPP[k], fmul(w.cPP[k], V[mur_off(g, w.nyPP, ps)]));
    }
}

// the flat apply launch: every wall's points (or listed columns) in one 1-D grid
static __global__ void k_mur_apply(GridDev g, MurDev m, const unsigned* __restrict__ numTS)
{
    const unsigned b = blockIdx.x;
    int wi = 0;
    while (wi + 1 < m.nwall && b >= m.afirst[wi + 1]) ++wi;
    mur_apply_point(g, m, wi, (b - m.afirst[wi]) * blockDim.x + threadIdx.x, *numTS);
}

// ---------------------------------------------------------------------------------------------
// Engine_Ext_LorentzMaterial pre hooks (engine_ext_lorentzmaterial.cpp:79-168) and
// Engine_Ext_Dispersive apply hooks (engine_ext_dispersive.cpp:76-127) for one order.
struct LorDev {
    unsigned count;
    const unsigned char* skip;       // optional: bit n set = the apply leaves component n alone
    const unsigned long long* off;   // field offset of component 0 at each position (or off32)
    const unsigned* off32;           // the same in 32 bits when every offset fits (off is null)
    int lor;                         // Lorentz pole term on
    const float* c_int;              // [3][count] (null when cls is set)
    const float* c_ext;
    const float* c_lor;
    const unsigned short* cls;       // per position: coefficient class, or null
    const float4* ctab;              // [class][3]: int 0..2, ext 0..2, lor 0..2, pad
    float* ade;                      // [3][count]
    float* lade;
};

__device__ __forceinline__ unsigned long long lor_off(const LorDev& l, unsigned i)
{
    return l.off32 ? (unsigned long long)__ldg(l.off32 + i) : __ldg(l.off + i);
}

// the position's coefficients of component n: int, ext, lor
struct LorCoef {
    float ci[3], ce[3], cl[3];
};
__device__ __forceinline__ LorCoef lor_coef(const LorDev& l, unsigned i)
{
    LorCoef c;
    if (l.cls) {
        const float4* t = l.ctab + 3u * __ldg(l.cls + i);
        const float4 a = __ldg(t), b = __ldg(t + 1), d = __ldg(t + 2);
        c.ci[0] = a.x; c.ci[1] = a.y; c.ci[2] = a.z;
        c.ce[0] = a.w; c.ce[1] = b.x; c.ce[2] = b.y;
        c.cl[0] = b.z; c.cl[1] = b.w; c.cl[2] = d.x;
    } else {
#pragma unroll
        for (int n = 0; n < 3; ++n) {
            const unsigned k = n * l.count + i;
            c.ci[n] = __ldg(l.c_int + k);
            c.ce[n] = __ldg(l.c_ext + k);
            c.cl[n] = l.lor ? __ldg(l.c_lor + k) : 0.f;
        }
    }
    return c;
}

// the pre hook of one component: the ADE current from the field before the update (a the ADE
// value, la the pole term's, f the field value); returns the new ADE value, la updated in place
__device__ __forceinline__ float lor_pre_one(const LorDev& l, const LorCoef& c, int n, float a, float& la, float f)
{
    if (l.lor) {
        la = fadd(la, fmul(c.cl[n], a));
        a = fmul(a, c.ci[n]);
        return fadd(a, fmul(c.ce[n], fsub(f, la)));
    }
    a = fmul(a, c.ci[n]);
    return fadd(a, fmul(c.ce[n], f));
}

static __global__ void k_lorentz_pre(const float* __restrict__ F, unsigned long long S, LorDev l)
{
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= l.count) return;
    const unsigned long long o = lor_off(l, i);
    const LorCoef c = lor_coef(l, i);
    float f[3], a[3], la[3];
#pragma unroll
    for (int n = 0; n < 3; ++n) {
        f[n] = F[o + n * S];
        a[n] = l.ade[n * l.count + i];
        la[n] = l.lor ? l.lade[n * l.count + i] : 0.f;
    }
#pragma unroll
    for (int n = 0; n < 3; ++n) {
        l.ade[n * l.count + i] = lor_pre_one(l, c, n, a[n], la[n], f[n]);
        if (l.lor) l.lade[n * l.count + i] = la[n];
    }
}

// the apply hook: F -= ade
__device__ __forceinline__ void lor_apply_point(float* __restrict__ F, unsigned long long S, const LorDev& l, unsigned i)
{
    if (i >= l.count) return;
    const unsigned long long o = lor_off(l, i);
    const unsigned sk = l.skip ? l.skip[i] : 0u;
#pragma unroll
    for (int n = 0; n < 3; ++n) {
        if (sk & (1u << n)) continue;
        const unsigned long long q = o + n * S;
        F[q] = fsub(F[q], l.ade[n * l.count + i]);
    }
}

static __global__ void k_lorentz_apply(float* __restrict__ F, unsigned long long S, LorDev l)
{
    lor_apply_point(F, S, l, blockIdx.x * blockDim.x + threadIdx.x);
}

// This step's apply and the next step's pre in one pass, launched at the end of the field's
// half-step (after every later apply hook: the host allows it only where no excitation edge is a
// position's component and the Mur walls' components are in skip).  Between the two nothing
// else writes the field at these positions, so the pre reads the same values as it would at the
// start of the next half-step; the ADE values stay in registers between them.
__device__ __forceinline__ void lor_carry_point(float* __restrict__ F, unsigned long long S, const LorDev& l, unsigned i)
{
    if (i >= l.count) return;
    const unsigned long long o = lor_off(l, i);
    const unsigned sk = l.skip ? l.skip[i] : 0u;
    const LorCoef c = lor_coef(l, i);
    float f[3], a[3], la[3];
#pragma unroll
    for (int n = 0; n < 3; ++n) {
        f[n] = F[o + n * S];
        a[n] = l.ade[n * l.count + i];
        la[n] = l.lor ? l.lade[n * l.count + i] : 0.f;
    }
#pragma unroll
    for (int n = 0; n < 3; ++n) {
        if (!(sk & (1u << n))) {
            f[n] = fsub(f[n], a[n]);
            F[o + n * S] = f[n];
        }
        l.ade[n * l.count + i] = lor_pre_one(l, c, n, a[n], la[n], f[n]);
        if (l.lor) l.lade[n * l.count + i] = la[n];
    }
}

static __global__ void k_lorentz_carry(float* __restrict__ F, unsigned long long S, LorDev l)
{
    lor_carry_point(F, S, l, blockIdx.x * blockDim.x + threadIdx.x);
}

// The end of a voltage half-step as one launch: the Mur apply (blocks [0, lor0)), the
// dispersive carry (CARRY, inside a sequence) or apply (the sequence's last step) ([lor0, exc0))
// and the excitation (from exc0).  The host allows it only where the three touch disjoint
// values: one dispersive order, no dispersive position on a Mur line (skip is empty), no
// excitation edge on a dispersive position or on a Mur line's tangential component; the order
// among them then does not matter.
template <bool CARRY>
__global__ void k_vtail(GridDev g, MurDev m, LorDev l, ExcDev x, const unsigned* __restrict__ numTS, unsigned lor0,
                        unsigned exc0)
{
    const unsigned b = blockIdx.x;
    if (b < lor0) {
        int wi = 0;
        while (wi + 1 < m.nwall && b >= m.afirst[wi + 1]) ++wi;
        mur_apply_point(g, m, wi, (b - m.afirst[wi]) * blockDim.x + threadIdx.x, *numTS);
    } else if (b < exc0) {
        const unsigned i = (b - lor0) * blockDim.x + threadIdx.x;
        if (CARRY) lor_carry_point(g.V, g.S, l, i);
        else lor_apply_point(g.V, g.S, l, i);
    } else {
        exc_point(g.V, x, (b - exc0) * blockDim.x + threadIdx.x, *numTS);
    }
}

// ---------------------------------------------------------------------------------------------
// Processing at the end of a timestep: probes (ProcessIntegral::Process,
// Common/processintegral.cpp:134-171), FD field dumps (ProcessFieldsFD::Process,
// Common/processfields_fd.cpp:72-107) and the numTS increment.
struct ProbeDev {
    int type;                        // 0 voltage (double sum), 1 current (float sum), 2/3 E/H field
    unsigned ncomp;                  // values per sample: 1, or 3 (field probes)
    double el[3];                    // field probes: edge length of each component
    unsigned nterm;
    const unsigned long long* term;  // field offsets in reference summation order
    const signed char* sign;         // +1 / -1
    double weight;
    unsigned interval, start_ts, stop_ts, nslots;
    double* series;                  // [nslots][ncomp]
    unsigned fd_interval, nf, nsamp;
    const double2* phasor;           // [nsamp][nf] = exp(-2j*pi*f*t)
    double* dft;                     // [nf][ncomp][2]
    double dt;
    // newest sample in mapped host memory (device address), with its slot: a host read of the
    // newest slot needs no copy after the stream synchronisation
    double* latest;                  // [ncomp]
    unsigned* latest_slot;
};

struct DumpDev {
    int field;                       // 0 E (uses V), 1 H (uses I)
    int interp;                      // 0 none, 1 node, 2 cell interpolation
    unsigned start[3], sz[3];
    unsigned npos;
    unsigned fd_interval, nf, nsamp;
    const float2* phasor;            // [nsamp][nf], includes *2 and *dt*fd_interval
    const double* el;                // GetEdgeLength per line, concatenated x,y,z (E: main, H: dual)
    const double* rho;               // cylindrical mesh (no interpolation): rho per x line, else null
    float2* acc;                     // [nf][3][npos]
    // time-domain dump (ProcessFieldsTD): td = 1; sample ts (ts % td_interval == 0 within
    // [td_start, td_stop]) goes to ring slot (ts / td_interval) % nslot as float [3][npos]
    unsigned td, td_interval, td_start, td_stop, nslot;
    float* ring;
};

struct StepEndDev {
    int nprobe;
    const ProbeDev* probes;          // device array
    int ndump;
    const DumpDev* dumps;            // device array
    const unsigned* dump_block0;     // first block of each dump (prefix sums), size ndump+1
    unsigned* numTS;
    unsigned* blocks_done;
};

// Record value*weight `a` of component c: the time series slot and the DFT accumulation
// (ProcessIntegral::Process, Common/processintegral.cpp:144-167), double arithmetic in its order.
static __device__ void probe_record(const ProbeDev& p, unsigned ts, unsigned c, double a, bool do_td, bool do_fd)
{
    if (do_td) {
        const unsigned slot = ts / p.interval;
        if (slot < p.nslots) {
            p.series[(unsigned long long)slot * p.ncomp + c] = a;
            if (p.latest) {
                p.latest[c] = a;
                if (c == 0) *p.latest_slot = slot;
            }
        }
    }
    if (do_fd) {
        const unsigned smp = ts / p.fd_interval;
        if (smp < p.nsamp) {
            for (unsigned f = 0; f < p.nf; ++f) {
                const double2 e = p.phasor[(unsigned long long)smp * p.nf + f];
                double re = __dmul_rn(e.x, a), im = __dmul_rn(e.y, a);
                re = __dmul_rn(re, 2.0); im = __dmul_rn(im, 2.0);
                re = __dmul_rn(re, p.dt); im = __dmul_rn(im, p.dt);
                re = __dmul_rn(re, (double)p.fd_interval); im = __dmul_rn(im, (double)p.fd_interval);
                double* acc = p.dft + 2 * ((unsigned long long)f * p.ncomp + c);
                acc[0] = __dadd_rn(acc[0], re);
                acc[1] = __dadd_rn(acc[1], im);
            }
        }
    }
}

static __device__ void probe_eval(const GridDev& g, const ProbeDev& p, unsigned ts, int lane)
{
    if (ts < p.start_ts || ts > p.stop_ts) return;
    const bool do_td = (ts % p.interval) == 0;
    const bool do_fd = p.fd_interval && (ts % p.fd_interval) == 0;
    if (!do_td && !do_fd) return;
    const float* F = (p.type == 0 || p.type == 2) ? g.V : g.I;
    if (p.type >= 2) {
        // ProcessFieldProbe: lane n evaluates component n (GetRawField / GetRawDualField)
        if (lane >= 3) return;
        const double value = (double)__ldcg(F + p.term[lane]);
        const double delta = p.el[lane];
        probe_record(p, ts, lane, __dmul_rn(delta != 0.0 ? __ddiv_rn(value, delta) : 0.0, p.weight), do_td, do_fd);
        return;
    }
    // lanes fetch terms in parallel, lane 0 accumulates them in the reference's order
    double accd = 0.0;
    float accf = 0.0f;
    for (unsigned base = 0; base < p.nterm; base += 32) {
        const unsigned k = base + lane;
        float v = 0.0f;
        int s = 0;
        if (k < p.nterm) { v = __ldcg(F + p.term[k]); s = p.sign[k]; }
        const unsigned cnt = min(32u, p.nterm - base);
        for (unsigned j = 0; j < cnt; ++j) {
            const float vj = __shfl_sync(0xffffffffu, v, j);
            const int sj = __shfl_sync(0xffffffffu, s, j);
            if (lane == 0) {
                if (p.type == 0) accd = sj > 0 ? __dadd_rn(accd, (double)vj) : __dsub_rn(accd, (double)vj);
                else accf = sj > 0 ? fadd(accf, vj) : fsub(accf, vj);
            }
        }
    }
    if (lane != 0) return;
    const double val = p.type == 0 ? accd : (double)accf;
    probe_record(p, ts, 0, __dmul_rn(val, p.weight), do_td, do_fd);
}

// E (Engine_Interface_FDTD::GetRawInterpolatedField, FDTD/engine_interface_fdtd.cpp:63-123) or
// H (GetRawInterpolatedDualField, :140-204) at pos with the dump's interpolation: 0 the raw Yee
// value over its edge length, 1 node interpolation, 2 cell interpolation.  Double arithmetic in
// the reference's order.
static __device__ void dump_field(const GridDev& g, const DumpDev& d, const unsigned pos[3], double out[3])
{
    const unsigned N[3] = {g.Nx, g.Ny, g.Nz};
    const unsigned eoff[3] = {0u, g.Nx, g.Nx + g.Ny};
    const float* F = d.field == 0 ? g.V : g.I;
    // GetRawField / GetRawDualField: value / edge length (0 for a zero length)
    auto raw = [&](int n, const unsigned* p) -> double {
        double delta = d.el[eoff[n] + p[n]];
        if (n == 1 && d.rho) delta = __dmul_rn(delta, d.rho[p[0]]);   // Operator_Cylinder::GetEdgeLength
        const float v = F[(unsigned long long)n * g.S + ((unsigned long long)p[0] * g.Ny + p[1]) * g.Pz + p[2]];
        return delta != 0.0 ? __ddiv_rn((double)v, delta) : 0.0;
    };
    const bool edge = pos[0] == N[0] - 1 || pos[1] == N[1] - 1 || pos[2] == N[2] - 1;
#pragma unroll
    for (int n = 0; n < 3; ++n) {
        const int nP = (n + 1) % 3, nPP = (n + 2) % 3;
        unsigned ip[3] = {pos[0], pos[1], pos[2]};
        if (d.interp == 0) { out[n] = raw(n, ip); continue; }
        if (d.field == 0) {
            if (d.interp == 1) {
                if (pos[n] == N[n] - 1) { --ip[n]; out[n] = raw(n, ip); continue; }   // the lower value
                const double delta = d.el[eoff[n] + ip[n]];
                out[n] = raw(n, ip);
                if (delta == 0.0) { out[n] = 0.0; continue; }
                if (pos[n] == 0) continue;                                              // the upper value
                --ip[n];
                const double deltaDown = d.el[eoff[n] + ip[n]];
                const double deltaRel = __ddiv_rn(delta, __dadd_rn(delta, deltaDown));
                out[n] = __dadd_rn(__dmul_rn(out[n], __dsub_rn(1.0, deltaRel)), __dmul_rn(raw(n, ip), deltaRel));
            } else {
                if (edge) { out[n] = 0.0; continue; }
                double acc = raw(n, ip);
                ++ip[nP];
                acc = __dadd_rn(acc, raw(n, ip));
                ++ip[nPP];
                acc = __dadd_rn(acc, raw(n, ip));
                --ip[nP];
                acc = __dadd_rn(acc, raw(n, ip));
                out[n] = __ddiv_rn(acc, 4.0);
            }
        } else {
            if (d.interp == 1) {
                if (edge || pos[nP] == 0 || pos[nPP] == 0) { out[n] = 0.0; continue; }
                double acc = raw(n, ip);
                --ip[nP];
                acc = __dadd_rn(acc, raw(n, ip));
                --ip[nPP];
                acc = __dadd_rn(acc, raw(n, ip));
                ++ip[nP];
                acc = __dadd_rn(acc, raw(n, ip));
                out[n] = __ddiv_rn(acc, 4.0);
            } else {
                const double delta = d.el[eoff[n] + ip[n]];
                const double o = raw(n, ip);
                if (pos[n] >= N[n] - 1) { out[n] = 0.0; continue; }
                ++ip[n];
                const double deltaUp = d.el[eoff[n] + ip[n]];
                const double deltaRel = __ddiv_rn(delta, __dadd_rn(delta, deltaUp));
                out[n] = __dadd_rn(__dmul_rn(o, __dsub_rn(1.0, deltaRel)), __dmul_rn(raw(n, ip), deltaRel));
            }
        }
    }
}

// One launch: block 0 warps evaluate the probes; blocks [dump_block0[k], dump_block0[k+1])
// handle dump k (one thread per box position, all frequencies).  The last block to finish
// increments numTS (threadfence + completion counter), so every block read the same ts.
// part -1: everything; part 0: the probes and dumps that read V (voltage and E-field probes, E
// dumps); part 1: those that read I (current and H-field probes, H dumps) and the numTS
// increment.  The parts let the engine run part 0 beside the current update (which does not
// write V) and part 1 beside the next voltage update (which does not write I).
static __global__ void __launch_bounds__(256) k_step_end(GridDev g, StepEndDev s, int part = -1)
{
    const unsigned ts = *s.numTS + 1;   // the step just completed
    if (blockIdx.x == 0) {
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        for (int p = warp; p < s.nprobe; p += blockDim.x >> 5) {
            const ProbeDev& q = s.probes[p];
            const int side = (q.type == 1 || q.type == 3) ? 1 : 0;
            if (part < 0 || part == side) probe_eval(g, q, ts, lane);
        }
    } else {
        // find the dump of this block
        int k = 0;
        while (k + 1 < s.ndump && blockIdx.x >= s.dump_block0[k + 1]) ++k;
        if (s.ndump > 0 && (part < 0 || part == (s.dumps[k].field == 1 ? 1 : 0))) {
            const DumpDev& d = s.dumps[k];
            const unsigned q = (blockIdx.x - s.dump_block0[k]) * blockDim.x + threadIdx.x;
            if (d.td) {
                if (q < d.npos && ts >= d.td_start && ts <= d.td_stop && (ts % d.td_interval) == 0) {
                    const unsigned a = q / (d.sz[1] * d.sz[2]);
                    const unsigned rem = q - a * d.sz[1] * d.sz[2];
                    const unsigned b = rem / d.sz[2], c = rem - b * d.sz[2];
                    const unsigned pos[3] = {d.start[0] + a, d.start[1] + b, d.start[2] + c};
                    double out[3];
                    dump_field(g, d, pos, out);
                    float* slot = d.ring + (unsigned long long)((ts / d.td_interval) % d.nslot) * 3 * d.npos;
#pragma unroll
                    for (int n = 0; n < 3; ++n) slot[(unsigned long long)n * d.npos + q] = (float)out[n];
                }
            } else if (q < d.npos && d.fd_interval && (ts % d.fd_interval) == 0) {
                const unsigned smp = ts / d.fd_interval;
                if (smp < d.nsamp) {
                    const unsigned a = q / (d.sz[1] * d.sz[2]);
                    const unsigned rem = q - a * d.sz[1] * d.sz[2];
                    const unsigned b = rem / d.sz[2], c = rem - b * d.sz[2];
                    const unsigned pos[3] = {d.start[0] + a, d.start[1] + b, d.start[2] + c};
                    double out[3];
                    dump_field(g, d, pos, out);
                    for (unsigned f = 0; f < d.nf; ++f) {
                        const float2 e = d.phasor[(unsigned long long)smp * d.nf + f];
#pragma unroll
                        for (int n = 0; n < 3; ++n) {
                            const float td = (float)out[n];
                            float2* acc = d.acc + ((unsigned long long)f * 3 + n) * d.npos + q;
                            float2 v = *acc;
                            v.x = fadd(v.x, fmul(td, e.x));
                            v.y = fadd(v.y, fmul(td, e.y));
                            *acc = v;
                        }
                    }
                }
            }
        }
    }
    // completion: last block bumps numTS
    if (part == 0) return;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned done = atomicAdd(s.blocks_done, 1u);
        if (done == gridDim.x - 1) {
            *s.blocks_done = 0u;
            __threadfence();
            *s.numTS = ts;
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Engine_Interface_FDTD::CalcFastEnergy (FDTD/engine_interface_fdtd.cpp:302-347): double
// accumulation of float squares over [0,N-1)^3; block partials then one final reduction.
static __global__ void __launch_bounds__(256) k_energy(GridDev g, double* __restrict__ partial)
{
    double e = 0.0, h = 0.0;
    const unsigned long long plane = (unsigned long long)g.Ny * g.Pz;
    const unsigned long long total = (unsigned long long)(g.Nx - 1) * plane;
    for (unsigned long long t = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned long long x = t / plane;
        const unsigned long long r = t - x * plane;
        const unsigned y = (unsigned)(r / g.Pz), z = (unsigned)(r - (unsigned long long)y * g.Pz);
        if (y + 1 >= g.Ny || z + 1 >= g.Nz) continue;
#pragma unroll
        for (int n = 0; n < 3; ++n) {
            const float v = g.V[n * g.S + t], c = g.I[n * g.S + t];
            e += (double)fmul(v, v);
            h += (double)fmul(c, c);
        }
    }
    __shared__ double se[256], sh[256];
    se[threadIdx.x] = e;
    sh[threadIdx.x] = h;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) { se[threadIdx.x] += se[threadIdx.x + w]; sh[threadIdx.x] += sh[threadIdx.x + w]; }
        __syncthreads();
    }
    if (threadIdx.x == 0) { partial[2 * blockIdx.x] = se[0]; partial[2 * blockIdx.x + 1] = sh[0]; }
}

}  // namespace oems
