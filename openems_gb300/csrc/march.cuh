// march.cuh -- one kernel per timestep, staged by the Tensor Memory Accelerator.
//
// A whole timestep of Engine::UpdateVoltages / UpdateCurrents (FDTD/engine.cpp:110-222) with the
// soft excitation (FDTD/extensions/engine_ext_excitation.cpp:33-94) in one pass over the mesh,
// for engines whose operator is compressed and which carry no UPML, Mur, dispersive, TFSF,
// lumped-RLC or cylinder hooks.  The step reads V, I and the class index once and writes V and
// I once (52 bytes per cell-step against 80 for the two half-step kernels), so the fields
// ping-pong between two buffer sets (the fused step's plumbing, fused.cuh).
//
// Decomposition: a block owns `ty` rows of y over the whole z extent (Pz <= 256, the TMA box
// limit) and marches over a chunk of x-planes.  Per plane p:
//   1. I_old(p) of rows y0-1 .. y0+ty (all three components) arrives in shared memory through one
//      cp.async.bulk.tensor load, issued two planes ahead into a three-slot ring and completed on
//      an mbarrier; I_old(p-1) is still in the previous slot (the -x neighbour);
//   2. each thread computes V'(p) of four consecutive z cells (a float4 group) on rows y0 .. y0+ty
//      -- the +y halo row is recomputed rather than exchanged -- from the staged I planes and from
//      V_old(p) and the class index of its cells, which it loaded into registers one plane ahead
//      (the register queue); the soft sources are added, V'(p) goes to shared memory and, for the
//      block's own rows, to the output buffer;
//   3. after a barrier, the thread computes I'(p-1) of the same four cells from V'(p-1), V'(p)
//      (both in shared memory) and I_old(p-1) (the previous ring slot), and stores it.
// Arithmetic is update_v_cell / update_i_cell's, lane by lane, so results are bit-identical to the
// separate kernels.  Boundary reads follow the reference: at index 0 the -x/-y/-z neighbour is the
// cell itself.
//
// Every wait on an mbarrier is bounded: past the limit the block sets the error flag, waits (again
// bounded) for its own copies still in flight and returns; the host reports OEMS_ERR_DEVICE.
#pragma once

#include <cuda.h>

#include "fused.cuh"
#include "march_dev.h"

namespace oems {

constexpr int MARCH_SLOTS = 3;
constexpr unsigned MARCH_SPIN_LIMIT = 1u << 26;        // tries of one wait, at most
constexpr unsigned long long MARCH_WAIT_NS = 2000000000ull;   // and two seconds of %globaltimer

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// bounded wait for phase `parity` of the barrier; false when the limit ran out
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity)
{
    const unsigned a = smem_addr(bar);
    unsigned long long t0 = 0;
    for (unsigned it = 0; it < MARCH_SPIN_LIMIT; ++it) {
        unsigned done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if ((it & 63u) == 63u) {
            const unsigned long long now = global_ns();
            if (!t0) t0 = now;
            else if (now - t0 > MARCH_WAIT_NS) return false;
        }
    }
    return false;
}

// I_old of x-plane q, rows y0-1 .. y0+ty, all z, all components, into a ring slot
__device__ __forceinline__ void march_load(const CUtensorMap* map, float* slot, unsigned long long* bar, unsigned bytes,
                                           int y0, int q)
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(bar, bytes);
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];" ::
            "r"(smem_addr(slot)),
        "l"(map), "r"(0), "r"(y0 - 1), "r"(q), "r"(0), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ float4 lds4(const float* p) { return *reinterpret_cast<const float4*>(p); }

// V'(x, y, z0..z0+3): update_v_cell's arithmetic on the staged planes Ic = I_old(x), Ip = I_old(x-1)
// (slot rows: slot row r holds y = y0 - 1 + r), then the soft sources
__device__ __forceinline__ void march_v(const MarchDev& m, const float* Ic, const float* Ip, unsigned x, unsigned y,
                                        unsigned z0, unsigned r, const float4 vold[3], uint4 ci, int ts, float4 out[3])
{
    const FusedDev& f = m.f;
    const GridDev& g = f.g;
    const unsigned Pz = g.Pz, rows = m.ty + 2;
    const float* c0p = Ic + (0 * rows + r) * Pz + z0;
    const float* c1p = Ic + (1 * rows + r) * Pz + z0;
    const float* c2p = Ic + (2 * rows + r) * Pz + z0;
    const float4 i0 = lds4(c0p), i1 = lds4(c1p), i2 = lds4(c2p);
    // -y neighbour (the cell itself at y = 0), -x neighbour (Ip: I_old(x-1), or x itself at x = 0)
    const float4 i2y = y ? lds4(c2p - Pz) : i2, i0y = y ? lds4(c0p - Pz) : i0;
    const float4 i2x = lds4(Ip + (2 * rows + r) * Pz + z0), i1x = lds4(Ip + (1 * rows + r) * Pz + z0);
    const float i1m = z0 ? c1p[-1] : i1.x, i0m = z0 ? c0p[-1] : i0.x;
    out[0] = vold[0];
    out[1] = vold[1];
    out[2] = vold[2];
    const unsigned cls[4] = {ci.x, ci.y, ci.z, ci.w};
    const unsigned long long S = g.S;
    const unsigned long long o0 = ((unsigned long long)x * g.Ny + y) * Pz + z0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (z0 + k >= g.Nz) break;
        const float4 ca = __ldg(g.tabV + 2 * cls[k]), cb = __ldg(g.tabV + 2 * cls[k] + 1);
        const float i1z = k ? f4(i1, k - 1) : i1m, i0z = k ? f4(i0, k - 1) : i0m;
        const float c0 = fadd(fsub(fsub(f4(i2, k), f4(i2y, k)), f4(i1, k)), i1z);
        const float c1 = fadd(fsub(fsub(f4(i0, k), i0z), f4(i2, k)), f4(i2x, k));
        const float c2 = fadd(fsub(fsub(f4(i1, k), f4(i1x, k)), f4(i0, k)), f4(i0y, k));
        float v[3] = {fadd(fmul(f4(out[0], k), ca.x), fmul(ca.w, c0)), fadd(fmul(f4(out[1], k), ca.y), fmul(cb.x, c1)),
                      fadd(fmul(f4(out[2], k), ca.z), fmul(cb.y, c2))};
        add_excitation(f.excV, f.srcV_cell, f.srcV_lo, f.srcV_hi, o0 + k, S, ts, v);
        set4(out[0], k, v[0]);
        set4(out[1], k, v[1]);
        set4(out[2], k, v[2]);
    }
}

// I'(x, y, z0..z0+3) from V'(x) (Vp), V'(x+1) (Vc) and I_old(x) (slot Ip): update_i_cell's
// arithmetic lane by lane (lanes at or past z = Nz-1 keep I_old), then the soft sources
__device__ __forceinline__ void march_i(const MarchDev& m, const float* Vp, const float* Vc, const float* Ip, unsigned x,
                                        unsigned y, unsigned z0, unsigned rv, uint4 ci, int ts, float4 out[3])
{
    const FusedDev& f = m.f;
    const GridDev& g = f.g;
    const unsigned Pz = g.Pz, vrows = m.ty + 1, irows = m.ty + 2;
    const float* w0p = Vp + (0 * vrows + rv) * Pz + z0;
    const float* w1p = Vp + (1 * vrows + rv) * Pz + z0;
    const float* w2p = Vp + (2 * vrows + rv) * Pz + z0;
    const float4 w0 = lds4(w0p), w1 = lds4(w1p), w2 = lds4(w2p);
    const float4 w2y = lds4(w2p + Pz), w0y = lds4(w0p + Pz);       // +y: the next V' row
    const float4 w2x = lds4(Vc + (2 * vrows + rv) * Pz + z0), w1x = lds4(Vc + (1 * vrows + rv) * Pz + z0);
    const float w0z4 = (z0 + 4 < Pz) ? w0p[4] : 0.f, w1z4 = (z0 + 4 < Pz) ? w1p[4] : 0.f;
    const unsigned r = rv + 1;
    out[0] = lds4(Ip + (0 * irows + r) * Pz + z0);
    out[1] = lds4(Ip + (1 * irows + r) * Pz + z0);
    out[2] = lds4(Ip + (2 * irows + r) * Pz + z0);
    const unsigned cls[4] = {ci.x, ci.y, ci.z, ci.w};
    const unsigned long long S = g.S;
    const unsigned long long o0 = ((unsigned long long)x * g.Ny + y) * Pz + z0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (z0 + k + 1 >= g.Nz) break;
        const float4 ca = __ldg(g.tabI + 2 * cls[k]), cb = __ldg(g.tabI + 2 * cls[k] + 1);
        const float v1z = k < 3 ? f4(w1, k + 1) : w1z4, v0z = k < 3 ? f4(w0, k + 1) : w0z4;
        const float c0 = fadd(fsub(fsub(f4(w2, k), f4(w2y, k)), f4(w1, k)), v1z);
        const float c1 = fadd(fsub(fsub(f4(w0, k), v0z), f4(w2, k)), f4(w2x, k));
        const float c2 = fadd(fsub(fsub(f4(w1, k), f4(w1x, k)), f4(w0, k)), f4(w0y, k));
        float v[3] = {fadd(fmul(f4(out[0], k), ca.x), fmul(ca.w, c0)), fadd(fmul(f4(out[1], k), ca.y), fmul(cb.x, c1)),
                      fadd(fmul(f4(out[2], k), ca.z), fmul(cb.y, c2))};
        add_excitation(f.excI, f.srcI_cell, f.srcI_lo, f.srcI_hi, o0 + k, S, ts, v);
        set4(out[0], k, v[0]);
        set4(out[1], k, v[1]);
        set4(out[2], k, v[2]);
    }
}

__device__ __forceinline__ void st4(float* p, const float4 v) { *reinterpret_cast<float4*>(p) = v; }

// Grid: (tiles of ty rows along y, chunks of xchunk planes along x).  Block: (ty+1) * groups
// threads, rounded up to warps.  Dynamic shared memory: three I ring slots, two V' buffers and
// the three mbarriers (host: march_smem_bytes).
// MINB: blocks per SM the register budget is sized for (1: about 108 registers a thread, no
// spills; 2: 64 registers)
template <int MINB>
__global__ void __launch_bounds__(512, MINB) k_step_march(const __grid_constant__ MarchDev m,
                                                     const __grid_constant__ CUtensorMap mapI)
{
    extern __shared__ __align__(128) float smem[];
    const FusedDev& f = m.f;
    const GridDev& g = f.g;
    const unsigned Pz = g.Pz, G = m.groups, ty = m.ty;
    // ring slot s at smem + s * slot_floats, V' buffer b after the ring (no pointer arrays: they
    // would be indexed at run time and live in local memory)
    const unsigned SF = m.slot_floats, VF = m.vbuf_floats;
    float* const vbase = smem + MARCH_SLOTS * SF;
    unsigned long long* bar = reinterpret_cast<unsigned long long*>(vbase + 2 * VF);
    const unsigned bytes = m.box_bytes;

    const unsigned t = threadIdx.x;
    const unsigned rv = t / G, gz = t - rv * G, z0 = gz * 4;
    const unsigned y0 = blockIdx.x * ty;
    const unsigned y = y0 + rv;
    const unsigned xa = blockIdx.y * m.xchunk;
    if (xa >= g.Nx) return;
    const unsigned xb = min(g.Nx, xa + m.xchunk);          // own planes [xa, xb)
    const unsigned xend = min(xb + 1, g.Nx);               // V' planes [xa, xend)
    const bool inV = rv <= ty && y < g.Ny;                 // this thread's V' group exists
    const bool ownV = rv < ty && y < g.Ny;                 // ... and is stored by this block
    const bool inI = rv < ty && y + 1 < g.Ny;              // I is updated on this row
    const unsigned long long S = g.S, plane = (unsigned long long)g.Ny * Pz;
    const unsigned long long yz = (unsigned long long)y * Pz + z0;
    const int ts = (int)*f.numTS;

    // ring slot of plane q: (q - xa + 1) % 3 (the -x neighbour plane of xa sits in slot 0); each
    // slot's barrier completes once per load, so its phase is the load count of that slot, mod 2.
    // Every thread waits on the barriers itself (the completed phase makes the copied data
    // visible to it); the per-plane __syncthreads_and makes the verdict of a bounded wait uniform.
    unsigned phase = 0u, pending = 0u;                      // bit s: slot s's phase / a copy in flight
    if (t == 0) {
        for (int s = 0; s < MARCH_SLOTS; ++s) mbar_init(&bar[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (t == 0) {
        march_load(&mapI, smem, &bar[0], bytes, (int)y0, (int)(xa > 0 ? xa - 1 : 0));
        march_load(&mapI, smem + SF, &bar[1], bytes, (int)y0, (int)xa);
        if (xa + 1 < xend) march_load(&mapI, smem + 2 * SF, &bar[2], bytes, (int)y0, (int)(xa + 1));
    }
    pending = xa + 1 < xend ? 7u : 3u;
    bool ok = true;
    // register queue: V_old and the class index of the next plane
    float4 vq[3] = {make_float4(0.f, 0.f, 0.f, 0.f), make_float4(0.f, 0.f, 0.f, 0.f), make_float4(0.f, 0.f, 0.f, 0.f)};
    uint4 cq = make_uint4(0u, 0u, 0u, 0u), cprev = make_uint4(0u, 0u, 0u, 0u);
    if (inV) {
        const unsigned long long o = xa * plane + yz;
        vq[0] = ldg4(g.V + o);
        vq[1] = ldg4(g.V + S + o);
        vq[2] = ldg4(g.V + 2 * S + o);
        cq = op_cls4(g, o);
    }
    bool w = mbar_wait(&bar[0], 0u);
    if (w) {                                                // a copy whose wait ran out is still in flight
        pending &= ~1u;
        phase ^= 1u;
    }
    for (unsigned x = xa; x < xend; ++x) {
        const unsigned sc = (x - xa + 1) % MARCH_SLOTS, sp = (x - xa) % MARCH_SLOTS;
        if (w) {
            w = mbar_wait(&bar[sc], (phase >> sc) & 1u);
            if (w) {
                pending &= ~(1u << sc);
                phase ^= 1u << sc;
            }
        }
        const float* Ic = smem + sc * SF;
        float* Ipl = smem + sp * SF;
        float4 vcur[3] = {vq[0], vq[1], vq[2]};
        const uint4 ccur = cq;
        if (inV && x + 1 < xend) {                          // next plane's V_old and classes
            const unsigned long long o = (x + 1) * plane + yz;
            vq[0] = ldg4(g.V + o);
            vq[1] = ldg4(g.V + S + o);
            vq[2] = ldg4(g.V + 2 * S + o);
            cq = op_cls4(g, o);
        }
        float* Vc = vbase + ((x - xa) & 1u) * VF;
        const float* Vp = vbase + ((x - xa + 1) & 1u) * VF;
        if (inV && w) {
            float4 out[3];
            march_v(m, Ic, Ipl, x, y, z0, rv + 1, vcur, ccur, ts, out);
#pragma unroll
            for (int c = 0; c < 3; ++c) st4(Vc + (c * (ty + 1) + rv) * Pz + z0, out[c]);
            if (ownV && x < xb) {
                const unsigned long long o = x * plane + yz;
                st4(f.Vo + o, out[0]);
                st4(f.Vo + S + o, out[1]);
                st4(f.Vo + 2 * S + o, out[2]);
            }
        }
        if (!__syncthreads_and(w)) {
            ok = false;
            break;
        }
        if (x > xa && ownV) {
            const unsigned long long o = (x - 1) * plane + yz;
            float4 out[3];
            if (inI) {
                march_i(m, Vp, Vc, Ipl, x - 1, y, z0, rv, cprev, ts, out);
            } else {                                        // I is never updated on this row: carry it over
                const unsigned r = rv + 1, rows = ty + 2;
                out[0] = lds4(Ipl + (0 * rows + r) * Pz + z0);
                out[1] = lds4(Ipl + (1 * rows + r) * Pz + z0);
                out[2] = lds4(Ipl + (2 * rows + r) * Pz + z0);
            }
            st4(f.Io + o, out[0]);
            st4(f.Io + S + o, out[1]);
            st4(f.Io + 2 * S + o, out[2]);
        }
        __syncthreads();
        // slot sp (plane x-1) is free: plane x+2 goes there
        if (x + 2 < xend) {
            if (t == 0) march_load(&mapI, Ipl, &bar[sp], bytes, (int)y0, (int)(x + 2));
            pending |= 1u << sp;
        }
        cprev = ccur;
    }
    if (!ok) {
        if (t == 0) atomicOr(m.err, 1u);
        // wait (bounded) for this block's copies still in flight before the block ends
        for (unsigned s = 0; s < MARCH_SLOTS; ++s)
            if ((pending >> s) & 1u) mbar_wait(&bar[s], (phase >> s) & 1u);
        return;
    }
    if (xb == g.Nx && ownV) {                               // the last plane: I is never updated
        const unsigned x = g.Nx - 1;
        const float* Il = smem + ((x - xa + 1) % MARCH_SLOTS) * SF;
        const unsigned r = rv + 1, rows = ty + 2;
        const unsigned long long o = x * plane + yz;
        st4(f.Io + o, lds4(Il + (0 * rows + r) * Pz + z0));
        st4(f.Io + S + o, lds4(Il + (1 * rows + r) * Pz + z0));
        st4(f.Io + 2 * S + o, lds4(Il + (2 * rows + r) * Pz + z0));
    }
}

}  // namespace oems
