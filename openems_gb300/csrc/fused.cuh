// fused.cuh -- the plumbing of a one-kernel timestep (k_step_march, march.cuh): the buffer sets
// the step ping-pongs between and the soft excitation applied inside it.
//
// A one-kernel step reads V and I once and writes them once (52 bytes per cell-step with the class
// index, against 80 for the two separate half-step kernels), so it cannot update in place: the
// step reads (V, I) from one buffer set and writes the other.  The K-step graph alternates the
// two; K is even, so the state is in the primary set whenever the host sees it.  The soft sources
// of Engine_Ext_Excitation::Apply2Voltages / Apply2Current (FDTD/extensions/
// engine_ext_excitation.cpp:33-94) are added by the thread that updates the source cell, with
// k_excitation's arithmetic, so results stay bit-identical.
#pragma once

#include "kernels.cuh"

namespace oems {

constexpr int FT_MAX_SRC = 64;   // sources the one-kernel step adds inline (engines with more keep the separate kernels)

struct FusedDev {
    GridDev g;                 // V, I: the buffers read by this step
    float* Vo;                 // written by this step
    float* Io;
    ExcDev excV, excI;
    const unsigned long long* srcV_cell;   // excitation cells (component removed), per source
    const unsigned long long* srcI_cell;
    unsigned long long srcV_lo, srcV_hi, srcI_lo, srcI_hi;
    const unsigned* numTS;
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

}  // namespace oems
