// march_dev.h -- launch parameters of the TMA-staged plane-march step (k_step_march, march.cuh).
#pragma once

#include "fused.cuh"

namespace oems {

struct MarchDev {
    FusedDev f;            // input set (f.g), output buffers, sources, step counter
    unsigned ty;           // output rows per tile
    unsigned groups;       // float4 groups per row (Pz / 4)
    unsigned xchunk;       // x-planes per block
    unsigned slot_floats;  // floats of one ring slot: 3 * (ty + 2) * Pz, rounded up to 128 bytes
    unsigned box_bytes;    // bytes one load delivers: 12 * (ty + 2) * Pz
    unsigned vbuf_floats;  // floats of one V' buffer: 3 * (ty + 1) * Pz, rounded up to 128 bytes
    unsigned* err;         // device error flag
};

}  // namespace oems
