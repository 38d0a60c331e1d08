// engine_impl.h -- private definition of the engine handle, shared by engine.cu and batch.cu.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include "../../include/oems_cuda.h"
#include "kernels.cuh"
#include "fused.cuh"
#include "march_dev.h"

using namespace oems;

namespace oems_host {

const double kPI = 3.14159265358979323846;  // M_PI as used by Common/processintegral.cpp:161

struct UpmlHost {
    unsigned start[3], nl[3];
    std::vector<float> tab[6];  // vv, vvfo, vvfn, ii, iifo, iifn
};
struct ProbeCache {
    double* pin = nullptr;           // pinned host copy of slots [first, first + count) per probe
    size_t cap = 0;
    std::vector<size_t> off;         // per probe: offset in pin, or SIZE_MAX
    bool valid = false;
    unsigned long long ts = 0;
    unsigned gen = 0;
    size_t first = 0, count = 0;
};
struct MurHost {
    int ny;
    unsigned line, shift, start_ts;
    std::vector<float> cP, cPP;
};
struct LorHost {
    unsigned count;
    std::vector<unsigned> pos;
    int von, con, vlon, clon;
    std::vector<float> vint, vext, vlor, iint, iext, ilor;
};
struct ProbeHost {
    int type;                      // 0 voltage, 1 current, 2 E field, 3 H field
    unsigned start[3], stop[3];
    double el[3] = {0, 0, 0};      // field probes: edge lengths at start
    int nd, si[3], ei[3];
    double weight;
    unsigned interval, start_ts, stop_ts;
    unsigned fd_interval = 0;
    std::vector<double> freqs;
};
struct TfsfHost {
    // terms in the reference's application order: target offset, delay, delta, amp
    std::vector<unsigned long long> off;
    std::vector<unsigned> delay;
    std::vector<float> delta, amp;
};
struct RlcHost {
    std::vector<unsigned long long> off;
    std::vector<float> c;   // [9][count]
};
struct DumpHost {
    int field;
    int interp = 2;          // 0 none, 1 node, 2 cell interpolation
    // time-domain dump (oems_cuda_add_td_dump): samples written to VTK files by the writer
    bool td = false;
    unsigned td_interval = 1, td_start = 0, td_stop = 0xFFFFFFFFu;
    std::string prefix;
    std::vector<double> coords;   // sample coordinates in metres, x then y then z
    unsigned start[3], stop[3];
    unsigned fd_interval;
    std::vector<double> freqs;
    std::vector<double> el;  // edge lengths used by this field type, concatenated x,y,z
    std::vector<double> rho; // cylindrical mesh: rho per x line of the dump's mesh (empty otherwise)
};

}  // namespace oems_host

using namespace oems_host;

// adjoint state (adjoint.cu); freed by oems_cuda_destroy
struct oems_adjoint_state;
void oems_adjoint_free(oems_adjoint_state* s);

// time-domain dump pipeline (tddump.cu): device ring -> pinned host buffers -> writer thread
struct oems_td_pipeline;
struct oems_cuda_engine;
int td_start_pipeline(oems_cuda_engine* e);            // after the device structs exist
int td_iterate(oems_cuda_engine* e, unsigned n);        // oems_cuda_iterate for engines with TD dumps
int td_flush(oems_cuda_engine* e);                      // enqueue the copies of every pending sample
int td_wait(oems_cuda_engine* e);                       // wait until every enqueued sample is written
void td_free(oems_cuda_engine* e);

struct oems_cuda_engine {
    int device = 0;
    cudaStream_t stream = nullptr;
    unsigned N[3] = {0, 0, 0};
    unsigned Pz = 0;
    unsigned long long S = 0;
    double dt = 0;
    std::string err;

    // fields
    float* dV = nullptr;
    float* dI = nullptr;

    // operator
    bool op_set = false;
    bool compressed = false;
    unsigned nclasses = 0;
    unsigned* didx = nullptr;
    float4* dtabV = nullptr;
    float4* dtabI = nullptr;
    float *dvv = nullptr, *dvi = nullptr, *dii = nullptr, *div = nullptr;

    // extensions (host copies until init)
    bool has_exc = false;
    std::vector<unsigned long long> exc_voff, exc_ioff;
    std::vector<float> exc_vamp, exc_iamp, sig_v, sig_i;
    std::vector<unsigned> exc_vdelay, exc_idelay;
    unsigned sig_len = 0, period = 0;
    std::vector<UpmlHost> upml;
    std::vector<MurHost> mur;
    std::vector<LorHost> lor;
    std::vector<ProbeHost> probes;
    std::vector<DumpHost> dumps;
    // TFSF plane wave (one per engine, as Operator_Ext_TFSF builds one)
    bool has_tfsf = false;
    TfsfHost tfsf_v, tfsf_i;
    std::vector<float> tfsf_sig_v, tfsf_sig_i;
    unsigned tfsf_len = 0, tfsf_period = 0;
    // lumped RLC loads
    RlcHost rlc_host;
    // cylinder extension: closed alpha mesh, rho = 0 on it, axis coefficients [Nz]
    int cyl_closed = 0, cyl_r0 = 0;
    std::vector<float> cyl_vv_r0, cyl_vi_r0;

    // device state after init
    bool inited = false;
    unsigned max_ts = 0;
    unsigned* d_numTS = nullptr;
    unsigned* d_zero = nullptr;       // a device 0 (the lane-parallel Mur hooks' step)
    unsigned* d_blocks_done = nullptr;
    unsigned host_numTS = 0;
    GridDev grid{};
    ExcDev excV{}, excI{};
    TfsfDev tfsfV{}, tfsfI{};
    RlcDev rlc{};
    CylDev cyl{};
    MurDev murdev{};
    std::vector<LorDev> lorV, lorI;
    StepEndDev stepend{};
    unsigned stepend_blocks = 1;
    std::vector<ProbeDev> probe_dev;   // host mirror of device structs
    std::vector<DumpDev> dump_dev;
    unsigned launches = 0;
    cudaGraphExec_t graph1 = nullptr;
    cudaGraphExec_t graphK = nullptr;
    unsigned K = 16;
    double* d_energy_partial = nullptr;
    unsigned energy_blocks = 0;

    std::vector<void*> allocs;                            // freed on destroy
    std::vector<std::pair<void*, size_t>> state;          // snapshot regions (device)
    oems_adjoint_state* adj = nullptr;
    oems_td_pipeline* td = nullptr;
    bool has_td = false;
    // UPML work split of the update launches (used when the engine has UPML regions)
    bool use_split = false;
    SplitDev splitV{}, splitI{};
    // float4 split: the region kernel's branch stream and its fork/join events
    cudaStream_t stream_r = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // Mur pre/post hooks as separate launches (k_mur phases 0/1) instead of inside the voltage
    // update; set by OEMS_CUDA_MUR_SEPARATE=1 at init
    bool mur_separate = false;
    // float4 forms of the update kernels (4 z cells per thread) where they exist
    bool vec4 = true;
    // the voltage update with the Mur hooks in the float4 form (k_update_v4w)
    bool mur_v4 = false;
    unsigned i4_block = 128;         // threads per block of k_update_i4
    unsigned v4_block = 64;          // threads per block of k_update_v4 / k_update_v4w
    unsigned box_block = 128;        // threads per block of k_update_box4
    unsigned reg_block = 128;        // threads per block of k_update_reg4 (128 or 256)
    unsigned adj_box_block = 128, adj_reg_block = 128;   // the same for k_adj_box4 / k_adj_reg4
    // dispersive apply + next pre as one launch inside enqueued sequences (k_lorentz_carry)
    bool lor_carry_v = false, lor_carry_i = false;
    bool vtail = false;              // k_vtail: Mur apply + carry + excitation as one launch
    // newest-sample reads of the probes (oems_cuda_read_probe_range): one pinned fetch per step
    ProbeCache pcache;
    double* latest_host = nullptr;   // mapped: each probe's newest sample (ProbeDev::latest)
    unsigned* latest_slot_host = nullptr;
    unsigned series_gen = 0;         // bumped by restore
    // the step end in two parts on a side stream (k_step_end part 0 beside the current update,
    // part 1 beside the next voltage update); se_pending: part 1 forked, not yet joined
    bool se_split = false, se_pending = false;
    cudaStream_t stream_se = nullptr;
    cudaEvent_t ev_se_fork = nullptr, ev_se_a = nullptr, ev_se_b = nullptr;

    // one-kernel step (the plane march, march.cuh): the K-step graph alternates buffer sets A
    // (dV, dI) and B (dV2, dI2); K is even, so the state is in A whenever the host sees it
    bool use_fused = false;
    float* dV2 = nullptr;
    float* dI2 = nullptr;
    FusedDev fused[2]{};
    unsigned fused_launches = 0;
    // TMA-staged plane march (march.cuh): the buffer sets and parities above, one kernel per
    // step, for compressed engines with PEC/PMC walls only; the maps describe I of sets A and B
    bool use_march = false;
    MarchDev march[2]{};
    CUtensorMap march_map[2]{};                 // 64-byte aligned by its own declaration
    dim3 march_grid{1, 1, 1};
    unsigned march_threads = 0, march_smem = 0;
    int march_minb = 1;
    unsigned* d_march_err = nullptr;
    // the march and the separate kernels both captured, the faster chosen on the first iterate
    // that runs at least four K-step graphs (OEMS_CUDA_MARCH unset); graphK_alt holds the other
    bool march_tune = false;
    cudaGraphExec_t graphK_alt = nullptr;
    float march_tune_ms[2] = {0.f, 0.f};   // one K-step graph: march, separate kernels
};

// enqueue one one-kernel timestep on e->stream: parity 0 reads set A and writes B, parity 1 the reverse
int enqueue_fused_step(oems_cuda_engine* e, int parity, unsigned* nlaunch);

// the split for update range R (V: the mesh, I: one cell less per axis)
void make_split(const oems_cuda_engine* e, const unsigned R[3], SplitDev& sp);
// one update launch (V or I) of the engine's kernel configuration on stream s
// name != nullptr: only report the kernel name this configuration launches.  fac != nullptr: the
// voltage update's float4 main box also writes the design-box factors of the reverse sweep (used
// by the recomputation when the engine runs the split with a float4 main box)
void launch_update(oems_cuda_engine* e, bool curr, cudaStream_t s, const char** name = nullptr,
                   const FacOut* fac = nullptr);
// per-cell coefficient classes of dense N-I-J-K arrays on the device (compress.cu): 0 = built,
// 1 = more than `cap` classes, else an OEMS error code
int compress_dense_device(oems_cuda_engine* e, const float* vv, const float* vi, const float* ii, const float* iv,
                          unsigned cap);


// per-launch events for oems_cuda_profile_steps (never used inside a captured graph)
struct StepProfiler {
    cudaEvent_t ev[2 * 64];
    int cls[64];
    int n = 0;
};

// enqueue one timestep of `e` on e->stream (defined in engine.cu)
int enqueue_step(oems_cuda_engine* e, unsigned* nlaunch, StepProfiler* prof = nullptr, unsigned seq = 3);
