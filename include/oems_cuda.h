/*
 * oems_cuda.h -- C ABI of the GB300 EC-FDTD engine (CUDA, sm_103a).
 *
 * The engine is a drop-in for openEMS's Engine path: it consumes the coefficients an openEMS
 * Operator builds (vv/vi/ii/iv, or the compressed operator) plus the tables its operator
 * extensions build, and runs Engine::IterateTS with the extension hooks fused into device
 * kernels.  Every entry point is extern "C", takes plain pointers and sizes, never throws and
 * returns an int status (OEMS_OK = 0).  Host arrays are owned by the caller and copied during
 * the call; device memory is owned by the engine handle.
 *
 * Layouts (all little-endian, C order):
 *   fields / dense coefficients : float [3][Nx][Ny][Nz]   (ArrayNIJK, tools/arraylib/array_nijk.h:58-62)
 *   index triples               : unsigned [3][count]     (x row, y row, z row)
 *
 * Threading: one handle belongs to one host thread and one CUDA stream (the engine's own).
 * Calls on different handles may run concurrently.
 *
 * Every declaration cites the reference interface it replaces.
 */
#ifndef OEMS_CUDA_H
#define OEMS_CUDA_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OEMS_OK               0
#define OEMS_ERR_ARG          1   /* invalid argument (sizes, indices, NULL pointers)          */
#define OEMS_ERR_CUDA         2   /* a CUDA runtime call failed; see oems_cuda_last_error      */
#define OEMS_ERR_STATE        3   /* call not allowed in the current state (e.g. before init)  */
#define OEMS_ERR_UNSUPPORTED  4   /* extension/feature not supported by this engine            */
#define OEMS_ERR_DEVICE       5   /* device-side status flag raised (non-finite field, ...)    */
#define OEMS_ERR_NOMEM        6   /* device allocation failed                                   */
#define OEMS_ERR_IO           8   /* a dump file could not be written                           */

/* which field for read/write calls */
#define OEMS_VOLT 0
#define OEMS_CURR 1

typedef struct oems_cuda_engine oems_cuda_engine;

/* ---- lifecycle ------------------------------------------------------------------------ */

/* Engine::New + Engine::Init (FDTD/engine.cpp:27-59): allocate zeroed fields for
 * numLines[0]*numLines[1]*numLines[2] mesh lines on device `device`. dt is the Operator's
 * timestep (Operator_Base::GetTimestep, Common/operator_base.h:37). */
int oems_cuda_create(const unsigned int num_lines[3], double dt, int device, oems_cuda_engine** out);

/* Engine::~Engine / Engine::Reset (FDTD/engine.cpp:100-108). Safe on NULL. */
void oems_cuda_destroy(oems_cuda_engine* eng);

/* Human-readable description of the last error on this handle (never NULL). */
const char* oems_cuda_last_error(const oems_cuda_engine* eng);

/* ---- operator coefficients ------------------------------------------------------------- */

/* Operator::vv_ptr/vi_ptr/ii_ptr/iv_ptr (FDTD/operator.h:364-367): dense float [3][Nx][Ny][Nz].
 * The engine deduplicates the per-cell 12-tuples like Operator_SSE_Compressed::CompressOperator
 * (FDTD/operator_sse_compressed.cpp:114-175, bitwise equality) and keeps the per-cell class
 * index on device; if the number of distinct tuples exceeds max_classes (0 = engine default)
 * the dense arrays are kept instead. */
int oems_cuda_set_operator(oems_cuda_engine* eng, const float* vv, const float* vi,
                           const float* ii, const float* iv, unsigned int max_classes);

/* Operator_SSE_Compressed's own tables (FDTD/operator_sse_compressed.h:70-85):
 * f4_{vv,vi,ii,iv}_Compressed[3] as float [3][num_vec_classes][4] and m_Op_index as
 * unsigned [Nx][Ny][nv], nv = ceil(Nz/4), with the lane-strided z mapping of
 * Engine_sse (FDTD/engine_sse.h:38-47): cell z lives in vector z % nv, lane z / nv. */
int oems_cuda_set_operator_sse_compressed(oems_cuda_engine* eng, unsigned int num_vec_classes,
                                          const float* f4_vv, const float* f4_vi,
                                          const float* f4_ii, const float* f4_iv,
                                          const unsigned int* op_index);

/* Number of coefficient classes in use (0 when dense arrays are used). */
int oems_cuda_operator_classes(const oems_cuda_engine* eng, unsigned int* num_classes);

/* ---- engine extensions (built tables of the matching Operator_Ext_*) --------------------- */

/* Engine_Ext_Excitation (FDTD/extensions/engine_ext_excitation.cpp:33-94) fed with
 * Operator_Ext_Excitation's Volt_* / Curr_* arrays (operator_ext_excitation.h:80-94) and the
 * Excitation signal (FDTD/excitation.h): sig_volt/sig_curr[length]; period = steps per signal
 * period (0 = aperiodic, p = numTS+1). Replaces any previous excitation. */
int oems_cuda_set_excitation(oems_cuda_engine* eng,
                             unsigned int volt_count, const unsigned int* volt_index,
                             const unsigned short* volt_dir, const float* volt_amp,
                             const unsigned int* volt_delay,
                             unsigned int curr_count, const unsigned int* curr_index,
                             const unsigned short* curr_dir, const float* curr_amp,
                             const unsigned int* curr_delay,
                             const float* sig_volt, const float* sig_curr, unsigned int length,
                             unsigned int period);

/* Engine_Ext_UPML (FDTD/extensions/engine_ext_upml.cpp:52-229) for one region of
 * Operator_Ext_UPML (operator_ext_upml.h:74-96): six float [3][rx][ry][rz] tables. Regions
 * must not overlap (Create_UPML builds them disjoint). At most 6 regions. */
int oems_cuda_add_upml(oems_cuda_engine* eng, const unsigned int start[3], const unsigned int num_lines[3],
                       const float* vv, const float* vvfo, const float* vvfn,
                       const float* ii, const float* iifo, const float* iifn);

/* Engine_Ext_Mur_ABC (FDTD/extensions/engine_ext_mur_abc.cpp:82-178) for one wall of
 * Operator_Ext_Mur_ABC: normal direction ny, wall line, shifted line, first active timestep,
 * coefficients float [numLines[nyP]][numLines[nyPP]]. Walls are applied in reverse call
 * order, as the reference's priority sort does. At most 6 walls. */
int oems_cuda_add_mur(oems_cuda_engine* eng, int ny, unsigned int line_nr, unsigned int line_nr_shift,
                      unsigned int start_ts, const float* coeff_nyP, const float* coeff_nyPP);

/* Engine_Ext_LorentzMaterial + Engine_Ext_Dispersive (engine_ext_lorentzmaterial.cpp:79-168,
 * engine_ext_dispersive.cpp:76-127) for one dispersion order of Operator_Ext_LorentzMaterial:
 * pos unsigned [3][count]; coefficient tables float [3][count] (NULL where the flag is off). */
int oems_cuda_add_lorentz_order(oems_cuda_engine* eng, unsigned int count, const unsigned int* pos,
                                int volt_ade_on, int curr_ade_on, int volt_lor_on, int curr_lor_on,
                                const float* v_int, const float* v_ext, const float* v_lor,
                                const float* i_int, const float* i_ext, const float* i_lor);

/* Engine_Ext_TFSF::DoPostVoltageUpdates / DoPostCurrentUpdates (FDTD/extensions/engine_ext_tfsf.cpp:36-215)
 * fed with Operator_Ext_TFSF's tables (FDTD/extensions/operator_ext_tfsf.h:55-84), flattened to one
 * term per (face plane, position, component) in the order the reference applies them: directions
 * n = x, y, z; lower plane before upper; the nP line outer, the nPP line inner; component nP before
 * nPP. Term k adds to field component dir[k] at cell index[.][k] ([3][count] like the excitation):
 *   F += (1.0 - delta)*amp*sig[lookup(delay)]  +  delta*amp*sig[lookup(delay + 1)]
 * with lookup(d) = m_DelayLookup[d] of the reference for the current numTS. The voltage terms add
 * the current signal sig_curr and the current terms the voltage signal sig_volt, as the reference
 * does. period = steps per signal period (0 = aperiodic); max_delay = m_maxDelay (every delay must
 * be below it). Replaces any previous TFSF setup. Engines with a TFSF source run the Mur pre/post
 * hooks as separate launches (the plane wave is added between the update and the Mur post hook). */
int oems_cuda_set_tfsf(oems_cuda_engine* eng, unsigned int volt_count, const unsigned int* volt_index,
                       const unsigned short* volt_dir, const unsigned int* volt_delay, const float* volt_delta,
                       const float* volt_amp, unsigned int curr_count, const unsigned int* curr_index,
                       const unsigned short* curr_dir, const unsigned int* curr_delay, const float* curr_delta,
                       const float* curr_amp, const float* sig_volt, const float* sig_curr, unsigned int length,
                       unsigned int period, unsigned int max_delay);

/* Engine_Ext_Cylinder (FDTD/extensions/engine_ext_cylinder.cpp:45-101) with Operator_Ext_Cylinder's
 * tables (FDTD/extensions/operator_ext_cylinder.cpp:44-112), for a mesh in cylindrical coordinates
 * (x = rho, y = alpha, z) whose operator Operator_Cylinder built. closed_alpha: the alpha lines
 * span 2*pi and line Ny-2 repeats line 0; after each voltage update the rho and z voltages of
 * line Ny-2 are copied onto line 0, after each current update the rho and z currents of line 0
 * onto line Ny-2. r0_included (closed meshes only): rho = 0 is the first line and the axis z
 * voltage becomes V*vv_r0[z] + sum over alpha lines 0..Ny-2 of vi_r0[z]*I_alpha (float, in that
 * order), written to every alpha line, with the alpha voltages on the axis set to zero; vv_r0 and
 * vi_r0 hold Nz floats. The post-voltage hook runs before the TFSF and Mur post hooks (priority
 * 1e5). Batched and adjoint runs reject it. */
int oems_cuda_set_cylinder(oems_cuda_engine* eng, int closed_alpha, int r0_included, const float* vv_r0,
                           const float* vi_r0);

/* Engine_Ext_LumpedRLC (FDTD/extensions/engine_ext_lumpedRLC.cpp:80-147) fed with
 * Operator_Ext_LumpedRLC's tables (FDTD/extensions/operator_ext_lumpedRLC.h:58-82): count lumped
 * edges, pos unsigned [3][count] (v_RLC_pos), dir int [count] (v_RLC_dir) and the float [count]
 * coefficient arrays v_RLC_ilv, v_RLC_i2v, v_RLC_vv2, v_RLC_vj1, v_RLC_vj2, v_RLC_vvd, v_RLC_ib0,
 * v_RLC_b1, v_RLC_b2. The engine keeps the parallel inductor current and the last three node
 * voltages and auxiliary currents of every edge; they start at zero and are part of a snapshot.
 * The apply hook runs after the post-voltage hooks and before the dispersive, Mur and excitation
 * apply hooks, as the reference's priority order has it. Two elements on one edge give
 * OEMS_ERR_ARG. Replaces any previous table. */
int oems_cuda_set_lumped_rlc(oems_cuda_engine* eng, unsigned int count, const unsigned int* pos, const int* dir,
                             const float* ilv, const float* i2v, const float* vv2, const float* vj1, const float* vj2,
                             const float* vvd, const float* ib0, const float* b1, const float* b2);

/* ---- processing: probes, DFTs, FD field dumps --------------------------------------------- */

/* ProcessVoltage (Common/processvoltage.cpp:38-48) -> Engine_Interface_FDTD::CalcVoltageIntegral
 * (FDTD/engine_interface_fdtd.cpp:206-232) on snapped start/stop indices (exactly one axis may
 * differ). Sampled when numTS % interval == 0 within [start_ts, stop_ts]; value*weight is
 * recorded as double. Returns the probe id (>= 0) through *id. */
int oems_cuda_add_voltage_probe(oems_cuda_engine* eng, const unsigned int start[3], const unsigned int stop[3],
                                double weight, unsigned int interval, unsigned int start_ts,
                                unsigned int stop_ts, int* id);

/* ProcessCurrent::CalcIntegral (Common/processcurrent.cpp:96-171): loop integral of currents in
 * the plane normal to norm_dir with the snapped dual-mesh box and inside flags. Time is the
 * dual time (numTS+0.5)*dt. */
int oems_cuda_add_current_probe(oems_cuda_engine* eng, const unsigned int start[3], const unsigned int stop[3],
                                int norm_dir, const int start_inside[3], const int stop_inside[3],
                                double weight, unsigned int interval, unsigned int start_ts,
                                unsigned int stop_ts, int* id);

/* ProcessFieldProbe (Common/processfieldprobe.cpp:77-92), probe types 2/3 of openems.cpp:541-544:
 * the E (field 0) or H (field 1) field at one Yee position without interpolation, i.e.
 * GetRawField / GetRawDualField (FDTD/engine_interface_fdtd.cpp:263-268, 136-142) = value /
 * el[n] (0 where el[n] == 0), el = GetEdgeLength(n, pos) of the main (E) or dual (H) mesh.
 * Three values per sample (series [slot][3], DFT [nf][3][re,im]); H uses the dual time. */
int oems_cuda_add_field_probe(oems_cuda_engine* eng, int field, const unsigned int pos[3], const double el[3],
                              double weight, unsigned int interval, unsigned int start_ts,
                              unsigned int stop_ts, int* id);

/* ProcessIntegral FD part (Common/processintegral.cpp:156-167): complex<double> DFT at
 * num_freqs frequencies, accumulated every fd_interval steps. */
int oems_cuda_set_probe_dft(oems_cuda_engine* eng, int probe_id, unsigned int fd_interval,
                            unsigned int num_freqs, const double* freqs);

/* ProcessFieldsFD (Common/processfields_fd.cpp:72-107) over the box start..stop (inclusive):
 * field 0 = E (main time), 1 = H (dual time); interp = the dump mode, i.e. the interpolation of
 * Engine_Interface_FDTD (FDTD/engine_interface_fdtd.cpp:63-204): 0 none (the raw Yee values),
 * 1 node interpolation, 2 cell interpolation. start/stop are the box snapped the way
 * ProcessFields snaps it (the dual mesh for cell interpolation and for H without interpolation).
 * edge_len[n] / dual_edge_len[n] are the mesh edge lengths in metres per line
 * (Operator::GetEdgeLength, FDTD/operator.cpp:212-215), float64 [numLines[n]] each,
 * concatenated x,y,z. Returns the dump id through *id. */
int oems_cuda_add_fd_dump(oems_cuda_engine* eng, int field, int interp, const unsigned int start[3],
                          const unsigned int stop[3], unsigned int fd_interval, unsigned int num_freqs,
                          const double* freqs, const double* edge_len, const double* dual_edge_len, int* id);

/* ProcessFieldsTD (Common/processfields_td.cpp:50-91): the dump box's E (field 0, main time) or H
 * (field 1, dual time) with interpolation `interp` (as for oems_cuda_add_fd_dump) at every step
 * numTS with numTS % interval == 0 within [start_ts, stop_ts] (Processing::CheckTimestep), numTS = 0
 * included. Each sample is written by a writer thread of the engine to
 * <file_prefix>_<numTS as 8 digits>.vtr, a VTK XML rectilinear grid (tools/vtk_file_writer.cpp:
 * 312-371 names the files the same way) holding the sample coordinates `coords` (metres, the
 * dump's x lines, then y, then z: stop-start+1 values per axis) and the vector field "E-Field" or
 * "H-Field" in float32, raw appended binary. The samples reach the host by asynchronous copies
 * into pinned buffers enqueued after each chunk of steps; the simulation does not wait for the
 * disk unless the writer falls four samples behind. Shares the id space of the FD dumps.
 * oems_cuda_profile_steps, the batched and the adjoint forms reject engines with TD dumps. */
int oems_cuda_add_td_dump(oems_cuda_engine* eng, int field, int interp, const unsigned int start[3],
                          const unsigned int stop[3], unsigned int interval, unsigned int start_ts,
                          unsigned int stop_ts, const double* edge_len, const double* dual_edge_len,
                          const double* coords, const char* file_prefix, int* id);

/* A dump (FD or time-domain) on a cylindrical mesh (x = rho, y = alpha), without interpolation
 * only: rho[N0] holds GetDiscLine(0, x) of the dump's mesh (main for E, dual for H) in drawing
 * units; the raw alpha value is divided by its edge length times rho, as
 * Operator_Cylinder::GetEdgeLength (FDTD/operator_cylinder.cpp:204-210) has it. Call before
 * oems_cuda_init. */
int oems_cuda_set_dump_rho(oems_cuda_engine* eng, int id, const double* rho);

/* Wait until every time-domain dump sample of the steps issued so far is written to its file;
 * OEMS_ERR_IO (with oems_cuda_last_error) if a file could not be written. oems_cuda_destroy
 * also finishes the pending files. */
int oems_cuda_flush_dumps(oems_cuda_engine* eng);

/* ---- run ------------------------------------------------------------------------------------ */

/* Finalise the setup: upload tables, size probe buffers for max_timesteps steps, capture the
 * per-step CUDA graph and record the probes at numTS = 0 (ProcessingArray::Process before the
 * first IterateTS, openems.cpp:1424-1425). */
int oems_cuda_init(oems_cuda_engine* eng, unsigned int max_timesteps);

/* Engine::IterateTS (FDTD/engine.cpp:267-286): n_steps full timesteps, asynchronous on the
 * engine's stream; probes/DFTs are recorded on device after each step. */
int oems_cuda_iterate(oems_cuda_engine* eng, unsigned int n_steps);

/* Wait for the engine's stream; returns OEMS_ERR_DEVICE if a device status flag was raised. */
int oems_cuda_sync(oems_cuda_engine* eng);

/* Engine::GetNumberOfTimesteps (FDTD/engine.h:49). Host-side count of issued steps. */
unsigned int oems_cuda_num_timesteps(const oems_cuda_engine* eng);

/* ---- field access (Engine::GetVolt/GetCurr/SetVolt/SetCurr, FDTD/engine.h:55-101) -------------- */
int oems_cuda_read_field(oems_cuda_engine* eng, int which, float* host_nijk);
int oems_cuda_write_field(oems_cuda_engine* eng, int which, const float* host_nijk);
int oems_cuda_get_value(oems_cuda_engine* eng, int which, unsigned int n, unsigned int x, unsigned int y,
                        unsigned int z, float* value);
int oems_cuda_set_value(oems_cuda_engine* eng, int which, unsigned int n, unsigned int x, unsigned int y,
                        unsigned int z, float value);

/* ---- results ---------------------------------------------------------------------------------- */

/* Probe time series: out[k] = value*weight at numTS = k*interval (NaN where not sampled),
 * k < cap; *count = number of slots written. */
int oems_cuda_read_probe(oems_cuda_engine* eng, int probe_id, double* out, size_t cap, size_t* count);

/* Slots [first, first+count) of a probe time series (same slot meaning as above). Used by a
 * caller that, like ProcessingArray::Process (Common/processing.cpp:355-366), fetches the newest
 * samples after every IterateTS chunk. Synchronises the engine stream. The newest sample
 * (count = 1, the slot of the last step) comes from a mapped host copy the step writes, with no
 * device copy; other short ranges (count <= 64) are fetched for every probe at once into pinned
 * memory and served from there until the engine steps again or is restored. */
int oems_cuda_read_probe_range(oems_cuda_engine* eng, int probe_id, size_t first, size_t count, double* out);

/* Probe DFT: out[2*f], out[2*f+1] = real, imag at frequency f (double). */
int oems_cuda_read_probe_dft(oems_cuda_engine* eng, int probe_id, double* out);

/* FD dump: complex<float> [num_freqs][3][sx][sy][sz] as interleaved re/im floats. */
int oems_cuda_read_fd_dump(oems_cuda_engine* eng, int dump_id, float* out, size_t cap_floats);

/* ProcessFieldsFD::DumpFDData with the VTK file type (Common/processfields_fd.cpp:114-215): writes
 * the accumulated FD dump as VTK XML rectilinear-grid files, per frequency 21 phase snapshots
 * <prefix>_f=<freq>_p=<degrees>.vtr plus <prefix>_f=<freq>_abs.vtr and _arg.vtr, with the
 * reference's names and complex<float> arithmetic.  coords: the sample coordinates in metres,
 * x then y then z (sx + sy + sz values).  Errors writing a file give OEMS_ERR_IO. */
int oems_cuda_write_fd_dump(oems_cuda_engine* eng, int dump_id, const char* prefix, const double* coords);

/* Engine_Interface_FDTD::CalcFastEnergy (FDTD/engine_interface_fdtd.cpp:302-347):
 * eps0*sum(V^2) + mu0*sum(I^2) over [0,N-1)^3, device reduction in double. */
int oems_cuda_energy(oems_cuda_engine* eng, double* energy);

/* Allocation-free variant of the energy reduction, with no counterpart in the reference. It
 * serves callers that must not call cudaMalloc: their device memory is owned by a host
 * framework's pool or arena (a raw allocation would bypass its accounting), or their deployment
 * forbids device allocation after start-up. The caller passes its own
 * device fields volt_dev/curr_dev, float [3][Nx][Ny][z_stride] with z_stride >= Nz, and a host
 * `energy`. The reduction uses a fixed 128 KB scratch array that is part of the library image,
 * so the entry point allocates nothing. Limit: Nx-1 <= OEMS_NOALLOC_MAX_PLANES x-planes; larger
 * meshes return OEMS_ERR_TOO_LARGE. The first call on a device resolves the scratch address
 * with that device current, so make it before any stream capture. All calls share the scratch,
 * so calls that overlap on the GPU (different streams at once) race. `stream` is a
 * cudaStream_t, or NULL for the default stream. The call synchronizes that stream. */
#define OEMS_NOALLOC_MAX_PLANES 8192
#define OEMS_ERR_TOO_LARGE    7
int oems_cuda_energy_noalloc(const float* volt_dev, const float* curr_dev, const unsigned int num_lines[3],
                             unsigned int z_stride, void* stream, double* energy);

/* ---- batched form ------------------------------------------------------------------------------ */

/* Many independent simulations (engine handles already through oems_cuda_init, same device),
 * advanced together. Replaces running openEMS once per excitation/geometry variant (the loop a
 * user writes around openEMS.Run, python/openEMS/openEMS.pyx:513-564, e.g. one run per port of an
 * S-parameter sweep). Supported per instance: excitation, UPML, probes and probe DFTs;
 * instances with Mur walls, dispersive materials or FD dumps give OEMS_ERR_UNSUPPORTED. The
 * batch references the engines' device state; destroy it before the engines. */
typedef struct oems_cuda_batch oems_cuda_batch;
int oems_cuda_batch_create(oems_cuda_engine* const* engines, unsigned int count, oems_cuda_batch** out);

/* Advance instance k by steps[k] timesteps (uneven counts allowed), in chunks over the instances
 * active throughout each chunk. Execution modes: persistent cooperative launches (one per
 * chunk, all chunks in one CUDA graph); per-phase launches over every instance (depth flag
 * 0x80000000) or over L2-sized instance groups (0xC0000000); concurrent graph branches, one per
 * instance with its own step kernels (0x20000000), or the same over L2-sized groups
 * (0x10000000). block_size/depth = 0 lets the built-in autotuner time the candidate (mode,
 * block size, x-planes per work item) sets on the first steps and keep the fastest (the tuning
 * steps are real steps). Results are bit-identical to running each engine alone with
 * oems_cuda_iterate. */
int oems_cuda_batch_run(oems_cuda_batch* b, const unsigned int* steps, unsigned int block_size, unsigned int depth);

/* The configuration in use, whether the launches ran from a captured graph, and the autotuner's
 * per-candidate timings (ms for the same number of steps each). */
int oems_cuda_batch_config(const oems_cuda_batch* b, unsigned int* block_size, unsigned int* depth, int* used_graph,
                           float* tune_ms, unsigned int* num_candidates);

void oems_cuda_batch_destroy(oems_cuda_batch* b);

/* ---- adjoint (reverse-mode) form --------------------------------------------------------------- */

/* Gradients of an objective built from probe samples with respect to the voltage coefficients
 * vv/vi of the edges in a design box. No reference counterpart: openEMS has no derivative
 * path; this is what an optimisation loop around python/openEMS/openEMS.pyx:513-564 (one
 * forward run per trial design) would call instead of finite differences.
 *
 * setup: after oems_cuda_init on a fresh engine. The design box covers the mesh nodes
 * box_start..box_stop-1 and may not overlap a UPML region; engines with Mur walls or dispersive
 * materials give OEMS_ERR_UNSUPPORTED. checkpoint_every = K: the forward run stores the full
 * state every K steps, the reverse sweep recomputes one K-step segment at a time. */
int oems_cuda_adjoint_setup(oems_cuda_engine* eng, unsigned int checkpoint_every, const unsigned int box_start[3],
                            const unsigned int box_stop[3]);
/* Forward run of `steps` timesteps from numTS = 0 with checkpoints; probes record as usual. */
int oems_cuda_adjoint_forward(oems_cuda_engine* eng, unsigned int steps);
/* Reverse sweep. sources[k*(steps+1) + n] = dJ/d(sample of probe probe_ids[k] at numTS = n)
 * (the weighted line integral of the probe, before any DFT). Writes dJ/dvv and dJ/dvi of the
 * design box edges, double [3][bx][by][bz] each (component-major, z fastest). The engine is
 * left at its forward end state. */
int oems_cuda_adjoint_backward(oems_cuda_engine* eng, unsigned int nprobe, const int* probe_ids, const double* sources,
                               double* grad_vv, double* grad_vi);
/* Device time (CUDA events on the engine stream) of the last adjoint forward and backward calls,
 * and the kernel launches per reverse step (any pointer may be NULL). */
int oems_cuda_adjoint_timing(const oems_cuda_engine* eng, float* forward_ms, float* backward_ms,
                             unsigned int* launches_per_reverse_step);

/* ---- NF2FF far-field transform ------------------------------------------------------------------ */

/* Replaces nf2ff_calc (nf2ff/nf2ff_calc.cpp:41-160, 329-530) run on the HDF5 FD dumps of an
 * NF2FF box: the transform reads the E/H FD-dump accumulators on the device directly. Face f
 * is the pair (e_dumps[f], h_dumps[f]) of FD dumps (E and H, same planar box, more than two
 * lines per tangential axis). coords holds, face after face, the sample coordinates in metres
 * along x, then y, then z (the dual mesh lines of a cell-interpolated dump). Cartesian meshes,
 * no mirror planes. freq_index selects the dumps' frequency, freq is its value in Hz. Outputs
 * for theta[i], phi[j] at index i*nphi + j: e_theta and e_phi (complex, re/im interleaved),
 * p_rad (W/m^2 at `radius` metres); rad_power (W, through the faces) and max_dir may be NULL. */
int oems_cuda_nf2ff(oems_cuda_engine* eng, unsigned int nface, const int* e_dumps, const int* h_dumps,
                    const double* coords, unsigned int freq_index, double freq, unsigned int ntheta,
                    const double* theta, unsigned int nphi, const double* phi, const double center[3], double radius,
                    double eps_r, double mu_r, double* e_theta, double* e_phi, double* p_rad, double* rad_power,
                    double* max_dir);

/* ---- operator numerics on the device --------------------------------------------------------------- */

/* Replaces the per-edge loops of Operator::CalcECOperator (FDTD/operator.cpp:986-1097):
 * AverageMatQuarterCell (:1447-1564), Calc_ECPos (:1189-1254), CalcTimestep_Var3 (:1956-2030) and
 * Calc_ECOperatorPos (:956-984), for geometries described as material boxes. lines: the mesh lines
 * of x, then y, then z (drawing units, num_lines each), unit: metres per drawing unit. Paint
 * records in painting order, the last record containing a sample point wins (ascending priority,
 * among equal priorities the earliest-defined box last): rec_lo/rec_hi [nrec][3] (drawing units,
 * inclusive), rec_par [nrec][4] = eps_r, kappa, mu_r, sigma; background [4] the same for points
 * outside every record. Results are bit-identical to the host restatement. */
typedef struct oems_cuda_opbuild oems_cuda_opbuild;
int oems_cuda_opbuild_create(const unsigned int num_lines[3], const double* lines, double unit, unsigned int nrec,
                             const double* rec_lo, const double* rec_hi, const double* rec_par,
                             const double background[4], oems_cuda_opbuild** out);
/* C, G, L, R of every edge (float [3][Nx][Ny][Nz] each, x,y,z order; any may be NULL) and, if
 * dt_var3 is not NULL, the Var3 timestep (1e200 if no node gives a finite positive one). */
int oems_cuda_opbuild_ec(oems_cuda_opbuild* b, float* C, float* G, float* L, float* R, double* dt_var3);
/* vv, vi, ii, iv for timestep dt (float [3][Nx][Ny][Nz] each), before boundary conditions. */
int oems_cuda_opbuild_coefficients(oems_cuda_opbuild* b, double dt, float* vv, float* vi, float* ii, float* iv);
const char* oems_cuda_opbuild_last_error(const oems_cuda_opbuild* b);
void oems_cuda_opbuild_destroy(oems_cuda_opbuild* b);

/* ---- checkpoint / resume --------------------------------------------------------------------- */

/* Size in bytes of a snapshot of the full engine state (fields, UPML fluxes, Mur buffers,
 * dispersive states, numTS, probe and DFT accumulators). */
int oems_cuda_snapshot_size(const oems_cuda_engine* eng, size_t* bytes);
/* Copy the state to host memory (`bytes` must be >= snapshot size). */
int oems_cuda_snapshot(oems_cuda_engine* eng, void* host, size_t bytes);
/* Restore a state written by oems_cuda_snapshot of an engine with the same setup. */
int oems_cuda_restore(oems_cuda_engine* eng, const void* host, size_t bytes);

/* ---- introspection ----------------------------------------------------------------------------- */

/* Number of kernel launches issued per timestep by the captured step graph. */
int oems_cuda_launches_per_step(const oems_cuda_engine* eng, unsigned int* launches);

/* The kernels that carry the voltage and current updates in this engine's configuration (after
 * oems_cuda_init), e.g. "k_update_v4w" / "k_update_i4", or "k_step_march" for both: NUL-terminated
 * names written into `volt` and `curr`, each buffer `cap` bytes. */
int oems_cuda_update_kernels(oems_cuda_engine* eng, char* volt, char* curr, size_t cap);

/* Run n_steps through the captured step graph and return their device time in ms (CUDA events
 * on the engine stream). */
int oems_cuda_timed_iterate(oems_cuda_engine* eng, unsigned int n_steps, float* ms);

/* Kernel classes reported by oems_cuda_profile_steps. */
#define OEMS_KC_UPDATE_V  0
#define OEMS_KC_UPDATE_I  1
#define OEMS_KC_MUR       2   /* boundary hooks: Mur walls and the cylinder's alpha seam / axis */
#define OEMS_KC_LORENTZ   3   /* auxiliary-equation kernels: Drude/Lorentz and lumped RLC */
#define OEMS_KC_EXCITE    4
#define OEMS_KC_STEP_END  5
#define OEMS_KC_COUNT     6

/* Run n_steps with every kernel launched directly on the engine stream, bracketed by CUDA events;
 * ms[k] = summed device time of kernel class k, launches[k] = number of launches (either may be
 * NULL). Same results as oems_cuda_iterate. */
int oems_cuda_profile_steps(oems_cuda_engine* eng, unsigned int n_steps, float* ms, unsigned int* launches);

#ifdef __cplusplus
}
#endif

#endif /* OEMS_CUDA_H */
