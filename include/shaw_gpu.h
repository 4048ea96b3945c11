/*
 * shaw_gpu.h -- C ABI of the GB300 (sm_103a) implementation of SHAW's two
 * data-parallel hot paths:
 *   (a) the full-order (FOM) velocity-stress leapfrog on the staggered
 *       axisymmetric (r, theta) grid, rank-1 (one forcing) and rank-2 (M forcings);
 *   (b) the Galerkin ROM leapfrog on the reduced operators.
 *
 * Conventions (the same for every entry point):
 *   - every function returns an int status (SHAW_OK == 0); no exception crosses
 *     the ABI.  shaw_last_error() gives a one-line message for the calling thread.
 *     The status codes mirror the reference's throw sites.
 *   - caller-owned host arrays are copied in; the library owns all device memory.
 *   - one CUDA stream per handle (shaw_*_stream); a handle is not thread-safe.
 *   - gids follow the reference's mesh files: vp gid = j*nth + i (theta fastest),
 *     sp gids interleaved per cell (srp, then stp), see meshing/helpers/full_mesh_utils.py.
 *   - multi-column host arrays are column-major ("LayoutLeft"), as the
 *     reference's host views are when written to file.
 *
 * Reference interfaces replaced (paths inside the reference project):
 *   ShWavePP ctor + fillVpJacobian/fillSpJacobian  src/kokkos/shwavepp.hpp:100-148,319-466
 *   updateVelocity / updateStress                  src/kokkos/fom_update_kernels.hpp:60-181
 *   runFom                                         src/kokkos/fom_run.hpp:66-161
 *   RankOneForcing / RankTwoForcing                src/kokkos/forcing_rank_one.hpp:56-179,
 *                                                  src/kokkos/forcing_rank_two.hpp:56-173
 *   Seismogram                                     src/kokkos/seismogram.hpp:82-233
 *   StateObserver                                  src/kokkos/state_observer.hpp:81-231
 *   computeRomOperatorsUsingFomJacsWithMatProp     src/kokkos/rom_compute_jacobians.hpp:59-109
 *   runRomRankOneForcing                           src/kokkos/rom_run_rank_one.hpp:91-162
 *   runRomRankTwoForcing                           src/kokkos/torevise/run_rom_rank_two_forcing.hpp:119-201
 *   reconstructSeismogram (ROM seismogram)         src/tools/main_reconstruct_seismo.cc:147-190
 *   computeThinSVD (POD)                           src/tools/main_eigen_svd.cc:113-197
 */
#ifndef SHAW_GPU_H_
#define SHAW_GPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define SHAW_OK                 0
#define SHAW_ERR_INVALID_ARG    1  /* bad pointer / size / enum value                        */
#define SHAW_ERR_CUDA           2  /* a CUDA runtime call failed                              */
#define SHAW_ERR_MESH           3  /* mesh files missing/malformed, or not a full structured mesh */
#define SHAW_ERR_FREQ_DIVISOR   4  /* sampling freq does not divide the step count
                                      (seismogram.hpp:163-169, state_observer.hpp:130-143)   */
#define SHAW_ERR_CFL            5  /* check_cfl.hpp:66-73                                     */
#define SHAW_ERR_DISPERSION     6  /* check_dispersion_criterion.hpp:68-81                    */
#define SHAW_ERR_FORCING_SETS   7  /* realizations not divisible by forcingSize
                                      (fom_problem_rank_two.hpp:136-139)                      */
#define SHAW_ERR_NONFINITE      8  /* NaN/Inf seen in a sampled state                         */
#define SHAW_ERR_IO             9  /* file could not be opened / written                      */
#define SHAW_ERR_PARSE         10  /* input file invalid (throw sites of src/shared/parser/)  */
#define SHAW_ERR_UNSUPPORTED   11  /* valid input outside what this build implements          */
#define SHAW_ERR_OUT_OF_MEMORY 12
#define SHAW_ERR_STATE         13  /* call order violated (e.g. run before set_sources)      */

/* ---- signal kinds (src/shared/enums/supported_signal_enums.hpp) --------- */
#define SHAW_SIGNAL_RICKER    0
#define SHAW_SIGNAL_SINUSOID  1
#define SHAW_SIGNAL_GAUSS_DER 2

/* ---- arithmetic of a run ------------------------------------------------ */
#define SHAW_FP64             0  /* plain FP64 (the oracle-parity path)                     */
#define SHAW_MIXED_TF32X3     1  /* EXPERIMENTAL, ROM rank 2 only: split TF32x3 products with
                                    FP32 accumulation.  Kept as a measured negative result:
                                    the tensor pipe's truncating FP32 accumulation drifts
                                    (7.5e-6 relative seismogram error after 100 steps at
                                    k = 512), so it does NOT meet the 1e-6 mixed-precision
                                    bar; use SHAW_MIXED_OZAKI_BF16.  (Value 2 is unused:
                                    no BF16x3 form is built, for the same reason.)        */
#define SHAW_MIXED_FP32       3  /* ROM rank 1: FP32 hi+lo arithmetic; FOM: FP32 state     */
#define SHAW_MIXED_OZAKI_BF16 4  /* ROM rank 2: BF16 tensor cores, 6 six-bit slices per
                                    operand (Ozaki scheme), exact FP32 accumulation,
                                    compensated FP32 state (~2^-36 products)             */
#define SHAW_OZAKI_FP64       5  /* ROM rank 2: BF16 tensor cores, 9 six-bit slices per
                                    operand, exact FP32 accumulation, FP64 state:
                                    FP64-grade results at tensor-core speed               */

const char* shaw_last_error(void);
const char* shaw_version(void);

/* ======================================================================== *
 *  FOM                                                                      *
 * ======================================================================== */

/* What ShWavePP reads from the mesh directory and the material model
 * (src/kokkos/shwavepp.hpp:100-146).  Arrays are indexed by gid. */
typedef struct {
  uint64_t nth, nr;             /* grid points along theta / r (mesh_info.dat)          */
  uint64_t nvp, nsp;            /* numPtsVp, numPtsSp                                    */
  double dth_inv;               /* 1/dth  [1/rad]                                        */
  double drr_inv;               /* 1/dr   [1/m]                                          */
  const int64_t* graph_vp;      /* nvp x 5 row-major: gid, W, N, E, S  (graph_vp.dat)    */
  const int64_t* graph_sp;      /* nsp x 3 row-major: gid, first, second (graph_sp.dat)  */
  const int32_t* labels_sp;     /* nsp: 1 = srp (sigma_r,phi), 2 = stp (sigma_theta,phi) */
  const double* coords_vp;      /* nvp x 2: theta [rad], 1/r [1/m]                       */
  const double* coords_sp;      /* nsp x 2                                               */
  const double* cot_vp;         /* nvp: cot(theta), 0 on the symmetry axis               */
  const double* cot_sp;         /* nsp                                                   */
  const double* coeff_vp;       /* nvp x 4: boundary factors c0..c3 (coeff_vp.dat)       */
  const double* rho_inv_vp;     /* nvp: 1/density                                        */
  const double* shear_mod_sp;   /* nsp: density * vs^2                                   */
} shaw_fom_operator_desc;

typedef struct shaw_fom_s* shaw_fom_t;

/* ShWavePP ctor + state allocation of FomProblemRank{One,Two}Forcing.
 * rank 1: one forcing, vector state, source added as KokkosBlas::mult does;
 * rank 2: num_forcings columns, source added as AddForcingRank2 does.
 * precision: SHAW_FP64, or SHAW_MIXED_FP32: FP32 state and dt-folded stencil values
 * (rounded from the FP64 values), FP32 FMAs, source increments computed in FP64 and
 * rounded once; half the HBM bytes of FP64.  Snapshots, seismograms and states are
 * returned in FP64.  Not an oracle-parity path: its seismograms differ from FP64 by
 * ~1e-6 relative (measured, grows slowly with grid size and step count). */
int shaw_fom_create(const shaw_fom_operator_desc* desc, int rank, uint32_t num_forcings, int precision,
                    shaw_fom_t* out);
void shaw_fom_destroy(shaw_fom_t h);

/* RankOneForcing / RankTwoForcing: one source per column (vp gid from the
 * reference's point-source mapper) and its signal.  The signal is evaluated
 * on the device at t = (n-1)*dt at step n, as the reference does. */
int shaw_fom_set_sources(shaw_fom_t h, const uint64_t* vp_gid, const int32_t* kind,
                         const double* period, const double* delay);

/* Seismogram: receivers' vp gids; every `freq` steps x_vp[gid_r, :] is stored.
 * nsteps % freq must be 0.  R == 0 disables. */
int shaw_fom_set_receivers(shaw_fom_t h, const uint64_t* vp_gid, uint32_t num_receivers,
                           uint64_t freq, uint64_t nsteps);

/* StateObserver: snapshot matrices written straight into caller host arrays,
 * vp: nvp x (nsteps/freq_vp) x M, sp: nsp x (nsteps/freq_sp) x M (LayoutLeft).
 * The arrays must stay valid until the handle is destroyed or snapshots are
 * disabled (freq 0).  They are page-locked by the library while registered. */
int shaw_fom_set_snapshots(shaw_fom_t h, uint64_t freq_vp, uint64_t freq_sp, uint64_t nsteps,
                           double* host_vp, double* host_sp);

/* runFom: zero the states, then nsteps leapfrog steps (blocking). */
int shaw_fom_run(shaw_fom_t h, double dt, uint64_t nsteps);
/* Zero states and counters (the start of runFom). */
int shaw_fom_reset(shaw_fom_t h);
/* Enqueue nsteps more leapfrog steps on the handle's stream (non-blocking). */
int shaw_fom_advance(shaw_fom_t h, double dt, uint64_t nsteps);
/* updateVelocity for step `step` (1-based; forcing at t=(step-1)*dt) and
 * updateStress: one half-step each, on the handle's stream. */
int shaw_fom_update_velocity(shaw_fom_t h, double dt, uint64_t step);
int shaw_fom_update_stress(shaw_fom_t h, double dt);
int shaw_fom_synchronize(shaw_fom_t h);

/* Copy out the seismogram, R x (nsteps/freq) x M (LayoutLeft). */
int shaw_fom_get_seismogram(shaw_fom_t h, double* out);
/* Copy the states out / in: vp nvp x M, sp nsp x M (LayoutLeft). */
int shaw_fom_get_state(shaw_fom_t h, double* vp, double* sp);
int shaw_fom_set_state(shaw_fom_t h, const double* vp, const double* sp);
/* Schedule of the FOM leapfrog (no counterpart in the reference, which always runs
 * its two CRS products per step, fom_update_kernels.hpp:60-181).
 *   SHAW_FOM_SCHEDULE_TWO_PASS: the two half-step kernels (in place).
 *   SHAW_FOM_SCHEDULE_SWEEP: one kernel per step (forcing columns a multiple of 32).  It
 *     reads and writes every state value once per step (16 B per FP64 DOF-update, 8 B per
 *     FP32 one) and alternates between two state buffers.  Same FMAs in the same order as
 *     the two-pass kernels: bit-identical results.
 *   SHAW_FOM_SCHEDULE_PERSISTENT: rank 1, FP64, small grids: all the steps of a call in
 *     one cooperative launch (one CTA per SM, each a band of r rows -- or of theta
 *     columns, on grids wider than tall -- in shared memory, halo lines exchanged through
 *     L2 as tagged words); bit-identical to the two-pass kernels; runs with snapshots keep
 *     the two-pass kernels.
 *   SHAW_FOM_SCHEDULE_AUTO (the default): the fastest for the handle on GB300: the
 *     persistent launch for rank-1 FP64 handles whose grid fits (at least two bands of at
 *     most 1024 points with the halo line), the sweep for SHAW_MIXED_FP32 (HBM-bound,
 *     when the column count allows it), otherwise the two-pass kernels (for FP64 both
 *     the sweep and the two-pass kernels are bound by the FP64 pipe, and the two-pass
 *     kernels keep it busier).
 * SHAW_FOM_SCHEDULE_SWEEP and SHAW_FOM_SCHEDULE_PERSISTENT return SHAW_ERR_UNSUPPORTED
 * when the handle does not allow them.  Synchronizes the handle's stream. */
#define SHAW_FOM_SCHEDULE_AUTO            0
#define SHAW_FOM_SCHEDULE_TWO_PASS        1
#define SHAW_FOM_SCHEDULE_SWEEP           2
#define SHAW_FOM_SCHEDULE_PERSISTENT      3
int shaw_fom_set_schedule(shaw_fom_t h, int schedule);
/* The handle's cudaStream_t, for callers that time with CUDA events. */
void* shaw_fom_stream(shaw_fom_t h);
/* Kernels this handle has launched since creation (graph replays count each node). */
uint64_t shaw_fom_kernel_launches(shaw_fom_t h);

/* ======================================================================== *
 *  ROM                                                                      *
 * ======================================================================== */

typedef struct shaw_rom_s* shaw_rom_t;

/* computeRomOperatorsUsingFomJacsWithMatProp (rom_compute_jacobians.hpp:83-102)
 * in FP64 on the GPU with the FOM handle's operators:
 *   rom_jvp (kv x ks, row-major) = PhiVp^T (Jvp PhiSp)
 *   rom_jsp (ks x kv, row-major) = PhiSp^T (Jsp PhiVp)
 * phi_vp: nvp x kv, phi_sp: nsp x ks, both LayoutLeft (the lsv_* file layout). */
int shaw_rom_project(shaw_fom_t fom, const double* phi_vp, uint64_t kv, const double* phi_sp, uint64_t ks,
                     double* rom_jvp, double* rom_jsp);

/* The same projection without any allocation.  It has no counterpart in the
 * reference.  It exists for callers that cannot allocate device memory while
 * they run: an application that hands the library a fixed memory budget up
 * front, a code path where an allocation would synchronise the device, or a
 * runtime that owns every device allocation itself.
 *   - Every array is a DEVICE pointer owned by the caller: d_phi_vp nvp x kv and
 *     d_phi_sp nsp x ks (LayoutLeft), d_rom_jvp kv x ks and d_rom_jsp ks x kv
 *     (row-major).  The work is enqueued on `stream` (a cudaStream_t; 0 is the
 *     default stream) and the call returns without waiting for it.
 *   - The intermediate J*Phi passes, one block of mesh rows at a time with every
 *     mode column, through one fixed 16 MiB FP64 device array inside the library;
 *     every GPU that loads the library holds it until the process exits.  A block
 *     holds 2097152 / k values per column (k = ks for romJvp, kv for romJsp), so
 *     any mesh size works; kv and ks must be at most 65535, otherwise the call
 *     returns SHAW_ERR_INVALID_ARG.  Cost: about 2 (nvp + nsp) kv ks FP64 flops,
 *     like the allocating path, each basis value read about once.
 *   - It calls no cudaMalloc or cudaFree and no library routine that allocates.
 *   - Each call looks up the array's device address on the current device
 *     (cudaGetSymbolAddress, which does not allocate); the first lookup on a
 *     device may load the module, so make the first call before any stream
 *     capture.  The FOM handle is only read: its stencil values do not change
 *     after shaw_fom_create.
 *   - All calls share the one array: calls whose work overlaps on the GPU (other
 *     streams, or unordered threads) race on it. */
int shaw_rom_project_noalloc(shaw_fom_t fom, const double* d_phi_vp, uint64_t kv, const double* d_phi_sp,
                             uint64_t ks, double* d_rom_jvp, double* d_rom_jsp, void* stream);

/* The reduced system of runRomRankOneForcing (rank 1, M == 1) and
 * runRomRankTwoForcing (rank 2, M columns):
 *   xv += dt Av xs ;  xv[:,j] += (f_j(t_{n-1}) dt) b[:,j] ;  xs += dt As xv
 * rom_jvp kv x ks and rom_jsp ks x kv row-major; b kv x M LayoutLeft with
 * b[:,j] = rhoInv[src_j] * PhiVp[src_j, :] (rom_problem_rank_one.hpp:137-147).
 * precision: SHAW_FP64, or SHAW_MIXED_FP32 (rank 1: FP32 hi+lo operators and
 * state, error-free products and compensated sums); rank 2 also SHAW_MIXED_TF32X3,
 * SHAW_MIXED_OZAKI_BF16 and SHAW_OZAKI_FP64 (tensor cores, one persistent launch). */
int shaw_rom_create(uint64_t kv, uint64_t ks, const double* rom_jvp, const double* rom_jsp, int rank,
                    uint32_t num_forcings, const double* b, int precision, shaw_rom_t* out);
void shaw_rom_destroy(shaw_rom_t h);
/* Signal of each column (kind, period, delay); evaluated on the device. */
int shaw_rom_set_signals(shaw_rom_t h, const int32_t* kind, const double* period, const double* delay);
/* Reduced-state snapshots (the ROM's StateObserver): kv x (nsteps/freq_vp) x M and
 * ks x (nsteps/freq_sp) x M, LayoutLeft, filled by shaw_rom_run / _synchronize. */
int shaw_rom_set_snapshots(shaw_rom_t h, uint64_t freq_vp, uint64_t freq_sp, uint64_t nsteps, double* host_vp,
                           double* host_sp);
/* In-loop ROM seismogram S(r, t, j) = PhiVp[gid_r, :] . xv(:, j) at every freq
 * steps (reconstructSeismogram, main_reconstruct_seismo.cc:157-185, whose rank-2 form
 * the reference leaves unimplemented at :187-190); phi_rows is R x kv row-major (the
 * basis rows of the receivers' vp gids).  FP64 and rank-1 mixed: FP64 / double-float
 * dots; SHAW_MIXED_OZAKI_BF16 / SHAW_OZAKI_FP64: an exact sliced product on the tensor
 * cores inside the persistent kernel; SHAW_MIXED_TF32X3: SHAW_ERR_UNSUPPORTED (use
 * snapshots). */
int shaw_rom_set_receivers(shaw_rom_t h, const double* phi_rows, uint32_t num_receivers, uint64_t freq,
                           uint64_t nsteps);
int shaw_rom_run(shaw_rom_t h, double dt, uint64_t nsteps);
int shaw_rom_reset(shaw_rom_t h);
/* The launch of a rank-1 FP64 handle (bit-identical results either way):
 * SHAW_ROM_SCHEDULE_CLUSTER one thread-block cluster of up to 16 CTAs, the new rows
 * exchanged through distributed shared memory; SHAW_ROM_SCHEDULE_BANDS one cooperative
 * launch of a few rows per CTA over up to every SM, the new rows gathered through L2 as
 * tagged words (at most 1024 modes per dof).  AUTO (the default) takes the bands when
 * they fit.  Other handles accept AUTO only. */
#define SHAW_ROM_SCHEDULE_AUTO            0
#define SHAW_ROM_SCHEDULE_CLUSTER         1
#define SHAW_ROM_SCHEDULE_BANDS           2
int shaw_rom_set_schedule(shaw_rom_t h, int schedule);
int shaw_rom_advance(shaw_rom_t h, double dt, uint64_t nsteps);
int shaw_rom_synchronize(shaw_rom_t h);
/* States out: xv kv x M, xs ks x M (LayoutLeft). */
int shaw_rom_get_state(shaw_rom_t h, double* xv, double* xs);
/* Seismogram out: R x (nsteps/freq) x M (LayoutLeft). */
int shaw_rom_get_seismogram(shaw_rom_t h, double* out);
void* shaw_rom_stream(shaw_rom_t h);
uint64_t shaw_rom_kernel_launches(shaw_rom_t h);

/* ---- Batched ROM: many rank-2 reduced systems of uneven size ---------------
 * No counterpart in the reference, which runs one reduced system per process
 * (runRomRankTwoForcing, src/kokkos/torevise/run_rom_rank_two_forcing.hpp:119-201).
 * Every instance is that system with its own kv, ks, operators, forcing vectors b
 * (kv x M LayoutLeft, column j = rhoInv[src_j] PhiVp[src_j, :]) and per-column
 * signals; all advance with one dt.  precision: SHAW_FP64 (cuBLAS DGEMMs per
 * instance), or SHAW_MIXED_OZAKI_BF16 / SHAW_OZAKI_FP64 (all instances, all steps, one
 * persistent tensor-core launch; kv, ks <= 1024). */
typedef struct shaw_rom_batch_s* shaw_rom_batch_t;
typedef struct {
  uint64_t kv, ks;
  uint32_t num_forcings;
  const double* rom_jvp; /* kv x ks row-major */
  const double* rom_jsp; /* ks x kv row-major */
  const double* b;       /* kv x num_forcings LayoutLeft */
  const int32_t* kind;   /* num_forcings signal kinds, periods and delays */
  const double* period;
  const double* delay;
} shaw_rom_instance_desc;
int shaw_rom_batch_create(uint32_t num_instances, const shaw_rom_instance_desc* inst, int precision,
                          shaw_rom_batch_t* out);
void shaw_rom_batch_destroy(shaw_rom_batch_t h);
/* Autotuner (tensor-core batches): times tile widths of 16, 32 and 64 forcing columns,
 * each with a model-cost and a measured-cost longest-first schedule, over trial_steps
 * steps; keeps the fastest and leaves the batch reset.  A report of the candidates
 * goes to report[cap] (may be NULL). */
int shaw_rom_batch_tune(shaw_rom_batch_t h, double dt, uint64_t trial_steps, char* report, size_t cap);
/* Fixed tiling of a tensor-core batch (e.g. one the autotuner chose before): tiles of
 * width 16, 32 or 64 forcing columns; paired != 0 splits every tile's rows across two
 * co-resident CTAs (needs >= 256 modes per dof and 2 x tiles <= SMs, else
 * SHAW_ERR_UNSUPPORTED).  SHAW_ERR_UNSUPPORTED on FP64 batches. */
int shaw_rom_batch_set_tiling(shaw_rom_batch_t h, uint32_t width, int paired);
/* Diagnostic of failure detection: every wait of the persistent kernels is bounded and
 * reports a timeout instead of hanging.  One small launch waits, with the same helpers,
 * on an mbarrier phase that nothing completes and on a global counter that nothing
 * increments, each for `polls` polls, and on a tagged exchange word that nothing writes
 * (the row exchange of the band kernels) for min(polls, 2^22) rounds; *status receives
 * the bits they set (64, 128 -- the codes the ROM kernels report -- and 256).  The device
 * stays usable afterwards.  polls must be in 1 .. 16777216 (2^24, the kernels' own wait
 * limit), else SHAW_ERR_INVALID_ARG. */
int shaw_selftest_bounded_waits(uint64_t polls, uint32_t* status);
/* Reduced-state snapshots of instance i: kv x (nsteps/freq_vp) x M and
 * ks x (nsteps/freq_sp) x M LayoutLeft host arrays, filled by _synchronize. */
int shaw_rom_batch_set_snapshots(shaw_rom_batch_t h, uint32_t i, uint64_t freq_vp, uint64_t freq_sp,
                                 uint64_t nsteps, double* host_vp, double* host_sp);
/* In-loop seismogram of instance i (shaw_rom_set_receivers semantics): phi_rows R x kv
 * row-major; the seismogram R x (nsteps/freq) x M (LayoutLeft) is read back with
 * shaw_rom_batch_get_seismogram. */
int shaw_rom_batch_set_receivers(shaw_rom_batch_t h, uint32_t i, const double* phi_rows, uint32_t num_receivers,
                                 uint64_t freq, uint64_t nsteps);
int shaw_rom_batch_get_seismogram(shaw_rom_batch_t h, uint32_t i, double* out);
int shaw_rom_batch_reset(shaw_rom_batch_t h);
int shaw_rom_batch_advance(shaw_rom_batch_t h, double dt, uint64_t nsteps);
int shaw_rom_batch_run(shaw_rom_batch_t h, double dt, uint64_t nsteps);
int shaw_rom_batch_synchronize(shaw_rom_batch_t h);
/* States of instance i: xv kv x M, xs ks x M (LayoutLeft, host arrays). */
int shaw_rom_batch_get_state(shaw_rom_batch_t h, uint32_t i, double* xv, double* xs);
int shaw_rom_batch_describe(shaw_rom_batch_t h, char* out, size_t cap);
void* shaw_rom_batch_stream(shaw_rom_batch_t h);
uint64_t shaw_rom_batch_kernel_launches(shaw_rom_batch_t h);
uint64_t shaw_rom_batch_step(shaw_rom_batch_t h);

/* ======================================================================== *
 *  Host-side setup (the reference's main.cc + MeshInfo + material + mappers) *
 * ======================================================================== */

typedef struct shaw_mesh_s* shaw_mesh_t;

/* MeshInfo + readFullMeshGraphFile + readFullMeshCoeffFile
 * (src/shared/mesh_helpers/mesh_info.hpp:116-214, read_graph_file.hpp:54-124,
 *  read_vpcoeff_file.hpp:52-81). */
int shaw_mesh_load(const char* mesh_dir, shaw_mesh_t* out);
/* The full-mesh generator (meshing/create_single_mesh.py -> helpers/full_mesh_utils.py,
 * build_graph_impl.py), in memory. Angles in degrees, radii in km. */
int shaw_mesh_generate(uint64_t nth, uint64_t nr, double th_left_deg, double th_right_deg,
                       double r_cmb_km, double r_surf_km, shaw_mesh_t* out);
/* Write mesh_info.dat, graph_vp.dat, graph_sp.dat, coeff_vp.dat into dir
 * (meshing/helpers/write_files.py formats). */
int shaw_mesh_write(shaw_mesh_t m, const char* dir);
/* out[14]: thL, thR [deg], rCmb, rSurf [m], dth [rad], dr [m], 1/dth, 1/dr,
 * nvp, nsp, nth, nr, minArc, maxArc [m]. */
int shaw_mesh_info(shaw_mesh_t m, double* out);
/* Material models (src/shared/material_models/material_model_{unilayer,bilayer,prem}.hpp):
 *   SHAW_MATERIAL_UNILAYER params: rho[3], vs[3]           (depth in metres)
 *   SHAW_MATERIAL_BILAYER  params: rho1[3], vs1[3], disc_km, rho2[3], vs2[3]
 *   SHAW_MATERIAL_PREM     params: none
 * Fills 1/rho at vp points and rho*vs^2 at sp points (shwavepp.hpp:246-286). */
#define SHAW_MATERIAL_UNILAYER 0
#define SHAW_MATERIAL_BILAYER  1
#define SHAW_MATERIAL_PREM     2
int shaw_mesh_set_material(shaw_mesh_t m, int kind, const double* params, uint32_t nparams);
/* Caller-computed material (the reference's "custom" kind): per-point arrays. */
int shaw_mesh_set_material_arrays(shaw_mesh_t m, const double* rho_inv_vp, const double* shear_mod_sp);
/* min/max shear velocity seen while setting the material (for the checkers). */
int shaw_mesh_min_max_vs(shaw_mesh_t m, double* minmax);
/* Views into the mesh's arrays, valid while the mesh lives. */
int shaw_mesh_operator_desc(shaw_mesh_t m, shaw_fom_operator_desc* out);
/* mapPointSourceToGridPoint / mapNominalLocationToVelocityGridPoint. */
int shaw_mesh_map_source(shaw_mesh_t m, double depth_km, double angle_deg, uint64_t* gid);
int shaw_mesh_map_receiver(shaw_mesh_t m, double angle_deg, uint64_t* gid);
/* checkCfl (returns SHAW_ERR_CFL on violation) and checkDispersionCriterion
 * (SHAW_ERR_DISPERSION); *value receives the cfl number. */
int shaw_mesh_check_cfl(shaw_mesh_t m, double dt, double* value);
int shaw_mesh_check_dispersion(shaw_mesh_t m, double max_freq);
void shaw_mesh_destroy(shaw_mesh_t m);

/* shawExe <input.yaml>: parse the YAML input, run the FOM (rank-1 single or
 * multi-forcing, rank-2 sets) or the ROM, and write the reference's output
 * files into the current directory. */
int shaw_run_input_file(const char* yaml_path);
/* InputParser (src/shared/parser/input_parser.hpp:52-70): parse and validate an
 * input file without running it; writes "key=value" lines (one per parsed
 * field, the reference's getter names) into out[cap].  Returns SHAW_ERR_PARSE
 * with the reference's message on invalid input. */
int shaw_parse_input(const char* yaml_path, char* out, size_t cap);

/* ---- POD: thin SVD of a snapshot matrix ------------------------------------
 * Replaces doThinSVDm0 (method 1, BDCSVD) and doThinSVDm1 (method 2, Householder
 * QR then SVD of R) of src/tools/main_eigen_svd.cc:113-197.  snaps is the host
 * n x t snapshot matrix (LayoutLeft, one snapshot per column); on return lsv holds
 * the n x min(n,t) left singular vectors (LayoutLeft) and sv the min(n,t) singular
 * values in decreasing order.  Computed in FP64 on the GPU (QR, SVD of the triangle,
 * back-transformation).  Each singular vector is determined up to its sign: compare
 * subspaces, not raw vectors, with the reference's output.  Method 2 needs n >= t
 * (SHAW_ERR_UNSUPPORTED otherwise), as in the reference. */
int shaw_pod(const double* snaps, uint64_t n, uint64_t t, int method, double* lsv, double* sv);
/* computeThinSVD --dirs ... --informat ... --outformat ... --method ...
 * (main_eigen_svd.cc:199-305): for "vp" then "sp", concatenate the columns of
 * <dir>/snaps_<dof>_0 over dirs, run shaw_pod, write sva_<dof> (text, one value per
 * line, 17 significant digits) and lsv_<dof> (binary with size_t extents) into the
 * current directory.  As in the reference, the snapshot reader receives the
 * `outformat` string (main_eigen_svd.cc:302 passes the two formats in swapped order)
 * and reads only "binary"; the sva/lsv formats do not depend on either string. */
int shaw_pod_tool(const char* const* dirs, uint32_t ndirs, const char* informat, const char* outformat,
                  int method);

#ifdef __cplusplus
}
#endif
#endif /* SHAW_GPU_H_ */
