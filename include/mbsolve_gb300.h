/*
 * mbsolve_gb300 — C-ABI of the GB300 Maxwell–Bloch time loop.
 *
 * This is the drop-in boundary between a host program (mbsolve-lib's solver
 * factory in C++, the Python layer, or any FFI) and the CUDA engine.  Every
 * entry point is `extern "C"`, takes plain pointers and sizes, returns an
 * int status (MBG_OK on success) and never lets a C++ exception cross the
 * boundary; the text of the last error of the calling thread is available
 * from mbg_last_error().
 *
 * The input is a flat, read-only description of the reference's objects:
 *   mbg_qm        <- mbsolve::qm_description / qm_lindblad_relaxation
 *                    (mbsolve-lib/include/mbsolve/lib/qm_description.hpp:38-332)
 *   mbg_material  <- mbsolve::material (material.hpp:38-130)
 *   mbg_region    <- mbsolve::region   (device.hpp:82-150)
 *   mbg_device    <- mbsolve::device   (device.hpp:152-216); materials are
 *                    listed in the order of device::get_used_materials(),
 *                    i.e. sorted by material id (a std::set<std::string>)
 *   mbg_source    <- mbsolve::source / sech_pulse / gaussian_pulse
 *                    (source.hpp:35-261)
 *   mbg_record    <- mbsolve::record (record.hpp:37-140, record.cpp:27-69)
 *   mbg_scenario  <- mbsolve::scenario (scenario.hpp:164-335)
 * All numbers are SI, FP64, with the reference's meaning.  Pointers are only
 * read during the call that receives them.
 */
#ifndef MBSOLVE_GB300_H
#define MBSOLVE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */

#define MBG_OK 0
/* a configuration error; the C++ layer rethrows std::invalid_argument
 * (the reference throws it at common_fdtd.hpp:92,121, solver.cpp:181,
 * algo_lindblad_cvr_rodr.hpp:155,203, algo_lindblad_reg_cayley.hpp:135,154) */
#define MBG_ERR_INVALID_ARGUMENT 1
/* a CUDA runtime error; rethrown as std::runtime_error("CUDA: ...")
 * (pattern of solver-cuda/include/common_cuda.hpp:60-66) */
#define MBG_ERR_CUDA 2
/* any other runtime failure (device wait timed out, non-finite probe) */
#define MBG_ERR_RUNTIME 3

/* ------------------------------------------------------------------- enums */

/* source::type, source.hpp:41-45 */
enum { MBG_SOURCE_HARD = 0, MBG_SOURCE_SOFT = 1 };
/* waveform of a source: a value table of n_t entries (what the reference
 * precomputes in solver_cpu_fdtd.tpp:185-202), or the two analytic pulses */
enum { MBG_SHAPE_TABLE = 0, MBG_SHAPE_SECH = 1, MBG_SHAPE_GAUSSIAN = 2 };
/* record::type, record.hpp:43-50 */
enum {
    MBG_RECORD_ELECTRIC = 0,
    MBG_RECORD_POLAR_DT = 1,
    MBG_RECORD_MAGNETIC = 2,
    MBG_RECORD_DENSITY = 3,
    MBG_RECORD_INVERSION = 4
};
/* relaxation superoperator: the base qm_superop (zero action,
 * qm_description.hpp:127-132) or qm_lindblad_relaxation (:144-253) */
enum { MBG_RELAX_NONE = 0, MBG_RELAX_LINDBLAD = 1 };
/* field initial condition: ic_field_const (scenario.hpp:99-117) or one value
 * per grid point (what ic_field_random draws, scenario.hpp:125-157) */
enum { MBG_FIELD_IC_CONST = 0, MBG_FIELD_IC_VALUES = 1 };

/* ------------------------------------------------------- scenario objects */

/* qm_description (qm_description.hpp:259-332).  Operators use the
 * reference's qm_operator packing (qm_description.hpp:38-87): the main
 * diagonal, then the upper triangle in column-major order as (re, im)
 * pairs: (0,1), (0,2), (1,2), (0,3), ...  The relaxation arrays hold what
 * qm_lindblad_relaxation::get_scattering_rates()/get_dephasing_rates()
 * return, i.e. after its constructor replaced the diagonal with the
 * negative total out-scattering and folded the lifetime into the dephasing
 * (qm_description.hpp:166-204). */
typedef struct mbg_qm {
    uint32_t num_levels;      /* N (2..6) */
    double carrier_density;   /* m^-3 */
    const double* h_diag;     /* [N]            J            */
    const double* h_off;      /* [N(N-1)/2][2]  J            */
    const double* mu_diag;    /* [N]            C m          */
    const double* mu_off;     /* [N(N-1)/2][2]  C m          */
    int32_t relax_kind;       /* MBG_RELAX_*                 */
    const double* scattering; /* [N][N] row-major, 1/s       */
    const double* dephasing;  /* [N(N-1)/2], 1/s (<= 0)      */
} mbg_qm;

/* material (material.hpp:38-130) */
typedef struct mbg_material {
    double rel_permittivity;
    double rel_permeability;
    double overlap_factor;
    double losses;
    const mbg_qm* qm; /* NULL: no quantum-mechanical description */
} mbg_material;

/* region (device.hpp:82-150); `material` indexes mbg_device.materials */
typedef struct mbg_region {
    uint32_t material;
    double x_start;
    double x_end;
} mbg_region;

/* field boundary conditions (bc_field, device.hpp:38-79) */
#define MBG_BC_PMC 0    /* H = 0 beyond both ends: what every reference
                           solver applies (bc_field_reflectivity is stored,
                           and ignored, solver_cpu_fdtd.tpp:263-275) */
#define MBG_BC_MIRROR 1 /* no reference counterpart: semi-transparent
                           mirrors of power reflectivity refl_left and
                           refl_right at the ends. The H value beyond each
                           end is tied to the end point's E as an impedance
                           wall: H = +k E (left), H = -k E (right) with
                           k Z = (1 - r)/(1 + r), r = sqrt(refl), Z the wave
                           impedance of the end point's material. refl = 1
                           is the PMC boundary, refl = 0 absorbs. */

/* device (device.hpp:152-216) */
typedef struct mbg_device {
    uint32_t num_materials;
    const mbg_material* materials;
    uint32_t num_regions;
    const mbg_region* regions;
    int32_t bc_kind;    /* MBG_BC_*; 0 (PMC) reproduces the reference */
    double refl_left;   /* MBG_BC_MIRROR: power reflectivities in [0, 1] */
    double refl_right;
} mbg_device;

/* source (source.hpp:35-261).  SECH: A*sech(beta t - phase)*sin(2 pi f t -
 * phase_sin); GAUSSIAN: A*exp(-(t - phase)^2/tau^2)*sin(2 pi f t) with
 * tau = beta_or_tau. TABLE: `table` holds n_t values, entry j for t = j*dt. */
typedef struct mbg_source {
    int32_t type;  /* MBG_SOURCE_* */
    int32_t shape; /* MBG_SHAPE_*  */
    double position;
    double ampl;
    double freq;
    double phase;
    double beta_or_tau;
    double phase_sin;
    const double* table;
    uint32_t table_len;
} mbg_source;

/* record (record.hpp:37-140); row/col are zero-based density indices */
typedef struct mbg_record {
    int32_t type; /* MBG_RECORD_* */
    uint32_t row;
    uint32_t col;
    double interval;
    double position;
    int32_t is_complex;
    int32_t coherence; /* density records with row != col: 0 records zero,
                          as every reference solver (solver_cpu_fdtd.tpp:
                          314-318); 1 records rho[row][col] (real and
                          imaginary part; no reference counterpart) */
} mbg_record;

/* scenario (scenario.hpp:164-335) with constant density initial condition
 * (ic_density_const, scenario.hpp:54-78) */
typedef struct mbg_scenario {
    uint32_t num_gridpoints;
    double endtime;
    uint32_t num_timesteps; /* only read for 0-D (one grid point) runs */
    const double* rho_diag; /* [rho_levels] */
    const double* rho_off;  /* [rho_num_off][2] */
    uint32_t rho_levels;    /* main-diagonal entries (0: no density IC) */
    uint32_t rho_num_off;   /* off-diagonal entries; a qm_operator may hold
                               any count (qm_description.hpp:54-66) */
    int32_t e_init_kind;    /* MBG_FIELD_IC_* */
    double e_init_value;
    const double* e_init_values; /* [num_gridpoints] */
    int32_t h_init_kind;
    double h_init_value;
    const double* h_init_values; /* [num_gridpoints] */
    uint32_t num_sources;
    const mbg_source* sources;
    uint32_t num_records;
    const mbg_record* records;
} mbg_scenario;

/* What init_fdtd_simulation (common_fdtd.hpp:52-123) writes back into the
 * scenario; a caller copies it into its own scenario object. */
typedef struct mbg_grid {
    uint32_t num_gridpoints;
    uint32_t num_timesteps;
    double gridpoint_size;
    double timestep_size;
    double endtime;
} mbg_grid;

/* Launch shape of the tiled time-step kernel (0 fields = autotuned).
 * cells_per_thread x threads cells form a tile; `depth` time steps run in
 * shared memory/registers per launch (temporal blocking). `staging`: 0 =
 * the tile state is loaded into registers (default), 1 = it is staged in
 * shared memory by bulk asynchronous (TMA) copies, for the 2-level FP32
 * solvers (elsewhere 0 is used); the environment variable
 * MBG_TILE_STAGING=bulk asks for 1 as well. mbg_ensemble_info reports the
 * staging in use. */
typedef struct mbg_tuning {
    uint32_t cells_per_thread;
    uint32_t threads;
    uint32_t depth;
    uint32_t launches_per_graph; /* kernel launches captured in one CUDA graph */
    uint32_t staging;
    uint32_t persistent; /* where the launch shape has a persistent
                            kernel (2-level FP32 4 x 256, tensor-core 4-6
                            levels, FP32 Cayley 4-6 levels): 1 = each
                            advance runs its full launches
                            as one persistent kernel (CTAs take the tiles of
                            successive launches in order, each waiting for
                            its neighbour tiles; bit-identical results),
                            2 = one launch per `depth` steps in CUDA graphs,
                            0 = automatic (persistent when a launch has
                            fewer than 4 waves of tiles). The environment
                            variable MBG_PERSISTENT=1 / =0 forces 1 / 2. */
} mbg_tuning;

/* ------------------------------------------------------------ entry points */

/* Version string and the thread-local text of the last failed call. */
const char* mbg_version(void);
const char* mbg_last_error(void);

/* Solver names this library serves, '\n'-separated (replaces the name list
 * that solver_cpu_loader registers, solver-cpu/src/solver_cpu_loader.cpp:
 * 32-89). Names: gpu-fdtd-noop-{fp32,fp64},
 * gpu-fdtd-{2..6}lvl-{cvr-rodr,reg-cayley}-{fp32,fp64}. Returns the length
 * needed (including the final NUL); writes nothing when buf is NULL. */
size_t mbg_solver_names(char* buf, size_t len);

typedef struct mbg_solver mbg_solver;

/* Grid derivation alone, on the host (no GPU needed): what
 * init_fdtd_simulation(dev, scen, 0.5) (common_fdtd.hpp:52-123, called with
 * Courant number 0.5 by solver_cpu_fdtd.tpp:67) writes into the scenario. */
int mbg_scenario_grid(
    const mbg_device* dev,
    const mbg_scenario* scen,
    mbg_grid* out);

/* Replaces the constructor of solver_cpu_fdtd
 * (solver-cpu/include/mbsolve/solver-cpu/solver_cpu_fdtd.tpp:36-203):
 * grid derivation, per-material FDTD and Lindblad constants (computed in
 * FP64 on the GPU), material map, initial state, record plan, source table.
 * Everything is resident on the GPU after this call. */
int mbg_solver_create(
    const char* name,
    const mbg_device* dev,
    const mbg_scenario* scen,
    const mbg_tuning* tuning, /* may be NULL */
    mbg_solver** out);

/* Grid as written back by init_fdtd_simulation. */
int mbg_solver_grid(const mbg_solver* s, mbg_grid* out);

/* Replaces solver_cpu_fdtd::run (solver_cpu_fdtd.tpp:223-338): all
 * num_timesteps steps on the GPU; like the reference, a second call
 * continues from the state the first left. Returns MBG_ERR_RUNTIME when a
 * recorded value was NaN or Inf (the run diverged) or a device wait ran
 * out; the results stay readable. Device waits are bounded: the
 * environment variable MBG_WAIT_LIMIT (read when a solver or ensemble is
 * created) sets how many times a kernel polls before it gives up, where
 * 0 or unset keeps the kernels' defaults (2^24 polls for a neighbour tile
 * of the persistent kernel, 2^22 for a tensor-core or bulk-copy
 * completion). MBG_TEST_STALL_PERSIST=1 exists for tests only: every wait
 * of the persistent kernel then asks for progress no tile reaches and runs
 * out. */
int mbg_solver_run(mbg_solver* s);

/* Results, one per scenario record in record order (solver_cpu_fdtd.tpp:
 * 157-179, 329-337): rows = time samples, cols = grid points, row-major. */
int mbg_solver_num_results(const mbg_solver* s, uint32_t* n);
int mbg_solver_result_shape(
    const mbg_solver* s,
    uint32_t k,
    uint32_t* rows,
    uint32_t* cols,
    int32_t* is_complex);
/* imag may be NULL for real results */
int mbg_solver_copy_result(
    const mbg_solver* s,
    uint32_t k,
    double* real,
    double* imag);

void mbg_solver_destroy(mbg_solver* s);

/* ----------------------------------------------------------- ensembles */

/* A batch of independent runs (no reference counterpart: the reference
 * runs one scenario per solver object; this is the batched launch model,
 * replacing n calls of solver::create_instance + run). All runs use one
 * solver name; each has its own device and scenario (length, sources,
 * materials, records). Runs share one packed ragged layout in HBM and are
 * advanced in lock-step; a run whose num_timesteps is reached is frozen. */
typedef struct mbg_ensemble mbg_ensemble;

int mbg_ensemble_create(
    const char* name,
    uint32_t num_runs,
    const mbg_device* const* devs,
    const mbg_scenario* const* scens,
    const mbg_tuning* tuning, /* may be NULL */
    mbg_ensemble** out);

/* Advance every run by up to n_steps time steps (all on the GPU; the call
 * returns once the work is queued: mbg_ensemble_status reports device
 * errors). */
int mbg_ensemble_advance(mbg_ensemble* e, uint32_t n_steps);
/* Advance to the end of the longest run; MBG_ERR_RUNTIME as for
 * mbg_solver_run. */
int mbg_ensemble_run(mbg_ensemble* e);
/* Time steps done so far and the maximum over runs. */
int mbg_ensemble_progress(
    const mbg_ensemble* e,
    uint64_t* steps_done,
    uint64_t* steps_total);
int mbg_ensemble_grid(const mbg_ensemble* e, uint32_t run, mbg_grid* out);
int mbg_ensemble_result_shape(
    const mbg_ensemble* e,
    uint32_t run,
    uint32_t k,
    uint32_t* rows,
    uint32_t* cols,
    int32_t* is_complex);
int mbg_ensemble_copy_result(
    const mbg_ensemble* e,
    uint32_t run,
    uint32_t k,
    double* real,
    double* imag);
/* Copy rows [row0, row0+nrows) of result k of every run whose result has
 * exactly one column (a probe) into out[run][nrows] (FP64). */
int mbg_ensemble_copy_probe_rows(
    const mbg_ensemble* e,
    uint32_t k,
    uint64_t row0,
    uint64_t nrows,
    double* out);
/* Total grid points over all runs and the tile plan in use. */
int mbg_ensemble_info(
    const mbg_ensemble* e,
    uint64_t* cells,
    uint32_t* tiles,
    mbg_tuning* tuning_used);
/* Kernel timing: CUDA events around every time-step kernel launch on the
 * ensemble's stream; returns launches and summed milliseconds since the
 * last reset. Enabled by mbg_ensemble_set_timing(e, 1). */
int mbg_ensemble_set_timing(mbg_ensemble* e, int enable);
int mbg_ensemble_kernel_time(
    mbg_ensemble* e,
    uint64_t* launches,
    double* milliseconds,
    int reset);
/* Device time of a region of work on the ensemble's stream: begin = 1
 * records a start event, begin = 0 records a stop event, waits for it and
 * writes the milliseconds between the two. */
int mbg_ensemble_stream_time(mbg_ensemble* e, int begin, double* milliseconds);
/* Kernels this library launched on the ensemble's stream so far (time-step
 * kernels and the small clock/gather kernels around them). */
int mbg_ensemble_launches(const mbg_ensemble* e, uint64_t* launches);
/* Status flags raised on the device (bit 0: a recorded value was NaN or
 * Inf; bit 3: a tensor-core or bulk-copy completion wait ran out; bit 4: a
 * persistent-kernel wait for neighbour tiles ran out). */
int mbg_ensemble_status(mbg_ensemble* e, uint32_t* flags);
/* Checkpoint and resume (no reference counterpart; the reference has no
 * checkpointing). The state is every field, density and record value plus
 * the step index, in host memory: mbg_ensemble_state_size gives the bytes,
 * mbg_ensemble_save_state writes them (after the queued work finishes),
 * mbg_ensemble_load_state restores them into an ensemble created from the
 * same descriptions (refused with MBG_ERR_INVALID_ARGUMENT otherwise);
 * advancing it then continues exactly where the saved one stood. */
int mbg_ensemble_state_size(const mbg_ensemble* e, uint64_t* bytes);
int mbg_ensemble_save_state(mbg_ensemble* e, void* host, uint64_t bytes);
int mbg_ensemble_load_state(mbg_ensemble* e, const void* host, uint64_t bytes);
void mbg_ensemble_destroy(mbg_ensemble* e);

/* ------------------------------------------------------------ inspection */

/* The per-material constants the time-step kernel consumes, computed by
 * the library's FP64 precompute (same code the GPU runs).  on_device = 1
 * runs it on the GPU, 0 runs the identical host instantiation (used by
 * tests on machines without a GPU; the solvers always use the GPU).
 * Writes up to `cap` doubles into out and the needed count to *len.
 * Layout is given by mbg_material_layout(). */
int mbg_material_constants(
    const char* algo, /* "cvr-rodr" or "reg-cayley" */
    const mbg_material* mat,
    double timestep,
    int on_device,
    double* out,
    size_t cap,
    size_t* len);

/* Allocation-free variant of mbg_material_constants (no counterpart in the
 * reference). For callers that cannot call cudaMalloc: their device memory
 * belongs to another allocator (a framework's pool, or memory reserved up
 * front), or the path cannot take the device-wide synchronisation that
 * cudaMalloc/cudaFree imply. The constant block is computed on the current
 * device into `out_device`, a device buffer of `cap` doubles the caller
 * owns, on `stream` (NULL: the legacy default stream); the call returns
 * when it is done. The FP64 workspace is a fixed array of about 160 KB in
 * this library's device memory (enough for 6 levels); larger workspaces
 * are refused with MBG_ERR_INVALID_ARGUMENT. Each call looks up the
 * array's address on the current device and synchronizes `stream` before
 * it returns. Every call uses the same array: calls that overlap on the
 * GPU race. With out_device NULL only *len (the block size) is written. */
int mbg_material_constants_noalloc(
    const char* algo,
    const mbg_material* mat,
    double timestep,
    double* out_device,
    size_t cap,
    size_t* len,
    void* stream);

/* Offsets of the fields in mbg_material_constants' output for N levels:
 * writes name=offset pairs as text ("a=0\nb=1\n..."). */
size_t mbg_material_layout(
    const char* algo,
    uint32_t num_levels,
    char* buf,
    size_t len);

#ifdef __cplusplus
}
#endif

#endif
