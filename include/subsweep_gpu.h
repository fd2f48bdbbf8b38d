/*
 * subsweep_gpu.h — C ABI of the GB300 sweep library.
 *
 * Drop-in for the reference's radiative-transfer sweep + hydrogen-only chemistry
 * (Tehforsch/subsweep, src/sweep/ and src/chemistry/).  The Rust host keeps its
 * ECS/plugin framework and calls these entry points through `extern "C"` from a
 * `GpuSweepPlugin` whose two systems replace the reference's:
 *
 *   init_sweep_system  (src/sweep/mod.rs:634-692)  ->  sw_create
 *   run_sweep_system   (src/sweep/mod.rs:694-739)  ->  sw_step + sw_get_fields
 *
 * Plain pointers and sizes only; no CUDA or torch types cross the boundary.  The
 * library owns all device memory.  One host thread per handle; calls on a handle
 * are not re-entrant.  All quantities are SI doubles (m, kg, s, K), as the
 * reference's diman quantities store them.  Every entry point makes the handle's
 * device current while it runs and makes the caller's current device current again
 * before it returns.
 */
#ifndef SUBSWEEP_GPU_H
#define SUBSWEEP_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The reference aborts (panic!/assert!/unwrap) where these return. */
typedef enum {
  SW_OK = 0,
  SW_ERR_INVALID_ARG = 1, /* bad parameters / grid / fields (reference: panic) */
  SW_ERR_CUDA = 2,        /* CUDA runtime error; sw_last_error has the message */
  SW_ERR_STALLED = 3,     /* a level sweep could not finish: dependency cycle
                             (reference: deadlock; check_deadlock analogue) or a
                             device wait that ran past its time limit */
  SW_ERR_OOM = 4,         /* device allocation failed */
  SW_ERR_UNSUPPORTED = 5  /* rotate_directions, > 128 directions, > 64 faces/cell */
} sw_status;

/* Arithmetic of the transport sweep.  FP64 is the plain drop-in (FP64 end to end).
 * MIXED runs the sweep in FP32 (scaled photon rates, FP32 face weights, compensated
 * per-cell rate sums) and keeps FP64 for the chemistry solve, the neutral fraction
 * (carried as 1 - x_HII) and the timescale-to-level assignment. */
typedef enum { SW_PRECISION_FP64 = 0, SW_PRECISION_MIXED = 1 } sw_precision;

/* Neighbour kinds of a face, as src/sweep/grid/cell.rs:16-23 on a single rank. */
enum { SW_FACE_LOCAL = 0, SW_FACE_LOCAL_PERIODIC = 1, SW_FACE_BOUNDARY = 2 };

/* Mirrors SweepParameters (src/sweep/parameters.rs:8-46) plus the scale factor
 * (Cosmology::scale_factor) and the precision choice.  sw_default_params fills the
 * reference's serde defaults (parameters.rs:64-78). */
typedef struct {
  /* DirectionsSpecification::Num (parameters.rs:48-62): 1, 16, 21, 32, 64 or 84. */
  int32_t num_directions;
  /* DirectionsSpecification::Explicit: if non-NULL, num_directions vectors
   * (xyz interleaved); each is normalised as Directions::from does (direction/mod.rs:97-108). */
  const double* explicit_directions;
  int32_t num_timestep_levels; /* >= 1, <= 16 */
  int32_t periodic;            /* informational; periodicity is carried by face kinds */
  double max_timestep;         /* s */
  int32_t rotate_directions;   /* must be 0 */
  double significant_rate_threshold;       /* photons/s, default 0 */
  double timestep_safety_factor;           /* default 0.1 */
  double chemistry_timestep_safety_factor; /* default 0.1 */
  int32_t check_deadlock;      /* 1: verify the dependency graph is acyclic at sw_create */
  int32_t prevent_cooling;     /* default 1 */
  int64_t num_tasks_to_solve_before_send_receive; /* MPI batching knob; accepted, unused */
  double scale_factor;         /* Cosmology::scale_factor(); 1 when non-cosmological */
  int32_t precision;           /* sw_precision */
  int32_t device;              /* CUDA device ordinal; -1 = the calling thread's current device */
  int32_t use_graphs;          /* replay each step as one CUDA graph (captured again
                                  when the step's set of sweeps changes); the transport kernel
                                  time is still recorded, the sweep / chemistry split is not.
                                  Default 0. */
  int32_t autotune;            /* mixed path: the first dense sweeps (each step opens with one)
                                  try each transport kernel variant (lanes per task, prefetch
                                  depth, resident blocks per SM; three candidates, so tuning
                                  ends within three steps)
                                  and keep the fastest per task; every variant computes
                                  identical results.  Default 1. */
} sw_params;

/* Face-neighbour CSR uploaded once (replaces the Cell component, grid/cell.rs:92-97).
 * Faces of cell c are row_ptr[c] .. row_ptr[c+1]-1.  Normals must be exactly
 * antisymmetric between the two sides of a face (true for generator-difference
 * normals).  The host owns these arrays; sw_create copies them. */
typedef struct {
  int64_t num_cells;
  const int64_t* row_ptr; /* [num_cells + 1] */
  const int32_t* nbr;     /* [E] neighbour index (ignored for boundary faces) */
  const uint8_t* kind;    /* [E] SW_FACE_* */
  const double* area;     /* [E] m^2 */
  const double* normal;   /* [E * 3] unit normals, xyz interleaved */
  const double* volume;   /* [num_cells] m^3 */
  const double* size;     /* [num_cells] m (cbrt(3V / 4pi) for Voronoi cells) */
} sw_grid_csr;

/* Per-cell initial components read by init_sweep_system (src/sweep/mod.rs:656-671). */
typedef struct {
  const double* density;                   /* kg/m^3 */
  const double* ionized_hydrogen_fraction; /* dimensionless */
  const double* temperature;               /* K */
  const double* source;                    /* photons/s */
} sw_cell_init;

typedef struct sw_handle sw_handle;

/* Cumulative work and timing counters of a handle. */
typedef struct {
  int64_t steps;
  int64_t level_sweeps;
  int64_t tasks;          /* solved (cell, direction) tasks */
  int64_t chem_cells;     /* chemistry cell updates */
  int64_t chem_attempts;  /* try_timestep_update calls */
  int64_t chem_failures;  /* cells whose chemistry did not converge (reference: log::error) */
  double sweep_ms;        /* device time in transport kernels (incl. counting, folding) */
  double chem_ms;         /* device time in chemistry kernels */
  double level_ms;        /* device time in level reassignment */
  double simulation_time; /* s, SimulationTime accumulated by sw_step */
  double step_ms;         /* device time of whole sw_step calls (CUDA events on the library's stream) */
  double transport_kernel_ms;  /* device time of the persistent transport kernel alone */
  int64_t transport_launches;  /* launches of the persistent transport kernel */
  int64_t kernel_launches;     /* all kernel launches made by sw_step */
  int64_t levelled_sweeps;     /* level sweeps run on the precomputed levelled schedule */
  int64_t schedule_levels;     /* Kahn levels of the schedule (0: cyclic grid, no schedule) */
  int64_t transport_attempts;  /* pull-path task attempts, retries included (tasks = success) */
  int64_t upwind_slots;        /* precomputed (face, direction) pairs of the grid: upwind LOCAL
                                  ones on the pull path, downwind LOCAL / LOCAL_PERIODIC ones on
                                  the push path (0 when the push path computes geometry) */
  int64_t graph_launches;      /* steps replayed from a CUDA graph */
  int64_t pull_variant;        /* mixed path: transport kernel variant in use (autotuned or set);
                                  0 in the compact state (the geometry kernel) */
  int64_t task_spaces;         /* mixed path, compact state: task spaces the directions are split
                                  into (0: the full state with task records and upwind slots) */
  int64_t device_bytes;        /* device memory the handle holds (grid, state, schedule) */
} sw_stats;

/* Fill the reference's defaults (num_directions 84, levels 1, max_timestep 1 Myr). */
sw_status sw_default_params(sw_params* p);

/* Batched mode (many independent small simulations, the C3 configuration): one handle
 * over the block-diagonal union of n_boxes grids, each with its own initial fields.
 * Box b's cells occupy the index range [sum of the earlier boxes' num_cells, + its own)
 * in every per-cell array of the handle (sw_get_fields, ...), and its neighbour indices
 * are local to the box.  Every box evolves exactly as a handle over that box alone
 * would (same parameters); one launch per sweep covers all boxes.  The reference has no
 * batched mode; this is the batch entry point planned for its GPU plugin. */
sw_status sw_create_batch(const sw_params* params, int32_t n_boxes, const sw_grid_csr* grids,
                          const sw_cell_init* inits, sw_handle** out);

/* Directions::from_num (src/sweep/direction/mod.rs:58-75): writes num*3 doubles. */
sw_status sw_directions_from_num(int32_t num, double* out);

/* init_sweep_system (src/sweep/mod.rs:634-692) + Sweep::new (194-232). */
sw_status sw_create(const sw_params* params, const sw_grid_csr* grid, const sw_cell_init* init,
                    sw_handle** out);

/* Sweep::run_sweeps (src/sweep/mod.rs:258-272): every level sweep of one step, the
 * chemistry, TimestepState::advance_allowed_levels and update_timestep_levels.  Writes
 * the elapsed time (TimestepState::current_max_timestep) and adds it to the handle's
 * simulation time.  (The reference skips the very first run_sweep_system call so the
 * initial conditions can be written; that is host-plugin logic.) */
sw_status sw_step(sw_handle* h, double* time_elapsed_out);

/* Write-back of run_sweep_system (src/sweep/mod.rs:718-738): x_HII, T, the species
 * timestep and PhotonRate = sum over directions of the incoming rate.  Any pointer
 * may be NULL.  Arrays have num_cells entries. */
sw_status sw_get_fields(sw_handle* h, double* ionized_hydrogen_fraction, double* temperature,
                        double* timestep, double* photon_rate);

/* Further per-cell state: change timescale (Site::change_timescale), timestep level,
 * and IonizationTime (time at which x_HII first exceeded 0.5, +inf before). */
sw_status sw_get_cell_state(sw_handle* h, double* change_timescale, uint8_t* level,
                            double* ionization_time);

/* Overwrite x_HII and T (remap / restart); either pointer may be NULL. */
sw_status sw_set_fields(sw_handle* h, const double* ionized_hydrogen_fraction,
                        const double* temperature);

/* Number of cells at each level >= l (Sweep::get_cell_counts_per_level,
 * src/sweep/mod.rs:240-245); per_level has num_timestep_levels entries. */
sw_status sw_get_level_counts(sw_handle* h, int64_t* per_level);

/* Dependency counts of Sweep::init_counts (src/sweep/mod.rs:346-386) for `level` with
 * the current cell levels: counts[cell * D + dir], 0 for inactive cells. */
sw_status sw_get_dependency_counts(sw_handle* h, int32_t level, uint8_t* counts);

/* Per-(cell, direction) transport state in [cell][dir] layout, converted to FP64
 * photons/s: Site::incoming_total_rate, outgoing_total_rate, periodic_source
 * (src/sweep/site.rs:12-23).  Any pointer may be NULL. */
sw_status sw_get_rates(sw_handle* h, double* incoming, double* outgoing, double* periodic);

sw_status sw_get_stats(sw_handle* h, sw_stats* out);

/* Global averages of the current state as the reference's time-series systems report
 * them (compute_time_series_system, src/sweep/time_series.rs:61-155), reduced on the
 * device: cell mass = density * volume (src/main.rs:195-203); a cell's photoionization
 * rate is Solver::photoionization_rate over one year (src/sweep/chemistry_output.rs:15-28)
 * with the rate summed over directions as Sweep::get_solver forms it
 * (src/sweep/mod.rs:613-631).  Copies 48 bytes to the host, nothing per cell. */
typedef struct {
  double hydrogen_ionization_mass_average;
  double hydrogen_ionization_volume_average;
  double temperature_mass_average;       /* K */
  double temperature_volume_average;     /* K */
  double photoionization_rate_volume_average;           /* 1/s */
  double weighted_photoionization_rate_volume_average;  /* 1/s, weighted by x_HII */
} sw_time_series;
sw_status sw_get_time_series(sw_handle* h, sw_time_series* out);

/* Checkpoint and restart of the evolving state (no counterpart in the reference, which
 * only remaps initial conditions): per-cell species, timestep levels, previous rates,
 * change timescales, ionization times; the per-(cell, direction) transport state of the
 * handle's precision; TimestepState, simulation time and sweep counter.  The grid,
 * parameters and precision are not stored: load into a handle created from the same
 * inputs (checked through cell, face, direction and level counts).  Statistics are not
 * part of the state.  sw_checkpoint_size gives the buffer size in bytes. */
sw_status sw_checkpoint_size(sw_handle* h, size_t* bytes);
sw_status sw_save_state(sw_handle* h, void* buffer, size_t bytes);
/* Rejects (SW_ERR_INVALID_ARG) a buffer whose header does not match the handle, that
 * is shorter than the checkpoint, or that holds a timestep level >= num_timestep_levels,
 * before any of it reaches the device. */
sw_status sw_load_state(sw_handle* h, const void* buffer, size_t bytes);

/* Same result as sw_get_dependency_counts, for callers that cannot allocate device
 * memory (a host engine whose GPU memory is owned by its own pool, code that must not
 * trigger the synchronisation cudaMalloc/cudaFree can cause): it stages the counts in
 * a fixed 16 MiB __device__ array of the library instead of a cudaMalloc'd buffer and
 * allocates nothing.  num_cells * directions must not exceed 16 MiB (SW_ERR_INVALID_ARG
 * otherwise).  The first call on a device looks up the array's device address; make it
 * before any stream capture.  That address is kept for the life of the device's primary
 * context: do not call this again after a cudaDeviceReset in the same process.  Calls
 * share the array, so calls that overlap on the GPU race.  This entry point has no
 * counterpart in the reference. */
sw_status sw_get_dependency_counts_noalloc(sw_handle* h, int32_t level, uint8_t* counts);

/* Message of the last error on this handle ("" if none); with h == NULL, the last
 * error of sw_create on this thread. */
const char* sw_last_error(const sw_handle* h);

void sw_destroy(sw_handle* h);

#ifdef __cplusplus
}
#endif
#endif
