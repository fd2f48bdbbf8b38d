/*
 * CPU FP64 oracle for the subsweep radiative-transfer sweep + hydrogen-only
 * chemistry hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is a line-by-line restatement of the
 * reference algorithm (Tehforsch/subsweep, Rust) and exists so that the CUDA
 * implementation can be checked against it.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load it; the product never does.
 *
 * Parity pinning: the reference (Rust nightly, unpinned git dependencies) cannot
 * be built here, so the oracle is pinned against the reference's own known-answer
 * tests (timestep level assignment, sweep level order, chemistry derivative
 * consistency, chemistry extreme-input runs) plus analytic transport checks; the
 * sweep transport and the coupled x_HII/T evolution have no reference golden
 * vectors ("parity unpinned" for those quantities).
 *
 * Units: plain SI doubles (m, kg, s, K, J), as the reference's diman quantities
 * store them.
 */
#ifndef SUBSWEEP_ORACLE_H
#define SUBSWEEP_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Neighbour kinds, mirroring src/sweep/grid/cell.rs:16-23 (single rank: no Remote kinds). */
enum { ORC_LOCAL = 0, ORC_LOCAL_PERIODIC = 1, ORC_BOUNDARY = 2 };

/* Periodic-source semantics. SNAPSHOT: contributions written through periodic faces
 * during a level sweep become visible to transport in the next sweep (and to the
 * chemistry of this sweep).  IMMEDIATE: the reference's literal behaviour, where
 * visibility depends on the (unstable) task order; kept to measure the deviation. */
enum { ORC_PERIODIC_SNAPSHOT = 0, ORC_PERIODIC_IMMEDIATE = 1 };

/* Task order within a level sweep.  FIFO: per direction (highest first), a FIFO queue
 * of ready tasks.  HEAP: the reference's std BinaryHeap keyed by direction only
 * (src/sweep/mod.rs:104, task.rs:25-35), restated from the Rust standard library, fed
 * in the reference's order (get_initial_tasks, mod.rs:388-398); with one thread and
 * ORC_PERIODIC_IMMEDIATE this is the reference's single-rank computation, task for
 * task. */
enum { ORC_ORDER_FIFO = 0, ORC_ORDER_HEAP = 1 };

/* How worker threads share a level sweep.  DIRECTIONS: directions t, t + T, ... to
 * worker t, each with its own queue or heap (with ORC_ORDER_FIFO the results do not
 * depend on the thread count).  DOMAINS: the reference's parallel scheme, one rank per
 * thread owning a contiguous block of cell ids, with the reference's own heap per rank
 * and batched rate-correction messages between ranks (summation order then depends on
 * timing; for CPU timing). */
enum { ORC_PARTITION_DIRECTIONS = 0, ORC_PARTITION_DOMAINS = 1 };

typedef struct {
  int64_t num_cells;
  const int64_t* row_ptr; /* [num_cells+1] */
  const int32_t* nbr;     /* [E] neighbour cell index (ignored for boundary faces) */
  const uint8_t* kind;    /* [E] ORC_LOCAL / ORC_LOCAL_PERIODIC / ORC_BOUNDARY */
  const double* area;     /* [E] face area (m^2) */
  const double* normal;   /* [E*3] face normal, interleaved xyz */
  const double* volume;   /* [num_cells] m^3 */
  const double* size;     /* [num_cells] m */
} orc_grid;

typedef struct {
  int32_t num_directions;
  const double* directions; /* [D*3] direction vectors, used as given */
  int32_t num_timestep_levels;
  double max_timestep;                     /* s */
  double significant_rate_threshold;       /* 1/s */
  double timestep_safety_factor;           /* dimensionless */
  double chemistry_timestep_safety_factor; /* dimensionless */
  int32_t prevent_cooling;
  double scale_factor;
  int32_t periodic_mode; /* ORC_PERIODIC_* */
  int32_t order;         /* ORC_ORDER_* */
  /* Worker threads (<= 1: one).  A level sweep's transport is shared as `partition`
   * says; the chemistry splits the cells. */
  int32_t num_threads;
  int32_t partition; /* ORC_PARTITION_* */
} orc_params;

typedef struct orc_sim orc_sim;

/* Sweep driver (src/sweep/mod.rs).  density kg/m^3, source photons/s. */
orc_sim* orc_sim_create(const orc_params* p, const orc_grid* g, const double* density,
                        const double* xhii, const double* temperature, const double* source);
void orc_sim_destroy(orc_sim* s);
/* One Sweep::run_sweeps (mod.rs:258-272). Returns 0 on success, 1 if a level sweep
 * could not finish (dependency cycle: the reference would deadlock). */
int orc_sim_step(orc_sim* s, double* time_elapsed);
/* Fields after the last step: x_HII, T, species timestep, PhotonRate = sum_d incoming
 * (mod.rs:718-730), change timescale, timestep level.  Any pointer may be NULL. */
void orc_sim_get_fields(const orc_sim* s, double* xhii, double* temperature, double* timestep,
                        double* rate, double* change_timescale, uint8_t* level);
/* Per-(cell,dir) transport state, [cell][dir] layout.  Any pointer may be NULL. */
void orc_sim_get_rates(const orc_sim* s, double* incoming, double* outgoing, double* periodic);
/* time series (src/sweep/time_series.rs:61-155): mass / volume averaged x_HII, mass /
   volume averaged T, volume averaged photoionization rate and its x_HII-weighted form */
void orc_sim_time_series(const orc_sim* s, double* out6);
/* Dependency counts of Sweep::init_counts (mod.rs:346-386) for the given level with the
 * current cell levels: out[cell*D + dir] (0 for inactive cells); returns #active cells. */
int64_t orc_sim_init_counts(const orc_sim* s, int32_t level, uint8_t* out);
/* Number of cells at each level >= l, as Sweep::get_cell_counts_per_level (mod.rs:240-245). */
void orc_sim_level_counts(const orc_sim* s, int64_t* counts);
/* Cumulative solved-task and chemistry-update counters. */
void orc_sim_work(const orc_sim* s, int64_t* tasks, int64_t* chem_cells);
/* Number of levels swept by the next step (TimestepState::iter_levels_in_sweep_order). */
int32_t orc_sim_sweep_order(const orc_sim* s, int32_t* levels_out, int32_t cap);
/* Run a single level sweep + chemistry at `level` (mod.rs:274-289) on the current state,
 * for bounded CPU timing samples.  Returns tasks solved. */
int64_t orc_sim_single_sweep(orc_sim* s, int32_t level);
/* A bounded sample of one level sweep, for CPU timing: the transport of directions
 * dir_first .. dir_first + dir_count - 1 (mod D) over every active cell, then the
 * chemistry of the same share of the active cells (dir_count / D of them, from the
 * chem_first-th active cell on, wrapping).  Returns the tasks solved (-1 on invalid
 * arguments); *chem_cells gets the chemistry updates. */
int64_t orc_sim_sample_sweep(orc_sim* s, int32_t level, int32_t dir_first, int32_t dir_count, int64_t chem_first,
                             int64_t* chem_cells);

/* --- Known-answer-test entry points ---------------------------------------- */
/* TimestepLevel::from_max_timestep_and_desired_timestep (timestep_level.rs:27-36). */
int32_t orc_timestep_level(int32_t max_num_levels, double max_timestep, double desired);
/* TimestepState: sweep order for `num_levels` levels after `advances` calls of
 * advance_allowed_levels.  Writes up to cap levels, returns count. */
int32_t orc_sweep_order_after(int32_t num_levels, int32_t advances, int32_t* out, int32_t cap);
int32_t orc_lowest_allowed_after(int32_t num_levels, int32_t advances);

/* Rate fits of hydrogen_only/mod.rs:161-273 at temperature T (K) and scale factor a.
 * which: 0 case-B recombination rate, 1 its derivative, 2 collisional ionization rate,
 * 3 derivative, 4 collisional ionization cooling, 5 derivative, 6 collisional excitation
 * cooling, 7 derivative, 8 case-B recombination cooling, 9 derivative, 10 bremsstrahlung
 * cooling, 11 derivative, 12 Compton cooling, 13 derivative.  SI units. */
double orc_rate_fit(int32_t which, double temperature, double scale_factor);

/* Solver::perform_timestep (hydrogen_only/mod.rs:426-441). Returns the chosen timescale
 * in *timescale_out and its process (0 temperature, 1 ionization fraction, 2 photon rate);
 * return value 0 ok, 1 convergence failed (pessimistic dt/10 returned). */
int32_t orc_solver_perform_timestep(double* xhii, double* temperature, double density,
                                    double volume, double length, double rate,
                                    double scale_factor, int32_t has_floor, double floor_t,
                                    double floor_x, double timestep, double safety,
                                    double* timescale_out, int32_t* process_out);

/* The task heap on its own: BinaryHeap::from of n_init tasks with directions
 * init_dirs (task i gets cell id i), then ops in order: a value >= 0 pushes a task of
 * that direction (cell ids continue from n_init), -1 pops and writes the popped cell
 * id to out (in order).  Returns the number of ids written; -1 on a pop of an empty
 * heap. */
int64_t orc_heap_replay(const int64_t* init_dirs, int64_t n_init, const int64_t* ops, int64_t n_ops,
                        int64_t* out);

/* Periodic Voronoi tessellation of n generators in [0, box)^3 (voronoi_oracle.cpp),
 * built on num_threads threads, as face-neighbour CSR with the kinds above.  NULL on
 * invalid arguments; failed cells (none expected) and faces dropped for want of a
 * reciprocal are counted. */
typedef struct orc_voronoi orc_voronoi;
orc_voronoi* orc_voronoi_build(const double* points, int64_t n, double box, int32_t num_threads);
int64_t orc_voronoi_num_faces(const orc_voronoi* g);
int64_t orc_voronoi_failed_cells(const orc_voronoi* g);
int64_t orc_voronoi_dropped_faces(const orc_voronoi* g);
void orc_voronoi_copy(const orc_voronoi* g, int64_t* row_ptr, int32_t* nbr, uint8_t* kind, double* area,
                      double* normal, double* volume, double* size);
void orc_voronoi_free(orc_voronoi* g);

/* Directions::from_num (src/sweep/direction/mod.rs:58-75): the reference's direction
 * table for num in {1, 16, 21, 32, 64, 84} into out[num*3]; 0 on success, -1 otherwise. */
int32_t orc_directions_from_num(int32_t num, double* out);

/* Outgoing rate of one task (hydrogen_only/mod.rs:72-88). */
double orc_outgoing_rate(double density, double xhii, double size, double incoming_rate,
                         double threshold);

#ifdef __cplusplus
}
#endif
#endif
