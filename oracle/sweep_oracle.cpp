// CPU FP64 oracle: restatement of the subsweep sweep + hydrogen-only chemistry.
//
// TEST INFRASTRUCTURE ONLY (see oracle.h).  Every function cites the reference
// file:line it restates (paths within Tehforsch/subsweep).  Compile with
// -O2 -fno-fast-math -ffp-contract=off so that every expression rounds exactly as
// the Rust reference's (which never contracts to FMA) does.  The transcendental
// functions are glibc's, which is what Rust's std uses on Linux.
#include "oracle.h"

// The reference's direction tables (src/sweep/direction/healpix.rs), as the generated
// data file the library is built with; the tests hold its digests against the reference.
#include "../subsweep_gb300/csrc/direction_bins.inc"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <chrono>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <utility>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// Units and constants: src/units/mod.rs:14-108.  Every quantity is a plain SI
// double; a unit constructor multiplies the literal by the unit's SI factor.
// ---------------------------------------------------------------------------
const double kMeters = 1.0;
const double kCentimeters = 0.01 * kMeters;                       // mod.rs:19
const double kCentimetersSquared = kCentimeters * kCentimeters;   // mod.rs:91
const double kCubicMeters = 1.0;                                  // mod.rs:75
const double kCubicCentimeters = 1e-6 * kCubicMeters;             // mod.rs:76
const double kSeconds = 1.0 * 1.0;                                // mod.rs:44
const double kCentimetersCubedPerS = kCubicCentimeters / kSeconds;  // mod.rs:93
const double kJoules = 1.0 * 1.0;                                 // mod.rs:59
const double kErgs = 1e-7 * kJoules;                              // mod.rs:60
const double kErgsCentimetersCubedPerS = kErgs * kCentimetersCubedPerS;  // mod.rs:95
const double kErgsPerS = kErgs / kSeconds;                        // mod.rs:72
const double kElectronVolts = 1.602176634e-19 * kJoules;          // mod.rs:61
const double kKelvins = 1.0;
const double kKilograms = 1.0;
const double BOLTZMANN_CONSTANT = 1.380649e-23 * kJoules / kKelvins;  // mod.rs:101
const double PROTON_MASS = 1.67262192369e-27 * kKilograms;             // mod.rs:102
const double GAMMA = 5.0 / 3.0;                                        // mod.rs:104
const double SIGMA = 2.9580524545305314e-18 * kCentimetersSquared;     // mod.rs:105
const double PHOTON_AVERAGE_ENERGY = 18.028356312818811 * kElectronVolts;  // mod.rs:107
const double RYDBERG_CONSTANT = 13.65693 * kElectronVolts;                 // mod.rs:108

const int MAX_DEPTH = 100;                        // hydrogen_only/mod.rs:34
const double IONIZED_FRACTION_EPSILON = 1e-10;    // hydrogen_only/mod.rs:38
const double HYDROGEN_MASS_FRACTION = 1.0;        // hydrogen_only/mod.rs:32

enum Process { PROC_TEMPERATURE = 0, PROC_IONIZATION = 1, PROC_PHOTON_RATE = 2 };

struct Timescale {
  double time;
  int process;
  // chemistry/timescale.rs:114-120 (strict <, NaN picks `other`)
  Timescale min(const Timescale& other) const { return time < other.time ? *this : other; }
};

inline double powi2(double x) { return x * x; }
inline double powi3(double x) { return x * x * x; }
inline double powi4(double x) { double x2 = x * x; return x2 * x2; }

// glam DVec3::dot: (x*x') + (y*y') + (z*z')
inline double dot3(const double* a, const double* b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

// ---------------------------------------------------------------------------
// Solver: src/chemistry/hydrogen_only/mod.rs:125-461
// ---------------------------------------------------------------------------
struct Solver {
  double x, temperature, density, volume, length, rate, scale_factor;
  bool has_floor;
  double floor_t, floor_x;
  bool clamp_panicked = false;

  double hydrogen_number_density() const { return density / PROTON_MASS; }            // 139-141
  double ionized_number_density() const { return hydrogen_number_density() * x; }     // 143-145
  double neutral_number_density() const { return hydrogen_number_density() * (1.0 - x); }  // 147-149
  double electron_number_density() const { return ionized_number_density(); }          // 151-154
  double mu() const { return 1.0 / (x + 1.0); }                                        // 156-159

  double collision_fit_function() const {  // 161-164
    double t = temperature;
    return std::sqrt(t) / (1.0 + std::sqrt(t / 1e5)) * std::exp(-157809.1 / t);
  }
  double collision_fit_function_derivative() const {  // 166-173
    double const1 = 1.0 / 1e5;
    double const2 = 157809.1;
    double t = temperature;
    return (std::exp(-const2 / t) *
            (const1 * const2 * t + 0.5 * std::sqrt(const1 * t) * (2.0 * const2 + t))) /
           (std::sqrt(powi3(t)) * std::sqrt(const1 * t) * powi2(std::sqrt(const1 * t) + 1.0));
  }
  double case_b_recombination_rate() const {  // 175-180
    double lambda = 315614.0 * kKelvins / temperature;
    return (2.753e-14 * std::pow(lambda, 1.5) /
            std::pow(1.0 + std::pow(lambda / 2.74, 0.407), 2.242)) *
           kCentimetersCubedPerS;
  }
  double case_b_recombination_rate_derivative() const {  // 182-194
    double lambda = 315614.0 * kKelvins / temperature;
    double dlambda_dt = -(315614.0 * kKelvins) / (temperature * temperature);
    double c1 = 1.0 / 2.74;
    double c2 = 0.407;
    double c3 = 2.242;
    double d = -std::sqrt(lambda) * std::pow(std::pow(c1 * lambda, c2) + 1.0, -c3 - 1.0) *
               (c2 * c3 * std::pow(c1 * lambda, c2) - 1.5 * std::pow(c1 * lambda, c2) - 1.5);
    return ((2.753e-14 * d) * kCentimetersCubedPerS) * dlambda_dt;
  }
  double case_b_recombination_cooling_rate() const {  // 196-202
    double lambda = 315614.0 * kKelvins / temperature;
    return (3.435e-30 * temperature * std::pow(lambda, 1.97) /
            std::pow(1.0 + std::pow(lambda / 2.25, 0.376), 3.72)) *
           kErgsCentimetersCubedPerS;
  }
  double case_b_recombination_cooling_rate_derivative() const {  // 204-216
    double c1 = 315614.0, c2 = 1.97, c3 = 0.376, c4 = 3.72, c5 = 2.25;
    double t = temperature;
    double derivative = std::pow(1.0 + std::pow(c1 / (c5 * t), c3), -1.0 - c4) *
                        (1.0 - 1.0 * c2 + (1.0 - 1.0 * c2 + c3 * c4) * std::pow(c1 / (c5 * t), c3)) *
                        std::pow(c1 / t, c2);
    return ((3.435e-30 * derivative) * kErgsCentimetersCubedPerS) / kKelvins;
  }
  double collisional_ionization_rate() const {  // 218-220
    return (5.85e-11 * collision_fit_function()) * kCentimetersCubedPerS;
  }
  double collisional_ionization_rate_derivative() const {  // 222-225
    return ((5.85e-11 * collision_fit_function_derivative()) * kCentimetersCubedPerS) / kKelvins;
  }
  double collisional_ionization_cooling_rate() const {  // 227-229
    return (1.27e-21 * collision_fit_function()) * kErgsCentimetersCubedPerS;
  }
  double collisional_ionization_cooling_rate_derivative() const {  // 231-235
    return ((1.27e-21 * collision_fit_function_derivative()) * kErgsCentimetersCubedPerS) /
           kKelvins;
  }
  double collisional_excitation_cooling_rate() const {  // 237-242
    double t = temperature;
    return (7.5e-19 / (1.0 + std::sqrt(t / 1e5)) * std::exp(-118348.0 / t)) *
           kErgsCentimetersCubedPerS;
  }
  double collisional_excitation_cooling_rate_derivative() const {  // 244-253
    double t = temperature;
    double c1 = 7.5e-19, c2 = 118348.0, c3 = 1.0 / 1e5;
    double v = (c1 * std::exp(-c2 / t) *
                (c2 * c3 * t - 0.5 * c3 * powi2(t) + c2 * std::sqrt(c3 * t))) /
               (powi2(t) * std::sqrt(c3 * t) * powi2(1.0 + std::sqrt(c3 * t)));
    return (v * kErgsCentimetersCubedPerS) / kKelvins;
  }
  double bremsstrahlung_cooling_rate() const {  // 255-257
    return (1.42e-27 * std::sqrt(temperature)) * kErgsCentimetersCubedPerS;
  }
  double bremsstrahlung_cooling_rate_derivative() const {  // 259-263
    return ((1.42e-27 / (2.0 * std::sqrt(temperature))) * kErgsCentimetersCubedPerS) / kKelvins;
  }
  double compton_cooling_rate() const {  // 265-268
    double xx = 2.727 / scale_factor;
    return (1.017e-37 * powi4(xx) * (temperature - xx)) * kErgsPerS;
  }
  double compton_cooling_rate_derivative() const {  // 270-273
    double xx = 2.727 / scale_factor;
    return ((1.017e-37 * powi4(xx)) * kErgsPerS) / kKelvins;
  }
  double cooling_rate() const {  // 275-287
    double ne = electron_number_density();
    double nh_neutral = neutral_number_density();
    double nh_ionized = ionized_number_density();
    double collisional =
        (collisional_excitation_cooling_rate() + collisional_ionization_cooling_rate()) * ne *
        nh_neutral;
    double recombination = case_b_recombination_cooling_rate() * ne * nh_ionized;
    double bremsstrahlung = bremsstrahlung_cooling_rate() * ne * nh_ionized;
    double compton = compton_cooling_rate() * ne;
    return collisional + recombination + bremsstrahlung + compton;
  }
  double cooling_rate_derivative() const {  // 289-302
    double ne = electron_number_density();
    double nh_neutral = neutral_number_density();
    double nh_ionized = ionized_number_density();
    double collisional = (collisional_excitation_cooling_rate_derivative() +
                          collisional_ionization_cooling_rate_derivative()) *
                         ne * nh_neutral;
    double recombination = case_b_recombination_cooling_rate_derivative() * ne * nh_ionized;
    double bremsstrahlung = bremsstrahlung_cooling_rate_derivative() * ne * nh_ionized;
    double compton = compton_cooling_rate_derivative() * ne;
    return collisional + recombination + bremsstrahlung + compton;
  }
  double num_newly_ionized_hydrogen_atoms(double timestep) const {  // 312-319
    double nhn = neutral_number_density();
    double absorbed_fraction = 1.0 - std::exp(-nhn * SIGMA * length);
    double num_photons = timestep * rate;
    return num_photons * absorbed_fraction;
  }
  double photoheating_rate(double timestep) const {  // 321-325
    double num = num_newly_ionized_hydrogen_atoms(timestep);
    double ionization_density = num / volume;
    return ionization_density * (PHOTON_AVERAGE_ENERGY - RYDBERG_CONSTANT) / timestep;
  }
  double photoionization_rate(double timestep) const {  // 327-332
    double num = num_newly_ionized_hydrogen_atoms(timestep);
    double fraction = num / (neutral_number_density() * volume);
    return fraction / timestep;
  }
  double temperature_change(double timestep) const {  // 304-310
    double k = (GAMMA - 1.0) * PROTON_MASS / (density * BOLTZMANN_CONSTANT);
    double lambda = photoheating_rate(timestep) - cooling_rate();
    double dlambdadt = -cooling_rate_derivative();
    double m = mu();
    return k * m * lambda * timestep / (1.0 - k * m * dlambdadt * timestep);
  }
  double ionized_fraction_change(double timestep) const {  // 334-354
    double nh = hydrogen_number_density();
    double ne = electron_number_density();
    double alpha = case_b_recombination_rate();
    double dalpha = case_b_recombination_rate_derivative();
    double beta = collisional_ionization_rate();
    double dbeta = collisional_ionization_rate_derivative();
    double photo = photoionization_rate(timestep);
    double c = beta * ne + photo;
    double m = mu();
    double d = alpha * ne;
    double xhii = x;
    double rhsc = ne * temperature * m * HYDROGEN_MASS_FRACTION * dbeta;
    double dcdx = nh * beta - rhsc;
    double rhsd = ne * temperature * m * HYDROGEN_MASS_FRACTION * dalpha;
    double dddx = nh * alpha - rhsd;
    double j = dcdx - (c + d) - xhii * (dcdx + dddx);
    return timestep * (c - xhii * (c + d)) / (1.0 - j * timestep);
  }
  void clamp() {  // 356-369, with f64::clamp semantics (asserts min <= max)
    double xf = has_floor ? floor_x : IONIZED_FRACTION_EPSILON;
    double xmax = 1.0 - IONIZED_FRACTION_EPSILON;
    if (!(xf <= xmax)) clamp_panicked = true;  // the reference panics here
    if (x < xf) x = xf;
    if (x > xmax) x = xmax;
    if (has_floor && temperature < floor_t) temperature = floor_t;
  }
  // update() 444-461. Returns false on TimestepCriterionViolated.
  static bool update(double& value, double change, double max_allowed, double timestep,
                     double& recommendation) {
    double relative_change = std::fmin(std::fabs(change / value), 1.0 / DBL_EPSILON);
    if (relative_change > max_allowed) return false;
    value += change;
    recommendation = timestep * (max_allowed / relative_change);
    return true;
  }
  bool try_timestep_update(double timestep, double safety, Timescale& out) {  // 371-392
    double tc = temperature_change(timestep);
    double rec_t;
    if (!update(temperature, tc, safety, timestep, rec_t)) return false;
    Timescale ideal_t{rec_t, PROC_TEMPERATURE};
    double xc = ionized_fraction_change(timestep);
    double rec_x;
    if (!update(x, xc, safety, timestep, rec_x)) return false;
    Timescale ideal_x{rec_x, PROC_IONIZATION};
    clamp();
    out = ideal_t.min(ideal_x);
    return true;
  }
  // perform_timestep_internal 394-424; false = TimestepConvergenceFailed.
  bool perform_internal(double timestep, double safety, int depth, Timescale& out,
                        int64_t& attempts) {
    clamp();
    double init_t = temperature, init_x = x;
    if (depth > MAX_DEPTH) return false;
    ++attempts;
    if (!try_timestep_update(timestep, safety, out)) {
      temperature = init_t;
      x = init_x;
      if (!perform_internal(timestep / 2.0, safety, depth + 1, out, attempts)) return false;
      return perform_internal(timestep / 2.0, safety, depth + 1, out, attempts);
    }
    return true;
  }
  // perform_timestep 426-441
  Timescale perform_timestep(double timestep, double safety, bool* failed, int64_t& attempts) {
    Timescale out{0.0, PROC_TEMPERATURE};
    if (!perform_internal(timestep, safety, 0, out, attempts)) {
      *failed = true;
      return Timescale{timestep / 10.0, PROC_TEMPERATURE};
    }
    *failed = false;
    return out;
  }
};

// TimestepLevel::from_max_timestep_and_desired_timestep, timestep_level.rs:27-36,
// with Rust's saturating float->usize cast.
int32_t timestep_level(int32_t max_num_levels, double max_timestep, double desired) {
  double ratio = max_timestep / desired;
  double v = std::ceil(std::log2(ratio));
  int64_t level;
  if (std::isnan(v) || v <= 0.0)
    level = 0;
  else if (v >= 9.2e18)
    level = INT64_MAX;
  else
    level = (int64_t)v;
  if (level > max_num_levels - 1) level = max_num_levels - 1;
  return (int32_t)level;
}

// TimestepState, timestep_state.rs:5-90
struct TimestepState {
  double max_timestep;
  int32_t max_num_levels;
  int32_t lowest;
  bool first_done = false;
  TimestepState(double m, int32_t n) : max_timestep(m), max_num_levels(n), lowest(n - 1) {}
  std::vector<int32_t> sweep_order() const {  // 22-27, 70-75
    int32_t num = max_num_levels - lowest;
    std::vector<int32_t> out;
    for (uint32_t i = 0; i < (1u << (num - 1)); ++i) {
      uint32_t first_bit = (uint32_t)(num - 1);
      for (uint32_t b = 0; b < 32; ++b)
        if (i & (1u << b)) { first_bit = b; break; }
      out.push_back(lowest + (int32_t)(num - 1 - first_bit));
    }
    return out;
  }
  void advance() {  // 37-48
    if (first_done && lowest > 0) lowest -= 1;
    if (!first_done) first_done = true;
  }
  double timestep_at_level(int32_t level) const {  // timestep_level.rs:42-48
    return max_timestep * std::pow(0.5, level);
  }
  double current_max_timestep() const { return max_timestep * std::pow(0.5, lowest); }  // 77-79
  int32_t desired_level(double desired) const {  // 54-64
    int32_t level = timestep_level(max_num_levels, max_timestep, desired);
    if (level < lowest) level = lowest;
    return level;
  }
};

}  // namespace

// ---------------------------------------------------------------------------
// The reference's task queue: std::collections::BinaryHeap<Task> (src/sweep/mod.rs:104)
// with Task ordered by direction alone (task.rs:25-35), so every task of a direction
// compares equal.  Restated from the Rust standard library's published source
// (library/alloc/src/collections/binary_heap/mod.rs): FromIterator collects into a
// Vec and heapifies it (`rebuild`: sift_down from len/2 - 1 down to 0), `push` sifts
// the new element up, `pop` swaps the last element into the root, sifts that hole down
// to the bottom always taking the greater child (the right one on ties) and sifts it
// back up.  Equal keys stop both sifts, which is what fixes the order of equal tasks.
// ---------------------------------------------------------------------------
struct Task {
  int64_t cell;
  int64_t dir;
};

class TaskHeap {
 public:
  // BinaryHeap::from(Vec): rebuild()
  void assign(std::vector<Task>&& v) {
    data_ = std::move(v);
    size_t n = data_.size() / 2;
    while (n > 0) {
      --n;
      sift_down_range(n, data_.size());
    }
  }
  bool empty() const { return data_.empty(); }
  size_t size() const { return data_.size(); }
  // BinaryHeap::push: push then sift_up(0, old_len)
  void push(Task t) {
    data_.push_back(t);
    sift_up(0, data_.size() - 1);
  }
  // BinaryHeap::pop: swap the last element into the root, sift_down_to_bottom(0)
  Task pop() {
    Task item = data_.back();
    data_.pop_back();
    if (!data_.empty()) {
      std::swap(item, data_[0]);
      sift_down_to_bottom(0);
    }
    return item;
  }

 private:
  std::vector<Task> data_;

  size_t sift_up(size_t start, size_t pos) {
    const Task elem = data_[pos];
    while (pos > start) {
      size_t parent = (pos - 1) / 2;
      if (elem.dir <= data_[parent].dir) break;
      data_[pos] = data_[parent];
      pos = parent;
    }
    data_[pos] = elem;
    return pos;
  }
  size_t sift_down_range(size_t pos, size_t end) {
    const Task elem = data_[pos];
    size_t child = 2 * pos + 1;
    while (child + 2 <= end) {  // child <= end.saturating_sub(2)
      if (data_[child].dir <= data_[child + 1].dir) child += 1;
      if (elem.dir >= data_[child].dir) {
        data_[pos] = elem;
        return pos;
      }
      data_[pos] = data_[child];
      pos = child;
      child = 2 * pos + 1;
    }
    if (child + 1 == end && elem.dir < data_[child].dir) {
      data_[pos] = data_[child];
      pos = child;
    }
    data_[pos] = elem;
    return pos;
  }
  void sift_down_to_bottom(size_t pos) {
    const size_t end = data_.size(), start = pos;
    const Task elem = data_[pos];
    size_t child = 2 * pos + 1;
    while (child + 2 <= end) {
      if (data_[child].dir <= data_[child + 1].dir) child += 1;
      data_[pos] = data_[child];
      pos = child;
      child = 2 * pos + 1;
    }
    if (child + 1 == end) {
      data_[pos] = data_[child];
      pos = child;
    }
    data_[pos] = elem;
    sift_up(start, pos);
  }
};

// FIFO queue of one direction's ready tasks (the oracle's default order).
struct FifoQueue {
  std::deque<Task> q;
  bool empty() const { return q.empty(); }
  void push(Task t) { q.push_back(t); }
  Task pop() {
    Task t = q.front();
    q.pop_front();
    return t;
  }
};

// Work counters of one worker thread.
struct WorkCount {
  int64_t tasks = 0, chem_cells = 0, chem_attempts = 0, chem_failures = 0;
  bool panicked = false;
};

// ---------------------------------------------------------------------------
// Sweep<HydrogenOnly>: src/sweep/mod.rs:171-610
// ---------------------------------------------------------------------------
struct orc_sim {
  orc_params p;
  std::vector<double> dirs;
  int64_t n;
  int32_t D;
  std::vector<int64_t> row_ptr;
  std::vector<int32_t> nbr;
  std::vector<uint8_t> kind;
  std::vector<double> area, normal, volume, size;
  // Site (site.rs:12-23) in SoA form; per-(cell, dir) arrays are direction-major,
  // [dir * n + cell], so the threads of a level sweep (one set of directions each)
  // write disjoint memory
  std::vector<double> density, source, xhii, temperature, species_timestep, change_timescale,
      previous_rate;
  std::vector<double> incoming, outgoing, periodic, periodic_pending;
  std::vector<uint32_t> missing;
  std::vector<uint8_t> level;
  TimestepState ts;
  int64_t tasks_solved = 0, chem_cells = 0, chem_attempts = 0, chem_failures = 0;
  bool panicked = false;

  explicit orc_sim(const orc_params* pp) : p(*pp), ts(pp->max_timestep, pp->num_timestep_levels) {}

  size_t at(int64_t c, int32_t d) const { return (size_t)d * (size_t)n + (size_t)c; }
  int threads() const { return p.num_threads > 1 ? p.num_threads : 1; }

  double get_rate(int64_t c, int32_t d) const {  // site.rs:53-56
    double src = source[c] / (double)D;
    return incoming[at(c, d)] + src + periodic[at(c, d)];
  }
  bool active(int64_t c, int32_t current) const { return level[c] >= current; }

  // ActiveList::enumerate_active (active_list.rs:55-66): the bins of levels current..L-1
  // in turn, each bin in index order (update_bins, 143-153)
  std::vector<int64_t> active_in_bin_order(int32_t current) const {
    std::vector<int64_t> order;
    for (int32_t l = current; l < p.num_timestep_levels; ++l)
      for (int64_t c = 0; c < n; ++c)
        if (level[c] == l) order.push_back(c);
    return order;
  }

  // Sweep::init_counts (mod.rs:346-386) for one direction: upwind faces whose neighbour
  // is LOCAL and active.
  void init_counts_dir(int32_t current, int32_t d, const std::vector<int64_t>& act,
                       std::vector<uint32_t>& out) const {
    const double* dir = &dirs[3 * d];
    for (int64_t c : act) {
      uint32_t cnt = 0;
      for (int64_t f = row_ptr[c]; f < row_ptr[c + 1]; ++f) {
        bool upwind = dot3(&normal[3 * f], dir) < 0.0;
        if (!upwind || kind[f] == ORC_BOUNDARY) continue;
        if (!active(nbr[f], current)) continue;
        if (kind[f] == ORC_LOCAL) cnt += 1;
      }
      out[at(c, d)] = cnt;
    }
  }

  // HydrogenOnly::get_outgoing_rate, hydrogen_only/mod.rs:72-88
  double outgoing_rate(int64_t c, double incoming_rate) const {
    double nhn = density[c] / PROTON_MASS * (1.0 - xhii[c]);
    if (incoming_rate < p.significant_rate_threshold) return 0.0;
    double non_absorbed = std::exp(-nhn * SIGMA * size[c]);
    return incoming_rate * non_absorbed;
  }

  // handle_local_neighbour (mod.rs:487-503) and handle_local_periodic_neighbour
  // (505-513): a rate correction arriving at (nb, d), from a task of this rank or in a
  // message from another.
  template <typename Queue>
  void deliver(int64_t nb, int32_t d, double w, bool periodic_face, int32_t current, Queue& queue) {
    if (periodic_face) {
      if (p.periodic_mode == ORC_PERIODIC_IMMEDIATE)
        periodic[at(nb, d)] += w;
      else
        periodic_pending[at(nb, d)] += w;
      return;
    }
    incoming[at(nb, d)] += w;
    if (active(nb, current)) {
      uint32_t& m = missing[at(nb, d)];
      m -= 1;
      if (m == 0) queue.push(Task{nb, d});
    }
  }

  // Sweep::solve_task, mod.rs:423-485 (+ get_outgoing_rate 412-421).  With `ranks`,
  // corrections for cells another rank owns become messages to it (handle_remote_
  // neighbour / handle_remote_periodic_neighbour, mod.rs:515-547).
  template <typename Queue>
  void solve_task(int64_t c, int32_t d, int32_t current, Queue& queue, WorkCount& work,
                  struct RankCtx* ranks = nullptr);

  // Run `body(worker, work)` on every worker thread (worker 0 on the calling thread).
  template <typename Body>
  void on_threads(Body body, std::vector<WorkCount>& work) {
    const int T = threads();
    work.assign(T, WorkCount{});
    std::vector<std::thread> pool;
    for (int t = 1; t < T; ++t) pool.emplace_back([&, t] { body(t, work[t]); });
    body(0, work[0]);
    for (std::thread& th : pool) th.join();
  }

  // Sweep::update_chemistry, mod.rs:549-574 (+ HydrogenOnly::update_abundances 90-119),
  // for the active cells in [begin, end)
  void update_chemistry_range(int32_t current, int64_t begin, int64_t end, WorkCount& work) {
    for (int64_t c = begin; c < end; ++c) {
      if (!active(c, current)) continue;
      double timestep = ts.timestep_at_level(level[c]);
      double rate = 0.0;
      for (int32_t d = 0; d < D; ++d) rate += get_rate(c, d);
      double relative_change;
      if (std::fabs(rate) < std::fabs(p.significant_rate_threshold)) {  // chemistry/mod.rs:79-81
        relative_change = 0.0;
      } else {  // chemistry/mod.rs:73-77
        relative_change = std::fabs(
            std::fmin(std::fabs(std::fabs(rate - previous_rate[c]) / rate), 1.0 / DBL_EPSILON));
      }
      previous_rate[c] = rate;
      Timescale rate_ts{timestep / relative_change, PROC_PHOTON_RATE};
      Solver s;
      s.x = xhii[c];
      s.temperature = temperature[c];
      s.density = density[c];
      s.volume = volume[c];
      s.length = size[c];
      s.rate = rate;
      s.scale_factor = p.scale_factor;
      s.has_floor = p.prevent_cooling != 0;
      s.floor_t = temperature[c];
      s.floor_x = xhii[c];
      bool failed = false;
      Timescale chem_ts = s.perform_timestep(timestep, p.chemistry_timestep_safety_factor, &failed,
                                             work.chem_attempts);
      if (failed) ++work.chem_failures;
      if (s.clamp_panicked) work.panicked = true;
      temperature[c] = s.temperature;
      xhii[c] = s.x;
      species_timestep[c] = chem_ts.time;
      Timescale change = rate_ts.min(chem_ts);
      change_timescale[c] = change.time;
      ++work.chem_cells;
    }
  }

  void add_work(const std::vector<WorkCount>& work) {
    for (const WorkCount& w : work) {
      tasks_solved += w.tasks;
      chem_cells += w.chem_cells;
      chem_attempts += w.chem_attempts;
      chem_failures += w.chem_failures;
      panicked = panicked || w.panicked;
    }
  }

  // Directions of worker t among `dset`: dset[t], dset[t + T], ...
  std::vector<int32_t> worker_dirs(int t, const std::vector<int32_t>& dset) const {
    std::vector<int32_t> out;
    for (size_t k = (size_t)t; k < dset.size(); k += (size_t)threads()) out.push_back(dset[k]);
    return out;
  }

  // One worker's share of a level sweep when the workers split the directions.
  // ORDER_HEAP: the reference's queue, get_initial_tasks (mod.rs:388-398: directions
  // outer, active sites in bin order inner) collected into the BinaryHeap restated
  // above and popped to exhaustion (solve, mod.rs:291-314; on one rank the
  // send/receive pauses do not change the order); with one worker this is the
  // reference's task order exactly, with several each worker runs that heap over its
  // own directions.  ORDER_FIFO: per direction, highest first (the heap's key order),
  // a FIFO queue seeded in index order.
  void sweep_worker(int32_t current, const std::vector<int32_t>& mine, const std::vector<int64_t>& act,
                    WorkCount& work) {
    for (int32_t d : mine) init_counts_dir(current, d, act, missing);
    if (p.order == ORC_ORDER_HEAP) {
      std::vector<Task> initial;
      for (int32_t d : mine)
        for (int64_t c : act)
          if (missing[at(c, d)] == 0) initial.push_back(Task{c, d});
      TaskHeap heap;
      heap.assign(std::move(initial));
      while (!heap.empty()) {
        Task task = heap.pop();
        solve_task(task.cell, (int32_t)task.dir, current, heap, work);
      }
      return;
    }
    for (auto it = mine.rbegin(); it != mine.rend(); ++it) {
      const int32_t d = *it;
      FifoQueue queue;
      for (int64_t c = 0; c < n; ++c)  // get_initial_tasks, mod.rs:388-398
        if (active(c, current) && missing[at(c, d)] == 0) queue.push(Task{c, d});
      while (!queue.empty()) {
        Task task = queue.pop();
        solve_task(task.cell, d, current, queue, work);
      }
    }
  }

  void domain_rank(int32_t current, const std::vector<int32_t>& dset, const std::vector<int64_t>& act,
                   struct Domains& dom, int rank, WorkCount& work);

  // The transport of one level sweep over the directions `dset`; returns the tasks
  // solved.  PARTITION_DIRECTIONS: each worker sweeps its own directions.
  // PARTITION_DOMAINS: each worker is a rank owning a contiguous block of cell ids
  // (a spatially compact domain on Morton-ordered grids) and sweeps every direction of
  // its cells, exchanging rate corrections with the other ranks as the reference's
  // MPI ranks do.
  int64_t sweep_transport(int32_t current, const std::vector<int32_t>& dset, const std::vector<int64_t>& act);

  // Sweep::update_chemistry over the active cells act[first .. first + count) (indices
  // taken modulo the active count), split between the workers.
  void chemistry(int32_t current, const std::vector<int64_t>& act, int64_t first, int64_t count) {
    const int T = threads();
    const int64_t na = (int64_t)act.size();
    if (na == 0 || count <= 0) return;
    std::vector<int64_t> cells;
    if (first == 0 && count >= na) {
      cells = act;
      std::sort(cells.begin(), cells.end());
    } else {
      for (int64_t k = 0; k < count && k < na; ++k) cells.push_back(act[(size_t)((first + k) % na)]);
    }
    std::vector<WorkCount> work;
    on_threads(
        [&](int t, WorkCount& w) {
          const int64_t m = (int64_t)cells.size(), chunk = (m + T - 1) / T;
          for (int64_t k = std::min(m, t * chunk); k < std::min(m, (t + 1) * chunk); ++k)
            update_chemistry_range(current, cells[k], cells[k] + 1, w);
        },
        work);
    add_work(work);
  }

  // Snapshot semantics: the periodic contributions of the sweep's directions become
  // visible now.
  void merge_periodic_pending(const std::vector<int32_t>& dset) {
    if (p.periodic_mode != ORC_PERIODIC_SNAPSHOT) return;
    std::vector<WorkCount> work;
    on_threads(
        [&](int t, WorkCount&) {
          for (size_t k = (size_t)t; k < dset.size(); k += (size_t)threads())
            for (int64_t c = 0; c < n; ++c) {
              const size_t i = at(c, dset[k]);
              periodic[i] += periodic_pending[i];
              periodic_pending[i] = 0.0;
            }
        },
        work);
  }

  // Sweep::single_sweep, mod.rs:274-289.
  bool single_sweep(int32_t current) {
    std::vector<int32_t> all(D);
    for (int32_t d = 0; d < D; ++d) all[d] = d;
    const std::vector<int64_t> act = active_in_bin_order(current);
    const int64_t solved = sweep_transport(current, all, act);
    merge_periodic_pending(all);
    chemistry(current, act, 0, (int64_t)act.size());
    return solved == (int64_t)act.size() * (int64_t)D;
  }

  // Sweep::update_timestep_levels, mod.rs:576-589
  void update_timestep_levels() {
    for (int64_t c = 0; c < n; ++c) {
      double desired = p.timestep_safety_factor * change_timescale[c];
      level[c] = (uint8_t)ts.desired_level(desired);
    }
  }

  void level_counts(int64_t* counts) const {
    for (int32_t l = 0; l < p.num_timestep_levels; ++l) counts[l] = 0;
    for (int64_t c = 0; c < n; ++c)
      for (int32_t l = 0; l <= level[c]; ++l) counts[l] += 1;
  }

  // Sweep::run_sweeps, mod.rs:258-272
  int run_sweeps(double* time_elapsed) {
    std::vector<int64_t> counts(p.num_timestep_levels);
    level_counts(counts.data());
    int status = 0;
    for (int32_t l : ts.sweep_order())
      if (counts[l] > 0)
        if (!single_sweep(l)) status = 1;
    *time_elapsed = ts.current_max_timestep();
    ts.advance();
    update_timestep_levels();
    return status;
  }
};

// ---------------------------------------------------------------------------
// Domain decomposition on threads: the reference's parallel scheme (MPI ranks owning
// spatial domains, src/sweep/mod.rs:291-314 and 515-547, communicator.rs) with one
// thread per rank and per-rank inboxes in place of MPI messages.  Each rank counts
// a neighbour in another domain like a local one (Remote, mod.rs:364-371), solves its
// own tasks from its own queue, sends the corrections for other ranks' cells in
// batches after every num_tasks_to_solve_before_send_receive tasks (default 10000,
// parameters.rs:64-78) or when its queue runs dry, and keeps receiving until every
// rank is done (periodic corrections carry no count, so they may arrive late).
// ---------------------------------------------------------------------------
struct Message {
  int64_t cell;
  int32_t dir;
  int32_t periodic;
  double w;
};

struct Domains {
  int ranks;
  int64_t chunk;  // cells per rank: rank r owns [r * chunk, (r + 1) * chunk)
  std::vector<std::unique_ptr<std::mutex>> lock;
  std::vector<std::vector<Message>> inbox;
  std::atomic<int> done{0};
  std::atomic<bool> stalled{false};
  Domains(int r, int64_t n) : ranks(r), chunk((n + r - 1) / r), inbox(r) {
    for (int k = 0; k < r; ++k) lock.emplace_back(new std::mutex());
  }
  int owner(int64_t c) const { return (int)(c / chunk); }
};

struct RankCtx {
  int rank;
  Domains* dom;
  std::vector<std::vector<Message>> outbox;
};

template <typename Queue>
void orc_sim::solve_task(int64_t c, int32_t d, int32_t current, Queue& queue, WorkCount& work, RankCtx* ranks) {
  double& inc = incoming[at(c, d)];
  if (inc < 0.0) inc = 0.0;  // Photons::make_positive, chemistry/mod.rs:61-65
  double out_new = outgoing_rate(c, get_rate(c, d));
  double corr = out_new - outgoing[at(c, d)];
  outgoing[at(c, d)] = out_new;
  const double* dir = &dirs[3 * d];
  double total_effective_area = 0.0;
  for (int64_t f = row_ptr[c]; f < row_ptr[c + 1]; ++f) {
    double dt = dot3(&normal[3 * f], dir);
    if (dt > 0.0) total_effective_area += area[f] * dt;
  }
  for (int64_t f = row_ptr[c]; f < row_ptr[c + 1]; ++f) {
    double dt = dot3(&normal[3 * f], dir);
    if (!(dt > 0.0)) continue;
    double effective_area = area[f] * dt;
    double w = corr * (effective_area / total_effective_area);
    if (kind[f] == ORC_BOUNDARY) continue;
    const int64_t nb = nbr[f];
    const bool periodic_face = kind[f] == ORC_LOCAL_PERIODIC;
    if (ranks && ranks->dom->owner(nb) != ranks->rank)
      ranks->outbox[ranks->dom->owner(nb)].push_back(Message{nb, d, periodic_face ? 1 : 0, w});
    else
      deliver(nb, d, w, periodic_face, current, queue);
  }
  ++work.tasks;
}

void orc_sim::domain_rank(int32_t current, const std::vector<int32_t>& dset, const std::vector<int64_t>& act,
                          Domains& dom, int rank, WorkCount& work) {
  RankCtx ctx{rank, &dom, std::vector<std::vector<Message>>(dom.ranks)};
  std::vector<int64_t> mine;  // this rank's active cells, in the global bin order
  for (int64_t c : act)
    if (dom.owner(c) == rank) mine.push_back(c);
  for (int32_t d : dset) init_counts_dir(current, d, mine, missing);
  std::vector<Task> initial;
  for (int32_t d : dset)
    for (int64_t c : mine)
      if (missing[at(c, d)] == 0) initial.push_back(Task{c, d});
  TaskHeap heap;
  heap.assign(std::move(initial));
  const int64_t total = (int64_t)mine.size() * (int64_t)dset.size();
  const int64_t batch = 10000;
  std::vector<Message> got;
  auto flush = [&] {
    for (int u = 0; u < dom.ranks; ++u) {
      if (ctx.outbox[u].empty()) continue;
      std::lock_guard<std::mutex> g(*dom.lock[u]);
      dom.inbox[u].insert(dom.inbox[u].end(), ctx.outbox[u].begin(), ctx.outbox[u].end());
      ctx.outbox[u].clear();
    }
  };
  auto drain = [&] {
    got.clear();
    {
      std::lock_guard<std::mutex> g(*dom.lock[rank]);
      got.swap(dom.inbox[rank]);
    }
    for (const Message& m : got) deliver(m.cell, m.dir, m.w, m.periodic != 0, current, heap);
    return !got.empty();
  };
  int64_t solved = 0;
  auto idle_since = std::chrono::steady_clock::now();
  while (solved < total && !dom.stalled.load(std::memory_order_relaxed)) {
    if (heap.empty() && !drain()) {
      // a dependency cycle would leave every rank waiting (the reference deadlocks)
      if (std::chrono::steady_clock::now() - idle_since > std::chrono::seconds(120)) dom.stalled = true;
      std::this_thread::yield();
      continue;
    }
    for (int64_t k = 0; k < batch && !heap.empty(); ++k) {
      Task task = heap.pop();
      solve_task(task.cell, (int32_t)task.dir, current, heap, work, &ctx);
      ++solved;
    }
    flush();
    idle_since = std::chrono::steady_clock::now();
  }
  flush();
  dom.done.fetch_add(1);
  while (dom.done.load() < dom.ranks && !dom.stalled.load(std::memory_order_relaxed)) {
    drain();
    std::this_thread::yield();
  }
  drain();
}

int64_t orc_sim::sweep_transport(int32_t current, const std::vector<int32_t>& dset, const std::vector<int64_t>& act) {
  std::vector<WorkCount> work;
  if (p.partition == ORC_PARTITION_DOMAINS && threads() > 1) {
    Domains dom(threads(), n);
    on_threads([&](int t, WorkCount& w) { domain_rank(current, dset, act, dom, t, w); }, work);
  } else {
    on_threads([&](int t, WorkCount& w) { sweep_worker(current, worker_dirs(t, dset), act, w); }, work);
  }
  int64_t solved = 0;
  for (const WorkCount& w : work) solved += w.tasks;
  add_work(work);
  return solved;
}

extern "C" {

orc_sim* orc_sim_create(const orc_params* p, const orc_grid* g, const double* density,
                        const double* xhii, const double* temperature, const double* source) {
  orc_sim* s = new orc_sim(p);
  s->D = p->num_directions;
  s->dirs.assign(p->directions, p->directions + 3 * p->num_directions);
  s->p.directions = s->dirs.data();
  s->n = g->num_cells;
  int64_t E = g->row_ptr[g->num_cells];
  s->row_ptr.assign(g->row_ptr, g->row_ptr + s->n + 1);
  s->nbr.assign(g->nbr, g->nbr + E);
  s->kind.assign(g->kind, g->kind + E);
  s->area.assign(g->area, g->area + E);
  s->normal.assign(g->normal, g->normal + 3 * E);
  s->volume.assign(g->volume, g->volume + s->n);
  s->size.assign(g->size, g->size + s->n);
  s->density.assign(density, density + s->n);
  s->xhii.assign(xhii, xhii + s->n);
  s->temperature.assign(temperature, temperature + s->n);
  s->source.assign(source, source + s->n);
  s->species_timestep.assign(s->n, 0.0);   // HydrogenOnlySpecies::new, hydrogen_only/mod.rs:56-65
  s->change_timescale.assign(s->n, 0.0);   // Site::new, site.rs:26-43
  s->previous_rate.assign(s->n, 0.0);
  size_t nd = (size_t)s->n * (size_t)s->D;
  s->incoming.assign(nd, 0.0);
  s->outgoing.assign(nd, 0.0);
  s->periodic.assign(nd, 0.0);
  s->periodic_pending.assign(nd, 0.0);
  s->missing.assign(nd, 0);
  // Sweep::new: every cell starts at the highest level (mod.rs:206)
  s->level.assign(s->n, (uint8_t)(p->num_timestep_levels - 1));
  return s;
}

void orc_sim_destroy(orc_sim* s) { delete s; }

int orc_sim_step(orc_sim* s, double* time_elapsed) {
  double te = 0.0;
  int st = s->run_sweeps(&te);
  if (time_elapsed) *time_elapsed = te;
  if (s->panicked) st = 2;
  return st;
}

void orc_sim_get_fields(const orc_sim* s, double* xhii, double* temperature, double* timestep,
                        double* rate, double* change_timescale, uint8_t* level) {
  for (int64_t c = 0; c < s->n; ++c) {
    if (xhii) xhii[c] = s->xhii[c];
    if (temperature) temperature[c] = s->temperature[c];
    if (timestep) timestep[c] = s->species_timestep[c];
    if (rate) {  // mod.rs:727-730: sum of incoming over directions
      double r = 0.0;
      for (int32_t d = 0; d < s->D; ++d) r += s->incoming[s->at(c, d)];
      rate[c] = r;
    }
    if (change_timescale) change_timescale[c] = s->change_timescale[c];
    if (level) level[c] = s->level[c];
  }
}

// Time series of the sweep (src/sweep/time_series.rs:61-155) at the current state:
// out[0] mass-averaged and out[1] volume-averaged ionized hydrogen fraction, out[2]
// mass- and out[3] volume-averaged temperature, out[4] volume-averaged
// photoionization rate and out[5] the same weighted by the ionized fraction.  The
// cell mass is density * volume (main.rs:195-203); a cell's photoionization rate is
// Solver::photoionization_rate over one year (chemistry_output.rs:15-28) of the solver
// that get_solver builds (mod.rs:613-631: the rate summed over directions, no floor).
// Each sum runs over the cells in order, as compute_global_sum does on one rank.
void orc_sim_time_series(const orc_sim* s, double* out) {
  const double year = 3.15576e7;  // units/mod.rs: one year in seconds
  double ionized_mass = 0.0, total_mass = 0.0, ionized_volume = 0.0, total_volume = 0.0;
  double mass_weighted_t = 0.0, volume_weighted_t = 0.0, volume_weighted_rate = 0.0, weighted_rate = 0.0;
  for (int64_t c = 0; c < s->n; ++c) {
    const double mass = s->density[c] * s->volume[c];
    double rate = 0.0;
    for (int32_t d = 0; d < s->D; ++d) rate += s->get_rate(c, d);
    Solver sv;
    sv.x = s->xhii[c];
    sv.temperature = s->temperature[c];
    sv.density = s->density[c];
    sv.volume = s->volume[c];
    sv.length = s->size[c];
    sv.rate = rate;
    sv.scale_factor = s->p.scale_factor;
    sv.has_floor = false;
    const double gamma = sv.photoionization_rate(year);
    ionized_mass += mass * s->xhii[c];
    total_mass += mass;
    ionized_volume += s->volume[c] * s->xhii[c];
    total_volume += s->volume[c];
    mass_weighted_t += s->temperature[c] * mass;
    volume_weighted_t += s->temperature[c] * s->volume[c];
    volume_weighted_rate += gamma * s->volume[c];
    weighted_rate += gamma * s->xhii[c] * s->volume[c];
  }
  out[0] = ionized_mass / total_mass;
  out[1] = ionized_volume / total_volume;
  out[2] = mass_weighted_t / total_mass;
  out[3] = volume_weighted_t / total_volume;
  out[4] = volume_weighted_rate / total_volume;
  out[5] = weighted_rate / total_volume;
}

void orc_sim_get_rates(const orc_sim* s, double* incoming, double* outgoing, double* periodic) {
  const std::vector<double>* src[3] = {&s->incoming, &s->outgoing, &s->periodic};
  double* dst[3] = {incoming, outgoing, periodic};
  for (int k = 0; k < 3; ++k) {
    if (!dst[k]) continue;
    for (int64_t c = 0; c < s->n; ++c)
      for (int32_t d = 0; d < s->D; ++d) dst[k][c * s->D + d] = (*src[k])[s->at(c, d)];
  }
}

int64_t orc_sim_init_counts(const orc_sim* s, int32_t level, uint8_t* out) {
  std::vector<uint32_t> tmp((size_t)s->n * s->D, 0);
  const std::vector<int64_t> act = s->active_in_bin_order(level);
  for (int32_t d = 0; d < s->D; ++d) s->init_counts_dir(level, d, act, tmp);
  for (int64_t c = 0; c < s->n; ++c)
    for (int32_t d = 0; d < s->D; ++d) {
      uint32_t v = tmp[s->at(c, d)];
      out[c * s->D + d] = (uint8_t)(v > 255 ? 255 : v);
    }
  return (int64_t)act.size();
}

void orc_sim_level_counts(const orc_sim* s, int64_t* counts) { s->level_counts(counts); }

void orc_sim_work(const orc_sim* s, int64_t* tasks, int64_t* chem_cells) {
  if (tasks) *tasks = s->tasks_solved;
  if (chem_cells) *chem_cells = s->chem_cells;
}

int32_t orc_sim_sweep_order(const orc_sim* s, int32_t* levels_out, int32_t cap) {
  std::vector<int32_t> o = s->ts.sweep_order();
  for (int32_t i = 0; i < (int32_t)o.size() && i < cap; ++i) levels_out[i] = o[i];
  return (int32_t)o.size();
}

int64_t orc_sim_sample_sweep(orc_sim* s, int32_t level, int32_t dir_first, int32_t dir_count, int64_t chem_first,
                             int64_t* chem_cells) {
  if (dir_count < 1 || dir_count > s->D || level < 0 || level >= s->p.num_timestep_levels) return -1;
  std::vector<int32_t> dset;
  for (int32_t k = 0; k < dir_count; ++k) dset.push_back(((dir_first % s->D) + s->D + k) % s->D);
  const std::vector<int64_t> act = s->active_in_bin_order(level);
  const int64_t solved = s->sweep_transport(level, dset, act);
  s->merge_periodic_pending(dset);
  const int64_t before = s->chem_cells;
  s->chemistry(level, act, chem_first, (int64_t)act.size() * dir_count / s->D);
  if (chem_cells) *chem_cells = s->chem_cells - before;
  return solved;
}

int64_t orc_sim_single_sweep(orc_sim* s, int32_t level) {
  int64_t before = s->tasks_solved;
  s->single_sweep(level);
  return s->tasks_solved - before;
}

int32_t orc_timestep_level(int32_t max_num_levels, double max_timestep, double desired) {
  return timestep_level(max_num_levels, max_timestep, desired);
}

int32_t orc_sweep_order_after(int32_t num_levels, int32_t advances, int32_t* out, int32_t cap) {
  TimestepState st(1.0, num_levels);
  for (int32_t i = 0; i < advances; ++i) st.advance();
  std::vector<int32_t> o = st.sweep_order();
  for (int32_t i = 0; i < (int32_t)o.size() && i < cap; ++i) out[i] = o[i];
  return (int32_t)o.size();
}

int32_t orc_lowest_allowed_after(int32_t num_levels, int32_t advances) {
  TimestepState st(1.0, num_levels);
  for (int32_t i = 0; i < advances; ++i) st.advance();
  return st.lowest;
}

double orc_rate_fit(int32_t which, double temperature, double scale_factor) {
  Solver s{};
  s.temperature = temperature;
  s.scale_factor = scale_factor;
  switch (which) {
    case 0: return s.case_b_recombination_rate();
    case 1: return s.case_b_recombination_rate_derivative();
    case 2: return s.collisional_ionization_rate();
    case 3: return s.collisional_ionization_rate_derivative();
    case 4: return s.collisional_ionization_cooling_rate();
    case 5: return s.collisional_ionization_cooling_rate_derivative();
    case 6: return s.collisional_excitation_cooling_rate();
    case 7: return s.collisional_excitation_cooling_rate_derivative();
    case 8: return s.case_b_recombination_cooling_rate();
    case 9: return s.case_b_recombination_cooling_rate_derivative();
    case 10: return s.bremsstrahlung_cooling_rate();
    case 11: return s.bremsstrahlung_cooling_rate_derivative();
    case 12: return s.compton_cooling_rate();
    case 13: return s.compton_cooling_rate_derivative();
    default: return NAN;
  }
}

int32_t orc_solver_perform_timestep(double* xhii, double* temperature, double density,
                                    double volume, double length, double rate,
                                    double scale_factor, int32_t has_floor, double floor_t,
                                    double floor_x, double timestep, double safety,
                                    double* timescale_out, int32_t* process_out) {
  Solver s{};
  s.x = *xhii;
  s.temperature = *temperature;
  s.density = density;
  s.volume = volume;
  s.length = length;
  s.rate = rate;
  s.scale_factor = scale_factor;
  s.has_floor = has_floor != 0;
  s.floor_t = floor_t;
  s.floor_x = floor_x;
  bool failed = false;
  int64_t attempts = 0;
  Timescale t = s.perform_timestep(timestep, safety, &failed, attempts);
  *xhii = s.x;
  *temperature = s.temperature;
  if (timescale_out) *timescale_out = t.time;
  if (process_out) *process_out = t.process;
  return failed ? 1 : 0;
}

int32_t orc_directions_from_num(int32_t num, double* out) {
  static const double one[1][3] = {{1.0, 0.0, 0.0}};
  const double(*tab)[3] = nullptr;
  switch (num) {  // Directions::from_num, src/sweep/direction/mod.rs:58-75
    case 1: tab = one; break;
    case 16: tab = kDirectionBins16; break;
    case 21: tab = kDirectionBins21; break;
    case 32: tab = kDirectionBins32; break;
    case 64: tab = kDirectionBins64; break;
    case 84: tab = kDirectionBins84; break;
    default: return -1;
  }
  for (int32_t i = 0; i < 3 * num; ++i) out[i] = tab[0][i];
  return 0;
}

int64_t orc_heap_replay(const int64_t* init_dirs, int64_t n_init, const int64_t* ops, int64_t n_ops,
                        int64_t* out) {
  std::vector<Task> v;
  for (int64_t i = 0; i < n_init; ++i) v.push_back(Task{i, init_dirs[i]});
  TaskHeap heap;
  heap.assign(std::move(v));
  int64_t next = n_init, written = 0;
  for (int64_t k = 0; k < n_ops; ++k) {
    if (ops[k] >= 0) {
      heap.push(Task{next++, ops[k]});
    } else {
      if (heap.empty()) return -1;
      out[written++] = heap.pop().cell;
    }
  }
  return written;
}

double orc_outgoing_rate(double density, double xhii, double size, double incoming_rate,
                         double threshold) {
  double nhn = density / PROTON_MASS * (1.0 - xhii);
  if (incoming_rate < threshold) return 0.0;
  return incoming_rate * std::exp(-nhn * SIGMA * size);
}

}  // extern "C"
