// Device side of the sweep: dependency counting, the persistent dependency-driven
// transport kernel, periodic-source folding, chemistry and level reassignment.
//
// Layout in HBM (all per-(cell, direction) arrays are [cell][dir] with a padded
// direction stride Dp = round_up(D, 8), so one cell's directions are contiguous and
// a warp working on 32 directions of one cell touches consecutive addresses):
//   faces:   geo64[E] = {nx, ny, nz, area} (Geo64), geo32[E] = same in float4 with the
//            area scaled by a power of two (the FP32 path only uses area ratios),
//            nbr[E] = neighbour index | kind << 30
//   cells:   level (u8), density, x_HII, (1 - x_HII), T, source, volume, size,
//            attenuation factor, previous rate, change timescale, species timestep
//   tasks:   incoming / outgoing / periodic / periodic_pending rates (R = double in
//            the FP64 drop-in, float in the mixed path), dependency counters (u8,
//            packed 4 per u32 word), ready-direction masks (4 x u32 per cell) and a
//            queued flag per cell.
//
// Transport (Sweep::single_sweep, src/sweep/mod.rs:274-289) runs as one persistent
// cooperative kernel.  A cell is a unit of work: when a producer's decrement brings
// a dependency counter (cell n, dir d) to zero it sets bit d in n's ready mask and,
// if n is not queued yet, appends n to the next round's frontier.  A warp that takes
// n from the frontier grabs all of n's ready bits at once and solves those
// directions together (lanes = directions), with n's faces staged in shared memory.
// Rounds are separated by a grid barrier; all cross-warp data (incoming rates,
// counters, masks) is exchanged through device-scope atomics before the barrier.
// The sweep ends when a round produces no new work; the number of solved tasks is
// then compared with the active (cell, dir) count to detect dependency cycles.
#pragma once

#include <cstdint>

#include "chemistry_device.cuh"
#include "sweep_types.h"

namespace swk {

template <typename R>
struct SweepArgs {
  // geometry
  const long long* row_ptr;
  const Geo64* geo64;
  const float4* geo32;
  const uint32_t* nbr;
  const double* size;
  // directions (D x 3, padded to Dp rows) in both precisions
  const double* dir64;
  const float* dir32;
  int D, Dp, words;      // words = ceil(D / 32)
  float guard;           // |dot32| above this has the sign of the FP64 dot
  // cell state
  const uint8_t* level;
  const uint32_t* order;   // cells sorted by level, highest first
  const double* source;
  const double* att;       // per-cell attenuation factor exp(-n_HI sigma size)
  double rate_scale;       // photons/s per unit of R (1 in FP64)
  R threshold;             // significant_rate_threshold / rate_scale
  // per-(cell, dir) state
  R* incoming;
  R* outgoing;
  R* periodic;
  R* pending;
  uint32_t* counters;      // Dp/4 words per cell
  uint32_t* ready;         // kMaxDirWords words per cell
  uint32_t* queued;        // round stamp: (round the cell is queued for) + 1
  uint32_t* frontier0;
  uint32_t* frontier1;
  SweepCtl* ctl;
  int current_level;
  unsigned long long timeout_ns;
  uint32_t max_rounds;
};

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint32_t ld_volatile(const uint32_t* p) {
  return *reinterpret_cast<const volatile uint32_t*>(p);
}

template <typename R>
__device__ __forceinline__ R ld_cg(const R* p) {
  return __ldcg(p);
}

// Exact classification of a face against a direction: returns the FP64 dot
// (n.x*d.x + n.y*d.y) + n.z*d.z, whose sign the reference tests with strict < 0 and
// > 0 (grid/cell.rs:125-132).  The FP32 dot decides whenever it is farther from zero
// than its rounding error bound; only near-perpendicular faces pay for FP64.
__device__ __forceinline__ double dot64(const Geo64& g, double dx, double dy, double dz) {
  return g.x * dx + g.y * dy + g.z * dz;
}

__device__ __forceinline__ int face_sign(const float4& g32, const Geo64& g64, float dx32, float dy32,
                                         float dz32, double dx, double dy, double dz, float guard) {
  float d = g32.x * dx32 + g32.y * dy32 + g32.z * dz32;
  if (d > guard) return 1;
  if (d < -guard) return -1;
  double e = dot64(g64, dx, dy, dz);
  return (e > 0.0) - (e < 0.0);
}

// Bounded grid barrier for the cooperative kernel.  Returns false if the kernel must
// stop (a wait ran out, or another block flagged an error).
__device__ __forceinline__ bool grid_barrier(SweepCtl* ctl, uint32_t& gen, unsigned long long deadline_ns) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    __threadfence();
    uint32_t arrived = atomicAdd(&ctl->bar_count, 1u);
    if (arrived == gridDim.x - 1) {
      atomicExch(&ctl->bar_count, 0u);
      __threadfence();
      atomicAdd(&ctl->bar_gen, 1u);
    } else {
      unsigned long long t0 = globaltimer_ns();
      while (ld_volatile(&ctl->bar_gen) == gen) {
        if (ld_volatile(&ctl->error) != 0) { ok = 0; break; }
        if (globaltimer_ns() - t0 > deadline_ns) {
          atomicOr(&ctl->error, kErrStall);
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    gen += 1;
    if (ld_volatile(&ctl->error) != 0) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Per-warp shared-memory stage of one cell's faces.
struct FaceStage {
  Geo64 g64[kMaxFaces];
  float4 g32[kMaxFaces];
  uint32_t nbr[kMaxFaces];
  uint8_t active[kMaxFaces];  // LOCAL neighbour that is active in this sweep
};

__device__ __forceinline__ int stage_faces(FaceStage& st, long long beg, int nf, const Geo64* geo64,
                                           const float4* geo32, const uint32_t* nbr, const uint8_t* level,
                                           int current, int lane) {
  __syncwarp();  // the previous cell's stage may still be read by other lanes
  for (int f = lane; f < nf; f += 32) {
    st.g64[f] = geo64[beg + f];
    st.g32[f] = geo32[beg + f];
    uint32_t nb = nbr[beg + f];
    st.nbr[f] = nb;
    uint32_t kind = nb >> kKindShift;
    st.active[f] = (kind == kKindLocal) && (level[nb & kNbrMask] >= current);
  }
  __syncwarp();
  return nf;
}

// ---------------------------------------------------------------------------
// Sweep::init_counts (src/sweep/mod.rs:346-386): for every active cell and direction,
// the number of upwind faces whose neighbour is LOCAL and active.  Cells with ready
// directions seed the first frontier.
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
k_init_counts(SweepArgs<R> a, uint8_t* debug_counts) {
  __shared__ FaceStage stage[kWarpsPerBlock];
  const uint32_t n_active = a.ctl->n_ge[a.current_level];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  FaceStage& st = stage[wib];
  const uint32_t nwarps = gridDim.x * kWarpsPerBlock;
  for (uint32_t i = blockIdx.x * kWarpsPerBlock + wib; i < n_active; i += nwarps) {
    uint32_t c = a.order[i];
    long long beg = a.row_ptr[c];
    int nf = (int)(a.row_ptr[c + 1] - beg);
    stage_faces(st, beg, nf, a.geo64, a.geo32, a.nbr, a.level, a.current_level, lane);
    uint32_t any_ready = 0;
    for (int k = 0; k < a.words; ++k) {
      int d = 32 * k + lane;
      bool valid = d < a.D;
      double dx = 0, dy = 0, dz = 0;
      float fx = 0, fy = 0, fz = 0;
      if (valid) {
        dx = a.dir64[3 * d]; dy = a.dir64[3 * d + 1]; dz = a.dir64[3 * d + 2];
        fx = a.dir32[3 * d]; fy = a.dir32[3 * d + 1]; fz = a.dir32[3 * d + 2];
      }
      uint32_t cnt = 0;
      if (valid)
        for (int f = 0; f < nf; ++f)
          if (st.active[f] && face_sign(st.g32[f], st.g64[f], fx, fy, fz, dx, dy, dz, a.guard) < 0) ++cnt;
      // pack 4 counters per word: lanes 4j..4j+3 -> word 8k + j
      uint32_t byte = valid ? cnt : 0u;
      uint32_t w = byte << (8 * (lane & 3));
      w |= __shfl_xor_sync(0xffffffffu, w, 1);
      w |= __shfl_xor_sync(0xffffffffu, w, 2);
      if ((lane & 3) == 0 && 32 * k + lane < a.Dp)
        a.counters[(size_t)c * (a.Dp / 4) + 8 * k + (lane >> 2)] = w;
      if (debug_counts && valid) debug_counts[(size_t)c * a.D + d] = (uint8_t)cnt;
      uint32_t rb = __ballot_sync(0xffffffffu, valid && cnt == 0);
      if (lane == 0) a.ready[(size_t)c * kMaxDirWords + k] = rb;
      any_ready |= rb;
    }
    if (lane == 0) {
      for (int k = a.words; k < kMaxDirWords; ++k) a.ready[(size_t)c * kMaxDirWords + k] = 0u;
      a.queued[c] = any_ready ? 1u : 0u;  // queued for round 0
      if (any_ready) {
        uint32_t slot = atomicAdd(&a.ctl->count[0], 1u);
        a.frontier0[slot] = c;
      }
    }
    __syncwarp();
  }
}

// Solve all ready directions of one cell (Sweep::solve_task, src/sweep/mod.rs:423-485,
// with get_outgoing_rate 412-421, handle_local_neighbour 487-503 and
// handle_local_periodic_neighbour 505-513).  Returns the number of tasks solved.
template <typename R>
__device__ __forceinline__ uint32_t process_cell(const SweepArgs<R>& a, FaceStage& st, uint32_t c,
                                                 const uint32_t* masks, uint32_t* next_frontier,
                                                 uint32_t* next_count, uint32_t stamp, int lane) {
  long long beg = a.row_ptr[c];
  int nf = (int)(a.row_ptr[c + 1] - beg);
  stage_faces(st, beg, nf, a.geo64, a.geo32, a.nbr, a.level, a.current_level, lane);
  const double att = a.att[c];
  const double src_per_dir = a.source[c] / (double)a.D;  // site.rs:49-51
  const size_t row = (size_t)c * a.Dp;
  uint32_t solved = 0;
  for (int k = 0; k < a.words; ++k) {
    const uint32_t m = masks[k];
    if (m == 0) continue;
    solved += __popc(m);
    const int d = 32 * k + lane;
    const bool act = (m >> lane) & 1u;
    double dx = 0, dy = 0, dz = 0;
    float fx = 0, fy = 0, fz = 0;
    if (act) {
      dx = a.dir64[3 * d]; dy = a.dir64[3 * d + 1]; dz = a.dir64[3 * d + 2];
      fx = a.dir32[3 * d]; fy = a.dir32[3 * d + 1]; fz = a.dir32[3 * d + 2];
    }
    // outgoing rate and its correction
    R corr = R(0);
    if (act) {
      R inc = ld_cg(a.incoming + row + d);
      if (inc < R(0)) {  // Photons::make_positive (chemistry/mod.rs:61-65)
        inc = R(0);
        a.incoming[row + d] = inc;
      }
      R r = (inc + R(src_per_dir / a.rate_scale)) + ld_cg(a.periodic + row + d);
      R out_new = (r < a.threshold) ? R(0) : r * R(att);
      corr = out_new - a.outgoing[row + d];
      a.outgoing[row + d] = out_new;
    }
    // total effective downwind area, summed in face order
    R total = R(0);
    uint64_t down = 0;
    if (act) {
      for (int f = 0; f < nf; ++f) {
        if (face_sign(st.g32[f], st.g64[f], fx, fy, fz, dx, dy, dz, a.guard) > 0) {
          down |= 1ull << f;
          if (sizeof(R) == 8) {
            total += R(st.g64[f].w * dot64(st.g64[f], dx, dy, dz));
          } else {
            total += R(st.g32[f].w * (st.g32[f].x * fx + st.g32[f].y * fy + st.g32[f].z * fz));
          }
        }
      }
    }
    // distribute to downwind neighbours; the face loop is warp-uniform so that the
    // lanes of one face hit consecutive directions of the same neighbour row.
    for (int f = 0; f < nf; ++f) {
      const bool dn = (down >> f) & 1ull;
      if (!__any_sync(0xffffffffu, dn)) continue;
      const uint32_t nb = st.nbr[f];
      const uint32_t kind = nb >> kKindShift;
      if (kind == kKindBoundary) continue;
      const uint32_t n = nb & kNbrMask;
      R w = R(0);
      if (dn) {
        R eff;
        if (sizeof(R) == 8) {
          eff = R(st.g64[f].w * dot64(st.g64[f], dx, dy, dz));
        } else {
          eff = R(st.g32[f].w * (st.g32[f].x * fx + st.g32[f].y * fy + st.g32[f].z * fz));
        }
        w = corr * (eff / total);
      }
      const size_t nrow = (size_t)n * a.Dp;
      if (kind == kKindPeriodic) {
        if (dn) atomicAdd(a.pending + nrow + d, w);
        continue;
      }
      if (dn) atomicAdd(a.incoming + nrow + d, w);
      if (!st.active[f]) continue;
      // dependency counters, 4 per word: combine the lanes of one word into one atomic
      uint32_t dec = dn ? (1u << (8 * (lane & 3))) : 0u;
      dec += __shfl_xor_sync(0xffffffffu, dec, 1);
      dec += __shfl_xor_sync(0xffffffffu, dec, 2);
      uint32_t old = 0;
      if ((lane & 3) == 0 && dec != 0u)
        old = atomicSub(a.counters + (size_t)n * (a.Dp / 4) + 8 * k + (lane >> 2), dec);
      old = __shfl_sync(0xffffffffu, old, lane & ~3);
      const bool became_ready = dn && (((old >> (8 * (lane & 3))) & 0xffu) == 1u);
      const uint32_t rb = __ballot_sync(0xffffffffu, became_ready);
      if (rb != 0u && lane == __ffs(rb) - 1) {
        // queued[n] holds (round for which n is queued) + 1; the first producer of
        // this round to raise it appends n, so a cell enters a frontier at most once.
        atomicOr(a.ready + (size_t)n * kMaxDirWords + k, rb);
        if (atomicMax(a.queued + n, stamp) < stamp) {
          uint32_t slot = atomicAdd(next_count, 1u);
          next_frontier[slot] = n;
        }
      }
    }
  }
  return solved;
}

// The persistent transport kernel (cooperative launch).  Round r takes the cells of
// frontier[r & 1] (count[r % 3]) and appends newly ready cells to frontier[(r+1) & 1]
// (count[(r+1) % 3]); count[(r+2) % 3] is cleared during round r for round r+1.
template <typename R>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
k_sweep(SweepArgs<R> a) {
  __shared__ FaceStage stage[kWarpsPerBlock];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  FaceStage& st = stage[wib];
  const uint32_t gwarp = blockIdx.x * kWarpsPerBlock + wib;
  const uint32_t nwarps = gridDim.x * kWarpsPerBlock;
  uint32_t gen = ld_volatile(&a.ctl->bar_gen);
  unsigned long long solved = 0, visits = 0;
  uint32_t round = 0;
  for (;; ++round) {
    if (round >= a.max_rounds) {
      if (threadIdx.x == 0 && blockIdx.x == 0) atomicOr(&a.ctl->error, kErrRounds);
      break;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) a.ctl->count[(round + 2) % 3] = 0u;
    const uint32_t cnt = ld_volatile(&a.ctl->count[round % 3]);
    const uint32_t* cur = (round & 1) ? a.frontier1 : a.frontier0;
    uint32_t* nxt = (round & 1) ? a.frontier0 : a.frontier1;
    uint32_t* nxt_count = &a.ctl->count[(round + 1) % 3];
    // cells queued during this round for the next one carry stamp round + 2
    const uint32_t stamp = round + 2;
    for (uint32_t i = gwarp; i < cnt; i += nwarps) {
      const uint32_t c = __ldcg(cur + i);
      uint32_t m = 0;
      if (lane < a.words) m = atomicExch(a.ready + (size_t)c * kMaxDirWords + lane, 0u);
      uint32_t masks[kMaxDirWords];
#pragma unroll
      for (int k = 0; k < kMaxDirWords; ++k) masks[k] = __shfl_sync(0xffffffffu, m, k);
      ++visits;
      solved += process_cell<R>(a, st, c, masks, nxt, nxt_count, stamp, lane);
    }
    if (!grid_barrier(a.ctl, gen, a.timeout_ns)) break;
    if (ld_volatile(&a.ctl->count[(round + 1) % 3]) == 0u) break;
  }
  if (lane == 0) {
    atomicAdd(&a.ctl->tasks, solved);
    atomicAdd(&a.ctl->visits, visits);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) a.ctl->rounds = round + 1;
}

// Snapshot semantics of periodic sources: contributions written through periodic
// faces during a level sweep are added to periodic_source after the transport, so
// transport reads the previous sweeps' contributions and the chemistry all of them.
template <typename R>
__global__ void k_fold_periodic(R* periodic, R* pending, const uint32_t* cells, uint32_t n_cells, int Dp) {
  size_t total = (size_t)n_cells * Dp;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    size_t c = cells[i / Dp];
    size_t idx = c * Dp + (i % Dp);
    R p = pending[idx];
    if (p != R(0)) {
      periodic[idx] += p;
      pending[idx] = R(0);
    }
  }
}

// Per-cell attenuation factor exp(-n_HI sigma size) of HydrogenOnly::get_outgoing_rate
// (hydrogen_only/mod.rs:72-88); direction-independent, so computed once per cell.
template <bool kCarryNeutral>
__global__ void k_attenuation(const uint32_t* order, const SweepCtl* ctl, int current_level,
                              const double* density, const double* xhii, const double* yneu,
                              const double* size, double* att) {
  uint32_t n_active = ctl->n_ge[current_level];
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_active; i += gridDim.x * blockDim.x) {
    uint32_t c = order[i];
    double neutral = kCarryNeutral ? yneu[c] : (1.0 - xhii[c]);
    double nhn = density[c] / Units::kProtonMass * neutral;
    att[c] = exp(-nhn * Units::kSigma * size[c]);
  }
}

template <typename R>
struct ChemArgs {
  const uint32_t* order;
  SweepCtl* ctl;
  int current_level;
  int D, Dp;
  const R* incoming;
  const R* periodic;
  double rate_scale;
  const double* source;
  const double* density;
  const double* volume;
  const double* size;
  const uint8_t* level;
  double* xhii;
  double* yneu;
  double* temperature;
  double* previous_rate;
  double* change_timescale;
  double* species_timestep;
  double max_timestep;
  double threshold;
  double safety;
  double scale_factor;
  int prevent_cooling;
};

// Sweep::update_chemistry (src/sweep/mod.rs:549-574) + HydrogenOnly::update_abundances
// (hydrogen_only/mod.rs:90-119), one thread per active cell.
template <typename R, bool kCarryNeutral>
__global__ void k_chemistry(ChemArgs<R> a) {
  uint32_t n_active = a.ctl->n_ge[a.current_level];
  uint32_t attempts = 0, failures = 0, cells = 0, invalid = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_active; i += gridDim.x * blockDim.x) {
    const uint32_t c = a.order[i];
    const double timestep = ldexp(a.max_timestep, -(int)a.level[c]);  // timestep_level.rs:42-48
    const double src = a.source[c] / (double)a.D;
    const size_t row = (size_t)c * a.Dp;
    double rate;
    if (sizeof(R) == 8) {
      rate = 0.0;  // sum over directions of Site::get_rate, in direction order
      for (int d = 0; d < a.D; ++d) rate += ((double)a.incoming[row + d] + src) + (double)a.periodic[row + d];
    } else {
      // compensated FP32 sum of the scaled rates, then the source in FP64
      float s = 0.f, comp = 0.f;
      for (int d = 0; d < a.D; ++d) {
        float v = (float)a.incoming[row + d] + (float)a.periodic[row + d];
        float yv = v - comp;
        float t = s + yv;
        comp = (t - s) - yv;
        s = t;
      }
      rate = (double)s * a.rate_scale + a.source[c];
    }
    double relative_change;
    if (fabs(rate) < fabs(a.threshold)) {  // chemistry/mod.rs:79-81
      relative_change = 0.0;
    } else {  // chemistry/mod.rs:73-77
      relative_change = fabs(fmin(fabs(fabs(rate - a.previous_rate[c]) / rate), 1.0 / DBL_EPSILON));
    }
    a.previous_rate[c] = rate;
    Timescale rate_ts{timestep / relative_change, kProcPhotonRate};
    ChemSolver<kCarryNeutral> s;
    s.x = a.xhii[c];
    s.y = kCarryNeutral ? a.yneu[c] : 0.0;
    s.temperature = a.temperature[c];
    s.density = a.density[c];
    s.volume = a.volume[c];
    s.length = a.size[c];
    s.rate = rate;
    s.scale_factor = a.scale_factor;
    s.has_floor = a.prevent_cooling != 0;
    s.floor_t = s.temperature;
    s.floor_x = s.x;
    s.clamp_invalid = false;
    bool failed = false;
    Timescale chem_ts = s.perform_timestep(timestep, a.safety, failed, attempts);
    failures += failed ? 1u : 0u;
    invalid |= s.clamp_invalid ? 1u : 0u;
    a.temperature[c] = s.temperature;
    a.xhii[c] = s.x;
    if (kCarryNeutral) a.yneu[c] = s.y;
    a.species_timestep[c] = chem_ts.time;
    a.change_timescale[c] = ts_min(rate_ts, chem_ts).time;
    ++cells;
  }
  // warp-aggregated counters
  for (int o = 16; o > 0; o >>= 1) {
    attempts += __shfl_xor_sync(0xffffffffu, attempts, o);
    failures += __shfl_xor_sync(0xffffffffu, failures, o);
    cells += __shfl_xor_sync(0xffffffffu, cells, o);
    invalid |= __shfl_xor_sync(0xffffffffu, invalid, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (attempts) atomicAdd(&a.ctl->chem_attempts, (unsigned long long)attempts);
    if (failures) atomicAdd(&a.ctl->chem_failures, (unsigned long long)failures);
    if (cells) atomicAdd(&a.ctl->chem_cells, (unsigned long long)cells);
    if (invalid) atomicOr(&a.ctl->error, kErrClamp);
  }
}

// TimestepLevel::from_max_timestep_and_desired_timestep (timestep_level.rs:27-36)
// with Rust's saturating float->usize cast, floored at the lowest allowed level
// (TimestepState::get_desired_level_from_desired_timestep, timestep_state.rs:54-64).
// ceil(log2(r)) is taken exactly from the binary exponent: r = m * 2^e with m in
// [0.5, 1) gives e - 1 when m == 0.5 (r a power of two) and e otherwise.
__device__ __forceinline__ int desired_level(double max_timestep, double desired, int num_levels, int lowest) {
  double ratio = max_timestep / desired;
  long long level;
  if (isnan(ratio) || ratio <= 1.0) {
    level = 0;  // log2 <= 0, NaN -> 0
  } else if (isinf(ratio)) {
    level = num_levels - 1;
  } else {
    int e;
    double m = frexp(ratio, &e);
    level = (m == 0.5) ? (e - 1) : e;
  }
  if (level > num_levels - 1) level = num_levels - 1;
  if (level < lowest) level = lowest;
  return (int)level;
}

// Sweep::update_timestep_levels (src/sweep/mod.rs:576-589) for all cells, plus the
// level histogram used to rebuild the active ordering.
static __global__ void k_update_levels(uint32_t n, const double* change_timescale, uint8_t* level, double safety,
                                double max_timestep, int num_levels, int lowest, SweepCtl* ctl) {
  __shared__ uint32_t hist[32];
  if (threadIdx.x < 32) hist[threadIdx.x] = 0;
  __syncthreads();
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    int l = desired_level(max_timestep, safety * change_timescale[c], num_levels, lowest);
    level[c] = (uint8_t)l;
    atomicAdd(&hist[l], 1u);
  }
  __syncthreads();
  if (threadIdx.x < num_levels && hist[threadIdx.x]) atomicAdd(&ctl->hist[threadIdx.x], hist[threadIdx.x]);
}

// Histogram of the current levels (used at creation and after sw_set_fields).
static __global__ void k_level_hist(uint32_t n, const uint8_t* level, int num_levels, SweepCtl* ctl) {
  __shared__ uint32_t hist[32];
  if (threadIdx.x < 32) hist[threadIdx.x] = 0;
  __syncthreads();
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x)
    atomicAdd(&hist[level[c]], 1u);
  __syncthreads();
  if (threadIdx.x < num_levels && hist[threadIdx.x]) atomicAdd(&ctl->hist[threadIdx.x], hist[threadIdx.x]);
}

// n_ge[l] = #cells with level >= l; fill[l] = start of level l in the order (highest first).
static __global__ void k_level_offsets(SweepCtl* ctl, int num_levels) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    uint32_t acc = 0;
    for (int l = num_levels - 1; l >= 0; --l) {
      ctl->fill[l] = acc;
      acc += ctl->hist[l];
      ctl->n_ge[l] = acc;
    }
    for (int l = 0; l < 32; ++l) ctl->hist[l] = 0;
  }
}

// Scatter cells into the level ordering (cells of the highest level first).
static __global__ void k_level_scatter(uint32_t n, const uint8_t* level, SweepCtl* ctl, uint32_t* order) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    uint32_t slot = atomicAdd(&ctl->fill[level[c]], 1u);
    order[slot] = c;
  }
}

// IonizationTime write-back of run_sweep_system (src/sweep/mod.rs:731-738).
static __global__ void k_ionization_time(uint32_t n, const double* xhii, double* ionization_time, double time) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x)
    if (xhii[c] > 0.5 && isinf(ionization_time[c])) ionization_time[c] = time;
}

// PhotonRate = sum over directions of the incoming rate (src/sweep/mod.rs:727-730).
template <typename R>
__global__ void k_photon_rate(uint32_t n, const R* incoming, int D, int Dp, double rate_scale, double* out) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    double r = 0.0;
    const size_t row = (size_t)c * Dp;
    for (int d = 0; d < D; ++d) r += (double)incoming[row + d];
    out[c] = r * rate_scale;
  }
}

// Convert a per-(cell, dir) array to FP64 photons/s in [cell][D] layout.
template <typename R>
__global__ void k_export_rates(uint32_t n, const R* src, int D, int Dp, double rate_scale, double* out) {
  size_t total = (size_t)n * D;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    size_t c = i / D, d = i % D;
    out[i] = (double)src[c * Dp + d] * rate_scale;
  }
}

}  // namespace swk
