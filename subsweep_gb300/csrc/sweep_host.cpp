// Host runtime of the GB300 sweep library and its C ABI (include/subsweep_gpu.h).
//
// Mirrors the reference's Sweep<HydrogenOnly> driver (src/sweep/mod.rs:171-610): the
// sweep parameters, the hierarchical timestep state and the per-step sequence of
// level sweeps live here on the host; every per-cell and per-(cell, direction)
// computation runs in the kernels of sweep_fp64.cu / sweep_mixed.cu.  There is no
// CPU fallback: every entry point fails with SW_ERR_CUDA when no device is usable.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/subsweep_gpu.h"
#include "host_checks.h"
#include "launch.h"
#include "sweep_types.h"

#include "direction_bins.inc"

namespace {

thread_local std::string g_create_error;

// TimestepState, src/sweep/timestep_state.rs:5-90.
struct TimestepState {
  double max_timestep = 0.0;
  int max_num_levels = 1;
  int lowest = 0;
  bool first_done = false;

  void init(double m, int n) {
    max_timestep = m;
    max_num_levels = n;
    lowest = n - 1;
    first_done = false;
  }
  // iter_levels_in_sweep_order (22-27) with lowest_active_from_iteration (70-75)
  std::vector<int> sweep_order() const {
    int num = max_num_levels - lowest;
    std::vector<int> out;
    for (uint32_t i = 0; i < (1u << (num - 1)); ++i) {
      int first_bit = (i == 0) ? (num - 1) : __builtin_ctz(i);
      out.push_back(lowest + (num - 1 - first_bit));
    }
    return out;
  }
  // advance_allowed_levels (37-48)
  void advance() {
    if (first_done && lowest > 0) lowest -= 1;
    if (!first_done) first_done = true;
  }
  // current_max_timestep (77-79): max_timestep * 0.5^lowest
  double current_max_timestep() const { return std::ldexp(max_timestep, -lowest); }
};

template <typename T>
cudaError_t dalloc(T** p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  return cudaMalloc((void**)p, count * sizeof(T));
}

}  // namespace

int32_t sw_host_sweep_order(int32_t num_levels, int32_t advances, int32_t* out, int32_t cap) {
  if (num_levels < 1 || num_levels > 16 || advances < 0 || cap < 0 || (cap > 0 && !out)) return -1;
  TimestepState ts;
  ts.init(1.0, num_levels);
  for (int32_t i = 0; i < advances; ++i) ts.advance();
  const std::vector<int> order = ts.sweep_order();
  for (size_t i = 0; i < order.size() && (int32_t)i < cap; ++i) out[i] = order[i];
  return (int32_t)order.size();
}

int32_t sw_host_lowest_allowed(int32_t num_levels, int32_t advances) {
  if (num_levels < 1 || num_levels > 16 || advances < 0) return -1;
  TimestepState ts;
  ts.init(1.0, num_levels);
  for (int32_t i = 0; i < advances; ++i) ts.advance();
  return ts.lowest;
}

struct sw_handle {
  sw_params params{};
  const swh::PrecisionOps* ops = nullptr;
  std::vector<double> dirs;
  int D = 0, L = 1;
  uint32_t Np = 0;
  int64_t N = 0, E = 0;
  TimestepState ts;
  double sim_time = 0.0;
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[8] = {};
  swh::DevicePtrs p{};
  std::vector<void*> allocations;
  std::vector<uint32_t> n_ge_host;  // cells with level >= l at the start of the next step
  swk::SweepCtl ctl_host{};
  sw_stats stats{};
  std::string last_error;
  double* scratch = nullptr;  // N doubles for field export
  uint32_t stats_schedule_levels = 0;
  // fingerprint of the levelled schedule (direction groups and segment offsets): the pull
  // path's checkpointed words are indexed by schedule position
  uint64_t schedule_hash = 0;
  int64_t device_bytes = 0;  // device memory held by the handle (its allocations)
  int64_t stats_upwind_slots = 0;
  int force_path = 0;  // 0 automatic, 1 always levelled, 2 always dependency-driven
  bool trace = false;  // SUBSWEEP_TRACE: one stderr line per level sweep
  uint32_t act_valid = 0;  // pull path: levels whose compacted list is current this step
  double* series_dev = nullptr;  // time-series partial sums and result (allocated on first use)
  // graph replay of a step (pull path): the instantiated graph, the step shape it was
  // captured for, and the pinned scalars its first node copies to the control block
  bool graph_mode = false;
  cudaGraphExec_t graph_exec = nullptr;
  std::vector<int64_t> graph_key;
  struct GraphScalars {
    uint32_t epoch_base, pad;
    double time;
  }* graph_scalars = nullptr;
  int64_t graph_captures = 0;
  int64_t graph_kernels = 0;  // kernel launches in the captured step
  // autotuning of the pull transport kernel: trials of ops->tune_variants, one per sweep
  bool autotune = false;
  bool tuned = false;
  int tune_index = 0;
  std::vector<double> tune_ns;  // ns per task of each candidate
  std::vector<cudaEvent_t> graph_ev;  // start / end of each sweep's transport inside the graph
  uint32_t last_epoch = 0;  // pull path: sweep number of the last sweep of the last step

  ~sw_handle() {
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    for (cudaEvent_t e : graph_ev) cudaEventDestroy(e);
    if (graph_scalars) cudaFreeHost(graph_scalars);
    for (void* a : allocations) cudaFree(a);
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
    if (stream) cudaStreamDestroy(stream);
  }

  template <typename T>
  bool alloc(T** ptr, size_t count) {
    cudaError_t e = dalloc(ptr, count);
    if (e != cudaSuccess) return false;
    allocations.push_back((void*)*ptr);
    device_bytes += (int64_t)(count * sizeof(T));
    return true;
  }

  sw_status fail(sw_status st, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    last_error = buf;
    return st;
  }
  sw_status cuda_fail(cudaError_t e, const char* where) {
    return fail(e == cudaErrorMemoryAllocation ? SW_ERR_OOM : SW_ERR_CUDA, "%s: %s", where,
                cudaGetErrorString(e));
  }
};

namespace {

#define SW_CUDA(h, call, where)                   \
  do {                                            \
    cudaError_t _e = (call);                      \
    if (_e != cudaSuccess) return (h)->cuda_fail(_e, where); \
  } while (0)

// The handle's device is current until the entry point returns; the caller's device
// is current again afterwards.
#define SW_DEVICE_SCOPE(h)                                    \
  swh::DeviceScope _device_scope((h)->device);                \
  if (_device_scope.status != cudaSuccess) return (h)->cuda_fail(_device_scope.status, "select device")

sw_status create_fail(sw_status st, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_create_error = buf;
  return st;
}

bool directions_for(int num, std::vector<double>& out) {
  const double(*tab)[3] = nullptr;
  static const double one[1][3] = {{1.0, 0.0, 0.0}};
  switch (num) {  // Directions::from_num, src/sweep/direction/mod.rs:58-75
    case 1: tab = one; break;
    case 16: tab = kDirectionBins16; break;
    case 21: tab = kDirectionBins21; break;
    case 32: tab = kDirectionBins32; break;
    case 64: tab = kDirectionBins64; break;
    case 84: tab = kDirectionBins84; break;
    default: return false;
  }
  out.assign(&tab[0][0], &tab[0][0] + 3 * num);
  return true;
}

// Each LOCAL / LOCAL_PERIODIC face c -> n needs a face n -> c with the bitwise negated
// normal: the reference counts upwind faces from c's side and delivers fluxes from
// n's side, so without it a level sweep could never finish.
bool check_reciprocal_faces(const sw_grid_csr* g, std::string& why) {
  std::atomic<int64_t> bad{-1};
  int nt = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  std::vector<std::thread> th;
  for (int t = 0; t < nt; ++t)
    th.emplace_back([&, t]() {
      for (int64_t c = t; c < g->num_cells; c += nt) {
        if (bad.load(std::memory_order_relaxed) >= 0) return;
        for (int64_t f = g->row_ptr[c]; f < g->row_ptr[c + 1]; ++f) {
          if (g->kind[f] == SW_FACE_BOUNDARY) continue;
          int64_t n = g->nbr[f];
          bool found = false;
          for (int64_t q = g->row_ptr[n]; q < g->row_ptr[n + 1] && !found; ++q)
            found = g->kind[q] != SW_FACE_BOUNDARY && g->nbr[q] == c &&
                    g->normal[3 * q] == -g->normal[3 * f] && g->normal[3 * q + 1] == -g->normal[3 * f + 1] &&
                    g->normal[3 * q + 2] == -g->normal[3 * f + 2];
          if (!found) {
            int64_t expected = -1;
            bad.compare_exchange_strong(expected, f);
            return;
          }
        }
      }
    });
  for (auto& x : th) x.join();
  if (bad.load() >= 0) {
    char buf[200];
    snprintf(buf, sizeof(buf), "face %lld has no reciprocal face with a negated normal",
             (long long)bad.load());
    why = buf;
    return false;
  }
  return true;
}

// check_deadlock analogue (src/sweep/deadlock_detection.rs): with every cell active,
// each direction's dependency graph must be acyclic (Kahn's algorithm on the host).
bool check_acyclic(const sw_grid_csr* g, const std::vector<double>& dirs, int D, std::string& why) {
  int64_t n = g->num_cells;
  std::vector<uint32_t> cnt(n);
  std::vector<int64_t> queue(n);
  for (int d = 0; d < D; ++d) {
    const double* dv = &dirs[3 * d];
    auto dotf = [&](int64_t f) {
      return g->normal[3 * f] * dv[0] + g->normal[3 * f + 1] * dv[1] + g->normal[3 * f + 2] * dv[2];
    };
    int64_t qh = 0, qt = 0;
    for (int64_t c = 0; c < n; ++c) {
      uint32_t k = 0;
      for (int64_t f = g->row_ptr[c]; f < g->row_ptr[c + 1]; ++f)
        if (g->kind[f] == SW_FACE_LOCAL && dotf(f) < 0.0) ++k;
      cnt[c] = k;
      if (k == 0) queue[qt++] = c;
    }
    while (qh < qt) {
      int64_t c = queue[qh++];
      for (int64_t f = g->row_ptr[c]; f < g->row_ptr[c + 1]; ++f)
        if (g->kind[f] == SW_FACE_LOCAL && dotf(f) > 0.0)
          if (--cnt[g->nbr[f]] == 0) queue[qt++] = g->nbr[f];
    }
    if (qt != n) {
      char buf[200];
      snprintf(buf, sizeof(buf), "direction %d: %lld cells lie on dependency cycles", d, (long long)(n - qt));
      why = buf;
      return false;
    }
  }
  return true;
}

sw_status sync_ctl(sw_handle* h) {
  SW_CUDA(h, cudaMemcpyAsync(&h->ctl_host, h->p.ctl, sizeof(swk::SweepCtl), cudaMemcpyDeviceToHost, h->stream),
          "read control block");
  SW_CUDA(h, cudaStreamSynchronize(h->stream), "synchronize");
  h->n_ge_host.assign(h->ctl_host.n_ge, h->ctl_host.n_ge + h->L);
  return SW_OK;
}

// Tasks t in [t0, t1) with t % Np < N listed by level from order[base] on, in id order
// within a level (so each level lists one direction's cells after another in increasing
// order along the space-filling curve, and consecutive tasks touch neighbouring 32-byte
// sectors): each thread counts its contiguous share of the range per level, an
// exclusive scan over (level, thread) gives every share its first slot in each level,
// and the shares are written in parallel.  Returns the tasks per level ([L]).
static std::vector<uint64_t> stable_level_order(const uint16_t* level, uint32_t Np, uint32_t N, uint64_t t0,
                                                uint64_t t1, size_t L, uint64_t base, uint32_t* order) {
  const int nt = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  std::vector<std::vector<uint64_t>> cnt(nt, std::vector<uint64_t>(L, 0u));
  auto range = [&](int t, uint64_t& b, uint64_t& e) {
    b = t0 + (t1 - t0) * t / nt;
    e = t0 + (t1 - t0) * (t + 1) / nt;
  };
  std::vector<std::thread> th;
  for (int t = 0; t < nt; ++t)
    th.emplace_back([&, t]() {
      uint64_t b, e;
      range(t, b, e);
      for (uint64_t i = b; i < e; ++i)
        if (i % Np < N) ++cnt[t][level[i]];
    });
  for (auto& x : th) x.join();
  th.clear();
  std::vector<uint64_t> per_level(L, 0u);
  uint64_t at = base;
  for (size_t l = 0; l < L; ++l) {
    for (int t = 0; t < nt; ++t) {
      const uint64_t n = cnt[t][l];
      cnt[t][l] = at;
      at += n;
      per_level[l] += n;
    }
  }
  for (int t = 0; t < nt; ++t)
    th.emplace_back([&, t]() {
      uint64_t b, e;
      range(t, b, e);
      std::vector<uint64_t>& cur = cnt[t];
      for (uint64_t i = b; i < e; ++i)
        if (i % Np < N) order[cur[level[i]]++] = (uint32_t)i;
    });
  for (auto& x : th) x.join();
  return per_level;
}

// The positions of one task space: its D directions cut into `groups` contiguous
// groups, each group's tasks after the previous group's, by Kahn level (`level`, L
// levels), in task-id order within a level.  Writes order[N * D] and appends the end of
// every non-empty (group, level) segment to seg (which starts with 0); returns the
// number of positions written.
static uint64_t grouped_level_order(const uint16_t* level, uint32_t Np, uint32_t N, uint32_t D, size_t L,
                                    int groups, uint32_t* order, std::vector<uint32_t>& seg) {
  uint64_t base = 0;
  for (int g = 0; g < groups; ++g) {
    const uint64_t d0 = (uint64_t)D * g / groups, d1 = (uint64_t)D * (g + 1) / groups;
    const std::vector<uint64_t> n = stable_level_order(level, Np, N, d0 * Np, d1 * Np, L, base, order);
    for (size_t l = 0; l < L; ++l)
      if (n[l]) {
        base += n[l];
        seg.push_back((uint32_t)base);
      }
  }
  return base;
}

// Compact state (mixed path): task spaces hold fewer than kSpaceTasks tasks each.  The
// fewest spaces of evenly split directions that do, 0 when kMaxSpaces are not enough.
constexpr uint64_t kSpaceTasks = 1ull << 31;
static int min_task_spaces(uint32_t Np, int D) {
  for (int s = 1; s <= std::min(D, swh::kMaxSpaces); ++s)
    if ((uint64_t)Np * (uint64_t)((D + s - 1) / s) < kSpaceTasks) return s;
  return 0;
}

// Number of direction groups of the schedule: SUBSWEEP_DIR_GROUPS, else as many as keep
// a group's levels about 40 K tasks wide on average (one per 40 K tasks of the average
// level, rounded).  That is about the number of tasks the lockstep kernels hold in
// flight (152 SMs x 32 warps x 8 tasks), so a task seldom waits for an upwind word, and
// a level's records, slots and words (~100 bytes a task) stay a small part of L2.
// Measured on the C4 generator at 256^3 x 84 (4,927 levels, 286 K tasks per level):
// 1, 4, 7 and 12 groups move 367, 169, 121 and 106 B of DRAM traffic per task in a
// level-0 sweep of 105, 94, 91 and 93 ms.
static int schedule_dir_groups(int D, uint64_t tasks, size_t levels) {
  constexpr uint64_t kGroupWidth = 40960;
  int g = (int)std::min<uint64_t>((tasks / std::max<size_t>(levels, 1) + kGroupWidth / 2) / kGroupWidth, (uint64_t)D);
  if (const char* env = std::getenv("SUBSWEEP_DIR_GROUPS")) g = std::atoi(env);
  return std::max(1, std::min(g, D));
}

// Levelled schedule (Kahn levels of all N*D tasks with every cell active), built once
// per grid on the device, per task space (one space unless the compact state splits the
// directions; task ids and positions are local to a space).  A dependency cycle leaves
// tasks unscheduled; such a grid keeps only the dependency-driven path, whose sweep then
// reports the stall as the reference would deadlock (the compact state, which has no
// such path, refuses the grid).
sw_status build_schedule(sw_handle* h) {
  swh::DevicePtrs& p = h->p;
  struct DeviceScratch {
    void* ptr = nullptr;
    ~DeviceScratch() {
      if (ptr) cudaFree(ptr);
    }
  } level_scratch;
  int max_ds = 0;
  for (int sp = 0; sp < p.num_spaces; ++sp) max_ds = std::max(max_ds, p.space_d0[sp + 1] - p.space_d0[sp]);
  SW_CUDA(h, cudaMalloc(&level_scratch.ptr, (size_t)h->Np * max_ds * sizeof(uint16_t)), "schedule scratch");
  uint16_t* task_level = static_cast<uint16_t*>(level_scratch.ptr);
  uint64_t hash = 0xcbf29ce484222325ull;  // FNV-1a over the state kind, spaces, groups and offsets
  auto mix = [&](uint32_t v) {
    for (int k = 0; k < 4; ++k) hash = (hash ^ ((v >> (8 * k)) & 0xffu)) * 0x100000001b3ull;
  };
  mix((uint32_t)p.geo_mode);
  mix((uint32_t)p.num_spaces);
  uint32_t depth = 0;
  for (int sp = 0; sp < p.num_spaces; ++sp) {
    const swh::DevicePtrs q = swh::space_view(p, sp);
    const uint64_t total = (uint64_t)h->N * (uint64_t)q.D;
    SW_CUDA(h, cudaMemsetAsync(p.ctl, 0, offsetof(swk::SweepCtl, tasks), h->stream), "reset control");
    SW_CUDA(h, cudaMemsetAsync(task_level, 0, (size_t)h->Np * q.D * sizeof(uint16_t), h->stream), "schedule scratch");
    SW_CUDA(h, h->ops->schedule_seed(q, h->stream), "schedule seed kernel");
    std::vector<uint32_t> lvl = {0};
    unsigned long long tail = 0;
    SW_CUDA(h, cudaMemcpyAsync(&tail, &p.ctl->tail, sizeof(tail), cudaMemcpyDeviceToHost, h->stream), "read tail");
    SW_CUDA(h, cudaStreamSynchronize(h->stream), "schedule seed");
    uint32_t begin = 0;
    uint32_t round = 0;
    while (tail > begin) {
      const uint32_t end = (uint32_t)tail;
      lvl.push_back(end);
      if (round + 1 >= 0xffffu) return h->fail(SW_ERR_UNSUPPORTED, "dependency graph deeper than 65534 levels");
      SW_CUDA(h, h->ops->kahn_round(q, begin, end, task_level, round, h->stream), "schedule round kernel");
      ++round;
      SW_CUDA(h, cudaMemcpyAsync(&tail, &p.ctl->tail, sizeof(tail), cudaMemcpyDeviceToHost, h->stream), "read tail");
      SW_CUDA(h, cudaStreamSynchronize(h->stream), "schedule round");
      begin = end;
    }
    uint32_t err = 0;
    SW_CUDA(h, cudaMemcpy(&err, &p.ctl->error, sizeof(err), cudaMemcpyDeviceToHost), "read error flag");
    if (tail != total || err != 0) {
      if (p.geo_mode) return h->fail(SW_ERR_STALLED, "the dependency graph has a cycle (compact state)");
      // cyclic dependency graph: no schedule.  The push path falls back to the
      // dependency-driven queue; the pull path visits tasks in id order and its waits run
      // out, so either reports the stall at the first sweep, where the reference deadlocks.
      p.num_sched_levels = 0;
      if (h->ops->pull) {
        std::vector<uint32_t> ids;
        ids.reserve(total);
        for (uint32_t d = 0; d < (uint32_t)h->D; ++d)
          for (uint32_t c = 0; c < (uint32_t)h->N; ++c) ids.push_back(d * h->Np + c);
        SW_CUDA(h, cudaMemcpy(p.order, ids.data(), ids.size() * sizeof(uint32_t), cudaMemcpyHostToDevice), "order");
      }
      SW_CUDA(h, cudaMemsetAsync(p.ctl, 0, offsetof(swk::SweepCtl, tasks), h->stream), "reset control");
      return SW_OK;
    }
    // The positions: the space's directions are cut into `groups` contiguous groups,
    // each group's tasks listed after the previous group's, by Kahn level, in task-id
    // order within a level.  Directions never depend on one another, so this is a
    // topological order, and its segments (one per non-empty (group, level)) are levels
    // of a valid levelled schedule.  Fewer directions per level keep the words a level
    // reads (written one or a few levels before) in L2 on large grids; the compact
    // state's geometry kernel pays a grid barrier per segment and keeps one group.  The
    // order is a stable counting sort on the host, so every handle on the same grid
    // gets the same schedule: the pull path's words are indexed by schedule position,
    // and checkpoints hold them in that order.
    const size_t L = lvl.size() - 1;
    depth = std::max(depth, (uint32_t)L);
    int groups = schedule_dir_groups(q.D, total, L);
    if (p.geo_mode && !std::getenv("SUBSWEEP_DIR_GROUPS")) groups = 1;
    std::vector<uint32_t> seg = {0};
    {
      std::vector<uint16_t> tl((size_t)h->Np * q.D);
      SW_CUDA(h, cudaMemcpy(tl.data(), task_level, tl.size() * sizeof(uint16_t), cudaMemcpyDeviceToHost),
              "read task levels");
      std::vector<uint32_t> order(total);
      const uint64_t base =
          grouped_level_order(tl.data(), h->Np, (uint32_t)h->N, (uint32_t)q.D, L, groups, order.data(), seg);
      if (base != total) return h->fail(SW_ERR_CUDA, "schedule order incomplete");
      SW_CUDA(h, cudaMemcpy(q.order, order.data(), order.size() * sizeof(uint32_t), cudaMemcpyHostToDevice),
              "upload order");
    }
    uint32_t* d_lvl;
    // padded to a multiple of four entries: the staged wavefront kernel copies them whole
    const size_t lvl_words = (seg.size() + 3) & ~(size_t)3;
    if (!h->alloc(&d_lvl, lvl_words)) return h->fail(SW_ERR_OOM, "device allocation of the schedule failed");
    SW_CUDA(h, cudaMemset(d_lvl, 0, lvl_words * sizeof(uint32_t)), "schedule");
    SW_CUDA(h, cudaMemcpy(d_lvl, seg.data(), seg.size() * sizeof(uint32_t), cudaMemcpyHostToDevice),
            "upload schedule");
    p.space_lvl[sp] = d_lvl;
    p.space_segments[sp] = (uint32_t)(seg.size() - 1);
    p.space_lvl_words[sp] = (uint32_t)lvl_words;
    mix((uint32_t)groups);
    for (uint32_t o : seg) mix(o);
  }
  SW_CUDA(h, cudaMemsetAsync(p.ctl, 0, offsetof(swk::SweepCtl, tasks), h->stream), "reset control");
  p.lvl = p.space_lvl[0];
  p.num_sched_levels = p.space_segments[0];
  p.lvl_words = p.space_lvl_words[0];
  h->stats_schedule_levels = depth;  // the dependency depth
  h->schedule_hash = hash;
  return SW_OK;
}

// Push path: precomputed downwind fractions of every schedule position, when they fit
// in the free device memory less a reserve of 1/16 of the device (at least 4 GiB) for
// later allocations (SUBSWEEP_FP64_RECORDS=0 never builds them, =1 always tries).
// Without them the transport computes the geometry on the fly.
sw_status build_push_records(sw_handle* h) {
  swh::DevicePtrs& p = h->p;
  if (!h->ops->push_records || p.num_sched_levels == 0) return SW_OK;
  int mode = -1;
  if (const char* env = std::getenv("SUBSWEEP_FP64_RECORDS")) mode = std::atoi(env) != 0 ? 1 : 0;
  if (mode == 0) return SW_OK;
  const int64_t positions = h->N * (int64_t)h->D;
  const size_t nc = (size_t)((positions + swk::kCompactChunk - 1) / swk::kCompactChunk);
  const size_t rec_bytes = (size_t)positions * sizeof(uint4);
  size_t free_b = 0, total_b = 0;
  SW_CUDA(h, cudaMemGetInfo(&free_b, &total_b), "memory info");
  const size_t reserve = std::max(total_b / 16, (size_t)4 << 30);
  const size_t room = free_b > reserve ? free_b - reserve : 0;
  if (mode < 0 && rec_bytes > room) return SW_OK;
  struct DeviceScratch {
    void* ptr = nullptr;
    ~DeviceScratch() {
      if (ptr) cudaFree(ptr);
    }
  } rec_mem, off_mem;
  if (cudaMalloc(&rec_mem.ptr, rec_bytes) != cudaSuccess) {
    (void)cudaGetLastError();
    return SW_OK;  // no room: the geometry path
  }
  SW_CUDA(h, cudaMalloc(&off_mem.ptr, (nc + 1) * sizeof(unsigned long long)), "record scratch");
  auto* chunk_off = static_cast<unsigned long long*>(off_mem.ptr);
  p.push_rec = rec_mem.ptr;
  cudaError_t ce = h->ops->push_records(p, 0, chunk_off, h->stream);
  unsigned long long total = 0;
  if (ce == cudaSuccess)
    ce = cudaMemcpyAsync(&total, chunk_off + nc, sizeof(total), cudaMemcpyDeviceToHost, h->stream);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(h->stream);
  p.push_rec = nullptr;
  if (ce != cudaSuccess) return h->cuda_fail(ce, "downwind fraction count kernels");
  const size_t slot_bytes = (size_t)total * (sizeof(uint32_t) + sizeof(double));
  if (mode < 0 && rec_bytes + slot_bytes > room) return SW_OK;
  uint32_t* tgt = nullptr;
  double* frac = nullptr;
  if (!h->alloc(&tgt, std::max<unsigned long long>(total, 1)) || !h->alloc(&frac, std::max<unsigned long long>(total, 1))) {
    (void)cudaGetLastError();
    return SW_OK;
  }
  p.push_rec = rec_mem.ptr;
  p.push_tgt = tgt;
  p.push_frac = frac;
  ce = h->ops->push_records(p, 1, chunk_off, h->stream);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(h->stream);
  uint32_t err = 0;
  if (ce == cudaSuccess) ce = cudaMemcpy(&err, &p.ctl->error, sizeof(err), cudaMemcpyDeviceToHost);
  if (ce != cudaSuccess) {
    p.push_rec = nullptr;
    return h->cuda_fail(ce, "downwind fraction kernel");
  }
  if (err & swk::kErrRecords) {
    p.push_rec = nullptr;
    return h->fail(SW_ERR_CUDA, "downwind classification disagrees with its count");
  }
  h->allocations.push_back(rec_mem.ptr);  // kept for the handle's lifetime
  rec_mem.ptr = nullptr;
  h->stats_upwind_slots = (int64_t)total;
  return SW_OK;
}

// Pull path: task records and upwind slots of every schedule position (after the
// schedule, or the id order of a cyclic grid, is in place).
sw_status build_records(sw_handle* h) {
  if (!h->ops->records) return SW_OK;
  swh::DevicePtrs& p = h->p;
  if (p.geo_mode) {  // compact state: only the periodic fold's entries
    SW_CUDA(h, h->ops->records(p, 1, nullptr, h->stream), "periodic fold entries");
    SW_CUDA(h, cudaStreamSynchronize(h->stream), "periodic fold entries");
    return SW_OK;
  }
  const size_t nc = (size_t)((h->N * (int64_t)h->D + swk::kCompactChunk - 1) / swk::kCompactChunk);
  struct DeviceScratch {
    void* ptr = nullptr;
    ~DeviceScratch() {
      if (ptr) cudaFree(ptr);
    }
  } off_scratch;
  SW_CUDA(h, cudaMalloc(&off_scratch.ptr, (nc + 1) * sizeof(unsigned long long)), "record scratch");
  auto* chunk_off = static_cast<unsigned long long*>(off_scratch.ptr);
  SW_CUDA(h, h->ops->records(p, 0, chunk_off, h->stream), "task record kernels");
  unsigned long long total = 0;
  SW_CUDA(h, cudaMemcpyAsync(&total, chunk_off + nc, sizeof(total), cudaMemcpyDeviceToHost, h->stream),
          "read slot total");
  SW_CUDA(h, cudaStreamSynchronize(h->stream), "task records");
  uint2* slots = nullptr;
  // two slots of padding: the staged wavefront kernel copies 16-byte aligned ranges
  if (!h->alloc(&slots, total + 2))
    return h->fail(SW_ERR_OOM, "device allocation of the upwind slots (%llu MB) failed", (total * 8) >> 20);
  p.pull_slots = slots;
  SW_CUDA(h, h->ops->records(p, 1, chunk_off, h->stream), "upwind slot kernel");
  SW_CUDA(h, cudaStreamSynchronize(h->stream), "upwind slots");
  uint32_t err = 0;
  SW_CUDA(h, cudaMemcpy(&err, &p.ctl->error, sizeof(err), cudaMemcpyDeviceToHost), "read error flag");
  if (err & swk::kErrRecords) return h->fail(SW_ERR_CUDA, "upwind slot classification disagrees with its count");
  h->stats_upwind_slots = (int64_t)total;
  return SW_OK;
}

}  // namespace


namespace swh {

bool handle_view(sw_handle* h, HandleView* out) {
  if (!h || !out) return false;
  out->p = &h->p;
  out->ops = h->ops;
  out->stream = h->stream;
  out->device = h->device;
  out->num_cells = h->N;
  out->num_directions = h->D;
  out->num_levels = h->L;
  return true;
}

sw_status handle_fail(sw_handle* h, sw_status st, const char* message) {
  if (h) h->last_error = message;
  return st;
}

void handle_clear_error(sw_handle* h) {
  if (h) h->last_error.clear();
}

}  // namespace swh

extern "C" {

sw_status sw_default_params(sw_params* p) {
  if (!p) return SW_ERR_INVALID_ARG;
  std::memset(p, 0, sizeof(*p));
  p->num_directions = 84;
  p->explicit_directions = nullptr;
  p->num_timestep_levels = 1;
  p->periodic = 0;
  p->max_timestep = 1e6 * 3.15576e7;  // 1 Myr
  p->rotate_directions = 0;               // parameters.rs:64-78
  p->significant_rate_threshold = 0.0;
  p->timestep_safety_factor = 0.01 * 10.0;  // Dimensionless::percent(10.0)
  p->chemistry_timestep_safety_factor = 0.01 * 10.0;
  p->check_deadlock = 0;
  p->prevent_cooling = 1;
  p->num_tasks_to_solve_before_send_receive = 10000;
  p->scale_factor = 1.0;
  p->precision = SW_PRECISION_FP64;
  p->device = -1;
  p->use_graphs = 0;
  p->autotune = 1;
  return SW_OK;
}

sw_status sw_directions_from_num(int32_t num, double* out) {
  std::vector<double> d;
  if (!out || !directions_for(num, d)) return SW_ERR_INVALID_ARG;
  std::memcpy(out, d.data(), d.size() * sizeof(double));
  return SW_OK;
}

sw_status sw_create(const sw_params* params, const sw_grid_csr* grid, const sw_cell_init* init,
                    sw_handle** out) {
  g_create_error.clear();
  if (!out) return create_fail(SW_ERR_INVALID_ARG, "out is NULL");
  *out = nullptr;
  if (!params || !grid || !init) return create_fail(SW_ERR_INVALID_ARG, "NULL argument");
  const sw_params& P = *params;
  if (P.rotate_directions)
    return create_fail(SW_ERR_UNSUPPORTED, "rotate_directions is not supported by the GPU sweep");
  if (P.num_timestep_levels < 1 || P.num_timestep_levels > 16)
    return create_fail(SW_ERR_INVALID_ARG, "num_timestep_levels must be in 1..16");
  if (!(P.max_timestep > 0.0) || !std::isfinite(P.max_timestep))
    return create_fail(SW_ERR_INVALID_ARG, "max_timestep must be positive");
  if (P.precision != SW_PRECISION_FP64 && P.precision != SW_PRECISION_MIXED)
    return create_fail(SW_ERR_INVALID_ARG, "unknown precision");
  std::vector<double> dirs;
  int D = P.num_directions;
  if (P.explicit_directions) {
    if (D < 1) return create_fail(SW_ERR_INVALID_ARG, "num_directions must be >= 1");
    dirs.assign(P.explicit_directions, P.explicit_directions + 3 * D);
    for (int d = 0; d < D; ++d) {  // glam normalize: v * (1 / |v|)
      double* v = &dirs[3 * d];
      double inv = 1.0 / std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
      if (!std::isfinite(inv)) return create_fail(SW_ERR_INVALID_ARG, "direction %d has zero length", d);
      v[0] *= inv;
      v[1] *= inv;
      v[2] *= inv;
    }
  } else if (!directions_for(D, dirs)) {
    return create_fail(SW_ERR_INVALID_ARG, "num_directions %d has no direction table (1,16,21,32,64,84)", D);
  }
  if (D > swk::kMaxDirections) return create_fail(SW_ERR_UNSUPPORTED, "at most 128 directions");

  const int64_t N = grid->num_cells;
  if (N < 1 || N >= (int64_t)1 << 30) return create_fail(SW_ERR_INVALID_ARG, "num_cells must be in 1..2^30-1");
  const uint32_t Np = (uint32_t)((N + 31) / 32 * 32);
  // The FP64 path keeps 32-bit task ids; the mixed path splits larger grids into task
  // spaces of fewer than 2^31 tasks each (compact state).
  const uint64_t task_ids = (uint64_t)Np * (uint64_t)D;
  if (P.precision == SW_PRECISION_FP64 && task_ids >= 0xffffffffull)
    return create_fail(SW_ERR_UNSUPPORTED, "num_cells * directions must stay below 2^32 task ids (FP64 path)");
  if (min_task_spaces(Np, D) == 0)
    return create_fail(SW_ERR_UNSUPPORTED, "num_cells * directions needs more than %d task spaces of 2^31 tasks",
                       swh::kMaxSpaces);
  if (!grid->row_ptr || !grid->nbr || !grid->kind || !grid->area || !grid->normal || !grid->volume || !grid->size)
    return create_fail(SW_ERR_INVALID_ARG, "grid array is NULL");
  if (!init->density || !init->ionized_hydrogen_fraction || !init->temperature || !init->source)
    return create_fail(SW_ERR_INVALID_ARG, "cell init array is NULL");
  if (grid->row_ptr[0] != 0) return create_fail(SW_ERR_INVALID_ARG, "row_ptr[0] must be 0");
  double max_normal = 0.0;
  for (int64_t c = 0; c < N; ++c) {
    int64_t nf = grid->row_ptr[c + 1] - grid->row_ptr[c];
    if (nf < 0) return create_fail(SW_ERR_INVALID_ARG, "row_ptr not monotone at cell %lld", (long long)c);
    if (nf > swk::kMaxFaces)
      return create_fail(SW_ERR_UNSUPPORTED, "cell %lld has %lld faces (max %d)", (long long)c, (long long)nf,
                         swk::kMaxFaces);
  }
  const int64_t E = grid->row_ptr[N];
  if (E >= 0xffffffffll) return create_fail(SW_ERR_UNSUPPORTED, "at most 2^32-1 faces");
  for (int64_t f = 0; f < E; ++f) {
    uint8_t k = grid->kind[f];
    if (k > SW_FACE_BOUNDARY) return create_fail(SW_ERR_INVALID_ARG, "face %lld has invalid kind", (long long)f);
    if (k != SW_FACE_BOUNDARY && (grid->nbr[f] < 0 || grid->nbr[f] >= N))
      return create_fail(SW_ERR_INVALID_ARG, "face %lld neighbour out of range", (long long)f);
    const double* nv = &grid->normal[3 * f];
    double l = std::sqrt(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]);
    if (!std::isfinite(l) || !std::isfinite(grid->area[f]))
      return create_fail(SW_ERR_INVALID_ARG, "face %lld has non-finite geometry", (long long)f);
    max_normal = std::max(max_normal, l);
  }
  std::string why;
  if (!check_reciprocal_faces(grid, why)) return create_fail(SW_ERR_INVALID_ARG, "%s", why.c_str());
  if (P.check_deadlock && !check_acyclic(grid, dirs, D, why)) return create_fail(SW_ERR_STALLED, "%s", why.c_str());
  if (P.prevent_cooling) {
    // HydrogenOnly clamps x_HII into [x_floor, 1 - 1e-10] and f64::clamp panics when
    // the floor (the current x_HII) is above that range.
    for (int64_t c = 0; c < N; ++c)
      if (init->ionized_hydrogen_fraction[c] > 1.0 - 1e-10)
        return create_fail(SW_ERR_INVALID_ARG,
                           "cell %lld: x_HII above 1 - 1e-10 with prevent_cooling (reference panics)",
                           (long long)c);
  }

  sw_handle* h = new sw_handle();
  h->params = P;
  h->params.explicit_directions = nullptr;
  h->ops = (P.precision == SW_PRECISION_MIXED) ? &swh::kOpsMixed : &swh::kOpsFP64;
  h->dirs = dirs;
  h->D = D;
  h->Np = Np;
  h->L = P.num_timestep_levels;
  h->N = N;
  h->E = E;
  h->ts.init(P.max_timestep, P.num_timestep_levels);

  auto bail = [&](sw_status st) {
    g_create_error = h->last_error;
    delete h;
    return st;
  };
  cudaError_t ce = cudaSuccess;
  if (P.device >= 0)
    h->device = P.device;
  else
    ce = cudaGetDevice(&h->device);
  if (ce != cudaSuccess) {
    h->cuda_fail(ce, "select device");
    return bail(SW_ERR_CUDA);
  }
  // the handle's device is current while the handle is built (and freed on failure)
  swh::DeviceScope device_scope(h->device);
  if (device_scope.status != cudaSuccess) {
    h->cuda_fail(device_scope.status, "select device");
    return bail(SW_ERR_CUDA);
  }
  int coop = 0, sms = 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, h->device);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
  if (!coop) {
    h->fail(SW_ERR_CUDA, "device does not support cooperative launches");
    return bail(SW_ERR_CUDA);
  }
  int bps = 0;
  ce = h->ops->occupancy(&bps);
  if (ce != cudaSuccess || bps < 1) {
    h->cuda_fail(ce == cudaSuccess ? cudaErrorInvalidConfiguration : ce, "occupancy");
    return bail(SW_ERR_CUDA);
  }
  if ((ce = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) != cudaSuccess) {
    h->cuda_fail(ce, "stream");
    return bail(SW_ERR_CUDA);
  }
  for (auto& e : h->ev) cudaEventCreate(&e);

  swh::DevicePtrs& p = h->p;
  p.num_cells = N;
  p.D = D;
  p.Np = Np;
  p.num_levels = h->L;
  for (int i = 0; i < 3 * D; ++i) p.dir32_host[i] = (float)dirs[i];
  p.threshold = P.significant_rate_threshold;
  p.max_timestep = P.max_timestep;
  p.timestep_safety = P.timestep_safety_factor;
  p.chem_safety = P.chemistry_timestep_safety_factor;
  p.scale_factor = P.scale_factor;
  p.prevent_cooling = P.prevent_cooling;
  // Resident blocks of the persistent transport kernel: at most the occupancy limit;
  // SUBSWEEP_SWEEP_BLOCKS_PER_SM lowers it (launch-shape tuning).
  // The dependency-driven kernel is bound by contention on its queue counters, not by
  // occupancy: one resident block per SM measured fastest.
  int want = 1;
  if (const char* env = std::getenv("SUBSWEEP_SWEEP_BLOCKS_PER_SM")) want = std::atoi(env);
  if (want >= 1 && want < bps) bps = want;
  p.coop_blocks = bps * sms;
  int lbps = 0;
  ce = h->ops->occupancy_levels(&lbps);
  if (ce != cudaSuccess || lbps < 1) {
    h->cuda_fail(ce == cudaSuccess ? cudaErrorInvalidConfiguration : ce, "occupancy");
    return bail(SW_ERR_CUDA);
  }
  if (const char* env = std::getenv("SUBSWEEP_LEVEL_BLOCKS_PER_SM")) {
    int v = std::atoi(env);
    if (v >= 1 && v < lbps) lbps = v;
  }
  p.level_blocks = lbps * sms;
  // SUBSWEEP_TRANSPORT=levels|queue pins the transport kernel (tests and tuning).
  if (const char* env = std::getenv("SUBSWEEP_TRANSPORT")) {
    if (std::strcmp(env, "levels") == 0) h->force_path = 1;
    if (std::strcmp(env, "queue") == 0) h->force_path = 2;
  }
  // transport kernel variant: SUBSWEEP_PULL_VARIANT fixes it, else the autotuner picks
  // it (sw_params.autotune; SUBSWEEP_AUTOTUNE=0|1 overrides)
  p.num_sms = sms;
  if (const char* env = std::getenv("SUBSWEEP_LEVEL_BLOCKS_PER_SM")) p.level_bps_cap = std::atoi(env);
  h->autotune = P.autotune != 0;
  if (const char* env = std::getenv("SUBSWEEP_AUTOTUNE")) h->autotune = std::atoi(env) != 0;
  if (const char* env = std::getenv("SUBSWEEP_PULL_VARIANT")) {
    p.pull_variant = std::atoi(env);
    h->autotune = false;
  }
  if (h->ops->num_tune_variants == 0) h->autotune = false;
  // graph replay of steps (SUBSWEEP_GRAPH=0|1 overrides the parameter)
  h->graph_mode = P.use_graphs != 0;
  if (const char* env = std::getenv("SUBSWEEP_GRAPH")) h->graph_mode = std::atoi(env) != 0;
  // SUBSWEEP_COMPACT=always|never overrides the mixed path's choice between compacting
  // the active positions and stamping inactive tasks in the sweep (tests and tuning).
  if (const char* env = std::getenv("SUBSWEEP_COMPACT")) {
    if (std::strcmp(env, "always") == 0) p.compact_mode = 1;
    if (std::strcmp(env, "never") == 0) p.compact_mode = 2;
  }
  // SUBSWEEP_TRACE=1 prints one line per level sweep to stderr (level, active tasks,
  // transport kernel / transport / chemistry milliseconds, transport attempts).
  if (const char* env = std::getenv("SUBSWEEP_TRACE")) h->trace = env[0] != '\0' && env[0] != '0';
  p.timeout_ns = 2ull * 1000 * 1000 * 1000;  // a lane waits at most 2 s for its queue slot
  double max_dir = 0.0;
  for (int d = 0; d < D; ++d)
    max_dir = std::max(max_dir, std::sqrt(dirs[3 * d] * dirs[3 * d] + dirs[3 * d + 1] * dirs[3 * d + 1] +
                                          dirs[3 * d + 2] * dirs[3 * d + 2]));
  // FP32 dot of FP32-rounded vectors: |error| <= ~5 * 2^-24 * |n| |d|; 4x margin.
  p.guard = (float)(20.0 * std::ldexp(1.0, -24) * std::max(1.0, max_normal) * std::max(1.0, max_dir));
  // Stored rate unit: photons/s in the FP64 drop-in; a power of two in the mixed path,
  // so that rates up to the total source (times 2^32 headroom) stay finite in FP32 and
  // the smallest normal float is ~2^-126 of the largest source.
  double total_source = 0.0;
  for (int64_t c = 0; c < N; ++c) total_source += std::fabs(init->source[c]);
  p.rate_scale = 1.0;
  if (P.precision == SW_PRECISION_MIXED && total_source > 0.0) {
    int e = 0;
    std::frexp(total_source, &e);
    p.rate_scale = std::ldexp(1.0, e - 96);
  }

  // geometry upload in kernel layout.  FP32 areas carry a power-of-two scale that maps
  // the largest face area to ~1 (areas of ~1e42 m^2 overflow FP32); the FP32 transport
  // only uses ratios of areas within a cell, which the scale leaves exact.
  double max_area = 0.0;
  for (int64_t f = 0; f < E; ++f) max_area = std::max(max_area, std::fabs(grid->area[f]));
  int area_exp = 0;
  if (max_area > 0.0) std::frexp(max_area, &area_exp);
  {
    std::vector<double> geo64(4 * (size_t)E);
    std::vector<float> geo32(4 * (size_t)E);
    std::vector<uint32_t> geo16(h->ops->pull ? 4 * (size_t)E : 0);
    std::vector<uint32_t> nbr(E);
    std::vector<uint32_t> row(N + 1);
    for (int64_t i = 0; i <= N; ++i) row[i] = (uint32_t)grid->row_ptr[i];
    for (int64_t f = 0; f < E; ++f) {
      for (int a = 0; a < 3; ++a) {
        geo64[4 * f + a] = grid->normal[3 * f + a];
        geo32[4 * f + a] = (float)grid->normal[3 * f + a];
      }
      geo64[4 * f + 3] = grid->area[f];
      geo32[4 * f + 3] = (float)std::ldexp(grid->area[f], -area_exp);
      uint32_t kind = grid->kind[f];
      uint32_t nb = (kind == SW_FACE_BOUNDARY) ? 0u : (uint32_t)grid->nbr[f];
      nbr[f] = nb | (kind << swk::kKindShift);
      if (h->ops->pull) {  // {area * n in the scaled FP32 area unit, neighbour | kind}
        const double a = std::ldexp(grid->area[f], -area_exp);
        for (int c3 = 0; c3 < 3; ++c3) {
          const float v = (float)(a * grid->normal[3 * f + c3]);
          std::memcpy(&geo16[4 * f + c3], &v, sizeof(float));
        }
        geo16[4 * f + 3] = nbr[f];
      }
    }
    uint32_t* d_row;
    double* d_geo64;
    float* d_geo32;
    uint32_t* d_nbr;
    if (!h->alloc(&d_row, N + 1) || !h->alloc(&d_geo64, 4 * (size_t)E) || !h->alloc(&d_geo32, 4 * (size_t)E) ||
        !h->alloc(&d_nbr, E)) {
      h->fail(SW_ERR_OOM, "device allocation of the grid failed");
      return bail(SW_ERR_OOM);
    }
    cudaMemcpy(d_row, row.data(), (N + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice);
    cudaMemcpy(d_geo64, geo64.data(), geo64.size() * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(d_geo32, geo32.data(), geo32.size() * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(d_nbr, nbr.data(), E * sizeof(uint32_t), cudaMemcpyHostToDevice);
    if (h->ops->pull) {
      uint32_t* d_geo16;
      if (!h->alloc(&d_geo16, geo16.size())) {
        h->fail(SW_ERR_OOM, "device allocation of the grid failed");
        return bail(SW_ERR_OOM);
      }
      cudaMemcpy(d_geo16, geo16.data(), geo16.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
      p.geo16 = d_geo16;
    }
    p.off = d_row;
    p.geo64 = d_geo64;
    p.geo32 = d_geo32;
    p.nbr = d_nbr;
    // cells that receive periodic contributions
    std::vector<uint32_t> pcells;
    for (int64_t c = 0; c < N; ++c)
      for (int64_t f = grid->row_ptr[c]; f < grid->row_ptr[c + 1]; ++f)
        if (grid->kind[f] == SW_FACE_LOCAL_PERIODIC) {
          pcells.push_back((uint32_t)c);
          break;
        }
    uint32_t* d_pc;
    if (!h->alloc(&d_pc, pcells.size())) {
      h->fail(SW_ERR_OOM, "device allocation failed");
      return bail(SW_ERR_OOM);
    }
    if (!pcells.empty()) cudaMemcpy(d_pc, pcells.data(), pcells.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
    p.periodic_cells = d_pc;
    p.n_periodic_cells = (uint32_t)pcells.size();
    if (h->ops->pull && !pcells.empty()) {  // the fold's precomputed upwind periodic faces
      uint8_t *fcnt = nullptr, *fchanged = nullptr;
      uint2* fslots = nullptr;
      const size_t entries = pcells.size() * (size_t)D;
      if (!h->alloc(&fcnt, entries) || !h->alloc(&fslots, entries * 4) || !h->alloc(&fchanged, pcells.size())) {
        h->fail(SW_ERR_OOM, "device allocation of the periodic fold slots failed");
        return bail(SW_ERR_OOM);
      }
      p.fold_cnt = fcnt;
      p.fold_slots = fslots;
      p.fold_changed = fchanged;
    }
  }
  // directions
  {
    std::vector<float> d32(dirs.begin(), dirs.end());
    double* d_dir64;
    float* d_dir32;
    if (!h->alloc(&d_dir64, dirs.size()) || !h->alloc(&d_dir32, dirs.size())) {
      h->fail(SW_ERR_OOM, "device allocation failed");
      return bail(SW_ERR_OOM);
    }
    cudaMemcpy(d_dir64, dirs.data(), dirs.size() * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(d_dir32, d32.data(), d32.size() * sizeof(float), cudaMemcpyHostToDevice);
    p.dir64 = d_dir64;
    p.dir32 = d_dir32;
  }
  // cells
  {
    double *d_size, *d_volume, *d_density, *d_source, *d_x, *d_y, *d_T, *d_att, *d_prev, *d_cts, *d_sdt, *d_ion;
    uint8_t* d_level;
    char* d_src_dir;
    const size_t rb = (size_t)h->ops->rate_bytes;
    bool ok = h->alloc(&d_size, N) && h->alloc(&d_volume, N) && h->alloc(&d_density, N) && h->alloc(&d_source, N) &&
              h->alloc(&d_x, N) && h->alloc(&d_y, N) && h->alloc(&d_T, N) && h->alloc(&d_att, N) &&
              h->alloc(&d_prev, N) && h->alloc(&d_cts, N) && h->alloc(&d_sdt, N) && h->alloc(&d_ion, N) &&
              h->alloc(&d_level, N) && h->alloc(&d_src_dir, N * rb) && h->alloc(&h->scratch, N);
    if (!ok) {
      h->fail(SW_ERR_OOM, "device allocation of cell state failed");
      return bail(SW_ERR_OOM);
    }
    std::vector<double> y(N), inf(N, INFINITY);
    for (int64_t c = 0; c < N; ++c) y[c] = 1.0 - init->ionized_hydrogen_fraction[c];
    // Site::source_per_direction_bin (site.rs:49-51), in stored rate units
    if (rb == 8) {
      std::vector<double> sd(N);
      for (int64_t c = 0; c < N; ++c) sd[c] = init->source[c] / (double)D;
      cudaMemcpy(d_src_dir, sd.data(), N * sizeof(double), cudaMemcpyHostToDevice);
    } else {
      std::vector<float> sd(N);
      for (int64_t c = 0; c < N; ++c) sd[c] = (float)(init->source[c] / (double)D / p.rate_scale);
      cudaMemcpy(d_src_dir, sd.data(), N * sizeof(float), cudaMemcpyHostToDevice);
    }
    cudaMemcpy(d_size, grid->size, N * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(d_volume, grid->volume, N * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(d_density, init->density, N * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(d_source, init->source, N * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(d_x, init->ionized_hydrogen_fraction, N * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(d_y, y.data(), N * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(d_T, init->temperature, N * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(d_ion, inf.data(), N * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemset(d_att, 0, N * sizeof(double));
    cudaMemset(d_prev, 0, N * sizeof(double));  // Site::new: zero previous rate
    cudaMemset(d_cts, 0, N * sizeof(double));   // change_timescale = 0
    cudaMemset(d_sdt, 0, N * sizeof(double));   // species timestep = 0
    cudaMemset(d_level, h->L - 1, N);           // Sweep::new: all cells at level n-1
    p.size = d_size;
    p.volume = d_volume;
    p.density = d_density;
    p.source = d_source;
    p.xhii = d_x;
    p.yneu = d_y;
    p.temperature = d_T;
    p.att = d_att;
    p.previous_rate = d_prev;
    p.change_timescale = d_cts;
    p.species_timestep = d_sdt;
    p.ionization_time = d_ion;
    p.level = d_level;
    p.src_dir = d_src_dir;
  }
  // per-(cell, direction) state, [dir][cell]
  // Compact state of the mixed path (no task records, upwind slots or inverse order;
  // words by task; the geometry kernel): for grids of 2^31 tasks or more, for grids whose
  // full state would not fit in the free device memory (records, slots, schedule, words,
  // rates and the active lists of the levels: ~44 + 4 * faces per cell + 4 * (levels - 1)
  // bytes per task), and on request (SUBSWEEP_COMPACT_STATE=1; SUBSWEEP_TASK_SPACES asks
  // for more task spaces than the grid needs).
  p.num_spaces = 1;
  p.space_d0[0] = 0;
  p.space_d0[1] = D;
  if (h->ops->pull) {
    const uint64_t tasks = (uint64_t)Np * (uint64_t)D;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) (void)cudaGetLastError();
    const double full = (44.0 + 4.0 * (double)E / (double)N + 4.0 * (h->L - 1)) * (double)tasks;
    bool geo = tasks >= kSpaceTasks || (free_b > 0 && full > 0.92 * (double)free_b);
    if (const char* env = std::getenv("SUBSWEEP_COMPACT_STATE")) geo = geo || std::atoi(env) != 0;
    if (geo) {
      int spaces = min_task_spaces(Np, D);
      if (const char* env = std::getenv("SUBSWEEP_TASK_SPACES"))
        spaces = std::max(spaces, std::min(std::atoi(env), std::min(D, swh::kMaxSpaces)));
      p.geo_mode = 1;
      p.num_spaces = spaces;
      for (int sp = 0; sp <= spaces; ++sp) p.space_d0[sp] = D * sp / spaces;
      p.compact_mode = 2;  // every sweep visits every position
      p.pull_variant = 0;
      h->autotune = false;
    }
  }
  {
    const size_t nd = (size_t)Np * D;
    const size_t rb = (size_t)h->ops->rate_bytes;
    // push path (FP64): incoming, outgoing, periodic, pending rates and the ready queue;
    // pull path (mixed): incoming and periodic rates and the {q, sweep} words (words
    // indexed by schedule position).
    const bool pull = h->ops->pull;
    char *inc = nullptr, *outg = nullptr, *per = nullptr, *pend = nullptr;
    uint32_t *cnt = nullptr, *queue = nullptr, *order = nullptr;
    unsigned long long* qe = nullptr;
    swk::SweepCtl* ctl = nullptr;
    bool ok = h->alloc(&inc, nd * rb) && h->alloc(&per, nd * rb) && h->alloc(&cnt, nd / 4) &&
              h->alloc(&order, nd) && h->alloc(&ctl, 1);
    uint4* rec = nullptr;
    uint32_t *act_counts = nullptr, *chunk = nullptr, *pos_of_task = nullptr, *act_bits = nullptr;
    uint32_t* cell_sweep = nullptr;
    uint2* cellpack = nullptr;
    float* per_pos = nullptr;
    const size_t chunks = (nd + swk::kCompactChunk - 1) / swk::kCompactChunk + 1;
    if (ok) ok = h->alloc(&chunk, chunks);
    if (ok && pull && p.geo_mode)  // compact state: words by task, no records or inverse order
      ok = h->alloc(&qe, nd) && h->alloc(&act_counts, 32) && h->alloc(&cell_sweep, (size_t)h->Np) &&
           h->alloc(&cellpack, (size_t)h->Np);
    else if (ok && pull)
      ok = h->alloc(&qe, nd) && h->alloc(&rec, nd) && h->alloc(&act_counts, 32) && h->alloc(&pos_of_task, nd) &&
           h->alloc(&act_bits, (nd + 31) / 32) && h->alloc(&cell_sweep, (size_t)h->Np) &&
           h->alloc(&cellpack, (size_t)h->Np) &&
           // per-position periodic sources: only for the staged wavefront kernel (78)
           (p.pull_variant != 78 || h->alloc(&per_pos, (size_t)h->N * h->D + 4));
    if (ok && !pull) ok = h->alloc(&outg, nd * rb) && h->alloc(&pend, nd * rb) && h->alloc(&queue, nd);
    if (!ok) {
      h->fail(SW_ERR_OOM, "device allocation of the transport state (%zu MB) failed",
              (pull ? (p.geo_mode ? 2 * rb + 13 : 2 * rb + 41) : 4 * rb + 9) * nd >> 20);
      return bail(SW_ERR_OOM);
    }
    cudaMemset(inc, 0, nd * rb);
    cudaMemset(per, 0, nd * rb);
    cudaMemset(cnt, 0, nd);
    if (pull) {
      cudaMemset(qe, 0, nd * sizeof(unsigned long long));
      cudaMemset(cell_sweep, 0, (size_t)h->Np * sizeof(uint32_t));
      if (per_pos) cudaMemset(per_pos, 0, ((size_t)h->N * h->D + 4) * sizeof(float));
    } else {
      cudaMemset(outg, 0, nd * rb);
      cudaMemset(pend, 0, nd * rb);
      cudaMemset(queue, 0xff, nd * sizeof(uint32_t));  // every slot empty
    }
    cudaMemset(ctl, 0, sizeof(swk::SweepCtl));
    p.qe = qe;
    p.pull_rec = rec;
    p.act_counts = act_counts;
    p.pos_of_task = pos_of_task;
    p.act_bits = act_bits;
    p.cell_sweep = cell_sweep;
    p.cellpack = cellpack;
    p.per_pos = per_pos;
    p.chunk = chunk;
    p.incoming = inc;
    p.outgoing = outg;
    p.periodic = per;
    p.pending = pend;
    p.counters = cnt;
    p.queue = queue;
    p.order = order;
    p.ctl = ctl;
  }
  ce = cudaDeviceSynchronize();
  if (ce != cudaSuccess) {
    h->cuda_fail(ce, "upload");
    return bail(ce == cudaErrorMemoryAllocation ? SW_ERR_OOM : SW_ERR_CUDA);
  }
  if (swh::launch_level_hist(p, h->stream) != cudaSuccess || sync_ctl(h) != SW_OK) {
    if (h->last_error.empty()) h->fail(SW_ERR_CUDA, "level ordering failed");
    return bail(SW_ERR_CUDA);
  }
  {
    sw_status st = build_schedule(h);
    if (st == SW_OK) st = build_records(h);
    if (st == SW_OK) st = build_push_records(h);
    if (st != SW_OK) return bail(st);
  }
  *out = h;
  return SW_OK;
}

// One step replayed as a CUDA graph: the same launches as sw_step (per sweep: control
// reset, attenuation, dependency counts on the push path, transport, periodic fold,
// chemistry; then the level update and the ionization times), captured once per step
// shape (lowest allowed level before and after, and each sweep's level and kernel
// choice).  The sweep
// numbers and the end time live in the control block, copied from pinned host memory by
// the graph's first node; the error flag stays set across the step's sweeps, so a stall
// ends the remaining sweeps at once, and is read when the step has finished.  Event
// nodes around each sweep's transport give the transport kernel time.
// Pull path: whether the sweep of `level` runs over the compacted list of its active
// positions (above level 0 with fewer than half of the cells active; SUBSWEEP_COMPACT
// overrides), and that list's buffer, allocated on first use.
static bool pull_sparse(sw_handle* h, int level) {
  const swh::DevicePtrs& p = h->p;
  if (level <= 0) return false;
  if (p.compact_mode == 1) return true;
  if (p.compact_mode == 2) return false;
  return h->n_ge_host[level] * 2 < h->N;
}

static sw_status ensure_act_list(sw_handle* h, int level) {
  if (h->p.act_lv[level]) return SW_OK;
  uint32_t* buf = nullptr;
  if (!h->alloc(&buf, (size_t)h->Np * h->D))
    return h->fail(SW_ERR_OOM, "device allocation of the active positions of level %d failed", level);
  h->p.act_lv[level] = buf;
  return SW_OK;
}

static sw_status step_graph(sw_handle* h, double* time_elapsed_out) {
  const swh::PrecisionOps& ops = *h->ops;
  swh::DevicePtrs& p = h->p;
  std::vector<int> levels;
  std::vector<bool> variants;
  uint64_t expected = 0;
  TimestepState after = h->ts;
  after.advance();
  std::vector<int64_t> key = {h->ts.lowest, after.lowest, p.pull_variant};
  for (int level : h->ts.sweep_order()) {
    if (h->n_ge_host[level] == 0) continue;  // Sweep::run_sweeps skips empty levels (mod.rs:262)
    levels.push_back(level);
    expected += (uint64_t)h->n_ge_host[level] * (uint64_t)h->D;
    // pull path: compaction or not; push path: levelled schedule or ready queue
    bool variant;
    if (ops.pull) {
      variant = pull_sparse(h, level);
      if (variant) {
        sw_status st = ensure_act_list(h, level);  // allocations stay outside the capture
        if (st != SW_OK) return st;
      }
    } else {
      variant = p.num_sched_levels > 0 && (uint64_t)h->n_ge_host[level] * 16 >= (uint64_t)h->N;
      if (h->force_path == 1) variant = p.num_sched_levels > 0;
      if (h->force_path == 2) variant = false;
    }
    variants.push_back(variant);
    key.push_back(level * 2 + (variant ? 1 : 0));
  }
  if (!h->graph_scalars) {
    void* ptr = nullptr;
    SW_CUDA(h, cudaMallocHost(&ptr, sizeof(sw_handle::GraphScalars)), "pinned graph scalars");
    h->graph_scalars = static_cast<sw_handle::GraphScalars*>(ptr);
  }
  if (!h->graph_exec || key != h->graph_key) {
    if (h->graph_exec) {
      cudaGraphExecDestroy(h->graph_exec);
      h->graph_exec = nullptr;
    }
    while (h->graph_ev.size() < 2 * levels.size()) {
      cudaEvent_t e;
      SW_CUDA(h, cudaEventCreate(&e), "event");
      h->graph_ev.push_back(e);
    }
    SW_CUDA(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal), "begin graph capture");
    cudaError_t ce = cudaMemcpyAsync(&p.ctl->epoch_base, h->graph_scalars, sizeof(sw_handle::GraphScalars),
                                     cudaMemcpyHostToDevice, h->stream);
    if (ce == cudaSuccess) ce = cudaMemsetAsync(&p.ctl->error, 0, sizeof(uint32_t), h->stream);
    swh::DevicePtrs q = p;
    q.epoch_base = &p.ctl->epoch_base;
    int64_t kernels = 3;  // level update (two kernels) and ionization times
    uint32_t compacted = 0;  // pull path: levels whose list the step has built so far
    std::vector<int> compact_now(levels.size(), 0);
    for (size_t k = 0; k < levels.size(); ++k) {
      // attenuation, transport, chemistry, the periodic fold, and the counts (push) or
      // the compaction at a sparse level's first sweep (pull)
      kernels += 3 + (p.n_periodic_cells > 0 ? 1 : 0);
      // the fold's mark pass after a sweep that leaves cells inactive (pull path)
      if (ops.pull && p.n_periodic_cells > 0 && h->n_ge_host[levels[k]] < h->N) kernels += 1;
      if (!ops.pull) {
        kernels += 1;
      } else if (variants[k] && !((compacted >> levels[k]) & 1u)) {
        compact_now[k] = 1;
        compacted |= 1u << levels[k];
        kernels += 4;
      }
    }
    for (size_t k = 0; k < levels.size() && ce == cudaSuccess; ++k) {
      const int level = levels[k];
      q.epoch = (uint32_t)(k + 1);
      q.active_cells = h->n_ge_host[level];
      q.sparse_sweep = (ops.pull && variants[k]) ? 1 : 0;
      q.compact_now = compact_now[k];
      ce = cudaMemsetAsync(p.ctl, 0, offsetof(swk::SweepCtl, error), h->stream);
      if (ce == cudaSuccess) ce = ops.attenuation(q, level, h->stream);
      if (ce == cudaSuccess && !ops.pull) ce = ops.init_counts(q, level, nullptr, !variants[k], h->stream);
      // external records: event nodes that are recorded when the graph runs
      if (ce == cudaSuccess) ce = cudaEventRecordWithFlags(h->graph_ev[2 * k], h->stream, cudaEventRecordExternal);
      if (ce == cudaSuccess) ce = (ops.pull || variants[k]) ? ops.sweep_levels(q, level, h->stream)
                                                            : ops.sweep(q, level, h->stream);
      if (ce == cudaSuccess) ce = cudaEventRecordWithFlags(h->graph_ev[2 * k + 1], h->stream, cudaEventRecordExternal);
      if (ce == cudaSuccess) ce = ops.fold_periodic(q, h->stream);
      if (ce == cudaSuccess) ce = ops.chemistry(q, level, h->stream);
    }
    if (ce == cudaSuccess) ce = swh::launch_update_levels(p, after.lowest, h->stream);
    if (ce == cudaSuccess) ce = swh::launch_ionization_time(p, 0.0, h->stream, &p.ctl->time);
    cudaGraph_t graph = nullptr;
    const cudaError_t end = cudaStreamEndCapture(h->stream, &graph);
    if (ce == cudaSuccess) ce = end;
    if (ce == cudaSuccess) ce = cudaGraphInstantiate(&h->graph_exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (ce != cudaSuccess) {
      h->graph_exec = nullptr;
      return h->cuda_fail(ce, "graph capture of a step");
    }
    h->graph_key = key;
    h->graph_captures += 1;
    h->graph_kernels = kernels;
  }
  const double elapsed = h->ts.current_max_timestep();
  h->graph_scalars->epoch_base = p.epoch;
  h->graph_scalars->time = h->sim_time + elapsed;
  const unsigned long long tasks_before = h->ctl_host.tasks;
  SW_CUDA(h, cudaEventRecord(h->ev[5], h->stream), "event");
  SW_CUDA(h, cudaGraphLaunch(h->graph_exec, h->stream), "graph launch");
  SW_CUDA(h, cudaEventRecord(h->ev[1], h->stream), "event");
  sw_status st = sync_ctl(h);
  if (st != SW_OK) return st;
  p.epoch += (uint32_t)levels.size();
  h->last_epoch = p.epoch;
  const uint32_t err = h->ctl_host.error;
  if (err & (swk::kErrStall | swk::kErrQueue)) {
    // leave the queue empty so the handle stays usable for inspection
    if (p.queue) cudaMemsetAsync(p.queue, 0xff, (size_t)h->Np * h->D * sizeof(uint32_t), h->stream);
    cudaStreamSynchronize(h->stream);
    return h->fail(SW_ERR_STALLED, "a sweep of the step stalled: tasks left unsolved after a %.1f s wait "
                   "(dependency cycle; flags 0x%x)", p.timeout_ns * 1e-9, err);
  }
  if (err & swk::kErrClamp)
    return h->fail(SW_ERR_INVALID_ARG, "x_HII floor above 1 - 1e-10 in the chemistry clamp (reference panics)");
  h->ts = after;
  h->sim_time += elapsed;
  h->act_valid = 0;  // the step's level update changed the active sets
  float step_ms = 0.f;
  cudaEventElapsedTime(&step_ms, h->ev[5], h->ev[1]);
  const int64_t n = (int64_t)levels.size();
  for (int64_t k = 0; k < n; ++k) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, h->graph_ev[2 * k], h->graph_ev[2 * k + 1]) == cudaSuccess)
      h->stats.transport_kernel_ms += ms;
  }
  (void)cudaGetLastError();  // a failed timing query must not surface at the next launch
  h->stats.step_ms += step_ms;
  h->stats.steps += 1;
  h->stats.level_sweeps += n;
  for (bool v : variants) h->stats.levelled_sweeps += (ops.pull || v) ? 1 : 0;
  h->stats.transport_launches += n;
  h->stats.graph_launches += 1;
  h->stats.kernel_launches += h->graph_kernels;
  h->stats.tasks = (int64_t)h->ctl_host.tasks;
  h->stats.chem_cells = (int64_t)h->ctl_host.chem_cells;
  h->stats.chem_attempts = (int64_t)h->ctl_host.chem_attempts;
  h->stats.chem_failures = (int64_t)h->ctl_host.chem_failures;
  h->stats.transport_attempts = (int64_t)h->ctl_host.attempts;
  h->stats.simulation_time = h->sim_time;
  if (time_elapsed_out) *time_elapsed_out = elapsed;
  const uint64_t solved = h->ctl_host.tasks - tasks_before;
  if (solved != expected)
    return h->fail(SW_ERR_STALLED, "sweep solved %llu of %llu tasks: the dependency graph has a cycle",
                   (unsigned long long)solved, (unsigned long long)expected);
  return SW_OK;
}

sw_status sw_create_batch(const sw_params* params, int32_t n_boxes, const sw_grid_csr* grids,
                          const sw_cell_init* inits, sw_handle** out) {
  if (!out) return create_fail(SW_ERR_INVALID_ARG, "out is NULL");
  *out = nullptr;
  if (!params || !grids || !inits || n_boxes < 1) return create_fail(SW_ERR_INVALID_ARG, "invalid batch arguments");
  int64_t n = 0, e = 0;
  for (int32_t b = 0; b < n_boxes; ++b) {
    const sw_grid_csr& g = grids[b];
    const sw_cell_init& in = inits[b];
    if (g.num_cells < 1 || !g.row_ptr || !g.nbr || !g.kind || !g.area || !g.normal || !g.volume || !g.size ||
        !in.density || !in.ionized_hydrogen_fraction || !in.temperature || !in.source)
      return create_fail(SW_ERR_INVALID_ARG, "box %d: missing array", b);
    if (g.row_ptr[0] != 0 || g.row_ptr[g.num_cells] < 0) return create_fail(SW_ERR_INVALID_ARG, "box %d: bad row_ptr", b);
    // neighbour indices must stay inside the box before they are offset into the union
    for (int64_t f = 0; f < g.row_ptr[g.num_cells]; ++f)
      if (g.kind[f] != SW_FACE_BOUNDARY && (g.nbr[f] < 0 || g.nbr[f] >= g.num_cells))
        return create_fail(SW_ERR_INVALID_ARG, "box %d: face %lld has neighbour %d outside the box", b,
                           (long long)f, g.nbr[f]);
    n += g.num_cells;
    e += g.row_ptr[g.num_cells];
  }
  if (n > (int64_t)INT32_MAX) return create_fail(SW_ERR_UNSUPPORTED, "batch of %lld cells", (long long)n);
  std::vector<int64_t> row_ptr(n + 1);
  std::vector<int32_t> nbr(e);
  std::vector<uint8_t> kind(e);
  std::vector<double> area(e), normal(3 * e), volume(n), size(n), density(n), x(n), t(n), src(n);
  int64_t c0 = 0, f0 = 0;
  for (int32_t b = 0; b < n_boxes; ++b) {
    const sw_grid_csr& g = grids[b];
    const sw_cell_init& in = inits[b];
    const int64_t nb = g.num_cells, eb = g.row_ptr[nb];
    for (int64_t c = 0; c < nb; ++c) row_ptr[c0 + c] = f0 + g.row_ptr[c];
    for (int64_t f = 0; f < eb; ++f) {
      kind[f0 + f] = g.kind[f];
      nbr[f0 + f] = g.kind[f] == SW_FACE_BOUNDARY ? g.nbr[f] : (int32_t)(g.nbr[f] + c0);
    }
    std::copy(g.area, g.area + eb, area.begin() + f0);
    std::copy(g.normal, g.normal + 3 * eb, normal.begin() + 3 * f0);
    std::copy(g.volume, g.volume + nb, volume.begin() + c0);
    std::copy(g.size, g.size + nb, size.begin() + c0);
    std::copy(in.density, in.density + nb, density.begin() + c0);
    std::copy(in.ionized_hydrogen_fraction, in.ionized_hydrogen_fraction + nb, x.begin() + c0);
    std::copy(in.temperature, in.temperature + nb, t.begin() + c0);
    std::copy(in.source, in.source + nb, src.begin() + c0);
    c0 += nb;
    f0 += eb;
  }
  row_ptr[n] = e;
  const sw_grid_csr u = {n, row_ptr.data(), nbr.data(), kind.data(), area.data(), normal.data(), volume.data(),
                         size.data()};
  const sw_cell_init ui = {density.data(), x.data(), t.data(), src.data()};
  return sw_create(params, &u, &ui, out);
}

sw_status sw_step(sw_handle* h, double* time_elapsed_out) {
  if (!h) return SW_ERR_INVALID_ARG;
  h->last_error.clear();
  const swh::PrecisionOps& ops = *h->ops;
  SW_DEVICE_SCOPE(h);
  if (h->graph_mode && (h->tuned || !h->autotune)) return step_graph(h, time_elapsed_out);
  uint64_t expected = 0;
  std::vector<int> order = h->ts.sweep_order();
  unsigned long long tasks_before = h->ctl_host.tasks;
  float sweep_ms = 0.f, chem_ms = 0.f, level_ms = 0.f, kernel_ms = 0.f;
  int64_t launches = 0;
  SW_CUDA(h, cudaEventRecord(h->ev[5], h->stream), "event");
  for (int level : order) {
    // Sweep::run_sweeps skips levels without active cells (mod.rs:262)
    if (h->n_ge_host[level] == 0) continue;
    expected += (uint64_t)h->n_ge_host[level] * (uint64_t)h->D;
    SW_CUDA(h, cudaMemsetAsync(h->p.ctl, 0, offsetof(swk::SweepCtl, tasks), h->stream), "reset queue");
    SW_CUDA(h, cudaEventRecord(h->ev[0], h->stream), "event");
    // Sweeps with at least 1/16 of the cells active walk the precomputed schedule;
    // sparser ones use the dependency-driven queue, which touches only active tasks.
    bool levelled = h->p.num_sched_levels > 0 && (uint64_t)h->n_ge_host[level] * 16 >= (uint64_t)h->N;
    if (h->force_path == 1) levelled = h->p.num_sched_levels > 0;
    if (h->force_path == 2) levelled = false;
    // autotuning trials on dense sweeps only: sparse ones always run the lockstep kernel
    const bool trial = ops.pull && h->autotune && !h->tuned && !pull_sparse(h, level);
    if (trial) h->p.pull_variant = ops.tune_variants[h->tune_index];
    if (ops.pull) {
      levelled = true;  // the pull path always walks the schedule (or the id order)
      h->p.epoch += 1;
      h->last_epoch = h->p.epoch;
      h->p.active_cells = h->n_ge_host[level];
      h->p.sparse_sweep = pull_sparse(h, level) ? 1 : 0;
      h->p.compact_now = 0;
      if (h->p.sparse_sweep) {
        sw_status st = ensure_act_list(h, level);
        if (st != SW_OK) return st;
        if (!((h->act_valid >> level) & 1u)) {  // first sweep of this level in the step
          h->p.compact_now = 1;
          h->act_valid |= 1u << level;
          launches += 4;  // compaction of the active positions
        }
      }
    }
    // after the pull path's sweep number advanced: attenuation records it per solved cell
    SW_CUDA(h, ops.attenuation(h->p, level, h->stream), "attenuation kernel");
    if (!ops.pull) {
      SW_CUDA(h, ops.init_counts(h->p, level, nullptr, !levelled, h->stream), "init_counts kernel");
      launches += 1;
    }
    SW_CUDA(h, cudaEventRecord(h->ev[6], h->stream), "event");
    if (levelled) {
      SW_CUDA(h, ops.sweep_levels(h->p, level, h->stream), "levelled sweep kernel");
      h->stats.levelled_sweeps += 1;
    } else {
      SW_CUDA(h, ops.sweep(h->p, level, h->stream), "sweep kernel");
    }
    SW_CUDA(h, cudaEventRecord(h->ev[7], h->stream), "event");
    SW_CUDA(h, ops.fold_periodic(h->p, h->stream), "periodic fold kernel");
    launches += 3 + (h->p.n_periodic_cells > 0 ? 1 : 0);
    if (ops.pull && h->p.n_periodic_cells > 0 && h->p.active_cells < h->N) launches += 1;  // fold marks
    SW_CUDA(h, cudaEventRecord(h->ev[1], h->stream), "event");
    SW_CUDA(h, ops.chemistry(h->p, level, h->stream), "chemistry kernel");
    SW_CUDA(h, cudaEventRecord(h->ev[2], h->stream), "event");
    SW_CUDA(h, cudaStreamSynchronize(h->stream), "level sweep");
    float a = 0.f, b = 0.f, k = 0.f;
    cudaEventElapsedTime(&a, h->ev[0], h->ev[1]);
    cudaEventElapsedTime(&b, h->ev[1], h->ev[2]);
    cudaEventElapsedTime(&k, h->ev[6], h->ev[7]);
    (void)cudaGetLastError();  // timing queries are best effort
    sweep_ms += a;
    chem_ms += b;
    kernel_ms += k;
    if (trial) {  // one autotuning trial per sweep; the fastest variant per task is kept
      h->tune_ns.push_back(1e6 * k / std::max(1.0, (double)h->n_ge_host[level] * h->D));
      if (++h->tune_index == ops.num_tune_variants) {
        int best = 0;
        for (int i = 1; i < ops.num_tune_variants; ++i)
          if (h->tune_ns[i] < h->tune_ns[best]) best = i;
        h->p.pull_variant = ops.tune_variants[best];
        h->tuned = true;
      }
    }
    h->stats.transport_launches += 1;
    if (h->trace) {
      swk::SweepCtl c{};
      cudaMemcpy(&c, h->p.ctl, sizeof(c), cudaMemcpyDeviceToHost);
      std::fprintf(stderr,
                   "subsweep sweep level=%d active_tasks=%llu kernel_ms=%.3f transport_ms=%.3f chem_ms=%.3f "
                   "attempts=%llu chem_cells=%llu chem_attempts=%llu\n",
                   level, (unsigned long long)h->n_ge_host[level] * (unsigned long long)h->D, k, a, b,
                   (unsigned long long)c.attempts, (unsigned long long)c.chem_cells,
                   (unsigned long long)c.chem_attempts);
    }
    uint32_t err = 0;
    SW_CUDA(h, cudaMemcpy(&err, &h->p.ctl->error, sizeof(err), cudaMemcpyDeviceToHost), "read error flag");
    h->stats.level_sweeps += 1;
    if (err & (swk::kErrStall | swk::kErrQueue)) {
      // leave the queue empty so the handle stays usable for inspection
      if (h->p.queue) cudaMemsetAsync(h->p.queue, 0xff, (size_t)h->Np * h->D * sizeof(uint32_t), h->stream);
      cudaStreamSynchronize(h->stream);
      return h->fail(SW_ERR_STALLED,
                     "level %d sweep stalled: tasks left unsolved after a %.1f s wait (dependency cycle; flags 0x%x)",
                     level, h->p.timeout_ns * 1e-9, err);
    }
    if (err & swk::kErrClamp)
      return h->fail(SW_ERR_INVALID_ARG, "x_HII floor above 1 - 1e-10 in the chemistry clamp (reference panics)");
  }
  // TimestepState bookkeeping and level reassignment (mod.rs:268-270)
  double elapsed = h->ts.current_max_timestep();
  h->ts.advance();
  SW_CUDA(h, cudaEventRecord(h->ev[3], h->stream), "event");
  SW_CUDA(h, swh::launch_update_levels(h->p, h->ts.lowest, h->stream), "level kernels");
  h->act_valid = 0;  // levels change: the compacted lists are rebuilt next step
  SW_CUDA(h, cudaEventRecord(h->ev[4], h->stream), "event");
  h->sim_time += elapsed;
  SW_CUDA(h, swh::launch_ionization_time(h->p, h->sim_time, h->stream), "ionization time kernel");
  launches += 3;
  SW_CUDA(h, cudaEventRecord(h->ev[1], h->stream), "event");
  sw_status st = sync_ctl(h);
  if (st != SW_OK) return st;
  cudaEventElapsedTime(&level_ms, h->ev[3], h->ev[4]);
  float step_ms = 0.f;
  cudaEventElapsedTime(&step_ms, h->ev[5], h->ev[1]);
  (void)cudaGetLastError();
  h->stats.step_ms += step_ms;
  h->stats.transport_kernel_ms += kernel_ms;
  h->stats.kernel_launches += launches;
  uint64_t solved = h->ctl_host.tasks - tasks_before;
  h->stats.steps += 1;
  h->stats.tasks = (int64_t)h->ctl_host.tasks;
  h->stats.chem_cells = (int64_t)h->ctl_host.chem_cells;
  h->stats.chem_attempts = (int64_t)h->ctl_host.chem_attempts;
  h->stats.chem_failures = (int64_t)h->ctl_host.chem_failures;
  h->stats.transport_attempts = (int64_t)h->ctl_host.attempts;
  h->stats.sweep_ms += sweep_ms;
  h->stats.chem_ms += chem_ms;
  h->stats.level_ms += level_ms;
  h->stats.simulation_time = h->sim_time;
  if (time_elapsed_out) *time_elapsed_out = elapsed;
  if (solved != expected)
    return h->fail(SW_ERR_STALLED, "sweep solved %llu of %llu tasks: the dependency graph has a cycle",
                   (unsigned long long)solved, (unsigned long long)expected);
  return SW_OK;
}

sw_status sw_get_fields(sw_handle* h, double* x, double* T, double* dt, double* rate) {
  if (!h) return SW_ERR_INVALID_ARG;
  h->last_error.clear();
  SW_DEVICE_SCOPE(h);
  size_t nb = (size_t)h->N * sizeof(double);
  if (x) SW_CUDA(h, cudaMemcpyAsync(x, h->p.xhii, nb, cudaMemcpyDeviceToHost, h->stream), "copy x");
  if (T) SW_CUDA(h, cudaMemcpyAsync(T, h->p.temperature, nb, cudaMemcpyDeviceToHost, h->stream), "copy T");
  if (dt) SW_CUDA(h, cudaMemcpyAsync(dt, h->p.species_timestep, nb, cudaMemcpyDeviceToHost, h->stream), "copy dt");
  if (rate) {
    SW_CUDA(h, h->ops->photon_rate(h->p, h->last_epoch, h->scratch, h->stream), "photon rate kernel");
    SW_CUDA(h, cudaMemcpyAsync(rate, h->scratch, nb, cudaMemcpyDeviceToHost, h->stream), "copy rate");
  }
  SW_CUDA(h, cudaStreamSynchronize(h->stream), "synchronize");
  return SW_OK;
}

sw_status sw_get_cell_state(sw_handle* h, double* change_timescale, uint8_t* level, double* ionization_time) {
  if (!h) return SW_ERR_INVALID_ARG;
  h->last_error.clear();
  SW_DEVICE_SCOPE(h);
  size_t nb = (size_t)h->N * sizeof(double);
  if (change_timescale)
    SW_CUDA(h, cudaMemcpyAsync(change_timescale, h->p.change_timescale, nb, cudaMemcpyDeviceToHost, h->stream), "copy");
  if (level) SW_CUDA(h, cudaMemcpyAsync(level, h->p.level, h->N, cudaMemcpyDeviceToHost, h->stream), "copy");
  if (ionization_time)
    SW_CUDA(h, cudaMemcpyAsync(ionization_time, h->p.ionization_time, nb, cudaMemcpyDeviceToHost, h->stream), "copy");
  SW_CUDA(h, cudaStreamSynchronize(h->stream), "synchronize");
  return SW_OK;
}

sw_status sw_set_fields(sw_handle* h, const double* x, const double* T) {
  if (!h) return SW_ERR_INVALID_ARG;
  h->last_error.clear();
  SW_DEVICE_SCOPE(h);
  size_t nb = (size_t)h->N * sizeof(double);
  if (x) {
    std::vector<double> y(h->N);
    for (int64_t c = 0; c < h->N; ++c) y[c] = 1.0 - x[c];
    SW_CUDA(h, cudaMemcpy(h->p.xhii, x, nb, cudaMemcpyHostToDevice), "copy x");
    SW_CUDA(h, cudaMemcpy(h->p.yneu, y.data(), nb, cudaMemcpyHostToDevice), "copy y");
  }
  if (T) SW_CUDA(h, cudaMemcpy(h->p.temperature, T, nb, cudaMemcpyHostToDevice), "copy T");
  return SW_OK;
}

sw_status sw_get_level_counts(sw_handle* h, int64_t* per_level) {
  if (!h || !per_level) return SW_ERR_INVALID_ARG;
  for (int l = 0; l < h->L; ++l) per_level[l] = h->n_ge_host[l];
  return SW_OK;
}

sw_status sw_get_dependency_counts(sw_handle* h, int32_t level, uint8_t* counts) {
  if (!h || !counts || level < 0 || level >= h->L) return SW_ERR_INVALID_ARG;
  h->last_error.clear();
  SW_DEVICE_SCOPE(h);
  uint8_t* d_counts = nullptr;
  size_t nb = (size_t)h->N * h->D;
  SW_CUDA(h, cudaMalloc(&d_counts, nb), "alloc");
  cudaError_t e = cudaSuccess;
  if (h->p.num_spaces <= 1) {
    // inactive cells' entries are not written by the counting kernel: start from zero
    e = cudaMemsetAsync(d_counts, 0, nb, h->stream);
    if (e == cudaSuccess) e = h->ops->init_counts(h->p, level, d_counts, false, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(counts, d_counts, nb, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  } else {  // task spaces: each space's [cell][its directions] block, interleaved on the host
    std::vector<uint8_t> part;
    for (int sp = 0; sp < h->p.num_spaces && e == cudaSuccess; ++sp) {
      const swh::DevicePtrs v = swh::space_view(h->p, sp);
      const size_t ns = (size_t)h->N * v.D;
      part.resize(ns);
      e = cudaMemsetAsync(d_counts, 0, ns, h->stream);
      if (e == cudaSuccess) e = h->ops->init_counts(v, level, d_counts, false, h->stream);
      if (e == cudaSuccess) e = cudaMemcpyAsync(part.data(), d_counts, ns, cudaMemcpyDeviceToHost, h->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
      const int d0 = h->p.space_d0[sp];
      for (int64_t c = 0; c < h->N && e == cudaSuccess; ++c)
        std::memcpy(counts + (size_t)c * h->D + d0, part.data() + (size_t)c * v.D, v.D);
    }
  }
  cudaFree(d_counts);
  if (e != cudaSuccess) return h->cuda_fail(e, "dependency counts");
  return SW_OK;
}

sw_status sw_get_rates(sw_handle* h, double* incoming, double* outgoing, double* periodic) {
  if (!h) return SW_ERR_INVALID_ARG;
  h->last_error.clear();
  SW_DEVICE_SCOPE(h);
  size_t nb = (size_t)h->N * h->D * sizeof(double);
  double* d_out = nullptr;
  SW_CUDA(h, cudaMalloc(&d_out, nb), "alloc");
  double* dsts[3] = {incoming, outgoing, periodic};
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < 3 && e == cudaSuccess; ++i) {
    if (!dsts[i]) continue;
    e = h->ops->export_rates(h->p, i, h->last_epoch, d_out, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dsts[i], d_out, nb, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  }
  cudaFree(d_out);
  if (e != cudaSuccess) return h->cuda_fail(e, "export rates");
  return SW_OK;
}

// Checkpoint layout: a header, then the device arrays of checkpoint_sections in order.
struct CheckpointHeader {
  uint64_t magic;
  uint32_t version, precision;
  int64_t num_cells, num_faces;
  int32_t num_directions, num_levels;
  uint32_t np, rate_bytes;
  double sim_time;
  int32_t ts_lowest, ts_first_done;
  uint32_t epoch, last_epoch;
  uint64_t schedule_hash;  // pull path: fingerprint of the schedule the words are ordered by
};
constexpr uint64_t kCheckpointMagic = 0x3154504357535553ull;  // "SUSWCPT1"
// 2: the mixed path's words (8 bytes, by schedule position) and incoming rates (4 bytes,
// by task) in two sections
constexpr uint32_t kCheckpointVersion = 2;

struct CheckpointSection {
  void* dev;
  size_t bytes;
};

static std::vector<CheckpointSection> checkpoint_sections(sw_handle* h) {
  const swh::DevicePtrs& p = h->p;
  const size_t n = (size_t)h->N, nd = (size_t)h->Np * h->D, rb = (size_t)h->ops->rate_bytes;
  std::vector<CheckpointSection> v = {
      {p.xhii, n * 8},           {p.yneu, n * 8},          {p.temperature, n * 8}, {p.previous_rate, n * 8},
      {p.change_timescale, n * 8}, {p.species_timestep, n * 8}, {p.ionization_time, n * 8}, {p.level, n},
      {p.periodic, nd * rb},
  };
  if (h->ops->pull) {
    v.push_back({p.qe, nd * 8});  // words, by schedule position
    v.push_back({p.incoming, nd * 4});
    v.push_back({p.cell_sweep, n * 4});
  } else {
    v.push_back({p.incoming, nd * rb});
    v.push_back({p.outgoing, nd * rb});
    v.push_back({p.pending, nd * rb});
  }
  return v;
}

static size_t checkpoint_bytes(sw_handle* h) {
  size_t total = sizeof(CheckpointHeader);
  for (const CheckpointSection& s : checkpoint_sections(h)) total += s.bytes;
  return total;
}

// The per-cell level bytes follow seven per-cell double arrays (checkpoint_sections).
static size_t checkpoint_level_offset(int64_t num_cells) {
  return sizeof(CheckpointHeader) + 7 * (size_t)num_cells * sizeof(double);
}

// Checkpoint length implied by a header's counts, in the order of checkpoint_sections;
// 0 for counts no handle can have.
static size_t checkpoint_bytes_for(const CheckpointHeader& hd) {
  if (hd.num_cells < 1 || hd.num_cells >= ((int64_t)1 << 30) || hd.num_directions < 1 ||
      hd.num_directions > swk::kMaxDirections || hd.num_levels < 1 || hd.num_levels > 16 ||
      (int64_t)hd.np < hd.num_cells || (hd.rate_bytes != 4 && hd.rate_bytes != 8) ||
      (hd.precision != SW_PRECISION_FP64 && hd.precision != SW_PRECISION_MIXED))
    return 0;
  const size_t n = (size_t)hd.num_cells, nd = (size_t)hd.np * (size_t)hd.num_directions, rb = hd.rate_bytes;
  size_t total = checkpoint_level_offset(hd.num_cells) + n + nd * rb;
  total += hd.precision == SW_PRECISION_MIXED ? nd * 12 + n * 4 : 3 * nd * rb;
  return total;
}

// Header, length and level checks of a checkpoint buffer, before any byte of it reaches
// the device: a level >= num_levels would index past the per-level histograms.
static int32_t check_checkpoint(const void* buffer, size_t bytes, CheckpointHeader* hd_out) {
  if (bytes < sizeof(CheckpointHeader)) return 2;
  CheckpointHeader hd;
  std::memcpy(&hd, buffer, sizeof(hd));
  if (hd_out) *hd_out = hd;
  if (hd.magic != kCheckpointMagic || hd.version != kCheckpointVersion) return 1;
  const size_t need = checkpoint_bytes_for(hd);
  if (need == 0 || hd.ts_lowest < 0 || hd.ts_lowest >= hd.num_levels) return 1;
  if (bytes < need) return 2;
  const uint8_t* level = static_cast<const uint8_t*>(buffer) + checkpoint_level_offset(hd.num_cells);
  for (int64_t c = 0; c < hd.num_cells; ++c)
    if (level[c] >= hd.num_levels) return 3;
  return 0;
}

int64_t sw_host_schedule_order(const uint16_t* task_level, uint32_t np, uint32_t n, uint32_t d, int32_t levels,
                                int32_t groups, uint32_t* order, uint32_t* seg, int64_t seg_cap) {
  if (!task_level || !order || !seg || n == 0 || np < n || d == 0 || levels < 1 || groups < 1 ||
      groups > (int32_t)d || (uint64_t)np * d >= (1ull << 32))
    return -1;
  for (uint64_t t = 0; t < (uint64_t)np * d; ++t)
    if (t % np < n && task_level[t] >= levels) return -1;
  std::vector<uint32_t> s = {0};
  grouped_level_order(task_level, np, n, d, (size_t)levels, groups, order, s);
  for (size_t i = 0; i < s.size() && (int64_t)i < seg_cap; ++i) seg[i] = s[i];
  return (int64_t)s.size() - 1;
}

int32_t sw_host_task_spaces(uint32_t np, int32_t d) {
  if (np == 0 || d < 1) return -1;
  return min_task_spaces(np, d);
}

int32_t sw_host_dir_groups(int32_t d, uint64_t tasks, int64_t levels) {
  if (d < 1 || levels < 1) return -1;
  return schedule_dir_groups(d, tasks, (size_t)levels);
}

int32_t sw_host_check_checkpoint(const void* buffer, size_t bytes) {
  if (!buffer) return 1;
  return check_checkpoint(buffer, bytes, nullptr);
}

sw_status sw_checkpoint_size(sw_handle* h, size_t* bytes) {
  if (!h || !bytes) return SW_ERR_INVALID_ARG;
  *bytes = checkpoint_bytes(h);
  return SW_OK;
}

sw_status sw_save_state(sw_handle* h, void* buffer, size_t bytes) {
  if (!h || !buffer) return SW_ERR_INVALID_ARG;
  h->last_error.clear();
  if (bytes < checkpoint_bytes(h)) return h->fail(SW_ERR_INVALID_ARG, "checkpoint buffer too small");
  SW_DEVICE_SCOPE(h);
  CheckpointHeader hd{};
  hd.magic = kCheckpointMagic;
  hd.version = kCheckpointVersion;
  hd.precision = (uint32_t)h->params.precision;
  hd.num_cells = h->N;
  hd.num_faces = h->E;
  hd.num_directions = h->D;
  hd.num_levels = h->L;
  hd.np = h->Np;
  hd.rate_bytes = (uint32_t)h->ops->rate_bytes;
  hd.sim_time = h->sim_time;
  hd.ts_lowest = h->ts.lowest;
  hd.ts_first_done = h->ts.first_done ? 1 : 0;
  hd.epoch = h->p.epoch;
  hd.last_epoch = h->last_epoch;
  hd.schedule_hash = h->ops->pull ? h->schedule_hash : 0;
  char* out = static_cast<char*>(buffer);
  std::memcpy(out, &hd, sizeof(hd));
  size_t off = sizeof(hd);
  for (const CheckpointSection& s : checkpoint_sections(h)) {
    SW_CUDA(h, cudaMemcpyAsync(out + off, s.dev, s.bytes, cudaMemcpyDeviceToHost, h->stream), "save state");
    off += s.bytes;
  }
  SW_CUDA(h, cudaStreamSynchronize(h->stream), "save state");
  return SW_OK;
}

sw_status sw_load_state(sw_handle* h, const void* buffer, size_t bytes) {
  if (!h || !buffer) return SW_ERR_INVALID_ARG;
  h->last_error.clear();
  CheckpointHeader hd{};
  const int32_t check = check_checkpoint(buffer, bytes, &hd);
  if (check == 2 && bytes < sizeof(CheckpointHeader))
    return h->fail(SW_ERR_INVALID_ARG, "checkpoint buffer too small");
  if (hd.magic != kCheckpointMagic || hd.version != kCheckpointVersion) return h->fail(SW_ERR_INVALID_ARG, "not a checkpoint");
  if (hd.precision != (uint32_t)h->params.precision || hd.num_cells != h->N || hd.num_faces != h->E ||
      hd.num_directions != h->D || hd.num_levels != h->L || hd.np != h->Np ||
      hd.rate_bytes != (uint32_t)h->ops->rate_bytes)
    return h->fail(SW_ERR_INVALID_ARG, "checkpoint was written by a handle with another grid, parameters or precision");
  if (checkpoint_bytes_for(hd) != checkpoint_bytes(h))
    return h->fail(SW_ERR_INVALID_ARG, "checkpoint layout does not match this handle");
  if (h->ops->pull && hd.schedule_hash != h->schedule_hash)
    return h->fail(SW_ERR_INVALID_ARG, "checkpoint was written with another transport schedule (direction groups)");
  if (check == 1) return h->fail(SW_ERR_INVALID_ARG, "corrupt checkpoint header");
  if (check == 2) return h->fail(SW_ERR_INVALID_ARG, "checkpoint buffer too small");
  if (check == 3) return h->fail(SW_ERR_INVALID_ARG, "corrupt checkpoint: a cell's timestep level is out of range");
  SW_DEVICE_SCOPE(h);
  const char* in = static_cast<const char*>(buffer);
  size_t off = sizeof(hd);
  for (const CheckpointSection& s : checkpoint_sections(h)) {
    SW_CUDA(h, cudaMemcpyAsync(s.dev, in + off, s.bytes, cudaMemcpyHostToDevice, h->stream), "load state");
    off += s.bytes;
  }
  SW_CUDA(h, cudaStreamSynchronize(h->stream), "load state");
  h->sim_time = hd.sim_time;
  h->ts.lowest = hd.ts_lowest;
  h->ts.first_done = hd.ts_first_done != 0;
  h->p.epoch = hd.epoch;
  h->last_epoch = hd.last_epoch;
  // pull path: the periodic sources by schedule position follow from the restored words
  // (between steps the periodic array is the fold of the current words, so this
  // rewrites it unchanged)
  if (h->ops->pull) {
    swh::DevicePtrs q = h->p;
    q.active_cells = h->N;  // every entry
    SW_CUDA(h, h->ops->fold_periodic(q, h->stream), "periodic fold kernel");
  }
  // cells per level for the next step
  h->act_valid = 0;
  SW_CUDA(h, swh::launch_level_hist(h->p, h->stream), "level histogram");
  return sync_ctl(h);
}

sw_status sw_get_time_series(sw_handle* h, sw_time_series* out) {
  if (!h || !out) return SW_ERR_INVALID_ARG;
  h->last_error.clear();
  SW_DEVICE_SCOPE(h);
  if (!h->series_dev && !h->alloc(&h->series_dev, swh::kTimeSeriesPartials + 8))
    return h->fail(SW_ERR_OOM, "device allocation of the time-series buffer failed");
  double* partial = h->series_dev;
  double* out6 = h->series_dev + swh::kTimeSeriesPartials;
  SW_CUDA(h, h->ops->cell_rates(h->p, h->last_epoch, h->scratch, h->stream), "cell rate kernel");
  SW_CUDA(h, swh::launch_time_series(h->p, h->scratch, h->ops->carry_neutral, partial, out6, h->stream),
          "time series kernels");
  double v[6];
  SW_CUDA(h, cudaMemcpyAsync(v, out6, sizeof(v), cudaMemcpyDeviceToHost, h->stream), "read time series");
  SW_CUDA(h, cudaStreamSynchronize(h->stream), "time series");
  out->hydrogen_ionization_mass_average = v[0];
  out->hydrogen_ionization_volume_average = v[1];
  out->temperature_mass_average = v[2];
  out->temperature_volume_average = v[3];
  out->photoionization_rate_volume_average = v[4];
  out->weighted_photoionization_rate_volume_average = v[5];
  return SW_OK;
}

sw_status sw_get_stats(sw_handle* h, sw_stats* out) {
  if (!h || !out) return SW_ERR_INVALID_ARG;
  h->stats.schedule_levels = h->stats_schedule_levels;
  h->stats.upwind_slots = h->stats_upwind_slots;
  h->stats.pull_variant =
      h->ops->pull && !h->p.geo_mode ? (h->p.pull_variant > 0 ? h->p.pull_variant : swh::kDefaultPullVariant) : 0;
  h->stats.task_spaces = h->p.geo_mode ? h->p.num_spaces : 0;
  h->stats.device_bytes = h->device_bytes;
  *out = h->stats;
  return SW_OK;
}

const char* sw_last_error(const sw_handle* h) {
  if (!h) return g_create_error.c_str();
  return h->last_error.c_str();
}

void sw_destroy(sw_handle* h) {
  if (!h) return;
  swh::DeviceScope device_scope(h->device);  // frees on the handle's device
  cudaStreamSynchronize(h->stream);
  delete h;
}

}  // extern "C"
