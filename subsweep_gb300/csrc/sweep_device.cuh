// Device side of the sweep: dependency counting, the persistent dependency-driven
// transport kernel, periodic-source folding, chemistry and level reassignment.
//
// Layout in HBM.  Per-(cell, direction) arrays are direction-major, [dir][cell] with
// the cell stride Np = round_up(N, 32), and a task (cell c, direction d) is the
// index t = d * Np + c into all of them.  Cells are numbered along a space-filling
// curve, so the 8 FP32 rates sharing a 32-byte sector belong to neighbouring cells,
// which a direction's sweep front reaches at nearly the same time.
//   faces:  off[N+1] (u32 CSR offsets), geo32[E] = {nx, ny, nz, area * 2^-k} (float4,
//           area scaled so the FP32 path never overflows; it only uses area ratios),
//           geo64[E] = {nx, ny, nz, area}, nbr[E] = index | kind << 30
//   cells:  level (u8), density, x_HII, 1 - x_HII, T, source per direction bin,
//           attenuation factor, previous rate, change timescale, species timestep
//   tasks:  incoming / outgoing / periodic / periodic_pending rates (R = double in the
//           FP64 drop-in, float in the mixed path), u8 dependency counters (4 per u32
//           word) and the ready queue (u32 task ids, one slot per task and sweep).
//
// Transport (Sweep::single_sweep, src/sweep/mod.rs:274-289) runs as one persistent
// cooperative kernel over an asynchronous ready queue.  k_init_counts counts every
// active task's upwind dependencies (Sweep::init_counts) and enqueues the tasks that
// have none.  Warps of k_sweep claim 32 consecutive queue slots, one per lane, and each
// lane solves its task as soon as its slot is filled: outgoing rate, correction,
// distribution of the correction over the downwind faces (float atomics on the
// neighbours' incoming rates), then a release-ordered decrement of each active local
// neighbour's counter; the decrement that reaches zero enqueues that neighbour's task.
// Every task is enqueued exactly once, so the queue needs no wrap-around and the sweep
// is complete when N_active * D slots have been consumed.  There are no grid-wide
// barriers: the only waits are lanes spinning on their own slot, bounded by a
// globaltimer limit after which the kernel flags a stall and exits (a dependency cycle
// leaves slots unfilled).
#pragma once

#include <cstdint>

#include "chemistry_device.cuh"
#include "sweep_types.h"

namespace swk {

constexpr int kSweepThreads = 256;

struct DirParam {
  float v[kMaxDirections * 3];  // FP32 directions, passed by value (uniform reads)
};

template <typename R>
struct SweepArgs {
  const uint32_t* off;     // CSR offsets [N+1]
  const float4* geo32;
  const Geo64* geo64;
  const uint32_t* nbr;
  const double* dir64;     // [D*3]
  const float* dir32;      // [D*3]
  int D;
  uint32_t Np;
  uint32_t N;
  float guard;             // |dot32| above this has the sign of the FP64 dot
  const uint8_t* level;
  const R* src_dir;        // source / D per cell, in stored rate units
  const double* att;       // exp(-n_HI sigma size) per cell
  R threshold;             // significant_rate_threshold in stored rate units
  R* incoming;
  R* outgoing;
  R* periodic;
  R* pending;
  uint32_t* counters;      // u8 per task, 4 per word
  uint32_t* queue;
  SweepCtl* ctl;
  int current_level;
  unsigned long long timeout_ns;
};

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Device-scope relaxed accesses (served by L2, never by a stale L1 line).  Acquire
// loads are avoided on the polling path: at GPU scope they invalidate the SM's L1,
// which the face geometry relies on.
__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned long long ld_relaxed64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release(uint32_t* p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Dependency counter decrement with release semantics: this lane's incoming-rate
// additions (performed at L2) complete before the decrement.  The decrement that
// reaches zero is followed by a release store of the task into its queue slot; the
// consumer reads the slot and then, through the task id it loaded (an address
// dependency), the incoming rate from L2, which by then holds every upstream
// contribution.
__device__ __forceinline__ uint32_t atom_sub_release(uint32_t* p, uint32_t v) {
  uint32_t old;
  asm volatile("atom.release.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(0u - v) : "memory");
  return old;
}

// (n.x*d.x + n.y*d.y) + n.z*d.z with every product and sum rounded separately, as the
// reference evaluates it, in translation units compiled with and without contraction
__device__ __forceinline__ double dot64(const Geo64& g, double dx, double dy, double dz) {
  return __dadd_rn(__dadd_rn(__dmul_rn(g.x, dx), __dmul_rn(g.y, dy)), __dmul_rn(g.z, dz));
}

// Exact classification of a face against a direction: the sign of the FP64 dot
// (n.x*d.x + n.y*d.y) + n.z*d.z, which the reference tests with strict < 0 and > 0
// (grid/cell.rs:125-132).  The FP32 dot decides whenever it is farther from zero than
// its rounding-error bound; only near-perpendicular faces read the FP64 normal.
__device__ __forceinline__ int face_sign(float s32, const Geo64* g64, double dx, double dy, double dz, float guard) {
  if (s32 > guard) return 1;
  if (s32 < -guard) return -1;
  double e = dot64(*g64, dx, dy, dz);
  return (e > 0.0) - (e < 0.0);
}

// Warp-aggregated append of the predicated lanes' task ids to the ready queue.
__device__ __forceinline__ void enqueue(bool pred, uint32_t task, SweepCtl* ctl, uint32_t* queue,
                                        unsigned long long capacity) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t m = __ballot_sync(0xffffffffu, pred);
  if (m == 0) return;
  unsigned long long base = 0;
  const uint32_t leader = __ffs(m) - 1;
  if (lane == leader) base = atomicAdd(&ctl->tail, (unsigned long long)__popc(m));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (pred) {
    unsigned long long slot = base + __popc(m & ((1u << lane) - 1u));
    if (slot < capacity) {
      st_release(queue + slot, task);
    } else {
      atomicOr(&ctl->error, kErrQueue);
    }
  }
}

// ---------------------------------------------------------------------------
// Sweep::init_counts (src/sweep/mod.rs:346-386): for every active cell and direction,
// the number of upwind faces whose neighbour is LOCAL and active; tasks without
// dependencies are enqueued.  One thread per cell; each face is read once and tested
// against all directions (uniform direction reads from the kernel parameters);
// per-thread counters live in shared memory as bytes, [dir][thread].
// ---------------------------------------------------------------------------
constexpr int kCountThreads = 128;

template <typename R>
__global__ void __launch_bounds__(kCountThreads) k_init_counts(SweepArgs<R> a, DirParam dirs,
                                                               unsigned long long capacity,
                                                               uint8_t* debug_counts) {
  __shared__ uint8_t cnt[kMaxDirections * kCountThreads];
  const int tid = threadIdx.x;
  const uint32_t c = blockIdx.x * kCountThreads + tid;
  const bool active = c < a.N && a.level[c] >= a.current_level;
  for (int d = 0; d < a.D; ++d) cnt[d * kCountThreads + tid] = 0;
  if (active) {
    const uint32_t beg = a.off[c], end = a.off[c + 1];
    for (uint32_t f = beg; f < end; ++f) {
      const uint32_t nb = a.nbr[f];
      if ((nb >> kKindShift) != kKindLocal) continue;           // periodic / boundary: not counted
      if (a.level[nb & kNbrMask] < a.current_level) continue;   // inactive neighbour
      const float4 g = a.geo32[f];
      for (int d = 0; d < a.D; ++d) {
        const float s = g.x * dirs.v[3 * d] + g.y * dirs.v[3 * d + 1] + g.z * dirs.v[3 * d + 2];
        const bool up = face_sign(s, a.geo64 + f, a.dir64[3 * d], a.dir64[3 * d + 1], a.dir64[3 * d + 2],
                                  a.guard) < 0;
        cnt[d * kCountThreads + tid] += up ? 1 : 0;
      }
    }
  }
  for (int d = 0; d < a.D; ++d) {
    const uint8_t k = cnt[d * kCountThreads + tid];
    const uint32_t t = (uint32_t)d * a.Np + c;
    if (c < a.N) {
      // inactive cells get a sentinel that no sweep's decrements (<= 64) can exhaust,
      // so producers may decrement a LOCAL neighbour's counter without checking its level
      reinterpret_cast<uint8_t*>(a.counters)[t] = active ? k : (uint8_t)0x80;
      if (debug_counts && active) debug_counts[(size_t)c * a.D + d] = k;
    }
    if (capacity) enqueue(active && k == 0, t, a.ctl, a.queue, capacity);
  }
}

// Solve the tasks of the predicated lanes (Sweep::solve_task, src/sweep/mod.rs:423-485,
// with get_outgoing_rate 412-421, handle_local_neighbour 487-503 and
// handle_local_periodic_neighbour 505-513).  Called by all 32 lanes of a warp.
template <typename R>
__device__ __forceinline__ void solve_task(const SweepArgs<R>& a, bool pred, uint32_t t,
                                           unsigned long long capacity) {
  const bool fp64 = sizeof(R) == 8;
  uint32_t c = 0, d = 0, beg = 0, end = 0;
  double dx = 0, dy = 0, dz = 0;
  float fx = 0, fy = 0, fz = 0;
  R corr = R(0), total = R(0);
  if (pred) {
    d = t / a.Np;
    c = t - d * a.Np;
    beg = a.off[c];
    end = a.off[c + 1];
    fx = a.dir32[3 * d]; fy = a.dir32[3 * d + 1]; fz = a.dir32[3 * d + 2];
    dx = a.dir64[3 * d]; dy = a.dir64[3 * d + 1]; dz = a.dir64[3 * d + 2];
    R inc = __ldcg(a.incoming + t);
    if (inc < R(0)) {  // Photons::make_positive (chemistry/mod.rs:61-65)
      inc = R(0);
      a.incoming[t] = inc;
    }
    const R r = (inc + a.src_dir[c]) + __ldcg(a.periodic + t);  // Site::get_rate, site.rs:53-56
    const R out_new = (r < a.threshold) ? R(0) : r * R(a.att[c]);
    corr = out_new - a.outgoing[t];
    a.outgoing[t] = out_new;
    // total effective downwind area, summed in face order
    for (uint32_t f = beg; f < end; ++f) {
      const float4 g = a.geo32[f];
      const float s = g.x * fx + g.y * fy + g.z * fz;
      if (face_sign(s, a.geo64 + f, dx, dy, dz, a.guard) > 0) {
        if (fp64) {
          const Geo64 h = a.geo64[f];
          total += R(h.w * dot64(h, dx, dy, dz));
        } else {
          total += R(g.w * s);
        }
      }
    }
  }
  // Distribute the correction: incoming rates of LOCAL neighbours, pending periodic
  // sources of LOCAL_PERIODIC ones (boundary faces drop it).  The loop runs to the
  // warp's largest face count so that the enqueue stays warp-collective.
  const uint32_t nf = pred ? end - beg : 0u;
  uint32_t maxf = nf;
  for (int o = 16; o > 0; o >>= 1) maxf = max(maxf, __shfl_xor_sync(0xffffffffu, maxf, o));
  for (uint32_t i = 0; i < maxf; ++i) {
    bool ready = false;
    uint32_t task_n = 0;
    if (i < nf) {
      const uint32_t f = beg + i;
      const float4 g = a.geo32[f];
      const float s = g.x * fx + g.y * fy + g.z * fz;
      const uint32_t nb = a.nbr[f];
      const uint32_t kind = nb >> kKindShift;
      if (kind != kKindBoundary && face_sign(s, a.geo64 + f, dx, dy, dz, a.guard) > 0) {
        R eff;
        if (fp64) {
          const Geo64 h = a.geo64[f];
          eff = R(h.w * dot64(h, dx, dy, dz));
        } else {
          eff = R(g.w * s);
        }
        const uint32_t n = nb & kNbrMask;
        const uint32_t tn = d * a.Np + n;
        const R w = corr * (eff / total);
        if (kind == kKindPeriodic) {
          atomicAdd(a.pending + tn, w);
        } else {
          atomicAdd(a.incoming + tn, w);
          if (a.level[n] >= a.current_level) {
            const uint32_t shift = 8u * (tn & 3u);
            const uint32_t old = atom_sub_release(a.counters + (tn >> 2), 1u << shift);
            ready = ((old >> shift) & 0xffu) == 1u;
            task_n = tn;
          }
        }
      }
    }
    enqueue(ready, task_n, a.ctl, a.queue, capacity);
  }
}

// The persistent transport kernel (cooperative launch: every block is resident, so a
// lane waiting on its slot is always eventually served by the lanes that produce).
// A warp claims 32 slots only when the queue shows unclaimed work, and idle warps
// back off exponentially, so waiting costs little L2 bandwidth.
template <typename R>
__global__ void __launch_bounds__(kSweepThreads) k_sweep(SweepArgs<R> a) {
  const uint32_t lane = threadIdx.x & 31;
  const unsigned long long total = (unsigned long long)a.ctl->n_ge[a.current_level] * (unsigned long long)a.D;
  const unsigned long long capacity = (unsigned long long)a.D * a.Np;
  unsigned long long solved = 0;
  unsigned long long t0 = 0;
  uint32_t backoff = 32;
  bool stop = false;
  while (!stop) {
    // wait until the queue shows work beyond the claimed slots (or the sweep is done)
    int claim = 0;
    if (lane == 0) {
      const unsigned long long head = ld_relaxed64(&a.ctl->head);
      if (head >= total) {
        claim = -1;
      } else if (ld_relaxed64(&a.ctl->tail) > head) {
        claim = 1;
      } else {
        const unsigned long long now = globaltimer_ns();
        if (t0 == 0) t0 = now;
        if (now - t0 > a.timeout_ns || *(volatile uint32_t*)&a.ctl->error != 0) claim = -2;
      }
    }
    claim = __shfl_sync(0xffffffffu, claim, 0);
    if (claim == -1) break;
    if (claim == -2) {
      if (lane == 0) atomicOr(&a.ctl->error, kErrStall);
      break;
    }
    if (claim == 0) {
      __nanosleep(backoff);
      backoff = min(backoff * 2, 2048u);
      continue;
    }
    backoff = 32;
    t0 = 0;
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(&a.ctl->head, 32ull);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= total) break;
    const unsigned long long slot = base + lane;
    bool waiting = slot < total;
    uint32_t t = kEmptySlot;
    unsigned long long w0 = 0;
    uint32_t wait_ns = 32;
    while (__any_sync(0xffffffffu, waiting)) {
      bool got = false;
      if (waiting) {
        t = ld_relaxed(a.queue + slot);
        got = t != kEmptySlot;
      }
      if (__any_sync(0xffffffffu, got)) {
        solve_task<R>(a, got, t, capacity);
        if (got) {
          a.queue[slot] = kEmptySlot;  // leave the queue clean for the next sweep
          waiting = false;
          ++solved;
        }
        w0 = 0;
        wait_ns = 32;
      } else {
        int expired = 0;
        if (lane == 0) {
          const unsigned long long now = globaltimer_ns();
          if (w0 == 0) w0 = now;
          expired = (now - w0 > a.timeout_ns) || (*(volatile uint32_t*)&a.ctl->error != 0);
        }
        if (__shfl_sync(0xffffffffu, expired, 0)) {
          if (lane == 0) atomicOr(&a.ctl->error, kErrStall);
          stop = true;
          break;
        }
        __nanosleep(wait_ns);
        wait_ns = min(wait_ns * 2, 1024u);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) solved += __shfl_xor_sync(0xffffffffu, solved, o);
  if (lane == 0 && solved) atomicAdd(&a.ctl->tasks, solved);
}

// ---------------------------------------------------------------------------
// Levelled schedule.  The dependency graph of every direction depends only on the
// geometry, so a topological order of all N*D tasks (Kahn levels: a task's level is
// the length of the longest upwind chain ending in it) is computed once per grid.
// It stays valid for any active subset: every dependency among active cells is also
// an edge of the full graph, so it goes from a lower level to a higher one.
// ---------------------------------------------------------------------------

// One Kahn round: release the downwind dependents of the tasks order[begin, end)
// (all cells active), appending the tasks that become free at ctl->tail and recording
// their level (round + 1) in task_level.
template <typename R>
__global__ void k_kahn_round(SweepArgs<R> a, uint32_t* order, uint32_t begin, uint32_t end,
                             unsigned long long capacity, uint16_t* task_level, uint32_t round) {
  const uint32_t nthreads = gridDim.x * blockDim.x;
  const uint32_t span = end - begin;
  const uint32_t iters = (span + nthreads - 1) / nthreads;
  for (uint32_t it = 0; it < iters; ++it) {
    const uint32_t i = begin + it * nthreads + blockIdx.x * blockDim.x + threadIdx.x;
    const bool have = i < end;
    uint32_t beg = 0, nf = 0, d = 0;
    double dx = 0, dy = 0, dz = 0;
    float fx = 0, fy = 0, fz = 0;
    if (have) {
      const uint32_t t = order[i];
      d = t / a.Np;
      const uint32_t c = t - d * a.Np;
      beg = a.off[c];
      nf = a.off[c + 1] - beg;
      fx = a.dir32[3 * d]; fy = a.dir32[3 * d + 1]; fz = a.dir32[3 * d + 2];
      dx = a.dir64[3 * d]; dy = a.dir64[3 * d + 1]; dz = a.dir64[3 * d + 2];
    }
    uint32_t maxf = nf;
    for (int o = 16; o > 0; o >>= 1) maxf = max(maxf, __shfl_xor_sync(0xffffffffu, maxf, o));
    for (uint32_t k = 0; k < maxf; ++k) {
      bool ready = false;
      uint32_t tn = 0;
      if (k < nf) {
        const uint32_t f = beg + k;
        const uint32_t nb = a.nbr[f];
        if ((nb >> kKindShift) == kKindLocal) {
          const float4 g = a.geo32[f];
          const float s = g.x * fx + g.y * fy + g.z * fz;
          if (face_sign(s, a.geo64 + f, dx, dy, dz, a.guard) > 0) {
            tn = d * a.Np + (nb & kNbrMask);
            const uint32_t shift = 8u * (tn & 3u);
            const uint32_t old = atomicSub(a.counters + (tn >> 2), 1u << shift);
            ready = ((old >> shift) & 0xffu) == 1u;
            if (ready) task_level[tn] = (uint16_t)(round + 1);
          }
        }
      }
      enqueue(ready, tn, a.ctl, order, capacity);
    }
  }
}

constexpr int kGroup = 8;                   // lanes per task in the scheduled sweep
constexpr int kGroupsPerWarp = 32 / kGroup;
constexpr int kLevelThreads = 256;
constexpr int kLevelWarps = kLevelThreads / 32;

// Solve one task per group of kGroup lanes (Sweep::solve_task, src/sweep/mod.rs:423-485):
// lane j of the group handles faces j, j + kGroup, ...; the group leader handles the
// cell's rates.  The FP64 total downwind area is summed by the leader in face order
// from shared memory, as the reference sums it; the FP32 one by a group reduction.
// The correction goes to the downwind neighbours' incoming rates (LOCAL) or pending
// periodic sources (LOCAL_PERIODIC); each LOCAL neighbour's dependency counter is then
// decremented with release semantics.
template <typename R>
__device__ __forceinline__ void solve_group(const SweepArgs<R>& a, bool have, uint32_t t, R* eff_stage) {
  const bool fp64 = sizeof(R) == 8;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t gl = lane & (kGroup - 1);
  uint32_t c = 0, d = 0, beg = 0, nf = 0;
  if (have) {
    d = t / a.Np;
    c = t - d * a.Np;
    if (gl == 0) {
      beg = a.off[c];
      nf = a.off[c + 1] - beg;
    }
  }
  beg = __shfl_sync(0xffffffffu, beg, 0, kGroup);
  nf = __shfl_sync(0xffffffffu, nf, 0, kGroup);
  double dx = 0, dy = 0, dz = 0;
  float fx = 0, fy = 0, fz = 0;
  R inc = R(0), per = R(0), outo = R(0), src = R(0);
  double att = 0.0;
  if (have) {
    fx = a.dir32[3 * d]; fy = a.dir32[3 * d + 1]; fz = a.dir32[3 * d + 2];
    dx = a.dir64[3 * d]; dy = a.dir64[3 * d + 1]; dz = a.dir64[3 * d + 2];
    if (gl == 0) {
      inc = __ldcg(a.incoming + t);
      per = __ldcg(a.periodic + t);
      outo = a.outgoing[t];
      att = a.att[c];
      src = a.src_dir[c];
    }
  }
  uint32_t rounds = (nf + kGroup - 1) / kGroup;
  for (int o = 16; o > 0; o >>= 1) rounds = max(rounds, __shfl_xor_sync(0xffffffffu, rounds, o));
  // phase 1: classify this lane's faces, effective areas of the downwind ones
  uint32_t down = 0;
  R part = R(0);
  for (uint32_t k = 0; k < rounds; ++k) {
    const uint32_t fl = gl + k * kGroup;
    if (fl < nf) {
      const uint32_t f = beg + fl;
      const float4 g = a.geo32[f];
      const float s = g.x * fx + g.y * fy + g.z * fz;
      R eff = R(0);
      if (face_sign(s, a.geo64 + f, dx, dy, dz, a.guard) > 0) {
        down |= 1u << k;
        if (fp64) {
          const Geo64 h = a.geo64[f];
          eff = R(h.w * dot64(h, dx, dy, dz));
        } else {
          eff = R(g.w * s);
        }
      }
      if (fp64) eff_stage[fl] = eff; else part += eff;
    }
  }
  R total;
  if (fp64) {
    __syncwarp();
    total = R(0);
    if (gl == 0)
      for (uint32_t fl = 0; fl < nf; ++fl) total += eff_stage[fl];  // face order, zeros for others
    total = __shfl_sync(0xffffffffu, total, 0, kGroup);
  } else {
    part += __shfl_xor_sync(0xffffffffu, part, 1, kGroup);
    part += __shfl_xor_sync(0xffffffffu, part, 2, kGroup);
    part += __shfl_xor_sync(0xffffffffu, part, 4, kGroup);
    total = part;
  }
  // outgoing rate and correction (leader), broadcast to the group
  R corr = R(0);
  if (have && gl == 0) {
    if (inc < R(0)) {  // Photons::make_positive (chemistry/mod.rs:61-65)
      inc = R(0);
      a.incoming[t] = inc;
    }
    const R r = (inc + src) + per;  // Site::get_rate, site.rs:53-56
    const R out_new = (r < a.threshold) ? R(0) : r * R(att);
    corr = out_new - outo;
    a.outgoing[t] = out_new;
  }
  corr = __shfl_sync(0xffffffffu, corr, 0, kGroup);
  // phase 2: distribute the correction over the downwind faces
  for (uint32_t k = 0; k < rounds; ++k) {
    if (!((down >> k) & 1u)) continue;
    const uint32_t fl = gl + k * kGroup;
    const uint32_t f = beg + fl;
    const uint32_t nb = a.nbr[f];
    const uint32_t kind = nb >> kKindShift;
    if (kind == kKindBoundary) continue;
    R eff;
    if (fp64) {
      eff = eff_stage[fl];
    } else {
      const float4 g = a.geo32[f];
      eff = R(g.w * (g.x * fx + g.y * fy + g.z * fz));
    }
    const R w = corr * (eff / total);
    const uint32_t tn = d * a.Np + (nb & kNbrMask);
    if (kind == kKindPeriodic) {
      atomicAdd(a.pending + tn, w);
    } else {
      atomicAdd(a.incoming + tn, w);
      atom_sub_release(a.counters + (tn >> 2), 1u << (8u * (tn & 3u)));
    }
  }
  __syncwarp();
}

// The scheduled transport kernel (cooperative launch: all blocks resident).  Group g
// solves schedule positions g, g + G, g + 2G, ... of the levelled order, each as soon
// as its dependency counter reads zero; inactive cells' tasks are skipped.  Every
// dependency points to an earlier position, and every group walks its positions in
// increasing order, so the earliest unsolved task can always proceed.  There are no
// barriers and no queue atomics; a group waits only for its own task's upwind
// neighbours, with exponential backoff and a globaltimer limit.  The counter is read
// with a relaxed load and the task's rates are read only after it reads zero (a control
// dependency); the producers' rate additions precede their release decrements.
template <typename R>
__global__ void __launch_bounds__(kLevelThreads) k_sweep_sched(SweepArgs<R> a, const uint32_t* order,
                                                                uint32_t total_sched) {
  __shared__ R eff_stage[kLevelWarps * kGroupsPerWarp][sizeof(R) == 8 ? kMaxFaces : 1];
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t gl = lane & (kGroup - 1);
  R* stage = eff_stage[(threadIdx.x >> 5) * kGroupsPerWarp + (lane / kGroup)];
  const uint32_t groups = gridDim.x * (kLevelThreads / kGroup);
  uint32_t i = blockIdx.x * (kLevelThreads / kGroup) + (threadIdx.x / kGroup);
  const uint8_t* cnt8 = reinterpret_cast<const uint8_t*>(a.counters);
  unsigned long long solved = 0;
  bool stop = false;
  while (!stop && __any_sync(0xffffffffu, i < total_sched)) {
    bool pending = false;
    uint32_t t = 0;
    if (i < total_sched) {
      t = order[i];
      const uint32_t c = t - (t / a.Np) * a.Np;
      pending = a.level[c] >= a.current_level;
    }
    unsigned long long w0 = 0;
    uint32_t wait_ns = 32;
    while (__any_sync(0xffffffffu, pending)) {
      bool ready = false;
      if (pending && gl == 0) {
        uint32_t v;
        asm volatile("ld.relaxed.gpu.global.u8 %0, [%1];" : "=r"(v) : "l"(cnt8 + t) : "memory");
        ready = (v & 0xffu) == 0u;
      }
      ready = __shfl_sync(0xffffffffu, ready ? 1 : 0, 0, kGroup) != 0;
      if (__any_sync(0xffffffffu, ready)) {
        solve_group<R>(a, ready, t, stage);
        if (ready) {
          pending = false;
          if (gl == 0) ++solved;
        }
        w0 = 0;
        wait_ns = 32;
      } else {
        int expired = 0;
        if (lane == 0) {
          const unsigned long long now = globaltimer_ns();
          if (w0 == 0) w0 = now;
          expired = (now - w0 > a.timeout_ns) || (*(volatile uint32_t*)&a.ctl->error != 0);
        }
        if (__shfl_sync(0xffffffffu, expired, 0)) {
          if (lane == 0) atomicOr(&a.ctl->error, kErrStall);
          stop = true;
          break;
        }
        __nanosleep(wait_ns);
        wait_ns = min(wait_ns * 2, 512u);
      }
    }
    i += groups;
  }
  for (int o = 16; o > 0; o >>= 1) solved += __shfl_xor_sync(0xffffffffu, solved, o);
  if (lane == 0 && solved) atomicAdd(&a.ctl->tasks, solved);
}

// Snapshot semantics of periodic sources: contributions written through periodic
// faces during a level sweep are added to periodic_source after the transport, so
// transport reads the previous sweeps' contributions and the chemistry all of them.
template <typename R>
__global__ void k_fold_periodic(R* periodic, R* pending, const uint32_t* cells, uint32_t n_cells, int D,
                                uint32_t Np) {
  const size_t totalw = (size_t)n_cells * D;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < totalw; i += (size_t)gridDim.x * blockDim.x) {
    const size_t idx = (size_t)(i / n_cells) * Np + cells[i % n_cells];
    const R p = pending[idx];
    if (p != R(0)) {
      periodic[idx] += p;
      pending[idx] = R(0);
    }
  }
}

// Per-cell attenuation factor exp(-n_HI sigma size) of HydrogenOnly::get_outgoing_rate
// (hydrogen_only/mod.rs:72-88); direction-independent, so computed once per cell.
template <bool kCarryNeutral>
__global__ void k_attenuation(uint32_t n, const uint8_t* level, int current_level, const double* density,
                              const double* xhii, const double* yneu, const double* size, double* att,
                              uint32_t* cell_sweep, const uint32_t* epoch_base, uint32_t epoch, uint2* cellpack,
                              const float* src32) {
  // pull path: the number of the sweep that solves each active cell, and per cell the
  // pair {(float) attenuation, source / D} (attenuation 0xffffffff: inactive)
  const uint32_t sweep = cell_sweep ? (epoch_base ? *epoch_base + epoch : epoch) : 0u;
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    if (level[c] < current_level) {
      if (cellpack) cellpack[c] = make_uint2(0xffffffffu, 0u);
      continue;
    }
    if (cell_sweep) cell_sweep[c] = sweep;
    const double neutral = kCarryNeutral ? yneu[c] : (1.0 - xhii[c]);
    const double nhn = density[c] / Units::kProtonMass * neutral;
    const double at = exp(-nhn * Units::kSigma * size[c]);
    att[c] = at;
    if (cellpack) cellpack[c] = make_uint2(__float_as_uint((float)at), __float_as_uint(src32[c]));
  }
}

template <typename R>
struct ChemArgs {
  uint32_t n;
  SweepCtl* ctl;
  int current_level;
  int D;
  uint32_t Np;
  const R* incoming;           // incoming rate of task t at incoming[t]
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
  double rate_floor;       // mixed path: rates below it count as below the threshold (0: FP64)
  double safety;
  double scale_factor;
  int prevent_cooling;
};

// Sweep::update_chemistry (src/sweep/mod.rs:549-574) + HydrogenOnly::update_abundances
// (hydrogen_only/mod.rs:90-119), one thread per cell (inactive cells skip).
template <typename R, bool kCarryNeutral>
__global__ void k_chemistry(ChemArgs<R> a) {
  uint32_t attempts = 0, failures = 0, cells = 0, invalid = 0;
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < a.n; c += gridDim.x * blockDim.x) {
    if (a.level[c] < a.current_level) continue;
    const double timestep = ldexp(a.max_timestep, -(int)a.level[c]);  // timestep_level.rs:42-48
    double rate;
    if (sizeof(R) == 8) {
      const double src = a.source[c] / (double)a.D;
      rate = 0.0;  // sum over directions of Site::get_rate, in direction order
      for (int d = 0; d < a.D; ++d) {
        const size_t t = (size_t)d * a.Np + c;
        rate += ((double)a.incoming[t] + src) + (double)a.periodic[t];
      }
    } else {
      // compensated FP32 sum of the scaled transported rates in direction order, the
      // source added in FP64; the rates are loaded eight directions at a time
      constexpr int kBatch = 8;
      float s = 0.f, comp = 0.f;
      for (int d0 = 0; d0 < a.D; d0 += kBatch) {
        float v[kBatch];
#pragma unroll
        for (int j = 0; j < kBatch; ++j) {
          const size_t t = (size_t)(d0 + j) * a.Np + c;
          v[j] = d0 + j < a.D ? (float)a.incoming[t] + (float)a.periodic[t] : 0.f;
        }
#pragma unroll
        for (int j = 0; j < kBatch; ++j) {
          if (d0 + j >= a.D) break;
          const float yv = v[j] - comp;
          const float tt = s + yv;
          comp = (tt - s) - yv;
          s = tt;
        }
      }
      rate = (double)s * a.rate_scale + a.source[c];
    }
    double relative_change;
    // chemistry/mod.rs:79-81.  The mixed path also treats a rate below the smallest
    // value its FP32 transport carries at full precision as insignificant: there the
    // FP64 path sees a smooth exponential tail, FP32 an underflowed zero, and the
    // reference's relative change of a zero rate (0/0, capped at 1/epsilon) would send
    // the cell to the deepest level.
    if (fabs(rate) < fabs(a.threshold) || fabs(rate) < a.rate_floor) {
      relative_change = 0.0;
    } else {  // chemistry/mod.rs:73-77
      relative_change = fabs(fmin(fabs(fabs(rate - a.previous_rate[c]) / rate), 1.0 / DBL_EPSILON));
    }
    a.previous_rate[c] = rate;
    const Timescale rate_ts{timestep / relative_change, kProcPhotonRate};
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
    s.prepare();
    bool failed = false;
    const Timescale chem_ts = s.perform_timestep(timestep, a.safety, failed, attempts);
    failures += failed ? 1u : 0u;
    invalid |= s.clamp_invalid ? 1u : 0u;
    a.temperature[c] = s.temperature;
    a.xhii[c] = s.x;
    if (kCarryNeutral) a.yneu[c] = s.y;
    a.species_timestep[c] = chem_ts.time;
    a.change_timescale[c] = ts_min(rate_ts, chem_ts).time;
    ++cells;
  }
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
  const double ratio = max_timestep / desired;
  long long level;
  if (isnan(ratio) || ratio <= 1.0) {
    level = 0;  // log2 <= 0, NaN -> 0
  } else if (isinf(ratio)) {
    level = num_levels - 1;
  } else {
    int e;
    const double m = frexp(ratio, &e);
    level = (m == 0.5) ? (e - 1) : e;
  }
  if (level > num_levels - 1) level = num_levels - 1;
  if (level < lowest) level = lowest;
  return (int)level;
}

// Sweep::update_timestep_levels (src/sweep/mod.rs:576-589) for all cells, plus the
// level histogram.
static __global__ void k_update_levels(uint32_t n, const double* change_timescale, uint8_t* level, double safety,
                                       double max_timestep, int num_levels, int lowest, SweepCtl* ctl) {
  __shared__ uint32_t hist[32];
  if (threadIdx.x < 32) hist[threadIdx.x] = 0;
  __syncthreads();
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    const int l = desired_level(max_timestep, safety * change_timescale[c], num_levels, lowest);
    level[c] = (uint8_t)l;
    atomicAdd(&hist[l], 1u);
  }
  __syncthreads();
  if (threadIdx.x < num_levels && hist[threadIdx.x]) atomicAdd(&ctl->hist[threadIdx.x], hist[threadIdx.x]);
}

// Histogram of the current levels (used at creation).
static __global__ void k_level_hist(uint32_t n, const uint8_t* level, int num_levels, SweepCtl* ctl) {
  __shared__ uint32_t hist[32];
  if (threadIdx.x < 32) hist[threadIdx.x] = 0;
  __syncthreads();
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x)
    atomicAdd(&hist[level[c]], 1u);
  __syncthreads();
  if (threadIdx.x < num_levels && hist[threadIdx.x]) atomicAdd(&ctl->hist[threadIdx.x], hist[threadIdx.x]);
}

// n_ge[l] = #cells with level >= l, from the histogram (which is then cleared).
static __global__ void k_level_counts(SweepCtl* ctl, int num_levels) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    uint32_t acc = 0;
    for (int l = num_levels - 1; l >= 0; --l) {
      acc += ctl->hist[l];
      ctl->n_ge[l] = acc;
    }
    for (int l = 0; l < 32; ++l) ctl->hist[l] = 0;
  }
}

// IonizationTime write-back of run_sweep_system (src/sweep/mod.rs:731-738).
static __global__ void k_ionization_time(uint32_t n, const double* xhii, double* ionization_time, double time,
                                         const double* time_dev) {
  if (time_dev) time = *time_dev;
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x)
    if (xhii[c] > 0.5 && isinf(ionization_time[c])) ionization_time[c] = time;
}

// PhotonRate = sum over directions of the incoming rate (src/sweep/mod.rs:727-730).
template <typename R>
__global__ void k_photon_rate(uint32_t n, const R* incoming, int D, uint32_t Np, double rate_scale, double* out) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    double r = 0.0;
    for (int d = 0; d < D; ++d) r += (double)incoming[(size_t)d * Np + c];
    out[c] = r * rate_scale;
  }
}

// Rate of every cell summed over directions as Sweep::get_solver forms it
// (src/sweep/mod.rs:616-620): sum over d of get_rate(d) = (incoming + source/D) +
// periodic (site.rs:53-56), in photons/s.
template <typename R>
__global__ void k_cell_rates(uint32_t n, const R* incoming, const R* periodic, const R* src_dir, int D, uint32_t Np,
                             double rate_scale, double* out) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    double r = 0.0;
    for (int d = 0; d < D; ++d) {
      const size_t t = (size_t)d * Np + c;
      r += ((double)incoming[t] + (double)src_dir[c]) + (double)periodic[t];
    }
    out[c] = r * rate_scale;
  }
}

// Time series of the sweep (src/sweep/time_series.rs:61-155), two stages with a fixed
// grid so the sums are deterministic: per-block partial sums of
//   [0] mass * x, [1] mass, [2] volume * x, [3] volume, [4] T * mass, [5] T * volume,
//   [6] Gamma * volume, [7] Gamma * x * volume,
// with mass = density * volume (main.rs:195-203) and Gamma the photoionization rate
// over one year of the cell's solver (chemistry_output.rs:15-28, hydrogen_only/mod.rs
// 312-332), then the ratios.  `yneu`, when given, is the carried neutral fraction.
constexpr int kSeriesThreads = 256;
constexpr int kSeriesBlocks = 256;
constexpr int kSeriesSums = 8;

static __global__ void __launch_bounds__(kSeriesThreads) k_time_series_partial(
    uint32_t n, const double* density, const double* volume, const double* size, const double* xhii,
    const double* yneu, const double* temperature, const double* cell_rate, double* partial) {
  const double year = 3.15576e7;  // units/mod.rs: one year in seconds
  double acc[kSeriesSums] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    const double x = xhii[c], v = volume[c], t = temperature[c];
    const double mass = density[c] * v;
    const double neutral = yneu ? yneu[c] : 1.0 - x;
    const double nhn = density[c] / Units::kProtonMass * neutral;
    const double absorbed = 1.0 - exp(-nhn * Units::kSigma * size[c]);
    const double num = (year * cell_rate[c]) * absorbed;
    const double gamma = (num / (nhn * v)) / year;
    acc[0] += mass * x;
    acc[1] += mass;
    acc[2] += v * x;
    acc[3] += v;
    acc[4] += t * mass;
    acc[5] += t * v;
    acc[6] += gamma * v;
    acc[7] += gamma * x * v;
  }
  __shared__ double sh[kSeriesSums][kSeriesThreads];
  for (int k = 0; k < kSeriesSums; ++k) sh[k][threadIdx.x] = acc[k];
  __syncthreads();
  for (int stride = kSeriesThreads / 2; stride > 0; stride >>= 1) {
    if ((int)threadIdx.x < stride)
      for (int k = 0; k < kSeriesSums; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + stride];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < kSeriesSums; ++k) partial[blockIdx.x * kSeriesSums + k] = sh[k][0];
}

static __global__ void k_time_series_final(const double* partial, int blocks, double* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s[kSeriesSums] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int b = 0; b < blocks; ++b)
    for (int k = 0; k < kSeriesSums; ++k) s[k] += partial[b * kSeriesSums + k];
  out[0] = s[0] / s[1];
  out[1] = s[2] / s[3];
  out[2] = s[4] / s[1];
  out[3] = s[5] / s[3];
  out[4] = s[6] / s[3];
  out[5] = s[7] / s[3];
}

// Convert a per-task array to FP64 photons/s in [cell][D] layout.
template <typename R>
__global__ void k_export_rates(uint32_t n, const R* src, int D, uint32_t Np, double rate_scale, double* out) {
  const size_t total = (size_t)n * D;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const size_t c = i / D, d = i % D;
    out[i] = (double)src[d * (size_t)Np + c] * rate_scale;
  }
}

}  // namespace swk
