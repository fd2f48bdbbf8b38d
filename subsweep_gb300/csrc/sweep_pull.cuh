// Pull-form transport of the mixed-precision path (FP32 rates).
//
// The reference distributes each task's outgoing-rate *correction* over its downwind
// faces (push, src/sweep/mod.rs:423-485).  Summed over a sweep's history, the incoming
// rate of (cell c, direction d) is the sum over c's upwind LOCAL faces f (neighbour n)
// of  area_f |n_f . d| * out(n, d) / A(n, d),  where A(n, d) is n's total effective
// downwind area.  This path evaluates that sum directly: every task publishes
//   q(c, d) = out(c, d) / A(c, d)
// together with the number of the sweep that produced it, as one 64-bit word
// {q bits, sweep << 1 | stamped}, and a task gathers q from its upwind neighbours once
// every active one's word carries the current sweep number; an inactive neighbour keeps
// the q of its last solve (its flux persists, as in the reference).  In a sweep above
// level 0 over all positions the tasks of inactive cells stamp their words with the
// sweep number (stamped bit set); over a compacted list of the active positions the
// consumer tests the neighbour's level instead.  The word is
// written and read in single 64-bit accesses, so there are no atomics, no counters and
// no fences on this path.  Tasks are visited in the levelled schedule order, every
// upwind task lies at an earlier schedule position, and a task whose inputs are not
// all published yet is retried.
//
// Geometry is one 16-byte load per face: {area * n (FP32, area scaled by 2^-k),
// neighbour | kind << 30}.  The sign of n . d decides up/downwind exactly: the FP32 dot
// decides when it exceeds its rounding bound, else the FP64 normal does.  The sweep
// itself reads precomputed per-position records and upwind slots.
//
// The path's kernels: records, upwind slots and the compaction of active positions in
// sweep_pull_setup.cuh; the warp-lockstep sweep kernels in sweep_pull_lockstep.cuh; the
// level-synchronous (wavefront) ones in sweep_pull_wavefront.cuh; the periodic fold and
// the field export in sweep_pull_fold.cuh.
#pragma once

#include <cuda/atomic>

#include "sweep_device.cuh"

namespace swk {

struct PullArgs {
  const uint32_t* off;
  const uint4* geo16;       // {area*n (float bits) x3, nbr | kind << 30}
  const Geo64* geo64;
  const double* dir64;
  const float* dir32;
  int D;
  uint32_t Np;
  uint32_t N;
  const uint8_t* level;
  const float* src_dir;     // source / D per cell, stored rate units
  const double* att;
  float threshold;
  const float* periodic;
  // per schedule position p: the word {q (float bits) low, sweep number high} at qe[p];
  // per task t: its incoming rate at inc[t]
  unsigned long long* qe;
  float* inc;
  SweepCtl* ctl;
  int current_level;
  uint32_t epoch;
  unsigned long long timeout_ns;
  // sweep kernel
  const uint4* rec;           // per schedule position: {task, 1/A_down, slot offset lo, count | offset hi << 8}
  const uint2* slots;         // upwind LOCAL faces of every position: {cell, |area n . d| (FP32)}
  const uint32_t* act;        // compacted active positions, or nullptr: every position
  const uint32_t* act_count;  // device count of act (written by the compaction)
  uint32_t count;             // number of positions when act is nullptr
  const uint32_t* epoch_base; // graph replay: the sweep number is *epoch_base + epoch
  const uint32_t* cell_sweep; // number of the last sweep that solved each cell
  const uint32_t* lvl;        // schedule level offsets into the positions [num_sched + 1]
  uint32_t num_sched;         // schedule levels (0: no levelled schedule)
  // staged wavefront kernel
  const uint2* cellpack;      // per cell: {(float) attenuation bits or kInactiveCell, source / D bits}
  float* per_pos;             // periodic source of every position (written by the fold)
  // schedule position of every task, or null in the compact state, whose words are
  // indexed by task
  const uint32_t* pos_of_task;
  const uint32_t* order;      // compact state: the task at every schedule position
};

// cellpack.x of a cell that is not active in the sweep (no attenuation is computed)
constexpr uint32_t kInactiveCell = 0xffffffffu;

// the sweep number of a launch (a step replayed from a graph keeps its base on the device)
__device__ __forceinline__ uint32_t sweep_number(const PullArgs& a) {
  return a.epoch_base ? *a.epoch_base + a.epoch : a.epoch;
}

// The words are only ever read and written whole (relaxed, device scope), and nothing
// else is ordered against them inside a sweep.
using WordRef = cuda::atomic_ref<unsigned long long, cuda::thread_scope_device>;

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
  return WordRef(*const_cast<unsigned long long*>(p)).load(cuda::memory_order_relaxed);
}

__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v) {
  WordRef(*p).store(v, cuda::memory_order_relaxed);
}

// Position p's word (8 bytes, four to a 32-byte sector, so neighbouring tasks' upwind
// words share sectors).  The incoming rates are kept apart, by task: a sweep reads only
// words, and the incoming rates are read after the sweep (chemistry, periodic fold,
// export), the chemistry's per-cell sum over directions in coalesced rows.  A commit
// writes the word with one relaxed device-scope store, so readers see the old or the
// new word whole.
__device__ __forceinline__ unsigned long long* word_ptr(unsigned long long* qe, size_t p) { return qe + p; }
__device__ __forceinline__ const unsigned long long* word_ptr(const unsigned long long* qe, size_t p) {
  return qe + p;
}

// {q, sweep << 1}: solved in `sweep`; {q, sweep << 1 | 1}: stamped (inactive in `sweep`)
__device__ __forceinline__ unsigned long long pack_qe(float q, uint32_t sweep) {
  return ((unsigned long long)(sweep << 1) << 32) | (unsigned long long)__float_as_uint(q);
}
__device__ __forceinline__ bool word_current(unsigned long long w, uint32_t sweep) {
  return (uint32_t)(w >> 33) == sweep;
}

// Signed effective area s = (area n) . d of one face, with the exact sign of n . d:
// returns +|s| downwind, -|s| upwind, 0 when n . d == 0.
__device__ __forceinline__ float face_eff(const uint4& g, float fx, float fy, float fz, const Geo64* g64,
                                          double dx, double dy, double dz) {
  // explicit roundings: every kernel that classifies a face gets the same answer
  const float ax = __uint_as_float(g.x), ay = __uint_as_float(g.y), az = __uint_as_float(g.z);
  const float s = __fmaf_rn(az, fz, __fmaf_rn(ay, fy, __fmul_rn(ax, fx)));
  const float bound =
      __fmul_rn(8.0e-7f, __fadd_rn(__fadd_rn(fabsf(__fmul_rn(ax, fx)), fabsf(__fmul_rn(ay, fy))), fabsf(__fmul_rn(az, fz))));
  if (s > bound) return s;
  if (s < -bound) return s;
  const double e = dot64(*g64, dx, dy, dz);
  if (e > 0.0) return fabsf(s);
  if (e < 0.0) return -fabsf(s);
  return 0.0f;
}

constexpr int kPullThreads = 256;
constexpr int kPullPartials = 8;   // partial sums of a task's incoming rate (slot j into partial j mod 8)
constexpr int kPullRegSlots = 16;  // upwind slots a task holds in registers (more are read from memory)

// t = d * Np + c  ->  (c, d) without a runtime integer division: FP32 estimate of the
// quotient (t / Np <= 128, so it is off by at most one), then an exact correction.
__device__ __forceinline__ void split_task(uint32_t t, uint32_t Np, float inv_np, uint32_t& c, uint32_t& d) {
  int q = (int)(__uint2float_rn(t) * inv_np);
  long long r = (long long)t - (long long)q * Np;
  if (r < 0) { --q; r += Np; }
  if (r >= (long long)Np) { ++q; r -= Np; }
  d = (uint32_t)q;
  c = (uint32_t)r;
}

// record word w: upwind count (7 bits) | direction << 7 (7 bits) | slot offset >> 32 << 14
// (17 bits) | 1 << 31 when an upwind face of the task is LOCAL_PERIODIC (its periodic
// source can be non-zero; every other task's stays 0)
constexpr uint32_t kRecPeriodic = 1u << 31;
__device__ __forceinline__ unsigned long long rec_offset(const uint4& r) {
  return (unsigned long long)r.z | ((unsigned long long)((r.w >> 14) & 0x1ffffu) << 32);
}
__device__ __forceinline__ uint32_t rec_count(const uint4& r) { return r.w & 0x7fu; }
__device__ __forceinline__ uint32_t rec_dir(const uint4& r) { return (r.w >> 7) & 0x7fu; }
__device__ __forceinline__ bool rec_periodic(const uint4& r) { return (r.w & kRecPeriodic) != 0u; }

// index of task t's word: its schedule position, or t in the compact state
__device__ __forceinline__ size_t word_of_task(const PullArgs& a, size_t t) {
  return a.pos_of_task ? (size_t)a.pos_of_task[t] : t;
}

// commit of the task with record r at position p
__device__ __forceinline__ void commit_slot(const PullArgs& a, size_t p, const uint4& r, unsigned long long word,
                                            float in) {
  a.inc[(size_t)rec_dir(r) * a.Np + r.x] = in;
  st_relaxed_u64(a.qe + p, word);
}

}  // namespace swk
