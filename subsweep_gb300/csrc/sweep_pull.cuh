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
// itself reads precomputed per-position records and upwind slots (below).
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
  // per task t, 16 bytes at qe + 2 t: the word {q (float bits) low, sweep number high}
  // and the task's incoming rate (float bits, low half of the second 8 bytes)
  unsigned long long* qe;
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
  const uint32_t* pos_of_task;
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

// predicated form: returns 0 without touching memory when pred is false
__device__ __forceinline__ unsigned long long ld_relaxed_u64_if(bool pred, const unsigned long long* p) {
  return pred ? ld_relaxed_u64(p) : 0ull;
}

__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v) {
  WordRef(*p).store(v, cuda::memory_order_relaxed);
}

// Task t's slot: its word, and beside it its incoming rate.  A commit writes both with
// one 16-byte store; each 8-byte element of a vector access is single-copy atomic, so
// readers of the word see either the old or the new word whole.
__device__ __forceinline__ unsigned long long* word_ptr(unsigned long long* qe, size_t t) { return qe + 2 * t; }
__device__ __forceinline__ const unsigned long long* word_ptr(const unsigned long long* qe, size_t t) {
  return qe + 2 * t;
}
__device__ __forceinline__ float stored_incoming(const unsigned long long* qe, size_t t) {
  return __uint_as_float((uint32_t)qe[2 * t + 1]);
}
__device__ __forceinline__ void commit_slot(unsigned long long* qe, size_t t, unsigned long long word, float in) {
  asm volatile("st.relaxed.gpu.global.v2.u64 [%0], {%1, %2};" ::"l"(qe + 2 * t), "l"(word),
               "l"((unsigned long long)__float_as_uint(in))
               : "memory");
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
constexpr int kPullGroup = 8;   // lanes per task
constexpr int kPullRounds = 2;  // slots per lane held in registers (tasks with <= 16 upwind faces)

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

// ---------------------------------------------------------------------------------------
// Task records and upwind slots, built once per grid from the schedule (geometry only).
// Position p of the schedule (task t = order[p] = d * Np + c) gets
//   rec[p]   = {c, bits of 1 / A_down (FP32; 0 when no face is downwind),
//               slot offset (low 32 bits), upwind count | d << 7 | offset >> 32 << 14
//               | kRecPeriodic}
//   slots[offset + k] = {upwind task d * Np + n, |area n . d| in FP32}, k < count,
// for the upwind LOCAL faces of c in face order (exact sign of n . d).  A_down is
// summed in face order.  Counts, a chunked 64-bit exclusive scan, then the writes.

__device__ __forceinline__ void classify_task(const PullArgs& a, uint32_t t, float inv_np, uint32_t& c,
                                              uint32_t& d, uint32_t& beg, uint32_t& nf) {
  split_task(t, a.Np, inv_np, c, d);
  beg = a.off[c];
  nf = a.off[c + 1] - beg;
}

__global__ void k_pull_rec_count(PullArgs a, const uint32_t* order, uint32_t total, uint4* rec) {
  const float inv_np = 1.0f / (float)a.Np;
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < total; p += gridDim.x * blockDim.x) {
    const uint32_t t = order[p];
    uint32_t c, d, beg, nf;
    classify_task(a, t, inv_np, c, d, beg, nf);
    const float fx = a.dir32[3 * d], fy = a.dir32[3 * d + 1], fz = a.dir32[3 * d + 2];
    const double dx = a.dir64[3 * d], dy = a.dir64[3 * d + 1], dz = a.dir64[3 * d + 2];
    float area_down = 0.f;
    uint32_t n_up = 0, periodic_up = 0;
    for (uint32_t j = 0; j < nf; ++j) {
      const uint4 g = a.geo16[beg + j];
      const float sj = face_eff(g, fx, fy, fz, a.geo64 + beg + j, dx, dy, dz);
      if (sj > 0.f) area_down += sj;
      else if (sj < 0.f && (g.w >> kKindShift) == kKindLocal) ++n_up;
      else if (sj < 0.f && (g.w >> kKindShift) == kKindPeriodic) periodic_up = kRecPeriodic;
    }
    const float inv = area_down > 0.f ? 1.0f / area_down : 0.f;
    rec[p] = make_uint4(c, __float_as_uint(inv), 0u, n_up | (d << 7) | periodic_up);
  }
}

// per chunk of kCompactChunk positions: total upwind count
__global__ void __launch_bounds__(kCompactThreads) k_pull_slot_chunks(const uint4* rec, uint32_t total,
                                                                      uint32_t* chunk) {
  const uint32_t first = blockIdx.x * kCompactChunk + threadIdx.x * kCompactPer;
  uint32_t n = 0;
  for (int k = 0; k < kCompactPer; ++k)
    if (first + k < total) n += rec_count(rec[first + k]);
  for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
  __shared__ uint32_t ws[kCompactThreads / 32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = n;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t s = 0;
    for (int w = 0; w < kCompactThreads / 32; ++w) s += ws[w];
    chunk[blockIdx.x] = s;
  }
}

// exclusive 64-bit scan of the chunk totals (one block); the grand total at out[n]
constexpr int kScanThreads = 1024;
__global__ void __launch_bounds__(kScanThreads) k_scan_chunks64(const uint32_t* chunk, uint32_t n,
                                                                unsigned long long* out) {
  __shared__ unsigned long long warp_sum[kScanThreads / 32];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long carry = 0;
  for (uint32_t base = 0; base < n; base += kScanThreads) {
    const uint32_t i = base + threadIdx.x;
    const unsigned long long v = i < n ? chunk[i] : 0ull;
    unsigned long long x = v;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) warp_sum[warp] = x;
    __syncthreads();
    unsigned long long wbase = 0, tot = 0;
    for (int w = 0; w < kScanThreads / 32; ++w) {
      const unsigned long long s = warp_sum[w];
      if ((uint32_t)w < warp) wbase += s;
      tot += s;
    }
    if (i < n) out[i] = carry + wbase + x - v;
    carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) out[n] = carry;
}

// Writes at most the counted number of slots per position; a classification that
// disagrees with the count flags kErrRecords.
__global__ void __launch_bounds__(kCompactThreads) k_pull_slots(PullArgs a, uint4* rec, uint32_t total,
                                                                const unsigned long long* chunk_off,
                                                                uint2* slots) {
  const uint32_t first = blockIdx.x * kCompactChunk + threadIdx.x * kCompactPer;
  uint32_t mine = 0;
  for (int k = 0; k < kCompactPer; ++k)
    if (first + k < total) mine += rec_count(rec[first + k]);
  // block-exclusive prefix of the per-thread totals
  __shared__ uint32_t ws[kCompactThreads / 32];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = mine;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) ws[warp] = x;
  __syncthreads();
  uint32_t wbase = 0;
  for (uint32_t w = 0; w < warp; ++w) wbase += ws[w];
  unsigned long long o = chunk_off[blockIdx.x] + wbase + x - mine;
  for (int k = 0; k < kCompactPer; ++k) {
    const uint32_t p = first + k;
    if (p >= total) break;
    uint4 r = rec[p];
    const uint32_t n_up = rec_count(r);
    const uint32_t c = r.x, d = rec_dir(r);
    r.z = (uint32_t)o;
    r.w = n_up | (d << 7) | ((uint32_t)(o >> 32) << 14) | (r.w & kRecPeriodic);
    rec[p] = r;
    const uint32_t beg = a.off[c], nf = a.off[c + 1] - beg;
    const uint32_t dnp = d * a.Np;
    const float fx = a.dir32[3 * d], fy = a.dir32[3 * d + 1], fz = a.dir32[3 * d + 2];
    const double dx = a.dir64[3 * d], dy = a.dir64[3 * d + 1], dz = a.dir64[3 * d + 2];
    uint32_t written = 0;
    for (uint32_t j = 0; j < nf; ++j) {
      const uint4 g = a.geo16[beg + j];
      if ((g.w >> kKindShift) != kKindLocal) continue;
      const float sj = face_eff(g, fx, fy, fz, a.geo64 + beg + j, dx, dy, dz);
      if (sj < 0.f) {
        if (written < n_up) slots[o + written] = make_uint2(dnp + (g.w & kNbrMask), __float_as_uint(-sj));
        ++written;
      }
    }
    if (written != n_up) atomicOr(&a.ctl->error, kErrRecords);
    o += n_up;
  }
}

// ---------------------------------------------------------------------------------------
// exclusive scan of the chunk counts in place (one block); the total goes to *count
__global__ void __launch_bounds__(kScanThreads) k_compact_scan(uint32_t* chunk, uint32_t n, uint32_t* count) {
  __shared__ uint32_t warp_sum[kScanThreads / 32];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t carry = 0;
  for (uint32_t base = 0; base < n; base += kScanThreads) {
    const uint32_t i = base + threadIdx.x;
    const uint32_t v = i < n ? chunk[i] : 0u;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) warp_sum[warp] = x;
    __syncthreads();
    uint32_t wbase = 0, total = 0;
    for (int w = 0; w < kScanThreads / 32; ++w) {
      const uint32_t ws = warp_sum[w];
      if ((uint32_t)w < warp) wbase += ws;
      total += ws;
    }
    if (i < n) chunk[i] = carry + wbase + x - v;
    carry += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) *count = carry;
}

// ---------------------------------------------------------------------------------------
// Compaction of a sparse level from a bitmap: the inverse of the schedule order gives
// each active cell's D positions, which set one bit each; a count / scan / scatter over
// the bitmap words then yields the active positions in schedule order.  The work is the
// active cells' tasks plus one pass over N*D/8 bytes.

__global__ void k_invert_order(const uint32_t* order, uint32_t total, uint32_t* pos_of_task) {
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < total; p += gridDim.x * blockDim.x)
    pos_of_task[order[p]] = p;
}

__global__ void k_mark_active(const uint8_t* level, int cur, uint32_t n, int D, uint32_t Np,
                              const uint32_t* pos_of_task, uint32_t* bitmap) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    if (level[c] < cur) continue;
    for (int d = 0; d < D; ++d) {
      const uint32_t p = pos_of_task[(size_t)d * Np + c];
      atomicOr(bitmap + (p >> 5), 1u << (p & 31u));
    }
  }
}

constexpr int kBitsThreads = 256;  // one bitmap word per thread, kBitsThreads words per chunk

__global__ void __launch_bounds__(kBitsThreads) k_bits_count(const uint32_t* bitmap, uint32_t words, uint32_t* chunk) {
  const uint32_t w = blockIdx.x * kBitsThreads + threadIdx.x;
  uint32_t n = w < words ? __popc(bitmap[w]) : 0u;
  for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
  __shared__ uint32_t ws[kBitsThreads / 32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = n;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t s = 0;
    for (int i = 0; i < kBitsThreads / 32; ++i) s += ws[i];
    chunk[blockIdx.x] = s;
  }
}

__global__ void __launch_bounds__(kBitsThreads) k_bits_scatter(const uint32_t* bitmap, uint32_t words,
                                                               const uint32_t* chunk, uint32_t* act) {
  const uint32_t w = blockIdx.x * kBitsThreads + threadIdx.x;
  uint32_t bits = w < words ? bitmap[w] : 0u;
  // block-exclusive prefix of the per-thread counts
  __shared__ uint32_t ws[kBitsThreads / 32];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t mine = __popc(bits);
  uint32_t x = mine;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) ws[warp] = x;
  __syncthreads();
  uint32_t base = 0;
  for (uint32_t i = 0; i < warp; ++i) base += ws[i];
  uint32_t o = chunk[blockIdx.x] + base + x - mine;
  while (bits) {
    const int k = __ffs(bits) - 1;
    act[o++] = w * 32u + (uint32_t)k;
    bits &= bits - 1;
  }
}

// ---------------------------------------------------------------------------------------
// Scheduled pull sweep (cooperative launch; every block resident).
//
// Groups of kPullGroup lanes visit the active positions in schedule order.  For its
// current task a group gathers the upwind tasks' words through the task's slots (lane
// l: slots l, l + 8, ...) and commits
//   in = sum_slots |area n . d| q(n, d),   out = (in + source/D + periodic) * attenuation
// (zero below the threshold), q = out / A_down, once every word carries the current
// sweep number; otherwise it retries.  The next positions' records and slots are
// loaded one block ahead, so a task waits only for its neighbours' words.  Every
// dependency lies at an earlier position and every warp walks its positions in order,
// so the earliest unsolved task can always commit.

__device__ __forceinline__ uint32_t pull_pos(const PullArgs& a, uint32_t j) { return a.act ? a.act[j] : j; }

__device__ __forceinline__ void load_slots(const PullArgs& a, const uint4& r, uint32_t gl, uint2 (&s)[kPullRounds]) {
  const uint32_t n = rec_count(r);
  const uint2* base = a.slots + rec_offset(r);
#pragma unroll
  for (int k = 0; k < kPullRounds; ++k)
    if (gl + k * kPullGroup < n) s[k] = __ldg(base + gl + k * kPullGroup);
}

// Warp-lockstep variant of the pull sweep: warp w owns the blocks of four consecutive
// positions b = w, w + W, ... (group g of the warp takes position 4b + g) and advances
// all four together once every one has committed, so the pipeline shift is a
// warp-uniform branch and the four groups' records and slots are contiguous.
// this lane's slots l, l + G, ... (RR of them) of the task whose record is r
template <int G, int RR>
__device__ __forceinline__ void load_slots_g(const PullArgs& a, const uint4& r, uint32_t gl, uint2 (&s)[RR]) {
  const uint32_t n = rec_count(r);
  const uint2* base = a.slots + rec_offset(r);
#pragma unroll
  for (int k = 0; k < RR; ++k)
    if (gl + k * G < n) s[k] = __ldg(base + gl + k * G);
}

template <int kMinBlocks, int G = kPullGroup>
__global__ void __launch_bounds__(kPullThreads, kMinBlocks) k_sweep_pull_lock(PullArgs a) {
  constexpr int RR = kPullGroup * kPullRounds / G;  // slot rounds per lane (16 slots in registers)
  constexpr uint32_t kGroups = 32 / G;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t gl = lane & (G - 1);
  const uint32_t g = lane / G;
  const uint32_t gfirst = g * G;
  const uint32_t gmask = ((1u << G) - 1u) << gfirst;
  const uint32_t W = gridDim.x * (kPullThreads / 32);
  const uint32_t count = a.act ? *a.act_count : a.count;
  const uint32_t sweep = sweep_number(a);
  uint32_t b = blockIdx.x * (kPullThreads / 32) + threadIdx.x / 32;
  // this group's position index in block bb
  auto idx = [&](uint32_t bb) { return bb * kGroups + g; };
  const uint4 z = make_uint4(0u, 0u, 0u, 0u);
  uint4 cur = z, n1 = z, n2 = z;
  uint2 s[RR], ns[RR];
  uint32_t p3 = 0;
  if (idx(b) < count) cur = a.rec[pull_pos(a, idx(b))];
  if (idx(b + W) < count) n1 = a.rec[pull_pos(a, idx(b + W))];
  if (idx(b + 2 * W) < count) n2 = a.rec[pull_pos(a, idx(b + 2 * W))];
  if (idx(b + 3 * W) < count) p3 = pull_pos(a, idx(b + 3 * W));
  load_slots_g<G, RR>(a, cur, gl, s);
  if (idx(b + W) < count) load_slots_g<G, RR>(a, n1, gl, ns);
  bool have = idx(b) < count;
  // the leader's cell data of the current task, loaded once per block.  Above level 0,
  // a sweep over every position tests each task's cell level here and stamps the
  // words of inactive tasks; a sweep over a compacted list of active positions
  // (`sparse`) instead tests the upwind cells' levels when their words are not current.
  const bool check_level = a.act == nullptr && a.current_level > 0;
  const bool sparse = a.act != nullptr && a.current_level > 0;
  float src = 0.f, per = 0.f, att = 0.f;
  bool active = true;
  // One 8-byte load per cell gives {(float) attenuation or the inactive mark, source}
  // (written by the attenuation kernel); the periodic source only for tasks with an
  // upwind periodic face.
  auto load_cell = [&]() {
    active = true;
    if (have && (check_level || gl == 0)) {
      const uint2 cp = __ldg(a.cellpack + cur.x);
      active = cp.x != kInactiveCell;
      att = __uint_as_float(cp.x);
      src = __uint_as_float(cp.y);
      per = (gl == 0 && rec_periodic(cur)) ? __ldcg(a.periodic + rec_dir(cur) * a.Np + cur.x) : 0.f;
    }
  };
  load_cell();
  unsigned long long solved = 0, attempts = 0, w0 = 0;
  uint32_t wait_ns = 32;
  while (b * kGroups < count) {
    if (have && !active) {  // inactive cell: keep its q, stamp the word with this sweep
      if (gl == 0) {
        const uint32_t t = rec_dir(cur) * a.Np + cur.x;
        const unsigned long long own = ld_relaxed_u64(word_ptr(a.qe, t));
        st_relaxed_u64(word_ptr(a.qe, t), (own & 0xffffffffull) | ((unsigned long long)((sweep << 1) | 1u) << 32));
      }
      have = false;
    }
    const uint32_t n_up = have ? rec_count(cur) : 0u;
    const uint32_t dnp = rec_dir(cur) * a.Np;
    unsigned long long w[RR];
    uint32_t lv[RR];
#pragma unroll
    for (int r = 0; r < RR; ++r) {
      const bool pr = gl + r * G < n_up;
      w[r] = ld_relaxed_u64_if(pr, word_ptr(a.qe, s[r].x));
      lv[r] = (sparse && pr) ? a.level[s[r].x - dnp] : 0xffu;
    }
    float in = 0.f;
    bool bad = false;
#pragma unroll
    for (int r = 0; r < RR; ++r) {
      if (gl + r * G < n_up) {
        // an upwind cell inactive in this sweep keeps the q of its last solve
        bad = bad || (!word_current(w[r], sweep) && lv[r] >= (uint32_t)a.current_level);
        in = fmaf(__uint_as_float(s[r].y), __uint_as_float((uint32_t)w[r]), in);
      }
    }
    for (uint32_t j = gl + RR * G; j < n_up; j += G) {
      const uint2 sj = a.slots[rec_offset(cur) + j];
      const unsigned long long wn = ld_relaxed_u64(word_ptr(a.qe, sj.x));
      const uint32_t lj = sparse ? a.level[sj.x - dnp] : 0xffu;
      bad = bad || (!word_current(wn, sweep) && lj >= (uint32_t)a.current_level);
      in = fmaf(__uint_as_float(sj.y), __uint_as_float((uint32_t)wn), in);
    }
    const uint32_t badmask = __ballot_sync(0xffffffffu, bad);
#pragma unroll
    for (int o = 1; o < G; o <<= 1) in += __shfl_xor_sync(0xffffffffu, in, o, G);
    const bool commit = have && (badmask & gmask) == 0u;
    if (have && gl == 0) ++attempts;
    if (commit && gl == 0) {
      const uint32_t t = rec_dir(cur) * a.Np + cur.x;
      const float rt = (in + src) + per;                   // Site::get_rate, site.rs:53-56
      const float out = (rt < a.threshold) ? 0.f : rt * att;  // get_outgoing_rate
      commit_slot(a.qe, t, pack_qe(out * __uint_as_float(cur.y), sweep), in);
      ++solved;
    }
    have = have && !commit;
    const bool any_commit = __any_sync(0xffffffffu, commit);
    if (!__any_sync(0xffffffffu, have)) {  // every group of the block done: advance the warp
      b += W;
      cur = n1;
#pragma unroll
      for (int r = 0; r < RR; ++r) s[r] = ns[r];
      n1 = n2;
      have = idx(b) < count;
      if (idx(b + W) < count) load_slots_g<G, RR>(a, n1, gl, ns);
      if (idx(b + 2 * W) < count) n2 = a.rec[p3];
      if (idx(b + 3 * W) < count) p3 = pull_pos(a, idx(b + 3 * W));
      load_cell();
    }
    if (any_commit) {
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
        break;
      }
      __nanosleep(wait_ns);
      wait_ns = min(wait_ns * 2, 256u);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    solved += __shfl_xor_sync(0xffffffffu, solved, o);
    attempts += __shfl_xor_sync(0xffffffffu, attempts, o);
  }
  if (lane == 0 && solved) atomicAdd(&a.ctl->tasks, solved);
  if (lane == 0 && attempts) atomicAdd(&a.ctl->attempts, attempts);
}

// Lockstep variant with an outer loop over blocks and an inner retry loop: everything
// a retry does not change (word addresses, predicates, weights, commit address, cell
// data) is set up once per block, and the next block's record and slot loads are issued
// when a block starts, so they overlap its waits.  Same additions in the same order as
// the other variants.
template <int kMinBlocks>
__global__ void __launch_bounds__(kPullThreads, kMinBlocks) k_sweep_pull_lock2(PullArgs a) {
  constexpr uint32_t kGroups = 32 / kPullGroup;
  static_assert(kPullRounds == 2, "two slot rounds per lane");
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t gl = lane & (kPullGroup - 1);
  const uint32_t g = lane / kPullGroup;
  const uint32_t gmask = ((1u << kPullGroup) - 1u) << (g * kPullGroup);
  const uint32_t W = gridDim.x * (kPullThreads / 32);
  const uint32_t count = a.act ? *a.act_count : a.count;
  const uint32_t sweep = sweep_number(a);
  const bool check_level = a.act == nullptr && a.current_level > 0;
  // over a compacted list of active positions: an upwind cell below the sweep's level is
  // inactive and keeps the q of its last solve, its word is accepted as it is
  const bool sparse = a.act != nullptr && a.current_level > 0;
  uint32_t b = blockIdx.x * (kPullThreads / 32) + threadIdx.x / 32;
  auto idx = [&](uint32_t bb) { return bb * kGroups + g; };
  // pipeline: record + slots of block b, record of b + W, position of b + 2W
  const uint4 z = make_uint4(0u, 0u, 0u, 0u);
  uint4 cur = z, n1 = z;
  uint2 s[kPullRounds];
  uint32_t p2 = 0;
  if (idx(b) < count) cur = a.rec[pull_pos(a, idx(b))];
  if (idx(b + W) < count) n1 = a.rec[pull_pos(a, idx(b + W))];
  if (idx(b + 2 * W) < count) p2 = pull_pos(a, idx(b + 2 * W));
  load_slots(a, cur, gl, s);
  uint32_t solved = 0, attempts = 0;
  bool stop = false;
  while (!stop && b * kGroups < count) {
    // next block's pipeline stages, issued now
    uint2 ns[kPullRounds];
    uint4 n2 = z;
    uint32_t p3 = 0;
    if (idx(b + W) < count) load_slots(a, n1, gl, ns);
    if (idx(b + 2 * W) < count) n2 = a.rec[p2];
    if (idx(b + 3 * W) < count) p3 = pull_pos(a, idx(b + 3 * W));
    // this block's task
    bool have = idx(b) < count;
    const uint32_t t = rec_dir(cur) * a.Np + cur.x;
    float src = 0.f, per = 0.f, att = 0.f;
    if (have && (check_level || gl == 0)) {
      const uint2 cp = __ldg(a.cellpack + cur.x);  // {(float) attenuation or inactive mark, source}
      if (cp.x == kInactiveCell) {  // inactive: keep q, stamp the word
        if (gl == 0) {
          const unsigned long long own = ld_relaxed_u64(word_ptr(a.qe, t));
          st_relaxed_u64(word_ptr(a.qe, t), (own & 0xffffffffull) | ((unsigned long long)((sweep << 1) | 1u) << 32));
        }
        have = false;
      } else if (gl == 0) {
        src = __uint_as_float(cp.y);
        per = rec_periodic(cur) ? __ldcg(a.periodic + t) : 0.f;
        att = __uint_as_float(cp.x);
      }
    }
    const uint32_t n_up = have ? rec_count(cur) : 0u;
    const bool p0 = gl < n_up, p1 = gl + kPullGroup < n_up;
    const unsigned long long* q0 = word_ptr(a.qe, s[0].x);
    const unsigned long long* q1 = word_ptr(a.qe, s[1].x);
    const float wt0 = __uint_as_float(s[0].y), wt1 = __uint_as_float(s[1].y);
    const bool big = n_up > (uint32_t)(kPullRounds * kPullGroup);
    const uint32_t dnp = rec_dir(cur) * a.Np;
    const bool keep0 = sparse && p0 && a.level[s[0].x - dnp] < (uint32_t)a.current_level;
    const bool keep1 = sparse && p1 && a.level[s[1].x - dnp] < (uint32_t)a.current_level;
    unsigned long long w0 = 0;
    uint32_t wait_ns = 32;
    // a word that carries the current sweep number (or of an inactive upwind cell) is
    // final for the sweep: a retry reloads only the words that were not
    unsigned long long x0 = 0, x1 = 0;
    bool need0 = p0, need1 = p1;
    while (true) {
      if (need0) x0 = ld_relaxed_u64(q0);
      if (need1) x1 = ld_relaxed_u64(q1);
      need0 = p0 && !keep0 && !word_current(x0, sweep);
      need1 = p1 && !keep1 && !word_current(x1, sweep);
      bool bad = need0 || need1;
      float in = p0 ? fmaf(wt0, __uint_as_float((uint32_t)x0), 0.f) : 0.f;
      if (p1) in = fmaf(wt1, __uint_as_float((uint32_t)x1), in);
      if (big) {
        for (uint32_t j = gl + kPullRounds * kPullGroup; j < n_up; j += kPullGroup) {
          const uint2 sj = a.slots[rec_offset(cur) + j];
          const unsigned long long wn = ld_relaxed_u64(word_ptr(a.qe, sj.x));
          bad = bad || (!word_current(wn, sweep) &&
                        !(sparse && a.level[sj.x - dnp] < (uint32_t)a.current_level));
          in = fmaf(__uint_as_float(sj.y), __uint_as_float((uint32_t)wn), in);
        }
      }
      const uint32_t badmask = __ballot_sync(0xffffffffu, bad);
#pragma unroll
      for (int o = 1; o < kPullGroup; o <<= 1) in += __shfl_xor_sync(0xffffffffu, in, o, kPullGroup);
      const bool commit = have && (badmask & gmask) == 0u;
      if (have && gl == 0) ++attempts;
      if (commit && gl == 0) {
        const float rt = (in + src) + per;                      // Site::get_rate, site.rs:53-56
        const float out = (rt < a.threshold) ? 0.f : rt * att;  // get_outgoing_rate
        commit_slot(a.qe, t, pack_qe(out * __uint_as_float(cur.y), sweep), in);
        ++solved;
      }
      have = have && !commit;
      if (!__any_sync(0xffffffffu, have)) break;
      if (__any_sync(0xffffffffu, commit)) {
        w0 = 0;
        wait_ns = 32;
        continue;
      }
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
      wait_ns = min(wait_ns * 2, 256u);
    }
    // advance the pipeline by one block
    b += W;
    cur = n1;
#pragma unroll
    for (int r = 0; r < kPullRounds; ++r) s[r] = ns[r];
    n1 = n2;
    p2 = p3;
  }
  unsigned long long ts = solved, ta = attempts;
  for (int o = 16; o > 0; o >>= 1) {
    ts += __shfl_xor_sync(0xffffffffu, ts, o);
    ta += __shfl_xor_sync(0xffffffffu, ta, o);
  }
  if (lane == 0 && ts) atomicAdd(&a.ctl->tasks, ts);
  if (lane == 0 && ta) atomicAdd(&a.ctl->attempts, ta);
}

// Wavefront form of the dense pull sweep: one thread per task, schedule level by
// schedule level, with a grid-wide barrier between levels (cooperative launch).  Every
// upwind task lies at an earlier level, so after the barrier a task's inputs are all
// published and no readiness test or retry is needed.  Thread j solves positions
// lvl[k] + j, lvl[k] + j + T, ... of level k; its first position of level k + 1
// (record, upwind slots and cell data, none of which a sweep writes) is loaded before
// the barrier, so only the neighbours' q words are read after it.  The sum of a task is
// formed exactly as the lockstep kernels form it: eight partial sums over the slots
// j = l, l + 8, ... (FMA in slot order), combined pairwise ((0+1)+(2+3))+((4+5)+(6+7)).
// Inactive cells of a sweep above level 0 are skipped: their words keep the q of their
// last solve, and no consumer in this kernel tests sweep numbers.
constexpr int kWaveThreads = 256;
constexpr int kWaveSlots = 16;  // upwind slots held in registers (two rounds of eight)

// Barrier k of the wavefront kernel: arrivals counted in ctl->head (zeroed before each
// sweep), all gridDim.x blocks have arrived when it reaches target = (k + 1) * gridDim.x.
// Release: the block's stores, ordered before thread 0 by __syncthreads, are made
// visible at GPU scope by the fence before the arrival; acquire: the fence after the
// wait.  The wait is bounded: on a timeout or an error raised elsewhere it sets kErrStall
// and the block returns false.
__device__ __forceinline__ bool wave_barrier(const PullArgs& a, unsigned long long target, int* flag) {
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    asm volatile("fence.acq_rel.gpu;" ::: "memory");
    atomicAdd(&a.ctl->head, 1ull);
    unsigned long long w0 = 0;
    while (ld_relaxed64(&a.ctl->head) < target) {
      const unsigned long long now = globaltimer_ns();
      if (w0 == 0) w0 = now;
      if (now - w0 > a.timeout_ns || *(volatile uint32_t*)&a.ctl->error != 0) {
        atomicOr(&a.ctl->error, kErrStall);
        ok = 0;
        break;
      }
    }
    asm volatile("fence.acq_rel.gpu;" ::: "memory");
    *flag = ok;
  }
  __syncthreads();
  return *flag != 0;
}

// one task of the wavefront kernel with its loads that no sweep result changes
struct WaveTask {
  uint4 r;
  uint2 s[kWaveSlots];
  float src, per, att;
  bool live;
};

__device__ __forceinline__ void wave_fetch(const PullArgs& a, uint32_t i, bool check_level, WaveTask& w) {
  w.r = __ldg(a.rec + i);
  const uint32_t c = w.r.x;
  const uint2 cp = __ldg(a.cellpack + c);  // {(float) attenuation or inactive mark, source}
  w.live = cp.x != kInactiveCell;
  const uint32_t n = w.live ? rec_count(w.r) : 0u;
  const uint2* base = a.slots + rec_offset(w.r);
#pragma unroll
  for (int j = 0; j < kWaveSlots; ++j)
    if ((uint32_t)j < n) w.s[j] = __ldg(base + j);
  w.src = __uint_as_float(cp.y);
  w.att = __uint_as_float(cp.x);
  w.per = (w.live && rec_periodic(w.r)) ? __ldcg(a.periodic + rec_dir(w.r) * a.Np + c) : 0.f;
}

__device__ __forceinline__ void wave_solve(const PullArgs& a, const WaveTask& w, uint32_t sweep,
                                           unsigned long long& solved) {
  if (!w.live) return;
  const uint32_t n = rec_count(w.r);
  uint32_t q[kWaveSlots];
#pragma unroll
  for (int j = 0; j < kWaveSlots; ++j)
    q[j] = (uint32_t)j < n ? ld_relaxed(reinterpret_cast<const uint32_t*>(word_ptr(a.qe, w.s[j].x))) : 0u;
  float p[8];
#pragma unroll
  for (int l = 0; l < 8; ++l) p[l] = 0.f;
#pragma unroll
  for (int j = 0; j < kWaveSlots; ++j)
    if ((uint32_t)j < n) p[j & 7] = fmaf(__uint_as_float(w.s[j].y), __uint_as_float(q[j]), p[j & 7]);
  if (n > (uint32_t)kWaveSlots) {  // the rest from memory, eight at a time
    const uint2* base = a.slots + rec_offset(w.r);
    for (uint32_t j0 = kWaveSlots; j0 < n; j0 += 8) {
#pragma unroll
      for (int l = 0; l < 8; ++l)
        if (j0 + l < n) {
          const uint2 sl = __ldg(base + j0 + l);
          const float qv = __uint_as_float(ld_relaxed(reinterpret_cast<const uint32_t*>(word_ptr(a.qe, sl.x))));
          p[l] = fmaf(__uint_as_float(sl.y), qv, p[l]);
        }
    }
  }
  const float in = ((p[0] + p[1]) + (p[2] + p[3])) + ((p[4] + p[5]) + (p[6] + p[7]));
  const uint32_t t = rec_dir(w.r) * a.Np + w.r.x;
  const float rt = (in + w.src) + w.per;                    // Site::get_rate, site.rs:53-56
  const float out = (rt < a.threshold) ? 0.f : rt * w.att;  // get_outgoing_rate
  commit_slot(a.qe, t, pack_qe(out * __uint_as_float(w.r.y), sweep), in);
  ++solved;
}

template <int kMinBlocks>
__global__ void __launch_bounds__(kWaveThreads, kMinBlocks) k_sweep_pull_wave(PullArgs a) {
  __shared__ int flag;
  const uint32_t T = gridDim.x * kWaveThreads;
  const uint32_t j = blockIdx.x * kWaveThreads + threadIdx.x;
  const uint32_t L = a.num_sched;
  const uint32_t sweep = sweep_number(a);
  const bool check_level = a.current_level > 0;
  unsigned long long solved = 0;
  WaveTask cur;
  uint32_t lo = __ldg(a.lvl), hi = L ? __ldg(a.lvl + 1) : lo;
  bool have = lo + j < hi;
  if (have) wave_fetch(a, lo + j, check_level, cur);
  for (uint32_t k = 0; k < L; ++k) {
    if (have) wave_solve(a, cur, sweep, solved);
    for (uint32_t i = lo + j + T; i < hi; i += T) {  // levels wider than the grid
      WaveTask extra;
      wave_fetch(a, i, check_level, extra);
      wave_solve(a, extra, sweep, solved);
    }
    if (k + 1 == L) break;
    lo = hi;
    hi = __ldg(a.lvl + k + 2);
    have = lo + j < hi;
    if (have) wave_fetch(a, lo + j, check_level, cur);
    if (!wave_barrier(a, (unsigned long long)(k + 1) * gridDim.x, &flag)) break;
  }
  const uint32_t lane = threadIdx.x & 31;
  for (int o = 16; o > 0; o >>= 1) solved += __shfl_xor_sync(0xffffffffu, solved, o);
  if (lane == 0 && solved) {
    atomicAdd(&a.ctl->tasks, solved);
    atomicAdd(&a.ctl->attempts, solved);
  }
}

// TMA bulk copies into shared memory with mbarrier completion (used by the staged
// wavefront kernel below).
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// bounded wait for the phase of `parity`; false (and kErrStall) on a timeout
__device__ __forceinline__ bool mbar_wait(const PullArgs& a, uint64_t* bar, uint32_t parity) {
  if (mbar_test(bar, parity)) return true;
  const unsigned long long w0 = globaltimer_ns();
  while (!mbar_test(bar, parity)) {
    if (globaltimer_ns() - w0 > a.timeout_ns) {
      atomicOr(&a.ctl->error, kErrStall);
      return false;
    }
  }
  return true;
}

// bytes (a multiple of 16) from global src to shared dst (both 16-byte aligned)
__device__ __forceinline__ void bulk_to_shared(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

struct StgCell {
  float src, per, att;
  bool live;
};


__device__ __forceinline__ void stg_commit(const PullArgs& a, const uint4& r, const StgCell& c, float in,
                                           uint32_t sweep) {
  const uint32_t t = rec_dir(r) * a.Np + r.x;
  const float rt = (in + c.src) + c.per;                    // Site::get_rate, site.rs:53-56
  const float out = (rt < a.threshold) ? 0.f : rt * c.att;  // get_outgoing_rate
  commit_slot(a.qe, t, pack_qe(out * __uint_as_float(r.y), sweep), in);
}

// Fully staged wavefront kernel (one block of 1024 threads per SM).  A plain load still
// in flight at the grid barrier costs its whole latency there, so everything a level
// needs that the previous level did not write arrives through the async (TMA) proxy:
//  * the level offsets, once, into shared memory;
//  * per unit (one pass of a block over its share of a level: the level is cut into
//    gridDim.x contiguous chunks of ceil(width / gridDim.x) positions, so every SM works
//    on every level, and a block takes its chunk B positions per pass; all blocks make
//    the same number of passes), the block's records and periodic sources, two units
//    ahead, and its
//    contiguous range of upwind slots, one unit ahead (records in shared memory give the
//    range), each completing on an mbarrier (three record stages, two slot stages).
// After the barrier a thread reads its record and slots from shared memory and loads
// only the neighbours' q words and its cell's {attenuation, source} pack (L2), all
// consumed before the next barrier.  Warp 0 takes no tasks: its thread 0 generates the
// units, issues the copies and runs the grid barrier while the other 31 warps solve.
// Sums, roundings and skipped inactive cells are the wavefront kernel's.
constexpr int kStgThreads = 1024;
constexpr uint32_t kStgTasks = kStgThreads - 32;  // task threads per block (warps 1-31)
constexpr uint32_t kStgPers = kStgThreads + 4;  // periodic sources per stage (16-byte aligned copy)

struct StgUnit {
  uint32_t first, n, peroff, flags;  // flags: 1 last pass of its level, 2 last unit
};

struct StgShared {
  uint64_t rec_bar[3], slot_bar[2], lvl_bar;
  StgUnit unit[3];
  unsigned long long base[2];
  int staged[2];
  int flag;
};

// dynamic shared memory: slot stages [2][cap] uint2 | records [3][B] uint4 |
// periodic [3][kStgPers] float | level offsets [lvl_words]
__host__ __device__ constexpr size_t stg_smem_bytes(uint32_t cap, uint32_t lvl_words) {
  return 2 * (size_t)cap * 8 + 3 * (size_t)kStgThreads * 16 + 3 * (size_t)kStgPers * 4 + (size_t)lvl_words * 4;
}

// q of a word published before the last grid barrier.  No word of an earlier level is
// written during a level, and the barrier's acquire fence leaves no stale line in L1, so
// the load may be served by L1: neighbouring tasks of a block share many upwind words.
__device__ __forceinline__ uint32_t stg_word(const PullArgs& a, uint32_t t) {
  return *reinterpret_cast<const unsigned int*>(word_ptr(a.qe, t));
}

// incoming rate of one task (the lockstep kernels' sum): the first 16 neighbours' words
// are requested together, the weights re-read from the slots afterwards
__device__ __forceinline__ float stg_gather(const PullArgs& a, const uint2* sl, uint32_t n) {
  constexpr int K = 16;
  uint32_t q[K];
#pragma unroll
  for (int j = 0; j < K; ++j) q[j] = (uint32_t)j < n ? stg_word(a, sl[j].x) : 0u;
  float p[8];
#pragma unroll
  for (int l = 0; l < 8; ++l) p[l] = 0.f;
#pragma unroll
  for (int j = 0; j < K; ++j)
    if ((uint32_t)j < n) p[j & 7] = fmaf(__uint_as_float(sl[j].y), __uint_as_float(q[j]), p[j & 7]);
  for (uint32_t j0 = K; j0 < n; j0 += 8) {
#pragma unroll
    for (int l = 0; l < 8; ++l)
      if (j0 + l < n) {
        const uint2 v = sl[j0 + l];
        p[l] = fmaf(__uint_as_float(v.y), __uint_as_float(stg_word(a, v.x)), p[l]);
      }
  }
  return ((p[0] + p[1]) + (p[2] + p[3])) + ((p[4] + p[5]) + (p[6] + p[7]));
}

__global__ void __launch_bounds__(kStgThreads, 1) k_sweep_pull_staged(PullArgs a, uint32_t cap, uint32_t lvl_words) {
  extern __shared__ __align__(128) unsigned char dyn[];
  __shared__ StgShared sh;
  constexpr uint32_t B = kStgThreads;   // stage rows (kStgTasks used)
  constexpr uint32_t BT = kStgTasks;
  uint2* slot_st = reinterpret_cast<uint2*>(dyn);
  uint4* rec_st = reinterpret_cast<uint4*>(dyn + 2 * (size_t)cap * 8);
  float* per_st = reinterpret_cast<float*>(dyn + 2 * (size_t)cap * 8 + 3 * (size_t)B * 16);
  uint32_t* lvl_s = reinterpret_cast<uint32_t*>(dyn + 2 * (size_t)cap * 8 + 3 * (size_t)B * 16 + 3 * (size_t)kStgPers * 4);
  const uint32_t tid = threadIdx.x;
  const uint32_t L = a.num_sched;
  const uint32_t sweep = sweep_number(a);
  unsigned long long solved = 0;
  // thread 0: unit generator (level gk, pass gp), issued-copy parities and the stages
  // with a copy it has not waited for (bits 0-2 records, 3-4 slots)
  uint32_t gk = 0, gp = 0, iss = 0, outstanding = 0;
  auto generate = [&](StgUnit& u) -> bool {
    if (gk >= L) return false;
    const uint32_t lo = lvl_s[gk], hi = lvl_s[gk + 1];
    const uint32_t chunk = (hi - lo + gridDim.x - 1) / gridDim.x;
    const unsigned long long cfirst = lo + (unsigned long long)blockIdx.x * chunk;
    const unsigned long long cend = min(cfirst + chunk, (unsigned long long)hi);
    const unsigned long long first = cfirst + (unsigned long long)gp * BT;
    const unsigned long long end = min(first + BT, cend);
    u.first = first < end ? (uint32_t)first : 0u;
    u.n = first < end ? (uint32_t)(end - first) : 0u;
    u.peroff = u.first & 3u;
    u.flags = 0;
    if ((unsigned long long)(gp + 1) * BT < chunk) {
      ++gp;
    } else {
      u.flags = (gk + 1 == L) ? 3u : 1u;
      ++gk;
      gp = 0;
    }
    return true;
  };
  auto issue_rec = [&](int s, const StgUnit& u) {
    sh.unit[s] = u;
    if (u.n == 0) return;
    const uint32_t p0 = u.first & ~3u, p1 = (u.first + u.n + 3u) & ~3u;
    const uint32_t rb = u.n * 16u, pb = (p1 - p0) * 4u;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(&sh.rec_bar[s], rb + pb);
    bulk_to_shared(rec_st + s * B, a.rec + u.first, rb, &sh.rec_bar[s]);
    bulk_to_shared(per_st + s * kStgPers, a.per_pos + p0, pb, &sh.rec_bar[s]);
    iss ^= 1u << s;
    outstanding |= 1u << s;
  };
  // thread 0: the slots of the unit whose records are in stage s3, into slot stage s2
  auto issue_slots = [&](int s2, int s3) {
    const uint32_t n = sh.unit[s3].n;
    int ok = 0;
    if (n > 0) {
      if (outstanding & (1u << s3)) {  // its records (issued a unit ago)
        if (!mbar_wait(a, &sh.rec_bar[s3], ((iss >> s3) & 1u) ^ 1u)) {
          sh.staged[s2] = 0;
          return;
        }
        outstanding &= ~(1u << s3);
      }
      const uint4 r0 = rec_st[s3 * B], r1 = rec_st[s3 * B + n - 1];
      const unsigned long long lo = rec_offset(r0) & ~1ull, hi = (rec_offset(r1) + rec_count(r1) + 1ull) & ~1ull;
      if (hi > lo && hi - lo <= cap) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(&sh.slot_bar[s2], (uint32_t)((hi - lo) * 8));
        bulk_to_shared(slot_st + s2 * (size_t)cap, a.slots + lo, (uint32_t)((hi - lo) * 8), &sh.slot_bar[s2]);
        sh.base[s2] = lo;
        iss ^= 1u << (3 + s2);
        outstanding |= 1u << (3 + s2);
        ok = 1;
      }
    }
    sh.staged[s2] = ok;
  };
  bool alive = true;
  if (tid == 0) {
    for (int s = 0; s < 3; ++s) mbar_init(&sh.rec_bar[s], 1);
    for (int s = 0; s < 2; ++s) mbar_init(&sh.slot_bar[s], 1);
    mbar_init(&sh.lvl_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(&sh.lvl_bar, lvl_words * 4u);
    bulk_to_shared(lvl_s, a.lvl, lvl_words * 4u, &sh.lvl_bar);
    alive = mbar_wait(a, &sh.lvl_bar, 0u);
    if (alive) {
      StgUnit u;
      if (generate(u)) issue_rec(0, u);
      if (!(u.flags & 2u) && generate(u)) issue_rec(1, u);
      issue_slots(0, 0);
    }
    sh.flag = alive ? 1 : 0;
  }
  __syncthreads();
  alive = sh.flag != 0 && L > 0;
  uint32_t rec_par = 0, slot_par = 0, nbar = 0;
  for (uint32_t u = 0; alive; ++u) {
    const int s3 = u % 3, s2 = u & 1;
    const StgUnit cu = sh.unit[s3];
    if (tid == 0 && !(cu.flags & 2u)) {
      issue_slots(s2 ^ 1, (s3 + 1) % 3);  // unit u + 1
      StgUnit nu;
      if (!(sh.unit[(s3 + 1) % 3].flags & 2u) && generate(nu)) issue_rec((s3 + 2) % 3, nu);  // unit u + 2
    }
    // task thread tt = tid - 32 solves position cu.first + tt
    const uint32_t tt = tid - 32u;
    const bool task = tid >= 32 && tt < cu.n;
    bool ok = true;
    if (cu.n > 0) {
      if (task || tid == 0) ok = mbar_wait(a, &sh.rec_bar[s3], (rec_par >> s3) & 1u);
      if (tid == 0 && ok) outstanding &= ~(1u << s3);
      rec_par ^= 1u << s3;
    }
    const int stg = sh.staged[s2];
    if (stg) {
      if (ok && (task || tid == 0)) ok = mbar_wait(a, &sh.slot_bar[s2], (slot_par >> s2) & 1u);
      if (tid == 0 && ok) outstanding &= ~(1u << (3 + s2));
      slot_par ^= 1u << s2;
    }
    if (ok && task) {
      const uint4 r = rec_st[s3 * B + tt];
      const uint2 cp = __ldg(a.cellpack + r.x);
      if (cp.x != kInactiveCell) {
        const uint32_t n = rec_count(r);
        const uint2* sl = stg ? slot_st + s2 * (size_t)cap + (rec_offset(r) - sh.base[s2]) : a.slots + rec_offset(r);
        const float in = stg_gather(a, sl, n);
        StgCell c;
        c.src = __uint_as_float(cp.y);
        c.att = __uint_as_float(cp.x);
        c.per = per_st[s3 * kStgPers + cu.peroff + tt];
        c.live = true;
        stg_commit(a, r, c, in, sweep);
        ++solved;
      }
    }
    if (cu.flags & 2u) break;
    if (cu.flags & 1u) {
      if (!wave_barrier(a, (unsigned long long)(++nbar) * gridDim.x, &sh.flag)) break;
    } else {
      __syncthreads();
    }
  }
  if (tid == 0) {  // copies issued and never waited for (after an error): wait, bounded
    for (int s = 0; s < 5; ++s)
      if (outstanding & (1u << s))
        (void)mbar_wait(a, s < 3 ? &sh.rec_bar[s] : &sh.slot_bar[s - 3], ((iss >> s) & 1u) ^ 1u);
  }
  const uint32_t lane = tid & 31;
  for (int o = 16; o > 0; o >>= 1) solved += __shfl_xor_sync(0xffffffffu, solved, o);
  if (lane == 0 && solved) {
    atomicAdd(&a.ctl->tasks, solved);
    atomicAdd(&a.ctl->attempts, solved);
  }
}

// Gathered incoming rate of (c, d): sum over upwind LOCAL faces of |s| q(n, d), or
// over LOCAL_PERIODIC faces when `periodic_faces`.
__device__ __forceinline__ float gather_in(const PullArgs& a, uint32_t c, uint32_t d, bool periodic_faces) {
  const float fx = a.dir32[3 * d], fy = a.dir32[3 * d + 1], fz = a.dir32[3 * d + 2];
  const double dx = a.dir64[3 * d], dy = a.dir64[3 * d + 1], dz = a.dir64[3 * d + 2];
  const uint32_t want = periodic_faces ? kKindPeriodic : kKindLocal;
  float in = 0.f;
  for (uint32_t f = a.off[c]; f < a.off[c + 1]; ++f) {
    const uint4 g = a.geo16[f];
    if ((g.w >> kKindShift) != want) continue;
    const float s = face_eff(g, fx, fy, fz, a.geo64 + f, dx, dy, dz);
    if (s < 0.f) in = fmaf(-s, __uint_as_float((uint32_t)*word_ptr(a.qe, (size_t)d * a.Np + (g.w & kNbrMask))), in);
  }
  return in;
}

// Periodic sources after a sweep (snapshot semantics): for every cell with periodic
// faces and every direction, the flux arriving through its LOCAL_PERIODIC upwind faces.
// Entry e = d * n_cells + (index of the cell in `cells`).  The upwind periodic faces of
// an entry are precomputed once per grid (k_fold_build: up to kFoldSlots of them, in
// face order, as {upwind task, |area n . d|}); an entry with more is gathered from the
// geometry.  Both sum in face order with the same roundings.
constexpr int kFoldSlots = 4;
constexpr uint8_t kFoldOverflow = 0xffu;

__global__ void k_fold_build(PullArgs a, const uint32_t* cells, uint32_t n_cells, uint8_t* cnt, uint2* slots) {
  const size_t total = (size_t)n_cells * a.D;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const uint32_t d = (uint32_t)(e / n_cells);
    const uint32_t c = cells[e % n_cells];
    const float fx = a.dir32[3 * d], fy = a.dir32[3 * d + 1], fz = a.dir32[3 * d + 2];
    const double dx = a.dir64[3 * d], dy = a.dir64[3 * d + 1], dz = a.dir64[3 * d + 2];
    uint32_t n = 0;
    for (uint32_t f = a.off[c]; f < a.off[c + 1]; ++f) {
      const uint4 g = a.geo16[f];
      if ((g.w >> kKindShift) != kKindPeriodic) continue;
      const float sf = face_eff(g, fx, fy, fz, a.geo64 + f, dx, dy, dz);
      if (!(sf < 0.f)) continue;
      if (n < (uint32_t)kFoldSlots)
        slots[e * kFoldSlots + n] = make_uint2(d * a.Np + (g.w & kNbrMask), __float_as_uint(-sf));
      ++n;
    }
    cnt[e] = n > (uint32_t)kFoldSlots ? kFoldOverflow : (uint8_t)n;
  }
}

// grid: (periodic cells / blockDim.x, D)
// After a sweep that left cells inactive: marks the periodic cells with a periodic
// neighbour that was active (attenuation's inactive mark in `cellpack`).  Only their
// entries can change; every other entry is the same sum of the same words.
__global__ void k_fold_mark(PullArgs a, const uint32_t* cells, uint32_t n_cells, uint8_t* changed) {
  for (uint32_t pc = blockIdx.x * blockDim.x + threadIdx.x; pc < n_cells; pc += gridDim.x * blockDim.x) {
    const uint32_t c = cells[pc];
    uint8_t ch = 0;
    for (uint32_t f = a.off[c]; f < a.off[c + 1] && !ch; ++f) {
      const uint32_t w = a.geo16[f].w;
      if ((w >> kKindShift) == kKindPeriodic && a.cellpack[w & kNbrMask].x != kInactiveCell) ch = 1;
    }
    changed[pc] = ch;
  }
}

// changed: null after a sweep of every cell, else the marks of k_fold_mark
__global__ void k_fold_pull(PullArgs a, float* periodic, const uint32_t* cells, uint32_t n_cells,
                            const uint8_t* cnt, const uint2* slots, const uint8_t* changed) {
  const uint32_t d = blockIdx.y;
  const uint32_t pc = blockIdx.x * blockDim.x + threadIdx.x;
  if (pc < n_cells && (!changed || changed[pc])) {
    const size_t e = (size_t)d * n_cells + pc;
    const uint32_t c = cells[pc];
    const uint32_t n = cnt[e];
    float in = 0.f;
    if (n == kFoldOverflow) {
      in = gather_in(a, c, d, true);
    } else {
      for (uint32_t k = 0; k < n; ++k) {
        const uint2 sl = slots[e * kFoldSlots + k];
        in = fmaf(__uint_as_float(sl.y), __uint_as_float((uint32_t)*word_ptr(a.qe, sl.x)), in);
      }
    }
    periodic[(size_t)d * a.Np + c] = in;
    if (a.per_pos) a.per_pos[a.pos_of_task[(size_t)d * a.Np + c]] = in;
  }
}

// Whether every incoming rate stored for cell c is current: a neighbour's q changes only
// when the neighbour is solved, so if no LOCAL neighbour was solved in a later sweep than
// c, each (c, d) still holds the sum it formed at c's last solve.
__device__ __forceinline__ bool cell_current(const PullArgs& a, uint32_t c) {
  const uint32_t mine = a.cell_sweep[c];
  for (uint32_t f = a.off[c]; f < a.off[c + 1]; ++f) {
    const uint32_t w = a.geo16[f].w;
    if ((w >> kKindShift) == kKindLocal && a.cell_sweep[w & kNbrMask] > mine) return false;
  }
  return true;
}

// Incoming rate of every (c, d) as the reference holds it after a step: the stored
// value if the cell is current or the task was solved in the step's last sweep, else
// gathered from the neighbours' current q (the reference keeps adding corrections to
// inactive cells).
__device__ __forceinline__ float current_incoming(const PullArgs& a, uint32_t c, uint32_t d, uint32_t last_epoch,
                                                  bool cell_is_current) {
  const size_t t = (size_t)d * a.Np + c;
  if (cell_is_current) return stored_incoming(a.qe, t);
  if ((uint32_t)(*word_ptr(a.qe, t) >> 32) == (last_epoch << 1)) return stored_incoming(a.qe, t);  // solved, not stamped
  return gather_in(a, c, d, false);
}

__global__ void k_photon_rate_pull(PullArgs a, uint32_t last_epoch, double rate_scale, double* out) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < a.N; c += gridDim.x * blockDim.x) {
    double r = 0.0;
    const bool cur = cell_current(a, c);
    for (int d = 0; d < a.D; ++d) r += (double)current_incoming(a, c, d, last_epoch, cur);
    out[c] = r * rate_scale;
  }
}

// Rate of every cell summed over directions as Sweep::get_solver forms it
// (src/sweep/mod.rs:616-620): sum over d of (incoming + source/D) + periodic, photons/s.
__global__ void k_cell_rates_pull(PullArgs a, uint32_t last_epoch, double rate_scale, double* out) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < a.N; c += gridDim.x * blockDim.x) {
    double r = 0.0;
    const bool cur = cell_current(a, c);
    for (int d = 0; d < a.D; ++d)
      r += ((double)current_incoming(a, c, d, last_epoch, cur) + (double)a.src_dir[c]) +
           (double)a.periodic[(size_t)d * a.Np + c];
    out[c] = r * rate_scale;
  }
}

// Export of per-task rates in [cell][D] layout, photons/s: which = 0 incoming,
// 1 outgoing (q * A), 2 periodic.
__global__ void k_export_pull(PullArgs a, uint32_t last_epoch, int which, double rate_scale, double* out) {
  const size_t total = (size_t)a.N * a.D;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const uint32_t c = (uint32_t)(i / a.D), d = (uint32_t)(i % a.D);
    const size_t t = (size_t)d * a.Np + c;
    float v;
    if (which == 0) {
      v = current_incoming(a, c, d, last_epoch, cell_current(a, c));
    } else if (which == 2) {
      v = a.periodic[t];
    } else {
      const float fx = a.dir32[3 * d], fy = a.dir32[3 * d + 1], fz = a.dir32[3 * d + 2];
      const double dx = a.dir64[3 * d], dy = a.dir64[3 * d + 1], dz = a.dir64[3 * d + 2];
      float area_down = 0.f;
      for (uint32_t f = a.off[c]; f < a.off[c + 1]; ++f) {
        const float s = face_eff(a.geo16[f], fx, fy, fz, a.geo64 + f, dx, dy, dz);
        if (s > 0.f) area_down += s;
      }
      v = __uint_as_float((uint32_t)*word_ptr(a.qe, t)) * area_down;
    }
    out[i] = (double)v * rate_scale;
  }
}

}  // namespace swk
