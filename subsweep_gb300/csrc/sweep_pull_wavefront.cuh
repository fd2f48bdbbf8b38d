// The level-synchronous (wavefront) pull sweep kernels (pull path).
// Part of the pull-form transport of the mixed path; the shared definitions
// (PullArgs, words, records) are in sweep_pull.cuh.
#pragma once

#include "sweep_pull.cuh"

namespace swk {

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
    uint32_t spins = 0;
    // the pollers share the arrivals' cache line: poll it alone, with a short sleep,
    // and look at the clock and the error flag every 16th poll
    while (ld_relaxed64(&a.ctl->head) < target) {
      if ((++spins & 15u) == 0) {
        const unsigned long long now = globaltimer_ns();
        if (w0 == 0) w0 = now;
        if (now - w0 > a.timeout_ns || *(volatile uint32_t*)&a.ctl->error != 0) {
          atomicOr(&a.ctl->error, kErrStall);
          ok = 0;
          break;
        }
      }
      __nanosleep(20);
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
  uint32_t pos;  // schedule position (the index of the task's word)
  bool live;
};

__device__ __forceinline__ void wave_fetch(const PullArgs& a, uint32_t i, bool check_level, WaveTask& w) {
  w.r = __ldg(a.rec + i);
  w.pos = i;
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
  const float rt = (in + w.src) + w.per;                    // Site::get_rate, site.rs:53-56
  const float out = (rt < a.threshold) ? 0.f : rt * w.att;  // get_outgoing_rate
  commit_slot(a, w.pos, w.r, pack_qe(out * __uint_as_float(w.r.y), sweep), in);
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


// `pos`: the task's schedule position (the index of its word)
__device__ __forceinline__ void stg_commit(const PullArgs& a, const uint4& r, const StgCell& c, float in,
                                           uint32_t sweep, uint32_t pos) {
  const float rt = (in + c.src) + c.per;                    // Site::get_rate, site.rs:53-56
  const float out = (rt < a.threshold) ? 0.f : rt * c.att;  // get_outgoing_rate
  commit_slot(a, pos, r, pack_qe(out * __uint_as_float(r.y), sweep), in);
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
__device__ __forceinline__ uint32_t stg_word(const PullArgs& a, uint32_t p) {
  return *reinterpret_cast<const unsigned int*>(word_ptr(a.qe, p));
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
        stg_commit(a, r, c, in, sweep, cu.first + tt);
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

}  // namespace swk
