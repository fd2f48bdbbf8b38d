// The warp-lockstep pull sweep kernels (pull path).
// Part of the pull-form transport of the mixed path; the shared definitions
// (PullArgs, words, records) are in sweep_pull.cuh.
#pragma once

#include "sweep_pull.cuh"

namespace swk {

// ---------------------------------------------------------------------------------------
// Scheduled pull sweep (cooperative launch; every block resident).
//
// Groups of kPullGroup lanes visit the active positions in schedule order.  For its
// current task a group gathers the upwind tasks' words through the task's slots (lane
// l: slots l, l + 8, ...) and commits
//   in = sum_slots |area n . d| q(n, d),   out = (in + source/D + periodic) * attenuation
// (zero below the threshold), q = out / A_down, once every word carries the current
// sweep number; otherwise it retries.  The next positions' records, slots and cell data
// are loaded one block ahead, so a task waits only for its neighbours' words.  Every
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
  // upwind periodic face.  Both are loaded one block ahead, with the slots: whether the
  // cell is active decides which lanes load words, so a pack loaded in the block itself
  // would hold back its word loads.
  const bool cell_lane = check_level || gl == 0;
  uint2 cp = make_uint2(0u, 0u), ncp = make_uint2(0u, 0u);
  float nper = 0.f;
  auto fetch_cell = [&](const uint4& r, uint2& pk, float& pr) {
    pk = __ldg(a.cellpack + r.x);
    pr = (gl == 0 && rec_periodic(r)) ? __ldcg(a.periodic + rec_dir(r) * a.Np + r.x) : 0.f;
  };
  auto take_cell = [&]() {
    active = true;
    if (have && cell_lane) {
      active = cp.x != kInactiveCell;
      att = __uint_as_float(cp.x);
      src = __uint_as_float(cp.y);
    }
  };
  if (have && cell_lane) fetch_cell(cur, cp, per);
  if (idx(b + W) < count && cell_lane) fetch_cell(n1, ncp, nper);
  take_cell();
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
      cp = ncp;
      per = nper;
      have = idx(b) < count;
      if (idx(b + W) < count) {
        load_slots_g<G, RR>(a, n1, gl, ns);
        if (cell_lane) fetch_cell(n1, ncp, nper);
      }
      if (idx(b + 2 * W) < count) n2 = a.rec[p3];
      if (idx(b + 3 * W) < count) p3 = pull_pos(a, idx(b + 3 * W));
      take_cell();
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
// data) is set up once per block, and the next block's record, slots, cell pack and
// periodic source are loaded when a block starts, so they overlap its waits and a block
// waits only for its neighbours' words (a cell pack loaded in the block itself would
// hold back the word loads: whether the cell is active decides which lanes load).  Same
// additions in the same order as the other variants.
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
  // the cell pack {(float) attenuation or inactive mark, source} of a block's task (every
  // lane above level 0, else the leader) and its periodic source (leader, periodic tasks)
  const bool cell_lane = check_level || gl == 0;
  uint2 cp = make_uint2(0u, 0u);
  float per = 0.f;
  auto load_cell = [&](const uint4& r, uint2& pk, float& pr) {
    pk = __ldg(a.cellpack + r.x);
    pr = (gl == 0 && rec_periodic(r)) ? __ldcg(a.periodic + rec_dir(r) * a.Np + r.x) : 0.f;
  };
  if (idx(b) < count && cell_lane) load_cell(cur, cp, per);
  uint32_t solved = 0, attempts = 0;
  bool stop = false;
  while (!stop && b * kGroups < count) {
    // next block's pipeline stages, issued now
    uint2 ns[kPullRounds];
    uint4 n2 = z;
    uint32_t p3 = 0;
    uint2 ncp = make_uint2(0u, 0u);
    float nper = 0.f;
    if (idx(b + W) < count) {
      load_slots(a, n1, gl, ns);
      if (cell_lane) load_cell(n1, ncp, nper);
    }
    if (idx(b + 2 * W) < count) n2 = a.rec[p2];
    if (idx(b + 3 * W) < count) p3 = pull_pos(a, idx(b + 3 * W));
    // this block's task
    bool have = idx(b) < count;
    const uint32_t t = rec_dir(cur) * a.Np + cur.x;
    float src = 0.f, att = 0.f;
    if (have && cell_lane) {
      if (cp.x == kInactiveCell) {  // inactive: keep q, stamp the word
        if (gl == 0) {
          const unsigned long long own = ld_relaxed_u64(word_ptr(a.qe, t));
          st_relaxed_u64(word_ptr(a.qe, t), (own & 0xffffffffull) | ((unsigned long long)((sweep << 1) | 1u) << 32));
        }
        have = false;
      } else if (gl == 0) {
        src = __uint_as_float(cp.y);
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
    cp = ncp;
    per = nper;
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

}  // namespace swk

namespace swk {

// ---------------------------------------------------------------------------------------
// The nested-loop lockstep kernel with its shape as template parameters, for the
// autotuner: G lanes per task (4, 8 or 16: 8, 4 or 2 tasks per warp block) and the
// prefetch depth PF of the slots and cell data (1: the next block's, 2: also the one
// after; 3: the next block's cell data, its slots only into L1) and CS, whether the
// records and slots are loaded with the streaming (evict-first) cache hint.  Whatever the shape, the incoming rate is summed in one fixed order, so every
// shape gives the same bits: eight partial sums, partial j over the slots j, j + 8 (and
// j + 16, j + 24, ... for tasks with more than 16 upwind faces) by fused multiply-adds
// in slot order, then combined pairwise as an eight-lane butterfly (xor 1, 2, 4).  With
// G = 4 a lane holds partials j and j + 4; with G = 16 lanes 8..15 hand their slot's
// weight and word to lanes 0..7.
template <int kMinBlocks, int G, int PF, bool CS = false>
__global__ void __launch_bounds__(kPullThreads, kMinBlocks) k_sweep_pull_lockg(PullArgs a) {
  static_assert(G == 4 || G == 8 || G == 16, "4, 8 or 16 lanes per task");
  static_assert(PF == 1 || PF == 2 || PF == 3, "prefetch depth 1 or 2, or 3: next slots into L1 only");
  static_assert(kPullGroup == 8 && kPullRounds == 2, "eight partial sums of two register slots");
  constexpr uint32_t kGroups = 32 / G;
  constexpr int V = G <= 8 ? 8 / G : 1;  // partial sums per lane
  constexpr int S = G <= 8 ? 2 * V : 1;  // slots per lane in registers
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t gl = lane & (G - 1);
  const uint32_t g = lane / G;
  const uint32_t gmask = (uint32_t)(((1ull << G) - 1ull) << (g * G));
  const uint32_t W = gridDim.x * (kPullThreads / 32);
  const uint32_t count = a.act ? *a.act_count : a.count;
  const uint32_t sweep = sweep_number(a);
  const bool check_level = a.act == nullptr && a.current_level > 0;
  const bool sparse = a.act != nullptr && a.current_level > 0;
  uint32_t b = blockIdx.x * (kPullThreads / 32) + threadIdx.x / 32;
  auto idx = [&](uint32_t bb) { return bb * kGroups + g; };
  // CS: records and slots are read once per sweep, so they are loaded with the
  // evict-first (streaming) hint and leave L2 to the words and cell packs
  auto ld_rec = [&](uint32_t pos) -> uint4 { return CS ? __ldcs(a.rec + pos) : a.rec[pos]; };
  // slot index held in register k of this lane
  auto slot_of = [&](int k) -> uint32_t {
    if constexpr (G <= 8) return gl + (uint32_t)(k / 2) * G + (uint32_t)(k & 1) * 8u;
    return gl;
  };
  auto load_s = [&](const uint4& r, uint2 (&s)[S]) {
    const uint32_t n = rec_count(r);
    const uint2* base = a.slots + rec_offset(r);
#pragma unroll
    for (int k = 0; k < S; ++k)
      if (slot_of(k) < n) s[k] = CS ? __ldcs(base + slot_of(k)) : __ldg(base + slot_of(k));
  };
  // PF = 3: the next block's slots are only brought into L1 (three lanes of the group
  // touch the lines of its first 24 slots) and loaded from there when the block starts,
  // which keeps them out of the registers
  auto prefetch_s = [&](const uint4& r) {
    const uint32_t n = rec_count(r);
    if (gl < 3 && gl * 8 < n)
      asm volatile("prefetch.global.L1 [%0];" ::"l"(a.slots + rec_offset(r) + gl * 8));
  };
  const bool cell_lane = check_level || gl == 0;
  auto load_cell = [&](const uint4& r, uint2& pk, float& pr) {
    pk = __ldg(a.cellpack + r.x);
    pr = (gl == 0 && rec_periodic(r)) ? __ldcg(a.periodic + rec_dir(r) * a.Np + r.x) : 0.f;
  };
  const uint4 z = make_uint4(0u, 0u, 0u, 0u);
  // pipeline: block b (cur, s, cp, per), b + W (n1; with PF = 2 also its slots and cell
  // data), b + 2W (record n2), position of b + 3W
  uint4 cur = z, n1 = z, n2 = z;
  uint2 s[S], s1[S];
  uint2 cp = make_uint2(0u, 0u), cp1 = make_uint2(0u, 0u);
  float per = 0.f, per1 = 0.f;
  uint32_t p3 = 0;
  if (idx(b) < count) cur = ld_rec(pull_pos(a, idx(b)));
  if (idx(b + W) < count) n1 = ld_rec(pull_pos(a, idx(b + W)));
  if constexpr (PF == 2) {
    if (idx(b + 2 * W) < count) n2 = ld_rec(pull_pos(a, idx(b + 2 * W)));
    if (idx(b + 3 * W) < count) p3 = pull_pos(a, idx(b + 3 * W));
  } else {
    if (idx(b + 2 * W) < count) p3 = pull_pos(a, idx(b + 2 * W));
  }
  load_s(cur, s);
  if (idx(b) < count && cell_lane) load_cell(cur, cp, per);
  if constexpr (PF == 2) {
    if (idx(b + W) < count) {
      load_s(n1, s1);
      if (cell_lane) load_cell(n1, cp1, per1);
    }
  }
  uint32_t solved = 0, attempts = 0;
  bool stop = false;
  while (!stop && b * kGroups < count) {
    // the next stages, issued before this block's words
    uint2 sn[S];
    uint2 cpn = make_uint2(0u, 0u);
    float pern = 0.f;
    uint4 nn = z;
    uint32_t pn = 0;
    if constexpr (PF == 2) {
      if (idx(b + 2 * W) < count) {
        load_s(n2, sn);
        if (cell_lane) load_cell(n2, cpn, pern);
      }
      if (idx(b + 3 * W) < count) nn = ld_rec(p3);
      if (idx(b + 4 * W) < count) pn = pull_pos(a, idx(b + 4 * W));
    } else {
      if (idx(b + W) < count) {
        if constexpr (PF == 3)
          prefetch_s(n1);
        else
          load_s(n1, sn);
        if (cell_lane) load_cell(n1, cpn, pern);
      }
      if (idx(b + 2 * W) < count) nn = ld_rec(p3);
      if (idx(b + 3 * W) < count) pn = pull_pos(a, idx(b + 3 * W));
    }
    bool have = idx(b) < count;
    const uint32_t t = rec_dir(cur) * a.Np + cur.x;
    float src = 0.f, att = 0.f;
    if (have && cell_lane) {
      if (cp.x == kInactiveCell) {  // inactive: keep q, stamp the word
        if (gl == 0) {
          const unsigned long long own = ld_relaxed_u64(word_ptr(a.qe, t));
          st_relaxed_u64(word_ptr(a.qe, t), (own & 0xffffffffull) | ((unsigned long long)((sweep << 1) | 1u) << 32));
        }
        have = false;
      } else if (gl == 0) {
        src = __uint_as_float(cp.y);
        att = __uint_as_float(cp.x);
      }
    }
    const uint32_t n_up = have ? rec_count(cur) : 0u;
    const uint32_t dnp = rec_dir(cur) * a.Np;
    bool pk[S], keep[S], need[S];
    unsigned long long x[S];
#pragma unroll
    for (int k = 0; k < S; ++k) {
      pk[k] = slot_of(k) < n_up;
      keep[k] = sparse && pk[k] && a.level[s[k].x - dnp] < (uint32_t)a.current_level;
      need[k] = pk[k];
      x[k] = 0;
    }
    const bool big = n_up > 16u;
    unsigned long long w0 = 0;
    uint32_t wait_ns = 32;
    while (true) {
#pragma unroll
      for (int k = 0; k < S; ++k)
        if (need[k]) x[k] = ld_relaxed_u64(word_ptr(a.qe, s[k].x));
      bool bad = false;
#pragma unroll
      for (int k = 0; k < S; ++k) {
        need[k] = pk[k] && !keep[k] && !word_current(x[k], sweep);
        bad = bad || need[k];
      }
      // the eight partial sums of this lane (G <= 8: V of them; G = 16: lanes 0..7 one)
      float part[V];
      if constexpr (G <= 8) {
#pragma unroll
        for (int v = 0; v < V; ++v) {
          part[v] = pk[2 * v] ? fmaf(__uint_as_float(s[2 * v].y), __uint_as_float((uint32_t)x[2 * v]), 0.f) : 0.f;
          if (pk[2 * v + 1])
            part[v] = fmaf(__uint_as_float(s[2 * v + 1].y), __uint_as_float((uint32_t)x[2 * v + 1]), part[v]);
        }
      } else {
        const float wt = pk[0] ? __uint_as_float(s[0].y) : 0.f;
        const float xv = __uint_as_float((uint32_t)x[0]);
        const float wt_hi = __shfl_down_sync(0xffffffffu, wt, 8, 16);
        const float x_hi = __shfl_down_sync(0xffffffffu, xv, 8, 16);
        const bool p_hi = __shfl_down_sync(0xffffffffu, (int)pk[0], 8, 16) != 0;
        part[0] = pk[0] ? fmaf(wt, xv, 0.f) : 0.f;
        if (p_hi && gl < 8) part[0] = fmaf(wt_hi, x_hi, part[0]);
      }
      if (big) {
#pragma unroll
        for (int v = 0; v < V; ++v) {
          const uint32_t j0 = (G <= 8 ? gl + (uint32_t)v * G : gl) + 16u;
          if (G == 16 && gl >= 8) break;
          for (uint32_t j = j0; j < n_up; j += 8) {
            const uint2 sj = a.slots[rec_offset(cur) + j];
            const unsigned long long wn = ld_relaxed_u64(word_ptr(a.qe, sj.x));
            bad = bad || (!word_current(wn, sweep) && !(sparse && a.level[sj.x - dnp] < (uint32_t)a.current_level));
            part[v] = fmaf(__uint_as_float(sj.y), __uint_as_float((uint32_t)wn), part[v]);
          }
        }
      }
      const uint32_t badmask = __ballot_sync(0xffffffffu, bad);
      // butterfly over the eight partials: xor 1 and 2 between lanes (xor 4 between lanes
      // for G >= 8, within the lane for G = 4)
      float in;
      if constexpr (G == 4) {
#pragma unroll
        for (int o = 1; o < 4; o <<= 1) {
          part[0] += __shfl_xor_sync(0xffffffffu, part[0], o, 4);
          part[1] += __shfl_xor_sync(0xffffffffu, part[1], o, 4);
        }
        in = part[0] + part[1];
      } else {
        in = part[0];
#pragma unroll
        for (int o = 1; o < 8; o <<= 1) in += __shfl_xor_sync(0xffffffffu, in, o, G);
      }
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
    if constexpr (PF == 2) {
#pragma unroll
      for (int k = 0; k < S; ++k) {
        s[k] = s1[k];
        s1[k] = sn[k];
      }
      cp = cp1;
      per = per1;
      cp1 = cpn;
      per1 = pern;
      n1 = n2;
      n2 = nn;
    } else {
      if constexpr (PF == 3) {
        if (idx(b) < count) load_s(cur, s);
      } else {
#pragma unroll
        for (int k = 0; k < S; ++k) s[k] = sn[k];
      }
      cp = cpn;
      per = pern;
      n1 = nn;
    }
    p3 = pn;
  }
  unsigned long long ts = solved, ta = attempts;
  for (int o = 16; o > 0; o >>= 1) {
    ts += __shfl_xor_sync(0xffffffffu, ts, o);
    ta += __shfl_xor_sync(0xffffffffu, ta, o);
  }
  if (lane == 0 && ts) atomicAdd(&a.ctl->tasks, ts);
  if (lane == 0 && ta) atomicAdd(&a.ctl->attempts, ta);
}

}  // namespace swk
