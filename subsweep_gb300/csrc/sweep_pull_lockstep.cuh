// The warp-lockstep pull sweep kernels (pull path).
// Part of the pull-form transport of the mixed path; the shared definitions
// (PullArgs, words, records) are in sweep_pull.cuh.
#pragma once

#include "sweep_pull.cuh"

namespace swk {

// ---------------------------------------------------------------------------------------
// Scheduled pull sweep (cooperative launch; every block resident).
//
// Groups of G lanes (a shape parameter below) visit the active positions in schedule
// order.  For its current task a group gathers the upwind tasks' words through the
// task's slots and commits
//   in = sum_slots |area n . d| q(n, d),   out = (in + source/D + periodic) * attenuation
// (zero below the threshold), q = out / A_down, once every word carries the current
// sweep number; otherwise it retries.  The next positions' records, slots and cell data
// are loaded one block ahead, so a task waits only for its neighbours' words.  Every
// dependency lies at an earlier position and every warp walks its positions in order,
// so the earliest unsolved task can always commit.

__device__ __forceinline__ uint32_t pull_pos(const PullArgs& a, uint32_t j) { return a.act ? a.act[j] : j; }

// Cell of the task at schedule position p (the first word of its record): the level
// test of an upwind task in a sweep over a compacted list of active positions.
__device__ __forceinline__ uint32_t cell_at(const PullArgs& a, uint32_t p) {
  return __ldg(reinterpret_cast<const uint32_t*>(a.rec) + 4 * (size_t)p);
}


// ---------------------------------------------------------------------------------------
// The nested-loop lockstep kernel with its shape as template parameters, for the
// autotuner: G lanes per task (2, 4, 8 or 16: 16, 8, 4 or 2 tasks per warp block) and the
// prefetch depth PF of the slots and cell data (1: the next block's, 2: also the one
// after; 3: the next block's cell data, its slots only into L1) and CS, whether the
// records and slots are loaded with the streaming (evict-first) cache hint, and SP
// (with PF = 2), whether the next block's upwind words are loaded one block ahead, as
// soon as its slots are in registers: a block whose words were already current then
// commits without a round trip of its own, and a word that was not is loaded again.
// Whatever the shape, the incoming rate is summed in one fixed order, so every shape
// gives the same bits: eight partial sums, partial j over the slots j, j + 8 (and
// j + 16, j + 24, ... for tasks with more than 16 upwind faces) by fused multiply-adds
// in slot order, then combined pairwise as an eight-lane butterfly (xor 1, 2, 4).  With
// G = 4 a lane holds partials j and j + 4 (xor 4 within the lane); with G = 2 lane j
// holds partials j, j + 2, j + 4, j + 6 (xor 2 and 4 within the lane); with G = 16
// lanes 8..15 hand their slot's weight and word to lanes 0..7.
template <int kMinBlocks, int G, int PF, bool CS = false, bool SP = false>
__global__ void __launch_bounds__(kPullThreads, kMinBlocks) k_sweep_pull_lockg(PullArgs a) {
  static_assert(G == 2 || G == 4 || G == 8 || G == 16, "2, 4, 8 or 16 lanes per task");
  static_assert(PF == 1 || PF == 2 || PF == 3, "prefetch depth 1 or 2, or 3: next slots into L1 only");
  static_assert(kPullPartials == 8 && kPullRegSlots == 16, "eight partial sums over sixteen register slots");
  static_assert(!SP || PF == 2, "words one block ahead need the slots two blocks ahead");
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
  // SP: the upwind words of the next block (slots s1), loaded during this block
  unsigned long long xp[S], xq[S];
#pragma unroll
  for (int k = 0; k < S; ++k) xp[k] = xq[k] = 0ull;
  bool pre = false;
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
      if constexpr (SP) {
        if (idx(b + W) < count) {
          const uint32_t n1_up = rec_count(n1);
#pragma unroll
          for (int k = 0; k < S; ++k)
            if (slot_of(k) < n1_up) xq[k] = ld_relaxed_u64(word_ptr(a.qe, s1[k].x));
        }
      }
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
    const uint32_t pos = have ? pull_pos(a, idx(b)) : 0u;  // this task's word
    float src = 0.f, att = 0.f;
    if (have && cell_lane) {
      if (cp.x == kInactiveCell) {  // inactive: keep q, stamp the word
        if (gl == 0) {
          const unsigned long long own = ld_relaxed_u64(word_ptr(a.qe, pos));
          st_relaxed_u64(word_ptr(a.qe, pos), (own & 0xffffffffull) | ((unsigned long long)((sweep << 1) | 1u) << 32));
        }
        have = false;
      } else if (gl == 0) {
        src = __uint_as_float(cp.y);
        att = __uint_as_float(cp.x);
      }
    }
    const uint32_t n_up = have ? rec_count(cur) : 0u;
    bool pk[S], keep[S], need[S];
    unsigned long long x[S];
#pragma unroll
    for (int k = 0; k < S; ++k) {
      pk[k] = slot_of(k) < n_up;
      keep[k] = sparse && pk[k] && a.level[cell_at(a, s[k].x)] < (uint32_t)a.current_level;
      need[k] = pk[k];
      x[k] = 0;
    }
    const bool big = n_up > 16u;
    unsigned long long w0 = 0;
    uint32_t wait_ns = 32;
    bool first = true;
    while (true) {
      if (SP && first && pre) {  // the words loaded during the previous block
#pragma unroll
        for (int k = 0; k < S; ++k)
          if (need[k]) x[k] = xp[k];
      } else {
#pragma unroll
        for (int k = 0; k < S; ++k)
          if (need[k]) x[k] = ld_relaxed_u64(word_ptr(a.qe, s[k].x));
      }
      first = false;
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
            bad = bad ||
                  (!word_current(wn, sweep) && !(sparse && a.level[cell_at(a, sj.x)] < (uint32_t)a.current_level));
            part[v] = fmaf(__uint_as_float(sj.y), __uint_as_float((uint32_t)wn), part[v]);
          }
        }
      }
      const uint32_t badmask = __ballot_sync(0xffffffffu, bad);
      // butterfly over the eight partials: xor 1 between lanes; xor 2 between lanes for
      // G >= 4, within the lane for G = 2; xor 4 between lanes for G >= 8, within the lane
      // for G <= 4
      float in;
      if constexpr (G == 2) {
#pragma unroll
        for (int v = 0; v < 4; ++v) part[v] += __shfl_xor_sync(0xffffffffu, part[v], 1, 2);
        in = (part[0] + part[1]) + (part[2] + part[3]);
      } else if constexpr (G == 4) {
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
        commit_slot(a, pos, cur, pack_qe(out * __uint_as_float(cur.y), sweep), in);
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
      if constexpr (SP) {
#pragma unroll
        for (int k = 0; k < S; ++k) xp[k] = xq[k];
        pre = true;
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
