// The lane-per-task pull sweep kernel (pull path).
// Part of the pull-form transport of the mixed path; the shared definitions
// (PullArgs, words, records) are in sweep_pull.cuh, pull_pos in sweep_pull_lockstep.cuh.
#pragma once

#include "sweep_pull.cuh"
#include "sweep_pull_lockstep.cuh"

namespace swk {

// ---------------------------------------------------------------------------------------
// One lane per task, each lane with its own cursor (cooperative launch; every block
// resident).  Lane i of the grid takes the positions i, i + L, i + 2L, ... (L lanes in
// the grid) in order; for its current task it loads the cell pack and the upwind slots,
// then the upwind words, and commits once every word carries the sweep number (else it
// tries again; only its own task waits).  A warp executes one attempt of each of its 32
// lanes' tasks per iteration, so an instruction serves 32 tasks, where the group
// kernels serve 4 or 8; the lanes' positions start out consecutive, so their records
// and slots arrive in whole sectors.  Every dependency lies at an earlier position and
// the earliest unsolved task's lane can always commit, so the sweep cannot deadlock.
//
// The incoming rate is summed in the order of the group kernels, so every variant gives
// the same bits: eight partial sums, partial j over the slots j, j + 8, j + 16, ... by
// fused multiply-adds, combined as ((p0 + p1) + (p2 + p3)) + ((p4 + p5) + (p6 + p7)).
template <int kMinBlocks>
__global__ void __launch_bounds__(kPullThreads, kMinBlocks) k_sweep_pull_lane(PullArgs a) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t L = gridDim.x * kPullThreads;
  const uint32_t count = a.act ? *a.act_count : a.count;
  const uint32_t sweep = sweep_number(a);
  const bool check_level = a.act == nullptr && a.current_level > 0;
  const bool sparse = a.act != nullptr && a.current_level > 0;
  uint32_t p = blockIdx.x * kPullThreads + threadIdx.x;
  const uint4 z = make_uint4(0u, 0u, 0u, 0u);
  uint4 cur = z, nxt = z;
  uint32_t pn = 0;  // position index of the task after next
  if (p < count) cur = a.rec[pull_pos(a, p)];
  if (p + L < count) nxt = a.rec[pull_pos(a, p + L)];
  if (p + 2 * L < count) pn = pull_pos(a, p + 2 * L);
  bool have = p < count;
  uint32_t solved = 0, attempts = 0;
  unsigned long long w0 = 0;
  uint32_t wait_ns = 32;
  while (__any_sync(0xffffffffu, have)) {
    bool done = false;  // this lane's task committed (or stamped) in this iteration
    if (have) {
      const uint32_t t = rec_dir(cur) * a.Np + cur.x;
      const uint32_t dnp = rec_dir(cur) * a.Np;
      const uint2 cp = __ldg(a.cellpack + cur.x);
      const float per = rec_periodic(cur) ? __ldcg(a.periodic + t) : 0.f;
      const uint32_t n_up = rec_count(cur);
      const uint2* base = a.slots + rec_offset(cur);
      if (check_level && cp.x == kInactiveCell) {  // inactive: keep q, stamp the word
        const unsigned long long own = ld_relaxed_u64(word_ptr(a.qe, t));
        st_relaxed_u64(word_ptr(a.qe, t), (own & 0xffffffffull) | ((unsigned long long)((sweep << 1) | 1u) << 32));
        done = true;
      } else {
        ++attempts;
        // slot j goes into partial j mod 8, in increasing j, eight slots per round
        float part[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) part[k] = 0.f;
        bool bad = false;
        for (uint32_t j = 0; j < n_up; j += 8) {
          uint2 sl[8];
          unsigned long long w[8];
#pragma unroll
          for (int k = 0; k < 8; ++k)
            if (j + k < n_up) sl[k] = __ldg(base + j + k);
#pragma unroll
          for (int k = 0; k < 8; ++k) w[k] = (j + k < n_up) ? ld_relaxed_u64(word_ptr(a.qe, sl[k].x)) : 0ull;
#pragma unroll
          for (int k = 0; k < 8; ++k) {
            if (j + k < n_up) {
              bad = bad ||
                    (!word_current(w[k], sweep) && !(sparse && a.level[sl[k].x - dnp] < (uint32_t)a.current_level));
              part[k] = fmaf(__uint_as_float(sl[k].y), __uint_as_float((uint32_t)w[k]), part[k]);
            }
          }
        }
        if (!bad) {
          const float in = ((part[0] + part[1]) + (part[2] + part[3])) + ((part[4] + part[5]) + (part[6] + part[7]));
          const float att = __uint_as_float(cp.x), src = __uint_as_float(cp.y);
          const float rt = (in + src) + per;                      // Site::get_rate, site.rs:53-56
          const float out = (rt < a.threshold) ? 0.f : rt * att;  // get_outgoing_rate
          commit_slot(a.qe, t, pack_qe(out * __uint_as_float(cur.y), sweep), in);
          ++solved;
          done = true;
        }
      }
    }
    if (done) {  // advance this lane's cursor
      p += L;
      cur = nxt;
      have = p < count;
      if (p + L < count) nxt = a.rec[pn];
      if (p + 2 * L < count) pn = pull_pos(a, p + 2 * L);
    }
    if (__any_sync(0xffffffffu, done)) {
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
      break;
    }
    __nanosleep(wait_ns);
    wait_ns = min(wait_ns * 2, 256u);
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
