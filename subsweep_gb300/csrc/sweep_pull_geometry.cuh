// The geometry pull sweep kernel of the compact state (pull path).
// Part of the pull-form transport of the mixed path; the shared definitions
// (PullArgs, words, records) are in sweep_pull.cuh, the grid barrier in
// sweep_pull_wavefront.cuh.
#pragma once

#include "sweep_pull.cuh"
#include "sweep_pull_wavefront.cuh"

namespace swk {

// ---------------------------------------------------------------------------------------
// Compact state: grids whose per-position records and upwind slots (~78 bytes per task)
// do not fit next to the rest of the state, or whose tasks exceed 32-bit ids, keep only
// the words (by task), the incoming and periodic rates and the schedule.  The sweep
// then classifies each task's faces itself, as the record and slot kernels do once per
// grid: one thread per task, segment by segment of the task spaces' levelled schedules
// (segment k of every space together: the spaces never depend on one another), with a
// grid barrier between segments (cooperative launch), so every upwind word is final
// when it is read and no readiness test is needed.  Every position is visited; a task whose cell is inactive in the sweep keeps its word (its flux
// persists, as in the reference), and nothing in this state tests sweep numbers inside
// a sweep.
//
// A task walks its cell's faces in face order: the FP32 effective area s of each face
// (exact sign as everywhere), s > 0 summed into the total downwind area, each upwind
// LOCAL face k adding |s| q(n, d) into partial k mod 8 by FMA, an upwind LOCAL_PERIODIC
// face flagging the periodic source.  The faces are taken eight upwind faces at a time,
// so eight upwind words are in flight per thread.  Partial sums, their combination
// ((p0 + p1) + (p2 + p3)) + ((p4 + p5) + (p6 + p7)), 1 / A_down and the commit are those
// of the record kernels, so both states give the same bits.
constexpr int kGeoThreads = 1024;  // one block per SM: few arrivals at each grid barrier
constexpr int kGeoMaxSpaces = 8;

// The arrays of one task space (directions [d0, d1)): its schedule, and its slices of
// the per-task arrays and of the directions.  Task ids in a space are local to it.
struct GeoSpace {
  const uint32_t* order;
  const uint32_t* lvl;  // segment offsets into order [num_levels + 1]
  uint32_t num_levels;
  unsigned long long* qe;
  float* inc;
  const float* periodic;
  const float* dir32;
  const double* dir64;
};

// One launch over every task space: segment k of all spaces, then a grid barrier.
struct GeoArgs {
  PullArgs a;  // grid, cells, threshold, control block, sweep number
  GeoSpace sp[kGeoMaxSpaces];
  int num_spaces;
  uint32_t max_levels;
};

__device__ __forceinline__ void geo_solve(const PullArgs& a, const GeoSpace& sp, uint32_t t, uint32_t sweep,
                                          unsigned long long& solved) {
  const uint32_t d = t / a.Np, c = t - d * a.Np;
  // inactive in this sweep: the level (1 byte per cell, L2-resident) decides before the
  // cell pack (8 bytes per cell) is read; attenuation marks exactly these cells inactive
  if (a.level[c] < (uint32_t)a.current_level) return;
  const uint2 cp = __ldg(a.cellpack + c);  // {(float) attenuation, source / D}
  const float fx = sp.dir32[3 * d], fy = sp.dir32[3 * d + 1], fz = sp.dir32[3 * d + 2];
  const double dx = sp.dir64[3 * d], dy = sp.dir64[3 * d + 1], dz = sp.dir64[3 * d + 2];
  const size_t dnp = (size_t)d * a.Np;
  const uint32_t end = a.off[c + 1];
  uint32_t f = a.off[c];
  float part[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) part[j] = 0.f;
  float area_down = 0.f;
  bool periodic_up = false;
  bool more = true;
  while (more) {  // one round: the next eight upwind LOCAL faces
    float w[8], q[8];
    bool have[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      have[j] = false;
      w[j] = 0.f;
      q[j] = 0.f;
      while (f < end) {
        const uint4 g = __ldg(a.geo16 + f);
        const float s = face_eff(g, fx, fy, fz, a.geo64 + f, dx, dy, dz);
        ++f;
        if (s > 0.f) {
          area_down += s;
        } else if (s < 0.f) {
          const uint32_t kind = g.w >> kKindShift;
          if (kind == kKindLocal) {
            w[j] = -s;
            q[j] = __uint_as_float((uint32_t)ld_relaxed_u64(word_ptr(sp.qe, dnp + (g.w & kNbrMask))));
            have[j] = true;
            break;
          }
          if (kind == kKindPeriodic) periodic_up = true;
        }
      }
    }
#pragma unroll
    for (int j = 0; j < 8; ++j)
      if (have[j]) part[j] = fmaf(w[j], q[j], part[j]);
    more = have[7] && f < end;
  }
  const float in = ((part[0] + part[1]) + (part[2] + part[3])) + ((part[4] + part[5]) + (part[6] + part[7]));
  const float inv = area_down > 0.f ? 1.0f / area_down : 0.f;
  const float per = periodic_up ? __ldcg(sp.periodic + t) : 0.f;
  const float rt = (in + __uint_as_float(cp.y)) + per;                  // Site::get_rate, site.rs:53-56
  const float out = (rt < a.threshold) ? 0.f : rt * __uint_as_float(cp.x);  // get_outgoing_rate
  sp.inc[t] = in;
  st_relaxed_u64(word_ptr(sp.qe, t), pack_qe(out * inv, sweep));
  ++solved;
}

// grid: every block resident (cooperative); ctl->head zeroed before the launch
template <int kMinBlocks>
__global__ void __launch_bounds__(kGeoThreads, kMinBlocks) k_sweep_pull_geo(GeoArgs g) {
  __shared__ int flag;
  const PullArgs& a = g.a;
  const uint32_t T = gridDim.x * kGeoThreads;
  const uint32_t j = blockIdx.x * kGeoThreads + threadIdx.x;
  const uint32_t sweep = sweep_number(a);
  unsigned long long solved = 0;
  for (uint32_t k = 0; k < g.max_levels; ++k) {
    uint32_t lo[kGeoMaxSpaces], n[kGeoMaxSpaces], total = 0;
#pragma unroll
    for (int s = 0; s < kGeoMaxSpaces; ++s) {
      lo[s] = 0;
      n[s] = 0;
      if (s < g.num_spaces && k < g.sp[s].num_levels) {
        lo[s] = __ldg(g.sp[s].lvl + k);
        n[s] = __ldg(g.sp[s].lvl + k + 1) - lo[s];
      }
      total += n[s];
    }
    for (uint32_t i = j; i < total; i += T) {  // position i of the spaces' segments k, concatenated
      uint32_t r = i;
      int s = 0;
      while (r >= n[s]) r -= n[s++];
      geo_solve(a, g.sp[s], __ldg(g.sp[s].order + lo[s] + r), sweep, solved);
    }
    if (k + 1 < g.max_levels && !wave_barrier(a, (unsigned long long)(k + 1) * gridDim.x, &flag)) break;
  }
  const uint32_t lane = threadIdx.x & 31;
  for (int o = 16; o > 0; o >>= 1) solved += __shfl_xor_sync(0xffffffffu, solved, o);
  if (lane == 0 && solved) {
    atomicAdd(&a.ctl->tasks, solved);
    atomicAdd(&a.ctl->attempts, solved);
  }
}

}  // namespace swk
