// Pull-form transport of the mixed-precision path (FP32 rates).
//
// The reference distributes each task's outgoing-rate *correction* over its downwind
// faces (push, src/sweep/mod.rs:423-485).  Summed over a sweep's history, the incoming
// rate of (cell c, direction d) is the sum over c's upwind LOCAL faces f (neighbour n)
// of  area_f |n_f . d| * out(n, d) / A(n, d),  where A(n, d) is n's total effective
// downwind area.  This path evaluates that sum directly: every task publishes
//   q(c, d) = out(c, d) / A(c, d)
// together with the number of the sweep that produced it, as one 64-bit word, and a
// task gathers q from its upwind neighbours.  A neighbour that is active in the
// current sweep is ready once its word carries the current sweep number; an inactive
// one keeps the q of its last solve (its flux persists, as in the reference).  The
// 64-bit word is written and read in single accesses, so there are no atomics, no
// counters and no fences on this path.  Tasks are visited in the levelled schedule
// order, every upwind task lies at an earlier schedule position, and a task whose
// inputs are not all published yet is retried.
//
// Geometry is one 16-byte load per face: {area * n (FP32, area scaled by 2^-k),
// neighbour | kind << 30}.  The sign of n . d decides up/downwind exactly: the FP32 dot
// decides when it exceeds its rounding bound, else the FP64 normal does.
#pragma once

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
  float* incoming;
  const float* periodic;
  unsigned long long* qe;   // {q (float bits) low, sweep number high}
  SweepCtl* ctl;
  int current_level;
  uint32_t epoch;
  unsigned long long timeout_ns;
};

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ unsigned long long pack_qe(float q, uint32_t epoch) {
  return ((unsigned long long)epoch << 32) | (unsigned long long)__float_as_uint(q);
}

// Signed effective area s = (area n) . d of one face, with the exact sign of n . d:
// returns +|s| downwind, -|s| upwind, 0 when n . d == 0.
__device__ __forceinline__ float face_eff(const uint4& g, float fx, float fy, float fz, const Geo64* g64,
                                          double dx, double dy, double dz) {
  const float ax = __uint_as_float(g.x), ay = __uint_as_float(g.y), az = __uint_as_float(g.z);
  const float s = ax * fx + ay * fy + az * fz;
  const float bound = 8.0e-7f * (fabsf(ax * fx) + fabsf(ay * fy) + fabsf(az * fz));
  if (s > bound) return s;
  if (s < -bound) return s;
  const double e = dot64(*g64, dx, dy, dz);
  if (e > 0.0) return fabsf(s);
  if (e < 0.0) return -fabsf(s);
  return 0.0f;
}

constexpr int kPullThreads = 256;

// One attempt at the tasks of the warp's groups (kGroup lanes each).  Returns, per
// group, whether the task was committed (all active upwind inputs published).
__device__ __forceinline__ bool try_solve_pull(const PullArgs& a, bool have, uint32_t t) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t gl = lane & (kGroup - 1);
  uint32_t c = 0, d = 0, beg = 0, nf = 0;
  float per = 0.f, src = 0.f;
  double att = 0.0;
  if (have) {
    d = t / a.Np;
    c = t - d * a.Np;
    if (gl == 0) {
      beg = a.off[c];
      nf = a.off[c + 1] - beg;
      per = __ldcg(a.periodic + t);
      src = a.src_dir[c];
      att = a.att[c];
    }
  }
  beg = __shfl_sync(0xffffffffu, beg, 0, kGroup);
  nf = __shfl_sync(0xffffffffu, nf, 0, kGroup);
  float fx = 0.f, fy = 0.f, fz = 0.f;
  double dx = 0.0, dy = 0.0, dz = 0.0;
  if (have) {
    fx = a.dir32[3 * d]; fy = a.dir32[3 * d + 1]; fz = a.dir32[3 * d + 2];
    dx = a.dir64[3 * d]; dy = a.dir64[3 * d + 1]; dz = a.dir64[3 * d + 2];
  }
  uint32_t rounds = (nf + kGroup - 1) / kGroup;
  for (int o = 16; o > 0; o >>= 1) rounds = max(rounds, __shfl_xor_sync(0xffffffffu, rounds, o));
  float area_down = 0.f, in = 0.f;
  bool ok = true;
  for (uint32_t k = 0; k < rounds; ++k) {
    const uint32_t fl = gl + k * kGroup;
    if (fl >= nf) continue;
    const uint32_t f = beg + fl;
    const uint4 g = a.geo16[f];
    const float s = face_eff(g, fx, fy, fz, a.geo64 + f, dx, dy, dz);
    if (s > 0.f) {
      area_down += s;
    } else if (s < 0.f && (g.w >> kKindShift) == kKindLocal) {
      const uint32_t n = g.w & kNbrMask;
      const unsigned long long w = ld_relaxed_u64(a.qe + (size_t)d * a.Np + n);
      if ((uint32_t)(w >> 32) != a.epoch && a.level[n] >= a.current_level) {
        ok = false;  // active upwind neighbour not solved yet in this sweep
      } else {
        in += -s * __uint_as_float((uint32_t)w);
      }
    }
  }
  // group reductions
  for (int o = 1; o < kGroup; o <<= 1) {
    area_down += __shfl_xor_sync(0xffffffffu, area_down, o, kGroup);
    in += __shfl_xor_sync(0xffffffffu, in, o, kGroup);
    ok = (__shfl_xor_sync(0xffffffffu, ok ? 1 : 0, o, kGroup) != 0) && ok;
  }
  const bool commit = have && ok;
  if (commit && gl == 0) {
    const float r = (in + src) + per;  // Site::get_rate, site.rs:53-56
    const float out = (r < a.threshold) ? 0.f : r * (float)att;  // get_outgoing_rate
    const float q = area_down > 0.f ? out / area_down : 0.f;
    a.incoming[t] = in;
    st_relaxed_u64(a.qe + t, pack_qe(q, a.epoch));
  }
  return commit;
}

// Scheduled pull sweep (cooperative launch; every block resident).  Group g visits
// schedule positions g, g + G, ...; inactive cells' tasks are skipped.
__global__ void __launch_bounds__(kPullThreads) k_sweep_pull(PullArgs a, const uint32_t* order, uint32_t total_sched) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t gl = lane & (kGroup - 1);
  const uint32_t groups = gridDim.x * (kPullThreads / kGroup);
  uint32_t i = blockIdx.x * (kPullThreads / kGroup) + (threadIdx.x / kGroup);
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
      const bool done = try_solve_pull(a, pending, t);
      if (__any_sync(0xffffffffu, done)) {
        if (done) {
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
    if (s < 0.f) in += -s * __uint_as_float((uint32_t)a.qe[(size_t)d * a.Np + (g.w & kNbrMask)]);
  }
  return in;
}

// Periodic sources after a sweep (snapshot semantics): for every cell with periodic
// faces and every direction, the flux arriving through its LOCAL_PERIODIC upwind faces.
__global__ void k_fold_pull(PullArgs a, float* periodic, const uint32_t* cells, uint32_t n_cells) {
  const size_t total = (size_t)n_cells * a.D;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const uint32_t d = (uint32_t)(i / n_cells);
    const uint32_t c = cells[i % n_cells];
    periodic[(size_t)d * a.Np + c] = gather_in(a, c, d, true);
  }
}

// Incoming rate of every (c, d) as the reference holds it after a step: the value
// stored by the task if it was solved in the step's last sweep, else gathered from the
// neighbours' current q (the reference keeps adding corrections to inactive cells).
__device__ __forceinline__ float current_incoming(const PullArgs& a, uint32_t c, uint32_t d, uint32_t last_epoch) {
  const size_t t = (size_t)d * a.Np + c;
  if ((uint32_t)(a.qe[t] >> 32) == last_epoch) return a.incoming[t];
  return gather_in(a, c, d, false);
}

__global__ void k_photon_rate_pull(PullArgs a, uint32_t last_epoch, double rate_scale, double* out) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < a.N; c += gridDim.x * blockDim.x) {
    double r = 0.0;
    for (int d = 0; d < a.D; ++d) r += (double)current_incoming(a, c, d, last_epoch);
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
      v = current_incoming(a, c, d, last_epoch);
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
      v = __uint_as_float((uint32_t)a.qe[t]) * area_down;
    }
    out[i] = (double)v * rate_scale;
  }
}

}  // namespace swk
