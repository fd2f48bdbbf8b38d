// Periodic fold and field export of the pull path.
// Part of the pull-form transport of the mixed path; the shared definitions
// (PullArgs, words, records) are in sweep_pull.cuh.
#pragma once

#include "sweep_pull.cuh"

namespace swk {

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
    if (s < 0.f)
      in = fmaf(-s, __uint_as_float((uint32_t)*word_ptr(a.qe, word_of_task(a, (size_t)d * a.Np + (g.w & kNbrMask)))),
                in);
  }
  return in;
}

// Periodic sources after a sweep (snapshot semantics): for every cell with periodic
// faces and every direction, the flux arriving through its LOCAL_PERIODIC upwind faces.
// Entry e = d * n_cells + (index of the cell in `cells`).  The upwind periodic faces of
// an entry are precomputed once per grid (k_fold_build: up to kFoldSlots of them, in
// face order, as {upwind task's word index, |area n . d|}); an entry with more is
// gathered from the geometry.  Both sum in face order with the same roundings.
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
        slots[e * kFoldSlots + n] =
            make_uint2((uint32_t)word_of_task(a, (size_t)d * a.Np + (g.w & kNbrMask)), __float_as_uint(-sf));
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
  if (cell_is_current) return a.inc[t];
  if ((uint32_t)(*word_ptr(a.qe, word_of_task(a, t)) >> 32) == (last_epoch << 1)) return a.inc[t];  // solved
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
      v = __uint_as_float((uint32_t)*word_ptr(a.qe, word_of_task(a, t))) * area_down;
    }
    out[i] = (double)v * rate_scale;
  }
}

}  // namespace swk
