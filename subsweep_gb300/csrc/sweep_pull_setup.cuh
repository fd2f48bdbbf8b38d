// Task records, upwind slots and the compaction of active positions (pull path).
// Part of the pull-form transport of the mixed path; the shared definitions
// (PullArgs, words, records) are in sweep_pull.cuh.
#pragma once

#include "sweep_pull.cuh"

namespace swk {

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
        if (written < n_up)
          slots[o + written] = make_uint2(a.pos_of_task[dnp + (g.w & kNbrMask)], __float_as_uint(-sj));
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

}  // namespace swk
