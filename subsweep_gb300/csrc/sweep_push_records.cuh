// Precomputed downwind fractions for the FP64 push transport.
//
// Sweep::solve_task (src/sweep/mod.rs:423-485) hands each downwind face the share
// corr * (eff_f / total) of a task's outgoing-rate correction, with eff_f = area_f
// (n_f . d) and total the sum of eff over the downwind faces in face order (boundary
// faces included).  Both depend on geometry only, so they are computed once per grid:
// for every schedule position, the LOCAL and LOCAL_PERIODIC downwind faces in face
// order as {target = neighbour | kind << 30, fraction = eff_f / total} (FP64, the same
// roundings as the transport kernel computes them), stored in position order with
// 64-bit offsets.  The transport then multiplies the correction by the stored
// fraction, so every contribution is the same double as when computed on the fly,
// without the FP64 dot products and divisions of the geometry path.
//
// Record per position: {task, slot offset low, count | slot offset high << 8, 0}.
#pragma once

#include "sweep_device.cuh"

namespace swk {

__device__ __forceinline__ unsigned long long prec_offset(const uint4& r) {
  return (unsigned long long)r.y | ((unsigned long long)(r.z >> 8) << 32);
}
__device__ __forceinline__ uint32_t prec_count(const uint4& r) { return r.z & 0xffu; }

// Exact classification and effective area of face j of cell c for direction d, as
// solve_group evaluates them.  Returns eff > 0 for a downwind face, 0 otherwise.
template <typename R>
__device__ __forceinline__ double push_eff(const SweepArgs<R>& a, uint32_t f, double dx, double dy, double dz,
                                           float fx, float fy, float fz) {
  const float4 g = a.geo32[f];
  const float s = g.x * fx + g.y * fy + g.z * fz;
  if (face_sign(s, a.geo64 + f, dx, dy, dz, a.guard) <= 0) return 0.0;
  const Geo64 h = a.geo64[f];
  return h.w * dot64(h, dx, dy, dz);
}

// Per position: the number of LOCAL / LOCAL_PERIODIC downwind faces.
template <typename R>
__global__ void k_push_rec_count(SweepArgs<R> a, const uint32_t* order, uint32_t total, uint4* rec) {
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < total; p += gridDim.x * blockDim.x) {
    const uint32_t t = order[p];
    const uint32_t d = t / a.Np, c = t - d * a.Np;
    const double dx = a.dir64[3 * d], dy = a.dir64[3 * d + 1], dz = a.dir64[3 * d + 2];
    const float fx = a.dir32[3 * d], fy = a.dir32[3 * d + 1], fz = a.dir32[3 * d + 2];
    uint32_t n = 0;
    for (uint32_t f = a.off[c]; f < a.off[c + 1]; ++f)
      if (push_eff(a, f, dx, dy, dz, fx, fy, fz) > 0.0 && (a.nbr[f] >> kKindShift) != kKindBoundary) ++n;
    rec[p] = make_uint4(t, 0u, n, 0u);
  }
}

// per chunk of kCompactChunk positions: the total count
template <typename R>
__global__ void __launch_bounds__(kCompactThreads) k_push_chunk_sums(const uint4* rec, uint32_t total,
                                                                     uint32_t* chunk) {
  const uint32_t first = blockIdx.x * kCompactChunk + threadIdx.x * kCompactPer;
  uint32_t n = 0;
  for (int k = 0; k < kCompactPer; ++k)
    if (first + k < total) n += prec_count(rec[first + k]);
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

// exclusive 64-bit scan of the chunk totals (one block of 1024); grand total at out[n]
template <typename R>
__global__ void __launch_bounds__(1024) k_push_scan64(const uint32_t* chunk, uint32_t n, unsigned long long* out) {
  __shared__ unsigned long long warp_sum[32];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long carry = 0;
  for (uint32_t base = 0; base < n; base += 1024) {
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
    for (int w = 0; w < 32; ++w) {
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

// Offsets into the records and the slots: targets and fractions in face order.  Writes
// at most the counted number per position; a mismatch flags kErrRecords.
template <typename R>
__global__ void __launch_bounds__(kCompactThreads) k_push_slots(SweepArgs<R> a, uint4* rec, uint32_t total,
                                                                const unsigned long long* chunk_off,
                                                                uint32_t* tgt, double* frac) {
  const uint32_t first = blockIdx.x * kCompactChunk + threadIdx.x * kCompactPer;
  uint32_t mine = 0;
  for (int k = 0; k < kCompactPer; ++k)
    if (first + k < total) mine += prec_count(rec[first + k]);
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
    const uint32_t n = prec_count(r);
    r.y = (uint32_t)o;
    r.z = n | ((uint32_t)(o >> 32) << 8);
    rec[p] = r;
    const uint32_t t = r.x;
    const uint32_t d = t / a.Np, c = t - d * a.Np;
    const double dx = a.dir64[3 * d], dy = a.dir64[3 * d + 1], dz = a.dir64[3 * d + 2];
    const float fx = a.dir32[3 * d], fy = a.dir32[3 * d + 1], fz = a.dir32[3 * d + 2];
    const uint32_t beg = a.off[c], end = a.off[c + 1];
    double tot = 0.0;  // face order, zeros for the other faces (solve_group)
    for (uint32_t f = beg; f < end; ++f) tot += push_eff(a, f, dx, dy, dz, fx, fy, fz);
    uint32_t written = 0;
    for (uint32_t f = beg; f < end; ++f) {
      const double eff = push_eff(a, f, dx, dy, dz, fx, fy, fz);
      const uint32_t nb = a.nbr[f];
      if (eff > 0.0 && (nb >> kKindShift) != kKindBoundary) {
        if (written < n) {
          tgt[o + written] = nb;
          frac[o + written] = eff / tot;
        }
        ++written;
      }
    }
    if (written != n) atomicOr(&a.ctl->error, kErrRecords);
    o += n;
  }
}

// Solve one task per group of kGroup lanes with the precomputed fractions: the leader
// forms the outgoing rate and the correction (as solve_group); lane j adds
// corr * fraction to the targets of slots j, j + kGroup, ... and decrements the LOCAL
// targets' dependency counters with release semantics.
template <typename R>
__device__ __forceinline__ void solve_group_rec(const SweepArgs<R>& a, bool have, const uint4& r,
                                                const uint32_t* tgt, const double* frac) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t gl = lane & (kGroup - 1);
  const uint32_t t = r.x;
  const uint32_t d = t / a.Np, c = t - d * a.Np;
  R corr = R(0);
  if (have && gl == 0) {
    R inc = __ldcg(a.incoming + t);
    const R per = __ldcg(a.periodic + t);
    const R outo = a.outgoing[t];
    const double att = a.att[c];
    const R src = a.src_dir[c];
    if (inc < R(0)) {  // Photons::make_positive (chemistry/mod.rs:61-65)
      inc = R(0);
      a.incoming[t] = inc;
    }
    const R rt = (inc + src) + per;  // Site::get_rate, site.rs:53-56
    const R out_new = (rt < a.threshold) ? R(0) : rt * R(att);
    corr = out_new - outo;
    a.outgoing[t] = out_new;
  }
  corr = __shfl_sync(0xffffffffu, corr, 0, kGroup);
  const uint32_t n = have ? prec_count(r) : 0u;
  const unsigned long long off = prec_offset(r);
  for (uint32_t k = gl; k < n; k += kGroup) {
    const uint32_t nb = tgt[off + k];
    const R w = corr * R(frac[off + k]);
    const uint32_t tn = d * a.Np + (nb & kNbrMask);
    if ((nb >> kKindShift) == kKindPeriodic) {
      atomicAdd(a.pending + tn, w);
    } else {
      atomicAdd(a.incoming + tn, w);
      atom_sub_release(a.counters + (tn >> 2), 1u << (8u * (tn & 3u)));
    }
  }
  __syncwarp();
}

// k_sweep_sched over the precomputed records (cooperative launch): group g solves the
// positions g, g + G, ... whose cells are active, each once its dependency counter
// reads zero; the record of the next position is loaded while the group waits.
template <typename R>
__global__ void __launch_bounds__(kLevelThreads) k_sweep_sched_rec(SweepArgs<R> a, const uint4* rec,
                                                                    uint32_t total_sched, const uint32_t* tgt,
                                                                    const double* frac) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t gl = lane & (kGroup - 1);
  const uint32_t groups = gridDim.x * (kLevelThreads / kGroup);
  uint32_t i = blockIdx.x * (kLevelThreads / kGroup) + (threadIdx.x / kGroup);
  const uint8_t* cnt8 = reinterpret_cast<const uint8_t*>(a.counters);
  unsigned long long solved = 0;
  bool stop = false;
  uint4 nxt = i < total_sched ? rec[i] : make_uint4(0u, 0u, 0u, 0u);
  while (!stop && __any_sync(0xffffffffu, i < total_sched)) {
    const uint4 r = nxt;
    bool pending = false;
    if (i < total_sched) {
      const uint32_t t = r.x;
      const uint32_t c = t - (t / a.Np) * a.Np;
      pending = a.level[c] >= a.current_level;
    }
    if (i + groups < total_sched) nxt = rec[i + groups];
    unsigned long long w0 = 0;
    uint32_t wait_ns = 32;
    while (__any_sync(0xffffffffu, pending)) {
      bool ready = false;
      if (pending && gl == 0) {
        uint32_t v;
        asm volatile("ld.relaxed.gpu.global.u8 %0, [%1];" : "=r"(v) : "l"(cnt8 + r.x) : "memory");
        ready = (v & 0xffu) == 0u;
      }
      ready = __shfl_sync(0xffffffffu, ready ? 1 : 0, 0, kGroup) != 0;
      if (__any_sync(0xffffffffu, ready)) {
        solve_group_rec<R>(a, ready, r, tgt, frac);
        if (ready) {
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

}  // namespace swk
