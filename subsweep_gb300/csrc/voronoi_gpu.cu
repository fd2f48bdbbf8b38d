// Voronoi tessellation on the GPU: the grid producer of csrc/grid_host.cpp (periodic
// or walled box, half-space clipping of a bounding polyhedron by the bisector planes of
// nearby generators in order of distance, stopped by the security radius), one thread
// per cell, then the face-neighbour CSR assembled on the device.
//
// Same face conventions as the host producer (and the reference, src/voronoi/cell.rs):
// normal = (p_neighbour + image shift - p_cell) * (1 / |.|), so the two sides of a face
// have bitwise negated normals; the area of a face is taken from the lower-index cell
// for both sides; size = cbrt(3 V / (4 pi)); faces of a cell sorted by (neighbour,
// image shift, wall).  Differences from the host producer: candidates are taken from
// bucket shells starting at Chebyshev radius 1 (the host starts at 2) and each shell's
// candidates are popped from a min-heap on (distance^2, index, shift), so the clipping
// order, and with it the last bits of vertex positions, can differ: the topology is the
// same, areas and volumes agree to rounding.
//
// Every per-thread buffer has a fixed capacity; a cell that would exceed one, or whose
// clipping becomes topologically inconsistent, is counted as failed and writes no faces.
// Compiled with -fmad=false: no fused multiply-adds, as the host producer.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "voronoi_gpu.h"

namespace vgpu {

constexpr int kMaxV = 192;     // vertices of a cell polyhedron, crossings of a clip included
constexpr int kMaxF = 72;      // faces
constexpr int kMaxFV = 640;    // vertex references over all faces
constexpr int kMaxCand = 512;  // candidates of one bucket shell
constexpr int kMaxOut = 64;    // faces per cell in the CSR (the sweep's limit)
constexpr int kMaxSeg = kMaxF;
constexpr int kThreads = 64;
constexpr int64_t kWallTagBase = -1;  // walls -1..-6 (x-, x+, y-, y+, z-, z+)

struct Poly {
  double x[kMaxV], y[kMaxV], z[kMaxV];
  int nv;
  uint16_t off[kMaxF + 1];
  uint8_t fv[kMaxFV];
  int64_t tag[kMaxF];
  int nf;
};

struct Cand {
  double d2;
  int32_t j;
  int32_t code;  // (sx + 1) * 9 + (sy + 1) * 3 + (sz + 1)
};

struct RawFace {
  int32_t nbr;  // neighbour, or -1 for a wall
  int8_t sx, sy, sz, wall;
  double area;
};

struct Params {
  const double* pts;
  int64_t n;
  double L[3];
  int periodic;
  int nb[3];
  double h[3];
  const int64_t* bucket_start;
  const int32_t* bucket_pts;
  RawFace* raw;      // [n][kMaxOut]
  int32_t* count;    // faces per cell, -1 when the cell failed
  double* volume;
  unsigned long long* failures;
};

__device__ __forceinline__ double dot3(double ax, double ay, double az, double bx, double by, double bz) {
  return ax * bx + ay * by + az * bz;
}

__device__ __forceinline__ bool cand_less(const Cand& a, const Cand& b) {
  if (a.d2 != b.d2) return a.d2 < b.d2;
  if (a.j != b.j) return a.j < b.j;
  return a.code < b.code;
}

__device__ void heap_down(Cand* h, int n, int i) {
  while (true) {
    int l = 2 * i + 1, r = l + 1, m = i;
    if (l < n && cand_less(h[l], h[m])) m = l;
    if (r < n && cand_less(h[r], h[m])) m = r;
    if (m == i) return;
    const Cand t = h[i];
    h[i] = h[m];
    h[m] = t;
    i = m;
  }
}

__device__ void box_poly(Poly& P, double lx, double ly, double lz, double hx, double hy, double hz) {
  const double vx[8] = {lx, hx, hx, lx, lx, hx, hx, lx};
  const double vy[8] = {ly, ly, hy, hy, ly, ly, hy, hy};
  const double vz[8] = {lz, lz, lz, lz, hz, hz, hz, hz};
  for (int k = 0; k < 8; ++k) {
    P.x[k] = vx[k];
    P.y[k] = vy[k];
    P.z[k] = vz[k];
  }
  P.nv = 8;
  const uint8_t faces[6][4] = {{0, 4, 7, 3}, {1, 2, 6, 5}, {0, 1, 5, 4}, {3, 7, 6, 2}, {0, 3, 2, 1}, {4, 5, 6, 7}};
  P.nf = 6;
  for (int f = 0; f < 6; ++f) {
    P.off[f] = (uint16_t)(4 * f);
    for (int k = 0; k < 4; ++k) P.fv[4 * f + k] = faces[f][k];
    P.tag[f] = kWallTagBase - f;
  }
  P.off[6] = 24;
}

// Keep {x : n.x <= b}: the host producer's Poly::clip with fixed buffers.  The clipped
// polyhedron is written to Q (vertices compacted in order of first use over the faces).
__device__ bool clip(const Poly& P, Poly& Q, double nx, double ny, double nz, double b, int64_t new_tag,
                     double* s, double* cx, double* cy, double* cz) {
  int nv = P.nv;
  bool any_out = false;
  for (int i = 0; i < nv; ++i) {
    s[i] = dot3(nx, ny, nz, P.x[i], P.y[i], P.z[i]) - b;
    if (s[i] > 0.0) any_out = true;
  }
  if (!any_out) {
    Q = P;
    return true;
  }
  // working vertex list: P's vertices then the crossings (cx/cy/cz hold P's copy + new)
  for (int i = 0; i < nv; ++i) {
    cx[i] = P.x[i];
    cy[i] = P.y[i];
    cz[i] = P.z[i];
  }
  uint32_t ckey[kMaxSeg * 2];
  int cval[kMaxSeg * 2];
  int ncache = 0;
  bool ok = true;
  auto crossing = [&](int a, int c) -> int {
    const uint32_t key = a < c ? ((uint32_t)a << 16) | (uint32_t)c : ((uint32_t)c << 16) | (uint32_t)a;
    for (int k = 0; k < ncache; ++k)
      if (ckey[k] == key) return cval[k];
    if (nv >= kMaxV || ncache >= kMaxSeg * 2) {
      ok = false;
      return a;
    }
    const double t = s[a] / (s[a] - s[c]);
    cx[nv] = cx[a] + (cx[c] - cx[a]) * t;
    cy[nv] = cy[a] + (cy[c] - cy[a]) * t;
    cz[nv] = cz[a] + (cz[c] - cz[a]) * t;
    s[nv] = 0.0;
    ckey[ncache] = key;
    cval[ncache] = nv;
    ++ncache;
    return nv++;
  };
  int seg_in[kMaxSeg], seg_out[kMaxSeg];
  int nseg = 0;
  // faces of the result, vertex indices into the working list
  uint16_t noff[kMaxF + 1];
  int64_t ntag[kMaxF];
  uint8_t nfv[kMaxFV];
  int nnf = 0, nref = 0;
  for (int fi = 0; fi < P.nf && ok; ++fi) {
    const int beg = P.off[fi], m = P.off[fi + 1] - beg;
    const int start_ref = nref;
    int exitv = -1, entryv = -1;
    for (int k = 0; k < m && ok; ++k) {
      const int a = P.fv[beg + k], c = P.fv[beg + (k + 1) % m];
      const bool ain = s[a] <= 0.0, cin = s[c] <= 0.0;
      if (ain) {
        if (nref >= kMaxFV) { ok = false; break; }
        nfv[nref++] = (uint8_t)a;
      }
      if (ain && !cin) {
        const int xv = (s[a] == 0.0) ? a : crossing(a, c);
        if (xv != a) {
          if (nref >= kMaxFV) { ok = false; break; }
          nfv[nref++] = (uint8_t)xv;
        }
        exitv = xv;
      } else if (!ain && cin) {
        const int yv = (s[c] == 0.0) ? c : crossing(a, c);
        if (yv != c) {
          if (nref >= kMaxFV) { ok = false; break; }
          nfv[nref++] = (uint8_t)yv;
        }
        entryv = yv;
      }
    }
    if (!ok) break;
    if (exitv >= 0 && entryv >= 0 && exitv != entryv) {
      if (nseg >= kMaxSeg) { ok = false; break; }
      seg_in[nseg] = entryv;
      seg_out[nseg] = exitv;
      ++nseg;
    }
    if (nref - start_ref >= 3) {
      if (nnf >= kMaxF) { ok = false; break; }
      noff[nnf] = (uint16_t)start_ref;
      ntag[nnf] = P.tag[fi];
      ++nnf;
    } else {
      nref = start_ref;  // degenerate remainder of a face: dropped
    }
  }
  if (!ok) return false;
  if (nseg >= 3) {
    // cap: follow entry -> exit around the new face
    for (int a2 = 0; a2 < nseg; ++a2)
      for (int b2 = a2 + 1; b2 < nseg; ++b2)
        if (seg_in[a2] == seg_in[b2]) return false;
    if (nnf >= kMaxF || nref + nseg > kMaxFV) return false;
    const int start_ref = nref;
    int cur = seg_in[0];
    const int start = cur;
    int steps = 0;
    for (int guard = 0; guard <= nseg; ++guard) {
      if (nref >= kMaxFV) return false;
      nfv[nref++] = (uint8_t)cur;
      ++steps;
      int nxt = -1;
      for (int k = 0; k < nseg; ++k)
        if (seg_in[k] == cur) { nxt = seg_out[k]; break; }
      if (nxt < 0) return false;
      cur = nxt;
      if (cur == start) break;
    }
    if (cur != start || steps != nseg) return false;
    noff[nnf] = (uint16_t)start_ref;
    ntag[nnf] = new_tag;
    ++nnf;
  }
  noff[nnf] = (uint16_t)nref;
  // compact vertices in order of first use over the faces
  int16_t remap[kMaxV];
  for (int i = 0; i < nv; ++i) remap[i] = -1;
  int q = 0;
  Q.nf = nnf;
  int r = 0;
  for (int f = 0; f < nnf; ++f) {
    Q.off[f] = (uint16_t)r;
    Q.tag[f] = ntag[f];
    for (int k = noff[f]; k < noff[f + 1]; ++k) {
      const int idx = nfv[k];
      if (remap[idx] < 0) {
        remap[idx] = (int16_t)q;
        Q.x[q] = cx[idx];
        Q.y[q] = cy[idx];
        Q.z[q] = cz[idx];
        ++q;
      }
      Q.fv[r++] = (uint8_t)remap[idx];
    }
  }
  Q.off[nnf] = (uint16_t)r;
  Q.nv = q;
  return true;
}

__device__ double max_radius(const Poly& P, double px, double py, double pz) {
  double r = 0.0;
  for (int i = 0; i < P.nv; ++i) {
    const double dx = P.x[i] - px, dy = P.y[i] - py, dz = P.z[i] - pz;
    r = fmax(r, sqrt(dot3(dx, dy, dz, dx, dy, dz)));
  }
  return r;
}

__device__ __forceinline__ void delta(const Params& p, int64_t i, int64_t j, int sx, int sy, int sz, double& dx,
                                      double& dy, double& dz) {
  dx = (p.pts[3 * j] - p.pts[3 * i]) + (double)sx * p.L[0];
  dy = (p.pts[3 * j + 1] - p.pts[3 * i + 1]) + (double)sy * p.L[1];
  dz = (p.pts[3 * j + 2] - p.pts[3 * i + 2]) + (double)sz * p.L[2];
}

// candidates of the Chebyshev bucket shell range (r_lo, r_hi] within distance^2 max_d2
// into c (false on overflow).  Farther ones can never clip: the security test compares
// against 4 R^2 and R only shrinks.
__device__ bool gather(const Params& p, int64_t i, int r_lo, int r_hi, double max_d2, Cand* c, int& nc) {
  nc = 0;
  const double px = p.pts[3 * i], py = p.pts[3 * i + 1], pz = p.pts[3 * i + 2];
  const int b0 = min(max((int)floor(px / p.h[0]), 0), p.nb[0] - 1);
  const int b1 = min(max((int)floor(py / p.h[1]), 0), p.nb[1] - 1);
  const int b2 = min(max((int)floor(pz / p.h[2]), 0), p.nb[2] - 1);
  for (int ox = -r_hi; ox <= r_hi; ++ox)
    for (int oy = -r_hi; oy <= r_hi; ++oy)
      for (int oz = -r_hi; oz <= r_hi; ++oz) {
        const int cheb = max(abs(ox), max(abs(oy), abs(oz)));
        if (cheb <= r_lo) continue;
        int q[3] = {b0 + ox, b1 + oy, b2 + oz};
        int sh[3] = {0, 0, 0};
        bool skip = false;
        for (int a = 0; a < 3; ++a) {
          if (q[a] < 0 || q[a] >= p.nb[a]) {
            if (!p.periodic) { skip = true; break; }
            const int w = ((q[a] % p.nb[a]) + p.nb[a]) % p.nb[a];
            sh[a] = (q[a] - w) / p.nb[a];
            q[a] = w;
          }
        }
        if (skip) continue;
        const int64_t bk = ((int64_t)q[0] * p.nb[1] + q[1]) * p.nb[2] + q[2];
        for (int64_t k = p.bucket_start[bk]; k < p.bucket_start[bk + 1]; ++k) {
          const int32_t j = p.bucket_pts[k];
          if (j == i && sh[0] == 0 && sh[1] == 0 && sh[2] == 0) continue;
          double dx, dy, dz;
          delta(p, i, j, sh[0], sh[1], sh[2], dx, dy, dz);
          const double d2 = dot3(dx, dy, dz, dx, dy, dz);
          if (d2 > max_d2) continue;
          if (nc >= kMaxCand) return false;
          c[nc].d2 = d2;
          c[nc].j = j;
          c[nc].code = (sh[0] + 1) * 9 + (sh[1] + 1) * 3 + (sh[2] + 1);
          ++nc;
        }
      }
  return true;
}

__device__ double polygon_area(const Poly& P, int f) {
  const int beg = P.off[f], m = P.off[f + 1] - beg;
  double ax = 0, ay = 0, az = 0;
  const int o = P.fv[beg];
  for (int k = 1; k + 1 < m; ++k) {
    const int a = P.fv[beg + k], c = P.fv[beg + k + 1];
    const double ux = P.x[a] - P.x[o], uy = P.y[a] - P.y[o], uz = P.z[a] - P.z[o];
    const double vx = P.x[c] - P.x[o], vy = P.y[c] - P.y[o], vz = P.z[c] - P.z[o];
    ax = ax + (uy * vz - uz * vy);
    ay = ay + (uz * vx - ux * vz);
    az = az + (ux * vy - uy * vx);
  }
  return 0.5 * sqrt(dot3(ax, ay, az, ax, ay, az));
}

__device__ double poly_volume(const Poly& P, double px, double py, double pz) {
  double vol = 0.0;
  for (int f = 0; f < P.nf; ++f) {
    const int beg = P.off[f], m = P.off[f + 1] - beg;
    const int o = P.fv[beg];
    const double ox = P.x[o] - px, oy = P.y[o] - py, oz = P.z[o] - pz;
    for (int k = 1; k + 1 < m; ++k) {
      const int a = P.fv[beg + k], c = P.fv[beg + k + 1];
      const double ax = P.x[a] - px, ay = P.y[a] - py, az = P.z[a] - pz;
      const double bx = P.x[c] - px, by = P.y[c] - py, bz = P.z[c] - pz;
      const double cxx = ay * bz - az * by, cyy = az * bx - ax * bz, czz = ax * by - ay * bx;
      vol += fabs(dot3(ox, oy, oz, cxx, cyy, czz)) / 6.0;
    }
  }
  return vol;
}

__device__ __forceinline__ bool face_less(const RawFace& a, const RawFace& b) {
  if (a.nbr != b.nbr) return a.nbr < b.nbr;
  if (a.sx != b.sx) return a.sx < b.sx;
  if (a.sy != b.sy) return a.sy < b.sy;
  if (a.sz != b.sz) return a.sz < b.sz;
  return a.wall < b.wall;
}

struct CellScratch {
  Poly A, B;
  double s[kMaxV], cx[kMaxV], cy[kMaxV], cz[kMaxV];
  Cand cand[kMaxCand];
};

__device__ bool build_cell(const Params& p, int64_t i, CellScratch& w, RawFace* out, int& nout, double& vol) {
  const double px = p.pts[3 * i], py = p.pts[3 * i + 1], pz = p.pts[3 * i + 2];
  const int max_r = p.periodic ? min(p.nb[0], min(p.nb[1], p.nb[2])) : max(p.nb[0], max(p.nb[1], p.nb[2]));
  const double hmin = fmin(p.h[0], fmin(p.h[1], p.h[2]));
  Poly* cur = &w.A;
  Poly* nxt = &w.B;
  if (p.periodic) {
    const double wd = (max_r + 1) * fmax(p.h[0], fmax(p.h[1], p.h[2]));
    box_poly(*cur, px - wd, py - wd, pz - wd, px + wd, py + wd, pz + wd);
  } else {
    box_poly(*cur, 0.0, 0.0, 0.0, p.L[0], p.L[1], p.L[2]);
  }
  int r_done = -1;
  int r = min(1, max_r);
  while (true) {
    int nc = 0;
    double R = max_radius(*cur, px, py, pz);
    if (!gather(p, i, r_done, r, 4.0 * R * R, w.cand, nc)) return false;
    for (int k = nc / 2 - 1; k >= 0; --k) heap_down(w.cand, nc, k);
    while (nc > 0) {
      const Cand c = w.cand[0];
      w.cand[0] = w.cand[nc - 1];
      --nc;
      heap_down(w.cand, nc, 0);
      if (c.d2 > 4.0 * R * R) break;
      const int sx = c.code / 9 - 1, sy = (c.code / 3) % 3 - 1, sz = c.code % 3 - 1;
      double dx, dy, dz;
      delta(p, i, c.j, sx, sy, sz, dx, dy, dz);
      const double mx = px + dx * 0.5, my = py + dy * 0.5, mz = pz + dz * 0.5;
      const int64_t tag = (int64_t)c.j * 27 + c.code;
      if (!clip(*cur, *nxt, dx, dy, dz, dot3(dx, dy, dz, mx, my, mz), tag, w.s, w.cx, w.cy, w.cz)) return false;
      Poly* t = cur;
      cur = nxt;
      nxt = t;
      R = max_radius(*cur, px, py, pz);
    }
    r_done = r;
    R = max_radius(*cur, px, py, pz);
    if (2.0 * R <= r * hmin) break;
    if (r >= max_r) {
      if (p.periodic) return false;
      break;
    }
    r = min(r + 1, max_r);
  }
  if (cur->nf > kMaxOut) return false;
  nout = 0;
  for (int f = 0; f < cur->nf; ++f) {
    RawFace rf;
    rf.area = polygon_area(*cur, f);
    const int64_t tag = cur->tag[f];
    if (tag < 0) {
      if (p.periodic) return false;  // the bounding box survived
      rf.nbr = -1;
      rf.sx = rf.sy = rf.sz = 0;
      rf.wall = (int8_t)(kWallTagBase - tag);
    } else {
      rf.nbr = (int32_t)(tag / 27);
      const int code = (int)(tag % 27);
      rf.sx = (int8_t)(code / 9 - 1);
      rf.sy = (int8_t)((code / 3) % 3 - 1);
      rf.sz = (int8_t)(code % 3 - 1);
      rf.wall = -1;
    }
    // insertion in (neighbour, shift, wall) order
    int k = nout++;
    while (k > 0 && face_less(rf, out[k - 1])) {
      out[k] = out[k - 1];
      --k;
    }
    out[k] = rf;
  }
  vol = poly_volume(*cur, px, py, pz);
  return true;
}

__global__ void __launch_bounds__(kThreads) k_voronoi_cells(Params p, int64_t first, int64_t last) {
  const int64_t i = first + (int64_t)blockIdx.x * kThreads + threadIdx.x;
  if (i >= last) return;
  CellScratch w;
  int nout = 0;
  double vol = 0.0;
  RawFace* out = p.raw + i * kMaxOut;
  if (build_cell(p, i, w, out, nout, vol)) {
    p.count[i] = nout;
    p.volume[i] = vol;
  } else {
    p.count[i] = -1;
    p.volume[i] = 0.0;
    atomicAdd(p.failures, 1ull);
  }
}

// index of the face of cell j towards (i, -shift), or -1
__device__ int find_recip(const Params& p, int32_t j, int64_t i, int sx, int sy, int sz) {
  const int nj = p.count[j];
  const RawFace* fj = p.raw + (int64_t)j * kMaxOut;
  for (int k = 0; k < nj; ++k)
    if (fj[k].nbr == (int32_t)i && fj[k].sx == -sx && fj[k].sy == -sy && fj[k].sz == -sz) return k;
  return -1;
}

// kept faces per cell (a neighbour face needs its reciprocal); dropped ones counted
__global__ void k_voronoi_keep(Params p, int32_t* kept, unsigned long long* dropped) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < p.n; i += (int64_t)gridDim.x * blockDim.x) {
    const int ni = p.count[i];
    int k = 0;
    unsigned long long d = 0;
    for (int f = 0; f < ni; ++f) {
      const RawFace& rf = p.raw[i * kMaxOut + f];
      if (rf.nbr < 0 || (p.count[rf.nbr] >= 0 && find_recip(p, rf.nbr, i, rf.sx, rf.sy, rf.sz) >= 0)) ++k;
      else ++d;
    }
    kept[i] = k;
    if (d) atomicAdd(dropped, d);
  }
}

__global__ void k_voronoi_csr(Params p, const int64_t* row_ptr, int32_t* nbr, uint8_t* kind, double* area,
                              double* normal, double* size) {
  const double kPi = 3.14159265358979323846;
  const double wn[6][3] = {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < p.n; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t o = row_ptr[i];
    const int ni = p.count[i];
    for (int f = 0; f < ni; ++f) {
      const RawFace& rf = p.raw[i * kMaxOut + f];
      if (rf.nbr >= 0) {
        if (p.count[rf.nbr] < 0) continue;
        const int rk = find_recip(p, rf.nbr, i, rf.sx, rf.sy, rf.sz);
        if (rk < 0) continue;
        double a = rf.area;
        if (rf.nbr < i) a = p.raw[(int64_t)rf.nbr * kMaxOut + rk].area;
        double dx, dy, dz;
        delta(p, i, rf.nbr, rf.sx, rf.sy, rf.sz, dx, dy, dz);
        const double inv = 1.0 / sqrt(dot3(dx, dy, dz, dx, dy, dz));
        nbr[o] = rf.nbr;
        kind[o] = (rf.sx | rf.sy | rf.sz) ? 1 : 0;
        normal[3 * o] = dx * inv;
        normal[3 * o + 1] = dy * inv;
        normal[3 * o + 2] = dz * inv;
        area[o] = a;
      } else {
        nbr[o] = -1;
        kind[o] = 2;
        normal[3 * o] = wn[rf.wall][0];
        normal[3 * o + 1] = wn[rf.wall][1];
        normal[3 * o + 2] = wn[rf.wall][2];
        area[o] = rf.area;
      }
      ++o;
    }
    size[i] = cbrt(3.0 * p.volume[i] / (4.0 * kPi));
  }
}

}  // namespace vgpu

struct sw_gpu_grid {
  int64_t n = 0;
  std::vector<int64_t> row_ptr;
  std::vector<int32_t> nbr;
  std::vector<uint8_t> kind;
  std::vector<double> area, normal, volume, size;
  int64_t failed_cells = 0, dropped_faces = 0;
  int status = 0;  // 0 ok, else a cudaError_t
};

namespace {

template <typename T>
cudaError_t dalloc(T** p, size_t count) {
  return cudaMalloc(reinterpret_cast<void**>(p), std::max<size_t>(count, 1) * sizeof(T));
}

struct DeviceBuffers {
  std::vector<void*> ptrs;
  ~DeviceBuffers() {
    for (void* q : ptrs) cudaFree(q);
  }
  template <typename T>
  cudaError_t get(T** p, size_t count) {
    cudaError_t e = dalloc(p, count);
    if (e == cudaSuccess) ptrs.push_back(*p);
    return e;
  }
};

}  // namespace

extern "C" {

sw_gpu_grid* sw_gpu_grid_voronoi(const double* points, int64_t n, const double box_size[3], int32_t periodic,
                                  int32_t device) {
  if (n <= 0 || !points || n >= (int64_t)INT32_MAX) return nullptr;
  sw_gpu_grid* g = new sw_gpu_grid();
  g->n = n;
  {
    const cudaError_t de = cudaSetDevice(device);
    if (de != cudaSuccess) {
      g->status = (int)de;
      return g;
    }
  }
  vgpu::Params p{};
  p.n = n;
  for (int a = 0; a < 3; ++a) p.L[a] = box_size[a];
  p.periodic = periodic != 0;
  // buckets on the host, as the host producer forms them (edge 1.5 x mean spacing)
  const double mean_spacing = std::cbrt(p.L[0] * p.L[1] * p.L[2] / (double)n);
  for (int a = 0; a < 3; ++a) {
    p.nb[a] = std::max(1, (int)std::floor(p.L[a] / (1.5 * mean_spacing)));
    p.h[a] = p.L[a] / p.nb[a];
  }
  const int64_t nbt = (int64_t)p.nb[0] * p.nb[1] * p.nb[2];
  std::vector<int64_t> start(nbt + 1, 0);
  std::vector<int64_t> bid(n);
  for (int64_t i = 0; i < n; ++i) {
    int b[3];
    for (int a = 0; a < 3; ++a) {
      b[a] = (int)std::floor(points[3 * i + a] / p.h[a]);
      b[a] = std::min(std::max(b[a], 0), p.nb[a] - 1);
    }
    bid[i] = ((int64_t)b[0] * p.nb[1] + b[1]) * p.nb[2] + b[2];
    start[bid[i] + 1]++;
  }
  for (int64_t k = 0; k < nbt; ++k) start[k + 1] += start[k];
  std::vector<int32_t> bpts(n);
  {
    std::vector<int64_t> fill(start.begin(), start.end() - 1);
    for (int64_t i = 0; i < n; ++i) bpts[fill[bid[i]]++] = (int32_t)i;
  }
  DeviceBuffers buf;
  double* d_pts = nullptr;
  int64_t *d_start = nullptr, *d_row = nullptr;
  int32_t *d_bpts = nullptr, *d_count = nullptr, *d_kept = nullptr, *d_nbr = nullptr;
  vgpu::RawFace* d_raw = nullptr;
  double *d_vol = nullptr, *d_area = nullptr, *d_normal = nullptr, *d_size = nullptr;
  uint8_t* d_kind = nullptr;
  unsigned long long* d_ctr = nullptr;
  cudaError_t e = cudaSuccess;
  auto step = [&](cudaError_t r) {
    if (e == cudaSuccess) e = r;
  };
  step(buf.get(&d_pts, 3 * n));
  step(buf.get(&d_start, nbt + 1));
  step(buf.get(&d_bpts, n));
  step(buf.get(&d_raw, (size_t)n * vgpu::kMaxOut));
  step(buf.get(&d_count, n));
  step(buf.get(&d_kept, n));
  step(buf.get(&d_vol, n));
  step(buf.get(&d_ctr, 2));
  if (e == cudaSuccess) {
    step(cudaMemcpy(d_pts, points, 3 * n * sizeof(double), cudaMemcpyHostToDevice));
    step(cudaMemcpy(d_start, start.data(), (nbt + 1) * sizeof(int64_t), cudaMemcpyHostToDevice));
    step(cudaMemcpy(d_bpts, bpts.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice));
    step(cudaMemset(d_ctr, 0, 2 * sizeof(unsigned long long)));
  }
  p.pts = d_pts;
  p.bucket_start = d_start;
  p.bucket_pts = d_bpts;
  p.raw = d_raw;
  p.count = d_count;
  p.volume = d_vol;
  p.failures = d_ctr;
  // cells in launches of at most 1 Mi threads, each a short kernel
  const int64_t chunk = 1 << 20;
  for (int64_t first = 0; first < n && e == cudaSuccess; first += chunk) {
    const int64_t last = std::min(n, first + chunk);
    const unsigned blocks = (unsigned)((last - first + vgpu::kThreads - 1) / vgpu::kThreads);
    vgpu::k_voronoi_cells<<<blocks, vgpu::kThreads>>>(p, first, last);
    step(cudaGetLastError());
  }
  const unsigned grid = (unsigned)std::min<int64_t>((n + 255) / 256, 152 * 32);
  if (e == cudaSuccess) {
    vgpu::k_voronoi_keep<<<grid, 256>>>(p, d_kept, d_ctr + 1);
    step(cudaGetLastError());
  }
  std::vector<int32_t> kept(n);
  unsigned long long ctr[2] = {0, 0};
  if (e == cudaSuccess) step(cudaMemcpy(kept.data(), d_kept, n * sizeof(int32_t), cudaMemcpyDeviceToHost));
  if (e == cudaSuccess) step(cudaMemcpy(ctr, d_ctr, sizeof(ctr), cudaMemcpyDeviceToHost));
  g->failed_cells = (int64_t)ctr[0];
  g->dropped_faces = (int64_t)ctr[1];
  g->row_ptr.assign(n + 1, 0);
  for (int64_t i = 0; i < n; ++i) g->row_ptr[i + 1] = g->row_ptr[i] + kept[i];
  const int64_t E = g->row_ptr[n];
  if (e == cudaSuccess) {
    step(buf.get(&d_row, n + 1));
    step(buf.get(&d_nbr, E));
    step(buf.get(&d_kind, E));
    step(buf.get(&d_area, E));
    step(buf.get(&d_normal, 3 * E));
    step(buf.get(&d_size, n));
  }
  if (e == cudaSuccess) {
    step(cudaMemcpy(d_row, g->row_ptr.data(), (n + 1) * sizeof(int64_t), cudaMemcpyHostToDevice));
    vgpu::k_voronoi_csr<<<grid, 256>>>(p, d_row, d_nbr, d_kind, d_area, d_normal, d_size);
    step(cudaGetLastError());
    step(cudaDeviceSynchronize());
  }
  if (e == cudaSuccess) {
    g->nbr.resize(E);
    g->kind.resize(E);
    g->area.resize(E);
    g->normal.resize(3 * E);
    g->volume.resize(n);
    g->size.resize(n);
    step(cudaMemcpy(g->nbr.data(), d_nbr, E * sizeof(int32_t), cudaMemcpyDeviceToHost));
    step(cudaMemcpy(g->kind.data(), d_kind, E, cudaMemcpyDeviceToHost));
    step(cudaMemcpy(g->area.data(), d_area, E * sizeof(double), cudaMemcpyDeviceToHost));
    step(cudaMemcpy(g->normal.data(), d_normal, 3 * E * sizeof(double), cudaMemcpyDeviceToHost));
    step(cudaMemcpy(g->volume.data(), d_vol, n * sizeof(double), cudaMemcpyDeviceToHost));
    step(cudaMemcpy(g->size.data(), d_size, n * sizeof(double), cudaMemcpyDeviceToHost));
  }
  g->status = (int)e;
  return g;
}

int32_t sw_gpu_grid_status(const sw_gpu_grid* g) { return g ? g->status : -1; }
int64_t sw_gpu_grid_num_faces(const sw_gpu_grid* g) { return g ? (int64_t)g->nbr.size() : 0; }
int64_t sw_gpu_grid_failed_cells(const sw_gpu_grid* g) { return g ? g->failed_cells : -1; }
int64_t sw_gpu_grid_dropped_faces(const sw_gpu_grid* g) { return g ? g->dropped_faces : -1; }

void sw_gpu_grid_copy(const sw_gpu_grid* g, int64_t* row_ptr, int32_t* nbr, uint8_t* kind, double* area,
                      double* normal, double* volume, double* size) {
  if (!g || g->status != 0) return;
  const size_t E = g->nbr.size();
  if (row_ptr) std::memcpy(row_ptr, g->row_ptr.data(), (g->n + 1) * sizeof(int64_t));
  if (nbr) std::memcpy(nbr, g->nbr.data(), E * sizeof(int32_t));
  if (kind) std::memcpy(kind, g->kind.data(), E);
  if (area) std::memcpy(area, g->area.data(), E * sizeof(double));
  if (normal) std::memcpy(normal, g->normal.data(), 3 * E * sizeof(double));
  if (volume) std::memcpy(volume, g->volume.data(), g->n * sizeof(double));
  if (size) std::memcpy(size, g->size.data(), g->n * sizeof(double));
}

void sw_gpu_grid_free(sw_gpu_grid* g) { delete g; }

}  // extern "C"
