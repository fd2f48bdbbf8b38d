// Host-side grid producers for the sweep: periodic / bounded 3D Voronoi
// tessellations built by half-space clipping, and the reference's cartesian grid.
//
// Grid construction stays on the host and is uploaded once as face-neighbour CSR
// (the sweep library takes any CSR with exactly antisymmetric normals).  The
// reference builds its Voronoi grids from an incremental Delaunay triangulation
// (src/voronoi/); this producer computes the same cells directly, one at a time,
// by clipping a bounding polyhedron with the bisector planes of nearby generators
// in order of distance until the security radius (2 x the farthest vertex) is
// passed.  Face conventions follow the reference:
//   * normal = (p_neighbour - p_cell).normalize()  (src/voronoi/cell.rs:63-71,
//     glam's normalize = v * (1/|v|)); the periodic image offset is added to the
//     generator difference, so the two sides of a face get bitwise negated normals;
//   * size = cbrt(3 V / (4 pi))  (src/voronoi/cell.rs:186-188);
//   * each face's area is taken from the lower-index cell for both sides.
// The cartesian grid restates src/sweep/grid/cartesian.rs:220-395 for one rank.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <unordered_map>
#include <vector>

#include "grid_host.h"

namespace {

struct V3 {
  double x, y, z;
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double norm(V3 a) { return std::sqrt(dot(a, a)); }

const int64_t kWallTagBase = -1;  // walls: -1..-6 (x-, x+, y-, y+, z-, z+)

// A convex polyhedron as vertex list + faces (vertex cycles, counter-clockwise seen
// from outside) with a tag per face.
struct Poly {
  std::vector<V3> v;
  std::vector<std::vector<int>> f;
  std::vector<int64_t> tag;

  void box(V3 lo, V3 hi) {
    v = {{lo.x, lo.y, lo.z}, {hi.x, lo.y, lo.z}, {hi.x, hi.y, lo.z}, {lo.x, hi.y, lo.z},
         {lo.x, lo.y, hi.z}, {hi.x, lo.y, hi.z}, {hi.x, hi.y, hi.z}, {lo.x, hi.y, hi.z}};
    f = {{0, 4, 7, 3}, {1, 2, 6, 5}, {0, 1, 5, 4}, {3, 7, 6, 2}, {0, 3, 2, 1}, {4, 5, 6, 7}};
    tag = {kWallTagBase - 0, kWallTagBase - 1, kWallTagBase - 2,
           kWallTagBase - 3, kWallTagBase - 4, kWallTagBase - 5};
  }

  // Keep {x : n.x <= b}; the new face gets `new_tag`.  Returns false on a topological
  // inconsistency (the caller reports the cell as failed).
  bool clip(V3 n, double b, int64_t new_tag, std::vector<double>& s,
            std::unordered_map<uint64_t, int>& cache) {
    size_t nv = v.size();
    s.resize(nv);
    bool any_out = false;
    for (size_t i = 0; i < nv; ++i) {
      s[i] = dot(n, v[i]) - b;
      if (s[i] > 0.0) any_out = true;
    }
    if (!any_out) return true;
    cache.clear();
    auto crossing = [&](int a, int c) -> int {
      uint64_t key = a < c ? ((uint64_t)a << 32) | (uint32_t)c : ((uint64_t)c << 32) | (uint32_t)a;
      auto it = cache.find(key);
      if (it != cache.end()) return it->second;
      double t = s[a] / (s[a] - s[c]);
      V3 p = v[a] + (v[c] - v[a]) * t;
      int idx = (int)v.size();
      v.push_back(p);
      s.push_back(0.0);
      cache.emplace(key, idx);
      return idx;
    };
    std::vector<std::vector<int>> nf;
    std::vector<int64_t> ntag;
    std::vector<std::pair<int, int>> segs;  // cap edges entry -> exit
    for (size_t fi = 0; fi < f.size(); ++fi) {
      const std::vector<int>& face = f[fi];
      std::vector<int> out;
      int exitv = -1, entryv = -1;
      size_t m = face.size();
      for (size_t k = 0; k < m; ++k) {
        int a = face[k], c = face[(k + 1) % m];
        bool ain = s[a] <= 0.0, cin = s[c] <= 0.0;
        if (ain) out.push_back(a);
        if (ain && !cin) {
          int x = (s[a] == 0.0) ? a : crossing(a, c);
          if (x != a) out.push_back(x);
          exitv = x;
        } else if (!ain && cin) {
          int y = (s[c] == 0.0) ? c : crossing(a, c);
          if (y != c) out.push_back(y);
          entryv = y;
        }
      }
      if (exitv >= 0 && entryv >= 0 && exitv != entryv) segs.push_back({entryv, exitv});
      if (out.size() >= 3) {
        nf.push_back(std::move(out));
        ntag.push_back(tag[fi]);
      }
    }
    if (segs.size() >= 3) {
      std::unordered_map<int, int> next;
      for (auto& sg : segs) {
        if (next.count(sg.first)) return false;
        next[sg.first] = sg.second;
      }
      std::vector<int> cap;
      int start = segs[0].first, cur = start;
      for (size_t guard = 0; guard <= segs.size(); ++guard) {
        cap.push_back(cur);
        auto it = next.find(cur);
        if (it == next.end()) return false;
        cur = it->second;
        if (cur == start) break;
      }
      if (cur != start || cap.size() != segs.size()) return false;
      nf.push_back(std::move(cap));
      ntag.push_back(new_tag);
    }
    f.swap(nf);
    tag.swap(ntag);
    // compact vertices
    std::vector<int> remap(v.size(), -1);
    std::vector<V3> nvtx;
    for (auto& face : f)
      for (int& idx : face) {
        if (remap[idx] < 0) {
          remap[idx] = (int)nvtx.size();
          nvtx.push_back(v[idx]);
        }
        idx = remap[idx];
      }
    v.swap(nvtx);
    return true;
  }

  double max_radius(V3 p) const {
    double r = 0.0;
    for (const V3& q : v) r = std::max(r, norm(q - p));
    return r;
  }
};

double polygon_area(const Poly& P, const std::vector<int>& face) {
  V3 acc{0, 0, 0};
  V3 o = P.v[face[0]];
  for (size_t k = 1; k + 1 < face.size(); ++k)
    acc = acc + cross(P.v[face[k]] - o, P.v[face[k + 1]] - o);
  return 0.5 * norm(acc);
}

double poly_volume(const Poly& P, V3 p) {
  double vol = 0.0;
  for (const auto& face : P.f) {
    V3 o = P.v[face[0]] - p;
    for (size_t k = 1; k + 1 < face.size(); ++k) {
      V3 a = P.v[face[k]] - p, b = P.v[face[k + 1]] - p;
      vol += std::fabs(dot(o, cross(a, b))) / 6.0;
    }
  }
  return vol;
}

struct RawFace {
  int32_t nbr;      // neighbour index, or -1 for a wall
  int8_t sx, sy, sz;  // periodic image shift of the neighbour, in box lengths
  int8_t wall;      // wall index 0..5 for boundary faces
  double area;
};

struct Builder {
  const double* pts;
  int64_t n;
  V3 L;
  bool periodic;
  int nb[3];
  double h[3];
  std::vector<int64_t> bucket_start;
  std::vector<int32_t> bucket_pts;
  std::vector<std::vector<RawFace>> faces;
  std::vector<double> volume;
  std::atomic<int64_t> failures{0};

  V3 P(int64_t i) const { return {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]}; }

  void bucketize() {
    double mean_spacing = std::cbrt(L.x * L.y * L.z / (double)n);
    double Ls[3] = {L.x, L.y, L.z};
    for (int a = 0; a < 3; ++a) {
      nb[a] = std::max(1, (int)std::floor(Ls[a] / (1.5 * mean_spacing)));
      h[a] = Ls[a] / nb[a];
    }
    int64_t nbt = (int64_t)nb[0] * nb[1] * nb[2];
    std::vector<int64_t> cnt(nbt + 1, 0);
    std::vector<int64_t> bid(n);
    for (int64_t i = 0; i < n; ++i) {
      int b[3];
      double c[3] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
      for (int a = 0; a < 3; ++a) {
        b[a] = (int)std::floor(c[a] / h[a]);
        b[a] = std::min(std::max(b[a], 0), nb[a] - 1);
      }
      bid[i] = ((int64_t)b[0] * nb[1] + b[1]) * nb[2] + b[2];
      cnt[bid[i] + 1]++;
    }
    for (int64_t k = 0; k < nbt; ++k) cnt[k + 1] += cnt[k];
    bucket_start = cnt;
    bucket_pts.assign(n, 0);
    std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1);
    for (int64_t i = 0; i < n; ++i) bucket_pts[fill[bid[i]]++] = (int32_t)i;
  }

  struct Cand {
    double d2;
    int32_t j;
    int8_t sx, sy, sz;
  };

  // Collect candidates in the Chebyshev bucket shell range (r_lo, r_hi].
  void gather(int64_t i, int r_lo, int r_hi, std::vector<Cand>& out) const {
    V3 p = P(i);
    int b[3] = {std::min(std::max((int)std::floor(p.x / h[0]), 0), nb[0] - 1),
                std::min(std::max((int)std::floor(p.y / h[1]), 0), nb[1] - 1),
                std::min(std::max((int)std::floor(p.z / h[2]), 0), nb[2] - 1)};
    for (int ox = -r_hi; ox <= r_hi; ++ox)
      for (int oy = -r_hi; oy <= r_hi; ++oy)
        for (int oz = -r_hi; oz <= r_hi; ++oz) {
          int cheb = std::max(std::abs(ox), std::max(std::abs(oy), std::abs(oz)));
          if (cheb <= r_lo) continue;
          int q[3] = {b[0] + ox, b[1] + oy, b[2] + oz};
          int sh[3] = {0, 0, 0};
          bool skip = false;
          for (int a = 0; a < 3; ++a) {
            if (q[a] < 0 || q[a] >= nb[a]) {
              if (!periodic) { skip = true; break; }
              int w = ((q[a] % nb[a]) + nb[a]) % nb[a];
              sh[a] = (q[a] - w) / nb[a];
              q[a] = w;
            }
          }
          if (skip) continue;
          int64_t bk = ((int64_t)q[0] * nb[1] + q[1]) * nb[2] + q[2];
          for (int64_t k = bucket_start[bk]; k < bucket_start[bk + 1]; ++k) {
            int32_t j = bucket_pts[k];
            if (j == i && sh[0] == 0 && sh[1] == 0 && sh[2] == 0) continue;
            V3 dlt = delta(i, j, sh[0], sh[1], sh[2]);
            out.push_back({dot(dlt, dlt), j, (int8_t)sh[0], (int8_t)sh[1], (int8_t)sh[2]});
          }
        }
  }

  // Generator difference p_j(+image) - p_i, evaluated as (p_j - p_i) + shift * L so that
  // the reverse face yields exactly the negated vector.
  V3 delta(int64_t i, int64_t j, int sx, int sy, int sz) const {
    V3 pi = P(i), pj = P(j);
    return {(pj.x - pi.x) + (double)sx * L.x, (pj.y - pi.y) + (double)sy * L.y,
            (pj.z - pi.z) + (double)sz * L.z};
  }

  bool build_cell(int64_t i, Poly& poly, std::vector<double>& s,
                  std::unordered_map<uint64_t, int>& cache, std::vector<Cand>& cands) {
    V3 p = P(i);
    // Periodic images are limited to one box length in each direction (shift -1..1),
    // which bucket offsets up to nb guarantee.
    int max_r = periodic ? std::min(nb[0], std::min(nb[1], nb[2]))
                         : std::max(nb[0], std::max(nb[1], nb[2]));
    double hmin = std::min(h[0], std::min(h[1], h[2]));
    if (periodic) {
      double w = (max_r + 1) * std::max(h[0], std::max(h[1], h[2]));
      poly.box(p - V3{w, w, w}, p + V3{w, w, w});
    } else {
      poly.box({0, 0, 0}, L);
    }
    int r_done = -1;
    int r = std::min(2, max_r);
    while (true) {
      cands.clear();
      gather(i, r_done, r, cands);
      std::sort(cands.begin(), cands.end(), [](const Cand& a, const Cand& b) {
        if (a.d2 != b.d2) return a.d2 < b.d2;
        return a.j < b.j;
      });
      double R = poly.max_radius(p);
      for (const Cand& c : cands) {
        if (c.d2 > 4.0 * R * R) break;
        V3 d = delta(i, c.j, c.sx, c.sy, c.sz);
        // bisector: keep x with d.(x - p) <= |d|^2 / 2
        V3 mid = p + d * 0.5;
        int64_t tag = (int64_t)c.j * 27 + ((c.sx + 1) * 9 + (c.sy + 1) * 3 + (c.sz + 1));
        if (!poly.clip(d, dot(d, mid), tag, s, cache)) return false;
        R = poly.max_radius(p);
      }
      r_done = r;
      R = poly.max_radius(p);
      if (2.0 * R <= r * hmin) break;
      if (r >= max_r) {
        if (periodic) return false;
        break;
      }
      r = std::min(r + 1, max_r);
    }
    // assemble faces
    std::vector<RawFace>& out = faces[i];
    out.clear();
    for (size_t fi = 0; fi < poly.f.size(); ++fi) {
      int64_t tag = poly.tag[fi];
      RawFace rf{};
      rf.area = polygon_area(poly, poly.f[fi]);
      if (tag < 0) {
        if (periodic) return false;  // bounding box survived: search radius too small
        rf.nbr = -1;
        rf.wall = (int8_t)(kWallTagBase - tag);
      } else {
        rf.nbr = (int32_t)(tag / 27);
        int code = (int)(tag % 27);
        rf.sx = (int8_t)(code / 9 - 1);
        rf.sy = (int8_t)((code / 3) % 3 - 1);
        rf.sz = (int8_t)(code % 3 - 1);
        rf.wall = -1;
      }
      out.push_back(rf);
    }
    std::sort(out.begin(), out.end(), [](const RawFace& a, const RawFace& b) {
      if (a.nbr != b.nbr) return a.nbr < b.nbr;
      if (a.sx != b.sx) return a.sx < b.sx;
      if (a.sy != b.sy) return a.sy < b.sy;
      if (a.sz != b.sz) return a.sz < b.sz;
      return a.wall < b.wall;
    });
    volume[i] = poly_volume(poly, p);
    return true;
  }

  void run(int nthreads) {
    faces.assign(n, {});
    volume.assign(n, 0.0);
    std::atomic<int64_t> next{0};
    auto worker = [&]() {
      Poly poly;
      std::vector<double> s;
      std::unordered_map<uint64_t, int> cache;
      std::vector<Cand> cands;
      while (true) {
        int64_t start = next.fetch_add(256);
        if (start >= n) break;
        int64_t end = std::min(n, start + 256);
        for (int64_t i = start; i < end; ++i)
          if (!build_cell(i, poly, s, cache, cands)) failures++;
      }
    };
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; ++t) th.emplace_back(worker);
    for (auto& t : th) t.join();
  }
};

}  // namespace

struct sw_host_grid {
  int64_t n = 0;
  std::vector<int64_t> row_ptr;
  std::vector<int32_t> nbr;
  std::vector<uint8_t> kind;
  std::vector<double> area, normal, volume, size, position;
  int64_t dropped_faces = 0;
  int64_t failed_cells = 0;
};

extern "C" {

sw_host_grid* sw_grid_voronoi(const double* points, int64_t n, const double box_size[3],
                              int32_t periodic, int32_t nthreads) {
  if (n <= 0 || !points) return nullptr;
  Builder B;
  B.pts = points;
  B.n = n;
  B.L = {box_size[0], box_size[1], box_size[2]};
  B.periodic = periodic != 0;
  B.bucketize();
  if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
  B.run(nthreads);

  sw_host_grid* g = new sw_host_grid();
  g->n = n;
  g->failed_cells = B.failures.load();
  g->row_ptr.assign(n + 1, 0);
  // Keep only faces whose reciprocal exists; take the area from the lower-index cell.
  auto find_recip = [&](int64_t j, int64_t i, int sx, int sy, int sz) -> const RawFace* {
    const auto& fj = B.faces[j];
    RawFace key{};
    key.nbr = (int32_t)i;
    key.sx = (int8_t)-sx;
    key.sy = (int8_t)-sy;
    key.sz = (int8_t)-sz;
    key.wall = -1;
    auto it = std::lower_bound(fj.begin(), fj.end(), key, [](const RawFace& a, const RawFace& b) {
      if (a.nbr != b.nbr) return a.nbr < b.nbr;
      if (a.sx != b.sx) return a.sx < b.sx;
      if (a.sy != b.sy) return a.sy < b.sy;
      if (a.sz != b.sz) return a.sz < b.sz;
      return a.wall < b.wall;
    });
    if (it != fj.end() && it->nbr == key.nbr && it->sx == key.sx && it->sy == key.sy &&
        it->sz == key.sz)
      return &*it;
    return nullptr;
  };
  for (int64_t i = 0; i < n; ++i) {
    for (const RawFace& rf : B.faces[i]) {
      double area = rf.area;
      if (rf.nbr >= 0) {
        const RawFace* rp = find_recip(rf.nbr, i, rf.sx, rf.sy, rf.sz);
        if (!rp) {
          g->dropped_faces++;
          continue;
        }
        if (rf.nbr < i) area = rp->area;
        V3 d = B.delta(i, rf.nbr, rf.sx, rf.sy, rf.sz);
        double inv = 1.0 / std::sqrt(dot(d, d));
        g->nbr.push_back(rf.nbr);
        g->kind.push_back((rf.sx | rf.sy | rf.sz) ? SW_HOST_LOCAL_PERIODIC : SW_HOST_LOCAL);
        g->normal.push_back(d.x * inv);
        g->normal.push_back(d.y * inv);
        g->normal.push_back(d.z * inv);
      } else {
        static const double wn[6][3] = {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0},
                                        {0, 1, 0},  {0, 0, -1}, {0, 0, 1}};
        g->nbr.push_back(-1);
        g->kind.push_back(SW_HOST_BOUNDARY);
        g->normal.push_back(wn[rf.wall][0]);
        g->normal.push_back(wn[rf.wall][1]);
        g->normal.push_back(wn[rf.wall][2]);
      }
      g->area.push_back(area);
    }
    g->row_ptr[i + 1] = (int64_t)g->nbr.size();
  }
  g->volume = B.volume;
  g->size.resize(n);
  const double kPi = 3.14159265358979323846;
  for (int64_t i = 0; i < n; ++i) g->size[i] = std::cbrt(3.0 * g->volume[i] / (4.0 * kPi));
  g->position.assign(points, points + 3 * n);
  return g;
}

sw_host_grid* sw_grid_cartesian(int32_t nx, int32_t ny, int32_t nz, double cell_size,
                                int32_t periodic) {
  if (nx <= 0 || ny <= 0 || nz <= 0) return nullptr;
  sw_host_grid* g = new sw_host_grid();
  int64_t n = (int64_t)nx * ny * nz;
  g->n = n;
  g->row_ptr.assign(n + 1, 0);
  // SimulationBox side lengths are num_cells * cell_size; positions are L * i / n
  // (cartesian.rs:160-177); face area cell_size^2, volume cell_size^3 (56-75).
  double Lx = cell_size * nx, Ly = cell_size * ny, Lz = cell_size * nz;
  auto pos = [&](int x, int y, int z) -> V3 {
    return {Lx * (double)x / (double)nx, Ly * (double)y / (double)ny, Lz * (double)z / (double)nz};
  };
  auto index = [&](int x, int y, int z) -> int64_t { return ((int64_t)x * ny + y) * nz + z; };
  double area = cell_size * cell_size;
  double vol = cell_size * cell_size * cell_size;
  for (int x = 0; x < nx; ++x)
    for (int y = 0; y < ny; ++y)
      for (int z = 0; z < nz; ++z) {
        int64_t i = index(x, y, z);
        V3 p = pos(x, y, z);
        const int nbrs[6][3] = {{x - 1, y, z}, {x + 1, y, z}, {x, y - 1, z},
                                {x, y + 1, z}, {x, y, z - 1}, {x, y, z + 1}};
        for (const auto& q : nbrs) {
          V3 qp = pos(q[0], q[1], q[2]);
          V3 d = qp - p;
          double inv = 1.0 / std::sqrt(dot(d, d));
          bool contained = q[0] >= 0 && q[1] >= 0 && q[2] >= 0 && q[0] < nx && q[1] < ny && q[2] < nz;
          int wx = ((q[0] % nx) + nx) % nx, wy = ((q[1] % ny) + ny) % ny, wz = ((q[2] % nz) + nz) % nz;
          uint8_t kind = contained ? SW_HOST_LOCAL : (periodic ? SW_HOST_LOCAL_PERIODIC : SW_HOST_BOUNDARY);
          g->nbr.push_back(kind == SW_HOST_BOUNDARY ? -1 : (int32_t)index(wx, wy, wz));
          g->kind.push_back(kind);
          g->area.push_back(area);
          g->normal.push_back(d.x * inv);
          g->normal.push_back(d.y * inv);
          g->normal.push_back(d.z * inv);
        }
        g->row_ptr[i + 1] = (int64_t)g->nbr.size();
        g->position.push_back(p.x);
        g->position.push_back(p.y);
        g->position.push_back(p.z);
      }
  g->volume.assign(n, vol);
  g->size.assign(n, cell_size);
  return g;
}

int64_t sw_grid_num_cells(const sw_host_grid* g) { return g ? g->n : 0; }
int64_t sw_grid_num_faces(const sw_host_grid* g) { return g ? (int64_t)g->nbr.size() : 0; }
int64_t sw_grid_failed_cells(const sw_host_grid* g) { return g ? g->failed_cells : -1; }
int64_t sw_grid_dropped_faces(const sw_host_grid* g) { return g ? g->dropped_faces : -1; }

void sw_grid_copy(const sw_host_grid* g, int64_t* row_ptr, int32_t* nbr, uint8_t* kind,
                  double* area, double* normal, double* volume, double* size, double* position) {
  if (!g) return;
  size_t E = g->nbr.size();
  if (row_ptr) std::memcpy(row_ptr, g->row_ptr.data(), (g->n + 1) * sizeof(int64_t));
  if (nbr) std::memcpy(nbr, g->nbr.data(), E * sizeof(int32_t));
  if (kind) std::memcpy(kind, g->kind.data(), E);
  if (area) std::memcpy(area, g->area.data(), E * sizeof(double));
  if (normal) std::memcpy(normal, g->normal.data(), 3 * E * sizeof(double));
  if (volume) std::memcpy(volume, g->volume.data(), g->n * sizeof(double));
  if (size) std::memcpy(size, g->size.data(), g->n * sizeof(double));
  if (position) std::memcpy(position, g->position.data(), 3 * g->n * sizeof(double));
}

void sw_grid_free(sw_host_grid* g) { delete g; }

}  // extern "C"
