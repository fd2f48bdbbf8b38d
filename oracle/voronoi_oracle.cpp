// Periodic 3-D Voronoi tessellation for the CPU oracle's own workloads.
//
// TEST INFRASTRUCTURE ONLY (see oracle.h): it builds the grids of the CPU reference
// arm of the benchmark, so that arm runs the oracle alone, and it is an independent
// check of the library's grid producers.  The reference builds its grids from an
// incremental Delaunay triangulation (src/voronoi/); this file computes each cell
// directly as the intersection of the bisector half-spaces of its generator,
// clipping a cube face polygon by face polygon (Sutherland-Hodgman) and closing every
// cut with a cap polygon whose vertices are ordered by angle.  Candidates come from a
// bucket grid, shell by shell, until no unvisited generator can be closer than twice
// the cell's farthest vertex.  Face conventions follow the reference:
//   * normal = (p_neighbour - p_cell).normalize() (src/voronoi/cell.rs:63-71), with the
//     periodic image offset added to the generator difference so the two sides of a
//     face get bitwise negated normals;
//   * size = cbrt(3 V / (4 pi)) (src/voronoi/cell.rs:186-188);
//   * a face is kept when both cells have it, with the lower-index cell's area.
#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <thread>
#include <vector>

#include "oracle.h"

namespace {

struct P3 {
  double x, y, z;
};
inline P3 add(P3 a, P3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline P3 sub(P3 a, P3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline P3 scale(P3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dotp(P3 a, P3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline P3 crossp(P3 a, P3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }

// One face of the cell being clipped: its polygon (cyclic order) and the generator it
// is shared with (neighbour index and periodic image shift); neighbour -1 for the
// faces of the starting cube.
struct Facet {
  std::vector<P3> poly;
  int64_t nbr;
  int sx, sy, sz;
};

struct Cell {
  std::vector<Facet> facets;
  std::vector<Facet> next;
  std::vector<P3> cap;

  void cube(double w) {
    facets.clear();
    const P3 c[8] = {{-w, -w, -w}, {w, -w, -w}, {w, w, -w}, {-w, w, -w},
                     {-w, -w, w},  {w, -w, w},  {w, w, w},  {-w, w, w}};
    const int q[6][4] = {{0, 3, 2, 1}, {4, 5, 6, 7}, {0, 1, 5, 4}, {2, 3, 7, 6}, {0, 4, 7, 3}, {1, 2, 6, 5}};
    for (const auto& f : q) facets.push_back(Facet{{c[f[0]], c[f[1]], c[f[2]], c[f[3]]}, -1, 0, 0, 0});
  }

  double radius2() const {
    double r = 0.0;
    for (const Facet& f : facets)
      for (const P3& v : f.poly) r = std::max(r, dotp(v, v));
    return r;
  }

  // Keep {q : n.q <= b}.  The cap is the polygon where the plane cuts the cell.
  void clip(P3 n, double b, int64_t nbr, int sx, int sy, int sz, double eps) {
    bool outside = false;
    for (const Facet& f : facets)
      for (const P3& v : f.poly)
        if (dotp(n, v) - b > 0.0) outside = true;
    if (!outside) return;
    next.clear();
    cap.clear();
    for (const Facet& f : facets) {
      Facet g{{}, f.nbr, f.sx, f.sy, f.sz};
      const size_t m = f.poly.size();
      for (size_t k = 0; k < m; ++k) {
        const P3 a = f.poly[k], c = f.poly[(k + 1) % m];
        const double sa = dotp(n, a) - b, sc = dotp(n, c) - b;
        if (sa <= 0.0) {
          g.poly.push_back(a);
          if (sa == 0.0) cap.push_back(a);
        }
        if ((sa <= 0.0) != (sc <= 0.0) && sa != 0.0 && sc != 0.0) {
          const P3 x = add(a, scale(sub(c, a), sa / (sa - sc)));
          g.poly.push_back(x);
          cap.push_back(x);
        }
      }
      if (g.poly.size() >= 3) next.push_back(std::move(g));
    }
    // distinct cap points, ordered by angle around their centroid in the plane
    std::vector<P3> pts;
    for (const P3& v : cap) {
      bool dup = false;
      for (const P3& u : pts)
        if (std::fabs(u.x - v.x) <= eps && std::fabs(u.y - v.y) <= eps && std::fabs(u.z - v.z) <= eps) dup = true;
      if (!dup) pts.push_back(v);
    }
    if (pts.size() >= 3) {
      P3 o{0, 0, 0};
      for (const P3& v : pts) o = add(o, v);
      o = scale(o, 1.0 / (double)pts.size());
      const P3 nn = scale(n, 1.0 / std::sqrt(dotp(n, n)));
      P3 u = std::fabs(nn.x) < 0.9 ? crossp(nn, P3{1, 0, 0}) : crossp(nn, P3{0, 1, 0});
      u = scale(u, 1.0 / std::sqrt(dotp(u, u)));
      const P3 w = crossp(nn, u);
      std::vector<std::pair<double, P3>> ang;
      for (const P3& v : pts) ang.push_back({std::atan2(dotp(sub(v, o), w), dotp(sub(v, o), u)), v});
      std::sort(ang.begin(), ang.end(), [](const auto& a, const auto& c) { return a.first < c.first; });
      Facet g{{}, nbr, sx, sy, sz};
      for (const auto& a : ang) g.poly.push_back(a.second);
      next.push_back(std::move(g));
    }
    facets.swap(next);
  }
};

double facet_area(const std::vector<P3>& poly) {
  P3 acc{0, 0, 0};
  for (size_t k = 1; k + 1 < poly.size(); ++k) acc = add(acc, crossp(sub(poly[k], poly[0]), sub(poly[k + 1], poly[0])));
  return 0.5 * std::sqrt(dotp(acc, acc));
}

struct FaceOut {
  int64_t nbr;
  int sx, sy, sz;
  double area;
};

bool face_less(const FaceOut& a, const FaceOut& b) {
  if (a.nbr != b.nbr) return a.nbr < b.nbr;
  if (a.sx != b.sx) return a.sx < b.sx;
  if (a.sy != b.sy) return a.sy < b.sy;
  return a.sz < b.sz;
}

struct Tessellation {
  const double* pts;
  int64_t n;
  double L;
  int nb;       // buckets per side
  double h;     // bucket width
  std::vector<int64_t> start;
  std::vector<int64_t> members;
  std::vector<std::vector<FaceOut>> faces;
  std::vector<double> volume;
  std::atomic<int64_t> failed{0};

  P3 at(int64_t i) const { return {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]}; }
  int bucket_of(double c) const { return std::min(std::max((int)std::floor(c / h), 0), nb - 1); }

  void bucketize() {
    nb = std::max(1, (int)std::floor(std::cbrt((double)n)));
    h = L / nb;
    const int64_t nbt = (int64_t)nb * nb * nb;
    start.assign(nbt + 1, 0);
    std::vector<int64_t> id(n);
    for (int64_t i = 0; i < n; ++i) {
      P3 p = at(i);
      id[i] = ((int64_t)bucket_of(p.x) * nb + bucket_of(p.y)) * nb + bucket_of(p.z);
      start[id[i] + 1]++;
    }
    for (int64_t k = 0; k < nbt; ++k) start[k + 1] += start[k];
    members.assign(n, 0);
    std::vector<int64_t> fill(start.begin(), start.end() - 1);
    for (int64_t i = 0; i < n; ++i) members[fill[id[i]]++] = i;
  }

  // (p_j + shift * L) - p_i, evaluated as (p_j - p_i) + shift * L
  P3 delta(int64_t i, int64_t j, int sx, int sy, int sz) const {
    P3 pi = at(i), pj = at(j);
    return {(pj.x - pi.x) + sx * L, (pj.y - pi.y) + sy * L, (pj.z - pi.z) + sz * L};
  }

  bool build(int64_t i, Cell& cell, std::vector<std::pair<double, std::array<int64_t, 4>>>& cand) {
    const P3 p = at(i);
    const int b[3] = {bucket_of(p.x), bucket_of(p.y), bucket_of(p.z)};
    const int max_shell = std::max(1, nb);  // images up to one box length away
    cell.cube((max_shell + 1) * h);
    const double eps = 1e-12 * h;
    for (int r = 0; r <= max_shell; ++r) {
      cand.clear();
      for (int ox = -r; ox <= r; ++ox)
        for (int oy = -r; oy <= r; ++oy)
          for (int oz = -r; oz <= r; ++oz) {
            if (std::max(std::abs(ox), std::max(std::abs(oy), std::abs(oz))) != r) continue;
            int q[3] = {b[0] + ox, b[1] + oy, b[2] + oz}, s[3];
            for (int a = 0; a < 3; ++a) {
              int w = ((q[a] % nb) + nb) % nb;
              s[a] = (q[a] - w) / nb;
              q[a] = w;
            }
            const int64_t bk = ((int64_t)q[0] * nb + q[1]) * nb + q[2];
            for (int64_t k = start[bk]; k < start[bk + 1]; ++k) {
              const int64_t j = members[k];
              if (j == i && s[0] == 0 && s[1] == 0 && s[2] == 0) continue;
              const P3 d = delta(i, j, s[0], s[1], s[2]);
              cand.push_back({dotp(d, d), {j, s[0], s[1], s[2]}});
            }
          }
      std::sort(cand.begin(), cand.end(), [](const auto& a, const auto& c) {
        return a.first != c.first ? a.first < c.first : a.second < c.second;
      });
      double r2 = cell.radius2();
      for (const auto& c : cand) {
        if (c.first > 4.0 * r2) break;
        const int64_t j = c.second[0];
        const int sx = (int)c.second[1], sy = (int)c.second[2], sz = (int)c.second[3];
        const P3 d = delta(i, j, sx, sy, sz);
        // bisector half-space around the origin p_i: d.q <= |d|^2 / 2
        cell.clip(d, 0.5 * dotp(d, d), j, sx, sy, sz, eps);
        r2 = cell.radius2();
      }
      // every generator beyond shell r is at least r * h away
      if (4.0 * r2 <= (double)r * r * h * h) break;
      if (r == max_shell) return false;
    }
    std::vector<FaceOut>& out = faces[i];
    out.clear();
    double vol = 0.0;
    for (const Facet& f : cell.facets) {
      if (f.nbr < 0) return false;  // a face of the starting cube survived
      const double a = facet_area(f.poly);
      const P3 d = delta(i, f.nbr, f.sx, f.sy, f.sz);
      vol += a * (0.5 * std::sqrt(dotp(d, d))) / 3.0;  // pyramid over the face, apex p_i
      out.push_back(FaceOut{f.nbr, f.sx, f.sy, f.sz, a});
    }
    std::sort(out.begin(), out.end(), face_less);
    volume[i] = vol;
    return true;
  }

  void run(int threads) {
    faces.assign(n, {});
    volume.assign(n, 0.0);
    std::atomic<int64_t> next{0};
    auto worker = [&] {
      Cell cell;
      std::vector<std::pair<double, std::array<int64_t, 4>>> cand;
      for (;;) {
        const int64_t s = next.fetch_add(512);
        if (s >= n) break;
        for (int64_t i = s; i < std::min(n, s + 512); ++i)
          if (!build(i, cell, cand)) failed++;
      }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; ++t) pool.emplace_back(worker);
    worker();
    for (std::thread& t : pool) t.join();
  }
};

}  // namespace

struct orc_voronoi {
  int64_t n = 0, failed = 0, dropped = 0;
  std::vector<int64_t> row_ptr;
  std::vector<int32_t> nbr;
  std::vector<uint8_t> kind;
  std::vector<double> area, normal, volume, size;
};

extern "C" {

orc_voronoi* orc_voronoi_build(const double* points, int64_t n, double box, int32_t num_threads) {
  if (!points || n < 1 || n >= ((int64_t)1 << 31) || !(box > 0.0)) return nullptr;
  Tessellation T;
  T.pts = points;
  T.n = n;
  T.L = box;
  T.bucketize();
  T.run(num_threads > 1 ? num_threads : 1);
  orc_voronoi* g = new orc_voronoi();
  g->n = n;
  g->failed = T.failed.load();
  g->row_ptr.assign(n + 1, 0);
  for (int64_t i = 0; i < n; ++i) {
    for (const FaceOut& f : T.faces[i]) {
      const std::vector<FaceOut>& other = T.faces[f.nbr];
      const FaceOut key{i, -f.sx, -f.sy, -f.sz, 0.0};
      auto it = std::lower_bound(other.begin(), other.end(), key, face_less);
      if (it == other.end() || it->nbr != i || it->sx != key.sx || it->sy != key.sy || it->sz != key.sz) {
        g->dropped++;
        continue;
      }
      const P3 d = T.delta(i, f.nbr, f.sx, f.sy, f.sz);
      const double inv = 1.0 / std::sqrt(dotp(d, d));
      g->nbr.push_back((int32_t)f.nbr);
      g->kind.push_back((f.sx | f.sy | f.sz) ? ORC_LOCAL_PERIODIC : ORC_LOCAL);
      g->area.push_back(f.nbr < i ? it->area : f.area);
      g->normal.push_back(d.x * inv);
      g->normal.push_back(d.y * inv);
      g->normal.push_back(d.z * inv);
    }
    g->row_ptr[i + 1] = (int64_t)g->nbr.size();
  }
  g->volume = T.volume;
  g->size.resize(n);
  const double kPi = 3.14159265358979323846;
  for (int64_t i = 0; i < n; ++i) g->size[i] = std::cbrt(3.0 * g->volume[i] / (4.0 * kPi));
  return g;
}

int64_t orc_voronoi_num_faces(const orc_voronoi* g) { return g ? (int64_t)g->nbr.size() : -1; }
int64_t orc_voronoi_failed_cells(const orc_voronoi* g) { return g ? g->failed : -1; }
int64_t orc_voronoi_dropped_faces(const orc_voronoi* g) { return g ? g->dropped : -1; }

void orc_voronoi_copy(const orc_voronoi* g, int64_t* row_ptr, int32_t* nbr, uint8_t* kind, double* area,
                      double* normal, double* volume, double* size) {
  std::copy(g->row_ptr.begin(), g->row_ptr.end(), row_ptr);
  std::copy(g->nbr.begin(), g->nbr.end(), nbr);
  std::copy(g->kind.begin(), g->kind.end(), kind);
  std::copy(g->area.begin(), g->area.end(), area);
  std::copy(g->normal.begin(), g->normal.end(), normal);
  std::copy(g->volume.begin(), g->volume.end(), volume);
  std::copy(g->size.begin(), g->size.end(), size);
}

void orc_voronoi_free(orc_voronoi* g) { delete g; }

}  // extern "C"
