// meshgen.cpp — synthetic dyad meshes written in the reference's mesh file set.
//
// Two layouts share one tetrahedralisation and writer: the box dyad (one
// cleft footprint) and the multi-site release unit (several footprints with
// their own RyR clusters over one box, JSR caps joined by thin JSR sheets).
//
// The reference builds its meshes with TetGen from a T-tubule/JSR geometry
// (mesh/main.cpp:26-507) and writes <base>.node, <base>.ele,
// <base>_tet_properties.txt, <base>_face_properties.txt, <base>_ryr.txt and
// <base>_lcc.txt (mesh/main.cpp:498-505, 511-567, 1305-1364).  This generator
// writes the same six files for a box dyad instead:
//   * an axis-aligned box cut by graded planes into hexahedra, each split into
//     six tetrahedra along its main diagonal (Kuhn/Freudenthal split, which is
//     conforming between neighbouring cells);
//   * the bottom face z = 0 is a flat T-tubule membrane (face type 2), the
//     other box faces are domain boundaries (type 1);
//   * a cleft slab [0, cleft_h] over a rectangular footprint, capped by a JSR
//     slab [cleft_h, cleft_h + jsr_h] (region 1) whose faces toward the
//     cytosol are JSR membrane (type 3);
//   * troponin C in cytosolic tets farther than r_trpn from the membrane;
//   * RyRs on a square lattice or a Poisson-disk cluster in the cleft, each
//     assigned to the nearest cytosolic / JSR tet centroid, and LCCs placed
//     uniformly at random in the footprint, assigned to the nearest centroid
//     (the reference's nearest-centroid rule, mesh/main.cpp:679-733).
// Per-face geometry (area vector, r1, r2, e_xi, d_xi and the coefficient
// |A_f|^2 / (d_xi A_f.e_xi)) follows the reference's definitions at
// mesh/main.cpp:334-481 so the solver sees the same kind of operator.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "srs_host.h"

namespace srs {

namespace {

struct V3 {
  double x, y, z;
};
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 scl(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double norm(V3 a) { return std::sqrt(dot(a, a)); }

// splitmix64: small deterministic generator for placement only.
struct SplitMix {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

// Plane positions on [lo, hi] with n_in uniform cells on [-half, half]
// (centred on 0) and geometric grading outside.  Requires lo < -half, hi > half.
std::vector<double> graded_axis_sym(double lo, double hi, double half, int n_in, int n_out_lo,
                                    int n_out_hi) {
  std::vector<double> p;
  auto grow = [](double start, double end, int n, double h0) {
    // n cells from start to end, first cell ~h0, geometric ratio solved by bisection.
    std::vector<double> w(n);
    double L = std::fabs(end - start);
    double g = 1.0;
    if (n > 1 && h0 * n < L) {
      double a = 1.0, b = 10.0;
      for (int it = 0; it < 200; ++it) {
        double m = 0.5 * (a + b);
        double s = h0 * (std::pow(m, n) - 1.0) / (m - 1.0);
        if (s > L) b = m; else a = m;
      }
      g = 0.5 * (a + b);
    }
    double acc = 0.0;
    for (int i = 0; i < n; ++i) {
      w[i] = (g == 1.0) ? L / n : h0 * std::pow(g, i);
      acc += w[i];
    }
    for (int i = 0; i < n; ++i) w[i] *= L / acc;
    return w;
  };
  double h_in = 2.0 * half / n_in;
  std::vector<double> wl = grow(-half, lo, n_out_lo, h_in);
  std::vector<double> wh = grow(half, hi, n_out_hi, h_in);
  double x = -half;
  std::vector<double> left;
  for (int i = 0; i < n_out_lo; ++i) {
    x -= wl[i];
    left.push_back(x);
  }
  left.back() = lo;
  for (int i = (int)left.size() - 1; i >= 0; --i) p.push_back(left[i]);
  for (int i = 0; i <= n_in; ++i) p.push_back(-half + h_in * i);
  x = half;
  for (int i = 0; i < n_out_hi; ++i) {
    x += wh[i];
    p.push_back(x);
  }
  p.back() = hi;
  return p;
}


// Tetrahedra of a tensor grid of hexahedra and the per-tet properties.
struct Body {
  int nx = 0, ny = 0, nz = 0, NN = 0, NE = 0;
  std::vector<V3> P, cen;
  std::vector<int> tv, region, tropc;
  std::vector<double> V0;
};

// region_of(x0, x1, y0, y1, z0, z1): 0 cytosol, 1 JSR for the hexahedron
// with those bounds.
template <class RegionOf>
Body build_body(const std::vector<double>& X, const std::vector<double>& Y,
                const std::vector<double>& Z, RegionOf region_of, double r_trpn) {
  Body B;
  const int nx = (int)X.size() - 1, ny = (int)Y.size() - 1, nz = (int)Z.size() - 1;
  const int NXp = nx + 1, NYp = ny + 1, NZp = nz + 1;
  auto vid = [&](int i, int j, int k) { return (k * NYp + j) * NXp + i; };
  const int NN = NXp * NYp * NZp;
  std::vector<V3> P(NN);
  for (int k = 0; k < NZp; ++k)
    for (int j = 0; j < NYp; ++j)
      for (int i = 0; i < NXp; ++i) P[vid(i, j, k)] = {X[i], Y[j], Z[k]};

  // ---- tetrahedra (6 per hexahedron, along the v000-v111 diagonal) ---------
  const int NE = nx * ny * nz * 6;
  std::vector<int> tv(4 * (size_t)NE);
  std::vector<int> region(NE);
  const int perms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  int e = 0;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const int reg = region_of(X[i], X[i + 1], Y[j], Y[j + 1], Z[k], Z[k + 1]);
        for (int p = 0; p < 6; ++p) {
          int c[3] = {i, j, k};
          tv[4 * e + 0] = vid(c[0], c[1], c[2]);
          for (int q = 0; q < 2; ++q) {
            c[perms[p][q]] += 1;
            tv[4 * e + 1 + q] = vid(c[0], c[1], c[2]);
          }
          tv[4 * e + 3] = vid(i + 1, j + 1, k + 1);
          region[e] = reg;
          ++e;
        }
      }

  // ---- per-tet properties ---------------------------------------------------
  std::vector<V3> cen(NE);
  std::vector<double> V0(NE);
  std::vector<int> tropc(NE);
  for (int t = 0; t < NE; ++t) {
    V3 a = P[tv[4 * t]], b = P[tv[4 * t + 1]], c = P[tv[4 * t + 2]], d = P[tv[4 * t + 3]];
    cen[t] = {(a.x + b.x + c.x + d.x) / 4, (a.y + b.y + c.y + d.y) / 4, (a.z + b.z + c.z + d.z) / 4};
    V3 u = sub(a, d), v = sub(b, d), w = sub(c, d);
    V0[t] = std::fabs(dot(u, cross(v, w))) / 6.0;
    tropc[t] = (region[t] == 0 && cen[t].z > r_trpn) ? 1 : 0;
  }

  B.nx = nx;
  B.ny = ny;
  B.nz = nz;
  B.NN = NN;
  B.NE = NE;
  B.P = std::move(P);
  B.cen = std::move(cen);
  B.tv = std::move(tv);
  B.region = std::move(region);
  B.tropc = std::move(tropc);
  B.V0 = std::move(V0);
  return B;
}

// Nearest tet centroid to p (first minimum in tet order) of region
// want_region (-1: any), among `cand` (every tet when null).
int nearest_tet(const Body& B, V3 p, int want_region, const std::vector<int>* cand) {
  double best = 1e300;
  int bi = -1;
  const int n = cand ? (int)cand->size() : B.NE;
  for (int q = 0; q < n; ++q) {
    const int t = cand ? (*cand)[q] : q;
    if (want_region >= 0 && B.region[t] != want_region) continue;
    V3 d = sub(B.cen[t], p);
    double r2 = dot(d, d);
    if (r2 < best) {
      best = r2;
      bi = t;
    }
  }
  return bi;
}

// Channel placement: RyR cleft / JSR tets, lattice neighbours, LCC tets.
struct Chan {
  std::vector<int> ryr_ele, ryr_jsr, ryr_nb, lcc_ele;
};

// Poisson-disk dart throwing of `count` points at least `pitch` apart inside
// the disc of radius `radius` around (cx, cy); false when it cannot place them.
bool poisson_disc(SplitMix& rng, double cx, double cy, double radius, double pitch, int count,
                  std::vector<V3>* out) {
  std::vector<V3> pts;
  int tries = 0;
  while ((int)pts.size() < count && tries < 2000000) {
    ++tries;
    double x = (2.0 * rng.uniform() - 1.0) * radius;
    double y = (2.0 * rng.uniform() - 1.0) * radius;
    if (x * x + y * y > radius * radius) continue;
    bool ok = true;
    for (auto& p : pts) {
      double dx = p.x - x, dy = p.y - y;
      if (dx * dx + dy * dy < pitch * pitch) {
        ok = false;
        break;
      }
    }
    if (ok) pts.push_back({x + cx, y + cy, 0.0});
  }
  if ((int)pts.size() < count) return false;
  *out = pts;
  return true;
}

// Lattice neighbours of a Poisson-disk cluster: up to four nearest within
// 1.5 x pitch, nearest first; indices offset by `base`.
void disc_neighbours(const std::vector<V3>& pts, double pitch, int base, std::vector<int>* nb) {
  const int n = (int)pts.size();
  for (int a = 0; a < n; ++a) {
    std::vector<std::pair<double, int>> d;
    for (int b = 0; b < n; ++b) {
      if (a == b) continue;
      double dx = pts[a].x - pts[b].x, dy = pts[a].y - pts[b].y;
      double r = std::sqrt(dx * dx + dy * dy);
      if (r < 1.5 * pitch) d.push_back({r, b});
    }
    std::sort(d.begin(), d.end());
    for (int q = 0; q < 4; ++q) nb->push_back(q < (int)d.size() ? base + d[q].second : -1);
  }
}

// Faces, face geometry and the six files of the reference's mesh set.
int write_mesh(const Body& B, const Chan& ch, int flag_tt, const char* base, MeshGenReport* rep) {
  const int NE = B.NE, NN = B.NN;
  const std::vector<int>& tv = B.tv;
  const std::vector<int>& region = B.region;
  const std::vector<V3>& P = B.P;
  const std::vector<V3>& cen = B.cen;
  const std::vector<double>& V0 = B.V0;
  const std::vector<int>& tropc = B.tropc;
  const std::vector<int>& ryr_ele = ch.ryr_ele;
  const std::vector<int>& ryr_jsr = ch.ryr_jsr;
  const std::vector<int>& ryr_nb = ch.ryr_nb;
  const std::vector<int>& lcc_ele = ch.lcc_ele;
  const int NR = (int)ryr_ele.size();
  std::vector<double> TT(NE, 0.0), SR(NE, 0.0);
  // ---- faces ---------------------------------------------------------------
  struct FaceRec {
    int t1, t2;
    int v[3];
  };
  std::vector<FaceRec> faces;
  faces.reserve((size_t)NE * 2 + 1024);
  std::unordered_map<uint64_t, int> fmap;
  fmap.reserve((size_t)NE * 3);
  const int fl[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};
  for (int t = 0; t < NE; ++t) {
    for (int f = 0; f < 4; ++f) {
      int a = tv[4 * t + fl[f][0]], b = tv[4 * t + fl[f][1]], c = tv[4 * t + fl[f][2]];
      int s3[3] = {a, b, c};
      std::sort(s3, s3 + 3);
      uint64_t key = ((uint64_t)s3[0] * (uint64_t)NN + (uint64_t)s3[1]) * (uint64_t)NN + (uint64_t)s3[2];
      auto it = fmap.find(key);
      if (it == fmap.end()) {
        FaceRec r;
        r.t1 = t;
        r.t2 = -2;
        r.v[0] = a;
        r.v[1] = b;
        r.v[2] = c;
        fmap.emplace(key, (int)faces.size());
        faces.push_back(r);
      } else {
        faces[it->second].t2 = t;
      }
    }
  }
  const int NF = (int)faces.size();


  // ---- face geometry + types, TT/SR areas ------------------------------------
  std::string b(base);
  FILE* ff = std::fopen((b + "_face_properties.txt").c_str(), "w");
  if (!ff) return SRS_ERR_IO;
  std::fprintf(ff, "%d\n", NF);
  std::fprintf(ff,
               "Neighb1 Neighb2 NormX NormY NormZ CentX CentY CentZ Area AfX AfY AfZ r1X r1Y r1Z "
               "r2X r2Y r2Z eXiX eXiY eXiZ dXi FaceCoeff FaceType bElectroDiff\n");
  double max_a0 = 0.0;
  std::vector<double> a0(NE, 0.0);
  int n_type[4] = {0, 0, 0, 0};
  for (int f = 0; f < NF; ++f) {
    FaceRec r = faces[f];
    int t1 = r.t1, t2 = r.t2, type;
    V3 p1 = P[r.v[0]], p2 = P[r.v[1]], p3 = P[r.v[2]];
    V3 c = scl(add(add(p1, p2), p3), 1.0 / 3.0);
    if (t2 >= 0) {
      if (region[t1] == region[t2]) {
        type = 0;
      } else {
        type = 3;  // JSR membrane; list the cytosolic side first
        if (region[t1] == 1) std::swap(t1, t2);
      }
    } else {
      type = (std::fabs(c.z) < 1e-12) ? 2 : 1;
    }
    V3 n = cross(sub(p2, p1), sub(p3, p1));
    double area = norm(n) / 2.0;
    V3 Af = scl(n, 0.5);
    V3 xs = cen[t1];
    if (norm(sub(add(c, Af), xs)) < norm(sub(sub(c, Af), xs))) Af = scl(Af, -1.0);
    double an = norm(Af);
    V3 nrm = scl(Af, 1.0 / an);
    V3 r1 = sub(c, xs);
    V3 r2 = {0, 0, 0}, xi;
    if (t2 >= 0) {
      r2 = sub(c, cen[t2]);
      xi = sub(cen[t2], xs);
    } else {
      xi = sub(c, xs);
    }
    double dxi = norm(xi);
    V3 exi = scl(xi, 1.0 / dxi);
    double coeff = dot(Af, Af) / (dxi * dot(Af, exi));
    if (type == 2 && flag_tt) TT[t1] += area;
    if (type == 3) SR[t1] += area;
    if (type == 0) {
      a0[t1] += coeff / V0[t1];
      a0[t2] += coeff / V0[t2];
    }
    n_type[type]++;
    std::fprintf(ff,
                 "%d %d %.10g %.10g %.10g %.10g %.10g %.10g %.10g %.10g %.10g %.10g %.10g %.10g "
                 "%.10g %.10g %.10g %.10g %.10g %.10g %.10g %.10g %.10g %d\n",
                 t1, t2, nrm.x, nrm.y, nrm.z, c.x, c.y, c.z, area, Af.x, Af.y, Af.z, r1.x, r1.y,
                 r1.z, r2.x, r2.y, r2.z, exi.x, exi.y, exi.z, dxi, coeff, type);
  }
  std::fclose(ff);
  for (int t = 0; t < NE; ++t) max_a0 = std::max(max_a0, a0[t]);

  FILE* ft = std::fopen((b + "_tet_properties.txt").c_str(), "w");
  if (!ft) return SRS_ERR_IO;
  std::fprintf(ft, "%d\n", NE);
  std::fprintf(ft, "CentX CentY CentZ V0 TTSurfaceArea SRSurfaceArea bTroponinC Type\n");
  for (int t = 0; t < NE; ++t)
    std::fprintf(ft, "%.10g %.10g %.10g %.10g %.10g %.10g %d %d\n", cen[t].x, cen[t].y, cen[t].z,
                 V0[t], TT[t], SR[t], tropc[t], region[t]);
  std::fclose(ft);

  FILE* fn = std::fopen((b + ".node").c_str(), "w");
  if (!fn) return SRS_ERR_IO;
  std::fprintf(fn, "%d  3  0  0\n", NN);
  for (int v = 0; v < NN; ++v)
    std::fprintf(fn, "%d  %.10g  %.10g  %.10g\n", v + 1, P[v].x, P[v].y, P[v].z);
  std::fclose(fn);

  FILE* fe = std::fopen((b + ".ele").c_str(), "w");
  if (!fe) return SRS_ERR_IO;
  std::fprintf(fe, "%d  4  1\n", NE);
  for (int t = 0; t < NE; ++t)
    std::fprintf(fe, "%d  %d  %d  %d  %d  %d\n", t + 1, tv[4 * t] + 1, tv[4 * t + 1] + 1,
                 tv[4 * t + 2] + 1, tv[4 * t + 3] + 1, region[t]);
  std::fclose(fe);

  FILE* fr = std::fopen((b + "_ryr.txt").c_str(), "w");
  if (!fr) return SRS_ERR_IO;
  std::fprintf(fr, "%d\n", NR);
  for (int r = 0; r < NR; ++r)
    std::fprintf(fr, "%d %d %d %d %d %d\n", ryr_ele[r], ryr_jsr[r], ryr_nb[4 * r],
                 ryr_nb[4 * r + 1], ryr_nb[4 * r + 2], ryr_nb[4 * r + 3]);
  std::fclose(fr);

  FILE* fl2 = std::fopen((b + "_lcc.txt").c_str(), "w");
  if (!fl2) return SRS_ERR_IO;
  std::fprintf(fl2, "%d\n", (int)lcc_ele.size());
  for (int l : lcc_ele) std::fprintf(fl2, "%d\n", l);
  std::fclose(fl2);

  if (rep) {
    rep->n_tets = NE;
    rep->n_faces = NF;
    rep->n_nodes = NN;
    rep->n_ryr = NR;
    rep->n_lcc = (int)lcc_ele.size();
    int nj = 0;
    for (int t = 0; t < NE; ++t) nj += region[t];
    rep->n_jsr_tets = nj;
    rep->max_a0 = max_a0;
    for (int q = 0; q < 4; ++q) rep->n_face_type[q] = n_type[q];
  }
  return SRS_OK;
}

// Cell widths of a graded segment of length L: sizes start at h0 on the
// left and h1 on the right and grow by `growth` toward the middle, capped at
// hmax; the middle cell takes the remainder (merged into a neighbour when
// it would be a sliver).
std::vector<double> graded_widths(double L, double h0, double h1, double hmax, double growth) {
  std::vector<double> wl, wr;
  double rem = L, sl = std::min(h0, hmax), sr = std::min(h1, hmax);
  while (true) {
    const double smin = std::min(sl, sr);
    if (rem <= 1.5 * smin) break;
    if (sl <= sr) {
      wl.push_back(sl);
      rem -= sl;
      sl = std::min(hmax, sl * growth);
    } else {
      wr.push_back(sr);
      rem -= sr;
      sr = std::min(hmax, sr * growth);
    }
  }
  std::vector<double> w = wl;
  if (rem > 0.5 * std::min(sl, sr) || (w.empty() && wr.empty())) {
    w.push_back(rem);
  } else if (!w.empty()) {
    w.back() += rem;
  } else {
    wr.back() += rem;
  }
  for (int i = (int)wr.size() - 1; i >= 0; --i) w.push_back(wr[i]);
  return w;
}

// Planes on [lo, hi]: uniform cells of about h inside each of the intervals
// (merged where they overlap), graded cells between them and toward the ends.
std::vector<double> axis_multi(double lo, double hi, std::vector<std::pair<double, double>> iv,
                               double h, double hmax, double growth) {
  for (auto& q : iv) {
    q.first = std::max(q.first, lo);
    q.second = std::min(q.second, hi);
  }
  std::sort(iv.begin(), iv.end());
  std::vector<std::pair<double, double>> m;
  for (auto& q : iv) {
    if (q.second <= q.first) continue;
    if (!m.empty() && q.first <= m.back().second + 2.0 * h)
      m.back().second = std::max(m.back().second, q.second);
    else
      m.push_back(q);
  }
  std::vector<double> p{lo};
  double x = lo;
  auto add_widths = [&](const std::vector<double>& w, double end) {
    for (size_t i = 0; i < w.size(); ++i) {
      x += w[i];
      p.push_back(i + 1 == w.size() ? end : x);
    }
    x = end;
  };
  for (size_t k = 0; k <= m.size(); ++k) {
    const double g0 = x, g1 = k < m.size() ? m[k].first : hi;
    if (g1 > g0 + 1e-12)
      add_widths(graded_widths(g1 - g0, k == 0 ? hmax : h, k < m.size() ? h : hmax, hmax, growth), g1);
    if (k < m.size()) {
      const int n = std::max(1, (int)std::lround((m[k].second - m[k].first) / h));
      add_widths(std::vector<double>(n, (m[k].second - m[k].first) / n), m[k].second);
    }
  }
  return p;
}

}  // namespace

int meshgen_box(const MeshGenSpec& s, const char* base, MeshGenReport* rep) {
  // ---- planes -------------------------------------------------------------
  std::vector<double> X = graded_axis_sym(-0.5 * s.box_x, 0.5 * s.box_x, s.foot_half_x,
                                          s.n_foot_x, s.n_out_x, s.n_out_x);
  std::vector<double> Y = graded_axis_sym(-0.5 * s.box_y, 0.5 * s.box_y, s.foot_half_y,
                                          s.n_foot_y, s.n_out_y, s.n_out_y);
  std::vector<double> Z;
  {
    Z.push_back(0.0);
    double zc = s.cleft_h;
    for (int i = 1; i <= s.n_cleft_z; ++i) Z.push_back(zc * i / s.n_cleft_z);
    double zj = s.cleft_h + s.jsr_h;
    for (int i = 1; i <= s.n_jsr_z; ++i) Z.push_back(zc + s.jsr_h * i / s.n_jsr_z);
    // geometric grading above the JSR up to box_z
    int n = s.n_above_z;
    double L = s.box_z - zj, h0 = s.jsr_h / s.n_jsr_z;
    double g = 1.0;
    if (n > 1 && h0 * n < L) {
      double a = 1.0, b = 10.0;
      for (int it = 0; it < 200; ++it) {
        double m = 0.5 * (a + b);
        double sum = h0 * (std::pow(m, n) - 1.0) / (m - 1.0);
        if (sum > L) b = m; else a = m;
      }
      g = 0.5 * (a + b);
    }
    std::vector<double> w(n);
    double acc = 0.0;
    for (int i = 0; i < n; ++i) {
      w[i] = (g == 1.0) ? L / n : h0 * std::pow(g, i);
      acc += w[i];
    }
    double z = zj;
    for (int i = 0; i < n; ++i) {
      z += w[i] * L / acc;
      Z.push_back(i == n - 1 ? s.box_z : z);
    }
  }
  const double zc_hi = s.cleft_h, zj_hi = s.cleft_h + s.jsr_h;
  const Body B = build_body(
      X, Y, Z,
      [&](double x0, double x1, double y0, double y1, double z0, double z1) {
        const double xm = 0.5 * (x0 + x1), ym = 0.5 * (y0 + y1), zm = 0.5 * (z0 + z1);
        bool foot = std::fabs(xm) < s.foot_half_x && std::fabs(ym) < s.foot_half_y;
        return (foot && zm > zc_hi && zm < zj_hi) ? 1 : 0;
      },
      s.r_trpn);

  // ---- channels ------------------------------------------------------------
  std::vector<V3> ryr_pt, ryr_jpt;
  std::vector<int> ryr_nb;
  SplitMix rng{s.seed};
  if (s.ryr_mode == 0) {
    // square lattice nx x ny at pitch, centred on (cx, cy)
    for (int i = 0; i < s.ryr_ny; ++i)
      for (int j = 0; j < s.ryr_nx; ++j) {
        double x = s.ryr_cx + (j - 0.5 * (s.ryr_nx - 1)) * s.ryr_pitch;
        double y = s.ryr_cy + (0.5 * (s.ryr_ny - 1) - i) * s.ryr_pitch;
        ryr_pt.push_back({x, y, s.cleft_h - s.ryr_depth});
        ryr_jpt.push_back({x, y, s.cleft_h});
      }
    for (int i = 0; i < s.ryr_ny; ++i)
      for (int j = 0; j < s.ryr_nx; ++j) {
        ryr_nb.push_back(i > 0 ? (i - 1) * s.ryr_nx + j : -1);
        ryr_nb.push_back(i < s.ryr_ny - 1 ? (i + 1) * s.ryr_nx + j : -1);
        ryr_nb.push_back(j > 0 ? i * s.ryr_nx + j - 1 : -1);
        ryr_nb.push_back(j < s.ryr_nx - 1 ? i * s.ryr_nx + j + 1 : -1);
      }
  } else {
    // Poisson-disk dart throwing inside a disc of radius ryr_radius
    std::vector<V3> pts;
    if (!poisson_disc(rng, s.ryr_cx, s.ryr_cy, s.ryr_radius, s.ryr_pitch, s.ryr_count, &pts))
      return SRS_ERR_INPUT;
    for (auto& p : pts) {
      ryr_pt.push_back({p.x, p.y, s.cleft_h - s.ryr_depth});
      ryr_jpt.push_back({p.x, p.y, s.cleft_h});
    }
    disc_neighbours(pts, s.ryr_pitch, 0, &ryr_nb);
  }
  auto nearest = [&](V3 p, int want_region) { return nearest_tet(B, p, want_region, nullptr); };
  const int NR = (int)ryr_pt.size();
  Chan ch;
  ch.ryr_nb = ryr_nb;
  ch.ryr_ele.resize(NR);
  ch.ryr_jsr.resize(NR);
  for (int r = 0; r < NR; ++r) {
    ch.ryr_ele[r] = nearest(ryr_pt[r], 0);
    ch.ryr_jsr[r] = nearest(ryr_jpt[r], 1);
  }
  SplitMix lrng{s.lcc_seed};
  for (int l = 0; l < s.n_lcc; ++l) {
    double x = s.ryr_cx + (2.0 * lrng.uniform() - 1.0) * s.lcc_half;
    double y = s.ryr_cy + (2.0 * lrng.uniform() - 1.0) * s.lcc_half;
    ch.lcc_ele.push_back(nearest({x, y, 0.0}, -1));
  }


  return write_mesh(B, ch, s.flag_tt, base, rep);
}

int meshgen_multisite(const MultiSiteSpec& s, const char* base, MeshGenReport* rep) {
  if (s.n_sites < 1 || s.n_sites > SRS_MAX_SITES || !(s.h_fine > 0) || !(s.h_max >= s.h_fine) ||
      !(s.growth > 1.0) || s.n_cleft_z < 1 || s.n_jsr_z < 1)
    return SRS_ERR_INPUT;
  std::vector<double> half(s.n_sites);
  std::vector<std::pair<double, double>> ix, iy;
  for (int k = 0; k < s.n_sites; ++k) {
    half[k] = s.site_radius[k] + s.foot_margin;
    ix.push_back({s.site_x[k] - half[k], s.site_x[k] + half[k]});
    iy.push_back({s.site_y[k] - half[k], s.site_y[k] + half[k]});
  }
  const std::vector<double> X = axis_multi(-0.5 * s.box_x, 0.5 * s.box_x, ix, s.h_fine, s.h_max, s.growth);
  const std::vector<double> Y = axis_multi(-0.5 * s.box_y, 0.5 * s.box_y, iy, s.h_fine, s.h_max, s.growth);
  std::vector<double> Z{0.0};
  for (int i = 1; i <= s.n_cleft_z; ++i) Z.push_back(s.cleft_h * i / s.n_cleft_z);
  const double zj = s.cleft_h + s.jsr_h;
  for (int i = 1; i <= s.n_jsr_z; ++i) Z.push_back(s.cleft_h + s.jsr_h * i / s.n_jsr_z);
  {
    const double hz = s.jsr_h / s.n_jsr_z;
    const std::vector<double> w = graded_widths(s.box_z - zj, hz, s.h_max, s.h_max, s.growth);
    double z = zj;
    for (size_t i = 0; i < w.size(); ++i) {
      z += w[i];
      Z.push_back(i + 1 == w.size() ? s.box_z : z);
    }
  }
  // JSR: the cap over every footprint, and sheets joining consecutive sites
  // along an L-shaped path (x first, then y); a cell belongs to a sheet when
  // it overlaps the strip, so sheets stay connected where cells are coarse.
  auto overlaps = [](double a0, double a1, double b0, double b1) { return a0 < b1 && b0 < a1; };
  const Body B = build_body(
      X, Y, Z,
      [&](double x0, double x1, double y0, double y1, double z0, double z1) {
        const double zm = 0.5 * (z0 + z1);
        if (!(zm > s.cleft_h && zm < zj)) return 0;
        const double xm = 0.5 * (x0 + x1), ym = 0.5 * (y0 + y1);
        for (int k = 0; k < s.n_sites; ++k)
          if (std::fabs(xm - s.site_x[k]) < half[k] && std::fabs(ym - s.site_y[k]) < half[k]) return 1;
        for (int k = 0; k + 1 < s.n_sites; ++k) {
          const double xa = std::min(s.site_x[k], s.site_x[k + 1]), xb = std::max(s.site_x[k], s.site_x[k + 1]);
          const double ya = std::min(s.site_y[k], s.site_y[k + 1]), yb = std::max(s.site_y[k], s.site_y[k + 1]);
          const double w = s.sheet_half;
          if (overlaps(x0, x1, xa - w, xb + w) && overlaps(y0, y1, s.site_y[k] - w, s.site_y[k] + w)) return 1;
          if (overlaps(x0, x1, s.site_x[k + 1] - w, s.site_x[k + 1] + w) && overlaps(y0, y1, ya - w, yb + w))
            return 1;
        }
        return 0;
      },
      s.r_trpn);

  Chan ch;
  for (int k = 0; k < s.n_sites; ++k) {
    // candidate tets: centroid over the footprint, below the top of the JSR
    std::vector<int> cand;
    for (int t = 0; t < B.NE; ++t)
      if (std::fabs(B.cen[t].x - s.site_x[k]) < half[k] + s.h_fine &&
          std::fabs(B.cen[t].y - s.site_y[k]) < half[k] + s.h_fine && B.cen[t].z < zj)
        cand.push_back(t);
    SplitMix rng{s.seed + (uint64_t)k};
    std::vector<V3> pts;
    if (!poisson_disc(rng, s.site_x[k], s.site_y[k], s.site_radius[k], s.ryr_pitch, s.site_ryr[k], &pts))
      return SRS_ERR_INPUT;
    const int base_idx = (int)ch.ryr_ele.size();
    for (auto& p : pts) {
      const int ce = nearest_tet(B, {p.x, p.y, s.cleft_h - s.ryr_depth}, 0, &cand);
      const int je = nearest_tet(B, {p.x, p.y, s.cleft_h}, 1, &cand);
      if (ce < 0 || je < 0) return SRS_ERR_INPUT;
      ch.ryr_ele.push_back(ce);
      ch.ryr_jsr.push_back(je);
    }
    disc_neighbours(pts, s.ryr_pitch, base_idx, &ch.ryr_nb);
    SplitMix lrng{s.seed + 100 + (uint64_t)k};
    const int n_lcc = std::max(1, (int)std::lround(s.site_ryr[k] / 7.0));
    for (int l = 0; l < n_lcc; ++l) {
      const double x = s.site_x[k] + (2.0 * lrng.uniform() - 1.0) * half[k];
      const double y = s.site_y[k] + (2.0 * lrng.uniform() - 1.0) * half[k];
      const int le = nearest_tet(B, {x, y, 0.0}, -1, &cand);
      if (le < 0) return SRS_ERR_INPUT;
      ch.lcc_ele.push_back(le);
    }
  }
  return write_mesh(B, ch, s.flag_tt, base, rep);
}

void meshgen_default_spec(MeshGenSpec* s) {
  // 2 x 2 x 2 um box of 12^3 hexahedra (10,368 tets): a 15 nm cleft under a
  // 50 nm JSR cap over a 400 x 400 nm footprint, 7x7 RyRs at 31 nm, 7 LCCs.
  std::memset(s, 0, sizeof(*s));
  s->box_x = 2.0;
  s->box_y = 2.0;
  s->box_z = 2.0;
  s->foot_half_x = 0.2;
  s->foot_half_y = 0.2;
  s->n_foot_x = 8;
  s->n_foot_y = 8;
  s->n_out_x = 2;
  s->n_out_y = 2;
  s->cleft_h = 0.015;
  s->jsr_h = 0.050;
  s->n_cleft_z = 1;
  s->n_jsr_z = 1;
  s->n_above_z = 10;
  s->r_trpn = 0.20;
  s->flag_tt = 1;
  s->ryr_mode = 0;
  s->ryr_nx = 7;
  s->ryr_ny = 7;
  s->ryr_pitch = 0.031;
  s->ryr_depth = 0.010;
  s->ryr_cx = 0.0;
  s->ryr_cy = 0.0;
  s->ryr_count = 49;
  s->ryr_radius = 0.1;
  s->n_lcc = 7;
  s->lcc_half = 0.2;
  s->lcc_seed = 1;
  s->seed = 1;
}

}  // namespace srs
