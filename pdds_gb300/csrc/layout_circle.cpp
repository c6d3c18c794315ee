// Host-side layout of a disk split into rings and sectors (a CircleMesh).
//
// The reference builds rectangular layouts only (Fullfill_interfaces,
// PDDAlgorithms/PDDSparseGM.cpp:346-689; its Circle* mesh files are empty
// stubs).  This layout applies the same rules in polar coordinates:
//   * interfaces are the arcs rho = rho_i between rings (one per sector) and
//     the rays phi = theta_j between sectors (one per ring outside the
//     central disk, which is one subdomain: sectors meeting at the centre make
//     (I + G) nearly singular, cond ~1e4 against ~30 on rectangles), nnode
//     knots per segment with shared end points (cross points);
//   * knots on the central disk's boundary take the disk of radius rho_2 as
//     stencil, whose one side is the whole second arc (periodic);
//   * a knot's stencil is the union of the subdomains next to its
//     interfaces (two for a segment knot, four for a cross point), a polar
//     rectangle {rho0, phi0, rho1, phi1};
//   * a stencil side holds the knots of the interfaces along it plus half of
//     the next interface on either end (STEN_ELONG = 0.5, the index rule of
//     Compute_Stencil, PDDSparseGM.cpp:1845-2041), and its kind counts them
//     as the reference does (-3, +2 per interface, +1 per elongation);
//   * the outer arc rho = R is the domain boundary: the boundary knots take
//     B = g and a stencil side on it has no knots (its exits score g);
//   * sides are ordered N (outer arc), S (inner arc), E (ray at phi1),
//     W (ray at phi0) for the G row, the order G_return_withrep uses.
// Sides are arcs (coordinate along = angle, RBF distance = chord
// 2 r sin(dphi / 2)) or rays (coordinate along = radius); arcs of one radius
// with the same knot spacing and exit extent share one shape by rotation.
#include <algorithm>
#include <array>
#include <cmath>
#include <map>
#include <tuple>

#include "pdds_internal.h"

namespace pdds {

namespace {

struct PolarIface {
  std::vector<int> index;      // knot indices along the interface
  std::vector<double> along;   // angle (arc) or radius (ray) of each knot
};

// Stencils, sides, G rows and side shapes of a polar layout.  kst[v] =
// {p, q, s, w}: rings [p, q), sectors [s, s + w) (s may be -1: angles are
// unwrapped, sector indices taken modulo NS).
std::string circle_stencils(HostLayout& L, const std::vector<double>& rad, int NR, int NS, int n,
                            const double kappa[4], int bps, bool graded, const std::vector<PolarIface>& arcs,
                            const std::vector<PolarIface>& rays, const std::vector<std::array<int, 4>>& kst) {
  const double PI = 3.141592653589793;
  const double dth = 2.0 * PI / NS;
  const double STEN_ELONG = 0.5;
  auto wrap = [&](int j) { return ((j % NS) + NS) % NS; };
  const int K = L.K;
  std::map<std::array<int, 4>, int> stencil_key;
  std::map<std::pair<int, std::vector<int>>, int> side_key;
  // side knots of one stencil side, in the reference's insertion order:
  // second half of the interface before, the interfaces, first half of the
  // interface after; consecutive repeats (shared end points) dropped
  struct Pending {
    std::vector<int> idx;
    std::vector<double> along, px, py;
    int kind = -3;
  };
  auto add_from = [&](Pending& P, const PolarIface& f, double shift, int from, int to, bool arc, double fixed) {
    for (int k = from; k < to; k++) {
      const int v = f.index[k];
      const double a = f.along[k] + shift;
      if (!P.idx.empty() && P.idx.back() == v) continue;
      P.idx.push_back(v);
      P.along.push_back(a);
      P.px.push_back(arc ? fixed * std::cos(a) : a * std::cos(fixed));
      P.py.push_back(arc ? fixed * std::sin(a) : a * std::sin(fixed));
    }
  };
  auto arc_side = [&](int ring, int s, int w) {  // arc rho_ring over sectors [s, s + w)
    Pending P;
    const double r = rad[ring];
    auto iface = [&](int jj) -> const PolarIface& { return arcs[(size_t)ring * NS + wrap(jj)]; };
    auto shift = [&](int jj) { return dth * (jj - wrap(jj)); };
    {
      const PolarIface& a = iface(s - 1);
      P.kind++;
      add_from(P, a, shift(s - 1), (int)((1 - STEN_ELONG) * (a.index.size() - 1)), (int)a.index.size(), true, r);
    }
    for (int jj = s; jj < s + w; jj++) {
      add_from(P, iface(jj), shift(jj), 0, (int)iface(jj).index.size(), true, r);
      P.kind += 2;
    }
    {
      const PolarIface& a = iface(s + w);
      P.kind++;
      add_from(P, a, shift(s + w), 0, (int)(STEN_ELONG * a.index.size()), true, r);
    }
    return P;
  };
  auto ray_side = [&](int p, int q, int jj) {  // ray theta_jj over rings [p, q)
    Pending P;
    const double ang = dth * jj;
    const int j = wrap(jj);
    if (p >= 2) {  // ring 0 has no rays
      const PolarIface& a = rays[(size_t)(p - 1) * NS + j];
      P.kind++;
      add_from(P, a, 0.0, (int)((1 - STEN_ELONG) * (a.index.size() - 1)), (int)a.index.size(), false, ang);
    }
    for (int i = p; i < q; i++) {
      const PolarIface& a = rays[(size_t)i * NS + j];
      add_from(P, a, 0.0, 0, (int)a.index.size(), false, ang);
      P.kind += 2;
    }
    if (q < NR) {
      const PolarIface& a = rays[(size_t)q * NS + j];
      P.kind++;
      add_from(P, a, 0.0, 0, (int)(STEN_ELONG * a.index.size()), false, ang);
    }
    return P;
  };
  L.knot_stencil.assign(K, -1);
  for (int v = 0; v < K; v++) {
    const std::array<int, 4> st4 = kst[v];
    if (st4[0] < 0) return "internal: knot without a stencil";
    const std::array<int, 4> key = {st4[0], st4[1], wrap(st4[2]), st4[3]};
    auto it = stencil_key.find(key);
    if (it != stencil_key.end()) {
      L.knot_stencil[v] = it->second;
      continue;
    }
    const int p = st4[0], q = st4[1], s = st4[2], w = st4[3];
    const bool full = (w == NS);  // the disk of radius rho_q: one periodic arc side
    StencilRec st;
    st.rect[0] = rad[p];
    st.rect[1] = dth * s;
    st.rect[2] = rad[q];
    st.rect[3] = dth * (s + w);
    Pending sides[4];
    bool has[4] = {false, false, false, false};
    for (int d = 0; d < 4; d++) st.glob[d] = 0;
    if (full) {
      if (q >= NR) return "internal: full-circle stencil on the boundary";
      Pending& P = sides[DIR_N];
      for (int jj = 0; jj < NS; jj++) add_from(P, arcs[(size_t)q * NS + jj], 0.0, 0,
                                               (int)arcs[(size_t)q * NS + jj].index.size() - 1, true, rad[q]);
      P.kind = 3;
      has[DIR_N] = true;
    } else {
      if (q < NR) { sides[DIR_N] = arc_side(q, s, w); has[DIR_N] = true; } else { st.glob[DIR_N] = 1; }
      if (p > 0) { sides[DIR_S] = arc_side(p, s, w); has[DIR_S] = true; }
      sides[DIR_E] = ray_side(p, q, s + w);
      has[DIR_E] = true;
      sides[DIR_W] = ray_side(p, q, s);
      has[DIR_W] = true;
    }
    for (int d = 0; d < 4; d++) {
      st.side[d] = -1;
      st.kind[d] = has[d] ? sides[d].kind : -3;
      if (!has[d] || sides[d].idx.empty()) continue;
      Pending& P = sides[d];
      const int kd = P.kind;
      if (kd < 0 || kd > 3) return "internal: circle stencil side kind out of range";
      auto skey = std::make_pair(kd, P.idx);
      auto sit = side_key.find(skey);
      if (sit != side_key.end()) {
        st.side[d] = sit->second;
        continue;
      }
      const bool arc = (d == DIR_N || d == DIR_S);
      SideRec sr;
      sr.n = (int)P.idx.size();
      sr.orient = arc ? 0 : 1;
      sr.kind = kd;
      const double rr = arc ? rad[d == DIR_N ? q : p] : 0.0;
      double spacing = arc ? 2.0 * rr * std::sin(0.5 * dth / (n - 1)) : (rad[1] - rad[0]) / (n - 1);
      if (graded && !arc) {  // a ray crosses rings of different widths: its finest spacing
        spacing = 0.0;
        for (size_t k = 1; k < P.along.size(); k++) {
          const double g = P.along[k] - P.along[k - 1];
          if (g > 0.0 && (spacing == 0.0 || g < spacing)) spacing = g;
        }
      }
      sr.c = kappa[kd] * spacing;
      sr.shape = -1;
      sr.knot_off = (int64_t)L.side_knot.size();
      sr.origin = P.along[0];
      sr.fixed = arc ? rr : dth * (d == DIR_E ? s + w : s);
      for (size_t k = 0; k < P.idx.size(); k++) {
        L.side_knot.push_back(P.idx[k]);
        L.side_px.push_back(P.px[k]);
        L.side_py.push_back(P.py[k]);
        L.side_along.push_back(P.along[k] - sr.origin);
      }
      L.max_side = std::max(L.max_side, sr.n);
      side_key[skey] = (int)L.sides.size();
      st.side[d] = (int)L.sides.size();
      L.sides.push_back(sr);
    }
    // G row: sorted union of the side knots; positions and owners in side
    // order N, S, E, W (later sides overwrite shared knots)
    std::vector<int> cols;
    for (int d = 0; d < 4; d++)
      if (st.side[d] >= 0) {
        const SideRec& sr = L.sides[st.side[d]];
        for (int k = 0; k < sr.n; k++) cols.push_back(L.side_knot[sr.knot_off + k]);
      }
    std::sort(cols.begin(), cols.end());
    cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
    st.cols = cols;
    st.row_len = (int)cols.size();
    st.map_off = (int64_t)L.map_pos.size();
    std::map<int, int64_t> last_writer;
    for (int d = 0; d < 4; d++) {
      if (st.side[d] < 0) continue;
      const SideRec& sr = L.sides[st.side[d]];
      for (int k = 0; k < sr.n; k++) {
        const int v2 = L.side_knot[sr.knot_off + k];
        last_writer[v2] = (int64_t)L.map_pos.size();
        L.map_pos.push_back((int)(std::lower_bound(cols.begin(), cols.end(), v2) - cols.begin()));
        L.map_owner.push_back(0);
      }
    }
    for (auto& kv : last_writer) L.map_owner[kv.second] = 1;
    const int sid = (int)L.stencils.size();
    stencil_key[key] = sid;
    L.knot_stencil[v] = sid;
    L.stencils.push_back(st);
  }
  L.row_ptr.assign(K + 1, 0);
  for (int v = 0; v < K; v++) {
    const int len = L.knot_boundary[v] ? 0 : L.stencils[L.knot_stencil[v]].row_len;
    L.row_ptr[v + 1] = L.row_ptr[v] + len;
  }
  // shapes: sides equal up to rotation (arcs) or translation (rays)
  std::map<std::tuple<int, int, long long, long long, long long, long long, long long, long long>, int> shape_key;
  std::vector<std::vector<std::pair<int, int>>> uses(L.sides.size());
  for (size_t si = 0; si < L.stencils.size(); si++)
    for (int d = 0; d < 4; d++)
      if (L.stencils[si].side[d] >= 0) uses[L.stencils[si].side[d]].push_back({(int)si, d});
  for (size_t sd = 0; sd < L.sides.size(); sd++) {
    SideRec& sr = L.sides[sd];
    std::vector<double> t(L.side_along.begin() + sr.knot_off, L.side_along.begin() + sr.knot_off + sr.n);
    const double gap = sr.n > 1 ? t[1] - t[0] : 1.0;
    long long sig = 0;  // the knots' positions along the side (graded rays differ inside)
    for (int k = 0; k < sr.n; k++) sig = sig * 1000003LL + std::llround(t[k] / gap * 1e6);
    double lo = 1e300, hi = -1e300;
    for (auto& u : uses[sd]) {
      const StencilRec& st = L.stencils[u.first];
      double a = sr.orient == 0 ? st.rect[1] : st.rect[0];
      double b = sr.orient == 0 ? st.rect[3] : st.rect[2];
      if (sr.orient == 0) {  // bring the stencil's angles next to the side's origin
        const double off = a - sr.origin - std::remainder(a - sr.origin, 2.0 * PI);
        a -= off;
        b -= off;
      }
      lo = std::min(lo, a - sr.origin);
      hi = std::max(hi, b - sr.origin);
    }
    const double Rs = sr.orient == 0 ? sr.fixed : 0.0;
    auto key = std::make_tuple(sr.n, sr.orient, (long long)std::llround(gap * 1e12), (long long)std::llround(sr.c * 1e12),
                               (long long)std::llround(Rs * 1e12), (long long)std::llround(lo / gap * 1e6),
                               (long long)std::llround(hi / gap * 1e6), sig);
    auto it = shape_key.find(key);
    if (it == shape_key.end()) {
      ShapeRec sh;
      sh.n = sr.n;
      sh.c = sr.c;
      sh.R = Rs;
      sh.t = t;
      sh.lo = lo;
      sh.hi = hi;
      shape_key[key] = (int)L.shapes.size();
      sr.shape = (int)L.shapes.size();
      L.shapes.push_back(sh);
    } else {
      sr.shape = it->second;
    }
  }
  int64_t ip = 0;
  for (auto& sh : L.shapes) {
    sh.ipsi_off = ip;
    ip += (int64_t)sh.n * sh.n;
  }
  set_shape_bins(L, bps);
  return "";
}

}  // namespace

std::string build_circle_layout(HostLayout& L, double R, int NR, int NS, int n, const double kappa[4], int bps,
                                double ring_ratio) {
  if (!(R > 0.0)) return "circle layout needs R > 0";
  if (NR < 2 || NS < 3 || n < 3) return "circle layout needs nrings >= 2, nsectors >= 3, nnode >= 3";
  if (NS < 5) return "circle layout needs nsectors >= 5 (stencils span two sectors each side)";
  L = HostLayout();
  L.geom = 1;
  L.radius = R;
  L.nrings = NR;
  L.nsectors = NS;
  L.nsub = NR;
  L.nnode = n;
  L.sw[0] = L.sw[1] = -R;
  L.ne[0] = L.ne[1] = R;
  for (int i = 0; i < 4; i++) L.fac[i] = kappa[i];
  const double PI = 3.141592653589793;
  const double dth = 2.0 * PI / NS, drho = R / NR;
  // ring boundaries: equal rings, or ring i ring_ratio^i times as wide as the
  // central disk's radius (the outer boundary exactly R)
  const bool graded = ring_ratio != 1.0;
  if (!(ring_ratio > 0.0)) return "circle layout needs ring_ratio > 0";
  std::vector<double> rad(NR + 1);
  {
    double tot = 0.0, w = 1.0;
    for (int i = 0; i < NR; i++, w *= ring_ratio) tot += w;
    double acc = 0.0;
    w = 1.0;
    for (int i = 0; i <= NR; i++, w *= ring_ratio) {
      rad[i] = graded ? (i == NR ? R : R * acc / tot) : drho * i;
      acc += w;
    }
  }
  auto rho = [&](int i) { return rad[i]; };
  auto theta = [&](int j) { return dth * j; };
  auto wrap = [&](int j) { return ((j % NS) + NS) % NS; };
  // ---- knots: cross points, arc interiors, ray interiors, boundary points
  int K = 0;
  std::vector<int> cross((size_t)(NR + 1) * NS, -1);  // [i][j], rings 1 .. NR-1
  std::vector<double> kx, ky;
  auto add_knot = [&](double r, double a) {
    kx.push_back(r * std::cos(a));
    ky.push_back(r * std::sin(a));
    return K++;
  };
  std::vector<PolarIface> arcs((size_t)(NR + 1) * NS), rays((size_t)NR * NS);  // arcs[i][j], rays[i][j]
  for (int i = 1; i < NR; i++)
    for (int j = 0; j < NS; j++) cross[(size_t)i * NS + j] = add_knot(rho(i), theta(j));
  for (int i = 1; i < NR; i++)
    for (int j = 0; j < NS; j++) {
      PolarIface& f = arcs[(size_t)i * NS + j];
      f.index.push_back(cross[(size_t)i * NS + j]);
      f.along.push_back(theta(j));
      for (int k = 1; k < n - 1; k++) {
        const double a = theta(j) + dth * k / (n - 1);
        f.index.push_back(add_knot(rho(i), a));
        f.along.push_back(a);
      }
      f.index.push_back(cross[(size_t)i * NS + wrap(j + 1)]);
      f.along.push_back(theta(j + 1));
    }
  std::vector<int> bnd(NS);
  for (int j = 0; j < NS; j++) bnd[j] = add_knot(R, theta(j));
  for (int i = 1; i < NR; i++)  // the central disk (ring 0) has no rays
    for (int j = 0; j < NS; j++) {
      PolarIface& f = rays[(size_t)i * NS + j];
      f.index.push_back(cross[(size_t)i * NS + j]);
      f.along.push_back(rho(i));
      for (int k = 1; k < n - 1; k++) {
        const double r = rho(i) + (graded ? rad[i + 1] - rad[i] : drho) * k / (n - 1);
        f.index.push_back(add_knot(r, theta(j)));
        f.along.push_back(r);
      }
      f.index.push_back(i + 1 < NR ? cross[(size_t)(i + 1) * NS + j] : bnd[j]);
      f.along.push_back(rho(i + 1));
    }
  L.K = K;
  L.kx = kx;
  L.ky = ky;
  L.order.resize(K);
  for (int v = 0; v < K; v++) L.order[v] = v;
  L.knot_boundary.assign(K, 0);
  for (int j = 0; j < NS; j++) L.knot_boundary[bnd[j]] = 1;
  L.nboundary = NS;
  // ---- stencil of every knot: rings [p, q), sectors [s, s + w)
  std::vector<std::array<int, 4>> kst(K, {-1, -1, -1, -1});
  // knots on the first arc (the central disk's boundary): the disk of radius
  // rho_2 (the central disk and the first ring), a stencil with one side,
  // the whole second arc
  for (int i = 1; i < NR; i++)
    for (int j = 0; j < NS; j++) {
      const PolarIface& f = arcs[(size_t)i * NS + j];
      for (size_t k = 1; k + 1 < f.index.size(); k++) kst[f.index[k]] = i == 1 ? std::array<int, 4>{0, 2, 0, NS}
                                                                               : std::array<int, 4>{i - 1, i + 1, j, 1};
      kst[cross[(size_t)i * NS + j]] = i == 1 ? std::array<int, 4>{0, 2, 0, NS} : std::array<int, 4>{i - 1, i + 1, j - 1, 2};
    }
  for (int i = 1; i < NR; i++)
    for (int j = 0; j < NS; j++) {
      const PolarIface& f = rays[(size_t)i * NS + j];
      for (size_t k = 1; k + 1 < f.index.size(); k++) kst[f.index[k]] = {i, i + 1, j - 1, 2};
      if (i == NR - 1) kst[f.index.back()] = {i, i + 1, j - 1, 2};  // boundary knot: no paths, B = g
    }
  return circle_stencils(L, rad, NR, NS, n, kappa, bps, graded, arcs, rays, kst);
}

}  // namespace pdds
