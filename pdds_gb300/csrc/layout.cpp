// Host-side layout of the PDDSparse interface system: knots, stencils, stencil
// sides and side shapes.  Follows the reference's construction exactly,
// including its floating-point order, so knot coordinates are bit-identical:
//   Fullfill_interfaces      PDDAlgorithms/PDDSparseGM.cpp:346-689 (INTERSECTIONS_YES)
//   server hand-out order    PDDAlgorithms/PDDSparseGM.cpp:705-756
//   Get_Interfaces, Labels_Stencil  PDDAlgorithms/PDDSparseGM.cpp:1316-1433
//   Compute_Stencil          PDDAlgorithms/PDDSparseGM.cpp:1845-2041 (STEN_ELONG 0.5)
//   Interface::N/S/E/W       Meshes/interface.cpp:16-93
//   Stencil::Init            Meshes/stencil.cpp:11-85
//   G_return_withrep order   Meshes/stencil.cpp:343-406 (sides N, S, E, W; later overwrites)
// The reference rebuilds a stencil for every knot; here knots that belong to
// the same interface (or the same cross point) share one stencil record, and
// stencil sides with identical knot lists share one side record.
#include <algorithm>
#include <climits>
#include <cstdint>
#include <cstring>
#include <cmath>
#include <map>
#include <string>
#include <thread>
#include <tuple>
#include <unordered_map>

#include "pdds_internal.h"

namespace pdds {

namespace {

struct Lab {
  int a, b;
};

// Position of interface [a, b] in the reference's interfaces vector, or -1.
int lab_id(int nsub, Lab l) {
  if (l.b >= 0 && (l.b % 2) == 1) {  // horizontal [j, 2i+1]
    const int i = (l.b - 1) / 2, j = l.a;
    if (i < 0 || i > nsub - 2 || j < 0 || j > nsub - 1) return -1;
    return 2 * (i * nsub + j);
  }
  if (l.b >= 0 && (l.b % 2) == 0) {  // vertical [i, 2j]
    const int i = l.a, j = l.b / 2;
    if (i < 0 || i > nsub - 2 || j < 0 || j > nsub - 1) return -1;
    return 2 * (i * nsub + j) + 1;
  }
  return -1;
}

// Interface::N/S/E/W; label[1] % 2 == 0 means vertical.
void lab_N(Lab l, std::vector<Lab>& o) {
  o.clear();
  if (l.b % 2 == 0) { o.push_back({l.a, l.b + 1}); o.push_back({l.a + 1, l.b + 1}); }
  else o.push_back({l.a, l.b + 2});
}
void lab_S(Lab l, std::vector<Lab>& o) {
  o.clear();
  if (l.b % 2 == 0) { o.push_back({l.a, l.b - 1}); o.push_back({l.a + 1, l.b - 1}); }
  else o.push_back({l.a, l.b - 2});
}
void lab_E(Lab l, std::vector<Lab>& o) {
  o.clear();
  if (l.b % 2 == 0) o.push_back({l.a + 1, l.b});
  else { o.push_back({l.a, l.b - 1}); o.push_back({l.a, l.b + 1}); }
}
void lab_W(Lab l, std::vector<Lab>& o) {
  o.clear();
  if (l.b % 2 == 0) o.push_back({l.a - 1, l.b});
  else { o.push_back({l.a - 1, l.b - 1}); o.push_back({l.a - 1, l.b + 1}); }
}

struct Iface {
  Lab label;
  std::vector<int> index;
  std::vector<double> px, py;
};

// One stencil side before side records are shared: its knot list (repeats
// dropped) and each knot's last written position.
struct SideWork {
  bool present = false;
  uint64_t hash = 0;  // FNV-1a of the side kind and knot list
  std::vector<int> idx;
  std::vector<double> px, py;
};

struct StencilWork {
  std::string err;
  StencilRec st;
  SideWork side[4];
  std::vector<int32_t> map_pos;
  std::vector<uint8_t> map_owner;
};

// Rectangle2D signed distance (BVPs/Domains/rectangle.hpp:7-229), distance only.
double rect_dist(const double* p, double x, double y) {
  const double c0 = 0.5 * (p[0] + p[2]), c1 = 0.5 * (p[1] + p[3]);
  const double h0 = p[2] - c0, h1 = p[3] - c1;
  const double d0 = std::fabs(x - c0), d1 = std::fabs(y - c1);
  if (d0 <= h0 && d1 <= h1) return (d0 - h0 > d1 - h1) ? d0 - h0 : d1 - h1;
  if (d0 > h0) {
    if (d1 > h1) return std::sqrt((d0 - h0) * (d0 - h0) + (d1 - h1) * (d1 - h1));
    return d0 - h0;
  }
  return d1 - h1;
}

}  // namespace

// Knot spacing of a side from its local coordinates: the smallest positive
// gap (sides of graded layouts and caller-built stencils are not uniform; a
// uniform side's gaps agree to rounding), 1 for a single knot or knots that
// all coincide.
double side_gap(const std::vector<double>& t) {
  double g = 0.0;
  for (size_t k = 1; k < t.size(); k++) {
    const double d = t[k] - t[k - 1];
    if (d > 0.0 && (g == 0.0 || d < g)) g = d;
  }
  return g > 0.0 ? g : 1.0;
}

void set_shape_bins(HostLayout& L, int bps) {
  if (bps <= 0) bps = 16;
  int64_t tab = 0;
  for (auto& sh : L.shapes) {
    const double gap = side_gap(sh.t);
    sh.delta = gap / bps;
    const int inner = (int)std::ceil((sh.hi - sh.lo) / sh.delta - 1e-9);
    sh.nbins = inner + 4;  // grid covers [lo - delta, hi + 2 delta]
    sh.tab_off = tab;
    tab += (int64_t)sh.nbins * sh.n;
  }
}

// Derived parts of a layout whose knots, stencils and sides are set:
// boundary knots (Solve_OMP_Analytic: |dist| <= 1e-8 -> B = g, no row), row
// offsets of G, side shapes (translates with equal knot spacing, size, c and
// exit extent share one) with their inverse and table offsets and bin grids.
void finish_layout(HostLayout& L, const double gparams[4], int bps) {
  L.row_ptr.assign(L.K + 1, 0);
  for (int v = 0; v < L.K; v++) {
    L.knot_boundary[v] = !(std::fabs(rect_dist(gparams, L.kx[v], L.ky[v])) > 1e-08);
    L.nboundary += L.knot_boundary[v];
    const int len = L.knot_boundary[v] ? 0 : L.stencils[L.knot_stencil[v]].row_len;
    L.row_ptr[v + 1] = L.row_ptr[v] + len;
  }
  // side shapes: translates with equal knot spacing, size, c and exit extent
  std::map<std::tuple<int, long long, long long, long long, long long>, int> shape_key;
  std::vector<std::vector<std::pair<int, int>>> uses(L.sides.size());  // (stencil, dir)
  for (size_t s = 0; s < L.stencils.size(); s++)
    for (int d = 0; d < 4; d++)
      if (L.stencils[s].side[d] >= 0) uses[L.stencils[s].side[d]].push_back({(int)s, d});
  for (size_t sd = 0; sd < L.sides.size(); sd++) {
    SideRec& sr = L.sides[sd];
    std::vector<double> t(sr.n);
    const double* crd = (sr.orient == 0) ? &L.side_px[sr.knot_off] : &L.side_py[sr.knot_off];
    for (int q = 0; q < sr.n; q++) t[q] = crd[q] - sr.origin;
    const double gap = side_gap(t);
    bool uniform = sr.n < 2 || t[1] - t[0] > 0.0;
    for (int q = 0; q < sr.n; q++)
      if (std::fabs(t[q] - q * gap) > 1e-9 * (1.0 + std::fabs(t[q]))) uniform = false;
    double lo = 1e300, hi = -1e300;
    for (auto& u : uses[sd]) {
      const StencilRec& st = L.stencils[u.first];
      const double a = (sr.orient == 0) ? st.rect[0] : st.rect[1];
      const double b = (sr.orient == 0) ? st.rect[2] : st.rect[3];
      lo = std::min(lo, a - sr.origin);
      hi = std::max(hi, b - sr.origin);
    }
    auto key = std::make_tuple(sr.n, (long long)std::llround(gap * 1e12),
                               (long long)std::llround(sr.c * 1e12),
                               (long long)std::llround(lo / gap * 1e6),
                               uniform ? (long long)std::llround(hi / gap * 1e6) : -1 - (long long)sd);
    auto it = shape_key.find(key);
    if (it == shape_key.end()) {
      ShapeRec sh;
      sh.n = sr.n;
      sh.c = sr.c;
      sh.t = t;
      sh.lo = lo;
      sh.hi = hi;
      shape_key[key] = (int)L.shapes.size();
      sr.shape = (int)L.shapes.size();
      L.shapes.push_back(sh);
    } else {
      sr.shape = it->second;
      ShapeRec& sh = L.shapes[it->second];
      sh.lo = std::min(sh.lo, lo);
      sh.hi = std::max(sh.hi, hi);
    }
  }
  int64_t ip = 0;
  for (auto& sh : L.shapes) {
    sh.ipsi_off = ip;
    ip += (int64_t)sh.n * sh.n;
  }
  set_shape_bins(L, bps);
}


std::string build_rect_layout(HostLayout& L, const double sw[2], const double ne[2], int nsub,
                              int nnode, const double fac[4], int bps, int max_threads) {
  if (nsub < 2 || nnode < 3) return "layout needs nsub >= 2 and nnode >= 3";
  if (!(ne[0] > sw[0] && ne[1] > sw[1])) return "layout needs NE > SW";
  L = HostLayout();
  for (int i = 0; i < 2; i++) { L.sw[i] = sw[i]; L.ne[i] = ne[i]; }
  for (int i = 0; i < 4; i++) L.fac[i] = fac[i];
  L.nsub = nsub;
  L.nnode = nnode;
  const int iN = nsub, nN = nnode;
  const int nif = iN * (iN - 1) * 2;
  std::vector<Iface> ifs(nif);
  std::vector<double> sx(nif), sy(nif), ex(nif), ey(nif);
  // interface end points (PDDSparseGM.cpp:363-437); P0 accumulates in y, P1 in x
  const double lx = (ne[0] - sw[0]) / (1.0 * iN), ly = (ne[1] - sw[1]) / (1.0 * iN);
  double P0[2] = {sw[0], sw[1]}, P1[2] = {sw[0], sw[1]};
  P0[0] += 0.0; P0[1] += ly;
  P1[0] += lx; P1[1] += 0.0;
  int cen = 0;
  for (int i = 0; i < iN - 1; i++) {
    for (int j = 0; j < iN; j++) {
      sx[cen] = P0[0] + lx * j; sy[cen] = P0[1] + 0.0 * j;
      ex[cen] = P0[0] + lx * (j + 1); ey[cen] = P0[1] + 0.0 * (j + 1);
      ifs[cen].label = {j, 2 * i + 1};
      cen++;
      sx[cen] = P1[0] + 0.0 * j; sy[cen] = P1[1] + ly * j;
      ex[cen] = P1[0] + 0.0 * (j + 1); ey[cen] = P1[1] + ly * (j + 1);
      ifs[cen].label = {i, 2 * j};
      cen++;
    }
    P0[0] += 0.0; P0[1] += ly;
    P1[0] += lx; P1[1] += 0.0;
  }
  // knot numbering with shared cross points (:493-543)
  std::vector<int> cross((iN - 1) * (iN - 1), 0);
  int knot = 0, cc = 0;
  for (int i = 0; i < iN - 1; i++)
    for (int j = 0; j <= 2 * iN - 2; j += 2) {
      Iface& f = ifs[lab_id(iN, {i, j})];
      f.index.push_back(knot);
      if (j != 0) cross[(j / 2 - 1) * (iN - 1) + i] = knot;
      for (int k = 0; k < nN - 1; k++) f.index.push_back(++knot);
      if (j == 2 * iN - 2) knot++;
    }
  for (int j = 1; j <= 2 * iN - 3; j += 2)
    for (int i = 0; i < iN; i++) {
      Iface& f = ifs[lab_id(iN, {i, j})];
      if (i != 0) f.index.push_back(cross[cc++]);
      else f.index.push_back(knot++);
      for (int k = 1; k < nN - 1; k++) f.index.push_back(knot++);
      if (i != iN - 1) f.index.push_back(cross[cc]);
      else f.index.push_back(knot++);
    }
  L.K = knot;
  // positions by repeated addition (:641-686)
  for (int id = 0; id < nif; id++) {
    Iface& f = ifs[id];
    const size_t n = f.index.size();
    const double den = (double)(n - 1);
    const double ix = (ex[id] - sx[id]) / den, iy = (ey[id] - sy[id]) / den;
    double vx = sx[id], vy = sy[id];
    f.px.resize(n);
    f.py.resize(n);
    for (size_t k = 0; k < n; k++) {
      f.px[k] = vx;
      f.py[k] = vy;
      vx += ix;
      vy += iy;
    }
  }
  // hand-out order and the positions sent with the knots (:705-756)
  L.kx.assign(L.K, 0.0);
  L.ky.assign(L.K, 0.0);
  for (int Iy = 0; Iy <= 2 * iN - 2; Iy++) {
    const bool vert = (Iy % 2 == 0);
    for (int Ix = 0; Ix <= (vert ? iN - 2 : iN - 1); Ix++) {
      const Iface& f = ifs[lab_id(iN, {Ix, Iy})];
      size_t b = 1, e = f.index.size();
      if (vert) { if (Iy == 0) b = 0; }
      else {
        if (Ix == 0) { b = 0; e = f.index.size() - 1; }
        else if (Ix != iN - 1) e = f.index.size() - 1;
      }
      for (size_t k = b; k < e; k++) {
        L.order.push_back(f.index[k]);
        L.kx[f.index[k]] = f.px[k];
        L.ky[f.index[k]] = f.py[k];
      }
    }
  }
  if ((int)L.order.size() != L.K) return "internal: hand-out list does not cover all knots";
  // interfaces of every knot, in interface-vector order (Get_Interfaces): one
  // for a knot inside an interface, four for a cross point; kif_n counts
  // them, the first four are kept (more is reported as an error below)
  std::vector<int> kif((size_t)L.K * 4, -1), kif_n(L.K, 0);
  for (int id = 0; id < nif; id++)
    for (int v : ifs[id].index) {
      int& n = kif_n[v];
      if (n > 0 && n <= 4 && kif[(size_t)v * 4 + n - 1] == id) continue;
      if (n < 4) kif[(size_t)v * 4 + n] = id;
      n++;
    }

  const double gparams[4] = {sw[0], sw[1], ne[0], ne[1]};
  // 1. stencil ids in knot order: knots with the same interfaces share one
  //    (one-interface knots by interface id, the others by their id list)
  std::vector<int> sid_of_if(nif, -1);
  std::map<std::vector<int>, int> multi_key;
  std::vector<int> rep;  // first knot of each stencil
  L.knot_stencil.assign(L.K, -1);
  L.knot_boundary.assign(L.K, 0);
  for (int v = 0; v < L.K; v++) {
    const int n = kif_n[v];
    int* slot;
    if (n == 1) {
      slot = &sid_of_if[kif[(size_t)v * 4]];
    } else {
      std::vector<int> key(kif.begin() + (size_t)v * 4, kif.begin() + (size_t)v * 4 + std::min(n, 4));
      if (n > 4) key.push_back(-n);
      slot = &multi_key.emplace(std::move(key), -1).first->second;
    }
    if (*slot < 0) {
      *slot = (int)rep.size();
      rep.push_back(v);
    }
    L.knot_stencil[v] = *slot;
  }
  // 2. every stencil on its own (host threads): rect, sides' knot lists with
  //    their last written positions, G row, row positions and owner flags
  const int nst = (int)rep.size();
  const double STEN_ELONG = 0.5;
  std::vector<StencilWork> work(nst);
  // per-thread scratch of build_one: knot-indexed arrays and side lists
  struct Scratch {
    std::vector<Lab> tmp, lab[4];
    std::vector<int> lastq, col_pos, sidx;
    std::vector<int64_t> last_writer;
    std::vector<double> spx, spy;
  };
  auto build_one = [&](int sid, Scratch& sc) {
    StencilWork& W = work[sid];
    const int* ki = &kif[(size_t)rep[sid] * 4];
    const int nki = kif_n[rep[sid]];
    std::vector<Lab>& tmp = sc.tmp;
    std::vector<int>& lastq = sc.lastq;
    std::vector<int>& col_pos = sc.col_pos;
    std::vector<int64_t>& last_writer = sc.last_writer;
    // Labels_Stencil
    std::vector<Lab>* lab = sc.lab;
    for (int d = 0; d < 4; d++) lab[d].clear();
    auto push_if = [&](int d, Lab l) { if (lab_id(iN, l) >= 0) lab[d].push_back(l); };
    if (nki == 1) {
      const Lab l = ifs[ki[0]].label;
      lab_N(l, tmp); for (auto& q : tmp) push_if(DIR_N, q);
      lab_S(l, tmp); for (auto& q : tmp) push_if(DIR_S, q);
      lab_E(l, tmp); for (auto& q : tmp) push_if(DIR_E, q);
      lab_W(l, tmp); for (auto& q : tmp) push_if(DIR_W, q);
    } else if (nki == 4) {
      int max_h = -1 << 30, max_v = -1 << 30;
      for (int q = 0; q < 4; q++) {
        max_h = std::max(max_h, ifs[ki[q]].label.a);
        max_v = std::max(max_v, ifs[ki[q]].label.b);
      }
      Lab ie{0, 0}, iw{0, 0}, in{0, 0}, is{0, 0};
      for (int q = 0; q < 4; q++) {
        const Lab l = ifs[ki[q]].label;
        if (l.b % 2 == 1) { if (l.a == max_h) ie = l; else iw = l; }
        else { if (l.b == max_v) in = l; else is = l; }
      }
      lab_N(iw, tmp); push_if(DIR_N, tmp[0]);
      lab_N(ie, tmp); push_if(DIR_N, tmp[0]);
      lab_S(iw, tmp); push_if(DIR_S, tmp[0]);
      lab_S(ie, tmp); push_if(DIR_S, tmp[0]);
      lab_E(is, tmp); push_if(DIR_E, tmp[0]);
      lab_E(in, tmp); push_if(DIR_E, tmp[0]);
      lab_W(is, tmp); push_if(DIR_W, tmp[0]);
      lab_W(in, tmp); push_if(DIR_W, tmp[0]);
    } else {
      W.err = "internal: knot on " + std::to_string(nki) + " interfaces";
      return;
    }
    auto IF = [&](Lab l) -> const Iface& { return ifs[lab_id(iN, l)]; };
    // Compute_Stencil
    StencilRec& st = W.st;
    for (int i = 0; i < 4; i++) st.rect[i] = gparams[i];
    if (!lab[DIR_S].empty()) st.rect[1] = IF(lab[DIR_S][0]).py[0];
    if (!lab[DIR_W].empty()) st.rect[0] = IF(lab[DIR_W][0]).px[0];
    if (!lab[DIR_N].empty()) st.rect[3] = IF(lab[DIR_N].back()).py.back();
    if (!lab[DIR_E].empty()) st.rect[2] = IF(lab[DIR_E].back()).px.back();
    std::vector<int>& sidx = sc.sidx;
    std::vector<double>& spx = sc.spx;
    std::vector<double>& spy = sc.spy;
    for (int d = 0; d < 4; d++) {
      int kind = -3;
      st.side[d] = -1;
      if (lab[d].empty()) {
        st.kind[d] = kind;
        continue;
      }
      sidx.clear();
      spx.clear();
      spy.clear();
      const bool horiz = (d == DIR_N || d == DIR_S);
      auto add = [&](const Iface& f, int from, int to) {
        for (int k = from; k < to; k++) {
          sidx.push_back(f.index[k]);
          spx.push_back(f.px[k]);
          spy.push_back(f.py[k]);
        }
      };
      Lab first = lab[d][0];
      Lab pre = horiz ? Lab{first.a - 1, first.b} : Lab{first.a, first.b - 2};
      if (lab_id(iN, pre) >= 0) {
        kind++;
        const Iface& f = IF(pre);
        add(f, (int)((1 - STEN_ELONG) * (f.index.size() - 1)), (int)f.index.size());
      }
      for (const Lab& l : lab[d]) {
        add(IF(l), 0, (int)IF(l).index.size());
        kind += 2;
      }
      Lab last = lab[d].back();
      Lab post = horiz ? Lab{last.a + 1, last.b} : Lab{last.a, last.b + 2};
      if (lab_id(iN, post) >= 0) {
        const Iface& f = IF(post);
        kind++;
        add(f, 0, (int)(STEN_ELONG * (f.index.size())));
      }
      st.kind[d] = kind;
      // Stencil::Init: keep the last written position of an index; drop
      // consecutive repeats of an index
      if (sidx.empty()) continue;
      if (kind < 0 || kind > 3) {
        W.err = "internal: stencil side kind out of range";
        return;
      }
      SideWork& S = W.side[d];
      S.present = true;
      S.idx = sidx;
      S.idx.erase(std::unique(S.idx.begin(), S.idx.end()), S.idx.end());
      for (size_t q = 0; q < sidx.size(); q++) lastq[sidx[q]] = (int)q;
      S.px.reserve(S.idx.size());
      S.py.reserve(S.idx.size());
      for (int v2 : S.idx) {
        S.px.push_back(spx[lastq[v2]]);
        S.py.push_back(spy[lastq[v2]]);
      }
      for (int v2 : sidx) lastq[v2] = -1;
      uint64_t h = 1469598103934665603ull ^ (uint64_t)kind;
      for (int v2 : S.idx) h = (h ^ (uint64_t)(uint32_t)v2) * 1099511628211ull;
      S.hash = h;
    }
    // global-boundary flags of the rect sides: midpoint within 1e-8 of the
    // domain boundary (Reduce_Analytic's test, EMFKACSolver.hpp:559)
    {
      const double mx = 0.5 * (st.rect[0] + st.rect[2]), my = 0.5 * (st.rect[1] + st.rect[3]);
      st.glob[DIR_N] = rect_dist(gparams, mx, st.rect[3]) >= -1e-08;
      st.glob[DIR_S] = rect_dist(gparams, mx, st.rect[1]) >= -1e-08;
      st.glob[DIR_E] = rect_dist(gparams, st.rect[2], my) >= -1e-08;
      st.glob[DIR_W] = rect_dist(gparams, st.rect[0], my) >= -1e-08;
    }
    // G row: sorted union of side indices
    std::vector<int>& cols = st.cols;
    for (int d = 0; d < 4; d++)
      if (W.side[d].present) cols.insert(cols.end(), W.side[d].idx.begin(), W.side[d].idx.end());
    std::sort(cols.begin(), cols.end());
    cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
    st.row_len = (int)cols.size();
    // row position of every (side, knot) entry, sides in N, S, E, W order;
    // the last side that wrote a knot owns its entry
    for (int p = 0; p < (int)cols.size(); p++) col_pos[cols[p]] = p;
    size_t nmap = 0;
    for (int d = 0; d < 4; d++)
      if (W.side[d].present) nmap += W.side[d].idx.size();
    W.map_pos.resize(nmap);
    W.map_owner.assign(nmap, 0);
    size_t m = 0;
    for (int d = 0; d < 4; d++) {
      if (!W.side[d].present) continue;
      for (int v2 : W.side[d].idx) {
        last_writer[v2] = (int64_t)m;
        W.map_pos[m++] = col_pos[v2];
      }
    }
    for (int v2 : cols) {
      W.map_owner[last_writer[v2]] = 1;
      last_writer[v2] = -1;
    }
  };
  {
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const int cap = max_threads > 0 ? max_threads : 8;  // 8 and 16 measured alike
    const int nth = std::max(1, std::min({(int)hw, cap, nst / 8}));
    std::vector<std::string> terr(nth);
    auto worker = [&](int t) {
      try {
        Scratch sc;
        sc.lastq.assign(L.K, -1);
        sc.col_pos.assign(L.K, 0);
        sc.last_writer.assign(L.K, -1);
        for (int sid = t; sid < nst; sid += nth) build_one(sid, sc);
      } catch (const std::exception& e) {
        terr[t] = std::string("layout worker: ") + e.what();
      }
    };
    std::vector<std::thread> pool;
    int t = 1;
    try {
      for (; t < nth; t++) pool.emplace_back(worker, t);
    } catch (const std::exception&) {  // no thread: the workers left run here
    }
    for (int r = t; r < nth; r++) worker(r);
    worker(0);
    for (auto& th : pool) th.join();
    for (auto& e : terr)
      if (!e.empty()) return e;
  }
  // 3. in stencil order: side records shared by equal (kind, knot list), the
  //    first stencil that meets a side giving its knot positions; records
  //    with one hash are chained (side_next) and compared in full
  size_t nside_knots = 0, nmap = 0;
  for (int sid = 0; sid < nst; sid++) {
    if (!work[sid].err.empty()) return work[sid].err;
    for (int d = 0; d < 4; d++)
      if (work[sid].side[d].present) nside_knots += work[sid].side[d].idx.size();
    nmap += work[sid].map_pos.size();
  }
  std::unordered_map<uint64_t, int> side_by_hash;
  std::vector<int> side_next;
  side_by_hash.reserve(4 * (size_t)nst);
  L.side_knot.reserve(nside_knots);
  L.side_px.reserve(nside_knots);
  L.side_py.reserve(nside_knots);
  L.map_pos.resize(nmap);
  L.map_owner.resize(nmap);
  L.stencils.reserve(nst);
  int64_t moff = 0;
  for (int sid = 0; sid < nst; sid++) {
    StencilWork& W = work[sid];
    StencilRec& st = W.st;
    for (int d = 0; d < 4; d++) {
      SideWork& S = W.side[d];
      if (!S.present) continue;
      const int kd = st.kind[d];
      const int n = (int)S.idx.size();
      auto hit = side_by_hash.find(S.hash);
      int found = -1;
      if (hit != side_by_hash.end())
        for (int c = hit->second; c >= 0; c = side_next[c]) {
          const SideRec& r = L.sides[c];
          if (r.kind == kd && r.n == n && std::equal(S.idx.begin(), S.idx.end(), L.side_knot.begin() + r.knot_off)) {
            found = c;
            break;
          }
        }
      if (found >= 0) {
        st.side[d] = found;
        continue;
      }
      SideRec sr;
      sr.n = n;
      sr.orient = (d == DIR_N || d == DIR_S) ? 0 : 1;
      sr.kind = kd;
      sr.c = fac[kd];
      sr.shape = -1;
      sr.knot_off = (int64_t)L.side_knot.size();
      L.side_knot.insert(L.side_knot.end(), S.idx.begin(), S.idx.end());
      L.side_px.insert(L.side_px.end(), S.px.begin(), S.px.end());
      L.side_py.insert(L.side_py.end(), S.py.begin(), S.py.end());
      sr.origin = (sr.orient == 0) ? L.side_px[sr.knot_off] : L.side_py[sr.knot_off];
      sr.fixed = (sr.orient == 0) ? L.side_py[sr.knot_off] : L.side_px[sr.knot_off];
      L.max_side = std::max(L.max_side, sr.n);
      const int id = (int)L.sides.size();
      st.side[d] = id;
      if (hit != side_by_hash.end()) {
        side_next.push_back(hit->second);
        hit->second = id;
      } else {
        side_next.push_back(-1);
        side_by_hash.emplace(S.hash, id);
      }
      L.sides.push_back(sr);
    }
    st.map_off = moff;
    std::copy(W.map_pos.begin(), W.map_pos.end(), L.map_pos.begin() + moff);
    std::copy(W.map_owner.begin(), W.map_owner.end(), L.map_owner.begin() + moff);
    moff += (int64_t)W.map_pos.size();
    L.stencils.push_back(std::move(st));
  }
  finish_layout(L, gparams, bps);
  return "";
}

std::string build_custom_layout(HostLayout& L, const double domain[4], int nknots, const double* x,
                                const double* y, const int32_t* knot_id, const CustomStencil* cst, int bps) {
  if (nknots < 1 || !x || !y || !cst) return "stencils need nknots >= 1 and knot positions";
  if (!(domain[2] > domain[0] && domain[3] > domain[1])) return "domain needs x1 > x0 and y1 > y0";
  L = HostLayout();
  L.custom = true;
  L.sw[0] = domain[0];
  L.sw[1] = domain[1];
  L.ne[0] = domain[2];
  L.ne[1] = domain[3];
  for (int q = 0; q < 4; q++) L.fac[q] = 0.0;
  L.K = nknots;
  L.kx.assign(x, x + nknots);
  L.ky.assign(y, y + nknots);
  L.order.resize(nknots);
  L.knot_stencil.resize(nknots);
  L.knot_boundary.assign(nknots, 0);
  for (int i = 0; i < nknots; i++) {
    L.order[i] = i;
    L.knot_stencil[i] = i;
    if (knot_id && knot_id[i] < 0) return "knot ids must be >= 0";
  }
  if (knot_id) L.knot_rng.assign(knot_id, knot_id + nknots);
  const double* gparams = domain;
  struct SideKeyHash {
    size_t operator()(const std::pair<std::vector<double>, std::vector<int>>& k) const {
      uint64_t h = 1469598103934665603ull;
      for (double v : k.first) {
        uint64_t b;
        std::memcpy(&b, &v, sizeof b);
        h = (h ^ b) * 1099511628211ull;
      }
      for (int v : k.second) h = (h ^ (uint64_t)(uint32_t)v) * 1099511628211ull;
      return (size_t)h;
    }
  };
  // identical sides (same shape c, knot list and positions) share one record
  std::unordered_map<std::pair<std::vector<double>, std::vector<int>>, int, SideKeyHash> side_key;
  std::map<int, int> lastq, last_writer;
  std::map<int, double> posx, posy;
  for (int k = 0; k < nknots; k++) {
    const CustomStencil& cs = cst[k];
    const std::string at = "stencil " + std::to_string(k) + ": ";
    if (!(cs.rect[2] > cs.rect[0] && cs.rect[3] > cs.rect[1])) return at + "rect needs x1 > x0 and y1 > y0";
    StencilRec st;
    for (int q = 0; q < 4; q++) st.rect[q] = cs.rect[q];
    std::vector<int> idx[4];
    std::vector<double> px[4], py[4];
    for (int d = 0; d < 4; d++) {
      st.side[d] = -1;
      st.kind[d] = -3;
      if (cs.n[d] < 0) return at + "negative side size";
      if (cs.n[d] == 0) continue;
      if (!cs.index[d] || !cs.x[d] || !cs.y[d]) return at + "side arrays missing";
      if (!(cs.c2[d] > 0.0)) return at + "RBF shape c2 must be positive";
      // Stencil::Init: a repeated index keeps its last position, consecutive
      // repeats are dropped
      posx.clear();
      posy.clear();
      for (int q = 0; q < cs.n[d]; q++) {
        if (cs.index[d][q] < 0) return at + "knot indices must be >= 0";
        posx[cs.index[d][q]] = cs.x[d][q];
        posy[cs.index[d][q]] = cs.y[d][q];
        idx[d].push_back(cs.index[d][q]);
      }
      idx[d].erase(std::unique(idx[d].begin(), idx[d].end()), idx[d].end());
      for (int v : idx[d]) {
        px[d].push_back(posx[v]);
        py[d].push_back(posy[v]);
      }
      // the binned exit weights of the MIXED form take the side's knots on
      // the side's line, in increasing order along it
      const bool horiz = (d == DIR_N || d == DIR_S);
      const double line = horiz ? (d == DIR_N ? cs.rect[3] : cs.rect[1]) : (d == DIR_E ? cs.rect[2] : cs.rect[0]);
      const double tol = 1e-9 * (1.0 + std::fabs(line));
      for (size_t q = 0; q < idx[d].size(); q++) {
        const double off = horiz ? py[d][q] : px[d][q];
        if (std::fabs(off - line) > tol) return at + "a side knot does not lie on its side of the rectangle";
        if (q > 0 && (horiz ? px[d][q] < px[d][q - 1] : py[d][q] < py[d][q - 1]))
          return at + "side knots must be in increasing order along the side";
      }
      if ((int)idx[d].size() > 160) return at + "stencil side larger than 160 knots";
      st.kind[d] = 0;
    }
    {
      const double mx = 0.5 * (st.rect[0] + st.rect[2]), my = 0.5 * (st.rect[1] + st.rect[3]);
      st.glob[DIR_N] = rect_dist(gparams, mx, st.rect[3]) >= -1e-08;
      st.glob[DIR_S] = rect_dist(gparams, mx, st.rect[1]) >= -1e-08;
      st.glob[DIR_E] = rect_dist(gparams, st.rect[2], my) >= -1e-08;
      st.glob[DIR_W] = rect_dist(gparams, st.rect[0], my) >= -1e-08;
    }
    std::vector<int32_t>& cols = st.cols;
    for (int d = 0; d < 4; d++) cols.insert(cols.end(), idx[d].begin(), idx[d].end());
    std::sort(cols.begin(), cols.end());
    cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
    st.row_len = (int)cols.size();
    if (!cols.empty()) L.max_col = std::max(L.max_col, cols.back());
    // row positions of the (side, knot) entries, sides N, S, E, W; the last
    // side that lists a knot owns its entry (G_return_withrep)
    st.map_off = (int64_t)L.map_pos.size();
    for (int d = 0; d < 4; d++)
      for (int v : idx[d]) {
        last_writer[v] = (int)L.map_pos.size();
        L.map_pos.push_back((int32_t)(std::lower_bound(cols.begin(), cols.end(), v) - cols.begin()));
        L.map_owner.push_back(0);
      }
    for (auto& lw : last_writer) L.map_owner[lw.second] = 1;
    last_writer.clear();
    for (int d = 0; d < 4; d++) {
      if (idx[d].empty()) continue;
      // (the positions fix the orientation: an N side of one stencil and
      // the S side of the next share their record, as built layouts do)
      std::vector<double> pk;
      pk.push_back(cs.c2[d]);
      pk.insert(pk.end(), px[d].begin(), px[d].end());
      pk.insert(pk.end(), py[d].begin(), py[d].end());
      auto key = std::make_pair(std::move(pk), idx[d]);
      auto it = side_key.find(key);
      if (it != side_key.end()) {
        st.side[d] = it->second;
        continue;
      }
      SideRec sr;
      sr.n = (int)idx[d].size();
      sr.orient = (d == DIR_N || d == DIR_S) ? 0 : 1;
      sr.kind = 0;
      sr.c = cs.c2[d];
      sr.shape = -1;
      sr.knot_off = (int64_t)L.side_knot.size();
      L.side_knot.insert(L.side_knot.end(), idx[d].begin(), idx[d].end());
      L.side_px.insert(L.side_px.end(), px[d].begin(), px[d].end());
      L.side_py.insert(L.side_py.end(), py[d].begin(), py[d].end());
      sr.origin = (sr.orient == 0) ? px[d][0] : py[d][0];
      sr.fixed = (sr.orient == 0) ? py[d][0] : px[d][0];
      L.max_side = std::max(L.max_side, sr.n);
      st.side[d] = (int)L.sides.size();
      side_key.emplace(std::move(key), (int)L.sides.size());
      L.sides.push_back(sr);
    }
    L.stencils.push_back(std::move(st));
  }
  finish_layout(L, gparams, bps);
  return "";
}

void layout_csr_cols(const HostLayout& L, int32_t* out) {
  auto rows = [&](int v0, int v1) {
    for (int v = v0; v < v1; v++) {
      const int64_t len = L.row_ptr[v + 1] - L.row_ptr[v];
      if (len == 0) continue;
      const auto& cols = L.stencils[L.knot_stencil[v]].cols;
      std::copy(cols.begin(), cols.begin() + len, out + L.row_ptr[v]);
    }
  };
  // host threads over row ranges of equal entry counts once the copy is
  // large (4.0 M entries, 16 MB on the 12x12/43 layout)
  const int64_t nnz = L.row_ptr[L.K];
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const int nth = (int)std::min<int64_t>({(int64_t)hw, 8, nnz >> 18});
  if (nth <= 1) {
    rows(0, L.K);
    return;
  }
  std::vector<int> cut(nth + 1, L.K);
  cut[0] = 0;
  for (int t = 1; t < nth; t++)
    cut[t] = (int)(std::lower_bound(L.row_ptr.begin(), L.row_ptr.end(), nnz * t / nth) - L.row_ptr.begin());
  std::vector<std::thread> pool;
  int t = 1;
  try {
    for (; t < nth; t++) pool.emplace_back(rows, cut[t], cut[t + 1]);
  } catch (const std::exception&) {  // no thread: the ranges left run here
  }
  for (int r = t; r < nth; r++) rows(cut[r], cut[r + 1]);
  rows(0, cut[1]);
  for (auto& th : pool) th.join();
}

void layout_stencil_cols(const HostLayout& L, std::vector<int64_t>& off, std::vector<int32_t>& cols) {
  off.assign(L.stencils.size() + 1, 0);
  for (size_t s = 0; s < L.stencils.size(); s++) off[s + 1] = off[s] + (int64_t)L.stencils[s].cols.size();
  cols.clear();
  cols.reserve(off.back());
  for (const auto& st : L.stencils) cols.insert(cols.end(), st.cols.begin(), st.cols.end());
}

std::string merge_layouts(HostLayout& out, const std::vector<HostLayout>& parts, int bps) {
  out = HostLayout();
  if (parts.empty()) return "a batch needs at least one instance";
  const HostLayout& p0 = parts[0];
  for (int i = 0; i < 2; i++) { out.sw[i] = p0.sw[i]; out.ne[i] = p0.ne[i]; }
  for (int i = 0; i < 4; i++) out.fac[i] = p0.fac[i];
  out.nsub = p0.nsub;
  out.nnode = p0.nnode;
  out.row_ptr.push_back(0);
  for (const HostLayout& P : parts) {
    const int k0 = out.K;
    const int s0 = (int)out.stencils.size();
    const int d0 = (int)out.sides.size();
    const int h0 = (int)out.shapes.size();
    const int64_t e0 = out.row_ptr.back();
    const int64_t sk0 = (int64_t)out.side_knot.size();
    const int64_t m0 = (int64_t)out.map_pos.size();
    if ((int64_t)out.K + P.K > (int64_t)INT32_MAX) return "batch has more than 2^31 knots";
    out.K += P.K;
    out.kx.insert(out.kx.end(), P.kx.begin(), P.kx.end());
    out.ky.insert(out.ky.end(), P.ky.begin(), P.ky.end());
    for (int v : P.order) out.order.push_back(v + k0);
    for (int v : P.knot_stencil) out.knot_stencil.push_back(v + s0);
    out.knot_boundary.insert(out.knot_boundary.end(), P.knot_boundary.begin(), P.knot_boundary.end());
    out.nboundary += P.nboundary;
    for (int v = 0; v < P.K; v++) out.row_ptr.push_back(e0 + P.row_ptr[v + 1]);
    for (StencilRec st : P.stencils) {
      for (int d = 0; d < 4; d++)
        if (st.side[d] >= 0) st.side[d] += d0;
      st.map_off += m0;
      for (int& c : st.cols) c += k0;
      out.stencils.push_back(std::move(st));
    }
    for (SideRec sr : P.sides) {
      sr.shape += h0;
      sr.knot_off += sk0;
      out.sides.push_back(sr);
    }
    for (int v : P.side_knot) out.side_knot.push_back(v + k0);
    out.side_px.insert(out.side_px.end(), P.side_px.begin(), P.side_px.end());
    out.side_py.insert(out.side_py.end(), P.side_py.begin(), P.side_py.end());
    out.map_pos.insert(out.map_pos.end(), P.map_pos.begin(), P.map_pos.end());
    out.map_owner.insert(out.map_owner.end(), P.map_owner.begin(), P.map_owner.end());
    out.shapes.insert(out.shapes.end(), P.shapes.begin(), P.shapes.end());
    out.max_side = std::max(out.max_side, P.max_side);
  }
  int64_t ip = 0;
  for (auto& sh : out.shapes) {
    sh.ipsi_off = ip;
    ip += (int64_t)sh.n * sh.n;
  }
  set_shape_bins(out, bps);
  return "";
}

}  // namespace pdds
