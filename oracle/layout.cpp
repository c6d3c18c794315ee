// CPU ORACLE -- TEST INFRASTRUCTURE ONLY (see oracle_internal.h).
// Interface/knot layout and per-knot stencils, restated from
//   PDDAlgorithms/PDDSparseGM.cpp:346-689  Fullfill_interfaces (INTERSECTIONS_YES)
//   PDDAlgorithms/PDDSparseGM.cpp:705-756  server loop (knot hand-out order)
//   PDDAlgorithms/PDDSparseGM.cpp:1316-1433 Get_Interfaces / Labels_Stencil
//   PDDAlgorithms/PDDSparseGM.cpp:1845-2041 Compute_Stencil (STEN_ELONG 0.5)
//   Meshes/interface.cpp:7-93              Interface::In/N/S/E/W
//   Meshes/stencil.cpp:11-85               Stencil::Init (std::unique dedup)
// Floating-point order follows the reference (positions are accumulated by
// repeated addition of the knot increment), so knot coordinates match bit for
// bit.
#include "oracle_internal.h"

#include <algorithm>
#include <cmath>

namespace orc {

namespace {

using Lab = std::vector<int>;

bool is_in(const Interface& it, int node) {  // interface.cpp:7-14
  for (int v : it.index)
    if (v == node) return true;
  return false;
}
std::vector<Lab> lab_N(const Lab& l) {  // interface.cpp:16-34
  std::vector<Lab> out;
  Lab a = l;
  if (l[1] % 2 == 0) {
    a[1]++; out.push_back(a);
    a[0]++; out.push_back(a);
  } else {
    a[1] += 2; out.push_back(a);
  }
  return out;
}
std::vector<Lab> lab_S(const Lab& l) {  // interface.cpp:35-53
  std::vector<Lab> out;
  Lab a = l;
  if (l[1] % 2 == 0) {
    a[1] -= 1; out.push_back(a);
    a[0]++; out.push_back(a);
  } else {
    a[1] -= 2; out.push_back(a);
  }
  return out;
}
std::vector<Lab> lab_E(const Lab& l) {  // interface.cpp:54-72
  std::vector<Lab> out;
  Lab a = l;
  if (l[1] % 2 == 0) {
    a[0]++; out.push_back(a);
  } else {
    a[1]--; out.push_back(a);
    a[1] += 2; out.push_back(a);
  }
  return out;
}
std::vector<Lab> lab_W(const Lab& l) {  // interface.cpp:73-93
  std::vector<Lab> out;
  Lab a = l;
  if (l[1] % 2 == 0) {
    a[0]--; out.push_back(a);
  } else {
    a[0]--; a[1]--; out.push_back(a);
    a[1] += 2; out.push_back(a);
  }
  return out;
}

}  // namespace

void build_layout(Layout& L, double swx, double swy, double nex, double ney, int nsub, int nnode) {
  L.SW[0] = swx; L.SW[1] = swy; L.NE[0] = nex; L.NE[1] = ney;
  L.iN[0] = L.iN[1] = nsub;   // the reference reads one value for both (:303-305)
  L.nN[0] = L.nN[1] = nnode;  // (:326-328)
  const int* iN = L.iN;
  const int* nN = L.nN;
  const int nif = iN[0] * (iN[1] - 1) + iN[1] * (iN[0] - 1);
  L.interfaces.assign(nif, Interface());
  L.interface_map.clear();
  std::vector<std::vector<int>> node_index(nif);
  std::vector<std::array<double, 2>> start, end;
  // long increments (:376-393): lincrement[i] has (NE-SW)/iN in component i
  double linc[2][2] = {{(L.NE[0] - L.SW[0]) / (1.0 * iN[0]), 0.0},
                       {0.0, (L.NE[1] - L.SW[1]) / (1.0 * iN[1])}};
  double P0[2] = {L.SW[0], L.SW[1]}, P1[2] = {L.SW[0], L.SW[1]};
  P0[0] += linc[1][0]; P0[1] += linc[1][1];
  P1[0] += linc[0][0]; P1[1] += linc[0][1];
  int cen = 0;
  for (int i = 0; i < iN[1] - 1; i++) {  // :409-437
    for (int j = 0; j < iN[0]; j++) {
      start.push_back({P0[0] + linc[0][0] * j, P0[1] + linc[0][1] * j});
      end.push_back({P0[0] + linc[0][0] * (j + 1), P0[1] + linc[0][1] * (j + 1)});
      L.interfaces[cen].label = {j, 2 * i + 1};
      cen++;
      start.push_back({P1[0] + linc[1][0] * j, P1[1] + linc[1][1] * j});
      end.push_back({P1[0] + linc[1][0] * (j + 1), P1[1] + linc[1][1] * (j + 1)});
      L.interfaces[cen].label = {i, 2 * j};
      cen++;
    }
    P0[0] += linc[1][0]; P0[1] += linc[1][1];
    P1[0] += linc[0][0]; P1[1] += linc[0][1];
  }
  for (int i = 0; i < nif; i++) L.interface_map[L.interfaces[i].label] = i;

  // knot numbering with shared cross points (:493-543)
  std::vector<int> cross((iN[0] - 1) * (iN[1] - 1), 0);
  unsigned cent = 0, cross_cent = 0;
  for (int i = 0; i < iN[0] - 1; i++) {
    for (int j = 0; j <= iN[1] * 2 - 2; j += 2) {
      const int index = L.interface_map.at({i, j});
      node_index[index].push_back(cent);
      if (j != 0) cross[(j / 2 - 1) * (iN[1] - 1) + i] = cent;
      for (int k = 0; k < nN[1] - 1; k++) {
        cent++;
        node_index[index].push_back(cent);
      }
      if (j == iN[1] * 2 - 2) cent++;
    }
  }
  for (int j = 1; j <= 2 * iN[1] - 3; j += 2) {
    for (int i = 0; i < iN[0]; i++) {
      const int index = L.interface_map.at({i, j});
      if (i != 0) {
        node_index[index].push_back(cross[cross_cent]);
        cross_cent++;
      } else {
        node_index[index].push_back(cent);
        cent++;
      }
      for (int k = 1; k < nN[0] - 1; k++) {
        node_index[index].push_back(cent);
        cent++;
      }
      if (i != iN[0] - 1) {
        node_index[index].push_back(cross[cross_cent]);
      } else {
        node_index[index].push_back(cent);
        cent++;
      }
    }
  }
  L.nNodes = (int)cent;
  // positions by repeated addition of the increment (:641-686)
  for (auto& it : L.interfaces) {
    const int index = L.interface_map.at(it.label);
    const size_t n = node_index[index].size();
    it.index = node_index[index];
    it.position.resize(n);
    const double den = (double)(n - 1);
    const double inc[2] = {(end[index][0] - start[index][0]) / den,
                           (end[index][1] - start[index][1]) / den};
    double v[2] = {start[index][0], start[index][1]};
    for (size_t i = 0; i < n; i++) {
      it.position[i] = {v[0], v[1]};
      v[0] += inc[0];
      v[1] += inc[1];
    }
  }
  // hand-out order of the server loop (:705-756)
  L.work_index.clear();
  L.work_pos.clear();
  for (int Iy = 0; Iy <= 2 * iN[1] - 2; Iy++) {
    if (Iy % 2 == 0) {
      for (int Ix = 0; Ix <= iN[0] - 2; Ix++) {
        const Interface& it = L.interfaces[L.interface_map.at({Ix, Iy})];
        const size_t b = (Iy == 0) ? 0 : 1;
        for (size_t k = b; k < it.index.size(); k++) {
          L.work_index.push_back(it.index[k]);
          L.work_pos.push_back(it.position[k]);
        }
      }
    } else {
      for (int Ix = 0; Ix <= iN[0] - 1; Ix++) {
        const Interface& it = L.interfaces[L.interface_map.at({Ix, Iy})];
        size_t b = 1, e = it.index.size() - 1;
        if (Ix == 0) b = 0;
        else if (Ix == iN[0] - 1) e = it.index.size();
        for (size_t k = b; k < e; k++) {
          L.work_index.push_back(it.index[k]);
          L.work_pos.push_back(it.position[k]);
        }
      }
    }
  }
}

namespace {

std::map<Dir, std::vector<Lab>> labels_stencil(const Layout& L, int index) {  // :1330-1433
  std::map<Dir, std::vector<Lab>> out;
  std::vector<Lab> ni;
  for (const auto& it : L.interfaces)  // Get_Interfaces :1316-1329
    if (is_in(it, index)) ni.push_back(it.label);
  auto exists = [&](const Lab& l) { return L.interface_map.count(l) > 0; };
  if (ni.size() == 1) {
    const Lab& l = ni[0];
    for (const auto& a : lab_N(l)) if (exists(a)) out[North].push_back(a);
    for (const auto& a : lab_S(l)) if (exists(a)) out[South].push_back(a);
    for (const auto& a : lab_E(l)) if (exists(a)) out[East].push_back(a);
    for (const auto& a : lab_W(l)) if (exists(a)) out[West].push_back(a);
  } else if (ni.size() == 4) {
    int max_h = std::max(std::max(ni[0][0], ni[1][0]), std::max(ni[2][0], ni[3][0]));
    int max_v = std::max(std::max(ni[0][1], ni[1][1]), std::max(ni[2][1], ni[3][1]));
    Lab ie, iw, in, is;
    for (int q = 0; q < 4; q++) {
      if (ni[q][1] % 2 == 1) {
        if (ni[q][0] == max_h) ie = ni[q]; else iw = ni[q];
      } else {
        if (ni[q][1] == max_v) in = ni[q]; else is = ni[q];
      }
    }
    if (exists(lab_N(iw)[0])) out[North].push_back(lab_N(iw)[0]);
    if (exists(lab_N(ie)[0])) out[North].push_back(lab_N(ie)[0]);
    if (exists(lab_S(iw)[0])) out[South].push_back(lab_S(iw)[0]);
    if (exists(lab_S(ie)[0])) out[South].push_back(lab_S(ie)[0]);
    if (exists(lab_E(is)[0])) out[East].push_back(lab_E(is)[0]);
    if (exists(lab_E(in)[0])) out[East].push_back(lab_E(in)[0]);
    if (exists(lab_W(is)[0])) out[West].push_back(lab_W(is)[0]);
    if (exists(lab_W(in)[0])) out[West].push_back(lab_W(in)[0]);
  }
  return out;
}

}  // namespace

Stencil compute_stencil(const Layout& L, int index) {  // :1845-2041
  const double STEN_ELONG = 0.5;  // PDDSparseGM.hpp:5
  auto labels = labels_stencil(L, index);
  auto IF = [&](const Lab& l) -> const Interface& { return L.interfaces[L.interface_map.at(l)]; };
  Stencil st;
  double sp[4] = {L.SW[0], L.SW[1], L.NE[0], L.NE[1]};
  if (labels[South].size() > 0) sp[1] = IF(labels[South][0]).position[0][1];
  if (labels[West].size() > 0) sp[0] = IF(labels[West][0]).position[0][0];
  if (labels[North].size() > 0) sp[3] = IF(labels[North].back()).position.back()[1];
  if (labels[East].size() > 0) sp[2] = IF(labels[East].back()).position.back()[0];
  std::map<Dir, std::vector<int>> s_index;
  std::map<Dir, std::vector<std::array<double, 2>>> s_pos;
  int kind[4] = {-3, -3, -3, -3};
  const Dir order[4] = {North, South, East, West};
  for (Dir d : order) {
    if (labels[d].empty()) continue;
    const Interface* s_inter = &IF(labels[d][0]);
    Lab aux = s_inter->label;
    // elongation before the first interface
    if (d == North || d == South) aux[0]--; else aux[1] -= 2;
    if (L.interface_map.count(aux) > 0) {
      kind[d]++;
      const Interface& a = IF(aux);
      for (int i = (int)((1 - STEN_ELONG) * (a.index.size() - 1)); i < (int)a.index.size(); i++) {
        s_index[d].push_back(a.index[i]);
        s_pos[d].push_back(a.position[i]);
      }
    }
    for (const auto& lab : labels[d]) {
      s_inter = &IF(lab);
      for (size_t j = 0; j < s_inter->index.size(); j++) {
        s_index[d].push_back(s_inter->index[j]);
        s_pos[d].push_back(s_inter->position[j]);
      }
      kind[d] += 2;
    }
    // elongation after the last interface
    aux = s_inter->label;
    if (d == North || d == South) aux[0]++; else aux[1] += 2;
    if (L.interface_map.count(aux) > 0) {
      const Interface& a = IF(aux);
      if (d != West || a.index.size() > 0) kind[d]++;
      for (int i = 0; i < (int)(STEN_ELONG * (a.index.size())); i++) {
        s_index[d].push_back(a.index[i]);
        s_pos[d].push_back(a.position[i]);
      }
    }
  }
  // Stencil::Init (stencil.cpp:11-85): the position kept for an index is the
  // last one written to the map; std::unique drops consecutive repeats only.
  for (int i = 0; i < 4; i++) st.params[i] = sp[i];
  st.global[0] = L.SW[0]; st.global[1] = L.SW[1]; st.global[2] = L.NE[0]; st.global[3] = L.NE[1];
  for (int d = 0; d < 4; d++) {
    st.kind[d] = kind[d];
    const Dir dd = (Dir)d;
    if (s_index[dd].empty()) continue;
    std::map<int, std::array<double, 2>> sten_map;
    std::vector<int> idx;
    for (size_t i = 0; i < s_index[dd].size(); i++) {
      sten_map[s_index[dd][i]] = s_pos[dd][i];
      idx.push_back(s_index[dd][i]);
    }
    idx.erase(std::unique(idx.begin(), idx.end()), idx.end());
    st.index[d] = idx;
    for (int v : idx) st.pos[d].push_back(sten_map[v]);
  }
  return st;
}

}  // namespace orc
