// CPU ORACLE -- TEST INFRASTRUCTURE ONLY.
// A plain C++17 restatement of the reference PDDSparse hot path (Feynman-Kac
// estimation of the interface system G/B and its solve).  It is the checker
// for the CUDA library: only tests/, __graft_entry__.smoke() and bench.py's
// CPU-baseline leg may load it.  Nothing in pdds_gb300/ links to it.
//
// Parity status: the reference cannot be built here (Eigen3, GSL, Boost.Random
// and MPI are absent), so this restatement is pinned against the reference's
// own recorded run (Output/Debug/cond.txt, G.csv, B.csv, G_var.csv, B_var.csv,
// Output/solution.csv of the 4x4 / 8-knot Monegros configuration), see
// tests/golden/.  Eigen's FullPivLU, BiCGSTAB and Boost's normal sampler are
// restated from their published algorithms; bit parity with those third-party
// libraries is not claimed.
#pragma once
#include <array>
#include <cstdint>
#include <map>
#include <vector>

namespace orc {

// Stencil side order of Meshes/stencil.hpp:13 (enum direction).
enum Dir { North = 0, South = 1, East = 2, West = 3 };

struct Interface {
  std::vector<int> label;                      // [i, 2j(+1)]
  std::vector<int> index;                      // knot indices
  std::vector<std::array<double, 2>> position; // knot positions
};

struct Layout {
  double SW[2], NE[2];
  int iN[2], nN[2];
  int nNodes = 0;
  std::vector<Interface> interfaces;
  std::map<std::vector<int>, int> interface_map;
  // Knots in the order the reference's server hands them to workers
  // (PDDAlgorithms/PDDSparseGM.cpp:705-756), with the position sent along.
  std::vector<int> work_index;
  std::vector<std::array<double, 2>> work_pos;
};

struct Stencil {
  double params[4];   // stencil rectangle {x0, y0, x1, y1}
  double global[4];   // domain rectangle
  int kind[4];        // per Dir
  std::vector<int> index[4];
  std::vector<std::array<double, 2>> pos[4];
};

void build_layout(Layout& L, double swx, double swy, double nex, double ney, int nsub, int nnode);
Stencil compute_stencil(const Layout& L, int knot);

}  // namespace orc
