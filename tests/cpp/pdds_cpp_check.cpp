// C++ host usage of pdds_gb300 through include/pdds.hpp, the way a caller of
// the reference's PDDSparseGM would use it: build the layout, estimate every
// knot, read the reference-shaped outputs, solve the interface system.
//   pdds_cpp_check host   layout only (no GPU): prints K, nnz and a checksum
//   pdds_cpp_check gpu    Poisson on [-1,1]^2, 4x4 subdomains, 11 knots per
//                         segment: prints the interface RMSE
//   pdds_cpp_check knot F one knot through pdds::EMFKACSolver::Solve_GPU_Analytic
//                         in the replay mode, as the reference's worker calls
//                         Solve_OMP_Analytic: the stencil, X0, paths and RBF
//                         inverses are read from the text file F; prints B,
//                         BB and the G row as hexadecimal floats
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>

#include "pdds.hpp"

// File F: x0 y0 knot_id / domain x0 y0 x1 y1 / rect x0 y0 x1 y1 / N h seed /
// per side N, S, E, W: n c2 then n lines "index x y" / per present side its
// n x n inverse, row-major (j, i).
static int run_knot(const char* path) {
  std::ifstream f(path);
  double x0, y0, h;
  int knot_id, N;
  unsigned long long seed;
  double dom[4], rect[4];
  f >> x0 >> y0 >> knot_id;
  for (double& v : dom) f >> v;
  for (double& v : rect) f >> v;
  f >> N >> h >> seed;
  std::map<pdds::direction, std::vector<int>> idx;
  std::map<pdds::direction, std::vector<double>> sx, sy;
  double c2[4];
  std::vector<double> ipsi;
  int sizes[4];
  for (int d = 0; d < 4; d++) {
    const auto dd = static_cast<pdds::direction>(d);
    f >> sizes[d] >> c2[d];
    for (int q = 0; q < sizes[d]; q++) {
      int i;
      double x, y;
      f >> i >> x >> y;
      idx[dd].push_back(i);
      sx[dd].push_back(x);
      sy[dd].push_back(y);
    }
  }
  for (int d = 0; d < 4; d++)
    for (int q = 0; q < sizes[d] * sizes[d]; q++) {
      double v;
      f >> v;
      ipsi.push_back(v);
    }
  if (!f) {
    std::fprintf(stderr, "bad knot file\n");
    return 3;
  }
  pdds::Stencil st;
  st.Init(idx, sx, sy, rect);
  for (int i = 0; i < 4; i++) st.global_parameters[i] = dom[i];
  st.Compute_ipsi(c2);
  pdds::EMFKACSolver solver(0);
  solver.options = pdds::estimate_desc(N, h, PDDS_MODE_REPLAY_FP64, seed);
  solver.options.want_var = 1;
  solver.options.ipsi_override = ipsi.data();
  solver.options.ipsi_override_len = (int64_t)ipsi.size();
  solver.knot_id = knot_id;
  std::vector<double> G, Gv;
  std::vector<int> Gj;
  double B = 0, BB = 0;
  solver.Solve_GPU_Analytic({x0, y0}, (unsigned)N, h, 0.0, pdds::problem(PDDS_POISSON_SINCOS), st, 0.0, G, Gv, Gj, B,
                            BB);
  std::printf("B %a BB %a nnz %zu\n", B, BB, G.size());
  for (size_t e = 0; e < G.size(); e++) std::printf("%d %a %a\n", Gj[e], G[e], Gv[e]);
  return 0;
}

int main(int argc, char** argv) {
  if (argc > 2 && std::strcmp(argv[1], "knot") == 0) {
    try {
      return run_knot(argv[2]);
    } catch (const pdds::Error& e) {
      std::fprintf(stderr, "pdds error %d: %s\n", (int)e.status, e.what());
      return 2;
    }
  }
  const bool gpu = argc > 1 && std::strcmp(argv[1], "gpu") == 0;
  const double gap = 2.0 / (10 * 4);
  const double k3 = 3.164;
  try {
    pdds::PDDSparseGM pd({-1.0, -1.0}, {1.0, 1.0}, 4, 11, {4.2 * gap, 3.556 * gap, 3.36 * gap, k3 * gap},
                         gpu ? 0 : -1);
    double sum = 0.0;
    for (int k = 0; k < pd.nNodes(); k++) sum += pd.x()[k] * (k + 1) + pd.y()[k];
    std::printf("K %d nnz %lld checksum %.17g\n", pd.nNodes(), (long long)pd.layout().nnz, sum);
    if (!gpu) return 0;
    auto bvp = pdds::problem(PDDS_POISSON_SINCOS);
    auto d = pdds::estimate_desc(4000, 1e-3);
    d.adaptive_h = 1;
    d.richardson = 1;
    d.want_var = 1;
    std::vector<double> u = pd.Solve(bvp, d);
    double se = 0.0;
    for (int k = 0; k < pd.nNodes(); k++) {
      const double x = pd.x()[k], y = pd.y()[k];
      const double ex = std::sin(M_PI * x) * std::cos(M_PI * y) + x * y;
      se += (u[k] - ex) * (u[k] - ex);
    }
    // one knot the way Solve_OMP_Analytic hands it back
    std::vector<double> G, Gv;
    std::vector<int> Gj;
    double B = 0, BB = 0;
    const int knot = pd.handout_order()[pd.nNodes() / 2];
    pd.Solve_Knot(knot, G, Gv, Gj, B, BB);
    const pdds::Triplets t = pd.G_triplets();
    std::printf("rmse %.6e iterations %d row %zu triplets %zu B %.6f\n", std::sqrt(se / pd.nNodes()),
                pd.solve_info().iterations, G.size(), t.val.size(), B);
    return 0;
  } catch (const pdds::Error& e) {
    std::fprintf(stderr, "pdds error %d: %s\n", (int)e.status, e.what());
    return 2;
  }
}
