// C++ host usage of pdds_gb300 through include/pdds.hpp, the way a caller of
// the reference's PDDSparseGM would use it: build the layout, estimate every
// knot, read the reference-shaped outputs, solve the interface system.
//   pdds_cpp_check host   layout only (no GPU): prints K, nnz and a checksum
//   pdds_cpp_check gpu    Poisson on [-1,1]^2, 4x4 subdomains, 11 knots per
//                         segment: prints the interface RMSE
#include <cmath>
#include <cstdio>
#include <cstring>

#include "pdds.hpp"

int main(int argc, char** argv) {
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
