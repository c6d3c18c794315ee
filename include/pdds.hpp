/* pdds_gb300 -- header-only C++17 host interface over the C ABI of pdds.h.
 *
 * Mirrors the call surface of the reference's PDDSparseGM
 * (PDDAlgorithms/PDDSparseGM.hpp:103-280) for the GPU path:
 *
 *   reference                                  here
 *   PDDSparseGM(configuration file)            pdds::PDDSparseGM(SW, NE, N_subdo, N_node, fac)
 *   Solve(bvp): worker loop :795-848           Solve(problem, N, h, ...): every knot in one estimate
 *     triplets (knot, j, G), (knot, j, G_var),   G_triplets(), G_var_triplets(), B(), B_var()
 *     B, B_var = B^2 - BB per knot
 *   Compute_Solution :3168-3246                Compute_Solution(method, tol) -> u
 *   EMFKACSolver::Solve_OMP_Analytic           Solve_Knot(k, ...): one knot's G row, G_var, G_j, B, BB
 *     (Solvers/EMFKACSolver.hpp:711-729)          read from the all-knot estimate, and
 *                                              pdds::EMFKACSolver::Solve_GPU_Analytic: one knot from
 *                                              any X0 and a caller-built pdds::Stencil
 *   Stencil (Meshes/stencil.hpp:13-98)         pdds::Stencil (Init, Compute_ipsi)
 *
 * Errors are thrown as pdds::Error (status + the library's message).
 */
#ifndef PDDS_HPP
#define PDDS_HPP

#include <array>
#include <cmath>
#include <map>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "pdds.h"

namespace pdds {

class Error : public std::runtime_error {
 public:
  Error(pdds_status s, const std::string& msg) : std::runtime_error(msg), status(s) {}
  pdds_status status;
};

struct Triplets {
  std::vector<int> row, col;
  std::vector<double> val;
};

inline pdds_problem_desc problem(pdds_problem_kind kind, std::initializer_list<double> p = {}, bool use_cv = true) {
  pdds_problem_desc d{};
  d.kind = kind;
  d.use_cv = use_cv ? 1 : 0;
  int i = 0;
  for (double v : p)
    if (i < 8) d.p[i++] = v;
  return d;
}

inline pdds_estimate_desc estimate_desc(int N, double h, pdds_mode mode = PDDS_MODE_MIXED, uint64_t seed = 1234) {
  pdds_estimate_desc d{};
  d.mode = mode;
  d.npaths = N;
  d.h = h;
  d.seed = seed;
  return d;
}

class PDDSparseGM {
 public:
  // device < 0: host-only context (layout queries, no estimation)
  PDDSparseGM(std::array<double, 2> SW, std::array<double, 2> NE, int N_subdo, int N_node,
              std::array<double, 4> fac, int device = 0) {
    check(pdds_create(&ctx_, device, 0), "pdds_create");
    pdds_layout_desc d{};
    d.sw[0] = SW[0];
    d.sw[1] = SW[1];
    d.ne[0] = NE[0];
    d.ne[1] = NE[1];
    d.nsub = N_subdo;
    d.nnode = N_node;
    for (int i = 0; i < 4; i++) d.fac[i] = fac[i];
    check(pdds_layout_build(ctx_, &d, &info_), "pdds_layout_build");
    const int K = info_.nknots;
    x_.assign(K, 0.0);
    y_.assign(K, 0.0);
    order_.assign(K, 0);
    check(pdds_layout_knots(ctx_, x_.data(), y_.data(), order_.data()), "pdds_layout_knots");
    row_ptr_.assign(K + 1, 0);
    col_.assign(info_.nnz > 0 ? info_.nnz : 1, 0);
    check(pdds_layout_csr(ctx_, row_ptr_.data(), col_.data()), "pdds_layout_csr");
    col_.resize(info_.nnz);
  }
  PDDSparseGM(const PDDSparseGM&) = delete;
  PDDSparseGM& operator=(const PDDSparseGM&) = delete;
  PDDSparseGM(PDDSparseGM&& o) noexcept { *this = std::move(o); }
  PDDSparseGM& operator=(PDDSparseGM&& o) noexcept {
    std::swap(ctx_, o.ctx_);
    info_ = o.info_;
    x_ = std::move(o.x_);
    y_ = std::move(o.y_);
    order_ = std::move(o.order_);
    row_ptr_ = std::move(o.row_ptr_);
    col_ = std::move(o.col_);
    G_ = std::move(o.G_);
    Gvar_ = std::move(o.Gvar_);
    B_ = std::move(o.B_);
    BB_ = std::move(o.BB_);
    return *this;
  }
  ~PDDSparseGM() {
    if (ctx_) pdds_destroy(ctx_);
  }

  int nNodes() const { return info_.nknots; }
  const pdds_layout_info& layout() const { return info_; }
  const std::vector<double>& x() const { return x_; }
  const std::vector<double>& y() const { return y_; }
  const std::vector<int32_t>& handout_order() const { return order_; }
  const std::vector<int64_t>& row_ptr() const { return row_ptr_; }
  const std::vector<int32_t>& col() const { return col_; }

  // Estimation of every knot's G row and B entry (the worker loop of Solve).
  const pdds_estimate_info& Estimate(const pdds_problem_desc& bvp, const pdds_estimate_desc& d) {
    check(pdds_problem_set(ctx_, &bvp), "pdds_problem_set");
    const size_t nnz = col_.size() > 0 ? col_.size() : 1;
    G_.assign(nnz, 0.0);
    Gvar_.assign(nnz, 0.0);
    B_.assign(x_.size(), 0.0);
    BB_.assign(x_.size(), 0.0);
    check(pdds_estimate(ctx_, &d, G_.data(), d.want_var ? Gvar_.data() : nullptr, B_.data(), BB_.data(), &est_),
          "pdds_estimate");
    G_.resize(col_.size());
    Gvar_.resize(col_.size());
    return est_;
  }

  // (I + G) u = B for the last estimate (Compute_Solution).
  std::vector<double> Compute_Solution(pdds_solve_method method = PDDS_SOLVE_GMRES_FP32_IR, double tol = 1e-10) {
    pdds_solve_desc d{};
    d.method = method;
    d.tol = tol;
    std::vector<double> u(x_.size(), 0.0);
    check(pdds_solve_interface(ctx_, &d, u.data(), &solve_), "pdds_solve_interface");
    return u;
  }

  // Solve(bvp): estimation and interface solve.
  std::vector<double> Solve(const pdds_problem_desc& bvp, const pdds_estimate_desc& d,
                            pdds_solve_method method = PDDS_SOLVE_GMRES_FP32_IR, double tol = 1e-10) {
    Estimate(bvp, d);
    return Compute_Solution(method, tol);
  }

  // The reference's outputs of the last estimate.
  const std::vector<double>& G() const { return G_; }          // CSR values (row_ptr(), col())
  const std::vector<double>& G_var() const { return Gvar_; }
  const std::vector<double>& B() const { return B_; }
  const std::vector<double>& BB() const { return BB_; }
  std::vector<double> B_var() const {  // B^2 - BB, the sign convention of PDDSparseGM.cpp:833
    std::vector<double> v(B_.size());
    for (size_t k = 0; k < B_.size(); k++) v[k] = B_[k] * B_[k] - BB_[k];
    return v;
  }
  Triplets G_triplets() const { return triplets(G_); }
  Triplets G_var_triplets() const { return triplets(Gvar_); }

  // One knot as Solve_OMP_Analytic returns it: G, G_var, G_j, B, BB.
  void Solve_Knot(int knot, std::vector<double>& G, std::vector<double>& G_var, std::vector<int>& G_j, double& B,
                  double& BB) const {
    if (knot < 0 || knot >= (int)x_.size()) throw Error(PDDS_ERR_INVALID, "knot out of range");
    G.clear();
    G_var.clear();
    G_j.clear();
    for (int64_t e = row_ptr_[knot]; e < row_ptr_[knot + 1]; e++) {
      G.push_back(G_[e]);
      G_var.push_back(Gvar_[e]);
      G_j.push_back(col_[e]);
    }
    B = B_[knot];
    BB = BB_[knot];
  }

  const pdds_estimate_info& estimate_info() const { return est_; }
  const pdds_solve_info& solve_info() const { return solve_; }
  pdds_ctx* handle() { return ctx_; }

 private:
  void check(pdds_status s, const char* what) const {
    if (s != PDDS_OK) throw Error(s, std::string(what) + ": " + (ctx_ ? pdds_last_error(ctx_) : "no context"));
  }
  Triplets triplets(const std::vector<double>& v) const {
    Triplets t;
    for (size_t k = 0; k + 1 < row_ptr_.size(); k++)
      for (int64_t e = row_ptr_[k]; e < row_ptr_[k + 1]; e++) {
        t.row.push_back((int)k);
        t.col.push_back(col_[e]);
        t.val.push_back(v.empty() ? 0.0 : v[e]);
      }
    return t;
  }

  pdds_ctx* ctx_ = nullptr;
  pdds_layout_info info_{};
  pdds_estimate_info est_{};
  pdds_solve_info solve_{};
  std::vector<double> x_, y_;
  std::vector<int32_t> order_;
  std::vector<int64_t> row_ptr_;
  std::vector<int32_t> col_;
  std::vector<double> G_, Gvar_, B_, BB_;
};

// Side directions of a stencil, the reference's enum (Meshes/stencil.hpp:13).
enum direction { North, South, East, West };

// A knot's stencil as the reference's Stencil class receives it
// (Meshes/stencil.hpp:13-98): Init with the side knot lists, Compute_ipsi
// with the RBF shapes, the rectangle stencil_parameters and the problem's
// rectangle global_parameters.  The library factorises the RBF matrices.
class Stencil {
 public:
  double stencil_parameters[4] = {0, 0, 0, 0};
  double global_parameters[4] = {0, 0, 0, 0};

  void Init(std::map<direction, std::vector<int>> s_index, std::map<direction, std::vector<double>> s_x,
            std::map<direction, std::vector<double>> s_y, const double* parameters) {
    for (int i = 0; i < 4; i++) stencil_parameters[i] = parameters[i];
    for (int d = 0; d < 4; d++) {
      const direction dd = static_cast<direction>(d);
      index_[d] = s_index[dd];
      x_[d] = s_x[dd];
      y_[d] = s_y[dd];
      if (x_[d].size() != index_[d].size() || y_[d].size() != index_[d].size())
        throw Error(PDDS_ERR_INVALID, "Stencil::Init: index, x and y differ in length");
    }
  }
  // c2[4] in the order North, South, East, West (Stencil::Compute_ipsi)
  void Compute_ipsi(const double c2[4]) {
    for (int d = 0; d < 4; d++) c2_[d] = c2[d];
  }
  void Compute_ipsi(double c2) {
    for (int d = 0; d < 4; d++) c2_[d] = c2;
  }
  pdds_stencil_desc desc() const {
    pdds_stencil_desc s{};
    for (int i = 0; i < 4; i++) s.rect[i] = stencil_parameters[i];
    for (int d = 0; d < 4; d++) {
      s.n[d] = (int32_t)index_[d].size();
      s.index[d] = index_[d].empty() ? nullptr : index_[d].data();
      s.x[d] = x_[d].empty() ? nullptr : x_[d].data();
      s.y[d] = y_[d].empty() ? nullptr : y_[d].data();
      s.c2[d] = c2_[d];
    }
    return s;
  }
  size_t side_size(direction d) const { return index_[d].size(); }

 private:
  std::vector<int32_t> index_[4];
  std::vector<double> x_[4], y_[4];
  double c2_[4] = {1, 1, 1, 1};
};

// The reference's per-knot solver (Solvers/EMFKACSolver.hpp) on the GPU.
// Solve_GPU_Analytic has the argument list of Solve_OMP_Analytic
// (:711-729); the choices it has no argument for -- precision mode, seed,
// weight rule, replay inverses, the Philox knot word -- are the members
// `options` and `knot_id`.  rho and c2 are accepted and, as in the
// reference's G_update, unused: the side shapes come from the stencil.
class EMFKACSolver {
 public:
  explicit EMFKACSolver(int device = 0) {
    options = estimate_desc(1, 1e-3, PDDS_MODE_FP64);
    options.want_var = 1;
    const pdds_status s = pdds_create(&ctx_, device, 0);
    if (s != PDDS_OK) throw Error(s, "pdds_create");
  }
  EMFKACSolver(const EMFKACSolver&) = delete;
  EMFKACSolver& operator=(const EMFKACSolver&) = delete;
  ~EMFKACSolver() {
    if (ctx_) pdds_destroy(ctx_);
  }

  pdds_estimate_desc options;  // mode, seed, instance, dup_sum, want_var, ipsi_override, diagnostics, ...
  int32_t knot_id = 0;         // Philox knot word of the knot
  // the reduction's diagnostic sums of the last solve, slots PDDS_DIAG_*
  // (the reference's sums[] member, Solvers/EMFKACSolver.hpp:60); filled
  // when options.diagnostics is set
  double sums[PDDS_DIAG_N] = {};

  void Solve_GPU_Analytic(std::array<double, 2> X0, unsigned int N_tray, double time_discretization, double rho,
                          const pdds_problem_desc& BoundaryValueProblem, Stencil& stencil_knot, double c2,
                          std::vector<double>& G, std::vector<double>& G_var, std::vector<int>& G_j, double& B,
                          double& BB) {
    (void)rho;
    (void)c2;
    check(pdds_problem_set(ctx_, &BoundaryValueProblem), "pdds_problem_set");
    pdds_estimate_desc d = options;
    d.npaths = (int32_t)N_tray;
    d.h = time_discretization;
    const pdds_stencil_desc sd = stencil_knot.desc();
    size_t cap = 1;
    for (int q = 0; q < 4; q++) cap += stencil_knot.side_size(static_cast<direction>(q));
    std::vector<int32_t> gj(cap);
    G.assign(cap, 0.0);
    G_var.assign(cap, 0.0);
    int32_t nnz = 0;
    check(pdds_estimate_knot(ctx_, stencil_knot.global_parameters, X0[0], X0[1], knot_id, &sd, &d, gj.data(),
                             G.data(), G_var.data(), (int32_t)cap, &nnz, &B, &BB, &info_),
          "pdds_estimate_knot");
    G.resize(nnz);
    G_var.resize(nnz);
    G_j.assign(gj.begin(), gj.begin() + nnz);
    if (d.diagnostics) check(pdds_estimate_diagnostics(ctx_, sums), "pdds_estimate_diagnostics");
  }

  const pdds_estimate_info& info() const { return info_; }

 private:
  void check(pdds_status s, const char* what) const {
    if (s != PDDS_OK) throw Error(s, std::string(what) + ": " + pdds_last_error(ctx_));
  }
  pdds_ctx* ctx_ = nullptr;
  pdds_estimate_info info_{};
};

}  // namespace pdds

#endif /* PDDS_HPP */
