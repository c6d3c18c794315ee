// Internal data model of the pdds_gb300 library (host side).
//
// HBM layout (struct-of-arrays, all device copies made once per layout):
//   knots    K      : x, y (FP64 and FP32), stencil id, boundary flag, row offset
//   stencils S      : rect {x0,y0,x1,y1} (FP64 and FP32), global-side flags,
//                     side id per direction N,S,E,W (-1 = none), row length,
//                     offset into the (side knot -> row column) map
//   sides    D      : shape id, orientation, origin (coordinate of side knot 0),
//                     knot offset into side_knot/side_px/side_py
//   shapes   P      : side knots that are translates of each other share one
//                     shape: n, c, local knot coordinates t_j, exit extent,
//                     bin grid, FP64 inverse of Psi and the FP32 table of
//                     cardinal functions H[b][i] on the bin grid.
#pragma once
#include <stdint.h>

#include <array>
#include <string>
#include <vector>

namespace pdds {

enum Dir { DIR_N = 0, DIR_S = 1, DIR_E = 2, DIR_W = 3 };

struct StencilRec {
  double rect[4];
  int32_t side[4];   // side id per Dir, -1 if the side has no knots
  int32_t kind[4];   // reference's kind per Dir (-3 .. 3)
  int32_t glob[4];   // 1 if that rect side lies on the domain boundary
  int32_t row_len;   // entries of the G row (sorted unique knot indices)
  int64_t map_off;   // offset of per-(side, knot) row positions, 4 blocks of n_side
  std::vector<int32_t> cols;  // sorted unique columns
};

struct SideRec {
  int32_t n;
  int32_t orient;    // 0: horizontal side (N/S), coordinate along = x; 1: vertical (E/W), along = y
  int32_t shape;
  int32_t kind;
  double c;          // RBF shape parameter (fac[kind])
  double origin;     // coordinate along the side of knot 0
  double fixed;      // the other coordinate (constant along the side)
  int64_t knot_off;  // into side_knot / side_px / side_py
};

struct ShapeRec {
  int32_t n;
  double c;
  double R = 0.0;         // 0: straight side (distance |t_i - t_j|); > 0: arc of radius R, t in radians
  std::vector<double> t;  // local coordinates of the knots (representative side)
  double lo, hi;          // exit extent in local coordinates (union over its sides)
  double delta;           // bin spacing
  int32_t nbins;          // grid points lo - delta + b*delta, b = 0 .. nbins-1
  int64_t tab_off;        // FP32 table offset: H[b*n + i]
  int64_t ipsi_off;       // FP64 inverse offset: ipsi[j*n + i]
};

struct HostLayout {
  // 0: rectangle split into nsub x nsub subdomains (the reference's layout);
  // 1: disk of radius `radius` split into nrings x nsectors annular sectors,
  //    stencils are polar rectangles rect = {rho0, phi0, rho1, phi1}, sides
  //    are arcs (orient 0, coordinate along = angle) and rays (orient 1,
  //    coordinate along = radius)
  int32_t geom = 0;
  double radius = 0.0;
  int32_t nrings = 0, nsectors = 0;
  double sw[2], ne[2];
  int32_t nsub = 0, nnode = 0;
  double fac[4];
  int32_t K = 0;
  std::vector<double> kx, ky;
  std::vector<int32_t> order;          // reference hand-out order
  std::vector<int32_t> knot_stencil;
  std::vector<uint8_t> knot_boundary;
  std::vector<int64_t> row_ptr;        // K+1; the columns of row k are stencils[knot_stencil[k]].cols
  std::vector<StencilRec> stencils;
  std::vector<SideRec> sides;
  std::vector<int32_t> side_knot;
  std::vector<double> side_px, side_py;
  std::vector<double> side_along;      // polar layouts: coordinate along the side (angle or radius) - origin
  std::vector<int32_t> map_pos;        // per stencil, per side, per side knot: row position
  std::vector<uint8_t> map_owner;      // 1 if this (side, knot) writes the entry (overwrite rule)
  std::vector<ShapeRec> shapes;
  int32_t max_side = 0;
  int32_t nboundary = 0;
  // layouts built from caller stencils (pdds_stencils_set): no subdomain
  // grid; knot i draws the Philox knot word knot_rng[i] (empty: i) and G's
  // columns are the caller's knot indices (max_col: the largest)
  bool custom = false;
  std::vector<int32_t> knot_rng;
  int32_t max_col = -1;
};

// Derived parts of a layout whose knots, stencils and sides are set: boundary
// knots, G row offsets, side shapes and their bin grids.
void finish_layout(HostLayout& L, const double gparams[4], int bins_per_gap);

// A caller-built stencil: rectangle, and per side N, S, E, W the knot
// indices and positions as Stencil::Init receives them, and the RBF shape.
struct CustomStencil {
  double rect[4];
  int32_t n[4];
  const int32_t* index[4];
  const double* x[4];
  const double* y[4];
  double c2[4];
};

// Layout of caller-built knots and stencils (pdds_stencils_set): knot i at
// (x[i], y[i]) with stencil st[i] and Philox knot word knot_id[i] (null: i);
// domain = {x0, y0, x1, y1}.  Empty string on success, else the error text.
std::string build_custom_layout(HostLayout& L, const double domain[4], int nknots, const double* x,
                                const double* y, const int32_t* knot_id, const CustomStencil* st,
                                int bins_per_gap);

// CSR column indices of G (nnz = row_ptr[K] values) written into out: row k
// is its stencil's sorted column list (empty for boundary knots).
void layout_csr_cols(const HostLayout& L, int32_t* out);
// Every stencil's column list, concatenated (off: stencils + 1 offsets).
void layout_stencil_cols(const HostLayout& L, std::vector<int64_t>& off, std::vector<int32_t>& cols);

// Builds the rectangular layout of PDDSparseGM (Fullfill_interfaces,
// Labels_Stencil, Compute_Stencil, Stencil::Init) and the derived tables.
// Returns an empty string on success, else the error text.
std::string build_rect_layout(HostLayout& L, const double sw[2], const double ne[2], int nsub,
                              int nnode, const double fac[4], int bins_per_gap, int max_threads = 0);

// Disk of radius R split into nrings x nsectors annular sectors (a
// CircleMesh): knots on the arcs between rings and on the rays between
// sectors, nnode knots per segment (shared end points; no knot at the
// centre), stencils = the union of the subdomains next to a knot's
// interfaces, sides elongated by half a segment as the rectangular rule
// does.  kappa[kind] scales the RBF shape to the side's knot spacing:
// c = kappa[kind] * chord between neighbouring side knots.
// ring_ratio (0 or 1: equal rings): ring i is ring_ratio^i times as wide as
// the central disk's radius.
std::string build_circle_layout(HostLayout& L, double R, int nrings, int nsectors, int nnode,
                                const double kappa[4], int bins_per_gap, double ring_ratio = 1.0);

// Block-diagonal union of independent layouts (a batch of instances): knots,
// stencils, sides and shapes of part i follow those of part i-1 with all
// indices shifted; G columns stay inside their part's knot range.
std::string merge_layouts(HostLayout& out, const std::vector<HostLayout>& parts, int bins_per_gap);

// Re-derives the shape bin grids for a new bins-per-gap value.
void set_shape_bins(HostLayout& L, int bins_per_gap);

}  // namespace pdds
