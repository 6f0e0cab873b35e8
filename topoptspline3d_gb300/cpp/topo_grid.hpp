// topo_grid.hpp -- C++ facade over the C ABI of libtopo_gb300 with the names the
// reference driver uses (NanXYZH/TopOptSpline3D: grid::HierarchyGrid and
// grid::Grid in grid/Grid.h:214-1037, initTemplateMatrix in
// element/templateMatrix.h:15-21, and the free functions of
// optimization/optimization.h:41-126).  A driver written against the reference
// classes compiles against this header with the listed argument changes; every
// call forwards to one topo_* entry point and throws grid::TopoError on a
// non-OK status instead of printing and exiting.
#pragma once

#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/topo_gb300.h"

namespace grid {

struct TopoError : std::runtime_error {
  int code;
  TopoError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(topo_handle* h, int rc, const char* what) {
  if (rc != TOPO_OK) throw TopoError(rc, std::string(what) + ": " + (h ? topo_last_error(h) : "no handle"));
}

class HierarchyGrid;

// One level of the hierarchy (reference grid::Grid).  Level 0 carries the design
// field; coarse levels carry the Galerkin stencils.
class Grid {
 public:
  Grid(HierarchyGrid* owner, int layer) : owner_(owner), layer_(layer) {}
  int layer() const { return layer_; }
  // reference Grid::coeff2density (grid/Grid.cu:3361-3456)
  void coeff2density();
  // reference Grid::compliance (grid/Grid.cpp:4035-4038)
  double compliance();
  // reference Grid::volumeRatio (grid/Grid.cu:5462-5470)
  float volumeRatio();
  // reference Grid::filterSensitivity (grid/Grid.cu:4218-4246)
  void filterSensitivity(double radii);
  // reference Grid::ddensity2dcoeff_update (grid/Grid.cu:3643-3748)
  void ddensity2dcoeff_update();
  // reference Grid::update_residual / relative_residual (grid/Grid.cu:2420-2454, 2722-2727)
  void update_residual();
  double relative_residual();
  // reference Grid::gs_relax (grid/Grid.cu:1844-1887)
  void gs_relax(int n_times = 1);
  // reference Grid::reset_displacement (grid/Grid.cu:2693-2699)
  void reset_displacement();
  // reference Grid::init_coeff (grid/Grid.cu:4926-4931)
  void init_coeff(double coeff);
  // Host copies of the reference getters (getRho/getCoeff/getSens/getCSens/
  // getDisplacement/getForce return device pointers there; here: copies, or
  // the borrowed device pointer through devicePtr).
  std::vector<double> get(int which) const;
  void put(int which, const std::vector<double>& v);
  void* devicePtr(int which) const;
  int n_cijk() const;
  int n_rho() const;

 private:
  HierarchyGrid* owner_;
  int layer_;
};

// reference grid::HierarchyGrid (grid/Grid.h:782-1037)
class HierarchyGrid {
 public:
  // genFromMesh(const std::vector<unsigned>& solid_bit, int out_reso[3]) (grid/Grid.cpp:977)
  // takes a bit mask on a power-of-two cube; here a byte mask on the box nx*ny*nz.
  HierarchyGrid(const topo_config& cfg, const std::vector<uint8_t>& eactive = {}) {
    check(nullptr, topo_create(&cfg, eactive.empty() ? nullptr : eactive.data(), &h_), "topo_create");
    int n = 0;
    check(h_, topo_num_levels(h_, &n), "topo_num_levels");
    for (int l = 0; l < n; ++l) layers_.emplace_back(this, l);
  }
  ~HierarchyGrid() { topo_destroy(h_); }
  HierarchyGrid(const HierarchyGrid&) = delete;
  HierarchyGrid& operator=(const HierarchyGrid&) = delete;

  Grid* operator[](int i) { return &layers_.at(i); }
  int n_grid() const { return (int)layers_.size(); }
  topo_handle* handle() const { return h_; }

  // setBoundaryCondition + setForceSupport (optimization/optimization.cpp:1023-1028,
  // optimization/projection.cu:344-368): per-vertex fixed-DOF bits and loads [3][nv].
  void setBoundaryCondition(const std::vector<uint8_t>& fixed, const std::vector<double>& loads) {
    check(h_, topo_set_bc(h_, fixed.data(), loads.data()), "topo_set_bc");
  }
  // set_spline_partition + set_spline_knot_series (grid/Grid.cu:3134-3203, grid/Grid.cpp:3253-3377)
  void set_spline(int order, const int partition[3], const double bmin[3], const double bmax[3]) {
    check(h_, topo_set_spline(h_, order, partition, bmin, bmax), "topo_set_spline");
  }
  // reference HierarchyGrid::update_stencil (grid/Grid.cpp:4167-4178)
  void update_stencil() { check(h_, topo_update_operators(h_), "topo_update_operators"); }
  // reference HierarchyGrid::v_cycle (grid/Grid.cpp:2399-2444)
  double v_cycle(int pre_relax = 1, int post_relax = 1) {
    double rr = 0;
    check(h_, topo_vcycle(h_, pre_relax, post_relax, &rr), "topo_vcycle");
    return rr;
  }
  // the driver's solve loop (utils/test_utils.cpp:937-941) and its MG-PCG / mixed replacements
  topo_solve_stats solve(const topo_solve_opts& o) {
    topo_solve_stats s{};
    const int rc = topo_solve(h_, &o, &s);
    if (rc != TOPO_OK && rc != TOPO_E_NOT_CONVERGED) check(h_, rc, "topo_solve");
    return s;
  }

 private:
  topo_handle* h_ = nullptr;
  std::vector<Grid> layers_;
};

inline void Grid::coeff2density() { check(owner_->handle(), topo_coeff_to_density(owner_->handle()), "coeff2density"); }
inline double Grid::compliance() {
  double c = 0;
  check(owner_->handle(), topo_compliance(owner_->handle(), &c), "compliance");
  return c;
}
inline float Grid::volumeRatio() {
  double v = 0;
  check(owner_->handle(), topo_volume(owner_->handle(), 1, &v), "volumeRatio");
  return (float)v;
}
inline void Grid::filterSensitivity(double r) { check(owner_->handle(), topo_filter(owner_->handle(), r), "filterSensitivity"); }
inline void Grid::ddensity2dcoeff_update() {
  check(owner_->handle(), topo_spline_adjoint(owner_->handle()), "ddensity2dcoeff_update");
}
inline void Grid::update_residual() { check(owner_->handle(), topo_residual(owner_->handle(), layer_), "update_residual"); }
inline double Grid::relative_residual() {
  std::vector<double> r = get(TOPO_R), f = get(TOPO_F);
  double rr = 0, ff = 0;
  for (double x : r) rr += x * x;
  for (double x : f) ff += x * x;
  return ff > 0 ? std::sqrt(rr / ff) : 0.0;
}
inline void Grid::gs_relax(int n) { check(owner_->handle(), topo_smooth(owner_->handle(), layer_, n, 0), "gs_relax"); }
inline void Grid::reset_displacement() {
  std::vector<double> z(get(TOPO_U).size(), 0.0);
  put(TOPO_U, z);
}
inline void Grid::init_coeff(double c) {
  std::vector<double> v((size_t)n_cijk(), c);
  put(TOPO_COEFF, v);
}
inline std::vector<double> Grid::get(int which) const {
  size_t n = 0;
  check(owner_->handle(), topo_array_size(owner_->handle(), which, layer_, &n), "topo_array_size");
  std::vector<double> out(n);
  check(owner_->handle(), topo_get_array(owner_->handle(), which, layer_, out.data(), n), "topo_get_array");
  return out;
}
inline void Grid::put(int which, const std::vector<double>& v) {
  check(owner_->handle(), topo_put_array(owner_->handle(), which, layer_, v.data(), v.size()), "topo_put_array");
}
inline void* Grid::devicePtr(int which) const {
  void* p = nullptr;
  check(owner_->handle(), topo_device_ptr(owner_->handle(), which, layer_, &p), "topo_device_ptr");
  return p;
}
inline int Grid::n_cijk() const {
  int n = 0;
  check(owner_->handle(), topo_num_coeffs(owner_->handle(), &n), "topo_num_coeffs");
  return n;
}
inline int Grid::n_rho() const {
  size_t n = 0;
  check(owner_->handle(), topo_array_size(owner_->handle(), TOPO_RHO, 0, &n), "topo_array_size");
  return (int)n;
}

}  // namespace grid

// reference initTemplateMatrix / getTemplateMatrixElements (element/templateMatrix.h:15-21)
inline std::vector<double> initTemplateMatrix(double element_len, double ymodu, double ps_ratio) {
  std::vector<double> Ke(576);
  grid::check(nullptr, topo_element_template(ymodu, ps_ratio, element_len, Ke.data()), "topo_element_template");
  return Ke;
}

// reference computeSensitivity() (optimization/optimization.cu:185-241): element
// sensitivity, filter, and the spline adjoint.
inline void computeSensitivity(grid::HierarchyGrid& grids, double filter_radius) {
  grid::check(grids.handle(), topo_sensitivity(grids.handle()), "computeSensitivity");
  grids[0]->filterSensitivity(filter_radius);
  grids[0]->ddensity2dcoeff_update();
}

// reference projectDensities(beta) (optimization/optimization.cu:313-353).
inline void projectDensities(grid::HierarchyGrid& grids, double beta) {
  grid::check(grids.handle(), topo_heaviside_project(grids.handle(), beta), "projectDensities");
}

// reference computeSensitivity2(beta) (optimization/optimization.cu:243-311):
// sensitivity and the projected volume's gradient through the projection's
// derivative, the filter and the spline adjoint (volume gradient scaled by
// vol_scale into the VOLCSENS array).
inline void computeSensitivity2(grid::HierarchyGrid& grids, double beta, double filter_radius, double vol_scale) {
  grid::check(grids.handle(), topo_sensitivity(grids.handle()), "computeSensitivity2");
  grid::check(grids.handle(), topo_heaviside_sensitivity(grids.handle(), beta), "computeSensitivity2");
  grids[0]->filterSensitivity(filter_radius);
  grids[0]->ddensity2dcoeff_update();
  grid::check(grids.handle(), topo_heaviside_volume_csens(grids.handle(), beta, 1, filter_radius, vol_scale, nullptr),
              "computeSensitivity2");
}

// reference deal_surface_points(beta) + global_selfsupp_constraint() +
// global_drip_constraint() (optimization/optimization.cpp:1103-1127,
// grid/Grid.cu:6101-6145, 6485-6534): the constraint values; their gradients
// are left in the SSCSENS and DRIPCSENS arrays.
inline topo_support_stats deal_surface_points(grid::HierarchyGrid& grids, const topo_support_opts& o) {
  topo_support_stats st{};
  grid::check(grids.handle(), topo_support_constraints(grids.handle(), &o, &st), "deal_surface_points");
  return st;
}

// reference updateCoeff(Vgoal) (optimization/optimization.cu:589-695); returns the multiplier.
inline double updateCoeff(grid::HierarchyGrid& grids, double vgoal, double damp = 0.5, double step = 0.03,
                          double cmin = 0.0, double cmax = 1.0, bool reference_double_step = false) {
  topo_oc_opts o{vgoal, damp, step, cmin, cmax, reference_double_step ? 1 : 0, 1};
  topo_oc_stats s{};
  grid::check(grids.handle(), topo_oc_update(grids.handle(), &o, &s), "updateCoeff");
  return s.lambda;
}

namespace MMA {

// reference MMA::mma_t (optimization/mma_t.h:159-266): the optimiser lives on the
// GPU; gradients are device pointers, constraint values host scalars.
class mma_t {
 public:
  // mma_t(ndim, nConstrain): standalone, own stream on `device`
  mma_t(int ndim, int nconstrain, int device = 0) {
    const int rc = topo_mma_create(ndim, nconstrain, device, &m_);
    if (rc != TOPO_OK) throw grid::TopoError(rc, "topo_mma_create");
  }
  // over the spline coefficients of `grids`, on its stream
  mma_t(grid::HierarchyGrid& grids, int nconstrain) {
    grid::check(grids.handle(), topo_mma_create_for(grids.handle(), nconstrain, &m_), "topo_mma_create_for");
  }
  mma_t(const mma_t&) = delete;
  mma_t& operator=(const mma_t&) = delete;
  ~mma_t() { topo_mma_destroy(m_); }

  void init(double lower_bound, double upper_bound) { ck(topo_mma_init_uniform(m_, lower_bound, upper_bound)); }
  void init(const double* lower_bound, const double* upper_bound) { ck(topo_mma_init(m_, lower_bound, upper_bound)); }
  void set_constrain_amplifier(double prefer_c, double prefer_d) {
    ck(topo_mma_set_constraint_amplifier(m_, prefer_c, prefer_d));
  }
  // returns "converged" as the reference's update does (optimization/mma_t.cpp:18-51)
  bool update(const double* dev_df, const double* const* dev_dg, const double* g) {
    ck(topo_mma_update(m_, dev_df, dev_dg, g, &last_));
    return last_.converged != 0;
  }
  void get_x(double* dst_dev) { ck(topo_mma_get_x(m_, dst_dev)); }
  std::vector<double> get_x() {
    int n = 0, m = 0;
    ck(topo_mma_size(m_, &n, &m));
    std::vector<double> x(n);
    ck(topo_mma_read_x(m_, x.data()));
    return x;
  }
  const topo_mma_stats& last_stats() const { return last_; }

 private:
  void ck(int rc) {
    if (rc != TOPO_OK) throw grid::TopoError(rc, std::string("mma: ") + topo_mma_last_error(m_));
  }
  topo_mma* m_ = nullptr;
  topo_mma_stats last_{};
};

}  // namespace MMA
