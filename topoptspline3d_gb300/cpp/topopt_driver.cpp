// topopt_driver -- C++ driver of the spline OC topology optimisation, the loop of
// TestSuit::testOrdinarySplineTopopt (utils/test_utils.cpp:878-970) written
// against the grid::HierarchyGrid facade of topo_grid.hpp.
//
//   topopt_driver [--case cantilever|mbb] [--nx N --ny N --nz N] [--iters K]
//                 [--mode vcycle|pcg64|mixed] [--vf 0.4] [--filter 2] [--order 3]
//                 [--lattice LX LY LZ] [--optimizer oc|mma]
//                 [--heaviside BETA] [--selfsupport] [--print-angle R]
//                 [--ss-mode M] [--drip-mode M] [--surface-lattice N]
//
// --optimizer mma runs the loop of TestSuit::testOrdinarySplineTopoptMMA
// (utils/test_utils.cpp:972-1217): MMA on the coefficients with the volume
// constraint 1e3 * (vol - vf) <= 0 and coefficient bounds [1e-3, 1].
// --heaviside projects the density (ENABLE_HEAVISIDE: beta doubled every 10
// iterations up to 32) and --selfsupport adds the self-support and drip
// constraints (ENABLE_SELFSUPPORT: scales 1e-1 / 1e2, raised to 1e0 / 1e3
// after 30 iterations and 1e1 / 1e4 after 80).
//
// Prints one line per design iteration and a JSON summary line.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "topo_grid.hpp"

namespace {

struct Args {
  std::string kase = "cantilever";
  int nx = 48, ny = 24, nz = 24, iters = 10, order = 3;
  int lattice[3] = {13, 7, 7};
  std::string mode = "mixed";
  std::string optimizer = "oc";
  double vf = 0.4, filter = 2.0;
  double heaviside = 0.0;        // initial beta (0 = no projection)
  bool selfsupport = false;
  double print_angle = 0.75;     // in units of pi
  int ss_mode = 4, drip_mode = 6, surface_lattice = 64;
};

Args parse(int argc, char** argv) {
  Args a;
  for (int i = 1; i < argc; ++i) {
    std::string s = argv[i];
    auto next = [&]() -> const char* {
      if (i + 1 >= argc) { std::fprintf(stderr, "missing value for %s\n", s.c_str()); std::exit(2); }
      return argv[++i];
    };
    if (s == "--case") a.kase = next();
    else if (s == "--nx") a.nx = std::atoi(next());
    else if (s == "--ny") a.ny = std::atoi(next());
    else if (s == "--nz") a.nz = std::atoi(next());
    else if (s == "--iters") a.iters = std::atoi(next());
    else if (s == "--mode") a.mode = next();
    else if (s == "--vf") a.vf = std::atof(next());
    else if (s == "--filter") a.filter = std::atof(next());
    else if (s == "--order") a.order = std::atoi(next());
    else if (s == "--lattice") { for (int k = 0; k < 3; ++k) a.lattice[k] = std::atoi(next()); }
    else if (s == "--optimizer") a.optimizer = next();
    else if (s == "--heaviside") a.heaviside = std::atof(next());
    else if (s == "--selfsupport") a.selfsupport = true;
    else if (s == "--print-angle") a.print_angle = std::atof(next());
    else if (s == "--ss-mode") a.ss_mode = std::atoi(next());
    else if (s == "--drip-mode") a.drip_mode = std::atoi(next());
    else if (s == "--surface-lattice") a.surface_lattice = std::atoi(next());
    else { std::fprintf(stderr, "unknown argument %s\n", s.c_str()); std::exit(2); }
  }
  if (a.optimizer != "oc" && a.optimizer != "mma") { std::fprintf(stderr, "--optimizer oc|mma\n"); std::exit(2); }
  if ((a.selfsupport || a.heaviside > 0) && a.optimizer != "mma") {
    std::fprintf(stderr, "--heaviside and --selfsupport need --optimizer mma\n");
    std::exit(2);
  }
  return a;
}

// Boundary conditions of the two benchmark cases (same as workloads.py).
void make_bc(const Args& a, std::vector<uint8_t>& fixed, std::vector<double>& loads) {
  const int vx = a.nx + 1, vy = a.ny + 1, vz = a.nz + 1;
  const int64_t nv = (int64_t)vx * vy * vz;
  fixed.assign(nv, 0);
  loads.assign(3 * nv, 0.0);
  auto vid = [&](int x, int y, int z) { return x + (int64_t)vx * (y + (int64_t)vy * z); };
  if (a.kase == "cantilever") {
    // x = 0 face fixed; unit downward force over the bottom edge of the x = nx face
    for (int z = 0; z < vz; ++z)
      for (int y = 0; y < vy; ++y) fixed[vid(0, y, z)] = 7;
    for (int y = 0; y < vy; ++y) loads[2 * nv + vid(a.nx, y, 0)] = -1.0 / vy;
  } else {
    // half-MBB: u_x = 0 on x = 0; u_y = u_z = 0 on the bottom edge at x = nx; line load at the top of x = 0
    for (int z = 0; z < vz; ++z)
      for (int y = 0; y < vy; ++y) fixed[vid(0, y, z)] |= 1;
    for (int y = 0; y < vy; ++y) fixed[vid(a.nx, y, 0)] |= 6;
    for (int y = 0; y < vy; ++y) loads[2 * nv + vid(0, y, a.nz)] = -1.0 / vy;
  }
}

}  // namespace

int main(int argc, char** argv) {
  const Args a = parse(argc, argv);
  try {
    topo_config cfg{a.nx, a.ny, a.nz, 1.0, 1e6, 0.4, 3.0, 1e-3, 400, 0};
    grid::HierarchyGrid grids(cfg);
    std::vector<uint8_t> fixed;
    std::vector<double> loads;
    make_bc(a, fixed, loads);
    grids.setBoundaryCondition(fixed, loads);
    const int part[3] = {a.lattice[0] - a.order, a.lattice[1] - a.order, a.lattice[2] - a.order};
    const double bmin[3] = {0, 0, 0}, bmax[3] = {(double)a.nx, (double)a.ny, (double)a.nz};
    grids.set_spline(a.order, part, bmin, bmax);
    grids[0]->init_coeff(a.vf);  // initCoeffs(volume_ratio), optimization/optimization.cpp:1045-1058
    grids[0]->coeff2density();

    topo_solve_opts so{};
    so.mode = a.mode == "vcycle" ? TOPO_SOLVE_VCYCLE : a.mode == "pcg64" ? TOPO_SOLVE_PCG64 : TOPO_SOLVE_MIXED;
    so.smoother = so.mode == TOPO_SOLVE_VCYCLE ? TOPO_SMOOTH_GS : TOPO_SMOOTH_CHEBYSHEV;
    so.pre = so.mode == TOPO_SOLVE_VCYCLE ? 5 : 2;
    so.post = so.pre;
    so.rtol = so.mode == TOPO_SOLVE_VCYCLE ? 1e-3 : 1e-6;
    so.max_iter = so.mode == TOPO_SOLVE_VCYCLE ? 50 : 300;
    so.inner_rtol = 0.1;
    so.inner_max = 4;
    so.cheb_degree = 2;
    so.cheb_lo = 0.3;
    so.cheb_hi = 1.1;
    if (so.mode == TOPO_SOLVE_MIXED) grid::check(grids.handle(), topo_set_operator_precision(grids.handle(), 2), "precision");

    std::vector<double> crec;
    double total_ms = 0;
    const bool use_mma = a.optimizer == "mma";
    const double vol_scale = 1e3;  // volScale, utils/test_utils.cpp:1059
    std::unique_ptr<MMA::mma_t> mma;
    double* dcoeff = nullptr;
    double* dvol = nullptr;
    const int ncon = a.selfsupport ? 3 : 1;
    double beta = a.heaviside;
    double ss_scale = 1e-1, drip_scale = 1e2;  // SSScale, dripScale (utils/test_utils.cpp:1058-1061)
    topo_support_opts sup{};
    sup.lattice = a.surface_lattice;
    sup.max_points = 200000;
    sup.print_angle = a.print_angle;
    sup.ss_mode = a.ss_mode;
    sup.drip_mode = a.drip_mode;
    if (use_mma) {
      mma.reset(new MMA::mma_t(grids, ncon));
      mma->init(1e-3, 1.0);
      dcoeff = static_cast<double*>(grids[0]->devicePtr(TOPO_COEFF));
      dvol = static_cast<double*>(grids[0]->devicePtr(TOPO_VOLCSENS));
      if (beta <= 0) grid::check(grids.handle(), topo_volume_csens(grids.handle(), 1, vol_scale, nullptr), "dvol2dcoeff");
    }
    for (int itn = 1; itn <= a.iters; ++itn) {
      const auto t0 = std::chrono::steady_clock::now();
      double vol = 0;
      if (use_mma) {
        mma->get_x(dcoeff);  // setCoeff(mma.get_x())
        grids[0]->coeff2density();
        if (beta > 0) projectDensities(grids, beta);
        vol = grids[0]->volumeRatio();
      }
      grids.update_stencil();
      topo_solve_stats st = grids.solve(so);
      const double c = grids[0]->compliance();
      topo_support_stats sst{};
      if (a.selfsupport) {
        if (itn > 80) { ss_scale = 1e1; drip_scale = 1e4; }
        else if (itn > 30) { ss_scale = 1e0; drip_scale = 1e3; }
        sup.beta = beta > 0 ? beta : 4.0;
        sst = deal_surface_points(grids, sup);
      }
      if (beta > 0) computeSensitivity2(grids, beta, a.filter, vol_scale);
      else computeSensitivity(grids, a.filter);
      if (use_mma) {
        std::vector<double> g = {vol_scale * (vol - a.vf)};
        std::vector<const double*> dg = {dvol};
        if (a.selfsupport) {
          // the constraint gradients scaled in place (scaleVector in the reference)
          double* dss = static_cast<double*>(grids[0]->devicePtr(TOPO_SSCSENS));
          double* ddr = static_cast<double*>(grids[0]->devicePtr(TOPO_DRIPCSENS));
          std::vector<double> hv(grids[0]->n_cijk());
          grid::check(grids.handle(), topo_get_array(grids.handle(), TOPO_SSCSENS, 0, hv.data(), hv.size()), "ss");
          for (double& v : hv) v *= ss_scale;
          grid::check(grids.handle(), topo_put_array(grids.handle(), TOPO_SSCSENS, 0, hv.data(), hv.size()), "ss");
          grid::check(grids.handle(), topo_get_array(grids.handle(), TOPO_DRIPCSENS, 0, hv.data(), hv.size()), "drip");
          for (double& v : hv) v *= drip_scale;
          grid::check(grids.handle(), topo_put_array(grids.handle(), TOPO_DRIPCSENS, 0, hv.data(), hv.size()), "drip");
          g.push_back(ss_scale * (sst.ss_value - 1.0));
          g.push_back(drip_scale * sst.drip_value);
          dg.push_back(dss);
          dg.push_back(ddr);
        }
        mma->update(static_cast<const double*>(grids[0]->devicePtr(TOPO_CSENS)), dg.data(), g.data());
        if (beta > 0 && itn % 10 == 0 && itn > 2 && beta < 32) beta *= 2;  // utils/test_utils.cpp:1174-1177
      } else {
        updateCoeff(grids, a.vf);
        vol = grids[0]->volumeRatio();
      }
      const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
      total_ms += ms;
      crec.push_back(c);
      std::printf("-- iter %3d  c = %.10e  v = %.6f  its = %d  r = %.2e  %.2f ms", itn, c, vol, st.iterations,
                  st.relres, ms);
      if (a.selfsupport) std::printf("  ss = %.6f  drip = %.3e  points = %d", sst.ss_value, sst.drip_value, sst.points);
      std::printf("\n");
    }
    std::printf("{\"driver\": \"topopt_driver\", \"case\": \"%s\", \"grid\": [%d, %d, %d], \"iters\": %d, "
                "\"mode\": \"%s\", \"optimizer\": \"%s\", \"ms_per_iter\": %.4f, \"compliance\": [",
                a.kase.c_str(), a.nx, a.ny, a.nz, a.iters, a.mode.c_str(), a.optimizer.c_str(),
                total_ms / a.iters);
    for (size_t k = 0; k < crec.size(); ++k) std::printf("%s%.15e", k ? ", " : "", crec[k]);
    std::printf("]}\n");
  } catch (const grid::TopoError& e) {
    std::fprintf(stderr, "topopt_driver: %s\n", e.what());
    return 1;
  }
  return 0;
}
