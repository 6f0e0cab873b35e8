// Boundary conditions from region predicates: the reference's JSON "fixedarea",
// "loadarea" and "force" sections (config_parser.cpp:389-455) evaluated on the
// surface vertices of the active domain (grid/Grid.cpp:2660-2726).
//
// Region semantics follow boundary/BoundaryCondition.h:
//   sphere     |p - c|^2 < r^2, or within 1e-8 of the sphere when closed   (:38-59, :401-425)
//   box        strictly inside the axis box spanned by corners p and q, or on
//              its boundary when closed                                     (:94-131, :428-461)
//   halfspace  positive side of the plane through p1, p2, p3 (normal
//              (p2-p1) x (p3-p1)), or on it when closed                    (:62-91, :464-505)
//   cylinder   0 <= (p - b).z <= |h| and distance to the axis < r; closed
//              and complement are ignored, as in the reference              (:147-173, :509-529)
// complement negates the predicate; a region list is a union (:176-210, :535-550).
// Force fields (:555-700): value = norm(p) * dir(p) where the region contains p,
// summed over fields; directions are normalised.
// A surface vertex inside the fixed union has all three DOFs fixed and gets no
// load; otherwise, inside the load union, it gets the summed field value as its
// nodal force (grid/Grid.cpp:2689-2721).  Surface vertices are those whose eight
// incident elements have, along some axis, no pair of active neighbours
// (mark_surface_nodes_kernel, grid/Grid.cu:2781-2815).
#include <cmath>
#include <cstdint>
#include <vector>

#include "topo_gb300.h"

namespace topo {

namespace {

bool region_contains(const topo_region& g, const double p[3]) {
  bool in = false;
  switch (g.type) {
    case TOPO_REGION_SPHERE: {
      double d2 = 0;
      for (int k = 0; k < 3; ++k) d2 += (p[k] - g.a[k]) * (p[k] - g.a[k]);
      const double r2 = g.r * g.r;
      in = d2 < r2 || (g.closed && (d2 - r2) < 1e-8);
      break;
    }
    case TOPO_REGION_BOX: {
      bool strict = true, closed_in = true;
      for (int k = 0; k < 3; ++k) {
        const double lo = std::fmin(g.a[k], g.b[k]), hi = std::fmax(g.a[k], g.b[k]);
        strict = strict && lo < p[k] && p[k] < hi;
        closed_in = closed_in && lo <= p[k] && p[k] <= hi;
      }
      in = strict || (g.closed && closed_in);
      break;
    }
    case TOPO_REGION_HALFSPACE: {
      double u[3], v[3], n[3];
      for (int k = 0; k < 3; ++k) { u[k] = g.b[k] - g.a[k]; v[k] = g.c[k] - g.a[k]; }
      n[0] = u[1] * v[2] - u[2] * v[1];
      n[1] = u[2] * v[0] - u[0] * v[2];
      n[2] = u[0] * v[1] - u[1] * v[0];
      const double s = n[0] * (p[0] - g.a[0]) + n[1] * (p[1] - g.a[1]) + n[2] * (p[2] - g.a[2]);
      in = s > 0 || (g.closed && s == 0);
      break;
    }
    case TOPO_REGION_CYLINDER: {
      const double hl = std::sqrt(g.b[0] * g.b[0] + g.b[1] * g.b[1] + g.b[2] * g.b[2]);
      if (!(hl > 0)) return false;
      double z[3], w[3];
      for (int k = 0; k < 3; ++k) { z[k] = g.b[k] / hl; w[k] = p[k] - g.a[k]; }
      const double proj = w[0] * z[0] + w[1] * z[1] + w[2] * z[2];
      if (proj > hl || proj < 0) return false;
      const double cx = w[1] * z[2] - w[2] * z[1], cy = w[2] * z[0] - w[0] * z[2], cz = w[0] * z[1] - w[1] * z[0];
      return std::sqrt(cx * cx + cy * cy + cz * cz) < g.r;
    }
    default: return false;
  }
  return g.complement ? !in : in;
}

bool union_contains(const topo_region* r, int n, const double p[3]) {
  for (int i = 0; i < n; ++i)
    if (region_contains(r[i], p)) return true;
  return false;
}

void normalise(double v[3]) {
  const double n = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  if (n > 0) for (int k = 0; k < 3; ++k) v[k] /= n;
}

// radial_normGen_t: amplifier * exp(-|c - p|^(2 damp))
double radial_norm(const double c[3], double amp, double damp, const double p[3]) {
  double d2 = 0;
  for (int k = 0; k < 3; ++k) d2 += (c[k] - p[k]) * (c[k] - p[k]);
  return amp * std::exp(-std::pow(std::sqrt(d2), damp * 2));
}

void field_value(const topo_force_field& f, const double p[3], double out[3]) {
  double dir[3] = {0, 0, 0}, nrm = 0;
  switch (f.type) {
    case TOPO_FIELD_CONST:
      for (int k = 0; k < 3; ++k) dir[k] = f.direction[k];
      normalise(dir);
      nrm = f.norm;
      break;
    case TOPO_FIELD_RADIAL_NORM_CONST_DIR:
      for (int k = 0; k < 3; ++k) dir[k] = f.direction[k];
      normalise(dir);
      nrm = radial_norm(f.center, f.amplifier, f.damp_ratio, p);
      break;
    case TOPO_FIELD_CONST_NORM_RADIAL_DIR:
      for (int k = 0; k < 3; ++k) dir[k] = f.center[k] - p[k];
      normalise(dir);
      nrm = f.norm;
      break;
    case TOPO_FIELD_RADIAL_NORM_RADIAL_DIR:
      for (int k = 0; k < 3; ++k) dir[k] = f.center2[k] - p[k];
      normalise(dir);
      nrm = radial_norm(f.center, f.amplifier, f.damp_ratio, p);
      break;
    case TOPO_FIELD_TWIST: {
      // axis from center (start) to center2 (end)
      double ax[3], w[3];
      for (int k = 0; k < 3; ++k) { ax[k] = f.center2[k] - f.center[k]; w[k] = p[k] - f.center[k]; }
      dir[0] = w[1] * ax[2] - w[2] * ax[1];
      dir[1] = w[2] * ax[0] - w[0] * ax[2];
      dir[2] = w[0] * ax[1] - w[1] * ax[0];
      double axn[3] = {ax[0], ax[1], ax[2]};
      normalise(axn);
      const double cx = w[1] * axn[2] - w[2] * axn[1], cy = w[2] * axn[0] - w[0] * axn[2],
                   cz = w[0] * axn[1] - w[1] * axn[0];
      nrm = std::sqrt(cx * cx + cy * cy + cz * cz) * f.amplifier;
      normalise(dir);
      break;
    }
    default: break;
  }
  for (int k = 0; k < 3; ++k) out[k] = nrm * dir[k];
}

}  // namespace

// fixed[nv] (bits 0-2) and loads[3][nv] for the active vertices of an nx*ny*nz
// element box; returns the support and load vertex counts.
int bc_from_regions(int nx, int ny, int nz, const uint8_t* eactive, const topo_bc_regions* s, uint8_t* fixed,
                    double* loads, int* nfixed, int* nloaded) {
  const int vx = nx + 1, vy = ny + 1, vz = nz + 1;
  const int64_t nv = (int64_t)vx * vy * vz;
  auto solid = [&](int ex, int ey, int ez) -> bool {
    if (ex < 0 || ey < 0 || ez < 0 || ex >= nx || ey >= ny || ez >= nz) return false;
    return eactive ? eactive[ex + (int64_t)nx * (ey + (int64_t)ny * ez)] != 0 : true;
  };
  int nf = 0, nl = 0;
  for (int64_t v = 0; v < nv; ++v) {
    fixed[v] = 0;
    loads[v] = loads[nv + v] = loads[2 * nv + v] = 0.0;
  }
  for (int z = 0; z < vz; ++z)
    for (int y = 0; y < vy; ++y)
      for (int x = 0; x < vx; ++x) {
        bool sf[2][2][2], any = false;
        for (int k = 0; k < 8; ++k) {
          const int i = k & 1, j = (k >> 1) & 1, l = k >> 2;
          sf[i][j][l] = solid(x - 1 + i, y - 1 + j, z - 1 + l);
          any = any || sf[i][j][l];
        }
        if (!any) continue;  // not a vertex of the active domain
        bool ax[3] = {false, false, false};
        for (int i = 0; i < 2; ++i)
          for (int j = 0; j < 2; ++j) {
            ax[0] = ax[0] || (sf[0][i][j] && sf[1][i][j]);
            ax[1] = ax[1] || (sf[i][0][j] && sf[i][1][j]);
            ax[2] = ax[2] || (sf[i][j][0] && sf[i][j][1]);
          }
        if (ax[0] && ax[1] && ax[2]) continue;  // interior vertex
        const double p[3] = {s->origin[0] + x * s->spacing, s->origin[1] + y * s->spacing,
                             s->origin[2] + z * s->spacing};
        const int64_t v = x + (int64_t)vx * (y + (int64_t)vy * z);
        if (union_contains(s->fixed, s->nfixed, p)) {
          fixed[v] = 7;
          ++nf;
          continue;
        }
        if (union_contains(s->load, s->nload, p)) {
          double f[3] = {0, 0, 0};
          for (int i = 0; i < s->nforce; ++i) {
            if (!region_contains(s->force[i].region, p)) continue;
            double fi[3];
            field_value(s->force[i], p, fi);
            for (int k = 0; k < 3; ++k) f[k] += fi[k];
          }
          for (int k = 0; k < 3; ++k) loads[k * nv + v] = f[k];
          ++nl;
        }
      }
  if (nfixed) *nfixed = nf;
  if (nloaded) *nloaded = nl;
  return TOPO_OK;
}

}  // namespace topo
