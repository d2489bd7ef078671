/*
 * metrics.cpp -- packing fraction and mean coordination number of a bed.
 *
 * The reference computes neither; these are the quantities a packing's
 * accuracy is stated in (against an all-FP64 run).  Definitions:
 *  - probe: the cylinder coaxial with the container, radius R - 3 d_max, from
 *    3 d_max above the floor to 3 d_max below the free surface; the free
 *    surface is the 98th percentile of the sphere tops (a few particles
 *    bouncing above the bed do not move it);
 *  - packing fraction: sum of the sphere volume inside the probe / probe
 *    volume.  Each sphere is clipped exactly at the two flat ends (spherical
 *    caps) and at the curved wall by integrating the circle-circle lens area
 *    of its z-slices (16-point Gauss-Legendre per sphere);
 *  - coordination number Z: mean number of p-p contacts (centre distance below
 *    the sum of radii) of the spheres whose centres lie in the probe.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <unordered_map>
#include <vector>

#include "dem_internal.h"

namespace {

constexpr double kPiExact = 3.14159265358979323846;

/* area of the intersection of two discs (radii a, b, centre distance d) */
double lens_area(double a, double b, double d) {
  if (d >= a + b) return 0.0;
  if (d <= std::fabs(a - b)) {
    const double m = std::min(a, b);
    return kPiExact * m * m;
  }
  const double a2 = a * a, b2 = b * b;
  const double alpha = std::acos(std::clamp((d * d + a2 - b2) / (2.0 * d * a), -1.0, 1.0));
  const double beta = std::acos(std::clamp((d * d + b2 - a2) / (2.0 * d * b), -1.0, 1.0));
  return a2 * (alpha - std::sin(2.0 * alpha) / 2.0) + b2 * (beta - std::sin(2.0 * beta) / 2.0);
}

/* volume of the part of a sphere (centre height zc, axial distance rho,
 * radius r) inside the probe cylinder (radius Rp, heights [z0, z1]) */
double clipped_volume(double zc, double rho, double r, double Rp, double z0, double z1) {
  const double lo = std::max(zc - r, z0), hi = std::min(zc + r, z1);
  if (hi <= lo) return 0.0;
  if (rho + r <= Rp) {
    /* only the flat ends clip: V(z) = pi (r^2 (z - zc) - (z - zc)^3 / 3) */
    auto prim = [&](double z) {
      const double t = z - zc;
      return kPiExact * (r * r * t - t * t * t / 3.0);
    };
    return prim(hi) - prim(lo);
  }
  if (rho - r >= Rp) return 0.0;
  static const double gx[8] = {0.0950125098376374, 0.2816035507792589, 0.4580167776572274, 0.6178762444026438,
                               0.7554044083550030, 0.8656312023878318, 0.9445750230732326, 0.9894009349916499};
  static const double gw[8] = {0.1894506104550685, 0.1826034150449236, 0.1691565193950025, 0.1495959888165767,
                               0.1246289712555339, 0.0951585116824928, 0.0622535239386479, 0.0271524594117541};
  const double mid = 0.5 * (hi + lo), half = 0.5 * (hi - lo);
  double sum = 0.0;
  for (int k = 0; k < 8; k++) {
    for (int sgn = -1; sgn <= 1; sgn += 2) {
      const double z = mid + sgn * half * gx[k];
      const double s2 = r * r - (z - zc) * (z - zc);
      if (s2 <= 0.0) continue;
      sum += gw[k] * lens_area(std::sqrt(s2), Rp, rho);
    }
  }
  return sum * half;
}

}  // namespace

extern "C" dem_status dem_packing_metrics(int n, const double3* pos, const double* rad, const CylinderBC* cyl,
                                          double* phi, double* z_mean, int* n_probe) {
  if (n <= 0 || !pos || !rad || !cyl) return dem::fail(DEM_ERR_ARG, "dem_packing_metrics: bad argument");
  double dmax = 0.0;
  std::vector<double> tops((size_t)n);
  for (int i = 0; i < n; i++) {
    dmax = std::max(dmax, 2.0 * rad[i]);
    tops[(size_t)i] = pos[i].z + rad[i];
  }
  const size_t k98 = (size_t)(0.98 * (n - 1));
  std::nth_element(tops.begin(), tops.begin() + (long)k98, tops.end());
  const double surf = tops[k98];
  const double Rp = cyl->R - 3.0 * dmax;
  const double z0 = cyl->Bw + 3.0 * dmax, z1 = surf - 3.0 * dmax;
  if (Rp <= 0.0 || z1 <= z0) return dem::fail(DEM_ERR_ARG, "dem_packing_metrics: bed too small for the probe");
  /* volume */
  double vol = 0.0;
  for (int i = 0; i < n; i++) {
    const double rho = std::hypot(pos[i].x - cyl->cir.x, pos[i].y - cyl->cir.y);
    vol += clipped_volume(pos[i].z, rho, rad[i], Rp, z0, z1);
  }
  const double probe = kPiExact * Rp * Rp * (z1 - z0);
  /* contacts of the spheres centred in the probe, through a uniform grid */
  const double cell = dmax;
  auto key = [&](long long ix, long long iy, long long iz) {
    return (uint64_t)((ix + (1 << 20)) & 0x1fffff) | ((uint64_t)((iy + (1 << 20)) & 0x1fffff) << 21) |
           ((uint64_t)((iz + (1 << 20)) & 0x1fffff) << 42);
  };
  std::unordered_map<uint64_t, std::vector<int>> grid;
  grid.reserve((size_t)n);
  for (int i = 0; i < n; i++)
    grid[key((long long)std::floor(pos[i].x / cell), (long long)std::floor(pos[i].y / cell),
             (long long)std::floor(pos[i].z / cell))]
        .push_back(i);
  long long contacts = 0, inside = 0;
  for (int i = 0; i < n; i++) {
    const double rho = std::hypot(pos[i].x - cyl->cir.x, pos[i].y - cyl->cir.y);
    if (rho > Rp || pos[i].z < z0 || pos[i].z > z1) continue;
    inside++;
    const long long ix = (long long)std::floor(pos[i].x / cell), iy = (long long)std::floor(pos[i].y / cell),
                    iz = (long long)std::floor(pos[i].z / cell);
    for (long long dz = -1; dz <= 1; dz++)
      for (long long dy = -1; dy <= 1; dy++)
        for (long long dx = -1; dx <= 1; dx++) {
          auto it = grid.find(key(ix + dx, iy + dy, iz + dz));
          if (it == grid.end()) continue;
          for (int j : it->second) {
            if (j == i) continue;
            const double ex = pos[i].x - pos[j].x, ey = pos[i].y - pos[j].y, ez = pos[i].z - pos[j].z;
            const double s = rad[i] + rad[j];
            if (ex * ex + ey * ey + ez * ez < s * s) contacts++;
          }
        }
  }
  if (phi) *phi = vol / probe;
  if (z_mean) *z_mean = inside ? (double)contacts / (double)inside : 0.0;
  if (n_probe) *n_probe = (int)inside;
  return DEM_OK;
}
