// sep_spinor_host.cpp -- neighbour lists of the spin-orbit operator (host).
//
// For each atom, the grid points within sqrt(rnlcut2) with r, r^2, Vso(r) =
// vso_a exp(-r^2 / 0.49) and the l = 1 harmonics, entry for entry what the
// reference's init_list computes (spinors/filterSpinors/init.c:114-181,
// compiled with -ffp-contract=off so every expression rounds as there).
// The reference visits every grid point for every atom; here each axis is
// first reduced to the coordinates whose own square is below rnlcut2.  A
// point outside that box cannot pass (the sum of the three squares is never
// below one of them), so the points and their order (x fastest) are the
// same, at natom x box cost instead of natom x N.
#include <cmath>
#include <string>
#include <vector>

#include "../../include/sep_gb300.h"

namespace sep {
void set_error(const std::string& msg);
}

namespace {
constexpr double kPie = 3.14159265358979323846;    // filterSpinors/fd.h PIE
constexpr double kTwoPi = 6.28318530717958647692;  // filterSpinors/fd.h TWOPI
constexpr double kEpsDx = 1.0e-20;                 // filterSpinors/fd.h EPSDX

int fail(const char* msg) {
  sep::set_error(msg);
  return SEP_ERR_ARG;
}

// indices j whose (v[j] - r)^2 is below rnlcut2
std::vector<long> axis_candidates(const double* v, long n, double r, double rnlcut2) {
  std::vector<long> out;
  for (long j = 0; j < n; ++j) {
    const double d = v[j] - r;
    if (d * d < rnlcut2) out.push_back(j);
  }
  return out;
}
}  // namespace

extern "C" int sep_spinor_neighbour_lists(long nx, long ny, long nz, const double* vx,
                                          const double* vy, const double* vz, long natom,
                                          const double* rxyz, const double* vso, double rnlcut2,
                                          long nnlc, sep_nlc* nlc, long* nl) {
  if (nx < 1 || ny < 1 || nz < 1 || !vx || !vy || !vz || natom < 0 || (natom && !rxyz) || !nl ||
      (nlc && (!vso || nnlc < 0)))
    return fail("sep_spinor_neighbour_lists: bad arguments");
  const double tmp1 = 0.5 * std::sqrt(3.0 / kPie);
  const double tmp2 = 0.5 * std::sqrt(3.0 / kTwoPi);
  const double tmp49 = 1.0 / 0.49;
  for (long a = 0; a < natom; ++a) {
    const double rx = rxyz[3 * a], ry = rxyz[3 * a + 1], rz = rxyz[3 * a + 2];
    const std::vector<long> cx = axis_candidates(vx, nx, rx, rnlcut2);
    const std::vector<long> cy = axis_candidates(vy, ny, ry, rnlcut2);
    const std::vector<long> cz = axis_candidates(vz, nz, rz, rnlcut2);
    long count = 0;
    for (long jz : cz) {
      const double dz = vz[jz] - rz;
      const double dzeps = dz + kEpsDx;
      for (long jy : cy) {
        const long jyz = nx * (ny * jz + jy);
        const double dy = vy[jy] - ry;
        const double dyeps = dy + kEpsDx;
        for (long jx : cx) {
          const double dx = vx[jx] - rx;
          const double dxeps = dx + kEpsDx;
          const double dr2 = dx * dx + dy * dy + dz * dz;
          if (!(dr2 < rnlcut2)) continue;
          if (nlc) {
            if (count >= nnlc) return fail("sep_spinor_neighbour_lists: nnlc is too small");
            sep_nlc& e = nlc[a * nnlc + count];
            e.jxyz = jyz + jx;
            e.Vr = vso[a] * std::exp(-tmp49 * dr2);
            e.r = std::sqrt(dr2);
            double dr_1 = 1.0 / std::sqrt(dx * dx + dy * dy + dzeps * dzeps);
            e.y10[0] = tmp1 * dzeps * dr_1;
            e.y10[1] = 0.0;
            dr_1 = 1.0 / std::sqrt(dxeps * dxeps + dy * dy + dz * dz);
            e.y11[0] = -tmp2 * dxeps * dr_1;
            e.y1_1[0] = tmp2 * dxeps * dr_1;
            dr_1 = 1.0 / std::sqrt(dx * dx + dyeps * dyeps + dz * dz);
            e.y11[1] = -tmp2 * dyeps * dr_1;
            e.y1_1[1] = -tmp2 * dyeps * dr_1;
            if (dr2 > kEpsDx) {
              e.r2_1 = dr_1 * dr_1;
              e.r2 = dr2;
            } else {
              e.r2_1 = 0.0;
              e.r2 = 1.0 / kEpsDx;
            }
            e.Vs0G1 = 0.0;
            e.Vs0G_2 = 0.0;
          }
          ++count;
        }
      }
    }
    nl[a] = count;
  }
  return SEP_OK;
}
