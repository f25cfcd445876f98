// sep_host.h -- host-side numerics of the filter path that must match the
// reference bit for bit (compiled with -ffp-contract=off).
#pragma once

#include <cstdint>
#include <utility>
#include <vector>

namespace sep {
namespace host {

// filter/coeff.c:82-134 (samp_points_ashkenazy, imaginary range 0)
void leja_points(long nc, double* zre, double* zim);
// filter/coeff.c:16-63
void coefficients(long ms, long nc, double dE, double vmin, double dt, const double* el,
                  double* an_re, double* an_im, double* zn);

// filter/rand.c:28-66 with its statics held in an object
struct Rand {
  long idum = 0, idum2 = 123456789, iy = 0;
  long iv[32] = {};
  explicit Rand(long seed) : idum(seed) {}
  double next();
};
// filter/init.c:236-251 (normalize of norm.c:9-36 divides by the norm)
void init_psi(Rand& r, long ngrid, double dv, double* out);

// The reference's ran_nrc keeps its second stream and shuffle table in
// statics shared by the whole process (filter/rand.c:32-34); these two entry
// points reproduce that, with *idum as the caller's running seed.
double global_ran_nrc(long* idum);
void global_init_psi(long* idum, long ngrid, double dv, double* out);

// filter/init.c:124-144: per-axis tables and the cap
struct KTables {
  std::vector<double> kx, ky, kz;
  double cap = 0.0;
};
KTables k_tables(long nx, long ny, long nz, double dx, double dy, double dz, double ekinmax);
void ksqr_grid(const KTables& t, long nx, long ny, long nz, double* ksqr);

// exp(-2 pi i m / L) for m < L, as interleaved doubles (2L values)
std::vector<double> twiddles(int L);

// pseudopotFitting/pot.c:35-63 + pseudopotFitting/hamiltonian.c:91-94
void form_factor_table(const double a[4], double vol_per_atom, double* r, double* v);

// filter/init.c:157-159 grid coordinates (running sums from the minimum)
std::vector<double> axis_coords(long n, double min, double step);

// The filter's chunks of pairs (first, count): at most bc each.  With host
// buffers each chunk's output copy runs under the next chunk's filter and the
// last chunk's copy is not overlapped; small chunks filter fewer pairs per
// second, so the last chunk splits off a tail:
//  - ratio >= 0 (output copy time over filter time per pair, measured by an
//    earlier call): the smallest tail t >= 4 with ratio (c - t) <= t, at most
//    half the chunk;
//  - ratio < 0 (not measured yet): halved while it has 8 pairs or more.
std::vector<std::pair<long long, long long>> filter_chunks(long long pairs, long long bc,
                                                           bool host, double ratio);

}  // namespace host
}  // namespace sep
