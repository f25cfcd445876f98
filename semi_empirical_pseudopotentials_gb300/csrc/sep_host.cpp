// sep_host.cpp -- host numerics that must reproduce the reference exactly.
// Build with -ffp-contract=off: every expression keeps the reference's order
// of operations so the results are identical on any IEEE-754 host.
#include "sep_host.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

namespace sep {
namespace host {

namespace {
constexpr double kPi = 3.14159265358979323846;     // filter/fd.h PIE
constexpr double kTwoPi = 6.28318530717958647692;  // filter/fd.h TWOPI

// sqrt(dt/pi) exp(-x^2 dt), filter/coeff.c:11
inline double gaussian(double x, double dt) { return std::sqrt(dt / kPi) * std::exp(-(x * x) * dt); }
}  // namespace

namespace {

// threads for the host numerics: the hardware threads, at most 16
int host_threads() {
  const unsigned h = std::thread::hardware_concurrency();
  return (int)std::max(1u, std::min(16u, h));
}

// a reusable barrier for a fixed team of threads (spins with yields)
class SpinBarrier {
 public:
  explicit SpinBarrier(int n) : n_(n) {}
  void wait() {
    const int g = gen_.load(std::memory_order_acquire);
    if (count_.fetch_add(1, std::memory_order_acq_rel) == n_ - 1) {
      count_.store(0, std::memory_order_relaxed);
      gen_.fetch_add(1, std::memory_order_release);
    } else {
      while (gen_.load(std::memory_order_acquire) == g) std::this_thread::yield();
    }
  }

 private:
  int n_;
  std::atomic<int> count_{0}, gen_{0};
};

// runs f(t) for t in [0, n) on n threads (the caller runs t = 0)
template <typename F> void run_team(int n, F&& f) {
  std::vector<std::thread> team;
  for (int t = 1; t < n; ++t) team.emplace_back(f, t);
  f(0);
  for (auto& th : team) th.join();
}

// The Leja points of filter/coeff.c:83-134 (samp_points_ashkenazy).  The
// candidates are split over a team of threads: each updates its share of the
// log-distance sums and finds its first maximum, and the team takes the
// maximum of those in thread order, which is the first maximum overall: the
// same points as one sequential scan.
void leja_compute(long nc, double* zre, double* zim) {
  // 32 nc candidates: 7/8 evenly spaced on [-2, 2], 1/8 at the origin (the
  // reference spreads them over an imaginary interval of zero width).
  const long total = 32 * nc;
  const long at_origin = total / 8;
  const double lo = -2.0, hi = 2.0;
  const double im_lo = 0.0 * lo, im_hi = 0.0 * hi;
  const double step = (hi - lo) / (double)(total - 1 - at_origin);
  const double im_step = (im_hi - im_lo) / (double)(at_origin - 1);
  std::vector<double> re(total, 0.0), im(total, 0.0), logsum(total, 0.0);
  for (long k = 0; k < total - at_origin; ++k) re[k] = lo + (double)k * step;
  for (long k = total - at_origin; k < total; ++k)
    im[k] = im_lo + (double)(k - total + at_origin) * im_step;
  zre[0] = re[0];
  zim[0] = im[0];
  const int T = (int)std::max<long>(1, std::min<long>(host_threads(), total / 4096));
  std::vector<double> best_v(T);
  std::vector<long> best_k(T);
  SpinBarrier bar(T);
  run_team(T, [&](int t) {
    const long k0 = total * t / T, k1 = total * (t + 1) / T;
    auto update = [&](double pr, double pi, bool first) {
      for (long k = k0; k < k1; ++k) {
        const double a = re[k] - pr, b = im[k] - pi;
        const double d2 = a * a + b * b;
        if (d2 < 1.0e-10) logsum[k] = -1.0e30;
        else logsum[k] = first ? std::log(d2) : logsum[k] + std::log(d2);
      }
    };
    update(re[0], im[0], true);
    for (long j = 1; j < nc; ++j) {
      long arg = k0;
      double best = -2.0e30;
      for (long k = k0; k < k1; ++k)
        if (logsum[k] > best) {
          best = logsum[k];
          arg = k;
        }
      best_v[t] = best;
      best_k[t] = arg;
      bar.wait();
      long g = best_k[0];
      double gb = best_v[0];
      for (int u = 1; u < T; ++u)
        if (best_v[u] > gb) {
          gb = best_v[u];
          g = best_k[u];
        }
      if (gb <= -2.0e30) g = 0;  // no candidate above the floor: the scan's initial index
      if (t == 0) {
        zre[j] = re[g];
        zim[j] = im[g];
      }
      bar.wait();  // the team has read best_v before the next round writes it
      update(re[g], im[g], false);
    }
  });
}
}  // namespace

void leja_points(long nc, double* zre, double* zim) {
  // they depend on nc only: computed once per nc and process
  static std::mutex mu;
  static std::map<long, std::vector<double>> cache;
  std::lock_guard<std::mutex> lock(mu);
  auto it = cache.find(nc);
  if (it == cache.end()) {
    std::vector<double> z(2 * (size_t)nc);
    leja_compute(nc, z.data(), z.data() + nc);
    it = cache.emplace(nc, std::move(z)).first;
  }
  std::memcpy(zre, it->second.data(), sizeof(double) * nc);
  std::memcpy(zim, it->second.data() + nc, sizeof(double) * nc);
}

void coefficients(long ms, long nc, double dE, double vmin, double dt, const double* el,
                  double* an_re, double* an_im, double* zn) {
  std::vector<double> zi(nc);
  leja_points(nc, zn, zi.data());
  const double scale = (2.0 - (-2.0)) / dE;
  auto energy_of = [&](long j) { return (zn[j] + 2.0) / scale + vmin; };
  // the targets are independent: one thread per target (up to the team size)
  const int T = (int)std::max<long>(1, std::min<long>(host_threads(), ms));
  run_team(T, [&](int t) {
  for (long e = t; e < ms; e += T) {
    double* cr = an_re + e * nc;
    double* ci = an_im + e * nc;
    cr[0] = gaussian(energy_of(0) - el[e], dt);
    ci[0] = 0.0;
    if (nc < 2) continue;
    cr[1] = (gaussian(energy_of(1) - el[e], dt) - cr[0]) / (zn[1] - zn[0]);
    ci[1] = (-ci[0]) / (zn[1] - zn[0]);
    for (long j = 2; j < nc; ++j) {
      // Newton divided differences: the basis polynomial at z_j is the
      // running product of (z_j - z_{i-1})
      double w = 1.0, sr = 0.0, si = 0.0;
      for (long i = 1; i < j; ++i) {
        w *= (zn[j] - zn[i - 1]);
        sr += cr[i] * w;
        si += ci[i] * w;
      }
      w *= (zn[j] - zn[j - 1]);
      cr[j] = (gaussian(energy_of(j) - el[e], dt) - cr[0] - sr) / w;
      ci[j] = (-ci[0] - si) / w;
    }
  }
  });
}

// L'Ecuyer's two multiplicative congruential streams, combined through a
// 32-entry Bays-Durham table (the published ran2 scheme of Numerical Recipes).
double Rand::next() {
  constexpr long m1 = 2147483563, m2 = 2147483399;
  constexpr long a1 = 40014, a2 = 40692, q1 = 53668, q2 = 52774, r1 = 12211, r2 = 3791;
  constexpr long ntab = 32, ndiv = 1 + (m1 - 1) / ntab;
  auto step = [](long v, long a, long q, long r, long m) {
    const long k = v / q;
    v = a * (v - k * q) - k * r;  // a v mod m without overflow (Schrage)
    return v < 0 ? v + m : v;
  };
  if (idum <= 0) {
    idum = (-idum < 1) ? 1 : -idum;
    idum2 = idum;
    for (long j = ntab + 7; j >= 0; --j) {
      idum = step(idum, a1, q1, r1, m1);
      if (j < ntab) iv[j] = idum;
    }
    iy = iv[0];
  }
  idum = step(idum, a1, q1, r1, m1);
  idum2 = step(idum2, a2, q2, r2, m2);
  const long j = iy / ndiv;
  iy = iv[j] - idum2;
  iv[j] = idum;
  if (iy < 1) iy += m1 - 1;
  const double t = (1.0 / (double)m1) * (double)iy;
  const double top = 1.0 - 1.2e-7;
  return t > top ? top : t;
}

namespace {
Rand& global_rand() {
  static Rand r(0);
  return r;
}
}  // namespace

double global_ran_nrc(long* idum) {
  Rand& r = global_rand();
  r.idum = *idum;
  const double v = r.next();
  *idum = r.idum;
  return v;
}

void global_init_psi(long* idum, long ngrid, double dv, double* out) {
  // init_psi copies *idum into a local, draws, and writes it back (init.c:239-249)
  Rand& r = global_rand();
  r.idum = *idum;
  init_psi(r, ngrid, dv, out);
  *idum = r.idum;
}

void init_psi(Rand& r, long ngrid, double dv, double* out) {
  for (long g = 0; g < ngrid; ++g) out[g] = -1.0 + 2.0 * r.next();
  double s = 0.0;
  for (long g = 0; g < ngrid; ++g) s += out[g] * out[g];
  const double nrm = std::sqrt(s * dv);
  for (long g = 0; g < ngrid; ++g) out[g] /= nrm;
}

KTables k_tables(long nx, long ny, long nz, double dx, double dy, double dz, double ekinmax) {
  KTables t;
  t.kx.assign(nx, 0.0);
  t.ky.assign(ny, 0.0);
  t.kz.assign(nz, 0.0);
  const double ix = 1.0 / (double)nx, iy = 1.0 / (double)ny, iz = 1.0 / (double)nz;
  const double gx = kTwoPi / ((double)nx * dx), gy = kTwoPi / ((double)ny * dy),
               gz = kTwoPi / ((double)nz * dz);
  // each axis multiplies its 1/n factors in the reference's order
  for (long j = 1; j <= nx / 2; ++j) {
    const double k = (double)j * gx;
    t.kx[j] = t.kx[nx - j] = 0.5 * (k * k) * ix * iy * iz / 1.0;
  }
  for (long j = 1; j <= ny / 2; ++j) {
    const double k = (double)j * gy;
    t.ky[j] = t.ky[ny - j] = 0.5 * (k * k) * iy * ix * iz / 1.0;
  }
  for (long j = 1; j <= nz / 2; ++j) {
    const double k = (double)j * gz;
    t.kz[j] = t.kz[nz - j] = 0.5 * (k * k) * iz * ix * iy / 1.0;
  }
  t.cap = ekinmax * (iy * ix * iz);
  return t;
}

void ksqr_grid(const KTables& t, long nx, long ny, long nz, double* ksqr) {
  for (long jz = 0; jz < nz; ++jz)
    for (long jy = 0; jy < ny; ++jy)
      for (long jx = 0; jx < nx; ++jx) {
        const double v = t.kx[jx] + t.ky[jy] + t.kz[jz];
        ksqr[nx * (ny * jz + jy) + jx] = v > t.cap ? t.cap : v;
      }
}

std::vector<double> twiddles(int L) {
  std::vector<double> w(2 * (size_t)L);
  const long double tp = 6.283185307179586476925286766559005768L;
  for (int m = 0; m < L; ++m) {
    double c, s;
    if (m == 0) { c = 1.0; s = 0.0; }
    else if (2 * m == L) { c = -1.0; s = 0.0; }
    else if (4 * m == L) { c = 0.0; s = 1.0; }
    else if (4 * m == 3 * L) { c = 0.0; s = -1.0; }
    else {
      const long double a = tp * (long double)m / (long double)L;
      c = (double)cosl(a);
      s = (double)sinl(a);
    }
    w[2 * m] = c;
    w[2 * m + 1] = -s;
  }
  return w;
}

void form_factor_table(const double a[4], double vol_per_atom, double* r, double* v) {
  constexpr int n = 1024;
  const double dq = (5.0 - 0.0) / (double)n;
  const double dr = 0.02 * kTwoPi / ((double)n * dq);
  std::vector<double> q(n), vq(n);
  double run = 0.0;
  for (int i = 0; i < n; ++i, run += dq) q[i] = run;
  run = 0.0;
  for (int i = 0; i < n; ++i, run += dr) r[i] = run;
  for (int i = 0; i < n; ++i)
    vq[i] = a[0] * (q[i] * q[i] - a[1]) / (a[2] * std::exp(a[3] * q[i] * q[i]) + 1.0) *
            vol_per_atom;
  const double cube = std::pow(kTwoPi, 3.0);
  for (int k = 1; k < n; ++k) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += q[i] * std::sin(q[i] * r[k]) * vq[i];
    v[k] = s * (dq * 4.0 * kPi / (cube * r[k]));
  }
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += q[i] * q[i] * vq[i];
  v[0] = s * (dq * 4.0 * kPi / cube);
}

std::vector<double> axis_coords(long n, double min, double step) {
  std::vector<double> c(n);
  double run = min;
  for (long j = 0; j < n; ++j, run += step) c[j] = run;
  return c;
}

std::vector<std::pair<long long, long long>> filter_chunks(long long pairs, long long bc,
                                                           bool host, double ratio) {
  std::vector<std::pair<long long, long long>> chunks;
  if (pairs < 1 || bc < 1) return chunks;
  for (long long b0 = 0; b0 < pairs; b0 += bc)
    chunks.push_back({b0, std::min<long long>(bc, pairs - b0)});
  if (!host) return chunks;
  if (ratio >= 0.0) {
    auto& last = chunks.back();
    if (last.second >= 8) {
      long long t = (long long)std::ceil(ratio * (double)last.second / (1.0 + ratio));
      t = std::max<long long>(t, 4);
      t = std::min<long long>(t, last.second / 2);
      last.second -= t;
      chunks.push_back({last.first + last.second, t});
    }
  } else {
    while (chunks.back().second >= 8) {
      auto& last = chunks.back();
      const long long second = last.second / 2;
      last.second -= second;
      chunks.push_back({last.first + last.second, second});
    }
  }
  return chunks;
}

}  // namespace host
}  // namespace sep
