// sep_dft.cuh -- complex arithmetic and in-register DFT butterflies.
//
// Building blocks of the line FFTs that apply the kinetic operator of
// filter/hamiltonian.c:27-44 (the reference calls FFTW there).  Conventions
// follow FFTW: forward transforms use exp(-2 pi i jk/n) (S = -1), backward
// ones exp(+2 pi i jk/n) (S = +1), neither is normalised.
//
// Roots of unity used inside the butterflies are compile-time constants:
// cos/sin(2 pi k/n) are reduced to an angle in [0, pi/4] by exact octant
// symmetries and evaluated by a Taylor series in double precision (error
// below 2 ulp), so no run-time math function is involved.
#pragma once

#include <cuda_runtime.h>

namespace sep {

// ---------------------------------------------------------------------------
// complex types: double2 / float2 so that loads and stores are vectorised
template <typename T> struct cvec;
template <> struct cvec<double> { using type = double2; };
template <> struct cvec<float> { using type = float2; };
template <typename T> using cx = typename cvec<T>::type;

template <typename T> __host__ __device__ __forceinline__ cx<T> mk(T a, T b) {
  cx<T> r;
  r.x = a;
  r.y = b;
  return r;
}
template <typename T> __device__ __forceinline__ cx<T> add(cx<T> a, cx<T> b) {
  return mk<T>(a.x + b.x, a.y + b.y);
}
template <typename T> __device__ __forceinline__ cx<T> sub(cx<T> a, cx<T> b) {
  return mk<T>(a.x - b.x, a.y - b.y);
}
template <typename T> __device__ __forceinline__ cx<T> mul(cx<T> a, cx<T> b) {
  return mk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename T> __device__ __forceinline__ cx<T> mulc(cx<T> a, cx<T> b) {
  return mk<T>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
// a * (s i), s = +1 or -1
template <int S, typename T> __device__ __forceinline__ cx<T> muli(cx<T> a) {
  return (S > 0) ? mk<T>(-a.y, a.x) : mk<T>(a.y, -a.x);
}
// o = alpha (t + v p) + beta p, the Newton step's epilogue (filter/hnorm.c:11-39),
// with its multiply-adds fixed so that every kernel rounds it the same way
__device__ __forceinline__ float fma_t(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_t(double a, double b, double c) { return __fma_rn(a, b, c); }
template <typename T>
__device__ __forceinline__ cx<T> newton_epi(cx<T> t, T v, cx<T> p, T alpha, T beta) {
  const T hx = fma_t(v, p.x, t.x), hy = fma_t(v, p.y, t.y);
  return mk<T>(fma_t(alpha, hx, beta * p.x), fma_t(alpha, hy, beta * p.y));
}
template <typename T> __device__ __forceinline__ cx<T> scale(cx<T> a, T s) {
  return mk<T>(a.x * s, a.y * s);
}

// ---------------------------------------------------------------------------
// compile-time cos / sin of 2 pi k / n
namespace ct {
constexpr double kQuarterPi = 0.78539816339744830961566084581987572;

constexpr double cos_series(double t) {
  // sum_{j} (-1)^j t^(2j) / (2j)!, |t| <= pi/4, 12 terms
  double t2 = t * t, term = 1.0, sum = 1.0;
  for (int j = 1; j <= 12; ++j) {
    term = -term * t2 / double((2 * j - 1) * (2 * j));
    sum += term;
  }
  return sum;
}
constexpr double sin_series(double t) {
  double t2 = t * t, term = t, sum = t;
  for (int j = 1; j <= 12; ++j) {
    term = -term * t2 / double((2 * j) * (2 * j + 1));
    sum += term;
  }
  return sum;
}
// returns cos (want_sin = false) or sin of 2 pi k / n
constexpr double root(long k, long n, bool want_sin) {
  long m = k % n;
  if (m < 0) m += n;
  // theta = (8m/n) * pi/4 ; octant q, remainder r8 / n
  long q = (8 * m) / n;
  long r8 = 8 * m - q * n;
  // theta = q pi/4 + psi with psi = (r8/n) pi/4; odd q reflects:
  // theta = (q+1) pi/4 - psi' with psi' = ((n - r8)/n) pi/4
  long p = 0;  // theta = p pi/2 + s * a
  int s = 1;
  long num = 0;  // a = (num / n) * pi/4
  if (q % 2 == 0) { p = q / 2; s = 1; num = r8; }
  else { p = (q + 1) / 2; s = -1; num = n - r8; }
  double a = (num == 0) ? 0.0 : kQuarterPi * double(num) / double(n);
  double c = (num == 0) ? 1.0 : cos_series(a);
  double sn = (num == 0) ? 0.0 : double(s) * sin_series(a);
  if (num == n) { c = 0.70710678118654752440; sn = double(s) * 0.70710678118654752440; }
  double rc = c, rs = sn;  // rotate by p * pi/2
  switch (p % 4) {
    case 0: rc = c; rs = sn; break;
    case 1: rc = -sn; rs = c; break;
    case 2: rc = -c; rs = -sn; break;
    default: rc = sn; rs = -c; break;
  }
  return want_sin ? rs : rc;
}
}  // namespace ct

template <long K, long N> struct Root {
  static constexpr double c = ct::root(K, N, false);
  static constexpr double s = ct::root(K, N, true);
};

// multiply by exp(S 2 pi i K / N) with the trivial cases folded away
template <int S, long K, long N, typename T>
__device__ __forceinline__ cx<T> twiddle(cx<T> a) {
  constexpr long m = ((K % N) + N) % N;
  if constexpr (m == 0) {
    return a;
  } else if constexpr (2 * m == N) {
    return mk<T>(-a.x, -a.y);
  } else if constexpr (4 * m == N) {
    return muli<S, T>(a);
  } else if constexpr (4 * m == 3 * N) {
    return muli<-S, T>(a);
  } else if constexpr (8 * m == N || 8 * m == 3 * N || 8 * m == 5 * N || 8 * m == 7 * N) {
    // (+-1 +- i)/sqrt(2): 2 adds + 2 multiplies
    constexpr T h = T(0.70710678118654752440);
    constexpr double c = Root<m, N>::c;
    constexpr double s = double(S) * Root<m, N>::s;
    if constexpr (c > 0 && s > 0) return mk<T>((a.x - a.y) * h, (a.x + a.y) * h);
    else if constexpr (c > 0 && s < 0) return mk<T>((a.x + a.y) * h, (a.y - a.x) * h);
    else if constexpr (c < 0 && s > 0) return mk<T>(-(a.x + a.y) * h, (a.x - a.y) * h);
    else return mk<T>((a.y - a.x) * h, -(a.x + a.y) * h);
  } else {
    constexpr T c = T(Root<m, N>::c);
    constexpr T s = T(double(S) * Root<m, N>::s);
    return mk<T>(a.x * c - a.y * s, a.x * s + a.y * c);
  }
}

// ---------------------------------------------------------------------------
// In-register DFT of length R, natural order in and out:
//   v[k] <- sum_j v[j] exp(S 2 pi i j k / R)
template <int R, int S, typename T> struct Dft;

template <int S, typename T> struct Dft<1, S, T> {
  static __device__ __forceinline__ void run(cx<T>*) {}
};

template <int S, typename T> struct Dft<2, S, T> {
  static __device__ __forceinline__ void run(cx<T>* v) {
    cx<T> a = v[0], b = v[1];
    v[0] = add<T>(a, b);
    v[1] = sub<T>(a, b);
  }
};

template <int S, typename T> struct Dft<3, S, T> {
  static __device__ __forceinline__ void run(cx<T>* v) {
    constexpr T h = T(0.86602540378443864676);  // sin(2 pi / 3)
    cx<T> t = add<T>(v[1], v[2]);
    cx<T> d = sub<T>(v[1], v[2]);
    cx<T> m = mk<T>(v[0].x - T(0.5) * t.x, v[0].y - T(0.5) * t.y);
    cx<T> r = muli<S, T>(scale<T>(d, h));
    v[0] = add<T>(v[0], t);
    v[1] = add<T>(m, r);
    v[2] = sub<T>(m, r);
  }
};

template <int S, typename T> struct Dft<4, S, T> {
  static __device__ __forceinline__ void run(cx<T>* v) {
    cx<T> t0 = add<T>(v[0], v[2]), t1 = sub<T>(v[0], v[2]);
    cx<T> t2 = add<T>(v[1], v[3]), t3 = muli<S, T>(sub<T>(v[1], v[3]));
    v[0] = add<T>(t0, t2);
    v[2] = sub<T>(t0, t2);
    v[1] = add<T>(t1, t3);
    v[3] = sub<T>(t1, t3);
  }
};

// odd prime R: pair j with R - j
template <int R, int S, typename T> struct DftOdd {
  template <int P, int Q>
  static __device__ __forceinline__ void acc(const cx<T>* sm, const cx<T>* df, cx<T>& cr,
                                             cx<T>& er) {
    if constexpr (Q <= (R - 1) / 2) {
      constexpr T c = T(Root<(long)P * Q, R>::c);
      constexpr T s = T(double(S) * Root<(long)P * Q, R>::s);
      cr.x += c * sm[Q].x;
      cr.y += c * sm[Q].y;
      er.x -= s * df[Q].y;  // i s d
      er.y += s * df[Q].x;
      acc<P, Q + 1>(sm, df, cr, er);
    }
  }
  template <int P>
  static __device__ __forceinline__ void out(const cx<T>& x0, const cx<T>* sm, const cx<T>* df,
                                             cx<T>* v) {
    if constexpr (P <= (R - 1) / 2) {
      cx<T> cr = x0, er = mk<T>(T(0), T(0));
      acc<P, 1>(sm, df, cr, er);
      v[P] = add<T>(cr, er);
      v[R - P] = sub<T>(cr, er);
      out<P + 1>(x0, sm, df, v);
    }
  }
  static __device__ __forceinline__ void run(cx<T>* v) {
    constexpr int H = (R - 1) / 2;
    cx<T> sm[H + 1], df[H + 1];
#pragma unroll
    for (int q = 1; q <= H; ++q) {
      sm[q] = add<T>(v[q], v[R - q]);
      df[q] = sub<T>(v[q], v[R - q]);
    }
    cx<T> x0 = v[0], s0 = v[0];
#pragma unroll
    for (int q = 1; q <= H; ++q) s0 = add<T>(s0, sm[q]);
    out<1>(x0, sm, df, v);
    v[0] = s0;
  }
};
template <int S, typename T> struct Dft<5, S, T> : DftOdd<5, S, T> {};
template <int S, typename T> struct Dft<7, S, T> : DftOdd<7, S, T> {};

// composite R = P * Q in registers (four-step):
//   n = n1 + P n2, k = k2 + Q k1
//   Y[n1][k2] = DFT_Q over n2 of v[n1 + P n2], times w_R^(S n1 k2)
//   v[k2 + Q k1] = DFT_P over n1 of Y[n1][k2]
template <int P, int Q, int S, typename T> struct DftPQ {
  template <int N1, int K2>
  static __device__ __forceinline__ void tw(cx<T> (&y)[P][Q]) {
    if constexpr (N1 < P) {
      if constexpr (K2 < Q) {
        y[N1][K2] = twiddle<S, (long)N1 * K2, (long)P * Q, T>(y[N1][K2]);
        tw<N1, K2 + 1>(y);
      } else {
        tw<N1 + 1, 0>(y);
      }
    }
  }
  static __device__ __forceinline__ void run(cx<T>* v) {
    cx<T> y[P][Q];
#pragma unroll
    for (int n1 = 0; n1 < P; ++n1) {
#pragma unroll
      for (int n2 = 0; n2 < Q; ++n2) y[n1][n2] = v[n1 + P * n2];
      Dft<Q, S, T>::run(y[n1]);
    }
    tw<1, 1>(y);
#pragma unroll
    for (int k2 = 0; k2 < Q; ++k2) {
      cx<T> z[P];
#pragma unroll
      for (int n1 = 0; n1 < P; ++n1) z[n1] = y[n1][k2];
      Dft<P, S, T>::run(z);
#pragma unroll
      for (int k1 = 0; k1 < P; ++k1) v[k2 + Q * k1] = z[k1];
    }
  }
};
template <int S, typename T> struct Dft<6, S, T> : DftPQ<2, 3, S, T> {};
template <int S, typename T> struct Dft<8, S, T> : DftPQ<2, 4, S, T> {};
template <int S, typename T> struct Dft<9, S, T> : DftPQ<3, 3, S, T> {};
template <int S, typename T> struct Dft<10, S, T> : DftPQ<2, 5, S, T> {};
template <int S, typename T> struct Dft<12, S, T> : DftPQ<3, 4, S, T> {};
template <int S, typename T> struct Dft<14, S, T> : DftPQ<2, 7, S, T> {};
template <int S, typename T> struct Dft<16, S, T> : DftPQ<4, 4, S, T> {};
template <int S, typename T> struct Dft<20, S, T> : DftPQ<4, 5, S, T> {};
template <int S, typename T> struct Dft<24, S, T> : DftPQ<8, 3, S, T> {};
template <int S, typename T> struct Dft<32, S, T> : DftPQ<4, 8, S, T> {};

}  // namespace sep
