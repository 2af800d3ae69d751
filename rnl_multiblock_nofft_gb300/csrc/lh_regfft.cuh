// lh_regfft.cuh — DFTs held in one thread's registers, for the two-stage transform kernels.
//
// dft_reg<R, INV>(v) transforms R complex values in place, natural order in and out:
// X[k] = sum_n x[n] exp(-+2 pi i n k / R) (INV = true: the + sign, unscaled). R = A * B is
// split Cooley-Tukey style into B-point DFTs (recursively) and A-point butterflies (dftR of
// lh_internal.cuh, A in {8, 6, 4, 3, 2}) with the twiddles exp(-2 pi i m / R) as compile-time
// constants: every index is a template parameter, so the data stay in registers and the
// permutations between the two steps cost no instruction. The constants are computed here
// from the Taylor series of sine and cosine on the first octant (constexpr, double).
#pragma once
#include <utility>

#include "lh_internal.cuh"

namespace regfft {

constexpr double kPi = 3.14159265358979323846264338327950288;

// sine and cosine of |x| <= pi/4 from their Taylor series (30 terms: below the double ulp)
__host__ __device__ constexpr double taylor_sin(double x) {
  double t = x, s = x;
  for (int n = 1; n < 30; ++n) { t *= -x * x / ((2.0 * n) * (2.0 * n + 1.0)); s += t; }
  return s;
}
__host__ __device__ constexpr double taylor_cos(double x) {
  double t = 1.0, s = 1.0;
  for (int n = 1; n < 30; ++n) { t *= -x * x / ((2.0 * n - 1.0) * (2.0 * n)); s += t; }
  return s;
}
// cos and sin of 2 pi m / r: reduced to an octant by the exact symmetries of the circle
// (8 m / r split into the octant index and the remainder, in integers)
__host__ __device__ constexpr double cos2pi(long m, long r) {
  m %= r; if (m < 0) m += r;
  const long o = (8 * m) / r;          // octant 0..7
  const long rem = 8 * m - o * r;      // 0 <= rem < r: angle = (o + rem / r) * pi / 4
  const double x = kPi / 4.0 * (double)rem / (double)r;
  const double c = taylor_cos(x), s = taylor_sin(x);
  const double cq = taylor_cos(kPi / 4.0 - x), sq = taylor_sin(kPi / 4.0 - x);
  switch (o) {
    case 0: return c;
    case 1: return sq;
    case 2: return -s;
    case 3: return -cq;
    case 4: return -c;
    case 5: return -sq;
    case 6: return s;
    default: return cq;
  }
}
// sin(2 pi m / r) = cos(2 pi (4 m - r) / (4 r)), exact in integers
__host__ __device__ constexpr double sin2pi(long m, long r) { return cos2pi(4 * m - r, 4 * r); }

template <int I, int N, typename F>
__host__ __device__ __forceinline__ void static_for(F &&f) {
  if constexpr (I < N) {
    f(std::integral_constant<int, I>{});
    static_for<I + 1, N>(f);
  }
}

// v *= exp(-+2 pi i M / R) (INV: +), M and R compile-time; trivial angles cost no multiply
template <int M, int R, bool INV, typename V>
__host__ __device__ __forceinline__ void twiddle_c(V &v) {
  typedef decltype(v.x) S;
  constexpr int m = ((M % R) + R) % R;
  if constexpr (m == 0) {
    return;
  } else if constexpr ((4 * m) % R == 0) {
    constexpr int q = (4 * m) / R;  // quarter turns of the forward (clockwise) rotation
    if constexpr (q == 2) { v.x = -v.x; v.y = -v.y; }
    else if constexpr ((q == 1) != INV) { const S t = v.x; v.x = v.y; v.y = -t; }   // * (-i)
    else { const S t = v.x; v.x = -v.y; v.y = t; }                                   // * (+i)
  } else {
    constexpr double c = cos2pi(m, R), s = INV ? sin2pi(m, R) : -sin2pi(m, R);
    const S cc = (S)c, ss = (S)s;
    const S x = v.x * cc - v.y * ss;
    v.y = v.x * ss + v.y * cc;
    v.x = x;
  }
}

template <int R> struct first_factor {
  static constexpr int value = (R % 8 == 0 && R > 8) ? 8 : (R % 6 == 0 && R > 6) ? 6 : (R % 4 == 0 && R > 4) ? 4
                             : (R % 3 == 0 && R > 3) ? 3 : (R % 2 == 0 && R > 2) ? 2 : R;
};

template <int R, bool INV, typename V>
__host__ __device__ __forceinline__ void dft_reg(V *v) {
  if constexpr (R == 1) {
    return;
  } else if constexpr (R == 2 || R == 3 || R == 4 || R == 6 || R == 8) {
    dftR<R, INV>(v);
  } else {
    constexpr int A = first_factor<R>::value, B = R / A;
    static_assert(A * B == R && A >= 2 && A <= 8, "register DFT length must factor into 2, 3, 4, 6, 8");
    V z[A][B];
    // B-point DFTs over n1 of x[n2 + A n1], then the twiddles exp(-2 pi i n2 k2 / R)
    static_for<0, A>([&](auto n2_) {
      constexpr int n2 = decltype(n2_)::value;
      static_for<0, B>([&](auto n1_) {
        constexpr int n1 = decltype(n1_)::value;
        z[n2][n1] = v[n2 + A * n1];
      });
      dft_reg<B, INV>(z[n2]);
      static_for<0, B>([&](auto k2_) {
        constexpr int k2 = decltype(k2_)::value;
        twiddle_c<n2 * k2, R, INV>(z[n2][k2]);
      });
    });
    // A-point DFTs over n2: X[B k1 + k2]
    static_for<0, B>([&](auto k2_) {
      constexpr int k2 = decltype(k2_)::value;
      V s[A];
      static_for<0, A>([&](auto n2_) { s[decltype(n2_)::value] = z[decltype(n2_)::value][k2]; });
      dftR<A, INV>(s);
      static_for<0, A>([&](auto k1_) { v[B * decltype(k1_)::value + k2] = s[decltype(k1_)::value]; });
    });
  }
}

}  // namespace regfft
