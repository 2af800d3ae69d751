// Host check of the register DFTs of lh_regfft.cuh (tests/test_fft_host.py builds and runs it):
// dft_reg<R> in both directions, FP64 and FP32, against a direct DFT in long double, and the
// compile-time twiddle constants against cosl/sinl. Prints "R err64_fwd err64_inv err32_fwd
// err32_inv" per length (max abs error / max abs value) and "tw <max error>" last.
#include "../rnl_multiblock_nofft_gb300/csrc/lh_regfft.cuh"

#include <cmath>
#include <cstdio>
#include <random>

template <int R, bool INV, typename V>
static double check() {
  typedef decltype(V().x) S;
  std::mt19937 rng(R * 7 + INV);
  std::normal_distribution<double> nd;
  double x[R][2];
  V v[R];
  for (int n = 0; n < R; ++n) {
    x[n][0] = nd(rng); x[n][1] = nd(rng);
    v[n].x = (S)x[n][0]; v[n].y = (S)x[n][1];
  }
  regfft::dft_reg<R, INV>(v);
  double err = 0.0, mx = 0.0;
  const long double tp = 6.283185307179586476925286766559L * (INV ? 1.0L : -1.0L);
  for (int k = 0; k < R; ++k) {
    long double re = 0, im = 0;
    for (int n = 0; n < R; ++n) {
      const long double a = tp * (long double)((long)n * k % R) / R;
      re += x[n][0] * cosl(a) - x[n][1] * sinl(a);
      im += x[n][0] * sinl(a) + x[n][1] * cosl(a);
    }
    err = fmax(err, fmax(fabs((double)(v[k].x - re)), fabs((double)(v[k].y - im))));
    mx = fmax(mx, fmax(fabs((double)re), fabs((double)im)));
  }
  return err / mx;
}

template <int R>
static void row() {
  printf("%d %.3e %.3e %.3e %.3e\n", R, check<R, false, double2>(), check<R, true, double2>(),
         check<R, false, float2>(), check<R, true, float2>());
}

int main() {
  row<2>(); row<3>(); row<4>(); row<6>(); row<8>(); row<9>(); row<12>(); row<16>(); row<18>();
  row<24>(); row<32>(); row<36>(); row<48>(); row<64>(); row<72>(); row<96>(); row<144>();
  double tw = 0.0;
  for (long r = 1; r <= 1200; ++r)
    for (long m = -r; m <= 2 * r; m += (r > 100 ? 7 : 1)) {
      const long double a = 6.283185307179586476925286766559L * (long double)m / (long double)r;
      tw = fmax(tw, fabs(regfft::cos2pi(m, r) - (double)cosl(a)));
      tw = fmax(tw, fabs(regfft::sin2pi(m, r) - (double)sinl(a)));
    }
  printf("tw %.3e\n", tw);
  return 0;
}
