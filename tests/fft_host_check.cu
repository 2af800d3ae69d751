// Host check of the shared-memory FFT's plan (tests/test_fft_host.py builds and runs it).
// It replays fft_stage_c / fft_rec_c of lh_internal.cuh on the CPU with the same radix
// plan, index formulas, first-pass rule and swizzle, calling the library's own dftR / cmul /
// fft_swz, and compares every compiled length with a direct DFT in long double.
#include "../rnl_multiblock_nofft_gb300/csrc/lh_internal.cuh"

#include <cmath>
#include <complex>
#include <cstdio>
#include <vector>

template <int R, bool INV, int N, int Ns, int NL, bool IL, bool SWI, bool SWO, typename V>
static void stage(const V *src, V *dst, const V *tw) {
  constexpr int nb = N / R, total = nb * NL, step = N / (Ns * R);
  for (int idx = 0; idx < total; ++idx) {  // every thread's work items, in order
    int line, j;
    if (IL) { j = idx / NL; line = idx - j * NL; }
    else { line = idx / nb; j = idx - line * nb; }
    const int k = j % Ns;
    V v[R];
    for (int t = 0; t < R; ++t) {
      const int i = IL ? (j + t * nb) * NL + line : line * N + j + t * nb;
      v[t] = src[SWI ? fft_swz(i) : i];
    }
    if (Ns > 1)
      for (int t = 1; t < R; ++t) {
        V w = tw[k * step * t];
        if (INV) w.y = -w.y;
        v[t] = cmul(v[t], w);
      }
    dftR<R, INV>(v);
    const int base = (j / Ns) * Ns * R + k;
    for (int t = 0; t < R; ++t) {
      const int i = IL ? (base + t * Ns) * NL + line : line * N + base + t * Ns;
      dst[SWO ? fft_swz(i) : i] = v[t];
    }
  }
}

template <bool INV, int N, int Ns, int NL, bool IL, typename V>
static V *rec(V *a, V *b, const V *tw) {
  if constexpr (Ns >= N) {
    return a;
  } else {
    constexpr int rem = N / Ns;
    constexpr int R = (rem % 8 == 0) ? 8 : ((rem % 6 == 0) ? 6 : ((rem % 4 == 0) ? 4 : ((rem % 2 == 0) ? 2 : 3)));
    constexpr bool first = (Ns == 1), last = (Ns * R >= N);
    stage<R, INV, N, Ns, NL, IL, !first, !last>(a, b, tw);
    return rec<INV, N, Ns * R, NL, IL>(b, a, tw);
  }
}

template <typename V, int N, bool IL, bool INV>
static double check() {
  typedef decltype(V().x) S;
  constexpr int NL = 3;
  const long double PI = 3.14159265358979323846264338327950288L;
  std::vector<V> a(N * NL), b(N * NL), tw(N);
  std::vector<std::complex<long double>> in(N * NL);
  for (int e = 0; e < N; ++e) {
    const long double ang = -2.0L * PI * e / N;
    tw[e].x = (S)cosl(ang); tw[e].y = (S)sinl(ang);
  }
  unsigned s = 12345u;
  for (int l = 0; l < NL; ++l)
    for (int e = 0; e < N; ++e) {
      s = s * 1103515245u + 12345u; const double re = (s >> 8) / 16777216.0 - 0.5;
      s = s * 1103515245u + 12345u; const double im = (s >> 8) / 16777216.0 - 0.5;
      V x; x.x = (S)re; x.y = (S)im;
      a[IL ? e * NL + l : l * N + e] = x;
      in[l * N + e] = std::complex<long double>((long double)x.x, (long double)x.y);
    }
  const V *res = rec<INV, N, 1, NL, IL>(a.data(), b.data(), tw.data());
  long double err = 0, mx = 0;
  for (int l = 0; l < NL; ++l)
    for (int k = 0; k < N; ++k) {
      std::complex<long double> sum = 0;
      for (int e = 0; e < N; ++e) {
        const long double ang = (INV ? 2.0L : -2.0L) * PI * (long double)((long)e * k % N) / N;
        sum += in[l * N + e] * std::complex<long double>(cosl(ang), sinl(ang));
      }
      const V r = res[IL ? k * NL + l : l * N + k];
      err = fmaxl(err, std::abs(sum - std::complex<long double>(r.x, r.y)));
      mx = fmaxl(mx, std::abs(sum));
    }
  return (double)(err / mx);
}

template <int N>
static void all() {
  printf("%d %.3e %.3e %.3e %.3e %.3e %.3e %.3e %.3e\n", N, check<double2, N, false, false>(),
         check<double2, N, false, true>(), check<double2, N, true, false>(), check<double2, N, true, true>(),
         check<float2, N, false, false>(), check<float2, N, false, true>(), check<float2, N, true, false>(),
         check<float2, N, true, true>());
}

int main() {
  all<24>(); all<48>(); all<72>(); all<96>(); all<144>(); all<192>(); all<288>(); all<384>();
  all<576>(); all<768>(); all<1152>();
  return 0;
}
