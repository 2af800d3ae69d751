// lh_internal.cuh — device-side data model of one channel and the shared-memory FFT.
//
// Layout in HBM: every spectral field is plane-major, complex [level][col] with
// col = ikz * (N1/2+1) + ikx. A y-level of a field is therefore one spectral x/z
// plane (what the reference builds with modes_to_planes_*, FOU3D.f90:1000-1098),
// and for a fixed level consecutive columns are consecutive in memory, so the
// per-column tridiagonal solves (one thread per column) load coalesced.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/lh.h"

// Geometry and coefficients, passed to kernels by value.
struct Geo {
  int N1, N2, N1h, G1, G2, dny, nu, nv, np, ncol, nuI, nvI, nn;
  int N3[4], N4[4];
  const double *yu, *yv, *thu, *thv, *d2u, *d2v, *k1x, *k2x, *k1z, *k2z;
  // stagger interpolation: u-level q (v -> centre): (iua*v[q] + iub*v[q-1]) / iud
  const double *iua, *iub, *iud;
  // v-level q (centre -> face): (iva*u[q+1] + ivb*u[q]) / ivd
  const double *iva, *ivb, *ivd;
  const double *thud;  // dd * thu (the divergence's y factor)
  // FP32 copies for the mixed form (no conversion in the kernels): wavenumbers,
  // interpolation weights, metrics, difference coefficients and their row sums
  const float *k1xf, *k1zf, *iuaf, *iubf, *ivaf, *ivbf, *thuf, *thvf, *d2uf, *d2vf, *sdgu, *sdgv;
  double Re, CFL, dtv, dd, dthetavi, alp, bet, Kib;
  double aRK[3], bRK[3], cRK[3], dRK[3], gRK[3];
  double gw[3][2];
  double gwbc1, gwbc3;
  int flag_ctpress;
  // ---- multiblock and plane views ----
  // The state lives on the wall-band mode grid: level stride ncolF = N1hF * N2F columns
  // (column = kz row * N1hF + kx). A nonlinear launch sees one class of planes (a
  // "view"): N1h, N2, G1, G2 and ncol are the view's, mode (r, kx) of the view is
  // wall-grid column gcol(); slotq maps the launch's slots to levels (null: slot + 1
  // for u slots, slot - nuI + 1 for v slots).
  int mb;
  int N1hF, N2F, ncolF;
  const int *slotq;
  // Column segments of the solve kernels: virtual column vc -> (column, band 0..2);
  // a long column has band 1 (all levels), a short column bands 0 and 2 (the wall
  // bands' levels). vcol null: vc = column, band 1.
  int nvc;
  const int2 *vcol;
  int bq[3][6];  // per band: u lo, u hi, v lo, v hi, p lo, p hi (array indices, inclusive)
};

// wall-grid column of mode (r, kx) of the view g (r: the view's own kz row)
__host__ __device__ __forceinline__ int gcol(const Geo &g, int r, int kx) {
  return (r < g.N2 / 2 ? r : r + g.N2F - g.N2) * g.N1hF + kx;
}
// wall-grid kz row of the view's row r (index of k1z)
__host__ __device__ __forceinline__ int grow(const Geo &g, int r) { return r < g.N2 / 2 ? r : r + g.N2F - g.N2; }
// level of a nonlinear slot
__device__ __forceinline__ int slot_level(const Geo &g, int slot, bool isU) {
  return g.slotq ? g.slotq[slot] : (isU ? slot + 1 : slot - g.nuI + 1);
}
// The slot of launch row y in the inverse z passes: u and v slots interleaved (u slot i, then
// v slot i), so the levels a staggered interpolation reads (v faces q - 1, q for u level q;
// u levels q, q + 1 for v level q) are also read by the neighbouring rows and come from L2
// the second time; a bijection of [0, nuI + nvI).
__host__ __device__ __forceinline__ int zinv_slot(const Geo &g, int y) {
  const int m = g.nuI < g.nvI ? g.nuI : g.nvI;
  if (y < 2 * m) return (y & 1) ? g.nuI + (y >> 1) : (y >> 1);
  return g.nuI > g.nvI ? y - m : g.nuI + (y - m);
}
// column and band of a virtual column
__device__ __forceinline__ void vcol_of(const Geo &g, int vc, int &c, int &b) {
  if (g.vcol) { const int2 e = g.vcol[vc]; c = e.x; b = e.y; }
  else { c = vc; b = 1; }
}

// Scalars kept on the device (no host round trip inside a step).
struct DevScalars {
  double t, dt, dti, dtc, err, mpgx, QxT, Qx;
  double dgx;          // the last flow-rate correction g of flowrate_corr (the history's dpgx)
  double Umax, Uslip;  // maxvel and the slip velocity of mode (0,0), formed by lh_history_record
  long long iter;
  unsigned long long u1m, u2m, u3m;  // bit patterns of non-negative doubles (atomicMax)
  unsigned long long errbits;
  int status;
  int pad;
};

// ---------------------------------------------------------------------------
// double <-> float on the integer pipe. On this part conversion instructions
// issue on the FP64 pipe, which the mixed form keeps for the arithmetic that
// needs it; these do the IEEE-754 bit manipulation with integer operations.
// d2f_alu: round to nearest even; |x| < 2^-126 becomes a signed zero; Inf/NaN
// preserved. f2d_alu: exact (FP32 denormals read as zero).
// ---------------------------------------------------------------------------
__device__ __forceinline__ float d2f_alu(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned int hi = (unsigned int)(b >> 32);
  const unsigned int ed = (hi >> 20) & 0x7ffu;  // biased double exponent
  // round to nearest even on the 29 dropped mantissa bits (adding half an ulp minus one, plus
  // the kept lowest bit; a carry runs into the exponent), then drop them; bits 23-31 of the
  // shifted word hold the low 9 exponent bits, and subtracting 896 << 23 (mod 2^32) rebiases
  // them for every exponent of the normal float range
  const unsigned long long r = b + 0x0fffffffull + ((b >> 29) & 1ull);
  unsigned int f = (unsigned int)(r >> 29) - 0xc0000000u;
  if (ed - 897u > 253u)  // below 2^-126: zero; above the float range: inf, or NaN for a NaN
    f = ed < 897u ? 0u : ((ed == 0x7ffu && (b << 12) != 0ull) ? 0x7fc00000u : 0x7f800000u);
  return __uint_as_float((hi & 0x80000000u) | f);
}
__device__ __forceinline__ double f2d_alu(float x) {
  const unsigned int u = __float_as_uint(x);
  const unsigned int sign = u & 0x80000000u;
  const unsigned int e = (u >> 23) & 0xffu;
  const unsigned int m = u & 0x7fffffu;
  unsigned int hi, lo;
  if (e == 0u) { hi = sign; lo = 0u; }
  else if (e == 255u) { hi = sign | 0x7ff00000u | (m >> 3) | (m ? 0x80000u : 0u); lo = m << 29; }
  else { hi = sign | ((e + 896u) << 20) | (m >> 3); lo = m << 29; }
  return __longlong_as_double((long long)(((unsigned long long)hi << 32) | lo));
}
template <typename T> __device__ __forceinline__ T to_t(double x);
template <> __device__ __forceinline__ double to_t<double>(double x) { return x; }
template <> __device__ __forceinline__ float to_t<float>(double x) { return d2f_alu(x); }
__device__ __forceinline__ double to_d(double x) { return x; }
__device__ __forceinline__ double to_d(float x) { return f2d_alu(x); }

// ---------------------------------------------------------------------------
// complex helpers (double2 / float2)
// ---------------------------------------------------------------------------
template <typename T> struct C2;
template <> struct C2<double> { typedef double2 t; };
template <> struct C2<float> { typedef float2 t; };

template <typename V> __host__ __device__ __forceinline__ V cadd(V a, V b) { V r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename V> __host__ __device__ __forceinline__ V csub(V a, V b) { V r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename V> __host__ __device__ __forceinline__ V cmul(V a, V b) {
  V r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}
template <typename V, typename S> __device__ __forceinline__ V cscale(V a, S s) { V r; r.x = a.x * s; r.y = a.y * s; return r; }
template <typename V> __device__ __forceinline__ V cconj(V a) { a.y = -a.y; return a; }
template <typename V> __device__ __forceinline__ V czero() { V r; r.x = 0; r.y = 0; return r; }
// i*k*a for a real k: (-k*a.y, k*a.x)
template <typename V, typename S> __device__ __forceinline__ V cimul(S k, V a) { V r; r.x = -k * a.y; r.y = k * a.x; return r; }

// ---------------------------------------------------------------------------
// Stockham mixed-radix (2, 3, 4) FFT of NL lines of length N held in shared
// memory, ping-ponging between two buffers. tw[e] = exp(-2 pi i e / N).
// INV = true: backward (exp(+i)), unscaled. Returns the buffer holding the result.
// ---------------------------------------------------------------------------
template <int R, bool INV, typename V>
__host__ __device__ __forceinline__ void dftR(V *v) {
  if (R == 8) {
    // two radix-4 DFTs on the even and odd elements, then W8^k on the odd ones
    typedef decltype(v[0].x) S;
    const S h = (S)0.70710678118654752440084436210485;  // 1/sqrt(2)
    V e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
    dftR<4, INV>(e);
    dftR<4, INV>(o);
    V t1, t2, t3;
    // forward W8 = (1 - i)/sqrt2, W8^2 = -i, W8^3 = (-1 - i)/sqrt2; backward conjugate
    if (INV) {
      t1.x = h * (o[1].x - o[1].y); t1.y = h * (o[1].x + o[1].y);
      t2.x = -o[2].y; t2.y = o[2].x;
      t3.x = -h * (o[3].x + o[3].y); t3.y = h * (o[3].x - o[3].y);
    } else {
      t1.x = h * (o[1].x + o[1].y); t1.y = h * (o[1].y - o[1].x);
      t2.x = o[2].y; t2.y = -o[2].x;
      t3.x = h * (o[3].y - o[3].x); t3.y = -h * (o[3].x + o[3].y);
    }
    v[0] = cadd(e[0], o[0]); v[4] = csub(e[0], o[0]);
    v[1] = cadd(e[1], t1); v[5] = csub(e[1], t1);
    v[2] = cadd(e[2], t2); v[6] = csub(e[2], t2);
    v[3] = cadd(e[3], t3); v[7] = csub(e[3], t3);
  } else if (R == 6) {
    // two radix-3 DFTs on the even and odd elements, then W6^k on the odd ones
    typedef decltype(v[0].x) S;
    const S s3 = (S)0.86602540378443864676372317075294;  // sin(2 pi / 6)
    V e[3] = {v[0], v[2], v[4]}, o[3] = {v[1], v[3], v[5]};
    dftR<3, INV>(e);
    dftR<3, INV>(o);
    V t1, t2;
    // forward W6 = (1/2, -s3), W6^2 = (-1/2, -s3); backward conjugate
    if (INV) {
      t1.x = (S)0.5 * o[1].x - s3 * o[1].y; t1.y = (S)0.5 * o[1].y + s3 * o[1].x;
      t2.x = (S)-0.5 * o[2].x - s3 * o[2].y; t2.y = (S)-0.5 * o[2].y + s3 * o[2].x;
    } else {
      t1.x = (S)0.5 * o[1].x + s3 * o[1].y; t1.y = (S)0.5 * o[1].y - s3 * o[1].x;
      t2.x = (S)-0.5 * o[2].x + s3 * o[2].y; t2.y = (S)-0.5 * o[2].y - s3 * o[2].x;
    }
    v[0] = cadd(e[0], o[0]); v[3] = csub(e[0], o[0]);
    v[1] = cadd(e[1], t1); v[4] = csub(e[1], t1);
    v[2] = cadd(e[2], t2); v[5] = csub(e[2], t2);
  } else if (R == 2) {
    V a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  } else if (R == 4) {
    V a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
    V a2 = cadd(v[1], v[3]), a3 = csub(v[1], v[3]);
    V rot;  // forward: -i*a3 = (a3.y, -a3.x); backward: +i*a3 = (-a3.y, a3.x)
    if (INV) { rot.x = -a3.y; rot.y = a3.x; } else { rot.x = a3.y; rot.y = -a3.x; }
    v[0] = cadd(a0, a2);
    v[2] = csub(a0, a2);
    v[1] = cadd(a1, rot);
    v[3] = csub(a1, rot);
  } else if (R == 3) {
    typedef decltype(v[0].x) S;
    const S c = (S)-0.5;
    const S s = (S)0.86602540378443864676372317075294;  // sin(2 pi / 3)
    V t1 = cadd(v[1], v[2]), t2 = csub(v[1], v[2]);
    V m = v[0];
    v[0] = cadd(m, t1);
    V b; b.x = m.x + c * t1.x; b.y = m.y + c * t1.y;
    V st;  // forward: -i*s*t2 = (s*t2.y, -s*t2.x)
    if (INV) { st.x = -s * t2.y; st.y = s * t2.x; } else { st.x = s * t2.y; st.y = -s * t2.x; }
    v[1] = cadd(b, st);
    v[2] = csub(b, st);
  }
}

// ---------------------------------------------------------------------------
// N and NL are compile-time (index arithmetic becomes shifts and multiplies); the
// radices run 8, ..., then 6, 4, 2 or 3 as the remaining length allows (384 = 8*8*6). IL selects the layout
// of the lines in shared memory: IL = false, line-contiguous (element e of line
// l at l*N + e, threads over e); IL = true, interleaved (at e*NL + l, threads
// over l first), which makes every stage's loads and stores bank-conflict free.
// ---------------------------------------------------------------------------
// Intermediate buffers between two stages are XOR-swizzled, element i stored at
// i ^ ((i >> 4) & 7) (a permutation within each aligned group of 8 elements, so any
// multiple of 8 elements maps onto itself): a radix-8 stage stores the 8 outputs of a
// butterfly 8 elements apart, and without the swizzle the lanes of a warp would all hit the
// same banks (16-way for 8-byte elements). A stage's first input and last output are not
// swizzled, so the buffers the kernels fill and read keep their plain layout.
__host__ __device__ __forceinline__ int fft_swz(int i) { return i ^ ((i >> 4) & 7); }

template <int R, bool INV, int N, int Ns, int NL, bool IL, bool SWI, bool SWO, typename V>
__device__ __forceinline__ void fft_stage_c(const V *__restrict__ src, V *__restrict__ dst,
                                            const V *__restrict__ tw) {
  constexpr int nb = N / R;
  constexpr int total = nb * NL;
  constexpr int step = N / (Ns * R);
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    int line, j;
    if (IL) { j = idx / NL; line = idx - j * NL; }
    else { line = idx / nb; j = idx - line * nb; }
    const int k = j % Ns;
    V v[R];
#pragma unroll
    for (int t = 0; t < R; ++t) {
      const int i = IL ? (j + t * nb) * NL + line : line * N + j + t * nb;
      v[t] = src[SWI ? fft_swz(i) : i];
    }
    if constexpr (Ns > 1) {  // the first stage's twiddles are all 1
#pragma unroll
      for (int t = 1; t < R; ++t) {
        V w = tw[k * step * t];
        if (INV) w.y = -w.y;
        v[t] = cmul(v[t], w);
      }
    }
    dftR<R, INV>(v);
    const int base = (j / Ns) * Ns * R + k;
#pragma unroll
    for (int t = 0; t < R; ++t) {
      const int i = IL ? (base + t * Ns) * NL + line : line * N + base + t * Ns;
      dst[SWO ? fft_swz(i) : i] = v[t];
    }
  }
}

template <bool INV, int N, int Ns, int NL, bool IL, typename V>
__device__ __forceinline__ V *fft_rec_c(V *a, V *b, const V *__restrict__ tw) {
  static_assert(N % 8 == 0, "the stage swizzle permutes aligned groups of 8 elements");
  if constexpr (Ns >= N) {
    return a;
  } else {
    constexpr int rem = N / Ns;
    constexpr int R = (rem % 8 == 0) ? 8 : ((rem % 6 == 0) ? 6 : ((rem % 4 == 0) ? 4 : ((rem % 2 == 0) ? 2 : 3)));
    constexpr bool first = (Ns == 1), last = (Ns * R >= N);
    fft_stage_c<R, INV, N, Ns, NL, IL, !first, !last>(a, b, tw);
    __syncthreads();
    return fft_rec_c<INV, N, Ns * R, NL, IL>(b, a, tw);
  }
}

template <bool INV, int N, int NL, bool IL, typename V>
__device__ __forceinline__ V *line_fft(V *a, V *b, const V *__restrict__ tw) {
  return fft_rec_c<INV, N, 1, NL, IL>(a, b, tw);
}

// plane row (physical z index, 0-based) of spectral kz-row r
__device__ __forceinline__ int prow(const Geo &g, int r) { return r < g.N2 / 2 ? r : r - g.N2 + g.G2; }

