// lh_kernels.cuh — CUDA kernels of the RK3 substep (FP64 plain form; transforms
// templated on the transform precision).
//
// Per substep (littleharsh.f90:174-217):
//   k_zinv_nl   : stagger interpolation (FOU3D.f90:427-474) fused into the inverse z
//                 transforms of the six velocity planes of every level (cft, iopt>=0)
//   k_xpass_nl  : inverse x transforms (rft, iopt>=0), physical products
//                 (ops_in_planes2, FOU3D.f90:2090-2251), CFL maxima (dtc_calc), forward x
//                 transforms (rft, iopt<0) of the products
//   k_zfwd_nl   : forward z transforms (cft, iopt<0) + der_x/der_z (FOU3D.f90:476-593):
//                 N_xz of u, v, w and the y-flux products uv, vv, wv
//   k_dt        : dt = min(2.5 dtv, CFL dtc) on the device (FOU3D.f90:291-297)
//   k_helm_uw   : RHS0_u1/u3 + der_yu_h + du += -gRK N + solveU_W, one thread per column
//   k_helm_v    : RHS0_u2 + der_yv_h + du += -gRK N + solveV
//   k_meanflow  : flowrate_corr on mode (0,0) (constant flow rate)
//   k_press2    : divergence + solveP (LUsolP with the stored factors, k_build_dg) + v_corr
//                 + divergence of the corrected field in the third substep (max |div| -> err)
//   k_ib_du(_mx), k_spec_zinv, k_ib_xforce, k_zfwd_spec : immersed-boundary forcing of du
//                 (imm_bounds_u/v, FOU3D.f90:806-998) when the geometry has posts
//   Mixed form (LH_PREC_MIXED): FP32 transforms, and k_helm_u_mx2 / k_helm_v_mx2 solve
//   the Helmholtz systems for the increment in FP32 on top of the FP64 state.
// On request: k_xstats, k_wx_stats, k_spectra, k_slip (statistics), k_band_io, k_transpose
// (state I/O).
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "lh_internal.cuh"

#define NTHR 256
// blocks per SM the compiler leaves registers for in the immersed-boundary kernels (sweep knobs)
#ifndef LH_IBDU_MINB
#define LH_IBDU_MINB 1
#endif
#ifndef LH_IBX_MINB
#define LH_IBX_MINB 1
#endif

__device__ __forceinline__ void atomic_max_pos(unsigned long long *addr, double v) {
  atomicMax(addr, (unsigned long long)__double_as_longlong(v));
}

// max that keeps a NaN (fmax drops it): the CFL and divergence maxima must carry a
// non-finite state to dt and err, where the blow-up guard sees it
template <typename T>
__device__ __forceinline__ T nmax(T a, T b) { return (b > a || b != b) ? b : a; }
// running maximum of non-negative doubles (or NaN) kept as their bit patterns: the integer
// order of those patterns is the order of the values, a NaN above every number, so the
// comparisons stay off the FP64 pipe; warp_max_bits reduces it over the warp
__device__ __forceinline__ void bits_max(unsigned long long &m, double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  m = b > m ? b : m;
}
__device__ __forceinline__ unsigned long long warp_max_bits(unsigned long long m) {
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long w = __shfl_xor_sync(0xffffffffu, m, o);
    m = w > m ? w : m;
  }
  return m;
}
template <typename T>
__device__ __forceinline__ T warp_max(T v) {
  for (int o = 16; o > 0; o >>= 1) {
    T w = __shfl_xor_sync(0xffffffffu, v, o);
    v = (w > v || isnan((double)w)) ? w : v;
  }
  return v;
}

// Lines per block of the transform kernels, from a shared-memory budget per
// kernel (same values on the host and the device). The budgets set how many
// blocks share an SM; the defaults are the fastest of a sweep on GB300 at C1.
#ifndef LH_BUDGET_ZINV
#define LH_BUDGET_ZINV 49152
#endif
#ifndef LH_BUDGET_XPASS
#define LH_BUDGET_XPASS 24576
#endif
#ifndef LH_BUDGET_ZFWD
#define LH_BUDGET_ZFWD 49152
#endif
__host__ __device__ constexpr int lh_clamp(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
template <typename V> __host__ __device__ constexpr int kb_zinv(int n) {
  return lh_clamp(LH_BUDGET_ZINV / (2 * n * (int)sizeof(V)), 1, 16);
}
template <typename V> __host__ __device__ constexpr int pb_xpass(int n) {
  return lh_clamp(LH_BUDGET_XPASS / (8 * n * (int)sizeof(V)), 1, 8);
}
template <typename V> __host__ __device__ constexpr int kb_zfwd(int n) {
  return lh_clamp(LH_BUDGET_ZFWD / (8 * n * (int)sizeof(V)), 1, 8);
}

// ============================================================================
// T1: inverse z transforms of the velocity planes (with stagger interpolation).
// grid: x = kx group of KB lines, y = level slot (u-levels then v-levels), z = field.
// A layout: [(slot*3 + f)][l][kx], l = 0..G2-1, kx = 0..N1h-1.
// Lines are interleaved in shared memory (element l of line kk at l*KB + kk).
// ============================================================================
// Levels loaded ahead in the y sweeps of the column solves (0: a plain loop). Without it
// a sweep's loads wait for the previous level's stores (the compiler cannot separate the
// addresses), one memory latency per level. Deeper prefetch costs registers, i.e. resident
// warps; the depths below were the fastest of a sweep at 256x256x301 (mixed form).
#ifndef LH_PF_PRESS
#define LH_PF_PRESS 1
#endif
#ifndef LH_PF_HU
#define LH_PF_HU 1
#endif
#ifndef LH_PF_HU_BACK
#define LH_PF_HU_BACK 2
#endif
#ifndef LH_PF_HV
#define LH_PF_HV 4
#endif
#ifndef LH_PF_HV_BACK
#define LH_PF_HV_BACK 2
#endif
#ifndef LH_PRESS_MINB
#define LH_PRESS_MINB 1
#endif
#ifndef LH_ZINV_THREADS
#define LH_ZINV_THREADS 256
#endif
#ifndef LH_ZFWD_THREADS
#define LH_ZFWD_THREADS 256
#endif
template <typename T, int N>
__global__ void __launch_bounds__(LH_ZINV_THREADS) k_zinv_nl(const double2 *__restrict__ u1, const double2 *__restrict__ u2,
                                                  const double2 *__restrict__ u3, typename C2<T>::t *__restrict__ A,
                                                  Geo g, const typename C2<T>::t *__restrict__ twz) {
  typedef typename C2<T>::t V;
  constexpr int KB = kb_zinv<V>(N);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V *b0 = reinterpret_cast<V *>(smem_raw);
  V *b1 = b0 + KB * N;
  const int slot = zinv_slot(g, blockIdx.y), f = blockIdx.z, kx0 = blockIdx.x * KB;
  const bool isU = slot < g.nuI;
  const int q = slot_level(g, slot, isU);
  const int nc = g.ncolF;
  for (int i = threadIdx.x; i < KB * N; i += blockDim.x) b0[i] = czero<V>();
  __syncthreads();
  for (int idx = threadIdx.x; idx < g.N2 * KB; idx += blockDim.x) {
    const int r = idx / KB, kk = idx - r * KB, kx = kx0 + kk;
    if (kx >= g.N1h) continue;
    const int c = gcol(g, r, kx);
    V v;
    if (isU) {
      if (f == 0) { const double2 x = u1[(size_t)q * nc + c]; v.x = to_t<T>(x.x); v.y = to_t<T>(x.y); }
      else if (f == 2) { const double2 x = u3[(size_t)q * nc + c]; v.x = to_t<T>(x.x); v.y = to_t<T>(x.y); }
      else {  // interp_v: v faces -> centre q
        const double2 v0 = u2[(size_t)q * nc + c], vm = u2[(size_t)(q - 1) * nc + c];
        if (sizeof(T) == 8) {
          const double a = g.iua[q], b = g.iub[q];
          v.x = (T)(a * v0.x + b * vm.x);
          v.y = (T)(a * v0.y + b * vm.y);
        } else {
          const T a = (T)g.iuaf[q], b = (T)g.iubf[q];
          v.x = a * to_t<T>(v0.x) + b * to_t<T>(vm.x);
          v.y = a * to_t<T>(v0.y) + b * to_t<T>(vm.y);
        }
      }
    } else {
      if (f == 1) { const double2 x = u2[(size_t)q * nc + c]; v.x = to_t<T>(x.x); v.y = to_t<T>(x.y); }
      else {  // interp_u: centres -> face q
        const double2 *src = (f == 0) ? u1 : u3;
        const double2 up = src[(size_t)(q + 1) * nc + c], u0 = src[(size_t)q * nc + c];
        if (sizeof(T) == 8) {
          const double a = g.iva[q], b = g.ivb[q];
          v.x = (T)(a * up.x + b * u0.x);
          v.y = (T)(a * up.y + b * u0.y);
        } else {
          const T a = (T)g.ivaf[q], b = (T)g.ivbf[q];
          v.x = a * to_t<T>(up.x) + b * to_t<T>(u0.x);
          v.y = a * to_t<T>(up.y) + b * to_t<T>(u0.y);
        }
      }
    }
    b0[prow(g, r) * KB + kk] = v;
  }
  __syncthreads();
  V *res = line_fft<true, N, KB, true>(b0, b1, twz);
  V *dst = A + (size_t)(slot * 3 + f) * N * g.N1h;
  for (int idx = threadIdx.x; idx < N * KB; idx += blockDim.x) {
    const int l = idx / KB, kk = idx - l * KB, kx = kx0 + kk;
    if (kx < g.N1h) dst[(size_t)l * g.N1h + kx] = res[l * KB + kk];
  }
}

// ============================================================================
// T2: x pass. PB row pairs per block; each pair of rows (l, l+1) of a field is
// carried by one complex line (row l in .x, row l+1 in .y after the transform).
// B layout: [pslot][l/2][kx][l%2] (the two rows of a pair interleaved, so that the z pass
// reads a few columns of a row pair as one contiguous run); pslot = slot*4 + p (u levels),
// nuI*4 + (slot-nuI)*2 + p (v).
// capture (optional): physical velocities of selected levels, [cap][f][l][m].
// ============================================================================
// x pass: one row pair per block (FP32) in 4 warps: a Stockham pass over the few lines
// of a block then spreads evenly over the threads (the fastest of a sweep at C1)
#ifndef LH_XPASS_THREADS
#define LH_XPASS_THREADS 128
#endif
template <typename T, int N>
__global__ void __launch_bounds__(LH_XPASS_THREADS) k_xpass_nl(const typename C2<T>::t *__restrict__ A,
                                                   typename C2<T>::t *__restrict__ B, Geo g,
                                                   const typename C2<T>::t *__restrict__ twx, int doCFL,
                                                   DevScalars *sc, const int *__restrict__ capslot,
                                                   T *__restrict__ cap) {
  typedef typename C2<T>::t V;
  constexpr int PB = pb_xpass<V>(N);
  constexpr int G1 = N, H = N / 2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int G2 = g.G2, N1h = g.N1h;
  V *b0 = reinterpret_cast<V *>(smem_raw);
  V *b1 = b0 + 4 * PB * G1;
  const int slot = blockIdx.y;
  const bool isU = slot < g.nuI;
  const int q = slot_level(g, slot, isU);
  const int l0 = blockIdx.x * PB * 2;
  const int npairs = min(PB, (G2 - l0) / 2);
  const size_t fstride = (size_t)G2 * N1h;
  const V *Af = A + (size_t)slot * 3 * fstride;
  // gather Hermitian-completed lines of the 3 fields: line f*PB + pb. One work item per
  // retained x-mode k writes element k (a + i b) and element G1 - k (conj(a) + i conj(b));
  // elements N1h .. G1 - N1h (the dealiasing band) are zero. N1 = 2 (Ngal1 / 3) (lh_create
  // checks it), so N1h = G1 / 3 + 1 is a compile-time constant here.
  constexpr int NK = G1 / 3 + 1, NZ = G1 - 2 * NK + 1;
  static_assert(NK <= H, "retained x-modes below the Nyquist index");
  for (int idx = threadIdx.x; idx < 3 * PB * NK; idx += blockDim.x) {
    const int line = idx / NK, k = idx - line * NK;
    const int f = line / PB, pb = line - f * PB;
    V zd = czero<V>(), zc = czero<V>();
    if (pb < npairs) {
      const int l = l0 + 2 * pb;
      V a = Af[f * fstride + (size_t)l * NK + k];
      V b = Af[f * fstride + (size_t)(l + 1) * NK + k];
      if (k == 0) { a.y = 0; b.y = 0; }
      zd.x = a.x - b.y; zd.y = a.y + b.x;   // a + i b
      zc.x = a.x + b.y; zc.y = -a.y + b.x;  // conj(a) + i conj(b)
    }
    b0[line * G1 + k] = zd;
    if (k > 0) b0[line * G1 + G1 - k] = zc;
  }
  for (int idx = threadIdx.x; idx < 3 * PB * NZ; idx += blockDim.x) {
    const int line = idx / NZ, m = idx - line * NZ;
    b0[line * G1 + NK + m] = czero<V>();
  }
  __syncthreads();
  V *res = line_fft<true, N, 3 * PB, false>(b0, b1, twx);
  V *oth = (res == b0) ? b1 : b0;
  if (capslot) {
    const int cs = capslot[slot];
    if (cs >= 0) {
      for (int idx = threadIdx.x; idx < 3 * PB * G1; idx += blockDim.x) {
        const int line = idx / G1, m = idx - line * G1;
        const int f = line / PB, pb = line - f * PB;
        if (pb >= npairs) continue;
        const int l = l0 + 2 * pb;
        T *cp = cap + ((size_t)cs * 3 + f) * (size_t)G2 * G1;
        const V z = res[idx];
        cp[(size_t)l * G1 + m] = z.x;
        cp[(size_t)(l + 1) * G1 + m] = z.y;
      }
    }
  }
  T m1 = 0, m2 = 0, m3 = 0;
  const T thv = isU ? (T)0 : (sizeof(T) == 8 ? (T)g.thv[q] : (T)g.thvf[q]);
  for (int idx = threadIdx.x; idx < PB * G1; idx += blockDim.x) {
    const int pb = idx / G1, m = idx - pb * G1;
    const V u = res[(0 * PB + pb) * G1 + m], v = res[(1 * PB + pb) * G1 + m], w = res[(2 * PB + pb) * G1 + m];
    const bool valid = pb < npairs;
    if (isU) {
      V p0, p1, p2, p3;
      p0.x = u.x * u.x; p0.y = u.y * u.y;
      p1.x = u.x * w.x; p1.y = u.y * w.y;
      p2.x = v.x * v.x; p2.y = v.y * v.y;
      p3.x = w.x * w.x; p3.y = w.y * w.y;
      oth[(0 * PB + pb) * G1 + m] = p0;
      oth[(1 * PB + pb) * G1 + m] = p1;
      oth[(2 * PB + pb) * G1 + m] = p2;
      oth[(3 * PB + pb) * G1 + m] = p3;
      if (valid && doCFL) {
        m1 = nmax(m1, nmax(fabs(u.x), fabs(u.y)));
        m3 = nmax(m3, nmax(fabs(w.x), fabs(w.y)));
      }
    } else {
      V p0, p1;
      p0.x = u.x * v.x; p0.y = u.y * v.y;
      p1.x = w.x * v.x; p1.y = w.y * v.y;
      oth[(0 * PB + pb) * G1 + m] = p0;
      oth[(1 * PB + pb) * G1 + m] = p1;
      if (valid && doCFL) m2 = nmax(m2, nmax(fabs(v.x), fabs(v.y)) * thv);
    }
  }
  if (doCFL) {
    m1 = warp_max(m1); m2 = warp_max(m2); m3 = warp_max(m3);
    if ((threadIdx.x & 31) == 0) {
      if (isU) { atomic_max_pos(&sc->u1m, to_d(m1)); atomic_max_pos(&sc->u3m, to_d(m3)); }
      else atomic_max_pos(&sc->u2m, to_d(m2));
    }
  }
  __syncthreads();
  V *pres = isU ? line_fft<false, N, 4 * PB, false>(oth, res, twx) : line_fft<false, N, 2 * PB, false>(oth, res, twx);
  const int nprod = isU ? 4 : 2;
  const T s1 = (T)1 / (T)G1;
  const int pbase = isU ? slot * 4 : g.nuI * 4 + (slot - g.nuI) * 2;
  // separate the two rows of each pair, keep kx = 0..N1h-1; kx fastest (coalesced rows).
  // N1 = 2 (Ngal1 / 3) (lh_create checks it), so N1h = G1 / 3 + 1 is a compile-time
  // constant here and the index split needs no runtime division.
  // One work item per x-mode k writes both rows of the pair, which sit next to each other
  // in B (one 16-byte store in the mixed form).
  constexpr int NH = G1 / 3 + 1;
  for (int idx = threadIdx.x; idx < nprod * PB * NH; idx += blockDim.x) {
    const int k = idx % NH;
    const int r2 = idx / NH;
    const int pb = r2 % PB, p = r2 / PB;
    if (pb >= npairs) continue;
    const V *L = pres + (p * PB + pb) * G1;
    const V z = L[k], zc = cconj(L[k == 0 ? 0 : G1 - k]);
    V o0, o1;
    o0.x = (T)0.5 * (z.x + zc.x) * s1; o0.y = (T)0.5 * (z.y + zc.y) * s1;
    o1.x = (T)0.5 * (z.y - zc.y) * s1; o1.y = (T)-0.5 * (z.x - zc.x) * s1;  // -0.5 i (z - zc)
    if (k == 0) { o0.y = 0; o1.y = 0; }
    V *dst = B + (((size_t)(pbase + p) * (G2 / 2) + (l0 >> 1) + pb) * N1h + k) * 2;
    if constexpr (sizeof(T) == 4) {
      *reinterpret_cast<float4 *>(dst) = make_float4(o0.x, o0.y, o1.x, o1.y);
    } else {
      dst[0] = o0;
      dst[1] = o1;
    }
  }
}

// ============================================================================
// Statistics (stats.f90:1-250) of one plane class: the x pass's gather and inverse
// transform, then the plane sums (per level) and the tile-conditioned sums (wall-band
// planes: conddown1/2 at the bottom, condup1/2 mirrored at the top with V's sign
// flipped). u slots hold (u, v interpolated, w), v slots (u interpolated, v, w
// interpolated). Sums: block reduction, one FP64 atomic per quantity and block; the
// conditioned sums add the ntilex tiles of a row in registers first.
// pl: [11][nu] (quantities 0-8 here); cd: [9][ncl][dnz][dnx].
// ============================================================================
template <typename T, int N>
__global__ void __launch_bounds__(NTHR) k_xstats(const typename C2<T>::t *__restrict__ A, Geo g,
                                                 const typename C2<T>::t *__restrict__ twx, double *__restrict__ pl,
                                                 double *__restrict__ cd, int ncl, int dnx, int dnz, int ntx) {
  typedef typename C2<T>::t V;
  constexpr int PB = pb_xpass<V>(N);
  constexpr int G1 = N, H = N / 2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[NTHR / 32][6];
  const int G2 = g.G2, N1h = g.N1h;
  V *b0 = reinterpret_cast<V *>(smem_raw);
  V *b1 = b0 + 4 * PB * G1;
  const int slot = blockIdx.y;
  const bool isU = slot < g.nuI;
  const int q = slot_level(g, slot, isU);
  const int l0 = blockIdx.x * PB * 2;
  const int npairs = min(PB, (G2 - l0) / 2);
  const size_t fstride = (size_t)G2 * N1h;
  const V *Af = A + (size_t)slot * 3 * fstride;
  for (int idx = threadIdx.x; idx < 3 * PB * G1; idx += blockDim.x) {
    const int line = idx / G1, m = idx - line * G1;
    const int f = line / PB, pb = line - f * PB;
    V z = czero<V>();
    if (pb < npairs) {
      const int l = l0 + 2 * pb;
      int k = m;
      bool conjpart = false;
      if (m > H) { k = G1 - m; conjpart = true; }
      if (k < N1h) {
        V a = Af[f * fstride + (size_t)l * N1h + k];
        V b = Af[f * fstride + (size_t)(l + 1) * N1h + k];
        if (k == 0 || k == H) { a.y = 0; b.y = 0; }
        if (!conjpart) { z.x = a.x - b.y; z.y = a.y + b.x; }
        else { z.x = a.x + b.y; z.y = -a.y + b.x; }
      }
    }
    b0[idx] = z;
  }
  __syncthreads();
  const V *res = line_fft<true, N, 3 * PB, false>(b0, b1, twx);
  // plane sums
  double s[6] = {0, 0, 0, 0, 0, 0};
  for (int idx = threadIdx.x; idx < PB * G1; idx += blockDim.x) {
    const int pb = idx / G1, m = idx - pb * G1;
    if (pb >= npairs) continue;
    const V u = res[(0 * PB + pb) * G1 + m], v = res[(1 * PB + pb) * G1 + m], w = res[(2 * PB + pb) * G1 + m];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const double a = to_d(h ? u.y : u.x), b = to_d(h ? v.y : v.x), c = to_d(h ? w.y : w.x);
      if (isU) { s[0] += a; s[1] += a * a; s[2] += c; s[3] += c * c; s[4] += a * b; s[5] += a * c; }
      else { s[0] += b; s[1] += b * b; s[2] += b * c; }
    }
  }
  const int nq = isU ? 6 : 3, qb = isU ? 0 : 6;
  for (int t = 0; t < nq; ++t) {
    double x = s[t];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][t] = x;
  }
  __syncthreads();
  if (threadIdx.x < nq) {
    double x = 0;
    for (int wi = 0; wi < (int)(blockDim.x >> 5); ++wi) x += red[wi][threadIdx.x];
    atomicAdd(&pl[(size_t)(qb + threadIdx.x) * g.nu + q], x);
  }
  // tile-conditioned sums on the wall-band planes
  if (!dnx) return;
  const int j = q - g.dny;
  const int *NN = isU ? g.N4 : g.N3;
  int j1, sv;
  if (j <= NN[1]) { j1 = j - NN[0]; sv = 1; }
  else if (j > NN[2]) { j1 = NN[3] + 1 - j; sv = -1; }
  else return;
  for (int idx = threadIdx.x; idx < 2 * npairs * dnx; idx += blockDim.x) {
    const int rr = idx / dnx, i = idx - rr * dnx;
    const int pb = rr >> 1, h = rr & 1;
    const int k = (l0 + rr) % dnz;
    double c[6] = {0, 0, 0, 0, 0, 0};
    for (int ix = 0; ix < ntx; ++ix) {
      const int m = i + dnx * ix;
      const V u = res[(0 * PB + pb) * G1 + m], v = res[(1 * PB + pb) * G1 + m], w = res[(2 * PB + pb) * G1 + m];
      const double a = to_d(h ? u.y : u.x), b = to_d(h ? v.y : v.x) * sv, cc = to_d(h ? w.y : w.x);
      if (isU) { c[0] += a; c[1] += a * a; c[2] += cc; c[3] += cc * cc; c[4] += a * b; c[5] += a * cc; }
      else { c[0] += b; c[1] += b * b; c[2] += b * cc; }
    }
    for (int t = 0; t < nq; ++t)
      atomicAdd(&cd[(((size_t)(qb + t) * ncl + (j1 - 1)) * dnz + k) * dnx + i], c[t]);
  }
}

// ============================================================================
// T3: forward z transforms + der_x/der_z. grid: x = kx group (KB), y = level slot.
// u level: products uu, uw, vv, ww -> N1xz, N3xz, vvc.   v level: uv, wv -> N2xz, uvf, wvf.
// Outputs are complex in the transform precision (TO = T).
// ============================================================================
template <typename T, int N, int NP>
__device__ __forceinline__ void zfwd_body(const typename C2<T>::t *__restrict__ B, const Geo &g,
                                          const typename C2<T>::t *__restrict__ twz, int slot, int q, int pbase,
                                          typename C2<T>::t *o0, typename C2<T>::t *o1, typename C2<T>::t *o2,
                                          typename C2<T>::t *o3, typename C2<T>::t *o4, typename C2<T>::t *o5) {
  typedef typename C2<T>::t V;
  constexpr int KB = kb_zfwd<V>(N);
  constexpr int NL = NP * KB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int N1h = g.N1h, N2 = g.N2;
  const int kx0 = blockIdx.x * KB;
  V *b0 = reinterpret_cast<V *>(smem_raw);
  V *b1 = b0 + 4 * KB * N;
  // line = p*KB + kk; element l at l*NL + line. B holds the rows of a pair next to each
  // other ([product][l/2][kx][l%2]): the KB columns of a row pair are 2*KB contiguous values.
  for (int idx = threadIdx.x; idx < N * NL; idx += blockDim.x) {
    const int h = idx & 1;
    int rest = idx >> 1;
    const int kk = rest % KB;
    rest /= KB;
    const int lp = rest % (N / 2), p = rest / (N / 2);
    const int l = 2 * lp + h, kx = kx0 + kk;
    V z = czero<V>();
    if (kx < N1h) z = B[(((size_t)(pbase + p) * (N / 2) + lp) * N1h + kx) * 2 + h];
    b0[l * NL + p * KB + kk] = z;
  }
  __syncthreads();
  V *res = line_fft<false, N, NL, true>(b0, b1, twz);
  const T s2 = (T)1 / (T)N;
  const size_t off = (size_t)q * g.ncolF;
  for (int idx = threadIdx.x; idx < N2 * KB; idx += blockDim.x) {
    const int r = idx / KB, kk = idx - r * KB, kx = kx0 + kk;
    if (kx >= N1h) continue;
    const int row = prow(g, r);
    const int c = gcol(g, r, kx), rg = grow(g, r);
    const T kxv = sizeof(T) == 8 ? (T)g.k1x[kx] : (T)g.k1xf[kx];
    const T kzv = sizeof(T) == 8 ? (T)g.k1z[rg] : (T)g.k1zf[rg];
    const bool zr = (r == N2 / 2);  // der_x/der_z zero the kz = -N2/2 row
    if (NP == 4) {
      const V uu = cscale(res[row * NL + 0 * KB + kk], s2), uw = cscale(res[row * NL + 1 * KB + kk], s2);
      const V vv = cscale(res[row * NL + 2 * KB + kk], s2), ww = cscale(res[row * NL + 3 * KB + kk], s2);
      V n1 = czero<V>(), n3 = czero<V>();
      if (!zr) {
        n1 = cadd(cimul(kxv, uu), cimul(kzv, uw));
        n3 = cadd(cimul(kxv, uw), cimul(kzv, ww));
      }
      o0[off + c] = n1;  // N1xz
      o2[off + c] = n3;  // N3xz
      o4[off + c] = vv;  // vvc
    } else {
      const V uv = cscale(res[row * NL + 0 * KB + kk], s2), wv = cscale(res[row * NL + 1 * KB + kk], s2);
      V n2 = czero<V>();
      if (!zr) n2 = cadd(cimul(kxv, uv), cimul(kzv, wv));
      o1[off + c] = n2;  // N2xz
      o3[off + c] = uv;  // uvf
      o5[off + c] = wv;  // wvf
    }
  }
}

template <typename T, int N>
__global__ void __launch_bounds__(LH_ZFWD_THREADS) k_zfwd_nl(const typename C2<T>::t *__restrict__ B, Geo g,
                                                  const typename C2<T>::t *__restrict__ twz,
                                                  typename C2<T>::t *__restrict__ N1xz, typename C2<T>::t *__restrict__ N2xz,
                                                  typename C2<T>::t *__restrict__ N3xz, typename C2<T>::t *__restrict__ uvf,
                                                  typename C2<T>::t *__restrict__ vvc, typename C2<T>::t *__restrict__ wvf) {
  const int slot = blockIdx.y;
  const bool isU = slot < g.nuI;
  const int q = slot_level(g, slot, isU);
  const int pbase = isU ? slot * 4 : g.nuI * 4 + (slot - g.nuI) * 2;
  if (isU) zfwd_body<T, N, 4>(B, g, twz, slot, q, pbase, N1xz, N2xz, N3xz, uvf, vvc, wvf);
  else zfwd_body<T, N, 2>(B, g, twz, slot, q, pbase, N1xz, N2xz, N3xz, uvf, vvc, wvf);
}

// ============================================================================
// dt (kRK = 1): dtc_calc + MPI_ALLREDUCE(MIN) + dt = min(2.5 dtv, CFL dtc)
// ============================================================================
__global__ void k_dt(Geo g, DevScalars *sc) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const double u1m = __longlong_as_double((long long)sc->u1m);
  const double u3m = __longlong_as_double((long long)sc->u3m);
  double u2m = __longlong_as_double((long long)sc->u2m);
  if (!(u2m > 1e-6)) u2m = (u2m != u2m) ? u2m : 1e-6;
  const double a = 1.0 / (g.alp * (double)(g.N1 / 2) * u1m);
  const double b = 1.0 / (g.bet * (double)(g.N2 / 2) * u3m);
  const double cv = 1.0 / (u2m * g.dthetavi);
  double d = fmin(a, b);
  d = fmin(d, cv);
  if (a != a || b != b || cv != cv) d = a + b + cv;  // propagate a NaN of any of the three maxima
  sc->dtc = d;
  const double lim = 2.5 * g.dtv, cfl = g.CFL * d;
  const double dt = (cfl != cfl) ? cfl : fmin(lim, cfl);
  sc->dt = dt;
  sc->dti = 1.0 / dt;
  sc->t = sc->t + dt;
  if (!(dt == dt)) sc->status = LH_ENONFINITE;  // the guard fires in the substep that forms dt
}

__global__ void k_reset_cfl(DevScalars *sc) {
  if (threadIdx.x == 0 && blockIdx.x == 0) { sc->u1m = 0ull; sc->u2m = 0ull; sc->u3m = 0ull; }
}

// ============================================================================
// Helmholtz u and w (shared matrix), one thread per column.
// Levels q = 0 .. nu-1 (ghosts at 0 and nu-1). For interior q the right-hand side
// is u + dt * du with du = RHS0 (laplacian, -cRK Nu_old, -dRK grad p, -dRK mpgx on
// (0,0)) - gRK Nu_new, Nu_new = N_xz + d/dy(uv or wv); Nu_new replaces Nu.
// The forward sweep stores y in u and the upper factor in `a3s`; the backward
// sweep writes the solution in place. At immersed-boundary levels du is read from
// `duib` (assembled and forced beforehand) instead of being formed here.
// ============================================================================
template <typename VN>
__device__ __forceinline__ double2 ld2(const VN &v) { return make_double2((double)v.x, (double)v.y); }

template <typename TN>
__global__ void __launch_bounds__(NTHR) k_helm_uw(double2 *__restrict__ u1, double2 *__restrict__ u3,
                                                  double2 *__restrict__ Nu1, double2 *__restrict__ Nu3,
                                                  const typename C2<TN>::t *__restrict__ N1xz, const typename C2<TN>::t *__restrict__ N3xz,
                                                  const typename C2<TN>::t *__restrict__ uvf, const typename C2<TN>::t *__restrict__ wvf,
                                                  const double2 *__restrict__ p, double *__restrict__ a3s, Geo g,
                                                  const DevScalars *__restrict__ sc, int kRK,
                                                  const int *__restrict__ ibslot_u, const double2 *__restrict__ duib) {
  const int vc = blockIdx.x * blockDim.x + threadIdx.x;
  const int nc = g.ncol;
  if (vc >= g.nvc) return;
  int c, bd;
  vcol_of(g, vc, c, bd);
  const int qlo = g.bq[bd][0], qhi = g.bq[bd][1];
  const int r = c / g.N1h, kx = c - r * g.N1h;
  const double k2x = g.k2x[kx], k2z = g.k2z[r];
  const double C1 = g.aRK[kRK - 1] / g.Re, C2 = -g.cRK[kRK - 1], dR = g.dRK[kRK - 1];
  const double G = -g.gRK[kRK - 1];
  const double dt = sc->dt;
  const double beta = g.bRK[kRK - 1] * dt / g.Re;
  const double C3x = -dR * g.k1x[kx], C3z = -dR * g.k1z[r];  // imaginary parts of -dRK*k1F
  const double mp = (c == 0) ? -dR * sc->mpgx : 0.0;
  const int nu = g.nu;
  const double *d0 = g.d2u, *d1 = g.d2u + nu, *d2 = g.d2u + 2 * nu;
  // first row: [1, gw(b,1)], rhs 0
  double a3raw = g.gw[bd][0];
  double a2p = 1.0;  // 1/a2(0)
  double2 y1 = czero<double2>(), y3 = czero<double2>();
  const size_t o0 = (size_t)qlo * nc + c;
  double2 um1 = u1[o0], u0 = u1[o0 + nc];
  double2 wm1 = u3[o0], w0 = u3[o0 + nc];
  u1[o0] = y1;
  u3[o0] = y3;
  double2 uvm = ld2(uvf[o0]), wvm = ld2(wvf[o0]);
  for (int q = qlo + 1; q <= qhi - 1; ++q) {
    const size_t o = (size_t)q * nc + c;
    const double2 up1 = u1[o + nc], wp1 = u3[o + nc];
    const double2 uvq = ld2(uvf[o]), wvq = ld2(wvf[o]);
    double2 du1, du3;
    const int ibs = ibslot_u ? ibslot_u[q] : -1;
    if (ibs < 0) {
      const double a = d0[q], dg = (k2x + k2z) + d1[q], cc = d2[q];
      double2 L1, L3;
      L1.x = (a * um1.x + dg * u0.x) + cc * up1.x; L1.y = (a * um1.y + dg * u0.y) + cc * up1.y;
      L3.x = (a * wm1.x + dg * w0.x) + cc * wp1.x; L3.y = (a * wm1.y + dg * w0.y) + cc * wp1.y;
      const double2 pj = p[(size_t)(q - 1) * nc + c];
      const double2 no1 = Nu1[o], no3 = Nu3[o];
      du1.x = (C1 * L1.x + C2 * no1.x) + (-C3x * pj.y);
      du1.y = (C1 * L1.y + C2 * no1.y) + (C3x * pj.x);
      du3.x = (C1 * L3.x + C2 * no3.x) + (-C3z * pj.y);
      du3.y = (C1 * L3.y + C2 * no3.y) + (C3z * pj.x);
      du1.x += mp;
      const double th = g.thu[q];
      const double2 x1 = ld2(N1xz[o]), x3 = ld2(N3xz[o]);
      double2 n1, n3;
      n1.x = x1.x + (uvq.x - uvm.x) * th * g.dd; n1.y = x1.y + (uvq.y - uvm.y) * th * g.dd;
      n3.x = x3.x + (wvq.x - wvm.x) * th * g.dd; n3.y = x3.y + (wvq.y - wvm.y) * th * g.dd;
      Nu1[o] = n1;
      Nu3[o] = n3;
      du1.x = du1.x + G * n1.x; du1.y = du1.y + G * n1.y;
      du3.x = du3.x + G * n3.x; du3.y = du3.y + G * n3.y;
    } else {
      du1 = duib[((size_t)ibs * 3 + 0) * nc + c];
      du3 = duib[((size_t)ibs * 3 + 2) * nc + c];
    }
    double2 rhs1, rhs3;
    rhs1.x = u0.x + dt * du1.x; rhs1.y = u0.y + dt * du1.y;
    rhs3.x = w0.x + dt * du3.x; rhs3.y = w0.y + dt * du3.y;
    const double a1 = -beta * d0[q];
    const double a2 = 1.0 - beta * ((d1[q] + k2x) + k2z);
    const double a3p = a3raw * a2p;  // a3'(q-1)
    a3s[(size_t)(q - 1) * nc + c] = a3p;
    a2p = 1.0 / (a2 - a1 * a3p);
    y1.x = (rhs1.x - a1 * y1.x) * a2p; y1.y = (rhs1.y - a1 * y1.y) * a2p;
    y3.x = (rhs3.x - a1 * y3.x) * a2p; y3.y = (rhs3.y - a1 * y3.y) * a2p;
    u1[o] = y1;
    u3[o] = y3;
    a3raw = -beta * d2[q];
    um1 = u0; u0 = up1; wm1 = w0; w0 = wp1;
    uvm = uvq; wvm = wvq;
  }
  {  // last row: [gw(b,2), 1], rhs 0
    const int q = qhi;
    const double a1 = g.gw[bd][1];
    const double a3p = a3raw * a2p;
    a3s[(size_t)(q - 1) * nc + c] = a3p;
    a2p = 1.0 / (1.0 - a1 * a3p);
    y1.x = (0.0 - a1 * y1.x) * a2p; y1.y = (0.0 - a1 * y1.y) * a2p;
    y3.x = (0.0 - a1 * y3.x) * a2p; y3.y = (0.0 - a1 * y3.y) * a2p;
    u1[(size_t)q * nc + c] = y1;
    u3[(size_t)q * nc + c] = y3;
  }
  double2 x1 = y1, x3 = y3;
  for (int q = qhi - 1; q >= qlo; --q) {
    const size_t o = (size_t)q * nc + c;
    const double a3p = a3s[o];
    const double2 yy1 = u1[o], yy3 = u3[o];
    x1.x = yy1.x - a3p * x1.x; x1.y = yy1.y - a3p * x1.y;
    x3.x = yy3.x - a3p * x3.x; x3.y = yy3.y - a3p * x3.y;
    u1[o] = x1;
    u3[o] = x3;
  }
}

// ============================================================================
// Helmholtz v, one thread per column. Levels q = 0 .. nv-1 (walls at both ends).
// ============================================================================
template <typename TN>
__global__ void __launch_bounds__(NTHR) k_helm_v(double2 *__restrict__ u2, double2 *__restrict__ Nu2,
                                                 const typename C2<TN>::t *__restrict__ N2xz, const typename C2<TN>::t *__restrict__ vvc,
                                                 const double2 *__restrict__ p, double *__restrict__ a3s, Geo g,
                                                 const DevScalars *__restrict__ sc, int kRK,
                                                 const int *__restrict__ ibslot_v, const double2 *__restrict__ duib) {
  const int vc = blockIdx.x * blockDim.x + threadIdx.x;
  const int nc = g.ncol;
  if (vc >= g.nvc) return;
  int c, bd;
  vcol_of(g, vc, c, bd);
  const int qlo = g.bq[bd][2], qhi = g.bq[bd][3];
  const int r = c / g.N1h, kx = c - r * g.N1h;
  const double k2x = g.k2x[kx], k2z = g.k2z[r];
  const double C1 = g.aRK[kRK - 1] / g.Re, C2 = -g.cRK[kRK - 1], dR = g.dRK[kRK - 1];
  const double G = -g.gRK[kRK - 1];
  const double dt = sc->dt;
  const double beta = g.bRK[kRK - 1] * dt / g.Re;
  const int nv = g.nv;
  const double *d0 = g.d2v, *d1 = g.d2v + nv, *d2 = g.d2v + 2 * nv;
  double a3raw = 0.0, a2p = 1.0;
  double2 y = czero<double2>();
  const size_t o0 = (size_t)qlo * nc + c;
  double2 vm1 = u2[o0], v0 = u2[o0 + nc];
  u2[o0] = y;
  double2 vvq = ld2(vvc[o0 + nc]);  // vv at u level q (interior starts at qlo + 1)
  for (int q = qlo + 1; q <= qhi - 1; ++q) {
    const size_t o = (size_t)q * nc + c;
    const double2 vp1 = u2[o + nc];
    const double2 vvp = ld2(vvc[o + nc]);  // vv at u level q+1
    double2 du;
    const int ibs = ibslot_v ? ibslot_v[q] : -1;
    if (ibs < 0) {
      const double a = d0[q], dg = (k2x + k2z) + d1[q], cc = d2[q];
      double2 L;
      L.x = (a * vm1.x + dg * v0.x) + cc * vp1.x; L.y = (a * vm1.y + dg * v0.y) + cc * vp1.y;
      const double C3 = -dR * g.dd * g.thv[q];
      const double2 pp = p[(size_t)q * nc + c], pm = p[(size_t)(q - 1) * nc + c];
      const double2 no = Nu2[o];
      du.x = (C1 * L.x + C2 * no.x) + C3 * (pp.x - pm.x);
      du.y = (C1 * L.y + C2 * no.y) + C3 * (pp.y - pm.y);
      const double th = g.thv[q];
      const double2 x2 = ld2(N2xz[o]);
      double2 n2;
      n2.x = x2.x + (vvp.x - vvq.x) * th * g.dd; n2.y = x2.y + (vvp.y - vvq.y) * th * g.dd;
      Nu2[o] = n2;
      du.x = du.x + G * n2.x; du.y = du.y + G * n2.y;
    } else {
      du = duib[((size_t)ibs * 3 + 1) * nc + c];
    }
    double2 rhs;
    rhs.x = v0.x + dt * du.x; rhs.y = v0.y + dt * du.y;
    const double a1 = -beta * d0[q];
    const double a2 = 1.0 - beta * ((d1[q] + k2x) + k2z);
    const double a3p = a3raw * a2p;
    a3s[(size_t)(q - 1) * nc + c] = a3p;
    a2p = 1.0 / (a2 - a1 * a3p);
    y.x = (rhs.x - a1 * y.x) * a2p; y.y = (rhs.y - a1 * y.y) * a2p;
    u2[o] = y;
    a3raw = -beta * d2[q];
    vm1 = v0; v0 = vp1; vvq = vvp;
  }
  {
    const int q = qhi;
    const double a3p = a3raw * a2p;
    a3s[(size_t)(q - 1) * nc + c] = a3p;
    a2p = 1.0 / (1.0 - 0.0 * a3p);
    y.x = (0.0 - 0.0 * y.x) * a2p; y.y = (0.0 - 0.0 * y.y) * a2p;
    u2[(size_t)q * nc + c] = y;
  }
  double2 x = y;
  for (int q = qhi - 1; q >= qlo; --q) {
    const size_t o = (size_t)q * nc + c;
    const double a3p = a3s[o];
    const double2 yy = u2[o];
    x.x = yy.x - a3p * x.x; x.y = yy.y - a3p * x.y;
    u2[o] = x;
  }
}

// ============================================================================
// Mixed form of the Helmholtz solves: the same equations written for the
// increment d = u_new - u, (I - beta L) d = dt du + beta L(u), with the BC rows
// d(0) + gw1 d(1) = -(u(0) + gw1 u(1)) (and the top row alike). d is small, so
// the right-hand side, the factorisation and both sweeps run in FP32; L(u) is
// formed from FP64 neighbour differences (u(j+-1) - u(j)); u_new = u + d in FP64.
// ============================================================================
__device__ __forceinline__ float2 f2d(double2 a) { return make_float2((float)a.x, (float)a.y); }
__device__ __forceinline__ float2 f2sub(double2 a, double2 b) { return make_float2((float)(a.x - b.x), (float)(a.y - b.y)); }

// Backward sweep of the mixed-form solves: x(q) = y(q) - a3'(q) x(q+1), u(q) += x(q) for
// q = qhi-1 .. qlo, with ys(q) = (y(q), a3'(q)). The loads of level q are issued
// D levels ahead, before the stores of the levels in between (D = 0: a plain loop).
template <int D>
__device__ __forceinline__ void back_sweep_mx(double *__restrict__ u, const float2 *__restrict__ ys, size_t lstride,
                                              size_t ci, int qlo, int qhi, float x) {
  if constexpr (D == 0) {
#pragma unroll 4
    for (int q = qhi - 1; q >= qlo; --q) {
      const size_t e = (size_t)q * lstride + ci;
      const float2 ya = ys[e];
      x = ya.x - ya.y * x;
      u[e] = u[e] + f2d_alu(x);
    }
    return;
  } else {
  float2 bys[D];
  double bu[D];
#pragma unroll
  for (int s_ = 0; s_ < D; ++s_) {
    const int q = qhi - 1 - s_;
    if (q >= qlo) { const size_t e = (size_t)q * lstride + ci; bys[s_] = ys[e]; bu[s_] = u[e]; }
  }
  for (int qb = qhi - 1; qb >= qlo; qb -= D) {
#pragma unroll
    for (int s_ = 0; s_ < D; ++s_) {
      const int q = qb - s_;
      if (q < qlo) break;
      const float2 ya = bys[s_];
      const double uq = bu[s_];
      if (q - D >= qlo) { const size_t en = (size_t)(q - D) * lstride + ci; bys[s_] = ys[en]; bu[s_] = u[en]; }
      x = ya.x - ya.y * x;
      u[(size_t)q * lstride + ci] = uq + f2d_alu(x);
    }
  }
  }
}

// ============================================================================
// Mode (0,0) of the mixed form in FP64. The mean flow and its -dRK mpgx forcing live in
// column 0, so its Helmholtz systems are solved in FP64 as the plain form solves them
// (LUsolU_W / LUsolV, tridLU_3D.f90:55-189, right-hand sides of RHS0_u1/u2/u3,
// littleharsh.f90:635-788): FP64 right-hand side, FP64 solve, the column's previous
// nonlinear term kept in FP64. Only the transforms' products (X, Fl) are the form's FP32
// values. k = 0, so there are no i*k couplings and the real and imaginary parts are six
// independent real systems (u, w, v x 2 parts): one block each, rows built in parallel and
// solved by parallel cyclic reduction (log2(levels) steps) so that the column costs a few
// microseconds instead of a serial FP64 recurrence over the levels. The mixed solve
// kernels skip column 0.
// Scalar views as the mixed kernels': element (q, col, part) at (q*ncol + col)*2 + part.
// nuo: the previous nonlinear term of the column, [u re, u im, w re, w im, v re, v im][nu].
// Shared memory: 8 (nu + 1) doubles.
// ============================================================================
__device__ __forceinline__ int fw2f(int fw) { return fw == 0 ? 0 : (fw == 1 ? 2 : 1); }
__global__ void __launch_bounds__(512) k_helm00_pcr(double *__restrict__ u1, double *__restrict__ u3,
                                                    double *__restrict__ u2, const float *__restrict__ N1xz,
                                                    const float *__restrict__ N3xz, const float *__restrict__ N2xz,
                                                    const float *__restrict__ uvf, const float *__restrict__ wvf,
                                                    const float *__restrict__ vvc, const double *__restrict__ p,
                                                    const float2 *__restrict__ duib, const int *__restrict__ ibslot_u,
                                                    const int *__restrict__ ibslot_v, Geo g,
                                                    const DevScalars *__restrict__ sc, int kRK,
                                                    double *__restrict__ nuo_all) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int fw = blockIdx.x >> 1, part = blockIdx.x & 1;  // fw 0: u, 1: w, 2: v
  const bool isv = fw == 2;
  const int qlo = isv ? g.bq[1][2] : g.bq[1][0], qhi = isv ? g.bq[1][3] : g.bq[1][1];
  const int n = qhi - qlo + 1, ny = isv ? g.nv : g.nu;
  double *A = reinterpret_cast<double *>(smem_raw), *B = A + n, *Cc = B + n, *D = Cc + n;
  double *A2 = D + n, *B2 = A2 + n, *C2b = B2 + n, *D2 = C2b + n;
  const size_t ls = (size_t)g.ncol * 2;
  double *u = fw == 0 ? u1 : (fw == 1 ? u3 : u2);
  const float *X = fw == 0 ? N1xz : (fw == 1 ? N3xz : N2xz);
  const float *Fl = fw == 0 ? uvf : (fw == 1 ? wvf : vvc);
  const int *ibslot = isv ? ibslot_v : ibslot_u;
  double *nuo = nuo_all + (size_t)blockIdx.x * g.nu;
  const double *d2 = isv ? g.d2v : g.d2u;
  const double dt = sc->dt;
  const double C1 = g.aRK[kRK - 1] / g.Re, C2 = -g.cRK[kRK - 1], dR = g.dRK[kRK - 1], G = -g.gRK[kRK - 1];
  const double beta = g.bRK[kRK - 1] * dt / g.Re;
  const double mp = (fw == 0 && part == 0) ? -dR * sc->mpgx : 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int q = qlo + i;
    double a, b, c, d;
    if (q == qlo || q == qhi) {  // boundary rows: [1, gw(b,1)] / [gw(b,2), 1] (u, w); v = 0 (v)
      a = 0.0; b = 1.0; c = 0.0; d = 0.0;
      if (!isv) { if (q == qlo) c = g.gw[1][0]; else a = g.gw[1][1]; }
    } else {
      const size_t e = q * ls + part;
      const double um = u[e - ls], u0 = u[e], up = u[e + ls];
      const double d0q = d2[q], d1q = d2[ny + q], d2q = d2[2 * ny + q];
      const int ibs = ibslot ? ibslot[q] : -1;
      double du;
      if (ibs < 0) {
        const double L = (d0q * um + d1q * u0) + d2q * up;
        double nq, rest;
        if (!isv) {
          nq = (double)X[e] + ((double)Fl[e] - (double)Fl[e - ls]) * g.thu[q] * g.dd;
          rest = mp;
        } else {
          nq = (double)X[e] + ((double)Fl[e + ls] - (double)Fl[e]) * g.thv[q] * g.dd;
          rest = (-dR * g.dd * g.thv[q]) * (p[e] - p[e - ls]);
        }
        du = ((C1 * L + C2 * nuo[q]) + rest) + G * nq;
        nuo[q] = nq;
      } else {
        const float2 di = duib[((size_t)ibs * 3 + fw2f(fw)) * g.ncol];
        du = f2d_alu(part ? di.y : di.x);
      }
      a = -beta * d0q; b = 1.0 - beta * d1q; c = -beta * d2q;
      d = u0 + dt * du;
    }
    A[i] = a; B[i] = b; Cc[i] = c; D[i] = d;
  }
  __syncthreads();
  for (int st = 1; st < n; st *= 2) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const int im = i - st, ip = i + st;
      double a = 0.0, b = B[i], c = 0.0, d = D[i];
      if (im >= 0) {
        const double al = -A[i] / B[im];
        a = al * A[im];
        b += al * Cc[im];
        d += al * D[im];
      }
      if (ip < n) {
        const double ga = -Cc[i] / B[ip];
        c = ga * Cc[ip];
        b += ga * A[ip];
        d += ga * D[ip];
      }
      A2[i] = a; B2[i] = b; C2b[i] = c; D2[i] = d;
    }
    __syncthreads();
    double *t;
    t = A; A = A2; A2 = t;
    t = B; B = B2; B2 = t;
    t = Cc; Cc = C2b; C2b = t;
    t = D; D = D2; D2 = t;
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) u[(qlo + i) * ls + part] = D[i] / B[i];
}

// cp.async copies from global to shared memory (8 and 4 bytes), their commit groups and waits
__device__ __forceinline__ void cpa8(void *dst, const void *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cpa4(void *dst, const void *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cpa_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ __forceinline__ void cpa_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// ============================================================================
// Mixed-form solves with one lane per (column, real/imaginary part): the matrix
// is real, so the two parts are independent systems; each lane repeats the FP32
// factorisation. Scalar views: element (q, col, part) at (q*ncol + col)*2 + part.
// ys2 holds (y(q), upper factor(q)) per lane.
// k_helm_u_mx2: one field (u when F == 0, w when F == 2) per launch row (blockIdx.y).
// ============================================================================
__global__ void __launch_bounds__(NTHR) k_helm_u_mx2(double *__restrict__ u1, double *__restrict__ u3,
                                                     float *__restrict__ Nu1, float *__restrict__ Nu3,
                                                     const float *__restrict__ N1xz, const float *__restrict__ N3xz,
                                                     const float *__restrict__ uvf, const float *__restrict__ wvf,
                                                     const double2 *__restrict__ p, float2 *__restrict__ ys2, Geo g,
                                                     const DevScalars *__restrict__ sc, int kRK,
                                                     const int *__restrict__ ibslot_u, const float2 *__restrict__ duib) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int vc = tid >> 1, part = tid & 1;
  const int nc = g.ncol;
  if (vc >= g.nvc) return;
  int c, bd;
  vcol_of(g, vc, c, bd);
  const int qlo = g.bq[bd][0], qhi = g.bq[bd][1];
  const int fw = blockIdx.y;  // 0: u, 1: w
  double *u = fw ? u3 : u1;
  float *Nu = fw ? Nu3 : Nu1;
  const float *X = fw ? N3xz : N1xz;
  const float *Fl = fw ? wvf : uvf;
  if (c == 0) return;  // mode (0,0): k_helm00_pcr (FP64)
  float2 *ys = ys2 + (size_t)fw * g.nu * nc * 2;
  const int r = c / g.N1h, kx = c - r * g.N1h;
  const float k2f = (float)(g.k2x[kx] + g.k2z[r]);
  const float C1 = (float)(g.aRK[kRK - 1] / g.Re), C2 = (float)(-g.cRK[kRK - 1]);
  const double dR = g.dRK[kRK - 1];
  const float G = (float)(-g.gRK[kRK - 1]);
  const double dt = sc->dt;
  const float dtf = (float)dt;
  const float beta = (float)(g.bRK[kRK - 1] * dt / g.Re);
  const float C3 = (float)(-dR * (fw ? g.k1z[r] : g.k1x[kx]));
  const float dd = (float)g.dd;
  const int nu = g.nu;
  const double gw1 = g.gw[bd][0], gw2 = g.gw[bd][1];
  const size_t lstride = (size_t)nc * 2;
  const size_t ci = (size_t)c * 2 + part;
  const size_t e0 = (size_t)qlo * lstride + ci;
  double um = u[e0], u0 = u[e0 + lstride];
  float y = d2f_alu(-(um + gw1 * u0));  // first row
  // um - u0 at level q is -(up1 - u0) of level q-1: one FP64 difference per level
  float fdm = d2f_alu(um - u0);
  float yprev = y;
  float a3raw = (float)gw1, a2p = 1.f;
  float flm = Fl[e0];
  // the inputs of level q are loaded LH_PF_HU levels ahead of their use, before the
  // stores of the levels in between (the sweep's own stores would otherwise order them)
#if LH_PF_HU > 0
  constexpr int D = LH_PF_HU;
  double fu[D];
  float ffl[D], fa[D], fb[D], fc[D], fsd[D], fth[D], fnu[D], fx[D];
  int fib[D];
  double fp[D];                       // the other part of p: i*C3*p = (-C3 p.y, C3 p.x)
  const double *pc = reinterpret_cast<const double *>(p);
#define HU_FETCH(s_, qq_)                                                        \
  {                                                                              \
    const int q_ = (qq_);                                                        \
    const size_t e_ = (size_t)q_ * lstride + ci;                                 \
    fu[s_] = u[e_ + lstride];                                                    \
    ffl[s_] = Fl[e_];                                                            \
    fa[s_] = g.d2uf[q_]; fb[s_] = g.d2uf[nu + q_]; fc[s_] = g.d2uf[2 * nu + q_]; \
    fsd[s_] = g.sdgu[q_]; fth[s_] = g.thuf[q_];                                  \
    fib[s_] = ibslot_u ? ibslot_u[q_] : -1;                                      \
    fp[s_] = pc[((size_t)(q_ - 1) * nc + c) * 2 + (part ^ 1)];                   \
    fnu[s_] = Nu[e_]; fx[s_] = X[e_];                                            \
  }
#pragma unroll
  for (int s_ = 0; s_ < D; ++s_)
    if (qlo + 1 + s_ <= qhi - 1) HU_FETCH(s_, qlo + 1 + s_)
  for (int qb = qlo + 1; qb <= qhi - 1; qb += D) {
#pragma unroll
    for (int s_ = 0; s_ < D; ++s_) {
      const int q = qb + s_;
      if (q > qhi - 1) break;
      const size_t e = (size_t)q * lstride + ci;
      const double up1 = fu[s_];
      const float flq = ffl[s_], a = fa[s_], b = fb[s_], cc = fc[s_], sdg = fsd[s_] + k2f, thq = fth[s_];
      const float nuq = fnu[s_], xq = fx[s_];
      const int ibs = fib[s_];
      const double po = fp[s_];
      if (q + D <= qhi - 1) HU_FETCH(s_, q + D)
      const float fdp = d2f_alu(up1 - u0);
      const float L = a * fdm + cc * fdp + sdg * d2f_alu(u0);
      fdm = -fdp;
      float du;
      if (ibs < 0) {
        const float pt = part ? d2f_alu(po) : -d2f_alu(po);
        du = (C1 * L + C2 * nuq) + C3 * pt;
        const float n = xq + (flq - flm) * thq * dd;
        Nu[e] = n;
        du += G * n;
      } else {
        const float2 di = duib[((size_t)ibs * 3 + (fw ? 2 : 0)) * nc + c];
        du = part ? di.y : di.x;
      }
      const float rr = dtf * du + beta * L;
      const float a1 = -beta * a;
      const float a2 = 1.f - beta * (b + k2f);
      const float a3p = a3raw * a2p;
      ys[(size_t)(q - 1) * lstride + ci] = make_float2(yprev, a3p);
      a2p = 1.f / (a2 - a1 * a3p);
      y = (rr - a1 * y) * a2p;
      yprev = y;
      a3raw = -beta * cc;
      um = u0; u0 = up1;
      flm = flq;
    }
  }
#undef HU_FETCH
#else
#pragma unroll 4
  for (int q = qlo + 1; q <= qhi - 1; ++q) {
    const size_t e = (size_t)q * lstride + ci;
    const double up1 = u[e + lstride];
    const float flq = Fl[e];
    const float a = g.d2uf[q], b = g.d2uf[nu + q], cc = g.d2uf[2 * nu + q];
    const float sdg = g.sdgu[q] + k2f;
    const float fdp = d2f_alu(up1 - u0);
    const float L = a * fdm + cc * fdp + sdg * d2f_alu(u0);
    fdm = -fdp;
    float du;
    const int ibs = ibslot_u ? ibslot_u[q] : -1;
    if (ibs < 0) {
      const double2 pj = p[(size_t)(q - 1) * nc + c];
      const float pt = part ? d2f_alu(pj.x) : -d2f_alu(pj.y);  // i*C3*p: (-C3 p.y, C3 p.x)
      du = (C1 * L + C2 * Nu[e]) + C3 * pt;
      const float n = X[e] + (flq - flm) * g.thuf[q] * dd;
      Nu[e] = n;
      du += G * n;
    } else {
      const float2 di = duib[((size_t)ibs * 3 + (fw ? 2 : 0)) * nc + c];
      du = part ? di.y : di.x;
    }
    const float rr = dtf * du + beta * L;
    const float a1 = -beta * a;
    const float a2 = 1.f - beta * (b + k2f);
    const float a3p = a3raw * a2p;
    ys[(size_t)(q - 1) * lstride + ci] = make_float2(yprev, a3p);
    a2p = 1.f / (a2 - a1 * a3p);
    y = (rr - a1 * y) * a2p;
    yprev = y;
    a3raw = -beta * cc;
    um = u0; u0 = up1;
    flm = flq;
  }
#endif
  {  // last row: gw2 d(n-2) + d(n-1) = -(gw2 u(n-2) + u(n-1))
    const int q = qhi;
    const float a1 = (float)gw2;
    const float rl = d2f_alu(-(gw2 * um + u0));
    const float a3p = a3raw * a2p;
    ys[(size_t)(q - 1) * lstride + ci] = make_float2(yprev, a3p);
    a2p = 1.f / (1.f - a1 * a3p);
    y = (rl - a1 * y) * a2p;
    u[(size_t)q * lstride + ci] = u0 + f2d_alu(y);
  }
  back_sweep_mx<LH_PF_HU_BACK>(u, ys, lstride, ci, qlo, qhi, y);
}

__global__ void __launch_bounds__(NTHR) k_helm_v_mx2(double *__restrict__ u2, float *__restrict__ Nu2,
                                                     const float *__restrict__ N2xz, const float *__restrict__ vvc,
                                                     const double *__restrict__ p, float2 *__restrict__ ys, Geo g,
                                                     const DevScalars *__restrict__ sc, int kRK,
                                                     const int *__restrict__ ibslot_v, const float2 *__restrict__ duib) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int vc = tid >> 1, part = tid & 1;
  const int nc = g.ncol;
  if (vc >= g.nvc) return;
  int c, bd;
  vcol_of(g, vc, c, bd);
  if (c == 0) return;  // mode (0,0): k_helm00_pcr (FP64)
  const int qlo = g.bq[bd][2], qhi = g.bq[bd][3];
  const int r = c / g.N1h, kx = c - r * g.N1h;
  const float k2f = (float)(g.k2x[kx] + g.k2z[r]);
  const float C1 = (float)(g.aRK[kRK - 1] / g.Re), C2 = (float)(-g.cRK[kRK - 1]);
  const double dR = g.dRK[kRK - 1];
  const float G = (float)(-g.gRK[kRK - 1]);
  const double dt = sc->dt;
  const float dtf = (float)dt;
  const float beta = (float)(g.bRK[kRK - 1] * dt / g.Re);
  const float dd = (float)g.dd;
  const int nv = g.nv;
  const size_t ci = (size_t)c * 2 + part;
  const size_t lstride = (size_t)nc * 2;
  const size_t e0 = (size_t)qlo * lstride + ci;
  double vm = u2[e0], v0 = u2[e0 + lstride];
  const float dRf = (float)dR;
  float y = d2f_alu(-vm);
  float fdm = d2f_alu(vm - v0);  // carried as -(vp1 - v0) of the level below
  float yprev = y;
  float a3raw = 0.f, a2p = 1.f;
  float vvq = vvc[e0 + lstride];
  constexpr int D = LH_PF_HV > 0 ? LH_PF_HV : 1;
  double fv[D];
  float fvv[D], fa[D], fb[D], fc[D], fsd[D], fth[D], fnu[D], fx[D], fpd[D];
  int fib[D];
#define HV_FETCH(s_, qq_)                                                        \
  {                                                                              \
    const int q_ = (qq_);                                                        \
    const size_t e_ = (size_t)q_ * lstride + ci;                                 \
    fv[s_] = u2[e_ + lstride];                                                   \
    fvv[s_] = vvc[e_ + lstride];                                                 \
    fa[s_] = g.d2vf[q_]; fb[s_] = g.d2vf[nv + q_]; fc[s_] = g.d2vf[2 * nv + q_]; \
    fsd[s_] = g.sdgv[q_]; fth[s_] = g.thvf[q_];                                  \
    fib[s_] = ibslot_v ? ibslot_v[q_] : -1;                                      \
    fpd[s_] = d2f_alu(p[e_]) - d2f_alu(p[e_ - lstride]);                         \
    fnu[s_] = Nu2[e_]; fx[s_] = N2xz[e_];                                        \
  }
#pragma unroll
  for (int s_ = 0; s_ < D; ++s_)
    if (qlo + 1 + s_ <= qhi - 1) HV_FETCH(s_, qlo + 1 + s_)
  for (int qb = qlo + 1; qb <= qhi - 1; qb += D) {
#pragma unroll
    for (int s_ = 0; s_ < D; ++s_) {
      const int q = qb + s_;
      if (q > qhi - 1) break;
      const size_t e = (size_t)q * lstride + ci;
      const double vp1 = fv[s_];
      const float vvp = fvv[s_], a = fa[s_], b = fb[s_], cc = fc[s_], sdg = fsd[s_] + k2f, thq = fth[s_];
      const float nuq = fnu[s_], xq = fx[s_], pd = fpd[s_];
      const int ibs = fib[s_];
      if (q + D <= qhi - 1) HV_FETCH(s_, q + D)
      const float fdp = d2f_alu(vp1 - v0);
      const float L = a * fdm + cc * fdp + sdg * d2f_alu(v0);
      fdm = -fdp;
      float du;
      if (ibs < 0) {
        const float C3 = -dRf * dd * thq;
        du = (C1 * L + C2 * nuq) + C3 * pd;
        const float n = xq + (vvp - vvq) * thq * dd;
        Nu2[e] = n;
        du += G * n;
      } else {
        const float2 di = duib[((size_t)ibs * 3 + 1) * nc + c];
        du = part ? di.y : di.x;
      }
      const float rr = dtf * du + beta * L;
      const float a1 = -beta * a;
      const float a2 = 1.f - beta * (b + k2f);
      const float a3p = a3raw * a2p;
      ys[(size_t)(q - 1) * lstride + ci] = make_float2(yprev, a3p);
      a2p = 1.f / (a2 - a1 * a3p);
      y = (rr - a1 * y) * a2p;
      yprev = y;
      a3raw = -beta * cc;
      vm = v0; v0 = vp1; vvq = vvp;
    }
  }
#undef HV_FETCH
  {  // last row: d(n-1) = -v(n-1)
    const int q = qhi;
    const float a3p = a3raw * a2p;
    ys[(size_t)(q - 1) * lstride + ci] = make_float2(yprev, a3p);
    y = d2f_alu(-v0);
    u2[(size_t)q * lstride + ci] = v0 + f2d_alu(y);
  }
  back_sweep_mx<LH_PF_HV_BACK>(u2, ys, lstride, ci, qlo, qhi, y);
}

// ============================================================================
// The mixed-form solves with their y-columns staged through shared memory (the arithmetic of
// k_helm_u_mx2 / k_helm_v_mx2, so the same results bit for bit): every lane keeps a ring of
// D + 1 levels of its inputs, filled by cp.async copies D levels ahead (into the slot not being
// read), and the per-level coefficient tables sit in shared memory; the backward sweep stages
// (y, upper factor) and the state the same way. Shared memory: 6 nu tables + the ring,
// 24 (D + 1) bytes per thread.
// ============================================================================
template <int D>
__device__ __forceinline__ void back_sweep_staged(double *__restrict__ u, const float2 *__restrict__ ys, size_t lstride,
                                                  size_t ci, int qlo, int qhi, float x, unsigned char *ring, int nt) {
  constexpr int NS = D + 1;
  float2 *ry = reinterpret_cast<float2 *>(ring);          // [NS][nt]
  double *ru = reinterpret_cast<double *>(ring) + NS * nt;  // [NS][nt]
  auto fetch = [&](int q) {
    const int s_ = (qhi - 1 - q) % NS;
    const size_t e = (size_t)q * lstride + ci;
    cpa8(&ry[s_ * nt + threadIdx.x], ys + e);
    cpa8(&ru[s_ * nt + threadIdx.x], u + e);
  };
#pragma unroll
  for (int s_ = 0; s_ < D; ++s_) {
    if (qhi - 1 - s_ >= qlo) fetch(qhi - 1 - s_);
    cpa_commit();
  }
  for (int q = qhi - 1; q >= qlo; --q) {
    cpa_wait<D - 1>();
    const int s_ = (qhi - 1 - q) % NS;
    const float2 ya = ry[s_ * nt + threadIdx.x];
    const double uq = ru[s_ * nt + threadIdx.x];
    if (q - D >= qlo) fetch(q - D);
    cpa_commit();
    x = ya.x - ya.y * x;
    u[(size_t)q * lstride + ci] = uq + f2d_alu(x);
  }
  cpa_wait<0>();
}

template <int D>
__global__ void __launch_bounds__(NTHR) k_helm_u_mx3(double *__restrict__ u1, double *__restrict__ u3,
                                                     float *__restrict__ Nu1, float *__restrict__ Nu3,
                                                     const float *__restrict__ N1xz, const float *__restrict__ N3xz,
                                                     const float *__restrict__ uvf, const float *__restrict__ wvf,
                                                     const double2 *__restrict__ p, float2 *__restrict__ ys2, Geo g,
                                                     const DevScalars *__restrict__ sc, int kRK,
                                                     const int *__restrict__ ibslot_u, const float2 *__restrict__ duib) {
  constexpr int NS = D + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nu = g.nu, nt = blockDim.x;
  float *ta = reinterpret_cast<float *>(smem_raw), *tb = ta + nu, *tc = tb + nu, *tsd = tc + nu, *tth = tsd + nu;
  int *tib = reinterpret_cast<int *>(tth + nu);
  unsigned char *ring = smem_raw + (((size_t)6 * nu * 4 + 15) & ~(size_t)15);
  for (int i = threadIdx.x; i < nu; i += nt) {
    ta[i] = g.d2uf[i]; tb[i] = g.d2uf[nu + i]; tc[i] = g.d2uf[2 * nu + i]; tsd[i] = g.sdgu[i]; tth[i] = g.thuf[i];
    tib[i] = ibslot_u ? ibslot_u[i] : -1;
  }
  __syncthreads();
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int vc = tid >> 1, part = tid & 1;
  const int nc = g.ncol;
  if (vc >= g.nvc) return;
  int c, bd;
  vcol_of(g, vc, c, bd);
  if (c == 0) return;  // mode (0,0): k_helm00_pcr (FP64)
  const int qlo = g.bq[bd][0], qhi = g.bq[bd][1];
  const int fw = blockIdx.y;  // 0: u, 1: w
  double *u = fw ? u3 : u1;
  float *Nu = fw ? Nu3 : Nu1;
  const float *X = fw ? N3xz : N1xz;
  const float *Fl = fw ? wvf : uvf;
  float2 *ys = ys2 + (size_t)fw * g.nu * nc * 2;
  const int r = c / g.N1h, kx = c - r * g.N1h;
  const float k2f = (float)(g.k2x[kx] + g.k2z[r]);
  const float C1 = (float)(g.aRK[kRK - 1] / g.Re), C2 = (float)(-g.cRK[kRK - 1]);
  const double dR = g.dRK[kRK - 1];
  const float G = (float)(-g.gRK[kRK - 1]);
  const double dt = sc->dt;
  const float dtf = (float)dt;
  const float beta = (float)(g.bRK[kRK - 1] * dt / g.Re);
  const float C3 = (float)(-dR * (fw ? g.k1z[r] : g.k1x[kx]));
  const float dd = (float)g.dd;
  const double gw1 = g.gw[bd][0], gw2 = g.gw[bd][1];
  const size_t lstride = (size_t)nc * 2;
  const size_t ci = (size_t)c * 2 + part;
  const size_t e0 = (size_t)qlo * lstride + ci;
  const double *pc = reinterpret_cast<const double *>(p);
  double um = u[e0], u0 = u[e0 + lstride];
  float y = d2f_alu(-(um + gw1 * u0));  // first row
  float fdm = d2f_alu(um - u0);
  float yprev = y;
  float a3raw = (float)gw1, a2p = 1.f;
  float flm = Fl[e0];
  // ring: doubles [NS][2][nt] (u of the level above, p of the other part), floats [NS][3][nt] (Fl, Nu, X)
  double *rd = reinterpret_cast<double *>(ring);
  float *rf = reinterpret_cast<float *>(rd + 2 * NS * nt);
  auto fetch = [&](int q) {
    const int s_ = (q - qlo - 1) % NS;
    const size_t e = (size_t)q * lstride + ci;
    cpa8(&rd[(s_ * 2 + 0) * nt + threadIdx.x], u + e + lstride);
    cpa8(&rd[(s_ * 2 + 1) * nt + threadIdx.x], pc + ((size_t)(q - 1) * nc + c) * 2 + (part ^ 1));
    cpa4(&rf[(s_ * 3 + 0) * nt + threadIdx.x], Fl + e);
    cpa4(&rf[(s_ * 3 + 1) * nt + threadIdx.x], Nu + e);
    cpa4(&rf[(s_ * 3 + 2) * nt + threadIdx.x], X + e);
  };
#pragma unroll
  for (int s_ = 0; s_ < D; ++s_) {
    if (qlo + 1 + s_ <= qhi - 1) fetch(qlo + 1 + s_);
    cpa_commit();
  }
  for (int q = qlo + 1; q <= qhi - 1; ++q) {
    cpa_wait<D - 1>();
    const int s_ = (q - qlo - 1) % NS;
    const size_t e = (size_t)q * lstride + ci;
    const double up1 = rd[(s_ * 2 + 0) * nt + threadIdx.x], po = rd[(s_ * 2 + 1) * nt + threadIdx.x];
    const float flq = rf[(s_ * 3 + 0) * nt + threadIdx.x], nuq = rf[(s_ * 3 + 1) * nt + threadIdx.x],
                xq = rf[(s_ * 3 + 2) * nt + threadIdx.x];
    if (q + D <= qhi - 1) fetch(q + D);
    cpa_commit();
    const float a = ta[q], b = tb[q], cc = tc[q], sdg = tsd[q] + k2f, thq = tth[q];
    const int ibs = tib[q];
    const float fdp = d2f_alu(up1 - u0);
    const float L = a * fdm + cc * fdp + sdg * d2f_alu(u0);
    fdm = -fdp;
    float du;
    if (ibs < 0) {
      const float pt = part ? d2f_alu(po) : -d2f_alu(po);
      du = (C1 * L + C2 * nuq) + C3 * pt;
      const float n = xq + (flq - flm) * thq * dd;
      Nu[e] = n;
      du += G * n;
    } else {
      const float2 di = duib[((size_t)ibs * 3 + (fw ? 2 : 0)) * nc + c];
      du = part ? di.y : di.x;
    }
    const float rr = dtf * du + beta * L;
    const float a1 = -beta * a;
    const float a2 = 1.f - beta * (b + k2f);
    const float a3p = a3raw * a2p;
    ys[(size_t)(q - 1) * lstride + ci] = make_float2(yprev, a3p);
    a2p = 1.f / (a2 - a1 * a3p);
    y = (rr - a1 * y) * a2p;
    yprev = y;
    a3raw = -beta * cc;
    um = u0; u0 = up1;
    flm = flq;
  }
  cpa_wait<0>();
  {  // last row: gw2 d(n-2) + d(n-1) = -(gw2 u(n-2) + u(n-1))
    const int q = qhi;
    const float a1 = (float)gw2;
    const float rl = d2f_alu(-(gw2 * um + u0));
    const float a3p = a3raw * a2p;
    ys[(size_t)(q - 1) * lstride + ci] = make_float2(yprev, a3p);
    a2p = 1.f / (1.f - a1 * a3p);
    y = (rl - a1 * y) * a2p;
    u[(size_t)q * lstride + ci] = u0 + f2d_alu(y);
  }
  __threadfence_block();  // the backward sweep's copies read ys written above by this thread
  back_sweep_staged<D>(u, ys, lstride, ci, qlo, qhi, y, ring, nt);
}

template <int D>
__global__ void __launch_bounds__(NTHR) k_helm_v_mx3(double *__restrict__ u2, float *__restrict__ Nu2,
                                                     const float *__restrict__ N2xz, const float *__restrict__ vvc,
                                                     const double *__restrict__ p, float2 *__restrict__ ys, Geo g,
                                                     const DevScalars *__restrict__ sc, int kRK,
                                                     const int *__restrict__ ibslot_v, const float2 *__restrict__ duib) {
  constexpr int NS = D + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nv = g.nv, nt = blockDim.x;
  float *ta = reinterpret_cast<float *>(smem_raw), *tb = ta + nv, *tc = tb + nv, *tsd = tc + nv, *tth = tsd + nv;
  int *tib = reinterpret_cast<int *>(tth + nv);
  unsigned char *ring = smem_raw + (((size_t)6 * nv * 4 + 15) & ~(size_t)15);
  for (int i = threadIdx.x; i < nv; i += nt) {
    ta[i] = g.d2vf[i]; tb[i] = g.d2vf[nv + i]; tc[i] = g.d2vf[2 * nv + i]; tsd[i] = g.sdgv[i]; tth[i] = g.thvf[i];
    tib[i] = ibslot_v ? ibslot_v[i] : -1;
  }
  __syncthreads();
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int vc = tid >> 1, part = tid & 1;
  const int nc = g.ncol;
  if (vc >= g.nvc) return;
  int c, bd;
  vcol_of(g, vc, c, bd);
  if (c == 0) return;  // mode (0,0): k_helm00_pcr (FP64)
  const int qlo = g.bq[bd][2], qhi = g.bq[bd][3];
  const int r = c / g.N1h, kx = c - r * g.N1h;
  const float k2f = (float)(g.k2x[kx] + g.k2z[r]);
  const float C1 = (float)(g.aRK[kRK - 1] / g.Re), C2 = (float)(-g.cRK[kRK - 1]);
  const double dR = g.dRK[kRK - 1];
  const float G = (float)(-g.gRK[kRK - 1]);
  const double dt = sc->dt;
  const float dtf = (float)dt;
  const float beta = (float)(g.bRK[kRK - 1] * dt / g.Re);
  const float dd = (float)g.dd;
  const size_t ci = (size_t)c * 2 + part;
  const size_t lstride = (size_t)nc * 2;
  const size_t e0 = (size_t)qlo * lstride + ci;
  double vm = u2[e0], v0 = u2[e0 + lstride];
  const float dRf = (float)dR;
  float y = d2f_alu(-vm);
  float fdm = d2f_alu(vm - v0);
  float yprev = y;
  float a3raw = 0.f, a2p = 1.f;
  float vvq = vvc[e0 + lstride];
  float pprev = d2f_alu(p[e0]);  // p of the level below (the pressure difference of level q)
  // ring: doubles [NS][2][nt] (v of the level above, p), floats [NS][3][nt] (vv above, Nu, X)
  double *rd = reinterpret_cast<double *>(ring);
  float *rf = reinterpret_cast<float *>(rd + 2 * NS * nt);
  auto fetch = [&](int q) {
    const int s_ = (q - qlo - 1) % NS;
    const size_t e = (size_t)q * lstride + ci;
    cpa8(&rd[(s_ * 2 + 0) * nt + threadIdx.x], u2 + e + lstride);
    cpa8(&rd[(s_ * 2 + 1) * nt + threadIdx.x], p + e);
    cpa4(&rf[(s_ * 3 + 0) * nt + threadIdx.x], vvc + e + lstride);
    cpa4(&rf[(s_ * 3 + 1) * nt + threadIdx.x], Nu2 + e);
    cpa4(&rf[(s_ * 3 + 2) * nt + threadIdx.x], N2xz + e);
  };
#pragma unroll
  for (int s_ = 0; s_ < D; ++s_) {
    if (qlo + 1 + s_ <= qhi - 1) fetch(qlo + 1 + s_);
    cpa_commit();
  }
  for (int q = qlo + 1; q <= qhi - 1; ++q) {
    cpa_wait<D - 1>();
    const int s_ = (q - qlo - 1) % NS;
    const size_t e = (size_t)q * lstride + ci;
    const double vp1 = rd[(s_ * 2 + 0) * nt + threadIdx.x];
    const float pq = d2f_alu(rd[(s_ * 2 + 1) * nt + threadIdx.x]);
    const float vvp = rf[(s_ * 3 + 0) * nt + threadIdx.x], nuq = rf[(s_ * 3 + 1) * nt + threadIdx.x],
                xq = rf[(s_ * 3 + 2) * nt + threadIdx.x];
    if (q + D <= qhi - 1) fetch(q + D);
    cpa_commit();
    const float a = ta[q], b = tb[q], cc = tc[q], sdg = tsd[q] + k2f, thq = tth[q];
    const int ibs = tib[q];
    const float pd = pq - pprev;
    pprev = pq;
    const float fdp = d2f_alu(vp1 - v0);
    const float L = a * fdm + cc * fdp + sdg * d2f_alu(v0);
    fdm = -fdp;
    float du;
    if (ibs < 0) {
      const float C3 = -dRf * dd * thq;
      du = (C1 * L + C2 * nuq) + C3 * pd;
      const float n = xq + (vvp - vvq) * thq * dd;
      Nu2[e] = n;
      du += G * n;
    } else {
      const float2 di = duib[((size_t)ibs * 3 + 1) * nc + c];
      du = part ? di.y : di.x;
    }
    const float rr = dtf * du + beta * L;
    const float a1 = -beta * a;
    const float a2 = 1.f - beta * (b + k2f);
    const float a3p = a3raw * a2p;
    ys[(size_t)(q - 1) * lstride + ci] = make_float2(yprev, a3p);
    a2p = 1.f / (a2 - a1 * a3p);
    y = (rr - a1 * y) * a2p;
    yprev = y;
    a3raw = -beta * cc;
    vm = v0; v0 = vp1; vvq = vvp;
  }
  cpa_wait<0>();
  {  // last row: d(n-1) = -v(n-1)
    const int q = qhi;
    const float a3p = a3raw * a2p;
    ys[(size_t)(q - 1) * lstride + ci] = make_float2(yprev, a3p);
    y = d2f_alu(-v0);
    u2[(size_t)q * lstride + ci] = v0 + f2d_alu(y);
  }
  __threadfence_block();
  back_sweep_staged<D>(u2, ys, lstride, ci, qlo, qhi, y, ring, nt);
}

// ============================================================================
// flowrate_corr (littleharsh.f90:476-509) on mode (0,0) of u1. The block stages the
// coefficients, the level widths and u(0,0) in `w` (shared memory when it fits,
// else global scratch); thread 0 runs the recurrence and the sums in the
// reference's order; the block applies the correction.
// w: 6*(nn+3) doubles: u11, a1, a2, a3, dy, ur
// ============================================================================
__global__ void k_meanflow(double2 *__restrict__ u1, Geo g, DevScalars *sc, int kRK, double *__restrict__ wg,
                           int use_smem) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nn = g.nn, n = nn + 3, dny = g.dny, nc = g.ncol, nu = g.nu;
  double *w = use_smem ? reinterpret_cast<double *>(smem_raw) : wg;
  double *u11 = w, *a1 = w + n, *a2 = w + 2 * n, *a3 = w + 3 * n, *dy = w + 4 * n, *ur = w + 5 * n;
  __shared__ double gg_sh;
  const double dt = sc->dt;
  const double bdt = -g.dRK[kRK - 1] * dt;
  const double beta = g.bRK[kRK - 1] * dt / g.Re;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    if (j == 0) { a1[j] = 0.0; a2[j] = 1.0; a3[j] = g.gw[1][0]; u11[j] = 0.0; }
    else if (j == nn + 2) { a1[j] = g.gw[1][1]; a2[j] = 1.0; a3[j] = 0.0; u11[j] = 0.0; }
    else {
      a1[j] = -beta * g.d2u[j + dny];
      a2[j] = 1.0 - beta * g.d2u[nu + j + dny];
      a3[j] = -beta * g.d2u[2 * nu + j + dny];
      u11[j] = bdt;
    }
    dy[j] = (j >= 1 && j <= nn + 1) ? (g.yv[j + dny] - g.yv[j - 1 + dny]) : 0.0;
    ur[j] = u1[(size_t)(j + dny) * nc].x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    a2[0] = 1.0 / a2[0];
    for (int j = 1; j < n; ++j) {
      a3[j - 1] = a3[j - 1] * a2[j - 1];
      a2[j] = 1.0 / (a2[j] - a1[j] * a3[j - 1]);
    }
    u11[0] = u11[0] * a2[0];
    for (int j = 1; j < n; ++j) u11[j] = (u11[j] - a1[j] * u11[j - 1]) * a2[j];
    for (int j = n - 2; j >= 0; --j) u11[j] = u11[j] - a3[j] * u11[j + 1];
    double Qx1 = 0.0, Qx0 = 0.0;
    for (int j = 1; j <= nn + 1; ++j) Qx1 = Qx1 + dy[j] * u11[j];
    for (int j = 1; j <= nn + 1; ++j) Qx0 = Qx0 + dy[j] * ur[j];
    const double gg = (sc->QxT - Qx0) / Qx1;
    sc->mpgx = sc->mpgx + gg;
    sc->dgx = gg;
    gg_sh = gg;
  }
  __syncthreads();
  const double gg = gg_sh;
  for (int j = threadIdx.x; j <= nn + 2; j += blockDim.x) u1[(size_t)(j + dny) * nc].x = ur[j] + gg * u11[j];
}

// flowrate_corr with the tridiagonal system solved by parallel cyclic reduction in one
// block (log2(n) steps) instead of k_meanflow's serial recurrence (its FP64 divisions
// were the latency); same system and correction, the solution's rounding differs.
// Shared memory: 8 n doubles (two copies of the four diagonals/rhs).
__global__ void __launch_bounds__(512) k_meanflow_pcr(double2 *__restrict__ u1, Geo g, DevScalars *sc, int kRK) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double gg_sh;
  const int nn = g.nn, n = nn + 3, dny = g.dny, nc = g.ncol, nu = g.nu;
  double *A = reinterpret_cast<double *>(smem_raw), *B = A + n, *Cc = B + n, *D = Cc + n;
  double *A2 = D + n, *B2 = A2 + n, *C2b = B2 + n, *D2 = C2b + n;
  const double dt = sc->dt;
  const double bdt = -g.dRK[kRK - 1] * dt;
  const double beta = g.bRK[kRK - 1] * dt / g.Re;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    if (j == 0) { A[j] = 0.0; B[j] = 1.0; Cc[j] = g.gw[1][0]; D[j] = 0.0; }
    else if (j == nn + 2) { A[j] = g.gw[1][1]; B[j] = 1.0; Cc[j] = 0.0; D[j] = 0.0; }
    else {
      A[j] = -beta * g.d2u[j + dny];
      B[j] = 1.0 - beta * g.d2u[nu + j + dny];
      Cc[j] = -beta * g.d2u[2 * nu + j + dny];
      D[j] = bdt;
    }
  }
  __syncthreads();
  for (int st = 1; st < n; st *= 2) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const int im = i - st, ip = i + st;
      double a = 0.0, b = B[i], c = 0.0, d = D[i];
      if (im >= 0) {
        const double al = -A[i] / B[im];
        a = al * A[im];
        b += al * Cc[im];
        d += al * D[im];
      }
      if (ip < n) {
        const double ga = -Cc[i] / B[ip];
        c = ga * Cc[ip];
        b += ga * A[ip];
        d += ga * D[ip];
      }
      A2[i] = a; B2[i] = b; C2b[i] = c; D2[i] = d;
    }
    __syncthreads();
    double *t;
    t = A; A = A2; A2 = t;
    t = B; B = B2; B2 = t;
    t = Cc; Cc = C2b; C2b = t;
    t = D; D = D2; D2 = t;
  }
  // u11 = D / B; the flow-rate sums Qx1 = sum dy u11, Qx0 = sum dy u(0,0) (j = 1..nn+1)
  // run serially in the reference's order: QxT - Qx0 cancels, so its rounding matters
  // (the level widths and u(0,0) are staged in shared memory first: the serial loop then
  // runs on shared-memory loads)
  double *dy = A2, *ur = B2;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    D[j] = D[j] / B[j];
    dy[j] = (j >= 1 && j <= nn + 1) ? (g.yv[j + dny] - g.yv[j - 1 + dny]) : 0.0;
    ur[j] = u1[(size_t)(j + dny) * nc].x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double Qx1 = 0.0, Qx0 = 0.0;
    for (int j = 1; j <= nn + 1; ++j) Qx1 = Qx1 + dy[j] * D[j];
    for (int j = 1; j <= nn + 1; ++j) Qx0 = Qx0 + dy[j] * ur[j];
    const double gg = (sc->QxT - Qx0) / Qx1;
    sc->mpgx = sc->mpgx + gg;
    sc->dgx = gg;
    gg_sh = gg;
  }
  __syncthreads();
  const double gg = gg_sh;
  for (int j = threadIdx.x; j <= nn + 2; j += blockDim.x) u1[(size_t)(j + dny) * nc].x += gg * D[j];
}

// flowrateIm of u1 (0,0): Qx (meanflow_ctP, littleharsh.f90:529-545; getini)
__global__ void k_flowrate(const double2 *__restrict__ u1, Geo g, DevScalars *sc, int setQxT) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double Q = 0.0;
  for (int j = 1; j <= g.nn + 1; ++j) Q = Q + (g.yv[j + g.dny] - g.yv[j - 1 + g.dny]) * u1[(size_t)(j + g.dny) * g.ncol].x;
  sc->Qx = Q;
  if (setQxT) sc->QxT = Q;
}

// The scalar part of record_out (FOU3D.f90:3040-3070) from mode (0,0) of u1: Qx by flowrateIm,
// Umax by maxvel (littleharsh.f90:511-527: the largest Re u(j), j = 0..nn+2, not below 0) and
// the slip velocity Uslip, u(0,0) extrapolated linearly from levels 0 and 1 to y = -1.
__global__ void k_history(const double2 *__restrict__ u1, Geo g, DevScalars *sc) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int dny = g.dny, nc = g.ncol;
  double Q = 0.0, um = 0.0;
  for (int j = 1; j <= g.nn + 1; ++j) Q = Q + (g.yv[j + dny] - g.yv[j - 1 + dny]) * u1[(size_t)(j + dny) * nc].x;
  for (int j = 0; j <= g.nn + 2; ++j) um = fmax(um, u1[(size_t)(j + dny) * nc].x);
  const double u0 = u1[(size_t)dny * nc].x, u1v = u1[(size_t)(1 + dny) * nc].x;
  const double y0 = g.yu[dny], y1 = g.yu[1 + dny];
  sc->Qx = Q;
  sc->Umax = um;
  sc->Uslip = (u1v * (-1.0 - y0) + u0 * (y1 + 1.0)) / (y1 - y0);
}

__global__ void k_step_end(DevScalars *sc) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  sc->iter += 1;
  const double e = sqrt(__longlong_as_double((long long)sc->errbits));
  sc->err = e;
  if (!(e == e) || isinf(e) || !(sc->dt == sc->dt)) sc->status = LH_ENONFINITE;
}

// ============================================================================
// LU_buildP + LU_decP (tridLU_3D.f90:333-407, 477-518), once per channel: the
// pressure matrix does not depend on time. dg1 = a1 (lower), dg2 = 1/pivot,
// dg3 = upper factor; [qp][col], qp = 0..np-1 <-> p level N(4,0)+1+qp.
// ============================================================================
__global__ void __launch_bounds__(NTHR) k_build_dg(double *__restrict__ dg1, double *__restrict__ dg2,
                                                   double *__restrict__ dg3, Geo g) {
  const int vc = blockIdx.x * blockDim.x + threadIdx.x;
  const int nc = g.ncol;
  if (vc >= g.nvc) return;
  int c, bd;
  vcol_of(g, vc, c, bd);
  const int plo = g.bq[bd][4], phi = g.bq[bd][5];
  const int r = c / g.N1h, kx = c - r * g.N1h;
  const double k2x = g.k2x[kx], k2z = g.k2z[r];
  const double dd = g.dd;
  double a3raw = 0.0, a2p = 0.0;
  for (int qp = plo; qp <= phi; ++qp) {
    const int q = qp + 1;
    const double Dt = dd * g.thu[q];
    const double Gb = -dd * g.thv[q];
    double A1, A2, A3;
    if (qp == plo) {
      A1 = 0.0;
      A2 = (Dt * Gb) + k2x + k2z;
      A3 = (Dt * (dd * g.thv[q]));
      if (c == 0 && bd == 1) {  // gauge of mode (0,0)
        const double h = g.yu[2 + g.dny] - g.yu[1 + g.dny];
        A1 = 0.0; A2 = 1.0 / (h * h); A3 = 0.0;
      }
    } else {
      const double Db = -dd * g.thu[q];
      const double Gt = dd * g.thv[q - 1];
      const double Gbm = -dd * g.thv[q - 1];
      if (qp == phi) { A2 = (Db * Gt) + k2x + k2z; A1 = (Db * Gbm); A3 = 0.0; }
      else { A2 = (Db * Gt) + (Dt * Gb) + k2x + k2z; A1 = (Db * Gbm); A3 = (Dt * (dd * g.thv[q])); }
    }
    if (qp == plo) a2p = 1.0 / A2;
    else {
      const double a3p = a3raw * a2p;
      dg3[(size_t)(qp - 1) * nc + c] = a3p;
      a2p = 1.0 / (A2 - A1 * a3p);
    }
    dg1[(size_t)qp * nc + c] = A1;
    dg2[(size_t)qp * nc + c] = a2p;
    a3raw = A3;
  }
  dg3[(size_t)phi * nc + c] = 0.0;
}

// ============================================================================
// Pressure: divergence, psi = dti/(a+b) div (gauge on (0,0)), LUsolP with the
// stored factors, p += psi, v_corr, and the divergence of the corrected field
// (max |div|^2 -> errbits) when need_div: the reference recomputes div after
// every v_corr but only reads it (error()) at the start of a step, so it is
// formed in the third substep. p levels qp <-> u/v index q = qp + 1;
// `psi` holds the forward-sweep values (psi itself stays in registers).
// ============================================================================
// One lane per (column, real/imaginary part): the pressure matrix is real, so the two
// parts are independent systems; the i*k couplings of the divergence and of v_corr
// exchange the other part through a shuffle within the lane pair. Two lanes per column
// double the warps in flight (the solves are latency-bound at the 384x192 wall grid).
// Scalar views: element (level, col, part) at (level*ncol + col)*2 + part.
__global__ void __launch_bounds__(NTHR, LH_PRESS_MINB) k_press2(double *__restrict__ u1, double *__restrict__ u2,
                                                 double *__restrict__ u3, double *__restrict__ p,
                                                 double *__restrict__ psi, const double *__restrict__ dg1,
                                                 const double *__restrict__ dg2, const double *__restrict__ dg3, Geo g,
                                                 DevScalars *sc, int kRK, int need_div) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int vc = tid >> 1, part = tid & 1;
  const unsigned pm = 3u << ((threadIdx.x & 31) & ~1);  // the lane pair
  const int nc = g.ncol;
  unsigned long long dmax = 0ull;  // max |div|^2 as bits
  // per-level factors of this substep: dti/(a+b) dd thu (divergence -> right-hand side)
  // and dt (a+b) dd thv (v_corr), so that the lanes spend no FP64 multiply on them
  extern __shared__ double ptab[];
  {
    const double aRb0 = g.aRK[kRK - 1] + g.bRK[kRK - 1];
    const double dti0 = sc->dti / aRb0, dtk0 = sc->dt * aRb0 * g.dd;
    for (int i = threadIdx.x; i < g.nu; i += blockDim.x) ptab[i] = dti0 * g.thud[i];
    for (int i = threadIdx.x; i < g.nv; i += blockDim.x) ptab[g.nu + i] = dtk0 * g.thv[i];
    __syncthreads();
  }
  if (vc < g.nvc) {
    int c, bd;
    vcol_of(g, vc, c, bd);
    const int plo = g.bq[bd][4], phi = g.bq[bd][5];
    const int ulo = g.bq[bd][0], uhi = g.bq[bd][1], vlo = g.bq[bd][2], vhi = g.bq[bd][3];
    const int r = c / g.N1h, kx = c - r * g.N1h;
    const double kxv = g.k1x[kx], kzv = g.k1z[r];
    // i*k*z: real part -k*z.y, imaginary part k*z.x; lane `part` reads the other part
    const double sgn = part ? 1.0 : -1.0;
    const double skx = sgn * kxv, skz = sgn * kzv;  // sgn*(a+b) = sgn*a + sgn*b exactly
    const double aRb = g.aRK[kRK - 1] + g.bRK[kRK - 1];
    const double dtirk = sc->dti / aRb;
    const double dt = sc->dt;
    const size_t ls = (size_t)nc * 2;
    const size_t ci = (size_t)c * 2 + part, co = (size_t)c * 2 + (part ^ 1);
    constexpr int D = LH_PF_PRESS > 0 ? LH_PF_PRESS : 1;
    const double dskx = dtirk * skx, dskz = dtirk * skz;
#define HP_TH(q_) ptab[q_]
#define HP_TV(q_) ptab[g.nu + (q_)]
    double y = 0.0;
    double vm = u2[(size_t)plo * ls + ci];
    {  // forward sweep; the inputs of a level are loaded D levels ahead
      double fa[D], fw[D], fv[D], f1[D], f2[D], ft[D];
#define HP_FETCH(s_, qq_)                                              \
  {                                                                    \
    const int qp_ = (qq_);                                             \
    const size_t e_ = (size_t)(qp_ + 1) * ls;                          \
    fa[s_] = u1[e_ + co]; fw[s_] = u3[e_ + co]; fv[s_] = u2[e_ + ci];  \
    f1[s_] = dg1[(size_t)qp_ * nc + c]; f2[s_] = dg2[(size_t)qp_ * nc + c]; \
    ft[s_] = HP_TH(qp_ + 1);                                           \
  }
#pragma unroll
      for (int s_ = 0; s_ < D; ++s_)
        if (plo + s_ <= phi) HP_FETCH(s_, plo + s_)
      for (int qb = plo; qb <= phi; qb += D) {
#pragma unroll
        for (int s_ = 0; s_ < D; ++s_) {
          const int qp = qb + s_;
          if (qp > phi) break;
          const double ao = fa[s_], wo = fw[s_], v = fv[s_], A1 = f1[s_], a2p = f2[s_];
          const double th = ft[s_];
          if (qp + D <= phi) HP_FETCH(s_, qp + D)
          double rhs = (dskx * ao + dskz * wo) + th * (v - vm);
          vm = v;
          if (qp == plo && c == 0 && bd == 1) rhs = 0.0;
          y = (qp == plo) ? rhs * a2p : (rhs - A1 * y) * a2p;
          psi[(size_t)qp * ls + ci] = y;
        }
      }
#undef HP_FETCH
    }
    const double dtrk = dt * aRb;
    const double kxd = dtrk * kxv, kzd = dtrk * kzv;
    double xn = y;
    double vup = 0.0, aup_o = 0.0, wup_o = 0.0;
    {  // backward sweep, v_corr and the divergence of the corrected field; loads D levels ahead
      double bs[D], b3[D], bp[D], bu[D], bw[D], bv[D], btv[D], btu[D];
#define HB_FETCH(s_, qq_)                                                   \
  {                                                                         \
    const int qp_ = (qq_);                                                  \
    const size_t e_ = (size_t)(qp_ + 1) * ls + ci;                          \
    bs[s_] = psi[(size_t)qp_ * ls + ci]; b3[s_] = dg3[(size_t)qp_ * nc + c]; \
    bp[s_] = p[(size_t)qp_ * ls + ci];                                      \
    bu[s_] = u1[e_]; bw[s_] = u3[e_]; bv[s_] = u2[e_];                      \
    btv[s_] = HP_TV(qp_ + 1); btu[s_] = g.thud[qp_ + 2];                    \
  }
#pragma unroll
      for (int s_ = 0; s_ < D; ++s_)
        if (phi - s_ >= plo) HB_FETCH(s_, phi - s_)
      for (int qb = phi; qb >= plo; qb -= D) {
#pragma unroll
        for (int s_ = 0; s_ < D; ++s_) {
          const int qp = qb - s_;
          if (qp < plo) break;
          const int q = qp + 1;
          const size_t e = (size_t)q * ls;
          const double ps = bs[s_], d3 = b3[s_], pq = bp[s_], uq = bu[s_], wq = bw[s_];
          const double thv = btv[s_], thu1 = btu[s_];
          double v = bv[s_];
          if (qp - D >= plo) HB_FETCH(s_, qp - D)
          const double x = (qp == phi) ? xn : ps - d3 * xn;
          p[(size_t)qp * ls + ci] = pq + x;
          // u -= dtrk i kx psi: the real part gains kxd*psi.y, the imaginary part loses kxd*psi.x
          const double xo = __shfl_xor_sync(pm, x, 1);
          const double a = uq - sgn * kxd * xo;
          const double w = wq - sgn * kzd * xo;
          u1[e + ci] = a;
          u3[e + ci] = w;
          if (q <= vhi - 1) {
            v = v - thv * (xn - x);
            u2[e + ci] = v;
          }
          // divergence of the corrected field at the level above (p level qp + 1)
          const double ao = __shfl_xor_sync(pm, a, 1), wo = __shfl_xor_sync(pm, w, 1);
          if (need_div && qp < phi) {
            const double th = thu1;
            const double dvp = (skx * aup_o + skz * wup_o) + th * (vup - v);
            const double d2 = dvp * dvp;
            bits_max(dmax, d2 + __shfl_xor_sync(pm, d2, 1));
          }
          aup_o = ao; wup_o = wo; vup = v;
          xn = x;
        }
      }
#undef HB_FETCH
#undef HP_TH
#undef HP_TV
    }
    if (need_div) {
      const double th = g.thud[plo + 1];
      const double vb = u2[(size_t)plo * ls + ci];
      const double dvp = (skx * aup_o + skz * wup_o) + th * (vup - vb);
      const double d2 = dvp * dvp;
      bits_max(dmax, d2 + __shfl_xor_sync(pm, d2, 1));
    }
    if (bd <= 1) {
      u1[(size_t)ulo * ls + ci] = g.gwbc1 * u1[(size_t)(ulo + 1) * ls + ci];
      u3[(size_t)ulo * ls + ci] = g.gwbc3 * u3[(size_t)(ulo + 1) * ls + ci];
    }
    if (bd >= 1) {
      u1[(size_t)uhi * ls + ci] = g.gwbc1 * u1[(size_t)(uhi - 1) * ls + ci];
      u3[(size_t)uhi * ls + ci] = g.gwbc3 * u3[(size_t)(uhi - 1) * ls + ci];
    }
    u2[(size_t)vlo * ls + ci] = 0.0;
    u2[(size_t)vhi * ls + ci] = 0.0;
  }
  // |div|^2 = re^2 + im^2 per level, summed over the lane pair above
  dmax = warp_max_bits(dmax);
  if ((threadIdx.x & 31) == 0) atomicMax(&sc->errbits, dmax);
}

// ============================================================================
// The pressure step of k_press2 with the y-columns staged through shared memory: every lane
// keeps a ring of D + 1 levels of its inputs, filled by cp.async copies issued D levels ahead
// of the sweep (into the slot not being read), so that D memory latencies overlap without
// holding the prefetched values in registers (the solves have few warps per SM: one lane per
// column and part). Same arithmetic as k_press2, so the same results bit for bit. Shared
// memory: the per-level factor tables (nu + nv doubles) and the ring, 6 (D + 1) doubles per
// thread.
// ============================================================================

template <int D>
__global__ void __launch_bounds__(NTHR) k_press3(double *__restrict__ u1, double *__restrict__ u2,
                                                 double *__restrict__ u3, double *__restrict__ p,
                                                 double *__restrict__ psi, const double *__restrict__ dg1,
                                                 const double *__restrict__ dg2, const double *__restrict__ dg3, Geo g,
                                                 DevScalars *sc, int kRK, int need_div) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int vc = tid >> 1, part = tid & 1;
  const unsigned pm = 3u << ((threadIdx.x & 31) & ~1);  // the lane pair
  const int nc = g.ncol;
  unsigned long long dmax = 0ull;  // max |div|^2 as bits
  extern __shared__ double ptab[];
  const int nt = blockDim.x;
  double *ring = ptab + ((g.nu + g.nv + 1) & ~1);  // [D + 1][6][nt]
  constexpr int NS = D + 1;
  {
    const double aRb0 = g.aRK[kRK - 1] + g.bRK[kRK - 1];
    const double dti0 = sc->dti / aRb0, dtk0 = sc->dt * aRb0 * g.dd;
    for (int i = threadIdx.x; i < g.nu; i += blockDim.x) ptab[i] = dti0 * g.thud[i];
    for (int i = threadIdx.x; i < g.nv; i += blockDim.x) ptab[g.nu + i] = dtk0 * g.thv[i];
    __syncthreads();
  }
#define RS(s_, f_) ring[((s_) * 6 + (f_)) * nt + threadIdx.x]
  if (vc < g.nvc) {
    int c, bd;
    vcol_of(g, vc, c, bd);
    const int plo = g.bq[bd][4], phi = g.bq[bd][5];
    const int ulo = g.bq[bd][0], uhi = g.bq[bd][1], vlo = g.bq[bd][2], vhi = g.bq[bd][3];
    const int r = c / g.N1h, kx = c - r * g.N1h;
    const double kxv = g.k1x[kx], kzv = g.k1z[r];
    const double sgn = part ? 1.0 : -1.0;
    const double skx = sgn * kxv, skz = sgn * kzv;
    const double aRb = g.aRK[kRK - 1] + g.bRK[kRK - 1];
    const double dtirk = sc->dti / aRb;
    const double dt = sc->dt;
    const size_t ls = (size_t)nc * 2;
    const size_t ci = (size_t)c * 2 + part, co = (size_t)c * 2 + (part ^ 1);
    const double dskx = dtirk * skx, dskz = dtirk * skz;
    double y = 0.0;
    double vm = u2[(size_t)plo * ls + ci];
    // forward sweep: level qp's inputs (u1, u3 of the other part, v, dg1, dg2) in ring slot qp % D
    auto fetch_f = [&](int qp) {
      const int s_ = (qp - plo) % NS;
      const size_t e_ = (size_t)(qp + 1) * ls;
      cpa8(&RS(s_, 0), u1 + e_ + co); cpa8(&RS(s_, 1), u3 + e_ + co); cpa8(&RS(s_, 2), u2 + e_ + ci);
      cpa8(&RS(s_, 3), dg1 + (size_t)qp * nc + c); cpa8(&RS(s_, 4), dg2 + (size_t)qp * nc + c);
    };
#pragma unroll
    for (int s_ = 0; s_ < D; ++s_) {
      if (plo + s_ <= phi) fetch_f(plo + s_);
      cpa_commit();
    }
    for (int qp = plo; qp <= phi; ++qp) {
      cpa_wait<D - 1>();
      const int s_ = (qp - plo) % NS;
      const double ao = RS(s_, 0), wo = RS(s_, 1), v = RS(s_, 2), A1 = RS(s_, 3), a2p = RS(s_, 4);
      const double th = ptab[qp + 1];
      if (qp + D <= phi) fetch_f(qp + D);
      cpa_commit();
      double rhs = (dskx * ao + dskz * wo) + th * (v - vm);
      vm = v;
      if (qp == plo && c == 0 && bd == 1) rhs = 0.0;
      y = (qp == plo) ? rhs * a2p : (rhs - A1 * y) * a2p;
      psi[(size_t)qp * ls + ci] = y;
    }
    cpa_wait<0>();
    __threadfence_block();  // the backward sweep's copies read psi written above by this thread
    const double dtrk = dt * aRb;
    const double kxd = dtrk * kxv, kzd = dtrk * kzv;
    double xn = y;
    double vup = 0.0, aup_o = 0.0, wup_o = 0.0;
    // backward sweep: level qp's inputs (psi, dg3, p, u1, u3, v of this part) in slot (phi - qp) % D
    auto fetch_b = [&](int qp) {
      const int s_ = (phi - qp) % NS;
      const size_t e_ = (size_t)(qp + 1) * ls + ci;
      cpa8(&RS(s_, 0), psi + (size_t)qp * ls + ci); cpa8(&RS(s_, 1), dg3 + (size_t)qp * nc + c);
      cpa8(&RS(s_, 2), p + (size_t)qp * ls + ci);
      cpa8(&RS(s_, 3), u1 + e_); cpa8(&RS(s_, 4), u3 + e_); cpa8(&RS(s_, 5), u2 + e_);
    };
#pragma unroll
    for (int s_ = 0; s_ < D; ++s_) {
      if (phi - s_ >= plo) fetch_b(phi - s_);
      cpa_commit();
    }
    for (int qp = phi; qp >= plo; --qp) {
      cpa_wait<D - 1>();
      const int s_ = (phi - qp) % NS;
      const int q = qp + 1;
      const size_t e = (size_t)q * ls;
      const double ps = RS(s_, 0), d3 = RS(s_, 1), pq = RS(s_, 2), uq = RS(s_, 3), wq = RS(s_, 4);
      double v = RS(s_, 5);
      const double thv = ptab[g.nu + q], thu1 = g.thud[qp + 2];
      if (qp - D >= plo) fetch_b(qp - D);
      cpa_commit();
      const double x = (qp == phi) ? xn : ps - d3 * xn;
      p[(size_t)qp * ls + ci] = pq + x;
      const double xo = __shfl_xor_sync(pm, x, 1);
      const double a = uq - sgn * kxd * xo;
      const double w = wq - sgn * kzd * xo;
      u1[e + ci] = a;
      u3[e + ci] = w;
      if (q <= vhi - 1) {
        v = v - thv * (xn - x);
        u2[e + ci] = v;
      }
      const double ao = __shfl_xor_sync(pm, a, 1), wo = __shfl_xor_sync(pm, w, 1);
      if (need_div && qp < phi) {
        const double dvp = (skx * aup_o + skz * wup_o) + thu1 * (vup - v);
        const double d2 = dvp * dvp;
        bits_max(dmax, d2 + __shfl_xor_sync(pm, d2, 1));
      }
      aup_o = ao; wup_o = wo; vup = v;
      xn = x;
    }
    cpa_wait<0>();
    if (need_div) {
      const double th = g.thud[plo + 1];
      const double vb = u2[(size_t)plo * ls + ci];
      const double dvp = (skx * aup_o + skz * wup_o) + th * (vup - vb);
      const double d2 = dvp * dvp;
      bits_max(dmax, d2 + __shfl_xor_sync(pm, d2, 1));
    }
    if (bd <= 1) {
      u1[(size_t)ulo * ls + ci] = g.gwbc1 * u1[(size_t)(ulo + 1) * ls + ci];
      u3[(size_t)ulo * ls + ci] = g.gwbc3 * u3[(size_t)(ulo + 1) * ls + ci];
    }
    if (bd >= 1) {
      u1[(size_t)uhi * ls + ci] = g.gwbc1 * u1[(size_t)(uhi - 1) * ls + ci];
      u3[(size_t)uhi * ls + ci] = g.gwbc3 * u3[(size_t)(uhi - 1) * ls + ci];
    }
    u2[(size_t)vlo * ls + ci] = 0.0;
    u2[(size_t)vhi * ls + ci] = 0.0;
  }
#undef RS
  dmax = warp_max_bits(dmax);
  if ((threadIdx.x & 31) == 0) atomicMax(&sc->errbits, dmax);
}

__global__ void k_reset_err(DevScalars *sc) {
  if (threadIdx.x == 0 && blockIdx.x == 0) sc->errbits = 0ull;
}

// max |div| of the current state (getini's divergence + error())
__global__ void __launch_bounds__(NTHR) k_divmax(const double2 *__restrict__ u1, const double2 *__restrict__ u2,
                                                 const double2 *__restrict__ u3, Geo g, DevScalars *sc) {
  const int vc = blockIdx.x * blockDim.x + threadIdx.x;
  double dmax = 0.0;
  if (vc < g.nvc) {
    int c, bd;
    vcol_of(g, vc, c, bd);
    const int r = c / g.N1h, kx = c - r * g.N1h;
    const double kxv = g.k1x[kx], kzv = g.k1z[r];
    for (int q = g.bq[bd][4] + 1; q <= g.bq[bd][5] + 1; ++q) {
      const size_t o = (size_t)q * g.ncol + c;
      const double2 a = u1[o], w = u3[o], v = u2[o], vm = u2[o - g.ncol];
      const double th = g.dd * g.thu[q];
      double2 dv;
      dv.x = (-kxv * a.y + -kzv * w.y) + th * (v.x - vm.x);
      dv.y = (kxv * a.x + kzv * w.x) + th * (v.y - vm.y);
      dmax = nmax(dmax, dv.x * dv.x + dv.y * dv.y);
    }
  }
  dmax = warp_max(dmax);
  if ((threadIdx.x & 31) == 0) atomic_max_pos(&sc->errbits, dmax);
}

// err = max |div| (errbits holds the maximum of |div|^2)
__global__ void k_err_from_bits(DevScalars *sc) {
  if (threadIdx.x == 0 && blockIdx.x == 0) sc->err = sqrt(__longlong_as_double((long long)sc->errbits));
}

// one band's host cfield [k][l] (staged) <-> device [lev0 + l][cols[k]]; put = 1 writes the device
// ============================================================================
// The other sums of the statistics step, formed from the spectral state (FP64 in both
// forms; launched on request only, LH_STAT_THREADS threads per block).
// ============================================================================
#define LH_STAT_THREADS 256
// omega_x = -der_z_N(v) + der_yv_h_wx(w) at every v level (FOU3D.f90:300-327), and its
// plane sums over the N1 x N2 points of four_to_phys_N (stats.f90:56-63), by Parseval:
// sum f = N1 N2 Re c(0,0); sum f^2 = N1 N2 [ sum over 0 < kx < N1/2 of 2 |c|^2, plus for
// kx = 0 and N1/2 (whose Im the real transform drops) 1/2 |c(kz)|^2 + 1/2 Re c(kz) c(-kz) ].
// One block per level; the level's plane class gives N1, N2 (wall bands: nhw, n2w; the
// core band: nhc, n2c). pl: [11][nu], quantities 9 and 10.
__device__ __forceinline__ double2 wx_mode(const double2 *__restrict__ u2, const double2 *__restrict__ u3,
                                           const Geo &g, int q, int c, int fr, double fy) {
  const double2 v = u2[(size_t)q * g.ncolF + c];
  const double2 a = u3[(size_t)(q + 1) * g.ncolF + c], b = u3[(size_t)q * g.ncolF + c];
  const double kz = g.k1z[fr];
  // -(i kz v) + (a - b) fy
  return make_double2(kz * v.y + (a.x - b.x) * fy, -kz * v.x + (a.y - b.y) * fy);
}
__global__ void __launch_bounds__(LH_STAT_THREADS) k_wx_stats(const double2 *__restrict__ u2, const double2 *__restrict__ u3,
                                                     Geo g, int nhc, int n2c, double *__restrict__ pl) {
  __shared__ double red[LH_STAT_THREADS / 32][2];
  const int q = blockIdx.x;
  const int j = q - g.dny;
  const bool fine = !g.mb || j <= g.N3[1] || j > g.N3[2];
  const int nh = fine ? g.N1hF : nhc, n2 = fine ? g.N2F : n2c, n1 = 2 * (nh - 1);
  const double fy = g.thv[q] * g.dd;
  double s = 0.0, s2 = 0.0;
  for (int e = threadIdx.x; e < nh * n2; e += blockDim.x) {
    const int r = e / nh, kx = e - r * nh;
    const int fr = r < n2 / 2 ? r : r + g.N2F - n2;
    const double2 cv = wx_mode(u2, u3, g, q, fr * g.N1hF + kx, fr, fy);
    const double m2 = cv.x * cv.x + cv.y * cv.y;
    if (kx == 0 || kx == nh - 1) {
      const int rm = (n2 - r) % n2;
      const int frm = rm < n2 / 2 ? rm : rm + g.N2F - n2;
      const double2 cm = wx_mode(u2, u3, g, q, frm * g.N1hF + kx, frm, fy);
      s2 += 0.5 * m2 + 0.5 * (cv.x * cm.x - cv.y * cm.y);
      if (e == 0) s = cv.x;
    } else {
      s2 += 2.0 * m2;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  }
  if ((threadIdx.x & 31) == 0) { red[threadIdx.x >> 5][0] = s; red[threadIdx.x >> 5][1] = s2; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < LH_STAT_THREADS / 32; ++w) { a += red[w][0]; b += red[w][1]; }
    const double nn = (double)n1 * (double)n2;
    pl[9 * (size_t)g.nu + q] += nn * a;
    pl[10 * (size_t)g.nu + q] += nn * b;
  }
}

// Pressure plane sums (stats.f90:43-50 over the physical pressure): one block per p level q
// (reference level j = q + 1 - dny). Wall-band planes (j <= N(4,1)-1, j >= N(4,2)+2, the
// pgrid plane ranges of the outer bands) hold every mode of the wall-band grid, on the
// Gf = G1 x G2 dealiased points; core planes the long columns (nhc x n2c) on Gc points.
// Parseval on the padded grid: sum p = G p(0,0); sum p^2 = G (sum over kx >= 1 of 2|p|^2,
// kx = N1/2 included, + the kx = 0 column's Hermitian part, whose row -N2/2 has no mirror).
// pp: [2][np].
__global__ void __launch_bounds__(LH_STAT_THREADS) k_p_stats(const double2 *__restrict__ p, Geo g, int nhc, int n2c,
                                                    double Gf, double Gc, double *__restrict__ pp) {
  __shared__ double red[LH_STAT_THREADS / 32][2];
  const int q = blockIdx.x;
  const int j = q + 1 - g.dny;
  const bool fine = !g.mb || j <= g.N4[1] - 1 || j >= g.N4[2] + 2;
  const int nh = fine ? g.N1hF : nhc, n2 = fine ? g.N2F : n2c;
  const double2 *P = p + (size_t)q * g.ncolF;
  double s = 0.0, s2 = 0.0;
  for (int e = threadIdx.x; e < nh * n2; e += blockDim.x) {
    const int r = e / nh, kx = e - r * nh;
    const int fr = r < n2 / 2 ? r : r + g.N2F - n2;
    const double2 a = P[fr * g.N1hF + kx];
    const double m2 = a.x * a.x + a.y * a.y;
    if (kx > 0) {
      s2 += 2.0 * m2;
    } else if (r == n2 / 2) {
      s2 += 0.5 * m2;
    } else {
      const int rm = (n2 - r) % n2;
      const int frm = rm < n2 / 2 ? rm : rm + g.N2F - n2;
      const double2 b = P[frm * g.N1hF];
      s2 += 0.5 * m2 + 0.5 * (a.x * b.x - a.y * b.y);
      if (r == 0) s = a.x;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  }
  if ((threadIdx.x & 31) == 0) { red[threadIdx.x >> 5][0] = s; red[threadIdx.x >> 5][1] = s2; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < LH_STAT_THREADS / 32; ++w) { a += red[w][0]; b += red[w][1]; }
    const double G = fine ? Gf : Gc;
    pp[q] += G * a;
    pp[(size_t)g.np + q] += G * b;
  }
}

// Spectral planes of the tile-conditioned P and omega_x sums: plane b of the chunk is
// list[b] = (kind, level, j1): kind 0 copies p level `level`; kind 1 forms omega_x at v level
// `level` (-i kz v + (w(q+1) - w(q)) dthdyv ddthetavi, FOU3D.f90:300-327). spec: [nb][ncolF].
__global__ void __launch_bounds__(LH_STAT_THREADS) k_cond_spec(const double2 *__restrict__ u2, const double2 *__restrict__ u3,
                                                      const double2 *__restrict__ p, Geo g,
                                                      const int4 *__restrict__ list, double2 *__restrict__ spec) {
  const int4 d = list[blockIdx.y];
  const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= (size_t)g.ncolF) return;
  double2 *o = spec + (size_t)blockIdx.y * g.ncolF + c;
  if (d.x == 0) {
    *o = p[(size_t)d.y * g.ncolF + c];
  } else {
    *o = wx_mode(u2, u3, g, d.y, (int)c, (int)(c / g.N1hF), g.thv[d.y] * g.dd);
  }
}

// conddown1 / condup1 with xsign 1 (stats.f90:109-138, 178-210) of the chunk's physical
// planes (phys [nb][G2][G1]): one thread per tile position (i, k), summing the value and
// its square over the ntx x ntz tiles into the pair 2 kind, 2 kind + 1 of
// cd4 [4][ncl1][dnz][dnx] at level j1 (bottom and top planes of a level add into one cell).
__global__ void __launch_bounds__(LH_STAT_THREADS) k_cond_phys(const double *__restrict__ phys, const int4 *__restrict__ list,
                                                      int G1, int G2, int dnx, int dnz, int ncl1,
                                                      double *__restrict__ cd4) {
  const int4 d = list[blockIdx.y];
  const int cell = blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= dnx * dnz) return;
  const int k = cell / dnx, i = cell - k * dnx;
  const double *f = phys + (size_t)blockIdx.y * G1 * G2;
  double s = 0.0, s2 = 0.0;
  for (int l = k; l < G2; l += dnz)
    for (int m = i; m < G1; m += dnx) {
      const double x = f[(size_t)l * G1 + m];
      s += x;
      s2 += x * x;
    }
  const size_t lv = (size_t)dnz * dnx;
  atomicAdd(&cd4[((size_t)(2 * d.x) * ncl1 + d.z) * lv + cell], s);
  atomicAdd(&cd4[((size_t)(2 * d.x + 1) * ncl1 + d.z) * lv + cell], s2);
}

// spectra (spectra.f90:1-56): band 2's levels x the long columns (cols[0..nlong)),
// sp(level, column) += |u|^2 (U, V, W, P) and Re u1 Re v + Im u1 Im v with v interpolated
// to the centres (interp_v, FOU3D.f90:427-474; band 2's end levels extrapolated with
// gridweighting_interp(2, 1:2) = gi0, gi1). sp: 5 arrays [level][nlong] at offsets off[].
__device__ __forceinline__ double2 itp_v(const double2 *__restrict__ u2, const Geo &g, int q, int c) {
  const double2 a = u2[(size_t)q * g.ncolF + c], b = u2[(size_t)(q - 1) * g.ncolF + c];
  const double w0 = g.yu[q] - g.yv[q - 1], w1 = g.yv[q] - g.yu[q], d = g.yv[q] - g.yv[q - 1];
  return make_double2((w0 * a.x + w1 * b.x) / d, (w0 * a.y + w1 * b.y) / d);
}
__global__ void __launch_bounds__(LH_STAT_THREADS) k_spectra(const double2 *__restrict__ u1, const double2 *__restrict__ u2,
                                                    const double2 *__restrict__ u3, const double2 *__restrict__ p,
                                                    Geo g, const int *__restrict__ cols, int nlong, double gi0,
                                                    double gi1, double *__restrict__ sp) {
  const int ulo = g.bq[1][0], uhi = g.bq[1][1], vlo = g.bq[1][2], vhi = g.bq[1][3];
  const int plo = g.bq[1][4], phi = g.bq[1][5];
  const int nlu = uhi - ulo + 1, nlv = vhi - vlo + 1, nlp = phi - plo + 1;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)nlu * nlong) return;
  const int l = (int)(i / nlong), k = (int)(i - (size_t)l * nlong);
  const int c = cols[k];
  const size_t nc = g.ncolF;
  double *sU = sp, *sV = sU + (size_t)nlu * nlong, *sW = sV + (size_t)nlv * nlong, *sUV = sW + (size_t)nlu * nlong;
  double *sP = sUV + (size_t)nlu * nlong;
  const int q = ulo + l;
  const double2 a = u1[q * nc + c], w = u3[q * nc + c];
  double2 v;
  if (q > ulo && q < uhi) v = itp_v(u2, g, q, c);
  else if (q == ulo) {
    const double2 i1 = itp_v(u2, g, ulo + 1, c), b = u2[(size_t)vlo * nc + c];
    v = make_double2(gi0 * (b.x - i1.x) + i1.x, gi0 * (b.y - i1.y) + i1.y);
  } else {
    const double2 i2 = itp_v(u2, g, uhi - 1, c), b = u2[(size_t)vhi * nc + c];
    v = make_double2(gi1 * (b.x - i2.x) + i2.x, gi1 * (b.y - i2.y) + i2.y);
  }
  sU[i] = sU[i] + a.x * a.x + a.y * a.y;
  sW[i] = sW[i] + w.x * w.x + w.y * w.y;
  sUV[i] = sUV[i] + a.x * v.x + a.y * v.y;
  if (l < nlv) {
    const double2 b = u2[(size_t)(vlo + l) * nc + c];
    sV[i] = sV[i] + b.x * b.x + b.y * b.y;
  }
  if (l < nlp) {
    const double2 b = p[(size_t)(plo + l) * nc + c];
    sP[i] = sP[i] + b.x * b.x + b.y * b.y;
  }
}

// slip statistics (sl_stats2.f90:33-121, inst_sl_stats.f90:1-62) at the wall faces
// jlim(1, vgrid, 2) and jlim(2, vgrid, 2) (v array indices qb, qt), every wall-grid column:
// u1 and u3 interpolated to the face (interp_u) and (u(q+1) - u(q)) dthdyv ddthetavi,
// negated at the top. out: [2][4][ncolF]; acc: add (sl_stats) or store (inst_sl_stats).
__global__ void __launch_bounds__(LH_STAT_THREADS) k_slip(const double2 *__restrict__ u1, const double2 *__restrict__ u3, Geo g,
                                                 int qb, int qt, double2 *__restrict__ out, int acc) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.ncolF) return;
  const size_t nc = g.ncolF;
  for (int w = 0; w < 2; ++w) {
    const int q = w ? qt : qb;
    const double sg = w ? -1.0 : 1.0;
    const double fy = g.thv[q] * g.dd;
    const double ya = g.yu[q], yb = g.yu[q + 1], yv = g.yv[q];
    for (int f = 0; f < 2; ++f) {
      const double2 *u = f ? u3 : u1;
      const double2 hi = u[(size_t)(q + 1) * nc + c], lo = u[(size_t)q * nc + c];
      const double2 it = make_double2(((yv - ya) * hi.x + (yb - yv) * lo.x) / (yb - ya),
                                      ((yv - ya) * hi.y + (yb - yv) * lo.y) / (yb - ya));
      const double2 dy = make_double2(sg * ((hi.x - lo.x) * fy), sg * ((hi.y - lo.y) * fy));
      double2 *o0 = out + ((size_t)(w * 4 + 2 * f) * nc + c), *o1 = o0 + nc;
      if (acc) {
        *o0 = make_double2(o0->x + it.x, o0->y + it.y);
        *o1 = make_double2(o1->x + dy.x, o1->y + dy.y);
      } else {
        *o0 = it;
        *o1 = dy;
      }
    }
  }
}

__global__ void k_band_io(double2 *__restrict__ dev, double2 *__restrict__ stage, const int *__restrict__ cols,
                          int ncb, int nlev, int lev0, int ncol, int put) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)ncb * nlev) return;
  const int k = (int)(i / nlev), l = (int)(i - (size_t)k * nlev);
  double2 *d = dev + (size_t)(lev0 + l) * ncol + cols[k];
  if (put) *d = stage[i];
  else stage[i] = *d;
}

// host cfield [col][lev] <-> device [lev][col] (complex), tiled transpose
__global__ void k_transpose(const double2 *__restrict__ src, double2 *__restrict__ dst, int rows, int cols) {
  __shared__ double2 tile[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int rr = by + i, cc = bx + threadIdx.x;
    if (rr < rows && cc < cols) tile[i][threadIdx.x] = src[(size_t)rr * cols + cc];
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int rr = bx + i, cc = by + threadIdx.x;  // dst is cols x rows
    if (rr < cols && cc < rows) dst[(size_t)rr * rows + cc] = tile[threadIdx.x][i];
  }
}

// ============================================================================
// Generic plane transforms (leaves lh_four_to_phys / lh_phys_to_four and the
// immersed-boundary round trip of du). spec [plane][N2][N1h] complex128, phys
// [plane][G2][G1] double, scratch A/B [plane][l][kx] in the transform precision.
// ============================================================================
template <typename T, int N>
__global__ void __launch_bounds__(NTHR) k_spec_zinv(const double2 *__restrict__ spec, typename C2<T>::t *__restrict__ A,
                                                    Geo g, const typename C2<T>::t *__restrict__ twz) {
  typedef typename C2<T>::t V;
  constexpr int KB = kb_zinv<V>(N);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V *b0 = reinterpret_cast<V *>(smem_raw);
  V *b1 = b0 + KB * N;
  const int pl = blockIdx.y, kx0 = blockIdx.x * KB;
  for (int i = threadIdx.x; i < KB * N; i += blockDim.x) b0[i] = czero<V>();
  __syncthreads();
  const double2 *S = spec + (size_t)pl * g.ncol;
  for (int idx = threadIdx.x; idx < g.N2 * KB; idx += blockDim.x) {
    const int r = idx / KB, kk = idx - r * KB, kx = kx0 + kk;
    if (kx >= g.N1h) continue;
    const double2 val = S[r * g.N1h + kx];
    V v; v.x = to_t<T>(val.x); v.y = to_t<T>(val.y);
    b0[prow(g, r) * KB + kk] = v;
  }
  __syncthreads();
  V *res = line_fft<true, N, KB, true>(b0, b1, twz);
  V *dst = A + (size_t)pl * N * g.N1h;
  for (int idx = threadIdx.x; idx < N * KB; idx += blockDim.x) {
    const int l = idx / KB, kk = idx - l * KB, kx = kx0 + kk;
    if (kx < g.N1h) dst[(size_t)l * g.N1h + kx] = res[l * KB + kk];
  }
}

template <typename T, int N>
__global__ void __launch_bounds__(NTHR) k_xinv_phys(const typename C2<T>::t *__restrict__ A, double *__restrict__ phys,
                                                    Geo g, const typename C2<T>::t *__restrict__ twx) {
  typedef typename C2<T>::t V;
  constexpr int PB = 4 * pb_xpass<V>(N);
  constexpr int G1 = N, H = N / 2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int G2 = g.G2, N1h = g.N1h;
  V *b0 = reinterpret_cast<V *>(smem_raw);
  V *b1 = b0 + PB * G1;
  const int pl = blockIdx.y, l0 = blockIdx.x * PB * 2;
  const int npairs = min(PB, (G2 - l0) / 2);
  const V *Ap = A + (size_t)pl * G2 * N1h;
  for (int idx = threadIdx.x; idx < PB * G1; idx += blockDim.x) {
    const int pb = idx / G1, m = idx - pb * G1;
    V z = czero<V>();
    if (pb < npairs) {
      const int l = l0 + 2 * pb;
      int k = m; bool cj = false;
      if (m > H) { k = G1 - m; cj = true; }
      if (k < N1h) {
        V a = Ap[(size_t)l * N1h + k], b = Ap[(size_t)(l + 1) * N1h + k];
        if (k == 0 || k == H) { a.y = 0; b.y = 0; }
        if (!cj) { z.x = a.x - b.y; z.y = a.y + b.x; } else { z.x = a.x + b.y; z.y = -a.y + b.x; }
      }
    }
    b0[idx] = z;
  }
  __syncthreads();
  V *res = line_fft<true, N, PB, false>(b0, b1, twx);
  double *P = phys + (size_t)pl * G2 * G1;
  for (int idx = threadIdx.x; idx < PB * G1; idx += blockDim.x) {
    const int pb = idx / G1, m = idx - pb * G1;
    if (pb >= npairs) continue;
    const int l = l0 + 2 * pb;
    P[(size_t)l * G1 + m] = to_d(res[idx].x);
    P[(size_t)(l + 1) * G1 + m] = to_d(res[idx].y);
  }
}

template <typename T, int N>
__global__ void __launch_bounds__(NTHR) k_xfwd_phys(const double *__restrict__ phys, typename C2<T>::t *__restrict__ B,
                                                    Geo g, const typename C2<T>::t *__restrict__ twx) {
  typedef typename C2<T>::t V;
  constexpr int PB = 4 * pb_xpass<V>(N);
  constexpr int G1 = N;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int G2 = g.G2, N1h = g.N1h;
  V *b0 = reinterpret_cast<V *>(smem_raw);
  V *b1 = b0 + PB * G1;
  const int pl = blockIdx.y, l0 = blockIdx.x * PB * 2;
  const int npairs = min(PB, (G2 - l0) / 2);
  const double *P = phys + (size_t)pl * G2 * G1;
  for (int idx = threadIdx.x; idx < PB * G1; idx += blockDim.x) {
    const int pb = idx / G1, m = idx - pb * G1;
    V z = czero<V>();
    if (pb < npairs) {
      const int l = l0 + 2 * pb;
      z.x = to_t<T>(P[(size_t)l * G1 + m]);
      z.y = to_t<T>(P[(size_t)(l + 1) * G1 + m]);
    }
    b0[idx] = z;
  }
  __syncthreads();
  V *res = line_fft<false, N, PB, false>(b0, b1, twx);
  const T s1 = (T)1 / (T)G1;
  for (int idx = threadIdx.x; idx < PB * 2 * N1h; idx += blockDim.x) {
    const int k = idx % N1h, rest = idx / N1h;
    const int half = rest & 1, pb = rest >> 1;
    if (pb >= npairs) continue;
    const V *L = res + pb * G1;
    const V z = L[k], zc = cconj(L[(G1 - k) % G1]);
    V o;
    if (!half) { o.x = (T)0.5 * (z.x + zc.x) * s1; o.y = (T)0.5 * (z.y + zc.y) * s1; }
    else { o.x = (T)0.5 * (z.y - zc.y) * s1; o.y = (T)-0.5 * (z.x - zc.x) * s1; }
    if (k == 0) o.y = 0;
    B[((size_t)pl * G2 + l0 + 2 * pb + half) * N1h + k] = o;
  }
}

template <typename T, int N>
__global__ void __launch_bounds__(NTHR) k_zfwd_spec(const typename C2<T>::t *__restrict__ B, double2 *__restrict__ spec,
                                                    Geo g, const typename C2<T>::t *__restrict__ twz) {
  typedef typename C2<T>::t V;
  constexpr int KB = kb_zinv<V>(N);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int N1h = g.N1h, N2 = g.N2;
  V *b0 = reinterpret_cast<V *>(smem_raw);
  V *b1 = b0 + KB * N;
  const int pl = blockIdx.y, kx0 = blockIdx.x * KB;
  for (int idx = threadIdx.x; idx < N * KB; idx += blockDim.x) {
    const int l = idx / KB, kk = idx - l * KB, kx = kx0 + kk;
    V z = czero<V>();
    if (kx < N1h) z = B[((size_t)pl * N + l) * N1h + kx];
    b0[idx] = z;
  }
  __syncthreads();
  V *res = line_fft<false, N, KB, true>(b0, b1, twz);
  const double s2 = 1.0 / (double)N;
  double2 *S = spec + (size_t)pl * g.ncol;
  for (int idx = threadIdx.x; idx < N2 * KB; idx += blockDim.x) {
    const int r = idx / KB, kk = idx - r * KB, kx = kx0 + kk;
    if (kx >= N1h) continue;
    const V t = res[prow(g, r) * KB + kk];
    double2 o; o.x = to_d(t.x) * s2; o.y = to_d(t.y) * s2;
    S[r * N1h + kx] = o;
  }
}

// ============================================================================
// Immersed boundaries (FOU3D.f90:806-998): assemble du at the listed levels,
// then (after the inverse transform) the forcing at the solid points.
// duib layout: [ibslot][field 0..2][col], complex128 (FP64 form) or complex64 (mixed form, whose
// values are FP32); ib levels of u (fields 0, 2) and v (1).
// ============================================================================
template <typename TN>
__global__ void __launch_bounds__(NTHR) k_ib_du(const double2 *__restrict__ u1, const double2 *__restrict__ u2,
                                                const double2 *__restrict__ u3, typename C2<TN>::t *__restrict__ Nu1o,
                                                typename C2<TN>::t *__restrict__ Nu2o, typename C2<TN>::t *__restrict__ Nu3o,
                                                const typename C2<TN>::t *__restrict__ N1xz, const typename C2<TN>::t *__restrict__ N2xz,
                                                const typename C2<TN>::t *__restrict__ N3xz, const typename C2<TN>::t *__restrict__ uvf,
                                                const typename C2<TN>::t *__restrict__ vvc, const typename C2<TN>::t *__restrict__ wvf,
                                                const double2 *__restrict__ p, double2 *__restrict__ duib,
                                                const int *__restrict__ iblev, int nib, Geo g,
                                                const DevScalars *__restrict__ sc, int kRK) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = blockIdx.y;  // ib slot
  const int nc = g.ncol;
  if (c >= nc || s >= nib) return;
  const int r = c / g.N1h, kx = c - r * g.N1h;
  const double k2x = g.k2x[kx], k2z = g.k2z[r];
  const double C1 = g.aRK[kRK - 1] / g.Re, C2 = -g.cRK[kRK - 1], dR = g.dRK[kRK - 1];
  const double G = -g.gRK[kRK - 1];
  const int qu = iblev[2 * s], qv = iblev[2 * s + 1];
  if (qu > 0) {  // u and w at u-level qu
    const double *d0 = g.d2u, *d1 = g.d2u + g.nu, *d2 = g.d2u + 2 * g.nu;
    const size_t o = (size_t)qu * nc + c;
    const double a = d0[qu], dg = (k2x + k2z) + d1[qu], cc = d2[qu];
    const double2 pj = p[(size_t)(qu - 1) * nc + c];
    const double C3x = -dR * g.k1x[kx], C3z = -dR * g.k1z[r];
    const double th = g.thu[qu];
    for (int f = 0; f < 2; ++f) {
      const double2 *U = f ? u3 : u1;
      typename ::C2<TN>::t *No = f ? Nu3o : Nu1o;
      const typename ::C2<TN>::t *X = f ? N3xz : N1xz;
      const typename ::C2<TN>::t *F = f ? wvf : uvf;
      const double C3 = f ? C3z : C3x;
      const double2 um = U[o - nc], u0 = U[o], up = U[o + nc];
      double2 L;
      L.x = (a * um.x + dg * u0.x) + cc * up.x; L.y = (a * um.y + dg * u0.y) + cc * up.y;
      const double2 no = ld2(No[o]);
      double2 du;
      du.x = (C1 * L.x + C2 * no.x) + (-C3 * pj.y);
      du.y = (C1 * L.y + C2 * no.y) + (C3 * pj.x);
      if (f == 0 && c == 0) du.x += -dR * sc->mpgx;
      const double2 x = ld2(X[o]), fq = ld2(F[o]), fm = ld2(F[o - nc]);
      double2 n;
      n.x = x.x + (fq.x - fm.x) * th * g.dd; n.y = x.y + (fq.y - fm.y) * th * g.dd;
      No[o].x = n.x; No[o].y = n.y;  // N of this substep (the next substep's -cRK term)
      du.x = du.x + G * n.x; du.y = du.y + G * n.y;
      duib[((size_t)s * 3 + (f ? 2 : 0)) * nc + c] = du;
    }
  }
  if (qv > 0) {
    const double *d0 = g.d2v, *d1 = g.d2v + g.nv, *d2 = g.d2v + 2 * g.nv;
    const size_t o = (size_t)qv * nc + c;
    const double a = d0[qv], dg = (k2x + k2z) + d1[qv], cc = d2[qv];
    const double2 vm = u2[o - nc], v0 = u2[o], vp = u2[o + nc];
    double2 L;
    L.x = (a * vm.x + dg * v0.x) + cc * vp.x; L.y = (a * vm.y + dg * v0.y) + cc * vp.y;
    const double C3 = -dR * g.dd * g.thv[qv];
    const double2 pp = p[(size_t)qv * nc + c], pm = p[(size_t)(qv - 1) * nc + c];
    const double2 no = ld2(Nu2o[o]);
    double2 du;
    du.x = (C1 * L.x + C2 * no.x) + C3 * (pp.x - pm.x);
    du.y = (C1 * L.y + C2 * no.y) + C3 * (pp.y - pm.y);
    const double th = g.thv[qv];
    const double2 x = ld2(N2xz[o]), vp1 = ld2(vvc[o + nc]), vq = ld2(vvc[o]);
    double2 n;
    n.x = x.x + (vp1.x - vq.x) * th * g.dd; n.y = x.y + (vp1.y - vq.y) * th * g.dd;
    Nu2o[o].x = n.x; Nu2o[o].y = n.y;
    du.x = du.x + G * n.x; du.y = du.y + G * n.y;
    duib[((size_t)s * 3 + 1) * nc + c] = du;
  }
}

// Mixed form of k_ib_du: the same right-hand side in FP32 (FP64 neighbour
// differences for the Laplacian, integer-pipe conversions), N and du stored in FP32.
__global__ void __launch_bounds__(NTHR, LH_IBDU_MINB) k_ib_du_mx(const double2 *__restrict__ u1, const double2 *__restrict__ u2,
                                                   const double2 *__restrict__ u3, float2 *__restrict__ Nu1o,
                                                   float2 *__restrict__ Nu2o, float2 *__restrict__ Nu3o,
                                                   const float2 *__restrict__ N1xz, const float2 *__restrict__ N2xz,
                                                   const float2 *__restrict__ N3xz, const float2 *__restrict__ uvf,
                                                   const float2 *__restrict__ vvc, const float2 *__restrict__ wvf,
                                                   const double2 *__restrict__ p, float2 *__restrict__ duib,
                                                   const int *__restrict__ iblev, int nib, Geo g,
                                                   const DevScalars *__restrict__ sc, int kRK) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = blockIdx.y;
  const int nc = g.ncol;
  if (c >= nc || s >= nib) return;
  const int r = c / g.N1h, kx = c - r * g.N1h;
  const float k2f = (float)(g.k2x[kx] + g.k2z[r]);
  const float C1 = (float)(g.aRK[kRK - 1] / g.Re), C2 = (float)(-g.cRK[kRK - 1]);
  const double dR = g.dRK[kRK - 1];
  const float dRf = (float)dR;
  const float G = (float)(-g.gRK[kRK - 1]);
  const float dd = (float)g.dd;
  const int qu = iblev[2 * s], qv = iblev[2 * s + 1];
  // every input of the thread is loaded before the first store, so that the latencies of the
  // u-level and v-level loads overlap (the kernel is bound by them, not by bandwidth)
  const size_t ou = (size_t)qu * nc + c, ov = (size_t)qv * nc + c;
  double2 um[2], u0[2], up[2], pj, vm, v0, vp, pp, pm;
  float2 no[2], xq[2], fq[2], fm[2], nov, xv, vp1, vq;
  double mpgx = 0.0;
  if (qu > 0) {
    pj = p[(size_t)(qu - 1) * nc + c];
    if (c == 0) mpgx = sc->mpgx;
#pragma unroll
    for (int f = 0; f < 2; ++f) {
      const double2 *U = f ? u3 : u1;
      const float2 *F = f ? wvf : uvf;
      um[f] = U[ou - nc]; u0[f] = U[ou]; up[f] = U[ou + nc];
      no[f] = (f ? Nu3o : Nu1o)[ou];
      xq[f] = (f ? N3xz : N1xz)[ou];
      fq[f] = F[ou]; fm[f] = F[ou - nc];
    }
  }
  if (qv > 0) {
    vm = u2[ov - nc]; v0 = u2[ov]; vp = u2[ov + nc];
    pp = p[(size_t)qv * nc + c]; pm = p[(size_t)(qv - 1) * nc + c];
    nov = Nu2o[ov]; xv = N2xz[ov]; vp1 = vvc[ov + nc]; vq = vvc[ov];
  }
  if (qu > 0) {
    const int nu = g.nu;
    const float a = g.d2uf[qu], cc = g.d2uf[2 * nu + qu], sdg = g.sdgu[qu] + k2f;
    const float pjx = d2f_alu(pj.x), pjy = d2f_alu(pj.y);
    const float C3x = (float)(-dR * g.k1x[kx]), C3z = (float)(-dR * g.k1z[r]);
    const float th = g.thuf[qu];
#pragma unroll
    for (int f = 0; f < 2; ++f) {
      const float C3 = f ? C3z : C3x;
      float2 L;
      L.x = a * d2f_alu(um[f].x - u0[f].x) + cc * d2f_alu(up[f].x - u0[f].x) + sdg * d2f_alu(u0[f].x);
      L.y = a * d2f_alu(um[f].y - u0[f].y) + cc * d2f_alu(up[f].y - u0[f].y) + sdg * d2f_alu(u0[f].y);
      float2 du;
      du.x = (C1 * L.x + C2 * no[f].x) + (-C3 * pjy);
      du.y = (C1 * L.y + C2 * no[f].y) + (C3 * pjx);
      if (f == 0 && c == 0) du.x += (float)(-dR * mpgx);
      float2 n;
      n.x = xq[f].x + (fq[f].x - fm[f].x) * th * dd; n.y = xq[f].y + (fq[f].y - fm[f].y) * th * dd;
      (f ? Nu3o : Nu1o)[ou] = n;
      du.x += G * n.x; du.y += G * n.y;
      duib[((size_t)s * 3 + (f ? 2 : 0)) * nc + c] = du;
    }
  }
  if (qv > 0) {
    const int nv = g.nv;
    const float a = g.d2vf[qv], cc = g.d2vf[2 * nv + qv], sdg = g.sdgv[qv] + k2f;
    float2 L;
    L.x = a * d2f_alu(vm.x - v0.x) + cc * d2f_alu(vp.x - v0.x) + sdg * d2f_alu(v0.x);
    L.y = a * d2f_alu(vm.y - v0.y) + cc * d2f_alu(vp.y - v0.y) + sdg * d2f_alu(v0.y);
    const float C3 = -dRf * dd * g.thvf[qv];
    float2 du;
    du.x = (C1 * L.x + C2 * nov.x) + C3 * (d2f_alu(pp.x) - d2f_alu(pm.x));
    du.y = (C1 * L.y + C2 * nov.y) + C3 * (d2f_alu(pp.y) - d2f_alu(pm.y));
    const float th = g.thvf[qv];
    float2 n;
    n.x = xv.x + (vp1.x - vq.x) * th * dd; n.y = xv.y + (vp1.y - vq.y) * th * dd;
    Nu2o[ov] = n;
    du.x += G * n.x; du.y += G * n.y;
    duib[((size_t)s * 3 + 1) * nc + c] = du;
  }
}

// ============================================================================
// Immersed-boundary forcing in one x pass (imm_bounds_u/v, FOU3D.f90:806-998): the rows
// of du's planes (z pass done, A layout) go to physical space, the forced points of the
// rows are overwritten with Kib/dt (A u(i1,k1,j1) - u(i,k,j)) from the captured physical
// velocities, and the rows go back (B layout for the z pass). Forced points come as
// records sorted by (plane, row): rec_off[plane * G2 + row] .. rec_off[... + 1];
// cap [capslot][field][G2][G1] holds the physical u, v, w the x pass captured, in the
// transform precision (FP32 in the mixed form: the values are FP32 there).
// ============================================================================
struct IbRec {
  int i, k;        // 0-based point of the plane: x index, row
  long long src;   // cap offset of u at the point
  long long ref;   // cap offset of u at the reference point (i1, k1, j1)
  double A;
};
template <typename T, int N>
__global__ void __launch_bounds__(NTHR, LH_IBX_MINB) k_ib_xforce(const typename C2<T>::t *__restrict__ A, typename C2<T>::t *__restrict__ B,
                                                    Geo g, const typename C2<T>::t *__restrict__ twx,
                                                    const IbRec *__restrict__ rec, const int *__restrict__ rec_off,
                                                    const T *__restrict__ cap, const DevScalars *__restrict__ sc) {
  typedef typename C2<T>::t V;
  constexpr int PB = 4 * pb_xpass<V>(N);
  constexpr int G1 = N, H = N / 2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int G2 = g.G2, N1h = g.N1h;
  V *b0 = reinterpret_cast<V *>(smem_raw);
  V *b1 = b0 + PB * G1;
  const int pl = blockIdx.y, l0 = blockIdx.x * PB * 2;
  const int npairs = min(PB, (G2 - l0) / 2);
  const V *Ap = A + (size_t)pl * G2 * N1h;
  // one work item per retained x-mode (N1h = G1 / 3 + 1), the dealiasing band zeroed
  constexpr int NK = G1 / 3 + 1, NZ = G1 - 2 * NK + 1;
  static_assert(NK <= H, "retained x-modes below the Nyquist index");
  for (int idx = threadIdx.x; idx < PB * NK; idx += blockDim.x) {
    const int pb = idx / NK, k = idx - pb * NK;
    V zd = czero<V>(), zc = czero<V>();
    if (pb < npairs) {
      const int l = l0 + 2 * pb;
      V a = Ap[(size_t)l * NK + k], b = Ap[(size_t)(l + 1) * NK + k];
      if (k == 0) { a.y = 0; b.y = 0; }
      zd.x = a.x - b.y; zd.y = a.y + b.x;
      zc.x = a.x + b.y; zc.y = -a.y + b.x;
    }
    b0[pb * G1 + k] = zd;
    if (k > 0) b0[pb * G1 + G1 - k] = zc;
  }
  for (int idx = threadIdx.x; idx < PB * NZ; idx += blockDim.x) {
    const int pb = idx / NZ, m = idx - pb * NZ;
    b0[pb * G1 + NK + m] = czero<V>();
  }
  __syncthreads();
  V *res = line_fft<true, N, PB, false>(b0, b1, twx);
  V *oth = (res == b0) ? b1 : b0;
  {
    const double Kibdt = g.Kib / sc->dt;
    const float Kibdtf = d2f_alu(Kibdt);
    const int r0 = rec_off[(size_t)pl * G2 + l0], r1 = rec_off[(size_t)pl * G2 + l0 + 2 * npairs];
    for (int e = r0 + threadIdx.x; e < r1; e += blockDim.x) {
      const IbRec R = rec[e];
      T val;
      if constexpr (sizeof(T) == 4) {  // FP32 values: one rounding of A u_ref - u (fused), one of the scaling
        val = Kibdtf * fmaf(d2f_alu(R.A), cap[R.ref], -cap[R.src]);
      } else {
        val = Kibdt * (R.A * cap[R.ref] - cap[R.src]);
      }
      const int rr = R.k - l0;
      V *z = res + (rr >> 1) * G1 + R.i;
      if (rr & 1) z->y = val;
      else z->x = val;
    }
  }
  __syncthreads();
  V *fres = line_fft<false, N, PB, false>(res, oth, twx);
  const T s1 = (T)1 / (T)G1;
  for (int idx = threadIdx.x; idx < PB * 2 * N1h; idx += blockDim.x) {
    const int k = idx % N1h, rest = idx / N1h;
    const int half = rest & 1, pb = rest >> 1;
    if (pb >= npairs) continue;
    const V *L = fres + pb * G1;
    const V z = L[k], zc = cconj(L[k == 0 ? 0 : G1 - k]);
    V o;
    if (!half) { o.x = (T)0.5 * (z.x + zc.x) * s1; o.y = (T)0.5 * (z.y + zc.y) * s1; }
    else { o.x = (T)0.5 * (z.y - zc.y) * s1; o.y = (T)-0.5 * (z.x - zc.x) * s1; }
    if (k == 0) o.y = 0;
    B[((size_t)pl * G2 + l0 + 2 * pb + half) * N1h + k] = o;
  }
}


