// lh_xpass2.cuh — the x pass of the mixed form as a two-stage transform held in registers.
//
// Same work as k_xpass_nl (lh_kernels.cuh) for one level's plane: the inverse x transforms
// (rft, iopt >= 0) of u, v, w row pairs, the physical products of ops_in_planes2
// (FOU3D.f90:2090-2251), the CFL maxima (dtc_calc) and the forward x transforms (rft,
// iopt < 0) of the products, with the same A input and B output layouts. Two rows l, l+1 of
// a field travel as one complex line (row l in .x, row l+1 in .y).
//
// The length-N transform is split N = XA * XB with XB = 8 (Stockham, two stages):
//   inverse stage 1: XB threads per line, each an XA-point DFT of elements jj + XB t, read
//                    straight from A with the Hermitian completion (the gather) -> shared E1
//   inverse stage 2 + products + forward stage 1 (fused, registers): XA threads per row pair,
//                    thread jj holds physical points jj + XA t (t < 8) of at most two of u, v,
//                    w at a time, forms the products there and transforms them with the forward
//                    8-point DFT, written over the E1 elements it has read (a fourth line for a
//                    u level's fourth product)
//   forward stage 2: XB threads per product line, each an XA-point DFT; the thread holds
//                    outputs jj + XB t, the conjugate-symmetric partner N - k of every output k
//                    is in lane (XB - jj) mod XB of the same 8-lane group, fetched by shuffle,
//                    and the two rows of the pair are separated and written to B.
// So the block exchanges data through shared memory once per direction, and every element
// address inside a stage is an immediate offset from the thread's base.
#pragma once
#include "lh_internal.cuh"
#include "lh_regfft.cuh"

// Blocks per SM the compiler must leave registers for (the second __launch_bounds__ argument)
// of the x pass, the inverse z pass and the forward z pass: as many blocks as a register budget
// per thread allows (x pass 128; z passes 56, none from 768 on, whose 24- to 36-point register
// DFTs need more), capped (5 / 6 / 3). At 384 (the fastest of a sweep at 256²×301 with posts):
// x pass 5 blocks of 96 threads, inverse z pass 6 of 192, forward z pass 3 of 384.
// LH_*_MINB override them for sweeps.
#ifndef LH_SPECZ_MINB  // the z transforms of the immersed levels' du planes (sweep knob; 1: unconstrained)
#define LH_SPECZ_MINB(N) 1
#endif
__host__ __device__ constexpr int lh_minb(int threads, int regs, int cap) {
  const int b = 65536 / (regs * threads);
  return b < 1 ? 1 : (b > cap ? cap : b);
}

// row pairs per block (one block: 96 threads at N = 384)
template <int N> struct xp2 {
  static constexpr int XB = 8, XA = N / XB;
  static constexpr int PB = XA >= 36 ? 2 : (XA >= 18 ? 4 : 8);
  // threads: enough for every stage (fused: XA PB; the first and last stages: 3 and 4 lines x
  // PB pairs x XB), in whole warps (the shuffles of the fused and last stages)
  static constexpr int NT = ((XA * PB > 4 * PB * XB ? XA * PB : 4 * PB * XB) + 31) / 32 * 32;
  // padded shared-memory lines E1 (stage-1 output e = jj XA + t at e + e / XA; the fused stage's
  // outputs in place); line strides = 8 (mod 16) float2 so that the lanes of two lines fall on
  // different banks
  static constexpr int pad16(int v) { return v + ((8 - v % 16) + 16) % 16; }
  static constexpr int LS1 = pad16(N + N / XA);
  static constexpr int SMEM = 4 * LS1 * PB * 8;  // 3 field lines + 1 product line per pair
#ifdef LH_XPASS2_MINB
  static constexpr int MINB = LH_XPASS2_MINB;
#else
  static constexpr int MINB = lh_minb(NT, 128, 5);
#endif
};

template <int N>
__global__ void __launch_bounds__(xp2<N>::NT, xp2<N>::MINB) k_xpass2(const float2 *__restrict__ A, float2 *__restrict__ B, Geo g,
                                                        const float2 *__restrict__ tw, int doCFL, DevScalars *sc,
                                                        const int *__restrict__ capslot, float *__restrict__ cap) {
  using P = xp2<N>;
  constexpr int XA = P::XA, XB = P::XB, PB = P::PB, LS1 = P::LS1;
  constexpr int NK = N / 3 + 1;  // retained x-modes 0..N1/2 (N1 = 2 (Ngal1 / 3), checked at create)
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *E = reinterpret_cast<float2 *>(smem_raw);
  const int G2 = g.G2, N1h = g.N1h;
  const int slot = blockIdx.y;
  const bool isU = slot < g.nuI;
  const int q = slot_level(g, slot, isU);
  const int l0 = blockIdx.x * PB * 2;
  const int npairs = min(PB, (G2 - l0) / 2);
  const size_t fstride = (size_t)G2 * N1h;
  const int tid = threadIdx.x;

  // ---- inverse stage 1: line (f, pb), thread jj < 8: XA-point DFT of elements jj + 8 t ----
  if (tid < 3 * PB * XB) {
    const int line = tid / XB, jj = tid - line * XB;
    const int f = line / PB, pb = line - f * PB;
    float2 v[XA];
    if (pb < npairs) {
      const float2 *ra = A + (size_t)(slot * 3 + f) * fstride + (size_t)(l0 + 2 * pb) * N1h;
      const float2 *rb = ra + N1h;
      regfft::static_for<0, XA>([&](auto t_) {
        constexpr int t = decltype(t_)::value;
        // element m = jj + 8 t: retained mode k = m (m < NK), conjugate of mode N - m (m > N - NK), else 0
        constexpr int mlo = XB * t, mhi = XB * t + XB - 1;
        constexpr bool direct = mlo < NK, conj = mhi > N - NK;  // possible for some lane
        const int m = jj + mlo;
        float2 z = make_float2(0.f, 0.f);
        if (direct && m < NK) {
          float2 a = __ldg(ra + m), b = __ldg(rb + m);
          if (m == 0) { a.y = 0.f; b.y = 0.f; }
          z = make_float2(a.x - b.y, a.y + b.x);  // a + i b
        } else if (conj && m > N - NK) {
          const float2 a = __ldg(ra + (N - m)), b = __ldg(rb + (N - m));
          z = make_float2(a.x + b.y, -a.y + b.x);  // conj(a) + i conj(b)
        }
        v[t] = z;
      });
    } else {
      regfft::static_for<0, XA>([&](auto t_) { v[decltype(t_)::value] = make_float2(0.f, 0.f); });
    }
    regfft::dft_reg<XA, true>(v);
    float2 *e1 = E + line * LS1 + jj * (XA + 1);
    regfft::static_for<0, XA>([&](auto t_) { e1[decltype(t_)::value] = v[decltype(t_)::value]; });
  }
  __syncthreads();

  // ---- fused: inverse stage 2 (8-point DFTs), products, CFL maxima, forward stage 1 ----
  // thread (pb, jj) reads element jj of the 8 stage-1 regions of each field line (positions
  // jj + (XA + 1) t) and writes each product's 8 outputs back there, over a field line it has
  // finished reading (the positions only it reads; a u level's fourth product into line 3),
  // holding at most two fields: u level: v -> vv; u, w -> uu, uw, ww; v level: v; u -> uv; w -> wv
  const int pb = tid / XA, jj = tid - pb * XA;
  const bool act = pb < PB;  // the threads that round the block up to whole warps only take part in the shuffles
  const bool valid = act && pb < npairs;
  const int cs = (capslot && valid) ? capslot[slot] : -1;
  float m1 = 0.f, m2 = 0.f, m3 = 0.f;
  if (act) {
    // inverse stage 2 of field f: twiddles exp(+2 pi i jj t / N), 8-point DFT -> points jj + XA t
    auto field = [&](int f, float2 *ph) {
      const float2 *e1 = E + (f * PB + pb) * LS1 + jj;
#pragma unroll
      for (int t = 0; t < XB; ++t) {
        const float2 x = e1[t * (XA + 1)];
        if (t == 0) {
          ph[0] = x;
        } else {
          const float2 w = __ldg(tw + jj * t);
          ph[t] = make_float2(x.x * w.x + x.y * w.y, x.y * w.x - x.x * w.y);  // x * conj(w)
        }
      }
      regfft::dft_reg<XB, true>(ph);
      if (cs >= 0) {
        const int l = l0 + 2 * pb;
        float *cp = cap + ((size_t)cs * 3 + f) * (size_t)G2 * N + (size_t)l * N + jj;
#pragma unroll
        for (int t = 0; t < XB; ++t) {
          cp[t * XA] = ph[t].x;
          cp[N + t * XA] = ph[t].y;
        }
      }
    };
    // product of two fields (row a in .x, row b in .y), forward 8-point DFT, into line L
    auto product = [&](const float2 *x0, const float2 *x1, int L) {
      float2 pr[XB];
#pragma unroll
      for (int t = 0; t < XB; ++t) pr[t] = make_float2(x0[t].x * x1[t].x, x0[t].y * x1[t].y);
      regfft::dft_reg<XB, false>(pr);
      float2 *e = E + (L * PB + pb) * LS1 + jj;
#pragma unroll
      for (int t = 0; t < XB; ++t) e[t * (XA + 1)] = pr[t];
    };
    auto amax = [](const float2 *x) {
      float m = 0.f;
#pragma unroll
      for (int t = 0; t < XB; ++t) m = nmax(m, nmax(fabsf(x[t].x), fabsf(x[t].y)));
      return m;
    };
    float2 pa[XB], pc[XB];
    if (isU) {
      field(1, pa);
      product(pa, pa, 1);
      field(0, pa);
      field(2, pc);
      if (valid) { m1 = amax(pa); m3 = amax(pc); }
      product(pa, pa, 0);
      product(pa, pc, 3);
      product(pc, pc, 2);
    } else {
      field(1, pc);
      if (valid) m2 = amax(pc) * g.thvf[q];
      field(0, pa);
      product(pa, pc, 0);
      field(2, pa);
      product(pa, pc, 2);
    }
  }
  if (doCFL) {
    m1 = warp_max(m1); m2 = warp_max(m2); m3 = warp_max(m3);
    if ((tid & 31) == 0) {
      if (isU) { atomic_max_pos(&sc->u1m, f2d_alu(m1)); atomic_max_pos(&sc->u3m, f2d_alu(m3)); }
      else atomic_max_pos(&sc->u2m, f2d_alu(m2));
    }
  }
  __syncthreads();
  const int nprod = isU ? 4 : 2;

  // ---- forward stage 2: line (p, pb), thread jj < 8: twiddles, XA-point DFT of jj + 8 t ----
  if (tid < nprod * PB * XB) {
    const int line = tid / XB, jj2 = tid - line * XB;
    const int p = line / PB, pb2 = line - p * PB;
    const int L = isU ? (p == 0 ? 0 : p == 1 ? 3 : p == 2 ? 1 : 2) : (p == 0 ? 0 : 2);
    float2 v[XA];
    // element t (the fused thread t's output jj2) at position t + (XA + 1) jj2 of line L
    const float2 *e2 = E + (L * PB + pb2) * LS1 + jj2 * (XA + 1);
    regfft::static_for<0, XA>([&](auto t_) {
      constexpr int t = decltype(t_)::value;
      const float2 x = e2[t];
      if constexpr (t == 0) {
        v[0] = x;
      } else {
        const float2 w = __ldg(tw + jj2 * t);
        v[t] = make_float2(x.x * w.x - x.y * w.y, x.x * w.y + x.y * w.x);
      }
    });
    regfft::dft_reg<XA, false>(v);
    // outputs k = jj2 + 8 t; the partner N - k = (8 - jj2) + 8 (XA - 1 - t) sits in lane
    // (8 - jj2) mod 8 of this 8-lane group (lane jj2 = 0: its own entry XA - t)
    const int lane = tid & 31, src = (lane & ~(XB - 1)) | ((XB - jj2) & (XB - 1));
    const int pbase = isU ? slot * 4 : g.nuI * 4 + (slot - g.nuI) * 2;
    float2 *dst = B + (((size_t)(pbase + p) * (G2 / 2) + (l0 >> 1) + pb2) * N1h) * 2;
    const float s1 = 1.f / (float)N;
    const bool ok = pb2 < npairs;
    regfft::static_for<0, (NK + XB - 1) / XB>([&](auto t_) {
      constexpr int t = decltype(t_)::value;
      float2 zp;
      zp.x = __shfl_sync(0xffffffffu, v[XA - 1 - t].x, src);
      zp.y = __shfl_sync(0xffffffffu, v[XA - 1 - t].y, src);
      if (jj2 == 0) zp = t == 0 ? v[0] : v[(XA - t) % XA];
      const int k = jj2 + XB * t;
      if (ok && k < NK) {
        const float2 z = v[t];
        float4 o;
        o.x = 0.5f * (z.x + zp.x) * s1; o.y = 0.5f * (z.y - zp.y) * s1;   // (z + conj zp) / 2
        o.z = 0.5f * (z.y + zp.y) * s1; o.w = -0.5f * (z.x - zp.x) * s1;  // -i (z - conj zp) / 2
        if (k == 0) { o.y = 0.f; o.w = 0.f; }
        *reinterpret_cast<float4 *>(dst + (size_t)k * 2) = o;
      }
    });
  }
}

// ============================================================================
// The inverse z pass of the mixed form as a two-stage transform (the work of k_zinv_nl:
// stagger interpolation (interp_u/v, FOU3D.f90:427-474) and the inverse z transforms (cft,
// iopt >= 0) of one field's kx columns at one level, written to A [slot*3 + f][l][kx]).
// N = ZA * ZB; stage 1: ZB threads per line, each a ZA-point DFT of rows jj + ZB t, gathered
// straight from the FP64 state (retained kz rows only; the dealiasing rows are zero and the
// loads of the rows that are zero for every lane are left out at compile time); stage 2: ZA
// threads per line, each a ZB-point DFT, writing rows jj + ZA t of A. KB kx lines per block,
// kx the fastest thread index (coalesced state loads and A stores).
// ============================================================================
template <int N> struct zp2 {
  static constexpr int ZA = N == 24 ? 4 : N == 48 ? 6 : N == 72 ? 8 : N == 96 ? 8 : N == 144 ? 12 : N == 192 ? 12
                          : N == 288 ? 16 : N == 384 ? 16 : N == 576 ? 24 : N == 768 ? 24 : 32;
  static constexpr int ZB = N / ZA;
#ifdef LH_ZP2_KB
  static constexpr int KB = LH_ZP2_KB;
#else
  static constexpr int KB = 8;
#endif
  static constexpr int NT = ((ZA > ZB ? ZA : ZB) * KB + 31) / 32 * 32;
  static constexpr int SMEM = (N + ZB) * KB * 8;  // float2, one pad element per ZA-block
#ifdef LH_ZINV2_MINB
  static constexpr int MINB = LH_ZINV2_MINB;
#else
  static constexpr int MINB = lh_minb(NT, N >= 768 ? 255 : 56, 6);
#endif
};

// The two stages of the inverse z pass for one block of KB kx columns: gather(r, kx) gives
// spectral row r (0..N2-1) of column kx in FP32; the physical rows l go to dst[l * N1h + kx].
template <int N, typename Gather>
__device__ __forceinline__ void zinv2_body(Gather &&gather, float2 *__restrict__ dst, int N1h, int kx0,
                                           const float2 *__restrict__ tw) {
  using P = zp2<N>;
  constexpr int ZA = P::ZA, ZB = P::ZB, KB = P::KB;
  static_assert(ZA * ZB == N, "z plan");
  constexpr int H = N / 3;  // N2 / 2 retained kz rows on each side (N2 = 2 (Ngal2 / 3), checked at create)
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *E = reinterpret_cast<float2 *>(smem_raw);
  const int tid = threadIdx.x;
  if (tid < ZB * KB) {
    const int jj = tid / KB, kk = tid - jj * KB, kx = kx0 + kk;
    float2 v[ZA];
    const bool ok = kx < N1h;
    regfft::static_for<0, ZA>([&](auto t_) {
      constexpr int t = decltype(t_)::value;
      constexpr int mlo = ZB * t, mhi = ZB * t + ZB - 1;
      constexpr bool lo = mlo < H, hi = mhi >= N - H;  // possible for some lane
      const int m = jj + mlo;
      float2 z = make_float2(0.f, 0.f);
      int r = -1;
      if (lo && m < H) r = m;
      else if (hi && m >= N - H) r = m - N + 2 * H;
      if ((lo || hi) && ok && r >= 0) z = gather(r, kx);
      v[t] = z;
    });
    regfft::dft_reg<ZA, true>(v);
    float2 *e = E + jj * (ZA + 1) * KB + kk;
    regfft::static_for<0, ZA>([&](auto t_) { e[decltype(t_)::value * KB] = v[decltype(t_)::value]; });
  }
  __syncthreads();
  if (tid < ZA * KB) {
    const int jj = tid / KB, kk = tid - jj * KB, kx = kx0 + kk;
    float2 v[ZB];
    const float2 *e = E + jj * KB + kk;
    regfft::static_for<0, ZB>([&](auto t_) {
      constexpr int t = decltype(t_)::value;
      const float2 x = e[t * (ZA + 1) * KB];
      if constexpr (t == 0) {
        v[0] = x;
      } else {
        const float2 w = __ldg(tw + jj * t);  // conj: the inverse direction
        v[t] = make_float2(x.x * w.x + x.y * w.y, x.y * w.x - x.x * w.y);
      }
    });
    regfft::dft_reg<ZB, true>(v);
    if (kx < N1h) {
      regfft::static_for<0, ZB>([&](auto t_) {
        constexpr int t = decltype(t_)::value;
        dst[(size_t)(jj + ZA * t) * N1h + kx] = v[t];
      });
    }
  }
}

template <int N>
__global__ void __launch_bounds__(zp2<N>::NT, zp2<N>::MINB) k_zinv2(const double2 *__restrict__ u1, const double2 *__restrict__ u2,
                                                       const double2 *__restrict__ u3, float2 *__restrict__ A, Geo g,
                                                       const float2 *__restrict__ tw) {
  const int slot = zinv_slot(g, blockIdx.y), f = blockIdx.z, kx0 = blockIdx.x * zp2<N>::KB;
  const bool isU = slot < g.nuI;
  const int q = slot_level(g, slot, isU);
  const size_t nc = g.ncolF;
  // field f at level q (interpolated to the level's grid), FP32
  const double2 *s0, *s1 = nullptr;
  float ca = 1.f, cb = 0.f;
  size_t o0 = (size_t)q * nc, o1 = 0;
  if (isU) {
    if (f == 0) s0 = u1;
    else if (f == 2) s0 = u3;
    else { s0 = u2; s1 = u2; o1 = (size_t)(q - 1) * nc; ca = g.iuaf[q]; cb = g.iubf[q]; }  // v faces -> centre
  } else {
    if (f == 1) s0 = u2;
    else { s0 = s1 = (f == 0) ? u1 : u3; o0 = (size_t)(q + 1) * nc; o1 = (size_t)q * nc; ca = g.ivaf[q]; cb = g.ivbf[q]; }
  }
  auto gather = [&](int r, int kx) {
    const int c = gcol(g, r, kx);
    const double2 a = s0[o0 + c];
    if (s1) {
      const double2 b = s1[o1 + c];
      return make_float2(ca * d2f_alu(a.x) + cb * d2f_alu(b.x), ca * d2f_alu(a.y) + cb * d2f_alu(b.y));
    }
    return make_float2(d2f_alu(a.x), d2f_alu(a.y));
  };
  zinv2_body<N>(gather, A + (size_t)(slot * 3 + f) * N * g.N1h, g.N1h, kx0, tw);
}

// The inverse z transforms of spectral planes [pl][N2][N1h] complex64 (the immersed-boundary
// du planes of the mixed form) into A [pl][l][kx] in FP32, as k_spec_zinv<float, N>.
template <int N>
__global__ void __launch_bounds__(zp2<N>::NT, LH_SPECZ_MINB(N)) k_spec_zinv2(const float2 *__restrict__ spec, float2 *__restrict__ A,
                                                            Geo g, const float2 *__restrict__ tw) {
  const int pl = blockIdx.y, kx0 = blockIdx.x * zp2<N>::KB;
  const float2 *S = spec + (size_t)pl * g.ncol;
  const int N1h = g.N1h;
  auto gather = [&](int r, int kx) { return S[(size_t)r * N1h + kx]; };
  zinv2_body<N>(gather, A + (size_t)pl * N * N1h, N1h, kx0, tw);
}

// ============================================================================
// The forward z pass of the mixed form as a two-stage transform (the work of k_zfwd_nl:
// forward z transforms (cft, iopt < 0) of the x pass's products and der_x / der_z,
// FOU3D.f90:476-593, 2253-2272). Per block: KF kx columns of the NP products of one level
// (u level: uu, uw, vv, ww -> N1xz, N3xz, vvc; v level: uv, wv -> N2xz, uvf, wvf).
// Stage 1: ZA threads per line, each a ZB-point DFT of rows jj + ZA t read from B (the two
// rows of a pair adjacent there); stage 2: ZB threads per line, each a ZA-point DFT; the
// retained kz rows go to shared memory, where one thread per (row, kx) combines the products.
// ============================================================================
template <int N> struct zf2 {
  using Z = zp2<N>;
  static constexpr int ZA = Z::ZA, ZB = Z::ZB, KF = 4;
  static constexpr int NTH = ((ZA > ZB ? ZA : ZB) * 4 * KF + 31) / 32 * 32;
  // line stride of the stage-1 output (e = jj ZB + t at e + e / ZB), = 4 (mod 16) float2 so that
  // the KF lines of a half-warp start 8 banks apart
  static constexpr int LSE = (N + N / ZB) + ((4 - (N + N / ZB) % 16) + 16) % 16;
  static constexpr int SMEM = 4 * KF * LSE * 8;
#ifdef LH_ZFWD2_MINB
  static constexpr int MINB = LH_ZFWD2_MINB;
#else
  static constexpr int MINB = lh_minb(NTH, N >= 768 ? 255 : 56, 3);
#endif
};

template <int N>
__global__ void __launch_bounds__(zf2<N>::NTH, zf2<N>::MINB) k_zfwd2(const float2 *__restrict__ B, Geo g, const float2 *__restrict__ tw,
                                                        float2 *__restrict__ N1xz, float2 *__restrict__ N2xz,
                                                        float2 *__restrict__ N3xz, float2 *__restrict__ uvf,
                                                        float2 *__restrict__ vvc, float2 *__restrict__ wvf) {
  using P = zf2<N>;
  constexpr int ZA = P::ZA, ZB = P::ZB, KF = P::KF, LSE = P::LSE;
  constexpr int H = N / 3;  // N2 / 2
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *E = reinterpret_cast<float2 *>(smem_raw);
  const int slot = blockIdx.y;
  const bool isU = slot < g.nuI;
  // a v level has two products: its blocks take twice the kx lines (the grid's second half
  // of v-level blocks has none and returns), so that every level fills the block
  const int NP = isU ? 4 : 2, KE = isU ? KF : 2 * KF;
  const int kx0 = blockIdx.x * KE;
  const int N1h = g.N1h;
  if (kx0 >= N1h) return;
  const int q = slot_level(g, slot, isU);
  const int pbase = isU ? slot * 4 : g.nuI * 4 + (slot - g.nuI) * 2;
  const int tid = threadIdx.x;
  // stage 1: thread (p, jj, kk), kk fastest
  if (tid < NP * ZA * KE) {
    const int kk = tid % KE, r1 = tid / KE, jj = r1 % ZA, p = r1 / ZA, kx = kx0 + kk;
    float2 v[ZB];
    const float2 *src = B + ((size_t)(pbase + p) * (N / 2) * N1h + kx) * 2;
    const bool ok = kx < N1h;
    regfft::static_for<0, ZB>([&](auto t_) {
      constexpr int t = decltype(t_)::value;
      const int l = jj + ZA * t;
      v[t] = ok ? src[(size_t)(l >> 1) * N1h * 2 + (l & 1)] : make_float2(0.f, 0.f);
    });
    regfft::dft_reg<ZB, false>(v);
    float2 *e = E + (p * KE + kk) * LSE + jj * (ZB + 1);
    regfft::static_for<0, ZB>([&](auto t_) { e[decltype(t_)::value] = v[decltype(t_)::value]; });
  }
  __syncthreads();
  // stage 2: thread (p, jj2, kk); the inputs are read before the block reuses E for the rows
  const bool s2 = tid < NP * ZB * KE;
  const int kk = tid % KE, r2 = tid / KE, jj2 = r2 % ZB, p = r2 / ZB;
  float2 v[ZA];
  if (s2) {
    const float2 *e = E + (p * KE + kk) * LSE + jj2;
    regfft::static_for<0, ZA>([&](auto t_) {
      constexpr int t = decltype(t_)::value;
      const float2 x = e[t * (ZB + 1)];
      if constexpr (t == 0) {
        v[0] = x;
      } else {
        const float2 w = __ldg(tw + jj2 * t);
        v[t] = make_float2(x.x * w.x - x.y * w.y, x.x * w.y + x.y * w.x);
      }
    });
  }
  __syncthreads();
  float2 *R = E;  // [p][r][kk], the 2H retained kz rows
  if (s2) {
    regfft::dft_reg<ZA, false>(v);
    regfft::static_for<0, ZA>([&](auto t_) {
      constexpr int t = decltype(t_)::value;
      constexpr int mlo = ZB * t, mhi = ZB * t + ZB - 1;
      const int m = jj2 + mlo;
      int r = -1;
      if (mlo < H && m < H) r = m;
      else if (mhi >= N - H && m >= N - H) r = m - N + 2 * H;
      if (r >= 0) R[((size_t)p * 2 * H + r) * KE + kk] = v[t];
    });
  }
  __syncthreads();
  // der_x / der_z and the stores, one thread per (kz row, kx)
  const float s = 1.f / (float)N;
  const size_t off = (size_t)q * g.ncolF;
  for (int idx = tid; idx < 2 * H * KE; idx += blockDim.x) {
    const int r = idx / KE, k2 = idx - r * KE, kx = kx0 + k2;
    if (kx >= N1h) continue;
    const int c = gcol(g, r, kx), rg = grow(g, r);
    const float kxv = g.k1xf[kx], kzv = g.k1zf[rg];
    const bool zr = (r == H);  // der_x / der_z zero the kz = -N2/2 row
    if (isU) {
      const float2 uu = cscale(R[((size_t)0 * 2 * H + r) * KE + k2], s), uw = cscale(R[((size_t)1 * 2 * H + r) * KE + k2], s);
      const float2 vv = cscale(R[((size_t)2 * 2 * H + r) * KE + k2], s), ww = cscale(R[((size_t)3 * 2 * H + r) * KE + k2], s);
      float2 n1 = make_float2(0.f, 0.f), n3 = make_float2(0.f, 0.f);
      if (!zr) {
        n1 = cadd(cimul(kxv, uu), cimul(kzv, uw));
        n3 = cadd(cimul(kxv, uw), cimul(kzv, ww));
      }
      N1xz[off + c] = n1;
      N3xz[off + c] = n3;
      vvc[off + c] = vv;
    } else {
      const float2 uv = cscale(R[((size_t)0 * 2 * H + r) * KE + k2], s), wv = cscale(R[((size_t)1 * 2 * H + r) * KE + k2], s);
      float2 n2 = make_float2(0.f, 0.f);
      if (!zr) n2 = cadd(cimul(kxv, uv), cimul(kzv, wv));
      N2xz[off + c] = n2;
      uvf[off + c] = uv;
      wvf[off + c] = wv;
    }
  }
}

// ============================================================================
// The forward z transforms of physical-x planes B [pl][l][kx] (FP32) into spectral planes
// [pl][N2][N1h] complex64, x 1/N, the retained kz rows only (as k_zfwd_spec<float, N>).
// ============================================================================
template <int N>
__global__ void __launch_bounds__(zp2<N>::NT, LH_SPECZ_MINB(N)) k_zfwd_spec2(const float2 *__restrict__ Bp, float2 *__restrict__ spec,
                                                            Geo g, const float2 *__restrict__ tw) {
  using P = zp2<N>;
  // the inverse pass's plan read backwards: stage 1 ZA threads per line (ZB-point DFTs of rows
  // jj + ZA t), stage 2 ZB threads per line (ZA-point DFTs), KB kx lines per block
  constexpr int ZA = P::ZA, ZB = P::ZB, KB = P::KB;
  constexpr int H = N / 3;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *E = reinterpret_cast<float2 *>(smem_raw);
  const int pl = blockIdx.y, kx0 = blockIdx.x * KB, N1h = g.N1h;
  const float2 *src = Bp + (size_t)pl * N * N1h;
  const int tid = threadIdx.x;
  if (tid < ZA * KB) {
    const int jj = tid / KB, kk = tid - jj * KB, kx = kx0 + kk;
    float2 v[ZB];
    const bool ok = kx < N1h;
    regfft::static_for<0, ZB>([&](auto t_) {
      constexpr int t = decltype(t_)::value;
      v[t] = ok ? src[(size_t)(jj + ZA * t) * N1h + kx] : make_float2(0.f, 0.f);
    });
    regfft::dft_reg<ZB, false>(v);
    float2 *e = E + jj * (ZB + 1) * KB + kk;  // e = jj ZB + t at e + e / ZB
    regfft::static_for<0, ZB>([&](auto t_) { e[decltype(t_)::value * KB] = v[decltype(t_)::value]; });
  }
  __syncthreads();
  if (tid < ZB * KB) {
    const int jj2 = tid / KB, kk = tid - jj2 * KB, kx = kx0 + kk;
    float2 v[ZA];
    const float2 *e = E + jj2 * KB + kk;
    regfft::static_for<0, ZA>([&](auto t_) {
      constexpr int t = decltype(t_)::value;
      const float2 x = e[t * (ZB + 1) * KB];
      if constexpr (t == 0) {
        v[0] = x;
      } else {
        const float2 w = __ldg(tw + jj2 * t);
        v[t] = make_float2(x.x * w.x - x.y * w.y, x.x * w.y + x.y * w.x);
      }
    });
    regfft::dft_reg<ZA, false>(v);
    if (kx < N1h) {
      const float s = 1.f / (float)N;
      float2 *dst = spec + (size_t)pl * g.ncol + kx;
      regfft::static_for<0, ZA>([&](auto t_) {
        constexpr int t = decltype(t_)::value;
        constexpr int mlo = ZB * t, mhi = ZB * t + ZB - 1;
        const int m = jj2 + mlo;
        int r = -1;
        if (mlo < H && m < H) r = m;
        else if (mhi >= N - H && m >= N - H) r = m - N + 2 * H;
        if (r >= 0) dst[(size_t)r * N1h] = make_float2(v[t].x * s, v[t].y * s);
      });
    }
  }
}

// ============================================================================
// The x pass of the mixed form at the long lengths (576, 768, 1152) as a three-stage register
// transform, N = XA * XM * 8, one row pair per block (the work of k_xpass_nl, same A and B
// layouts). Stages, each a register DFT between padded shared-memory lines:
//   inverse: XA-point DFTs gathered straight from A (Hermitian completion) -> XM-point DFTs ->
//            8-point DFTs fused with the products, the CFL maxima and the forward 8-point DFTs
//   forward: -> XM-point DFTs -> XA-point DFTs -> natural order, from where the two rows of the
//            pair are separated (output k with its partner N - k) into B.
// The element e of a stage's output sits at e + e / D in its line (D the stage's contiguous
// block), so the lanes of one store or load fall on different banks.
// ============================================================================
template <int N> struct xp3 {
  static constexpr int XA = N == 576 ? 12 : 16, XM = N / (8 * XA), XB = 8;
  static constexpr int L1 = N / XA, LM = N / XM, LB = N / XB;  // threads per line of the stages
  static constexpr int NT = 288;  // the fused stage's 2 LB work items in one round at 1152
  static constexpr int pad16(int v) { return v + ((8 - v % 16) + 16) % 16; }
  static constexpr int LS = pad16(N + N / 8 + 1);            // line stride (float2), >= every padded size
  static constexpr int SMEM = 2 * 4 * LS * 8;                // two buffers of 4 lines
#ifdef LH_XPASS3_MINB
  static constexpr int MINB = LH_XPASS3_MINB;
#else
  static constexpr int MINB = 3;  // 72 registers, no spills (1 block per SM unconstrained: 105 registers, 1.8x slower)
#endif
};

template <int N>
__global__ void __launch_bounds__(xp3<N>::NT, xp3<N>::MINB) k_xpass3(const float2 *__restrict__ A, float2 *__restrict__ B, Geo g,
                                                        const float2 *__restrict__ tw, int doCFL, DevScalars *sc,
                                                        const int *__restrict__ capslot, float *__restrict__ cap) {
  using P = xp3<N>;
  constexpr int XA = P::XA, XM = P::XM, XB = P::XB, L1 = P::L1, LM = P::LM, LB = P::LB, NT = P::NT, LS = P::LS;
  static_assert(XA * XM * XB == N, "x plan");
  constexpr int NK = N / 3 + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *BA = reinterpret_cast<float2 *>(smem_raw), *BB = BA + 4 * LS;  // the two buffers [line][LS]
  const int G2 = g.G2, N1h = g.N1h;
  const int slot = blockIdx.y;
  const bool isU = slot < g.nuI;
  const int q = slot_level(g, slot, isU);
  const int l = blockIdx.x * 2;  // the row pair (l, l + 1)
  const size_t fstride = (size_t)G2 * N1h;
  const int tid = threadIdx.x;
  // ---- inverse stage 1 (XA-point, Ns = 1): line f, thread j < L1, elements j + L1 t -> BA at e + e / XA ----
  for (int it = tid; it < 3 * L1; it += NT) {
    const int f = it / L1, j = it - f * L1;
    const float2 *ra = A + (size_t)(slot * 3 + f) * fstride + (size_t)l * N1h, *rb = ra + N1h;
    float2 v[XA];
    regfft::static_for<0, XA>([&](auto t_) {
      constexpr int t = decltype(t_)::value;
      constexpr int mlo = L1 * t, mhi = L1 * t + L1 - 1;
      constexpr bool direct = mlo < NK, conj = mhi > N - NK;
      const int m = j + mlo;
      float2 z = make_float2(0.f, 0.f);
      if (direct && m < NK) {
        float2 a = __ldg(ra + m), b = __ldg(rb + m);
        if (m == 0) { a.y = 0.f; b.y = 0.f; }
        z = make_float2(a.x - b.y, a.y + b.x);
      } else if (conj && m > N - NK) {
        const float2 a = __ldg(ra + (N - m)), b = __ldg(rb + (N - m));
        z = make_float2(a.x + b.y, -a.y + b.x);
      }
      v[t] = z;
    });
    regfft::dft_reg<XA, true>(v);
    float2 *o = BA + f * LS + j * (XA + 1);  // e = j XA + t
    regfft::static_for<0, XA>([&](auto t_) { o[decltype(t_)::value] = v[decltype(t_)::value]; });
  }
  __syncthreads();
  // ---- inverse stage 2 (XM-point, Ns = XA): thread j < LM, k = j % XA, elements j + LM t ----
  for (int it = tid; it < 3 * LM; it += NT) {
    const int f = it / LM, j = it - f * LM, k = j % XA;
    float2 v[XM];
    const float2 *in = BA + f * LS;
    regfft::static_for<0, XM>([&](auto t_) {
      constexpr int t = decltype(t_)::value;
      const int e = j + LM * t;
      const float2 x = in[e + e / XA];
      if constexpr (t == 0) {
        v[0] = x;
      } else {
        const float2 w = __ldg(tw + k * t * XB);  // exp(+2 pi i k t / (XA XM)): conj of the table
        v[t] = make_float2(x.x * w.x + x.y * w.y, x.y * w.x - x.x * w.y);
      }
    });
    regfft::dft_reg<XM, true>(v);
    float2 *o = BB + f * LS;
    const int base = (j / XA) * XA * XM + k;
    regfft::static_for<0, XM>([&](auto t_) {
      constexpr int t = decltype(t_)::value;
      const int e = base + XA * t;
      o[e + e / (XA * XM)] = v[t];
    });
  }
  __syncthreads();
  // ---- fused: inverse stage 3 (8-point, Ns = LB), products, CFL, forward stage 1 -> BA at e + e / 8 ----
  // two work items per point set j, each holding at most two fields: u level: (u, w -> uu, uw,
  // ww) and (v -> vv); v level: (u, v -> uv) and (w, v -> wv), v transformed by both
  const int nprod = isU ? 4 : 2;
  const int cs = capslot ? capslot[slot] : -1;
  float m1 = 0.f, m2 = 0.f, m3 = 0.f;
  for (int it = tid; it < 2 * LB; it += NT) {
    const int grp = it / LB, j = it - grp * LB;
    float2 w[XB];
    w[0] = make_float2(1.f, 0.f);
    regfft::static_for<1, XB>([&](auto t_) {
      constexpr int t = decltype(t_)::value;
      const float2 x = __ldg(tw + j * t);
      w[t] = make_float2(x.x, -x.y);
    });
    // inverse stage 3 of field f -> physical points j + LB t (captured for the forcing if asked)
    auto field = [&](int f, float2 *ph, bool capture) {
      const float2 *in = BB + f * LS;
      regfft::static_for<0, XB>([&](auto t_) {
        constexpr int t = decltype(t_)::value;
        const int e = j + LB * t;
        const float2 x = in[e + e / (XA * XM)];
        ph[t] = t == 0 ? x : make_float2(x.x * w[t].x - x.y * w[t].y, x.x * w[t].y + x.y * w[t].x);
      });
      regfft::dft_reg<XB, true>(ph);
      if (capture && cs >= 0) {
        float *cp = cap + ((size_t)cs * 3 + f) * (size_t)G2 * N + (size_t)l * N + j;
        regfft::static_for<0, XB>([&](auto t_) {
          constexpr int t = decltype(t_)::value;
          cp[t * LB] = ph[t].x;
          cp[N + t * LB] = ph[t].y;
        });
      }
    };
    // product of two fields (row l in .x, row l + 1 in .y), forward 8-point DFT -> BA line p
    auto product = [&](const float2 *x0, const float2 *x1, int p) {
      float2 pr[XB];
#pragma unroll
      for (int t = 0; t < XB; ++t) pr[t] = make_float2(x0[t].x * x1[t].x, x0[t].y * x1[t].y);
      regfft::dft_reg<XB, false>(pr);
      float2 *o = BA + p * LS + j * (XB + 1);  // e = j 8 + t
#pragma unroll
      for (int t = 0; t < XB; ++t) o[t] = pr[t];
    };
    auto amax = [](const float2 *x) {
      float m = 0.f;
#pragma unroll
      for (int t = 0; t < XB; ++t) m = nmax(m, nmax(fabsf(x[t].x), fabsf(x[t].y)));
      return m;
    };
    float2 pa[XB], pc[XB];
    if (isU) {
      if (grp == 0) {
        field(0, pa, true);
        field(2, pc, true);
        if (doCFL) { m1 = nmax(m1, amax(pa)); m3 = nmax(m3, amax(pc)); }
        product(pa, pa, 0);
        product(pa, pc, 1);
        product(pc, pc, 3);
      } else {
        field(1, pa, true);
        product(pa, pa, 2);
      }
    } else {
      field(1, pc, grp == 0);
      if (grp == 0) {
        if (doCFL) m2 = nmax(m2, amax(pc) * g.thvf[q]);
        field(0, pa, true);
        product(pa, pc, 0);
      } else {
        field(2, pa, true);
        product(pa, pc, 1);
      }
    }
  }
  if (doCFL) {
    m1 = warp_max(m1); m2 = warp_max(m2); m3 = warp_max(m3);
    if ((tid & 31) == 0) {
      if (isU) { atomic_max_pos(&sc->u1m, f2d_alu(m1)); atomic_max_pos(&sc->u3m, f2d_alu(m3)); }
      else atomic_max_pos(&sc->u2m, f2d_alu(m2));
    }
  }
  __syncthreads();
  // ---- forward stage 2 (XM-point, Ns = 8): thread j < LM, k = j % 8, elements j + LM t -> BB at e + e / (8 XM) ----
  for (int it = tid; it < nprod * LM; it += NT) {
    const int p = it / LM, j = it - p * LM, k = j % XB;
    float2 v[XM];
    const float2 *in = BA + p * LS;
    regfft::static_for<0, XM>([&](auto t_) {
      constexpr int t = decltype(t_)::value;
      const int e = j + LM * t;
      const float2 x = in[e + e / XB];
      if constexpr (t == 0) {
        v[0] = x;
      } else {
        const float2 w = __ldg(tw + k * t * XA);  // exp(-2 pi i k t / (8 XM))
        v[t] = make_float2(x.x * w.x - x.y * w.y, x.x * w.y + x.y * w.x);
      }
    });
    regfft::dft_reg<XM, false>(v);
    float2 *o = BB + p * LS;
    const int base = (j / XB) * XB * XM + k;
    regfft::static_for<0, XM>([&](auto t_) {
      constexpr int t = decltype(t_)::value;
      const int e = base + XB * t;
      o[e + e / (XB * XM)] = v[t];
    });
  }
  __syncthreads();
  // ---- forward stage 3 (XA-point, Ns = 8 XM = L1): thread j < L1, elements j + L1 t -> BA natural (k + k / 32) ----
  for (int it = tid; it < nprod * L1; it += NT) {
    const int p = it / L1, j = it - p * L1;
    float2 v[XA];
    const float2 *in = BB + p * LS;
    regfft::static_for<0, XA>([&](auto t_) {
      constexpr int t = decltype(t_)::value;
      const int e = j + L1 * t;
      const float2 x = in[e + e / (XB * XM)];
      if constexpr (t == 0) {
        v[0] = x;
      } else {
        const float2 w = __ldg(tw + j * t);
        v[t] = make_float2(x.x * w.x - x.y * w.y, x.x * w.y + x.y * w.x);
      }
    });
    regfft::dft_reg<XA, false>(v);
    float2 *o = BA + p * LS;
    regfft::static_for<0, XA>([&](auto t_) {
      constexpr int t = decltype(t_)::value;
      const int k = j + L1 * t;
      o[k + k / 32] = v[t];
    });
  }
  __syncthreads();
  // ---- the two rows of the pair: output k with its partner N - k, written to B ----
  const int pbase = isU ? slot * 4 : g.nuI * 4 + (slot - g.nuI) * 2;
  const float s1 = 1.f / (float)N;
  for (int it = tid; it < nprod * NK; it += NT) {
    const int p = it / NK, k = it - p * NK;
    const float2 *L = BA + p * LS;
    const int kp = k == 0 ? 0 : N - k;
    const float2 z = L[k + k / 32], zp = L[kp + kp / 32];
    float4 o;
    o.x = 0.5f * (z.x + zp.x) * s1; o.y = 0.5f * (z.y - zp.y) * s1;
    o.z = 0.5f * (z.y + zp.y) * s1; o.w = -0.5f * (z.x - zp.x) * s1;
    if (k == 0) { o.y = 0.f; o.w = 0.f; }
    float2 *dst = B + (((size_t)(pbase + p) * (G2 / 2) + (l >> 1)) * N1h + k) * 2;
    *reinterpret_cast<float4 *>(dst) = o;
  }
}
