// lh_triads.cuh — triad-list nonlinear term (the reference's as-run form):
// ops_in_planes + nonlinInter (FOU3D.f90:1724-2088) over the lists nonlinRead loads
// (start.f90:2983-3069).
//
// For every product X of a plane, and every target mode t = (lt, kt) with lt in
// 0..nx, kt in -nz..nz:
//   X(t) = linear advection (FOU3D.f90:1781-1800, 1926-1937)
//        + [t = (0,0) of vv, uv, wv] zeroth-mode sum (FOU3D.f90:1755-1772, 1902-1920)
//        + sum over the listed triads that land on t, in list order (nonlinInter).
// A list triad (la, ka, lp, kp) lands twice: pass p = 0 on (la+lp, -(ka+kp)) from
// A(la,-ka) P(lp,-kp), pass p = 1 on (la+lp, ka+kp) from A(la,ka) P(lp,kp) (p = 1
// skipped when ka+kp = 0). A mode with l < 0 is conj of mode (|l|, -k).
//
// GPU layout. On the host each list is expanded into its terms, grouped by target
// with a stable counting sort (so every target sums its terms in the reference's
// order), and laid out warp-striped: the 32 targets of a warp own rows of 32
// terms, row i holding term i of each lane (padding terms read a zero slot), so
// every warp load of terms is one coalesced 128-byte line. Targets are assigned to
// thread slots in decreasing order of their complete-list term count, so the lanes
// of a warp carry similar counts and little padding. A term is 32 bits:
// two 15-bit shared-memory indices (field * P + row * (N1/2+1) + |l|) and two
// conjugate flags. One block per plane stages the plane's three velocity fields
// (interpolated where the stagger needs it, FOU3D.f90:427-474) in shared memory;
// one thread per target accumulates its five (u planes) or four (v planes)
// products and writes the x/z derivatives (der_x, der_z) and the y-flux products
// in the layout the Helmholtz kernels read.
#pragma once
#include <stdint.h>

#include <algorithm>
#include <string>
#include <vector>

#include "lh_internal.cuh"

struct TriadGeo {
  const uint32_t *terms;  // warp-striped term rows, 32 terms per row
  const int *wb;          // [nlists][Tw+1] first row of each warp of each expanded list
  const int *lid;         // [(nu + nv) * 9] expanded list of (level, type), -1 if none
  const int *tmap;        // [T] target of each thread slot (slots ordered by expected term count)
  int Tw, T, nx, nz, P;   // warps, targets, list header, plane size (N2 * (N1/2+1))
};

__host__ __device__ __forceinline__ int tri_krow(int k, int N2) { return k >= 0 ? k : k + N2; }

// conjugation by flipping the sign bit on the integer pipe
__device__ __forceinline__ double tri_flip(double v, uint32_t code) {
  return __longlong_as_double(__double_as_longlong(v) ^ ((long long)(code & 0x8000u) << 48));
}
__device__ __forceinline__ float tri_flip(float v, uint32_t code) {
  return __int_as_float(__float_as_int(v) ^ (int)((code & 0x8000u) << 16));
}
__device__ __forceinline__ double tri_fma(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float tri_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }

template <typename V>
__device__ __forceinline__ V tri_ld(const V *F, uint32_t code) {
  V a = F[code & 0x7fffu];
  a.y = tri_flip(a.y, code);
  return a;
}

// acc += a * p, in the reference's order: re (+ ar pr) (- ai pi), im (+ ar pi) (+ ai pr)
template <typename V>
__device__ __forceinline__ void tri_mac(V &acc, V a, V p) {
  acc.x = tri_fma(a.x, p.x, acc.x);
  acc.x = tri_fma(-a.y, p.y, acc.x);
  acc.y = tri_fma(a.x, p.y, acc.y);
  acc.y = tri_fma(a.y, p.x, acc.y);
}

template <typename V>
__device__ __forceinline__ void tri_list(V &acc, const V *F, const TriadGeo &tg, int lid, int w, int lane) {
  const int *wb = tg.wb + (size_t)lid * (tg.Tw + 1);
  const int r0 = wb[w], r1 = wb[w + 1];
  const uint32_t *t = tg.terms + (size_t)r0 * 32 + lane;
  for (int r = r0; r < r1; ++r, t += 32) {
    const uint32_t code = __ldg(t);
    tri_mac(acc, tri_ld(F, code), tri_ld(F, code >> 16));
  }
}

// zeroth mode: sum over i = -N1/2..N1/2, k = klo..N2/2-1 of A(i, k) P(-i, -k)
template <typename V>
__device__ V tri_zeroth(const V *A, const V *Pf, int klo, int N1, int N2, int N1h) {
  V acc;
  acc.x = 0;
  acc.y = 0;
  for (int i = -(N1 / 2); i <= N1 / 2; ++i) {
    const int ia = i < 0 ? -i : i;
    const bool ca = i < 0, cp = -i < 0;
    for (int k = klo; k <= N2 / 2 - 1; ++k) {
      V a = A[tri_krow(ca ? -k : k, N2) * N1h + ia];
      V p = Pf[tri_krow(cp ? k : -k, N2) * N1h + ia];
      if (ca) a.y = -a.y;
      if (cp) p.y = -p.y;
      tri_mac(acc, a, p);
    }
  }
  return acc;
}

template <typename T>
__device__ __forceinline__ typename C2<T>::t tri_lin(T s1, typename C2<T>::t x1, T s2, typename C2<T>::t x2) {
  typename C2<T>::t r;
  r.x = s1 * x1.x + s2 * x2.x;
  r.y = s1 * x1.y + s2 * x2.y;
  return r;
}

// one block per plane: blockIdx.x < nuI -> u level blockIdx.x + 1, else v level
template <typename T>
__global__ void __launch_bounds__(512) k_triad(const double2 *__restrict__ u1, const double2 *__restrict__ u2,
                                               const double2 *__restrict__ u3, Geo g, TriadGeo tg,
                                               typename C2<T>::t *__restrict__ N1xz, typename C2<T>::t *__restrict__ N2xz,
                                               typename C2<T>::t *__restrict__ N3xz, typename C2<T>::t *__restrict__ uvf,
                                               typename C2<T>::t *__restrict__ vvc, typename C2<T>::t *__restrict__ wvf) {
  typedef typename C2<T>::t V;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V *F = reinterpret_cast<V *>(smem_raw);  // [3][P] + zero slot
  const bool isU = blockIdx.x < (unsigned)g.nuI;
  const int q = isU ? blockIdx.x + 1 : blockIdx.x - g.nuI + 1;
  const int nc = g.ncol, N1h = g.N1h, N2 = g.N2, P = tg.P;
  const size_t off = (size_t)q * nc;
  // stage the three fields: u planes (u1, v at the centre, u3); v planes (u1 at the face, u2, u3 at the face)
  for (int c = threadIdx.x; c < nc; c += blockDim.x) {
    V f0, f1, f2;
    if (isU) {
      const double2 a = u1[off + c], b = u3[off + c], v0 = u2[off + c], vm = u2[off - nc + c];
      f0.x = to_t<T>(a.x); f0.y = to_t<T>(a.y);
      f2.x = to_t<T>(b.x); f2.y = to_t<T>(b.y);
      if (sizeof(T) == 8) {
        const double ia = g.iua[q], ib = g.iub[q];
        f1.x = (T)(ia * v0.x + ib * vm.x);
        f1.y = (T)(ia * v0.y + ib * vm.y);
      } else {
        const T ia = (T)g.iuaf[q], ib = (T)g.iubf[q];
        f1.x = ia * to_t<T>(v0.x) + ib * to_t<T>(vm.x);
        f1.y = ia * to_t<T>(v0.y) + ib * to_t<T>(vm.y);
      }
    } else {
      const double2 v = u2[off + c];
      const double2 ap = u1[off + nc + c], a0 = u1[off + c], bp = u3[off + nc + c], b0 = u3[off + c];
      f1.x = to_t<T>(v.x); f1.y = to_t<T>(v.y);
      if (sizeof(T) == 8) {
        const double ia = g.iva[q], ib = g.ivb[q];
        f0.x = (T)(ia * ap.x + ib * a0.x); f0.y = (T)(ia * ap.y + ib * a0.y);
        f2.x = (T)(ia * bp.x + ib * b0.x); f2.y = (T)(ia * bp.y + ib * b0.y);
      } else {
        const T ia = (T)g.ivaf[q], ib = (T)g.ivbf[q];
        f0.x = ia * to_t<T>(ap.x) + ib * to_t<T>(a0.x); f0.y = ia * to_t<T>(ap.y) + ib * to_t<T>(a0.y);
        f2.x = ia * to_t<T>(bp.x) + ib * to_t<T>(b0.x); f2.y = ia * to_t<T>(bp.y) + ib * to_t<T>(b0.y);
      }
    }
    F[c] = f0;
    F[P + c] = f1;
    F[2 * P + c] = f2;
  }
  if (threadIdx.x == 0) F[3 * P] = czero<V>();
  __syncthreads();
  const V *F0 = F, *F1 = F + P, *F2 = F + 2 * P;
  const T a00 = F0[0].x, b00 = F1[0].x, c00 = F2[0].x;  // real parts of the (0,0) modes
  const int kw = 2 * tg.nz + 1;
  const int *lid = tg.lid + (size_t)(isU ? q : g.nu + q) * 9;
  const int lane = threadIdx.x & 31;
  // targets: (lt, kt) with list terms
  for (int sl = threadIdx.x; sl < tg.Tw * 32; sl += blockDim.x) {
    if (sl >= tg.T) continue;
    const int w = sl >> 5;
    const int tt = tg.tmap[sl];
    const int lt = tt / kw, kt = tt - lt * kw - tg.nz;
    const int r = tri_krow(kt, N2), c = r * N1h + lt;
    const bool z0 = (lt == 0 && kt == 0);
    const T kxv = sizeof(T) == 8 ? (T)g.k1x[lt] : (T)g.k1xf[lt];
    const T kzv = sizeof(T) == 8 ? (T)g.k1z[r] : (T)g.k1zf[r];
    if (isU) {
      // F0 = u, F1 = v (interpolated), F2 = w; lists 1 uu, 3 uw, 5 vv, 7 wu, 9 ww
      V uu = tri_lin<T>((T)2 * a00, F0[c], (T)0, F0[c]);
      V ww = tri_lin<T>((T)2 * c00, F2[c], (T)0, F2[c]);
      V uw = tri_lin<T>(a00, F2[c], c00, F0[c]);
      V wu = uw;
      V vv = z0 ? tri_zeroth(F1, F1, -(N2 / 2), g.N1, N2, N1h) : tri_lin<T>((T)2 * b00, F1[c], (T)0, F1[c]);
      tri_list(uu, F, tg, lid[0], w, lane);
      tri_list(uw, F, tg, lid[2], w, lane);
      tri_list(vv, F, tg, lid[4], w, lane);
      tri_list(wu, F, tg, lid[6], w, lane);
      tri_list(ww, F, tg, lid[8], w, lane);
      N1xz[off + c] = cadd(cimul(kxv, uu), cimul(kzv, uw));
      N3xz[off + c] = cadd(cimul(kxv, wu), cimul(kzv, ww));
      vvc[off + c] = vv;
    } else {
      // F0 = u (interpolated), F1 = v, F2 = w (interpolated); lists 2 uv, 4 vu, 6 vw, 8 wv
      V vu = tri_lin<T>(a00, F1[c], b00, F0[c]);
      V vw = tri_lin<T>(b00, F2[c], c00, F1[c]);
      V uv = z0 ? tri_zeroth(F0, F1, -(N2 / 2 - 1), g.N1, N2, N1h) : vu;
      V wv = z0 ? tri_zeroth(F2, F1, -(N2 / 2 - 1), g.N1, N2, N1h) : vw;
      tri_list(uv, F, tg, lid[1], w, lane);
      tri_list(vu, F, tg, lid[3], w, lane);
      tri_list(vw, F, tg, lid[5], w, lane);
      tri_list(wv, F, tg, lid[7], w, lane);
      N2xz[off + c] = cadd(cimul(kxv, vu), cimul(kzv, vw));
      uvf[off + c] = uv;
      wvf[off + c] = wv;
    }
  }
  // the other modes (x-mode N1/2, z-mode -N2/2): linear advection only
  const int nrest = N2 + (N1h - 1);
  for (int i = threadIdx.x; i < nrest; i += blockDim.x) {
    const int kx = i < N2 ? N1h - 1 : i - N2;
    const int r = i < N2 ? i : N2 / 2;
    const int c = r * N1h + kx;
    const bool zr = (r == N2 / 2);
    const T kxv = sizeof(T) == 8 ? (T)g.k1x[kx] : (T)g.k1xf[kx];
    const T kzv = sizeof(T) == 8 ? (T)g.k1z[r] : (T)g.k1zf[r];
    if (isU) {
      const V uu = tri_lin<T>((T)2 * a00, F0[c], (T)0, F0[c]);
      const V ww = tri_lin<T>((T)2 * c00, F2[c], (T)0, F2[c]);
      const V uw = tri_lin<T>(a00, F2[c], c00, F0[c]);
      N1xz[off + c] = zr ? czero<V>() : cadd(cimul(kxv, uu), cimul(kzv, uw));
      N3xz[off + c] = zr ? czero<V>() : cadd(cimul(kxv, uw), cimul(kzv, ww));
      vvc[off + c] = tri_lin<T>((T)2 * b00, F1[c], (T)0, F1[c]);
    } else {
      const V vu = tri_lin<T>(a00, F1[c], b00, F0[c]);
      const V vw = tri_lin<T>(b00, F2[c], c00, F1[c]);
      N2xz[off + c] = zr ? czero<V>() : cadd(cimul(kxv, vu), cimul(kzv, vw));
      uvf[off + c] = vu;
      wvf[off + c] = vw;
    }
  }
}

// ---------------------------------------------------------------------------
// host: expansion of the lists into warp-striped term rows
// ---------------------------------------------------------------------------
struct TriadHost {
  std::vector<uint32_t> terms;
  std::vector<int> wb;   // [nlists][Tw+1]
  std::vector<int> lid;  // [(nu + nv) * 9]
  std::vector<int> tmap;  // [T] slot -> target
  int Tw = 0, T = 0, P = 0, nlists = 0;
  long long nterms = 0;  // list terms (both passes), without padding
};

// fields of (type): u planes F0 = u, F1 = v, F2 = w; v planes F0 = u, F1 = v, F2 = w
// (interpolated where needed). Active field a, passive field p as nonlinInter's
// arguments uaPL, upPL (FOU3D.f90:1845-1849, 1943-1946).
static inline void triad_fields(int type, int &fa, int &fp) {
  static const int A[9] = {0, 1, 2, 0, 1, 2, 0, 1, 2};
  static const int Pp[9] = {0, 0, 0, 1, 1, 1, 2, 2, 2};
  // uu(U,U) uv(V,U) uw(W,U) vu(U,V) vv(V,V) vw(W,V) wu(U,W) wv(V,W) ww(W,W)
  fa = A[type - 1];
  fp = Pp[type - 1];
}

static std::string build_triads(const lh_config *cfg, const Geo &g, TriadHost &th) {
  const int nx = cfg->triad_nx, nz = cfg->triad_nz, ns = cfg->triad_nsets;
  if (nx != g.N1 / 2 - 1) return "nx number does not agree between list and simulation";
  if (nz != g.N2 / 2 - 1) return "nz number does not agree between list and simulation";
  if (ns <= 0 || !cfg->triad_off || !cfg->triad_len || !cfg->triad_data || !cfg->triad_set_u || !cfg->triad_set_v)
    return "triad lists missing";
  if (cfg->dny != 0) return "triad lists need dny = 0 (no lists file covers the immersed region)";
  const int N1h = g.N1h, N2 = g.N2;
  th.P = N1h * N2;
  if (3 * th.P + 1 > 0x7fff) return "plane too large for the triad form";
  const int kw = 2 * nz + 1;
  th.T = (nx + 1) * kw;
  th.Tw = (th.T + 31) / 32;
  // slots: targets by decreasing complete-list count (2nx+1-lt)(2nz+1-|kt|), stable
  th.tmap.resize(th.T);
  for (int t = 0; t < th.T; ++t) th.tmap[t] = t;
  auto key = [&](int t) { const int lt = t / kw, kt = t - lt * kw - nz; return (2 * nx + 1 - lt) * (kw - abs(kt)); };
  std::stable_sort(th.tmap.begin(), th.tmap.end(), [&](int a, int b) { return key(a) > key(b); });
  std::vector<int> slot_of(th.T);
  for (int sl = 0; sl < th.T; ++sl) slot_of[th.tmap[sl]] = sl;
  const uint32_t zero = (uint32_t)(3 * th.P);
  const uint32_t pad = zero | (zero << 16);
  th.lid.assign((size_t)(g.nu + g.nv) * 9, -1);
  struct Key { int64_t off, len; int type; };
  std::vector<Key> keys;
  std::vector<uint32_t> bucket;
  std::vector<int> cnt, start, tgt;
  std::vector<uint32_t> code;
  auto expand = [&](const Key &k) -> std::string {
    const int8_t *l = cfg->triad_data + 4 * k.off;
    const int64_t L = k.len;
    int fa, fp;
    triad_fields(k.type, fa, fp);
    tgt.clear();
    code.clear();
    for (int64_t e = 0; e < L; ++e) {
      const int la = l[e], ka0 = l[L + e], lp = l[2 * L + e], kp0 = l[3 * L + e];
      if (abs(la) > nx || abs(lp) > nx || abs(ka0) > nz || abs(kp0) > nz || la + lp < 0 || la + lp > nx ||
          abs(ka0 + kp0) > nz)
        return "triad outside the retained modes";
      const int sa = la < 0 ? -1 : 1, sp = lp < 0 ? -1 : 1;
      for (int p = 0; p <= 1; ++p) {
        if (ka0 + kp0 == 0 && p == 1) continue;
        const int pn = 2 * p - 1;
        const int ra = tri_krow(pn * sa * ka0, N2), rp = tri_krow(pn * sp * kp0, N2);
        const uint32_t ia = (uint32_t)(fa * th.P + ra * N1h + abs(la)) | (la < 0 ? 0x8000u : 0u);
        const uint32_t ip = (uint32_t)(fp * th.P + rp * N1h + abs(lp)) | (lp < 0 ? 0x8000u : 0u);
        tgt.push_back(slot_of[(la + lp) * kw + pn * (ka0 + kp0) + nz]);
        code.push_back(ia | (ip << 16));
      }
    }
    // stable counting sort by slot, then warp striping
    cnt.assign(th.Tw * 32, 0);
    for (int t : tgt) ++cnt[t];
    start.assign(th.Tw * 32 + 1, 0);
    for (int t = 0; t < th.Tw * 32; ++t) start[t + 1] = start[t] + cnt[t];
    bucket.resize(code.size());
    {
      std::vector<int> pos(start.begin(), start.end() - 1);
      for (size_t i = 0; i < code.size(); ++i) bucket[pos[tgt[i]]++] = code[i];
    }
    const size_t row0 = th.terms.size() / 32;
    th.wb.push_back((int)row0);
    size_t rows = row0;
    for (int w = 0; w < th.Tw; ++w) {
      int Lw = 0;
      for (int j = 0; j < 32; ++j) Lw = std::max(Lw, cnt[w * 32 + j]);
      const size_t base = th.terms.size();
      th.terms.resize(base + (size_t)Lw * 32, pad);
      for (int j = 0; j < 32; ++j) {
        const int t = w * 32 + j;
        for (int i = 0; i < cnt[t]; ++i) th.terms[base + (size_t)i * 32 + j] = bucket[start[t] + i];
      }
      rows += Lw;
      if (rows > 0x7fffffffULL) return "triad lists too large";
      th.wb.push_back((int)rows);
    }
    th.nterms += (long long)code.size();
    return "";
  };
  for (int i = 0; i < 9 * ns; ++i)
    if (cfg->triad_off[i] < 0 || cfg->triad_len[i] < 0) return "negative list offset or length";
  auto list_of = [&](int set, int type, int &out) -> std::string {
    if (set < 0 || set >= ns) return "level without a lists set";
    const Key k{cfg->triad_off[set * 9 + type - 1], cfg->triad_len[set * 9 + type - 1], type};
    for (size_t i = 0; i < keys.size(); ++i)
      if (keys[i].off == k.off && keys[i].len == k.len && keys[i].type == k.type) { out = (int)i; return ""; }
    std::string e = expand(k);
    if (!e.empty()) return e;
    keys.push_back(k);
    out = (int)keys.size() - 1;
    return "";
  };
  for (int q = 1; q <= g.nu - 2; ++q)
    for (int t : {1, 3, 5, 7, 9}) {
      std::string e = list_of(cfg->triad_set_u[q], t, th.lid[(size_t)q * 9 + t - 1]);
      if (!e.empty()) return e;
    }
  for (int q = 1; q <= g.nv - 2; ++q)
    for (int t : {2, 4, 6, 8}) {
      std::string e = list_of(cfg->triad_set_v[q], t, th.lid[(size_t)(g.nu + q) * 9 + t - 1]);
      if (!e.empty()) return e;
    }
  th.nlists = (int)keys.size();
  if (th.wb.size() != (size_t)th.nlists * (th.Tw + 1)) return "internal: warp table size";
  if (th.terms.empty()) th.terms.assign(32, pad);
  return "";
}
