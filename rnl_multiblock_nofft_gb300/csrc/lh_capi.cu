// lh_capi.cu — the C ABI of include/lh.h: one handle = one channel on one GPU.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <atomic>
#include <mutex>
#include <string>
#include <algorithm>
#include <vector>

#include "lh_internal.cuh"

#include "lh_kernels.cuh"
#include "lh_triads.cuh"
#include "lh_xpass2.cuh"

namespace {
const int NTHR_H = 256;
}


struct lh_handle {
  lh_config cfg;
  std::vector<double> h_yu, h_yv, h_thu, h_thv, h_d2u, h_d2v, h_k1x, h_k2x, h_k1z, h_k2z;
  std::vector<int> h_lu, h_lv;
  std::vector<double> h_Au, h_Av;
  Geo g;
  int prec;  // LH_PREC_*
  size_t vsz;  // bytes of one complex value in the transforms
  cudaStream_t st;
  cudaStream_t st2;            // side stream: mean-flow correction overlapped with the v solve
  cudaEvent_t ev_fork, ev_join;
  // device buffers
  double2 *u1, *u2, *u3, *p, *psi;
  void *Nu1, *Nu2, *Nu3;  // nonlinear term of the last substep, transform precision
  double *dg1, *dg2, *dg3;  // factorised pressure matrices (constant)
  void *ysf, *ysv;  // FP32 scratch of the mixed-form solves (u and w; v)
  void *N1xz, *N2xz, *N3xz, *uvf, *vvc, *wvf;  // transform outputs, transform precision
  double *a3s, *a3v, *mfw;
  void *A, *B, *twx, *twz, *twx64, *twz64;
  size_t Abytes, Bbytes;
  long long graph_nodes_per_step;
  double *geo_pool;
  float *geo_poolf;
  DevScalars *sc;
  double2 *stage;  // staging for transposes
  // asynchronous state I/O (allocated on first use): staged copies of the whole state in
  // each direction, copy streams, and the events that order them against the main stream
  double2 *stage_in, *stage_out;
  cudaStream_t st_in, st_out;
  // per staging slot: 0 the whole state, 1..3 the bands (each band its own region)
  cudaEvent_t ev_in_copied[4], ev_in_used[4], ev_out_ready[4], ev_out_copied[4];
  // immersed boundaries
  int ib, nib, ncap;
  int *d_ibslot_u, *d_ibslot_v, *d_iblev, *d_lev2cap_u, *d_lev2cap_v;
  void *cap;  // captured physical planes of the immersed levels, in the transform precision
  IbRec *d_ibrec;   // forced points, sorted by (plane of du, row)
  int *d_iboff;     // [3 nib G2 + 1] record ranges per (plane, row)
  void *duib;  // du of the immersed levels [ibslot][3][col], complex in the transform precision
  // plane views of the nonlinear launches: wall-band planes, then core planes
  // (multiblock); one view when single-resolution
  Geo gv[2];
  int nviews;
  int *d_slotq, *d_capv;    // slot -> level of the views; capture slot of view 0's slots
  void *twv[2][2];          // twiddles of the views (x, z) in the transform precision
  int2 *d_vcol;             // virtual columns of the solve kernels (multiblock)
  int *d_bcols;             // long columns, then short columns (band I/O)
  int nlong, nshort;
  // statistics
  double *st_pl, *st_cd;
  double *st_pp, *st_cd4;    // pressure plane sums [2][np]; conditioned P, omega_x [4][ncl + 1][dnz][dnx]
  int4 *d_cond_list;         // planes of the conditioned P, omega_x sums: (kind, level, j1) (first use)
  int n_cond;
  void *d_cond_scr;          // their spectral and physical planes, one chunk of cond_chunk planes
  int cond_chunk;
  double *d_sp;              // spectra accumulators: U, V, W, UV, P, each [level][nlong] (allocated on first use)
  double2 *d_slip, *d_slip_inst;  // slip statistics [2][4][ncol]: accumulated / instantaneous
  int st_ncl, st_dnx, st_dnz, st_ntx;
  long long istat;
  // triad-list nonlinear form
  int triad;
  TriadGeo tg;
  uint32_t *d_terms;
  int *d_wb, *d_lid, *d_tmap;
  int tri_threads;
  size_t tri_smem;
  long long tri_nterms;
  cudaGraph_t graph;
  cudaGraphExec_t gexec;
  bool graph_ready;
  long long launches;
  int tb_uw, tb_v, tb_p;  // threads per block of the one-thread-per-column kernels (lh_autotune)
  // levels the solve kernels stage ahead through shared memory (0: the kernels that prefetch into
  // registers instead), per kernel: u/w, v (mixed form) and pressure (lh_autotune)
  int pf_uw, pf_v, pf_p;
  std::string err;
  // per-kernel timing (lh_profile_steps): events around each launch
  bool prof;
  std::vector<std::pair<const char *, std::pair<cudaEvent_t, cudaEvent_t>>> prof_ev;
  const char *cur_name;
};

// message of the last failure on this host thread (lh_last_error(NULL))
static thread_local std::string t_last_err;

static int fail(lh_handle *h, int code, const std::string &msg) {
  if (h) h->err = msg;
  t_last_err = msg;
  return code;
}

#define CK(call)                                                                            \
  do {                                                                                      \
    cudaError_t e__ = (call);                                                               \
    if (e__ != cudaSuccess)                                                                 \
      return fail(h, LH_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e__));        \
  } while (0)

template <typename T>
static void twiddles(int n, std::vector<T> &out) {
  out.resize(2 * (size_t)n);
  for (int e = 0; e < n; ++e) {
    long double a = -2.0L * 3.14159265358979323846264338327950288L * (long double)e / (long double)n;
    out[2 * e] = (T)cosl(a);
    out[2 * e + 1] = (T)sinl(a);
  }
}

template <typename T>
static void *upload_vec(const std::vector<T> &v, cudaError_t &err) {
  void *d = nullptr;
  err = cudaMalloc(&d, sizeof(T) * (v.size() ? v.size() : 1));
  if (err == cudaSuccess && v.size()) err = cudaMemcpy(d, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice);
  return d;
}

static void prof_begin(lh_handle *h, const char *name) {
  if (!h->prof) return;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a, h->st);
  h->prof_ev.push_back({name, {a, b}});
}
static int count_launch(lh_handle *h) {
  h->launches++;
  if (h->prof && !h->prof_ev.empty()) cudaEventRecord(h->prof_ev.back().second.second, h->st);
  cudaError_t e = cudaGetLastError();  // this launch's error (and clears it)
  if (e != cudaSuccess) return fail(h, LH_ECUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  return LH_OK;
}
// KL(name, kernel<<<...>>>(...)): launch on the handle's stream, counted and (when
// profiling) bracketed by CUDA events
#define KL(name, ...)                 \
  do {                                \
    prof_begin(h, name);              \
    __VA_ARGS__;                      \
    int rc__ = count_launch(h);       \
    if (rc__ != LH_OK) return rc__;   \
  } while (0)

// FFT lengths compiled into the library (Ngal values of every workload)
#define LH_FOR_SIZES(X) X(24) X(48) X(72) X(96) X(144) X(192) X(288) X(384) X(576) X(768) X(1152)
static bool size_supported(int n) {
  switch (n) {
#define LH_CASE_TRUE(n_) case n_: return true;
    LH_FOR_SIZES(LH_CASE_TRUE)
#undef LH_CASE_TRUE
    default: return false;
  }
}
// run CALL with the compile-time constant N equal to n
#define LH_DISPATCH(n, ...)                               \
  switch (n) {                                            \
    case 24: { constexpr int N = 24; __VA_ARGS__; } break;       \
    case 48: { constexpr int N = 48; __VA_ARGS__; } break;       \
    case 72: { constexpr int N = 72; __VA_ARGS__; } break;       \
    case 96: { constexpr int N = 96; __VA_ARGS__; } break;       \
    case 144: { constexpr int N = 144; __VA_ARGS__; } break;     \
    case 192: { constexpr int N = 192; __VA_ARGS__; } break;     \
    case 288: { constexpr int N = 288; __VA_ARGS__; } break;     \
    case 384: { constexpr int N = 384; __VA_ARGS__; } break;     \
    case 576: { constexpr int N = 576; __VA_ARGS__; } break;     \
    case 768: { constexpr int N = 768; __VA_ARGS__; } break;     \
    case 1152: { constexpr int N = 1152; __VA_ARGS__; } break;   \
    default: break;                                       \
  }

template <typename T, int N>
static cudaError_t set_attrs_sized(int lim) {
  cudaError_t e = cudaSuccess;
  const cudaFuncAttribute A = cudaFuncAttributeMaxDynamicSharedMemorySize;
  // k_xstats also holds a small static reduction array
  if (e == cudaSuccess) e = cudaFuncSetAttribute((const void *)k_xstats<T, N>, A, lim - 1024);
  if (e == cudaSuccess) e = cudaFuncSetAttribute((const void *)k_ib_xforce<T, N>, A, lim);
  if constexpr (sizeof(T) == 8) {  // the Stockham passes (FP64 form and the FP64 leaf transforms)
    if (e == cudaSuccess) e = cudaFuncSetAttribute((const void *)k_zinv_nl<T, N>, A, lim);
    if (e == cudaSuccess) e = cudaFuncSetAttribute((const void *)k_xpass_nl<T, N>, A, lim);
    if (e == cudaSuccess) e = cudaFuncSetAttribute((const void *)k_zfwd_nl<T, N>, A, lim);
    if (e == cudaSuccess) e = cudaFuncSetAttribute((const void *)k_spec_zinv<T, N>, A, lim);
    if (e == cudaSuccess) e = cudaFuncSetAttribute((const void *)k_xinv_phys<T, N>, A, lim);
    if (e == cudaSuccess) e = cudaFuncSetAttribute((const void *)k_xfwd_phys<T, N>, A, lim);
    if (e == cudaSuccess) e = cudaFuncSetAttribute((const void *)k_zfwd_spec<T, N>, A, lim);
  }
  if constexpr (sizeof(T) == 4) {  // the two-stage mixed-form passes
    if (e == cudaSuccess) e = cudaFuncSetAttribute((const void *)k_zinv2<N>, A, lim);
    if (e == cudaSuccess) e = cudaFuncSetAttribute((const void *)k_zfwd2<N>, A, lim);
    if (e == cudaSuccess) e = cudaFuncSetAttribute((const void *)k_spec_zinv2<N>, A, lim);
    if constexpr (N == 576 || N == 768 || N == 1152)
      if (e == cudaSuccess) e = cudaFuncSetAttribute((const void *)k_xpass3<N>, A, lim);
    if (e == cudaSuccess) e = cudaFuncSetAttribute((const void *)k_zfwd_spec2<N>, A, lim);
    if constexpr (N <= 384)
      if (e == cudaSuccess) e = cudaFuncSetAttribute((const void *)k_xpass2<N>, A, lim);
  }
  return e;
}

static int smem_optin(int *lim) {
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return -1;
  *lim = optin > 0 ? optin : 49152;
  return 0;
}

static int set_smem_attrs_all(lh_handle *h) {
  int lim = 0;
  if (smem_optin(&lim)) return fail(h, LH_ECUDA, "cudaDeviceGetAttribute");
  cudaError_t e = cudaSuccess;
  for (int n : {h->g.G1, h->g.G2, h->gv[1].G1, h->gv[1].G2}) {
    if (n <= 0) continue;
    LH_DISPATCH(n, e = set_attrs_sized<double, N>(lim); if (e == cudaSuccess) e = set_attrs_sized<float, N>(lim));
    if (e != cudaSuccess) return fail(h, LH_ECUDA, std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
  }
  return LH_OK;
}


extern "C" int lh_create(const lh_config *cfg, lh_handle **out) {
  lh_handle *h = nullptr;
  if (!cfg || !out) return fail(nullptr, LH_EINVAL, "null argument");
  *out = nullptr;
  if (cfg->abi_version != LH_ABI_VERSION) return fail(nullptr, LH_EINVAL, "abi_version mismatch");
  if (cfg->precision != LH_PREC_FP64 && cfg->precision != LH_PREC_MIXED)
    return fail(nullptr, LH_EINVAL, "unknown precision");
  if (cfg->nonlin_form != LH_NONLIN_PRODUCTS && cfg->nonlin_form != LH_NONLIN_TRIADS)
    return fail(nullptr, LH_EINVAL, "unknown nonlinear form");
  if (cfg->N1 <= 0 || cfg->N2 <= 0 || (cfg->N1 & 1) || (cfg->N2 & 1) || cfg->Ngal1 <= cfg->N1 ||
      cfg->Ngal2 <= cfg->N2 || (cfg->Ngal1 & 1) || (cfg->Ngal2 & 1) || cfg->dny < 0)
    return fail(nullptr, LH_EINVAL, "bad N / Ngal / dny");
  if (cfg->N1 != 2 * (cfg->Ngal1 / 3) || cfg->N2 != 2 * (cfg->Ngal2 / 3) || cfg->N1c != 2 * (cfg->Ngal1c / 3) ||
      cfg->N2c != 2 * (cfg->Ngal2c / 3))
    return fail(nullptr, LH_EINVAL, "N must be 2 (Ngal / 3) in every band (start.f90:110-114)");
  if (cfg->nyu != cfg->N4[3] + 1 - cfg->N4[0] + 1 || cfg->nyv != cfg->N3[3] + 1 - cfg->N3[0] + 1 ||
      cfg->nyv != cfg->nyu - 1 || cfg->N4[0] != -cfg->dny || cfg->N3[0] != -cfg->dny || cfg->nyu < 5)
    return fail(nullptr, LH_EINVAL, "band limits inconsistent with nyu / nyv / dny");
  const int mb = (cfg->N1c != cfg->N1 || cfg->N2c != cfg->N2 || cfg->Ngal1c != cfg->Ngal1 || cfg->Ngal2c != cfg->Ngal2);
  if (mb) {
    if (cfg->N1c <= 0 || cfg->N2c <= 0 || cfg->N1c > cfg->N1 || cfg->N2c > cfg->N2 || (cfg->N1c & 1) ||
        (cfg->N2c & 1) || cfg->Ngal1c <= cfg->N1c || cfg->Ngal2c <= cfg->N2c || !size_supported(cfg->Ngal1c) ||
        !size_supported(cfg->Ngal2c))
      return fail(nullptr, LH_EINVAL, "core band: need N1c <= N1, N2c <= N2, even, Ngal1c/Ngal2c supported sizes");
    if (cfg->N4[2] <= cfg->N4[1] + 1 || cfg->N3[2] <= cfg->N3[1] + 1 || cfg->N4[1] <= cfg->N4[0] + 1)
      return fail(nullptr, LH_EINVAL, "multiblock: every band needs interior levels");
    if (cfg->nonlin_form == LH_NONLIN_TRIADS)
      return fail(nullptr, LH_EINVAL, "triad lists need one x/z resolution in every band");
  }
  h = new lh_handle();
  memset(&h->g, 0, sizeof(Geo));
  h->cfg = *cfg;
  h->prec = cfg->precision;
  h->vsz = (h->prec == LH_PREC_FP64) ? sizeof(double2) : sizeof(float2);
  h->graph_ready = false;
  h->launches = 0;
  h->tb_uw = h->tb_v = h->tb_p = 128;
  h->pf_uw = h->pf_v = h->pf_p = 4;
  if (!size_supported(cfg->Ngal1) || !size_supported(cfg->Ngal2)) {
    int rc = fail(h, LH_EINVAL, "Ngal must be one of 24 48 72 96 144 192 288 384 576 768 1152");
    delete h;
    return rc;
  }
  Geo &g = h->g;
  g.N1 = cfg->N1; g.N2 = cfg->N2; g.N1h = cfg->N1 / 2 + 1; g.G1 = cfg->Ngal1; g.G2 = cfg->Ngal2;
  g.dny = cfg->dny; g.nu = cfg->nyu; g.nv = cfg->nyv; g.np = cfg->nyu - 2; g.ncol = g.N1h * g.N2;
  g.nuI = g.nu - 2; g.nvI = g.nv - 2; g.nn = cfg->nn;
  for (int b = 0; b < 4; ++b) { g.N3[b] = cfg->N3[b]; g.N4[b] = cfg->N4[b]; }
  g.Re = cfg->Re; g.CFL = cfg->CFL; g.dtv = cfg->dtv; g.dd = cfg->ddthetavi; g.dthetavi = cfg->dthetavi;
  g.alp = cfg->alp; g.bet = cfg->bet; g.Kib = cfg->Kib;
  for (int k = 0; k < 3; ++k) {
    g.aRK[k] = cfg->aRK[k]; g.bRK[k] = cfg->bRK[k]; g.cRK[k] = cfg->cRK[k]; g.dRK[k] = cfg->dRK[k]; g.gRK[k] = cfg->gRK[k];
  }
  for (int b = 0; b < 3; ++b) { g.gw[b][0] = cfg->gw[b][0]; g.gw[b][1] = cfg->gw[b][1]; }
  g.gwbc1 = cfg->gw_bc_u1; g.gwbc3 = cfg->gw_bc_u3;
  // multiblock description: wall-band grid, band level ranges (jlim, start.f90:1675-1709)
  g.mb = mb;
  g.N1hF = g.N1h; g.N2F = g.N2; g.ncolF = g.ncol;
  g.slotq = nullptr;
  {
    const int d = cfg->dny, *N3 = cfg->N3, *N4 = cfg->N4;
    const int bq[3][6] = {{N4[0] + d, N4[1] + 1 + d, N3[0] + d, N3[1] + 1 + d, N4[0] + d, N4[1] + d - 1},
                          {N4[0] + d, N4[3] + 1 + d, N3[0] + d, N3[3] + 1 + d, N4[0] + d, N4[3] + d - 1},
                          {N4[2] + d, N4[3] + 1 + d, N3[2] + d, N3[3] + 1 + d, N4[2] + d, N4[3] + d - 1}};
    memcpy(g.bq, bq, sizeof(bq));
  }
  // long columns (modes of the core band) and short columns (wall bands only)
  std::vector<int> longc, shortc;
  for (int c = 0; c < g.ncol; ++c) {
    const int r = c / g.N1h, kx = c - r * g.N1h;
    const bool lg = !mb || (kx <= cfg->N1c / 2 && (r < cfg->N2c / 2 || r >= g.N2 - cfg->N2c / 2));
    (lg ? longc : shortc).push_back(c);
  }
  h->nlong = (int)longc.size(); h->nshort = (int)shortc.size();
  g.nvc = mb ? h->nlong + 2 * h->nshort : g.ncol;
  g.vcol = nullptr;
  // plane views: u planes N(4,0)+1..N(4,1), N(4,2)+1..N(4,3) and v planes N(3,0)+1..N(3,1),
  // N(3,2)+1..N(3,3) are wall-band planes (proc_lims_planes, start.f90:1836-1916)
  std::vector<int> vsl[2][2];
  for (int q = 1; q <= g.nu - 2; ++q) {
    const int j = q - cfg->dny;
    vsl[(!mb || j <= cfg->N4[1] || j > cfg->N4[2]) ? 0 : 1][0].push_back(q);
  }
  for (int q = 1; q <= g.nv - 2; ++q) {
    const int j = q - cfg->dny;
    vsl[(!mb || j <= cfg->N3[1] || j > cfg->N3[2]) ? 0 : 1][1].push_back(q);
  }
  h->nviews = mb ? 2 : 1;
  // view sizes (the views themselves are filled once the geometry pools exist)
  const int vN1h[2] = {g.N1h, cfg->N1c / 2 + 1}, vG2[2] = {g.G2, cfg->Ngal2c};
  g.flag_ctpress = cfg->flag_ctpress;
  const int nu = g.nu, nv = g.nv;
  // geometry pool: yu yv thu thv d2u(3nu) d2v(3nv) k1x k2x k1z k2z iua iub iud iva ivb ivd
  std::vector<double> pool;
  auto put = [&](const double *src, size_t n) { size_t o = pool.size(); pool.insert(pool.end(), src, src + n); return o; };
  std::vector<double> iua(nu, 1.0), iub(nu, 0.0), iud(nu, 1.0), iva(nv, 1.0), ivb(nv, 0.0), ivd(nv, 1.0);
  // interp_v / interp_u weights (FOU3D.f90:427-474) as ratios: one multiply-add per value
  for (int q = 1; q <= nu - 2; ++q) {
    iud[q] = cfg->yv[q] - cfg->yv[q - 1];
    iua[q] = (cfg->yu[q] - cfg->yv[q - 1]) / iud[q];
    iub[q] = (cfg->yv[q] - cfg->yu[q]) / iud[q];
  }
  for (int q = 0; q <= nv - 1; ++q) {
    ivd[q] = cfg->yu[q + 1] - cfg->yu[q];
    iva[q] = (cfg->yv[q] - cfg->yu[q]) / ivd[q];
    ivb[q] = (cfg->yu[q + 1] - cfg->yv[q]) / ivd[q];
  }
  size_t o_yu = put(cfg->yu, nu), o_yv = put(cfg->yv, nv), o_thu = put(cfg->dthdyu, nu), o_thv = put(cfg->dthdyv, nv);
  size_t o_d2u = put(cfg->dyu2i, 3 * (size_t)nu), o_d2v = put(cfg->dyv2i, 3 * (size_t)nv);
  size_t o_k1x = put(cfg->k1x, g.N1h), o_k2x = put(cfg->k2x, g.N1h), o_k1z = put(cfg->k1z, g.N2), o_k2z = put(cfg->k2z, g.N2);
  size_t o_iua = put(iua.data(), nu), o_iub = put(iub.data(), nu), o_iud = put(iud.data(), nu);
  size_t o_iva = put(iva.data(), nv), o_ivb = put(ivb.data(), nv), o_ivd = put(ivd.data(), nv);
  std::vector<double> thud(nu);  // ddthetavi * dthdyu, the divergence's y factor
  for (int q = 0; q < nu; ++q) thud[q] = cfg->ddthetavi * cfg->dthdyu[q];
  size_t o_thud = put(thud.data(), nu);
  cudaError_t ce;
  h->geo_pool = (double *)upload_vec(pool, ce);
  if (ce != cudaSuccess) { int rc = fail(h, LH_ECUDA, cudaGetErrorString(ce)); lh_destroy(h); return rc; }
  double *P = h->geo_pool;
  g.yu = P + o_yu; g.yv = P + o_yv; g.thu = P + o_thu; g.thv = P + o_thv; g.d2u = P + o_d2u; g.d2v = P + o_d2v;
  g.k1x = P + o_k1x; g.k2x = P + o_k2x; g.k1z = P + o_k1z; g.k2z = P + o_k2z;
  g.iua = P + o_iua; g.iub = P + o_iub; g.iud = P + o_iud; g.iva = P + o_iva; g.ivb = P + o_ivb; g.ivd = P + o_ivd;
  g.thud = P + o_thud;
  {  // FP32 copies for the mixed form
    std::vector<float> pf;
    auto putf = [&](const double *src, size_t n) { size_t o = pf.size(); for (size_t i = 0; i < n; ++i) pf.push_back((float)src[i]); return o; };
    std::vector<double> sdgu(nu, 0.0), sdgv(nv, 0.0);
    for (int q = 0; q < nu; ++q) sdgu[q] = (cfg->dyu2i[q] + cfg->dyu2i[nu + q]) + cfg->dyu2i[2 * nu + q];
    for (int q = 0; q < nv; ++q) sdgv[q] = (cfg->dyv2i[q] + cfg->dyv2i[nv + q]) + cfg->dyv2i[2 * nv + q];
    size_t f_k1x = putf(cfg->k1x, g.N1h), f_k1z = putf(cfg->k1z, g.N2);
    size_t f_iua = putf(iua.data(), nu), f_iub = putf(iub.data(), nu), f_iva = putf(iva.data(), nv), f_ivb = putf(ivb.data(), nv);
    size_t f_thu = putf(cfg->dthdyu, nu), f_thv = putf(cfg->dthdyv, nv);
    size_t f_d2u = putf(cfg->dyu2i, 3 * (size_t)nu), f_d2v = putf(cfg->dyv2i, 3 * (size_t)nv);
    size_t f_su = putf(sdgu.data(), nu), f_sv = putf(sdgv.data(), nv);
    h->geo_poolf = (float *)upload_vec(pf, ce);
    if (ce != cudaSuccess) { int rc = fail(h, LH_ECUDA, cudaGetErrorString(ce)); lh_destroy(h); return rc; }
    float *F = h->geo_poolf;
    g.k1xf = F + f_k1x; g.k1zf = F + f_k1z; g.iuaf = F + f_iua; g.iubf = F + f_iub; g.ivaf = F + f_iva; g.ivbf = F + f_ivb;
    g.thuf = F + f_thu; g.thvf = F + f_thv; g.d2uf = F + f_d2u; g.d2vf = F + f_d2v; g.sdgu = F + f_su; g.sdgv = F + f_sv;
  }

  const size_t vs = h->vsz;

  size_t nc = g.ncol;
  auto zalloc = [&](void **ptr, size_t bytes) -> cudaError_t {
    cudaError_t e = cudaMalloc(ptr, bytes ? bytes : 16);
    if (e == cudaSuccess) e = cudaMemset(*ptr, 0, bytes ? bytes : 16);
    return e;
  };
#define ZA(ptr, bytes)                                                                       \
  do {                                                                                       \
    cudaError_t e__ = zalloc((void **)&(ptr), (bytes));                                      \
    if (e__ != cudaSuccess) {                                                                \
      int rc__ = fail(h, e__ == cudaErrorMemoryAllocation ? LH_ENOMEM : LH_ECUDA,            \
                      std::string("cudaMalloc: ") + cudaGetErrorString(e__));                \
      lh_destroy(h);                                                                         \
      return rc__;                                                                           \
    }                                                                                        \
  } while (0)
  const size_t cz = sizeof(double2);
  ZA(h->u1, cz * nu * nc); ZA(h->u3, cz * nu * nc); ZA(h->u2, cz * nv * nc); ZA(h->p, cz * g.np * nc);
  ZA(h->Nu1, vs * nu * nc); ZA(h->Nu3, vs * nu * nc); ZA(h->Nu2, vs * nv * nc);
  ZA(h->dg1, sizeof(double) * g.np * nc); ZA(h->dg2, sizeof(double) * g.np * nc); ZA(h->dg3, sizeof(double) * g.np * nc);
  if (h->prec == LH_PREC_MIXED) { ZA(h->ysf, 2 * sizeof(float4) * nu * nc); ZA(h->ysv, 2 * sizeof(float2) * nv * nc); }
  ZA(h->N1xz, vs * nu * nc); ZA(h->N3xz, vs * nu * nc); ZA(h->vvc, vs * nu * nc);
  ZA(h->N2xz, vs * nv * nc); ZA(h->uvf, vs * nv * nc); ZA(h->wvf, vs * nv * nc);
  // a3s: the FP64 solves' upper factors; in the mixed form the previous nonlinear term of mode
  // (0,0) in FP64 (k_helm00_pcr: 6 x nu doubles; nc >= 8 always)
  ZA(h->psi, cz * g.np * nc); ZA(h->a3s, sizeof(double) * nu * nc); ZA(h->a3v, sizeof(double) * nv * nc);
  ZA(h->mfw, sizeof(double) * 6 * (size_t)(g.nn + 3));
  h->Abytes = h->Bbytes = 0;
  for (int vi = 0; vi < h->nviews; ++vi) {
    const size_t nuv = vsl[vi][0].size(), nvv = vsl[vi][1].size();
    h->Abytes = std::max(h->Abytes, vs * (nuv + nvv) * 3 * vG2[vi] * vN1h[vi]);
    h->Bbytes = std::max(h->Bbytes, vs * (4 * nuv + 2 * nvv) * vN1h[vi] * vG2[vi]);
  }
  {  // the immersed-boundary round trip transforms 3 * 2 * dny planes through A and B
    const size_t ibp = (cfg->ib_enable && cfg->dny > 0) ? (size_t)6 * cfg->dny : 0;
    h->Abytes = std::max(h->Abytes, sizeof(double2) * ibp * g.G2 * g.N1h);
    h->Bbytes = std::max(h->Bbytes, sizeof(double2) * ibp * g.G2 * g.N1h);
  }
  ZA(h->A, h->Abytes);
  ZA(h->B, h->Bbytes);
  ZA(h->sc, sizeof(DevScalars));
  ZA(h->stage, cz * nu * nc);
  {
    if (h->prec == LH_PREC_FP64) {
      std::vector<double> tx, tz;
      twiddles(g.G1, tx); twiddles(g.G2, tz);
      h->twx = upload_vec(tx, ce); if (ce == cudaSuccess) h->twz = upload_vec(tz, ce);
    } else {
      std::vector<float> tx, tz;
      twiddles(g.G1, tx); twiddles(g.G2, tz);
      h->twx = upload_vec(tx, ce); if (ce == cudaSuccess) h->twz = upload_vec(tz, ce);
    }
    if (ce != cudaSuccess) { int rc = fail(h, LH_ECUDA, cudaGetErrorString(ce)); lh_destroy(h); return rc; }
  }
  {  // FP64 twiddles for the leaves and the immersed-boundary round trip
    std::vector<double> tx, tz;
    twiddles(g.G1, tx); twiddles(g.G2, tz);
    h->twx64 = upload_vec(tx, ce); if (ce == cudaSuccess) h->twz64 = upload_vec(tz, ce);
    if (ce != cudaSuccess) { int rc = fail(h, LH_ECUDA, cudaGetErrorString(ce)); lh_destroy(h); return rc; }
  }
  // immersed boundaries
  h->ib = (cfg->ib_enable && cfg->dny > 0) ? 1 : 0;
  h->nib = 0; h->ncap = 0;
  h->d_sp = nullptr;
  h->d_slip = h->d_slip_inst = nullptr;
  h->stage_in = h->stage_out = nullptr;
  h->st_in = h->st_out = nullptr;
  for (int i = 0; i < 4; ++i) h->ev_in_copied[i] = h->ev_in_used[i] = h->ev_out_ready[i] = h->ev_out_copied[i] = nullptr;
  h->d_ibslot_u = h->d_ibslot_v = h->d_iblev = h->d_lev2cap_u = h->d_lev2cap_v = nullptr;
  h->cap = nullptr;
  h->d_ibrec = nullptr;
  h->d_iboff = nullptr;
  h->duib = nullptr;
  std::vector<int> lev2cap_u(nu, -1), lev2cap_v(nv, -1);  // captured physical planes of the IB forcing
  if (h->ib) {
    const int d = cfg->dny;
    h->nib = 2 * d;
    std::vector<int> iblev(2 * h->nib), ibslot_u(nu, -1), ibslot_v(nv, -1);
    for (int s = 0; s < h->nib; ++s) {
      int qu = (s < d) ? 1 + s : nu - 1 - d + (s - d);
      int qv = (s < d) ? 1 + s : nv - 1 - d + (s - d);
      iblev[2 * s] = qu; iblev[2 * s + 1] = qv;
      ibslot_u[qu] = s; ibslot_v[qv] = s;
    }
    // captured levels: u ib levels + the two tip reference levels; v ib levels
    int nc2 = 0;
    for (int q = 1; q <= nu - 2; ++q) {
      bool need = ibslot_u[q] >= 0 || q == d + 1 || q == cfg->nn + 1 + d;
      if (need) { lev2cap_u[q] = nc2; ++nc2; }
    }
    for (int q = 1; q <= nv - 2; ++q)
      if (ibslot_v[q] >= 0) { lev2cap_v[q] = nc2; ++nc2; }
    h->ncap = nc2;
    std::vector<int> lu(cfg->list_ib_u, cfg->list_ib_u + 6 * (size_t)cfg->nib_u);
    std::vector<int> lv(cfg->list_ib_v, cfg->list_ib_v + 6 * (size_t)cfg->nib_v);
    // validate list indices against the plane and the level ranges
    for (size_t e = 0; e < lu.size() / 6; ++e) {
      const int *L = &lu[6 * e];
      if (L[0] < 1 || L[0] > g.G1 || L[1] < 1 || L[1] > g.G2 || L[3] < 1 || L[3] > g.G1 || L[4] < 1 || L[4] > g.G2 ||
          L[2] + d < 0 || L[2] + d >= nu || L[5] + d < 0 || L[5] + d >= nu) {
        int rc = fail(h, LH_EINVAL, "immersed-boundary u list index out of range"); lh_destroy(h); return rc;
      }
    }
    for (size_t e = 0; e < lv.size() / 6; ++e) {
      const int *L = &lv[6 * e];
      if (L[0] < 1 || L[0] > g.G1 || L[1] < 1 || L[1] > g.G2 || L[3] < 1 || L[3] > g.G1 || L[4] < 1 || L[4] > g.G2 ||
          L[2] + d < 0 || L[2] + d >= nv || L[5] + d < 0 || L[5] + d >= nv) {
        int rc = fail(h, LH_EINVAL, "immersed-boundary v list index out of range"); lh_destroy(h); return rc;
      }
    }
    // forced points as records of du's planes (slot s, field f) sorted by (plane, row), in
    // list order within a row: a u-list point forces u1 and u3, a v-list point v. Points
    // whose level is not an immersed level or whose reference level is not captured are
    // skipped (the reference's lists never hold such points).
    const size_t pp = (size_t)g.G1 * g.G2;
    const size_t nrow = (size_t)3 * h->nib * g.G2;
    std::vector<std::vector<IbRec>> rows(nrow);
    auto add = [&](const int *L, double A, const std::vector<int> &slot, const std::vector<int> &l2c, int f) {
      const int q = L[2] + d, q1 = L[5] + d;
      const int s = slot[q], cs = l2c[q], cs1 = l2c[q1];
      if (s < 0 || cs < 0 || cs1 < 0) return;
      IbRec R;
      R.i = L[0] - 1; R.k = L[1] - 1;
      R.src = (long long)((size_t)(cs * 3 + f) * pp + (size_t)R.k * g.G1 + R.i);
      R.ref = (long long)((size_t)(cs1 * 3 + f) * pp + (size_t)(L[4] - 1) * g.G1 + (L[3] - 1));
      R.A = A;
      rows[((size_t)s * 3 + f) * g.G2 + R.k].push_back(R);
    };
    for (size_t e = 0; e < lu.size() / 6; ++e) {
      add(&lu[6 * e], cfg->A_ib_u[e], ibslot_u, lev2cap_u, 0);
      add(&lu[6 * e], cfg->A_ib_u[e], ibslot_u, lev2cap_u, 2);
    }
    for (size_t e = 0; e < lv.size() / 6; ++e) add(&lv[6 * e], cfg->A_ib_v[e], ibslot_v, lev2cap_v, 1);
    std::vector<IbRec> rec;
    std::vector<int> off(nrow + 1, 0);
    for (size_t r = 0; r < nrow; ++r) {
      off[r] = (int)rec.size();
      rec.insert(rec.end(), rows[r].begin(), rows[r].end());
    }
    off[nrow] = (int)rec.size();
    if (rec.empty()) rec.push_back(IbRec{0, 0, 0, 0, 0.0});  // a valid pointer; no range refers to it
    h->d_ibrec = (IbRec *)upload_vec(rec, ce);
    if (ce == cudaSuccess) h->d_iboff = (int *)upload_vec(off, ce);
    h->d_ibslot_u = (int *)upload_vec(ibslot_u, ce); h->d_ibslot_v = (int *)upload_vec(ibslot_v, ce);
    h->d_iblev = (int *)upload_vec(iblev, ce);
    h->d_lev2cap_u = (int *)upload_vec(lev2cap_u, ce); h->d_lev2cap_v = (int *)upload_vec(lev2cap_v, ce);
    if (ce != cudaSuccess) { int rc = fail(h, LH_ECUDA, cudaGetErrorString(ce)); lh_destroy(h); return rc; }
    ZA(h->cap, h->vsz / 2 * (size_t)h->ncap * 3 * pp);
    ZA(h->duib, vs * (size_t)h->nib * 3 * nc);
  }
  if (cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&h->st2, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming) != cudaSuccess) {
    int rc = fail(h, LH_ECUDA, "cudaStreamCreate/cudaEventCreate"); lh_destroy(h); return rc;
  }
  {  // views: slot tables, capture slots of view 0, twiddles; solve segments; band columns
    std::vector<int> slotq, capv;
    size_t off[2];
    for (int vi = 0; vi < 2; ++vi) {
      off[vi] = slotq.size();
      slotq.insert(slotq.end(), vsl[vi][0].begin(), vsl[vi][0].end());
      slotq.insert(slotq.end(), vsl[vi][1].begin(), vsl[vi][1].end());
    }
    for (int q : vsl[0][0]) capv.push_back(lev2cap_u[q]);
    for (int q : vsl[0][1]) capv.push_back(lev2cap_v[q]);
    // every captured level must be a plane of view 0 (the immersed region is in the wall bands)
    int ncapv = 0;
    for (int x : capv) ncapv += (x >= 0);
    if (ncapv != h->ncap) { int rc = fail(h, LH_EINVAL, "immersed region outside the wall bands"); lh_destroy(h); return rc; }
    h->d_slotq = (int *)upload_vec(slotq, ce);
    if (ce == cudaSuccess) h->d_capv = (int *)upload_vec(capv, ce);
    std::vector<int2> vcol;
    if (mb) {
      for (int c : longc) vcol.push_back(make_int2(c, 1));
      for (int c : shortc) vcol.push_back(make_int2(c, 0));
      for (int c : shortc) vcol.push_back(make_int2(c, 2));
      if (ce == cudaSuccess) h->d_vcol = (int2 *)upload_vec(vcol, ce);
    }
    std::vector<int> bcols(longc);
    bcols.insert(bcols.end(), shortc.begin(), shortc.end());
    if (ce == cudaSuccess) h->d_bcols = (int *)upload_vec(bcols, ce);
    h->twv[0][0] = h->twx; h->twv[0][1] = h->twz;
    h->twv[1][0] = h->twv[1][1] = nullptr;
    if (mb && ce == cudaSuccess) {
      if (h->prec == LH_PREC_FP64) {
        std::vector<double> tx, tz;
        twiddles(cfg->Ngal1c, tx); twiddles(cfg->Ngal2c, tz);
        h->twv[1][0] = upload_vec(tx, ce); if (ce == cudaSuccess) h->twv[1][1] = upload_vec(tz, ce);
      } else {
        std::vector<float> tx, tz;
        twiddles(cfg->Ngal1c, tx); twiddles(cfg->Ngal2c, tz);
        h->twv[1][0] = upload_vec(tx, ce); if (ce == cudaSuccess) h->twv[1][1] = upload_vec(tz, ce);
      }
    }
    if (ce != cudaSuccess) { int rc = fail(h, LH_ECUDA, cudaGetErrorString(ce)); lh_destroy(h); return rc; }
    g.vcol = mb ? h->d_vcol : nullptr;
    for (int vi = 0; vi < 2; ++vi) {
      Geo &gv = h->gv[vi];
      gv = g;
      gv.nuI = (int)vsl[vi][0].size(); gv.nvI = (int)vsl[vi][1].size();
      gv.slotq = mb ? h->d_slotq + off[vi] : nullptr;
      if (vi == 1) {
        gv.N1 = cfg->N1c; gv.N2 = cfg->N2c; gv.N1h = cfg->N1c / 2 + 1;
        gv.G1 = cfg->Ngal1c; gv.G2 = cfg->Ngal2c; gv.ncol = gv.N1h * gv.N2;
      }
    }
  }
  {  // statistics accumulators
    const int *N3 = cfg->N3, *N4 = cfg->N4;
    int ncl = std::max(std::max(N4[1] - N4[0], N4[3] - N4[2]), std::max(N3[1] - N3[0], N3[3] - N3[2]));
    const bool tiles = cfg->ntilex > 0 && cfg->ntilez > 0 && g.G1 % cfg->ntilex == 0 && g.G2 % cfg->ntilez == 0;
    h->st_ncl = ncl;
    h->st_ntx = tiles ? cfg->ntilex : 0;
    h->st_dnx = tiles ? g.G1 / cfg->ntilex : 0;
    h->st_dnz = tiles ? g.G2 / cfg->ntilez : 0;
    h->istat = 0;
    ZA(h->st_pl, sizeof(double) * 11 * (size_t)nu);
    ZA(h->st_cd, sizeof(double) * 9 * (size_t)ncl * (tiles ? (size_t)h->st_dnx * h->st_dnz : 1));
    ZA(h->st_pp, sizeof(double) * 2 * (size_t)(nu - 2));
    ZA(h->st_cd4, sizeof(double) * 4 * (size_t)(ncl + 1) * (tiles ? (size_t)h->st_dnx * h->st_dnz : 1));
  }
  int rc = set_smem_attrs_all(h);
  if (rc != LH_OK) { lh_destroy(h); return rc; }
  {
    int lim = 0;
    if (smem_optin(&lim) || cudaFuncSetAttribute((const void *)k_press3<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess ||
        cudaFuncSetAttribute((const void *)k_press3<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess ||
        cudaFuncSetAttribute((const void *)k_press3<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess ||
        cudaFuncSetAttribute((const void *)k_helm_u_mx3<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess ||
        cudaFuncSetAttribute((const void *)k_helm_u_mx3<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess ||
        cudaFuncSetAttribute((const void *)k_helm_u_mx3<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess ||
        cudaFuncSetAttribute((const void *)k_helm_v_mx3<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess ||
        cudaFuncSetAttribute((const void *)k_helm_v_mx3<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess ||
        cudaFuncSetAttribute((const void *)k_helm_v_mx3<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess) {
      rc = fail(h, LH_ECUDA, "cudaFuncSetAttribute(k_press3)"); lh_destroy(h); return rc;
    }
  }
  {  // function attributes are per process, not per handle: the device's limit serves every channel
    int lim = 0;
    if (smem_optin(&lim) || (size_t)lim < 8 * sizeof(double) * (size_t)(std::max(nu, nv) + 1)) {
      rc = fail(h, LH_EINVAL, "too many levels for the (0,0) solve's shared memory"); lh_destroy(h); return rc;
    }
    if (cudaFuncSetAttribute((const void *)k_helm00_pcr, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess) {
      rc = fail(h, LH_ECUDA, "cudaFuncSetAttribute(k_helm00_pcr)"); lh_destroy(h); return rc;
    }
  }
  if (cudaFuncSetAttribute((const void *)k_meanflow_pcr, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024) !=
      cudaSuccess) {
    rc = fail(h, LH_ECUDA, "cudaFuncSetAttribute(k_meanflow_pcr)"); lh_destroy(h); return rc;
  }
  h->triad = (cfg->nonlin_form == LH_NONLIN_TRIADS) ? 1 : 0;
  h->d_terms = nullptr; h->d_wb = h->d_lid = h->d_tmap = nullptr; h->tri_nterms = 0;
  if (h->triad) {  // expand and upload the triad lists (nonlinRead, start.f90:2983-3069)
    TriadHost th;
    std::string e = build_triads(cfg, g, th);
    if (!e.empty()) { rc = fail(h, LH_EINVAL, e); lh_destroy(h); return rc; }
    h->d_terms = (uint32_t *)upload_vec(th.terms, ce);
    if (ce == cudaSuccess) h->d_wb = (int *)upload_vec(th.wb, ce);
    if (ce == cudaSuccess) h->d_lid = (int *)upload_vec(th.lid, ce);
    if (ce == cudaSuccess) h->d_tmap = (int *)upload_vec(th.tmap, ce);
    if (ce != cudaSuccess) {
      rc = fail(h, ce == cudaErrorMemoryAllocation ? LH_ENOMEM : LH_ECUDA, std::string("triad lists: ") + cudaGetErrorString(ce));
      lh_destroy(h);
      return rc;
    }
    h->tg.terms = h->d_terms; h->tg.wb = h->d_wb; h->tg.lid = h->d_lid; h->tg.tmap = h->d_tmap;
    h->tg.Tw = th.Tw; h->tg.T = th.T; h->tg.nx = cfg->triad_nx; h->tg.nz = cfg->triad_nz; h->tg.P = th.P;
    h->tri_nterms = th.nterms;
    h->tri_threads = std::min(32 * th.Tw, 512);
    h->tri_smem = (size_t)(3 * th.P + 1) * h->vsz;
    int lim = 0;
    if (smem_optin(&lim) || h->tri_smem > (size_t)lim) {
      rc = fail(h, LH_EINVAL, "plane too large for the triad form (shared memory)"); lh_destroy(h); return rc;
    }
    // the device's limit, not this channel's need: the attribute is shared by every handle
    cudaError_t ea = (h->prec == LH_PREC_FP64)
                         ? cudaFuncSetAttribute(k_triad<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim)
                         : cudaFuncSetAttribute(k_triad<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    if (ea != cudaSuccess) { rc = fail(h, LH_ECUDA, std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(ea)); lh_destroy(h); return rc; }
  }
  {  // pressure factors, once (start.f90:656-658)
    const int nb = (g.nvc + NTHR_H - 1) / NTHR_H;
    k_build_dg<<<nb, NTHR_H, 0, h->st>>>(h->dg1, h->dg2, h->dg3, g);
    cudaError_t e = cudaStreamSynchronize(h->st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) { rc = fail(h, LH_ECUDA, std::string("k_build_dg: ") + cudaGetErrorString(e)); lh_destroy(h); return rc; }
  }
  // keep host copies of the arrays
  h->h_yu.assign(cfg->yu, cfg->yu + nu);
  h->h_yv.assign(cfg->yv, cfg->yv + nv);
  h->cfg.yu = h->h_yu.data(); h->cfg.yv = h->h_yv.data();
  h->cfg.dthdyu = h->cfg.dthdyv = h->cfg.dyu2i = h->cfg.dyv2i = nullptr;
  h->cfg.k1x = h->cfg.k2x = h->cfg.k1z = h->cfg.k2z = nullptr;
  h->cfg.list_ib_u = h->cfg.list_ib_v = nullptr;
  h->cfg.A_ib_u = h->cfg.A_ib_v = nullptr;
  h->cfg.triad_off = h->cfg.triad_len = nullptr;
  h->cfg.triad_data = nullptr;
  h->cfg.triad_set_u = h->cfg.triad_set_v = nullptr;
  *out = h;
  return LH_OK;
}

extern "C" int lh_destroy(lh_handle *h) {
  if (!h) return LH_EINVAL;
  if (h->graph_ready) { cudaGraphExecDestroy(h->gexec); cudaGraphDestroy(h->graph); }
  void *bufs[] = {h->u1, h->u2, h->u3, h->p, h->Nu1, h->Nu2, h->Nu3, h->dg1, h->dg2, h->dg3, h->ysf, h->N1xz, h->N2xz, h->N3xz, h->uvf, h->vvc,
                  h->wvf, h->psi, h->a3s, h->mfw, h->A, h->B, h->twx, h->twz, h->twx64, h->twz64, h->geo_pool, h->geo_poolf, h->sc, h->stage,
                  h->d_ibslot_u, h->d_ibslot_v, h->d_iblev, h->d_lev2cap_u,
                  h->d_lev2cap_v, h->d_ibrec, h->d_iboff, h->cap, h->duib, h->d_terms, h->d_wb, h->d_lid, h->d_tmap,
                  h->d_slotq, h->d_capv, h->d_vcol, h->d_bcols, h->twv[1][0], h->twv[1][1],
                  h->ysv, h->a3v, h->st_pl, h->st_cd, h->st_pp, h->st_cd4, h->d_cond_list, h->d_cond_scr, h->d_sp, h->d_slip, h->d_slip_inst, h->stage_in, h->stage_out};
  for (void *b : bufs)
    if (b) cudaFree(b);
  for (int i = 0; i < 4; ++i)
    for (cudaEvent_t e : {h->ev_in_copied[i], h->ev_in_used[i], h->ev_out_ready[i], h->ev_out_copied[i]})
      if (e) cudaEventDestroy(e);
  if (h->st_in) cudaStreamDestroy(h->st_in);
  if (h->st_out) cudaStreamDestroy(h->st_out);
  if (h->ev_fork) cudaEventDestroy(h->ev_fork);
  if (h->ev_join) cudaEventDestroy(h->ev_join);
  if (h->st2) cudaStreamDestroy(h->st2);
  if (h->st) cudaStreamDestroy(h->st);
  delete h;
  return LH_OK;
}

extern "C" const char *lh_last_error(lh_handle *h) { return h ? h->err.c_str() : t_last_err.c_str(); }

extern "C" void *lh_stream(lh_handle *h) { return h ? (void *)h->st : nullptr; }

extern "C" int64_t lh_kernel_launches(lh_handle *h) { return h ? h->launches : -1; }

extern "C" int lh_device_state(lh_handle *h, void **u1, void **u2, void **u3, void **p) {
  if (!h) return LH_EINVAL;
  if (u1) *u1 = h->u1;
  if (u2) *u2 = h->u2;
  if (u3) *u3 = h->u3;
  if (p) *p = h->p;
  return LH_OK;
}

// host [col][lev] -> device [lev][col]
static int put_field(lh_handle *h, double2 *dst, int nlev, const double *src) {
  const int nc = h->g.ncol;
  CK(cudaMemcpyAsync(h->stage, src, sizeof(double2) * (size_t)nc * nlev, cudaMemcpyHostToDevice, h->st));
  dim3 grid((nlev + 31) / 32, (nc + 31) / 32), blk(32, 8);
  KL("k_transpose", k_transpose<<<grid, blk, 0, h->st>>>(h->stage, dst, nc, nlev));
  return LH_OK;
}
static int get_field(lh_handle *h, const double2 *srcd, int nlev, double *dst) {
  const int nc = h->g.ncol;
  dim3 grid((nc + 31) / 32, (nlev + 31) / 32), blk(32, 8);
  KL("k_transpose", k_transpose<<<grid, blk, 0, h->st>>>(srcd, h->stage, nlev, nc));
  CK(cudaMemcpyAsync(dst, h->stage, sizeof(double2) * (size_t)nc * nlev, cudaMemcpyDeviceToHost, h->st));
  return LH_OK;
}

extern "C" int lh_upload_state(lh_handle *h, const double *u1, const double *u2, const double *u3, const double *p) {
  if (!h) return LH_EINVAL;
  if (h->g.mb) return fail(h, LH_EINVAL, "multiblock channel: use lh_upload_band");
  int rc;
  if (u1 && (rc = put_field(h, h->u1, h->g.nu, u1))) return rc;
  if (u2 && (rc = put_field(h, h->u2, h->g.nv, u2))) return rc;
  if (u3 && (rc = put_field(h, h->u3, h->g.nu, u3))) return rc;
  if (p && (rc = put_field(h, h->p, h->g.np, p))) return rc;
  CK(cudaStreamSynchronize(h->st));
  return LH_OK;
}

extern "C" int lh_download_state(lh_handle *h, double *u1, double *u2, double *u3, double *p) {
  if (!h) return LH_EINVAL;
  if (h->g.mb) return fail(h, LH_EINVAL, "multiblock channel: use lh_download_band");
  int rc;  // stream order protects the staging buffer between the fields
  if (u1 && (rc = get_field(h, h->u1, h->g.nu, u1))) return rc;
  if (u2 && (rc = get_field(h, h->u2, h->g.nv, u2))) return rc;
  if (u3 && (rc = get_field(h, h->u3, h->g.nu, u3))) return rc;
  if (p && (rc = get_field(h, h->p, h->g.np, p))) return rc;
  CK(cudaStreamSynchronize(h->st));
  return LH_OK;
}

// ---- asynchronous state I/O ----
// The host->device copy of an upload runs on its own stream as soon as the previous
// upload's transposes have consumed the input staging; only its transposes into the
// state wait for the work already queued (the previous step, the previous download's
// transposes). A download's transposes follow the queued steps on the main stream and its
// device->host copy runs on a second copy stream, overlapping the steps queued after it.
static int async_io_init(lh_handle *h) {
  if (h->ev_out_copied[3]) return LH_OK;  // the last resource created below
  const size_t n = (size_t)(2 * h->g.nu + h->g.nv + h->g.np) * h->g.ncol;
  // each resource on its own, so that a failure part-way is completed by the next call
  if (!h->stage_in) CK(cudaMalloc(&h->stage_in, sizeof(double2) * n));
  if (!h->stage_out) CK(cudaMalloc(&h->stage_out, sizeof(double2) * n));
  if (!h->st_in) CK(cudaStreamCreateWithFlags(&h->st_in, cudaStreamNonBlocking));
  if (!h->st_out) CK(cudaStreamCreateWithFlags(&h->st_out, cudaStreamNonBlocking));
  for (int i = 0; i < 4; ++i) {
    for (cudaEvent_t *e : {&h->ev_in_copied[i], &h->ev_in_used[i], &h->ev_out_ready[i], &h->ev_out_copied[i]}) {
      if (*e) continue;
      CK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
      CK(cudaEventRecord(*e, h->st));  // completed once the work queued so far is done
    }
  }
  return LH_OK;
}
// a slot's staging may be refilled once its previous contents are consumed; the whole-state
// slot overlaps every band slot
static int wait_slot(lh_handle *h, cudaStream_t st, cudaEvent_t *ev, int slot) {
  if (slot == 0) {
    for (int i = 0; i < 4; ++i) CK(cudaStreamWaitEvent(st, ev[i], 0));
  } else {
    CK(cudaStreamWaitEvent(st, ev[slot], 0));
    CK(cudaStreamWaitEvent(st, ev[0], 0));
  }
  return LH_OK;
}
// field f of the state: device array, levels, offset in the staging
static void state_field(lh_handle *h, int f, double2 *&dev, int &nlev, size_t &off) {
  const size_t nc = h->g.ncol, nu = h->g.nu, nv = h->g.nv;
  double2 *F[4] = {h->u1, h->u2, h->u3, h->p};
  const int L[4] = {h->g.nu, h->g.nv, h->g.nu, h->g.np};
  const size_t O[4] = {0, nu * nc, (nu + nv) * nc, (2 * nu + nv) * nc};
  dev = F[f]; nlev = L[f]; off = O[f];
}

extern "C" int lh_upload_state_async(lh_handle *h, const double *u1, const double *u2, const double *u3,
                                     const double *p) {
  if (!h) return LH_EINVAL;
  if (h->g.mb) return fail(h, LH_EINVAL, "multiblock channel: use lh_upload_band");
  int rc = async_io_init(h);
  if (rc) return rc;
  const double *H[4] = {u1, u2, u3, p};
  const int nc = h->g.ncol;
  if ((rc = wait_slot(h, h->st_in, h->ev_in_used, 0))) return rc;
  for (int f = 0; f < 4; ++f) {
    if (!H[f]) continue;
    double2 *dev; int nl; size_t off;
    state_field(h, f, dev, nl, off);
    CK(cudaMemcpyAsync(h->stage_in + off, H[f], sizeof(double2) * (size_t)nc * nl, cudaMemcpyHostToDevice, h->st_in));
  }
  CK(cudaEventRecord(h->ev_in_copied[0], h->st_in));
  CK(cudaStreamWaitEvent(h->st, h->ev_in_copied[0], 0));
  for (int f = 0; f < 4; ++f) {
    if (!H[f]) continue;
    double2 *dev; int nl; size_t off;
    state_field(h, f, dev, nl, off);
    dim3 grid((nl + 31) / 32, (nc + 31) / 32), blk(32, 8);
    KL("k_transpose", k_transpose<<<grid, blk, 0, h->st>>>(h->stage_in + off, dev, nc, nl));
  }
  CK(cudaEventRecord(h->ev_in_used[0], h->st));
  return LH_OK;
}

extern "C" int lh_download_state_async(lh_handle *h, double *u1, double *u2, double *u3, double *p) {
  if (!h) return LH_EINVAL;
  if (h->g.mb) return fail(h, LH_EINVAL, "multiblock channel: use lh_download_band");
  int rc = async_io_init(h);
  if (rc) return rc;
  double *H[4] = {u1, u2, u3, p};
  const int nc = h->g.ncol;
  if ((rc = wait_slot(h, h->st, h->ev_out_copied, 0))) return rc;
  for (int f = 0; f < 4; ++f) {
    if (!H[f]) continue;
    double2 *dev; int nl; size_t off;
    state_field(h, f, dev, nl, off);
    dim3 grid((nc + 31) / 32, (nl + 31) / 32), blk(32, 8);
    KL("k_transpose", k_transpose<<<grid, blk, 0, h->st>>>(dev, h->stage_out + off, nl, nc));
  }
  CK(cudaEventRecord(h->ev_out_ready[0], h->st));
  CK(cudaStreamWaitEvent(h->st_out, h->ev_out_ready[0], 0));
  for (int f = 0; f < 4; ++f) {
    if (!H[f]) continue;
    double2 *dev; int nl; size_t off;
    state_field(h, f, dev, nl, off);
    CK(cudaMemcpyAsync(H[f], h->stage_out + off, sizeof(double2) * (size_t)nc * nl, cudaMemcpyDeviceToHost, h->st_out));
  }
  CK(cudaEventRecord(h->ev_out_copied[0], h->st_out));
  return LH_OK;
}

// one band's cfield [column][level] (staged on the device) <-> the wall-grid layout
static int band_field(lh_handle *h, int band, int field, double2 *dev, const double *hin, double *hout) {
  const int b = band - 1;
  const int ncb = (band == 2) ? h->nlong : h->nshort;
  const int *cols = h->d_bcols + ((band == 2) ? 0 : h->nlong);
  const int lo = h->g.bq[b][field == 3 ? 4 : (field == 1 ? 2 : 0)];
  const int hi = h->g.bq[b][field == 3 ? 5 : (field == 1 ? 3 : 1)];
  const int nl = hi - lo + 1;
  const size_t n = (size_t)ncb * nl;
  if (n == 0) return LH_OK;
  const int nb = (int)((n + NTHR_H - 1) / NTHR_H);
  if (hin) {
    CK(cudaMemcpyAsync(h->stage, hin, sizeof(double2) * n, cudaMemcpyHostToDevice, h->st));
    KL("k_band_io", k_band_io<<<nb, NTHR_H, 0, h->st>>>(dev, h->stage, cols, ncb, nl, lo, h->g.ncol, 1));
  } else {
    KL("k_band_io", k_band_io<<<nb, NTHR_H, 0, h->st>>>(dev, h->stage, cols, ncb, nl, lo, h->g.ncol, 0));
    CK(cudaMemcpyAsync(hout, h->stage, sizeof(double2) * n, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
  }
  return LH_OK;
}

extern "C" int lh_upload_band(lh_handle *h, int band, const double *u1, const double *u2, const double *u3,
                              const double *p) {
  if (!h) return LH_EINVAL;
  if (band < 1 || band > 3) return fail(h, LH_EINVAL, "band must be 1, 2 or 3");
  double2 *F[4] = {h->u1, h->u2, h->u3, h->p};
  const double *H[4] = {u1, u2, u3, p};
  for (int f = 0; f < 4; ++f) {
    if (!H[f]) continue;
    int rc = band_field(h, band, f, F[f], H[f], nullptr);
    if (rc) return rc;
    CK(cudaStreamSynchronize(h->st));  // the staging buffer is reused by the next field
  }
  return LH_OK;
}

extern "C" int lh_download_band(lh_handle *h, int band, double *u1, double *u2, double *u3, double *p) {
  if (!h) return LH_EINVAL;
  if (band < 1 || band > 3) return fail(h, LH_EINVAL, "band must be 1, 2 or 3");
  double2 *F[4] = {h->u1, h->u2, h->u3, h->p};
  double *H[4] = {u1, u2, u3, p};
  for (int f = 0; f < 4; ++f) {
    if (!H[f]) continue;
    int rc = band_field(h, band, f, F[f], nullptr, H[f]);
    if (rc) return rc;
  }
  return LH_OK;
}

// ---- asynchronous band I/O: as the state calls above, one staging region per band ----
// band b's field f: its columns, level range and size; regions laid out band after band
static void band_geom(lh_handle *h, int band, int field, const int *&cols, int &ncb, int &lo, int &nl) {
  const int b = band - 1;
  ncb = (band == 2) ? h->nlong : h->nshort;
  cols = h->d_bcols + ((band == 2) ? 0 : h->nlong);
  lo = h->g.bq[b][field == 3 ? 4 : (field == 1 ? 2 : 0)];
  const int hi = h->g.bq[b][field == 3 ? 5 : (field == 1 ? 3 : 1)];
  nl = hi - lo + 1;
}
static size_t band_offset(lh_handle *h, int band, int field) {
  size_t off = 0;
  for (int b = 1; b <= 3; ++b)
    for (int f = 0; f < 4; ++f) {
      if (b == band && f == field) return off;
      const int *cols; int ncb, lo, nl;
      band_geom(h, b, f, cols, ncb, lo, nl);
      off += (size_t)ncb * nl;
    }
  return off;
}

extern "C" int lh_upload_band_async(lh_handle *h, int band, const double *u1, const double *u2, const double *u3,
                                    const double *p) {
  if (!h) return LH_EINVAL;
  if (band < 1 || band > 3) return fail(h, LH_EINVAL, "band must be 1, 2 or 3");
  int rc = async_io_init(h);
  if (rc) return rc;
  if (band_offset(h, 4, 0) > (size_t)(2 * h->g.nu + h->g.nv + h->g.np) * h->g.ncol)
    return fail(h, LH_EINVAL, "band layouts larger than the staging buffer");
  double2 *F[4] = {h->u1, h->u2, h->u3, h->p};
  const double *H[4] = {u1, u2, u3, p};
  if ((rc = wait_slot(h, h->st_in, h->ev_in_used, band))) return rc;
  for (int f = 0; f < 4; ++f) {
    const int *cols; int ncb, lo, nl;
    band_geom(h, band, f, cols, ncb, lo, nl);
    if (!H[f] || (size_t)ncb * nl == 0) continue;
    CK(cudaMemcpyAsync(h->stage_in + band_offset(h, band, f), H[f], sizeof(double2) * (size_t)ncb * nl,
                       cudaMemcpyHostToDevice, h->st_in));
  }
  CK(cudaEventRecord(h->ev_in_copied[band], h->st_in));
  CK(cudaStreamWaitEvent(h->st, h->ev_in_copied[band], 0));
  for (int f = 0; f < 4; ++f) {
    const int *cols; int ncb, lo, nl;
    band_geom(h, band, f, cols, ncb, lo, nl);
    const size_t n = (size_t)ncb * nl;
    if (!H[f] || n == 0) continue;
    const int nb = (int)((n + NTHR_H - 1) / NTHR_H);
    KL("k_band_io", k_band_io<<<nb, NTHR_H, 0, h->st>>>(F[f], h->stage_in + band_offset(h, band, f), cols, ncb, nl, lo,
                                                         h->g.ncol, 1));
  }
  CK(cudaEventRecord(h->ev_in_used[band], h->st));
  return LH_OK;
}

extern "C" int lh_download_band_async(lh_handle *h, int band, double *u1, double *u2, double *u3, double *p) {
  if (!h) return LH_EINVAL;
  if (band < 1 || band > 3) return fail(h, LH_EINVAL, "band must be 1, 2 or 3");
  int rc = async_io_init(h);
  if (rc) return rc;
  double2 *F[4] = {h->u1, h->u2, h->u3, h->p};
  double *H[4] = {u1, u2, u3, p};
  if ((rc = wait_slot(h, h->st, h->ev_out_copied, band))) return rc;
  for (int f = 0; f < 4; ++f) {
    const int *cols; int ncb, lo, nl;
    band_geom(h, band, f, cols, ncb, lo, nl);
    const size_t n = (size_t)ncb * nl;
    if (!H[f] || n == 0) continue;
    const int nb = (int)((n + NTHR_H - 1) / NTHR_H);
    KL("k_band_io", k_band_io<<<nb, NTHR_H, 0, h->st>>>(F[f], h->stage_out + band_offset(h, band, f), cols, ncb, nl, lo,
                                                         h->g.ncol, 0));
  }
  CK(cudaEventRecord(h->ev_out_ready[band], h->st));
  CK(cudaStreamWaitEvent(h->st_out, h->ev_out_ready[band], 0));
  for (int f = 0; f < 4; ++f) {
    const int *cols; int ncb, lo, nl;
    band_geom(h, band, f, cols, ncb, lo, nl);
    const size_t n = (size_t)ncb * nl;
    if (!H[f] || n == 0) continue;
    CK(cudaMemcpyAsync(H[f], h->stage_out + band_offset(h, band, f), sizeof(double2) * n, cudaMemcpyDeviceToHost,
                       h->st_out));
  }
  CK(cudaEventRecord(h->ev_out_copied[band], h->st_out));
  return LH_OK;
}

extern "C" int lh_set_scalars(lh_handle *h, const lh_scalars *s) {
  if (!h || !s) return LH_EINVAL;
  DevScalars d;
  memset(&d, 0, sizeof(d));
  d.t = s->t; d.dt = s->dt; d.dti = s->dti; d.dtc = s->dtc; d.err = s->err; d.mpgx = s->mpgx;
  d.QxT = s->QxT; d.Qx = s->Qx; d.iter = s->iter;
  CK(cudaMemcpyAsync(h->sc, &d, sizeof(d), cudaMemcpyHostToDevice, h->st));
  KL("k_flowrate", k_flowrate<<<1, 32, 0, h->st>>>(h->u1, h->g, h->sc, h->g.flag_ctpress != 1 ? 1 : 0));
  const int nb = (h->g.nvc + NTHR_H - 1) / NTHR_H;
  KL("k_reset_err", k_reset_err<<<1, 32, 0, h->st>>>(h->sc));
  KL("k_divmax", k_divmax<<<nb, NTHR_H, 0, h->st>>>(h->u1, h->u2, h->u3, h->g, h->sc));
  KL("k_err_from_bits", k_err_from_bits<<<1, 32, 0, h->st>>>(h->sc));
  CK(cudaStreamSynchronize(h->st));
  return LH_OK;
}

extern "C" int lh_get_scalars(lh_handle *h, lh_scalars *s) {
  if (!h || !s) return LH_EINVAL;
  DevScalars d;
  CK(cudaMemcpyAsync(&d, h->sc, sizeof(d), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  s->t = d.t; s->dt = d.dt; s->dti = d.dti; s->dtc = d.dtc; s->err = d.err; s->mpgx = d.mpgx;
  s->QxT = d.QxT; s->Qx = d.Qx; s->iter = d.iter;
  return LH_OK;
}

extern "C" int lh_history_record(lh_handle *h, lh_history *out) {
  if (!h || !out) return LH_EINVAL;
  KL("k_history", k_history<<<1, 32, 0, h->st>>>(h->u1, h->g, h->sc));
  DevScalars d;
  CK(cudaMemcpyAsync(&d, h->sc, sizeof(d), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  out->flag_ctpress = h->g.flag_ctpress;
  out->iter = (int32_t)d.iter;
  out->t = d.t; out->dtv = h->g.dtv; out->dtc = d.dtc; out->dt = d.dt; out->err = d.err;
  out->Qx = d.Qx; out->QxT = d.QxT; out->mpgx = d.mpgx; out->dgx = d.dgx;
  out->Umax = d.Umax; out->Uslip = d.Uslip;
  return LH_OK;
}

// ---------------------------------------------------------------------------
// one substep
// ---------------------------------------------------------------------------
template <typename T, int N>
static int launch_zinv(lh_handle *h, const Geo &g, int nslots, const void *twz) {
  typedef typename C2<T>::t V;
  if constexpr (sizeof(T) == 4) {  // the two-stage register form of the mixed inverse z pass
    using P = zp2<N>;
    dim3 grid((g.N1h + P::KB - 1) / P::KB, nslots, 3);
    KL("k_zinv_nl", k_zinv2<N><<<grid, P::NT, P::SMEM, h->st>>>(h->u1, h->u2, h->u3, (float2 *)h->A, g,
                                                                (const float2 *)twz));
  } else {  // FP64: Stockham
    constexpr int KB = kb_zinv<V>(N);
    dim3 grid((g.N1h + KB - 1) / KB, nslots, 3);
    KL("k_zinv_nl", k_zinv_nl<T, N><<<grid, LH_ZINV_THREADS, 2 * (size_t)KB * N * sizeof(V), h->st>>>(
                        h->u1, h->u2, h->u3, (V *)h->A, g, (const V *)twz));
  }
  return LH_OK;
}
template <typename T, int N>
static int launch_xpass(lh_handle *h, const Geo &g, int nslots, int doCFL, const int *capslot, const void *twx) {
  typedef typename C2<T>::t V;
  if constexpr (sizeof(T) == 4 && N <= 384) {  // the two-stage register form of the mixed x pass
    using P = xp2<N>;
    dim3 grid((g.G2 / 2 + P::PB - 1) / P::PB, nslots);
    KL("k_xpass_nl", k_xpass2<N><<<grid, P::NT, P::SMEM, h->st>>>((const float2 *)h->A, (float2 *)h->B, g,
                                                                  (const float2 *)twx, doCFL, h->sc, capslot, (float *)h->cap));
  } else if constexpr (sizeof(T) == 4 && (N == 576 || N == 768 || N == 1152)) {  // three-stage register form
    using P = xp3<N>;
    dim3 grid(g.G2 / 2, nslots);
    KL("k_xpass_nl", k_xpass3<N><<<grid, P::NT, P::SMEM, h->st>>>((const float2 *)h->A, (float2 *)h->B, g,
                                                                  (const float2 *)twx, doCFL, h->sc, capslot, (float *)h->cap));
  } else {  // FP64: Stockham
    static_assert(sizeof(T) == 8, "the mixed x pass has a register form for every compiled length");
    constexpr int PB = pb_xpass<V>(N);
    dim3 grid((g.G2 / 2 + PB - 1) / PB, nslots);
    KL("k_xpass_nl", k_xpass_nl<T, N><<<grid, LH_XPASS_THREADS, 8 * (size_t)PB * N * sizeof(V), h->st>>>(
                         (const V *)h->A, (V *)h->B, g, (const V *)twx, doCFL, h->sc, capslot, (T *)h->cap));
  }
  return LH_OK;
}
template <typename T, int N>
static int launch_zfwd(lh_handle *h, const Geo &g, int nslots, const void *twz) {
  typedef typename C2<T>::t V;
  if constexpr (sizeof(T) == 4) {  // the two-stage register form of the mixed forward z pass
    using P = zf2<N>;
    dim3 grid((g.N1h + P::KF - 1) / P::KF, nslots);
    KL("k_zfwd_nl", k_zfwd2<N><<<grid, P::NTH, P::SMEM, h->st>>>(
                        (const float2 *)h->B, g, (const float2 *)twz, (float2 *)h->N1xz, (float2 *)h->N2xz,
                        (float2 *)h->N3xz, (float2 *)h->uvf, (float2 *)h->vvc, (float2 *)h->wvf));
  } else {  // FP64: Stockham
    constexpr int KB = kb_zfwd<V>(N);
    dim3 grid((g.N1h + KB - 1) / KB, nslots);
    KL("k_zfwd_nl", k_zfwd_nl<T, N><<<grid, LH_ZFWD_THREADS, 8 * (size_t)KB * N * sizeof(V), h->st>>>(
                        (const V *)h->B, g, (const V *)twz, (V *)h->N1xz, (V *)h->N2xz, (V *)h->N3xz, (V *)h->uvf,
                        (V *)h->vvc, (V *)h->wvf));
  }
  return LH_OK;
}

// inverse transforms, products (and CFL maxima at kRK = 1) of one view's planes
template <typename T>
static int view_products(lh_handle *h, int vi, int kRK, bool forward) {
  const Geo &g = h->gv[vi];
  const int nslots = g.nuI + g.nvI;
  if (nslots == 0) return LH_OK;
  const int *capslot = (h->ib && vi == 0) ? h->d_capv : nullptr;
  int rc = LH_EINVAL;
  const void *twx = h->twv[vi][0], *twz = h->twv[vi][1];
  LH_DISPATCH(g.G2, rc = launch_zinv<T, N>(h, g, nslots, twz));
  if (rc) return rc;
  rc = LH_EINVAL;
  LH_DISPATCH(g.G1, rc = launch_xpass<T, N>(h, g, nslots, kRK == 1 ? 1 : 0, capslot, twx));
  if (rc || !forward) return rc;
  rc = LH_EINVAL;
  LH_DISPATCH(g.G2, rc = launch_zfwd<T, N>(h, g, nslots, twz));
  return rc;
}

template <typename T>
static int nonlinear_transforms(lh_handle *h, int kRK) {
  if (kRK == 1) KL("k_reset_cfl", k_reset_cfl<<<1, 32, 0, h->st>>>(h->sc));
  for (int vi = 0; vi < h->nviews; ++vi) {
    const int rc = view_products<T>(h, vi, kRK, true);
    if (rc) return rc;
  }
  return LH_OK;
}

// triad-list form (ops_in_planes): the products come from the lists; the inverse
// transforms still run where the physical velocities are needed (dtc_calc at kRK = 1)
template <typename T>
static int triad_nonlinear(lh_handle *h, int kRK) {
  typedef typename C2<T>::t V;
  const Geo &g = h->g;
  const int nslots = g.nuI + g.nvI;
  if (kRK == 1) {
    KL("k_reset_cfl", k_reset_cfl<<<1, 32, 0, h->st>>>(h->sc));
    const int rc = view_products<T>(h, 0, kRK, false);
    if (rc) return rc;
  }
  KL("k_triad", k_triad<T><<<nslots, h->tri_threads, h->tri_smem, h->st>>>(
                    h->u1, h->u2, h->u3, g, h->tg, (V *)h->N1xz, (V *)h->N2xz, (V *)h->N3xz, (V *)h->uvf,
                    (V *)h->vvc, (V *)h->wvf));
  return LH_OK;
}

// plane transforms through scratch buffers in precision T (leaves: FP64; immersed
// boundaries: the form's transform precision)
template <typename T, int N>
static int launch_spec_zinv(lh_handle *h, const void *spec, void *Ascr, int npl, const void *twz) {
  typedef typename C2<T>::t V;
  if constexpr (sizeof(T) == 4) {  // the two-stage register form (immersed boundaries, mixed form)
    using P = zp2<N>;
    dim3 g1((h->g.N1h + P::KB - 1) / P::KB, npl);
    KL("k_spec_zinv", k_spec_zinv2<N><<<g1, P::NT, P::SMEM, h->st>>>((const float2 *)spec, (float2 *)Ascr, h->g, (const float2 *)twz));
  } else {  // FP64: Stockham
    constexpr int KB = kb_zinv<V>(N);
    dim3 g1((h->g.N1h + KB - 1) / KB, npl);
    KL("k_spec_zinv", k_spec_zinv<T, N><<<g1, NTHR_H, 2 * (size_t)KB * N * sizeof(V), h->st>>>((const double2 *)spec, (V *)Ascr, h->g, (const V *)twz));
  }
  return LH_OK;
}
template <typename T, int N>
static int launch_xinv_phys(lh_handle *h, const void *Ascr, double *phys, int npl, const void *twx) {
  typedef typename C2<T>::t V;
  constexpr int PB = 4 * pb_xpass<V>(N);
  dim3 g2((h->g.G2 / 2 + PB - 1) / PB, npl);
  KL("k_xinv_phys", k_xinv_phys<T, N><<<g2, NTHR_H, 2 * (size_t)PB * N * sizeof(V), h->st>>>((const V *)Ascr, phys, h->g, (const V *)twx));
  return LH_OK;
}
template <typename T, int N>
static int launch_xfwd_phys(lh_handle *h, const double *phys, void *Bscr, int npl, const void *twx) {
  typedef typename C2<T>::t V;
  constexpr int PB = 4 * pb_xpass<V>(N);
  dim3 g1((h->g.G2 / 2 + PB - 1) / PB, npl);
  KL("k_xfwd_phys", k_xfwd_phys<T, N><<<g1, NTHR_H, 2 * (size_t)PB * N * sizeof(V), h->st>>>(phys, (V *)Bscr, h->g, (const V *)twx));
  return LH_OK;
}
template <typename T, int N>
static int launch_zfwd_spec(lh_handle *h, const void *Bscr, void *spec, int npl, const void *twz) {
  typedef typename C2<T>::t V;
  if constexpr (sizeof(T) == 4) {  // the two-stage register form (immersed boundaries, mixed form)
    using P = zp2<N>;
    dim3 g2((h->g.N1h + P::KB - 1) / P::KB, npl);
    KL("k_zfwd_spec", k_zfwd_spec2<N><<<g2, P::NT, P::SMEM, h->st>>>((const float2 *)Bscr, (float2 *)spec, h->g, (const float2 *)twz));
  } else {  // FP64: Stockham
    constexpr int KB = kb_zinv<V>(N);
    dim3 g2((h->g.N1h + KB - 1) / KB, npl);
    KL("k_zfwd_spec", k_zfwd_spec<T, N><<<g2, NTHR_H, 2 * (size_t)KB * N * sizeof(V), h->st>>>((const V *)Bscr, (double2 *)spec, h->g, (const V *)twz));
  }
  return LH_OK;
}

template <typename T, int N>
static int launch_ib_xforce(lh_handle *h, int npl) {
  typedef typename C2<T>::t V;
  constexpr int PB = 4 * pb_xpass<V>(N);
  dim3 g2((h->g.G2 / 2 + PB - 1) / PB, npl);
  KL("k_ib_xforce", k_ib_xforce<T, N><<<g2, NTHR_H, 2 * (size_t)PB * N * sizeof(V), h->st>>>(
                        (const V *)h->A, (V *)h->B, h->g, (const V *)h->twx, h->d_ibrec, h->d_iboff, (const T *)h->cap, h->sc));
  return LH_OK;
}
template <typename T>
static int spec_to_phys(lh_handle *h, const double2 *spec, double *phys, int npl, void *Ascr, const void *twx,
                        const void *twz) {
  int rc = LH_EINVAL;
  LH_DISPATCH(h->g.G2, rc = launch_spec_zinv<T, N>(h, spec, Ascr, npl, twz));
  if (rc) return rc;
  rc = LH_EINVAL;
  LH_DISPATCH(h->g.G1, rc = launch_xinv_phys<T, N>(h, Ascr, phys, npl, twx));
  return rc;
}
template <typename T>
static int phys_to_spec(lh_handle *h, const double *phys, double2 *spec, int npl, void *Bscr, const void *twx,
                        const void *twz) {
  int rc = LH_EINVAL;
  LH_DISPATCH(h->g.G1, rc = launch_xfwd_phys<T, N>(h, phys, Bscr, npl, twx));
  if (rc) return rc;
  rc = LH_EINVAL;
  LH_DISPATCH(h->g.G2, rc = launch_zfwd_spec<T, N>(h, Bscr, spec, npl, twz));
  return rc;
}

static const void *fp64_tw(lh_handle *h, bool x) { return x ? h->twx64 : h->twz64; }

// flowrate_corr after solveU_W, on the side stream (joined before solveP); on the
// main stream when kernels are being timed one by one
// flowrate_corr on the main stream, after the u solve (constant flow rate only)
static int meanflow(lh_handle *h, int kRK) {
  const Geo &g = h->g;
  if (g.flag_ctpress != 0) return LH_OK;
  const size_t pcr = 8 * sizeof(double) * (size_t)(g.nn + 3);
  if (pcr <= 96 * 1024) {  // parallel cyclic reduction in one block
    KL("k_meanflow", k_meanflow_pcr<<<1, 512, pcr, h->st>>>(h->u1, g, h->sc, kRK));
    return LH_OK;
  }
  const size_t mb = 6 * sizeof(double) * (size_t)(g.nn + 3);
  const int sm = mb <= 48 * 1024 ? 1 : 0;
  KL("k_meanflow", k_meanflow<<<1, 256, sm ? mb : 0, h->st>>>(h->u1, g, h->sc, kRK, h->mfw, sm));
  return LH_OK;
}

// shared memory of the staged mixed solves (k_helm_u_mx3 / k_helm_v_mx3): six per-level tables
// and a ring of 28 bytes per thread and slot (D + 1 slots)
static size_t staged_smem(int nlev, int pf, int tb) {
  return pf == 0 ? 0 : (((size_t)6 * nlev * 4 + 15) & ~(size_t)15) + (size_t)28 * (pf + 1) * tb;
}
static size_t press_smem(const Geo &g, int pf, int tb) {
  return sizeof(double) * (((size_t)g.nu + g.nv + 1) & ~(size_t)1) + sizeof(double) * 6 * (size_t)(pf + 1) * tb;
}

template <typename T>
static int substep_launches_t(lh_handle *h, int kRK) {
  typedef typename C2<T>::t V;
  const Geo &g = h->g;
  int rc = h->triad ? triad_nonlinear<T>(h, kRK) : nonlinear_transforms<T>(h, kRK);
  if (rc) return rc;
  if (kRK == 1) KL("k_dt", k_dt<<<1, 32, 0, h->st>>>(g, h->sc));
  const int nb = (g.ncol + NTHR_H - 1) / NTHR_H;
  const int nbu = (g.nvc + h->tb_uw - 1) / h->tb_uw, nbv = (g.nvc + h->tb_v - 1) / h->tb_v;
  if (h->ib) {
    dim3 gd(nb, h->nib);
    if (h->prec == LH_PREC_FP64) {
      KL("k_ib_du", k_ib_du<T><<<gd, NTHR_H, 0, h->st>>>(h->u1, h->u2, h->u3, (V *)h->Nu1, (V *)h->Nu2, (V *)h->Nu3,
                                                         (const V *)h->N1xz, (const V *)h->N2xz, (const V *)h->N3xz,
                                                         (const V *)h->uvf, (const V *)h->vvc, (const V *)h->wvf, h->p,
                                                         (double2 *)h->duib, h->d_iblev, h->nib, g, h->sc, kRK));
    } else {
      KL("k_ib_du", k_ib_du_mx<<<gd, NTHR_H, 0, h->st>>>(h->u1, h->u2, h->u3, (float2 *)h->Nu1, (float2 *)h->Nu2,
                                                         (float2 *)h->Nu3, (const float2 *)h->N1xz, (const float2 *)h->N2xz,
                                                         (const float2 *)h->N3xz, (const float2 *)h->uvf,
                                                         (const float2 *)h->vvc, (const float2 *)h->wvf, h->p, (float2 *)h->duib,
                                                         h->d_iblev, h->nib, g, h->sc, kRK));
    }
    rc = LH_EINVAL;
    LH_DISPATCH(g.G2, rc = launch_spec_zinv<T, N>(h, h->duib, h->A, 3 * h->nib, h->twz));
    if (rc) return rc;
    rc = LH_EINVAL;
    LH_DISPATCH(g.G1, rc = launch_ib_xforce<T, N>(h, 3 * h->nib));
    if (rc) return rc;
    rc = LH_EINVAL;
    LH_DISPATCH(g.G2, rc = launch_zfwd_spec<T, N>(h, h->B, h->duib, 3 * h->nib, h->twz));
    if (rc) return rc;
  }
  // The u/w and v solves are independent: v runs on the side stream while u/w and the
  // mean-flow correction (which follows u) run on the main stream; each solve has its
  // own scratch. In the mixed form mode (0,0) is solved in FP64 by its own kernel on the
  // side stream after v (the other solves skip column 0), overlapping the longer u/w solve;
  // the mean-flow correction, which reads u(0,0), follows the join. (Sequential on the main
  // stream while per-kernel times are profiled.)
  const bool fork = !h->prof;
  cudaStream_t sv = fork ? h->st2 : h->st;
  if (fork) {
    CK(cudaEventRecord(h->ev_fork, h->st));
    CK(cudaStreamWaitEvent(h->st2, h->ev_fork, 0));
  }
  if (!fork) prof_begin(h, "k_helm_v");
  if (h->prec == LH_PREC_FP64) {
    k_helm_v<T><<<nbv, h->tb_v, 0, sv>>>(h->u2, (double2 *)h->Nu2, (const V *)h->N2xz, (const V *)h->vvc, h->p,
                                         h->a3v, g, h->sc, kRK, h->ib ? h->d_ibslot_v : nullptr, (const double2 *)h->duib);
  } else {
    const int nb2v = (2 * g.nvc + h->tb_v - 1) / h->tb_v;
    const size_t sm = staged_smem(g.nv, h->pf_v, h->tb_v);
    const int *ibv = h->ib ? h->d_ibslot_v : nullptr;
    double *V = (double *)h->u2;
    float *NV = (float *)h->Nu2;
    const float *XV = (const float *)h->N2xz, *VV = (const float *)h->vvc;
    const double *PP = (const double *)h->p;
    float2 *YS = (float2 *)h->ysv;
    switch (h->pf_v) {
      case 0: k_helm_v_mx2<<<nb2v, h->tb_v, 0, sv>>>(V, NV, XV, VV, PP, YS, g, h->sc, kRK, ibv, (const float2 *)h->duib); break;
      case 2: k_helm_v_mx3<2><<<nb2v, h->tb_v, sm, sv>>>(V, NV, XV, VV, PP, YS, g, h->sc, kRK, ibv, (const float2 *)h->duib); break;
      case 8: k_helm_v_mx3<8><<<nb2v, h->tb_v, sm, sv>>>(V, NV, XV, VV, PP, YS, g, h->sc, kRK, ibv, (const float2 *)h->duib); break;
      default: k_helm_v_mx3<4><<<nb2v, h->tb_v, sm, sv>>>(V, NV, XV, VV, PP, YS, g, h->sc, kRK, ibv, (const float2 *)h->duib); break;
    }
  }
  if ((rc = count_launch(h))) return rc;
  const bool mixed00 = h->prec == LH_PREC_MIXED;
  if (mixed00) {
    const size_t sm00 = 8 * sizeof(double) * (size_t)(std::max(g.nu, g.nv) + 1);
    KL("k_helm00", k_helm00_pcr<<<6, 512, sm00, sv>>>(
                       (double *)h->u1, (double *)h->u3, (double *)h->u2, (const float *)h->N1xz, (const float *)h->N3xz,
                       (const float *)h->N2xz, (const float *)h->uvf, (const float *)h->wvf, (const float *)h->vvc,
                       (const double *)h->p, (const float2 *)h->duib, h->ib ? h->d_ibslot_u : nullptr, h->ib ? h->d_ibslot_v : nullptr,
                       g, h->sc, kRK, h->a3s));
  }
  if (fork) CK(cudaEventRecord(h->ev_join, h->st2));
  if (h->prec == LH_PREC_FP64) {
    KL("k_helm_uw", k_helm_uw<T><<<nbu, h->tb_uw, 0, h->st>>>(h->u1, h->u3, (double2 *)h->Nu1, (double2 *)h->Nu3,
                                                           (const V *)h->N1xz, (const V *)h->N3xz, (const V *)h->uvf,
                                                           (const V *)h->wvf, h->p, h->a3s, g, h->sc, kRK,
                                                           h->ib ? h->d_ibslot_u : nullptr, (const double2 *)h->duib));
  } else {
    const int nb2u = (2 * g.nvc + h->tb_uw - 1) / h->tb_uw;
    const size_t sm = staged_smem(g.nu, h->pf_uw, h->tb_uw);
    const dim3 gr(nb2u, 2);
    double *U1 = (double *)h->u1, *U3 = (double *)h->u3;
    float *N1 = (float *)h->Nu1, *N3 = (float *)h->Nu3;
    const float *X1 = (const float *)h->N1xz, *X3 = (const float *)h->N3xz, *F1 = (const float *)h->uvf,
                *F3 = (const float *)h->wvf;
    const int *ibu = h->ib ? h->d_ibslot_u : nullptr;
    float2 *YS = (float2 *)h->ysf;
    switch (h->pf_uw) {
      case 0: KL("k_helm_uw", k_helm_u_mx2<<<gr, h->tb_uw, 0, h->st>>>(U1, U3, N1, N3, X1, X3, F1, F3, h->p, YS, g, h->sc, kRK, ibu, (const float2 *)h->duib)); break;
      case 2: KL("k_helm_uw", k_helm_u_mx3<2><<<gr, h->tb_uw, sm, h->st>>>(U1, U3, N1, N3, X1, X3, F1, F3, h->p, YS, g, h->sc, kRK, ibu, (const float2 *)h->duib)); break;
      case 8: KL("k_helm_uw", k_helm_u_mx3<8><<<gr, h->tb_uw, sm, h->st>>>(U1, U3, N1, N3, X1, X3, F1, F3, h->p, YS, g, h->sc, kRK, ibu, (const float2 *)h->duib)); break;
      default: KL("k_helm_uw", k_helm_u_mx3<4><<<gr, h->tb_uw, sm, h->st>>>(U1, U3, N1, N3, X1, X3, F1, F3, h->p, YS, g, h->sc, kRK, ibu, (const float2 *)h->duib)); break;
    }
  }
  if (fork) CK(cudaStreamWaitEvent(h->st, h->ev_join, 0));
  if ((rc = meanflow(h, kRK))) return rc;
  const int need_div = (kRK == 3) ? 1 : 0;
  if (need_div) KL("k_reset_err", k_reset_err<<<1, 32, 0, h->st>>>(h->sc));
  const int nbp2 = (2 * g.nvc + h->tb_p - 1) / h->tb_p;
  {  // the pressure step with its y-columns staged pf_p levels ahead (k_press3)
    const size_t sm = press_smem(g, h->pf_p, h->tb_p);
    double *U1 = (double *)h->u1, *U2 = (double *)h->u2, *U3 = (double *)h->u3, *P = (double *)h->p;
    double *PS = (double *)h->psi;
    switch (h->pf_p) {
      case 0: KL("k_press", k_press2<<<nbp2, h->tb_p, sizeof(double) * ((size_t)g.nu + g.nv), h->st>>>(U1, U2, U3, P, PS, h->dg1, h->dg2, h->dg3, g, h->sc, kRK, need_div)); break;
      case 2: KL("k_press", k_press3<2><<<nbp2, h->tb_p, sm, h->st>>>(U1, U2, U3, P, PS, h->dg1, h->dg2, h->dg3, g, h->sc, kRK, need_div)); break;
      case 8: KL("k_press", k_press3<8><<<nbp2, h->tb_p, sm, h->st>>>(U1, U2, U3, P, PS, h->dg1, h->dg2, h->dg3, g, h->sc, kRK, need_div)); break;
      default: KL("k_press", k_press3<4><<<nbp2, h->tb_p, sm, h->st>>>(U1, U2, U3, P, PS, h->dg1, h->dg2, h->dg3, g, h->sc, kRK, need_div)); break;
    }
  }
  if (need_div) KL("k_err_from_bits", k_err_from_bits<<<1, 32, 0, h->st>>>(h->sc));
  return LH_OK;
}

static int substep_launches(lh_handle *h, int kRK) {
  return (h->prec == LH_PREC_FP64) ? substep_launches_t<double>(h, kRK) : substep_launches_t<float>(h, kRK);
}

extern "C" int lh_substep(lh_handle *h, int kRK) {
  if (!h) return LH_EINVAL;
  if (kRK < 1 || kRK > 3) return fail(h, LH_EINVAL, "kRK must be 1, 2 or 3");
  return substep_launches(h, kRK);
}

static int step_launches(lh_handle *h) {
  int rc;
  for (int k = 1; k <= 3; ++k)
    if ((rc = substep_launches(h, k))) return rc;
  if (h->g.flag_ctpress == 1) { KL("k_flowrate", k_flowrate<<<1, 32, 0, h->st>>>(h->u1, h->g, h->sc, 0)); }
  KL("k_step_end", k_step_end<<<1, 32, 0, h->st>>>(h->sc));
  return LH_OK;
}

extern "C" int lh_step(lh_handle *h) {
  if (!h) return LH_EINVAL;
  if (!h->graph_ready) {
    // capture once; every later step replays the graph
    long long before = h->launches;
    CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
    int rc = step_launches(h);
    cudaGraph_t gr;
    cudaError_t e = cudaStreamEndCapture(h->st, &gr);
    if (rc) return rc;
    if (e != cudaSuccess) return fail(h, LH_ECUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&h->gexec, gr, 0);
    if (e != cudaSuccess) { cudaGraphDestroy(gr); return fail(h, LH_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(e)); }
    h->graph = gr;
    h->graph_ready = true;
    h->launches = before;  // the captured launches run below
    h->graph_nodes_per_step = 0;
    size_t n = 0;
    if (cudaGraphGetNodes(gr, nullptr, &n) == cudaSuccess) h->graph_nodes_per_step = (long long)n;
  }
  CK(cudaGraphLaunch(h->gexec, h->st));
  h->launches += h->graph_nodes_per_step;
  return LH_OK;
}

extern "C" int lh_profile_steps(lh_handle *h, int nsteps, lh_kernel_time *out, int nmax, int *nout) {
  if (!h || nsteps <= 0 || !out || nmax <= 0 || !nout) return LH_EINVAL;
  CK(cudaStreamSynchronize(h->st));
  h->prof = true;
  h->prof_ev.clear();
  int rc = LH_OK;
  for (int k = 0; k < nsteps && rc == LH_OK; ++k) rc = step_launches(h);
  h->prof = false;
  cudaError_t e = cudaStreamSynchronize(h->st);
  int n = 0;
  for (auto &pe : h->prof_ev) {
    float ms = 0.f;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, pe.second.first, pe.second.second);
    cudaEventDestroy(pe.second.first);
    cudaEventDestroy(pe.second.second);
    int i = 0;
    for (; i < n; ++i)
      if (strncmp(out[i].name, pe.first, sizeof(out[i].name)) == 0) break;
    if (i == n) {
      if (n >= nmax) continue;
      memset(&out[n], 0, sizeof(out[n]));
      strncpy(out[n].name, pe.first, sizeof(out[n].name) - 1);
      ++n;
    }
    out[i].launches += 1;
    out[i].total_ms += ms;
  }
  h->prof_ev.clear();
  *nout = n;
  if (rc != LH_OK) return rc;
  if (e != cudaSuccess) return fail(h, LH_ECUDA, cudaGetErrorString(e));
  return LH_OK;
}

// statistics of the current state: the inverse transforms of the nonlinear stage, then
// the sums of stats.f90 (k_xstats), per plane class
template <typename T, int N>
static int launch_xstats(lh_handle *h, const Geo &g, int nslots, const void *twx) {
  typedef typename C2<T>::t V;
  constexpr int PB = pb_xpass<V>(N);
  dim3 grid((g.G2 / 2 + PB - 1) / PB, nslots);
  KL("k_xstats", k_xstats<T, N><<<grid, NTHR_H, 8 * (size_t)PB * N * sizeof(V), h->st>>>(
                     (const V *)h->A, g, (const V *)twx, h->st_pl, h->st_cd, h->st_ncl, h->st_dnx, h->st_dnz,
                     h->st_ntx));
  return LH_OK;
}
template <typename T>
static int stats_launches(lh_handle *h) {
  for (int vi = 0; vi < h->nviews; ++vi) {
    const Geo &g = h->gv[vi];
    const int nslots = g.nuI + g.nvI;
    if (nslots == 0) continue;
    int rc = LH_EINVAL;
    LH_DISPATCH(g.G2, rc = launch_zinv<T, N>(h, g, nslots, h->twv[vi][1]));
    if (rc) return rc;
    rc = LH_EINVAL;
    LH_DISPATCH(g.G1, rc = launch_xstats<T, N>(h, g, nslots, h->twv[vi][0]));
    if (rc) return rc;
  }
  return LH_OK;
}

// band 2's level counts of U, V, W, UV, P (jlim(1:2, grid, midband))
static void spectra_levels(const lh_handle *h, int nl[5]) {
  const int(*bq)[6] = h->g.bq;
  nl[0] = nl[2] = nl[3] = bq[1][1] - bq[1][0] + 1;
  nl[1] = bq[1][3] - bq[1][2] + 1;
  nl[4] = bq[1][5] - bq[1][4] + 1;
}
static size_t spectra_size(const lh_handle *h) {
  int nl[5];
  spectra_levels(h, nl);
  return (size_t)(nl[0] + nl[1] + nl[2] + nl[3] + nl[4]) * h->nlong;
}
// the accumulators of spectra and slip statistics, zeroed, on first use
static int spectral_stats_buffers(lh_handle *h) {
  if (h->d_sp && h->d_slip && h->d_slip_inst) return LH_OK;
  const size_t nsp = spectra_size(h), nsl = 8 * (size_t)h->g.ncolF;
  // each buffer on its own, allocated into a local and published only once it is zeroed:
  // a failed allocation or memset leaves the member null, and the next call retries it
  if (!h->d_sp) {
    double *d = nullptr;
    CK(cudaMalloc(&d, sizeof(double) * nsp));
    const cudaError_t e = cudaMemsetAsync(d, 0, sizeof(double) * nsp, h->st);
    if (e != cudaSuccess) { cudaFree(d); return fail(h, LH_ECUDA, std::string("zeroing the spectra: ") + cudaGetErrorString(e)); }
    h->d_sp = d;
  }
  if (!h->d_slip) {
    double2 *d = nullptr;
    CK(cudaMalloc(&d, sizeof(double2) * nsl));
    const cudaError_t e = cudaMemsetAsync(d, 0, sizeof(double2) * nsl, h->st);
    if (e != cudaSuccess) { cudaFree(d); return fail(h, LH_ECUDA, std::string("zeroing the slip sums: ") + cudaGetErrorString(e)); }
    h->d_slip = d;
  }
  if (!h->d_slip_inst) CK(cudaMalloc(&h->d_slip_inst, sizeof(double2) * nsl));
  return LH_OK;
}
// the wall faces jlim(1, vgrid, 2), jlim(2, vgrid, 2) as v array indices
static void slip_faces(const lh_handle *h, int &qb, int &qt) { qb = h->g.bq[1][2]; qt = h->g.bq[1][3]; }

// the planes of the tile-conditioned P and omega_x sums, and a scratch chunk for their
// spectral and physical forms (first use): p levels of the wall bands (N(4,0)+1 .. N(4,1)-1,
// j1 = j - N(4,0) - 1; N(4,2)+2 .. N(4,3), j1 = N(4,3) - j) and the v levels of omega_x
// (N(3,0) .. N(3,1), j1 = j - N(3,0); N(3,2)+1 .. N(3,3)+1, j1 = N(3,3) + 1 - j)
static int cond_planes(lh_handle *h) {
  if (h->d_cond_list) return LH_OK;
  const Geo &g = h->g;
  const int *N3 = g.N3, *N4 = g.N4;
  std::vector<int4> L;
  for (int j = N4[0] + 1; j <= N4[3]; ++j) {
    if (j <= N4[1] - 1) L.push_back(make_int4(0, j + g.dny - 1, j - N4[0] - 1, 0));
    else if (j >= N4[2] + 2) L.push_back(make_int4(0, j + g.dny - 1, N4[3] - j, 0));
  }
  for (int j = N3[0]; j <= N3[3] + 1; ++j) {
    if (j <= N3[1]) L.push_back(make_int4(1, j + g.dny, j - N3[0], 0));
    else if (j > N3[2]) L.push_back(make_int4(1, j + g.dny, N3[3] + 1 - j, 0));
  }
  for (const int4 &d : L)
    if (d.z < 0 || d.z > h->st_ncl || d.y < 0 || d.y >= (d.x ? g.nv : g.np))
      return fail(h, LH_EINVAL, "conditioned statistics: plane outside the grid");
  const size_t per = sizeof(double2) * (size_t)g.G2 * g.N1h;  // z-transformed plane in the A scratch
  const int chunk = (int)std::min<size_t>({(size_t)32, L.size(), h->Abytes / per});
  if (chunk < 1) return fail(h, LH_EINVAL, "conditioned statistics: scratch too small");
  void *scr = nullptr;
  int4 *dl = nullptr;
  CK(cudaMalloc(&scr, (size_t)chunk * (sizeof(double2) * g.ncolF + sizeof(double) * (size_t)g.G1 * g.G2)));
  cudaError_t e = cudaMalloc(&dl, sizeof(int4) * L.size());
  if (e == cudaSuccess) e = cudaMemcpy(dl, L.data(), sizeof(int4) * L.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(scr);
    if (dl) cudaFree(dl);
    return fail(h, LH_ECUDA, std::string("conditioned statistics: ") + cudaGetErrorString(e));
  }
  h->d_cond_scr = scr;
  h->cond_chunk = chunk;
  h->n_cond = (int)L.size();
  h->d_cond_list = dl;
  return LH_OK;
}

// pressure plane sums (every p level, Parseval) and the tile-conditioned P and omega_x sums
// (wall-band planes transformed to the dealiased grid in FP64, then summed per tile position)
static int pressure_wx_stats(lh_handle *h, int nhc, int n2c) {
  const Geo &g = h->g;
  const double Gf = (double)g.G1 * g.G2;
  const double Gc = h->nviews > 1 ? (double)h->gv[1].G1 * h->gv[1].G2 : Gf;
  KL("k_p_stats", k_p_stats<<<g.np, LH_STAT_THREADS, 0, h->st>>>(h->p, g, nhc, n2c, Gf, Gc, h->st_pp));
  if (!h->st_dnx) return LH_OK;
  int rc = cond_planes(h);
  if (rc) return rc;
  double2 *spec = (double2 *)h->d_cond_scr;
  double *phys = (double *)(spec + (size_t)h->cond_chunk * g.ncolF);
  const int cells = h->st_dnx * h->st_dnz;
  for (int b0 = 0; b0 < h->n_cond; b0 += h->cond_chunk) {
    const int nb = std::min(h->cond_chunk, h->n_cond - b0);
    KL("k_cond_spec", k_cond_spec<<<dim3((g.ncolF + LH_STAT_THREADS - 1) / LH_STAT_THREADS, nb), LH_STAT_THREADS, 0,
                                     h->st>>>(h->u2, h->u3, h->p, g, h->d_cond_list + b0, spec));
    if ((rc = spec_to_phys<double>(h, spec, phys, nb, h->A, fp64_tw(h, true), fp64_tw(h, false)))) return rc;
    KL("k_cond_phys", k_cond_phys<<<dim3((cells + LH_STAT_THREADS - 1) / LH_STAT_THREADS, nb), LH_STAT_THREADS, 0,
                                     h->st>>>(phys, h->d_cond_list + b0, g.G1, g.G2, h->st_dnx, h->st_dnz,
                                              h->st_ncl + 1, h->st_cd4));
  }
  return LH_OK;
}

// stats() + spectra() + sl_stats() of the current state (FOU3D.f90:127-130, 298-373)
extern "C" int lh_stats_accumulate(lh_handle *h) {
  if (!h) return LH_EINVAL;
  int rc = (h->prec == LH_PREC_FP64) ? stats_launches<double>(h) : stats_launches<float>(h);
  if (rc) return rc;
  if ((rc = spectral_stats_buffers(h))) return rc;
  const Geo &g = h->g;
  const int nhc = h->nviews > 1 ? h->gv[1].N1h : g.N1hF, n2c = h->nviews > 1 ? h->gv[1].N2 : g.N2F;
  KL("k_wx_stats", k_wx_stats<<<g.nv, LH_STAT_THREADS, 0, h->st>>>(h->u2, h->u3, g, nhc, n2c, h->st_pl));
  if ((rc = pressure_wx_stats(h, nhc, n2c))) return rc;
  int nl[5];
  spectra_levels(h, nl);
  const size_t ne = (size_t)nl[0] * h->nlong;
  KL("k_spectra", k_spectra<<<(unsigned)((ne + LH_STAT_THREADS - 1) / LH_STAT_THREADS), LH_STAT_THREADS, 0, h->st>>>(
                      h->u1, h->u2, h->u3, h->p, g, h->d_bcols, h->nlong, h->cfg.gw_interp[1][0],
                      h->cfg.gw_interp[1][1], h->d_sp));
  int qb, qt;
  slip_faces(h, qb, qt);
  KL("k_slip", k_slip<<<(g.ncolF + LH_STAT_THREADS - 1) / LH_STAT_THREADS, LH_STAT_THREADS, 0, h->st>>>(
                   h->u1, h->u3, g, qb, qt, h->d_slip, 1));
  h->istat += 1;
  return LH_OK;
}

extern "C" int lh_stats_reset(lh_handle *h) {
  if (!h) return LH_EINVAL;
  const size_t ncd = 9 * (size_t)h->st_ncl * (h->st_dnx ? (size_t)h->st_dnx * h->st_dnz : 1);
  CK(cudaMemsetAsync(h->st_pl, 0, sizeof(double) * 11 * (size_t)h->g.nu, h->st));
  CK(cudaMemsetAsync(h->st_cd, 0, sizeof(double) * ncd, h->st));
  CK(cudaMemsetAsync(h->st_pp, 0, sizeof(double) * 2 * (size_t)h->g.np, h->st));
  CK(cudaMemsetAsync(h->st_cd4, 0, sizeof(double) * 4 * (size_t)(h->st_ncl + 1) * (h->st_dnx ? (size_t)h->st_dnx * h->st_dnz : 1), h->st));
  if (h->d_sp) CK(cudaMemsetAsync(h->d_sp, 0, sizeof(double) * spectra_size(h), h->st));
  if (h->d_slip) CK(cudaMemsetAsync(h->d_slip, 0, sizeof(double2) * 8 * (size_t)h->g.ncolF, h->st));
  h->istat = 0;
  return LH_OK;
}

extern "C" int lh_stats_dims(lh_handle *h, int *ncl, int *dnx, int *dnz) {
  if (!h) return LH_EINVAL;
  if (ncl) *ncl = h->st_ncl;
  if (dnx) *dnx = h->st_dnx;
  if (dnz) *dnz = h->st_dnz;
  return LH_OK;
}

extern "C" int lh_stats_get(lh_handle *h, double *plane, double *cond, int64_t *istat) {
  if (!h) return LH_EINVAL;
  if (plane) CK(cudaMemcpyAsync(plane, h->st_pl, sizeof(double) * 11 * (size_t)h->g.nu, cudaMemcpyDeviceToHost, h->st));
  if (cond && h->st_dnx)
    CK(cudaMemcpyAsync(cond, h->st_cd, sizeof(double) * 9 * (size_t)h->st_ncl * h->st_dnx * h->st_dnz,
                       cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  if (istat) *istat = h->istat;
  return LH_OK;
}

extern "C" int lh_stats_get_pw(lh_handle *h, double *pplane, double *cond4) {
  if (!h) return LH_EINVAL;
  if (pplane) CK(cudaMemcpyAsync(pplane, h->st_pp, sizeof(double) * 2 * (size_t)h->g.np, cudaMemcpyDeviceToHost, h->st));
  if (cond4 && h->st_dnx)
    CK(cudaMemcpyAsync(cond4, h->st_cd4, sizeof(double) * 4 * (size_t)(h->st_ncl + 1) * h->st_dnx * h->st_dnz,
                       cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  return LH_OK;
}

extern "C" int lh_spectra_dims(lh_handle *h, int *nlev, int *nlong) {
  if (!h) return LH_EINVAL;
  if (nlev) spectra_levels(h, nlev);
  if (nlong) *nlong = h->nlong;
  return LH_OK;
}

extern "C" int lh_spectra_get(lh_handle *h, double *sU, double *sV, double *sW, double *sUV, double *sP) {
  if (!h) return LH_EINVAL;
  int nl[5];
  spectra_levels(h, nl);
  double *dst[5] = {sU, sV, sW, sUV, sP};
  const size_t nlg = h->nlong;
  std::vector<double> buf;
  size_t off = 0;
  for (int q = 0; q < 5; ++q) {
    const size_t n = (size_t)nl[q] * nlg;
    if (dst[q]) {
      if (!h->d_sp) {
        memset(dst[q], 0, sizeof(double) * n);
      } else {
        buf.resize(n);
        CK(cudaMemcpyAsync(buf.data(), h->d_sp + off, sizeof(double) * n, cudaMemcpyDeviceToHost, h->st));
        CK(cudaStreamSynchronize(h->st));
        // device [level][column] -> sp(level, column), level fastest
        for (size_t k = 0; k < nlg; ++k)
          for (int l = 0; l < nl[q]; ++l) dst[q][k * nl[q] + l] = buf[(size_t)l * nlg + k];
      }
    }
    off += n;
  }
  return LH_OK;
}

extern "C" int lh_slip_get(lh_handle *h, double *acc) {
  if (!h) return LH_EINVAL;
  const size_t n = 8 * (size_t)h->g.ncolF;
  if (!acc) return LH_OK;
  if (!h->d_slip) { memset(acc, 0, sizeof(double2) * n); return LH_OK; }
  CK(cudaMemcpyAsync(acc, h->d_slip, sizeof(double2) * n, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  return LH_OK;
}

extern "C" int lh_slip_planes(lh_handle *h, double *out) {
  if (!h || !out) return LH_EINVAL;
  int rc = spectral_stats_buffers(h);
  if (rc) return rc;
  int qb, qt;
  slip_faces(h, qb, qt);
  KL("k_slip", k_slip<<<(h->g.ncolF + LH_STAT_THREADS - 1) / LH_STAT_THREADS, LH_STAT_THREADS, 0, h->st>>>(
                   h->u1, h->u3, h->g, qb, qt, h->d_slip_inst, 0));
  CK(cudaMemcpyAsync(out, h->d_slip_inst, sizeof(double2) * 8 * (size_t)h->g.ncolF, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  return LH_OK;
}

extern "C" int lh_synchronize(lh_handle *h) {
  if (!h) return LH_EINVAL;
  CK(cudaStreamSynchronize(h->st));
  if (h->st_in) CK(cudaStreamSynchronize(h->st_in));
  if (h->st_out) CK(cudaStreamSynchronize(h->st_out));
  int status = 0;
  CK(cudaMemcpy(&status, &h->sc->status, sizeof(int), cudaMemcpyDeviceToHost));
  if (status == LH_ENONFINITE) return fail(h, LH_ENONFINITE, "non-finite state (divergence or dt)");
  return LH_OK;
}

extern "C" int lh_four_to_phys(lh_handle *h, const void *spec, void *phys, int nplanes) {
  if (!h || !spec || !phys || nplanes <= 0) return LH_EINVAL;
  const size_t need = sizeof(double2) * (size_t)nplanes * h->g.G2 * h->g.N1h;
  if (need > h->Abytes) return fail(h, LH_EINVAL, "too many planes for the scratch buffer");
  return spec_to_phys<double>(h, (const double2 *)spec, (double *)phys, nplanes, h->A, fp64_tw(h, true), fp64_tw(h, false));
}

extern "C" int lh_phys_to_four(lh_handle *h, const void *phys, void *spec, int nplanes) {
  if (!h || !spec || !phys || nplanes <= 0) return LH_EINVAL;
  const size_t need = sizeof(double2) * (size_t)nplanes * h->g.G2 * h->g.N1h;
  if (need > h->Bbytes) return fail(h, LH_EINVAL, "too many planes for the scratch buffer");
  return phys_to_spec<double>(h, (const double *)phys, (double2 *)spec, nplanes, h->B, fp64_tw(h, true), fp64_tw(h, false));
}

// ---------------------------------------------------------------------------
// Autotuner: threads per block of the one-thread-per-column kernels. Each
// candidate runs one eager step with CUDA events around every launch on a copy of
// the state; the state and the scalars are restored afterwards.
// ---------------------------------------------------------------------------
extern "C" int lh_autotune(lh_handle *h) {
  if (!h) return LH_EINVAL;
  const Geo &g = h->g;
  const size_t nc = g.ncol, cz = sizeof(double2);
  const size_t bu = cz * g.nu * nc, bv = cz * g.nv * nc, bp = cz * g.np * nc, bn = h->vsz * g.nu * nc,
               bnv = h->vsz * g.nv * nc;
  void *save = nullptr;
  const size_t total = 2 * bu + bv + bp + 2 * bn + bnv + sizeof(DevScalars);
  CK(cudaStreamSynchronize(h->st));
  CK(cudaMalloc(&save, total));
  char *sp = (char *)save;
  void *src[] = {h->u1, h->u3, h->u2, h->p, h->Nu1, h->Nu3, h->Nu2, h->sc};
  const size_t sz[] = {bu, bu, bv, bp, bn, bn, bnv, sizeof(DevScalars)};
  auto copy_all = [&](bool to_save) -> cudaError_t {
    size_t off = 0;
    for (int i = 0; i < 8; ++i) {
      cudaError_t e = to_save ? cudaMemcpyAsync(sp + off, src[i], sz[i], cudaMemcpyDeviceToDevice, h->st)
                              : cudaMemcpyAsync(src[i], sp + off, sz[i], cudaMemcpyDeviceToDevice, h->st);
      if (e != cudaSuccess) return e;
      off += sz[i];
    }
    return cudaStreamSynchronize(h->st);
  };
  cudaError_t e = copy_all(true);
  if (e != cudaSuccess) { cudaFree(save); return fail(h, LH_ECUDA, cudaGetErrorString(e)); }
  // trials: every block size with every staging depth (0: the register-prefetch kernels); each
  // solve kernel keeps the configuration of its fastest trial. The FP64 form's Helmholtz kernels
  // depend on the block size only.
  const int cand[] = {64, 128, 256}, cpf[] = {0, 2, 4, 8};
  double best[3] = {1e30, 1e30, 1e30};
  int pick[3] = {h->tb_uw, h->tb_v, h->tb_p}, pickpf[3] = {h->pf_uw, h->pf_v, h->pf_p};
  const char *names[3] = {"k_helm_uw", "k_helm_v", "k_press"};
  lh_kernel_time kt[64];
  int rc = LH_OK;
  int optin = 0;
  if (smem_optin(&optin)) optin = 49152;
  for (int ti = 0; ti < 12 && rc == LH_OK; ++ti) {
    const int tb = cand[ti % 3], pf = cpf[ti / 3];
    if (press_smem(g, pf, tb) > (size_t)optin || staged_smem(g.nu, pf, tb) > (size_t)optin) continue;
    h->tb_uw = h->tb_v = h->tb_p = tb;
    h->pf_uw = h->pf_v = h->pf_p = pf;
    int n = 0;
    rc = lh_profile_steps(h, 1, kt, 64, &n);
    for (int k = 0; k < 3 && rc == LH_OK; ++k)
      for (int i = 0; i < n; ++i)
        if (strncmp(kt[i].name, names[k], 32) == 0 && kt[i].total_ms < best[k]) {
          best[k] = kt[i].total_ms;
          pick[k] = tb;
          pickpf[k] = pf;
        }
    if (copy_all(false) != cudaSuccess) rc = fail(h, LH_ECUDA, "state restore failed");
  }
  cudaFree(save);
  h->tb_uw = pick[0]; h->tb_v = pick[1]; h->tb_p = pick[2];
  h->pf_uw = pickpf[0]; h->pf_v = pickpf[1]; h->pf_p = pickpf[2];
  if (h->graph_ready) {  // recapture with the chosen configuration
    cudaGraphExecDestroy(h->gexec);
    cudaGraphDestroy(h->graph);
    h->graph_ready = false;
  }
  return rc;
}

extern "C" int lh_get_tuning(lh_handle *h, int32_t *cfg) {
  if (!h || !cfg) return LH_EINVAL;
  cfg[0] = h->tb_uw; cfg[1] = h->tb_v; cfg[2] = h->tb_p;
  cfg[3] = h->pf_uw; cfg[4] = h->pf_v; cfg[5] = h->pf_p;
  return LH_OK;
}

// ---------------------------------------------------------------------------
// Batches: one RK3 step of many independent channels (any sizes) as one CUDA
// graph; every channel is a branch on its own stream.
// ---------------------------------------------------------------------------
struct lh_batch {
  std::vector<lh_handle *> hs;
  cudaStream_t root = nullptr;
  cudaEvent_t ev0 = nullptr;
  std::vector<cudaEvent_t> evs;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  long long nodes = 0;
  std::string err;
};
extern "C" int lh_batch_destroy(lh_batch *b);

// failure of a batch call: the message goes to lh_last_error(NULL)
static int batch_fail(lh_batch *b, int code, const std::string &msg) {
  t_last_err = msg;
  if (b) b->err = msg;
  return code;
}

extern "C" int lh_batch_create(lh_handle *const *handles, int n, lh_batch **out) {
  if (!handles || n <= 0 || !out) return batch_fail(nullptr, LH_EINVAL, "lh_batch_create: no handles");
  *out = nullptr;
  lh_batch *b = new lh_batch();
  b->hs.assign(handles, handles + n);
  for (lh_handle *h : b->hs)
    if (!h) { delete b; return batch_fail(nullptr, LH_EINVAL, "lh_batch_create: a null handle"); }
  cudaError_t e = cudaStreamCreateWithFlags(&b->root, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev0, cudaEventDisableTiming);
  b->evs.resize(n);
  for (int i = 0; i < n && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&b->evs[i], cudaEventDisableTiming);
  if (e != cudaSuccess) {
    lh_batch_destroy(b);
    return batch_fail(nullptr, LH_ECUDA, std::string("lh_batch_create: streams/events: ") + cudaGetErrorString(e));
  }
  for (int i = 0; i < n; ++i)
    if ((e = cudaStreamSynchronize(b->hs[i]->st)) != cudaSuccess) {
      lh_batch_destroy(b);
      return batch_fail(nullptr, LH_ECUDA, "lh_batch_create: channel " + std::to_string(i) + " has a failed launch: " +
                                               cudaGetErrorString(e));
    }
  if ((e = cudaStreamBeginCapture(b->root, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) {
    lh_batch_destroy(b);
    return batch_fail(nullptr, LH_ECUDA, std::string("lh_batch_create: begin capture: ") + cudaGetErrorString(e));
  }
  cudaEventRecord(b->ev0, b->root);
  int rc = LH_OK;
  std::string why;
  for (int i = 0; i < n && rc == LH_OK; ++i) {
    lh_handle *h = b->hs[i];
    cudaStreamWaitEvent(h->st, b->ev0, 0);
    long long before = h->launches;
    rc = step_launches(h);
    h->launches = before;
    if (rc != LH_OK) why = "channel " + std::to_string(i) + ": " + h->err;
    cudaEventRecord(b->evs[i], h->st);
    cudaStreamWaitEvent(b->root, b->evs[i], 0);
  }
  cudaGraph_t gr = nullptr;
  e = cudaStreamEndCapture(b->root, &gr);
  if (rc != LH_OK || e != cudaSuccess) {
    if (gr) cudaGraphDestroy(gr);
    lh_batch_destroy(b);
    return rc != LH_OK ? batch_fail(nullptr, rc, "lh_batch_create: " + why)
                       : batch_fail(nullptr, LH_ECUDA, std::string("lh_batch_create: end capture: ") + cudaGetErrorString(e));
  }
  e = cudaGraphInstantiate(&b->gexec, gr, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(gr);
    lh_batch_destroy(b);
    return batch_fail(nullptr, LH_ECUDA, std::string("lh_batch_create: graph instantiate: ") + cudaGetErrorString(e));
  }
  b->graph = gr;
  size_t nn = 0;
  cudaGraphGetNodes(gr, nullptr, &nn);
  b->nodes = (long long)nn;
  *out = b;
  return LH_OK;
}

extern "C" int lh_batch_step(lh_batch *b) {
  if (!b) return LH_EINVAL;
  if (cudaGraphLaunch(b->gexec, b->root) != cudaSuccess) return LH_ECUDA;
  for (lh_handle *h : b->hs) h->launches += b->nodes / (long long)b->hs.size();
  return LH_OK;
}

extern "C" int lh_batch_synchronize(lh_batch *b) {
  if (!b) return LH_EINVAL;
  if (cudaStreamSynchronize(b->root) != cudaSuccess) return LH_ECUDA;
  int worst = LH_OK;
  for (lh_handle *h : b->hs) {
    int rc = lh_synchronize(h);
    if (rc != LH_OK) worst = rc;
  }
  return worst;
}

extern "C" int lh_batch_destroy(lh_batch *b) {
  if (!b) return LH_EINVAL;
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (cudaEvent_t e : b->evs) if (e) cudaEventDestroy(e);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->root) cudaStreamDestroy(b->root);
  delete b;
  return LH_OK;
}

extern "C" void *lh_batch_stream(lh_batch *b) { return b ? (void *)b->root : nullptr; }

// ===========================================================================
// lh_four_to_phys_noalloc: the four_to_phys transform without a handle and
// without any device allocation.
//
// Who needs it: hosts that own every byte of device memory themselves (a
// Fortran solver that sizes HBM once at start-up and forbids later allocation,
// or an application running at the edge of the device's capacity) cannot call
// cudaMalloc, and so cannot create a handle (lh_create allocates the whole
// channel state). This entry point takes only the caller's input and output
// buffers; its working memory is the fixed array below, which every GPU that
// loads the library holds until the process exits.
// ===========================================================================
static __device__ __align__(256) unsigned char lh_noalloc_scratch[LH_NOALLOC_SCRATCH_BYTES];

// exp(-2 pi i e / n) for the two transform lengths, written by every call
__global__ void k_noalloc_twiddles(double2 *twx, int n1, double2 *twz, int n2) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n1) { double s, c; sincospi(-2.0 * (double)e / (double)n1, &s, &c); twx[e] = make_double2(c, s); }
  if (e < n2) { double s, c; sincospi(-2.0 * (double)e / (double)n2, &s, &c); twz[e] = make_double2(c, s); }
}

namespace {
const int LH_NOALLOC_MAX_DEVICES = 256;
// per device: the scratch array's device address, published by the set-up under the lock
std::mutex g_noalloc_mu;
std::atomic<unsigned char *> g_noalloc_ptr[LH_NOALLOC_MAX_DEVICES];

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// the shared-memory limit both kernels need at every supported length (the largest
// request, k_xinv_phys at Ngal1 = 1152 in FP64, is above the default 48 KB)
int noalloc_smem_limit(int dev) {
  int optin = 0;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) optin = 49152;
  return optin;
}

// true when the set-up of this device is still in force: a cudaDeviceReset reloads the
// module and clears the kernels' shared-memory attribute, which is detected here
bool noalloc_attr_set(int lim) {
  cudaFuncAttributes fa;
  if (cudaFuncGetAttributes(&fa, (const void *)k_xinv_phys<double, 24>) != cudaSuccess) return false;
  return fa.maxDynamicSharedSizeBytes >= lim;
}

// Set-up, once per device (again after a device reset), with that device current: the
// device address of the scratch array (a host-side name of a __device__ array is not a
// device address) and the shared-memory limit of the two kernels. Host threads making
// their first call at the same time are serialised by the lock; later calls read the
// published address without it.
int noalloc_setup(int dev, unsigned char **ptr, const char **err) {
  if (dev < 0 || dev >= LH_NOALLOC_MAX_DEVICES) { if (err) *err = "device index out of range"; return LH_EINVAL; }
  const int lim = noalloc_smem_limit(dev);
  unsigned char *cur = g_noalloc_ptr[dev].load(std::memory_order_acquire);
  if (cur && noalloc_attr_set(lim)) { *ptr = cur; return LH_OK; }
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  cur = g_noalloc_ptr[dev].load(std::memory_order_acquire);
  if (cur && noalloc_attr_set(lim)) { *ptr = cur; return LH_OK; }
  void *p = nullptr;
  if (cudaGetSymbolAddress(&p, lh_noalloc_scratch) != cudaSuccess || !p) {
    if (err) *err = "cudaGetSymbolAddress of the scratch array failed";
    return LH_ECUDA;
  }
  cudaError_t e = cudaSuccess;
#define LH_NOALLOC_ATTR(n_)                                                                                   \
  if (e == cudaSuccess) e = cudaFuncSetAttribute((const void *)k_spec_zinv<double, n_>,                      \
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, lim);          \
  if (e == cudaSuccess) e = cudaFuncSetAttribute((const void *)k_xinv_phys<double, n_>,                      \
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
  LH_FOR_SIZES(LH_NOALLOC_ATTR)
#undef LH_NOALLOC_ATTR
  if (e != cudaSuccess) {
    if (err) *err = "cudaFuncSetAttribute failed";
    return LH_ECUDA;
  }
  g_noalloc_ptr[dev].store((unsigned char *)p, std::memory_order_release);
  *ptr = (unsigned char *)p;
  return LH_OK;
}
}  // namespace

static size_t noalloc_max_planes(int N1, int N2, int Ngal1, int Ngal2) {
  if (N1 <= 0 || N2 <= 0 || Ngal1 <= 0 || Ngal2 <= 0) return 0;
  const size_t tw = align256(sizeof(double2) * (size_t)Ngal1) + align256(sizeof(double2) * (size_t)Ngal2);
  const size_t plane = sizeof(double2) * (size_t)Ngal2 * (size_t)(N1 / 2 + 1);
  if (tw >= LH_NOALLOC_SCRATCH_BYTES || plane == 0) return 0;
  return (LH_NOALLOC_SCRATCH_BYTES - tw) / plane;
}

extern "C" int lh_four_to_phys_noalloc(int N1, int N2, int Ngal1, int Ngal2, const void *spec, void *phys,
                                       int nplanes, void *stream, const char **err) {
  if (err) *err = "";
  if (N1 <= 0 || N2 <= 0 || (N1 & 1) || (N2 & 1) || Ngal1 <= N1 || Ngal2 <= N2 || !size_supported(Ngal1) ||
      !size_supported(Ngal2) || !spec || !phys || nplanes <= 0) {
    if (err) *err = "invalid sizes or pointers (N even, Ngal > N and one of 24 48 72 96 144 192 288 384 576 768 1152)";
    return LH_EINVAL;
  }
  if ((size_t)nplanes > noalloc_max_planes(N1, N2, Ngal1, Ngal2)) {
    if (err) *err = "too many planes for the fixed scratch of LH_NOALLOC_SCRATCH_BYTES; split the call";
    return LH_EINVAL;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) { if (err) *err = "cudaGetDevice failed"; return LH_ECUDA; }
  unsigned char *base = nullptr;
  int rc = noalloc_setup(dev, &base, err);
  if (rc != LH_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  (void)cudaGetLastError();  // an earlier, unrelated launch error is not this call's
  double2 *twx = (double2 *)base;
  double2 *twz = (double2 *)(base + align256(sizeof(double2) * (size_t)Ngal1));
  double2 *Ascr = (double2 *)(base + align256(sizeof(double2) * (size_t)Ngal1) + align256(sizeof(double2) * (size_t)Ngal2));
  Geo g;
  memset(&g, 0, sizeof(g));
  g.N1 = N1; g.N2 = N2; g.N1h = N1 / 2 + 1; g.G1 = Ngal1; g.G2 = Ngal2; g.ncol = g.N1h * N2;
  const int nt = Ngal1 > Ngal2 ? Ngal1 : Ngal2;
  k_noalloc_twiddles<<<(nt + 255) / 256, 256, 0, st>>>(twx, Ngal1, twz, Ngal2);
  {
    LH_DISPATCH(Ngal2, {
      constexpr int KB = kb_zinv<double2>(N);
      dim3 g1((g.N1h + KB - 1) / KB, nplanes);
      k_spec_zinv<double, N><<<g1, NTHR_H, 2 * (size_t)KB * N * sizeof(double2), st>>>((const double2 *)spec, Ascr, g, twz);
    });
    LH_DISPATCH(Ngal1, {
      constexpr int PB = 4 * pb_xpass<double2>(N);
      dim3 g2((g.G2 / 2 + PB - 1) / PB, nplanes);
      k_xinv_phys<double, N><<<g2, NTHR_H, 2 * (size_t)PB * N * sizeof(double2), st>>>(Ascr, (double *)phys, g, twx);
    });
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { if (err) *err = "kernel launch failed"; return LH_ECUDA; }
  return LH_OK;
}
