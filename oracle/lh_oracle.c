/*
 * lh_oracle.c — CPU FP64 restatement of the reference's RK3 substep.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the oracle the tests, smoke() and the
 * CPU-baseline leg of bench.py check the CUDA library against. It is never linked
 * into, loaded by, or called from the product path.
 *
 * It follows, loop by loop and in the same floating-point evaluation order:
 *   littleharsh.f90:174-217  substep sequence
 *   littleharsh.f90:237-272  divergence
 *   littleharsh.f90:274-340  laplacian_U / laplacian_V
 *   littleharsh.f90:435-509  flowrateIm / flowrateRe / flowrate_corr
 *   littleharsh.f90:529-562  meanflow_ctP / meanflow_ctU
 *   littleharsh.f90:581-633  solveP
 *   littleharsh.f90:635-788  RHS0_u1 / RHS0_u2 / RHS0_u3
 *   littleharsh.f90:791-907  solveU_W / solveV
 *   littleharsh.f90:956-1052 v_corr
 *   FOU3D.f90:41-425         nonlinear, with either form of the products:
 *   FOU3D.f90:2090-2251        ops_in_planes2 (pseudo-spectral products, 3/2 dealiasing)
 *   FOU3D.f90:1724-2088        ops_in_planes + nonlinInter (the as-run triad-list
 *                              convolution; lists as nonlinRead loads them, start.f90:2983-3069)
 *   FOU3D.f90:427-474        interp_u / interp_v
 *   FOU3D.f90:476-593        der_x / der_z
 *   FOU3D.f90:636-676        der_yu_h / der_yv_h
 *   FOU3D.f90:699-736        dtc_calc (dthetavi is never assigned in the reference, so the
 *                            wall-normal term is 1/(u2m*0) = +inf; reproduced)
 *   FOU3D.f90:738-764, 2253-2272 four_to_phys_u / phys_to_four_du
 *   FOU3D.f90:806-998        imm_bounds_u / imm_bounds_v (disabled in the reference: the call
 *                            is commented out at FOU3D.f90:413-423; restated here, switchable)
 *   tridLU_3D.f90:55-537     LUsolU_W, LUsolV, LUsolP, LUsol0, LU_build*, LU_dec*
 * The x/z transforms follow the mathematics of rft_buff.f:24-86 and cft_buff.f:1-65
 * (forward scaled by 1/n, Im of x-modes 0 and n/2 zeroed, inverse unscaled); the FFT
 * itself is written here from the DFT definition (mixed radix 2/3/4 Cooley-Tukey),
 * not taken from FFTPACK.
 *
 * Layout: every spectral field is plane-major, complex [level][kz][kx].
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "lh_oracle.h"

typedef double complex cplx;

/* ------------------------------------------------------------------------- */
/* FFT: recursive mixed-radix decimation in time, twiddles exp(-2 pi i e/n).  */
/* ------------------------------------------------------------------------- */
typedef struct {
  int n;
  int nfac;
  int fac[32];
  cplx *tw; /* [n] exp(-2 pi i e / n) */
} fftplan;

static int plan_init(fftplan *P, int n) {
  P->n = n;
  P->nfac = 0;
  int m = n;
  while (m > 1) {
    int f;
    if (m % 4 == 0) f = 4;
    else if (m % 2 == 0) f = 2;
    else if (m % 3 == 0) f = 3;
    else if (m % 5 == 0) f = 5;
    else f = m; /* generic prime */
    P->fac[P->nfac++] = f;
    m /= f;
  }
  P->tw = (cplx *)malloc(sizeof(cplx) * (size_t)n);
  if (!P->tw) return -1;
  for (int e = 0; e < n; ++e) {
    double a = -2.0 * M_PI * (double)e / (double)n;
    P->tw[e] = cos(a) + I * sin(a);
  }
  return 0;
}

static void plan_free(fftplan *P) { free(P->tw); P->tw = NULL; }

/* out[0..m*p) from in[] with stride `st`; `ts` = twiddle stride (n / current length). */
static void fft_rec(const fftplan *P, const cplx *in, cplx *out, int len, int st, int fi,
                    int sgn, cplx *scr) {
  if (len == 1) { out[0] = in[0]; return; }
  int p = P->fac[fi];
  int m = len / p;
  for (int r = 0; r < p; ++r) fft_rec(P, in + (size_t)r * st, out + (size_t)r * m, m, st * p, fi + 1, sgn, scr);
  int ts = P->n / len; /* W_len^e = tw[e*ts] */
  const cplx *tw = P->tw;
  for (int k = 0; k < m; ++k) {
    cplx t[64];
    for (int r = 0; r < p; ++r) {
      cplx w = tw[(size_t)r * k * ts % P->n];
      if (sgn > 0) w = conj(w);
      t[r] = (r == 0) ? out[k] : w * out[r * m + k];
    }
    if (p == 2) {
      out[k] = t[0] + t[1];
      out[k + m] = t[0] - t[1];
    } else if (p == 4) {
      cplx a0 = t[0] + t[2], a1 = t[0] - t[2], a2 = t[1] + t[3], a3 = t[1] - t[3];
      cplx rot = (sgn > 0) ? I * a3 : -I * a3; /* W_4^1 = -i (forward), +i (backward) */
      out[k] = a0 + a2;
      out[k + m] = a1 + rot;
      out[k + 2 * m] = a0 - a2;
      out[k + 3 * m] = a1 - rot;
    } else {
      for (int q = 0; q < p; ++q) {
        cplx s = 0;
        for (int r = 0; r < p; ++r) {
          cplx w = tw[(size_t)((r * q) % p) * (P->n / p)];
          if (sgn > 0) w = conj(w);
          s += w * t[r];
        }
        scr[q] = s;
      }
      for (int q = 0; q < p; ++q) out[k + q * m] = scr[q];
    }
  }
}

/* in-place complex transform of x[0..n) with element stride 1 */
/* Test hook: uniform noise of amplitude eps x (the line's largest modulus) added to every
 * transform output, standing in for the rounding of a transform less accurate than FP64
 * (orc_set_transform_noise; 0 = off). The noise is a hash of the value, so runs repeat. */
static double g_transform_noise = 0.0;
static inline double noise_unit(double v) {
  uint64_t b;
  memcpy(&b, &v, 8);
  b ^= b >> 33; b *= 0xff51afd7ed558ccdULL; b ^= b >> 33; b *= 0xc4ceb9fe1a85ec53ULL; b ^= b >> 33;
  return (double)(b >> 11) / 4503599627370496.0 - 1.0;  /* [-1, 1) */
}
int orc_set_transform_noise(double eps) { g_transform_noise = eps; return 0; }

static void fft_inplace(const fftplan *P, cplx *x, int sgn, cplx *tmp) {
  cplx scr[64];
  memcpy(tmp, x, sizeof(cplx) * (size_t)P->n);
  fft_rec(P, tmp, x, P->n, 1, 0, sgn, scr);
  if (g_transform_noise != 0.0) {
    double mx = 0.0;
    for (int i = 0; i < P->n; ++i) if (cabs(x[i]) > mx) mx = cabs(x[i]);
    const double a = g_transform_noise * mx;
    for (int i = 0; i < P->n; ++i) {
      const double re = creal(x[i]), im = cimag(x[i]);
      x[i] = (re + a * noise_unit(re)) + I * (im + a * noise_unit(im));
    }
  }
}

/* ------------------------------------------------------------------------- */
struct orc {
  lh_config c;
  /* owned copies of the config arrays */
  double *yu, *yv, *thu, *thv, *d2u, *d2v, *k1x, *k2x, *k1z, *k2z, *Au, *Av;
  int32_t *lu, *lv;
  int N1, N2, N1h, G1, G2, dny, nu, nv, np, ncol, nn;
  fftplan px, pz; /* complex plans of length G1 and G2 (wall bands) */
  /* multiblock: core band (band 2) resolution, its plans, the long-column flags of
   * the wall-band mode grid and jlim(lo/hi, grid, band) (start.f90:1675-1709) */
  int mb, N1c, N2c, G1c, G2c;
  fftplan pxc, pzc;
  unsigned char *lng;
  int bj[3][3][2]; /* [band 0..2][grid: 0 u, 1 v, 2 p][lo, hi], reference j */
  /* statistics (stats.f90): plane sums [11][nu], tile-conditioned sums [9][ncl][dnz][dnx];
   * pressure plane sums [2][np] and the conditioned P, omega_x sums [4][ncl + 1][dnz][dnx] */
  double *st_pl, *st_cd, *st_pp, *st_cd4;
  int st_ncl, st_dnx, st_dnz;
  int64_t istat;
  /* spectra (spectra.f90): sp(level, long column) of U, V, W, UV, P, level fastest */
  double *sp[5];
  int sp_nl[5], nlong;
  /* slip statistics (sl_stats2.f90): [wall 0 bottom, 1 top][u1_itp, du1dy, u3_itp, du3dy][column] */
  cplx *slip;
  /* plans of the unpadded N grids (four_to_phys_N): wall bands and core band */
  fftplan pxN, pzN, pxNc, pzNc;
  cplx *u1, *u2, *u3, *p;
  cplx *Nu1, *Nu2, *Nu3, *du1, *du2, *du3, *psi, *div;
  cplx *u1i, *u2i, *u3i; /* u1,u3 at v levels; u2 at u levels */
  cplx *uvf, *wvf, *vvc, *N1xz, *N2xz, *N3xz;
  double *DG; /* [np][ncol][3] factorised pressure matrices */
  double *phys_u1, *phys_u3, *phys_u2; /* physical planes, all levels (for IB) */
  /* owned copies of the triad lists */
  int8_t *tdata;
  int64_t *toff, *tlen;
  int32_t *tsu, *tsv;
  double t, dt, dti, dtc, err, mpgx, QxT, Qx;
  int64_t iter;
};

#define UIDX(j) ((j) + O->dny)          /* u or v level j -> array index */
#define PIDX(j) ((j) + O->dny - 1)      /* p level j -> array index */
#define PL(F, idx) ((F) + (size_t)(idx) * O->ncol)

/* column segments: a long column has one (band 2), a short column two (bands 1, 3) */
static inline int col_bands(const orc *O, int c, int b[2]) {
  if (!O->mb || O->lng[c]) { b[0] = 1; return 1; }
  b[0] = 0; b[1] = 2; return 2;
}

static double *dupd(const double *s, size_t n) {
  double *d = (double *)malloc(sizeof(double) * (n ? n : 1));
  if (n) memcpy(d, s, sizeof(double) * n);
  return d;
}

static cplx *zalloc(size_t n) { return (cplx *)calloc(n ? n : 1, sizeof(cplx)); }

/* pressure matrices of every band's columns over jlim(1:2, pgrid, band), LU_buildP +
 * LU_decP (tridLU_3D.f90:333-407, 477-518); gauge on mode (0,0) of band 2 */
static void build_DG(orc *O) {
  const double dd = O->c.ddthetavi;
  for (int c = 0; c < O->ncol; ++c) {
    int bs[2];
    const int nsg = col_bands(O, c, bs);
    const int r = c / O->N1h, kx = c % O->N1h;
    const double k2x = O->k2x[kx], k2z = O->k2z[r];
    for (int sgi = 0; sgi < nsg; ++sgi) {
      const int b = bs[sgi];
      const int ns = O->bj[b][2][0], ne = O->bj[b][2][1], n = ne - ns + 1;
      double *Db = (double *)malloc(sizeof(double) * (n + 2)); /* index m - (ns-1) */
      double *Gb = (double *)malloc(sizeof(double) * (n + 2));
      double *Dt = (double *)malloc(sizeof(double) * (n + 2));
      double *Gt = (double *)malloc(sizeof(double) * (n + 2));
#define X(m) ((m) - (ns - 1))
      for (int j = ns; j <= ne; ++j) {
        Db[X(j - 1)] = -dd * O->thu[UIDX(j)];
        Gb[X(j)] = -dd * O->thv[UIDX(j)];
        Dt[X(j)] = dd * O->thu[UIDX(j)];
        Gt[X(j + 1)] = dd * O->thv[UIDX(j)];
      }
#define A(cc, j) O->DG[((size_t)PIDX(j) * O->ncol + c) * 3 + (cc) - 1]
      A(1, ns) = 0.0;
      A(2, ns) = (Dt[X(ns)] * Gb[X(ns)]) + k2x + k2z;
      A(3, ns) = (Dt[X(ns)] * Gt[X(ns + 1)]);
      A(2, ne) = (Db[X(ne - 1)] * Gt[X(ne)]) + k2x + k2z;
      A(1, ne) = (Db[X(ne - 1)] * Gb[X(ne - 1)]);
      A(3, ne) = 0.0;
      for (int j = ns + 1; j <= ne - 1; ++j) {
        A(2, j) = (Db[X(j - 1)] * Gt[X(j)]) + (Dt[X(j)] * Gb[X(j)]) + k2x + k2z;
        A(1, j) = (Db[X(j - 1)] * Gb[X(j - 1)]);
        A(3, j) = (Dt[X(j)] * Gt[X(j + 1)]);
      }
      if (c == 0 && b == 1) { /* gauge of mode (0,0), tridLU_3D.f90:384-390 */
        double h = O->yu[UIDX(1 + 1)] - O->yu[UIDX(1)];
        A(1, ns) = 0.0;
        A(2, ns) = 1.0 / (h * h);
        A(3, ns) = 0.0;
      }
      A(2, ns) = 1.0 / A(2, ns);
      for (int j = ns + 1; j <= ne; ++j) {
        A(3, j - 1) = A(3, j - 1) * A(2, j - 1);
        A(2, j) = 1.0 / (A(2, j) - A(1, j) * A(3, j - 1));
      }
#undef A
#undef X
      free(Db); free(Gb); free(Dt); free(Gt);
    }
  }
}

void orc_destroy(orc *O);

/* Copies and checks the triad lists: header as nonlinRead checks it (start.f90:3040-3048),
 * every triad inside the retained modes with a target x-mode la + lp >= 0. */
static int copy_triads(orc *O, const lh_config *cfg) {
  if (cfg->triad_nx != O->N1 / 2 - 1 || cfg->triad_nz != O->N2 / 2 - 1) return -1;
  const int ns = cfg->triad_nsets, nx = cfg->triad_nx, nz = cfg->triad_nz;
  if (ns <= 0 || !cfg->triad_off || !cfg->triad_len || !cfg->triad_data) return -1;
  int64_t end = 0;
  for (int i = 0; i < 9 * ns; ++i) {
    if (cfg->triad_off[i] < 0 || cfg->triad_len[i] < 0) return -1;
    int64_t e = cfg->triad_off[i] + cfg->triad_len[i];
    if (e > end) end = e;
  }
  O->tdata = (int8_t *)malloc(4 * (size_t)end + 4);
  O->toff = (int64_t *)malloc(sizeof(int64_t) * 9 * ns);
  O->tlen = (int64_t *)malloc(sizeof(int64_t) * 9 * ns);
  O->tsu = (int32_t *)malloc(sizeof(int32_t) * O->nu);
  O->tsv = (int32_t *)malloc(sizeof(int32_t) * O->nv);
  memcpy(O->tdata, cfg->triad_data, 4 * (size_t)end);
  memcpy(O->toff, cfg->triad_off, sizeof(int64_t) * 9 * ns);
  memcpy(O->tlen, cfg->triad_len, sizeof(int64_t) * 9 * ns);
  memcpy(O->tsu, cfg->triad_set_u, sizeof(int32_t) * O->nu);
  memcpy(O->tsv, cfg->triad_set_v, sizeof(int32_t) * O->nv);
  for (int i = 0; i < 9 * ns; ++i) {
    const int8_t *l = O->tdata + 4 * O->toff[i];
    const int64_t L = O->tlen[i];
    for (int64_t e = 0; e < L; ++e) {
      int la = l[e], ka = l[L + e], lp = l[2 * L + e], kp = l[3 * L + e];
      if (abs(la) > nx || abs(lp) > nx || abs(ka) > nz || abs(kp) > nz) return -1;
      if (la + lp < 0 || la + lp > nx || abs(ka + kp) > nz) return -1;
    }
  }
  for (int q = 1; q < O->nu - 1; ++q) if (O->tsu[q] < 0 || O->tsu[q] >= ns) return -1;
  for (int q = 1; q < O->nv - 1; ++q) if (O->tsv[q] < 0 || O->tsv[q] >= ns) return -1;
  O->c.triad_data = O->tdata; O->c.triad_off = O->toff; O->c.triad_len = O->tlen;
  O->c.triad_set_u = O->tsu; O->c.triad_set_v = O->tsv;
  return 0;
}

orc *orc_create(const lh_config *cfg) {
  orc *O = (orc *)calloc(1, sizeof(orc));
  if (!O) return NULL;
  O->c = *cfg;
  O->N1 = cfg->N1; O->N2 = cfg->N2; O->N1h = cfg->N1 / 2 + 1;
  O->G1 = cfg->Ngal1; O->G2 = cfg->Ngal2; O->dny = cfg->dny;
  O->nu = cfg->nyu; O->nv = cfg->nyv; O->np = cfg->nyu - 2; O->nn = cfg->nn;
  O->ncol = O->N1h * O->N2;
  O->N1c = cfg->N1c; O->N2c = cfg->N2c; O->G1c = cfg->Ngal1c; O->G2c = cfg->Ngal2c;
  O->mb = (O->N1c != O->N1 || O->N2c != O->N2 || O->G1c != O->G1 || O->G2c != O->G2);
  if (O->N1c <= 0 || O->N2c <= 0 || O->N1c > O->N1 || O->N2c > O->N2 || (O->N1c & 1) || (O->N2c & 1) ||
      O->G1c <= O->N1c || O->G2c <= O->N2c || (O->mb && cfg->nonlin_form == LH_NONLIN_TRIADS)) {
    free(O);
    return NULL;
  }
  {
    const int *N3 = cfg->N3, *N4 = cfg->N4;
    const int bj[3][3][2] = {{{N4[0], N4[1] + 1}, {N3[0], N3[1] + 1}, {N4[0] + 1, N4[1]}},
                             {{N4[0], N4[3] + 1}, {N3[0], N3[3] + 1}, {N4[0] + 1, N4[3]}},
                             {{N4[2], N4[3] + 1}, {N3[2], N3[3] + 1}, {N4[2] + 1, N4[3]}}};
    memcpy(O->bj, bj, sizeof(bj));
    O->lng = (unsigned char *)malloc((size_t)O->ncol);
    for (int c = 0; c < O->ncol; ++c) {
      const int r = c / O->N1h, kx = c % O->N1h;
      O->lng[c] = (kx <= O->N1c / 2) && (r < O->N2c / 2 || r >= O->N2 - O->N2c / 2);
    }
  }
  O->yu = dupd(cfg->yu, O->nu); O->yv = dupd(cfg->yv, O->nv);
  O->thu = dupd(cfg->dthdyu, O->nu); O->thv = dupd(cfg->dthdyv, O->nv);
  O->d2u = dupd(cfg->dyu2i, 3 * (size_t)O->nu); O->d2v = dupd(cfg->dyv2i, 3 * (size_t)O->nv);
  O->k1x = dupd(cfg->k1x, O->N1h); O->k2x = dupd(cfg->k2x, O->N1h);
  O->k1z = dupd(cfg->k1z, O->N2); O->k2z = dupd(cfg->k2z, O->N2);
  O->lu = (int32_t *)malloc(sizeof(int32_t) * (6 * (size_t)cfg->nib_u + 1));
  O->lv = (int32_t *)malloc(sizeof(int32_t) * (6 * (size_t)cfg->nib_v + 1));
  if (cfg->nib_u) memcpy(O->lu, cfg->list_ib_u, sizeof(int32_t) * 6 * (size_t)cfg->nib_u);
  if (cfg->nib_v) memcpy(O->lv, cfg->list_ib_v, sizeof(int32_t) * 6 * (size_t)cfg->nib_v);
  O->Au = dupd(cfg->A_ib_u, cfg->nib_u); O->Av = dupd(cfg->A_ib_v, cfg->nib_v);
  O->c.yu = O->yu; O->c.yv = O->yv; O->c.dthdyu = O->thu; O->c.dthdyv = O->thv;
  O->c.dyu2i = O->d2u; O->c.dyv2i = O->d2v; O->c.k1x = O->k1x; O->c.k2x = O->k2x;
  O->c.k1z = O->k1z; O->c.k2z = O->k2z; O->c.list_ib_u = O->lu; O->c.list_ib_v = O->lv;
  O->c.A_ib_u = O->Au; O->c.A_ib_v = O->Av;
  if (plan_init(&O->px, O->G1) || plan_init(&O->pz, O->G2) || plan_init(&O->pxc, O->G1c) ||
      plan_init(&O->pzc, O->G2c) || plan_init(&O->pxN, O->N1) || plan_init(&O->pzN, O->N2) ||
      plan_init(&O->pxNc, O->N1c) || plan_init(&O->pzNc, O->N2c))
    return NULL;
  size_t nc = (size_t)O->ncol;
  O->u1 = zalloc(nc * O->nu); O->u3 = zalloc(nc * O->nu); O->u2 = zalloc(nc * O->nv);
  O->p = zalloc(nc * O->np);
  O->Nu1 = zalloc(nc * O->nu); O->Nu3 = zalloc(nc * O->nu); O->Nu2 = zalloc(nc * O->nv);
  O->du1 = zalloc(nc * O->nu); O->du3 = zalloc(nc * O->nu); O->du2 = zalloc(nc * O->nv);
  O->psi = zalloc(nc * O->np); O->div = zalloc(nc * O->np);
  O->u1i = zalloc(nc * O->nv); O->u3i = zalloc(nc * O->nv); O->u2i = zalloc(nc * O->nu);
  O->uvf = zalloc(nc * O->nv); O->wvf = zalloc(nc * O->nv); O->vvc = zalloc(nc * O->nu);
  O->N1xz = zalloc(nc * O->nu); O->N3xz = zalloc(nc * O->nu); O->N2xz = zalloc(nc * O->nv);
  O->DG = (double *)calloc(3 * nc * O->np, sizeof(double));
  size_t pp = (size_t)O->G1 * O->G2;
  O->phys_u1 = (double *)calloc(pp * O->nu, sizeof(double));
  O->phys_u3 = (double *)calloc(pp * O->nu, sizeof(double));
  O->phys_u2 = (double *)calloc(pp * O->nv, sizeof(double));
  if (cfg->nonlin_form == LH_NONLIN_TRIADS && copy_triads(O, cfg)) { orc_destroy(O); return NULL; }
  build_DG(O);
  O->dt = 0; O->t = 0; O->mpgx = cfg->Re * 0; O->iter = 0;
  return O;
}

void orc_destroy(orc *O) {
  if (!O) return;
  void *ptrs[] = {O->yu, O->yv, O->thu, O->thv, O->d2u, O->d2v, O->k1x, O->k2x, O->k1z, O->k2z,
                  O->Au, O->Av, O->lu, O->lv, O->u1, O->u2, O->u3, O->p, O->Nu1, O->Nu2, O->Nu3,
                  O->du1, O->du2, O->du3, O->psi, O->div, O->u1i, O->u2i, O->u3i, O->uvf, O->wvf,
                  O->vvc, O->N1xz, O->N2xz, O->N3xz, O->DG, O->phys_u1, O->phys_u3, O->phys_u2,
                  O->tdata, O->toff, O->tlen, O->tsu, O->tsv, O->lng, O->st_pl, O->st_cd, O->st_pp, O->st_cd4,
                  O->sp[0], O->sp[1], O->sp[2], O->sp[3], O->sp[4], O->slip};
  for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); ++i) free(ptrs[i]);
  plan_free(&O->px); plan_free(&O->pz); plan_free(&O->pxc); plan_free(&O->pzc);
  plan_free(&O->pxN); plan_free(&O->pzN); plan_free(&O->pxNc); plan_free(&O->pzNc);
  free(O);
}

/* ------------------------------------------------------------------------- */
/* transforms of one plane                                                     */
/* ------------------------------------------------------------------------- */
/* A plane's resolution: the wall bands' (every mode of the wall-band grid) or the
 * core band's (the long columns only). Mode (r, kx) of a view, r its own kz index,
 * lives at wall-grid column frow(r) * (N1/2+1) + kx (the dk shift, start.f90:1722-1734). */
typedef struct { int N1h, N2, G1, G2; const fftplan *px, *pz; } pview;
static inline size_t vcol(const orc *O, const pview *v, int r, int kx) {
  const int fr = r < v->N2 / 2 ? r : r + O->N2 - v->N2;
  return (size_t)fr * O->N1h + kx;
}
static inline void view_of(const orc *O, int fine, pview *v) {
  if (fine) { v->N1h = O->N1h; v->N2 = O->N2; v->G1 = O->G1; v->G2 = O->G2; v->px = &O->px; v->pz = &O->pz; }
  else { v->N1h = O->N1c / 2 + 1; v->N2 = O->N2c; v->G1 = O->G1c; v->G2 = O->G2c; v->px = &O->pxc; v->pz = &O->pzc; }
}
/* band of planes (proc_lims_planes, start.f90:1836-1916): u plane j is a wall-band plane
 * for j <= N(4,1) or j > N(4,2); v plane j for j <= N(3,1) or j > N(3,2) */
static inline int fine_u(const orc *O, int j) { return !O->mb || j <= O->c.N4[1] || j > O->c.N4[2]; }
static inline int fine_v(const orc *O, int j) { return !O->mb || j <= O->c.N3[1] || j > O->c.N3[2]; }

/* plane row (0-based, physical z index) of kz-index r of a view */
static inline int prow(const pview *v, int r) { return r < v->N2 / 2 ? r : r - v->N2 + v->G2; }



/* work buffers for one thread (sized for the wall-band planes, the largest) */
typedef struct { cplx *A; cplx *line; cplx *tmp; } pwork;

static void pwork_init(const orc *O, pwork *w) {
  int n = O->G1 > O->G2 ? O->G1 : O->G2;
  w->A = zalloc((size_t)O->G2 * (O->G1 / 2 + 1));
  w->line = zalloc((size_t)n);
  w->tmp = zalloc((size_t)n);
}
static void pwork_free(pwork *w) { free(w->A); free(w->line); free(w->tmp); }

/* four_to_phys (FOU3D.f90:738-781): the modes of view v of spectral plane S -> phys[l][m]
 * (G2 x G1 of the view). z: backward complex transform of the N1/2+1 retained x-modes; x:
 * backward real transform of every row, Im of x-modes 0 and G1/2 ignored. */
static void four_to_phys_plane(const orc *O, const pview *v, const cplx *S, double *phys, pwork *w) {
  const int G1 = v->G1, G2 = v->G2, Gh = G1 / 2 + 1, N1h = v->N1h;
  memset(w->A, 0, sizeof(cplx) * (size_t)G2 * Gh);
  for (int kx = 0; kx < N1h; ++kx) {
    for (int l = 0; l < G2; ++l) w->line[l] = 0;
    for (int r = 0; r < v->N2; ++r) w->line[prow(v, r)] = S[vcol(O, v, r, kx)];
    w->line[G2 / 2] = 0; /* zeroed z 'oddball' row */
    fft_inplace(v->pz, w->line, +1, w->tmp);
    for (int l = 0; l < G2; ++l) w->A[(size_t)l * Gh + kx] = w->line[l];
  }
  /* x: pair rows (a, b) into one complex backward transform */
  for (int l = 0; l < G2; l += 2) {
    const cplx *a = w->A + (size_t)l * Gh;
    const cplx *b = (l + 1 < G2) ? w->A + (size_t)(l + 1) * Gh : NULL;
    for (int k = 0; k < G1; ++k) w->line[k] = 0;
    for (int k = 0; k <= G1 / 2; ++k) {
      cplx ak = a[k], bk = b ? b[k] : 0;
      if (k == 0 || k == G1 / 2) { ak = creal(ak); bk = creal(bk); }
      w->line[k] = ak + I * bk;
      if (k > 0 && k < G1 / 2) w->line[G1 - k] = conj(ak) + I * conj(bk);
    }
    fft_inplace(v->px, w->line, +1, w->tmp);
    for (int m = 0; m < G1; ++m) {
      phys[(size_t)l * G1 + m] = creal(w->line[m]);
      if (b) phys[(size_t)(l + 1) * G1 + m] = cimag(w->line[m]);
    }
  }
}

/* phys_to_four (FOU3D.f90:2253-2272) restricted to the retained modes of view v: writes
 * C at the view's columns for all its N2 rows (the zeroed row G2/2 is never retained). */
static void phys_to_four_plane(const orc *O, const pview *v, const double *phys, cplx *C, pwork *w) {
  const int G1 = v->G1, G2 = v->G2, Gh = G1 / 2 + 1, N1h = v->N1h;
  const double s1 = 1.0 / G1, s2 = 1.0 / G2;
  for (int l = 0; l < G2; l += 2) {
    int hasb = (l + 1 < G2);
    for (int m = 0; m < G1; ++m)
      w->line[m] = phys[(size_t)l * G1 + m] + I * (hasb ? phys[(size_t)(l + 1) * G1 + m] : 0.0);
    fft_inplace(v->px, w->line, -1, w->tmp);
    for (int k = 0; k <= G1 / 2; ++k) {
      cplx z = w->line[k], zc = conj(w->line[(G1 - k) % G1]);
      cplx A = 0.5 * (z + zc), B = -0.5 * I * (z - zc);
      A *= s1; B *= s1;
      if (k == 0 || k == G1 / 2) { A = creal(A); B = creal(B); }
      w->A[(size_t)l * Gh + k] = A;
      if (hasb) w->A[(size_t)(l + 1) * Gh + k] = B;
    }
  }
  for (int kx = 0; kx < N1h; ++kx) {
    for (int l = 0; l < G2; ++l) w->line[l] = w->A[(size_t)l * Gh + kx];
    fft_inplace(v->pz, w->line, -1, w->tmp);
    for (int r = 0; r < v->N2; ++r) C[vcol(O, v, r, kx)] = w->line[prow(v, r)] * s2;
  }
}

/* der_x / der_z (FOU3D.f90:476-593) of the view's modes, summed:
 * out = i kx * X + i kz * Z, with the row kz = -N2/2 of the view zeroed. */
static void derxz(const orc *O, const pview *v, const cplx *X, const cplx *Z, cplx *out) {
  for (int r = 0; r < v->N2; ++r)
    for (int kx = 0; kx < v->N1h; ++kx) {
      size_t c = vcol(O, v, r, kx);
      if (r == v->N2 / 2) { out[c] = 0; continue; }
      cplx kxF = I * O->k1x[kx], kzF = I * O->k1z[c / O->N1h];
      out[c] = kxF * X[c] + kzF * Z[c];
    }
}

/* ------------------------------------------------------------------------- */
/* triad-list products (ops_in_planes + nonlinInter, FOU3D.f90:1724-2088)      */
/* ------------------------------------------------------------------------- */
/* plane row of z-mode k in -N2/2..N2/2: kLkup (start.f90:1155-1163) on the compact
 * [kz row][kx] plane, where row N2/2 holds kz = -N2/2 (= +N2/2) */
static inline int krow(const orc *O, int k) { return k >= 0 ? k : k + O->N2; }

/* nonlinInter (FOU3D.f90:1983-2012): X(la+lp, +-(ka+kp)) += A(la, +-ka) P(lp, +-kp) for every
 * listed triad, mirrored pass p = 0 first; x-mode l < 0 reads conj of mode (|l|, -k).
 * Evaluation order as the Fortran expression. */
static void nonlin_inter(const orc *O, int set, int type, cplx *X, const cplx *A, const cplx *P) {
  const int N1h = O->N1h;
  const int64_t L = O->tlen[set * 9 + type - 1];
  const int8_t *l = O->tdata + 4 * O->toff[set * 9 + type - 1];
  double *x = (double *)X;
  const double *a = (const double *)A, *pp = (const double *)P;
  for (int64_t e = 0; e < L; ++e) {
    const int la = l[e], ka0 = l[L + e], lp = l[2 * L + e], kp0 = l[3 * L + e];
    const int sa = la < 0 ? -1 : 1, sp = lp < 0 ? -1 : 1;
    const int ia = abs(la), ip = abs(lp), it = la + lp;
    for (int p = 0; p <= 1; ++p) {
      if (ka0 + kp0 == 0 && p == 1) continue;
      const int pn = p * 2 - 1;
      const int ka = krow(O, pn * sa * ka0), kp = krow(O, pn * sp * kp0), kt = krow(O, pn * (ka0 + kp0));
      const double ar = a[2 * (ka * N1h + ia)], ai = a[2 * (ka * N1h + ia) + 1];
      const double pr = pp[2 * (kp * N1h + ip)], pi = pp[2 * (kp * N1h + ip) + 1];
      double *xt = x + 2 * (kt * N1h + it);
      xt[0] = (xt[0] + ar * pr) - ((double)(sa * sp) * ai) * pi;
      xt[1] = (xt[1] + ((double)sp * ar) * pi) + ((double)sa * ai) * pr;
    }
  }
}

/* zeroth mode of a product, sum over i = -N1/2..N1/2, k = klo..N2/2-1 of
 * A(i, k) P(-i, -k) (FOU3D.f90:1755-1772, 1902-1920) */
static void zeroth_mode(const orc *O, int klo, cplx *X, const cplx *A, const cplx *P) {
  const int N1h = O->N1h;
  const double *a = (const double *)A, *pp = (const double *)P;
  double xr = creal(X[0]), xi = cimag(X[0]);
  for (int i = -(O->N1 / 2); i <= O->N1 / 2; ++i)
    for (int k = klo; k <= O->N2 / 2 - 1; ++k) {
      const int sa = i < 0 ? -1 : 1, sp = -i < 0 ? -1 : 1;
      const int ia = abs(i), ip = abs(i);
      const int ka = krow(O, sa * k), kp = krow(O, sp * (-k));
      const double ar = a[2 * (ka * N1h + ia)], ai = a[2 * (ka * N1h + ia) + 1];
      const double pr = pp[2 * (kp * N1h + ip)], pi = pp[2 * (kp * N1h + ip) + 1];
      xr = (xr + ar * pr) - ((double)(sa * sp) * ai) * pi;
      xi = (xi + (ar * pi) * (double)sp) + ((double)sa * ai) * pr;
    }
  X[0] = CMPLX(xr, xi);
}

/* ops_in_planes: products of every u plane (uu, uw, vv, wu, ww) and v plane (uv, vu, vw,
 * wv) by linear advection + zeroth mode + listed triads, then der_x / der_z; the physical
 * planes feed dtc_calc and the immersed boundaries as in the transform form. */
static void triad_products(orc *O, double *pu1m, double *pu3m, double *pu2m) {
  const int nc = O->ncol, N2 = O->N2;
  const size_t pp = (size_t)O->G1 * O->G2;
  const int ulo = O->c.N4[0] + 1, uhi = O->c.N4[3], vlo = O->c.N3[0] + 1, vhi = O->c.N3[3];
  double u1m = *pu1m, u3m = *pu3m, u2m = *pu2m;
  pview vf;
  view_of(O, 1, &vf);
#pragma omp parallel reduction(max : u1m, u3m, u2m)
  {
    pwork w; pwork_init(O, &w);
    double *f = (double *)malloc(sizeof(double) * pp);
    cplx *t1 = zalloc(nc), *t2 = zalloc(nc), *t3 = zalloc(nc), *t4 = zalloc(nc);
#pragma omp for schedule(dynamic)
    for (int j = ulo; j <= uhi; ++j) {
      const int q = UIDX(j), set = O->tsu[q];
      const cplx *U = PL(O->u1, q), *V = PL(O->u2i, q), *W = PL(O->u3, q);
      cplx *uu = t1, *uw = t2, *wu = t3, *ww = t4, *vv = PL(O->vvc, q);
      vv[0] = 0;
      zeroth_mode(O, -(N2 / 2), vv, V, V);
      const double u00 = creal(U[0]), v00 = creal(V[0]), w00 = creal(W[0]);
      for (int c = 0; c < nc; ++c) {
        const double ur = creal(U[c]), ui = cimag(U[c]), vr = creal(V[c]), vi = cimag(V[c]);
        const double wr = creal(W[c]), wi = cimag(W[c]);
        uu[c] = CMPLX(2 * (u00 * ur), 2 * (u00 * ui));
        ww[c] = CMPLX(2 * (w00 * wr), 2 * (w00 * wi));
        if (c != 0) vv[c] = CMPLX(2 * (v00 * vr), 2 * (v00 * vi));
        uw[c] = CMPLX(u00 * wr + w00 * ur, u00 * wi + w00 * ui);
        wu[c] = uw[c];
      }
      nonlin_inter(O, set, 1, uu, U, U);
      nonlin_inter(O, set, 3, uw, W, U);
      nonlin_inter(O, set, 5, vv, V, V);
      nonlin_inter(O, set, 7, wu, U, W);
      nonlin_inter(O, set, 9, ww, W, W);
      derxz(O, &vf, uu, uw, PL(O->N1xz, q));
      derxz(O, &vf, wu, ww, PL(O->N3xz, q));
      four_to_phys_plane(O, &vf, U, f, &w);
      for (size_t e = 0; e < pp; ++e) if (fabs(f[e]) > u1m) u1m = fabs(f[e]);
      memcpy(O->phys_u1 + pp * q, f, sizeof(double) * pp);
      four_to_phys_plane(O, &vf, W, f, &w);
      for (size_t e = 0; e < pp; ++e) if (fabs(f[e]) > u3m) u3m = fabs(f[e]);
      memcpy(O->phys_u3 + pp * q, f, sizeof(double) * pp);
    }
#pragma omp for schedule(dynamic)
    for (int j = vlo; j <= vhi; ++j) {
      const int q = UIDX(j), set = O->tsv[q];
      const cplx *Ui = PL(O->u1i, q), *V = PL(O->u2, q), *Wi = PL(O->u3i, q);
      cplx *uv = PL(O->uvf, q), *wv = PL(O->wvf, q), *vu = t1, *vw = t2;
      uv[0] = 0;
      wv[0] = 0;
      zeroth_mode(O, -(N2 / 2 - 1), uv, Ui, V);
      zeroth_mode(O, -(N2 / 2 - 1), wv, Wi, V);
      const double u00 = creal(Ui[0]), v00 = creal(V[0]), w00 = creal(Wi[0]);
      for (int c = 0; c < nc; ++c) {
        const double ur = creal(Ui[c]), ui = cimag(Ui[c]), vr = creal(V[c]), vi = cimag(V[c]);
        const double wr = creal(Wi[c]), wi = cimag(Wi[c]);
        vu[c] = CMPLX(u00 * vr + v00 * ur, u00 * vi + v00 * ui);
        vw[c] = CMPLX(v00 * wr + w00 * vr, v00 * wi + w00 * vi);
        if (c != 0) { uv[c] = vu[c]; wv[c] = vw[c]; }
      }
      nonlin_inter(O, set, 2, uv, V, Ui);
      nonlin_inter(O, set, 4, vu, Ui, V);
      nonlin_inter(O, set, 6, vw, Wi, V);
      nonlin_inter(O, set, 8, wv, V, Wi);
      derxz(O, &vf, vu, vw, PL(O->N2xz, q));
      four_to_phys_plane(O, &vf, V, f, &w);
      const double th = O->thv[q];
      for (size_t e = 0; e < pp; ++e) {
        double a = fabs(f[e]) * th;
        if (a > u2m) u2m = a;
      }
      memcpy(O->phys_u2 + pp * q, f, sizeof(double) * pp);
    }
    free(f); free(t1); free(t2); free(t3); free(t4);
    pwork_free(&w);
  }
  *pu1m = u1m; *pu3m = u3m; *pu2m = u2m;
}

/* ------------------------------------------------------------------------- */
/* nonlinear (FOU3D.f90:41-425 with ops_in_planes2)                          */
/* ------------------------------------------------------------------------- */
/* interp_u (u1,u3 -> v levels) and interp_v (u2 -> u levels) of every band's columns
 * over the band's levels, FOU3D.f90:427-474 */
static void interp_all(orc *O) {
  const int nc = O->ncol;
#pragma omp parallel for schedule(static)
  for (int c = 0; c < nc; ++c) {
    int bs[2];
    const int ns = col_bands(O, c, bs);
    for (int sgi = 0; sgi < ns; ++sgi) {
      const int b = bs[sgi];
      for (int jv = O->bj[b][1][0]; jv <= O->bj[b][1][1]; ++jv) {
        double yv = O->yv[UIDX(jv)], yuj = O->yu[UIDX(jv)], yu1 = O->yu[UIDX(jv + 1)];
        cplx a = PL(O->u1, UIDX(jv + 1))[c], bb = PL(O->u1, UIDX(jv))[c];
        PL(O->u1i, UIDX(jv))[c] = ((yv - yuj) * a + (yu1 - yv) * bb) / (yu1 - yuj);
        a = PL(O->u3, UIDX(jv + 1))[c]; bb = PL(O->u3, UIDX(jv))[c];
        PL(O->u3i, UIDX(jv))[c] = ((yv - yuj) * a + (yu1 - yv) * bb) / (yu1 - yuj);
      }
      const int lo = O->bj[b][0][0], hi = O->bj[b][0][1], vlo = O->bj[b][1][0], vhi = O->bj[b][1][1];
      for (int ju = lo + 1; ju <= hi - 1; ++ju) {
        double yuj = O->yu[UIDX(ju)], yvm = O->yv[UIDX(ju - 1)], yvj = O->yv[UIDX(ju)];
        PL(O->u2i, UIDX(ju))[c] = ((yuj - yvm) * PL(O->u2, UIDX(ju))[c]
                                   + (yvj - yuj) * PL(O->u2, UIDX(ju - 1))[c]) / (yvj - yvm);
      }
      cplx i1 = PL(O->u2i, UIDX(lo + 1))[c], i2 = PL(O->u2i, UIDX(hi - 1))[c];
      PL(O->u2i, UIDX(lo))[c] = O->c.gw_interp[b][0] * (PL(O->u2, UIDX(vlo))[c] - i1) + i1;
      PL(O->u2i, UIDX(hi))[c] = O->c.gw_interp[b][1] * (PL(O->u2, UIDX(vhi))[c] - i2) + i2;
    }
  }
}

static void nonlinear(orc *O, int kRK) {
  const int nc = O->ncol;
  const double dd = O->c.ddthetavi;
  interp_all(O);

  const size_t ppF = (size_t)O->G1 * O->G2;
  double u1m = 0.0, u3m = 0.0, u2m = 1e-6;
  int ulo = O->c.N4[0] + 1, uhi = O->c.N4[3];
  int vlo = O->c.N3[0] + 1, vhi = O->c.N3[3];

  if (O->c.nonlin_form == LH_NONLIN_TRIADS) triad_products(O, &u1m, &u3m, &u2m);
  else
#pragma omp parallel reduction(max : u1m, u3m, u2m)
  {
    pwork w; pwork_init(O, &w);
    double *f1 = (double *)malloc(sizeof(double) * ppF), *f2 = (double *)malloc(sizeof(double) * ppF);
    double *f3 = (double *)malloc(sizeof(double) * ppF);
    double *q1 = (double *)malloc(sizeof(double) * ppF), *q2 = (double *)malloc(sizeof(double) * ppF);
    double *q3 = (double *)malloc(sizeof(double) * ppF), *q4 = (double *)malloc(sizeof(double) * ppF);
    cplx *c1 = zalloc(nc), *c2 = zalloc(nc), *c3 = zalloc(nc), *c4 = zalloc(nc);
#pragma omp for schedule(dynamic)
    for (int ju = ulo; ju <= uhi; ++ju) {
      pview v;
      view_of(O, fine_u(O, ju), &v);
      const size_t pp = (size_t)v.G1 * v.G2;
      four_to_phys_plane(O, &v, PL(O->u1, UIDX(ju)), f1, &w);
      four_to_phys_plane(O, &v, PL(O->u2i, UIDX(ju)), f2, &w);
      four_to_phys_plane(O, &v, PL(O->u3, UIDX(ju)), f3, &w);
      for (size_t e = 0; e < pp; ++e) {
        q1[e] = f1[e] * f1[e];
        q2[e] = f1[e] * f3[e];
        q3[e] = f2[e] * f2[e];
        q4[e] = f3[e] * f3[e];
        if (fabs(f1[e]) > u1m) u1m = fabs(f1[e]);
        if (fabs(f3[e]) > u3m) u3m = fabs(f3[e]);
      }
      memcpy(O->phys_u1 + ppF * UIDX(ju), f1, sizeof(double) * pp);
      memcpy(O->phys_u3 + ppF * UIDX(ju), f3, sizeof(double) * pp);
      phys_to_four_plane(O, &v, q1, c1, &w);
      phys_to_four_plane(O, &v, q2, c2, &w);
      phys_to_four_plane(O, &v, q3, PL(O->vvc, UIDX(ju)), &w);
      phys_to_four_plane(O, &v, q4, c4, &w);
      derxz(O, &v, c1, c2, PL(O->N1xz, UIDX(ju)));
      derxz(O, &v, c2, c4, PL(O->N3xz, UIDX(ju)));
    }
#pragma omp for schedule(dynamic)
    for (int jv = vlo; jv <= vhi; ++jv) {
      pview v;
      view_of(O, fine_v(O, jv), &v);
      const size_t pp = (size_t)v.G1 * v.G2;
      four_to_phys_plane(O, &v, PL(O->u1i, UIDX(jv)), f1, &w);
      four_to_phys_plane(O, &v, PL(O->u2, UIDX(jv)), f2, &w);
      four_to_phys_plane(O, &v, PL(O->u3i, UIDX(jv)), f3, &w);
      double th = O->thv[UIDX(jv)];
      for (size_t e = 0; e < pp; ++e) {
        q1[e] = f1[e] * f2[e];
        q2[e] = f3[e] * f2[e];
        double a = fabs(f2[e]) * th;
        if (a > u2m) u2m = a;
      }
      memcpy(O->phys_u2 + ppF * UIDX(jv), f2, sizeof(double) * pp);
      phys_to_four_plane(O, &v, q1, PL(O->uvf, UIDX(jv)), &w);
      phys_to_four_plane(O, &v, q2, PL(O->wvf, UIDX(jv)), &w);
      derxz(O, &v, PL(O->uvf, UIDX(jv)), PL(O->wvf, UIDX(jv)), PL(O->N2xz, UIDX(jv)));
    }
    free(f1); free(f2); free(f3); free(q1); free(q2); free(q3); free(q4);
    free(c1); free(c2); free(c3); free(c4);
    pwork_free(&w);
  }
  /* product wall planes are never computed: zero (v = 0 at the walls) */
  memset(PL(O->uvf, UIDX(O->c.N3[0])), 0, sizeof(cplx) * nc);
  memset(PL(O->wvf, UIDX(O->c.N3[0])), 0, sizeof(cplx) * nc);
  memset(PL(O->uvf, UIDX(O->c.N3[3] + 1)), 0, sizeof(cplx) * nc);
  memset(PL(O->wvf, UIDX(O->c.N3[3] + 1)), 0, sizeof(cplx) * nc);

  /* y-derivatives and assembly over every band's interior levels (FOU3D.f90:262-283,
   * 636-676); a short column's band-end flux level lies on a core plane, which holds
   * no short modes: its flux is zero, as the reference's transposes leave it */
#pragma omp parallel for schedule(static)
  for (int c = 0; c < nc; ++c) {
    int bs[2];
    const int ns = col_bands(O, c, bs);
    for (int sgi = 0; sgi < ns; ++sgi) {
      const int b = bs[sgi];
      for (int ju = O->bj[b][0][0] + 1; ju <= O->bj[b][0][1] - 1; ++ju) {
        double th = O->thu[UIDX(ju)];
        cplx d1 = (PL(O->uvf, UIDX(ju))[c] - PL(O->uvf, UIDX(ju - 1))[c]) * th * dd;
        cplx d3 = (PL(O->wvf, UIDX(ju))[c] - PL(O->wvf, UIDX(ju - 1))[c]) * th * dd;
        PL(O->Nu1, UIDX(ju))[c] = PL(O->N1xz, UIDX(ju))[c] + d1;
        PL(O->Nu3, UIDX(ju))[c] = PL(O->N3xz, UIDX(ju))[c] + d3;
      }
      for (int jv = O->bj[b][1][0] + 1; jv <= O->bj[b][1][1] - 1; ++jv) {
        double th = O->thv[UIDX(jv)];
        cplx d2 = (PL(O->vvc, UIDX(jv + 1))[c] - PL(O->vvc, UIDX(jv))[c]) * th * dd;
        PL(O->Nu2, UIDX(jv))[c] = PL(O->N2xz, UIDX(jv))[c] + d2;
      }
    }
  }

  if (kRK == 1) {
    double a = 1.0 / (O->c.alp * (double)(O->N1 / 2) * u1m);
    double b = 1.0 / (O->c.bet * (double)(O->N2 / 2) * u3m);
    double cv = 1.0 / (u2m * O->c.dthetavi);
    double d = a < b ? a : b;
    O->dtc = d < cv ? d : cv;
    double lim = 2.5 * O->c.dtv, cfl = O->c.CFL * O->dtc;
    O->dt = lim < cfl ? lim : cfl;
    O->dti = 1.0 / O->dt;
    O->t = O->t + O->dt;
  }
}

/* immersed-boundary forcing (FOU3D.f90:806-998), one grid */
static void imm_bounds(orc *O, cplx *du, const double *uphys, int nlist, const int32_t *list,
                       const double *A, int lo0, int hi0, int lo1, int hi1) {
  const int G1 = O->G1, G2 = O->G2;
  const size_t pp = (size_t)G1 * G2;
  const double Kibdt = O->c.Kib / O->dt;
  int ranges[2][2] = {{lo0, hi0}, {lo1, hi1}};
  for (int rg = 0; rg < 2; ++rg) {
#pragma omp parallel
    {
      pwork w; pwork_init(O, &w);
      pview vf;
      view_of(O, 1, &vf);
      double *ph = (double *)malloc(sizeof(double) * pp);
#pragma omp for schedule(dynamic)
      for (int j = ranges[rg][0]; j <= ranges[rg][1]; ++j) {
        four_to_phys_plane(O, &vf, PL(du, UIDX(j)), ph, &w);
        for (int e = 0; e < nlist; ++e) {
          const int32_t *L = list + 6 * (size_t)e;
          if (L[2] != j) continue;
          double V = A[e] * uphys[pp * UIDX(L[5]) + (size_t)(L[4] - 1) * G1 + (L[3] - 1)];
          double u = uphys[pp * UIDX(j) + (size_t)(L[1] - 1) * G1 + (L[0] - 1)];
          ph[(size_t)(L[1] - 1) * G1 + (L[0] - 1)] = Kibdt * (V - u);
        }
        phys_to_four_plane(O, &vf, ph, PL(du, UIDX(j)), &w);
      }
      free(ph);
      pwork_free(&w);
    }
  }
}

/* tridiagonal LU of one column (LU_dec, tridLU_3D.f90:437-474) and both sweeps */
static void lu_dec(double *a1, double *a2, double *a3, int n) {
  a2[0] = 1.0 / a2[0];
  for (int j = 1; j < n; ++j) {
    a3[j - 1] = a3[j - 1] * a2[j - 1];
    a2[j] = 1.0 / (a2[j] - a1[j] * a3[j - 1]);
  }
}
static void lu_sol(const double *a1, const double *a2, const double *a3, cplx *x, int n,
                   size_t stride) {
  x[0] = x[0] * a2[0];
  for (int j = 1; j < n; ++j) x[j * stride] = (x[j * stride] - a1[j] * x[(j - 1) * stride]) * a2[j];
  for (int j = n - 2; j >= 0; --j) x[j * stride] = x[j * stride] - a3[j] * x[(j + 1) * stride];
}

static void flowrate_corr(orc *O, int kRK) {
  int nn = O->nn;
  int n = nn + 3; /* levels 0..nn+2 */
  double *u11 = (double *)calloc(n, sizeof(double));
  double *a1 = (double *)calloc(n, sizeof(double)), *a2 = (double *)calloc(n, sizeof(double));
  double *a3 = (double *)calloc(n, sizeof(double));
  double bdt = -O->c.dRK[kRK - 1] * O->dt;
  u11[0] = 0.0;
  for (int j = 1; j <= nn + 1; ++j) u11[j] = bdt;
  u11[nn + 2] = 0.0;
  double beta = O->c.bRK[kRK - 1] * O->dt / O->c.Re;
  a1[0] = 0.0; a2[0] = 1.0; a3[0] = O->c.gw[1][0];
  for (int j = 1; j <= nn + 1; ++j) {
    a1[j] = -beta * O->d2u[0 * O->nu + UIDX(j)];
    a2[j] = 1.0 - beta * O->d2u[1 * O->nu + UIDX(j)];
    a3[j] = -beta * O->d2u[2 * O->nu + UIDX(j)];
  }
  a1[nn + 2] = O->c.gw[1][1]; a2[nn + 2] = 1.0; a3[nn + 2] = 0.0;
  lu_dec(a1, a2, a3, n);
  u11[0] = u11[0] * a2[0];
  for (int j = 1; j < n; ++j) u11[j] = (u11[j] - a1[j] * u11[j - 1]) * a2[j];
  for (int j = n - 2; j >= 0; --j) u11[j] = u11[j] - a3[j] * u11[j + 1];
  double Qx1 = 0.0, Qx0 = 0.0;
  for (int j = 1; j <= nn + 1; ++j) Qx1 = Qx1 + (O->yv[UIDX(j)] - O->yv[UIDX(j - 1)]) * u11[j];
  for (int j = 1; j <= nn + 1; ++j)
    Qx0 = Qx0 + (O->yv[UIDX(j)] - O->yv[UIDX(j - 1)]) * creal(PL(O->u1, UIDX(j))[0]);
  double g = (O->QxT - Qx0) / Qx1;
  O->mpgx = O->mpgx + g;
  for (int j = 0; j <= nn + 2; ++j) PL(O->u1, UIDX(j))[0] = PL(O->u1, UIDX(j))[0] + g * u11[j];
  free(u11); free(a1); free(a2); free(a3);
}

static double flowrateIm(const orc *O) {
  double Q = 0.0;
  for (int j = 1; j <= O->nn + 1; ++j)
    Q = Q + (O->yv[UIDX(j)] - O->yv[UIDX(j - 1)]) * creal(PL(O->u1, UIDX(j))[0]);
  return Q;
}

static void divergence(orc *O) {
  const double dd = O->c.ddthetavi;
#pragma omp parallel for schedule(static)
  for (int c = 0; c < O->ncol; ++c) {
    const int r = c / O->N1h, kx = c % O->N1h;
    cplx kxF = I * O->k1x[kx], kzF = I * O->k1z[r];
    int bs[2];
    const int ns = col_bands(O, c, bs);
    for (int sgi = 0; sgi < ns; ++sgi)
      for (int j = O->bj[bs[sgi]][2][0]; j <= O->bj[bs[sgi]][2][1]; ++j) {
        double th = dd * O->thu[UIDX(j)];
        PL(O->div, PIDX(j))[c] = kxF * PL(O->u1, UIDX(j))[c] + kzF * PL(O->u3, UIDX(j))[c]
                                 + th * (PL(O->u2, UIDX(j))[c] - PL(O->u2, UIDX(j - 1))[c]);
      }
  }
}

static double max_abs_div(const orc *O) {
  double m = 0.0;
  size_t n = (size_t)O->ncol * O->np;
  for (size_t e = 0; e < n; ++e) { double a = cabs(O->div[e]); if (a > m) m = a; }
  return m;
}

int orc_substep(orc *O, int kRK) {
  if (kRK < 1 || kRK > 3) return -1;
  const int nc = O->ncol, N1h = O->N1h;
  const double C1 = O->c.aRK[kRK - 1] / O->c.Re, C2 = -O->c.cRK[kRK - 1];
  const double dR = O->c.dRK[kRK - 1];

  /* RHS0_u1 / RHS0_u3 / RHS0_u2 (littleharsh.f90:635-788) over every band's interior levels */
#pragma omp parallel for schedule(static)
  for (int c = 0; c < nc; ++c) {
    const int r = c / N1h, kx = c % N1h;
    int bs[2];
    const int ns = col_bands(O, c, bs);
    for (int sgi = 0; sgi < ns; ++sgi) {
      const int b = bs[sgi];
      for (int j = O->bj[b][0][0] + 1; j <= O->bj[b][0][1] - 1; ++j) {
        const double a = O->d2u[0 * O->nu + UIDX(j)], bb = O->d2u[1 * O->nu + UIDX(j)];
        const double cc = O->d2u[2 * O->nu + UIDX(j)];
        double dg = O->k2x[kx] + O->k2z[r] + bb;
        cplx L1 = a * PL(O->u1, UIDX(j - 1))[c] + dg * PL(O->u1, UIDX(j))[c] + cc * PL(O->u1, UIDX(j + 1))[c];
        cplx L3 = a * PL(O->u3, UIDX(j - 1))[c] + dg * PL(O->u3, UIDX(j))[c] + cc * PL(O->u3, UIDX(j + 1))[c];
        cplx C3x = -dR * (I * O->k1x[kx]);
        cplx C3z = -dR * (I * O->k1z[r]);
        cplx pj = PL(O->p, PIDX(j))[c];
        PL(O->du1, UIDX(j))[c] = C1 * L1 + C2 * PL(O->Nu1, UIDX(j))[c] + C3x * pj;
        PL(O->du3, UIDX(j))[c] = C1 * L3 + C2 * PL(O->Nu3, UIDX(j))[c] + C3z * pj;
        if (c == 0) PL(O->du1, UIDX(j))[0] = PL(O->du1, UIDX(j))[0] + (-dR * O->mpgx);
      }
      for (int j = O->bj[b][1][0] + 1; j <= O->bj[b][1][1] - 1; ++j) {
        const double a = O->d2v[0 * O->nv + UIDX(j)], bb = O->d2v[1 * O->nv + UIDX(j)];
        const double cc = O->d2v[2 * O->nv + UIDX(j)];
        const double C3 = -dR * O->c.ddthetavi * O->thv[UIDX(j)];
        double dg = O->k2x[kx] + O->k2z[r] + bb;
        cplx L2 = a * PL(O->u2, UIDX(j - 1))[c] + dg * PL(O->u2, UIDX(j))[c] + cc * PL(O->u2, UIDX(j + 1))[c];
        PL(O->du2, UIDX(j))[c] = C1 * L2 + C2 * PL(O->Nu2, UIDX(j))[c]
                                 + C3 * (PL(O->p, PIDX(j + 1))[c] - PL(O->p, PIDX(j))[c]);
      }
    }
  }

  nonlinear(O, kRK);

  /* du += -gRK * Nu (FOU3D.f90:399-410) */
  const double G = -O->c.gRK[kRK - 1];
#pragma omp parallel for schedule(static)
  for (int c = 0; c < nc; ++c) {
    int bs[2];
    const int ns = col_bands(O, c, bs);
    for (int sgi = 0; sgi < ns; ++sgi) {
      const int b = bs[sgi];
      for (int j = O->bj[b][0][0] + 1; j <= O->bj[b][0][1] - 1; ++j) {
        PL(O->du1, UIDX(j))[c] = PL(O->du1, UIDX(j))[c] + G * PL(O->Nu1, UIDX(j))[c];
        PL(O->du3, UIDX(j))[c] = PL(O->du3, UIDX(j))[c] + G * PL(O->Nu3, UIDX(j))[c];
      }
      for (int j = O->bj[b][1][0] + 1; j <= O->bj[b][1][1] - 1; ++j)
        PL(O->du2, UIDX(j))[c] = PL(O->du2, UIDX(j))[c] + G * PL(O->Nu2, UIDX(j))[c];
    }
  }

  if (O->c.ib_enable && O->dny > 0) {
    int d = O->dny, nn = O->nn;
    imm_bounds(O, O->du1, O->phys_u1, O->c.nib_u, O->lu, O->Au, -d + 1, 0, nn + 2, nn + 1 + d);
    imm_bounds(O, O->du2, O->phys_u2, O->c.nib_v, O->lv, O->Av, -d + 1, 0, nn + 1, nn + d);
    imm_bounds(O, O->du3, O->phys_u3, O->c.nib_u, O->lu, O->Au, -d + 1, 0, nn + 2, nn + 1 + d);
  }

  /* solveU_W and solveV per band (littleharsh.f90:791-907, tridLU_3D.f90:55-189, 257-329):
   * rows jlim(1)..jlim(2) of the band, BC rows [1, gridweighting(b,1)] and
   * [gridweighting(b,2), 1] for u and w, identity rows for v */
  const double dt = O->dt;
  const double beta = O->c.bRK[kRK - 1] * dt / O->c.Re;
#pragma omp parallel
  {
    const int nmax = O->nu + 2;
    double *a1 = (double *)malloc(sizeof(double) * nmax), *a2 = (double *)malloc(sizeof(double) * nmax);
    double *a3 = (double *)malloc(sizeof(double) * nmax);
#pragma omp for schedule(static)
    for (int c = 0; c < nc; ++c) {
      int r = c / N1h, kx = c % N1h;
      double k2x = O->k2x[kx], k2z = O->k2z[r];
      int bs[2];
      const int ns = col_bands(O, c, bs);
      for (int sgi = 0; sgi < ns; ++sgi) {
        const int b = bs[sgi];
        int lo = O->bj[b][0][0], hi = O->bj[b][0][1], n = hi - lo + 1;
        PL(O->du1, UIDX(lo))[c] = 0; PL(O->du3, UIDX(lo))[c] = 0;
        for (int j = lo + 1; j <= hi - 1; ++j) {
          PL(O->du1, UIDX(j))[c] = PL(O->u1, UIDX(j))[c] + dt * PL(O->du1, UIDX(j))[c];
          PL(O->du3, UIDX(j))[c] = PL(O->u3, UIDX(j))[c] + dt * PL(O->du3, UIDX(j))[c];
        }
        PL(O->du1, UIDX(hi))[c] = 0; PL(O->du3, UIDX(hi))[c] = 0;
        a1[0] = 0.0; a2[0] = 1.0; a3[0] = O->c.gw[b][0];
        for (int j = lo + 1; j <= hi - 1; ++j) {
          int q = j - lo;
          a1[q] = -beta * O->d2u[0 * O->nu + UIDX(j)];
          a2[q] = 1.0 - beta * (O->d2u[1 * O->nu + UIDX(j)] + k2x + k2z);
          a3[q] = -beta * O->d2u[2 * O->nu + UIDX(j)];
        }
        a1[n - 1] = O->c.gw[b][1]; a2[n - 1] = 1.0; a3[n - 1] = 0.0;
        lu_dec(a1, a2, a3, n);
        for (int j = 0; j < n; ++j) {
          PL(O->u1, UIDX(lo + j))[c] = PL(O->du1, UIDX(lo + j))[c];
          PL(O->u3, UIDX(lo + j))[c] = PL(O->du3, UIDX(lo + j))[c];
        }
        lu_sol(a1, a2, a3, PL(O->u1, UIDX(lo)) + c, n, (size_t)nc);
        lu_sol(a1, a2, a3, PL(O->u3, UIDX(lo)) + c, n, (size_t)nc);

        int vlo0 = O->bj[b][1][0], vhi0 = O->bj[b][1][1], nvv = vhi0 - vlo0 + 1;
        PL(O->du2, UIDX(vlo0))[c] = 0;
        for (int j = vlo0 + 1; j <= vhi0 - 1; ++j)
          PL(O->du2, UIDX(j))[c] = PL(O->u2, UIDX(j))[c] + dt * PL(O->du2, UIDX(j))[c];
        PL(O->du2, UIDX(vhi0))[c] = 0;
        a1[0] = 0.0; a2[0] = 1.0; a3[0] = 0.0;
        for (int j = vlo0 + 1; j <= vhi0 - 1; ++j) {
          int q = j - vlo0;
          a1[q] = -beta * O->d2v[0 * O->nv + UIDX(j)];
          a2[q] = 1.0 - beta * (O->d2v[1 * O->nv + UIDX(j)] + k2x + k2z);
          a3[q] = -beta * O->d2v[2 * O->nv + UIDX(j)];
        }
        a1[nvv - 1] = 0.0; a2[nvv - 1] = 1.0; a3[nvv - 1] = 0.0;
        lu_dec(a1, a2, a3, nvv);
        for (int j = 0; j < nvv; ++j) PL(O->u2, UIDX(vlo0 + j))[c] = PL(O->du2, UIDX(vlo0 + j))[c];
        lu_sol(a1, a2, a3, PL(O->u2, UIDX(vlo0)) + c, nvv, (size_t)nc);
      }
    }
    free(a1); free(a2); free(a3);
  }

  if (O->c.flag_ctpress == 0) flowrate_corr(O, kRK);

  /* solveP (littleharsh.f90:581-633): per band, LUsolP over jlim(1:2, pgrid, b) */
  divergence(O);
  const double dtirk = O->dti / (O->c.aRK[kRK - 1] + O->c.bRK[kRK - 1]);
  for (size_t e = 0; e < (size_t)nc * O->np; ++e) O->psi[e] = dtirk * O->div[e];
  PL(O->psi, PIDX(O->c.N4[0] + 1))[0] = 0.0;
#pragma omp parallel for schedule(static)
  for (int c = 0; c < nc; ++c) {
    int bs[2];
    const int ns = col_bands(O, c, bs);
    for (int sgi = 0; sgi < ns; ++sgi) {
      const int b = bs[sgi];
      const int q0 = PIDX(O->bj[b][2][0]), npn = O->bj[b][2][1] - O->bj[b][2][0] + 1;
      cplx *x = PL(O->psi, q0) + c;
      const double *D = O->DG;
#define DGA(cc, q) D[((size_t)(q0 + (q)) * nc + c) * 3 + (cc) - 1]
      x[0] = x[0] * DGA(2, 0);
      for (int q = 1; q < npn; ++q) x[(size_t)q * nc] = (x[(size_t)q * nc] - DGA(1, q) * x[(size_t)(q - 1) * nc]) * DGA(2, q);
      for (int q = npn - 2; q >= 0; --q) x[(size_t)q * nc] = x[(size_t)q * nc] - DGA(3, q) * x[(size_t)(q + 1) * nc];
#undef DGA
    }
  }
  for (size_t e = 0; e < (size_t)nc * O->np; ++e) O->p[e] = O->p[e] + O->psi[e];

  /* v_corr (littleharsh.f90:956-1052): interior of every band; the wall ghosts of
   * bands 1, 2 (bottom) and 2, 3 (top) from gridweighting_bc; v = 0 at band ends */
  const double dtrk = dt * (O->c.aRK[kRK - 1] + O->c.bRK[kRK - 1]);
  const double dtrk_u2 = dtrk * O->c.ddthetavi;
#pragma omp parallel for schedule(static)
  for (int c = 0; c < nc; ++c) {
    const int r = c / N1h, kx = c % N1h;
    cplx kxc = (cplx)dtrk * (I * O->k1x[kx]);
    cplx kzc = (cplx)dtrk * (I * O->k1z[r]);
    int bs[2];
    const int ns = col_bands(O, c, bs);
    for (int sgi = 0; sgi < ns; ++sgi) {
      const int b = bs[sgi];
      const int lo = O->bj[b][0][0], hi = O->bj[b][0][1];
      for (int j = lo + 1; j <= hi - 1; ++j) {
        PL(O->u1, UIDX(j))[c] = PL(O->u1, UIDX(j))[c] - kxc * PL(O->psi, PIDX(j))[c];
        PL(O->u3, UIDX(j))[c] = PL(O->u3, UIDX(j))[c] - kzc * PL(O->psi, PIDX(j))[c];
      }
      if (b <= 1) {
        PL(O->u1, UIDX(lo))[c] = O->c.gw_bc_u1 * PL(O->u1, UIDX(lo + 1))[c];
        PL(O->u3, UIDX(lo))[c] = O->c.gw_bc_u3 * PL(O->u3, UIDX(lo + 1))[c];
      }
      if (b >= 1) {
        PL(O->u1, UIDX(hi))[c] = O->c.gw_bc_u1 * PL(O->u1, UIDX(hi - 1))[c];
        PL(O->u3, UIDX(hi))[c] = O->c.gw_bc_u3 * PL(O->u3, UIDX(hi - 1))[c];
      }
      const int vlo0 = O->bj[b][1][0], vhi0 = O->bj[b][1][1];
      for (int j = vlo0 + 1; j <= vhi0 - 1; ++j) {
        double f = dtrk_u2 * O->thv[UIDX(j)];
        PL(O->u2, UIDX(j))[c] = PL(O->u2, UIDX(j))[c] - f * (PL(O->psi, PIDX(j + 1))[c] - PL(O->psi, PIDX(j))[c]);
      }
      PL(O->u2, UIDX(vlo0))[c] = 0;
      PL(O->u2, UIDX(vhi0))[c] = 0;
    }
  }
  divergence(O);
  return 0;
}

int orc_step(orc *O) {
  for (int k = 1; k <= 3; ++k)
    if (orc_substep(O, k)) return -1;
  if (O->c.flag_ctpress == 1) O->Qx = flowrateIm(O);
  O->iter += 1;
  return 0;
}

/* ------------------------------------------------------------------------- */
/* state access: host cfield layout f(level, column), level fastest           */
/* ------------------------------------------------------------------------- */
static void put_field(orc *O, cplx *F, int nlev, const double *src) {
  const int nc = O->ncol;
  for (int c = 0; c < nc; ++c)
    for (int l = 0; l < nlev; ++l) {
      const double *s = src + 2 * ((size_t)c * nlev + l);
      F[(size_t)l * nc + c] = s[0] + I * s[1];
    }
}
static void get_field(const orc *O, const cplx *F, int nlev, double *dst) {
  const int nc = O->ncol;
  for (int c = 0; c < nc; ++c)
    for (int l = 0; l < nlev; ++l) {
      double *d = dst + 2 * ((size_t)c * nlev + l);
      cplx v = F[(size_t)l * nc + c];
      d[0] = creal(v); d[1] = cimag(v);
    }
}

int orc_set_state(orc *O, const double *u1, const double *u2, const double *u3, const double *p) {
  if (u1) put_field(O, O->u1, O->nu, u1);
  if (u2) put_field(O, O->u2, O->nv, u2);
  if (u3) put_field(O, O->u3, O->nu, u3);
  if (p) put_field(O, O->p, O->np, p);
  return 0;
}
int orc_get_state(orc *O, double *u1, double *u2, double *u3, double *p) {
  if (u1) get_field(O, O->u1, O->nu, u1);
  if (u2) get_field(O, O->u2, O->nv, u2);
  if (u3) get_field(O, O->u3, O->nu, u3);
  if (p) get_field(O, O->p, O->np, p);
  return 0;
}
/* one band's cfield f(level, column) <-> the wall-grid layout: the band's columns in
 * wall-grid order (columns_i/k, start.f90:1566-1609) over its jlim levels */
static int band_io(orc *O, int band, int put, double *u1, double *u2, double *u3, double *p) {
  if (band < 1 || band > 3) return -1;
  const int b = band - 1;
  cplx *F[4] = {O->u1, O->u2, O->u3, O->p};
  double *H[4] = {u1, u2, u3, p};
  const int grid[4] = {0, 1, 0, 2};
  for (int f = 0; f < 4; ++f) {
    if (!H[f]) continue;
    const int lo = O->bj[b][grid[f]][0], hi = O->bj[b][grid[f]][1], nl = hi - lo + 1;
    const int base = (f == 3) ? PIDX(lo) : UIDX(lo);
    size_t k = 0;
    for (int c = 0; c < O->ncol; ++c) {
      const int isl = !O->mb || O->lng[c];
      if ((b == 1) != isl) continue;
      for (int l = 0; l < nl; ++l) {
        double *h = H[f] + 2 * (k * nl + l);
        cplx *d = &F[f][(size_t)(base + l) * O->ncol + c];
        if (put) *d = h[0] + I * h[1];
        else { h[0] = creal(*d); h[1] = cimag(*d); }
      }
      ++k;
    }
  }
  return 0;
}
int orc_set_band(orc *O, int band, const double *u1, const double *u2, const double *u3, const double *p) {
  return band_io(O, band, 1, (double *)u1, (double *)u2, (double *)u3, (double *)p);
}
int orc_get_band(orc *O, int band, double *u1, double *u2, double *u3, double *p) {
  return band_io(O, band, 0, u1, u2, u3, p);
}

/* Nu1/Nu2/Nu3 of the last substep, same layout (levels of u, v, u) */
int orc_get_nonlinear(orc *O, double *n1, double *n2, double *n3) {
  if (n1) get_field(O, O->Nu1, O->nu, n1);
  if (n2) get_field(O, O->Nu2, O->nv, n2);
  if (n3) get_field(O, O->Nu3, O->nu, n3);
  return 0;
}

int orc_set_scalars(orc *O, const lh_scalars *s) {
  O->t = s->t; O->dt = s->dt; O->dti = s->dti; O->dtc = s->dtc; O->mpgx = s->mpgx;
  O->iter = s->iter;
  /* getini: Qx from the (0,0) mode, QxT = Qx for constant flow rate, initial divergence */
  O->Qx = flowrateIm(O);
  O->QxT = (O->c.flag_ctpress != 1) ? O->Qx : s->QxT;
  divergence(O);
  O->err = max_abs_div(O);
  return 0;
}
int orc_get_scalars(orc *O, lh_scalars *s) {
  O->err = max_abs_div(O);
  s->t = O->t; s->dt = O->dt; s->dti = O->dti; s->dtc = O->dtc; s->err = O->err;
  s->mpgx = O->mpgx; s->QxT = O->QxT; s->Qx = O->Qx; s->iter = O->iter;
  return 0;
}

/* leaves: batched plane transforms, spectral [N2][N1/2+1] <-> physical [G2][G1] */
int orc_four_to_phys(orc *O, const double *spec, double *phys, int nplanes) {
  const size_t ns = (size_t)O->ncol, pp = (size_t)O->G1 * O->G2;
#pragma omp parallel
  {
    pwork w; pwork_init(O, &w);
    pview vf;
    view_of(O, 1, &vf);
#pragma omp for
    for (int q = 0; q < nplanes; ++q)
      four_to_phys_plane(O, &vf, (const cplx *)spec + ns * q, phys + pp * q, &w);
    pwork_free(&w);
  }
  return 0;
}
int orc_phys_to_four(orc *O, const double *phys, double *spec, int nplanes) {
  const size_t ns = (size_t)O->ncol, pp = (size_t)O->G1 * O->G2;
#pragma omp parallel
  {
    pwork w; pwork_init(O, &w);
    pview vf;
    view_of(O, 1, &vf);
#pragma omp for
    for (int q = 0; q < nplanes; ++q)
      phys_to_four_plane(O, &vf, phys + pp * q, (cplx *)spec + ns * q, &w);
    pwork_free(&w);
  }
  return 0;
}

/* ------------------------------------------------------------------------- */
/* statistics (stats.f90:1-250) of the current state over the interior planes  */
/* ------------------------------------------------------------------------- */
static void stats_alloc(orc *O) {
  const int *N3 = O->c.N3, *N4 = O->c.N4;
  int ncl = N4[1] - N4[0];
  if (N4[3] - N4[2] > ncl) ncl = N4[3] - N4[2];
  if (N3[1] - N3[0] > ncl) ncl = N3[1] - N3[0];
  if (N3[3] - N3[2] > ncl) ncl = N3[3] - N3[2];
  const int tx = O->c.ntilex, tz = O->c.ntilez;
  O->st_ncl = ncl;
  O->st_dnx = (tx > 0 && tz > 0) ? O->G1 / tx : 0;
  O->st_dnz = (tx > 0 && tz > 0) ? O->G2 / tz : 0;
  O->st_pl = (double *)calloc((size_t)11 * O->nu, sizeof(double));
  O->st_cd = (double *)calloc((size_t)9 * ncl * (O->st_dnx ? O->st_dnx * O->st_dnz : 1), sizeof(double));
  O->st_pp = (double *)calloc((size_t)2 * O->np, sizeof(double));
  O->st_cd4 = (double *)calloc((size_t)4 * (ncl + 1) * (O->st_dnx ? O->st_dnx * O->st_dnz : 1), sizeof(double));
  O->istat = 0;
  O->nlong = 0;
  for (int c = 0; c < O->ncol; ++c) O->nlong += (!O->mb || O->lng[c]);
  /* band 2's levels: jlim(1:2, grid, midband) (start.f90:1675-1709) */
  const int nl[5] = {O->bj[1][0][1] - O->bj[1][0][0] + 1, O->bj[1][1][1] - O->bj[1][1][0] + 1,
                     O->bj[1][0][1] - O->bj[1][0][0] + 1, O->bj[1][0][1] - O->bj[1][0][0] + 1,
                     O->bj[1][2][1] - O->bj[1][2][0] + 1};
  for (int q = 0; q < 5; ++q) {
    O->sp_nl[q] = nl[q];
    O->sp[q] = (double *)calloc((size_t)nl[q] * O->nlong, sizeof(double));
  }
  O->slip = zalloc((size_t)8 * O->ncol);
}

/* one plane's sums: the plane statistics of stats(), and conddown/condup
 * (stats.f90:109-250) on wall-band planes: tile position (i, k) = (m mod dnx, l mod dnz),
 * level j1 = j - Ny(grid,0) at the bottom, Ny(grid,nband) + 1 - j at the top, where V
 * enters with the sign -1 (xsign) */
static void stats_plane(orc *O, int isU, int j, const double *a, const double *b, const double *c3, int G1,
                        int G2, int fine) {
  const size_t pp = (size_t)G1 * G2;
  double s[3] = {0, 0, 0}, s2[3] = {0, 0, 0};
  double *P = O->st_pl;
  const int q = UIDX(j), nu = O->nu;
  for (size_t e = 0; e < pp; ++e) {
    if (isU) {
      s[0] += a[e]; s2[0] += a[e] * a[e];
      s[1] += c3[e]; s2[1] += c3[e] * c3[e];
      s[2] += a[e] * b[e];
      s2[2] += a[e] * c3[e];
    } else {
      s[0] += b[e]; s2[0] += b[e] * b[e];
      s[1] += b[e] * c3[e];
    }
  }
  if (isU) {
    P[0 * nu + q] += s[0]; P[1 * nu + q] += s2[0]; P[2 * nu + q] += s[1]; P[3 * nu + q] += s2[1];
    P[4 * nu + q] += s[2]; P[5 * nu + q] += s2[2];
  } else {
    P[6 * nu + q] += s[0]; P[7 * nu + q] += s2[0]; P[8 * nu + q] += s[1];
  }
  const int dnx = O->st_dnx, dnz = O->st_dnz;
  if (!dnx || !fine) return;
  const int *NN = isU ? O->c.N4 : O->c.N3;
  int j1, sv;
  if (j <= NN[1]) { j1 = j - NN[0]; sv = 1; }
  else if (j > NN[2]) { j1 = NN[3] + 1 - j; sv = -1; }
  else return;
  const int ncl = O->st_ncl;
#define CD(qty, k, i) O->st_cd[(((size_t)(qty) * ncl + (j1 - 1)) * dnz + (k)) * dnx + (i)]
  for (int l = 0; l < G2; ++l)
    for (int m = 0; m < G1; ++m) {
      const size_t e = (size_t)l * G1 + m;
      const int i = m % dnx, k = l % dnz;
      if (isU) {
        CD(0, k, i) += a[e]; CD(1, k, i) += a[e] * a[e];
        CD(2, k, i) += c3[e]; CD(3, k, i) += c3[e] * c3[e];
        CD(4, k, i) += a[e] * (b[e] * sv); CD(5, k, i) += a[e] * c3[e];
      } else {
        CD(6, k, i) += b[e] * sv; CD(7, k, i) += b[e] * b[e];
        CD(8, k, i) += (b[e] * sv) * c3[e];
      }
    }
#undef CD
}

/* omega_x at v plane j (FOU3D.f90:300-327): -der_z_N(v) + der_yv_h_wx(w) in the plane band's
 * unpadded N1 x N2 layout, four_to_phys_N (FOU3D.f90:786-804: z backward complex transform
 * of the N1/2+1 x-modes, no zeroed row, then x backward real transform), summed over the
 * N1 x N2 points in the order of stats.f90:56-63 (k outer, i inner). */
static void wx_plane(orc *O, int j, double *phys, pwork *w, double *ps, double *ps2) {
  const int fine = fine_v(O, j);
  const int N1 = fine ? O->N1 : O->N1c, N2 = fine ? O->N2 : O->N2c, N1h = N1 / 2 + 1;
  const fftplan *px = fine ? &O->pxN : &O->pxNc, *pz = fine ? &O->pzN : &O->pzNc;
  pview v;
  view_of(O, fine, &v);
  const int q = UIDX(j);
  const double fy = O->thv[q] * O->c.ddthetavi;
  for (int kx = 0; kx < N1h; ++kx) {
    for (int r = 0; r < N2; ++r) {
      const size_t c = vcol(O, &v, r, kx);
      const int fr = (int)(c / O->N1h);
      const cplx dz = (I * O->k1z[fr]) * PL(O->u2, q)[c];
      const cplx dy = (PL(O->u3, q + 1)[c] - PL(O->u3, q)[c]) * fy;
      w->line[r] = -dz + dy;
    }
    fft_inplace(pz, w->line, +1, w->tmp);
    for (int l = 0; l < N2; ++l) w->A[(size_t)l * N1h + kx] = w->line[l];
  }
  for (int l = 0; l < N2; ++l) {
    const cplx *a = w->A + (size_t)l * N1h;
    for (int k = 0; k < N1; ++k) w->line[k] = 0;
    for (int k = 0; k <= N1 / 2; ++k) {
      cplx ak = a[k];
      if (k == 0 || k == N1 / 2) ak = creal(ak);
      w->line[k] = ak;
      if (k > 0 && k < N1 / 2) w->line[N1 - k] = conj(ak);
    }
    fft_inplace(px, w->line, +1, w->tmp);
    for (int m = 0; m < N1; ++m) phys[(size_t)l * N1 + m] = creal(w->line[m]);
  }
  double s = 0, s2 = 0;
  for (int l = 0; l < N2; ++l)
    for (int m = 0; m < N1; ++m) {
      const double x = phys[(size_t)l * N1 + m];
      s += x;
      s2 += x * x;
    }
  *ps = s;
  *ps2 = s2;
}

/* p plane j of the wall bands: N(4,0)+1 .. N(4,1)-1 and N(4,2)+2 .. N(4,3), the pgrid
 * plane ranges of the bottom and top bands (start.f90:1995-2049); the others are core-band
 * planes */
static inline int fine_p(const orc *O, int j) { return !O->mb || j <= O->c.N4[1] - 1 || j >= O->c.N4[2] + 2; }

/* conddown1 / condup1 with xsign 1 (stats.f90:109-138, 178-210) of one physical plane on
 * the G1 x G2 grid: tile position (i mod dnx, l mod dnz), level j1 (0 = the first plane of
 * the band, the file's level 0), into the pair qa, qa + 1 of st_cd4 */
static void cond_plane(orc *O, int qa, int j1, const double *f, int G1, int G2) {
  const int dnx = O->st_dnx, dnz = O->st_dnz, ncl1 = O->st_ncl + 1;
  double *m = O->st_cd4 + ((size_t)qa * ncl1 + j1) * dnz * dnx;
  double *m2 = O->st_cd4 + ((size_t)(qa + 1) * ncl1 + j1) * dnz * dnx;
  for (int l = 0; l < G2; ++l)
    for (int i = 0; i < G1; ++i) {
      const double x = f[(size_t)l * G1 + i];
      const size_t e = (size_t)(l % dnz) * dnx + (i % dnx);
      m[e] += x;
      m2[e] += x * x;
    }
}

/* Pressure statistics (stats.f90:43-50 and the PmC / wxmC calls, stats.f90:91-92, 100-101). The
 * reference sums ppPL, which holds the spectral packing of p left by record_out
 * (FOU3D.f90:156-157); here the physical pressure is formed the way the velocities are
 * (four_to_phys on the plane's dealiased grid) and summed over its points: every p plane
 * for P, P^2 (st_pp [2][np]), the wall-band planes for the conditioned sums (st_cd4 pairs
 * 0, 1). omega_x (FOU3D.f90:300-327) of the wall-band v planes j = N(3,0) .. N(3,1) and
 * N(3,2)+1 .. N(3,3)+1 is transformed on the same dealiased grid (its spectrum padded like
 * the velocities') and conditioned into pairs 2, 3. */
static void pressure_wx_stats(orc *O, double *f, pwork *w) {
  const int *N3 = O->c.N3, *N4 = O->c.N4;
  for (int j = N4[0] + 1; j <= N4[3]; ++j) {
    pview v;
    const int fine = fine_p(O, j);
    view_of(O, fine, &v);
    four_to_phys_plane(O, &v, PL(O->p, PIDX(j)), f, w);
    const size_t pp = (size_t)v.G1 * v.G2;
    double s = 0, s2 = 0;
    for (size_t e = 0; e < pp; ++e) {
      s += f[e];
      s2 += f[e] * f[e];
    }
    O->st_pp[PIDX(j)] += s;
    O->st_pp[(size_t)O->np + PIDX(j)] += s2;
    if (!O->st_dnx || !fine) continue;
    if (j <= N4[1] - 1) cond_plane(O, 0, j - N4[0] - 1, f, v.G1, v.G2);
    else if (j >= N4[2] + 2) cond_plane(O, 0, N4[3] - j, f, v.G1, v.G2);
  }
  if (!O->st_dnx) return;
  cplx *ws = zalloc((size_t)O->ncol);
  pview v;
  view_of(O, 1, &v);
  for (int j = N3[0]; j <= N3[3] + 1; ++j) {
    int j1;
    if (j <= N3[1]) j1 = j - N3[0];
    else if (j > N3[2]) j1 = N3[3] + 1 - j;
    else continue;
    const int q = UIDX(j);
    const double fy = O->thv[q] * O->c.ddthetavi;
    for (int c = 0; c < O->ncol; ++c) {
      const cplx dz = (I * O->k1z[c / O->N1h]) * PL(O->u2, q)[c];
      ws[c] = -dz + (PL(O->u3, q + 1)[c] - PL(O->u3, q)[c]) * fy;
    }
    four_to_phys_plane(O, &v, ws, f, w);
    cond_plane(O, 2, j1, f, v.G1, v.G2);
  }
  free(ws);
}

/* spectra (spectra.f90:1-56): buildsp / buildspUV over band 2's columns (the long
 * columns, in the order of columns_long_list) and levels, sp(j, column) += |u|^2,
 * spUV += Re u1 Re u2_itp + Im u1 Im u2_itp (u2_itp: v interpolated to the centres) */
static void spectra_accumulate(orc *O) {
  const int ulo = UIDX(O->bj[1][0][0]), vlo = UIDX(O->bj[1][1][0]), plo = PIDX(O->bj[1][2][0]);
  int k = 0;
  for (int c = 0; c < O->ncol; ++c) {
    if (O->mb && !O->lng[c]) continue;
    double *sU = O->sp[0] + (size_t)k * O->sp_nl[0], *sV = O->sp[1] + (size_t)k * O->sp_nl[1];
    double *sW = O->sp[2] + (size_t)k * O->sp_nl[2], *sUV = O->sp[3] + (size_t)k * O->sp_nl[3];
    double *sP = O->sp[4] + (size_t)k * O->sp_nl[4];
    for (int l = 0; l < O->sp_nl[0]; ++l) {
      const cplx a = PL(O->u1, ulo + l)[c], b = PL(O->u3, ulo + l)[c], v = PL(O->u2i, ulo + l)[c];
      sU[l] = sU[l] + creal(a) * creal(a) + cimag(a) * cimag(a);
      sW[l] = sW[l] + creal(b) * creal(b) + cimag(b) * cimag(b);
      sUV[l] = sUV[l] + creal(a) * creal(v) + cimag(a) * cimag(v);
    }
    for (int l = 0; l < O->sp_nl[1]; ++l) {
      const cplx a = PL(O->u2, vlo + l)[c];
      sV[l] = sV[l] + creal(a) * creal(a) + cimag(a) * cimag(a);
    }
    for (int l = 0; l < O->sp_nl[4]; ++l) {
      const cplx a = PL(O->p, plo + l)[c];
      sP[l] = sP[l] + creal(a) * creal(a) + cimag(a) * cimag(a);
    }
    ++k;
  }
}

/* sl_stats / inst_sl_stats (sl_stats2.f90:33-121, inst_sl_stats.f90:1-62) at the two wall
 * faces jlim(1, vgrid, 2) and jlim(2, vgrid, 2), every column of the wall-band grid (the
 * columns of bands 1+2 at the bottom, 2+3 at the top): u1_itp, du1dy, u3_itp, du3dy with
 * du/dy = (u(j+1) - u(j)) dthdyv(j) ddthetavi, negated at the top. out: [2][4][ncol];
 * acc: add (sl_stats) or overwrite (inst_sl_stats). interp_all must have run. */
static void slip_planes(orc *O, cplx *out, int acc) {
  const int jw[2] = {O->c.N3[0], O->c.N3[3] + 1};
  const double sg[2] = {1.0, -1.0};
  const size_t nc = (size_t)O->ncol;
  for (int w = 0; w < 2; ++w) {
    const int q = UIDX(jw[w]);
    const double fy = O->thv[q] * O->c.ddthetavi;
    cplx *o = out + (size_t)w * 4 * nc;
    for (size_t c = 0; c < nc; ++c) {
      const cplx v[4] = {PL(O->u1i, q)[c], sg[w] * ((PL(O->u1, q + 1)[c] - PL(O->u1, q)[c]) * fy),
                         PL(O->u3i, q)[c], sg[w] * ((PL(O->u3, q + 1)[c] - PL(O->u3, q)[c]) * fy)};
      for (int f = 0; f < 4; ++f) o[f * nc + c] = acc ? o[f * nc + c] + v[f] : v[f];
    }
  }
}

int orc_stats_accumulate(orc *O) {
  if (!O->st_pl) stats_alloc(O);
  interp_all(O);
  const size_t ppF = (size_t)O->G1 * O->G2;
  double *f1 = (double *)malloc(sizeof(double) * ppF), *f2 = (double *)malloc(sizeof(double) * ppF);
  double *f3 = (double *)malloc(sizeof(double) * ppF);
  pwork w; pwork_init(O, &w);
  for (int j = O->c.N4[0] + 1; j <= O->c.N4[3]; ++j) {
    pview v;
    const int fine = fine_u(O, j);
    view_of(O, fine, &v);
    four_to_phys_plane(O, &v, PL(O->u1, UIDX(j)), f1, &w);
    four_to_phys_plane(O, &v, PL(O->u2i, UIDX(j)), f2, &w);
    four_to_phys_plane(O, &v, PL(O->u3, UIDX(j)), f3, &w);
    stats_plane(O, 1, j, f1, f2, f3, v.G1, v.G2, fine);
  }
  for (int j = O->c.N3[0] + 1; j <= O->c.N3[3]; ++j) {
    pview v;
    const int fine = fine_v(O, j);
    view_of(O, fine, &v);
    four_to_phys_plane(O, &v, PL(O->u1i, UIDX(j)), f1, &w);
    four_to_phys_plane(O, &v, PL(O->u2, UIDX(j)), f2, &w);
    four_to_phys_plane(O, &v, PL(O->u3i, UIDX(j)), f3, &w);
    stats_plane(O, 0, j, f1, f2, f3, v.G1, v.G2, fine);
  }
  for (int j = O->c.N3[0]; j <= O->c.N3[3] + 1; ++j) {
    double s = 0, s2 = 0;
    wx_plane(O, j, f1, &w, &s, &s2);
    O->st_pl[9 * (size_t)O->nu + UIDX(j)] += s;
    O->st_pl[10 * (size_t)O->nu + UIDX(j)] += s2;
  }
  pressure_wx_stats(O, f1, &w);
  pwork_free(&w);
  free(f1); free(f2); free(f3);
  spectra_accumulate(O);
  slip_planes(O, O->slip, 1);
  O->istat += 1;
  return 0;
}

int orc_stats_get(orc *O, double *plane, double *cond, int64_t *istat, int *dims) {
  if (!O->st_pl) stats_alloc(O);
  if (plane) memcpy(plane, O->st_pl, sizeof(double) * 11 * (size_t)O->nu);
  const size_t nc = (size_t)9 * O->st_ncl * (O->st_dnx ? O->st_dnx * O->st_dnz : 1);
  if (cond && O->st_dnx) memcpy(cond, O->st_cd, sizeof(double) * nc);
  if (istat) *istat = O->istat;
  if (dims) { dims[0] = O->st_ncl; dims[1] = O->st_dnx; dims[2] = O->st_dnz; }
  return 0;
}

/* pressure plane sums [2][np] and conditioned P, P^2, omega_x, omega_x^2 [4][ncl + 1][dnz][dnx]
 * (NULL skips one; cond only with tiles) */
int orc_stats_get_pw(orc *O, double *pplane, double *cond4) {
  if (!O->st_pl) stats_alloc(O);
  if (pplane) memcpy(pplane, O->st_pp, sizeof(double) * 2 * (size_t)O->np);
  if (cond4 && O->st_dnx)
    memcpy(cond4, O->st_cd4, sizeof(double) * 4 * (size_t)(O->st_ncl + 1) * O->st_dnx * O->st_dnz);
  return 0;
}

/* sp(level, long column) of U, V, W, UV, P (NULL skips one); nl: band 2's level counts */
int orc_spectra_get(orc *O, double *sU, double *sV, double *sW, double *sUV, double *sP, int *nl, int *nlong) {
  if (!O->st_pl) stats_alloc(O);
  double *dst[5] = {sU, sV, sW, sUV, sP};
  for (int q = 0; q < 5; ++q) {
    if (dst[q]) memcpy(dst[q], O->sp[q], sizeof(double) * (size_t)O->sp_nl[q] * O->nlong);
    if (nl) nl[q] = O->sp_nl[q];
  }
  if (nlong) *nlong = O->nlong;
  return 0;
}

/* accumulated slip statistics [2][4][ncol] complex (NULL skips) */
int orc_slip_get(orc *O, double *acc) {
  if (!O->st_pl) stats_alloc(O);
  if (acc) memcpy(acc, O->slip, sizeof(cplx) * 8 * (size_t)O->ncol);
  return 0;
}

/* instantaneous slip planes of the current state [2][4][ncol] complex */
int orc_slip_planes(orc *O, double *out) {
  interp_all(O);
  slip_planes(O, (cplx *)out, 0);
  return 0;
}

int orc_stats_reset(orc *O) {
  if (!O->st_pl) stats_alloc(O);
  memset(O->st_pl, 0, sizeof(double) * 11 * (size_t)O->nu);
  memset(O->st_cd, 0, sizeof(double) * 9 * (size_t)O->st_ncl * (O->st_dnx ? O->st_dnx * O->st_dnz : 1));
  memset(O->st_pp, 0, sizeof(double) * 2 * (size_t)O->np);
  memset(O->st_cd4, 0, sizeof(double) * 4 * (size_t)(O->st_ncl + 1) * (O->st_dnx ? O->st_dnx * O->st_dnz : 1));
  for (int q = 0; q < 5; ++q) memset(O->sp[q], 0, sizeof(double) * (size_t)O->sp_nl[q] * O->nlong);
  memset(O->slip, 0, sizeof(cplx) * 8 * (size_t)O->ncol);
  O->istat = 0;
  return 0;
}

int orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}
