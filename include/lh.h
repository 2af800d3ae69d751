/*
 * lh.h — C ABI of the GB300 RK3 substep of the "littleharsh" channel DNS.
 *
 * The reference (Fortran 90 + MPI) has no plugin API: its boundary is the set of
 * Fortran subroutines `program littleharsh` calls once per RK3 substep
 * (littleharsh.f90:174-217), with all shared data in `module declaration`
 * (declaration.f90). This header replaces that boundary with plain C entry points
 * that a Fortran host binds through an ISO_C_BINDING interface module and that
 * the Python package binds through ctypes.
 *
 * Conventions
 *  - A "level" j is a reference y-index. u/w live on levels N(4,0)..N(4,3)+1
 *    (ghosts included), v on N(3,0)..N(3,3)+1 (walls included), p/psi/div on
 *    N(4,0)+1..N(4,3). N(3,0) = N(4,0) = -dny (dny > 0 only with posts).
 *  - Spectral state arrays on the host use the reference's `type(cfield)` layout
 *    of the midband (long-column) band: f(level, column), complex(8),
 *    column-major with the level fastest, one column per (kx, kz) mode in the
 *    order of proc_lims_columns with one process (start.f90:1610-1631):
 *    column = ikz * (N1/2+1) + ikx, ikz = 0..N2-1 in k1F_z order.
 *  - All entry points return LH_OK or a negative error code; lh_last_error()
 *    returns a message for the last failure on that handle, lh_last_error(NULL)
 *    the last failure on the calling thread (e.g. of lh_create).
 *  - One handle per host thread. No internal threads.
 */
#ifndef LH_H
#define LH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LH_ABI_VERSION 2

enum {
  LH_OK = 0,
  LH_EINVAL = -1,      /* bad argument or unsupported configuration */
  LH_ENONFINITE = -2,  /* a NaN/Inf appeared in the state (blow-up guard) */
  LH_ETIMEOUT = -3,    /* a bounded device wait gave up */
  LH_ECUDA = -4,       /* a CUDA runtime call failed */
  LH_ENOMEM = -5
};

enum {
  LH_PREC_FP64 = 0,    /* plain form: every kernel in FP64 */
  LH_PREC_MIXED = 1    /* precision form: FP32 transforms/products, FP64 state, solves and (0,0) mode */
};

enum {
  LH_NONLIN_PRODUCTS = 0,  /* FFT products (ops_in_planes2) */
  LH_NONLIN_TRIADS = 1     /* triad-list convolution (ops_in_planes) */
};

/* Everything the substep reads from `module declaration`, for one channel whose
 * three bands share one x/z resolution (start.f90:36-691 computes these). */
typedef struct lh_config {
  int32_t abi_version;            /* LH_ABI_VERSION */
  int32_t precision;              /* LH_PREC_* */
  int32_t N1, N2;                 /* retained Fourier modes N(1,b), N(2,b) */
  int32_t Ngal1, Ngal2;           /* physical points Ngal(1,b), Ngal(2,b) */
  int32_t dny;                    /* depth of the immersed region: N(3,0) = N(4,0) = -dny */
  int32_t nn;                     /* N(3,nband) before the immersed region is added (= ny-2) */
  int32_t N3[4], N4[4];           /* band limits N(3,0:3), N(4,0:3) */
  int32_t nyu, nyv;               /* number of u levels and v levels */
  const double *yu, *yv;          /* [nyu], [nyv] : yu(j), yv(j) at index j+dny */
  const double *dthdyu, *dthdyv;  /* [nyu], [nyv] */
  const double *dyu2i, *dyv2i;    /* [3][nyu], [3][nyv] : dyu2i(c, j) at [c-1][j+dny] */
  const double *k1x, *k2x;        /* [N1/2+1] : Im k1F_x(i), k2F_x(i) */
  const double *k1z, *k2z;        /* [N2]     : Im k1F_z(k), k2F_z(k) */
  double Re, CFL, dtv, ddthetavi, dthetavi, alp, bet, Kib;
  double aRK[3], bRK[3], cRK[3], dRK[3], gRK[3];
  double gw[3][2];                /* gridweighting(band, 1:2) */
  double gw_interp[3][2];         /* gridweighting_interp(band, 1:2) */
  double gw_bc_u1, gw_bc_u3;      /* gridweighting_bc_u1/u3 */
  int32_t flag_ctpress;           /* 0 constant flow rate, 1 constant pressure gradient */
  int32_t ib_enable;              /* apply the immersed-boundary forcing */
  int32_t nib_u, nib_v;           /* number of listed solid points, u/w grid and v grid */
  const int32_t *list_ib_u;       /* [nib_u][6] : i, k, j, i1, k1, j1 (i,k 1-based physical) */
  const int32_t *list_ib_v;       /* [nib_v][6] */
  const double *A_ib_u, *A_ib_v;  /* [nib_u], [nib_v] */
  /* Nonlinear-term form. LH_NONLIN_PRODUCTS: pseudo-spectral products with 3/2
   * dealiasing (ops_in_planes2, FOU3D.f90:2090-2251). LH_NONLIN_TRIADS: the
   * as-run triad-list convolution (ops_in_planes + nonlinInter, FOU3D.f90:1724-2088)
   * over the interaction lists that nonlinRead loads (start.f90:2983-3069). */
  int32_t nonlin_form;            /* LH_NONLIN_* */
  int32_t triad_nx, triad_nz;     /* list header: largest |kx| and |kz| index (N1/2-1, N2/2-1) */
  int32_t triad_nsets;            /* number of lists files (one per distinct plane) */
  const int64_t *triad_off;       /* [nsets][9] triad offset of list `type` 1..9 in triad_data */
  const int64_t *triad_len;       /* [nsets][9] number of triads L of that list */
  const int8_t *triad_data;       /* list of L triads at offset o: bytes 4*o .. 4*o+4L-1, stored as
                                     the lists file stores it (column-major list(L,4)): la[L],
                                     ka[L], lp[L], kp[L]. Lists may share storage. */
  const int32_t *triad_set_u;     /* [nyu] set (0-based) of each u level, -1 on the ghost levels */
  const int32_t *triad_set_v;     /* [nyv] set of each v level, -1 on the wall levels */
  /* Multiblock: N1, N2, Ngal1, Ngal2 above are the wall bands' (bands 1 and 3,
   * N(1:2,1), Ngal(1:2,1)); these are the core band's (band 2). Equal values give a
   * single-resolution channel. The core modes must be a subset of the wall modes. */
  int32_t N1c, N2c, Ngal1c, Ngal2c;
  /* Post tiles of the wall texture (ntilex, ntilez of boundary_post_coll.f90; 0 = none):
   * the tile-conditioned statistics average over them. */
  int32_t ntilex, ntilez;
} lh_config;

/* Scalars of the time integration (module declaration: t, dt, dti, dtc, err, mpgx, QxT, Qx, iter).
 * err = max |div u| of the state (error(), littleharsh.f90:342-375): the reference
 * reads it only at the start of a step, so it is refreshed at the end of the third
 * substep (and by lh_set_scalars). */
typedef struct lh_scalars {
  double t, dt, dti, dtc, err, mpgx, QxT, Qx;
  int64_t iter;
} lh_scalars;

typedef struct lh_handle lh_handle;

/* Replaces `start` + the allocations of littleharsh.f90:110-152 and the pressure
 * factorisation LU_buildP/LU_decP (start.f90:656-658, tridLU_3D.f90:333-518).
 * The config's arrays are copied; the caller may free them afterwards. */
int lh_create(const lh_config *cfg, lh_handle **out);
int lh_destroy(lh_handle *h);
const char *lh_last_error(lh_handle *h);

/* Upload / download the state (u1, u2, u3, p) in the host cfield layout
 * (replaces getini's planes_to_modes_UVP, start.f90:2226-2229, and the
 * modes_to_planes_UVP feeding record_out, littleharsh.f90:398-402).
 * u1, u3: complex(8) [ncols][nyu]; u2: [ncols][nyv]; p: [ncols][nyu-2]
 * (interleaved re/im doubles, level fastest). Any pointer may be NULL to skip
 * that field. Blocking. */
int lh_upload_state(lh_handle *h, const double *u1, const double *u2,
                    const double *u3, const double *p);
int lh_download_state(lh_handle *h, double *u1, double *u2, double *u3, double *p);
/* The same, queued without blocking: an upload takes effect before the steps queued after
 * it, a download reads the state left by the steps queued before it. The host->device
 * copy runs on a copy stream of its own (overlapping the steps already queued) and the
 * device->host copy on another (overlapping the steps queued later). The host arrays must
 * stay valid, and unread/unwritten by the host, until lh_synchronize; page-locked host
 * memory makes the copies asynchronous. Two full-state staging buffers are allocated on
 * first use. Single-resolution channels only. */
int lh_upload_state_async(lh_handle *h, const double *u1, const double *u2,
                          const double *u3, const double *p);
int lh_download_state_async(lh_handle *h, double *u1, double *u2, double *u3, double *p);

/* Per-band state, the reference's cfield of one band (u1(iband)%f etc.,
 * declaration.f90:137-139): band 1 (bottom wall band) and 3 (top) hold the short
 * columns (wall-band modes the core band lacks) over their jlim levels
 * (start.f90:1675-1709); band 2 the long columns over all levels. Columns in the
 * order of columns_i/k with one process (start.f90:1566-1609): row-major over
 * (kz index, kx) of the wall-band modes. Shapes [ncols_b][nlev_b] complex(8),
 * nlev_b = jlim(2,grid,b) - jlim(1,grid,b) + 1 for u/w, v and p. Bands 1 and 3
 * are empty for a single-resolution channel, and band 2 is then lh_upload_state's
 * layout. Blocking. */
int lh_upload_band(lh_handle *h, int band, const double *u1, const double *u2,
                   const double *u3, const double *p);
int lh_download_band(lh_handle *h, int band, double *u1, double *u2, double *u3, double *p);
/* The same, queued without blocking (as lh_upload_state_async / lh_download_state_async):
 * each band has its own staging region, so the copies of one band overlap the scatter of
 * another and the steps queued around them. */
int lh_upload_band_async(lh_handle *h, int band, const double *u1, const double *u2,
                         const double *u3, const double *p);
int lh_download_band_async(lh_handle *h, int band, double *u1, double *u2, double *u3, double *p);

/* Scalars: lh_set_scalars also (re)computes Qx, and QxT when flag_ctpress == 0,
 * as getini does (start.f90:2170-2176), and the initial divergence. */
int lh_set_scalars(lh_handle *h, const lh_scalars *s);
int lh_get_scalars(lh_handle *h, lh_scalars *s);

/* One record of the history file (hist_*.dat), the scalar part of record_out
 * (FOU3D.f90:3040-3070): with flag_ctpress == 0 the file record is
 * flag_ctpress, iter, t, dtv, dtc, dt, err, Qx, QxT, mpgx, dgx, Umax, Uslip, and with
 * flag_ctpress == 1 QxT and dgx are left out. */
typedef struct lh_history {
  int32_t flag_ctpress, iter;
  double t, dtv, dtc, dt, err, Qx, QxT, mpgx, dgx, Umax, Uslip;
} lh_history;
/* Forms the record of the current state as record_out does at an output step: Qx by
 * flowrateIm (which also refreshes the scalar Qx), Umax by maxvel (littleharsh.f90:511-527)
 * and the slip velocity of mode (0,0); dgx is the last flowrate_corr correction. Called
 * between steps, after lh_step n it is the record the reference writes at iteration n.
 * Blocking. */
int lh_history_record(lh_handle *h, lh_history *out);

/* One RK3 substep kRK = 1..3: RHS0_u1/u2/u3, nonlinear, solveU_W, solveV,
 * [meanflow_ctU], solveP, v_corr (littleharsh.f90:176-215). Asynchronous on the
 * handle's stream; dt and err stay on the device. */
int lh_substep(lh_handle *h, int kRK);

/* One full step: three substeps, then meanflow_ctP when flag_ctpress == 1,
 * then iter += 1 (littleharsh.f90:174-226). Replayed from a CUDA graph after
 * the first call. Asynchronous. */
int lh_step(lh_handle *h);

/* Block until the handle's work is done; returns LH_ENONFINITE if the blow-up
 * guard fired (max|div| or a velocity became non-finite). */
int lh_synchronize(lh_handle *h);

/* Device-resident views for callers that keep the state on the GPU (e.g. a
 * PyTorch host). Plane-major layout [level][kz][kx] complex128. */
int lh_device_state(lh_handle *h, void **u1, void **u2, void **u3, void **p);
/* The CUDA stream the handle runs on (cudaStream_t as void*). */
void *lh_stream(lh_handle *h);

/* ---- leaves, for per-kernel parity checks (device pointers, handle's stream) ----
 * Batched x/z transforms of `nplanes` spectral planes [N2][N1/2+1] complex to
 * physical planes [Ngal2][Ngal1] real and back: four_to_phys_du / phys_to_four_du
 * (FOU3D.f90:766-781, 2253-2272) over cft/rft (cft_buff.f:1-65, rft_buff.f:24-86). */
int lh_four_to_phys(lh_handle *h, const void *spec, void *phys, int nplanes);
int lh_phys_to_four(lh_handle *h, const void *phys, void *spec, int nplanes);

/* ---- statistics (stats.f90, spectra.f90, sl_stats2.f90), accumulated on the device ----
 * lh_stats_accumulate adds the current state's statistics (istat += 1), as the statistics
 * step of nonlinear does at kRK = 1 when flagst is set (FOU3D.f90:127-130, 298-373):
 * stats(), spectra() and sl_stats() together.
 * Plane sums (stats.f90:1-107), per level:
 *   0 U, 1 U^2, 2 W, 3 W^2, 4 U V, 5 U W   (interior u levels; V interpolated to the centres)
 *   6 V, 7 V^2, 8 V W                      (interior v levels; W interpolated to the faces)
 *   9 omega_x, 10 omega_x^2                (every v level: omega_x = -dv/dz + dw/dy on the
 *                                           plane's unpadded N1 x N2 grid, FOU3D.f90:300-327)
 * and the sums 0-8 conditioned on the position inside a post tile (conddown1/2, condup1/2,
 * stats.f90:109-250): wall-band planes only, indexed by the distance j1 = 1.. from the
 * wall, the top band mirrored onto the bottom with the sign of V flipped. Sums 0-8 are in
 * FP64 from planes in the form's transform precision; 9-10 from the FP64 state. The
 * pressure sums and the tile-conditioned omega_x sums are accumulated by the same call and
 * read with lh_stats_get_pw. */
int lh_stats_accumulate(lh_handle *h);
/* zeroes every accumulator (plane, conditioned, spectra, slip) and istat */
int lh_stats_reset(lh_handle *h);
/* Pressure plane sums P, P^2 (stats.f90:43-50) and the tile-conditioned P, P^2, omega_x,
 * omega_x^2 (PmC, P2mC, wxmC, wx2mC: stats.f90:91-92, 100-101), from the FP64 state. The
 * reference sums ppPL, which holds the spectral packing of p left by record_out
 * (FOU3D.f90:156-157), and conditions wx, allocated (N1+2) x N2, through an igal x kgal dummy;
 * here p is transformed the way the velocities are (the plane's dealiased grid; the p planes
 * of the wall bands are N(4,0)+1 .. N(4,1)-1 and N(4,2)+2 .. N(4,3), the others core planes)
 * and omega_x of the wall-band v planes N(3,0) .. N(3,1), N(3,2)+1 .. N(3,3)+1 on the same
 * dealiased grid, conditioned like the velocities with xsign 1.
 * pplane: [2][nyu - 2] (p level index); cond4: [4][ncl + 1][dnz][dnx], level j1 = 0 .. ncl
 * (0: the first plane from the wall, the file's level 0); NULL skips one. Blocking. */
int lh_stats_get_pw(lh_handle *h, double *pplane, double *cond4);
/* ncl: conditioned levels; dnx, dnz: tile size in physical points (0 without tiles) */
int lh_stats_dims(lh_handle *h, int *ncl, int *dnx, int *dnz);
/* plane: [11][nyu] (u-level quantities at u index j+dny, v-level ones at v index j+dny);
 * cond: [9][ncl][dnz][dnx] (may be NULL); istat: number of accumulations. Blocking. */
int lh_stats_get(lh_handle *h, double *plane, double *cond, int64_t *istat);

/* Spectra (spectra.f90:1-56, buildsp / buildspUV): over band 2 (the long columns, in the
 * order of columns_long_list, start.f90:1606-1631) and band 2's levels jlim(1:2, grid, 2),
 * sp(j, column) += |u|^2 of U, V, W, P, and spUV += Re u1 Re v + Im u1 Im v with v
 * interpolated to the centres. nlev: [5] level counts of U, V, W, UV, P; nlong: columns. */
int lh_spectra_dims(lh_handle *h, int *nlev, int *nlong);
/* each array [nlong][nlev[q]] (level fastest, the layout of sp(j, column)); NULL skips one.
 * Folding onto |kz| for the file is the host's (recvwrspec, spectra.f90:124-182). Blocking. */
int lh_spectra_get(lh_handle *h, double *spU, double *spV, double *spW, double *spUV, double *spP);

/* Slip statistics (sl_stats2.f90:33-121) at the wall faces jlim(1, vgrid, 2) (bottom) and
 * jlim(2, vgrid, 2) (top), every mode of the wall-band grid: u1 and u3 interpolated to the
 * face and du1/dy, du3/dy = (u(j+1) - u(j)) dthdyv(j) ddthetavi, negated at the top.
 * acc: [2 faces][4: u1, du1dy, u3, du3dy][N2][N1+2] (re/im of x-modes 0..N1/2, the
 * bslip_*_M layout), accumulated by lh_stats_accumulate. Blocking. */
int lh_slip_get(lh_handle *h, double *acc);
/* the same four planes of the current state, not accumulated (inst_sl_stats.f90:1-62) */
int lh_slip_planes(lh_handle *h, double *out);

/* Number of CUDA kernel launches issued by the handle since creation (graph
 * replays count every kernel node). */
int64_t lh_kernel_launches(lh_handle *h);

/* Diagnostic, no counterpart in the reference: run `nsteps` steps eagerly (not
 * from the graph) with CUDA events around every launch on the handle's stream and
 * return the time per kernel name. Advances the state like lh_step. */
typedef struct lh_kernel_time {
  char name[32];
  int32_t launches;
  double total_ms;
} lh_kernel_time;
int lh_profile_steps(lh_handle *h, int nsteps, lh_kernel_time *out, int nmax, int *nout);

/* Autotuner, no counterpart in the reference: times the candidate block sizes of
 * the one-thread-per-column kernels (solves, pressure) on this handle's channel,
 * keeps the fastest, and restores the state. Allocates a temporary copy of the
 * state. Call before the first lh_step (or it recaptures the step graph). */
int lh_autotune(lh_handle *h);

/* The configuration lh_autotune chose (or the defaults): threads per block of the u/w
 * Helmholtz, v Helmholtz and pressure kernels, then the levels each stages ahead through shared
 * memory (0: the variant that prefetches into registers). cfg: [6]. No counterpart in the
 * reference. */
int lh_get_tuning(lh_handle *h, int32_t *cfg);

/* Batches (the ensemble form; no counterpart in the reference): one RK3 step of
 * each of `n` independent channels, of any sizes, captured once into a single
 * CUDA graph in which every channel is a branch on its own stream, and replayed
 * by lh_batch_step with one graph launch. The handles stay owned by the caller and
 * must outlive the batch; upload their states before lh_batch_create. */
typedef struct lh_batch lh_batch;
int lh_batch_create(lh_handle *const *handles, int n, lh_batch **out);
int lh_batch_step(lh_batch *b);
int lh_batch_synchronize(lh_batch *b);
int lh_batch_destroy(lh_batch *b);
void *lh_batch_stream(lh_batch *b);

/* ---- four_to_phys without a handle and without allocating ----
 * No counterpart in the reference. For callers that cannot call cudaMalloc: hosts
 * that own every byte of device memory themselves (a solver that sizes HBM once at
 * start-up and forbids later allocation, or one running at the edge of the
 * device's capacity) and therefore cannot create a handle, since lh_create
 * allocates the whole channel state. Same transform as lh_four_to_phys on
 * `nplanes` spectral planes [N2][N1/2+1] complex128 -> physical [Ngal2][Ngal1]
 * double, caller-owned device buffers, on `stream` (cudaStream_t as void*,
 * NULL = default stream). Its working memory is a fixed device array of
 * LH_NOALLOC_SCRATCH_BYTES inside the library, which every GPU that loads the
 * library holds until exit. It must hold the two twiddle tables and the
 * intermediate planes: 16*Ngal1 and 16*Ngal2 bytes (each rounded up to 256) plus
 * nplanes * Ngal2 * (N1/2+1) * 16 bytes; larger requests are rejected with
 * LH_EINVAL and *err (if not NULL) points to a static message. The first call on a device
 * does a one-time set-up for that device (looks up the array's device address and
 * sets the kernels' shared-memory limit); make that first call before any stream
 * capture. Host threads that make their first calls at the same time are serialised
 * during the set-up, and it runs again after a cudaDeviceReset (which clears it).
 * Every call shares the one array and overwrites what it needs, so calls
 * that overlap on the GPU (other streams, other host threads) race: serialise them. */
#define LH_NOALLOC_SCRATCH_BYTES (32u << 20)
int lh_four_to_phys_noalloc(int N1, int N2, int Ngal1, int Ngal2, const void *spec, void *phys,
                            int nplanes, void *stream, const char **err);

#ifdef __cplusplus
}
#endif
#endif /* LH_H */
