/* lh_oracle.h — CPU FP64 restatement of the reference RK3 substep.
 * TEST INFRASTRUCTURE ONLY: used by tests/, smoke() and bench.py's CPU-baseline leg
 * as the checker; never by the product path. */
#ifndef LH_ORACLE_H
#define LH_ORACLE_H
#include "../include/lh.h"
typedef struct orc orc;
orc *orc_create(const lh_config *cfg);
void orc_destroy(orc *O);
int orc_set_state(orc *O, const double *u1, const double *u2, const double *u3, const double *p);
int orc_get_state(orc *O, double *u1, double *u2, double *u3, double *p);
int orc_set_band(orc *O, int band, const double *u1, const double *u2, const double *u3, const double *p);
int orc_get_band(orc *O, int band, double *u1, double *u2, double *u3, double *p);
int orc_get_nonlinear(orc *O, double *n1, double *n2, double *n3);
int orc_set_scalars(orc *O, const lh_scalars *s);
int orc_get_scalars(orc *O, lh_scalars *s);
int orc_substep(orc *O, int kRK);
int orc_step(orc *O);
int orc_four_to_phys(orc *O, const double *spec, double *phys, int nplanes);
int orc_phys_to_four(orc *O, const double *phys, double *spec, int nplanes);
int orc_set_threads(int n);
/* test hook: noise eps x max|line| on every transform output (0: off), process-wide */
int orc_set_transform_noise(double eps);
int orc_stats_accumulate(orc *O);
/* plane: [11][nu]; dims: ncl, dnx, dnz */
int orc_stats_get(orc *O, double *plane, double *cond, int64_t *istat, int *dims);
int orc_stats_reset(orc *O);
/* pplane: [2][np] (P, P^2); cond4: [4][ncl + 1][dnz][dnx] (P, P^2, omega_x, omega_x^2) */
int orc_stats_get_pw(orc *O, double *pplane, double *cond4);
int orc_spectra_get(orc *O, double *sU, double *sV, double *sW, double *sUV, double *sP, int *nl, int *nlong);
int orc_slip_get(orc *O, double *acc);
int orc_slip_planes(orc *O, double *out);
#endif
