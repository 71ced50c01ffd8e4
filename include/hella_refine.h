/*
 * hella_refine.h -- differentiable refinement of FRB candidates on GB300
 * (sm_103a).  No counterpart in casm-hella, whose search stops at the
 * detection grid (peaks.cu:31-117 reports a DM trial index, a boxcar width
 * index and a sample); this stage fits continuous burst parameters to each
 * detection's dynamic-spectrum cutout.
 *
 * Cutout i is fp32 [nchan][nsamp], channel 0 the highest frequency f0,
 * each channel row already shifted by the integer delay of the detection
 * DM dm_ref[i]: off_c = (int)(dm_ref * tab[c] + 0.5f), tab[c] =
 * 4.148808e3 (1/f_c^2 - 1/f0^2) / tsamp samples per unit DM (the
 * dedispersion plan's rounding, hella_dedisp.h).  The model is a dispersed
 * Gaussian at fractional delays:
 *   m[c][t] = amp * (f_c/f0)^index * exp(-u^2/2),
 *   u = (t - mu_c) / sigma,  mu_c = t0 + dm * tab[c] - off_c,
 *   sigma = width / (2 sqrt(2 ln 2)) in samples (width = FWHM in ms),
 * and chi2 = sum over c, t of (d - m)^2 (unit-variance noise).
 * theta[i] = {dm (pc cm^-3), t0 (samples), width (ms), amp, index}.
 * All pointers are device pointers; work is issued on the context's
 * stream and every call returns once it is queued. */
#ifndef HELLA_REFINE_H
#define HELLA_REFINE_H

#include "hella_search.h"

#ifdef __cplusplus
extern "C" {
#endif

#define HELLA_REFINE_NPAR 5

typedef struct hella_refine hella_refine;

typedef struct {
  int ncut;          /* cutouts per call (capacity) */
  int nchan;         /* channels per cutout, a multiple of 16 */
  int nsamp;         /* samples per channel, a multiple of 128 */
  double tsamp;      /* s */
  double f0_mhz;     /* frequency of channel 0 */
  double df_mhz;     /* channel width (sign ignored: descending) */
  int device;
} hella_refine_params;

hella_status hella_refine_create(hella_refine **r, const hella_refine_params *p);
void hella_refine_destroy(hella_refine *r);
hella_status hella_refine_set_stream(hella_refine *r, void *stream);
/* Host copy of the per-unit-DM delay table tab[nchan] the model uses. */
hella_status hella_refine_delay_table(const hella_refine *r, float *tab);

/* Forward: chi2[i] for the first n cutouts. */
hella_status hella_refine_forward(hella_refine *r, int n, const float *cutouts, const float *dm_ref,
                                  const float *theta, float *chi2);
/* Adjoint: gtheta[i][k] = gchi2[i] * d chi2_i / d theta[i][k], the model
 * recomputed from theta (nothing is kept from the forward call). */
hella_status hella_refine_adjoint(hella_refine *r, int n, const float *cutouts, const float *dm_ref,
                                  const float *theta, const float *gchi2, float *gtheta);
/* `steps` Adam steps on chi2 (betas 0.9/0.999, eps 1e-8, per-parameter
 * learning rates lr[5], host memory) updating theta in place; every step
 * is one fused forward + adjoint pass over the cutouts.  width is kept
 * >= 0.05 ms and dm >= 0.  chi2 (may be NULL) receives the chi2 of the
 * last step's starting point. */
hella_status hella_refine_fit(hella_refine *r, int n, const float *cutouts, const float *dm_ref,
                              float *theta, int steps, const float *lr, float *chi2);

#ifdef __cplusplus
}
#endif
#endif
