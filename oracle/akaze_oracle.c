/*
 * akaze_oracle.c - CPU oracle for the A-KAZE hot path of francoto/akaze.
 *
 * TEST INFRASTRUCTURE ONLY: a checker for the GPU library and the timed CPU
 * baseline, never part of the product.  See akaze_oracle.h for what each
 * stage restates and how far parity is pinned.  Build with
 * -ffp-contract=off so that no multiply-add is fused on any host.
 */
#include "akaze_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../akaze_gb300/csrc/akz_fmath.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
#define AKO_CV_PI 3.1415926535897932384626433832795

static inline int ako_clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* cv::BORDER_REFLECT_101 for offsets of at most n-1. */
static inline int ako_refl101(int i, int n)
{
  if (n == 1) return 0;
  if (i < 0) return -i;
  if (i >= n) return 2 * n - 2 - i;
  return i;
}

/* Per-axis INTER_AREA weight table (pixel-area relation): for each
 * destination index the source indices and weights, in ascending order.
 * The reference half-samples odd sizes with cv::resize(INTER_AREA)
 * (nldiffusion_functions.cpp:320-324); to give its bits, the table follows
 * the construction of OpenCV's computeResizeAreaTab (modules/imgproc/src/
 * resize.cpp; OpenCV, Apache License 2.0 for 4.x, 3-clause BSD before):
 * destination cell [d*scale, (d+1)*scale) clipped to the source, a leading
 * and a trailing partial pixel kept only when their overlap exceeds 1e-3,
 * weights = overlap / cell width. */
typedef struct {
  int *start; /* dsize+1 */
  int *si;
  float *alpha;
} ako_area_table;

static void ako_area_tab(int ssize, int dsize, ako_area_table *t)
{
  const double scale = (double)ssize / dsize;
  const int cap = 2 * ssize + 2 * dsize + 4;
  t->start = (int *)malloc(sizeof(int) * (size_t)(dsize + 1));
  t->si = (int *)malloc(sizeof(int) * (size_t)cap);
  t->alpha = (float *)malloc(sizeof(float) * (size_t)cap);
  int k = 0;
  for (int dx = 0; dx < dsize; dx++) {
    t->start[dx] = k;
    const double fsx1 = dx * scale;
    const double fsx2 = fsx1 + scale;
    const double cellWidth = fmin(scale, ssize - fsx1);
    int sx1 = (int)ceil(fsx1), sx2 = (int)floor(fsx2);
    sx2 = sx2 < ssize - 1 ? sx2 : ssize - 1;
    sx1 = sx1 < sx2 ? sx1 : sx2;
    if (sx1 - fsx1 > 1e-3) {
      t->si[k] = sx1 - 1;
      t->alpha[k++] = (float)((sx1 - fsx1) / cellWidth);
    }
    for (int sx = sx1; sx < sx2; sx++) {
      t->si[k] = sx;
      t->alpha[k++] = (float)(1.0 / cellWidth);
    }
    if (fsx2 - sx2 > 1e-3) {
      t->si[k] = sx2;
      t->alpha[k++] = (float)(fmin(fmin(fsx2 - sx2, 1.), cellWidth) / cellWidth);
    }
  }
  t->start[dsize] = k;
}

static void ako_area_free(ako_area_table *t)
{
  free(t->start);
  free(t->si);
  free(t->alpha);
}

/* ---- FP32 instantiation (reference CPU semantics) ---- */
#define REAL float
#define AKO_SFX _f32
#define AKO_SQRT sqrtf
#define AKO_FLOOR floorf
#define AKO_EXP akz_expf
#include "ako_scale_impl.h"
#undef REAL
#undef AKO_SFX
#undef AKO_SQRT
#undef AKO_FLOOR
#undef AKO_EXP

/* ---- FP64 instantiation (error report) ---- */
#define REAL double
#define AKO_SFX _f64
#define AKO_SQRT sqrt
#define AKO_FLOOR floor
#define AKO_EXP exp
#include "ako_scale_impl.h"
#undef REAL
#undef AKO_SFX
#undef AKO_SQRT
#undef AKO_FLOOR
#undef AKO_EXP

/* ------------------------------------------------------------------------ */
/* FED schedule, fed.cpp:41-148                                              */

static int ako_is_prime(int number)
{
  if (number <= 1) return 0;
  if (number == 2 || number == 3 || number == 5 || number == 7) return 1;
  if ((number % 2) == 0 || (number % 3) == 0 || (number % 5) == 0 || (number % 7) == 0) return 0;
  const int upper = (int)sqrt(number + 1.0);
  for (int d = 11; d <= upper; d += 2)
    if (number % d == 0) return 0;
  return 1;
}

static int ako_fed_tau_internal(int n, float scale, float tau_max, int reordering, float *tau, int cap)
{
  if (n <= 0 || n > cap) return 0;
  float *tauh = (float *)malloc(sizeof(float) * (size_t)n);
  const float c = 1.0f / (4.0f * (float)n + 2.0f);
  const float d = scale * tau_max / 2.0f;
  for (int k = 0; k < n; ++k) {
    const float h = (float)cos(M_PI * (double)(2.0f * (float)k + 1.0f) * (double)c);
    tauh[k] = d / (h * h);
  }
  if (!reordering) {
    memcpy(tau, tauh, sizeof(float) * (size_t)n);
  } else if (n == 1) {
    /* the reference's kappa-cycle with kappa = n/2 = 0 indexes tauh[-1]; the
     * single step is taken as is */
    tau[0] = tauh[0];
  } else {
    const int kappa = n / 2;
    int prime = n + 1;
    while (!ako_is_prime(prime)) prime++;
    for (int k = 0, l = 0; l < n; ++k, ++l) {
      int index;
      while ((index = ((k + 1) * kappa) % prime - 1) >= n) k++;
      tau[l] = tauh[index];
    }
  }
  free(tauh);
  return n;
}

int ako_fed_tau_by_process_time(float T, int M, float tau_max, int reordering, float *tau, int cap)
{
  const float t = T / (float)M;
  const int n = (int)(ceil(sqrt(3.0 * t / tau_max + 0.25f) - 0.5f - 1.0e-8f) + 0.5f);
  const float scale = (float)(3.0 * t / (tau_max * (float)(n * (n + 1))));
  return ako_fed_tau_internal(n, scale, tau_max, reordering, tau, cap);
}

/* Gaussian kernel size (nldiffusion_functions.cpp:33-43) and taps: the
 * normalised samples of exp(-x^2/(2 sigma^2)) computed in double, as
 * cv::getGaussianKernel does, then rounded to float. */
static int ako_gauss_R(float sigma)
{
  long ks = (long)ceil(2.0 * (1.0 + (sigma - 0.8) / (0.3)));
  if (ks % 2 == 0) ks += 1;
  return (int)(ks / 2);
}

static void ako_gauss_taps_d(float sigma, int R, double *k)
{
  const double scale2 = -0.5 / ((double)sigma * (double)sigma);
  double sum = 0;
  for (int i = 0; i <= 2 * R; i++) {
    const double x = i - R;
    k[i] = exp(scale2 * x * x);
    sum += k[i];
  }
  for (int i = 0; i <= 2 * R; i++) k[i] = k[i] / sum;
}

int ako_gaussian_taps(float sigma, float *taps, int cap)
{
  const int R = ako_gauss_R(sigma);
  if (2 * R + 1 > cap || R > 64) return -1;
  double k[129];
  ako_gauss_taps_d(sigma, R, k);
  for (int i = 0; i <= 2 * R; i++) taps[i] = (float)k[i];
  return 2 * R + 1;
}

/* ------------------------------------------------------------------------ */

struct ako_ctx {
  ako_options opt;
  int W, H, nlev;
  ako_level lev[AKO_MAX_LEVELS];
  float *tau[AKO_MAX_LEVELS];
  size_t off[AKO_MAX_LEVELS + 1];
  float *Lt, *Ls, *Lf, *Lx, *Ly, *Ld; /* all levels, dense, concatenated */
  double *Lt64;
  float kcontrast;
  double kcontrast64;
  int built;
  ako_extremum *ext;
  int next;
  int ext_off[AKO_MAX_LEVELS + 1];
  int *state;
  ako_keypoint *kp;
  int nkp;
  uint8_t *desc;
  int ndesc;
  int desc_bytes; /* bytes of one descriptor row */
};

void ako_options_default(ako_options *o)
{
  o->omax = 4;
  o->nsublevels = 4;
  o->soffset = 1.6f;
  o->derivative_factor = 1.5f;
  o->sderivatives = 1.0f;
  o->diffusivity = 1;
  o->dthreshold = 0.001f;
  o->min_dthreshold = 0.00001f;
  o->descriptor = 5;
  o->descriptor_size = 0;
  o->descriptor_channels = 3;
  o->descriptor_pattern_size = 10;
  o->kcontrast_percentile = 0.7f;
  o->kcontrast_nbins = 300;
  o->extrema_3d = 0;
}

void ako_set_threads(int n)
{
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* AKAZE.cpp:146-197: level geometry, evolution times, FED schedules. */
ako_ctx *ako_create(const ako_options *o, int W, int H)
{
  if (!o || W < 8 || H < 8 || o->omax < 1 || o->nsublevels < 1 || o->omax * o->nsublevels > AKO_MAX_LEVELS) return NULL;
  if (o->soffset < 0.65f || o->kcontrast_nbins < 1) return NULL;
  ako_ctx *c = (ako_ctx *)calloc(1, sizeof(ako_ctx));
  c->opt = *o;
  c->W = W;
  c->H = H;
  int nlev = 0;
  for (int i = 0; i <= o->omax - 1; i++) {
    const float rfactor = (float)(1.0 / pow(2.0, i));
    const int lh = (int)((float)H * rfactor);
    const int lw = (int)((float)W * rfactor);
    if ((lw < 80 || lh < 40) && i != 0) break;
    for (int j = 0; j < o->nsublevels; j++) {
      ako_level *L = &c->lev[nlev];
      L->width = lw;
      L->height = lh;
      L->octave = i;
      L->sublevel = j;
      L->esigma = o->soffset * powf(2.0f, (float)j / (float)o->nsublevels + (float)i);
      L->etime = (float)(0.5 * (double)(L->esigma * L->esigma));
      const float ratio = powf(2.0f, (float)i);
      L->deriv_step = (int)(L->esigma * o->derivative_factor / ratio + 0.5f);
      L->size = L->esigma * o->derivative_factor;
      const float smax = (float)(10.0 * (double)sqrtf(2.0f));
      L->border = smax * (float)(int)(L->size / ratio + 0.5f);
      nlev++;
    }
  }
  c->nlev = nlev;
  for (int i = 1; i < nlev; i++) {
    float tmp[4096];
    const float ttime = c->lev[i].etime - c->lev[i - 1].etime;
    const int n = ako_fed_tau_by_process_time(ttime, 1, 0.25f, 1, tmp, 4096);
    c->lev[i].nsteps = n;
    c->tau[i] = (float *)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1));
    memcpy(c->tau[i], tmp, sizeof(float) * (size_t)n);
  }
  c->off[0] = 0;
  for (int i = 0; i < nlev; i++) c->off[i + 1] = c->off[i] + (size_t)c->lev[i].width * c->lev[i].height;
  const size_t tot = c->off[nlev];
  c->Lt = (float *)calloc(tot, sizeof(float));
  c->Ls = (float *)calloc(tot, sizeof(float));
  c->Lf = (float *)calloc(tot, sizeof(float));
  c->Lx = (float *)calloc(tot, sizeof(float));
  c->Ly = (float *)calloc(tot, sizeof(float));
  c->Ld = (float *)calloc(tot, sizeof(float));
  if (!c->Lt || !c->Ls || !c->Lf || !c->Lx || !c->Ly || !c->Ld) {
    ako_destroy(c);
    return NULL;
  }
  return c;
}

void ako_destroy(ako_ctx *c)
{
  if (!c) return;
  for (int i = 0; i < AKO_MAX_LEVELS; i++) free(c->tau[i]);
  free(c->Lt);
  free(c->Ls);
  free(c->Lf);
  free(c->Lx);
  free(c->Ly);
  free(c->Ld);
  free(c->Lt64);
  free(c->ext);
  free(c->state);
  free(c->kp);
  free(c->desc);
  free(c);
}

int ako_num_levels(const ako_ctx *c) { return c ? c->nlev : -1; }

int ako_get_level(const ako_ctx *c, int i, ako_level *out)
{
  if (!c || i < 0 || i >= c->nlev) return -1;
  *out = c->lev[i];
  return 0;
}

int ako_get_tau(const ako_ctx *c, int i, float *tau, int cap)
{
  if (!c || i < 1 || i >= c->nlev) return 0;
  const int n = c->lev[i].nsteps;
  for (int k = 0; k < n && k < cap; k++) tau[k] = c->tau[i][k];
  return n;
}

void ako_u8_to_unit(const uint8_t *src, float *dst, long n)
{
  const float s = (float)(1.0 / 255.0);
  for (long i = 0; i < n; i++) dst[i] = (float)src[i] * s;
}

/* ------------------------------------------------------------------------ */
/* The oracle's scale-space stages on single planes, exported so that the
 * reference's own nldiffusion_functions.cpp, compiled by oracle/Makefile
 * target "ref" over an OpenCV-shaped shim, can be checked against them
 * (its GaussianBlur, Scharr and resize calls route here). */

/* Gaussian of sigma with the oracle's kernel-size rule; *ksize receives the
 * kernel size used. */
int ako_plane_gaussian(const float *src, float *dst, int w, int h, float sigma, int *ksize)
{
  const int R = ako_gauss_R(sigma);
  if (R > 64 || w < 1 || h < 1) return -1;
  double kd[129];
  float k[129];
  ako_gauss_taps_d(sigma, R, kd);
  for (int i = 0; i <= 2 * R; i++) k[i] = (float)kd[i];
  float *tmp = (float *)malloc(sizeof(float) * (size_t)w * h);
  if (!tmp) return -1;
  ako_gauss_f32(src, dst, tmp, w, h, k, R);
  free(tmp);
  if (ksize) *ksize = 2 * R + 1;
  return 0;
}

void ako_plane_scharr(const float *src, float *lx, float *ly, int w, int h) { ako_scharr_f32(src, lx, ly, w, h); }

void ako_plane_halfsample(const float *src, int sw, int sh, float *dst, int dw, int dh)
{
  ako_halfsample_f32(src, sw, sh, dst, dw, dh);
}

void ako_plane_conductance(const float *lx, const float *ly, float *dst, long n, float k, int type)
{
  ako_conductance_f32(lx, ly, dst, (size_t)n, k, type);
}

void ako_plane_nld_step(float *Ld, const float *c, int w, int h, float stepsize)
{
  float *Lstep = (float *)calloc((size_t)w * h, sizeof(float));
  if (!Lstep) return;
  ako_nld_step_f32(Ld, c, Lstep, w, h, stepsize);
  free(Lstep);
}

/* compute_k_percentile(img, perc, gscale, nbins, 0, 0) as the oracle
 * evaluates it. */
float ako_plane_k_percentile(const float *img, int w, int h, float perc, int nbins, float gscale)
{
  const int R = ako_gauss_R(gscale);
  if (R > 64) return -1.0f;
  double kd[129];
  float k[129];
  ako_gauss_taps_d(gscale, R, kd);
  for (int i = 0; i <= 2 * R; i++) k[i] = (float)kd[i];
  const size_t n = (size_t)w * h;
  float *buf = (float *)malloc(sizeof(float) * n * 4);
  if (!buf) return -1.0f;
  const float r = ako_k_percentile_f32(img, w, h, perc, nbins, k, R, buf, buf + n, buf + 2 * n, buf + 3 * n);
  free(buf);
  return r;
}

/* AKAZE.cpp:211-276 with the reference CPU functions (the upstream CPU
 * orchestration the fork's GPU code mirrors): level 0 is the soffset Gaussian
 * of the image, each later level starts from the previous level's final image
 * (half-sampled at an octave change, where the contrast factor is scaled by
 * 0.75), is smoothed with sigma 1 (Lsmooth), gives the PM-g2 conductance and
 * evolves by the level's FED steps. */
int ako_build(ako_ctx *c, const float *img)
{
  if (!c || !img) return -1;
  const int W = c->W, H = c->H;
  const size_t n0 = (size_t)W * H;
  float *tmp = (float *)malloc(sizeof(float) * n0);
  float *g = (float *)malloc(sizeof(float) * n0);
  float *lx = (float *)malloc(sizeof(float) * n0);
  float *ly = (float *)malloc(sizeof(float) * n0);
  float taps1[129], taps0[129];
  double td[129];
  const int R1 = ako_gauss_R(1.0f);
  ako_gauss_taps_d(1.0f, R1, td);
  for (int i = 0; i <= 2 * R1; i++) taps1[i] = (float)td[i];
  const int R0 = ako_gauss_R(c->opt.soffset);
  ako_gauss_taps_d(c->opt.soffset, R0, td);
  for (int i = 0; i <= 2 * R0; i++) taps0[i] = (float)td[i];

  float kc = ako_k_percentile_f32(img, W, H, c->opt.kcontrast_percentile, c->opt.kcontrast_nbins, taps1, R1, g, lx, ly, tmp);
  c->kcontrast = kc;
  ako_gauss_f32(img, c->Lt, tmp, W, H, taps0, R0);
  memcpy(c->Ls, c->Lt, sizeof(float) * n0);
  memset(c->Lf, 0, sizeof(float) * n0);
  c->lev[0].kcontrast = kc;
  for (int i = 1; i < c->nlev; i++) {
    const ako_level *L = &c->lev[i], *P = &c->lev[i - 1];
    float *Lt = c->Lt + c->off[i], *Lp = c->Lt + c->off[i - 1];
    const size_t n = (size_t)L->width * L->height;
    if (L->octave > P->octave) {
      ako_halfsample_f32(Lp, P->width, P->height, Lt, L->width, L->height);
      kc = (float)(kc * 0.75);
    } else {
      memcpy(Lt, Lp, sizeof(float) * n);
    }
    c->lev[i].kcontrast = kc;
    float *Ls = c->Ls + c->off[i];
    ako_gauss_f32(Lt, Ls, tmp, L->width, L->height, taps1, R1);
    ako_scharr_f32(Ls, lx, ly, L->width, L->height);
    float *Lf = c->Lf + c->off[i];
    ako_conductance_f32(lx, ly, Lf, n, kc, c->opt.diffusivity);
    for (int j = 0; j < L->nsteps; j++) ako_nld_step_f32(Lt, Lf, tmp, L->width, L->height, c->tau[i][j]);
  }
  free(tmp);
  free(g);
  free(lx);
  free(ly);
  c->built = 1;
  return 0;
}

int ako_build_f64(ako_ctx *c, const float *img)
{
  if (!c || !img) return -1;
  const int W = c->W, H = c->H;
  const size_t n0 = (size_t)W * H, tot = c->off[c->nlev];
  free(c->Lt64);
  c->Lt64 = (double *)malloc(sizeof(double) * tot);
  double *im = (double *)malloc(sizeof(double) * n0);
  double *tmp = (double *)malloc(sizeof(double) * n0);
  double *g = (double *)malloc(sizeof(double) * n0);
  double *lx = (double *)malloc(sizeof(double) * n0);
  double *ly = (double *)malloc(sizeof(double) * n0);
  double *Ls = (double *)malloc(sizeof(double) * n0);
  double *Lf = (double *)malloc(sizeof(double) * n0);
  for (size_t i = 0; i < n0; i++) im[i] = img[i];
  double taps1[129], taps0[129];
  const int R1 = ako_gauss_R(1.0f), R0 = ako_gauss_R(c->opt.soffset);
  ako_gauss_taps_d(1.0f, R1, taps1);
  ako_gauss_taps_d(c->opt.soffset, R0, taps0);
  double kc = ako_k_percentile_f64(im, W, H, (double)c->opt.kcontrast_percentile, c->opt.kcontrast_nbins, taps1, R1, g, lx, ly, tmp);
  c->kcontrast64 = kc;
  ako_gauss_f64(im, c->Lt64, tmp, W, H, taps0, R0);
  for (int i = 1; i < c->nlev; i++) {
    const ako_level *L = &c->lev[i], *P = &c->lev[i - 1];
    double *Lt = c->Lt64 + c->off[i], *Lp = c->Lt64 + c->off[i - 1];
    const size_t n = (size_t)L->width * L->height;
    if (L->octave > P->octave) {
      ako_halfsample_f64(Lp, P->width, P->height, Lt, L->width, L->height);
      kc = kc * 0.75;
    } else {
      memcpy(Lt, Lp, sizeof(double) * n);
    }
    ako_gauss_f64(Lt, Ls, tmp, L->width, L->height, taps1, R1);
    ako_scharr_f64(Ls, lx, ly, L->width, L->height);
    ako_conductance_f64(lx, ly, Lf, n, kc, c->opt.diffusivity);
    for (int j = 0; j < L->nsteps; j++) ako_nld_step_f64(Lt, Lf, tmp, L->width, L->height, c->tau[i][j]);
  }
  free(im);
  free(tmp);
  free(g);
  free(lx);
  free(ly);
  free(Ls);
  free(Lf);
  return 0;
}

float ako_kcontrast(const ako_ctx *c) { return c ? c->kcontrast : 0.0f; }
double ako_kcontrast_f64(const ako_ctx *c) { return c ? c->kcontrast64 : 0.0; }

int ako_get_plane(const ako_ctx *c, int level, int plane, float *out)
{
  if (!c || level < 0 || level >= c->nlev || !out) return -1;
  const float *base[6] = {c->Lt, c->Ls, c->Lf, c->Lx, c->Ly, c->Ld};
  if (plane < 0 || plane > 5) return -1;
  memcpy(out, base[plane] + c->off[level], sizeof(float) * (c->off[level + 1] - c->off[level]));
  return 0;
}

int ako_get_plane_f64(const ako_ctx *c, int level, double *out)
{
  if (!c || !c->Lt64 || level < 0 || level >= c->nlev || !out) return -1;
  memcpy(out, c->Lt64 + c->off[level], sizeof(double) * (c->off[level + 1] - c->off[level]));
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Detector: cuda_akaze.cu:651-725 (scaled Scharr derivatives with step
 * sigma_size and reflect-101 border, Hessian determinant).                  */

static void ako_deriv_pair(const float *s, float *dx, float *dy, int w, int h, int step, float fac1, float fac2)
{
  int y;
#pragma omp parallel for schedule(static)
  for (y = 0; y < h; y++) {
    const int yl = y < step ? step - y : y - step;
    const int yh = y >= h - step ? 2 * h - y - step - 2 : y + step;
    for (int x = 0; x < w; x++) {
      const int xl = x < step ? step - x : x - step;
      const int xh = x >= w - step ? 2 * w - x - step - 2 : x + step;
      const float ul = s[(size_t)yl * w + xl], ur = s[(size_t)yl * w + xh];
      const float ll = s[(size_t)yh * w + xl], lr = s[(size_t)yh * w + xh];
      const float cl = s[(size_t)y * w + xl], cr = s[(size_t)y * w + xh];
      const float uc = s[(size_t)yl * w + x], lc = s[(size_t)yh * w + x];
      dx[(size_t)y * w + x] = fac1 * (ur + lr - ul - ll) + fac2 * (cr - cl);
      dy[(size_t)y * w + x] = fac1 * (lr + ll - ur - ul) + fac2 * (lc - uc);
    }
  }
}

static void ako_hessian(const float *lx, const float *ly, float *det, int w, int h, int step, float fac1, float fac2)
{
  int y;
#pragma omp parallel for schedule(static)
  for (y = 0; y < h; y++) {
    const int yl = y < step ? step - y : y - step;
    const int yh = y >= h - step ? 2 * h - y - step - 2 : y + step;
    for (int x = 0; x < w; x++) {
      const int xl = x < step ? step - x : x - step;
      const int xh = x >= w - step ? 2 * w - x - step - 2 : x + step;
      float ul = lx[(size_t)yl * w + xl], ur = lx[(size_t)yl * w + xh];
      float ll = lx[(size_t)yh * w + xl], lr = lx[(size_t)yh * w + xh];
      const float cl = lx[(size_t)y * w + xl], cr = lx[(size_t)y * w + xh];
      const float lxx = fac1 * (ur + lr - ul - ll) + fac2 * (cr - cl);
      float uc = lx[(size_t)yl * w + x], lc = lx[(size_t)yh * w + x];
      const float lyx = fac1 * (lr + ll - ur - ul) + fac2 * (lc - uc);
      ul = ly[(size_t)yl * w + xl];
      ur = ly[(size_t)yl * w + xh];
      ll = ly[(size_t)yh * w + xl];
      lr = ly[(size_t)yh * w + xh];
      uc = ly[(size_t)yl * w + x];
      lc = ly[(size_t)yh * w + x];
      const float lyy = fac1 * (lr + ll - ur - ul) + fac2 * (lc - uc);
      det[(size_t)y * w + x] = lxx * lyy - lyx * lyx;
    }
  }
}

/* 1 when v exceeds the 9 values of the 3 x 3 block at p of the level plane
 * A (same size as the current level), or when there is no such level. */
static int ako_above3x3(const float *A, size_t p, int w, float v)
{
  if (!A) return 1;
  for (int dy = -1; dy <= 1; dy++)
    for (int dx = -1; dx <= 1; dx++)
      if (!(v > A[(long)p + (long)dy * w + dx])) return 0;
  return 1;
}

/* cuda_akaze.cu:727-774 for one level, in raster order (the order the
 * reference's per-level bitonic sort by (y, x) produces, :884-939).  With
 * Dp / Dn (the determinants of the previous and next level of the same
 * octave, NULL where there is none) a candidate must also exceed their 3 x 3
 * blocks at its position: the 3 x 3 x 3 rule for which the reference passes
 * those planes to FindExtrema and leaves them unused (AKAZE.cpp:340-367). */
static int ako_find_extrema(const float *D, const float *Dp, const float *Dn, int w, int h, const ako_level *L,
                            int level, float thr, ako_extremum *out, int cap)
{
  int n = 0;
  const float border = L->border;
  const int octave = L->octave;
  for (int y = 0; y < h; y++) {
    for (int x = 0; x < w; x++) {
      const int left_x = (int)((float)x - border + 0.5f) - 1;
      const int right_x = (int)((float)x + border + 0.5f) + 1;
      const int up_y = (int)((float)y - border + 0.5f) - 1;
      const int down_y = (int)((float)y + border + 0.5f) + 1;
      if (left_x < 0 || right_x >= w || up_y < 0 || down_y >= h) continue;
      const size_t p = (size_t)y * w + x;
      const float v = D[p];
      if (v > thr && v > D[p - w - 1] && v > D[p + w + 1] && v > D[p + w - 1] && v > D[p - w + 1] && v > D[p - 1] &&
          v > D[p + 1] && v > D[p + w] && v > D[p - w] && ako_above3x3(Dp, p, w, v) && ako_above3x3(Dn, p, w, v)) {
        const float dx = 0.5f * (D[p + 1] - D[p - 1]);
        const float dy = 0.5f * (D[p + w] - D[p - w]);
        const float dxx = D[p + 1] + D[p - 1] - 2.0f * v;
        const float dyy = D[p + w] + D[p - w] - 2.0f * v;
        const float dxy = 0.25f * (D[p + w + 1] + D[p - w - 1] - D[p + w - 1] - D[p - w + 1]);
        const float det = dxx * dyy - dxy * dxy;
        const float idet = (det != 0.0f ? 1.0f / det : 0.0f);
        const float dst0 = idet * (dxy * dy - dyy * dx);
        const float dst1 = idet * (dxy * dx - dxx * dy);
        const int weak = !(dst0 >= -1.0f && dst0 <= 1.0f && dst1 >= -1.0f && dst1 <= 1.0f);
        if (n < cap) {
          ako_extremum *e = &out[n];
          e->x = x;
          e->y = y;
          e->level = level;
          e->octave = octave;
          e->response = v;
          e->size = (float)((weak ? -1 : 1) * 2.0 * (double)L->size);
          const float octsub = (float)(dst0 < 0 ? -1 : 1) * ((float)octave + fabsf(dst0));
          e->octsub = weak ? (float)octave : octsub;
          e->dst1 = dst1;
        }
        n++;
      }
    }
  }
  return n;
}

/* Neighbourhood suppression, cuda_akaze.cu:1005-1316, as the sequential
 * rule its round-based kernels compute (each round lets every point whose
 * earlier neighbours are all settled act, and lets only the lowest-indexed
 * challenger of a slot act on it, which is the sequential order):
 *   points in (level, y, x) order; neighbours of i are earlier points of the
 *   same level and any points of the previous level within distance
 *   |size_i|/2 (none for weak points, whose size is negative);
 *   no neighbour holding a slot -> i takes its own slot;
 *   otherwise compare with the neighbour whose slot value is smallest: if i's
 *   response is larger, i takes that neighbour's index as its slot value and
 *   the neighbour is dropped (-2), else i is dropped.
 * Emission (sortFiltered_kernel, :1227-1316) walks the slots in chunks of
 * 2048, sorts each chunk's non-negative slot values and emits the original
 * point at each value when its size is positive. */
static void ako_nms(ako_ctx *c)
{
  const int n = c->next;
  free(c->state);
  c->state = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  int *state = c->state;
  float *px = (float *)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1));
  float *py = (float *)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1));
  for (int i = 0; i < n; i++) {
    const int ratio = 1 << c->ext[i].octave;
    px[i] = (float)(ratio * c->ext[i].x);
    py[i] = (float)(ratio * c->ext[i].y);
    state[i] = -1;
  }
  for (int i = 0; i < n; i++) {
    const ako_extremum *e = &c->ext[i];
    const int l = e->level;
    const float size = e->size;
    const float hs = size * .5f;
    const double lim = (double)(size * size) * 0.25;
    int best = -1;
    for (int j = i - 1; j >= c->ext_off[l]; j--) {
      if (py[i] - py[j] > hs) break;
      const float ddx = px[i] - px[j], ddy = py[i] - py[j];
      const float dist = ddx * ddx + ddy * ddy;
      if ((double)dist < lim && state[j] >= 0 && (best < 0 || state[j] < state[best])) best = j;
    }
    if (l > 0) {
      for (int j = c->ext_off[l] - 1; j >= c->ext_off[l - 1]; j--) {
        if (py[j] - py[i] > hs) continue;
        if (py[i] - py[j] > hs) break;
        const float ddx = px[i] - px[j], ddy = py[i] - py[j];
        const float dist = ddx * ddx + ddy * ddy;
        if ((double)dist < lim && state[j] >= 0 && (best < 0 || state[j] < state[best])) best = j;
      }
    }
    if (best < 0) {
      state[i] = i;
    } else if (e->response > c->ext[best].response) {
      state[i] = best;
      state[best] = -2;
    } else {
      state[i] = -2;
    }
  }
  /* emission */
  free(c->kp);
  c->kp = (ako_keypoint *)malloc(sizeof(ako_keypoint) * (size_t)(n > 0 ? n : 1));
  int nk = 0;
  int vals[2048];
  for (int cs = 0; cs < n; cs += 2048) {
    int m = 0;
    for (int s = cs; s < cs + 2048 && s < n; s++) {
      const int v = state[s];
      if (v >= 0 && c->ext[v].size >= 0) vals[m++] = v;
    }
    for (int a = 1; a < m; a++) { /* insertion sort, ascending */
      const int t = vals[a];
      int b = a - 1;
      while (b >= 0 && vals[b] > t) {
        vals[b + 1] = vals[b];
        b--;
      }
      vals[b + 1] = t;
    }
    for (int a = 0; a < m; a++) {
      const ako_extremum *e = &c->ext[vals[a]];
      const float octsub = fabsf(e->octsub);
      const int octave = (int)octsub;
      const float subp = (e->octsub < 0 ? -1 : 1) * (octsub - (float)octave);
      const float ratio = (float)(1 << octave);
      ako_keypoint *k = &c->kp[nk++];
      k->y = ratio * ((float)(int)(0.5f + py[vals[a]] / ratio) + e->dst1);
      k->x = ratio * ((float)(int)(0.5f + px[vals[a]] / ratio) + subp);
      k->class_id = e->level;
      k->octave = octave;
      k->response = e->response;
      k->size = e->size;
      k->angle = 0.0f;
    }
  }
  c->nkp = nk;
  free(px);
  free(py);
}

/* Orientation, cuda_akaze.cu:2114-2167: 109 samples (radius < 6 on a grid
 * of spacing step) weighted by a sigma-2.5 Gaussian, 42 angular bins, a
 * 7-bin circular window sum, the strongest window's direction in [0, 2pi). */
static void ako_orientation(ako_ctx *c)
{
  float gw[36];
  for (int r2 = 0; r2 < 36; r2++) gw[r2] = akz_expf((float)(-r2) / (2.5f * 2.5f * 2.0f));
  int p;
#pragma omp parallel for schedule(dynamic, 16)
  for (p = 0; p < c->nkp; p++) {
    ako_keypoint *k = &c->kp[p];
    const int lev = k->class_id;
    const int w = c->lev[lev].width;
    const float *dxd = c->Lx + c->off[lev], *dyd = c->Ly + c->off[lev];
    const int octave = k->octave;
    const int step = (int)(0.5f * k->size + 0.5f) >> octave;
    const int x = (int)(k->x + 0.5f) >> octave;
    const int y = (int)(k->y + 0.5f) >> octave;
    float resx[42], resy[42], re8x[42], re8y[42];
    for (int b = 0; b < 42; b++) resx[b] = resy[b] = 0.0f;
    for (int tx = 0; tx < 208; tx++) {
      const int i = (tx & 15) - 6, j = (tx / 16) - 6;
      const int r2 = i * i + j * j;
      if (r2 < 36) {
        const int sx = ako_clampi(x + step * i, 0, w - 1), sy = ako_clampi(y + step * j, 0, c->lev[lev].height - 1);
        const size_t pos = (size_t)sy * w + sx;
        const float dx = gw[r2] * dxd[pos];
        const float dy = gw[r2] * dyd[pos];
        const float angle = akz_atan2f(dy, dx);
        int a = (int)((double)angle * (21 / AKO_CV_PI)) + 21;
        a = a > 41 ? 41 : a;
        a = a < 0 ? 0 : a;
        resx[a] += dx;
        resy[a] += dy;
      }
    }
    for (int t = 0; t < 42; t++) {
      re8x[t] = resx[t];
      re8y[t] = resy[t];
      for (int q = t + 1; q < t + 7; q++) {
        re8x[t] += resx[q < 42 ? q : q - 42];
        re8y[t] += resy[q < 42 ? q : q - 42];
      }
    }
    float maxr = 0.0f;
    int maxk = 0;
    for (int q = 0; q < 42; q++) {
      const float r = re8x[q] * re8x[q] + re8y[q] * re8y[q];
      if (r > maxr) {
        maxr = r;
        maxk = q;
      }
    }
    const float angle = akz_atan2f(re8y[maxk], re8x[maxk]);
    k->angle = angle < 0.0f ? (float)((double)angle + 2.0 * AKO_CV_PI) : angle;
  }
}

int ako_detect(ako_ctx *c)
{
  if (!c || !c->built) return -1;
  const float w = (float)(10.0 / 3.0);
  const float fac1 = (float)(1.0 / (2.0 * ((double)w + 2.0)));
  const float fac2 = w * fac1;
  const float thr = c->opt.dthreshold > c->opt.min_dthreshold ? c->opt.dthreshold : c->opt.min_dthreshold;
  for (int i = 0; i < c->nlev; i++) {
    const ako_level *L = &c->lev[i];
    ako_deriv_pair(c->Ls + c->off[i], c->Lx + c->off[i], c->Ly + c->off[i], L->width, L->height, L->deriv_step, fac1, fac2);
    ako_hessian(c->Lx + c->off[i], c->Ly + c->off[i], c->Ld + c->off[i], L->width, L->height, L->deriv_step, fac1, fac2);
  }
  /* adjacent levels of the same octave for the 3 x 3 x 3 rule */
  const float *Dp[AKO_MAX_LEVELS], *Dn[AKO_MAX_LEVELS];
  for (int i = 0; i < c->nlev; i++) {
    const int same_p = c->opt.extrema_3d && i > 0 && c->lev[i - 1].octave == c->lev[i].octave;
    const int same_n = c->opt.extrema_3d && i + 1 < c->nlev && c->lev[i + 1].octave == c->lev[i].octave;
    Dp[i] = same_p ? c->Ld + c->off[i - 1] : NULL;
    Dn[i] = same_n ? c->Ld + c->off[i + 1] : NULL;
  }
  int total = 0;
  for (int i = 0; i < c->nlev; i++) {
    const ako_level *L = &c->lev[i];
    total += ako_find_extrema(c->Ld + c->off[i], Dp[i], Dn[i], L->width, L->height, L, i, thr, NULL, 0);
  }
  free(c->ext);
  c->ext = (ako_extremum *)malloc(sizeof(ako_extremum) * (size_t)(total > 0 ? total : 1));
  int n = 0;
  for (int i = 0; i < c->nlev; i++) {
    const ako_level *L = &c->lev[i];
    c->ext_off[i] = n;
    n += ako_find_extrema(c->Ld + c->off[i], Dp[i], Dn[i], L->width, L->height, L, i, thr, c->ext + n, total - n);
  }
  c->ext_off[c->nlev] = n;
  c->next = n;
  ako_nms(c);
  if (c->opt.descriptor == 5) ako_orientation(c);
  return c->nkp;
}

int ako_num_extrema(const ako_ctx *c) { return c ? c->next : -1; }

int ako_get_extrema(const ako_ctx *c, ako_extremum *out, int cap)
{
  if (!c) return -1;
  const int n = c->next < cap ? c->next : cap;
  memcpy(out, c->ext, sizeof(ako_extremum) * (size_t)n);
  return n;
}

int ako_get_level_offsets(const ako_ctx *c, int *out, int cap)
{
  if (!c || cap < c->nlev + 1) return -1;
  for (int i = 0; i <= c->nlev; i++) out[i] = c->ext_off[i];
  return c->nlev + 1;
}

int ako_get_nms_state(const ako_ctx *c, int *out, int cap)
{
  if (!c || !c->state) return -1;
  const int n = c->next < cap ? c->next : cap;
  memcpy(out, c->state, sizeof(int) * (size_t)n);
  return n;
}

int ako_num_keypoints(const ako_ctx *c) { return c ? c->nkp : -1; }

int ako_get_keypoints(const ako_ctx *c, ako_keypoint *out, int cap)
{
  if (!c) return -1;
  const int n = c->nkp < cap ? c->nkp : cap;
  memcpy(out, c->kp, sizeof(ako_keypoint) * (size_t)n);
  return n;
}

/* ------------------------------------------------------------------------ */
/* M-LDB: cuda_akaze.cu:1420-1533 (samples and cell sums), :1786-1807 (bits)
 * and :2034-2111 (comparison order).  Cell sums in the reference's order
 * (ExtractDescriptors, cuda_akaze.cu:1456-1523): 64 threads, thread t sums
 * the window samples i = t, t + 64, ... of each cell in increasing i; per
 * cell, lane j < 32 adds the partials of threads j and j + 32, and a
 * __shfl_down tree with offsets 1, 2, 4, 8, 16 sums the 32 lanes. */

static int ako_cmp_pairs(int *i1, int *i2)
{
  int n = 0;
  const int g0[3] = {0, 4, 13}, g1[3] = {4, 13, 29};
  for (int grid = 0; grid < 3; grid++)
    for (int ch = 0; ch < 3; ch++)
      for (int j = g0[grid]; j < g1[grid] - 1; j++)
        for (int i = j + 1; i < g1[grid]; i++) {
          i1[n] = 3 * j + ch;
          i2[n] = 3 * i + ch;
          n++;
        }
  return n;
}

/* The generator behind srand()/rand() of the GNU C library (its TYPE_3
 * additive feedback generator, which the reference's
 * generateDescriptorSubsample uses through srand(1024), AKAZE.cpp:535):
 * r[0] = seed, r[i] = 16807 r[i-1] mod (2^31 - 1) for i < 31,
 * r[i] = r[i-31] for i = 31..33, then r[i] = r[i-31] + r[i-3] (mod 2^32);
 * the first 310 of those are discarded and output k is r[344+k] >> 1. */
typedef struct {
  uint32_t r[34];
  int i;
} ako_glibc_rand;

static void ako_glibc_srand(ako_glibc_rand *g, uint32_t seed)
{
  int32_t v[344];
  v[0] = (int32_t)(seed ? seed : 1);
  for (int i = 1; i < 31; i++) {
    const int64_t t = (16807LL * v[i - 1]) % 2147483647LL;
    v[i] = (int32_t)(t < 0 ? t + 2147483647LL : t);
  }
  for (int i = 31; i < 34; i++) v[i] = v[i - 31];
  uint32_t u[344];
  for (int i = 0; i < 34; i++) u[i] = (uint32_t)v[i];
  for (int i = 34; i < 344; i++) u[i] = u[i - 31] + u[i - 3];
  for (int k = 0; k < 34; k++) g->r[k] = u[310 + k];
  g->i = 0;
}

static int ako_glibc_rand_next(ako_glibc_rand *g)
{
  /* the ring holds r[n-34 .. n-1]; next = r[n-31] + r[n-3] */
  const uint32_t a = g->r[(g->i + 3) % 34], b = g->r[(g->i + 31) % 34];
  const uint32_t v = a + b;
  g->r[g->i] = v;
  g->i = (g->i + 1) % 34;
  return (int)(v >> 1);
}

int ako_glibc_rand_sequence(uint32_t seed, int *out, int n)
{
  ako_glibc_rand g;
  ako_glibc_srand(&g, seed);
  for (int k = 0; k < n; k++) out[k] = ako_glibc_rand_next(&g);
  return n;
}

/* Comparison table of the M-LDB bits: value indices 3*cell + channel into
 * the 29 x 3 cell sums (cells 0-3 the 2x2 grid, 4-12 the 3x3, 13-28 the 4x4,
 * each row-major in the rotated frame: row = the sample offset along the
 * keypoint direction).  Returns the bit count.
 *  - descriptor_size 0: every pair i < j of each grid, per channel in
 *    increasing channel order (AKAZE.cpp:412-418: (6+36+120)*channels bits);
 *  - descriptor_size n > 0: the random selection of generateDescriptorSubsample
 *    (AKAZE.cpp:498-603): of the 162 grid pairs, pick k = rand() % (162 - i)
 *    (forced to i for the first 6 picks) from a list shrunk by moving its
 *    last live row into the picked one; each pick's two cells become samples
 *    (reused when already listed) and give `channels` comparisons, channel c
 *    of the first cell against channel c of the second; the first n kept.
 *    The subset's cell with list index j of a g x g grid lies at row j % g
 *    and column j / g (Get_MLDB_Descriptor_Subset, the upstream libAKAZE
 *    routine the reference's table feeds, takes the sample's first offset
 *    along the keypoint direction). */
int ako_mldb_table(int channels, int nbits_subset, int *c1, int *c2)
{
  static const int g0[3] = {0, 4, 13};
  if (nbits_subset <= 0) {
    int n = 0;
    for (int grid = 0; grid < 3; grid++) {
      const int gs = (grid + 2) * (grid + 2);
      for (int ch = 0; ch < channels; ch++)
        for (int j = 0; j < gs - 1; j++)
          for (int i = j + 1; i < gs; i++) {
            c1[n] = 3 * (g0[grid] + j) + ch;
            c2[n] = 3 * (g0[grid] + i) + ch;
            n++;
          }
    }
    return n;
  }
  /* the 162 grid pairs as (grid, cell a, cell b) in the reference's order */
  int full[162][3], nf = 0;
  for (int grid = 0; grid < 3; grid++) {
    const int gs = (grid + 2) * (grid + 2);
    for (int j = 0; j < gs; j++)
      for (int k = j + 1; k < gs; k++) {
        full[nf][0] = grid;
        full[nf][1] = j;
        full[nf][2] = k;
        nf++;
      }
  }
  const int npicks = (nbits_subset + channels - 1) / channels;
  int samp[29][2], count = 0; /* listed samples: (grid, cell index in the subset's order) */
  int *cm1 = (int *)malloc(sizeof(int) * (size_t)npicks * channels), *cm2 = (int *)malloc(sizeof(int) * (size_t)npicks * channels);
  ako_glibc_rand g;
  ako_glibc_srand(&g, 1024);
  for (int i = 0; i < npicks; i++) {
    int k = ako_glibc_rand_next(&g) % (nf - i);
    if (i < 6) k = i;
    int which[2];
    for (int e = 0; e < 2; e++) {
      const int grid = full[k][0], cell = full[k][1 + e];
      int j;
      for (j = 0; j < count; j++)
        if (samp[j][0] == grid && samp[j][1] == cell) break;
      if (j == count) {
        samp[count][0] = grid;
        samp[count][1] = cell;
        count++;
      }
      which[e] = j;
    }
    for (int ch = 0; ch < channels; ch++) {
      cm1[i * channels + ch] = which[0] * 3 + ch; /* sample index * 3 + channel, mapped below */
      cm2[i * channels + ch] = which[1] * 3 + ch;
    }
    for (int q = 0; q < 3; q++) full[k][q] = full[nf - i - 1][q];
  }
  for (int b = 0; b < nbits_subset; b++) {
    const int s1 = cm1[b] / 3, ch = cm1[b] % 3, s2 = cm2[b] / 3;
    const int gd1 = samp[s1][0] + 2, gd2 = samp[s2][0] + 2;
    const int cell1 = g0[samp[s1][0]] + (samp[s1][1] % gd1) * gd1 + samp[s1][1] / gd1;
    const int cell2 = g0[samp[s2][0]] + (samp[s2][1] % gd2) * gd2 + samp[s2][1] / gd2;
    c1[b] = 3 * cell1 + ch;
    c2[b] = 3 * cell2 + ch;
  }
  free(cm1);
  free(cm2);
  return nbits_subset;
}

int ako_describe(ako_ctx *c)
{
  if (!c || !c->built) return -1;
  int i1[486], i2[486];
  const int channels = c->opt.descriptor_channels;
  if (channels < 1 || channels > 3 || c->opt.descriptor_size < 0 || c->opt.descriptor_size > 162 * channels) return -1;
  const int nbits = ako_mldb_table(channels, c->opt.descriptor_size, i1, i2);
  const int rb = (nbits + 7) / 8;
  c->desc_bytes = rb;
  free(c->desc);
  c->desc = (uint8_t *)calloc((size_t)(c->nkp > 0 ? c->nkp : 1), (size_t)rb);
  const int ps = c->opt.descriptor_pattern_size;
  const int size2 = ps;
  const int size3 = (int)ceilf(2.0f * (float)ps / 3.0f);
  const int size4 = (int)ceilf(0.5f * (float)ps);
  const int win = 3 * size3 > 4 * size4 ? 3 * size3 : 4 * size4;
  const int upright = c->opt.descriptor == 4;
  int p;
#pragma omp parallel for schedule(dynamic, 16)
  for (p = 0; p < c->nkp; p++) {
    const ako_keypoint *k = &c->kp[p];
    const int lev = k->class_id;
    const int w = c->lev[lev].width, h = c->lev[lev].height;
    const float *imd = c->Lt + c->off[lev], *dxd = c->Lx + c->off[lev], *dyd = c->Ly + c->off[lev];
    const float iratio = 1.0f / (float)(1 << k->octave);
    const int scale = (int)(0.5f * k->size * iratio + 0.5f);
    const float xf = k->x * iratio, yf = k->y * iratio;
    float co = 1.0f, si = 0.0f;
    if (!upright) akz_sincosf(k->angle, &si, &co);
    float vals[87];
    float part[64][87];
    memset(part, 0, sizeof(part));
    for (int y = 0; y < win; y++) {
      for (int x = 0; x < win; x++) {
        float *pv = part[(y * win + x) & 63];
        const int m = x > y ? x : y;
        const int l = x - size2, kk = y - size2;
        int xp = (int)(xf + (float)scale * ((float)kk * co - (float)l * si) + 0.5f);
        int yp = (int)(yf + (float)scale * ((float)kk * si + (float)l * co) + 0.5f);
        xp = ako_clampi(xp, 0, w - 1);
        yp = ako_clampi(yp, 0, h - 1);
        const size_t pos = (size_t)yp * w + xp;
        const float im = imd[pos], dx = dxd[pos], dy = dyd[pos];
        /* channels 2 and 3 of the cells: the rotated derivatives, or for a
         * 2-channel descriptor the gradient magnitude (MLDB_Fill_Values of
         * upstream libAKAZE; the reference's own kernel is 3-channel only) */
        const float rx = channels == 2 ? sqrtf(dx * dx + dy * dy) : -dx * si + dy * co;
        const float ry = dx * co + dy * si;
        if (m < 2 * size2) {
          const int x2 = x < size2 ? 0 : 1, y2 = y < size2 ? 0 : 1;
          const int cell = y2 * 2 + x2;
          pv[3 * cell] += im;
          pv[3 * cell + 1] += rx;
          pv[3 * cell + 2] += ry;
        }
        if (m < 3 * size3) {
          const int x3 = x < size3 ? 0 : (x < 2 * size3 ? 1 : 2), y3 = y < size3 ? 0 : (y < 2 * size3 ? 1 : 2);
          const int cell = 4 + y3 * 3 + x3;
          pv[3 * cell] += im;
          pv[3 * cell + 1] += rx;
          pv[3 * cell + 2] += ry;
        }
        if (m < 4 * size4) {
          const int x4 = x < 2 * size4 ? (x < size4 ? 0 : 1) : (x < 3 * size4 ? 2 : 3);
          const int y4 = y < 2 * size4 ? (y < size4 ? 0 : 1) : (y < 3 * size4 ? 2 : 3);
          const int cell = 13 + y4 * 4 + x4;
          pv[3 * cell] += im;
          pv[3 * cell + 1] += rx;
          pv[3 * cell + 2] += ry;
        }
      }
    }
    for (int q = 0; q < 87; q++) {
      float a[32];
      for (int j = 0; j < 32; j++) a[j] = part[j][q] + part[j + 32][q];
      for (int d = 1; d < 32; d <<= 1)
        for (int j = 0; j < 32; j += 2 * d) a[j] = a[j] + a[j + d];
      vals[q] = a[0];
    }
    uint8_t *d = c->desc + (size_t)p * rb;
    for (int b = 0; b < nbits; b++)
      if (vals[i1[b]] > vals[i2[b]]) d[b >> 3] |= (uint8_t)(1u << (b & 7));
  }
  c->ndesc = c->nkp;
  return c->nkp;
}

int ako_descriptor_bytes(const ako_ctx *c) { return c ? c->desc_bytes : -1; }

int ako_get_descriptors(const ako_ctx *c, uint8_t *out, int cap_rows)
{
  if (!c || !c->desc) return -1;
  const int n = c->ndesc < cap_rows ? c->ndesc : cap_rows;
  memcpy(out, c->desc, (size_t)n * c->desc_bytes);
  return n;
}

int ako_run_u8(ako_ctx *c, const uint8_t *img)
{
  if (!c || !img) return -1;
  const long n = (long)c->W * c->H;
  float *f = (float *)malloc(sizeof(float) * (size_t)n);
  ako_u8_to_unit(img, f, n);
  int r = ako_build(c, f);
  free(f);
  if (r) return r;
  r = ako_detect(c);
  if (r < 0) return r;
  return ako_describe(c);
}

/* ------------------------------------------------------------------------ */
/* 2-NN Hamming matcher, cuda_akaze.cu:1843-1967 and AKAZE.cpp:36-79: two
 * matches per query, the closest and second-closest train rows with ties to
 * the lower train index (the cv::BFMatcher knnMatch rule); a missing match is
 * {trainIdx 0, distance 512}. */
int ako_bfmatch(const uint8_t *q, int nq, const uint8_t *t, int nt, int row_bytes, ako_dmatch *out)
{
  if (nq < 0 || nt < 0 || row_bytes < 1 || row_bytes > 64) return -1;
  /* Rows zero-padded to 8 64-bit words: the Hamming distance is the sum of
   * the words' xor popcounts, the same integer as the byte-wise sum. */
  uint64_t *tw = (uint64_t *)calloc((size_t)(nt > 0 ? nt : 1) * 8, sizeof(uint64_t));
  if (!tw) return -1;
  for (int j = 0; j < nt; j++) memcpy(tw + (size_t)j * 8, t + (size_t)j * row_bytes, (size_t)row_bytes);
  int i;
#pragma omp parallel for schedule(dynamic, 64)
  for (i = 0; i < nq; i++) {
    uint64_t a[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    memcpy(a, q + (size_t)i * row_bytes, (size_t)row_bytes);
    int bd = 512, bi = 0, sd = 512, si = 0;
    for (int j = 0; j < nt; j++) {
      const uint64_t *b = tw + (size_t)j * 8;
      int d = 0;
      for (int k = 0; k < 8; k++) d += __builtin_popcountll(a[k] ^ b[k]);
      if (d < bd) {
        sd = bd;
        si = bi;
        bd = d;
        bi = j;
      } else if (d < sd) {
        sd = d;
        si = j;
      }
    }
    out[2 * i] = (ako_dmatch){i, bi, 0, (float)bd};
    out[2 * i + 1] = (ako_dmatch){i, si, 0, (float)sd};
  }
  free(tw);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* The shared float routines, exported so tests can check them on the host. */
float ako_atan2f(float y, float x) { return akz_atan2f(y, x); }
void ako_sincosf(float x, float *s, float *c) { akz_sincosf(x, s, c); }
float ako_expf(float x) { return akz_expf(x); }
float ako_recip1pf(float f) { return akz_recip1pf(f); }

/* The 486 comparison pairs of the M-LDB bits in bit order (test hook). */
int ako_descriptor_pairs(int *i1, int *i2) { return ako_cmp_pairs(i1, i2); }
