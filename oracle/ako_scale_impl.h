/*
 * ako_scale_impl.h - nonlinear scale-space stages of the oracle, written once
 * and instantiated twice by akaze_oracle.c: REAL=float (the reference CPU
 * semantics, including its double-precision intermediates) and REAL=double
 * (the FP64 oracle used for the per-level error report).
 *
 * TEST INFRASTRUCTURE ONLY (see akaze_oracle.h).
 *
 * Evaluation orders are fixed and shared with the GPU kernels:
 *  - separable Gaussian: horizontal pass, then vertical pass, each
 *    acc = k[0]*(v[-R]+v[R]); acc += k[R-d]*(v[-d]+v[d]) for d=R-1..1;
 *    acc += k[R]*v[0]; replicate border (cv::BORDER_REPLICATE).
 *  - Scharr (scale 1, cv::BORDER_DEFAULT = reflect-101), horizontal filter
 *    first as cv::sepFilter2D does:
 *    Lx = 3*(rx[y-1]+rx[y+1]) + 10*rx[y], rx[y'] = s[y'][x+1]-s[y'][x-1];
 *    Ly = sy[y+1] - sy[y-1], sy[y'] = 3*(s[y'][x-1]+s[y'][x+1]) + 10*s[y'][x].
 */

#define AKO_CAT2(a, b) a##b
#define AKO_CAT(a, b) AKO_CAT2(a, b)
#define AKO_F(name) AKO_CAT(name, AKO_SFX)

/* nldiffusion_functions.cpp:29-47 through cv::GaussianBlur. */
static void AKO_F(ako_gauss)(const REAL *src, REAL *dst, REAL *tmp, int w, int h, const REAL *k, int R)
{
  int y;
#pragma omp parallel for schedule(static)
  for (y = 0; y < h; y++) {
    const REAL *s = src + (size_t)y * w;
    REAL *t = tmp + (size_t)y * w;
    for (int x = 0; x < w; x++) {
      REAL acc;
      if (R > 0) {
        acc = k[0] * (s[ako_clampi(x - R, 0, w - 1)] + s[ako_clampi(x + R, 0, w - 1)]);
        for (int d = R - 1; d >= 1; d--)
          acc = acc + k[R - d] * (s[ako_clampi(x - d, 0, w - 1)] + s[ako_clampi(x + d, 0, w - 1)]);
        acc = acc + k[R] * s[x];
      } else {
        acc = k[0] * s[x];
      }
      t[x] = acc;
    }
  }
#pragma omp parallel for schedule(static)
  for (y = 0; y < h; y++) {
    REAL *o = dst + (size_t)y * w;
    for (int x = 0; x < w; x++) {
      REAL acc;
      if (R > 0) {
        acc = k[0] * (tmp[(size_t)ako_clampi(y - R, 0, h - 1) * w + x] + tmp[(size_t)ako_clampi(y + R, 0, h - 1) * w + x]);
        for (int d = R - 1; d >= 1; d--)
          acc = acc + k[R - d] * (tmp[(size_t)ako_clampi(y - d, 0, h - 1) * w + x] + tmp[(size_t)ako_clampi(y + d, 0, h - 1) * w + x]);
        acc = acc + k[R] * tmp[(size_t)y * w + x];
      } else {
        acc = k[0] * tmp[(size_t)y * w + x];
      }
      o[x] = acc;
    }
  }
}

/* nldiffusion_functions.cpp:50-53 (cv::Scharr, xorder/yorder 1, scale 1). */
static void AKO_F(ako_scharr)(const REAL *s, REAL *lx, REAL *ly, int w, int h)
{
  int y;
#pragma omp parallel for schedule(static)
  for (y = 0; y < h; y++) {
    const int ym = ako_refl101(y - 1, h), yp = ako_refl101(y + 1, h);
    const REAL *rm = s + (size_t)ym * w, *r0 = s + (size_t)y * w, *rp = s + (size_t)yp * w;
    for (int x = 0; x < w; x++) {
      const int xm = ako_refl101(x - 1, w), xp = ako_refl101(x + 1, w);
      const REAL rxm = rm[xp] - rm[xm];
      const REAL rx0 = r0[xp] - r0[xm];
      const REAL rxp = rp[xp] - rp[xm];
      lx[(size_t)y * w + x] = (REAL)3 * (rxm + rxp) + (REAL)10 * rx0;
      const REAL syp = (REAL)3 * (rp[xm] + rp[xp]) + (REAL)10 * rp[x];
      const REAL sym = (REAL)3 * (rm[xm] + rm[xp]) + (REAL)10 * rm[x];
      ly[(size_t)y * w + x] = syp - sym;
    }
  }
}

/* nldiffusion_functions.cpp:121-201, compute_k_percentile(img, perc, gscale,
 * nbins, 0, 0), written with the reference's own types: the histogram and
 * npoints are float, the counters size_t. */
static REAL AKO_F(ako_k_percentile)(const REAL *img, int w, int h, REAL perc, int nbins, const REAL *taps, int R,
                                    REAL *g, REAL *lx, REAL *ly, REAL *tmp)
{
  size_t nbin = 0, nelements = 0, nthreshold = 0, k = 0;
  REAL kperc = 0, modg = 0, npoints = 0, hmax = 0;
  REAL *hist = (REAL *)calloc((size_t)nbins, sizeof(REAL));
  AKO_F(ako_gauss)(img, g, tmp, w, h, taps, R);
  AKO_F(ako_scharr)(g, lx, ly, w, h);
  for (int y = 1; y < h - 1; y++) {
    for (int x = 1; x < w - 1; x++) {
      const size_t p = (size_t)y * w + x;
      modg = lx[p] * lx[p] + ly[p] * ly[p];
      if (modg > hmax) hmax = modg;
    }
  }
  hmax = AKO_SQRT(hmax);
  for (int y = 1; y < h - 1; y++) {
    for (int x = 1; x < w - 1; x++) {
      const size_t p = (size_t)y * w + x;
      modg = AKO_SQRT(lx[p] * lx[p] + ly[p] * ly[p]);
      if (modg != 0.0) {
        nbin = (size_t)AKO_FLOOR((REAL)nbins * (modg / hmax));
        if (nbin == (size_t)nbins) nbin--;
        hist[nbin]++;
        npoints++;
      }
    }
  }
  nthreshold = (size_t)(npoints * perc);
  for (k = 0; nelements < nthreshold && k < (size_t)nbins; k++) nelements = (size_t)((REAL)nelements + hist[k]);
  if (nelements < nthreshold)
    kperc = (REAL)0.03;
  else
    kperc = hmax * ((REAL)k / (REAL)nbins);
  free(hist);
  return kperc;
}

/* Conductance, nldiffusion_functions.cpp:56-118 (PM_G2 is :72-83). */
static void AKO_F(ako_conductance)(const REAL *lx, const REAL *ly, REAL *dst, size_t n, REAL k, int type)
{
  const REAL inv_k = (REAL)(1.0 / (k * k));
  long i;
#pragma omp parallel for schedule(static)
  for (i = 0; i < (long)n; i++) {
    const REAL m = lx[i] * lx[i] + ly[i] * ly[i];
    if (type == 1) {
      dst[i] = (REAL)(1.0 / (1.0 + inv_k * m));
    } else if (type == 0) {
      dst[i] = AKO_EXP(-inv_k * m);
    } else if (type == 2) {
      const REAL dL = inv_k * m;
      const REAL t = (REAL)(-3.315 / (dL * dL * dL * dL));
      dst[i] = (REAL)(1.0 - AKO_EXP(t));
    } else {
      const REAL den = (REAL)sqrt(1.0 + inv_k * m);
      dst[i] = (REAL)(1.0 / den);
    }
  }
}

/* One FED step, nldiffusion_functions.cpp:213-317, written the way the
 * reference writes it: separate formulas for the image border, the step
 * 0.5*stepsize*(...) evaluated in double, then Ld += Lstep. */
static void AKO_F(ako_nld_step)(REAL *Ld, const REAL *c, REAL *Lstep, int cols, int rows, float stepsize)
{
  int y;
#define AKO_AT(P, yy, xx) (P)[(size_t)(yy) * cols + (xx)]
#pragma omp parallel for schedule(static)
  for (y = 1; y < rows - 1; y++) {
    for (int x = 1; x < cols - 1; x++) {
      const REAL xpos = (AKO_AT(c, y, x) + AKO_AT(c, y, x + 1)) * (AKO_AT(Ld, y, x + 1) - AKO_AT(Ld, y, x));
      const REAL xneg = (AKO_AT(c, y, x - 1) + AKO_AT(c, y, x)) * (AKO_AT(Ld, y, x) - AKO_AT(Ld, y, x - 1));
      const REAL ypos = (AKO_AT(c, y, x) + AKO_AT(c, y + 1, x)) * (AKO_AT(Ld, y + 1, x) - AKO_AT(Ld, y, x));
      const REAL yneg = (AKO_AT(c, y - 1, x) + AKO_AT(c, y, x)) * (AKO_AT(Ld, y, x) - AKO_AT(Ld, y - 1, x));
      AKO_AT(Lstep, y, x) = (REAL)(0.5 * stepsize * (xpos - xneg + ypos - yneg));
    }
  }
  /* first row (neighbour below is row 1), then last row (neighbour row rows-2) */
  for (int pass = 0; pass < 2; pass++) {
    const int r = pass == 0 ? 0 : rows - 1;
    const int rp = pass == 0 ? 1 : rows - 2;
    for (int x = 1; x < cols - 1; x++) {
      const REAL xpos = (AKO_AT(c, r, x) + AKO_AT(c, r, x + 1)) * (AKO_AT(Ld, r, x + 1) - AKO_AT(Ld, r, x));
      const REAL xneg = (AKO_AT(c, r, x - 1) + AKO_AT(c, r, x)) * (AKO_AT(Ld, r, x) - AKO_AT(Ld, r, x - 1));
      const REAL ypos = (AKO_AT(c, r, x) + AKO_AT(c, rp, x)) * (AKO_AT(Ld, rp, x) - AKO_AT(Ld, r, x));
      AKO_AT(Lstep, r, x) = (REAL)(0.5 * stepsize * (xpos - xneg + ypos));
    }
    {
      const REAL xpos = (AKO_AT(c, r, 0) + AKO_AT(c, r, 1)) * (AKO_AT(Ld, r, 1) - AKO_AT(Ld, r, 0));
      const REAL ypos = (AKO_AT(c, r, 0) + AKO_AT(c, rp, 0)) * (AKO_AT(Ld, rp, 0) - AKO_AT(Ld, r, 0));
      AKO_AT(Lstep, r, 0) = (REAL)(0.5 * stepsize * (xpos + ypos));
    }
    {
      const int x = cols - 1;
      const REAL xneg = (AKO_AT(c, r, x - 1) + AKO_AT(c, r, x)) * (AKO_AT(Ld, r, x) - AKO_AT(Ld, r, x - 1));
      const REAL ypos = (AKO_AT(c, r, x) + AKO_AT(c, rp, x)) * (AKO_AT(Ld, rp, x) - AKO_AT(Ld, r, x));
      AKO_AT(Lstep, r, x) = (REAL)(0.5 * stepsize * (-xneg + ypos));
    }
  }
  /* first and last columns */
  for (int i = 1; i < rows - 1; i++) {
    {
      const REAL xpos = (AKO_AT(c, i, 0) + AKO_AT(c, i, 1)) * (AKO_AT(Ld, i, 1) - AKO_AT(Ld, i, 0));
      const REAL ypos = (AKO_AT(c, i, 0) + AKO_AT(c, i + 1, 0)) * (AKO_AT(Ld, i + 1, 0) - AKO_AT(Ld, i, 0));
      const REAL yneg = (AKO_AT(c, i - 1, 0) + AKO_AT(c, i, 0)) * (AKO_AT(Ld, i, 0) - AKO_AT(Ld, i - 1, 0));
      AKO_AT(Lstep, i, 0) = (REAL)(0.5 * stepsize * (xpos + ypos - yneg));
    }
    {
      const int x = cols - 1;
      const REAL xneg = (AKO_AT(c, i, x - 1) + AKO_AT(c, i, x)) * (AKO_AT(Ld, i, x) - AKO_AT(Ld, i, x - 1));
      const REAL ypos = (AKO_AT(c, i, x) + AKO_AT(c, i + 1, x)) * (AKO_AT(Ld, i + 1, x) - AKO_AT(Ld, i, x));
      const REAL yneg = (AKO_AT(c, i - 1, x) + AKO_AT(c, i, x)) * (AKO_AT(Ld, i, x) - AKO_AT(Ld, i - 1, x));
      AKO_AT(Lstep, i, x) = (REAL)(0.5 * stepsize * (-xneg + ypos - yneg));
    }
  }
#undef AKO_AT
  long p;
#pragma omp parallel for schedule(static)
  for (p = 0; p < (long)rows * cols; p++) Ld[p] = Ld[p] + Lstep[p];
}

/* nldiffusion_functions.cpp:320-324, cv::resize(INTER_AREA) to the next
 * octave's size.  Exact 2x: the area-fast path 0.25*(((a+b)+c)+d).  Other
 * ratios: the pixel-area weights of INTER_AREA (per-axis tables built by
 * ako_area_tab), horizontal sum per source row, then the weighted row sum. */
static void AKO_F(ako_halfsample)(const REAL *src, int sw, int sh, REAL *dst, int dw, int dh)
{
  if (sw == 2 * dw && sh == 2 * dh) {
    int y;
#pragma omp parallel for schedule(static)
    for (y = 0; y < dh; y++) {
      for (int x = 0; x < dw; x++) {
        const REAL *p0 = src + (size_t)(2 * y) * sw + 2 * x;
        const REAL *p1 = p0 + sw;
        dst[(size_t)y * dw + x] = (REAL)0.25 * (((p0[0] + p0[1]) + p1[0]) + p1[1]);
      }
    }
    return;
  }
  ako_area_table tx, ty;
  ako_area_tab(sw, dw, &tx);
  ako_area_tab(sh, dh, &ty);
  REAL *row = (REAL *)malloc(sizeof(REAL) * (size_t)dw);
  for (int dy = 0; dy < dh; dy++) {
    REAL *o = dst + (size_t)dy * dw;
    int first_y = 1;
    for (int ky = ty.start[dy]; ky < ty.start[dy + 1]; ky++) {
      const REAL *s = src + (size_t)ty.si[ky] * sw;
      const REAL beta = (REAL)ty.alpha[ky];
      for (int dx = 0; dx < dw; dx++) {
        REAL acc = 0;
        int first_x = 1;
        for (int kx = tx.start[dx]; kx < tx.start[dx + 1]; kx++) {
          const REAL v = (REAL)tx.alpha[kx] * s[tx.si[kx]];
          acc = first_x ? v : acc + v;
          first_x = 0;
        }
        row[dx] = acc;
      }
      for (int dx = 0; dx < dw; dx++) o[dx] = first_y ? beta * row[dx] : o[dx] + beta * row[dx];
      first_y = 0;
    }
  }
  free(row);
  ako_area_free(&tx);
  ako_area_free(&ty);
}

#undef AKO_F
