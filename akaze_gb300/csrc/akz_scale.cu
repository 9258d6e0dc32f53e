/*
 * akz_scale.cu - nonlinear scale space on sm_103a.
 *
 *   contrast  (nldiffusion_functions.cpp:121-201): sigma-1 Gaussian of the
 *             input, Scharr gradient, max |grad|^2 (pass 0) and the histogram
 *             of |grad|/max (pass 1), recomputed from the u8 tile each pass;
 *             the percentile is evaluated on the device with the reference's
 *             float arithmetic (no host round trip).
 *   level 0   (AKAZE.cpp:234): soffset Gaussian of the input.
 *   level i   (AKAZE.cpp:244-270): one fused kernel per FED chunk. The first
 *             chunk reads the predecessor level (or its 2x half-sample), forms
 *             the sigma-1 smoothing Lsmooth, the Scharr gradient and the PM-g2
 *             conductance in shared memory and then runs up to AKZ_MAX_CHUNK
 *             explicit FED steps on the tile (temporal blocking: the tile
 *             carries a halo of one pixel per step), writing only the final
 *             level, Lsmooth and (when more chunks follow) the conductance.
 *
 * Bytes that must cross HBM per level pixel: predecessor read (4 B, 16 B at
 * an octave start), Lt write (4 B), Lsmooth write (4 B).
 */
#include <cuda_runtime.h>

#include "akz_device.cuh"
#include "akz_fmath.h"

/* ------------------------------------------------------------------------ */
/* Contrast factor                                                          */

template <int PASS>
__global__ void __launch_bounds__(256) k_contrast(akz_contrast_params p)
{
  constexpr int TW = AKZ_CONTRAST_TW, TH = AKZ_CONTRAST_TH;
  constexpr int PW = TW + 6, PH = TH + 6; /* input region: tile +- 3 */
  constexpr int GW = TW + 2, GH = TH + 2; /* Gaussian region: tile +- 1 */
  __shared__ float sP[PH * PW];
  __shared__ float sT[PH * GW];
  __shared__ float sG[GH * GW];
  __shared__ unsigned int sHist[PASS == 1 ? AKZ_MAX_NBINS : 1];
  __shared__ float sRed[8];

  const int tid = threadIdx.x;
  const int si = akz_find_seg(p.segs, p.nsegs, blockIdx.x);
  const akz_tile_seg sg = p.segs[si];
  const int img = sg.level_desc;
  const akz_image_desc I = p.t.im[img];
  const int W = I.width, H = I.height;
  const int lt = blockIdx.x - sg.tile_begin;
  const int tx0 = (lt % sg.tiles_x) * TW, ty0 = (lt / sg.tiles_x) * TH;
  const int gx0 = max(tx0 - 1, 0), gx1 = min(tx0 + TW + 1, W), gy0 = max(ty0 - 1, 0), gy1 = min(ty0 + TH + 1, H);
  const int px0 = max(gx0 - 2, 0), px1 = min(gx1 + 2, W), py0 = max(gy0 - 2, 0), py1 = min(gy1 + 2, H);

  if (PASS == 1)
    for (int b = tid; b < p.nbins; b += 256) sHist[b] = 0;
  for (int i = tid; i < (py1 - py0) * (px1 - px0); i += 256) {
    const int y = py0 + i / (px1 - px0), x = px0 + i % (px1 - px0);
    sP[(y - py0) * PW + (x - px0)] = akz_fetch_input(p.t, I, x, y, p.inv255);
  }
  __syncthreads();
  const float k0 = p.taps[0], k1 = p.taps[1], k2 = p.taps[2];
  for (int i = tid; i < (py1 - py0) * (gx1 - gx0); i += 256) {
    const int y = py0 + i / (gx1 - gx0), x = gx0 + i % (gx1 - gx0);
    const float *r = sP + (y - py0) * PW - px0;
    float acc = k0 * (r[max(x - 2, 0)] + r[min(x + 2, W - 1)]);
    acc = acc + k1 * (r[max(x - 1, 0)] + r[min(x + 1, W - 1)]);
    acc = acc + k2 * r[x];
    sT[(y - py0) * GW + (x - gx0)] = acc;
  }
  __syncthreads();
  for (int i = tid; i < (gy1 - gy0) * (gx1 - gx0); i += 256) {
    const int y = gy0 + i / (gx1 - gx0), x = gx0 + i % (gx1 - gx0);
    const float *c = sT + (x - gx0) - py0 * GW;
    float acc = k0 * (c[max(y - 2, 0) * GW] + c[min(y + 2, H - 1) * GW]);
    acc = acc + k1 * (c[max(y - 1, 0) * GW] + c[min(y + 1, H - 1) * GW]);
    acc = acc + k2 * c[y * GW];
    sG[(y - gy0) * GW + (x - gx0)] = acc;
  }
  __syncthreads();

  const int ix0 = max(tx0, 1), ix1 = min(tx0 + TW, W - 1), iy0 = max(ty0, 1), iy1 = min(ty0 + TH, H - 1);
  float mx = 0.0f, hmax = 0.0f;
  if (PASS == 1) hmax = sqrtf(__uint_as_float(p.t.stats[img].hmax2_bits));
  const float nb = (float)p.nbins;
  for (int i = tid; i < max(iy1 - iy0, 0) * max(ix1 - ix0, 0); i += 256) {
    const int y = iy0 + i / (ix1 - ix0), x = ix0 + i % (ix1 - ix0);
    const float *rm = sG + (y - 1 - gy0) * GW - gx0, *r0 = sG + (y - gy0) * GW - gx0, *rp = sG + (y + 1 - gy0) * GW - gx0;
    const float rxm = rm[x + 1] - rm[x - 1];
    const float rx0 = r0[x + 1] - r0[x - 1];
    const float rxp = rp[x + 1] - rp[x - 1];
    const float lx = 3.0f * (rxm + rxp) + 10.0f * rx0;
    const float syp = 3.0f * (rp[x - 1] + rp[x + 1]) + 10.0f * rp[x];
    const float sym = 3.0f * (rm[x - 1] + rm[x + 1]) + 10.0f * rm[x];
    const float ly = syp - sym;
    if (PASS == 0) {
      const float m = lx * lx + ly * ly;
      mx = fmaxf(mx, m);
    } else {
      const float modg = sqrtf(lx * lx + ly * ly);
      if (modg != 0.0f) {
        int nbin = (int)floorf(nb * (modg / hmax));
        if (nbin == p.nbins) nbin--;
        atomicAdd(&sHist[nbin], 1u);
      }
    }
  }
  if (PASS == 0) {
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((tid & 31) == 0) sRed[tid >> 5] = mx;
    __syncthreads();
    if (tid == 0) {
      float m = sRed[0];
      for (int w = 1; w < 8; w++) m = fmaxf(m, sRed[w]);
      atomicMax(&p.t.stats[img].hmax2_bits, __float_as_uint(m));
    }
  } else {
    __syncthreads();
    for (int b = tid; b < p.nbins; b += 256)
      if (sHist[b]) atomicAdd(&p.hist[(long long)img * p.nbins + b], sHist[b]);
  }
}

/* Percentile and per-octave factors, with the reference's types: histogram
 * and point count as float (exact up to 2^24), counters as size_t. */
__global__ void k_contrast_final(akz_tables t, const unsigned int *hist, int nbins, float perc, float2 *kc)
{
  const int img = blockIdx.x * blockDim.x + threadIdx.x;
  if (img >= t.nimg) return;
  const float hmax = sqrtf(__uint_as_float(t.stats[img].hmax2_bits));
  const unsigned int *h = hist + (long long)img * nbins;
  unsigned long long tot = 0;
  for (int b = 0; b < nbins; b++) tot += h[b];
  const float npoints = tot >= (1ull << 24) ? 16777216.0f : (float)tot;
  const unsigned long long nthreshold = (unsigned long long)(npoints * perc);
  unsigned long long nelements = 0;
  int k;
  for (k = 0; nelements < nthreshold && k < nbins; k++) {
    const float hk = h[k] >= (1u << 24) ? 16777216.0f : (float)h[k];
    nelements = (unsigned long long)((float)nelements + hk);
  }
  float kperc;
  if (nelements < nthreshold)
    kperc = (float)0.03;
  else
    kperc = hmax * ((float)k / (float)nbins);
  t.stats[img].kcontrast = kperc;
  float kk = kperc;
  for (int o = 0; o < 16; o++) {
    kc[img * 16 + o] = make_float2(kk, (float)(1.0 / (double)(kk * kk)));
    kk = (float)((double)kk * 0.75);
  }
}

/* ------------------------------------------------------------------------ */
/* Level 0: soffset Gaussian of the input (replicate border).               */

__global__ void __launch_bounds__(256) k_gauss0(akz_gauss_params p)
{
  constexpr int TW = AKZ_GAUSS_TW, TH = AKZ_GAUSS_TH;
  extern __shared__ float sm[];
  const int R = p.R;
  const int PW = TW + 2 * R;
  float *sP = sm;                        /* (TH+2R) x (TW+2R) */
  float *sT = sm + (TH + 2 * R) * PW;    /* (TH+2R) x TW */
  const int tid = threadIdx.x;
  const int si = akz_find_seg(p.segs, p.nsegs, blockIdx.x);
  const akz_tile_seg sg = p.segs[si];
  const akz_level_desc L = p.t.lv[sg.level_desc];
  const akz_image_desc I = p.t.im[L.image];
  const int W = L.width, H = L.height;
  const int lt = blockIdx.x - sg.tile_begin;
  const int tx0 = (lt % sg.tiles_x) * TW, ty0 = (lt / sg.tiles_x) * TH;
  const int tx1 = min(tx0 + TW, W), ty1 = min(ty0 + TH, H);
  const int px0 = max(tx0 - R, 0), px1 = min(tx1 + R, W), py0 = max(ty0 - R, 0), py1 = min(ty1 + R, H);
  for (int i = tid; i < (py1 - py0) * (px1 - px0); i += 256) {
    const int y = py0 + i / (px1 - px0), x = px0 + i % (px1 - px0);
    sP[(y - py0) * PW + (x - px0)] = akz_fetch_input(p.t, I, x, y, p.inv255);
  }
  __syncthreads();
  for (int i = tid; i < (py1 - py0) * (tx1 - tx0); i += 256) {
    const int y = py0 + i / (tx1 - tx0), x = tx0 + i % (tx1 - tx0);
    const float *r = sP + (y - py0) * PW - px0;
    float acc;
    if (R > 0) {
      acc = p.taps[0] * (r[max(x - R, 0)] + r[min(x + R, W - 1)]);
      for (int d = R - 1; d >= 1; d--) acc = acc + p.taps[R - d] * (r[max(x - d, 0)] + r[min(x + d, W - 1)]);
      acc = acc + p.taps[R] * r[x];
    } else {
      acc = p.taps[0] * r[x];
    }
    sT[(y - py0) * TW + (x - tx0)] = acc;
  }
  __syncthreads();
  float *out = p.t.planes + L.lt;
  for (int i = tid; i < (ty1 - ty0) * (tx1 - tx0); i += 256) {
    const int y = ty0 + i / (tx1 - tx0), x = tx0 + i % (tx1 - tx0);
    const float *c = sT + (x - tx0) - py0 * TW;
    float acc;
    if (R > 0) {
      acc = p.taps[0] * (c[max(y - R, 0) * TW] + c[min(y + R, H - 1) * TW]);
      for (int d = R - 1; d >= 1; d--) acc = acc + p.taps[R - d] * (c[max(y - d, 0) * TW] + c[min(y + d, H - 1) * TW]);
      acc = acc + p.taps[R] * c[y * TW];
    } else {
      acc = p.taps[0] * c[y * TW];
    }
    out[(long long)y * L.pitch + x] = acc;
  }
}

/* ------------------------------------------------------------------------ */
/* Level i >= 1: Lsmooth, conductance and a chunk of FED steps per tile.     */

__device__ __forceinline__ float akz_conductance(float lx, float ly, float inv_k, int type)
{
  const float m = lx * lx + ly * ly;
  if (type == 1) return akz_recip1pf(inv_k * m);
  if (type == 0) return akz_expf(-inv_k * m);
  if (type == 2) {
    const float dL = inv_k * m;
    const float t = (float)(-3.315 / (double)(dL * dL * dL * dL));
    return (float)(1.0 - (double)akz_expf(t));
  }
  const float den = (float)sqrt(1.0 + (double)(inv_k * m));
  return (float)(1.0 / (double)den);
}

/* One explicit FED step over [ax0,ax1)x[ay0,ay1) with replicate borders
 * (the reference's border formulas of nld_step_scalar equal the generic
 * formula with clamped neighbours: a clamped difference is exactly zero). */
__device__ __forceinline__ void akz_fed_step(const akz_smem_acc &src, float *dst, int dx0, int dy0, int dstride,
                                             const float *g, int gx0, int gy0, int gstride, int ax0, int ax1, int ay0,
                                             int ay1, int W, int H, float h)
{
  for (int y = ay0 + (int)threadIdx.y; y < ay1; y += 8) {
    const int ym = max(y - 1, 0), yp = min(y + 1, H - 1);
    const float *gr = g + (y - gy0) * gstride - gx0;
    const float *gm = g + (ym - gy0) * gstride - gx0;
    const float *gp = g + (yp - gy0) * gstride - gx0;
    for (int x = ax0 + (int)threadIdx.x; x < ax1; x += 32) {
      const int xm = max(x - 1, 0), xp = min(x + 1, W - 1);
      const float Lc = src(x, y), Le = src(xp, y), Lw = src(xm, y), Ls = src(x, yp), Ln = src(x, ym);
      const float gc = gr[x];
      const float xpos = (gc + gr[xp]) * (Le - Lc);
      const float xneg = (gr[xm] + gc) * (Lc - Lw);
      const float ypos = (gc + gp[x]) * (Ls - Lc);
      const float yneg = (gm[x] + gc) * (Lc - Ln);
      const float step = h * (xpos - xneg + ypos - yneg);
      dst[(y - dy0) * dstride + (x - dx0)] = Lc + step;
    }
  }
}

size_t akz_fed_smem_bytes(int tw, int th, int d, int first)
{
  const size_t r0 = (size_t)(tw + 2 * d) * (th + 2 * d);
  if (!first) return 3 * r0 * sizeof(float);
  const size_t P = (size_t)(tw + 2 * d + 6) * (th + 2 * d + 6);
  const size_t T = (size_t)(th + 2 * d + 6) * (tw + 2 * d + 2);
  const size_t S = (size_t)(tw + 2 * d + 2) * (th + 2 * d + 2);
  return (P + T + S + r0) * sizeof(float);
}

template <int TW, int TH>
__global__ void __launch_bounds__(256) k_fed(akz_fed_params p)
{
  extern __shared__ float sm[];
  const int tid = threadIdx.y * 32 + threadIdx.x;
  const int si = akz_find_seg(p.segs, p.nsegs, blockIdx.x);
  const akz_tile_seg sg = p.segs[si];
  const akz_level_desc L = p.t.lv[sg.level_desc];
  const akz_image_desc I = p.t.im[L.image];
  const int W = L.width, H = L.height;
  const int lt = blockIdx.x - sg.tile_begin;
  const int tx0 = (lt % sg.tiles_x) * TW, ty0 = (lt / sg.tiles_x) * TH;
  const int tx1 = min(tx0 + TW, W), ty1 = min(ty0 + TH, H);
  const int d = p.steps;
  const int srck = p.first ? sg.aux : p.src; /* first chunk: per-image source kind */
  const int rx0 = max(tx0 - d, 0), rx1 = min(tx1 + d, W), ry0 = max(ty0 - d, 0), ry1 = min(ty1 + d, H);
  const int rw = rx1 - rx0;
  float *planes = p.t.planes;

  float *gbuf, *bufA, *bufB;
  akz_smem_acc src;
  if (p.first) {
    const int sx0 = max(rx0 - 1, 0), sx1 = min(rx1 + 1, W), sy0 = max(ry0 - 1, 0), sy1 = min(ry1 + 1, H);
    const int px0 = max(sx0 - 2, 0), px1 = min(sx1 + 2, W), py0 = max(sy0 - 2, 0), py1 = min(sy1 + 2, H);
    const int PWm = TW + 2 * d + 6, PHm = TH + 2 * d + 6, SWm = TW + 2 * d + 2, SHm = TH + 2 * d + 2;
    float *sP = sm;
    float *sT = sP + PWm * PHm;
    float *sS = sT + PHm * SWm;
    gbuf = sS + SWm * SHm;
    const int pw = px1 - px0, sw = sx1 - sx0;
    /* predecessor: same-size copy, exact 2x half-sample, or a prepared plane */
    if (srck == 1) {
      const akz_level_desc Lp = p.t.lv[sg.level_desc - 1];
      const float *pp = planes + Lp.lt;
      for (int i = tid; i < (py1 - py0) * pw; i += 256) {
        const int y = py0 + i / pw, x = px0 + i % pw;
        const float *q0 = pp + (long long)(2 * y) * Lp.pitch + 2 * x;
        const float *q1 = q0 + Lp.pitch;
        sP[(y - py0) * pw + (x - px0)] = 0.25f * (((__ldg(q0) + __ldg(q0 + 1)) + __ldg(q1)) + __ldg(q1 + 1));
      }
    } else {
      const float *pp;
      long long pitch;
      if (srck == 0) {
        const akz_level_desc Lp = p.t.lv[sg.level_desc - 1];
        pp = planes + Lp.lt;
        pitch = Lp.pitch;
      } else {
        pp = planes + I.t2;
        pitch = L.pitch;
      }
      for (int i = tid; i < (py1 - py0) * pw; i += 256) {
        const int y = py0 + i / pw, x = px0 + i % pw;
        sP[(y - py0) * pw + (x - px0)] = __ldg(pp + (long long)y * pitch + x);
      }
    }
    __syncthreads();
    const float k0 = p.taps1[0], k1 = p.taps1[1], k2 = p.taps1[2];
    for (int i = tid; i < (py1 - py0) * sw; i += 256) {
      const int y = py0 + i / sw, x = sx0 + i % sw;
      const float *r = sP + (y - py0) * pw - px0;
      float acc = k0 * (r[max(x - 2, 0)] + r[min(x + 2, W - 1)]);
      acc = acc + k1 * (r[max(x - 1, 0)] + r[min(x + 1, W - 1)]);
      acc = acc + k2 * r[x];
      sT[(y - py0) * sw + (x - sx0)] = acc;
    }
    __syncthreads();
    float *lsp = planes + L.ls;
    for (int i = tid; i < (sy1 - sy0) * sw; i += 256) {
      const int y = sy0 + i / sw, x = sx0 + i % sw;
      const float *c = sT + (x - sx0) - py0 * sw;
      float acc = k0 * (c[max(y - 2, 0) * sw] + c[min(y + 2, H - 1) * sw]);
      acc = acc + k1 * (c[max(y - 1, 0) * sw] + c[min(y + 1, H - 1) * sw]);
      acc = acc + k2 * c[y * sw];
      sS[(y - sy0) * sw + (x - sx0)] = acc;
      if (x >= tx0 && x < tx1 && y >= ty0 && y < ty1) lsp[(long long)y * L.pitch + x] = acc;
    }
    __syncthreads();
    const float inv_k = p.kc[L.image * 16 + L.octave].y;
    float *gp = planes + I.g;
    for (int i = tid; i < (ry1 - ry0) * rw; i += 256) {
      const int y = ry0 + i / rw, x = rx0 + i % rw;
      const int xm = akz_refl101(x - 1, W), xp = akz_refl101(x + 1, W);
      const int ym = akz_refl101(y - 1, H), yp = akz_refl101(y + 1, H);
      const float *rm = sS + (ym - sy0) * sw - sx0, *r0 = sS + (y - sy0) * sw - sx0, *rp = sS + (yp - sy0) * sw - sx0;
      const float hm = rm[xp] - rm[xm];
      const float h0 = r0[xp] - r0[xm];
      const float hp = rp[xp] - rp[xm];
      const float lx = 3.0f * (hm + hp) + 10.0f * h0;
      const float syp = 3.0f * (rp[xm] + rp[xp]) + 10.0f * rp[x];
      const float sym = 3.0f * (rm[xm] + rm[xp]) + 10.0f * rm[x];
      const float ly = syp - sym;
      const float gv = akz_conductance(lx, ly, inv_k, p.diffusivity);
      gbuf[(y - ry0) * rw + (x - rx0)] = gv;
      if (p.write_g && x >= tx0 && x < tx1 && y >= ty0 && y < ty1) gp[(long long)y * L.pitch + x] = gv;
    }
    __syncthreads();
    src = akz_smem_acc{sP, px0, py0, pw};
    bufA = sT; /* rowtmp region, free now, holds >= R0 */
    bufB = sS; /* smoothing region, free now */
  } else {
    gbuf = sm;
    bufA = sm + (TW + 2 * d) * (TH + 2 * d);
    bufB = bufA + (TW + 2 * d) * (TH + 2 * d);
    const float *lp = planes + (p.src == 1 ? I.t1 : I.t2);
    const float *gp = planes + I.g;
    for (int i = tid; i < (ry1 - ry0) * rw; i += 256) {
      const int y = ry0 + i / rw, x = rx0 + i % rw;
      bufB[(y - ry0) * rw + (x - rx0)] = __ldg(lp + (long long)y * L.pitch + x);
      gbuf[(y - ry0) * rw + (x - rx0)] = __ldg(gp + (long long)y * L.pitch + x);
    }
    __syncthreads();
    src = akz_smem_acc{bufB, rx0, ry0, rw};
  }
  /* steps: write into bufA, then alternate */
  float *dstb = bufA, *other = bufB;
  for (int s = 1; s <= d; s++) {
    const int ax0 = max(tx0 - (d - s), 0), ax1 = min(tx1 + (d - s), W);
    const int ay0 = max(ty0 - (d - s), 0), ay1 = min(ty1 + (d - s), H);
    akz_fed_step(src, dstb, rx0, ry0, rw, gbuf, rx0, ry0, rw, ax0, ax1, ay0, ay1, W, H, p.h[s - 1]);
    __syncthreads();
    src = akz_smem_acc{dstb, rx0, ry0, rw};
    float *t = dstb;
    dstb = other;
    other = t;
  }
  float *out = planes + (p.dst == 0 ? L.lt : (p.dst == 1 ? I.t1 : I.t2));
  for (int i = tid; i < (ty1 - ty0) * (tx1 - tx0); i += 256) {
    const int y = ty0 + i / (tx1 - tx0), x = tx0 + i % (tx1 - tx0);
    out[(long long)y * L.pitch + x] = src(x, y);
  }
}

/* Half-sample by the INTER_AREA pixel-area tables when the predecessor is not
 * exactly twice the size; writes the level's starting image into T2. */
__global__ void k_area(akz_area_params p)
{
  const akz_area_seg sg = p.segs[blockIdx.z];
  const akz_level_desc L = p.t.lv[sg.ld];
  const akz_level_desc Lp = p.t.lv[sg.ld - 1];
  const akz_image_desc I = p.t.im[L.image];
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= L.width || y >= L.height) return;
  const int *xs = p.start + sg.xs, *ys = p.start + sg.ys;
  const int *xi = p.si, *yi = p.si;
  const float *xa = p.alpha, *ya = p.alpha;
  const float *src = p.t.planes + Lp.lt;
  float o = 0.0f;
  for (int ky = ys[y]; ky < ys[y + 1]; ky++) {
    const float *s = src + (long long)yi[ky] * Lp.pitch;
    float acc = 0.0f;
    for (int kx = xs[x]; kx < xs[x + 1]; kx++) {
      const float v = xa[kx] * s[xi[kx]];
      acc = kx == xs[x] ? v : acc + v;
    }
    const float t = ya[ky] * acc;
    o = ky == ys[y] ? t : o + t;
  }
  p.t.planes[I.t2 + (long long)y * L.pitch + x] = o;
}

/* ------------------------------------------------------------------------ */

cudaError_t akz_launch_contrast(const akz_contrast_params &p, int ntiles, int pass, cudaStream_t s)
{
  if (ntiles <= 0) return cudaSuccess;
  if (pass == 0)
    k_contrast<0><<<ntiles, 256, 0, s>>>(p);
  else
    k_contrast<1><<<ntiles, 256, 0, s>>>(p);
  return cudaGetLastError();
}

cudaError_t akz_launch_contrast_final(const akz_tables &t, const unsigned int *hist, int nbins, float perc, float2 *kc, cudaStream_t s)
{
  k_contrast_final<<<(t.nimg + 127) / 128, 128, 0, s>>>(t, hist, nbins, perc, kc);
  return cudaGetLastError();
}

cudaError_t akz_launch_gauss0(const akz_gauss_params &p, int ntiles, cudaStream_t s)
{
  if (ntiles <= 0) return cudaSuccess;
  const size_t smem = (size_t)((AKZ_GAUSS_TH + 2 * p.R) * (AKZ_GAUSS_TW + 2 * p.R) + (AKZ_GAUSS_TH + 2 * p.R) * AKZ_GAUSS_TW) * sizeof(float);
  cudaFuncSetAttribute(k_gauss0, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_gauss0<<<ntiles, 256, smem, s>>>(p);
  return cudaGetLastError();
}

cudaError_t akz_launch_fed(const akz_fed_params &p, int ntiles, int tw, int th, cudaStream_t s)
{
  if (ntiles <= 0) return cudaSuccess;
  const size_t smem = akz_fed_smem_bytes(tw, th, p.steps, p.first);
  const dim3 block(32, 8);
  if (tw == 128 && th == 32) {
    cudaFuncSetAttribute(k_fed<128, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_fed<128, 32><<<ntiles, block, smem, s>>>(p);
  } else if (tw == 64 && th == 32) {
    cudaFuncSetAttribute(k_fed<64, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_fed<64, 32><<<ntiles, block, smem, s>>>(p);
  } else if (tw == 64 && th == 64) {
    cudaFuncSetAttribute(k_fed<64, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_fed<64, 64><<<ntiles, block, smem, s>>>(p);
  } else {
    return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t akz_launch_area(const akz_area_params &p, int maxw, int maxh, cudaStream_t s)
{
  if (p.nsegs <= 0) return cudaSuccess;
  const dim3 block(32, 8);
  const dim3 grid((maxw + 31) / 32, (maxh + 7) / 8, p.nsegs);
  k_area<<<grid, block, 0, s>>>(p);
  return cudaGetLastError();
}
