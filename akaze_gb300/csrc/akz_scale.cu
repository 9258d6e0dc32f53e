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
  const int lane = tid & 31, warp = tid >> 5;
  for (int y = py0 + warp; y < py1; y += 8)
    for (int x = px0 + lane; x < px1; x += 32) sP[(y - py0) * PW + (x - px0)] = akz_fetch_input(p.t, I, x, y, p.inv255);
  __syncthreads();
  const float k0 = p.taps[0], k1 = p.taps[1], k2 = p.taps[2];
  for (int y = py0 + warp; y < py1; y += 8)
    for (int x = gx0 + lane; x < gx1; x += 32) {
    const float *r = sP + (y - py0) * PW - px0;
    float acc = k0 * (r[max(x - 2, 0)] + r[min(x + 2, W - 1)]);
    acc = acc + k1 * (r[max(x - 1, 0)] + r[min(x + 1, W - 1)]);
    acc = acc + k2 * r[x];
    sT[(y - py0) * GW + (x - gx0)] = acc;
  }
  __syncthreads();
  for (int y = gy0 + warp; y < gy1; y += 8)
    for (int x = gx0 + lane; x < gx1; x += 32) {
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
  for (int y = iy0 + warp; y < iy1; y += 8)
    for (int x = ix0 + lane; x < ix1; x += 32) {
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
  const int lane = tid & 31, warp = tid >> 5;
  for (int y = py0 + warp; y < py1; y += 8)
    for (int x = px0 + lane; x < px1; x += 32) sP[(y - py0) * PW + (x - px0)] = akz_fetch_input(p.t, I, x, y, p.inv255);
  __syncthreads();
  for (int y = py0 + warp; y < py1; y += 8)
    for (int x = tx0 + lane; x < tx1; x += 32) {
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
  for (int y = ty0 + warp; y < ty1; y += 8)
    for (int x = tx0 + lane; x < tx1; x += 32) {
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

/* FED level kernel.
 *
 * Every CTA owns a fixed 128 x 40 region R0 = tile +- d (d = FED steps of the
 * launch, tile (128-2d) x (40-2d)), so one thread geometry serves every
 * chunk size: 512 threads, 4 column groups of 32 lanes x 4 bands of 10 rows;
 * each thread keeps the 10 level values of its column in registers together
 * with the conductance pair sums (c_x + c_x+1), (c_x-1 + c_x), (c_y + c_y+1)
 * of the reference's flux terms, which do not change across steps.  A step
 * reads the east/west neighbours (and the band's outer rows) from a
 * double-buffered shared plane: 3 shared-memory operations and 13 FP32
 * operations per pixel-step, one barrier per step.  Pixels outside
 * tile +- (d - s) after step s are not needed and may hold anything; image
 * borders are replicate (clamped) neighbours, whose flux is exactly zero, as
 * in the reference's border formulas (nldiffusion_functions.cpp:241-307).
 */
#define AKZ_FED_RW 128
#define AKZ_FED_RH 40
#define AKZ_FED_RB 10
#define AKZ_FED_THREADS 512

size_t akz_fed_smem_bytes(int, int, int, int first)
{
  if (!first) return 2 * AKZ_FED_RW * AKZ_FED_RH * sizeof(float);
  const size_t P = (size_t)(AKZ_FED_RH + 6) * (AKZ_FED_RW + 6);
  const size_t T = (size_t)(AKZ_FED_RH + 6) * (AKZ_FED_RW + 2);
  const size_t S = (size_t)(AKZ_FED_RH + 2) * (AKZ_FED_RW + 2);
  return (P + T + S) * sizeof(float);
}

/* First-chunk prologue of k_fed for a tile whose input region (R0 +- 3)
 * lies inside the image: every region has its full compile-time size and no
 * neighbour needs clamping or reflecting, so the loops are straight-line.
 * Same arithmetic, in the same order, as the general path in k_fed. */
template <int SRCK>
__device__ __forceinline__ void akz_fed_prologue_interior(const akz_fed_params &p, const akz_level_desc &L,
                                                          const akz_image_desc &I, int level_desc, float *sm, int ox,
                                                          int oy, int tx0, int ty0, int tx1, int ty1, int lx, int ly0,
                                                          float *Lr, float *gE, float *gW, float *gS, float &gN0)
{
  constexpr int RW = AKZ_FED_RW, RH = AKZ_FED_RH, RB = AKZ_FED_RB;
  constexpr int PS = RW + 6, SS = RW + 2;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float *sP = sm, *sT = sm + (RH + 6) * PS, *sS = sT + (RH + 6) * SS;
  const float *planes = p.t.planes;
  if (SRCK == 1) {
    const akz_level_desc Lp = p.t.lv[level_desc - 1];
    const float *pp = planes + Lp.lt + (long long)(2 * (oy - 3)) * Lp.pitch + 2 * (ox - 3);
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const int ly = warp + 16 * k;
      if (ly < RH + 6) {
        const float *q0 = pp + (long long)(2 * ly) * Lp.pitch, *q1 = q0 + Lp.pitch;
#pragma unroll
        for (int j = 0; j < 5; j++) {
          const int l = lane + 32 * j;
          if (l < PS) {
            const float2 a = __ldg((const float2 *)(q0 + 2 * l)), b = __ldg((const float2 *)(q1 + 2 * l));
            sP[ly * PS + l] = 0.25f * (((a.x + a.y) + b.x) + b.y);
          }
        }
      }
    }
  } else {
    const float *pp;
    long long pitch;
    if (SRCK == 0) {
      const akz_level_desc Lp = p.t.lv[level_desc - 1];
      pp = planes + Lp.lt;
      pitch = Lp.pitch;
    } else {
      pp = planes + I.t2;
      pitch = L.pitch;
    }
    pp += (long long)(oy - 3) * pitch + (ox - 3);
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const int ly = warp + 16 * k;
      if (ly < RH + 6) {
        const float *q = pp + (long long)ly * pitch;
#pragma unroll
        for (int j = 0; j < 5; j++) {
          const int l = lane + 32 * j;
          if (l < PS) sP[ly * PS + l] = __ldg(q + l);
        }
      }
    }
  }
  __syncthreads();
  const float k0 = p.taps1[0], k1 = p.taps1[1], k2 = p.taps1[2];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const int ly = warp + 16 * k;
    if (ly < RH + 6) {
      const float *r = sP + ly * PS;
#pragma unroll
      for (int j = 0; j < 5; j++) {
        const int m = lane + 32 * j;
        if (m < SS) {
          float acc = k0 * (r[m] + r[m + 4]);
          acc = acc + k1 * (r[m + 1] + r[m + 3]);
          acc = acc + k2 * r[m + 2];
          sT[ly * SS + m] = acc;
        }
      }
    }
  }
  __syncthreads();
  float *lsp = p.t.planes + L.ls + (long long)(oy - 1) * L.pitch + (ox - 1);
  const int d = tx0 - ox;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const int n = warp + 16 * k;
    if (n < RH + 2) {
      const float *c = sT + n * SS;
      const bool yt = n >= d + 1 && n < d + 1 + (ty1 - ty0);
#pragma unroll
      for (int j = 0; j < 5; j++) {
        const int m = lane + 32 * j;
        if (m < SS) {
          float acc = k0 * (c[m] + c[m + 4 * SS]);
          acc = acc + k1 * (c[m + SS] + c[m + 3 * SS]);
          acc = acc + k2 * c[m + 2 * SS];
          sS[n * SS + m] = acc;
          if (yt && m >= d + 1 && m < d + 1 + (tx1 - tx0)) lsp[(long long)n * L.pitch + m] = acc;
        }
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < RB; r++) Lr[r] = sP[(ly0 + r + 3) * PS + lx + 3];
  __syncthreads();
  float *sG = sP;
  const float inv_k = p.kc[L.image * 16 + L.octave].y;
  float *gp = p.t.planes + I.g + (long long)oy * L.pitch + ox;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const int ly = warp + 16 * k;
    if (ly < RH) {
      const float *rm = sS + ly * SS, *r0 = rm + SS, *rp = r0 + SS;
      const bool yt = p.write_g && ly >= d && ly < d + (ty1 - ty0);
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const int l = lane + 32 * j;
        const float hm = rm[l + 2] - rm[l];
        const float h0 = r0[l + 2] - r0[l];
        const float hp = rp[l + 2] - rp[l];
        const float gx = 3.0f * (hm + hp) + 10.0f * h0;
        const float syp = 3.0f * (rp[l] + rp[l + 2]) + 10.0f * rp[l + 1];
        const float sym = 3.0f * (rm[l] + rm[l + 2]) + 10.0f * rm[l + 1];
        const float gy = syp - sym;
        const float gv = akz_conductance(gx, gy, inv_k, p.diffusivity);
        sG[ly * RW + l] = gv;
        if (yt && l >= d && l < d + (tx1 - tx0)) gp[(long long)ly * L.pitch + l] = gv;
      }
    }
  }
  __syncthreads();
  const int lxe = min(lx + 1, RW - 1), lxw = max(lx - 1, 0);
#pragma unroll
  for (int r = 0; r < RB; r++) {
    const int ly = ly0 + r;
    const float gc = sG[ly * RW + lx];
    gE[r] = gc + sG[ly * RW + lxe];
    gW[r] = sG[ly * RW + lxw] + gc;
    gS[r] = gc + sG[min(ly + 1, RH - 1) * RW + lx];
  }
  gN0 = sG[max(ly0 - 1, 0) * RW + lx] + sG[ly0 * RW + lx];
  __syncthreads();
}

__global__ void __launch_bounds__(AKZ_FED_THREADS, 2) k_fed(akz_fed_params p)
{
  extern __shared__ float sm[];
  constexpr int RW = AKZ_FED_RW, RH = AKZ_FED_RH, RB = AKZ_FED_RB;
  constexpr int PS = RW + 6, SS = RW + 2; /* strides of the input and smoothing regions */
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int si = akz_find_seg(p.segs, p.nsegs, blockIdx.x);
  const akz_tile_seg sg = p.segs[si];
  const akz_level_desc L = p.t.lv[sg.level_desc];
  const akz_image_desc I = p.t.im[L.image];
  const int W = L.width, H = L.height;
  const int d = p.steps;
  const int TW = RW - 2 * d, TH = RH - 2 * d;
  const int lt = blockIdx.x - sg.tile_begin;
  const int tx0 = (lt % sg.tiles_x) * TW, ty0 = (lt / sg.tiles_x) * TH;
  const int tx1 = min(tx0 + TW, W), ty1 = min(ty0 + TH, H);
  const int ox = tx0 - d, oy = ty0 - d; /* R0 origin (may lie outside the image) */
  const int srck = p.first ? sg.aux : p.src;
  float *planes = p.t.planes;

  /* this thread: column lx of R0, rows ly0 .. ly0+RB-1 */
  const int lx = (warp & 3) * 32 + lane;
  const int ly0 = (warp >> 2) * RB;
  const int x = ox + lx;
  const bool xin = x >= 0 && x < W;
  const int ytop = oy + ly0;
  const int lxe = min(lx + 1, RW - 1), lxw = max(lx - 1, 0);

  /* level values and the conductance pair sums of the reference's flux terms:
   *   xpos uses (c_x + c_x+1), xneg (c_x-1 + c_x), ypos (c_y + c_y+1), yneg (c_y-1 + c_y).
   * A pair that crosses the image border is zero: its flux is exactly zero
   * there (the reference omits the term), whatever the neighbour value is. */
  float Lr[RB], gE[RB], gW[RB], gS[RB];
  float gN0;
  float *cur, *nxt;

  const bool interior = ox >= 3 && oy >= 3 && ox + RW + 3 <= W && oy + RH + 3 <= H;
  if (p.first && interior) {
    if (srck == 1)
      akz_fed_prologue_interior<1>(p, L, I, sg.level_desc, sm, ox, oy, tx0, ty0, tx1, ty1, lx, ly0, Lr, gE, gW, gS, gN0);
    else if (srck == 0)
      akz_fed_prologue_interior<0>(p, L, I, sg.level_desc, sm, ox, oy, tx0, ty0, tx1, ty1, lx, ly0, Lr, gE, gW, gS, gN0);
    else
      akz_fed_prologue_interior<2>(p, L, I, sg.level_desc, sm, ox, oy, tx0, ty0, tx1, ty1, lx, ly0, Lr, gE, gW, gS, gN0);
    cur = sm + (RH + 6) * PS;                 /* row-pass buffer */
    nxt = cur + (RH + 6) * SS;                /* smoothing buffer */
  } else if (p.first) {
    float *sP = sm, *sT = sm + (RH + 6) * PS, *sS = sT + (RH + 6) * SS;
    const int px0 = max(ox - 3, 0), px1 = min(ox + RW + 3, W), py0 = max(oy - 3, 0), py1 = min(oy + RH + 3, H);
    const int sx0 = max(ox - 1, 0), sx1 = min(ox + RW + 1, W), sy0 = max(oy - 1, 0), sy1 = min(oy + RH + 1, H);
    /* input region: predecessor copy, its exact 2x half-sample, or a prepared plane */
    if (srck == 1) {
      const akz_level_desc Lp = p.t.lv[sg.level_desc - 1];
      const float *pp = planes + Lp.lt;
      for (int y = py0 + warp; y < py1; y += 16) {
        const float *q0 = pp + (long long)(2 * y) * Lp.pitch;
        const float *q1 = q0 + Lp.pitch;
        float *o = sP + (y - oy + 3) * PS - ox + 3;
        for (int xx = px0 + lane; xx < px1; xx += 32) {
          const float2 a = __ldg((const float2 *)(q0 + 2 * xx)), b = __ldg((const float2 *)(q1 + 2 * xx));
          o[xx] = 0.25f * (((a.x + a.y) + b.x) + b.y);
        }
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
      for (int y = py0 + warp; y < py1; y += 16) {
        const float *q = pp + (long long)y * pitch;
        float *o = sP + (y - oy + 3) * PS - ox + 3;
        for (int xx = px0 + lane; xx < px1; xx += 32) o[xx] = __ldg(q + xx);
      }
    }
    __syncthreads();
    /* sigma-1 Gaussian, horizontal then vertical, replicate border */
    const float k0 = p.taps1[0], k1 = p.taps1[1], k2 = p.taps1[2];
    for (int y = py0 + warp; y < py1; y += 16) {
      const float *r = sP + (y - oy + 3) * PS - ox + 3;
      float *o = sT + (y - oy + 3) * SS - ox + 1;
      for (int xx = sx0 + lane; xx < sx1; xx += 32) {
        float acc = k0 * (r[max(xx - 2, 0)] + r[min(xx + 2, W - 1)]);
        acc = acc + k1 * (r[max(xx - 1, 0)] + r[min(xx + 1, W - 1)]);
        acc = acc + k2 * r[xx];
        o[xx] = acc;
      }
    }
    __syncthreads();
    float *lsp = planes + L.ls;
    for (int y = sy0 + warp; y < sy1; y += 16) {
      const float *c2m = sT + (max(y - 2, 0) - oy + 3) * SS - ox + 1, *c2p = sT + (min(y + 2, H - 1) - oy + 3) * SS - ox + 1;
      const float *c1m = sT + (max(y - 1, 0) - oy + 3) * SS - ox + 1, *c1p = sT + (min(y + 1, H - 1) - oy + 3) * SS - ox + 1;
      const float *c0 = sT + (y - oy + 3) * SS - ox + 1;
      float *o = sS + (y - oy + 1) * SS - ox + 1;
      const bool yt = y >= ty0 && y < ty1;
      float *lo = lsp + (long long)y * L.pitch;
      for (int xx = sx0 + lane; xx < sx1; xx += 32) {
        float acc = k0 * (c2m[xx] + c2p[xx]);
        acc = acc + k1 * (c1m[xx] + c1p[xx]);
        acc = acc + k2 * c0[xx];
        o[xx] = acc;
        if (yt && xx >= tx0 && xx < tx1) lo[xx] = acc;
      }
    }
    __syncthreads();
    /* conductance on R0 from the Scharr gradient of Lsmooth (reflect-101) */
    float *sG = sP; /* the input region is not read any more except for L0 below */
    const float inv_k = p.kc[L.image * 16 + L.octave].y;
    float *gp = planes + I.g;
    /* L0 of this thread's pixels before sG overwrites the input region */
    for (int r = 0; r < RB; r++) {
      const int y = ytop + r;
      Lr[r] = (xin && y >= 0 && y < H) ? sP[(ly0 + r + 3) * PS + lx + 3] : 0.0f;
    }
    __syncthreads();
    for (int ly = warp; ly < RH; ly += 16) {
      const int y = oy + ly;
      const bool yin = y >= 0 && y < H;
      const int ym = y > 0 ? y - 1 : 1, yp = y < H - 1 ? y + 1 : H - 2;
      const float *rm = sS + (ym - oy + 1) * SS - ox + 1, *r0 = sS + (y - oy + 1) * SS - ox + 1;
      const float *rp = sS + (yp - oy + 1) * SS - ox + 1;
      const bool yt = y >= ty0 && y < ty1 && p.write_g;
      for (int l = lane; l < RW; l += 32) {
        const int xx = ox + l;
        float gv = 0.0f;
        if (yin && xx >= 0 && xx < W) {
          const int xm = xx > 0 ? xx - 1 : 1, xp = xx < W - 1 ? xx + 1 : W - 2;
          const float hm = rm[xp] - rm[xm];
          const float h0 = r0[xp] - r0[xm];
          const float hp = rp[xp] - rp[xm];
          const float gx = 3.0f * (hm + hp) + 10.0f * h0;
          const float syp = 3.0f * (rp[xm] + rp[xp]) + 10.0f * rp[xx];
          const float sym = 3.0f * (rm[xm] + rm[xp]) + 10.0f * rm[xx];
          const float gy = syp - sym;
          gv = akz_conductance(gx, gy, inv_k, p.diffusivity);
          if (yt && xx >= tx0 && xx < tx1) gp[(long long)y * L.pitch + xx] = gv;
        }
        sG[ly * RW + l] = gv;
      }
    }
    __syncthreads();
    const bool xe_in = xin && x + 1 < W, xw_in = xin && x >= 1;
    for (int r = 0; r < RB; r++) {
      const int ly = ly0 + r, y = ytop + r;
      const float gc = sG[ly * RW + lx];
      const bool yin = y >= 0 && y < H;
      gE[r] = (yin && xe_in) ? gc + sG[ly * RW + lxe] : 0.0f;
      gW[r] = (yin && xw_in) ? sG[ly * RW + lxw] + gc : 0.0f;
      gS[r] = (xin && y >= 0 && y + 1 < H) ? gc + sG[min(ly + 1, RH - 1) * RW + lx] : 0.0f;
    }
    gN0 = (xin && ytop >= 1 && ytop < H) ? sG[max(ly0 - 1, 0) * RW + lx] + sG[ly0 * RW + lx] : 0.0f;
    cur = sT; /* the row-pass buffer is free now and larger than R0 */
    nxt = sS; /* so is the smoothing buffer, once the conductance is done */
    __syncthreads();
  } else {
    cur = sm;
    nxt = sm + RW * RH;
    const float *lp = planes + (p.src == 1 ? I.t1 : I.t2);
    const float *gp = planes + I.g;
    const long long pitch = L.pitch;
    const int xc = min(max(x, 0), W - 1);
    for (int r = 0; r < RB; r++) {
      const int y = ytop + r;
      Lr[r] = 0.0f;
      gE[r] = gW[r] = gS[r] = 0.0f;
      if (xin && y >= 0 && y < H) {
        const float *gr = gp + (long long)y * pitch;
        const float gc = __ldg(gr + xc);
        Lr[r] = __ldg(lp + (long long)y * pitch + xc);
        if (x + 1 < W) gE[r] = gc + __ldg(gr + xc + 1);
        if (x >= 1) gW[r] = __ldg(gr + xc - 1) + gc;
        if (y + 1 < H) gS[r] = gc + __ldg(gr + pitch + xc);
      }
    }
    gN0 = (xin && ytop >= 1 && ytop < H) ? __ldg(gp + (long long)(ytop - 1) * pitch + xc) + __ldg(gp + (long long)ytop * pitch + xc) : 0.0f;
  }
  for (int r = 0; r < RB; r++) cur[(ly0 + r) * RW + lx] = Lr[r];
  __syncthreads();

  /* FED steps: xpos - xneg + ypos - yneg, scaled by tau/2, added to L
   * (nld_step_scalar, nldiffusion_functions.cpp:232-237 and :309-316) */
  const int lyn = max(ly0 - 1, 0), lys = min(ly0 + RB, RH - 1);
  for (int s = 0; s < d; s++) {
    const float h = p.h[s];
    float prev = cur[lyn * RW + lx];
    const float below = cur[lys * RW + lx];
#pragma unroll
    for (int r = 0; r < RB; r++) {
      const int ly = ly0 + r;
      const float Lc = Lr[r];
      const float Le = cur[ly * RW + lxe];
      const float Lw = cur[ly * RW + lxw];
      const float Ls = r < RB - 1 ? Lr[r + 1] : below;
      const float gn = r == 0 ? gN0 : gS[r - 1];
      const float xpos = gE[r] * (Le - Lc);
      const float xneg = gW[r] * (Lc - Lw);
      const float ypos = gS[r] * (Ls - Lc);
      const float yneg = gn * (Lc - prev);
      const float nv = Lc + h * (xpos - xneg + ypos - yneg);
      nxt[ly * RW + lx] = nv;
      prev = Lc;
      Lr[r] = nv;
    }
    __syncthreads();
    float *t = cur;
    cur = nxt;
    nxt = t;
  }
  /* tile interior from registers */
  float *out = planes + (p.dst == 0 ? L.lt : (p.dst == 1 ? I.t1 : I.t2));
  if (x >= tx0 && x < tx1) {
#pragma unroll
    for (int r = 0; r < RB; r++) {
      const int y = ytop + r;
      if (y >= ty0 && y < ty1) out[(long long)y * L.pitch + x] = Lr[r];
    }
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

cudaError_t akz_launch_fed(const akz_fed_params &p, int ntiles, int, int, cudaStream_t s)
{
  if (ntiles <= 0) return cudaSuccess;
  if (p.steps < 1 || p.steps > 8) return cudaErrorInvalidValue;
  const size_t smem = akz_fed_smem_bytes(0, 0, p.steps, p.first);
  cudaError_t e = cudaFuncSetAttribute(k_fed, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_fed<<<ntiles, AKZ_FED_THREADS, smem, s>>>(p);
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
