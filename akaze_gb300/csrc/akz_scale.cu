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

#include "../../include/akaze_gb300.h"
#include "akz_device.cuh"
#include "akz_fmath.h"

akz_status akz_report(akz_status s, const char *msg);

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
__global__ void __launch_bounds__(32) k_contrast_final(akz_tables t, const unsigned int *hist, int nbins, float perc,
                                                        float2 *kc)
{
  /* one warp per image: the histogram staged in shared memory by the warp
   * and its (integer) total summed across the lanes, then lane 0 walks the
   * bins in order with the reference's float accumulation */
  extern __shared__ unsigned int h[]; /* nbins words: a CTA this small fits beside the other groups' kernels */
  const int img = blockIdx.x, lane = threadIdx.x;
  const unsigned int *hg = hist + (long long)img * nbins;
  unsigned long long tot = 0;
  for (int b = lane; b < nbins; b += 32) {
    const unsigned int v = hg[b];
    h[b] = v;
    tot += v;
  }
  for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
  __syncwarp();
  if (lane != 0) return;
  const float hmax = sqrtf(__uint_as_float(t.stats[img].hmax2_bits));
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
/* Level 0 and the contrast gradient from one staging of the input.
 *
 * k_level0: per 128 x 32 tile, the input region tile +- 4 is staged once
 * with replicate (clamped) coordinates; from it
 *   Lt0 = the soffset Gaussian (AKAZE.cpp:234, radius <= 4; a smaller kernel
 *         is zero-padded at its outer end, which adds exact zeros first), and
 *   m   = Lx^2 + Ly^2 of the Scharr gradient of the sigma-1 Gaussian
 *         (compute_k_percentile, nldiffusion_functions.cpp:121-170) at every
 *         interior pixel, written to the image's T1 plane, with the image's
 *         maximum of m.
 * k_contrast_hist then bins sqrt(m) / max (nldiffusion_functions.cpp:
 * 172-197).  Column pairs with packed FP32x2 additions, scalar products, in
 * the reference's operation order, so every value equals the per-pixel
 * kernels k_gauss0 / k_contrast. */

template <bool FUSED>
__global__ void __launch_bounds__(256) k_level0(akz_level0_params p)
{
  constexpr int TW = AKZ_L0_TW, TH = AKZ_L0_TH;
  constexpr int PW = TW + 8, PH = TH + 8;  /* input: tile +- 4 */
  constexpr int BW = TW + 2, BH = TH + 6;  /* sigma-1 rows pass: cols tile +- 1, rows tile +- 3 */
  extern __shared__ __align__(16) float l0sm[];
  float *sP = l0sm, *sA = sP + PH * PW, *sB = sA + PH * TW;
  __shared__ float sRed[8];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int si = akz_find_seg_warp(p.segs, p.nsegs, blockIdx.x);
  const akz_tile_seg sg = p.segs[si];
  const akz_level_desc L = p.t.lv[sg.level_desc];
  const akz_image_desc I = p.t.im[L.image];
  const int W = L.width, H = L.height;
  const int lt = blockIdx.x - sg.tile_begin;
  const int tx0 = (lt % sg.tiles_x) * TW, ty0 = (lt / sg.tiles_x) * TH;

  if (!p.t.input_f32 && tx0 >= 4 && tx0 + TW + 4 <= W && ty0 >= 4 && ty0 + TH + 4 <= H) {
    /* interior tile: a row per warp, 4 bytes per lane (tx0 - 4 is a
     * multiple of 4 and u8 rows are 16-byte aligned), 4 floats per store */
    static_assert(PW == 136 && TW % 4 == 0, "k_level0 staging");
    const uint8_t *u8 = p.t.u8 + I.u8_off + tx0 - 4;
#pragma unroll
    for (int k = 0; k < PH / 8; k++) {
      const int r = warp + 8 * k;
      const uchar4 *src = reinterpret_cast<const uchar4 *>(u8 + (long long)(ty0 - 4 + r) * I.u8_pitch);
#pragma unroll
      for (int j = 0; j < 2; j++) {
        const int q = lane + 32 * j;
        if (q < PW / 4) {
          const uchar4 b = __ldg(src + q);
          *reinterpret_cast<float4 *>(sP + r * PW + 4 * q) =
              make_float4((float)b.x * p.inv255, (float)b.y * p.inv255, (float)b.z * p.inv255, (float)b.w * p.inv255);
        }
      }
    }
  } else {
    for (int i = tid; i < PH * PW; i += 256) {
      const int r = i / PW, c = i - r * PW;
      const int y = akz_clampi(ty0 - 4 + r, 0, H - 1), x = akz_clampi(tx0 - 4 + c, 0, W - 1);
      sP[i] = akz_fetch_input(p.t, I, x, y, p.inv255);
    }
  }
  __syncthreads();
  /* rows passes from one window per column pair: soffset Gaussian on tile
   * columns (all PH rows), sigma-1 on the same columns for rows tile +- 3
   * (sB column d is x = tx0 - 1 + d, sB row r is sP row r + 1) */
  const float t0 = p.taps0[0], t1 = p.taps0[1], t2 = p.taps0[2], t3 = p.taps0[3], t4 = p.taps0[4];
  const float k0 = p.taps1[0], k1 = p.taps1[1], k2 = p.taps1[2];
  for (int i = tid; i < PH * (TW / 2); i += 256) {
    const int r = i / (TW / 2), c = 2 * (i - r * (TW / 2));
    const float *q = sP + r * PW + c; /* sP column c + 4 is tile column c */
    const float2 A0 = ld2(q), A1 = ld2(q + 2), A2 = ld2(q + 4), A3 = ld2(q + 6), A4 = ld2(q + 8);
    const float2 s08 = f2add(A0, A4);
    const float2 s17 = f2add(make_float2(A0.y, A1.x), make_float2(A3.y, A4.x));
    const float2 s26 = f2add(A1, A3);
    const float2 s35 = f2add(make_float2(A1.y, A2.x), make_float2(A2.y, A3.x));
    float2 acc = akz_k2<FUSED>(t0, s08);
    acc = akz_axpy2<FUSED>(t1, s17, acc);
    acc = akz_axpy2<FUSED>(t2, s26, acc);
    acc = akz_axpy2<FUSED>(t3, s35, acc);
    acc = akz_axpy2<FUSED>(t4, A2, acc);
    st2(sA + r * TW + c, acc);
    if (r >= 1 && r <= BH) { /* sigma 1 at x = tx0 + c, c + 1: taps sP columns c + 2 .. c + 7 */
      const float2 s15 = s26, s24 = s35;
      float2 g = akz_k2<FUSED>(k0, s15);
      g = akz_axpy2<FUSED>(k1, s24, g);
      g = akz_axpy2<FUSED>(k2, A2, g);
      float *o = sB + (r - 1) * BW + c + 1;
      o[0] = g.x;
      o[1] = g.y;
    }
  }
  if (tid < 2 * BH) { /* sigma 1 at the two columns outside the tile, x = tx0 - 1 and tx0 + TW */
    const int r = tid >> 1, d = (tid & 1) ? BW - 1 : 0;
    const float *q = sP + (r + 1) * PW + d + 3; /* centre */
    float g = k0 * (q[-2] + q[2]);
    if (FUSED) {
      g = __fmaf_rn(k1, q[-1] + q[1], g);
      g = __fmaf_rn(k2, q[0], g);
    } else {
      g = g + k1 * (q[-1] + q[1]);
      g = g + k2 * q[0];
    }
    sB[r * BW + d] = g;
  }
  __syncthreads();
  /* columns passes, 8 rows x one column pair per thread: Lt0 for the tile
   * (to HBM); the sigma-1 image of rows y - 1 .. y + 8 on columns x - 1 ..
   * x + 2 from sB rows y - 3 .. y + 10, and from it the Scharr gradient
   * magnitude^2 at interior pixels */
  float mx = 0.0f;
  {
    const int c = 2 * (tid & 63), g = tid >> 6; /* 64 column pairs x 4 groups of 8 rows */
    const int x = tx0 + c;
    float *out = p.t.planes + L.lt;
    {
      float2 v[16];
#pragma unroll
      for (int j = 0; j < 16; j++) v[j] = ld2(sA + (g * 8 + j) * TW + c);
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const float2 s08 = f2add(v[j], v[j + 8]), s17 = f2add(v[j + 1], v[j + 7]);
        const float2 s26 = f2add(v[j + 2], v[j + 6]), s35 = f2add(v[j + 3], v[j + 5]);
        float2 acc = akz_k2<FUSED>(t0, s08);
        acc = akz_axpy2<FUSED>(t1, s17, acc);
        acc = akz_axpy2<FUSED>(t2, s26, acc);
        acc = akz_axpy2<FUSED>(t3, s35, acc);
        acc = akz_axpy2<FUSED>(t4, v[j + 4], acc);
        const int y = ty0 + g * 8 + j;
        if (y < H) {
          float *o = out + (long long)y * L.pitch + x;
          if (x + 1 < W)
            st2(o, acc);
          else if (x < W)
            o[0] = acc.x;
        }
      }
    }
    float *mp = p.t.planes + I.t1;
    const bool mx0 = x >= 1 && x < W - 1, mx1 = x + 1 >= 1 && x + 1 < W - 1;
    float2 ba[5], bb[5], ga[3], gb[3]; /* sB rows and sigma-1 rows; a: x - 1, x; b: x + 1, x + 2 */
#pragma unroll
    for (int k = 0; k < 14; k++) { /* sB row 8 g + k */
      const float *q = sB + (g * 8 + k) * BW + c;
#pragma unroll
      for (int i = 0; i < 4; i++) {
        ba[i] = ba[i + 1];
        bb[i] = bb[i + 1];
      }
      ba[4] = ld2(q);
      bb[4] = ld2(q + 2);
      if (k < 4) continue;
      { /* sigma-1 row y - 1 + (k - 4), y = ty0 + 8 g */
        const float2 sa04 = f2add(ba[0], ba[4]), sa13 = f2add(ba[1], ba[3]);
        const float2 sb04 = f2add(bb[0], bb[4]), sb13 = f2add(bb[1], bb[3]);
        float2 a = akz_k2<FUSED>(k0, sa04), b = akz_k2<FUSED>(k0, sb04);
        a = akz_axpy2<FUSED>(k1, sa13, a);
        b = akz_axpy2<FUSED>(k1, sb13, b);
        a = akz_axpy2<FUSED>(k2, ba[2], a);
        b = akz_axpy2<FUSED>(k2, bb[2], b);
        ga[0] = ga[1];
        ga[1] = ga[2];
        ga[2] = a;
        gb[0] = gb[1];
        gb[1] = gb[2];
        gb[2] = b;
      }
      if (k < 6) continue;
      /* Scharr at row y = ty0 + 8 g + k - 6 */
      const float2 m0 = ga[0], m1 = gb[0], c0 = ga[1], c1 = gb[1], p0 = ga[2], p1 = gb[2];
      const float2 hm = f2sub(m1, m0), h0 = f2sub(c1, c0), hp = f2sub(p1, p0); /* v[x+1] - v[x-1] */
      const float2 u = f2add(hm, hp);
      const float2 lx = akz_lin2<FUSED>(3.0f, u, 10.0f, h0);
      const float2 sp = f2add(p0, p1), sm = f2add(m0, m1); /* (v[x-1] + v[x+1]) */
      const float2 syp = akz_lin2<FUSED>(3.0f, sp, 10.0f, make_float2(p0.y, p1.x));
      const float2 sym = akz_lin2<FUSED>(3.0f, sm, 10.0f, make_float2(m0.y, m1.x));
      const float2 ly = f2sub(syp, sym);
      const float2 m = akz_sq2sum<FUSED>(lx, ly);
      const int y = ty0 + g * 8 + k - 6;
      if (y < 1 || y >= H - 1) continue;
      float *o = mp + (long long)y * L.pitch + x;
      if (mx0 && mx1) {
        st2(o, m);
        mx = fmaxf(fmaxf(mx, m.x), m.y);
      } else if (mx0) {
        o[0] = m.x;
        mx = fmaxf(mx, m.x);
      } else if (mx1) {
        o[1] = m.y;
        mx = fmaxf(mx, m.y);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (lane == 0) sRed[warp] = mx;
  __syncthreads();
  if (tid == 0) {
    float m = sRed[0];
    for (int w = 1; w < 8; w++) m = fmaxf(m, sRed[w]);
    atomicMax(&p.t.stats[L.image].hmax2_bits, __float_as_uint(m));
  }
}

__global__ void __launch_bounds__(256) k_contrast_hist(akz_level0_params p)
{
  constexpr int TW = AKZ_L0_TW, TH = AKZ_L0_TH;
  __shared__ unsigned int sHist[AKZ_MAX_NBINS];
  const int tid = threadIdx.x;
  const int si = akz_find_seg_warp(p.segs, p.nsegs, blockIdx.x);
  const akz_tile_seg sg = p.segs[si];
  const akz_level_desc L = p.t.lv[sg.level_desc];
  const akz_image_desc I = p.t.im[L.image];
  const int W = L.width, H = L.height;
  const int lt = blockIdx.x - sg.tile_begin;
  const int tx0 = (lt % sg.tiles_x) * TW, ty0 = (lt / sg.tiles_x) * TH;
  for (int b = tid; b < p.nbins; b += 256) sHist[b] = 0;
  __syncthreads();
  const float hmax = sqrtf(__uint_as_float(p.t.stats[L.image].hmax2_bits));
  const float nb = (float)p.nbins;
  const float *mp = p.t.planes + I.t1;
  const int x0 = max(tx0, 1), x1 = min(tx0 + TW, W - 1), y0 = max(ty0, 1), y1 = min(ty0 + TH, H - 1);
  /* a run of 16 consecutive pixels per thread (8 threads per 128-pixel row
   * segment, 32 rows): neighbouring pixels mostly share a bin, so one shared
   * atomic per run of equal bins instead of one per pixel */
  static_assert(TW == 128 && TH == 32, "k_contrast_hist runs");
  const int y = ty0 + (tid >> 3), xs = tx0 + 16 * (tid & 7);
  if (y >= y0 && y < y1) {
    const float *row = mp + (long long)y * L.pitch;
    int cur = -1;
    unsigned int cnt = 0;
    float v[16];
    if (xs >= x0 && xs + 16 <= x1) { /* pitch is a multiple of 32 floats: 16-byte aligned */
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const float4 f = __ldg(reinterpret_cast<const float4 *>(row + xs) + q);
        v[4 * q] = f.x;
        v[4 * q + 1] = f.y;
        v[4 * q + 2] = f.z;
        v[4 * q + 3] = f.w;
      }
    } else {
#pragma unroll
      for (int k = 0; k < 16; k++) v[k] = (xs + k >= x0 && xs + k < x1) ? __ldg(row + xs + k) : 0.0f;
    }
#pragma unroll
    for (int k = 0; k < 16; k++) {
      const float modg = sqrtf(v[k]); /* 0 outside the interior: skipped like a zero gradient */
      if (modg != 0.0f) {
        int nbin = (int)floorf(nb * (modg / hmax));
        if (nbin == p.nbins) nbin--;
        if (nbin != cur) {
          if (cnt) atomicAdd(&sHist[cur], cnt);
          cur = nbin;
          cnt = 0;
        }
        cnt++;
      }
    }
    if (cnt) atomicAdd(&sHist[cur], cnt);
  }
  __syncthreads();
  for (int b = tid; b < p.nbins; b += 256)
    if (sHist[b]) atomicAdd(&p.hist[(long long)L.image * p.nbins + b], sHist[b]);
}

cudaError_t akz_launch_level0(const akz_level0_params &p, int ntiles, cudaStream_t s)
{
  if (ntiles <= 0) return cudaSuccess;
  constexpr int smem = ((AKZ_L0_TH + 8) * (AKZ_L0_TW + 8) + (AKZ_L0_TH + 8) * AKZ_L0_TW + (AKZ_L0_TH + 6) * (AKZ_L0_TW + 2)) *
                       (int)sizeof(float);
  cudaError_t e0;
  if (p.fused) {
    e0 = cudaFuncSetAttribute(k_level0<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e0 != cudaSuccess) return e0;
    k_level0<true><<<ntiles, 256, smem, s>>>(p);
  } else {
    e0 = cudaFuncSetAttribute(k_level0<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e0 != cudaSuccess) return e0;
    k_level0<false><<<ntiles, 256, smem, s>>>(p);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_contrast_hist<<<ntiles, 256, 0, s>>>(p);
  return cudaGetLastError();
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

/* FED level kernel.
 *
 * Every CTA owns a fixed 128 x 48 region R0 = tile +- d (d = FED steps of the
 * launch; the region's left edge is rounded down to a multiple of 4 columns,
 * akz_fed_tile_w), so one thread geometry serves every chunk size: 512
 * threads, each with 4 columns x 3 rows of R0 (a warp spans the region's
 * 128 columns, 16 warps its 48 rows).  A thread keeps its level values and
 * the conductance pair sums (c_x + c_x+1), (c_y + c_y+1) of the reference's
 * flux terms in registers for the whole launch.  A step takes the west and
 * east neighbours from the adjacent lanes (shuffles) and the rows above and
 * below the warp's band from a double-buffered shared exchange of every
 * warp's first and last row: one barrier per step, 6 shuffles and 2 128-bit
 * shared loads and stores per thread and step.  Pixels outside
 * tile +- (d - s) after step s are not needed and may hold anything (the
 * region's outer columns and rows take their own values as stand-ins);
 * image borders are replicate (clamped) neighbours, whose flux is exactly
 * zero, as in the reference's border formulas (nldiffusion_functions.cpp:
 * 241-307).  Column groups start at multiples of 4 image columns, so every
 * global load or store of a thread's row is one 128-bit access.
 */
#define AKZ_FED_RW 128
#define AKZ_FED_RH 48
#define AKZ_FED_RB 3
#define AKZ_FED_THREADS 512
#define AKZ_FED_PS (AKZ_FED_RW + 8) /* input plane: columns R0 - 4 .. R0 + 131 */
#define AKZ_FED_SS (AKZ_FED_RW + 4) /* Gaussian planes: columns R0 - 2 .. R0 + 129 */
#define AKZ_FED_XB (2 * 2 * 16 * AKZ_FED_RW) /* exchange rows: [step parity][first, last row][warp][column] */
#define AKZ_FED_TMA_SPIN (1 << 22)  /* bounded wait for the input box */
static_assert(AKZ_FED_PS == AKZ_FED_BOX_W && AKZ_FED_RH + 6 == AKZ_FED_BOX_H, "k_fed input box");
static_assert(AKZ_FED_RB * 16 == AKZ_FED_RH && AKZ_FED_THREADS == 512, "k_fed thread geometry");

size_t akz_fed_smem_bytes(int, int, int, int first)
{
  if (!first) return AKZ_FED_XB * sizeof(float) + 128; /* the kernel aligns its base to 128 bytes */
  const size_t P = (size_t)(AKZ_FED_RH + 6) * AKZ_FED_PS;
  const size_t T = (size_t)(AKZ_FED_RH + 6) * AKZ_FED_SS;
  const size_t S = (size_t)(AKZ_FED_RH + 2) * AKZ_FED_SS;
  static_assert((size_t)AKZ_FED_XB <= (size_t)(AKZ_FED_RH + 6) * (AKZ_FED_PS + AKZ_FED_SS), "exchange rows fit sP + sT");
  return (P + T + S) * sizeof(float) + 128 + 16; /* 128-byte alignment of the TMA box, the mbarrier */
}

/* Conductance of |grad|^2 = m (AKAZE.cpp:259-268 with pm_g1, pm_g2,
 * weickert_diffusivity, charbonnier_diffusivity, nldiffusion_functions.cpp:58-118). */
__device__ __forceinline__ float akz_conductance_m(float m, float inv_k, int type)
{
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

/* PM-g2 conductance of two pixels, (float)(1.0 / (1.0 + (double)f)) with
 * f = inv_k * m per lane, exactly as akz_recip1pf gives it.  The reciprocal
 * of s = fl(1 + f) starts from the hardware approximation (relative error
 * below 2^-22); one Newton step against the exact float-float sum s + lo
 * (TwoSum) gives v = q + q r within about 2^-43 (relative) of 1 / (1 + f).
 * The final rounding is taken twice, at v - q 2^-41 and v + q 2^-41 (r +- 2^-41
 * is exact in float: |r| < 2^-21).  The true quotient lies between them, so
 * where both round to the same float that float is its correct rounding; the
 * lanes where they differ (a rounding midpoint within 2^-41 of v, about one
 * in 2^17) take the double evaluation. */
template <bool FUSED>
__device__ __forceinline__ float2 akz_pm_g2_pair(float2 m, float inv_k)
{
  if (FUSED) { /* one rounding of 1 + f, the hardware reciprocal (relative error below 2^-22) */
    const float2 s = f2fma(make_float2(inv_k, inv_k), m, make_float2(1.0f, 1.0f));
    float2 q;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(q.x) : "f"(s.x));
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(q.y) : "f"(s.y));
    return q;
  }
  const float2 f = make_float2(inv_k * m.x, inv_k * m.y);
  const float2 one = make_float2(1.0f, 1.0f);
  const float2 s = f2add(one, f);
  const float2 bb = f2sub(s, one); /* TwoSum: lo = 1 + f - s exactly, for any order of magnitude */
  const float2 lo = f2add(f2sub(one, f2sub(s, bb)), f2sub(f, bb));
  float2 q;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(q.x) : "f"(s.x));
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(q.y) : "f"(s.y));
  const float2 nq = make_float2(-q.x, -q.y);
  const float2 r = f2fma(nq, lo, f2fma(nq, s, one)); /* 1 - q (s + lo) */
  const float2 band = make_float2(0x1p-41f, 0x1p-41f);
  const float2 lo_r = f2fma(q, f2sub(r, band), q), hi_r = f2fma(q, f2add(r, band), q);
  float out[2] = {lo_r.x, lo_r.y};
  const float ff[2] = {f.x, f.y}, hh[2] = {hi_r.x, hi_r.y};
#pragma unroll
  for (int k = 0; k < 2; k++)
    if (!(ff[k] <= 0x1p100f) || out[k] != hh[k]) out[k] = (float)(1.0 / (1.0 + (double)ff[k]));
  return make_float2(out[0], out[1]);
}

/* First-chunk prologue of k_fed: the level's starting image on R0 +- 3 rows
 * and R0 +- 4 columns, its sigma-1 smoothing Lsmooth (written to HBM for the
 * tile) and the conductance on R0 (written to HBM for the tile when more
 * chunks follow).
 *
 * The input is the predecessor level (SRCK 0) or the INTER_AREA plane
 * prepared in T2 (SRCK 2), fetched as one TMA box; or the exact 2x
 * half-sample of the predecessor (SRCK 1), formed by the threads.  Rows and
 * columns outside the image take the nearest image row and column
 * (replicate), which makes the Gaussian's replicate border
 * (gaussian_2D_convolution, nldiffusion_functions.cpp:29-47) exact for every
 * pixel inside the image; Lsmooth's row and column just outside the image
 * are then replaced by their reflect-101 mirrors (x = -1 by x = 1, x = W by
 * x = W - 2), the border of the Scharr gradient (nldiffusion_functions.cpp:
 * 50-53).  Values outside the image are finite and unused: their
 * conductance pair sums are zero.
 *
 * Leaves the level values of R0 in sP (stride AKZ_FED_PS, R0 at row 3,
 * column 4), the conductance in sT (stride RW) and this thread's 3 x 4
 * conductances in g.  Filter passes work on
 * column pairs with packed FP32x2 additions and scalar products, in the
 * reference's operation order:
 *   Gaussian  k0*(v[-2] + v[+2]) + k1*(v[-1] + v[+1]) + k2*v[0], rows then columns;
 *   Scharr    gx = 3*(d[y-1] + d[y+1]) + 10*d[y],  d = v[x+1] - v[x-1],
 *             gy = s[y+1] - s[y-1],  s = 3*(v[x-1] + v[x+1]) + 10*v[x].
 * Returns false when the input box did not arrive within the bounded wait
 * (the image's status is then AKZ_ERR_TIMEOUT). */
template <int SRCK, bool FUSED>
__device__ __forceinline__ bool akz_fed_prologue(const akz_fed_params &p, const akz_level_desc &L,
                                                 const akz_image_desc &I, int level_desc, float *sm, int ox, int oy,
                                                 int tx0, int ty0, int tx1, int ty1, int lx0, int ly0, float (&g)[3][4])
{
  constexpr int RW = AKZ_FED_RW, RH = AKZ_FED_RH, NT = AKZ_FED_THREADS;
  constexpr int PS = AKZ_FED_PS, SS = AKZ_FED_SS, PH = RH + 6, SH = RH + 2;
  constexpr int NP = SS / 2;          /* column pairs of the smoothing regions */
  /* rows per thread and row groups of the vertical pass: 7 groups of 8 rows
   * (the last one 2 rows) keep 462 of the 512 threads busy */
  constexpr int VR = 8, VG = (SH + VR - 1) / VR;
  static_assert(NP * VG <= NT && NP == 66 && NT == 512 && (VG - 1) * VR < SH, "k_fed prologue geometry");
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int W = L.width, H = L.height;
  float *sP = sm, *sT = sm + PH * PS, *sS = sT + PH * SS;
  uint64_t *mbar = reinterpret_cast<uint64_t *>(sS + SH * SS);
  const float *planes = p.t.planes;

  /* 1. starting image on columns ox - 4 .. ox + 131, rows oy - 3 .. oy + 42 */
  if (SRCK == 1) {
    const akz_level_desc Lp = p.t.lv[level_desc - 1];
    const float *pp = planes + Lp.lt;
    const long long pitch = Lp.pitch;
#pragma unroll
    for (int k = 0; k < (PH + 15) / 16; k++) {
      const int ly = warp + 16 * k;
      if (ly < PH) {
        const int y = akz_clampi(oy - 3 + ly, 0, H - 1);
        const float *q0 = pp + (long long)(2 * y) * pitch;
#pragma unroll
        for (int j = 0; j < (PS + 31) / 32; j++) {
          const int l = lane + 32 * j;
          if (l < PS) {
            const int x = akz_clampi(ox - 4 + l, 0, W - 1);
            const float2 a = __ldg((const float2 *)(q0 + 2 * x)), b = __ldg((const float2 *)(q0 + pitch + 2 * x));
            sP[ly * PS + l] = 0.25f * (((a.x + a.y) + b.x) + b.y);
          }
        }
      }
    }
    __syncthreads();
  } else {
    /* one TMA box; out-of-image parts arrive as zeros and are replaced below */
    const char *tmap = (const char *)p.tmaps + 128 * (SRCK == 2 ? 2 * level_desc + 1 : 2 * (level_desc - 1));
    const uint32_t mb = (uint32_t)__cvta_generic_to_shared(mbar);
    if (tid == 0) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb));
      asm volatile("fence.mbarrier_init.release.cluster;");
    }
    __syncthreads();
    if (tid == 0) {
      const uint32_t dst = (uint32_t)__cvta_generic_to_shared(sP);
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(PH * PS * 4) : "memory");
      asm volatile(
          "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
              "r"(dst), "l"(tmap), "r"(ox - 4), "r"(oy - 3), "r"(mb)
          : "memory");
    }
    /* one warp polls the barrier; the others wait at the block barrier,
     * where they issue nothing (the SM's other CTA keeps the slots) */
    uint32_t done = 1;
    if (warp == 0) {
      done = 0;
      for (int it = 0; it < AKZ_FED_TMA_SPIN && !done; it++)
        asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\nselp.u32 %0, 1, 0, p;\n}"
                     : "=r"(done)
                     : "r"(mb)
                     : "memory");
    }
    if (__syncthreads_or(!done)) { /* (CTA-uniform) record it, give the copy one more bounded wait, and leave */
      if (tid == 0) {
        atomicExch(&p.t.stats[L.image].status, (int)AKZ_ERR_TIMEOUT);
        done = 0;
        for (int it = 0; it < AKZ_FED_TMA_SPIN && !done; it++)
          asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\nselp.u32 %0, 1, 0, p;\n}"
                       : "=r"(done)
                       : "r"(mb)
                       : "memory");
      }
      __syncthreads();
      return false;
    }
    /* replicate border: columns first (each row from its own clamped
     * column), then whole rows; the box always contains column and row 0
     * or W-1 / H-1 where it crosses the image edge */
    if (ox - 4 < 0 || ox + 132 > W || oy - 3 < 0 || oy - 3 + PH > H) {
      /* only the box columns left of x = 0 (nl) and from x = W on (from
       * cr), then the rows above y = 0 (nt) and from y = H on (from rb) */
      const int nl = max(0, 4 - ox), cr = min(PS, W - (ox - 4));
      const int nc = nl + (PS - cr);
      if (nc > 0) {
        for (int i = tid; i < PH * nc; i += NT) {
          const int r = i / nc, k = i - r * nc, c = k < nl ? k : cr + (k - nl);
          const int xc = akz_clampi(ox - 4 + c, 0, W - 1);
          sP[r * PS + c] = sP[r * PS + (xc - (ox - 4))];
        }
        __syncthreads();
      }
      const int nt = max(0, 3 - oy), rb = min(PH, H - (oy - 3));
      const int nr = nt + (PH - rb);
      if (nr > 0) {
        for (int i = tid; i < nr * PS; i += NT) {
          const int k = i / PS, c = i - k * PS, r = k < nt ? k : rb + (k - nt);
          const int yc = akz_clampi(oy - 3 + r, 0, H - 1);
          sP[r * PS + c] = sP[(yc - (oy - 3)) * PS + c];
        }
        __syncthreads();
      }
    }
  }

  /* 2. rows of the Gaussian on columns R0 - 2 .. R0 + 129 (sT column c is
   *    x = ox - 2 + c, its taps sP c .. c + 4): column pairs 0..63 by
   *    (tid & 63) on rows (tid >> 6) + 8k, pairs 64 and 65 by the last
   *    2 PH threads, whose row groups 6 and 7 have one row fewer (so no
   *    thread has more than 7 rows; an even spread over all threads costs
   *    more in index arithmetic than it saves) */
  const float k0 = p.taps1[0], k1 = p.taps1[1], k2 = p.taps1[2];
  auto hrow = [&](int row, int c) {
    const float *r = sP + row * PS + c;
    const float2 A = ld2(r), B = ld2(r + 2), C = ld2(r + 4);
    const float2 s04 = f2add(A, C);
    const float2 s13 = f2add(make_float2(A.y, B.x), make_float2(B.y, C.x));
    float2 acc = akz_k2<FUSED>(k0, s04);
    acc = akz_axpy2<FUSED>(k1, s13, acc);
    acc = akz_axpy2<FUSED>(k2, B, acc);
    st2(sT + row * SS + c, acc);
  };
  {
    const int c = 2 * (tid & 63), r0 = tid >> 6;
#pragma unroll
    for (int k = 0; k < (PH + 7) / 8; k++)
      if (r0 + 8 * k < PH) hrow(r0 + 8 * k, c);
    static_assert(NT - 2 * PH >= 6 * 64 && (PH + 7) / 8 == 7 && PH % 8 == 6, "k_fed rows pass: extra pairs on the 6-row groups");
    if (tid >= NT - 2 * PH) {
      const int e = tid - (NT - 2 * PH);
      hrow(e >> 1, 2 * (64 + (e & 1)));
    }
  }
  __syncthreads();

  /* 3. columns of the Gaussian: Lsmooth on rows R0 +- 1 (sS row n is y = oy - 1 + n); the
   *    tile's Lsmooth goes to HBM from step 5, by the threads that own its pixels */
  if (tid < NP * VG) {
    const int g = tid / NP, c = 2 * (tid - g * NP);
    const float *col = sT + c;
    float2 v[VR + 4];
#pragma unroll
    for (int j = 0; j < VR + 4; j++) v[j] = ld2(col + min(g * VR + j, PH - 1) * SS); /* rows past sT: unused */
#pragma unroll
    for (int j = 0; j < VR; j++) {
      const int n = g * VR + j;
      if (n >= SH) break;
      const float2 s04 = f2add(v[j], v[j + 4]);
      const float2 s13 = f2add(v[j + 1], v[j + 3]);
      float2 acc = akz_k2<FUSED>(k0, s04);
      acc = akz_axpy2<FUSED>(k1, s13, acc);
      acc = akz_axpy2<FUSED>(k2, v[j + 2], acc);
      st2(sS + n * SS + c, acc);
    }
  }
  __syncthreads();

  /* 4. the reflect-101 border of Lsmooth: columns first, then whole rows
   *    (which fixes the corners) */
  const int cm = 1 - ox, cp = W - ox + 2; /* sS columns of x = -1 and x = W */
  const int nm = -oy, np = H - oy + 1;    /* sS rows of y = -1 and y = H */
  if (cm >= 0 || cp < SS) { /* (CTA-uniform) */
    if (tid < SH) {
      float *row = sS + tid * SS;
      if (cm >= 0) row[cm] = row[cm + 2];
      if (cp < SS) row[cp] = row[cp - 2];
    }
    __syncthreads();
  }
  if (nm >= 0 || np < SH) {
    if (tid < SS) {
      if (nm >= 0) sS[nm * SS + tid] = sS[(nm + 2) * SS + tid];
      if (np < SH) sS[np * SS + tid] = sS[(np - 2) * SS + tid];
    }
    __syncthreads();
  }

  /* 5. Scharr gradient of Lsmooth and the conductance on R0, in this
   *    thread's k_fed geometry: columns x0 .. x0+3 (x0 = ox + lx0, sS
   *    columns lx0 + 2 ..), rows ly0 .. ly0+2; kept in g, stored to sT
   *    (free since pass 3; neighbours read it after the barrier) and, for
   *    later chunks, to HBM; first the thread's own Lsmooth pixels go to
   *    HBM */
  float *sG = sT;
  const float inv_k = p.kc[L.image * 16 + L.octave].y;
  const int x0 = ox + lx0; /* a multiple of 4 */
  const bool xfull = x0 >= tx0 && x0 + 4 <= tx1, xany = x0 + 4 > tx0 && x0 < tx1;
#pragma unroll
  for (int r = 0; r < 3; r++) { /* the thread's Lsmooth pixels (sS row ly0 + r + 1, columns lx0 + 2 ..) */
    const int y = oy + ly0 + r;
    if (y >= ty0 && y < ty1 && xany) {
      const float *row = sS + (ly0 + r + 1) * SS + lx0 + 2;
      const float2 a = ld2(row), b = ld2(row + 2);
      float *o = p.t.planes + L.ls + (long long)y * L.pitch + x0;
      if (xfull) {
        *reinterpret_cast<float4 *>(o) = make_float4(a.x, a.y, b.x, b.y);
      } else {
        const float v[4] = {a.x, a.y, b.x, b.y};
#pragma unroll
        for (int k = 0; k < 4; k++)
          if (x0 + k >= tx0 && x0 + k < tx1) o[k] = v[k];
      }
    }
  }
#pragma unroll
  for (int h = 0; h < 2; h++) { /* column pairs (x0, x0+1), (x0+2, x0+3) */
    float2 dh[5], sh[5];
#pragma unroll
    for (int j = 0; j < 5; j++) {
      const float *row = sS + (ly0 + j) * SS + lx0 + 2 * h; /* x0 + 2h - 2 .. x0 + 2h + 3 */
      const float2 A = ld2(row), B = ld2(row + 2), C = ld2(row + 4);
      const float2 P = make_float2(A.y, B.x), Q = make_float2(B.y, C.x);
      dh[j] = f2sub(Q, P);
      const float2 t = f2add(P, Q);
      sh[j] = akz_lin2<FUSED>(3.0f, t, 10.0f, make_float2(P.y, Q.x));
    }
#pragma unroll
    for (int r = 0; r < 3; r++) {
      const float2 u = f2add(dh[r], dh[r + 2]);
      const float2 gx = akz_lin2<FUSED>(3.0f, u, 10.0f, dh[r + 1]);
      const float2 gy = f2sub(sh[r + 2], sh[r]);
      const float2 m = akz_sq2sum<FUSED>(gx, gy);
      const float2 gv = p.diffusivity == 1 ? akz_pm_g2_pair<FUSED>(m, inv_k)
                                           : make_float2(akz_conductance_m(m.x, inv_k, p.diffusivity),
                                                         akz_conductance_m(m.y, inv_k, p.diffusivity));
      g[r][2 * h] = gv.x;
      g[r][2 * h + 1] = gv.y;
    }
  }
#pragma unroll
  for (int r = 0; r < 3; r++) {
    *reinterpret_cast<float4 *>(sG + (ly0 + r) * RW + lx0) = make_float4(g[r][0], g[r][1], g[r][2], g[r][3]);
    const int y = oy + ly0 + r;
    if (p.write_g && y >= ty0 && y < ty1 && xany) {
      float *og = p.t.planes + I.g + (long long)y * L.pitch + x0;
      if (xfull) {
        *reinterpret_cast<float4 *>(og) = make_float4(g[r][0], g[r][1], g[r][2], g[r][3]);
      } else {
#pragma unroll
        for (int k = 0; k < 4; k++)
          if (x0 + k >= tx0 && x0 + k < tx1) og[k] = g[r][k];
      }
    }
  }
  __syncthreads();
  return true;
}

/* The flux pair sums of one thread (columns x0 .. x0+3, rows ytop ..
 * ytop+2) from its conductances g, the rows above (ga) and below (gb) its
 * band and the lanes' neighbours (shuffles):
 *   gh[r][e]  c(x0+e-1) + c(x0+e) for e = 0..4, the fluxes west of column e
 *             (e = 4: east of column 3);
 *   gs[r][k]  c(x, y) + c(x, y+1);   gn[k] the pair above row 0.
 * A pair that crosses the image border is zero: the reference omits that
 * flux term (nldiffusion_functions.cpp:241-307), and zero times any finite
 * difference adds nothing. */
template <bool INTERIOR>
__device__ __forceinline__ void akz_fed_pairs(const float (&g)[3][4], const float4 ga, const float4 gb, int x0, int ytop,
                                              int W, int H, float (&gh)[3][5], float (&gs)[3][4], float (&gn)[4])
{
  const float ra[4] = {ga.x, ga.y, ga.z, ga.w}, rb[4] = {gb.x, gb.y, gb.z, gb.w};
#pragma unroll
  for (int r = 0; r < 3; r++) {
    const float gw = __shfl_up_sync(0xffffffffu, g[r][3], 1), ge = __shfl_down_sync(0xffffffffu, g[r][0], 1);
    const int y = ytop + r;
    const bool yin = y >= 0 && y < H, ys = y >= 0 && y + 1 < H;
#pragma unroll
    for (int e = 0; e < 5; e++) {
      const float a = e == 0 ? gw : g[r][e - 1], b = e == 4 ? ge : g[r][e];
      const int xl = x0 + e - 1; /* the pair (xl, xl + 1) */
      gh[r][e] = (INTERIOR || (yin && xl >= 0 && xl + 1 < W)) ? a + b : 0.0f;
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const float b = r < 2 ? g[r + 1][k] : rb[k];
      gs[r][k] = (INTERIOR || (ys && x0 + k >= 0 && x0 + k < W)) ? g[r][k] + b : 0.0f;
    }
  }
  const bool nin = ytop >= 1 && ytop < H;
#pragma unroll
  for (int k = 0; k < 4; k++) gn[k] = (INTERIOR || (nin && x0 + k >= 0 && x0 + k < W)) ? ra[k] + g[0][k] : 0.0f;
}

/* One FED step of this thread's 3 x 4 pixels (nld_step_scalar,
 * nldiffusion_functions.cpp:232-237, :309-316):
 *   L += h * (((xpos - xneg) + ypos) - yneg)
 * Each flux product is formed once and used twice, which is exact: the
 * reference's xneg at x+1 is (c(x) + c(x+1)) * (L(x+1) - L(x)), the same
 * operands in the same order as xpos at x, and likewise yneg at y+1 and ypos
 * at y.  Additions run as packed FP32x2 pairs; products stay scalar (with
 * FUSED: packed products and L + h * t as one packed multiply-add).  above
 * and below are the rows next to the band (old values). */
template <bool FUSED>
__device__ __forceinline__ void akz_fed_step4(float (&Lp)[3][4], float4 above, float4 below, float h,
                                              const float (&gh)[3][5], const float (&gs)[3][4], const float (&gn)[4])
{
  float Lw[3], Le[3];
#pragma unroll
  for (int r = 0; r < 3; r++) {
    Lw[r] = __shfl_up_sync(0xffffffffu, Lp[r][3], 1);
    Le[r] = __shfl_down_sync(0xffffffffu, Lp[r][0], 1);
  }
  const float ab[4] = {above.x, above.y, above.z, above.w}, bl[4] = {below.x, below.y, below.z, below.w};
  float Fn[4];
  {
    const float2 d0 = f2sub(make_float2(Lp[0][0], Lp[0][1]), make_float2(ab[0], ab[1]));
    const float2 d1 = f2sub(make_float2(Lp[0][2], Lp[0][3]), make_float2(ab[2], ab[3]));
    const float2 f0 = akz_mul2<FUSED>(make_float2(gn[0], gn[1]), d0), f1 = akz_mul2<FUSED>(make_float2(gn[2], gn[3]), d1);
    Fn[0] = f0.x;
    Fn[1] = f0.y;
    Fn[2] = f1.x;
    Fn[3] = f1.y;
  }
  float nv[3][4];
#pragma unroll
  for (int r = 0; r < 3; r++) {
    const float *L = Lp[r];
    /* horizontal differences L(x) - L(x-1) at the 5 edges */
    const float2 e01 = f2sub(make_float2(L[0], L[1]), make_float2(Lw[r], L[0]));
    const float2 e23 = f2sub(make_float2(L[2], L[3]), make_float2(L[1], L[2]));
    const float e4 = Le[r] - L[3];
    const float2 F01 = akz_mul2<FUSED>(make_float2(gh[r][0], gh[r][1]), e01);
    const float2 F23 = akz_mul2<FUSED>(make_float2(gh[r][2], gh[r][3]), e23);
    const float F0 = F01.x, F1 = F01.y, F2 = F23.x, F3 = F23.y, F4 = gh[r][4] * e4;
    const float2 xs01 = f2sub(make_float2(F1, F2), make_float2(F0, F1)); /* xpos - xneg */
    const float2 xs23 = f2sub(make_float2(F3, F4), make_float2(F2, F3));
    float nb[4];
#pragma unroll
    for (int k = 0; k < 4; k++) nb[k] = r < 2 ? Lp[r + 1][k] : bl[k];
    const float2 ds01 = f2sub(make_float2(nb[0], nb[1]), make_float2(L[0], L[1]));
    const float2 ds23 = f2sub(make_float2(nb[2], nb[3]), make_float2(L[2], L[3]));
    const float2 Fs01 = akz_mul2<FUSED>(make_float2(gs[r][0], gs[r][1]), ds01); /* ypos */
    const float2 Fs23 = akz_mul2<FUSED>(make_float2(gs[r][2], gs[r][3]), ds23);
    const float Fs[4] = {Fs01.x, Fs01.y, Fs23.x, Fs23.y};
    const float2 t01 = f2sub(f2add(xs01, Fs01), make_float2(Fn[0], Fn[1]));
    const float2 t23 = f2sub(f2add(xs23, Fs23), make_float2(Fn[2], Fn[3]));
    const float2 n01 = akz_axpy2<FUSED>(h, t01, make_float2(L[0], L[1]));
    const float2 n23 = akz_axpy2<FUSED>(h, t23, make_float2(L[2], L[3]));
    nv[r][0] = n01.x;
    nv[r][1] = n01.y;
    nv[r][2] = n23.x;
    nv[r][3] = n23.y;
#pragma unroll
    for (int k = 0; k < 4; k++) Fn[k] = Fs[k];
  }
#pragma unroll
  for (int r = 0; r < 3; r++)
#pragma unroll
    for (int k = 0; k < 4; k++) Lp[r][k] = nv[r][k];
}

/* The flux pair sums of akz_fed_pairs as register pairs, formed once per
 * launch for the fused step (the packed operations then find their
 * loop-invariant operands already paired). */
struct akz_fed_pairs2 {
  float2 h01[3], h23[3]; /* horizontal sums west of columns 0, 1 and 2, 3 */
  float h4[3];           /* east of column 3 */
  float2 s01[3], s23[3]; /* below rows 0..2 */
  float2 n01, n23;       /* above row 0 */
};

__device__ __forceinline__ akz_fed_pairs2 akz_fed_pack_pairs(const float (&gh)[3][5], const float (&gs)[3][4],
                                                            const float (&gn)[4])
{
  akz_fed_pairs2 P;
#pragma unroll
  for (int r = 0; r < 3; r++) {
    P.h01[r] = make_float2(gh[r][0], gh[r][1]);
    P.h23[r] = make_float2(gh[r][2], gh[r][3]);
    P.h4[r] = gh[r][4];
    P.s01[r] = make_float2(gs[r][0], gs[r][1]);
    P.s23[r] = make_float2(gs[r][2], gs[r][3]);
  }
  P.n01 = make_float2(gn[0], gn[1]);
  P.n23 = make_float2(gn[2], gn[3]);
  return P;
}

/* The fused step of akz_fed_step4 on the paired state: the same operations
 * (so the same results), with the image rows held as pairs (L0, L1), (L2, L3)
 * and the flux pair sums as P. */
__device__ __forceinline__ void akz_fed_step4_paired(float2 (&Lq)[3][2], float4 above, float4 below, float h,
                                                     const akz_fed_pairs2 &P)
{
  float Lw[3], Le[3];
#pragma unroll
  for (int r = 0; r < 3; r++) {
    Lw[r] = __shfl_up_sync(0xffffffffu, Lq[r][1].y, 1);
    Le[r] = __shfl_down_sync(0xffffffffu, Lq[r][0].x, 1);
  }
  float2 Fn01 = f2mul(P.n01, f2sub(Lq[0][0], make_float2(above.x, above.y)));
  float2 Fn23 = f2mul(P.n23, f2sub(Lq[0][1], make_float2(above.z, above.w)));
  const float2 hh = make_float2(h, h);
  float2 nv[3][2];
#pragma unroll
  for (int r = 0; r < 3; r++) {
    const float2 A = Lq[r][0], B = Lq[r][1];
    const float2 e01 = f2sub(A, make_float2(Lw[r], A.x));
    const float2 e23 = f2sub(B, make_float2(A.y, B.x));
    const float2 F01 = f2mul(P.h01[r], e01), F23 = f2mul(P.h23[r], e23);
    const float F4 = P.h4[r] * (Le[r] - B.y);
    const float2 xs01 = make_float2(F01.y - F01.x, F23.x - F01.y); /* xpos - xneg */
    const float2 xs23 = make_float2(F23.y - F23.x, F4 - F23.y);
    const float2 nA = r < 2 ? Lq[r + 1][0] : make_float2(below.x, below.y);
    const float2 nB = r < 2 ? Lq[r + 1][1] : make_float2(below.z, below.w);
    const float2 Fs01 = f2mul(P.s01[r], f2sub(nA, A)), Fs23 = f2mul(P.s23[r], f2sub(nB, B)); /* ypos */
    const float2 t01 = f2sub(f2add(xs01, Fs01), Fn01), t23 = f2sub(f2add(xs23, Fs23), Fn23);
    nv[r][0] = f2fma(hh, t01, A);
    nv[r][1] = f2fma(hh, t23, B);
    Fn01 = Fs01;
    Fn23 = Fs23;
  }
#pragma unroll
  for (int r = 0; r < 3; r++) {
    Lq[r][0] = nv[r][0];
    Lq[r][1] = nv[r][1];
  }
}

/* D > 0: the launch's FED depth as a compile-time constant (p.steps == D),
 * so that the step loop unrolls (the step size of each step is a constant
 * parameter offset, the exchange parity a constant, and the new values
 * land in renamed registers); D == 0: the depth from p.steps at run time. */
template <bool FUSED, int D>
__global__ void __launch_bounds__(AKZ_FED_THREADS, 2) k_fed(akz_fed_params p)
{
  extern __shared__ __align__(128) float sm_raw[];
  constexpr int RW = AKZ_FED_RW, RH = AKZ_FED_RH, PS = AKZ_FED_PS;
  if (p.gate && *p.gate <= p.gate_tol) return; /* a gated fallback that is not needed */
  /* the TMA box wants a 128-byte aligned destination */
  float *sm = sm_raw + ((128u - ((uint32_t)__cvta_generic_to_shared(sm_raw) & 127u)) & 127u) / 4;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int si = akz_find_seg_warp(p.segs, p.nsegs, blockIdx.x);
  const akz_tile_seg sg = p.segs[si];
  const akz_level_desc L = p.t.lv[sg.level_desc];
  const akz_image_desc I = p.t.im[L.image];
  const int W = L.width, H = L.height;
  const int d = D > 0 ? D : p.steps;
  const int TW = akz_fed_tile_w(d), TH = akz_fed_tile_h(d);
  const int lt = blockIdx.x - sg.tile_begin;
  const int tx0 = (lt % sg.tiles_x) * TW, ty0 = (lt / sg.tiles_x) * TH;
  const int tx1 = min(tx0 + TW, W), ty1 = min(ty0 + TH, H);
  const int ox = tx0 - d - akz_fed_delta(d), oy = ty0 - d; /* R0 origin (a multiple of 4; may lie outside the image) */
  const int srck = p.first ? sg.aux : p.src;
  float *planes = p.t.planes;

  /* this thread: columns lx0 .. lx0+3 of R0, rows ly0 .. ly0+2 */
  const int lx0 = 4 * lane, ly0 = 3 * warp;
  const int x0 = ox + lx0; /* a multiple of 4 */
  const int ytop = oy + ly0;
  const bool interior = ox >= 1 && oy >= 1 && ox + RW + 1 <= W && oy + RH + 1 <= H;

  float Lp[3][4], g[3][4];
  float4 ga, gb; /* conductances of the rows above and below the band */
  if (p.first) {
    float *sP = sm, *sT = sm + (RH + 6) * PS;
    bool ok;
    if (srck == 1)
      ok = akz_fed_prologue<1, FUSED>(p, L, I, sg.level_desc, sm, ox, oy, tx0, ty0, tx1, ty1, lx0, ly0, g);
    else if (srck == 0)
      ok = akz_fed_prologue<0, FUSED>(p, L, I, sg.level_desc, sm, ox, oy, tx0, ty0, tx1, ty1, lx0, ly0, g);
    else
      ok = akz_fed_prologue<2, FUSED>(p, L, I, sg.level_desc, sm, ox, oy, tx0, ty0, tx1, ty1, lx0, ly0, g);
    if (!ok) return; /* uniform: every thread saw the same barrier state */
    const float *sL = sP + 3 * PS + 4; /* level values of R0 */
#pragma unroll
    for (int r = 0; r < 3; r++) {
      const float4 v = *reinterpret_cast<const float4 *>(sL + (ly0 + r) * PS + lx0);
      Lp[r][0] = v.x;
      Lp[r][1] = v.y;
      Lp[r][2] = v.z;
      Lp[r][3] = v.w;
    }
    ga = *reinterpret_cast<const float4 *>(sT + max(ly0 - 1, 0) * RW + lx0);
    gb = *reinterpret_cast<const float4 *>(sT + min(ly0 + 3, RH - 1) * RW + lx0);
    __syncthreads(); /* sP and sT are the exchange rows from here */
  } else {
    const float *lp = planes + (p.src == 1 ? I.t1 : I.t2);
    const float *gp = planes + I.g;
    const long long pitch = L.pitch;
    const bool full = x0 >= 0 && x0 + 4 <= W;
    auto row4 = [&](const float *base, int y) -> float4 { /* 4 values of row y from column x0, 0 outside */
      if (y < 0 || y >= H) return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      const float *q = base + (long long)y * pitch + x0;
      if (full) return __ldg(reinterpret_cast<const float4 *>(q));
      float v[4];
#pragma unroll
      for (int k = 0; k < 4; k++) v[k] = (x0 + k >= 0 && x0 + k < W) ? __ldg(q + k) : 0.0f;
      return make_float4(v[0], v[1], v[2], v[3]);
    };
#pragma unroll
    for (int r = 0; r < 3; r++) {
      const float4 l4 = row4(lp, ytop + r), g4 = row4(gp, ytop + r);
      Lp[r][0] = l4.x;
      Lp[r][1] = l4.y;
      Lp[r][2] = l4.z;
      Lp[r][3] = l4.w;
      g[r][0] = g4.x;
      g[r][1] = g4.y;
      g[r][2] = g4.z;
      g[r][3] = g4.w;
    }
    ga = row4(gp, ytop - 1);
    gb = row4(gp, ytop + 3);
  }
  float gh[3][5], gs[3][4], gn[4];
  if (interior)
    akz_fed_pairs<true>(g, ga, gb, x0, ytop, W, H, gh, gs, gn);
  else
    akz_fed_pairs<false>(g, ga, gb, x0, ytop, W, H, gh, gs, gn);

  /* exchange rows: xb[((par * 2 + last) * 16 + warp) * RW + column] */
  float *xb = sm;
  if constexpr (FUSED) { /* the fused steps on paired registers */
    const akz_fed_pairs2 P = akz_fed_pack_pairs(gh, gs, gn);
    float2 Lq[3][2];
#pragma unroll
    for (int r = 0; r < 3; r++) {
      Lq[r][0] = make_float2(Lp[r][0], Lp[r][1]);
      Lq[r][1] = make_float2(Lp[r][2], Lp[r][3]);
    }
    auto putq = [&](int par) {
      *reinterpret_cast<float4 *>(xb + ((par * 2 + 0) * 16 + warp) * RW + lx0) =
          make_float4(Lq[0][0].x, Lq[0][0].y, Lq[0][1].x, Lq[0][1].y);
      *reinterpret_cast<float4 *>(xb + ((par * 2 + 1) * 16 + warp) * RW + lx0) =
          make_float4(Lq[2][0].x, Lq[2][0].y, Lq[2][1].x, Lq[2][1].y);
    };
    if (d > 0) {
      putq(0);
      __syncthreads();
    }
    auto stepq = [&](int s) {
      const int par = s & 1;
      const float4 above = warp > 0 ? *reinterpret_cast<const float4 *>(xb + ((par * 2 + 1) * 16 + warp - 1) * RW + lx0)
                                    : make_float4(Lq[0][0].x, Lq[0][0].y, Lq[0][1].x, Lq[0][1].y);
      const float4 below = warp < 15 ? *reinterpret_cast<const float4 *>(xb + ((par * 2 + 0) * 16 + warp + 1) * RW + lx0)
                                     : make_float4(Lq[2][0].x, Lq[2][0].y, Lq[2][1].x, Lq[2][1].y);
      akz_fed_step4_paired(Lq, above, below, p.h[s], P);
      if (s + 1 < d) {
        putq(par ^ 1);
        __syncthreads();
      }
    };
    if constexpr (D > 0) {
#pragma unroll
      for (int s = 0; s < D; s++) stepq(s);
    } else {
      for (int s = 0; s < d; s++) stepq(s);
    }
#pragma unroll
    for (int r = 0; r < 3; r++) {
      Lp[r][0] = Lq[r][0].x;
      Lp[r][1] = Lq[r][0].y;
      Lp[r][2] = Lq[r][1].x;
      Lp[r][3] = Lq[r][1].y;
    }
  } else {
  auto put = [&](int par) {
    *reinterpret_cast<float4 *>(xb + ((par * 2 + 0) * 16 + warp) * RW + lx0) = make_float4(Lp[0][0], Lp[0][1], Lp[0][2], Lp[0][3]);
    *reinterpret_cast<float4 *>(xb + ((par * 2 + 1) * 16 + warp) * RW + lx0) = make_float4(Lp[2][0], Lp[2][1], Lp[2][2], Lp[2][3]);
  };
  if (d > 0) {
    put(0);
    __syncthreads();
  }
  auto step = [&](int s) {
    const int par = s & 1;
    const float4 above = warp > 0 ? *reinterpret_cast<const float4 *>(xb + ((par * 2 + 1) * 16 + warp - 1) * RW + lx0)
                                  : make_float4(Lp[0][0], Lp[0][1], Lp[0][2], Lp[0][3]);
    const float4 below = warp < 15 ? *reinterpret_cast<const float4 *>(xb + ((par * 2 + 0) * 16 + warp + 1) * RW + lx0)
                                   : make_float4(Lp[2][0], Lp[2][1], Lp[2][2], Lp[2][3]);
    akz_fed_step4<FUSED>(Lp, above, below, p.h[s], gh, gs, gn);
    if (s + 1 < d) {
      put(par ^ 1);
      __syncthreads();
    }
  };
  if constexpr (D > 0) {
#pragma unroll
    for (int s = 0; s < D; s++) step(s);
  } else {
    for (int s = 0; s < d; s++) step(s);
  }
  }
  /* tile interior from registers, one 128-bit store per row */
  float *out = p.dst == 3 ? p.chk : planes + (p.dst == 0 ? L.lt : (p.dst == 1 ? I.t1 : I.t2));
#pragma unroll
  for (int r = 0; r < 3; r++) {
    const int y = ytop + r;
    if (y < ty0 || y >= ty1) continue;
    float *o = out + (long long)y * L.pitch + x0;
    if (x0 >= tx0 && x0 + 4 <= tx1) {
      *reinterpret_cast<float4 *>(o) = make_float4(Lp[r][0], Lp[r][1], Lp[r][2], Lp[r][3]);
    } else {
#pragma unroll
      for (int k = 0; k < 4; k++)
        if (x0 + k >= tx0 && x0 + k < tx1) o[k] = Lp[r][k];
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
  if (nbins < 1 || nbins > AKZ_MAX_NBINS) return cudaErrorInvalidValue;
  k_contrast_final<<<t.nimg, 32, (size_t)nbins * sizeof(unsigned int), s>>>(t, hist, nbins, perc, kc);
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
  if (p.steps < 0 || p.steps > 8) return cudaErrorInvalidValue; /* 0: Lsmooth, conductance and the start image only */
  if (p.first && !p.tmaps) return cudaErrorInvalidValue;         /* the input box needs the tensor maps */
  const size_t smem = akz_fed_smem_bytes(0, 0, p.steps, p.first);
  auto go = [&](auto kern) -> cudaError_t {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<ntiles, AKZ_FED_THREADS, smem, s>>>(p);
    return cudaGetLastError();
  };
  if (!p.fused) {
    switch (p.steps) { /* both modes unroll their depth */
    case 1: return go(k_fed<false, 1>);
    case 2: return go(k_fed<false, 2>);
    case 3: return go(k_fed<false, 3>);
    case 4: return go(k_fed<false, 4>);
    case 5: return go(k_fed<false, 5>);
    case 6: return go(k_fed<false, 6>);
    case 7: return go(k_fed<false, 7>);
    case 8: return go(k_fed<false, 8>);
    default: return go(k_fed<false, 0>);
    }
  }
  switch (p.steps) {
  case 1: return go(k_fed<true, 1>);
  case 2: return go(k_fed<true, 2>);
  case 3: return go(k_fed<true, 3>);
  case 4: return go(k_fed<true, 4>);
  case 5: return go(k_fed<true, 5>);
  case 6: return go(k_fed<true, 6>);
  case 7: return go(k_fed<true, 7>);
  case 8: return go(k_fed<true, 8>);
  default: return go(k_fed<true, 0>);
  }
}

cudaError_t akz_launch_area(const akz_area_params &p, int maxw, int maxh, cudaStream_t s)
{
  if (p.nsegs <= 0) return cudaSuccess;
  const dim3 block(32, 8);
  const dim3 grid((maxw + 31) / 32, (maxh + 7) / 8, p.nsegs);
  k_area<<<grid, block, 0, s>>>(p);
  return cudaGetLastError();
}

/* ------------------------------------------------------------------------ */
/* Device self-check of the exact PM-g2 reciprocal: out[i] = the conductance
 * of f = in[i] (inv_k = 1) from the pair routine (fn 0) or the scalar one
 * (fn 1), for comparison with (float)(1 / (1 + (double)f)) on the host. */
__global__ void k_pm_g2_check(const float *in, float *out, int n, int fn)
{
  const int i = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
  if (i >= n) return;
  const float a = in[i], b = i + 1 < n ? in[i + 1] : 0.0f;
  float2 r;
  if (fn == 0)
    r = akz_pm_g2_pair<false>(make_float2(a, b), 1.0f);
  else
    r = make_float2(akz_recip1pf(a), akz_recip1pf(b));
  out[i] = r.x;
  if (i + 1 < n) out[i + 1] = r.y;
}

extern "C" AKZ_API akz_status akz_selfcheck_pm_g2(const float *in, float *out, int n, int fn, void *stream)
{
  if (n < 0 || (n > 0 && (!in || !out)) || fn < 0 || fn > 1) return akz_report(AKZ_ERR_INVALID_ARG, "akz_selfcheck_pm_g2: bad arguments");
  if (n == 0) return AKZ_OK;
  k_pm_g2_check<<<((n + 1) / 2 + 255) / 256, 256, 0, (cudaStream_t)stream>>>(in, out, n, fn);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? AKZ_OK : akz_report(AKZ_ERR_CUDA, cudaGetErrorString(e));
}
