/*
 * akz_detect.cu - Hessian detector, extrema, ordering and suppression.
 *
 *   k_detect   one fused tile kernel per launch over every (image, level):
 *              Lsmooth tile -> scaled Scharr derivatives Lx, Ly with step
 *              sigma_size and reflect-101 border (cuda_akaze.cu:651-671,
 *              written to HBM for orientation and M-LDB) -> Hessian
 *              determinant in shared memory (:673-701) -> strict 3x3 maxima
 *              above the threshold inside the border (:727-743), recorded as
 *              one bit per pixel plus a per-row count.
 *   k_rowscan  exclusive scan of the row counts of each image: the raw
 *              extrema come out in (level, y, x) order, which is the order
 *              the reference's per-level bitonic sort gives (:884-939),
 *              with no per-level cap.
 *   k_extract  one warp per row: subpixel fit and record (:744-769), the
 *              determinant recomputed from Lx, Ly at the 3x3 neighbourhood.
 *   k_nms      one CTA per image: the reference's round-based suppression
 *              (:1005-1224) with an exact per-slot minimum (atomicMin), then
 *              the 2048-slot chunked emission and subpixel restore
 *              (:1227-1316).
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>

#include "akz_device.cuh"
#include "akz_fmath.h"

/* ------------------------------------------------------------------------ */

/* The reference's border test for an extremum at coordinate v of a level of
 * size n (cuda_akaze.cu:734-740):
 *   (int)((float)v - border + 0.5f) - 1 >= 0  and  (int)((float)v + border + 0.5f) + 1 < n.
 * Both sides are monotone in v, so the accepted coordinates form one range;
 * these return its ends, found with the same float expressions. */
__device__ __forceinline__ int akz_border_lo(float border)
{
  int v = max((int)border - 2, 0);
  while ((int)((float)v - border + 0.5f) - 1 < 0) v++;
  return v;
}

__device__ __forceinline__ int akz_border_hi(float border, int n)
{
  int v = min(n - 1 - (int)border + 2, n - 1);
  while (v >= 0 && (int)((float)v + border + 0.5f) + 1 >= n) v--;
  return v;
}

/* k_detect for every tile of a level with derivative step ST (2..4, the steps
 * of the default options): compile-time region sizes, straight-line loops,
 * column pairs with packed FP32x2 additions (products scalar), in the
 * reference's operation order.
 *
 * Borders: the Lsmooth region is staged with reflect-101 coordinates, which
 * makes Lx and Ly exact at every pixel inside the image (their taps at +-ST
 * are the reference's reflect-101 indices, cuda_akaze.cu:657-660).  The
 * determinant reads Lx and Ly at reflect-101 indices too, i.e. the mirrored
 * in-image value, not a derivative of the mirrored image, so after the
 * derivative pass the entries just outside the image (within ST) are
 * replaced by their in-image mirrors.
 *
 * Layout: tile (62 - 2 ST) x 32, so the Lx, Ly region is exactly 64 columns
 * (32 pairs): one warp per row in both passes, no row wraps inside a warp,
 * hence no shared-memory bank conflicts for the 64-bit pair accesses. */
template <int ST, bool BORDER>
__device__ __forceinline__ void akz_detect_tile(const akz_detect_params &p, const akz_level_desc &L, float *sm, int tx0,
                                                int ty0)
{
  constexpr int TW = 62 - 2 * ST, TH = AKZ_DETECT_TH;
  constexpr int DW = TW + 2 * ST + 2, DH = TH + 2 * ST + 2; /* Lx, Ly:  tile +- (ST+1)  */
  constexpr int SW = TW + 4 * ST + 2, SH = TH + 4 * ST + 2; /* Lsmooth: tile +- (2ST+1) */
  constexpr int SWS = SW;                                   /* Lsmooth row stride */
  constexpr int EW = TW + 2, EH = TH + 2;                   /* Ldet:    tile +- 1       */
  constexpr int DP = DW / 2, EP = EW / 2;                   /* column pairs */
  static_assert(DW == 64 && EP <= 32 && EW % 2 == 0 && SW % 2 == 0, "pair layout");
  static_assert(EW * EH <= SWS * SH, "determinant plane fits the Lsmooth region");
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int W = L.width, H = L.height;
  /* the determinant plane reuses the Lsmooth region, dead after the derivative pass */
  float *sS = sm, *sX = sm + SWS * SH, *sY = sX + DW * DH, *sD = sm;
  const float fac1 = p.fac1, fac2 = p.fac2;
  const float *ls = p.t.planes + L.ls;
  if (BORDER) {
#pragma unroll
    for (int n = warp; n < SH; n += 8) {
      const int y = akz_refl101(min(ty0 - 2 * ST - 1 + n, H + 2 * ST), H);
      const float *q = ls + (long long)y * L.pitch;
#pragma unroll
      for (int j = 0; j < (SW + 31) / 32; j++) {
        const int m = lane + 32 * j;
        if (m < SW) sS[n * SWS + m] = __ldg(q + akz_refl101(min(tx0 - 2 * ST - 1 + m, W + 2 * ST), W));
      }
    }
  } else {
    const float *q0 = ls + (long long)(ty0 - 2 * ST - 1) * L.pitch + (tx0 - 2 * ST - 1);
#pragma unroll
    for (int n = warp; n < SH; n += 8) {
      const float *q = q0 + (long long)n * L.pitch;
#pragma unroll
      for (int j = 0; j < (SW + 31) / 32; j++) {
        const int m = lane + 32 * j;
        if (m < SW) sS[n * SWS + m] = __ldg(q + m);
      }
    }
  }
  __syncthreads();
  /* Lx, Ly on the tile +- (ST+1), two columns per item: D column d is
   * Lsmooth column d + ST; its taps sit at d, d + ST and d + 2ST, so the
   * outer taps are aligned pairs for every ST (cuda_akaze.cu:651-671) */
  const int dx0 = tx0 - ST - 1, dy0 = ty0 - ST - 1; /* image coordinates of D (0, 0) */
  float *lxp = p.t.planes + L.lx, *lyp = p.t.planes + L.ly;
  for (int n = warp; n < DH; n += 8) {
    const int d = 2 * lane;
    const float *su = sS + n * SWS + d, *sc = su + ST * SWS, *sd = su + 2 * ST * SWS;
    const float2 ul = ld2(su), ur = ld2(su + 2 * ST), ll = ld2(sd), lr = ld2(sd + 2 * ST);
    const float2 cl = ld2(sc), cr = ld2(sc + 2 * ST);
    const float2 uc = (ST & 1) ? make_float2(su[ST], su[ST + 1]) : ld2(su + ST);
    const float2 lc = (ST & 1) ? make_float2(sd[ST], sd[ST + 1]) : ld2(sd + ST);
    const float2 ax = f2sub(f2sub(f2add(ur, lr), ul), ll), bx = f2sub(cr, cl);
    const float2 ay = f2sub(f2sub(f2add(lr, ll), ur), ul), by = f2sub(lc, uc);
    const float2 a = f2add(make_float2(fac1 * ax.x, fac1 * ax.y), make_float2(fac2 * bx.x, fac2 * bx.y));
    const float2 b = f2add(make_float2(fac1 * ay.x, fac1 * ay.y), make_float2(fac2 * by.x, fac2 * by.y));
    st2(sX + n * DW + d, a);
    st2(sY + n * DW + d, b);
    const int y = dy0 + n, x = dx0 + d;
    if (n >= ST + 1 && n < ST + 1 + TH && (!BORDER || y < H)) {
      float *ox = lxp + (long long)y * L.pitch + x, *oy = lyp + (long long)y * L.pitch + x;
      if (d >= ST + 1 && d < ST + 1 + TW && (!BORDER || x < W)) {
        ox[0] = a.x;
        oy[0] = b.x;
      }
      if (d + 1 >= ST + 1 && d + 1 < ST + 1 + TW && (!BORDER || x + 1 < W)) {
        ox[1] = a.y;
        oy[1] = b.y;
      }
    }
  }
  __syncthreads();
  /* reflect-101 mirrors of Lx, Ly within ST outside the image: columns
   * first, then whole rows (which covers the corners); the sources are
   * in-image entries, which these passes do not write */
  if (BORDER && (dx0 < 0 || dx0 + DW > W)) {
    for (int i = tid; i < DH * DW; i += 256) {
      const int n = i / DW, c = i - n * DW, x = dx0 + c;
      const int xm = x < 0 ? -x : (x >= W && x <= W - 1 + ST ? 2 * W - 2 - x : -1);
      if (xm >= 0) {
        sX[n * DW + c] = sX[n * DW + xm - dx0];
        sY[n * DW + c] = sY[n * DW + xm - dx0];
      }
    }
    __syncthreads();
  }
  if (BORDER && (dy0 < 0 || dy0 + DH > H)) {
    for (int i = tid; i < DH * DW; i += 256) {
      const int n = i / DW, c = i - n * DW, y = dy0 + n;
      const int ym = y < 0 ? -y : (y >= H && y <= H - 1 + ST ? 2 * H - 2 - y : -1);
      if (ym >= 0) {
        sX[n * DW + c] = sX[(ym - dy0) * DW + c];
        sY[n * DW + c] = sY[(ym - dy0) * DW + c];
      }
    }
    __syncthreads();
  }
  /* Hessian determinant on the tile +- 1 (cuda_akaze.cu:673-701): E column e
   * is D column e + ST */
  for (int n = warp; n < EH; n += 8) {
    const int e = 2 * lane;
    if (lane >= EP) continue;
    const float *xu = sX + n * DW + e, *xc = xu + ST * DW, *xd = xu + 2 * ST * DW;
    const float *yu = sY + n * DW + e, *yd = yu + 2 * ST * DW;
    const float2 ul = ld2(xu), ur = ld2(xu + 2 * ST), ll = ld2(xd), lr = ld2(xd + 2 * ST);
    const float2 cl = ld2(xc), cr = ld2(xc + 2 * ST);
    const float2 xuc = (ST & 1) ? make_float2(xu[ST], xu[ST + 1]) : ld2(xu + ST);
    const float2 xdc = (ST & 1) ? make_float2(xd[ST], xd[ST + 1]) : ld2(xd + ST);
    const float2 ax = f2sub(f2sub(f2add(ur, lr), ul), ll), bx = f2sub(cr, cl);
    const float2 ay = f2sub(f2sub(f2add(lr, ll), ur), ul), by = f2sub(xdc, xuc);
    const float2 lxx = f2add(make_float2(fac1 * ax.x, fac1 * ax.y), make_float2(fac2 * bx.x, fac2 * bx.y));
    const float2 lyx = f2add(make_float2(fac1 * ay.x, fac1 * ay.y), make_float2(fac2 * by.x, fac2 * by.y));
    const float2 vul = ld2(yu), vur = ld2(yu + 2 * ST), vll = ld2(yd), vlr = ld2(yd + 2 * ST);
    const float2 yuc = (ST & 1) ? make_float2(yu[ST], yu[ST + 1]) : ld2(yu + ST);
    const float2 ydc = (ST & 1) ? make_float2(yd[ST], yd[ST + 1]) : ld2(yd + ST);
    const float2 cy = f2sub(f2sub(f2add(vlr, vll), vur), vul), dy = f2sub(ydc, yuc);
    const float2 lyy = f2add(make_float2(fac1 * cy.x, fac1 * cy.y), make_float2(fac2 * dy.x, fac2 * dy.y));
    st2(sD + n * EW + e, f2sub(make_float2(lxx.x * lyy.x, lxx.y * lyy.y), make_float2(lyx.x * lyx.x, lyx.y * lyx.y)));
  }
  __syncthreads();
  /* strict 3x3 maxima above the threshold inside the border (cuda_akaze.cu:727-743);
   * the border range also rejects tile pixels outside the image */
  const int xlo = akz_border_lo(L.border), xhi = akz_border_hi(L.border, W);
  const int ylo = akz_border_lo(L.border), yhi = akz_border_hi(L.border, H);
  for (int j = warp; j < TH; j += 8) {
    const int y = ty0 + j;
    if (y < ylo || y > yhi) continue;
#pragma unroll
    for (int k = 0; k < (TW + 31) / 32; k++) {
      const int i = lane + 32 * k;
      const int x = tx0 + i;
      if (i >= TW || x < xlo || x > xhi) continue;
      const float *c = sD + (j + 1) * EW + (i + 1);
      const float v = c[0];
      if (v > p.thr) {
        if (v > c[-EW - 1] && v > c[EW + 1] && v > c[EW - 1] && v > c[-EW + 1] && v > c[-1] && v > c[1] &&
            v > c[EW] && v > c[-EW]) {
          atomicOr(&p.bitmap[L.bitmap + (long long)y * L.bitmap_pitch + (x >> 5)], 1u << (x & 31));
          atomicAdd(&p.rowcnt[L.rows + y], 1);
        }
      }
    }
  }
}

__global__ void __launch_bounds__(256) k_detect(akz_detect_params p, int max_step)
{
  constexpr int TW = AKZ_DETECT_TW, TH = AKZ_DETECT_TH;
  extern __shared__ float sm[];
  const int tid = threadIdx.x;
  const int si = akz_find_seg(p.segs, p.nsegs, blockIdx.x);
  const akz_tile_seg sg = p.segs[si];
  const akz_level_desc L = p.t.lv[sg.level_desc];
  const int W = L.width, H = L.height, st = L.deriv_step;
  const int lt = blockIdx.x - sg.tile_begin;
  const int tw = akz_detect_tile_width(st);
  const int tx0 = (lt % sg.tiles_x) * tw, ty0 = (lt / sg.tiles_x) * TH;
  const int tx1 = min(tx0 + TW, W), ty1 = min(ty0 + TH, H);
  const int sx0 = max(tx0 - 2 * st - 1, 0), sx1 = min(tx1 + 2 * st + 1, W);
  const int sy0 = max(ty0 - 2 * st - 1, 0), sy1 = min(ty1 + 2 * st + 1, H);
  const int dx0 = max(tx0 - st - 1, 0), dx1 = min(tx1 + st + 1, W);
  const int dy0 = max(ty0 - st - 1, 0), dy1 = min(ty1 + st + 1, H);
  const int ex0 = max(tx0 - 1, 0), ex1 = min(tx1 + 1, W), ey0 = max(ty0 - 1, 0), ey1 = min(ty1 + 1, H);
  const int sw = sx1 - sx0, dw = dx1 - dx0, ew = ex1 - ex0;
  if (st >= 2 && st <= 4 && st <= max_step) {
    const bool border = tx0 - 2 * st - 1 < 0 || ty0 - 2 * st - 1 < 0 || tx0 + tw + 2 * st + 1 > W ||
                        ty0 + TH + 2 * st + 1 > H;
    if (border) {
      if (st == 2)
        akz_detect_tile<2, true>(p, L, sm, tx0, ty0);
      else if (st == 3)
        akz_detect_tile<3, true>(p, L, sm, tx0, ty0);
      else
        akz_detect_tile<4, true>(p, L, sm, tx0, ty0);
    } else {
      if (st == 2)
        akz_detect_tile<2, false>(p, L, sm, tx0, ty0);
      else if (st == 3)
        akz_detect_tile<3, false>(p, L, sm, tx0, ty0);
      else
        akz_detect_tile<4, false>(p, L, sm, tx0, ty0);
    }
    return;
  }
  const int SM = (TW + 4 * max_step + 2) * (TH + 4 * max_step + 2);
  const int DM = (TW + 2 * max_step + 2) * (TH + 2 * max_step + 2);
  float *sS = sm, *sX = sm + SM, *sY = sX + DM, *sD = sm; /* determinant plane over the dead Lsmooth region */

  const int lane = tid & 31, warp = tid >> 5;
  const float *ls = p.t.planes + L.ls;
  for (int y = sy0 + warp; y < sy1; y += 8)
    for (int x = sx0 + lane; x < sx1; x += 32) sS[(y - sy0) * sw + (x - sx0)] = __ldg(ls + (long long)y * L.pitch + x);
  __syncthreads();
  float *lxp = p.t.planes + L.lx, *lyp = p.t.planes + L.ly;
  const float fac1 = p.fac1, fac2 = p.fac2;
  /* Lx, Ly on the tile +- (step+1): scaled Scharr with step sigma_size and
   * reflect-101 offsets (cuda_akaze.cu:651-671) */
  for (int y = dy0 + warp; y < dy1; y += 8) {
    const int yl = y < st ? st - y : y - st;
    const int yh = y >= H - st ? 2 * H - y - st - 2 : y + st;
    const float *su = sS + (yl - sy0) * sw - sx0, *sc = sS + (y - sy0) * sw - sx0, *sd = sS + (yh - sy0) * sw - sx0;
    float *ox = sX + (y - dy0) * dw - dx0, *oy = sY + (y - dy0) * dw - dx0;
    const bool yt = y >= ty0 && y < ty1;
    for (int x = dx0 + lane; x < dx1; x += 32) {
      const int xl = x < st ? st - x : x - st;
      const int xh = x >= W - st ? 2 * W - x - st - 2 : x + st;
      const float ul = su[xl], ur = su[xh], ll = sd[xl], lr = sd[xh];
      const float cl = sc[xl], cr = sc[xh], uc = su[x], lc = sd[x];
      const float a = fac1 * (ur + lr - ul - ll) + fac2 * (cr - cl);
      const float b = fac1 * (lr + ll - ur - ul) + fac2 * (lc - uc);
      ox[x] = a;
      oy[x] = b;
      if (yt && x >= tx0 && x < tx1) {
        lxp[(long long)y * L.pitch + x] = a;
        lyp[(long long)y * L.pitch + x] = b;
      }
    }
  }
  __syncthreads();
  /* Hessian determinant on the tile +- 1 (cuda_akaze.cu:673-701) */
  for (int y = ey0 + warp; y < ey1; y += 8) {
    const int yl = y < st ? st - y : y - st;
    const int yh = y >= H - st ? 2 * H - y - st - 2 : y + st;
    const float *xu = sX + (yl - dy0) * dw - dx0, *xc = sX + (y - dy0) * dw - dx0, *xd = sX + (yh - dy0) * dw - dx0;
    const float *yu = sY + (yl - dy0) * dw - dx0, *yd = sY + (yh - dy0) * dw - dx0;
    float *o = sD + (y - ey0) * ew - ex0;
    for (int x = ex0 + lane; x < ex1; x += 32) {
      const int xl = x < st ? st - x : x - st;
      const int xh = x >= W - st ? 2 * W - x - st - 2 : x + st;
      float ul = xu[xl], ur = xu[xh], ll = xd[xl], lr = xd[xh];
      const float lxx = fac1 * (ur + lr - ul - ll) + fac2 * (xc[xh] - xc[xl]);
      const float lyx = fac1 * (lr + ll - ur - ul) + fac2 * (xd[x] - xu[x]);
      ul = yu[xl];
      ur = yu[xh];
      ll = yd[xl];
      lr = yd[xh];
      const float lyy = fac1 * (lr + ll - ur - ul) + fac2 * (yd[x] - yu[x]);
      o[x] = lxx * lyy - lyx * lyx;
    }
  }
  __syncthreads();
  const float border = L.border;
  for (int y = ty0 + warp; y < ty1; y += 8)
    for (int x = tx0 + lane; x < tx1; x += 32) {
    const int left_x = (int)((float)x - border + 0.5f) - 1;
    const int right_x = (int)((float)x + border + 0.5f) + 1;
    const int up_y = (int)((float)y - border + 0.5f) - 1;
    const int down_y = (int)((float)y + border + 0.5f) + 1;
    if (left_x < 0 || right_x >= W || up_y < 0 || down_y >= H) continue;
    const float *c = sD + (y - ey0) * ew + (x - ex0);
    const float v = c[0];
    if (v > p.thr && v > c[-ew - 1] && v > c[ew + 1] && v > c[ew - 1] && v > c[-ew + 1] && v > c[-1] && v > c[1] &&
        v > c[ew] && v > c[-ew]) {
      atomicOr(&p.bitmap[L.bitmap + (long long)y * L.bitmap_pitch + (x >> 5)], 1u << (x & 31));
      atomicAdd(&p.rowcnt[L.rows + y], 1);
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Exclusive scan of each image's row counts (rows of all its levels,
 * concatenated, plus one closing entry).                                   */

__global__ void __launch_bounds__(1024) k_rowscan(akz_tables t, const int *rowcnt, int *rowscan)
{
  __shared__ int sWarp[32];
  __shared__ int sCarry;
  const akz_image_desc I = t.im[blockIdx.x];
  const int n = I.rows_total;
  const int *c = rowcnt + I.rows_base;
  int *o = rowscan + I.rows_base;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (threadIdx.x == 0) sCarry = 0;
  __syncthreads();
  for (int base = 0; base < n; base += 1024) {
    const int i = base + threadIdx.x;
    const int v = i < n ? c[i] : 0;
    int x = v;
    for (int d = 1; d < 32; d <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, d);
      if (lane >= d) x += y;
    }
    if (lane == 31) sWarp[wid] = x;
    __syncthreads();
    if (wid == 0) {
      int w = sWarp[lane];
      for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, w, d);
        if (lane >= d) w += y;
      }
      sWarp[lane] = w;
    }
    __syncthreads();
    const int incl = x + (wid > 0 ? sWarp[wid - 1] : 0);
    if (i < n) o[i] = sCarry + incl - v;
    __syncthreads();
    if (threadIdx.x == 1023) sCarry += incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    o[n] = sCarry;
    akz_image_stats *s = &t.stats[blockIdx.x];
    s->nraw = sCarry;
    s->overflow = sCarry > I.raw_cap ? 1 : 0;
    if (s->overflow) s->status = 4; /* AKZ_ERR_OVERFLOW */
  }
}

/* ------------------------------------------------------------------------ */

__global__ void __launch_bounds__(256) k_extract(akz_extract_params p, int nrows)
{
  const int lane = threadIdx.x & 31;
  const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (r >= nrows) return;
  const int si = akz_find_seg(p.segs, p.nsegs, r);
  const akz_tile_seg sg = p.segs[si];
  const akz_level_desc L = p.t.lv[sg.level_desc];
  const akz_image_desc I = p.t.im[L.image];
  const int y = r - sg.tile_begin;
  const int W = L.width, H = L.height, st = L.deriv_step;
  const int words = L.bitmap_pitch;
  const uint32_t *row = p.bitmap + L.bitmap + (long long)y * words;
  const int rank0 = p.rowscan[L.rows + y];
  akz_raw *out = p.raw + I.raw_base;
  const akz_plane_acc X{p.t.planes + L.lx, L.pitch}, Y{p.t.planes + L.ly, L.pitch};
  const int ratio = 1 << L.octave;
  int running = 0;
  for (int w0 = 0; w0 < words; w0 += 32) {
    const int w = w0 + lane;
    uint32_t bits = w < words ? row[w] : 0u;
    const int cnt = __popc(bits);
    int pre = cnt;
    for (int d = 1; d < 32; d <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, pre, d);
      if (lane >= d) pre += t;
    }
    const int total = __shfl_sync(0xffffffffu, pre, 31);
    int k = running + pre - cnt;
    while (bits) {
      const int b = __ffs(bits) - 1;
      bits &= bits - 1;
      const int x = w * 32 + b;
      const int idx = rank0 + k++;
      if (idx >= I.raw_cap) continue;
      float D[3][3];
      for (int j = -1; j <= 1; j++)
        for (int i = -1; i <= 1; i++) D[j + 1][i + 1] = akz_det_at(X, Y, W, H, st, x + i, y + j, p.fac1, p.fac2);
      const float v = D[1][1];
      const float dx = 0.5f * (D[1][2] - D[1][0]);
      const float dy = 0.5f * (D[2][1] - D[0][1]);
      const float dxx = D[1][2] + D[1][0] - 2.0f * v;
      const float dyy = D[2][1] + D[0][1] - 2.0f * v;
      const float dxy = 0.25f * (D[2][2] + D[0][0] - D[2][0] - D[0][2]);
      const float det = dxx * dyy - dxy * dxy;
      const float idet = (det != 0.0f ? 1.0f / det : 0.0f);
      const float dst0 = idet * (dxy * dy - dyy * dx);
      const float dst1 = idet * (dxy * dx - dxx * dy);
      const bool weak = !(dst0 >= -1.0f && dst0 <= 1.0f && dst1 >= -1.0f && dst1 <= 1.0f);
      akz_raw e;
      e.x = x;
      e.y = y;
      e.level = L.level;
      e.octave = L.octave;
      e.response = v;
      e.size = (float)((weak ? -1 : 1) * 2.0 * (double)L.size);
      const float octsub = (float)(dst0 < 0 ? -1 : 1) * ((float)L.octave + fabsf(dst0));
      e.octsub = weak ? (float)L.octave : octsub;
      e.dst1 = dst1;
      out[idx] = e;
    }
    running += total;
  }
  (void)ratio;
}

/* ------------------------------------------------------------------------ */
/* Suppression.                                                             */

struct akz_nms_ctx {
  const akz_raw *R;
  const int *state;
  const int *rs; /* image-local row scan */
  const akz_level_desc *lv;
  int first_level;
  long long rows_base;
};

/* Decision of unsettled point i: 0 wait (an earlier neighbour is unsettled),
 * 1 take its own slot, 2 challenge *target (the settled neighbour with the
 * smallest slot value). Neighbours: FindNeighbors, cuda_akaze.cu:1005-1070. */
/* Visits the neighbours of raw extremum i in the reference's sense
 * (cuda_akaze.cu:1005-1070): earlier points of the same level and points of
 * the previous level whose squared distance is below (size/2)^2; weak points
 * (negative size) have none.  f(j) returns false to stop; visit returns
 * false when stopped. */
template <class F>
__device__ __forceinline__ bool akz_nms_visit(const akz_nms_ctx &c, int i, F f)
{
  const akz_raw e = c.R[i];
  const float size = e.size;
  if (!(size >= 0.0f)) return true;
  const float hs = size * .5f;
  const float lim = size * size * 0.25f;
  const akz_level_desc L = c.lv[c.first_level + e.level];
  const int r = 1 << e.octave;
  const float px = (float)(r * e.x), py = (float)(r * e.y);
  const long long rowb = L.rows - c.rows_base;
  /* same level: earlier points whose rows are within hs */
  for (int yy = e.y; yy >= 0; yy--) {
    const float pyj = (float)(r * yy);
    if (py - pyj > hs) break;
    const int j0 = c.rs[rowb + yy];
    const int j1 = yy == e.y ? i : c.rs[rowb + yy + 1];
    for (int j = j0; j < j1; j++) {
      const float ddx = px - (float)(r * c.R[j].x), ddy = py - pyj;
      if (ddx * ddx + ddy * ddy < lim && !f(j)) return false;
    }
  }
  /* previous level: points whose rows are within hs either way */
  if (e.level > 0) {
    const akz_level_desc P = c.lv[c.first_level + e.level - 1];
    const int rp = 1 << P.octave;
    const long long rowp = P.rows - c.rows_base;
    const int ylo = max((int)floorf((py - hs) / (float)rp) - 1, 0);
    const int yhi = min((int)floorf((py + hs) / (float)rp) + 1, P.height - 1);
    for (int yy = ylo; yy <= yhi; yy++) {
      const float pyj = (float)(rp * yy);
      if (pyj - py > hs) continue;
      if (py - pyj > hs) continue;
      const int j0 = c.rs[rowp + yy], j1 = c.rs[rowp + yy + 1];
      for (int j = j0; j < j1; j++) {
        const float ddx = px - (float)(rp * c.R[j].x), ddy = py - pyj;
        if (ddx * ddx + ddy * ddy < lim && !f(j)) return false;
      }
    }
  }
  return true;
}

/* One point's decision in a round: 0 wait (an unsettled neighbour), 1 take
 * its own slot (no settled neighbour), 2 challenge *target, the settled
 * neighbour with the smallest slot value. */
struct akz_nms_pick {
  const int *state;
  int best, bestv;
  bool wait;
  __device__ __forceinline__ bool operator()(int j)
  {
    const int sj = state[j];
    if (sj == -1) {
      wait = true;
      return false;
    }
    if (sj >= 0 && sj < bestv) {
      bestv = sj;
      best = j;
    }
    return true;
  }
};

__device__ __forceinline__ int akz_nms_decide(const akz_nms_ctx &c, int i, int *target)
{
  akz_nms_pick pk{c.state, -1, INT_MAX, false};
  akz_nms_visit(c, i, [&](int j) { return pk(j); });
  if (pk.wait) return 0;
  if (pk.best < 0) return 1;
  *target = pk.best;
  return 2;
}

__device__ __forceinline__ void akz_bitonic2048(int *v)
{
  const int t = threadIdx.x; /* 1024 threads */
  for (int k = 2; k <= 2048; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      const int i = ((t & ~(j - 1)) << 1) | (t & (j - 1));
      const int l = i | j;
      const bool up = (i & k) == 0;
      const int a = v[i], b = v[l];
      if ((a > b) == up) {
        v[i] = b;
        v[l] = a;
      }
      __syncthreads();
    }
  }
}

__global__ void __launch_bounds__(AKZ_NMS_THREADS) k_nms(akz_nms_params p)
{
  __shared__ int sv[2048];
  const int img = blockIdx.x;
  const int tid = threadIdx.x;
  const akz_image_desc I = p.t.im[img];
  akz_image_stats *stats = &p.t.stats[img];
  if (stats->overflow) {
    if (tid == 0) stats->nkp = 0;
    return;
  }
  const int n = stats->nraw;
  const akz_raw *R = p.raw + I.raw_base;
  int *state = p.state + I.raw_base;
  int *minc = p.aux + I.raw_base;
  signed char *dec = p.decision + I.raw_base;
  for (int i = tid; i < n; i += AKZ_NMS_THREADS) {
    state[i] = -1;
    minc[i] = INT_MAX;
  }
  __syncthreads();
  const akz_nms_ctx c{R, state, p.rowscan + I.rows_base, p.t.lv, I.first_level, I.rows_base};
  /* neighbour sets, found once (the rounds then cost O(neighbours) each);
   * a point with more than AKZ_NMS_NB neighbours is decided by scanning */
  int *nbr = p.nbr + (long long)I.raw_base * AKZ_NMS_NB;
  unsigned char *nbc = p.nbc + I.raw_base;
  for (int i = tid; i < n; i += AKZ_NMS_THREADS) {
    int cnt = 0;
    int *li = nbr + (long long)i * AKZ_NMS_NB;
    const bool all = akz_nms_visit(c, i, [&](int j) {
      if (cnt == AKZ_NMS_NB) return false;
      li[cnt++] = j;
      return true;
    });
    nbc[i] = (unsigned char)(all ? cnt : AKZ_NMS_NB + 1);
  }
  __syncthreads();
  int rounds = 0;
  for (;;) {
    int any = 0;
    for (int i = tid; i < n; i += AKZ_NMS_THREADS) {
      if (state[i] != -1) continue;
      any = 1;
      int target = -1, d;
      const int cnt = nbc[i];
      if (cnt <= AKZ_NMS_NB) {
        akz_nms_pick pk{state, -1, INT_MAX, false};
        const int *li = nbr + (long long)i * AKZ_NMS_NB;
        for (int k = 0; k < cnt && pk(li[k]); k++) {
        }
        d = pk.wait ? 0 : (pk.best < 0 ? 1 : 2);
        target = pk.best;
      } else {
        d = akz_nms_decide(c, i, &target);
      }
      dec[i] = (signed char)d;
      if (d == 2) atomicMin(&minc[target], i);
    }
    if (!__syncthreads_or(any)) break;
    for (int i = tid; i < n; i += AKZ_NMS_THREADS)
      if (state[i] == -1 && dec[i] == 1) state[i] = i;
    __syncthreads();
    for (int s = tid; s < n; s += AKZ_NMS_THREADS) {
      const int ch = minc[s];
      if (ch != INT_MAX) {
        minc[s] = INT_MAX;
        if (R[ch].response > R[s].response) {
          state[ch] = s;
          state[s] = -2;
        } else {
          state[ch] = -2;
        }
      }
    }
    __syncthreads();
    if (++rounds > p.max_rounds) {
      if (tid == 0) stats->status = 5; /* AKZ_ERR_TIMEOUT */
      break;
    }
  }
  /* emission in chunks of 2048 slots, each chunk's slot values ascending */
  akz_kp *kp = p.kp + I.kp_base;
  int out = 0;
  for (int cs = 0; cs < n; cs += 2048) {
    for (int k = tid; k < 2048; k += AKZ_NMS_THREADS) {
      const int s = cs + k;
      int v = INT_MAX;
      if (s < n) {
        const int st = state[s];
        if (st >= 0 && R[st].size >= 0.0f) v = st;
      }
      sv[k] = v;
    }
    __syncthreads();
    akz_bitonic2048(sv);
    const int c0 = __syncthreads_count(sv[tid] != INT_MAX);
    const int c1 = __syncthreads_count(sv[tid + 1024] != INT_MAX);
    for (int k = tid; k < c0 + c1; k += AKZ_NMS_THREADS) {
      const akz_raw e = R[sv[k]];
      const float octsub = fabsf(e.octsub);
      const int octave = (int)octsub;
      const float subp = (float)(e.octsub < 0 ? -1 : 1) * (octsub - (float)octave);
      const float ratio = (float)(1 << octave);
      const int r0 = 1 << e.octave;
      const float px = (float)(r0 * e.x), py = (float)(r0 * e.y);
      akz_kp o;
      o.y = ratio * ((float)(int)(0.5f + py / ratio) + e.dst1);
      o.x = ratio * ((float)(int)(0.5f + px / ratio) + subp);
      o.class_id = e.level;
      o.octave = octave;
      o.response = e.response;
      o.size = e.size;
      o.angle = 0.0f;
      kp[out + k] = o;
    }
    out += c0 + c1;
    __syncthreads();
  }
  if (tid == 0) {
    stats->nkp = out;
    stats->nms_rounds = rounds;
  }
}

/* ------------------------------------------------------------------------ */

cudaError_t akz_launch_detect(const akz_detect_params &p, int ntiles, int max_step, cudaStream_t s)
{
  if (ntiles <= 0) return cudaSuccess;
  /* Lsmooth region + Lx, Ly regions; the determinant plane reuses the
   * Lsmooth region.  General path at AKZ_DETECT_TW, akz_detect_tile at its
   * narrower per-step width. */
  size_t words = 0;
  for (int st = 1; st <= max_step; st++) {
    const size_t tw = (size_t)akz_detect_tile_width(st);
    words = std::max(words, (tw + 4 * st + 2) * (AKZ_DETECT_TH + 4 * st + 2) + 2 * (tw + 2 * st + 2) * (AKZ_DETECT_TH + 2 * st + 2));
  }
  const size_t smem = words * sizeof(float);
  cudaError_t e = cudaFuncSetAttribute(k_detect, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_detect<<<ntiles, 256, smem, s>>>(p, max_step);
  return cudaGetLastError();
}

cudaError_t akz_launch_rowscan(const akz_tables &t, const int *rowcnt, int *rowscan, cudaStream_t s)
{
  k_rowscan<<<t.nimg, 1024, 0, s>>>(t, rowcnt, rowscan);
  return cudaGetLastError();
}

cudaError_t akz_launch_extract(const akz_extract_params &p, int nrows, cudaStream_t s)
{
  if (nrows <= 0) return cudaSuccess;
  const int warps_per_block = 8;
  k_extract<<<(nrows + warps_per_block - 1) / warps_per_block, 32 * warps_per_block, 0, s>>>(p, nrows);
  return cudaGetLastError();
}

cudaError_t akz_launch_nms(const akz_nms_params &p, cudaStream_t s)
{
  k_nms<<<p.t.nimg, AKZ_NMS_THREADS, 0, s>>>(p);
  return cudaGetLastError();
}
