/*
 * akz_detect.cu - Hessian detector, extrema, ordering and suppression.
 *
 *   k_detect_strip  one launch over every (image, level) with derivative
 *              step 2..4 (all levels of the default options): each CTA
 *              streams down a column strip, Lsmooth rows -> scaled Scharr
 *              derivatives Lx, Ly with step sigma_size and reflect-101
 *              border (cuda_akaze.cu:651-671, written to HBM for orientation
 *              and M-LDB) -> Hessian determinant (:673-701) -> strict 3x3
 *              maxima above the threshold inside the border (:727-743),
 *              recorded as one bit per pixel plus a per-row count.
 *   k_detect   the same per 64 x 32 tile for any other step.
 *   k_rowscan  exclusive scan of the row counts of each image: the raw
 *              extrema come out in (level, y, x) order, which is the order
 *              the reference's per-level bitonic sort gives (:884-939),
 *              with no per-level cap.
 *   k_extract  one warp per 4 rows: the raw extrema's positions in (level, y, x)
 *              order at their scanned indices.
 *   k_extract_fit  one thread per raw extremum of the batch: subpixel fit and
 *              record (:744-769), the determinant recomputed from Lx, Ly at
 *              the 3x3 neighbourhood.
 *   k_nms      one cluster of 8 CTAs per image: the reference's round-based suppression
 *              (:1005-1224) with an exact per-slot minimum (atomicMin), then
 *              the 2048-slot chunked emission and subpixel restore
 *              (:1227-1316).
 */
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>

#include "../../include/akaze_gb300.h"
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

/* ------------------------------------------------------------------------ */
/* Streaming detector for derivative steps 2..4 (every level of the default
 * options).
 *
 * A CTA owns a strip of TW output columns and AKZ_STRIP_CH rows and walks
 * down it in blocks of BH rows (8; 6 for step 3):
 *   Lsmooth rows  -> ring of 32 rows (cp.async, issued one block ahead)
 *   Lx, Ly rows   -> ring of 16 rows, and to HBM for the strip's own pixels
 *   determinant   -> ring of 16 rows
 *   3x3 maxima above the threshold inside the border range.
 * Lx, Ly and the determinant are formed for row pairs (r, r + ST), which
 * share their two middle tap rows; a warp takes one pair on half of the
 * columns.  Block k + 1's Lx, Ly rows are formed in the same phase as block
 * k's maxima, so a block costs two barriers.
 * Column grids (image x of column 0):
 *   D (Lx, Ly)     tx0 - A,        128 columns = 64 aligned pairs, A = ST+1 rounded up to even
 *   S (Lsmooth)    tx0 - A - ST,   128 + 2 ST columns; D column d has its taps at S d, d+ST, d+2ST
 *   E (det)        tx0 + EO,       2 NEP columns, EO = -1 for odd ST, -2 otherwise; E column e
 *                                  has its centre at D column e + EO + A, an offset of ST's parity,
 *                                  so its outer taps (+-ST) are aligned pairs
 * The strip's vertical halo is paid once per AKZ_STRIP_CH rows instead of
 * once per tile.  Lsmooth rows and columns outside the image are read at
 * their reflect-101 index (clamped into the image where the reflection
 * itself would leave it), so Lx and Ly are exact at every pixel inside the
 * image (cuda_akaze.cu:651-671).  The determinant is exact wherever the
 * maxima test reads it: the border range of a level with step ST starts at
 * x >= 10 sqrt(2) ST (cuda_akaze.cu:734-740), and the determinant at
 * distance <= 1 from it reads Lx, Ly inside the image only, so no mirrored
 * Lx, Ly value is ever needed.  Same expressions, same order as the
 * reference's kernels (cuda_akaze.cu:651-701, :727-743). */
template <int ST>
struct akz_strip_geo {
  static constexpr int A = (ST + 2) & ~1;
  static constexpr int TW = (127 - A - ST) & ~1;
  static constexpr int SW = 128 + 2 * ST;
  /* Lsmooth ring rows: column SO + c holds x = tx0 - A - ST + c.  For even
   * steps the ring row starts 2 columns earlier, on a 16-byte boundary of the
   * image row (tx0 is a multiple of 4), so interior strips load it in 16-byte
   * chunks; SWR is the ring row stride. */
  static constexpr int SO = (ST & 1) ? 0 : 2;
  static constexpr int SWR = (ST & 1) ? SW : ((SW + SO + 3) & ~3);
  static constexpr int EO = (ST & 1) ? -1 : -2;
  static constexpr int NEP = (128 - ST - EO - A) / 2; /* E pairs: right tap pair of the last one ends at D 127 */
  static_assert(TW - EO + 1 <= 2 * NEP, "E covers tx0 - 1 .. tx0 + TW");
  static_assert(EO + A - ST >= 0 && 2 * (NEP - 1) + EO + A + ST + 1 <= 127, "E taps inside the D ring row");
  static_assert(A >= ST + 1 && TW + A + ST <= 127 && A % 2 == 0 && TW % 2 == 0, "D covers tx0 - ST - 1 .. tx0 + TW + ST");
  static_assert(2 * ST < 9, "ring depths (S 32, D 16, E 16 rows) hold every live row");
};

static inline __host__ __device__ int akz_strip_tile_width_rt(int st)
{
  return st == 2 ? akz_strip_geo<2>::TW : st == 3 ? akz_strip_geo<3>::TW : st == 4 ? akz_strip_geo<4>::TW : 0;
}
int akz_strip_tile_width(int st) { return akz_strip_tile_width_rt(st); }

#define AKZ_STRIP_NS 32 /* Lsmooth ring rows */
#define AKZ_STRIP_ND 16 /* Lx, Ly ring rows */
#define AKZ_STRIP_NE 16 /* determinant ring rows */
#define AKZ_STRIP_EW 128

__device__ __forceinline__ void akz_cp_async16(float *dst, const float *src)
{
  const unsigned int d = (unsigned int)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void akz_cp_async4(float *dst, const float *src)
{
  const unsigned int d = (unsigned int)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void akz_cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void akz_cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

/* reflect-101 into [0, n), clamped where the reflection would leave it */
__device__ __forceinline__ int akz_refl_clamp(int i, int n)
{
  if (i < 0) i = -i;
  if (i >= n) i = 2 * n - 2 - i;
  return akz_clampi(i, 0, n - 1);
}

template <int ST, bool FUSED>
__device__ __forceinline__ void akz_detect_strip(const akz_detect_params &p, const akz_level_desc &L, float *sm, int tx0,
                                                 int ty0)
{
  using G = akz_strip_geo<ST>;
  constexpr int A = G::A, TW = G::TW, SO = G::SO, SWR = G::SWR, EO = G::EO, NEP = G::NEP;
  constexpr int NS = AKZ_STRIP_NS, ND = AKZ_STRIP_ND, NE = AKZ_STRIP_NE, EW = AKZ_STRIP_EW;
  constexpr int SJ = (SWR + 31) / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int W = L.width, H = L.height;
  constexpr int BH = ST == 3 ? 6 : 8; /* rows per block: pairs (o, o + ST) tile it */
  static_assert(BH % (2 * ST) == 0, "row pairs tile the block");
  const int ch = min(AKZ_STRIP_CH, H - ty0); /* rows of this CTA */
  const int iters = (ch + BH - 1) / BH;
  float *sS = sm, *sX = sS + NS * SWR, *sY = sX + ND * 128, *sE = sY + ND * 128;
  const float fac1 = p.fac1, fac2 = p.fac2;
  const float *ls = p.t.planes + L.ls;
  float *lxyp = p.t.planes + L.lx; /* interleaved (Lx, Ly), row pitch 2 * pitch */
  const long long pitch = L.pitch;

  const int xs0 = tx0 - A - ST - SO; /* image column of ring column 0 */
  int xs[SJ]; /* source column of this lane's ring columns lane + 32 j */
#pragma unroll
  for (int j = 0; j < SJ; j++) xs[j] = akz_refl_clamp(xs0 + lane + 32 * j, W);
  /* (CTA-uniform) the ring row lies inside the image row: 16-byte copies */
  const bool vec = !(ST & 1) && xs0 >= 0 && xs0 + SWR <= W;

  auto load_s = [&](int r) { /* S row r into its ring slot */
    const float *src = ls + (long long)akz_refl_clamp(r, H) * pitch;
    float *dst = sS + (r & (NS - 1)) * SWR;
    if (vec) {
#pragma unroll
      for (int j = 0; j < (SWR / 4 + 31) / 32; j++) {
        const int q = lane + 32 * j;
        if (q < SWR / 4) akz_cp_async16(dst + 4 * q, src + xs0 + 4 * q);
      }
    } else {
#pragma unroll
      for (int j = 0; j < SJ; j++) {
        const int c = lane + 32 * j;
        if (c < SWR) akz_cp_async4(dst + c, src + xs[j]);
      }
    }
  };
  auto comp_d = [&](int r) { /* Lx, Ly row r; HBM for the strip's own pixels */
    const float *su = sS + ((r - ST) & (NS - 1)) * SWR + SO, *sc = sS + (r & (NS - 1)) * SWR + SO,
                *sd = sS + ((r + ST) & (NS - 1)) * SWR + SO;
    float *ox = sX + (r & (ND - 1)) * 128, *oy = sY + (r & (ND - 1)) * 128;
    const bool wrow = r >= ty0 && r < ty0 + ch;
#pragma unroll
    for (int k = 0; k < 2; k++) {
      const int d = 2 * (lane + 32 * k);
      const float2 ul = ld2(su + d), ur = ld2(su + d + 2 * ST), ll = ld2(sd + d), lr = ld2(sd + d + 2 * ST);
      const float2 cl = ld2(sc + d), cr = ld2(sc + d + 2 * ST);
      const float2 uc = (ST & 1) ? make_float2(su[d + ST], su[d + ST + 1]) : ld2(su + d + ST);
      const float2 lc = (ST & 1) ? make_float2(sd[d + ST], sd[d + ST + 1]) : ld2(sd + d + ST);
      const float2 ax = f2sub(f2sub(f2add(ur, lr), ul), ll), bx = f2sub(cr, cl);
      const float2 ay = f2sub(f2sub(f2add(lr, ll), ur), ul), by = f2sub(lc, uc);
      const float2 a = akz_lin2<FUSED>(fac1, ax, fac2, bx);
      const float2 b = akz_lin2<FUSED>(fac1, ay, fac2, by);
      st2(ox + d, a);
      st2(oy + d, b);
      const int x = tx0 - A + d; /* even */
      if (wrow && d >= A && d < A + TW && x < W) {
        float *o = lxyp + (long long)r * (2 * pitch) + 2 * x; /* x even: 16-byte aligned */
        if (x + 1 < W)
          *reinterpret_cast<float4 *>(o) = make_float4(a.x, b.x, a.y, b.y);
        else
          st2(o, make_float2(a.x, b.x));
      }
    }
  };
  auto comp_e = [&](int r) { /* determinant row r */
    const float *xu = sX + ((r - ST) & (ND - 1)) * 128, *xc = sX + (r & (ND - 1)) * 128,
                *xd = sX + ((r + ST) & (ND - 1)) * 128;
    const float *yu = sY + ((r - ST) & (ND - 1)) * 128, *yd = sY + ((r + ST) & (ND - 1)) * 128;
    float *o = sE + (r & (NE - 1)) * EW;
#pragma unroll
    for (int k = 0; k < 2; k++) {
      const int q = lane + 32 * k;
      if (q >= NEP) continue;
      const int e = 2 * q, d = e + EO + A; /* centre D column */
      const float2 ul = ld2(xu + d - ST), ur = ld2(xu + d + ST), ll = ld2(xd + d - ST), lr = ld2(xd + d + ST);
      const float2 cl = ld2(xc + d - ST), cr = ld2(xc + d + ST);
      const float2 xuc = (ST & 1) ? make_float2(xu[d], xu[d + 1]) : ld2(xu + d);
      const float2 xdc = (ST & 1) ? make_float2(xd[d], xd[d + 1]) : ld2(xd + d);
      const float2 ax = f2sub(f2sub(f2add(ur, lr), ul), ll), bx = f2sub(cr, cl);
      const float2 ay = f2sub(f2sub(f2add(lr, ll), ur), ul), by = f2sub(xdc, xuc);
      const float2 lxx = akz_lin2<FUSED>(fac1, ax, fac2, bx);
      const float2 lyx = akz_lin2<FUSED>(fac1, ay, fac2, by);
      const float2 vul = ld2(yu + d - ST), vur = ld2(yu + d + ST), vll = ld2(yd + d - ST), vlr = ld2(yd + d + ST);
      const float2 yuc = (ST & 1) ? make_float2(yu[d], yu[d + 1]) : ld2(yu + d);
      const float2 ydc = (ST & 1) ? make_float2(yd[d], yd[d + 1]) : ld2(yd + d);
      const float2 cy = f2sub(f2sub(f2add(vlr, vll), vur), vul), dy = f2sub(ydc, yuc);
      const float2 lyy = akz_lin2<FUSED>(fac1, cy, fac2, dy);
      st2(o + e, akz_det2<FUSED>(lxx, lyy, lyx));
    }
  };
  /* a centre tap of a ring row: a pair, or two floats for odd ST */
  auto tap = [&](const float *row, int c) -> float2 { return (ST & 1) ? make_float2(row[c], row[c + 1]) : ld2(row + c); };
  /* Lx, Ly rows rA and rA + ST for column pair d: the two share their
   * middle Lsmooth rows, 12 pair loads instead of 16 */
  auto comp_d2 = [&](int rA, int d) {
    const float *s0 = sS + ((rA - ST) & (NS - 1)) * SWR + SO, *s1 = sS + (rA & (NS - 1)) * SWR + SO,
                *s2 = sS + ((rA + ST) & (NS - 1)) * SWR + SO, *s3 = sS + ((rA + 2 * ST) & (NS - 1)) * SWR + SO;
    const float2 L0 = ld2(s0 + d), C0 = tap(s0, d + ST), R0 = ld2(s0 + d + 2 * ST);
    const float2 L1 = ld2(s1 + d), C1 = tap(s1, d + ST), R1 = ld2(s1 + d + 2 * ST);
    const float2 L2 = ld2(s2 + d), C2 = tap(s2, d + ST), R2 = ld2(s2 + d + 2 * ST);
    const float2 L3 = ld2(s3 + d), C3 = tap(s3, d + ST), R3 = ld2(s3 + d + 2 * ST);
    const int x = tx0 - A + d; /* even */
    const bool wcol = d >= A && d < A + TW && x < W;
#pragma unroll
    for (int t = 0; t < 2; t++) { /* row rA (u, c, d = rows 0, 1, 2), row rA + ST (rows 1, 2, 3) */
      const float2 ul = t ? L1 : L0, uc = t ? C1 : C0, ur = t ? R1 : R0;
      const float2 cl = t ? L2 : L1, cr = t ? R2 : R1;
      const float2 ll = t ? L3 : L2, lc = t ? C3 : C2, lr = t ? R3 : R2;
      const float2 ax = f2sub(f2sub(f2add(ur, lr), ul), ll), bx = f2sub(cr, cl);
      const float2 ay = f2sub(f2sub(f2add(lr, ll), ur), ul), by = f2sub(lc, uc);
      const float2 a = akz_lin2<FUSED>(fac1, ax, fac2, bx);
      const float2 b = akz_lin2<FUSED>(fac1, ay, fac2, by);
      const int r = rA + t * ST;
      st2(sX + (r & (ND - 1)) * 128 + d, a);
      st2(sY + (r & (ND - 1)) * 128 + d, b);
      if (wcol && r >= ty0 && r < ty0 + ch) {
        float *o = lxyp + (long long)r * (2 * pitch) + 2 * x; /* x even: 16-byte aligned */
        if (x + 1 < W)
          *reinterpret_cast<float4 *>(o) = make_float4(a.x, b.x, a.y, b.y);
        else
          st2(o, make_float2(a.x, b.x));
      }
    }
  };
  /* determinant rows rA and rA + ST for E pair q: they share two Lx rows */
  auto comp_e2 = [&](int rA, int q) {
    if (q >= NEP) return;
    const int e = 2 * q, d = e + EO + A; /* centre D column */
    const float *x0 = sX + ((rA - ST) & (ND - 1)) * 128, *x1 = sX + (rA & (ND - 1)) * 128,
                *x2 = sX + ((rA + ST) & (ND - 1)) * 128, *x3 = sX + ((rA + 2 * ST) & (ND - 1)) * 128;
    const float *y0 = sY + ((rA - ST) & (ND - 1)) * 128, *y1 = sY + (rA & (ND - 1)) * 128,
                *y2 = sY + ((rA + ST) & (ND - 1)) * 128, *y3 = sY + ((rA + 2 * ST) & (ND - 1)) * 128;
    const float2 XL0 = ld2(x0 + d - ST), XC0 = tap(x0, d), XR0 = ld2(x0 + d + ST);
    const float2 XL1 = ld2(x1 + d - ST), XC1 = tap(x1, d), XR1 = ld2(x1 + d + ST);
    const float2 XL2 = ld2(x2 + d - ST), XC2 = tap(x2, d), XR2 = ld2(x2 + d + ST);
    const float2 XL3 = ld2(x3 + d - ST), XC3 = tap(x3, d), XR3 = ld2(x3 + d + ST);
    const float2 YL0 = ld2(y0 + d - ST), YC0 = tap(y0, d), YR0 = ld2(y0 + d + ST);
    const float2 YL1 = ld2(y1 + d - ST), YC1 = tap(y1, d), YR1 = ld2(y1 + d + ST);
    const float2 YL2 = ld2(y2 + d - ST), YC2 = tap(y2, d), YR2 = ld2(y2 + d + ST);
    const float2 YL3 = ld2(y3 + d - ST), YC3 = tap(y3, d), YR3 = ld2(y3 + d + ST);
#pragma unroll
    for (int t = 0; t < 2; t++) {
      const float2 ul = t ? XL1 : XL0, ur = t ? XR1 : XR0, ll = t ? XL3 : XL2, lr = t ? XR3 : XR2;
      const float2 cl = t ? XL2 : XL1, cr = t ? XR2 : XR1, xuc = t ? XC1 : XC0, xdc = t ? XC3 : XC2;
      const float2 vul = t ? YL1 : YL0, vur = t ? YR1 : YR0, vll = t ? YL3 : YL2, vlr = t ? YR3 : YR2;
      const float2 yuc = t ? YC1 : YC0, ydc = t ? YC3 : YC2;
      const float2 ax = f2sub(f2sub(f2add(ur, lr), ul), ll), bx = f2sub(cr, cl);
      const float2 ay = f2sub(f2sub(f2add(lr, ll), ur), ul), by = f2sub(xdc, xuc);
      const float2 lxx = akz_lin2<FUSED>(fac1, ax, fac2, bx);
      const float2 lyx = akz_lin2<FUSED>(fac1, ay, fac2, by);
      const float2 cy = f2sub(f2sub(f2add(vlr, vll), vur), vul), dy = f2sub(ydc, yuc);
      const float2 lyy = akz_lin2<FUSED>(fac1, cy, fac2, dy);
      st2(sE + ((rA + t * ST) & (NE - 1)) * EW + e,
          akz_det2<FUSED>(lxx, lyy, lyx));
    }
  };
  const int xlo = max(akz_border_lo(L.border), tx0), xhi = min(akz_border_hi(L.border, W), tx0 + TW - 1);
  const int ylo = max(akz_border_lo(L.border), ty0), yhi = min(akz_border_hi(L.border, H), ty0 + ch - 1);
  auto maxima = [&](int y) {
    if (p.store_det && y >= ty0 && y < ty0 + ch) { /* the strip's own determinants, for the 3 x 3 x 3 rule */
      const float *ec = sE + (y & (NE - 1)) * EW;
      float *o = p.t.planes + L.ldet + (long long)y * pitch;
#pragma unroll
      for (int j = 0; j < (TW + 31) / 32; j++) {
        const int x = tx0 + lane + 32 * j;
        if (lane + 32 * j < TW && x < W) o[x] = ec[x - tx0 - EO];
      }
    }
    if (y < ylo || y > yhi) return;
    const float *eu = sE + ((y - 1) & (NE - 1)) * EW, *ec = sE + (y & (NE - 1)) * EW, *ed = sE + ((y + 1) & (NE - 1)) * EW;
#pragma unroll
    for (int j = 0; j < (TW + 31) / 32; j++) {
      const int x = tx0 + lane + 32 * j;
      if (x < xlo || x > xhi) continue;
      const int e = x - tx0 - EO;
      const float v = ec[e];
      if (v > p.thr) {
        if (v > eu[e - 1] && v > ed[e + 1] && v > ed[e - 1] && v > eu[e + 1] && v > ec[e - 1] && v > ec[e + 1] &&
            v > ed[e] && v > eu[e]) {
          atomicOr(&p.bitmap[L.bitmap + (long long)y * L.bitmap_pitch + (x >> 5)], 1u << (x & 31));
          atomicAdd(&p.rowcnt[L.rows + y], 1);
        }
      }
    }
  };

  /* pre-roll: S rows ty0-1-2ST .. ty0+2ST, D rows ty0-1-ST .. ty0+ST,
   * E rows ty0-1, ty0; then block 0's Lx, Ly and determinant rows.
   * Blocks of BH rows; warp w < BH takes row pair (o, o + ST) of a block,
   * o = (q / ST) 2 ST + q % ST with q = w / 2, and column half w % 2 */
  const int q = warp >> 1, half = warp & 1, o = (q / ST) * 2 * ST + q % ST;
  for (int r = ty0 - 1 - 2 * ST + warp; r <= ty0 + 2 * ST; r += 8) load_s(r);
  akz_cp_async_commit();
  akz_cp_async_wait_all();
  __syncthreads();
  if (warp < BH) load_s(ty0 + 2 * ST + 1 + warp);
  akz_cp_async_commit();
  for (int r = ty0 - 1 - ST + warp; r <= ty0 + ST; r += 8) comp_d(r);
  __syncthreads();
  if (warp < 2) comp_e(ty0 - 1 + warp);
  akz_cp_async_wait_all();
  __syncthreads(); /* block 0's S rows landed */
  if (iters > 1 && warp < BH) load_s(ty0 + 2 * ST + BH + 1 + warp);
  akz_cp_async_commit();
  if (warp < BH) comp_d2(ty0 + ST + 1 + o, 2 * (32 * half + lane));
  __syncthreads();
  if (warp < BH) comp_e2(ty0 + 1 + o, 32 * half + lane);
  /* iteration k: block k + 1's Lx, Ly next to block k's maxima, then block
   * k + 1's determinant; block k + 2's S rows in flight */
  for (int k = 0; k < iters; k++) {
    const int r = ty0 + BH * k;
    akz_cp_async_wait_all();
    __syncthreads(); /* S rows up to r+2BH+2ST landed; E rows up to r+BH visible */
    if (k + 2 < iters && warp < BH) load_s(r + 2 * ST + 2 * BH + 1 + warp);
    akz_cp_async_commit();
    if (k + 1 < iters && warp < BH) comp_d2(r + BH + ST + 1 + o, 2 * (32 * half + lane));
    if (warp < BH) maxima(r + warp);
    __syncthreads();
    if (k + 1 < iters && warp < BH) comp_e2(r + BH + 1 + o, 32 * half + lane);
  }
  akz_cp_async_wait_all();
}

template <bool FUSED>
__global__ void __launch_bounds__(256, 4) k_detect_strip(akz_detect_params p)
{
  extern __shared__ float sm[];
  const int si = akz_find_seg_warp(p.segs, p.nsegs, blockIdx.x);
  const akz_tile_seg sg = p.segs[si];
  const akz_level_desc L = p.t.lv[sg.level_desc];
  const int st = L.deriv_step;
  const int lt = blockIdx.x - sg.tile_begin;
  const int tx0 = (lt % sg.tiles_x) * akz_strip_tile_width_rt(st), ty0 = (lt / sg.tiles_x) * AKZ_STRIP_CH;
  if (st == 2)
    akz_detect_strip<2, FUSED>(p, L, sm, tx0, ty0);
  else if (st == 3)
    akz_detect_strip<3, FUSED>(p, L, sm, tx0, ty0);
  else if (st == 4)
    akz_detect_strip<4, FUSED>(p, L, sm, tx0, ty0);
}

size_t akz_detect_strip_smem()
{
  static_assert(akz_strip_geo<4>::SWR >= akz_strip_geo<2>::SWR && akz_strip_geo<4>::SWR >= akz_strip_geo<3>::SWR,
                "the step-4 ring row is the widest");
  return (size_t)(AKZ_STRIP_NS * akz_strip_geo<4>::SWR + 2 * AKZ_STRIP_ND * 128 + AKZ_STRIP_NE * AKZ_STRIP_EW) *
         sizeof(float);
}

cudaError_t akz_launch_detect_strip(const akz_detect_params &p, int ntiles, cudaStream_t s)
{
  if (ntiles <= 0) return cudaSuccess;
  const size_t smem = akz_detect_strip_smem();
  cudaError_t e;
  if (p.fused) {
    e = cudaFuncSetAttribute(k_detect_strip<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_detect_strip<true><<<ntiles, 256, smem, s>>>(p);
  } else {
    e = cudaFuncSetAttribute(k_detect_strip<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_detect_strip<false><<<ntiles, 256, smem, s>>>(p);
  }
  return cudaGetLastError();
}

__global__ void __launch_bounds__(256) k_detect(akz_detect_params p, int max_step)
{
  constexpr int TW = AKZ_DETECT_TW, TH = AKZ_DETECT_TH;
  extern __shared__ float sm[];
  const int tid = threadIdx.x;
  const int si = akz_find_seg_warp(p.segs, p.nsegs, blockIdx.x);
  const akz_tile_seg sg = p.segs[si];
  const akz_level_desc L = p.t.lv[sg.level_desc];
  const int W = L.width, H = L.height, st = L.deriv_step;
  const int lt = blockIdx.x - sg.tile_begin;
  const int tx0 = (lt % sg.tiles_x) * TW, ty0 = (lt / sg.tiles_x) * TH;
  const int tx1 = min(tx0 + TW, W), ty1 = min(ty0 + TH, H);
  const int sx0 = max(tx0 - 2 * st - 1, 0), sx1 = min(tx1 + 2 * st + 1, W);
  const int sy0 = max(ty0 - 2 * st - 1, 0), sy1 = min(ty1 + 2 * st + 1, H);
  const int dx0 = max(tx0 - st - 1, 0), dx1 = min(tx1 + st + 1, W);
  const int dy0 = max(ty0 - st - 1, 0), dy1 = min(ty1 + st + 1, H);
  const int ex0 = max(tx0 - 1, 0), ex1 = min(tx1 + 1, W), ey0 = max(ty0 - 1, 0), ey1 = min(ty1 + 1, H);
  const int sw = sx1 - sx0, dw = dx1 - dx0, ew = ex1 - ex0;
  const int SM = (TW + 4 * max_step + 2) * (TH + 4 * max_step + 2);
  const int DM = (TW + 2 * max_step + 2) * (TH + 2 * max_step + 2);
  float *sS = sm, *sX = sm + SM, *sY = sX + DM, *sD = sm; /* determinant plane over the dead Lsmooth region */

  const int lane = tid & 31, warp = tid >> 5;
  const float *ls = p.t.planes + L.ls;
  for (int y = sy0 + warp; y < sy1; y += 8)
    for (int x = sx0 + lane; x < sx1; x += 32) sS[(y - sy0) * sw + (x - sx0)] = __ldg(ls + (long long)y * L.pitch + x);
  __syncthreads();
  float *lxyp = p.t.planes + L.lx; /* interleaved (Lx, Ly), row pitch 2 * pitch */
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
      if (yt && x >= tx0 && x < tx1) st2(lxyp + (long long)y * (2 * L.pitch) + 2 * x, make_float2(a, b));
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
  if (p.store_det) /* the tile's determinants, for the 3 x 3 x 3 rule */
    for (int y = ty0 + warp; y < ty1; y += 8)
      for (int x = tx0 + lane; x < tx1; x += 32)
        p.t.planes[L.ldet + (long long)y * L.pitch + x] = sD[(y - ey0) * ew + (x - ex0)];
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
/* The 3 x 3 x 3 extrema rule (akz_options.extrema_3d): a candidate of the
 * 3 x 3 rule stays only if it also exceeds the 3 x 3 blocks of the
 * determinant at its position in the previous and the next level of its
 * octave (where those exist); AKAZE.cpp:340-367 hands FindExtrema those
 * planes, cuda_akaze.cu:727-774 does not read them.  One warp per bitmap
 * row (grid: x = level descriptor, y = groups of 8 rows), one lane per
 * 32-bit word; the warp's removals leave the row count in one add.  The
 * candidates lie inside the level's border range (>= 10 sqrt(2) pixels
 * from every edge), so their neighbours' blocks are inside the image. */
__global__ void __launch_bounds__(256) k_extrema3d(akz_detect_params p, int nlev_total)
{
  const int ld = blockIdx.x;
  const akz_level_desc L = p.t.lv[ld];
  const int lane = threadIdx.x & 31, y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (y >= L.height) return;
  const float *adj[2] = {nullptr, nullptr};
  if (ld > 0) {
    const akz_level_desc P = p.t.lv[ld - 1];
    if (P.image == L.image && P.octave == L.octave) adj[0] = p.t.planes + P.ldet;
  }
  if (ld + 1 < nlev_total) {
    const akz_level_desc N = p.t.lv[ld + 1];
    if (N.image == L.image && N.octave == L.octave) adj[1] = p.t.planes + N.ldet;
  }
  const long long pitch = L.pitch;
  const float *det = p.t.planes + L.ldet;
  uint32_t *row = p.bitmap + L.bitmap + (long long)y * L.bitmap_pitch;
  int removed = 0;
  for (int wd = lane; wd < L.bitmap_pitch; wd += 32) {
    uint32_t bits = row[wd], keep = bits;
    while (bits) {
      const int b = __ffs(bits) - 1;
      bits &= bits - 1;
      const int x = 32 * wd + b;
      const float v = det[(long long)y * pitch + x];
      bool ok = true;
#pragma unroll
      for (int a = 0; a < 2; a++) {
        if (!adj[a]) continue;
#pragma unroll
        for (int dy = -1; dy <= 1; dy++)
#pragma unroll
          for (int dx = -1; dx <= 1; dx++) ok = ok && v > adj[a][(long long)(y + dy) * pitch + x + dx];
      }
      if (!ok) {
        keep &= ~(1u << b);
        removed++;
      }
    }
    if (keep != row[wd]) row[wd] = keep;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) removed += __shfl_down_sync(0xffffffffu, removed, o);
  if (lane == 0 && removed) p.rowcnt[L.rows + y] -= removed;
}

cudaError_t akz_launch_extrema3d(const akz_detect_params &p, int nlevels_total, int max_level_h, cudaStream_t s)
{
  if (nlevels_total <= 0) return cudaSuccess;
  k_extrema3d<<<dim3(nlevels_total, (max_level_h + 7) / 8), 256, 0, s>>>(p, nlevels_total);
  return cudaGetLastError();
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

/* Raw extrema positions in (image, level, row, column) order: a warp takes
 * AKZ_EXTRACT_RPW consecutive rows of the row list (one per level row of
 * every image) and writes each set bit of their bitmap rows at its rank
 * (the row's exclusive scan plus the bits before it).  Every row's
 * descriptors, rank and first two 32-word chunks of bitmap are loaded before
 * the first row is written, so the rows' load chains overlap. */
#define AKZ_EXTRACT_RPW 4
__global__ void __launch_bounds__(256) k_extract(akz_extract_params p, int nrows)
{
  constexpr int R = AKZ_EXTRACT_RPW;
  const int lane = threadIdx.x & 31;
  const int r0 = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * R;
  if (r0 >= nrows) return;
  int si = akz_find_seg_warp(p.segs, p.nsegs, r0);
  int y[R], words[R], rank0[R], level[R], cap[R];
  long long raw_base[R];
  const uint32_t *row[R];
  uint32_t b0[R], b1[R];
#pragma unroll
  for (int k = 0; k < R; k++) {
    const int r = min(r0 + k, nrows - 1); /* rows past the list: a copy of the last, skipped below */
    while (si + 1 < p.nsegs && __ldg(&p.segs[si + 1].tile_begin) <= r) si++;
    const akz_tile_seg sg = p.segs[si];
    const akz_level_desc &L = p.t.lv[sg.level_desc];
    y[k] = r - sg.tile_begin;
    words[k] = L.bitmap_pitch;
    level[k] = L.level;
    const akz_image_desc &I = p.t.im[L.image];
    raw_base[k] = I.raw_base;
    cap[k] = I.raw_cap;
    row[k] = p.bitmap + L.bitmap + (long long)y[k] * words[k];
    rank0[k] = p.rowscan[L.rows + y[k]];
    b0[k] = lane < words[k] ? row[k][lane] : 0u;
    b1[k] = 32 + lane < words[k] ? row[k][32 + lane] : 0u;
  }
#pragma unroll
  for (int k = 0; k < R; k++) {
    if (r0 + k >= nrows) break;
    akz_raw *out = p.raw + raw_base[k];
    int running = 0;
    for (int w0 = 0; w0 < words[k]; w0 += 32) {
      const int w = w0 + lane;
      uint32_t bits = w0 == 0 ? b0[k] : (w0 == 32 ? b1[k] : (w < words[k] ? row[k][w] : 0u));
      const int cnt = __popc(bits);
      int pre = cnt;
      for (int d = 1; d < 32; d <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, pre, d);
        if (lane >= d) pre += t;
      }
      const int total = __shfl_sync(0xffffffffu, pre, 31);
      int j = running + pre - cnt;
      while (bits) {
        const int bt = __ffs(bits) - 1;
        bits &= bits - 1;
        const int idx = rank0[k] + j++;
        if (idx >= cap[k]) continue;
        /* position only; k_extract_fit completes the record */
        out[idx].x = w * 32 + bt;
        out[idx].y = y[k];
        out[idx].level = level[k];
      }
      running += total;
    }
  }
}

/* Subpixel fit of every raw extremum (cuda_akaze.cu:744-769), one thread
 * each over the whole batch: the determinant recomputed from Lx, Ly at the
 * 3x3 neighbourhood, its gradient and Hessian, the offset (dst0, dst1) and
 * the record. */
__global__ void __launch_bounds__(256) k_extract_fit(akz_extract_params p)
{
  __shared__ int sOff[AKZ_FIT_MAXIMG + 1]; /* raw extrema before each image (capped at each image's capacity) */
  const int nimg = p.t.nimg;
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int i = 0; i < nimg; i++) {
      sOff[i] = acc;
      acc += min(p.t.stats[i].nraw, p.t.im[i].raw_cap);
    }
    sOff[nimg] = acc;
  }
  __syncthreads();
  const int total = sOff[nimg];
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
    int lo = 0, hi = nimg - 1; /* last image with sOff <= g */
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (sOff[mid] <= g)
        lo = mid;
      else
        hi = mid - 1;
    }
    const akz_image_desc I = p.t.im[lo];
    akz_raw *rec = p.raw + I.raw_base + (g - sOff[lo]);
    const int x = rec->x, y = rec->y;
    const akz_level_desc L = p.t.lv[I.first_level + rec->level];
    const int W = L.width, H = L.height, st = L.deriv_step;
    const float *lxy = p.t.planes + L.lx;
    const long long pitch2 = 2LL * L.pitch;
    float D[3][3];
#pragma unroll
    for (int j = -1; j <= 1; j++)
#pragma unroll
      for (int i = -1; i <= 1; i++) D[j + 1][i + 1] = akz_det_at2(lxy, pitch2, W, H, st, x + i, y + j, p.fac1, p.fac2);
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
    *rec = e;
  }
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
    const int sj = __ldcg(state + j); /* other CTAs of the cluster write it */
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
  for (int k = 2; k <= 2048; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int t = threadIdx.x; t < 1024; t += blockDim.x) { /* 1024 compare-exchanges per step */
        const int i = ((t & ~(j - 1)) << 1) | (t & (j - 1));
        const int l = i | j;
        const bool up = (i & k) == 0;
        const int a = v[i], b = v[l];
        if ((a > b) == up) {
          v[i] = b;
          v[l] = a;
        }
      }
      __syncthreads();
    }
  }
}

/* Suppression of one image per cluster of AKZ_NMS_CL CTAs (a point per
 * thread of the cluster, strided): the reference's rounds (cuda_akaze.cu:
 * 1005-1224) with a cluster barrier between their phases, so the image with
 * the most raw extrema no longer runs on one SM while the others idle.
 * Points' states live in global memory; they are read through L2
 * (__ldcg) after each barrier's release/acquire, since another SM of the
 * cluster may have written them.  Emission: every chunk of 2048 slots is
 * counted first (any CTA), the counts are prefixed, then each CTA sorts its
 * own chunks and writes them at their offsets (cuda_akaze.cu:1227-1316). */
__global__ void __cluster_dims__(AKZ_NMS_CL, 1, 1) __launch_bounds__(AKZ_NMS_THREADS) k_nms(akz_nms_params p)
{
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  __shared__ int sv[2048];
  __shared__ int sflag[2];
  const int rank = (int)cl.block_rank();
  const int img = blockIdx.x / AKZ_NMS_CL;
  const int tid = threadIdx.x;
  const int gt = rank * AKZ_NMS_THREADS + tid, GT = AKZ_NMS_CL * AKZ_NMS_THREADS;
  const akz_image_desc I = p.t.im[img];
  akz_image_stats *stats = &p.t.stats[img];
  if (__ldcg(&stats->overflow)) { /* the same for every CTA of the cluster */
    if (rank == 0 && tid == 0) stats->nkp = 0;
    return;
  }
  const int n = __ldcg(&stats->nraw);
  const akz_raw *R = p.raw + I.raw_base;
  int *state = p.state + I.raw_base;
  int *minc = p.aux + I.raw_base;
  signed char *dec = p.decision + I.raw_base;
  if (tid < 2) sflag[tid] = 0;
  for (int i = gt; i < n; i += GT) {
    state[i] = -1;
    minc[i] = INT_MAX;
  }
  cl.sync();
  const akz_nms_ctx c{R, state, p.rowscan + I.rows_base, p.t.lv, I.first_level, I.rows_base};
  /* neighbour sets, found once (the rounds then cost O(neighbours) each);
   * a point with more than AKZ_NMS_NB neighbours is decided by scanning;
   * point i is always handled by the same thread */
  int *nbr = p.nbr + (long long)I.raw_base * AKZ_NMS_NB;
  unsigned char *nbc = p.nbc + I.raw_base;
  for (int i = gt; i < n; i += GT) {
    int cnt = 0;
    int *li = nbr + (long long)i * AKZ_NMS_NB;
    const bool all = akz_nms_visit(c, i, [&](int j) {
      if (cnt == AKZ_NMS_NB) return false;
      li[cnt++] = j;
      return true;
    });
    nbc[i] = (unsigned char)(all ? cnt : AKZ_NMS_NB + 1);
  }
  int *flag0 = cl.map_shared_rank(sflag, 0);
  int rounds = 0;
  for (;;) {
    int any = 0;
    for (int i = gt; i < n; i += GT) {
      if (__ldcg(state + i) != -1) continue;
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
    /* cluster-wide "any point unsettled": an OR into rank 0's flag of this
     * round's parity; rank 0 clears the other parity, last read a round ago */
    if (__syncthreads_or(any) && tid == 0) atomicOr(flag0 + (rounds & 1), 1);
    cl.sync();
    const int anyc = *(volatile int *)(flag0 + (rounds & 1));
    if (rank == 0 && tid == 0) sflag[(rounds + 1) & 1] = 0;
    if (!anyc) break;
    for (int i = gt; i < n; i += GT)
      if (__ldcg(state + i) == -1 && dec[i] == 1) state[i] = i;
    cl.sync();
    for (int s2 = gt; s2 < n; s2 += GT) {
      const int ch = __ldcg(minc + s2);
      if (ch != INT_MAX) {
        minc[s2] = INT_MAX;
        if (R[ch].response > R[s2].response) {
          state[ch] = s2;
          state[s2] = -2;
        } else {
          state[ch] = -2;
        }
      }
    }
    cl.sync();
    if (++rounds > p.max_rounds) {
      if (rank == 0 && tid == 0) stats->status = (int)AKZ_ERR_TIMEOUT;
      break;
    }
  }
  /* emission in chunks of 2048 slots, each chunk's slot values ascending:
   * counts of every chunk (into minc[chunk], free again), then offsets */
  const int nchunks = (n + 2047) / 2048;
  __shared__ int scnt;
  for (int ck = rank; ck < nchunks; ck += AKZ_NMS_CL) {
    if (tid == 0) scnt = 0;
    __syncthreads();
    int cnt = 0;
    for (int k = tid; k < 2048; k += AKZ_NMS_THREADS) {
      const int s2 = ck * 2048 + k;
      if (s2 < n) {
        const int st = __ldcg(state + s2);
        cnt += st >= 0 && R[st].size >= 0.0f;
      }
    }
    if (cnt) atomicAdd(&scnt, cnt);
    __syncthreads();
    if (tid == 0) minc[ck] = scnt;
    __syncthreads();
  }
  cl.sync();
  akz_kp *kp = p.kp + I.kp_base;
  int total = 0;
  for (int ck = 0; ck < nchunks; ck++) total += __ldcg(minc + ck);
  for (int ck = rank; ck < nchunks; ck += AKZ_NMS_CL) {
    int out = 0;
    for (int q = 0; q < ck; q++) out += __ldcg(minc + q);
    for (int k = tid; k < 2048; k += AKZ_NMS_THREADS) {
      const int s2 = ck * 2048 + k;
      int v = INT_MAX;
      if (s2 < n) {
        const int st = __ldcg(state + s2);
        if (st >= 0 && R[st].size >= 0.0f) v = st;
      }
      sv[k] = v;
    }
    __syncthreads();
    akz_bitonic2048(sv);
    const int cnt = __ldcg(minc + ck);
    for (int k = tid; k < cnt; k += AKZ_NMS_THREADS) {
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
    __syncthreads();
  }
  if (rank == 0 && tid == 0) {
    stats->nkp = total;
    stats->nms_rounds = rounds;
  }
  cl.sync(); /* no CTA leaves while another may still read rank 0's flags */
}

/* ------------------------------------------------------------------------ */

cudaError_t akz_launch_detect(const akz_detect_params &p, int ntiles, int max_step, cudaStream_t s)
{
  if (ntiles <= 0) return cudaSuccess;
  /* Lsmooth region + Lx, Ly regions; the determinant plane reuses the
   * Lsmooth region */
  const size_t tw = AKZ_DETECT_TW, th = AKZ_DETECT_TH, ms = (size_t)max_step;
  const size_t smem = ((tw + 4 * ms + 2) * (th + 4 * ms + 2) + 2 * (tw + 2 * ms + 2) * (th + 2 * ms + 2)) * sizeof(float);
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
  const int rows_per_block = 8 * AKZ_EXTRACT_RPW; /* 8 warps */
  k_extract<<<(nrows + rows_per_block - 1) / rows_per_block, 256, 0, s>>>(p, nrows);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (p.t.nimg > AKZ_FIT_MAXIMG) return cudaErrorInvalidValue;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  k_extract_fit<<<8 * std::max(nsm, 1), 256, 0, s>>>(p);
  return cudaGetLastError();
}

cudaError_t akz_launch_nms(const akz_nms_params &p, cudaStream_t s)
{
  k_nms<<<p.t.nimg * AKZ_NMS_CL, AKZ_NMS_THREADS, 0, s>>>(p);
  return cudaGetLastError();
}
