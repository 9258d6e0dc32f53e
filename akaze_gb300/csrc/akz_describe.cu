/*
 * akz_describe.cu - orientation and M-LDB, one warp per keypoint.
 *
 * Orientation (cuda_akaze.cu:2114-2167): 109 gradient samples of radius < 6
 * on a grid of spacing round(size/2) >> octave, Gaussian weights sigma 2.5,
 * 42 angular bins, the strongest 7-bin circular window, atan2 in [0, 2 pi).
 * M-LDB (cuda_akaze.cu:1420-1533, :1786-1807, :2034-2111): a 21x21 grid of
 * samples rotated by the orientation at spacing round(size/2 / 2^octave),
 * three channels (L, rotated dx, rotated dy) summed into 2x2, 3x3 and 4x4
 * cells (87 sums) and 486 pairwise comparisons, written as 64-byte rows
 * (bits 486..511 zero) that the matcher reads directly.  The comparisons
 * come from a per-batch table: the full descriptor of 1, 2 or 3 channels
 * (162 bits per channel; the second channel of a 2-channel descriptor is the
 * gradient magnitude) or the random-bit subset of descriptor_size bits
 * (AKAZE.cpp:412-423, :498-603).
 *
 * Sums are formed in a fixed order: sample order for the orientation bins,
 * and for the cells the reference's order (64 strided per-thread partials,
 * pairs t and t + 32, then the shuffle-down tree).  The CPU restatement uses
 * the same orders, so angles and descriptors are reproducible bit for bit.
 *
 * The grid is one wave of resident CTAs (AKZ_DESC_CTAS per SM), each warp
 * looping over keypoints.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "akz_device.cuh"
#include "akz_fmath.h"

#define AKZ_DESC_WARPS 4
#define AKZ_DESC_ITERS 14 /* 14 x 32 = 448 >= 21 x 21 window samples */
#define AKZ_DESC_MAXIMG 1024 /* images whose keypoint offsets a CTA keeps in shared memory */
#ifndef AKZ_DESC_CTAS
#define AKZ_DESC_CTAS 5 /* resident CTAs per SM: at most 96 registers, ~34 KB of shared memory each */
#endif
#define AKZ_CV_PI 3.1415926535897932384626433832795

/* orientation samples in the reference's thread order: tx = 16*(j+6) + (i+6) */
__constant__ signed char c_oi[109], c_oj[109], c_or2[109];
/* the M-LDB window's samples in the order the warp gathers them: 4 x 8
 * blocks of the window, so one gather instruction touches a compact patch
 * of the level (its sectors) rather than one and a half rotated rows; each
 * entry is (row << 8) | column, the stores keep the raster index */
#define AKZ_DESC_MAXWIN 21 /* window of pattern size 10 */
__device__ unsigned short g_smp_order[AKZ_DESC_MAXWIN + 1][32 * AKZ_DESC_ITERS]; /* per window size */

struct akz_warp_smem {
  float s[3][441];
  float v[87];
  union {
    struct {
      float bx[42], by[42];
      float wx[42], wy[42];
    } o;                /* orientation bins */
    float acc[16 * 33]; /* cell partials of one grid, channel and thread parity: [cell][lane] */
  } u;
};

/* One grid (C cells) of the M-LDB cell sums, all three channels, in the
 * reference's order (ExtractDescriptors, cuda_akaze.cu:1456-1523): its 64
 * threads each sum the samples i = t, t + 64, ... of a cell in increasing
 * i; then for every cell, lane j (j < 32) adds the partials of threads j and
 * j + 32 and a __shfl_down tree (offsets 1, 2, 4, 8, 16) sums the 32 lanes.
 * Here lane l holds the samples i = l + 32 m: even m belong to thread l,
 * odd m to thread l + 32, so each lane keeps both partials of every cell
 * (lane-private columns of acc; the sample's column offset is decoded once
 * per grid) and forms its tree leaf.  The leaves of a small grid go through
 * the shuffle tree itself; those of a larger one are transposed through acc
 * (row stride 33: conflict-free both ways) so that lane c sums cell c's 32
 * leaves in the tree's association. */
template <int C, int SHIFT, int MASK, int BASE>
__device__ __forceinline__ void akz_mldb_cells(float *acc, const float (*src)[441], const unsigned short *cells, int lane,
                                               int nsmp, float *vout)
{
  int off[AKZ_DESC_ITERS]; /* acc column offset of each sample of this lane, -1 outside the grid */
#pragma unroll
  for (int m = 0; m < AKZ_DESC_ITERS; m++) {
    const int i = lane + 32 * m;
    const int c = i < nsmp ? (cells[i] >> SHIFT) & MASK : MASK;
    off[m] = c < C ? c * 32 + lane : -1;
  }
#pragma unroll 1
  for (int ch = 0; ch < 3; ch++) {
    const float *sc = src[ch];
    float a[C];
#pragma unroll
    for (int par = 0; par < 2; par++) { /* thread l (even m), then thread l + 32 (odd m) */
#pragma unroll
      for (int r = 0; r < C; r++) acc[r * 32 + lane] = 0.0f;
#pragma unroll
      for (int m = par; m < AKZ_DESC_ITERS; m += 2)
        if (off[m] >= 0) acc[off[m]] += sc[lane + 32 * m];
#pragma unroll
      for (int c = 0; c < C; c++) a[c] = par ? a[c] + acc[c * 32 + lane] : acc[c * 32 + lane];
    }
    if (C <= 4) {
#pragma unroll
      for (int c = 0; c < C; c++) {
        float v = a[c];
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) v += __shfl_down_sync(0xffffffffu, v, d);
        if (lane == 0) vout[3 * (BASE + c) + ch] = v;
      }
    } else {
      __syncwarp();
#pragma unroll
      for (int c = 0; c < C; c++) acc[c * 33 + lane] = a[c];
      __syncwarp();
      if (lane < C) { /* the tree's two halves of 16 leaves, then their sum (its last level) */
        float h[2];
#pragma unroll
        for (int q = 0; q < 2; q++) {
          float t[16];
#pragma unroll
          for (int k = 0; k < 16; k++) t[k] = acc[lane * 33 + 16 * q + k];
#pragma unroll
          for (int d = 1; d < 16; d <<= 1)
#pragma unroll
            for (int j = 0; j < 16; j += 2 * d) t[j] = t[j] + t[j + d];
          h[q] = t[0];
        }
        vout[3 * (BASE + lane) + ch] = h[0] + h[1];
      }
    }
    __syncwarp();
  }
}

__global__ void __launch_bounds__(32 * AKZ_DESC_WARPS, AKZ_DESC_CTAS) k_describe(akz_describe_params p)
{
  __shared__ akz_warp_smem sm_all[AKZ_DESC_WARPS];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  akz_warp_smem &S = sm_all[wib];
  const int nwarps = gridDim.x * AKZ_DESC_WARPS;
  /* keypoint offsets of the images, once per CTA: sOff[i] = sum_{j<i} nkp_j */
  extern __shared__ int sOff[]; /* nimg + 1 entries when nimg <= AKZ_DESC_MAXIMG */
  const bool table = p.t.nimg <= AKZ_DESC_MAXIMG;
  if (table) {
    if (threadIdx.x == 0) {
      int acc = 0;
      for (int b = 0; b < p.t.nimg; b++) {
        sOff[b] = acc;
        acc += p.t.stats[b].nkp;
      }
      sOff[p.t.nimg] = acc;
    }
    __syncthreads();
  }
  /* orientation sample offsets (packed i, j) and Gaussian weights, indexed
   * by sample: lane-consecutive shared loads instead of divergent constant
   * reads */
  __shared__ int sOrIJ[112];
  __shared__ float sOrW[112];
  __shared__ unsigned short sOrd[32 * AKZ_DESC_ITERS];
  for (int t = threadIdx.x; t < 109; t += blockDim.x) {
    sOrIJ[t] = ((int)c_oi[t] & 0xffff) + (int)c_oj[t] * 65536;
    sOrW[t] = p.gw[c_or2[t]];
  }
  {
    const int ps0 = p.pattern_size;
    const int w0 = max(3 * (int)ceilf(2.0f * (float)ps0 / 3.0f), 4 * (int)ceilf(0.5f * (float)ps0));
    const unsigned short *ord = g_smp_order[min(w0, AKZ_DESC_MAXWIN)];
    for (int t = threadIdx.x; t < 32 * AKZ_DESC_ITERS; t += blockDim.x) sOrd[t] = ord[t];
  }
  __syncthreads();
  int total = 0;
  if (table)
    total = sOff[p.t.nimg];
  else
    for (int b = 0; b < p.t.nimg; b++) total += p.t.stats[b].nkp;
  const int ps = p.pattern_size;
  const int size2 = ps, size3 = (int)ceilf(2.0f * (float)ps / 3.0f), size4 = (int)ceilf(0.5f * (float)ps);
  const int win = max(3 * size3, 4 * size4);
  /* each window sample's cell in the 2x2, 3x3 and 4x4 grids (7, 15, 31:
   * outside that grid's range), the rules of cuda_akaze.cu:1470-1497 */
  __shared__ unsigned short sCell[32 * AKZ_DESC_ITERS];
  for (int i = threadIdx.x; i < 32 * AKZ_DESC_ITERS; i += blockDim.x) {
    int c = 0xffff;
    if (i < win * win) {
      const int y = i / win, x = i - y * win, m = max(x, y);
      const int c2 = m < 2 * size2 ? (x < size2 ? 0 : 1) + 2 * (y < size2 ? 0 : 1) : 7;
      const int x3 = x < size3 ? 0 : (x < 2 * size3 ? 1 : 2), y3 = y < size3 ? 0 : (y < 2 * size3 ? 1 : 2);
      const int c3 = m < 3 * size3 ? x3 + 3 * y3 : 15;
      const int x4 = x < 2 * size4 ? (x < size4 ? 0 : 1) : (x < 3 * size4 ? 2 : 3);
      const int y4 = y < 2 * size4 ? (y < size4 ? 0 : 1) : (y < 3 * size4 ? 2 : 3);
      const int c4 = m < 4 * size4 ? x4 + 4 * y4 : 31;
      c = c2 | (c3 << 3) | (c4 << 7);
    }
    sCell[i] = (unsigned short)c;
  }
  __syncthreads();
  for (int g = blockIdx.x * AKZ_DESC_WARPS + wib; g < total; g += nwarps) {
    int img = 0, k = g;
    if (table) {
      int lo = 0, hi = p.t.nimg - 1; /* last image with sOff <= g */
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (sOff[mid] <= g)
          lo = mid;
        else
          hi = mid - 1;
      }
      img = lo;
      k = g - sOff[lo];
    } else {
      while (k >= p.t.stats[img].nkp) {
        k -= p.t.stats[img].nkp;
        img++;
      }
    }
    const akz_image_desc I = p.t.im[img];
    akz_kp *kpp = p.kp + I.kp_base + k;
    const akz_kp kp = *kpp;
    const akz_level_desc L = p.t.lv[I.first_level + kp.class_id];
    const int W = L.width, H = L.height, pitch = L.pitch;
    const float *lxyp = p.t.planes + L.lx, *ltp = p.t.planes + L.lt; /* (Lx, Ly) interleaved, row pitch 2 * pitch */
    float angle = 0.0f;
    if (!p.upright) {
      const int octave = kp.octave;
      const int step = (int)(0.5f * kp.size + 0.5f) >> octave;
      const int x = (int)(kp.x + 0.5f) >> octave;
      const int y = (int)(kp.y + 0.5f) >> octave;
      /* every gather of the 109 samples in flight before the first use */
      float gxv[4], gyv[4];
#pragma unroll
      for (int it = 0; it < 4; it++) {
        const int s = lane + 32 * it;
        if (s < 109) {
          const int ij = sOrIJ[s];
          const int sx = akz_clampi(x + step * (int)(short)(ij & 0xffff), 0, W - 1);
          const int sy = akz_clampi(y + step * (ij >> 16), 0, H - 1);
          const float2 g2 = __ldg(reinterpret_cast<const float2 *>(lxyp + (long long)sy * (2 * pitch) + 2 * sx));
          gxv[it] = g2.x;
          gyv[it] = g2.y;
        }
      }
      /* per bin, a 109-bit mask of its samples (4 words in the third
       * sample channel, free until the M-LDB samples) */
      uint32_t *bm = reinterpret_cast<uint32_t *>(S.s[2]);
      for (int t = lane; t < 42 * 4; t += 32) bm[t] = 0u;
      __syncwarp();
#pragma unroll
      for (int it = 0; it < 4; it++) {
        const int s = lane + 32 * it;
        int bin = 64; /* no sample */
        if (s < 109) {
          const float w = sOrW[s];
          const float dx = w * gxv[it];
          const float dy = w * gyv[it];
          const float a = akz_atan2f(dy, dx);
          /* (int)((double)a * (21 / pi)): the float product is within
           * 2.5e-6 of the double one, so away from integers their
           * truncations agree; near an integer the double product decides */
          const float tf = a * (float)(21 / AKZ_CV_PI);
          const int ib = fabsf(tf - rintf(tf)) > 0x1p-17f ? (int)tf : (int)((double)a * (21 / AKZ_CV_PI));
          bin = ib + 21;
          bin = bin > 41 ? 41 : (bin < 0 ? 0 : bin);
          S.s[0][s] = dx;
          S.s[1][s] = dy;
        }
        const uint32_t grp = __match_any_sync(0xffffffffu, bin);
        if (bin < 42 && (grp & ((1u << lane) - 1u)) == 0u) bm[bin * 4 + it] = grp; /* the group's lowest lane */
      }
      __syncwarp();
      {
        /* bins lane and lane + 32, each summed over its samples in sample order */
        const int b1 = lane + 32;
        float rx0 = 0.0f, ry0 = 0.0f, rx1 = 0.0f, ry1 = 0.0f;
#pragma unroll
        for (int w = 0; w < 4; w++) {
          uint32_t m0 = bm[lane * 4 + w], m1 = b1 < 42 ? bm[b1 * 4 + w] : 0u;
          while (m0) {
            const int s = 32 * w + __ffs(m0) - 1;
            m0 &= m0 - 1u;
            rx0 += S.s[0][s];
            ry0 += S.s[1][s];
          }
          while (m1) {
            const int s = 32 * w + __ffs(m1) - 1;
            m1 &= m1 - 1u;
            rx1 += S.s[0][s];
            ry1 += S.s[1][s];
          }
        }
        S.u.o.bx[lane] = rx0;
        S.u.o.by[lane] = ry0;
        if (b1 < 42) {
          S.u.o.bx[b1] = rx1;
          S.u.o.by[b1] = ry1;
        }
      }
      __syncwarp();
      float best = -1.0f;
      int bk = 0;
      for (int t = lane; t < 42; t += 32) {
        float ex = S.u.o.bx[t], ey = S.u.o.by[t];
        for (int q = t + 1; q < t + 7; q++) {
          ex += S.u.o.bx[q < 42 ? q : q - 42];
          ey += S.u.o.by[q < 42 ? q : q - 42];
        }
        S.u.o.wx[t] = ex;
        S.u.o.wy[t] = ey;
        const float r = ex * ex + ey * ey;
        if (r > best) {
          best = r;
          bk = t;
        }
      }
      /* the reference keeps the first k with r > maxr (maxr starts at 0) */
      for (int o = 16; o > 0; o >>= 1) {
        const float ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int ok = __shfl_xor_sync(0xffffffffu, bk, o);
        if (ob > best || (ob == best && ok < bk)) {
          best = ob;
          bk = ok;
        }
      }
      if (!(best > 0.0f)) bk = 0;
      __syncwarp();
      const float a = akz_atan2f(S.u.o.wy[bk], S.u.o.wx[bk]);
      angle = a < 0.0f ? (float)((double)a + 2.0 * AKZ_CV_PI) : a;
      if (lane == 0) kpp->angle = angle;
      __syncwarp();
    }
    /* M-LDB samples */
    float co = 1.0f, si = 0.0f;
    if (!p.upright) akz_sincosf(angle, &si, &co);
    const float iratio = 1.0f / (float)(1 << kp.octave);
    const int scale = (int)(0.5f * kp.size * iratio + 0.5f);
    const float xf = kp.x * iratio, yf = kp.y * iratio;
    const float fs = (float)scale;
    /* the window's samples, every gather in flight before the first use
     * (the window has at most 21 x 21 <= 14 x 32 samples: pattern size
     * <= 10), in the block order of g_smp_order */
    const int nsmp = win * win;
    {
      float vi[AKZ_DESC_ITERS], vx[AKZ_DESC_ITERS], vy[AKZ_DESC_ITERS];
#pragma unroll
      for (int it = 0; it < AKZ_DESC_ITERS; it++) {
        const int idx = lane + 32 * it;
        if (idx < nsmp) {
          const int o = sOrd[idx], yy = o >> 8, xx = o & 255;
          const int l = xx - size2, kk = yy - size2;
          int xp = (int)(xf + fs * ((float)kk * co - (float)l * si) + 0.5f);
          int yp = (int)(yf + fs * ((float)kk * si + (float)l * co) + 0.5f);
          xp = akz_clampi(xp, 0, W - 1);
          yp = akz_clampi(yp, 0, H - 1);
          vi[it] = __ldg(ltp + (long long)yp * pitch + xp);
          const float2 g2 = __ldg(reinterpret_cast<const float2 *>(lxyp + (long long)yp * (2 * pitch) + 2 * xp));
          vx[it] = g2.x;
          vy[it] = g2.y;
        }
      }
#pragma unroll
      for (int it = 0; it < AKZ_DESC_ITERS; it++) {
        const int idx = lane + 32 * it;
        if (idx < nsmp) {
          const int o = sOrd[idx], s = (o >> 8) * win + (o & 255);
          const float dx = vx[it], dy = vy[it];
          S.s[0][s] = vi[it];
          /* a 2-channel descriptor's second channel is the gradient magnitude (upstream libAKAZE's MLDB_Fill_Values) */
          S.s[1][s] = p.channels == 2 ? __fsqrt_rn(dx * dx + dy * dy) : -dx * si + dy * co;
          S.s[2][s] = dx * co + dy * si;
        }
      }
    }
    for (int s = lane + 32 * AKZ_DESC_ITERS; s < nsmp; s += 32) { /* larger windows: not reached for pattern size <= 10 */
      const int yy = s / win, xx = s - yy * win;
      const int l = xx - size2, kk = yy - size2;
      const int xp = akz_clampi((int)(xf + fs * ((float)kk * co - (float)l * si) + 0.5f), 0, W - 1);
      const int yp = akz_clampi((int)(yf + fs * ((float)kk * si + (float)l * co) + 0.5f), 0, H - 1);
      const float2 g2 = __ldg(reinterpret_cast<const float2 *>(lxyp + (long long)yp * (2 * pitch) + 2 * xp));
      const float dx = g2.x, dy = g2.y;
      S.s[0][s] = __ldg(ltp + (long long)yp * pitch + xp);
      S.s[1][s] = p.channels == 2 ? __fsqrt_rn(dx * dx + dy * dy) : -dx * si + dy * co;
      S.s[2][s] = dx * co + dy * si;
    }
    __syncwarp();
    akz_mldb_cells<4, 0, 7, 0>(S.u.acc, S.s, sCell, lane, nsmp, S.v);
    akz_mldb_cells<9, 3, 15, 4>(S.u.acc, S.s, sCell, lane, nsmp, S.v);
    akz_mldb_cells<16, 7, 31, 13>(S.u.acc, S.s, sCell, lane, nsmp, S.v);
    __syncwarp();
    /* word w holds bits 32w .. 32w+31, LSB first: one ballot per word */
    uint32_t myword = 0;
#pragma unroll 4
    for (int w = 0; w < 16; w++) {
      const int bit = w * 32 + lane;
      const bool v = bit < p.nbits && S.v[__ldg(&p.cmp1[bit])] > S.v[__ldg(&p.cmp2[bit])];
      const uint32_t word = __ballot_sync(0xffffffffu, v);
      if (lane == w) myword = word;
    }
    if (lane < 16) p.desc[(long long)(I.kp_base + k) * 16 + lane] = myword;
    __syncwarp();
  }
}

#define AKZ_DESC_MAXDEV 64
static bool akz_describe_tables_ready[AKZ_DESC_MAXDEV];
static int akz_describe_grid[AKZ_DESC_MAXDEV]; /* resident CTAs of the device (with the largest offset table) */
static std::mutex akz_describe_tables_mutex;

static cudaError_t akz_init_describe_tables()
{
  static unsigned short ord[AKZ_DESC_MAXWIN + 1][32 * AKZ_DESC_ITERS];
  for (int win = 1; win <= AKZ_DESC_MAXWIN; win++) {
    int no = 0;
    for (int tr = 0; tr < win; tr += 4)
      for (int tc = 0; tc < win; tc += 8)
        for (int r = tr; r < tr + 4 && r < win; r++)
          for (int c = tc; c < tc + 8 && c < win; c++) ord[win][no++] = (unsigned short)((r << 8) | c);
    while (no < 32 * AKZ_DESC_ITERS) ord[win][no++] = 0;
  }
  signed char oi[109], oj[109], orr[109];
  int n = 0;
  for (int tx = 0; tx < 208; tx++) {
    const int i = (tx & 15) - 6, j = (tx / 16) - 6;
    if (i * i + j * j < 36) {
      oi[n] = (signed char)i;
      oj[n] = (signed char)j;
      orr[n] = (signed char)(i * i + j * j);
      n++;
    }
  }
  cudaError_t e;
  if ((e = cudaMemcpyToSymbol(c_oi, oi, sizeof(oi))) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(c_oj, oj, sizeof(oj))) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(c_or2, orr, sizeof(orr))) != cudaSuccess) return e;
  return cudaMemcpyToSymbol(g_smp_order, ord, sizeof(ord));
}

cudaError_t akz_launch_describe(const akz_describe_params &p, int nblocks, cudaStream_t s)
{
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= AKZ_DESC_MAXDEV || p.pattern_size < 1 || p.pattern_size > 10) return cudaErrorInvalidValue;
  int resident = 0;
  {
    std::lock_guard<std::mutex> lock(akz_describe_tables_mutex);
    if (!akz_describe_tables_ready[dev]) {
      cudaError_t e = akz_init_describe_tables();
      if (e != cudaSuccess) return e;
      /* a grid-stride loop over the keypoints: one wave of resident CTAs,
       * counted once per device with the largest keypoint-offset table */
      int per_sm = 0, nsm = 0;
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_describe, 32 * AKZ_DESC_WARPS,
                                                        (AKZ_DESC_MAXIMG + 1) * sizeof(int));
      if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
      if (e != cudaSuccess) return e;
      akz_describe_grid[dev] = std::max(1, per_sm) * std::max(1, nsm);
      akz_describe_tables_ready[dev] = true;
    }
    resident = akz_describe_grid[dev];
  }
  if (nblocks <= 0) return cudaSuccess;
  const size_t dyn = p.t.nimg <= AKZ_DESC_MAXIMG ? (size_t)(p.t.nimg + 1) * sizeof(int) : 0;
  const int grid = std::min(nblocks, resident);
  k_describe<<<grid, 32 * AKZ_DESC_WARPS, dyn, s>>>(p);
  return cudaGetLastError();
}

/* Packs every image's keypoints and descriptor rows (rb <= 64 bytes each)
 * contiguously (image i at offset sum_{j<i} nkp_j): blockIdx.x is the image,
 * blockIdx.y a slice of its words.  The keypoint records are copied as
 * words; the descriptor rows are written as the 4-byte words of the packed
 * byte stream, consecutive threads on consecutive words (coalesced), each
 * word gathered from the one or two 64-byte source rows it spans.  An
 * image's first and last words may hold its neighbours' bytes too: those
 * two go byte by byte, every byte by the CTAs of its own image. */
__global__ void k_pack_results(akz_tables t, const akz_kp *kp, const uint32_t *desc, akz_kp *kp_out, uint8_t *desc_out,
                               int rb)
{
  static_assert(sizeof(akz_kp) % 4 == 0, "keypoint records are whole words");
  constexpr int KW = sizeof(akz_kp) / 4;
  const int img = blockIdx.x;
  long long off = 0;
  for (int j = 0; j < img; j++) off += t.stats[j].nkp;
  const int n = t.stats[img].nkp;
  if (n <= 0) return;
  const akz_image_desc I = t.im[img];
  const long long tid = (long long)blockIdx.y * blockDim.x + threadIdx.x, nt = (long long)gridDim.y * blockDim.x;
  const uint32_t *ks = reinterpret_cast<const uint32_t *>(kp + I.kp_base);
  uint32_t *kd = reinterpret_cast<uint32_t *>(kp_out + off);
  for (long long w = tid; w < (long long)n * KW; w += nt) kd[w] = ks[w];
  const uint8_t *ds = reinterpret_cast<const uint8_t *>(desc) + (long long)I.kp_base * 64;
  const long long b0 = off * rb, b1 = b0 + (long long)n * rb; /* this image's bytes of the stream */
  for (long long w = (b0 >> 2) + tid; w < (b1 + 3) >> 2; w += nt) {
    const long long b = w << 2;
    if (b >= b0 && b + 4 <= b1) {
      long long r = (b - b0) / rb;
      int c = (int)(b - b0 - r * rb);
      uint32_t v = 0;
#pragma unroll
      for (int k = 0; k < 4; k++) {
        v |= (uint32_t)ds[r * 64 + c] << (8 * k);
        if (++c == rb) {
          c = 0;
          r++;
        }
      }
      reinterpret_cast<uint32_t *>(desc_out)[w] = v;
    } else {
      for (int k = 0; k < 4; k++) {
        const long long bb = b + k;
        if (bb < b0 || bb >= b1) continue;
        const long long r = (bb - b0) / rb;
        desc_out[bb] = ds[r * 64 + (bb - b0 - r * rb)];
      }
    }
  }
}

cudaError_t akz_launch_pack_results(const akz_tables &t, const akz_kp *kp, const uint32_t *desc, akz_kp *kp_out,
                                    uint8_t *desc_out, int row_bytes, cudaStream_t s)
{
  if (row_bytes < 1 || row_bytes > 64) return cudaErrorInvalidValue;
  if (((uintptr_t)kp_out | (uintptr_t)desc_out) & 3) return cudaErrorInvalidValue; /* word stores */
  /* 64 slices per image: a few words per thread, so the gathers of a
   * thread's loop iterations do not queue behind one another */
  k_pack_results<<<dim3(t.nimg, 64), 256, 0, s>>>(t, kp, desc, kp_out, desc_out, row_bytes);
  return cudaGetLastError();
}
