/*
 * akz_surrogate_infer.cu - inference of the FED surrogate on a whole level,
 * BF16 tensor-core implicit GEMM with FP32 accumulation.
 *
 * Per level:   im2col  (L_start, g, dt feature) -> A1 [pixel][32] bf16
 *              (k = tap*3 + channel, 27 used), replicate border;
 *              conv 1  1x1 GEMM  32 -> 32, ReLU;
 *              conv 2-4 3x3 implicit GEMM 32 -> 32, ReLU (k = tap*32 + ci);
 *              conv 5  3x3 32 -> 1 (padded to 8 outputs), then
 *              L_end = L_start + s_out * (net output).
 * Every 3x3 layer extends its input by replicate padding at the image border.
 *
 * The 3 x 3 layers 2-4 run on tcgen05 (k_sg_conv_tcp below, the default);
 * layers 1 and 5, and layers 2-4 when tcgen05 is switched off, on mma.sync.
 *
 * mma.sync kernel: a CTA computes a 32 x 4 pixel block (4 warps, one pixel row
 * each, two m16 tiles per warp) for all outputs.  Its input region (with a
 * one-pixel halo for 3x3) is staged in shared memory as 64-byte pixel rows
 * whose four 16-byte channel chunks are XOR-swizzled by (pixel >> 1) & 3, so
 * the eight rows of an ldmatrix 8x8 read land on distinct banks.  Weights
 * are staged as [n][k] rows padded by 16 bytes (also conflict-free).
 * mma.sync m16n8k16 bf16 -> f32.
 */
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/akaze_gb300.h"

akz_status akz_report(akz_status s, const char *msg);

struct akz_sg_level {
  const float *l0, *g;
  long long pitch;
  int W, H;
  float dtf, s_out;
  float *out;
};

__device__ __forceinline__ int sg_clamp(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

__global__ void k_sg_im2col(akz_sg_level lv, __nv_bfloat16 *act)
{
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= lv.W) return;
  __align__(16) __nv_bfloat16 v[32];
#pragma unroll
  for (int t = 0; t < 9; t++) {
    const int yy = sg_clamp(y + t / 3 - 1, 0, lv.H - 1), xx = sg_clamp(x + t % 3 - 1, 0, lv.W - 1);
    const long long o = (long long)yy * lv.pitch + xx;
    v[3 * t] = __float2bfloat16_rn(lv.l0[o]);
    v[3 * t + 1] = __float2bfloat16_rn(lv.g[o]);
    v[3 * t + 2] = __float2bfloat16_rn(lv.dtf);
  }
#pragma unroll
  for (int k = 27; k < 32; k++) v[k] = __float2bfloat16_rn(0.0f);
  uint4 *dst = (uint4 *)(act + ((long long)y * lv.W + x) * 32);
  const uint4 *src = (const uint4 *)v;
#pragma unroll
  for (int c = 0; c < 4; c++) dst[c] = src[c];
}

__device__ __forceinline__ void sg_ldsm_x4(unsigned int (&r)[4], const void *p)
{
  const unsigned int a = (unsigned int)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(a));
}

__device__ __forceinline__ void sg_ldsm_x2(unsigned int (&r)[2], const void *p)
{
  const unsigned int a = (unsigned int)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0, %1}, [%2];" : "=r"(r[0]), "=r"(r[1]) : "r"(a));
}

__device__ __forceinline__ void sg_mma(float (&d)[4], const unsigned int (&a)[4], unsigned int b0, unsigned int b1)
{
  asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
               "{%0, %1, %2, %3};"
               : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
               : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

#define SG_BX 32
#define SG_BY 4

/* NTAPS 1 (1x1) or 9 (3x3); NT n8 output tiles (4 -> 32 outputs, 1 -> 8);
 * FINAL: write L_start + s_out * output channel 0 to the level plane,
 * otherwise bias + ReLU -> bf16 NHWC. */
template <int NTAPS, int NT, bool FINAL>
__global__ void __launch_bounds__(128) k_sg_conv_mma(const __nv_bfloat16 *__restrict__ in, const __nv_bfloat16 *__restrict__ wt,
                                                     const float *__restrict__ bias, __nv_bfloat16 *__restrict__ out,
                                                     akz_sg_level lv)
{
  constexpr int K = NTAPS * 32, KS = K + 8; /* weight row stride (bf16): 16-byte pad */
  constexpr int HALO = NTAPS == 9 ? 1 : 0;
  constexpr int RX = SG_BX + 2 * HALO, RY = SG_BY + 2 * HALO;
  __shared__ __align__(16) __nv_bfloat16 sW[NT * 8 * KS];
  __shared__ __align__(16) unsigned char sA[RX * RY * 64];
  __shared__ float sBias[NT * 8];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int W = lv.W, H = lv.H;
  const int x0 = blockIdx.x * SG_BX, y0 = blockIdx.y * SG_BY;
  for (int i = tid; i < NT * 8 * (K / 8); i += 128) {
    const int n = i / (K / 8), c = i - n * (K / 8);
    *(uint4 *)(sW + n * KS + c * 8) = *(const uint4 *)(wt + n * K + c * 8);
  }
  if (tid < NT * 8) sBias[tid] = bias[tid];
  for (int i = tid; i < RX * RY * 4; i += 128) {
    const int q = i >> 2, c = i & 3;
    const int ry = q / RX, rx = q - ry * RX;
    const int yy = sg_clamp(y0 - HALO + ry, 0, H - 1), xx = sg_clamp(x0 - HALO + rx, 0, W - 1);
    const uint4 v = *(const uint4 *)(in + ((long long)yy * W + xx) * 32 + c * 8);
    *(uint4 *)(sA + q * 64 + ((c ^ ((q >> 1) & 3)) << 4)) = v;
  }
  __syncthreads();

  float acc[2][NT][4];
#pragma unroll
  for (int mt = 0; mt < 2; mt++)
#pragma unroll
    for (int nt = 0; nt < NT; nt++)
#pragma unroll
      for (int j = 0; j < 4; j++) acc[mt][nt][j] = 0.0f;

#pragma unroll 1
  for (int t = 0; t < NTAPS; t++) {
    const int dy = NTAPS == 9 ? t / 3 : 0, dx = NTAPS == 9 ? t % 3 : 0;
#pragma unroll
    for (int h = 0; h < 2; h++) {
      unsigned int a[2][4];
#pragma unroll
      for (int mt = 0; mt < 2; mt++) {
        const int q = (warp + dy) * RX + mt * 16 + (lane & 15) + dx;
        const int c = h * 2 + (lane >> 4);
        sg_ldsm_x4(a[mt], sA + q * 64 + ((c ^ ((q >> 1) & 3)) << 4));
      }
      const int kb = t * 32 + h * 16;
      if (NT >= 2) {
#pragma unroll
        for (int np = 0; np < NT / 2; np++) {
          unsigned int b[4];
          const int n = np * 16 + ((lane >> 4) & 1) * 8 + (lane & 7);
          sg_ldsm_x4(b, sW + n * KS + kb + ((lane >> 3) & 1) * 8);
#pragma unroll
          for (int mt = 0; mt < 2; mt++) {
            sg_mma(acc[mt][2 * np], a[mt], b[0], b[1]);
            sg_mma(acc[mt][2 * np + 1], a[mt], b[2], b[3]);
          }
        }
      } else {
        unsigned int b[2];
        const int n = lane & 7;
        sg_ldsm_x2(b, sW + n * KS + kb + ((lane >> 3) & 1) * 8);
#pragma unroll
        for (int mt = 0; mt < 2; mt++) sg_mma(acc[mt][0], a[mt], b[0], b[1]);
      }
    }
  }

  const int y = y0 + warp;
  if (y >= H) return;
#pragma unroll
  for (int mt = 0; mt < 2; mt++)
#pragma unroll
    for (int half = 0; half < 2; half++) {
      const int x = x0 + mt * 16 + (lane >> 2) + half * 8;
      if (x >= W) continue;
      if (FINAL) {
        if ((lane & 3) == 0) {
          const long long o = (long long)y * lv.pitch + x;
          lv.out[o] = lv.l0[o] + lv.s_out * (acc[mt][0][half * 2] + sBias[0]);
        }
      } else {
#pragma unroll
        for (int nt = 0; nt < NT; nt++) {
          const int ch = nt * 8 + (lane & 3) * 2;
          const float v0 = fmaxf(acc[mt][nt][half * 2] + sBias[ch], 0.0f);
          const float v1 = fmaxf(acc[mt][nt][half * 2 + 1] + sBias[ch + 1], 0.0f);
          *(__nv_bfloat162 *)(out + ((long long)y * W + x) * 32 + ch) = __floats2bfloat162_rn(v0, v1);
        }
      }
    }
}

/* ------------------------------------------------------------------------ */
/* tcgen05 helpers.  Shared-memory operands use the canonical K-major layout
 * without swizzle: 8-row x 16-byte core matrices, row r of a core matrix at
 * r * 16 bytes; LBO is the byte distance of core matrices adjacent in K,
 * SBO of those adjacent in M / N. */

#define AKZ_SG_TC_SPIN (1 << 24)

__device__ __forceinline__ uint64_t sg_smem_desc(const void *p, uint32_t lbo, uint32_t sbo)
{
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
  uint64_t d = 0;
  d |= (uint64_t)((a & 0x3FFFF) >> 4);          /* start address, bits 0-13 */
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;   /* leading dimension byte offset */
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;   /* stride dimension byte offset */
  d |= (uint64_t)1 << 46;                       /* descriptor version */
  return d;                                     /* base offset 0, no swizzle */
}

/* kind::f16 instruction descriptor: D F32, A and B BF16, both K-major */
__host__ __device__ constexpr uint32_t sg_idesc(int M, int N)
{
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

/* ------------------------------------------------------------------------ */
/* Persistent, pipelined tcgen05 kernel for the 3 x 3 layers (32 -> 32).
 *
 * Work item: a 128-pixel column block and rc consecutive rows.  The CTA
 * walks the rows downwards; each input row (the block's 128 pixels plus one
 * on each side, replicate-clamped) is staged once, by cp.async, into a ring
 * of SG_TP_R rows laid out as [channel group][pixel] 16-byte cells.  In that
 * layout the K-major core matrices of a row are SBO = 128 bytes apart along
 * M (8 pixels) and LBO = SG_TP_NPIX * 16 bytes apart along K, so the three
 * horizontal taps of a row are the same row at start offsets 0, 16 and 32
 * bytes: no im2col copy.  Row y's 18 MMAs (9 taps x 2 K-steps of 16) read
 * ring rows y - 1 .. y + 1 and accumulate into one of two 32-column TMEM
 * buffers; while they run, the threads wait for row y - 1's MMAs, load row
 * y + 4 into the slot row y - 2 left (rows y + 2 and y + 3 are on their
 * way), and write row y - 1 from TMEM (bias, ReLU, bf16); one barrier per
 * row.  rc is chosen by the host so that every CTA gets at most one item.
 * Every mbarrier wait is bounded; a timeout records the error flag, ends the
 * CTA's loop at the next barrier, and TMEM is freed after one more bounded
 * wait. */

#define SG_TP_R 6                      /* ring rows */
#define SG_TP_NPIX 130                 /* staged pixels per row */
#define SG_TP_SLOT (4 * SG_TP_NPIX * 16) /* bytes per ring row */
#define SG_TP_SMEM (32 * 288 * 2 + SG_TP_R * SG_TP_SLOT)

__device__ __forceinline__ void sg_cp_async16(void *dst, const void *src)
{
  const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}

__device__ __forceinline__ bool sg_mbar_wait(const unsigned long long *mbar, uint32_t parity)
{
  const uint32_t mb = (uint32_t)__cvta_generic_to_shared(mbar);
  uint32_t done = 0;
  for (int it = 0; it < AKZ_SG_TC_SPIN && !done; it++)
    asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
                 : "=r"(done)
                 : "r"(mb), "r"(parity)
                 : "memory");
  return done != 0;
}

__global__ void __launch_bounds__(128) k_sg_conv_tcp(const __nv_bfloat16 *__restrict__ in,
                                                     const __nv_bfloat16 *__restrict__ wt, const float *__restrict__ bias,
                                                     __nv_bfloat16 *__restrict__ out, akz_sg_level lv, int rc, int *err)
{
  constexpr int K = 288, NP = SG_TP_NPIX, R = SG_TP_R;
  extern __shared__ __align__(1024) unsigned char tpsm[];
  unsigned char *sB = tpsm, *sR = tpsm + 32 * K * 2;
  __shared__ __align__(8) unsigned long long mbar[2];
  __shared__ uint32_t tbase;
  __shared__ float sBias[32];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int W = lv.W, H = lv.H;
  const int nxb = (W + 127) / 128, nitems = nxb * ((H + rc - 1) / rc);

  /* weights: row n, K group kg -> core matrix (n / 8, kg), row n % 8 */
  for (int i = tid; i < 32 * (K / 8); i += 128) {
    const int n = i / (K / 8), kg = i - n * (K / 8);
    *(uint4 *)(sB + (n >> 3) * (K * 16) + kg * 128 + (n & 7) * 16) = *(const uint4 *)(wt + n * K + kg * 8);
  }
  if (tid < 32) sBias[tid] = bias[tid];
  if (warp == 0) {
    const uint32_t dst = (uint32_t)__cvta_generic_to_shared(&tbase);
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 64;" ::"r"(dst));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int b = 0; b < 2; b++) {
      const uint32_t mb = (uint32_t)__cvta_generic_to_shared(&mbar[b]);
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb));
    }
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  asm volatile("fence.proxy.async.shared::cta;");
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tbase;
  constexpr uint32_t idesc = sg_idesc(128, 32);
  const uint64_t adesc0 = sg_smem_desc(sR, NP * 16, 128), bdesc0 = sg_smem_desc(sB, 128, K * 16);

  auto load_row = [&](int yrow, int slot, int x0) { /* 16-byte chunks, pixel-major over the threads */
    const __nv_bfloat16 *src = in + (long long)sg_clamp(yrow, 0, H - 1) * W * 32;
    unsigned char *dst = sR + slot * SG_TP_SLOT;
    for (int c = tid; c < 4 * NP; c += 128) {
      const int px = c >> 2, kg = c & 3;
      sg_cp_async16(dst + kg * (NP * 16) + px * 16, src + (long long)sg_clamp(x0 - 1 + px, 0, W - 1) * 32 + kg * 8);
    }
  };
  /* landed rows -> tensor core; all threads past their TMEM reads; returns
   * (CTA-uniform) whether any thread saw an MMA wait run out */
  auto sync_ring = [&](int pending, bool bad) -> bool {
    if (pending)
      asm volatile("cp.async.wait_group 2;" ::: "memory");
    else
      asm volatile("cp.async.wait_group 0;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;");
    asm volatile("tcgen05.fence::before_thread_sync;");
    const bool any = __syncthreads_or(bad) != 0;
    asm volatile("tcgen05.fence::after_thread_sync;");
    return any;
  };
  auto epilogue = [&](uint32_t c, int y, int x0) { /* batch c's accumulator: warp w has pixels 32w .. 32w+31 */
    uint32_t r[32];
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (c & 1u) * 32u;
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;");
    const int x = x0 + warp * 32 + lane;
    if (x < W && y < H) {
      __align__(16) __nv_bfloat162 v[16];
#pragma unroll
      for (int k = 0; k < 16; k++)
        v[k] = __floats2bfloat162_rn(fmaxf(__uint_as_float(r[2 * k]) + sBias[2 * k], 0.0f),
                                     fmaxf(__uint_as_float(r[2 * k + 1]) + sBias[2 * k + 1], 0.0f));
      uint4 *dst = (uint4 *)(out + ((long long)y * W + x) * 32);
      const uint4 *src = (const uint4 *)v;
#pragma unroll
      for (int k = 0; k < 4; k++) dst[k] = src[k];
    }
  };

  uint32_t issued = 0, retired = 0; /* MMA batches issued / known complete (batch c: mbar[c & 1], its (c >> 1)-th phase) */
  bool ok = true;
  for (int item = blockIdx.x; item < nitems && ok; item += gridDim.x) {
    const int xb = item % nxb, yb = (item / nxb) * rc, n = min(rc, H - yb), x0 = xb * 128;
    /* ring row j holds image row yb - 1 + j, slot j % R; row y's MMAs need rows up to y + 1 */
    load_row(yb - 1, 0, x0);
    load_row(yb, 1, x0);
    load_row(yb + 1, 2, x0);
    asm volatile("cp.async.commit_group;" ::: "memory");
    if (n >= 2) load_row(yb + 2, 3, x0);
    asm volatile("cp.async.commit_group;" ::: "memory");
    if (n >= 3) load_row(yb + 3, 4, x0);
    asm volatile("cp.async.commit_group;" ::: "memory");
    sync_ring(1, false);
    for (int i = 0; i < n; i++) {
      if (tid == 0) { /* row yb + i: ring rows i .. i + 2, taps (dy, dx) at slot (i + dy) % R, offset 16 dx */
        const uint32_t d = tmem + (issued & 1u) * 32u;
        const uint32_t so[3] = {(uint32_t)((i % R) * SG_TP_SLOT), (uint32_t)(((i + 1) % R) * SG_TP_SLOT),
                                (uint32_t)(((i + 2) % R) * SG_TP_SLOT)};
#pragma unroll
        for (int s = 0; s < 18; s++) {
          const int t = s >> 1, kc = s & 1, dy = t / 3, dx = t - 3 * dy;
          /* the start address field counts 16-byte units in the low bits: offsets add to it */
          const uint64_t ad = adesc0 + ((so[dy] + (uint32_t)((2 * kc) * (NP * 16) + dx * 16)) >> 4);
          const uint64_t bd = bdesc0 + (uint64_t)((2 * s * 128) >> 4);
          const uint32_t acc = s > 0 ? 1u : 0u;
          asm volatile(
              "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
              "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d),
              "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
        }
        const uint32_t mb = (uint32_t)__cvta_generic_to_shared(&mbar[issued & 1u]);
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mb));
      }
      issued++;
      bool bad = false;
      if (i >= 1) { /* row yb + i - 1's MMAs: then its ring row yb + i - 2 is free and its accumulator ready */
        const uint32_t c = issued - 2;
        bad = !sg_mbar_wait(&mbar[c & 1u], (c >> 1) & 1u);
        if (!bad) retired = c + 1;
      }
      if (i + 4 <= n && !bad) load_row(yb + i + 4, (i + 5) % R, x0);
      asm volatile("cp.async.commit_group;" ::: "memory");
      if (i >= 1) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        epilogue(issued - 2, yb + i - 1, x0);
      }
      if (sync_ring(1, bad)) {
        ok = false;
        break;
      }
    }
    if (!ok) break;
    { /* the item's last row */
      const uint32_t c = issued - 1;
      const bool bad = !sg_mbar_wait(&mbar[c & 1u], (c >> 1) & 1u);
      if (!bad) retired = c + 1;
      asm volatile("tcgen05.fence::after_thread_sync;");
      epilogue(c, yb + n - 1, x0);
      if (sync_ring(0, bad)) {
        ok = false;
        break;
      }
    }
  }
  if (!ok) {
    if (tid == 0) atomicExch(err, 1);
    if (retired < issued) { /* batches complete in order: wait (bounded) for the last one */
      const uint32_t c = issued - 1;
      sg_mbar_wait(&mbar[c & 1u], (c >> 1) & 1u);
    }
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;" ::"r"(tmem));
}

/* tensor path of the 3 x 3 layers 2-4 (on: k_sg_conv_tcp, off: mma.sync),
 * and the flag the tcgen05 kernel sets when an MMA wait ran out. */
static int g_sg_tc = 1;
static __device__ int g_sg_tc_err;

extern "C" AKZ_API akz_status akz_sg_set_tcgen05(int on)
{
  g_sg_tc = on ? 1 : 0;
  return AKZ_OK;
}

extern "C" AKZ_API akz_status akz_sg_tcgen05_status(int *timed_out)
{
  if (!timed_out) return akz_report(AKZ_ERR_INVALID_ARG, "akz_sg_tcgen05_status: NULL");
  int v = 0;
  cudaError_t e = cudaMemcpyFromSymbol(&v, g_sg_tc_err, sizeof(int));
  if (e == cudaSuccess) {
    const int z = 0;
    e = cudaMemcpyToSymbol(g_sg_tc_err, &z, sizeof(int));
  }
  if (e != cudaSuccess) return akz_report(AKZ_ERR_CUDA, cudaGetErrorString(e));
  *timed_out = v;
  return AKZ_OK;
}

/* Packed weights (bf16): layer 1 [32][32], layers 2-4 [32][288], layer 5
 * [8][288] (rows 1-7 zero); biases (f32): 4 x 32 + 8. */
#define SG_W1 (32 * 32)
#define SG_W3 (32 * 288)
#define SG_W5 (8 * 288)

extern "C" AKZ_API size_t akz_sg_weight_elems(void) { return SG_W1 + 3 * SG_W3 + SG_W5; }

extern "C" AKZ_API akz_status akz_sg_infer_level(const float *l0, const float *g, size_t pitch, int width, int height,
                                                 float dt_feature, float s_out, const void *weights_bf16,
                                                 const float *biases, void *scratch, float *out, void *stream)
{
  if (!l0 || !g || !weights_bf16 || !biases || !scratch || !out || width < 1 || height < 1 || pitch < (size_t)width)
    return akz_report(AKZ_ERR_INVALID_ARG, "akz_sg_infer_level: bad arguments");
  if (((uintptr_t)weights_bf16 & 15) || ((uintptr_t)scratch & 15))
    return akz_report(AKZ_ERR_INVALID_ARG, "akz_sg_infer_level: weights and scratch must be 16-byte aligned");
  cudaStream_t s = (cudaStream_t)stream;
  akz_sg_level lv;
  lv.l0 = l0;
  lv.g = g;
  lv.pitch = (long long)pitch;
  lv.W = width;
  lv.H = height;
  lv.dtf = dt_feature;
  lv.s_out = s_out;
  lv.out = out;
  const __nv_bfloat16 *w = (const __nv_bfloat16 *)weights_bf16;
  __nv_bfloat16 *a0 = (__nv_bfloat16 *)scratch, *a1 = a0 + (size_t)width * height * 32;
  k_sg_im2col<<<dim3((width + 127) / 128, height), 128, 0, s>>>(lv, a0);
  const dim3 grid((width + SG_BX - 1) / SG_BX, (height + SG_BY - 1) / SG_BY);
  if (g_sg_tc) {
    int *err = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void **)&err, g_sg_tc_err);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_sg_conv_tcp, cudaFuncAttributeMaxDynamicSharedMemorySize, SG_TP_SMEM);
    /* all of the unified L1 as shared memory, so that 3 CTAs fit an SM */
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_sg_conv_tcp, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
    int dev = 0, nsm = 0, smem_sm = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    if (e != cudaSuccess) return akz_report(AKZ_ERR_CUDA, cudaGetErrorString(e));
    /* resident CTAs per SM: shared memory (operands, ring, ~1 KB static and 1 KB reserved each), at most 8
     * (8 x 64 TMEM columns = 512) */
    const int per_sm = std::max(1, std::min(8, smem_sm / (SG_TP_SMEM + 2048)));
    /* rows per item: every resident CTA gets at most one item, of at least 2 rows */
    const int nxb = (width + 127) / 128, ctas = per_sm * nsm;
    const int rc = std::max(2, (height + std::max(1, ctas / nxb) - 1) / std::max(1, ctas / nxb));
    const int items = nxb * ((height + rc - 1) / rc);
    const int gp = std::max(1, std::min(items, ctas));
    k_sg_conv_mma<1, 4, false><<<grid, 128, 0, s>>>(a0, w, biases, a1, lv);
    k_sg_conv_tcp<<<gp, 128, SG_TP_SMEM, s>>>(a1, w + SG_W1, biases + 32, a0, lv, rc, err);
    k_sg_conv_tcp<<<gp, 128, SG_TP_SMEM, s>>>(a0, w + SG_W1 + SG_W3, biases + 64, a1, lv, rc, err);
    k_sg_conv_tcp<<<gp, 128, SG_TP_SMEM, s>>>(a1, w + SG_W1 + 2 * SG_W3, biases + 96, a0, lv, rc, err);
  } else {
    k_sg_conv_mma<1, 4, false><<<grid, 128, 0, s>>>(a0, w, biases, a1, lv);
    k_sg_conv_mma<9, 4, false><<<grid, 128, 0, s>>>(a1, w + SG_W1, biases + 32, a0, lv);
    k_sg_conv_mma<9, 4, false><<<grid, 128, 0, s>>>(a0, w + SG_W1 + SG_W3, biases + 64, a1, lv);
    k_sg_conv_mma<9, 4, false><<<grid, 128, 0, s>>>(a1, w + SG_W1 + 2 * SG_W3, biases + 96, a0, lv);
  }
  k_sg_conv_mma<9, 1, true><<<grid, 128, 0, s>>>(a0, w + SG_W1 + 3 * SG_W3, biases + 128, nullptr, lv);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return akz_report(AKZ_ERR_CUDA, cudaGetErrorString(e));
  return AKZ_OK;
}

/* max |a - b| over a level plane into *slot (non-negative float bits, so an
 * integer atomicMax orders them); NaN or infinity counts as infinity */
__global__ void k_sg_maxdiff(const float *a, const float *b, int pitch, int W, int H, float *slot)
{
  float m = 0.0f;
  for (long long i = blockIdx.x * 256LL + threadIdx.x; i < (long long)W * H; i += (long long)gridDim.x * 256) {
    const long long o = (i / W) * pitch + i % W;
    float d = fabsf(a[o] - b[o]);
    if (!(d <= 3.0e38f)) d = __int_as_float(0x7f800000);
    m = fmaxf(m, d);
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax((int *)slot, __float_as_int(m));
}

cudaError_t akz_sg_maxdiff(const float *a, const float *b, int pitch, int width, int height, float *slot, cudaStream_t s)
{
  const long long n = (long long)width * height;
  const int blocks = (int)std::min<long long>((n + 255) / 256, 1024);
  k_sg_maxdiff<<<blocks, 256, 0, s>>>(a, b, pitch, width, height, slot);
  return cudaGetLastError();
}
