/*
 * akz_match_tc.cu - the 2-NN Hamming matcher on the tensor cores.
 *
 * Same result as k_match (akz_match.cu; reference MatchDescriptors,
 * cuda_akaze.cu:1843-1967, and Matcher::bfmatch, AKAZE.cpp:36-79), bit for
 * bit, with the pair distances formed by tcgen05 FP8 matrix multiplies
 * instead of 16 xor + popc per pair.
 *
 * For 512-bit rows q (query) and t (train), with a, b their bits:
 *   hamming(q, t) = popc(q) + sum_k b_k (1 - 2 a_k).
 * Train bits become E4M3 values b w_k (w_k a power of two chosen by the
 * bit's position in its byte) and query bits (1 - 2a) / w_k, so every
 * product is 0 or +-1; one K = 512 product per pair gives the sums, exact in
 * the FP32 accumulator (integers of magnitude <= 512).  The result is the
 * popc kernel's: the two smallest (distance, train index) pairs, ties to
 * the lower index (the cv::BFMatcher rule), starting from two entries
 * {distance 512, index 0}.
 *
 * A CTA (one per SM: it holds all 512 TMEM columns) loops over work items of
 * 256 queries x one train split.  Eight warps expand operands and read
 * accumulators; a ninth issues the MMAs.  Per item each thread expands its
 * query row once into tensor memory (the MMAs' A operand, 2 x 128 rows x
 * 512 bytes).  The split's train rows stream through shared memory in tiles
 * of 64: each expanding thread loads its quarter of a row's 64 packed bytes
 * into registers one tile ahead and expands it into one of two 32 KB
 * operand buffers (K-major 8-row x 16-byte core matrices); the MMA warp then
 * issues the tile's 32 MMAs (two query halves x K 512 / 32, M 128, N 64)
 * into one of two pairs of 64-column TMEM accumulators; while they run,
 * every expanding warp takes the previous tile's accumulator of its query
 * half (warp w: TMEM lanes of quarter w % 4, half w / 4) through
 * tcgen05.ld.  Shared memory carries only the train operand: the query
 * operand, read by every MMA, stays in TMEM.  The roles hand over through
 * mbarriers only.  Each thread owns one query and keeps its top two as packed
 * (key, column) words, so equal distances keep the lower train index.  Every
 * mbarrier wait is bounded; a wait that runs out sets the error flag, every
 * role leaves its loop, and the CTA frees its TMEM after waiting (bounded)
 * for its last MMAs.
 */
#include <cuda_runtime.h>

#include "akz_device.cuh"

#define AKZ_TC_CWARPS 8                        /* expanding / epilogue warps; one more issues the MMAs */
#define AKZ_TC_CTHREADS (32 * AKZ_TC_CWARPS)
#define AKZ_TC_THREADS (AKZ_TC_CTHREADS + 32)
#define AKZ_TC_ITEM_COST 16                    /* fixed cost of an item, in tiles (split choice) */
#define AKZ_TC_Q 256                          /* queries per item */
#define AKZ_TC_N 64                           /* train rows per tile */
#define AKZ_TC_B_BYTES (AKZ_TC_N * 512)       /* one train tile */
#define AKZ_TC_STAGES 2                        /* train buffers = accumulator sets = barrier sets */
#define AKZ_TC_LAG (AKZ_TC_STAGES - 1)          /* tiles between a hand-over and its epilogue */
#define AKZ_TC_SMEM (AKZ_TC_STAGES * AKZ_TC_B_BYTES + 1024)
/* requested at launch: more than half an SM's shared memory, so that one CTA
 * per SM holds the whole TMEM (a second CTA's allocation would wait) */
#define AKZ_TC_SMEM_LAUNCH (AKZ_TC_SMEM > 120 * 1024 ? AKZ_TC_SMEM : 120 * 1024)
#define AKZ_TC_ACOL 256                        /* TMEM column of the query operand (half h: + 128 h) */
#define AKZ_TC_SPIN (1 << 24)

/* set when an MMA wait of k_match_tc ran out (read and cleared by
 * akz_matcher_tensor_status) */
__device__ int g_akz_tc_err;

struct akz_tc_top2 {
  int bd, bi, sd, si;
};

/* Shared-memory matrix descriptor of a K-major operand without swizzle. */
__device__ __forceinline__ uint64_t tc_smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46; /* descriptor version; base offset 0, no swizzle */
  return d;
}

/* kind::f8f6f4 instruction descriptor: D F32, A and B E4M3, both K-major */
__host__ __device__ constexpr uint32_t tc_idesc(int M, int N)
{
  return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ bool tc_mbar_wait(uint32_t mb, uint32_t parity)
{
  uint32_t done = 0;
  for (int it = 0; it < AKZ_TC_SPIN && !done; it++)
    asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
                 : "=r"(done)
                 : "r"(mb), "r"(parity)
                 : "memory");
  return done != 0;
}

/* The K order and the operand values.  Source byte i of a row (bits
 * b0..b7) gives K positions 8 i .. 8 i + 7 = bits 3, 4, 5, 6, 7, 0, 1, 2.
 * A train byte there is the source byte masked to that one bit, moved (for
 * bits 7, 0, 1, 2, by a nibble swap) to bit position 3, 4, 5 or 6: E4M3
 * 0x08, 0x10, 0x20, 0x40 = 2^-6, 2^-5, 2^-3, 2^1 when the bit is set, else
 * 0.  The query byte at the same K position is (1 - 2a) / w with w that
 * weight: 0x68, 0x60, 0x50, 0x30 = 64, 32, 8, 0.5, with the sign bit when
 * a = 1.  Every product is 0 or +-1 exactly.  The masked word is one
 * byte-permute and one AND per 4 K bytes. */
#define AKZ_TC_WMASK 0x40201008u /* bytes 0..3: bit 3, 4, 5, 6 */
#define AKZ_TC_QMAG 0x30506068u  /* bytes 0..3: 64, 32, 8, 0.5 */

__device__ __forceinline__ uint32_t tc_nibswap(uint32_t w)
{
  return ((w >> 4) & 0x0f0f0f0fu) | ((w << 4) & 0xf0f0f0f0u);
}

/* source word w (bytes 0..3) -> the 32 K bytes of its 4 bytes, as two
 * 16-byte chunks */
__device__ __forceinline__ void tc_expand_word(uint32_t w, bool query, uint4 &c0, uint4 &c1)
{
  const uint32_t y = tc_nibswap(w);
  uint32_t o[8];
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const uint32_t a = __byte_perm(w, 0, 0x1111u * (uint32_t)i) & AKZ_TC_WMASK;
    const uint32_t b = __byte_perm(y, 0, 0x1111u * (uint32_t)i) & AKZ_TC_WMASK;
    if (query) { /* a set bit (<= 0x40) plus 0x7f reaches bit 7, without carry into the next byte */
      o[2 * i] = AKZ_TC_QMAG | ((a + 0x7f7f7f7fu) & 0x80808080u);
      o[2 * i + 1] = AKZ_TC_QMAG | ((b + 0x7f7f7f7fu) & 0x80808080u);
    } else {
      o[2 * i] = a;
      o[2 * i + 1] = b;
    }
  }
  c0 = make_uint4(o[0], o[1], o[2], o[3]);
  c1 = make_uint4(o[4], o[5], o[6], o[7]);
}

/* Writes NW consecutive 32-bit words of a packed row (starting at word w0)
 * into an operand of `rows` rows: row r, K byte k at core matrix (r / 8,
 * k / 16), K-adjacent core matrices rows * 16 bytes apart (LBO), row-adjacent
 * 128 (SBO).  The 32 lanes of a warp take 32 consecutive rows: each 16-byte
 * store of the warp covers 512 contiguous bytes. */
template <int NW>
__device__ __forceinline__ void tc_expand_words(const uint32_t (&w)[NW], int r, int w0, int rows, unsigned char *op,
                                                bool query)
{
  const uint32_t ro = (uint32_t)((r >> 3) * 128 + (r & 7) * 16), kstride = (uint32_t)rows * 16;
#pragma unroll
  for (int m = 0; m < NW; m++) {
    const uint32_t c = (uint32_t)(2 * (w0 + m)); /* core column of the word's first 16 K bytes */
    uint4 c0, c1;
    tc_expand_word(w[m], query, c0, c1);
    *reinterpret_cast<uint4 *>(op + c * kstride + ro) = c0;
    *reinterpret_cast<uint4 *>(op + (c + 1) * kstride + ro) = c1;
  }
}

/* Waits (bounded) for phase `parity` of the mbarrier at mb; gives up early
 * when another thread of the CTA has flagged a failure, and flags one when
 * its own limit runs out. */
__device__ __forceinline__ bool tc_wait(uint32_t mb, uint32_t parity, volatile int *bad, int spin)
{
  for (int it = 0; it < spin; it++) {
    uint32_t done;
    asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
                 : "=r"(done)
                 : "r"(mb), "r"(parity)
                 : "memory");
    if (done) return true;
    if (*bad) return false;
  }
  *bad = 1;
  return false;
}

__device__ __forceinline__ void tc_arrive(uint32_t mb)
{
  asm volatile("{\n.reg .b64 st;\nmbarrier.arrive.shared::cta.b64 st, [%0];\n}" ::"r"(mb) : "memory");
}

/* 32 consecutive accumulator columns of this warp's 32 TMEM lanes (no wait) */
__device__ __forceinline__ void tc_ld32(uint32_t taddr, uint32_t (&r)[32])
{
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}

/* 32 consecutive TMEM columns of this warp's 32 lanes (no wait) */
__device__ __forceinline__ void tc_st32(uint32_t taddr, const uint32_t (&r)[32])
{
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
      "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]),
      "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]), "r"(r[16]), "r"(r[17]), "r"(r[18]),
      "r"(r[19]), "r"(r[20]), "r"(r[21]), "r"(r[22]), "r"(r[23]), "r"(r[24]), "r"(r[25]), "r"(r[26]), "r"(r[27]),
      "r"(r[28]), "r"(r[29]), "r"(r[30]), "r"(r[31])
      : "memory");
}

/* Running top two of one query as packed keys: (hamming - popc(q) + 512)
 * in bits 21..31, the column within the split in bits 0..20, so that the
 * unsigned order is the (distance, train index) order of the popc kernel
 * and min / max keep the lexicographic top two in any processing order.
 * kf is the float key of the second entry: a column whose value is not
 * below kf cannot enter. */
struct tc_top2 {
  uint32_t ub, us;
  float kf;
};

/* one 32-column half of a tile's accumulator row: v[cc] = key of column
 * col0 + cc; PART: columns cc >= lim lie past the split */
template <bool PART>
__device__ __forceinline__ void tc_scan32(const uint32_t (&r)[32], uint32_t col0, int lim, tc_top2 &st)
{
  /* (0x4B400000 + key) << 21 + BIAS = (key + 512) << 21 (mod 2^32) */
  constexpr uint32_t BIAS = (512u - 0x4B400000u) << 21;
  float m8[4];
#pragma unroll
  for (int g = 0; g < 4; g++) {
    float v[8];
#pragma unroll
    for (int e = 0; e < 8; e++) v[e] = __uint_as_float(r[8 * g + e]);
    m8[g] = fminf(fminf(fminf(v[0], v[1]), fminf(v[2], v[3])), fminf(fminf(v[4], v[5]), fminf(v[6], v[7])));
  }
  if (fminf(fminf(m8[0], m8[1]), fminf(m8[2], m8[3])) < st.kf) {
    const uint32_t cb = col0 + BIAS;
#pragma unroll
    for (int g = 0; g < 4; g++) {
      if (m8[g] < st.kf) {
#pragma unroll
        for (int e = 0; e < 8; e++) {
          const int cc = 8 * g + e;
          /* the key is an integer of magnitude <= 512: adding 1.5 * 2^23 puts it in the low mantissa bits */
          const uint32_t x = __float_as_uint(__uint_as_float(r[cc]) + 12582912.0f);
          uint32_t u = (x << 21) + cb + (uint32_t)cc;
          if (PART && cc >= lim) u = 0xffffffffu;
          const uint32_t hi = max(st.ub, u);
          st.ub = min(st.ub, u);
          st.us = min(st.us, hi);
        }
        st.kf = (float)((int)(st.us >> 21) - 512);
      }
    }
  }
}

/* Warp roles: warps 0..7 expand the operands and run the epilogue (warp w
 * owns TMEM lane quarter w % 4 of query half w / 4: its query rows of the
 * operand and its accumulator rows); warp 8 issues the MMAs (the whole warp
 * runs the loop, elect.sync picks the issuing lane).
 * TMEM: accumulator sets at columns 0..255 (set s, half h: 128 s + 64 h),
 * the expanded queries at 256..511 (half h: 256 + 128 h, 4 K bytes per
 * column).  Tile batch c over the CTA's lifetime uses stage c % 2: train
 * buffer, accumulator set and the barriers, at phase (c / 2) & 1:
 *   full:    each expanding warp arrives once its lanes have written the
 *            train tile (and, for an item's first tile, their query rows);
 *   done:    the MMA batch's commit;
 *   accfree: each expanding warp arrives once its lanes have read the
 *            batch's accumulators, which batch c + 2 overwrites.
 * The expanding warps read batch c - 1's accumulators after handing over
 * tile c.  A thread rewrites train buffer c % 2 only after it has seen batch
 * c - 2 done, and its query row (at an item's start) after every batch of
 * the previous item. */
__global__ void __launch_bounds__(AKZ_TC_THREADS, 1) k_match_tc(const uint4 *__restrict__ q, const uint4 *__restrict__ t,
                                                             int nq, int nt, int split_len, int nsplit,
                                                             akz_tc_top2 *partial, int4 *out, int spin, int no_mma)
{
  extern __shared__ __align__(1024) unsigned char tcsm[];
  unsigned char *base = tcsm + ((1024u - ((uint32_t)__cvta_generic_to_shared(tcsm) & 1023u)) & 1023u);
  unsigned char *sB = base; /* the train stages */
  __shared__ __align__(8) unsigned long long mbar[3 * AKZ_TC_STAGES]; /* full, done, accfree */
  __shared__ uint32_t tbase;
  __shared__ volatile int sBad;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (warp == 0) {
    const uint32_t dst = (uint32_t)__cvta_generic_to_shared(&tbase);
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(dst));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  const uint32_t mfull = (uint32_t)__cvta_generic_to_shared(&mbar[0]), mdone = mfull + 8u * AKZ_TC_STAGES,
                 mfree = mdone + 8u * AKZ_TC_STAGES;
  if (tid == 0) {
    for (int b = 0; b < AKZ_TC_STAGES; b++) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mfull + 8u * b), "r"(AKZ_TC_CWARPS));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mdone + 8u * b));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mfree + 8u * b), "r"(AKZ_TC_CWARPS));
    }
    asm volatile("fence.mbarrier_init.release.cluster;");
    sBad = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tbase;
  const uint32_t baddr = (uint32_t)__cvta_generic_to_shared(sB);
  const int nqb = (nq + AKZ_TC_Q - 1) / AKZ_TC_Q;
  const int nitems = nqb * nsplit;
  uint32_t committed = 0; /* MMA lane: batches committed */

  if (warp == AKZ_TC_CWARPS) {
    /* the whole warp runs the loop, so that the operands are warp-uniform;
     * elect.sync inside each asm picks the one lane that issues (a lone
     * lane's issue costs about twice as many cycles per MMA) */
    constexpr uint32_t idesc = tc_idesc(128, AKZ_TC_N);
    uint32_t c = 0;
    bool ok = true;
    for (int item = blockIdx.x; item < nitems && ok; item += gridDim.x) {
      const int sp = item / nqb;
      const int j0 = sp * split_len, j1 = min(nt, j0 + split_len);
      const int ntile = j1 > j0 ? (j1 - j0 + AKZ_TC_N - 1) / AKZ_TC_N : 0;
      for (int k = 0; k < ntile; k++, c++) {
        const uint32_t st = c % AKZ_TC_STAGES, ph = (c / AKZ_TC_STAGES) & 1u;
        ok = __all_sync(0xffffffffu, tc_wait(mfull + 8u * st, ph, &sBad, spin));
        if (ok && c >= AKZ_TC_STAGES) ok = __all_sync(0xffffffffu, tc_wait(mfree + 8u * st, ph ^ 1u, &sBad, spin));
        if (no_mma) ok = false; /* self-check: no batch is ever committed */
        if (!ok) {
          if (!no_mma) sBad = 1; /* (the self-check leaves the timeout to the epilogue's wait) */
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t bb = baddr + st * (uint32_t)AKZ_TC_B_BYTES;
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const uint32_t d = tmem + (st * 2u + (uint32_t)h) * AKZ_TC_N;
          const uint32_t ah = tmem + (uint32_t)(AKZ_TC_ACOL + 128 * h);
#pragma unroll
          for (int s = 0; s < 16; s++) { /* K step s: bytes 32 s .. 32 s + 31: A columns 8 s .. 8 s + 7, B two core columns */
            const uint64_t bd = tc_smem_desc(bb + (uint32_t)(s * 2048), 1024, 128);
            const uint32_t acc = s > 0 ? 1u : 0u;
            asm volatile(
                "{\n.reg .pred p, e;\nsetp.ne.b32 p, %4, 0;\nelect.sync _|e, 0xffffffff;\n"
                "@e tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], [%1], %2, %3, p;\n}" ::"r"(d),
                "r"(ah + 8u * (uint32_t)s), "l"(bd), "r"(idesc), "r"(acc));
          }
        }
        asm volatile(
            "{\n.reg .pred e;\nelect.sync _|e, 0xffffffff;\n"
            "@e tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n}" ::"r"(mdone + 8u * st));
        committed = c + 1;
      }
    }
  } else {
    const int quarter = warp & 3, qh = warp >> 2; /* TMEM lane quarter, query half */
    /* expansion roles: train tiles, row er = tid % 64 and words 4 eh .. 4 eh + 3 */
    const int er = tid & 63, eh = tid >> 6;
    uint32_t c = 0;
    for (int item = blockIdx.x; item < nitems && !sBad; item += gridDim.x) {
      const int qb = item % nqb, sp = item / nqb;
      const int j0 = sp * split_len, j1 = min(nt, j0 + split_len);
      const int ntile = j1 > j0 ? (j1 - j0 + AKZ_TC_N - 1) / AKZ_TC_N : 0;
      const int myq = qb * AKZ_TC_Q + qh * 128 + quarter * 32 + lane; /* this thread's query */

      auto load_tile = [&](int k, uint4 &v) { /* row er of tile k, words 4 eh .. 4 eh + 3; zeros past the split */
        const int j = j0 + k * AKZ_TC_N + er;
        v = j < j1 ? __ldg(t + (long long)j * 4 + eh) : make_uint4(0, 0, 0, 0);
      };
      uint4 cur = make_uint4(0, 0, 0, 0), nxt = cur;
      if (ntile > 0) {
        load_tile(0, cur);
        /* this thread's query row into its TMEM lane of the query operand:
         * source word m -> columns 8 m .. 8 m + 7 (K bytes 32 m .. 32 m + 31) */
        uint4 qv[4];
#pragma unroll
        for (int w = 0; w < 4; w++) qv[w] = myq < nq ? __ldg(q + (long long)myq * 4 + w) : make_uint4(0, 0, 0, 0);
        const uint32_t ta = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(AKZ_TC_ACOL + 128 * qh);
#pragma unroll
        for (int w = 0; w < 4; w++) {
          const uint32_t src[4] = {qv[w].x, qv[w].y, qv[w].z, qv[w].w};
          uint32_t o[32];
#pragma unroll
          for (int m = 0; m < 4; m++) {
            uint4 c0, c1;
            tc_expand_word(src[m], true, c0, c1);
            o[8 * m] = c0.x, o[8 * m + 1] = c0.y, o[8 * m + 2] = c0.z, o[8 * m + 3] = c0.w;
            o[8 * m + 4] = c1.x, o[8 * m + 5] = c1.y, o[8 * m + 6] = c1.z, o[8 * m + 7] = c1.w;
          }
          tc_st32(ta + 32u * (uint32_t)w, o);
        }
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
      }
      int pq = 0;
      if (myq < nq) {
#pragma unroll
        for (int w = 0; w < 4; w++) {
          const uint4 v = __ldg(q + (long long)myq * 4 + w);
          pq += __popc(v.x) + __popc(v.y) + __popc(v.z) + __popc(v.w);
        }
      }
      tc_top2 top; /* both entries start as {distance 512, index 0} */
      top.ub = top.us = (uint32_t)(1024 - pq) << 21;
      top.kf = (float)(512 - pq);

      auto epilogue = [&](uint32_t cb, int k) -> bool { /* batch cb = tile k of this item */
        const uint32_t st = cb % AKZ_TC_STAGES;
        /* tcgen05.ld is warp-collective: the warp goes on only if every lane saw the batch done */
        if (!__all_sync(0xffffffffu, tc_wait(mdone + 8u * st, (cb / AKZ_TC_STAGES) & 1u, &sBad, spin))) {
          sBad = 1;
          return false;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        uint32_t r0[32], r1[32];
        const uint32_t taddr = tmem + ((uint32_t)(quarter * 32) << 16) + (st * 2u + (uint32_t)qh) * AKZ_TC_N;
        tc_ld32(taddr, r0);
        tc_ld32(taddr + 32u, r1);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncwarp();
        if (lane == 0) tc_arrive(mfree + 8u * st);
        const int lim = j1 - (j0 + k * AKZ_TC_N);
        const uint32_t col0 = (uint32_t)(k * AKZ_TC_N);
        if (lim >= AKZ_TC_N) {
          tc_scan32<false>(r0, col0, lim, top);
          tc_scan32<false>(r1, col0 + 32u, lim - 32, top);
        } else {
          tc_scan32<true>(r0, col0, lim, top);
          tc_scan32<true>(r1, col0 + 32u, lim - 32, top);
        }
        return true;
      };

      /* tile k: expand, hand over, then read batch c - 1's accumulators */
      auto step = [&](int k, const uint4 &v) -> bool {
        {
          const uint32_t w[4] = {v.x, v.y, v.z, v.w};
          tc_expand_words<4>(w, er, 4 * eh, AKZ_TC_N, sB + (c % AKZ_TC_STAGES) * AKZ_TC_B_BYTES, false);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncwarp();
        if (lane == 0) tc_arrive(mfull + 8u * (c % AKZ_TC_STAGES));
        const bool r = k < AKZ_TC_LAG || epilogue(c - AKZ_TC_LAG, k - AKZ_TC_LAG);
        c++;
        return r;
      };
      /* two register sets in turn: each tile's rows are loaded one step ahead
       * and used where they landed, with no copy that would wait for them */
      bool ok = true;
      for (int k = 0; k < ntile && ok; k += 2) {
        if (k + 1 < ntile) load_tile(k + 1, nxt);
        ok = step(k, cur);
        if (!ok || k + 1 >= ntile) break;
        if (k + 2 < ntile) load_tile(k + 2, cur);
        ok = step(k + 1, nxt);
      }
      if (!ok) break;
      for (int k = max(0, ntile - AKZ_TC_LAG); k < ntile && ok; k++) ok = epilogue(c - (uint32_t)(ntile - k), k);
      if (!ok) break;
      if (myq < nq) {
        const int bd = pq + (int)(top.ub >> 21) - 512, sd = pq + (int)(top.us >> 21) - 512;
        const int bi = j0 + (int)(top.ub & 0x1fffffu), si = j0 + (int)(top.us & 0x1fffffu);
        if (nsplit == 1) {
          out[2 * myq] = make_int4(myq, bi, 0, __float_as_int((float)bd));
          out[2 * myq + 1] = make_int4(myq, si, 0, __float_as_int((float)sd));
        } else {
          partial[(long long)myq * nsplit + sp] = akz_tc_top2{bd, bi, sd, si};
        }
      }
    }
  }
  if (warp == AKZ_TC_CWARPS && committed > 0) {
    /* every batch's MMAs finished before the CTA frees TMEM and exits; on
     * the normal path the epilogue has already seen the last one */
    const uint32_t cp = committed - 1;
    tc_mbar_wait(mdone + 8u * (cp % AKZ_TC_STAGES), (cp / AKZ_TC_STAGES) & 1u);
  }
  if (tid == 0 && sBad) atomicExch(&g_akz_tc_err, 1);
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem));
}

/* Train splits for the tensor path: items of 256 queries x one split are
 * spread over one CTA per SM, so the cost is waves x (tiles per split + a
 * fixed cost per item: the query expansion, and the first columns of a split,
 * where the top two change often).  A split's columns must fit 21 bits. */
int akz_match_tc_splits(int nq, int nt, int nsm)
{
  const long long nqb = (nq + AKZ_TC_Q - 1) / AKZ_TC_Q;
  const int smax = (1 << 21) - 1;
  const int min_s = nt > smax ? (nt + smax - 1) / smax : 1;
  int best = min_s;
  long long bestc = -1;
  for (int ns = min_s; ns <= 64; ns++) {
    const long long len = ((long long)nt + ns - 1) / ns;
    if (ns > min_s && len < 4 * AKZ_TC_N) break;
    const long long waves = (nqb * ns + nsm - 1) / nsm;
    const long long cost = waves * ((len + AKZ_TC_N - 1) / AKZ_TC_N + AKZ_TC_ITEM_COST);
    if (bestc < 0 || cost < bestc) {
      bestc = cost;
      best = ns;
    }
  }
  return best;
}

/* Launches k_match_tc over nq queries and nt >= 1 train rows split in nsplit
 * parts (split length < 2^21), at most one CTA per SM; with nsplit > 1 the
 * caller merges partial (nq x nsplit records in the popc kernel's akz_top2
 * layout). */
cudaError_t akz_match_tc_launch(const void *dq, int nq, const void *dt, int nt, void *dout, void *partial, int nsplit,
                                int nsm, cudaStream_t s, int spin, int no_mma)
{
  const int split_len = (nt + nsplit - 1) / nsplit;
  if (split_len >= (1 << 21)) return cudaErrorInvalidValue;
  const int nitems = ((nq + AKZ_TC_Q - 1) / AKZ_TC_Q) * nsplit;
  const int grid = nitems < nsm ? nitems : nsm;
  cudaError_t e =
      cudaFuncSetAttribute(k_match_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)AKZ_TC_SMEM_LAUNCH);
  if (e != cudaSuccess) return e;
  k_match_tc<<<grid, AKZ_TC_THREADS, AKZ_TC_SMEM_LAUNCH, s>>>((const uint4 *)dq, (const uint4 *)dt, nq, nt, split_len,
                                                             nsplit, (akz_tc_top2 *)partial, (int4 *)dout,
                                                             spin > 0 ? spin : AKZ_TC_SPIN, no_mma);
  return cudaGetLastError();
}

/* reads and clears the timeout flag (synchronous) */
cudaError_t akz_match_tc_status(int *timed_out)
{
  int v = 0, z = 0;
  cudaError_t e = cudaMemcpyFromSymbol(&v, g_akz_tc_err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_akz_tc_err, &z, sizeof(int));
  *timed_out = v;
  return e;
}
