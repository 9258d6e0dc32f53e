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
 * Query rows are expanded to E4M3 values 1 - 2a in {+1, -1}, train rows to
 * b in {0, +1}; one K = 512 product per pair gives the sums, exact in the FP32
 * accumulator (integers of magnitude <= 512).  The epilogue keeps the running
 * best and second best per query in train order with strict <, so equal
 * distances keep the lower train index (the cv::BFMatcher rule of the popc
 * kernel); the initial entry is {distance 512, index 0}, as there.
 *
 * A CTA (8 warps, one per SM: it holds 256 TMEM columns) loops over work
 * items of 256 queries x one train split.  Per item the queries are expanded
 * once into shared memory (two 64 KB operands of 128 rows, K-major 8-row x
 * 16-byte core matrices).  The split's train rows stream through in tiles of
 * 64: each thread loads its quarter of a row's 64 packed bytes into
 * registers one tile ahead and expands it into one of two 32 KB operand
 * buffers; one thread then issues the tile's 32 MMAs (two query halves x
 * K 512 / 32, M 128, N 64) into one of two pairs of 64-column TMEM
 * accumulators; while they run, every warp takes the previous tile's
 * accumulator of its query half (warp w: TMEM lanes of quarter w % 4, half
 * w / 4) through tcgen05.ld.  Each thread owns one query and sees every
 * train column in order.  Every mbarrier wait is bounded; a wait that runs
 * out sets the error flag, ends the loop, and the CTA frees its TMEM after
 * waiting (bounded) for its last MMAs.
 */
#include <cuda_runtime.h>

#include "akz_device.cuh"

#define AKZ_TC_THREADS 256
#define AKZ_TC_Q 256                          /* queries per item */
#define AKZ_TC_N 64                           /* train rows per tile */
#define AKZ_TC_A_BYTES (128 * 512)            /* one query half: 128 rows x 512 E4M3 values */
#define AKZ_TC_B_BYTES (AKZ_TC_N * 512)       /* one train tile */
#define AKZ_TC_SMEM (2 * AKZ_TC_A_BYTES + 2 * AKZ_TC_B_BYTES + 1024)
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

/* 16 row bits -> 16 E4M3 bytes: train 0 / +1 (0x38), query +1 / -1 (0x38 / 0xB8) */
__device__ __forceinline__ uint4 tc_expand16(uint32_t bits, bool query)
{
  uint32_t w[4];
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const uint32_t ones = (((bits >> (4 * i)) & 15u) * 0x00204081u) & 0x01010101u; /* byte j = bit 4i + j */
    w[i] = query ? (0x38383838u | (ones << 7)) : ones * 0x38u;
  }
  return make_uint4(w[0], w[1], w[2], w[3]);
}

/* Writes nw consecutive 32-bit words of a packed row (starting at word w0)
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
    const uint32_t c = (uint32_t)(2 * (w0 + m)); /* core column of the word's first 16 bits */
    *reinterpret_cast<uint4 *>(op + c * kstride + ro) = tc_expand16(w[m] & 0xffffu, query);
    *reinterpret_cast<uint4 *>(op + (c + 1) * kstride + ro) = tc_expand16(w[m] >> 16, query);
  }
}

__global__ void __launch_bounds__(AKZ_TC_THREADS, 1) k_match_tc(const uint4 *__restrict__ q, const uint4 *__restrict__ t,
                                                             int nq, int nt, int split_len, int nsplit,
                                                             akz_tc_top2 *partial, int4 *out)
{
  extern __shared__ __align__(1024) unsigned char tcsm[];
  unsigned char *base = tcsm + ((1024u - ((uint32_t)__cvta_generic_to_shared(tcsm) & 1023u)) & 1023u);
  unsigned char *sA = base, *sB = base + 2 * AKZ_TC_A_BYTES; /* sA: halves 0 and 1; sB: tiles 0 and 1 */
  __shared__ __align__(8) unsigned long long mbar[2];
  __shared__ uint32_t tbase;
  __shared__ int sBad;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int quarter = warp & 3, qh = warp >> 2; /* TMEM lane quarter, query half */

  if (warp == 0) {
    const uint32_t dst = (uint32_t)__cvta_generic_to_shared(&tbase);
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(dst));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int b = 0; b < 2; b++)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"((uint32_t)__cvta_generic_to_shared(&mbar[b])));
    asm volatile("fence.mbarrier_init.release.cluster;");
    sBad = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tbase;
  constexpr uint32_t idesc = tc_idesc(128, AKZ_TC_N);
  const uint32_t aaddr = (uint32_t)__cvta_generic_to_shared(sA), baddr = (uint32_t)__cvta_generic_to_shared(sB);
  const uint32_t mb0 = (uint32_t)__cvta_generic_to_shared(&mbar[0]);
  /* MMA batches (one per tile) committed by thread 0 / seen complete, over
   * the CTA's lifetime: batch c uses mbar[c & 1], phase (c >> 1) & 1 */
  uint32_t issued = 0, committed = 0, retired = 0;
  bool ok = true;

  const int nqb = (nq + AKZ_TC_Q - 1) / AKZ_TC_Q;
  const int nitems = nqb * nsplit;
  /* expansion roles: train tiles, row er = tid % 64 and words 4 eh .. 4 eh + 3 */
  const int er = tid & 63, eh = tid >> 6;
  for (int item = blockIdx.x; item < nitems && ok; item += gridDim.x) {
    const int qb = item % nqb, sp = item / nqb;
    const int j0 = sp * split_len, j1 = min(nt, j0 + split_len);
    const int ntile = j1 > j0 ? (j1 - j0 + AKZ_TC_N - 1) / AKZ_TC_N : 0;
    const int myq = qb * AKZ_TC_Q + qh * 128 + quarter * 32 + lane; /* this thread's query */

    auto load_tile = [&](int k, uint4 &v) { /* row er of tile k, words 4 eh .. 4 eh + 3; zeros past the split */
      const int j = j0 + k * AKZ_TC_N + er;
      v = j < j1 ? __ldg(t + (long long)j * 4 + eh) : make_uint4(0, 0, 0, 0);
    };
    uint4 cur = make_uint4(0, 0, 0, 0), nxt = cur;
    if (ntile > 0) load_tile(0, cur);
    { /* the 256 queries: thread i expands rows i % 128 of both halves, words 8 (i / 128) .. + 7 */
      const int r = tid & 127, h = tid >> 7;
#pragma unroll
      for (int half = 0; half < 2; half++) {
        const int qi = qb * AKZ_TC_Q + half * 128 + r;
        uint4 a = make_uint4(0, 0, 0, 0), b = a;
        if (qi < nq) {
          a = __ldg(q + (long long)qi * 4 + 2 * h);
          b = __ldg(q + (long long)qi * 4 + 2 * h + 1);
        }
        const uint32_t w[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
        tc_expand_words<8>(w, r, 8 * h, 128, sA + half * AKZ_TC_A_BYTES, true);
      }
    }
    int pq = 0;
    if (myq < nq) {
#pragma unroll
      for (int c = 0; c < 4; c++) {
        const uint4 v = __ldg(q + (long long)myq * 4 + c);
        pq += __popc(v.x) + __popc(v.y) + __popc(v.z) + __popc(v.w);
      }
    }
    float bk = (float)(512 - pq), sk = bk; /* keys: hamming - popc(q) */
    int bi = 0, si = 0;

    auto epilogue = [&](uint32_t c, int k) { /* batch c = tile k's accumulators */
      const int jt = j0 + k * AKZ_TC_N;
      const int lim0 = j1 - jt;
#pragma unroll
      for (int h = 0; h < 2; h++) {
        uint32_t r[32];
        const uint32_t taddr =
            tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)((((c & 1u) * 2u + (uint32_t)qh) * AKZ_TC_N) + 32 * h);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
              "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]),
              "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
              "=r"(r[30]), "=r"(r[31])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;");
        const int lim = lim0 - 32 * h; /* columns past the split are not candidates */
#pragma unroll
        for (int cc = 0; cc < 32; cc++) {
          const float v = __uint_as_float(r[cc]);
          if (cc < lim && v < sk) {
            const int j = jt + 32 * h + cc;
            if (v < bk) {
              sk = bk;
              si = bi;
              bk = v;
              bi = j;
            } else {
              sk = v;
              si = j;
            }
          }
        }
      }
    };

    for (int k = 0; k < ntile; k++) {
      if (k + 1 < ntile) load_tile(k + 1, nxt); /* in flight while tile k is expanded */
      /* operand buffer k & 1: its last reader, tile k - 2's MMAs, retired before tile k - 1's barrier */
      {
        const uint32_t w[4] = {cur.x, cur.y, cur.z, cur.w};
        tc_expand_words<4>(w, er, 4 * eh, AKZ_TC_N, sB + (k & 1) * AKZ_TC_B_BYTES, false);
      }
      cur = nxt;
      asm volatile("fence.proxy.async.shared::cta;");
      asm volatile("tcgen05.fence::before_thread_sync;");
      __syncthreads();
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t c = issued++;
      if (tid == 0) {
        const uint32_t bb = baddr + (uint32_t)((k & 1) * AKZ_TC_B_BYTES);
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const uint32_t d = tmem + (uint32_t)(((c & 1u) * 2u + (uint32_t)h) * AKZ_TC_N);
          const uint32_t ah = aaddr + (uint32_t)(h * AKZ_TC_A_BYTES);
#pragma unroll
          for (int s = 0; s < 16; s++) { /* K step s: bytes 32 s .. 32 s + 31, two core columns */
            const uint64_t ad = tc_smem_desc(ah + (uint32_t)(s * 4096), 2048, 128);
            const uint64_t bd = tc_smem_desc(bb + (uint32_t)(s * 2048), 1024, 128);
            const uint32_t acc = s > 0 ? 1u : 0u;
            asm volatile(
                "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}" ::"r"(d),
                "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
          }
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mb0 + 8u * (c & 1u)));
        committed = c + 1;
      }
      if (k >= 1) { /* tile k - 1's accumulators while tile k's MMAs run */
        const uint32_t cp = c - 1;
        if (!tc_mbar_wait(mb0 + 8u * (cp & 1u), (cp >> 1) & 1u)) {
          sBad = 1;
        } else {
          retired = cp + 1;
          asm volatile("tcgen05.fence::after_thread_sync;");
          epilogue(cp, k - 1);
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      __syncthreads();
      if (sBad) {
        ok = false;
        break;
      }
    }
    if (!ok) break;
    if (ntile > 0) { /* the last tile */
      const uint32_t cp = issued - 1;
      if (!tc_mbar_wait(mb0 + 8u * (cp & 1u), (cp >> 1) & 1u)) {
        sBad = 1;
      } else {
        retired = cp + 1;
        asm volatile("tcgen05.fence::after_thread_sync;");
        epilogue(cp, ntile - 1);
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads(); /* sA and the accumulators are reused by the next item */
    if (sBad) {
      ok = false;
      break;
    }
    if (myq < nq) {
      const int bd = pq + (int)bk, sd = pq + (int)sk;
      if (nsplit == 1) {
        out[2 * myq] = make_int4(myq, bi, 0, __float_as_int((float)bd));
        out[2 * myq + 1] = make_int4(myq, si, 0, __float_as_int((float)sd));
      } else {
        partial[(long long)myq * nsplit + sp] = akz_tc_top2{bd, bi, sd, si};
      }
    }
  }
  if (!ok && tid == 0) {
    atomicExch(&g_akz_tc_err, 1);
    if (retired < committed) { /* batches complete in order: wait (bounded) for the last one */
      const uint32_t cp = committed - 1;
      tc_mbar_wait(mb0 + 8u * (cp & 1u), (cp >> 1) & 1u);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tmem));
}

/* Launches k_match_tc over nq queries and nt >= 1 train rows split in nsplit
 * parts, at most one CTA per SM; with nsplit > 1 the caller merges partial
 * (nq x nsplit records in the popc kernel's akz_top2 layout). */
cudaError_t akz_match_tc_launch(const void *dq, int nq, const void *dt, int nt, void *dout, void *partial, int nsplit,
                                int nsm, cudaStream_t s)
{
  const int split_len = (nt + nsplit - 1) / nsplit;
  const int nitems = ((nq + AKZ_TC_Q - 1) / AKZ_TC_Q) * nsplit;
  const int grid = nitems < nsm ? nitems : nsm;
  cudaError_t e = cudaFuncSetAttribute(k_match_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)AKZ_TC_SMEM);
  if (e != cudaSuccess) return e;
  k_match_tc<<<grid, AKZ_TC_THREADS, AKZ_TC_SMEM, s>>>((const uint4 *)dq, (const uint4 *)dt, nq, nt, split_len, nsplit,
                                                      (akz_tc_top2 *)partial, (int4 *)dout);
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
