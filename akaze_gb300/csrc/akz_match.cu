/*
 * akz_match.cu - brute-force 2-NN Hamming matcher on 64-byte rows.
 *
 * Reference: MatchDescriptors, cuda_akaze.cu:1843-1967, and Matcher::bfmatch,
 * AKAZE.cpp:36-79.  For every query the closest and second-closest train rows
 * by Hamming distance; equal distances go to the lower train index (the
 * cv::BFMatcher knnMatch rule), a missing candidate is {trainIdx 0,
 * distance 512}.
 *
 * Layout: one query per thread (its 512 bits in 16 registers), train rows
 * staged through shared memory 256 at a time and read as broadcasts, 16
 * xor+popc per pair.  The train set is split across blockIdx.y so that small
 * query sets still fill the GPU; the per-split top-2 lists are merged in
 * split order with a (distance, index) comparison, which equals one
 * sequential scan.
 */
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/akaze_gb300.h"
#include "akz_device.cuh"

akz_status akz_report(akz_status s, const char *msg);

#define AKZ_MQ 256
#define AKZ_MT 256

struct akz_top2 {
  int bd, bi, sd, si;
};

__device__ __forceinline__ bool akz_lex_less(int d1, int i1, int d2, int i2) { return d1 < d2 || (d1 == d2 && i1 < i2); }

__global__ void __launch_bounds__(AKZ_MQ) k_match(const uint4 *__restrict__ q, const uint4 *__restrict__ t, int nq, int nt,
                                                  int split_len, int nsplit, akz_top2 *partial, int4 *out)
{
  __shared__ uint4 sT[AKZ_MT * 4];
  const int qi = blockIdx.x * AKZ_MQ + threadIdx.x;
  uint4 a0 = make_uint4(0, 0, 0, 0), a1 = a0, a2 = a0, a3 = a0;
  if (qi < nq) {
    a0 = __ldg(q + (long long)qi * 4 + 0);
    a1 = __ldg(q + (long long)qi * 4 + 1);
    a2 = __ldg(q + (long long)qi * 4 + 2);
    a3 = __ldg(q + (long long)qi * 4 + 3);
  }
  const int j0 = blockIdx.y * split_len, j1 = min(nt, j0 + split_len);
  int bd = 512, bi = 0, sd = 512, si = 0;
  for (int tile = j0; tile < j1; tile += AKZ_MT) {
    const int cnt = min(AKZ_MT, j1 - tile);
    __syncthreads();
    for (int i = threadIdx.x; i < cnt * 4; i += AKZ_MQ) sT[i] = __ldg(t + (long long)tile * 4 + i);
    __syncthreads();
#pragma unroll 4
    for (int r = 0; r < cnt; r++) {
      const uint4 b0 = sT[r * 4 + 0], b1 = sT[r * 4 + 1], b2 = sT[r * 4 + 2], b3 = sT[r * 4 + 3];
      int d = __popc(a0.x ^ b0.x) + __popc(a0.y ^ b0.y) + __popc(a0.z ^ b0.z) + __popc(a0.w ^ b0.w);
      d += __popc(a1.x ^ b1.x) + __popc(a1.y ^ b1.y) + __popc(a1.z ^ b1.z) + __popc(a1.w ^ b1.w);
      d += __popc(a2.x ^ b2.x) + __popc(a2.y ^ b2.y) + __popc(a2.z ^ b2.z) + __popc(a2.w ^ b2.w);
      d += __popc(a3.x ^ b3.x) + __popc(a3.y ^ b3.y) + __popc(a3.z ^ b3.z) + __popc(a3.w ^ b3.w);
      const int j = tile + r;
      if (d < bd) {
        sd = bd;
        si = bi;
        bd = d;
        bi = j;
      } else if (d < sd) {
        sd = d;
        si = j;
      }
    }
  }
  if (qi >= nq) return;
  if (nsplit == 1) {
    out[2 * qi] = make_int4(qi, bi, 0, __float_as_int((float)bd));
    out[2 * qi + 1] = make_int4(qi, si, 0, __float_as_int((float)sd));
  } else {
    partial[(long long)qi * nsplit + blockIdx.y] = akz_top2{bd, bi, sd, si};
  }
}

__global__ void k_match_merge(const akz_top2 *partial, int nq, int nsplit, int4 *out)
{
  const int qi = blockIdx.x * blockDim.x + threadIdx.x;
  if (qi >= nq) return;
  akz_top2 r = partial[(long long)qi * nsplit];
  for (int s = 1; s < nsplit; s++) {
    const akz_top2 o = partial[(long long)qi * nsplit + s];
    /* candidates: r.b, r.s, o.b, o.s ; r entries come from lower indices */
    int c[4][2] = {{r.bd, r.bi}, {r.sd, r.si}, {o.bd, o.bi}, {o.sd, o.si}};
    int b = 0;
    for (int k = 1; k < 4; k++)
      if (akz_lex_less(c[k][0], c[k][1], c[b][0], c[b][1])) b = k;
    int s2 = b == 0 ? 1 : 0;
    for (int k = 0; k < 4; k++)
      if (k != b && akz_lex_less(c[k][0], c[k][1], c[s2][0], c[s2][1])) s2 = k;
    r = akz_top2{c[b][0], c[b][1], c[s2][0], c[s2][1]};
  }
  out[2 * qi] = make_int4(qi, r.bi, 0, __float_as_int((float)r.bd));
  out[2 * qi + 1] = make_int4(qi, r.si, 0, __float_as_int((float)r.sd));
}

cudaError_t akz_match_tc_launch(const void *dq, int nq, const void *dt, int nt, void *dout, void *partial, int nsplit,
                                int nsm, cudaStream_t s, int spin, int no_mma);
cudaError_t akz_match_tc_status(int *timed_out);
int akz_match_tc_splits(int nq, int nt, int nsm);

/* Process-wide choice of the pair-distance engine for large calls: the
 * tensor-core kernels (akz_match_tc.cu, on by default) or xor + popc. */
static int g_akz_match_tc_on = 1;
#define AKZ_TC_MIN_PAIRS (1LL << 20) /* below ~1 M pairs one popc launch is latency-bound either way */

static bool akz_match_tensor_path(int nq, int nt)
{
  return g_akz_match_tc_on && nt >= 128 && (long long)nq * nt >= AKZ_TC_MIN_PAIRS;
}

/* out: 2*nq records {queryIdx, trainIdx, imgIdx, distance(float bits)};
 * partial: scratch of nq*nsplit top-2 records (may be null when nsplit==1). */
cudaError_t akz_match_run(const void *dq, int nq, const void *dt, int nt, void *dout, void *partial, int nsplit, cudaStream_t s)
{
  if (nq <= 0) return cudaSuccess;
  if (nsplit < 1) nsplit = 1;
  if (akz_match_tensor_path(nq, nt) && (nt + nsplit - 1) / nsplit < (1 << 21)) {
    int dev = 0, nsm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = akz_match_tc_launch(dq, nq, dt, nt, dout, partial, nsplit, nsm, s, 0, 0);
    if (e != cudaSuccess || nsplit == 1) return e;
    k_match_merge<<<(nq + 255) / 256, 256, 0, s>>>((const akz_top2 *)partial, nq, nsplit, (int4 *)dout);
    return cudaGetLastError();
  }
  const int split_len = nt > 0 ? (nt + nsplit - 1) / nsplit : 0;
  const dim3 grid((nq + AKZ_MQ - 1) / AKZ_MQ, nsplit);
  k_match<<<grid, AKZ_MQ, 0, s>>>((const uint4 *)dq, (const uint4 *)dt, nq, nt, split_len, nsplit, (akz_top2 *)partial,
                                  (int4 *)dout);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || nsplit == 1) return e;
  k_match_merge<<<(nq + 255) / 256, 256, 0, s>>>((const akz_top2 *)partial, nq, nsplit, (int4 *)dout);
  return cudaGetLastError();
}

/* Number of train splits.  Tensor path: akz_match_tc_splits (whole waves of
 * 256-query items).  Popc path: about 4 CTAs per SM, with at least 64 train
 * rows per split: a small query set is otherwise a handful of CTAs each
 * walking the whole train set, bound by the latency of one row. */
int akz_match_splits(int nq, int nt, int nsm)
{
  if (akz_match_tensor_path(nq, nt)) return akz_match_tc_splits(nq, nt, nsm);
  const int qb = (nq + AKZ_MQ - 1) / AKZ_MQ;
  int ns = (4 * nsm + qb - 1) / qb;
  const int maxs = (nt + 63) / 64;
  if (ns > maxs) ns = maxs;
  if (ns < 1) ns = 1;
  return ns;
}

size_t akz_match_partial_bytes(int nq, int nsplit) { return (size_t)nq * nsplit * sizeof(akz_top2); }

/* ------------------------------------------------------------------------ */
/* Allocation-free 2-NN match.
 *
 * For callers that cannot call cudaMalloc: a plugin that runs inside a host
 * application which owns all device memory and hands out fixed buffers (a
 * video or inference pipeline with a planned memory budget), or code on a
 * latency-critical path where an allocation would synchronise the device.
 * The caller passes the query and train rows and the output in device
 * memory; the per-split top-2 scratch lives in the library's own
 * statically sized device array below, so the call allocates nothing.
 *
 * Limit: nq * splits top-2 records must fit the array, i.e. at most
 * AKZ_NOALLOC_MAX_RECORDS (131072) query rows per call; larger nq is
 * rejected with AKZ_ERR_INVALID_ARG.  Every GPU that loads the library holds
 * the array (2 MiB) until the process exits.  All calls share it: each call
 * rewrites every record it reads (nothing needs to start at zero), and calls
 * whose kernels overlap on the GPU (different streams, or another host
 * thread) race on it and must be serialised by the caller.
 */
#define AKZ_NOALLOC_MAX_RECORDS 131072
#define AKZ_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) akz_top2 g_akz_noalloc_scratch[AKZ_NOALLOC_MAX_RECORDS];

static std::mutex g_noalloc_mutex;
static void *g_noalloc_addr[AKZ_NOALLOC_MAX_DEVICES];
static int g_noalloc_sms[AKZ_NOALLOC_MAX_DEVICES];

/* Device address of the scratch array on the current device, resolved once
 * per device (host code cannot use the symbol itself as a device pointer).
 * The address is kept for the life of the process; a cudaDeviceReset
 * invalidates it, so the entry point is not for use after a reset. */
static cudaError_t akz_noalloc_setup(int *dev_out, void **addr, int *nsm)
{
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= AKZ_NOALLOC_MAX_DEVICES) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_addr[dev]) {
    void *ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_akz_noalloc_scratch);
    if (e != cudaSuccess) return e;
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    g_noalloc_sms[dev] = sms;
    g_noalloc_addr[dev] = ptr;
  }
  *dev_out = dev;
  *addr = g_noalloc_addr[dev];
  *nsm = g_noalloc_sms[dev];
  return cudaSuccess;
}

extern "C" AKZ_API akz_status akz_matcher_bfmatch_noalloc(const uint8_t *query64, int nq, const uint8_t *train64, int nt,
                                                         akz_dmatch *out, void *stream)
{
  if (nq < 0 || nt < 0) return akz_report(AKZ_ERR_INVALID_ARG, "akz_matcher_bfmatch_noalloc: negative size");
  if (nq > AKZ_NOALLOC_MAX_RECORDS)
    return akz_report(AKZ_ERR_INVALID_ARG,
                      "akz_matcher_bfmatch_noalloc: more than 131072 query rows (the fixed scratch limit); "
                      "use akz_matcher_bfmatch_device");
  if (nq == 0) return AKZ_OK;
  if (!query64 || !out || (nt > 0 && !train64))
    return akz_report(AKZ_ERR_INVALID_ARG, "akz_matcher_bfmatch_noalloc: NULL device buffer");
  int dev = 0, nsm = 0;
  void *scratch = nullptr;
  cudaError_t e = akz_noalloc_setup(&dev, &scratch, &nsm);
  if (e != cudaSuccess) return akz_report(AKZ_ERR_CUDA, cudaGetErrorString(e));
  int ns = akz_match_splits(nq, nt, nsm);
  const int fit = AKZ_NOALLOC_MAX_RECORDS / nq;
  if (ns > fit) ns = fit;
  e = akz_match_run(query64, nq, train64, nt, out, scratch, ns, (cudaStream_t)stream);
  if (e != cudaSuccess) return akz_report(AKZ_ERR_CUDA, cudaGetErrorString(e));
  return AKZ_OK;
}

extern "C" AKZ_API akz_status akz_matcher_set_tensor_cores(int on)
{
  if (on != 0 && on != 1) return akz_report(AKZ_ERR_INVALID_ARG, "akz_matcher_set_tensor_cores: on must be 0 or 1");
  g_akz_match_tc_on = on;
  return AKZ_OK;
}

/* Self-check of the tensor-core matcher's failure path: one launch on 256
 * query and 128 train rows whose MMA warp issues nothing, with `spin` polls
 * per wait, so the epilogue's wait for the first batch runs out.  The
 * kernel must flag it, free its tensor memory and return. */
extern "C" AKZ_API akz_status akz_selfcheck_matcher_timeout(int spin, int *timed_out)
{
  if (!timed_out || spin < 1) return akz_report(AKZ_ERR_INVALID_ARG, "akz_selfcheck_matcher_timeout: bad arguments");
  *timed_out = -1;
  int v = 0;
  cudaError_t e = akz_match_tc_status(&v); /* clear a flag left by an earlier call */
  void *dq = nullptr, *dt = nullptr, *dout = nullptr;
  const int nq = 256, nt = 128;
  if (e == cudaSuccess) e = cudaMalloc(&dq, (size_t)nq * 64);
  if (e == cudaSuccess) e = cudaMalloc(&dt, (size_t)nt * 64);
  if (e == cudaSuccess) e = cudaMalloc(&dout, (size_t)nq * 2 * sizeof(int4));
  if (e == cudaSuccess) e = cudaMemset(dq, 0x5a, (size_t)nq * 64);
  if (e == cudaSuccess) e = cudaMemset(dt, 0xa5, (size_t)nt * 64);
  int dev = 0, nsm = 0;
  if (e == cudaSuccess) e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = akz_match_tc_launch(dq, nq, dt, nt, dout, nullptr, 1, nsm, 0, spin, 1);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = akz_match_tc_status(&v);
  cudaFree(dq);
  cudaFree(dt);
  cudaFree(dout);
  if (e != cudaSuccess) return akz_report(AKZ_ERR_CUDA, cudaGetErrorString(e));
  *timed_out = v;
  return AKZ_OK;
}

extern "C" AKZ_API akz_status akz_matcher_tensor_status(int *timed_out)
{
  if (!timed_out) return akz_report(AKZ_ERR_INVALID_ARG, "akz_matcher_tensor_status: NULL");
  cudaError_t e = akz_match_tc_status(timed_out);
  if (e != cudaSuccess) return akz_report(AKZ_ERR_CUDA, cudaGetErrorString(e));
  return AKZ_OK;
}
