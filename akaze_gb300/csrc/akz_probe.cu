/*
 * akz_probe.cu - throughput probe for the matcher's roofline.
 *
 * The 2-NN Hamming matcher spends 16 x (xor, popc, add) on 32-bit words per
 * query/train pair (64-byte rows).  Its roofline is therefore the rate at
 * which one GPU sustains that triple, measured here rather than taken from a
 * table: every thread runs 8 independent dependency chains
 *     acc[k] += popc(acc[k] ^ key[k])
 * so that each iteration issues exactly one xor, one popc and one add per
 * chain, and 8 CTAs of 256 threads per SM keep every scheduler busy.
 */
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/akaze_gb300.h"

akz_status akz_report(akz_status s, const char *msg);

#define AKZ_POPC_CHAINS 8

__global__ void __launch_bounds__(256) k_popc_rate(unsigned int seed, int iters, unsigned int *sink)
{
  unsigned int acc[AKZ_POPC_CHAINS], key[AKZ_POPC_CHAINS];
  const unsigned int t = blockIdx.x * blockDim.x + threadIdx.x;
#pragma unroll
  for (int k = 0; k < AKZ_POPC_CHAINS; k++) {
    acc[k] = t * 2654435761u + (unsigned int)k;
    key[k] = seed ^ (0x9e3779b9u * (unsigned int)(k + 1));
  }
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < AKZ_POPC_CHAINS; k++) acc[k] += (unsigned int)__popc(acc[k] ^ key[k]);
  }
  unsigned int s = 0;
#pragma unroll
  for (int k = 0; k < AKZ_POPC_CHAINS; k++) s ^= acc[k];
  if (s == 0x5eed5eedu) sink[0] = s; /* keeps the chains live; practically never taken */
}

extern "C" AKZ_API akz_status akz_measure_popc_rate(int iters, double *triples_per_s, void *stream)
{
  if (iters < 1 || !triples_per_s) return akz_report(AKZ_ERR_INVALID_ARG, "akz_measure_popc_rate: iters < 1 or NULL output");
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0, nsm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  unsigned int *sink = nullptr;
  if (e == cudaSuccess) e = cudaMalloc(&sink, sizeof(unsigned int));
  cudaEvent_t a = nullptr, b = nullptr;
  if (e == cudaSuccess) e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  float ms = 0.0f;
  const int blocks = nsm * 8, threads = 256;
  if (e == cudaSuccess) {
    k_popc_rate<<<blocks, threads, 0, s>>>(1u, iters, sink); /* warm-up */
    cudaEventRecord(a, s);
    k_popc_rate<<<blocks, threads, 0, s>>>(2u, iters, sink);
    cudaEventRecord(b, s);
    e = cudaEventSynchronize(b);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
  }
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (sink) cudaFree(sink);
  if (e != cudaSuccess) return akz_report(AKZ_ERR_CUDA, cudaGetErrorString(e));
  *triples_per_s = (double)blocks * threads * AKZ_POPC_CHAINS * (double)iters / (ms * 1e-3);
  return AKZ_OK;
}

/* The bounded mbarrier wait of k_fed's TMA input and of the tcgen05 kernels:
 * poll try_wait at most spin times, then record a timeout and go on. */
__global__ void k_wait_selfcheck(int arrive, int spin, int *timed_out)
{
  __shared__ __align__(8) unsigned long long mbar;
  const uint32_t mb = (uint32_t)__cvta_generic_to_shared(&mbar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  __syncthreads();
  if (arrive && threadIdx.x == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mb) : "memory");
  uint32_t done = 0;
  for (int it = 0; it < spin && !done; it++)
    asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\nselp.u32 %0, 1, 0, p;\n}"
                 : "=r"(done)
                 : "r"(mb)
                 : "memory");
  if (__syncthreads_or(!done) && threadIdx.x == 0) *timed_out = 1;
}

static __device__ int g_wait_selfcheck;

extern "C" AKZ_API akz_status akz_selfcheck_bounded_wait(int arrive, int spin, int *timed_out)
{
  if (!timed_out || spin < 1) return akz_report(AKZ_ERR_INVALID_ARG, "akz_selfcheck_bounded_wait: bad arguments");
  int *flag = nullptr;
  const int zero = 0;
  cudaError_t e = cudaGetSymbolAddress((void **)&flag, g_wait_selfcheck);
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_wait_selfcheck, &zero, sizeof(int));
  if (e == cudaSuccess) {
    k_wait_selfcheck<<<1, 128>>>(arrive ? 1 : 0, spin, flag);
    e = cudaGetLastError();
  }
  int v = 0;
  if (e == cudaSuccess) e = cudaMemcpyFromSymbol(&v, g_wait_selfcheck, sizeof(int));
  if (e != cudaSuccess) return akz_report(AKZ_ERR_CUDA, cudaGetErrorString(e));
  *timed_out = v;
  return AKZ_OK;
}
