/*
 * akz_surrogate.cu - the learned FED surrogate: a 5-layer 3x3 convolutional
 * net (3 -> 32 -> 32 -> 32 -> 32 -> 1 channels, ReLU between layers) that
 * maps one level's starting image, its conductance and the level's FED time
 * span to the residual L_end - L_start of the level's whole FED cycle
 * (AKAZE.cpp:244-270 computes that cycle step by step).
 *
 * This file holds the training kernels, FP32 throughout:
 *   k_sg_conv_fwd   valid 3x3 convolution, bias, optional ReLU;
 *   k_sg_conv_bwd_data  gradient with respect to the input, times the ReLU
 *                   derivative of that input (the previous layer's output);
 *   k_sg_conv_bwd_w gradient with respect to weights and bias, per-block
 *                   partial sums reduced with atomics;
 *   k_sg_adam       Adam update.
 * Tensors are NCHW float32 on the device; weights are [cout][cin][3][3].
 * The inference kernel (BF16 tensor cores) lives in akz_surrogate_infer.cu.
 */
#include <cuda_runtime.h>

#include "../../include/akaze_gb300.h"

akz_status akz_report(akz_status s, const char *msg);

#define SG_T 16       /* output tile edge of the convolution kernels */
#define SG_MAXC 32    /* channel limit */

/* out[b, co, y, x] = bias[co] + sum_ci sum_k w[co, ci, k] * in[b, ci, y + ky, x + kx] */
__global__ void __launch_bounds__(SG_T *SG_T) k_sg_conv_fwd(const float *__restrict__ in, const float *__restrict__ w,
                                                           const float *__restrict__ bias, float *__restrict__ out,
                                                           int cin, int cout, int hi, int wi, int relu)
{
  __shared__ float sIn[(SG_T + 2) * (SG_T + 2)];
  __shared__ float sW[SG_MAXC * 9];
  const int ho = hi - 2, wo = wi - 2;
  const int tx = threadIdx.x % SG_T, ty = threadIdx.x / SG_T;
  const int ox0 = blockIdx.x * SG_T, oy0 = blockIdx.y * SG_T, b = blockIdx.z;
  const int ox = ox0 + tx, oy = oy0 + ty;
  float acc[SG_MAXC];
#pragma unroll
  for (int co = 0; co < SG_MAXC; co++) acc[co] = co < cout ? bias[co] : 0.0f;
  for (int ci = 0; ci < cin; ci++) {
    const float *src = in + ((long long)b * cin + ci) * hi * wi;
    for (int i = threadIdx.x; i < (SG_T + 2) * (SG_T + 2); i += SG_T * SG_T) {
      const int yy = oy0 + i / (SG_T + 2), xx = ox0 + i % (SG_T + 2);
      sIn[i] = (yy < hi && xx < wi) ? src[(long long)yy * wi + xx] : 0.0f;
    }
    for (int i = threadIdx.x; i < cout * 9; i += SG_T * SG_T) sW[i] = w[((i / 9) * cin + ci) * 9 + i % 9];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 9; k++) {
      const float v = sIn[(ty + k / 3) * (SG_T + 2) + tx + k % 3];
#pragma unroll
      for (int co = 0; co < SG_MAXC; co++)
        if (co < cout) acc[co] += sW[co * 9 + k] * v;
    }
    __syncthreads();
  }
  if (ox >= wo || oy >= ho) return;
#pragma unroll
  for (int co = 0; co < SG_MAXC; co++)
    if (co < cout) {
      const float v = relu ? fmaxf(acc[co], 0.0f) : acc[co];
      out[(((long long)b * cout + co) * ho + oy) * wo + ox] = v;
    }
}

/* din[b, ci, y, x] = (mask[b, ci, y, x] > 0) * sum_co sum_k w[co, ci, k] * dout[b, co, y - ky, x - kx]
 * (mask NULL: no ReLU factor) */
__global__ void __launch_bounds__(SG_T *SG_T) k_sg_conv_bwd_data(const float *__restrict__ dout, const float *__restrict__ w,
                                                                const float *__restrict__ mask, float *__restrict__ din,
                                                                int cin, int cout, int hi, int wi)
{
  __shared__ float sG[(SG_T + 2) * (SG_T + 2)];
  __shared__ float sW[SG_MAXC * 9];
  const int ho = hi - 2, wo = wi - 2;
  const int tx = threadIdx.x % SG_T, ty = threadIdx.x / SG_T;
  const int x0 = blockIdx.x * SG_T, y0 = blockIdx.y * SG_T, b = blockIdx.z;
  const int x = x0 + tx, y = y0 + ty;
  float acc[SG_MAXC];
#pragma unroll
  for (int ci = 0; ci < SG_MAXC; ci++) acc[ci] = 0.0f;
  for (int co = 0; co < cout; co++) {
    const float *g = dout + ((long long)b * cout + co) * ho * wo;
    /* dout rows y0-2 .. y0+SG_T-1, columns x0-2 .. x0+SG_T-1 */
    for (int i = threadIdx.x; i < (SG_T + 2) * (SG_T + 2); i += SG_T * SG_T) {
      const int yy = y0 - 2 + i / (SG_T + 2), xx = x0 - 2 + i % (SG_T + 2);
      sG[i] = (yy >= 0 && yy < ho && xx >= 0 && xx < wo) ? g[(long long)yy * wo + xx] : 0.0f;
    }
    for (int i = threadIdx.x; i < cin * 9; i += SG_T * SG_T) sW[i] = w[(co * cin + i / 9) * 9 + i % 9];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 9; k++) {
      /* output (y - ky, x - kx) used input (y, x) with tap k */
      const float gv = sG[(ty + 2 - k / 3) * (SG_T + 2) + tx + 2 - k % 3];
#pragma unroll
      for (int ci = 0; ci < SG_MAXC; ci++)
        if (ci < cin) acc[ci] += sW[ci * 9 + k] * gv;
    }
    __syncthreads();
  }
  if (x >= wi || y >= hi) return;
#pragma unroll
  for (int ci = 0; ci < SG_MAXC; ci++)
    if (ci < cin) {
      const long long o = (((long long)b * cin + ci) * hi + y) * wi + x;
      const float m = mask ? (mask[o] > 0.0f ? 1.0f : 0.0f) : 1.0f;
      din[o] = acc[ci] * m;
    }
}

/* dw[co, ci, k] += sum_{b,y,x} dout[b, co, y, x] * in[b, ci, y + ky, x + kx];  db[co] += sum dout.
 * One block per (co, ci) pair and a slice of the batch; 9 + 1 partial sums
 * reduced in shared memory, then added with atomics. */
__global__ void __launch_bounds__(256) k_sg_conv_bwd_w(const float *__restrict__ in, const float *__restrict__ dout,
                                                      float *__restrict__ dw, float *__restrict__ db, int nb, int cin,
                                                      int cout, int hi, int wi, int bslice)
{
  const int co = blockIdx.x / cin, ci = blockIdx.x % cin;
  const int b0 = blockIdx.y * bslice, b1 = min(nb, b0 + bslice);
  const int ho = hi - 2, wo = wi - 2;
  float acc[10];
#pragma unroll
  for (int k = 0; k < 10; k++) acc[k] = 0.0f;
  for (int b = b0; b < b1; b++) {
    const float *g = dout + ((long long)b * cout + co) * ho * wo;
    const float *src = in + ((long long)b * cin + ci) * hi * wi;
    for (int p = threadIdx.x; p < ho * wo; p += 256) {
      const int y = p / wo, x = p % wo;
      const float gv = g[p];
#pragma unroll
      for (int k = 0; k < 9; k++) acc[k] += gv * src[(long long)(y + k / 3) * wi + x + k % 3];
      acc[9] += gv;
    }
  }
  __shared__ float red[8][10];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 10; k++) {
    float v = acc[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[wid][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < 10) {
    float v = 0.0f;
    for (int i = 0; i < 8; i++) v += red[i][threadIdx.x];
    if (threadIdx.x < 9)
      atomicAdd(&dw[(co * cin + ci) * 9 + threadIdx.x], v);
    else if (ci == 0)
      atomicAdd(&db[co], v);
  }
}

__global__ void k_sg_adam(float *p, const float *g, float *m, float *v, int n, float lr, float b1, float b2, float eps,
                          float c1, float c2)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.0f - b1) * gi;
  const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

static akz_status sg_check(const char *what)
{
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return akz_report(AKZ_ERR_CUDA, cudaGetErrorString(e));
  (void)what;
  return AKZ_OK;
}

static bool sg_shape_ok(int nb, int cin, int cout, int hi, int wi)
{
  return nb >= 1 && cin >= 1 && cin <= SG_MAXC && cout >= 1 && cout <= SG_MAXC && hi >= 3 && wi >= 3 && nb <= 65535;
}

extern "C" AKZ_API akz_status akz_sg_conv_forward(const float *in, const float *w, const float *bias, float *out, int nb,
                                                  int cin, int cout, int hi, int wi, int relu, void *stream)
{
  if (!sg_shape_ok(nb, cin, cout, hi, wi) || !in || !w || !bias || !out)
    return akz_report(AKZ_ERR_INVALID_ARG, "akz_sg_conv_forward: bad shape or NULL pointer");
  const dim3 grid((wi - 2 + SG_T - 1) / SG_T, (hi - 2 + SG_T - 1) / SG_T, nb);
  k_sg_conv_fwd<<<grid, SG_T * SG_T, 0, (cudaStream_t)stream>>>(in, w, bias, out, cin, cout, hi, wi, relu);
  return sg_check("conv_forward");
}

extern "C" AKZ_API akz_status akz_sg_conv_backward_data(const float *dout, const float *w, const float *mask, float *din,
                                                        int nb, int cin, int cout, int hi, int wi, void *stream)
{
  if (!sg_shape_ok(nb, cin, cout, hi, wi) || !dout || !w || !din)
    return akz_report(AKZ_ERR_INVALID_ARG, "akz_sg_conv_backward_data: bad shape or NULL pointer");
  const dim3 grid((wi + SG_T - 1) / SG_T, (hi + SG_T - 1) / SG_T, nb);
  k_sg_conv_bwd_data<<<grid, SG_T * SG_T, 0, (cudaStream_t)stream>>>(dout, w, mask, din, cin, cout, hi, wi);
  return sg_check("conv_backward_data");
}

extern "C" AKZ_API akz_status akz_sg_conv_backward_weights(const float *in, const float *dout, float *dw, float *db, int nb,
                                                           int cin, int cout, int hi, int wi, void *stream)
{
  if (!sg_shape_ok(nb, cin, cout, hi, wi) || !in || !dout || !dw || !db)
    return akz_report(AKZ_ERR_INVALID_ARG, "akz_sg_conv_backward_weights: bad shape or NULL pointer");
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(dw, 0, (size_t)cout * cin * 9 * sizeof(float), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(db, 0, (size_t)cout * sizeof(float), s);
  if (e != cudaSuccess) return akz_report(AKZ_ERR_CUDA, cudaGetErrorString(e));
  const int bslice = 4;
  const dim3 grid(cout * cin, (nb + bslice - 1) / bslice);
  k_sg_conv_bwd_w<<<grid, 256, 0, s>>>(in, dout, dw, db, nb, cin, cout, hi, wi, bslice);
  return sg_check("conv_backward_weights");
}

extern "C" AKZ_API akz_status akz_sg_adam(float *param, const float *grad, float *m, float *v, int n, float lr, float beta1,
                                         float beta2, float eps, int step, void *stream)
{
  if (n < 1 || !param || !grad || !m || !v || step < 1) return akz_report(AKZ_ERR_INVALID_ARG, "akz_sg_adam: bad arguments");
  const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
  k_sg_adam<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(param, grad, m, v, n, lr, beta1, beta2, eps, c1, c2);
  return sg_check("adam");
}

/* dout = scale * (out - target); partial sums of (out - target)^2 per block
 * into loss_parts[blockIdx.x] (the host adds them) */
__global__ void __launch_bounds__(256) k_sg_mse_grad(const float *out, const float *target, float *dout, int n, float scale,
                                                    float *loss_parts)
{
  __shared__ float red[8];
  float acc = 0.0f;
  for (int i = blockIdx.x * 256 + threadIdx.x; i < n; i += gridDim.x * 256) {
    const float d = out[i] - target[i];
    dout[i] = scale * d;
    acc += d * d;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    float s = 0.0f;
    for (int i = 0; i < 8; i++) s += red[i];
    loss_parts[blockIdx.x] = s;
  }
}

extern "C" AKZ_API akz_status akz_sg_mse_grad(const float *out, const float *target, float *dout, int n, float scale,
                                             float *loss_parts, int nparts, void *stream)
{
  if (n < 1 || nparts < 1 || !out || !target || !dout || !loss_parts)
    return akz_report(AKZ_ERR_INVALID_ARG, "akz_sg_mse_grad: bad arguments");
  k_sg_mse_grad<<<nparts, 256, 0, (cudaStream_t)stream>>>(out, target, dout, n, scale, loss_parts);
  return sg_check("mse_grad");
}
