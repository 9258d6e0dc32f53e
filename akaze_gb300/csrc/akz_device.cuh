/*
 * akz_device.cuh - small device helpers shared by the kernels.
 *
 * All kernels are compiled with -fmad=false: every float expression is
 * evaluated as written, with one rounding per operation, so the GPU results
 * equal the CPU restatement of the reference operation for operation.
 */
#ifndef AKZ_DEVICE_CUH
#define AKZ_DEVICE_CUH

#include <cuda_runtime.h>
#include <stdint.h>

#include "akz_internal.h"
#include "akz_kernels.h"

__device__ __forceinline__ int akz_clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* cv::BORDER_REFLECT_101 for offsets of at most n-1. */
__device__ __forceinline__ int akz_refl101(int i, int n)
{
  if (n == 1) return 0;
  if (i < 0) return -i;
  if (i >= n) return 2 * n - 2 - i;
  return i;
}

/* Segment of a tiled launch that owns tile t (segments sorted by tile_begin). */
__device__ __forceinline__ int akz_find_seg(const akz_tile_seg *segs, int nsegs, int t)
{
  int lo = 0, hi = nsegs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(&segs[mid].tile_begin) <= t)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

/* akz_find_seg as a 32-way search by the (full) warp: each round every lane
 * reads one segment start, so up to 32 segments cost one load round trip and
 * up to 1024 two, instead of a chain of log2(nsegs) dependent loads. */
__device__ __forceinline__ int akz_find_seg_warp(const akz_tile_seg *segs, int nsegs, int t)
{
  const int lane = threadIdx.x & 31;
  int lo = 0, n = nsegs; /* the answer lies in [lo, lo + n); segs[lo] starts at or before t */
  while (n > 32) {
    const int stride = (n + 31) >> 5, i = lo + lane * stride;
    const int c = __popc(__ballot_sync(0xffffffffu, i < lo + n && __ldg(&segs[i].tile_begin) <= t));
    const int nlo = lo + (c - 1) * stride; /* starts are sorted: the lanes at or below t form a prefix */
    n = min(stride, lo + n - nlo);
    lo = nlo;
  }
  const int i = lo + lane;
  return lo + __popc(__ballot_sync(0xffffffffu, i < lo + n && __ldg(&segs[i].tile_begin) <= t)) - 1;
}

/* Input pixel of image img as float in [0,1]: u8 * (float)(1/255) or f32.
 * Both staging arrays use the same element offsets and pitches. */
__device__ __forceinline__ float akz_fetch_input(const akz_tables &t, const akz_image_desc &I, int x, int y, float inv255)
{
  if (t.input_f32) return __ldg(t.f32 + I.u8_off + (long long)y * I.u8_pitch + x);
  return (float)__ldg(t.u8 + I.u8_off + (long long)y * I.u8_pitch + x) * inv255;
}

/* Detector derivative pair at (x, y) from a plane s with reflect-101 offsets
 * of +-step (cuda_akaze.cu:651-671):
 *   dx = fac1*(ur + lr - ul - ll) + fac2*(cr - cl)
 *   dy = fac1*(lr + ll - ur - ul) + fac2*(lc - uc)
 * The accessor A(x, y) returns the plane value. */
template <class A>
__device__ __forceinline__ void akz_deriv_at(const A &s, int W, int H, int step, int x, int y, float fac1, float fac2,
                                             float *dx, float *dy)
{
  const int xl = x < step ? step - x : x - step;
  const int xh = x >= W - step ? 2 * W - x - step - 2 : x + step;
  const int yl = y < step ? step - y : y - step;
  const int yh = y >= H - step ? 2 * H - y - step - 2 : y + step;
  const float ul = s(xl, yl), ur = s(xh, yl), ll = s(xl, yh), lr = s(xh, yh);
  const float cl = s(xl, y), cr = s(xh, y), uc = s(x, yl), lc = s(x, yh);
  *dx = fac1 * (ur + lr - ul - ll) + fac2 * (cr - cl);
  *dy = fac1 * (lr + ll - ur - ul) + fac2 * (lc - uc);
}

/* Hessian determinant at (x, y) from Lx, Ly accessors (cuda_akaze.cu:673-701). */
template <class A>
__device__ __forceinline__ float akz_det_at(const A &lx, const A &ly, int W, int H, int step, int x, int y, float fac1, float fac2)
{
  const int xl = x < step ? step - x : x - step;
  const int xh = x >= W - step ? 2 * W - x - step - 2 : x + step;
  const int yl = y < step ? step - y : y - step;
  const int yh = y >= H - step ? 2 * H - y - step - 2 : y + step;
  float ul = lx(xl, yl), ur = lx(xh, yl), ll = lx(xl, yh), lr = lx(xh, yh);
  const float cl = lx(xl, y), cr = lx(xh, y);
  const float lxx = fac1 * (ur + lr - ul - ll) + fac2 * (cr - cl);
  float uc = lx(x, yl), lc = lx(x, yh);
  const float lyx = fac1 * (lr + ll - ur - ul) + fac2 * (lc - uc);
  ul = ly(xl, yl);
  ur = ly(xh, yl);
  ll = ly(xl, yh);
  lr = ly(xh, yh);
  uc = ly(x, yl);
  lc = ly(x, yh);
  const float lyy = fac1 * (lr + ll - ur - ul) + fac2 * (lc - uc);
  return lxx * lyy - lyx * lyx;
}

/* Hessian determinant at (x, y) from the interleaved (Lx, Ly) plane lxy
 * (row pitch pitch2 floats): the expressions of akz_det_at, each tap's pair
 * read with one 64-bit load. */
__device__ __forceinline__ float akz_det_at2(const float *lxy, long long pitch2, int W, int H, int step, int x, int y,
                                             float fac1, float fac2)
{
  const int xl = x < step ? step - x : x - step;
  const int xh = x >= W - step ? 2 * W - x - step - 2 : x + step;
  const int yl = y < step ? step - y : y - step;
  const int yh = y >= H - step ? 2 * H - y - step - 2 : y + step;
  auto at = [&](int xx, int yy) { return __ldg(reinterpret_cast<const float2 *>(lxy + yy * pitch2 + 2 * xx)); };
  const float2 ul = at(xl, yl), ur = at(xh, yl), ll = at(xl, yh), lr = at(xh, yh);
  const float2 cl = at(xl, y), cr = at(xh, y), uc = at(x, yl), lc = at(x, yh);
  const float lxx = fac1 * (ur.x + lr.x - ul.x - ll.x) + fac2 * (cr.x - cl.x);
  const float lyx = fac1 * (lr.x + ll.x - ur.x - ul.x) + fac2 * (lc.x - uc.x);
  const float lyy = fac1 * (lr.y + ll.y - ur.y - ul.y) + fac2 * (lc.y - uc.y);
  return lxx * lyy - lyx * lyx;
}

/* Packed FP32x2 additions (sm_100+ add/sub .f32x2): two independent IEEE
 * float additions per instruction, each rounded exactly like the scalar one.
 * There is deliberately no packed multiply: the assembler of CUDA 13.0
 * contracts a packed multiply (mul.rn.f32x2, or fma.rn.f32x2 with a -0
 * addend) feeding a packed add into a packed fused multiply-add despite the
 * .rn modifier and -fmad=false (measured on sm_103a: 9-14% of random operands
 * differ from the scalar result), while scalar products feeding a packed add
 * are kept as written (0 of 2^20 differ). */
__device__ __forceinline__ unsigned long long akz_f2u(float2 v)
{
  return ((unsigned long long)__float_as_uint(v.y) << 32) | __float_as_uint(v.x);
}
__device__ __forceinline__ float2 akz_u2f(unsigned long long u)
{
  return make_float2(__uint_as_float((unsigned int)u), __uint_as_float((unsigned int)(u >> 32)));
}
__device__ __forceinline__ float2 f2add(float2 a, float2 b)
{
  unsigned long long r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(akz_f2u(a)), "l"(akz_f2u(b)));
  return akz_u2f(r);
}
__device__ __forceinline__ float2 f2sub(float2 a, float2 b)
{
  unsigned long long r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(akz_f2u(a)), "l"(akz_f2u(b)));
  return akz_u2f(r);
}
/* Explicit packed fused multiply-add (one rounding per lane, as fmaf). */
__device__ __forceinline__ float2 f2fma(float2 a, float2 b, float2 c)
{
  unsigned long long r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(akz_f2u(a)), "l"(akz_f2u(b)), "l"(akz_f2u(c)));
  return akz_u2f(r);
}
__device__ __forceinline__ float2 ld2(const float *p) { return *reinterpret_cast<const float2 *>(p); }
__device__ __forceinline__ void st2(float *p, float2 v) { *reinterpret_cast<float2 *>(p) = v; }
/* Packed product, for the fused-arithmetic kernels only (see above). */
__device__ __forceinline__ float2 f2mul(float2 a, float2 b)
{
  unsigned long long r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(akz_f2u(a)), "l"(akz_f2u(b)));
  return akz_u2f(r);
}

/* Products and multiply-adds of the level and detector kernels in their two
 * arithmetic modes.  FUSED = false: the reference's operation order, every
 * product and sum rounded on its own (scalar products, packed sums), which
 * reproduces the CPU restatement bit for bit.  FUSED = true: packed products
 * and packed fused multiply-adds (one rounding per multiply-add), about half
 * the instructions; results stay within the tolerances the fused mode is
 * tested to (levels 1e-4 relative). */
template <bool FUSED>
__device__ __forceinline__ float2 akz_k2(float k, float2 v) /* k * v */
{
  if (FUSED) return f2mul(make_float2(k, k), v);
  return make_float2(k * v.x, k * v.y);
}
template <bool FUSED>
__device__ __forceinline__ float2 akz_axpy2(float k, float2 v, float2 acc) /* acc + k * v */
{
  if (FUSED) return f2fma(make_float2(k, k), v, acc);
  return f2add(acc, make_float2(k * v.x, k * v.y));
}
template <bool FUSED>
__device__ __forceinline__ float2 akz_mul2(float2 a, float2 b) /* a * b */
{
  if (FUSED) return f2mul(a, b);
  return make_float2(a.x * b.x, a.y * b.y);
}
template <bool FUSED>
__device__ __forceinline__ float2 akz_sq2sum(float2 a, float2 b) /* a^2 + b^2 */
{
  if (FUSED) return f2fma(a, a, f2mul(b, b));
  return f2add(make_float2(a.x * a.x, a.y * a.y), make_float2(b.x * b.x, b.y * b.y));
}
template <bool FUSED>
__device__ __forceinline__ float2 akz_lin2(float ka, float2 a, float kb, float2 b) /* ka * a + kb * b */
{
  if (FUSED) return f2fma(make_float2(ka, ka), a, f2mul(make_float2(kb, kb), b));
  return f2add(make_float2(ka * a.x, ka * a.y), make_float2(kb * b.x, kb * b.y));
}
template <bool FUSED>
__device__ __forceinline__ float2 akz_det2(float2 a, float2 b, float2 c) /* a * b - c * c */
{
  if (FUSED) return f2fma(a, b, f2mul(make_float2(-c.x, -c.y), c));
  return f2sub(make_float2(a.x * b.x, a.y * b.y), make_float2(c.x * c.x, c.y * c.y));
}

struct akz_plane_acc {
  const float *p;
  int pitch;
  __device__ __forceinline__ float operator()(int x, int y) const { return __ldg(p + (long long)y * pitch + x); }
};

struct akz_smem_acc {
  const float *p;
  int x0, y0, stride;
  __device__ __forceinline__ float operator()(int x, int y) const { return p[(y - y0) * stride + (x - x0)]; }
};

#endif
