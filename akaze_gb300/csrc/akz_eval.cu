/*
 * akz_eval.cu - evaluation helpers around the matcher, and keypoint output.
 *
 *   akz_nndr_homography_inliers  the reference's match evaluation
 *     (matches2points_nndr and compute_inliers_homography, utils.cpp:154-243,
 *     as akaze_match.cpp:161-168 uses them) on the device, one thread per
 *     query, over the matcher's 2-NN output;
 *   akz_save_keypoints  the Krystian Mikolajczyk text format of
 *     save_keypoints (utils.cpp:97-152).
 */
#include <cuda_runtime.h>

#include <fstream>

#include "../../include/akaze_gb300.h"

akz_status akz_report(akz_status s, const char *msg);

struct akz_h3 {
  float h[9];
};

/* status: 0 not an NNDR match, 1 match, 2 match and homography inlier.
 * Arithmetic as in the reference: NNDR in float; the projection in float,
 * left to right; the squared distance terms in double (pow of a float
 * difference), the square root in double, then rounded to float. */
__global__ void k_nndr_inliers(const akz_dmatch *m, int nq, const akz_keypoint *kq, const akz_keypoint *kt, akz_h3 H,
                               float nndr, float min_error, signed char *status, int *counts)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nq) return;
  const akz_dmatch a = m[2 * i], b = m[2 * i + 1];
  signed char st = 0;
  if (a.distance < nndr * b.distance) {
    st = 1;
    const float x1 = kq[a.queryIdx].x, y1 = kq[a.queryIdx].y;
    const float x2 = kt[a.trainIdx].x, y2 = kt[a.trainIdx].y;
    const float s = __fadd_rn(__fadd_rn(__fmul_rn(H.h[6], x1), __fmul_rn(H.h[7], y1)), H.h[8]);
    const float x2m = __fdiv_rn(__fadd_rn(__fadd_rn(__fmul_rn(H.h[0], x1), __fmul_rn(H.h[1], y1)), H.h[2]), s);
    const float y2m = __fdiv_rn(__fadd_rn(__fadd_rn(__fmul_rn(H.h[3], x1), __fmul_rn(H.h[4], y1)), H.h[5]), s);
    const double dx = (double)__fsub_rn(x2m, x2), dy = (double)__fsub_rn(y2m, y2);
    const float dist = (float)__dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
    if (dist <= min_error) st = 2;
  }
  status[i] = st;
  if (st) {
    atomicAdd(&counts[0], 1);
    if (st == 2) atomicAdd(&counts[1], 1);
  }
}

extern "C" AKZ_API akz_status akz_nndr_homography_inliers(const akz_dmatch *matches, int nq, const akz_keypoint *kp_query,
                                                          const akz_keypoint *kp_train, const float *H, float nndr,
                                                          float min_error, int8_t *status, int *counts, void *stream)
{
  if (nq < 0 || !H || !counts || (nq > 0 && (!matches || !kp_query || !kp_train || !status)))
    return akz_report(AKZ_ERR_INVALID_ARG, "akz_nndr_homography_inliers: bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(counts, 0, 2 * sizeof(int), s);
  if (e != cudaSuccess) return akz_report(AKZ_ERR_CUDA, cudaGetErrorString(e));
  if (nq == 0) return AKZ_OK;
  akz_h3 h;
  for (int k = 0; k < 9; k++) h.h[k] = H[k];
  k_nndr_inliers<<<(nq + 255) / 256, 256, 0, s>>>(matches, nq, kp_query, kp_train, h, nndr, min_error,
                                                  (signed char *)status, counts);
  e = cudaGetLastError();
  if (e != cudaSuccess) return akz_report(AKZ_ERR_CUDA, cudaGetErrorString(e));
  return AKZ_OK;
}

extern "C" AKZ_API akz_status akz_save_keypoints(const char *path, const akz_keypoint *kpts, int n, const uint8_t *desc,
                                                int desc_bytes, int save_desc)
{
  if (!path || n < 0 || (n > 0 && !kpts) || desc_bytes < 0 || (n > 0 && desc_bytes > 0 && !desc))
    return akz_report(AKZ_ERR_INVALID_ARG, "akz_save_keypoints: bad arguments");
  std::ofstream f(path);
  if (!f) return akz_report(AKZ_ERR_INVALID_ARG, "akz_save_keypoints: cannot open the file");
  /* As the reference writes it: the header says 1 without save_desc, yet
   * every row carries the descriptor bytes it is given (utils.cpp:103,
   * :114-118, :133-141). */
  const int dsize = desc_bytes;
  f << (save_desc ? dsize : 1) << std::endl << n << std::endl;
  for (int i = 0; i < n; i++) {
    float sc = kpts[i].size;
    sc *= sc;
    f << kpts[i].x << " " << kpts[i].y << " " << 1.0 / sc << " " << 0.0 << " " << 1.0 / sc;
    for (int j = 0; j < dsize; j++) f << " " << (int)desc[(size_t)i * desc_bytes + j];
    f << std::endl;
  }
  if (!f) return akz_report(AKZ_ERR_INVALID_ARG, "akz_save_keypoints: write failed");
  return AKZ_OK;
}
