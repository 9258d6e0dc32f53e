/*
 * akz_internal.h - device-visible tables and launch helpers shared by the
 * akaze_gb300 kernels and the host engine.
 *
 * HBM layout of one batch (one arena, 256-byte aligned sub-buffers):
 *   u8 staging   images packed row-major, pitch = width rounded up to 16
 *   float planes per (image, level): Lt (evolved level), Ls (pre-diffusion
 *                sigma-1 smoothing used by the detector; level 0 aliases Lt),
 *                Lx, Ly (scaled first derivatives, kept for orientation and
 *                M-LDB); row pitch rounded up to 32 floats (128 B)
 *   per image    scratch planes T1, T2, G (conductance) of level-0 size
 *   per image    extrema bitmap (1 bit per level pixel, rows padded to 32
 *                bits), per-row extremum counts and their exclusive scan
 *   per image    raw extrema records, suppression state, keypoints,
 *                64-byte descriptor rows
 */
#ifndef AKZ_INTERNAL_H
#define AKZ_INTERNAL_H

#include <stdint.h>

#define AKZ_MAX_LEVELS 64
#define AKZ_MAX_NBINS 4096
#define AKZ_NMS_THREADS 512
#define AKZ_NMS_CL 8
#define AKZ_FIT_MAXIMG 4096 /* images of one batch the fit kernel indexes */ /* CTAs per image in the suppression kernel (a thread-block cluster) */
#define AKZ_NMS_NB 8 /* neighbour list capacity per raw extremum */

/* One (image, level). */
struct akz_level_desc {
  int width, height, pitch; /* pitch in floats */
  int image, level, octave, sublevel;
  int deriv_step;           /* detector step sigma_size */
  float border;             /* extrema border */
  float size;               /* esigma * derivative_factor */
  long long lt, ls, lx, ly; /* float offsets into the plane arena; Lx and Ly are one interleaved
                             * plane of (Lx, Ly) pairs with row pitch 2 * pitch (ly = lx + 1) */
  long long rows;           /* offset of this level's rows in the row-count arrays */
  long long bitmap;         /* word offset of the bitmap */
  int bitmap_pitch;         /* 32-bit words per row */
  int pad;
  long long ldet;           /* float offset of the determinant plane (row pitch `pitch`), kept only for
                             * the 3 x 3 x 3 extrema rule; -1 otherwise */
};

/* One image of the batch. */
struct akz_image_desc {
  int width, height, nlev, first_level; /* first_level: index into the level table */
  long long u8_off;                     /* byte offset of the u8 image in the staging area */
  int u8_pitch;                         /* bytes */
  int pad0;
  long long t1, t2, g;                  /* float offsets of the scratch planes */
  long long raw_base;                   /* record offset of this image's raw extrema */
  int raw_cap;                          /* capacity in records */
  int kp_cap;
  long long kp_base;                    /* keypoint/descriptor row offset */
  long long rows_base;                  /* first row-count entry of this image */
  int rows_total;                       /* rows over all levels of this image */
  int pad1;
};

/* Raw extremum as the reference's FindExtrema writes it (cuda_akaze.cu:758-769),
 * plus level coordinates. */
struct akz_raw {
  int x, y, level, octave;
  float response, size, octsub, dst1;
};

/* cv::KeyPoint layout. */
struct akz_kp {
  float x, y, size, angle, response;
  int octave, class_id;
};

/* Per-image results written by the device. */
struct akz_image_stats {
  unsigned int hmax2_bits; /* max |grad|^2 over the interior, as float bits */
  int nraw;                /* raw extrema over all levels */
  int nkp;                 /* keypoints after suppression */
  int overflow;            /* raw extrema beyond capacity */
  float kcontrast;         /* contrast factor of octave 0 */
  int nms_rounds;
  int status;              /* 0 ok, otherwise an akz_status code */
  int pad;
};

/* Work list entry of a tiled launch: tiles of one (image, level). */
struct akz_tile_seg {
  int level_desc;   /* index into the level table */
  int tiles_x;
  int tile_begin;   /* first tile index of this segment in the launch */
  int aux;          /* launch specific */
};

#ifdef __CUDACC__
#define AKZ_CUDA_CHECK(x)                                                     \
  do {                                                                        \
    cudaError_t e_ = (x);                                                     \
    if (e_ != cudaSuccess) return akz_fail_cuda(e_, #x, __FILE__, __LINE__); \
  } while (0)
#endif

#endif
