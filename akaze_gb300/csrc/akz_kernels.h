/*
 * akz_kernels.h - launch parameters and launchers of the akaze_gb300 kernels.
 * Every launcher enqueues on the given stream and returns the launch error.
 */
#ifndef AKZ_KERNELS_H
#define AKZ_KERNELS_H

#include <cuda_runtime.h>
#include <stdint.h>

#include "akz_internal.h"

#define AKZ_MAX_TAPS 33 /* Gaussian radius up to 16 */
#define AKZ_MAX_CHUNK 32

struct akz_tables {
  const akz_level_desc *lv;
  const akz_image_desc *im;
  akz_image_stats *stats;
  float *planes;
  const uint8_t *u8;
  const float *f32;    /* float input staging (when the input is f32) */
  int input_f32;
  int nimg;
};

struct akz_contrast_params {
  akz_tables t;
  const akz_tile_seg *segs;
  int nsegs;
  int nbins;
  unsigned int *hist; /* nimg x nbins */
  float inv255;
  float taps[5];      /* sigma 1, radius 2 */
};

/* Level 0 and the contrast gradient in one pass (akz_scale.cu k_level0):
 * tiles of AKZ_L0_TW x AKZ_L0_TH over level 0 of every image. */
#define AKZ_L0_TW 128
#define AKZ_L0_TH 32
struct akz_level0_params {
  akz_tables t;
  const akz_tile_seg *segs;
  int nsegs;
  float inv255;
  float taps0[5]; /* soffset Gaussian, outermost tap first, zero-padded to radius 4 */
  float taps1[3]; /* sigma 1 */
  int nbins;
  unsigned int *hist;
  int fused; /* 1: the fused-arithmetic kernel (akz_options.fast_math) */
};

struct akz_gauss_params {
  akz_tables t;
  const akz_tile_seg *segs;
  int nsegs;
  float inv255;
  int R;
  float taps[AKZ_MAX_TAPS];
};

/* k_fed geometry: a 128 x 48 region R0 = tile +- d per CTA (d = FED steps of
 * the launch).  The region's left edge tx0 - d - delta sits on a multiple of
 * 4 columns (delta = (-d) mod 4, tile origins are multiples of 4), so every
 * column pair is 8-byte aligned in shared and global memory and the TMA box
 * of the input (x = region - 4) starts on a 16-byte boundary; the tile
 * width is what remains, rounded down to a multiple of 4. */
static inline __host__ __device__ int akz_fed_delta(int d) { return (4 - (d & 3)) & 3; }
static inline __host__ __device__ int akz_fed_tile_w(int d) { return (128 - 2 * d - akz_fed_delta(d)) & ~3; }
static inline __host__ __device__ int akz_fed_tile_h(int d) { return 48 - 2 * d; }
#define AKZ_FED_BOX_W 136 /* input box: region +- 4 columns */
#define AKZ_FED_BOX_H 54  /* region +- 3 rows */

struct akz_fed_params {
  akz_tables t;
  /* two 128-byte CUtensorMaps per level descriptor l: [2l] the level's Lt
   * plane, [2l + 1] its image's T2 plane at the level's size; boxes of
   * AKZ_FED_BOX_W x AKZ_FED_BOX_H floats */
  const void *tmaps;
  const akz_tile_seg *segs;
  int nsegs;
  const float2 *kc;   /* per image x 16 octaves: (k, 1/k^2) */
  int steps;          /* FED steps in this launch */
  int first;          /* 1: start from the predecessor (copy / 2x half-sample / prepared T2) */
  int src;            /* first: 0 predecessor Lt, 1 2x half-sample of it, 2 prepared T2; else 1 T1, 2 T2 */
  int dst;            /* 0 Lt of the level, 1 T1, 2 T2, 3 chk */
  int write_g;        /* store the conductance for later launches */
  int diffusivity;
  int fused;          /* 1: the fused-arithmetic kernel (akz_options.fast_math) */
  float taps1[5];
  float h[AKZ_MAX_CHUNK]; /* 0.5 * tau per step */
  float *chk;         /* dst 3: a plane with the level's pitch */
  const float *gate;  /* non-NULL: the launch runs only if !(*gate <= gate_tol) */
  float gate_tol;
};

/* INTER_AREA tables of one octave start: start[] indices are absolute into
 * si/alpha; xs/ys are offsets of the per-axis start arrays in start[]. */
struct akz_area_seg {
  int ld; /* level descriptor of the octave-start level */
  int xs, ys;
  int pad;
};

struct akz_area_params {
  akz_tables t;
  const akz_area_seg *segs;
  int nsegs;
  const int *start;
  const int *si;
  const float *alpha;
};

struct akz_detect_params {
  akz_tables t;
  const akz_tile_seg *segs;
  int nsegs;
  uint32_t *bitmap;
  int *rowcnt;
  float thr, fac1, fac2;
  int store_det; /* 1: keep every level's determinant in its plane (L.ldet) for the 3 x 3 x 3 rule */
  int fused;     /* 1: the strip detector's fused-arithmetic kernel (akz_options.fast_math) */
};

struct akz_extract_params {
  akz_tables t;
  const akz_tile_seg *segs; /* one entry per (image, level); tiles = rows */
  int nsegs;
  const uint32_t *bitmap;
  const int *rowscan;
  akz_raw *raw;
  float fac1, fac2;
};

struct akz_nms_params {
  akz_tables t;
  const int *rowscan;
  const akz_raw *raw;
  int *state;
  int *aux; /* minimum challenger per slot */
  signed char *decision;
  akz_kp *kp;
  int max_rounds;
  int *nbr;           /* AKZ_NMS_NB neighbours per raw extremum */
  unsigned char *nbc; /* their count; AKZ_NMS_NB + 1: more, decided by scanning */
};

struct akz_describe_params {
  akz_tables t;
  akz_kp *kp;
  uint32_t *desc; /* 16 words per keypoint */
  int upright;
  int pattern_size;
  int channels;   /* 1 (L), 2 (L, |grad|) or 3 (L, rotated dx, dy) */
  int nbits;      /* bits of a descriptor row (<= 486) */
  const unsigned char *cmp1, *cmp2; /* bit b: cell value cmp1[b] > cmp2[b] (3 * cell + channel) */
  float gw[36];   /* Gaussian weights exp(-r2/12.5) of the orientation samples */
};

cudaError_t akz_launch_contrast(const akz_contrast_params &p, int ntiles, int pass, cudaStream_t s);
cudaError_t akz_launch_contrast_final(const akz_tables &t, const unsigned int *hist, int nbins, float perc, float2 *kc, cudaStream_t s);
cudaError_t akz_launch_gauss0(const akz_gauss_params &p, int ntiles, cudaStream_t s);
cudaError_t akz_launch_level0(const akz_level0_params &p, int ntiles, cudaStream_t s);
cudaError_t akz_launch_fed(const akz_fed_params &p, int ntiles, int tw, int th, cudaStream_t s);
size_t akz_fed_smem_bytes(int tw, int th, int steps, int first);
cudaError_t akz_launch_area(const akz_area_params &p, int maxw, int maxh, cudaStream_t s);
cudaError_t akz_launch_detect(const akz_detect_params &p, int ntiles, int max_step, cudaStream_t s);
/* streaming detector for derivative steps 2..4: strips of
 * akz_strip_tile_width(st) columns and AKZ_STRIP_CH rows */
#define AKZ_STRIP_CH 256
int akz_strip_tile_width(int st); /* 0 for steps the strip kernel does not compile */
cudaError_t akz_launch_detect_strip(const akz_detect_params &p, int ntiles, cudaStream_t s);
/* the 3 x 3 x 3 extrema rule: clears the bitmap bits (and row counts) of
 * candidates that do not exceed the 3 x 3 blocks of the adjacent levels of
 * their octave; after both detector launches with store_det set */
cudaError_t akz_launch_extrema3d(const akz_detect_params &p, int nlevels_total, int max_level_h, cudaStream_t s);
cudaError_t akz_launch_rowscan(const akz_tables &t, const int *rowcnt, int *rowscan, cudaStream_t s);
cudaError_t akz_launch_extract(const akz_extract_params &p, int nrows, cudaStream_t s);
cudaError_t akz_launch_nms(const akz_nms_params &p, cudaStream_t s);
cudaError_t akz_launch_describe(const akz_describe_params &p, int nblocks, cudaStream_t s);

#define AKZ_DETECT_TW 64
#define AKZ_DETECT_TH 32
#define AKZ_GAUSS_TW 64
#define AKZ_GAUSS_TH 32
#define AKZ_CONTRAST_TW 64
#define AKZ_CONTRAST_TH 32

#endif
