/*
 * cvshim_prims.h -- ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C restatements of the OpenCV 3.2 image primitives that ORB-SLAM2's
 * feature front-end calls (OpenCV itself is not available here).  Each one is
 * written from the published definition of the OpenCV routine it stands in for:
 *
 *   shim_resize_linear_u8   cv::resize(..., INTER_LINEAR) on CV_8UC1, the
 *                           fixed-point (11-bit coefficient) separable bilinear
 *                           path with half-pixel centres
 *                           (called at src/ORBextractor.cc:1677).
 *   shim_gauss7_u8          cv::GaussianBlur(Size(7,7), 2, 2, BORDER_REFLECT_101)
 *                           on CV_8UC1: separable, float kernel rounded to 8-bit
 *                           fixed point, (sum + 2^15) >> 16
 *                           (src/ORBextractor.cc:1610).
 *   shim_fast9_u8           cv::FAST(img, kps, th, true): FAST-9/16 segment test,
 *                           score = largest arc threshold - 1, 3x3 non-max
 *                           suppression inside the image passed
 *                           (src/ORBextractor.cc:1111,1120).
 *   shim_fast_atan2         cv::fastAtan2: 7th-order odd minimax polynomial for
 *                           atan on [0,1], in degrees (src/ORBextractor.cc:140).
 *   shim_border_reflect101  BORDER_REFLECT_101 index mapping.
 *
 * The CUDA kernels of this repository implement the same definitions; parity
 * with a real OpenCV build is not pinned because OpenCV is absent.
 * Nothing in the product links this file: tests, smoke() and bench.py's CPU
 * baseline use it as the checker only.
 */
#ifndef CVSHIM_PRIMS_H
#define CVSHIM_PRIMS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* round half to even, as cvRound (lrint under the default rounding mode) */
int shim_cvround_f(float v);
int shim_cvround_d(double v);

int shim_border_reflect101(int p, int len);

/* Bilinear INTER_LINEAR resize, u8 -> u8. */
void shim_resize_linear_u8(const uint8_t* src, size_t sstep, int sw, int sh,
                           uint8_t* dst, size_t dstep, int dw, int dh);

/* The 7 integer taps of the 8-bit fixed-point Gaussian (sigma 2). */
void shim_gauss7_taps(int taps[7]);

/* 7x7 sigma-2 Gaussian blur, u8 -> u8, BORDER_REFLECT_101 at the image edge.
 * src and dst may alias. */
void shim_gauss7_u8(const uint8_t* src, size_t sstep, int w, int h,
                    uint8_t* dst, size_t dstep);

/* FAST-9/16 with non-max suppression over a w x h image.
 * Writes up to cap keypoints (x, y, score), in the detector's emission
 * order (row-major), returns the number found (may exceed cap: only the
 * first cap are written). */
typedef struct { int x, y, score; } shim_corner;
int shim_fast9_u8(const uint8_t* img, size_t step, int w, int h, int threshold,
                  shim_corner* out, int cap);

/* Max over the 16 nine-pixel arcs of the minimum absolute difference with a
 * consistent sign (0 if no arc has a consistent sign).  A pixel is a FAST
 * corner at threshold t iff this value exceeds t, and its score is then
 * value - 1. */
int shim_fast_arc_strength(const uint8_t* center, size_t step);

float shim_fast_atan2(float y, float x);

#ifdef __cplusplus
}
#endif
#endif
