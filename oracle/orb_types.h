/*
 * orb_types.h -- ORACLE / TEST INFRASTRUCTURE ONLY.
 * Plain C records shared by the oracle restatement (orb_oracle.cpp) and the
 * harness around the reference's own sources (refbuild/ref_harness.cpp).
 */
#ifndef ORB_ORACLE_TYPES_H
#define ORB_ORACLE_TYPES_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Field-for-field the layout of cv::KeyPoint (pt.x, pt.y, size, angle,
 * response, octave, class_id). */
typedef struct {
    float x, y, size, angle, response;
    int32_t octave, class_id;
} orc_kp;

typedef struct {
    int nfeatures;
    float scale_factor;
    int nlevels;
    int ini_th_fast;
    int min_th_fast;
} orc_params;

/* One map point of ORBmatcher::SearchByProjection(Frame&, vector<MapPoint*>,
 * th) as the tracking thread leaves it before the call
 * (src/Tracking.cc:1731-1807 via Frame::isInFrustum, src/Frame.cc:491-578). */
typedef struct {
    float proj_x, proj_y, proj_xr, view_cos;
    int32_t track_scale_level;
    int32_t track_in_view; /* mbTrackInView */
    int32_t bad;           /* isBad() */
    int32_t pad;
} orc_mappoint;

/* One entry of LastFrame.mvpMapPoints for ORBmatcher::SearchByProjection(
 * Frame& CurrentFrame, const Frame& LastFrame, th, bMono)
 * (src/ORBmatcher.cc:1710-1879), indexed like LastFrame's keypoints. */
typedef struct {
    float x, y, z;  /* MapPoint::GetWorldPos() */
    int32_t flags;  /* ORC_MP_PRESENT | ORC_MP_OUTLIER | ORC_MP_OBSERVED */
} orc_frame_mappoint;
#define ORC_MP_PRESENT 1  /* LastFrame.mvpMapPoints[i] != NULL */
#define ORC_MP_OUTLIER 2  /* LastFrame.mvbOutlier[i] */
#define ORC_MP_OBSERVED 4 /* MapPoint::Observations() > 0 */

/* Camera data of that search: rows 0-2 of both frames' mTcw (row-major
 * 3 x 4) and the current frame's fx, fy, cx, cy, mbf, mb. */
typedef struct {
    float Tcw[12];
    float Tlw[12];
    float fx, fy, cx, cy, bf, b;
} orc_frame_motion;

/* The map point fields Frame::isInFrustum reads (src/Frame.cc:491-578). */
typedef struct {
    float x, y, z;       /* GetWorldPos() */
    float nx, ny, nz;    /* GetNormal() */
    float min_distance;  /* mfMinDistance */
    float max_distance;  /* mfMaxDistance */
} orc_mp_geometry;

/* The frame of isInFrustum: rows 0-2 of mTcw (row-major 3 x 4), Frame::fx,
 * fy, cx, cy, mbf, mnMinX, mnMaxX, mnMinY, mnMaxY, mfScaleFactor and
 * mnScaleLevels. */
typedef struct {
    float Tcw[12];
    float fx, fy, cx, cy, bf;
    float min_x, max_x, min_y, max_y;
    float scale_factor;
    int32_t nlevels;
} orc_frustum_camera;

#ifdef __cplusplus
}
#endif
#endif
