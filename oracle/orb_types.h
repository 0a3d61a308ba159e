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

#ifdef __cplusplus
}
#endif
#endif
