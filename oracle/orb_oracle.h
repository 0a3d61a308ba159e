/*
 * orb_oracle.h -- ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * This repository's CPU restatement of ORB-SLAM2's feature front-end, written
 * from the reference's behaviour (each function cites the reference lines it
 * follows).  It is the checker the GPU path is compared with: only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.  It is
 * pinned against the reference's own sources (refbuild/, built where they are
 * present) and through them against the committed golden fixtures.
 *
 * Every entry point mirrors the harness entry point of the same name with a
 * ref_ prefix (refbuild/ref_harness.cpp).
 */
#ifndef ORB_ORACLE_H
#define ORB_ORACLE_H
#include "orb_types.h"

#ifdef __cplusplus
extern "C" {
#endif

int orc_extract(const uint8_t* img, int w, int h, size_t step, const orc_params* p, orc_kp* kps, uint8_t* desc,
                int cap, int* n_out, uint8_t* pyr, size_t pyr_cap);
int orc_extractor_tables(const orc_params* p, float* scale, float* inv_scale, float* sigma2, float* inv_sigma2,
                         int* features_per_level, int* umax16);
int orc_descriptor_distance(const uint8_t* a, const uint8_t* b);
int orc_features_in_area(const orc_params* p, const orc_kp* kps, int n, int w, int h, float x, float y, float r,
                         int minLevel, int maxLevel, int* out, int cap);
int orc_search_for_initialization(const orc_params* p, const orc_kp* kps1, const uint8_t* desc1, int n1,
                                  const orc_kp* kps2, const uint8_t* desc2, int n2, int w, int h,
                                  float* prev_matched_xy, int window, float nnratio, int check_ori, int* matches12);
int orc_search_by_projection(const orc_params* p, const orc_kp* kps, const uint8_t* desc, const float* uright, int n,
                             int w, int h, const orc_mappoint* mps, const uint8_t* mp_desc, int m, float th,
                             float nnratio, const uint8_t* claimed, int* match_out);
/* match_out per current keypoint: >= 0 the LastFrame keypoint whose map point
 * now fills CurrentFrame.mvpMapPoints[i2]; -1 untouched; -2 claimed before the
 * call (untouched); -4 assigned, then reset to NULL by the rotation check. */
int orc_search_by_projection_frame(const orc_params* p, const orc_kp* kps, const uint8_t* desc, const float* uright,
                                   int n, int w, int h, const orc_kp* last_kps, int n_last,
                                   const orc_frame_mappoint* last_mps, const uint8_t* last_mp_desc,
                                   const orc_frame_motion* mo, float th, int mono, int check_ori,
                                   const uint8_t* claimed, int* match_out);
int orc_compute_stereo_matches(const orc_params* p, const orc_kp* kpsL, const uint8_t* descL, int nL,
                               const orc_kp* kpsR, const uint8_t* descR, int nR, const uint8_t* pyrL,
                               const uint8_t* pyrR, const int* level_w, const int* level_h, int w, int h, float bf,
                               float fx, float* uright, float* depth);
int orc_knn2(const uint8_t* q, int nq, const uint8_t* t, int nt, int* idx1, int* d1, int* idx2, int* d2);
/* MapPoint::ComputeDistinctiveDescriptors (src/MapPoint.cc:365-447) over
 * ragged observation lists of pool rows (-1 = observation of a bad keyframe).
 * best_rows: chosen row, -1 none valid, -2 invalid list (the harness version
 * reports -3: the reference exposes only the descriptor).  desc_inout
 * (nullable) gets the chosen descriptor, unchanged where best_rows < 0. */
/* DBoW2 (Thirdparty/DBoW2/DBoW2/TemplatedVocabulary.h): loads a text
 * vocabulary (loadFromTextFile) under its path, returns its word count or -1;
 * orc_bow_transform is transform(features, BowVector, FeatureVector,
 * levelsup) on n descriptors with the vocabulary loaded from path (see
 * orb_oracle.cpp for the output layout). */
int orc_vocabulary_load(const char* path);
int orc_vocabulary_from_arrays(const char* name, int k, int L, int scoring, int weighting, int nnodes,
                               const int* parents, const uint8_t* is_leaf, const uint8_t* descriptors,
                               const double* weights);
int orc_bow_transform(const char* path, const uint8_t* desc, int n, int levelsup, int* word_ids, double* weights,
                      int* node_ids, int* bow_n, int* bow_words, double* bow_values, int* fv_n, int* fv_nodes,
                      int* fv_offsets, int* fv_features);
/* ORBmatcher::SearchByProjection(Frame&, KeyFrame*, sAlreadyFound, th,
 * ORBdist) (src/ORBmatcher.cc:1891-2010).  T: rows 0-2 of mTcw; cam: fx, fy,
 * cx, cy; mp_state: 0 none, 1 usable, 2 bad, 3 already found. */
int orc_search_by_projection_kf(const orc_params* p, const orc_kp* kps, const uint8_t* desc, int n, int w, int h,
                                const float* T, const float* cam, const orc_kp* kf_kps, int m,
                                const orc_mp_geometry* mps, const uint8_t* mp_desc, const uint8_t* mp_state, float th,
                                int orbdist, int check_ori, const uint8_t* claimed, int* match_out);
/* ORBmatcher::SearchForTriangulation(pKF1, pKF2, F12, pairs, bOnlyStereo)
 * (src/ORBmatcher.cc:884-1040): see orb_oracle.cpp for the arguments. */
int orc_search_for_triangulation(const orc_kp* kps1, const uint8_t* desc1, const uint8_t* mp1, const float* ur1, int n1,
                                  int fv1_n, const int* fv1_nodes, const int* fv1_offsets, const int* fv1_features,
                                  const orc_kp* kps2, const uint8_t* desc2, const uint8_t* mp2, const float* ur2, int n2,
                                  int fv2_n, const int* fv2_nodes, const int* fv2_offsets, const int* fv2_features,
                                  const float* Cw1, const float* T2, const float* K2, const float* F12,
                                  const float* scale, const float* sigma2, int only_stereo, int check_ori,
                                  int* match_out);
/* ORBmatcher::SearchByProjection(KeyFrame*, Scw, vpPoints, vpMatched, th)
 * (src/ORBmatcher.cc:423-560).  Scw: rows 0-2 (3 x 4); cam: fx, fy, cx, cy;
 * pstate: 1 usable, 2 bad. */
int orc_search_by_projection_sim3(const orc_params* p, const orc_kp* kps, const uint8_t* desc, int n, int w, int h,
                                  const float* Scw, const float* cam, const orc_mp_geometry* pts,
                                  const uint8_t* pdesc, const uint8_t* pstate, int npts, int th,
                                  const uint8_t* claimed, int* match_out);
/* ORBmatcher::Fuse(KeyFrame*, vpMapPoints, th) (src/ORBmatcher.cc:1107-1220):
 * the keyframe feature each map point fuses with (target), -1 none; returns
 * the count.  cam: fx, fy, cx, cy, bf; mp_state 1 usable. */
int orc_fuse_candidates(const orc_params* p, const orc_kp* kps, const uint8_t* desc, const float* uright, int n,
                          int w, int h, const float* T, const float* cam, const orc_mp_geometry* mps,
                          const uint8_t* mp_desc, const uint8_t* mp_state, int m, float th, int* target);
/* ORBmatcher::Fuse(KeyFrame*, Scw, vpPoints, th, vpReplacePoint)
 * (src/ORBmatcher.cc:1290-1380): each point's choice; cam fx, fy, cx, cy. */
int orc_fuse_sim3_candidates(const orc_params* p, const orc_kp* kps, const uint8_t* desc, int n, int w, int h,
                               const float* Scw, const float* cam, const orc_mp_geometry* pts, const uint8_t* pdesc,
                               const uint8_t* pstate, int npts, float th, int* target);
/* ORBmatcher::SearchBySim3 (src/ORBmatcher.cc:1441-1640), vpMatches12 empty
 * on entry; match12: the pKF2 feature per pKF1 feature or -1. */
int orc_search_by_sim3(const orc_params* p, const orc_kp* kps1, const uint8_t* desc1, int n1, const orc_kp* kps2,
                           const uint8_t* desc2, int n2, int w, int h, const float* T1w, const float* T2w, float s12,
                           const float* R12, const float* t12, const float* cam, const orc_mp_geometry* mps1,
                           const uint8_t* mpd1, const uint8_t* st1, const orc_mp_geometry* mps2, const uint8_t* mpd2,
                           const uint8_t* st2, float th, int* match12);
/* ORBmatcher::SearchByBoW(KeyFrame*, Frame&, vpMapPointMatches)
 * (src/ORBmatcher.cc:247-380) on two FeatureVectors (nodes ascending, node i
 * owning features [offsets[i], offsets[i + 1]) of *_fv_features).  kf_mp:
 * 0 no map point, 1 a map point, 2 a bad one.  match_out: f_n keyframe
 * feature indices or -1.  Returns nmatches. */
int orc_search_by_bow(const orc_kp* kf_kps, const uint8_t* kf_desc, const uint8_t* kf_mp, int kf_n, int kf_fv_n,
                      const int* kf_fv_nodes, const int* kf_fv_offsets, const int* kf_fv_features, const orc_kp* f_kps,
                      const uint8_t* f_desc, int f_n, int f_fv_n, const int* f_fv_nodes, const int* f_fv_offsets,
                      const int* f_fv_features, float nnratio, int check_ori, int* match_out);
/* ORBmatcher::SearchByBoW(KeyFrame* pKF1, KeyFrame* pKF2, vpMatches12)
 * (src/ORBmatcher.cc:729-880): match_out has n1 entries, the pKF2 feature
 * matched to each pKF1 feature or -1. */
int orc_search_by_bow_kf(const orc_kp* kps1, const uint8_t* desc1, const uint8_t* mp1, int n1, int fv1_n,
                         const int* fv1_nodes, const int* fv1_offsets, const int* fv1_features, const orc_kp* kps2,
                         const uint8_t* desc2, const uint8_t* mp2, int n2, int fv2_n, const int* fv2_nodes,
                         const int* fv2_offsets, const int* fv2_features, float nnratio, int check_ori,
                         int* match_out);
/* Frame::UndistortKeyPoints (src/Frame.cc:724-776) and ComputeImageBounds
 * (:778-819) with cv::undistortPoints restated from OpenCV 3.2.  K4 = fx, fy,
 * cx, cy; dist = k1 k2 p1 p2 [k3] (ndist 4 or 5); bounds = mnMinX, mnMaxX,
 * mnMinY, mnMaxY. */
int orc_undistort_keypoints(const float* K4, const float* dist, int ndist, const orc_kp* kps, int n, orc_kp* out);
int orc_compute_image_bounds(int cols, int rows, const float* K4, const float* dist, int ndist, float* bounds);
/* Frame::isInFrustum(pMP, cos_limit) (src/Frame.cc:491-578, pose matrices of
 * Frame::UpdatePoseMatrices :454-470, MapPoint::PredictScale
 * src/MapPoint.cc:604-619) for m map points of one frame; out holds the map
 * points' tracking fields before the call and after it (bad untouched).
 * Returns the number in view. */
int orc_is_in_frustum(const orc_frustum_camera* cam, const orc_mp_geometry* mps, int m, float cos_limit,
                      orc_mappoint* out);
/* MapPoint::PredictScale (src/MapPoint.cc:604-619) on n ratios
 * mfMaxDistance / currentDist (oracle only; no harness counterpart). */
void orc_predict_scale(const float* ratio, int n, float scale_factor, int nlevels, int* out);
int orc_distinctive_descriptors(const uint8_t* pool, int pool_rows, const int* offsets, const int* rows, int m,
                                int* best_rows, uint8_t* desc_inout);

/* Stage-level checkers for the kernel tests. */
/* 7x7 sigma-2 blur of one level (GaussianBlur, src/ORBextractor.cc:1607-1615). */
void orc_blur_level(const uint8_t* src, int w, int h, uint8_t* dst);
/* FAST candidates of one level in the order the cell loop of
 * src/ORBextractor.cc:1069-1142 emits them (coordinates relative to the
 * 16-pixel border, as handed to DistributeOctTree); returns the count. */
int orc_fast_level(const uint8_t* level, int w, int h, int ini_th, int min_th, orc_kp* out, int cap);
/* DistributeOctTree (src/ORBextractor.cc:688-1033) on given candidates. */
int orc_distribute(const orc_kp* cand, int n, int minX, int maxX, int minY, int maxY, int N, orc_kp* out, int cap);
/* glibc cosf/sinf of the descriptor angle, for the GPU's rotation check. */
void orc_sincos_table(const float* x, int n, float* c, float* s);

#ifdef __cplusplus
}
#endif
#endif
