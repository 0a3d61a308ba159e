/*
 * orbgpu.h -- C ABI of the GB300 ORB front-end (liborbgpu.so).
 *
 * Drop-in boundary for ORB-SLAM2's feature hot path: each entry point names
 * the reference interface it replaces (file:line in the reference tree).
 * Plain pointers and sizes only.  Every call is asynchronous on the handle's
 * CUDA stream unless it says otherwise; calls that return host results
 * synchronise that stream before returning.
 *
 * Memory flags: ORBGPU_MEM_HOST means the pointer is host memory (pageable or
 * pinned) and the library copies through its own device buffers;
 * ORBGPU_MEM_DEVICE means the pointer is device memory of the current device.
 *
 * Error convention: every function returns an orbgpu_status; 0 is success.
 * orbgpu_last_error() returns a thread-local description of the last failure.
 * There is no CPU fallback: without a usable CUDA device every call fails
 * with ORBGPU_ERR_CUDA.
 */
#ifndef ORBGPU_H
#define ORBGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    ORBGPU_OK = 0,
    ORBGPU_ERR_BAD_ARG = 1,  /* invalid argument (the reference asserts or has undefined behaviour) */
    ORBGPU_ERR_OOM = 2,      /* device allocation failed */
    ORBGPU_ERR_CUDA = 3,     /* CUDA runtime error (no device, launch failure, ...) */
    ORBGPU_ERR_TIMEOUT = 4,  /* a bounded device-side wait gave up */
    ORBGPU_ERR_CAPACITY = 5  /* caller's output capacity too small; *n_* holds the needed size */
} orbgpu_status;

enum { ORBGPU_MEM_HOST = 0, ORBGPU_MEM_DEVICE = 1 };

/* Field for field the layout of cv::KeyPoint: pt.x, pt.y, size, angle,
 * response, octave, class_id (28 bytes). */
typedef struct {
    float x, y, size, angle, response;
    int32_t octave, class_id;
} orbgpu_keypoint;

const char* orbgpu_last_error(void);
int orbgpu_version(void);

/* ------------------------------------------------------------ extractor */
typedef struct orbgpu_extractor orbgpu_extractor;

/* ORBextractor::ORBextractor(int nfeatures, float scaleFactor, int nlevels,
 *                            int iniThFAST, int minThFAST)
 * -- include/ORBextractor.h:93, src/ORBextractor.cc:469-571.
 * max_width/max_height bound the images this handle accepts (device buffers
 * are sized for them once).  stream: a cudaStream_t, or NULL for a stream the
 * handle creates and owns. */
int orbgpu_extractor_create(int nfeatures, float scale_factor, int nlevels, int ini_th_fast, int min_th_fast,
                            int max_width, int max_height, void* stream, orbgpu_extractor** out);
int orbgpu_extractor_destroy(orbgpu_extractor* ex);

/* ORBextractor::operator()(InputArray image, InputArray mask,
 *                          vector<KeyPoint>& keypoints, OutputArray descriptors)
 * -- include/ORBextractor.h:111, src/ORBextractor.cc:1533-1649.
 * image: width x height uint8, row pitch 'step' bytes, host or device per
 * image_mem.  keypoints (capacity entries) and descriptors (capacity x 32
 * bytes, row-major) are host or device per out_mem.  The mask is ignored by
 * the reference and has no parameter here.  An empty image (width or height
 * 0) returns OK with *n_keypoints = 0.  Output order is the reference's:
 * level-major, each level in DistributeOctTree's list order; coordinates
 * scaled to level 0.  Synchronises the handle's stream. */
int orbgpu_extract(orbgpu_extractor* ex, const uint8_t* image, int width, int height, size_t step, int image_mem,
                   orbgpu_keypoint* keypoints, uint8_t* descriptors, int capacity, int out_mem, int* n_keypoints);

/* GetLevels / GetScaleFactors / GetInverseScaleFactors / GetScaleSigmaSquares
 * / GetInverseScaleSigmaSquares -- include/ORBextractor.h:119-159.
 * Arrays receive nlevels floats each (any may be NULL). */
int orbgpu_extractor_tables(const orbgpu_extractor* ex, int* nlevels, float* scale_factors, float* inv_scale_factors,
                            float* sigma2, float* inv_sigma2, int* features_per_level);

/* mvImagePyramid[level] of the last extraction -- include/ORBextractor.h:162.
 * Returns the device pointer of the unblurred level, its size and row pitch. */
int orbgpu_extractor_pyramid_level(const orbgpu_extractor* ex, int level, const uint8_t** dev_ptr, int* width,
                                   int* height, size_t* pitch);

/* The CUDA stream of the handle (a cudaStream_t). */
void* orbgpu_extractor_stream(const orbgpu_extractor* ex);

/* ------------------------------------------------------------ batched extraction */
/* Many frames of uneven size through one pipeline: a ragged list of
 * (frame, level) and (frame, level, cell) work items processed by one launch
 * per stage, replayed as a CUDA graph when the frame list repeats.
 * images: one pointer per frame to device memory or to page-locked host
 * memory (read in place over the host link by the first kernel of the
 * pipeline), widths/heights/steps per frame.
 * Output for frame f starts at keypoints + f * per_frame_capacity (and the
 * same row of descriptors); n_keypoints[f] receives its count (device or
 * host per out_mem). */
typedef struct orbgpu_batch orbgpu_batch;
int orbgpu_batch_create(int max_frames, int max_width, int max_height, int max_nfeatures, void* stream,
                        orbgpu_batch** out);
int orbgpu_batch_destroy(orbgpu_batch* b);
int orbgpu_batch_extract(orbgpu_batch* b, int nframes, const uint8_t* const* images, const int* widths,
                         const int* heights, const size_t* steps, const int* nfeatures, float scale_factor,
                         int nlevels, int ini_th_fast, int min_th_fast, orbgpu_keypoint* keypoints,
                         uint8_t* descriptors, int per_frame_capacity, int out_mem, int* n_keypoints);
/* orbgpu_batch_extract without waiting: returns once the work is queued on
 * the batch's stream (orbgpu_batch_stream), so further work on that stream
 * (the batched searches) follows it without a host round trip.  The
 * extraction's status (capacity checks) is returned by orbgpu_batch_wait,
 * which synchronises the stream; the next extraction on the batch waits for
 * it first. */
int orbgpu_batch_extract_async(orbgpu_batch* b, int nframes, const uint8_t* const* images, const int* widths,
                               const int* heights, const size_t* steps, const int* nfeatures, float scale_factor,
                               int nlevels, int ini_th_fast, int min_th_fast, orbgpu_keypoint* keypoints,
                               uint8_t* descriptors, int per_frame_capacity, int out_mem, int* n_keypoints);
int orbgpu_batch_wait(orbgpu_batch* b);

/* ------------------------------------------------------------ matcher */
typedef struct orbgpu_matcher orbgpu_matcher;

/* A frame as the matchers read it (the fields of ORB_SLAM2::Frame that the
 * searches use): undistorted keypoints, descriptors (n x 32), optional
 * mvuRight (n floats, NULL = none), image bounds for the 64 x 48 grid
 * (src/Frame.cc:783-819 without distortion: [0, width] x [0, height]) and the
 * scale factors of its extractor.  All pointers share one memory flag. */
typedef struct {
    const orbgpu_keypoint* keypoints;
    const uint8_t* descriptors;
    const float* uright;
    int n;
    int width, height;
    int nlevels;
    float scale_factors[16];
    int mem;
} orbgpu_frame;

/* ORBmatcher::ORBmatcher(float nnratio, bool checkOri) -- include/ORBmatcher.h. */
int orbgpu_matcher_create(float nnratio, int check_orientation, void* stream, orbgpu_matcher** out);
int orbgpu_matcher_destroy(orbgpu_matcher* m);

/* ORBmatcher::SearchForInitialization(Frame& F1, Frame& F2,
 *     vector<Point2f>& vbPrevMatched, vector<int>& vnMatches12, int windowSize)
 * -- src/ORBmatcher.cc:573-717.  prev_matched: n1 x 2 floats (in/out),
 * matches12: n1 ints (out), both host memory.  Returns OK and *nmatches. */
int orbgpu_search_for_initialization(orbgpu_matcher* m, const orbgpu_frame* f1, const orbgpu_frame* f2,
                                     float* prev_matched, int* matches12, int window_size, int* nmatches);

/* One map point of ORBmatcher::SearchByProjection(Frame&, vector<MapPoint*>, th)
 * as Frame::isInFrustum leaves it (src/Frame.cc:491-578). */
typedef struct {
    float proj_x, proj_y, proj_xr, view_cos;
    int32_t track_scale_level;
    int32_t track_in_view;
    int32_t bad;
    int32_t pad;
} orbgpu_mappoint;

/* ORBmatcher::SearchByProjection(Frame& F, const vector<MapPoint*>& vpMapPoints,
 *     const float th) -- src/ORBmatcher.cc:72-183.
 * mappoints/mp_descriptors: m records and m x 32 bytes.  claimed: n bytes,
 * non-zero where F.mvpMapPoints[i] already holds a map point with
 * observations (NULL = none).  match_out: n ints, receives the index of the
 * map point assigned to keypoint i, -2 where claimed, -1 otherwise.
 * Host memory (mem = ORBGPU_MEM_HOST) or device memory. */
int orbgpu_search_by_projection(orbgpu_matcher* m, const orbgpu_frame* f, const orbgpu_mappoint* mappoints,
                                const uint8_t* mp_descriptors, int n_mappoints, float th, const uint8_t* claimed,
                                int* match_out, int mem, int* nmatches);

/* A DBoW2 vocabulary tree (ORBVocabulary, include/ORBVocabulary.h) resident
 * on the device. */
typedef struct orbgpu_vocabulary orbgpu_vocabulary;

/* TemplatedVocabulary::loadFromTextFile (Thirdparty/DBoW2/DBoW2/
 * TemplatedVocabulary.h:1368-1460): "k L scoring weighting", then one line
 * "parent is_leaf d0 .. d31 weight" per node after the root, in node order.
 * A line the reference would read only partly (an empty or short line: it
 * appends a node with unset descriptor bytes) is ORBGPU_ERR_BAD_ARG. */
int orbgpu_vocabulary_load_text(const char* path, orbgpu_vocabulary** out);
/* The same tree from arrays: nnodes counts the root; entry i of parents /
 * is_leaf / descriptors (32 bytes) / weights describes node i + 1, whose
 * parent must precede it.  scoring: DBoW2::ScoringType (L1_NORM 0 ..
 * DOT_PRODUCT 5); weighting: DBoW2::WeightingType (TF_IDF 0, TF 1, IDF 2,
 * BINARY 3).  Host arrays; the tree is copied to the device. */
int orbgpu_vocabulary_create(int k, int L, int scoring, int weighting, int nnodes, const int* parents,
                             const uint8_t* is_leaf, const uint8_t* descriptors, const double* weights,
                             orbgpu_vocabulary** out);
/* Waits for all device work (transforms run on the callers' streams), then
 * frees the tree. */
int orbgpu_vocabulary_destroy(orbgpu_vocabulary* v);
/* TemplatedVocabulary::size() (words) and the node count. */
int orbgpu_vocabulary_size(const orbgpu_vocabulary* v, int* nwords, int* nnodes);

/* Frame::ComputeBoW -- src/Frame.cc:704-718 -- i.e.
 * TemplatedVocabulary::transform(features, BowVector, FeatureVector,
 * levelsup) (TemplatedVocabulary.h:1136-1290) for the features of nframes
 * frames: frame f owns descriptor rows [offsets[f], offsets[f + 1]) of desc
 * (at most 8192 per frame).  Per feature i: word_ids[i], weights[i] (the
 * word's weight) and node_ids[i] (the node of level L - levelsup on its path;
 * the root when that level is <= 0).  Per frame f, written from index
 * offsets[f] on:
 *   BowVector      bow_counts[f] entries (word, value) in ascending word
 *                  order in bow_words / bow_values -- the reference's
 *                  std::map, doubles bit-identical (weights of repeated words
 *                  summed in sequence, normalised as the vocabulary's scoring
 *                  requires);
 *   FeatureVector  fv_counts[f] nodes in ascending order in fv_nodes, node j
 *                  owning fv_features[fv_starts[j] .. + fv_sizes[j]) (feature
 *                  indices within the frame, ascending; fv_starts are absolute
 *                  indices into fv_features).
 * Features whose word has weight 0 (stopped words) appear in neither, as in
 * the reference.  A frame of more than 8192 features gets counts of -1.
 * All arrays device or page-locked host memory (desc 16-byte aligned);
 * asynchronous on 'stream'; two kernel launches. */
int orbgpu_bow_transform(const orbgpu_vocabulary* v, const uint8_t* desc, const int* offsets, int nframes,
                         int levelsup, int* word_ids, double* weights, int* node_ids, int* bow_counts, int* bow_words,
                         double* bow_values, int* fv_counts, int* fv_nodes, int* fv_starts, int* fv_sizes,
                         int* fv_features, void* stream);

/* ORBmatcher::SearchByBoW(KeyFrame* pKF, Frame& F, vector<MapPoint*>&
 * vpMapPointMatches) -- src/ORBmatcher.cc:247-380 -- for npairs (keyframe,
 * frame) pairs in one launch, with the matcher's nnratio and checkOri.
 * Keyframes and frames are entries of one set laid out as
 * orbgpu_bow_transform's inputs and outputs: entry s owns keypoints /
 * descriptor rows [offsets[s], offsets[s + 1]) (at most 8192) and its
 * FeatureVector (fv_counts[s] nodes at fv_nodes / fv_starts / fv_sizes from
 * offsets[s], feature lists in fv_features).  pairs: 2 * npairs ints
 * (keyframe entry, frame entry).  kf_mappoints: one byte per row, 1 where
 * the keyframe's GetMapPointMatches()[i] is a map point that is not bad.
 * match_out: for pair p, the frame's rows at out_offsets[p]: the keyframe
 * feature whose map point vpMapPointMatches[i] receives, or -1.
 * nmatches[p]: the reference's return value (-1 for an entry beyond 8192
 * features).  Device or page-locked host memory; asynchronous; one launch. */
int orbgpu_search_by_bow(const orbgpu_keypoint* kps, const uint8_t* desc, const int* offsets, const int* fv_counts,
                         const int* fv_nodes, const int* fv_starts, const int* fv_sizes, const int* fv_features,
                         const uint8_t* kf_mappoints, const int* pairs, int npairs, float nnratio, int check_ori,
                         const int* out_offsets, int* match_out, int* nmatches, void* stream);

/* ORBmatcher::SearchByBoW(KeyFrame* pKF1, KeyFrame* pKF2, vector<MapPoint*>&
 * vpMatches12) -- src/ORBmatcher.cc:729-880 -- for npairs keyframe pairs:
 * the same set layout; pairs hold (pKF1 entry, pKF2 entry); kf_mappoints is
 * read for both sides (candidates in pKF2 need a map point that is not bad
 * too).  match_out: for pair p, pKF1's rows at out_offsets[p]: the pKF2
 * feature whose map point vpMatches12[i] receives, or -1. */
int orbgpu_search_by_bow_keyframes(const orbgpu_keypoint* kps, const uint8_t* desc, const int* offsets,
                                   const int* fv_counts, const int* fv_nodes, const int* fv_starts,
                                   const int* fv_sizes, const int* fv_features, const uint8_t* kf_mappoints,
                                   const int* pairs, int npairs, float nnratio, int check_ori, const int* out_offsets,
                                   int* match_out, int* nmatches, void* stream);

/* ORBmatcher::SearchForTriangulation(pKF1, pKF2, F12, vMatchedPairs,
 * bOnlyStereo) -- src/ORBmatcher.cc:884-1040, CheckDistEpipolarLine
 * :205-232 -- for npairs keyframe pairs: the set layout of
 * orbgpu_search_by_bow; has_mappoint: one byte per row, non-zero where
 * GetMapPoint(i) is not NULL (such features take no part); uright: one float
 * per row (mvuRight, >= 0 for stereo); pair_params: 11 floats per pair, F12
 * row-major then the epipole (ex, ey) in pKF2 (orbgpu_triangulation_epipole);
 * scale_factors / level_sigma2: pKF2's mvScaleFactors / mvLevelSigma2
 * (nlevels, host).  match_out: for pair p, pKF1's rows at out_offsets[p]: the
 * pKF2 feature paired with it (vMatchedPairs), or -1.  nmatches[p]: the
 * reference's return value.  The candidate a pKF1 feature takes is the last
 * at the least distance among those passing the tests, as the reference's
 * "dist > bestDist" skip leaves it. */
int orbgpu_search_for_triangulation(const orbgpu_keypoint* kps, const uint8_t* desc, const int* offsets,
                                    const int* fv_counts, const int* fv_nodes, const int* fv_starts,
                                    const int* fv_sizes, const int* fv_features, const uint8_t* has_mappoint,
                                    const float* uright, const int* pairs, int npairs, const float* pair_params,
                                    const float* scale_factors, const float* level_sigma2, int nlevels,
                                    int only_stereo, int check_ori, const int* out_offsets, int* match_out,
                                    int* nmatches, void* stream);
/* The epipole of SearchForTriangulation: pKF1's camera centre Cw1 seen by
 * pKF2 (T2: rows 0-2 of its Tcw; K2: fx, fy, cx, cy), as the reference
 * computes it (src/ORBmatcher.cc:897-906).  Host only. */
int orbgpu_triangulation_epipole(const float* Cw1, const float* T2, const float* K2, float* ex, float* ey);

/* Frame::UndistortKeyPoints() -- src/Frame.cc:724-776 -- for n keypoints of
 * one camera: out[i] = kps[i] with x, y through cv::undistortPoints(pts, pts,
 * mK, mDistCoef, cv::Mat(), mK) (OpenCV 3.2's algorithm: double precision,
 * five fixed-point rounds).  K4 = fx, fy, cx, cy (mK); dist = mDistCoef, k1
 * k2 p1 p2 [k3] (ndist 4 or 5); host arrays.  A zero k1 copies the keypoints
 * unchanged, as the reference does whatever the other coefficients.
 * kps / out: device or page-locked host memory (out may be kps).
 * Asynchronous on 'stream'; one kernel launch. */
int orbgpu_undistort_keypoints(const orbgpu_keypoint* kps, int n, const float* K4, const float* dist, int ndist,
                               orbgpu_keypoint* out, void* stream);

/* Frame::ComputeImageBounds(imLeft) -- src/Frame.cc:778-819 -- for an image
 * of cols x rows: bounds = mnMinX, mnMaxX, mnMinY, mnMaxY (the undistorted
 * corners, or the image rectangle when k1 is zero).  Host only, with the
 * same arithmetic as orbgpu_undistort_keypoints. */
int orbgpu_compute_image_bounds(int cols, int rows, const float* K4, const float* dist, int ndist, float* bounds);

/* The map point fields Frame::isInFrustum reads (src/Frame.cc:491-578). */
typedef struct {
    float x, y, z;          /* MapPoint::GetWorldPos() */
    float nx, ny, nz;       /* MapPoint::GetNormal() */
    float min_distance;     /* mfMinDistance (GetMinDistanceInvariance() is 0.8f times it) */
    float max_distance;     /* mfMaxDistance (GetMaxDistanceInvariance() is 1.2f times it) */
} orbgpu_mappoint_geometry;

/* The frame data isInFrustum and MapPoint::PredictScale(dist, Frame*) read:
 * mRcw, mtcw and mOw as Frame::UpdatePoseMatrices derives them from mTcw,
 * Frame::fx, fy, cx, cy, mbf, the image bounds mnMinX, mnMaxX, mnMinY,
 * mnMaxY, mnScaleLevels, and the predicted-level thresholds: PredictScale
 * returns #{n < nlevels - 1 : ratio > level_above[n]} (ratio =
 * mfMaxDistance / dist), the thresholds being where ceil(log(ratio) /
 * mfLogScaleFactor) steps, found with the host's logf.  Fill it with
 * orbgpu_frustum_frame_init. */
typedef struct {
    float Rcw[9];
    float tcw[3];
    float Ow[3];
    float fx, fy, cx, cy, bf;
    float min_x, max_x, min_y, max_y;
    int32_t nlevels;
    float level_above[15];
} orbgpu_frustum_frame;

/* Fills *out from rows 0-2 of the frame's mTcw (row-major 3 x 4), the
 * camera constants, the image bounds and the extractor's scale factor and
 * level count (Frame::mfScaleFactor, mnScaleLevels; mfLogScaleFactor =
 * logf(scale_factor) as in the Frame constructors).  Host only; nlevels 1-16,
 * scale_factor > 1. */
int orbgpu_frustum_frame_init(const float* Tcw, float fx, float fy, float cx, float cy, float bf, float min_x,
                              float max_x, float min_y, float max_y, float scale_factor, int nlevels,
                              orbgpu_frustum_frame* out);

/* Frame::isInFrustum(pMP, viewingCosLimit) -- src/Frame.cc:491-578, with
 * MapPoint::PredictScale(dist, this) (src/MapPoint.cc:604-619) -- for the map
 * points of nframes frames in one launch: frame f tests mps[mp_offsets[f] ..
 * mp_offsets[f + 1]).  For every map point it writes mappoints[i] as the
 * reference leaves the MapPoint: track_in_view (mbTrackInView), and where it
 * is 1 also proj_x, proj_y, proj_xr, view_cos and track_scale_level
 * (mTrackProjX, mTrackProjY, mTrackProjXR, mTrackViewCos,
 * mnTrackScaleLevel); where it is 0 those fields keep their values, and
 * 'bad' is never written -- so the records go straight to
 * orbgpu_search_by_projection / orbgpu_batch_search_by_projection.
 * in_view (nullable, device, nframes ints) receives the number of map points
 * in view per frame (Tracking::SearchLocalPoints' nToMatch).  frames,
 * mp_offsets, mps and mappoints may be device or page-locked host memory.
 * Asynchronous on 'stream'; one kernel launch (plus a memset of in_view). */
int orbgpu_is_in_frustum(const orbgpu_frustum_frame* frames, int nframes, const int* mp_offsets,
                         const orbgpu_mappoint_geometry* mps, float viewing_cos_limit, orbgpu_mappoint* mappoints,
                         int* in_view, void* stream);

/* ORBmatcher::SearchByProjection(Frame& CurrentFrame, KeyFrame* pKF, const
 * set<MapPoint*>& sAlreadyFound, th, ORBdist) -- src/ORBmatcher.cc:1891-2010
 * (relocalisation) -- with the matcher's checkOri.  current: the frame
 * searched; pose: its mTcw / camera / PredictScale thresholds as
 * orbgpu_frustum_frame_init fills them (the image bounds are the frame's
 * 0..width x 0..height); per keyframe feature i (n_kf of them):
 * kf_keypoints[i] (its angle is read), mappoints[i] / mp_descriptors[i] (the
 * map point's position, distances and GetDescriptor()), usable[i] = 1 where
 * GetMapPointMatches()[i] is a map point that is not bad and not in
 * sAlreadyFound.  claimed: current->n bytes, non-zero where
 * CurrentFrame.mvpMapPoints[i] is already set (NULL = none).  match_out:
 * current->n ints: >= 0 the keyframe feature whose map point now fills
 * CurrentFrame.mvpMapPoints[i]; -1 not assigned; -2 claimed before; -4
 * assigned and reset by the rotation check.  Host or device memory per
 * 'mem'; returns after the result is complete. */
int orbgpu_search_by_projection_keyframe(orbgpu_matcher* m, const orbgpu_frame* current,
                                         const orbgpu_frustum_frame* pose, const orbgpu_keypoint* kf_keypoints,
                                         const orbgpu_mappoint_geometry* mappoints, const uint8_t* mp_descriptors,
                                         const uint8_t* usable, int n_kf, float th, int orbdist,
                                         const uint8_t* claimed, int* match_out, int mem, int* nmatches);

/* ORBmatcher::SearchByProjection(KeyFrame* pKF, cv::Mat Scw, const
 * vector<MapPoint*>& vpPoints, vector<MapPoint*>& vpMatched, int th) --
 * src/ORBmatcher.cc:423-560 (loop closing).  keyframe: pKF's keypoints and
 * descriptors (image bounds 0..width x 0..height); Scw: rows 0-2 of the Sim3
 * (row-major 3 x 4, scale in the rotation block); fx..cy, scale_factor,
 * nlevels: pKF's camera and pyramid.  points / point_descriptors: vpPoints
 * (position, normal, distances; GetDescriptor()); usable[i] = 1 where
 * vpPoints[i] is not bad and not already in vpMatched.  matched:
 * keyframe->n bytes, non-zero where vpMatched[i] is set before the call
 * (NULL = none).  match_out: keyframe->n ints: >= 0 the vpPoints index now in
 * vpMatched[i], -2 set before, -1 none.  Host or device memory per 'mem'. */
int orbgpu_search_by_projection_sim3(orbgpu_matcher* m, const orbgpu_frame* keyframe, const float* Scw, float fx,
                                     float fy, float cx, float cy, float scale_factor, int nlevels,
                                     const orbgpu_mappoint_geometry* points, const uint8_t* point_descriptors,
                                     const uint8_t* usable, int npoints, int th, const uint8_t* matched,
                                     int* match_out, int mem, int* nmatches);

/* ORBmatcher::Fuse(KeyFrame* pKF, const vector<MapPoint*>& vpMapPoints,
 * th) -- src/ORBmatcher.cc:1107-1245 -- the search half: for every map point
 * the keyframe feature it fuses with (target[i], -1 for none; dist[i] its
 * distance, nullable), i.e. the first feature at the least distance among
 * those of its window (levels predicted - 1 .. predicted) that pass the
 * reprojection gate (chi-square 7.8 with mvuRight, 5.99 without), kept when
 * <= TH_LOW.  The choice does not depend on the other map points; the map
 * updates it leads to (MapPoint::Replace when the feature holds a map point
 * that is not bad, else AddObservation / AddMapPoint; the count nFused)
 * mutate the map and are applied by the caller in vpMapPoints order,
 * re-checking isBad() and IsInKeyFrame(pKF) at each step as the reference
 * does.  keyframe: pKF's keypoints, descriptors and mvuRight (uright);
 * Tcw: rows 0-2 of its pose; fx..bf: its camera; scale_factor, nlevels,
 * inv_level_sigma2 (nlevels floats, host): its pyramid.  usable[i] = 1 where
 * vpMapPoints[i] exists, is not bad and not in pKF at the start of the call.
 * Host or device memory per 'mem'. */
int orbgpu_fuse_candidates(orbgpu_matcher* m, const orbgpu_frame* keyframe, const float* Tcw, float fx, float fy,
                           float cx, float cy, float bf, float scale_factor, int nlevels,
                           const float* inv_level_sigma2, const orbgpu_mappoint_geometry* mappoints,
                           const uint8_t* mp_descriptors, const uint8_t* usable, int n_mp, float th, int* target,
                           int* dist, int mem);

/* ORBmatcher::Fuse(KeyFrame* pKF, cv::Mat Scw, const vector<MapPoint*>&
 * vpPoints, float th, vector<MapPoint*>& vpReplacePoint) --
 * src/ORBmatcher.cc:1290-1380 (loop correction) -- the search half: per
 * point the keyframe feature it fuses with (target, -1 none; dist
 * nullable), as orbgpu_fuse_candidates but through the de-scaled Sim3 and
 * without a reprojection gate.  usable[i] = 1 where vpPoints[i] is not bad
 * and not among pKF->GetMapPoints() at the start.  The caller applies, in
 * order, vpReplacePoint[i] = GetMapPoint(target) when that is a map point
 * not bad, else AddObservation / AddMapPoint.  Scw: rows 0-2 of the Sim3. */
int orbgpu_fuse_sim3_candidates(orbgpu_matcher* m, const orbgpu_frame* keyframe, const float* Scw, float fx,
                                float fy, float cx, float cy, float scale_factor, int nlevels,
                                const orbgpu_mappoint_geometry* points, const uint8_t* point_descriptors,
                                const uint8_t* usable, int npoints, float th, int* target, int* dist, int mem);

/* ORBmatcher::SearchBySim3(KeyFrame* pKF1, KeyFrame* pKF2, vpMatches12,
 * s12, R12, t12, th) -- src/ORBmatcher.cc:1441-1640: pKF1's map points
 * projected into pKF2 through the Sim3 and pKF2's into pKF1, each taking the
 * first least distance in its window (<= TH_HIGH), kept where the two agree.
 * kf1 / kf2: the keyframes' keypoints and descriptors (image bounds
 * 0..width x 0..height); T1w / T2w: rows 0-2 of their poses; s12, R12
 * (row-major 3 x 3), t12: the Sim3; fx..cy: pKF1's camera (the reference
 * projects into both with it); scale_factor, nlevels: the pyramid.  Per
 * keyframe feature: mps / mpd (its map point's geometry and descriptor),
 * usable1[i] = 1 where pKF1's map point i exists, is not bad and
 * vpMatches12[i] is NULL; usable2[i] = 1 where pKF2's map point i exists, is
 * not bad and i is not vpMatches12[j]->GetIndexInKeyFrame(pKF2) for any
 * non-NULL vpMatches12[j] (the reference's vbAlreadyMatched2,
 * src/ORBmatcher.cc:1478-1490: the pKF2 index of an already matched map
 * point, not the map point's own slot).  match12 (host, kf1->n ints): the
 * pKF2 feature whose map point vpMatches12[i] receives, or -1 (also for
 * entries that were already set); *nfound the reference's return value (new
 * matches only).
 * Host arrays; returns after the result is complete. */
int orbgpu_search_by_sim3(orbgpu_matcher* m, const orbgpu_frame* kf1, const orbgpu_frame* kf2, const float* T1w,
                          const float* T2w, float s12, const float* R12, const float* t12, float fx, float fy,
                          float cx, float cy, float scale_factor, int nlevels, const orbgpu_mappoint_geometry* mps1,
                          const uint8_t* mpd1, const uint8_t* usable1, const orbgpu_mappoint_geometry* mps2,
                          const uint8_t* mpd2, const uint8_t* usable2, float th, int* match12, int* nfound);

/* One entry of LastFrame.mvpMapPoints for orbgpu_search_by_projection_frame,
 * indexed like LastFrame's keypoints. */
typedef struct {
    float x, y, z; /* MapPoint::GetWorldPos() */
    int32_t flags; /* ORBGPU_MP_* */
} orbgpu_frame_mappoint;
#define ORBGPU_MP_PRESENT 1  /* LastFrame.mvpMapPoints[i] != NULL */
#define ORBGPU_MP_OUTLIER 2  /* LastFrame.mvbOutlier[i] */
#define ORBGPU_MP_OBSERVED 4 /* MapPoint::Observations() > 0 */

/* Camera data of that search: rows 0-2 of CurrentFrame.mTcw and
 * LastFrame.mTcw (row-major 3 x 4), Frame::fx, fy, cx, cy and the current
 * frame's mbf and mb. */
typedef struct {
    float Tcw[12];
    float Tlw[12];
    float fx, fy, cx, cy;
    float bf, b;
} orbgpu_frame_motion;

/* ORBmatcher::SearchByProjection(Frame& CurrentFrame, const Frame& LastFrame,
 *     const float th, const bool bMono) -- src/ORBmatcher.cc:1710-1879,
 * with the matcher's checkOri for the rotation check.
 * current: the frame searched (keypoints, descriptors, optional mvuRight);
 * last: LastFrame's keypoints (octave and angle are read; descriptors may be
 * NULL); last_mappoints / last_mp_descriptors: last->n records and
 * last->n x 32 bytes (MapPoint::GetDescriptor()).  claimed: current->n bytes,
 * non-zero where CurrentFrame.mvpMapPoints[i] already holds a map point with
 * observations (NULL = none).  match_out: current->n ints: >= 0 the LastFrame
 * keypoint whose map point now fills CurrentFrame.mvpMapPoints[i]; -1 not
 * assigned by this call; -2 claimed; -4 assigned and then reset to NULL by
 * the rotation check.  *nmatches: the reference's return value (it counts
 * reassignments, as the reference does).  last_mappoints, last_mp_descriptors,
 * claimed and match_out are host or device memory per 'mem'; the frames
 * carry their own flag. */
int orbgpu_search_by_projection_frame(orbgpu_matcher* m, const orbgpu_frame* current, const orbgpu_frame* last,
                                      const orbgpu_frame_mappoint* last_mappoints, const uint8_t* last_mp_descriptors,
                                      const orbgpu_frame_motion* motion, float th, int mono, const uint8_t* claimed,
                                      int* match_out, int mem, int* nmatches);

/* Frame::ComputeStereoMatches() -- src/Frame.cc:831-1082.
 * left/right: the two extractor handles that produced the frames (their
 * pyramids are read in place).  bf = mbf, fx = K(0,0); mb = bf/fx.
 * uright/depth: nL floats each (host or device per 'mem'). */
int orbgpu_compute_stereo_matches(orbgpu_matcher* m, const orbgpu_extractor* left, const orbgpu_extractor* right,
                                  const orbgpu_frame* fl, const orbgpu_frame* fr, float bf, float fx, float* uright,
                                  float* depth, int mem);

/* Brute-force k = 2 Hamming nearest neighbours over ORBmatcher::DescriptorDistance
 * semantics (src/ORBmatcher.cc:2083): for each query row, the best and the
 * second-best train rows, ties to the lower train index.  Not a reference
 * function: the build's batched matcher.  algo: 0 = popcount kernel, 1 =
 * tensor cores (+-1 FP8 dot products, tcgen05), -1 = automatic (the tensor
 * cores from the tuned problem size on, see orbgpu_tune_set); all give the
 * same results.  All arrays on the device. */
int orbgpu_knn2(orbgpu_matcher* m, const uint8_t* query, int nq, const uint8_t* train, int nt, int* idx1, int* d1,
                int* idx2, int* d2, int algo);

/* The ratio test of a k = 2 result in the reference's form
 * (src/ORBmatcher.cc:647: bestDist < bestDist2 * nnratio, as floats):
 * accept[i] = 1 where d1[i] < ratio * d2[i] (a query without a second
 * neighbour is rejected).  Device arrays; returns after the stream finished. */
int orbgpu_knn2_accept(const int* d1, const int* d2, int n, float ratio, uint8_t* accept, void* stream);

/* The same k = 2 search as orbgpu_knn2 (popcount kernel), for callers that
 * cannot allocate device memory: processes whose device memory is reserved up
 * front by their own allocator (a library cudaMalloc would fail or fragment
 * it) and real-time paths where cudaMalloc/cudaFree's implicit device-wide
 * synchronisation would stall other streams.  No counterpart in the
 * reference.
 * It allocates nothing: its scratch is a fixed 16 MiB device array inside
 * the library, one (best, second) pair per query row per train slice, so nq
 * is limited to 1048576 (ORBGPU_ERR_BAD_ARG beyond).  Every GPU that loads
 * the library holds that array until the process exits.  The first call on
 * a device looks up the array's device address (cudaGetSymbolAddress) with
 * that device current; make that first call before any stream capture.
 * The address is kept for the life of the process: after a cudaDeviceReset
 * of that device (which ends the context the address belongs to) this entry
 * point must not be called again in the same process.
 * All calls share the one array: calls that overlap on the GPU (different
 * streams, or host threads) race and give wrong results; serialise them.
 * Asynchronous on 'stream' (NULL = the legacy default stream); all arrays on
 * the device. */
int orbgpu_knn2_noalloc(const uint8_t* query, int nq, const uint8_t* train, int nt, int* idx1, int* d1, int* idx2,
                        int* d2, void* stream);

/* ORBmatcher::DescriptorDistance for n row pairs (device arrays). */
int orbgpu_descriptor_distance(const uint8_t* a, const uint8_t* b, int n, int* out, void* stream);

/* MapPoint::ComputeDistinctiveDescriptors (src/MapPoint.cc:365-447) for m map
 * points in one launch.  Each map point's observations are a list of rows of
 * a descriptor pool (pool_rows x 32 bytes: the observing keyframes'
 * mDescriptors, e.g. their extraction outputs left resident), given in CSR
 * form -- map point i owns obs_rows[obs_offsets[i] .. obs_offsets[i + 1]) --
 * in the order MapPoint::mObservations iterates them; a row of -1 is an
 * observation whose keyframe is bad (skipped, as KeyFrame::isBad() at
 * src/MapPoint.cc:391).  For every map point the descriptor with the least
 * median Hamming distance to the others is chosen, the first such in list
 * order (the reference's strict '<'), with the median taken as element
 * (size_t)(0.5 * (N - 1)) of the sorted distance row of the N valid
 * descriptors.
 *   best_rows[i]   the chosen pool row; -1 when the list has no valid
 *                  observation (the reference returns early and keeps
 *                  mDescriptor); -2 when the list is malformed (a row outside
 *                  [-1, pool_rows), offsets decreasing, negative or beyond
 *                  n_obs), where the reference would index out of range.
 *   descriptors    (nullable, m x 32) the chosen descriptor of every map point
 *                  with best_rows[i] >= 0; other rows are left unchanged, as
 *                  mDescriptor is.
 * No counterpart is needed for the per-map-point call: one list is m = 1.
 * Arrays may be device memory or page-locked host memory (read in place);
 * pool and descriptors 16-byte aligned.  Asynchronous on 'stream' (NULL = the
 * legacy default stream); one kernel launch, no allocation. */
int orbgpu_distinctive_descriptors(const uint8_t* pool, int pool_rows, const int* obs_offsets, const int* obs_rows,
                                   int n_obs, int m, int* best_rows, uint8_t* descriptors, void* stream);

#ifdef __cplusplus
}
#endif
#endif
