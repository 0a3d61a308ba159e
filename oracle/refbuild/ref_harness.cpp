// ORACLE / TEST INFRASTRUCTURE ONLY.
//
// C entry points around the reference's own, unmodified ORB-SLAM2 sources
// (src/ORBextractor.cc, src/ORBmatcher.cc, src/Frame.cc, src/MapPoint.cc),
// compiled against the
// cv stand-in in ../cvshim.  Used to pin the oracle restatement
// (../orb_oracle.cpp) and to generate the golden fixtures under tests/golden.
//
// Determinism of DistributeOctTree: src/ORBextractor.cc:926 sorts
// (size, ExtractorNode*) pairs, so equal-size nodes are ordered by heap
// address.  This library replaces the global allocator with a monotonic arena,
// which makes address order equal allocation order, i.e. the order in which
// the std::list nodes were created.  The restatement and the CUDA kernels use
// that creation order explicitly.
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <list>
#include <map>
#include <mutex>
#include <new>
#include <set>
#include <string>
#include <thread>
#include <vector>
#include <sys/mman.h>

#include <opencv2/core/core.hpp>

// The harness needs Frame::AssignFeaturesToGrid (private), MapPoint's
// protected fields and KeyFrame::mbBad (protected) to build frames, keyframes
// and map points from recorded data; the reference files themselves are
// compiled unchanged.
#define private public
#define protected public
#include "Frame.h"
#include "KeyFrame.h"
#include "Map.h"
#include "MapPoint.h"
#include "ORBextractor.h"
#include "ORBmatcher.h"
#undef private
#undef protected

#include "../orb_types.h"

// ------------------------------------------------------------------ arena
namespace {
struct Arena {
    char* base = nullptr;
    size_t cap = 0;
    size_t top = 0;
    size_t mark = 0;
    long live_since_mark = 0;
    Arena() {
        cap = (size_t)64 << 30;
        void* p = mmap(nullptr, cap, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS | MAP_NORESERVE, -1, 0);
        if (p == MAP_FAILED) { std::fprintf(stderr, "ref arena: mmap failed\n"); std::abort(); }
        base = (char*)p;
    }
    void* alloc(size_t n) {
        n = (n + 15) & ~(size_t)15;
        if (n == 0) n = 16;
        if (top + n > cap) { std::fprintf(stderr, "ref arena exhausted\n"); std::abort(); }
        void* p = base + top;
        top += n;
        live_since_mark++;
        return p;
    }
    bool owns(void* p) const { return (char*)p >= base && (char*)p < base + cap; }
    void release(void* p) {
        if ((size_t)((char*)p - base) >= mark) live_since_mark--;
    }
};
Arena& arena() {
    static Arena* a = new (std::malloc(sizeof(Arena))) Arena();
    return *a;
}
// Scope of one harness call: everything allocated inside and freed before the
// end is reclaimed, so repeated calls do not grow the arena.
struct ArenaScope {
    size_t saved_mark;
    long saved_live;
    ArenaScope() {
        Arena& a = arena();
        saved_mark = a.mark;
        saved_live = a.live_since_mark;
        a.mark = a.top;
        a.live_since_mark = 0;
    }
    ~ArenaScope() {
        Arena& a = arena();
        if (a.live_since_mark == 0) {
            const size_t page = 4096;
            size_t lo = (a.mark + page - 1) & ~(page - 1);
            if (a.top > lo) madvise(a.base + lo, a.top - lo, MADV_DONTNEED);
            a.top = a.mark;
        }
        a.mark = saved_mark;
        a.live_since_mark = saved_live + a.live_since_mark;
    }
};
}  // namespace

void* operator new(size_t n) { return arena().alloc(n); }
void* operator new[](size_t n) { return arena().alloc(n); }
void* operator new(size_t n, const std::nothrow_t&) noexcept { return arena().alloc(n); }
void* operator new[](size_t n, const std::nothrow_t&) noexcept { return arena().alloc(n); }
void operator delete(void* p) noexcept {
    if (!p) return;
    if (arena().owns(p)) arena().release(p);
    else std::free(p);
}
void operator delete[](void* p) noexcept { operator delete(p); }
void operator delete(void* p, size_t) noexcept { operator delete(p); }
void operator delete[](void* p, size_t) noexcept { operator delete(p); }

using namespace ORB_SLAM2;

namespace {

void copy_kps_out(const std::vector<cv::KeyPoint>& kps, orc_kp* out) {
    for (size_t i = 0; i < kps.size(); i++) {
        out[i].x = kps[i].pt.x;
        out[i].y = kps[i].pt.y;
        out[i].size = kps[i].size;
        out[i].angle = kps[i].angle;
        out[i].response = kps[i].response;
        out[i].octave = kps[i].octave;
        out[i].class_id = kps[i].class_id;
    }
}

std::vector<cv::KeyPoint> kps_in(const orc_kp* kps, int n) {
    std::vector<cv::KeyPoint> v(n);
    for (int i = 0; i < n; i++)
        v[i] = cv::KeyPoint(kps[i].x, kps[i].y, kps[i].size, kps[i].angle, kps[i].response, kps[i].octave,
                            kps[i].class_id);
    return v;
}

// Map points built through the reference's own constructor
// (src/MapPoint.cc:39-67), which reads its reference keyframe's ids and locks
// the map's point-creation mutex: one map and one reference keyframe per
// harness call.  The matchers read only Observations() > 0 of a map point, so
// make() sets nObs directly.
struct MapPointMaker {
    Map* map;
    Frame* frame;
    KeyFrame* kf;
    MapPointMaker() : map(new Map()), frame(new Frame()) {
        frame->mnId = 0;
        frame->N = 0;
        kf = new KeyFrame(*frame, map, nullptr);
    }
    ~MapPointMaker() {
        delete kf;
        delete frame;
        delete map;
    }
    MapPoint* make(const cv::Mat& pos, int nobs) {
        MapPoint* mp = new MapPoint(pos, kf, map);
        mp->nObs = nobs;
        return mp;
    }
};

// A Frame as the reference's constructors leave it (src/Frame.cc:313-393 for
// an image without distortion), built from recorded keypoints/descriptors.
Frame* make_frame(ORBextractor* ext, const orc_kp* kps, const uint8_t* desc, int n, int w, int h, const float* uright) {
    Frame* F = new Frame();
    F->mpORBextractorLeft = ext;
    F->mpORBextractorRight = nullptr;
    F->N = n;
    F->mvKeys = kps_in(kps, n);
    F->mvKeysUn = F->mvKeys;
    F->mDescriptors = cv::Mat(n, 32, CV_8U);
    if (n) std::memcpy(F->mDescriptors.data, desc, (size_t)n * 32);
    F->mvuRight = std::vector<float>(n, -1.f);
    if (uright)
        for (int i = 0; i < n; i++) F->mvuRight[i] = uright[i];
    F->mvDepth = std::vector<float>(n, -1.f);
    F->mvpMapPoints = std::vector<MapPoint*>(n, static_cast<MapPoint*>(NULL));
    F->mvbOutlier = std::vector<bool>(n, false);
    F->mnScaleLevels = ext->GetLevels();
    F->mfScaleFactor = ext->GetScaleFactor();
    F->mvScaleFactors = ext->GetScaleFactors();
    F->mvInvScaleFactors = ext->GetInverseScaleFactors();
    F->mvLevelSigma2 = ext->GetScaleSigmaSquares();
    F->mvInvLevelSigma2 = ext->GetInverseScaleSigmaSquares();
    // ComputeImageBounds without distortion + the grid constants
    // (src/Frame.cc:783-819, :372-388).
    Frame::mnMinX = 0.0f;
    Frame::mnMaxX = w;
    Frame::mnMinY = 0.0f;
    Frame::mnMaxY = h;
    Frame::mfGridElementWidthInv = static_cast<float>(FRAME_GRID_COLS) / static_cast<float>(Frame::mnMaxX - Frame::mnMinX);
    Frame::mfGridElementHeightInv = static_cast<float>(FRAME_GRID_ROWS) / static_cast<float>(Frame::mnMaxY - Frame::mnMinY);
    F->AssignFeaturesToGrid();
    return F;
}

}  // namespace

extern "C" {

// ORBextractor(...)(image, Mat(), keypoints, descriptors) -- src/ORBextractor.cc:1533.
// pyr (optional) receives the unblurred pyramid levels back to back.
int ref_extract(const uint8_t* img, int w, int h, size_t step, const orc_params* p, orc_kp* kps, uint8_t* desc,
                int cap, int* n_out, uint8_t* pyr, size_t pyr_cap) {
    ArenaScope scope;
    int rc = 0;
    {
        ORBextractor ext(p->nfeatures, p->scale_factor, p->nlevels, p->ini_th_fast, p->min_th_fast);
        cv::Mat image(h, w, CV_8UC1, (void*)img, step);
        std::vector<cv::KeyPoint> keys;
        cv::Mat descriptors;
        ext(image, cv::Mat(), keys, descriptors);
        *n_out = (int)keys.size();
        if ((int)keys.size() > cap) rc = -1;
        else {
            copy_kps_out(keys, kps);
            if (!keys.empty()) std::memcpy(desc, descriptors.data, keys.size() * 32);
        }
        if (pyr) {
            size_t off = 0;
            for (int l = 0; l < p->nlevels && rc == 0; l++) {
                const cv::Mat& L = ext.mvImagePyramid[l];
                if (off + (size_t)L.rows * L.cols > pyr_cap) { rc = -2; break; }
                for (int y = 0; y < L.rows; y++) std::memcpy(pyr + off + (size_t)y * L.cols, L.ptr(y), L.cols);
                off += (size_t)L.rows * L.cols;
            }
        }
    }
    return rc;
}

// Scale tables and per-level budgets of the ORBextractor constructor
// (src/ORBextractor.cc:469-571).
int ref_extractor_tables(const orc_params* p, float* scale, float* inv_scale, float* sigma2, float* inv_sigma2,
                         int* features_per_level, int* umax16) {
    ArenaScope scope;
    {
        ORBextractor ext(p->nfeatures, p->scale_factor, p->nlevels, p->ini_th_fast, p->min_th_fast);
        for (int l = 0; l < p->nlevels; l++) {
            scale[l] = ext.mvScaleFactor[l];
            inv_scale[l] = ext.mvInvScaleFactor[l];
            sigma2[l] = ext.mvLevelSigma2[l];
            inv_sigma2[l] = ext.mvInvLevelSigma2[l];
            features_per_level[l] = ext.mnFeaturesPerLevel[l];
        }
        for (int v = 0; v < 16; v++) umax16[v] = ext.umax[v];
    }
    return 0;
}

int ref_descriptor_distance(const uint8_t* a, const uint8_t* b) {
    ArenaScope scope;
    int d;
    {
        cv::Mat A(1, 32, CV_8U, (void*)a), B(1, 32, CV_8U, (void*)b);
        d = ORBmatcher::DescriptorDistance(A, B);
    }
    return d;
}

// Frame::GetFeaturesInArea (src/Frame.cc:590) on a frame built from keypoints.
int ref_features_in_area(const orc_params* p, const orc_kp* kps, int n, int w, int h, float x, float y, float r,
                         int minLevel, int maxLevel, int* out, int cap) {
    ArenaScope scope;
    int cnt;
    {
        ORBextractor ext(p->nfeatures, p->scale_factor, p->nlevels, p->ini_th_fast, p->min_th_fast);
        std::vector<uint8_t> desc((size_t)n * 32 + 32, 0);
        Frame* F = make_frame(&ext, kps, desc.data(), n, w, h, nullptr);
        std::vector<size_t> v = F->GetFeaturesInArea(x, y, r, minLevel, maxLevel);
        cnt = (int)v.size();
        for (int i = 0; i < cnt && i < cap; i++) out[i] = (int)v[i];
        delete F;
    }
    return cnt;
}

// ORBmatcher(nnratio, checkOri).SearchForInitialization(F1, F2, vbPrevMatched,
// vnMatches12, windowSize) -- src/ORBmatcher.cc:573-717.
int ref_search_for_initialization(const orc_params* p, const orc_kp* kps1, const uint8_t* desc1, int n1,
                                  const orc_kp* kps2, const uint8_t* desc2, int n2, int w, int h,
                                  float* prev_matched_xy, int window, float nnratio, int check_ori,
                                  int* matches12) {
    ArenaScope scope;
    int nm;
    {
        ORBextractor ext(p->nfeatures, p->scale_factor, p->nlevels, p->ini_th_fast, p->min_th_fast);
        Frame* F1 = make_frame(&ext, kps1, desc1, n1, w, h, nullptr);
        Frame* F2 = make_frame(&ext, kps2, desc2, n2, w, h, nullptr);
        std::vector<cv::Point2f> prev(n1);
        for (int i = 0; i < n1; i++) prev[i] = cv::Point2f(prev_matched_xy[2 * i], prev_matched_xy[2 * i + 1]);
        std::vector<int> m12;
        ORBmatcher matcher(nnratio, check_ori != 0);
        nm = matcher.SearchForInitialization(*F1, *F2, prev, m12, window);
        for (int i = 0; i < n1; i++) {
            matches12[i] = m12[i];
            prev_matched_xy[2 * i] = prev[i].x;
            prev_matched_xy[2 * i + 1] = prev[i].y;
        }
        delete F1;
        delete F2;
    }
    return nm;
}

// ORBmatcher(nnratio).SearchByProjection(F, vpMapPoints, th) -- src/ORBmatcher.cc:72-183.
// claimed[i] != 0 marks frame keypoints that already hold a map point with
// observations (skipped by :128-130).  match_out[i] receives the index of the
// map point now assigned to keypoint i, -2 for a pre-claimed keypoint, -1 for none.
int ref_search_by_projection(const orc_params* p, const orc_kp* kps, const uint8_t* desc, const float* uright,
                             int n, int w, int h, const orc_mappoint* mps, const uint8_t* mp_desc, int m,
                             float th, float nnratio, const uint8_t* claimed, int* match_out) {
    ArenaScope scope;
    int nm;
    {
        ORBextractor ext(p->nfeatures, p->scale_factor, p->nlevels, p->ini_th_fast, p->min_th_fast);
        Frame* F = make_frame(&ext, kps, desc, n, w, h, uright);
        cv::Mat pos = cv::Mat::zeros(3, 1, CV_32F);
        MapPointMaker maker;
        MapPoint* preclaimed = maker.make(pos, 1);
        std::vector<MapPoint*> vmp(m);
        std::map<MapPoint*, int> index;
        for (int i = 0; i < m; i++) {
            MapPoint* mp = maker.make(pos, 1);
            mp->mTrackProjX = mps[i].proj_x;
            mp->mTrackProjY = mps[i].proj_y;
            mp->mTrackProjXR = mps[i].proj_xr;
            mp->mTrackViewCos = mps[i].view_cos;
            mp->mnTrackScaleLevel = mps[i].track_scale_level;
            mp->mbTrackInView = mps[i].track_in_view != 0;
            mp->mbBad = mps[i].bad != 0;
            mp->mDescriptor = cv::Mat(1, 32, CV_8U);
            std::memcpy(mp->mDescriptor.data, mp_desc + (size_t)i * 32, 32);
            vmp[i] = mp;
            index[mp] = i;
        }
        for (int i = 0; i < n; i++)
            if (claimed && claimed[i]) F->mvpMapPoints[i] = preclaimed;
        ORBmatcher matcher(nnratio, true);
        nm = matcher.SearchByProjection(*F, vmp, th);
        for (int i = 0; i < n; i++) {
            MapPoint* mp = F->mvpMapPoints[i];
            match_out[i] = mp == nullptr ? -1 : (mp == preclaimed ? -2 : index[mp]);
        }
        for (int i = 0; i < m; i++) delete vmp[i];
        delete preclaimed;
        delete F;
    }
    return nm;
}

// ORBmatcher::SearchByProjection(Frame& CurrentFrame, const Frame& LastFrame,
// th, bMono) -- src/ORBmatcher.cc:1710-1879.  Current keypoints without a
// pre-claimed map point start with a sentinel map point that has no
// observations (it blocks nothing, exactly like NULL), so that an entry the
// rotation check resets to NULL can be told from an untouched one.
int ref_search_by_projection_frame(const orc_params* p, const orc_kp* kps, const uint8_t* desc, const float* uright,
                                   int n, int w, int h, const orc_kp* last_kps, int n_last,
                                   const orc_frame_mappoint* last_mps, const uint8_t* last_mp_desc,
                                   const orc_frame_motion* mo, float th, int mono, int check_ori,
                                   const uint8_t* claimed, int* match_out) {
    ArenaScope scope;
    int nm;
    {
        ORBextractor ext(p->nfeatures, p->scale_factor, p->nlevels, p->ini_th_fast, p->min_th_fast);
        std::vector<uint8_t> no_desc((size_t)std::max(1, n_last) * 32, 0);
        Frame* LF = make_frame(&ext, last_kps, no_desc.data(), n_last, w, h, nullptr);
        Frame* CF = make_frame(&ext, kps, desc, n, w, h, uright);
        CF->mTcw = cv::Mat::eye(4, 4, CV_32F);
        LF->mTcw = cv::Mat::eye(4, 4, CV_32F);
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 4; c++) {
                CF->mTcw.at<float>(r, c) = mo->Tcw[4 * r + c];
                LF->mTcw.at<float>(r, c) = mo->Tlw[4 * r + c];
            }
        Frame::fx = mo->fx;
        Frame::fy = mo->fy;
        Frame::cx = mo->cx;
        Frame::cy = mo->cy;
        Frame::invfx = 1.0f / mo->fx;
        Frame::invfy = 1.0f / mo->fy;
        CF->mbf = mo->bf;
        CF->mb = mo->b;
        cv::Mat zero = cv::Mat::zeros(3, 1, CV_32F);
        MapPointMaker maker;
        MapPoint* preclaimed = maker.make(zero, 1);
        MapPoint* sentinel = maker.make(zero, 0);
        std::vector<MapPoint*> owned;
        std::map<MapPoint*, int> index;
        for (int i = 0; i < n_last; i++) {
            const orc_frame_mappoint& q = last_mps[i];
            LF->mvbOutlier[i] = (q.flags & ORC_MP_OUTLIER) != 0;
            if (!(q.flags & ORC_MP_PRESENT)) continue;
            cv::Mat pos(3, 1, CV_32F);
            pos.at<float>(0) = q.x;
            pos.at<float>(1) = q.y;
            pos.at<float>(2) = q.z;
            MapPoint* mp = maker.make(pos, (q.flags & ORC_MP_OBSERVED) ? 1 : 0);
            mp->mDescriptor = cv::Mat(1, 32, CV_8U);
            std::memcpy(mp->mDescriptor.data, last_mp_desc + (size_t)i * 32, 32);
            LF->mvpMapPoints[i] = mp;
            owned.push_back(mp);
            index[mp] = i;
        }
        for (int i = 0; i < n; i++) CF->mvpMapPoints[i] = (claimed && claimed[i]) ? preclaimed : sentinel;
        ORBmatcher matcher(0.9f, check_ori != 0);
        nm = matcher.SearchByProjection(*CF, *LF, th, mono != 0);
        for (int i = 0; i < n; i++) {
            MapPoint* mp = CF->mvpMapPoints[i];
            match_out[i] = mp == nullptr ? -4 : mp == sentinel ? -1 : mp == preclaimed ? -2 : index[mp];
        }
        for (MapPoint* mp : owned) delete mp;
        delete preclaimed;
        delete sentinel;
        delete CF;
        delete LF;
    }
    return nm;
}

// Frame::ComputeStereoMatches -- src/Frame.cc:831-1082, on frames built from
// recorded keypoints and the unblurred pyramids (levels back to back).  mb is
// set to mbf/fx first: the stereo constructor reads it before assigning it
// (src/Frame.cc:154 vs :202), and mbf/fx is its value for every later frame.
int ref_compute_stereo_matches(const orc_params* p, const orc_kp* kpsL, const uint8_t* descL, int nL,
                               const orc_kp* kpsR, const uint8_t* descR, int nR, const uint8_t* pyrL,
                               const uint8_t* pyrR, const int* level_w, const int* level_h, int w, int h, float bf,
                               float fx, float* uright, float* depth) {
    ArenaScope scope;
    {
        ORBextractor extL(p->nfeatures, p->scale_factor, p->nlevels, p->ini_th_fast, p->min_th_fast);
        ORBextractor extR(p->nfeatures, p->scale_factor, p->nlevels, p->ini_th_fast, p->min_th_fast);
        size_t off = 0;
        for (int l = 0; l < p->nlevels; l++) {
            extL.mvImagePyramid[l] = cv::Mat(level_h[l], level_w[l], CV_8UC1, (void*)(pyrL + off));
            extR.mvImagePyramid[l] = cv::Mat(level_h[l], level_w[l], CV_8UC1, (void*)(pyrR + off));
            off += (size_t)level_w[l] * level_h[l];
        }
        Frame* F = make_frame(&extL, kpsL, descL, nL, w, h, nullptr);
        F->mpORBextractorRight = &extR;
        F->mvKeysRight = kps_in(kpsR, nR);
        F->mDescriptorsRight = cv::Mat(nR, 32, CV_8U);
        if (nR) std::memcpy(F->mDescriptorsRight.data, descR, (size_t)nR * 32);
        F->mbf = bf;
        Frame::fx = fx;
        F->mb = F->mbf / Frame::fx;
        F->ComputeStereoMatches();
        for (int i = 0; i < nL; i++) {
            uright[i] = F->mvuRight[i];
            depth[i] = F->mvDepth[i];
        }
        delete F;
    }
    return 0;
}

// Brute-force k=2 over ORBmatcher::DescriptorDistance (src/ORBmatcher.cc:2083):
// for each query, best and second-best train rows, ties to the lower index.
int ref_knn2(const uint8_t* q, int nq, const uint8_t* t, int nt, int* idx1, int* d1, int* idx2, int* d2) {
    ArenaScope scope;
    {
        for (int i = 0; i < nq; i++) {
            cv::Mat Q(1, 32, CV_8U, (void*)(q + (size_t)i * 32));
            int b1 = INT_MAX, b2 = INT_MAX, i1 = -1, i2 = -1;
            for (int j = 0; j < nt; j++) {
                cv::Mat T(1, 32, CV_8U, (void*)(t + (size_t)j * 32));
                int d = ORBmatcher::DescriptorDistance(Q, T);
                if (d < b1) { b2 = b1; i2 = i1; b1 = d; i1 = j; }
                else if (d < b2) { b2 = d; i2 = j; }
            }
            idx1[i] = i1; d1[i] = b1; idx2[i] = i2; d2[i] = b2;
        }
    }
    return 0;
}

// A frame carrying only the camera of the undistortion functions: mK and
// mDistCoef as the Frame constructors store them (src/Frame.cc:121-206).
static Frame* camera_frame(const float* K4, const float* dist, int ndist) {
    Frame* F = new Frame();
    F->mK = cv::Mat::eye(3, 3, CV_32F);
    F->mK.at<float>(0, 0) = K4[0];
    F->mK.at<float>(1, 1) = K4[1];
    F->mK.at<float>(0, 2) = K4[2];
    F->mK.at<float>(1, 2) = K4[3];
    F->mDistCoef = cv::Mat(ndist, 1, CV_32F);
    for (int i = 0; i < ndist; i++) F->mDistCoef.at<float>(i) = dist[i];
    return F;
}

// Frame::UndistortKeyPoints -- src/Frame.cc:724-776.  K4 = fx, fy, cx, cy;
// dist = k1 k2 p1 p2 [k3] (ndist 4 or 5).
int ref_undistort_keypoints(const float* K4, const float* dist, int ndist, const orc_kp* kps, int n, orc_kp* out) {
    ArenaScope scope;
    {
        Frame* F = camera_frame(K4, dist, ndist);
        F->N = n;
        F->mvKeys = kps_in(kps, n);
        F->UndistortKeyPoints();
        copy_kps_out(F->mvKeysUn, out);
        delete F;
    }
    return 0;
}

// Frame::ComputeImageBounds -- src/Frame.cc:778-819; bounds = mnMinX,
// mnMaxX, mnMinY, mnMaxY.
int ref_compute_image_bounds(int cols, int rows, const float* K4, const float* dist, int ndist, float* bounds) {
    ArenaScope scope;
    {
        Frame* F = camera_frame(K4, dist, ndist);
        cv::Mat im(rows, cols, CV_8U);
        F->ComputeImageBounds(im);
        bounds[0] = Frame::mnMinX;
        bounds[1] = Frame::mnMaxX;
        bounds[2] = Frame::mnMinY;
        bounds[3] = Frame::mnMaxY;
        delete F;
    }
    return 0;
}

// DBoW2 vocabularies loaded by ORBVocabulary::loadFromTextFile, by path
// (allocated outside any call's arena scope: they live until exit).
static std::map<std::string, ORBVocabulary*> g_ref_vocabs;

int ref_vocabulary_load(const char* path) {
    ORBVocabulary* v = new ORBVocabulary();
    if (!v->loadFromTextFile(path)) return -1;
    g_ref_vocabs[path] = v;
    return (int)v->size();
}

// ORBVocabulary::transform(features, mBowVec, mFeatVec, levelsup) as
// Frame::ComputeBoW calls it (src/Frame.cc:704-718), plus the per-feature
// transform(feature, word, weight, &nid, levelsup) for the word / weight /
// node of every feature.  Output layout as orc_bow_transform.
int ref_bow_transform(const char* path, const uint8_t* desc, int n, int levelsup, int* word_ids, double* weights,
                      int* node_ids, int* bow_n, int* bow_words, double* bow_values, int* fv_n, int* fv_nodes,
                      int* fv_offsets, int* fv_features) {
    auto it = g_ref_vocabs.find(path);
    if (it == g_ref_vocabs.end()) return -1;
    ORBVocabulary* voc = it->second;
    ArenaScope scope;
    {
        std::vector<cv::Mat> feats;
        for (int i = 0; i < n; i++) feats.push_back(cv::Mat(1, 32, CV_8U, (void*)(desc + (size_t)i * 32)));
        DBoW2::BowVector bv;
        DBoW2::FeatureVector fv;
        voc->transform(feats, bv, fv, levelsup);
        for (int i = 0; i < n; i++) {
            DBoW2::WordId wid = 0;
            DBoW2::WordValue w = 0;
            DBoW2::NodeId nid = 0;
            voc->transform(feats[i], wid, w, &nid, levelsup);
            word_ids[i] = (int)wid;
            weights[i] = w;
            node_ids[i] = (int)nid;
        }
        int b = 0;
        for (auto& e : bv) {
            bow_words[b] = (int)e.first;
            bow_values[b] = e.second;
            b++;
        }
        *bow_n = b;
        int nn = 0, off = 0;
        for (auto& e : fv) {
            fv_nodes[nn] = (int)e.first;
            fv_offsets[nn] = off;
            for (unsigned f : e.second) fv_features[off++] = (int)f;
            nn++;
        }
        fv_offsets[nn] = off;
        *fv_n = nn;
    }
    return 0;
}

static DBoW2::FeatureVector feature_vector(int n, const int* nodes, const int* offsets, const int* features) {
    DBoW2::FeatureVector fv;
    for (int i = 0; i < n; i++)
        for (int p = offsets[i]; p < offsets[i + 1]; p++) fv.addFeature((DBoW2::NodeId)nodes[i], (unsigned)features[p]);
    return fv;
}

// ORBmatcher::SearchByBoW(KeyFrame*, Frame&, vpMapPointMatches) --
// src/ORBmatcher.cc:247-380.  The keyframe is built from a frame holding its
// keypoints (mvKeysUn) and descriptors; its map points are real MapPoints
// (kf_mp 1), bad ones (2) or NULL (0).  match_out as orc_search_by_bow.
int ref_search_by_bow(const orc_kp* kf_kps, const uint8_t* kf_desc, const uint8_t* kf_mp, int kf_n, int kf_fv_n,
                      const int* kf_fv_nodes, const int* kf_fv_offsets, const int* kf_fv_features, const orc_kp* f_kps,
                      const uint8_t* f_desc, int f_n, int f_fv_n, const int* f_fv_nodes, const int* f_fv_offsets,
                      const int* f_fv_features, float nnratio, int check_ori, int* match_out) {
    ArenaScope scope;
    int nm;
    {
        MapPointMaker maker;
        cv::Mat pos = cv::Mat::zeros(3, 1, CV_32F);
        Frame* KFsrc = new Frame();
        KFsrc->N = kf_n;
        KFsrc->mvKeys = kps_in(kf_kps, kf_n);
        KFsrc->mvKeysUn = KFsrc->mvKeys;
        KFsrc->mvuRight.assign(kf_n, -1.0f);
        KFsrc->mDescriptors = cv::Mat(kf_n, 32, CV_8U);
        std::memcpy(KFsrc->mDescriptors.data, kf_desc, (size_t)kf_n * 32);
        KeyFrame* KF = new KeyFrame(*KFsrc, maker.map, nullptr);
        KF->mFeatVec = feature_vector(kf_fv_n, kf_fv_nodes, kf_fv_offsets, kf_fv_features);
        KF->mvpMapPoints.assign(kf_n, static_cast<MapPoint*>(NULL));
        std::map<MapPoint*, int> index;
        for (int i = 0; i < kf_n; i++) {
            if (kf_mp[i] == 0) continue;
            MapPoint* mp = maker.make(pos, 1);
            mp->mbBad = kf_mp[i] == 2;
            KF->mvpMapPoints[i] = mp;
            index[mp] = i;
        }
        Frame* F = new Frame();
        F->N = f_n;
        F->mvKeys = kps_in(f_kps, f_n);
        F->mvKeysUn = F->mvKeys;
        F->mDescriptors = cv::Mat(f_n, 32, CV_8U);
        std::memcpy(F->mDescriptors.data, f_desc, (size_t)f_n * 32);
        F->mFeatVec = feature_vector(f_fv_n, f_fv_nodes, f_fv_offsets, f_fv_features);
        std::vector<MapPoint*> matches;
        ORBmatcher matcher(nnratio, check_ori != 0);
        nm = matcher.SearchByBoW(KF, *F, matches);
        for (int i = 0; i < f_n; i++) match_out[i] = matches[i] ? index[matches[i]] : -1;
        for (auto& e : index) delete e.first;
        delete F;
        delete KF;
        delete KFsrc;
    }
    return nm;
}

// A keyframe built from recorded keypoints / descriptors / FeatureVector with
// real map points where mp[i] is 1 (bad ones where 2); index maps them back.
static KeyFrame* make_keyframe(MapPointMaker& maker, const orc_kp* kps, const uint8_t* desc, const uint8_t* mp, int n,
                               int fv_n, const int* fv_nodes, const int* fv_offsets, const int* fv_features,
                               std::map<MapPoint*, int>& index, Frame*& src) {
    cv::Mat pos = cv::Mat::zeros(3, 1, CV_32F);
    src = new Frame();
    src->N = n;
    src->mvKeys = kps_in(kps, n);
    src->mvKeysUn = src->mvKeys;
    src->mvuRight.assign(n, -1.0f);
    src->mDescriptors = cv::Mat(n, 32, CV_8U);
    std::memcpy(src->mDescriptors.data, desc, (size_t)n * 32);
    KeyFrame* KF = new KeyFrame(*src, maker.map, nullptr);
    KF->mFeatVec = feature_vector(fv_n, fv_nodes, fv_offsets, fv_features);
    KF->mvpMapPoints.assign(n, static_cast<MapPoint*>(NULL));
    for (int i = 0; i < n; i++) {
        if (mp[i] == 0) continue;
        MapPoint* p = maker.make(pos, 1);
        p->mbBad = mp[i] == 2;
        KF->mvpMapPoints[i] = p;
        index[p] = i;
    }
    return KF;
}

// ORBmatcher::SearchByBoW(KeyFrame* pKF1, KeyFrame* pKF2, vpMatches12) --
// src/ORBmatcher.cc:729-880.  match_out[i]: the pKF2 feature whose map point
// vpMatches12[i] holds, or -1.
int ref_search_by_bow_kf(const orc_kp* kps1, const uint8_t* desc1, const uint8_t* mp1, int n1, int fv1_n,
                         const int* fv1_nodes, const int* fv1_offsets, const int* fv1_features, const orc_kp* kps2,
                         const uint8_t* desc2, const uint8_t* mp2, int n2, int fv2_n, const int* fv2_nodes,
                         const int* fv2_offsets, const int* fv2_features, float nnratio, int check_ori,
                         int* match_out) {
    ArenaScope scope;
    int nm;
    {
        MapPointMaker maker;
        std::map<MapPoint*, int> index1, index2;
        Frame *s1, *s2;
        KeyFrame* KF1 = make_keyframe(maker, kps1, desc1, mp1, n1, fv1_n, fv1_nodes, fv1_offsets, fv1_features,
                                      index1, s1);
        KeyFrame* KF2 = make_keyframe(maker, kps2, desc2, mp2, n2, fv2_n, fv2_nodes, fv2_offsets, fv2_features,
                                      index2, s2);
        std::vector<MapPoint*> matches;
        ORBmatcher matcher(nnratio, check_ori != 0);
        nm = matcher.SearchByBoW(KF1, KF2, matches);
        for (int i = 0; i < n1; i++) match_out[i] = matches[i] ? index2[matches[i]] : -1;
        for (auto& e : index1) delete e.first;
        for (auto& e : index2) delete e.first;
        delete KF1;
        delete KF2;
        delete s1;
        delete s2;
    }
    return nm;
}

// ORBmatcher::SearchByProjection(Frame&, KeyFrame*, sAlreadyFound, th,
// ORBdist) -- src/ORBmatcher.cc:1891-2010.  The keyframe holds real map
// points (bad ones for mp_state 2, those of state 3 also in sAlreadyFound).
// match_out: >= 0 the keyframe feature whose map point fills the keypoint,
// -2 claimed before, -1 otherwise (a reset by the rotation check leaves NULL,
// like an untouched keypoint).
int ref_search_by_projection_kf(const orc_params* p, const orc_kp* kps, const uint8_t* desc, int n, int w, int h,
                                const float* T, const float* cam, const orc_kp* kf_kps, int m,
                                const orc_mp_geometry* mps, const uint8_t* mp_desc, const uint8_t* mp_state, float th,
                                int orbdist, int check_ori, const uint8_t* claimed, int* match_out) {
    ArenaScope scope;
    int nm;
    {
        ORBextractor ext(p->nfeatures, p->scale_factor, p->nlevels, p->ini_th_fast, p->min_th_fast);
        Frame* F = make_frame(&ext, kps, desc, n, w, h, nullptr);
        Frame::fx = cam[0];
        Frame::fy = cam[1];
        Frame::cx = cam[2];
        Frame::cy = cam[3];
        Frame::invfx = 1.0f / cam[0];
        Frame::invfy = 1.0f / cam[1];
        F->mfLogScaleFactor = std::log(F->mfScaleFactor);
        cv::Mat Tcw = cv::Mat::eye(4, 4, CV_32F);
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 4; c++) Tcw.at<float>(r, c) = T[4 * r + c];
        F->SetPose(Tcw);
        MapPointMaker maker;
        cv::Mat zero = cv::Mat::zeros(3, 1, CV_32F);
        MapPoint* preclaimed = maker.make(zero, 1);
        for (int i = 0; i < n; i++)
            if (claimed && claimed[i]) F->mvpMapPoints[i] = preclaimed;
        Frame* src = new Frame();
        src->N = m;
        src->mvKeys = kps_in(kf_kps, m);
        src->mvKeysUn = src->mvKeys;
        src->mvuRight.assign(m, -1.0f);
        src->mDescriptors = cv::Mat(m, 32, CV_8U);
        KeyFrame* KF = new KeyFrame(*src, maker.map, nullptr);
        KF->mvpMapPoints.assign(m, static_cast<MapPoint*>(NULL));
        std::set<MapPoint*> found;
        std::map<MapPoint*, int> index;
        for (int i = 0; i < m; i++) {
            if (mp_state[i] == 0) continue;
            cv::Mat pos(3, 1, CV_32F);
            pos.at<float>(0) = mps[i].x;
            pos.at<float>(1) = mps[i].y;
            pos.at<float>(2) = mps[i].z;
            MapPoint* mp = maker.make(pos, 1);
            mp->mfMinDistance = mps[i].min_distance;
            mp->mfMaxDistance = mps[i].max_distance;
            mp->mDescriptor = cv::Mat(1, 32, CV_8U);
            std::memcpy(mp->mDescriptor.data, mp_desc + (size_t)i * 32, 32);
            mp->mbBad = mp_state[i] == 2;
            if (mp_state[i] == 3) found.insert(mp);
            KF->mvpMapPoints[i] = mp;
            index[mp] = i;
        }
        ORBmatcher matcher(0.9f, check_ori != 0);
        nm = matcher.SearchByProjection(*F, KF, found, th, orbdist);
        for (int i = 0; i < n; i++) {
            MapPoint* mp = F->mvpMapPoints[i];
            match_out[i] = mp == nullptr ? -1 : mp == preclaimed ? -2 : index[mp];
        }
        for (auto& e : index) delete e.first;
        delete KF;
        delete src;
        delete F;
    }
    return nm;
}

// ORBmatcher::SearchForTriangulation(pKF1, pKF2, F12, vMatchedPairs,
// bOnlyStereo) -- src/ORBmatcher.cc:884-1040.  Arguments as
// orc_search_for_triangulation; pKF1's camera centre and pKF2's pose are set
// on the keyframes, pKF2's camera constants and scale tables through the
// frame they are built from.
int ref_search_for_triangulation(const orc_kp* kps1, const uint8_t* desc1, const uint8_t* mp1, const float* ur1, int n1,
                                  int fv1_n, const int* fv1_nodes, const int* fv1_offsets, const int* fv1_features,
                                  const orc_kp* kps2, const uint8_t* desc2, const uint8_t* mp2, const float* ur2, int n2,
                                  int fv2_n, const int* fv2_nodes, const int* fv2_offsets, const int* fv2_features,
                                  const float* Cw1, const float* T2, const float* K2, const float* F12,
                                  const float* scale, const float* sigma2, int only_stereo, int check_ori,
                                  int* match_out) {
    ArenaScope scope;
    int nm;
    {
        MapPointMaker maker;
        Frame::fx = K2[0];
        Frame::fy = K2[1];
        Frame::cx = K2[2];
        Frame::cy = K2[3];
        std::map<MapPoint*, int> index1, index2;
        Frame *s1, *s2;
        KeyFrame* KF1 = make_keyframe(maker, kps1, desc1, mp1, n1, fv1_n, fv1_nodes, fv1_offsets, fv1_features,
                                      index1, s1);
        KeyFrame* KF2 = make_keyframe(maker, kps2, desc2, mp2, n2, fv2_n, fv2_nodes, fv2_offsets, fv2_features,
                                      index2, s2);
        // stereo flags and pKF2's scale tables live in const members: rebuild
        // the keyframes from frames carrying them
        s1->mvuRight.assign(ur1, ur1 + n1);
        s2->mvuRight.assign(ur2, ur2 + n2);
        s2->mvScaleFactors.assign(scale, scale + 16);
        s2->mvLevelSigma2.assign(sigma2, sigma2 + 16);
        KeyFrame* A = new KeyFrame(*s1, maker.map, nullptr);
        KeyFrame* B = new KeyFrame(*s2, maker.map, nullptr);
        A->mFeatVec = KF1->mFeatVec;
        B->mFeatVec = KF2->mFeatVec;
        A->mvpMapPoints = KF1->mvpMapPoints;
        B->mvpMapPoints = KF2->mvpMapPoints;
        A->Ow = cv::Mat(3, 1, CV_32F);
        for (int r = 0; r < 3; r++) A->Ow.at<float>(r) = Cw1[r];
        B->Tcw = cv::Mat::eye(4, 4, CV_32F);
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 4; c++) B->Tcw.at<float>(r, c) = T2[4 * r + c];
        cv::Mat F(3, 3, CV_32F);
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) F.at<float>(r, c) = F12[3 * r + c];
        std::vector<std::pair<size_t, size_t> > pairs;
        ORBmatcher matcher(0.6f, check_ori != 0);
        nm = matcher.SearchForTriangulation(A, B, F, pairs, only_stereo != 0);
        for (int i = 0; i < n1; i++) match_out[i] = -1;
        for (auto& pr : pairs) match_out[pr.first] = (int)pr.second;
        for (auto& e : index1) delete e.first;
        for (auto& e : index2) delete e.first;
        delete A;
        delete B;
        delete KF1;
        delete KF2;
        delete s1;
        delete s2;
    }
    return nm;
}

// ORBmatcher::SearchByProjection(KeyFrame* pKF, Scw, vpPoints, vpMatched, th)
// -- src/ORBmatcher.cc:423-560, on a keyframe built from a frame of the
// given keypoints (grid, bounds 0..w x 0..h); claimed keypoints hold other
// map points in vpMatched.  match_out as orc_search_by_projection_sim3.
int ref_search_by_projection_sim3(const orc_params* p, const orc_kp* kps, const uint8_t* desc, int n, int w, int h,
                                  const float* Scw, const float* cam, const orc_mp_geometry* pts,
                                  const uint8_t* pdesc, const uint8_t* pstate, int npts, int th,
                                  const uint8_t* claimed, int* match_out) {
    ArenaScope scope;
    int nm;
    {
        ORBextractor ext(p->nfeatures, p->scale_factor, p->nlevels, p->ini_th_fast, p->min_th_fast);
        Frame::fx = cam[0];
        Frame::fy = cam[1];
        Frame::cx = cam[2];
        Frame::cy = cam[3];
        Frame* F = make_frame(&ext, kps, desc, n, w, h, nullptr);
        F->mfLogScaleFactor = std::log(F->mfScaleFactor);
        MapPointMaker maker;
        KeyFrame* KF = new KeyFrame(*F, maker.map, nullptr);
        cv::Mat zero = cv::Mat::zeros(3, 1, CV_32F);
        MapPoint* outside = maker.make(zero, 1);
        std::vector<MapPoint*> matched(n, static_cast<MapPoint*>(NULL));
        for (int i = 0; i < n; i++)
            if (claimed && claimed[i]) matched[i] = outside;
        std::vector<MapPoint*> points(npts);
        std::map<MapPoint*, int> index;
        for (int i = 0; i < npts; i++) {
            cv::Mat pos(3, 1, CV_32F);
            pos.at<float>(0) = pts[i].x;
            pos.at<float>(1) = pts[i].y;
            pos.at<float>(2) = pts[i].z;
            MapPoint* mp = maker.make(pos, 1);
            mp->mNormalVector = cv::Mat(3, 1, CV_32F);
            mp->mNormalVector.at<float>(0) = pts[i].nx;
            mp->mNormalVector.at<float>(1) = pts[i].ny;
            mp->mNormalVector.at<float>(2) = pts[i].nz;
            mp->mfMinDistance = pts[i].min_distance;
            mp->mfMaxDistance = pts[i].max_distance;
            mp->mDescriptor = cv::Mat(1, 32, CV_8U);
            std::memcpy(mp->mDescriptor.data, pdesc + (size_t)i * 32, 32);
            mp->mbBad = pstate[i] == 2;
            points[i] = mp;
            index[mp] = i;
        }
        cv::Mat S = cv::Mat::eye(4, 4, CV_32F);
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 4; c++) S.at<float>(r, c) = Scw[4 * r + c];
        ORBmatcher matcher(0.9f, true);
        nm = matcher.SearchByProjection(KF, S, points, matched, th);
        for (int i = 0; i < n; i++)
            match_out[i] = matched[i] == nullptr ? -1 : matched[i] == outside ? -2 : index[matched[i]];
        for (MapPoint* mp : points) delete mp;
        delete KF;
        delete F;
    }
    return nm;
}

// ORBmatcher::Fuse(KeyFrame*, vpMapPoints, th) -- src/ORBmatcher.cc:1107-1245,
// run on one map point at a time against the keyframe with no map points (so
// the reference adds the observation): target[i] is the feature where
// AddMapPoint put map point i, or -1.
int ref_fuse_candidates(const orc_params* p, const orc_kp* kps, const uint8_t* desc, const float* uright, int n,
                          int w, int h, const float* T, const float* cam, const orc_mp_geometry* mps,
                          const uint8_t* mp_desc, const uint8_t* mp_state, int m, float th, int* target) {
    ArenaScope scope;
    int nf = 0;
    {
        ORBextractor ext(p->nfeatures, p->scale_factor, p->nlevels, p->ini_th_fast, p->min_th_fast);
        Frame::fx = cam[0];
        Frame::fy = cam[1];
        Frame::cx = cam[2];
        Frame::cy = cam[3];
        Frame* F = make_frame(&ext, kps, desc, n, w, h, uright);
        F->mfLogScaleFactor = std::log(F->mfScaleFactor);
        F->mbf = cam[4];
        MapPointMaker maker;
        KeyFrame* KF = new KeyFrame(*F, maker.map, nullptr);
        KF->Tcw = cv::Mat::eye(4, 4, CV_32F);
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 4; c++) KF->Tcw.at<float>(r, c) = T[4 * r + c];
        // Ow = -Rcw' tcw as KeyFrame::SetPose computes it
        cv::Mat Rcw = KF->Tcw.rowRange(0, 3).colRange(0, 3);
        cv::Mat tcw = KF->Tcw.rowRange(0, 3).col(3);
        KF->Ow = -Rcw.t() * tcw;
        ORBmatcher matcher(0.6f, true);
        for (int i = 0; i < m; i++) {
            target[i] = -1;
            if (mp_state[i] != 1) continue;
            cv::Mat pos(3, 1, CV_32F);
            pos.at<float>(0) = mps[i].x;
            pos.at<float>(1) = mps[i].y;
            pos.at<float>(2) = mps[i].z;
            MapPoint* mp = maker.make(pos, 0);
            mp->mNormalVector = cv::Mat(3, 1, CV_32F);
            mp->mNormalVector.at<float>(0) = mps[i].nx;
            mp->mNormalVector.at<float>(1) = mps[i].ny;
            mp->mNormalVector.at<float>(2) = mps[i].nz;
            mp->mfMinDistance = mps[i].min_distance;
            mp->mfMaxDistance = mps[i].max_distance;
            mp->mDescriptor = cv::Mat(1, 32, CV_8U);
            std::memcpy(mp->mDescriptor.data, mp_desc + (size_t)i * 32, 32);
            KF->mvpMapPoints.assign(n, static_cast<MapPoint*>(NULL));
            std::vector<MapPoint*> one(1, mp);
            nf += matcher.Fuse(KF, one, th);
            for (int k = 0; k < n; k++)
                if (KF->mvpMapPoints[k] == mp) target[i] = k;
            delete mp;
        }
        delete KF;
        delete F;
    }
    return nf;
}

// ORBmatcher::Fuse(KeyFrame*, Scw, vpPoints, th, vpReplacePoint) --
// src/ORBmatcher.cc:1290-1380, one point at a time against the keyframe with
// no map points: target[i] is where AddMapPoint put point i, or -1.
int ref_fuse_sim3_candidates(const orc_params* p, const orc_kp* kps, const uint8_t* desc, int n, int w, int h,
                               const float* Scw, const float* cam, const orc_mp_geometry* pts, const uint8_t* pdesc,
                               const uint8_t* pstate, int npts, float th, int* target) {
    ArenaScope scope;
    int nf = 0;
    {
        ORBextractor ext(p->nfeatures, p->scale_factor, p->nlevels, p->ini_th_fast, p->min_th_fast);
        Frame::fx = cam[0];
        Frame::fy = cam[1];
        Frame::cx = cam[2];
        Frame::cy = cam[3];
        Frame* F = make_frame(&ext, kps, desc, n, w, h, nullptr);
        F->mfLogScaleFactor = std::log(F->mfScaleFactor);
        MapPointMaker maker;
        KeyFrame* KF = new KeyFrame(*F, maker.map, nullptr);
        cv::Mat S = cv::Mat::eye(4, 4, CV_32F);
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 4; c++) S.at<float>(r, c) = Scw[4 * r + c];
        ORBmatcher matcher(0.6f, true);
        for (int i = 0; i < npts; i++) {
            target[i] = -1;
            if (pstate[i] != 1) continue;
            cv::Mat pos(3, 1, CV_32F);
            pos.at<float>(0) = pts[i].x;
            pos.at<float>(1) = pts[i].y;
            pos.at<float>(2) = pts[i].z;
            MapPoint* mp = maker.make(pos, 0);
            mp->mNormalVector = cv::Mat(3, 1, CV_32F);
            mp->mNormalVector.at<float>(0) = pts[i].nx;
            mp->mNormalVector.at<float>(1) = pts[i].ny;
            mp->mNormalVector.at<float>(2) = pts[i].nz;
            mp->mfMinDistance = pts[i].min_distance;
            mp->mfMaxDistance = pts[i].max_distance;
            mp->mDescriptor = cv::Mat(1, 32, CV_8U);
            std::memcpy(mp->mDescriptor.data, pdesc + (size_t)i * 32, 32);
            KF->mvpMapPoints.assign(n, static_cast<MapPoint*>(NULL));
            std::vector<MapPoint*> one(1, mp), replace(1, static_cast<MapPoint*>(NULL));
            nf += matcher.Fuse(KF, S, one, th, replace);
            for (int k = 0; k < n; k++)
                if (KF->mvpMapPoints[k] == mp) target[i] = k;
            delete mp;
        }
        delete KF;
        delete F;
    }
    return nf;
}

// ORBmatcher::SearchBySim3 -- src/ORBmatcher.cc:1441-1640, two keyframes
// built from frames of the given keypoints, vpMatches12 empty on entry.
int ref_search_by_sim3(const orc_params* p, const orc_kp* kps1, const uint8_t* desc1, int n1, const orc_kp* kps2,
                           const uint8_t* desc2, int n2, int w, int h, const float* T1w, const float* T2w, float s12,
                           const float* R12, const float* t12, const float* cam, const orc_mp_geometry* mps1,
                           const uint8_t* mpd1, const uint8_t* st1, const orc_mp_geometry* mps2, const uint8_t* mpd2,
                           const uint8_t* st2, float th, const int* pre12, int* match12) {
    ArenaScope scope;
    int nf;
    {
        ORBextractor ext(p->nfeatures, p->scale_factor, p->nlevels, p->ini_th_fast, p->min_th_fast);
        Frame::fx = cam[0];
        Frame::fy = cam[1];
        Frame::cx = cam[2];
        Frame::cy = cam[3];
        MapPointMaker maker;
        Frame* F1 = make_frame(&ext, kps1, desc1, n1, w, h, nullptr);
        F1->mfLogScaleFactor = std::log(F1->mfScaleFactor);
        KeyFrame* K1 = new KeyFrame(*F1, maker.map, nullptr);
        Frame* F2 = make_frame(&ext, kps2, desc2, n2, w, h, nullptr);
        F2->mfLogScaleFactor = std::log(F2->mfScaleFactor);
        KeyFrame* K2 = new KeyFrame(*F2, maker.map, nullptr);
        std::map<MapPoint*, int> index2;
        std::vector<MapPoint*> owned;
        auto fill = [&](KeyFrame* K, const float* T, int n, const orc_mp_geometry* mps, const uint8_t* mpd,
                        const uint8_t* st, std::map<MapPoint*, int>* index) {
            K->Tcw = cv::Mat::eye(4, 4, CV_32F);
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 4; c++) K->Tcw.at<float>(r, c) = T[4 * r + c];
            K->mvpMapPoints.assign(n, static_cast<MapPoint*>(NULL));
            for (int i = 0; i < n; i++) {
                if (st[i] == 0) continue;
                cv::Mat pos(3, 1, CV_32F);
                pos.at<float>(0) = mps[i].x;
                pos.at<float>(1) = mps[i].y;
                pos.at<float>(2) = mps[i].z;
                MapPoint* mp = maker.make(pos, 1);
                mp->mfMinDistance = mps[i].min_distance;
                mp->mfMaxDistance = mps[i].max_distance;
                mp->mDescriptor = cv::Mat(1, 32, CV_8U);
                std::memcpy(mp->mDescriptor.data, mpd + (size_t)i * 32, 32);
                mp->mbBad = st[i] == 2;
                K->mvpMapPoints[i] = mp;
                owned.push_back(mp);
                if (index) (*index)[mp] = i;
            }
        };
        fill(K1, T1w, n1, mps1, mpd1, st1, nullptr);
        fill(K2, T2w, n2, mps2, mpd2, st2, &index2);
        cv::Mat R(3, 3, CV_32F), tt(3, 1, CV_32F);
        for (int k = 0; k < 9; k++) R.at<float>(k / 3, k % 3) = R12[k];
        for (int k = 0; k < 3; k++) tt.at<float>(k) = t12[k];
        std::vector<MapPoint*> matches(n1, static_cast<MapPoint*>(NULL));
        // vpMatches12 entries already set: pKF2's map point pre12[i], observed
        // by pKF2 at that feature (what GetIndexInKeyFrame(pKF2) reports)
        if (pre12)
            for (int i = 0; i < n1; i++)
                if (pre12[i] >= 0 && pre12[i] < n2 && K2->mvpMapPoints[pre12[i]]) {
                    MapPoint* mp = K2->mvpMapPoints[pre12[i]];
                    mp->AddObservation(K2, pre12[i]);
                    matches[i] = mp;
                }
        ORBmatcher matcher(0.75f, true);
        const float s = s12;
        nf = matcher.SearchBySim3(K1, K2, matches, s, R, tt, th);
        for (int i = 0; i < n1; i++) match12[i] = matches[i] ? index2[matches[i]] : -1;
        for (MapPoint* mp : owned) delete mp;
        delete K1;
        delete K2;
        delete F1;
        delete F2;
    }
    return nf;
}

// Frame::isInFrustum -- src/Frame.cc:491-578, on a Frame posed by SetPose
// (UpdatePoseMatrices) and real map points whose tracking fields start from
// out[i] (the reference leaves them unchanged where it returns false).
int ref_is_in_frustum(const orc_frustum_camera* cam, const orc_mp_geometry* mps, int m, float cos_limit,
                      orc_mappoint* out) {
    ArenaScope scope;
    int nin = 0;
    {
        MapPointMaker maker;
        Frame* F = new Frame();
        cv::Mat Tcw = cv::Mat::eye(4, 4, CV_32F);
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 4; c++) Tcw.at<float>(r, c) = cam->Tcw[4 * r + c];
        F->SetPose(Tcw);
        Frame::fx = cam->fx;
        Frame::fy = cam->fy;
        Frame::cx = cam->cx;
        Frame::cy = cam->cy;
        Frame::invfx = 1.0f / cam->fx;
        Frame::invfy = 1.0f / cam->fy;
        Frame::mnMinX = cam->min_x;
        Frame::mnMaxX = cam->max_x;
        Frame::mnMinY = cam->min_y;
        Frame::mnMaxY = cam->max_y;
        F->mbf = cam->bf;
        F->mnScaleLevels = cam->nlevels;
        F->mfScaleFactor = cam->scale_factor;
        F->mfLogScaleFactor = std::log(cam->scale_factor);
        for (int i = 0; i < m; i++) {
            cv::Mat pos(3, 1, CV_32F);
            pos.at<float>(0) = mps[i].x;
            pos.at<float>(1) = mps[i].y;
            pos.at<float>(2) = mps[i].z;
            MapPoint* mp = maker.make(pos, 1);
            mp->mNormalVector = cv::Mat(3, 1, CV_32F);
            mp->mNormalVector.at<float>(0) = mps[i].nx;
            mp->mNormalVector.at<float>(1) = mps[i].ny;
            mp->mNormalVector.at<float>(2) = mps[i].nz;
            mp->mfMinDistance = mps[i].min_distance;
            mp->mfMaxDistance = mps[i].max_distance;
            mp->mTrackProjX = out[i].proj_x;
            mp->mTrackProjY = out[i].proj_y;
            mp->mTrackProjXR = out[i].proj_xr;
            mp->mTrackViewCos = out[i].view_cos;
            mp->mnTrackScaleLevel = out[i].track_scale_level;
            const bool in = F->isInFrustum(mp, cos_limit);
            nin += in ? 1 : 0;
            out[i].track_in_view = mp->mbTrackInView ? 1 : 0;
            out[i].proj_x = mp->mTrackProjX;
            out[i].proj_y = mp->mTrackProjY;
            out[i].proj_xr = mp->mTrackProjXR;
            out[i].view_cos = mp->mTrackViewCos;
            out[i].track_scale_level = mp->mnTrackScaleLevel;
            delete mp;
        }
        delete F;
    }
    return nin;
}

// MapPoint::ComputeDistinctiveDescriptors -- src/MapPoint.cc:365-447, run on a
// real MapPoint whose observations are one keyframe per list entry (each
// keyframe holding that entry's descriptor as its row 0; a -1 row becomes a
// keyframe flagged bad).  mObservations is a std::map keyed by KeyFrame*; the
// arena makes address order equal creation order, so the map iterates in list
// order.  desc_inout holds each map point's descriptor before the call
// (zeros when NULL is passed) and receives mDescriptor after it.  best_rows:
// -2 invalid list (the reference is not run), -1 no valid observation, else
// -3 (the reference exposes the chosen descriptor, not its index).
int ref_distinctive_descriptors(const uint8_t* pool, int pool_rows, const int* offsets, const int* rows, int m,
                                int* best_rows, uint8_t* desc_inout) {
    ArenaScope scope;
    {
        MapPointMaker maker;
        cv::Mat pos = cv::Mat::zeros(3, 1, CV_32F);
        for (int i = 0; i < m; i++) {
            const int o0 = offsets[i], o1 = offsets[i + 1];
            bool bad_input = o1 < o0, any_valid = false;
            for (int t = o0; t < o1 && !bad_input; t++) {
                if (rows[t] < -1 || rows[t] >= pool_rows) bad_input = true;
                any_valid |= rows[t] >= 0;
            }
            if (bad_input) {
                best_rows[i] = -2;
                continue;
            }
            std::vector<KeyFrame*> kfs;
            for (int t = o0; t < o1; t++) {
                Frame f;
                f.mnId = (long unsigned int)t;
                f.N = 1;
                f.mvuRight.assign(1, -1.0f);
                f.mDescriptors = cv::Mat::zeros(1, 32, CV_8U);
                if (rows[t] >= 0) std::memcpy(f.mDescriptors.data, pool + (size_t)rows[t] * 32, 32);
                KeyFrame* kf = new KeyFrame(f, maker.map, nullptr);
                kf->mbBad = rows[t] < 0;
                if (!kfs.empty() && kf < kfs.back()) {
                    std::fprintf(stderr, "ref_distinctive_descriptors: keyframes not in address order\n");
                    std::abort();
                }
                kfs.push_back(kf);
            }
            MapPoint* mp = new MapPoint(pos, kfs.empty() ? maker.kf : kfs[0], maker.map);
            mp->mDescriptor = cv::Mat::zeros(1, 32, CV_8U);
            if (desc_inout) std::memcpy(mp->mDescriptor.data, desc_inout + (size_t)i * 32, 32);
            for (KeyFrame* kf : kfs) mp->AddObservation(kf, 0);
            mp->ComputeDistinctiveDescriptors();
            if (desc_inout) std::memcpy(desc_inout + (size_t)i * 32, mp->mDescriptor.data, 32);
            best_rows[i] = any_valid ? -3 : -1;
            delete mp;
            for (KeyFrame* kf : kfs) delete kf;
        }
    }
    return 0;
}

}  // extern "C"
