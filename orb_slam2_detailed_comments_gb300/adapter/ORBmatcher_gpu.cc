// ORB_SLAM2::ORBmatcher's searches of the front-end path on the GPU library,
// compiled against the reference's unchanged include/ORBmatcher.h and
// include/Frame.h.  Defines the member functions
//   SearchForInitialization                    (src/ORBmatcher.cc:573-717)
//   SearchByProjection(Frame&, vector<MapPoint*>, th)   (src/ORBmatcher.cc:72-183)
//   SearchByProjection(Frame&, const Frame&, th, bMono) (src/ORBmatcher.cc:1710-1879)
// which a host removes from its src/ORBmatcher.cc (the constructor, the
// TH_LOW / TH_HIGH / HISTO_LENGTH constants, DescriptorDistance and the other
// searches stay there), and the free function orbgpu_cv::ComputeStereoMatches
// for Frame::ComputeStereoMatches (src/Frame.cc:831-1082).  Each reads the
// Frame / MapPoint fields the reference reads, calls the library, and applies
// the result to mvpMapPoints (or mvuRight / mvDepth) as the reference does.
// Frames must have the undistorted bounds [0, cols] x [0, rows] (the
// library's grid); others are rejected with an exception.
#include <cmath>
#include <cstring>
#include <map>
#include <utility>
#include <vector>

#include "Frame.h"
#include "MapPoint.h"
#include "ORBmatcher.h"
#include "orbgpu_cv.hpp"

namespace orbgpu_cv {
namespace {

// One library matcher per (nnratio, checkOri) and host thread: the reference
// constructs ORBmatcher objects on the stack all over Tracking, so handles
// are cached rather than tied to objects.
struct MatcherCache {
    std::map<std::pair<float, bool>, orbgpu_matcher*> handles;
    ~MatcherCache() {
        for (auto& kv : handles) orbgpu_matcher_destroy(kv.second);
    }
};

orbgpu_matcher* matcher_for(float nnratio, bool check_ori) {
    thread_local MatcherCache cache;
    const auto key = std::make_pair(nnratio, check_ori);
    auto it = cache.handles.find(key);
    if (it != cache.handles.end()) return it->second;
    orbgpu_matcher* h = nullptr;
    check(orbgpu_matcher_create(nnratio, check_ori ? 1 : 0, nullptr, &h), "ORBmatcher");
    cache.handles[key] = h;
    return h;
}

// The Frame fields the searches read, as the library's frame view (host
// memory, read in place).
orbgpu_frame frame_view(const std::vector<cv::KeyPoint>& kps, const cv::Mat& desc, const ORB_SLAM2::Frame& F,
                        const float* uright) {
    if (F.mnMinX != 0.f || F.mnMinY != 0.f || F.mnMaxX != std::floor(F.mnMaxX) ||
        F.mnMaxY != std::floor(F.mnMaxY))
        throw Error(ORBGPU_ERR_BAD_ARG, "orbgpu adapter: only undistorted image bounds [0, cols] x [0, rows]");
    if (!kps.empty() && (desc.rows != (int)kps.size() || desc.cols != 32 || desc.type() != CV_8U ||
                         !desc.isContinuous()))
        throw Error(ORBGPU_ERR_BAD_ARG, "orbgpu adapter: descriptors must be a continuous N x 32 CV_8U matrix");
    if (F.mnScaleLevels < 1 || F.mnScaleLevels > 16)
        throw Error(ORBGPU_ERR_BAD_ARG, "orbgpu adapter: 1 to 16 pyramid levels");
    orbgpu_frame v;
    std::memset(&v, 0, sizeof(v));
    v.keypoints = reinterpret_cast<const orbgpu_keypoint*>(kps.data());
    v.descriptors = kps.empty() ? nullptr : desc.ptr<uint8_t>(0);
    v.uright = uright;
    v.n = (int)kps.size();
    v.width = (int)F.mnMaxX;
    v.height = (int)F.mnMaxY;
    v.nlevels = F.mnScaleLevels;
    for (int l = 0; l < F.mnScaleLevels; l++) v.scale_factors[l] = F.mvScaleFactors[l];
    v.mem = ORBGPU_MEM_HOST;
    return v;
}

// CurrentFrame.mvpMapPoints[i] already holds a map point with observations
// (the searches skip such keypoints).
std::vector<uint8_t> claimed_of(const ORB_SLAM2::Frame& F) {
    std::vector<uint8_t> c(F.mvKeysUn.size(), 0);
    for (size_t i = 0; i < c.size() && i < F.mvpMapPoints.size(); i++)
        c[i] = F.mvpMapPoints[i] && F.mvpMapPoints[i]->Observations() > 0;
    return c;
}

void rows_of(const cv::Mat& T, float* out12) {
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 4; c++) out12[4 * r + c] = T.at<float>(r, c);
}

}  // namespace

void ComputeStereoMatches(ORB_SLAM2::Frame& F) {
    orbgpu_extractor* L = extractor_handle(F.mpORBextractorLeft);
    orbgpu_extractor* R = extractor_handle(F.mpORBextractorRight);
    if (!L || !R) throw Error(ORBGPU_ERR_BAD_ARG, "ComputeStereoMatches: the frame's extractors are not the adapter's");
    const orbgpu_frame fl = frame_view(F.mvKeys, F.mDescriptors, F, nullptr);
    const orbgpu_frame fr = frame_view(F.mvKeysRight, F.mDescriptorsRight, F, nullptr);
    F.mvuRight.assign(F.N, -1.0f);
    F.mvDepth.assign(F.N, -1.0f);
    if (F.N == 0) return;
    check(orbgpu_compute_stereo_matches(matcher_for(0.6f, true), L, R, &fl, &fr, F.mbf, F.fx, F.mvuRight.data(),
                                        F.mvDepth.data(), ORBGPU_MEM_HOST),
          "ComputeStereoMatches");
}

}  // namespace orbgpu_cv

namespace ORB_SLAM2 {

int ORBmatcher::SearchForInitialization(Frame& F1, Frame& F2, std::vector<cv::Point2f>& vbPrevMatched,
                                        std::vector<int>& vnMatches12, int windowSize) {
    const orbgpu_frame f1 = orbgpu_cv::frame_view(F1.mvKeysUn, F1.mDescriptors, F1, nullptr);
    const orbgpu_frame f2 = orbgpu_cv::frame_view(F2.mvKeysUn, F2.mDescriptors, F2, nullptr);
    vnMatches12.assign(F1.mvKeysUn.size(), -1);
    if (vbPrevMatched.size() < F1.mvKeysUn.size())
        throw orbgpu_cv::Error(ORBGPU_ERR_BAD_ARG, "SearchForInitialization: vbPrevMatched shorter than F1's keypoints");
    if (F1.mvKeysUn.empty()) return 0;
    int nm = 0;
    orbgpu_cv::check(orbgpu_search_for_initialization(orbgpu_cv::matcher_for(mfNNratio, mbCheckOrientation), &f1, &f2,
                                                      reinterpret_cast<float*>(vbPrevMatched.data()),
                                                      vnMatches12.data(), windowSize, &nm),
                     "SearchForInitialization");
    return nm;
}

int ORBmatcher::SearchByProjection(Frame& F, const std::vector<MapPoint*>& vpMapPoints, const float th) {
    const orbgpu_frame f =
        orbgpu_cv::frame_view(F.mvKeysUn, F.mDescriptors, F, F.mvuRight.empty() ? nullptr : F.mvuRight.data());
    const size_t M = vpMapPoints.size();
    std::vector<orbgpu_mappoint> rec(std::max<size_t>(M, 1));
    std::vector<uint8_t> desc(std::max<size_t>(M, 1) * 32, 0);
    for (size_t i = 0; i < M; i++) {
        MapPoint* p = vpMapPoints[i];
        orbgpu_mappoint& r = rec[i];
        std::memset(&r, 0, sizeof(r));
        if (!p || !p->mbTrackInView) continue;  // track_in_view 0: skipped, as the reference does
        r.track_in_view = 1;
        r.bad = p->isBad() ? 1 : 0;
        r.proj_x = p->mTrackProjX;
        r.proj_y = p->mTrackProjY;
        r.proj_xr = p->mTrackProjXR;
        r.view_cos = p->mTrackViewCos;
        r.track_scale_level = p->mnTrackScaleLevel;
        if (!r.bad) {
            const cv::Mat d = p->GetDescriptor();
            std::memcpy(&desc[i * 32], d.ptr<uint8_t>(0), 32);
        }
    }
    const std::vector<uint8_t> claimed = orbgpu_cv::claimed_of(F);
    std::vector<int> match(std::max<size_t>(F.mvKeysUn.size(), 1), -1);
    if (F.mvKeysUn.empty() || M == 0) return 0;
    int nm = 0;
    orbgpu_cv::check(orbgpu_search_by_projection(orbgpu_cv::matcher_for(mfNNratio, mbCheckOrientation), &f, rec.data(),
                                                 desc.data(), (int)M, th, claimed.data(), match.data(),
                                                 ORBGPU_MEM_HOST, &nm),
                     "SearchByProjection(Frame&, vector<MapPoint*>)");
    for (size_t i = 0; i < F.mvKeysUn.size(); i++)
        if (match[i] >= 0) F.mvpMapPoints[i] = vpMapPoints[match[i]];
    return nm;
}

int ORBmatcher::SearchByProjection(Frame& CurrentFrame, const Frame& LastFrame, const float th, const bool bMono) {
    const orbgpu_frame cur = orbgpu_cv::frame_view(CurrentFrame.mvKeysUn, CurrentFrame.mDescriptors, CurrentFrame,
                                                   CurrentFrame.mvuRight.empty() ? nullptr
                                                                                 : CurrentFrame.mvuRight.data());
    const orbgpu_frame last = orbgpu_cv::frame_view(LastFrame.mvKeysUn, LastFrame.mDescriptors, LastFrame, nullptr);
    const size_t NL = LastFrame.mvKeysUn.size();
    std::vector<orbgpu_frame_mappoint> mps(std::max<size_t>(NL, 1));
    std::vector<uint8_t> desc(std::max<size_t>(NL, 1) * 32, 0);
    for (size_t i = 0; i < NL; i++) {
        orbgpu_frame_mappoint& r = mps[i];
        std::memset(&r, 0, sizeof(r));
        MapPoint* p = i < LastFrame.mvpMapPoints.size() ? LastFrame.mvpMapPoints[i] : nullptr;
        if (!p) continue;
        r.flags = ORBGPU_MP_PRESENT;
        if (i < LastFrame.mvbOutlier.size() && LastFrame.mvbOutlier[i]) r.flags |= ORBGPU_MP_OUTLIER;
        if (p->Observations() > 0) r.flags |= ORBGPU_MP_OBSERVED;
        const cv::Mat x = p->GetWorldPos();
        r.x = x.at<float>(0);
        r.y = x.at<float>(1);
        r.z = x.at<float>(2);
        const cv::Mat d = p->GetDescriptor();
        std::memcpy(&desc[i * 32], d.ptr<uint8_t>(0), 32);
    }
    orbgpu_frame_motion mo;
    std::memset(&mo, 0, sizeof(mo));
    orbgpu_cv::rows_of(CurrentFrame.mTcw, mo.Tcw);
    orbgpu_cv::rows_of(LastFrame.mTcw, mo.Tlw);
    mo.fx = CurrentFrame.fx;
    mo.fy = CurrentFrame.fy;
    mo.cx = CurrentFrame.cx;
    mo.cy = CurrentFrame.cy;
    mo.bf = CurrentFrame.mbf;
    mo.b = CurrentFrame.mb;
    const std::vector<uint8_t> claimed = orbgpu_cv::claimed_of(CurrentFrame);
    std::vector<int> match(std::max<size_t>(CurrentFrame.mvKeysUn.size(), 1), -1);
    if (CurrentFrame.mvKeysUn.empty() || NL == 0) return 0;
    int nm = 0;
    orbgpu_cv::check(orbgpu_search_by_projection_frame(orbgpu_cv::matcher_for(mfNNratio, mbCheckOrientation), &cur,
                                                       &last, mps.data(), desc.data(), &mo, th, bMono ? 1 : 0,
                                                       claimed.data(), match.data(), ORBGPU_MEM_HOST, &nm),
                     "SearchByProjection(Frame&, const Frame&)");
    for (size_t i = 0; i < CurrentFrame.mvKeysUn.size(); i++) {
        if (match[i] >= 0) CurrentFrame.mvpMapPoints[i] = LastFrame.mvpMapPoints[match[i]];
        else if (match[i] == -4) CurrentFrame.mvpMapPoints[i] = static_cast<MapPoint*>(NULL);
    }
    return nm;
}

}  // namespace ORB_SLAM2
