// ORACLE / TEST INFRASTRUCTURE ONLY.
// Link stubs for the reference classes that src/ORBmatcher.cc and src/Frame.cc
// reference but whose own sources (src/MapPoint.cc, src/KeyFrame.cc,
// src/Converter.cc) need Eigen/g2o/DBoW2 vocabularies and are off the feature
// path.  The accessors the path does use (MapPoint::isBad, Observations,
// GetDescriptor, GetWorldPos) return the stored fields exactly as the
// reference's src/MapPoint.cc does (without its locking); everything else
// aborts if called.
#include "MapPoint.h"
#include "KeyFrame.h"
#include "Converter.h"

#include <cstdio>
#include <cstdlib>

namespace ORB_SLAM2 {

[[noreturn]] static void stub_unreachable(const char* what) {
    std::fprintf(stderr, "reference stub reached: %s\n", what);
    std::abort();
}

long unsigned int MapPoint::nNextId = 0;
std::mutex MapPoint::mGlobalMutex;

// Only the harness constructs map points: a point with one observation
// (src/MapPoint.cc keeps nObs as the number of keyframe observations).
MapPoint::MapPoint(const cv::Mat& Pos, KeyFrame* pRefKF, Map* pMap)
    : mnFirstKFid(0), mnFirstFrame(0), nObs(1), mnTrackReferenceForFrame(0), mnLastFrameSeen(0),
      mnBALocalForKF(0), mnFuseCandidateForKF(0), mnLoopPointForKF(0), mnCorrectedByKF(0),
      mnCorrectedReference(0), mnBAGlobalForKF(0), mpRefKF(pRefKF), mnVisible(1), mnFound(1), mbBad(false),
      mpReplaced(static_cast<MapPoint*>(NULL)), mfMinDistance(0), mfMaxDistance(0), mpMap(pMap) {
    Pos.copyTo(mWorldPos);
    mNormalVector = cv::Mat::zeros(3, 1, CV_32F);
    mnId = nNextId++;
}

bool MapPoint::isBad() { return mbBad; }
int MapPoint::Observations() { return nObs; }
cv::Mat MapPoint::GetDescriptor() { return mDescriptor.clone(); }
cv::Mat MapPoint::GetWorldPos() { return mWorldPos.clone(); }
cv::Mat MapPoint::GetNormal() { return mNormalVector.clone(); }
void MapPoint::AddObservation(KeyFrame*, size_t) { stub_unreachable("MapPoint::AddObservation"); }
int MapPoint::GetIndexInKeyFrame(KeyFrame*) { stub_unreachable("MapPoint::GetIndexInKeyFrame"); }
bool MapPoint::IsInKeyFrame(KeyFrame*) { stub_unreachable("MapPoint::IsInKeyFrame"); }
float MapPoint::GetMinDistanceInvariance() { stub_unreachable("MapPoint::GetMinDistanceInvariance"); }
float MapPoint::GetMaxDistanceInvariance() { stub_unreachable("MapPoint::GetMaxDistanceInvariance"); }
int MapPoint::PredictScale(const float&, KeyFrame*) { stub_unreachable("MapPoint::PredictScale"); }
int MapPoint::PredictScale(const float&, Frame*) { stub_unreachable("MapPoint::PredictScale"); }
void MapPoint::Replace(MapPoint*) { stub_unreachable("MapPoint::Replace"); }

void KeyFrame::AddMapPoint(MapPoint*, const size_t&) { stub_unreachable("KeyFrame::AddMapPoint"); }
cv::Mat KeyFrame::GetCameraCenter() { stub_unreachable("KeyFrame::GetCameraCenter"); }
std::vector<size_t> KeyFrame::GetFeaturesInArea(const float&, const float&, const float&) const {
    stub_unreachable("KeyFrame::GetFeaturesInArea");
}
MapPoint* KeyFrame::GetMapPoint(const size_t&) { stub_unreachable("KeyFrame::GetMapPoint"); }
std::vector<MapPoint*> KeyFrame::GetMapPointMatches() { stub_unreachable("KeyFrame::GetMapPointMatches"); }
std::set<MapPoint*> KeyFrame::GetMapPoints() { stub_unreachable("KeyFrame::GetMapPoints"); }
cv::Mat KeyFrame::GetRotation() { stub_unreachable("KeyFrame::GetRotation"); }
cv::Mat KeyFrame::GetTranslation() { stub_unreachable("KeyFrame::GetTranslation"); }
bool KeyFrame::IsInImage(const float&, const float&) const { stub_unreachable("KeyFrame::IsInImage"); }

std::vector<cv::Mat> Converter::toDescriptorVector(const cv::Mat&) { stub_unreachable("Converter::toDescriptorVector"); }

}  // namespace ORB_SLAM2
