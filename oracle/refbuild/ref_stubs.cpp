// ORACLE / TEST INFRASTRUCTURE ONLY.
// Link stubs for the reference classes that src/ORBmatcher.cc, src/Frame.cc
// and src/MapPoint.cc reference but whose own sources (src/KeyFrame.cc,
// src/Map.cc, src/Converter.cc) need Eigen/g2o/DBoW2 vocabularies and are off
// the feature path.  The keyframe constructor copies only the fields the
// compiled reference code reads (mnFrameId, fx, fy, cx, cy, mvKeysUn, mvuRight,
// mDescriptors, mvScaleFactors, mvLevelSigma2) and zeroes the rest; the
// accessors the path uses (isBad, GetMapPointMatches, GetMapPoint,
// GetCameraCenter, GetRotation, GetTranslation) return the stored fields
// exactly as src/KeyFrame.cc does (without its locking);
// everything else aborts if called.
#include "MapPoint.h"
#include "KeyFrame.h"
#include "Map.h"
#include "Converter.h"

#include <cstdio>
#include <cstdlib>

namespace ORB_SLAM2 {

[[noreturn]] static void stub_unreachable(const char* what) {
    std::fprintf(stderr, "reference stub reached: %s\n", what);
    std::abort();
}

long unsigned int KeyFrame::nNextId = 0;

KeyFrame::KeyFrame(Frame& F, Map* pMap, KeyFrameDatabase* pKFDB)
    : mnFrameId(F.mnId), mTimeStamp(0), mnGridCols(0), mnGridRows(0), mfGridElementWidthInv(0),
      mfGridElementHeightInv(0), mnTrackReferenceForFrame(0), mnFuseTargetForKF(0), mnBALocalForKF(0),
      mnBAFixedForKF(0), mnLoopQuery(0), mnLoopWords(0), mLoopScore(0), mnRelocQuery(0), mnRelocWords(0),
      mRelocScore(0), mnBAGlobalForKF(0), fx(F.fx), fy(F.fy), cx(F.cx), cy(F.cy), invfx(0), invfy(0), mbf(0), mb(0),
      mThDepth(0), N(F.N), mvKeysUn(F.mvKeysUn), mvuRight(F.mvuRight), mDescriptors(F.mDescriptors.clone()),
      mnScaleLevels(0), mvScaleFactors(F.mvScaleFactors), mvLevelSigma2(F.mvLevelSigma2),
      mfScaleFactor(0), mfLogScaleFactor(0), mnMinX(0), mnMinY(0), mnMaxX(0), mnMaxY(0), mpKeyFrameDB(pKFDB),
      mpORBvocabulary(nullptr), mbFirstConnection(true), mpParent(nullptr), mbNotErase(false),
      mbToBeErased(false), mbBad(false), mHalfBaseline(0), mpMap(pMap) {
    mnId = nNextId++;
}

bool KeyFrame::isBad() { return mbBad; }
void KeyFrame::AddMapPoint(MapPoint*, const size_t&) { stub_unreachable("KeyFrame::AddMapPoint"); }
void KeyFrame::EraseMapPointMatch(const size_t&) { stub_unreachable("KeyFrame::EraseMapPointMatch"); }
void KeyFrame::EraseMapPointMatch(MapPoint*) { stub_unreachable("KeyFrame::EraseMapPointMatch"); }
void KeyFrame::ReplaceMapPointMatch(const size_t&, MapPoint*) { stub_unreachable("KeyFrame::ReplaceMapPointMatch"); }
cv::Mat KeyFrame::GetCameraCenter() { return Ow.clone(); }
std::vector<size_t> KeyFrame::GetFeaturesInArea(const float&, const float&, const float&) const {
    stub_unreachable("KeyFrame::GetFeaturesInArea");
}
MapPoint* KeyFrame::GetMapPoint(const size_t& idx) { return mvpMapPoints[idx]; }
std::vector<MapPoint*> KeyFrame::GetMapPointMatches() { return mvpMapPoints; }
std::set<MapPoint*> KeyFrame::GetMapPoints() { stub_unreachable("KeyFrame::GetMapPoints"); }
cv::Mat KeyFrame::GetRotation() { return Tcw.rowRange(0, 3).colRange(0, 3).clone(); }
cv::Mat KeyFrame::GetTranslation() { return Tcw.rowRange(0, 3).col(3).clone(); }
bool KeyFrame::IsInImage(const float&, const float&) const { stub_unreachable("KeyFrame::IsInImage"); }

Map::Map() : mnMaxKFid(0), mnBigChangeIdx(0) {}
void Map::EraseMapPoint(MapPoint*) { stub_unreachable("Map::EraseMapPoint"); }

std::vector<cv::Mat> Converter::toDescriptorVector(const cv::Mat&) { stub_unreachable("Converter::toDescriptorVector"); }

}  // namespace ORB_SLAM2
