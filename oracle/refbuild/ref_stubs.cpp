// ORACLE / TEST INFRASTRUCTURE ONLY.
// Link stubs for the reference classes that src/ORBmatcher.cc, src/Frame.cc
// and src/MapPoint.cc reference but whose own sources (src/KeyFrame.cc,
// src/Map.cc, src/Converter.cc) need Eigen/g2o/DBoW2 vocabularies and are off
// the feature path.  The keyframe constructor copies only the fields the
// compiled reference code reads (mnFrameId, mvKeysUn, mvuRight, mDescriptors)
// and zeroes the rest; the accessors the path uses (KeyFrame::isBad,
// GetMapPointMatches) return the stored fields exactly as src/KeyFrame.cc
// does (without its locking);
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
      mRelocScore(0), mnBAGlobalForKF(0), fx(0), fy(0), cx(0), cy(0), invfx(0), invfy(0), mbf(0), mb(0),
      mThDepth(0), N(F.N), mvKeysUn(F.mvKeysUn), mvuRight(F.mvuRight), mDescriptors(F.mDescriptors.clone()),
      mnScaleLevels(0),
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
cv::Mat KeyFrame::GetCameraCenter() { stub_unreachable("KeyFrame::GetCameraCenter"); }
std::vector<size_t> KeyFrame::GetFeaturesInArea(const float&, const float&, const float&) const {
    stub_unreachable("KeyFrame::GetFeaturesInArea");
}
MapPoint* KeyFrame::GetMapPoint(const size_t&) { stub_unreachable("KeyFrame::GetMapPoint"); }
std::vector<MapPoint*> KeyFrame::GetMapPointMatches() { return mvpMapPoints; }
std::set<MapPoint*> KeyFrame::GetMapPoints() { stub_unreachable("KeyFrame::GetMapPoints"); }
cv::Mat KeyFrame::GetRotation() { stub_unreachable("KeyFrame::GetRotation"); }
cv::Mat KeyFrame::GetTranslation() { stub_unreachable("KeyFrame::GetTranslation"); }
bool KeyFrame::IsInImage(const float&, const float&) const { stub_unreachable("KeyFrame::IsInImage"); }

Map::Map() : mnMaxKFid(0), mnBigChangeIdx(0) {}
void Map::EraseMapPoint(MapPoint*) { stub_unreachable("Map::EraseMapPoint"); }

std::vector<cv::Mat> Converter::toDescriptorVector(const cv::Mat&) { stub_unreachable("Converter::toDescriptorVector"); }

}  // namespace ORB_SLAM2
