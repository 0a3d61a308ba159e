// ORACLE / TEST INFRASTRUCTURE ONLY.
// Link stubs for the reference classes that src/ORBmatcher.cc, src/Frame.cc
// and src/MapPoint.cc reference but whose own sources (src/KeyFrame.cc,
// src/Map.cc, src/Converter.cc) need Eigen/g2o/DBoW2 vocabularies and are off
// the feature path.  The keyframe constructor copies only the fields the
// compiled reference code reads (mnFrameId, fx, fy, cx, cy, mvKeysUn, mvuRight,
// mDescriptors, mvScaleFactors, mvLevelSigma2) and zeroes the rest; the
// accessors the path uses (isBad, GetMapPointMatches, GetMapPoint,
// GetCameraCenter, GetRotation, GetTranslation, IsInImage,
// GetFeaturesInArea) compute exactly as src/KeyFrame.cc does (without its
// locking); the constructor also copies the grid, image bounds and pyramid
// constants;
// everything else aborts if called.
#include "MapPoint.h"
#include "KeyFrame.h"
#include "Map.h"
#include "Converter.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>

namespace ORB_SLAM2 {

[[noreturn]] static void stub_unreachable(const char* what) {
    std::fprintf(stderr, "reference stub reached: %s\n", what);
    std::abort();
}

long unsigned int KeyFrame::nNextId = 0;

KeyFrame::KeyFrame(Frame& F, Map* pMap, KeyFrameDatabase* pKFDB)
    : mnFrameId(F.mnId), mTimeStamp(0), mnGridCols(FRAME_GRID_COLS), mnGridRows(FRAME_GRID_ROWS),
      mfGridElementWidthInv(F.mfGridElementWidthInv), mfGridElementHeightInv(F.mfGridElementHeightInv), mnTrackReferenceForFrame(0), mnFuseTargetForKF(0), mnBALocalForKF(0),
      mnBAFixedForKF(0), mnLoopQuery(0), mnLoopWords(0), mLoopScore(0), mnRelocQuery(0), mnRelocWords(0),
      mRelocScore(0), mnBAGlobalForKF(0), fx(F.fx), fy(F.fy), cx(F.cx), cy(F.cy), invfx(0), invfy(0), mbf(F.mbf), mb(0),
      mThDepth(0), N(F.N), mvKeysUn(F.mvKeysUn), mvuRight(F.mvuRight), mDescriptors(F.mDescriptors.clone()),
      mnScaleLevels(F.mnScaleLevels), mvScaleFactors(F.mvScaleFactors), mvLevelSigma2(F.mvLevelSigma2),
      mvInvLevelSigma2(F.mvInvLevelSigma2),
      mfScaleFactor(F.mfScaleFactor), mfLogScaleFactor(F.mfLogScaleFactor), mnMinX(F.mnMinX), mnMinY(F.mnMinY),
      mnMaxX(F.mnMaxX), mnMaxY(F.mnMaxY), mpKeyFrameDB(pKFDB),
      mpORBvocabulary(nullptr), mbFirstConnection(true), mpParent(nullptr), mbNotErase(false),
      mbToBeErased(false), mbBad(false), mHalfBaseline(0), mpMap(pMap) {
    mnId = nNextId++;
    mGrid.resize(mnGridCols);
    for (int i = 0; i < mnGridCols; i++) {
        mGrid[i].resize(mnGridRows);
        for (int j = 0; j < mnGridRows; j++) mGrid[i][j] = F.mGrid[i][j];
    }
}

bool KeyFrame::isBad() { return mbBad; }
// src/KeyFrame.cc: mvpMapPoints[idx] = pMP
void KeyFrame::AddMapPoint(MapPoint* pMP, const size_t& idx) { mvpMapPoints[idx] = pMP; }
void KeyFrame::EraseMapPointMatch(const size_t&) { stub_unreachable("KeyFrame::EraseMapPointMatch"); }
void KeyFrame::EraseMapPointMatch(MapPoint*) { stub_unreachable("KeyFrame::EraseMapPointMatch"); }
void KeyFrame::ReplaceMapPointMatch(const size_t&, MapPoint*) { stub_unreachable("KeyFrame::ReplaceMapPointMatch"); }
cv::Mat KeyFrame::GetCameraCenter() { return Ow.clone(); }
// src/KeyFrame.cc:785-830: the grid cells overlapping the square window,
// then |dx| < r and |dy| < r on every keypoint of them.
std::vector<size_t> KeyFrame::GetFeaturesInArea(const float& x, const float& y, const float& r) const {
    std::vector<size_t> out;
    const int x0 = std::max(0, (int)floor((x - mnMinX - r) * mfGridElementWidthInv));
    if (x0 >= mnGridCols) return out;
    const int x1 = std::min((int)mnGridCols - 1, (int)ceil((x - mnMinX + r) * mfGridElementWidthInv));
    if (x1 < 0) return out;
    const int y0 = std::max(0, (int)floor((y - mnMinY - r) * mfGridElementHeightInv));
    if (y0 >= mnGridRows) return out;
    const int y1 = std::min((int)mnGridRows - 1, (int)ceil((y - mnMinY + r) * mfGridElementHeightInv));
    if (y1 < 0) return out;
    for (int ix = x0; ix <= x1; ix++)
        for (int iy = y0; iy <= y1; iy++)
            for (size_t k : mGrid[ix][iy]) {
                const cv::KeyPoint& kp = mvKeysUn[k];
                if (fabs(kp.pt.x - x) < r && fabs(kp.pt.y - y) < r) out.push_back(k);
            }
    return out;
}
MapPoint* KeyFrame::GetMapPoint(const size_t& idx) { return mvpMapPoints[idx]; }
std::vector<MapPoint*> KeyFrame::GetMapPointMatches() { return mvpMapPoints; }
// src/KeyFrame.cc: the map points of the keyframe that are not bad
std::set<MapPoint*> KeyFrame::GetMapPoints() {
    std::set<MapPoint*> s;
    for (MapPoint* pMP : mvpMapPoints)
        if (pMP && !pMP->isBad()) s.insert(pMP);
    return s;
}
cv::Mat KeyFrame::GetRotation() { return Tcw.rowRange(0, 3).colRange(0, 3).clone(); }
cv::Mat KeyFrame::GetTranslation() { return Tcw.rowRange(0, 3).col(3).clone(); }
// src/KeyFrame.cc:832-835
bool KeyFrame::IsInImage(const float& x, const float& y) const {
    return x >= mnMinX && x < mnMaxX && y >= mnMinY && y < mnMaxY;
}

Map::Map() : mnMaxKFid(0), mnBigChangeIdx(0) {}
void Map::EraseMapPoint(MapPoint*) { stub_unreachable("Map::EraseMapPoint"); }

std::vector<cv::Mat> Converter::toDescriptorVector(const cv::Mat&) { stub_unreachable("Converter::toDescriptorVector"); }

}  // namespace ORB_SLAM2
