// ORACLE / TEST INFRASTRUCTURE ONLY: cv feature-detection stand-ins (see cvshim_prims.h).
#ifndef CVSHIM_FEATURES2D_HPP
#define CVSHIM_FEATURES2D_HPP
#include "../core/core.hpp"
namespace cv {
void FAST(InputArray image, std::vector<KeyPoint>& keypoints, int threshold, bool nonmaxSuppression = true);
class KeyPointsFilter {
public:
    static void retainBest(std::vector<KeyPoint>& keypoints, int npoints);
};
}  // namespace cv
#endif
