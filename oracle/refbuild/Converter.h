// ORACLE / TEST INFRASTRUCTURE ONLY.
// Stand-in for the reference's include/Converter.h, which needs Eigen and g2o.
// src/Frame.cc only uses Converter::toDescriptorVector (in Frame::ComputeBoW,
// src/Frame.cc:711), which the feature path never reaches.
#ifndef ORB_SLAM2_CONVERTER_STUB_H
#define ORB_SLAM2_CONVERTER_STUB_H
#include <opencv2/core/core.hpp>
#include <vector>
namespace ORB_SLAM2 {
class Converter {
public:
    static std::vector<cv::Mat> toDescriptorVector(const cv::Mat& Descriptors);
};
}  // namespace ORB_SLAM2
#endif
