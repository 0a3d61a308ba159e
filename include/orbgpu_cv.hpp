/* orbgpu_cv.hpp -- the C++ side of the drop-in boundary.
 *
 * For hosts built against the reference's headers (include/ORBextractor.h,
 * include/ORBmatcher.h, include/Frame.h) and an OpenCV-compatible cv::
 * namespace.  The adapter sources (orb_slam2_detailed_comments_gb300/adapter/)
 * define ORB_SLAM2::ORBextractor's constructor and operator(), and
 * ORBmatcher's SearchForInitialization and two SearchByProjection overloads,
 * on top of the C ABI in orbgpu.h.  This header holds what they share: the
 * layout checks that let keypoint records cross the ABI by memcpy, the status
 * check that turns a library error into an exception (there is no CPU
 * fallback: without the library or a device every call throws), and the
 * extractor-handle registry.
 */
#ifndef ORBGPU_CV_HPP
#define ORBGPU_CV_HPP

#include <cstddef>
#include <stdexcept>
#include <string>

#include <opencv2/core/core.hpp>
#include <opencv2/features2d/features2d.hpp>

#include "orbgpu.h"

namespace ORB_SLAM2 {
class Frame;
}

namespace orbgpu_cv {

/* cv::KeyPoint crosses the ABI as orbgpu_keypoint (pt.x, pt.y, size, angle,
 * response, octave, class_id: 28 bytes), cv::Point2f as two floats. */
static_assert(sizeof(cv::KeyPoint) == sizeof(orbgpu_keypoint), "cv::KeyPoint is not 28 bytes");
static_assert(offsetof(cv::KeyPoint, pt) == offsetof(orbgpu_keypoint, x), "cv::KeyPoint::pt.x offset");
static_assert(offsetof(cv::KeyPoint, size) == offsetof(orbgpu_keypoint, size), "cv::KeyPoint::size offset");
static_assert(offsetof(cv::KeyPoint, angle) == offsetof(orbgpu_keypoint, angle), "cv::KeyPoint::angle offset");
static_assert(offsetof(cv::KeyPoint, response) == offsetof(orbgpu_keypoint, response),
              "cv::KeyPoint::response offset");
static_assert(offsetof(cv::KeyPoint, octave) == offsetof(orbgpu_keypoint, octave), "cv::KeyPoint::octave offset");
static_assert(offsetof(cv::KeyPoint, class_id) == offsetof(orbgpu_keypoint, class_id),
              "cv::KeyPoint::class_id offset");
static_assert(sizeof(cv::Point2f) == 2 * sizeof(float), "cv::Point2f is not two floats");

/* A library status other than ORBGPU_OK as an exception carrying the
 * library's last error message. */
class Error : public std::runtime_error {
public:
    Error(int code, const std::string& what) : std::runtime_error(what), code_(code) {}
    int code() const { return code_; }

private:
    int code_;
};

inline void check(int rc, const char* where) {
    if (rc != ORBGPU_OK) {
        const char* m = orbgpu_last_error();
        throw Error(rc, std::string(where) + ": orbgpu status " + std::to_string(rc) + " (" + (m ? m : "") + ")");
    }
}

/* The library handle behind an ORB_SLAM2::ORBextractor object (created by the
 * adapter's constructor).  The reference's destructor is defined inline in
 * its header and cannot release it; release_extractor() does, and
 * handles of destroyed objects are otherwise kept until the process exits. */
orbgpu_extractor* extractor_handle(const void* orb_extractor);
void release_extractor(const void* orb_extractor);

/* Whether operator() also copies the unblurred pyramid to the host into
 * mvImagePyramid (the reference's public member, read by the reference's own
 * Frame::ComputeStereoMatches).  On by default; hosts that run the stereo
 * search through the library (ComputeStereoMatches below) can turn it off. */
void set_copy_pyramid(bool on);
bool copy_pyramid();

/* Frame::ComputeStereoMatches() (src/Frame.cc:831-1082) through the library:
 * fills F.mvuRight and F.mvDepth from F.mvKeys / F.mvKeysRight and the
 * pyramids the frame's two adapter extractors left on the device.  A host
 * calls it where the stereo Frame constructor calls ComputeStereoMatches(). */
void ComputeStereoMatches(ORB_SLAM2::Frame& F);

}  // namespace orbgpu_cv

#endif  // ORBGPU_CV_HPP
