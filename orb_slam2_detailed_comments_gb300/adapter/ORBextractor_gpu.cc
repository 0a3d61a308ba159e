// ORB_SLAM2::ORBextractor on the GPU library: a replacement for the
// reference's src/ORBextractor.cc, compiled against its unchanged
// include/ORBextractor.h.  The constructor (include/ORBextractor.h:93,
// src/ORBextractor.cc:469-571) creates a library extractor and reads the
// scale tables from it (the library computes them with the reference's
// arithmetic); operator() (include/ORBextractor.h:111,
// src/ORBextractor.cc:1533-1649) runs the whole extraction in the library
// and fills keypoints, descriptors and mvImagePyramid as the reference does.
// The protected helpers (ComputePyramid, ComputeKeyPointsOctTree,
// DistributeOctTree, ComputeKeyPointsOld) are only called from inside the
// reference's operator() and are not defined here; 'pattern' and 'umax' stay
// empty (the library holds its own copies).
#include <cassert>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "ORBextractor.h"
#include "orbgpu_cv.hpp"
#include "orbgpu_ext.h"

namespace orbgpu_cv {
namespace {
std::mutex g_mu;
std::map<const void*, orbgpu_extractor*> g_handles;
bool g_copy_pyramid = true;
}  // namespace

orbgpu_extractor* extractor_handle(const void* ex) {
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_handles.find(ex);
    return it == g_handles.end() ? nullptr : it->second;
}

void release_extractor(const void* ex) {
    orbgpu_extractor* h = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        auto it = g_handles.find(ex);
        if (it == g_handles.end()) return;
        h = it->second;
        g_handles.erase(it);
    }
    orbgpu_extractor_destroy(h);
}

static void register_extractor(const void* ex, orbgpu_extractor* h) {
    orbgpu_extractor* old = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        // a new object at the address of a destroyed one replaces its handle
        auto it = g_handles.find(ex);
        if (it != g_handles.end()) old = it->second;
        g_handles[ex] = h;
    }
    if (old) orbgpu_extractor_destroy(old);
}

void set_copy_pyramid(bool on) { g_copy_pyramid = on; }
bool copy_pyramid() { return g_copy_pyramid; }

}  // namespace orbgpu_cv

namespace ORB_SLAM2 {

ORBextractor::ORBextractor(int _nfeatures, float _scaleFactor, int _nlevels, int _iniThFAST, int _minThFAST)
    : nfeatures(_nfeatures), scaleFactor(_scaleFactor), nlevels(_nlevels), iniThFAST(_iniThFAST),
      minThFAST(_minThFAST) {
    orbgpu_extractor* h = nullptr;
    // max size 0 x 0: the handle sizes its buffers for each image it sees
    orbgpu_cv::check(orbgpu_extractor_create(nfeatures, _scaleFactor, nlevels, iniThFAST, minThFAST, 0, 0, nullptr, &h),
                     "ORBextractor::ORBextractor");
    orbgpu_cv::register_extractor(this, h);
    mvScaleFactor.resize(nlevels);
    mvInvScaleFactor.resize(nlevels);
    mvLevelSigma2.resize(nlevels);
    mvInvLevelSigma2.resize(nlevels);
    mnFeaturesPerLevel.resize(nlevels);
    int nl = 0;
    orbgpu_cv::check(orbgpu_extractor_tables(h, &nl, mvScaleFactor.data(), mvInvScaleFactor.data(),
                                             mvLevelSigma2.data(), mvInvLevelSigma2.data(), mnFeaturesPerLevel.data()),
                     "ORBextractor tables");
    mvImagePyramid.resize(nlevels);
}

void ORBextractor::operator()(cv::InputArray _image, cv::InputArray _mask, std::vector<cv::KeyPoint>& _keypoints,
                              cv::OutputArray _descriptors) {
    (void)_mask;  // ignored by the reference too
    if (_image.empty()) return;
    cv::Mat image = _image.getMat();
    assert(image.type() == CV_8UC1);
    orbgpu_extractor* h = orbgpu_cv::extractor_handle(this);
    if (!h) throw orbgpu_cv::Error(ORBGPU_ERR_BAD_ARG, "ORBextractor: no library handle for this object");
    // DistributeOctTree may keep a few more keypoints per level than asked
    int cap = nfeatures + 64 * nlevels + 64;
    std::vector<orbgpu_keypoint> kps;
    std::vector<uint8_t> desc;
    int n = 0;
    for (;;) {
        kps.resize(cap);
        desc.resize((size_t)cap * 32);
        const int rc = orbgpu_extract(h, image.data, image.cols, image.rows, image.step[0], ORBGPU_MEM_HOST,
                                      kps.data(), desc.data(), cap, ORBGPU_MEM_HOST, &n);
        if (rc == ORBGPU_ERR_CAPACITY && n > cap) {
            cap = n;
            continue;
        }
        orbgpu_cv::check(rc, "ORBextractor::operator()");
        break;
    }
    // keypoints level-major in the reference's order, coordinates at level 0
    _keypoints.resize(n);
    if (n > 0) std::memcpy(_keypoints.data(), kps.data(), sizeof(orbgpu_keypoint) * (size_t)n);
    if (n == 0) {
        _descriptors.release();
    } else {
        _descriptors.create(n, 32, CV_8U);
        cv::Mat d = _descriptors.getMat();
        for (int i = 0; i < n; i++) std::memcpy(d.ptr<uint8_t>(i), desc.data() + (size_t)i * 32, 32);
    }
    if (orbgpu_cv::copy_pyramid()) {
        mvImagePyramid.resize(nlevels);
        for (int l = 0; l < nlevels; l++) {
            const uint8_t* p = nullptr;
            int w = 0, hh = 0;
            size_t pitch = 0;
            orbgpu_cv::check(orbgpu_extractor_pyramid_level(h, l, &p, &w, &hh, &pitch), "mvImagePyramid");
            mvImagePyramid[l] = cv::Mat(hh, w, CV_8U);
            std::vector<uint8_t> rows((size_t)hh * pitch);
            orbgpu_cv::check(orbgpu_copy_to_host(rows.data(), p, rows.size()), "mvImagePyramid copy");
            for (int r = 0; r < hh; r++) std::memcpy(mvImagePyramid[l].ptr<uint8_t>(r), rows.data() + (size_t)r * pitch, w);
        }
    }
}

}  // namespace ORB_SLAM2
