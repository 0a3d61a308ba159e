// TEST INFRASTRUCTURE: the build check of the C++ adapter.  Linked with the
// adapter sources, the reference's own src/Frame.cc, src/MapPoint.cc and
// src/ORBmatcher.cc (that file compiled with the three replaced searches
// renamed away, as a host removes them) against the cv stand-in, and
// liborbgpu.so.
//
//   adapter_check layout     prints the record sizes (the static_asserts of
//                            orbgpu_cv.hpp already held at compile time)
//   adapter_check nodevice   constructs an ORBextractor and expects the
//                            library's error as an exception (no fallback)
//   adapter_check run W H A.raw B.raw
//                            on a GPU: two monocular Frames through the
//                            adapter's ORBextractor, SearchForInitialization
//                            (window 100, nnratio 0.9), prints counts
#include <cstdio>
#include <cstring>
#include <fstream>
#include <vector>

#include "Frame.h"
#include "ORBextractor.h"
#include "ORBmatcher.h"
#include "orbgpu_cv.hpp"

using namespace ORB_SLAM2;

static cv::Mat read_raw(const char* path, int w, int h) {
    cv::Mat m(h, w, CV_8U);
    std::ifstream f(path, std::ios::binary);
    f.read(reinterpret_cast<char*>(m.data), (std::streamsize)w * h);
    return m;
}

int main(int argc, char** argv) {
    const char* mode = argc > 1 ? argv[1] : "layout";
    if (!std::strcmp(mode, "layout")) {
        std::printf("keypoint %zu %zu point2f %zu\n", sizeof(cv::KeyPoint), sizeof(orbgpu_keypoint),
                    sizeof(cv::Point2f));
        return 0;
    }
    if (!std::strcmp(mode, "nodevice")) {
        try {
            ORBextractor ex(1000, 1.2f, 8, 20, 7);
            std::printf("constructed without error\n");
            return 1;
        } catch (const orbgpu_cv::Error& e) {
            std::printf("threw %d: %s\n", e.code(), e.what());
            return 0;
        }
    }
    if (!std::strcmp(mode, "run") && argc >= 6) {
        const int w = std::atoi(argv[2]), h = std::atoi(argv[3]);
        cv::Mat a = read_raw(argv[4], w, h), b = read_raw(argv[5], w, h);
        ORBextractor ex(1000, 1.2f, 8, 20, 7);
        cv::Mat K = cv::Mat::eye(3, 3, CV_32F);
        K.at<float>(0, 0) = 500.f;
        K.at<float>(1, 1) = 500.f;
        K.at<float>(0, 2) = w / 2.f;
        K.at<float>(1, 2) = h / 2.f;
        cv::Mat dist = cv::Mat::zeros(4, 1, CV_32F);
        Frame F1(a, 0.0, &ex, nullptr, K, dist, 0.f, 0.f);
        Frame F2(b, 0.1, &ex, nullptr, K, dist, 0.f, 0.f);
        std::vector<cv::Point2f> prev(F1.mvKeysUn.size());
        for (size_t i = 0; i < prev.size(); i++) prev[i] = F1.mvKeysUn[i].pt;
        std::vector<int> m12;
        ORBmatcher matcher(0.9f, true);
        const int nm = matcher.SearchForInitialization(F1, F2, prev, m12, 100);
        std::printf("keypoints %d %d matches %d\n", F1.N, F2.N, nm);
        return 0;
    }
    std::fprintf(stderr, "usage: adapter_check layout | nodevice | run W H A.raw B.raw\n");
    return 2;
}
