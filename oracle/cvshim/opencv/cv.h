// ORACLE / TEST INFRASTRUCTURE ONLY: OpenCV 2.x/3.x compatibility umbrella of the cv stand-in.
#ifndef CVSHIM_CV_H
#define CVSHIM_CV_H
#include "../opencv2/opencv.hpp"
#endif
