// ORACLE / TEST INFRASTRUCTURE ONLY: umbrella header of the cv stand-in.
#ifndef CVSHIM_OPENCV_HPP
#define CVSHIM_OPENCV_HPP
#include "core/core.hpp"
#include "imgproc/imgproc.hpp"
#include "features2d/features2d.hpp"
#include "calib3d/calib3d.hpp"
#include "highgui/highgui.hpp"
#endif
