// ORACLE / TEST INFRASTRUCTURE ONLY: declared so the reference compiles; aborts if called.
#ifndef CVSHIM_CALIB3D_HPP
#define CVSHIM_CALIB3D_HPP
#include "../core/core.hpp"
namespace cv {
void undistortPoints(InputArray src, OutputArray dst, InputArray cameraMatrix, InputArray distCoeffs,
                     InputArray R = noArray(), InputArray P = noArray());
}
#endif
