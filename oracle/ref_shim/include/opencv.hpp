// Minimal stand-in for <opencv.hpp>: the reference's Tracking/Reduction.h
// names cv::cuda::GpuMat only in a declaration the recipe never calls.
#pragma once
namespace cv { namespace cuda { struct GpuMat {}; } }
