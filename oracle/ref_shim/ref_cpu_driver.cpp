// The reference's device code compiled as host C++ by build_ref.py (the CUDA
// emulation header in SHIM_OMP mode: OpenMP over each launch's blocks),
// driven in System::GrabImage's order by ref_loop.h: the reference's own
// loop on the host cores, the benchmark's CPU baseline.  ICP-only tracking.
// Test and benchmark infrastructure, never shipped.
#include <omp.h>

#include "ref_loop.h"

thread_local uint3 threadIdx;
thread_local uint3 blockIdx;
thread_local dim3 blockDim;
thread_local dim3 gridDim;

extern "C" void *refcpu_create(int cols, int rows, const float *K, float depth_scale, float cutoff,
                               const double *init_pose) {
  return refloop_create(cols, rows, K, depth_scale, cutoff, init_pose);
}
// One frame of System::GrabImage; returns 1 when the frame was tracked.
extern "C" int refcpu_grab(void *h, const uint16_t *depth, const uint8_t *rgb, double *pose_out) {
  return refloop_grab(h, depth, rgb, pose_out);
}
extern "C" void refcpu_destroy(void *h) { refloop_destroy(h); }
// Host threads the OpenMP launches use.
extern "C" int refcpu_threads() { return omp_get_max_threads(); }
