// The reference's own CUDA launchers, compiled for sm_103a from the copies
// that build_ref_gpu.py makes of Tracking/Pyrdown.cu, Reduction.cu,
// Mapping/FuseMap.cu, RenderScene.cu and DeviceMap.cu, driven in
// System::GrabImage's order by ref_loop.h.  Test infrastructure: a timing
// baseline and a parity reference, never shipped.
#include "ref_loop.h"

extern "C" void *refgpu_create(int cols, int rows, const float *K, float depth_scale, float cutoff,
                               const double *init_pose) {
  return refloop_create(cols, rows, K, depth_scale, cutoff, init_pose);
}
// One frame of System::GrabImage; returns 1 when the frame was tracked.
extern "C" int refgpu_grab(void *h, const uint16_t *depth, const uint8_t *rgb, double *pose_out) {
  return refloop_grab(h, depth, rgb, pose_out);
}
extern "C" void refgpu_destroy(void *h) { refloop_destroy(h); }
extern "C" void refgpu_set_rgb(void *h, int on) { refloop_set_rgb(h, on); }
extern "C" void refgpu_map_arrays(void *h, void **out6, long long *sizes2) { refloop_map_arrays(h, out6, sizes2); }
