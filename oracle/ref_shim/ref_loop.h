// The reference's per-frame loop driven through its own launchers, in
// System::GrabImage's order (Core/System.cc:131-270):
//   Tracker::GrabFrame  -> LastFrame->ResizeImages, NextFrame->FillImages
//                          (Core/Frame.cc:68-98)
//   Tracker::Track      -> first frame: InitTracking + SwapFrame; then
//                          TrackFrame / ComputeSE3 (Tracking/Tracking.cc
//                          :65-173, 369-517) and SwapFrame on success
//   Mapping::FuseColor, Mapping::RayTrace (Mapping/Mapping.cc:76-161) on
//                          the last frame.
// Compiled twice by the recipes under oracle/ref_shim: with nvcc against the
// reference's CUDA sources (ref_gpu_driver.cu, the reference CUDA build), and
// with g++ against the same sources compiled as host C++ through the CUDA
// emulation header (ref_cpu_driver.cpp, OpenMP over each launch's blocks).
//
// ComputeSE3 runs ICP-only (its icpOnly = true path), or on the GPU, after
// set_rgb(1), with the photometric term (icpOnly = false, the reference's
// default): the reference's RGBStep before ICPStep in every iteration and
// the combined solve.  On the GPU the ICP sums are ICPStep's (the
// reference's Reduce / ReduceSum kernels and download); on the host they
// are the reference's ICPReduce::getRow for every pixel summed in FP64 per
// host thread (ref_icp_sums_impl, appended to Reduction.cu's host copy by
// build_ref.py), because the warp-shuffle block reduction has no serial
// form.  The host 6x6 solve, SE(3) update, divergence guard and acceptance
// gate are semantic_icpslam_gb300/csrc/sf_solve.h's FP64 restatement of
// Eigen LDLT and Sophus (the reference's Eigen/Sophus/OpenCV host code
// cannot be built here).  Keypoints, keyframes and the viewer are not part
// of the loop.  Test infrastructure: a timing baseline, never shipped.
#ifndef REF_LOOP_H_
#define REF_LOOP_H_
#include <cstdint>
#include <cstring>
#include <new>

#include "Reduction.h"
#include "RenderScene.h"
#include "sf_solve.h"

#ifdef REF_SHIM_CUDA_RUNTIME_H_
extern "C" void ref_icp_sums_impl(const float *vc, const float *vl, const float *nc, const float *nl, int cols,
                                  int rows, const float *Rc, const float *tc, const float *Rl, const float *RlInv,
                                  const float *tl, float fx, float fy, float cx, float cy, double *sums29);
#endif

namespace {

constexpr int kLevels = 3;
const int kIters[kLevels] = {10, 5, 4};          // ITERATIONS_SE3 (level 0 first)
const int kMinCount[kLevels] = {2000, 1000, 100};  // MIN_ICP_COUNT
constexpr float kThreshICP = 1e-4f;              // THRESH_ICP_SE3

struct RefFrame {
  DeviceArray2D<unsigned short> temp;
  DeviceArray2D<uchar3> color;
  DeviceArray2D<float> range;
  DeviceArray2D<float> depth[kLevels];
  DeviceArray2D<unsigned char> image[kLevels];
  DeviceArray2D<float4> vmap[kLevels], nmap[kLevels];
  DeviceArray2D<short> dIdx[kLevels], dIdy[kLevels];
  double pose[16];
  void create(int cols, int rows) {
    temp.create(cols, rows);
    color.create(cols, rows);
    range.create(cols, rows);
    for (int i = 0; i < kLevels; ++i) {
      const int c = cols >> i, r = rows >> i;
      depth[i].create(c, r);
      image[i].create(c, r);
      vmap[i].create(c, r);
      nmap[i].create(c, r);
      dIdx[i].create(c, r);
      dIdy[i].create(c, r);
    }
  }
};

// Frame::GpuRotation / GpuInvRotation / GpuTranslation (Core/Frame.cc:626-645)
Matrix3f rot(const double *P) {
  Matrix3f M;
  M.rowx = make_float3((float)P[0], (float)P[1], (float)P[2]);
  M.rowy = make_float3((float)P[4], (float)P[5], (float)P[6]);
  M.rowz = make_float3((float)P[8], (float)P[9], (float)P[10]);
  return M;
}
Matrix3f rot_inv(const double *P) {
  Matrix3f M;
  M.rowx = make_float3((float)P[0], (float)P[4], (float)P[8]);
  M.rowy = make_float3((float)P[1], (float)P[5], (float)P[9]);
  M.rowz = make_float3((float)P[2], (float)P[6], (float)P[10]);
  return M;
}
float3 trans(const double *P) { return make_float3((float)P[3], (float)P[7], (float)P[11]); }

struct RefSystem {
  int cols, rows;
  float fx, fy, cx, cy, depth_scale, cutoff;
  RefFrame fr[2];
  RefFrame *next = &fr[0], *last = &fr[1];
  bool have_last = false;
  int state = 1;
  double init_pose[16];
  // Mapping::Create (Mapping/Mapping.cc:11-51), the loop's arrays
  DeviceArray<int> heapCounter, hashCounter, heap, bucketMutex;
  DeviceArray<uint> noVisibleEntries, noRenderingBlocks;
  DeviceArray<Voxel> sdfBlock;
  DeviceArray<HashEntry> hashEntries, visibleEntries;
  DeviceArray2D<float> zRangeMin, zRangeMax;
  DeviceArray<RenderingBlock> renderingBlockList;
  DeviceArray2D<unsigned char> mask;
  DeviceArray<int> labels;
  // Tracker scratch (Tracking.cc:36-41)
  DeviceArray2D<float> sumSE3;
  DeviceArray<float> outSE3;
  DeviceArray2D<int> sumRes;
  DeviceArray<int> outRes;
  int rgb = 0;

  DeviceMap dmap() const {  // Mapping::operator DeviceMap (Mapping.cc:363-377)
    DeviceMap m;
    m.heapMem = heap;
    m.heapCounter = heapCounter;
    m.noVisibleBlocks = noVisibleEntries;
    m.bucketMutex = bucketMutex;
    m.hashEntries = hashEntries;
    m.visibleEntries = visibleEntries;
    m.voxelBlocks = sdfBlock;
    m.entryPtr = hashCounter;
    return m;
  }

  Intrinsics K(int level) const { return Intrinsics(fx, fy, cx, cy)(level); }

  // CreateMatrix<6,7>'s 27 sums (Reduction.cu:6-16) back from A, b, and
  // the residual pair
  static void to_sums(const double *A, const double *b, const float *residual, double *sums) {
    int k = 0;
    for (int r = 0; r < 6; ++r)
      for (int q = r; q < 7; ++q) sums[k++] = q == 6 ? b[r] : A[r * 6 + q];
    sums[27] = residual[0];
    sums[28] = residual[1];
  }

  // Tracker::ComputeSE3(icpOnly = !rgb) with the FP64 solve of sf_solve.h
  bool compute_se3() {
    sf::TrackCtl c;
    sf::ctl_begin(c, last->pose);
    float residual[2], rres[2];
    double A[36], b[6], sums[29], rsums[29];
    for (int i = kLevels - 1; i >= 0; --i) {
      for (int j = 0; j < kIters[i]; ++j) {
#ifndef REF_SHIM_CUDA_RUNTIME_H_
        if (rgb) {
          RGBStep(next->image[i], last->image[i], next->vmap[i], last->vmap[i], next->dIdx[i], next->dIdy[i],
                  rot(c.next_pose), rot_inv(c.next_pose), rot(last->pose), rot_inv(last->pose),
                  trans(c.next_pose), trans(last->pose), K(i), sumSE3, outSE3, sumRes, outRes, rres, A, b);
          to_sums(A, b, rres, rsums);
        }
#endif
#ifdef REF_SHIM_CUDA_RUNTIME_H_
        {
          const Matrix3f Rc = rot(c.next_pose), Rl = rot(last->pose), RlI = rot_inv(last->pose);
          const float3 tc = trans(c.next_pose), tl = trans(last->pose);
          const Intrinsics Ki = K(i);
          ref_icp_sums_impl((const float *)next->vmap[i].data, (const float *)last->vmap[i].data,
                            (const float *)next->nmap[i].data, (const float *)last->nmap[i].data,
                            next->vmap[i].cols, next->vmap[i].rows, (const float *)&Rc, (const float *)&tc,
                            (const float *)&Rl, (const float *)&RlI, (const float *)&tl, Ki.fx, Ki.fy, Ki.cx,
                            Ki.cy, sums);
          (void)residual; (void)A; (void)b;
        }
#else
        ICPStep(next->vmap[i], last->vmap[i], next->nmap[i], last->nmap[i], rot(c.next_pose),
                trans(c.next_pose), rot(last->pose), rot_inv(last->pose), trans(last->pose), K(i), sumSE3,
                outSE3, residual, A, b);
        to_sums(A, b, residual, sums);
#endif
        if (!sf::ctl_step(c, sums, kMinCount[i], rgb ? rsums : nullptr)) break;
      }
      if (c.stop) break;
    }
    sf::ctl_finish(c, kThreshICP);
    std::memcpy(next->pose, c.next_pose, sizeof(next->pose));
    return c.accepted != 0;
  }
};

}  // namespace

inline void *refloop_create(int cols, int rows, const float *K, float depth_scale, float cutoff,
                               const double *init_pose) {
  RefSystem *s = new (std::nothrow) RefSystem();
  if (!s) return nullptr;
  s->cols = cols; s->rows = rows;
  s->fx = K[0]; s->fy = K[1]; s->cx = K[2]; s->cy = K[3];
  s->depth_scale = depth_scale; s->cutoff = cutoff;
  std::memcpy(s->init_pose, init_pose, sizeof(s->init_pose));
  s->fr[0].create(cols, rows);
  s->fr[1].create(cols, rows);
  s->heapCounter.create(1);
  s->hashCounter.create(1);
  s->noVisibleEntries.create(1);
  s->heap.create(DeviceMap::NumSdfBlocks);
  s->sdfBlock.create(DeviceMap::NumVoxels);
  s->bucketMutex.create(DeviceMap::NumBuckets);
  s->hashEntries.create(DeviceMap::NumEntries);
  s->visibleEntries.create(DeviceMap::NumEntries);
  s->zRangeMin.create(80, 60);
  s->zRangeMax.create(80, 60);
  s->noRenderingBlocks.create(1);
  s->renderingBlockList.create(DeviceMap::MaxRenderingBlocks);
  s->mask.create(cols, rows);
  s->labels.create(1);
  s->sumSE3.create(29, 96);
  s->outSE3.create(29);
  s->sumRes.create(2, 96);
  s->outRes.create(2);
  ResetMap(s->dmap());  // Mapping::Reset
  return s;
}

// One frame of System::GrabImage; returns 1 when the frame was tracked.
inline int refloop_grab(void *h, const uint16_t *depth, const uint8_t *rgb, double *pose_out) {
  RefSystem &s = *static_cast<RefSystem *>(h);
  // Tracker::GrabFrame
  if (s.have_last)
    for (int i = 1; i < kLevels; ++i)
      ResizeMap(s.last->vmap[i - 1], s.last->nmap[i - 1], s.last->vmap[i], s.last->nmap[i]);
  RefFrame &f = *s.next;
  f.temp.upload(depth, sizeof(uint16_t) * s.cols);
  f.color.upload(rgb, 3 * s.cols);
  FilterDepth(f.temp, f.range, f.depth[0], s.depth_scale, s.cutoff);
  ImageToIntensity(f.color, f.image[0]);
  for (int i = 1; i < kLevels; ++i) {
    PyrDownGauss(f.depth[i - 1], f.depth[i]);
    PyrDownGauss(f.image[i - 1], f.image[i]);
  }
  for (int i = 0; i < kLevels; ++i) {
    const Intrinsics K = s.K(i);
    ComputeVMap(f.depth[i], f.vmap[i], K.fx, K.fy, K.cx, K.cy, s.cutoff);
    ComputeNMap(f.vmap[i], f.nmap[i]);
    ComputeDerivativeImage(f.image[i], f.dIdx[i], f.dIdy[i]);
  }
  // Tracker::Track
  int tracked = 0;
  if (s.state == 1) {
    std::memcpy(f.pose, s.init_pose, sizeof(f.pose));
    s.state = 0;
    tracked = 1;
  } else {
    std::memcpy(f.pose, s.last->pose, sizeof(f.pose));
    tracked = s.compute_se3() ? 1 : 0;
  }
  if (tracked) {
    std::swap(s.next, s.last);
    s.have_last = true;
  }
  // Mapping::FuseColor + Mapping::RayTrace on the last frame
  RefFrame &l = *s.last;
  uint no = 0;
  const Intrinsics K = s.K(0);
  FuseMapColor(l.range, l.color, l.nmap[0], s.mask, s.labels, 0, s.noVisibleEntries, rot(l.pose), rot_inv(l.pose),
               trans(l.pose), s.dmap(), K.fx, K.fy, K.cx, K.cy, DeviceMap::DepthMax, DeviceMap::DepthMin, &no);
  if (CreateRenderingBlocks(s.visibleEntries, s.zRangeMin, s.zRangeMax, DeviceMap::DepthMax, DeviceMap::DepthMin,
                            s.renderingBlockList, s.noRenderingBlocks, rot_inv(l.pose), trans(l.pose), no, K.fx,
                            K.fy, K.cx, K.cy))
    Raycast(s.dmap(), l.vmap[0], l.nmap[0], s.zRangeMin, s.zRangeMax, rot(l.pose), rot_inv(l.pose), trans(l.pose),
            1.0 / K.fx, 1.0 / K.fy, K.cx, K.cy);
  if (pose_out) std::memcpy(pose_out, l.pose, sizeof(l.pose));
  return tracked;
}

inline void refloop_destroy(void *h) { delete static_cast<RefSystem *>(h); }

// The map's arrays (device pointers in the CUDA build): hashEntries,
// sdfBlock (voxels), visibleEntries, noVisibleEntries, heapCounter,
// hashCounter (entryPtr); and the sizes NumEntries, NumSdfBlocks.
inline void refloop_map_arrays(void *h, void **out6, long long *sizes2) {
  RefSystem &s = *static_cast<RefSystem *>(h);
  out6[0] = s.hashEntries.data;
  out6[1] = s.sdfBlock.data;
  out6[2] = s.visibleEntries.data;
  out6[3] = s.noVisibleEntries.data;
  out6[4] = s.heapCounter.data;
  out6[5] = s.hashCounter.data;
  sizes2[0] = DeviceMap::NumEntries;
  sizes2[1] = DeviceMap::NumSdfBlocks;
}

inline void refloop_set_rgb(void *h, int on) { static_cast<RefSystem *>(h)->rgb = on != 0; }

#endif  // REF_LOOP_H_
