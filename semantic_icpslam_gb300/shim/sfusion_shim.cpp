// The reference-side binding of the C ABI: the host launchers that
// Tracking/Reduction.h and Mapping/RenderScene.h declare, forwarding to
// include/sfusion.h.  A maintainer compiles this file inside
// YuhangMing/semantic_icpSLAM, next to Mapping/ and Tracking/, in place of
// the host launchers of Tracking/Pyrdown.cu, Tracking/Reduction.cu,
// Mapping/FuseMap.cu and Mapping/RenderScene.cu (whose kernels are then no
// longer compiled), and links libsfusion.so.  Frame, Tracker and Mapping
// compile unchanged against the same declarations.  Each function converts
// the reference's containers (DeviceArray2D's pitched rows, DeviceMap's
// PtrSz views, Matrix3f rows) into sf_image / sf_device_map views and maps
// a non-zero status to the reference's own error behaviour: print, then
// exit(0), as SafeCall does (Utility/SafeCall.h:13-16).
#include "Reduction.h"
#include "RenderScene.h"
#include "sfusion.h"
#include <cstdio>
#include <cstdlib>

namespace {
template <class T> sf_image view(const DeviceArray2D<T> &a) {
  return sf_image{a.data, a.step, a.cols, a.rows};
}
sf_mat3 m3(const Matrix3f &m) {
  return sf_mat3{{m.rowx.x, m.rowx.y, m.rowx.z}, {m.rowy.x, m.rowy.y, m.rowy.z}, {m.rowz.x, m.rowz.y, m.rowz.z}};
}
sf_float3 f3(const float3 &v) { return sf_float3{v.x, v.y, v.z}; }
void check(int st, const char *fn) {           // SafeCall's behaviour (Utility/SafeCall.h:13-16)
  if (st != SF_OK) { std::printf("%s failed with status %d\n", fn, st); std::exit(0); }
}
sf_context *ctx() {                            // one context per host thread
  thread_local sf_context *c = nullptr;
  if (!c) check(sf_context_create(&c), "sf_context_create");
  return c;
}
thread_local sf_map *g_last_map = nullptr;     // the map wrap() last returned
sf_map *wrap(DeviceMap &m) {                   // the Mapping's own arrays, sizes from DeviceMap.h:166-189
  thread_local sf_map *w = nullptr;
  thread_local void *key = nullptr;
  if (w && key == m.hashEntries.data) return g_last_map = w;
  if (w) sf_map_destroy(w);
  sf_map_config c{DeviceMap::VoxelSize, DeviceMap::TruncateDist, DeviceMap::DepthMin, DeviceMap::DepthMax,
                  DeviceMap::NumBuckets, DeviceMap::NumExcess, DeviceMap::NumSdfBlocks,
                  DeviceMap::MaxRenderingBlocks};
  sf_device_map a{m.heapMem.data, m.entryPtr.data, m.heapCounter.data, m.bucketMutex.data,
                  (sf_voxel *)m.voxelBlocks.data, m.noVisibleBlocks.data,
                  (sf_hash_entry *)m.hashEntries.data, (sf_hash_entry *)m.visibleEntries.data};
  check(sf_map_wrap(&c, &a, &w), "sf_map_wrap");
  check(sf_map_rebuild_index(ctx(), w), "sf_map_rebuild_index");
  key = m.hashEntries.data;
  return g_last_map = w;
}
}  // namespace

void FilterDepth(const DeviceArray2D<unsigned short> &depth, DeviceArray2D<float> &rawDepth,
                 DeviceArray2D<float> &filteredDepth, float depthScale, float depthCutoff) {
  check(sf_FilterDepth(ctx(), view(depth), view(rawDepth), view(filteredDepth), depthScale, depthCutoff),
        "FilterDepth");
}
void ComputeVMap(const DeviceArray2D<float> &depth, DeviceArray2D<float4> &vmap, float fx, float fy, float cx,
                 float cy, float depthCutoff) {
  check(sf_ComputeVMap(ctx(), view(depth), view(vmap), fx, fy, cx, cy, depthCutoff), "ComputeVMap");
}
void ComputeNMap(const DeviceArray2D<float4> &vmap, DeviceArray2D<float4> &nmap) {
  check(sf_ComputeNMap(ctx(), view(vmap), view(nmap)), "ComputeNMap");
}
void PyrDownGauss(const DeviceArray2D<float> &src, DeviceArray2D<float> &dst) {
  check(sf_PyrDownGauss(ctx(), view(src), view(dst)), "PyrDownGauss");
}
void PyrDownGauss(const DeviceArray2D<unsigned char> &src, DeviceArray2D<unsigned char> &dst) {
  check(sf_PyrDownGauss_u8(ctx(), view(src), view(dst)), "PyrDownGauss");
}
void ImageToIntensity(const DeviceArray2D<uchar3> &rgb, DeviceArray2D<unsigned char> &image) {
  check(sf_ImageToIntensity(ctx(), view(rgb), view(image)), "ImageToIntensity");
}
void ComputeDerivativeImage(DeviceArray2D<unsigned char> &image, DeviceArray2D<short> &dx, DeviceArray2D<short> &dy) {
  check(sf_ComputeDerivativeImage(ctx(), view(image), view(dx), view(dy)), "ComputeDerivativeImage");
}
void RGBStep(const DeviceArray2D<unsigned char> &nextImage, const DeviceArray2D<unsigned char> &lastImage,
             const DeviceArray2D<float4> &nextVMap, const DeviceArray2D<float4> &lastVMap,
             const DeviceArray2D<short> &dIdx, const DeviceArray2D<short> &dIdy, Matrix3f Rcurr, Matrix3f RcurrInv,
             Matrix3f Rlast, Matrix3f RlastInv, float3 tcurr, float3 tlast, Intrinsics K, DeviceArray2D<float> &,
             DeviceArray<float> &, DeviceArray2D<int> &, DeviceArray<int> &, float *residual, double *matrixA_host,
             double *vectorB_host) {
  // the reduction scratch arguments are not needed; nor is the reference's per-call Residual array
  check(sf_RGBStep(ctx(), view(nextImage), view(lastImage), view(nextVMap), view(lastVMap), view(dIdx), view(dIdy),
                   m3(Rcurr), m3(RcurrInv), m3(Rlast), m3(RlastInv), f3(tcurr), f3(tlast),
                   sf_intrinsics{K.fx, K.fy, K.cx, K.cy}, residual, matrixA_host, vectorB_host), "RGBStep");
}
void ResizeMap(const DeviceArray2D<float4> &vsrc, const DeviceArray2D<float4> &nsrc, DeviceArray2D<float4> &vdst,
               DeviceArray2D<float4> &ndst) {
  check(sf_ResizeMap(ctx(), view(vsrc), view(nsrc), view(vdst), view(ndst)), "ResizeMap");
}
void ICPStep(DeviceArray2D<float4> &nextVMap, DeviceArray2D<float4> &lastVMap, DeviceArray2D<float4> &nextNMap,
             DeviceArray2D<float4> &lastNMap, Matrix3f Rcurr, float3 tcurr, Matrix3f Rlast, Matrix3f RlastInv,
             float3 tlast, Intrinsics K, DeviceArray2D<float> &, DeviceArray<float> &, float *residual,
             double *matrixA_host, double *vectorB_host) {
  // sum / out (the reference's reduction scratch) are not needed: the context holds its own
  check(sf_ICPStep(ctx(), view(nextVMap), view(lastVMap), view(nextNMap), view(lastNMap), m3(Rcurr), f3(tcurr),
                   m3(Rlast), m3(RlastInv), f3(tlast), sf_intrinsics{K.fx, K.fy, K.cx, K.cy}, residual,
                   matrixA_host, vectorB_host), "ICPStep");
}
void ResetMap(DeviceMap map) { check(sf_ResetMap(ctx(), wrap(map)), "ResetMap"); }
void CheckBlockVisibility(DeviceMap map, DeviceArray<uint> &, Matrix3f Rview, Matrix3f RviewInv, float3 tview,
                          int cols, int rows, float fx, float fy, float cx, float cy, float depthMax,
                          float depthMin, uint *host_data) {
  check(sf_CheckBlockVisibility(ctx(), wrap(map), m3(Rview), m3(RviewInv), f3(tview), cols, rows, fx, fy, cx, cy,
                                depthMax, depthMin, host_data), "CheckBlockVisibility");
}
void FuseMapColor(const DeviceArray2D<float> &depth, const DeviceArray2D<uchar3> &color,
                  const DeviceArray2D<float4> &nmap, const DeviceArray2D<unsigned char> &mask,
                  const DeviceArray<int> &, int numDetection, DeviceArray<uint> &, Matrix3f Rview,
                  Matrix3f RviewInv, float3 tview, DeviceMap map, float fx, float fy, float cx, float cy,
                  float depthMax, float depthMin, uint *host_data) {
  // `labels` is stored by the reference but read by no kernel (FuseMap.cu:1086)
  check(sf_FuseMapColor(ctx(), wrap(map), view(depth), view(color), view(nmap), view(mask), numDetection,
                        m3(Rview), m3(RviewInv), f3(tview), fx, fy, cx, cy, depthMax, depthMin, host_data),
        "FuseMapColor");
}
void AnalyzeMapSemantics(const DeviceArray2D<float> &depth, const DeviceArray2D<uchar3> &color,
                         const DeviceArray2D<float4> &nmap, const DeviceArray2D<unsigned char> &mask,
                         const DeviceArray<int> &, int numDetection, DeviceArray<uint> &, Matrix3f Rview,
                         Matrix3f RviewInv, float3 tview, DeviceMap map, float fx, float fy, float cx, float cy,
                         float depthMax, float depthMin) {
  check(sf_AnalyzeMapSemantics(ctx(), wrap(map), view(depth), view(color), view(nmap), view(mask), numDetection,
                               m3(Rview), m3(RviewInv), f3(tview), fx, fy, cx, cy, depthMax, depthMin),
        "AnalyzeMapSemantics");
}
bool CreateRenderingBlocks(const DeviceArray<HashEntry> &, DeviceArray2D<float> &zRangeX,
                           DeviceArray2D<float> &zRangeY, const float &depthMax, const float &depthMin,
                           DeviceArray<RenderingBlock> &list, DeviceArray<uint> &noRenderingBlocks,
                           Matrix3f RviewInv, float3 tview, uint noVisibleBlocks, float fx, float fy, float cx,
                           float cy) {
  int ok = 0;   // the visible list is the map's own: the map the last launcher wrapped
  check(sf_CreateRenderingBlocks(ctx(), g_last_map, view(zRangeX), view(zRangeY), depthMax, depthMin,
                                 (sf_rendering_block *)list.data, (uint32_t *)noRenderingBlocks.data, m3(RviewInv),
                                 f3(tview), noVisibleBlocks,
                                 fx, fy, cx, cy, &ok), "CreateRenderingBlocks");
  return ok != 0;
}
void Raycast(DeviceMap map, DeviceArray2D<float4> &vmap, DeviceArray2D<float4> &nmap,
             DeviceArray2D<float> &zRangeX, DeviceArray2D<float> &zRangeY, Matrix3f Rview, Matrix3f RviewInv,
             float3 tview, float invfx, float invfy, float cx, float cy) {
  check(sf_Raycast(ctx(), wrap(map), view(vmap), view(nmap), view(zRangeX), view(zRangeY), m3(Rview), m3(RviewInv),
                   f3(tview), invfx, invfy, cx, cy), "Raycast");
}
