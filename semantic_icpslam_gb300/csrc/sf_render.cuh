// Projection of a voxel block into the subsampled z-range image and the
// z-range tiles it lays down (Mapping/RenderScene.cu:54-190).
#ifndef SF_RENDER_CUH_
#define SF_RENDER_CUH_

#include "sf_kernels.cuh"

namespace sf {

// ------------------------------------------------- block-pointer window
// Bounding box, in block coordinates, of the camera frustum between depth
// dmin and dmax (+ margins for the raycast's interpolation and normal
// offsets).  Float arithmetic is fine here: the window only accelerates
// lookups; any block outside it is found through the hash table.
__device__ __forceinline__ void window_setup(const Cam &c, float bw, float dmin, float dmax,
                                             uint32_t cap, int *win) {
  float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
  const float us[2] = {0.f, (float)c.cols}, vs[2] = {0.f, (float)c.rows};
  const float zs[2] = {dmin, dmax + 2.0f * bw};
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b)
      for (int k = 0; k < 2; ++k) {
        f3 pc = mk3((us[a] - c.cx) / c.fx * zs[k], (vs[b] - c.cy) / c.fy * zs[k], zs[k]);
        f3 pw = mul(c.R, pc) + c.t;
        const float p[3] = {pw.x, pw.y, pw.z};
        for (int d = 0; d < 3; ++d) { lo[d] = fminf(lo[d], p[d]); hi[d] = fmaxf(hi[d], p[d]); }
      }
  int o[3], n[3];
  long long total = 1;
  for (int d = 0; d < 3; ++d) {
    if (!(lo[d] > -1.0e7f && hi[d] < 1.0e7f)) { win[3] = win[4] = win[5] = 0; return; }
    int a = (int)floorf(lo[d] / bw) - 1, b = (int)floorf(hi[d] / bw) + 1;
    o[d] = a;
    n[d] = b - a + 1;
    total *= n[d];
  }
  if (total > (long long)cap) { win[3] = win[4] = win[5] = 0; return; }
  win[0] = o[0]; win[1] = o[1]; win[2] = o[2];
  win[3] = n[0]; win[4] = n[1]; win[5] = n[2];
}

// Cell of block bp in the window, or -1 when outside.
__device__ __forceinline__ int window_cell(const int *win, i3 bp) {
  const unsigned x = (unsigned)(bp.x - win[0]), y = (unsigned)(bp.y - win[1]), z = (unsigned)(bp.z - win[2]);
  if (x >= (unsigned)win[3] || y >= (unsigned)win[4] || z >= (unsigned)win[5]) return -1;
  return (int)((z * (unsigned)win[4] + y) * (unsigned)win[3] + x);
}

// Projection::projectBlock (RenderScene.cu:54-112).
__device__ __forceinline__ bool project_block(i3 pos, float voxel, const m3 &Rinv, f3 t, float fx, float fy,
                              float cx, float cy, int zc, int zr, float dmax, float dmin,
                              sf_rendering_block &b) {
  b.ulx = (int16_t)zc; b.uly = (int16_t)zr; b.lrx = -1; b.lry = -1;
  b.zmin = dmax; b.zmax = dmin;
  for (int corner = 0; corner < 8; ++corner) {
    int tx = pos.x + ((corner & 1) ? 1 : 0);
    int ty = pos.y + ((corner & 2) ? 1 : 0);
    int tz = pos.z + ((corner & 4) ? 1 : 0);
    f3 p3 = mk3((float)(int)((unsigned)tx * 8u) * voxel, (float)(int)((unsigned)ty * 8u) * voxel,
                (float)(int)((unsigned)tz * 8u) * voxel);
    p3 = mul(Rinv, p3 - t);
    if (p3.z < 0.2f) continue;  // (double)z < 2e-1: no float lies in [0.2, 0.2f)
    float px = (fx * p3.x / p3.z + cx) / 8.0f;
    float py = (fy * p3.y / p3.z + cy) / 8.0f;
    if ((float)b.ulx > floorf(px)) b.ulx = (int16_t)(int)floorf(px);
    if ((float)b.lrx < ceilf(px)) b.lrx = (int16_t)(int)ceilf(px);
    if ((float)b.uly > floorf(py)) b.uly = (int16_t)(int)floorf(py);
    if ((float)b.lry < ceilf(py)) b.lry = (int16_t)(int)ceilf(py);
    if (b.zmin > p3.z) b.zmin = p3.z;
    if (b.zmax < p3.z) b.zmax = p3.z;
  }
  if (b.ulx < 0) b.ulx = 0;
  if (b.uly < 0) b.uly = 0;
  if (b.lrx >= zc) b.lrx = (int16_t)(zc - 1);
  if (b.lry >= zr) b.lry = (int16_t)(zr - 1);
  if (b.ulx > b.lrx) return false;
  if (b.uly > b.lry) return false;
  if (b.zmin < dmin) b.zmin = dmin;
  if (b.zmax < dmin) return false;
  return true;
}

// Tiles of createRenderingBlockList (RenderScene.cu:114-132: x < ny bound
// and un-offset lowerRight kept) filled as fillBlocks does (:167-190).
// nx, ny from RenderScene.cu:147-151.
__device__ __forceinline__ void fill_block_tiles(const sf_rendering_block &b, const sf_image &zmin,
                                 const sf_image &zmax) {
  float dy = (float)b.lry - (float)b.uly + 1.0f;
  int ny = (int)ceilf(dy / 16.0f);
  const int zc = zmin.cols, zr = zmin.rows;
  for (int ty_ = 0; ty_ < ny; ++ty_)
    for (int tx_ = 0; tx_ < ny; ++tx_) {
      int ulx = (int16_t)(b.ulx + tx_ * 16), uly = (int16_t)(b.uly + ty_ * 16);
      int lrx = (int16_t)(b.ulx + 16), lry = (int16_t)(b.uly + 16);
      if (lrx > b.lrx) lrx = b.lrx;
      if (lry > b.lry) lry = b.lry;
      int xe = min(min(ulx + 15, lrx), zc - 1);
      int ye = min(min(uly + 15, lry), zr - 1);
      for (int yy = uly; yy <= ye; ++yy)
        for (int xx = ulx; xx <= xe; ++xx) {
          atomicMin(row_ptr<int>(zmin, yy) + xx, __float_as_int(b.zmin));
          atomicMax(row_ptr<int>(zmax, yy) + xx, __float_as_int(b.zmax));
        }
    }
}

}  // namespace sf
#endif
