// Tracker::ValidatePose (Tracking/Tracking.cc:750-790) for n candidate poses
// against one frame, batched on the GPU.
//
// For each candidate the reference runs, one after another:
// UpdateVisibility at the candidate pose (the visible-block count `no`),
// and when no >= 512, RayTrace into LastFrame's level-0 maps,
// LastFrame->ResizeImages, and ComputeSE3(icpOnly = true, ITERATIONS_RELOC
// {3, 3, 2}, THRESH_ICP_RELOC 1e-3) from the candidate, recording
// lastIcpError and the candidate pose of every accepted candidate.
//
// Here every stage runs for all candidates at once: one visibility and
// z-range launch, one raycast launch (each candidate draws into its own
// slice of a stacked model map), one resize launch per level, and two
// launches per ComputeSE3 iteration.  Only the candidates the reference
// would evaluate take part in each stage.  A candidate whose RayTrace draws
// nothing (CreateRenderingBlocks found no rendering block) tracks, as in
// the reference, against whatever LastFrame held: the maps of the closest
// earlier candidate that drew, else the caller's last maps.
//
// The candidate ValidatePose keeps is the first accepted one in candidate
// order: the reference sorts the N x 1 matrix of ICP errors with
// cv::sortIdx(..., CV_SORT_DESCENDING), which sorts each ROW (one element),
// so index 0 always names the first accepted candidate (Tracking.cc:774-778).
#include <cstring>
#include <new>
#include <vector>

#include "sf_kernels.cuh"

namespace sf {
cudaStream_t ctx_stream(sf_context *c);
DevMap &map_dev(sf_map *m);
FuseScratch &map_scratch(sf_map *m);
int map_ensure_scratch(sf_map *m, int pixels);
const sf_map_config &map_cfg(sf_map *m);

struct VpWorkspace {
  int n_cap = 0, cols = 0, rows = 0, levels = 0, zc = 0, zr = 0;
  Cam *cams = nullptr;       // [n]
  TrackCtl *ctl = nullptr;   // [n]
  unsigned *vis = nullptr;   // [2n]: visible counts, then rendered flags
  int *src = nullptr;        // [n] model-map source (c, an earlier candidate, -1 the caller's maps, -2 skipped)
  int *box = nullptr;        // [8] bounding box of the allocated blocks
  float4 *mv[kMaxLevels] = {}, *mn[kMaxLevels] = {};  // stacked model maps per level
  float *zmin = nullptr, *zmax = nullptr;             // stacked z-range images
  double *part = nullptr;    // [n][29][stride] ICP partials
  int stride = 0;
  TrackCtl *h_ctl = nullptr;  // pinned [n]
  unsigned *h_vis = nullptr;  // pinned [2n]
};

void vp_workspace_free(VpWorkspace *w) {
  if (!w) return;
  cudaFree(w->cams); cudaFree(w->ctl); cudaFree(w->vis); cudaFree(w->src); cudaFree(w->box);
  for (int l = 0; l < kMaxLevels; ++l) { cudaFree(w->mv[l]); cudaFree(w->mn[l]); }
  cudaFree(w->zmin); cudaFree(w->zmax); cudaFree(w->part);
  if (w->h_ctl) cudaFreeHost(w->h_ctl);
  if (w->h_vis) cudaFreeHost(w->h_vis);
  delete w;
}

namespace {

int vp_workspace_ensure(VpWorkspace *&w, int n, int cols, int rows, int levels, int zc, int zr) {
  if (w && n <= w->n_cap && w->cols == cols && w->rows == rows && w->levels >= levels && w->zc == zc &&
      w->zr == zr)
    return SF_OK;
  vp_workspace_free(w);
  w = new (std::nothrow) VpWorkspace();
  if (!w) return SF_ERR_INVALID;
  w->n_cap = n; w->cols = cols; w->rows = rows; w->levels = levels; w->zc = zc; w->zr = zr;
  w->stride = vp_icp_blocks(cols * rows);
  auto A = [](void **p, size_t b) { return cudaMalloc(p, b) == cudaSuccess; };
  bool ok = A((void **)&w->cams, sizeof(Cam) * n) && A((void **)&w->ctl, sizeof(TrackCtl) * n) &&
            A((void **)&w->vis, sizeof(unsigned) * 2 * n) && A((void **)&w->src, sizeof(int) * n) &&
            A((void **)&w->box, sizeof(int) * 8) &&
            A((void **)&w->zmin, sizeof(float) * (size_t)n * zc * zr) &&
            A((void **)&w->zmax, sizeof(float) * (size_t)n * zc * zr) &&
            A((void **)&w->part, sizeof(double) * (size_t)n * 29 * w->stride);
  for (int l = 0; ok && l < levels; ++l) {
    const size_t px = (size_t)(cols >> l) * (rows >> l) * n;
    ok = A((void **)&w->mv[l], sizeof(float4) * px) && A((void **)&w->mn[l], sizeof(float4) * px);
  }
  ok = ok && cudaMallocHost(&w->h_ctl, sizeof(TrackCtl) * n) == cudaSuccess &&
       cudaMallocHost(&w->h_vis, sizeof(unsigned) * 2 * n) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    vp_workspace_free(w);
    w = nullptr;
    return SF_ERR_CUDA;
  }
  return SF_OK;
}

inline sf_image tall(void *p, int cols, int rows, size_t elem) {
  sf_image i;
  i.data = p;
  i.step = (size_t)cols * elem;
  i.cols = cols;
  i.rows = rows;
  return i;
}

inline f3 h3(float x, float y, float z) {
  f3 v;
  v.x = x; v.y = y; v.z = z;
  return v;
}

inline bool img16(const sf_image &im, int cols, int rows) {
  return im.data && im.cols == cols && im.rows == rows && im.step >= (size_t)cols * 16;
}

}  // namespace

VpWorkspace *&ctx_vp(sf_context *c);

}  // namespace sf

using namespace sf;

extern "C" int sf_ValidatePoseBatch(sf_context *ctx, sf_map *m, int levels, const sf_image *next_vmaps,
                                    const sf_image *next_nmaps, const sf_image *last_vmaps,
                                    const sf_image *last_nmaps, sf_intrinsics K, const double *poses, int n,
                                    const int *iters, const int *min_count, float thresh, uint32_t min_visible,
                                    sf_reloc_candidate *out, int *chosen) {
  if (!ctx || !m || levels < 1 || levels > kMaxLevels || !next_vmaps || !next_nmaps || !last_vmaps ||
      !last_nmaps || !poses || n < 1 || n > 65535 || !iters || !min_count || !out || K.fx <= 0 || K.fy <= 0)
    return SF_ERR_INVALID;
  const int cols = next_vmaps[0].cols, rows = next_vmaps[0].rows;
  if (cols < 1 || rows < 1 || (cols >> (levels - 1)) < 1 || (rows >> (levels - 1)) < 1) return SF_ERR_INVALID;
  for (int l = 0; l < levels; ++l) {
    const int c = cols >> l, r = rows >> l;
    if (!img16(next_vmaps[l], c, r) || !img16(next_nmaps[l], c, r) || !img16(last_vmaps[l], c, r) ||
        !img16(last_nmaps[l], c, r) || iters[l] < 0)
      return SF_ERR_INVALID;
  }
  cudaStream_t st = ctx_stream(ctx);
  const sf_map_config &mc = map_cfg(m);
  const int zc = (cols + 7) / 8, zr = (rows + 7) / 8;
  VpWorkspace *&w = ctx_vp(ctx);
  if (cudaStreamSynchronize(st) != cudaSuccess) return SF_ERR_CUDA;
  int e = vp_workspace_ensure(w, n, cols, rows, levels, zc, zr);
  if (e != SF_OK) return e;
  if ((e = map_ensure_scratch(m, cols * rows)) != SF_OK) return e;
  DevMap &dm = map_dev(m);
  FuseScratch &fs = map_scratch(m);
  // cameras (Frame::GpuRotation / GpuInvRotation / GpuTranslation,
  // Frame.cc:626-645) and ComputeSE3's starting state per candidate:
  // LastFrame->pose = NextFrame->pose = the candidate (Tracking.cc:757,763)
  std::vector<Cam> cams((size_t)n);
  for (int k = 0; k < n; ++k) {
    const double *P = poses + 16 * (size_t)k;
    Cam &c = cams[k];
    memset(&c, 0, sizeof(c));
    c.R.rx = h3((float)P[0], (float)P[1], (float)P[2]);
    c.R.ry = h3((float)P[4], (float)P[5], (float)P[6]);
    c.R.rz = h3((float)P[8], (float)P[9], (float)P[10]);
    c.Rinv.rx = h3((float)P[0], (float)P[4], (float)P[8]);
    c.Rinv.ry = h3((float)P[1], (float)P[5], (float)P[9]);
    c.Rinv.rz = h3((float)P[2], (float)P[6], (float)P[10]);
    c.t = h3((float)P[3], (float)P[7], (float)P[11]);
    c.fx = K.fx; c.fy = K.fy; c.cx = K.cx; c.cy = K.cy;
    c.invfx = (float)(1.0 / (double)K.fx);
    c.invfy = (float)(1.0 / (double)K.fy);
    c.cols = cols; c.rows = rows;
    c.dmin = mc.depth_min; c.dmax = mc.depth_max;
    ctl_begin(w->h_ctl[k], P);
  }
  if (cudaMemcpyAsync(w->cams, cams.data(), sizeof(Cam) * n, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(w->ctl, w->h_ctl, sizeof(TrackCtl) * n, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemsetAsync(w->vis, 0, sizeof(unsigned) * 2 * n, st) != cudaSuccess)
    return SF_ERR_CUDA;
  // UpdateVisibility and the z-range of CreateRenderingBlocks
  const sf_image zmin = tall(w->zmin, zc, zr * n, 4), zmax = tall(w->zmax, zc, zr * n, 4);
  launch_zrange_init(zmin, zmax, st);
  launch_vp_visibility(dm, w->cams, n, zmin, zmax, zr, w->vis, w->vis + n, st);
  if (cudaMemcpyAsync(w->h_vis, w->vis, sizeof(unsigned) * 2 * n, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return SF_ERR_CUDA;
  // which maps each candidate tracks against (see the file comment)
  std::vector<int> src((size_t)n);
  int last_drawn = -1;
  for (int k = 0; k < n; ++k) {
    if (w->h_vis[k] < min_visible) {
      src[k] = -2;
    } else if (w->h_vis[n + k]) {
      src[k] = k;
      last_drawn = k;
    } else {
      src[k] = last_drawn;
    }
  }
  if (cudaMemcpyAsync(w->src, src.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st) != cudaSuccess)
    return SF_ERR_CUDA;
  // RayTrace of every drawing candidate through one block window over the
  // whole map, then ResizeImages
  launch_window_alloc_box(dm, fs, w->box, st);
  launch_raycast_batch(dm, fs, tall(w->mv[0], cols, rows * n, 16), tall(w->mn[0], cols, rows * n, 16), rows, zmin,
                       zmax, zr, w->cams, n, w->src, st);
  for (int l = 1; l < levels; ++l) {
    const int cs = cols >> (l - 1), rs = rows >> (l - 1), cd = cols >> l, rd = rows >> l;
    launch_resize_batch(tall(w->mv[l - 1], cs, rs * n, 16), tall(w->mn[l - 1], cs, rs * n, 16),
                        tall(w->mv[l], cd, rd * n, 16), tall(w->mn[l], cd, rd * n, 16), rs, rd, n, w->src, st);
  }
  // ComputeSE3(icpOnly = true, iters, thresh): coarse to fine
  for (int l = levels - 1; l >= 0; --l) {
    const int c = cols >> l, r = rows >> l;
    VpLevel V;
    V.vc = next_vmaps[l]; V.nc = next_nmaps[l];
    V.mv = tall(w->mv[l], c, r * n, 16); V.mn = tall(w->mn[l], c, r * n, 16);
    V.fv = last_vmaps[l]; V.fn = last_nmaps[l];
    V.rows = r;
    const float div = (float)(1 << l);
    V.fx = K.fx / div; V.fy = K.fy / div; V.cx = K.cx / div; V.cy = K.cy / div;
    V.min_count = min_count[l];
    const int nb = vp_icp_blocks(c * r);
    for (int j = 0; j < iters[l]; ++j) launch_vp_icp_iteration(V, w->src, w->ctl, w->part, nb, w->stride, n, st);
  }
  launch_vp_icp_finish(w->ctl, w->src, thresh, n, st);
  if (cudaGetLastError() != cudaSuccess) return SF_ERR_CUDA;
  if (cudaMemcpyAsync(w->h_ctl, w->ctl, sizeof(TrackCtl) * n, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return SF_ERR_CUDA;
  int pick = -1;
  for (int k = 0; k < n; ++k) {
    const TrackCtl &c = w->h_ctl[k];
    sf_reloc_candidate &o = out[k];
    memset(&o, 0, sizeof(o));
    o.visible = w->h_vis[k];
    o.rendered = src[k] == k;
    o.evaluated = src[k] != -2;
    if (o.evaluated) {
      o.accepted = c.accepted;
      o.fail = c.stop;
      o.iterations = c.iters_run;
      o.icp_error = c.icpError;
      o.icp_count = c.icpCount;
      for (int q = 0; q < 16; ++q) o.pose[q] = c.next_pose[q];
      if (o.accepted && pick < 0) pick = k;
    } else {
      for (int q = 0; q < 16; ++q) o.pose[q] = poses[16 * (size_t)k + q];
    }
  }
  if (chosen) *chosen = pick;
  return SF_OK;
}
