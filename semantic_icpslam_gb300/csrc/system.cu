// The per-frame loop: System::GrabImage (Core/System.cc:131-270) with
// Tracker::GrabFrame / Track / TrackFrame / ComputeSE3(icpOnly)
// (Tracking/Tracking.cc:65-173, 246-280, 369-517), Mapping::FuseColor and
// Mapping::RayTrace (Mapping/Mapping.cc:76-161).
//
// Buffers: the current frame's measured pyramid (raw + filtered depth,
// vertex and normal maps per level) and the model maps (the last tracked
// frame's raycast at level 0, 2x2-downsampled below).  The reference keeps
// two Frame objects and swaps them after a tracked frame; here the model
// maps are written in place (raycast, or the measured level-0 maps when no
// block renders), which leaves the same data where ICP reads it.
//
// Three execution forms of the same kernels:
//  * plain   - host-driven: ICP downloads 29 sums per iteration and solves
//              on the host; the visible count is downloaded as the
//              reference does.  The "plain per-launch" comparison form.
//  * eager   - device-driven: one persistent ICP kernel, tracking decision
//              and camera on the device, no host synchronisation.
//  * graph   - the eager form captured once as a CUDA graph and replayed.
#include <cstddef>
#include <cstring>
#include <new>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "sf_frame.cuh"

namespace {
// NVTX range over a host scope (a profiler shows which stage issued which
// launches; without a tool attached the calls return at once).
struct Range {
  explicit Range(const char *name) { nvtxRangePushA(name); }
  ~Range() { nvtxRangePop(); }
};
}  // namespace

namespace sf {
cudaStream_t ctx_stream(sf_context *c);
IcpWorkspace &ctx_icp(sf_context *c);
uint32_t *ctx_flags(sf_context *c);
DevMap &map_dev(sf_map *m);
FuseScratch &map_scratch(sf_map *m);
int map_ensure_scratch(sf_map *m, int pixels);
const sf_map_config &map_cfg(sf_map *m);

namespace {

__global__ void k_sys_post(SysDev *s, const TrackCtl *ctl, Cam tmpl, FuseScratch f) { sys_post(s, *ctl, tmpl, f); }

__global__ void k_sys_stats(const SysDev *s, const TrackCtl *ctl, DevMap m, const uint32_t *flags,
                            sf_frame_stats *out, sf_frame_stats *host_out, uint32_t *host_ready,
                            uint32_t *seq) {
  sys_stats(s, *ctl, m, flags, out, host_out, host_ready, seq);
}

template <class T>
inline T *dev_field(SysDev *base, size_t off) {
  return (T *)((char *)base + off);
}

inline sf_image img(void *p, int cols, int rows, size_t elem) {
  sf_image i;
  i.data = p;
  i.step = (size_t)cols * elem;
  i.cols = cols;
  i.rows = rows;
  return i;
}

}  // namespace
}  // namespace sf

using namespace sf;

struct sf_system {
  sf_context *ctx = nullptr;
  sf_map *map = nullptr;
  sf_system_config cfg;
  int L = 3, zc = 0, zr = 0;
  // device buffers
  uint16_t *d_depth16 = nullptr;
  uint8_t *d_rgb = nullptr, *d_mask = nullptr;
  float *d_raw = nullptr;
  float *d_depth[kMaxLevels] = {};
  float4 *d_vmap[kMaxLevels] = {}, *d_nmap[kMaxLevels] = {};
  float4 *d_mv[kMaxLevels] = {}, *d_mn[kMaxLevels] = {};
  // photometric term: this frame's and the last frame's intensity pyramids,
  // this frame's derivative images and correspondence candidate flags
  uint8_t *d_int[kMaxLevels] = {}, *d_int_last[kMaxLevels] = {}, *d_cand[kMaxLevels] = {};
  int16_t *d_dx[kMaxLevels] = {}, *d_dy[kMaxLevels] = {};
  float4 *d_corr = nullptr;  // per-iteration correspondences (level-0 size)
  float *d_rdepth = nullptr;  // rendered depth (localisation mode's label pass)
  int mapping = 1;            // 0: localisation mode (Tracker::mappingDisabled)
  float *d_zmin = nullptr, *d_zmax = nullptr;
  SysDev *d_sys = nullptr;
  sf_frame_stats *d_stats = nullptr;
  // pinned host staging
  uint16_t *h_depth16 = nullptr;
  uint8_t *h_rgb = nullptr, *h_mask = nullptr;
  sf_frame_stats *h_stats = nullptr;
  // plain-form host state
  double last_pose[16];
  int state = 1;        // the next frame's state (Tracker::state), as SysDev::state
  int prev_state = 0;   // the state the last frame ran in
  int missed = 0;       // Tracker::noMissedFrames
  TrackCtl ctl;
  // relocalisation: the caller's candidate poses (n x 16, camera -> world),
  // tried by every frame that starts lost; the device forms' next state as
  // last read back (-2 = unknown)
  std::vector<double> reloc;
  int dev_state = -2;
  bool host_driven = false;  // this frame ran host-driven (its stats are copied, not flagged)
  Cam tmpl;
  // graph
  cudaGraphExec_t gexec = nullptr;
  int graph_sem = -1;  // semantics flag the graph was captured with
  int graph_mapping = -1;  // mapping flag the graph was captured with
  unsigned long long graph_kernels = 0;  // kernel launches recorded in the graph
  int num_detection_captured = 0;
  // stage timing (eager form only): events at the stage boundaries
  int timing = 0;
  cudaEvent_t ev[8] = {};
  // colour (and mask) uploads of sf_system_grab run on their own stream,
  // overlapping the pyramid and ICP; integration waits for ev_inputs
  cudaStream_t cstream = nullptr;
  cudaEvent_t ev_inputs = nullptr, ev_prev = nullptr;
  // the photometric term's intensity pyramid runs on its own stream beside
  // the depth pyramid (fork / join events)
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // A device-driven frame with mapping takes its stats before the final
  // RayTrace (which changes none of them); the graph form also writes them
  // to h_stats there and then sets *h_ready, so sf_system_grab returns
  // while the raycast and ResizeMap still run and the next frame's uploads
  // and launch overlap them.
  uint32_t *h_ready = nullptr;  // pinned; the sequence number of the last frame that wrote h_stats
  uint32_t *d_seq = nullptr;    // device: graph frames run so far (k_sys_stats counts them)
  uint32_t graph_seq = 0;       // host: graph frames launched so far
  bool capturing = false;    // enqueue_device_frame is being captured
  bool stats_taken = false;  // this frame's enqueue took the stats early
  bool graph_early = false;  // the frame graph writes h_stats and h_ready
  // launch shapes (sf_system_autotune / sf_system_set_tune): the raycast's
  // (an index into raycast_tune's candidates) and the integration's CTAs per SM
  RaycastTune rc_tune;
  int rc_index = 0;
  int int_ctas = 8;
  int alloc_tile = 0;           // the allocation walk's pixel tile (alloc_tile())
  long long frames = 0;  // frames run (any form)
};

namespace {

// Stage boundary marker: 0 start, 1 pyramid, 2 ICP, 3 allocation,
// 4 visibility + z-range, 5 integration, 6 raycast, 7 resize + stats.
void mark(sf_system *s, cudaStream_t st, int i) {
  if (s->timing && s->ev[i]) cudaEventRecord(s->ev[i], st);
}

int alloc_all(sf_system *s) {
  const int C = s->cfg.cols, R = s->cfg.rows;
  const size_t np = (size_t)C * R;
  auto A = [&](void **p, size_t bytes) { return cudaMalloc(p, bytes) == cudaSuccess; };
  bool ok = A((void **)&s->d_depth16, np * 2) && A((void **)&s->d_rgb, np * 3) &&
            A((void **)&s->d_mask, np) && A((void **)&s->d_raw, np * 4) && A((void **)&s->d_rdepth, np * 4) &&
            A((void **)&s->d_zmin, (size_t)s->zc * s->zr * 4) &&
            A((void **)&s->d_zmax, (size_t)s->zc * s->zr * 4) &&
            A((void **)&s->d_sys, sizeof(SysDev)) && A((void **)&s->d_stats, sizeof(sf_frame_stats)) &&
            A((void **)&s->d_seq, sizeof(uint32_t)) && cudaMemset(s->d_seq, 0, sizeof(uint32_t)) == cudaSuccess;
  for (int l = 0; ok && l < s->L; ++l) {
    const size_t n = (size_t)(C >> l) * (R >> l);
    ok = A((void **)&s->d_depth[l], n * 4) && A((void **)&s->d_vmap[l], n * 16) &&
         A((void **)&s->d_nmap[l], n * 16) && A((void **)&s->d_mv[l], n * 16) &&
         A((void **)&s->d_mn[l], n * 16);
    if (ok && s->cfg.rgb_term)
      ok = A((void **)&s->d_int[l], n) && A((void **)&s->d_int_last[l], n) && A((void **)&s->d_cand[l], n) &&
           A((void **)&s->d_dx[l], n * 2) && A((void **)&s->d_dy[l], n * 2) &&
           cudaMemset(s->d_int[l], 0, n) == cudaSuccess && cudaMemset(s->d_int_last[l], 0, n) == cudaSuccess;
  }
  if (ok && s->cfg.rgb_term) ok = A((void **)&s->d_corr, np * sizeof(float4));
  ok = ok && cudaMallocHost(&s->h_depth16, np * 2) == cudaSuccess &&
       cudaMallocHost(&s->h_rgb, np * 3) == cudaSuccess &&
       cudaMallocHost(&s->h_mask, np) == cudaSuccess &&
       cudaMallocHost(&s->h_stats, sizeof(sf_frame_stats)) == cudaSuccess &&
       cudaMallocHost(&s->h_ready, sizeof(uint32_t)) == cudaSuccess;
  if (ok) ok = cudaMemset(s->d_mask, 0, np) == cudaSuccess;
  if (ok) *s->h_ready = 0u;
  ok = ok && cudaStreamCreateWithFlags(&s->cstream, cudaStreamNonBlocking) == cudaSuccess &&
       cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking) == cudaSuccess &&
       cudaEventCreateWithFlags(&s->ev_fork, cudaEventDisableTiming) == cudaSuccess &&
       cudaEventCreateWithFlags(&s->ev_join, cudaEventDisableTiming) == cudaSuccess &&
       cudaEventCreateWithFlags(&s->ev_inputs, cudaEventDisableTiming) == cudaSuccess &&
       cudaEventCreateWithFlags(&s->ev_prev, cudaEventDisableTiming) == cudaSuccess;
  return ok ? SF_OK : SF_ERR_CUDA;
}

void free_all(sf_system *s) {
  cudaFree(s->d_depth16); cudaFree(s->d_rgb); cudaFree(s->d_mask); cudaFree(s->d_raw); cudaFree(s->d_rdepth);
  cudaFree(s->d_zmin); cudaFree(s->d_zmax); cudaFree(s->d_sys); cudaFree(s->d_stats); cudaFree(s->d_corr);
  cudaFree(s->d_seq);
  for (int l = 0; l < kMaxLevels; ++l) {
    cudaFree(s->d_depth[l]); cudaFree(s->d_vmap[l]); cudaFree(s->d_nmap[l]);
    cudaFree(s->d_mv[l]); cudaFree(s->d_mn[l]);
    cudaFree(s->d_int[l]); cudaFree(s->d_int_last[l]); cudaFree(s->d_cand[l]);
    cudaFree(s->d_dx[l]); cudaFree(s->d_dy[l]);
  }
  if (s->h_depth16) cudaFreeHost(s->h_depth16);
  if (s->h_rgb) cudaFreeHost(s->h_rgb);
  if (s->h_mask) cudaFreeHost(s->h_mask);
  if (s->h_stats) cudaFreeHost(s->h_stats);
  if (s->h_ready) cudaFreeHost(s->h_ready);
  if (s->gexec) cudaGraphExecDestroy(s->gexec);
  for (auto &e : s->ev)
    if (e) cudaEventDestroy(e);
  if (s->cstream) cudaStreamSynchronize(s->cstream);
  if (s->ev_inputs) cudaEventDestroy(s->ev_inputs);
  if (s->ev_prev) cudaEventDestroy(s->ev_prev);
  if (s->cstream) cudaStreamDestroy(s->cstream);
  if (s->side) cudaStreamSynchronize(s->side);
  if (s->ev_fork) cudaEventDestroy(s->ev_fork);
  if (s->ev_join) cudaEventDestroy(s->ev_join);
  if (s->side) cudaStreamDestroy(s->side);
}

// The frame's colour (and mask) upload on the copy stream; captured as an
// external event wait in the frame graph.
void wait_inputs(sf_system *s, cudaStream_t st) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(st, &cs);
  cudaStreamWaitEvent(st, s->ev_inputs, cs == cudaStreamCaptureStatusActive ? cudaEventWaitExternal : 0);
}

// Frame::FillImages intensity part (Core/Frame.cc:74-84), with the
// photometric term only: this frame's intensity pyramid, saving the one it
// replaces as the last frame's when the previous frame was tracked
// (SwapFrame, Tracking.cc:65-119; SysDev.run still holds that frame's
// outcome here), then the derivative images and candidate flags.
void enqueue_intensity(sf_system *s, cudaStream_t st) {
  const int C = s->cfg.cols, R = s->cfg.rows;
  sf_image im[kMaxLevels], sv[kMaxLevels], dx[kMaxLevels], dy[kMaxLevels], cd[kMaxLevels];
  for (int l = 0; l < s->L; ++l) {
    im[l] = img(s->d_int[l], C >> l, R >> l, 1);
    sv[l] = img(s->d_int_last[l], C >> l, R >> l, 1);
    dx[l] = img(s->d_dx[l], C >> l, R >> l, 2);
    dy[l] = img(s->d_dy[l], C >> l, R >> l, 2);
    cd[l] = img(s->d_cand[l], C >> l, R >> l, 1);
  }
  wait_inputs(s, st);
  launch_intensity_pyramid(img(s->d_rgb, C, R, 3), im, sv, dev_field<int>(s->d_sys, offsetof(SysDev, run)), dx,
                           dy, cd, s->L, st);
}

void rgb_levels(sf_system *s, RgbLevelArgs *rg) {
  const int C = s->cfg.cols, R = s->cfg.rows;
  for (int l = 0; l < s->L; ++l) {
    const int c = C >> l, r = R >> l;
    rg[l].inext = img(s->d_int[l], c, r, 1);
    rg[l].ilast = img(s->d_int_last[l], c, r, 1);
    rg[l].dx = img(s->d_dx[l], c, r, 2);
    rg[l].dy = img(s->d_dy[l], c, r, 2);
    rg[l].cand = img(s->d_cand[l], c, r, 1);
    rg[l].corr = s->d_corr;
  }
}

// Frame::FillImages (Core/Frame.cc:68-92): the depth pyramid, and with the
// photometric term the intensity pyramid forked onto the side stream so
// that the two run side by side (joined before this returns).
void enqueue_depth_pyramid(sf_system *s, cudaStream_t st);
void enqueue_pyramid(sf_system *s, cudaStream_t st) {
  Range nvtx_range("sf pyramid");
  if (!s->cfg.rgb_term) {
    enqueue_depth_pyramid(s, st);
    return;
  }
  cudaEventRecord(s->ev_fork, st);
  cudaStreamWaitEvent(s->side, s->ev_fork, 0);
  enqueue_intensity(s, s->side);
  cudaEventRecord(s->ev_join, s->side);
  enqueue_depth_pyramid(s, st);
  cudaStreamWaitEvent(st, s->ev_join, 0);
}

// Frame::FillImages depth part.
void enqueue_depth_pyramid(sf_system *s, cudaStream_t st) {
  const int C = s->cfg.cols, R = s->cfg.rows;
  launch_filter_depth(img(s->d_depth16, C, R, 2), img(s->d_raw, C, R, 4), img(s->d_depth[0], C, R, 4),
                      s->cfg.depth_scale, s->cfg.depth_cutoff, st);
  if (s->L >= 2) {
    sf_image d[kMaxLevels], v[kMaxLevels], n[kMaxLevels];
    for (int l = 0; l < s->L; ++l) {
      d[l] = img(s->d_depth[l], C >> l, R >> l, 4);
      v[l] = img(s->d_vmap[l], C >> l, R >> l, 16);
      n[l] = img(s->d_nmap[l], C >> l, R >> l, 16);
    }
    launch_pyramid_levels(d, v, n, s->L, s->cfg.K.fx, s->cfg.K.fy, s->cfg.K.cx, s->cfg.K.cy, s->cfg.depth_cutoff,
                          st);
    return;
  }
  for (int l = 0; l < s->L; ++l) {
    const int c = C >> l, r = R >> l;
    if (l > 0)
      launch_pyrdown(img(s->d_depth[l - 1], C >> (l - 1), R >> (l - 1), 4), img(s->d_depth[l], c, r, 4), st);
    const float div = (float)(1 << l);
    launch_vnmap(img(s->d_depth[l], c, r, 4), img(s->d_vmap[l], c, r, 16), img(s->d_nmap[l], c, r, 16),
                 s->cfg.K.fx / div, s->cfg.K.fy / div, s->cfg.K.cx / div, s->cfg.K.cy / div,
                 s->cfg.depth_cutoff, st);
  }
}

void icp_levels(sf_system *s, IcpLevelArgs *lv) {
  const int C = s->cfg.cols, R = s->cfg.rows;
  for (int l = 0; l < s->L; ++l) {
    const int c = C >> l, r = R >> l;
    const float div = (float)(1 << l);
    lv[l].vc = img(s->d_vmap[l], c, r, 16);
    lv[l].nc = img(s->d_nmap[l], c, r, 16);
    lv[l].vl = img(s->d_mv[l], c, r, 16);
    lv[l].nl = img(s->d_mn[l], c, r, 16);
    lv[l].fx = s->cfg.K.fx / div; lv[l].fy = s->cfg.K.fy / div;
    lv[l].cx = s->cfg.K.cx / div; lv[l].cy = s->cfg.K.cy / div;
    lv[l].iters = s->cfg.iters[l];
    lv[l].min_count = s->cfg.min_count[l];
  }
}

// The frame's stats (k_sys_stats); in a captured frame also written to
// h_stats (pinned, device-accessible) and flagged in h_ready.
cudaError_t enqueue_stats(sf_system *s, cudaStream_t st) {
  k_sys_stats<<<1, 1, 0, st>>>(s->d_sys, ctx_icp(s->ctx).ctl, map_dev(s->map), ctx_flags(s->ctx), s->d_stats,
                               s->capturing ? s->h_stats : nullptr, s->h_ready, s->d_seq);
  note_launch();
  return cudaGetLastError();
}

// Mapping::FuseColor (FuseMapColor) and Mapping::RayTrace of the frame's
// mapping stage.  `first` marks the stage boundaries and joins the colour
// upload; `plain` downloads the visible count and skips the integration
// when it is zero, as FuseMapColor does (FuseMap.cu:1116-1120).  `last`:
// the frame's final pass, whose raycast a device-driven frame's stats
// precede.
int fuse_and_raytrace(sf_system *s, const Cam *cam, const int *run, int num_detection, const sf_image &nmap,
                      bool first, bool last, bool plain, cudaStream_t st) {
  const int C = s->cfg.cols, R = s->cfg.rows;
  DevMap &m = map_dev(s->map);
  FuseScratch &f = map_scratch(s->map);
  uint32_t *flags = ctx_flags(s->ctx);
  sf_image depth = img(s->d_raw, C, R, 4), rgb = img(s->d_rgb, C, R, 3), mask = img(s->d_mask, C, R, 1);
  sf_image zmin = img(s->d_zmin, s->zc, s->zr, 4), zmax = img(s->d_zmax, s->zc, s->zr, 4);
  // the first pass of a device-driven frame starts its allocation epoch in
  // k_sys_post
  // the insert pass's launch also starts the visibility pass (counters,
  // window box, cleared window cells and z-range)
  launch_alloc(m, f, depth, cam, run, flags, st, /*begin=*/!first || run == nullptr, s->alloc_tile, &zmin, &zmax);
  if (first) mark(s, st, 3);
  launch_visibility(m, f, cam, &zmin, &zmax, run, flags, st, /*started=*/true);
  if (first) {
    mark(s, st, 4);
    // the frame's colour and mask (already waited for by the intensity
    // pyramid with the photometric term)
    if (!s->cfg.rgb_term) wait_inputs(s, st);
  }
  bool integrate = true;
  if (plain) {
    uint32_t nvis = 0;
    if (cudaMemcpyAsync(&nvis, m.no_visible, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return SF_ERR_CUDA;
    integrate = nvis > 0;
  }
  if (integrate) {
    launch_integrate(m, depth, rgb, &nmap, &mask, num_detection, cam, true, num_detection > 0, run, st,
                     s->int_ctas);
    if (num_detection > 0) launch_unify_neighbor(m, f, run, st);  // FuseMap.cu:1141-1160
  }
  if (first) mark(s, st, 5);
  // a device-driven frame's stats, final here, are written by the first
  // thread of its last raycast (k_sys_stats's work, without its launch)
  FrameStatsArgs stats;
  const bool with_stats = last && !plain;
  if (with_stats) {
    stats.sys = s->d_sys;
    stats.ctl = ctx_icp(s->ctx).ctl;
    stats.flags = ctx_flags(s->ctx);
    stats.out = s->d_stats;
    stats.host_out = s->capturing ? s->h_stats : nullptr;
    stats.host_ready = s->h_ready;
    stats.seq = s->d_seq;
    s->stats_taken = true;
  }
  sf_image fv = img(s->d_vmap[0], C, R, 16), fn = img(s->d_nmap[0], C, R, 16);
  launch_raycast(m, f, img(s->d_mv[0], C, R, 16), img(s->d_mn[0], C, R, 16), zmin, zmax, cam,
                 f.counters + 3, &fv, &fn, run, st, s->rc_tune, with_stats ? &stats : nullptr);
  if (with_stats && cudaGetLastError() != cudaSuccess) return SF_ERR_CUDA;
  if (first) mark(s, st, 6);
  return SF_OK;
}

// The mapping stage of System::GrabImage (Core/System.cc:161-212) and the
// next frame's Frame::ResizeImages, every launch gated by `run` (device)
// when given.  Mapping: FuseColor + RayTrace; with detections (the
// semantic mode, gap_semantic = 1) FuseColor again with the labels, its
// label pass reading the raycast normals, and RayTrace.  Localisation
// (mapping disabled): UpdateVisibility + RayTrace; with detections
// Mapping::SemanticAnalysis: AnalyzeMapSemantics on the rendered depth
// (vmap[0].z, Mapping.cc:99-123).
int enqueue_mapping(sf_system *s, const Cam *cam, const int *run, int num_detection, bool plain,
                    cudaStream_t st) {
  Range nvtx_range("sf mapping");
  const int C = s->cfg.cols, R = s->cfg.rows;
  DevMap &m = map_dev(s->map);
  FuseScratch &f = map_scratch(s->map);
  uint32_t *flags = ctx_flags(s->ctx);
  const sf_image mn0 = img(s->d_mn[0], C, R, 16);
  int e = SF_OK;
  if (s->mapping) {
    e = fuse_and_raytrace(s, cam, run, 0, img(s->d_nmap[0], C, R, 16), true, num_detection == 0, plain, st);
    if (e == SF_OK && num_detection > 0)
      e = fuse_and_raytrace(s, cam, run, num_detection, mn0, false, true, plain, st);
  } else {
    sf_image zmin = img(s->d_zmin, s->zc, s->zr, 4), zmax = img(s->d_zmax, s->zc, s->zr, 4);
    mark(s, st, 3);
    launch_visibility(m, f, cam, &zmin, &zmax, run, flags, st);
    mark(s, st, 4);
    if (!s->cfg.rgb_term) wait_inputs(s, st);
    mark(s, st, 5);
    sf_image fv = img(s->d_vmap[0], C, R, 16), fn = img(s->d_nmap[0], C, R, 16);
    launch_raycast(m, f, img(s->d_mv[0], C, R, 16), mn0, zmin, zmax, cam, f.counters + 3, &fv, &fn, run, st,
                   s->rc_tune);
    mark(s, st, 6);
    if (num_detection > 0) {
      const sf_image rd = img(s->d_rdepth, C, R, 4), rgb = img(s->d_rgb, C, R, 3), mask = img(s->d_mask, C, R, 1);
      launch_vmap_depth(img(s->d_mv[0], C, R, 16), rd, run, st);
      launch_visibility(m, f, cam, nullptr, nullptr, run, flags, st);
      launch_integrate(m, rd, rgb, &mn0, &mask, num_detection, cam, false, true, run, st, s->int_ctas);
      launch_unify_neighbor(m, f, run, st);
    }
  }
  if (e != SF_OK) return e;
  int l = 1;
  if (s->L >= 3) {  // levels 1 and 2 in one launch
    launch_resize2(img(s->d_mv[0], C, R, 16), img(s->d_mn[0], C, R, 16), img(s->d_mv[1], C >> 1, R >> 1, 16),
                   img(s->d_mn[1], C >> 1, R >> 1, 16), img(s->d_mv[2], C >> 2, R >> 2, 16),
                   img(s->d_mn[2], C >> 2, R >> 2, 16), st);
    l = 3;
  }
  for (; l < s->L; ++l)
    launch_resize(img(s->d_mv[l - 1], C >> (l - 1), R >> (l - 1), 16),
                  img(s->d_mn[l - 1], C >> (l - 1), R >> (l - 1), 16),
                  img(s->d_mv[l], C >> l, R >> l, 16), img(s->d_mn[l], C >> l, R >> l, 16), st);
  return SF_OK;
}

// Device-driven frame (eager and graph forms).
cudaError_t enqueue_device_frame(sf_system *s, int num_detection, cudaStream_t st) {
  Range nvtx_range("sf frame (device-driven)");
  IcpWorkspace &w = ctx_icp(s->ctx);
  mark(s, st, 0);
  enqueue_pyramid(s, st);
  mark(s, st, 1);
  IcpLevelArgs lv[kMaxLevels];
  icp_levels(s, lv);
  cudaError_t e = icp_persistent_reset(w, st);
  if (e != cudaSuccess) return e;
  RgbLevelArgs rg[kMaxLevels];
  if (s->cfg.rgb_term) rgb_levels(s, rg);
  // the tracker's state update after ComputeSE3 (Track) runs at the
  // kernel's end
  FramePost post;
  post.sys = s->d_sys;
  post.tmpl = s->tmpl;
  post.f = map_scratch(s->map);
  e = launch_icp_persistent(w, lv, s->L, s->cfg.icp_thresh, dev_field<double>(s->d_sys, offsetof(SysDev, last_pose)),
                            dev_field<int>(s->d_sys, offsetof(SysDev, state)),
                            ctx_flags(s->ctx), st, s->cfg.rgb_term ? rg : nullptr, &post);
  if (e != cudaSuccess) return e;
  mark(s, st, 2);
  s->stats_taken = false;
  if (enqueue_mapping(s, dev_field<Cam>(s->d_sys, offsetof(SysDev, cam)),
                      dev_field<int>(s->d_sys, offsetof(SysDev, run)), num_detection, false, st) != SF_OK)
    return cudaErrorUnknown;
  if (!s->stats_taken) {
    e = enqueue_stats(s, st);
    if (e != cudaSuccess) return e;
  }
  mark(s, st, 7);
  return cudaGetLastError();
}

// Host-driven frame (plain per-launch form).
int run_plain_frame(sf_system *s, int num_detection) {
  Range nvtx_range("sf frame (plain)");
  cudaStream_t st = ctx_stream(s->ctx);
  IcpWorkspace &w = ctx_icp(s->ctx);
  enqueue_pyramid(s, st);
  const int state = s->state;
  int ok = 0;
  if (state == 1) {
    ctl_begin(s->ctl, s->last_pose);
    s->ctl.accepted = 1;
    ok = 1;
  } else if (state == -1) {
    // lost, and no candidates to relocalise against: the frame is skipped
  } else {
    IcpLevelArgs lv[kMaxLevels];
    icp_levels(s, lv);
    RgbLevelArgs rg[kMaxLevels];
    if (s->cfg.rgb_term) rgb_levels(s, rg);
    ctl_begin(s->ctl, s->last_pose);
    double sums[58];  // ICP, then RGB
    for (int l = s->L - 1; l >= 0 && !s->ctl.stop; --l) {
      for (int j = 0; j < lv[l].iters; ++j) {
        m3 Rc, Rci, Rl, Rli;
        f3 tc, tl;
        auto tofl = [](const double *P, m3 &R, m3 &Ri, f3 &t) {
          R.rx = {(float)P[0], (float)P[1], (float)P[2]};
          R.ry = {(float)P[4], (float)P[5], (float)P[6]};
          R.rz = {(float)P[8], (float)P[9], (float)P[10]};
          Ri.rx = {(float)P[0], (float)P[4], (float)P[8]};
          Ri.ry = {(float)P[1], (float)P[5], (float)P[9]};
          Ri.rz = {(float)P[2], (float)P[6], (float)P[10]};
          t = {(float)P[3], (float)P[7], (float)P[11]};
        };
        tofl(s->ctl.next_pose, Rc, Rci, tc);
        tofl(s->ctl.last_pose, Rl, Rli, tl);
        const bool rgb = s->cfg.rgb_term != 0;
        // RGBStep then ICPStep (Tracking.cc:400-447), each downloading its sums
        if (rgb) launch_rgb_step(w, lv[l], rg[l], Rc, Rci, tc, Rl, Rli, tl, st);
        launch_icp_step(w, lv[l], Rc, tc, Rl, Rli, tl, st);
        if (cudaMemcpyAsync(sums, w.sums, (rgb ? 58 : 29) * sizeof(double), cudaMemcpyDeviceToHost, st) !=
                cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
          return SF_ERR_CUDA;
        if (!ctl_step(s->ctl, sums, lv[l].min_count, rgb ? sums + 29 : nullptr)) break;
      }
    }
    ctl_finish(s->ctl, s->cfg.icp_thresh);
    ok = s->ctl.accepted;
  }
  int next = 0;
  const int tracked = track_transition(state, s->prev_state, ok, next, s->missed);
  if (state == 0 && tracked) memcpy(s->last_pose, s->ctl.next_pose, sizeof(s->last_pose));
  s->prev_state = state;
  s->state = next;
  // host -> device state (camera, pose, decision) for the mapping pass
  SysDev sd;
  memset(&sd, 0, sizeof(sd));
  memcpy(sd.last_pose, s->last_pose, sizeof(sd.last_pose));
  sd.state = next;
  sd.prev_state = state;
  sd.missed = s->missed;
  sd.run = tracked;
  sd.accepted = ok;
  sd.first = state == 1 ? 1 : 0;
  sd.icp_ran = state == 0 ? 1 : 0;
  const double *P = s->last_pose;
  sd.cam = s->tmpl;
  sd.cam.R.rx = {(float)P[0], (float)P[1], (float)P[2]};
  sd.cam.R.ry = {(float)P[4], (float)P[5], (float)P[6]};
  sd.cam.R.rz = {(float)P[8], (float)P[9], (float)P[10]};
  sd.cam.Rinv.rx = {(float)P[0], (float)P[4], (float)P[8]};
  sd.cam.Rinv.ry = {(float)P[1], (float)P[5], (float)P[9]};
  sd.cam.Rinv.rz = {(float)P[2], (float)P[6], (float)P[10]};
  sd.cam.t = {(float)P[3], (float)P[7], (float)P[11]};
  if (cudaMemcpyAsync(s->d_sys, &sd, sizeof(sd), cudaMemcpyHostToDevice, st) != cudaSuccess)
    return SF_ERR_CUDA;
  if (cudaMemcpyAsync(w.ctl, &s->ctl, sizeof(TrackCtl), cudaMemcpyHostToDevice, st) != cudaSuccess)
    return SF_ERR_CUDA;
  if (tracked) {
    int e = enqueue_mapping(s, dev_field<Cam>(s->d_sys, offsetof(SysDev, cam)), nullptr, num_detection, true, st);
    if (e != SF_OK) return e;
  }
  k_sys_stats<<<1, 1, 0, st>>>(s->d_sys, w.ctl, map_dev(s->map), ctx_flags(s->ctx), s->d_stats, nullptr, nullptr,
                               nullptr);
  note_launch();
  return cudaGetLastError() == cudaSuccess ? SF_OK : SF_ERR_CUDA;
}

// ValidatePose's constants (Tracking.h:111,119; Tracking.cc:758):
// ITERATIONS_RELOC per level (level 0 first; levels beyond the reference's
// three run none), THRESH_ICP_RELOC, and the visible-block floor.
constexpr int kRelocIters[kMaxLevels] = {3, 3, 2, 0};
constexpr float kRelocThresh = 1e-3f;
constexpr uint32_t kRelocMinVisible = 512;

void set_cam(Cam &c, const Cam &tmpl, const double *P) {
  c = tmpl;
  c.R.rx = {(float)P[0], (float)P[1], (float)P[2]};
  c.R.ry = {(float)P[4], (float)P[5], (float)P[6]};
  c.R.rz = {(float)P[8], (float)P[9], (float)P[10]};
  c.Rinv.rx = {(float)P[0], (float)P[4], (float)P[8]};
  c.Rinv.ry = {(float)P[1], (float)P[5], (float)P[9]};
  c.Rinv.rz = {(float)P[2], (float)P[6], (float)P[10]};
  c.t = {(float)P[3], (float)P[7], (float)P[11]};
}

// A frame that starts lost, with candidate poses registered: Track()'s
// state -1, Tracker::Relocalise's validation and final refinement
// (Tracking.cc:107-116, 750-790), host-driven in every form.  The caller's
// candidates stand in for the poses Relocalise estimates from SURF matches
// (keypoint matching is outside this loop).  ValidatePose runs as one
// batched call; the pose it keeps becomes LastFrame's pose (whether or not
// the final ComputeSE3 then accepts), LastFrame's model maps are ray traced
// and resized there, and ComputeSE3(icpOnly = true) with the loop's
// iterations and threshold refines it.  Accepted, the frame is tracked and
// mapped like any other.
int run_reloc_frame(sf_system *s, int num_detection) {
  Range nvtx_range("sf frame (relocalise)");
  cudaStream_t st = ctx_stream(s->ctx);
  IcpWorkspace &w = ctx_icp(s->ctx);
  const int C = s->cfg.cols, R = s->cfg.rows, L = s->L;
  const bool plain = s->cfg.use_graph == 0;
  DevMap &m = map_dev(s->map);
  FuseScratch &f = map_scratch(s->map);
  s->host_driven = true;
  SysDev sd;
  if (plain) {
    memset(&sd, 0, sizeof(sd));
    memcpy(sd.last_pose, s->last_pose, sizeof(sd.last_pose));
    sd.prev_state = s->prev_state;
    sd.missed = s->missed;
  } else if (cudaMemcpyAsync(&sd, s->d_sys, sizeof(sd), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
             cudaStreamSynchronize(st) != cudaSuccess) {
    return SF_ERR_CUDA;
  }
  enqueue_pyramid(s, st);
  sf_image nv[kMaxLevels], nn[kMaxLevels], lv[kMaxLevels], ln[kMaxLevels];
  int iters[kMaxLevels], minc[kMaxLevels];
  for (int l = 0; l < L; ++l) {
    nv[l] = img(s->d_vmap[l], C >> l, R >> l, 16);
    nn[l] = img(s->d_nmap[l], C >> l, R >> l, 16);
    lv[l] = img(s->d_mv[l], C >> l, R >> l, 16);
    ln[l] = img(s->d_mn[l], C >> l, R >> l, 16);
    iters[l] = kRelocIters[l];
    minc[l] = s->cfg.min_count[l];
  }
  const int n = (int)(s->reloc.size() / 16);
  std::vector<sf_reloc_candidate> out((size_t)n);
  int chosen = -1;
  int e = sf_ValidatePoseBatch(s->ctx, s->map, L, nv, nn, lv, ln, s->cfg.K, s->reloc.data(), n, iters, minc,
                               kRelocThresh, kRelocMinVisible, out.data(), &chosen);
  if (e != SF_OK) return e;
  const Cam *cam = dev_field<Cam>(s->d_sys, offsetof(SysDev, cam));
  int ok = 0;
  TrackCtl &ctl = s->ctl;
  if (chosen >= 0) {
    // LastFrame->pose = the kept candidate; UpdateVisibility, RayTrace and
    // ResizeImages there (Tracking.cc:780-785)
    memcpy(sd.last_pose, s->reloc.data() + 16 * (size_t)chosen, sizeof(sd.last_pose));
    set_cam(sd.cam, s->tmpl, sd.last_pose);
    if (cudaMemcpyAsync(s->d_sys, &sd, sizeof(sd), cudaMemcpyHostToDevice, st) != cudaSuccess) return SF_ERR_CUDA;
    const sf_image zmin = img(s->d_zmin, s->zc, s->zr, 4), zmax = img(s->d_zmax, s->zc, s->zr, 4);
    launch_visibility(m, f, cam, &zmin, &zmax, nullptr, ctx_flags(s->ctx), st);
    launch_raycast(m, f, lv[0], ln[0], zmin, zmax, cam, f.counters + 3, nullptr, nullptr, nullptr, st, s->rc_tune);
    for (int l = 1; l < L; ++l) launch_resize(lv[l - 1], ln[l - 1], lv[l], ln[l], st);
    // ComputeSE3(true, ITERATIONS_SE3, THRESH_ICP_SE3) from it (Tracking.cc:789)
    IcpLevelArgs il[kMaxLevels];
    icp_levels(s, il);
    if (icp_persistent_reset(w, st) != cudaSuccess ||
        launch_icp_persistent(w, il, L, s->cfg.icp_thresh, dev_field<double>(s->d_sys, offsetof(SysDev, last_pose)),
                              nullptr, ctx_flags(s->ctx), st) != cudaSuccess ||
        cudaMemcpyAsync(&ctl, w.ctl, sizeof(TrackCtl), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return SF_ERR_CUDA;
    ok = ctl.accepted;
  }
  int next = -1, missed = sd.missed;
  const int tracked = track_transition(-1, sd.prev_state, ok, next, missed);
  if (tracked) memcpy(sd.last_pose, ctl.next_pose, sizeof(sd.last_pose));
  sd.state = next;
  sd.prev_state = -1;
  sd.missed = missed;
  sd.run = tracked;
  sd.accepted = ok;
  sd.first = 0;
  sd.relocalised = tracked;
  sd.icp_ran = chosen >= 0 ? 1 : 0;
  set_cam(sd.cam, s->tmpl, sd.last_pose);
  if (cudaMemcpyAsync(s->d_sys, &sd, sizeof(sd), cudaMemcpyHostToDevice, st) != cudaSuccess) return SF_ERR_CUDA;
  if (plain) {
    memcpy(s->last_pose, sd.last_pose, sizeof(s->last_pose));
    s->state = next;
    s->prev_state = -1;
    s->missed = missed;
  } else {
    s->dev_state = next;
  }
  if (tracked) {
    e = enqueue_mapping(s, cam, nullptr, num_detection, true, st);
    if (e != SF_OK) return e;
  } else if (!s->cfg.rgb_term) {
    wait_inputs(s, st);  // the colour upload is not left behind the frame
  }
  k_sys_stats<<<1, 1, 0, st>>>(s->d_sys, w.ctl, m, ctx_flags(s->ctx), s->d_stats, nullptr, nullptr, nullptr);
  note_launch();
  return cudaGetLastError() == cudaSuccess ? SF_OK : SF_ERR_CUDA;
}

// The state the next frame starts in, when candidates are registered: the
// plain form keeps it on the host; the device forms read it back when the
// last frame's stats did not bring it.
int upcoming_state(sf_system *s, int *state) {
  if (s->cfg.use_graph == 0) {
    *state = s->state;
    return SF_OK;
  }
  if (s->dev_state == -2) {
    int v = 0;
    if (cudaMemcpyAsync(&v, dev_field<int>(s->d_sys, offsetof(SysDev, state)), sizeof(int), cudaMemcpyDeviceToHost,
                        ctx_stream(s->ctx)) != cudaSuccess ||
        cudaStreamSynchronize(ctx_stream(s->ctx)) != cudaSuccess)
      return SF_ERR_CUDA;
    s->dev_state = v;
  }
  *state = s->dev_state;
  return SF_OK;
}

int run_frame(sf_system *s, int num_detection) {
  cudaStream_t st = ctx_stream(s->ctx);
  ++s->frames;
  s->host_driven = false;
  if (num_detection > 0) {  // UnifyNeighbor's output buffer, before any capture
    int e = fuse_scratch_unify(map_scratch(s->map), map_dev(s->map).c);
    if (e != SF_OK) return e;
  }
  if (!s->reloc.empty()) {
    int state = 0;
    int e = upcoming_state(s, &state);
    if (e != SF_OK) return e;
    if (state == -1) return run_reloc_frame(s, num_detection);
  }
  s->dev_state = -2;  // a device-form frame decides the next state on the device
  if (s->cfg.use_graph == 0) return run_plain_frame(s, num_detection);
  if (s->cfg.use_graph == 2) {  // eager device-driven
    return enqueue_device_frame(s, num_detection, st) == cudaSuccess ? SF_OK : SF_ERR_CUDA;
  }
  const int sem = num_detection > 0 ? 1 : 0;
  if (!s->gexec || s->graph_sem != sem || s->graph_mapping != s->mapping ||
      (sem && s->num_detection_captured != num_detection)) {
    if (s->gexec) { cudaGraphExecDestroy(s->gexec); s->gexec = nullptr; }
    cudaGraph_t g = nullptr;
    const unsigned long long before = launches_total();
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return SF_ERR_CUDA;
    s->capturing = true;
    s->graph_early = false;
    cudaError_t e = enqueue_device_frame(s, num_detection, st);
    s->capturing = false;
    cudaError_t e2 = cudaStreamEndCapture(st, &g);
    // captured launches are recorded, not run: count them per replay instead
    s->graph_kernels = launches_total() - before;
    note_launch(0ull - s->graph_kernels);
    if (e != cudaSuccess || e2 != cudaSuccess || !g) {
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
      return SF_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&s->gexec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { s->gexec = nullptr; return SF_ERR_CUDA; }
    s->graph_sem = sem;
    s->graph_mapping = s->mapping;
    s->graph_early = true;  // every captured frame writes h_stats and h_ready
    s->num_detection_captured = num_detection;
  }
  Range nvtx_range("sf frame (graph replay)");
  if (cudaGraphLaunch(s->gexec, st) != cudaSuccess) return SF_ERR_CUDA;
  ++s->graph_seq;  // this replay's k_sys_stats writes this number to h_ready
  note_launch(s->graph_kernels);
  return SF_OK;
}

}  // namespace

extern "C" {

int sf_system_create(sf_context *ctx, const sf_system_config *cfg, const double init_pose[16],
                     sf_system **out) {
  if (!ctx || !cfg || !out) return SF_ERR_INVALID;
  *out = nullptr;
  if (cfg->cols <= 0 || cfg->rows <= 0 || cfg->levels < 1 || cfg->levels > kMaxLevels ||
      (cfg->cols >> (cfg->levels - 1)) < 2 || (cfg->rows >> (cfg->levels - 1)) < 2 ||
      cfg->depth_scale <= 0 || cfg->K.fx <= 0 || cfg->K.fy <= 0 || cfg->rgb_term < 0 || cfg->rgb_term > 1 ||
      (cfg->rgb_term && ((size_t)cfg->cols >= 65536 || (size_t)cfg->rows >= 32768)))
    return SF_ERR_INVALID;
  sf_system *s = new (std::nothrow) sf_system();
  if (!s) return SF_ERR_INVALID;
  s->ctx = ctx;
  s->cfg = *cfg;
  s->L = cfg->levels;
  s->zc = cfg->zrange_cols > 0 ? cfg->zrange_cols : (cfg->cols + 7) / 8;
  s->zr = cfg->zrange_rows > 0 ? cfg->zrange_rows : (cfg->rows + 7) / 8;
  for (int k = 0; k < 16; ++k) s->last_pose[k] = init_pose ? init_pose[k] : (k % 5 == 0 ? 1.0 : 0.0);
  int st = sf_map_create(&cfg->map, &s->map);
  if (st == SF_OK) st = alloc_all(s);
  if (st == SF_OK) st = map_ensure_scratch(s->map, cfg->cols * cfg->rows);
  if (st == SF_OK) {
    Cam &c = s->tmpl;
    memset(&c, 0, sizeof(c));
    c.fx = cfg->K.fx; c.fy = cfg->K.fy; c.cx = cfg->K.cx; c.cy = cfg->K.cy;
    c.invfx = (float)(1.0 / (double)cfg->K.fx);
    c.invfy = (float)(1.0 / (double)cfg->K.fy);
    c.cols = cfg->cols; c.rows = cfg->rows;
    c.dmin = cfg->map.depth_min; c.dmax = cfg->map.depth_max;
    SysDev sd;
    memset(&sd, 0, sizeof(sd));
    memcpy(sd.last_pose, s->last_pose, sizeof(sd.last_pose));
    sd.state = 1;
    if (cudaMemcpy(s->d_sys, &sd, sizeof(sd), cudaMemcpyHostToDevice) != cudaSuccess) st = SF_ERR_CUDA;
    ctl_begin(s->ctl, s->last_pose);
  }
  if (st != SF_OK) {
    sf_system_destroy(s);
    return st;
  }
  *out = s;
  return SF_OK;
}

int sf_system_destroy(sf_system *s) {
  if (!s) return SF_ERR_INVALID;
  if (s->ctx) cudaStreamSynchronize(ctx_stream(s->ctx));
  free_all(s);
  if (s->map) sf_map_destroy(s->map);
  delete s;
  return SF_OK;
}

int sf_system_grab(sf_system *s, const uint16_t *depth, const uint8_t *rgb, const uint8_t *mask,
                   int num_detection, sf_frame_stats *stats) {
  if (!s || !depth || !rgb) return SF_ERR_INVALID;
  if (num_detection > 0 && !mask) return SF_ERR_INVALID;
  cudaStream_t st = ctx_stream(s->ctx);
  const size_t np = (size_t)s->cfg.cols * s->cfg.rows;
  // host -> device: straight from the caller's buffer when it is pinned
  // (page-locked or registered), through the pinned staging buffer when not
  auto upload = [&](void *dst, const void *src, void *staging, size_t n, cudaStream_t on) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, src) == cudaSuccess && a.type == cudaMemoryTypeHost)
      return cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, on);
    cudaGetLastError();  // an unregistered pointer is not an error here
    memcpy(staging, src, n);
    return cudaMemcpyAsync(dst, staging, n, cudaMemcpyHostToDevice, on);
  };
  // Depth on the frame's stream; colour and mask on the copy stream after
  // the previous frame's work (their buffers are read by its integration),
  // overlapping this frame's pyramid and ICP.
  if (cudaEventRecord(s->ev_prev, st) != cudaSuccess || cudaStreamWaitEvent(s->cstream, s->ev_prev, 0) != cudaSuccess)
    return SF_ERR_CUDA;
  if (upload(s->d_depth16, depth, s->h_depth16, np * 2, st) != cudaSuccess ||
      upload(s->d_rgb, rgb, s->h_rgb, np * 3, s->cstream) != cudaSuccess)
    return SF_ERR_CUDA;
  if (num_detection > 0 && upload(s->d_mask, mask, s->h_mask, np, s->cstream) != cudaSuccess) return SF_ERR_CUDA;
  if (cudaEventRecord(s->ev_inputs, s->cstream) != cudaSuccess) return SF_ERR_CUDA;
  int r = run_frame(s, num_detection);
  if (r) return r;
  if (s->cfg.use_graph == 1 && s->graph_early && !s->host_driven) {
    // the graph wrote them before its final raycast; the wait ends with this
    // frame's sequence number in the flag (an earlier frame's number, left
    // by a replay that sf_system_grab_device launched and nobody waited for,
    // does not end it), or with the stream (done, or failed)
    const uint32_t want = s->graph_seq;
    while (__atomic_load_n(s->h_ready, __ATOMIC_ACQUIRE) != want) {
      const cudaError_t q = cudaStreamQuery(st);
      if (q == cudaErrorNotReady) continue;
      if (q != cudaSuccess || __atomic_load_n(s->h_ready, __ATOMIC_ACQUIRE) != want) return SF_ERR_CUDA;
    }
  } else if (cudaMemcpyAsync(s->h_stats, s->d_stats, sizeof(sf_frame_stats), cudaMemcpyDeviceToHost, st) !=
                 cudaSuccess ||
             cudaStreamSynchronize(st) != cudaSuccess) {
    return SF_ERR_CUDA;
  }
  if (s->cfg.use_graph != 0) s->dev_state = s->h_stats->state;
  if (stats) *stats = *s->h_stats;
  return s->h_stats->fail == 3 ? SF_ERR_TIMEOUT : SF_OK;
}

int sf_system_grab_device(sf_system *s, const uint16_t *depth, const uint8_t *rgb,
                          const uint8_t *mask, int num_detection) {
  if (!s || !depth || !rgb) return SF_ERR_INVALID;
  if (num_detection > 0 && !mask) return SF_ERR_INVALID;
  cudaStream_t st = ctx_stream(s->ctx);
  const size_t np = (size_t)s->cfg.cols * s->cfg.rows;
  if (depth != s->d_depth16 &&
      cudaMemcpyAsync(s->d_depth16, depth, np * 2, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
    return SF_ERR_CUDA;
  if (rgb != s->d_rgb && cudaMemcpyAsync(s->d_rgb, rgb, np * 3, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
    return SF_ERR_CUDA;
  if (num_detection > 0 && mask != s->d_mask &&
      cudaMemcpyAsync(s->d_mask, mask, np, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
    return SF_ERR_CUDA;
  return run_frame(s, num_detection);
}

int sf_system_set_reloc_candidates(sf_system *s, const double *poses, int n) {
  if (!s || n < 0 || n > 65535 || (n > 0 && !poses)) return SF_ERR_INVALID;
  s->reloc.assign(poses, poses + 16 * (size_t)n);
  s->dev_state = -2;
  return SF_OK;
}

int sf_system_set_mapping(sf_system *s, int enabled) {
  if (!s || (enabled != 0 && enabled != 1)) return SF_ERR_INVALID;
  s->mapping = enabled;  // the frame graph is captured again on the next frame
  return SF_OK;
}

int sf_system_autotune(sf_system *s, int reps, sf_autotune_report *report) {
  Range nvtx_range("sf autotune");
  if (!s || reps < 1 || reps > 1000) return SF_ERR_INVALID;
  if (s->frames < 1) return SF_ERR_INVALID;  // needs one grabbed frame: the stages' inputs
  cudaStream_t st = ctx_stream(s->ctx);
  const int C = s->cfg.cols, R = s->cfg.rows;
  DevMap &m = map_dev(s->map);
  FuseScratch &f = map_scratch(s->map);
  const sf_image mv = img(s->d_mv[0], C, R, 16), mn = img(s->d_mn[0], C, R, 16);
  const sf_image zmin = img(s->d_zmin, s->zc, s->zr, 4), zmax = img(s->d_zmax, s->zc, s->zr, 4);
  const sf_image fv = img(s->d_vmap[0], C, R, 16), fn = img(s->d_nmap[0], C, R, 16);
  const sf_image depth = img(s->d_raw, C, R, 4), rgb = img(s->d_rgb, C, R, 3), mask = img(s->d_mask, C, R, 1);
  const Cam *cam = dev_field<Cam>(s->d_sys, offsetof(SysDev, cam));
  const int *run = dev_field<int>(s->d_sys, offsetof(SysDev, run));
  static const int kIntCtas[4] = {2, 4, 8, 16};
  sf_autotune_report rep;
  memset(&rep, 0, sizeof(rep));
  rep.candidates = kRaycastTunes;
  rep.integrate_chosen = -1;
  // The last frame's integration and raycast run again as the frame ran
  // them: the visible blocks' voxels are saved first and restored before
  // every run, and L2 is flushed after the restore, so each timed launch
  // starts from the frame's state; the raycast is timed right after an
  // integration, as in the frame.  At the end the voxels are restored and
  // the raycast rerun with the frame's shape, which rewrites the same model
  // maps: the loop's state is unchanged.
  unsigned nvis = 0;
  int win[6] = {0, 0, 0, 0, 0, 0};
  cudaError_t e = cudaMemcpyAsync(&nvis, m.no_visible, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(win, f.win, sizeof(win), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return SF_ERR_CUDA;
  nvis = nvis < m.c.num_entries ? nvis : m.c.num_entries;
  const bool fuse = s->mapping && nvis > 0;
  const size_t flush_bytes = 256u << 20;
  void *save = nullptr, *flush = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess) e = cudaMalloc(&flush, flush_bytes);
  if (e == cudaSuccess && fuse) e = cudaMalloc(&save, (size_t)nvis * 512 * sizeof(sf_voxel));
  if (e == cudaSuccess && fuse) launch_save_visible(m, save, nvis, false, st);
  // the frame's visibility pass has just written the block-pointer window
  // when its integration and raycast run: after the flush, the window is
  // read back into L2 (copied into the flush buffer) to stand in for it
  const size_t win_bytes = sizeof(int) * (size_t)win[3] * (size_t)win[4] * (size_t)win[5];
  auto prepare = [&]() {
    if (fuse) launch_save_visible(m, save, nvis, true, st);
    cudaError_t q = cudaMemsetAsync(flush, 0, flush_bytes, st);
    if (q == cudaSuccess && win_bytes > 0 && win_bytes <= flush_bytes)
      q = cudaMemcpyAsync(flush, f.win_cells, win_bytes, cudaMemcpyDeviceToDevice, st);
    return q;
  };
  auto timed = [&](auto &&launch, float &ms_out) {
    float total = 0.f;
    for (int k = 0; k <= reps && e == cudaSuccess; ++k) {  // k = 0 warms up
      e = launch(true);
      if (e != cudaSuccess) break;
      cudaEventRecord(e0, st);
      launch(false);
      cudaEventRecord(e1, st);
      e = cudaEventSynchronize(e1);
      float ms = 0.f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
      if (k > 0) total += ms;
    }
    ms_out = total / (float)reps;
  };
  int best = 0;
  for (int i = 0; i < kRaycastTunes && e == cudaSuccess; ++i) {
    const RaycastTune t = raycast_tune(i);
    timed([&](bool before) -> cudaError_t {
      if (before) {
        cudaError_t q = prepare();
        if (fuse) launch_integrate(m, depth, rgb, &fn, &mask, 0, cam, true, false, run, st, s->int_ctas);
        return q;
      }
      launch_raycast(m, f, mv, mn, zmin, zmax, cam, f.counters + 3, &fv, &fn, run, st, t);
      return cudaSuccess;
    }, rep.ms[i]);
    rep.minb[i] = t.minb;
    rep.tile_x[i] = t.tx;
    rep.tile_y[i] = t.ty;
    if (rep.ms[i] < rep.ms[best]) best = i;
  }
  rep.chosen = best;
  int ibest = 2;
  if (fuse) {
    rep.integrate_candidates = 4;
    for (int i = 0; i < 4 && e == cudaSuccess; ++i) {
      timed([&](bool before) -> cudaError_t {
        if (before) return prepare();
        launch_integrate(m, depth, rgb, &fn, &mask, 0, cam, true, false, run, st, kIntCtas[i]);
        return cudaSuccess;
      }, rep.integrate_ms[i]);
      rep.integrate_ctas[i] = kIntCtas[i];
      if (rep.integrate_ms[i] < rep.integrate_ms[ibest]) ibest = i;
    }
    rep.integrate_chosen = ibest;
  }
  // the allocation walk's probe pass over the frame's depth and pose: the
  // frame allocated every block it meets (and requested, in this epoch,
  // any it could not), so the reruns request nothing and change nothing
  int abest = s->alloc_tile;
  rep.alloc_chosen = -1;
  if (fuse) {
    rep.alloc_candidates = kAllocTileCount;
    abest = 0;
    for (int i = 0; i < kAllocTileCount && e == cudaSuccess; ++i) {
      timed([&](bool before) -> cudaError_t {
        if (before) return cudaMemsetAsync(flush, 0, flush_bytes, st);
        launch_alloc_probe(m, f, depth, cam, run, ctx_flags(s->ctx), st, i);
        return cudaSuccess;
      }, rep.alloc_ms[i]);
      rep.alloc_tile_x[i] = alloc_tile(i).x;
      rep.alloc_tile_y[i] = alloc_tile(i).y;
      if (rep.alloc_ms[i] < rep.alloc_ms[abest]) abest = i;
    }
    rep.alloc_chosen = abest;
  }
  // the frame's state back
  if (e == cudaSuccess && fuse) launch_save_visible(m, save, nvis, true, st);
  if (e == cudaSuccess) launch_raycast(m, f, mv, mn, zmin, zmax, cam, f.counters + 3, &fv, &fn, run, st, s->rc_tune);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(save);
  cudaFree(flush);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return SF_ERR_CUDA;
  }
  sf_frame_tune tune;
  tune.raycast = best;
  tune.integrate_ctas_per_sm = fuse ? kIntCtas[ibest] : s->int_ctas;
  tune.alloc_tile = abest;
  const int r = sf_system_set_tune(s, &tune);
  if (report) *report = rep;
  return r;
}

int sf_system_get_tune(sf_system *s, sf_frame_tune *t) {
  if (!s || !t) return SF_ERR_INVALID;
  t->raycast = s->rc_index;
  t->integrate_ctas_per_sm = s->int_ctas;
  t->alloc_tile = s->alloc_tile;
  return SF_OK;
}

int sf_system_set_tune(sf_system *s, const sf_frame_tune *t) {
  if (!s || !t || t->raycast < 0 || t->raycast >= kRaycastTunes || t->integrate_ctas_per_sm < 1 ||
      t->integrate_ctas_per_sm > 64 || t->alloc_tile < 0 || t->alloc_tile >= kAllocTileCount)
    return SF_ERR_INVALID;
  const RaycastTune rt = raycast_tune(t->raycast);
  const bool changed = rt.minb != s->rc_tune.minb || rt.tx != s->rc_tune.tx || rt.ty != s->rc_tune.ty ||
                       t->integrate_ctas_per_sm != s->int_ctas || t->alloc_tile != s->alloc_tile;
  s->rc_tune = rt;
  s->rc_index = t->raycast;
  s->int_ctas = t->integrate_ctas_per_sm;
  s->alloc_tile = t->alloc_tile;
  if (changed && s->gexec) {  // recaptured with the new shapes on the next frame
    cudaGraphExecDestroy(s->gexec);
    s->gexec = nullptr;
  }
  return SF_OK;
}

int sf_system_stats(sf_system *s, sf_frame_stats *stats) {
  if (!s || !stats) return SF_ERR_INVALID;
  cudaStream_t st = ctx_stream(s->ctx);
  if (cudaMemcpyAsync(s->h_stats, s->d_stats, sizeof(sf_frame_stats), cudaMemcpyDeviceToHost, st) !=
          cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return SF_ERR_CUDA;
  *stats = *s->h_stats;
  return SF_OK;
}

int sf_system_model_maps(sf_system *s, int level, sf_image *vmap, sf_image *nmap) {
  if (!s || level < 0 || level >= s->L || !vmap || !nmap) return SF_ERR_INVALID;
  const int c = s->cfg.cols >> level, r = s->cfg.rows >> level;
  *vmap = img(s->d_mv[level], c, r, 16);
  *nmap = img(s->d_mn[level], c, r, 16);
  return SF_OK;
}

int sf_system_frame_maps(sf_system *s, int level, sf_image *vmap, sf_image *nmap, sf_image *depth) {
  if (!s || level < 0 || level >= s->L) return SF_ERR_INVALID;
  const int c = s->cfg.cols >> level, r = s->cfg.rows >> level;
  if (vmap) *vmap = img(s->d_vmap[level], c, r, 16);
  if (nmap) *nmap = img(s->d_nmap[level], c, r, 16);
  if (depth) *depth = img(s->d_depth[level], c, r, 4);
  return SF_OK;
}

int sf_system_set_timing(sf_system *s, int enable) {
  if (!s) return SF_ERR_INVALID;
  if (enable && s->cfg.use_graph == 1) return SF_ERR_STATE;  // events are not captured
  if (enable && !s->ev[0])
    for (auto &e : s->ev)
      if (cudaEventCreate(&e) != cudaSuccess) return SF_ERR_CUDA;
  s->timing = enable ? 1 : 0;
  return SF_OK;
}

int sf_system_stage_ms(sf_system *s, float ms[7]) {
  if (!s || !ms || !s->timing) return SF_ERR_INVALID;
  if (cudaEventSynchronize(s->ev[7]) != cudaSuccess) return SF_ERR_CUDA;
  for (int i = 0; i < 7; ++i)
    if (cudaEventElapsedTime(&ms[i], s->ev[i], s->ev[i + 1]) != cudaSuccess) return SF_ERR_CUDA;
  return SF_OK;
}

int sf_system_get_map(sf_system *s, sf_map **map) {
  if (!s || !map) return SF_ERR_INVALID;
  *map = s->map;
  return SF_OK;
}

int sf_system_pose_device(sf_system *s, double **last_pose) {
  if (!s || !last_pose) return SF_ERR_INVALID;
  *last_pose = dev_field<double>(s->d_sys, offsetof(SysDev, last_pose));
  return SF_OK;
}

}  // extern "C"
