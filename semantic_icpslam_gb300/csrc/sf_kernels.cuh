// Internal (C++) interface between the kernel files and the C ABI layer.
#ifndef SF_KERNELS_CUH_
#define SF_KERNELS_CUH_

#include "sf_device.cuh"
#include "sf_solve.h"

namespace sf {

constexpr int kMaxLevels = 4;

// ------------------------------------------------------------- pyramid
void launch_filter_depth(const sf_image &depth, const sf_image &raw, const sf_image &filt,
                         float depth_scale, float cutoff, cudaStream_t s);
void launch_pyrdown(const sf_image &src, const sf_image &dst, cudaStream_t s);
void launch_vnmap(const sf_image &depth, const sf_image &vmap, const sf_image &nmap, float fx,
                  float fy, float cx, float cy, float cutoff, cudaStream_t s);
void launch_vmap(const sf_image &depth, const sf_image &vmap, float fx, float fy, float cx,
                 float cy, float cutoff, cudaStream_t s);
void launch_nmap(const sf_image &vmap, const sf_image &nmap, cudaStream_t s);
// The z channel of a vertex map as a depth image (rendered depth).
void launch_vmap_depth(const sf_image &vmap, const sf_image &depth, const int *run_flag, cudaStream_t s);
void launch_resize(const sf_image &vsrc, const sf_image &nsrc, const sf_image &vdst,
                   const sf_image &ndst, cudaStream_t s);
// Two ResizeMap levels (0 -> 1 -> 2) in one launch, bit-identical to two
// launch_resize calls.
void launch_resize2(const sf_image &v0, const sf_image &n0, const sf_image &v1, const sf_image &n1,
                    const sf_image &v2, const sf_image &n2, cudaStream_t s);

// Levels 1..levels-1 of the pyramid from the filtered depths[0], and every
// level's vertex and normal maps, in one launch (2 <= levels <= kMaxLevels;
// the level sizes must halve (floor) and the maps match their depth).
// fx .. cy are level 0's intrinsics.
struct PyramidLevelK {
  float invfx, invfy, cx, cy;
};
struct PyramidArgs {
  sf_image depth[kMaxLevels], vmap[kMaxLevels], nmap[kMaxLevels];
  PyramidLevelK k[kMaxLevels];
  float cutoff;
};
bool pyramid_levels_fusable(const sf_image *depths, const sf_image *vmaps, const sf_image *nmaps, int levels);
void launch_pyramid_levels(const sf_image *depths, const sf_image *vmaps, const sf_image *nmaps, int levels,
                           float fx, float fy, float cx, float cy, float cutoff, cudaStream_t s);

// ----------------------------------------------------------------- ICP
struct IcpLevelArgs {
  sf_image vc, nc, vl, nl;   // current (measured) and last (model) maps
  float fx, fy, cx, cy;
  int iters, min_count;
};

// Photometric term of one level (RGBStep, Tracking/Reduction.cu:387-642):
// the next and last frames' intensities (uint8), the next frame's
// derivative images (int16) and candidate flags (uint8, see
// launch_derivatives), and the per-pixel correspondences of the current
// iteration (float4: the last frame's vertex in the current camera, and
// the intensity difference as int bits, INT_MIN when none).
struct RgbLevelArgs {
  sf_image inext, ilast, dx, dy, cand;
  float4 *corr;
};

struct IcpWorkspace {
  double *partials = nullptr;  // [2][29][max_blocks]
  double *sums = nullptr;      // [29] (photometric: [2][29], ICP then RGB)
  unsigned *barrier = nullptr; // persistent kernel: arrival count, then (at +256 B) fix
  unsigned long long *fix = nullptr;  // [3][8][29][4] fixed-point accumulators (sets, CTA groups)
  unsigned long long *fix_rgb = nullptr;  // the same for the photometric sums
  unsigned *rgb_res = nullptr;  // [3][8][2] correspondence count and sum of diff^2 (sets, groups)
  TrackCtl *ctl = nullptr;     // device copy of the tracking state
  int max_blocks = 0;          // co-resident CTAs of the persistent kernel
  int max_blocks_rgb = 0;      // the same for the photometric form
  int threads = 0;
  unsigned long long *prof = nullptr;  // [64][16] per-iteration phase clocks (sf_icp_profile)
  int profile = 0;                     // record phase clocks when set
  // grid barrier bounds of the persistent kernel (sf_icp_barrier_limits)
  unsigned barrier_poll_limit = 1u << 22;
  unsigned barrier_extra = 0;
  int predict = 1;  // next-pose prediction of the persistent kernel (sf_icp_predict)
  void *pub = nullptr;  // persistent kernel: the solving CTA's publications (inside barrier)
  // photometric scratch, grown on demand: correspondences of the largest
  // level, and candidate flags of every level for callers that pass none
  float4 *corr = nullptr;
  uint8_t *cand = nullptr;
  size_t rgb_pixels = 0;
};

// Grows the photometric scratch to `pixels` (level 0) pixels.
int icp_workspace_rgb(IcpWorkspace &w, size_t pixels);

// Photometric images (csrc/photometric.cu).  save (may be null) receives
// each pixel's previous value first when *save_flag is nonzero.
void launch_intensity(const sf_image &rgb, const sf_image &out, const sf_image *save, const int *save_flag,
                      cudaStream_t s);
void launch_pyrdown_u8(const sf_image &src, const sf_image &dst, const sf_image *save, const int *save_flag,
                       cudaStream_t s);
// Derivative images of every level in one launch; cand (may be null) gets
// the per-pixel flag of FindCorresp's pose-independent tests.
void launch_derivatives(const sf_image *img, const sf_image *dx, const sf_image *dy, const sf_image *cand,
                        int levels, cudaStream_t s);
void launch_intensity_pyramid(const sf_image &rgb, const sf_image *img, const sf_image *save,
                              const int *save_flag, const sf_image *dx, const sf_image *dy,
                              const sf_image *cand, int levels, cudaStream_t s);

int icp_workspace_init(IcpWorkspace &w);
void icp_workspace_free(IcpWorkspace &w);

// Plain form: one partial-sum launch + one reduction launch; the 29 FP64
// sums land in w.sums (device).  Pose given as float matrices.
void launch_icp_step(const IcpWorkspace &w, const IcpLevelArgs &L, const m3 &Rc, f3 tc,
                     const m3 &Rl, const m3 &RlInv, f3 tl, cudaStream_t s);

// Plain form of RGBStep: the correspondence pass (its count and sum of
// diff^2 land in w.rgb_res[0..1]), then, with sigma computed from them on
// the device, the 29 sums of the photometric rows in w.sums + 29.
void launch_rgb_step(const IcpWorkspace &w, const IcpLevelArgs &L, const RgbLevelArgs &R, const m3 &Rc,
                     const m3 &RcInv, f3 tc, const m3 &Rl, const m3 &RlInv, f3 tl, cudaStream_t s);
// Candidate flags of FindCorresp's pose-independent tests from an
// intensity image and its derivatives (callers that have none).
void launch_rgb_cand(const sf_image &inext, const sf_image &dx, const sf_image &dy, const sf_image &cand,
                     cudaStream_t s);

// Zeroes the persistent kernel's barrier count and accumulators (one memset);
// enqueue it before each launch_icp_persistent.
cudaError_t icp_persistent_reset(const IcpWorkspace &w, cudaStream_t s);

struct FramePost;        // sf_frame.cuh
struct FrameStatsArgs;   // sf_frame.cuh

// Persistent form: every level and iteration of Tracker::ComputeSE3 in one
// cooperative launch.  last_pose: device double[16]; result in *w.ctl.
// skip_flag (device int, may be null): when nonzero the kernel does nothing.
// rgb (may be null): per-level photometric inputs; then each iteration
// adds RGBStep's rows (ComputeSE3 with icpOnly = false).  post (may be
// null): the frame loop's state update after ComputeSE3 (sys_post), run by
// the kernel at its end, skipped or not.
cudaError_t launch_icp_persistent(const IcpWorkspace &w, const IcpLevelArgs *levels, int nlevels,
                                  float thresh, const double *last_pose, const int *skip_flag,
                                  uint32_t *flags, cudaStream_t s, const RgbLevelArgs *rgb = nullptr,
                                  const FramePost *post = nullptr);

// -------------------------------------------------------------- fusion
struct FuseScratch {
  // allocation requests (lock-free dedupe set keyed by epoch | block pos)
  unsigned long long *req_set = nullptr;  // [req_cap] (power of 2)
  uint32_t req_cap = 0;
  int4 *pending = nullptr;                // [pend_cap] {x, y, z, bucket}
  int *pending_next = nullptr;            // [pend_cap]
  uint32_t pend_cap = 0;
  int *bucket_head = nullptr;             // [num_buckets], -1 when idle
  int *dirty = nullptr;                   // [pend_cap] buckets with requests
  unsigned *counters = nullptr;           // [4] pending, dirty, epoch, any_rendered
  // Dense block-pointer window over the camera frustum's bounding box,
  // rebuilt with the visible set every frame: cell = the block's voxel
  // index (ptr) or -1.  win = {ox, oy, oz, nx, ny, nz}.  Lookups outside the
  // window go to the hash table, so the window only accelerates.
  int *win = nullptr;                     // [8]
  int *win_cells = nullptr;               // [win_cap]
  uint32_t win_cap = 0;
  // UnifyNeighbor's new {label, count, label_2, count_2} words, indexed like
  // the voxel array; allocated on the first pass with labels.
  uint32_t *unify_out = nullptr;          // [num_sdf_blocks * 512]
  int *unify_list = nullptr;              // [num_sdf_blocks] blocks of the pass (inside unify_out's allocation)
  unsigned *unify_count = nullptr;        // [1]
};

// Start of a frame's allocation pass: clears the per-frame counters and
// advances the request epoch (skipping 0, the empty-slot value).  Run by
// one thread before the probe pass.
__device__ __forceinline__ void alloc_frame_begin(const FuseScratch &f) {
  f.counters[0] = 0;
  f.counters[1] = 0;
  unsigned e = (f.counters[2] + 1u) & 0xffffu;
  if (e == 0) e = 1;
  f.counters[2] = e;
}


int fuse_scratch_init(FuseScratch &f, const MapConst &c, int max_pixels);
void fuse_scratch_free(FuseScratch &f);

struct Cam {
  m3 R, Rinv;
  f3 t;
  float fx, fy, cx, cy, invfx, invfy;
  int cols, rows;
  float dmin, dmax;
};

void launch_map_reset(const DevMap &m, cudaStream_t s);
void launch_rebuild_index(const DevMap &m, cudaStream_t s);
// Fusion::CreateBlocks (FuseMap.cu:92-132) as probe + insert passes.  With
// begin = false the caller has run alloc_frame_begin itself (in its own
// single-thread kernel, gated by the same run flag).
// tile: the probe's 256-thread pixel tile, kAllocTiles[tile] (every tile
// allocates the same blocks; sf_system_autotune times them).
constexpr int kAllocTileCount = 4;
struct AllocTile {
  int x, y;
};
AllocTile alloc_tile(int tile);
// The start of the next visibility pass run by the insert pass's launch
// (k_alloc_insert): on when vis_zmin / vis_zmax are given; the visibility
// pass is then launched with started = true.
struct VisStartArgs {
  int on;
  const Cam *cam;
  unsigned *rendered;
  sf_image zmin, zmax;
  int do_z;
};
void launch_alloc(const DevMap &m, const FuseScratch &f, const sf_image &depth, const Cam *c,
                  const int *run_flag, uint32_t *flags, cudaStream_t s, bool begin = true, int tile = 0,
                  const sf_image *vis_zmin = nullptr, const sf_image *vis_zmax = nullptr);
// The probe pass alone (no epoch start, no insert pass), for the autotuner.
void launch_alloc_probe(const DevMap &m, const FuseScratch &f, const sf_image &depth, const Cam *c,
                        const int *run_flag, uint32_t *flags, cudaStream_t s, int tile);
// CheckFullVisibility (FuseMap.cu:134-168) over the allocated-entry index.
// When zmin/zmax images are given, also lays down the z-range tiles of
// Projection + fillBlocks (RenderScene.cu:54-190) for each visible block.
void launch_visibility(const DevMap &m, const FuseScratch &f, const Cam *c, const sf_image *zmin,
                       const sf_image *zmax, const int *run_flag, uint32_t *flags,
                       cudaStream_t s, bool started = false);
// createVoxels (+ analyzeSemantics when mask != null), FuseMap.cu:432-668.
// MeshScene's marching cubes over the allocated blocks: up to max_tri
// triangles (3 vertices, normals, colours each) appended at *count.
void launch_mesh(const DevMap &m, float3 *vert, float3 *norm, uchar3 *col, uint32_t max_tri, uint32_t *count,
                 cudaStream_t s);
// Fusion::UnifyNeighbor over hash slots [0, *no_visible) from the pass-start
// state (three launches: the block list, the pass, the copy back); needs
// fuse_scratch_unify first.
int fuse_scratch_unify(FuseScratch &f, const MapConst &c);
void launch_unify_neighbor(const DevMap &m, const FuseScratch &f, const int *run_flag, cudaStream_t s);
// ctas_per_sm: the launch's CTAs per SM (grid-stride over the visible
// blocks; every shape computes the same voxels).
void launch_integrate(const DevMap &m, const sf_image &depth, const sf_image &rgb,
                      const sf_image *nmap, const sf_image *mask, int num_detection, const Cam *c,
                      bool integrate, bool semantics, const int *run_flag, cudaStream_t s, int ctas_per_sm = 8);
// Copies the voxels of visible blocks [0, nvis) to scratch (nvis x 8 KiB),
// or back with restore.
void launch_save_visible(const DevMap &m, void *scratch, unsigned nvis, bool restore, cudaStream_t s);
void launch_zrange_init(const sf_image &zmin, const sf_image &zmax, cudaStream_t s);

// -------------------------------------------------------------- raycast
// Projection over the visible list into a rendering-block list + fill.
void launch_rendering_blocks(const DevMap &m, uint32_t nvis, const sf_image &zmin,
                             sf_rendering_block *list, uint32_t *count, const Cam *c,
                             uint32_t *flags, cudaStream_t s);
void launch_fill_blocks(const sf_image &zmin, const sf_image &zmax,
                        const sf_rendering_block *list, uint32_t nblocks, cudaStream_t s);
// Rendering (RenderScene.cu:291-489).  fallback_v/n (may be null): when
// *rendered == 0 the output is a copy of the fallback maps (the reference
// skips the raycast and keeps the frame's own maps).
// Launch shape of the raycast: CTAs per SM the registers are sized for
// (minb) and the pixel tile of a 128-thread CTA.  Every shape computes the
// same maps; sf_system_autotune picks the fastest on the device at hand.
struct RaycastTune {
  int minb = 8;
  int tx = 8, ty = 16;
};
constexpr int kRaycastTunes = 6;
RaycastTune raycast_tune(int i);  // candidate i < kRaycastTunes; 0 is the default
// stats (may be null): the frame's statistics (sys_stats), written by the
// kernel's first thread before anything else.
void launch_raycast(const DevMap &m, const FuseScratch &f, const sf_image &vmap, const sf_image &nmap,
                    const sf_image &zmin, const sf_image &zmax, const Cam *c,
                    const unsigned *rendered, const sf_image *fallback_v,
                    const sf_image *fallback_n, const int *run_flag, cudaStream_t s,
                    const RaycastTune &tune = RaycastTune(), const FrameStatsArgs *stats = nullptr);
// RaycastAdjoint: gradients of launch_raycast's maps w.r.t. the pose (left
// se(3) perturbation, 6 doubles into pose_out) and TSDF values (added into
// grad_sdf, one float per voxel index; may be null).  pose_part holds
// raycast_adjoint_blocks() x 6 floats.
int raycast_adjoint_blocks(int cols, int rows);
void launch_raycast_adjoint(const DevMap &m, const FuseScratch &f, const sf_image &zmin, const sf_image &zmax,
                            const Cam *c, const sf_image &gv, const sf_image &gn, float *grad_sdf,
                            float *pose_part, double *pose_out, cudaStream_t s);
// Block-pointer window for camera c from the allocated-entry index (the
// per-frame path builds it inside launch_visibility).
void launch_window_build(const DevMap &m, const FuseScratch &f, const Cam *c, cudaStream_t s);

// ------------------------------------------------------ relocalisation
// n candidate poses (float rows R | t, 12 per pose) scored, each candidate
// over reloc_score_parts() CTAs whose partials go to part
// [n][reloc_score_parts()], then added in a fixed order into out.
int reloc_score_parts();
void launch_reloc_score(const DevMap &m, const sf_image &vmap, int stride, const float *poses, int n,
                        float inlier_sdf, sf_reloc_score *part, sf_reloc_score *out, cudaStream_t s);

// Tracker::ValidatePose (Tracking.cc:750-790) batched over n candidate
// poses (csrc/validate.cu).  The candidates' model maps and z-range images
// are stacked: candidate c's image of h rows is rows [c h, c h + h) of one
// tall image.  cams: n device cameras (Frame::GpuRotation of each pose).
//
// UpdateVisibility + CreateRenderingBlocks' z-range per candidate:
// vis[c] (zero on entry) gets the visible-block count, rendered[c] (zero
// on entry) is set when a block projected; zmin / zmax hold 100 / 0 on
// entry (launch_zrange_init on the tall images).
void launch_vp_visibility(const DevMap &m, const Cam *cams, int n, const sf_image &zmin, const sf_image &zmax,
                          int zr, unsigned *vis, unsigned *rendered, cudaStream_t s);
// Block-pointer window over the bounding box of every allocated block
// (box: device int[8] scratch), so the candidates' raycasts share one.
void launch_window_alloc_box(const DevMap &m, const FuseScratch &f, int *box, cudaStream_t s);
// Raycast of every candidate whose src[c] == c (drawn) into its rows of
// the tall level-0 model maps.
void launch_raycast_batch(const DevMap &m, const FuseScratch &f, const sf_image &vmap, const sf_image &nmap,
                          int rows, const sf_image &zmin, const sf_image &zmax, int zr, const Cam *cams, int n,
                          const int *src, cudaStream_t s);
// ResizeMap of every drawn candidate (src[c] == c) from its src_rows-row
// slice of the tall source maps into its dst_rows-row slice of the tall
// destination maps.
void launch_resize_batch(const sf_image &vsrc, const sf_image &nsrc, const sf_image &vdst, const sf_image &ndst,
                         int src_rows, int dst_rows, int n, const int *src, cudaStream_t s);
// One ComputeSE3 iteration of every evaluated candidate (src[c] != -2,
// ctl[c].stop == 0) at one level: mv / mn are the tall model maps of this
// level (candidate src[c]'s slice of `rows` rows), fv / fn the fallback
// model maps (src[c] == -1); vc / nc the frame's maps.
struct VpWorkspace;
void vp_workspace_free(VpWorkspace *w);
struct VpLevel {
  sf_image vc, nc, mv, mn, fv, fn;
  int rows;
  float fx, fy, cx, cy;
  int min_count;
};
int vp_icp_blocks(int pixels);  // CTAs per candidate of launch_vp_icp_partials
void launch_vp_icp_iteration(const VpLevel &L, const int *src, TrackCtl *ctl, double *part, int nb, int stride,
                             int n, cudaStream_t s);
// ComputeSE3's acceptance gate of every evaluated candidate.
void launch_vp_icp_finish(TrackCtl *ctl, const int *src, float thresh, int n, cudaStream_t s);

// Converts host map config into device constants (DeviceMap.h:166-189).
MapConst make_map_const(const sf_map_config &cfg);

// Process-wide count of kernel launches issued by this library (graph
// replays add the kernel nodes of the replayed graph).
void note_launch(unsigned long long n = 1);
unsigned long long launches_total();

}  // namespace sf
#endif
