// ORACLE — test infrastructure only (tests/, __graft_entry__.smoke() and
// bench.py's CPU-baseline leg).  Nothing in semantic_icpslam_gb300/ links,
// loads or calls this code.
//
// CPU restatement of YuhangMing/semantic_icpSLAM's dense per-frame
// tracking-and-fusion loop.  Every function cites the reference file:line it
// follows.  Arithmetic is strict IEEE-754 per operation (built with
// -ffp-contract=off): FP32 where the reference computes in float, FP64 where
// the reference promotes to double; the "fp64" variants compute everything in
// double and serve as the error-budget oracle.
#ifndef SFO_H_
#define SFO_H_
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { int x, y, z, ptr, offset, pad_[3]; } sfo_entry;   // 32 B
typedef struct {
  float sdf; uint8_t weight; uint8_t color[3];
  uint8_t label, count, label_2, count_2; uint8_t color_2[3]; uint8_t obj_idx;
} sfo_voxel;                                                        // 16 B

typedef struct {
  float voxel_size, trunc_dist, depth_min, depth_max;
  uint32_t num_buckets, num_excess, num_sdf_blocks, max_rendering_blocks;
} sfo_config;

typedef struct sfo_map sfo_map;

// ---- pyramid (Tracking/Pyrdown.cu) ----
void sfo_filter_depth(const uint16_t *d, int cols, int rows, float depth_scale,
                      float cutoff, float *raw, float *filtered);
void sfo_pyrdown(const float *src, int sc, int sr, float *dst, int dc, int dr);
void sfo_vmap(const float *depth, int cols, int rows, float fx, float fy,
              float cx, float cy, float cutoff, float *vmap);
void sfo_nmap(const float *vmap, int cols, int rows, float *nmap);
void sfo_resize(const float *vsrc, const float *nsrc, int sc, int sr,
                float *vdst, float *ndst, int dc, int dr);

// ---- ICP (Tracking/Reduction.cu) ----
// R* are row-major 3x3 float; t* are float[3].  out[29] in double.
// fp64 != 0 computes the per-pixel terms in double (error-budget oracle).
void sfo_icp_sums(const float *vcurr, const float *vlast, const float *ncurr,
                  const float *nlast, int cols, int rows, const float *Rcurr,
                  const float *tcurr, const float *Rlast, const float *RlastInv,
                  const float *tlast, float fx, float fy, float cx, float cy,
                  int fp64, double *out29);
// Per-pixel rows (29 floats per pixel) in FP32 reference semantics.
void sfo_icp_rows(const float *vcurr, const float *vlast, const float *ncurr,
                  const float *nlast, int cols, int rows, const float *Rcurr,
                  const float *tcurr, const float *Rlast, const float *RlastInv,
                  const float *tlast, float fx, float fy, float cx, float cy,
                  float *rows29);
// CreateMatrix<6,7> (Reduction.cu:6-16) from 29 sums.
void sfo_create_matrix(const double *sums29, double *A36, double *b6);
// LDLT solve (Eigen semantics, Tracking.cc:493) and SE3 exp (Sophus, :494).
void sfo_ldlt_solve6(const double *A36, const double *b6, double *x6);
void sfo_se3_exp(const double *xi6, double *T16);
// Tracker::ComputeSE3, icpOnly (Tracking.cc:369-517).
// levels vmaps/nmaps (float4) for next & last frames; poses row-major 4x4.
// Returns 1 if accepted; next_pose is updated in place (rolled back on
// failure exactly as the reference does).  stats[4] = {icpError, count,
// iterations run, failure code}.
int sfo_compute_se3(int levels, const int *cols, const int *rows,
                    const float *const *vnext, const float *const *nnext,
                    const float *const *vlast, const float *const *nlast,
                    const float *K /*fx,fy,cx,cy level 0*/, const int *iters,
                    const int *min_count, float thresh, const double *last_pose,
                    double *next_pose, int fp64, double *stats);

// ---- photometric term (Pyrdown.cu:201-316, Reduction.cu:387-642) ----
void sfo_intensity(const uint8_t *rgb, int cols, int rows, uint8_t *out);
void sfo_pyrdown_u8(const uint8_t *src, int sc, int sr, uint8_t *dst, int dc, int dr);
void sfo_sobel(const uint8_t *img, int cols, int rows, int16_t *dx, int16_t *dy);
// RGBStep at the 4x4 poses Pc (current estimate) and Pl (last frame):
// out29 sums, res2 = {count, sum of diff^2}, sigma; rows29 (optional) the
// per-pixel FP32 29-vectors.  fp64 != 0 computes the rows in double.
void sfo_rgb_step(const uint8_t *inext, const uint8_t *ilast, const float *vnext,
                  const float *vlast, const int16_t *dIdx, const int16_t *dIdy,
                  int cols, int rows, const double *Pc, const double *Pl, float fx,
                  float fy, float cx, float cy, int fp64, double *out29, int *res2,
                  float *sigma, float *rows29);
// ComputeSE3 with the photometric term when inext != NULL (icpOnly = false);
// stats[6] then ends with {rgbError, rgbCount}.
int sfo_compute_se3_ex(int levels, const int *cols, const int *rows,
                       const float *const *vnext, const float *const *nnext,
                       const float *const *vlast, const float *const *nlast,
                       const uint8_t *const *inext, const uint8_t *const *ilast,
                       const int16_t *const *dIdx, const int16_t *const *dIdy,
                       const float *K, const int *iters, const int *min_count,
                       float thresh, const double *last_pose, double *next_pose,
                       int fp64, double *stats);

// ---- marching cubes (Mapping/MeshScene.cu) ----
// The triangle / vertex-count / edge tables of this restatement's rule.
void sfo_mc_tables(int *tri4096, int *nverts256, int *edges256);

// ---- map (Mapping/DeviceMap.cu, FuseMap.cu, RenderScene.cu) ----
sfo_map *sfo_map_create(const sfo_config *cfg);
void sfo_map_destroy(sfo_map *m);
void sfo_map_reset(sfo_map *m);
sfo_entry *sfo_map_entries(sfo_map *m);
// Sets the visible count a state loaded into the map's arrays carries.
void sfo_map_set_no_visible(sfo_map *m, unsigned n);
sfo_voxel *sfo_map_voxels(sfo_map *m);
sfo_entry *sfo_map_visible(sfo_map *m);
int *sfo_map_heap(sfo_map *m);
// {heapCounter, entryPtr, noVisible, allocated}
void sfo_map_counters(sfo_map *m, int *out4);
// Pose as R (row-major 3x3 float, world<-camera), Rinv, t (float[3]).
void sfo_alloc(sfo_map *m, const float *depth, int cols, int rows,
               const float *R, const float *t, float fx, float fy, float cx,
               float cy);
unsigned sfo_visibility(sfo_map *m, const float *R, const float *Rinv,
                        const float *t, int cols, int rows, float fx, float fy,
                        float cx, float cy, float depth_max, float depth_min);
void sfo_integrate(sfo_map *m, const float *depth, const uint8_t *rgb, int cols,
                   int rows, const float *Rinv, const float *t, float fx,
                   float fy, float cx, float cy, float depth_max,
                   float depth_min);
void sfo_semantics(sfo_map *m, const float *depth, const uint8_t *rgb,
                   const float *nmap, const uint8_t *mask, int num_detection,
                   int cols, int rows, const float *Rinv, const float *t,
                   float fx, float fy, float cx, float cy, float depth_max,
                   float depth_min);
// MeshScene's marching cubes over the allocated entries in table order:
// up to max_tri triangles, 9 floats of vertices and of normals and 9 bytes
// of colour each.  Returns the triangle count.
unsigned sfo_mesh(sfo_map *m, unsigned max_tri, float *vert, float *nrm, uint8_t *col);
// Fusion::UnifyNeighbor over hash entries [0, noVisible) (FuseMap.cu:757-896).
void sfo_unify_neighbor(sfo_map *m);
// FuseMapColor order (FuseMap.cu:1039-1162): alloc, visibility, integrate,
// [semantics, and UnifyNeighbor when unify != 0].  Returns the visible count.
unsigned sfo_fuse(sfo_map *m, const float *depth, const uint8_t *rgb,
                  const float *nmap, const uint8_t *mask, int num_detection,
                  int cols, int rows, const float *R, const float *Rinv,
                  const float *t, float fx, float fy, float cx, float cy,
                  int unify);
// CreateRenderingBlocks (RenderScene.cu:210-289) into zmin/zmax images of
// zc x zr floats.  Returns the reference's bool.  blocks_out (optional,
// 4 shorts + 2 floats each) receives the rendering-block list; *nblocks the
// count.
int sfo_zrange(sfo_map *m, float *zmin, float *zmax, int zc, int zr,
               float depth_max, float depth_min, const float *Rinv,
               const float *t, float fx, float fy, float cx, float cy,
               void *blocks_out, int max_blocks, unsigned *nblocks);
// Raycast (RenderScene.cu:291-537).
void sfo_reloc_score(sfo_map *m, const float *vmap, int cols, int rows, int stride,
                     const float *poses, int n, float inlier_sdf, void *out);
double sfo_raycast_smooth_f64(sfo_map *m, const float *gv, const float *gn, int cols, int rows,
                              const float *zmin, const float *zmax, int zc, int zr, const double *T,
                              float invfx, float invfy, float cx, float cy, const double *xi,
                              long long vox, double delta);
void sfo_raycast(sfo_map *m, float *vmap, float *nmap, int cols, int rows,
                 const float *zmin, const float *zmax, int zc, int zr,
                 const float *R, const float *Rinv, const float *t, float invfx,
                 float invfy, float cx, float cy);

// ---- whole loop (Core/System.cc:131-270, icp-only tracking) ----
typedef struct sfo_system sfo_system;
sfo_system *sfo_system_create(const sfo_config *cfg, int cols, int rows,
                              int levels, const float *K, float depth_scale,
                              float depth_cutoff, const int *iters,
                              const int *min_count, float icp_thresh,
                              const double *init_pose);
void sfo_system_destroy(sfo_system *s);
// on != 0: track with the photometric term (ComputeSE3(icpOnly = false),
// the reference's default, Tracking.cc:170).
void sfo_system_set_rgb(sfo_system *s, int on);
// on == 0: localisation mode (Tracker::mappingDisabled): UpdateVisibility
// and RayTrace instead of FuseColor, labels by AnalyzeMapSemantics on the
// rendered depth (System.cc:161-212).
void sfo_system_set_mapping(sfo_system *s, int on);
// Returns the tracking result (1 tracked / 0 lost); pose_out = the frame's
// pose after tracking; stats[8] = {icpError, count, iters, fail, visible,
// heapCounter, entryPtr, allocated}, with the photometric term
// stats[10] (stats[8..9] = {rgbError, rgbCount}).
int sfo_system_grab(sfo_system *s, const uint16_t *depth, const uint8_t *rgb,
                    const uint8_t *mask, int num_detection, double *pose_out,
                    double *stats);
sfo_map *sfo_system_map(sfo_system *s);
// Level-l maps of the "last" frame (the model prediction after raycast).
const float *sfo_system_vmap(sfo_system *s, int level);
const float *sfo_system_nmap(sfo_system *s, int level);

#ifdef __cplusplus
}
#endif
#endif
