/*
 * sfusion.h — C ABI of the GB300 (sm_103a) dense tracking-and-fusion loop.
 *
 * Every entry point is `extern "C"`, takes plain pointers / POD structs and
 * returns an int status (SF_OK == 0).  Device buffers are raw CUDA device
 * pointers; images are (data, step in bytes, cols, rows) like the reference's
 * pitched DeviceArray2D / PtrStepSz.  No torch or C++ types cross this line.
 *
 * Reference interfaces replaced (paths inside YuhangMing/semantic_icpSLAM):
 *   Tracking/Reduction.h    FilterDepth :18, ComputeVMap :22, ComputeNMap :26,
 *                           PyrDownGauss(float) :29, ResizeMap :40, ICPStep :74
 *   Mapping/RenderScene.h   ResetMap :3, Raycast :13, CreateRenderingBlocks :20,
 *                           CheckBlockVisibility :40, FuseMapColor :45,
 *                           AnalyzeMapSemantics :57
 *   Tracking/Tracking.cc    Tracker::ComputeSE3 :369-517 (whole ICP loop)
 *   Core/System.cc          System::GrabImage :131-270 (per-frame order)
 * Error convention: the reference prints and exit(0)s on a CUDA error
 * (Utility/SafeCall.h:13-16); here every call returns a status instead.
 */
#ifndef SFUSION_H_
#define SFUSION_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
enum {
  SF_OK = 0,
  SF_ERR_INVALID = 1,   /* bad argument / size / config                   */
  SF_ERR_CUDA = 2,      /* a CUDA runtime call failed                      */
  SF_ERR_OVERFLOW = 3,  /* a fixed-capacity list overflowed (counted)      */
  SF_ERR_TIMEOUT = 4,   /* a bounded device wait gave up                   */
  SF_ERR_NO_DEVICE = 5, /* no CUDA device                                  */
  SF_ERR_STATE = 6,     /* call not valid in the object's current state    */
  SF_ERR_TOO_LARGE = 7, /* input beyond a fixed buffer's stated maximum    */
  SF_ERR_IO = 8         /* a file could not be opened, read or written     */
};

/* ----------------------------------------------------------- POD layouts */
/* Matrix3f: three float3 rows, row-major (Utility/VectorMath.h:360-375). */
typedef struct { float x, y, z; } sf_float3;
typedef struct { sf_float3 rowx, rowy, rowz; } sf_mat3;
/* Intrinsics (Utility/Intrinsics.h:4-18); level l uses fx/2^l etc. */
typedef struct { float fx, fy, cx, cy; } sf_intrinsics;
/* Pitched 2-D image view (Utility/DeviceArray.h:31-42 PtrStepSz). */
typedef struct { void *data; size_t step; int cols, rows; } sf_image;

/* HashEntry, 32 bytes (Mapping/DeviceMap.h:20-60): int3 pos, int ptr
 * (voxel index = heap block * 512; -1 = free), int offset (1-based excess
 * link; 0 = end of chain), 12 bytes padding from __align__(16). */
typedef struct { int x, y, z, ptr, offset, pad_[3]; } sf_hash_entry;
/* Voxel, 16 bytes (Mapping/DeviceMap.h:63-123). */
typedef struct {
  float sdf;
  uint8_t weight;
  uint8_t color[3];
  uint8_t label, count, label_2, count_2;
  uint8_t color_2[3];
  uint8_t obj_idx;
} sf_voxel;
/* RenderingBlock, 16 bytes (Mapping/DeviceMap.h:11-18). */
typedef struct { int16_t ulx, uly, lrx, lry; float zmin, zmax; } sf_rendering_block;

/* Runtime replacement of DeviceMap's static constexpr constants
 * (Mapping/DeviceMap.h:166-189).  Derived constants are computed exactly
 * as the reference's constexpr expressions are. */
typedef struct {
  float voxel_size;          /* VoxelSize (m)                           */
  float trunc_dist;          /* TruncateDist (m)                        */
  float depth_min;           /* DepthMin (m)                            */
  float depth_max;           /* DepthMax (m)                            */
  uint32_t num_buckets;      /* NumBuckets                              */
  uint32_t num_excess;       /* NumExcess                               */
  uint32_t num_sdf_blocks;   /* NumSdfBlocks (heap capacity)            */
  uint32_t max_rendering_blocks; /* MaxRenderingBlocks                 */
} sf_map_config;

/* DeviceMap's arrays (Mapping/DeviceMap.h:191-198) as raw device pointers. */
typedef struct {
  int *heap_mem;               /* [num_sdf_blocks]                      */
  int *entry_ptr;              /* [1] next excess slot, starts at 1     */
  int *heap_counter;           /* [1] top of the free-block stack       */
  int *bucket_mutex;           /* [num_buckets]                         */
  sf_voxel *voxel_blocks;      /* [num_sdf_blocks * 512]                */
  uint32_t *no_visible_blocks; /* [1]                                   */
  sf_hash_entry *hash_entries; /* [num_buckets + num_excess]            */
  sf_hash_entry *visible_entries; /* [num_buckets + num_excess]         */
} sf_device_map;

typedef struct sf_context sf_context; /* stream + per-call scratch       */
typedef struct sf_map sf_map;         /* voxel-block hash map            */
typedef struct sf_system sf_system;   /* whole per-frame loop            */

/* ------------------------------------------------------------- context */
/* A context owns one non-default CUDA stream on the current device and
 * the scratch every launcher below needs.  Not thread-safe; one per host
 * thread.  (Reference: default stream + caller-owned DeviceArrays.) */
int sf_context_create(sf_context **out);
int sf_context_destroy(sf_context *ctx);
int sf_context_stream(sf_context *ctx, void **stream_out);
int sf_context_sync(sf_context *ctx);
/* Last device-side overflow / error flags recorded by the context. */
int sf_context_flags(sf_context *ctx, uint32_t *flags_out);
/* Process-wide number of kernels this library has launched (a CUDA-graph
 * replay counts the kernel nodes it runs). */
int sf_kernel_launches(uint64_t *out);
/* Tracing of the persistent ICP kernel: when enabled, the first pixel CTA
 * records SM clocks at five phase boundaries of each iteration (round
 * start, rows accumulated, block total written, grid barrier passed, sums
 * and the solving CTA's pose in hand) into slots 0-4 of 64 x 16 slots, the
 * global timer (ns) at the round start into slot 6, whether the rows came
 * from a predicted pose into slot 7 and the start of the rows after the
 * prediction into slot 14; the solving CTA records clocks inside the
 * iteration's solve into slots 8-13; out (may be NULL, else 64 * 16
 * values) receives them. */
int sf_icp_profile(sf_context *ctx, int enable, uint64_t *out);
/* Bounds of the persistent ICP kernel's grid barriers (a diagnostic hook
 * for testing failure detection; no counterpart in the reference).  Each
 * barrier polls an arrival count at most poll_limit times (0 restores the
 * default, 2^22, about a second) and waits for extra_arrivals arrivals
 * beyond the grid's (0 by default; a test sets it so that no wait can end).
 * A barrier that gives up records SF_FLAG_BARRIER_TIMEOUT, every CTA leaves
 * its iterations, the tracking fails, and sf_ComputeSE3 /
 * sf_ComputeSE3_rgbd return SF_ERR_TIMEOUT (sf_system_grab too, with the
 * frame's stats.fail = 3); the context stays usable.  Takes effect for
 * later launches (a frame graph captured before keeps its bounds). */
int sf_icp_barrier_limits(sf_context *ctx, uint32_t poll_limit, uint32_t extra_arrivals);
/* Next-pose prediction of the persistent ICP kernel (a diagnostic switch;
 * no counterpart in the reference; on by default).  One CTA runs each
 * iteration's FP64 solve while the others predict the float pose it will
 * give (FP32 / float-float arithmetic) and accumulate the next iteration's
 * rows on the prediction; the rows are kept only when the prediction
 * equals the float form of the solved FP64 pose in every bit, else they
 * are accumulated again on that pose.  Poses, sums and decisions are the
 * same with the prediction on or off; off, every iteration takes two grid
 * rounds (the solve, then the rows).  Takes effect for later launches (a
 * frame graph captured before keeps its setting).  Phase-clock slot 7 of
 * sf_icp_profile records per iteration whether its rows came from a
 * prediction. */
int sf_icp_predict(sf_context *ctx, int enable);
/* Copies `bytes` between any two host/device pointers (unified addressing)
 * on the context stream and waits for it. */
int sf_memcpy(sf_context *ctx, void *dst, const void *src, size_t bytes);

/* ----------------------------------------------------------------- map */
/* Mapping::Create (Mapping/Mapping.cc:11-51): allocates every map array. */
int sf_map_create(const sf_map_config *cfg, sf_map **out);
/* Wraps caller-owned arrays (a reference Mapping's DeviceArrays). */
int sf_map_wrap(const sf_map_config *cfg, const sf_device_map *arrays, sf_map **out);
int sf_map_destroy(sf_map *map);
int sf_map_arrays(const sf_map *map, sf_device_map *out);
/* Bounds-checked build (no counterpart in the reference, whose race
 * analysis would need a memory checker): the library built with
 * SF_BOUNDS_CHECK (semantic_icpslam_gb300/build.py, debug_bounds) checks
 * every hash-chain link and every block pointer taken from the table or the
 * block window before use; a bad one sets a bit in the map's status word
 * (SF_BOUND_CHAIN 1: a chain link beyond the table; SF_BOUND_PTR 2: a block
 * pointer outside the voxel array or not a multiple of 512) and the access
 * is skipped.  sf_map_bounds_status reads the word (always 0 in the
 * release build); sf_build_flags tells which build is loaded. */
#define SF_BUILD_BOUNDS_CHECK 1u
int sf_map_bounds_status(sf_context *ctx, const sf_map *map, uint32_t *out);
int sf_build_flags(uint32_t *out);
/* Rebuilds the allocated-entry index after the hash table was written
 * outside this library (e.g. a map loaded from disk). */
int sf_map_rebuild_index(sf_context *ctx, sf_map *map);
/* Host copies of the map's counters: heapCounter, entryPtr, visible count,
 * allocated (ptr >= 0) entry count. */
int sf_map_counters(sf_context *ctx, const sf_map *map, int out[4]);
/* map.bin, byte for byte as System::WriteMapToDisk writes it
 * (Core/System.cc:327-361, arrays of Mapping::DownloadToRAM,
 * Mapping/Mapping.cc:220-235): four ints NumSdfBlocks, NumBuckets,
 * NumVoxels, NumEntries; heapCounter, entryPtr (hashCounter), noVisibleBlocks;
 * heapMem, bucketMutex, the voxels (16 B each), hashEntries and
 * visibleEntries (32 B each); then the keypoint map (KeyMap::MaxKeys mutex
 * ints and KeyMap::maxEntries 288-byte SURF records), which this library
 * does not keep: it is written as a reset key map (mutexes -1, records
 * zero, so every key invalid). */
int sf_map_write(sf_context *ctx, const sf_map *map, const char *path);
/* System::ReadMapFromDisk (Core/System.cc:363-403): the dense part of a
 * map.bin into a map of the same sizes (header checked against the map's
 * config, else SF_ERR_INVALID); the keypoint section is skipped.  The
 * allocated-entry index is rebuilt.  SF_ERR_IO when the file cannot be
 * read or is shorter than the dense part. */
int sf_map_read(sf_context *ctx, sf_map *map, const char *path);

/* ResetMap (Mapping/RenderScene.h:3; FuseMap.cu:1251-1304). */
int sf_ResetMap(sf_context *ctx, sf_map *map);

/* ------------------------------------------------------------- pyramid */
/* FilterDepth (Tracking/Reduction.h:18; Pyrdown.cu:72-121).
 * depth: uint16; raw, filtered: float. */
int sf_FilterDepth(sf_context *ctx, sf_image depth, sf_image raw_depth,
                   sf_image filtered_depth, float depth_scale, float depth_cutoff);
/* ComputeVMap (Reduction.h:22; Pyrdown.cu:123-158). vmap: float4. */
int sf_ComputeVMap(sf_context *ctx, sf_image depth, sf_image vmap, float fx,
                   float fy, float cx, float cy, float depth_cutoff);
/* ComputeNMap (Reduction.h:26; Pyrdown.cu:160-192). */
int sf_ComputeNMap(sf_context *ctx, sf_image vmap, sf_image nmap);
/* PyrDownGauss, float overload (Reduction.h:29; Pyrdown.cu:201-236). */
int sf_PyrDownGauss(sf_context *ctx, sf_image src, sf_image dst);
/* ResizeMap (Reduction.h:40; Pyrdown.cu:318-358). */
int sf_ResizeMap(sf_context *ctx, sf_image vsrc, sf_image nsrc, sf_image vdst,
                 sf_image ndst);
/* Frame::FillImages depth part (Core/Frame.cc:68-92) fused: raw + filtered
 * depth, Gaussian levels, vertex and normal maps of `levels` levels.
 * depth_levels/vmaps/nmaps: arrays of `levels` images. */
int sf_BuildPyramid(sf_context *ctx, sf_image depth_u16, sf_image raw_depth,
                    const sf_image *depth_levels, const sf_image *vmaps,
                    const sf_image *nmaps, int levels, sf_intrinsics K0,
                    float depth_scale, float depth_cutoff);

/* ----------------------------------------------------------------- ICP */
/* ICPStep (Tracking/Reduction.h:74; Reduction.cu:213-385): one projective
 * point-to-plane step.  Writes residual[2] = {sum r^2, count},
 * matrixA[36] (row-major symmetric) and vectorB[6] to HOST memory.
 * Per-pixel terms FP32; block partials Kahan-compensated FP32; the
 * cross-block sum FP64. */
int sf_ICPStep(sf_context *ctx, sf_image next_vmap, sf_image last_vmap,
               sf_image next_nmap, sf_image last_nmap, sf_mat3 Rcurr,
               sf_float3 tcurr, sf_mat3 Rlast, sf_mat3 RlastInv,
               sf_float3 tlast, sf_intrinsics K, float residual[2],
               double matrixA[36], double vectorB[6]);

/* sf_ICPStep without any device allocation.  No counterpart in the
 * reference: it is for callers that cannot allocate device memory, such as
 * a host application whose allocator owns all device memory, or a
 * real-time loop that must not pay for cudaMalloc's implicit device
 * synchronisation.  Such callers cannot create an sf_context either, so
 * this call takes only a stream (a cudaStream_t; NULL = the legacy default
 * stream) and the same inputs and host outputs as sf_ICPStep.
 * Its scratch (one FP64 partial per CTA for each of the 29 sums, plus the
 * sums) is a fixed array of 464.25 KiB inside the library's device
 * image.  Every GPU that loads the library holds it until the process
 * exits.  Images of more than SF_ICP_STATIC_MAX_PIXELS pixels return
 * SF_ERR_TOO_LARGE before any GPU work.
 * The first call on each device looks up the array's device address.
 * Under CUDA's lazy module loading (the default since CUDA 12) that first
 * call, or any earlier first use of this library's kernels, also loads the
 * library's device image, which allocates device memory for its code and
 * this array once and may synchronise the device.  A caller that can allow
 * neither in its loop makes one warm-up call at initialisation (or sets
 * CUDA_MODULE_LOADING=EAGER); later calls allocate nothing.  Make that
 * first call before any stream capture.
 * All calls share the one array, so calls that overlap on the GPU (other
 * streams, other host threads) race and give wrong sums.  The call
 * synchronises `stream` before it returns. */
#define SF_ICP_STATIC_MAX_PIXELS 4194304 /* 2048 x 2048 */
int sf_ICPStep_static(void *stream, sf_image next_vmap, sf_image last_vmap,
                      sf_image next_nmap, sf_image last_nmap, sf_mat3 Rcurr,
                      sf_float3 tcurr, sf_mat3 Rlast, sf_mat3 RlastInv,
                      sf_float3 tlast, sf_intrinsics K, float residual[2],
                      double matrixA[36], double vectorB[6]);

/* Tracker::ComputeSE3(icpOnly = true, iter, thresh) (Tracking/Tracking.cc
 * :369-517) as ONE persistent cooperative launch: every level (coarse to
 * fine) and iteration, the divergence guard, the FP64 6x6 LDLT solve and
 * SE(3) update, and the acceptance gate, with no host round trip.
 * next_* / last_*: `levels` images each (level 0 first), float4.
 * last_pose: host double[16] (camera->world).  next_pose_out: host
 * double[16], rolled back to last_pose on failure as the reference does.
 * stats_out (may be NULL): {accepted, fail (0/1 count-NaN/2 diverged),
 * iterations, icp_count}; icp_error_out (may be NULL). */
int sf_ComputeSE3(sf_context *ctx, int levels, const sf_image *next_vmaps,
                  const sf_image *next_nmaps, const sf_image *last_vmaps,
                  const sf_image *last_nmaps, sf_intrinsics K0, const int *iters,
                  const int *min_count, float thresh, const double last_pose[16],
                  double next_pose_out[16], int stats_out[4], float *icp_error_out);

/* ----------------------------------------------------------------- mesh */
/* MeshScene (RenderScene.h:29; MeshScene.cu:299-356, Mapping::CreateModel
 * Mapping.cc:183-192): marching cubes over every allocated block.  Writes
 * up to max_triangles triangles, three vertices each, to DEVICE arrays:
 * vertices and normals float[3 * 3 * max_triangles] (metres, unit
 * normals), colors uint8[3 * 3 * max_triangles]; *num_triangles = the
 * triangles written.  Vertices, normals and colours are the reference's
 * per cube; each cube's polygons are those of the reference's tables, split
 * into triangles by this library's own rule (a fan from the polygon's
 * lowest edge).  Triangle order is not defined. */
int sf_MeshScene(sf_context *ctx, sf_map *map, float *vertices, float *normals,
                 uint8_t *colors, uint32_t max_triangles,
                 uint32_t *num_triangles);
/* System::WriteMeshToDisk (Core/System.cc:272-325): the mesh (DEVICE
 * arrays as sf_MeshScene writes them) as an ASCII PLY file, the reference's
 * layout. */
int sf_mesh_write_ply(sf_context *ctx, const char *path, const float *vertices,
                      const float *normals, const uint8_t *colors,
                      uint32_t num_triangles);

/* ----------------------------------------------------- photometric term */
/* ImageToIntensity (Tracking/Reduction.h:34; Pyrdown.cu:250-271): uchar3
 * colour -> uint8 intensity, (int)(0.2125 g + 0.7154 r + 0.0721 b) with the
 * reference's channel order. */
int sf_ImageToIntensity(sf_context *ctx, sf_image rgb, sf_image image);
/* PyrDownGauss(unsigned char) (Reduction.h:31; Pyrdown.cu:201-245). */
int sf_PyrDownGauss_u8(sf_context *ctx, sf_image src, sf_image dst);
/* ComputeDerivativeImage (Reduction.h:37; Pyrdown.cu:262-316): 3x3 Sobel
 * of a uint8 image into int16 dx, dy. */
int sf_ComputeDerivativeImage(sf_context *ctx, sf_image image, sf_image dx,
                              sf_image dy);
/* RGBStep (Reduction.h:81; Reduction.cu:561-642): the photometric rows of
 * one level.  Images uint8 (intensity), float4 (vertex maps), int16 (the
 * next frame's derivatives).  Writes residual = {sum of weighted squared
 * differences, correspondences}, matrixA[36] and vectorB[6] to HOST memory,
 * as ICPStep does.  Correspondences and sigma are exact; the sums agree
 * with the reference's to FP32 rounding. */
int sf_RGBStep(sf_context *ctx, sf_image next_image, sf_image last_image,
               sf_image next_vmap, sf_image last_vmap, sf_image dIdx,
               sf_image dIdy, sf_mat3 Rcurr, sf_mat3 RcurrInv, sf_mat3 Rlast,
               sf_mat3 RlastInv, sf_float3 tcurr, sf_float3 tlast,
               sf_intrinsics K, float residual[2], double matrixA[36],
               double vectorB[6]);
/* Tracker::ComputeSE3(icpOnly = false, ...) (Tracking/Tracking.cc:369-517),
 * the reference's default tracking: sf_ComputeSE3 with RGBStep run in every
 * iteration (its error and count tested first) and the solve of
 * A_rgb 1e-4 + A_icp.  Per level: the next and last intensity images and
 * the next frame's derivative images.  stats_out (may be NULL): {accepted,
 * fail, iterations, icp_count, rgb_count, 0}; errors_out (may be NULL):
 * {icp_error, rgb_error}. */
int sf_ComputeSE3_rgbd(sf_context *ctx, int levels, const sf_image *next_vmaps,
                       const sf_image *next_nmaps, const sf_image *last_vmaps,
                       const sf_image *last_nmaps, const sf_image *next_images,
                       const sf_image *last_images, const sf_image *next_dIdx,
                       const sf_image *next_dIdy, sf_intrinsics K0,
                       const int *iters, const int *min_count, float thresh,
                       const double last_pose[16], double next_pose_out[16],
                       int stats_out[6], float errors_out[2]);

/* --------------------------------------------------------------- fusion */
/* CheckBlockVisibility (RenderScene.h:40; FuseMap.cu:991-1037). */
int sf_CheckBlockVisibility(sf_context *ctx, sf_map *map, sf_mat3 Rview,
                            sf_mat3 RviewInv, sf_float3 tview, int cols,
                            int rows, float fx, float fy, float cx, float cy,
                            float depth_max, float depth_min,
                            uint32_t *host_data);
/* FuseMapColor (RenderScene.h:45; FuseMap.cu:1039-1162): allocate blocks
 * along each raw-depth ray, compact the visible blocks, integrate
 * TSDF/weight/colour and, when num_detection > 0, fuse labels from `mask`
 * and run the UnifyNeighbor pass (sf_UnifyNeighbor).
 * depth: float (raw metres), color: uchar3, nmap: float4, mask: uint8. */
int sf_FuseMapColor(sf_context *ctx, sf_map *map, sf_image depth,
                    sf_image color, sf_image nmap, sf_image mask,
                    int num_detection, sf_mat3 Rview, sf_mat3 RviewInv,
                    sf_float3 tview, float fx, float fy, float cx, float cy,
                    float depth_max, float depth_min, uint32_t *host_data);
/* AnalyzeMapSemantics (RenderScene.h:57; FuseMap.cu:1164-1247): visible
 * blocks, the label pass, then the UnifyNeighbor pass. */
int sf_AnalyzeMapSemantics(sf_context *ctx, sf_map *map, sf_image depth,
                           sf_image color, sf_image nmap, sf_image mask,
                           int num_detection, sf_mat3 Rview, sf_mat3 RviewInv,
                           sf_float3 tview, float fx, float fy, float cx,
                           float cy, float depth_max, float depth_min);
/* UnifyNeighborKernel (FuseMap.cu:757-896, launched at :1158-1160 and
 * :1244-1246): every labelled voxel (weight > 0) of the blocks in hash slots
 * [0, visible count of the map's last visibility pass) takes the label most
 * of its 26 neighbours carry.  Each voxel updates from the state at the
 * start of the pass (the reference's in-place kernel races with its own
 * neighbour reads).  The first call allocates 4 bytes per voxel of the
 * block pool as the pass's output buffer. */
int sf_UnifyNeighbor(sf_context *ctx, sf_map *map);
/* Mapping::SemanticAnalysis(const Frame *) (Mapping/Mapping.cc:99-123), the
 * localisation mode's label pass (System.cc:206-212): AnalyzeMapSemantics
 * on the rendered depth, the z channel of the raycast vertex map `vmap`,
 * with the raycast normals `nmap`. */
int sf_SemanticAnalysis(sf_context *ctx, sf_map *map, sf_image vmap,
                        sf_image color, sf_image nmap, sf_image mask,
                        int num_detection, sf_mat3 Rview, sf_mat3 RviewInv,
                        sf_float3 tview, float fx, float fy, float cx,
                        float cy);

/* -------------------------------------------------------------- raycast */
/* CreateRenderingBlocks (RenderScene.h:20; RenderScene.cu:210-289).
 * zrange_min/zrange_max: float images (cols/8 x rows/8 in the reference),
 * rendering_blocks: device array of max_rendering_blocks entries,
 * no_rendering_blocks: device uint32[1].  *ok_out = reference's bool. */
int sf_CreateRenderingBlocks(sf_context *ctx, sf_map *map, sf_image zrange_min,
                             sf_image zrange_max, float depth_max,
                             float depth_min, sf_rendering_block *rendering_blocks,
                             uint32_t *no_rendering_blocks, sf_mat3 RviewInv,
                             sf_float3 tview, uint32_t no_visible_blocks,
                             float fx, float fy, float cx, float cy, int *ok_out);
/* Raycast (RenderScene.h:13; RenderScene.cu:291-537). */
int sf_Raycast(sf_context *ctx, sf_map *map, sf_image vmap, sf_image nmap,
               sf_image zrange_min, sf_image zrange_max, sf_mat3 Rview,
               sf_mat3 RviewInv, sf_float3 tview, float invfx, float invfy,
               float cx, float cy);

/* RaycastAdjoint: gradient of sf_Raycast's outputs (same map, z-range,
 * pose and intrinsics) with respect to the camera pose and the TSDF values
 * the rendering read.  No kernel of the reference corresponds; the raycast
 * it differentiates is Rendering::operator() (RenderScene.cu:380-488).
 * grad_vmap / grad_nmap: float4 images of dL/d(vertex) and dL/d(normal)
 * (w ignored, NaN treated as 0; grad_nmap.data may be NULL).  Each ray is
 * marched again and its discrete outcome held fixed; the gradient flows
 * through the two refinement steps, the normal's six interpolations and
 * the ray's ends and direction.  grad_pose_out (host double[6]): dL/dxi for
 * T(xi) = exp(xi) T, T = [Rview | tview] camera -> world, xi = (rho, omega)
 * translation first, summed over pixels in a fixed order.  grad_sdf
 * (device, may be NULL): one float per voxel index (heap block * 512 +
 * local), ADDED to (float atomics, so the order of additions varies). */
int sf_RaycastAdjoint(sf_context *ctx, sf_map *map, sf_image zrange_min,
                      sf_image zrange_max, sf_mat3 Rview, sf_mat3 RviewInv,
                      sf_float3 tview, float invfx, float invfy, float cx,
                      float cy, sf_image grad_vmap, sf_image grad_nmap,
                      float *grad_sdf, double grad_pose_out[6]);

/* -------------------------------------------------------- relocalisation */
/* RelocScoreBatch: scores n candidate poses against one frame in a single
 * launch (no kernel of the reference corresponds; the reference relocalises
 * with SURF keypoints outside this loop).  poses: host double[n][16],
 * camera -> world as Tracker's poses are; vmap: the frame's float4 vertex
 * map in its camera frame (any pyramid level).  For every stride-th column
 * and row, a vertex moved into the map by a candidate is sampled with
 * readSdfInterped (Mapping/RenderScene.cu:310-343); a valid, finite sample
 * counts in `valid` and, when |sdf| < inlier_sdf (normalised TSDF), in
 * `inliers`.  sum_abs_sdf is summed in a fixed order (deterministic),
 * mean_abs_sdf = sum / valid (NaN when valid is 0).  scores_out: host [n].
 * 1 <= n <= 65536. */
typedef struct {
  uint32_t valid, inliers;
  float sum_abs_sdf, mean_abs_sdf;
} sf_reloc_score;
int sf_RelocScoreBatch(sf_context *ctx, sf_map *map, sf_image vmap, int stride,
                       const double *poses, int n, float inlier_sdf,
                       sf_reloc_score *scores_out);

/* Tracker::ValidatePose (Tracking/Tracking.cc:750-790) for n candidate
 * poses against one frame, batched into a few launches over all candidates.
 * For each candidate (host double[16], camera -> world): UpdateVisibility
 * at the pose (`visible`); when visible >= min_visible (512 in the
 * reference), RayTrace into the candidate's own model maps (`rendered`;
 * a candidate that draws nothing tracks, as in the reference, against the
 * maps of the closest earlier candidate that drew, else last_vmaps /
 * last_nmaps), ResizeMap, and ComputeSE3(icpOnly = true, iters, thresh)
 * from the pose (ITERATIONS_RELOC {3, 3, 2} and THRESH_ICP_RELOC 1e-3 in
 * the reference, Tracking.h:111,119) against the frame's next_vmaps /
 * next_nmaps (`levels` images each, level 0 first; float4).  out (host
 * [n]) gets each candidate's result; *chosen (may be NULL) the candidate
 * ValidatePose keeps, or -1: the first accepted one in candidate order
 * (the reference's cv::sortIdx of its N x 1 error matrix sorts each row,
 * so its index 0 always names the first).  The reference then runs the
 * full ComputeSE3 from that candidate's pose (not its refined pose).  The
 * map is read, not changed; its block-pointer window is rebuilt.
 * 1 <= n <= 65535; the call allocates its workspace on first use (about
 * 13 MB per candidate at 640x480) and synchronises the context stream. */
typedef struct {
  uint32_t visible;   /* UpdateVisibility's count at the candidate pose   */
  int rendered;       /* RayTrace drew this candidate's own model maps    */
  int evaluated;      /* visible >= min_visible: ComputeSE3 ran           */
  int accepted;       /* ComputeSE3 accepted the refined pose             */
  int fail;           /* 0 ok, 1 ICP count/NaN failure, 2 diverged        */
  int iterations;     /* ICP iterations run                               */
  float icp_error;    /* lastIcpError: sqrt(sum r^2) / count              */
  int icp_count;
  double pose[16];    /* NextFrame->pose after ComputeSE3 (the candidate
                         itself when rejected or not evaluated)           */
} sf_reloc_candidate;
int sf_ValidatePoseBatch(sf_context *ctx, sf_map *map, int levels,
                         const sf_image *next_vmaps, const sf_image *next_nmaps,
                         const sf_image *last_vmaps, const sf_image *last_nmaps,
                         sf_intrinsics K0, const double *poses, int n,
                         const int *iters, const int *min_count, float thresh,
                         uint32_t min_visible, sf_reloc_candidate *out,
                         int *chosen);

/* ------------------------------------------------------- whole frame loop */
/* System::GrabImage (Core/System.cc:131-270) with Tracker::GrabFrame /
 * Track / ComputeSE3(icpOnly) (Tracking/Tracking.cc:65-173,246-280,369-517),
 * Mapping::FuseColor and Mapping::RayTrace (Mapping/Mapping.cc:76-161).
 * Keyframes, SURF matching, relocalisation by features and the viewer are
 * not part of this loop. */
typedef struct {
  sf_map_config map;
  int cols, rows;          /* level-0 image size                          */
  int levels;              /* pyramid levels (<= 4; reference: 3)          */
  sf_intrinsics K;         /* level-0 intrinsics                           */
  float depth_scale;       /* raw depth units per metre                   */
  float depth_cutoff;      /* Frame::mDepthCutoff                          */
  int iters[4];            /* ICP iterations per level (level 0 first)     */
  int min_count[4];        /* MIN_ICP_COUNT per level                      */
  float icp_thresh;        /* THRESH_ICP_SE3                               */
  int zrange_cols;         /* z-range image (0: ceil(cols / 8))            */
  int zrange_rows;         /* z-range image (0: ceil(rows / 8))            */
  int use_graph;           /* 1: one CUDA graph per frame; 0: per launch  */
  int rgb_term;            /* 1: ComputeSE3(icpOnly = false), the
                              reference's default (Tracking.cc:170): RGBStep
                              beside ICPStep every iteration; 0: ICP only   */
} sf_system_config;

typedef struct {
  int tracked;             /* Track() result for this frame                */
  int accepted;            /* ComputeSE3 acceptance (1 on the first frame) */
  int fail;                /* 0 ok, 1 ICP count/NaN failure, 2 diverged,
                              3 a bounded device wait gave up (the grab
                              returns SF_ERR_TIMEOUT)                      */
  int iterations;          /* ICP iterations run                           */
  float icp_error;         /* sqrt(sum r^2) / count of the last iteration  */
  int icp_count;
  uint32_t visible;        /* visible blocks                               */
  int heap_counter;        /* DeviceMap heapCounter                        */
  int entry_ptr;           /* DeviceMap entryPtr                           */
  int allocated;           /* entries with ptr >= 0                        */
  uint32_t flags;          /* SF_FLAG_* overflow / timeout bits            */
  double pose[16];         /* camera->world pose after this frame          */
  float rgb_error;         /* photometric error of the last iteration      */
  int rgb_count;           /* photometric correspondences                  */
  int state;               /* Tracker state of the NEXT frame: 1 initialise,
                              0 track, -1 lost (Tracking.cc:65-119)        */
  int missed;              /* Tracker::noMissedFrames                      */
  int relocalised;         /* this frame was relocalised (Relocalise)      */
} sf_frame_stats;

int sf_system_create(sf_context *ctx, const sf_system_config *cfg,
                     const double init_pose[16], sf_system **out);
int sf_system_destroy(sf_system *sys);
/* One frame from HOST buffers: depth uint16[rows*cols], rgb uint8[rows*cols*3],
 * mask uint8[rows*cols] (may be NULL).  Copies in, runs the frame, copies
 * the stats (pose included) out.  Returns when the stats are final: in the
 * graph form (use_graph = 1) the frame's last raycast and ResizeMap may still
 * run on the context's stream, and work ordered on that stream (the next
 * frame, sf_memcpy, sf_context_sync) comes after them. */
int sf_system_grab(sf_system *sys, const uint16_t *depth, const uint8_t *rgb,
                   const uint8_t *mask, int num_detection, sf_frame_stats *stats);
/* One frame from DEVICE buffers (already resident); asynchronous on the
 * context stream.  Read results with sf_system_stats. */
int sf_system_grab_device(sf_system *sys, const uint16_t *depth, const uint8_t *rgb,
                          const uint8_t *mask, int num_detection);
int sf_system_stats(sf_system *sys, sf_frame_stats *stats);
/* Relocalisation candidates (Tracker::Relocalise, Tracking/Tracking.cc
 * :107-116, 560-790): host double[n][16] camera -> world poses, copied.
 * Track() counts frames in a row whose ComputeSE3 fails; after ten the
 * tracker is lost (stats.state == -1).  Every later frame that starts lost
 * and finds candidates registered runs Relocalise's validation as
 * sf_ValidatePoseBatch does, then the final ComputeSE3 from the candidate
 * it keeps; accepted, the frame is tracked and mapped (stats.relocalised).
 * The candidates stand in for the poses the reference estimates from SURF
 * matches, which are outside this loop.  Such frames run host-driven in
 * every form.  n = 0 clears the candidates (lost frames are then skipped).
 * With candidates registered, sf_system_grab_device reads the tracker state
 * back before each frame (a stream synchronisation). */
int sf_system_set_reloc_candidates(sf_system *sys, const double *poses, int n);
/* Device views of the model maps (the last frame's raycast prediction,
 * level l) and of the current frame's measured maps. */
int sf_system_model_maps(sf_system *sys, int level, sf_image *vmap, sf_image *nmap);
int sf_system_frame_maps(sf_system *sys, int level, sf_image *vmap, sf_image *nmap,
                         sf_image *depth);
int sf_system_get_map(sf_system *sys, sf_map **map);
/* Stage timing with CUDA events on the system's stream (eager device form,
 * use_graph == 2): ms[7] = pyramid, ICP, allocation, visibility + z-range,
 * integration, raycast, resize + stats of the last frame. */
/* Autotune (new entry point; no counterpart in the reference).  Times the
 * raycast of the last grabbed frame under each of its launch shapes
 * (registers sized for 8 or 6 CTAs per SM; 8x16, 16x8 or 32x4 pixel
 * tiles), reps launches each, on the system's stream, and keeps the
 * fastest for the following frames (a captured frame graph is re-captured).
 * Every shape computes the same maps, and the timing runs rewrite the same
 * model maps, so the loop's results do not change.  Needs one grabbed
 * frame; 1 <= reps <= 1000.  report (may be NULL) receives the timings. */
typedef struct {
  int candidates;
  int chosen;
  float ms[16];
  int minb[16], tile_x[16], tile_y[16];
  /* the integration's grid: CTAs per SM 2, 4, 8, 16, timed by rerunning
   * the last frame's integration from the visible voxels as they stand
   * (saved before and restored after each run, so the map is unchanged;
   * a workspace of 8 KiB per visible block is allocated for the call);
   * integrate_chosen = -1 when no block was visible */
  int integrate_candidates;
  int integrate_chosen;
  float integrate_ms[8];
  int integrate_ctas[8];
  /* the allocation walk's pixel tile (256 threads: 32x8, 64x4, 16x16,
   * 128x2), timed by rerunning the last frame's probe pass over its depth
   * and pose after the frame allocated (it finds every block and requests
   * none, so the map is unchanged); alloc_chosen = -1 when the last frame
   * was not mapped */
  int alloc_candidates;
  int alloc_chosen;
  float alloc_ms[8];
  int alloc_tile_x[8], alloc_tile_y[8];
} sf_autotune_report;
int sf_system_autotune(sf_system *sys, int reps, sf_autotune_report *report);
/* The frame's launch shapes: the raycast's (index of its candidate,
 * 0..5: registers for 8 or 6 CTAs per SM x tiles 8x16, 16x8, 32x4), the
 * integration's CTAs per SM (1..64) and the allocation walk's pixel tile
 * (0..3: 32x8, 64x4, 16x16, 128x2).  Every shape computes the same maps.
 * sf_system_autotune picks them on the device at hand; a caller that cached
 * a choice for a configuration sets it back with sf_system_set_tune (the
 * frame graph is captured again on the next frame). */
typedef struct {
  int raycast;
  int integrate_ctas_per_sm;
  int alloc_tile;
} sf_frame_tune;
int sf_system_get_tune(sf_system *sys, sf_frame_tune *tune);
int sf_system_set_tune(sf_system *sys, const sf_frame_tune *tune);
/* Tracker::mappingDisabled (Tracking.h:51, toggled by the viewer,
 * GUI/Viewer.cc:151-156): enabled = 0 switches the loop to localisation,
 * UpdateVisibility and RayTrace instead of FuseColor, and with detections
 * the rendered-depth label pass of sf_SemanticAnalysis (System.cc:161-212);
 * 1 switches back.  Takes effect on the next frame. */
int sf_system_set_mapping(sf_system *sys, int enabled);

int sf_system_set_timing(sf_system *sys, int enable);
int sf_system_stage_ms(sf_system *sys, float ms[7]);
/* Device pointers to the pose state: last (tracked) pose, double[16]. */
int sf_system_pose_device(sf_system *sys, double **last_pose);

#ifdef __cplusplus
}
#endif
#endif /* SFUSION_H_ */
