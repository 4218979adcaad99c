// C ABI: context, map, reference-shaped launchers and the per-frame system.
//
// The launchers keep the reference's argument meaning (Tracking/Reduction.h,
// Mapping/RenderScene.h) and return a status instead of exit(0)-ing
// (Utility/SafeCall.h:13-16).  Launchers whose reference version writes a
// host output (ICPStep, FuseMapColor, CheckBlockVisibility,
// CreateRenderingBlocks) synchronise the context stream; the others are
// asynchronous on it.  The context stream is a blocking stream, so work the
// caller issues on the legacy default stream orders after it, as the
// reference's default-stream cudaMemcpy calls expect.
#include <atomic>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "sf_kernels.cuh"

using namespace sf;

struct sf_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  IcpWorkspace icp;
  uint32_t *flags = nullptr;    // device [1]
  Cam *cam = nullptr;           // device camera for reference-shaped calls
  uint32_t *u32 = nullptr;      // device scratch [4]
  double *host_sums = nullptr;  // pinned [29]
  double *pose = nullptr;       // device [16]
  TrackCtl *host_ctl = nullptr; // pinned
  float *reloc_poses = nullptr;           // device [reloc_cap][12]
  sf_reloc_score *reloc_scores = nullptr; // device [reloc_cap]
  sf_reloc_score *reloc_part = nullptr;   // device [reloc_cap][reloc_score_parts()]
  int reloc_cap = 0;
  float *adj_part = nullptr;              // device [adj_cap][6] pose partials
  double *adj_pose = nullptr;             // device [6]
  int adj_cap = 0;
  float *rdepth = nullptr;                // device rendered depth (sf_SemanticAnalysis)
  size_t rdepth_px = 0;
  VpWorkspace *vp = nullptr;              // sf_ValidatePoseBatch's workspace
};

struct sf_map {
  sf_map_config cfg;
  DevMap d;
  bool owned = false;
  FuseScratch scratch;
  int scratch_pixels = 0;
};

namespace {

inline int cuda_ok(cudaError_t e) {
  if (e == cudaSuccess) return SF_OK;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return SF_ERR_NO_DEVICE;
  return SF_ERR_CUDA;
}
#define SF_CHECK(x)                     \
  do {                                  \
    cudaError_t _e = (x);               \
    if (_e != cudaSuccess) return cuda_ok(_e); \
  } while (0)

inline bool img_ok(const sf_image &im, size_t elem) {
  return im.data && im.cols > 0 && im.rows > 0 && im.step >= (size_t)im.cols * elem;
}

Cam make_cam(const sf_mat3 &R, const sf_mat3 &Rinv, const sf_float3 &t, float fx, float fy,
             float cx, float cy, int cols, int rows, float dmin, float dmax) {
  Cam c;
  c.R = to_m3(R);
  c.Rinv = to_m3(Rinv);
  c.t = to_f3(t);
  c.fx = fx; c.fy = fy; c.cx = cx; c.cy = cy;
  c.invfx = (float)(1.0 / (double)fx);  // Fusion: invfx = 1.0 / fx (FuseMap.cu:1072)
  c.invfy = (float)(1.0 / (double)fy);
  c.cols = cols; c.rows = rows;
  c.dmin = dmin; c.dmax = dmax;
  return c;
}

int upload_cam(sf_context *ctx, const Cam &c) {
  SF_CHECK(cudaMemcpyAsync(ctx->cam, &c, sizeof(Cam), cudaMemcpyHostToDevice, ctx->stream));
  return SF_OK;
}

int ensure_scratch(sf_map *m, int pixels) {
  if (m->scratch.req_set && pixels <= m->scratch_pixels) return SF_OK;
  cudaDeviceSynchronize();
  fuse_scratch_free(m->scratch);
  int st = fuse_scratch_init(m->scratch, m->d.c, pixels);
  m->scratch_pixels = pixels;
  return st;
}

bool valid_cfg(const sf_map_config *c) {
  return c && c->voxel_size > 0 && c->trunc_dist > 0 && c->depth_min > 0 &&
         c->depth_max > c->depth_min && c->num_buckets > 0 && c->num_sdf_blocks > 0 &&
         c->num_excess > 0 && c->max_rendering_blocks > 0 &&
         (uint64_t)c->num_buckets + c->num_excess < (1ull << 31) &&
         (uint64_t)c->num_sdf_blocks * 512ull < (1ull << 31);
}

}  // namespace

extern "C" {

// ------------------------------------------------------------- context
int sf_context_create(sf_context **out) {
  if (!out) return SF_ERR_INVALID;
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) return SF_ERR_NO_DEVICE;
  sf_context *c = new (std::nothrow) sf_context();
  if (!c) return SF_ERR_INVALID;
  cudaGetDevice(&c->device);
  int st = SF_OK;
  if (cudaStreamCreate(&c->stream) != cudaSuccess) st = SF_ERR_CUDA;
  if (st == SF_OK) st = icp_workspace_init(c->icp);
  if (st == SF_OK && cudaMalloc(&c->flags, sizeof(uint32_t)) != cudaSuccess) st = SF_ERR_CUDA;
  if (st == SF_OK && cudaMemset(c->flags, 0, sizeof(uint32_t)) != cudaSuccess) st = SF_ERR_CUDA;
  if (st == SF_OK && cudaMalloc(&c->cam, sizeof(Cam)) != cudaSuccess) st = SF_ERR_CUDA;
  if (st == SF_OK && cudaMalloc(&c->u32, 4 * sizeof(uint32_t)) != cudaSuccess) st = SF_ERR_CUDA;
  if (st == SF_OK && cudaMallocHost(&c->host_sums, 29 * sizeof(double)) != cudaSuccess) st = SF_ERR_CUDA;
  if (st == SF_OK && cudaMalloc(&c->pose, 16 * sizeof(double)) != cudaSuccess) st = SF_ERR_CUDA;
  if (st == SF_OK && cudaMallocHost(&c->host_ctl, sizeof(TrackCtl)) != cudaSuccess) st = SF_ERR_CUDA;
  if (st != SF_OK) {
    sf_context_destroy(c);
    return st;
  }
  *out = c;
  return SF_OK;
}

int sf_context_destroy(sf_context *ctx) {
  if (!ctx) return SF_ERR_INVALID;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  icp_workspace_free(ctx->icp);
  cudaFree(ctx->flags);
  cudaFree(ctx->cam);
  cudaFree(ctx->u32);
  if (ctx->host_sums) cudaFreeHost(ctx->host_sums);
  cudaFree(ctx->pose);
  if (ctx->host_ctl) cudaFreeHost(ctx->host_ctl);
  cudaFree(ctx->reloc_poses);
  cudaFree(ctx->reloc_scores);
  cudaFree(ctx->reloc_part);
  cudaFree(ctx->adj_part);
  cudaFree(ctx->adj_pose);
  cudaFree(ctx->rdepth);
  vp_workspace_free(ctx->vp);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return SF_OK;
}

int sf_context_stream(sf_context *ctx, void **stream_out) {
  if (!ctx || !stream_out) return SF_ERR_INVALID;
  *stream_out = (void *)ctx->stream;
  return SF_OK;
}

int sf_context_sync(sf_context *ctx) {
  if (!ctx) return SF_ERR_INVALID;
  SF_CHECK(cudaStreamSynchronize(ctx->stream));
  return SF_OK;
}

int sf_context_flags(sf_context *ctx, uint32_t *flags_out) {
  if (!ctx || !flags_out) return SF_ERR_INVALID;
  SF_CHECK(cudaMemcpyAsync(flags_out, ctx->flags, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
  SF_CHECK(cudaStreamSynchronize(ctx->stream));
  return SF_OK;
}

int sf_icp_barrier_limits(sf_context *ctx, uint32_t poll_limit, uint32_t extra_arrivals) {
  if (!ctx || extra_arrivals > 65536) return SF_ERR_INVALID;
  ctx->icp.barrier_poll_limit = poll_limit ? poll_limit : (1u << 22);
  ctx->icp.barrier_extra = extra_arrivals;
  return SF_OK;
}

int sf_icp_predict(sf_context *ctx, int enable) {
  if (!ctx) return SF_ERR_INVALID;
  ctx->icp.predict = enable ? 1 : 0;
  return SF_OK;
}

int sf_icp_profile(sf_context *ctx, int enable, uint64_t *out) {
  if (!ctx) return SF_ERR_INVALID;
  ctx->icp.profile = enable ? 1 : 0;
  if (out) {
    SF_CHECK(cudaMemcpyAsync(out, ctx->icp.prof, sizeof(uint64_t) * 64 * 16, cudaMemcpyDeviceToHost,
                             ctx->stream));
    SF_CHECK(cudaStreamSynchronize(ctx->stream));
  }
  return SF_OK;
}

int sf_kernel_launches(uint64_t *out) {
  if (!out) return SF_ERR_INVALID;
  *out = (uint64_t)launches_total();
  return SF_OK;
}

int sf_memcpy(sf_context *ctx, void *dst, const void *src, size_t bytes) {
  if (!ctx || (!dst && bytes) || (!src && bytes)) return SF_ERR_INVALID;
  if (bytes == 0) return SF_OK;
  SF_CHECK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, ctx->stream));
  SF_CHECK(cudaStreamSynchronize(ctx->stream));
  return SF_OK;
}

// ----------------------------------------------------------------- map
static int map_alloc_index(sf_map *m) {
  const size_t ne = m->d.c.num_entries;
  SF_CHECK(cudaMalloc(&m->d.alloc_list, sizeof(int) * ne));
  SF_CHECK(cudaMalloc(&m->d.alloc_count, sizeof(int)));
  SF_CHECK(cudaMemset(m->d.alloc_count, 0, sizeof(int)));
  SF_CHECK(cudaMalloc(&m->d.status, sizeof(uint32_t)));
  SF_CHECK(cudaMemset(m->d.status, 0, sizeof(uint32_t)));
  return SF_OK;
}

int sf_map_create(const sf_map_config *cfg, sf_map **out) {
  if (!out || !valid_cfg(cfg)) return SF_ERR_INVALID;
  *out = nullptr;
  sf_map *m = new (std::nothrow) sf_map();
  if (!m) return SF_ERR_INVALID;
  m->cfg = *cfg;
  m->owned = true;
  m->d.c = make_map_const(*cfg);
  const size_t ne = m->d.c.num_entries, nb = cfg->num_buckets, nsb = cfg->num_sdf_blocks;
  int st = SF_OK;
  auto alloc = [&](void **p, size_t bytes) {
    if (st == SF_OK && cudaMalloc(p, bytes) != cudaSuccess) st = SF_ERR_CUDA;
  };
  alloc((void **)&m->d.entries, sizeof(sf_hash_entry) * ne);
  alloc((void **)&m->d.visible, sizeof(sf_hash_entry) * ne);
  alloc((void **)&m->d.voxels, sizeof(sf_voxel) * nsb * 512);
  alloc((void **)&m->d.heap, sizeof(int) * nsb);
  alloc((void **)&m->d.heap_counter, sizeof(int));
  alloc((void **)&m->d.entry_ptr, sizeof(int));
  alloc((void **)&m->d.bucket_mutex, sizeof(int) * nb);
  alloc((void **)&m->d.no_visible, sizeof(uint32_t));
  if (st == SF_OK) st = map_alloc_index(m);
  // voxels start zeroed once so obj_idx (never written by the loop) is 0
  if (st == SF_OK && cudaMemset(m->d.voxels, 0, sizeof(sf_voxel) * nsb * 512) != cudaSuccess) st = SF_ERR_CUDA;
  if (st == SF_OK) {
    launch_map_reset(m->d, 0);
    if (cudaDeviceSynchronize() != cudaSuccess) st = SF_ERR_CUDA;
  }
  if (st != SF_OK) {
    sf_map_destroy(m);
    return st;
  }
  *out = m;
  return SF_OK;
}

int sf_map_wrap(const sf_map_config *cfg, const sf_device_map *a, sf_map **out) {
  if (!out || !a || !valid_cfg(cfg)) return SF_ERR_INVALID;
  if (!a->heap_mem || !a->entry_ptr || !a->heap_counter || !a->bucket_mutex || !a->voxel_blocks ||
      !a->no_visible_blocks || !a->hash_entries || !a->visible_entries)
    return SF_ERR_INVALID;
  *out = nullptr;
  sf_map *m = new (std::nothrow) sf_map();
  if (!m) return SF_ERR_INVALID;
  m->cfg = *cfg;
  m->owned = false;
  m->d.c = make_map_const(*cfg);
  m->d.entries = a->hash_entries;
  m->d.visible = a->visible_entries;
  m->d.voxels = a->voxel_blocks;
  m->d.heap = a->heap_mem;
  m->d.heap_counter = a->heap_counter;
  m->d.entry_ptr = a->entry_ptr;
  m->d.bucket_mutex = a->bucket_mutex;
  m->d.no_visible = a->no_visible_blocks;
  int st = map_alloc_index(m);
  if (st == SF_OK) {
    launch_rebuild_index(m->d, 0);
    if (cudaDeviceSynchronize() != cudaSuccess) st = SF_ERR_CUDA;
  }
  if (st != SF_OK) {
    sf_map_destroy(m);
    return st;
  }
  *out = m;
  return SF_OK;
}

int sf_map_destroy(sf_map *m) {
  if (!m) return SF_ERR_INVALID;
  cudaDeviceSynchronize();
  if (m->owned) {
    cudaFree(m->d.entries);
    cudaFree(m->d.visible);
    cudaFree(m->d.voxels);
    cudaFree(m->d.heap);
    cudaFree(m->d.heap_counter);
    cudaFree(m->d.entry_ptr);
    cudaFree(m->d.bucket_mutex);
    cudaFree(m->d.no_visible);
  }
  cudaFree(m->d.alloc_list);
  cudaFree(m->d.alloc_count);
  cudaFree(m->d.status);
  fuse_scratch_free(m->scratch);
  delete m;
  return SF_OK;
}

int sf_map_bounds_status(sf_context *ctx, const sf_map *m, uint32_t *out) {
  if (!ctx || !m || !out) return SF_ERR_INVALID;
  SF_CHECK(cudaMemcpyAsync(out, m->d.status, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
  SF_CHECK(cudaStreamSynchronize(ctx->stream));
  return SF_OK;
}

int sf_build_flags(uint32_t *out) {
  if (!out) return SF_ERR_INVALID;
#ifdef SF_BOUNDS_CHECK
  *out = SF_BUILD_BOUNDS_CHECK;
#else
  *out = 0;
#endif
  return SF_OK;
}

int sf_map_arrays(const sf_map *m, sf_device_map *o) {
  if (!m || !o) return SF_ERR_INVALID;
  o->heap_mem = m->d.heap;
  o->entry_ptr = m->d.entry_ptr;
  o->heap_counter = m->d.heap_counter;
  o->bucket_mutex = m->d.bucket_mutex;
  o->voxel_blocks = m->d.voxels;
  o->no_visible_blocks = m->d.no_visible;
  o->hash_entries = m->d.entries;
  o->visible_entries = m->d.visible;
  return SF_OK;
}

int sf_map_rebuild_index(sf_context *ctx, sf_map *m) {
  if (!ctx || !m) return SF_ERR_INVALID;
  launch_rebuild_index(m->d, ctx->stream);
  SF_CHECK(cudaGetLastError());
  return SF_OK;
}

// ------------------------------------------------------------- map.bin
namespace {

constexpr int kRefMaxKeys = 100000;                  // KeyMap::MaxKeys (Mapping/DeviceMap.h:207)
constexpr long long kRefKeyEntries = kRefMaxKeys * 5LL;  // KeyMap::maxEntries (:208-209)
constexpr size_t kRefSurfBytes = 288;  // SURF: bool valid, float3 pos, float4 normal, float[64] (:129-138)
constexpr size_t kMapIoChunk = 32u << 20;

struct MapBinHeader {
  int num_sdf_blocks, num_buckets, num_voxels, num_entries;
};

MapBinHeader map_bin_header(const sf_map_config &c) {
  MapBinHeader h;
  h.num_sdf_blocks = (int)c.num_sdf_blocks;
  h.num_buckets = (int)c.num_buckets;
  h.num_voxels = (int)(c.num_sdf_blocks * 512u);
  h.num_entries = (int)(c.num_buckets + c.num_excess);
  return h;
}

// Device array <-> file through a pinned staging buffer, chunk by chunk.
int dev_to_file(std::FILE *f, const void *dev, size_t bytes, char *stage, cudaStream_t st) {
  for (size_t off = 0; off < bytes; off += kMapIoChunk) {
    const size_t n = bytes - off < kMapIoChunk ? bytes - off : kMapIoChunk;
    SF_CHECK(cudaMemcpyAsync(stage, (const char *)dev + off, n, cudaMemcpyDeviceToHost, st));
    SF_CHECK(cudaStreamSynchronize(st));
    if (std::fwrite(stage, 1, n, f) != n) return SF_ERR_IO;
  }
  return SF_OK;
}

int file_to_dev(std::FILE *f, void *dev, size_t bytes, char *stage, cudaStream_t st) {
  for (size_t off = 0; off < bytes; off += kMapIoChunk) {
    const size_t n = bytes - off < kMapIoChunk ? bytes - off : kMapIoChunk;
    SF_CHECK(cudaStreamSynchronize(st));  // the previous chunk has left the staging buffer
    if (std::fread(stage, 1, n, f) != n) return SF_ERR_IO;
    SF_CHECK(cudaMemcpyAsync((char *)dev + off, stage, n, cudaMemcpyHostToDevice, st));
  }
  SF_CHECK(cudaStreamSynchronize(st));
  return SF_OK;
}

struct FileCloser {
  std::FILE *f;
  ~FileCloser() {
    if (f) std::fclose(f);
  }
};
struct PinnedBuffer {
  char *p = nullptr;
  ~PinnedBuffer() {
    if (p) cudaFreeHost(p);
  }
};

}  // namespace

int sf_map_write(sf_context *ctx, const sf_map *m, const char *path) {
  if (!ctx || !m || !path) return SF_ERR_INVALID;
  const MapBinHeader h = map_bin_header(m->cfg);
  FileCloser fc{std::fopen(path, "wb")};
  if (!fc.f) return SF_ERR_IO;
  PinnedBuffer stage;
  SF_CHECK(cudaMallocHost(&stage.p, kMapIoChunk));
  cudaStream_t st = ctx->stream;
  int counters[3];
  SF_CHECK(cudaMemcpyAsync(&counters[0], m->d.heap_counter, sizeof(int), cudaMemcpyDeviceToHost, st));
  SF_CHECK(cudaMemcpyAsync(&counters[1], m->d.entry_ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
  SF_CHECK(cudaMemcpyAsync(&counters[2], m->d.no_visible, sizeof(int), cudaMemcpyDeviceToHost, st));
  SF_CHECK(cudaStreamSynchronize(st));
  if (std::fwrite(&h, sizeof(h), 1, fc.f) != 1 || std::fwrite(counters, sizeof(int), 3, fc.f) != 3)
    return SF_ERR_IO;
  int r;
  if ((r = dev_to_file(fc.f, m->d.heap, sizeof(int) * (size_t)h.num_sdf_blocks, stage.p, st)) ||
      (r = dev_to_file(fc.f, m->d.bucket_mutex, sizeof(int) * (size_t)h.num_buckets, stage.p, st)) ||
      (r = dev_to_file(fc.f, m->d.voxels, sizeof(sf_voxel) * (size_t)h.num_voxels, stage.p, st)) ||
      (r = dev_to_file(fc.f, m->d.entries, sizeof(sf_hash_entry) * (size_t)h.num_entries, stage.p, st)) ||
      (r = dev_to_file(fc.f, m->d.visible, sizeof(sf_hash_entry) * (size_t)h.num_entries, stage.p, st)))
    return r;
  // the keypoint map, reset (ResetKeyPoints, Mapping/FuseMap.cu:1306-1322)
  std::memset(stage.p, 0xff, sizeof(int) * (size_t)kRefMaxKeys);
  if (std::fwrite(stage.p, sizeof(int), kRefMaxKeys, fc.f) != (size_t)kRefMaxKeys) return SF_ERR_IO;
  std::memset(stage.p, 0, kMapIoChunk);
  for (long long left = kRefKeyEntries * (long long)kRefSurfBytes; left > 0;) {
    const size_t n = left < (long long)kMapIoChunk ? (size_t)left : kMapIoChunk;
    if (std::fwrite(stage.p, 1, n, fc.f) != n) return SF_ERR_IO;
    left -= (long long)n;
  }
  if (std::fflush(fc.f) != 0) return SF_ERR_IO;
  return SF_OK;
}

int sf_map_read(sf_context *ctx, sf_map *m, const char *path) {
  if (!ctx || !m || !path) return SF_ERR_INVALID;
  const MapBinHeader want = map_bin_header(m->cfg);
  FileCloser fc{std::fopen(path, "rb")};
  if (!fc.f) return SF_ERR_IO;
  MapBinHeader h;
  int counters[3];
  if (std::fread(&h, sizeof(h), 1, fc.f) != 1) return SF_ERR_IO;
  if (h.num_sdf_blocks != want.num_sdf_blocks || h.num_buckets != want.num_buckets ||
      h.num_voxels != want.num_voxels || h.num_entries != want.num_entries)
    return SF_ERR_INVALID;
  if (std::fread(counters, sizeof(int), 3, fc.f) != 3) return SF_ERR_IO;
  PinnedBuffer stage;
  SF_CHECK(cudaMallocHost(&stage.p, kMapIoChunk));
  cudaStream_t st = ctx->stream;
  int r;
  if ((r = file_to_dev(fc.f, m->d.heap, sizeof(int) * (size_t)h.num_sdf_blocks, stage.p, st)) ||
      (r = file_to_dev(fc.f, m->d.bucket_mutex, sizeof(int) * (size_t)h.num_buckets, stage.p, st)) ||
      (r = file_to_dev(fc.f, m->d.voxels, sizeof(sf_voxel) * (size_t)h.num_voxels, stage.p, st)) ||
      (r = file_to_dev(fc.f, m->d.entries, sizeof(sf_hash_entry) * (size_t)h.num_entries, stage.p, st)) ||
      (r = file_to_dev(fc.f, m->d.visible, sizeof(sf_hash_entry) * (size_t)h.num_entries, stage.p, st)))
    return r;
  SF_CHECK(cudaMemcpyAsync(m->d.heap_counter, &counters[0], sizeof(int), cudaMemcpyHostToDevice, st));
  SF_CHECK(cudaMemcpyAsync(m->d.entry_ptr, &counters[1], sizeof(int), cudaMemcpyHostToDevice, st));
  SF_CHECK(cudaMemcpyAsync(m->d.no_visible, &counters[2], sizeof(int), cudaMemcpyHostToDevice, st));
  launch_rebuild_index(m->d, st);
  SF_CHECK(cudaGetLastError());
  SF_CHECK(cudaStreamSynchronize(st));
  return SF_OK;
}

int sf_map_counters(sf_context *ctx, const sf_map *m, int out[4]) {
  if (!ctx || !m || !out) return SF_ERR_INVALID;
  SF_CHECK(cudaMemcpyAsync(out + 0, m->d.heap_counter, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  SF_CHECK(cudaMemcpyAsync(out + 1, m->d.entry_ptr, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  SF_CHECK(cudaMemcpyAsync(out + 2, m->d.no_visible, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  SF_CHECK(cudaMemcpyAsync(out + 3, m->d.alloc_count, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  SF_CHECK(cudaStreamSynchronize(ctx->stream));
  return SF_OK;
}

int sf_ResetMap(sf_context *ctx, sf_map *m) {
  if (!ctx || !m) return SF_ERR_INVALID;
  launch_map_reset(m->d, ctx->stream);
  SF_CHECK(cudaGetLastError());
  return SF_OK;
}

// ------------------------------------------------------------- pyramid
int sf_FilterDepth(sf_context *ctx, sf_image depth, sf_image raw, sf_image filt, float depth_scale,
                   float depth_cutoff) {
  if (!ctx || !img_ok(depth, 2) || !img_ok(raw, 4) || !img_ok(filt, 4)) return SF_ERR_INVALID;
  if (raw.cols != depth.cols || raw.rows != depth.rows || filt.cols != depth.cols ||
      filt.rows != depth.rows || depth_scale <= 0)
    return SF_ERR_INVALID;
  launch_filter_depth(depth, raw, filt, depth_scale, depth_cutoff, ctx->stream);
  SF_CHECK(cudaGetLastError());
  return SF_OK;
}

int sf_ComputeVMap(sf_context *ctx, sf_image depth, sf_image vmap, float fx, float fy, float cx,
                   float cy, float depth_cutoff) {
  if (!ctx || !img_ok(depth, 4) || !img_ok(vmap, 16) || vmap.cols != depth.cols ||
      vmap.rows != depth.rows)
    return SF_ERR_INVALID;
  launch_vmap(depth, vmap, fx, fy, cx, cy, depth_cutoff, ctx->stream);
  SF_CHECK(cudaGetLastError());
  return SF_OK;
}

int sf_ComputeNMap(sf_context *ctx, sf_image vmap, sf_image nmap) {
  if (!ctx || !img_ok(vmap, 16) || !img_ok(nmap, 16) || vmap.cols != nmap.cols ||
      vmap.rows != nmap.rows)
    return SF_ERR_INVALID;
  launch_nmap(vmap, nmap, ctx->stream);
  SF_CHECK(cudaGetLastError());
  return SF_OK;
}

int sf_PyrDownGauss(sf_context *ctx, sf_image src, sf_image dst) {
  if (!ctx || !img_ok(src, 4) || !img_ok(dst, 4) || dst.cols * 2 > src.cols ||
      dst.rows * 2 > src.rows)
    return SF_ERR_INVALID;
  launch_pyrdown(src, dst, ctx->stream);
  SF_CHECK(cudaGetLastError());
  return SF_OK;
}

int sf_ResizeMap(sf_context *ctx, sf_image vsrc, sf_image nsrc, sf_image vdst, sf_image ndst) {
  if (!ctx || !img_ok(vsrc, 16) || !img_ok(nsrc, 16) || !img_ok(vdst, 16) || !img_ok(ndst, 16))
    return SF_ERR_INVALID;
  if (vdst.cols * 2 > vsrc.cols || vdst.rows * 2 > vsrc.rows || nsrc.cols != vsrc.cols ||
      nsrc.rows != vsrc.rows || ndst.cols != vdst.cols || ndst.rows != vdst.rows)
    return SF_ERR_INVALID;
  launch_resize(vsrc, nsrc, vdst, ndst, ctx->stream);
  SF_CHECK(cudaGetLastError());
  return SF_OK;
}

int sf_BuildPyramid(sf_context *ctx, sf_image depth_u16, sf_image raw, const sf_image *depths,
                    const sf_image *vmaps, const sf_image *nmaps, int levels, sf_intrinsics K,
                    float depth_scale, float depth_cutoff) {
  if (!ctx || !depths || !vmaps || !nmaps || levels < 1 || levels > kMaxLevels) return SF_ERR_INVALID;
  for (int l = 0; l < levels; ++l)
    if (!img_ok(depths[l], 4) || !img_ok(vmaps[l], 16) || !img_ok(nmaps[l], 16)) return SF_ERR_INVALID;
  int st = sf_FilterDepth(ctx, depth_u16, raw, depths[0], depth_scale, depth_cutoff);
  if (st) return st;
  if (pyramid_levels_fusable(depths, vmaps, nmaps, levels)) {
    launch_pyramid_levels(depths, vmaps, nmaps, levels, K.fx, K.fy, K.cx, K.cy, depth_cutoff, ctx->stream);
    SF_CHECK(cudaGetLastError());
    return SF_OK;
  }
  for (int l = 0; l < levels; ++l) {
    if (l > 0) launch_pyrdown(depths[l - 1], depths[l], ctx->stream);
    const float div = (float)(1 << l);
    launch_vnmap(depths[l], vmaps[l], nmaps[l], K.fx / div, K.fy / div, K.cx / div, K.cy / div,
                 depth_cutoff, ctx->stream);
  }
  SF_CHECK(cudaGetLastError());
  return SF_OK;
}

// ----------------------------------------------------------------- ICP
int sf_ICPStep(sf_context *ctx, sf_image next_vmap, sf_image last_vmap, sf_image next_nmap,
               sf_image last_nmap, sf_mat3 Rcurr, sf_float3 tcurr, sf_mat3 Rlast,
               sf_mat3 RlastInv, sf_float3 tlast, sf_intrinsics K, float residual[2],
               double matrixA[36], double vectorB[6]) {
  if (!ctx || !residual || !matrixA || !vectorB) return SF_ERR_INVALID;
  const sf_image *ims[4] = {&next_vmap, &last_vmap, &next_nmap, &last_nmap};
  for (auto im : ims)
    if (!img_ok(*im, 16) || im->cols != next_vmap.cols || im->rows != next_vmap.rows)
      return SF_ERR_INVALID;
  IcpLevelArgs L;
  L.vc = next_vmap; L.nc = next_nmap; L.vl = last_vmap; L.nl = last_nmap;
  L.fx = K.fx; L.fy = K.fy; L.cx = K.cx; L.cy = K.cy;
  L.iters = 1; L.min_count = 0;
  launch_icp_step(ctx->icp, L, to_m3(Rcurr), to_f3(tcurr), to_m3(Rlast), to_m3(RlastInv),
                  to_f3(tlast), ctx->stream);
  SF_CHECK(cudaGetLastError());
  SF_CHECK(cudaMemcpyAsync(ctx->host_sums, ctx->icp.sums, 29 * sizeof(double),
                           cudaMemcpyDeviceToHost, ctx->stream));
  SF_CHECK(cudaStreamSynchronize(ctx->stream));
  create_matrix(ctx->host_sums, matrixA, vectorB);
  residual[0] = (float)ctx->host_sums[27];
  residual[1] = (float)ctx->host_sums[28];
  return SF_OK;
}

int sf_ComputeSE3(sf_context *ctx, int levels, const sf_image *nv, const sf_image *nn,
                  const sf_image *lv, const sf_image *ln, sf_intrinsics K, const int *iters,
                  const int *min_count, float thresh, const double last_pose[16],
                  double next_pose_out[16], int stats_out[4], float *icp_error_out) {
  if (!ctx || levels < 1 || levels > kMaxLevels || !nv || !nn || !lv || !ln || !iters ||
      !min_count || !last_pose || !next_pose_out)
    return SF_ERR_INVALID;
  IcpLevelArgs L[kMaxLevels];
  for (int l = 0; l < levels; ++l) {
    const sf_image *ims[4] = {&nv[l], &nn[l], &lv[l], &ln[l]};
    for (auto im : ims)
      if (!img_ok(*im, 16) || im->cols != nv[l].cols || im->rows != nv[l].rows) return SF_ERR_INVALID;
    if (iters[l] < 0) return SF_ERR_INVALID;
    const float div = (float)(1 << l);
    L[l].vc = nv[l]; L[l].nc = nn[l]; L[l].vl = lv[l]; L[l].nl = ln[l];
    L[l].fx = K.fx / div; L[l].fy = K.fy / div; L[l].cx = K.cx / div; L[l].cy = K.cy / div;
    L[l].iters = iters[l];
    L[l].min_count = min_count[l];
  }
  SF_CHECK(cudaMemcpyAsync(ctx->pose, last_pose, 16 * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  SF_CHECK(icp_persistent_reset(ctx->icp, ctx->stream));
  SF_CHECK(launch_icp_persistent(ctx->icp, L, levels, thresh, ctx->pose, nullptr, ctx->flags, ctx->stream));
  SF_CHECK(cudaMemcpyAsync(ctx->host_ctl, ctx->icp.ctl, sizeof(TrackCtl), cudaMemcpyDeviceToHost, ctx->stream));
  SF_CHECK(cudaStreamSynchronize(ctx->stream));
  const TrackCtl &c = *ctx->host_ctl;
  for (int k = 0; k < 16; ++k) next_pose_out[k] = c.next_pose[k];
  if (stats_out) {
    stats_out[0] = c.accepted;
    stats_out[1] = c.stop;
    stats_out[2] = c.iters_run;
    stats_out[3] = c.icpCount;
  }
  if (icp_error_out) *icp_error_out = c.icpError;
  return c.timeout ? SF_ERR_TIMEOUT : SF_OK;
}

// ------------------------------------------------------ photometric term
int sf_ImageToIntensity(sf_context *ctx, sf_image rgb, sf_image image) {
  if (!ctx || !img_ok(rgb, 3) || !img_ok(image, 1) || rgb.cols != image.cols || rgb.rows != image.rows)
    return SF_ERR_INVALID;
  launch_intensity(rgb, image, nullptr, nullptr, ctx->stream);
  SF_CHECK(cudaGetLastError());
  return SF_OK;
}

int sf_PyrDownGauss_u8(sf_context *ctx, sf_image src, sf_image dst) {
  if (!ctx || !img_ok(src, 1) || !img_ok(dst, 1) || dst.cols > src.cols || dst.rows > src.rows)
    return SF_ERR_INVALID;
  launch_pyrdown_u8(src, dst, nullptr, nullptr, ctx->stream);
  SF_CHECK(cudaGetLastError());
  return SF_OK;
}

int sf_ComputeDerivativeImage(sf_context *ctx, sf_image image, sf_image dx, sf_image dy) {
  if (!ctx || !img_ok(image, 1) || !img_ok(dx, 2) || !img_ok(dy, 2) || dx.cols != image.cols ||
      dx.rows != image.rows || dy.cols != image.cols || dy.rows != image.rows)
    return SF_ERR_INVALID;
  launch_derivatives(&image, &dx, &dy, nullptr, 1, ctx->stream);
  SF_CHECK(cudaGetLastError());
  return SF_OK;
}

namespace {
// Photometric inputs of one level, checked against the level's vertex map;
// the candidate flags go to `cand` (rows x cols bytes of scratch).
int rgb_level(sf_context *ctx, const sf_image &vmap, const sf_image &inext, const sf_image &ilast,
              const sf_image &dx, const sf_image &dy, uint8_t *cand, RgbLevelArgs &R) {
  const sf_image *u8[2] = {&inext, &ilast}, *s16[2] = {&dx, &dy};
  for (auto im : u8)
    if (!img_ok(*im, 1) || im->cols != vmap.cols || im->rows != vmap.rows) return SF_ERR_INVALID;
  for (auto im : s16)
    if (!img_ok(*im, 2) || im->cols != vmap.cols || im->rows != vmap.rows) return SF_ERR_INVALID;
  R.inext = inext; R.ilast = ilast; R.dx = dx; R.dy = dy;
  R.cand.data = cand; R.cand.step = (size_t)vmap.cols; R.cand.cols = vmap.cols; R.cand.rows = vmap.rows;
  R.corr = ctx->icp.corr;
  launch_rgb_cand(inext, dx, dy, R.cand, ctx->stream);
  return SF_OK;
}
}  // namespace

int sf_RGBStep(sf_context *ctx, sf_image next_image, sf_image last_image, sf_image next_vmap,
               sf_image last_vmap, sf_image dIdx, sf_image dIdy, sf_mat3 Rcurr, sf_mat3 RcurrInv,
               sf_mat3 Rlast, sf_mat3 RlastInv, sf_float3 tcurr, sf_float3 tlast, sf_intrinsics K,
               float residual[2], double matrixA[36], double vectorB[6]) {
  if (!ctx || !residual || !matrixA || !vectorB) return SF_ERR_INVALID;
  if (!img_ok(next_vmap, 16) || !img_ok(last_vmap, 16) || last_vmap.cols != next_vmap.cols ||
      last_vmap.rows != next_vmap.rows)
    return SF_ERR_INVALID;
  const size_t px = (size_t)next_vmap.cols * next_vmap.rows;
  int st = icp_workspace_rgb(ctx->icp, px);
  if (st) return st;
  IcpLevelArgs L;
  L.vc = next_vmap; L.vl = last_vmap; L.nc = next_vmap; L.nl = last_vmap;
  L.fx = K.fx; L.fy = K.fy; L.cx = K.cx; L.cy = K.cy;
  L.iters = 1; L.min_count = 0;
  RgbLevelArgs R;
  if ((st = rgb_level(ctx, next_vmap, next_image, last_image, dIdx, dIdy, ctx->icp.cand, R))) return st;
  launch_rgb_step(ctx->icp, L, R, to_m3(Rcurr), to_m3(RcurrInv), to_f3(tcurr), to_m3(Rlast), to_m3(RlastInv),
                  to_f3(tlast), ctx->stream);
  SF_CHECK(cudaGetLastError());
  SF_CHECK(cudaMemcpyAsync(ctx->host_sums, ctx->icp.sums + 29, 29 * sizeof(double), cudaMemcpyDeviceToHost,
                           ctx->stream));
  SF_CHECK(cudaStreamSynchronize(ctx->stream));
  create_matrix(ctx->host_sums, matrixA, vectorB);
  residual[0] = (float)ctx->host_sums[27];
  residual[1] = (float)ctx->host_sums[28];
  return SF_OK;
}

int sf_ComputeSE3_rgbd(sf_context *ctx, int levels, const sf_image *nv, const sf_image *nn,
                       const sf_image *lv, const sf_image *ln, const sf_image *next_images,
                       const sf_image *last_images, const sf_image *next_dIdx, const sf_image *next_dIdy,
                       sf_intrinsics K, const int *iters, const int *min_count, float thresh,
                       const double last_pose[16], double next_pose_out[16], int stats_out[6],
                       float errors_out[2]) {
  if (!ctx || levels < 1 || levels > kMaxLevels || !nv || !nn || !lv || !ln || !next_images || !last_images ||
      !next_dIdx || !next_dIdy || !iters || !min_count || !last_pose || !next_pose_out)
    return SF_ERR_INVALID;
  const size_t px0 = (size_t)nv[0].cols * nv[0].rows;
  int st = icp_workspace_rgb(ctx->icp, px0);
  if (st) return st;
  IcpLevelArgs L[kMaxLevels];
  RgbLevelArgs R[kMaxLevels];
  size_t cand_off = 0;
  for (int l = 0; l < levels; ++l) {
    const sf_image *ims[4] = {&nv[l], &nn[l], &lv[l], &ln[l]};
    for (auto im : ims)
      if (!img_ok(*im, 16) || im->cols != nv[l].cols || im->rows != nv[l].rows) return SF_ERR_INVALID;
    if (iters[l] < 0) return SF_ERR_INVALID;
    const size_t px = (size_t)nv[l].cols * nv[l].rows;
    if (px > px0 || cand_off + px > 2 * px0) return SF_ERR_INVALID;
    const float div = (float)(1 << l);
    L[l].vc = nv[l]; L[l].nc = nn[l]; L[l].vl = lv[l]; L[l].nl = ln[l];
    L[l].fx = K.fx / div; L[l].fy = K.fy / div; L[l].cx = K.cx / div; L[l].cy = K.cy / div;
    L[l].iters = iters[l];
    L[l].min_count = min_count[l];
    if ((st = rgb_level(ctx, nv[l], next_images[l], last_images[l], next_dIdx[l], next_dIdy[l],
                        ctx->icp.cand + cand_off, R[l])))
      return st;
    cand_off += px;
  }
  SF_CHECK(cudaMemcpyAsync(ctx->pose, last_pose, 16 * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  SF_CHECK(icp_persistent_reset(ctx->icp, ctx->stream));
  SF_CHECK(launch_icp_persistent(ctx->icp, L, levels, thresh, ctx->pose, nullptr, ctx->flags, ctx->stream, R));
  SF_CHECK(cudaMemcpyAsync(ctx->host_ctl, ctx->icp.ctl, sizeof(TrackCtl), cudaMemcpyDeviceToHost, ctx->stream));
  SF_CHECK(cudaStreamSynchronize(ctx->stream));
  const TrackCtl &c = *ctx->host_ctl;
  for (int k = 0; k < 16; ++k) next_pose_out[k] = c.next_pose[k];
  if (stats_out) {
    stats_out[0] = c.accepted;
    stats_out[1] = c.stop;
    stats_out[2] = c.iters_run;
    stats_out[3] = c.icpCount;
    stats_out[4] = c.rgbCount;
    stats_out[5] = 0;
  }
  if (errors_out) {
    errors_out[0] = c.icpError;
    errors_out[1] = c.rgbError;
  }
  return c.timeout ? SF_ERR_TIMEOUT : SF_OK;
}

// ------------------------------------------------------------- mesh
int sf_MeshScene(sf_context *ctx, sf_map *m, float *vertices, float *normals, uint8_t *colors,
                 uint32_t max_triangles, uint32_t *num_triangles) {
  if (!ctx || !m || !vertices || !normals || !colors || !num_triangles || max_triangles == 0) return SF_ERR_INVALID;
  launch_mesh(m->d, reinterpret_cast<float3 *>(vertices), reinterpret_cast<float3 *>(normals),
              reinterpret_cast<uchar3 *>(colors), max_triangles, ctx->u32, ctx->stream);
  SF_CHECK(cudaGetLastError());
  uint32_t n = 0;
  SF_CHECK(cudaMemcpyAsync(&n, ctx->u32, sizeof(n), cudaMemcpyDeviceToHost, ctx->stream));
  SF_CHECK(cudaStreamSynchronize(ctx->stream));
  *num_triangles = n < max_triangles ? n : max_triangles;  // MeshScene.cu:352-353
  return SF_OK;
}

int sf_mesh_write_ply(sf_context *ctx, const char *path, const float *vertices, const float *normals,
                      const uint8_t *colors, uint32_t num_triangles) {
  if (!ctx || !path || (num_triangles && (!vertices || !normals || !colors))) return SF_ERR_INVALID;
  FILE *fp = fopen(path, "w");
  if (!fp) return SF_ERR_IO;
  FileCloser close_fp{fp};
  const size_t nv = (size_t)num_triangles * 3;
  // System::WriteMeshToDisk's ASCII layout (Core/System.cc:283-322); the
  // numbers print as an ostream's defaults (%g)
  if (fprintf(fp,
              "ply\nformat ascii 1.0\nelement vertex %zu\nproperty float x\nproperty float y\nproperty float z\n"
              "property float nx\nproperty float ny\nproperty float nz\nproperty uchar red\nproperty uchar green\n"
              "property uchar blue\nelement face %u\nproperty list uchar uint vertex_indices\nend_header\n",
              nv, num_triangles) < 0)
    return SF_ERR_IO;
  const size_t chunk = 1 << 18;
  std::vector<float> v, n;
  std::vector<uint8_t> c;
  for (size_t i0 = 0; i0 < nv; i0 += chunk) {
    const size_t k = nv - i0 < chunk ? nv - i0 : chunk;
    v.resize(3 * k); n.resize(3 * k); c.resize(3 * k);
    SF_CHECK(cudaMemcpyAsync(v.data(), vertices + 3 * i0, 12 * k, cudaMemcpyDeviceToHost, ctx->stream));
    SF_CHECK(cudaMemcpyAsync(n.data(), normals + 3 * i0, 12 * k, cudaMemcpyDeviceToHost, ctx->stream));
    SF_CHECK(cudaMemcpyAsync(c.data(), colors + 3 * i0, 3 * k, cudaMemcpyDeviceToHost, ctx->stream));
    SF_CHECK(cudaStreamSynchronize(ctx->stream));
    for (size_t i = 0; i < k; ++i)
      if (fprintf(fp, "%g %g %g %g %g %g %d %d %d\n", v[3 * i], v[3 * i + 1], v[3 * i + 2], n[3 * i], n[3 * i + 1],
                  n[3 * i + 2], (int)c[3 * i], (int)c[3 * i + 1], (int)c[3 * i + 2]) < 0)
        return SF_ERR_IO;
  }
  for (uint32_t t = 0; t < num_triangles; ++t)
    if (fprintf(fp, "3 %d %d %d\n", (int)t * 3 + 0, (int)t * 3 + 1, (int)t * 3 + 2) < 0) return SF_ERR_IO;
  return SF_OK;
}

// -------------------------------------------------------- relocalisation
int sf_RelocScoreBatch(sf_context *ctx, sf_map *m, sf_image vmap, int stride, const double *poses, int n,
                       float inlier_sdf, sf_reloc_score *scores_out) {
  if (!ctx || !m || !poses || !scores_out || n < 1 || n > 65536 || stride < 1 || !img_ok(vmap, 16))
    return SF_ERR_INVALID;
  if (n > ctx->reloc_cap) {
    SF_CHECK(cudaStreamSynchronize(ctx->stream));
    cudaFree(ctx->reloc_poses);
    cudaFree(ctx->reloc_scores);
    cudaFree(ctx->reloc_part);
    ctx->reloc_poses = nullptr;
    ctx->reloc_scores = nullptr;
    ctx->reloc_part = nullptr;
    ctx->reloc_cap = 0;
    SF_CHECK(cudaMalloc(&ctx->reloc_poses, sizeof(float) * 12 * (size_t)n));
    SF_CHECK(cudaMalloc(&ctx->reloc_scores, sizeof(sf_reloc_score) * (size_t)n));
    SF_CHECK(cudaMalloc(&ctx->reloc_part, sizeof(sf_reloc_score) * (size_t)n * reloc_score_parts()));
    ctx->reloc_cap = n;
  }
  // Frame::GpuRotation / GpuTranslation (Core/Frame.cc:626-645) per candidate
  std::vector<float> hp(12 * (size_t)n);
  for (int k = 0; k < n; ++k) {
    const double *P = poses + 16 * (size_t)k;
    float *q = hp.data() + 12 * (size_t)k;
    const int src[12] = {0, 1, 2, 4, 5, 6, 8, 9, 10, 3, 7, 11};
    for (int i = 0; i < 12; ++i) q[i] = (float)P[src[i]];
  }
  SF_CHECK(cudaMemcpyAsync(ctx->reloc_poses, hp.data(), sizeof(float) * hp.size(), cudaMemcpyHostToDevice,
                           ctx->stream));
  launch_reloc_score(m->d, vmap, stride, ctx->reloc_poses, n, inlier_sdf, ctx->reloc_part, ctx->reloc_scores,
                     ctx->stream);
  SF_CHECK(cudaGetLastError());
  SF_CHECK(cudaMemcpyAsync(scores_out, ctx->reloc_scores, sizeof(sf_reloc_score) * (size_t)n,
                           cudaMemcpyDeviceToHost, ctx->stream));
  SF_CHECK(cudaStreamSynchronize(ctx->stream));
  return SF_OK;
}

// --------------------------------------------------------------- fusion
int sf_CheckBlockVisibility(sf_context *ctx, sf_map *m, sf_mat3 Rview, sf_mat3 RviewInv,
                            sf_float3 tview, int cols, int rows, float fx, float fy, float cx,
                            float cy, float depth_max, float depth_min, uint32_t *host_data) {
  if (!ctx || !m || !host_data || cols <= 0 || rows <= 0) return SF_ERR_INVALID;
  int st = upload_cam(ctx, make_cam(Rview, RviewInv, tview, fx, fy, cx, cy, cols, rows, depth_min, depth_max));
  if (st) return st;
  if ((st = ensure_scratch(m, cols * rows))) return st;
  launch_visibility(m->d, m->scratch, ctx->cam, nullptr, nullptr, nullptr, ctx->flags, ctx->stream);
  SF_CHECK(cudaGetLastError());
  SF_CHECK(cudaMemcpyAsync(host_data, m->d.no_visible, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
  SF_CHECK(cudaStreamSynchronize(ctx->stream));
  return SF_OK;
}

int sf_FuseMapColor(sf_context *ctx, sf_map *m, sf_image depth, sf_image color, sf_image nmap,
                    sf_image mask, int num_detection, sf_mat3 Rview, sf_mat3 RviewInv,
                    sf_float3 tview, float fx, float fy, float cx, float cy, float depth_max,
                    float depth_min, uint32_t *host_data) {
  (void)depth_max;
  (void)depth_min;  // FuseMapColor uses DeviceMap::DepthMax/DepthMin (FuseMap.cu:1080-1081)
  if (!ctx || !m || !host_data || !img_ok(depth, 4) || !img_ok(color, 3)) return SF_ERR_INVALID;
  if (num_detection > 0 && (!img_ok(nmap, 16) || !img_ok(mask, 1))) return SF_ERR_INVALID;
  int st = upload_cam(ctx, make_cam(Rview, RviewInv, tview, fx, fy, cx, cy, depth.cols, depth.rows,
                                    m->cfg.depth_min, m->cfg.depth_max));
  if (st) return st;
  if ((st = ensure_scratch(m, depth.cols * depth.rows))) return st;
  launch_alloc(m->d, m->scratch, depth, ctx->cam, nullptr, ctx->flags, ctx->stream);
  launch_visibility(m->d, m->scratch, ctx->cam, nullptr, nullptr, nullptr, ctx->flags, ctx->stream);
  SF_CHECK(cudaGetLastError());
  SF_CHECK(cudaMemcpyAsync(host_data, m->d.no_visible, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
  SF_CHECK(cudaStreamSynchronize(ctx->stream));
  if (host_data[0] == 0) return SF_OK;  // "no visible blocks found" early return
  launch_integrate(m->d, depth, color, num_detection > 0 ? &nmap : nullptr,
                   num_detection > 0 ? &mask : nullptr, num_detection, ctx->cam, true,
                   num_detection > 0, nullptr, ctx->stream);
  if (num_detection > 0) {  // FuseMap.cu:1141-1160
    if ((st = fuse_scratch_unify(m->scratch, m->d.c))) return st;
    launch_unify_neighbor(m->d, m->scratch, nullptr, ctx->stream);
  }
  SF_CHECK(cudaGetLastError());
  SF_CHECK(cudaStreamSynchronize(ctx->stream));
  return SF_OK;
}

int sf_AnalyzeMapSemantics(sf_context *ctx, sf_map *m, sf_image depth, sf_image color,
                           sf_image nmap, sf_image mask, int num_detection, sf_mat3 Rview,
                           sf_mat3 RviewInv, sf_float3 tview, float fx, float fy, float cx,
                           float cy, float depth_max, float depth_min) {
  (void)depth_max;
  (void)depth_min;
  if (!ctx || !m || !img_ok(depth, 4) || !img_ok(color, 3) || !img_ok(nmap, 16)) return SF_ERR_INVALID;
  if (num_detection > 0 && !img_ok(mask, 1)) return SF_ERR_INVALID;
  int st = upload_cam(ctx, make_cam(Rview, RviewInv, tview, fx, fy, cx, cy, depth.cols, depth.rows,
                                    m->cfg.depth_min, m->cfg.depth_max));
  if (st) return st;
  if ((st = ensure_scratch(m, depth.cols * depth.rows))) return st;
  launch_visibility(m->d, m->scratch, ctx->cam, nullptr, nullptr, nullptr, ctx->flags, ctx->stream);
  launch_integrate(m->d, depth, color, &nmap, num_detection > 0 ? &mask : nullptr, num_detection,
                   ctx->cam, false, true, nullptr, ctx->stream);
  if ((st = fuse_scratch_unify(m->scratch, m->d.c))) return st;
  launch_unify_neighbor(m->d, m->scratch, nullptr, ctx->stream);
  SF_CHECK(cudaGetLastError());
  SF_CHECK(cudaStreamSynchronize(ctx->stream));
  return SF_OK;
}

int sf_SemanticAnalysis(sf_context *ctx, sf_map *m, sf_image vmap, sf_image color, sf_image nmap, sf_image mask,
                        int num_detection, sf_mat3 Rview, sf_mat3 RviewInv, sf_float3 tview, float fx, float fy,
                        float cx, float cy) {
  if (!ctx || !m || !img_ok(vmap, 16) || !img_ok(color, 3) || !img_ok(nmap, 16)) return SF_ERR_INVALID;
  const size_t px = (size_t)vmap.cols * vmap.rows;
  if (px > ctx->rdepth_px) {
    SF_CHECK(cudaStreamSynchronize(ctx->stream));
    cudaFree(ctx->rdepth);
    ctx->rdepth = nullptr;
    ctx->rdepth_px = 0;
    SF_CHECK(cudaMalloc(&ctx->rdepth, px * sizeof(float)));
    ctx->rdepth_px = px;
  }
  sf_image rd;
  rd.data = ctx->rdepth; rd.step = (size_t)vmap.cols * sizeof(float); rd.cols = vmap.cols; rd.rows = vmap.rows;
  launch_vmap_depth(vmap, rd, nullptr, ctx->stream);
  SF_CHECK(cudaGetLastError());
  return sf_AnalyzeMapSemantics(ctx, m, rd, color, nmap, mask, num_detection, Rview, RviewInv, tview, fx, fy, cx,
                                cy, m->cfg.depth_max, m->cfg.depth_min);
}

int sf_UnifyNeighbor(sf_context *ctx, sf_map *m) {
  if (!ctx || !m) return SF_ERR_INVALID;
  int st = fuse_scratch_unify(m->scratch, m->d.c);
  if (st) return st;
  launch_unify_neighbor(m->d, m->scratch, nullptr, ctx->stream);
  SF_CHECK(cudaGetLastError());
  SF_CHECK(cudaStreamSynchronize(ctx->stream));
  return SF_OK;
}

// -------------------------------------------------------------- raycast
int sf_CreateRenderingBlocks(sf_context *ctx, sf_map *m, sf_image zmin, sf_image zmax,
                             float depth_max, float depth_min, sf_rendering_block *list,
                             uint32_t *no_blocks, sf_mat3 RviewInv, sf_float3 tview,
                             uint32_t no_visible, float fx, float fy, float cx, float cy,
                             int *ok_out) {
  if (!ctx || !m || !list || !no_blocks || !ok_out || !img_ok(zmin, 4) || !img_ok(zmax, 4))
    return SF_ERR_INVALID;
  *ok_out = 0;
  if (no_visible == 0) return SF_OK;
  sf_mat3 I = {};
  int st = upload_cam(ctx, make_cam(I, RviewInv, tview, fx, fy, cx, cy, zmin.cols * 8, zmin.rows * 8,
                                    depth_min, depth_max));
  if (st) return st;
  SF_CHECK(cudaMemsetAsync(no_blocks, 0, sizeof(uint32_t), ctx->stream));
  launch_zrange_init(zmin, zmax, ctx->stream);
  launch_rendering_blocks(m->d, no_visible, zmin, list, no_blocks, ctx->cam, ctx->flags, ctx->stream);
  uint32_t total = 0;
  SF_CHECK(cudaMemcpyAsync(&total, no_blocks, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
  SF_CHECK(cudaStreamSynchronize(ctx->stream));
  if (total == 0) return SF_OK;
  launch_fill_blocks(zmin, zmax, list, total, ctx->stream);
  SF_CHECK(cudaGetLastError());
  SF_CHECK(cudaStreamSynchronize(ctx->stream));
  *ok_out = 1;
  return SF_OK;
}

int sf_Raycast(sf_context *ctx, sf_map *m, sf_image vmap, sf_image nmap, sf_image zmin,
               sf_image zmax, sf_mat3 Rview, sf_mat3 RviewInv, sf_float3 tview, float invfx,
               float invfy, float cx, float cy) {
  if (!ctx || !m || !img_ok(vmap, 16) || !img_ok(nmap, 16) || !img_ok(zmin, 4) || !img_ok(zmax, 4))
    return SF_ERR_INVALID;
  Cam c = make_cam(Rview, RviewInv, tview, 1.0f, 1.0f, cx, cy, vmap.cols, vmap.rows,
                   m->cfg.depth_min, m->cfg.depth_max);
  c.invfx = invfx;  // the reference passes 1.0 / fx explicitly (Mapping.cc:158-159)
  c.invfy = invfy;
  int st = upload_cam(ctx, c);
  if (st) return st;
  if ((st = ensure_scratch(m, vmap.cols * vmap.rows))) return st;
  launch_window_build(m->d, m->scratch, ctx->cam, ctx->stream);
  launch_raycast(m->d, m->scratch, vmap, nmap, zmin, zmax, ctx->cam, nullptr, nullptr, nullptr, nullptr,
                 ctx->stream);
  SF_CHECK(cudaGetLastError());
  return SF_OK;
}

int sf_RaycastAdjoint(sf_context *ctx, sf_map *m, sf_image zmin, sf_image zmax, sf_mat3 Rview,
                      sf_mat3 RviewInv, sf_float3 tview, float invfx, float invfy, float cx, float cy,
                      sf_image grad_vmap, sf_image grad_nmap, float *grad_sdf, double grad_pose_out[6]) {
  if (!ctx || !m || !grad_pose_out || !img_ok(grad_vmap, 16) || !img_ok(zmin, 4) || !img_ok(zmax, 4))
    return SF_ERR_INVALID;
  if (grad_nmap.data && (!img_ok(grad_nmap, 16) || grad_nmap.cols != grad_vmap.cols ||
                         grad_nmap.rows != grad_vmap.rows))
    return SF_ERR_INVALID;
  Cam c = make_cam(Rview, RviewInv, tview, 1.0f, 1.0f, cx, cy, grad_vmap.cols, grad_vmap.rows,
                   m->cfg.depth_min, m->cfg.depth_max);
  c.invfx = invfx;
  c.invfy = invfy;
  int st = upload_cam(ctx, c);
  if (st) return st;
  if ((st = ensure_scratch(m, grad_vmap.cols * grad_vmap.rows))) return st;
  const int nb = raycast_adjoint_blocks(grad_vmap.cols, grad_vmap.rows);
  if (nb > ctx->adj_cap) {
    SF_CHECK(cudaStreamSynchronize(ctx->stream));
    cudaFree(ctx->adj_part);
    ctx->adj_part = nullptr;
    ctx->adj_cap = 0;
    SF_CHECK(cudaMalloc(&ctx->adj_part, sizeof(float) * 6 * (size_t)nb));
    ctx->adj_cap = nb;
  }
  if (!ctx->adj_pose) SF_CHECK(cudaMalloc(&ctx->adj_pose, sizeof(double) * 6));
  launch_window_build(m->d, m->scratch, ctx->cam, ctx->stream);
  launch_raycast_adjoint(m->d, m->scratch, zmin, zmax, ctx->cam, grad_vmap, grad_nmap, grad_sdf, ctx->adj_part,
                         ctx->adj_pose, ctx->stream);
  SF_CHECK(cudaGetLastError());
  SF_CHECK(cudaMemcpyAsync(grad_pose_out, ctx->adj_pose, sizeof(double) * 6, cudaMemcpyDeviceToHost,
                           ctx->stream));
  SF_CHECK(cudaStreamSynchronize(ctx->stream));
  return SF_OK;
}

}  // extern "C"

// Accessors used by system.cu.
namespace sf {
static std::atomic<unsigned long long> g_launches{0};
void note_launch(unsigned long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
unsigned long long launches_total() { return g_launches.load(std::memory_order_relaxed); }
cudaStream_t ctx_stream(sf_context *c) { return c->stream; }
IcpWorkspace &ctx_icp(sf_context *c) { return c->icp; }
uint32_t *ctx_flags(sf_context *c) { return c->flags; }
DevMap &map_dev(sf_map *m) { return m->d; }
FuseScratch &map_scratch(sf_map *m) { return m->scratch; }
int map_ensure_scratch(sf_map *m, int pixels) { return ensure_scratch(m, pixels); }
const sf_map_config &map_cfg(sf_map *m) { return m->cfg; }
VpWorkspace *&ctx_vp(sf_context *c) { return c->vp; }
}  // namespace sf
