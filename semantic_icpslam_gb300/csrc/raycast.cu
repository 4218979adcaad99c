// Rendering-block z-range and the block-skipping trilinear raycast.
//
// Reference: Mapping/RenderScene.cu (Projection :9-191,
// CreateRenderingBlocks :210-289, Rendering :291-489, Raycast :495-537)
// with DeviceMap::FindVoxel's per-ray entry cache (DeviceMap.cu:116-133).
//
// GB300 form: the per-frame path lays the z-range tiles down during the
// visibility pass (fusion.cu), so no rendering-block list is materialised,
// downloaded or re-read; the list form below serves the reference-shaped
// CreateRenderingBlocks entry point.  Float z-ranges are positive, so the
// reference's CAS-loop float min/max become single integer atomicMin/Max
// on the bit patterns.  The raycast reads only the first 8 bytes of a
// voxel (sdf, weight) per sample.
#include "sf_kernels.cuh"
#include "sf_render.cuh"

namespace sf {


namespace {

// Projection::operator() (RenderScene.cu:134-165) in list form: each valid
// block reserves nx*ny slots and fills them with the tiles (y < ny, x < ny)
// of createRenderingBlockList (:114-132); reserved slots beyond ny*ny hold
// empty tiles.
__global__ void k_project_blocks(DevMap m, uint32_t nvis, const Cam *cam, int zc, int zr,
                                 sf_rendering_block *list, uint32_t *count, uint32_t cap,
                                 uint32_t *flags) {
  const Cam c = *cam;
  for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < nvis; k += gridDim.x * blockDim.x) {
    int4 h = __ldcg((const int4 *)(m.visible + k));
    if (h.w == -1) continue;
    i3 pos; pos.x = h.x; pos.y = h.y; pos.z = h.z;
    sf_rendering_block b;
    if (!project_block(pos, m.c.voxel_size, c.Rinv, c.t, c.fx, c.fy, c.cx, c.cy, zc, zr, c.dmax,
                       c.dmin, b))
      continue;
    float dx = (float)b.lrx - (float)b.ulx + 1.0f;
    float dy = (float)b.lry - (float)b.uly + 1.0f;
    int nx = (int)ceilf(dx / 16.0f), ny = (int)ceilf(dy / 16.0f);
    unsigned required = (unsigned)(nx * ny);
    unsigned off = atomicAdd(count, required);
    if (off + required >= cap) {
      atomicOr(flags, SF_FLAG_RENDER_FULL);
      atomicSub(count, required);
      continue;
    }
    unsigned slot = 0;
    for (int y = 0; y < ny && slot < required; ++y)
      for (int x = 0; x < ny && slot < required; ++x) {
        sf_rendering_block t;
        t.ulx = (int16_t)(b.ulx + x * 16);
        t.uly = (int16_t)(b.uly + y * 16);
        t.lrx = (int16_t)(b.ulx + 16);
        t.lry = (int16_t)(b.uly + 16);
        if (t.lrx > b.lrx) t.lrx = b.lrx;
        if (t.lry > b.lry) t.lry = b.lry;
        t.zmin = b.zmin;
        t.zmax = b.zmax;
        list[off + slot++] = t;
      }
    for (; slot < required; ++slot) {
      sf_rendering_block e;
      e.ulx = 1; e.uly = 1; e.lrx = 0; e.lry = 0;
      e.zmin = b.zmin; e.zmax = b.zmax;
      list[off + slot] = e;
    }
  }
}

// Projection::fillBlocks (RenderScene.cu:167-190), one 16x16 CTA per tile.
__global__ void k_fill_blocks(sf_image zmin, sf_image zmax, const sf_rendering_block *list,
                              uint32_t n) {
  const unsigned blk = blockIdx.x;
  if (blk >= n) return;
  const sf_rendering_block b = list[blk];
  int xpos = b.ulx + (int)threadIdx.x;
  if (xpos > b.lrx || xpos >= zmin.cols) return;
  int ypos = b.uly + (int)threadIdx.y;
  if (ypos > b.lry || ypos >= zmin.rows) return;
  atomicMin(row_ptr<int>(zmin, ypos) + xpos, __float_as_int(b.zmin));
  atomicMax(row_ptr<int>(zmax, ypos) + xpos, __float_as_int(b.zmax));
}

// ---------------------------------------------------------------- raycast
// Block lookup for the ray: the frame's block-pointer window, the hash table
// (DeviceMap::FindEntry) outside it.  Equal to FindEntry for every block,
// so the per-ray entry cache of DeviceMap::FindVoxel (DeviceMap.cu:116-133)
// has nothing left to save and is not kept.  (The reference's cache starts
// as {pos (0,0,0), ptr -1}, which would alias block (0,0,0) to voxel index
// -1; that aliasing is not reproduced.)
struct RayCtx {
  const sf_voxel *voxels;
  const int *cells;
  int win[6];
  const sf_hash_entry *entries;
  uint32_t num_buckets, num_excess;
};

// Hash-table lookup (DeviceMap::FindEntry) for a block outside the window;
// rare, so kept out of line to keep the inlined sample code small.
__device__ __noinline__ int block_ptr_hash(const sf_hash_entry *entries, uint32_t num_buckets,
                                           uint32_t num_excess, int bx, int by, int bz) {
  DevMap m;
  m.entries = const_cast<sf_hash_entry *>(entries);
  m.c.num_buckets = num_buckets;
  m.c.num_excess = num_excess;
  i3 p;
  p.x = bx; p.y = by; p.z = bz;
  return find_block(m, p);
}

// Voxel index of block (bx, by, bz), or -1.
__device__ __forceinline__ int block_ptr(const RayCtx &r, int bx, int by, int bz) {
  const unsigned x = (unsigned)(bx - r.win[0]), y = (unsigned)(by - r.win[1]), z = (unsigned)(bz - r.win[2]);
  if (x < (unsigned)r.win[3] && y < (unsigned)r.win[4] && z < (unsigned)r.win[5])
    return __ldg(r.cells + (int)((z * (unsigned)r.win[4] + y) * (unsigned)r.win[3] + x));
  return block_ptr_hash(r.entries, r.num_buckets, r.num_excess, bx, by, bz);
}

struct VoxelRead {
  float sdf;
  unsigned weight;
  bool found;
};

// Voxel (vx, vy, vz) of the block whose voxel index is ptr (block
// coordinates are v >> 3, local ones v & 7, as worldPosToVoxelPos /
// voxelPosToLocalIdx compute them).  A missing block reads as Voxel()
// (sdf NaN, weight 0) with found = false, as DeviceMap::FindVoxel does.
__device__ __forceinline__ VoxelRead voxel_in(const RayCtx &r, int ptr, int vx, int vy, int vz) {
  VoxelRead v;
  if (ptr < 0) {
    v.sdf = nanf_bits();
    v.weight = 0;
    v.found = false;
    return v;
  }
  const uint2 raw = __ldg((const uint2 *)(r.voxels + ptr + ((vz & 7) * 64 + (vy & 7) * 8 + (vx & 7))));
  v.sdf = __uint_as_float(raw.x);
  v.weight = raw.y & 0xffu;
  v.found = true;
  return v;
}

__device__ __forceinline__ VoxelRead read_voxel(const RayCtx &r, f3 pt) {
  const i3 p = floor3(pt);
  return voxel_in(r, block_ptr(r, p.x >> 3, p.y >> 3, p.z >> 3), p.x, p.y, p.z);
}

// Rendering::readSdfInterped (RenderScene.cu:310-343).  The corners are
// the reference's floor3(pt + offset); per axis that is floor(pt) or
// floor(pt + 1), so six floors give all eight.  Corners that share a block
// share one lookup.  `valid` is the last corner's (pt + (1,1,1)), as each
// FindVoxel call overwrites it in the reference.
__device__ __forceinline__ float sdf_interp(const RayCtx &r, f3 pt, bool &valid) {
  const f3 xyz3 = pt - mk3(floorf(pt.x), floorf(pt.y), floorf(pt.z));
  const i3 a = floor3(pt);
  const i3 b = floor3(pt + mk3(1, 1, 1));
  const int ax = a.x >> 3, ay = a.y >> 3, az = a.z >> 3;
  const int bx = b.x >> 3, by = b.y >> 3, bz = b.z >> 3;
  const bool sx = ax == bx, sy = ay == by, sz = az == bz;
  const int p000 = block_ptr(r, ax, ay, az);
  const int p100 = sx ? p000 : block_ptr(r, bx, ay, az);
  const int p010 = sy ? p000 : block_ptr(r, ax, by, az);
  const int p110 = sx ? p010 : (sy ? p100 : block_ptr(r, bx, by, az));
  const int p001 = sz ? p000 : block_ptr(r, ax, ay, bz);
  const int p101 = sx ? p001 : (sz ? p100 : block_ptr(r, bx, ay, bz));
  const int p011 = sy ? p001 : (sz ? p010 : block_ptr(r, ax, by, bz));
  const int p111 = sx ? p011 : (sy ? p101 : (sz ? p110 : block_ptr(r, bx, by, bz)));
  const VoxelRead c000 = voxel_in(r, p000, a.x, a.y, a.z);
  const VoxelRead c100 = voxel_in(r, p100, b.x, a.y, a.z);
  const VoxelRead c010 = voxel_in(r, p010, a.x, b.y, a.z);
  const VoxelRead c110 = voxel_in(r, p110, b.x, b.y, a.z);
  const VoxelRead c001 = voxel_in(r, p001, a.x, a.y, b.z);
  const VoxelRead c101 = voxel_in(r, p101, b.x, a.y, b.z);
  const VoxelRead c011 = voxel_in(r, p011, a.x, b.y, b.z);
  const VoxelRead c111 = voxel_in(r, p111, b.x, b.y, b.z);
  float r0 = (1.0f - xyz3.x) * c000.sdf + xyz3.x * c100.sdf;
  float r1 = (1.0f - xyz3.x) * c010.sdf + xyz3.x * c110.sdf;
  const float r2 = (1.0f - xyz3.y) * r0 + xyz3.y * r1;
  r0 = (1.0f - xyz3.x) * c001.sdf + xyz3.x * c101.sdf;
  r1 = (1.0f - xyz3.x) * c011.sdf + xyz3.x * c111.sdf;
  const float r3 = (1.0f - xyz3.y) * r0 + xyz3.y * r1;
  valid = c111.found;
  return (1.0f - xyz3.z) * r2 + xyz3.z * r3;
}

struct SdfValid {
  float sdf;
  bool valid;
};

// Out-of-line copy for the marching loop and the surface refinement
// (arguments by value so the caller's context stays in registers).
__device__ __noinline__ SdfValid read_sdf_interp(const RayCtx r, f3 pt) {
  SdfValid o;
  o.sdf = sdf_interp(r, pt, o.valid);
  return o;
}

struct NormalOut {
  f3 n;
  bool ok;
};

// Rendering::readNormal (RenderScene.cu:345-378).  The six interpolations
// are independent, so all of them are issued before the reference's checks
// run in its order (the early returns only decide the output).
__device__ __noinline__ NormalOut read_normal(const RayCtx r, f3 pt, const m3 Rinv) {
  NormalOut o;
  o.ok = false;
  bool v0, v1, v2, v3, v4, v5;
  const float s0 = sdf_interp(r, pt + mk3(1, 0, 0), v0);
  const float s1 = sdf_interp(r, pt + mk3(-1, 0, 0), v1);
  const float s2 = sdf_interp(r, pt + mk3(0, 1, 0), v2);
  const float s3 = sdf_interp(r, pt + mk3(0, -1, 0), v3);
  const float s4 = sdf_interp(r, pt + mk3(0, 0, 1), v4);
  const float s5 = sdf_interp(r, pt + mk3(0, 0, -1), v5);
  if (isnan(s0) || s0 == 1.0f || !v0) return o;
  if (isnan(s1) || s1 == 1.0f || !v1) return o;
  if (isnan(s2) || s2 == 1.0f || !v2) return o;
  if (isnan(s3) || s3 == 1.0f || !v3) return o;
  if (isnan(s4) || s4 == 1.0f || !v4) return o;
  if (isnan(s5) || s5 == 1.0f || !v5) return o;
  o.n = normalised(mul(Rinv, mk3(s0 - s1, s2 - s3, s4 - s5)));
  o.ok = true;
  return o;
}

constexpr int kSpec = 4;  // march samples read ahead together

// Rendering::operator() (RenderScene.cu:380-488).  The march reads kSpec
// samples ahead at once, at the positions a run of 1-voxel steps would
// reach (the same float additions), then replays the reference's loop over
// them in order; an 8-voxel step or the end of the range ends the run.
__global__ void __launch_bounds__(128) k_raycast(DevMap m, FuseScratch f, sf_image vmap, sf_image nmap,
                                                 sf_image zmin, sf_image zmax, const Cam *cam,
                                                 const unsigned *rendered, sf_image fb_v,
                                                 sf_image fb_n, const int *run_flag) {
  if (run_flag && *run_flag == 0) return;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= vmap.cols || y >= vmap.rows) return;
  if (rendered && *rendered == 0u) {
    // Mapping::RayTrace skips Raycast: the maps keep the frame's own maps.
    if (fb_v.data) {
      row_ptr<float4>(vmap, y)[x] = __ldg(row_ptr<const float4>(fb_v, y) + x);
      row_ptr<float4>(nmap, y)[x] = __ldg(row_ptr<const float4>(fb_n, y) + x);
    }
    return;
  }
  const Cam c = *cam;
  RayCtx r;
  r.voxels = m.voxels;
  r.cells = f.win_cells;
  for (int k = 0; k < 6; ++k) r.win[k] = f.win[k];
  r.entries = m.entries;
  r.num_buckets = m.c.num_buckets;
  r.num_excess = m.c.num_excess;
  float4 vout = nan4(), nout = nan4();
  const int lx = (int)floorf((float)x / 8.0f), ly = (int)floorf((float)y / 8.0f);
  const float zx = __ldg(row_ptr<const float>(zmin, ly) + lx);
  const float zy = __ldg(row_ptr<const float>(zmax, ly) + lx);
  // (double)z < 1e-3 of the reference: no float lies in [1e-3, 0.001f), so
  // for a float z that is exactly z < 0.001f
  if (!(zy < 0.001f || zx < 0.001f || isnan(zx) || isnan(zy))) {
    const float vsi = m.c.voxel_size_inv;
    float sdf = 1.0f;
    f3 p;
    p.z = zx;
    p.x = p.z * ((float)x - c.cx) * c.invfx;
    p.y = p.z * ((float)y - c.cy) * c.invfy;
    float dist_s = norm(p) * vsi;
    const f3 block_s = (mul(c.R, p) + c.t) * vsi;
    p.z = zy;
    p.x = p.z * ((float)x - c.cx) * c.invfx;
    p.y = p.z * ((float)y - c.cy) * c.invfy;
    const float dist_e = norm(p) * vsi;
    const f3 block_e = (mul(c.R, p) + c.t) * vsi;
    const f3 dir = normalised(block_e - block_s);
    f3 result = block_s;
    bool valid_sdf = false, behind = false, done = false;
    while (!done && dist_s < dist_e) {
      f3 pos[kSpec];
      float ds[kSpec];
      VoxelRead v[kSpec];
      pos[0] = result;
      ds[0] = dist_s;
#pragma unroll
      for (int i = 1; i < kSpec; ++i) {
        pos[i] = pos[i - 1] + 1.0f * dir;
        ds[i] = ds[i - 1] + 1.0f;
      }
#pragma unroll
      for (int i = 0; i < kSpec; ++i) v[i] = read_voxel(r, pos[i]);
      bool run = true;  // still on the speculated run of 1-voxel steps
#pragma unroll
      for (int i = 0; i < kSpec; ++i) {
        if (!run) break;
        if (i > 0 && !(ds[i] < dist_e)) {  // the while condition fails here
          result = pos[i];
          dist_s = ds[i];
          done = true;
          break;
        }
        const float prev_sdf = sdf;
        sdf = v[i].sdf;
        valid_sdf = v[i].found && v[i].weight != 0;
        if (!valid_sdf) {  // 8-voxel step: the run ends
          result = pos[i] + 8.0f * dir;
          dist_s = ds[i] + 8.0f;
          run = false;
          break;
        }
        if (sdf <= 0.1f && sdf >= -0.5f) {
          const SdfValid sv = read_sdf_interp(r, pos[i]);
          sdf = sv.sdf;
          valid_sdf = sv.valid;
        }
        if (prev_sdf < 0.f && sdf >= 0.f) {
          behind = true;
          done = true;
          break;
        }
        if (prev_sdf > 0.f && sdf <= 0.f) {
          result = pos[i];
          done = true;
          break;
        }
        if (i == kSpec - 1) {  // every speculated sample consumed
          result = pos[i] + 1.0f * dir;
          dist_s = ds[i] + 1.0f;
        }
      }
    }
    if (!behind && sdf <= 0.0f) {
      float step = sdf * m.c.step_scale;
      result = result + step * dir;
      sdf = read_sdf_interp(r, result).sdf;
      step = sdf * m.c.step_scale;
      result = result + step * dir;
      const NormalOut no = read_normal(r, result, c.Rinv);
      if (no.ok) {
        const f3 q = mul(c.Rinv, result * m.c.voxel_size - c.t);
        vout = make_float4(q.x, q.y, q.z, 1.0f);
        nout = make_float4(no.n.x, no.n.y, no.n.z, 1.0f);
      }
    }
  }
  row_ptr<float4>(vmap, y)[x] = vout;
  row_ptr<float4>(nmap, y)[x] = nout;
}

// Builds the block window for the reference-shaped Raycast entry point.
__global__ void k_window_build_setup(DevMap m, FuseScratch f, const Cam *cam) {
  window_setup(*cam, m.c.block_width, m.c.depth_min, m.c.depth_max, f.win_cap, f.win);
}
__global__ void k_window_build_clear(FuseScratch f) {
  const unsigned n = (unsigned)f.win[3] * (unsigned)f.win[4] * (unsigned)f.win[5];
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    f.win_cells[i] = -1;
}
__global__ void k_window_build_fill(DevMap m, FuseScratch f) {
  const unsigned n = (unsigned)*m.alloc_count;
  int win[6];
  for (int k = 0; k < 6; ++k) win[k] = f.win[k];
  for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int4 h = entry_head(m.entries + m.alloc_list[k]);
    i3 pos; pos.x = h.x; pos.y = h.y; pos.z = h.z;
    const int cell = window_cell(win, pos);
    if (cell >= 0 && h.w >= 0) f.win_cells[cell] = h.w;
  }
}

}  // namespace

void launch_rendering_blocks(const DevMap &m, uint32_t nvis, const sf_image &zmin,
                             sf_rendering_block *list, uint32_t *count, const Cam *c,
                             uint32_t *flags, cudaStream_t s) {
  k_project_blocks<<<256, 256, 0, s>>>(m, nvis, c, zmin.cols, zmin.rows, list, count,
                                       m.c.max_rendering_blocks, flags); note_launch();
}

void launch_fill_blocks(const sf_image &zmin, const sf_image &zmax,
                        const sf_rendering_block *list, uint32_t nblocks, cudaStream_t s) {
  if (nblocks == 0) return;
  k_fill_blocks<<<nblocks, dim3(16, 16), 0, s>>>(zmin, zmax, list, nblocks); note_launch();
}

void launch_raycast(const DevMap &m, const FuseScratch &f, const sf_image &vmap, const sf_image &nmap,
                    const sf_image &zmin, const sf_image &zmax, const Cam *c,
                    const unsigned *rendered, const sf_image *fallback_v,
                    const sf_image *fallback_n, const int *run_flag, cudaStream_t s) {
  dim3 blk(8, 16);
  dim3 grd((vmap.cols + 7) / 8, (vmap.rows + 15) / 16);
  sf_image fv = fallback_v ? *fallback_v : sf_image{};
  sf_image fn = fallback_n ? *fallback_n : sf_image{};
  k_raycast<<<grd, blk, 0, s>>>(m, f, vmap, nmap, zmin, zmax, c, rendered, fv, fn, run_flag); note_launch();
}

void launch_window_build(const DevMap &m, const FuseScratch &f, const Cam *c, cudaStream_t s) {
  k_window_build_setup<<<1, 1, 0, s>>>(m, f, c); note_launch();
  k_window_build_clear<<<256, 256, 0, s>>>(f); note_launch();
  k_window_build_fill<<<256, 256, 0, s>>>(m, f); note_launch();
}

}  // namespace sf
