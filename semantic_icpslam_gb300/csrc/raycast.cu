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
  const DevMap *m;
  const int *cells;
  int win[6];
};

__device__ __forceinline__ int block_ptr(const RayCtx &r, i3 bp) {
  const int cell = window_cell(r.win, bp);
  if (cell >= 0) return __ldg(r.cells + cell);
  return find_block(*r.m, bp);
}

struct VoxelRead {
  float sdf;
  unsigned weight;
  bool found;
};

// DeviceMap::FindVoxel(float3, cache, valid): a missing block reads as
// Voxel() (sdf NaN, weight 0) and valid = false.
__device__ __forceinline__ VoxelRead read_voxel(const RayCtx &r, f3 pt) {
  const i3 p = floor3(pt);
  const int ptr = block_ptr(r, vox2block(p));
  VoxelRead v;
  if (ptr < 0) {
    v.sdf = nanf_bits();
    v.weight = 0;
    v.found = false;
    return v;
  }
  const uint2 raw = __ldg((const uint2 *)(r.m->voxels + ptr + vox2local(p)));
  v.sdf = __uint_as_float(raw.x);
  v.weight = raw.y & 0xffu;
  v.found = true;
  return v;
}

// Rendering::readSdf (RenderScene.cu:303-308).
__device__ __forceinline__ float read_sdf(const RayCtx &r, f3 pt, bool &valid) {
  VoxelRead v = read_voxel(r, pt);
  valid = v.found && v.weight != 0;
  return v.sdf;
}

// Rendering::readSdfInterped (RenderScene.cu:310-343).  The eight corner
// reads are independent; `valid` is the last corner's (pt + (1,1,1)), as
// each FindVoxel call overwrites it in the reference.
__device__ __forceinline__ float read_sdf_interp(const RayCtx &r, f3 pt, bool &valid) {
  const f3 xyz3 = pt - mk3(floorf(pt.x), floorf(pt.y), floorf(pt.z));
  const VoxelRead c000 = read_voxel(r, pt);
  const VoxelRead c100 = read_voxel(r, pt + mk3(1, 0, 0));
  const VoxelRead c010 = read_voxel(r, pt + mk3(0, 1, 0));
  const VoxelRead c110 = read_voxel(r, pt + mk3(1, 1, 0));
  const VoxelRead c001 = read_voxel(r, pt + mk3(0, 0, 1));
  const VoxelRead c101 = read_voxel(r, pt + mk3(1, 0, 1));
  const VoxelRead c011 = read_voxel(r, pt + mk3(0, 1, 1));
  const VoxelRead c111 = read_voxel(r, pt + mk3(1, 1, 1));
  float r0 = (1.0f - xyz3.x) * c000.sdf + xyz3.x * c100.sdf;
  float r1 = (1.0f - xyz3.x) * c010.sdf + xyz3.x * c110.sdf;
  const float r2 = (1.0f - xyz3.y) * r0 + xyz3.y * r1;
  r0 = (1.0f - xyz3.x) * c001.sdf + xyz3.x * c101.sdf;
  r1 = (1.0f - xyz3.x) * c011.sdf + xyz3.x * c111.sdf;
  const float r3 = (1.0f - xyz3.y) * r0 + xyz3.y * r1;
  valid = c111.found;
  return (1.0f - xyz3.z) * r2 + xyz3.z * r3;
}

// Rendering::readNormal (RenderScene.cu:345-378).
__device__ __forceinline__ bool read_normal(const RayCtx &r, f3 pt, const m3 &Rinv, f3 &n) {
  bool valid;
  const float s0 = read_sdf_interp(r, pt + mk3(1, 0, 0), valid);
  if (isnan(s0) || s0 == 1.0f || !valid) return false;
  const float s1 = read_sdf_interp(r, pt + mk3(-1, 0, 0), valid);
  if (isnan(s1) || s1 == 1.0f || !valid) return false;
  const float s2 = read_sdf_interp(r, pt + mk3(0, 1, 0), valid);
  if (isnan(s2) || s2 == 1.0f || !valid) return false;
  const float s3 = read_sdf_interp(r, pt + mk3(0, -1, 0), valid);
  if (isnan(s3) || s3 == 1.0f || !valid) return false;
  const float s4 = read_sdf_interp(r, pt + mk3(0, 0, 1), valid);
  if (isnan(s4) || s4 == 1.0f || !valid) return false;
  const float s5 = read_sdf_interp(r, pt + mk3(0, 0, -1), valid);
  if (isnan(s5) || s5 == 1.0f || !valid) return false;
  n = normalised(mul(Rinv, mk3(s0 - s1, s2 - s3, s4 - s5)));
  return true;
}

// Rendering::operator() (RenderScene.cu:380-488).
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
  r.m = &m;
  r.cells = f.win_cells;
  for (int k = 0; k < 6; ++k) r.win[k] = f.win[k];
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
    bool valid_sdf = false, behind = false;
    float step, prev_sdf;
    while (dist_s < dist_e) {
      prev_sdf = sdf;
      sdf = read_sdf(r, result, valid_sdf);
      if (!valid_sdf) {
        step = 8.0f;
      } else {
        if (sdf <= 0.1f && sdf >= -0.5f) sdf = read_sdf_interp(r, result, valid_sdf);
        if (prev_sdf < 0.f && sdf >= 0.f) { behind = true; break; }
        if (prev_sdf > 0.f && sdf <= 0.f) break;
        step = 1.0f;
      }
      result = result + step * dir;
      dist_s += step;
    }
    if (!behind && sdf <= 0.0f) {
      step = sdf * m.c.step_scale;
      result = result + step * dir;
      sdf = read_sdf_interp(r, result, valid_sdf);
      step = sdf * m.c.step_scale;
      result = result + step * dir;
      f3 n;
      if (read_normal(r, result, c.Rinv, n)) {
        const f3 q = mul(c.Rinv, result * m.c.voxel_size - c.t);
        vout = make_float4(q.x, q.y, q.z, 1.0f);
        nout = make_float4(n.x, n.y, n.z, 1.0f);
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
