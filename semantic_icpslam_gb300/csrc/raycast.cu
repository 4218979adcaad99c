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
#include "sf_frame.cuh"
#include "sf_render.cuh"
#include "sf_sample.cuh"

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

// One axis of readNormal's six interpolation points pt + e (e = (+-1, 0, 0)
// and so on): the coordinate is v0 = p + 0 for the four points that do not
// move along this axis and vP = p + 1, vM = p + (-1) for the two that do.
// For each, readSdfInterped's corners are floor(v) and floor(v + 1) (the
// reference's make_int3 floor of float sums) and its weight v - floorf(v).
// The axis is regular when the corners chain up, floor(vM + 1) = floor(v0)
// and floor(v0 + 1) = floor(vP), so that the six cubes use the four
// coordinates c[0] = floor(vM) .. c[3] = floor(vP + 1) and at most two
// blocks: c[0] >> 3 and c[3] >> 3 differ by at most one.
struct NormalAxis {
  int c[4];
  float f0, fP, fM;
  bool regular;
};

__device__ __forceinline__ int floor1(float a) {
  const int b = (int)a;
  return (float)b > a ? b - 1 : b;
}

__device__ __forceinline__ NormalAxis normal_axis(float p) {
  NormalAxis n;
  const float v0 = p + 0.0f, vP = p + 1.0f, vM = p + (-1.0f);
  const int a0 = floor1(v0), b0 = floor1(v0 + 1.0f);
  const int aP = floor1(vP), bP = floor1(vP + 1.0f);
  const int aM = floor1(vM), bM = floor1(vM + 1.0f);
  n.f0 = v0 - floorf(v0);
  n.fP = vP - floorf(vP);
  n.fM = vM - floorf(vM);
  n.c[0] = aM; n.c[1] = a0; n.c[2] = b0; n.c[3] = bP;
  n.regular = bM == a0 && b0 == aP && (unsigned)((bP >> 3) - (aM >> 3)) <= 1u;
  return n;
}

// readSdfInterped's trilinear form on the eight corner values (c000 ..
// c111 in the reference's order) with weights (fx, fy, fz).
__device__ __forceinline__ float trilerp(float fx, float fy, float fz, float c000, float c100, float c010,
                                         float c110, float c001, float c101, float c011, float c111) {
  float r0 = (1.0f - fx) * c000 + fx * c100;
  float r1 = (1.0f - fx) * c010 + fx * c110;
  const float r2 = (1.0f - fy) * r0 + fy * r1;
  r0 = (1.0f - fx) * c001 + fx * c101;
  r1 = (1.0f - fx) * c011 + fx * c111;
  const float r3 = (1.0f - fy) * r0 + fy * r1;
  return (1.0f - fz) * r2 + fz * r3;
}

// Rendering::readNormal (RenderScene.cu:345-378).  The six interpolations
// (pt +- one voxel along each axis) read 48 corners, of which 32 are
// distinct when every axis is regular (the usual case): the 2x2x2 cube
// around pt and a 2x2 face beyond it on each side.  Those 32 voxels are
// read once, through at most eight block lookups, and each interpolation
// takes its corners from them with the reference's arithmetic and order;
// otherwise the six interpolations run as readSdfInterped does.  The
// reference's checks then run in its order (the early returns only decide
// the output).
__device__ __noinline__ NormalOut read_normal(const RayCtx r, f3 pt, const m3 Rinv) {
  NormalOut o;
  o.ok = false;
  const NormalAxis X = normal_axis(pt.x), Y = normal_axis(pt.y), Z = normal_axis(pt.z);
  float s[6];
  bool v[6];
  if (X.regular && Y.regular && Z.regular) {
    // block pointers of the (lo | hi)^3 blocks; a bit per axis picks hi
    const int lx = X.c[0] >> 3, ly = Y.c[0] >> 3, lz = Z.c[0] >> 3;
    const int hx = X.c[3] >> 3, hy = Y.c[3] >> 3, hz = Z.c[3] >> 3;
    const bool sx = lx == hx, sy = ly == hy, sz = lz == hz;
    int P[8];
    P[0] = block_ptr(r, lx, ly, lz);
    P[1] = sx ? P[0] : block_ptr(r, hx, ly, lz);
    P[2] = sy ? P[0] : block_ptr(r, lx, hy, lz);
    P[3] = sx ? P[2] : (sy ? P[1] : block_ptr(r, hx, hy, lz));
    P[4] = sz ? P[0] : block_ptr(r, lx, ly, hz);
    P[5] = sx ? P[4] : (sz ? P[1] : block_ptr(r, hx, ly, hz));
    P[6] = sy ? P[4] : (sz ? P[2] : block_ptr(r, lx, hy, hz));
    P[7] = sx ? P[6] : (sy ? P[5] : (sz ? P[3] : block_ptr(r, hx, hy, hz)));
    // voxel (X.c[i], Y.c[j], Z.c[k])
    auto vox = [&](int i, int j, int k) {
      const int bi = (X.c[i] >> 3) != lx, bj = (Y.c[j] >> 3) != ly, bk = (Z.c[k] >> 3) != lz;
      const int q0 = bj ? (bk ? P[6] : P[2]) : (bk ? P[4] : P[0]);
      const int q1 = bj ? (bk ? P[7] : P[3]) : (bk ? P[5] : P[1]);
      return voxel_in(r, bi ? q1 : q0, X.c[i], Y.c[j], Z.c[k]);
    };
    // the 2x2x2 cube (coordinates 1, 2 on every axis)
    VoxelRead k000 = vox(1, 1, 1), k100 = vox(2, 1, 1), k010 = vox(1, 2, 1), k110 = vox(2, 2, 1);
    VoxelRead k001 = vox(1, 1, 2), k101 = vox(2, 1, 2), k011 = vox(1, 2, 2), k111 = vox(2, 2, 2);
    // faces beyond it: x = c[0] (xm) and c[3] (xp), the same for y and z
    VoxelRead xm00 = vox(0, 1, 1), xm10 = vox(0, 2, 1), xm01 = vox(0, 1, 2), xm11 = vox(0, 2, 2);
    VoxelRead xp00 = vox(3, 1, 1), xp10 = vox(3, 2, 1), xp01 = vox(3, 1, 2), xp11 = vox(3, 2, 2);
    VoxelRead ym00 = vox(1, 0, 1), ym10 = vox(2, 0, 1), ym01 = vox(1, 0, 2), ym11 = vox(2, 0, 2);
    VoxelRead yp00 = vox(1, 3, 1), yp10 = vox(2, 3, 1), yp01 = vox(1, 3, 2), yp11 = vox(2, 3, 2);
    VoxelRead zm00 = vox(1, 1, 0), zm10 = vox(2, 1, 0), zm01 = vox(1, 2, 0), zm11 = vox(2, 2, 0);
    VoxelRead zp00 = vox(1, 1, 3), zp10 = vox(2, 1, 3), zp01 = vox(1, 2, 3), zp11 = vox(2, 2, 3);
    // +x: x corners c[2], c[3]; -x: c[0], c[1]; y, z corners c[1], c[2]
    s[0] = trilerp(X.fP, Y.f0, Z.f0, k100.sdf, xp00.sdf, k110.sdf, xp10.sdf, k101.sdf, xp01.sdf, k111.sdf, xp11.sdf);
    v[0] = xp11.found;
    s[1] = trilerp(X.fM, Y.f0, Z.f0, xm00.sdf, k000.sdf, xm10.sdf, k010.sdf, xm01.sdf, k001.sdf, xm11.sdf, k011.sdf);
    v[1] = k011.found;
    s[2] = trilerp(X.f0, Y.fP, Z.f0, k010.sdf, k110.sdf, yp00.sdf, yp10.sdf, k011.sdf, k111.sdf, yp01.sdf, yp11.sdf);
    v[2] = yp11.found;
    s[3] = trilerp(X.f0, Y.fM, Z.f0, ym00.sdf, ym10.sdf, k000.sdf, k100.sdf, ym01.sdf, ym11.sdf, k001.sdf, k101.sdf);
    v[3] = k101.found;
    s[4] = trilerp(X.f0, Y.f0, Z.fP, k001.sdf, k101.sdf, k011.sdf, k111.sdf, zp00.sdf, zp10.sdf, zp01.sdf, zp11.sdf);
    v[4] = zp11.found;
    s[5] = trilerp(X.f0, Y.f0, Z.fM, zm00.sdf, zm10.sdf, zm01.sdf, zm11.sdf, k000.sdf, k100.sdf, k010.sdf, k110.sdf);
    v[5] = k110.found;
  } else {
    s[0] = sdf_interp(r, pt + mk3(1, 0, 0), v[0]);
    s[1] = sdf_interp(r, pt + mk3(-1, 0, 0), v[1]);
    s[2] = sdf_interp(r, pt + mk3(0, 1, 0), v[2]);
    s[3] = sdf_interp(r, pt + mk3(0, -1, 0), v[3]);
    s[4] = sdf_interp(r, pt + mk3(0, 0, 1), v[4]);
    s[5] = sdf_interp(r, pt + mk3(0, 0, -1), v[5]);
  }
#pragma unroll
  for (int k = 0; k < 6; ++k)
    if (isnan(s[k]) || s[k] == 1.0f || !v[k]) return o;
  o.n = normalised(mul(Rinv, mk3(s[0] - s[1], s[2] - s[3], s[4] - s[5])));
  o.ok = true;
  return o;
}

constexpr int kSpec = 4;  // march samples read ahead together

// One ray's march, Rendering::operator() (RenderScene.cu:395-447): the
// ray from the z-range's near to far point, 8-voxel steps through empty or
// unobserved space, 1-voxel steps in observed voxels, readSdfInterped near
// the surface, and the stop at a sign change.  The march reads kSpec
// samples ahead at once, at the positions a run of 1-voxel steps would
// reach (the same float additions), then replays the loop over them in
// order; an 8-voxel step or the end of the range ends the run.  Besides the
// reference's state it records, for the adjoint, how far along the ray the
// final position and the sample that gave the final sdf lie.
struct MarchState {
  f3 block_s, block_e, dir;  // ray ends and direction (voxel units)
  f3 ps, pe;                 // the same ends in the world frame (metres)
  f3 result;                 // final position
  float sdf;                 // final sdf
  f3 sample;                 // position of the sample that gave sdf
  float s_result, s_sample;  // distances of result and of sdf's sample from block_s
  bool interp;               // sdf came from readSdfInterped
  bool behind;
};

__device__ __forceinline__ void march_ray(const RayCtx &r, const Cam &c, float vsi, int x, int y, float zx,
                                          float zy, MarchState &ms) {
  float sdf = 1.0f;
  f3 p;
  p.z = zx;
  p.x = p.z * ((float)x - c.cx) * c.invfx;
  p.y = p.z * ((float)y - c.cy) * c.invfy;
  float dist_s = norm(p) * vsi;
  const float dist0 = dist_s;
  ms.ps = mul(c.R, p) + c.t;
  const f3 block_s = ms.ps * vsi;
  p.z = zy;
  p.x = p.z * ((float)x - c.cx) * c.invfx;
  p.y = p.z * ((float)y - c.cy) * c.invfy;
  const float dist_e = norm(p) * vsi;
  ms.pe = mul(c.R, p) + c.t;
  const f3 block_e = ms.pe * vsi;
  const f3 dir = normalised(block_e - block_s);
  f3 result = block_s;
  bool valid_sdf = false, behind = false, done = false, interp = false;
  float s_sample = 0.f;
  f3 sample = block_s;
  BlockCache cache;
  cache.bx = 0x7fffffff; cache.by = 0; cache.bz = 0; cache.ptr = -1;
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
    read_voxels<kSpec>(r, pos, v, cache);
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
      s_sample = ds[i] - dist0;
      sample = pos[i];
      interp = false;
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
        interp = true;
      }
      if (prev_sdf < 0.f && sdf >= 0.f) {
        behind = true;
        done = true;
        break;
      }
      if (prev_sdf > 0.f && sdf <= 0.f) {
        result = pos[i];
        dist_s = ds[i];
        done = true;
        break;
      }
      if (i == kSpec - 1) {  // every speculated sample consumed
        result = pos[i] + 1.0f * dir;
        dist_s = ds[i] + 1.0f;
      }
    }
  }
  ms.block_s = block_s;
  ms.block_e = block_e;
  ms.dir = dir;
  ms.result = result;
  ms.sdf = sdf;
  ms.s_result = dist_s - dist0;
  ms.s_sample = s_sample;
  ms.sample = sample;
  ms.interp = interp;
  ms.behind = behind;
}

__device__ __forceinline__ RayCtx ray_ctx(const DevMap &m, const FuseScratch &f) {
  RayCtx r;
  r.voxels = m.voxels;
  r.cells = f.win_cells;
  for (int k = 0; k < 6; ++k) r.win[k] = f.win[k];
  ray_ctx_map(r, m);
  return r;
}

// One pixel of Rendering::operator() (RenderScene.cu:380-488): the z-range
// test, the march, the two refinement steps, the normal, and the write.
__device__ __forceinline__ void raycast_pixel(const RayCtx &r, const Cam &c, const MapConst &mc,
                                              const sf_image &zmin, const sf_image &zmax, int x, int y,
                                              const sf_image &vmap, const sf_image &nmap) {
  float4 vout = nan4(), nout = nan4();
  const int lx = (int)floorf((float)x / 8.0f), ly = (int)floorf((float)y / 8.0f);
  const float zx = __ldg(row_ptr<const float>(zmin, ly) + lx);
  const float zy = __ldg(row_ptr<const float>(zmax, ly) + lx);
  // (double)z < 1e-3 of the reference: no float lies in [1e-3, 0.001f), so
  // for a float z that is exactly z < 0.001f
  if (!(zy < 0.001f || zx < 0.001f || isnan(zx) || isnan(zy))) {
    MarchState ms;
    march_ray(r, c, mc.voxel_size_inv, x, y, zx, zy, ms);
    f3 result = ms.result;
    const f3 dir = ms.dir;
    float sdf = ms.sdf;
    const bool behind = ms.behind;
    if (!behind && sdf <= 0.0f) {
      float step = sdf * mc.step_scale;
      result = result + step * dir;
      sdf = read_sdf_interp(r, result).sdf;
      step = sdf * mc.step_scale;
      result = result + step * dir;
      const NormalOut no = read_normal(r, result, c.Rinv);
      if (no.ok) {
        const f3 q = mul(c.Rinv, result * mc.voxel_size - c.t);
        vout = make_float4(q.x, q.y, q.z, 1.0f);
        nout = make_float4(no.n.x, no.n.y, no.n.z, 1.0f);
      }
    }
  }
  row_ptr<float4>(vmap, y)[x] = vout;
  row_ptr<float4>(nmap, y)[x] = nout;
}

// Rendering::operator() (RenderScene.cu:380-488).  The march reads kSpec
// samples ahead at once, at the positions a run of 1-voxel steps would
// reach (the same float additions), then replays the reference's loop over
// them in order; an 8-voxel step or the end of the range ends the run.
// 128-thread CTAs with the registers sized for MINB of them per SM: the
// march is latency-bound and gains more from the extra warps than it
// loses to a few spilled values (measured on GB300: 6 and 8 per SM are
// best, 10 and more spill too much); both are built and the autotuner
// picks between them and among tile shapes.
template <int MINB>
__global__ void __launch_bounds__(128, MINB) k_raycast(DevMap m, FuseScratch f, sf_image vmap, sf_image nmap,
                                                       sf_image zmin, sf_image zmax, const Cam *cam,
                                                       const unsigned *rendered, sf_image fb_v,
                                                       sf_image fb_n, const int *run_flag, FrameStatsArgs stats) {
  // the frame's statistics are final when its last raycast starts
  if (stats.sys && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0)
    sys_stats(stats.sys, *stats.ctl, m, stats.flags, stats.out, stats.host_out, stats.host_ready, stats.seq);
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
  raycast_pixel(ray_ctx(m, f), c, m.c, zmin, zmax, x, y, vmap, nmap);
}

// Tracker::ValidatePose's RayTrace of n candidates in one launch
// (Tracking.cc:759-761): grid.z is the candidate; a candidate draws into
// its `rows`-row slice of the tall model maps from its zr-row slice of the
// tall z-range images, and only when src[c] == c (its visible count
// reached the threshold and a block projected).
__global__ void __launch_bounds__(128, 8) k_raycast_batch(DevMap m, FuseScratch f, sf_image vmap, sf_image nmap,
                                                          int rows, sf_image zmin, sf_image zmax, int zr,
                                                          const Cam *cams, const int *src) {
  const int k = blockIdx.z;
  if (src[k] != k) return;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= vmap.cols || y >= rows) return;
  sf_image v = vmap, n = nmap, zn = zmin, zx = zmax;
  v.data = (char *)vmap.data + (size_t)k * rows * vmap.step;
  n.data = (char *)nmap.data + (size_t)k * rows * nmap.step;
  zn.data = (char *)zmin.data + (size_t)k * zr * zmin.step;
  zx.data = (char *)zmax.data + (size_t)k * zr * zmax.step;
  v.rows = n.rows = rows;
  zn.rows = zx.rows = zr;
  const Cam c = cams[k];
  raycast_pixel(ray_ctx(m, f), c, m.c, zn, zx, x, y, v, n);
}

// RaycastAdjoint: gradient of the raycast's vertex and normal maps with
// respect to the camera pose and the TSDF values the rendering read.  Each
// ray is marched again with march_ray (the same samples and decisions), so
// nothing is stored between the forward and backward passes.  The march's
// outcome (where the sign change lies, which samples were interpolated) is
// piecewise constant and held fixed; the gradient flows through
//   p1 = p0 + ss * sdf_c * dir,  p2 = p1 + ss * interp(p1) * dir,
//   v = R^T (p2 * voxel - t),  n = normalised(R^T g),
//   g = (s(p2+x) - s(p2-x), s(p2+y) - s(p2-y), s(p2+z) - s(p2-z)),
// the ray's ends (world points R p + t) and its direction.  The pose is
// perturbed on the left, T(xi) = exp(xi) T, with xi = (rho, omega) in
// Sophus's order (translation first).  TSDF gradients are added into
// grad_sdf at the voxel index (ptr + local) with atomics; the pose gradient
// is summed per CTA in a fixed order into pose_part.
__global__ void __launch_bounds__(128) k_raycast_adjoint(DevMap m, FuseScratch f, sf_image zmin,
                                                         sf_image zmax, const Cam *cam, sf_image gv_img,
                                                         sf_image gn_img, float *grad_sdf, float *pose_part) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  float gp[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (x < gv_img.cols && y < gv_img.rows) {
    const float4 gv4 = __ldg(row_ptr<const float4>(gv_img, y) + x);
    const float4 gn4 = gn_img.data ? __ldg(row_ptr<const float4>(gn_img, y) + x) : make_float4(0.f, 0.f, 0.f, 0.f);
    f3 gv = xyz(gv4), gn = xyz(gn4);
    if (isnan(gv.x) || isnan(gv.y) || isnan(gv.z)) gv = mk3(0.f, 0.f, 0.f);
    if (isnan(gn.x) || isnan(gn.y) || isnan(gn.z)) gn = mk3(0.f, 0.f, 0.f);
    const Cam c = *cam;
    const int lx = (int)floorf((float)x / 8.0f), ly = (int)floorf((float)y / 8.0f);
    const float zx = __ldg(row_ptr<const float>(zmin, ly) + lx);
    const float zy = __ldg(row_ptr<const float>(zmax, ly) + lx);
    const bool any = gv.x != 0.f || gv.y != 0.f || gv.z != 0.f || gn.x != 0.f || gn.y != 0.f || gn.z != 0.f;
    if (any && !(zy < 0.001f || zx < 0.001f || isnan(zx) || isnan(zy))) {
      RayCtx r;
      r.voxels = m.voxels;
      r.cells = f.win_cells;
      for (int k = 0; k < 6; ++k) r.win[k] = f.win[k];
      ray_ctx_map(r, m);
      MarchState ms;
      march_ray(r, c, m.c.voxel_size_inv, x, y, zx, zy, ms);
      if (!ms.behind && ms.sdf <= 0.0f) {
        const float ss = m.c.step_scale, vs = m.c.voxel_size;
        const f3 dir = ms.dir;
        const f3 p1 = ms.result + (ms.sdf * ss) * dir;
        const float s1 = read_sdf_interp(r, p1).sdf;
        const f3 p2 = p1 + (s1 * ss) * dir;
        const f3 ex = mk3(1, 0, 0), ey = mk3(0, 1, 0), ez = mk3(0, 0, 1);
        bool v0, v1, v2, v3, v4, v5;
        const float n0 = sdf_interp(r, p2 + ex, v0), n1 = sdf_interp(r, p2 + mk3(-1, 0, 0), v1);
        const float n2 = sdf_interp(r, p2 + ey, v2), n3 = sdf_interp(r, p2 + mk3(0, -1, 0), v3);
        const float n4 = sdf_interp(r, p2 + ez, v4), n5 = sdf_interp(r, p2 + mk3(0, 0, -1), v5);
        const bool ok = !(isnan(n0) || n0 == 1.0f || !v0) && !(isnan(n1) || n1 == 1.0f || !v1) &&
                        !(isnan(n2) || n2 == 1.0f || !v2) && !(isnan(n3) || n3 == 1.0f || !v3) &&
                        !(isnan(n4) || n4 == 1.0f || !v4) && !(isnan(n5) || n5 == 1.0f || !v5);
        if (ok) {
          // vertex v = R^T (q - t), q = p2 * voxel
          const f3 q = p2 * vs;
          const f3 gq = mul(c.R, gv);
          f3 grho = -gq;
          f3 gom = cross(gq, q);
          f3 gp2 = gq * vs;
          // normal n = u / |u|, u = R^T g
          const f3 gr = mk3(n0 - n1, n2 - n3, n4 - n5);
          const f3 u = mul(c.Rinv, gr);
          const float un = norm(u);
          const f3 nn = u / un;
          const f3 gu = (gn - nn * dot(nn, gn)) / un;
          const f3 ggr = mul(c.R, gu);
          gom = gom + cross(ggr, gr);
          gp2 = gp2 + ggr.x * sdf_interp_bwd(r, p2 + ex, ggr.x, grad_sdf);
          gp2 = gp2 - ggr.x * sdf_interp_bwd(r, p2 + mk3(-1, 0, 0), -ggr.x, grad_sdf);
          gp2 = gp2 + ggr.y * sdf_interp_bwd(r, p2 + ey, ggr.y, grad_sdf);
          gp2 = gp2 - ggr.y * sdf_interp_bwd(r, p2 + mk3(0, -1, 0), -ggr.y, grad_sdf);
          gp2 = gp2 + ggr.z * sdf_interp_bwd(r, p2 + ez, ggr.z, grad_sdf);
          gp2 = gp2 - ggr.z * sdf_interp_bwd(r, p2 + mk3(0, 0, -1), -ggr.z, grad_sdf);
          // p2 = p1 + ss * s1 * dir
          f3 gp1 = gp2;
          const float gs1 = ss * dot(dir, gp2);
          f3 gdir = (ss * s1) * gp2;
          gp1 = gp1 + gs1 * sdf_interp_bwd(r, p1, gs1, grad_sdf);
          // p1 = p0 + ss * sdf_c * dir; sdf_c read at ms.sample
          const f3 gp0 = gp1;
          const float gsc = ss * dot(dir, gp1);
          gdir = gdir + (ss * ms.sdf) * gp1;
          f3 gsmp = mk3(0.f, 0.f, 0.f);
          if (ms.interp) {
            gsmp = gsc * sdf_interp_bwd(r, ms.sample, gsc, grad_sdf);
          } else if (grad_sdf && gsc != 0.f) {
            const i3 pv = floor3(ms.sample);
            const int ptr = block_ptr(r, pv.x >> 3, pv.y >> 3, pv.z >> 3);
            if (ptr >= 0) atomicAdd(grad_sdf + ptr + ((pv.z & 7) * 64 + (pv.y & 7) * 8 + (pv.x & 7)), gsc);
          }
          // p0 = block_s + s_result * dir, sample = block_s + s_sample * dir
          f3 gbs = gp0 + gsmp;
          gdir = gdir + ms.s_result * gp0 + ms.s_sample * gsmp;
          // dir = normalised(block_e - block_s)
          const f3 d = ms.block_e - ms.block_s;
          const float dn = norm(d);
          const f3 gd = (gdir - dir * dot(dir, gdir)) / dn;
          const f3 gbe = gd;
          gbs = gbs - gd;
          // block_s = (R p + t) / voxel, block_e likewise; world points move by omega x w + rho
          const float vsi = m.c.voxel_size_inv;
          const f3 gws = gbs * vsi, gwe = gbe * vsi;
          grho = grho + gws + gwe;
          gom = gom + cross(ms.ps, gws) + cross(ms.pe, gwe);
          gp[0] = grho.x; gp[1] = grho.y; gp[2] = grho.z;
          gp[3] = gom.x; gp[4] = gom.y; gp[5] = gom.z;
        }
      }
    }
  }
  // fixed-order CTA sum of the pose gradient
  __shared__ float wpart[4][6];
  const int tid = threadIdx.y * blockDim.x + threadIdx.x, lane = tid & 31, warp = tid >> 5;
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    float v = gp[k];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if (lane == 0) wpart[warp][k] = v;
  }
  __syncthreads();
  if (tid < 6) {
    const float v = ((wpart[0][tid] + wpart[1][tid]) + wpart[2][tid]) + wpart[3][tid];
    pose_part[(size_t)(blockIdx.y * gridDim.x + blockIdx.x) * 6 + tid] = v;
  }
}

// Sum of the CTA pose partials in FP64, fixed order.
__global__ void k_pose_grad_sum(const float *part, int n, double *out) {
  __shared__ double w[8][6];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (int i = threadIdx.x; i < n; i += blockDim.x)
#pragma unroll
    for (int k = 0; k < 6; ++k) acc[k] += (double)part[(size_t)i * 6 + k];
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    double v = acc[k];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if (lane == 0) w[warp][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    double v = 0.0;
    for (int q = 0; q < (int)(blockDim.x / 32); ++q) v += w[q][threadIdx.x];
    out[threadIdx.x] = v;
  }
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

// Window over the bounding box of every allocated block: box[0..2] min,
// box[3..5] max block coordinates.
__global__ void k_window_box_init(int *box) {
  if (threadIdx.x < 3) box[threadIdx.x] = 0x7fffffff;
  else if (threadIdx.x < 6) box[threadIdx.x] = (int)0x80000000;
}
__global__ void k_window_box_reduce(DevMap m, int *box) {
  const unsigned n = (unsigned)*m.alloc_count;
  int lo[3] = {0x7fffffff, 0x7fffffff, 0x7fffffff}, hi[3] = {(int)0x80000000, (int)0x80000000, (int)0x80000000};
  for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int4 h = entry_head(m.entries + m.alloc_list[k]);
    if (h.w < 0) continue;
    const int p[3] = {h.x, h.y, h.z};
    for (int d = 0; d < 3; ++d) { lo[d] = min(lo[d], p[d]); hi[d] = max(hi[d], p[d]); }
  }
  for (int d = 0; d < 3; ++d) {
    lo[d] = __reduce_min_sync(0xffffffffu, lo[d]);
    hi[d] = __reduce_max_sync(0xffffffffu, hi[d]);
  }
  if ((threadIdx.x & 31) == 0) {
    for (int d = 0; d < 3; ++d) {
      atomicMin(box + d, lo[d]);
      atomicMax(box + 3 + d, hi[d]);
    }
  }
}
__global__ void k_window_box_setup(FuseScratch f, const int *box) {
  long long total = 1;
  int n[3];
  for (int d = 0; d < 3; ++d) {
    n[d] = box[3 + d] >= box[d] ? box[3 + d] - box[d] + 1 : 0;
    total *= n[d];
  }
  if (total <= 0 || total > (long long)f.win_cap) n[0] = n[1] = n[2] = 0;
  for (int d = 0; d < 3; ++d) {
    f.win[d] = n[0] ? box[d] : 0;
    f.win[3 + d] = n[d];
  }
}

}  // namespace

void launch_window_alloc_box(const DevMap &m, const FuseScratch &f, int *box, cudaStream_t s) {
  k_window_box_init<<<1, 32, 0, s>>>(box); note_launch();
  k_window_box_reduce<<<256, 256, 0, s>>>(m, box); note_launch();
  k_window_box_setup<<<1, 1, 0, s>>>(f, box); note_launch();
  k_window_build_clear<<<256, 256, 0, s>>>(f); note_launch();
  k_window_build_fill<<<256, 256, 0, s>>>(m, f); note_launch();
}

void launch_raycast_batch(const DevMap &m, const FuseScratch &f, const sf_image &vmap, const sf_image &nmap,
                          int rows, const sf_image &zmin, const sf_image &zmax, int zr, const Cam *cams, int n,
                          const int *src, cudaStream_t s) {
  const dim3 blk(8, 16);
  const dim3 grd((vmap.cols + 7) / 8, (rows + 15) / 16, n);
  k_raycast_batch<<<grd, blk, 0, s>>>(m, f, vmap, nmap, rows, zmin, zmax, zr, cams, src); note_launch();
}

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

RaycastTune raycast_tune(int i) {
  static const int shapes[3][2] = {{8, 16}, {16, 8}, {32, 4}};
  RaycastTune t;
  t.minb = i < 3 ? 8 : 6;
  t.tx = shapes[i % 3][0];
  t.ty = shapes[i % 3][1];
  return t;
}

void launch_raycast(const DevMap &m, const FuseScratch &f, const sf_image &vmap, const sf_image &nmap,
                    const sf_image &zmin, const sf_image &zmax, const Cam *c,
                    const unsigned *rendered, const sf_image *fallback_v,
                    const sf_image *fallback_n, const int *run_flag, cudaStream_t s,
                    const RaycastTune &tune, const FrameStatsArgs *stats) {
  const dim3 blk(tune.tx, tune.ty);
  const dim3 grd((vmap.cols + tune.tx - 1) / tune.tx, (vmap.rows + tune.ty - 1) / tune.ty);
  sf_image fv = fallback_v ? *fallback_v : sf_image{};
  sf_image fn = fallback_n ? *fallback_n : sf_image{};
  FrameStatsArgs st = {};
  if (stats) st = *stats;
  if (tune.minb == 6)
    k_raycast<6><<<grd, blk, 0, s>>>(m, f, vmap, nmap, zmin, zmax, c, rendered, fv, fn, run_flag, st);
  else
    k_raycast<8><<<grd, blk, 0, s>>>(m, f, vmap, nmap, zmin, zmax, c, rendered, fv, fn, run_flag, st);
  note_launch();
}

int raycast_adjoint_blocks(int cols, int rows) { return ((cols + 7) / 8) * ((rows + 15) / 16); }

void launch_raycast_adjoint(const DevMap &m, const FuseScratch &f, const sf_image &zmin, const sf_image &zmax,
                            const Cam *c, const sf_image &gv, const sf_image &gn, float *grad_sdf,
                            float *pose_part, double *pose_out, cudaStream_t s) {
  dim3 blk(8, 16);
  dim3 grd((gv.cols + 7) / 8, (gv.rows + 15) / 16);
  k_raycast_adjoint<<<grd, blk, 0, s>>>(m, f, zmin, zmax, c, gv, gn, grad_sdf, pose_part); note_launch();
  k_pose_grad_sum<<<1, 256, 0, s>>>(pose_part, (int)(grd.x * grd.y), pose_out); note_launch();
}

void launch_window_build(const DevMap &m, const FuseScratch &f, const Cam *c, cudaStream_t s) {
  k_window_build_setup<<<1, 1, 0, s>>>(m, f, c); note_launch();
  k_window_build_clear<<<256, 256, 0, s>>>(f); note_launch();
  k_window_build_fill<<<256, 256, 0, s>>>(m, f); note_launch();
}

}  // namespace sf
