// Map sampling shared by the raycast and the relocalisation scorer: block
// lookups through the frame's block-pointer window with the hash table
// behind it, voxel reads and readSdfInterped (RenderScene.cu:310-343).
#ifndef SF_SAMPLE_CUH_
#define SF_SAMPLE_CUH_

#include "sf_kernels.cuh"

namespace sf {
namespace {

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
#ifdef SF_BOUNDS_CHECK
  uint32_t *status;  // the map's bounds status word
  uint32_t num_sdf_blocks;
#endif
};

// The map fields a RayCtx carries besides the arrays.
__device__ __forceinline__ void ray_ctx_map(RayCtx &r, const DevMap &m) {
  r.entries = m.entries;
  r.num_buckets = m.c.num_buckets;
  r.num_excess = m.c.num_excess;
#ifdef SF_BOUNDS_CHECK
  r.status = m.status;
  r.num_sdf_blocks = m.c.num_sdf_blocks;
#endif
}

// Hash-table lookup (DeviceMap::FindEntry) for a block outside the window;
// rare, so kept out of line to keep the inlined sample code small.
#ifdef SF_BOUNDS_CHECK
__device__ __noinline__ int block_ptr_hash(const RayCtx r, int bx, int by, int bz) {
  DevMap m;
  m.entries = const_cast<sf_hash_entry *>(r.entries);
  m.c.num_buckets = r.num_buckets;
  m.c.num_excess = r.num_excess;
  m.c.num_sdf_blocks = r.num_sdf_blocks;
  m.status = r.status;
  i3 p;
  p.x = bx; p.y = by; p.z = bz;
  return find_block(m, p);
}
#else
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
#endif

// Voxel index of block (bx, by, bz), or -1.
__device__ __forceinline__ int block_ptr(const RayCtx &r, int bx, int by, int bz) {
  const unsigned x = (unsigned)(bx - r.win[0]), y = (unsigned)(by - r.win[1]), z = (unsigned)(bz - r.win[2]);
#ifdef SF_BOUNDS_CHECK
  if (x < (unsigned)r.win[3] && y < (unsigned)r.win[4] && z < (unsigned)r.win[5]) {
    const int v = __ldg(r.cells + (int)((z * (unsigned)r.win[4] + y) * (unsigned)r.win[3] + x));
    if (v < 0 || ((v & 511) == 0 && (uint32_t)v < r.num_sdf_blocks * 512u)) return v;
    atomicOr(r.status, SF_BOUND_PTR);
    return -1;
  }
  return block_ptr_hash(r, bx, by, bz);
#else
  if (x < (unsigned)r.win[3] && y < (unsigned)r.win[4] && z < (unsigned)r.win[5])
    return __ldg(r.cells + (int)((z * (unsigned)r.win[4] + y) * (unsigned)r.win[3] + x));
  return block_ptr_hash(r.entries, r.num_buckets, r.num_excess, bx, by, bz);
#endif
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

// A ray's last looked-up block (DeviceMap::FindVoxel's per-ray entry cache,
// DeviceMap.cu:116-133): consecutive samples mostly fall in one block, and
// a hit skips the lookup, so the voxel read is the sample's only dependent
// load.  The cache changes no value (block_ptr is exact for every block).
struct BlockCache {
  int bx, by, bz, ptr;
};

// The voxels at n consecutive sample points, their block lookups issued
// together: a sample in the cached block or in the previous sample's block
// reuses that pointer.  The cache then holds the last sample's block.
template <int N>
__device__ __forceinline__ void read_voxels(const RayCtx &r, const f3 *pt, VoxelRead *v, BlockCache &cache) {
  i3 p[N];
  int ptr[N];
#pragma unroll
  for (int i = 0; i < N; ++i) {
    p[i] = floor3(pt[i]);
    const int bx = p[i].x >> 3, by = p[i].y >> 3, bz = p[i].z >> 3;
    const bool same_prev =
        i > 0 && bx == (p[i - 1].x >> 3) && by == (p[i - 1].y >> 3) && bz == (p[i - 1].z >> 3);
    if (same_prev)
      ptr[i] = ptr[i > 0 ? i - 1 : 0];
    else if (bx == cache.bx && by == cache.by && bz == cache.bz)
      ptr[i] = cache.ptr;
    else
      ptr[i] = block_ptr(r, bx, by, bz);
  }
#pragma unroll
  for (int i = 0; i < N; ++i) v[i] = voxel_in(r, ptr[i], p[i].x, p[i].y, p[i].z);
  cache.bx = p[N - 1].x >> 3;
  cache.by = p[N - 1].y >> 3;
  cache.bz = p[N - 1].z >> 3;
  cache.ptr = ptr[N - 1];
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


// Adjoint of sdf_interp at pt: adds g * (corner weight) to grad_sdf at each
// corner's voxel index (ptr + local) and returns d sdf_interp / d pt.  The
// corners and weights are sdf_interp's.  Corners in missing blocks get no
// gradient (their NaN value already makes the forward output invalid).
__device__ __forceinline__ f3 sdf_interp_bwd(const RayCtx &r, f3 pt, float g, float *grad_sdf) {
  const f3 f = pt - mk3(floorf(pt.x), floorf(pt.y), floorf(pt.z));
  const i3 a = floor3(pt);
  const i3 b = floor3(pt + mk3(1, 1, 1));
  float c[8];
  int idx[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int vx = (k & 1) ? b.x : a.x, vy = (k & 2) ? b.y : a.y, vz = (k & 4) ? b.z : a.z;
    const int ptr = block_ptr(r, vx >> 3, vy >> 3, vz >> 3);
    idx[k] = ptr < 0 ? -1 : ptr + ((vz & 7) * 64 + (vy & 7) * 8 + (vx & 7));
    c[k] = ptr < 0 ? 0.f : __ldg(&r.voxels[idx[k]].sdf);
  }
  const float wx[2] = {1.0f - f.x, f.x}, wy[2] = {1.0f - f.y, f.y}, wz[2] = {1.0f - f.z, f.z};
  if (grad_sdf && g != 0.f) {
#pragma unroll
    for (int k = 0; k < 8; ++k)
      if (idx[k] >= 0) atomicAdd(grad_sdf + idx[k], g * (wx[k & 1] * wy[(k >> 1) & 1] * wz[(k >> 2) & 1]));
  }
  // d/dfx, d/dfy, d/dfz of the trilinear form
  const float dx = wz[0] * (wy[0] * (c[1] - c[0]) + wy[1] * (c[3] - c[2])) +
                   wz[1] * (wy[0] * (c[5] - c[4]) + wy[1] * (c[7] - c[6]));
  const float dy = wz[0] * (wx[0] * (c[2] - c[0]) + wx[1] * (c[3] - c[1])) +
                   wz[1] * (wx[0] * (c[6] - c[4]) + wx[1] * (c[7] - c[5]));
  const float dz = wy[0] * (wx[0] * (c[4] - c[0]) + wx[1] * (c[5] - c[1])) +
                   wy[1] * (wx[0] * (c[6] - c[2]) + wx[1] * (c[7] - c[3]));
  return mk3(dx, dy, dz);
}

}  // namespace
}  // namespace sf
#endif
