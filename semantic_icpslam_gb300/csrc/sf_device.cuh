// Device-side data model and exact-arithmetic helpers shared by the kernels.
//
// Every .cu file of the library is compiled with -fmad=false, so each float
// + - * / and sqrtf rounds once (IEEE-754, round to nearest) exactly as the
// reference's source states the expression; values the reference promotes
// to double are computed in double.  With that, integer outputs (allocated
// blocks, visible sets, weights, label counts) are bit-exact against the
// CPU oracle, which is built with -ffp-contract=off.
#ifndef SF_DEVICE_CUH_
#define SF_DEVICE_CUH_

#include <cuda_runtime.h>
#include <stdint.h>

#include "sfusion.h"

namespace sf {

// ------------------------------------------------------------ vector math
struct f3 { float x, y, z; };
struct m3 { f3 rx, ry, rz; };  // Matrix3f rows (Utility/VectorMath.h:360-375)
struct i3 { int x, y, z; };
__host__ __device__ __forceinline__ i3 mk_i3(int x, int y, int z) {
  i3 r;
  r.x = x; r.y = y; r.z = z;
  return r;
}

__device__ __forceinline__ f3 mk3(float x, float y, float z) { f3 r; r.x = x; r.y = y; r.z = z; return r; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ f3 operator-(f3 a) { return mk3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ f3 operator*(f3 a, float b) { return mk3(a.x * b, a.y * b, a.z * b); }
__device__ __forceinline__ f3 operator*(float a, f3 b) { return mk3(a * b.x, a * b.y, a * b.z); }
__device__ __forceinline__ f3 operator/(f3 a, float b) { return mk3(a.x / b, a.y / b, a.z / b); }
// float3 . float3 (VectorMath.h:195-197): ((ax*bx + ay*by) + az*bz)
__device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 cross(f3 a, f3 b) {  // VectorMath.h:312-316
  return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float norm(f3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ f3 normalised(f3 a) { return a / norm(a); }
__device__ __forceinline__ f3 mul(const m3 &m, f3 a) { return mk3(dot(m.rx, a), dot(m.ry, a), dot(m.rz, a)); }
__device__ __forceinline__ f3 xyz(float4 v) { return mk3(v.x, v.y, v.z); }

__host__ __device__ __forceinline__ m3 to_m3(const sf_mat3 &m) {
  m3 r;
  r.rx.x = m.rowx.x; r.rx.y = m.rowx.y; r.rx.z = m.rowx.z;
  r.ry.x = m.rowy.x; r.ry.y = m.rowy.y; r.ry.z = m.rowy.z;
  r.rz.x = m.rowz.x; r.rz.y = m.rowz.y; r.rz.z = m.rowz.z;
  return r;
}
__host__ __device__ __forceinline__ f3 to_f3(const sf_float3 &v) { f3 r; r.x = v.x; r.y = v.y; r.z = v.z; return r; }

// (int) casts compile to cvt.rzi: NaN -> 0, out-of-range saturates.
__device__ __forceinline__ int f2i(float v) { return (int)v; }
__device__ __forceinline__ int d2i(double v) { return (int)v; }
// make_int3(float3) == floor (VectorMath.h:36-42).
__device__ __forceinline__ i3 floor3(f3 a) {
  i3 b;
  b.x = (int)a.x; b.y = (int)a.y; b.z = (int)a.z;
  b.x = (float)b.x > a.x ? b.x - 1 : b.x;
  b.y = (float)b.y > a.y ? b.y - 1 : b.y;
  b.z = (float)b.z > a.z ? b.z - 1 : b.z;
  return b;
}
// make_uchar3(float3) (VectorMath.h:16-18): int cast, then uchar narrowing.
__device__ __forceinline__ uint8_t f2u8(float v) { return (uint8_t)(uint32_t)(int)v; }

__device__ __forceinline__ float nanf_bits() { return __int_as_float(0x7fffffff); }
__device__ __forceinline__ float4 nan4() { float n = nanf_bits(); return make_float4(n, n, n, n); }

// ------------------------------------------------------------- images
template <class T>
__device__ __forceinline__ T *row_ptr(const sf_image &im, int y) {
  return (T *)((char *)im.data + (size_t)y * im.step);
}

// ----------------------------------------------------------------- map
// Map constants: the reference's constexpr expressions evaluated at runtime
// with the same precision (Mapping/DeviceMap.h:166-189).
struct MapConst {
  float voxel_size, voxel_size_inv, block_width, trunc_dist, step_scale;
  float depth_min, depth_max;
  uint32_t num_buckets, num_excess, num_sdf_blocks, num_entries, max_rendering_blocks;
};

struct DevMap {
  sf_hash_entry *entries;   // [num_entries]
  sf_voxel *voxels;         // [num_sdf_blocks * 512]
  int *heap;                // [num_sdf_blocks]
  int *heap_counter;        // [1]
  int *entry_ptr;           // [1]
  int *bucket_mutex;        // [num_buckets] (layout only; allocation is lock-free)
  uint32_t *no_visible;     // [1]
  sf_hash_entry *visible;   // [num_entries]
  // index of allocated entries (ptr >= 0), in allocation order
  int *alloc_list;          // [num_entries]
  int *alloc_count;         // [1]
  uint32_t *status;         // [1] SF_BOUND_* bits of the bounds-checked build (else stays 0)
  MapConst c;
};

// ------------------------------------------------- bounds-checked build
// Built with -DSF_BOUNDS_CHECK (the debug library, build.py's
// debug_bounds), every hash-chain link and every voxel index taken from a
// hash entry or the block window is checked before use: an index outside
// its array, or a block pointer that is not a multiple of 512, records its
// SF_BOUND_* bit in the map's status word and the access is skipped (the
// lookup finds no block).  This stands in for a memory checker against
// corrupted maps and the reference's allocation races
// (Mapping/DeviceMap.cu:23-69).  The release build compiles the checks out.
enum : uint32_t {
  SF_BOUND_CHAIN = 1u << 0,   // an excess-chain link beyond the table
  SF_BOUND_PTR = 1u << 1,     // a block pointer outside the voxel array or not block-aligned
  SF_BOUND_VISIBLE = 1u << 2, // a visible-list index beyond the table
};
#ifdef SF_BOUNDS_CHECK
__device__ __forceinline__ bool bound_ok(const DevMap &m, bool ok, uint32_t bit) {
  if (!ok) atomicOr(m.status, bit);
  return ok;
}
#else
__device__ __forceinline__ bool bound_ok(const DevMap &, bool, uint32_t) { return true; }
#endif
// A block pointer read from the table or the window: -1 stays -1; a
// pointer the checked build rejects reads as -1 (no block).
__device__ __forceinline__ int checked_ptr(const DevMap &m, int ptr) {
  if (ptr < 0) return ptr;
  return bound_ok(m, (ptr & 511) == 0 && (uint32_t)ptr < m.c.num_sdf_blocks * 512u, SF_BOUND_PTR) ? ptr : -1;
}

// DeviceMap::Hash (Mapping/DeviceMap.cu:3-10).  NumBuckets is unsigned, so
// the signed product-xor is taken modulo NumBuckets as an unsigned value.
// A power-of-two bucket count (every shipped map size) takes the mask,
// which equals the remainder and avoids the ~20-instruction integer
// division; any other count divides.
__device__ __forceinline__ uint32_t hash_block(i3 p, uint32_t nb) {
  uint32_t h = ((uint32_t)p.x * 73856093u) ^ ((uint32_t)p.y * 19349669u) ^ ((uint32_t)p.z * 83492791u);
  return (nb & (nb - 1u)) == 0u ? (h & (nb - 1u)) : h % nb;
}
// voxelPosToBlockPos (DeviceMap.cu:169-180)
__device__ __forceinline__ i3 vox2block(i3 v) {
  if (v.x < 0) v.x -= 7;
  if (v.y < 0) v.y -= 7;
  if (v.z < 0) v.z -= 7;
  i3 r; r.x = v.x / 8; r.y = v.y / 8; r.z = v.z / 8;
  return r;
}
// voxelPosToLocalIdx (DeviceMap.cu:186-201,218-220)
__device__ __forceinline__ int vox2local(i3 v) {
  int lx = v.x % 8, ly = v.y % 8, lz = v.z % 8;
  if (lx < 0) lx += 8;
  if (ly < 0) ly += 8;
  if (lz < 0) lz += 8;
  return lz * 64 + ly * 8 + lx;
}

// 32-byte entry as two 16-byte loads: {x, y, z, ptr}, {offset, pad}.
__device__ __forceinline__ int4 entry_head(const sf_hash_entry *e) { return __ldcg((const int4 *)e); }
__device__ __forceinline__ int entry_offset(const sf_hash_entry *e) { return __ldcg(&e->offset); }

// DeviceMap::FindEntry (DeviceMap.cu:141-154).  Returns ptr (>= 0) or -1.
// The lookup given the head and offset of p's bucket entry, already loaded
// (so that several lookups can have their first loads in flight at once).
__device__ __forceinline__ int find_block_from(const DevMap &m, i3 p, int4 h, int off) {
  if (h.w != -1 && h.x == p.x && h.y == p.y && h.z == p.z) return checked_ptr(m, h.w);
  int guard = 0;
  while (off > 0) {
    if (!bound_ok(m, (uint32_t)off <= m.c.num_excess, SF_BOUND_CHAIN)) break;
    const sf_hash_entry *e = m.entries + (m.c.num_buckets + (uint32_t)off - 1u);
    h = entry_head(e);
    if (h.x == p.x && h.y == p.y && h.z == p.z && h.w != -1) return checked_ptr(m, h.w);
    off = entry_offset(e);
    if (++guard > (int)m.c.num_excess) break;  // corrupted chain: stop
  }
  return -1;
}
__device__ __forceinline__ int find_block(const DevMap &m, i3 p) {
  const sf_hash_entry *e = m.entries + hash_block(p, m.c.num_buckets);
  return find_block_from(m, p, entry_head(e), entry_offset(e));
}

// ------------------------------------------------------- device flags
enum : uint32_t {
  SF_FLAG_DEDUP_FULL = 1u << 0,      // allocation request set overflowed
  SF_FLAG_PENDING_FULL = 1u << 1,    // allocation pending list overflowed
  SF_FLAG_HEAP_EMPTY = 1u << 2,      // voxel-block heap exhausted
  SF_FLAG_EXCESS_FULL = 1u << 3,     // excess list exhausted
  SF_FLAG_VISIBLE_FULL = 1u << 4,    // visible list overflowed
  SF_FLAG_RENDER_FULL = 1u << 5,     // rendering-block list overflowed
  SF_FLAG_BARRIER_TIMEOUT = 1u << 6, // a bounded grid barrier gave up
  SF_FLAG_COORD_RANGE = 1u << 7,     // block coordinate outside +-32767
};

}  // namespace sf
#endif
