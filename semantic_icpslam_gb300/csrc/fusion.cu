// Voxel-block hash allocation, visible-block compaction and TSDF / weight /
// colour / label integration.
//
// Reference: Mapping/DeviceMap.cu (Hash :3-10, CreateEntry :12-21,
// CreateBlock :23-69, FindEntry :141-154), Mapping/FuseMap.cu
// (CreateBlocks :92-132, CheckFullVisibility :134-168, createVoxels
// :432-507, analyzeSemantics :509-668, UnifyNeighbor :757-896,
// ResetHash/ResetSdfBlock :1251-1304) and Utility/ParallelScan.h
// (ComputeOffset).
//
// GB300 form:
//  * Allocation is two lock-free passes.  Probe: every raw-depth pixel walks
//    its truncation segment; a block missing from the table is entered once
//    into an epoch-tagged request set (64-bit CAS) and pushed onto its
//    bucket's request list (atomicExch).  Insert: one thread per bucket with
//    requests runs the reference's CreateBlock serially for that bucket's
//    requests, so no allocation is lost to the bucket mutex race and no
//    block is entered twice; heap pops (atomicSub) and excess slots
//    (atomicAdd) are the reference's.
//  * An index of allocated entries replaces the full-table scan of
//    CheckFullVisibility; visible entries are appended with one atomic per
//    warp.  The z-range tiles of the raycast (Projection + fillBlocks) are
//    laid down in the same pass.
//  * Integration is a persistent grid over the visible list, one voxel per
//    thread with 128-bit loads and stores; label fusion runs on the same
//    voxel in the same pass.
//  * UnifyNeighbor is two launches around a 4-byte-per-voxel buffer, so
//    every voxel updates from the pass-start state.
#include "sf_kernels.cuh"
#include "sf_render.cuh"

namespace sf {

MapConst make_map_const(const sf_map_config &cfg) {
  MapConst c;
  c.voxel_size = cfg.voxel_size;
  c.voxel_size_inv = (float)(1.0 / (double)cfg.voxel_size);  // DeviceMap.h:186
  c.block_width = cfg.voxel_size * 8.0f;                     // :187
  c.trunc_dist = cfg.trunc_dist;
  c.step_scale = (float)(0.5 * (double)cfg.trunc_dist * (double)c.voxel_size_inv);  // :189
  c.depth_min = cfg.depth_min;
  c.depth_max = cfg.depth_max;
  c.num_buckets = cfg.num_buckets;
  c.num_excess = cfg.num_excess;
  c.num_sdf_blocks = cfg.num_sdf_blocks;
  c.num_entries = cfg.num_buckets + cfg.num_excess;
  c.max_rendering_blocks = cfg.max_rendering_blocks;
  return c;
}

namespace {

__device__ __forceinline__ unsigned grid_tid() { return blockIdx.x * blockDim.x + threadIdx.x; }
__device__ __forceinline__ unsigned grid_stride() { return gridDim.x * blockDim.x; }

// Warp-aggregated append: one atomicAdd per warp for the lanes in `active`.
__device__ __forceinline__ unsigned warp_append(unsigned *counter, bool want) {
  unsigned mask = __ballot_sync(__activemask(), want);
  if (!want) return 0;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(mask) - 1;
  unsigned base = 0;
  if (lane == leader) base = atomicAdd(counter, (unsigned)__popc(mask));
  base = __shfl_sync(mask, base, leader);
  return base + __popc(mask & ((1u << lane) - 1u));
}

// ---------------------------------------------------------------- reset
__global__ void k_reset_entries(DevMap m, int *bucket_head) {
  for (unsigned i = grid_tid(); i < m.c.num_entries; i += grid_stride()) {
    int4 *e = (int4 *)(m.entries + i);
    e[0] = make_int4(0, 0, 0, -1);
    e[1] = make_int4(0, 0, 0, 0);
    int4 *v = (int4 *)(m.visible + i);
    v[0] = make_int4(0, 0, 0, -1);
    v[1] = make_int4(0, 0, 0, 0);
    if (i < m.c.num_buckets) {
      m.bucket_mutex[i] = -1;
      if (bucket_head) bucket_head[i] = -1;
    }
  }
}

// ResetSdfBlockKernel (FuseMap.cu:1268-1289): heap[x] = N-1-x and every
// voxel released (sdf NaN, all counters 0; obj_idx is left as is).
__global__ void k_reset_voxels(DevMap m) {
  const size_t nvox = (size_t)m.c.num_sdf_blocks * 512;
  for (size_t i = grid_tid(); i < nvox; i += grid_stride()) {
    uint4 *p = (uint4 *)(m.voxels + i);
    uint4 v = *p;
    v.x = 0x7fffffffu;
    v.y = 0u;
    v.z = 0u;
    v.w &= 0xff000000u;
    *p = v;
    if (i < m.c.num_sdf_blocks) m.heap[i] = (int)m.c.num_sdf_blocks - (int)i - 1;
  }
  if (grid_tid() == 0) {
    *m.heap_counter = (int)m.c.num_sdf_blocks - 1;
    *m.entry_ptr = 1;
    *m.alloc_count = 0;
    *m.no_visible = 0;
  }
}

__global__ void k_rebuild_index(DevMap m) {
  for (unsigned i = grid_tid(); i < m.c.num_entries; i += grid_stride()) {
    int ptr = m.entries[i].ptr;
    bool alloc = ptr >= 0;
    unsigned slot = warp_append((unsigned *)m.alloc_count, alloc);
    if (alloc) m.alloc_list[slot] = (int)i;
  }
}

// ------------------------------------------------------------ allocation
constexpr int kProbeLimit = 128;

__device__ __forceinline__ unsigned long long req_key(i3 p, unsigned epoch) {
  return ((unsigned long long)(epoch & 0xffffu) << 48) |
         ((unsigned long long)((unsigned)p.x & 0xffffu) << 32) |
         ((unsigned long long)((unsigned)p.y & 0xffffu) << 16) | (unsigned long long)((unsigned)p.z & 0xffffu);
}

// Enters p into the request set.  Returns 1 if this thread entered it
// first, 0 if it was already requested this epoch, -1 if the set is full.
__device__ __forceinline__ int request_once(const FuseScratch &f, i3 p, unsigned epoch) {
  const unsigned long long key = req_key(p, epoch);
  uint32_t h = ((uint32_t)p.x * 0x9E3779B1u) ^ ((uint32_t)p.y * 0x85EBCA77u) ^ ((uint32_t)p.z * 0xC2B2AE3Du);
  h ^= h >> 15;
  const uint32_t mask = f.req_cap - 1;
  uint32_t idx = h & mask;
  for (int k = 0; k < kProbeLimit; ++k) {
    unsigned long long cur = __ldcg(f.req_set + idx);
    if (cur == key) return 0;
    if ((unsigned)(cur >> 48) != (epoch & 0xffffu)) {
      unsigned long long prev = atomicCAS(f.req_set + idx, cur, key);
      if (prev == cur) return 1;
      if (prev == key) return 0;
    }
    idx = (idx + 1) & mask;
  }
  return -1;
}

// Fusion::CreateBlocks (FuseMap.cu:92-132), probe pass.
// One block of the allocation walk: skip it if allocated (found >= 0),
// else request it once per frame and chain it into its bucket's pending
// list.
__device__ __forceinline__ void alloc_visit(const DevMap &m, const FuseScratch &f, uint32_t *flags,
                                            unsigned epoch, i3 bp, int found) {
  if (found >= 0) return;
  if (bp.x < -32767 || bp.x > 32767 || bp.y < -32767 || bp.y > 32767 || bp.z < -32767 ||
      bp.z > 32767) {
    atomicOr(flags, SF_FLAG_COORD_RANGE);
    return;
  }
  int r = request_once(f, bp, epoch);
  if (r < 0) { atomicOr(flags, SF_FLAG_DEDUP_FULL); return; }
  if (r == 0) return;
  unsigned slot = atomicAdd(&f.counters[0], 1u);
  if (slot >= f.pend_cap) { atomicOr(flags, SF_FLAG_PENDING_FULL); return; }
  int bucket = (int)hash_block(bp, m.c.num_buckets);
  f.pending[slot] = make_int4(bp.x, bp.y, bp.z, bucket);
  int prev = atomicExch(f.bucket_head + bucket, (int)slot);
  f.pending_next[slot] = prev;
  if (prev == -1) {
    unsigned d = atomicAdd(&f.counters[1], 1u);
    f.dirty[d] = bucket;  // d < pend_cap: one dirty bucket per pending slot at most
  }
}

constexpr int kAllocThreads = 256;  // a 32x8 tile of pixels per CTA

__global__ void __launch_bounds__(kAllocThreads, 5) k_alloc_probe(DevMap m, FuseScratch f, sf_image depth,
                                                               const Cam *cam,
                              const int *run_flag, uint32_t *flags) {
  if (run_flag && *run_flag == 0) return;  // the same for every thread
  const Cam c = *cam;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const unsigned epoch = f.counters[2];
  auto visit = [&](i3 bp, int found) { alloc_visit(m, f, flags, epoch, bp, found); };
  // The segment of the pixel's ray within trunc/2 of the measured depth,
  // sampled at half-voxel steps (the walk of FuseMapColor's allocation).
  int nSteps = 0;
  f3 pt_near = mk3(0.f, 0.f, 0.f), dir = pt_near;
  if (x < depth.cols && y < depth.rows) {
    const float dmin = m.c.depth_min, dmax = m.c.depth_max;
    const float z = row_ptr<const float>(depth, y)[x];
    const float thresh = m.c.trunc_dist / 2.0f;
    const float z_near = fmaxf(dmin, z - thresh);
    const float z_far = fminf(dmax, z + thresh);
    if (!isnan(z) && z >= dmin && z <= dmax && z_near < z_far) {
      f3 pn = mk3(z_near * ((float)x - c.cx) * c.invfx, z_near * ((float)y - c.cy) * c.invfy, z_near);
      f3 pf = mk3(z_far * ((float)x - c.cx) * c.invfx, z_far * ((float)y - c.cy) * c.invfy, z_far);
      pt_near = (mul(c.R, pn) + c.t) * m.c.voxel_size_inv;
      const f3 pt_far = (mul(c.R, pf) + c.t) * m.c.voxel_size_inv;
      dir = pt_far - pt_near;
      const float length = norm(dir);
      // A non-finite pose would make the walk unbounded; such a pixel is skipped.
      if (length < 65536.0f) {
        // (int)ceil(2.0 * length): 2*length is exact in float.
        nSteps = (int)ceilf(2.0f * length);
        dir = dir / (float)(nSteps - 1);
      }
    }
  }
  // The walk visits each run of samples in one block once.  The first
  // kAllocAhead distinct blocks are collected first (a ray through the
  // truncation band crosses two to four blocks).  Neighbouring pixels'
  // rays cross the same blocks, so within a warp only the lowest lane
  // holding a given block at a given position of its walk looks it up and
  // visits it (visits are idempotent within a frame: the others would find
  // it requested); the leaders' bucket entries are loaded together.  A
  // longer walk visits its further blocks as it meets them.
  //
  // Samples step by about half a voxel, so the walk tracks its block's
  // voxel bounds [8b, 8b + 8) and moves b by one per axis when a sample
  // leaves them: floor(floor(p) / 8) = b iff 8b <= p < 8b + 8, and the
  // bounds are exact floats while |b| < 2^20 (otherwise, or for the first
  // sample, the block comes from vox2block(floor3(p)) as in the reference).
  // Float-to-int conversions thus run once per ray, not once per sample.
  constexpr int kAllocAhead = 4;
  __shared__ i3 s_blk[kAllocThreads][kAllocAhead];
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  int nblk = 0;
  {
    i3 last;
    last.x = 0x7fffffff; last.y = 0; last.z = 0;
    f3 lo = mk3(1.f, 1.f, 1.f), hi = mk3(0.f, 0.f, 0.f);  // empty: no exact bounds
    bool exact = false;
    for (int i = 0; i < nSteps; ++i) {
      const f3 p = pt_near;
      pt_near = pt_near + dir;
      i3 bp;
      if (exact) {
        const int dx = (int)(p.x >= hi.x) - (int)(p.x < lo.x);
        const int dy = (int)(p.y >= hi.y) - (int)(p.y < lo.y);
        const int dz = (int)(p.z >= hi.z) - (int)(p.z < lo.z);
        if ((dx | dy | dz) == 0) continue;
        bp.x = last.x + dx; bp.y = last.y + dy; bp.z = last.z + dz;
      } else {
        bp = vox2block(floor3(p));
        if (bp.x == last.x && bp.y == last.y && bp.z == last.z) continue;
      }
      last = bp;
      const int lim = 1 << 20;
      exact = bp.x > -lim && bp.x < lim && bp.y > -lim && bp.y < lim && bp.z > -lim && bp.z < lim;
      if (exact) {
        lo = mk3((float)(8 * bp.x), (float)(8 * bp.y), (float)(8 * bp.z));
        hi = mk3((float)(8 * bp.x + 8), (float)(8 * bp.y + 8), (float)(8 * bp.z + 8));
      }
      if (nblk < kAllocAhead) {
        s_blk[tid][nblk] = bp;
        ++nblk;
      } else {
        visit(bp, find_block(m, bp));  // a fifth block or later (rare)
      }
    }
  }
  i3 blk[kAllocAhead];
#pragma unroll
  for (int k = 0; k < kAllocAhead; ++k) blk[k] = s_blk[tid][k];
  const int lane = (threadIdx.y * blockDim.x + threadIdx.x) & 31;
  bool lead[kAllocAhead];
  int4 head[kAllocAhead];
  int off[kAllocAhead];
#pragma unroll
  for (int k = 0; k < kAllocAhead; ++k) {
    const bool has = k < nblk;
    const unsigned long long key =
        has ? ((unsigned long long)(blk[k].x & 0x1fffff) | ((unsigned long long)(blk[k].y & 0x1fffff) << 21) |
               ((unsigned long long)(blk[k].z & 0x1fffff) << 42))
            : ~0ull;
    const unsigned same = __match_any_sync(0xffffffffu, key);
    const int src = __ffs(same) - 1;
    const int lx = __shfl_sync(0xffffffffu, blk[k].x, src), ly = __shfl_sync(0xffffffffu, blk[k].y, src),
              lz = __shfl_sync(0xffffffffu, blk[k].z, src);
    // a key shared by two different blocks (coordinates 2^21 blocks apart)
    // leaves both lanes leading
    lead[k] = has && (src == lane || lx != blk[k].x || ly != blk[k].y || lz != blk[k].z);
    if (lead[k]) {
      const sf_hash_entry *e = m.entries + hash_block(blk[k], m.c.num_buckets);
      head[k] = entry_head(e);
      off[k] = entry_offset(e);
    }
  }
#pragma unroll
  for (int k = 0; k < kAllocAhead; ++k)
    if (lead[k]) visit(blk[k], find_block_from(m, blk[k], head[k], off[k]));
}

// DeviceMap::CreateEntry (DeviceMap.cu:12-21).
__device__ __forceinline__ void create_entry(DevMap &m, i3 p, int offset, int4 &h0, int &off_out,
                                             uint32_t *flags) {
  int old = atomicSub(m.heap_counter, 1);
  if (old >= 0) {
    int ptr = m.heap[old];
    if (ptr != -1 && bound_ok(m, (uint32_t)ptr < m.c.num_sdf_blocks, SF_BOUND_PTR)) {
      h0 = make_int4(p.x, p.y, p.z, ptr * 512);
      off_out = offset;
      return;
    }
  }
  atomicOr(flags, SF_FLAG_HEAP_EMPTY);
  h0 = make_int4(p.x, p.y, p.z, -1);
  off_out = 0;
}

__device__ __forceinline__ void write_entry(DevMap &m, unsigned idx, int4 h0, int off) {
  int4 *e = (int4 *)(m.entries + idx);
  e[0] = h0;
  e[1] = make_int4(off, 0, 0, 0);
  if (h0.w >= 0) {
    int slot = atomicAdd(m.alloc_count, 1);
    m.alloc_list[slot] = (int)idx;
  }
}

// DeviceMap::CreateBlock (DeviceMap.cu:23-69) for one bucket, serially.
__device__ void create_block_serial(DevMap &m, i3 p, uint32_t bucket, uint32_t *flags) {
  unsigned idx = bucket;
  int4 h = entry_head(m.entries + idx);
  if (h.x == p.x && h.y == p.y && h.z == p.z && h.w != -1) return;
  int empty = (h.w == -1) ? (int)idx : -1;
  int off = m.entries[idx].offset;
  unsigned last = idx;
  int guard = 0;
  while (off > 0) {
    idx = m.c.num_buckets + (unsigned)off - 1u;
    h = entry_head(m.entries + idx);
    if (h.x == p.x && h.y == p.y && h.z == p.z && h.w != -1) return;
    if (h.w == -1 && empty < 0) empty = (int)idx;
    last = idx;
    off = m.entries[idx].offset;
    if (++guard > (int)m.c.num_excess) return;
  }
  int4 h0;
  int o;
  if (empty >= 0) {
    create_entry(m, p, m.entries[last].offset, h0, o, flags);
    write_entry(m, (unsigned)empty, h0, o);
  } else {
    int offset = atomicAdd(m.entry_ptr, 1);
    if (offset <= (int)m.c.num_excess) {
      create_entry(m, p, 0, h0, o, flags);
      write_entry(m, m.c.num_buckets + (unsigned)offset - 1u, h0, o);
      m.entries[last].offset = offset;
    } else {
      atomicOr(flags, SF_FLAG_EXCESS_FULL);
    }
  }
}

// Start of the visibility pass: resets the visible count and the rendered
// flag, sets the frame's block-pointer window (each CTA computes it for
// itself; CTA 0 publishes it for the later passes), then clears the window
// cells and (when given) the z-range images.  Run by every thread of the
// grid; win is shared memory of the calling CTA.
__device__ __forceinline__ void vis_start(const DevMap &m, const FuseScratch &f, const Cam *cam, unsigned *rendered,
                                          const sf_image &zmin, const sf_image &zmax, int do_z, int *win) {
  if (threadIdx.x == 0) {
    for (int k = 0; k < 8; ++k) win[k] = 0;
    window_setup(*cam, m.c.block_width, m.c.depth_min, m.c.depth_max, f.win_cap, win);
    if (blockIdx.x == 0) {
      *m.no_visible = 0u;
      if (rendered) *rendered = 0u;
      for (int k = 0; k < 6; ++k) f.win[k] = win[k];
    }
  }
  __syncthreads();
  const unsigned ncell = (unsigned)win[3] * (unsigned)win[4] * (unsigned)win[5];
  const unsigned nz = do_z ? (unsigned)(zmin.cols * zmin.rows) : 0u;
  const unsigned n = ncell > nz ? ncell : nz;
  for (unsigned i = grid_tid(); i < n; i += grid_stride()) {
    if (i < ncell) f.win_cells[i] = -1;
    if (i < nz) {
      const int y = (int)(i / (unsigned)zmin.cols), x = (int)(i % (unsigned)zmin.cols);
      row_ptr<float>(zmin, y)[x] = 100.f;
      row_ptr<float>(zmax, y)[x] = 0.f;
    }
  }
}

// With vs.on, the next visibility pass's start (vis_start) follows the
// inserts in the same launch: it touches none of the entries, heap or
// request set the inserts use.
__global__ void k_alloc_insert(DevMap m, FuseScratch f, const int *run_flag, uint32_t *flags, VisStartArgs vs) {
  if (run_flag && *run_flag == 0) return;
  const unsigned ndirty = min(f.counters[1], f.pend_cap);
  for (unsigned d = grid_tid(); d < ndirty; d += grid_stride()) {
    const int bucket = f.dirty[d];
    int i = f.bucket_head[bucket];
    int guard = 0;
    while (i >= 0 && guard++ < (int)f.pend_cap) {
      int4 q = f.pending[i];
      i3 p;
      p.x = q.x; p.y = q.y; p.z = q.z;
      create_block_serial(m, p, (uint32_t)bucket, flags);
      i = f.pending_next[i];
    }
    f.bucket_head[bucket] = -1;
  }
  // The 16-bit epoch wraps to 1 at the next frame: clear the request set
  // now (the probe pass is over), so no entry of 65535 frames ago matches.
  if (f.counters[2] == 0xffffu)
    for (unsigned i = grid_tid(); i < f.req_cap; i += grid_stride()) f.req_set[i] = 0ull;
  if (vs.on) {
    __shared__ int win[8];
    vis_start(m, f, vs.cam, vs.rendered, vs.zmin, vs.zmax, vs.do_z, win);
  }
}

// Clears the per-frame counters and advances the request epoch.  The
// probe pass reads counters[2]; the epoch skips 0 (the empty-slot value).
__global__ void k_alloc_begin(FuseScratch f, const int *run_flag) {
  if (run_flag && *run_flag == 0) return;
  alloc_frame_begin(f);
}

// ------------------------------------------------------------ visibility
// Fusion::CheckVertexVisibility (FuseMap.cu:46-56).
__device__ __forceinline__ bool vertex_visible(const Cam &c, f3 p3) {
  f3 pt = mul(c.Rinv, p3 - c.t);
  if (pt.z < 1e-3f) return false;
  float px = c.fx * pt.x / pt.z + c.cx;
  float py = c.fy * pt.y / pt.z + c.cy;
  return px >= 0 && py >= 0 && px < (float)c.cols && py < (float)c.rows && pt.z >= c.dmin &&
         pt.z <= c.dmax;
}

// Fusion::CheckBlockVisibility (FuseMap.cu:58-90), corner walk order kept.
__device__ __forceinline__ bool block_visible(const Cam &c, float s, i3 pos) {
  f3 k = mk3((float)pos.x * s, (float)pos.y * s, (float)pos.z * s);
  if (vertex_visible(c, k)) return true;
  k.z += s; if (vertex_visible(c, k)) return true;
  k.y += s; if (vertex_visible(c, k)) return true;
  k.x += s; if (vertex_visible(c, k)) return true;
  k.z -= s; if (vertex_visible(c, k)) return true;
  k.y -= s; if (vertex_visible(c, k)) return true;
  k.x -= s; k.y += s; if (vertex_visible(c, k)) return true;
  k.x += s; k.y -= s; k.z += s; if (vertex_visible(c, k)) return true;
  return false;
}

__global__ void k_visibility(DevMap m, FuseScratch f, const Cam *cam, sf_image zmin, sf_image zmax,
                             int do_z, unsigned *rendered, const int *run_flag, uint32_t *flags) {
  if (run_flag && *run_flag == 0) return;
  const Cam c = *cam;
  const unsigned n = (unsigned)*m.alloc_count;
  int win[6];
  for (int k = 0; k < 6; ++k) win[k] = f.win[k];
  // grid-stride with whole warps so warp_append sees converged lanes
  for (unsigned base = blockIdx.x * blockDim.x; base < n; base += grid_stride()) {
    const unsigned k = base + threadIdx.x;
    bool vis = false;
    int4 h0 = make_int4(0, 0, 0, -1);
    int4 h1 = make_int4(0, 0, 0, 0);
    unsigned idx = 0;
    if (k < n) {
      idx = (unsigned)m.alloc_list[k];
      h0 = entry_head(m.entries + idx);
      h1 = __ldcg((const int4 *)(m.entries + idx) + 1);
      i3 pos; pos.x = h0.x; pos.y = h0.y; pos.z = h0.z;
      vis = h0.w != -1 && block_visible(c, m.c.block_width, pos);
      // every allocated block inside the frustum box goes into the window
      const int cell = window_cell(win, pos);
      if (cell >= 0) f.win_cells[cell] = h0.w;
    }
    unsigned slot = warp_append(m.no_visible, vis);
    if (vis) {
      if (slot < m.c.num_entries) {
        int4 *o = (int4 *)(m.visible + slot);
        o[0] = h0;
        o[1] = h1;
      } else {
        atomicOr(flags, SF_FLAG_VISIBLE_FULL);
      }
      if (do_z) {
        sf_rendering_block b;
        i3 pos; pos.x = h0.x; pos.y = h0.y; pos.z = h0.z;
        if (project_block(pos, m.c.voxel_size, c.Rinv, c.t, c.fx, c.fy, c.cx, c.cy, zmin.cols,
                          zmin.rows, m.c.depth_max, m.c.depth_min, b)) {
          fill_block_tiles(b, zmin, zmax);
          if (*rendered == 0u) atomicExch(rendered, 1u);
        }
      }
    }
  }
}

__global__ void k_zrange_init(sf_image zmin, sf_image zmax) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= zmin.cols || y >= zmin.rows) return;
  row_ptr<float>(zmin, y)[x] = 100.f;
  row_ptr<float>(zmax, y)[x] = 0.f;
}

__global__ void k_vis_start(DevMap m, FuseScratch f, const Cam *cam, unsigned *rendered, sf_image zmin,
                            sf_image zmax, int do_z, const int *run_flag) {
  if (run_flag && *run_flag == 0) return;
  __shared__ int win[8];
  vis_start(m, f, cam, rendered, zmin, zmax, do_z, win);
}

// UpdateVisibility + CreateRenderingBlocks' z-range for n candidate
// cameras (Tracker::ValidatePose, Tracking.cc:756-762): grid.y is the
// candidate, grid.x strides over the allocated-entry index.  The count is
// CheckBlockVisibility's (FuseMap.cu:991-1037); the z-range tiles are
// Projection + fillBlocks' (RenderScene.cu:54-190), laid into the
// candidate's zr-row slice of the tall z-range images.
__global__ void k_vp_visibility(DevMap m, const Cam *cams, sf_image zmin, sf_image zmax, int zr, unsigned *vis,
                                unsigned *rendered) {
  const int c = blockIdx.y;
  const Cam cam = cams[c];
  sf_image zn = zmin, zx = zmax;
  zn.data = (char *)zmin.data + (size_t)c * zr * zmin.step;
  zx.data = (char *)zmax.data + (size_t)c * zr * zmax.step;
  zn.rows = zx.rows = zr;
  const unsigned n = (unsigned)*m.alloc_count;
  unsigned cnt = 0;
  bool drew = false;
  for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int4 h = entry_head(m.entries + m.alloc_list[k]);
    if (h.w == -1) continue;
    i3 pos; pos.x = h.x; pos.y = h.y; pos.z = h.z;
    if (!block_visible(cam, m.c.block_width, pos)) continue;
    ++cnt;
    sf_rendering_block b;
    if (project_block(pos, m.c.voxel_size, cam.Rinv, cam.t, cam.fx, cam.fy, cam.cx, cam.cy, zn.cols, zr,
                      m.c.depth_max, m.c.depth_min, b)) {
      fill_block_tiles(b, zn, zx);
      drew = true;
    }
  }
  cnt = __reduce_add_sync(0xffffffffu, cnt);
  drew = __any_sync(0xffffffffu, drew);
  if ((threadIdx.x & 31) == 0) {
    if (cnt) atomicAdd(vis + c, cnt);
    if (drew && rendered[c] == 0u) atomicExch(rendered + c, 1u);
  }
}

// -------------------------------------------------------------- integrate
union VoxelU {
  uint4 u;
  sf_voxel v;
};

// Fusion::createVoxels per voxel (FuseMap.cu:453-505).
__device__ __forceinline__ bool integrate_voxel(sf_voxel &prev, float sdf, f3 val) {
  if (prev.weight == 0) {
    prev.sdf = sdf;
    prev.weight = 1;
    prev.color[0] = f2u8(val.x); prev.color[1] = f2u8(val.y); prev.color[2] = f2u8(val.z);
    prev.label = 0; prev.count = 0; prev.label_2 = 0; prev.count_2 = 0;
    prev.color_2[0] = 0; prev.color_2[1] = 0; prev.color_2[2] = 0;
    return true;
  }
  if (prev.label == 0) {
    // make_float3(color) * weight is operator*(float3,int) -> int3
    // (VectorMath.h:231-233); int3 + float3 -> float3; / (w+1).
    const int w = prev.weight;
    float r0 = ((float)(int)((float)prev.color[0] * (float)w) + val.x) / (float)(w + 1);
    float r1 = ((float)(int)((float)prev.color[1] * (float)w) + val.y) / (float)(w + 1);
    float r2 = ((float)(int)((float)prev.color[2] * (float)w) + val.z) / (float)(w + 1);
    prev.color[0] = f2u8(r0); prev.color[1] = f2u8(r1); prev.color[2] = f2u8(r2);
  }
  prev.sdf = (prev.sdf * (float)prev.weight + sdf) / (float)(prev.weight + 1);
  prev.weight = (uint8_t)min(255, prev.weight + 1);
  return true;
}

// Fusion::analyzeSemantics per voxel (FuseMap.cu:582-664).
__device__ __forceinline__ void semantic_voxel(sf_voxel &prev, uint8_t label, f3 val, float4 nl,
                                               f3 pos) {
  if (prev.weight == 0) return;
  if (label != 0) {
    if (label == prev.label) {
      prev.count = (uint8_t)min(255, prev.count + 1);
      prev.color[0] = f2u8(val.x); prev.color[1] = f2u8(val.y); prev.color[2] = f2u8(val.z);
    } else {
      if (label == prev.label_2) {
        prev.count_2 = (uint8_t)min(255, prev.count_2 + 1);
        prev.color_2[0] = f2u8(val.x); prev.color_2[1] = f2u8(val.y); prev.color_2[2] = f2u8(val.z);
      } else if (prev.count_2 < 7) {
        prev.label_2 = label;
        prev.count_2 = 1;
        prev.color_2[0] = f2u8(val.x); prev.color_2[1] = f2u8(val.y); prev.color_2[2] = f2u8(val.z);
      }
      if ((prev.count < prev.count_2 && prev.label != 0) ||
          (prev.count < prev.count_2 * 2 && prev.label == 0)) {
        uint8_t t = prev.label; prev.label = prev.label_2; prev.label_2 = t;
        t = prev.count; prev.count = prev.count_2; prev.count_2 = t;
        for (int k = 0; k < 3; ++k) { t = prev.color[k]; prev.color[k] = prev.color_2[k]; prev.color_2[k] = t; }
      }
    }
  } else {
    // w = nl . normalised(make_float4(pos)) with the float4 norm.
    float len = sqrtf(pos.x * pos.x + pos.y * pos.y + pos.z * pos.z + 1.0f * 1.0f);
    float a0 = pos.x / len, a1 = pos.y / len, a2 = pos.z / len, a3 = 1.0f / len;
    float w = nl.x * a0 + nl.y * a1 + nl.z * a2 + nl.w * a3;
    if (prev.label != 0) {
      if (prev.count < 7) {
        prev.label_2 = prev.label;
        prev.color_2[0] = prev.color[0]; prev.color_2[1] = prev.color[1]; prev.color_2[2] = prev.color[2];
        prev.count_2 = prev.count;
        prev.label = 0;
        prev.count = 1;
        f3 vv = val / 255.f;
        f3 old = mk3((float)prev.color[0], (float)prev.color[1], (float)prev.color[2]) / 255.f;
        float a = w * 0.2f;
        f3 res = (a * vv + (1 - w * 0.2f) * old) * 255.f;
        prev.color[0] = f2u8(res.x); prev.color[1] = f2u8(res.y); prev.color[2] = f2u8(res.z);
      }
    } else {
      prev.count = (uint8_t)min(255, prev.count + 1);
    }
  }
}

// ------------------------------------------------------ neighbour labels
// Fusion::UnifyNeighbor + UpdateNeighborLabel (FuseMap.cu:757-896): for the
// hash slots [0, noVisible) (the kernel indexes hashEntries[blockIdx.x] over
// a grid of noVisibleBlocks), each labelled voxel takes the label most of
// its 26 neighbours carry.  One thread per (x, y) voxel column, as the
// (8, 8) launch; the 4-slot neighbour table lives across the column's z
// loop as in the reference.  k_unify_compute writes each processed voxel's
// new {label, count, label_2, count_2} word to `out` while reading only the
// voxel array, and k_unify_apply copies the words back, so every voxel
// updates from the pass-start state (in place, the reference's neighbours
// read voxels other threads are rewriting).
constexpr int kUnifyThreads = 64;

// UnifyNeighbor's 26 offsets in its order (FuseMap.cu:834-887), as
// (dx + 1) | (dy + 1) << 2 | (dz + 1) << 4.
__device__ __forceinline__ constexpr unsigned unify_order(int k) {
  return k == 0 ? 0x16u : k == 1 ? 0x1au : k == 2 ? 0x12u : k == 3 ? 0x26u : k == 4 ? 0x06u : k == 5 ? 0x2au : k == 6 ? 0x0au : k == 7 ? 0x22u : k == 8 ? 0x02u : k == 9 ? 0x14u : k == 10 ? 0x18u : k == 11 ? 0x10u : k == 12 ? 0x24u : k == 13 ? 0x04u : k == 14 ? 0x28u : k == 15 ? 0x08u : k == 16 ? 0x20u : k == 17 ? 0x00u : k == 18 ? 0x19u : k == 19 ? 0x29u : k == 20 ? 0x09u : k == 21 ? 0x11u : k == 22 ? 0x21u : k == 23 ? 0x01u : k == 24 ? 0x25u : 0x05u;
}

// make_int3(float) on one axis: floor (VectorMath.h:36-42).
__device__ __forceinline__ int floor1i(float a) {
  const int b = (int)a;
  return (float)b > a ? b - 1 : b;
}
// worldPosToVoxelPos of pos - step, pos, pos + step on one axis
// (DeviceMap.cu:156-159).
struct AxisCands {
  int lo, mid, hi;
  __device__ __forceinline__ AxisCands(float pos, float step, float vs)
      : lo(floor1i((pos - step) / vs)), mid(floor1i(pos / vs)), hi(floor1i((pos + step) / vs)) {}
  __device__ __forceinline__ int at(unsigned d) const { return d == 0u ? lo : (d == 1u ? mid : hi); }
};

// UpdateNeighborLabel's 4-slot table (FuseMap.cu:757-796) in registers:
// label (-1 = free), neighbours seen, and their largest count.
struct NeighborTable {
  int l0 = -1, l1 = -1, l2 = -1, l3 = -1;
  int c0 = 0, c1 = 0, c2 = 0, c3 = 0;
  int lc0 = 0, lc1 = 0, lc2 = 0, lc3 = 0;
  // The first slot holding `lab` counts it; else the first free slot takes
  // it; a full table drops it.
  __device__ __forceinline__ static bool slot(int &l, int &c, int &lc, int lab, int cnt) {
    if (l == lab) {
      ++c;
      lc = lc > cnt ? lc : cnt;
      return true;
    }
    if (l == -1) {
      l = lab;
      c = 1;
      lc = cnt;
      return true;
    }
    return false;
  }
  __device__ __forceinline__ void add(int lab, int cnt) {
    if (slot(l0, c0, lc0, lab, cnt)) return;
    if (slot(l1, c1, lc1, lab, cnt)) return;
    if (slot(l2, c2, lc2, lab, cnt)) return;
    slot(l3, c3, lc3, lab, cnt);
  }
  // The labelled slot (count > 0) seen most often; the first wins ties.
  __device__ __forceinline__ static void pick(int l, int c, int lc, int &best_l, int &best_c, int &best_lc) {
    if (l != -1 && lc != 0 && c > best_c) {
      best_l = l;
      best_c = c;
      best_lc = lc;
    }
  }
};

// A block's neighbourhood for the pass: its voxels and the ones whose
// float positions (pos +- VoxelSize) / VoxelSize can floor to -- offsets
// -2..+1 from a block voxel, so cells -2..8 per axis (11^3) -- each as
// {weight > 0, label, count} (0: no neighbour value: a missing block or
// weight 0), staged in shared memory by the whole CTA with every load in
// flight; the columns' 26-neighbour walks then read shared memory.
constexpr int kUnifyHalo = 11;
constexpr int kUnifyCells = kUnifyHalo * kUnifyHalo * kUnifyHalo;

__device__ __forceinline__ uint32_t unify_cell_value(const DevMap &m, int ptr, i3 v) {
  if (ptr < 0) return 0u;
  const uint4 w = __ldg((const uint4 *)(m.voxels + ptr + vox2local(v)));
  if ((w.y & 0xffu) == 0u) return 0u;  // weight 0: label -1
  return 0x10000u | (w.z & 0xffffu);   // valid | count << 8 | label
}

__device__ __forceinline__ void unify_block(const DevMap &m, uint32_t *out, int4 h, uint32_t *cells,
                                            int *bptr) {
  const int tx = threadIdx.x & 7, ty = threadIdx.x >> 3;
  const int bx = (int)((uint32_t)h.x * 8u), by = (int)((uint32_t)h.y * 8u), bz = (int)((uint32_t)h.z * 8u);
  const int ox = bx - 2, oy = by - 2, oz = bz - 2;  // the neighbourhood's first cell
  // the 27 blocks around this one (cells -2..-1 in block -1, 8 in block +1)
  if (threadIdx.x < 27) {
    const int dx = threadIdx.x % 3 - 1, dy = (threadIdx.x / 3) % 3 - 1, dz = threadIdx.x / 9 - 1;
    bptr[threadIdx.x] = (dx | dy | dz) == 0 ? h.w : find_block(m, mk_i3(h.x + dx, h.y + dy, h.z + dz));
  }
  __syncthreads();
  // four cells per thread per round, their loads issued together
  constexpr int kRound = 4 * kUnifyThreads;
  for (int c0 = 0; c0 < kUnifyCells; c0 += kRound) {
    uint4 w[4];
    int cell[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int c = c0 + q * kUnifyThreads + threadIdx.x;
      cell[q] = -1;
      w[q] = make_uint4(0u, 0u, 0u, 0u);
      if (c < kUnifyCells) {
        const int ix = c % kUnifyHalo, iy = (c / kUnifyHalo) % kUnifyHalo, iz = c / (kUnifyHalo * kUnifyHalo);
        const int sx = ix < 2 ? 0 : (ix < 10 ? 1 : 2), sy = iy < 2 ? 0 : (iy < 10 ? 1 : 2);
        const int sz = iz < 2 ? 0 : (iz < 10 ? 1 : 2);
        const int ptr = bptr[sx + 3 * sy + 9 * sz];
        cell[q] = c;
        if (ptr >= 0) {
          w[q] = __ldg((const uint4 *)(m.voxels + ptr + vox2local(mk_i3(ox + ix, oy + iy, oz + iz))));
          w[q].x = 1u;  // found
        }
      }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (cell[q] >= 0)
        cells[cell[q]] = (w[q].x == 0u || (w[q].y & 0xffu) == 0u) ? 0u : (0x10000u | (w[q].z & 0xffffu));
  }
  __syncthreads();
  const float vs = m.c.voxel_size;
  const float step = vs * (float)1;  // VoxelSize * r, r = 1
  const AxisCands cx((float)(bx + tx) * vs, step, vs), cy((float)(by + ty) * vs, step, vs);
  NeighborTable t;
  // the column's own label word, each loaded one voxel ahead (its weight
  // is in the staged cells: valid = weight > 0)
  const uint32_t *own = (const uint32_t *)(m.voxels + h.w + ty * 8 + tx) + 2;
  uint32_t next = __ldg(own);
#pragma unroll 1
  for (int i = 0; i < 8; ++i) {
    const int idx = h.w + i * 64 + ty * 8 + tx;
    const uint32_t w2 = next;
    if (i < 7) next = __ldg(own + (i + 1) * 64 * 4);
    uint32_t res = w2;
    if (cells[((i + 2) * kUnifyHalo + ty + 2) * kUnifyHalo + tx + 2] != 0u) {
      const int cur_label = (int)(w2 & 0xffu);
      const AxisCands cz((float)(bz + i) * vs, step, vs);
      // the 26 neighbour values first (independent shared-memory reads, all
      // in flight), then the table updates in UnifyNeighbor's order
      uint32_t nv[26];
      bool outside = false;
#pragma unroll
      for (int k = 0; k < 26; ++k) {
        const unsigned o = unify_order(k);
        const unsigned qx = (unsigned)(cx.at(o & 3u) - ox), qy = (unsigned)(cy.at((o >> 2) & 3u) - oy);
        const unsigned qz = (unsigned)(cz.at((o >> 4) & 3u) - oz);
        const bool in = qx < (unsigned)kUnifyHalo && qy < (unsigned)kUnifyHalo && qz < (unsigned)kUnifyHalo;
        outside |= !in;
        nv[k] = in ? cells[(qz * kUnifyHalo + qy) * kUnifyHalo + qx] : 0u;
      }
      if (outside) {  // a position outside the staged cells (not reached for |coordinates| < 2^21): the table
#pragma unroll
        for (int k = 0; k < 26; ++k) {
          const unsigned o = unify_order(k);
          const i3 v = mk_i3(cx.at(o & 3u), cy.at((o >> 2) & 3u), cz.at((o >> 4) & 3u));
          const unsigned qx = (unsigned)(v.x - ox), qy = (unsigned)(v.y - oy), qz = (unsigned)(v.z - oz);
          if (!(qx < (unsigned)kUnifyHalo && qy < (unsigned)kUnifyHalo && qz < (unsigned)kUnifyHalo))
            nv[k] = unify_cell_value(m, find_block(m, vox2block(v)), v);
        }
      }
#pragma unroll
      for (int k = 0; k < 26; ++k)
        if (nv[k] != 0u) t.add((int)(nv[k] & 0xffu), (int)((nv[k] >> 8) & 0xffu));
      int nei_label = -1, nei_count = 0, nei_lc = 0;
      t.pick(t.l0, t.c0, t.lc0, nei_label, nei_count, nei_lc);
      t.pick(t.l1, t.c1, t.lc1, nei_label, nei_count, nei_lc);
      t.pick(t.l2, t.c2, t.lc2, nei_label, nei_count, nei_lc);
      t.pick(t.l3, t.c3, t.lc3, nei_label, nei_count, nei_lc);
      const uint32_t count = (w2 >> 8) & 0xffu, label_2 = (w2 >> 16) & 0xffu, count_2 = w2 >> 24;
      if (cur_label != nei_label) {
        const int tmp = cur_label == (int)label_2 ? (nei_lc > (int)count_2 ? nei_lc : (int)count_2 + 5) : nei_lc;
        res = ((uint32_t)nei_label & 0xffu) | (((uint32_t)tmp & 0xffu) << 8) | ((uint32_t)cur_label << 16) |
              (count << 24);
      } else {
        res = (w2 & 0xffff00ffu) | (((uint32_t)nei_lc & 0xffu) << 8);
      }
    }
    out[idx] = res;
  }
  __syncthreads();  // before the cells are restaged
}

// The allocated entries among hash slots [0, visible count), in any order
// (each block's pass is independent): list[0..*count).
__global__ void k_unify_list(DevMap m, int *list, unsigned *count, const int *run_flag) {
  if (run_flag && *run_flag == 0) return;
  const unsigned n = min(*m.no_visible, m.c.num_entries);
  for (unsigned base = blockIdx.x * blockDim.x; base < n; base += grid_stride()) {
    const unsigned e = base + threadIdx.x;
    const bool occ = e < n && checked_ptr(m, __ldcg(&m.entries[e].ptr)) >= 0;
    const unsigned slot = warp_append(count, occ);
    if (occ) list[slot] = (int)e;
  }
}

// One CTA per listed block.
__global__ void __launch_bounds__(kUnifyThreads) k_unify_compute(DevMap m, uint32_t *out, const int *list,
                                                                  const unsigned *count, const int *run_flag) {
  if (run_flag && *run_flag == 0) return;
  __shared__ uint32_t s_cells[kUnifyCells];
  __shared__ int s_bptr[27];
  const unsigned n = __ldcg(count);
  for (unsigned j = blockIdx.x; j < n; j += gridDim.x)
    unify_block(m, out, entry_head(m.entries + __ldcg(list + j)), s_cells, s_bptr);
}

__global__ void k_unify_apply(DevMap m, const uint32_t *out, unsigned *list_count, const int *run_flag) {
  if (run_flag && *run_flag == 0) return;
  if (grid_tid() == 0) *list_count = 0u;  // the compute pass has read it; zero for the next pass
  const unsigned n = min(*m.no_visible, m.c.num_entries);
  const unsigned lane = threadIdx.x & 31u;
  const unsigned nwarps = (gridDim.x * blockDim.x) >> 5;
  for (unsigned e = grid_tid() >> 5; e < n; e += nwarps) {
    const int ptr = __ldcg(&m.entries[e].ptr);
    if (ptr < 0) continue;
    for (unsigned i = lane; i < 512u; i += 32u)
      ((uint32_t *)(m.voxels + ptr + i))[2] = __ldcg(out + ptr + i);
  }
}

constexpr int kIntThreads = 256;

// Eight 256-thread CTAs per SM (32 registers, a few spilled bytes) for the
// TSDF pass: the kernel waits on its depth and voxel loads, and full
// occupancy hides that best (measured on GB300 against 3-6 CTAs per SM);
// the label passes, with more state per voxel, take six.
#ifndef SF_INT_MINB
#define SF_INT_MINB 8
#endif
// One instantiation per pass (TSDF only, labels only, both): the TSDF pass
// carries none of the label update's registers.
template <bool do_int, bool do_sem>
__global__ void __launch_bounds__(kIntThreads, do_sem ? 6 : SF_INT_MINB) k_integrate(DevMap m, sf_image depth, sf_image rgb,
                                                           sf_image nmap, sf_image mask,
                                                           int num_detection, const Cam *cam,
                                                           const int *run_flag) {
  if (run_flag && *run_flag == 0) return;
  const Cam c = *cam;
  const unsigned nvis = min(*m.no_visible, m.c.num_entries);
  const float thresh = m.c.trunc_dist;
  const float voxel = m.c.voxel_size;
  const int pal0 = 33554431, pal1 = 32767, pal2 = 2097151;  // 2^25-1, 2^15-1, 2^21-1 (FuseMap.cu:18)
  for (unsigned b = blockIdx.x; b < nvis; b += gridDim.x) {
    int4 h = __ldcg((const int4 *)(m.visible + b));
    h.w = checked_ptr(m, h.w);
    if (h.w == -1) continue;
    // Each thread's two voxels (li = tid, tid + 256) in phases, so that
    // their dependent loads overlap: both projections and depth reads with
    // both voxel reads (issued before the depth tests decide which voxels
    // change: 1.3% faster than reading only those, for more DRAM bytes),
    // then the colour reads, then both updates.
    static_assert(kIntThreads * 2 == 512, "two voxels per thread");
    f3 pos[2];
    int u[2], v[2];
    float dp[2];
    bool ok[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const int li = threadIdx.x + k * kIntThreads;
      const int lx = li & 7, ly = (li >> 3) & 7, lz = li >> 6;
      f3 w3 = mk3((float)(h.x * 8 + lx) * voxel, (float)(h.y * 8 + ly) * voxel,
                  (float)(h.z * 8 + lz) * voxel);
      pos[k] = mul(c.Rinv, w3 - c.t);
      u[k] = (int)(c.fx * pos[k].x / pos[k].z + c.cx);
      v[k] = (int)(c.fy * pos[k].y / pos[k].z + c.cy);
      ok[k] = !(u[k] < 0 || v[k] < 0 || u[k] >= c.cols || v[k] >= c.rows);
      dp[k] = ok[k] ? __ldg(row_ptr<const float>(depth, v[k]) + u[k]) : 0.0f;
    }
    VoxelU vx[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) vx[k].u = *((const uint4 *)(m.voxels + h.w) + threadIdx.x + k * kIntThreads);
    uint8_t px[2][3];
    float sdf[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      ok[k] = ok[k] && !(isnan(dp[k]) || dp[k] > c.dmax || dp[k] < c.dmin);
      sdf[k] = dp[k] - pos[k].z;
      ok[k] = ok[k] && sdf[k] >= -thresh;
      if (ok[k]) {
        const uint8_t *p = row_ptr<const uint8_t>(rgb, v[k]) + 3 * u[k];
        px[k][0] = p[0]; px[k][1] = p[1]; px[k][2] = p[2];
      }
    }
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      if (!ok[k]) continue;
      bool dirty = false;
      if (do_int) {
        f3 val = mk3((float)px[k][0], (float)px[k][1], (float)px[k][2]);
        dirty = integrate_voxel(vx[k].v, fminf(1.0f, sdf[k] / thresh), val);
      }
      if (do_sem) {
        float4 nl = __ldg(row_ptr<const float4>(nmap, v[k]) + u[k]);
        if (!isnan(nl.x)) {
          uint8_t label;
          f3 val;
          if (num_detection > 0) {
            label = __ldg(row_ptr<const uint8_t>(mask, v[k]) + u[k]);
            if (label == 0) {
              val = mk3((float)px[k][0], (float)px[k][1], (float)px[k][2]);
            } else {
              int p0 = (int)((unsigned)pal0 * (unsigned)label) % 255;
              int p1 = (int)((unsigned)pal1 * (unsigned)label) % 255;
              int p2 = (int)((unsigned)pal2 * (unsigned)label) % 255;
              val = mk3((float)p0, (float)p1, (float)p2);
            }
          } else {
            label = 0;
            val = mk3((float)px[k][0], (float)px[k][1], (float)px[k][2]);
          }
          semantic_voxel(vx[k].v, label, val, nl, pos[k]);
          dirty = true;
        }
      }
      if (dirty) *((uint4 *)(m.voxels + h.w) + threadIdx.x + k * kIntThreads) = vx[k].u;
    }
  }
}

}  // namespace

// ---------------------------------------------------------------- host side
int fuse_scratch_init(FuseScratch &f, const MapConst &c, int max_pixels) {
  uint32_t want = 1;
  while (want < (uint32_t)max_pixels * 2u && want < (1u << 24)) want <<= 1;
  f.req_cap = want < (1u << 16) ? (1u << 16) : want;
  f.pend_cap = f.req_cap / 2;
  if (cudaMalloc(&f.req_set, sizeof(unsigned long long) * f.req_cap) != cudaSuccess) return SF_ERR_CUDA;
  if (cudaMemset(f.req_set, 0, sizeof(unsigned long long) * f.req_cap) != cudaSuccess) return SF_ERR_CUDA;
  if (cudaMalloc(&f.pending, sizeof(int4) * f.pend_cap) != cudaSuccess) return SF_ERR_CUDA;
  if (cudaMalloc(&f.pending_next, sizeof(int) * f.pend_cap) != cudaSuccess) return SF_ERR_CUDA;
  if (cudaMalloc(&f.dirty, sizeof(int) * f.pend_cap) != cudaSuccess) return SF_ERR_CUDA;
  if (cudaMalloc(&f.bucket_head, sizeof(int) * c.num_buckets) != cudaSuccess) return SF_ERR_CUDA;
  if (cudaMemset(f.bucket_head, 0xff, sizeof(int) * c.num_buckets) != cudaSuccess) return SF_ERR_CUDA;
  if (cudaMalloc(&f.counters, sizeof(unsigned) * 4) != cudaSuccess) return SF_ERR_CUDA;
  if (cudaMemset(f.counters, 0, sizeof(unsigned) * 4) != cudaSuccess) return SF_ERR_CUDA;
  f.win_cap = 1u << 23;
  if (cudaMalloc(&f.win, sizeof(int) * 8) != cudaSuccess) return SF_ERR_CUDA;
  if (cudaMemset(f.win, 0, sizeof(int) * 8) != cudaSuccess) return SF_ERR_CUDA;
  if (cudaMalloc(&f.win_cells, sizeof(int) * (size_t)f.win_cap) != cudaSuccess) return SF_ERR_CUDA;
  return SF_OK;
}

void fuse_scratch_free(FuseScratch &f) {
  cudaFree(f.req_set);
  cudaFree(f.pending);
  cudaFree(f.pending_next);
  cudaFree(f.dirty);
  cudaFree(f.bucket_head);
  cudaFree(f.counters);
  cudaFree(f.win);
  cudaFree(f.win_cells);
  cudaFree(f.unify_out);
  f = FuseScratch();
}

static int sm_count() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
  }
  return n;
}

void launch_map_reset(const DevMap &m, cudaStream_t s) {
  const int g = sm_count() * 8;
  k_reset_entries<<<g, 256, 0, s>>>(m, nullptr); note_launch();
  k_reset_voxels<<<g, 256, 0, s>>>(m); note_launch();
}

void launch_rebuild_index(const DevMap &m, cudaStream_t s) {
  cudaMemsetAsync(m.alloc_count, 0, sizeof(int), s);
  k_rebuild_index<<<sm_count() * 8, 256, 0, s>>>(m); note_launch();
}

AllocTile alloc_tile(int tile) {
  // 256 threads each (the probe's shared block lists are sized for that);
  // a warp covers 32, 32, 16 x 2 or 32 pixels of a row
  static const AllocTile kTiles[kAllocTileCount] = {{32, 8}, {64, 4}, {16, 16}, {128, 2}};
  return kTiles[tile >= 0 && tile < kAllocTileCount ? tile : 0];
}

void launch_alloc_probe(const DevMap &m, const FuseScratch &f, const sf_image &depth, const Cam *c,
                        const int *run_flag, uint32_t *flags, cudaStream_t s, int tile) {
  const AllocTile t = alloc_tile(tile);
  static_assert(kAllocThreads == 256, "alloc tiles hold 256 threads");
  dim3 blk(t.x, t.y);
  dim3 grd((depth.cols + t.x - 1) / t.x, (depth.rows + t.y - 1) / t.y);
  k_alloc_probe<<<grd, blk, 0, s>>>(m, f, depth, c, run_flag, flags); note_launch();
}

void launch_alloc(const DevMap &m, const FuseScratch &f, const sf_image &depth, const Cam *c,
                  const int *run_flag, uint32_t *flags, cudaStream_t s, bool begin, int tile,
                  const sf_image *vis_zmin, const sf_image *vis_zmax) {
  if (begin) {
    k_alloc_begin<<<1, 1, 0, s>>>(f, run_flag);
    note_launch();
  }
  launch_alloc_probe(m, f, depth, c, run_flag, flags, s, tile);
  VisStartArgs vs = {};
  if (vis_zmin && vis_zmax) {
    vs.on = 1;
    vs.cam = c;
    vs.rendered = f.counters + 3;
    vs.zmin = *vis_zmin;
    vs.zmax = *vis_zmax;
    vs.do_z = 1;
  }
  k_alloc_insert<<<sm_count() * 2, 128, 0, s>>>(m, f, run_flag, flags, vs); note_launch();
}

void launch_zrange_init(const sf_image &zmin, const sf_image &zmax, cudaStream_t s) {
  dim3 blk(32, 8);
  dim3 grd((zmin.cols + 31) / 32, (zmin.rows + 7) / 8);
  k_zrange_init<<<grd, blk, 0, s>>>(zmin, zmax); note_launch();
}

void launch_visibility(const DevMap &m, const FuseScratch &f, const Cam *c, const sf_image *zmin,
                       const sf_image *zmax, const int *run_flag, uint32_t *flags,
                       cudaStream_t s, bool started) {
  unsigned *rendered = f.counters + 3;
  const bool do_z = zmin && zmax;
  sf_image zn = do_z ? *zmin : sf_image{}, zx = do_z ? *zmax : sf_image{};
  if (!started) {
    k_vis_start<<<sm_count() * 8, 256, 0, s>>>(m, f, c, rendered, zn, zx, do_z ? 1 : 0, run_flag);
    note_launch();
  }
  k_visibility<<<sm_count() * 4, 256, 0, s>>>(m, f, c, zn, zx, do_z ? 1 : 0, rendered, run_flag,
                                              flags); note_launch();
}

void launch_vp_visibility(const DevMap &m, const Cam *cams, int n, const sf_image &zmin, const sf_image &zmax,
                          int zr, unsigned *vis, unsigned *rendered, cudaStream_t s) {
  k_vp_visibility<<<dim3(64, n), 256, 0, s>>>(m, cams, zmin, zmax, zr, vis, rendered); note_launch();
}

void launch_unify_neighbor(const DevMap &m, const FuseScratch &f, const int *run_flag, cudaStream_t s) {
  k_unify_list<<<sm_count() * 4, 256, 0, s>>>(m, f.unify_list, f.unify_count, run_flag); note_launch();
  k_unify_compute<<<sm_count() * 16, kUnifyThreads, 0, s>>>(m, f.unify_out, f.unify_list, f.unify_count,
                                                             run_flag); note_launch();
  k_unify_apply<<<sm_count() * 4, 256, 0, s>>>(m, f.unify_out, f.unify_count, run_flag); note_launch();
}

int fuse_scratch_unify(FuseScratch &f, const MapConst &c) {
  if (f.unify_out) return SF_OK;
  const size_t words = 512 * (size_t)c.num_sdf_blocks;
  // the new label words, then the block list and its count
  if (cudaMalloc(&f.unify_out, sizeof(uint32_t) * (words + c.num_sdf_blocks + 1)) != cudaSuccess) return SF_ERR_CUDA;
  f.unify_list = reinterpret_cast<int *>(f.unify_out + words);
  f.unify_count = reinterpret_cast<unsigned *>(f.unify_out + words + c.num_sdf_blocks);
  // zero before first use (the apply pass zeroes it for the next pass)
  if (cudaMemset(f.unify_count, 0, sizeof(unsigned)) != cudaSuccess) return SF_ERR_CUDA;
  return cudaDeviceSynchronize() == cudaSuccess ? SF_OK : SF_ERR_CUDA;
}

void launch_integrate(const DevMap &m, const sf_image &depth, const sf_image &rgb,
                      const sf_image *nmap, const sf_image *mask, int num_detection, const Cam *c,
                      bool integrate, bool semantics, const int *run_flag, cudaStream_t s, int ctas_per_sm) {
  sf_image nm = nmap ? *nmap : sf_image{};
  sf_image mk = mask ? *mask : sf_image{};
  const bool sem = semantics && nmap && (num_detection <= 0 || mask);
  const dim3 grid(sm_count() * ctas_per_sm);
  if (integrate && sem)
    k_integrate<true, true><<<grid, kIntThreads, 0, s>>>(m, depth, rgb, nm, mk, num_detection, c, run_flag);
  else if (integrate)
    k_integrate<true, false><<<grid, kIntThreads, 0, s>>>(m, depth, rgb, nm, mk, num_detection, c, run_flag);
  else if (sem)
    k_integrate<false, true><<<grid, kIntThreads, 0, s>>>(m, depth, rgb, nm, mk, num_detection, c, run_flag);
  else
    return;
  note_launch();
}

// The voxels of the visible blocks saved to / restored from scratch (the
// autotuner's timing runs of the integration, which changes them).
__global__ void k_save_visible(DevMap m, uint4 *scratch, unsigned nvis, int restore) {
  for (unsigned b = blockIdx.x; b < nvis; b += gridDim.x) {
    const int ptr = __ldcg(&m.visible[b].ptr);
    if (ptr < 0) continue;
    uint4 *v = (uint4 *)(m.voxels + ptr);
    uint4 *w = scratch + (size_t)b * 512;
    for (int i = threadIdx.x; i < 512; i += blockDim.x) {
      if (restore) v[i] = w[i];
      else w[i] = v[i];
    }
  }
}

void launch_save_visible(const DevMap &m, void *scratch, unsigned nvis, bool restore, cudaStream_t s) {
  k_save_visible<<<sm_count() * 8, 256, 0, s>>>(m, (uint4 *)scratch, nvis, restore ? 1 : 0); note_launch();
}

}  // namespace sf
