// Batched relocalisation scoring: n candidate camera poses scored against
// one frame's vertex map, each candidate spread over kRelocSplit CTAs.
//
// The reference's loop has no such kernel; this is the RelocScoreBatch of
// the GB300 loop.  Each candidate moves the frame's vertices (every
// stride-th column and row) into the map and reads the TSDF there with the
// raycast's readSdfInterped (Mapping/RenderScene.cu:310-343): a sample
// counts when the interpolation is valid and finite, and is an inlier when
// |sdf| < inlier_sdf.  The per-candidate sums use a fixed order, so a
// score is deterministic and the oracle restates it bit for bit: CTA c of
// a candidate has its thread t sum samples i = 256 c + t, + 256 kRelocSplit,
// ... in float, then a shuffle-down tree in each warp and over the eight
// warp sums gives the CTA's partial; a second launch adds a candidate's
// kRelocSplit partials with a shuffle-down tree (offsets 4, 2, 1).  Block
// lookups go to the hash table (candidates need not lie in the last
// frame's window).  One CTA per candidate filled 256 candidates into 1.7
// CTAs per SM.
#include "sf_kernels.cuh"
#include "sf_sample.cuh"

namespace sf {
namespace {

constexpr int kRelocThreads = 256;
constexpr int kRelocSplit = 8;

// Sum, valid and inlier counts of a CTA's threads: a shuffle-down tree in
// each warp, then over the warp sums (the result in thread 0).
__device__ __forceinline__ void reloc_block_tree(float &sum, unsigned &valid, unsigned &inl, float *wsum,
                                                 unsigned *wvalid, unsigned *winl) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    sum += __shfl_down_sync(0xffffffffu, sum, off);
    valid += __shfl_down_sync(0xffffffffu, valid, off);
    inl += __shfl_down_sync(0xffffffffu, inl, off);
  }
  if (lane == 0) {
    wsum[warp] = sum;
    wvalid[warp] = valid;
    winl[warp] = inl;
  }
  __syncthreads();
  if (warp == 0) {
    constexpr int NW = kRelocThreads / 32;
    sum = lane < NW ? wsum[lane] : 0.f;
    valid = lane < NW ? wvalid[lane] : 0u;
    inl = lane < NW ? winl[lane] : 0u;
#pragma unroll
    for (int off = NW / 2; off > 0; off >>= 1) {
      sum += __shfl_down_sync(0xffffffffu, sum, off);
      valid += __shfl_down_sync(0xffffffffu, valid, off);
      inl += __shfl_down_sync(0xffffffffu, inl, off);
    }
  }
}

// CTA (c, k): candidate k's samples 256 c + t + 256 kRelocSplit j; its
// partial to part[k][c].
__global__ void __launch_bounds__(kRelocThreads) k_reloc_score(DevMap m, sf_image vmap, int stride,
                                                                const float *poses, int n, float inlier_sdf,
                                                                sf_reloc_score *part) {
  const int k = blockIdx.y, cta = blockIdx.x;
  if (k >= n) return;
  __shared__ float P[12];
  __shared__ float wsum[kRelocThreads / 32];
  __shared__ unsigned wvalid[kRelocThreads / 32], winl[kRelocThreads / 32];
  if (threadIdx.x < 12) P[threadIdx.x] = poses[(size_t)k * 12 + threadIdx.x];
  __syncthreads();
  m3 R;
  R.rx = mk3(P[0], P[1], P[2]);
  R.ry = mk3(P[3], P[4], P[5]);
  R.rz = mk3(P[6], P[7], P[8]);
  const f3 t = mk3(P[9], P[10], P[11]);
  RayCtx r;
  r.voxels = m.voxels;
  r.cells = nullptr;
  for (int i = 0; i < 6; ++i) r.win[i] = 0;  // empty window: every lookup hashes
  ray_ctx_map(r, m);
  const float vsi = m.c.voxel_size_inv;
  const int sc = (vmap.cols + stride - 1) / stride, sr = (vmap.rows + stride - 1) / stride;
  const int N = sc * sr;
  unsigned valid = 0, inl = 0;
  float sum = 0.f;
  for (int i = cta * kRelocThreads + threadIdx.x; i < N; i += kRelocThreads * kRelocSplit) {
    const int y = (i / sc) * stride, x = (i % sc) * stride;
    const float4 v4 = __ldg(row_ptr<const float4>(vmap, y) + x);
    if (isnan(v4.x)) continue;
    const f3 pt = (mul(R, xyz(v4)) + t) * vsi;
    bool ok;
    const float s = sdf_interp(r, pt, ok);
    if (!ok || isnan(s)) continue;
    ++valid;
    const float a = fabsf(s);
    if (a < inlier_sdf) ++inl;
    sum += a;
  }
  reloc_block_tree(sum, valid, inl, wsum, wvalid, winl);
  if (threadIdx.x == 0) {
    sf_reloc_score o;
    o.valid = valid;
    o.inliers = inl;
    o.sum_abs_sdf = sum;
    o.mean_abs_sdf = 0.f;
    part[(size_t)k * kRelocSplit + cta] = o;
  }
}

// Warp k: candidate k's kRelocSplit partials added with a shuffle-down tree.
__global__ void k_reloc_finish(const sf_reloc_score *part, int n, sf_reloc_score *out) {
  const int k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (k >= n) return;  // uniform over the warp
  sf_reloc_score p = {};
  if (lane < kRelocSplit) p = part[(size_t)k * kRelocSplit + lane];
  float sum = p.sum_abs_sdf;
  unsigned valid = p.valid, inl = p.inliers;
#pragma unroll
  for (int off = kRelocSplit / 2; off > 0; off >>= 1) {
    sum += __shfl_down_sync(0xffffffffu, sum, off);
    valid += __shfl_down_sync(0xffffffffu, valid, off);
    inl += __shfl_down_sync(0xffffffffu, inl, off);
  }
  if (lane == 0) {
    sf_reloc_score o;
    o.valid = valid;
    o.inliers = inl;
    o.sum_abs_sdf = sum;
    o.mean_abs_sdf = valid ? __fdiv_rn(sum, (float)valid) : __int_as_float(0x7fffffff);
    out[k] = o;
  }
}

}  // namespace

int reloc_score_parts() { return kRelocSplit; }

void launch_reloc_score(const DevMap &m, const sf_image &vmap, int stride, const float *poses, int n,
                        float inlier_sdf, sf_reloc_score *part, sf_reloc_score *out, cudaStream_t s) {
  k_reloc_score<<<dim3(kRelocSplit, n), kRelocThreads, 0, s>>>(m, vmap, stride, poses, n, inlier_sdf, part);
  note_launch();
  k_reloc_finish<<<(n + 7) / 8, 256, 0, s>>>(part, n, out); note_launch();
}

}  // namespace sf
