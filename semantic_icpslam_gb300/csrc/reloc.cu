// Batched relocalisation scoring: n candidate camera poses scored against
// one frame's vertex map in a single launch, one CTA per candidate.
//
// The reference's loop has no such kernel; this is the RelocScoreBatch of
// the GB300 loop.  Each candidate moves the frame's vertices (every
// stride-th column and row) into the map and reads the TSDF there with the
// raycast's readSdfInterped (Mapping/RenderScene.cu:310-343): a sample
// counts when the interpolation is valid and finite, and is an inlier when
// |sdf| < inlier_sdf.  The per-candidate sums use a fixed order (per-thread
// float sums over samples i = t, t + 256, ..., then a shuffle-down tree in
// each warp and over the eight warp sums), so a score is deterministic and
// the oracle restates it bit for bit.  Block lookups go to the hash table
// (candidates need not lie in the last frame's window).
#include "sf_kernels.cuh"
#include "sf_sample.cuh"

namespace sf {
namespace {

constexpr int kRelocThreads = 256;

__global__ void __launch_bounds__(kRelocThreads) k_reloc_score(DevMap m, sf_image vmap, int stride,
                                                                const float *poses, int n,
                                                                float inlier_sdf, sf_reloc_score *out) {
  const int k = blockIdx.x;
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
  for (int i = threadIdx.x; i < N; i += kRelocThreads) {
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
    if (lane == 0) {
      sf_reloc_score o;
      o.valid = valid;
      o.inliers = inl;
      o.sum_abs_sdf = sum;
      o.mean_abs_sdf = valid ? __fdiv_rn(sum, (float)valid) : __int_as_float(0x7fffffff);
      out[k] = o;
    }
  }
}

}  // namespace

void launch_reloc_score(const DevMap &m, const sf_image &vmap, int stride, const float *poses, int n,
                        float inlier_sdf, sf_reloc_score *out, cudaStream_t s) {
  k_reloc_score<<<n, kRelocThreads, 0, s>>>(m, vmap, stride, poses, n, inlier_sdf, out); note_launch();
}

}  // namespace sf
