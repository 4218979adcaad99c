// Depth pyramid: bilateral filter, Gaussian pyramid, vertex and normal maps,
// and the 2x2 vertex/normal downsampling of the raycast maps.
//
// Reference: Tracking/Pyrdown.cu (FilterDepthKernel :72-108,
// ComputeVMapKernel :123-145, ComputeNMapKernel :160-181,
// PyrDownGaussKernel :201-225, ResizeMapKernel :318-346) driven by
// Frame::FillImages / ResizeImages (Core/Frame.cc:68-98).
//
// GB300 layout: the whole pyramid is two launches.  The bilateral filter
// stages its tile in shared memory; then one kernel makes every coarser
// level and every level's vertex and normal maps from tiles staged in
// shared memory (k_pyramid_levels_*), recomputing the halos it needs
// rather than round-tripping levels and vertex maps through memory.  The
// per-operation kernels (k_pyrdown, k_vnmap, k_vmap, k_nmap) serve the
// reference-shaped entry points.  All maps are dense (step = cols *
// sizeof), 16-byte float4 stores are coalesced across a warp.
#include "sf_kernels.cuh"

namespace sf {

__constant__ float c_gauss[25] = {1, 4, 6, 4, 1, 4, 16, 24, 16, 4, 6, 24, 36,
                                  24, 6, 4, 16, 24, 16, 4, 1, 4, 6, 4, 1};

// FilterDepthKernel (Pyrdown.cu:72-108).  sigSpace = 0.5/16, sigRange =
// 0.5/0.25 (Pyrdown.cu:3-4).  The window's upper bound is exclusive, as in
// the reference.
//
// A CTA filters a 32x8 tile.  The depths of the tile and its 2-pixel halo
// are converted to metres once and staged in shared memory; a pixel whose
// whole 5x5 window lies inside the image takes the fully unrolled taps
// (space2 * sigSpace is then a constant), the others the clipped loops.
// Both visit the taps in the reference's order with the same operations
// (space2 * 2^-5 and color2 * 2 are exact), so the filtered depth is the
// same as a per-pixel global-memory form's.
constexpr int kFiltTX = 32, kFiltTY = 8;
constexpr int kFiltSX = kFiltTX + 4, kFiltSY = kFiltTY + 4;

__global__ void __launch_bounds__(kFiltTX * kFiltTY) k_filter_depth(sf_image depth, sf_image raw, sf_image filt,
                                                                    float inv_scale, float cutoff) {
  __shared__ float s_m[kFiltSY][kFiltSX];
  const int x0 = blockIdx.x * kFiltTX, y0 = blockIdx.y * kFiltTY;
  const int tid = threadIdx.y * kFiltTX + threadIdx.x;
  constexpr int kN = kFiltSX * kFiltSY, kPer = (kN + kFiltTX * kFiltTY - 1) / (kFiltTX * kFiltTY);
  float stage[kPer];
#pragma unroll
  for (int k = 0; k < kPer; ++k) {
    const int i = tid + k * kFiltTX * kFiltTY;
    const int gx = x0 - 2 + i % kFiltSX, gy = y0 - 2 + i / kFiltSX;
    stage[k] = (i < kN && gx >= 0 && gy >= 0 && gx < depth.cols && gy < depth.rows)
                   ? (float)__ldg(row_ptr<const uint16_t>(depth, gy) + gx) * inv_scale
                   : 0.f;
  }
#pragma unroll
  for (int k = 0; k < kPer; ++k) {
    const int i = tid + k * kFiltTX * kFiltTY;
    if (i < kN) s_m[i / kFiltSX][i % kFiltSX] = stage[k];
  }
  __syncthreads();
  const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
  if (x >= depth.cols || y >= depth.rows) return;
  const float sig_space = 0.03125f, sig_range = 2.0f;
  const int lx = threadIdx.x + 2, ly = threadIdx.y + 2;
  const float center = s_m[ly][lx];
  row_ptr<float>(raw, y)[x] = center < cutoff ? center : nanf_bits();
  float sum1 = 0.f, sum2 = 0.f;
  if (x >= 2 && y >= 2 && x + 3 <= depth.cols - 1 && y + 3 <= depth.rows - 1) {
#pragma unroll
    for (int dy = -2; dy <= 2; ++dy) {
#pragma unroll
      for (int dx = -2; dx <= 2; ++dx) {
        const float val = s_m[ly + dy][lx + dx];
        const float space2 = (float)(dx * dx + dy * dy);
        const float color2 = (center - val) * (center - val);
        const float weight = expf(-(space2 * sig_space + color2 * sig_range));
        sum1 += val * weight;
        sum2 += weight;
      }
    }
  } else {
    const int tx = min(x + 3, depth.cols - 1);
    const int ty = min(y + 3, depth.rows - 1);
    for (int cy = max(y - 2, 0); cy < ty; ++cy) {
      for (int cx = max(x - 2, 0); cx < tx; ++cx) {
        const float val = s_m[cy - y0 + 2][cx - x0 + 2];
        const float space2 = (float)((x - cx) * (x - cx) + (y - cy) * (y - cy));
        const float color2 = (center - val) * (center - val);
        const float weight = expf(-(space2 * sig_space + color2 * sig_range));
        sum1 += val * weight;
        sum2 += weight;
      }
    }
  }
  const float fin = sum1 / sum2;
  row_ptr<float>(filt, y)[x] = fin < cutoff ? fin : nanf_bits();
}

// PyrDownGaussKernel<float,float> (Pyrdown.cu:201-225): NaN-skipping 5x5
// Gaussian normalised by the used weights, reversed kernel index.  The
// reference's count = (int)((float)count + k) only ever adds small integers
// (the weights sum to 256), so it is the integer sum of the used weights.
__device__ __forceinline__ float pyrdown_px(const sf_image &src, int x, int y) {
  const int tx = min(2 * x + 3, src.cols - 1);
  const int ty = min(2 * y + 3, src.rows - 1);
  float sum = 0.f;
  int count = 0;
  for (int cy = max(0, 2 * y - 2); cy < ty; ++cy) {
    const float *srow = row_ptr<const float>(src, cy);
    for (int cx = max(0, 2 * x - 2); cx < tx; ++cx) {
      float v = __ldg(srow + cx);
      if (!isnan(v)) {
        float k = c_gauss[(ty - cy - 1) * 5 + (tx - cx - 1)];
        sum += v * k;
        count += (int)k;
      }
    }
  }
  return sum / (float)count;
}

// The same with the whole window inside the source: p points at tap
// (2x - 2, 2y - 2) of a row-major array with row stride `stride`.  The
// weights are symmetric, so the reversed index reads the same table; the
// taps are selects, not branches (every library file is built without
// multiply-add contraction, so sum + v * k rounds twice as above).
__device__ __forceinline__ float pyrdown_interior(const float *p, int stride) {
  constexpr int g[5] = {1, 4, 6, 4, 1};
  float sum = 0.f;
  int count = 0;
#pragma unroll
  for (int r = 0; r < 5; ++r) {
#pragma unroll
    for (int c = 0; c < 5; ++c) {
      const float v = p[r * stride + c];
      const bool ok = !isnan(v);
      sum = ok ? sum + v * (float)(g[r] * g[c]) : sum;
      count += ok ? g[r] * g[c] : 0;
    }
  }
  return sum / (float)count;
}

__global__ void k_pyrdown(sf_image src, sf_image dst) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= dst.cols || y >= dst.rows) return;
  row_ptr<float>(dst, y)[x] = pyrdown_px(src, x, y);
}

// ComputeVMapKernel (Pyrdown.cu:123-145): z in (0.1, cutoff), where the
// reference compares (double)z > 0.1.  No float lies in (0.1, 0.1f], so for
// a float z that is exactly z >= 0.1f, with no FP64 instruction.
__device__ __forceinline__ float4 vertex_of(float z, int x, int y, float invfx, float invfy, float cx,
                                            float cy, float cutoff) {
  if (!isnan(z) && z >= 0.1f && z < cutoff) {
    return make_float4(z * ((float)x - cx) * invfx, z * ((float)y - cy) * invfy, z, 1.0f);
  }
  return nan4();
}
__device__ __forceinline__ float4 vertex_at(const sf_image &depth, int x, int y, float invfx,
                                            float invfy, float cx, float cy, float cutoff) {
  return vertex_of(__ldg(row_ptr<const float>(depth, y) + x), x, y, invfx, invfy, cx, cy, cutoff);
}

// ComputeNMapKernel's normal (Pyrdown.cu:160-181) from the vertex and its
// right and lower neighbours.
__device__ __forceinline__ float4 normal_of(float4 vc, float4 vr, float4 vd) {
  if (isnan(vc.x) || isnan(vr.x) || isnan(vd.x)) return nan4();
  f3 a = mk3(vr.x - vc.x, vr.y - vc.y, vr.z - vc.z);
  f3 b = mk3(vd.x - vc.x, vd.y - vc.y, vd.z - vc.z);
  f3 q = normalised(cross(a, b));
  return make_float4(q.x, q.y, q.z, 1.0f);
}

// ComputeVMap + ComputeNMap fused (Pyrdown.cu:123-181).
__global__ void k_vnmap(sf_image depth, sf_image vmap, sf_image nmap, float invfx, float invfy,
                        float cx, float cy, float cutoff) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= depth.cols || y >= depth.rows) return;
  float4 vc = vertex_at(depth, x, y, invfx, invfy, cx, cy, cutoff);
  row_ptr<float4>(vmap, y)[x] = vc;
  float4 n = nan4();
  if (x != depth.cols - 1 && y != depth.rows - 1) {
    float4 vr = vertex_at(depth, x + 1, y, invfx, invfy, cx, cy, cutoff);
    float4 vd = vertex_at(depth, x, y + 1, invfx, invfy, cx, cy, cutoff);
    n = normal_of(vc, vr, vd);
  }
  row_ptr<float4>(nmap, y)[x] = n;
}

// Levels 1..NL-1 of the Gaussian pyramid and the vertex and normal maps of
// every level, from the filtered level-0 depth, in one launch.  A CTA owns
// an 8x8 tile of the coarsest level and the 2^l times larger tiles under
// it; it stages in shared memory the region of each level that its windows
// reach (the 5x5 PyrDownGauss taps of the level below, the right and lower
// neighbours of the normals) and recomputes the halo instead of waiting
// for other CTAs.  Every value is computed with the same operations, in
// the same order, as k_pyrdown and k_vnmap, so the maps are bit-identical
// to theirs.
template <int NL>
struct PyrTile {
  // region of level l, relative to the tile origin: [lo, hi] inclusive
  __host__ __device__ static constexpr int lo(int l) { return l >= NL - 1 ? 0 : 2 * lo(l + 1) - 2; }
  __host__ __device__ static constexpr int hi(int l) { return l >= NL - 1 ? 8 : 2 * hi(l + 1) + 2; }
  __host__ __device__ static constexpr int n(int l) { return hi(l) - lo(l) + 1; }
  __host__ __device__ static constexpr int tile(int l) { return 8 << (NL - 1 - l); }
  __host__ __device__ static constexpr int off(int l) { return l == 0 ? 0 : off(l - 1) + n(l - 1) * n(l - 1); }
  __host__ __device__ static constexpr int total() { return off(NL); }
};

// 512 threads, two CTAs per SM: a 640x480 frame's 300 tiles run in one wave.
constexpr int kPyrThreads = 512;

template <int NL>
__device__ __forceinline__ void pyramid_levels(const PyramidArgs &a) {
  using T = PyrTile<NL>;
  __shared__ float s[T::total()];
  const int X = blockIdx.x, Y = blockIdx.y;
  {  // level 0 region: all of a thread's loads in flight before the stores
    constexpr int n = T::n(0), kPer = (n * n + kPyrThreads - 1) / kPyrThreads;
    const int ox = X * T::tile(0) + T::lo(0), oy = Y * T::tile(0) + T::lo(0);
    const sf_image &d = a.depth[0];
    float v[kPer];
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
      const int i = threadIdx.x + kPyrThreads * k;
      const int yy = i / n, xx = i - yy * n;
      const int gx = ox + xx, gy = oy + yy;
      v[k] = (i < n * n && gx >= 0 && gy >= 0 && gx < d.cols && gy < d.rows)
                 ? __ldg(row_ptr<const float>(d, gy) + gx)
                 : 0.f;
    }
#pragma unroll
    for (int k = 0; k < kPer; ++k)
      if (threadIdx.x + kPyrThreads * k < n * n) s[threadIdx.x + kPyrThreads * k] = v[k];
  }
  __syncthreads();
#pragma unroll
  for (int l = 1; l < NL; ++l) {
    const int n = T::n(l), np = T::n(l - 1);
    const int t = T::tile(l);
    const int ox = X * t + T::lo(l), oy = Y * t + T::lo(l);
    const int opx = 2 * X * t + T::lo(l - 1), opy = 2 * Y * t + T::lo(l - 1);
    const sf_image &d = a.depth[l];
    const int pc = a.depth[l - 1].cols, pr = a.depth[l - 1].rows;
    const float *src = s + T::off(l - 1);
    for (int i = threadIdx.x; i < n * n; i += blockDim.x) {
      const int yy = i / n, xx = i - yy * n;
      const int x = ox + xx, y = oy + yy;
      if (x < 0 || y < 0 || x >= d.cols || y >= d.rows) continue;
      // pyrdown_px over the staged level below
      float v;
      if (x >= 1 && y >= 1 && 2 * x + 3 <= pc - 1 && 2 * y + 3 <= pr - 1) {
        v = pyrdown_interior(src + (2 * y - 2 - opy) * np + (2 * x - 2 - opx), np);
      } else {
        const int tx = min(2 * x + 3, pc - 1);
        const int ty = min(2 * y + 3, pr - 1);
        float sum = 0.f;
        int count = 0;
        for (int cy = max(0, 2 * y - 2); cy < ty; ++cy) {
          const float *srow = src + (cy - opy) * np - opx;
          for (int cx = max(0, 2 * x - 2); cx < tx; ++cx) {
            float sv = srow[cx];
            if (!isnan(sv)) {
              float k = c_gauss[(ty - cy - 1) * 5 + (tx - cx - 1)];
              sum += sv * k;
              count += (int)k;
            }
          }
        }
        v = sum / (float)count;
      }
      s[T::off(l) + i] = v;
      if (xx >= -T::lo(l) && xx < t - T::lo(l) && yy >= -T::lo(l) && yy < t - T::lo(l))
        row_ptr<float>(d, y)[x] = v;
    }
    __syncthreads();
  }
#pragma unroll
  for (int l = 0; l < NL; ++l) {
    const int n = T::n(l), t = T::tile(l);
    const int ox = X * t + T::lo(l), oy = Y * t + T::lo(l);
    const sf_image &d = a.depth[l];
    const PyramidLevelK k = a.k[l];
    const float *z = s + T::off(l);
    for (int i = threadIdx.x; i < t * t; i += blockDim.x) {
      const int ty = i / t, tx = i - ty * t;
      const int x = X * t + tx, y = Y * t + ty;
      if (x >= d.cols || y >= d.rows) continue;
      const int r = (y - oy) * n + (x - ox);
      const float4 vc = vertex_of(z[r], x, y, k.invfx, k.invfy, k.cx, k.cy, a.cutoff);
      row_ptr<float4>(a.vmap[l], y)[x] = vc;
      float4 nm = nan4();
      if (x != d.cols - 1 && y != d.rows - 1) {
        const float4 vr = vertex_of(z[r + 1], x + 1, y, k.invfx, k.invfy, k.cx, k.cy, a.cutoff);
        const float4 vd = vertex_of(z[r + n], x, y + 1, k.invfx, k.invfy, k.cx, k.cy, a.cutoff);
        nm = normal_of(vc, vr, vd);
      }
      row_ptr<float4>(a.nmap[l], y)[x] = nm;
    }
  }
}

__global__ void __launch_bounds__(kPyrThreads, 2) k_pyramid_levels_2(PyramidArgs a) { pyramid_levels<2>(a); }
__global__ void __launch_bounds__(kPyrThreads, 2) k_pyramid_levels_3(PyramidArgs a) { pyramid_levels<3>(a); }
__global__ void __launch_bounds__(kPyrThreads, 2) k_pyramid_levels_4(PyramidArgs a) { pyramid_levels<4>(a); }
static_assert(PyrTile<3>::n(0) == 45 && PyrTile<3>::n(1) == 21 && PyrTile<3>::n(2) == 9, "tile regions");
static_assert(PyrTile<4>::total() * sizeof(float) <= 48 * 1024, "static shared memory");

// Separate vertex-map and normal-map kernels for the reference-shaped
// launchers (ComputeVMap / ComputeNMap).
__global__ void k_vmap(sf_image depth, sf_image vmap, float invfx, float invfy, float cx, float cy,
                       float cutoff) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= depth.cols || y >= depth.rows) return;
  row_ptr<float4>(vmap, y)[x] = vertex_at(depth, x, y, invfx, invfy, cx, cy, cutoff);
}

__global__ void k_nmap(sf_image vmap, sf_image nmap) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= vmap.cols || y >= vmap.rows) return;
  float4 n = nan4();
  if (x != vmap.cols - 1 && y != vmap.rows - 1) {
    float4 vc = row_ptr<const float4>(vmap, y)[x];
    float4 vr = row_ptr<const float4>(vmap, y)[x + 1];
    float4 vd = row_ptr<const float4>(vmap, y + 1)[x];
    if (!isnan(vc.x) && !isnan(vr.x) && !isnan(vd.x)) {
      f3 a = mk3(vr.x - vc.x, vr.y - vc.y, vr.z - vc.z);
      f3 b = mk3(vd.x - vc.x, vd.y - vc.y, vd.z - vc.z);
      f3 q = normalised(cross(a, b));
      n = make_float4(q.x, q.y, q.z, 1.0f);
    }
  }
  row_ptr<float4>(nmap, y)[x] = n;
}

// ResizeMapKernel (Pyrdown.cu:318-346): 2x2 mean, any NaN -> NaN; normals
// normalised as float4 (w included in the norm, VectorMath.h:328-346).
__device__ __forceinline__ float4 resize_vertex(float4 a, float4 b, float4 c, float4 d) {
  if (isnan(a.x) || isnan(b.x) || isnan(c.x) || isnan(d.x)) return nan4();
  float4 out;
  out.x = (((a.x + b.x) + c.x) + d.x) / 4.0f;
  out.y = (((a.y + b.y) + c.y) + d.y) / 4.0f;
  out.z = (((a.z + b.z) + c.z) + d.z) / 4.0f;
  out.w = (((a.w + b.w) + c.w) + d.w) / 4.0f;
  return out;
}

__device__ __forceinline__ float4 resize_normal(float4 a, float4 b, float4 c, float4 d) {
  if (isnan(a.x) || isnan(b.x) || isnan(c.x) || isnan(d.x)) return nan4();
  float s0 = (((a.x + b.x) + c.x) + d.x) / 4.0f;
  float s1 = (((a.y + b.y) + c.y) + d.y) / 4.0f;
  float s2 = (((a.z + b.z) + c.z) + d.z) / 4.0f;
  float s3 = (((a.w + b.w) + c.w) + d.w) / 4.0f;
  float len = sqrtf(s0 * s0 + s1 * s1 + s2 * s2 + s3 * s3);
  return make_float4(s0 / len, s1 / len, s2 / len, s3 / len);
}

// One destination pixel.  Guarded on the destination size (the reference
// guards on the source).
__device__ __forceinline__ void resize_px(const sf_image &vsrc, const sf_image &nsrc, const sf_image &vdst,
                                          const sf_image &ndst, int x, int y) {
  const float4 *v0 = row_ptr<const float4>(vsrc, 2 * y) + 2 * x;
  const float4 *v1 = row_ptr<const float4>(vsrc, 2 * y + 1) + 2 * x;
  const float4 *n0 = row_ptr<const float4>(nsrc, 2 * y) + 2 * x;
  const float4 *n1 = row_ptr<const float4>(nsrc, 2 * y + 1) + 2 * x;
  row_ptr<float4>(vdst, y)[x] = resize_vertex(v0[0], v0[1], v1[0], v1[1]);
  row_ptr<float4>(ndst, y)[x] = resize_normal(n0[0], n0[1], n1[0], n1[1]);
}

// Two ResizeMap levels in one launch (level 0 -> 1 -> 2): thread (x, y)
// makes the level-1 pixels (2x + i, 2y + j) that exist and, from those four
// values, level-2 pixel (x, y) when it exists; the same operations as two
// k_resize launches, so the maps are bit-identical.  The grid covers level
// 1 in 2x2 cells (an odd level-1 size leaves its last column or row to
// threads without a level-2 pixel).
__global__ void k_resize2(sf_image v0, sf_image n0, sf_image v1, sf_image n1, sf_image v2, sf_image n2) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (2 * x >= v1.cols || 2 * y >= v1.rows) return;
  float4 pv[4], pn[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int px = 2 * x + (k & 1), py = 2 * y + (k >> 1);
    if (px < v1.cols && py < v1.rows) {
      const float4 *a = row_ptr<const float4>(v0, 2 * py) + 2 * px;
      const float4 *b = row_ptr<const float4>(v0, 2 * py + 1) + 2 * px;
      const float4 *c = row_ptr<const float4>(n0, 2 * py) + 2 * px;
      const float4 *d = row_ptr<const float4>(n0, 2 * py + 1) + 2 * px;
      pv[k] = resize_vertex(a[0], a[1], b[0], b[1]);
      pn[k] = resize_normal(c[0], c[1], d[0], d[1]);
      row_ptr<float4>(v1, py)[px] = pv[k];
      row_ptr<float4>(n1, py)[px] = pn[k];
    }
  }
  if (x < v2.cols && y < v2.rows) {
    row_ptr<float4>(v2, y)[x] = resize_vertex(pv[0], pv[1], pv[2], pv[3]);
    row_ptr<float4>(n2, y)[x] = resize_normal(pn[0], pn[1], pn[2], pn[3]);
  }
}

__global__ void k_resize(sf_image vsrc, sf_image nsrc, sf_image vdst, sf_image ndst) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= vdst.cols || y >= vdst.rows) return;
  resize_px(vsrc, nsrc, vdst, ndst, x, y);
}

// Frame::ResizeImages of n stacked candidates (Tracker::ValidatePose,
// Tracking.cc:762): grid.z is the candidate; those with src[c] != c (not
// drawn this call) are left alone.
__global__ void k_resize_batch(sf_image vsrc, sf_image nsrc, sf_image vdst, sf_image ndst, int src_rows,
                               int dst_rows, const int *src) {
  const int k = blockIdx.z;
  if (src[k] != k) return;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= vdst.cols || y >= dst_rows) return;
  sf_image vs = vsrc, ns = nsrc, vd = vdst, nd = ndst;
  vs.data = (char *)vsrc.data + (size_t)k * src_rows * vsrc.step;
  ns.data = (char *)nsrc.data + (size_t)k * src_rows * nsrc.step;
  vd.data = (char *)vdst.data + (size_t)k * dst_rows * vdst.step;
  nd.data = (char *)ndst.data + (size_t)k * dst_rows * ndst.step;
  vs.rows = ns.rows = src_rows;
  vd.rows = nd.rows = dst_rows;
  resize_px(vs, ns, vd, nd, x, y);
}

// ------------------------------------------------------------- launchers
// Mapping::SemanticAnalysis' rendered depth (Mapping.cc:99-111): the z of
// the raycast vertex map, NaN where the ray found no surface.
__global__ void k_vmap_depth(sf_image vmap, sf_image depth, const int *run_flag) {
  if (run_flag && *run_flag == 0) return;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= depth.cols || y >= depth.rows) return;
  row_ptr<float>(depth, y)[x] = row_ptr<const float4>(vmap, y)[x].z;
}

static inline dim3 grid2d(int cols, int rows, dim3 blk) {
  return dim3((cols + blk.x - 1) / blk.x, (rows + blk.y - 1) / blk.y);
}

void launch_filter_depth(const sf_image &depth, const sf_image &raw, const sf_image &filt,
                         float depth_scale, float cutoff, cudaStream_t s) {
  dim3 blk(kFiltTX, kFiltTY);
  const float inv = (float)(1.0 / (double)depth_scale);
  k_filter_depth<<<grid2d(depth.cols, depth.rows, blk), blk, 0, s>>>(depth, raw, filt, inv, cutoff); note_launch();
}

void launch_pyrdown(const sf_image &src, const sf_image &dst, cudaStream_t s) {
  dim3 blk(32, 8);
  k_pyrdown<<<grid2d(dst.cols, dst.rows, blk), blk, 0, s>>>(src, dst); note_launch();
}

bool pyramid_levels_fusable(const sf_image *depths, const sf_image *vmaps, const sf_image *nmaps, int levels) {
  if (levels < 2 || levels > kMaxLevels) return false;
  for (int l = 0; l < levels; ++l) {
    if (vmaps[l].cols != depths[l].cols || vmaps[l].rows != depths[l].rows) return false;
    if (nmaps[l].cols != depths[l].cols || nmaps[l].rows != depths[l].rows) return false;
    if (l > 0 && (depths[l].cols != depths[l - 1].cols >> 1 || depths[l].rows != depths[l - 1].rows >> 1))
      return false;
  }
  return depths[0].cols > 0 && depths[0].rows > 0;
}

void launch_pyramid_levels(const sf_image *depths, const sf_image *vmaps, const sf_image *nmaps, int levels,
                           float fx, float fy, float cx, float cy, float cutoff, cudaStream_t s) {
  PyramidArgs a;
  for (int l = 0; l < levels; ++l) {
    a.depth[l] = depths[l];
    a.vmap[l] = vmaps[l];
    a.nmap[l] = nmaps[l];
    const float div = (float)(1 << l);  // the per-level intrinsics of launch_vnmap's callers
    a.k[l].invfx = (float)(1.0 / (double)(fx / div));
    a.k[l].invfy = (float)(1.0 / (double)(fy / div));
    a.k[l].cx = cx / div;
    a.k[l].cy = cy / div;
  }
  a.cutoff = cutoff;
  const int t0 = 8 << (levels - 1);
  const dim3 grid((depths[0].cols + t0 - 1) / t0, (depths[0].rows + t0 - 1) / t0);
  if (levels == 2) k_pyramid_levels_2<<<grid, kPyrThreads, 0, s>>>(a);
  else if (levels == 3) k_pyramid_levels_3<<<grid, kPyrThreads, 0, s>>>(a);
  else k_pyramid_levels_4<<<grid, kPyrThreads, 0, s>>>(a);
  note_launch();
}

void launch_vnmap(const sf_image &depth, const sf_image &vmap, const sf_image &nmap, float fx,
                  float fy, float cx, float cy, float cutoff, cudaStream_t s) {
  dim3 blk(32, 8);
  k_vnmap<<<grid2d(depth.cols, depth.rows, blk), blk, 0, s>>>(
      depth, vmap, nmap, (float)(1.0 / (double)fx), (float)(1.0 / (double)fy), cx, cy, cutoff); note_launch();
}

void launch_vmap(const sf_image &depth, const sf_image &vmap, float fx, float fy, float cx,
                 float cy, float cutoff, cudaStream_t s) {
  dim3 blk(32, 8);
  k_vmap<<<grid2d(depth.cols, depth.rows, blk), blk, 0, s>>>(
      depth, vmap, (float)(1.0 / (double)fx), (float)(1.0 / (double)fy), cx, cy, cutoff); note_launch();
}

void launch_nmap(const sf_image &vmap, const sf_image &nmap, cudaStream_t s) {
  dim3 blk(32, 8);
  k_nmap<<<grid2d(vmap.cols, vmap.rows, blk), blk, 0, s>>>(vmap, nmap); note_launch();
}

void launch_vmap_depth(const sf_image &vmap, const sf_image &depth, const int *run_flag, cudaStream_t s) {
  dim3 blk(32, 8);
  k_vmap_depth<<<grid2d(depth.cols, depth.rows, blk), blk, 0, s>>>(vmap, depth, run_flag); note_launch();
}

void launch_resize(const sf_image &vsrc, const sf_image &nsrc, const sf_image &vdst,
                   const sf_image &ndst, cudaStream_t s) {
  dim3 blk(32, 8);
  k_resize<<<grid2d(vdst.cols, vdst.rows, blk), blk, 0, s>>>(vsrc, nsrc, vdst, ndst); note_launch();
}

void launch_resize2(const sf_image &v0, const sf_image &n0, const sf_image &v1, const sf_image &n1,
                    const sf_image &v2, const sf_image &n2, cudaStream_t s) {
  const dim3 blk(16, 8);
  k_resize2<<<grid2d((v1.cols + 1) / 2, (v1.rows + 1) / 2, blk), blk, 0, s>>>(v0, n0, v1, n1, v2, n2);
  note_launch();
}

void launch_resize_batch(const sf_image &vsrc, const sf_image &nsrc, const sf_image &vdst, const sf_image &ndst,
                         int src_rows, int dst_rows, int n, const int *src, cudaStream_t s) {
  dim3 blk(32, 8);
  dim3 grd = grid2d(vdst.cols, dst_rows, blk);
  grd.z = n;
  k_resize_batch<<<grd, blk, 0, s>>>(vsrc, nsrc, vdst, ndst, src_rows, dst_rows, src); note_launch();
}

}  // namespace sf
