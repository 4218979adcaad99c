// Projective point-to-plane ICP.
//
// Reference: ICPReduce::searchPoint / getRow (Tracking/Reduction.cu:228-290),
// the 29-float block reduction (WarpReduce / BlockReduce / Reduce<float,29>,
// :18-65), ICPStep (:328-385) and the host loop Tracker::ComputeSE3
// (Tracking/Tracking.cc:369-517), which downloads 29 floats and solves a
// 6x6 system on the host every iteration.
//
// GB300 form: one persistent cooperative kernel runs every pyramid level and
// iteration.  Per iteration each CTA reduces its pixels' 29 products
// (FP32 per pixel, compensated FP32 warp and block trees), adds the block
// totals into exact fixed-point accumulators with fire-and-forget atomics
// and crosses a bounded grid barrier.  One CTA runs the FP64 6x6 solve and
// SE(3) update and publishes the pose before the next barrier, while the
// pixel CTAs accumulate the next iteration's rows on a float prediction of
// that pose and keep them only when it matches the published pose bit for
// bit (k_icp_persistent below).  Accumulators rotate over three sets.
#include <mutex>

#include "sf_frame.cuh"

// Tracing slots of the solve phases (set per iteration in CTA 0 when
// tracing is on, else null); read by SF_SOLVE_MARK inside the solve.
__shared__ unsigned long long *s_solve_marks;
#define SF_SOLVE_MARK(k)                                           \
  do {                                                             \
    if (threadIdx.x == 0 && s_solve_marks) s_solve_marks[k] = clock64(); \
  } while (0)
#include "sf_icp_solve.cuh"
#include "sf_icp_spec.cuh"

namespace sf {

namespace {

// Persistent-kernel CTA size (a multiple of 32, at most 1024).  512 threads
// with the registers that one CTA per SM allows (about 124) measured
// fastest on GB300, ahead of 768 and 1024 threads at 64-85 registers.
#ifndef SF_ICP_PTHREADS
#define SF_ICP_PTHREADS 512
#endif
constexpr int kThreads = 512;               // plain-form kernels
constexpr int kPThreads = SF_ICP_PTHREADS;  // persistent kernel
constexpr int kProfIters = 64;
constexpr int kProfSlots = 16;  // per iteration (prof_mark): phases, global timer, prediction, solve steps
constexpr int kWarps = kThreads / 32;
constexpr int kPWarps = kPThreads / 32;

struct PoseF {
  m3 Rc, Rl, RlI, RcI;
  f3 tc, tl;
};

// (int)((double)t + 0.5) of Reduction.cu:239-240 evaluated in float: the
// double sum is exact for every float t, so the result is floor(t) +
// (frac(t) >= 0.5) for t >= -0.5, 0 for t in (-1.5, -0.5), negative below.
__device__ __forceinline__ int round_half_up(float t) {
  if (t >= -0.5f) {
    float f = floorf(t);
    int i = (int)f;
    return (t - f >= 0.5f) ? i + 1 : i;
  }
  return (t > -1.5f) ? 0 : -1;
}

// Frame::GpuRotation / GpuInvRotation / GpuTranslation (Core/Frame.cc
// :626-645) of the current and last poses, one element per lane of the
// calling warp (one FP64 conversion instruction, not 21 in one thread).
__device__ __forceinline__ void pose_to_float_warp(const double *Pc, const double *Pl, PoseF &p) {
  const int lane = threadIdx.x & 31;
  if (lane < 9) {
    const int i = lane / 3, j = lane - 3 * (lane / 3);
    const float rc = (float)Pc[i * 4 + j], rl = (float)Pl[i * 4 + j];
    (&p.Rc.rx.x)[lane] = rc;
    (&p.RcI.rx.x)[j * 3 + i] = rc;
    (&p.Rl.rx.x)[lane] = rl;
    (&p.RlI.rx.x)[j * 3 + i] = rl;
  } else if (lane < 12) {
    const int i = lane - 9;
    (&p.tc.x)[i] = (float)Pc[i * 4 + 3];
    (&p.tl.x)[i] = (float)Pl[i * 4 + 3];
  }
}
static_assert(sizeof(m3) == 9 * sizeof(float) && sizeof(f3) == 3 * sizeof(float), "packed pose");

// ICPReduce::searchPoint + getRow (Reduction.cu:228-279), split at the
// dependent loads: icp_project maps a current vertex to the model pixel
// (u, v), icp_finish takes the three loads and returns the row.
struct IcpProj {
  f3 vg;  // current vertex in the world frame
  f3 vp;  // the same in the last camera's frame
  int u, v;
  bool ok;
};

__device__ __forceinline__ IcpProj icp_project(const IcpLevelArgs &L, const PoseF &p, float4 vc4) {
  IcpProj q;
  q.ok = false;
  q.u = 0;
  q.v = 0;
  const f3 vcurr_c = xyz(vc4);
  q.vg = mul(p.Rc, vcurr_c) + p.tc;
  // (double)z < 1e-3 of the reference is exactly z < 0.001f for a float z
  if (isnan(vcurr_c.x) || vcurr_c.z < 0.001f) return q;
  const f3 vcurr_p = mul(p.RlI, q.vg - p.tl);
  q.vp = vcurr_p;
  // (float)(1.0 / (double)z): double rounding is innocuous for division,
  // so this equals the correctly rounded float quotient.
  const float invz = __fdiv_rn(1.0f, vcurr_p.z);
  q.u = round_half_up(vcurr_p.x * invz * L.fx + L.cx);
  q.v = round_half_up(vcurr_p.y * invz * L.fy + L.cy);
  q.ok = !(q.u < 0 || q.v < 0 || q.u >= L.vc.cols || q.v >= L.vc.rows);
  return q;
}

__device__ __forceinline__ bool icp_finish(const PoseF &p, const IcpProj &q, float4 vl4, float4 nl4,
                                           float4 nc4, float row[7]) {
  const f3 vlast_g = mul(p.Rl, xyz(vl4)) + p.tl;
  const f3 ncurr_g = mul(p.Rc, xyz(nc4));
  const f3 nlast_g = mul(p.Rl, xyz(nl4));
  // dist = norm(vlast_g - vg) <= 0.1f and sine = norm(ncurr_g x nlast_g)
  // < 0.6f without the square roots: sqrtf is correctly rounded and
  // monotone, so sqrtf(d) <= 0.1f iff d <= 0x3c23d70b (0.010000001f) and
  // sqrtf(s) < 0.6f iff s < 0x3eb851ec (0.36f), the squared norms being
  // the same dot products norm() takes.
  const f3 dv = vlast_g - q.vg, cr_n = cross(ncurr_g, nlast_g);
  const float dist2 = dot(dv, dv), sine2 = dot(cr_n, cr_n);
  if (!(sine2 < __int_as_float(0x3eb851ec) && dist2 <= __int_as_float(0x3c23d70b) && !isnan(nc4.x) &&
        !isnan(nl4.x)))
    return false;
  const f3 nlast = mul(p.RlI, nlast_g);
  const f3 vcurr = q.vp;  // mul(p.RlI, q.vg - p.tl), computed by icp_project
  const f3 vlast = mul(p.RlI, vlast_g - p.tl);
  const f3 mn = -nlast;
  const f3 cr = cross(nlast, vlast);
  row[0] = mn.x; row[1] = mn.y; row[2] = mn.z;
  row[3] = cr.x; row[4] = cr.y; row[5] = cr.z;
  row[6] = dot(mn, vcurr - vlast);
  return true;
}

// The 28 products of the row, each fused into its running sum (one
// rounding per term; the per-thread order of pixels is kept).
__device__ __forceinline__ void icp_add_row(float acc[29], const float row[7]) {
  int k = 0;
#pragma unroll
  for (int a = 0; a < 7; ++a)
#pragma unroll
    for (int b = a; b < 7; ++b, ++k) acc[k] = fmaf(row[a], row[b], acc[k]);
  acc[28] += 1.0f;
}

// Accumulates the 29 terms (Reduction.cu:281-289) of this thread's pixels
// i = gtid, gtid + gstride, ... in that order.  Pixels go in batches of
// kIcpBatch: the batch's current vertices are loaded together, then its
// model gathers, so a thread waits for two memory round trips per batch
// instead of two per pixel.
#ifndef SF_ICP_BATCH
#define SF_ICP_BATCH 2
#endif
constexpr int kIcpBatch = SF_ICP_BATCH;

__device__ __forceinline__ void icp_accumulate(const IcpLevelArgs &L, const PoseF &p, int gtid,
                                               int gstride, float acc[29]) {
#pragma unroll
  for (int k = 0; k < 29; ++k) acc[k] = 0.f;
  const int cols = L.vc.cols;
  const int N = cols * L.vc.rows;
  // i / cols through the float reciprocal: for i < 2^24 the product's two
  // roundings put it within (i / cols) 2^-23 < 1 of the quotient, so the
  // truncated estimate is off by at most one, which the remainder test
  // corrects.  Larger images divide.
  const float inv_cols = 1.0f / (float)cols;
  const bool small = N < (1 << 24) - kIcpBatch * gstride;
  for (int i0 = gtid; i0 < N; i0 += kIcpBatch * gstride) {
    float4 vc[kIcpBatch];
    int xs[kIcpBatch], ys[kIcpBatch];
#pragma unroll
    for (int b = 0; b < kIcpBatch; ++b) {
      const int i = i0 + b * gstride;
      int y, x;
      if (small) {
        y = (int)((float)i * inv_cols);
        x = i - y * cols;
        if (x < 0) { --y; x += cols; }
        if (x >= cols) { ++y; x -= cols; }
      } else {
        y = i / cols;
        x = i - y * cols;
      }
      ys[b] = y;
      xs[b] = x;
      vc[b] = i < N ? __ldg(row_ptr<const float4>(L.vc, ys[b]) + xs[b]) : nan4();
    }
    IcpProj q[kIcpBatch];
    float4 vl[kIcpBatch], nl[kIcpBatch], nc[kIcpBatch];
#pragma unroll
    for (int b = 0; b < kIcpBatch; ++b) {
      q[b] = icp_project(L, p, vc[b]);
      if (q[b].ok) {
        vl[b] = __ldg(row_ptr<const float4>(L.vl, q[b].v) + q[b].u);
        nl[b] = __ldg(row_ptr<const float4>(L.nl, q[b].v) + q[b].u);
        nc[b] = __ldg(row_ptr<const float4>(L.nc, ys[b]) + xs[b]);
      }
    }
#pragma unroll
    for (int b = 0; b < kIcpBatch; ++b) {
      float row[7];
      if (q[b].ok && icp_finish(p, q[b], vl[b], nl[b], nc[b], row)) icp_add_row(acc, row);
    }
  }
}

// ------------------------------------------------------ photometric term
// Pixel (x, y) of index i: i / cols through the float reciprocal (exact
// after the remainder correction for i < 2^24), as icp_accumulate does.
__device__ __forceinline__ void pixel_xy(int i, int cols, float inv_cols, bool small, int &x, int &y) {
  if (small) {
    y = (int)((float)i * inv_cols);
    x = i - y * cols;
    if (x < 0) { --y; x += cols; }
    if (x >= cols) { ++y; x -= cols; }
  } else {
    y = i / cols;
    x = i - y * cols;
  }
}

// A pixel's correspondence for the iteration: the last frame's vertex in
// the current camera (the `point` of GetRow) and the intensity difference,
// or w = kNoCorr.
constexpr int kNoCorr = (int)0x80000000;

// RGBReduction::FindCorresp (Reduction.cu:412-463) for a pixel whose
// pose-independent tests passed (its candidate flag): the current vertex
// through the current and last poses to the last frame's pixel (u, v) --
// `+ 0.5` is double and the sum reaches __float2int_rd as a float; the
// double sum is exact, so that is the float sum rounded once -- then the
// two vertices' float4 distance below 0.1 and a nonzero last intensity.
// GetRow's pose-dependent point (Reduction.cu:497) is made here from the
// vertex just gathered.
__device__ __forceinline__ float4 rgb_find(const IcpLevelArgs &L, const RgbLevelArgs &R, const PoseF &p, int x,
                                           int y) {
  const float4 none = make_float4(0.f, 0.f, 0.f, __int_as_float(kNoCorr));
  const float4 vc = __ldg(row_ptr<const float4>(L.vc, y) + x);
  if (isnan(vc.x)) return none;
  const f3 vg = mul(p.Rc, xyz(vc)) + p.tc;
  const f3 vq = mul(p.RlI, vg - p.tl);
  const int u = __float2int_rd(__fadd_rn(__fadd_rn(__fdiv_rn(__fmul_rn(L.fx, vq.x), vq.z), L.cx), 0.5f));
  const int v = __float2int_rd(__fadd_rn(__fadd_rn(__fdiv_rn(__fmul_rn(L.fy, vq.y), vq.z), L.cy), 0.5f));
  if (u < 0 || v < 0 || u >= L.vc.cols || v >= L.vc.rows) return none;
  const float4 vl = __ldg(row_ptr<const float4>(L.vl, v) + u);
  if (isnan(vl.x)) return none;
  const float d0 = vl.x - vc.x, d1 = vl.y - vc.y, d2 = vl.z - vc.z, d3 = vl.w - vc.w;
  // (double)sqrtf(n2) < 0.1 iff n2 < 0x3c23d70a (0.01f): sqrtf is
  // correctly rounded and monotone
  if (!(d0 * d0 + d1 * d1 + d2 * d2 + d3 * d3 < __int_as_float(0x3c23d70a))) return none;
  const int il = __ldg(row_ptr<const uint8_t>(R.ilast, v) + u);
  if (il == 0) return none;
  const int in = __ldg(row_ptr<const uint8_t>(R.inext, y) + x);
  const f3 point = mul(p.RcI, (mul(p.Rl, xyz(vl)) + p.tl) - p.tc);
  return make_float4(point.x, point.y, point.z, __int_as_float(in - il));
}

// RGBReduction::GetRow (Reduction.cu:483-517) from a correspondence: w =
// 1 / (sigma + |diff|) (1 when that is below 1e-3, or when sigma < 1e-6),
// the gradient / 9 (the float quotient equals the reference's double one
// for every short), and the row [w left, w (point x left), -w diff].
__device__ __forceinline__ void rgb_row(const IcpLevelArgs &L, const RgbLevelArgs &R, float sigma, bool sigma_tiny,
                                        int x, int y, float4 c, float row[7]) {
  const int diff = __float_as_int(c.w);
  float w = sigma + (float)abs(diff);
  w = w < 0.001f ? 1.0f : __fdiv_rn(1.0f, w);  // (double)w < 1e-3 iff w < 0.001f
  if (sigma_tiny) w = 1.0f;
  const f3 point = mk3(c.x, c.y, c.z);
  const float gx = __fdiv_rn((float)__ldg(row_ptr<const short>(R.dx, y) + x), 9.0f);
  const float gy = __fdiv_rn((float)__ldg(row_ptr<const short>(R.dy, y) + x), 9.0f);
  const float invz = __fdiv_rn(1.0f, point.z);
  f3 left;
  left.x = gx * L.fx * invz;
  left.y = gy * L.fy * invz;
  left.z = -(left.x * point.x + left.y * point.y) * invz;
  const f3 cr = cross(point, left);
  row[0] = w * left.x; row[1] = w * left.y; row[2] = w * left.z;
  row[3] = w * cr.x; row[4] = w * cr.y; row[5] = w * cr.z;
  row[6] = -w * (float)diff;
}

// RGBStep's sigma (Reduction.cu:619-622) from the integer sums; sigma_tiny
// is (double)sigma < 1e-6, i.e. sigma <= 1e-6f.
__device__ __forceinline__ float rgb_sigma(unsigned cnt, unsigned ssq, bool &tiny) {
  const int c = (int)cnt, q = (int)ssq;
  const float sg = __fsqrt_rn(__fdiv_rn((float)q, (float)(c == 0 ? 1 : c)));
  tiny = sg <= 1e-6f;
  return sg;
}

// ComputeResidualKernel's pass (Reduction.cu:465-481) over this thread's
// pixels i = gtid, gtid + gstride, ...: the correspondence of each goes to
// R.corr[i]; cnt / ssq gather the count and sum of diff^2 (32-bit
// wrapping sums, as the reference's int sums).
__device__ __forceinline__ void rgb_residual_pass(const IcpLevelArgs &L, const RgbLevelArgs &R, const PoseF &p,
                                                  int gtid, int gstride, unsigned &cnt, unsigned &ssq) {
  const int cols = L.vc.cols, N = cols * L.vc.rows;
  const float inv_cols = 1.0f / (float)cols;
  const bool small = N < (1 << 24) - gstride;
  for (int i = gtid; i < N; i += gstride) {
    int x, y;
    pixel_xy(i, cols, inv_cols, small, x, y);
    float4 c = make_float4(0.f, 0.f, 0.f, __int_as_float(kNoCorr));
    if (__ldg(row_ptr<const uint8_t>(R.cand, y) + x)) c = rgb_find(L, R, p, x, y);
    __stcg(R.corr + i, c);
    const int d = __float_as_int(c.w);
    if (d != kNoCorr) {
      cnt += 1u;
      ssq += (unsigned)(d * d);
    }
  }
}

// RgbStepKernel's pass (Reduction.cu:519-551): the 29 terms of this
// thread's pixels' rows.
__device__ __forceinline__ void rgb_rows_pass(const IcpLevelArgs &L, const RgbLevelArgs &R, float sigma, bool tiny,
                                              int gtid, int gstride, float acc[29]) {
#pragma unroll
  for (int k = 0; k < 29; ++k) acc[k] = 0.f;
  const int cols = L.vc.cols, N = cols * L.vc.rows;
  const float inv_cols = 1.0f / (float)cols;
  const bool small = N < (1 << 24) - gstride;
  for (int i = gtid; i < N; i += gstride) {
    const float4 c = __ldcg(R.corr + i);
    if (__float_as_int(c.w) == kNoCorr) continue;
    int x, y;
    pixel_xy(i, cols, inv_cols, small, x, y);
    float row[7];
    rgb_row(L, R, sigma, tiny, x, y, c, row);
    icp_add_row(acc, row);
  }
}

// Block totals of the correspondence count and sum of diff^2 (wrapping
// 32-bit sums) in s2[0..1], which must be zero on entry; valid after the
// __syncthreads.
__device__ __forceinline__ void block_sum2(unsigned cnt, unsigned ssq, unsigned *s2) {
  cnt = __reduce_add_sync(0xffffffffu, cnt);
  ssq = __reduce_add_sync(0xffffffffu, ssq);
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(s2, cnt);
    atomicAdd(s2 + 1, ssq);
  }
  __syncthreads();
}

// Float-float (hi + lo) accumulation: Knuth's TwoSum on the leading parts,
// the rounding errors and trailing parts carried in lo.  About 2^-47
// relative per addition, on the FP32 pipe.
struct ff {
  float s, e;
};
__device__ __forceinline__ ff ff_add(ff a, ff b) {
  const float t = a.s + b.s;
  const float bb = t - a.s;
  const float err = (a.s - (t - bb)) + (b.s - bb);
  return ff{t, a.e + b.e + err};
}
__device__ __forceinline__ ff ff_shfl_xor(ff a, int off) {
  return ff{__shfl_xor_sync(0xffffffffu, a.s, off), __shfl_xor_sync(0xffffffffu, a.e, off)};
}
// (hi, lo) with |lo| <= ulp(hi) / 2.
__device__ __forceinline__ float2 ff_norm(ff a) {
  const float hi = a.s + a.e;
  return make_float2(hi, a.e - (hi - a.s));
}

// Transposing butterfly over the 29 accumulators of a warp: at each level
// a lane keeps half of its components, adds the partner's copy of them and
// hands over the other half, so lane l ends with the compensated warp total
// of component l (components 29..31 are zero) after 31 shuffle pairs
// instead of 29 separate trees.
__device__ __forceinline__ ff warp_transpose_reduce29(const float acc[29]) {
  const int lane = threadIdx.x & 31;
  ff v16[16];
  {
    const bool hi = lane & 16;
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      const float lo_c = acc[m];
      const float hi_c = (m + 16 < 29) ? acc[m + 16] : 0.f;
      const float send = hi ? lo_c : hi_c;
      const float keep = hi ? hi_c : lo_c;
      const float recv = __shfl_xor_sync(0xffffffffu, send, 16);
      v16[m] = ff_add(ff{keep, 0.f}, ff{recv, 0.f});
    }
  }
  ff v8[8];
  {
    const bool hi = lane & 8;
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      const ff send = hi ? v16[m] : v16[m + 8];
      const ff keep = hi ? v16[m + 8] : v16[m];
      v8[m] = ff_add(keep, ff_shfl_xor(send, 8));
    }
  }
  ff v4[4];
  {
    const bool hi = lane & 4;
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const ff send = hi ? v8[m] : v8[m + 4];
      const ff keep = hi ? v8[m + 4] : v8[m];
      v4[m] = ff_add(keep, ff_shfl_xor(send, 4));
    }
  }
  ff v2[2];
  {
    const bool hi = lane & 2;
#pragma unroll
    for (int m = 0; m < 2; ++m) {
      const ff send = hi ? v4[m] : v4[m + 2];
      const ff keep = hi ? v4[m + 2] : v4[m];
      v2[m] = ff_add(keep, ff_shfl_xor(send, 2));
    }
  }
  const bool hi = lane & 1;
  const ff send = hi ? v2[0] : v2[1];
  const ff keep = hi ? v2[1] : v2[0];
  return ff_add(keep, ff_shfl_xor(send, 1));
}

// Block total of the 29 terms as normalised float-float pairs in smem
// out[29]: warp butterflies, then for each component the NW warp totals
// are added with a shuffle tree (warp w takes components w, w + NW, ...).
// wpart rows are padded to 33 so the column reads hit distinct banks.
template <int NW>
__device__ __forceinline__ void block_reduce29(const float acc[29], ff (*wpart)[33], float2 *out) {
  static_assert(NW >= 1 && NW <= 32, "1..32 warps");
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  wpart[warp][lane] = warp_transpose_reduce29(acc);
  __syncthreads();
  for (int c = warp; c < 29; c += NW) {
    ff v = (lane < NW) ? wpart[lane][c] : ff{0.f, 0.f};
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v = ff_add(v, ff_shfl_xor(v, off));
    if (lane == 0) out[c] = ff_norm(v);
  }
  __syncthreads();
}

// Sum of FP64 partials[29][nb] per component, fixed order: warp w sums
// component w; lanes stride over CTAs, then a shuffle tree.
__device__ __forceinline__ void cross_block_sum(const double *part, int nb, int stride,
                                                double *sums) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int c = warp; c < 29; c += kWarps) {
    double t = 0.0;
    for (int b = lane; b < nb; b += 32) t += __ldcg(part + (size_t)c * stride + b);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) t += __shfl_down_sync(0xffffffffu, t, off);
    if (lane == 0) sums[c] = t;
  }
  __syncthreads();
}

// Exact cross-CTA sums.  A CTA's float-float total of a component becomes
// an integer, value * 2^kFixFrac (truncated below 2^-kFixFrac), cut into
// three kLimbBits-bit limbs (the top one signed) that are added into three
// 64-bit accumulators with fire-and-forget atomics.  Limbs of up to 2^21
// addends sum without overflow and without carries between limbs, and
// integer addition is exact and independent of order, so the totals do not
// depend on which CTA arrives first and every CTA reads the same 29 values
// once the barrier opens.  A fourth slot counts addends beyond 2^64 in
// magnitude (or not finite); such a component reads as NaN.
//
// Atomics on one address serialise in L2: with all CTAs adding into one
// set of 29 x 3 words, the adds and the fence behind them took ~4 us per
// iteration on GB300.  CTA b therefore adds into group b % kFixGroups, and
// readers sum the groups (integer sums, so still exact and order-free).
// Eight groups measured as fast as sixteen (about 1 us over a bare grid
// barrier) with half the reads.
constexpr int kFixFrac = 60;
constexpr int kLimbBits = 42;
constexpr int kFixSlots = 4;  // limbs 0-2, out-of-range count
constexpr int kFixGroups = 8;
constexpr int kFixSet = kFixGroups * 29 * kFixSlots;  // words per accumulator set
constexpr unsigned long long kLimbMask = (1ull << kLimbBits) - 1ull;

__device__ __forceinline__ __int128 f32_to_fix(float f, bool &bad) {
  const unsigned b = __float_as_uint(f);
  const int ex = (b >> 23) & 0xff;
  if (ex == 0) return 0;  // zero or subnormal: below 2^-126
  const int sh = ex - 150 + kFixFrac;  // |f| = m * 2^(ex - 150)
  if (sh > 100) {  // |f| >= 2^64, infinite or NaN
    bad = true;
    return 0;
  }
  const unsigned m = (b & 0x7fffffu) | 0x800000u;
  const __int128 v = sh >= 0 ? ((__int128)m << sh) : (sh > -24 ? (__int128)(m >> -sh) : (__int128)0);
  return (b >> 31) ? -v : v;
}

__device__ __forceinline__ void red_add_u64(unsigned long long *p, unsigned long long v) {
  asm volatile("red.relaxed.gpu.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Adds a CTA's float-float total (hi, lo) into the accumulator slots d.
__device__ __forceinline__ void fix_add(unsigned long long *d, float2 v) {
  bool bad = false;
  const __int128 x = f32_to_fix(v.x, bad) + f32_to_fix(v.y, bad);
  red_add_u64(d + 0, (unsigned long long)x & kLimbMask);
  red_add_u64(d + 1, (unsigned long long)(x >> kLimbBits) & kLimbMask);
  red_add_u64(d + 2, (unsigned long long)(long long)(x >> (2 * kLimbBits)));
  if (bad) red_add_u64(d + 3, 1ull);
}

// The total of the limb sums a0..a2 (and out-of-range count bad) as a
// double (one rounding when the integer fits 64 bits, else at most two,
// relative 2^-52).
__device__ __forceinline__ double fix_total(unsigned long long a0, unsigned long long a1, unsigned long long a2,
                                            unsigned long long bad) {
  if (bad != 0ull) return __longlong_as_double(0x7ff8000000000000ll);
  const __int128 t = ((__int128)(long long)a2 << (2 * kLimbBits)) + ((__int128)a1 << kLimbBits) + (__int128)a0;
  const long long hi = (long long)(t >> 64);
  const unsigned long long lo = (unsigned long long)t;
  if (hi == ((long long)lo >> 63)) return (double)(long long)lo * 0x1p-60;
  return fma((double)hi, 0x1p4, (double)lo * 0x1p-60);
}
static_assert(kFixFrac == 60, "fix_total's scale factors");

struct PersistentArgs {
  IcpLevelArgs lv[kMaxLevels];
  RgbLevelArgs rg[kMaxLevels];  // photometric form only
  int levels;
  float thresh;
  unsigned *arrivals;        // grid barrier count, zero at launch
  unsigned long long *fix;   // [3][kFixGroups][29][kFixSlots] accumulators, zero at launch
  unsigned long long *fix_rgb;  // the same for the photometric sums, zero at launch
  unsigned *rgb_res;         // [3][kFixGroups][2] count and sum of diff^2, zero at launch
  TrackCtl *ctl;
  const double *last_pose;
  const int *skip_flag;  // nonzero: the kernel does nothing
  uint32_t *flags;
  unsigned long long *prof;  // optional per-iteration phase clocks of CTA 0
  unsigned poll_limit;       // polls before a grid barrier gives up
  unsigned extra_arrivals;   // arrivals a barrier waits for beyond the grid (0; a test sets it to make
                             // every wait run out)
  int predict;               // predict each iteration's pose and accumulate its rows during the solve
  void *pub;                 // [3] IcpPub: the solving CTA's pose and decision per accumulator set
  FramePost post;            // the frame loop's state update at the end (post.sys null: none)
};

// Phase clocks of the first pixel CTA (SM cycles), per iteration (the
// last round that accumulated its rows): 0 round start, 1 rows
// accumulated, 2 block total sent, 3 barrier passed, 4 the 29 sums and the
// solving CTA's pose in hand; 6 the global timer at 0; 7 whether the rows
// came from a prediction; 14 the rows started (after the prediction).
// Slots 8-13 take clocks of CTA 0 inside the iteration's solve.
// SM clock read that the compiler keeps in place relative to barriers and
// memory operations (clock64() alone may be moved ahead of a barrier).
__device__ __forceinline__ unsigned long long prof_clock() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%clock64;" : "=l"(t)::"memory");
  return t;
}

__device__ __forceinline__ void prof_mark(const PersistentArgs &a, int it, int k) {
  if (a.prof && blockIdx.x == 1 && threadIdx.x == 0 && it < kProfIters) {
    a.prof[it * kProfSlots + k] = prof_clock();
    if (k == 0) {
      unsigned long long ns;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(ns));
      a.prof[it * kProfSlots + 6] = ns;
    }
  }
}

// Grid barrier number k (counted from 0 in this launch): the arrival
// count only grows, so the barrier is open once it reaches nb * (k + 1).
// Thread 0 releases the CTA's accumulator adds (and the stores its threads
// made before the __syncthreads) with its arrival and acquires everyone
// else's with the poll that sees the count.  A wait that runs past
// a.poll_limit polls (2^22 unless a test lowers it) records
// SF_FLAG_BARRIER_TIMEOUT and sets *abort (shared), after which the CTA
// leaves its iterations with the tracking failed; the host reports
// SF_ERR_TIMEOUT and the context stays usable.
__device__ __forceinline__ void grid_barrier(const PersistentArgs &a, int nb, int k, int *abort) {
  __syncthreads();
  if (threadIdx.x == 0) {
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(a.arrivals) : "memory");
    const unsigned target = ((unsigned)nb + a.extra_arrivals) * (unsigned)(k + 1);
    unsigned polls = 0, seen;
    for (;;) {
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(seen) : "l"(a.arrivals) : "memory");
      if ((int)(seen - target) >= 0) break;
      if (++polls > a.poll_limit) {
        atomicOr(a.flags, SF_FLAG_BARRIER_TIMEOUT);
        *abort = 1;
        break;
      }
      __nanosleep(32);
    }
  }
  __syncthreads();
}

// The 29 totals of accumulator set fx (kFixGroups groups) into out
// (threads 0..28); with sync_after the block then synchronises (else the
// caller does before reading out or reusing sfix).
__device__ __forceinline__ void read_fix_set(const unsigned long long *fx,
                                             unsigned long long (*sfix)[kFixSlots], double *out,
                                             bool sync_after) {
  for (int k = threadIdx.x; k < kFixGroups * 29; k += blockDim.x) {
    const ulonglong2 *d = reinterpret_cast<const ulonglong2 *>(fx + (size_t)k * kFixSlots);
    const ulonglong2 x = __ldcg(d), y = __ldcg(d + 1);
    sfix[k][0] = x.x; sfix[k][1] = x.y; sfix[k][2] = y.x; sfix[k][3] = y.y;
  }
  __syncthreads();
  if (threadIdx.x < 29) {
    unsigned long long t[kFixSlots] = {0ull, 0ull, 0ull, 0ull};
#pragma unroll
    for (int g = 0; g < kFixGroups; ++g)
#pragma unroll
      for (int q = 0; q < kFixSlots; ++q) t[q] += sfix[g * 29 + threadIdx.x][q];
    out[threadIdx.x] = fix_total(t[0], t[1], t[2], t[3]);
  }
  if (sync_after) __syncthreads();
}

// What the solving CTA publishes per accumulator set: the FP64 pose after
// its solve (rows 0..2) and whether the iterations stop there.
struct IcpPub {
  double pose[12];
  int stop;
  int pad[7];
};
static_assert(sizeof(IcpPub) == 128, "one publication per 128 B");

// The iteration after (l, j): its level in *nl and index in *nj (levels
// without iterations skipped); false after the last one.
__device__ __forceinline__ bool next_iteration(const PersistentArgs &a, int l, int j, int *nl, int *nj) {
  if (j + 1 < a.lv[l].iters) {
    *nl = l;
    *nj = j + 1;
    return true;
  }
  for (int m = l - 1; m >= 0; --m)
    if (a.lv[m].iters > 0) {
      *nl = m;
      *nj = 0;
      return true;
    }
  return false;
}

// Every level and iteration of ComputeSE3 in one cooperative launch.
//
// CTA 0 solves; CTAs 1.. take the pixels.  Each iteration's rows need the
// pose the previous iteration's FP64 solve gives, so rather than wait for
// it, the pixel CTAs predict that pose (its float form, from the same 29
// sums and the previous FP64 pose, with FP32 / float-float arithmetic in
// one warp: sf_icp_spec.cuh) and accumulate the iteration's rows on the
// prediction while CTA 0 runs the FP64 solve.  CTA 0 publishes the FP64
// pose (and the stop decision) before it arrives at the round's grid
// barrier; after the barrier every CTA compares the float form of the
// published pose with its prediction, bit for bit.  When they agree the
// round's sums are the iteration's sums; when they do not (or no
// prediction was made) the next round accumulates the rows again on the
// published pose.  So sums, poses and decisions are those of the FP64
// path whatever the prediction does.  Rounds rotate over three
// accumulator sets; a round's barrier index is its number (twice its
// number, and once more after the correspondence pass, with the
// photometric term).
//
// RGB: each iteration also runs RGBStep (Tracking.cc:400-431): the
// correspondence pass beside the ICP rows, a grid barrier for its count
// and sum of diff^2 (sigma), the photometric rows, a second barrier, and
// the solve of the combined system.
template <bool RGB>
__global__ void __launch_bounds__(kPThreads, 1) k_icp_persistent(PersistentArgs a) {
  __shared__ TrackCtl ctl;
  __shared__ IcpSolveSmem ssolve;
  __shared__ PoseF pose;          // the float pose of this round's rows
  __shared__ spec::f2f nff[12];   // the last solved FP64 pose (rows 0..2) as float-float
  __shared__ float spred[12];     // this round's prediction (row-major 3 x 4)
  __shared__ int made;            // a prediction was made this round
  __shared__ int pub_stop, hit;
  __shared__ float2 bsum[29];
  __shared__ double sums[29];
  __shared__ double rsums[RGB ? 29 : 1];
  __shared__ unsigned s2[2];
  __shared__ ff wpart[kPWarps][33];
  __shared__ unsigned long long sfix[kFixGroups * 29][kFixSlots];
  __shared__ int abort_wait;  // a grid barrier gave up
  if (a.skip_flag && *a.skip_flag != 0) {  // uniform across the grid
    if (a.post.sys && blockIdx.x == 0 && threadIdx.x == 0) sys_post(a.post.sys, *a.ctl, a.post.tmpl, a.post.f);
    return;
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool solver = blockIdx.x == 0;
  if (threadIdx.x == 0) {
    ctl_begin(ctl, a.last_pose);
    s_solve_marks = nullptr;
    abort_wait = 0;
    made = 0;
  }
  __syncthreads();
  if (warp == 0) {
    pose_to_float_warp(ctl.next_pose, ctl.last_pose, pose);
    if (lane < 12) nff[lane] = spec::split(ctl.next_pose[lane]);
  }
  __syncthreads();
  const int nb = gridDim.x;
  // Warp w of pixel CTA b takes the 32-pixel runs w * (nb - 1) + b - 1 (+
  // multiples of the pixel CTAs' threads): every CTA's work is spread over
  // the whole image, which evens out the CTAs' arrival at the barrier;
  // each warp's loads stay coalesced.
  const int gtid = (warp * (nb - 1) + (int)blockIdx.x - 1) * 32 + lane;
  const int gstride = (nb - 1) * kPThreads;
  IcpPub *const pubs = reinterpret_cast<IcpPub *>(a.pub);
  int l = a.levels - 1;  // level of iteration it (-1: none left)
  while (l >= 0 && a.lv[l].iters == 0) --l;
  int j = 0, it = 0, round = 0, set = 0;  // set = round % 3
  int sl = 0;             // level of the iteration whose sums are in `sums`
  bool predict = false;   // this round's rows go on a prediction (the sums of iteration it - 1 are in hand)
  for (;;) {
    const bool have = l >= 0;
    if (have) prof_mark(a, it, 0);
    if (predict) {
      if (solver) {
        // the FP64 solve of iteration it - 1, and the same prediction as the
        // pixel CTAs make (to check it after the barrier)
        if (warp < 3) {
          if (threadIdx.x == 0)
            s_solve_marks = (a.prof && it - 1 < kProfIters) ? a.prof + (it - 1) * kProfSlots + 8 : nullptr;
          __syncwarp();
          ctl_step_fast(ctl, sums, a.lv[sl].min_count, ssolve, RGB ? rsums : nullptr);
        } else if (warp == 3) {
          const bool m = a.predict && have && spec::predict_pose_warp(sums, nff, spred);
          if (lane == 0) made = m;
        }
        __syncthreads();
        if (!have) break;  // the last iteration's solve: done
        if (threadIdx.x < 12) __stcg(&pubs[set].pose[threadIdx.x], ctl.next_pose[threadIdx.x]);
        if (threadIdx.x == 0) __stcg(&pubs[set].stop, ctl.stop);
      } else {
        if (!have) break;  // the solving CTA finishes alone
        if (warp == 0) {
          const bool m = a.predict && spec::predict_pose_warp(sums, nff, spred);
          if (m && lane < 12) {  // the last pose's parts of pose stay as they are
            const int i = lane >> 2, c = lane & 3;
            if (c < 3) {
              (&pose.Rc.rx.x)[i * 3 + c] = spred[lane];
              (&pose.RcI.rx.x)[c * 3 + i] = spred[lane];
            } else {
              (&pose.tc.x)[i] = spred[lane];
            }
          }
          if (lane == 0) made = m;
        }
        __syncthreads();
      }
    }
    const bool rows = !solver && (!predict || made);
    if (a.prof && blockIdx.x == 1 && threadIdx.x == 0 && it < kProfIters) a.prof[it * kProfSlots + 14] = prof_clock();
    float acc[29];
    unsigned cnt = 0u, ssq = 0u;
    if (rows) {
      icp_accumulate(a.lv[l], pose, gtid, gstride, acc);
      if (RGB) rgb_residual_pass(a.lv[l], a.rg[l], pose, gtid, gstride, cnt, ssq);
    } else {
#pragma unroll
      for (int k = 0; k < 29; ++k) acc[k] = 0.f;
    }
    if (RGB && threadIdx.x < 2) s2[threadIdx.x] = 0u;
    prof_mark(a, it, 1);
    const int group = blockIdx.x % kFixGroups;
    unsigned long long *fx = a.fix + (size_t)set * kFixSet;
    unsigned *rres = a.rgb_res + (size_t)set * kFixGroups * 2;
    if (!solver) {  // uniform over the CTA (the solving CTA adds nothing)
      block_reduce29<kPWarps>(acc, wpart, bsum);
      if (rows && threadIdx.x < 29) fix_add(fx + (group * 29 + threadIdx.x) * kFixSlots, bsum[threadIdx.x]);
      if (RGB) {
        block_sum2(cnt, ssq, s2);
        if (rows && threadIdx.x < 2) atomicAdd(rres + group * 2 + threadIdx.x, s2[threadIdx.x]);
      }
    }
    prof_mark(a, it, 2);
    grid_barrier(a, nb, RGB ? 2 * round : round, &abort_wait);
    if (abort_wait) break;  // uniform: read after the barrier's __syncthreads
    prof_mark(a, it, 3);
    unsigned long long *fxr = a.fix_rgb + (size_t)set * kFixSet;
    if (RGB) {
      // sigma from the grid's count and sum of diff^2, then the rows
      if (threadIdx.x < 32) {
        const unsigned v = lane < kFixGroups * 2 ? __ldcg(rres + lane) : 0u;
        const unsigned c2 = __reduce_add_sync(0xffffffffu, (lane & 1) ? 0u : v);
        const unsigned q2 = __reduce_add_sync(0xffffffffu, (lane & 1) ? v : 0u);
        if (lane == 0) { s2[0] = c2; s2[1] = q2; }
      }
      __syncthreads();
      bool tiny;
      const float sigma = rgb_sigma(s2[0], s2[1], tiny);
      if (!solver) {
        if (rows) {
          rgb_rows_pass(a.lv[l], a.rg[l], sigma, tiny, gtid, gstride, acc);
        } else {
#pragma unroll
          for (int k = 0; k < 29; ++k) acc[k] = 0.f;
        }
        block_reduce29<kPWarps>(acc, wpart, bsum);
        if (rows && threadIdx.x < 29) fix_add(fxr + (group * 29 + threadIdx.x) * kFixSlots, bsum[threadIdx.x]);
      }
      grid_barrier(a, nb, 2 * round + 1, &abort_wait);
      if (abort_wait) break;
    }
    // the solving CTA's pose, loaded beside the accumulator sets
    double P = 0.0;
    int P_stop = 0;
    if (predict && warp == 0) {
      if (lane < 12) P = __ldcg(&pubs[set].pose[lane]);
      if (lane == 0) P_stop = __ldcg(&pubs[set].stop);
    }
    read_fix_set(fx, sfix, sums, RGB);
    if (RGB) {
      read_fix_set(fxr, sfix, rsums, true);
      // A = A_rgb w + A_icp, b = b_rgb w + b_icp (Tracking.cc:484-487)
      if (threadIdx.x < 27) sums[threadIdx.x] = __dadd_rn(__dmul_rn(rsums[threadIdx.x], (double)1e-4f), sums[threadIdx.x]);
    }
    // Every CTA read the previous round's sets before it arrived here, so
    // CTA 0 clears them for round + 2; its clearing is released with its
    // next arrival, before anyone can add into them.
    const int prev = set == 0 ? 2 : set - 1;
    if (solver) {
      for (int k = threadIdx.x; k < kFixSet; k += blockDim.x) __stcg(a.fix + (size_t)prev * kFixSet + k, 0ull);
      if (RGB) {
        for (int k = threadIdx.x; k < kFixSet; k += blockDim.x) __stcg(a.fix_rgb + (size_t)prev * kFixSet + k, 0ull);
        if (threadIdx.x < kFixGroups * 2) __stcg(a.rgb_res + (size_t)prev * kFixGroups * 2 + threadIdx.x, 0u);
      }
    }
    if (predict && warp == 0) {
      // the published FP64 pose: its float form against the prediction
      const float f = (float)P;
      const bool same = lane >= 12 || __float_as_uint(f) == __float_as_uint(spred[lane]);
      const bool agree = __all_sync(0xffffffffu, same);
      if (lane < 12) {
        nff[lane] = spec::split(P);
        if (!(made && agree)) {  // the next round accumulates on this pose
          const int i = lane >> 2, c = lane & 3;
          if (c < 3) {
            (&pose.Rc.rx.x)[i * 3 + c] = f;
            (&pose.RcI.rx.x)[c * 3 + i] = f;
          } else {
            (&pose.tc.x)[i] = f;
          }
        }
      }
      if (lane == 0) {
        pub_stop = P_stop;
        hit = made && agree;
      }
    }
    __syncthreads();
    prof_mark(a, it, 4);
    set = set == 2 ? 0 : set + 1;
    ++round;
    if (predict) {
      if (pub_stop) break;  // the solve of iteration it - 1 ended the iterations
      if (!hit) {           // the rows again, on the FP64 pose
        if (a.prof && blockIdx.x == 1 && threadIdx.x == 0 && it < kProfIters) a.prof[it * kProfSlots + 7] = 0;
        predict = false;
        continue;
      }
    }
    if (a.prof && blockIdx.x == 1 && threadIdx.x == 0 && it < kProfIters) a.prof[it * kProfSlots + 7] = predict;
    // the sums of iteration it are in hand
    predict = true;
    sl = l;
    int nl = 0, nj = 0;
    if (next_iteration(a, l, j, &nl, &nj)) {
      l = nl;
      j = nj;
    } else {
      l = -1;
    }
    ++it;
  }
  if (!solver) return;
  if (threadIdx.x == 0) {
    s_solve_marks = nullptr;
    if (abort_wait) {  // a barrier gave up: the tracking failed
      ctl.stop = 1;
      ctl.timeout = 1;
    }
  }
  __syncthreads();
  __syncwarp();
  if (threadIdx.x < 32) ctl_finish_fast(ctl, a.thresh, ssolve);
  __syncthreads();
  if (threadIdx.x == 0) {
    *a.ctl = ctl;
    if (a.post.sys) sys_post(a.post.sys, ctl, a.post.tmpl, a.post.f);
  }
}

// Plain form, launch 1: per-CTA FP64 partials.
__global__ void __launch_bounds__(kThreads) k_icp_partials(IcpLevelArgs L, PoseF p, double *part,
                                                           int stride) {
  __shared__ float2 bsum[29];
  __shared__ ff wpart[kWarps][33];
  float acc[29];
  icp_accumulate(L, p, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x, acc);
  block_reduce29<kWarps>(acc, wpart, bsum);
  if (threadIdx.x < 29)
    part[(size_t)threadIdx.x * stride + blockIdx.x] = (double)bsum[threadIdx.x].x + (double)bsum[threadIdx.x].y;
}

// Plain form, launch 2: FP64 sum of the partials (Reduce<float,29>).
__global__ void __launch_bounds__(kThreads) k_icp_reduce(const double *part, int nb, int stride,
                                                         double *out) {
  __shared__ double sums[29];
  cross_block_sum(part, nb, stride, sums);
  if (threadIdx.x < 29) out[threadIdx.x] = sums[threadIdx.x];
}

// Plain form of RGBStep, launch 1: correspondences, their count and sum of
// diff^2 added into res[0..1] (zero on entry).
__global__ void __launch_bounds__(kThreads) k_rgb_residual(IcpLevelArgs L, RgbLevelArgs R, PoseF p,
                                                           unsigned *res) {
  __shared__ unsigned s2[2];
  if (threadIdx.x < 2) s2[threadIdx.x] = 0u;
  __syncthreads();
  unsigned cnt = 0u, ssq = 0u;
  rgb_residual_pass(L, R, p, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x, cnt, ssq);
  block_sum2(cnt, ssq, s2);
  if (threadIdx.x < 2) atomicAdd(res + threadIdx.x, s2[threadIdx.x]);
}

// Plain form of RGBStep, launch 2: per-CTA FP64 partials of the rows'
// 29 terms, sigma from res.
__global__ void __launch_bounds__(kThreads) k_rgb_partials(IcpLevelArgs L, RgbLevelArgs R, PoseF p,
                                                           const unsigned *res, double *part, int stride) {
  __shared__ float2 bsum[29];
  __shared__ ff wpart[kWarps][33];
  bool tiny;
  const float sigma = rgb_sigma(__ldcg(res), __ldcg(res + 1), tiny);
  float acc[29];
  rgb_rows_pass(L, R, sigma, tiny, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x, acc);
  block_reduce29<kWarps>(acc, wpart, bsum);
  if (threadIdx.x < 29)
    part[(size_t)threadIdx.x * stride + blockIdx.x] = (double)bsum[threadIdx.x].x + (double)bsum[threadIdx.x].y;
}

// FindCorresp's pose-independent tests from an image and its derivatives
// (the flag launch_derivatives makes beside them).
__global__ void k_rgb_cand(sf_image img, sf_image dx, sf_image dy, sf_image cand) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= img.cols || y >= img.rows) return;
  bool ok = x >= 5 && x < img.cols - 5 && y >= 5 && y < img.rows - 5 &&
            (row_ptr<const short>(dx, y)[x] != 0 || row_ptr<const short>(dy, y)[x] != 0);
  if (ok)
    for (int u = y - 2; u < y + 2; ++u)
      for (int v = x - 2; v < x + 2; ++v) ok = ok && row_ptr<const uint8_t>(img, u)[v] > 0;
  row_ptr<uint8_t>(cand, y)[x] = ok ? 1 : 0;
}

// ------------------------------------- ValidatePose batch: ComputeSE3 part
// ComputeSE3(icpOnly = true, ITERATIONS_RELOC, THRESH_ICP_RELOC) of n
// candidates side by side (Tracker::ValidatePose, Tracking.cc:763-765).
// Each iteration is two launches: every candidate still running gets nb
// CTAs over the level's pixels (one FP64 partial per CTA and sum), then one
// 96-thread CTA that sums its partials in a fixed order and runs the
// persistent kernel's solve and stop logic (ctl_step_fast) on them.  The
// candidate's state stays in ctl[c] between launches.
struct VpArgs {
  IcpLevelArgs L;  // vc, nc: the frame; vl, nl: tall model maps (or the fallback)
  sf_image fv, fn;
  int rows;
  const int *src;
  const TrackCtl *ctl;
  double *part;
  int stride;
};

__global__ void __launch_bounds__(kThreads) k_vp_partials(VpArgs a) {
  const int c = blockIdx.y;
  const int src = a.src[c];
  if (src == -2 || a.ctl[c].stop) return;  // uniform over the CTA
  __shared__ PoseF pose;
  __shared__ float2 bsum[29];
  __shared__ ff wpart[kWarps][33];
  if (threadIdx.x < 32) pose_to_float_warp(a.ctl[c].next_pose, a.ctl[c].last_pose, pose);
  __syncthreads();
  IcpLevelArgs L = a.L;
  if (src >= 0) {
    L.vl.data = (char *)a.L.vl.data + (size_t)src * a.rows * a.L.vl.step;
    L.nl.data = (char *)a.L.nl.data + (size_t)src * a.rows * a.L.nl.step;
  } else {
    L.vl = a.fv;
    L.nl = a.fn;
  }
  L.vl.rows = L.nl.rows = a.rows;
  float acc[29];
  icp_accumulate(L, pose, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x, acc);
  block_reduce29<kWarps>(acc, wpart, bsum);
  if (threadIdx.x < 29)
    a.part[((size_t)c * 29 + threadIdx.x) * a.stride + blockIdx.x] =
        (double)bsum[threadIdx.x].x + (double)bsum[threadIdx.x].y;
}

__global__ void __launch_bounds__(96) k_vp_step(const double *part, int nb, int stride, const int *src,
                                                TrackCtl *ctl_g, int min_count) {
  const int c = blockIdx.x;
  if (src[c] == -2) return;
  __shared__ TrackCtl ctl;
  __shared__ IcpSolveSmem ssolve;
  __shared__ double sums[29];
  if (threadIdx.x == 0) {
    ctl = ctl_g[c];
    s_solve_marks = nullptr;
  }
  __syncthreads();
  if (ctl.stop) return;  // uniform
  if (threadIdx.x < 29) {
    // four interleaved chains, joined in a fixed order
    const double *p = part + ((size_t)c * 29 + threadIdx.x) * stride;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    int b = 0;
    for (; b + 4 <= nb; b += 4) {
      a0 += __ldcg(p + b);
      a1 += __ldcg(p + b + 1);
      a2 += __ldcg(p + b + 2);
      a3 += __ldcg(p + b + 3);
    }
    for (; b < nb; ++b) a0 += __ldcg(p + b);
    sums[threadIdx.x] = (a0 + a1) + (a2 + a3);
  }
  __syncthreads();
  ctl_step_fast(ctl, sums, min_count, ssolve, nullptr);
  __syncthreads();
  if (threadIdx.x == 0) ctl_g[c] = ctl;
}

__global__ void __launch_bounds__(32) k_vp_finish(TrackCtl *ctl_g, const int *src, float thresh) {
  const int c = blockIdx.x;
  if (src[c] == -2) return;
  __shared__ TrackCtl ctl;
  __shared__ IcpSolveSmem ssolve;
  if (threadIdx.x == 0) ctl = ctl_g[c];
  __syncwarp();
  ctl_finish_fast(ctl, thresh, ssolve);
  __syncwarp();
  if (threadIdx.x == 0) ctl_g[c] = ctl;
}

}  // namespace

// arrival count (256 B), ICP accumulator sets, photometric accumulator
// sets, photometric count / sum of diff^2 sets
constexpr size_t kFixBytes = sizeof(unsigned long long) * 3 * kFixSet;
constexpr size_t kResBytes = sizeof(unsigned) * 3 * kFixGroups * 2;
constexpr size_t kPubBytes = 3 * 128;  // IcpPub per accumulator set
constexpr size_t kBarrierBytes = 256 + 2 * kFixBytes + kResBytes + kPubBytes;

cudaError_t icp_persistent_reset(const IcpWorkspace &w, cudaStream_t s) {
  return cudaMemsetAsync(w.barrier, 0, kBarrierBytes, s);
}

int icp_workspace_init(IcpWorkspace &w) {
  int dev = 0, sms = 0, per_sm = 0, coop = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return SF_ERR_CUDA;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  int per_sm_rgb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_icp_persistent<false>, kPThreads, 0) !=
          cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_rgb, k_icp_persistent<true>, kPThreads, 0) !=
          cudaSuccess)
    return SF_ERR_CUDA;
  if (per_sm < 1 || per_sm_rgb < 1 || !coop) return SF_ERR_CUDA;
  w.max_blocks = sms * per_sm;
  w.max_blocks_rgb = sms * per_sm_rgb;
  w.threads = kPThreads;
  if (cudaMalloc(&w.partials, sizeof(double) * 2 * 29 * (size_t)w.max_blocks) != cudaSuccess) return SF_ERR_CUDA;
  if (cudaMalloc(&w.sums, sizeof(double) * 2 * 29) != cudaSuccess) return SF_ERR_CUDA;
  if (cudaMalloc(&w.barrier, kBarrierBytes) != cudaSuccess) return SF_ERR_CUDA;
  if (cudaMemset(w.barrier, 0, kBarrierBytes) != cudaSuccess) return SF_ERR_CUDA;
  char *base = reinterpret_cast<char *>(w.barrier);
  w.fix = reinterpret_cast<unsigned long long *>(base + 256);
  w.fix_rgb = reinterpret_cast<unsigned long long *>(base + 256 + kFixBytes);
  w.rgb_res = reinterpret_cast<unsigned *>(base + 256 + 2 * kFixBytes);
  w.pub = base + 256 + 2 * kFixBytes + kResBytes;
  if (cudaMalloc(&w.ctl, sizeof(TrackCtl)) != cudaSuccess) return SF_ERR_CUDA;
  if (cudaMalloc(&w.prof, sizeof(unsigned long long) * kProfSlots * kProfIters) != cudaSuccess) return SF_ERR_CUDA;
  if (cudaMemset(w.prof, 0, sizeof(unsigned long long) * kProfSlots * kProfIters) != cudaSuccess) return SF_ERR_CUDA;
  return SF_OK;
}

void icp_workspace_free(IcpWorkspace &w) {
  cudaFree(w.partials);
  cudaFree(w.sums);
  cudaFree(w.barrier);
  cudaFree(w.ctl);
  cudaFree(w.prof);
  cudaFree(w.corr);
  cudaFree(w.cand);
  w = IcpWorkspace();
}

int icp_workspace_rgb(IcpWorkspace &w, size_t pixels) {
  if (pixels <= w.rgb_pixels) return SF_OK;
  cudaFree(w.corr);
  cudaFree(w.cand);
  w.corr = nullptr;
  w.cand = nullptr;
  w.rgb_pixels = 0;
  // candidate flags of every level: at most 4/3 of level 0, padded
  if (cudaMalloc(&w.corr, sizeof(float4) * pixels) != cudaSuccess) return SF_ERR_CUDA;
  if (cudaMalloc(&w.cand, pixels * 2) != cudaSuccess) return SF_ERR_CUDA;
  w.rgb_pixels = pixels;
  return SF_OK;
}

void launch_rgb_step(const IcpWorkspace &w, const IcpLevelArgs &L, const RgbLevelArgs &R, const m3 &Rc,
                     const m3 &RcInv, f3 tc, const m3 &Rl, const m3 &RlInv, f3 tl, cudaStream_t s) {
  PoseF p;
  p.Rc = Rc; p.RcI = RcInv; p.tc = tc; p.Rl = Rl; p.RlI = RlInv; p.tl = tl;
  const int nb = w.max_blocks;
  cudaMemsetAsync(w.rgb_res, 0, 2 * sizeof(unsigned), s);
  k_rgb_residual<<<nb, kThreads, 0, s>>>(L, R, p, w.rgb_res); note_launch();
  k_rgb_partials<<<nb, kThreads, 0, s>>>(L, R, p, w.rgb_res, w.partials, w.max_blocks); note_launch();
  k_icp_reduce<<<1, kThreads, 0, s>>>(w.partials, nb, w.max_blocks, w.sums + 29); note_launch();
}

void launch_rgb_cand(const sf_image &inext, const sf_image &dx, const sf_image &dy, const sf_image &cand,
                     cudaStream_t s) {
  const dim3 blk(32, 8);
  const dim3 grd((inext.cols + 31) / 32, (inext.rows + 7) / 8);
  k_rgb_cand<<<grd, blk, 0, s>>>(inext, dx, dy, cand); note_launch();
}

int vp_icp_blocks(int pixels) {
  const int per = kThreads * 4;
  return (pixels + per - 1) / per;
}

void launch_vp_icp_iteration(const VpLevel &V, const int *src, TrackCtl *ctl, double *part, int nb, int stride,
                             int n, cudaStream_t s) {
  VpArgs a;
  a.L.vc = V.vc; a.L.nc = V.nc; a.L.vl = V.mv; a.L.nl = V.mn;
  a.L.fx = V.fx; a.L.fy = V.fy; a.L.cx = V.cx; a.L.cy = V.cy;
  a.L.iters = 1; a.L.min_count = V.min_count;
  a.fv = V.fv; a.fn = V.fn;
  a.rows = V.rows;
  a.src = src;
  a.ctl = ctl;
  a.part = part;
  a.stride = stride;
  k_vp_partials<<<dim3(nb, n), kThreads, 0, s>>>(a); note_launch();
  k_vp_step<<<n, 96, 0, s>>>(part, nb, stride, src, ctl, V.min_count); note_launch();
}

void launch_vp_icp_finish(TrackCtl *ctl, const int *src, float thresh, int n, cudaStream_t s) {
  k_vp_finish<<<n, 32, 0, s>>>(ctl, src, thresh); note_launch();
}

void launch_icp_step(const IcpWorkspace &w, const IcpLevelArgs &L, const m3 &Rc, f3 tc,
                     const m3 &Rl, const m3 &RlInv, f3 tl, cudaStream_t s) {
  PoseF p;
  p.Rc = Rc; p.tc = tc; p.Rl = Rl; p.RlI = RlInv; p.tl = tl;
  const int nb = w.max_blocks;
  k_icp_partials<<<nb, kThreads, 0, s>>>(L, p, w.partials, w.max_blocks); note_launch();
  k_icp_reduce<<<1, kThreads, 0, s>>>(w.partials, nb, w.max_blocks, w.sums); note_launch();
}

cudaError_t launch_icp_persistent(const IcpWorkspace &w, const IcpLevelArgs *levels, int nlevels,
                                  float thresh, const double *last_pose, const int *skip_flag,
                                  uint32_t *flags, cudaStream_t s, const RgbLevelArgs *rgb,
                                  const FramePost *post) {
  PersistentArgs a = {};
  if (post) a.post = *post;
  for (int l = 0; l < nlevels && l < kMaxLevels; ++l) {
    a.lv[l] = levels[l];
    if (rgb) a.rg[l] = rgb[l];
  }
  a.levels = nlevels;
  a.thresh = thresh;
  a.arrivals = w.barrier;
  a.fix = w.fix;
  a.fix_rgb = w.fix_rgb;
  a.rgb_res = w.rgb_res;
  a.ctl = w.ctl;
  a.last_pose = last_pose;
  a.skip_flag = skip_flag;
  a.flags = flags;
  a.prof = w.profile ? w.prof : nullptr;
  a.poll_limit = w.barrier_poll_limit;
  a.extra_arrivals = w.barrier_extra;
  a.predict = w.predict;
  a.pub = w.pub;
  if ((rgb ? w.max_blocks_rgb : w.max_blocks) < 2) return cudaErrorInvalidConfiguration;  // a solving CTA and pixel CTAs
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(rgb ? w.max_blocks_rgb : w.max_blocks);
  cfg.blockDim = dim3(kPThreads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  note_launch();
  return rgb ? cudaLaunchKernelEx(&cfg, k_icp_persistent<true>, a)
             : cudaLaunchKernelEx(&cfg, k_icp_persistent<false>, a);
}

}  // namespace sf

// ------------------------------------------------- ICP step, no allocation
// sf_ICPStep for callers that cannot allocate device memory (a host whose
// own allocator owns the device, or a loop that must not pay for
// cudaMalloc's implicit device synchronisation).  Its scratch is a fixed
// array in this library's device image instead of a context workspace:
// one CTA per kStaticPixPerCta pixels, each writing one FP64 partial per
// sum, then the 29 sums.  Every partial a call reads is written by the
// same call first, so nothing needs clearing between calls.  Calls that
// overlap on the GPU share the array and race.
namespace sf {
namespace {

constexpr int kStaticPixPerCta = kThreads * 4;
constexpr int kStaticMaxCtas = SF_ICP_STATIC_MAX_PIXELS / kStaticPixPerCta;
static_assert(kStaticMaxCtas * kStaticPixPerCta == SF_ICP_STATIC_MAX_PIXELS, "whole CTAs");
constexpr int kStaticSumsOffset = 29 * kStaticMaxCtas;

// [29][kStaticMaxCtas] partials, then 29 sums (padded): 464.25 KiB.
static __device__ __align__(256) double g_icp_static[kStaticSumsOffset + 32];

constexpr int kStaticMaxDevices = 64;
std::mutex g_icp_static_mu;
double *g_icp_static_addr[kStaticMaxDevices] = {};

// Device address of g_icp_static on the current device, looked up on the
// first call per device.  The name g_icp_static in host code is only a
// host-side stand-in, never a device pointer.
int icp_static_scratch(double **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return SF_ERR_NO_DEVICE;
  if (dev < 0 || dev >= kStaticMaxDevices) return SF_ERR_INVALID;
  std::lock_guard<std::mutex> lock(g_icp_static_mu);
  if (!g_icp_static_addr[dev]) {
    double *p = nullptr;
    if (cudaGetSymbolAddress((void **)&p, g_icp_static) != cudaSuccess || !p) {
      cudaGetLastError();  // leave no error of this lookup pending for the caller's next CUDA call
      return SF_ERR_CUDA;
    }
    g_icp_static_addr[dev] = p;
  }
  *out = g_icp_static_addr[dev];
  return SF_OK;
}

bool static_img_ok(const sf_image &im, const sf_image &like) {
  return im.data && im.cols > 0 && im.rows > 0 && im.step >= (size_t)im.cols * 16 &&
         im.cols == like.cols && im.rows == like.rows;
}

}  // namespace
}  // namespace sf

extern "C" int sf_ICPStep_static(void *stream, sf_image next_vmap, sf_image last_vmap,
                                 sf_image next_nmap, sf_image last_nmap, sf_mat3 Rcurr,
                                 sf_float3 tcurr, sf_mat3 Rlast, sf_mat3 RlastInv,
                                 sf_float3 tlast, sf_intrinsics K, float residual[2],
                                 double matrixA[36], double vectorB[6]) {
  using namespace sf;
  if (!residual || !matrixA || !vectorB) return SF_ERR_INVALID;
  const sf_image *ims[4] = {&next_vmap, &last_vmap, &next_nmap, &last_nmap};
  for (auto im : ims)
    if (!static_img_ok(*im, next_vmap)) return SF_ERR_INVALID;
  const long long pixels = (long long)next_vmap.cols * next_vmap.rows;
  if (pixels > SF_ICP_STATIC_MAX_PIXELS) return SF_ERR_TOO_LARGE;
  double *scratch = nullptr;
  int st = icp_static_scratch(&scratch);
  if (st != SF_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  IcpLevelArgs L;
  L.vc = next_vmap; L.nc = next_nmap; L.vl = last_vmap; L.nl = last_nmap;
  L.fx = K.fx; L.fy = K.fy; L.cx = K.cx; L.cy = K.cy;
  L.iters = 1; L.min_count = 0;
  PoseF p;
  p.Rc = to_m3(Rcurr); p.tc = to_f3(tcurr);
  p.Rl = to_m3(Rlast); p.RlI = to_m3(RlastInv); p.tl = to_f3(tlast);
  const int nb = (int)((pixels + kStaticPixPerCta - 1) / kStaticPixPerCta);
  double *sums_dev = scratch + kStaticSumsOffset;
  // Each launch's own status: cudaLaunchKernelEx returns it directly, so an
  // unrelated error the caller's earlier work left pending is neither
  // reported nor cleared here.  A failed launch's error is cleared before
  // returning, so it does not leak into the caller's next CUDA call.
  cudaLaunchConfig_t lc = {};
  lc.blockDim = dim3(kThreads);
  lc.stream = s;
  lc.gridDim = dim3(nb);
  if (cudaLaunchKernelEx(&lc, k_icp_partials, L, p, scratch, kStaticMaxCtas) != cudaSuccess) {
    cudaGetLastError();
    return SF_ERR_CUDA;
  }
  note_launch();
  lc.gridDim = dim3(1);
  if (cudaLaunchKernelEx(&lc, k_icp_reduce, (const double *)scratch, nb, kStaticMaxCtas, sums_dev) !=
      cudaSuccess) {
    cudaGetLastError();
    return SF_ERR_CUDA;
  }
  note_launch();
  double sums[29];
  if (cudaMemcpyAsync(sums, sums_dev, sizeof(sums), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return SF_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return SF_ERR_CUDA;
  create_matrix(sums, matrixA, vectorB);
  residual[0] = (float)sums[27];
  residual[1] = (float)sums[28];
  return SF_OK;
}
