// ORACLE — test infrastructure only.  Only tests/, __graft_entry__.smoke() and
// bench.py's CPU-baseline leg may load this library, and only as the checker
// (or the timed CPU baseline); the product (semantic_icpslam_gb300/) never
// links, loads or calls it.
//
// CPU restatement of the dense per-frame loop of YuhangMing/semantic_icpSLAM
// (pyramid -> projective point-to-plane ICP -> voxel-hash allocation ->
// visible-block compaction -> TSDF/weight/colour/label integration ->
// block-skipping raycast).  Each function cites the reference file:line it
// restates.  Build: g++ -O2 -ffp-contract=off (no FMA contraction), so every
// float operation is one IEEE-754 rounding, as the reference's source states
// it; values the reference promotes to double are computed in double.
//
// Parity pin: tests/golden/ holds outputs of the reference's own device code
// (compiled for the CPU from the reference sources by oracle/ref_shim/) and
// tests/test_oracle_golden.py checks this restatement against them.
#include "sfo.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <memory>
#include <mutex>
#include <vector>

namespace {

// ------------------------------------------------------------------ helpers
struct f3 { float x, y, z; };
struct f4 { float x, y, z, w; };
struct i3 { int x, y, z; };
struct m3 { f3 rx, ry, rz; };  // Matrix3f rows (Utility/VectorMath.h:360-375)

const float kNaN = [] { uint32_t u = 0x7fffffffu; float f; memcpy(&f, &u, 4); return f; }();

inline f3 mk3(float x, float y, float z) { return {x, y, z}; }
inline f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline f3 operator-(f3 a) { return {-a.x, -a.y, -a.z}; }
inline f3 operator*(f3 a, float b) { return {a.x * b, a.y * b, a.z * b}; }
inline f3 operator*(float a, f3 b) { return {a * b.x, a * b.y, a * b.z}; }
inline f3 operator/(f3 a, float b) { return {a.x / b, a.y / b, a.z / b}; }
// float3 . float3, VectorMath.h:195-197 (left-to-right sum)
inline float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline f3 cross(f3 a, f3 b) {  // VectorMath.h:312-316
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline float norm(f3 a) { return std::sqrt(dot(a, a)); }     // :324-326
inline f3 normalised(f3 a) { return a / norm(a); }           // :340-342
inline f3 mul(const m3 &m, f3 a) { return {dot(m.rx, a), dot(m.ry, a), dot(m.rz, a)}; }
inline f3 xyz(f4 v) { return {v.x, v.y, v.z}; }

// CUDA's cvt.rzi (the reference's (int) casts run on the GPU): NaN -> 0,
// out-of-range saturates.  Used wherever the reference casts float -> int.
inline int f2i(double v) {
  if (std::isnan(v)) return 0;
  if (v >= 2147483647.0) return 2147483647;
  if (v <= -2147483648.0) return (-2147483647 - 1);
  return (int)v;
}
// make_int3(float3) == floor, VectorMath.h:36-42.
inline i3 floor3(f3 a) {
  i3 b{f2i(a.x), f2i(a.y), f2i(a.z)};
  b.x = (float)b.x > a.x ? b.x - 1 : b.x;
  b.y = (float)b.y > a.y ? b.y - 1 : b.y;
  b.z = (float)b.z > a.z ? b.z - 1 : b.z;
  return b;
}
// make_uchar3(float3) (VectorMath.h:16-18): int cast then uchar narrowing.
inline uint8_t f2u8(float v) { return (uint8_t)(uint32_t)f2i(v); }

m3 m3_from(const float *R) { return {{R[0], R[1], R[2]}, {R[3], R[4], R[5]}, {R[6], R[7], R[8]}}; }
f3 f3_from(const float *t) { return {t[0], t[1], t[2]}; }

// __constant__ sigSpace / sigRange (Pyrdown.cu:3-4)
const float kSigSpace = (float)(0.5 / (4 * 4));
const float kSigRange = (float)(0.5 / (0.5 * 0.5));
// gaussKernel (Pyrdown.cu:194-200)
const float kGauss[25] = {1, 4, 6, 4, 1, 4, 16, 24, 16, 4, 6, 24, 36,
                          24, 6, 4, 16, 24, 16, 4, 1, 4, 6, 4, 1};

}  // namespace

// =================================================================== pyramid
// FilterDepthKernel, Tracking/Pyrdown.cu:72-108 (+ launcher :110-121 passes
// depthScaleInv = 1.0 / depthScale as a float).
extern "C" void sfo_filter_depth(const uint16_t *d, int cols, int rows,
                                 float depth_scale, float cutoff, float *raw,
                                 float *filtered) {
  const float inv = (float)(1.0 / (double)depth_scale);
#pragma omp parallel for schedule(static)
  for (int y = 0; y < rows; ++y)
    for (int x = 0; x < cols; ++x) {
      float center = (float)d[y * cols + x] * inv;
      raw[y * cols + x] = center < cutoff ? center : kNaN;
      if (std::isnan(center)) { filtered[y * cols + x] = kNaN; continue; }
      const int R = 2, D = R * 2 + 1;
      int tx = std::min(x - D / 2 + D, cols - 1);
      int ty = std::min(y - D / 2 + D, rows - 1);
      float sum1 = 0, sum2 = 0;
      for (int cy = std::max(y - D / 2, 0); cy < ty; ++cy)
        for (int cx = std::max(x - D / 2, 0); cx < tx; ++cx) {
          float val = (float)d[cy * cols + cx] * inv;
          float space2 = (float)((x - cx) * (x - cx) + (y - cy) * (y - cy));
          float color2 = (center - val) * (center - val);
          float weight = std::exp(-(space2 * kSigSpace + color2 * kSigRange));
          sum1 += val * weight;
          sum2 += weight;
        }
      float fin = sum1 / sum2;
      filtered[y * cols + x] = fin < cutoff ? fin : kNaN;
    }
}

// PyrDownGaussKernel<float,float>, Pyrdown.cu:201-225 (note the reversed
// kernel index (ty-cy-1)*5 + (tx-cx-1) and the exclusive window bound).
extern "C" void sfo_pyrdown(const float *src, int sc, int sr, float *dst, int dc,
                            int dr) {
#pragma omp parallel for schedule(static)
  for (int y = 0; y < dr; ++y)
    for (int x = 0; x < dc; ++x) {
      const int D = 5;
      int tx = std::min(2 * x - D / 2 + D, sc - 1);
      int ty = std::min(2 * y - D / 2 + D, sr - 1);
      float sum = 0;
      int count = 0;
      for (int cy = std::max(0, 2 * y - D / 2); cy < ty; ++cy)
        for (int cx = std::max(0, 2 * x - D / 2); cx < tx; ++cx) {
          float v = src[cy * sc + cx];
          if (!std::isnan(v)) {
            float k = kGauss[(ty - cy - 1) * 5 + (tx - cx - 1)];
            sum += v * k;
            count = (int)((float)count + k);
          }
        }
      dst[y * dc + x] = sum / (float)count;
    }
}

// ComputeVMapKernel, Pyrdown.cu:123-145; launcher :147-158 passes 1.0/fx.
// Invalid pixels are written as all-NaN (the reference sets only x = NaN
// and leaves y, w unset; every consumer tests x only).
extern "C" void sfo_vmap(const float *depth, int cols, int rows, float fx,
                         float fy, float cx, float cy, float cutoff, float *vmap) {
  const float invfx = (float)(1.0 / (double)fx), invfy = (float)(1.0 / (double)fy);
#pragma omp parallel for schedule(static)
  for (int y = 0; y < rows; ++y)
    for (int x = 0; x < cols; ++x) {
      float z = depth[y * cols + x];
      float *v = vmap + 4 * (y * cols + x);
      if (!std::isnan(z) && (double)z > 0.1 && z < cutoff) {
        v[0] = z * ((float)x - cx) * invfx;
        v[1] = z * ((float)y - cy) * invfy;
        v[2] = z;
        v[3] = 1.0f;
      } else {
        v[0] = v[1] = v[2] = v[3] = kNaN;
      }
    }
}

// ComputeNMapKernel, Pyrdown.cu:160-181.
extern "C" void sfo_nmap(const float *vmap, int cols, int rows, float *nmap) {
#pragma omp parallel for schedule(static)
  for (int y = 0; y < rows; ++y)
    for (int x = 0; x < cols; ++x) {
      float *n = nmap + 4 * (y * cols + x);
      if (x == cols - 1 || y == rows - 1) { n[0] = n[1] = n[2] = n[3] = kNaN; continue; }
      const float *c = vmap + 4 * (y * cols + x);
      const float *r = vmap + 4 * (y * cols + x + 1);
      const float *d = vmap + 4 * ((y + 1) * cols + x);
      if (!std::isnan(c[0]) && !std::isnan(r[0]) && !std::isnan(d[0])) {
        f3 a = {r[0] - c[0], r[1] - c[1], r[2] - c[2]};
        f3 b = {d[0] - c[0], d[1] - c[1], d[2] - c[2]};
        f3 q = normalised(cross(a, b));
        n[0] = q.x; n[1] = q.y; n[2] = q.z; n[3] = 1.0f;
      } else {
        n[0] = n[1] = n[2] = n[3] = kNaN;
      }
    }
}

// ResizeMapKernel, Pyrdown.cu:318-346.  normalised(float4) includes w in
// the norm (VectorMath.h:328-330, 344-346).  The reference guards on the
// source size but launches over the destination (an out-of-bounds access
// when a destination side is not a multiple of 8); here the loop runs over
// the destination, which yields the same in-bounds values.
extern "C" void sfo_resize(const float *vsrc, const float *nsrc, int sc, int sr,
                           float *vdst, float *ndst, int dc, int dr) {
  (void)sr;
#pragma omp parallel for schedule(static)
  for (int y = 0; y < dr; ++y)
    for (int x = 0; x < dc; ++x) {
      const float *v00 = vsrc + 4 * ((2 * y) * sc + 2 * x), *v01 = v00 + 4;
      const float *v10 = vsrc + 4 * ((2 * y + 1) * sc + 2 * x), *v11 = v10 + 4;
      const float *n00 = nsrc + 4 * ((2 * y) * sc + 2 * x), *n01 = n00 + 4;
      const float *n10 = nsrc + 4 * ((2 * y + 1) * sc + 2 * x), *n11 = n10 + 4;
      float *vd = vdst + 4 * (y * dc + x), *nd = ndst + 4 * (y * dc + x);
      if (std::isnan(v00[0]) || std::isnan(v01[0]) || std::isnan(v10[0]) || std::isnan(v11[0])) {
        vd[0] = vd[1] = vd[2] = vd[3] = kNaN;
      } else {
        for (int k = 0; k < 4; ++k) vd[k] = (((v00[k] + v01[k]) + v10[k]) + v11[k]) / 4.0f;
      }
      if (std::isnan(n00[0]) || std::isnan(n01[0]) || std::isnan(n10[0]) || std::isnan(n11[0])) {
        nd[0] = nd[1] = nd[2] = nd[3] = kNaN;
      } else {
        float s[4];
        for (int k = 0; k < 4; ++k) s[k] = (((n00[k] + n01[k]) + n10[k]) + n11[k]) / 4.0f;
        float len = std::sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2] + s[3] * s[3]);
        for (int k = 0; k < 4; ++k) nd[k] = s[k] / len;
      }
    }
}

// ======================================================================= ICP
namespace {

// ICPReduce::searchPoint + getRow, Tracking/Reduction.cu:228-290, FP32
// reference semantics.  `1.0 / z` and `+ 0.5` are double in the reference.
bool icp_row_f32(const float *vc4, const float *vl_map, const float *nc4,
                 const float *nl_map, int cols, int rows, const m3 &Rc,
                 f3 tc, const m3 &Rl, const m3 &RlInv, f3 tl, float fx,
                 float fy, float cx, float cy, float *row7) {
  f3 vcurr_c = {vc4[0], vc4[1], vc4[2]};
  if (std::isnan(vcurr_c.x) || (double)vcurr_c.z < 1e-3) return false;
  f3 vcurr_g = mul(Rc, vcurr_c) + tc;
  f3 vcurr_p = mul(RlInv, vcurr_g - tl);
  float invz = (float)(1.0 / (double)vcurr_p.z);
  int u = f2i((double)(vcurr_p.x * invz * fx + cx) + 0.5);
  int v = f2i((double)(vcurr_p.y * invz * fy + cy) + 0.5);
  if (u < 0 || v < 0 || u >= cols || v >= rows) return false;
  const float *vl4 = vl_map + 4 * (v * cols + u);
  const float *nl4 = nl_map + 4 * (v * cols + u);
  f3 vlast_g = mul(Rl, mk3(vl4[0], vl4[1], vl4[2])) + tl;
  f3 ncurr_c = {nc4[0], nc4[1], nc4[2]};
  f3 ncurr_g = mul(Rc, ncurr_c);
  f3 nlast_c = {nl4[0], nl4[1], nl4[2]};
  f3 nlast_g = mul(Rl, nlast_c);
  float dist = norm(vlast_g - vcurr_g);
  float sine = norm(cross(ncurr_g, nlast_g));
  const float angleThresh = (float)0.6, distThresh = (float)0.1;  // Reduction.cu:361-362
  if (!(sine < angleThresh && dist <= distThresh && !std::isnan(ncurr_c.x) &&
        !std::isnan(nlast_c.x)))
    return false;
  f3 nlast = mul(RlInv, nlast_g);
  f3 vcurr = mul(RlInv, vcurr_g - tl);
  f3 vlast = mul(RlInv, vlast_g - tl);
  f3 mn = -nlast;
  f3 cr = cross(nlast, vlast);
  row7[0] = mn.x; row7[1] = mn.y; row7[2] = mn.z;
  row7[3] = cr.x; row7[4] = cr.y; row7[5] = cr.z;
  row7[6] = dot(mn, vcurr - vlast);
  return true;
}

// The same row computed entirely in double (error-budget oracle).
struct d3 { double x, y, z; };
inline d3 operator+(d3 a, d3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline d3 operator-(d3 a, d3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline double ddot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline d3 dcross(d3 a, d3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double dnorm(d3 a) { return std::sqrt(ddot(a, a)); }
struct dm3 { double m[9]; };
inline d3 dmul(const dm3 &R, d3 a) {
  return {R.m[0] * a.x + R.m[1] * a.y + R.m[2] * a.z, R.m[3] * a.x + R.m[4] * a.y + R.m[5] * a.z,
          R.m[6] * a.x + R.m[7] * a.y + R.m[8] * a.z};
}
bool icp_row_f64(const float *vc4, const float *vl_map, const float *nc4,
                 const float *nl_map, int cols, int rows, const dm3 &Rc, d3 tc,
                 const dm3 &Rl, const dm3 &RlInv, d3 tl, double fx, double fy,
                 double cx, double cy, double *row7) {
  d3 vcurr_c = {vc4[0], vc4[1], vc4[2]};
  if (std::isnan(vcurr_c.x) || vcurr_c.z < 1e-3) return false;
  d3 vcurr_g = dmul(Rc, vcurr_c) + tc;
  d3 vcurr_p = dmul(RlInv, vcurr_g - tl);
  double invz = 1.0 / vcurr_p.z;
  int u = f2i(vcurr_p.x * invz * fx + cx + 0.5);
  int v = f2i(vcurr_p.y * invz * fy + cy + 0.5);
  if (u < 0 || v < 0 || u >= cols || v >= rows) return false;
  const float *vl4 = vl_map + 4 * (v * cols + u);
  const float *nl4 = nl_map + 4 * (v * cols + u);
  d3 vlast_g = dmul(Rl, d3{vl4[0], vl4[1], vl4[2]}) + tl;
  d3 ncurr_g = dmul(Rc, d3{nc4[0], nc4[1], nc4[2]});
  d3 nlast_g = dmul(Rl, d3{nl4[0], nl4[1], nl4[2]});
  double dist = dnorm(vlast_g - vcurr_g);
  double sine = dnorm(dcross(ncurr_g, nlast_g));
  if (!(sine < 0.6 && dist <= 0.1 && !std::isnan(nc4[0]) && !std::isnan(nl4[0]))) return false;
  d3 nlast = dmul(RlInv, nlast_g);
  d3 vcurr = dmul(RlInv, vcurr_g - tl);
  d3 vlast = dmul(RlInv, vlast_g - tl);
  d3 cr = dcross(nlast, vlast);
  row7[0] = -nlast.x; row7[1] = -nlast.y; row7[2] = -nlast.z;
  row7[3] = cr.x; row7[4] = cr.y; row7[5] = cr.z;
  row7[6] = -(nlast.x * (vcurr.x - vlast.x) + nlast.y * (vcurr.y - vlast.y) + nlast.z * (vcurr.z - vlast.z));
  return true;
}

}  // namespace

// Per-pixel 29-vectors (Reduction.cu:281-289): upper triangle of [J|r]^T[J|r]
// (28 products) and the found flag.
extern "C" void sfo_icp_rows(const float *vcurr, const float *vlast,
                             const float *ncurr, const float *nlast, int cols,
                             int rows, const float *Rcurr, const float *tcurr,
                             const float *Rlast, const float *RlastInv,
                             const float *tlast, float fx, float fy, float cx,
                             float cy, float *rows29) {
  m3 Rc = m3_from(Rcurr), Rl = m3_from(Rlast), RlI = m3_from(RlastInv);
  f3 tc = f3_from(tcurr), tl = f3_from(tlast);
  const int N = cols * rows;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < N; ++i) {
    float row[7] = {0, 0, 0, 0, 0, 0, 0};
    bool found = icp_row_f32(vcurr + 4 * i, vlast, ncurr + 4 * i, nlast, cols, rows, Rc, tc, Rl,
                             RlI, tl, fx, fy, cx, cy, row);
    float *o = rows29 + 29 * (size_t)i;
    int k = 0;
    for (int a = 0; a < 7; ++a)
      for (int b = a; b < 7; ++b) o[k++] = row[a] * row[b];
    o[28] = (float)found;
  }
}

// icpStepKernel + Reduce<float,29> (Reduction.cu:292-385): the 29 sums.  The
// reference sums in float in a launch-shape-dependent order; the oracle sums
// the same FP32 per-pixel products in double (per-thread partials combined
// in thread order, so the result is deterministic for a thread count).
namespace {
// Sum of the 29 per-pixel terms.  fp64 == 0: FP32 rows (reference
// semantics) from the float pose; fp64 == 1: rows in double from the
// double pose.  Per-chunk partials combined in chunk order.
void icp_sums_impl(const float *vcurr, const float *vlast, const float *ncurr,
                   const float *nlast, int cols, int rows, const m3 &Rc, f3 tc,
                   const m3 &Rl, const m3 &RlI, f3 tl, const dm3 &dRc, d3 dtc,
                   const dm3 &dRl, const dm3 &dRlI, d3 dtl, float fx, float fy,
                   float cx, float cy, int fp64, double *out29) {
  const int N = cols * rows;
  for (int k = 0; k < 29; ++k) out29[k] = 0;
  const int kChunks = 64;
  std::vector<double> part((size_t)kChunks * 29, 0.0);
#pragma omp parallel for schedule(static)
  for (int c = 0; c < kChunks; ++c) {
    double *p = &part[(size_t)c * 29];
    int i0 = (int)((long long)N * c / kChunks), i1 = (int)((long long)N * (c + 1) / kChunks);
    for (int i = i0; i < i1; ++i) {
      if (fp64) {
        double row[7] = {0, 0, 0, 0, 0, 0, 0};
        bool found = icp_row_f64(vcurr + 4 * i, vlast, ncurr + 4 * i, nlast, cols, rows, dRc, dtc,
                                 dRl, dRlI, dtl, fx, fy, cx, cy, row);
        if (!found) continue;
        int k = 0;
        for (int a = 0; a < 7; ++a)
          for (int b = a; b < 7; ++b) p[k++] += row[a] * row[b];
        p[28] += 1.0;
      } else {
        float row[7] = {0, 0, 0, 0, 0, 0, 0};
        bool found = icp_row_f32(vcurr + 4 * i, vlast, ncurr + 4 * i, nlast, cols, rows, Rc, tc,
                                 Rl, RlI, tl, fx, fy, cx, cy, row);
        if (!found) continue;
        int k = 0;
        for (int a = 0; a < 7; ++a)
          for (int b = a; b < 7; ++b) p[k++] += (double)(row[a] * row[b]);
        p[28] += 1.0;
      }
    }
  }
  for (int c = 0; c < kChunks; ++c)
    for (int k = 0; k < 29; ++k) out29[k] += part[(size_t)c * 29 + k];
}
}  // namespace

// icpStepKernel + Reduce<float,29> (Reduction.cu:292-385): the 29 sums.  The
// reference sums in float in a launch-shape-dependent order; the oracle sums
// the same FP32 per-pixel products in double.
extern "C" void sfo_icp_sums(const float *vcurr, const float *vlast,
                             const float *ncurr, const float *nlast, int cols,
                             int rows, const float *Rcurr, const float *tcurr,
                             const float *Rlast, const float *RlastInv,
                             const float *tlast, float fx, float fy, float cx,
                             float cy, int fp64, double *out29) {
  m3 Rc = m3_from(Rcurr), Rl = m3_from(Rlast), RlI = m3_from(RlastInv);
  f3 tc = f3_from(tcurr), tl = f3_from(tlast);
  dm3 dRc, dRl, dRlI;
  for (int k = 0; k < 9; ++k) { dRc.m[k] = Rcurr[k]; dRl.m[k] = Rlast[k]; dRlI.m[k] = RlastInv[k]; }
  d3 dtc{tcurr[0], tcurr[1], tcurr[2]}, dtl{tlast[0], tlast[1], tlast[2]};
  icp_sums_impl(vcurr, vlast, ncurr, nlast, cols, rows, Rc, tc, Rl, RlI, tl, dRc, dtc, dRl, dRlI,
                dtl, fx, fy, cx, cy, fp64, out29);
}

// ================================================= photometric (RGB) term
// ImageToIntensityKernel, Tracking/Pyrdown.cu:250-260: double weights, the
// first byte weighted 0.7154 and the second 0.2125, as written.
extern "C" void sfo_intensity(const uint8_t *rgb, int cols, int rows, uint8_t *out) {
  for (int i = 0; i < cols * rows; ++i) {
    const uint8_t *p = rgb + 3 * (size_t)i;
    out[i] = (uint8_t)(int)(0.2125 * p[1] + 0.7154 * p[0] + 0.0721 * p[2]);
  }
}

// PyrDownGaussKernel<unsigned char, unsigned char>, Pyrdown.cu:201-245.
extern "C" void sfo_pyrdown_u8(const uint8_t *src, int sc, int sr, uint8_t *dst, int dc, int dr) {
  for (int y = 0; y < dr; ++y)
    for (int x = 0; x < dc; ++x) {
      const int D = 5;
      int tx = std::min(2 * x - D / 2 + D, sc - 1);
      int ty = std::min(2 * y - D / 2 + D, sr - 1);
      float sum = 0;
      int count = 0;
      for (int cy = std::max(0, 2 * y - D / 2); cy < ty; ++cy)
        for (int cx = std::max(0, 2 * x - D / 2); cx < tx; ++cx) {
          float k = kGauss[(ty - cy - 1) * 5 + (tx - cx - 1)];
          sum += (float)src[cy * sc + cx] * k;
          count = (int)((float)count + k);
        }
      dst[y * dc + x] = (uint8_t)(int)(sum / (float)count);
    }
}

// ComputeDerivativeImageKernel, Pyrdown.cu:262-304: the 3x3 Sobel taps are
// taken from index 8 downwards over the window clipped to the image, so at
// the border the taps shift, as written.
extern "C" void sfo_sobel(const uint8_t *img, int cols, int rows, int16_t *dx, int16_t *dy) {
  static const float sx[9] = {1, 0, -1, 2, 0, -2, 1, 0, -1};
  static const float sy[9] = {1, 2, 1, 0, 0, 0, -1, -2, -1};
  for (int y = 0; y < rows; ++y)
    for (int x = 0; x < cols; ++x) {
      float dxv = 0, dyv = 0;
      int k = 8;
      for (int j = std::max(y - 1, 0); j <= std::min(y + 1, rows - 1); j++)
        for (int i = std::max(x - 1, 0); i <= std::min(x + 1, cols - 1); i++) {
          dxv += (float)img[j * cols + i] * sx[k];
          dyv += (float)img[j * cols + i] * sy[k];
          --k;
        }
      dx[y * cols + x] = (int16_t)f2i(dxv);
      dy[y * cols + x] = (int16_t)f2i(dyv);
    }
}

namespace {
struct RgbCorr { int u, v, diff; };
// Frame::GpuRotation / GpuInvRotation / GpuTranslation (Core/Frame.cc:626-645).
void pose_f32(const double *P, float *R, float *Rinv, float *t) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) { R[i * 3 + j] = (float)P[i * 4 + j]; Rinv[i * 3 + j] = (float)P[j * 4 + i]; }
  for (int i = 0; i < 3; ++i) t[i] = (float)P[i * 4 + 3];
}
// __float2int_rd: floor, saturating, NaN -> 0.
inline int floor_i(float v) { return f2i(std::floor(v)); }
// RGBReduction::FindCorresp, Reduction.cu:412-463.  `+ 0.5` is double and
// the sum goes to __float2int_rd as a float.
bool rgb_corresp(const uint8_t *inext, const uint8_t *ilast, const float *vnext, const float *vlast,
                 const int16_t *dIdx, const int16_t *dIdy, int cols, int rows, int x, int y, const m3 &Rc,
                 f3 tc, const m3 &RlI, f3 tl, float fx, float fy, float cx, float cy, RgbCorr &r) {
  if (!(x >= 5 && x < cols - 5 && y >= 5 && y < rows - 5)) return false;
  bool valid = true;
  for (int u = std::max(y - 2, 0); u < std::min(y + 2, rows); ++u)
    for (int v = std::max(x - 2, 0); v < std::min(x + 2, cols); ++v) valid = valid && (inext[u * cols + v] > 0);
  if (!valid) return false;
  const int gx = dIdx[y * cols + x], gy = dIdy[y * cols + x];
  if (!(std::sqrt((float)(gx * gx + gy * gy)) > 0)) return false;
  const float *vc = vnext + 4 * ((size_t)y * cols + x);
  if (std::isnan(vc[0])) return false;
  const f3 vcurr_g = mul(Rc, mk3(vc[0], vc[1], vc[2])) + tc;
  const f3 vcl = mul(RlI, vcurr_g - tl);
  const int u = floor_i((float)((double)(fx * vcl.x / vcl.z + cx) + 0.5));
  const int v = floor_i((float)((double)(fy * vcl.y / vcl.z + cy) + 0.5));
  if (!(u >= 0 && v >= 0 && u < cols && v < rows)) return false;
  const float *vl = vlast + 4 * ((size_t)v * cols + u);
  if (std::isnan(vl[0])) return false;
  const float d0 = vl[0] - vc[0], d1 = vl[1] - vc[1], d2 = vl[2] - vc[2], d3 = vl[3] - vc[3];
  if (!((double)std::sqrt(d0 * d0 + d1 * d1 + d2 * d2 + d3 * d3) < 0.1)) return false;
  if (ilast[v * cols + u] == 0) return false;
  r.u = u;
  r.v = v;
  r.diff = (int)inext[y * cols + x] - (int)ilast[v * cols + u];
  return true;
}
// RGBStep's sigma (Reduction.cu:621-622) from the two integer sums.
float rgb_sigma(int count, int sumsq) {
  return std::sqrt((float)sumsq / (float)(count == 0 ? 1 : count));
}
// RGBReduction::GetRow, Reduction.cu:483-517, FP32 reference semantics
// (`/ 9.0` is double).
void rgb_row_f32(const RgbCorr &r, float sigma, const float *vlast, const int16_t *dIdx, const int16_t *dIdy,
                 int cols, int x, int y, const m3 &RcI, const m3 &Rl, f3 tl, f3 tc, float fx, float fy,
                 float row[7]) {
  float w = sigma + (float)std::abs(r.diff);
  w = (double)w < 1e-3 ? 1.0f : 1.0f / w;
  if ((double)sigma < 1e-6) w = 1.0f;
  const float *vl = vlast + 4 * ((size_t)r.v * cols + r.u);
  const f3 point = mul(RcI, ((mul(Rl, mk3(vl[0], vl[1], vl[2])) + tl) - tc));
  const float gx = (float)((double)(float)dIdx[y * cols + x] / 9.0);
  const float gy = (float)((double)(float)dIdy[y * cols + x] / 9.0);
  const float invz = 1.0f / point.z;
  f3 left;
  left.x = gx * fx * invz;
  left.y = gy * fy * invz;
  left.z = -(left.x * point.x + left.y * point.y) * invz;
  const f3 a = w * left, c = w * cross(point, left);
  row[0] = a.x; row[1] = a.y; row[2] = a.z;
  row[3] = c.x; row[4] = c.y; row[5] = c.z;
  row[6] = -w * (float)r.diff;
}
// The same row in double from the double pose (error-budget oracle); the
// correspondence and sigma are the FP32 ones.
void rgb_row_f64(const RgbCorr &r, float sigma, const float *vlast, const int16_t *dIdx, const int16_t *dIdy,
                 int cols, int x, int y, const dm3 &RcI, const dm3 &Rl, d3 tl, d3 tc, double fx, double fy,
                 double row[7]) {
  double w = (double)sigma + std::abs(r.diff);
  w = w < 1e-3 ? 1.0 : 1.0 / w;
  if ((double)sigma < 1e-6) w = 1.0;
  const float *vl = vlast + 4 * ((size_t)r.v * cols + r.u);
  const d3 point = dmul(RcI, (dmul(Rl, d3{vl[0], vl[1], vl[2]}) + tl) - tc);
  const double gx = (double)dIdx[y * cols + x] / 9.0, gy = (double)dIdy[y * cols + x] / 9.0;
  const double invz = 1.0 / point.z;
  const d3 left = {gx * fx * invz, gy * fy * invz, 0.0};
  const d3 l2 = {left.x, left.y, -(left.x * point.x + left.y * point.y) * invz};
  const d3 c = dcross(point, l2);
  row[0] = w * l2.x; row[1] = w * l2.y; row[2] = w * l2.z;
  row[3] = w * c.x; row[4] = w * c.y; row[5] = w * c.z;
  row[6] = -w * r.diff;
}
// ComputeResidualKernel + RgbStepKernel + both reductions (Reduction.cu
// :465-481, :519-551, :561-642): res = {count, sum of diff^2} (int sums,
// wrapping as the reference's), sigma, and the 29 sums (FP32 rows summed in
// double, or FP64 rows).
void rgb_sums_impl(const uint8_t *inext, const uint8_t *ilast, const float *vnext, const float *vlast,
                   const int16_t *dIdx, const int16_t *dIdy, int cols, int rows, const double *Pc,
                   const double *Pl, float fx, float fy, float cx, float cy, int fp64, double *out29,
                   int *res2, float *sigma_out, float *rows29) {
  float Rc[9], RcI[9], tcf[3], Rl[9], RlI[9], tlf[3];
  pose_f32(Pc, Rc, RcI, tcf);
  pose_f32(Pl, Rl, RlI, tlf);
  const m3 mRc = m3_from(Rc), mRcI = m3_from(RcI), mRl = m3_from(Rl), mRlI = m3_from(RlI);
  const f3 tc = f3_from(tcf), tl = f3_from(tlf);
  dm3 dRcI, dRl;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) { dRcI.m[r * 3 + c] = Pc[c * 4 + r]; dRl.m[r * 3 + c] = Pl[r * 4 + c]; }
  const d3 dtc{Pc[3], Pc[7], Pc[11]}, dtl{Pl[3], Pl[7], Pl[11]};
  const int N = cols * rows;
  std::vector<RgbCorr> corr(N);
  std::vector<uint8_t> ok(N, 0);
  uint32_t cnt = 0, ssq = 0;
  for (int i = 0; i < N; ++i) {
    const int y = i / cols, x = i - y * cols;
    if (rgb_corresp(inext, ilast, vnext, vlast, dIdx, dIdy, cols, rows, x, y, mRc, tc, mRlI, tl, fx, fy, cx,
                    cy, corr[i])) {
      ok[i] = 1;
      cnt += 1u;
      ssq += (uint32_t)(corr[i].diff * corr[i].diff);
    }
  }
  res2[0] = (int)cnt;
  res2[1] = (int)ssq;
  const float sigma = rgb_sigma(res2[0], res2[1]);
  if (sigma_out) *sigma_out = sigma;
  for (int k = 0; k < 29; ++k) out29[k] = 0.0;
  for (int i = 0; i < N; ++i) {
    float *o = rows29 ? rows29 + 29 * (size_t)i : nullptr;
    if (!ok[i]) {
      if (o) for (int k = 0; k < 29; ++k) o[k] = 0.f;
      continue;
    }
    const int y = i / cols, x = i - y * cols;
    int k = 0;
    if (fp64) {
      double row[7];
      rgb_row_f64(corr[i], sigma, vlast, dIdx, dIdy, cols, x, y, dRcI, dRl, dtl, dtc, fx, fy, row);
      for (int a = 0; a < 7; ++a)
        for (int b = a; b < 7; ++b) out29[k++] += row[a] * row[b];
    } else {
      float row[7];
      rgb_row_f32(corr[i], sigma, vlast, dIdx, dIdy, cols, x, y, mRcI, mRl, tl, tc, fx, fy, row);
      for (int a = 0; a < 7; ++a)
        for (int b = a; b < 7; ++b, ++k) {
          const float p = row[a] * row[b];
          out29[k] += (double)p;
          if (o) o[k] = p;
        }
      if (o) o[28] = 1.f;
    }
    out29[28] += 1.0;
  }
}
}  // namespace

// RGBStep (Reduction.cu:561-642) at the poses Pc (current estimate) and Pl
// (last frame), 4x4 row-major double: the 29 sums, res = {count, sum of
// diff^2}, sigma, and optionally the per-pixel FP32 29-vectors.
extern "C" void sfo_rgb_step(const uint8_t *inext, const uint8_t *ilast, const float *vnext,
                             const float *vlast, const int16_t *dIdx, const int16_t *dIdy, int cols,
                             int rows, const double *Pc, const double *Pl, float fx, float fy, float cx,
                             float cy, int fp64, double *out29, int *res2, float *sigma, float *rows29) {
  rgb_sums_impl(inext, ilast, vnext, vlast, dIdx, dIdy, cols, rows, Pc, Pl, fx, fy, cx, cy, fp64, out29, res2,
                sigma, rows29);
}

// CreateMatrix<6,7>, Reduction.cu:6-16.
extern "C" void sfo_create_matrix(const double *s, double *A, double *b) {
  int shift = 0;
  for (int i = 0; i < 6; ++i)
    for (int j = i; j < 7; ++j) {
      double value = s[shift++];
      if (j == 6) b[i] = value;
      else A[j * 6 + i] = A[i * 6 + j] = value;
    }
}

// Eigen::LDLT (Tracking.cc:493): LDL^T with symmetric pivoting on the
// largest remaining diagonal; a zero pivot zeroes that component of the
// solution (Eigen's LDLT::solve rule).
extern "C" void sfo_ldlt_solve6(const double *A36, const double *b6, double *x6) {
  double a[6][6];
  int perm[6];
  for (int i = 0; i < 6; ++i) { perm[i] = i; for (int j = 0; j < 6; ++j) a[i][j] = A36[i * 6 + j]; }
  double d[6];
  // Right-looking: a[k..][k..] is the Schur complement, columns < k hold L.
  for (int k = 0; k < 6; ++k) {
    int piv = k;
    double best = std::fabs(a[k][k]);
    for (int i = k + 1; i < 6; ++i) if (std::fabs(a[i][i]) > best) { best = std::fabs(a[i][i]); piv = i; }
    if (piv != k) {
      for (int j = 0; j < 6; ++j) std::swap(a[k][j], a[piv][j]);
      for (int i = 0; i < 6; ++i) std::swap(a[i][k], a[i][piv]);
      std::swap(perm[k], perm[piv]);
    }
    double dk = a[k][k];
    d[k] = dk;
    double l[6] = {0, 0, 0, 0, 0, 0};
    for (int i = k + 1; i < 6; ++i) l[i] = (dk != 0.0) ? a[i][k] / dk : 0.0;
    for (int i = k + 1; i < 6; ++i)
      for (int j = k + 1; j < 6; ++j) a[i][j] -= l[i] * dk * l[j];
    for (int i = k + 1; i < 6; ++i) { a[i][k] = l[i]; a[k][i] = 0.0; }
  }
  double y[6];
  for (int i = 0; i < 6; ++i) y[i] = b6[perm[i]];
  for (int i = 0; i < 6; ++i) for (int j = 0; j < i; ++j) y[i] -= a[i][j] * y[j];
  const double tol = std::numeric_limits<double>::min();
  for (int i = 0; i < 6; ++i) y[i] = (std::fabs(d[i]) > tol) ? y[i] / d[i] : 0.0;
  for (int i = 5; i >= 0; --i) for (int j = i + 1; j < 6; ++j) y[i] -= a[j][i] * y[j];
  for (int i = 0; i < 6; ++i) x6[perm[i]] = y[i];
}

// Sophus::SE3d::exp (Tracking.cc:494): twist (upsilon, omega), rotation via
// the unit quaternion of SO3::expAndTheta, translation V * upsilon with the
// left Jacobian V = I + (1-cos t)/t^2 W + (t - sin t)/t^3 W^2.
extern "C" void sfo_se3_exp(const double *xi, double *T) {
  const double ups[3] = {xi[0], xi[1], xi[2]}, w[3] = {xi[3], xi[4], xi[5]};
  const double eps = 1e-10;
  double th2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
  double th = std::sqrt(th2);
  double real_f, imag_f;
  if (th2 < eps * eps) {
    double th4 = th2 * th2;
    imag_f = 0.5 - (1.0 / 48.0) * th2 + (1.0 / 3840.0) * th4;
    real_f = 1.0 - (1.0 / 8.0) * th2 + (1.0 / 384.0) * th4;
  } else {
    imag_f = std::sin(0.5 * th) / th;
    real_f = std::cos(0.5 * th);
  }
  double qw = real_f, qx = imag_f * w[0], qy = imag_f * w[1], qz = imag_f * w[2];
  double tx = 2 * qx, ty = 2 * qy, tz = 2 * qz;
  double twx = tx * qw, twy = ty * qw, twz = tz * qw, txx = tx * qx, txy = ty * qx, txz = tz * qx;
  double tyy = ty * qy, tyz = tz * qy, tzz = tz * qz;
  double R[9] = {1 - (tyy + tzz), txy - twz, txz + twy, txy + twz, 1 - (txx + tzz),
                 tyz - twx, txz - twy, tyz + twx, 1 - (txx + tyy)};
  double W[9] = {0, -w[2], w[1], w[2], 0, -w[0], -w[1], w[0], 0};
  double W2[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0;
      for (int k = 0; k < 3; ++k) s += W[i * 3 + k] * W[k * 3 + j];
      W2[i * 3 + j] = s;
    }
  double V[9];
  if (th < eps) {
    for (int k = 0; k < 9; ++k) V[k] = R[k];
  } else {
    double c1 = (1 - std::cos(th)) / th2, c2 = (th - std::sin(th)) / (th2 * th);
    for (int k = 0; k < 9; ++k) V[k] = (k % 4 == 0 ? 1.0 : 0.0) + c1 * W[k] + c2 * W2[k];
  }
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) T[i * 4 + j] = R[i * 3 + j];
    T[i * 4 + 3] = V[i * 3 + 0] * ups[0] + V[i * 3 + 1] * ups[1] + V[i * 3 + 2] * ups[2];
  }
  T[12] = T[13] = T[14] = 0; T[15] = 1;
}

namespace {
void mat4_mul(const double *A, const double *B, double *C) {
  double t[16];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      double s = 0;
      for (int k = 0; k < 4; ++k) s += A[i * 4 + k] * B[k * 4 + j];
      t[i * 4 + j] = s;
    }
  memcpy(C, t, sizeof(t));
}
void se3_inv(const double *T, double *I) {
  double t[16];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) t[i * 4 + j] = T[j * 4 + i];
  for (int i = 0; i < 3; ++i) t[i * 4 + 3] = -(t[i * 4 + 0] * T[3] + t[i * 4 + 1] * T[7] + t[i * 4 + 2] * T[11]);
  t[12] = t[13] = t[14] = 0; t[15] = 1;
  memcpy(I, t, sizeof(t));
}
// Frame::GpuRotation / GpuInvRotation / GpuTranslation, Core/Frame.cc:626-645.
void pose_to_gpu(const double *P, float *R, float *Rinv, float *t) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) { R[i * 3 + j] = (float)P[i * 4 + j]; Rinv[i * 3 + j] = (float)P[j * 4 + i]; }
  for (int i = 0; i < 3; ++i) t[i] = (float)P[i * 4 + 3];
}
// |sin(eulerAngles(0,1,2))| (Tracking.cc:505-510): the norm is the same for
// both of Eigen's solution branches.
double euler_sin_norm(const double *P) {
  double r02 = std::max(-1.0, std::min(1.0, P[2]));
  double b = std::asin(r02);
  double a = std::atan2(-P[6], P[10]);
  double c = std::atan2(-P[1], P[0]);
  double sa = std::sin(a), sb = std::sin(b), sc = std::sin(c);
  return std::sqrt(sa * sa + sb * sb + sc * sc);
}
}  // namespace

// Tracker::ComputeSE3(icpOnly, iter, thresh), Tracking.cc:369-517.  With
// inext == nullptr it is the icpOnly form; else each iteration first runs
// RGBStep (:402-431) on the intensity pyramids inext / ilast and the next
// frame's derivative images, fails on a NaN error or too few photometric
// correspondences, and solves (A_rgb w + A_icp) x = b_rgb w + b_icp with
// w = 1e-4f (:484-491).  stats[0..3] = {icpError, icpCount, iterations,
// failure code}; with the RGB term stats[4..5] = {rgbError, rgbCount}.
extern "C" int sfo_compute_se3_ex(int levels, const int *cols, const int *rows,
                                  const float *const *vnext, const float *const *nnext,
                                  const float *const *vlast, const float *const *nlast,
                                  const uint8_t *const *inext, const uint8_t *const *ilast,
                                  const int16_t *const *dIdx, const int16_t *const *dIdy,
                                  const float *K, const int *iters, const int *min_count,
                                  float thresh, const double *last_pose, double *next_pose,
                                  int fp64, double *stats) {
  const bool rgb = inext != nullptr;
  int rgbCount = 0;
  double lastPose[16], pose[16], delta[16], candidate[16];
  memcpy(lastPose, last_pose, sizeof(lastPose));
  memcpy(pose, next_pose, sizeof(pose));
  for (int k = 0; k < 16; ++k) delta[k] = (k % 5 == 0) ? 1.0 : 0.0;
  float rgbError = 0, icpError = 0, lastError = 100.f, currError = 0, candidateICP = 0;
  const float w = 1e-4f;
  int breakCount = 0, its = 0, icpCount = 0;
  float Rl[9], RlI[9], tl[3];
  pose_to_gpu(lastPose, Rl, RlI, tl);
  for (int i = levels - 1; i >= 0; --i) {
    const int div = 1 << i;
    const float fx = K[0] / (float)div, fy = K[1] / (float)div, cx = K[2] / (float)div, cy = K[3] / (float)div;
    for (int j = 0; j < iters[i]; ++j) {
      float Rc[9], RcI[9], tc[3];
      pose_to_gpu(next_pose, Rc, RcI, tc);
      double s[29], A[36], b[6], x[6], dT[16], dInv[16];
      {
        dm3 dRc, dRl, dRlI;
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c) {
            dRc.m[r * 3 + c] = next_pose[r * 4 + c];
            dRl.m[r * 3 + c] = lastPose[r * 4 + c];
            dRlI.m[r * 3 + c] = lastPose[c * 4 + r];
          }
        d3 dtc{next_pose[3], next_pose[7], next_pose[11]}, dtl{lastPose[3], lastPose[7], lastPose[11]};
        icp_sums_impl(vnext[i], vlast[i], nnext[i], nlast[i], cols[i], rows[i], m3_from(Rc),
                      f3_from(tc), m3_from(Rl), m3_from(RlI), f3_from(tl), dRc, dtc, dRl, dRlI,
                      dtl, fx, fy, cx, cy, fp64, s);
      }
      ++its;
      double Argb[36], brgb[6];
      if (rgb) {
        double srgb[29];
        int res2[2];
        rgb_sums_impl(inext[i], ilast[i], vnext[i], vlast[i], dIdx[i], dIdy[i], cols[i], rows[i], next_pose,
                      lastPose, fx, fy, cx, cy, fp64, srgb, res2, nullptr, nullptr);
        float rres[2] = {(float)srgb[27], (float)srgb[28]};
        sfo_create_matrix(srgb, Argb, brgb);
        rgbError = std::sqrt(rres[0]) / rres[1];
        rgbCount = (int)rres[1];
        if (std::isnan(rgbError) || rgbCount < min_count[i]) {
          memcpy(next_pose, lastPose, sizeof(lastPose));
          if (stats) {
            stats[0] = icpError; stats[1] = icpCount; stats[2] = its; stats[3] = 1;
            stats[4] = rgbError; stats[5] = rgbCount;
          }
          return 0;
        }
      }
      float residual[2] = {(float)s[27], (float)s[28]};
      sfo_create_matrix(s, A, b);
      icpError = std::sqrt(residual[0]) / residual[1];
      icpCount = (int)residual[1];
      if (std::isnan(icpError) || icpCount < min_count[i]) {
        memcpy(next_pose, lastPose, sizeof(lastPose));
        if (stats) {
          stats[0] = icpError; stats[1] = icpCount; stats[2] = its; stats[3] = 1;
          if (rgb) { stats[4] = rgbError; stats[5] = rgbCount; }
        }
        return 0;
      }
      currError = rgbError * w + icpError;
      if (lastError < currError) {
        breakCount++;
        if (breakCount == 1) memcpy(candidate, next_pose, sizeof(candidate));
        candidateICP = icpError;  // outside the inner if (Tracking.cc:463-465)
      } else {
        breakCount = 0;
      }
      if (breakCount > 2) {
        memcpy(next_pose, candidate, sizeof(candidate));
        icpError = candidateICP;
        break;
      }
      lastError = currError;
      if (rgb) {
        for (int k = 0; k < 36; ++k) A[k] = Argb[k] * (double)w + A[k];
        for (int k = 0; k < 6; ++k) b[k] = brgb[k] * (double)w + b[k];
      }
      sfo_ldlt_solve6(A, b, x);
      sfo_se3_exp(x, dT);
      mat4_mul(dT, delta, delta);
      se3_inv(delta, dInv);
      mat4_mul(lastPose, dInv, next_pose);
    }
    if (breakCount > 2) break;
  }
  double pinv[16], p[16];
  se3_inv(pose, pinv);
  mat4_mul(pinv, next_pose, p);
  double tn = std::sqrt(p[3] * p[3] + p[7] * p[7] + p[11] * p[11]);
  double an = euler_sin_norm(p);
  int ok = (icpError < thresh) && (an <= 0.1 && tn <= 0.1);
  if (!ok) memcpy(next_pose, lastPose, sizeof(lastPose));
  if (stats) {
    stats[0] = icpError; stats[1] = icpCount; stats[2] = its; stats[3] = ok ? 0 : 2;
    if (rgb) { stats[4] = rgbError; stats[5] = rgbCount; }
  }
  return ok;
}

// Tracker::ComputeSE3(icpOnly=true, iter, thresh).
extern "C" int sfo_compute_se3(int levels, const int *cols, const int *rows,
                               const float *const *vnext, const float *const *nnext,
                               const float *const *vlast, const float *const *nlast,
                               const float *K, const int *iters, const int *min_count,
                               float thresh, const double *last_pose, double *next_pose,
                               int fp64, double *stats) {
  return sfo_compute_se3_ex(levels, cols, rows, vnext, nnext, vlast, nlast, nullptr, nullptr, nullptr, nullptr,
                            K, iters, min_count, thresh, last_pose, next_pose, fp64, stats);
}

// ======================================================================= map
struct sfo_map {
  sfo_config c;
  float voxelSizeInv, blockWidth, stepScale;  // DeviceMap.h:186-189
  uint32_t numEntries;
  std::vector<sfo_entry> entries, visible;
  std::vector<sfo_voxel> voxels;
  std::vector<int> heap, mutex;
  int heapCounter = 0, entryPtr = 1;
  unsigned noVisible = 0;
};

namespace {
// DeviceMap::Hash, Mapping/DeviceMap.cu:3-10.  `% NumBuckets` is taken on
// the unsigned conversion of the signed product-xor (NumBuckets is uint).
inline uint32_t hash_pos(const sfo_map &m, i3 p) {
  uint32_t h = ((uint32_t)p.x * 73856093u) ^ ((uint32_t)p.y * 19349669u) ^ ((uint32_t)p.z * 83492791u);
  return h % m.c.num_buckets;
}
inline bool pos_eq(const sfo_entry &e, i3 p) { return e.x == p.x && e.y == p.y && e.z == p.z; }
// voxelPosToBlockPos, DeviceMap.cu:169-180.
inline i3 vox2block(i3 v) {
  if (v.x < 0) v.x -= 7;
  if (v.y < 0) v.y -= 7;
  if (v.z < 0) v.z -= 7;
  return {v.x / 8, v.y / 8, v.z / 8};
}
// voxelPosToLocalIdx, DeviceMap.cu:186-201,218-220.
inline int vox2local(i3 v) {
  int lx = v.x % 8, ly = v.y % 8, lz = v.z % 8;
  if (lx < 0) lx += 8;
  if (ly < 0) ly += 8;
  if (lz < 0) lz += 8;
  return lz * 64 + ly * 8 + lx;
}
// DeviceMap::CreateEntry, DeviceMap.cu:12-21.
sfo_entry create_entry(sfo_map &m, i3 p, int offset) {
  int old = m.heapCounter--;
  if (old >= 0) {
    int ptr = m.heap[old];
    if (ptr != -1) return {p.x, p.y, p.z, ptr * 512, offset, {0, 0, 0}};
  }
  return {p.x, p.y, p.z, -1, 0, {0, 0, 0}};
}
// DeviceMap::CreateBlock, DeviceMap.cu:23-69, executed serially (the bucket
// mutex never contends).
void create_block(sfo_map &m, i3 p) {
  uint32_t bucket = hash_pos(m, p);
  sfo_entry *e = &m.entries[bucket];
  sfo_entry *empty = nullptr;
  if (pos_eq(*e, p) && e->ptr != -1) return;
  if (e->ptr == -1) empty = e;
  while (e->offset > 0) {
    e = &m.entries[m.c.num_buckets + e->offset - 1];
    if (pos_eq(*e, p) && e->ptr != -1) return;
    if (e->ptr == -1 && !empty) empty = e;
  }
  if (empty) {
    *empty = create_entry(m, p, e->offset);
  } else {
    int offset = m.entryPtr++;
    if (offset <= (int)m.c.num_excess) {
      m.entries[m.c.num_buckets + offset - 1] = create_entry(m, p, 0);
      e->offset = offset;
    }
  }
}
// DeviceMap::FindEntry, DeviceMap.cu:141-154.
const sfo_entry *find_entry(const sfo_map &m, i3 p) {
  uint32_t bucket = hash_pos(m, p);
  const sfo_entry *e = &m.entries[bucket];
  if (e->ptr != -1 && pos_eq(*e, p)) return e;
  while (e->offset > 0) {
    e = &m.entries[m.c.num_buckets + e->offset - 1];
    if (pos_eq(*e, p) && e->ptr != -1) return e;
  }
  return nullptr;
}
}  // namespace

extern "C" sfo_map *sfo_map_create(const sfo_config *cfg) {
  sfo_map *m = new sfo_map();
  m->c = *cfg;
  m->voxelSizeInv = (float)(1.0 / (double)cfg->voxel_size);
  m->blockWidth = cfg->voxel_size * 8.0f;
  m->stepScale = (float)(0.5 * (double)cfg->trunc_dist * (double)m->voxelSizeInv);
  m->numEntries = cfg->num_buckets + cfg->num_excess;
  m->entries.resize(m->numEntries);
  m->visible.resize(m->numEntries);
  m->voxels.resize((size_t)cfg->num_sdf_blocks * 512);
  m->heap.resize(cfg->num_sdf_blocks);
  m->mutex.resize(cfg->num_buckets);
  sfo_map_reset(m);
  return m;
}
extern "C" void sfo_map_destroy(sfo_map *m) { delete m; }

// ResetHashKernel + ResetSdfBlockKernel, FuseMap.cu:1251-1289.  release()
// leaves `offset` untouched; the reference relies on freshly allocated
// (zeroed) memory, so reset writes offset = 0.
extern "C" void sfo_map_reset(sfo_map *m) {
  for (auto &e : m->entries) e = {0, 0, 0, -1, 0, {0, 0, 0}};
  for (auto &e : m->visible) e = {0, 0, 0, -1, 0, {0, 0, 0}};
  for (auto &x : m->mutex) x = -1;
  for (uint32_t x = 0; x < m->c.num_sdf_blocks; ++x) m->heap[x] = (int)m->c.num_sdf_blocks - (int)x - 1;
  sfo_voxel rel;
  memset(&rel, 0, sizeof(rel));
  rel.sdf = kNaN;
  for (auto &v : m->voxels) {
    uint8_t keep = v.obj_idx;  // release() does not touch obj_idx
    v = rel;
    v.obj_idx = keep;
  }
  m->heapCounter = (int)m->c.num_sdf_blocks - 1;
  m->entryPtr = 1;
  m->noVisible = 0;
}
extern "C" sfo_entry *sfo_map_entries(sfo_map *m) { return m->entries.data(); }
extern "C" sfo_voxel *sfo_map_voxels(sfo_map *m) { return m->voxels.data(); }
extern "C" sfo_entry *sfo_map_visible(sfo_map *m) { return m->visible.data(); }
extern "C" int *sfo_map_heap(sfo_map *m) { return m->heap.data(); }
extern "C" void sfo_map_counters(sfo_map *m, int *out) {
  int alloc = 0;
  for (auto &e : m->entries) alloc += e.ptr >= 0;
  out[0] = m->heapCounter; out[1] = m->entryPtr; out[2] = (int)m->noVisible; out[3] = alloc;
}

extern "C" void sfo_map_set_no_visible(sfo_map *m, unsigned n) { m->noVisible = n; }

// Fusion::CreateBlocks, FuseMap.cu:92-132 (unproject :35-44), run serially
// in the launch order of its (16, 8) thread blocks (FuseMap.cu:1093-1096):
// block rows, blocks, thread rows, threads.  The order decides which of two
// blocks new in the same frame with the same bucket holds the bucket slot
// (a race on the GPU); UnifyNeighbor's pass over hash slots [0, noVisible)
// depends on it.
extern "C" void sfo_alloc(sfo_map *m, const float *depth, int cols, int rows,
                          const float *R, const float *t, float fx, float fy,
                          float cx, float cy) {
  m3 Rv = m3_from(R);
  f3 tv = f3_from(t);
  const float invfx = (float)(1.0 / (double)fx), invfy = (float)(1.0 / (double)fy);
  const float dmin = m->c.depth_min, dmax = m->c.depth_max;
  const int tiles_x = (cols + 15) / 16, tiles_y = (rows + 7) / 8;
  for (int p = 0; p < tiles_x * tiles_y * 128; ++p) {
    const int tile = p / 128, in = p % 128;
    const int x = (tile % tiles_x) * 16 + in % 16, y = (tile / tiles_x) * 8 + in / 16;
    if (x >= cols || y >= rows) continue;
    float z = depth[y * cols + x];
    if (std::isnan(z) || z < dmin || z > dmax) continue;
    float thresh = m->c.trunc_dist / 2.0f;
    float z_near = std::fmax(dmin, z - thresh);
    float z_far = std::fmin(dmax, z + thresh);
    if (z_near >= z_far) continue;
    f3 pn = {z_near * ((float)x - cx) * invfx, z_near * ((float)y - cy) * invfy, z_near};
    f3 pf = {z_far * ((float)x - cx) * invfx, z_far * ((float)y - cy) * invfy, z_far};
    f3 pt_near = (mul(Rv, pn) + tv) * m->voxelSizeInv;
    f3 pt_far = (mul(Rv, pf) + tv) * m->voxelSizeInv;
    f3 dir = pt_far - pt_near;
    float length = norm(dir);
    int nSteps = f2i(std::ceil(2.0 * (double)length));
    dir = dir / (float)(nSteps - 1);
    for (int i = 0; i < nSteps; ++i) {
      create_block(*m, vox2block(floor3(pt_near)));
      pt_near = pt_near + dir;
    }
  }
}

namespace {
struct Cam {
  m3 R, Rinv;
  f3 t;
  float fx, fy, cx, cy;
  int cols, rows;
  float dmin, dmax;
};
// Fusion::CheckVertexVisibility, FuseMap.cu:46-56 (project :27-33).
inline bool vertex_visible(const Cam &c, f3 p3) {
  f3 pt = mul(c.Rinv, p3 - c.t);
  if (pt.z < 1e-3f) return false;
  float px = c.fx * pt.x / pt.z + c.cx;
  float py = c.fy * pt.y / pt.z + c.cy;
  return px >= 0 && py >= 0 && px < (float)c.cols && py < (float)c.rows && pt.z >= c.dmin &&
         pt.z <= c.dmax;
}
// Fusion::CheckBlockVisibility, FuseMap.cu:58-90 (the corner walk order).
bool block_visible(const Cam &c, const sfo_map &m, i3 pos) {
  float s = m.blockWidth;
  f3 k = {(float)pos.x * s, (float)pos.y * s, (float)pos.z * s};
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
}  // namespace

// Fusion::CheckFullVisibility + ComputeOffset, FuseMap.cu:134-168 and
// Utility/ParallelScan.h:1-49: the visible set, compacted in entry order.
extern "C" unsigned sfo_visibility(sfo_map *m, const float *R, const float *Rinv,
                                   const float *t, int cols, int rows, float fx,
                                   float fy, float cx, float cy, float depth_max,
                                   float depth_min) {
  Cam c{m3_from(R), m3_from(Rinv), f3_from(t), fx, fy, cx, cy, cols, rows, depth_min, depth_max};
  unsigned n = 0;
  for (uint32_t x = 0; x < m->numEntries; ++x) {
    const sfo_entry &e = m->entries[x];
    if (e.ptr != -1 && block_visible(c, *m, {e.x, e.y, e.z})) {
      if (n < m->numEntries) m->visible[n] = e;
      ++n;
    }
  }
  m->noVisible = n;
  return n;
}

namespace {
// project(): FuseMap.cu:27-33 then make_int2 (truncation, VectorMath.h:28-30).
inline bool voxel_pixel(const Cam &c, const sfo_map &m, i3 blk, int lx, int ly, int lz, f3 &pos,
                        int &u, int &v) {
  f3 w = {(float)(blk.x * 8 + lx) * m.c.voxel_size, (float)(blk.y * 8 + ly) * m.c.voxel_size,
          (float)(blk.z * 8 + lz) * m.c.voxel_size};
  pos = mul(c.Rinv, w - c.t);
  u = f2i(c.fx * pos.x / pos.z + c.cx);
  v = f2i(c.fy * pos.y / pos.z + c.cy);
  return !(u < 0 || v < 0 || u >= c.cols || v >= c.rows);
}
}  // namespace

// Fusion::createVoxels, FuseMap.cu:432-507 (one update per visible voxel).
extern "C" void sfo_integrate(sfo_map *m, const float *depth, const uint8_t *rgb,
                              int cols, int rows, const float *Rinv, const float *t,
                              float fx, float fy, float cx, float cy,
                              float depth_max, float depth_min) {
  Cam c{{}, m3_from(Rinv), f3_from(t), fx, fy, cx, cy, cols, rows, depth_min, depth_max};
  const float thresh = m->c.trunc_dist;
#pragma omp parallel for schedule(dynamic, 16)
  for (int b = 0; b < (int)m->noVisible; ++b) {
    const sfo_entry &entry = m->visible[b];
    if (entry.ptr == -1) continue;
    i3 blk = {entry.x, entry.y, entry.z};
    for (int lz = 0; lz < 8; ++lz)
      for (int ly = 0; ly < 8; ++ly)
        for (int lx = 0; lx < 8; ++lx) {
          f3 pos;
          int u, v;
          if (!voxel_pixel(c, *m, blk, lx, ly, lz, pos, u, v)) continue;
          float dp = depth[v * cols + u];
          if (std::isnan(dp) || dp > c.dmax || dp < c.dmin) continue;
          float sdf = dp - pos.z;
          if (!(sdf >= -thresh)) continue;
          sdf = std::fmin(1.0f, sdf / thresh);
          const uint8_t *px = rgb + 3 * (v * cols + u);
          f3 val = {(float)px[0], (float)px[1], (float)px[2]};
          sfo_voxel &prev = m->voxels[(size_t)entry.ptr + lz * 64 + ly * 8 + lx];
          if (prev.weight == 0) {
            uint8_t keep = prev.obj_idx;  // Voxel::operator= skips obj_idx
            memset(&prev, 0, sizeof(prev));
            prev.obj_idx = keep;
            prev.sdf = sdf;
            prev.weight = 1;
            prev.color[0] = f2u8(val.x); prev.color[1] = f2u8(val.y); prev.color[2] = f2u8(val.z);
          } else {
            if (prev.label == 0) {
              // (make_float3(color) * weight) resolves to operator*(float3,int)
              // -> int3 (VectorMath.h:231-233), then int3 + float3 -> float3.
              int wgt = prev.weight;
              float r0 = ((float)(f2i((float)prev.color[0] * (float)wgt)) + val.x) / (float)(wgt + 1);
              float r1 = ((float)(f2i((float)prev.color[1] * (float)wgt)) + val.y) / (float)(wgt + 1);
              float r2 = ((float)(f2i((float)prev.color[2] * (float)wgt)) + val.z) / (float)(wgt + 1);
              prev.color[0] = f2u8(r0); prev.color[1] = f2u8(r1); prev.color[2] = f2u8(r2);
            }
            prev.sdf = (prev.sdf * (float)prev.weight + sdf) / (float)(prev.weight + 1);
            prev.weight = (uint8_t)std::min(255, prev.weight + 1);
          }
        }
  }
}

// FP64 shadow of the TSDF (measurement only, not a reference kernel): for
// the voxels createVoxels updates this frame (the same gates, decided in
// FP32 as the reference decides them), the new TSDF in double: the voxel's
// camera depth from the FP64 pose and the voxel centre in double, and the
// running average in double.  Called before sfo_integrate of the same frame
// (it reads the pre-update weight).  The shadow is per heap block, made on
// first touch; sfo_tsdf_f64_error compares it with the FP32 voxels.
struct sfo_f64_shadow {
  std::vector<std::unique_ptr<double[]>> blocks;
};
static sfo_f64_shadow &f64_shadow(sfo_map *m) {
  static std::mutex mu;
  static std::vector<std::pair<sfo_map *, std::unique_ptr<sfo_f64_shadow>>> all;
  std::lock_guard<std::mutex> lock(mu);
  for (auto &e : all)
    if (e.first == m) return *e.second;
  all.emplace_back(m, std::unique_ptr<sfo_f64_shadow>(new sfo_f64_shadow()));
  all.back().second->blocks.resize(m->c.num_sdf_blocks);
  return *all.back().second;
}

extern "C" void sfo_integrate_f64(sfo_map *m, const float *depth, int cols, int rows, const float *Rinv,
                                  const float *t, const double *P64, float fx, float fy, float cx, float cy,
                                  float depth_max, float depth_min) {
  Cam c{{}, m3_from(Rinv), f3_from(t), fx, fy, cx, cy, cols, rows, depth_min, depth_max};
  const float thresh = m->c.trunc_dist;
  sfo_f64_shadow &sh = f64_shadow(m);
  // the visible blocks' shadows, made serially before the parallel pass
  for (unsigned b = 0; b < m->noVisible; ++b) {
    const sfo_entry &entry = m->visible[b];
    if (entry.ptr < 0) continue;
    auto &blk = sh.blocks[(size_t)entry.ptr / 512];
    if (!blk) {
      blk.reset(new double[512]);
      for (int k = 0; k < 512; ++k) blk[k] = 0.0;
    }
  }
#pragma omp parallel for schedule(dynamic, 16)
  for (int b = 0; b < (int)m->noVisible; ++b) {
    const sfo_entry &entry = m->visible[b];
    if (entry.ptr == -1) continue;
    i3 blk = {entry.x, entry.y, entry.z};
    double *s64 = sh.blocks[(size_t)entry.ptr / 512].get();
    for (int lz = 0; lz < 8; ++lz)
      for (int ly = 0; ly < 8; ++ly)
        for (int lx = 0; lx < 8; ++lx) {
          f3 pos;
          int u, v;
          if (!voxel_pixel(c, *m, blk, lx, ly, lz, pos, u, v)) continue;
          float dp = depth[v * cols + u];
          if (std::isnan(dp) || dp > c.dmax || dp < c.dmin) continue;
          float sdf = dp - pos.z;
          if (!(sdf >= -thresh)) continue;
          // camera depth of the voxel centre in double: z = row 2 of R^T (w - t)
          const double vs = (double)m->c.voxel_size;
          const double wx = (double)(blk.x * 8 + lx) * vs, wy = (double)(blk.y * 8 + ly) * vs,
                       wz = (double)(blk.z * 8 + lz) * vs;
          const double dx = wx - P64[3], dy = wy - P64[7], dz = wz - P64[11];
          const double z64 = P64[2] * dx + P64[6] * dy + P64[10] * dz;
          double sd = (double)dp - z64;
          sd = std::fmin(1.0, sd / (double)thresh);
          const size_t li = (size_t)(lz * 64 + ly * 8 + lx);
          const sfo_voxel &prev = m->voxels[(size_t)entry.ptr + li];
          if (prev.weight == 0)
            s64[li] = sd;
          else
            s64[li] = (s64[li] * (double)prev.weight + sd) / (double)(prev.weight + 1);
        }
  }
}

// out[0] = max |tsdf32 - tsdf64|, out[1] = RMS, out[2] = voxels compared
// (every voxel of a shadowed block with weight > 0).  The TSDF is the
// voxel's normalised distance in [-1, 1].
extern "C" void sfo_tsdf_f64_error(sfo_map *m, double *out) {
  sfo_f64_shadow &sh = f64_shadow(m);
  double mx = 0.0, ss = 0.0, n = 0.0;
  for (size_t b = 0; b < sh.blocks.size(); ++b) {
    if (!sh.blocks[b]) continue;
    for (int k = 0; k < 512; ++k) {
      const sfo_voxel &v = m->voxels[b * 512 + k];
      if (v.weight == 0) continue;
      const double e = std::fabs((double)v.sdf - sh.blocks[b][k]);
      mx = std::max(mx, e);
      ss += e * e;
      n += 1.0;
    }
  }
  out[0] = mx;
  out[1] = n > 0 ? std::sqrt(ss / n) : 0.0;
  out[2] = n;
}

// Fusion::analyzeSemantics, FuseMap.cu:509-668, one update per voxel (the
// (8,8) launch of AnalyzeMapSemantics, FuseMap.cu:1234-1236).
extern "C" void sfo_semantics(sfo_map *m, const float *depth, const uint8_t *rgb,
                              const float *nmap, const uint8_t *mask,
                              int num_detection, int cols, int rows,
                              const float *Rinv, const float *t, float fx,
                              float fy, float cx, float cy, float depth_max,
                              float depth_min) {
  Cam c{{}, m3_from(Rinv), f3_from(t), fx, fy, cx, cy, cols, rows, depth_min, depth_max};
  const float thresh = m->c.trunc_dist;
  const int pal[3] = {(int)(std::pow(2, 25) - 1), (int)(std::pow(2, 15) - 1), (int)(std::pow(2, 21) - 1)};
#pragma omp parallel for schedule(dynamic, 16)
  for (int b = 0; b < (int)m->noVisible; ++b) {
    const sfo_entry &entry = m->visible[b];
    if (entry.ptr == -1) continue;
    i3 blk = {entry.x, entry.y, entry.z};
    for (int lz = 0; lz < 8; ++lz)
      for (int ly = 0; ly < 8; ++ly)
        for (int lx = 0; lx < 8; ++lx) {
          f3 pos;
          int u, v;
          if (!voxel_pixel(c, *m, blk, lx, ly, lz, pos, u, v)) continue;
          float dp = depth[v * cols + u];
          if (std::isnan(dp) || dp > c.dmax || dp < c.dmin) continue;
          const float *nl = nmap + 4 * (v * cols + u);
          if (std::isnan(nl[0])) continue;
          float sdf = dp - pos.z;
          if (!(sdf >= -thresh)) continue;
          f3 val;
          uint8_t label;
          const uint8_t *px = rgb + 3 * (v * cols + u);
          if (num_detection > 0) {
            label = mask[v * cols + u];
            if (label == 0) {
              val = {(float)px[0], (float)px[1], (float)px[2]};
            } else {
              // pallete[k] * int(label) wraps in 32-bit on the GPU.
              int p0 = (int)((uint32_t)pal[0] * (uint32_t)label) % 255;
              int p1 = (int)((uint32_t)pal[1] * (uint32_t)label) % 255;
              int p2 = (int)((uint32_t)pal[2] * (uint32_t)label) % 255;
              val = {(float)p0, (float)p1, (float)p2};
            }
          } else {
            label = 0;
            val = {(float)px[0], (float)px[1], (float)px[2]};
          }
          sfo_voxel &prev = m->voxels[(size_t)entry.ptr + lz * 64 + ly * 8 + lx];
          if (prev.weight == 0) continue;
          if (label != 0) {
            if (label == prev.label) {
              prev.count = (uint8_t)std::min(255, prev.count + 1);
              prev.color[0] = f2u8(val.x); prev.color[1] = f2u8(val.y); prev.color[2] = f2u8(val.z);
            } else {
              if (label == prev.label_2) {
                prev.count_2 = (uint8_t)std::min(255, prev.count_2 + 1);
                prev.color_2[0] = f2u8(val.x); prev.color_2[1] = f2u8(val.y); prev.color_2[2] = f2u8(val.z);
              } else if (prev.count_2 < 7) {
                prev.label_2 = label;
                prev.count_2 = 1;
                prev.color_2[0] = f2u8(val.x); prev.color_2[1] = f2u8(val.y); prev.color_2[2] = f2u8(val.z);
              }
              if ((prev.count < prev.count_2 && prev.label != 0) ||
                  (prev.count < prev.count_2 * 2 && prev.label == 0)) {
                std::swap(prev.label, prev.label_2);
                std::swap(prev.count, prev.count_2);
                for (int k = 0; k < 3; ++k) std::swap(prev.color[k], prev.color_2[k]);
              }
            }
          } else {
            // w = nl . normalised(make_float4(pos)) (FuseMap.cu:641), float4 dot
            float len = std::sqrt(pos.x * pos.x + pos.y * pos.y + pos.z * pos.z + 1.0f * 1.0f);
            float a0 = pos.x / len, a1 = pos.y / len, a2 = pos.z / len, a3 = 1.0f / len;
            float wgt = nl[0] * a0 + nl[1] * a1 + nl[2] * a2 + nl[3] * a3;
            if (prev.label != 0) {
              if (prev.count < 7) {
                prev.label_2 = prev.label;
                for (int k = 0; k < 3; ++k) prev.color_2[k] = prev.color[k];
                prev.count_2 = prev.count;
                prev.label = 0;
                prev.count = 1;
                f3 vv = val / 255.f;
                f3 old = mk3((float)prev.color[0], (float)prev.color[1], (float)prev.color[2]) / 255.f;
                float a = wgt * 0.2f;
                f3 res = (a * vv + (1 - wgt * 0.2f) * old) * 255.f;
                prev.color[0] = f2u8(res.x); prev.color[1] = f2u8(res.y); prev.color[2] = f2u8(res.z);
              }
            } else {
              prev.count = (uint8_t)std::min(255, prev.count + 1);
            }
          }
        }
  }
}

// Fusion::UnifyNeighbor and UpdateNeighborLabel, FuseMap.cu:757-896: the
// (8, 8) launch over hash entries [0, noVisible) (the kernel indexes
// hashEntries[blockIdx.x] with a grid of noVisibleBlocks, FuseMap.cu:802-808,
// :1158-1160, :1244).  One thread per (x, y) voxel column, its 4-slot
// neighbour table kept across the column's z loop (declared outside it,
// FuseMap.cu:812-816).  Every voxel updates from the pass-start state: new
// label fields go to `out` and are applied after the pass.
extern "C" void sfo_unify_neighbor(sfo_map *m) {
  const float vs = m->c.voxel_size;
  const float step = vs * (float)1;  // VoxelSize * r, r = 1 (FuseMap.cu:833)
  const unsigned n = std::min<unsigned>(m->noVisible, m->numEntries);
  // the 26 neighbours in UnifyNeighbor's order (FuseMap.cu:834-887)
  static const int8_t kOrder[26][3] = {
      {1, 0, 0},  {1, 1, 0},  {1, -1, 0},  {1, 0, 1},  {1, 0, -1},  {1, 1, 1},   {1, 1, -1},
      {1, -1, 1}, {1, -1, -1}, {-1, 0, 0}, {-1, 1, 0}, {-1, -1, 0}, {-1, 0, 1},  {-1, 0, -1},
      {-1, 1, 1}, {-1, 1, -1}, {-1, -1, 1}, {-1, -1, -1}, {0, 1, 0}, {0, 1, 1},  {0, 1, -1},
      {0, -1, 0}, {0, -1, 1},  {0, -1, -1}, {0, 0, 1},  {0, 0, -1}};
  struct Upd { size_t idx; uint8_t label, count, label_2, count_2; };
  std::vector<Upd> out;
  for (unsigned b = 0; b < n; ++b) {
    const sfo_entry &entry = m->entries[b];
    if (entry.ptr == -1) continue;
    i3 bp = {(int)((uint32_t)entry.x * 8u), (int)((uint32_t)entry.y * 8u), (int)((uint32_t)entry.z * 8u)};
    for (int ty = 0; ty < 8; ++ty)
      for (int tx = 0; tx < 8; ++tx) {
        int nl[4] = {-1, -1, -1, -1}, nc[4] = {0, 0, 0, 0}, nlc[4] = {0, 0, 0, 0};
        for (int i = 0; i < 8; ++i) {
          const size_t idx = (size_t)entry.ptr + i * 64 + ty * 8 + tx;
          const sfo_voxel &cur = m->voxels[idx];
          const int cur_label = cur.weight == 0 ? -1 : (int)cur.label;
          if (cur_label == -1) continue;
          // voxelPosToWorldPos (DeviceMap.cu:165-167): int3 * float
          const f3 pos = {(float)(bp.x + tx) * vs, (float)(bp.y + ty) * vs, (float)(bp.z + i) * vs};
          for (int k = 0; k < 26; ++k) {
            f3 np = pos;
            if (kOrder[k][0]) np.x = kOrder[k][0] > 0 ? pos.x + step : pos.x - step;
            if (kOrder[k][1]) np.y = kOrder[k][1] > 0 ? pos.y + step : pos.y - step;
            if (kOrder[k][2]) np.z = kOrder[k][2] > 0 ? pos.z + step : pos.z - step;
            // FindVoxel(float3) -> worldPosToVoxelPos (DeviceMap.cu:83-95, 156-159)
            const i3 v = floor3({np.x / vs, np.y / vs, np.z / vs});
            const sfo_entry *e = find_entry(*m, vox2block(v));
            if (!e) continue;
            const sfo_voxel &nb = m->voxels[(size_t)e->ptr + vox2local(v)];
            const int tmp_label = nb.weight == 0 ? -1 : (int)nb.label;
            if (tmp_label == -1) continue;
            for (int l = 0; l < 4; ++l) {
              if (nl[l] == tmp_label) {
                nc[l]++;
                nlc[l] = nlc[l] > (int)nb.count ? nlc[l] : (int)nb.count;
                break;
              } else if (nl[l] == -1) {
                nl[l] = tmp_label;
                nc[l] = 1;
                nlc[l] = (int)nb.count;
                break;
              }
            }
          }
          int nei_label = -1, nei_count = 0, nei_lc = 0;
          for (int j = 0; j < 4; ++j)
            if (nl[j] != -1 && nlc[j] != 0 && nc[j] > nei_count) {
              nei_label = nl[j];
              nei_count = nc[j];
              nei_lc = nlc[j];
            }
          Upd u{idx, cur.label, cur.count, cur.label_2, cur.count_2};
          if (cur_label != nei_label) {
            const int tmp = cur_label == (int)cur.label_2
                                ? (nei_lc > (int)cur.count_2 ? nei_lc : (int)cur.count_2 + 5)
                                : nei_lc;
            u.label_2 = cur.label;
            u.count_2 = cur.count;
            u.label = (uint8_t)nei_label;
            u.count = (uint8_t)tmp;
          } else {
            u.count = (uint8_t)nei_lc;
          }
          out.push_back(u);
        }
      }
  }
  for (const Upd &u : out) {
    sfo_voxel &v = m->voxels[u.idx];
    v.label = u.label; v.count = u.count; v.label_2 = u.label_2; v.count_2 = u.count_2;
  }
}

extern "C" unsigned sfo_fuse(sfo_map *m, const float *depth, const uint8_t *rgb,
                             const float *nmap, const uint8_t *mask,
                             int num_detection, int cols, int rows, const float *R,
                             const float *Rinv, const float *t, float fx, float fy,
                             float cx, float cy, int unify) {
  sfo_alloc(m, depth, cols, rows, R, t, fx, fy, cx, cy);
  unsigned n = sfo_visibility(m, R, Rinv, t, cols, rows, fx, fy, cx, cy, m->c.depth_max, m->c.depth_min);
  if (n == 0) return 0;
  sfo_integrate(m, depth, rgb, cols, rows, Rinv, t, fx, fy, cx, cy, m->c.depth_max, m->c.depth_min);
  if (num_detection > 0) {
    sfo_semantics(m, depth, rgb, nmap, mask, num_detection, cols, rows, Rinv, t, fx, fy, cx, cy,
                  m->c.depth_max, m->c.depth_min);
    if (unify) sfo_unify_neighbor(m);  // FuseMapColor, FuseMap.cu:1155-1160
  }
  return n;
}

namespace {
struct RBlock { int16_t ulx, uly, lrx, lry; float zmin, zmax; };
// Projection::projectBlock, RenderScene.cu:54-112.
bool project_block(const sfo_map &m, i3 pos, const m3 &Rinv, f3 t, float fx, float fy, float cx,
                   float cy, int zc, int zr, float dmax, float dmin, RBlock &b) {
  b.ulx = (int16_t)zc; b.uly = (int16_t)zr; b.lrx = -1; b.lry = -1;
  b.zmin = dmax; b.zmax = dmin;
  for (int corner = 0; corner < 8; ++corner) {
    i3 tmp = pos;
    tmp.x += (corner & 1) ? 1 : 0;
    tmp.y += (corner & 2) ? 1 : 0;
    tmp.z += (corner & 4) ? 1 : 0;
    f3 p3 = {(float)(int)((uint32_t)tmp.x * 8u) * m.c.voxel_size,
             (float)(int)((uint32_t)tmp.y * 8u) * m.c.voxel_size,
             (float)(int)((uint32_t)tmp.z * 8u) * m.c.voxel_size};
    p3 = mul(Rinv, p3 - t);
    if ((double)p3.z < 2e-1) continue;
    float px = (fx * p3.x / p3.z + cx) / 8.0f;
    float py = (fy * p3.y / p3.z + cy) / 8.0f;
    if ((float)b.ulx > std::floor(px)) b.ulx = (int16_t)f2i(std::floor(px));
    if ((float)b.lrx < std::ceil(px)) b.lrx = (int16_t)f2i(std::ceil(px));
    if ((float)b.uly > std::floor(py)) b.uly = (int16_t)f2i(std::floor(py));
    if ((float)b.lry < std::ceil(py)) b.lry = (int16_t)f2i(std::ceil(py));
    if (b.zmin > p3.z) b.zmin = p3.z;
    if (b.zmax < p3.z) b.zmax = p3.z;
  }
  if (b.ulx < 0) b.ulx = 0;
  if (b.uly < 0) b.uly = 0;
  if (b.lrx >= zc) b.lrx = (int16_t)(zc - 1);
  if (b.lry >= zr) b.lry = (int16_t)(zr - 1);
  if (b.ulx > b.lrx) return false;
  if (b.uly > b.lry) return false;
  if (b.zmin < dmin) b.zmin = dmin;
  if (b.zmax < dmin) return false;
  return true;
}
}  // namespace

// Projection::operator() + createRenderingBlockList + fillBlocks,
// RenderScene.cu:114-190, and CreateRenderingBlocks :210-289.  Each
// visible block lays down the tiles (y < ny, x < ny) of
// createRenderingBlockList (its x < ny bound and the un-offset lowerRight
// kept), each tile filled as fillBlocks does; blocks do not overwrite each
// other's list slots and no slot beyond the count is filled.
extern "C" int sfo_zrange(sfo_map *m, float *zmin, float *zmax, int zc, int zr,
                          float depth_max, float depth_min, const float *Rinv,
                          const float *t, float fx, float fy, float cx, float cy,
                          void *blocks_out, int max_blocks, unsigned *nblocks) {
  if (nblocks) *nblocks = 0;
  if (m->noVisible == 0) return 0;
  for (int i = 0; i < zc * zr; ++i) { zmin[i] = 100.f; zmax[i] = 0.f; }
  m3 RI = m3_from(Rinv);
  f3 tv = f3_from(t);
  unsigned total = 0;
  RBlock *out = (RBlock *)blocks_out;
  for (unsigned k = 0; k < m->noVisible; ++k) {
    const sfo_entry &e = m->visible[k];
    if (e.ptr == -1) continue;
    RBlock b;
    if (!project_block(*m, {e.x, e.y, e.z}, RI, tv, fx, fy, cx, cy, zc, zr, depth_max, depth_min, b))
      continue;
    // RenderScene.cu:147-151: dx = (float)LR.x - UL.x + 1; __float2int_ru(dx/16)
    float dx = (float)b.lrx - (float)b.ulx + 1.0f;
    float dy = (float)b.lry - (float)b.uly + 1.0f;
    int nx = f2i(std::ceil(dx / 16.0f)), ny = f2i(std::ceil(dy / 16.0f));
    unsigned required = (unsigned)(nx * ny);
    if (total + required >= m->c.max_rendering_blocks) continue;
    unsigned slot = 0;
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < ny; ++x) {
        RBlock tb;
        tb.ulx = (int16_t)(b.ulx + x * 16);
        tb.uly = (int16_t)(b.uly + y * 16);
        tb.lrx = (int16_t)(b.ulx + 16);
        tb.lry = (int16_t)(b.uly + 16);
        if (tb.lrx > b.lrx) tb.lrx = b.lrx;
        if (tb.lry > b.lry) tb.lry = b.lry;
        tb.zmin = b.zmin; tb.zmax = b.zmax;
        if (slot < required) {
          if (out && (int)(total + slot) < max_blocks) out[total + slot] = tb;
          ++slot;
        }
        for (int ty = 0; ty < 16; ++ty)
          for (int tx = 0; tx < 16; ++tx) {
            int xpos = tb.ulx + tx, ypos = tb.uly + ty;
            if (xpos > tb.lrx || xpos >= zc) continue;
            if (ypos > tb.lry || ypos >= zr) continue;
            float &a = zmin[ypos * zc + xpos];
            float &c2 = zmax[ypos * zc + xpos];
            a = std::fmin(tb.zmin, a);
            c2 = std::fmax(tb.zmax, c2);
          }
      }
    for (; slot < required; ++slot) {
      RBlock eb{1, 1, 0, 0, b.zmin, b.zmax};
      if (out && (int)(total + slot) < max_blocks) out[total + slot] = eb;
    }
    total += required;
  }
  if (nblocks) *nblocks = total;
  return total > 0;
}

namespace {
// Rendering (RenderScene.cu:291-489) with DeviceMap::FindVoxel's per-ray
// entry cache (DeviceMap.cu:116-133).  The reference's cache starts as
// HashEntry() = {pos (0,0,0), ptr -1}; a ray entering block (0,0,0) before
// any other block would read voxelBlocks[idx - 1].  Here the cache starts
// empty, so such a lookup goes to the hash table.
struct RayCache { i3 pos; int ptr; bool set; };
struct VoxelRead { float sdf; uint8_t weight; };

inline VoxelRead find_voxel(const sfo_map &m, f3 pt, RayCache &cache, bool &valid) {
  i3 p = floor3(pt);
  i3 bp = vox2block(p);
  if (cache.set && bp.x == cache.pos.x && bp.y == cache.pos.y && bp.z == cache.pos.z) {
    valid = true;
    const sfo_voxel &v = m.voxels[(size_t)cache.ptr + vox2local(p)];
    return {v.sdf, v.weight};
  }
  const sfo_entry *e = find_entry(m, bp);
  if (!e) { valid = false; return {kNaN, 0}; }
  valid = true;
  cache.pos = bp; cache.ptr = e->ptr; cache.set = true;
  const sfo_voxel &v = m.voxels[(size_t)e->ptr + vox2local(p)];
  return {v.sdf, v.weight};
}
inline float read_sdf(const sfo_map &m, f3 pt, RayCache &c, bool &valid) {
  VoxelRead v = find_voxel(m, pt, c, valid);
  if (v.weight == 0) valid = false;
  return v.sdf;
}
inline float read_sdf_interp(const sfo_map &m, f3 pt, RayCache &c, bool &valid) {
  f3 fl = {std::floor(pt.x), std::floor(pt.y), std::floor(pt.z)};
  f3 xyz = pt - fl;
  float s0, s1, r0, r1, r2, r3;
  s0 = find_voxel(m, pt, c, valid).sdf;
  s1 = find_voxel(m, pt + mk3(1, 0, 0), c, valid).sdf;
  r0 = (1.0f - xyz.x) * s0 + xyz.x * s1;
  s0 = find_voxel(m, pt + mk3(0, 1, 0), c, valid).sdf;
  s1 = find_voxel(m, pt + mk3(1, 1, 0), c, valid).sdf;
  r1 = (1.0f - xyz.x) * s0 + xyz.x * s1;
  r2 = (1.0f - xyz.y) * r0 + xyz.y * r1;
  s0 = find_voxel(m, pt + mk3(0, 0, 1), c, valid).sdf;
  s1 = find_voxel(m, pt + mk3(1, 0, 1), c, valid).sdf;
  r0 = (1.0f - xyz.x) * s0 + xyz.x * s1;
  s0 = find_voxel(m, pt + mk3(0, 1, 1), c, valid).sdf;
  s1 = find_voxel(m, pt + mk3(1, 1, 1), c, valid).sdf;
  r1 = (1.0f - xyz.x) * s0 + xyz.x * s1;
  r3 = (1.0f - xyz.y) * r0 + xyz.y * r1;
  return (1.0f - xyz.z) * r2 + xyz.z * r3;
}
inline bool read_normal(const sfo_map &m, f3 pt, RayCache &c, const m3 &Rinv, f3 &n) {
  bool valid;
  float s[6];
  const f3 offs[6] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
  for (int k = 0; k < 6; ++k) {
    s[k] = read_sdf_interp(m, pt + offs[k], c, valid);
    if (std::isnan(s[k]) || s[k] == 1.0f || !valid) return false;
  }
  n = mk3(s[0] - s[1], s[2] - s[3], s[4] - s[5]);
  n = normalised(mul(Rinv, n));
  return true;
}
}  // namespace

extern "C" void sfo_raycast(sfo_map *m, float *vmap, float *nmap, int cols, int rows,
                            const float *zmin, const float *zmax, int zc, int zr,
                            const float *R, const float *Rinv, const float *t,
                            float invfx, float invfy, float cx, float cy) {
  m3 Rv = m3_from(R), RI = m3_from(Rinv);
  f3 tv = f3_from(t);
  const float vsi = m->voxelSizeInv;
  (void)zr;
#pragma omp parallel for schedule(dynamic, 4)
  for (int y = 0; y < rows; ++y)
    for (int x = 0; x < cols; ++x) {
      float *vo = vmap + 4 * (y * cols + x), *no = nmap + 4 * (y * cols + x);
      vo[0] = vo[1] = vo[2] = vo[3] = kNaN;
      no[0] = no[1] = no[2] = no[3] = kNaN;
      int lx = f2i(std::floor((float)x / 8.0f)), ly = f2i(std::floor((float)y / 8.0f));
      float zx = zmin[ly * zc + lx], zy = zmax[ly * zc + lx];
      if ((double)zy < 1e-3 || (double)zx < 1e-3 || std::isnan(zx) || std::isnan(zy)) continue;
      float sdf = 1.0f;
      f3 p;
      p.z = zx;
      p.x = p.z * ((float)x - cx) * invfx;
      p.y = p.z * ((float)y - cy) * invfy;
      float dist_s = norm(p) * vsi;
      f3 block_s = (mul(Rv, p) + tv) * vsi;
      p.z = zy;
      p.x = p.z * ((float)x - cx) * invfx;
      p.y = p.z * ((float)y - cy) * invfy;
      float dist_e = norm(p) * vsi;
      f3 block_e = (mul(Rv, p) + tv) * vsi;
      f3 dir = normalised(block_e - block_s);
      f3 result = block_s;
      bool valid_sdf = false, found_pt = false, behind = false;
      float step, prev_sdf;
      RayCache cache{{0, 0, 0}, -1, false};
      while (dist_s < dist_e) {
        prev_sdf = sdf;
        sdf = read_sdf(*m, result, cache, valid_sdf);
        if (!valid_sdf) {
          step = 8.0f;
        } else {
          if (sdf <= 0.1f && sdf >= -0.5f) sdf = read_sdf_interp(*m, result, cache, valid_sdf);
          if (prev_sdf < 0.f && sdf >= 0.f) { behind = true; break; }
          if (prev_sdf > 0.f && sdf <= 0.f) break;
          step = 1.0f;
        }
        result = result + step * dir;
        dist_s += step;
      }
      if (behind) continue;
      if (sdf <= 0.0f) {
        step = sdf * m->stepScale;
        result = result + step * dir;
        sdf = read_sdf_interp(*m, result, cache, valid_sdf);
        step = sdf * m->stepScale;
        result = result + step * dir;
        found_pt = true;
      }
      if (found_pt) {
        f3 n;
        if (read_normal(*m, result, cache, RI, n)) {
          f3 r = mul(RI, result * m->c.voxel_size - tv);
          vo[0] = r.x; vo[1] = r.y; vo[2] = r.z; vo[3] = 1.0f;
          no[0] = n.x; no[1] = n.y; no[2] = n.z; no[3] = 1.0f;
        }
      }
    }
}

// ========================================================= marching cubes
namespace {
// Corners (0,0,0) (1,0,0) (1,1,0) (0,1,0) (0,0,1) (1,0,1) (1,1,1) (0,1,1)
// and edges (0,1) (1,2) (2,3) (3,0) (4,5) (5,6) (6,7) (7,4) (0,4) (1,5)
// (2,6) (3,7), MeshScene.cu's numbering.
const int kMcA[12] = {0, 1, 2, 3, 4, 5, 6, 7, 0, 1, 2, 3};
const int kMcB[12] = {1, 2, 3, 0, 5, 6, 7, 4, 4, 5, 6, 7};
const int kMcCorner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
struct McTab { int tri[256][16]; int nverts[256]; int edges[256]; };
// The polygons of each configuration: on every face (corners taken
// counterclockwise from outside) a segment cuts off each inside corner
// (or run of them), from the crossing that leaves it to the crossing that
// enters it; the segments chain into loops, each fanned into triangles
// from its lowest edge.  The loops are those of the classic table
// Mapping/Constant.h holds (checked by tests/test_oracle_mesh.py).
McTab mc_tables() {
  static const int face[6][4] = {{0, 3, 2, 1}, {4, 5, 6, 7}, {0, 1, 5, 4}, {3, 7, 6, 2}, {0, 4, 7, 3}, {1, 2, 6, 5}};
  McTab t;
  auto edge_of = [](int a, int b) {
    for (int e = 0; e < 12; ++e)
      if ((kMcA[e] == a && kMcB[e] == b) || (kMcA[e] == b && kMcB[e] == a)) return e;
    return -1;
  };
  for (int ci = 0; ci < 256; ++ci) {
    int nxt[12];
    for (int e = 0; e < 12; ++e) nxt[e] = -1;
    int emask = 0;
    for (const auto &f : face) {
      std::vector<std::pair<int, int>> cr;  // (edge, leaves an inside corner)
      for (int k = 0; k < 4; ++k) {
        int a = f[k], b = f[(k + 1) % 4];
        int ia = (ci >> a) & 1, ib = (ci >> b) & 1;
        if (ia != ib) cr.push_back({edge_of(a, b), ia});
      }
      for (size_t j = 0; j < cr.size(); ++j) {
        emask |= 1 << cr[j].first;
        if (cr[j].second == 0) nxt[cr[(j + 1) % cr.size()].first] = cr[j].first;
      }
    }
    t.edges[ci] = emask;
    for (int k = 0; k < 16; ++k) t.tri[ci][k] = -1;
    int used = 0, nt = 0;
    for (int s0 = 0; s0 < 12; ++s0) {
      if (nxt[s0] < 0 || ((used >> s0) & 1)) continue;
      std::vector<int> loop;
      int e = s0;
      do { loop.push_back(e); used |= 1 << e; e = nxt[e]; } while (e != s0);
      for (size_t q = 1; q + 1 < loop.size(); ++q) {
        t.tri[ci][3 * nt] = loop[0]; t.tri[ci][3 * nt + 1] = loop[q]; t.tri[ci][3 * nt + 2] = loop[q + 1];
        ++nt;
      }
    }
    t.nverts[ci] = 3 * nt;
  }
  return t;
}
}  // namespace

extern "C" void sfo_mc_tables(int *tri4096, int *nverts256, int *edges256) {
  static const McTab t = mc_tables();
  memcpy(tri4096, t.tri, sizeof(t.tri));
  memcpy(nverts256, t.nverts, sizeof(t.nverts));
  memcpy(edges256, t.edges, sizeof(t.edges));
}

// MeshEngine (Mapping/MeshScene.cu:4-297) over the allocated entries in
// table order, the cubes of a block in its (8, 8) launch order (y, x, then
// z): up to max_tri triangles into vert / norm (float[9] each per
// triangle) and col (uint8[9]).  Returns the triangle count (capped).
extern "C" unsigned sfo_mesh(sfo_map *m, unsigned max_tri, float *vert, float *nrm_out, uint8_t *col) {
  static const McTab T = mc_tables();
  const float vs = m->c.voxel_size;
  auto voxel = [&](i3 v) -> const sfo_voxel * {
    const sfo_entry *e = find_entry(*m, vox2block(v));
    return e ? &m->voxels[(size_t)e->ptr + vox2local(v)] : nullptr;
  };
  auto sdf_at = [&](i3 v) {
    const sfo_voxel *p = voxel(v);
    return p ? p->sdf : std::nanf("");
  };
  // interp (MeshScene.cu:144-152), the 1e-6 tests in double
  auto interp = [](float v1, float v2) {
    if ((double)std::fabs(0.f - v1) < 1e-6) return 0.f;
    if ((double)std::fabs(0.f - v2) < 1e-6) return 1.f;
    if ((double)std::fabs(v1 - v2) < 1e-6) return 0.f;
    return (0.f - v1) / (v2 - v1);
  };
  unsigned count = 0;
  for (const sfo_entry &ent : m->entries) {
    if (ent.ptr < 0) continue;
    for (int ty = 0; ty < 8; ++ty)
      for (int tx = 0; tx < 8; ++tx)
        for (int z = 0; z < 8; ++z) {
          const i3 pos = {ent.x * 8 + tx, ent.y * 8 + ty, ent.z * 8 + z};
          // readVertexAndColor (:115-141)
          float sdf[8];
          uint8_t c[8][3];
          bool ok = true;
          for (int k = 0; k < 8 && ok; ++k) {
            const sfo_voxel *p = voxel({pos.x + kMcCorner[k][0], pos.y + kMcCorner[k][1], pos.z + kMcCorner[k][2]});
            sdf[k] = p ? p->sdf : std::nanf("");
            for (int q = 0; q < 3; ++q) c[k][q] = p ? p->color[q] : 0;
            ok = !(sdf[k] == 1.0 || std::isnan(sdf[k]));
          }
          if (!ok) continue;
          // readNormal (:43-113): per corner, the differences to the
          // outside neighbour along x, y, z (sdf[] of the in-cube one)
          f3 n[8];
          for (int k = 0; k < 8 && ok; ++k) {
            float d[3];
            for (int ax = 0; ax < 3; ++ax) {
              const int lo = kMcCorner[k][ax] == 0;  // the neighbour outside is below
              i3 q = {pos.x + kMcCorner[k][0], pos.y + kMcCorner[k][1], pos.z + kMcCorner[k][2]};
              int other = k;
              if (ax == 0) { q.x += lo ? -1 : 1; other = k ^ 1; }
              if (ax == 1) { q.y += lo ? -1 : 1; other = (k & 4) | (3 - (k & 3)); }
              if (ax == 2) { q.z += lo ? -1 : 1; other = k ^ 4; }
              const float v = sdf_at(q);
              if (std::isnan(v)) { ok = false; break; }
              d[ax] = lo ? sdf[other] - v : v - sdf[other];
            }
            if (ok) n[k] = {d[0], d[1], d[2]};
          }
          if (!ok) continue;
          int ci = 0;
          for (int k = 0; k < 8; ++k) ci |= (sdf[k] < 0) << k;
          if (T.edges[ci] == 0 || ci <= 0) continue;
          // buildVertexList (:172-247)
          f3 vl[12], nl[12];
          uint8_t cl[12][3];
          static const float dir[12][3] = {{1, 0, 0}, {0, 1, 0}, {-1, 0, 0}, {0, -1, 0}, {1, 0, 0}, {0, 1, 0},
                                           {-1, 0, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, 1}, {0, 0, 1}, {0, 0, 1}};
          for (int e = 0; e < 12; ++e) {
            if (!((T.edges[ci] >> e) & 1)) continue;
            const int a = kMcA[e], b = kMcB[e];
            const float val = interp(sdf[a], sdf[b]);
            // pos + make_float3(o): the corner a, plus val along the edge
            // (1 - val where the edge runs backwards)
            float o[3];
            for (int ax = 0; ax < 3; ++ax) {
              const float base = (float)kMcCorner[a][ax];
              o[ax] = dir[e][ax] > 0 ? val : (dir[e][ax] < 0 ? 1.f - val : base);
            }
            vl[e] = {(float)pos.x + o[0], (float)pos.y + o[1], (float)pos.z + o[2]};
            nl[e] = n[a] + val * (n[b] - n[a]);
            // uchar3 + val * (uchar3 - uchar3): val taken as an int
            const int s = (int)val;
            for (int q = 0; q < 3; ++q)
              cl[e][q] = (uint8_t)(c[a][q] + (uint8_t)((uint8_t)(c[b][q] - c[a][q]) * s));
          }
          const int nt = T.nverts[ci] / 3;
          for (int j = 0; j < nt; ++j) {
            if (count >= max_tri) return count;
            for (int q = 0; q < 3; ++q) {
              const int e = T.tri[ci][3 * j + q];
              const f3 v = vl[e] * vs;
              const f3 nn = nl[e] / norm(nl[e]);
              float *pv = vert + 9 * (size_t)count + 3 * q, *pn = nrm_out + 9 * (size_t)count + 3 * q;
              pv[0] = v.x; pv[1] = v.y; pv[2] = v.z;
              pn[0] = nn.x; pn[1] = nn.y; pn[2] = nn.z;
              for (int r = 0; r < 3; ++r) col[9 * (size_t)count + 3 * q + r] = cl[e][r];
            }
            ++count;
          }
        }
  }
  return count;
}


// RelocScoreBatch of the GB300 loop (no reference kernel; see
// semantic_icpslam_gb300/csrc/reloc.cu): per candidate, every stride-th
// vertex moved into the map by (R | t) and read with readSdfInterped
// (RenderScene.cu:310-343).  The float sums follow the kernel's order: the
// candidate's samples over 8 CTAs of 256 threads, thread t of CTA c
// summing samples i = 256 c + t, + 2048, ...; a shuffle-down tree per warp,
// then over the eight warp sums, gives CTA c's partial; the eight partials
// are added with a shuffle-down tree (offsets 4, 2, 1).  out: n records of
// {uint32 valid, uint32 inliers, float sum, float mean}.
extern "C" void sfo_reloc_score(sfo_map *m, const float *vmap, int cols, int rows, int stride,
                                const float *poses, int n, float inlier_sdf, void *out) {
  struct Rec { uint32_t valid, inliers; float sum, mean; };
  Rec *rec = static_cast<Rec *>(out);
  const int sc = (cols + stride - 1) / stride, sr = (rows + stride - 1) / stride;
  const int N = sc * sr;
  const float vsi = m->voxelSizeInv;
  constexpr int kSplit = 8, kThreads = 256;
#pragma omp parallel for schedule(dynamic, 1)
  for (int k = 0; k < n; ++k) {
    const float *P = poses + 12 * (size_t)k;
    m3 R;
    R.rx = {P[0], P[1], P[2]};
    R.ry = {P[3], P[4], P[5]};
    R.rz = {P[6], P[7], P[8]};
    const f3 t = {P[9], P[10], P[11]};
    float psum[kSplit];
    uint32_t pvalid[kSplit], pinl[kSplit];
    for (int c = 0; c < kSplit; ++c) {
      float tsum[kThreads];
      uint32_t tvalid[kThreads], tinl[kThreads];
      for (int th = 0; th < kThreads; ++th) {
        float sum = 0.f;
        uint32_t valid = 0, inl = 0;
        RayCache cache{{0, 0, 0}, -1, false};
        for (int i = c * kThreads + th; i < N; i += kThreads * kSplit) {
          const int y = (i / sc) * stride, x = (i % sc) * stride;
          const float *v = vmap + 4 * ((size_t)y * cols + x);
          if (std::isnan(v[0])) continue;
          const f3 pt = (mul(R, f3{v[0], v[1], v[2]}) + t) * vsi;
          bool ok;
          const float sdf = read_sdf_interp(*m, pt, cache, ok);
          if (!ok || std::isnan(sdf)) continue;
          ++valid;
          const float a = std::fabs(sdf);
          if (a < inlier_sdf) ++inl;
          sum += a;
        }
        tsum[th] = sum;
        tvalid[th] = valid;
        tinl[th] = inl;
      }
      float wsum[8];
      uint32_t wvalid[8], winl[8];
      for (int w = 0; w < 8; ++w) {
        float *v = tsum + 32 * w;
        uint32_t *a = tvalid + 32 * w, *b = tinl + 32 * w;
        for (int off = 16; off > 0; off >>= 1)
          for (int l = 0; l < off; ++l) {
            v[l] = v[l] + v[l + off];
            a[l] += a[l + off];
            b[l] += b[l + off];
          }
        wsum[w] = v[0];
        wvalid[w] = a[0];
        winl[w] = b[0];
      }
      for (int off = 4; off > 0; off >>= 1)
        for (int l = 0; l < off; ++l) {
          wsum[l] = wsum[l] + wsum[l + off];
          wvalid[l] += wvalid[l + off];
          winl[l] += winl[l + off];
        }
      psum[c] = wsum[0];
      pvalid[c] = wvalid[0];
      pinl[c] = winl[0];
    }
    for (int off = kSplit / 2; off > 0; off >>= 1)
      for (int l = 0; l < off; ++l) {
        psum[l] = psum[l] + psum[l + off];
        pvalid[l] += pvalid[l + off];
        pinl[l] += pinl[l + off];
      }
    rec[k].valid = pvalid[0];
    rec[k].inliers = pinl[0];
    rec[k].sum = psum[0];
    rec[k].mean = pvalid[0] ? psum[0] / (float)pvalid[0] : std::numeric_limits<float>::quiet_NaN();
  }
}

// RaycastAdjoint's FP64 reference (test infrastructure).  For every pixel
// the float march of sfo_raycast (same samples, same decisions) fixes where
// the surface lies, and the float forward fixes the interpolation cells
// (and the raw sample's voxel), as the adjoint holds them; the smooth rest
// of the raycast is then evaluated in double from the map's float values,
// for the pose exp(xi) T (xi = (rho, omega), translation first) and with
// voxel index `vox` moved by `delta`:
//   p0 = bs + S_res dir, sample = bs + S_smp dir, sdf_c = interp(sample) or
//   the sample's voxel, p1 = p0 + ss sdf_c dir, p2 = p1 + ss interp(p1) dir,
//   v = R^T (p2 voxel - t), n = normalised(R^T g) (g from the six
//   interpolations at p2 +- e).
// Returns L = sum over rendered pixels of gv . v + gn . n, whose central
// differences in xi and in delta check the GPU adjoint.
namespace {
inline d3 dd(f3 a) { return {a.x, a.y, a.z}; }
inline d3 operator*(d3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline d3 dmul(const double *R, d3 a) {  // R row-major 3x3 in a 4x4
  return {R[0] * a.x + R[1] * a.y + R[2] * a.z, R[4] * a.x + R[5] * a.y + R[6] * a.z,
          R[8] * a.x + R[9] * a.y + R[10] * a.z};
}
inline d3 dmulT(const double *R, d3 a) {
  return {R[0] * a.x + R[4] * a.y + R[8] * a.z, R[1] * a.x + R[5] * a.y + R[9] * a.z,
          R[2] * a.x + R[6] * a.y + R[10] * a.z};
}
inline double voxel_f64(const sfo_map &m, int vx, int vy, int vz, long long vox, double delta, bool &found) {
  i3 p{vx, vy, vz};
  const sfo_entry *e = find_entry(m, vox2block(p));
  if (!e) { found = false; return std::numeric_limits<double>::quiet_NaN(); }
  found = true;
  const long long idx = (long long)e->ptr + vox2local(p);
  return (double)m.voxels[idx].sdf + (idx == vox ? delta : 0.0);
}
// Trilinear interpolation over the cell with corner `base` (fixed by the
// float march), extended linearly when pt leaves the cell.
inline double interp_f64(const sfo_map &m, d3 pt, i3 base, long long vox, double delta, bool &valid) {
  const d3 f = {pt.x - base.x, pt.y - base.y, pt.z - base.z};
  const int ax = base.x, ay = base.y, az = base.z;
  double c[8];
  bool found = true;
  for (int k = 0; k < 8; ++k)
    c[k] = voxel_f64(m, ax + (k & 1), ay + ((k >> 1) & 1), az + ((k >> 2) & 1), vox, delta, found);
  valid = found;
  const double r0 = (1 - f.x) * c[0] + f.x * c[1], r1 = (1 - f.x) * c[2] + f.x * c[3];
  const double r2 = (1 - f.y) * r0 + f.y * r1;
  const double q0 = (1 - f.x) * c[4] + f.x * c[5], q1 = (1 - f.x) * c[6] + f.x * c[7];
  const double r3 = (1 - f.y) * q0 + f.y * q1;
  return (1 - f.z) * r2 + f.z * r3;
}
}  // namespace

extern "C" double sfo_raycast_smooth_f64(sfo_map *m, const float *gv, const float *gn, int cols, int rows,
                                         const float *zmin, const float *zmax, int zc, int zr,
                                         const double *T, float invfx, float invfy, float cx, float cy,
                                         const double *xi, long long vox, double delta) {
  (void)zr;
  // the float pose of the march (Frame::GpuRotation / GpuInvRotation / GpuTranslation)
  m3 Rv, RI;
  Rv.rx = {(float)T[0], (float)T[1], (float)T[2]};
  Rv.ry = {(float)T[4], (float)T[5], (float)T[6]};
  Rv.rz = {(float)T[8], (float)T[9], (float)T[10]};
  RI.rx = {(float)T[0], (float)T[4], (float)T[8]};
  RI.ry = {(float)T[1], (float)T[5], (float)T[9]};
  RI.rz = {(float)T[2], (float)T[6], (float)T[10]};
  const f3 tv = {(float)T[3], (float)T[7], (float)T[11]};
  // the perturbed FP64 pose
  double E[16], Tx[16];
  sfo_se3_exp(xi, E);
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      double a = 0;
      for (int k = 0; k < 4; ++k) a += E[i * 4 + k] * T[k * 4 + j];
      Tx[i * 4 + j] = a;
    }
  const d3 tx = {Tx[3], Tx[7], Tx[11]};
  const float vsi = m->voxelSizeInv;
  const double vs = m->c.voxel_size, ss = m->stepScale;
  double L = 0.0;
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : L)
  for (int y = 0; y < rows; ++y)
    for (int x = 0; x < cols; ++x) {
      const float *g1 = gv + 4 * ((size_t)y * cols + x);
      const float *g2 = gn ? gn + 4 * ((size_t)y * cols + x) : nullptr;
      int lx = f2i(std::floor((float)x / 8.0f)), ly = f2i(std::floor((float)y / 8.0f));
      float zx = zmin[ly * zc + lx], zy = zmax[ly * zc + lx];
      if ((double)zy < 1e-3 || (double)zx < 1e-3 || std::isnan(zx) || std::isnan(zy)) continue;
      // the float march (sfo_raycast's loop, with the positions recorded)
      float sdf = 1.0f;
      f3 p;
      p.z = zx;
      p.x = p.z * ((float)x - cx) * invfx;
      p.y = p.z * ((float)y - cy) * invfy;
      float dist_s = norm(p) * vsi;
      const float dist0 = dist_s;
      const f3 pcs = p;
      f3 block_s = (mul(Rv, p) + tv) * vsi;
      p.z = zy;
      p.x = p.z * ((float)x - cx) * invfx;
      p.y = p.z * ((float)y - cy) * invfy;
      float dist_e = norm(p) * vsi;
      const f3 pce = p;
      f3 block_e = (mul(Rv, p) + tv) * vsi;
      f3 dir = normalised(block_e - block_s);
      f3 result = block_s;
      bool valid_sdf = false, behind = false, interp = false;
      float step, prev_sdf, s_smp = 0.f, s_res = 0.f;
      f3 sample_pos = result;
      RayCache cache{{0, 0, 0}, -1, false};
      while (dist_s < dist_e) {
        prev_sdf = sdf;
        sdf = read_sdf(*m, result, cache, valid_sdf);
        s_smp = dist_s - dist0;
        sample_pos = result;
        interp = false;
        if (!valid_sdf) {
          step = 8.0f;
        } else {
          if (sdf <= 0.1f && sdf >= -0.5f) {
            sdf = read_sdf_interp(*m, result, cache, valid_sdf);
            interp = true;
          }
          if (prev_sdf < 0.f && sdf >= 0.f) { behind = true; break; }
          if (prev_sdf > 0.f && sdf <= 0.f) break;
          step = 1.0f;
        }
        result = result + step * dir;
        dist_s += step;
      }
      s_res = dist_s - dist0;
      if (behind || !(sdf <= 0.0f)) continue;
      // the float forward: its validity (sfo_raycast) and the cells it read
      i3 cell_smp, cell_p1, cell_n[6];
      {
        f3 r1 = result + (sdf * m->stepScale) * dir;
        float s1 = read_sdf_interp(*m, r1, cache, valid_sdf);
        f3 r2 = r1 + (s1 * m->stepScale) * dir;
        f3 n;
        if (!read_normal(*m, r2, cache, RI, n)) continue;
        cell_smp = floor3(sample_pos);
        cell_p1 = floor3(r1);
        const f3 offs[6] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
        for (int k = 0; k < 6; ++k) cell_n[k] = floor3(r2 + offs[k]);
      }
      // the smooth part in double at exp(xi) T
      const d3 ws = dmul(Tx, dd(pcs)) + tx, we = dmul(Tx, dd(pce)) + tx;
      const d3 bs = ws * (double)vsi, be = we * (double)vsi;
      const d3 dv = be - bs;
      const d3 dr = dv * (1.0 / std::sqrt(ddot(dv, dv)));
      const d3 p0 = bs + dr * (double)s_res, smp = bs + dr * (double)s_smp;
      bool ok;
      double sc;
      if (interp) {
        sc = interp_f64(*m, smp, cell_smp, vox, delta, ok);
      } else {
        sc = voxel_f64(*m, cell_smp.x, cell_smp.y, cell_smp.z, vox, delta, ok);
      }
      const d3 q1 = p0 + dr * (ss * sc);
      const double s1 = interp_f64(*m, q1, cell_p1, vox, delta, ok);
      const d3 q2 = q1 + dr * (ss * s1);
      const d3 v = dmulT(Tx, q2 * vs - tx);
      double Lp = g1[0] * v.x + g1[1] * v.y + g1[2] * v.z;
      if (g2) {
        const d3 e[6] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
        double sv[6];
        for (int k = 0; k < 6; ++k) sv[k] = interp_f64(*m, q2 + e[k], cell_n[k], vox, delta, ok);
        const d3 gr = {sv[0] - sv[1], sv[2] - sv[3], sv[4] - sv[5]};
        const d3 u = dmulT(Tx, gr);
        const d3 n = u * (1.0 / std::sqrt(ddot(u, u)));
        Lp += g2[0] * n.x + g2[1] * n.y + g2[2] * n.z;
      }
      // a pixel whose double evaluation reaches an unobserved voxel (NaN
      // sdf) where the float one did not is left out
      if (std::isfinite(Lp)) L += Lp;
    }
  return L;
}

// Tracker::ValidatePose (Tracking.cc:750-790) over n candidates, one after
// another as the reference runs them.  LastFrame's maps start as the
// caller's last maps (all levels); a candidate with at least min_visible
// visible blocks ray traces into level 0 when CreateRenderingBlocks finds a
// block (else level 0 keeps what the previous candidate left), ResizeImages
// remakes the levels below, and ComputeSE3(icpOnly = true, iters, thresh)
// runs from the candidate.  out per candidate, 24 doubles: visible,
// rendered, evaluated, accepted, fail code (ComputeSE3's: 1 count / NaN,
// 2 rejected or diverged, 0 accepted), iterations, icp error, icp count,
// then the pose after ComputeSE3 (16).  Returns the first accepted
// candidate, the one ValidatePose keeps, or -1.
extern "C" int sfo_validate_pose_batch(sfo_map *m, int levels, int cols, int rows, const float *const *nv,
                                       const float *const *nn, const float *const *lv, const float *const *ln,
                                       const float *K, const double *poses, int n, const int *iters,
                                       const int *min_count, float thresh, unsigned min_visible, double *out) {
  std::vector<std::vector<float>> wv(levels), wn(levels);
  std::vector<int> cs(levels), rs(levels);
  std::vector<const float *> pv(levels), pn(levels);
  for (int l = 0; l < levels; ++l) {
    cs[l] = cols >> l;
    rs[l] = rows >> l;
    const size_t e = 4 * (size_t)cs[l] * rs[l];
    wv[l].assign(lv[l], lv[l] + e);
    wn[l].assign(ln[l], ln[l] + e);
    pv[l] = wv[l].data();
    pn[l] = wn[l].data();
  }
  const int zc = (cols + 7) / 8, zr = (rows + 7) / 8;
  std::vector<float> zmin((size_t)zc * zr), zmax((size_t)zc * zr);
  const float invfx = (float)(1.0 / (double)K[0]), invfy = (float)(1.0 / (double)K[1]);
  int chosen = -1;
  for (int c = 0; c < n; ++c) {
    const double *P = poses + 16 * (size_t)c;
    double *o = out + 24 * (size_t)c;
    for (int k = 0; k < 24; ++k) o[k] = 0.0;
    for (int k = 0; k < 16; ++k) o[8 + k] = P[k];
    float R[9], RI[9], t[3];
    pose_to_gpu(P, R, RI, t);
    const unsigned no = sfo_visibility(m, R, RI, t, cols, rows, K[0], K[1], K[2], K[3], m->c.depth_max,
                                       m->c.depth_min);
    o[0] = no;
    if (no < min_visible) continue;
    o[2] = 1;
    const int drew = sfo_zrange(m, zmin.data(), zmax.data(), zc, zr, m->c.depth_max, m->c.depth_min, RI, t, K[0],
                                K[1], K[2], K[3], nullptr, 0, nullptr);
    if (drew)
      sfo_raycast(m, wv[0].data(), wn[0].data(), cols, rows, zmin.data(), zmax.data(), zc, zr, R, RI, t, invfx,
                  invfy, K[2], K[3]);
    o[1] = drew ? 1 : 0;
    for (int l = 1; l < levels; ++l)
      sfo_resize(wv[l - 1].data(), wn[l - 1].data(), cs[l - 1], rs[l - 1], wv[l].data(), wn[l].data(), cs[l], rs[l]);
    double np[16], st[6] = {0, 0, 0, 0, 0, 0};
    memcpy(np, P, sizeof(np));
    const int ok = sfo_compute_se3_ex(levels, cs.data(), rs.data(), nv, nn, pv.data(), pn.data(), nullptr, nullptr,
                                      nullptr, nullptr, K, iters, min_count, thresh, P, np, 0, st);
    o[3] = ok;
    o[4] = st[3];
    o[5] = st[2];
    o[6] = st[0];
    o[7] = st[1];
    for (int k = 0; k < 16; ++k) o[8 + k] = np[k];
    if (ok && chosen < 0) chosen = c;
  }
  return chosen;
}

// =============================================================== whole loop
struct sfo_frame {
  std::vector<float> raw;
  std::vector<std::vector<float>> depth, vmap, nmap;
  std::vector<std::vector<uint8_t>> image;        // intensity pyramid (photometric term)
  std::vector<std::vector<int16_t>> dIdx, dIdy;   // its derivative images
  double pose[16];
};
struct sfo_system {
  sfo_map *map = nullptr;
  int cols, rows, levels;
  float K[4], depth_scale, cutoff, icp_thresh;
  std::vector<int> iters, min_count;
  sfo_frame fa, fb;
  sfo_frame *next = &fa, *last = &fb;
  int state = 1;  // the next frame's state: 1 init, 0 tracking, -1 lost (Tracking.cc:65-119)
  int prev_state = 0;  // the state the last frame ran in
  int missed = 0;      // Tracker::noMissedFrames
  std::vector<double> reloc;  // relocalisation candidates, n x 16
  int rgb = 0;    // 1: ComputeSE3(icpOnly = false), the reference's default
  int mapping = 1;  // 0: localisation mode (Tracker::mappingDisabled)
  double init_pose[16];
  std::vector<float> zmin, zmax;
  int zc, zr;
};

namespace {
void frame_alloc(sfo_frame &f, int cols, int rows, int L) {
  f.raw.assign((size_t)cols * rows, 0);
  f.depth.resize(L); f.vmap.resize(L); f.nmap.resize(L);
  f.image.resize(L); f.dIdx.resize(L); f.dIdy.resize(L);
  for (int l = 0; l < L; ++l) {
    size_t n = (size_t)(cols >> l) * (rows >> l);
    f.depth[l].assign(n, 0); f.vmap[l].assign(4 * n, 0); f.nmap[l].assign(4 * n, 0);
    f.image[l].assign(n, 0); f.dIdx[l].assign(n, 0); f.dIdy[l].assign(n, 0);
  }
}
// Frame::FillImages intensity part, Core/Frame.cc:74-84 (run only with the
// photometric term: nothing else reads it).
void fill_intensity(sfo_system *s, sfo_frame &f, const uint8_t *rgb) {
  sfo_intensity(rgb, s->cols, s->rows, f.image[0].data());
  for (int l = 1; l < s->levels; ++l)
    sfo_pyrdown_u8(f.image[l - 1].data(), s->cols >> (l - 1), s->rows >> (l - 1), f.image[l].data(),
                   s->cols >> l, s->rows >> l);
  for (int l = 0; l < s->levels; ++l)
    sfo_sobel(f.image[l].data(), s->cols >> l, s->rows >> l, f.dIdx[l].data(), f.dIdy[l].data());
}
// Frame::FillImages depth part, Core/Frame.cc:68-92.
void fill_images(sfo_system *s, sfo_frame &f, const uint16_t *d) {
  sfo_filter_depth(d, s->cols, s->rows, s->depth_scale, s->cutoff, f.raw.data(), f.depth[0].data());
  for (int l = 1; l < s->levels; ++l)
    sfo_pyrdown(f.depth[l - 1].data(), s->cols >> (l - 1), s->rows >> (l - 1), f.depth[l].data(),
                s->cols >> l, s->rows >> l);
  for (int l = 0; l < s->levels; ++l) {
    float div = (float)(1 << l);
    sfo_vmap(f.depth[l].data(), s->cols >> l, s->rows >> l, s->K[0] / div, s->K[1] / div,
             s->K[2] / div, s->K[3] / div, s->cutoff, f.vmap[l].data());
    sfo_nmap(f.vmap[l].data(), s->cols >> l, s->rows >> l, f.nmap[l].data());
  }
}
// Frame::ResizeImages, Core/Frame.cc:94-98.
void resize_images(sfo_system *s, sfo_frame &f) {
  for (int l = 1; l < s->levels; ++l)
    sfo_resize(f.vmap[l - 1].data(), f.nmap[l - 1].data(), s->cols >> (l - 1), s->rows >> (l - 1),
               f.vmap[l].data(), f.nmap[l].data(), s->cols >> l, s->rows >> l);
}
}  // namespace

extern "C" sfo_system *sfo_system_create(const sfo_config *cfg, int cols, int rows,
                                         int levels, const float *K, float depth_scale,
                                         float depth_cutoff, const int *iters,
                                         const int *min_count, float icp_thresh,
                                         const double *init_pose) {
  sfo_system *s = new sfo_system();
  s->map = sfo_map_create(cfg);
  s->cols = cols; s->rows = rows; s->levels = levels;
  memcpy(s->K, K, sizeof(s->K));
  s->depth_scale = depth_scale; s->cutoff = depth_cutoff; s->icp_thresh = icp_thresh;
  s->iters.assign(iters, iters + levels);
  s->min_count.assign(min_count, min_count + levels);
  frame_alloc(s->fa, cols, rows, levels);
  frame_alloc(s->fb, cols, rows, levels);
  for (int k = 0; k < 16; ++k) s->init_pose[k] = init_pose ? init_pose[k] : (k % 5 == 0 ? 1.0 : 0.0);
  s->zc = (cols + 7) / 8; s->zr = (rows + 7) / 8;
  s->zmin.assign((size_t)s->zc * s->zr, 0); s->zmax.assign((size_t)s->zc * s->zr, 0);
  return s;
}
extern "C" void sfo_system_destroy(sfo_system *s) { sfo_map_destroy(s->map); delete s; }
extern "C" void sfo_system_set_rgb(sfo_system *s, int on) { s->rgb = on != 0; }
extern "C" void sfo_system_set_reloc(sfo_system *s, const double *poses, int n) {
  s->reloc.assign(poses, poses + 16 * (size_t)n);
}
extern "C" void sfo_system_set_mapping(sfo_system *s, int on) { s->mapping = on != 0; }
extern "C" sfo_map *sfo_system_map(sfo_system *s) { return s->map; }
extern "C" const float *sfo_system_vmap(sfo_system *s, int l) { return s->last->vmap[l].data(); }
extern "C" const float *sfo_system_nmap(sfo_system *s, int l) { return s->last->nmap[l].data(); }

// System::GrabImage (Core/System.cc:131-270) with Tracker::GrabFrame /
// Track / TrackFrame (Tracking.cc:65-173,246-280): icp-only tracking (or
// the photometric term, sfo_system_set_rgb), no keyframes or SURF.  A
// missed frame is skipped and the next frame is tracked against the same
// model; after ten misses in a row the tracker is lost, and a lost frame
// relocalises against the candidates of sfo_system_set_reloc (Relocalise's
// ValidatePose and final ComputeSE3, Tracking.cc:107-116, 750-790; the
// candidates stand in for its SURF pose estimates).  num_detection > 0
// stands for the semantic mode's detections of this frame (gap_semantic =
// 1).
extern "C" int sfo_system_grab(sfo_system *s, const uint16_t *depth, const uint8_t *rgb,
                               const uint8_t *mask, int num_detection, double *pose_out,
                               double *stats) {
  resize_images(s, *s->last);
  fill_images(s, *s->next, depth);
  if (s->rgb) fill_intensity(s, *s->next, rgb);
  double st[6] = {0, 0, 0, 0, 0, 0};
  const int state = s->state;
  int ok = 0, relocalised = 0;
  if (state == 1) {
    memcpy(s->next->pose, s->init_pose, sizeof(s->init_pose));
    ok = 1;
  } else if (state == -1) {
    const int n = (int)(s->reloc.size() / 16);
    if (n > 0) {
      std::vector<int> it(s->levels), mc(s->levels);
      std::vector<const float *> vn(s->levels), nn(s->levels), vl(s->levels), nl(s->levels);
      for (int l = 0; l < s->levels; ++l) {
        it[l] = l < 3 ? (l < 2 ? 3 : 2) : 0;  // ITERATIONS_RELOC {3, 3, 2} (Tracking.h:111)
        mc[l] = s->min_count[l];
        vn[l] = s->next->vmap[l].data(); nn[l] = s->next->nmap[l].data();
        vl[l] = s->last->vmap[l].data(); nl[l] = s->last->nmap[l].data();
      }
      std::vector<double> out(24 * (size_t)n);
      const int chosen = sfo_validate_pose_batch(s->map, s->levels, s->cols, s->rows, vn.data(), nn.data(), vl.data(),
                                                 nl.data(), s->K, s->reloc.data(), n, it.data(), mc.data(), 1e-3f,
                                                 512u, out.data());
      if (chosen >= 0) {
        // LastFrame->pose = the kept candidate; UpdateVisibility, RayTrace,
        // ResizeImages there; ComputeSE3 from it (Tracking.cc:780-789)
        sfo_frame &l = *s->last;
        memcpy(l.pose, s->reloc.data() + 16 * (size_t)chosen, sizeof(l.pose));
        float R[9], RI[9], t[3];
        pose_to_gpu(l.pose, R, RI, t);
        sfo_visibility(s->map, R, RI, t, s->cols, s->rows, s->K[0], s->K[1], s->K[2], s->K[3], s->map->c.depth_max,
                       s->map->c.depth_min);
        if (sfo_zrange(s->map, s->zmin.data(), s->zmax.data(), s->zc, s->zr, s->map->c.depth_max, s->map->c.depth_min,
                       RI, t, s->K[0], s->K[1], s->K[2], s->K[3], nullptr, 0, nullptr))
          sfo_raycast(s->map, l.vmap[0].data(), l.nmap[0].data(), s->cols, s->rows, s->zmin.data(), s->zmax.data(),
                      s->zc, s->zr, R, RI, t, (float)(1.0 / (double)s->K[0]), (float)(1.0 / (double)s->K[1]),
                      s->K[2], s->K[3]);
        resize_images(s, l);
        memcpy(s->next->pose, l.pose, sizeof(l.pose));
        std::vector<int> cols(s->levels), rows(s->levels);
        for (int k = 0; k < s->levels; ++k) { cols[k] = s->cols >> k; rows[k] = s->rows >> k; }
        ok = sfo_compute_se3_ex(s->levels, cols.data(), rows.data(), vn.data(), nn.data(), vl.data(), nl.data(),
                                nullptr, nullptr, nullptr, nullptr, s->K, s->iters.data(), s->min_count.data(),
                                s->icp_thresh, l.pose, s->next->pose, 0, st);
      }
    }
  } else {
    memcpy(s->next->pose, s->last->pose, sizeof(s->last->pose));
    std::vector<int> cols(s->levels), rows(s->levels);
    std::vector<const float *> vn(s->levels), nn(s->levels), vl(s->levels), nl(s->levels);
    std::vector<const uint8_t *> in(s->levels), il(s->levels);
    std::vector<const int16_t *> gx(s->levels), gy(s->levels);
    for (int l = 0; l < s->levels; ++l) {
      cols[l] = s->cols >> l; rows[l] = s->rows >> l;
      vn[l] = s->next->vmap[l].data(); nn[l] = s->next->nmap[l].data();
      vl[l] = s->last->vmap[l].data(); nl[l] = s->last->nmap[l].data();
      in[l] = s->next->image[l].data(); il[l] = s->last->image[l].data();
      gx[l] = s->next->dIdx[l].data(); gy[l] = s->next->dIdy[l].data();
    }
    ok = sfo_compute_se3_ex(s->levels, cols.data(), rows.data(), vn.data(), nn.data(), vl.data(),
                            nl.data(), s->rgb ? in.data() : nullptr, il.data(), gx.data(), gy.data(), s->K,
                            s->iters.data(), s->min_count.data(), s->icp_thresh, s->last->pose,
                            s->next->pose, 0, st);
  }
  // Track()'s state machine (Tracking.cc:65-119)
  int tracked = 0, next_state = 0;
  if (state == 1) {
    tracked = 1;
  } else if (state == 0) {
    if (ok) {
      s->missed = 0;
      tracked = s->prev_state != -1;
    } else if (++s->missed > 9) {
      next_state = -1;
    }
  } else {
    tracked = ok;
    next_state = ok ? 0 : -1;
    relocalised = ok;
  }
  s->prev_state = state;
  s->state = next_state;
  if (tracked) std::swap(s->next, s->last);
  unsigned nvis = 0;
  if (tracked) {
    sfo_frame &f = *s->last;
    float R[9], RI[9], t[3];
    pose_to_gpu(f.pose, R, RI, t);
    // Mapping::RayTrace (Mapping.cc:142-161): raycast only if the z-range
    // pass produced rendering blocks; else vmap[0]/nmap[0] keep the
    // measured maps.
    auto raytrace = [&]() {
      if (sfo_zrange(s->map, s->zmin.data(), s->zmax.data(), s->zc, s->zr, s->map->c.depth_max,
                     s->map->c.depth_min, RI, t, s->K[0], s->K[1], s->K[2], s->K[3], nullptr, 0, nullptr)) {
        sfo_raycast(s->map, f.vmap[0].data(), f.nmap[0].data(), s->cols, s->rows, s->zmin.data(),
                    s->zmax.data(), s->zc, s->zr, R, RI, t, (float)(1.0 / (double)s->K[0]),
                    (float)(1.0 / (double)s->K[1]), s->K[2], s->K[3]);
      }
    };
    if (s->mapping) {
      // FuseColor on the frame as grabbed (Frame::FillImages leaves
      // numDetection 0, Core/Frame.cc:86-91), RayTrace (System.cc:163-168)
      nvis = sfo_fuse(s->map, f.raw.data(), rgb, f.nmap[0].data(), mask, 0, s->cols, s->rows, R, RI, t,
                      s->K[0], s->K[1], s->K[2], s->K[3], 1);
      raytrace();
      if (num_detection > 0) {
        // with detections, FuseColor again with the labels (its label pass
        // reading the raycast normals now in nmap[0]) and RayTrace
        // (System.cc:184-205)
        nvis = sfo_fuse(s->map, f.raw.data(), rgb, f.nmap[0].data(), mask, num_detection, s->cols, s->rows,
                        R, RI, t, s->K[0], s->K[1], s->K[2], s->K[3], 1);
        raytrace();
      }
    } else {
      // localisation: UpdateVisibility + RayTrace (System.cc:169-172)
      nvis = sfo_visibility(s->map, R, RI, t, s->cols, s->rows, s->K[0], s->K[1], s->K[2], s->K[3],
                            s->map->c.depth_max, s->map->c.depth_min);
      raytrace();
      if (num_detection > 0) {
        // Mapping::SemanticAnalysis(f) (Mapping.cc:99-123, System.cc:206-212):
        // AnalyzeMapSemantics on the rendered depth, vmap[0].z
        std::vector<float> rdepth((size_t)s->cols * s->rows);
        for (size_t i = 0; i < rdepth.size(); ++i) rdepth[i] = f.vmap[0][4 * i + 2];
        if (sfo_visibility(s->map, R, RI, t, s->cols, s->rows, s->K[0], s->K[1], s->K[2], s->K[3],
                           s->map->c.depth_max, s->map->c.depth_min) > 0) {
          sfo_semantics(s->map, rdepth.data(), rgb, f.nmap[0].data(), mask, num_detection, s->cols, s->rows, RI, t,
                        s->K[0], s->K[1], s->K[2], s->K[3], s->map->c.depth_max, s->map->c.depth_min);
          sfo_unify_neighbor(s->map);
        }
      }
    }
  }
  if (pose_out) memcpy(pose_out, s->last->pose, sizeof(s->last->pose));
  if (stats) {
    int c[4];
    sfo_map_counters(s->map, c);
    stats[0] = st[0]; stats[1] = st[1]; stats[2] = st[2]; stats[3] = st[3];
    stats[4] = nvis; stats[5] = c[0]; stats[6] = c[1]; stats[7] = c[3];
    if (s->rgb) { stats[8] = st[4]; stats[9] = st[5]; }
    stats[10] = s->state; stats[11] = s->missed; stats[12] = relocalised;
  }
  return tracked;
}
