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
// (FP32 per-pixel, compensated FP32 warp trees, FP64 block total), writes one
// FP64 partial per component, and crosses a bounded grid barrier; then every
// CTA sums the partials in FP64 in the same fixed order and runs the same
// 6x6 LDLT solve and SE(3) update, so all CTAs hold the same pose without a
// second barrier.  Partials are double-buffered by iteration parity.
#include <mutex>

#include "sf_kernels.cuh"
#include "sf_solve_warp.cuh"

namespace sf {

namespace {

constexpr int kThreads = 512;
constexpr int kProfIters = 64;
constexpr int kWarps = kThreads / 32;

struct PoseF {
  m3 Rc, Rl, RlI;
  f3 tc, tl;
};

// Frame::GpuRotation / GpuInvRotation / GpuTranslation (Core/Frame.cc:626-645).
__host__ __device__ inline void pose_to_float(const double *P, m3 &R, m3 &Rinv, f3 &t) {
  R.rx.x = (float)P[0]; R.rx.y = (float)P[1]; R.rx.z = (float)P[2];
  R.ry.x = (float)P[4]; R.ry.y = (float)P[5]; R.ry.z = (float)P[6];
  R.rz.x = (float)P[8]; R.rz.y = (float)P[9]; R.rz.z = (float)P[10];
  Rinv.rx.x = (float)P[0]; Rinv.rx.y = (float)P[4]; Rinv.rx.z = (float)P[8];
  Rinv.ry.x = (float)P[1]; Rinv.ry.y = (float)P[5]; Rinv.ry.z = (float)P[9];
  Rinv.rz.x = (float)P[2]; Rinv.rz.y = (float)P[6]; Rinv.rz.z = (float)P[10];
  t.x = (float)P[3]; t.y = (float)P[7]; t.z = (float)P[11];
}

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

// ICPReduce::searchPoint + getRow (Reduction.cu:228-279).
__device__ __forceinline__ bool icp_row(const IcpLevelArgs &L, int x, int y, const PoseF &p,
                                        float row[7]) {
  float4 vc4 = __ldg(row_ptr<const float4>(L.vc, y) + x);
  f3 vcurr_c = xyz(vc4);
  if (isnan(vcurr_c.x) || (double)vcurr_c.z < 1e-3) return false;
  f3 vcurr_g = mul(p.Rc, vcurr_c) + p.tc;
  f3 vcurr_p = mul(p.RlI, vcurr_g - p.tl);
  // (float)(1.0 / (double)z): double rounding is innocuous for division,
  // so this equals the correctly rounded float quotient.
  float invz = __fdiv_rn(1.0f, vcurr_p.z);
  int u = round_half_up(vcurr_p.x * invz * L.fx + L.cx);
  int v = round_half_up(vcurr_p.y * invz * L.fy + L.cy);
  if (u < 0 || v < 0 || u >= L.vc.cols || v >= L.vc.rows) return false;
  float4 vl4 = __ldg(row_ptr<const float4>(L.vl, v) + u);
  float4 nl4 = __ldg(row_ptr<const float4>(L.nl, v) + u);
  float4 nc4 = __ldg(row_ptr<const float4>(L.nc, y) + x);
  f3 vlast_g = mul(p.Rl, xyz(vl4)) + p.tl;
  f3 ncurr_g = mul(p.Rc, xyz(nc4));
  f3 nlast_g = mul(p.Rl, xyz(nl4));
  float dist = norm(vlast_g - vcurr_g);
  float sine = norm(cross(ncurr_g, nlast_g));
  if (!(sine < 0.6f && dist <= 0.1f && !isnan(nc4.x) && !isnan(nl4.x))) return false;
  f3 nlast = mul(p.RlI, nlast_g);
  f3 vcurr = mul(p.RlI, vcurr_g - p.tl);
  f3 vlast = mul(p.RlI, vlast_g - p.tl);
  f3 mn = -nlast;
  f3 cr = cross(nlast, vlast);
  row[0] = mn.x; row[1] = mn.y; row[2] = mn.z;
  row[3] = cr.x; row[4] = cr.y; row[5] = cr.z;
  row[6] = dot(mn, vcurr - vlast);
  return true;
}

// Accumulates the 29 terms (Reduction.cu:281-289) of this thread's pixels.
__device__ __forceinline__ void icp_accumulate(const IcpLevelArgs &L, const PoseF &p, int gtid,
                                               int gstride, float acc[29]) {
#pragma unroll
  for (int k = 0; k < 29; ++k) acc[k] = 0.f;
  const int N = L.vc.cols * L.vc.rows;
  for (int i = gtid; i < N; i += gstride) {
    const int y = i / L.vc.cols;
    const int x = i - y * L.vc.cols;
    float row[7];
    if (!icp_row(L, x, y, p, row)) continue;
    int k = 0;
#pragma unroll
    for (int a = 0; a < 7; ++a)
#pragma unroll
      for (int b = a; b < 7; ++b) acc[k++] += row[a] * row[b];
    acc[28] += 1.0f;
  }
}

// Compensated warp tree: Knuth's TwoSum at every level, errors carried in a
// second float; lane 0 ends with (sum, err).
__device__ __forceinline__ void warp_reduce_comp(float &s, float &e) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    float s2 = __shfl_down_sync(0xffffffffu, s, off);
    float e2 = __shfl_down_sync(0xffffffffu, e, off);
    float t = s + s2;
    float bb = t - s;
    float err = (s - (t - bb)) + (s2 - bb);
    s = t;
    e = e + e2 + err;
  }
}

// Block total of the 29 terms as doubles in smem out[29].
__device__ __forceinline__ void block_reduce29(float acc[29], float2 (*wpart)[29], double *out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 29; ++k) {
    float s = acc[k], e = 0.f;
    warp_reduce_comp(s, e);
    if (lane == 0) wpart[warp][k] = make_float2(s, e);
  }
  __syncthreads();
  if (threadIdx.x < 29) {
    double t = 0.0;
    for (int w = 0; w < kWarps; ++w) t += (double)wpart[w][threadIdx.x].x + (double)wpart[w][threadIdx.x].y;
    out[threadIdx.x] = t;
  }
  __syncthreads();
}

// Bounded sense-reversing grid barrier.  All CTAs are co-resident (the
// kernel is launched cooperatively); the spin still gives up after a fixed
// number of polls and records SF_FLAG_BARRIER_TIMEOUT.
__device__ __forceinline__ void grid_barrier(unsigned *bar, unsigned nblocks, uint32_t *flags) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned *gen = bar + 1;
    unsigned g = *gen;
    __threadfence();
    unsigned arrived = atomicAdd(bar, 1u);
    if (arrived == nblocks - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      unsigned polls = 0;
      while (*gen == g) {
        if (++polls > (1u << 22)) {
          atomicOr(flags, SF_FLAG_BARRIER_TIMEOUT);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
}

// Sum of partials[29][nb] per component in FP64, fixed order: warp w sums
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

struct PersistentArgs {
  IcpLevelArgs lv[kMaxLevels];
  int levels;
  float thresh;
  double *partials;  // [2][29][max_blocks]
  int stride;        // max_blocks
  unsigned *barrier;
  TrackCtl *ctl;
  const double *last_pose;
  const int *run_flag;
  uint32_t *flags;
  unsigned long long *prof;  // optional per-iteration phase clocks of CTA 0
};

// Phase clock of CTA 0 (SM cycles): 0 iteration start, 1 pixels
// accumulated, 2 block total written, 3 grid barrier passed, 4 cross-block
// sum done, 5 solve done.
__device__ __forceinline__ void prof_mark(const PersistentArgs &a, int it, int k) {
  if (a.prof && blockIdx.x == 0 && threadIdx.x == 0 && it < kProfIters) a.prof[it * 8 + k] = clock64();
}

__global__ void __launch_bounds__(kThreads) k_icp_persistent(PersistentArgs a) {
  __shared__ TrackCtl ctl;
  __shared__ WarpSolveScratch wsolve;
  __shared__ PoseF pose;
  __shared__ double bsum[29];
  __shared__ double sums[29];
  __shared__ float2 wpart[kWarps][29];
  if (a.run_flag && *a.run_flag == 0) return;  // uniform across the grid
  if (threadIdx.x == 0) ctl_begin(ctl, a.last_pose);
  __syncthreads();
  const int nb = gridDim.x;
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const int gstride = nb * blockDim.x;
  int buf = 0, it = 0;
  for (int l = a.levels - 1; l >= 0; --l) {
    const IcpLevelArgs &L = a.lv[l];
    for (int j = 0; j < L.iters; ++j, ++it) {
      prof_mark(a, it, 0);
      if (threadIdx.x == 0) {
        m3 dummy;
        pose_to_float(ctl.next_pose, pose.Rc, dummy, pose.tc);
        pose_to_float(ctl.last_pose, pose.Rl, pose.RlI, pose.tl);
      }
      __syncthreads();
      float acc[29];
      icp_accumulate(L, pose, gtid, gstride, acc);
      prof_mark(a, it, 1);
      block_reduce29(acc, wpart, bsum);
      double *part = a.partials + (size_t)buf * 29 * a.stride;
      if (threadIdx.x < 29) part[(size_t)threadIdx.x * a.stride + blockIdx.x] = bsum[threadIdx.x];
      prof_mark(a, it, 2);
      grid_barrier(a.barrier, nb, a.flags);
      prof_mark(a, it, 3);
      cross_block_sum(part, nb, a.stride, sums);
      prof_mark(a, it, 4);
      if (threadIdx.x < 32) ctl_step_warp(ctl, sums, L.min_count, wsolve);
      __syncthreads();
      prof_mark(a, it, 5);
      buf ^= 1;
      if (ctl.stop) break;
    }
    if (ctl.stop) break;
  }
  if (threadIdx.x == 0) {
    ctl_finish(ctl, a.thresh);
    if (blockIdx.x == 0) *a.ctl = ctl;
  }
}

// Plain form, launch 1: per-CTA FP64 partials.
__global__ void __launch_bounds__(kThreads) k_icp_partials(IcpLevelArgs L, PoseF p, double *part,
                                                           int stride) {
  __shared__ double bsum[29];
  __shared__ float2 wpart[kWarps][29];
  float acc[29];
  icp_accumulate(L, p, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x, acc);
  block_reduce29(acc, wpart, bsum);
  if (threadIdx.x < 29) part[(size_t)threadIdx.x * stride + blockIdx.x] = bsum[threadIdx.x];
}

// Plain form, launch 2: FP64 sum of the partials (Reduce<float,29>).
__global__ void __launch_bounds__(kThreads) k_icp_reduce(const double *part, int nb, int stride,
                                                         double *out) {
  __shared__ double sums[29];
  cross_block_sum(part, nb, stride, sums);
  if (threadIdx.x < 29) out[threadIdx.x] = sums[threadIdx.x];
}

}  // namespace

int icp_workspace_init(IcpWorkspace &w) {
  int dev = 0, sms = 0, per_sm = 0, coop = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return SF_ERR_CUDA;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_icp_persistent, kThreads, 0) !=
      cudaSuccess)
    return SF_ERR_CUDA;
  if (per_sm < 1 || !coop) return SF_ERR_CUDA;
  w.max_blocks = sms * per_sm;
  w.threads = kThreads;
  if (cudaMalloc(&w.partials, sizeof(double) * 2 * 29 * (size_t)w.max_blocks) != cudaSuccess) return SF_ERR_CUDA;
  if (cudaMalloc(&w.sums, sizeof(double) * 29) != cudaSuccess) return SF_ERR_CUDA;
  if (cudaMalloc(&w.barrier, sizeof(unsigned) * 2) != cudaSuccess) return SF_ERR_CUDA;
  if (cudaMemset(w.barrier, 0, sizeof(unsigned) * 2) != cudaSuccess) return SF_ERR_CUDA;
  if (cudaMalloc(&w.ctl, sizeof(TrackCtl)) != cudaSuccess) return SF_ERR_CUDA;
  if (cudaMalloc(&w.prof, sizeof(unsigned long long) * 8 * kProfIters) != cudaSuccess) return SF_ERR_CUDA;
  if (cudaMemset(w.prof, 0, sizeof(unsigned long long) * 8 * kProfIters) != cudaSuccess) return SF_ERR_CUDA;
  return SF_OK;
}

void icp_workspace_free(IcpWorkspace &w) {
  cudaFree(w.partials);
  cudaFree(w.sums);
  cudaFree(w.barrier);
  cudaFree(w.ctl);
  cudaFree(w.prof);
  w = IcpWorkspace();
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
                                  float thresh, const double *last_pose, const int *run_flag,
                                  uint32_t *flags, cudaStream_t s) {
  PersistentArgs a;
  for (int l = 0; l < nlevels && l < kMaxLevels; ++l) a.lv[l] = levels[l];
  a.levels = nlevels;
  a.thresh = thresh;
  a.partials = w.partials;
  a.stride = w.max_blocks;
  a.barrier = w.barrier;
  a.ctl = w.ctl;
  a.last_pose = last_pose;
  a.run_flag = run_flag;
  a.flags = flags;
  a.prof = w.profile ? w.prof : nullptr;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(w.max_blocks);
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  note_launch();
  return cudaLaunchKernelEx(&cfg, k_icp_persistent, a);
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
    if (cudaGetSymbolAddress((void **)&p, g_icp_static) != cudaSuccess || !p) return SF_ERR_CUDA;
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
  k_icp_partials<<<nb, kThreads, 0, s>>>(L, p, scratch, kStaticMaxCtas); note_launch();
  k_icp_reduce<<<1, kThreads, 0, s>>>(scratch, nb, kStaticMaxCtas, sums_dev); note_launch();
  if (cudaGetLastError() != cudaSuccess) return SF_ERR_CUDA;
  double sums[29];
  if (cudaMemcpyAsync(sums, sums_dev, sizeof(sums), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return SF_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return SF_ERR_CUDA;
  create_matrix(sums, matrixA, vectorB);
  residual[0] = (float)sums[27];
  residual[1] = (float)sums[28];
  return SF_OK;
}
