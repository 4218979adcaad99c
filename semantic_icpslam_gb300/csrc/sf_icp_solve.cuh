// Per-iteration control, 6x6 solve and SE(3) update of the persistent ICP
// kernel, run by three warps.
//
// GB300's FP64 path is narrow: a warp has one FP64 instruction in flight
// at a time, about 64 cycles each whether the next one depends on it or
// not (conversions and compares to/from double included), and the SM
// retires one FP64 warp instruction per ~19 cycles.  Lanes are free, FP64
// instructions are not, so this form keeps the mathematics of
// sf::ctl_step (sf_solve.h), which restates Tracker::ComputeSE3
// (Tracking/Tracking.cc:449-499), with as few FP64 instructions per warp as
// it can:
//  - A x = b by Gauss-Jordan elimination of the augmented 6x7 matrix, one
//    element per thread over two warps (two schedulers issue their FP64
//    updates side by side), two FP64 instructions per element and step.  The
//    pivot order is LDLT's symmetric pivoting (largest remaining
//    |diagonal|; every uneliminated row carries the same scale, so the
//    comparison is LDLT's), a zero pivot zeroes its component as in the
//    LDLT solve, and instead of dividing, each step rescales the updated
//    rows by an exact power of two through exponent arithmetic.  The six
//    divisions x_i = b_i / a_ii run side by side.
//  - exp(x) in Rodrigues form, R = I + c_a W + c_1 W^2 and
//    t = u + c_1 (w x u) + c_2 (w x (w x u)), with c_a = sin(t)/t,
//    c_1 = (1 - cos t)/t^2, c_2 = (t - sin t)/t^3: the same rotation and
//    left Jacobian as Sophus's quaternion form.  For t < 0.1 rad the
//    coefficients are their Taylor series in x = t^2: the leading two
//    terms in FP64, the rest (below 1e-4 of the total, truncated below
//    1e-20) in FP32, which keeps each coefficient within 1e-13 absolute.
//    Larger angles take the trigonometric form.
//  - the pose as next = next * exp(-x), which equals the reference's
//    last * delta^-1 after delta = exp(x) delta (the accumulated delta is
//    not kept), as FMA chains, one matrix element per lane.
// Results agree with the host ctl_step to rounding (about 1e-15 relative
// on well-conditioned systems); they are not bit-identical.
#ifndef SF_ICP_SOLVE_CUH_
#define SF_ICP_SOLVE_CUH_

#include "sf_solve.h"

// Optional phase-clock hook (a no-op unless defined before inclusion).
#ifndef SF_SOLVE_MARK
#define SF_SOLVE_MARK(k)
#endif

namespace sf {

// Compares and conversions run on the FP64 pipe at the cost of an FP64
// operation; these integer forms take the exponent and mantissa bits
// instead.  nonneg_below: x < y for x >= 0 and finite y >= 0, as the bit
// patterns order those doubles (|x| < y for any x; NaN compares false).
__device__ __forceinline__ bool nonneg_below(double x, double y) {
  return (__double_as_longlong(x) & 0x7fffffffffffffffll) < __double_as_longlong(y);
}
// A non-negative double to float, truncating the mantissa (within one float
// ulp of the rounded conversion); values below the float normal range give 0.
__device__ __forceinline__ float nonneg_to_float_rz(double x) {
  const int hi = __double2hiint(x), lo = __double2loint(x);
  const int fe = ((hi >> 20) & 0x7ff) - 1023 + 127;
  if (fe <= 0) return 0.0f;
  if (fe >= 0xff) return __int_as_float(0x7f800000);
  return __int_as_float((fe << 23) | ((hi & 0xfffff) << 3) | (int)((unsigned)lo >> 29));
}
// A float to double, exactly, for zero and normal floats (subnormal floats
// give 0).
__device__ __forceinline__ double float_to_double_exact(float f) {
  const int b = __float_as_int(f);
  const int e = (b >> 23) & 0xff;
  if (e == 0) return 0.0;
  const int hi = (b & (int)0x80000000) | ((e - 127 + 1023) << 20) | ((b & 0x7fffff) >> 3);
  return __hiloint2double(hi, (b & 7) << 29);
}

struct IcpSolveSmem {
  double a[2][6][8];  // augmented [A | b], row stride 8, double-buffered
  int code, copy_cand;  // the stop decision of ctl_decide
  double R[9];       // rotation of exp(-x), row-major
  double delta[12];  // translation of exp(-x); the acceptance gate's relative pose
};

// v * 2^sh by exponent arithmetic on the high word (no FP64 instruction).
// Zero, subnormal, infinite and NaN inputs pass unchanged; a result below
// the normal range flushes to signed zero, one above it saturates to
// infinity.
__device__ __forceinline__ double scale_pow2(double v, int sh) {
  const int hi = __double2hiint(v), lo = __double2loint(v);
  const int e = (hi >> 20) & 0x7ff;
  const int ne = e + sh;
  int rhi = hi + (sh << 20), rlo = lo;
  if (ne <= 0) { rhi = hi & (int)0x80000000; rlo = 0; }
  if (ne >= 0x7ff) { rhi = (hi & (int)0x80000000) | 0x7ff00000; rlo = 0; }
  if (e == 0 || e == 0x7ff) { rhi = hi; rlo = lo; }
  return __hiloint2double(rhi, rlo);
}

// Solves A x = b for the 27 upper-triangle sums of CreateMatrix<6,7>
// (Tracking/Reduction.cu:6-16), run by threads 0..63 (two warps, named
// barrier 1); warp 0 returns x[0..5] in every lane.  Thread e < 42 owns
// element e = 7 i + j of the row-major augmented matrix, keeps it in a
// register and publishes it in s.a[buffer], double-buffered so that one
// barrier per step separates a step's reads from the next step's writes;
// the two warps' FP64 updates run on different schedulers side by side.
// The pivot is found with one warp max over keys made of the top 28 bits
// of |a_ii| (exponent and 17 mantissa bits) and 7 - i in the low 3 bits:
// diagonals within 2^-17 of each other count as equal and the lower index
// wins, as on an exact tie.
__device__ __forceinline__ void solve6_two_warps(const double *sums, double x[6], IcpSolveSmem &s) {
  const int lane = threadIdx.x & 31, e = threadIdx.x;
  auto sum_at = [&](int i, int j) {
    const int r = i < j ? i : j, q = i < j ? j : i;
    return j == 6 ? sums[7 * i - i * (i - 1) / 2 + (6 - i)] : sums[7 * r - r * (r - 1) / 2 + (q - r)];
  };
  const bool has = e < 42;
  const int i0 = has ? e / 7 : 5, j0 = has ? e - 7 * (e / 7) : 6;
  double r = has ? sum_at(i0, j0) : 0.0;
  if (has) s.a[0][i0][j0] = r;
  asm volatile("bar.sync 1, 64;" ::: "memory");
  unsigned done = 0, zero = 0;
  int cur = 0;
#pragma unroll 1
  for (int step = 0; step < 6; ++step) {
    const double(*A)[8] = s.a[cur];
    unsigned key = 0;
    if (lane < 6 && !((done >> lane) & 1u)) {
      const unsigned hi = (unsigned)__double2hiint(A[lane][lane]) & 0x7fffffffu;
      key = hi < 0x00100000u ? 0u : ((hi & ~7u) | (7u - lane));  // zero / subnormal: no pivot
    }
    const unsigned best = __reduce_max_sync(0xffffffffu, key);
    if (best == 0) {  // every remaining pivot is zero: those components are 0
      zero = 0x3fu & ~done;
      break;
    }
    const int k = 7 - (int)(best & 7u);
    done |= 1u << k;
    const double akk = A[k][k];
    const int ek = (__double2hiint(akk) >> 20) & 0x7ff;
    const int sh = 1023 - ek;  // |akk| * 2^sh in [1, 2)
    const double aik = A[i0][k], akj = A[k][j0];
    const double u = fma(akk, r, -(aik * akj));
    r = (i0 == k) ? r : ((j0 == k) ? 0.0 : scale_pow2(u, sh));
    cur ^= 1;
    if (has) s.a[cur][i0][j0] = r;
    asm volatile("bar.sync 1, 64;" ::: "memory");
  }
  // x_i = b_i / a_ii, the six divisions side by side in lanes 0..5 (of both warps)
  const int row = lane < 6 ? lane : 0;
  const double xi = ((zero >> row) & 1u) ? 0.0 : s.a[cur][row][6] / s.a[cur][row][row];
#pragma unroll
  for (int i = 0; i < 6; ++i) x[i] = __shfl_sync(0xffffffffu, xi, i);
}

// Tracker::ComputeSE3's per-iteration bookkeeping (Tracking.cc:449-479) for
// one lane: the residual and inlier count, the stop tests and the
// break-count / candidate logic.  Returns 0 to go on, 1 to stop on too few
// inliers or a NaN error (next = last), 2 to stop on three rises in a row
// (next = the candidate); *copy_cand asks for the current pose to become
// the candidate first.
__device__ __forceinline__ int ctl_decide(TrackCtl &c, const double *sums, int min_count, int *copy_cand,
                                          const double *rsums) {
  int code = 0;
  *copy_cand = 0;
  c.iters_run++;
  if (rsums) {  // RGBStep's error and count first (Tracking.cc:421-431)
    const float r0 = (float)rsums[27], r1 = (float)rsums[28];
    c.rgbError = sqrtf(r0) / r1;
    c.rgbCount = (int)r1;
    if (isnan(c.rgbError) || c.rgbCount < min_count) {
      c.stop = 1;
      return 1;
    }
  }
  float residual0 = (float)sums[27], residual1 = (float)sums[28];
  c.icpError = sqrtf(residual0) / residual1;
  c.icpCount = (int)residual1;
  if (isnan(c.icpError) || c.icpCount < min_count) {
    c.stop = 1;
    code = 1;
  } else {
    const float wgt = 1e-4f;
    float currError = c.rgbError * wgt + c.icpError;
    if (c.lastError < currError) {
      c.breakCount++;
      *copy_cand = (c.breakCount == 1);
      c.candidateICP = c.icpError;  // outside the inner if (Tracking.cc:463-465)
    } else {
      c.breakCount = 0;
    }
    if (c.breakCount > 2) {
      c.icpError = c.candidateICP;
      c.stop = 2;
      code = 2;
    } else {
      c.lastError = currError;
    }
  }
  return code;
}

// One iteration given the 29 sums in shared memory, run by threads 0..95
// (three warps): lane 0 of warp 2 takes the stop decision while warps 0
// and 1 solve and build exp(-x) (rotation on warp 0, translation on warp
// 1), so the three overlap; after named barrier 2, warp 0 applies the
// decision (or the update).  Same contract and state transitions as
// sf::ctl_step; warp 0 returns whether to go on.  With the photometric
// term, sums[0..26] already hold the combined system and rsums the RGB
// sums (for its error and count).
__device__ __noinline__ bool ctl_step_fast(TrackCtl &c, const double *sums, int min_count, IcpSolveSmem &s,
                              const double *rsums = nullptr) {
  const int lane = threadIdx.x & 31;
  if (threadIdx.x >= 64) {  // warp 2
    if (lane == 0) s.code = ctl_decide(c, sums, min_count, &s.copy_cand, rsums);
    asm volatile("bar.sync 2, 96;" ::: "memory");
    return false;
  }
  SF_SOLVE_MARK(0);
  SF_SOLVE_MARK(1);
  double x[6];
  solve6_two_warps(sums, x, s);
  // Warp 0 builds exp(-x)'s rotation, warp 1 its translation, side by side.
  const bool tw = threadIdx.x >= 32;  // the translation warp
  const double u0 = x[0], u1 = x[1], u2 = x[2];
  const double w0 = x[3], w1 = x[4], w2 = x[5];
  const double th2 = fma(w2, w2, fma(w1, w1, w0 * w0));
  const bool tiny = nonneg_below(th2, 1e-20);  // below 1e-10 rad Sophus's V is R
  double ca = 0.0, c1, c2 = 0.0;
  if (nonneg_below(th2, 0.01)) {
    // sin t / t = 1 - x/6 + x^2/120 - ..., (1 - cos t)/t^2 = 1/2 - x/24 + ...,
    // (t - sin t)/t^3 = 1/6 - x/120 + ..., x = t^2
    const float xf = nonneg_to_float_rz(th2);
    const float c1_tail = xf * (1.f / 720 + xf * (-1.f / 40320 + xf * (1.f / 3628800 + xf * (-1.f / 479001600))));
    c1 = fma(th2, -1.0 / 24 + float_to_double_exact(c1_tail), 0.5);
    if (!tw || tiny) {
      const float ca_tail = xf * (1.f / 120 + xf * (-1.f / 5040 + xf * (1.f / 362880 + xf * (-1.f / 39916800))));
      ca = fma(th2, -1.0 / 6 + float_to_double_exact(ca_tail), 1.0);
    }
    if (tw && !tiny) {
      const float c2_tail =
          xf * (1.f / 5040 + xf * (-1.f / 362880 + xf * (1.f / 39916800 + xf * (-1.f / 6227020800.f))));
      c2 = fma(th2, -1.0 / 120 + float_to_double_exact(c2_tail), 1.0 / 6);
    }
  } else {
    const double th = sqrt(th2);
    double v = 0.0;
    if (lane == 0) v = sin(th);
    if (lane == 1) v = cos(th);
    const double sn = __shfl_sync(0xffffffffu, v, 0), cs = __shfl_sync(0xffffffffu, v, 1);
    c1 = (1 - cs) / th2;
    if (tw)
      c2 = (th - sn) / (th2 * th);
    else
      ca = sn / th;
  }
  SF_SOLVE_MARK(3);
  // next = last * (exp(x) delta)^-1 = next * exp(x)^-1 = next * exp(-x):
  // exp(-x) = [R^T | t'] with R^T_ij = R_ji = delta_ij - c_a W_ij +
  // c_1 (w_i w_j - delta_ij t^2) (W = [w]x: W01 = -w2, W02 = w1, W12 = -w0,
  // W^T = -W) in lanes 0..8 of warp 0, and t' = -(u - c_1 (w x u) +
  // c_2 (w x (w x u))) (t' = -R^T u below 1e-10 rad) in lanes 0..2 of warp 1.
  auto rot_t = [&]() {  // R^T_ij for lane 3 i + j (lanes 0..8)
    const int i = lane < 9 ? lane / 3 : 0, j = lane < 9 ? lane - 3 * (lane / 3) : 0;
    const int kk = 3 - i - j;  // the third axis when i != j
    const double wi = i == 0 ? w0 : (i == 1 ? w1 : w2);
    const double wj = j == 0 ? w0 : (j == 1 ? w1 : w2);
    const double wk = kk == 0 ? w0 : (kk == 1 ? w1 : w2);
    const bool cyc = (j == i + 1) || (i == 2 && j == 0);
    const double Wij = (i == j) ? 0.0 : (cyc ? -wk : wk);
    const double dl = (i == j) ? 1.0 : 0.0;
    const double w2ij = fma(-dl, th2, wi * wj);
    return fma(c1, w2ij, fma(-ca, Wij, dl));
  };
  if (!tw) {
    const double r = rot_t();
    if (lane < 9) s.R[lane] = r;  // R^T, row-major
  } else {
    double ti;
    const int ci = lane < 3 ? lane : 0;
    if (tiny) {
      const double r = rot_t();
      ti = -(__shfl_sync(0xffffffffu, r, ci * 3 + 0) * u0);
      ti = fma(-__shfl_sync(0xffffffffu, r, ci * 3 + 1), u1, ti);
      ti = fma(-__shfl_sync(0xffffffffu, r, ci * 3 + 2), u2, ti);
    } else {
      // (cj, ck): the next two axes after ci, cyclically
      const int cj = ci == 2 ? 0 : ci + 1, ck = ci == 0 ? 2 : ci - 1;
      const double wj = cj == 0 ? w0 : (cj == 1 ? w1 : w2), wk = ck == 0 ? w0 : (ck == 1 ? w1 : w2);
      const double uj = cj == 0 ? u0 : (cj == 1 ? u1 : u2), uk = ck == 0 ? u0 : (ck == 1 ? u1 : u2);
      const double ui = ci == 0 ? u0 : (ci == 1 ? u1 : u2);
      const double a = fma(wj, uk, -(wk * uj));  // (w x u)_i
      const double aj = __shfl_sync(0xffffffffu, a, cj), ak = __shfl_sync(0xffffffffu, a, ck);
      const double b = fma(wj, ak, -(wk * aj));  // (w x (w x u))_i
      ti = fma(-c2, b, fma(c1, a, -ui));
    }
    if (lane < 3) s.delta[lane] = ti;  // t'
  }
  asm volatile("bar.sync 2, 96;" ::: "memory");
  if (tw) return false;
  {
    const int code = s.code;
    if (s.copy_cand && lane < 16) c.candidate[lane] = c.next_pose[lane];
    __syncwarp();
    if (code == 1) {
      if (lane < 16) c.next_pose[lane] = c.last_pose[lane];
      __syncwarp();
      return false;
    }
    if (code == 2) {
      if (lane < 16) c.next_pose[lane] = c.candidate[lane];
      __syncwarp();
      return false;
    }
  }
  SF_SOLVE_MARK(4);
  // next_ij = sum_k next_ik exp(-x)_kj, lanes 0..11 (the bottom row stays)
  double v = 0.0;
  if (lane < 12) {
    const int i = lane >> 2, j = lane & 3;
    const double *N = c.next_pose;
    if (j < 3) {
      v = N[i * 4 + 0] * s.R[0 * 3 + j];
      v = fma(N[i * 4 + 1], s.R[1 * 3 + j], v);
      v = fma(N[i * 4 + 2], s.R[2 * 3 + j], v);
    } else {
      v = fma(N[i * 4 + 0], s.delta[0], N[i * 4 + 3]);
      v = fma(N[i * 4 + 1], s.delta[1], v);
      v = fma(N[i * 4 + 2], s.delta[2], v);
    }
  }
  __syncwarp();
  if (lane < 12) c.next_pose[lane] = v;
  __syncwarp();
  SF_SOLVE_MARK(5);
  return true;
}

// Acceptance gate of sf::ctl_finish (Tracking.cc:505-516) for one warp.
// p = start^-1 * next = [S^T N, S^T (t_next - t_start)], one element per
// lane.  |sin| of the three Euler angles (eulerAngles(0, 1, 2)) comes from
// the matrix entries instead of asin / atan2 / sin: sin b = r02,
// |sin a| = |r12| / |(r12, r22)|, |sin c| = |r01| / |(r00, r01)|, the same
// for both of Eigen's solution branches.
__device__ __noinline__ void ctl_finish_fast(TrackCtl &c, float thresh, IcpSolveSmem &s) {
  const int lane = threadIdx.x & 31;
  if (c.stop == 1) {
    if (lane == 0) c.accepted = 0;
    __syncwarp();
    return;
  }
  if (lane < 12) {
    const int i = lane >> 2, j = lane & 3;
    const double *S = c.start_pose, *N = c.next_pose;
    double v;
    if (j < 3) {
      v = S[0 * 4 + i] * N[0 * 4 + j];
      v = fma(S[1 * 4 + i], N[1 * 4 + j], v);
      v = fma(S[2 * 4 + i], N[2 * 4 + j], v);
    } else {
      v = S[0 * 4 + i] * (N[3] - S[3]);
      v = fma(S[1 * 4 + i], N[7] - S[7], v);
      v = fma(S[2 * 4 + i], N[11] - S[11], v);
    }
    s.delta[lane] = v;
  }
  __syncwarp();
  int accepted = 0;
  if (lane == 0) {
    const double *p = s.delta;
    const double tn = sqrt(p[3] * p[3] + p[7] * p[7] + p[11] * p[11]);
    const double r02 = p[2] < -1.0 ? -1.0 : (p[2] > 1.0 ? 1.0 : p[2]);
    const double ha = p[6] * p[6] + p[10] * p[10], hc = p[0] * p[0] + p[1] * p[1];
    const double sa2 = ha > 0.0 ? (p[6] * p[6]) / ha : 0.0;
    const double sc2 = hc > 0.0 ? (p[1] * p[1]) / hc : 0.0;
    const double an = sqrt(sa2 + r02 * r02 + sc2);
    accepted = (c.icpError < thresh) && (an <= 0.1 && tn <= 0.1);
    c.accepted = accepted;
  }
  accepted = __shfl_sync(0xffffffffu, accepted, 0);
  if (!accepted && lane < 16) c.next_pose[lane] = c.last_pose[lane];
  __syncwarp();
}

}  // namespace sf
#endif
