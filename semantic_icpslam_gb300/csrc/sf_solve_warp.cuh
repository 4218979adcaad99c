// Warp-parallel form of sf::ctl_step (sf_solve.h) for the persistent ICP
// kernel: the FP64 6x6 LDLT solve, SE(3) exponential and pose products
// spread over the 32 lanes of one warp.  Every matrix element is computed
// with the same operations in the same order as the serial version, so the
// result is bit-identical to ctl_step on the host; only independent
// elements run side by side.  GB300's FP64 pipe is narrow and deep, so the
// serial chain (about 1500 dependent FP64 operations) is the cost this
// removes.
#ifndef SF_SOLVE_WARP_CUH_
#define SF_SOLVE_WARP_CUH_

#include "sf_solve.h"

namespace sf {

struct WarpSolveScratch {
  double a[36], b[6], y[6], d[6], l[6], x[6];
  double R[9], W[9], V[9], dT[16], tmp[16], dInv[16];
  double sc[4];  // sin(th/2), cos(th/2), cos(th), sin(th)
  int perm[6];
  int piv;
};

// start index of row i of the 27 upper-triangle sums (CreateMatrix<6,7>)
__device__ __forceinline__ int tri_start(int i) { return 7 * i - i * (i - 1) / 2; }

// mat4 product C = A * B with the serial summation order (k ascending).
__device__ __forceinline__ void warp_mat4_mul(const double *A, const double *B, double *C, int lane) {
  if (lane < 16) {
    const int i = lane >> 2, j = lane & 3;
    double s = 0;
    for (int k = 0; k < 4; ++k) s += A[i * 4 + k] * B[k * 4 + j];
    C[lane] = s;
  }
  __syncwarp();
}

// All 32 lanes of the calling warp; c, sums and w in shared memory.
// Returns true if the loop continues (same contract as ctl_step).
__device__ bool ctl_step_warp(TrackCtl &c, const double *sums, int min_count, WarpSolveScratch &w) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  int code = 0, copy_cand = 0;
  if (lane == 0) {
    c.iters_run++;
    float residual0 = (float)sums[27], residual1 = (float)sums[28];
    c.icpError = sqrtf(residual0) / residual1;
    c.icpCount = (int)residual1;
    if (isnan(c.icpError) || c.icpCount < min_count) {
      c.stop = 1;
      code = 1;
    } else {
      const float rgbError = 0.f, wgt = 1e-4f;
      float currError = rgbError * wgt + c.icpError;
      if (c.lastError < currError) {
        c.breakCount++;
        copy_cand = (c.breakCount == 1);
        c.candidateICP = c.icpError;
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
  }
  code = __shfl_sync(full, code, 0);
  copy_cand = __shfl_sync(full, copy_cand, 0);
  __syncwarp();
  if (copy_cand && lane < 16) c.candidate[lane] = c.next_pose[lane];
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
  // CreateMatrix<6,7>
  for (int e = lane; e < 36; e += 32) {
    const int i = e / 6, j = e % 6;
    const int r = i < j ? i : j, q = i < j ? j : i;
    w.a[e] = sums[tri_start(r) + (q - r)];
  }
  if (lane < 6) {
    w.b[lane] = sums[tri_start(lane) + (6 - lane)];
    w.perm[lane] = lane;
  }
  __syncwarp();
  // LDL^T with symmetric pivoting (ldlt_solve6)
  for (int k = 0; k < 6; ++k) {
    if (lane == 0) {
      int piv = k;
      double best = fabs(w.a[k * 6 + k]);
      for (int i = k + 1; i < 6; ++i) {
        double v = fabs(w.a[i * 6 + i]);
        if (v > best) { best = v; piv = i; }
      }
      w.piv = piv;
    }
    __syncwarp();
    const int piv = w.piv;
    if (piv != k) {
      if (lane < 6) {
        double t = w.a[k * 6 + lane]; w.a[k * 6 + lane] = w.a[piv * 6 + lane]; w.a[piv * 6 + lane] = t;
      }
      __syncwarp();
      if (lane < 6) {
        double t = w.a[lane * 6 + k]; w.a[lane * 6 + k] = w.a[lane * 6 + piv]; w.a[lane * 6 + piv] = t;
      }
      if (lane == 0) { int t = w.perm[k]; w.perm[k] = w.perm[piv]; w.perm[piv] = t; }
      __syncwarp();
    }
    const double dk = w.a[k * 6 + k];
    if (lane == 0) w.d[k] = dk;
    if (lane > k && lane < 6) w.l[lane] = (dk != 0.0) ? w.a[lane * 6 + k] / dk : 0.0;
    __syncwarp();
    const int n = 5 - k;
    if (lane < n * n) {
      const int i = k + 1 + lane / n, j = k + 1 + lane % n;
      w.a[i * 6 + j] -= w.l[i] * dk * w.l[j];
    }
    __syncwarp();
    if (lane > k && lane < 6) { w.a[lane * 6 + k] = w.l[lane]; w.a[k * 6 + lane] = 0.0; }
    __syncwarp();
  }
  if (lane < 6) w.y[lane] = w.b[w.perm[lane]];
  __syncwarp();
  for (int j = 0; j < 6; ++j) {
    if (lane > j && lane < 6) w.y[lane] -= w.a[lane * 6 + j] * w.y[j];
    __syncwarp();
  }
  const double tol = 2.2250738585072014e-308;
  if (lane < 6) w.y[lane] = (fabs(w.d[lane]) > tol) ? w.y[lane] / w.d[lane] : 0.0;
  __syncwarp();
  for (int j = 5; j >= 1; --j) {
    if (lane < j) w.y[lane] -= w.a[j * 6 + lane] * w.y[j];
    __syncwarp();
  }
  if (lane < 6) w.x[w.perm[lane]] = w.y[lane];
  __syncwarp();
  // se3_exp
  const double u0 = w.x[0], u1 = w.x[1], u2 = w.x[2];
  const double w0 = w.x[3], w1 = w.x[4], w2 = w.x[5];
  const double eps = 1e-10;
  const double th2 = w0 * w0 + w1 * w1 + w2 * w2;
  const double th = sqrt(th2);
  double real_f, imag_f;
  if (th2 < eps * eps) {
    double th4 = th2 * th2;
    imag_f = 0.5 - (1.0 / 48.0) * th2 + (1.0 / 3840.0) * th4;
    real_f = 1.0 - (1.0 / 8.0) * th2 + (1.0 / 384.0) * th4;
  } else {
    if (lane == 0) w.sc[0] = sin(0.5 * th);
    if (lane == 1) w.sc[1] = cos(0.5 * th);
    if (lane == 2) w.sc[2] = cos(th);
    if (lane == 3) w.sc[3] = sin(th);
    __syncwarp();
    imag_f = w.sc[0] / th;
    real_f = w.sc[1];
  }
  if (lane < 9) {
    const double qw = real_f, qx = imag_f * w0, qy = imag_f * w1, qz = imag_f * w2;
    const double tx = 2 * qx, ty = 2 * qy, tz = 2 * qz;
    const double twx = tx * qw, twy = ty * qw, twz = tz * qw, txx = tx * qx, txy = ty * qx, txz = tz * qx;
    const double tyy = ty * qy, tyz = tz * qy, tzz = tz * qz;
    double r;
    switch (lane) {
      case 0: r = 1 - (tyy + tzz); break;
      case 1: r = txy - twz; break;
      case 2: r = txz + twy; break;
      case 3: r = txy + twz; break;
      case 4: r = 1 - (txx + tzz); break;
      case 5: r = tyz - twx; break;
      case 6: r = txz - twy; break;
      case 7: r = tyz + twx; break;
      default: r = 1 - (txx + tyy); break;
    }
    w.R[lane] = r;
    const double Wv[9] = {0, -w2, w1, w2, 0, -w0, -w1, w0, 0};
    w.W[lane] = Wv[lane];
  }
  __syncwarp();
  if (lane < 9) {
    if (th < eps) {
      w.V[lane] = w.R[lane];
    } else {
      const int i = lane / 3, j = lane % 3;
      const double c1 = (1 - w.sc[2]) / th2, c2 = (th - w.sc[3]) / (th2 * th);
      const double w2ij = w.W[i * 3 + 0] * w.W[0 * 3 + j] + w.W[i * 3 + 1] * w.W[1 * 3 + j] +
                          w.W[i * 3 + 2] * w.W[2 * 3 + j];
      w.V[lane] = (i == j ? 1.0 : 0.0) + c1 * w.W[lane] + c2 * w2ij;
    }
  }
  __syncwarp();
  if (lane < 16) {
    const int i = lane >> 2, j = lane & 3;
    double v;
    if (i == 3) v = (j == 3) ? 1.0 : 0.0;
    else if (j < 3) v = w.R[i * 3 + j];
    else v = w.V[i * 3 + 0] * u0 + w.V[i * 3 + 1] * u1 + w.V[i * 3 + 2] * u2;
    w.dT[lane] = v;
  }
  __syncwarp();
  // delta = dT * delta
  warp_mat4_mul(w.dT, c.delta, w.tmp, lane);
  if (lane < 16) c.delta[lane] = w.tmp[lane];
  __syncwarp();
  // dInv = se3_inv(delta)
  if (lane < 16) {
    const int i = lane >> 2, j = lane & 3;
    const double *T = c.delta;
    double v;
    if (i == 3) v = (j == 3) ? 1.0 : 0.0;
    else if (j < 3) v = T[j * 4 + i];
    else v = -(T[0 * 4 + i] * T[3] + T[1 * 4 + i] * T[7] + T[2 * 4 + i] * T[11]);
    w.dInv[lane] = v;
  }
  __syncwarp();
  // next = last * dInv
  warp_mat4_mul(c.last_pose, w.dInv, w.tmp, lane);
  if (lane < 16) c.next_pose[lane] = w.tmp[lane];
  __syncwarp();
  return true;
}

}  // namespace sf
#endif
