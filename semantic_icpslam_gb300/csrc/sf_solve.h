// FP64 6x6 solve, SE(3) exponential and pose algebra shared by the host
// (plain per-launch tracking loop) and the device (persistent ICP kernel).
// These are the only FP64 steps of the loop.
//
// Reference: Tracker::ComputeSE3 (Tracking/Tracking.cc:481-499) solves
// A x = b with Eigen's LDLT and applies Sophus::SE3d::exp(x).  Both are
// restated from their mathematics here: LDL^T with symmetric pivoting on
// the largest remaining diagonal, a zero pivot zeroing that component; the
// exponential via the unit quaternion of the rotation vector and the left
// Jacobian V = I + (1 - cos t)/t^2 W + (t - sin t)/t^3 W^2 applied to the
// translational part (twist order: translation first, then rotation).
#ifndef SF_SOLVE_H_
#define SF_SOLVE_H_

#include <math.h>

#if defined(__CUDACC__)
#define SF_HD __host__ __device__ __forceinline__
#else
#define SF_HD inline
#endif

namespace sf {

// CreateMatrix<6,7> (Tracking/Reduction.cu:6-16): 27 upper-triangle sums
// -> symmetric A (row-major) and b.
SF_HD void create_matrix(const double *s, double *A, double *b) {
  int shift = 0;
  for (int i = 0; i < 6; ++i)
    for (int j = i; j < 7; ++j) {
      double v = s[shift++];
      if (j == 6) b[i] = v;
      else { A[j * 6 + i] = v; A[i * 6 + j] = v; }
    }
}

SF_HD void ldlt_solve6(const double *A36, const double *b6, double *x6) {
  double a[36];
  int perm[6];
  double d[6];
  for (int i = 0; i < 36; ++i) a[i] = A36[i];
  for (int i = 0; i < 6; ++i) perm[i] = i;
  for (int k = 0; k < 6; ++k) {
    int piv = k;
    double best = fabs(a[k * 6 + k]);
    for (int i = k + 1; i < 6; ++i) {
      double v = fabs(a[i * 6 + i]);
      if (v > best) { best = v; piv = i; }
    }
    if (piv != k) {
      for (int j = 0; j < 6; ++j) { double t = a[k * 6 + j]; a[k * 6 + j] = a[piv * 6 + j]; a[piv * 6 + j] = t; }
      for (int i = 0; i < 6; ++i) { double t = a[i * 6 + k]; a[i * 6 + k] = a[i * 6 + piv]; a[i * 6 + piv] = t; }
      int t = perm[k]; perm[k] = perm[piv]; perm[piv] = t;
    }
    double dk = a[k * 6 + k];
    d[k] = dk;
    double l[6] = {0, 0, 0, 0, 0, 0};
    for (int i = k + 1; i < 6; ++i) l[i] = (dk != 0.0) ? a[i * 6 + k] / dk : 0.0;
    for (int i = k + 1; i < 6; ++i)
      for (int j = k + 1; j < 6; ++j) a[i * 6 + j] -= l[i] * dk * l[j];
    for (int i = k + 1; i < 6; ++i) { a[i * 6 + k] = l[i]; a[k * 6 + i] = 0.0; }
  }
  double y[6];
  for (int i = 0; i < 6; ++i) y[i] = b6[perm[i]];
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < i; ++j) y[i] -= a[i * 6 + j] * y[j];
  const double tol = 2.2250738585072014e-308;  // smallest normal double
  for (int i = 0; i < 6; ++i) y[i] = (fabs(d[i]) > tol) ? y[i] / d[i] : 0.0;
  // back substitution with j descending (the order the warp-parallel
  // device version can reproduce bit for bit)
  for (int j = 5; j >= 1; --j)
    for (int i = j - 1; i >= 0; --i) y[i] -= a[j * 6 + i] * y[j];
  for (int i = 0; i < 6; ++i) x6[perm[i]] = y[i];
}

SF_HD void se3_exp(const double *xi, double *T) {
  const double u0 = xi[0], u1 = xi[1], u2 = xi[2];
  const double w0 = xi[3], w1 = xi[4], w2 = xi[5];
  const double eps = 1e-10;
  double th2 = w0 * w0 + w1 * w1 + w2 * w2;
  double th = sqrt(th2);
  double real_f, imag_f;
  if (th2 < eps * eps) {
    double th4 = th2 * th2;
    imag_f = 0.5 - (1.0 / 48.0) * th2 + (1.0 / 3840.0) * th4;
    real_f = 1.0 - (1.0 / 8.0) * th2 + (1.0 / 384.0) * th4;
  } else {
    imag_f = sin(0.5 * th) / th;
    real_f = cos(0.5 * th);
  }
  double qw = real_f, qx = imag_f * w0, qy = imag_f * w1, qz = imag_f * w2;
  double tx = 2 * qx, ty = 2 * qy, tz = 2 * qz;
  double twx = tx * qw, twy = ty * qw, twz = tz * qw, txx = tx * qx, txy = ty * qx, txz = tz * qx;
  double tyy = ty * qy, tyz = tz * qy, tzz = tz * qz;
  double R[9] = {1 - (tyy + tzz), txy - twz, txz + twy, txy + twz, 1 - (txx + tzz),
                 tyz - twx, txz - twy, tyz + twx, 1 - (txx + tyy)};
  double W[9] = {0, -w2, w1, w2, 0, -w0, -w1, w0, 0};
  double V[9];
  if (th < eps) {
    for (int k = 0; k < 9; ++k) V[k] = R[k];
  } else {
    double c1 = (1 - cos(th)) / th2, c2 = (th - sin(th)) / (th2 * th);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double w2ij = W[i * 3 + 0] * W[0 * 3 + j] + W[i * 3 + 1] * W[1 * 3 + j] + W[i * 3 + 2] * W[2 * 3 + j];
        V[i * 3 + j] = (i == j ? 1.0 : 0.0) + c1 * W[i * 3 + j] + c2 * w2ij;
      }
  }
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) T[i * 4 + j] = R[i * 3 + j];
    T[i * 4 + 3] = V[i * 3 + 0] * u0 + V[i * 3 + 1] * u1 + V[i * 3 + 2] * u2;
  }
  T[12] = 0; T[13] = 0; T[14] = 0; T[15] = 1;
}

SF_HD void mat4_mul(const double *A, const double *B, double *C) {
  double t[16];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      double s = 0;
      for (int k = 0; k < 4; ++k) s += A[i * 4 + k] * B[k * 4 + j];
      t[i * 4 + j] = s;
    }
  for (int k = 0; k < 16; ++k) C[k] = t[k];
}

// Inverse of a rigid transform: [R^T, -R^T t].
SF_HD void se3_inv(const double *T, double *I) {
  double t[16];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) t[i * 4 + j] = T[j * 4 + i];
  for (int i = 0; i < 3; ++i)
    t[i * 4 + 3] = -(t[i * 4 + 0] * T[3] + t[i * 4 + 1] * T[7] + t[i * 4 + 2] * T[11]);
  t[12] = 0; t[13] = 0; t[14] = 0; t[15] = 1;
  for (int k = 0; k < 16; ++k) I[k] = t[k];
}

// |sin(eulerAngles(0,1,2))| of the rotation part (Tracking.cc:505-510).
// Eigen's two solution branches give the same norm.
SF_HD double euler_sin_norm(const double *P) {
  double r02 = P[2] < -1.0 ? -1.0 : (P[2] > 1.0 ? 1.0 : P[2]);
  double b = asin(r02);
  double a = atan2(-P[6], P[10]);
  double c = atan2(-P[1], P[0]);
  double sa = sin(a), sb = sin(b), sc = sin(c);
  return sqrt(sa * sa + sb * sb + sc * sc);
}

// Tracker::ComputeSE3's per-iteration control (Tracking.cc:449-499,
// icpOnly): failure test, divergence guard with its candidate pose, solve,
// delta = exp(x) * delta, next = last * delta^-1.  The state is plain data
// so it can live in device memory between launches.
struct TrackCtl {
  double last_pose[16];   // LastFrame->pose
  double start_pose[16];  // NextFrame->pose at entry (== last pose)
  double next_pose[16];   // NextFrame->pose
  double delta[16];
  double candidate[16];
  float lastError, candidateICP, icpError;
  int breakCount, icpCount, iters_run;
  int stop;               // 0 running, 1 failed (rolled back), 2 diverged (candidate)
  int accepted;           // final decision (valid after finish)
  float rgbError;         // photometric term (icpOnly = false), else 0
  int rgbCount;
  int timeout;            // a bounded device wait gave up (the persistent kernel), stop = 1
};

SF_HD void ctl_begin(TrackCtl &c, const double *last_pose) {
  for (int k = 0; k < 16; ++k) {
    c.last_pose[k] = last_pose[k];
    c.start_pose[k] = last_pose[k];
    c.next_pose[k] = last_pose[k];
    c.delta[k] = (k % 5 == 0) ? 1.0 : 0.0;
    c.candidate[k] = last_pose[k];
  }
  c.lastError = 100.f;
  c.candidateICP = 0.f;
  c.icpError = 0.f;
  c.breakCount = 0;
  c.icpCount = 0;
  c.iters_run = 0;
  c.stop = 0;
  c.accepted = 0;
  c.rgbError = 0.f;
  c.timeout = 0;
  c.rgbCount = 0;
}

// One iteration given the 29 ICP sums and, with the photometric term
// (icpOnly = false), the 29 RGB sums (Tracking.cc:400-499): the RGB error
// and count are tested first, and the solve takes A_rgb w + A_icp,
// b_rgb w + b_icp with w = 1e-4f.  Returns false when the loop stops.
SF_HD bool ctl_step(TrackCtl &c, const double *sums29, int min_count, const double *rgb29 = nullptr) {
  c.iters_run++;
  if (rgb29) {
    const float r0 = (float)rgb29[27], r1 = (float)rgb29[28];
    c.rgbError = sqrtf(r0) / r1;
    c.rgbCount = (int)r1;
    if (isnan(c.rgbError) || c.rgbCount < min_count) {
      for (int k = 0; k < 16; ++k) c.next_pose[k] = c.last_pose[k];
      c.stop = 1;
      return false;
    }
  }
  float residual0 = (float)sums29[27], residual1 = (float)sums29[28];
  c.icpError = sqrtf(residual0) / residual1;
  c.icpCount = (int)residual1;
  if (isnan(c.icpError) || c.icpCount < min_count) {
    for (int k = 0; k < 16; ++k) c.next_pose[k] = c.last_pose[k];
    c.stop = 1;
    return false;
  }
  const float w = 1e-4f;
  float currError = c.rgbError * w + c.icpError;
  if (c.lastError < currError) {
    c.breakCount++;
    if (c.breakCount == 1)
      for (int k = 0; k < 16; ++k) c.candidate[k] = c.next_pose[k];
    c.candidateICP = c.icpError;  // outside the inner if (Tracking.cc:463-465)
  } else {
    c.breakCount = 0;
  }
  if (c.breakCount > 2) {
    for (int k = 0; k < 16; ++k) c.next_pose[k] = c.candidate[k];
    c.icpError = c.candidateICP;
    c.stop = 2;
    return false;
  }
  c.lastError = currError;
  double A[36], b[6], x[6], dT[16], dInv[16];
  create_matrix(sums29, A, b);
  if (rgb29) {
    double Ar[36], br[6];
    create_matrix(rgb29, Ar, br);
    for (int k = 0; k < 36; ++k) A[k] = Ar[k] * (double)w + A[k];
    for (int k = 0; k < 6; ++k) b[k] = br[k] * (double)w + b[k];
  }
  ldlt_solve6(A, b, x);
  se3_exp(x, dT);
  mat4_mul(dT, c.delta, c.delta);
  se3_inv(c.delta, dInv);
  mat4_mul(c.last_pose, dInv, c.next_pose);
  return true;
}

// Acceptance gate (Tracking.cc:505-516); rolls back on rejection.
SF_HD void ctl_finish(TrackCtl &c, float thresh) {
  if (c.stop == 1) { c.accepted = 0; return; }
  double pinv[16], p[16];
  se3_inv(c.start_pose, pinv);
  mat4_mul(pinv, c.next_pose, p);
  double tn = sqrt(p[3] * p[3] + p[7] * p[7] + p[11] * p[11]);
  double an = euler_sin_norm(p);
  c.accepted = (c.icpError < thresh) && (an <= 0.1 && tn <= 0.1);
  if (!c.accepted)
    for (int k = 0; k < 16; ++k) c.next_pose[k] = c.last_pose[k];
}

}  // namespace sf
#endif
