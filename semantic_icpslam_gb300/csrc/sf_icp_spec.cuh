// Next-pose prediction for the persistent ICP kernel.
//
// Every ICP iteration ends in the FP64 6x6 solve and SE(3) update
// (sf_icp_solve.cuh), a dependent chain of FP64 instructions of about
// 3.5 us on GB300 during which the pixel warps would idle: the next
// iteration's rows need the pose the solve produces, in float (the
// reference's GpuRotation / GpuTranslation, Core/Frame.cc:626-645).
// This warp predicts that float pose from the same 29 sums with FP32 and
// float-float (hi + lo) arithmetic only, off the FP64 pipe, in well under
// a microsecond, so that the pixel warps can accumulate the next
// iteration's rows while the FP64 solve runs.  The FP64 result stays the
// only result: once it is known, the prediction is compared with it bit
// for bit (all twelve floats), and a prediction that differs in any bit,
// or that was not made, is thrown away and the rows are accumulated again
// from the FP64 pose.  So the poses, sums and decisions of the kernel do
// not depend on the prediction; it only decides whether the next
// iteration's accumulation overlapped the solve.
//
// The prediction: A x = b by Gauss-Jordan elimination in FP32 on
// [A | b | I] (without pivoting: J^T J is symmetric positive definite),
// then one step of iterative refinement with the residual b - A x taken
// in float-float from the FP64 sums (mixed-precision iterative refinement,
// J. H. Wilkinson, Rounding Errors in Algebraic Processes, 1963; C. B.
// Moler, J. ACM 14(2), 1967), which brings x to about 2^-44 relative for
// the conditioning of these systems.  exp(-x) is taken as I + D with D and
// the translation in float-float, their leading terms (-[w]x, w w^T / 2,
// -u, (w x u) / 2) exact and the higher-order terms of the Rodrigues
// coefficients in FP32 (angles below 0.1 rad; larger steps are not
// predicted), and the pose as N + N D, N + N t' in float-float from the
// FP64 pose split into float-float by bit manipulation, rounded once to
// float.  The float-float operations are Knuth's TwoSum, Dekker's
// FastTwoSum and the FMA-based exact product (T. J. Dekker, Numer. Math.
// 18, 1971).  On the 640x480 benchmark sequence every prediction equalled
// the FP64 path's float pose.
#ifndef SF_ICP_SPEC_CUH_
#define SF_ICP_SPEC_CUH_

// Optional stage-clock hook of the prediction (a no-op unless defined
// before inclusion).
#ifndef SF_SPEC_MARK
#define SF_SPEC_MARK(k)
#endif

namespace sf {
namespace spec {

struct f2f {
  float h, l;
};

__device__ __forceinline__ f2f two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return f2f{s, (a - (s - bb)) + (b - bb)};
}
// |a| >= |b| (or a == 0)
__device__ __forceinline__ f2f fast_two_sum(float a, float b) {
  const float s = a + b;
  return f2f{s, b - (s - a)};
}
__device__ __forceinline__ f2f two_prod(float a, float b) {
  const float p = a * b;
  return f2f{p, fmaf(a, b, -p)};
}
__device__ __forceinline__ f2f add(f2f x, f2f y) {
  const f2f s = two_sum(x.h, y.h);
  return fast_two_sum(s.h, s.l + (x.l + y.l));
}
__device__ __forceinline__ f2f neg(f2f x) { return f2f{-x.h, -x.l}; }
__device__ __forceinline__ f2f mul(f2f x, f2f y) {
  const f2f p = two_prod(x.h, y.h);
  return fast_two_sum(p.h, p.l + (x.h * y.l + x.l * y.h));
}
__device__ __forceinline__ f2f mulf(f2f x, float f) {
  const f2f p = two_prod(x.h, f);
  return fast_two_sum(p.h, p.l + x.l * f);
}
__device__ __forceinline__ f2f half(f2f x) { return f2f{x.h * 0.5f, x.l * 0.5f}; }
__device__ __forceinline__ f2f shfl(f2f x, int src) {
  return f2f{__shfl_sync(0xffffffffu, x.h, src), __shfl_sync(0xffffffffu, x.l, src)};
}

// A double as float-float from its bits (no FP64 instruction): hi takes the
// sign, the exponent and the top 23 mantissa bits, lo the remaining 29 bits
// (rounded to 24).  Zero and subnormal doubles give zero; doubles outside
// the float range give NaN, which fails the comparison with the FP64 path.
// Branch-free, so that the lanes of a warp split side by side.
__device__ __forceinline__ f2f split(double d) {
  const int hi = __double2hiint(d), lo = __double2loint(d);
  const int e = (hi >> 20) & 0x7ff;
  const int fe = e - 1023 + 127;
  const unsigned sign = (unsigned)hi & 0x80000000u;
  const float h0 = __uint_as_float(sign | ((unsigned)fe << 23) | (((unsigned)hi & 0xfffffu) << 3) |
                                   ((unsigned)lo >> 29));
  const unsigned rest = (unsigned)lo & 0x1fffffffu;  // weight 2^(e - 1023 - 52)
  const int se = e - 1023 - 52 + 127;
  const float l0 = __uint2float_rn(rest) * __uint_as_float((unsigned)(se > 0 ? se : 0) << 23);
  const float l = se > 0 ? __uint_as_float(__float_as_uint(l0) ^ sign) : 0.f;
  const bool zero = e == 0, out_of_range = fe <= 0 || fe >= 255;
  return f2f{zero ? 0.f : (out_of_range ? __int_as_float(0x7fc00000) : h0), (zero || out_of_range) ? 0.f : l};
}

// Approximate reciprocal (MUFU.RCP, about one ulp): the prediction's
// elimination only has to be close, the refinement corrects it.
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Index of sum (i, j), i <= j <= 6, in CreateMatrix<6,7>'s upper-triangle
// order (Tracking/Reduction.cu:6-16).
__device__ __forceinline__ int sum_index(int i, int j) { return 7 * i - i * (i - 1) / 2 + (j - i); }

// The float pose of the iteration after the one whose sums are given:
// out[4 i + j] (i < 3, j < 4) is the prediction of
// (float)(N exp(-x))_ij for the FP64 pose N (as float-float in nff[4 i + j])
// and the solution x of A x = b.  Run by one whole warp; returns
// (warp-uniform) whether a prediction was made, and writes out (lanes
// 0..11) only then.  Every step is spread over the lanes so that the
// warp's dependent chain stays short (about a microsecond's fraction of
// the FP64 solve it races):
//  - elimination without pivoting (J^T J is symmetric positive definite;
//    a pivot that is not positive gives no prediction), lane c < 13 holding
//    column c of [A | b | I], the six steps unrolled, each one shuffle of
//    the pivot, five of its column, a reciprocal and five FMAs per lane;
//  - the refinement's residual of row i in lane i from its seven
//    float-float terms summed as a tree, the correction of x_j in lane
//    7 + j (row j of the inverse, which is symmetric);
//  - D = exp(-x)'s rotation - I in lanes 0..8 (entry (k, j) in lane
//    3 k + j), t' in lanes 9..11, then pose entry (i, j) in lane 4 i + j
//    from the three D or t' entries it needs.
__device__ __noinline__ bool predict_pose_warp(const double *sums, const f2f *nff, float *out) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const f2f sk = lane < 27 ? split(sums[lane]) : f2f{0.f, 0.f};
  SF_SPEC_MARK(6);
  // column c of [A | b | I] (lanes 13..31 repeat column 12)
  const int c = lane < 13 ? lane : 12;
  float M[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    const int src = c < 6 ? (i < c ? sum_index(i, c) : sum_index(c, i)) : sum_index(i, 6);
    const float v = __shfl_sync(full, sk.h, src);
    M[i] = c <= 6 ? v : ((c - 7 == i) ? 1.f : 0.f);
  }
  SF_SPEC_MARK(0);
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    const float pk = __shfl_sync(full, M[k], k);
    if (!(pk > 1e-30f) || !(pk < 3e38f)) return false;  // not positive definite (or not finite)
    const float rp = rcp_approx(pk);
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      if (i == k) continue;
      const float f = __shfl_sync(full, M[i], k) * rp;
      M[i] = fmaf(-f, M[k], M[i]);
    }
  }
  SF_SPEC_MARK(1);
  // x_i = b'_i / d_i in every lane; lane 7 + j keeps row j of A^-1
  float x0[6], inv[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    const float rd = rcp_approx(__shfl_sync(full, M[i], i));
    x0[i] = __shfl_sync(full, M[i], 6) * rd;
    inv[i] = M[i] * rd;
  }
  SF_SPEC_MARK(2);
  // refinement: lane i < 6 takes the residual of row i in float-float
  f2f x[6];
  {
    const int r = lane < 6 ? lane : 0;
    f2f t[7];
    t[6] = shfl(sk, sum_index(r, 6));
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      const f2f a = shfl(sk, r < j ? sum_index(r, j) : sum_index(j, r));
      t[j] = neg(mulf(a, x0[j]));
    }
    SF_SPEC_MARK(7);
    const f2f s01 = add(t[0], t[1]), s23 = add(t[2], t[3]), s45 = add(t[4], t[5]);
    const f2f res2 = add(add(s01, s23), add(s45, t[6]));
    const float res = res2.h + res2.l;
    SF_SPEC_MARK(8);
    // lane 7 + j: dx_j = sum_i (A^-1)_ji res_i
    float dx = 0.f;
#pragma unroll
    for (int i = 0; i < 6; ++i) dx = fmaf(inv[i], __shfl_sync(full, res, i), dx);
#pragma unroll
    for (int j = 0; j < 6; ++j) x[j] = shfl(two_sum(x0[j], dx), 7 + j);
  }
  SF_SPEC_MARK(3);
  const f2f u0 = x[0], u1 = x[1], u2 = x[2];
  const f2f w0 = x[3], w1 = x[4], w2 = x[5];
  const f2f th2 = add(add(mul(w0, w0), mul(w1, w1)), mul(w2, w2));
  if (!(th2.h < 0.01f)) return false;  // steps of 0.1 rad and more are not predicted
  SF_SPEC_MARK(9);
  // c_a - 1, c_1 - 1/2 and c_2 of the Rodrigues form (their series in t^2)
  const float t = th2.h;
  const float cap = t * (-1.f / 6 + t * (1.f / 120 + t * (-1.f / 5040 + t * (1.f / 362880))));
  const float c1p = t * (-1.f / 24 + t * (1.f / 720 + t * (-1.f / 40320 + t * (1.f / 3628800))));
  const float c2 = 1.f / 6 + t * (-1.f / 120 + t * (1.f / 5040 + t * (-1.f / 362880)));
  // Entry (k, j) of E = exp(-x) - I in lane 4 k + j (j < 3: the rotation's
  // D_kj; j = 3: the translation t'_k), each as -X + Y / 2 + s with X, Y
  // in float-float and the higher-order rest s in FP32:
  //   D_kj = -W_kj + (w_k w_j - delta_kj t^2) / 2 + [-(c_a - 1) W_kj + (c_1 - 1/2) Q_kj],
  //   t'_k = -u_k + (w x u)_k / 2 + [(c_1 - 1/2) (w x u)_k - c_2 (w x (w x u))_k],
  // W = [w]x, Q_kj = w_k w_j - delta_kj t^2.  Y = P1 Q1 - P2 Q2 (- t^2 on the
  // diagonal) covers both with operands chosen per lane.
  const int k = lane < 12 ? lane >> 2 : 0, jj = lane & 3;
  const int k1 = k == 2 ? 0 : k + 1, k2 = k == 0 ? 2 : k - 1;
  auto pick = [&](const f2f &v0, const f2f &v1, const f2f &v2, int q) { return q == 0 ? v0 : (q == 1 ? v1 : v2); };
  const bool rot = jj < 3;
  const f2f wk = pick(w0, w1, w2, k), wk1 = pick(w0, w1, w2, k1), wk2 = pick(w0, w1, w2, k2);
  const f2f wj = pick(w0, w1, w2, jj < 3 ? jj : 0);
  const f2f uk = pick(u0, u1, u2, k), uk1 = pick(u0, u1, u2, k1), uk2 = pick(u0, u1, u2, k2);
  // X: W_kj = -w_m for (k, j) cyclic (j = k + 1), w_m for j = k - 1, 0 on the diagonal; u_k
  const f2f zero = f2f{0.f, 0.f};
  const f2f X = rot ? (jj == k ? zero : (jj == k1 ? neg(wk2) : wk1)) : uk;
  const f2f Y = rot ? add(mul(wk, wj), jj == k ? neg(th2) : zero) : add(mul(wk1, uk2), neg(mul(wk2, uk1)));
  // (w x (w x u))_k from the lanes holding (w x u): lanes 4 k' + 3
  SF_SPEC_MARK(10);
  const float ak1 = __shfl_sync(full, Y.h, 4 * k1 + 3), ak2 = __shfl_sync(full, Y.h, 4 * k2 + 3);
  const float bk = wk1.h * ak2 - wk2.h * ak1;
  const float rest = rot ? (-cap * X.h + c1p * Y.h) : (c1p * Y.h - c2 * bk);
  const f2f e = add(add(neg(X), half(Y)), f2f{rest, 0.f});
  // pose entry (i, j) in lane 4 i + j: N_ij + sum_k N_ik E_kj
  const int i = lane < 12 ? lane >> 2 : 0, j = lane & 3;
  f2f p[3];
#pragma unroll
  for (int q = 0; q < 3; ++q) p[q] = mul(nff[4 * i + q], shfl(e, 4 * q + j));
  const f2f v = add(add(nff[lane < 12 ? lane : 0], p[0]), add(p[1], p[2]));
  if (lane < 12) out[lane] = v.h + v.l;
  SF_SPEC_MARK(5);
  return true;
}

}  // namespace spec
}  // namespace sf
#endif
