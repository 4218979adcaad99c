// Next-pose prediction for the persistent ICP kernel.
//
// Every ICP iteration ends in the FP64 6x6 solve and SE(3) update
// (sf_icp_solve.cuh), a dependent chain of FP64 instructions of about
// 3.3 us on GB300 during which the pixel warps would idle: the next
// iteration's rows need the pose the solve produces, in float (the
// reference's GpuRotation / GpuTranslation, Core/Frame.cc:626-645).
// This warp predicts that float pose from the same 29 sums with FP32 and
// float-float (hi + lo) arithmetic only, off the FP64 pipe, in about a
// third of the solve's time, so that the pixel warps can accumulate the next
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
// warp's dependent chain stays short against the FP64 solve it races:
//  - elimination without pivoting (J^T J is symmetric positive definite;
//    a pivot that is not positive gives no prediction), lane c < 13 holding
//    column c of [A | b | I], the six steps unrolled, each one shuffle of
//    the pivot, five of its column, an approximate reciprocal and five FMAs
//    per lane;
//  - the refinement's residual of row i in lane i from its seven
//    float-float terms summed as a tree, the correction of x_j in lane
//    7 + j (row j of the inverse, which is symmetric);
//  - E = exp(-x) - I, entry (k, j) in lane 4 k + j (rotation for j < 3,
//    translation for j = 3), then pose entry (i, j) in the same lane from
//    the three entries of E it needs.
// About 2,100 SM cycles alone on a GB300 (one warp, clock64), against
// about 6,600 for the FP64 solve.
__device__ __noinline__ bool predict_pose_warp(const double *sums, const f2f *nff, float *out) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const f2f sk = lane < 27 ? split(sums[lane]) : f2f{0.f, 0.f};
  SF_SPEC_MARK(6);
  // column c of [A | b | I] (lanes 13..31 repeat column 12); sum (i, c)
  // has index 6 i - i (i - 1) / 2 + c for i <= c, base_c + i for i > c
  const int c = lane < 13 ? lane : 12;
  const int base_c = 6 * c - (c * (c - 1)) / 2;
  float M[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    const int ci = 6 * i - (i * (i - 1)) / 2;
    const int src = c < 6 ? (i <= c ? ci + c : base_c + i) : ci + 6;
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
  // refinement: lane r < 6 takes the residual of row r in float-float
  f2f x[6];
  {
    const int r = lane < 6 ? lane : 0;
    const int base_r = 6 * r - (r * (r - 1)) / 2;
    f2f t[7];
    t[6] = shfl(sk, base_r + 6);
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      const int cj = 6 * j - (j * (j - 1)) / 2;
      const f2f a = shfl(sk, r <= j ? base_r + j : cj + r);
      t[j] = neg(mulf(a, x0[j]));
    }
    SF_SPEC_MARK(7);
    const f2f s01 = add(t[0], t[1]), s23 = add(t[2], t[3]), s45 = add(t[4], t[5]);
    const f2f res2 = add(add(s01, s23), add(s45, t[6]));
    const float res = res2.h + res2.l;
    SF_SPEC_MARK(8);
    // lane 7 + j: dx_j = sum_i (A^-1)_ji res_i, x_j = x0_j + dx_j
    float dx = 0.f;
#pragma unroll
    for (int i = 0; i < 6; ++i) dx = fmaf(inv[i], __shfl_sync(full, res, i), dx);
    float xo = x0[0];
#pragma unroll
    for (int j = 1; j < 6; ++j)
      if (lane == 7 + j) xo = x0[j];
    const f2f xs = two_sum(xo, dx);
#pragma unroll
    for (int j = 0; j < 6; ++j) x[j] = shfl(xs, 7 + j);
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
  // diagonal) covers both with operands chosen per lane, so every lane runs
  // the same instructions.
  const int k = lane < 12 ? lane >> 2 : 0, jj = lane & 3;
  const int k1 = k == 2 ? 0 : k + 1, k2 = k == 0 ? 2 : k - 1;
  const bool rot = jj < 3;
  const int jr = rot ? jj : 0;
  auto sel = [](f2f v0, f2f v1, f2f v2, int q) {
    f2f r = v0;
    if (q == 1) r = v1;
    if (q == 2) r = v2;
    return r;
  };
  const f2f wk = sel(w0, w1, w2, k), wk1 = sel(w0, w1, w2, k1), wk2 = sel(w0, w1, w2, k2);
  const f2f wj = sel(w0, w1, w2, jr);
  const f2f uk = sel(u0, u1, u2, k), uk1 = sel(u0, u1, u2, k1), uk2 = sel(u0, u1, u2, k2);
  const f2f P1 = rot ? wk : wk1, Q1 = rot ? wj : uk2;
  const f2f P2 = rot ? f2f{0.f, 0.f} : wk2, Q2 = rot ? f2f{0.f, 0.f} : uk1;
  const f2f diag = (rot && jj == k) ? th2 : f2f{0.f, 0.f};
  const f2f Y = add(add(mul(P1, Q1), neg(mul(P2, Q2))), neg(diag));
  // X: W_kj = -w_k2 for j = k + 1 (cyclic), w_k1 for j = k - 1, 0 on the diagonal; u_k
  f2f X = uk;
  if (rot) X = (jj == k) ? f2f{0.f, 0.f} : (jj == k1 ? neg(wk2) : wk1);
  SF_SPEC_MARK(10);
  // (w x (w x u))_k from the lanes holding (w x u) (lanes 4 k' + 3): of
  // order |w|^2 |u|, float suffices
  const float ak1 = __shfl_sync(full, Y.h, 4 * k1 + 3), ak2 = __shfl_sync(full, Y.h, 4 * k2 + 3);
  const float bk = wk1.h * ak2 - wk2.h * ak1;
  const float rest = rot ? (-cap * X.h + c1p * Y.h) : (c1p * Y.h - c2 * bk);
  const f2f e = add(add(neg(X), half(Y)), f2f{rest, 0.f});
  SF_SPEC_MARK(4);
  // pose entry (i, j) in lane 4 i + j: N_ij + sum_q N_iq E_qj, the
  // products N_iq.h E_qj.h exact (TwoProduct) and summed exactly, the cross
  // terms (about 2^-24 of them) in float
  const int i = lane < 12 ? lane >> 2 : 0, j = lane & 3;
  f2f p[3];
  float small = 0.f;
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    const f2f eq = shfl(e, 4 * q + j);
    const f2f n = nff[4 * i + q];
    p[q] = two_prod(n.h, eq.h);
    small += p[q].l + (n.h * eq.l + n.l * eq.h);
  }
  const f2f d = two_sum(p[0].h, p[1].h);
  const f2f d2 = two_sum(d.h, p[2].h);
  const f2f n0 = nff[lane < 12 ? lane : 0];
  const f2f v = add(n0, f2f{d2.h, d.l + d2.l + small});
  if (lane < 12) out[lane] = v.h + v.l;
  SF_SPEC_MARK(5);
  return true;
}
}  // namespace spec
}  // namespace sf
#endif
