// The FP64 tail of plbpd's AVX2 collision kernel, evaluated in FP32.
//
// plbpd's CollisionSRT::_collision_kernel_avx2 (src/CollisionSRT.cpp:93-148)
// updates directions k < 8*floor(Q/8) in 8-wide FP32 and the rest (k = 8 for
// D2Q9, 16-18 for D3Q19, 24-26 for D3Q27) in a scalar loop whose arithmetic
// is double (src/CollisionSRT.cpp:144-147):
//
//   wr  = w_k * rho                                         float product
//   B   = ((1.0 + 3.0*cu) + (4.5*cu)*cu) - 1.5*usq           double, three
//                                                             roundings (the
//                                                             products are exact)
//   neq = wr * B                                            double
//   x   = (double)((1.0f - omega) * n) + omega * neq          double; the first
//                                                             product is float
//   n'  = (float)x
//
// GB300 issues double-precision instructions at a small fraction of its FP32
// rate, so a kernel that runs this tail in FP64 is bound by the FP64 pipe
// (D3Q19 256^3: 13.3k MLUPS against 46k for FP32 arithmetic).  This file gives
// the same float n' from FP32 instructions alone:
//
//   1. The exact value X = a + (omega*wr) * (1 + 3cu + 4.5cu^2 - 1.5usq),
//      a = (1-omega)*n, is evaluated in double-float arithmetic (error-free
//      products by fused multiply-add, Dekker's Fast2Sum and Knuth's TwoSum)
//      to about 2^-42 of its terms.
//   2. The reference's x differs from X by its own six double roundings, at
//      most about 2^-50 of the terms.  E bounds the distance between x and the
//      double-float value s + low.
//   3. If s + low - 2E and s + low + 2E round to the same float, x rounds to it
//      too (rounding is monotone): that float is n'.  Otherwise -- x lies
//      within E of a rounding boundary, about once in 10^4 evaluations for
//      lattice flows -- the caller recomputes n' with the reference's own FP64
//      sequence (tail_fp64).
//
// Preconditions of the fast form, checked at run time (anything else takes
// the FP64 form, which reproduces the reference for every input, NaN and
// infinity included): usq <= 0.25 (|u| up to 0.5, beyond any stable lattice
// flow), so the last bracket sum meets Fast2Sum's ordering condition
// (1 + 3cu + 4.5cu^2 >= 1/2 > 1.5usq); E finite and at most 2^20, which keeps
// every intermediate finite.  Subnormal results are handled (the error bound
// carries an absolute 2^-144 for underflowing products); the code must not be
// compiled with flush-to-zero.
//
// Error bound, with u = 2^-24 and S = |1 + 3cu| + 4.5cu^2 + 1.5usq:
//   reference roundings   2^-53 |a| + 6 * 2^-53 |omega wr| S
//   bracket low part      6 roundings of terms below 2^-21.7 S   -> 2^-43 |P| S
//   product tails         P_lo*lo, rounding of P_lo*b3 and of the fma
//                                                                 -> 2^-44.6 |P| S
//   final low sum         2 roundings                            -> 2^-47 |a| + 2^-43.5 |P| S
// total below 2^-46.9 |a| + 2^-41.7 |P| S <= 2^-41 (|a| + 4 |P_hi| S_f), the E
// used here (S_f, S evaluated in float, and P_hi differ from S and P by
// 2^-22 at most; the factor 4 leaves a margin of 6).
// tests/cpp/test_tail_exact.cpp checks this function against the double
// sequence on random and near-boundary inputs.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define PLB_TX_FN __host__ __device__ __forceinline__
#else
#include <math.h>
#include <string.h>
#define PLB_TX_FN static inline
#endif

namespace plb {
namespace tx {

// Round-to-nearest single operations.  Host builds of this header must use
// -ffp-contract=off so that a*b+c stays two roundings.
PLB_TX_FN float add(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
PLB_TX_FN float sub(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
PLB_TX_FN float mul(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
PLB_TX_FN float fma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return fmaf(a, b, c);
#endif
}
PLB_TX_FN float fabs_(float a) {
#if defined(__CUDA_ARCH__)
    return fabsf(a);
#else
    return fabsf(a);
#endif
}
PLB_TX_FN uint32_t bits(float a) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(a);
#else
    uint32_t u;
    memcpy(&u, &a, 4);
    return u;
#endif
}
PLB_TX_FN double dadd(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
PLB_TX_FN double dsub(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dsub_rn(a, b);
#else
    return a - b;
#endif
}
PLB_TX_FN double dmul(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
PLB_TX_FN float d2f(double a) {
#if defined(__CUDA_ARCH__)
    return __double2float_rn(a);
#else
    return (float)a;
#endif
}

// The reference's tail, operation for operation in double.  wr = w*rho
// (float product), a = (1-omega)*n (float product), om = omega.
PLB_TX_FN float tail_fp64(float cu, float usq, float wr, float om, float a) {
    const double cud = (double)cu;
    // 3*cu, 4.5*cu and (4.5*cu)*cu are exact in double
    double br = dadd(1.0, dmul(3.0, cud));
    br = dadd(br, dmul(dmul(4.5, cud), cud));
    br = dsub(br, dmul(1.5, (double)usq));
    const double neq = dmul((double)wr, br);
    return d2f(dadd((double)a, dmul((double)om, neq)));
}

// Per-node part: 1.5*usq split exactly into vh + vl, and the guard.
struct TailNode {
    float vh, vl;
    bool ok;
};

PLB_TX_FN TailNode tail_node(float usq) {
    TailNode t;
    t.vh = mul(1.5f, usq);
    t.vl = fma(1.5f, usq, -t.vh);
    t.ok = usq <= 0.25f;  // false for NaN
    return t;
}

// The FP32 evaluation.  Returns true with *out = n' when the float result is
// decided; false when the caller must use tail_fp64.
PLB_TX_FN bool tail_fast(float cu, const TailNode& nd, float wr, float om, float a, float* out) {
    // exact pieces of the bracket: 3cu = qh + ql, cu^2 = sh + sl, 4.5 sh = th + tl
    const float qh = mul(3.0f, cu), ql = fma(3.0f, cu, -qh);
    const float sh = mul(cu, cu), sl = fma(cu, cu, -sh);
    const float th = mul(4.5f, sh), tl = fma(4.5f, sh, -th);
    // 1 + qh + th - vh with the rounding error of each sum kept: TwoSum for
    // the first two (no ordering condition), Fast2Sum for the last
    // (b2 ~ 1 + 3cu + 4.5cu^2 >= 1/2 > vh under the guard)
    const float b1 = add(1.0f, qh);
    const float z1 = sub(b1, 1.0f);
    const float e1 = add(sub(1.0f, sub(b1, z1)), sub(qh, z1));
    const float b2 = add(b1, th);
    const float z2 = sub(b2, b1);
    const float e2 = add(sub(b1, sub(b2, z2)), sub(th, z2));
    const float b3 = sub(b2, nd.vh), e3 = sub(sub(b2, b3), nd.vh);
    // the bracket is b3 + lo to about 2^-43 of its terms
    float lo = add(ql, tl);
    lo = fma(4.5f, sl, lo);
    lo = sub(lo, nd.vl);
    lo = add(lo, e1);
    lo = add(lo, e2);
    lo = add(lo, e3);
    // P = omega * wr = ph + pl exactly; P * bracket = mh + ml + ml2
    const float ph = mul(om, wr), pl = fma(om, wr, -ph);
    const float mh = mul(ph, b3), ml = fma(ph, b3, -mh);
    const float ml2 = fma(ph, lo, mul(pl, b3));
    // a + mh = s + se exactly (TwoSum: no ordering condition)
    const float s = add(a, mh);
    const float bb = sub(s, a);
    const float se = add(sub(a, sub(s, bb)), sub(mh, bb));
    const float low = add(add(se, ml), ml2);
    // |x - (s + low)| <= E; the round-to-nearest sums below move by at most
    // 2^-3 E from low -/+ 2E (|low| < 2^21 E), so they stay outside x -/+ E
    const float sf = add(add(fabs_(b1), th), nd.vh);
    const float E = fma(0x1p-41f, fma(mul(4.0f, fabs_(ph)), sf, fabs_(a)), 0x1p-144f);
    const float E2 = add(E, E);
    const float r0 = add(s, sub(low, E2));
    const float r1 = add(s, add(low, E2));
    *out = r0;
    return nd.ok && E <= 0x1p20f && bits(r0) == bits(r1);
}

// n' for one tail direction: the FP32 form when it decides the result, the
// reference's FP64 sequence otherwise.
PLB_TX_FN float tail_update(float cu, float usq, const TailNode& nd, float wr, float om, float a) {
    float r;
    if (tail_fast(cu, nd, wr, om, a, &r)) return r;
    return tail_fp64(cu, usq, wr, om, a);
}

}  // namespace tx
}  // namespace plb
