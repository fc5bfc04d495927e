// Lattice tables, device layout and the per-node arithmetic shared by every
// kernel of the engine.
//
// Tables: plbpd's LBModel (src/LBModel.cpp:23-165).  The order of the
// velocities, the weights (double literals rounded to float) and the reverse
// indices are the reference's, because populations are compared index by
// index; everything else in this file is this engine's own design.
#pragma once

#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "tail_exact.h"

namespace plb {

// ---------------------------------------------------------------------------
// lattice tables
// ---------------------------------------------------------------------------
template <int Q> struct Lattice;

template <> struct Lattice<9> {
    // D2Q9 moves in the x-z plane: c_y is zero for every direction.
    __host__ __device__ static constexpr int cx(int k) {
        constexpr int v[9] = {0, 1, -1, 0, 0, 1, -1, 1, -1};
        return v[k];
    }
    __host__ __device__ static constexpr int cy(int k) {
        constexpr int v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        return v[k];
    }
    __host__ __device__ static constexpr int cz(int k) {
        constexpr int v[9] = {0, 0, 0, 1, -1, 1, -1, -1, 1};
        return v[k];
    }
};
template <> struct Lattice<19> {
    __host__ __device__ static constexpr int cx(int k) {
        constexpr int v[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
        return v[k];
    }
    __host__ __device__ static constexpr int cy(int k) {
        constexpr int v[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1};
        return v[k];
    }
    __host__ __device__ static constexpr int cz(int k) {
        constexpr int v[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1};
        return v[k];
    }
};
template <> struct Lattice<27> {
    __host__ __device__ static constexpr int cx(int k) {
        constexpr int v[27] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0,
                                   1, -1, 1, -1, 1, -1, -1, 1};
        return v[k];
    }
    __host__ __device__ static constexpr int cy(int k) {
        constexpr int v[27] = {0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1,
                                   1, -1, 1, -1, -1, 1, 1, -1};
        return v[k];
    }
    __host__ __device__ static constexpr int cz(int k) {
        constexpr int v[27] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1,
                                   1, -1, -1, 1, 1, -1, 1, -1};
        return v[k];
    }
};

// Every table lists each velocity next to its opposite: 1<->2, 3<->4, ...
__host__ __device__ constexpr int rev_of(int k) { return k == 0 ? 0 : ((k & 1) ? k + 1 : k - 1); }

template <int Q>
__host__ __device__ constexpr int speed2(int k) {
    return Lattice<Q>::cx(k) * Lattice<Q>::cx(k) + Lattice<Q>::cy(k) * Lattice<Q>::cy(k) +
           Lattice<Q>::cz(k) * Lattice<Q>::cz(k);
}

// Weights, each the float nearest to the reference's double literal.
template <int Q>
__host__ __device__ constexpr float weight(int k) {
    return Q == 9 ? (speed2<Q>(k) == 0 ? float(4. / 9.) : speed2<Q>(k) == 1 ? float(1. / 9.) : float(1. / 36.))
         : Q == 19 ? (speed2<Q>(k) == 0 ? float(1. / 3.) : speed2<Q>(k) == 1 ? float(1. / 18.) : float(1. / 36.))
         : (speed2<Q>(k) == 0 ? float(8. / 27.) : speed2<Q>(k) == 1 ? float(2. / 27.)
            : speed2<Q>(k) == 2 ? float(1. / 54.) : float(1. / 216.));
}

// The exact weights in double, for FP64 storage: the float weights sum to
// 1 + O(1e-8), which an FP64 run would add to the mass at every collision.
template <int Q>
__host__ __device__ constexpr double weight_d(int k) {
    return Q == 9 ? (speed2<Q>(k) == 0 ? 4. / 9. : speed2<Q>(k) == 1 ? 1. / 9. : 1. / 36.)
         : Q == 19 ? (speed2<Q>(k) == 0 ? 1. / 3. : speed2<Q>(k) == 1 ? 1. / 18. : 1. / 36.)
         : (speed2<Q>(k) == 0 ? 8. / 27. : speed2<Q>(k) == 1 ? 2. / 27. : speed2<Q>(k) == 2 ? 1. / 54. : 1. / 216.);
}

// ---------------------------------------------------------------------------
// device layout
// ---------------------------------------------------------------------------
// Populations are structure-of-arrays: direction k occupies its own plane of
// ks elements.  Inside a plane the box is z-major, rows of `ys` elements
// (pitched), with `h` halo layers on every axis.  Interior coordinates are
// 0-based; the reference's coordinate is this + 1.  The first interior
// element of every row sits at element `xoff` of the row, which is 32-byte
// aligned, so warps read and write whole sectors.
struct Geo {
    int nx, ny, nz;   // interior extents
    int h;            // halo layers (1 under REFERENCE semantics, 0 under NATIVE)
    int xoff;         // element offset of x = 0 inside a row
    long long ys;     // row pitch (elements)
    long long zs;     // plane pitch (elements)
    long long fs;     // elements of one scalar field (zs * (nz + 2h))
    long long ks;     // plane pitch of every multi-component array: population
                      // direction k and velocity component d start at k*ks
                      // and d*ks (fs rounded up to 64 elements)
    int wrap_x, wrap_y, wrap_z;   // NATIVE: axis is periodic

    __host__ __device__ long long idx(int x, int y, int z) const {
        return (long long)(z + h) * zs + (long long)(y + h) * ys + (long long)(x + xoff);
    }
    __host__ __device__ long long cells() const { return (long long)nx * ny * nz; }
};

// ---------------------------------------------------------------------------
// per-node arithmetic
// ---------------------------------------------------------------------------
// Parameters of the collision, derived on the host exactly as plbpd does
// (src/CollisionSRT.cpp:19-20, src/Boundary.cpp:27).
struct CollideParams {
    float tau, omega, omc;    // omc = 1.0f - omega (float subtraction)
    float fx, fy, fz;         // body force
    // TRT: odd-moment rate 1/tau_m (float and double) and the source factors
    // gp = 1 - omega/2, gm = 1 - omega_m/2 (float arithmetic)
    float omega_m, gp, gm;
    double omega_m_d;
    // -0.0f, known only at run time: the addend that makes a fused
    // multiply-add an exact product the paired-FP32 code can use where a
    // product feeds a sum (native_impl.cuh, mulx2)
    float neg_zero = -0.0f;
};

// FP16 storage holds h = binary16(d * 2^12), d = f - w.  The power-of-2
// scale is exact both ways and moves binary16's normal range (down to
// 6.1e-5) to 1.5e-8 in d, so the small deviations of slow flows keep all 11
// bits instead of falling into subnormals; |d| must stay below 16.
constexpr int kHalfShift = 12;
constexpr float kHalfScale = 4096.0f;
constexpr float kHalfUnscale = 1.0f / 4096.0f;

// 2^sc and 2^-sc for the deviation arithmetic's scale (0 or kHalfShift).
__host__ __device__ constexpr float pow2f(int sc) { return sc == 0 ? 1.0f : sc == kHalfShift ? kHalfScale : 0.0f; }
__host__ __device__ constexpr float pow2f_neg(int sc) { return sc == 0 ? 1.0f : sc == kHalfShift ? kHalfUnscale : 0.0f; }

// Kernel arithmetic: plbpd's (FP32 body + FP64 tail), FP32 only, or the
// two-relaxation-time operator (FP32 arithmetic).
enum Arith : int { kArithReference = 0, kArithFP32 = 1, kArithTRT = 2 };

// Sums of one node in direction order: r = sum f_k, j = sum c_k f_k.  c is
// -1, 0 or 1, so f*c is exact and adding the zero products leaves every
// partial sum unchanged; they are skipped.
template <int Q>
__device__ __forceinline__ void node_sums(const float (&f)[Q], float& r, float& jx, float& jy, float& jz) {
    r = 0.0f; jx = 0.0f; jy = 0.0f; jz = 0.0f;
#pragma unroll
    for (int k = 0; k < Q; ++k) {
        r = __fadd_rn(r, f[k]);
        if (Lattice<Q>::cx(k) > 0) jx = __fadd_rn(jx, f[k]);
        if (Lattice<Q>::cx(k) < 0) jx = __fsub_rn(jx, f[k]);
        if (Lattice<Q>::cy(k) > 0) jy = __fadd_rn(jy, f[k]);
        if (Lattice<Q>::cy(k) < 0) jy = __fsub_rn(jy, f[k]);
        if (Lattice<Q>::cz(k) > 0) jz = __fadd_rn(jz, f[k]);
        if (Lattice<Q>::cz(k) < 0) jz = __fsub_rn(jz, f[k]);
    }
}

// Moments of one node, op for op as CalcMoments::_get_local_moments
// (src/CalcMoments.hpp:22-37): sums in direction order, then one reciprocal
// and three products.
template <int Q>
__device__ __forceinline__ void node_moments(const float (&f)[Q], float& rho, float& ux, float& uy, float& uz) {
    float r, jx, jy, jz;
    node_sums<Q>(f, r, jx, jy, jz);
    const float rinv = __fdiv_rn(1.0f, r);
    rho = r;
    ux = __fmul_rn(jx, rinv);
    uy = __fmul_rn(jy, rinv);
    uz = __fmul_rn(jz, rinv);
}

// c_k . u with plbpd's association ((c0 u0 + c1 u1) + c2 u2).  Products with
// c in {-1,0,1} are exact and a signed zero never changes a later sum except
// in its own sign, which no caller can observe, so only the nonzero terms are
// added, in order.
template <int Q>
__device__ __forceinline__ float dot_c(int k, float ux, float uy, float uz) {
    float acc = 0.0f;
    bool any = false;
    if (Lattice<Q>::cx(k) != 0) { acc = Lattice<Q>::cx(k) > 0 ? ux : -ux; any = true; }
    if (Lattice<Q>::cy(k) != 0) {
        const float t = Lattice<Q>::cy(k) > 0 ? uy : -uy;
        acc = any ? __fadd_rn(acc, t) : t;
        any = true;
    }
    if (Lattice<Q>::cz(k) != 0) {
        const float t = Lattice<Q>::cz(k) > 0 ? uz : -uz;
        acc = any ? __fadd_rn(acc, t) : t;
    }
    return acc;
}

// BGK collision of one node in place, with the rounding of plbpd's AVX2
// kernel (src/CollisionSRT.cpp:71-148):
//   u_eq = u + F * (tau / rho)                      (float)
//   usq  = ((ux*ux + uy*uy) + uz*uz)                (float)
//   body: neq = fma(3, cu, 1); neq = fma(4.5, cu*cu, neq); neq += -1.5*usq;
//         neq = (neq*rho)*w;  n = fma(1-omega, n, omega*neq)
//   tail (k >= 8*floor(Q/8), REFERENCE arithmetic only): the bracket
//         1 + 3cu + 4.5cu^2 - 1.5usq in FP64 times the float w*rho, then
//         (1-omega)*n (float) + omega*neq in FP64, rounded to float; the
//         result is formed from FP32 instructions (tail_exact.h).
// ---- TRT ----------------------------------------------------------------------
// Two relaxation times with a second-order force source (the oracle's
// orc_set_trt states the method); pairs (k, k + 1) with k odd are opposite
// directions.  DEV: populations are deviations d = f - w (FP16 storage), so
// the even equilibrium enters as e+ - w = w (drho + rho (4.5cu^2 - 1.5usq)).
// Op order, FP32:
//   hr = 0.5/rho; v = u + F hr; vsq = (vx^2 + vy^2) + vz^2; uF = (vx Fx + vy Fy) + vz Fz
//   kusq = -1.5 vsq; base = 1 + kusq; m3uF = -3 uF
//   e0 = (w0 rho) base | fma(w0 rho, kusq, w0 drho);  n0 = (n0 - om (n0 - e0)) + (gp w0) m3uF
//   per pair: t = 4.5 cu; e+ = (w rho) fma(t, cu, base) | fma(w rho, fma(t, cu, kusq), w drho)
//     e- = (w rho)(3 cu); s+ = 0.5 (nk + nr); s- = 0.5 (nk - nr)
//     a = om (s+ - e+); b = omm (s- - e-); S+ = (gp w) fma(9 cu, cF, m3uF); S- = (gm w)(3 cF)
//     nk = ((nk - a) - b) + (S+ + S-); nr = ((nr - a) + b) + (S+ - S-)
//
// SC: the populations (and drho) are deviations times 2^SC (FP16 storage
// keeps them so).  Every term is then the unscaled one times 2^SC: the
// weights that multiply rho, gp w and gm w carry the factor, which is exact,
// so the result is the unscaled operator's, times 2^SC, bit for bit.
template <int Q, bool DEV, int SC = 0>
__device__ __forceinline__ void collide_node_trt(float (&f)[Q], float drho, float rho, float ux, float uy, float uz,
                                                 const CollideParams& P) {
    constexpr float S = pow2f(SC);
    // 0.5 (1/rho) is 0.5/rho exactly (a power-of-2 factor), and 1/rho is the
    // moments' reciprocal, which the compiler shares
    const float hr = __fmul_rn(0.5f, __fdiv_rn(1.0f, rho));
    const float vx = __fadd_rn(ux, __fmul_rn(P.fx, hr));
    const float vy = __fadd_rn(uy, __fmul_rn(P.fy, hr));
    const float vz = __fadd_rn(uz, __fmul_rn(P.fz, hr));
    const float vsq = __fadd_rn(__fadd_rn(__fmul_rn(vx, vx), __fmul_rn(vy, vy)), __fmul_rn(vz, vz));
    const float uF = __fadd_rn(__fadd_rn(__fmul_rn(vx, P.fx), __fmul_rn(vy, P.fy)), __fmul_rn(vz, P.fz));
    const float kusq = __fmul_rn(-1.5f, vsq);
    const float base = __fadd_rn(1.0f, kusq);
    const float m3uF = __fmul_rn(-3.0f, uF);
    const float om = P.omega, omm = P.omega_m;
    {
        const float w0 = weight<Q>(0), wr0 = __fmul_rn(w0 * S, rho);
        const float e0 = DEV ? __fmaf_rn(wr0, kusq, __fmul_rn(w0, drho)) : __fmul_rn(wr0, base);
        f[0] = __fadd_rn(__fsub_rn(f[0], __fmul_rn(om, __fsub_rn(f[0], e0))),
                         __fmul_rn(__fmul_rn(__fmul_rn(P.gp, w0), S), m3uF));
    }
#pragma unroll
    for (int k = 1; k < Q; k += 2) {
        const float w = weight<Q>(k), wr = __fmul_rn(w * S, rho);
        const float cu = dot_c<Q>(k, vx, vy, vz);
        const float cF = dot_c<Q>(k, P.fx, P.fy, P.fz);
        const float t = __fmul_rn(4.5f, cu);
        const float ep = DEV ? __fmaf_rn(wr, __fmaf_rn(t, cu, kusq), __fmul_rn(w, drho))
                             : __fmul_rn(wr, __fmaf_rn(t, cu, base));
        const float em = __fmul_rn(wr, __fmul_rn(3.0f, cu));
        const float sp = __fmul_rn(0.5f, __fadd_rn(f[k], f[k + 1]));
        const float sm = __fmul_rn(0.5f, __fsub_rn(f[k], f[k + 1]));
        const float a = __fmul_rn(om, __fsub_rn(sp, ep));
        const float b = __fmul_rn(omm, __fsub_rn(sm, em));
        const float Sp = __fmul_rn(__fmul_rn(__fmul_rn(P.gp, w), S), __fmaf_rn(__fmul_rn(9.0f, cu), cF, m3uF));
        const float Sm = __fmul_rn(__fmul_rn(__fmul_rn(P.gm, w), S), __fmul_rn(3.0f, cF));
        const float nk = __fadd_rn(__fsub_rn(__fsub_rn(f[k], a), b), __fadd_rn(Sp, Sm));
        const float nr = __fadd_rn(__fadd_rn(__fsub_rn(f[k + 1], a), b), __fsub_rn(Sp, Sm));
        f[k] = nk;
        f[k + 1] = nr;
    }
}

// Under kArithFP32 the body's sequence is used for every direction; under
// kArithTRT the two-relaxation-time operator above replaces BGK.
template <int Q, int ARITH>
__device__ __forceinline__ void collide_node(float (&f)[Q], float rho, float ux, float uy, float uz,
                                             const CollideParams& P) {
    if constexpr (ARITH == kArithTRT) {
        collide_node_trt<Q, false>(f, 0.0f, rho, ux, uy, uz, P);
        return;
    }
    const float tr = __fdiv_rn(P.tau, rho);
    const float vx = __fadd_rn(ux, __fmul_rn(P.fx, tr));
    const float vy = __fadd_rn(uy, __fmul_rn(P.fy, tr));
    const float vz = __fadd_rn(uz, __fmul_rn(P.fz, tr));
    const float usq = __fadd_rn(__fadd_rn(__fmul_rn(vx, vx), __fmul_rn(vy, vy)), __fmul_rn(vz, vz));
    const float kusq = __fmul_rn(-1.5f, usq);
    const float om = P.omega, omc = P.omc;
    constexpr int kBody = (ARITH == kArithReference) ? (Q / 8) * 8 : Q;
    const tx::TailNode tnode = tx::tail_node(usq);
#pragma unroll
    for (int k = 0; k < Q; ++k) {
        const float cu = (k == 0) ? 0.0f : dot_c<Q>(k, vx, vy, vz);
        if (k < kBody) {
            const float cusq = __fmul_rn(cu, cu);
            float neq = __fmaf_rn(3.0f, cu, 1.0f);
            neq = __fmaf_rn(4.5f, cusq, neq);
            neq = __fadd_rn(neq, kusq);
            neq = __fmul_rn(neq, rho);
            neq = __fmul_rn(neq, weight<Q>(k));
            f[k] = __fmaf_rn(omc, f[k], __fmul_rn(om, neq));
        } else {
            // the reference's double-precision tail, reproduced bit for bit
            // from FP32 instructions (tail_exact.h); the rare lanes whose
            // result lies too close to a rounding boundary run it in FP64
            const float wr = __fmul_rn(weight<Q>(k), rho);
            const float a = __fmul_rn(omc, f[k]);
            f[k] = tx::tail_update(cu, usq, tnode, wr, om, a);
        }
    }
}

// Moving-wall term of plbpd's no-slip rule (src/Boundary.cpp:215-217):
//   2.0f * w_k * rho_nbr * (c_k . u_b) * (1/c_s^2), left to right in float.
template <int Q>
__device__ __forceinline__ float wall_term(int k, float rho_nbr, float cub, float cs2inv) {
    return __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(2.0f, weight<Q>(k)), rho_nbr), cub), cs2inv);
}

// c_k . u_b exactly as the reference forms it: ((c0*ub0 + c1*ub1) + c2*ub2)
// with the int velocity components converted to float.
template <int Q>
__device__ __forceinline__ float dot_c_full(int k, const float* ub) {
    const float a = __fmul_rn((float)Lattice<Q>::cx(k), ub[0]);
    const float b = __fmul_rn((float)Lattice<Q>::cy(k), ub[1]);
    const float c = __fmul_rn((float)Lattice<Q>::cz(k), ub[2]);
    return __fadd_rn(__fadd_rn(a, b), c);
}

}  // namespace plb
