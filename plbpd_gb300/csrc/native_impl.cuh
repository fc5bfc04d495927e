// Native-semantics kernel templates and their host-side dispatch, shared by
// kernels_native.cu (BGK instantiations) and kernels_trt.cu (TRT).
//
// The device holds P, the post-collision populations of the previous step.
// A step at node x gathers n[x][k] = P[x - c_k][k] (periodic axes wrap), or,
// when x - c_k is solid, the bounce-back value P[x][rev k] that node x itself
// stored with the moving-wall term already applied; then it computes the
// moments, collides and stores P[x][k] at its own node.  Reads of a shifted
// row are misaligned by one element, writes are whole aligned sectors.
//
// The bounce-back is plbpd's no-slip rule (src/Boundary.cpp:189-221) for a
// fluid node next to a solid one:
//   n[x][rev k] = P[x][k] - 2 w_k rho[x] (c_k . u_b) / c_s^2,  x + c_k solid,
// with rho[x] the density node x collided with -- available in registers when
// P[x][k] is stored, so the term is applied on the store side.
//
// Storage (template parameter ST):
//   0  FP32 populations, plbpd's FP32 arithmetic (or FP32-only, ARITH)
//   1  FP16 deviations d_k = f_k - w_k, arithmetic in FP32 in deviation form
//   2  FP64 populations and FP64 arithmetic: the reference run of the same
//      method that reduced-precision runs are measured against
//   3  FP32 deviations d_k = f_k - w_k, FP16's arithmetic without its rounding:
//      FP32 cost, with the precision kept where the flow is (f - w is small)
#pragma once

#include <type_traits>

#include "engine.h"

namespace plb {
namespace {

constexpr int kBlockX = 128;

// Thread blocks of the hot per-node kernels are one segment of a row: 4 warps
// along x (128 threads) when the row is a whole number of such blocks long,
// else one warp, so a row of any length leaves at most one warp partly idle.
// The row (y, z) comes from the block index alone, which keeps the row
// offsets warp-uniform (they live in uniform registers); a thread index in
// them costs registers and occupancy.  BX is the block width.
inline int block_x(const Geo& g, int nodes_per_thread) {
    return g.nx % (kBlockX * nodes_per_thread) == 0 ? kBlockX : 32;
}

inline dim3 seg_grid(const Geo& g, int bx, int nodes_per_thread) {
    const long long xs = (long long)bx * nodes_per_thread;
    return dim3((unsigned)((g.nx + xs - 1) / xs), (unsigned)g.ny, (unsigned)g.nz);
}

// Storage accessors: ld reads through the read-only path (buffers the kernel
// does not write), ldp is a plain load (the in-place AA kernels), st streams.
template <int ST> struct Store;
template <> struct Store<0> {
    using T = float;
    using R = float;
    __device__ static __forceinline__ float ld(const float* p, long long i) { return __ldg(p + i); }
    __device__ static __forceinline__ float ldp(const float* p, long long i) { return p[i]; }
    __device__ static __forceinline__ void st(float* p, long long i, float v) { __stcs(p + i, v); }
};
template <> struct Store<1> {
    using T = __half;
    using R = float;
    // the stored value x = 2^12 d; the kernels compute on x (SC = kHalfShift)
    __device__ static __forceinline__ float ld(const __half* p, long long i) { return __half2float(__ldg(p + i)); }
    __device__ static __forceinline__ float ldp(const __half* p, long long i) { return __half2float(p[i]); }
    __device__ static __forceinline__ void st(__half* p, long long i, float v) {
        __stcs(reinterpret_cast<unsigned short*>(p) + i, __half_as_ushort(__float2half_rn(v)));
    }
};
// FP32 deviations d = f - w: the FP16 storage's arithmetic without its rounding
template <> struct Store<3> {
    using T = float;
    using R = float;
    __device__ static __forceinline__ float ld(const float* p, long long i) { return __ldg(p + i); }
    __device__ static __forceinline__ float ldp(const float* p, long long i) { return p[i]; }
    __device__ static __forceinline__ void st(float* p, long long i, float v) { __stcs(p + i, v); }
};
// The scale of a storage's deviation arithmetic: FP16 computes on 2^12 d.
template <int ST>
__host__ __device__ constexpr int dev_shift() { return ST == 1 ? kHalfShift : 0; }

template <> struct Store<2> {
    using T = double;
    using R = double;
    __device__ static __forceinline__ double ld(const double* p, long long i) { return __ldg(p + i); }
    __device__ static __forceinline__ double ldp(const double* p, long long i) { return p[i]; }
    __device__ static __forceinline__ void st(double* p, long long i, double v) { __stcs(p + i, v); }
};

// A population load: through the read-only path (the buffer is not written
// while the kernel runs), or, CG, cached in L2 only -- the multi-step batch
// kernel reads in one step what other SMs wrote in the previous one, which
// an SM's L1 or read-only cache may still hold from two steps before.
template <int ST, bool CG>
__device__ __forceinline__ typename Store<ST>::R ld_pop(const typename Store<ST>::T* p, long long i) {
    if constexpr (!CG) return Store<ST>::ld(p, i);
    else if constexpr (ST == 1) return __half2float(__ldcg(p + i));
    else return __ldcg(p + i);
}

// A one-node kernel's pull of a whole row (the streaming loads): as ld_pop,
// with 256-byte L2 fills as the pair kernels' row loads.
template <int ST, bool CG>
__device__ __forceinline__ typename Store<ST>::R ld_pull(const typename Store<ST>::T* p, long long i) {
    if constexpr (CG || ST == 2) {
        return ld_pop<ST, CG>(p, i);
    } else if constexpr (ST == 1) {
        unsigned short r;
        asm("ld.global.nc.L2::256B.b16 %0, [%1];" : "=h"(r) : "l"(p + i));
        return __half2float(__ushort_as_half(r));
    } else {
        float r;
        asm("ld.global.nc.L2::256B.f32 %0, [%1];" : "=f"(r) : "l"(p + i));
        return r;
    }
}

// Neighbour index helper: element offsets of x-1, x, x+1 (and y, z) with the
// periodic axes wrapped.  A fluid node never has a neighbour outside the box
// along a walled axis, because the wall layer in between is solid, so kernels
// index a node's neighbours only after they know it is fluid.
struct Nbr {
    long long xo[3], yo[3], zo[3];
    __device__ __forceinline__ Nbr(const Geo& g, int x, int y, int z) {
        const int xm = (x == 0 && g.wrap_x) ? g.nx - 1 : x - 1;
        const int xp = (x == g.nx - 1 && g.wrap_x) ? 0 : x + 1;
        const int ym = (y == 0 && g.wrap_y) ? g.ny - 1 : y - 1;
        const int yp = (y == g.ny - 1 && g.wrap_y) ? 0 : y + 1;
        const int zm = (z == 0 && g.wrap_z) ? g.nz - 1 : z - 1;
        const int zp = (z == g.nz - 1 && g.wrap_z) ? 0 : z + 1;
        xo[0] = xm + g.xoff; xo[1] = x + g.xoff; xo[2] = xp + g.xoff;
        yo[0] = (long long)ym * g.ys; yo[1] = (long long)y * g.ys; yo[2] = (long long)yp * g.ys;
        zo[0] = (long long)zm * g.zs; zo[1] = (long long)z * g.zs; zo[2] = (long long)zp * g.zs;
    }
    // node at x + s*c_k, s = +1 (downstream) or -1 (upstream)
    template <int Q>
    __device__ __forceinline__ long long at(int k, int s) const {
        return zo[1 + s * Lattice<Q>::cz(k)] + yo[1 + s * Lattice<Q>::cy(k)] + xo[1 + s * Lattice<Q>::cx(k)];
    }
};

// ---- FP16 storage: deviation form -----------------------------------------
// d_k = f_k - w_k, drho = sum d_k, rho = 1 + drho, and
//   f_eq,k - w_k = w_k (drho + rho X_k),  X_k = 3 cu + 4.5 cu^2 - 1.5 usq,
//   d'_k = (1 - omega) d_k + omega (f_eq,k - w_k).
// Written for few operations: per weight class A = w (omega rho) and
// B = w (omega drho), then per direction
//   X = fma(cu, fma(4.5, cu, 3), -1.5 usq),  d' = fma(1 - omega, d, fma(A, X, B)).
// SC: d and drho are deviations times 2^SC (FP16 storage keeps x = 2^12 d);
// A then takes the factor through w 2^SC, B through drho, so every result is
// the unscaled one times 2^SC, bit for bit (power-of-2 factors are exact).
template <int Q, int SC = 0>
__device__ __forceinline__ void collide_node_dev(float (&d)[Q], float drho, float rho, float ux, float uy,
                                                 float uz, const CollideParams& P) {
    // tau (1/rho): the reciprocal is the moments' (the compiler shares it)
    const float tr = __fmul_rn(P.tau, __fdiv_rn(1.0f, rho));
    const float vx = __fadd_rn(ux, __fmul_rn(P.fx, tr));
    const float vy = __fadd_rn(uy, __fmul_rn(P.fy, tr));
    const float vz = __fadd_rn(uz, __fmul_rn(P.fz, tr));
    const float usq = __fadd_rn(__fadd_rn(__fmul_rn(vx, vx), __fmul_rn(vy, vy)), __fmul_rn(vz, vz));
    const float kusq = __fmul_rn(-1.5f, usq);
    const float orho = __fmul_rn(P.omega, rho);
    const float odrho = __fmul_rn(P.omega, drho);
#pragma unroll
    for (int k = 0; k < Q; ++k) {
        const float cu = (k == 0) ? 0.0f : dot_c<Q>(k, vx, vy, vz);
        const float A = __fmul_rn(weight<Q>(k) * pow2f(SC), orho);   // shared by a weight class after CSE
        const float B = __fmul_rn(weight<Q>(k), odrho);
        const float X = __fmaf_rn(cu, __fmaf_rn(4.5f, cu, 3.0f), kusq);
        d[k] = __fmaf_rn(P.omc, d[k], __fmaf_rn(A, X, B));
    }
}

// Moments from (scaled) deviations: drho comes back scaled, rho and u do not
// (rho = 1 + 2^-SC drho and 1/rho 2^-SC are exact rescalings).
template <int Q, int SC = 0>
__device__ __forceinline__ void node_moments_dev(const float (&d)[Q], float& drho, float& rho, float& ux,
                                                 float& uy, float& uz) {
    float jx, jy, jz;
    node_sums<Q>(d, drho, jx, jy, jz);
    rho = SC ? __fmaf_rn(drho, pow2f_neg(SC), 1.0f) : __fadd_rn(1.0f, drho);
    float rinv = __fdiv_rn(1.0f, rho);
    if (SC) rinv = __fmul_rn(rinv, pow2f_neg(SC));
    ux = __fmul_rn(jx, rinv);
    uy = __fmul_rn(jy, rinv);
    uz = __fmul_rn(jz, rinv);
}

// ---- FP64 storage: the same method in double ---------------------------------
// With the exact weights in double (weight_d).
// Op order: u_eq = u + F (tau/rho); usq = (ux^2 + uy^2) + uz^2;
// neq = (w rho)(((1 + 3cu) + (4.5cu)cu) - 1.5usq); n = (1-omega) n + omega neq.
template <int Q>
__device__ __forceinline__ double dot_c_d(int k, double ux, double uy, double uz) {
    double acc = 0.0;
    bool any = false;
    if (Lattice<Q>::cx(k) != 0) { acc = Lattice<Q>::cx(k) > 0 ? ux : -ux; any = true; }
    if (Lattice<Q>::cy(k) != 0) {
        const double t = Lattice<Q>::cy(k) > 0 ? uy : -uy;
        acc = any ? __dadd_rn(acc, t) : t;
        any = true;
    }
    if (Lattice<Q>::cz(k) != 0) {
        const double t = Lattice<Q>::cz(k) > 0 ? uz : -uz;
        acc = any ? __dadd_rn(acc, t) : t;
    }
    return acc;
}

template <int Q>
__device__ __forceinline__ void node_moments_d(const double (&f)[Q], double& rho, double& ux, double& uy,
                                               double& uz) {
    double r = 0.0, jx = 0.0, jy = 0.0, jz = 0.0;
#pragma unroll
    for (int k = 0; k < Q; ++k) {
        r = __dadd_rn(r, f[k]);
        if (Lattice<Q>::cx(k) > 0) jx = __dadd_rn(jx, f[k]);
        if (Lattice<Q>::cx(k) < 0) jx = __dsub_rn(jx, f[k]);
        if (Lattice<Q>::cy(k) > 0) jy = __dadd_rn(jy, f[k]);
        if (Lattice<Q>::cy(k) < 0) jy = __dsub_rn(jy, f[k]);
        if (Lattice<Q>::cz(k) > 0) jz = __dadd_rn(jz, f[k]);
        if (Lattice<Q>::cz(k) < 0) jz = __dsub_rn(jz, f[k]);
    }
    const double rinv = __ddiv_rn(1.0, r);
    rho = r;
    ux = __dmul_rn(jx, rinv);
    uy = __dmul_rn(jy, rinv);
    uz = __dmul_rn(jz, rinv);
}

template <int Q>
__device__ __forceinline__ void collide_node_d(double (&f)[Q], double rho, double ux, double uy, double uz,
                                               const CollideParams& P) {
    const double tau = (double)P.tau;
    const double omega = __ddiv_rn(1.0, tau);
    const double omc = __dsub_rn(1.0, omega);
    const double tr = __ddiv_rn(tau, rho);
    const double vx = __dadd_rn(ux, __dmul_rn((double)P.fx, tr));
    const double vy = __dadd_rn(uy, __dmul_rn((double)P.fy, tr));
    const double vz = __dadd_rn(uz, __dmul_rn((double)P.fz, tr));
    const double usq = __dadd_rn(__dadd_rn(__dmul_rn(vx, vx), __dmul_rn(vy, vy)), __dmul_rn(vz, vz));
    const double k15 = __dmul_rn(1.5, usq);
#pragma unroll
    for (int k = 0; k < Q; ++k) {
        const double cu = (k == 0) ? 0.0 : dot_c_d<Q>(k, vx, vy, vz);
        double br = __dadd_rn(1.0, __dmul_rn(3.0, cu));
        br = __dadd_rn(br, __dmul_rn(__dmul_rn(4.5, cu), cu));
        br = __dsub_rn(br, k15);
        const double neq = __dmul_rn(__dmul_rn(weight_d<Q>(k), rho), br);
        f[k] = __dadd_rn(__dmul_rn(omc, f[k]), __dmul_rn(omega, neq));
    }
}

// ---- TRT, FP64 storage (the FP32 operator is collide_node_trt in lattice.cuh) ----
// The same in double (FP64 storage): omega = 1/tau and gp = 1 - omega/2 in
// double, omm = omega_m_d, gm = 1 - omm/2; e+ = (w rho)((1 + (4.5cu)cu) - 1.5vsq),
// S+ = (gp w)((9cu) cF + m3uF); otherwise the FP32 order.
template <int Q>
__device__ __forceinline__ void collide_node_trt_d(double (&f)[Q], double rho, double ux, double uy, double uz,
                                                   const CollideParams& P) {
    const double om = __ddiv_rn(1.0, (double)P.tau), omm = P.omega_m_d;
    const double gp = __dsub_rn(1.0, __dmul_rn(0.5, om)), gm = __dsub_rn(1.0, __dmul_rn(0.5, omm));
    const double Fx = P.fx, Fy = P.fy, Fz = P.fz;
    const double hr = __ddiv_rn(0.5, rho);
    const double vx = __dadd_rn(ux, __dmul_rn(Fx, hr));
    const double vy = __dadd_rn(uy, __dmul_rn(Fy, hr));
    const double vz = __dadd_rn(uz, __dmul_rn(Fz, hr));
    const double vsq = __dadd_rn(__dadd_rn(__dmul_rn(vx, vx), __dmul_rn(vy, vy)), __dmul_rn(vz, vz));
    const double uF = __dadd_rn(__dadd_rn(__dmul_rn(vx, Fx), __dmul_rn(vy, Fy)), __dmul_rn(vz, Fz));
    const double k15 = __dmul_rn(1.5, vsq), m3uF = __dmul_rn(-3.0, uF);
    {
        const double w0 = weight_d<Q>(0);
        const double e0 = __dmul_rn(__dmul_rn(w0, rho), __dsub_rn(1.0, k15));
        f[0] = __dadd_rn(__dsub_rn(f[0], __dmul_rn(om, __dsub_rn(f[0], e0))), __dmul_rn(__dmul_rn(gp, w0), m3uF));
    }
#pragma unroll
    for (int k = 1; k < Q; k += 2) {
        const double w = weight_d<Q>(k), wr = __dmul_rn(w, rho);
        const double cu = dot_c_d<Q>(k, vx, vy, vz);
        const double cF = dot_c_d<Q>(k, Fx, Fy, Fz);
        const double ep = __dmul_rn(wr, __dsub_rn(__dadd_rn(1.0, __dmul_rn(__dmul_rn(4.5, cu), cu)), k15));
        const double em = __dmul_rn(wr, __dmul_rn(3.0, cu));
        const double sp = __dmul_rn(0.5, __dadd_rn(f[k], f[k + 1]));
        const double sm = __dmul_rn(0.5, __dsub_rn(f[k], f[k + 1]));
        const double a = __dmul_rn(om, __dsub_rn(sp, ep));
        const double b = __dmul_rn(omm, __dsub_rn(sm, em));
        const double Sp = __dmul_rn(__dmul_rn(gp, w), __dadd_rn(__dmul_rn(__dmul_rn(9.0, cu), cF), m3uF));
        const double Sm = __dmul_rn(__dmul_rn(gm, w), __dmul_rn(3.0, cF));
        const double nk = __dadd_rn(__dsub_rn(__dsub_rn(f[k], a), b), __dadd_rn(Sp, Sm));
        const double nr = __dadd_rn(__dadd_rn(__dsub_rn(f[k + 1], a), b), __dsub_rn(Sp, Sm));
        f[k] = nk;
        f[k + 1] = nr;
    }
}

// ---- per storage: moments + collision, and the moving-wall correction ---------
// Collision of one node from its moments, per storage and operator.
template <int Q, int ST, int ARITH>
__device__ __forceinline__ void collide_any(typename Store<ST>::R (&f)[Q], typename Store<ST>::R rho,
                                            typename Store<ST>::R ux, typename Store<ST>::R uy,
                                            typename Store<ST>::R uz, float drho, const CollideParams& cp) {
    if constexpr (ST == 0) {
        collide_node<Q, ARITH>(f, rho, ux, uy, uz, cp);
    } else if constexpr (ST == 1 || ST == 3) {
        if constexpr (ARITH == kArithTRT) collide_node_trt<Q, true, dev_shift<ST>()>(f, drho, rho, ux, uy, uz, cp);
        else collide_node_dev<Q, dev_shift<ST>()>(f, drho, rho, ux, uy, uz, cp);
    } else {
        if constexpr (ARITH == kArithTRT) collide_node_trt_d<Q>(f, rho, ux, uy, uz, cp);
        else collide_node_d<Q>(f, rho, ux, uy, uz, cp);
    }
}

// drho of a RAW state's rho field, in the deviation arithmetic's scale.
template <int ST>
__device__ __forceinline__ float raw_drho(float rho) {
    if constexpr (ST == 1) return __fmul_rn(__fsub_rn(rho, 1.0f), kHalfScale);
    else if constexpr (ST == 3) return __fsub_rn(rho, 1.0f);
    else return 0.0f;
}

template <int Q, int ST, int ARITH>
__device__ __forceinline__ void update_node(typename Store<ST>::R (&f)[Q], typename Store<ST>::R& rho,
                                            const CollideParams& cp) {
    if constexpr (ST == 0) {
        float ux, uy, uz;
        node_moments<Q>(f, rho, ux, uy, uz);
        collide_any<Q, ST, ARITH>(f, rho, ux, uy, uz, 0.0f, cp);
    } else if constexpr (ST == 1 || ST == 3) {
        float drho, ux, uy, uz;
        node_moments_dev<Q, dev_shift<ST>()>(f, drho, rho, ux, uy, uz);
        collide_any<Q, ST, ARITH>(f, rho, ux, uy, uz, drho, cp);
    } else {
        double ux, uy, uz;
        node_moments_d<Q>(f, rho, ux, uy, uz);
        collide_any<Q, ST, ARITH>(f, rho, ux, uy, uz, 0.0f, cp);
    }
}

// ---- two nodes per instruction: Blackwell's paired FP32 operations ----------
// add/sub/mul/fma.rn.f32x2 apply one FP32 operation to both halves of a
// float2, each half rounded exactly as the scalar operation.  The FP16 pair
// kernel holds two x-neighbour nodes per thread; updating them through these
// operations, op for op as the scalar update_node<Q, 1, ARITH>, gives the
// same bits with half the FP32 math instructions (the divisions stay scalar:
// there is no paired divide).
//
// ptxas merges a paired multiply into a paired add or subtract that consumes
// it (a fused multiply-add, one rounding instead of two) even when the PTX
// names the rounding mode and -fmad=false is given, and it also recognises a
// multiply-add with a constant -0 addend as a multiply.  A product that feeds
// a sum is therefore formed by mulx2: a multiply-add whose -0 addend comes
// from the kernel parameters, which rounds exactly as the product (x*y + -0
// is x*y, zeros keep their sign) and cannot be merged further.
__device__ __forceinline__ float2 bc2(float a) { return make_float2(a, a); }
__device__ __forceinline__ unsigned long long f2bits(float2 a) {
    return *reinterpret_cast<const unsigned long long*>(&a);
}
__device__ __forceinline__ float2 bits2f(unsigned long long d) { return *reinterpret_cast<const float2*>(&d); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) {
    unsigned long long d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2bits(a)), "l"(f2bits(b)));
    return bits2f(d);
}
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
    unsigned long long d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2bits(a)), "l"(f2bits(b)));
    return bits2f(d);
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) {
    unsigned long long d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2bits(a)), "l"(f2bits(b)));
    return bits2f(d);
}
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(f2bits(a)), "l"(f2bits(b)), "l"(f2bits(c)));
    return bits2f(d);
}
__device__ __forceinline__ float2 mulx2(float2 a, float2 b, float2 nz) { return fma2(a, b, nz); }
__device__ __forceinline__ float2 div2(float a, float2 b) { return make_float2(__fdiv_rn(a, b.x), __fdiv_rn(a, b.y)); }

// v = (vx, vy, vz) and its negation nv, so that every c_k . v is the scalar
// dot_c's sum: a leading negative term is read from nv, a later one is a
// subtraction (x + (-y) and x - y are the same IEEE operation).
struct Vel2 {
    float2 v[3], nv[3];
};
template <int Q>
__device__ __forceinline__ float2 dot_c2(int k, const Vel2& u) {
    const int c[3] = {Lattice<Q>::cx(k), Lattice<Q>::cy(k), Lattice<Q>::cz(k)};
    float2 acc = bc2(0.0f);
    bool any = false;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (c[a] == 0) continue;
        if (!any) acc = c[a] > 0 ? u.v[a] : u.nv[a];
        else acc = c[a] > 0 ? add2(acc, u.v[a]) : sub2(acc, u.v[a]);
        any = true;
    }
    return acc;
}

// c_k . v for a direction k whose reverse comes after it (k odd): the scalar
// dot_c's sum, with a leading negative term folded into the following
// positive one ((-a) + b and b - a are the same IEEE operation); two leading
// negative terms negate their sum, which can differ from dot_c only in the
// sign of a zero.
template <int Q>
__device__ __forceinline__ float2 dot_c2_fwd(int k, const float2 (&v)[3]) {
    const int c[3] = {Lattice<Q>::cx(k), Lattice<Q>::cy(k), Lattice<Q>::cz(k)};
    float2 acc = bc2(0.0f);
    int n = 0;          // terms summed so far
    int lead = -1;      // a leading negative term not yet summed
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (c[a] == 0) continue;
        if (n == 0 && lead < 0 && c[a] < 0) { lead = a; continue; }
        if (lead >= 0) {
            acc = c[a] > 0 ? sub2(v[a], v[lead]) : mul2(bc2(-1.0f), add2(v[lead], v[a]));
            lead = -1;
            n = 2;
            continue;
        }
        acc = n == 0 ? v[a] : (c[a] > 0 ? add2(acc, v[a]) : sub2(acc, v[a]));
        ++n;
    }
    if (lead >= 0) acc = mul2(bc2(-1.0f), v[lead]);
    return acc;
}

template <int Q, int SC>
__device__ __forceinline__ void node_moments_dev2(const float2 (&d)[Q], float2& drho, float2& rho, float2& ux,
                                                  float2& uy, float2& uz, float2 nz) {
    float2 r = bc2(0.0f), jx = bc2(0.0f), jy = bc2(0.0f), jz = bc2(0.0f);
#pragma unroll
    for (int k = 0; k < Q; ++k) {
        r = add2(r, d[k]);
        if (Lattice<Q>::cx(k) > 0) jx = add2(jx, d[k]);
        if (Lattice<Q>::cx(k) < 0) jx = sub2(jx, d[k]);
        if (Lattice<Q>::cy(k) > 0) jy = add2(jy, d[k]);
        if (Lattice<Q>::cy(k) < 0) jy = sub2(jy, d[k]);
        if (Lattice<Q>::cz(k) > 0) jz = add2(jz, d[k]);
        if (Lattice<Q>::cz(k) < 0) jz = sub2(jz, d[k]);
    }
    drho = r;
    rho = SC ? fma2(r, bc2(pow2f_neg(SC)), bc2(1.0f)) : add2(bc2(1.0f), r);
    float2 rinv = div2(1.0f, rho);
    if (SC) rinv = mul2(rinv, bc2(pow2f_neg(SC)));
    ux = mulx2(jx, rinv, nz);
    uy = mulx2(jy, rinv, nz);
    uz = mulx2(jz, rinv, nz);
}

// collide_node_dev for two nodes.  NEG selects how c.v is formed: from v
// and -v for every direction (0), or for an even direction as the negated
// previous one (1); the two give the same bits and differ in registers.
template <int Q, bool NEG, int SC>
__device__ __forceinline__ void collide_node_dev2(float2 (&d)[Q], float2 drho, float2 rho, float2 ux, float2 uy,
                                                  float2 uz, const CollideParams& P) {
    const float2 nz = bc2(P.neg_zero);
    const float2 tr = mul2(bc2(P.tau), div2(1.0f, rho));   // tau (1/rho), as collide_node_dev
    Vel2 u;
    float2 (&v)[3] = u.v;
    v[0] = add2(ux, mulx2(bc2(P.fx), tr, nz));
    v[1] = add2(uy, mulx2(bc2(P.fy), tr, nz));
    v[2] = add2(uz, mulx2(bc2(P.fz), tr, nz));
    if (!NEG) {
#pragma unroll
        for (int a = 0; a < 3; ++a) u.nv[a] = mul2(bc2(-1.0f), v[a]);
    }
    const float2 usq = add2(add2(mulx2(v[0], v[0], nz), mulx2(v[1], v[1], nz)), mulx2(v[2], v[2], nz));
    const float2 kusq = mul2(bc2(-1.5f), usq);
    const float2 orho = mul2(bc2(P.omega), rho);
    const float2 odrho = mul2(bc2(P.omega), drho);
    // c_{k+1} = -c_k for odd k, so the even directions negate the previous
    // c.v.  A zero's sign cannot reach the result: X = +-0*3 + kusq is kusq,
    // or +-0 when kusq is -0, and then A X + B is B (B is never -0: the sum
    // drho starts from +0).
    float2 cu_prev = bc2(0.0f);
#pragma unroll
    for (int k = 0; k < Q; ++k) {
        const float2 cu = (k == 0) ? bc2(0.0f)
                          : !NEG   ? dot_c2<Q>(k, u)
                          : (k & 1) ? dot_c2_fwd<Q>(k, v)
                                    : mul2(bc2(-1.0f), cu_prev);
        cu_prev = cu;
        const float2 A = mul2(bc2(weight<Q>(k) * pow2f(SC)), orho);
        const float2 B = mul2(bc2(weight<Q>(k)), odrho);
        const float2 X = fma2(cu, fma2(bc2(4.5f), cu, bc2(3.0f)), kusq);
        d[k] = fma2(bc2(P.omc), d[k], fma2(A, X, B));
    }
}

// collide_node_trt<Q, true, SC> for two nodes
template <int Q, int SC>
__device__ __forceinline__ void collide_node_trt_dev2(float2 (&f)[Q], float2 drho, float2 rho, float2 ux, float2 uy,
                                                      float2 uz, const CollideParams& P) {
    const float2 nz = bc2(P.neg_zero);
    const float2 hr = mul2(bc2(0.5f), div2(1.0f, rho));   // = 0.5/rho exactly (power-of-2 factor)
    Vel2 u;
    u.v[0] = add2(ux, mulx2(bc2(P.fx), hr, nz));
    u.v[1] = add2(uy, mulx2(bc2(P.fy), hr, nz));
    u.v[2] = add2(uz, mulx2(bc2(P.fz), hr, nz));
#pragma unroll
    for (int a = 0; a < 3; ++a) u.nv[a] = mul2(bc2(-1.0f), u.v[a]);
    const float2 vsq =
        add2(add2(mulx2(u.v[0], u.v[0], nz), mulx2(u.v[1], u.v[1], nz)), mulx2(u.v[2], u.v[2], nz));
    const float2 uF = add2(add2(mulx2(u.v[0], bc2(P.fx), nz), mulx2(u.v[1], bc2(P.fy), nz)),
                           mulx2(u.v[2], bc2(P.fz), nz));
    const float2 kusq = mul2(bc2(-1.5f), vsq);
    const float2 m3uF = mul2(bc2(-3.0f), uF);
    const float2 om = bc2(P.omega), omm = bc2(P.omega_m);
    {
        const float w0 = weight<Q>(0);
        const float2 wr0 = mul2(bc2(w0 * pow2f(SC)), rho);
        const float2 e0 = fma2(wr0, kusq, mul2(bc2(w0), drho));
        f[0] = add2(sub2(f[0], mulx2(om, sub2(f[0], e0), nz)),
                    mulx2(bc2(__fmul_rn(__fmul_rn(P.gp, w0), pow2f(SC))), m3uF, nz));
    }
#pragma unroll
    for (int k = 1; k < Q; k += 2) {
        const float w = weight<Q>(k);
        const float2 wr = mul2(bc2(w * pow2f(SC)), rho);
        const float2 cu = dot_c2<Q>(k, u);
        const float cF = dot_c<Q>(k, P.fx, P.fy, P.fz);
        const float2 t = mul2(bc2(4.5f), cu);
        const float2 ep = fma2(wr, fma2(t, cu, kusq), mul2(bc2(w), drho));
        const float2 em = mulx2(wr, mul2(bc2(3.0f), cu), nz);
        const float2 sp = mulx2(bc2(0.5f), add2(f[k], f[k + 1]), nz);
        const float2 sm = mulx2(bc2(0.5f), sub2(f[k], f[k + 1]), nz);
        const float2 a = mulx2(om, sub2(sp, ep), nz);
        const float2 b = mulx2(omm, sub2(sm, em), nz);
        const float2 Sp =
            mulx2(bc2(__fmul_rn(__fmul_rn(P.gp, w), pow2f(SC))), fma2(mul2(bc2(9.0f), cu), bc2(cF), m3uF), nz);
        const float2 Sm = bc2(__fmul_rn(__fmul_rn(__fmul_rn(P.gm, w), pow2f(SC)), __fmul_rn(3.0f, cF)));
        const float2 nk = add2(sub2(sub2(f[k], a), b), add2(Sp, Sm));
        const float2 nr = add2(add2(sub2(f[k + 1], a), b), sub2(Sp, Sm));
        f[k] = nk;
        f[k + 1] = nr;
    }
}

// update_node<Q, ST, ARITH> of deviation storage (ST 1 or 3, scale SC) for
// two nodes.  NEG as in collide_node_dev2.
template <int Q, int ARITH, bool NEG, int SC>
__device__ __forceinline__ void update_pair_dev(float2 (&d)[Q], float2& rho, const CollideParams& cp) {
    float2 drho, ux, uy, uz;
    node_moments_dev2<Q, SC>(d, drho, rho, ux, uy, uz, bc2(cp.neg_zero));
    if constexpr (ARITH == kArithTRT) collide_node_trt_dev2<Q, SC>(d, drho, rho, ux, uy, uz, cp);
    else collide_node_dev2<Q, NEG, SC>(d, drho, rho, ux, uy, uz, cp);
}

// node_moments + collide_node<Q, kArithFP32> (plbpd's FP32 body sequence
// for every direction) for two nodes, op for op.
template <int Q, bool NEG>
__device__ __forceinline__ void update_pair_fp32(float2 (&f)[Q], float2& rho, const CollideParams& P) {
    const float2 nz = bc2(P.neg_zero);
    float2 r = bc2(0.0f), jx = bc2(0.0f), jy = bc2(0.0f), jz = bc2(0.0f);
#pragma unroll
    for (int k = 0; k < Q; ++k) {
        r = add2(r, f[k]);
        if (Lattice<Q>::cx(k) > 0) jx = add2(jx, f[k]);
        if (Lattice<Q>::cx(k) < 0) jx = sub2(jx, f[k]);
        if (Lattice<Q>::cy(k) > 0) jy = add2(jy, f[k]);
        if (Lattice<Q>::cy(k) < 0) jy = sub2(jy, f[k]);
        if (Lattice<Q>::cz(k) > 0) jz = add2(jz, f[k]);
        if (Lattice<Q>::cz(k) < 0) jz = sub2(jz, f[k]);
    }
    const float2 rinv = div2(1.0f, r);
    rho = r;
    const float2 tr = div2(P.tau, rho);
    Vel2 u;
    float2 (&v)[3] = u.v;
    v[0] = add2(mulx2(jx, rinv, nz), mulx2(bc2(P.fx), tr, nz));
    v[1] = add2(mulx2(jy, rinv, nz), mulx2(bc2(P.fy), tr, nz));
    v[2] = add2(mulx2(jz, rinv, nz), mulx2(bc2(P.fz), tr, nz));
    if (!NEG) {
#pragma unroll
        for (int a = 0; a < 3; ++a) u.nv[a] = mul2(bc2(-1.0f), v[a]);
    }
    const float2 usq = add2(add2(mulx2(v[0], v[0], nz), mulx2(v[1], v[1], nz)), mulx2(v[2], v[2], nz));
    const float2 kusq = mulx2(bc2(-1.5f), usq, nz);
    const float2 om = bc2(P.omega), omc = bc2(P.omc);
    // a zero's sign in c.v cannot reach the result: cu^2 is +0 and 3 cu + 1 is 1
    float2 cu_prev = bc2(0.0f);
#pragma unroll
    for (int k = 0; k < Q; ++k) {
        const float2 cu = (k == 0) ? bc2(0.0f)
                          : !NEG   ? dot_c2<Q>(k, u)
                          : (k & 1) ? dot_c2_fwd<Q>(k, v)
                                    : mul2(bc2(-1.0f), cu_prev);
        cu_prev = cu;
        const float2 cusq = mul2(cu, cu);
        float2 neq = fma2(bc2(3.0f), cu, bc2(1.0f));
        neq = fma2(bc2(4.5f), cusq, neq);
        neq = add2(neq, kusq);
        neq = mul2(neq, rho);
        neq = mul2(neq, bc2(weight<Q>(k)));
        f[k] = fma2(omc, f[k], mul2(om, neq));
    }
}

// The update of a pair kernel: FORM 0 and 1 paired (NEG = FORM == 0),
// FORM 2 the scalar update of each node (other registers and schedule).
template <int Q, int ST, int ARITH, int FORM>
__device__ __forceinline__ void update_pair(float2 (&d)[Q], float2& rho, const CollideParams& cp) {
    if constexpr (FORM == 2) {
        float a[Q], b[Q];
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            a[k] = d[k].x;
            b[k] = d[k].y;
        }
        update_node<Q, ST, ARITH>(a, rho.x, cp);
        update_node<Q, ST, ARITH>(b, rho.y, cp);
#pragma unroll
        for (int k = 0; k < Q; ++k) d[k] = make_float2(a[k], b[k]);
    } else if constexpr (ST == 0) {
        static_assert(ARITH == kArithFP32, "paired FP32 storage runs plbpd's FP32 body arithmetic only");
        update_pair_fp32<Q, FORM == 0>(d, rho, cp);
    } else {
        update_pair_dev<Q, ARITH, FORM == 0, dev_shift<ST>()>(d, rho, cp);
    }
}

template <int Q, int ST>
__device__ __forceinline__ void moments_any(const typename Store<ST>::R (&f)[Q], typename Store<ST>::R& rho,
                                            typename Store<ST>::R& ux, typename Store<ST>::R& uy,
                                            typename Store<ST>::R& uz) {
    if constexpr (ST == 0) node_moments<Q>(f, rho, ux, uy, uz);
    else if constexpr (ST == 1 || ST == 3) { float drho; node_moments_dev<Q, dev_shift<ST>()>(f, drho, rho, ux, uy, uz); }
    else node_moments_d<Q>(f, rho, ux, uy, uz);
}

// v - 2 w_k rho (c_k . u_b) / c_s^2, in the storage's arithmetic
template <int Q, int ST>
__device__ __forceinline__ typename Store<ST>::R wall_corrected(int k, typename Store<ST>::R v,
                                                                typename Store<ST>::R rho, const float* ub,
                                                                float cs2inv) {
    if constexpr (ST == 2) {
        const double cu = __dadd_rn(__dadd_rn(__dmul_rn((double)Lattice<Q>::cx(k), (double)ub[0]),
                                              __dmul_rn((double)Lattice<Q>::cy(k), (double)ub[1])),
                                    __dmul_rn((double)Lattice<Q>::cz(k), (double)ub[2]));
        const double t = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(2.0, weight_d<Q>(k)), rho), cu), (double)cs2inv);
        return __dsub_rn(v, t);
    } else {
        // FP16 storage: v is 2^12 times the deviation, so is the term (exact)
        const float t = wall_term<Q>(k, rho, dot_c_full<Q>(k, ub), cs2inv);
        return __fsub_rn(v, ST == 1 ? __fmul_rn(t, kHalfScale) : t);
    }
}

// Stores the collided populations of a fluid node; a direction that points
// into a solid node becomes the bounce-back slot and carries the moving-wall
// term (src/Boundary.cpp:215-217).
template <int Q, int ST, bool MASK, bool MOVING = true>
__device__ __forceinline__ void store_node(typename Store<ST>::T* __restrict__ dst, const Geo& g,
                                           const NativeParams& np, const uint8_t* __restrict__ types,
                                           uint32_t links, const Nbr& nb, long long node,
                                           typename Store<ST>::R rho, const typename Store<ST>::R (&f)[Q]) {
#pragma unroll
    for (int k = 0; k < Q; ++k) {
        typename Store<ST>::R v = f[k];
        // a resting solid adds nothing (the term is a signed zero)
        if (MASK && MOVING && k != 0 && np.moving && ((links >> k) & 1u)) {
            const uint8_t t = __ldg(types + nb.at<Q>(k, +1));
            v = wall_corrected<Q, ST>(k, v, rho, np.vel[t & kVelMask], np.cs2inv);
        }
        Store<ST>::st(dst, k * g.ks + node, v);
    }
}

// A solid node that shares a store sector with a fluid node (kSectorMate)
// stores the rest equilibrium w_k (a zero deviation in the deviation
// storages).  No fluid node's result depends on it: a fluid neighbour's
// bounce-back takes its own reversed slot, and a solid node reads back as 0.
// It only feeds the update that the solid half of a pair kernel's pair runs,
// where rest values keep that update finite (zeros would give rho = 0 and,
// with plbpd's arithmetic, send the tail to its FP64 fallback).
// The kernels store it through the fluid path's own store loop: a separate
// loop of stores in the solid branch changed the register allocation of the
// fluid path (the masked one-node kernel went from 56 to 80 registers).
template <int Q, int ST>
__device__ __forceinline__ void rest_state(typename Store<ST>::R (&f)[Q], typename Store<ST>::R& rho) {
    using R = typename Store<ST>::R;
#pragma unroll
    for (int k = 0; k < Q; ++k) f[k] = (ST == 1 || ST == 3) ? R(0) : R(weight<Q>(k));
    rho = R(1);
}

// A row load of the pair kernels through the read-only path with a 256-byte
// L2 fill: the next warp of the row reads the other half of the block.
__device__ __forceinline__ __half2 ld_row_h2(const __half2* p) {
    unsigned int r;
    asm("ld.global.nc.L2::256B.b32 %0, [%1];" : "=r"(r) : "l"(p));
    return *reinterpret_cast<const __half2*>(&r);
}
__device__ __forceinline__ float2 ld_row_f2(const float2* p) {
    float2 r;
    asm("ld.global.nc.L2::256B.v2.f32 {%0, %1}, [%2];" : "=f"(r.x), "=f"(r.y) : "l"(p));
    return r;
}

// The solid-link mask of a node (0 for nodes away from solids).
template <bool MASK>
__device__ __forceinline__ uint32_t links_of(const uint8_t t, const uint32_t* __restrict__ links, long long node) {
    return (MASK && (t & kNearSolid)) ? __ldg(links + node) : 0u;
}

// Gathers n[x][*] from P for a fluid node: the streaming loads, then the
// bounce-back fix-up.  Every source is inside the box (a solid source is a
// node too), so the streaming loads are unconditional; bounce-back directions
// are then replaced by the node's own reversed slot.  `links` bit k is set
// when x + c_k is solid, so the source x - c_k is solid when bit rev(k) is.
template <int Q, int ST, bool CG = false>
__device__ __forceinline__ void stream_loads(const typename Store<ST>::T* __restrict__ src, const Geo& g,
                                             const Nbr& nb, typename Store<ST>::R (&f)[Q]) {
#pragma unroll
    for (int k = 0; k < Q; ++k) f[k] = ld_pull<ST, CG>(src, k * g.ks + nb.at<Q>(k, -1));
}

template <int Q, int ST, bool CG = false>
__device__ __forceinline__ void bounce_fixup(const typename Store<ST>::T* __restrict__ src, const Geo& g,
                                             uint32_t links, long long node, typename Store<ST>::R (&f)[Q]) {
    if (links) {
#pragma unroll
        for (int k = 1; k < Q; ++k)
            if ((links >> rev_of(k)) & 1u) f[k] = ld_pop<ST, CG>(src, rev_of(k) * g.ks + node);
    }
}

template <int Q, int ST, bool MASK, bool CG = false>
__device__ __forceinline__ void gather_node(const typename Store<ST>::T* __restrict__ src, const Geo& g,
                                            uint32_t links, const Nbr& nb, long long node,
                                            typename Store<ST>::R (&f)[Q]) {
    stream_loads<Q, ST, CG>(src, g, nb, f);
    if (MASK) bounce_fixup<Q, ST, CG>(src, g, links, node, f);
}

// ---------------------------------------------------------------------------
template <int Q, int ST, bool MASK, int ARITH, int BX>
__global__ void __launch_bounds__(BX)
nat_fused_k(Geo g, CollideParams cp, NativeParams np, const typename Store<ST>::T* __restrict__ src,
            typename Store<ST>::T* __restrict__ dst, const uint8_t* __restrict__ types) {
    using R = typename Store<ST>::R;
    const int x = blockIdx.x * BX + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= g.nx) return;
    const long long node = g.idx(x, y, z);
    // the type is read first: loading a solid node's sources would cost
    // traffic in obstacle-filled regions (measured 15% slower on D3Q27 with
    // 15% solid spheres), more than the round trip it saves; the link word
    // is read beside it, so the bounce-back fix-ups wait one round trip less
    uint32_t L = 0;
    bool solid = false;
    if (MASK) {
        const uint8_t t = __ldg(types + node);
        const uint32_t lw = __ldg(np.links + node);
        if ((t & (kSolid | kSectorMate)) == kSolid) return;
        L = (t & kNearSolid) ? lw : 0u;
        solid = t & kSolid;
    }
    const Nbr nb(g, x, y, z);
    R f[Q];
    R rho;
    if (MASK && solid) {
        rest_state<Q, ST>(f, rho);
    } else {
        gather_node<Q, ST, MASK>(src, g, L, nb, node, f);
        update_node<Q, ST, ARITH>(f, rho, cp);
    }
    store_node<Q, ST, MASK>(dst, g, np, types, L, nb, node, rho, f);
}

// FP16 storage, two x-neighbour nodes per thread (x0 even, x0 + 1).  Every
// direction is read as one aligned half2 of the source row, so a warp moves
// 128 B per access as the FP32 kernel does.  For c_x = +1 the pair needs
// (x0 - 1, x0): the high half of the previous lane's pair; for c_x = -1 it
// needs (x0 + 1, x0 + 2): the low half of the next lane's pair; lanes at a
// warp or row edge load that one value themselves.  Rows are whole warps of
// the same row, so neighbouring lanes hold neighbouring x.  nx must be even.
// Arithmetic, rounding and bounce-back are those of the one-node kernel.
//
// Every lane in the row loads all its source rows, also when its own pair is
// solid: its neighbours take values from it through the shuffles, and for a
// diagonal direction those come from another row, where the node may be
// fluid.  The loads share one guard (the lane is inside the row) so that they
// issue together; a guard per direction splits them into separate branches
// and measured 1.6x (D3Q19) to 2.3x (D3Q27) slower.  A source row outside a
// walled axis only occurs for pairs in a wall row, which are solid and store
// nothing; its address is clamped to the pair's own row.
// One lane's pair (x0, x0 + 1) of row (y, z); every lane of the warp calls
// it together (the shuffles), lanes past the end of their row with
// active = false.  A lane's neighbour lane holds the neighbouring pair of the
// same row unless x0 is 0 or x0 + 2 is nx, which the edge loads cover.
//
// The same two-node scheme serves FP32 and FP32-deviation storage (ST 0 and
// 3: one aligned float2 a lane and direction), where it halves the
// instructions a node takes and doubles the bytes a thread has in flight.
template <int Q, bool MASK, bool MOVING, int ARITH, int FORM = 0, int ST = 1, bool CG = false, bool VOTE = false>
__device__ __forceinline__ void h2_pair(const Geo& g, const CollideParams& cp, const NativeParams& np,
                                        const typename Store<ST>::T* __restrict__ src,
                                        typename Store<ST>::T* __restrict__ dst, const uint8_t* __restrict__ types,
                                        int lane, int x0, int y, int z, bool active) {
    const unsigned kFull = 0xffffffffu;
    const int ym = y == 0 ? (g.wrap_y ? g.ny - 1 : y) : y - 1;
    const int yp = y == g.ny - 1 ? (g.wrap_y ? 0 : y) : y + 1;
    const int zm = z == 0 ? (g.wrap_z ? g.nz - 1 : z) : z - 1;
    const int zp = z == g.nz - 1 ? (g.wrap_z ? 0 : z) : z + 1;
    const long long yo[3] = {(long long)ym * g.ys, (long long)y * g.ys, (long long)yp * g.ys};
    const long long zo[3] = {(long long)zm * g.zs, (long long)z * g.zs, (long long)zp * g.zs};
    // the values the neighbouring lanes cannot provide
    const int xm = x0 == 0 ? (g.wrap_x ? g.nx - 1 : -1) : x0 - 1;
    const int xp2 = x0 + 2 >= g.nx ? (g.wrap_x ? x0 + 2 - g.nx : -1) : x0 + 2;
    const bool edge_lo = lane == 0 || x0 == 0;
    const bool edge_hi = lane == 31 || x0 + 2 >= g.nx;
    const long long node0 = zo[1] + yo[1] + x0;

    bool skip = !active;
    uint8_t t0 = 0, t1 = 0;
    uint32_t L0 = 0, L1 = 0;
    if (MASK && active) {
        // the pair's two link words are read beside its types, not after
        // them: the fix-up loads wait for one round trip instead of two
        const unsigned short tt = __ldg(reinterpret_cast<const unsigned short*>(types + node0));
        const uint2 lw = __ldg(reinterpret_cast<const uint2*>(np.links + node0));
        t0 = (uint8_t)(tt & 0xff);
        t1 = (uint8_t)(tt >> 8);
        // a solid pair whose store sector holds a fluid node runs the update
        // on what it pulled and stores it, so that the sector is written
        // whole; not with plbpd's arithmetic, where such a pair (often at
        // rest, u = 0) would take the tail's FP64 fallback (measured 31k ->
        // 20k MLUPS on a D3Q19 duct with spheres)
        skip = (t0 & kSolid) && (t1 & kSolid) && (ARITH == kArithReference || !((t0 | t1) & kSectorMate));
        L0 = (t0 & kNearSolid) ? lw.x : 0u;
        L1 = (t1 & kNearSolid) ? lw.y : 0u;
    }
    // batch tasks: a warp of solid pairs (a wall plane or row of a small
    // domain, an obstacle's inside) needs no loads.  Not in the fused kernels:
    // there the vote makes every warp's population loads wait for its type
    // loads (D3Q27 duct with spheres, FP16: 40.5k -> 36.5k MLUPS), while
    // wall rows are few; a batch of small walled domains gained 4 %.
    if (MASK && VOTE && __all_sync(kFull, skip)) return;
    float2 f[Q];   // .x node x0, .y node x0 + 1
#pragma unroll
    for (int k = 0; k < Q; ++k) {
        const int cx = Lattice<Q>::cx(k), cy = Lattice<Q>::cy(k), cz = Lattice<Q>::cz(k);
        const long long row = (long long)k * g.ks + zo[1 - cz] + yo[1 - cy];
        float2 v = make_float2(0.0f, 0.0f);
        if (active) {
            if constexpr (ST == 1) {
                const __half2* a = reinterpret_cast<const __half2*>(src + row + x0);
                v = __half22float2(CG ? __ldcg(a) : ld_row_h2(a));
            } else {
                const float2* a = reinterpret_cast<const float2*>(src + row + x0);
                v = CG ? __ldcg(a) : ld_row_f2(a);
            }
        }
        if (cx == 0) {
            f[k] = v;
        } else if (cx > 0) {
            float prev = __shfl_up_sync(kFull, v.y, 1);
            if (edge_lo) prev = (active && xm >= 0) ? ld_pop<ST, CG>(src, row + xm) : 0.0f;
            f[k] = make_float2(prev, v.x);
        } else {
            float next = __shfl_down_sync(kFull, v.x, 1);
            if (edge_hi) next = (active && xp2 >= 0) ? ld_pop<ST, CG>(src, row + xp2) : 0.0f;
            f[k] = make_float2(v.y, next);
        }
    }
    if (skip) return;
    if (MASK && (L0 | L1)) {
#pragma unroll
        for (int k = 1; k < Q; ++k) {
            const long long slot = (long long)rev_of(k) * g.ks + node0;
            if ((L0 >> rev_of(k)) & 1u) f[k].x = ld_pop<ST, CG>(src, slot);
            if ((L1 >> rev_of(k)) & 1u) f[k].y = ld_pop<ST, CG>(src, slot + 1);
        }
    }
    float2 rho;
    update_pair<Q, ST, ARITH, FORM>(f, rho, cp);
    if (MASK && MOVING && (L0 | L1)) {
        const Nbr n0(g, x0, y, z), n1(g, x0 + 1, y, z);
#pragma unroll
        for (int k = 1; k < Q; ++k) {
            if ((L0 >> k) & 1u)
                f[k].x = wall_corrected<Q, ST>(k, f[k].x, rho.x, np.vel[__ldg(types + n0.at<Q>(k, +1)) & kVelMask],
                                               np.cs2inv);
            if ((L1 >> k) & 1u)
                f[k].y = wall_corrected<Q, ST>(k, f[k].y, rho.y, np.vel[__ldg(types + n1.at<Q>(k, +1)) & kVelMask],
                                               np.cs2inv);
        }
    }
#pragma unroll
    for (int k = 0; k < Q; ++k) {
        if constexpr (ST == 1) {
            const __half2 v = __float22half2_rn(f[k]);
            __stcs(reinterpret_cast<unsigned int*>(dst + (long long)k * g.ks + node0),
                   *reinterpret_cast<const unsigned int*>(&v));
        } else {
            __stcs(reinterpret_cast<float2*>(dst + (long long)k * g.ks + node0), f[k]);
        }
    }
}

// Pair-kernel variants: the same arithmetic and the same bits, compiled
// differently.  Which is fastest depends on the lattice, the mask, the block
// width and the domain (the compiler's register allocation and schedule
// shift with each), so the autotuner in capi.cu times them per lattice and
// size class.  form: the update's form (update_pair_dev); regs: a register
// cap per thread, 0 for the compiler's choice.  D2Q9 stays below every cap
// and has the first three.
struct H2Variant {
    int form;
    int regs;
};
constexpr int kH2Variants = kFusedVariants;
constexpr H2Variant kH2Variant[kH2Variants] = {{0, 0}, {1, 0}, {2, 0}, {0, 72}, {1, 72}, {0, 80}, {1, 80}};

template <int Q, bool MASK, bool MOVING, int ARITH, int BX, int FORM, int ST = 1>
__global__ void __launch_bounds__(BX)
nat_fused_h2_k(Geo g, CollideParams cp, NativeParams np, const typename Store<ST>::T* __restrict__ src,
               typename Store<ST>::T* __restrict__ dst, const uint8_t* __restrict__ types) {
    const int lane = threadIdx.x & 31;   // a warp is 32 consecutive pairs of one row
    const int x0 = 2 * (blockIdx.x * BX + threadIdx.x);
    h2_pair<Q, MASK, MOVING, ARITH, FORM, ST>(g, cp, np, src, dst, types, lane, x0, blockIdx.y, blockIdx.z,
                                              x0 < g.nx);
}

// The same kernel with at most NR registers a thread.
template <int Q, bool MASK, bool MOVING, int ARITH, int BX, int FORM, int NR, int ST = 1>
__global__ void __maxnreg__(NR)
nat_fused_h2_kr(Geo g, CollideParams cp, NativeParams np, const typename Store<ST>::T* __restrict__ src,
                typename Store<ST>::T* __restrict__ dst, const uint8_t* __restrict__ types) {
    const int lane = threadIdx.x & 31;
    const int x0 = 2 * (blockIdx.x * BX + threadIdx.x);
    h2_pair<Q, MASK, MOVING, ARITH, FORM, ST>(g, cp, np, src, dst, types, lane, x0, blockIdx.y, blockIdx.z,
                                              x0 < g.nx);
}

// First collision from a RAW state: n at the node itself and the rho/u fields.
template <int Q, int ST, bool MASK, int ARITH>
__global__ void __launch_bounds__(kBlockX)
nat_collide_raw_k(Geo g, CollideParams cp, NativeParams np, const typename Store<ST>::T* __restrict__ src,
                  typename Store<ST>::T* __restrict__ dst, const float* __restrict__ rho_f,
                  const float* __restrict__ u_f, const uint8_t* __restrict__ types) {
    using R = typename Store<ST>::R;
    const int x = blockIdx.x * kBlockX + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= g.nx) return;
    const long long node = g.idx(x, y, z);
    uint32_t L = 0;
    if (MASK) {
        const uint8_t t = __ldg(types + node);
        if (t & kSolid) return;
        L = links_of<MASK>(t, np.links, node);
    }
    const Nbr nb(g, x, y, z);
    R f[Q];
#pragma unroll
    for (int k = 0; k < Q; ++k) f[k] = Store<ST>::ld(src, k * g.ks + node);
    const R rho = (R)rho_f[node];
    const R ux = (R)u_f[node], uy = (R)u_f[g.ks + node], uz = (R)u_f[2 * g.ks + node];
    collide_any<Q, ST, ARITH>(f, rho, ux, uy, uz, raw_drho<ST>((float)rho), cp);
    store_node<Q, ST, MASK>(dst, g, np, types, L, nb, node, rho, f);
}

// ---- AA in-place streaming (one population buffer) ----------------------------
// Even step at node x: reads its own slots A[k][x] = n_k(x), collides, stores
// n*_k in A[rev k][x]; no neighbour is touched.  Odd step: gathers
// n_k(x) = A[rev k][x - c_k] (the even step's n*_k(x - c_k)), or A[k][x] when
// x - c_k is solid (x's own n*_{rev k}, bounced); collides; stores n*_k in
// A[k][x + c_k], or in A[rev k][x] when x + c_k is solid, where x's next even
// step reads it back as n_{rev k}.  Either step reads exactly the slots the
// same thread writes, so the update is in place without races, and after an
// odd step A holds the pre-collision populations in the natural layout.
// Bounce-back values carry the moving-wall term when stored.  Every value is
// the one the two-buffer kernel computes, so the two are bit-identical.
template <int Q, int ST, bool MASK, int ARITH, bool MOVING, bool RAW, int BX>
__global__ void __launch_bounds__(BX)
nat_aa_even_k(Geo g, CollideParams cp, NativeParams np, typename Store<ST>::T* __restrict__ A,
              const float* __restrict__ rho_f, const float* __restrict__ u_f, const uint8_t* __restrict__ types) {
    using R = typename Store<ST>::R;
    const int x = blockIdx.x * BX + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= g.nx) return;
    const long long node = g.idx(x, y, z);
    uint32_t L = 0;
    if (MASK) {
        const uint8_t t = __ldg(types + node);
        if (t & kSolid) return;
        L = links_of<MASK>(t, np.links, node);
    }
    R f[Q];
#pragma unroll
    for (int k = 0; k < Q; ++k) f[k] = Store<ST>::ldp(A, k * g.ks + node);
    R rho;
    if constexpr (RAW) {
        // the first collision of a RAW state uses the rho/u fields
        rho = (R)rho_f[node];
        const R ux = (R)u_f[node], uy = (R)u_f[g.ks + node], uz = (R)u_f[2 * g.ks + node];
        const float drho = raw_drho<ST>((float)rho);
        collide_any<Q, ST, ARITH>(f, rho, ux, uy, uz, drho, cp);
    } else {
        update_node<Q, ST, ARITH>(f, rho, cp);
    }
    const Nbr nb(g, x, y, z);
#pragma unroll
    for (int k = 0; k < Q; ++k) {
        typename Store<ST>::R v = f[k];
        if (MASK && MOVING && k != 0 && np.moving && ((L >> k) & 1u))
            v = wall_corrected<Q, ST>(k, v, rho, np.vel[__ldg(types + nb.at<Q>(k, +1)) & kVelMask], np.cs2inv);
        Store<ST>::st(A, rev_of(k) * g.ks + node, v);
    }
}

template <int Q, int ST, bool MASK, int ARITH, bool MOVING, int BX>
__global__ void __launch_bounds__(BX)
nat_aa_odd_k(Geo g, CollideParams cp, NativeParams np, typename Store<ST>::T* __restrict__ A,
             const uint8_t* __restrict__ types) {
    using R = typename Store<ST>::R;
    const int x = blockIdx.x * BX + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= g.nx) return;
    const long long node = g.idx(x, y, z);
    uint32_t L = 0;
    if (MASK) {
        const uint8_t t = __ldg(types + node);
        if (t & kSolid) return;
        L = links_of<MASK>(t, np.links, node);
    }
    const Nbr nb(g, x, y, z);
    R f[Q];
#pragma unroll
    for (int k = 0; k < Q; ++k) f[k] = Store<ST>::ldp(A, rev_of(k) * g.ks + nb.at<Q>(k, -1));
    if (MASK && L) {
#pragma unroll
        for (int k = 1; k < Q; ++k)
            if ((L >> rev_of(k)) & 1u) f[k] = Store<ST>::ldp(A, k * g.ks + node);
    }
    R rho;
    update_node<Q, ST, ARITH>(f, rho, cp);
#pragma unroll
    for (int k = 0; k < Q; ++k) {
        if (MASK && k != 0 && ((L >> k) & 1u)) {
            typename Store<ST>::R v = f[k];
            if (MOVING && np.moving)
                v = wall_corrected<Q, ST>(k, v, rho, np.vel[__ldg(types + nb.at<Q>(k, +1)) & kVelMask], np.cs2inv);
            Store<ST>::st(A, rev_of(k) * g.ks + node, v);
        } else {
            Store<ST>::st(A, k * g.ks + nb.at<Q>(k, +1), f[k]);
        }
    }
}

// Natural populations (storage format, into n_out, may be null) and moments
// with the solid-node resets (into rho/u, may be null) of an AA buffer in
// either layout: SWAPPED after an even step, natural after an odd one.
template <int Q, int ST, bool MASK, bool SWAPPED>
__global__ void __launch_bounds__(kBlockX)
nat_aa_gather_k(Geo g, NativeParams np, const typename Store<ST>::T* __restrict__ A,
                typename Store<ST>::T* __restrict__ n_out, float* __restrict__ rho_f, float* __restrict__ u_f,
                const uint8_t* __restrict__ types) {
    using R = typename Store<ST>::R;
    const int x = blockIdx.x * kBlockX + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= g.nx) return;
    const long long node = g.idx(x, y, z);
    uint32_t L = 0;
    if (MASK) {
        const uint8_t t = __ldg(types + node);
        if (t & kSolid) {
            if (rho_f) {
                const float* ub = np.vel[t & kVelMask];
                rho_f[node] = np.rho_solid;
                u_f[node] = ub[0]; u_f[g.ks + node] = ub[1]; u_f[2 * g.ks + node] = ub[2];
            }
            if (n_out) {
#pragma unroll
                for (int k = 0; k < Q; ++k)
                    Store<ST>::st(n_out, k * g.ks + node, (ST == 1 || ST == 3) ? -weight<Q>(k) : (R)0);
            }
            return;
        }
        L = links_of<MASK>(t, np.links, node);
    }
    R f[Q];
    if constexpr (SWAPPED) {
        const Nbr nb(g, x, y, z);
#pragma unroll
        for (int k = 0; k < Q; ++k) f[k] = Store<ST>::ld(A, rev_of(k) * g.ks + nb.at<Q>(k, -1));
        if (MASK && L) {
#pragma unroll
            for (int k = 1; k < Q; ++k)
                if ((L >> rev_of(k)) & 1u) f[k] = Store<ST>::ld(A, k * g.ks + node);
        }
    } else {
#pragma unroll
        for (int k = 0; k < Q; ++k) f[k] = Store<ST>::ld(A, k * g.ks + node);
    }
    if (n_out) {
#pragma unroll
        for (int k = 0; k < Q; ++k) Store<ST>::st(n_out, k * g.ks + node, f[k]);
    }
    if (rho_f) {
        R rho, ux, uy, uz;
        moments_any<Q, ST>(f, rho, ux, uy, uz);
        rho_f[node] = (float)rho;
        u_f[node] = (float)ux; u_f[g.ks + node] = (float)uy; u_f[2 * g.ks + node] = (float)uz;
    }
}

// Gather only: n (storage format) and/or moments, solid nodes reset to
// (rho_solid, u_b) as Boundary::reset does for walls.
template <int Q, int ST, bool MASK>
__global__ void __launch_bounds__(kBlockX)
nat_gather_k(Geo g, NativeParams np, const typename Store<ST>::T* __restrict__ src,
             typename Store<ST>::T* __restrict__ n_out, float* __restrict__ rho_f,
             float* __restrict__ u_f, const uint8_t* __restrict__ types) {
    using R = typename Store<ST>::R;
    const int x = blockIdx.x * kBlockX + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= g.nx) return;
    const long long node = g.idx(x, y, z);
    uint32_t L = 0;
    if (MASK) {
        const uint8_t t = __ldg(types + node);
        if (t & kSolid) {
            if (rho_f) {
                const float* ub = np.vel[t & kVelMask];
                rho_f[node] = np.rho_solid;
                u_f[node] = ub[0]; u_f[g.ks + node] = ub[1]; u_f[2 * g.ks + node] = ub[2];
            }
            if (n_out) {
                // a solid node holds no populations: they read back as 0
#pragma unroll
                for (int k = 0; k < Q; ++k)
                    Store<ST>::st(n_out, k * g.ks + node, (ST == 1 || ST == 3) ? -weight<Q>(k) : (R)0);
            }
            return;
        }
        L = links_of<MASK>(t, np.links, node);
    }
    const Nbr nb(g, x, y, z);
    R f[Q];
    gather_node<Q, ST, MASK>(src, g, L, nb, node, f);
    if (n_out) {
#pragma unroll
        for (int k = 0; k < Q; ++k) Store<ST>::st(n_out, k * g.ks + node, f[k]);
    }
    if (rho_f) {
        R rho, ux, uy, uz;
        moments_any<Q, ST>(f, rho, ux, uy, uz);
        rho_f[node] = (float)rho;
        u_f[node] = (float)ux; u_f[g.ks + node] = (float)uy; u_f[2 * g.ks + node] = (float)uz;
    }
}

// ---------------------------------------------------------------------------
// Batches: every domain of the batch advances one step in one launch.  The
// work is a list of warp tasks (domain, z, i0): 32 consecutive nodes i0 ..
// i0 + 31 of the plane z in x-fastest order, so rows shorter than a warp do
// not leave lanes idle and a warp's loads stay within one or two rows.
// Resident blocks take tasks round-robin.  Per node the work is that of
// nat_fused_k: the same gather, arithmetic and bounce-back, so a domain's
// result does not depend on which other domains share its batch.  Descriptor
// fields are read where they are used (every lane reads the same address).
//
// PAIRS: the batch also holds tasks of 64 consecutive nodes (task .w = 1,
// domains with even nx), which run the two-node pair kernel's work: a pair
// never straddles a row (nx is even), and the rows of a warp's pairs differ,
// so each lane forms its own row offsets.  A task's kind is the same for the
// whole warp.  FP16 pairs use the paired update (form 0), FP32 storages the
// scalar update of each node (form 2), which serves every arithmetic.
//
// KIND: the tasks a kernel runs.  A step launches one kernel for the pair
// tasks and one for the 32-node tasks (the host puts the pair tasks first):
// each kernel then holds only its own path's registers (D3Q19 FP32: 126
// registers for both paths in one kernel).  The multi-step kernel runs both
// kinds in one launch (kBatchMixed; .w says which).
enum BatchKind : int { kBatchSingles = 0, kBatchPairs = 1, kBatchMixed = 2 };

// The tasks of one step, walked by every resident warp (CG: L2-coherent
// population loads, for the multi-step kernel).
template <int Q, int ST, int ARITH, bool MOVING, int KIND, bool CG>
__device__ __forceinline__ void batch_tasks(const BatchDomain* __restrict__ doms, const int4* __restrict__ tasks,
                                            int ntasks, int parity) {
    using T = typename Store<ST>::T;
    using R = typename Store<ST>::R;
    const int lane = threadIdx.x & 31;
    const int warps = gridDim.x * (kBatchTile / 32);
    // the next task's descriptor is loaded while this one runs, so a task
    // does not start with a round trip for its own descriptor
    const int t0 = blockIdx.x * (kBatchTile / 32) + (threadIdx.x >> 5);
    int4 next = t0 < ntasks ? __ldg(tasks + t0) : make_int4(0, 0, 0, 0);
    for (int t = t0; t < ntasks; t += warps) {
        const int4 tk = next;
        if (t + warps < ntasks) next = __ldg(tasks + t + warps);
        const BatchDomain& D = doms[tk.x];
        const Geo g = D.g;
        if constexpr (KIND != kBatchSingles) {
            if (KIND == kBatchPairs || tk.w) {
                const int i = tk.z + 2 * lane;
                const bool active = i < g.nx * g.ny;
                const int y = active ? (int)((unsigned)i / (unsigned)g.nx) : 0;
                const int x0 = active ? i - y * g.nx : 0;
                h2_pair<Q, true, MOVING, ARITH, ST == 1 ? 0 : 2, ST, CG, true>(
                    g, D.cp, D.np, static_cast<const T*>(D.f[parity]), static_cast<T*>(D.f[parity ^ 1]), D.types,
                    lane, x0, y, tk.y, active);
                continue;
            }
        }
        if constexpr (KIND == kBatchPairs) continue;
        // 32 consecutive nodes of the plane z (flattened y * nx + x), so short
        // rows do not leave lanes idle
        const int i = tk.z + lane;
        if (i >= g.nx * g.ny) continue;
        const int y = (int)((unsigned)i / (unsigned)g.nx), x = i - y * g.nx, z = tk.y;
        const long long node = g.idx(x, y, z);
        const uint8_t* types = D.types;
        const NativeParams& np = D.np;
        const uint8_t tt = __ldg(types + node);
        const uint32_t lw = __ldg(np.links + node);   // beside the type, as nat_fused_k
        if ((tt & (kSolid | kSectorMate)) == kSolid) continue;
        const uint32_t L = (tt & kNearSolid) ? lw : 0u;
        const T* src = static_cast<const T*>(D.f[parity]);
        T* dst = static_cast<T*>(D.f[parity ^ 1]);
        const Nbr nb(g, x, y, z);
        R f[Q];
        R rho;
        if (tt & kSolid) {
            rest_state<Q, ST>(f, rho);   // completes its store sector, as nat_fused_k
        } else {
            gather_node<Q, ST, true, CG>(src, g, L, nb, node, f);
            update_node<Q, ST, ARITH>(f, rho, D.cp);
        }
        store_node<Q, ST, true, MOVING>(dst, g, np, types, L, nb, node, rho, f);
    }
}

// FP16 batches of D2Q9/D3Q19 at six blocks an SM (at most 80 registers):
// config 4's FP16 batch 33.6k -> 36.0k MLUPS.  FP32 storages, the most
// blocks an SM without spills: pair tasks five (D2Q9/D3Q19, 96 registers)
// and four (D3Q27, 128), one-node tasks six (D2Q9/D3Q19, 80); the
// compiler's choices were 122, 156 and 96.  These kernels are latency-bound
// (long-scoreboard stalls, ~31 % warps active at 96 registers).
template <int Q, int ST, int ARITH, bool MOVING, int KIND>
__global__ void __launch_bounds__(kBatchTile, (ST == 1 && Q <= 19) ? 6 : (KIND == kBatchPairs ? (Q <= 19 ? 5 : 4) : (Q <= 19 ? 6 : 1)))
nat_batch_k(const BatchDomain* __restrict__ doms, const int4* __restrict__ tasks, int ntasks, int parity) {
    batch_tasks<Q, ST, ARITH, MOVING, KIND, false>(doms, tasks, ntasks, parity);
}

// ---------------------------------------------------------------------------
// Multi-step batches: one launch runs n steps of the task list, the steps
// separated by a grid-wide barrier.  The grid is what can be resident at once
// (a cooperative launch), so every block reaches every barrier.  The wait at
// a barrier is bounded: a block that polls more than kBatchBarrierPolls times
// sets the error word and leaves, the others see the word and leave too, and
// the host reports PLB_ETIMEOUT; a step's own work never takes that long.
// Population loads bypass L1 (CG): a step reads what other SMs wrote in the
// previous one.
constexpr unsigned long long kBatchBarrierPolls = 1ull << 22;   // about 1-2 s with the back-off

__device__ __forceinline__ bool batch_grid_sync(BatchSync* bs, unsigned nblocks) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        volatile unsigned int* vgen = &bs->gen;
        volatile int* verr = &bs->error;
        const unsigned int g0 = *vgen;   // read before arriving: it cannot change until this block arrives
        __threadfence();                 // this block's stores before its arrival
        if (atomicAdd(&bs->count, 1u) == nblocks - 1) {
            atomicExch(&bs->count, 0u);
            __threadfence();
            atomicAdd(&bs->gen, 1u);
        } else {
            unsigned long long polls = 0;
            while (*vgen == g0) {
                if (*verr || ++polls > kBatchBarrierPolls) {
                    atomicExch(&bs->error, 1);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();                 // the other blocks' stores before this block's next loads
    }
    __syncthreads();
    return ok != 0;
}

template <int Q, int ST, int ARITH, bool MOVING, bool PAIRS = false>
__global__ void __launch_bounds__(kBatchTile)
nat_batch_multi_k(const BatchDomain* __restrict__ doms, const int4* __restrict__ tasks, int ntasks, int parity,
                  int nsteps, BatchSync* bs) {
    for (int s = 0; s < nsteps; ++s) {
        batch_tasks<Q, ST, ARITH, MOVING, PAIRS ? kBatchMixed : kBatchSingles, true>(doms, tasks, ntasks,
                                                                                   parity ^ (s & 1));
        if (s + 1 < nsteps && !batch_grid_sync(bs, gridDim.x)) return;
    }
}

dim3 cell_grid(const Geo& g) { return dim3((g.nx + kBlockX - 1) / kBlockX, g.ny, g.nz); }

template <int Q, int ST, bool MASK, int ARITH>
int launch_fused(const Geo& g, const CollideParams& cp, const NativeParams& np, const void* src, void* dst,
                 const uint8_t* types, cudaStream_t st) {
    using T = typename Store<ST>::T;
    if (block_x(g, 1) == kBlockX)
        nat_fused_k<Q, ST, MASK, ARITH, kBlockX><<<seg_grid(g, kBlockX, 1), kBlockX, 0, st>>>(
            g, cp, np, (const T*)src, (T*)dst, types);
    else
        nat_fused_k<Q, ST, MASK, ARITH, 32><<<seg_grid(g, 32, 1), 32, 0, st>>>(g, cp, np, (const T*)src, (T*)dst,
                                                                             types);
    return (int)cudaGetLastError();
}

template <int Q, int ST, bool MASK, int ARITH>
int launch_raw(const Geo& g, const CollideParams& cp, const NativeParams& np, const void* src, void* dst,
               const float* rho, const float* u, const uint8_t* types, cudaStream_t st) {
    using T = typename Store<ST>::T;
    nat_collide_raw_k<Q, ST, MASK, ARITH><<<cell_grid(g), kBlockX, 0, st>>>(
        g, cp, np, (const T*)src, (T*)dst, rho, u, types);
    return (int)cudaGetLastError();
}

template <int Q, int ST, bool MASK>
int launch_gather(const Geo& g, const NativeParams& np, const void* src, void* n_out, float* rho, float* u,
                  const uint8_t* types, cudaStream_t st) {
    using T = typename Store<ST>::T;
    nat_gather_k<Q, ST, MASK><<<cell_grid(g), kBlockX, 0, st>>>(g, np, (const T*)src, (T*)n_out, rho, u, types);
    return (int)cudaGetLastError();
}

// ---- host-side dispatch --------------------------------------------------------
// Calls f(ST, ARITH) (integral constants) with the kernel arithmetic of a
// storage: FP16 and FP64 storage have one BGK arithmetic each, FP32 storage
// plbpd's or the FP32-only one; under TRT every storage has the TRT one.
template <int V> using IC = std::integral_constant<int, V>;

template <bool TRT, class F>
auto with_storage_arith(int storage, int arith, F&& f) {
    if constexpr (TRT) {
        if (storage == 1) return f(IC<1>{}, IC<kArithTRT>{});
        if (storage == 2) return f(IC<2>{}, IC<kArithTRT>{});
        if (storage == 3) return f(IC<3>{}, IC<kArithTRT>{});
        return f(IC<0>{}, IC<kArithTRT>{});
    } else {
        if (storage == 1) return f(IC<1>{}, IC<kArithFP32>{});
        if (storage == 2) return f(IC<2>{}, IC<kArithFP32>{});
        if (storage == 3) return f(IC<3>{}, IC<kArithFP32>{});
        if (arith == kArithReference) return f(IC<0>{}, IC<kArithReference>{});
        return f(IC<0>{}, IC<kArithFP32>{});
    }
}

// Variants that exist for a kernel: BGK without moving walls has all of
// kH2Variant (D2Q9 the three without a cap); TRT and moving walls have
// variant 0.
template <int Q, int ARITH, bool MOVING>
constexpr int h2_variants() {
    return (ARITH == kArithTRT || MOVING) ? 1 : (Q == 9 ? 3 : kH2Variants);
}

inline int nat_h2_variant_count(int q, int arith, bool moving) {
    if (arith == kArithTRT || moving) return 1;
    return q == 9 ? 3 : kH2Variants;
}

template <int Q, int ARITH, bool MASK>
int launch_fused_h2(const Geo& g, const CollideParams& cp, const NativeParams& np, const void* src, void* dst,
                    const uint8_t* types, int variant, cudaStream_t st) {
    auto s2 = (const __half*)src;
    auto d2 = (__half*)dst;
    auto go = [&](auto bxc) {
        constexpr int BX = decltype(bxc)::value;
        const dim3 grid = seg_grid(g, BX, 2);
        if (MASK && np.moving) {
            nat_fused_h2_k<Q, true, true, ARITH, BX, 0><<<grid, BX, 0, st>>>(g, cp, np, s2, d2, types);
            return;
        }
        static_assert(kH2Variant[1].form == 1 && kH2Variant[2].form == 2 && kH2Variant[3].regs == 72 &&
                          kH2Variant[4].form == 1 && kH2Variant[5].regs == 80 && kH2Variant[6].form == 1,
                      "the launches below follow kH2Variant");
        constexpr int NV = h2_variants<Q, ARITH, false>();
        const int v = variant < NV ? variant : 0;
        if constexpr (NV >= 3) {
            if (v == 1) { nat_fused_h2_k<Q, MASK, false, ARITH, BX, 1><<<grid, BX, 0, st>>>(g, cp, np, s2, d2, types); return; }
            if (v == 2) { nat_fused_h2_k<Q, MASK, false, ARITH, BX, 2><<<grid, BX, 0, st>>>(g, cp, np, s2, d2, types); return; }
        }
        if constexpr (NV == kH2Variants) {
            switch (v) {
                case 3: nat_fused_h2_kr<Q, MASK, false, ARITH, BX, 0, 72><<<grid, BX, 0, st>>>(g, cp, np, s2, d2, types); return;
                case 4: nat_fused_h2_kr<Q, MASK, false, ARITH, BX, 1, 72><<<grid, BX, 0, st>>>(g, cp, np, s2, d2, types); return;
                case 5: nat_fused_h2_kr<Q, MASK, false, ARITH, BX, 0, 80><<<grid, BX, 0, st>>>(g, cp, np, s2, d2, types); return;
                case 6: nat_fused_h2_kr<Q, MASK, false, ARITH, BX, 1, 80><<<grid, BX, 0, st>>>(g, cp, np, s2, d2, types); return;
                default: break;
            }
        }
        nat_fused_h2_k<Q, MASK, false, ARITH, BX, 0><<<grid, BX, 0, st>>>(g, cp, np, s2, d2, types);
    };
    if (block_x(g, 2) == kBlockX) go(std::integral_constant<int, kBlockX>{});
    else go(std::integral_constant<int, 32>{});
    return (int)cudaGetLastError();
}

// FP32 and FP32-deviation storage (BGK, FP32 arithmetic) with even nx: the
// single-node kernel is variant 0, the pair kernel in forms 0, 1 and 2 are
// variants 1-3.  FP32 storage with plbpd's arithmetic has the single-node
// kernel and the pair kernel in form 2 (each node's own update, so the
// exact-tail emulation and its FP64 fallback run per node as in the
// single-node kernel): variants 0 and 1.  Moving walls, FP64 storage and TRT
// have the single-node kernel only.
constexpr int kPair32Variants = 4;
constexpr int kPairRefVariants = 2;

template <int Q, int ST, bool MASK, int ARITH = kArithFP32>
int launch_fused_pair32(const Geo& g, const CollideParams& cp, const NativeParams& np, const void* src, void* dst,
                        const uint8_t* types, int variant, cudaStream_t st) {
    static_assert(ST == 0 || ST == 3, "FP32 storages only");
    static_assert(ARITH == kArithFP32 || (ARITH == kArithReference && ST == 0), "BGK arithmetics of FP32 storage");
    using T = typename Store<ST>::T;
    auto s2 = (const T*)src;
    auto d2 = (T*)dst;
    auto go = [&](auto bxc) {
        constexpr int BX = decltype(bxc)::value;
        const dim3 grid = seg_grid(g, BX, 2);
        if constexpr (ARITH == kArithReference) {
            nat_fused_h2_k<Q, MASK, false, ARITH, BX, 2, ST><<<grid, BX, 0, st>>>(g, cp, np, s2, d2, types);
        } else {
            if (variant == 2) nat_fused_h2_k<Q, MASK, false, ARITH, BX, 1, ST><<<grid, BX, 0, st>>>(g, cp, np, s2, d2, types);
            else if (variant == 3) nat_fused_h2_k<Q, MASK, false, ARITH, BX, 2, ST><<<grid, BX, 0, st>>>(g, cp, np, s2, d2, types);
            else nat_fused_h2_k<Q, MASK, false, ARITH, BX, 0, ST><<<grid, BX, 0, st>>>(g, cp, np, s2, d2, types);
        }
    };
    if (block_x(g, 2) == kBlockX) go(std::integral_constant<int, kBlockX>{});
    else go(std::integral_constant<int, 32>{});
    return (int)cudaGetLastError();
}

// One fused step (FP16 storage with even nx: the pair kernel).
template <bool TRT, int Q>
int fused_q(int storage, int arith, bool m, const Geo& g, const CollideParams& cp, const NativeParams& np,
            const void* src, void* dst, const uint8_t* types, int variant, cudaStream_t st) {
    return with_storage_arith<TRT>(storage, arith, [&](auto stc, auto arc) {
        constexpr int ST = decltype(stc)::value, AR = decltype(arc)::value;
        if constexpr (ST == 1) {
            if (g.nx % 2 == 0) {
                if constexpr (TRT) {
                    return m ? launch_fused_h2<Q, AR, true>(g, cp, np, src, dst, types, 0, st)
                             : launch_fused_h2<Q, AR, false>(g, cp, np, src, dst, types, 0, st);
                } else {
                    if constexpr (Q == 9) return nat_fused_h2_bgk9(m, g, cp, np, src, dst, types, variant, st);
                    if constexpr (Q == 19) return nat_fused_h2_bgk19(m, g, cp, np, src, dst, types, variant, st);
                    if constexpr (Q == 27) return nat_fused_h2_bgk27(m, g, cp, np, src, dst, types, variant, st);
                }
            }
        }
        if constexpr (!TRT && (ST == 3 || ST == 0)) {
            if (variant > 0 && g.nx % 2 == 0 && !(m && np.moving)) {
                if constexpr (Q == 9) return nat_fused_pair32_q9(ST, AR, m, g, cp, np, src, dst, types, variant, st);
                if constexpr (Q == 19) return nat_fused_pair32_q19(ST, AR, m, g, cp, np, src, dst, types, variant, st);
                if constexpr (Q == 27) return nat_fused_pair32_q27(ST, AR, m, g, cp, np, src, dst, types, variant, st);
            }
        }
        return m ? launch_fused<Q, ST, true, AR>(g, cp, np, src, dst, types, st)
                 : launch_fused<Q, ST, false, AR>(g, cp, np, src, dst, types, st);
    });
}

template <bool TRT, int Q>
int raw_q(int storage, int arith, bool m, const Geo& g, const CollideParams& cp, const NativeParams& np,
          const void* src, void* dst, const float* rho, const float* u, const uint8_t* types, cudaStream_t st) {
    return with_storage_arith<TRT>(storage, arith, [&](auto stc, auto arc) {
        constexpr int ST = decltype(stc)::value, AR = decltype(arc)::value;
        return m ? launch_raw<Q, ST, true, AR>(g, cp, np, src, dst, rho, u, types, st)
                 : launch_raw<Q, ST, false, AR>(g, cp, np, src, dst, rho, u, types, st);
    });
}

// AA steps: kind 0 = even from a RAW state (fields), 1 = even, 2 = odd.
template <int Q, int ST, bool MASK, int AR>
int launch_aa(int kind, const Geo& g, const CollideParams& cp, const NativeParams& np, void* A, const float* rho,
              const float* u, const uint8_t* types, cudaStream_t st) {
    using T = typename Store<ST>::T;
    const bool mv = MASK && np.moving;
    auto go = [&](auto mvc, auto bxc) {
        constexpr bool MV = decltype(mvc)::value;
        constexpr int BX = decltype(bxc)::value;
        const dim3 grid = seg_grid(g, BX, 1);
        if (kind == 0)
            nat_aa_even_k<Q, ST, MASK, AR, MV, true, BX><<<grid, BX, 0, st>>>(g, cp, np, (T*)A, rho, u, types);
        else if (kind == 1)
            nat_aa_even_k<Q, ST, MASK, AR, MV, false, BX><<<grid, BX, 0, st>>>(g, cp, np, (T*)A, rho, u, types);
        else
            nat_aa_odd_k<Q, ST, MASK, AR, MV, BX><<<grid, BX, 0, st>>>(g, cp, np, (T*)A, types);
        return (int)cudaGetLastError();
    };
    using W = std::integral_constant<int, kBlockX>;
    using N = std::integral_constant<int, 32>;
    if (block_x(g, 1) == kBlockX) return mv ? go(std::true_type{}, W{}) : go(std::false_type{}, W{});
    return mv ? go(std::true_type{}, N{}) : go(std::false_type{}, N{});
}

template <bool TRT, int Q>
int aa_q(int kind, int storage, int arith, bool m, const Geo& g, const CollideParams& cp, const NativeParams& np,
         void* A, const float* rho, const float* u, const uint8_t* types, cudaStream_t st) {
    return with_storage_arith<TRT>(storage, arith, [&](auto stc, auto arc) {
        constexpr int ST = decltype(stc)::value, AR = decltype(arc)::value;
        return m ? launch_aa<Q, ST, true, AR>(kind, g, cp, np, A, rho, u, types, st)
                 : launch_aa<Q, ST, false, AR>(kind, g, cp, np, A, rho, u, types, st);
    });
}

// Batches hold FP32, FP32-deviation or FP16 storage; kind: the BatchKind of
// the one-step kernel.
template <bool TRT, bool MV>
const void* batch_kernel_for(int q, int storage, int arith, int kind) {
    if (storage == 2) return nullptr;
    const void* k = nullptr;
    with_storage_arith<TRT>(storage, arith, [&](auto stc, auto arc) {
        constexpr int ST = decltype(stc)::value == 2 ? 0 : decltype(stc)::value, AR = decltype(arc)::value;
        auto pick = [&](auto kc) {
            constexpr int K = decltype(kc)::value;
            k = q == 9 ? (const void*)nat_batch_k<9, ST, AR, MV, K>
              : q == 19 ? (const void*)nat_batch_k<19, ST, AR, MV, K>
              : q == 27 ? (const void*)nat_batch_k<27, ST, AR, MV, K> : nullptr;
        };
        if (kind == kBatchPairs) pick(IC<kBatchPairs>{});
        else if (kind == kBatchMixed) pick(IC<kBatchMixed>{});
        else pick(IC<kBatchSingles>{});
        return 0;
    });
    return k;
}

template <bool TRT>
int batch_blocks_per_sm(int q, int storage, int arith, bool moving, int kind) {
    const void* k = moving ? batch_kernel_for<TRT, true>(q, storage, arith, kind)
                           : batch_kernel_for<TRT, false>(q, storage, arith, kind);
    if (!k) return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, kBatchTile, 0) != cudaSuccess) return 0;
    return n;
}

// One step: the pair tasks tiles[0, npair) and the 32-node tasks
// tiles[npair, ntiles), each kind in its own kernel on `st` (at most
// blocks_pair / blocks_single resident blocks, one task per warp).
template <bool TRT>
int batch_step(int q, int storage, int arith, bool moving, const BatchDomain* doms, const int4* tiles, int ntiles,
               int npair, int parity, int blocks_pair, int blocks_single, cudaStream_t st) {
    if (ntiles <= 0) return 0;
    if (storage == 2) return (int)cudaErrorInvalidValue;
    auto grid = [](int tasks, int blocks) {
        const int need = (tasks + kBatchTile / 32 - 1) / (kBatchTile / 32);
        return blocks < need ? (blocks > 0 ? blocks : 1) : need;
    };
    return with_storage_arith<TRT>(storage, arith, [&](auto stc, auto arc) {
        constexpr int ST = decltype(stc)::value == 2 ? 0 : decltype(stc)::value, AR = decltype(arc)::value;
        auto go = [&](auto qc) {
            constexpr int Q = decltype(qc)::value;
            if (npair > 0) {
                const int gb = grid(npair, blocks_pair);
                if (moving) nat_batch_k<Q, ST, AR, true, kBatchPairs><<<gb, kBatchTile, 0, st>>>(doms, tiles, npair, parity);
                else nat_batch_k<Q, ST, AR, false, kBatchPairs><<<gb, kBatchTile, 0, st>>>(doms, tiles, npair, parity);
                const cudaError_t e = cudaGetLastError();
                if (e != cudaSuccess) return (int)e;
            }
            const int ns = ntiles - npair;
            if (ns > 0) {
                const int gb = grid(ns, blocks_single);
                const int4* t1 = tiles + npair;
                if (moving) nat_batch_k<Q, ST, AR, true, kBatchSingles><<<gb, kBatchTile, 0, st>>>(doms, t1, ns, parity);
                else nat_batch_k<Q, ST, AR, false, kBatchSingles><<<gb, kBatchTile, 0, st>>>(doms, t1, ns, parity);
            }
            return (int)cudaGetLastError();
        };
        return q == 9 ? go(IC<9>{}) : q == 19 ? go(IC<19>{}) : q == 27 ? go(IC<27>{}) : (int)cudaErrorInvalidValue;
    });
}

// The multi-step kernel for a configuration (nullptr if none).
template <bool TRT, bool MV>
const void* batch_multi_kernel_for(int q, int storage, int arith, bool pairs) {
    const void* k = nullptr;
    with_storage_arith<TRT>(storage == 2 ? 0 : storage, arith, [&](auto stc, auto arc) {
        constexpr int ST = decltype(stc)::value == 2 ? 0 : decltype(stc)::value, AR = decltype(arc)::value;
        if (pairs)
            k = q == 9 ? (const void*)nat_batch_multi_k<9, ST, AR, MV, true>
              : q == 19 ? (const void*)nat_batch_multi_k<19, ST, AR, MV, true>
              : q == 27 ? (const void*)nat_batch_multi_k<27, ST, AR, MV, true> : nullptr;
        else
            k = q == 9 ? (const void*)nat_batch_multi_k<9, ST, AR, MV>
              : q == 19 ? (const void*)nat_batch_multi_k<19, ST, AR, MV>
              : q == 27 ? (const void*)nat_batch_multi_k<27, ST, AR, MV> : nullptr;
        return 0;
    });
    return k;
}

// nsteps steps in one cooperative launch of at most `blocks` blocks (no more
// than are resident at once on the device); bs must hold count = 0 and
// error = 0.
template <bool TRT>
int batch_step_multi(int q, int storage, int arith, bool moving, bool pairs, const BatchDomain* doms,
                     const int4* tiles, int ntiles, int parity, int nsteps, int blocks, BatchSync* bs,
                     cudaStream_t st) {
    if (ntiles <= 0 || nsteps <= 0) return 0;
    if (storage == 2) return (int)cudaErrorInvalidValue;
    const void* k = moving ? batch_multi_kernel_for<TRT, true>(q, storage, arith, pairs)
                           : batch_multi_kernel_for<TRT, false>(q, storage, arith, pairs);
    if (!k) return (int)cudaErrorInvalidValue;
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kBatchTile, 0);
    if (e != cudaSuccess) return (int)e;
    const int resident = sms * per_sm;
    const int need = (ntiles + kBatchTile / 32 - 1) / (kBatchTile / 32);
    if (blocks > resident) blocks = resident;
    if (blocks > need) blocks = need;
    if (blocks < 1) return (int)cudaErrorInvalidConfiguration;
    void* args[] = {(void*)&doms, (void*)&tiles, (void*)&ntiles, (void*)&parity, (void*)&nsteps, (void*)&bs};
    return (int)cudaLaunchCooperativeKernel(k, dim3((unsigned)blocks), dim3(kBatchTile), args, 0, st);
}

#define PLB_Q_DISPATCH(q, CALL) \
    ((q) == 9 ? CALL(9) : (q) == 19 ? CALL(19) : (q) == 27 ? CALL(27) : (int)cudaErrorInvalidValue)

}  // namespace
}  // namespace plb
