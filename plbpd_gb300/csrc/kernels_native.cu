// Kernels for NATIVE semantics: one fused pull kernel per time step.
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
#include "engine.h"

namespace plb {
namespace {

constexpr int kBlockX = 128;

template <int ST> struct Store;
template <> struct Store<0> {
    using T = float;
    using R = float;
    __device__ static __forceinline__ float ld(const float* p, long long i) { return __ldg(p + i); }
    __device__ static __forceinline__ void st(float* p, long long i, float v) { __stcs(p + i, v); }
};
template <> struct Store<1> {
    using T = __half;
    using R = float;
    __device__ static __forceinline__ float ld(const __half* p, long long i) { return __half2float(__ldg(p + i)); }
    __device__ static __forceinline__ void st(__half* p, long long i, float v) {
        __stcs(reinterpret_cast<unsigned short*>(p) + i, __half_as_ushort(__float2half_rn(v)));
    }
};
template <> struct Store<2> {
    using T = double;
    using R = double;
    __device__ static __forceinline__ double ld(const double* p, long long i) { return __ldg(p + i); }
    __device__ static __forceinline__ void st(double* p, long long i, double v) { __stcs(p + i, v); }
};

// Neighbour index helper: element offsets of x-1, x, x+1 (and y, z) with the
// periodic axes wrapped.  A fluid node never has a neighbour outside the box
// along a walled axis, because the wall layer in between is solid.
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
template <int Q>
__device__ __forceinline__ void collide_node_dev(float (&d)[Q], float drho, float rho, float ux, float uy,
                                                 float uz, const CollideParams& P) {
    const float tr = __fdiv_rn(P.tau, rho);
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
        const float A = __fmul_rn(weight<Q>(k), orho);     // shared by a weight class after CSE
        const float B = __fmul_rn(weight<Q>(k), odrho);
        const float X = __fmaf_rn(cu, __fmaf_rn(4.5f, cu, 3.0f), kusq);
        d[k] = __fmaf_rn(P.omc, d[k], __fmaf_rn(A, X, B));
    }
}

template <int Q>
__device__ __forceinline__ void node_moments_dev(const float (&d)[Q], float& drho, float& rho, float& ux,
                                                 float& uy, float& uz) {
    float jx, jy, jz;
    node_sums<Q>(d, drho, jx, jy, jz);
    rho = __fadd_rn(1.0f, drho);
    const float rinv = __fdiv_rn(1.0f, rho);
    ux = __fmul_rn(jx, rinv);
    uy = __fmul_rn(jy, rinv);
    uz = __fmul_rn(jz, rinv);
}

// ---- FP64 storage: the same method in double ---------------------------------
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
        const double neq = __dmul_rn(__dmul_rn((double)weight<Q>(k), rho), br);
        f[k] = __dadd_rn(__dmul_rn(omc, f[k]), __dmul_rn(omega, neq));
    }
}

// ---- per storage: moments + collision, and the moving-wall correction ---------
template <int Q, int ST, int ARITH>
__device__ __forceinline__ void update_node(typename Store<ST>::R (&f)[Q], typename Store<ST>::R& rho,
                                            const CollideParams& cp) {
    if constexpr (ST == 0) {
        float ux, uy, uz;
        node_moments<Q>(f, rho, ux, uy, uz);
        collide_node<Q, ARITH>(f, rho, ux, uy, uz, cp);
    } else if constexpr (ST == 1) {
        float drho, ux, uy, uz;
        node_moments_dev<Q>(f, drho, rho, ux, uy, uz);
        collide_node_dev<Q>(f, drho, rho, ux, uy, uz, cp);
    } else {
        double ux, uy, uz;
        node_moments_d<Q>(f, rho, ux, uy, uz);
        collide_node_d<Q>(f, rho, ux, uy, uz, cp);
    }
}

template <int Q, int ST>
__device__ __forceinline__ void moments_any(const typename Store<ST>::R (&f)[Q], typename Store<ST>::R& rho,
                                            typename Store<ST>::R& ux, typename Store<ST>::R& uy,
                                            typename Store<ST>::R& uz) {
    if constexpr (ST == 0) node_moments<Q>(f, rho, ux, uy, uz);
    else if constexpr (ST == 1) { float drho; node_moments_dev<Q>(f, drho, rho, ux, uy, uz); }
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
        const double t = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(2.0, (double)weight<Q>(k)), rho), cu), (double)cs2inv);
        return __dsub_rn(v, t);
    } else {
        return __fsub_rn(v, wall_term<Q>(k, rho, dot_c_full<Q>(k, ub), cs2inv));
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

// The solid-link mask of a node (0 for nodes away from solids).
template <bool MASK>
__device__ __forceinline__ uint32_t links_of(const uint8_t t, const uint32_t* __restrict__ links, long long node) {
    return (MASK && (t & kNearSolid)) ? __ldg(links + node) : 0u;
}

// Gathers n[x][*] from P (streaming plus bounce-back).  `links` bit k is set
// when x + c_k is solid, so the source x - c_k is solid when bit rev(k) is.
template <int Q, int ST, bool MASK>
__device__ __forceinline__ void gather_node(const typename Store<ST>::T* __restrict__ src, const Geo& g,
                                            uint32_t links, const Nbr& nb, long long node,
                                            typename Store<ST>::R (&f)[Q]) {
    // every source is inside the box (a solid source is a node too), so the
    // streaming loads are unconditional; bounce-back directions are then
    // replaced by the node's own reversed slot
#pragma unroll
    for (int k = 0; k < Q; ++k) f[k] = Store<ST>::ld(src, k * g.ks + nb.at<Q>(k, -1));
    if (MASK && links) {
#pragma unroll
        for (int k = 1; k < Q; ++k)
            if ((links >> rev_of(k)) & 1u) f[k] = Store<ST>::ld(src, rev_of(k) * g.ks + node);
    }
}

// ---------------------------------------------------------------------------
template <int Q, int ST, bool MASK, int ARITH>
__global__ void __launch_bounds__(kBlockX)
nat_fused_k(Geo g, CollideParams cp, NativeParams np, const typename Store<ST>::T* __restrict__ src,
            typename Store<ST>::T* __restrict__ dst, const uint8_t* __restrict__ types) {
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
    gather_node<Q, ST, MASK>(src, g, L, nb, node, f);
    R rho;
    update_node<Q, ST, ARITH>(f, rho, cp);
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
template <int Q, bool MASK, bool MOVING>
__global__ void __launch_bounds__(kBlockX, (Q == 27 || MOVING) ? 4 : 6)
nat_fused_h2_k(Geo g, CollideParams cp, NativeParams np, const __half* __restrict__ src, __half* __restrict__ dst,
               const uint8_t* __restrict__ types) {
    const unsigned kFull = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int x0 = 2 * (blockIdx.x * kBlockX + threadIdx.x);
    const int y = blockIdx.y, z = blockIdx.z;
    const bool active = x0 < g.nx;
    const int ym = (y == 0 && g.wrap_y) ? g.ny - 1 : y - 1;
    const int yp = (y == g.ny - 1 && g.wrap_y) ? 0 : y + 1;
    const int zm = (z == 0 && g.wrap_z) ? g.nz - 1 : z - 1;
    const int zp = (z == g.nz - 1 && g.wrap_z) ? 0 : z + 1;
    // 32-bit element offsets (the host checks q * ks < 2^32)
    const unsigned ys = (unsigned)g.ys, zs = (unsigned)g.zs, ks = (unsigned)g.ks;
    const unsigned yo[3] = {(unsigned)ym * ys, (unsigned)y * ys, (unsigned)yp * ys};
    const unsigned zo[3] = {(unsigned)zm * zs, (unsigned)z * zs, (unsigned)zp * zs};
    // the values the neighbouring lanes cannot provide
    const int xm = x0 == 0 ? (g.wrap_x ? g.nx - 1 : -1) : x0 - 1;
    const int xp2 = x0 + 2 >= g.nx ? (g.wrap_x ? x0 + 2 - g.nx : -1) : x0 + 2;
    const bool edge_lo = lane == 0 || x0 == 0;
    const bool edge_hi = lane == 31 || x0 + 2 >= g.nx;
    const unsigned node0 = zo[1] + yo[1] + (unsigned)x0;

    bool skip = !active;
    uint8_t t0 = 0, t1 = 0;
    uint32_t L0 = 0, L1 = 0;
    if (MASK && active) {
        const unsigned short tt = __ldg(reinterpret_cast<const unsigned short*>(types + node0));
        t0 = (uint8_t)(tt & 0xff);
        t1 = (uint8_t)(tt >> 8);
        skip = (t0 & kSolid) && (t1 & kSolid);
        L0 = links_of<MASK>(t0, np.links, node0);
        L1 = links_of<MASK>(t1, np.links, node0 + 1);
    }
    // A lane loads every source row that exists even when its own pair is
    // solid: its neighbours take values from it through the shuffles, and for
    // a diagonal direction those come from another row, where the node may be
    // fluid.  Rows outside a walled axis only occur for pairs in a wall row,
    // whose neighbours in that row are walls too.
    const bool ym_ok = g.wrap_y || y > 0, yp_ok = g.wrap_y || y < g.ny - 1;
    const bool zm_ok = g.wrap_z || z > 0, zp_ok = g.wrap_z || z < g.nz - 1;
    float f0[Q], f1[Q];
#pragma unroll
    for (int k = 0; k < Q; ++k) {
        const int cx = Lattice<Q>::cx(k), cy = Lattice<Q>::cy(k), cz = Lattice<Q>::cz(k);
        const unsigned row = (unsigned)k * ks + zo[1 - cz] + yo[1 - cy];
        const bool row_ok = active && (cy > 0 ? ym_ok : cy < 0 ? yp_ok : true) &&
                            (cz > 0 ? zm_ok : cz < 0 ? zp_ok : true);
        float lo = 0.0f, hi = 0.0f;
        if (row_ok) {
            const __half2 v = __ldg(reinterpret_cast<const __half2*>(src + row + x0));
            lo = __low2float(v);
            hi = __high2float(v);
        }
        if (cx == 0) {
            f0[k] = lo;
            f1[k] = hi;
        } else if (cx > 0) {
            float prev = __shfl_up_sync(kFull, hi, 1);
            if (edge_lo) prev = (row_ok && xm >= 0) ? __half2float(__ldg(src + row + xm)) : 0.0f;
            f0[k] = prev;
            f1[k] = lo;
        } else {
            float next = __shfl_down_sync(kFull, lo, 1);
            if (edge_hi) next = (row_ok && xp2 >= 0) ? __half2float(__ldg(src + row + xp2)) : 0.0f;
            f0[k] = hi;
            f1[k] = next;
        }
    }
    if (skip) return;
    if (MASK && (L0 | L1)) {
#pragma unroll
        for (int k = 1; k < Q; ++k) {
            const unsigned slot = (unsigned)rev_of(k) * ks + node0;
            if ((L0 >> rev_of(k)) & 1u) f0[k] = __half2float(__ldg(src + slot));
            if ((L1 >> rev_of(k)) & 1u) f1[k] = __half2float(__ldg(src + slot + 1));
        }
    }
    float rho0, rho1;
    update_node<Q, 1, kArithFP32>(f0, rho0, cp);
    update_node<Q, 1, kArithFP32>(f1, rho1, cp);
    if (MASK && MOVING && (L0 | L1)) {
        const Nbr n0(g, x0, y, z), n1(g, x0 + 1, y, z);
#pragma unroll
        for (int k = 1; k < Q; ++k) {
            if ((L0 >> k) & 1u)
                f0[k] = wall_corrected<Q, 1>(k, f0[k], rho0, np.vel[__ldg(types + n0.at<Q>(k, +1)) & kVelMask],
                                             np.cs2inv);
            if ((L1 >> k) & 1u)
                f1[k] = wall_corrected<Q, 1>(k, f1[k], rho1, np.vel[__ldg(types + n1.at<Q>(k, +1)) & kVelMask],
                                             np.cs2inv);
        }
    }
#pragma unroll
    for (int k = 0; k < Q; ++k) {
        const __half2 v = __floats2half2_rn(f0[k], f1[k]);
        __stcs(reinterpret_cast<unsigned int*>(dst + ((unsigned)k * ks + node0)),
               *reinterpret_cast<const unsigned int*>(&v));
    }
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
    if constexpr (ST == 0) collide_node<Q, ARITH>(f, rho, ux, uy, uz, cp);
    else if constexpr (ST == 1) collide_node_dev<Q>(f, __fsub_rn(rho, 1.0f), rho, ux, uy, uz, cp);
    else collide_node_d<Q>(f, rho, ux, uy, uz, cp);
    store_node<Q, ST, MASK>(dst, g, np, types, L, nb, node, rho, f);
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
                for (int k = 0; k < Q; ++k) Store<ST>::st(n_out, k * g.ks + node, ST == 1 ? -weight<Q>(k) : (R)0);
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

// Node types: solid from the mask or a wall layer (velocity index = the last
// wall face in plbpd's face order, else obstacle); fluid nodes with a solid
// neighbour along any lattice direction are marked near-solid.
template <int Q>
__global__ void __launch_bounds__(kBlockX)
nat_types_solid_k(Geo g, const uint8_t* __restrict__ mask, int noslip_mask, uint8_t* __restrict__ types) {
    const int x = blockIdx.x * kBlockX + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= g.nx) return;
    uint8_t t = 0;
    if (mask && mask[((long long)z * g.ny + y) * g.nx + x]) t = kSolid | kObstacleVel;
    const bool in[6] = {x == g.nx - 1, x == 0, y == g.ny - 1, y == 0, z == g.nz - 1, z == 0};
    for (int f = 0; f < 6; ++f)
        if (((noslip_mask >> f) & 1) && in[f]) t = kSolid | (uint8_t)f;
    types[g.idx(x, y, z)] = t;
}

template <int Q>
__global__ void __launch_bounds__(kBlockX)
nat_types_near_k(Geo g, const uint8_t* __restrict__ types, uint8_t* __restrict__ out,
                 uint32_t* __restrict__ links) {
    const int x = blockIdx.x * kBlockX + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= g.nx) return;
    const long long node = g.idx(x, y, z);
    const uint8_t t = types[node];
    out[node] = t;
    links[node] = 0u;
    if (t & kSolid) return;
    const Nbr nb(g, x, y, z);
    uint32_t bits = 0u;   // bit k: x + c_k is solid
#pragma unroll
    for (int k = 1; k < Q; ++k) {
        const int xx = x + Lattice<Q>::cx(k), yy = y + Lattice<Q>::cy(k), zz = z + Lattice<Q>::cz(k);
        const bool inside = (g.wrap_x || (xx >= 0 && xx < g.nx)) && (g.wrap_y || (yy >= 0 && yy < g.ny)) &&
                            (g.wrap_z || (zz >= 0 && zz < g.nz));
        if (inside && (types[nb.at<Q>(k, +1)] & kSolid)) bits |= 1u << k;
    }
    if (bits) {
        out[node] = t | kNearSolid;
        links[node] = bits;
    }
}

// Solid nodes' fields: rho_solid and the wall velocity, as Boundary::reset
// leaves wall nodes (src/Boundary.cpp:58-89).
__global__ void __launch_bounds__(kBlockX)
nat_reset_fields_k(Geo g, NativeParams np, const uint8_t* __restrict__ types, float* __restrict__ rho_f,
                   float* __restrict__ u_f) {
    const int x = blockIdx.x * kBlockX + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= g.nx) return;
    const long long node = g.idx(x, y, z);
    const uint8_t t = types[node];
    if (!(t & kSolid)) return;
    const float* ub = np.vel[t & kVelMask];
    rho_f[node] = np.rho_solid;
    u_f[node] = ub[0]; u_f[g.ks + node] = ub[1]; u_f[2 * g.ks + node] = ub[2];
}

// ---------------------------------------------------------------------------
// Batches: every domain of the batch advances one step in one launch.  The
// work is a list of tiles of kBatchTile consecutive nodes of one domain (in
// its pitched node order, so a tile is a coalesced run of rows); resident
// blocks take tiles round-robin.  Per node the work is that of nat_fused_k:
// the same gather, arithmetic and bounce-back, so a domain's result does not
// depend on which other domains share its batch.
// Work items are warp tasks: (domain, y, z, x0) covering x0 .. x0+31 of one
// row, so no thread divides to find its node; descriptor fields are read
// where they are used (every lane reads the same address).
template <int Q, int ST, int ARITH, bool MOVING>
__global__ void __launch_bounds__(kBatchTile)
nat_batch_k(const BatchDomain* __restrict__ doms, const int4* __restrict__ tasks, int ntasks, int parity) {
    using T = typename Store<ST>::T;
    using R = typename Store<ST>::R;
    const int lane = threadIdx.x & 31;
    const int warps = gridDim.x * (kBatchTile / 32);
    for (int t = blockIdx.x * (kBatchTile / 32) + (threadIdx.x >> 5); t < ntasks; t += warps) {
        const int4 tk = __ldg(tasks + t);
        const BatchDomain& D = doms[tk.x];
        const Geo g = D.g;
        const int x = tk.w + lane, y = tk.y, z = tk.z;
        if (x >= g.nx) continue;
        const long long node = g.idx(x, y, z);
        const uint8_t* types = D.types;
        const uint8_t tt = __ldg(types + node);
        if (tt & kSolid) continue;
        const NativeParams& np = D.np;
        const uint32_t L = links_of<true>(tt, np.links, node);
        const T* src = static_cast<const T*>(D.f[parity]);
        T* dst = static_cast<T*>(D.f[parity ^ 1]);
        const Nbr nb(g, x, y, z);
        R f[Q];
        gather_node<Q, ST, true>(src, g, L, nb, node, f);
        R rho;
        update_node<Q, ST, ARITH>(f, rho, D.cp);
        store_node<Q, ST, true, MOVING>(dst, g, np, types, L, nb, node, rho, f);
    }
}

dim3 cell_grid(const Geo& g) { return dim3((g.nx + kBlockX - 1) / kBlockX, g.ny, g.nz); }

template <int Q, int ST, bool MASK, int ARITH>
int launch_fused(const Geo& g, const CollideParams& cp, const NativeParams& np, const void* src, void* dst,
                 const uint8_t* types, cudaStream_t st) {
    using T = typename Store<ST>::T;
    nat_fused_k<Q, ST, MASK, ARITH><<<cell_grid(g), kBlockX, 0, st>>>(g, cp, np, (const T*)src, (T*)dst, types);
    return (int)cudaGetLastError();
}

template <int Q, int ST, bool MASK, int ARITH>
int launch_raw(const Geo& g, const CollideParams& cp, const NativeParams& np, const void* src, void* dst,
               const float* rho, const float* u, const uint8_t* types, cudaStream_t st) {
    using T = typename Store<ST>::T;
    nat_collide_raw_k<Q, ST, MASK, ARITH><<<cell_grid(g), kBlockX, 0, st>>>(g, cp, np, (const T*)src, (T*)dst,
                                                                            rho, u, types);
    return (int)cudaGetLastError();
}

template <int Q, int ST, bool MASK>
int launch_gather(const Geo& g, const NativeParams& np, const void* src, void* n_out, float* rho, float* u,
                  const uint8_t* types, cudaStream_t st) {
    using T = typename Store<ST>::T;
    nat_gather_k<Q, ST, MASK><<<cell_grid(g), kBlockX, 0, st>>>(g, np, (const T*)src, (T*)n_out, rho, u, types);
    return (int)cudaGetLastError();
}

// storage x mask x arith expansion for one Q (FP16 and FP64 have one arithmetic each)
template <int Q, bool MASK>
int launch_fused_h2(const Geo& g, const CollideParams& cp, const NativeParams& np, const void* src, void* dst,
                    const uint8_t* types, cudaStream_t st) {
    const dim3 grid((g.nx + 2 * kBlockX - 1) / (2 * kBlockX), g.ny, g.nz);
    if (MASK && np.moving)
        nat_fused_h2_k<Q, true, true><<<grid, kBlockX, 0, st>>>(g, cp, np, (const __half*)src, (__half*)dst, types);
    else
        nat_fused_h2_k<Q, MASK, false><<<grid, kBlockX, 0, st>>>(g, cp, np, (const __half*)src, (__half*)dst, types);
    return (int)cudaGetLastError();
}

template <int Q>
int fused_q(int storage, int arith, bool m, const Geo& g, const CollideParams& cp, const NativeParams& np,
            const void* src, void* dst, const uint8_t* types, cudaStream_t st) {
    if (storage == 1 && g.nx % 2 == 0 && (long long)Q * g.ks < (1ll << 32))
        return m ? launch_fused_h2<Q, true>(g, cp, np, src, dst, types, st)
                 : launch_fused_h2<Q, false>(g, cp, np, src, dst, types, st);
    if (storage == 1)
        return m ? launch_fused<Q, 1, true, kArithFP32>(g, cp, np, src, dst, types, st)
                 : launch_fused<Q, 1, false, kArithFP32>(g, cp, np, src, dst, types, st);
    if (storage == 2)
        return m ? launch_fused<Q, 2, true, kArithFP32>(g, cp, np, src, dst, types, st)
                 : launch_fused<Q, 2, false, kArithFP32>(g, cp, np, src, dst, types, st);
    if (arith == kArithReference)
        return m ? launch_fused<Q, 0, true, kArithReference>(g, cp, np, src, dst, types, st)
                 : launch_fused<Q, 0, false, kArithReference>(g, cp, np, src, dst, types, st);
    return m ? launch_fused<Q, 0, true, kArithFP32>(g, cp, np, src, dst, types, st)
             : launch_fused<Q, 0, false, kArithFP32>(g, cp, np, src, dst, types, st);
}

template <int Q>
int raw_q(int storage, int arith, bool m, const Geo& g, const CollideParams& cp, const NativeParams& np,
          const void* src, void* dst, const float* rho, const float* u, const uint8_t* types, cudaStream_t st) {
    if (storage == 1)
        return m ? launch_raw<Q, 1, true, kArithFP32>(g, cp, np, src, dst, rho, u, types, st)
                 : launch_raw<Q, 1, false, kArithFP32>(g, cp, np, src, dst, rho, u, types, st);
    if (storage == 2)
        return m ? launch_raw<Q, 2, true, kArithFP32>(g, cp, np, src, dst, rho, u, types, st)
                 : launch_raw<Q, 2, false, kArithFP32>(g, cp, np, src, dst, rho, u, types, st);
    if (arith == kArithReference)
        return m ? launch_raw<Q, 0, true, kArithReference>(g, cp, np, src, dst, rho, u, types, st)
                 : launch_raw<Q, 0, false, kArithReference>(g, cp, np, src, dst, rho, u, types, st);
    return m ? launch_raw<Q, 0, true, kArithFP32>(g, cp, np, src, dst, rho, u, types, st)
             : launch_raw<Q, 0, false, kArithFP32>(g, cp, np, src, dst, rho, u, types, st);
}

template <int Q>
int gather_q(int storage, bool m, const Geo& g, const NativeParams& np, const void* src, void* n_out, float* rho,
             float* u, const uint8_t* types, cudaStream_t st) {
    if (storage == 1)
        return m ? launch_gather<Q, 1, true>(g, np, src, n_out, rho, u, types, st)
                 : launch_gather<Q, 1, false>(g, np, src, n_out, rho, u, types, st);
    if (storage == 2)
        return m ? launch_gather<Q, 2, true>(g, np, src, n_out, rho, u, types, st)
                 : launch_gather<Q, 2, false>(g, np, src, n_out, rho, u, types, st);
    return m ? launch_gather<Q, 0, true>(g, np, src, n_out, rho, u, types, st)
             : launch_gather<Q, 0, false>(g, np, src, n_out, rho, u, types, st);
}

}  // namespace

#define PLB_Q_DISPATCH(q, CALL) \
    ((q) == 9 ? CALL(9) : (q) == 19 ? CALL(19) : (q) == 27 ? CALL(27) : (int)cudaErrorInvalidValue)

int nat_fused_step(int q, int storage, int arith, bool has_mask, const Geo& g, const CollideParams& cp,
                   const NativeParams& np, const void* src, void* dst, const uint8_t* types, cudaStream_t st) {
#define CALL(Q) fused_q<Q>(storage, arith, has_mask, g, cp, np, src, dst, types, st)
    return PLB_Q_DISPATCH(q, CALL);
#undef CALL
}

int nat_collide_raw(int q, int storage, int arith, bool has_mask, const Geo& g, const CollideParams& cp,
                    const NativeParams& np, const void* src, void* dst, const float* rho, const float* u,
                    const uint8_t* types, cudaStream_t st) {
#define CALL(Q) raw_q<Q>(storage, arith, has_mask, g, cp, np, src, dst, rho, u, types, st)
    return PLB_Q_DISPATCH(q, CALL);
#undef CALL
}

int nat_gather(int q, int storage, bool has_mask, const Geo& g, const NativeParams& np, const void* src,
               void* n_out, float* rho, float* u, const uint8_t* types, cudaStream_t st) {
#define CALL(Q) gather_q<Q>(storage, has_mask, g, np, src, n_out, rho, u, types, st)
    return PLB_Q_DISPATCH(q, CALL);
#undef CALL
}

namespace {
template <int Q, int ST, int ARITH, bool MV>
const void* batch_kernel() { return (const void*)nat_batch_k<Q, ST, ARITH, MV>; }

template <bool MV>
const void* batch_kernel_for(int q, int storage, int arith) {
#define PICK(Q) (storage == 1 ? batch_kernel<Q, 1, kArithFP32, MV>() \
               : arith == kArithReference ? batch_kernel<Q, 0, kArithReference, MV>() \
                                          : batch_kernel<Q, 0, kArithFP32, MV>())
    return q == 9 ? PICK(9) : q == 19 ? PICK(19) : q == 27 ? PICK(27) : nullptr;
#undef PICK
}

template <int Q, bool MV>
void launch_batch(int storage, int arith, const BatchDomain* doms, const int4* tiles, int ntiles, int parity,
                  int blocks, cudaStream_t st) {
    if (storage == 1)
        nat_batch_k<Q, 1, kArithFP32, MV><<<blocks, kBatchTile, 0, st>>>(doms, tiles, ntiles, parity);
    else if (arith == kArithReference)
        nat_batch_k<Q, 0, kArithReference, MV><<<blocks, kBatchTile, 0, st>>>(doms, tiles, ntiles, parity);
    else
        nat_batch_k<Q, 0, kArithFP32, MV><<<blocks, kBatchTile, 0, st>>>(doms, tiles, ntiles, parity);
}
}  // namespace

int nat_batch_blocks_per_sm(int q, int storage, int arith, bool moving) {
    const void* k = moving ? batch_kernel_for<true>(q, storage, arith) : batch_kernel_for<false>(q, storage, arith);
    if (!k) return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, kBatchTile, 0) != cudaSuccess) return 0;
    return n;
}

int nat_batch_step(int q, int storage, int arith, bool moving, const BatchDomain* doms, const int4* tiles,
                   int ntiles, int parity, int blocks, cudaStream_t st) {
    if (ntiles <= 0) return 0;
    const int need = (ntiles + kBatchTile / 32 - 1) / (kBatchTile / 32);   // one task per warp
    if (blocks > need) blocks = need;
#define CALL(Q) (moving ? launch_batch<Q, true>(storage, arith, doms, tiles, ntiles, parity, blocks, st) \
                        : launch_batch<Q, false>(storage, arith, doms, tiles, ntiles, parity, blocks, st))
    if (q == 9) CALL(9);
    else if (q == 19) CALL(19);
    else if (q == 27) CALL(27);
    else return (int)cudaErrorInvalidValue;
#undef CALL
    return (int)cudaGetLastError();
}

int nat_reset_fields(const Geo& g, const NativeParams& np, const uint8_t* types, float* rho, float* u,
                     cudaStream_t st) {
    nat_reset_fields_k<<<cell_grid(g), kBlockX, 0, st>>>(g, np, types, rho, u);
    return (int)cudaGetLastError();
}

int nat_build_types(int q, const Geo& g, const uint8_t* mask, int noslip_mask, uint8_t* scratch,
                    uint8_t* types, uint32_t* links, cudaStream_t st) {
#define CALL(Q) (nat_types_solid_k<Q><<<cell_grid(g), kBlockX, 0, st>>>(g, mask, noslip_mask, scratch), \
                 nat_types_near_k<Q><<<cell_grid(g), kBlockX, 0, st>>>(g, scratch, types, links), \
                 (int)cudaGetLastError())
    return PLB_Q_DISPATCH(q, CALL);
#undef CALL
}

}  // namespace plb
