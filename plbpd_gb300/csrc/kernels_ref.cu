// Kernels for REFERENCE semantics: plbpd's operator sequence, bit for bit.
//
// One time step of plbpd (src/PLBPD.cpp:23-30) is
//   collide (in place) -> push into the other buffer, swap -> no-slip ->
//   periodic halo copies -> moments -> reset.
// Here it is three kinds of launch:
//   ref_fused_step_k : moments of the current populations (the previous
//                      step's CalcMoments), the resets, the collision and the
//                      push, for every interior node at once;
//   ref_noslip_k     : the no-slip rule on one or two wall faces;
//   ref_periodic_k   : both halo copies.
// The ρ field is written only where the no-slip rule reads it, and the
// moments are computed again by the next step, so the only per-cell traffic
// is one read and one write of each population.
#include "engine.h"
#include "ref_ops.cuh"

namespace plb {
namespace {

constexpr int kBlockX = 128;

// ---------------------------------------------------------------------------
template <int Q, int ARITH, bool FIRST>
__global__ void __launch_bounds__(kBlockX)
ref_fused_step_k(Geo g, CollideParams cp, FaceParams fp, float* __restrict__ cur,
                 float* __restrict__ nxt, float* __restrict__ rho_f, const float* __restrict__ u_f,
                 int wb_all) {
    const int x = blockIdx.x * kBlockX + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= g.nx) return;
    const long long node = g.idx(x, y, z);
    float f[Q];
#pragma unroll
    for (int k = 0; k < Q; ++k) f[k] = cur[k * g.ks + node];

    float rho, ux, uy, uz;
    if (FIRST) {
        // first step of a march: the fields as the caller left them
        rho = rho_f[node];
        ux = u_f[node]; uy = u_f[g.ks + node]; uz = u_f[2 * g.ks + node];
    } else {
        node_moments<Q>(f, rho, ux, uy, uz);
        apply_reset(fp, x, y, z, g, rho, ux, uy, uz);
    }
    // the no-slip rule of this step reads rho within one node of each wall
    bool near = false;
#pragma unroll
    for (int fc = 0; fc < 6; ++fc) near |= ((fp.noslip_mask >> fc) & 1) && near_face(fc, x, y, z, g);
    if (near && !FIRST) rho_f[node] = rho;

    collide_node<Q, ARITH>(f, rho, ux, uy, uz, cp);

#pragma unroll
    for (int k = 0; k < Q; ++k) nxt[k * g.ks + node + push_offset<Q>(k, g)] = f[k];

    // plbpd collides in place, so a slot that the next push leaves unwritten
    // still holds this step's collided value; only boundary-layer nodes own
    // such slots (D2Q9 never moves along y, so its y faces own none).  The
    // last step of a march writes every node back, which leaves the other
    // buffer exactly as plbpd's ntmp.
    const bool outer = x == 0 || x == g.nx - 1 || z == 0 || z == g.nz - 1 ||
                       (Q != 9 && (y == 0 || y == g.ny - 1));
    if (outer || wb_all) {
#pragma unroll
        for (int k = 0; k < Q; ++k) cur[k * g.ks + node] = f[k];
    }
}

// ---------------------------------------------------------------------------
// Boundary::_apply_noslip (src/Boundary.cpp:189-221) for one face: for every
// wall node A and kp = 1..Q-1, with B = A + c_kp and k = rev(kp),
//   n[B][kp] = n[A][k] - 2 w_k rho[B] (c_k . u_b) / c_s^2.
// plbpd visits A in (z, y, x) order.  When B is itself a wall node of the
// same face the two updates form a pair that shares slots: the node visited
// first reads the original value, the second reads what the first wrote.
// The thread of the first node of each pair performs both updates, so the
// result is the serial one and no slot is touched by two threads.
template <int Q>
__global__ void ref_noslip_k(Geo g, FaceParams fp, int f0, int f1, int nfaces,
                             float* __restrict__ n, const float* __restrict__ rho) {
    const int face = (blockIdx.z < (unsigned)((gridDim.z) / nfaces)) ? f0 : f1;
    const int zz = blockIdx.z % (gridDim.z / nfaces);
    // plane coordinates: (a, b) span the two in-plane axes
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    const int b = blockIdx.y * blockDim.y + threadIdx.y + zz * (gridDim.y * blockDim.y);
    int x, y, z, na, nb;
    if (face <= 1) { na = g.ny; nb = g.nz; y = a; z = b; x = face == 0 ? g.nx - 1 : 0; }
    else if (face <= 3) { na = g.nx; nb = g.nz; x = a; z = b; y = face == 2 ? g.ny - 1 : 0; }
    else { na = g.nx; nb = g.ny; x = a; y = b; z = face == 4 ? g.nz - 1 : 0; }
    if (a >= na || b >= nb) return;
    const float* ub = fp.vel[face];
    const long long A = g.idx(x, y, z);
#pragma unroll
    for (int kp = 1; kp < Q; ++kp) {
        const int k = rev_of(kp);
        const int bx = x + Lattice<Q>::cx(kp), by = y + Lattice<Q>::cy(kp), bz = z + Lattice<Q>::cz(kp);
        const long long B = g.idx(bx, by, bz);
        if (face_contains<Q>(face, bx, by, bz, g)) {
            // lexicographic (z, y, x) order of B - A = c_kp
            const int cz = Lattice<Q>::cz(kp), cy = Lattice<Q>::cy(kp), cx = Lattice<Q>::cx(kp);
            const bool a_first = cz > 0 || (cz == 0 && (cy > 0 || (cy == 0 && cx > 0)));
            if (!a_first) continue;   // the pair belongs to B's thread
            // A (first) writes (B, kp) from the original (A, k); B then writes
            // (A, k) from the value A just wrote.
            const float t1 = wall_term<Q>(k, rho[B], dot_c_full<Q>(k, ub), fp.cs2inv);
            const float vB = __fsub_rn(n[k * g.ks + A], t1);
            const float t2 = wall_term<Q>(kp, rho[A], dot_c_full<Q>(kp, ub), fp.cs2inv);
            const float vA = __fsub_rn(vB, t2);
            n[kp * g.ks + B] = vB;
            n[k * g.ks + A] = vA;
        } else {
            const float t = wall_term<Q>(k, rho[B], dot_c_full<Q>(k, ub), fp.cs2inv);
            n[kp * g.ks + B] = __fsub_rn(n[k * g.ks + A], t);
        }
    }
}

// ---------------------------------------------------------------------------
// Boundary::_apply_periodicity_east_west then _north_south
// (src/Boundary.cpp:234-281), merged: the north/south copy runs second in
// plbpd and overwrites the east/west copy on the slots both write, so the
// east/west part skips those; neither copy reads a slot the other writes.
template <int Q>
__global__ void ref_periodic_k(Geo g, FaceParams fp, float* __restrict__ n) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int z = blockIdx.y;
    const int n_ew = fp.ew_periodic ? g.ny : 0;
    const int n_ns = fp.ns_periodic ? g.nx : 0;
    if (t < n_ew) {
        const int y = t;
#pragma unroll
        for (int k = 1; k < Q; ++k) {
            const int cx = Lattice<Q>::cx(k), cy = Lattice<Q>::cy(k);
            if (cx == 0) continue;
            const int xd = cx > 0 ? 0 : g.nx - 1;
            const int xs = cx > 0 ? g.nx : -1;
            if (fp.ns_periodic && ((cy > 0 && y == 0) || (cy < 0 && y == g.ny - 1))) continue;
            n[k * g.ks + g.idx(xd, y, z)] = n[k * g.ks + g.idx(xs, y, z)];
        }
    } else if (t < n_ew + n_ns) {
        const int x = t - n_ew;
#pragma unroll
        for (int k = 1; k < Q; ++k) {
            const int cy = Lattice<Q>::cy(k);
            if (cy == 0) continue;
            const int yd = cy > 0 ? 0 : g.ny - 1;
            const int ysrc = cy > 0 ? g.ny : -1;
            n[k * g.ks + g.idx(x, yd, z)] = n[k * g.ks + g.idx(x, ysrc, z)];
        }
    }
}

// ---------------------------------------------------------------------------
// Unfused operators.
template <int Q, int ARITH>
__global__ void __launch_bounds__(kBlockX)
ref_collide_k(Geo g, CollideParams cp, float* __restrict__ n, const float* __restrict__ rho_f,
              const float* __restrict__ u_f) {
    const int x = blockIdx.x * kBlockX + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= g.nx) return;
    const long long node = g.idx(x, y, z);
    float f[Q];
#pragma unroll
    for (int k = 0; k < Q; ++k) f[k] = n[k * g.ks + node];
    collide_node<Q, ARITH>(f, rho_f[node], u_f[node], u_f[g.ks + node], u_f[2 * g.ks + node], cp);
#pragma unroll
    for (int k = 0; k < Q; ++k) n[k * g.ks + node] = f[k];
}

template <int Q>
__global__ void __launch_bounds__(kBlockX)
ref_push_k(Geo g, const float* __restrict__ n, float* __restrict__ nt) {
    const int x = blockIdx.x * kBlockX + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= g.nx) return;
    const long long node = g.idx(x, y, z);
#pragma unroll
    for (int k = 0; k < Q; ++k) nt[k * g.ks + node + push_offset<Q>(k, g)] = n[k * g.ks + node];
}

template <int Q>
__global__ void __launch_bounds__(kBlockX)
ref_moments_k(Geo g, const float* __restrict__ n, float* __restrict__ rho_f, float* __restrict__ u_f) {
    const int x = blockIdx.x * kBlockX + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= g.nx) return;
    const long long node = g.idx(x, y, z);
    float f[Q];
#pragma unroll
    for (int k = 0; k < Q; ++k) f[k] = n[k * g.ks + node];
    float r, ux, uy, uz;
    node_moments<Q>(f, r, ux, uy, uz);
    rho_f[node] = r;
    u_f[node] = ux; u_f[g.ks + node] = uy; u_f[2 * g.ks + node] = uz;
}

__global__ void __launch_bounds__(kBlockX)
ref_reset_k(Geo g, FaceParams fp, int velocity, int density, float* __restrict__ rho_f,
            float* __restrict__ u_f) {
    const int x = blockIdx.x * kBlockX + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= g.nx) return;
    const long long node = g.idx(x, y, z);
    if (velocity) {
        for (int f = 0; f < 6; ++f)
            if (((fp.vel_mask >> f) & 1) && in_face(f, x, y, z, g)) {
                u_f[node] = fp.vel[f][0]; u_f[g.ks + node] = fp.vel[f][1]; u_f[2 * g.ks + node] = fp.vel[f][2];
            }
    }
    if (density) {
        for (int f = 0; f < 6; ++f)
            if (((fp.noslip_mask >> f) & 1) && in_face(f, x, y, z, g)) rho_f[node] = fp.rho_solid;
    }
}

dim3 cell_grid(const Geo& g) { return dim3((g.nx + kBlockX - 1) / kBlockX, g.ny, g.nz); }

template <int Q>
int fused_dispatch(int arith, bool first, bool wb_all, const Geo& g, const CollideParams& cp,
                   const FaceParams& fp, float* cur, float* nxt, float* rho, float* u, cudaStream_t st) {
    const dim3 grid = cell_grid(g);
    const int wb = wb_all ? 1 : 0;
    if (arith == kArithReference) {
        if (first) ref_fused_step_k<Q, kArithReference, true><<<grid, kBlockX, 0, st>>>(g, cp, fp, cur, nxt, rho, u, wb);
        else ref_fused_step_k<Q, kArithReference, false><<<grid, kBlockX, 0, st>>>(g, cp, fp, cur, nxt, rho, u, wb);
    } else if (arith == kArithTRT) {
        if (first) ref_fused_step_k<Q, kArithTRT, true><<<grid, kBlockX, 0, st>>>(g, cp, fp, cur, nxt, rho, u, wb);
        else ref_fused_step_k<Q, kArithTRT, false><<<grid, kBlockX, 0, st>>>(g, cp, fp, cur, nxt, rho, u, wb);
    } else {
        if (first) ref_fused_step_k<Q, kArithFP32, true><<<grid, kBlockX, 0, st>>>(g, cp, fp, cur, nxt, rho, u, wb);
        else ref_fused_step_k<Q, kArithFP32, false><<<grid, kBlockX, 0, st>>>(g, cp, fp, cur, nxt, rho, u, wb);
    }
    return (int)cudaGetLastError();
}

}  // namespace

#define PLB_Q_DISPATCH(q, CALL) \
    ((q) == 9 ? CALL(9) : (q) == 19 ? CALL(19) : (q) == 27 ? CALL(27) : (int)cudaErrorInvalidValue)

int ref_fused_step(int q, int arith, bool first, bool wb_all, const Geo& g, const CollideParams& cp,
                   const FaceParams& fp, float* cur, float* nxt, float* rho, float* u,
                   cudaStream_t st) {
#define CALL(Q) fused_dispatch<Q>(arith, first, wb_all, g, cp, fp, cur, nxt, rho, u, st)
    return PLB_Q_DISPATCH(q, CALL);
#undef CALL
}

int ref_noslip(int q, const Geo& g, const FaceParams& fp, const int* face_list, int nfaces,
               float* n, const float* rho, cudaStream_t st) {
    if (nfaces <= 0) return 0;
    // plane extents of the first face (faces grouped together are parallel)
    const int f0 = face_list[0];
    const int f1 = nfaces > 1 ? face_list[1] : f0;
    int na, nb;
    if (f0 <= 1) { na = g.ny; nb = g.nz; }
    else if (f0 <= 3) { na = g.nx; nb = g.nz; }
    else { na = g.nx; nb = g.ny; }
    const dim3 block(32, 4);
    const int gy = (nb + block.y - 1) / block.y;
    // gridDim.y is capped at 65535; fold the rest of b into z
    const int gy_cap = gy > 16384 ? 16384 : gy;
    const int fold = (gy + gy_cap - 1) / gy_cap;
    const dim3 grid((na + block.x - 1) / block.x, gy_cap, fold * nfaces);
#define CALL(Q) (ref_noslip_k<Q><<<grid, block, 0, st>>>(g, fp, f0, f1, nfaces, n, rho), (int)cudaGetLastError())
    return PLB_Q_DISPATCH(q, CALL);
#undef CALL
}

int ref_periodic(int q, const Geo& g, const FaceParams& fp, float* n, cudaStream_t st) {
    const int total = (fp.ew_periodic ? g.ny : 0) + (fp.ns_periodic ? g.nx : 0);
    if (total == 0) return 0;
    const dim3 grid((total + 127) / 128, g.nz);
#define CALL(Q) (ref_periodic_k<Q><<<grid, 128, 0, st>>>(g, fp, n), (int)cudaGetLastError())
    return PLB_Q_DISPATCH(q, CALL);
#undef CALL
}

int ref_collide(int q, int arith, const Geo& g, const CollideParams& cp, float* n,
                const float* rho, const float* u, cudaStream_t st) {
    const dim3 grid = cell_grid(g);
#define CALL(Q) (arith == kArithReference \
    ? (ref_collide_k<Q, kArithReference><<<grid, kBlockX, 0, st>>>(g, cp, n, rho, u), 0) \
    : arith == kArithTRT ? (ref_collide_k<Q, kArithTRT><<<grid, kBlockX, 0, st>>>(g, cp, n, rho, u), 0) \
    : (ref_collide_k<Q, kArithFP32><<<grid, kBlockX, 0, st>>>(g, cp, n, rho, u), 0), (int)cudaGetLastError())
    return PLB_Q_DISPATCH(q, CALL);
#undef CALL
}

int ref_push(int q, const Geo& g, const float* n, float* nt, cudaStream_t st) {
    const dim3 grid = cell_grid(g);
#define CALL(Q) (ref_push_k<Q><<<grid, kBlockX, 0, st>>>(g, n, nt), (int)cudaGetLastError())
    return PLB_Q_DISPATCH(q, CALL);
#undef CALL
}

int ref_moments(int q, const Geo& g, const float* n, float* rho, float* u, cudaStream_t st) {
    const dim3 grid = cell_grid(g);
#define CALL(Q) (ref_moments_k<Q><<<grid, kBlockX, 0, st>>>(g, n, rho, u), (int)cudaGetLastError())
    return PLB_Q_DISPATCH(q, CALL);
#undef CALL
}

int ref_reset(const Geo& g, const FaceParams& fp, bool velocity, bool density, float* rho, float* u,
              cudaStream_t st) {
    ref_reset_k<<<cell_grid(g), kBlockX, 0, st>>>(g, fp, velocity ? 1 : 0, density ? 1 : 0, rho, u);
    return (int)cudaGetLastError();
}

}  // namespace plb
