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
#include <cstdlib>
#include <cstring>

#include "engine.h"
#include "ref_ops.cuh"

namespace plb {
namespace {

constexpr int kBlockX = 128;

// ---------------------------------------------------------------------------
// A node's population loads, with 256-byte L2 fills (the next warp of the row
// reads the other half).  Plain loads, not the read-only path: the step
// writes boundary-layer nodes' own slots of the same buffer back.
__device__ __forceinline__ float ld_row(const float* p) {
    float r;
    asm volatile("ld.global.L2::256B.f32 %0, [%1];" : "=f"(r) : "l"(p));
    return r;
}
__device__ __forceinline__ float2 ld_row2(const float* p) {
    float2 r;
    asm volatile("ld.global.L2::256B.v2.f32 {%0, %1}, [%2];" : "=f"(r.x), "=f"(r.y) : "l"(p));
    return r;
}

// One node's work before the push: its moments (or, on a march's first step,
// the fields as the caller left them), the resets, the density the no-slip
// rule of this step reads, and the collision in place.
template <int Q, int ARITH, bool FIRST>
__device__ __forceinline__ void ref_node_update(const Geo& g, const CollideParams& cp, const FaceParams& fp,
                                                float* __restrict__ rho_f, const float* __restrict__ u_f, int x,
                                                int y, int z, long long node, float (&f)[Q]) {
    float rho, ux, uy, uz;
    if (FIRST) {
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
}

// plbpd collides in place, so a slot that the next push leaves unwritten
// still holds this step's collided value; only boundary-layer nodes own such
// slots (D2Q9 never moves along y, so its y faces own none).  The last step
// of a march writes every node back, which leaves the other buffer exactly as
// plbpd's ntmp.
template <int Q>
__device__ __forceinline__ bool ref_outer(const Geo& g, int x, int y, int z) {
    return x == 0 || x == g.nx - 1 || z == 0 || z == g.nz - 1 || (Q != 9 && (y == 0 || y == g.ny - 1));
}

template <int Q, int ARITH, bool FIRST>
__global__ void __launch_bounds__(kBlockX, (Q == 19 && ARITH != kArithReference) ? 6 : 0)
ref_fused_step_k(Geo g, CollideParams cp, FaceParams fp, float* __restrict__ cur,
                 float* __restrict__ nxt, float* __restrict__ rho_f, const float* __restrict__ u_f,
                 int wb_all) {
    const int x = blockIdx.x * kBlockX + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= g.nx) return;
    const long long node = g.idx(x, y, z);
    float f[Q];
#pragma unroll
    for (int k = 0; k < Q; ++k) f[k] = ld_row(cur + k * g.ks + node);
    ref_node_update<Q, ARITH, FIRST>(g, cp, fp, rho_f, u_f, x, y, z, node, f);
#pragma unroll
    for (int k = 0; k < Q; ++k) nxt[k * g.ks + node + push_offset<Q>(k, g)] = f[k];
    if (ref_outer<Q>(g, x, y, z) || wb_all) {
#pragma unroll
        for (int k = 0; k < Q; ++k) cur[k * g.ks + node] = f[k];
    }
}

// The same step for two neighbouring nodes (x0, x0 + 1) a thread, nx even
// and x0 even: a row starts at element offset 8 and has a pitch of a
// multiple of 8, so every pair is an aligned float2, loaded in one access.
// Each node's update is ref_node_update, so the values are those of the
// one-node kernel.  The push of direction k moves the pair by c_k; along y
// and z that is another row, along x it is one element, so the stores are
// realigned through the neighbouring lanes: for c_x = +1 the pair slot
// (x0, x0 + 1) receives (the previous lane's x0 - 1, this lane's x0), for
// c_x = -1 (this lane's x0 + 1, the next lane's x0 + 2).  A slot whose source
// is in another warp or outside the row is stored alone by the lane that
// holds its source, and a slot whose source is a halo node is not stored at
// all -- exactly the slots the one-node kernel writes, each written once.
template <int Q, int ARITH, bool FIRST, int BX>
__global__ void __launch_bounds__(BX)
ref_fused_pair_k(Geo g, CollideParams cp, FaceParams fp, float* __restrict__ cur, float* __restrict__ nxt,
                 float* __restrict__ rho_f, const float* __restrict__ u_f, int wb_all) {
    const unsigned kFull = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int x0 = 2 * (blockIdx.x * BX + threadIdx.x);
    const int y = blockIdx.y, z = blockIdx.z;
    const bool active = x0 < g.nx;
    const long long node0 = g.idx(active ? x0 : 0, y, z);
    float a[Q], b[Q];   // nodes x0 and x0 + 1
    if (active) {
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            const float2 v = ld_row2(cur + k * g.ks + node0);
            a[k] = v.x;
            b[k] = v.y;
        }
        ref_node_update<Q, ARITH, FIRST>(g, cp, fp, rho_f, u_f, x0, y, z, node0, a);
        ref_node_update<Q, ARITH, FIRST>(g, cp, fp, rho_f, u_f, x0 + 1, y, z, node0 + 1, b);
    } else {
#pragma unroll
        for (int k = 0; k < Q; ++k) a[k] = b[k] = 0.0f;
    }
    const bool lo_edge = lane == 0 || x0 == 0;           // x0 - 1 is not the previous lane's
    const bool hi_edge = lane == 31 || x0 + 2 >= g.nx;   // x0 + 2 is not the next lane's
#pragma unroll
    for (int k = 0; k < Q; ++k) {
        const int cx = Lattice<Q>::cx(k);
        float* d = nxt + k * g.ks + node0 + (long long)Lattice<Q>::cy(k) * g.ys +
                   (long long)Lattice<Q>::cz(k) * g.zs;   // slot x0 of the destination row
        if (cx == 0) {
            if (active) *reinterpret_cast<float2*>(d) = make_float2(a[k], b[k]);
        } else if (cx > 0) {
            const float pb = __shfl_up_sync(kFull, b[k], 1);
            if (active) {
                if (!lo_edge) *reinterpret_cast<float2*>(d) = make_float2(pb, a[k]);
                else d[1] = a[k];
                if (hi_edge) d[2] = b[k];
            }
        } else {
            const float na = __shfl_down_sync(kFull, a[k], 1);
            if (active) {
                if (!hi_edge) *reinterpret_cast<float2*>(d) = make_float2(b[k], na);
                else d[0] = b[k];
                if (lo_edge) d[-1] = a[k];
            }
        }
    }
    if (active) {
        const bool oa = ref_outer<Q>(g, x0, y, z) || wb_all, ob = ref_outer<Q>(g, x0 + 1, y, z) || wb_all;
        if (oa || ob) {
#pragma unroll
            for (int k = 0; k < Q; ++k) {
                float* c = cur + k * g.ks + node0;
                if (oa && ob) *reinterpret_cast<float2*>(c) = make_float2(a[k], b[k]);
                else if (oa) c[0] = a[k];
                else c[1] = b[k];
            }
        }
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
    // every value this thread reads first: its stores go to slots no later
    // read of this thread (or of another thread, see above) touches, and
    // with the reads in between the compiler would have to keep each read
    // after the previous store (18 round trips in a row for D3Q19)
    float nA[Q];
#pragma unroll
    for (int kp = 1; kp < Q; ++kp) nA[kp] = n[rev_of(kp) * g.ks + A];
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
            const float vB = __fsub_rn(nA[kp], t1);
            const float t2 = wall_term<Q>(kp, rho[A], dot_c_full<Q>(kp, ub), fp.cs2inv);
            const float vA = __fsub_rn(vB, t2);
            n[kp * g.ks + B] = vB;
            n[k * g.ks + A] = vA;
        } else {
            const float t = wall_term<Q>(k, rho[B], dot_c_full<Q>(k, ub), fp.cs2inv);
            n[kp * g.ks + B] = __fsub_rn(nA[kp], t);
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
    // a thread reads halo slots and writes interior ones, so all its reads
    // go first (with a store between two reads the compiler keeps them in
    // order: one round trip after another)
    float v[Q];
    if (t < n_ew) {
        const int y = t;
#pragma unroll
        for (int k = 1; k < Q; ++k) {
            const int cx = Lattice<Q>::cx(k);
            if (cx != 0) v[k] = n[k * g.ks + g.idx(cx > 0 ? g.nx : -1, y, z)];
        }
#pragma unroll
        for (int k = 1; k < Q; ++k) {
            const int cx = Lattice<Q>::cx(k), cy = Lattice<Q>::cy(k);
            if (cx == 0) continue;
            if (fp.ns_periodic && ((cy > 0 && y == 0) || (cy < 0 && y == g.ny - 1))) continue;
            n[k * g.ks + g.idx(cx > 0 ? 0 : g.nx - 1, y, z)] = v[k];
        }
    } else if (t < n_ew + n_ns) {
        const int x = t - n_ew;
#pragma unroll
        for (int k = 1; k < Q; ++k) {
            const int cy = Lattice<Q>::cy(k);
            if (cy != 0) v[k] = n[k * g.ks + g.idx(x, cy > 0 ? g.ny : -1, z)];
        }
#pragma unroll
        for (int k = 1; k < Q; ++k) {
            const int cy = Lattice<Q>::cy(k);
            if (cy != 0) n[k * g.ks + g.idx(x, cy > 0 ? 0 : g.ny - 1, z)] = v[k];
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

// Which form of the step runs: the pair form whenever nx is even, unless
// PLB_REF_PAIR=0.  Measured on 256^3 / 192^3 / 2048^2 channels with plbpd's
// arithmetic, one-node against pair form: D3Q19 31.8k -> 33.7k MLUPS (FP32
// arithmetic 31.7k -> 34.0k), D3Q27 16.4k -> 19.4k, D2Q9 51.9k -> 62.5k.
bool ref_use_pair(int nx) {
    if (nx % 2 != 0) return false;
    const char* e = std::getenv("PLB_REF_PAIR");
    return !(e && std::strcmp(e, "0") == 0);
}

template <int Q, int ARITH>
int launch_ref_pair(bool first, const Geo& g, const CollideParams& cp, const FaceParams& fp, float* cur, float* nxt,
                    float* rho, float* u, int wb, cudaStream_t st) {
    auto go = [&](auto bxc) {
        constexpr int BX = decltype(bxc)::value;
        const dim3 grid((unsigned)((g.nx + 2 * BX - 1) / (2 * BX)), (unsigned)g.ny, (unsigned)g.nz);
        if (first) ref_fused_pair_k<Q, ARITH, true, BX><<<grid, BX, 0, st>>>(g, cp, fp, cur, nxt, rho, u, wb);
        else ref_fused_pair_k<Q, ARITH, false, BX><<<grid, BX, 0, st>>>(g, cp, fp, cur, nxt, rho, u, wb);
    };
    // whole 128-thread blocks when the row is a whole number of them, else one warp a block
    if (g.nx % (2 * kBlockX) == 0) go(std::integral_constant<int, kBlockX>{});
    else go(std::integral_constant<int, 32>{});
    return (int)cudaGetLastError();
}

template <int Q>
int fused_dispatch(int arith, bool first, bool wb_all, const Geo& g, const CollideParams& cp,
                   const FaceParams& fp, float* cur, float* nxt, float* rho, float* u, cudaStream_t st) {
    const dim3 grid = cell_grid(g);
    const int wb = wb_all ? 1 : 0;
    if (ref_use_pair(g.nx)) {
        if (arith == kArithReference) return launch_ref_pair<Q, kArithReference>(first, g, cp, fp, cur, nxt, rho, u, wb, st);
        if (arith == kArithTRT) return launch_ref_pair<Q, kArithTRT>(first, g, cp, fp, cur, nxt, rho, u, wb, st);
        return launch_ref_pair<Q, kArithFP32>(first, g, cp, fp, cur, nxt, rho, u, wb, st);
    }
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
