// Whole marches of small D2Q9 domains under REFERENCE semantics in one launch.
//
// A plbpd time step (src/PLBPD.cpp:23-30) on a small domain is a few
// microseconds of work split over three dependent launches (kernels_ref.cu:
// fused collide/push, no-slip, periodic copies), so a 128 x 64 channel runs
// at the launch rate, not the memory rate.  Here one thread-block cluster
// holds the domain's whole state in distributed shared memory -- both
// population buffers and the rho field over x = -1..nx and z = -1..nz of the
// y = 0 plane, the only plane a D2Q9 step touches (its velocities have no y
// component) -- and runs every step of the march.  Each CTA owns a band of
// rows; a push or a no-slip write that lands in another CTA's rows is a plain
// store through the cluster's shared-memory window.  Loads and stores of the
// populations at the start and end of the march are the only global-memory
// traffic.
//
// Per node the operations are those of the three-launch path, in the same
// order and with the same device functions, so the result is bit-identical
// to it (and to plbpd): the fused phase is ref_fused_step_k's body, the
// no-slip phase ref_noslip_k's (with its serial order of in-plane pairs), the
// periodic phase ref_periodic_k's east/west copy.  A step has one cluster
// barrier after the pushes, and one after each no-slip face group unless
// every no-slip access stays inside one CTA (up/down walls with two or more
// rows a CTA: then a CTA barrier); the periodic copies of a CTA's own rows
// end with a CTA barrier.  The barriers are the hardware's; no thread waits
// on a flag.
#include <cooperative_groups.h>

#include "engine.h"
#include "ref_ops.cuh"

namespace cg = cooperative_groups;

namespace plb {
namespace {

constexpr int Q9 = 9;
static_assert(Lattice<Q9>::cx(1) == 1 && Lattice<Q9>::cx(5) == 1 && Lattice<Q9>::cx(7) == 1 &&
                  Lattice<Q9>::cx(2) == -1 && Lattice<Q9>::cx(6) == -1 && Lattice<Q9>::cx(8) == -1 &&
                  Lattice<Q9>::cx(3) == 0 && Lattice<Q9>::cx(4) == 0,
              "the periodic phase takes the directions with c_x = +1 as the odd ones");

// The march's state in the cluster's shared memory.  Row z (-1..nz) lives in
// the CTA that owns it, at row slot z - owner * R + 1 of that CTA's arrays
// (slot 0 of CTA 0 is the halo row -1; the last CTA's last used slot is the
// halo row nz).  A CTA's arrays: population buffer b, direction k at
// pop + ((b * 9 + k) * slots + slot) * W + x + 1; rho at rho + slot * W + x + 1.
// Another CTA's element is reached through the cluster's shared-memory
// window (mapa); the CTA's own elements directly.
struct MarchView {
    cg::cluster_group cl;
    float* pop;   // this CTA's arrays
    float* rho;
    int me, C, R, W, slots;
    int row0, row1;   // the interior rows this CTA owns: [row0, row1)
    // owner of a row within one row of this CTA's band (every access of a
    // step: a node's neighbours, a wall node's partner), without a division
    __device__ __forceinline__ int owner(int z) const {
        if (z < row0) return me > 0 ? me - 1 : 0;        // row -1 is CTA 0's
        if (z >= row1) return me < C - 1 ? me + 1 : me;  // row nz is the last CTA's
        return me;
    }
    __device__ __forceinline__ float* at(float* base, int c, int off) const {
        return c == me ? base + off : cl.map_shared_rank(base + off, c);
    }
    __device__ __forceinline__ float* p(int b, int k, int x, int z) const {
        const int c = owner(z);
        return at(pop, c, ((b * Q9 + k) * slots + (z - c * R + 1)) * W + (x + 1));
    }
    __device__ __forceinline__ float* r(int x, int z) const {
        const int c = owner(z);
        return at(rho, c, (z - c * R + 1) * W + (x + 1));
    }
};

// u_b of a face, read with constant indices (a run-time index into the
// parameter block would copy it to local memory).
__device__ __forceinline__ void face_velocity(const FaceParams& fp, int face, float (&ub)[3]) {
#pragma unroll
    for (int f = 0; f < 6; ++f)
        if (f == face) {
            ub[0] = fp.vel[f][0];
            ub[1] = fp.vel[f][1];
            ub[2] = fp.vel[f][2];
        }
}

// ref_noslip_k's rule for the wall node A = (x, 0, z) of face `face`,
// against the cluster's state (buffer b).
__device__ __forceinline__ void noslip_node(const Geo& g, const FaceParams& fp, const MarchView& v, int b, int face,
                                            int x, int z) {
    float ub[3];
    face_velocity(fp, face, ub);
#pragma unroll
    for (int kp = 1; kp < Q9; ++kp) {
        const int k = rev_of(kp);
        const int bx = x + Lattice<Q9>::cx(kp), bz = z + Lattice<Q9>::cz(kp);
        if (face_contains<Q9>(face, bx, 0, bz, g)) {
            // an in-plane pair: the node first in (z, y, x) order does both
            const int cz = Lattice<Q9>::cz(kp), cx = Lattice<Q9>::cx(kp);
            const bool a_first = cz > 0 || (cz == 0 && cx > 0);
            if (!a_first) continue;
            const float t1 = wall_term<Q9>(k, *v.r(bx, bz), dot_c_full<Q9>(k, ub), fp.cs2inv);
            const float vB = __fsub_rn(*v.p(b, k, x, z), t1);
            const float t2 = wall_term<Q9>(kp, *v.r(x, z), dot_c_full<Q9>(kp, ub), fp.cs2inv);
            const float vA = __fsub_rn(vB, t2);
            *v.p(b, kp, bx, bz) = vB;
            *v.p(b, k, x, z) = vA;
        } else {
            const float t = wall_term<Q9>(k, *v.r(bx, bz), dot_c_full<Q9>(k, ub), fp.cs2inv);
            *v.p(b, kp, bx, bz) = __fsub_rn(*v.p(b, k, x, z), t);
        }
    }
}

template <int ARITH>
__global__ void __launch_bounds__(kRefClusterThreads)
ref_march_cluster_k(Geo g, CollideParams cp, FaceParams fp, RefNoslipPlan plan, float* b0, float* b1,
                    float* rho_g, const float* u_g, int cur0, int nsteps, int first, int wb_last, int R,
                    int local_noslip) {
    extern __shared__ float sm[];
    cg::cluster_group cl = cg::this_cluster();
    const int c = (int)cl.block_rank();
    const int C = (int)cl.num_blocks();
    const int W = g.nx + 2, plane = (R + 2) * W;
    float* my_pop = sm;
    float* my_rho = sm + 2 * Q9 * plane;
    const int row0 = c * R;                          // first interior row owned
    const int row1 = min(row0 + R, g.nz);            // one past the last
    const MarchView v{cl, my_pop, my_rho, c, C, R, W, R + 2, row0, row1};
    const int zlo = c == 0 ? -1 : row0;              // rows held, halo included
    const int zhi = c == C - 1 ? g.nz : row1 - 1;
    const int nrow = zhi - zlo + 1;

    // ---- global -> cluster --------------------------------------------------
    for (int i = threadIdx.x; i < 2 * Q9 * nrow * W; i += blockDim.x) {
        const int xw = i % W, rest = i / W;
        const int z = zlo + rest % nrow, bk = rest / nrow;
        const float* src = bk < Q9 ? b0 : b1;
        my_pop[(bk * v.slots + (z - row0 + 1)) * W + xw] = src[(bk % Q9) * g.ks + g.idx(xw - 1, 0, z)];
    }
    for (int i = threadIdx.x; i < nrow * W; i += blockDim.x) {
        const int xw = i % W, z = zlo + i / W;
        my_rho[(z - row0 + 1) * W + xw] = rho_g[g.idx(xw - 1, 0, z)];
    }
    cl.sync();

    const int own_nodes = (row1 - row0) * g.nx;
    int cur = cur0;
    for (int t = 0; t < nsteps; ++t) {
        const bool FIRST = first && t == 0;
        const bool wb = wb_last && t == nsteps - 1;
        // ---- phase 1: moments, resets, collision, push (ref_fused_step_k) ----
        for (int i = threadIdx.x; i < own_nodes; i += blockDim.x) {
            const int z = row0 + i / g.nx, x = i % g.nx;
            float* at = my_pop + (z - row0 + 1) * W + (x + 1);
            float f[Q9];
#pragma unroll
            for (int k = 0; k < Q9; ++k) f[k] = at[(cur * Q9 + k) * plane];
            float rho, ux, uy, uz;
            if (FIRST) {
                const long long node = g.idx(x, 0, z);
                rho = my_rho[(z - row0 + 1) * W + (x + 1)];
                ux = u_g[node]; uy = u_g[g.ks + node]; uz = u_g[2 * g.ks + node];
            } else {
                node_moments<Q9>(f, rho, ux, uy, uz);
                apply_reset(fp, x, 0, z, g, rho, ux, uy, uz);
                bool near = false;
#pragma unroll
                for (int fc = 0; fc < 6; ++fc) near |= ((fp.noslip_mask >> fc) & 1) && near_face(fc, x, 0, z, g);
                if (near) my_rho[(z - row0 + 1) * W + (x + 1)] = rho;
            }
            collide_node<Q9, ARITH>(f, rho, ux, uy, uz, cp);
#pragma unroll
            for (int k = 0; k < Q9; ++k) *v.p(cur ^ 1, k, x + Lattice<Q9>::cx(k), z + Lattice<Q9>::cz(k)) = f[k];
            const bool outer = x == 0 || x == g.nx - 1 || z == 0 || z == g.nz - 1;
            if (outer || wb) {
#pragma unroll
                for (int k = 0; k < Q9; ++k) at[(cur * Q9 + k) * plane] = f[k];
            }
        }
        cl.sync();
        cur ^= 1;
        // ---- phase 2: no-slip, face groups in plbpd's order (ref_noslip_k).
        // A wall node is handled by the CTA that owns its row, so most
        // accesses are to its own shared memory. ----
#pragma unroll
        for (int gi = 0; gi < 6; ++gi) {
            if (gi >= plan.ngroups) break;
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                if (j >= plan.len[gi]) break;
                const int face = plan.faces[gi][j];
                if (face >= 4) {   // up / down: one row, owned by one CTA
                    const int z = face == 4 ? g.nz - 1 : 0;
                    if (z >= row0 && z < row1)
                        for (int x = threadIdx.x; x < g.nx; x += blockDim.x) noslip_node(g, fp, v, cur, face, x, z);
                } else {           // east / west: a column, every CTA its rows
                    const int x = face == 0 ? g.nx - 1 : 0;
                    for (int z = row0 + threadIdx.x; z < row1; z += blockDim.x) noslip_node(g, fp, v, cur, face, x, z);
                }
            }
            // when every wall node's partners and their rho lie in its own
            // CTA's rows (up/down walls, two or more rows a CTA), no other
            // CTA takes part in this phase: a CTA barrier orders it
            if (local_noslip) __syncthreads();
            else cl.sync();
        }
        // ---- phase 3: east/west halo copies of this CTA's rows
        // (ref_periodic_k; D2Q9 has no north/south copy: no velocity moves
        // along y).  Only this CTA's rows are read and written, and the next
        // step's collision reads only them, so a CTA barrier suffices: the
        // next step's pushes into other CTAs go to the other buffer, and the
        // rho values they overwrite were read before the barrier above. ----
        if (fp.ew_periodic) {
            for (int i = threadIdx.x; i < (row1 - row0) * 6; i += blockDim.x) {
                const int z = row0 + i / 6, j = i % 6;
                // the directions with c_x != 0: 1, 5, 7 (c_x = +1) and 2, 6, 8 (c_x = -1)
                const int k = j < 2 ? j + 1 : j + 3;
                const bool east = (k & 1) != 0;
                const int xd = east ? 0 : g.nx - 1;
                const int xs = east ? g.nx : -1;
                float* rowp = my_pop + ((cur * Q9 + k) * v.slots + (z - row0 + 1)) * W;
                rowp[xd + 1] = rowp[xs + 1];
            }
        }
        __syncthreads();
    }

    // ---- cluster -> global (this CTA's rows).  The last cluster barrier
    // ended every access of other CTAs to this CTA's arrays, so no CTA exits
    // while another still reads or writes its shared memory. ----
    for (int i = threadIdx.x; i < 2 * Q9 * nrow * W; i += blockDim.x) {
        const int xw = i % W, rest = i / W;
        const int z = zlo + rest % nrow, bk = rest / nrow;
        float* dst = bk < Q9 ? b0 : b1;
        dst[(bk % Q9) * g.ks + g.idx(xw - 1, 0, z)] = my_pop[(bk * v.slots + (z - row0 + 1)) * W + xw];
    }
    for (int i = threadIdx.x; i < nrow * W; i += blockDim.x) {
        const int xw = i % W, z = zlo + i / W;
        rho_g[g.idx(xw - 1, 0, z)] = my_rho[(z - row0 + 1) * W + xw];
    }
}

size_t march_smem_bytes(int nx, int R) { return (size_t)(2 * Q9 + 1) * (size_t)(R + 2) * (size_t)(nx + 2) * 4; }

// Threads of a CTA: one a node of its band, in whole warps, at most
// kRefClusterThreads.
int march_threads(int nx, int R) {
    const long long n = ((long long)nx * R + 31) / 32 * 32;
    return (int)(n < kRefClusterThreads ? n : kRefClusterThreads);
}

// Whether a cluster of C CTAs with this shared memory can be resident.
bool cluster_fits(int C, int threads, size_t smem) {
    const void* k = (const void*)ref_march_cluster_k<kArithReference>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return false;
    if (C > 8 && cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)C, 1, 1);
    cfg.blockDim = dim3((unsigned)threads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, k, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return clusters >= 1;
}

}  // namespace

// Cluster shape for a march of a D2Q9 domain (nx, nz): as many CTAs (up to
// 16) as keep two rows or more in every CTA's band -- a step's collision is
// issue-bound on an SM, so more SMs shorten it, and two rows keep the
// up/down no-slip phase inside one CTA -- within a CTA's shared memory and
// the device's cluster limits; 0 when the domain does not fit 16 CTAs.
int ref_cluster_shape(int nx, int nz, int* C_out, int* R_out) {
    int dev = 0, smem_max = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
        return 0;
    for (int C = kRefClusterMax; C >= 1; C /= 2) {
        if (C > 1 && nz < 2 * C) continue;
        const int R = (nz + C - 1) / C;
        if ((long long)(C - 1) * R >= nz) continue;   // every CTA owns a row
        if ((long long)R * nx > 4LL * kRefClusterThreads) continue;   // at most 4 nodes a thread
        const size_t smem = march_smem_bytes(nx, R);
        if (smem > (size_t)smem_max) continue;
        if (!cluster_fits(C, march_threads(nx, R), smem)) continue;
        *C_out = C;
        *R_out = R;
        return 1;
    }
    return 0;
}

int ref_march_cluster(int arith, int C, int R, const Geo& g, const CollideParams& cp, const FaceParams& fp,
                      const RefNoslipPlan& plan, float* b0, float* b1, float* rho, const float* u, int cur0,
                      long long nsteps, bool first, bool wb_last, cudaStream_t st) {
    const size_t smem = march_smem_bytes(g.nx, R);
    // no-slip faces only up/down, and the first and last CTA own two rows or
    // more: every no-slip access stays in the wall row's CTA
    bool ud_only = true;
    for (int i = 0; i < plan.ngroups; ++i)
        for (int j = 0; j < plan.len[i]; ++j) ud_only &= plan.faces[i][j] >= 4;
    const int last_rows = g.nz - (C - 1) * R;
    const int local_noslip = (ud_only && R >= 2 && last_rows >= 2) ? 1 : 0;
    const int threads = march_threads(g.nx, R);
    auto launch = [&](auto kernel) -> int {
        cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess && C > 8) e = cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) return (int)e;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)C, 1, 1);
        cfg.blockDim = dim3((unsigned)threads, 1, 1);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = (unsigned)C;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int clusters = 0;
        e = cudaOccupancyMaxActiveClusters(&clusters, kernel, &cfg);
        if (e != cudaSuccess) return (int)e;
        if (clusters < 1) return (int)cudaErrorInvalidConfiguration;
        // steps in chunks that keep one launch well under a second
        long long done = 0;
        int cur = cur0;
        while (done < nsteps) {
            const long long n = nsteps - done < (1 << 20) ? nsteps - done : (1 << 20);
            e = cudaLaunchKernelEx(&cfg, kernel, g, cp, fp, plan, b0, b1, rho, u, cur, (int)n,
                                   (int)(first && done == 0), (int)(wb_last && done + n == nsteps), R,
                                   local_noslip);
            if (e != cudaSuccess) return (int)e;
            cur ^= (int)(n & 1);
            done += n;
        }
        return (int)cudaSuccess;
    };
    if (arith == kArithReference) return launch(ref_march_cluster_k<kArithReference>);
    if (arith == kArithTRT) return launch(ref_march_cluster_k<kArithTRT>);
    return launch(ref_march_cluster_k<kArithFP32>);
}

}  // namespace plb
