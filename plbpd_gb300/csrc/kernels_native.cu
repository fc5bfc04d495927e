// Kernels for NATIVE semantics: one fused pull kernel per time step (BGK
// instantiations; the TRT ones are in kernels_trt.cu).
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
//   3  FP32 deviations d_k = f_k - w_k with storage 1's arithmetic
#include "native_impl.cuh"

namespace plb {
namespace {

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
                 uint32_t* __restrict__ links, int esize) {
    const int x = blockIdx.x * kBlockX + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= g.nx) return;
    const long long node = g.idx(x, y, z);
    const uint8_t t = types[node];
    out[node] = t;
    links[node] = 0u;
    if (t & kSolid) {
        // rows start on a 32-byte boundary (the row pitch is a whole number of
        // sectors), so the sector of x is the run of 32 / esize nodes holding it
        const int S = 32 / esize, x0 = x - x % S, x1 = min(x0 + S, g.nx);
        for (int xx = x0; xx < x1; ++xx)
            if (!(types[node - x + xx] & kSolid)) {
                out[node] = t | kSectorMate;
                break;
            }
        return;
    }
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

}  // namespace

int nat_fused_step(int q, int storage, int arith, bool has_mask, const Geo& g, const CollideParams& cp,
                   const NativeParams& np, const void* src, void* dst, const uint8_t* types, int variant,
                   cudaStream_t st) {
    if (arith == kArithTRT) return nat_fused_step_trt(q, storage, has_mask, g, cp, np, src, dst, types, st);
#define CALL(Q) fused_q<false, Q>(storage, arith, has_mask, g, cp, np, src, dst, types, variant, st)
    return PLB_Q_DISPATCH(q, CALL);
#undef CALL
}

int nat_fused_variants(int q, int storage, int arith, bool moving, const Geo& g) {
    if (g.nx % 2 != 0) return 1;
    if (storage == 1) return nat_h2_variant_count(q, arith, moving);
    if ((storage == 3 && arith != kArithTRT) || (storage == 0 && arith == kArithFP32)) return moving ? 1 : kPair32Variants;
    if (storage == 0 && arith == kArithReference) return moving ? 1 : kPairRefVariants;
    return 1;
}

int nat_collide_raw(int q, int storage, int arith, bool has_mask, const Geo& g, const CollideParams& cp,
                    const NativeParams& np, const void* src, void* dst, const float* rho, const float* u,
                    const uint8_t* types, cudaStream_t st) {
    if (arith == kArithTRT) return nat_collide_raw_trt(q, storage, has_mask, g, cp, np, src, dst, rho, u, types, st);
#define CALL(Q) raw_q<false, Q>(storage, arith, has_mask, g, cp, np, src, dst, rho, u, types, st)
    return PLB_Q_DISPATCH(q, CALL);
#undef CALL
}

namespace {
template <int Q>
int gather_q(int storage, bool m, const Geo& g, const NativeParams& np, const void* src, void* n_out, float* rho,
             float* u, const uint8_t* types, cudaStream_t st) {
    if (storage == 1)
        return m ? launch_gather<Q, 1, true>(g, np, src, n_out, rho, u, types, st)
                 : launch_gather<Q, 1, false>(g, np, src, n_out, rho, u, types, st);
    if (storage == 2)
        return m ? launch_gather<Q, 2, true>(g, np, src, n_out, rho, u, types, st)
                 : launch_gather<Q, 2, false>(g, np, src, n_out, rho, u, types, st);
    if (storage == 3)
        return m ? launch_gather<Q, 3, true>(g, np, src, n_out, rho, u, types, st)
                 : launch_gather<Q, 3, false>(g, np, src, n_out, rho, u, types, st);
    return m ? launch_gather<Q, 0, true>(g, np, src, n_out, rho, u, types, st)
             : launch_gather<Q, 0, false>(g, np, src, n_out, rho, u, types, st);
}
}  // namespace

int nat_gather(int q, int storage, bool has_mask, const Geo& g, const NativeParams& np, const void* src,
               void* n_out, float* rho, float* u, const uint8_t* types, cudaStream_t st) {
#define CALL(Q) gather_q<Q>(storage, has_mask, g, np, src, n_out, rho, u, types, st)
    return PLB_Q_DISPATCH(q, CALL);
#undef CALL
}

int nat_aa_step(int kind, int q, int storage, int arith, bool has_mask, const Geo& g, const CollideParams& cp,
                const NativeParams& np, void* A, const float* rho, const float* u, const uint8_t* types,
                cudaStream_t st) {
    if (arith == kArithTRT) return nat_aa_step_trt(kind, q, storage, has_mask, g, cp, np, A, rho, u, types, st);
#define CALL(Q) aa_q<false, Q>(kind, storage, arith, has_mask, g, cp, np, A, rho, u, types, st)
    return PLB_Q_DISPATCH(q, CALL);
#undef CALL
}

namespace {
template <int Q, int ST>
int aa_gather_st(bool m, bool swapped, const Geo& g, const NativeParams& np, const void* A, void* n_out, float* rho,
                 float* u, const uint8_t* types, cudaStream_t st) {
    using T = typename Store<ST>::T;
    auto go = [&](auto mc, auto sc) {
        nat_aa_gather_k<Q, ST, decltype(mc)::value, decltype(sc)::value><<<cell_grid(g), kBlockX, 0, st>>>(
            g, np, (const T*)A, (T*)n_out, rho, u, types);
        return (int)cudaGetLastError();
    };
    if (m) return swapped ? go(std::true_type{}, std::true_type{}) : go(std::true_type{}, std::false_type{});
    return swapped ? go(std::false_type{}, std::true_type{}) : go(std::false_type{}, std::false_type{});
}

template <int Q>
int aa_gather_q(int storage, bool m, bool swapped, const Geo& g, const NativeParams& np, const void* A, void* n_out,
                float* rho, float* u, const uint8_t* types, cudaStream_t st) {
    switch (storage) {
        case 1: return aa_gather_st<Q, 1>(m, swapped, g, np, A, n_out, rho, u, types, st);
        case 2: return aa_gather_st<Q, 2>(m, swapped, g, np, A, n_out, rho, u, types, st);
        case 3: return aa_gather_st<Q, 3>(m, swapped, g, np, A, n_out, rho, u, types, st);
        default: return aa_gather_st<Q, 0>(m, swapped, g, np, A, n_out, rho, u, types, st);
    }
}
}  // namespace

int nat_aa_gather(int q, int storage, bool has_mask, bool swapped, const Geo& g, const NativeParams& np,
                  const void* A, void* n_out, float* rho, float* u, const uint8_t* types, cudaStream_t st) {
#define CALL(Q) aa_gather_q<Q>(storage, has_mask, swapped, g, np, A, n_out, rho, u, types, st)
    return PLB_Q_DISPATCH(q, CALL);
#undef CALL
}

int nat_batch_blocks_per_sm(int q, int storage, int arith, bool moving, int kind) {
    if (arith == kArithTRT) return nat_batch_blocks_per_sm_trt(q, storage, moving, kind);
    return batch_blocks_per_sm<false>(q, storage, arith, moving, kind);
}

int nat_batch_step(int q, int storage, int arith, bool moving, const BatchDomain* doms, const int4* tiles,
                   int ntiles, int npair, int parity, int blocks_pair, int blocks_single, cudaStream_t st) {
    if (arith == kArithTRT)
        return nat_batch_step_trt(q, storage, moving, doms, tiles, ntiles, npair, parity, blocks_pair, blocks_single,
                                  st);
    return batch_step<false>(q, storage, arith, moving, doms, tiles, ntiles, npair, parity, blocks_pair,
                             blocks_single, st);
}

int nat_batch_step_multi(int q, int storage, int arith, bool moving, bool pairs, const BatchDomain* doms,
                         const int4* tiles, int ntiles, int parity, int nsteps, int blocks, BatchSync* bs,
                         cudaStream_t st) {
    if (arith == kArithTRT)
        return nat_batch_step_multi_trt(q, storage, moving, pairs, doms, tiles, ntiles, parity, nsteps, blocks, bs, st);
    return batch_step_multi<false>(q, storage, arith, moving, pairs, doms, tiles, ntiles, parity, nsteps, blocks, bs,
                                   st);
}

int nat_reset_fields(const Geo& g, const NativeParams& np, const uint8_t* types, float* rho, float* u,
                     cudaStream_t st) {
    nat_reset_fields_k<<<cell_grid(g), kBlockX, 0, st>>>(g, np, types, rho, u);
    return (int)cudaGetLastError();
}

int nat_build_types(int q, const Geo& g, const uint8_t* mask, int noslip_mask, int esize, uint8_t* scratch,
                    uint8_t* types, uint32_t* links, cudaStream_t st) {
#define CALL(Q) (nat_types_solid_k<Q><<<cell_grid(g), kBlockX, 0, st>>>(g, mask, noslip_mask, scratch), \
                 nat_types_near_k<Q><<<cell_grid(g), kBlockX, 0, st>>>(g, scratch, types, links, esize), \
                 (int)cudaGetLastError())
    return PLB_Q_DISPATCH(q, CALL);
#undef CALL
}

}  // namespace plb
