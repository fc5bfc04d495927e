// Per-node pieces of plbpd's boundary operators shared by the
// REFERENCE-semantics kernels (kernels_ref.cu: one launch per operator group;
// kernels_ref_cluster.cu: whole marches of small domains in one launch).
// Faces are numbered east, west, north, south, up, down (src/Boundary.cpp:17-18).
#pragma once

#include "engine.h"

namespace plb {
namespace {

__device__ __forceinline__ bool in_face(int f, int x, int y, int z, const Geo& g) {
    switch (f) {
        case 0: return x == g.nx - 1;   // east
        case 1: return x == 0;          // west
        case 2: return y == g.ny - 1;   // north
        case 3: return y == 0;          // south
        case 4: return z == g.nz - 1;   // up
        default: return z == 0;         // down
    }
}

// Within one node of the face plane (the no-slip rule reads rho there).
__device__ __forceinline__ bool near_face(int f, int x, int y, int z, const Geo& g) {
    switch (f) {
        case 0: return x >= g.nx - 2;
        case 1: return x <= 1;
        case 2: return y >= g.ny - 2;
        case 3: return y <= 1;
        case 4: return z >= g.nz - 2;
        default: return z <= 1;
    }
}

// Boundary::reset (src/Boundary.cpp:58-89): u_b on faces with a velocity entry
// (later faces win), rho_solid on no-slip faces.
__device__ __forceinline__ void apply_reset(const FaceParams& fp, int x, int y, int z, const Geo& g,
                                            float& rho, float& ux, float& uy, float& uz) {
#pragma unroll
    for (int f = 0; f < 6; ++f) {
        if (((fp.vel_mask >> f) & 1) && in_face(f, x, y, z, g)) {
            ux = fp.vel[f][0]; uy = fp.vel[f][1]; uz = fp.vel[f][2];
        }
    }
#pragma unroll
    for (int f = 0; f < 6; ++f)
        if (((fp.noslip_mask >> f) & 1) && in_face(f, x, y, z, g)) rho = fp.rho_solid;
}

template <int Q>
__device__ __forceinline__ long long push_offset(int k, const Geo& g) {
    return (long long)Lattice<Q>::cx(k) + (long long)Lattice<Q>::cy(k) * g.ys +
           (long long)Lattice<Q>::cz(k) * g.zs;
}

template <int Q>
__device__ __forceinline__ bool face_contains(int f, int x, int y, int z, const Geo& g) {
    if (x < 0 || x >= g.nx || y < 0 || y >= g.ny || z < 0 || z >= g.nz) return false;
    return in_face(f, x, y, z, g);
}

}  // namespace
}  // namespace plb
