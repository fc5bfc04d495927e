// Initialization, layout conversion between the device layout and plbpd's
// AoS halo layout, and the FP64 conservation reduction.
#include "engine.h"

namespace plb {
namespace {

constexpr int kBlock = 256;

// Domain::initialize (src/Domain.cpp:46-63): every node of the box, halo
// included, gets rho0, u0 and the equilibrium; ntmp starts at zero
// (src/SimData.cpp:53-56).  Under FP16 and FP32 deviation storage the
// buffers hold f - w.
template <int ST>
__global__ void init_uniform_k(Geo g, int q, const float* __restrict__ feq, const float* __restrict__ wk,
                               float rho0, float u0x, float u0y, float u0z, void* __restrict__ n,
                               void* __restrict__ nt, float* __restrict__ rho, float* __restrict__ u) {
    const long long i = (long long)blockIdx.x * kBlock + threadIdx.x;
    if (i >= g.fs) return;
    rho[i] = rho0;
    u[i] = u0x; u[g.ks + i] = u0y; u[2 * g.ks + i] = u0z;
    for (int k = 0; k < q; ++k) {
        if (ST == 0) {
            static_cast<float*>(n)[k * g.ks + i] = feq[k];
            if (nt) static_cast<float*>(nt)[k * g.ks + i] = 0.0f;
        } else if (ST == 1) {
            static_cast<__half*>(n)[k * g.ks + i] = __float2half_rn(__fmul_rn(__fsub_rn(feq[k], wk[k]), kHalfScale));
            if (nt) static_cast<__half*>(nt)[k * g.ks + i] = __float2half_rn(__fmul_rn(-wk[k], kHalfScale));
        } else if (ST == 3) {
            static_cast<float*>(n)[k * g.ks + i] = __fsub_rn(feq[k], wk[k]);
            if (nt) static_cast<float*>(nt)[k * g.ks + i] = -wk[k];
        } else {
            static_cast<double*>(n)[k * g.ks + i] = (double)feq[k];
            if (nt) static_cast<double*>(nt)[k * g.ks + i] = 0.0;
        }
    }
}

// Device (SoA, pitched) -> plbpd layout (AoS, one halo layer on every axis).
// One thread per node of the plbpd box; nodes the device does not hold
// (halo under NATIVE semantics) are written as 0.
template <int ST>
__global__ void export_k(Geo g, int v, const void* __restrict__ src, const float* __restrict__ wk,
                         float* __restrict__ aos) {
    const long long X = g.nx + 2, Y = g.ny + 2, Z = g.nz + 2;
    const long long i = (long long)blockIdx.x * kBlock + threadIdx.x;
    if (i >= X * Y * Z) return;
    const int x = (int)(i % X) - 1;
    const int y = (int)((i / X) % Y) - 1;
    const int z = (int)(i / (X * Y)) - 1;
    const bool held = x >= -g.h && x < g.nx + g.h && y >= -g.h && y < g.ny + g.h && z >= -g.h && z < g.nz + g.h;
    const long long node = held ? g.idx(x, y, z) : 0;
    for (int c = 0; c < v; ++c) {
        float val = 0.0f;
        if (held) {
            if (ST == 0) val = static_cast<const float*>(src)[c * g.ks + node];
            else if (ST == 1)
                val = __fadd_rn(__fmul_rn(__half2float(static_cast<const __half*>(src)[c * g.ks + node]), kHalfUnscale),
                                wk[c]);
            else if (ST == 3) val = __fadd_rn(static_cast<const float*>(src)[c * g.ks + node], wk[c]);
            else val = __double2float_rn(static_cast<const double*>(src)[c * g.ks + node]);
        }
        aos[i * v + c] = val;
    }
}

template <int ST>
__global__ void import_k(Geo g, int v, const float* __restrict__ aos, const float* __restrict__ wk,
                         void* __restrict__ dst) {
    const long long X = g.nx + 2, Y = g.ny + 2, Z = g.nz + 2;
    const long long i = (long long)blockIdx.x * kBlock + threadIdx.x;
    if (i >= X * Y * Z) return;
    const int x = (int)(i % X) - 1;
    const int y = (int)((i / X) % Y) - 1;
    const int z = (int)(i / (X * Y)) - 1;
    if (!(x >= -g.h && x < g.nx + g.h && y >= -g.h && y < g.ny + g.h && z >= -g.h && z < g.nz + g.h)) return;
    const long long node = g.idx(x, y, z);
    for (int c = 0; c < v; ++c) {
        const float val = aos[i * v + c];
        if (ST == 0) static_cast<float*>(dst)[c * g.ks + node] = val;
        else if (ST == 1)
            static_cast<__half*>(dst)[c * g.ks + node] = __float2half_rn(__fmul_rn(__fsub_rn(val, wk[c]), kHalfScale));
        else if (ST == 3) static_cast<float*>(dst)[c * g.ks + node] = __fsub_rn(val, wk[c]);
        else static_cast<double*>(dst)[c * g.ks + node] = (double)val;
    }
}

// FP64 sums over fluid nodes.  Fluid: not solid (NATIVE, `types` given) or
// not on a no-slip face (REFERENCE).  Block partials are written to
// `partials`; a second one-block kernel adds them in a fixed order, so the
// result does not depend on scheduling.
constexpr int kRedBlocks = 1024;

template <int Q, int ST>
__global__ void __launch_bounds__(kBlock)
conservation_k(Geo g, const void* __restrict__ n, const uint8_t* __restrict__ types, int noslip_mask,
               double* __restrict__ partials) {
    double m = 0.0, px = 0.0, py = 0.0, pz = 0.0;
    const long long total = g.cells();
    for (long long c = (long long)blockIdx.x * kBlock + threadIdx.x; c < total; c += (long long)gridDim.x * kBlock) {
        const int x = (int)(c % g.nx);
        const int y = (int)((c / g.nx) % g.ny);
        const int z = (int)(c / ((long long)g.nx * g.ny));
        const long long node = g.idx(x, y, z);
        if (types) {
            if (types[node] & kSolid) continue;
        } else {
            const bool in[6] = {x == g.nx - 1, x == 0, y == g.ny - 1, y == 0, z == g.nz - 1, z == 0};
            bool wall = false;
            for (int f = 0; f < 6; ++f) wall |= ((noslip_mask >> f) & 1) && in[f];
            if (wall) continue;
        }
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            double v;
            if (ST == 0) v = (double)static_cast<const float*>(n)[k * g.ks + node];
            else if (ST == 1)
                v = (double)__fmul_rn(__half2float(static_cast<const __half*>(n)[k * g.ks + node]), kHalfUnscale) +
                    (double)weight<Q>(k);
            else if (ST == 3) v = (double)static_cast<const float*>(n)[k * g.ks + node] + (double)weight<Q>(k);
            else v = static_cast<const double*>(n)[k * g.ks + node];
            m += v;
            if (Lattice<Q>::cx(k)) px += Lattice<Q>::cx(k) * v;
            if (Lattice<Q>::cy(k)) py += Lattice<Q>::cy(k) * v;
            if (Lattice<Q>::cz(k)) pz += Lattice<Q>::cz(k) * v;
        }
    }
    __shared__ double sh[4][kBlock / 32];
    double vals[4] = {m, px, py, pz};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        double v = vals[j];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) sh[j][threadIdx.x >> 5] = v;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double s = 0.0;
        for (int w = 0; w < kBlock / 32; ++w) s += sh[threadIdx.x][w];
        partials[blockIdx.x * 4 + threadIdx.x] = s;
    }
}

__global__ void finish_sum_k(const double* __restrict__ partials, int nblocks, double* __restrict__ out4) {
    __shared__ double sh[4][kBlock / 32];
    double vals[4] = {0.0, 0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < nblocks; b += kBlock)
        for (int j = 0; j < 4; ++j) vals[j] += partials[b * 4 + j];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        double v = vals[j];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) sh[j][threadIdx.x >> 5] = v;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double s = 0.0;
        for (int w = 0; w < kBlock / 32; ++w) s += sh[threadIdx.x][w];
        out4[threadIdx.x] = s;
    }
}

unsigned blocks_for(long long n) { return (unsigned)((n + kBlock - 1) / kBlock); }

}  // namespace

int util_init_uniform(int q, int storage, const Geo& g, const float* feq_dev, float rho0, const float* u0,
                      void* n, void* nt, float* rho, float* u, cudaStream_t st) {
    // feq_dev holds 2*q floats: the equilibrium, then the weights
    const float* wk = feq_dev + q;
    if (storage == 0)
        init_uniform_k<0><<<blocks_for(g.fs), kBlock, 0, st>>>(g, q, feq_dev, wk, rho0, u0[0], u0[1], u0[2], n, nt, rho, u);
    else if (storage == 1)
        init_uniform_k<1><<<blocks_for(g.fs), kBlock, 0, st>>>(g, q, feq_dev, wk, rho0, u0[0], u0[1], u0[2], n, nt, rho, u);
    else if (storage == 3)
        init_uniform_k<3><<<blocks_for(g.fs), kBlock, 0, st>>>(g, q, feq_dev, wk, rho0, u0[0], u0[1], u0[2], n, nt, rho, u);
    else
        init_uniform_k<2><<<blocks_for(g.fs), kBlock, 0, st>>>(g, q, feq_dev, wk, rho0, u0[0], u0[1], u0[2], n, nt, rho, u);
    return (int)cudaGetLastError();
}

int util_export(int storage, int v, const Geo& g, const void* src, const float* wk, float* aos, cudaStream_t st) {
    const long long cells = (long long)(g.nx + 2) * (g.ny + 2) * (g.nz + 2);
    if (storage == 0) export_k<0><<<blocks_for(cells), kBlock, 0, st>>>(g, v, src, wk, aos);
    else if (storage == 1) export_k<1><<<blocks_for(cells), kBlock, 0, st>>>(g, v, src, wk, aos);
    else if (storage == 3) export_k<3><<<blocks_for(cells), kBlock, 0, st>>>(g, v, src, wk, aos);
    else export_k<2><<<blocks_for(cells), kBlock, 0, st>>>(g, v, src, wk, aos);
    return (int)cudaGetLastError();
}

int util_import(int storage, int v, const Geo& g, const float* aos, const float* wk, void* dst, cudaStream_t st) {
    const long long cells = (long long)(g.nx + 2) * (g.ny + 2) * (g.nz + 2);
    if (storage == 0) import_k<0><<<blocks_for(cells), kBlock, 0, st>>>(g, v, aos, wk, dst);
    else if (storage == 1) import_k<1><<<blocks_for(cells), kBlock, 0, st>>>(g, v, aos, wk, dst);
    else if (storage == 3) import_k<3><<<blocks_for(cells), kBlock, 0, st>>>(g, v, aos, wk, dst);
    else import_k<2><<<blocks_for(cells), kBlock, 0, st>>>(g, v, aos, wk, dst);
    return (int)cudaGetLastError();
}

int util_conservation_partials() { return kRedBlocks * 4; }

int util_conservation(int q, int storage, const Geo& g, const void* n, const uint8_t* types, int noslip_mask,
                      double* partials, double* out4, cudaStream_t st) {
    const long long cells = g.cells();
    int nb = (int)blocks_for(cells);
    if (nb > kRedBlocks) nb = kRedBlocks;
    if (nb < 1) nb = 1;
#define CALL(Q) (storage == 0 ? (conservation_k<Q, 0><<<nb, kBlock, 0, st>>>(g, n, types, noslip_mask, partials), 0) \
             : storage == 1 ? (conservation_k<Q, 1><<<nb, kBlock, 0, st>>>(g, n, types, noslip_mask, partials), 0) \
             : storage == 3 ? (conservation_k<Q, 3><<<nb, kBlock, 0, st>>>(g, n, types, noslip_mask, partials), 0) \
                            : (conservation_k<Q, 2><<<nb, kBlock, 0, st>>>(g, n, types, noslip_mask, partials), 0))
    if (q == 9) CALL(9);
    else if (q == 19) CALL(19);
    else if (q == 27) CALL(27);
    else return (int)cudaErrorInvalidValue;
#undef CALL
    finish_sum_k<<<1, kBlock, 0, st>>>(partials, nb, out4);
    return (int)cudaGetLastError();
}

}  // namespace plb
