// plb_conservation_static: the FP64 mass/momentum reduction for callers that
// cannot allocate device memory.
//
// Who needs it: code that owns every byte of device memory up front and may
// not call cudaMalloc once it is running -- a solver embedded in a host
// application with its own memory pool, a process under a hard device-memory
// quota, a caller whose allocator must not see foreign allocations.  For them
// plb_conservation is unusable (its solve handle allocates a block-partials
// buffer), so this entry point works on the caller's own device arrays and
// keeps its block partials in a fixed array that is part of the library image.
//
// The scratch array is a file-scope __device__ variable: every GPU that loads
// the library holds its 128 KiB until the process exits.  Host code must not
// pass the symbol itself to a kernel (on the host it names a host-side shadow,
// not device memory); the device address is looked up once per device with
// cudaGetSymbolAddress, with that device current, on the first call made on
// it.  That first call should therefore come before any stream capture.
//
// Every call shares the one array and it keeps whatever the last call left in
// it.  Each block writes its own partial before the final kernel reads it, so
// nothing has to start at zero; but two calls whose kernels overlap on the GPU
// (different streams, or different host threads without ordering) race on the
// array and may return wrong sums.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/plb.h"
#include "engine.h"
#include "lattice.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kCellsPerThread = 16;
constexpr long long kCellsPerBlock = (long long)kThreads * kCellsPerThread;   // 4096
constexpr int kMaxBlocks = 4096;                                                // 4096 x 4 doubles = 128 KiB
constexpr int kMaxDevices = 64;

// block partials: mass, momentum x, y, z per block
static __device__ __align__(256) double g_static_partials[kMaxBlocks * 4];

double* g_partials_addr[kMaxDevices] = {};
std::mutex g_setup_mutex;

template <int Q>
__global__ void __launch_bounds__(kThreads)
flat_sums_k(const float* __restrict__ n, long long ncells, long long plane, const uint8_t* __restrict__ solid,
            double* __restrict__ partials) {
    double m = 0.0, px = 0.0, py = 0.0, pz = 0.0;
    const long long base = (long long)blockIdx.x * kCellsPerBlock;
    for (int j = 0; j < kCellsPerThread; ++j) {
        const long long i = base + (long long)j * kThreads + threadIdx.x;
        if (i >= ncells) break;
        if (solid && solid[i]) continue;
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            const double v = (double)n[(long long)k * plane + i];
            m += v;
            if (plb::Lattice<Q>::cx(k)) px += plb::Lattice<Q>::cx(k) * v;
            if (plb::Lattice<Q>::cy(k)) py += plb::Lattice<Q>::cy(k) * v;
            if (plb::Lattice<Q>::cz(k)) pz += plb::Lattice<Q>::cz(k) * v;
        }
    }
    __shared__ double sh[4][kThreads / 32];
    double vals[4] = {m, px, py, pz};
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        double v = vals[c];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) sh[c][threadIdx.x >> 5] = v;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double s = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) s += sh[threadIdx.x][w];
        partials[blockIdx.x * 4 + threadIdx.x] = s;
    }
}

__global__ void __launch_bounds__(kThreads)
flat_finish_k(const double* __restrict__ partials, int nblocks, double* __restrict__ out4) {
    __shared__ double sh[4][kThreads / 32];
    double vals[4] = {0.0, 0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < nblocks; b += kThreads)
        for (int c = 0; c < 4; ++c) vals[c] += partials[b * 4 + c];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        double v = vals[c];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) sh[c][threadIdx.x >> 5] = v;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double s = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) s += sh[threadIdx.x][w];
        out4[threadIdx.x] = s;
    }
}

// messages go to the same per-thread slot plb_last_error() reads
int fail(int code, const std::string& msg) {
    plb::record_error(msg);
    return code;
}

// Device address of the scratch array on the current device, looked up once.
int partials_on_current_device(double** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(PLB_ECUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(PLB_EUNSUPPORTED, "device ordinal beyond 63");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_partials_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_static_partials);
        if (e != cudaSuccess || !p)
            return fail(PLB_ECUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        g_partials_addr[dev] = static_cast<double*>(p);
    }
    *out = g_partials_addr[dev];
    return PLB_OK;
}

}  // namespace

extern "C" int plb_conservation_static(int32_t q, const float* n, int64_t ncells, int64_t plane_stride,
                                       const uint8_t* solid, double* out4, void* stream) {
    if (q != 9 && q != 19 && q != 27) return fail(PLB_EINVAL, "q must be 9, 19 or 27");
    if (!n || !out4) return fail(PLB_EINVAL, "populations and output must be device pointers, not null");
    if (ncells < 1) return fail(PLB_EINVAL, "ncells must be at least 1");
    if (plane_stride < ncells) return fail(PLB_EINVAL, "plane_stride must be at least ncells");
    if (ncells > (int64_t)kMaxBlocks * kCellsPerBlock)
        return fail(PLB_EINVAL, "ncells " + std::to_string(ncells) + " exceeds the static scratch limit of " +
                                    std::to_string((long long)kMaxBlocks * kCellsPerBlock) + " cells");
    double* partials = nullptr;
    const int rc = partials_on_current_device(&partials);
    if (rc != PLB_OK) return rc;
    const int nb = (int)((ncells + kCellsPerBlock - 1) / kCellsPerBlock);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (q == 9) flat_sums_k<9><<<nb, kThreads, 0, st>>>(n, ncells, plane_stride, solid, partials);
    else if (q == 19) flat_sums_k<19><<<nb, kThreads, 0, st>>>(n, ncells, plane_stride, solid, partials);
    else flat_sums_k<27><<<nb, kThreads, 0, st>>>(n, ncells, plane_stride, solid, partials);
    flat_finish_k<<<1, kThreads, 0, st>>>(partials, nb, out4);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(PLB_ECUDA, std::string("plb_conservation_static launch: ") + cudaGetErrorString(e));
    return PLB_OK;
}
