// BGK instantiations of the FP16 pair kernel for D3Q19, every compiled variant
// (native_impl.cuh, kH2Variant), in a file of their own so the lattices
// build in parallel.
#include "native_impl.cuh"

namespace plb {

int nat_fused_h2_bgk19(bool mask, const Geo& g, const CollideParams& cp, const NativeParams& np, const void* src,
                       void* dst, const uint8_t* types, int variant, cudaStream_t st) {
    return mask ? launch_fused_h2<19, kArithFP32, true>(g, cp, np, src, dst, types, variant, st)
                : launch_fused_h2<19, kArithFP32, false>(g, cp, np, src, dst, types, variant, st);
}

}  // namespace plb
