// The two-node pair kernel for FP32 and FP32-deviation storage, D2Q9, BGK:
// variants 1-3 of the fused step with FP32 arithmetic, variant 1 with
// plbpd's arithmetic on FP32 storage (native_impl.cuh, launch_fused_pair32),
// in a file of their own so the lattices build in parallel.
#include "native_impl.cuh"

namespace plb {

int nat_fused_pair32_q9(int storage, int arith, bool mask, const Geo& g, const CollideParams& cp, const NativeParams& np,
                        const void* src, void* dst, const uint8_t* types, int variant, cudaStream_t st) {
    if (storage == 3)
        return mask ? launch_fused_pair32<9, 3, true>(g, cp, np, src, dst, types, variant, st)
                    : launch_fused_pair32<9, 3, false>(g, cp, np, src, dst, types, variant, st);
    if (arith == kArithReference)
        return mask ? launch_fused_pair32<9, 0, true, kArithReference>(g, cp, np, src, dst, types, variant, st)
                    : launch_fused_pair32<9, 0, false, kArithReference>(g, cp, np, src, dst, types, variant, st);
    return mask ? launch_fused_pair32<9, 0, true>(g, cp, np, src, dst, types, variant, st)
                : launch_fused_pair32<9, 0, false>(g, cp, np, src, dst, types, variant, st);
}

}  // namespace plb
