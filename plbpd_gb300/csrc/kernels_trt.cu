// TRT instantiations of the NATIVE-semantics kernels (native_impl.cuh),
// compiled apart from the BGK ones so the two build in parallel.
#include "native_impl.cuh"

namespace plb {

int nat_fused_step_trt(int q, int storage, bool has_mask, const Geo& g, const CollideParams& cp,
                       const NativeParams& np, const void* src, void* dst, const uint8_t* types, cudaStream_t st) {
#define CALL(Q) fused_q<true, Q>(storage, kArithTRT, has_mask, g, cp, np, src, dst, types, 0, st)
    return PLB_Q_DISPATCH(q, CALL);
#undef CALL
}

int nat_collide_raw_trt(int q, int storage, bool has_mask, const Geo& g, const CollideParams& cp,
                        const NativeParams& np, const void* src, void* dst, const float* rho, const float* u,
                        const uint8_t* types, cudaStream_t st) {
#define CALL(Q) raw_q<true, Q>(storage, kArithTRT, has_mask, g, cp, np, src, dst, rho, u, types, st)
    return PLB_Q_DISPATCH(q, CALL);
#undef CALL
}

int nat_aa_step_trt(int kind, int q, int storage, bool has_mask, const Geo& g, const CollideParams& cp,
                    const NativeParams& np, void* A, const float* rho, const float* u, const uint8_t* types,
                    cudaStream_t st) {
#define CALL(Q) aa_q<true, Q>(kind, storage, kArithTRT, has_mask, g, cp, np, A, rho, u, types, st)
    return PLB_Q_DISPATCH(q, CALL);
#undef CALL
}

int nat_batch_blocks_per_sm_trt(int q, int storage, bool moving, int kind) {
    return batch_blocks_per_sm<true>(q, storage, kArithTRT, moving, kind);
}

int nat_batch_step_trt(int q, int storage, bool moving, const BatchDomain* doms, const int4* tiles, int ntiles,
                       int npair, int parity, int blocks_pair, int blocks_single, cudaStream_t st) {
    return batch_step<true>(q, storage, kArithTRT, moving, doms, tiles, ntiles, npair, parity, blocks_pair,
                            blocks_single, st);
}

int nat_batch_step_multi_trt(int q, int storage, bool moving, bool pairs, const BatchDomain* doms,
                             const int4* tiles, int ntiles, int parity, int nsteps, int blocks, BatchSync* bs,
                             cudaStream_t st) {
    return batch_step_multi<true>(q, storage, kArithTRT, moving, pairs, doms, tiles, ntiles, parity, nsteps, blocks,
                                  bs, st);
}

}  // namespace plb
