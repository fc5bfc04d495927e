// Internal interface between the C ABI (capi.cu) and the kernel files.
#pragma once

#include <cstdint>
#include <string>
#include <cuda_runtime.h>

#include "lattice.cuh"

struct plb_params;
struct plb_solve;
struct plb_batch;

namespace plb {

// Stores the message plb_last_error() returns on this thread.
void record_error(const std::string& msg);

// plb_solve_create's checks of a parameter block: PLB_OK, or an error code
// with the message recorded.
int check_params(const plb_params* p);

// Moves a solve's / a batch's work onto a new stream of CUDA priority
// `priority` (after the old stream's work); the solve server ranks its lanes.
int set_solve_priority(plb_solve* s, int priority);
int set_batch_priority(plb_batch* b, int priority);
// Runs a batch's calls as multi-step cooperative launches (or one launch a
// step): the solve server's lanes, whose membership changes every few
// ticks, take one launch a tick instead of capturing a new graph.
int set_batch_multi(plb_batch* b, bool multi);
// rho and u of a solve in plbpd's layout (host memory), with one gather and
// one wait for both (the solve server's retirement).
int read_moments(plb_solve* s, float* rho, float* u);

// Boundary description handed to the REFERENCE-semantics kernels.  Faces are
// numbered east, west, north, south, up, down (plbpd's src/Boundary.cpp:17-18).
struct FaceParams {
    int noslip_mask;      // bit f: face f is a no-slip wall
    int vel_mask;         // bit f: face f has a velocity entry
    float vel[6][3];      // u_b per face
    float rho_solid;
    float cs2inv;         // 1.0f / c_s^2 (src/Boundary.cpp:27)
    int ew_periodic, ns_periodic;
};

// Node types under NATIVE semantics (one byte per interior node).
//   bit 7: solid; bits 0-2 then index the solid's wall velocity (0..5 = face,
//          6 = obstacle, zero velocity)
//   bit 6: fluid node with at least one solid neighbour
enum : uint8_t { kSolid = 0x80, kNearSolid = 0x40, kVelMask = 0x07, kObstacleVel = 6 };
// A solid node whose 32-byte sector of its row (in the population storage)
// also holds a fluid node: the fused kernels store into its slots (values
// that no fluid node reads) so that the sector is written whole.  A partly
// written sector makes the memory system read the sector from DRAM before
// it writes it back.
enum : uint8_t { kSectorMate = 0x20 };

struct NativeParams {
    float vel[8][3];      // solid velocities by index (6 = obstacle = 0)
    float rho_solid;
    float cs2inv;
    int moving;           // some wall velocity is nonzero
    const uint32_t* links;  // per node: bit k set when x + c_k is solid
};

// ---- REFERENCE semantics (kernels_ref.cu) ----------------------------------
// One fused step: moments (or the rho/u fields when `first`), resets, collision
// and push into `nxt`; boundary-layer nodes also write their collided values
// back into `cur` (every node when `wb_all`).  Returns a cudaError_t.
int ref_fused_step(int q, int arith, bool first, bool wb_all, const Geo& g, const CollideParams& cp,
                   const FaceParams& fp, float* cur, float* nxt, float* rho, float* u,
                   cudaStream_t st);
// No-slip for the faces in face_list[0..nfaces) in one launch (faces must not
// interact; the host groups them).
int ref_noslip(int q, const Geo& g, const FaceParams& fp, const int* face_list, int nfaces,
               float* n, const float* rho, cudaStream_t st);
// East/west then north/south halo copies, as one launch.
int ref_periodic(int q, const Geo& g, const FaceParams& fp, float* n, cudaStream_t st);

// ---- REFERENCE semantics, whole marches in one launch (kernels_ref_cluster.cu)
// The no-slip faces in launch groups, in plbpd's order (faces of a group
// touch disjoint slots).
struct RefNoslipPlan {
    int ngroups;
    int faces[6][2];
    int len[6];
};
constexpr int kRefClusterMax = 16;        // CTAs of a cluster (above 8: non-portable size)
constexpr int kRefClusterThreads = 1024;  // threads of a CTA
// Cluster shape (CTAs, interior rows a CTA) for a D2Q9 domain of nx x nz
// nodes held in distributed shared memory; 0 when it does not fit.
int ref_cluster_shape(int nx, int nz, int* C, int* R);
// n steps of plbpd's march on a D2Q9 domain (ny = 1, no north/south no-slip
// face) in one launch per 2^20 steps: the first step takes rho/u from the
// fields when `first`, the last writes every node back when `wb_last`, as
// ref_fused_step does.  b0/b1 are the two population buffers, cur0 the one
// holding n.  Returns a cudaError_t.
int ref_march_cluster(int arith, int C, int R, const Geo& g, const CollideParams& cp, const FaceParams& fp,
                      const RefNoslipPlan& plan, float* b0, float* b1, float* rho, const float* u, int cur0,
                      long long nsteps, bool first, bool wb_last, cudaStream_t st);
// Unfused operators.
int ref_collide(int q, int arith, const Geo& g, const CollideParams& cp, float* n,
                const float* rho, const float* u, cudaStream_t st);
int ref_push(int q, const Geo& g, const float* n, float* nt, cudaStream_t st);
int ref_moments(int q, const Geo& g, const float* n, float* rho, float* u, cudaStream_t st);
int ref_reset(const Geo& g, const FaceParams& fp, bool velocity, bool density, float* rho,
              float* u, cudaStream_t st);

// ---- NATIVE semantics (kernels_native.cu; TRT in kernels_trt.cu) -----------
// storage: 0 = FP32, 1 = FP16 deviations f - w, 2 = FP64.  arith: kArith*;
// kArithTRT selects the two-relaxation-time operator for any storage.
// Collision of a RAW state (n in `src`, rho/u fields), result P into `dst`.
int nat_collide_raw(int q, int storage, int arith, bool has_mask, const Geo& g,
                    const CollideParams& cp, const NativeParams& np, const void* src, void* dst,
                    const float* rho, const float* u, const uint8_t* types, cudaStream_t st);
// One fused step: gather P from `src` (streaming + bounce-back), moments,
// collision, store P into `dst`.  `variant` picks among the FP16 pair
// kernel's compiled variants (all give the same bits); other kernels have one.
int nat_fused_step(int q, int storage, int arith, bool has_mask, const Geo& g,
                   const CollideParams& cp, const NativeParams& np, const void* src, void* dst,
                   const uint8_t* types, int variant, cudaStream_t st);
// How many variants nat_fused_step has for a configuration (1 unless FP16
// storage with even nx takes the pair kernel).
int nat_fused_variants(int q, int storage, int arith, bool moving, const Geo& g);
// The most variants any configuration has.
constexpr int kFusedVariants = 7;
// The BGK pair-kernel step of one lattice (kernels_h2_q<Q>.cu: one file per
// lattice, so their variants compile in parallel).
int nat_fused_h2_bgk9(bool mask, const Geo& g, const CollideParams& cp, const NativeParams& np, const void* src,
                      void* dst, const uint8_t* types, int variant, cudaStream_t st);
int nat_fused_h2_bgk19(bool mask, const Geo& g, const CollideParams& cp, const NativeParams& np, const void* src,
                       void* dst, const uint8_t* types, int variant, cudaStream_t st);
int nat_fused_h2_bgk27(bool mask, const Geo& g, const CollideParams& cp, const NativeParams& np, const void* src,
                       void* dst, const uint8_t* types, int variant, cudaStream_t st);
// The FP32 / FP32-deviation pair kernel (storage 0 with FP32 or plbpd's
// arithmetic, or 3) of one lattice: variants 1-3 of nat_fused_step with FP32
// arithmetic, variant 1 with plbpd's (kernels_pair32_q<Q>.cu).
int nat_fused_pair32_q9(int storage, int arith, bool mask, const Geo& g, const CollideParams& cp,
                        const NativeParams& np, const void* src, void* dst, const uint8_t* types, int variant,
                        cudaStream_t st);
int nat_fused_pair32_q19(int storage, int arith, bool mask, const Geo& g, const CollideParams& cp,
                         const NativeParams& np, const void* src, void* dst, const uint8_t* types, int variant,
                         cudaStream_t st);
int nat_fused_pair32_q27(int storage, int arith, bool mask, const Geo& g, const CollideParams& cp,
                         const NativeParams& np, const void* src, void* dst, const uint8_t* types, int variant,
                         cudaStream_t st);
// Gather only: writes n (storage format, or nullptr) and the moments with the
// solid-node resets (rho/u, or nullptr).
int nat_gather(int q, int storage, bool has_mask, const Geo& g, const NativeParams& np,
               const void* src, void* n_out, float* rho, float* u, const uint8_t* types,
               cudaStream_t st);
// AA in-place streaming on one buffer A: kind 0 = even step from a RAW state
// (collides with the rho/u fields), 1 = even step, 2 = odd step.
int nat_aa_step(int kind, int q, int storage, int arith, bool has_mask, const Geo& g, const CollideParams& cp,
                const NativeParams& np, void* A, const float* rho, const float* u, const uint8_t* types,
                cudaStream_t st);
// Natural n (storage format, into n_out, or nullptr) and the moments with the
// solid-node resets (rho/u, or nullptr) of an AA buffer; `swapped`: A holds
// the layout an even step leaves.
int nat_aa_gather(int q, int storage, bool has_mask, bool swapped, const Geo& g, const NativeParams& np,
                  const void* A, void* n_out, float* rho, float* u, const uint8_t* types, cudaStream_t st);
// Solid nodes' fields = (rho_solid, wall velocity).
int nat_reset_fields(const Geo& g, const NativeParams& np, const uint8_t* types, float* rho,
                     float* u, cudaStream_t st);
// Node types from an obstacle mask (nz*ny*nx bytes, may be null) and the walls.
// `scratch` has the size of `types`; `links` gets one word per node; esize:
// bytes of one stored population (for kSectorMate).
int nat_build_types(int q, const Geo& g, const uint8_t* mask, int noslip_mask, int esize,
                    uint8_t* scratch, uint8_t* types, uint32_t* links, cudaStream_t st);

// ---- batches of NATIVE domains (kernels_native.cu) --------------------------
// One domain of a batch: its geometry, parameters and buffers.
struct BatchDomain {
    Geo g;
    CollideParams cp;
    NativeParams np;
    const uint8_t* types;
    void* f[2];
};
// A task is one warp's work: up to 32 consecutive nodes of one z plane of
// one domain, (domain index, z, first node of the plane in x-fastest order, 0).
// One launch advances every domain by one step, reading f[parity] and
// writing f[parity ^ 1]; `blocks` resident blocks walk the task list.
// `moving`: some member has a moving wall.
// The first npair tasks are 64-node pair tasks (task .w = 1, domains with
// even nx: the two-node pair kernel's work), the rest 32-node one-node tasks;
// each kind runs in its own kernel, on blocks_pair / blocks_single resident
// blocks.
int nat_batch_step(int q, int storage, int arith, bool moving, const BatchDomain* doms, const int4* tiles,
                   int ntiles, int npair, int parity, int blocks_pair, int blocks_single, cudaStream_t st);
// Resident blocks per SM of a batch kernel (for sizing the grid); kind 0:
// one-node tasks, 1: pair tasks, 2: both in one kernel.
int nat_batch_blocks_per_sm(int q, int storage, int arith, bool moving, int kind);
constexpr int kBatchTile = 128;
// The multi-step batch kernel's grid barrier (device memory; count and error
// start at 0; error becomes 1 when a barrier's wait ran out).
struct BatchSync {
    unsigned int count;
    unsigned int gen;
    int error;
};
// nsteps steps of the batch in one cooperative launch (at most `blocks`
// blocks, no more than can be resident), a grid barrier between steps; the
// parities alternate from `parity` as with nsteps calls of nat_batch_step.
int nat_batch_step_multi(int q, int storage, int arith, bool moving, bool pairs, const BatchDomain* doms,
                         const int4* tiles, int ntiles, int parity, int nsteps, int blocks, BatchSync* bs,
                         cudaStream_t st);

// The TRT instantiations behind the functions above (kernels_trt.cu).
int nat_fused_step_trt(int q, int storage, bool has_mask, const Geo& g, const CollideParams& cp,
                       const NativeParams& np, const void* src, void* dst, const uint8_t* types, cudaStream_t st);
int nat_collide_raw_trt(int q, int storage, bool has_mask, const Geo& g, const CollideParams& cp,
                        const NativeParams& np, const void* src, void* dst, const float* rho, const float* u,
                        const uint8_t* types, cudaStream_t st);
int nat_aa_step_trt(int kind, int q, int storage, bool has_mask, const Geo& g, const CollideParams& cp,
                    const NativeParams& np, void* A, const float* rho, const float* u, const uint8_t* types,
                    cudaStream_t st);
int nat_batch_blocks_per_sm_trt(int q, int storage, bool moving, int kind);
int nat_batch_step_trt(int q, int storage, bool moving, const BatchDomain* doms, const int4* tiles, int ntiles,
                       int npair, int parity, int blocks_pair, int blocks_single, cudaStream_t st);
int nat_batch_step_multi_trt(int q, int storage, bool moving, bool pairs, const BatchDomain* doms,
                             const int4* tiles, int ntiles, int parity, int nsteps, int blocks, BatchSync* bs,
                             cudaStream_t st);

// ---- shared (kernels_util.cu) ----------------------------------------------
// Every node of the box (halo included): rho0, u0, n = feq, ntmp = 0.
// `feq_dev` is a device array of 2q floats: the equilibrium, then the weights.
// u0 is a host array.  `nt` may be null.
int util_init_uniform(int q, int storage, const Geo& g, const float* feq_dev, float rho0,
                      const float* u0, void* n, void* nt, float* rho, float* u,
                      cudaStream_t st);
// Device layout <-> plbpd's AoS halo layout (`aos` is a device buffer of
// (nx+2)(ny+2)(nz+2)*v floats).  Halo slots the device does not hold read as
// 0.  Under FP16 storage (populations only) `wk` are the v weights (device).
int util_export(int storage, int v, const Geo& g, const void* src, const float* wk, float* aos,
                cudaStream_t st);
int util_import(int storage, int v, const Geo& g, const float* aos, const float* wk, void* dst,
                cudaStream_t st);
// FP64 sums of n_k and n_k c_k over fluid nodes.  `partials` holds at least
// util_conservation_partials() doubles; out4 is a device pointer.
int util_conservation_partials();
int util_conservation(int q, int storage, const Geo& g, const void* n, const uint8_t* types,
                      int noslip_mask, double* partials, double* out4, cudaStream_t st);

}  // namespace plb
