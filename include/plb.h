/*
 * plb.h -- C ABI of the GB300 lattice-Boltzmann engine (libplb_gb300.so).
 *
 * One opaque handle (plb_solve) is one lattice-Boltzmann problem whose state
 * lives in GPU memory.  Every entry point takes plain pointers and sizes,
 * returns an int status (PLB_OK == 0, negative on error) and records a
 * message readable with plb_last_error().  The C++ classes in
 * include/plbpd/ (LBModel, Domain, Boundary, SimData, CollisionSRT, Streaming,
 * CalcMoments, LBDynamics, PLBPD, Flow) sit on top of these calls and throw
 * the exception types plbpd throws.
 *
 * Each declaration names the plbpd interface it replaces (paths inside the
 * plbpd project).
 *
 * Coordinates, layouts and faces follow plbpd:
 *   - domain sizes nx, ny, nz are plbpd's Domain(x, y, z) (src/Domain.cpp:13-22);
 *   - host arrays use plbpd's Field layout (src/Field.hpp:37-47,91-93): AoS
 *     with one halo layer on every axis, element ((z*(ny+2)+y)*(nx+2)+x)*V+v,
 *     interior coordinates 1..n;
 *   - faces are numbered east, west, north, south, up, down
 *     (src/Boundary.cpp:17-18): east/west bound x, north/south bound y,
 *     up/down bound z.
 */
#ifndef PLB_GB300_PLB_H_
#define PLB_GB300_PLB_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define PLB_OK 0
#define PLB_EINVAL (-1)       /* bad argument: plbpd throws logic_error / invalid_argument */
#define PLB_ENOMEM (-2)       /* device or host allocation failed                       */
#define PLB_ECUDA (-3)        /* a CUDA call failed                                      */
#define PLB_ETIMEOUT (-4)     /* a bounded wait ran out                                  */
#define PLB_ESTATE (-5)       /* call not valid in the handle's current state            */
#define PLB_EUNSUPPORTED (-6) /* combination the engine does not implement               */

/* ---- enumerations -------------------------------------------------------- */
#define PLB_FACE_NONE 0
#define PLB_FACE_PERIODIC 1
#define PLB_FACE_NOSLIP 2

#define PLB_FACE_EAST 0
#define PLB_FACE_WEST 1
#define PLB_FACE_NORTH 2
#define PLB_FACE_SOUTH 3
#define PLB_FACE_UP 4
#define PLB_FACE_DOWN 5

/* Boundary semantics.
 * REFERENCE: plbpd's exact operator sequence -- halo-copy periodicity on
 *   east/west and north/south only (src/Boundary.cpp:91-99,234-281), no-slip
 *   on the wall layers in plbpd's serial order (src/Boundary.cpp:189-221),
 *   push streaming into a double buffer (src/Streaming.cpp:62-94).  Results
 *   reproduce plbpd bit for bit, seams included.  FP32 storage only.
 * NATIVE: every periodic axis (z included) wraps around; every other face is
 *   a no-slip wall layer; an optional obstacle mask adds solid nodes; one
 *   fused pull kernel per step.  FP32 or FP16 storage.                      */
#define PLB_SEMANTICS_REFERENCE 0
#define PLB_SEMANTICS_NATIVE 1

/* Collision arithmetic (src/CollisionSRT.cpp:93-148).
 * REFERENCE: plbpd's AVX2 kernel op for op -- FP32 8-wide body, FP64 bracket
 *   for the directions past the last multiple of 8 -- so populations match
 *   plbpd's AVX2 build with -ffp-contract=off bit for bit.
 * FP32: the FP32 body's sequence for every direction; no FP64 on the GPU.  */
#define PLB_ARITH_REFERENCE 0
#define PLB_ARITH_FP32 1

/* Population storage.  FP16_DEV keeps f_k - w_k in IEEE half precision and
 * does all collision arithmetic in FP32 (NATIVE semantics only).  FP64
 * keeps populations and arithmetic in double with the exact weights: the
 * reference run that reduced-precision runs are measured against (NATIVE
 * semantics only).  FP32_DEV keeps f_k - w_k in FP32 with FP16_DEV's
 * arithmetic: FP32's bytes, with the precision kept in the small deviation
 * that carries the flow (NATIVE semantics only).                          */
#define PLB_STORAGE_FP32 0
#define PLB_STORAGE_FP16_DEV 1
#define PLB_STORAGE_FP64 2
#define PLB_STORAGE_FP32_DEV 3

/* Collision operator.  BGK is plbpd's CollisionSRT (src/CollisionSRT.cpp),
 * body force as the velocity shift u + F tau/rho.  TRT is an extension
 * through plbpd's Collision base (src/Collision.hpp:10-21), under either
 * semantics, always in FP32 arithmetic (FP64 with FP64 storage; `arith` is
 * not used): the even part of each pair
 * of opposite directions relaxes with 1/tau, the odd part with 1/tau_m,
 * tau_m = trt_magic/(tau - 1/2) + 1/2 (trt_magic 0 selects 3/16, which puts
 * the half-way bounce-back wall exactly half way), and the force enters as a
 * second-order source with v = u + F/(2 rho) in the equilibrium.  Exported u
 * is sum(c_k f_k)/rho under both operators, as plbpd's CalcMoments reports it. */
#define PLB_COLLISION_BGK 0
#define PLB_COLLISION_TRT 1

/* Streaming (NATIVE semantics).  AB: two population buffers, each step
 * reads one and writes the other.  AA: one buffer updated in place,
 * alternating a step that touches only the node's own slots with one that
 * reads and writes the neighbours' (the reference's Streaming leaves its
 * pull variant unimplemented, src/Streaming.cpp:96-102): half the device
 * memory, the same bytes per step, bit-identical results.  Batches take AB
 * solves only. */
#define PLB_STREAMING_AB 0
#define PLB_STREAMING_AA 1

/* Field ids: plbpd's SimData members n, ntmp, rho, u (src/SimData.hpp:18-21). */
#define PLB_FIELD_N 0
#define PLB_FIELD_NTMP 1
#define PLB_FIELD_RHO 2
#define PLB_FIELD_U 3

typedef struct plb_solve plb_solve;

/* Problem description: plbpd's LBModel + Domain + Boundary constructor
 * arguments in one struct.  Replaces
 *   LBModel(std::string)                                   src/LBModel.hpp:25
 *   Domain(lbmodel, x, y, z, nu, rho, u0, F)               src/Domain.hpp:23-28
 *   Boundary(lbmodel, domain, rho_solid, types, velocities) src/Boundary.hpp:55-60 */
typedef struct plb_params {
    int32_t q;                  /* 9 (D2Q9), 19 (D3Q19) or 27 (D3Q27)              */
    int64_t nx, ny, nz;         /* interior extents, each >= 1                      */
    float nu;                   /* viscosity; tau = 3*nu + 0.5 in float             */
    float rho0;                 /* initial density                                  */
    float u0[3];                /* initial velocity                                 */
    float force[3];             /* body force, applied as u + F*tau/rho             */
    float rho_solid;            /* density written on no-slip faces                 */
    int32_t face_type[6];       /* PLB_FACE_*, order east..down                     */
    int32_t face_has_vel[6];    /* nonzero: face_vel[f] is given                    */
    float face_vel[6][3];       /* wall velocity u_b per face                       */
    int32_t semantics;          /* PLB_SEMANTICS_*                                  */
    int32_t arith;              /* PLB_ARITH_*                                      */
    int32_t storage;            /* PLB_STORAGE_*                                    */
    int32_t device;             /* CUDA device ordinal                              */
    int32_t collision;          /* PLB_COLLISION_* (0: BGK)                         */
    float trt_magic;            /* TRT: (tau - 1/2)(tau_m - 1/2); 0 selects 3/16    */
    int32_t streaming;          /* PLB_STREAMING_* (0: AB)                          */
} plb_params;

/* ---- library ----------------------------------------------------------- */
/* Message of the last failed call on this thread ("" if none). */
const char* plb_last_error(void);
/* Library version, major*10000 + minor*100 + patch. */
int plb_version(void);

/* Lattice tables of a named model.  Replaces LBModel(name) and its getters
 * (src/LBModel.cpp:8-19,167-189).  c: Q*3 int32, w: Q floats, rev: Q uint32.
 * Returns Q, or PLB_EINVAL for an unknown name (plbpd: "Model X not yet
 * implemented", src/LBModel.cpp:17).  Any output pointer may be NULL. */
int plb_model_tables(const char* name, int32_t* c, float* w, uint32_t* rev, float* cs2);

/* Equilibrium populations on one node.  Replaces EqlbDist::operator()
 * (src/EqlbDist.hpp:26-38), same rounding: float usq and c.u, FP64 bracket. */
int plb_equilibrium(int32_t q, float rho, const float* u3, float* out_q);

/* tau and omega as CollisionSRT derives them (src/CollisionSRT.cpp:19-20). */
int plb_relaxation(float nu, float* tau, float* omega);

/* ---- solve lifetime ------------------------------------------------------ */
/* Creates the solve and its device buffers.  Replaces constructing
 * SimData(dims, Q) (src/SimData.cpp:22-30) together with the operator objects
 * CollisionSRT, Streaming, CalcMoments, LBDynamics and PLBPD
 * (src/PLBPD.cpp:6-14).  Fields start as plbpd's do: n, ntmp, rho, u = 0. */
int plb_solve_create(const plb_params* params, plb_solve** out);
int plb_solve_destroy(plb_solve* s);

/* Replace the collision parameters of an existing solve.  plbpd configures
 * CollisionSRT from a Domain (src/CollisionSRT.cpp:14-21) independently of
 * the SimData it is applied to; this call lets one device state be driven by
 * whichever operator objects the caller applies to it. */
int plb_set_relaxation(plb_solve* s, float nu, const float* force3);
/* Replace the boundary description of an existing solve (REFERENCE
 * semantics), as constructing another Boundary (src/Boundary.cpp:20-32) and
 * applying it to the same SimData would.  Arguments as in plb_params. */
/* Switches the collision operator (PLB_COLLISION_*, with the TRT magic
 * parameter) of an existing solve; the façade's CollisionTRT uses it.  No
 * counterpart in plbpd, whose LBDynamics constructs its CollisionSRT. */
int plb_set_collision(plb_solve* s, int32_t collision, float trt_magic);
int plb_set_boundary(plb_solve* s, float rho_solid, const int32_t* face_type6, const int32_t* face_has_vel6,
                     const float* face_vel18);

/* Obstacle mask, nz*ny*nx bytes with x fastest, nonzero = solid.  NATIVE
 * semantics only (plbpd has no obstacle masks; its wall rule,
 * src/Boundary.cpp:189-221, is applied to every solid node). */
int plb_set_mask(plb_solve* s, const uint8_t* mask);

/* Domain::initialize + Boundary::reset (src/PLBPD.cpp:16-19,
 * src/Domain.cpp:46-63, src/Boundary.cpp:58-89): rho0, u0 and
 * EqlbDist(rho0, u0) on every node, then the wall resets. */
int plb_initialize(plb_solve* s);

/* PLBPD::march_in_time (src/PLBPD.cpp:21-33): nsteps of collide, push,
 * no-slip, periodic copy, moments, reset, fused.  Blocks until done. */
int plb_step(plb_solve* s, int64_t nsteps);
/* Same, enqueued on the solve's stream; returns without waiting. */
int plb_step_async(plb_solve* s, int64_t nsteps);
/* Waits for the solve's stream. */
int plb_synchronize(plb_solve* s);
/* The solve's CUDA stream (a cudaStream_t), for callers that order their own
 * work after plb_step_async. */
void* plb_stream_handle(plb_solve* s);

/* ---- kernel autotuning ----------------------------------------------------------
 * The NATIVE fused step with even nx comes in several compiled variants that
 * give bit-identical results: for FP16 storage seven forms of the two-node
 * pair kernel, for FP32 (FP32 arithmetic) and FP32_DEV storage the one-node
 * kernel and three forms of the pair kernel, for FP32 storage with plbpd's
 * arithmetic the one-node kernel and one form of the pair kernel.  Before a
 * solve's first fused step the library times each on the solve's own
 * buffers (the trial steps write only the buffer the next step overwrites)
 * and keeps the fastest per lattice, storage, collision, mask, block width
 * and size class (floor(log2 cells)) for the process; PLB_TUNE_CACHE=<file>
 * keeps the table across processes, PLB_TUNE=0 uses variant 0.  A choice
 * made by trials is timed once more after 256 fused steps, on the state the
 * solve has reached (a flow started from rest can favour another variant for
 * its first steps than for the rest of the run).  No plbpd counterpart:
 * plbpd's TBB loops have no launch configuration to tune. */
/* Number of variants the library compiles (valid ids are 0 .. n-1). */
int plb_tune_variants(void);
/* variant >= 0: every solve that has not chosen yet uses it (solves whose
 * kernel has fewer variants use 0); -1: tune (the default).  PLB_EINVAL
 * for other values. */
int plb_tune_force(int32_t variant);
/* The variant the solve runs, or -1 before its first fused step. */
int plb_tune_variant(const plb_solve* s, int32_t* variant);
/* Times the variants on the solve's current state now (synchronises the
 * solve's stream), keeps the fastest for this solve and records it in the
 * table; no later trial follows.  A caller that times its own steps calls
 * it after its warm-up so that no trial falls in the timed steps.  No-op
 * (PLB_OK) for REFERENCE semantics and AA streaming; under plb_tune_force or
 * PLB_TUNE=0 it takes that variant.  Must not be called while the stream is
 * being captured. */
int plb_tune(plb_solve* s);

/* ---- batches of solves --------------------------------------------------------
 * A batch advances many NATIVE solves of one lattice, storage and device
 * together: every time step is one launch of a persistent-grid kernel whose
 * resident blocks walk a list of 128-node tiles across all member domains,
 * and the step loop replays as a captured CUDA graph.  Each domain keeps its
 * own extents, tau, force, walls and mask, and its result is bit-identical
 * to advancing it alone.  The batch does not own its solves; their own entry
 * points (initialize, set/get field, set mask, conservation) still apply
 * between batch calls, and each member's stream waits for the batch's work
 * of the last call, so they see its result without plb_batch_synchronize.
 * A step is one launch, the step loop replayed as CUDA-graph chunks; with
 * PLB_BATCH_MULTI=1 a call's steps run as one cooperative launch with a
 * grid barrier between steps instead (its loads bypass L1, which costs a few
 * per cent), and a barrier whose wait runs out ends the launch and the next
 * plb_batch_synchronize returns PLB_ETIMEOUT.
 * A batch keeps the kernel chosen at creation: after a member's lattice
 * arithmetic or collision changes (plb_set_collision) or it gains a moving
 * wall, plb_batch_step refuses with PLB_ESTATE; create a new batch.
 * No counterpart in plbpd, which runs one problem per process. */
typedef struct plb_batch plb_batch;
int plb_batch_create(int32_t n, plb_solve* const* solves, plb_batch** out);
int plb_batch_step(plb_batch* b, int64_t nsteps);
int plb_batch_step_async(plb_batch* b, int64_t nsteps);
int plb_batch_synchronize(plb_batch* b);
int plb_batch_destroy(plb_batch* b);
/* Fault injection for tests of the timeout path (PLB_BATCH_MULTI=1): the
 * next plb_batch_step's multi-step launch starts its grid barrier in a state
 * no arrival completes, so the first barrier's bounded wait runs out (about
 * a second), the kernel ends, and plb_batch_synchronize returns
 * PLB_ETIMEOUT.  The members' state is then undefined (some steps ran, some
 * did not).  No counterpart in plbpd. */
int plb_batch_fault_barrier(plb_batch* b);
/* Cells of all member domains. */
int64_t plb_batch_cells(const plb_batch* b);
/* The batch's CUDA stream (a cudaStream_t). */
void* plb_batch_stream_handle(plb_batch* b);

/* ---- serving ------------------------------------------------------------------
 * A server runs a scheduler thread that takes solve requests as they arrive,
 * admits them while their device bytes fit a budget, keeps each admitted
 * solve resident in HBM, and advances the running solves a tick of steps
 * at a time: small solves of one lattice / storage / arithmetic class
 * together as one batch, large ones (PLB_SERVER_SOLO_CELLS cells or more,
 * default 2^19) alone with their own kernels.  Every batch and large solve
 * runs on its own stream, so their kernels overlap, and the scheduler
 * restarts each one as soon as its own tick ends.  A finished solve's rho
 * and u are copied out and its memory is freed at once, so queued requests
 * start as soon as room frees up.  Results are identical to running each
 * request alone.  No counterpart in plbpd. */
typedef struct plb_server plb_server;
typedef struct plb_request {
    plb_params params;      /* NATIVE semantics                                  */
    const uint8_t* mask;    /* nz*ny*nx obstacle bytes or NULL; copied on submit */
    int64_t steps;          /* time steps to run                                 */
} plb_request;
#define PLB_REQ_QUEUED 0
#define PLB_REQ_RUNNING 1
#define PLB_REQ_DONE 2
#define PLB_REQ_FAILED 3
#define PLB_REQ_CANCELLED 4
/* Device bytes a solve with these parameters holds while it runs. */
int64_t plb_solve_bytes(const plb_params* params);
/* tick_steps: most steps a class advances between admission checks. */
int plb_server_start(int32_t device, int64_t budget_bytes, int32_t tick_steps, plb_server** out);
/* Thread-safe; the request (and its mask) is copied.  *id names it later. */
int plb_server_submit(plb_server* srv, const plb_request* req, int64_t* id);
int plb_server_status(plb_server* srv, int64_t id, int32_t* state);
/* Cancels a request: a queued one never starts; a running one stops when its
 * current tick ends and its memory returns to the budget.  Either then
 * reports PLB_REQ_CANCELLED, and wait/result return PLB_ESTATE for it.
 * PLB_ESTATE for a request that already finished. */
int plb_server_cancel(plb_server* srv, int64_t id);
/* Blocks until the request is done or failed, or timeout_s passes (PLB_ETIMEOUT). */
int plb_server_wait(plb_server* srv, int64_t id, double timeout_s);
/* Copies a finished request's rho (plb_field_len RHO floats) and u (U floats)
 * in plbpd's layout, either may be NULL, and times3 = seconds since the
 * server started at submit, admission and completion; then forgets the
 * request.  PLB_ESTATE while it is not done. */
int plb_server_result(plb_server* srv, int64_t id, float* rho, float* u, double* times3);
/* Bytes of the budget in use now, and the most in use at any time. */
int plb_server_memory(plb_server* srv, int64_t* in_use, int64_t* peak);
/* Finishes nothing further: pending and running requests are dropped. */
int plb_server_stop(plb_server* srv);

/* ---- the unfused plbpd operators (REFERENCE semantics) ---------------------
 * Each runs one operator of plbpd's loop on the device state, with plbpd's
 * semantics, so the plbpd classes can be driven operator by operator.     */
/* CollisionSRT::operator() (src/CollisionSRT.cpp:25-69): in place on n with
 * the current rho and u fields. */
int plb_collide(plb_solve* s);
/* Streaming::operator()(simdata, "push") (src/Streaming.cpp:31-94): push into
 * ntmp, then n and ntmp swap. */
int plb_stream_push(plb_solve* s);
/* Boundary::apply_noslip (src/Boundary.cpp:101-111,189-221). */
int plb_apply_noslip(plb_solve* s);
/* Boundary::apply_periodicity (src/Boundary.cpp:91-99,234-281). */
int plb_apply_periodicity(plb_solve* s);
/* CalcMoments::operator() (src/CalcMoments.hpp:47-73). */
int plb_calc_moments(plb_solve* s);
/* Boundary::reset (src/Boundary.cpp:58-66): reset_velocity then reset_density. */
int plb_reset(plb_solve* s);
/* Boundary::reset_velocity / reset_density (src/Boundary.cpp:68-89). */
int plb_reset_velocity(plb_solve* s);
int plb_reset_density(plb_solve* s);

/* ---- state transfer (host buffers, plbpd's Field layout) ------------------
 * Replaces reading/writing SimData's public Field pointers
 * (src/SimData.hpp:18-21, Field::at/get src/Field.hpp:95-109).  `out`/`in`
 * hold plb_field_len() floats.  Under NATIVE semantics the halo slots carry
 * no state (read back as 0) and ntmp reads back as 0. */
size_t plb_field_len(const plb_solve* s, int32_t which);
int plb_get_field(plb_solve* s, int32_t which, float* out);
int plb_set_field(plb_solve* s, int32_t which, const float* in);

/* Sums over the fluid nodes of n_k (mass) and n_k c_k (momentum), in FP64 on
 * the device: out[0] = mass, out[1..3] = momentum.  No plbpd counterpart;
 * plbpd has no conservation diagnostics. */
int plb_conservation(plb_solve* s, double* out4);

/* The same FP64 sums for callers that cannot allocate device memory: a
 * process that may not call cudaMalloc once it runs (its own memory pool, a
 * hard memory quota, an allocator that must see every allocation) cannot use
 * plb_conservation, whose solve handle allocates scratch.  This entry point
 * allocates nothing.  No counterpart in plbpd, which has no conservation
 * diagnostics.
 *   n      device pointer, q planes of FP32 populations, plane k at
 *          n + k*plane_stride, cells 0..ncells-1 contiguous in each plane
 *   solid  device pointer to ncells bytes (nonzero = skip the cell), or NULL
 *   out4   device pointer to 4 doubles: mass, momentum x, y, z
 *   stream a cudaStream_t (NULL = legacy default stream); the call only
 *          enqueues work, synchronize before reading out4
 * Block partials live in a fixed 128 KiB __device__ array inside the library,
 * so ncells is limited to 16,777,216 (PLB_EINVAL beyond).  The first call on
 * a device looks that array's address up (cudaGetSymbolAddress, with the
 * device current) and keeps it for the life of the process; make that first
 * call before any stream capture.  The address belongs to the device's
 * context: after cudaDeviceReset on that device it is stale, so a process that
 * resets a device must not call this entry point on it again.  All calls
 * share the array: calls whose kernels overlap on the GPU race on it. */
int plb_conservation_static(int32_t q, const float* n, int64_t ncells, int64_t plane_stride,
                            const uint8_t* solid, double* out4, void* stream);

/* Pinned host memory for fast transfers (cudaHostAlloc / cudaFreeHost). */
int plb_host_alloc(size_t bytes, void** out);
int plb_host_free(void* p);

/* Device bytes the solve holds. */
int64_t plb_device_bytes(const plb_solve* s);

#ifdef __cplusplus
}
#endif

#endif /* PLB_GB300_PLB_H_ */
