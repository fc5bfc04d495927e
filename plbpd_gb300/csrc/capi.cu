// The C ABI (include/plb.h): handle lifetime, validation, state tracking,
// step orchestration (CUDA-graph chunks of fused steps) and transfers between
// host buffers in plbpd's layout and the device layout.
#include <array>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/plb.h"
#include "engine.h"

using namespace plb;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

#define PLB_CUDA(call)                                                                        \
    do {                                                                                      \
        const cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess)                                                                \
            return fail(PLB_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_));      \
    } while (0)

#define PLB_KERNEL(call)                                                                      \
    do {                                                                                      \
        const int e_ = (call);                                                                \
        if (e_ != 0)                                                                          \
            return fail(PLB_ECUDA, std::string(#call) + ": " +                                \
                                   cudaGetErrorString(static_cast<cudaError_t>(e_)));         \
    } while (0)

#define PLB_TRY(call)                 \
    do {                              \
        const int r_ = (call);        \
        if (r_ != PLB_OK) return r_;  \
    } while (0)

// ---- host-side lattice tables (the same constexpr tables the kernels use) --
template <int Q>
void tables_of(int32_t* c, float* w, uint32_t* rev) {
    for (int k = 0; k < Q; ++k) {
        if (c) { c[3 * k] = Lattice<Q>::cx(k); c[3 * k + 1] = Lattice<Q>::cy(k); c[3 * k + 2] = Lattice<Q>::cz(k); }
        if (w) w[k] = weight<Q>(k);
        if (rev) rev[k] = (uint32_t)rev_of(k);
    }
}

bool tables(int q, int32_t* c, float* w, uint32_t* rev) {
    if (q == 9) tables_of<9>(c, w, rev);
    else if (q == 19) tables_of<19>(c, w, rev);
    else if (q == 27) tables_of<27>(c, w, rev);
    else return false;
    return true;
}

// EqlbDist::operator() (src/EqlbDist.hpp:26-38): float usq and c.u, the
// bracket in double, times the float w*rho, rounded to float.
void host_eqlb(int q, float rho, const float* u, float* out) {
    int32_t c[27 * 3];
    float w[27];
    tables(q, c, w, nullptr);
    const float usq = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
    for (int k = 0; k < q; ++k) {
        const float cu = (float)c[3 * k] * u[0] + (float)c[3 * k + 1] * u[1] + (float)c[3 * k + 2] * u[2];
        const float wr = w[k] * rho;
        const double cud = (double)cu;
        out[k] = (float)((double)wr * (1.0 + 3.0 * cud + 4.5 * cud * cud - 1.5 * (double)usq));
    }
}

// CollisionSRT's constructor (src/CollisionSRT.cpp:19-20); this file is
// compiled with -ffp-contract=off, so each operation rounds separately.
void relaxation(float nu, float* tau, float* omega) {
    const float three_nu = 3.0f * nu;
    *tau = three_nu + 0.5f;
    *omega = (float)(1. / (double)*tau);
}

long long round_up(long long v, long long m) { return (v + m - 1) / m * m; }

int graph_steps_default() {
    const char* e = std::getenv("PLB_GRAPH_STEPS");
    if (!e) return 64;
    int v = std::atoi(e);
    if (v < 0) v = 0;
    return v & ~1;   // even, so a chunk returns the buffers to their parity
}

}  // namespace

void plb::record_error(const std::string& msg) { g_last_error = msg; }

// ---------------------------------------------------------------------------
struct plb_solve {
    plb_params p;
    int q = 0;
    bool native = false;
    int storage = 0;
    int karith = 0;          // kernel arithmetic: p.arith, or kArithTRT under TRT
    Geo g{};
    CollideParams cp{};
    FaceParams fp{};
    NativeParams np{};
    cudaStream_t stream = nullptr;
    void* f[2] = {nullptr, nullptr};
    int cur = 0;
    float* rho = nullptr;
    float* u = nullptr;
    float* consts = nullptr;     // 2q floats: equilibrium(rho0, u0), weights
    uint8_t* types = nullptr;    // NATIVE node types
    uint8_t* types_tmp = nullptr;
    uint32_t* links = nullptr;   // NATIVE solid-link masks
    uint8_t* mask_dev = nullptr;
    bool has_mask = false;       // NATIVE: walls or obstacles exist
    float* staging = nullptr;    // plbpd-layout transfer buffer
    size_t staging_len = 0;
    double* partials = nullptr;
    double* out4 = nullptr;
    double* out4_host = nullptr;
    // REFERENCE: rho/u fields hold what the next collision must use
    bool fields_valid = true;
    // NATIVE: false = RAW (buffer cur holds n), true = POST (holds P_{t-1})
    bool post = false;
    // NATIVE AA streaming: one buffer f[0]; `swapped` after an even step
    // (A[rev k][x] = n*_k(x)), natural after an odd one (A[k][x] = n_k(x))
    bool aa = false;
    bool swapped = false;
    // no-slip launch groups (REFERENCE)
    int groups[6][2];
    int group_len[6];
    int ngroups = 0;
    int graph_steps = 64;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    int64_t device_bytes = 0;
    // variant of the fused-step kernel (autotuner); -1 until chosen
    int variant = -1;
    // fused steps marched since the solve was made, and the count at which
    // the variants are timed once more (-1: no second trial)
    int64_t fused_steps = 0;
    int64_t retune_at = -1;
};

namespace {

size_t esize_of(int storage) {
    return storage == PLB_STORAGE_FP16_DEV ? 2 : storage == PLB_STORAGE_FP64 ? 8 : 4;
}

// Bytes of one population buffer.
size_t pop_bytes(const plb_solve* s) { return (size_t)s->q * (size_t)s->g.ks * esize_of(s->storage); }

int set_device(const plb_solve* s) {
    int cur = -1;
    PLB_CUDA(cudaGetDevice(&cur));
    if (cur != s->p.device) PLB_CUDA(cudaSetDevice(s->p.device));
    return PLB_OK;
}

// Device memory is stream-ordered (cudaMallocAsync on the solve's stream):
// destroying a solve then waits for that stream only, where cudaFree would
// wait for the whole device and stall every other solve running beside it.
// plb_solve_create synchronizes its stream before returning, so the memory is
// usable from any stream afterwards.
int dalloc(plb_solve* s, void** p, size_t bytes) {
    const cudaError_t e = cudaMallocAsync(p, bytes, s->stream);
    if (e != cudaSuccess) {
        *p = nullptr;
        return fail(PLB_ENOMEM, std::string("cudaMallocAsync(") + std::to_string(bytes) + "): " + cudaGetErrorString(e));
    }
    s->device_bytes += (int64_t)bytes;
    return PLB_OK;
}

void drop_graphs(plb_solve* s) {
    for (int i = 0; i < 2; ++i)
        if (s->graph[i]) { cudaGraphExecDestroy(s->graph[i]); s->graph[i] = nullptr; }
}

void release(plb_solve* s) {
    if (!s) return;
    drop_graphs(s);
    for (void* ptr : {s->f[0], s->f[1], (void*)s->rho, (void*)s->u, (void*)s->consts, (void*)s->types,
                      (void*)s->types_tmp, (void*)s->links, (void*)s->mask_dev, (void*)s->staging, (void*)s->partials,
                      (void*)s->out4})
        if (ptr) cudaFreeAsync(ptr, s->stream);
    if (s->out4_host) cudaFreeHost(s->out4_host);
    if (s->stream) {
        cudaStreamSynchronize(s->stream);
        cudaStreamDestroy(s->stream);
    }
    delete s;
}

// CollisionSRT's parameters (src/CollisionSRT.cpp:14-21).
// Under TRT also the odd-moment rate, tau_m = magic/(tau - 1/2) + 1/2 in
// double, and the source factors 1 - omega/2, 1 - omega_m/2 in float.
void set_collision_params(plb_solve* s, float nu, const float* force) {
    s->p.nu = nu;
    relaxation(nu, &s->cp.tau, &s->cp.omega);
    s->cp.omc = 1.0f - s->cp.omega;
    s->cp.fx = force[0]; s->cp.fy = force[1]; s->cp.fz = force[2];
    for (int i = 0; i < 3; ++i) s->p.force[i] = force[i];
    if (s->p.collision == PLB_COLLISION_TRT) {
        const double lam = s->p.trt_magic > 0.0f ? (double)s->p.trt_magic : 3.0 / 16.0;
        const double tau_m = lam / ((double)s->cp.tau - 0.5) + 0.5;
        s->cp.omega_m_d = 1.0 / tau_m;
        s->cp.omega_m = (float)s->cp.omega_m_d;
    } else {
        s->cp.omega_m_d = 1.0 / (double)s->cp.tau;
        s->cp.omega_m = s->cp.omega;
    }
    s->cp.gp = 1.0f - 0.5f * s->cp.omega;
    s->cp.gm = 1.0f - 0.5f * s->cp.omega_m;
    s->karith = s->p.collision == PLB_COLLISION_TRT ? (int)kArithTRT : (int)s->p.arith;
}

// Boundary's parameters (src/Boundary.cpp:20-32) and the no-slip launch
// groups: faces in plbpd's order; two parallel faces share a launch when they
// are far enough apart not to touch the same slots.
void set_face_params(plb_solve* s, float rho_solid, const int32_t* face_type, const int32_t* face_has_vel,
                     const float* face_vel) {
    const float cs2 = (float)(1. / 3.);
    const float cs2inv = 1.0f / cs2;   // src/Boundary.cpp:27
    s->fp.noslip_mask = 0; s->fp.vel_mask = 0;
    for (int f = 0; f < 6; ++f) {
        s->p.face_type[f] = face_type[f];
        s->p.face_has_vel[f] = face_has_vel[f];
        if (face_type[f] == PLB_FACE_NOSLIP) s->fp.noslip_mask |= 1 << f;
        if (face_has_vel[f]) s->fp.vel_mask |= 1 << f;
        for (int i = 0; i < 3; ++i) {
            s->fp.vel[f][i] = face_has_vel[f] ? face_vel[3 * f + i] : 0.0f;
            s->p.face_vel[f][i] = s->fp.vel[f][i];
        }
    }
    s->p.rho_solid = rho_solid;
    s->fp.rho_solid = rho_solid;
    s->fp.cs2inv = cs2inv;
    s->fp.ew_periodic = face_type[0] == PLB_FACE_PERIODIC && face_type[1] == PLB_FACE_PERIODIC;
    s->fp.ns_periodic = face_type[2] == PLB_FACE_PERIODIC && face_type[3] == PLB_FACE_PERIODIC;
    const uint32_t* links = s->np.links;
    std::memset(&s->np, 0, sizeof(s->np));
    s->np.links = links;
    for (int f = 0; f < 6; ++f)
        for (int i = 0; i < 3; ++i) {
            s->np.vel[f][i] = s->fp.vel[f][i];
            if (face_type[f] == PLB_FACE_NOSLIP && s->fp.vel[f][i] != 0.0f) s->np.moving = 1;
        }
    s->np.rho_solid = rho_solid;
    s->np.cs2inv = cs2inv;
    const long long ext[3] = {s->p.nx, s->p.ny, s->p.nz};
    s->ngroups = 0;
    int f = 0;
    while (f < 6) {
        if (!((s->fp.noslip_mask >> f) & 1)) { ++f; continue; }
        const int axis = f / 2;
        if ((f % 2) == 0 && ((s->fp.noslip_mask >> (f + 1)) & 1) && ext[axis] >= 4) {
            s->groups[s->ngroups][0] = f; s->groups[s->ngroups][1] = f + 1; s->group_len[s->ngroups++] = 2;
            f += 2;
        } else {
            s->groups[s->ngroups][0] = f; s->group_len[s->ngroups++] = 1;
            f += 1;
        }
    }
}

int validate(const plb_params* p) {
    if (!p) return fail(PLB_EINVAL, "params is null");
    if (p->q != 9 && p->q != 19 && p->q != 27)
        return fail(PLB_EINVAL, "Model with " + std::to_string(p->q) + " directions not yet implemented");
    if (p->nx < 1 || p->ny < 1 || p->nz < 1) return fail(PLB_EINVAL, "argument is zero");
    {
        // a request with a NaN or infinite parameter fails here, not in the kernels
        bool finite = std::isfinite(p->nu) && std::isfinite(p->rho0) && std::isfinite(p->rho_solid) &&
                      std::isfinite(p->trt_magic);
        for (int i = 0; i < 3; ++i) finite = finite && std::isfinite(p->u0[i]) && std::isfinite(p->force[i]);
        for (int f = 0; f < 6; ++f)
            for (int i = 0; i < 3; ++i) finite = finite && std::isfinite(p->face_vel[f][i]);
        if (!finite) return fail(PLB_EINVAL, "parameters must be finite");
        if (!(3.0f * p->nu + 0.5f > 0.0f)) return fail(PLB_EINVAL, "tau = 3 nu + 1/2 must be positive");
    }
    if (p->ny > 65535 || p->nz > 65535 || p->nx > (1ll << 30))
        return fail(PLB_EINVAL, "domain extent too large (ny, nz <= 65535)");
    for (int f = 0; f < 6; ++f) {
        if (p->face_type[f] < PLB_FACE_NONE || p->face_type[f] > PLB_FACE_NOSLIP)
            return fail(PLB_EINVAL, "invalid face type");
        // a NATIVE wall moves with its face velocity, so it needs one; under
        // REFERENCE semantics the lookup fails only when no-slip runs
        // (src/Boundary.cpp:197), which plb_apply_noslip and plb_step check
        if (p->semantics == PLB_SEMANTICS_NATIVE && p->face_type[f] == PLB_FACE_NOSLIP && !p->face_has_vel[f])
            return fail(PLB_EINVAL, "no-slip face " + std::to_string(f) + " has no velocity entry");
    }
    if (p->semantics != PLB_SEMANTICS_REFERENCE && p->semantics != PLB_SEMANTICS_NATIVE)
        return fail(PLB_EINVAL, "invalid semantics");
    if (p->arith != PLB_ARITH_REFERENCE && p->arith != PLB_ARITH_FP32) return fail(PLB_EINVAL, "invalid arith");
    if (p->storage != PLB_STORAGE_FP32 && p->storage != PLB_STORAGE_FP16_DEV && p->storage != PLB_STORAGE_FP64 &&
        p->storage != PLB_STORAGE_FP32_DEV)
        return fail(PLB_EINVAL, "invalid storage");
    if (p->storage != PLB_STORAGE_FP32 && p->semantics != PLB_SEMANTICS_NATIVE)
        return fail(PLB_EUNSUPPORTED, "FP16, FP64 and FP32 deviation storage need NATIVE semantics");
    if (p->collision != PLB_COLLISION_BGK && p->collision != PLB_COLLISION_TRT)
        return fail(PLB_EINVAL, "invalid collision operator");
    if (p->streaming != PLB_STREAMING_AB && p->streaming != PLB_STREAMING_AA)
        return fail(PLB_EINVAL, "invalid streaming");
    if (p->streaming == PLB_STREAMING_AA && p->semantics != PLB_SEMANTICS_NATIVE)
        return fail(PLB_EUNSUPPORTED, "AA streaming needs NATIVE semantics");
    if (p->collision == PLB_COLLISION_TRT) {
        if (!(p->trt_magic >= 0.0f) || p->trt_magic > 1e30f) return fail(PLB_EINVAL, "invalid TRT magic parameter");
        if (!(3.0f * p->nu + 0.5f > 0.5f)) return fail(PLB_EINVAL, "TRT needs tau > 1/2 (nu > 0)");
    }
    if (p->semantics == PLB_SEMANTICS_NATIVE) {
        int32_t c[27 * 3];
        tables(p->q, c, nullptr, nullptr);
        for (int a = 0; a < 3; ++a) {
            bool moves = false;
            for (int k = 0; k < p->q; ++k) moves |= c[3 * k + a] != 0;
            const int t0 = p->face_type[2 * a], t1 = p->face_type[2 * a + 1];
            const bool per = t0 == PLB_FACE_PERIODIC && t1 == PLB_FACE_PERIODIC;
            const bool wall = t0 == PLB_FACE_NOSLIP && t1 == PLB_FACE_NOSLIP;
            if (moves && !per && !wall)
                return fail(PLB_EINVAL, "NATIVE semantics: each axis the lattice moves along must be periodic on "
                                        "both faces or no-slip on both faces");
        }
    }
    return PLB_OK;
}

// Page-locked host memory that the device can address (plb_host_alloc,
// cudaHostAlloc, registered memory) is read or written by the layout kernels
// directly over the host link: one pass instead of a copy plus a pass.
// Returns null for other memory, which goes through the staging buffer.
// Page-locked host memory can be read and written by the layout kernels in
// place over the host link (PLB_PINNED_TRANSFER=direct), or moved by one
// bulk DMA copy through the device staging buffer with the layout conversion
// on the device (copy, the default: on GB300 the copy engines move a large
// pinned buffer several times faster than kernel loads and stores that cross
// the link).  Other host memory always takes the staging path.
bool pinned_direct() {
    static const bool direct = [] {
        const char* e = std::getenv("PLB_PINNED_TRANSFER");
        return e && std::strcmp(e, "direct") == 0;
    }();
    return direct;
}

float* device_view(const void* host) {
    if (!pinned_direct()) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
    return static_cast<float*>(a.devicePointer);
}

// Transfer buffer for one field of v components (grown on demand).
int ensure_staging(plb_solve* s, int v) {
    const size_t cells = (size_t)(s->p.nx + 2) * (s->p.ny + 2) * (s->p.nz + 2);
    const size_t need = cells * (size_t)v;
    if (s->staging && s->staging_len >= need) return PLB_OK;
    if (s->staging) { cudaFreeAsync(s->staging, s->stream); s->device_bytes -= (int64_t)(s->staging_len * sizeof(float)); s->staging = nullptr; }
    PLB_TRY(dalloc(s, (void**)&s->staging, need * sizeof(float)));
    s->staging_len = need;
    return PLB_OK;
}

// ---- REFERENCE semantics ---------------------------------------------------
// plbpd looks the wall velocity of every no-slip face up when no-slip runs
// (src/Boundary.cpp:197) and throws if it is missing.
int check_noslip_velocities(const plb_solve* s) {
    const int missing = s->fp.noslip_mask & ~s->fp.vel_mask;
    if (missing) {
        int f = 0;
        while (!((missing >> f) & 1)) ++f;
        return fail(PLB_EINVAL, "no-slip face " + std::to_string(f) + " has no velocity entry");
    }
    return PLB_OK;
}

int ref_noslip_all(plb_solve* s) {
    PLB_TRY(check_noslip_velocities(s));
    float* n = (float*)s->f[s->cur];
    for (int i = 0; i < s->ngroups; ++i)
        PLB_KERNEL(ref_noslip(s->q, s->g, s->fp, s->groups[i], s->group_len[i], n, s->rho, s->stream));
    return PLB_OK;
}

int ref_boundary(plb_solve* s) {
    PLB_TRY(ref_noslip_all(s));
    PLB_KERNEL(ref_periodic(s->q, s->g, s->fp, (float*)s->f[s->cur], s->stream));
    return PLB_OK;
}

int ref_one_step(plb_solve* s, bool first, bool wb_all) {
    PLB_KERNEL(ref_fused_step(s->q, s->karith, first, wb_all, s->g, s->cp, s->fp, (float*)s->f[s->cur],
                              (float*)s->f[1 - s->cur], s->rho, s->u, s->stream));
    s->cur = 1 - s->cur;
    return ref_boundary(s);
}

// rho/u fields = moments of n + resets, which is what plbpd holds after
// march_in_time.
int ref_materialize_fields(plb_solve* s) {
    if (s->fields_valid) return PLB_OK;
    PLB_KERNEL(ref_moments(s->q, s->g, (const float*)s->f[s->cur], s->rho, s->u, s->stream));
    PLB_KERNEL(ref_reset(s->g, s->fp, true, true, s->rho, s->u, s->stream));
    s->fields_valid = true;
    return PLB_OK;
}

// ---- autotuner of the fused-step kernel --------------------------------------
// The NATIVE fused step with even nx is compiled in several variants that
// give the same bits (native_impl.cuh: kH2Variant for FP16 storage; the
// one-node kernel and the pair kernel's forms for FP32 and FP32_DEV, either
// arithmetic); which is fastest depends on the lattice, the mask, the block
// width and the domain size.  Before a solve's
// first fused step the variants are timed on the solve's own buffers: a pull
// step reads buffer cur and writes the other one, which the next real step
// overwrites, so trial launches leave the state as it was.  The winner is
// kept per (lattice, storage, arithmetic, mask, moving walls, block width,
// size class = floor(log2 cells)) for the process, and in the file named by
// PLB_TUNE_CACHE across processes.  PLB_TUNE=0 turns tuning off (variant 0);
// plb_tune_force fixes one variant.
//
// The state a solve starts from can favour another variant than the state
// it runs in: with plbpd's arithmetic a masked flow at rest sends many tail
// evaluations to the FP64 fallback for its first steps, where the one-node
// kernel is faster, and the pair kernel is faster from then on.  So a
// choice made by trials is timed once more after kRetuneSteps fused steps,
// on the state the solve has reached, and that choice is kept (graphs
// captured with the first are dropped).  plb_tune times the variants on
// the current state at a moment the caller picks, and no second trial
// follows it.
constexpr int64_t kRetuneSteps = 256;
using TuneKey = std::array<int, 7>;
std::mutex g_tune_mu;
std::map<TuneKey, int> g_tune;
bool g_tune_loaded = false;
std::atomic<int> g_tune_force{-1};

std::string device_tag() {
    int dev = 0;
    cudaDeviceProp prop{};
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return "unknown";
    std::string n = prop.name;
    for (char& c : n)
        if (c == ' ') c = '_';
    return n + "_sm" + std::to_string(prop.multiProcessorCount);
}

// Loads PLB_TUNE_CACHE once (lines: plb-tune-v2 device q storage arith mask
// moving wide size_class variant); caller holds g_tune_mu.
void tune_load_locked() {
    if (g_tune_loaded) return;
    g_tune_loaded = true;
    const char* path = std::getenv("PLB_TUNE_CACHE");
    if (!path || !*path) return;
    std::ifstream in(path);
    const std::string dev = device_tag();
    std::string line;
    while (std::getline(in, line)) {
        std::istringstream ls(line);
        std::string magic, d;
        TuneKey k{};
        int v = -1;
        if (!(ls >> magic >> d) || magic != "plb-tune-v2" || d != dev) continue;
        bool ok = true;
        for (int& x : k) ok = ok && static_cast<bool>(ls >> x);
        if (ok && (ls >> v) && v >= 0) g_tune[k] = v;
    }
}

void tune_store_locked(const TuneKey& k, int v) {
    g_tune[k] = v;
    const char* path = std::getenv("PLB_TUNE_CACHE");
    if (!path || !*path) return;
    std::ofstream out(path, std::ios::app);
    out << "plb-tune-v2 " << device_tag();
    for (int x : k) out << ' ' << x;
    out << ' ' << v << '\n';
}

int fused_variants(const plb_solve* s) {
    if (!s->native || s->aa) return 1;
    return nat_fused_variants(s->q, s->storage, s->karith, s->has_mask && s->np.moving, s->g);
}

int launch_fused(plb_solve* s, int variant) {
    PLB_KERNEL(nat_fused_step(s->q, s->storage, s->karith, s->has_mask, s->g, s->cp, s->np, s->f[s->cur],
                              s->f[1 - s->cur], s->types, variant, s->stream));
    return PLB_OK;
}

// Mean time of `reps` launches of one variant, in ms.
int time_variant(plb_solve* s, int v, int reps, cudaEvent_t e0, cudaEvent_t e1, float* ms) {
    for (int i = 0; i < 2; ++i) PLB_TRY(launch_fused(s, v));
    PLB_CUDA(cudaEventRecord(e0, s->stream));
    for (int i = 0; i < reps; ++i) PLB_TRY(launch_fused(s, v));
    PLB_CUDA(cudaEventRecord(e1, s->stream));
    PLB_CUDA(cudaEventSynchronize(e1));
    PLB_CUDA(cudaEventElapsedTime(ms, e0, e1));
    *ms /= (float)reps;
    return PLB_OK;
}

TuneKey tune_key(const plb_solve* s) {
    const long long cells = (long long)s->g.nx * s->g.ny * s->g.nz;
    int cls = 0;
    while ((2LL << cls) <= cells) ++cls;
    return {s->q, s->storage, s->karith, (int)s->has_mask, (int)(s->has_mask && s->np.moving),
            (int)(s->g.nx % 256 == 0), cls};
}

// The variant a solve takes without trials: 0 for one variant or PLB_TUNE=0,
// the forced one, or -1 (trials decide).
int untimed_variant(const plb_solve* s, int nv) {
    const int forced = g_tune_force.load();
    if (nv <= 1) return 0;
    if (forced >= 0) return forced < nv ? forced : 0;
    const char* on = std::getenv("PLB_TUNE");
    if (on && std::strcmp(on, "0") == 0) return 0;
    return -1;
}

// Times every variant on the solve's current state, sets s->variant to the
// fastest and records it (not during a graph capture: the trials
// synchronise).
int tune_trials(plb_solve* s, int nv) {
    const long long cells = (long long)s->g.nx * s->g.ny * s->g.nz;
    // about 2^25 node updates a trial, 3 to 50 launches; two passes over the
    // variants, the second in reverse order, and each variant's faster pass
    // counts, so a clock that is still rising or another process's burst
    // does not decide the choice
    const long long r = (1LL << 25) / (cells > 0 ? cells : 1);
    const int reps = r < 3 ? 3 : (r > 50 ? 50 : (int)r);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    PLB_CUDA(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) { cudaEventDestroy(e0); return fail(PLB_ECUDA, "cudaEventCreate"); }
    std::vector<float> best_of(nv, 0.0f);
    int rc = PLB_OK;
    for (int pass = 0; pass < 2 && rc == PLB_OK; ++pass) {
        for (int i = 0; i < nv && rc == PLB_OK; ++i) {
            const int v = pass == 0 ? i : nv - 1 - i;
            float ms = 0.0f;
            rc = time_variant(s, v, reps, e0, e1, &ms);
            if (rc == PLB_OK && (pass == 0 || ms < best_of[v])) best_of[v] = ms;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != PLB_OK) return rc;
    int best = 0;
    for (int v = 1; v < nv; ++v)
        if (best_of[v] < best_of[best]) best = v;
    if (best != s->variant) drop_graphs(s);   // captured with the other variant
    s->variant = best;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    tune_store_locked(tune_key(s), best);
    return PLB_OK;
}

// Sets s->variant before the solve's first fused step: untimed, from the
// table, or by trials (then timed again after kRetuneSteps fused steps).
int choose_variant(plb_solve* s) {
    const int nv = fused_variants(s);
    const int fixed = untimed_variant(s, nv);
    if (fixed >= 0) { s->variant = fixed; return PLB_OK; }
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        tune_load_locked();
        auto it = g_tune.find(tune_key(s));
        if (it != g_tune.end() && it->second < nv) { s->variant = it->second; return PLB_OK; }
    }
    PLB_TRY(tune_trials(s, nv));
    s->retune_at = s->fused_steps + kRetuneSteps;
    return PLB_OK;
}

// The second trial of a choice made by trials, once the solve has marched
// kRetuneSteps fused steps.
int maybe_retune(plb_solve* s) {
    if (s->retune_at < 0 || s->fused_steps < s->retune_at) return PLB_OK;
    s->retune_at = -1;
    const int nv = fused_variants(s);
    if (untimed_variant(s, nv) >= 0) return PLB_OK;
    return tune_trials(s, nv);
}

// ---- NATIVE semantics ------------------------------------------------------
int nat_one_step(plb_solve* s) {
    if (s->aa) {
        PLB_KERNEL(nat_aa_step(s->swapped ? 2 : 1, s->q, s->storage, s->karith, s->has_mask, s->g, s->cp, s->np,
                               s->f[0], s->rho, s->u, s->types, s->stream));
        s->swapped = !s->swapped;
        return PLB_OK;
    }
    if (s->variant < 0) PLB_TRY(choose_variant(s));
    PLB_TRY(launch_fused(s, s->variant));
    s->cur = 1 - s->cur;
    return PLB_OK;
}

// n_t and its moments from P_{t-1}, into the other buffer and the fields;
// the state itself is left as it is (POST stays POST), so reading the state
// does not change the trajectory.
int nat_gather_to_other(plb_solve* s) {
    PLB_KERNEL(nat_gather(s->q, s->storage, s->has_mask, s->g, s->np, s->f[s->cur], s->f[1 - s->cur], s->rho,
                          s->u, s->types, s->stream));
    return PLB_OK;
}

// POST -> RAW: n_t and its moments become the state (before the caller
// replaces part of it).
int nat_materialize(plb_solve* s) {
    if (!s->post) return PLB_OK;
    if (s->aa) {
        if (s->swapped) {
            // the natural layout cannot be rebuilt in place: gather into a
            // transient buffer and copy it back
            const size_t bytes = pop_bytes(s);
            void* tmp = nullptr;
            PLB_CUDA(cudaMallocAsync(&tmp, bytes, s->stream));
            const int e = nat_aa_gather(s->q, s->storage, s->has_mask, true, s->g, s->np, s->f[0], tmp, s->rho, s->u,
                                        s->types, s->stream);
            const cudaError_t c = e == 0 ? cudaMemcpyAsync(s->f[0], tmp, bytes, cudaMemcpyDeviceToDevice, s->stream)
                                         : cudaSuccess;
            cudaFreeAsync(tmp, s->stream);
            if (e != 0) return fail(PLB_ECUDA, std::string("nat_aa_gather: ") + cudaGetErrorString((cudaError_t)e));
            if (c != cudaSuccess) return fail(PLB_ECUDA, std::string("cudaMemcpyAsync: ") + cudaGetErrorString(c));
        } else {
            PLB_KERNEL(nat_aa_gather(s->q, s->storage, s->has_mask, false, s->g, s->np, s->f[0], nullptr, s->rho,
                                     s->u, s->types, s->stream));
        }
        s->post = false;
        s->swapped = false;
        return PLB_OK;
    }
    PLB_TRY(nat_gather_to_other(s));
    s->cur = 1 - s->cur;
    s->post = false;
    return PLB_OK;
}

// ---- graphs of fused steps --------------------------------------------------
int capture_chunk(plb_solve* s, int parity) {
    cudaGraph_t graph = nullptr;
    PLB_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    int rc = PLB_OK;
    for (int i = 0; i < s->graph_steps && rc == PLB_OK; ++i)
        rc = s->native ? nat_one_step(s) : ref_one_step(s, false, false);
    const cudaError_t ec = cudaStreamEndCapture(s->stream, &graph);
    if (rc != PLB_OK) { if (graph) cudaGraphDestroy(graph); return rc; }
    if (ec != cudaSuccess) return fail(PLB_ECUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(ec));
    const cudaError_t ei = cudaGraphInstantiate(&s->graph[parity], graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) return fail(PLB_ECUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ei));
    return PLB_OK;
}

int run_chunk(plb_solve* s) {
    // a chunk has an even number of steps, so it ends in the state it began
    const int parity = s->aa ? (int)s->swapped : s->cur;
    if (!s->graph[parity]) {
        if (s->native && s->variant < 0) PLB_TRY(choose_variant(s));   // before the capture
        PLB_TRY(capture_chunk(s, parity));   // capture toggles cur an even number of times
    }
    PLB_CUDA(cudaGraphLaunch(s->graph[parity], s->stream));
    return PLB_OK;
}

// A REFERENCE march of a small D2Q9 domain runs in one cluster launch with
// its state in distributed shared memory (kernels_ref_cluster.cu), unless
// PLB_REF_CLUSTER=0.  D2Q9 moves in the x-z plane only; a north/south no-slip
// face would make the whole plane a wall and keeps the three-launch path.
bool ref_cluster_eligible(const plb_solve* s, int* C, int* R) {
    const char* e = std::getenv("PLB_REF_CLUSTER");
    if (e && std::strcmp(e, "0") == 0) return false;
    if (s->q != 9 || s->g.ny != 1 || (s->fp.noslip_mask & 0x0c)) return false;
    return ref_cluster_shape(s->g.nx, s->g.nz, C, R) != 0;
}

int ref_march_in_cluster(plb_solve* s, int C, int R, int64_t n) {
    RefNoslipPlan plan{};
    plan.ngroups = s->ngroups;
    for (int i = 0; i < s->ngroups; ++i) {
        plan.len[i] = s->group_len[i];
        for (int j = 0; j < s->group_len[i]; ++j) plan.faces[i][j] = s->groups[i][j];
    }
    PLB_KERNEL(ref_march_cluster(s->karith, C, R, s->g, s->cp, s->fp, plan, (float*)s->f[0], (float*)s->f[1],
                                 s->rho, s->u, s->cur, (long long)n, s->fields_valid, true, s->stream));
    if (n & 1) s->cur = 1 - s->cur;
    s->post = false;
    s->fields_valid = false;
    return PLB_OK;
}

int march(plb_solve* s, int64_t n) {
    if (n < 0) return fail(PLB_EINVAL, "negative step count");
    if (n == 0) return PLB_OK;
    const int64_t G = s->graph_steps;
    if (!s->native) {
        PLB_TRY(check_noslip_velocities(s));
        int C = 0, R = 0;
        if (ref_cluster_eligible(s, &C, &R)) return ref_march_in_cluster(s, C, R, n);
        // the first step reads the fields when they are the caller's; the
        // last writes every node back so the other buffer equals plbpd's ntmp
        int64_t done = 0;
        PLB_TRY(ref_one_step(s, s->fields_valid, n == 1));
        done = 1;
        while (G > 0 && n - done - 1 >= G) { PLB_TRY(run_chunk(s)); done += G; }
        while (done < n) { PLB_TRY(ref_one_step(s, false, done == n - 1)); ++done; }
        s->fields_valid = false;
        return PLB_OK;
    }
    int64_t done = 0;
    if (!s->post) {
        if (s->aa) {
            PLB_KERNEL(nat_aa_step(0, s->q, s->storage, s->karith, s->has_mask, s->g, s->cp, s->np, s->f[0], s->rho,
                                   s->u, s->types, s->stream));
            s->swapped = true;
        } else {
            PLB_KERNEL(nat_collide_raw(s->q, s->storage, s->karith, s->has_mask, s->g, s->cp, s->np, s->f[s->cur],
                                       s->f[1 - s->cur], s->rho, s->u, s->types, s->stream));
            s->cur = 1 - s->cur;
        }
        s->post = true;
        done = 1;
    }
    while (done < n) {
        PLB_TRY(maybe_retune(s));
        if (G > 0 && n - done >= G) {
            PLB_TRY(run_chunk(s));
            done += G;
            s->fused_steps += G;
        } else {
            PLB_TRY(nat_one_step(s));
            ++done;
            ++s->fused_steps;
        }
    }
    return PLB_OK;
}

int sync(plb_solve* s) {
    PLB_CUDA(cudaStreamSynchronize(s->stream));
    return PLB_OK;
}

}  // namespace

int plb::check_params(const plb_params* p) { return validate(p); }

namespace {
// Waits for `st`'s work, then replaces it with a stream of CUDA priority
// `priority`.  Captured graphs are not bound to a stream, and memory the old
// stream allocated is usable once its work is done.
int restream(cudaStream_t* st, int priority) {
    cudaStream_t ns = nullptr;
    PLB_CUDA(cudaStreamSynchronize(*st));
    PLB_CUDA(cudaStreamCreateWithPriority(&ns, cudaStreamNonBlocking, priority));
    cudaStreamDestroy(*st);
    *st = ns;
    return PLB_OK;
}
}  // namespace

int plb::set_solve_priority(plb_solve* s, int priority) {
    if (!s) return fail(PLB_EINVAL, "solve is null");
    PLB_CUDA(cudaSetDevice(s->p.device));
    return restream(&s->stream, priority);
}

// ===========================================================================
extern "C" {

const char* plb_last_error(void) { return g_last_error.c_str(); }

int plb_version(void) { return 10000; }

int plb_model_tables(const char* name, int32_t* c, float* w, uint32_t* rev, float* cs2) {
    if (!name) return fail(PLB_EINVAL, "model name is null");
    const std::string n(name);
    const int q = n == "D2Q9" ? 9 : n == "D3Q19" ? 19 : n == "D3Q27" ? 27 : 0;
    if (!q) return fail(PLB_EINVAL, "Model " + n + " not yet implemented");
    tables(q, c, w, rev);
    if (cs2) *cs2 = (float)(1. / 3.);
    return q;
}

int plb_equilibrium(int32_t q, float rho, const float* u3, float* out_q) {
    if (!tables(q, nullptr, nullptr, nullptr)) return fail(PLB_EINVAL, "invalid Q");
    if (!u3 || !out_q) return fail(PLB_EINVAL, "null pointer");
    host_eqlb(q, rho, u3, out_q);
    return PLB_OK;
}

int plb_relaxation(float nu, float* tau, float* omega) {
    float t, o;
    relaxation(nu, &t, &o);
    if (tau) *tau = t;
    if (omega) *omega = o;
    return PLB_OK;
}

int plb_solve_create(const plb_params* params, plb_solve** out) {
    if (!out) return fail(PLB_EINVAL, "out is null");
    *out = nullptr;
    PLB_TRY(validate(params));
    plb_solve* s = new plb_solve();
    s->p = *params;
    s->q = params->q;
    s->native = params->semantics == PLB_SEMANTICS_NATIVE;
    s->storage = params->storage;
    s->aa = s->native && params->streaming == PLB_STREAMING_AA;
    s->graph_steps = graph_steps_default();
    int rc = PLB_OK;
    auto bail = [&](int code) { release(s); return code; };
    {
        const cudaError_t e = cudaSetDevice(params->device);
        if (e != cudaSuccess) return bail(fail(PLB_ECUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e)));
    }
    // geometry
    Geo& g = s->g;
    g.nx = (int)params->nx; g.ny = (int)params->ny; g.nz = (int)params->nz;
    const size_t esize = esize_of(s->storage);
    if (s->native) {
        g.h = 0; g.xoff = 0;
        g.ys = round_up(g.nx, 32 / (long long)esize);
        g.zs = g.ys * g.ny;
        g.fs = g.zs * g.nz;
        g.ks = round_up(g.fs, 128);
        g.wrap_x = params->face_type[0] == PLB_FACE_PERIODIC && params->face_type[1] == PLB_FACE_PERIODIC;
        g.wrap_y = params->face_type[2] == PLB_FACE_PERIODIC && params->face_type[3] == PLB_FACE_PERIODIC;
        g.wrap_z = params->face_type[4] == PLB_FACE_PERIODIC && params->face_type[5] == PLB_FACE_PERIODIC;
    } else {
        g.h = 1; g.xoff = 8;
        g.ys = round_up(g.xoff + g.nx + 1, 8);
        g.zs = g.ys * (g.ny + 2);
        g.fs = g.zs * (g.nz + 2);
        g.ks = round_up(g.fs, 64);
    }
    // collision and boundary parameters, derived as plbpd derives them
    set_collision_params(s, params->nu, params->force);
    set_face_params(s, params->rho_solid, params->face_type, params->face_has_vel, &params->face_vel[0][0]);
    // device memory
    {
        const cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) return bail(fail(PLB_ECUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e)));
    }
    const size_t pbytes = pop_bytes(s);
    if ((rc = dalloc(s, &s->f[0], pbytes)) != PLB_OK) return bail(rc);
    if (!s->aa && (rc = dalloc(s, &s->f[1], pbytes)) != PLB_OK) return bail(rc);   // AA: one buffer
    if ((rc = dalloc(s, (void**)&s->rho, (size_t)g.ks * sizeof(float))) != PLB_OK) return bail(rc);
    if ((rc = dalloc(s, (void**)&s->u, 3 * (size_t)g.ks * sizeof(float))) != PLB_OK) return bail(rc);
    if ((rc = dalloc(s, (void**)&s->consts, 2 * 27 * sizeof(float))) != PLB_OK) return bail(rc);
    if ((rc = dalloc(s, (void**)&s->partials, (size_t)util_conservation_partials() * sizeof(double))) != PLB_OK)
        return bail(rc);
    if ((rc = dalloc(s, (void**)&s->out4, 4 * sizeof(double))) != PLB_OK) return bail(rc);
    if (cudaHostAlloc((void**)&s->out4_host, 4 * sizeof(double), cudaHostAllocDefault) != cudaSuccess)
        return bail(fail(PLB_ENOMEM, "cudaHostAlloc failed"));
    {
        // plbpd's SimData starts every field at 0 (src/SimData.cpp:53-56)
        cudaError_t e = cudaSuccess;
        if (e == cudaSuccess) e = cudaMemsetAsync(s->f[0], 0, pbytes, s->stream);
        if (e == cudaSuccess && s->f[1]) e = cudaMemsetAsync(s->f[1], 0, pbytes, s->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(s->rho, 0, (size_t)g.ks * sizeof(float), s->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(s->u, 0, 3 * (size_t)g.ks * sizeof(float), s->stream);
        if (e != cudaSuccess) return bail(fail(PLB_ECUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e)));
    }
    {
        // consts: EqlbDist(rho0, u0), then the weights
        float host[54];
        host_eqlb(s->q, params->rho0, params->u0, host);
        tables(s->q, nullptr, host + s->q, nullptr);
        if (cudaMemcpyAsync(s->consts, host, 2 * s->q * sizeof(float), cudaMemcpyHostToDevice, s->stream) !=
            cudaSuccess)
            return bail(fail(PLB_ECUDA, "cudaMemcpyAsync(consts)"));
    }
    if (s->native) {
        s->has_mask = s->fp.noslip_mask != 0;
        if ((rc = dalloc(s, (void**)&s->types, (size_t)g.ks)) != PLB_OK) return bail(rc);
        if ((rc = dalloc(s, (void**)&s->types_tmp, (size_t)g.ks)) != PLB_OK) return bail(rc);
        if ((rc = dalloc(s, (void**)&s->links, (size_t)g.ks * sizeof(uint32_t))) != PLB_OK) return bail(rc);
        s->np.links = s->links;
        if (cudaMemsetAsync(s->types, 0, (size_t)g.ks, s->stream) != cudaSuccess)
            return bail(fail(PLB_ECUDA, "cudaMemsetAsync(types)"));
        const int e = nat_build_types(s->q, g, nullptr, s->fp.noslip_mask, (int)esize_of(s->storage), s->types_tmp,
                                      s->types, s->links, s->stream);
        if (e != 0) return bail(fail(PLB_ECUDA, "nat_build_types"));
        s->post = false;
    }
    s->fields_valid = true;
    if (cudaStreamSynchronize(s->stream) != cudaSuccess) return bail(fail(PLB_ECUDA, "solve setup failed"));
    *out = s;
    return PLB_OK;
}

int plb_solve_destroy(plb_solve* s) {
    if (!s) return PLB_OK;
    set_device(s);
    cudaStreamSynchronize(s->stream);
    release(s);
    return PLB_OK;
}

int plb_set_relaxation(plb_solve* s, float nu, const float* force3) {
    if (!s || !force3) return fail(PLB_EINVAL, "null argument");
    if (s->p.nu == nu && s->p.force[0] == force3[0] && s->p.force[1] == force3[1] && s->p.force[2] == force3[2])
        return PLB_OK;
    if (s->p.collision == PLB_COLLISION_TRT && !(3.0f * nu + 0.5f > 0.5f))
        return fail(PLB_EINVAL, "TRT needs tau > 1/2 (nu > 0)");
    PLB_TRY(set_device(s));
    PLB_TRY(sync(s));
    set_collision_params(s, nu, force3);
    drop_graphs(s);   // captured launches carry the old parameters
    return PLB_OK;
}

int plb_set_collision(plb_solve* s, int32_t collision, float trt_magic) {
    if (!s) return fail(PLB_EINVAL, "solve is null");
    if (s->p.collision == collision && s->p.trt_magic == trt_magic) return PLB_OK;
    plb_params p = s->p;
    p.collision = collision;
    p.trt_magic = trt_magic;
    PLB_TRY(validate(&p));
    PLB_TRY(set_device(s));
    PLB_TRY(sync(s));
    s->p.collision = collision;
    s->p.trt_magic = trt_magic;
    set_collision_params(s, s->p.nu, s->p.force);
    drop_graphs(s);   // captured launches carry the old operator
    return PLB_OK;
}

int plb_set_boundary(plb_solve* s, float rho_solid, const int32_t* face_type6, const int32_t* face_has_vel6,
                     const float* face_vel18) {
    if (!s || !face_type6 || !face_has_vel6 || !face_vel18) return fail(PLB_EINVAL, "null argument");
    if (s->native) return fail(PLB_EUNSUPPORTED, "changing the boundary needs REFERENCE semantics");
    bool same = s->p.rho_solid == rho_solid;
    for (int f = 0; f < 6; ++f) {
        if (face_type6[f] < PLB_FACE_NONE || face_type6[f] > PLB_FACE_NOSLIP) return fail(PLB_EINVAL, "invalid face type");
        same = same && s->p.face_type[f] == face_type6[f] && (s->p.face_has_vel[f] != 0) == (face_has_vel6[f] != 0);
        for (int i = 0; i < 3; ++i)
            same = same && (!face_has_vel6[f] || s->p.face_vel[f][i] == face_vel18[3 * f + i]);
    }
    if (same) return PLB_OK;
    PLB_TRY(set_device(s));
    PLB_TRY(sync(s));
    PLB_TRY(ref_materialize_fields(s));   // the pending resets belong to the old boundary
    set_face_params(s, rho_solid, face_type6, face_has_vel6, face_vel18);
    drop_graphs(s);
    return PLB_OK;
}

int plb_set_mask(plb_solve* s, const uint8_t* mask) {
    if (!s) return fail(PLB_EINVAL, "solve is null");
    if (!s->native) return fail(PLB_EUNSUPPORTED, "obstacle masks need NATIVE semantics");
    PLB_TRY(set_device(s));
    PLB_TRY(nat_materialize(s));
    const size_t cells = (size_t)s->g.cells();
    if (!s->mask_dev) PLB_TRY(dalloc(s, (void**)&s->mask_dev, cells));
    if (mask) PLB_CUDA(cudaMemcpyAsync(s->mask_dev, mask, cells, cudaMemcpyHostToDevice, s->stream));
    PLB_KERNEL(nat_build_types(s->q, s->g, mask ? s->mask_dev : nullptr, s->fp.noslip_mask,
                               (int)esize_of(s->storage), s->types_tmp, s->types, s->links, s->stream));
    s->has_mask = mask != nullptr || s->fp.noslip_mask != 0;
    drop_graphs(s);
    return sync(s);
}

int plb_initialize(plb_solve* s) {
    if (!s) return fail(PLB_EINVAL, "solve is null");
    PLB_TRY(set_device(s));
    // Domain::initialize writes n, rho and u and leaves ntmp as it is
    if (s->native) { s->post = false; s->swapped = false; }
    PLB_KERNEL(util_init_uniform(s->q, s->storage, s->g, s->consts, s->p.rho0, s->p.u0, s->f[s->cur], nullptr,
                                 s->rho, s->u, s->stream));
    if (s->native) {
        if (s->has_mask) PLB_KERNEL(nat_reset_fields(s->g, s->np, s->types, s->rho, s->u, s->stream));
        s->post = false;
    } else {
        PLB_KERNEL(ref_reset(s->g, s->fp, true, true, s->rho, s->u, s->stream));
        s->fields_valid = true;
    }
    return sync(s);
}

int plb_step_async(plb_solve* s, int64_t nsteps) {
    if (!s) return fail(PLB_EINVAL, "solve is null");
    PLB_TRY(set_device(s));
    return march(s, nsteps);
}

int plb_tune_variants(void) { return kFusedVariants; }

int plb_tune_force(int32_t variant) {
    if (variant < -1 || variant >= kFusedVariants) return fail(PLB_EINVAL, "variant out of range");
    g_tune_force.store(variant);
    return PLB_OK;
}

int plb_tune_variant(const plb_solve* s, int32_t* variant) {
    if (!s || !variant) return fail(PLB_EINVAL, "null argument");
    *variant = s->variant;
    return PLB_OK;
}

int plb_tune(plb_solve* s) {
    if (!s) return fail(PLB_EINVAL, "solve is null");
    PLB_TRY(set_device(s));
    s->retune_at = -1;
    if (!s->native || s->aa) return PLB_OK;   // one kernel form, nothing to time
    const int nv = fused_variants(s);
    const int fixed = untimed_variant(s, nv);
    if (fixed >= 0) {
        if (fixed != s->variant) drop_graphs(s);
        s->variant = fixed;
        return PLB_OK;
    }
    return tune_trials(s, nv);
}

int plb_step(plb_solve* s, int64_t nsteps) {
    PLB_TRY(plb_step_async(s, nsteps));
    return sync(s);
}

int plb_synchronize(plb_solve* s) {
    if (!s) return fail(PLB_EINVAL, "solve is null");
    PLB_TRY(set_device(s));
    return sync(s);
}

void* plb_stream_handle(plb_solve* s) { return s ? (void*)s->stream : nullptr; }

// ---- unfused operators ------------------------------------------------------
#define PLB_REF_ONLY(s)                                                                   \
    do {                                                                                  \
        if (!(s)) return fail(PLB_EINVAL, "solve is null");                               \
        if ((s)->native) return fail(PLB_EUNSUPPORTED, "operator needs REFERENCE semantics"); \
        PLB_TRY(set_device(s));                                                           \
        PLB_TRY(ref_materialize_fields(s));                                               \
    } while (0)

int plb_collide(plb_solve* s) {
    PLB_REF_ONLY(s);
    PLB_KERNEL(ref_collide(s->q, s->karith, s->g, s->cp, (float*)s->f[s->cur], s->rho, s->u, s->stream));
    return sync(s);
}

int plb_stream_push(plb_solve* s) {
    PLB_REF_ONLY(s);
    PLB_KERNEL(ref_push(s->q, s->g, (const float*)s->f[s->cur], (float*)s->f[1 - s->cur], s->stream));
    s->cur = 1 - s->cur;
    return sync(s);
}

int plb_apply_noslip(plb_solve* s) {
    PLB_REF_ONLY(s);
    PLB_TRY(ref_noslip_all(s));
    return sync(s);
}

int plb_apply_periodicity(plb_solve* s) {
    PLB_REF_ONLY(s);
    PLB_KERNEL(ref_periodic(s->q, s->g, s->fp, (float*)s->f[s->cur], s->stream));
    return sync(s);
}

int plb_calc_moments(plb_solve* s) {
    PLB_REF_ONLY(s);
    PLB_KERNEL(ref_moments(s->q, s->g, (const float*)s->f[s->cur], s->rho, s->u, s->stream));
    return sync(s);
}

int plb_reset(plb_solve* s) {
    PLB_REF_ONLY(s);
    PLB_KERNEL(ref_reset(s->g, s->fp, true, true, s->rho, s->u, s->stream));
    return sync(s);
}

int plb_reset_velocity(plb_solve* s) {
    PLB_REF_ONLY(s);
    PLB_KERNEL(ref_reset(s->g, s->fp, true, false, s->rho, s->u, s->stream));
    return sync(s);
}

int plb_reset_density(plb_solve* s) {
    PLB_REF_ONLY(s);
    PLB_KERNEL(ref_reset(s->g, s->fp, false, true, s->rho, s->u, s->stream));
    return sync(s);
}

// ---- transfers ----------------------------------------------------------------
size_t plb_field_len(const plb_solve* s, int32_t which) {
    if (!s) return 0;
    const size_t cells = (size_t)(s->p.nx + 2) * (s->p.ny + 2) * (s->p.nz + 2);
    switch (which) {
        case PLB_FIELD_N: case PLB_FIELD_NTMP: return cells * (size_t)s->q;
        case PLB_FIELD_RHO: return cells;
        case PLB_FIELD_U: return cells * 3;
        default: return 0;
    }
}

}  // extern "C"

namespace {
// Enqueues a field read on the solve's stream (plb_get_field without the
// wait).  `gathered`: a NATIVE state's moments are already in the rho/u
// fields (a read of the other moment field came first).  `slot`: element
// offset of the field in the staging buffer, which must hold
// `staging_comps` components a cell.
int enqueue_get_field(plb_solve* s, int32_t which, float* out, bool gathered, size_t slot, int staging_comps) {
    const size_t len = plb_field_len(s, which);
    int n_buf = s->cur;   // buffer that holds n for FIELD_N
    void* tmp = nullptr;   // AA: transient natural copy of a swapped buffer
    if (s->native) {
        if (which == PLB_FIELD_NTMP) { std::memset(out, 0, len * sizeof(float)); return PLB_OK; }
        if (s->post && s->aa) {
            if (which == PLB_FIELD_N) {
                // also from the natural layout: the gather reads solid nodes as 0, as the two-buffer path does
                PLB_CUDA(cudaMallocAsync(&tmp, pop_bytes(s), s->stream));
                const int e = nat_aa_gather(s->q, s->storage, s->has_mask, s->swapped, s->g, s->np, s->f[0], tmp,
                                            nullptr, nullptr, s->types, s->stream);
                if (e != 0) {
                    cudaFreeAsync(tmp, s->stream);
                    return fail(PLB_ECUDA, std::string("nat_aa_gather: ") + cudaGetErrorString((cudaError_t)e));
                }
            } else if (!gathered) {
                PLB_KERNEL(nat_aa_gather(s->q, s->storage, s->has_mask, s->swapped, s->g, s->np, s->f[0], nullptr,
                                         s->rho, s->u, s->types, s->stream));
            }
        } else if (s->post) {
            if (which == PLB_FIELD_N) {
                PLB_TRY(nat_gather_to_other(s));
                n_buf = 1 - s->cur;
            } else if (!gathered) {
                // rho and u only: the gather writes no populations
                PLB_KERNEL(nat_gather(s->q, s->storage, s->has_mask, s->g, s->np, s->f[s->cur], nullptr, s->rho,
                                      s->u, s->types, s->stream));
            }
        }
    } else if (which == PLB_FIELD_RHO || which == PLB_FIELD_U) {
        PLB_TRY(ref_materialize_fields(s));
    }
    float* direct = device_view(out);
    if (!direct) PLB_TRY(ensure_staging(s, staging_comps));
    float* aos = direct ? direct : s->staging + slot;
    const float* wk = s->consts + s->q;
    if (which == PLB_FIELD_N || which == PLB_FIELD_NTMP) {
        const void* src = tmp ? tmp : s->f[which == PLB_FIELD_N ? n_buf : 1 - s->cur];
        const int e = util_export(s->storage, s->q, s->g, src, wk, aos, s->stream);
        if (tmp) cudaFreeAsync(tmp, s->stream);
        if (e != 0) return fail(PLB_ECUDA, std::string("util_export: ") + cudaGetErrorString((cudaError_t)e));
    } else {
        PLB_KERNEL(util_export(0, which == PLB_FIELD_RHO ? 1 : 3, s->g, which == PLB_FIELD_RHO ? s->rho : s->u,
                               nullptr, aos, s->stream));
    }
    if (!direct) PLB_CUDA(cudaMemcpyAsync(out, aos, len * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    return PLB_OK;
}
}  // namespace

int plb::read_moments(plb_solve* s, float* rho, float* u) {
    if (!s || !rho || !u) return fail(PLB_EINVAL, "null argument");
    PLB_TRY(set_device(s));
    const size_t cells = plb_field_len(s, PLB_FIELD_RHO);
    PLB_TRY(enqueue_get_field(s, PLB_FIELD_RHO, rho, false, 0, 4));
    PLB_TRY(enqueue_get_field(s, PLB_FIELD_U, u, true, cells, 4));
    return sync(s);
}

extern "C" {

int plb_get_field(plb_solve* s, int32_t which, float* out) {
    if (!s || !out) return fail(PLB_EINVAL, "null argument");
    if (which < PLB_FIELD_N || which > PLB_FIELD_U) return fail(PLB_EINVAL, "invalid field id");
    PLB_TRY(set_device(s));
    const size_t len = plb_field_len(s, which);
    const int comps = (int)(len / ((size_t)(s->p.nx + 2) * (s->p.ny + 2) * (s->p.nz + 2)));
    PLB_TRY(enqueue_get_field(s, which, out, false, 0, comps));
    return sync(s);
}

int plb_set_field(plb_solve* s, int32_t which, const float* in) {
    if (!s || !in) return fail(PLB_EINVAL, "null argument");
    if (which < PLB_FIELD_N || which > PLB_FIELD_U) return fail(PLB_EINVAL, "invalid field id");
    PLB_TRY(set_device(s));
    if (s->native) {
        if (which == PLB_FIELD_NTMP) return PLB_OK;   // NATIVE keeps no second population state
        PLB_TRY(nat_materialize(s));
    } else {
        PLB_TRY(ref_materialize_fields(s));
    }
    const size_t len = plb_field_len(s, which);
    const float* aos = device_view(in);
    if (!aos) {
        PLB_TRY(ensure_staging(s, (int)(len / ((size_t)(s->p.nx + 2) * (s->p.ny + 2) * (s->p.nz + 2)))));
        PLB_CUDA(cudaMemcpyAsync(s->staging, in, len * sizeof(float), cudaMemcpyHostToDevice, s->stream));
        aos = s->staging;
    }
    if (which == PLB_FIELD_N || which == PLB_FIELD_NTMP) {
        void* dst = s->f[which == PLB_FIELD_N ? s->cur : 1 - s->cur];
        PLB_KERNEL(util_import(s->storage, s->q, s->g, aos, s->consts + s->q, dst, s->stream));
    } else {
        PLB_KERNEL(util_import(0, which == PLB_FIELD_RHO ? 1 : 3, s->g, aos, nullptr,
                               which == PLB_FIELD_RHO ? (void*)s->rho : (void*)s->u, s->stream));
        if (!s->native) s->fields_valid = true;
    }
    return sync(s);
}

int plb_conservation(plb_solve* s, double* out4) {
    if (!s || !out4) return fail(PLB_EINVAL, "null argument");
    PLB_TRY(set_device(s));
    // the sums are of the current populations n_t; under NATIVE semantics the
    // state may be P_{t-1}, whose bounce-back slots hold reversed directions,
    // so n_t is gathered first (mass alone would not need it, momentum does)
    const void* src = s->f[s->cur];
    void* tmp = nullptr;
    if (s->native && s->post && s->aa) {
        if (s->swapped) {
            PLB_CUDA(cudaMallocAsync(&tmp, pop_bytes(s), s->stream));
            const int e = nat_aa_gather(s->q, s->storage, s->has_mask, true, s->g, s->np, s->f[0], tmp, nullptr,
                                        nullptr, s->types, s->stream);
            if (e != 0) {
                cudaFreeAsync(tmp, s->stream);
                return fail(PLB_ECUDA, std::string("nat_aa_gather: ") + cudaGetErrorString((cudaError_t)e));
            }
            src = tmp;
        }
    } else if (s->native && s->post) {
        PLB_KERNEL(nat_gather(s->q, s->storage, s->has_mask, s->g, s->np, s->f[s->cur], s->f[1 - s->cur], nullptr,
                              nullptr, s->types, s->stream));
        src = s->f[1 - s->cur];
    }
    const int ec = util_conservation(s->q, s->storage, s->g, src, s->native ? s->types : nullptr, s->fp.noslip_mask,
                                     s->partials, s->out4, s->stream);
    if (tmp) cudaFreeAsync(tmp, s->stream);
    if (ec != 0) return fail(PLB_ECUDA, std::string("util_conservation: ") + cudaGetErrorString((cudaError_t)ec));
    PLB_CUDA(cudaMemcpyAsync(s->out4_host, s->out4, 4 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    PLB_TRY(sync(s));
    std::memcpy(out4, s->out4_host, 4 * sizeof(double));
    return PLB_OK;
}

int plb_host_alloc(size_t bytes, void** out) {
    if (!out) return fail(PLB_EINVAL, "out is null");
    PLB_CUDA(cudaHostAlloc(out, bytes, cudaHostAllocDefault));
    return PLB_OK;
}

int plb_host_free(void* p) {
    if (p) PLB_CUDA(cudaFreeHost(p));
    return PLB_OK;
}

int64_t plb_device_bytes(const plb_solve* s) { return s ? s->device_bytes : 0; }

}  // extern "C"

// ===========================================================================
// batches
struct plb_batch {
    std::vector<plb_solve*> solves;
    int q = 0, storage = 0, arith = 0, device = 0;
    cudaStream_t stream = nullptr;
    BatchDomain* d_doms = nullptr;
    int4* d_tiles = nullptr;   // warp tasks (domain, z, first node of the plane, 1 for a pair task)
    int ntiles = 0;
    int npair = 0;             // the first npair tasks are pair tasks
    int blocks = 0;            // the multi-step kernel's grid (both kinds in one kernel)
    int blocks_pair = 0, blocks_single = 0;   // the one-step kernels' grids
    int64_t cells = 0;
    bool moving = false;   // some member has a moving wall
    bool pairs = false;    // some domain has even nx: 64-node pair tasks beside 32-node ones
    int graph_steps = 64;
    cudaGraphExec_t graph = nullptr;
    cudaEvent_t done = nullptr;   // recorded after each batch call's work
    std::vector<cudaEvent_t> member_ev;   // one per member: its own work so far
    std::vector<BatchDomain> h_doms;
    // multi-step launches (PLB_BATCH_MULTI=1: one cooperative launch runs a
    // call's steps, a grid barrier between them)
    bool multi = false;
    BatchSync* d_sync = nullptr;
    int* err_host = nullptr;   // the barrier's error word after the last launch (page-locked)
    bool fault_next = false;   // plb_batch_fault_barrier: the next launch's first barrier cannot complete
};

namespace {

void batch_release(plb_batch* b) {
    if (!b) return;
    if (b->graph) cudaGraphExecDestroy(b->graph);
    if (b->done) cudaEventDestroy(b->done);
    for (cudaEvent_t e : b->member_ev)
        if (e) cudaEventDestroy(e);
    if (b->d_sync) cudaFreeAsync(b->d_sync, b->stream);
    if (b->d_doms) cudaFreeAsync(b->d_doms, b->stream);
    if (b->d_tiles) cudaFreeAsync(b->d_tiles, b->stream);
    if (b->stream) {
        cudaStreamSynchronize(b->stream);
        cudaStreamDestroy(b->stream);
    }
    if (b->err_host) cudaFreeHost(b->err_host);
    delete b;
}

// Brings every member to the POST state with one step where needed: members
// in RAW take their first collision, members already in POST one fused step,
// so all advance by exactly one step.  Returns the step count consumed.
int batch_prepare(plb_batch* b, int64_t* consumed) {
    bool any_raw = false;
    for (plb_solve* s : b->solves) any_raw |= !s->post;
    *consumed = 0;
    if (!any_raw) return PLB_OK;
    for (plb_solve* s : b->solves) {
        if (!s->post) {
            PLB_KERNEL(nat_collide_raw(s->q, s->storage, s->karith, s->has_mask, s->g, s->cp, s->np, s->f[s->cur],
                                       s->f[1 - s->cur], s->rho, s->u, s->types, b->stream));
            s->post = true;
        } else {
            PLB_KERNEL(nat_fused_step(s->q, s->storage, s->karith, s->has_mask, s->g, s->cp, s->np, s->f[s->cur],
                                      s->f[1 - s->cur], s->types, s->variant < 0 ? 0 : s->variant, b->stream));
        }
        s->cur = 1 - s->cur;
    }
    *consumed = 1;
    return PLB_OK;
}

// The batch's kernel was chosen for the lattice, storage, kernel arithmetic
// (collision operator included) and moving walls its members had when it was
// created; a member changed since then (plb_set_collision, new faces) would
// run under the wrong kernel, so the call is refused instead.
int batch_check_members(const plb_batch* b) {
    for (const plb_solve* s : b->solves) {
        if (s->q != b->q || s->storage != b->storage || s->karith != b->arith || s->aa || !s->native)
            return fail(PLB_ESTATE, "a batch member's lattice, storage, arithmetic or collision changed after "
                                    "plb_batch_create; create a new batch");
        if (s->np.moving && !b->moving)
            return fail(PLB_ESTATE, "a batch member gained a moving wall after plb_batch_create; create a new batch");
    }
    return PLB_OK;
}

// Device table of the members, each with its buffers ordered so that
// f[0] is the one holding the current state.
int batch_upload_table(plb_batch* b) {
    for (size_t i = 0; i < b->solves.size(); ++i) {
        plb_solve* s = b->solves[i];
        BatchDomain& d = b->h_doms[i];
        d.g = s->g;
        d.cp = s->cp;
        d.np = s->np;
        d.types = s->types;
        d.f[0] = s->f[s->cur];
        d.f[1] = s->f[1 - s->cur];
    }
    PLB_CUDA(cudaMemcpyAsync(b->d_doms, b->h_doms.data(), b->h_doms.size() * sizeof(BatchDomain),
                             cudaMemcpyHostToDevice, b->stream));
    return PLB_OK;
}

int batch_capture(plb_batch* b) {
    cudaGraph_t graph = nullptr;
    PLB_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    int rc = 0;
    for (int i = 0; i < b->graph_steps && rc == 0; ++i)
        rc = nat_batch_step(b->q, b->storage, b->arith, b->moving, b->d_doms, b->d_tiles, b->ntiles, b->npair, i & 1,
                            b->blocks_pair, b->blocks_single, b->stream);
    const cudaError_t ec = cudaStreamEndCapture(b->stream, &graph);
    if (rc != 0) {
        if (graph) cudaGraphDestroy(graph);
        return fail(PLB_ECUDA, std::string("batch capture: ") + cudaGetErrorString((cudaError_t)rc));
    }
    if (ec != cudaSuccess) return fail(PLB_ECUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(ec));
    const cudaError_t ei = cudaGraphInstantiate(&b->graph, graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) return fail(PLB_ECUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ei));
    return PLB_OK;
}

}  // namespace

int plb::set_batch_multi(plb_batch* b, bool multi) {
    if (!b) return fail(PLB_EINVAL, "batch is null");
    b->multi = multi;
    return PLB_OK;
}

int plb::set_batch_priority(plb_batch* b, int priority) {
    if (!b) return fail(PLB_EINVAL, "batch is null");
    PLB_CUDA(cudaSetDevice(b->device));
    return restream(&b->stream, priority);
}

extern "C" {

int plb_batch_create(int32_t n, plb_solve* const* solves, plb_batch** out) {
    if (!out || !solves || n < 1) return fail(PLB_EINVAL, "a batch needs at least one solve");
    *out = nullptr;
    const plb_solve* s0 = solves[0];
    if (!s0) return fail(PLB_EINVAL, "null solve");
    for (int i = 0; i < n; ++i) {
        const plb_solve* s = solves[i];
        if (!s) return fail(PLB_EINVAL, "null solve");
        if (!s->native) return fail(PLB_EUNSUPPORTED, "batches need NATIVE semantics");
        if (s->q != s0->q || s->storage != s0->storage || s->karith != s0->karith || s->p.device != s0->p.device)
            return fail(PLB_EINVAL, "batch members must share lattice, storage, arithmetic and device");
        if (s->storage == PLB_STORAGE_FP64) return fail(PLB_EUNSUPPORTED, "FP64 storage is not batched");
        if (s->aa) return fail(PLB_EUNSUPPORTED, "AA streaming is not batched");
        if ((long long)s->g.ys * s->g.ny * s->g.nz >= (1ll << 31))
            return fail(PLB_EINVAL, "batch member too large for 32-bit tile indices");
    }
    plb_batch* b = new plb_batch();
    b->solves.assign(solves, solves + n);
    b->q = s0->q; b->storage = s0->storage; b->arith = s0->karith; b->device = s0->p.device;
    b->graph_steps = graph_steps_default();
    b->h_doms.resize(n);
    if (cudaSetDevice(b->device) != cudaSuccess) { batch_release(b); return fail(PLB_ECUDA, "cudaSetDevice"); }
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
        batch_release(b);
        return fail(PLB_ECUDA, "cudaStreamCreate");
    }
    b->member_ev.assign(n, nullptr);
    bool ev_ok = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming) == cudaSuccess;
    for (int i = 0; i < n && ev_ok; ++i)
        ev_ok = cudaEventCreateWithFlags(&b->member_ev[i], cudaEventDisableTiming) == cudaSuccess;
    if (!ev_ok) {
        batch_release(b);
        return fail(PLB_ECUDA, "cudaEventCreate");
    }
    // a domain with even nx runs as pair tasks (two nodes a lane, 64 a warp),
    // listed first: each kind has its own kernel
    std::vector<int4> tiles;
    for (int kind = 1; kind >= 0; --kind) {
        for (int i = 0; i < n; ++i) {
            const Geo& g = solves[i]->g;
            const bool pair = g.nx % 2 == 0;
            if ((int)pair != kind) continue;
            const int per_task = pair ? 64 : 32;
            b->pairs |= pair;
            const int plane = g.nx * g.ny;   // nodes of one z plane, x fastest
            for (int z = 0; z < g.nz; ++z)
                for (int i0 = 0; i0 < plane; i0 += per_task) tiles.push_back(make_int4(i, z, i0, pair ? 1 : 0));
            b->cells += g.cells();
        }
        if (kind == 1) b->npair = (int)tiles.size();
    }
    b->ntiles = (int)tiles.size();
    int dev_sms = 0;
    cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, b->device);
    if (dev_sms < 1) dev_sms = 1;
    for (int i = 0; i < n; ++i) b->moving |= solves[i]->np.moving != 0;
    auto grid_of = [&](int kind) {
        const int per_sm = nat_batch_blocks_per_sm(b->q, b->storage, b->arith, b->moving, kind);
        return dev_sms * (per_sm > 0 ? per_sm : 1);
    };
    b->blocks = grid_of(b->pairs ? 2 : 0);
    b->blocks_pair = grid_of(1);
    b->blocks_single = grid_of(0);
    // stream-ordered, like a solve's memory
    if (cudaMallocAsync(&b->d_doms, n * sizeof(BatchDomain), b->stream) != cudaSuccess ||
        cudaMallocAsync(&b->d_tiles, tiles.size() * sizeof(int4), b->stream) != cudaSuccess ||
        cudaMallocAsync(&b->d_sync, sizeof(BatchSync), b->stream) != cudaSuccess) {
        batch_release(b);
        return fail(PLB_ENOMEM, "batch tables");
    }
    if (cudaHostAlloc(&b->err_host, sizeof(int), cudaHostAllocDefault) != cudaSuccess) {
        b->err_host = nullptr;
        batch_release(b);
        return fail(PLB_ENOMEM, "batch error word");
    }
    *b->err_host = 0;
    {
        const char* e = std::getenv("PLB_BATCH_MULTI");
        b->multi = e && std::strcmp(e, "1") == 0;
    }
    // from pageable memory: the call returns once the tiles are staged, so
    // the vector may go; the stream orders the copy before the first step
    if (cudaMemcpyAsync(b->d_tiles, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice, b->stream) !=
        cudaSuccess) {
        batch_release(b);
        return fail(PLB_ECUDA, "batch tile upload");
    }
    *out = b;
    return PLB_OK;
}

int plb_batch_step_async(plb_batch* b, int64_t nsteps) {
    if (!b) return fail(PLB_EINVAL, "batch is null");
    if (nsteps < 0) return fail(PLB_EINVAL, "negative step count");
    if (nsteps == 0) return PLB_OK;
    PLB_CUDA(cudaSetDevice(b->device));
    PLB_TRY(batch_check_members(b));
    // members' own work comes first (stream order, no host wait)
    for (size_t m = 0; m < b->solves.size(); ++m) {
        PLB_CUDA(cudaEventRecord(b->member_ev[m], b->solves[m]->stream));
        PLB_CUDA(cudaStreamWaitEvent(b->stream, b->member_ev[m], 0));
    }
    int64_t done = 0;
    PLB_TRY(batch_prepare(b, &done));
    PLB_TRY(batch_upload_table(b));
    int64_t i = 0;
    const int64_t todo = nsteps - done;
    const int64_t G = b->graph_steps;
    // multi-step launches, chunks of at most 2^16 steps; a configuration
    // the cooperative launch refuses (too many blocks for co-residency)
    // falls back to one launch a step
    while (b->multi && i < todo) {
        const int n = (int)(todo - i < (1 << 16) ? todo - i : (1 << 16));
        BatchSync init{b->fault_next ? 0x7fffffffu : 0u, 0u, 0};
        b->fault_next = false;
        PLB_CUDA(cudaMemcpyAsync(b->d_sync, &init, sizeof(init), cudaMemcpyHostToDevice, b->stream));
        const int rc = nat_batch_step_multi(b->q, b->storage, b->arith, b->moving, b->pairs, b->d_doms, b->d_tiles,
                                            b->ntiles, (int)(i & 1), n, b->blocks, b->d_sync, b->stream);
        if (rc == (int)cudaErrorCooperativeLaunchTooLarge || rc == (int)cudaErrorInvalidConfiguration) {
            cudaGetLastError();
            b->multi = false;
            break;
        }
        if (rc != 0) return fail(PLB_ECUDA, std::string("nat_batch_step_multi: ") + cudaGetErrorString((cudaError_t)rc));
        PLB_CUDA(cudaMemcpyAsync(b->err_host, &b->d_sync->error, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
        i += n;
    }
    while (G > 0 && todo - i >= G) {
        if (!b->graph) PLB_TRY(batch_capture(b));
        PLB_CUDA(cudaGraphLaunch(b->graph, b->stream));
        i += G;
    }
    for (; i < todo; ++i)
        PLB_KERNEL(nat_batch_step(b->q, b->storage, b->arith, b->moving, b->d_doms, b->d_tiles, b->ntiles, b->npair,
                                  (int)(i & 1), b->blocks_pair, b->blocks_single, b->stream));
    if (todo & 1)
        for (plb_solve* s : b->solves) s->cur = 1 - s->cur;
    // a member's own calls (fields, conservation, steps) run on its stream:
    // order them after the batch's work on its buffers
    PLB_CUDA(cudaEventRecord(b->done, b->stream));
    for (plb_solve* s : b->solves) PLB_CUDA(cudaStreamWaitEvent(s->stream, b->done, 0));
    return PLB_OK;
}

int plb_batch_synchronize(plb_batch* b) {
    if (!b) return fail(PLB_EINVAL, "batch is null");
    PLB_CUDA(cudaStreamSynchronize(b->stream));
    if (*b->err_host) {
        *b->err_host = 0;
        return fail(PLB_ETIMEOUT, "a grid barrier of the multi-step batch kernel waited too long; the steps of "
                                  "that launch did not all run");
    }
    return PLB_OK;
}

int plb_batch_fault_barrier(plb_batch* b) {
    if (!b) return fail(PLB_EINVAL, "batch is null");
    b->fault_next = true;
    return PLB_OK;
}

int plb_batch_step(plb_batch* b, int64_t nsteps) {
    PLB_TRY(plb_batch_step_async(b, nsteps));
    return plb_batch_synchronize(b);
}

int plb_batch_destroy(plb_batch* b) {
    if (!b) return PLB_OK;
    cudaStreamSynchronize(b->stream);
    batch_release(b);
    return PLB_OK;
}

int64_t plb_batch_cells(const plb_batch* b) { return b ? b->cells : 0; }

void* plb_batch_stream_handle(plb_batch* b) { return b ? (void*)b->stream : nullptr; }

}  // extern "C"
