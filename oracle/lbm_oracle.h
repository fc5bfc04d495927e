/*
 * CPU restatement of plbpd's BGK/SRT time step (the oracle).
 *
 * TEST INFRASTRUCTURE ONLY.  The parity tests, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py load this library as the checker; the product
 * library never links, loads or calls it.
 *
 * Parity: pinned.  The float instantiation in mode ORC_MODE_REFERENCE is
 * checked bit-for-bit against the reference's own sources compiled in
 * oracle/_ref (tests/test_oracle_vs_reference.py) and against the golden
 * vectors in the reference's unit tests (tests/golden/).
 *
 * State lives in the reference's layout (src/Field.hpp:37-47,91-93): AoS with
 * one halo layer on every axis, index ((z*(Y+2)+y)*(X+2)+x)*V + v with
 * X = nx+2 etc., reference coordinates 1..n for the interior.
 *
 * Two boundary semantics:
 *   ORC_MODE_REFERENCE  the reference's exact operator sequence: halo-copy
 *                       periodicity on east/west and north/south only
 *                       (src/Boundary.cpp:91-99,234-281), no-slip on wall
 *                       layers in serial (z,y,x,kp) order
 *                       (src/Boundary.cpp:101-111,189-221), in-place collision
 *                       and push streaming into the other buffer.
 *   ORC_MODE_NATIVE     every periodic axis (z included) wraps around; every
 *                       other face is a no-slip wall layer; an optional
 *                       obstacle mask marks more solid nodes.  Bounce-back is
 *                       the reference's no-slip rule applied to each solid
 *                       node: n[S+c_kp][kp] = n[S][rev kp] - 2 w rho[S+c_kp]
 *                       (c.u_b)/c_s^2 for fluid S+c_kp.
 */
#ifndef PLB_ORACLE_LBM_ORACLE_H_
#define PLB_ORACLE_LBM_ORACLE_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_MODE_REFERENCE = 0, ORC_MODE_NATIVE = 1 };
/* Collision arithmetic of the float instantiation.
 *   ORC_ARITH_AVX2    FP32 8-wide body + FP64 tail (src/CollisionSRT.cpp:93-148)
 *   ORC_ARITH_SCALAR  FP64 bracket for every direction (src/CollisionSRT.cpp:151-176)
 *   ORC_ARITH_FP32    the FP32 body's sequence for every direction          */
enum { ORC_ARITH_AVX2 = 0, ORC_ARITH_SCALAR = 1, ORC_ARITH_FP32 = 2,
       /* ORC_MODE_NATIVE, float: populations held as deviations d = f - w
        * rounded to IEEE binary16 after every step, moments and collision in
        * FP32 in deviation form (the engine's FP16 storage):
        *   drho = sum d_k, rho = 1 + drho, u = (sum c_k d_k) / rho,
        *   d'_k = (1-omega) d_k + omega w_k (drho + rho (3cu + 4.5cu^2 - 1.5usq)) */
       ORC_ARITH_FP16DEV = 3,
       /* the same deviation form with d kept in FP32, not rounded to binary16
        * (the engine's FP32 deviation storage) */
       ORC_ARITH_FP32DEV = 4 };
enum { ORC_FACE_NONE = 0, ORC_FACE_PERIODIC = 1, ORC_FACE_NOSLIP = 2 };
/* field ids */
enum { ORC_N = 0, ORC_NTMP = 1, ORC_RHO = 2, ORC_U = 3 };

typedef struct orc_sim orc_sim;

/* Lattice tables (src/LBModel.cpp:23-165).  Returns Q or 0. */
int orc_model_tables(int q, int32_t* c, float* w, uint32_t* rev, float* cs2);

/* Equilibrium on one node exactly as src/EqlbDist.hpp:26-38 (float, FP64 bracket). */
void orc_eqlb(int q, float rho, const float* u, float* out);

/* face order: east, west, north, south, up, down (src/Boundary.cpp:17-18).
 * precision: 0 = float, 1 = double.  The double instantiation uses the exact
 * weights (4/9, 1/9, ... in double, not plbpd's float ones, whose sum 1 +
 * O(1e-8) would add mass at every collision): it is the accuracy reference
 * reduced-precision runs are measured against.  Returns NULL on invalid input. */
orc_sim* orc_create(int q, long nx, long ny, long nz, float nu, float rho0,
                    const float* u0, const float* force, float rho_solid,
                    const int* face_type, const int* face_has_vel,
                    const float* face_vel, int mode, int arith, int precision);
void orc_destroy(orc_sim* s);
void orc_set_threads(int n);
int orc_max_threads(void);

/* Two-relaxation-time collision (float arithmetic ORC_ARITH_FP32 or a
 * deviation form, or double precision), in either mode.  The even part
 * of each pair (k, r = rev k) relaxes with omega = 1/tau, the odd part with
 * omega_m = 1/tau_m, tau_m = magic/(tau - 1/2) + 1/2 (magic 0 selects 3/16),
 * and the body force enters as a second-order source (no velocity shift):
 *   v = u + F/(2 rho),  f+ = (f_k + f_r)/2,  f- = (f_k - f_r)/2,
 *   e+ = w rho (1 + 4.5(c.v)^2 - 1.5v^2),  e- = 3 w rho c.v,
 *   S+ = (1 - omega/2) w (9 (c.v)(c.F) - 3 v.F),  S- = (1 - omega_m/2) 3 w c.F,
 *   f_k' = f_k - omega (f+ - e+) - omega_m (f- - e-) + S+ + S-,
 *   f_r' = f_r - omega (f+ - e+) + omega_m (f- - e-) + S+ - S-.
 * With magic 3/16 and half-way bounce-back, plane Poiseuille flow is exact.
 * Returns 0, or -1 when the arithmetic or tau (must exceed 1/2) does not
 * allow it. */
int orc_set_trt(orc_sim* s, float magic);

/* Obstacle mask for ORC_MODE_NATIVE: nz*ny*nx bytes (x fastest), nonzero = solid. */
int orc_set_mask(orc_sim* s, const uint8_t* mask);

void orc_initialize(orc_sim* s);            /* Domain::initialize + Boundary::reset */
void orc_step(orc_sim* s, long nsteps);     /* PLBPD::march_in_time's loop body     */
void orc_collide(orc_sim* s);
void orc_stream(orc_sim* s);
void orc_noslip(orc_sim* s);
void orc_periodic(orc_sim* s);
void orc_moments(orc_sim* s);
void orc_reset(orc_sim* s);

size_t orc_field_len(const orc_sim* s, int which);
/* float views (double state is rounded on get, widened on set) */
void orc_get_field(const orc_sim* s, int which, float* out);
void orc_set_field(orc_sim* s, int which, const float* in);
/* double views (float state is widened on get) */
void orc_get_field_f64(const orc_sim* s, int which, double* out);
void orc_set_field_f64(orc_sim* s, int which, const double* in);

/* tau and omega as the reference derives them (src/CollisionSRT.cpp:19-20). */
void orc_relaxation(const orc_sim* s, float* tau, float* omega);

/* Nearest IEEE binary16 value of f (round to nearest even; overflow to inf),
 * returned as a float. */
float orc_round_half(float f);

/* The value FP16 storage keeps of a deviation d = f - w: the engine stores
 * binary16(d * 2^12) and reads it back times 2^-12 (both scalings exact). */
float orc_store_half(float d);

/* Sum over fluid interior nodes of n_k and n_k c_k, in double:
 * out[0] = mass, out[1..3] = momentum. */
void orc_conservation(const orc_sim* s, double* out);

#ifdef __cplusplus
}
#endif

#endif /* PLB_ORACLE_LBM_ORACLE_H_ */
