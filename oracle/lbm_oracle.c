/*
 * CPU restatement of plbpd's BGK/SRT time step: the oracle.
 * TEST INFRASTRUCTURE ONLY (see lbm_oracle.h).  Compiled with
 * -ffp-contract=off so that every float operation rounds where the source
 * says it does, on x86-64 and aarch64 alike.
 */
#include "lbm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#if defined(_OPENMP)
#include <omp.h>
#endif

struct orc_sim {
    int q;
    long nx, ny, nz;      /* interior extents                        */
    long X, Y, Z;         /* extents with the halo: n + 2             */
    int32_t c[27][3];
    float w[27];          /* plbpd's weights: double literals rounded to float */
    double wd[27];        /* the exact weights in double, for precision 1:
                             the float ones sum to 1 + O(1e-8), which a double
                             run would add to the mass every collision */
    uint32_t rev[27];
    float cs2, cs2inv;
    float nu, rho0, u0[3], force[3], rho_solid;
    float tau, omega;
    int trt;              /* NATIVE: two-relaxation-time collision       */
    float omega_m;        /* TRT: odd-moment rate, float arithmetic      */
    double omega_m_d;     /* TRT: odd-moment rate, double arithmetic     */
    int face_type[6], face_has_vel[6];
    float face_vel[6][3];
    int mode, arith, precision;
    int wrap[3];          /* NATIVE: axis x/y/z wraps around          */
    void *n, *ntmp, *rho, *u;
    uint8_t* solid;       /* per node of the halo box: 1 = solid      */
    uint8_t* solid_vel;   /* 0..5 = wall face, 6 = obstacle           */
    float* drho;          /* FP16 deviation arithmetic: sum of d_k    */
};

/* ---- lattice tables: src/LBModel.cpp:23-165 ------------------------------ */
/* Velocity order, weights (double literals rounded to float) and reverse
 * indices must be identical to the reference's for index-level parity. */
static const int32_t kD2Q9[9][3] = {
    {0, 0, 0}, {1, 0, 0}, {-1, 0, 0}, {0, 0, 1}, {0, 0, -1},
    {1, 0, 1}, {-1, 0, -1}, {1, 0, -1}, {-1, 0, 1}};
static const int32_t kD3Q19[19][3] = {
    {0, 0, 0}, {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1},
    {1, 1, 0}, {-1, -1, 0}, {1, -1, 0}, {-1, 1, 0}, {1, 0, 1}, {-1, 0, -1},
    {1, 0, -1}, {-1, 0, 1}, {0, 1, 1}, {0, -1, -1}, {0, 1, -1}, {0, -1, 1}};
static const int32_t kD3Q27[27][3] = {
    {0, 0, 0}, {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1},
    {1, 1, 0}, {-1, -1, 0}, {1, -1, 0}, {-1, 1, 0}, {1, 0, 1}, {-1, 0, -1},
    {1, 0, -1}, {-1, 0, 1}, {0, 1, 1}, {0, -1, -1}, {0, 1, -1}, {0, -1, 1},
    {1, 1, 1}, {-1, -1, -1}, {1, 1, -1}, {-1, -1, 1}, {1, -1, 1}, {-1, 1, -1},
    {-1, 1, 1}, {1, -1, -1}};

/* Populations held as deviations d = f - w (float instantiation). */
static int orc_dev(const orc_sim* s) {
    return !s->precision && (s->arith == ORC_ARITH_FP16DEV || s->arith == ORC_ARITH_FP32DEV);
}

/* Weight of a velocity with |c|^2 = sp, as the reference's double literal. */
static double weight_exact(int q, int sp) {
    if (q == 9) return sp == 0 ? 4. / 9. : (sp == 1 ? 1. / 9. : 1. / 36.);
    if (q == 19) return sp == 0 ? 1. / 3. : (sp == 1 ? 1. / 18. : 1. / 36.);
    return sp == 0 ? 8. / 27. : (sp == 1 ? 2. / 27. : (sp == 2 ? 1. / 54. : 1. / 216.));
}

int orc_model_tables(int q, int32_t* c, float* w, uint32_t* rev, float* cs2) {
    const int32_t(*cv)[3];
    if (q == 9) cv = kD2Q9;
    else if (q == 19) cv = kD3Q19;
    else if (q == 27) cv = kD3Q27;
    else return 0;
    for (int k = 0; k < q; ++k) {
        for (int i = 0; i < 3; ++i) c[3 * k + i] = cv[k][i];
        w[k] = (float)weight_exact(q, abs(cv[k][0]) + abs(cv[k][1]) + abs(cv[k][2]));
        /* every table lists each velocity directly before or after its opposite */
        rev[k] = k == 0 ? 0u : (uint32_t)(k % 2 == 1 ? k + 1 : k - 1);
    }
    *cs2 = (float)(1. / 3.);
    return q;
}

/* EqlbDist::operator() (src/EqlbDist.hpp:26-38): float usq and cu, FP64
 * bracket, product with the float w*rho, rounded to float on store. */
void orc_eqlb(int q, float rho, const float* u, float* out) {
    int32_t c[27 * 3];
    float w[27], cs2;
    uint32_t rev[27];
    if (!orc_model_tables(q, c, w, rev, &cs2)) return;
    const float usq = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
    for (int k = 0; k < q; ++k) {
        const float cu = (float)c[3 * k] * u[0] + (float)c[3 * k + 1] * u[1] +
                         (float)c[3 * k + 2] * u[2];
        const float wr = w[k] * rho;
        const double cud = (double)cu;
        out[k] = (float)((double)wr *
                         (1.0 + 3.0 * cud + 4.5 * cud * cud - 1.5 * (double)usq));
    }
}

/* ---- geometry helpers ----------------------------------------------------- */
static inline long orc_wrap(long v, long n, int wraps) {
    if (!wraps) return v;
    if (v < 1) return v + n;
    if (v > n) return v - n;
    return v;
}

/* Boundary::_get_boundary_extent (src/Boundary.cpp:113-148): a face is the
 * one-node-thick first or last interior layer.  e = {xmin,xmax,ymin,ymax,zmin,zmax},
 * half-open, reference coordinates. */
static void orc_face_extent(const orc_sim* s, int f, long* e) {
    e[0] = 1; e[1] = s->nx + 1; e[2] = 1; e[3] = s->ny + 1; e[4] = 1; e[5] = s->nz + 1;
    switch (f) {
        case 0: e[0] = s->nx; e[1] = s->nx + 1; break;   /* east  */
        case 1: e[0] = 1; e[1] = 2; break;               /* west  */
        case 2: e[2] = s->ny; e[3] = s->ny + 1; break;   /* north */
        case 3: e[2] = 1; e[3] = 2; break;               /* south */
        case 4: e[4] = s->nz; e[5] = s->nz + 1; break;   /* up    */
        default: e[4] = 1; e[5] = 2; break;              /* down  */
    }
}

static const float kZeroVel[3] = {0.0f, 0.0f, 0.0f};
static inline const float* orc_solid_velocity(const orc_sim* s, uint8_t v) {
    return v < 6 ? s->face_vel[v] : kZeroVel;
}

/* IEEE binary16 rounding, from the format's definition: 10 fraction bits,
 * exponent range -14..15, subnormal quantum 2^-24, round half to even. */
float orc_round_half(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    const uint32_t sign = u & 0x80000000u;
    uint32_t a = u & 0x7fffffffu;
    if (a >= 0x7f800000u) return f;                          /* inf, nan */
    if (a < 0x38800000u) {                                   /* below 2^-14: fixed quantum */
        float v;
        memcpy(&v, &a, 4);
        v = nearbyintf(v * 16777216.0f) * (1.0f / 16777216.0f);
        memcpy(&a, &v, 4);
    } else {
        a += 0x00000fffu + ((a >> 13) & 1u);                 /* round the 13 dropped bits */
        a &= ~0x00001fffu;
        if (a >= 0x47800000u) a = 0x7f800000u;               /* beyond 65504: inf */
    }
    a |= sign;
    float r;
    memcpy(&r, &a, 4);
    return r;
}

float orc_store_half(float d) { return orc_round_half(d * 4096.0f) * (1.0f / 4096.0f); }

/* ---- two instantiations ----------------------------------------------------- */
#define R float
#define FN(x) x##_f
#define ORC_IS_DOUBLE 0
#include "lbm_oracle_impl.h"
#undef R
#undef FN
#undef ORC_IS_DOUBLE
#define R double
#define FN(x) x##_d
#define ORC_IS_DOUBLE 1
#include "lbm_oracle_impl.h"
#undef R
#undef FN
#undef ORC_IS_DOUBLE

/* ---- API ------------------------------------------------------------------- */
void orc_set_threads(int n) {
#if defined(_OPENMP)
    omp_set_num_threads(n > 0 ? n : 1);
#else
    (void)n;
#endif
}

int orc_max_threads(void) {
#if defined(_OPENMP)
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Marks wall layers (and, in NATIVE mode, their velocities) in s->solid. */
static void orc_mark_walls(orc_sim* s) {
    for (int f = 0; f < 6; ++f) {
        if (s->face_type[f] != ORC_FACE_NOSLIP) continue;
        long e[6];
        orc_face_extent(s, f, e);
        for (long z = e[4]; z < e[5]; ++z)
            for (long y = e[2]; y < e[3]; ++y)
                for (long x = e[0]; x < e[1]; ++x) {
                    const size_t i = ((size_t)z * s->Y + y) * s->X + x;
                    s->solid[i] = 1;
                    s->solid_vel[i] = (uint8_t)f;   /* later faces win */
                }
    }
}

orc_sim* orc_create(int q, long nx, long ny, long nz, float nu, float rho0,
                    const float* u0, const float* force, float rho_solid,
                    const int* face_type, const int* face_has_vel,
                    const float* face_vel, int mode, int arith, int precision) {
    if (nx < 1 || ny < 1 || nz < 1) return NULL;   /* src/Field.hpp:28-31 */
    if (mode != ORC_MODE_REFERENCE && mode != ORC_MODE_NATIVE) return NULL;
    orc_sim* s = (orc_sim*)calloc(1, sizeof(orc_sim));
    if (!s) return NULL;
    int32_t c[27 * 3];
    if (!orc_model_tables(q, c, s->w, s->rev, &s->cs2)) { free(s); return NULL; }
    for (int k = 0; k < q; ++k) {
        for (int i = 0; i < 3; ++i) s->c[k][i] = c[3 * k + i];
        s->wd[k] = weight_exact(q, abs(c[3 * k]) + abs(c[3 * k + 1]) + abs(c[3 * k + 2]));
    }
    s->q = q;
    s->nx = nx; s->ny = ny; s->nz = nz;
    s->X = nx + 2; s->Y = ny + 2; s->Z = nz + 2;
    s->cs2inv = 1.0f / s->cs2;                       /* src/Boundary.cpp:27 */
    s->nu = nu; s->rho0 = rho0; s->rho_solid = rho_solid;
    for (int i = 0; i < 3; ++i) { s->u0[i] = u0[i]; s->force[i] = force[i]; }
    /* src/CollisionSRT.cpp:19-20 */
    {
        const float three_nu = 3.0f * nu;
        s->tau = three_nu + 0.5f;
        s->omega = (float)(1. / (double)s->tau);
    }
    for (int f = 0; f < 6; ++f) {
        s->face_type[f] = face_type[f];
        s->face_has_vel[f] = face_has_vel[f];
        for (int i = 0; i < 3; ++i) s->face_vel[f][i] = face_has_vel[f] ? face_vel[3 * f + i] : 0.0f;
        /* src/Boundary.cpp:197: a no-slip face needs a velocity entry */
        if (face_type[f] == ORC_FACE_NOSLIP && !face_has_vel[f]) { free(s); return NULL; }
    }
    s->mode = mode; s->arith = arith; s->precision = precision;
    if (mode == ORC_MODE_NATIVE) {
        /* each axis the lattice moves along must be periodic on both faces
         * or walled on both faces */
        for (int a = 0; a < 3; ++a) {
            int moves = 0;
            for (int k = 0; k < q; ++k) moves |= s->c[k][a] != 0;
            const int t0 = face_type[2 * a], t1 = face_type[2 * a + 1];
            s->wrap[a] = t0 == ORC_FACE_PERIODIC && t1 == ORC_FACE_PERIODIC;
            if (moves && !s->wrap[a] && !(t0 == ORC_FACE_NOSLIP && t1 == ORC_FACE_NOSLIP)) {
                free(s); return NULL;
            }
        }
    }
    const size_t cells = (size_t)s->X * s->Y * s->Z;
    const size_t rs = precision ? sizeof(double) : sizeof(float);
    s->n = calloc(cells * q, rs);
    s->ntmp = calloc(cells * q, rs);
    s->rho = calloc(cells, rs);
    s->u = calloc(cells * 3, rs);
    s->solid = (uint8_t*)calloc(cells, 1);
    s->solid_vel = (uint8_t*)calloc(cells, 1);
    s->drho = (float*)calloc(cells, sizeof(float));
    if (!s->n || !s->ntmp || !s->rho || !s->u || !s->solid || !s->solid_vel || !s->drho) {
        orc_destroy(s);
        return NULL;
    }
    orc_mark_walls(s);
    return s;
}

void orc_destroy(orc_sim* s) {
    if (!s) return;
    free(s->n); free(s->ntmp); free(s->rho); free(s->u);
    free(s->solid); free(s->solid_vel); free(s->drho);
    free(s);
}

int orc_set_trt(orc_sim* s, float magic) {
    if (!(s->tau > 0.5f)) return -1;
    if (s->precision == 0 && s->arith != ORC_ARITH_FP32 && !orc_dev(s)) return -1;
    const double lam = magic > 0.0f ? (double)magic : 3.0 / 16.0;
    const double tau_m = lam / ((double)s->tau - 0.5) + 0.5;
    s->trt = 1;
    s->omega_m_d = 1.0 / tau_m;
    s->omega_m = (float)s->omega_m_d;
    return 0;
}

int orc_set_mask(orc_sim* s, const uint8_t* mask) {
    if (s->mode != ORC_MODE_NATIVE) return -1;
    for (long z = 1; z <= s->nz; ++z)
        for (long y = 1; y <= s->ny; ++y)
            for (long x = 1; x <= s->nx; ++x) {
                const size_t i = ((size_t)z * s->Y + y) * s->X + x;
                const size_t m = ((size_t)(z - 1) * s->ny + (y - 1)) * s->nx + (x - 1);
                s->solid[i] = 0;
                s->solid_vel[i] = 0;
                if (mask[m]) { s->solid[i] = 1; s->solid_vel[i] = 6; }
            }
    orc_mark_walls(s);
    return 0;
}

#define ORC_DISPATCH(name) \
    void orc_##name(orc_sim* s) { if (s->precision) name##_d(s); else name##_f(s); }
ORC_DISPATCH(collide)
ORC_DISPATCH(stream)
ORC_DISPATCH(noslip)
ORC_DISPATCH(periodic)
ORC_DISPATCH(moments)
ORC_DISPATCH(reset)
ORC_DISPATCH(quantize)

void orc_initialize(orc_sim* s) {       /* PLBPD::initialize (src/PLBPD.cpp:16-19) */
    if (s->precision) init_fields_d(s); else init_fields_f(s);
    orc_reset(s);
}

void orc_step(orc_sim* s, long nsteps) {  /* src/PLBPD.cpp:23-30 */
    for (long t = 0; t < nsteps; ++t) {
        orc_collide(s);
        orc_stream(s);
        orc_noslip(s);
        orc_quantize(s);
        orc_periodic(s);
        orc_moments(s);
        orc_reset(s);
    }
}

size_t orc_field_len(const orc_sim* s, int which) {
    const size_t cells = (size_t)s->X * s->Y * s->Z;
    switch (which) {
        case ORC_N: case ORC_NTMP: return cells * s->q;
        case ORC_RHO: return cells;
        case ORC_U: return cells * 3;
        default: return 0;
    }
}

static void* orc_field_ptr(const orc_sim* s, int which) {
    switch (which) {
        case ORC_N: return s->n;
        case ORC_NTMP: return s->ntmp;
        case ORC_RHO: return s->rho;
        case ORC_U: return s->u;
        default: return NULL;
    }
}

static int orc_dev_pop(const orc_sim* s, int which) {
    return !s->precision && orc_dev(s) && (which == ORC_N || which == ORC_NTMP);
}

void orc_get_field(const orc_sim* s, int which, float* out) {
    const size_t len = orc_field_len(s, which);
    const void* p = orc_field_ptr(s, which);
    if (orc_dev_pop(s, which)) {   /* populations are w + d */
        const float* d = (const float*)p;
        for (size_t i = 0; i < len; ++i) out[i] = d[i] + s->w[i % (size_t)s->q];
        return;
    }
    if (s->precision) {
        const double* d = (const double*)p;
        for (size_t i = 0; i < len; ++i) out[i] = (float)d[i];
    } else {
        memcpy(out, p, len * sizeof(float));
    }
}

void orc_set_field(orc_sim* s, int which, const float* in) {
    const size_t len = orc_field_len(s, which);
    void* p = orc_field_ptr(s, which);
    if (orc_dev_pop(s, which)) {
        float* d = (float*)p;
        for (size_t i = 0; i < len; ++i) {
            const float v = in[i] - s->w[i % (size_t)s->q];
            d[i] = s->arith == ORC_ARITH_FP16DEV ? orc_store_half(v) : v;
        }
        return;
    }
    if (!s->precision && which == ORC_RHO)
        for (size_t i = 0; i < len; ++i) s->drho[i] = in[i] - 1.0f;
    if (s->precision) {
        double* d = (double*)p;
        for (size_t i = 0; i < len; ++i) d[i] = (double)in[i];
    } else {
        memcpy(p, in, len * sizeof(float));
    }
}

void orc_get_field_f64(const orc_sim* s, int which, double* out) {
    const size_t len = orc_field_len(s, which);
    const void* p = orc_field_ptr(s, which);
    if (s->precision) {
        memcpy(out, p, len * sizeof(double));
    } else {
        const float* f = (const float*)p;
        for (size_t i = 0; i < len; ++i) out[i] = (double)f[i];
    }
}

void orc_set_field_f64(orc_sim* s, int which, const double* in) {
    const size_t len = orc_field_len(s, which);
    void* p = orc_field_ptr(s, which);
    if (s->precision) {
        memcpy(p, in, len * sizeof(double));
    } else {
        float* f = (float*)p;
        for (size_t i = 0; i < len; ++i) f[i] = (float)in[i];
    }
}

void orc_relaxation(const orc_sim* s, float* tau, float* omega) {
    *tau = s->tau;
    *omega = s->omega;
}

void orc_conservation(const orc_sim* s, double* out) {
    if (s->precision) conservation_d(s, out); else conservation_f(s, out);
}
