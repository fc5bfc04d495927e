/*
 * Precision-generic body of the oracle (included twice by lbm_oracle.c with
 * R = float / double and FN(x) = x##_f / x##_d).  Test infrastructure only.
 *
 * Every loop restates one reference operator; the citations are paths inside
 * the plbpd project.  Loops whose order is observable (no-slip, periodic
 * copies) run serially in the reference's loop order; the others may run on
 * OpenMP threads because each output slot is written exactly once.
 */

/* ---- collision, one node ------------------------------------------------ */
/* CollisionSRT::_get_updated_u (src/CollisionSRT.cpp:71-81), _get_cu (:83-91),
 * _collision_kernel_avx2 (:93-148), _collision_kernel (:151-176). */
static void FN(collide_node)(const orc_sim* s, R* nl, R rho, const R* ul, R drho) {
    const int q = s->q;
#if ORC_IS_DOUBLE
    (void)drho;
    const double tau = (double)s->tau;
    const double omega = 1.0 / tau;
    const double trho = tau / rho;
    double uu[3];
    for (int i = 0; i < 3; ++i) uu[i] = ul[i] + (double)s->force[i] * trho;
    const double usq = uu[0] * uu[0] + uu[1] * uu[1] + uu[2] * uu[2];
    if (s->trt) {
        /* TRT with a second-order force source; pairs (k, k + 1), k odd
         * (every table lists a velocity next to its opposite) */
        const double omm = s->omega_m_d;
        const double gp = 1.0 - 0.5 * omega, gm = 1.0 - 0.5 * omm;
        const double hr = 0.5 / rho;
        double v[3], F[3];
        for (int i = 0; i < 3; ++i) { F[i] = (double)s->force[i]; v[i] = ul[i] + F[i] * hr; }
        const double vsq = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
        const double uF = v[0] * F[0] + v[1] * F[1] + v[2] * F[2];
        const double k15 = 1.5 * vsq, m3uF = -3.0 * uF;
        const double w0 = s->wd[0];
        const double e0 = (w0 * rho) * (1.0 - k15);
        nl[0] = (nl[0] - omega * (nl[0] - e0)) + (gp * w0) * m3uF;
        for (int k = 1; k < q; k += 2) {
            const double w = s->wd[k];
            const double cu = s->c[k][0] * v[0] + s->c[k][1] * v[1] + s->c[k][2] * v[2];
            const double cF = s->c[k][0] * F[0] + s->c[k][1] * F[1] + s->c[k][2] * F[2];
            const double wr = w * rho;
            const double ep = wr * ((1.0 + (4.5 * cu) * cu) - k15);
            const double em = wr * (3.0 * cu);
            const double sp = 0.5 * (nl[k] + nl[k + 1]);
            const double sm = 0.5 * (nl[k] - nl[k + 1]);
            const double a = omega * (sp - ep);
            const double b = omm * (sm - em);
            const double Sp = (gp * w) * ((9.0 * cu) * cF + m3uF);
            const double Sm = (gm * w) * (3.0 * cF);
            nl[k] = ((nl[k] - a) - b) + (Sp + Sm);
            nl[k + 1] = ((nl[k + 1] - a) + b) + (Sp - Sm);
        }
        return;
    }
    for (int k = 0; k < q; ++k) {
        const double cu = s->c[k][0] * uu[0] + s->c[k][1] * uu[1] + s->c[k][2] * uu[2];
        const double neq = s->wd[k] * rho *
                           (1.0 + 3.0 * cu + 4.5 * cu * cu - 1.5 * usq);
        nl[k] = (1.0 - omega) * nl[k] + omega * neq;
    }
#else
    const float tau = s->tau, omega = s->omega;
    /* the deviation form (FP16/FP32 deviation storage) takes tau (1/rho), one
     * reciprocal shared with the moments; plbpd's FP32 forms take tau/rho */
    const float tau_rhoinv = (orc_dev(s) && !s->trt) ? tau * (1.0f / rho) : tau / rho;
    float uu[3];
    for (int i = 0; i < 3; ++i) uu[i] = ul[i] + s->force[i] * tau_rhoinv;
    const float usq = uu[0] * uu[0] + uu[1] * uu[1] + uu[2] * uu[2];
    float cu[27];
    cu[0] = 0.0f;
    for (int k = 1; k < q; ++k)
        cu[k] = (float)s->c[k][0] * uu[0] + (float)s->c[k][1] * uu[1] +
                (float)s->c[k][2] * uu[2];
    if (s->trt) {
        /* TRT with a second-order force source; pairs (k, k + 1), k odd.
         * FP16DEV works on deviations d = f - w: e+ - w = w (drho + rho (4.5cu^2 - 1.5usq)) */
        const int dev = orc_dev(s);
        const float omm = s->omega_m;
        const float gp = 1.0f - 0.5f * omega, gm = 1.0f - 0.5f * omm;
        const float hr = 0.5f / rho;
        float v[3];
        for (int i = 0; i < 3; ++i) v[i] = ul[i] + s->force[i] * hr;
        const float vsq = (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2];
        const float uF = (v[0] * s->force[0] + v[1] * s->force[1]) + v[2] * s->force[2];
        const float kusq = -1.5f * vsq, base = 1.0f + kusq, m3uF = -3.0f * uF;
        const float w0 = s->w[0], wr0 = w0 * rho;
        const float e0 = dev ? fmaf(wr0, kusq, w0 * drho) : wr0 * base;
        nl[0] = (nl[0] - omega * (nl[0] - e0)) + (gp * w0) * m3uF;
        for (int k = 1; k < q; k += 2) {
            const float w = s->w[k], wr = w * rho;
            const float cuk = (float)s->c[k][0] * v[0] + (float)s->c[k][1] * v[1] + (float)s->c[k][2] * v[2];
            const float cF = (float)s->c[k][0] * s->force[0] + (float)s->c[k][1] * s->force[1] +
                             (float)s->c[k][2] * s->force[2];
            const float t = 4.5f * cuk;
            const float ep = dev ? fmaf(wr, fmaf(t, cuk, kusq), w * drho) : wr * fmaf(t, cuk, base);
            const float em = wr * (3.0f * cuk);
            const float sp = 0.5f * (nl[k] + nl[k + 1]);
            const float sm = 0.5f * (nl[k] - nl[k + 1]);
            const float a = omega * (sp - ep);
            const float b = omm * (sm - em);
            const float Sp = (gp * w) * fmaf(9.0f * cuk, cF, m3uF);
            const float Sm = (gm * w) * (3.0f * cF);
            nl[k] = ((nl[k] - a) - b) + (Sp + Sm);
            nl[k + 1] = ((nl[k + 1] - a) + b) + (Sp - Sm);
        }
        return;
    }
    if (orc_dev(s)) {
        /* deviation form: nl holds d = f - w;
         * X = 3cu + 4.5cu^2 - 1.5usq, d' = (1-omega) d + w (omega rho X + omega drho) */
        const float kusq16 = -1.5f * usq;
        const float orho = omega * rho;
        const float odrho = omega * drho;
        for (int k = 0; k < q; ++k) {
            const float A = s->w[k] * orho;
            const float B = s->w[k] * odrho;
            const float X = fmaf(cu[k], fmaf(4.5f, cu[k], 3.0f), kusq16);
            nl[k] = fmaf(1.0f - omega, nl[k], fmaf(A, X, B));
        }
        return;
    }
    int nbody;
    if (s->arith == ORC_ARITH_AVX2) nbody = (q / 8) * 8;
    else if (s->arith == ORC_ARITH_FP32) nbody = q;
    else nbody = 0;
    const float kusq = -1.5f * usq;
    const float omc = 1.0f - omega;
    for (int k = 0; k < nbody; ++k) {           /* 8-wide FP32 body */
        const float cusq = cu[k] * cu[k];
        float neq = fmaf(3.0f, cu[k], 1.0f);
        neq = fmaf(4.5f, cusq, neq);
        neq = neq + kusq;
        neq = neq * rho;
        neq = neq * s->w[k];
        nl[k] = fmaf(omc, nl[k], omega * neq);
    }
    for (int k = nbody; k < q; ++k) {           /* FP64 bracket */
        const float wr = s->w[k] * rho;
        const double cud = (double)cu[k];
        const double neq = (double)wr *
            (1.0 + 3.0 * cud + 4.5 * cud * cud - 1.5 * (double)usq);
        const float a = omc * nl[k];
        nl[k] = (float)((double)a + (double)omega * neq);
    }
#endif
}

/* ---- helpers -------------------------------------------------------------- */
static inline size_t FN(node)(const orc_sim* s, long z, long y, long x) {
    return ((size_t)z * (size_t)s->Y + (size_t)y) * (size_t)s->X + (size_t)x;
}

/* ---- operators ------------------------------------------------------------ */

/* CollisionSRT::_collision_tbb (src/CollisionSRT.cpp:49-69): in place on n over
 * the interior, wall layers included, with the current rho and u fields. */
static void FN(collide)(orc_sim* s) {
    R* n = (R*)s->n;
    const R* rho = (const R*)s->rho;
    const R* u = (const R*)s->u;
    const float* drho = s->drho;
    const int q = s->q;
#pragma omp parallel for schedule(static)
    for (long z = 1; z <= s->nz; ++z)
        for (long y = 1; y <= s->ny; ++y)
            for (long x = 1; x <= s->nx; ++x) {
                const size_t i = FN(node)(s, z, y, x);
                if (s->mode == ORC_MODE_NATIVE && s->solid[i]) continue;
                FN(collide_node)(s, n + i * q, rho[i], u + 3 * i, (R)drho[i]);
            }
}

/* FP16 storage: every fluid population rounds to the stored binary16 value
 * (orc_store_half) once per step, after the bounce-back writes (the engine
 * rounds when it stores). */
static void FN(quantize)(orc_sim* s) {
#if ORC_IS_DOUBLE
    (void)s;
#else
    if (s->arith != ORC_ARITH_FP16DEV) return;
    float* n = (float*)s->n;
    const int q = s->q;
#pragma omp parallel for schedule(static)
    for (long z = 1; z <= s->nz; ++z)
        for (long y = 1; y <= s->ny; ++y)
            for (long x = 1; x <= s->nx; ++x) {
                const size_t i = FN(node)(s, z, y, x);
                if (s->solid[i]) continue;
                for (int k = 0; k < q; ++k) n[i * q + k] = orc_store_half(n[i * q + k]);
            }
#endif
}

/* Streaming::_push_kernel / _push_tbb (src/Streaming.cpp:62-94):
 * ntmp[node + c_k][k] = n[node][k] for every interior node and every k, then
 * the two buffers swap.  NATIVE mode pushes from fluid nodes only and wraps
 * periodic axes. */
static void FN(stream)(orc_sim* s) {
    const R* n = (const R*)s->n;
    R* nt = (R*)s->ntmp;
    const int q = s->q;
    const int native = s->mode == ORC_MODE_NATIVE;
#pragma omp parallel for schedule(static)
    for (long z = 1; z <= s->nz; ++z)
        for (long y = 1; y <= s->ny; ++y)
            for (long x = 1; x <= s->nx; ++x) {
                const size_t i = FN(node)(s, z, y, x);
                if (native && s->solid[i]) continue;
                for (int k = 0; k < q; ++k) {
                    long zz = z + s->c[k][2], yy = y + s->c[k][1], xx = x + s->c[k][0];
                    if (native) {
                        zz = orc_wrap(zz, s->nz, s->wrap[2]);
                        yy = orc_wrap(yy, s->ny, s->wrap[1]);
                        xx = orc_wrap(xx, s->nx, s->wrap[0]);
                    }
                    nt[FN(node)(s, zz, yy, xx) * q + k] = n[i * q + k];
                }
            }
    void* t = s->n; s->n = s->ntmp; s->ntmp = t;
}

/* Boundary::_apply_noslip (src/Boundary.cpp:189-221), faces in the order
 * east, west, north, south, up, down (:17-18,101-111), each face's wall nodes
 * visited in serial (z, y, x, kp) order:
 *   n[W + c_kp][kp] = n[W][k] - 2 w_k rho[W + c_kp] (c_k . u_b) / c_s^2,  k = rev(kp).
 * NATIVE mode: the same rule for every solid node S whose neighbour S + c_kp
 * (wrapped) is a fluid node; u_b is the velocity of the wall the node belongs
 * to, zero for obstacles. */
static void FN(noslip)(orc_sim* s) {
    R* n = (R*)s->n;
    const R* rho = (const R*)s->rho;
    const int q = s->q;
    if (s->mode == ORC_MODE_REFERENCE) {
        for (int f = 0; f < 6; ++f) {
            if (s->face_type[f] != ORC_FACE_NOSLIP) continue;
            long e[6];
            orc_face_extent(s, f, e);
            const float* ub = s->face_vel[f];
            for (long z = e[4]; z < e[5]; ++z)
                for (long y = e[2]; y < e[3]; ++y)
                    for (long x = e[0]; x < e[1]; ++x)
                        for (int kp = 1; kp < q; ++kp) {
                            const long nz_ = z + s->c[kp][2], ny_ = y + s->c[kp][1],
                                       nx_ = x + s->c[kp][0];
                            const size_t nb = FN(node)(s, nz_, ny_, nx_);
                            const size_t w0 = FN(node)(s, z, y, x);
                            const int k = (int)s->rev[kp];
#if ORC_IS_DOUBLE
                            const double cu = s->c[k][0] * (double)ub[0] +
                                              s->c[k][1] * (double)ub[1] +
                                              s->c[k][2] * (double)ub[2];
                            n[nb * q + kp] = n[w0 * q + k] -
                                2.0 * s->wd[k] * rho[nb] * cu * (double)s->cs2inv;
#else
                            const float cu = (float)s->c[k][0] * ub[0] +
                                             (float)s->c[k][1] * ub[1] +
                                             (float)s->c[k][2] * ub[2];
                            n[nb * q + kp] = n[w0 * q + k] -
                                2.0f * s->w[k] * rho[nb] * cu * s->cs2inv;
#endif
                        }
        }
        return;
    }
#pragma omp parallel for schedule(static)
    for (long z = 1; z <= s->nz; ++z)
        for (long y = 1; y <= s->ny; ++y)
            for (long x = 1; x <= s->nx; ++x) {
                const size_t w0 = FN(node)(s, z, y, x);
                if (!s->solid[w0]) continue;
                const float* ub = orc_solid_velocity(s, s->solid_vel[w0]);
                for (int kp = 1; kp < q; ++kp) {
                    const long zz = orc_wrap(z + s->c[kp][2], s->nz, s->wrap[2]);
                    const long yy = orc_wrap(y + s->c[kp][1], s->ny, s->wrap[1]);
                    const long xx = orc_wrap(x + s->c[kp][0], s->nx, s->wrap[0]);
                    if (zz < 1 || zz > s->nz || yy < 1 || yy > s->ny || xx < 1 || xx > s->nx)
                        continue;
                    const size_t nb = FN(node)(s, zz, yy, xx);
                    if (s->solid[nb]) continue;
                    const int k = (int)s->rev[kp];
#if ORC_IS_DOUBLE
                    const double cu = s->c[k][0] * (double)ub[0] + s->c[k][1] * (double)ub[1] +
                                      s->c[k][2] * (double)ub[2];
                    n[nb * q + kp] = n[w0 * q + k] -
                        2.0 * s->wd[k] * rho[nb] * cu * (double)s->cs2inv;
#else
                    const float cu = (float)s->c[k][0] * ub[0] + (float)s->c[k][1] * ub[1] +
                                     (float)s->c[k][2] * ub[2];
                    n[nb * q + kp] = n[w0 * q + k] -
                        2.0f * s->w[k] * rho[nb] * cu * s->cs2inv;
#endif
                }
            }
}

/* Boundary::_apply_periodicity_east_west / _north_south
 * (src/Boundary.cpp:234-251,264-281): halo -> interior copies over interior
 * rows, rest direction excluded; no up/down periodicity exists there.
 * NATIVE mode wraps inside the push instead, so this is a no-op. */
static void FN(periodic)(orc_sim* s) {
    if (s->mode != ORC_MODE_REFERENCE) return;
    R* n = (R*)s->n;
    const int q = s->q;
    if (s->face_type[0] == ORC_FACE_PERIODIC && s->face_type[1] == ORC_FACE_PERIODIC) {
        for (long z = 1; z <= s->nz; ++z)
            for (long y = 1; y <= s->ny; ++y)
                for (int k = 1; k < q; ++k) {
                    const int ck0 = s->c[k][0];
                    if (ck0 > 0)
                        n[FN(node)(s, z, y, 1) * q + k] = n[FN(node)(s, z, y, s->nx + 1) * q + k];
                    if (ck0 < 0)
                        n[FN(node)(s, z, y, s->nx) * q + k] = n[FN(node)(s, z, y, 0) * q + k];
                }
    }
    if (s->face_type[2] == ORC_FACE_PERIODIC && s->face_type[3] == ORC_FACE_PERIODIC) {
        for (long z = 1; z <= s->nz; ++z)
            for (long x = 1; x <= s->nx; ++x)
                for (int k = 1; k < q; ++k) {
                    const int ck1 = s->c[k][1];
                    if (ck1 > 0)
                        n[FN(node)(s, z, 1, x) * q + k] = n[FN(node)(s, z, s->ny + 1, x) * q + k];
                    if (ck1 < 0)
                        n[FN(node)(s, z, s->ny, x) * q + k] = n[FN(node)(s, z, 0, x) * q + k];
                }
    }
}

/* CalcMoments::operator() / _get_local_moments (src/CalcMoments.hpp:22-37,47-73):
 * rho = sum_k n_k in k order, u_i = sum_k n_k c_ki, then u_i *= 1/rho. */
static void FN(moments)(orc_sim* s) {
    const R* n = (const R*)s->n;
    R* rho = (R*)s->rho;
    R* u = (R*)s->u;
    const int q = s->q;
#pragma omp parallel for schedule(static)
    for (long z = 1; z <= s->nz; ++z)
        for (long y = 1; y <= s->ny; ++y)
            for (long x = 1; x <= s->nx; ++x) {
                const size_t i = FN(node)(s, z, y, x);
                if (s->mode == ORC_MODE_NATIVE && s->solid[i]) continue;
                R r = 0, ux = 0, uy = 0, uz = 0;
                for (int k = 0; k < q; ++k) {
                    const R nk = n[i * q + k];
                    r += nk;
                    ux += nk * (R)s->c[k][0];
                    uy += nk * (R)s->c[k][1];
                    uz += nk * (R)s->c[k][2];
                }
#if !ORC_IS_DOUBLE
                if (orc_dev(s)) {   /* r is the density deviation */
                    s->drho[i] = r;
                    r = 1.0f + r;
                }
#endif
                const R rinv = (R)1 / r;
                rho[i] = r;
                u[3 * i + 0] = ux * rinv;
                u[3 * i + 1] = uy * rinv;
                u[3 * i + 2] = uz * rinv;
            }
}

/* Boundary::reset -> reset_velocity, reset_density (src/Boundary.cpp:58-89,
 * 150-187): u = u_b on every face with a velocity entry, then rho = rho_solid
 * on every no-slip face, faces in order.  NATIVE mode: every solid node gets
 * rho_solid and its wall velocity (zero for obstacles). */
static void FN(reset)(orc_sim* s) {
    R* rho = (R*)s->rho;
    R* u = (R*)s->u;
    if (s->mode == ORC_MODE_REFERENCE) {
        for (int f = 0; f < 6; ++f) {
            if (!s->face_has_vel[f]) continue;
            long e[6];
            orc_face_extent(s, f, e);
            for (long z = e[4]; z < e[5]; ++z)
                for (long y = e[2]; y < e[3]; ++y)
                    for (long x = e[0]; x < e[1]; ++x)
                        for (int i = 0; i < 3; ++i)
                            u[3 * FN(node)(s, z, y, x) + i] = (R)s->face_vel[f][i];
        }
        for (int f = 0; f < 6; ++f) {
            if (s->face_type[f] != ORC_FACE_NOSLIP) continue;
            long e[6];
            orc_face_extent(s, f, e);
            for (long z = e[4]; z < e[5]; ++z)
                for (long y = e[2]; y < e[3]; ++y)
                    for (long x = e[0]; x < e[1]; ++x)
                        rho[FN(node)(s, z, y, x)] = (R)s->rho_solid;
        }
        return;
    }
    for (long z = 1; z <= s->nz; ++z)
        for (long y = 1; y <= s->ny; ++y)
            for (long x = 1; x <= s->nx; ++x) {
                const size_t i = FN(node)(s, z, y, x);
                if (!s->solid[i]) continue;
                const float* ub = orc_solid_velocity(s, s->solid_vel[i]);
                rho[i] = (R)s->rho_solid;
                for (int d = 0; d < 3; ++d) u[3 * i + d] = (R)ub[d];
            }
}

/* Domain::initialize (src/Domain.cpp:46-63): rho0, u0 and EqlbDist(rho0, u0)
 * on every node, halo included; ntmp starts at zero (src/SimData.cpp:53-56). */
static void FN(init_fields)(orc_sim* s) {
    const size_t cells = (size_t)s->X * s->Y * s->Z;
    R* n = (R*)s->n;
    R* nt = (R*)s->ntmp;
    R* rho = (R*)s->rho;
    R* u = (R*)s->u;
    R feq[27];
#if ORC_IS_DOUBLE
    {
        const double ux = s->u0[0], uy = s->u0[1], uz = s->u0[2];
        const double usq = ux * ux + uy * uy + uz * uz;
        for (int k = 0; k < s->q; ++k) {
            const double cu = s->c[k][0] * ux + s->c[k][1] * uy + s->c[k][2] * uz;
            feq[k] = s->wd[k] * (double)s->rho0 *
                     (1.0 + 3.0 * cu + 4.5 * cu * cu - 1.5 * usq);
        }
    }
#else
    orc_eqlb(s->q, s->rho0, s->u0, feq);
    if (orc_dev(s))
        for (int k = 0; k < s->q; ++k) {
            feq[k] = feq[k] - s->w[k];
            if (s->arith == ORC_ARITH_FP16DEV) feq[k] = orc_store_half(feq[k]);
        }
#endif
    for (size_t i = 0; i < cells; ++i) {
        s->drho[i] = s->rho0 - 1.0f;
        rho[i] = (R)s->rho0;
        for (int d = 0; d < 3; ++d) u[3 * i + d] = (R)s->u0[d];
        for (int k = 0; k < s->q; ++k) {
            n[i * s->q + k] = feq[k];
            nt[i * s->q + k] = 0;
        }
    }
}

static void FN(conservation)(const orc_sim* s, double* out) {
    const R* n = (const R*)s->n;
    double m = 0, px = 0, py = 0, pz = 0;
    for (long z = 1; z <= s->nz; ++z)
        for (long y = 1; y <= s->ny; ++y)
            for (long x = 1; x <= s->nx; ++x) {
                const size_t i = FN(node)(s, z, y, x);
                if (s->solid[i]) continue;
                for (int k = 0; k < s->q; ++k) {
                    double v = (double)n[i * s->q + k];
                    if (orc_dev(s) && !ORC_IS_DOUBLE) v += (double)s->w[k];
                    m += v;
                    px += v * s->c[k][0];
                    py += v * s->c[k][1];
                    pz += v * s->c[k][2];
                }
            }
    out[0] = m; out[1] = px; out[2] = py; out[3] = pz;
}
