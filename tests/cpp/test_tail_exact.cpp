// Checks plb::tx::tail_update (plbpd_gb300/csrc/tail_exact.h), the FP32
// evaluation of the double-precision tail of plbpd's AVX2 collision kernel,
// against that tail written as the reference writes it
// (src/CollisionSRT.cpp:144-147), bit for bit.
//
//   test_tail_exact <samples> <seed>
//
// Input families: lattice-like nodes (velocities up to 0.1, densities near 1,
// every D3Q27 weight, tau from 0.5 to 3, populations near equilibrium); nodes
// with random exponents (tiny, huge and subnormal operands); special values
// (zeros of both signs, NaN, infinities); and nodes at rest.  Prints the
// number of mismatches, the number of evaluations that took the FP64 form,
// and how many decided evaluations lay within 2^-12 of a float spacing of a
// rounding boundary.  Build with -ffp-contract=off.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>

#include "../../plbpd_gb300/csrc/tail_exact.h"

static uint64_t g_state;
static uint64_t next_u64() {  // splitmix64
    uint64_t z = (g_state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double unif() { return (double)(next_u64() >> 11) * 0x1p-53; }
static float unif_f(float lo, float hi) { return (float)(lo + (hi - lo) * unif()); }
static float rand_exp_float(int emin, int emax) {
    const int e = emin + (int)(next_u64() % (uint64_t)(emax - emin + 1));
    float m = (float)(1.0 + unif());
    float v = std::ldexp(m, e);
    return (next_u64() & 1) ? -v : v;
}

// The reference's statement with its types: float weights, density, omega
// and population; the bracket and the sum in double.
static float reference_tail(float w, float rho, float cu, float usq, float omega, float n) {
    const double neq = w * rho * (1.0 + 3.0 * cu + 4.5 * cu * cu - 1.5 * usq);
    return (1.0f - omega) * n + omega * neq;
}

static uint32_t fbits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}

// Distance of the double x from the nearest float rounding boundary, in units
// of the float spacing there (0.5 means x is a float).
static double boundary_distance(float w, float rho, float cu, float usq, float omega, float n) {
    const double neq = w * rho * (1.0 + 3.0 * cu + 4.5 * cu * cu - 1.5 * usq);
    const double x = (double)((1.0f - omega) * n) + omega * neq;
    if (!std::isfinite(x) || x == 0.0) return 1.0;
    const float f = (float)x;
    const float up = std::nextafter(f, std::numeric_limits<float>::infinity());
    const float dn = std::nextafter(f, -std::numeric_limits<float>::infinity());
    const double gap_up = (double)up - (double)f, gap_dn = (double)f - (double)dn;
    const double d = x - (double)f;  // |d| <= half the spacing on its side
    return d >= 0 ? 0.5 - d / gap_up : 0.5 + d / gap_dn;
}

int main(int argc, char** argv) {
    const long long samples = argc > 1 ? atoll(argv[1]) : 1000000;
    g_state = argc > 2 ? strtoull(argv[2], nullptr, 10) : 20261203ull;
    const float weights[] = {8.f / 27.f, 2.f / 27.f, 1.f / 54.f, 1.f / 216.f, 1.f / 3.f, 1.f / 18.f, 1.f / 36.f,
                             4.f / 9.f, 1.f / 9.f};
    const float inf = std::numeric_limits<float>::infinity(), nan = std::numeric_limits<float>::quiet_NaN();
    long long mismatches = 0, fp64_evals = 0, near = 0, fp64_mismatch = 0;
    for (long long i = 0; i < samples; ++i) {
        const int family = (int)(i % 16);
        float w, rho, cu, usq, omega, n;
        if (family < 12) {  // lattice-like node
            const float scale = (family < 6) ? 0.1f : (family < 10 ? 0.02f : 1e-4f);
            const float ux = unif_f(-scale, scale), uy = unif_f(-scale, scale), uz = unif_f(-scale, scale);
            usq = (ux * ux + uy * uy) + uz * uz;
            const int k = (int)(next_u64() % 7);
            cu = (k == 0) ? ux : (k == 1) ? ux + uy : (k == 2) ? (ux - uy) + uz : (k == 3) ? -uy - uz
                : (k == 4) ? uz : (k == 5) ? -ux + uz : (ux + uy) - uz;
            w = weights[next_u64() % 9];
            rho = unif_f(0.7f, 1.3f);
            const float tau = unif_f(0.5001f, 3.0f);
            omega = (float)(1. / tau);
            const float eq = w * rho;
            n = (family == 11) ? eq : eq * (1.0f + unif_f(-0.3f, 0.3f));
            if (family == 11) { cu = 0.0f; usq = 0.0f; }  // at rest
        } else if (family < 15) {  // random exponents
            cu = (next_u64() & 7) ? rand_exp_float(-140, -2) : 0.0f;
            if (std::fabs(cu) > 0.17f) cu = 0.17f;
            usq = (next_u64() & 7) ? std::fabs(rand_exp_float(-149, -7)) : 0.0f;
            w = weights[next_u64() % 9];
            rho = rand_exp_float(-70, 60);
            omega = rand_exp_float(-12, 3);
            n = rand_exp_float(-149, 60);
        } else {  // special values
            const float specials[] = {0.0f, -0.0f, inf, -inf, nan, 1e-45f, -1e-45f, 3.4e38f, 1.0f, 0.5f};
            cu = specials[next_u64() % 10] * ((next_u64() & 1) ? 1.0f : 1e-3f);
            usq = std::fabs(specials[next_u64() % 10]);
            w = weights[next_u64() % 9];
            rho = specials[next_u64() % 10];
            omega = (next_u64() & 1) ? specials[next_u64() % 10] : 1.6f;
            n = specials[next_u64() % 10];
        }
        const float ref = reference_tail(w, rho, cu, usq, omega, n);
        const float wr = w * rho;
        const float a = (1.0f - omega) * n;
        const plb::tx::TailNode nd = plb::tx::tail_node(usq);
        float fast;
        const bool decided = plb::tx::tail_fast(cu, nd, wr, omega, a, &fast);
        const float got = decided ? fast : plb::tx::tail_fp64(cu, usq, wr, omega, a);
        const float slow = plb::tx::tail_fp64(cu, usq, wr, omega, a);
        const bool ref_nan = std::isnan(ref);
        if (ref_nan ? !std::isnan(got) : fbits(got) != fbits(ref)) {
            if (++mismatches <= 10)
                std::printf("mismatch: w=%a rho=%a cu=%a usq=%a omega=%a n=%a ref=%a got=%a decided=%d\n", w, rho, cu,
                            usq, omega, n, ref, got, (int)decided);
        }
        if (ref_nan ? !std::isnan(slow) : fbits(slow) != fbits(ref)) ++fp64_mismatch;
        if (!decided) ++fp64_evals;
        else if (boundary_distance(w, rho, cu, usq, omega, n) < 0x1p-12) ++near;
    }
    std::printf("samples %lld mismatches %lld fp64_mismatches %lld fp64_evals %lld near_boundary_decided %lld\n",
                samples, mismatches, fp64_mismatch, fp64_evals, near);
    return mismatches == 0 && fp64_mismatch == 0 ? 0 : 1;
}
