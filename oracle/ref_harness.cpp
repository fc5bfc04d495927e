// C entry points over the reference plbpd classes, compiled together with the
// reference sources (see oracle/Makefile) into oracle/_ref/libplbpd_ref*.so.
//
// Oracle-only test infrastructure: the parity tests and the CPU-baseline leg
// of bench.py load this library to run the reference's own code.  It never
// ships in, or links into, the product library.
//
// Reference interfaces driven here (paths inside the plbpd project):
//   LBModel(name)                                src/LBModel.cpp:8-19
//   Domain(model, x, y, z, nu, rho, u0, F)       src/Domain.cpp:13-22
//   Boundary(model, domain, rho_s, types, vels)  src/Boundary.cpp:20-32
//   SimData(dims(x,y,z), Q)                      src/SimData.cpp:22-30
//   PLBPD::initialize / march_in_time            src/PLBPD.cpp:16-33
//   LBDynamics::collide / stream                 src/LBDynamics.cpp:12-21
//   Boundary::apply_noslip / apply_periodicity / reset   src/Boundary.cpp:58-111
//   CalcMoments::operator()                      src/CalcMoments.hpp:47-73
#include <array>
#include <cstring>
#include <memory>
#include <string>
#include <tuple>
#if defined(_OPENMP)
#include <omp.h>
#endif

#include "Boundary.hpp"
#include "CalcMoments.hpp"
#include "Domain.hpp"
#include "LBDynamics.hpp"
#include "LBModel.hpp"
#include "PLBPD.hpp"
#include "EqlbDist.hpp"
#include "SimData.hpp"

namespace {

const char* kFaceNames[6] = {"east", "west", "north", "south", "up", "down"};

struct RefSim {
    std::unique_ptr<LBModel> model;
    std::unique_ptr<Domain> domain;
    std::unique_ptr<Boundary> boundary;
    std::unique_ptr<SimData> sim;
    std::unique_ptr<PLBPD> plbpd;
    std::unique_ptr<LBDynamics> dyn;
    std::unique_ptr<CalcMoments> moments;
    size_t nx, ny, nz, q;
};

Field::VectorField<float, 1>* field_of(RefSim* s, int which) {
    switch (which) {
        case 0: return s->sim->n;
        case 1: return s->sim->ntmp;
        case 2: return s->sim->rho;
        case 3: return s->sim->u;
        default: return nullptr;
    }
}

size_t field_len(RefSim* s, int which) {
    const size_t cells = (s->nx + 2) * (s->ny + 2) * (s->nz + 2);
    switch (which) {
        case 0: case 1: return cells * s->q;
        case 2: return cells;
        case 3: return cells * 3;
        default: return 0;
    }
}

}  // namespace

extern "C" {

// face_type[f]: 0 = not given, 1 = "periodic", 2 = "noslip"  (order E,W,N,S,up,down)
// face_has_vel[f] != 0 adds face_vel[3f..3f+2] to the BoundaryVelocity map.
void* refh_create(const char* model, size_t nx, size_t ny, size_t nz,
                  float nu, float rho0, const float* u0, const float* force,
                  float rho_solid, const int* face_type,
                  const int* face_has_vel, const float* face_vel) {
    auto s = new RefSim();
    s->nx = nx; s->ny = ny; s->nz = nz;
    s->model = std::make_unique<LBModel>(std::string(model));
    s->q = s->model->get_num_directions();
    std::array<float, 3> u0a = {u0[0], u0[1], u0[2]};
    std::array<float, 3> fa = {force[0], force[1], force[2]};
    s->domain = std::make_unique<Domain>(s->model.get(), nx, ny, nz, nu, rho0, u0a, fa);
    BoundaryType types;
    BoundaryVelocity vels;
    for (int f = 0; f < 6; ++f) {
        if (face_type[f] == 1) types[kFaceNames[f]] = "periodic";
        if (face_type[f] == 2) types[kFaceNames[f]] = "noslip";
        if (face_has_vel[f])
            vels[kFaceNames[f]] = {face_vel[3 * f], face_vel[3 * f + 1], face_vel[3 * f + 2]};
    }
    s->boundary = std::make_unique<Boundary>(s->model.get(), s->domain.get(),
                                             rho_solid, types, vels);
    s->sim = std::make_unique<SimData>(s->domain->get_dimensions(), s->q);
    s->plbpd = std::make_unique<PLBPD>(s->model.get(), s->domain.get(), s->boundary.get());
    s->dyn = std::make_unique<LBDynamics>(s->model.get(), s->domain.get());
    s->moments = std::make_unique<CalcMoments>(s->model.get());
    return s;
}

void refh_destroy(void* h) { delete static_cast<RefSim*>(h); }

void refh_set_threads(int n) {
#if defined(_OPENMP)
    omp_set_num_threads(n > 0 ? n : 1);
#else
    (void)n;
#endif
}

int refh_max_threads(void) {
#if defined(_OPENMP)
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void refh_initialize(void* h) {
    auto s = static_cast<RefSim*>(h);
    s->plbpd->initialize(*s->sim);
}

// PLBPD::march_in_time: the reference's own timed loop (it prints one line).
void refh_march(void* h, size_t nsteps) {
    auto s = static_cast<RefSim*>(h);
    s->plbpd->march_in_time(nsteps, *s->sim);
}

// The same six phases called one by one; `reference` selects the serial
// collision/streaming kernels (CollisionSRT.cpp:36-46, Streaming.cpp:76-83).
void refh_collide(void* h, int reference) {
    auto s = static_cast<RefSim*>(h);
    s->dyn->collide(*s->sim, reference != 0);
}
void refh_stream(void* h, int reference) {
    auto s = static_cast<RefSim*>(h);
    s->dyn->stream(*s->sim, "push", reference != 0);
}
void refh_noslip(void* h) {
    auto s = static_cast<RefSim*>(h);
    s->boundary->apply_noslip(*s->sim);
}
void refh_periodic(void* h) {
    auto s = static_cast<RefSim*>(h);
    s->boundary->apply_periodicity(*s->sim);
}
void refh_moments(void* h) {
    auto s = static_cast<RefSim*>(h);
    (*s->moments)(*s->sim);
}
void refh_reset(void* h) {
    auto s = static_cast<RefSim*>(h);
    s->boundary->reset(*s->sim);
}

// which: 0 = n, 1 = ntmp, 2 = rho, 3 = u.  Layout is the reference's own:
// AoS with one halo layer, index ((z*(Y+2)+y)*(X+2)+x)*V + v.
size_t refh_field_len(void* h, int which) {
    return field_len(static_cast<RefSim*>(h), which);
}
void refh_get_field(void* h, int which, float* out) {
    auto s = static_cast<RefSim*>(h);
    auto f = field_of(s, which);
    std::memcpy(out, f->get(0, 0, 0, 0), field_len(s, which) * sizeof(float));
}
void refh_set_field(void* h, int which, const float* in) {
    auto s = static_cast<RefSim*>(h);
    auto f = field_of(s, which);
    std::memcpy(f->get(0, 0, 0, 0), in, field_len(s, which) * sizeof(float));
}

// EqlbDist on one node (src/EqlbDist.hpp:26-38).
void refh_eqlb(const char* model, float rho, const float* u, float* out) {
    LBModel m{std::string(model)};
    std::vector<float> nl(m.get_num_directions(), 0.0f);
    EqlbDist e(&m);
    std::array<float, 3> ua = {u[0], u[1], u[2]};
    e(rho, ua, nl);
    std::memcpy(out, nl.data(), nl.size() * sizeof(float));
}

// LBModel tables (src/LBModel.cpp:23-165).
int refh_model_tables(const char* model, int* c, float* w, unsigned* rev, float* cs2) {
    LBModel m{std::string(model)};
    const int q = static_cast<int>(m.get_num_directions());
    for (int k = 0; k < q; ++k) {
        for (int i = 0; i < 3; ++i) c[3 * k + i] = m.get_directional_velocities()[k][i];
        w[k] = m.get_directional_weights()[k];
        rev[k] = m.get_reverse()[k];
    }
    *cs2 = m.get_speed_of_sound_squared();
    return q;
}

}  // extern "C"
