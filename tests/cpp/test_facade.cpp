// Drives plbpd's C++ classes as implemented over libplb_gb300 (include/plbpd).
//
//   test_facade cpu
//       checks that need no GPU: LBModel tables, EqlbDist known answer, Field
//       indexing (the reference's TestLBModel / TestEqlbDist / TestField /
//       TestDomain cases) and the reference's exception types; prints tables
//       and the equilibrium as JSON for the Python side to compare.
//   test_facade case <outdir> <model> nx ny nz nu rho0 u0x u0y u0z fx fy fz rho_s
//                    then 6 x (type has_vel vx vy vz), faces east..down,
//                    type 0 none / 1 periodic / 2 noslip
//       PLBPD::initialize, march_in_time to steps 1, 2, 5, 20, then one step
//       operator by operator; writes every field as raw float32.
//   test_facade preset <name> <outdir>
//       the reference's main.cpp flow on a Flow preset; writes the fields.
#include <cassert>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "Boundary.hpp"
#include "CalcMoments.hpp"
#include "CollisionTRT.hpp"
#include "Domain.hpp"
#include "EqlbDist.hpp"
#include "Field.hpp"
#include "Flow.hpp"
#include "LBDynamics.hpp"
#include "LBModel.hpp"
#include "PLBPD.hpp"
#include "SimData.hpp"

#define CHECK(cond)                                                            \
    do {                                                                       \
        if (!(cond)) {                                                         \
            std::fprintf(stderr, "CHECK failed at line %d: %s\n", __LINE__, #cond); \
            std::exit(1);                                                      \
        }                                                                      \
    } while (0)

template <typename E, typename F>
void expect_throw(F f, const char* what) {
    try {
        f();
    } catch (const E&) {
        return;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "%s: wrong exception type: %s\n", what, e.what());
        std::exit(1);
    }
    std::fprintf(stderr, "%s: no exception\n", what);
    std::exit(1);
}

static void dump(const std::string& path, const Field::VectorField<float, 1>* f) {
    std::ofstream o(path, std::ios::binary);
    const float* p = f->get(0, 0, 0, 0);
    o.write(reinterpret_cast<const char*>(p), (std::streamsize)(f->size() * sizeof(float)));
}

// Every byte of n, ntmp, rho and u of two SimData equal (const access: the
// host mirrors are read, downloaded first where the device is newer).
static bool same_bits(const SimData& a, const SimData& b) {
    const Field::VectorField<float, 1>* fa[4] = {a.n, a.ntmp, a.rho, a.u};
    const Field::VectorField<float, 1>* fb[4] = {b.n, b.ntmp, b.rho, b.u};
    for (int i = 0; i < 4; ++i) {
        if (fa[i]->size() != fb[i]->size()) return false;
        if (std::memcmp(fa[i]->get(0, 0, 0, 0), fb[i]->get(0, 0, 0, 0), fa[i]->size() * sizeof(float)) != 0) {
            std::fprintf(stderr, "field %d differs\n", i);
            return false;
        }
    }
    return true;
}

static void dump_all(const std::string& dir, const std::string& key, SimData& sd) {
    dump(dir + "/" + key + "_n.f32", sd.n);
    dump(dir + "/" + key + "_ntmp.f32", sd.ntmp);
    dump(dir + "/" + key + "_rho.f32", sd.rho);
    dump(dir + "/" + key + "_u.f32", sd.u);
}

static int run_cpu() {
    // TestField: extents and indexing with 0 and 1 halo layers
    {
        Field::ScalarField<float, 0> sf(4, 5, 7, 0);
        const auto e = sf.get_extents();
        CHECK(e.zbegin == 0 && e.zend == 4 && e.ybegin == 0 && e.yend == 5 && e.xbegin == 0 && e.xend == 7);
        float ctr = 0;
        for (auto z = e.zbegin; z < e.zend; ++z)
            for (auto y = e.ybegin; y < e.yend; ++y)
                for (auto x = e.xbegin; x < e.xend; ++x) sf.at(z, y, x) = ctr++;
        for (auto z = e.zbegin; z < e.zend; ++z)
            for (auto y = e.ybegin; y < e.yend; ++y)
                for (auto x = e.xbegin; x < e.xend; ++x) CHECK(sf.at(z, y, x) == sf.sub2ind(z, y, x));
        Field::VectorField<float, 0> vf(4, 5, 7, 2, 0.0f);
        CHECK(vf.get_vector_length() == 2);
        auto sf1 = std::make_unique<Field::ScalarField<float, 1> >(2, 2, 3, 0.0f);
        uint32_t zd, yd, xd;
        std::tie(zd, yd, xd) = sf1->get_dimensions();
        CHECK(zd == 4 && yd == 4 && xd == 5);
        const auto e1 = sf1->get_extents();
        for (auto z = e1.zbegin; z < e1.zend; ++z)
            for (auto y = e1.ybegin; y < e1.yend; ++y)
                for (auto x = e1.xbegin; x < e1.xend; ++x) sf1->at(z, y, x) = (float)sf1->sub2ind(z, y, x);
        CHECK(sf1->at(1, 2, 3) == 33);
        CHECK(sf1->at(2, 1, 3) == 48);
        auto nb = vf.get_neighbor(1, 1, 1, {1, 0, -1});
        CHECK(std::get<0>(nb) == 0 && std::get<1>(nb) == 1 && std::get<2>(nb) == 2);
    }
    // TestDomain: getters round-trip
    {
        auto m = std::make_unique<LBModel>("D3Q19");
        const std::array<float, 3> vel = {-1148.14f, 762.878f, 3.2f};
        const std::array<float, 3> force = {-0.145f, 0.0f, 4.2f};
        auto d = std::make_unique<Domain>(m.get(), 5, 4, 3, 0.5f, 1.0f, vel, force);
        CHECK(std::make_tuple((size_t)5, (size_t)4, (size_t)3) == d->get_dimensions());
        CHECK(d->get_fluid_viscosity() == 0.5f && d->get_fluid_density() == 1.0f);
        CHECK(d->get_init_flow_velocity() == vel && d->get_external_force() == force);
    }
    // error conventions
    expect_throw<std::logic_error>([] { LBModel m("D4Q1"); }, "unknown model");
    expect_throw<std::invalid_argument>([] { Field::VectorField<float, 1> f(0, 1, 1, 1, 0.0f); }, "zero extent");
    expect_throw<std::invalid_argument>([] { Flow f("Taylor3D"); }, "unknown flow");
    {
        LBModel m("D2Q9");
        Streaming st(&m);
        SimData sd(std::make_tuple((size_t)4, (size_t)1, (size_t)3), 9);
        expect_throw<std::logic_error>([&] { st(sd, "sideways"); }, "bad stream type");
        expect_throw<std::logic_error>([&] { st(sd, "pull"); }, "pull streaming");
        expect_throw<std::logic_error>([&] { st(sd, "pull", true); }, "pull streaming (reference)");
        Domain d(&m, 4, 1, 3, 0.1f, 1.0f, {0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f});
        expect_throw<std::invalid_argument>([&] { CollisionTRT c(&m, &d, -1.0f); }, "negative TRT magic");
    }
    // tables and the TestEqlbDist known answer, for the Python side
    std::printf("{");
    for (const char* name : {"D2Q9", "D3Q19", "D3Q27"}) {
        LBModel m(name);
        std::printf("\"%s\": {\"q\": %u, \"cs2\": %.9g, \"c\": [", name, m.get_num_directions(),
                    (double)m.get_speed_of_sound_squared());
        const auto& c = m.get_directional_velocities();
        for (size_t k = 0; k < c.size(); ++k)
            std::printf("%s%d, %d, %d", k ? ", " : "", c[k][0], c[k][1], c[k][2]);
        std::printf("], \"w\": [");
        for (size_t k = 0; k < c.size(); ++k) std::printf("%s%.9g", k ? ", " : "", (double)m.get_directional_weights()[k]);
        std::printf("], \"rev\": [");
        for (size_t k = 0; k < c.size(); ++k) std::printf("%s%u", k ? ", " : "", m.get_reverse()[k]);
        std::printf("]}, ");
    }
    LBModel m9("D2Q9");
    EqlbDist e(&m9);
    std::vector<float> nl(9, 0.0f);
    e(1.0f, {0.5f, 0.5f, -0.5f}, nl);
    std::printf("\"eqlb\": [");
    for (int k = 0; k < 9; ++k) std::printf("%s%.9g", k ? ", " : "", (double)nl[k]);
    std::printf("]}\n");
    return 0;
}

static const char* kFaceNames[6] = {"east", "west", "north", "south", "up", "down"};

static int run_case(int argc, char** argv) {
    const std::string dir = argv[2];
    const std::string model = argv[3];
    int a = 4;
    const size_t nx = std::stoul(argv[a++]), ny = std::stoul(argv[a++]), nz = std::stoul(argv[a++]);
    const float nu = std::stof(argv[a++]), rho0 = std::stof(argv[a++]);
    std::array<float, 3> u0, F;
    for (int i = 0; i < 3; ++i) u0[i] = std::stof(argv[a++]);
    for (int i = 0; i < 3; ++i) F[i] = std::stof(argv[a++]);
    const float rho_s = std::stof(argv[a++]);
    BoundaryType type;
    BoundaryVelocity vel;
    for (int f = 0; f < 6; ++f) {
        const int t = std::stoi(argv[a++]);
        const int hv = std::stoi(argv[a++]);
        std::array<float, 3> v;
        for (int i = 0; i < 3; ++i) v[i] = std::stof(argv[a++]);
        if (t == 1) type[kFaceNames[f]] = "periodic";
        if (t == 2) type[kFaceNames[f]] = "noslip";
        if (hv) vel[kFaceNames[f]] = v;
    }
    CHECK(a <= argc);
    auto lbmodel = std::make_unique<LBModel>(model);
    auto domain = std::make_unique<Domain>(lbmodel.get(), nx, ny, nz, nu, rho0, u0, F);
    auto boundary = std::make_unique<Boundary>(lbmodel.get(), domain.get(), rho_s, type, vel);
    auto problem = std::make_unique<PLBPD>(lbmodel.get(), domain.get(), boundary.get());
    auto simdata = SimData(domain->get_dimensions(), lbmodel->get_num_directions());
    problem->initialize(simdata);
    dump_all(dir, "init", simdata);
    size_t done = 0;
    for (size_t target : {1, 2, 5, 20}) {
        problem->march_in_time(target - done, simdata);
        done = target;
        dump_all(dir, "step" + std::to_string(target), simdata);
    }
    // one more step, operator by operator
    LBDynamics dyn(lbmodel.get(), domain.get());
    CalcMoments moments(lbmodel.get());
    dyn.collide(simdata);
    dump(dir + "/op_collide_n.f32", simdata.n);
    dyn.stream(simdata, "push");
    dump(dir + "/op_stream_n.f32", simdata.n);
    dump(dir + "/op_stream_ntmp.f32", simdata.ntmp);
    boundary->apply_noslip(simdata);
    dump(dir + "/op_noslip_n.f32", simdata.n);
    boundary->apply_periodicity(simdata);
    dump(dir + "/op_periodic_n.f32", simdata.n);
    moments(simdata);
    dump(dir + "/op_moments_rho.f32", simdata.rho);
    dump(dir + "/op_moments_u.f32", simdata.u);
    boundary->reset(simdata);
    dump(dir + "/op_reset_rho.f32", simdata.rho);
    dump(dir + "/op_reset_u.f32", simdata.u);
    // host edits between operators reach the device
    simdata.rho->at(1, 1, 1) = simdata.rho->at(1, 1, 1) + 0.0f;
    // state round trip
    simdata.write_state(dir + "/state.plb");
    SimData back(domain->get_dimensions(), lbmodel->get_num_directions());
    back.read_state(dir + "/state.plb");
    CHECK(same_bits(back, simdata));
    // resume: a march continued from a restored state equals the uninterrupted
    // march, bit for bit (odd step counts leave n and ntmp swapped)
    {
        auto whole = SimData(domain->get_dimensions(), lbmodel->get_num_directions());
        problem->initialize(whole);
        problem->march_in_time(13, whole);
        whole.write_state(dir + "/resume.plb");
        problem->march_in_time(17, whole);
        auto resumed = SimData(domain->get_dimensions(), lbmodel->get_num_directions());
        resumed.read_state(dir + "/resume.plb");
        problem->march_in_time(17, resumed);
        CHECK(same_bits(resumed, whole));
    }
    // a hand-written loop with the second Collision subclass in place of
    // CollisionSRT: 6 steps of collide, push, no-slip, periodicity, moments, reset
    {
        auto trt_data = SimData(domain->get_dimensions(), lbmodel->get_num_directions());
        problem->initialize(trt_data);
        const std::unique_ptr<Collision> collide = std::make_unique<CollisionTRT>(lbmodel.get(), domain.get());
        CHECK(static_cast<const CollisionTRT&>(*collide).get_magic() == 3.0f / 16.0f);
        Streaming stream(lbmodel.get());
        for (int t = 0; t < 6; ++t) {
            (*collide)(trt_data, false);
            stream(trt_data, "push");
            boundary->apply_noslip(trt_data);
            boundary->apply_periodicity(trt_data);
            moments(trt_data);
            boundary->reset(trt_data);
        }
        dump_all(dir, "trt6", trt_data);
    }
    problem->print_times();
    return 0;
}

static int run_preset(char** argv) {
    // the reference's main.cpp, on a named preset
    const auto flow = std::make_unique<Flow>(argv[2]);
    const auto lbmodel = flow->get_lbmodel();
    const auto domain = flow->get_domain();
    const auto boundary = flow->get_boundary();
    const auto problem = std::make_unique<PLBPD>(lbmodel, domain, boundary);
    auto simdata = SimData(domain->get_dimensions(), lbmodel->get_num_directions());
    problem->initialize(simdata);
    problem->march_in_time(flow->get_num_timesteps(), simdata);
    dump_all(argv[3], "final", simdata);
    problem->print_times();
    return 0;
}

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    const std::string mode = argv[1];
    try {
        if (mode == "cpu") return run_cpu();
        if (mode == "case" && argc >= 4 + 3 + 2 + 6 + 1 + 30) return run_case(argc, argv);
        if (mode == "preset" && argc >= 4) return run_preset(argv);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "exception: %s\n", e.what());
        return 3;
    }
    return 2;
}
