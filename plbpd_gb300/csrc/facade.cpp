// plbpd's C++ classes over the C ABI (include/plbpd/*.hpp).  Each class keeps
// the reference's public interface, error types and timers; the work runs on
// the GPU through plb_* calls on the SimData's device state.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>

#include "../../include/plb.h"
#include "../../include/plbpd/Boundary.hpp"
#include "../../include/plbpd/CalcMoments.hpp"
#include "../../include/plbpd/Collision.hpp"
#include "../../include/plbpd/CollisionSRT.hpp"
#include "../../include/plbpd/CollisionTRT.hpp"
#include "../../include/plbpd/Domain.hpp"
#include "../../include/plbpd/EqlbDist.hpp"
#include "../../include/plbpd/Flow.hpp"
#include "../../include/plbpd/LBDynamics.hpp"
#include "../../include/plbpd/LBModel.hpp"
#include "../../include/plbpd/PLBPD.hpp"
#include "../../include/plbpd/SimData.hpp"
#include "../../include/plbpd/Streaming.hpp"

namespace chrono = std::chrono;

namespace {

void check(int rc, const char* what) {
    if (rc >= 0) return;
    const std::string msg = std::string(what) + ": " + plb_last_error();
    if (rc == PLB_EINVAL) throw std::invalid_argument(msg);
    throw std::runtime_error(msg);
}

const char* kFaces[6] = {"east", "west", "north", "south", "up", "down"};

// Parameters a device state is created with when an operator first touches a
// SimData; every operator then installs its own parameters before it runs.
plb_params base_params(const SimData& sd) {
    plb_params p;
    std::memset(&p, 0, sizeof(p));
    size_t x, y, z;
    std::tie(x, y, z) = sd.dimensions();
    p.q = (int32_t)sd.num_directions();
    p.nx = (int64_t)x; p.ny = (int64_t)y; p.nz = (int64_t)z;
    p.nu = 0.1f;
    p.rho0 = 1.0f;
    p.rho_solid = 1.0f;
    p.semantics = PLB_SEMANTICS_REFERENCE;
    p.arith = PLB_ARITH_REFERENCE;
    p.storage = PLB_STORAGE_FP32;
    p.device = 0;
    return p;
}

// The collision operator and its parameters: BGK for CollisionSRT (and the
// fused march), TRT with its magic parameter for CollisionTRT.
void install_collision(plb_solve* s, const Domain* d, int32_t collision = PLB_COLLISION_BGK, float magic = 0.0f) {
    const auto& F = d->get_external_force();
    check(plb_set_collision(s, collision, magic), "plb_set_collision");
    check(plb_set_relaxation(s, d->get_fluid_viscosity(), F.data()), "plb_set_relaxation");
}

void install_boundary(plb_solve* s, const Boundary* b) {
    int32_t t[6], hv[6];
    float v[18];
    b->face_arrays(t, hv, v);
    check(plb_set_boundary(s, b->get_solid_density(), t, hv, v), "plb_set_boundary");
}

float seconds_since(chrono::system_clock::time_point t0) {
    chrono::duration<float> el = chrono::system_clock::now() - t0;
    return el.count();
}

}  // namespace

// ===========================================================================
// LBModel (src/LBModel.cpp:8-189)
LBModel::LBModel(std::string model_name) : _name(model_name) {
    int32_t c[27 * 3];
    float w[27];
    uint32_t rev[27];
    float cs2 = 0.0f;
    const int q = plb_model_tables(model_name.c_str(), c, w, rev, &cs2);
    if (q < 0) throw std::logic_error("Model " + model_name + " not yet implemented");
    _q = (uint32_t)q;
    _cs2 = cs2;
    for (int k = 0; k < q; ++k) {
        _c.push_back({c[3 * k], c[3 * k + 1], c[3 * k + 2]});
        _w.push_back(w[k]);
        _rev.push_back(rev[k]);
    }
}
LBModel::~LBModel() {}
std::string LBModel::get_model_name() const { return _name; }
uint32_t LBModel::get_num_directions() const { return _q; }
float LBModel::get_speed_of_sound_squared() const { return _cs2; }
const std::vector<std::array<int32_t, 3> >& LBModel::get_directional_velocities() const { return _c; }
const std::vector<float>& LBModel::get_directional_weights() const { return _w; }
const std::vector<uint32_t>& LBModel::get_reverse() const { return _rev; }

// ===========================================================================
// EqlbDist (src/EqlbDist.hpp:26-38)
EqlbDist::EqlbDist(const LBModel* lbmodel) : _kdim(lbmodel->get_num_directions()) {}

void EqlbDist::operator()(const float rholocal, const std::array<float, 3>& ulocal, std::vector<float>& nlocal) {
    if (nlocal.size() != _kdim) throw std::invalid_argument("nlocal has the wrong length");
    check(plb_equilibrium((int32_t)_kdim, rholocal, ulocal.data(), nlocal.data()), "plb_equilibrium");
}

// ===========================================================================
// SimData (src/SimData.cpp:22-164)
SimData::SimData(const std::tuple<size_t, size_t, size_t> domain_dimensions, const size_t num_directions)
    : rho(nullptr), u(nullptr), n(nullptr), ntmp(nullptr), _dims(domain_dimensions), _kdim(num_directions),
      _arith(PLB_ARITH_REFERENCE) {
    const char* env = std::getenv("PLB_FACADE_ARITH");
    if (env && std::string(env) == "fp32") _arith = PLB_ARITH_FP32;
    _bootstrap();
}

SimData::SimData(SimData&& o) noexcept
    : rho(o.rho), u(o.u), n(o.n), ntmp(o.ntmp), _dims(o._dims), _kdim(o._kdim), _arith(o._arith),
      _solve(o._solve), _hook(std::move(o._hook)) {
    o.rho = nullptr; o.u = nullptr; o.n = nullptr; o.ntmp = nullptr; o._solve = nullptr;
    if (_hook) _hook->owner = this;
}

SimData::~SimData() {
    if (_solve) plb_solve_destroy(_solve);
    delete rho; delete u; delete n; delete ntmp;
}

void SimData::_bootstrap() {
    size_t xd, yd, zd;
    std::tie(xd, yd, zd) = _dims;
    rho = new Field::ScalarField<float, 1>((uint32_t)zd, (uint32_t)yd, (uint32_t)xd, 0.0f);
    u = new Field::VectorField<float, 1>((uint32_t)zd, (uint32_t)yd, (uint32_t)xd, 3, 0.0f);
    n = new Field::VectorField<float, 1>((uint32_t)zd, (uint32_t)yd, (uint32_t)xd, (uint32_t)_kdim, 0.0f);
    ntmp = new Field::VectorField<float, 1>((uint32_t)zd, (uint32_t)yd, (uint32_t)xd, (uint32_t)_kdim, 0.0f);
    _hook.reset(new Field::AccessHook());
    _hook->owner = this;
    _hook->pull = [](Field::AccessHook* h) { static_cast<SimData*>(h->owner)->pull(); };
    _attach_hooks();
}

void SimData::_attach_hooks() {
    for (Field::VectorField<float, 1>* f : {static_cast<Field::VectorField<float, 1>*>(rho), u, n, ntmp})
        f->set_access_hook(_hook.get());
}

void SimData::set_arithmetic(int arith) {
    if (_solve) throw std::logic_error("set_arithmetic must come before the first operator");
    _arith = arith;
}

void SimData::_upload() {
    check(plb_set_field(_solve, PLB_FIELD_N, n->raw()), "plb_set_field(n)");
    check(plb_set_field(_solve, PLB_FIELD_NTMP, ntmp->raw()), "plb_set_field(ntmp)");
    check(plb_set_field(_solve, PLB_FIELD_RHO, rho->raw()), "plb_set_field(rho)");
    check(plb_set_field(_solve, PLB_FIELD_U, u->raw()), "plb_set_field(u)");
}

plb_solve* SimData::device_for(const plb_params& p) {
    if (!_solve) {
        plb_params q = p;
        q.arith = _arith;
        check(plb_solve_create(&q, &_solve), "plb_solve_create");
        _upload();
    } else if (_hook->host_dirty) {
        _upload();
    }
    _hook->host_dirty = false;
    return _solve;
}

void SimData::mark_device_newer() { _hook->device_newer = true; }

void SimData::pull() {
    _hook->device_newer = false;
    if (!_solve) return;
    check(plb_get_field(_solve, PLB_FIELD_N, n->raw()), "plb_get_field(n)");
    check(plb_get_field(_solve, PLB_FIELD_NTMP, ntmp->raw()), "plb_get_field(ntmp)");
    check(plb_get_field(_solve, PLB_FIELD_RHO, rho->raw()), "plb_get_field(rho)");
    check(plb_get_field(_solve, PLB_FIELD_U, u->raw()), "plb_get_field(u)");
}

// The "plb-state-v1" container: one JSON line naming the datasets in order,
// then their float32 data back to back.
void SimData::write_state(std::string dump_file) {
    if (_hook->device_newer) pull();
    size_t xd, yd, zd;
    std::tie(xd, yd, zd) = _dims;
    std::ostringstream h;
    h << "{\"format\": \"plb-state-v1\", \"dims_zyx\": [" << zd + 2 << ", " << yd + 2 << ", " << xd + 2
      << "], \"datasets\": [[\"/Density\", 1], [\"/FlowVelocity\", 3], [\"/ParticleDistribution\", " << _kdim
      << "], [\"/ParticleDistributionTmp\", " << _kdim << "]]}\n";
    std::ofstream f(dump_file, std::ios::binary | std::ios::trunc);
    if (!f) throw std::runtime_error("cannot open " + dump_file);
    const std::string hs = h.str();
    f.write(hs.data(), (std::streamsize)hs.size());
    for (const Field::VectorField<float, 1>* fld :
         {static_cast<const Field::VectorField<float, 1>*>(rho), static_cast<const Field::VectorField<float, 1>*>(u),
          static_cast<const Field::VectorField<float, 1>*>(n), static_cast<const Field::VectorField<float, 1>*>(ntmp)})
        f.write(reinterpret_cast<const char*>(fld->raw()), (std::streamsize)(fld->size() * sizeof(float)));
    if (!f) throw std::runtime_error("write failed: " + dump_file);
}

void SimData::read_state(std::string dump_file) {
    std::ifstream f(dump_file, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open " + dump_file);
    std::string header;
    std::getline(f, header);
    size_t xd, yd, zd;
    std::tie(xd, yd, zd) = _dims;
    std::ostringstream want;
    want << "\"dims_zyx\": [" << zd + 2 << ", " << yd + 2 << ", " << xd + 2 << "]";
    if (header.find("\"plb-state-v1\"") == std::string::npos || header.find(want.str()) == std::string::npos)
        throw std::invalid_argument("state file does not match this SimData: " + dump_file);
    if (_hook->device_newer) pull();
    for (Field::VectorField<float, 1>* fld : {static_cast<Field::VectorField<float, 1>*>(rho), u, n, ntmp})
        f.read(reinterpret_cast<char*>(fld->raw()), (std::streamsize)(fld->size() * sizeof(float)));
    if (!f) throw std::runtime_error("state file is truncated: " + dump_file);
    _hook->host_dirty = true;
}

// ===========================================================================
// Domain (src/Domain.cpp:13-63)
Domain::Domain(const LBModel* lbmodel, size_t xdim, size_t ydim, size_t zdim, float fluid_viscosity,
               float fluid_density, std::array<float, 3> init_flow_velocity, std::array<float, 3> external_force)
    : _lbmodel(lbmodel), _xdim((uint32_t)xdim), _ydim((uint32_t)ydim), _zdim((uint32_t)zdim),
      _fluid_viscosity(fluid_viscosity), _fluid_density(fluid_density), _init_flow_velocity(init_flow_velocity),
      _external_force(external_force) {}
Domain::~Domain() {}
std::tuple<size_t, size_t, size_t> Domain::get_dimensions() const {
    return std::make_tuple((size_t)_xdim, (size_t)_ydim, (size_t)_zdim);
}
float Domain::get_fluid_viscosity() const { return _fluid_viscosity; }
float Domain::get_fluid_density() const { return _fluid_density; }
const std::array<float, 3>& Domain::get_init_flow_velocity() const { return _init_flow_velocity; }
const std::array<float, 3>& Domain::get_external_force() const { return _external_force; }

void Domain::initialize(SimData& simdata) const {
    const uint32_t kdim = simdata.n->get_vector_length();
    std::vector<float> feq(kdim, 0.0f);
    check(plb_equilibrium((int32_t)kdim, _fluid_density, _init_flow_velocity.data(), feq.data()), "plb_equilibrium");
    float* r = simdata.rho->get(0, 0, 0);
    float* uu = simdata.u->get(0, 0, 0, 0);
    float* nn = simdata.n->get(0, 0, 0, 0);
    const size_t cells = simdata.rho->size();
    for (size_t i = 0; i < cells; ++i) {
        r[i] = _fluid_density;
        for (int d = 0; d < 3; ++d) uu[3 * i + d] = _init_flow_velocity[d];
        for (uint32_t k = 0; k < kdim; ++k) nn[i * kdim + k] = feq[k];
    }
}

// ===========================================================================
// Boundary (src/Boundary.cpp:12-305)
float Boundary::_time_noslip = 0.0f;
float Boundary::_time_periodicity = 0.0f;
float Boundary::_time_reset = 0.0f;
float Boundary::_time_velocity_reset = 0.0f;
float Boundary::_time_density_reset = 0.0f;
const std::vector<std::string> Boundary::_directions = {"east", "west", "north", "south", "up", "down"};

Boundary::Boundary(const LBModel* lbmodel, const Domain* domain, float solid_density, BoundaryType type,
                   BoundaryVelocity velocity)
    : _lbmodel(lbmodel), _domain(domain), _solid_density(solid_density), _type(type), _velocity(velocity) {}
Boundary::~Boundary() {}
const BoundaryType Boundary::get_boundary_type() const { return _type; }
const BoundaryVelocity Boundary::get_boundary_velocity() const { return _velocity; }

void Boundary::face_arrays(int32_t* type6, int32_t* has_vel6, float* vel18) const {
    for (int f = 0; f < 6; ++f) {
        type6[f] = PLB_FACE_NONE;
        auto t = _type.find(kFaces[f]);
        if (t != _type.end()) {
            if (t->second == "periodic") type6[f] = PLB_FACE_PERIODIC;
            if (t->second == "noslip") type6[f] = PLB_FACE_NOSLIP;
        }
        auto v = _velocity.find(kFaces[f]);
        has_vel6[f] = v != _velocity.end();
        for (int i = 0; i < 3; ++i) vel18[3 * f + i] = has_vel6[f] ? v->second[i] : 0.0f;
    }
}

void Boundary::check_noslip_velocities() const {
    for (const auto& d : _directions) {
        auto t = _type.find(d);
        if (t != _type.end() && t->second == "noslip") (void)_velocity.at(d);   // throws std::out_of_range
    }
}

namespace {
plb_solve* boundary_device(SimData& sd, const Boundary* b) {
    plb_solve* s = sd.device_for(base_params(sd));
    install_boundary(s, b);
    return s;
}
}  // namespace

void Boundary::reset(SimData& simdata) const {
    const auto t0 = chrono::system_clock::now();
    reset_velocity(simdata);
    reset_density(simdata);
    _time_reset += seconds_since(t0);
}

void Boundary::reset_velocity(SimData& simdata) const {
    const auto t0 = chrono::system_clock::now();
    plb_solve* s = boundary_device(simdata, this);
    check(plb_reset_velocity(s), "plb_reset_velocity");
    simdata.mark_device_newer();
    _time_velocity_reset += seconds_since(t0);
}

void Boundary::reset_density(SimData& simdata) const {
    const auto t0 = chrono::system_clock::now();
    plb_solve* s = boundary_device(simdata, this);
    check(plb_reset_density(s), "plb_reset_density");
    simdata.mark_device_newer();
    _time_density_reset += seconds_since(t0);
}

void Boundary::apply_periodicity(SimData& simdata) const {
    const auto t0 = chrono::system_clock::now();
    plb_solve* s = boundary_device(simdata, this);
    check(plb_apply_periodicity(s), "plb_apply_periodicity");
    simdata.mark_device_newer();
    _time_periodicity += seconds_since(t0);
}

void Boundary::apply_noslip(SimData& simdata) const {
    const auto t0 = chrono::system_clock::now();
    check_noslip_velocities();
    plb_solve* s = boundary_device(simdata, this);
    check(plb_apply_noslip(s), "plb_apply_noslip");
    simdata.mark_device_newer();
    _time_noslip += seconds_since(t0);
}

float Boundary::get_time_noslip() const { return _time_noslip; }
float Boundary::get_time_periodicity() const { return _time_periodicity; }
float Boundary::get_time_reset() const { return _time_reset; }
float Boundary::get_time_velocity_reset() const { return _time_velocity_reset; }
float Boundary::get_time_density_reset() const { return _time_density_reset; }
float Boundary::get_total_time() const { return _time_noslip + _time_periodicity + _time_reset; }

// ===========================================================================
// Collision, CollisionSRT (src/Collision.cpp, src/CollisionSRT.cpp:14-33)
float Collision::_time = 0.0f;
Collision::Collision() {}
Collision::~Collision() {}
float Collision::get_total_time() const { return _time; }

CollisionSRT::CollisionSRT(const LBModel* lbmodel, const Domain* domain) : _lbmodel(lbmodel), _domain(domain) {}
CollisionSRT::~CollisionSRT() {}

void CollisionSRT::operator()(SimData& simdata, bool /*reference*/) const {
    const auto t0 = chrono::system_clock::now();
    plb_solve* s = simdata.device_for(base_params(simdata));
    install_collision(s, _domain);
    check(plb_collide(s), "plb_collide");
    simdata.mark_device_newer();
    Collision::_time += seconds_since(t0);
}

// CollisionTRT: a second subclass of Collision (no counterpart in plbpd).
CollisionTRT::CollisionTRT(const LBModel* lbmodel, const Domain* domain, float magic)
    : _lbmodel(lbmodel), _domain(domain), _magic(magic) {
    if (!(magic >= 0.0f)) throw std::invalid_argument("CollisionTRT: the magic parameter must be >= 0");
}
CollisionTRT::~CollisionTRT() {}
float CollisionTRT::get_magic() const { return _magic > 0.0f ? _magic : 3.0f / 16.0f; }

void CollisionTRT::operator()(SimData& simdata, bool /*reference*/) const {
    const auto t0 = chrono::system_clock::now();
    plb_solve* s = simdata.device_for(base_params(simdata));
    install_collision(s, _domain, PLB_COLLISION_TRT, _magic);
    check(plb_collide(s), "plb_collide");
    simdata.mark_device_newer();
    Collision::_time += seconds_since(t0);
}

// ===========================================================================
// Streaming (src/Streaming.cpp:12-102)
float Streaming::_time = 0.0f;
Streaming::Streaming(const LBModel* lbmodel) : _lbmodel(lbmodel) {}
Streaming::~Streaming() {}
float Streaming::get_total_time() const { return _time; }

void Streaming::operator()(SimData& simdata, std::string stream_type, bool reference) const {
    const auto t0 = chrono::system_clock::now();
    if (stream_type != "push" && stream_type != "pull")
        throw std::logic_error("Invalid stream type: " + stream_type);
    if (stream_type == "pull")
        throw std::logic_error(reference ? "Streaming::_pull_ref has not yet been implemented"
                                         : "Streaming::_pull_tbb has not yet been implemented");
    plb_solve* s = simdata.device_for(base_params(simdata));
    check(plb_stream_push(s), "plb_stream_push");
    std::swap(simdata.ntmp, simdata.n);
    simdata.mark_device_newer();
    _time += seconds_since(t0);
}

// ===========================================================================
// LBDynamics (src/LBDynamics.cpp:5-33)
LBDynamics::LBDynamics(const LBModel* lbmodel, const Domain* domain) {
    _collide = std::make_unique<CollisionSRT>(lbmodel, domain);
    _stream = std::make_unique<Streaming>(lbmodel);
}
LBDynamics::~LBDynamics() {}
void LBDynamics::collide(SimData& simdata, bool reference) const { (*_collide)(simdata, reference); }
void LBDynamics::stream(SimData& simdata, std::string stream_type, bool reference) const {
    (*_stream)(simdata, stream_type, reference);
}
float LBDynamics::get_time_collide() const { return _collide->get_total_time(); }
float LBDynamics::get_time_stream() const { return _stream->get_total_time(); }
float LBDynamics::get_total_time() const { return _collide->get_total_time() + _stream->get_total_time(); }

// ===========================================================================
// CalcMoments (src/CalcMoments.hpp:47-73)
float CalcMoments::_time_calc_moment = 0.0f;
CalcMoments::CalcMoments(const LBModel* lbmodel) : _lbmodel(lbmodel) {}
CalcMoments::~CalcMoments() {}
float CalcMoments::get_total_time() const { return _time_calc_moment; }

void CalcMoments::operator()(SimData& simdata) const {
    const auto t0 = chrono::system_clock::now();
    plb_solve* s = simdata.device_for(base_params(simdata));
    check(plb_calc_moments(s), "plb_calc_moments");
    simdata.mark_device_newer();
    _time_calc_moment += seconds_since(t0);
}

// ===========================================================================
// PLBPD (src/PLBPD.cpp:6-48)
float PLBPD::_time_march = 0.0f;

PLBPD::PLBPD(const LBModel* lbmodel, const Domain* domain, const Boundary* boundary)
    : _lbmodel(lbmodel), _domain(domain), _boundary(boundary) {
    _lbdynamics = std::make_unique<LBDynamics>(lbmodel, domain);
    _calc_moments = std::make_unique<CalcMoments>(lbmodel);
}
PLBPD::~PLBPD() {}

void PLBPD::initialize(SimData& simdata) const {
    _domain->initialize(simdata);
    _boundary->reset(simdata);
}

void PLBPD::march_in_time(size_t num_timesteps, SimData& simdata) const {
    const auto t0 = chrono::system_clock::now();
    if (num_timesteps > 0) _boundary->check_noslip_velocities();
    plb_solve* s = simdata.device_for(base_params(simdata));
    install_collision(s, _domain);
    install_boundary(s, _boundary);
    check(plb_step(s, (int64_t)num_timesteps), "plb_step");
    // plbpd's streaming swaps n and ntmp once per step
    if (num_timesteps % 2 == 1) std::swap(simdata.ntmp, simdata.n);
    simdata.mark_device_newer();
    const float el = seconds_since(t0);
    _time_march += el;
    std::cout << "Time taken by timeloop: " << el << "s" << std::endl;
}

void PLBPD::print_times() const {
    std::cout << "LBDynamics: " << _lbdynamics->get_total_time() << "s\n";
    std::cout << "-collide: " << _lbdynamics->get_time_collide() << "s\n";
    std::cout << "-stream: " << _lbdynamics->get_time_stream() << "s\n";
    std::cout << "CalcMoments: " << _calc_moments->get_total_time() << "s\n";
    std::cout << "Boundary: " << _boundary->get_total_time() << "s\n";
    std::cout << "-noslip: " << _boundary->get_time_noslip() << "s\n";
    std::cout << "-periodicity: " << _boundary->get_time_periodicity() << "s\n";
    std::cout << "-reset: " << _boundary->get_time_reset() << "s\n";
    std::cout << "--velocity-reset: " << _boundary->get_time_velocity_reset() << "s\n";
    std::cout << "--density-reset: " << _boundary->get_time_density_reset() << "s\n";
    std::cout << "Fused time loop (all phases above, on the GPU): " << _time_march << "s\n";
}

// ===========================================================================
// Flow presets (src/Flow.cpp:5-122)
Flow::Flow(std::string flow_type) {
    const bool couette = flow_type == "Couette2D" || flow_type == "Couette3D";
    const bool poiseuille = flow_type == "Poiseuille2D" || flow_type == "Poiseuille3D";
    if (!couette && !poiseuille) throw std::invalid_argument("Flow type [" + flow_type + "] not recognized");
    const bool three_d = flow_type.back() == 'D' && flow_type[flow_type.size() - 2] == '3';
    _lbmodel = std::make_unique<LBModel>(three_d ? "D3Q19" : "D2Q9");
    BoundaryType type = {{"east", "periodic"}, {"west", "periodic"}, {"up", "noslip"}, {"down", "noslip"}};
    if (three_d) { type["north"] = "periodic"; type["south"] = "periodic"; }
    const std::array<float, 3> zero = {0.0f, 0.0f, 0.0f};
    if (couette) {
        // resting fluid between a lid moving at 0.5 in x and a resting wall
        BoundaryVelocity vel = {{"up", {0.5f, 0.0f, 0.0f}}, {"down", zero}};
        if (three_d) _domain = std::make_unique<Domain>(_lbmodel.get(), 200, 50, 50, 0.5f, 1.0f, zero, zero);
        else _domain = std::make_unique<Domain>(_lbmodel.get(), 100, 1, 25, 0.5f, 1.0f, zero, zero);
        _boundary = std::make_unique<Boundary>(_lbmodel.get(), _domain.get(), 1.0f, type, vel);
        _num_timesteps = three_d ? 200 : 20000;
    } else {
        // body-force driven channel between resting walls
        BoundaryVelocity vel = {{"up", zero}, {"down", zero}};
        const std::array<float, 3> force = {1.0e-5f, 0.0f, 0.0f};
        if (three_d) _domain = std::make_unique<Domain>(_lbmodel.get(), 256, 256, 48, 0.1f, 1.0f, zero, force);
        else _domain = std::make_unique<Domain>(_lbmodel.get(), 256, 1, 48, 0.1f, 1.0f, zero, force);
        _boundary = std::make_unique<Boundary>(_lbmodel.get(), _domain.get(), 1.0f, type, vel);
        _num_timesteps = three_d ? 10 : 5000;
    }
}
Flow::~Flow() {}
const Domain* Flow::get_domain() const { return _domain.get(); }
const Boundary* Flow::get_boundary() const { return _boundary.get(); }
const LBModel* Flow::get_lbmodel() const { return _lbmodel.get(); }
size_t Flow::get_num_timesteps() const { return _num_timesteps; }
