// plbpd's Domain interface (src/Domain.hpp:10-40): extents, fluid properties,
// initial velocity and body force; initialize() sets rho0, u0 and the
// equilibrium on every node, halo included (src/Domain.cpp:46-63).
#ifndef PLBPD_GB300_DOMAIN_HPP_
#define PLBPD_GB300_DOMAIN_HPP_

#include <array>
#include <cstdint>
#include <string>
#include <tuple>

#include "LBModel.hpp"
#include "SimData.hpp"

class Domain final {
 public:
    Domain() = delete;
    Domain(const LBModel* lbmodel, size_t xdim, size_t ydim, size_t zdim, float fluid_viscosity,
           float fluid_density, std::array<float, 3> init_flow_velocity, std::array<float, 3> external_force);
    Domain(Domain&) = delete;
    Domain& operator=(Domain&) = delete;
    ~Domain();
    std::tuple<size_t, size_t, size_t> get_dimensions() const;
    float get_fluid_viscosity() const;
    float get_fluid_density() const;
    const std::array<float, 3>& get_init_flow_velocity() const;
    const std::array<float, 3>& get_external_force() const;
    void initialize(SimData& simdata) const;
    const LBModel* get_lbmodel() const { return _lbmodel; }

 private:
    const LBModel* _lbmodel;
    uint32_t _xdim, _ydim, _zdim;
    float _fluid_viscosity;
    float _fluid_density;
    std::array<float, 3> _init_flow_velocity;
    std::array<float, 3> _external_force;
};

#endif  // PLBPD_GB300_DOMAIN_HPP_
