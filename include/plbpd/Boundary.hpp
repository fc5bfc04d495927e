// plbpd's Boundary interface (src/Boundary.hpp:14-79): face types
// ("periodic" / "noslip") and wall velocities by face name (east, west,
// north, south, up, down); no-slip, periodic copies and wall resets run on
// the GPU with plbpd's exact semantics.
#ifndef PLBPD_GB300_BOUNDARY_HPP_
#define PLBPD_GB300_BOUNDARY_HPP_

#include <array>
#include <string>
#include <unordered_map>
#include <vector>

#include "Domain.hpp"
#include "LBModel.hpp"
#include "SimData.hpp"

using fVectorField = Field::VectorField<float, 1>;
using fScalarField = Field::ScalarField<float, 1>;
using BoundaryType = std::unordered_map<std::string, std::string>;
using BoundaryVelocity = std::unordered_map<std::string, std::array<float, 3> >;

class Boundary final {
 public:
    Boundary() = delete;
    Boundary(const LBModel* lbmodel, const Domain* domain, const float solid_density, BoundaryType type,
             BoundaryVelocity velocity);
    Boundary(Boundary&) = delete;
    Boundary& operator=(Boundary&) = delete;
    ~Boundary();

    void reset(SimData& simdata) const;
    const BoundaryType get_boundary_type() const;
    const BoundaryVelocity get_boundary_velocity() const;
    void reset_velocity(SimData& simdata) const;
    void reset_density(SimData& simdata) const;
    void apply_periodicity(SimData& simdata) const;
    void apply_noslip(SimData& simdata) const;
    float get_time_noslip() const;
    float get_time_periodicity() const;
    float get_time_reset() const;
    float get_time_velocity_reset() const;
    float get_time_density_reset() const;
    float get_total_time() const;

    // -- GB300 additions ---------------------------------------------------
    // Face arrays in plbpd's face order for the C ABI.
    void face_arrays(int32_t* type6, int32_t* has_vel6, float* vel18) const;
    float get_solid_density() const { return _solid_density; }
    // Throws std::out_of_range, as plbpd's map lookup does, when a no-slip
    // face has no velocity entry (src/Boundary.cpp:197).
    void check_noslip_velocities() const;

 private:
    const LBModel* _lbmodel;
    const Domain* _domain;
    const float _solid_density;
    BoundaryType _type;
    BoundaryVelocity _velocity;
    static float _time_noslip;
    static float _time_periodicity;
    static float _time_reset;
    static float _time_velocity_reset;
    static float _time_density_reset;
    static const std::vector<std::string> _directions;
};

#endif  // PLBPD_GB300_BOUNDARY_HPP_
