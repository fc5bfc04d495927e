// plbpd's SimData interface (src/SimData.hpp:9-31): the four public fields
// rho, u, n and ntmp with one halo layer.  Here the state lives on the GPU
// while operators run: the host fields are a mirror that is brought up to
// date when accessed, and host changes are uploaded before the next device
// operator.  n and ntmp are swapped by streaming exactly as in plbpd.
#ifndef PLBPD_GB300_SIMDATA_HPP_
#define PLBPD_GB300_SIMDATA_HPP_

#include <cstdint>
#include <memory>
#include <string>
#include <tuple>

#include "Field.hpp"

struct plb_solve;
struct plb_params;

class SimData final {
 public:
    Field::ScalarField<float, 1>* rho;
    Field::VectorField<float, 1>* u;
    Field::VectorField<float, 1>* n;
    Field::VectorField<float, 1>* ntmp;

    SimData() = delete;
    SimData(const std::tuple<size_t, size_t, size_t> domain_dimensions, const size_t num_directions);
    SimData(SimData&& other) noexcept;
    SimData(const SimData&) = delete;
    SimData& operator=(SimData&) = delete;
    ~SimData();
    // Writes /Density (z+2, y+2, x+2) and /FlowVelocity (z+2, y+2, x+2, 3),
    // as plbpd does (src/SimData.cpp:83-160), plus the populations
    // /ParticleDistribution and /ParticleDistributionTmp, in the raw
    // "plb-state-v1" container (a JSON header line, then float32 data).
    void write_state(std::string dump_file);
    // Restores all four fields from a file written by write_state.
    void read_state(std::string dump_file);

    // -- GB300 additions ---------------------------------------------------
    // Collision arithmetic of the device state: PLB_ARITH_REFERENCE (default,
    // bit-exact with plbpd) or PLB_ARITH_FP32.  Set before the first operator.
    void set_arithmetic(int arith);
    // Device state for an operator: created on first use with `p`, host
    // changes uploaded.  Operators call this, then mark_device_newer().
    plb_solve* device_for(const plb_params& p);
    void mark_device_newer();
    // Brings the host fields up to date with the device.
    void pull();
    size_t num_directions() const { return _kdim; }
    std::tuple<size_t, size_t, size_t> dimensions() const { return _dims; }

 private:
    void _bootstrap();
    void _attach_hooks();
    void _upload();
    std::tuple<size_t, size_t, size_t> _dims;
    size_t _kdim;
    int _arith;
    plb_solve* _solve = nullptr;
    std::unique_ptr<Field::AccessHook> _hook;
};

#endif  // PLBPD_GB300_SIMDATA_HPP_
