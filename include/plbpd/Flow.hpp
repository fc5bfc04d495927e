// plbpd's flow presets (src/Flow.hpp:11-32): "Couette2D", "Couette3D",
// "Poiseuille2D", "Poiseuille3D" with the reference's parameters
// (src/Flow.cpp:20-106); an unknown name throws std::invalid_argument.
#ifndef PLBPD_GB300_FLOW_HPP_
#define PLBPD_GB300_FLOW_HPP_

#include <memory>
#include <string>

#include "Boundary.hpp"
#include "Domain.hpp"
#include "LBModel.hpp"

class Flow final {
 public:
    explicit Flow(std::string flow_type);
    Flow(Flow&) = delete;
    Flow& operator=(Flow&) = delete;
    ~Flow();
    const Domain* get_domain() const;
    const Boundary* get_boundary() const;
    const LBModel* get_lbmodel() const;
    size_t get_num_timesteps() const;

 private:
    std::unique_ptr<LBModel> _lbmodel;
    std::unique_ptr<Domain> _domain;
    std::unique_ptr<Boundary> _boundary;
    uint32_t _num_timesteps;
};

#endif  // PLBPD_GB300_FLOW_HPP_
