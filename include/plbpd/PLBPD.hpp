// plbpd's driver (src/PLBPD.hpp:12-29).  march_in_time runs the whole loop --
// collide, push, no-slip, periodic copy, moments, reset -- as fused GPU
// kernels, with plbpd's results bit for bit.
#ifndef PLBPD_GB300_PLBPD_HPP_
#define PLBPD_GB300_PLBPD_HPP_

#include <memory>

#include "Boundary.hpp"
#include "CalcMoments.hpp"
#include "Domain.hpp"
#include "Flow.hpp"
#include "LBDynamics.hpp"
#include "LBModel.hpp"
#include "SimData.hpp"

class PLBPD final {
 public:
    PLBPD(const LBModel* lbmodel, const Domain* domain, const Boundary* boundary);
    PLBPD(PLBPD&) = delete;
    PLBPD& operator=(PLBPD&) = delete;
    ~PLBPD();
    void initialize(SimData& simdata) const;
    void march_in_time(size_t num_timesteps, SimData& simdata) const;
    void print_times() const;

 private:
    const LBModel* _lbmodel;
    const Domain* _domain;
    const Boundary* _boundary;
    std::unique_ptr<LBDynamics> _lbdynamics;
    std::unique_ptr<CalcMoments> _calc_moments;
    static float _time_march;
};

#endif  // PLBPD_GB300_PLBPD_HPP_
