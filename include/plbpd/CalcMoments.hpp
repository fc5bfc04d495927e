// plbpd's CalcMoments interface (src/CalcMoments.hpp:15-74): rho and u on
// every interior node, summed in direction order.
#ifndef PLBPD_GB300_CALCMOMENTS_HPP_
#define PLBPD_GB300_CALCMOMENTS_HPP_

#include "LBModel.hpp"
#include "SimData.hpp"

class CalcMoments final {
 public:
    explicit CalcMoments(const LBModel* lbmodel);
    CalcMoments(const CalcMoments&) = delete;
    CalcMoments& operator=(const CalcMoments&) = delete;
    ~CalcMoments();
    float get_total_time() const;
    void operator()(SimData& simdata) const;

 private:
    const LBModel* _lbmodel;
    static float _time_calc_moment;
};

#endif  // PLBPD_GB300_CALCMOMENTS_HPP_
