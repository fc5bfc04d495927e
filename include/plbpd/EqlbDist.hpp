// plbpd's EqlbDist interface (src/EqlbDist.hpp:10-39): equilibrium populations
// of one node, with the reference's rounding (plb_equilibrium).
#ifndef PLBPD_GB300_EQLBDIST_HPP_
#define PLBPD_GB300_EQLBDIST_HPP_

#include <array>
#include <vector>

#include "LBModel.hpp"

class EqlbDist final {
 public:
    explicit EqlbDist(const LBModel* lbmodel);
    EqlbDist(const EqlbDist&) = delete;
    EqlbDist& operator=(const EqlbDist&) = delete;
    ~EqlbDist() {}
    void operator()(const float rholocal, const std::array<float, 3>& ulocal, std::vector<float>& nlocal);

 private:
    const uint32_t _kdim;
};

#endif  // PLBPD_GB300_EQLBDIST_HPP_
