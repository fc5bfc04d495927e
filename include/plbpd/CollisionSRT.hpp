// plbpd's CollisionSRT interface (src/CollisionSRT.hpp:11-45): BGK collision,
// tau = 3 nu + 0.5, omega = 1/tau, body force as a velocity shift.  Runs on
// the GPU in place on n; `reference` selects plbpd's serial kernel, which
// gives the same result here.
#ifndef PLBPD_GB300_COLLISIONSRT_HPP_
#define PLBPD_GB300_COLLISIONSRT_HPP_

#include <array>

#include "Collision.hpp"
#include "Domain.hpp"
#include "LBModel.hpp"

class CollisionSRT final : public Collision {
 public:
    CollisionSRT() = delete;
    CollisionSRT(const LBModel* lbmodel, const Domain* domain);
    CollisionSRT(CollisionSRT&) = delete;
    CollisionSRT& operator=(CollisionSRT&) = delete;
    ~CollisionSRT();
    void operator()(SimData& simdata, bool reference = false) const;

 private:
    const LBModel* _lbmodel;
    const Domain* _domain;
};

#endif  // PLBPD_GB300_COLLISIONSRT_HPP_
