// A two-relaxation-time collision through plbpd's Collision base
// (src/Collision.hpp:10-21), the extension point plbpd leaves for collision
// models other than CollisionSRT.  No counterpart in plbpd.
//
// The even part of each pair of opposite directions relaxes with 1/tau
// (tau = 3 nu + 0.5, as CollisionSRT derives it), the odd part with 1/tau_m,
// tau_m = magic/(tau - 1/2) + 1/2; magic 0 selects 3/16, for which the
// half-way bounce-back wall lies exactly half way between the wall layer and
// the first fluid layer.  The body force enters as a second-order source with
// u + F/(2 rho) in the equilibrium.  Runs on the GPU in place on n, like
// CollisionSRT; it can replace CollisionSRT in a hand-written time loop.
#ifndef PLBPD_GB300_COLLISIONTRT_HPP_
#define PLBPD_GB300_COLLISIONTRT_HPP_

#include "Collision.hpp"
#include "Domain.hpp"
#include "LBModel.hpp"

class CollisionTRT final : public Collision {
 public:
    CollisionTRT() = delete;
    CollisionTRT(const LBModel* lbmodel, const Domain* domain, float magic = 0.0f);
    CollisionTRT(CollisionTRT&) = delete;
    CollisionTRT& operator=(CollisionTRT&) = delete;
    ~CollisionTRT();
    void operator()(SimData& simdata, bool reference = false) const;
    float get_magic() const;

 private:
    const LBModel* _lbmodel;
    const Domain* _domain;
    float _magic;
};

#endif  // PLBPD_GB300_COLLISIONTRT_HPP_
