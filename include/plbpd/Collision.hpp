// plbpd's Collision base (src/Collision.hpp:10-21): the extension point for
// collision models, with a process-wide timer.
#ifndef PLBPD_GB300_COLLISION_HPP_
#define PLBPD_GB300_COLLISION_HPP_

#include "LBModel.hpp"
#include "SimData.hpp"

class Collision {
 protected:
    static float _time;

 public:
    Collision();
    Collision(Collision&) = delete;
    Collision& operator=(Collision&) = delete;
    virtual ~Collision();
    virtual void operator()(SimData& simdata, bool reference) const = 0;
    float get_total_time() const;
};

#endif  // PLBPD_GB300_COLLISION_HPP_
