// plbpd's LBDynamics facade (src/LBDynamics.hpp:13-33): collide and stream.
#ifndef PLBPD_GB300_LBDYNAMICS_HPP_
#define PLBPD_GB300_LBDYNAMICS_HPP_

#include <memory>
#include <string>

#include "CollisionSRT.hpp"
#include "Domain.hpp"
#include "LBModel.hpp"
#include "SimData.hpp"
#include "Streaming.hpp"

class LBDynamics final {
 public:
    LBDynamics() = delete;
    LBDynamics(const LBModel* lbmodel, const Domain* domain);
    LBDynamics(LBDynamics&) = delete;
    LBDynamics& operator=(LBDynamics&) = delete;
    ~LBDynamics();
    void collide(SimData& simdata, bool reference = false) const;
    void stream(SimData& simdata, std::string stream_type, bool reference = false) const;
    float get_time_collide() const;
    float get_time_stream() const;
    float get_total_time() const;

 private:
    std::unique_ptr<CollisionSRT> _collide;
    std::unique_ptr<Streaming> _stream;
};

#endif  // PLBPD_GB300_LBDYNAMICS_HPP_
