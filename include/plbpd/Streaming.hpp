// plbpd's Streaming interface (src/Streaming.hpp:10-34): "push" streaming into
// ntmp followed by the n/ntmp swap; "pull" is not implemented in plbpd and
// throws std::logic_error here too, and any other type is rejected.
#ifndef PLBPD_GB300_STREAMING_HPP_
#define PLBPD_GB300_STREAMING_HPP_

#include <string>

#include "LBModel.hpp"
#include "SimData.hpp"

class Streaming final {
 public:
    explicit Streaming(const LBModel* lbmodel);
    Streaming(Streaming&) = delete;
    Streaming& operator=(Streaming&) = delete;
    ~Streaming();
    void operator()(SimData& simdata, std::string stream_type, bool reference = false) const;
    float get_total_time() const;

 private:
    const LBModel* _lbmodel;
    static float _time;
};

#endif  // PLBPD_GB300_STREAMING_HPP_
