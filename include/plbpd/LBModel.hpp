// plbpd's LBModel interface (src/LBModel.hpp:8-35): lattice tables by name.
// The tables come from libplb_gb300 (plb_model_tables), the same ones the
// kernels use.  An unknown name throws std::logic_error, as plbpd does.
#ifndef PLBPD_GB300_LBMODEL_HPP_
#define PLBPD_GB300_LBMODEL_HPP_

#include <array>
#include <cstdint>
#include <string>
#include <vector>

class LBModel final {
 public:
    LBModel() = delete;
    explicit LBModel(std::string model_name);
    LBModel(LBModel&) = delete;
    LBModel& operator=(LBModel&) = delete;
    virtual ~LBModel();
    std::string get_model_name() const;
    uint32_t get_num_directions() const;
    float get_speed_of_sound_squared() const;
    const std::vector<std::array<int32_t, 3> >& get_directional_velocities() const;
    const std::vector<float>& get_directional_weights() const;
    const std::vector<uint32_t>& get_reverse() const;

 private:
    std::string _name;
    uint32_t _q;
    float _cs2;
    std::vector<std::array<int32_t, 3> > _c;
    std::vector<float> _w;
    std::vector<uint32_t> _rev;
};

#endif  // PLBPD_GB300_LBMODEL_HPP_
