// Field storage with plbpd's interface (src/Field.hpp:11-151): a z-major grid
// of V-vectors with `num_buffer_layers` halo layers on every axis, element
// index z*zf + y*yf + x*xf + v in uint32 arithmetic, extents that exclude the
// halo, and the neighbour rule (z + c2, y + c1, x + c0).
//
// When a Field belongs to a SimData whose state lives on the GPU, the
// SimData attaches an access hook: any access first brings the host copy up
// to date, and a non-const access marks the host copy as changed so the next
// device operator uploads it.  A Field without a hook is plain host storage.
#ifndef PLBPD_GB300_FIELD_HPP_
#define PLBPD_GB300_FIELD_HPP_

#include <array>
#include <cstdint>
#include <stdexcept>
#include <tuple>
#include <vector>

namespace Field {

struct FieldExtents {
    uint32_t zbegin, zend;
    uint32_t ybegin, yend;
    uint32_t xbegin, xend;
};

// Hook a device-backed owner installs on its fields.
struct AccessHook {
    bool device_newer = false;   // the device holds newer values than the host
    bool host_dirty = false;     // the host copy changed since the last upload
    void (*pull)(AccessHook*) = nullptr;
    void* owner = nullptr;
    inline void before(bool write) {
        if (device_newer && pull) pull(this);
        if (write) host_dirty = true;
    }
};

template <typename T, uint32_t num_buffer_layers>
class VectorField {
 public:
    VectorField(const uint32_t zlen, const uint32_t ylen, const uint32_t xlen, const uint32_t vlen,
                const T& value) {
        for (uint32_t a : {zlen, ylen, xlen, vlen})
            if (a == 0) throw std::invalid_argument("argument is zero");
        _zlen = zlen + 2 * num_buffer_layers;
        _ylen = ylen + 2 * num_buffer_layers;
        _xlen = xlen + 2 * num_buffer_layers;
        _vlen = vlen;
        _data.assign(static_cast<size_t>(_zlen) * _ylen * _xlen * _vlen, value);
        _xf = _vlen;
        _yf = _vlen * _xlen;
        _zf = _vlen * _xlen * _ylen;
        _e = {num_buffer_layers, _zlen - num_buffer_layers, num_buffer_layers, _ylen - num_buffer_layers,
              num_buffer_layers, _xlen - num_buffer_layers};
    }
    ~VectorField() {}
    VectorField(VectorField&) = delete;
    VectorField& operator=(VectorField&) = delete;

    inline std::tuple<uint32_t, uint32_t, uint32_t> get_dimensions() const {
        return std::make_tuple(_zlen, _ylen, _xlen);
    }
    inline uint32_t get_vector_length() const { return _vlen; }
    inline const FieldExtents& get_extents() const { return _e; }
    inline uint32_t sub2ind(uint32_t z, uint32_t y, uint32_t x, uint32_t v) {
        return z * _zf + y * _yf + x * _xf + v;
    }
    inline uint32_t sub2ind(uint32_t z, uint32_t y, uint32_t x, uint32_t v) const {
        return z * _zf + y * _yf + x * _xf + v;
    }
    inline T& at(uint32_t z, uint32_t y, uint32_t x, uint32_t v) {
        if (_hook) _hook->before(true);
        return _data[sub2ind(z, y, x, v)];
    }
    inline const T& at(uint32_t z, uint32_t y, uint32_t x, uint32_t v) const {
        if (_hook) _hook->before(false);
        return _data[sub2ind(z, y, x, v)];
    }
    inline const T* get(uint32_t z, uint32_t y, uint32_t x, uint32_t v) const {
        if (_hook) _hook->before(false);
        return &_data[sub2ind(z, y, x, v)];
    }
    inline T* get(uint32_t z, uint32_t y, uint32_t x, uint32_t v) {
        if (_hook) _hook->before(true);
        return &_data[sub2ind(z, y, x, v)];
    }
    inline std::tuple<uint32_t, uint32_t, uint32_t> get_neighbor(uint32_t z, uint32_t y, uint32_t x,
                                                                  const std::array<int32_t, 3>& ck) const {
        return std::make_tuple(z + ck[2], y + ck[1], x + ck[0]);
    }

    // -- for device-backed owners -------------------------------------------
    void set_access_hook(AccessHook* h) { _hook = h; }
    T* raw() { return _data.data(); }
    const T* raw() const { return _data.data(); }
    size_t size() const { return _data.size(); }

 private:
    uint32_t _zlen, _ylen, _xlen, _vlen;
    uint32_t _zf, _yf, _xf;
    FieldExtents _e;
    std::vector<T> _data;
    AccessHook* _hook = nullptr;
};

template <typename T, uint32_t num_buffer_layers>
class ScalarField : public VectorField<T, num_buffer_layers> {
    using Base = VectorField<T, num_buffer_layers>;

 public:
    ScalarField(uint32_t zlen, uint32_t ylen, uint32_t xlen, const T& value) : Base(zlen, ylen, xlen, 1, value) {}
    ~ScalarField() {}
    ScalarField(ScalarField&) = delete;
    ScalarField& operator=(ScalarField&) = delete;
    inline uint32_t sub2ind(uint32_t z, uint32_t y, uint32_t x) { return Base::sub2ind(z, y, x, 0); }
    inline T& at(uint32_t z, uint32_t y, uint32_t x) { return Base::at(z, y, x, 0); }
    inline const T& at(uint32_t z, uint32_t y, uint32_t x) const { return Base::at(z, y, x, 0); }
    inline const T* get(uint32_t z, uint32_t y, uint32_t x) const { return Base::get(z, y, x, 0); }
    inline T* get(uint32_t z, uint32_t y, uint32_t x) { return Base::get(z, y, x, 0); }
    using Base::at;
    using Base::get;
    using Base::sub2ind;
};

}  // namespace Field

#endif  // PLBPD_GB300_FIELD_HPP_
