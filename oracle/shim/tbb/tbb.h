// Stand-in for the Intel TBB pieces that the reference lattice-Boltzmann
// sources use.  TBB 2018 U2 (pinned by the reference's build environment) is
// not installed here, so this header supplies the same three names:
//
//   * tbb::parallel_for(first, last, f)              index form, f(size_t)
//   * tbb::parallel_for(tbb::blocked_range3d<T>, f)  f(const blocked_range3d&)
//   * tbb::tick_count::now() / (a - b).seconds()
//
// Parallelism comes from OpenMP when the translation unit is compiled with
// -fopenmp (the timed CPU baseline), otherwise every loop runs serially in
// ascending index order (the deterministic order the parity oracle relies on).
// Oracle-only test infrastructure: never linked into the product library.
#ifndef PLB_ORACLE_SHIM_TBB_H_
#define PLB_ORACLE_SHIM_TBB_H_

#include <chrono>
#include <cstddef>
#include <cstdint>
#if defined(_OPENMP)
#include <omp.h>
#endif

namespace tbb {

template <typename Value>
class blocked_range {
 public:
    blocked_range(Value b, Value e) : _b(b), _e(e) {}
    Value begin() const { return _b; }
    Value end() const { return _e; }
    size_t size() const { return static_cast<size_t>(_e - _b); }
 private:
    Value _b, _e;
};

template <typename Value>
class blocked_range3d {
 public:
    blocked_range3d(Value page_begin, Value page_end,
                    Value row_begin, Value row_end,
                    Value col_begin, Value col_end)
        : _pages(page_begin, page_end), _rows(row_begin, row_end),
          _cols(col_begin, col_end) {}
    const blocked_range<Value>& pages() const { return _pages; }
    const blocked_range<Value>& rows() const { return _rows; }
    const blocked_range<Value>& cols() const { return _cols; }
 private:
    blocked_range<Value> _pages, _rows, _cols;
};

// Index form: f(i) for i in [first, last).
template <typename Index, typename Func>
void parallel_for(Index first, Index last, const Func& f) {
#if defined(_OPENMP)
    const long long n = static_cast<long long>(last) - static_cast<long long>(first);
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; ++i)
        f(static_cast<size_t>(first + static_cast<Index>(i)));
#else
    for (Index i = first; i < last; ++i)
        f(static_cast<size_t>(i));
#endif
}

// Range form over a 3-D box: the pages (outermost) are split between threads;
// each thread sees whole rows and columns of its pages.
template <typename Value, typename Func>
void parallel_for(const blocked_range3d<Value>& r, const Func& f) {
#if defined(_OPENMP)
    const long long pb = r.pages().begin(), pe = r.pages().end();
    if (pe - pb > 1 && omp_get_max_threads() > 1) {
#pragma omp parallel for schedule(static)
        for (long long p = pb; p < pe; ++p) {
            blocked_range3d<Value> sub(static_cast<Value>(p), static_cast<Value>(p + 1),
                                       r.rows().begin(), r.rows().end(),
                                       r.cols().begin(), r.cols().end());
            f(sub);
        }
        return;
    }
#endif
    f(r);
}

class tick_count {
 public:
    class interval_t {
     public:
        explicit interval_t(double s) : _s(s) {}
        double seconds() const { return _s; }
     private:
        double _s;
    };
    static tick_count now() {
        tick_count t;
        t._t = std::chrono::steady_clock::now();
        return t;
    }
    interval_t operator-(const tick_count& o) const {
        return interval_t(std::chrono::duration<double>(_t - o._t).count());
    }
 private:
    std::chrono::steady_clock::time_point _t;
};

}  // namespace tbb

#endif  // PLB_ORACLE_SHIM_TBB_H_
