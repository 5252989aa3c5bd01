// Stand-in for the TBB calls of core/Grid.h and core/*.cpp (TEST INFRASTRUCTURE for oracle/_ref): every
// parallel_for runs its range serially, in index order.  Each loop body the reference runs through it writes
// only its own element, so the serial order gives the same results as any parallel schedule.
#pragma once
#include <type_traits>
namespace tbb {
template <class T> class blocked_range {
  public:
    blocked_range(T b, T e) : b_(b), e_(e) {}
    T begin() const { return b_; }
    T end() const { return e_; }

  private:
    T b_, e_;
};
template <class T> class blocked_range3d {
  public:
    blocked_range3d(T pb, T pe, T rb, T re, T cb, T ce) : p_(pb, pe), r_(rb, re), c_(cb, ce) {}
    const blocked_range<T> &pages() const { return p_; }
    const blocked_range<T> &rows() const { return r_; }
    const blocked_range<T> &cols() const { return c_; }

  private:
    blocked_range<T> p_, r_, c_;
};
template <class T, class F> inline void parallel_for(const blocked_range3d<T> &r, F &&f) { f(r); }
template <class T, class F> inline void parallel_for(const blocked_range<T> &r, F &&f) { f(r); }
template <class I, class J, class F>
    requires(std::is_integral_v<I> && std::is_integral_v<J>)
inline void parallel_for(I b, J e, F &&f) {
    for (I i = b; i < static_cast<I>(e); i++) f(i);
}
} // namespace tbb
