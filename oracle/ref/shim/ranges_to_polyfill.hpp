// Oracle build shim (test infrastructure only): g++ 13 lacks C++23
// std::ranges::to, which two reference translation units use to collect a
// view into a std::vector.  This minimal stand-in covers exactly those uses.
#pragma once
#include <ranges>
#include <vector>
#include <iterator>
#if !defined(__cpp_lib_ranges_to_container)
namespace std::ranges {
namespace mango_shim {
template <template <class...> class C> struct to_tmpl {};
template <class C> struct to_cont {};
template <template <class...> class C, class R>
auto operator|(R&& r, to_tmpl<C>) {
  using V = std::ranges::range_value_t<R>;
  C<V> out;
  for (auto&& e : r) out.push_back(e);
  return out;
}
template <class C, class R>
C operator|(R&& r, to_cont<C>) {
  C out;
  for (auto&& e : r) out.push_back(e);
  return out;
}
}  // namespace mango_shim
template <template <class...> class C> mango_shim::to_tmpl<C> to() { return {}; }
template <class C> mango_shim::to_cont<C> to() { return {}; }
template <class C, class R> C to(R&& r) { return std::forward<R>(r) | mango_shim::to_cont<C>{}; }
}  // namespace std::ranges
#endif
