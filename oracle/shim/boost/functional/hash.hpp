/* Stand-in for the one boost facility the reference tree code names: a hash
 * functor for std::pair<double, double>.  Test infrastructure. */
#ifndef ORACLE_SHIM_BOOST_HASH_HPP
#define ORACLE_SHIM_BOOST_HASH_HPP
#include <cstddef>
#include <functional>
#include <utility>
namespace boost {
template <class T> struct hash;
template <class A, class B> struct hash<std::pair<A, B>> {
  std::size_t operator()(const std::pair<A, B>& p) const {
    std::size_t h = std::hash<A>()(p.first);
    return h ^ (std::hash<B>()(p.second) + 0x9e3779b97f4a7c15ULL + (h << 6) + (h >> 2));
  }
};
}  // namespace boost
#endif
