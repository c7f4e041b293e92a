// Minimal stand-in for boost::hash / boost::hash_combine as used by the
// reference's hashed containers and its LRU key. Test infrastructure only.
// The combine step is the widely published golden-ratio mix
// (seed ^= h + 0x9e3779b9 + (seed << 6) + (seed >> 2)). Hash values only pick
// buckets and LRU keys; no result the oracle reports depends on them.
#ifndef LMC_ORACLE_SHIM_BOOST_HASH_
#define LMC_ORACLE_SHIM_BOOST_HASH_
#include <cstddef>
#include <functional>
#include <type_traits>
#include <utility>
namespace boost {
template <typename T>
inline typename std::enable_if<std::is_integral<T>::value || std::is_enum<T>::value, std::size_t>::type
hash_value(T v) {
  return static_cast<std::size_t>(v);
}
template <typename T>
struct hash;
template <typename T>
inline void hash_combine(std::size_t &seed, const T &v);
template <typename A, typename B>
inline std::size_t hash_value(const std::pair<A, B> &p) {
  std::size_t seed = 0;
  hash_combine(seed, p.first);
  hash_combine(seed, p.second);
  return seed;
}
template <typename T>
struct hash {
  std::size_t operator()(const T &v) const {
    using boost::hash_value;
    return hash_value(v);
  }
};
template <typename T>
inline void hash_combine(std::size_t &seed, const T &v) {
  const std::size_t h = boost::hash<T>()(v);
  seed ^= h + 0x9e3779b9u + (seed << 6) + (seed >> 2);
}
}  // namespace boost
#endif
