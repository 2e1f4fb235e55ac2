// Stand-in for the Boost.Serialization declarations that the reference headers
// name. Nothing here serializes: the reference's serialize() members are
// templates that are never instantiated by the oracle driver, so only the
// names they use have to exist.
#ifndef REFSHIM_BOOST_SERIALIZATION_HPP
#define REFSHIM_BOOST_SERIALIZATION_HPP
#include <cstddef>
#include <limits>
#include <iostream>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>
namespace boost {
namespace serialization {
class access {};
template <class Base, class Derived> Base& base_object(Derived& d) { return static_cast<Base&>(d); }
template <class Derived, class Base> inline const void* void_cast_register(const Derived*, const Base*) { return nullptr; }
template <class Archive, class T> inline void save_construct_data(Archive&, const T*, const unsigned int) {}
template <class Archive, class T> inline void load_construct_data(Archive&, T*, const unsigned int) {}
struct binary_object {
  binary_object(void* p, std::size_t n) : m_t(p), m_size(n) {}
  void* m_t;
  std::size_t m_size;
};
}  // namespace serialization
}  // namespace boost
#define BOOST_SERIALIZATION_SPLIT_MEMBER()
#define BOOST_CLASS_EXPORT(T)
#define BOOST_CLASS_EXPORT_GUID(T, K)
#define BOOST_CLASS_EXPORT_KEY(T)
#define BOOST_CLASS_EXPORT_IMPLEMENT(T)
#endif
