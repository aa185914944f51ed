// Stand-in archives: the harness never serialises, it only needs the names.
#pragma once
#include <iosfwd>
namespace boost { namespace archive {
struct binary_oarchive { explicit binary_oarchive(std::ostream &) {} template <class T> binary_oarchive &operator<<(const T &) { return *this; } template <class T> binary_oarchive &operator&(const T &) { return *this; } };
struct binary_iarchive { explicit binary_iarchive(std::istream &) {} template <class T> binary_iarchive &operator>>(T &) { return *this; } template <class T> binary_iarchive &operator&(T &) { return *this; } };
typedef binary_oarchive text_oarchive;
typedef binary_iarchive text_iarchive;
}}  // namespace boost::archive
