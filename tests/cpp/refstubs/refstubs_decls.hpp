// Declaration-only stand-ins for the third-party headers the LuxCore headers
// include (Boost serialization, archives, iostreams, filesystem, threads;
// LuxCore's generated cfg.h), so that those headers parse for the compile
// check of the LuxRays binding (luxcore_gb300/luxrays/gb300accel.cpp,
// tests/test_luxrays_binding.py).  Nothing here is ever linked or run: each
// name is only declared with the shape the headers use.
#pragma once
#include <fstream>
#include <istream>
#include <ostream>
#include <string>
#include <cmath>
#include <mutex>
#include <thread>
#include <unordered_map>
#define BOOST_VERSION 107400
#define BOOST_CLASS_IMPLEMENTATION(T, L)
#define BOOST_CLASS_EXPORT_KEY(T)
#define BOOST_CLASS_EXPORT_KEY2(T, K)
#define BOOST_CLASS_VERSION(T, N)
#define BOOST_CLASS_TRACKING(T, N)
#define BOOST_SERIALIZATION_SPLIT_MEMBER()
#define BOOST_SERIALIZATION_SPLIT_FREE(T)
#define BOOST_ASSERT(x) ((void)0)
#define BOOST_SERIALIZATION_ASSUME_ABSTRACT(T)
#define BOOST_SERIALIZATION_BASE_OBJECT_NVP(T) 0
#define BOOST_FOREACH(a, b) for (a : b)
namespace boost {
namespace serialization {
class access {};
enum level_type { not_serializable, primitive_type, object_serializable, object_class_info };
enum tracking_type { track_never, track_selectively, track_always };
template <class T> struct base_object_t {};
template <class B, class D> B &base_object(D &d) { return d; }
template <class T> int make_array(T *, std::size_t) { return 0; }
template <class T> int make_nvp(const char *, T &) { return 0; }
}
namespace archive {
class binary_oarchive { public: template <class T> binary_oarchive &operator&(const T &) { return *this; } template <class T> binary_oarchive &operator<<(const T &) { return *this; } };
class binary_iarchive { public: template <class T> binary_iarchive &operator&(T &) { return *this; } template <class T> binary_iarchive &operator>>(T &) { return *this; } };
}
namespace filesystem { typedef std::ofstream ofstream; typedef std::ifstream ifstream; class path { public: path() {} path(const std::string &) {} std::string string() const { return {}; } }; }
namespace iostreams { class filtering_ostream : public std::ostream { public: filtering_ostream() : std::ostream(nullptr) {} }; class filtering_istream : public std::istream { public: filtering_istream() : std::istream(nullptr) {} }; }
namespace math { template <class T> int signbit(T v) { return std::signbit(v); } }
typedef std::mutex mutex;
typedef std::thread thread;
template <class K, class V, class H = std::hash<K>> using unordered_map = std::unordered_map<K, V, H>;
template <class T> std::string lexical_cast_str(const T &) { return {}; }
template <class To, class From> To lexical_cast(const From &) { return To(); }
}
