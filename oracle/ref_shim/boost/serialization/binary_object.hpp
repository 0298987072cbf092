// Oracle-only stub: a do-nothing binary_object so the templated save/load members parse.
#pragma once
#include <cstddef>
namespace boost { namespace serialization {
struct binary_object { void *p; std::size_t n; };
inline binary_object make_binary_object(void *p, std::size_t n) { return binary_object{p, n}; }
inline binary_object make_binary_object(const void *p, std::size_t n) { return binary_object{const_cast<void *>(p), n}; }
} }
