// Declaration-only stand-in (see d_ary_heap.hpp).
#ifndef MCT_SHIM_BOOST_HEAP_FIBONACCI_HEAP_HPP
#define MCT_SHIM_BOOST_HEAP_FIBONACCI_HEAP_HPP
#include "policies.hpp"
namespace boost { namespace heap {
template <class T, class... Options> class fibonacci_heap { public: typedef void *handle_type; };
}}
#endif
