// Declaration-only stand-in: the reference names boost::heap::d_ary_heap in a
// class template that the compiled entry point never instantiates.
#ifndef MCT_SHIM_BOOST_HEAP_D_ARY_HEAP_HPP
#define MCT_SHIM_BOOST_HEAP_D_ARY_HEAP_HPP
#include "policies.hpp"
namespace boost { namespace heap {
template <class T, class... Options> class d_ary_heap { public: typedef void *handle_type; };
}}
#endif
