// Option tags used by the reference's heap typedefs (stand-in, see priority_queue.hpp).
#ifndef MCT_SHIM_BOOST_HEAP_POLICIES_HPP
#define MCT_SHIM_BOOST_HEAP_POLICIES_HPP
namespace boost { namespace heap {
template <class C> struct compare {};
template <bool B> struct mutable_ {};
template <unsigned N> struct arity {};
}}  // namespace boost::heap
#endif
