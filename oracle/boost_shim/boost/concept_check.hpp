// Stand-in for the one Boost facility the reference takes from this header:
// BOOST_CONCEPT_ASSERT((boost::Convertible<A, B>)) inside member functions.
// The check is dropped; the code it guards compiles only for valid types anyway.
#ifndef MCT_SHIM_BOOST_CONCEPT_CHECK_HPP
#define MCT_SHIM_BOOST_CONCEPT_CHECK_HPP
#define BOOST_CONCEPT_ASSERT(Model) ((void)0)
#endif
