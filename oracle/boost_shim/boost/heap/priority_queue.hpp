// Minimal stand-in for boost::heap::priority_queue, written for this project
// so the reference's fastMarching3D compiles without Boost. Only the calls the
// reference makes (push, top, pop, reserve, size, empty, clear) exist; they
// delegate to std::push_heap / std::pop_heap on a std::vector, which is how
// boost::heap::priority_queue stores and orders its elements.
#ifndef MCT_SHIM_BOOST_HEAP_PRIORITY_QUEUE_HPP
#define MCT_SHIM_BOOST_HEAP_PRIORITY_QUEUE_HPP
#include <algorithm>
#include <vector>
#include <cstddef>
#include "policies.hpp"
namespace boost { namespace heap {
template <class T, class... Options> class priority_queue;
template <class T, class Cmp> class priority_queue<T, compare<Cmp>> {
  std::vector<T> q_;
  Cmp cmp_;
 public:
  void reserve(std::size_t n) { q_.reserve(n); }
  void push(const T &v) { q_.push_back(v); std::push_heap(q_.begin(), q_.end(), cmp_); }
  const T &top() const { return q_.front(); }
  void pop() { std::pop_heap(q_.begin(), q_.end(), cmp_); q_.pop_back(); }
  std::size_t size() const { return q_.size(); }
  bool empty() const { return q_.empty(); }
  void clear() { q_.clear(); }
};
}}  // namespace boost::heap
#endif
