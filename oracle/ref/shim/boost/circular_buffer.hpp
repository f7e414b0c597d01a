// Minimal boost::circular_buffer stand-in (push_back, size, operator[])
// for the oracle's reference build.
#pragma once
#include <cstddef>
#include <deque>
namespace boost {
template <class T>
class circular_buffer {
 public:
  explicit circular_buffer(std::size_t capacity) : cap_(capacity) {}
  void push_back(const T& v) {
    if (cap_ == 0) return;
    if (d_.size() == cap_) d_.pop_front();
    d_.push_back(v);
  }
  std::size_t size() const { return d_.size(); }
  T& operator[](std::size_t i) { return d_[i]; }
  const T& operator[](std::size_t i) const { return d_[i]; }

 private:
  std::size_t cap_;
  std::deque<T> d_;
};
}  // namespace boost
