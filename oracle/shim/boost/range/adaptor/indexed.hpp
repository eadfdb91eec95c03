// Stand-in for boost::adaptors::indexed (test infrastructure only).
//
// The LPM reference iterates `range | indexed(0)` and reads `.index()` and
// `.value()` from each element (stiffness.h:239-246).  This header provides
// exactly that, written from Boost.Range's documented behaviour.
#pragma once

#include <cstddef>
#include <iterator>
#include <utility>

namespace boost {
namespace adaptors {

struct indexed {
  std::ptrdiff_t start;
  explicit indexed(std::ptrdiff_t s = 0) : start(s) {}
};

template <class Range>
class indexed_range {
 public:
  typedef decltype(std::declval<Range&>().begin()) base_iterator;
  typedef decltype(*std::declval<base_iterator>()) reference;

  struct element {
    std::ptrdiff_t i;
    base_iterator it;
    std::ptrdiff_t index() const { return i; }
    reference value() const { return *it; }
  };

  struct iterator {
    base_iterator it;
    std::ptrdiff_t i;
    element operator*() const { return element{i, it}; }
    iterator& operator++() {
      ++it;
      ++i;
      return *this;
    }
    bool operator!=(const iterator& o) const { return it != o.it; }
    bool operator==(const iterator& o) const { return it == o.it; }
  };

  indexed_range(Range& r, std::ptrdiff_t s) : r_(r), start_(s) {}
  iterator begin() const { return iterator{r_.begin(), start_}; }
  iterator end() const { return iterator{r_.end(), start_}; }

 private:
  Range& r_;
  std::ptrdiff_t start_;
};

template <class Range>
indexed_range<Range> operator|(Range& r, indexed f) {
  return indexed_range<Range>(r, f.start);
}

}  // namespace adaptors
}  // namespace boost
