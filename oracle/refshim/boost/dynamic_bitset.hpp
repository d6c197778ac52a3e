// Minimal stand-in for boost::dynamic_bitset<> as the CEOs reference sources
// use it (construction by size, element read/write through a proxy, ~proxy,
// count, find_first/find_next, npos, clear, size), written for this project
// from Boost's documented interface so those sources compile unchanged for
// parity pinning (test infrastructure only).
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

namespace boost {

template <typename Block = unsigned long>
class dynamic_bitset {
 public:
  typedef std::size_t size_type;
  static const size_type npos = static_cast<size_type>(-1);

  class reference {
   public:
    reference(dynamic_bitset& b, size_type i) : b_(b), i_(i) {}
    operator bool() const { return b_.test(i_); }
    bool operator~() const { return !b_.test(i_); }
    reference& operator=(bool v) {
      b_.set(i_, v);
      return *this;
    }
    reference& operator=(const reference& o) { return *this = bool(o); }

   private:
    dynamic_bitset& b_;
    size_type i_;
  };

  dynamic_bitset() : n_(0) {}
  explicit dynamic_bitset(size_type n) : n_(n), w_((n + 63) / 64, 0) {}

  size_type size() const { return n_; }
  void clear() {
    n_ = 0;
    w_.clear();
  }
  void resize(size_type n) {
    n_ = n;
    w_.resize((n + 63) / 64, 0);
  }
  bool test(size_type i) const { return (w_[i >> 6] >> (i & 63)) & 1u; }
  dynamic_bitset& set(size_type i, bool v = true) {
    if (v) w_[i >> 6] |= (uint64_t)1 << (i & 63);
    else w_[i >> 6] &= ~((uint64_t)1 << (i & 63));
    return *this;
  }
  dynamic_bitset& reset(size_type i) { return set(i, false); }
  bool operator[](size_type i) const { return test(i); }
  reference operator[](size_type i) { return reference(*this, i); }
  size_type count() const {
    size_type c = 0;
    for (uint64_t w : w_) c += (size_type)__builtin_popcountll(w);
    return c;
  }
  size_type find_first() const { return scan_from(0); }
  size_type find_next(size_type i) const { return i + 1 >= n_ ? npos : scan_from(i + 1); }

 private:
  size_type scan_from(size_type i) const {
    size_type wi = i >> 6;
    if (wi >= w_.size()) return npos;
    uint64_t w = w_[wi] & (~(uint64_t)0 << (i & 63));
    while (true) {
      if (w) {
        const size_type pos = (wi << 6) + (size_type)__builtin_ctzll(w);
        return pos < n_ ? pos : npos;
      }
      if (++wi >= w_.size()) return npos;
      w = w_[wi];
    }
  }
  size_type n_;
  std::vector<uint64_t> w_;
};

}  // namespace boost
