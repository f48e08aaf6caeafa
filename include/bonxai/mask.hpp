// Bonxai::Mask, the bit set of one grid node, with the interface of the
// reference's bonxai_core/include/bonxai/mask.hpp:19-140 so that caller code
// that walks nodes (rootMap(), getLeafGrid(), Serialize) compiles unchanged.
//
// On the GPU the masks live inside the device pools as plain 64-bit words;
// this class is the host-side form used by the node snapshots of
// include/bonxai/bonxai.hpp. A mask of log2dim has 2^(3*log2dim) bits stored
// in max(bits/64, 1) words; bit i is bit (i & 63) of word (i >> 6), the same
// word layout as the device pools and the serialized stream.
#pragma once

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <vector>

namespace Bonxai {

class Mask {
 public:
  explicit Mask(size_t log2dim) : Mask(log2dim, false) {}
  Mask(size_t log2dim, bool on)
      : size_(1u << (3 * log2dim)),
        words_(std::max<uint32_t>(size_ >> 6, 1u), on ? ~uint64_t(0) : uint64_t(0)) {
    trim();
  }

  size_t memUsage() const { return sizeof(Mask) + words_.size() * sizeof(uint64_t); }
  uint32_t bitCount() const { return size_; }
  uint32_t size() const { return size_; }
  uint32_t wordCount() const { return static_cast<uint32_t>(words_.size()); }
  uint64_t getWord(size_t n) const { return words_[n]; }
  void setWord(size_t n, uint64_t v) {
    words_[n] = v;
    trim();
  }

  uint32_t countOn() const {
    uint32_t c = 0;
    for (uint64_t w : words_) c += CountOn(w);
    return c;
  }

  /// Iterates the indices of the set bits, lowest first (mask.hpp:59-84).
  class Iterator {
   public:
    Iterator(const Mask* parent) : pos_(parent->size_), parent_(parent) {}
    Iterator(uint32_t pos, const Mask* parent) : pos_(pos), parent_(parent) {}
    Iterator& operator=(const Iterator&) = default;
    uint32_t operator*() const { return pos_; }
    operator bool() const { return pos_ != parent_->size_; }
    Iterator& operator++() {
      pos_ = parent_->findNextOn(pos_ + 1);
      return *this;
    }

   private:
    uint32_t pos_;
    const Mask* parent_;
  };

  bool operator==(const Mask& o) const { return size_ == o.size_ && words_ == o.words_; }
  bool operator!=(const Mask& o) const { return !(*this == o); }

  Iterator beginOn() const { return Iterator(findFirstOn(), this); }

  bool isOn(uint32_t n) const { return (words_[n >> 6] >> (n & 63)) & 1u; }
  /// Every bit on.
  bool isOn() const {
    const uint64_t full = size_ < 64 ? (uint64_t(1) << size_) - 1 : ~uint64_t(0);
    for (uint64_t w : words_)
      if (w != full) return false;
    return true;
  }
  /// Every bit off.
  bool isOff() const {
    for (uint64_t w : words_)
      if (w) return false;
    return true;
  }
  /// setOn / setOff return the previous state of the bit (mask.hpp:351-365).
  bool setOn(uint32_t n) {
    uint64_t& w = words_[n >> 6];
    const uint64_t b = uint64_t(1) << (n & 63);
    const bool was = (w & b) != 0;
    w |= b;
    return was;
  }
  bool setOff(uint32_t n) {
    uint64_t& w = words_[n >> 6];
    const uint64_t b = uint64_t(1) << (n & 63);
    const bool was = (w & b) != 0;
    w &= ~b;
    return was;
  }
  void set(uint32_t n, bool on) { on ? (void)setOn(n) : (void)setOff(n); }
  void setOn() {
    std::fill(words_.begin(), words_.end(), ~uint64_t(0));
    trim();
  }
  void setOff() { std::fill(words_.begin(), words_.end(), uint64_t(0)); }
  void set(bool on) { on ? setOn() : setOff(); }
  void toggle() {
    for (uint64_t& w : words_) w = ~w;
    trim();
  }
  void toggle(uint32_t n) { words_[n >> 6] ^= uint64_t(1) << (n & 63); }

  /// Index of the lowest set bit, or size() if none.
  uint32_t findFirstOn() const { return findNextOn(0); }
  /// Index of the lowest set bit at or above start, or size() if none.
  uint32_t findNextOn(uint32_t start) const {
    if (start >= size_) return size_;
    uint32_t n = start >> 6;
    uint64_t w = words_[n] & (~uint64_t(0) << (start & 63));
    while (!w) {
      if (++n >= words_.size()) return size_;
      w = words_[n];
    }
    return (n << 6) + FindLowestOn(w);
  }

  static uint32_t FindLowestOn(uint64_t v) { return static_cast<uint32_t>(__builtin_ctzll(v)); }
  static uint32_t CountOn(uint64_t v) { return static_cast<uint32_t>(__builtin_popcountll(v)); }

 private:
  // masks of fewer than 64 bits (log2dim 1) keep their unused high bits off
  void trim() {
    if (size_ < 64) words_[0] &= (uint64_t(1) << size_) - 1;
  }
  uint32_t size_;
  std::vector<uint64_t> words_;
};

}  // namespace Bonxai
