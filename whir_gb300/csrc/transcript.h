// Fiat-Shamir transcript on the host: PoseidonWriter over
// DuplexChallenger<KoalaBear, Poseidon2KoalaBear<16>, 16, 8>
// (crates/transcript/src/poseidon.rs:13-87, harness crates/whir/src/test.rs:190-200).
//
// Byte format (crates/transcript/src/field.rs:1-25, bincode 1.3): a field
// element is its 32-bit Montgomery word little-endian; an extension element
// is its 4 coefficients; a digest its 8 words.  write() appends the bytes and
// observes the elements; write_hint() only appends.
#pragma once
#include <stddef.h>
#include <stdint.h>

#include <vector>

#include "kb.cuh"

namespace whir {

class Challenger {
 public:
  Challenger();
  void observe(uint32_t v);
  uint32_t sample();
  size_t sample_bits(int bits);

 private:
  void duplexing();
  uint32_t state_[16];
  uint32_t in_[8];
  int n_in_ = 0;
  uint32_t out_[8];
  int n_out_ = 0;
};

class Transcript {
 public:
  void write_fe(uint32_t v) { put(v); ch_.observe(v); }
  void write_ext(const kb::E4 &e) {
    for (int i = 0; i < 4; i++) write_fe(e.c[i]);
  }
  void write_digest(const uint32_t *d) {
    for (int i = 0; i < 8; i++) write_fe(d[i]);
  }
  void hint_fe(uint32_t v) { put(v); }
  void hint_words(const uint32_t *v, size_t n);
  // Hints are never observed, so their bytes may be written after later
  // transcript operations: reserve n words now, fill them once known.
  size_t hint_reserve(size_t n) {
    size_t off = bytes_.size();
    bytes_.resize(off + 4 * n);
    return off;
  }
  void hint_fill(size_t off, const uint32_t *v, size_t n);
  kb::E4 draw_ext() {
    kb::E4 e;
    for (int i = 0; i < 4; i++) e.c[i] = ch_.sample();
    return e;
  }
  uint32_t draw_fe() { return ch_.sample(); }
  size_t draw_bits(int bits) { return ch_.sample_bits(bits); }
  const std::vector<uint8_t> &bytes() const { return bytes_; }
  // room for a proof of up to n bytes without reallocating
  void reserve(size_t n) { bytes_.reserve(n); }

 private:
  void put(uint32_t v) {
    uint8_t b[4] = {(uint8_t)v, (uint8_t)(v >> 8), (uint8_t)(v >> 16), (uint8_t)(v >> 24)};
    bytes_.insert(bytes_.end(), b, b + 4);
  }
  std::vector<uint8_t> bytes_;
  Challenger ch_;
};

// The verifier's side (crates/transcript/src/poseidon.rs:13-87): the proof
// bytes are read back in order; read_* observes what write_* observed,
// hint_* reads hints without observing.  A read past the end, or a word
// that is not a canonical field element, sets the error flag and yields 0.
class TranscriptReader {
 public:
  TranscriptReader(const uint8_t *bytes, size_t len) : p_(bytes), n_(len) {}
  uint32_t read_fe() {
    uint32_t v = take();
    ch_.observe(v);
    return v;
  }
  kb::E4 read_ext() {
    kb::E4 e;
    for (int i = 0; i < 4; i++) e.c[i] = read_fe();
    return e;
  }
  void read_digest(uint32_t *d) {
    for (int i = 0; i < 8; i++) d[i] = read_fe();
  }
  uint32_t hint_fe() { return take(); }
  // n hint words at once (out == nullptr: read and checked only); the same
  // words, offset and failure as n hint_fe() calls
  void hint_words(uint32_t *out, size_t n) {
    if (n > (n_ - off_) / 4) {
      for (size_t i = 0; i < n; i++) {
        const uint32_t v = take();
        if (out) out[i] = v;
      }
      return;
    }
    const uint8_t *q = p_ + off_;
    uint32_t bad = 0;
    if (out) {
      for (size_t i = 0; i < n; i++) {
        const uint32_t v = word_at(q + 4 * i);
        bad |= (uint32_t)(v >= kb::P);
        out[i] = v;
      }
    } else {
      for (size_t i = 0; i < n; i++) bad |= (uint32_t)(word_at(q + 4 * i) >= kb::P);
    }
    off_ += 4 * n;
    if (bad) err_ = true;
  }
  void hint_digest(uint32_t *d) {
    for (int i = 0; i < 8; i++) d[i] = take();
  }
  kb::E4 draw_ext() {
    kb::E4 e;
    for (int i = 0; i < 4; i++) e.c[i] = ch_.sample();
    return e;
  }
  uint32_t draw_fe() { return ch_.sample(); }
  size_t draw_bits(int bits) { return ch_.sample_bits(bits); }
  bool failed() const { return err_; }
  size_t remaining() const { return n_ - off_; }
  size_t offset() const { return off_; }  // bytes read so far

 private:
  uint32_t take() {
    if (off_ + 4 > n_) {
      err_ = true;
      off_ = n_;
      return 0;
    }
    uint32_t v = word_at(p_ + off_);
    off_ += 4;
    if (v >= kb::P) {
      err_ = true;
      return 0;
    }
    return v;
  }
  static uint32_t word_at(const uint8_t *b) {  // little-endian
    return (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) |
           ((uint32_t)b[3] << 24);
  }
  const uint8_t *p_;
  size_t n_, off_ = 0;
  bool err_ = false;
  Challenger ch_;
};

}  // namespace whir
