// Small host-side extension-field helpers shared by the prover and the
// verifier (crates/poly/src/lib.rs, crates/poly/src/point.rs,
// crates/whir/src/sumcheck/mod.rs, crates/common/src/utils.rs).
#pragma once
#include <stddef.h>

#include <vector>

#include "kb.cuh"

namespace whir {

inline kb::E4 e_inv2() { return kb::e_from(kb::inv(kb::from_canonical(2))); }
// Lagrange weights of the nodes 0, 1, 2 at r (mod.rs:25-28)
inline void lagrange012(const kb::E4 &r, kb::E4 w[3]) {
  using namespace kb;
  E4 it = e_inv2(), one = e_one(), two = e_dbl(e_one());
  w[0] = e_mul(e_mul(e_sub(r, one), e_sub(r, two)), it);
  w[1] = e_mul(r, e_sub(two, r));
  w[2] = e_mul(e_mul(r, e_sub(r, one)), it);
}
inline kb::E4 extrapolate012(const kb::E4 &e0, const kb::E4 &e1, const kb::E4 &e2,
                             const kb::E4 &r) {
  using namespace kb;
  E4 w[3];
  lagrange012(r, w);
  return e_add(e_add(e_mul(e0, w[0]), e_mul(e1, w[1])), e_mul(e2, w[2]));
}
// eq(z) * scale over k variables, LSB-first doubling (point.rs:110-126)
inline void eq_host(const kb::E4 *z, int k, const kb::E4 &scale, kb::E4 *out) {
  using namespace kb;
  out[0] = scale;
  for (int i = 0; i < k; i++) {
    size_t h = (size_t)1 << i;
    for (size_t j = 0; j < h; j++) {
      E4 hi = e_mul(out[j], z[i]);
      out[j + h] = hi;
      out[j] = e_sub(out[j], hi);
    }
  }
}
// eval_eq_xy: prod (2 x y - x - y + 1) (lib.rs:17-23)
inline kb::E4 eval_eq_xy(const kb::E4 *x, const kb::E4 *y, int n) {
  using namespace kb;
  E4 acc = e_one();
  for (int i = 0; i < n; i++) {
    E4 t = e_sub(e_sub(e_dbl(e_mul(y[i], x[i])), x[i]), y[i]);
    acc = e_mul(acc, e_add(t, e_one()));
  }
  return acc;
}
// eval_pow_xy with base-field x: prod (x y - y + 1) (lib.rs:25-31)
inline kb::E4 eval_pow_xy(const uint32_t *x, const kb::E4 *y, int n) {
  using namespace kb;
  E4 acc = e_one();
  for (int i = 0; i < n; i++) acc = e_mul(acc, e_add(e_sub(e_scale(y[i], x[i]), y[i]), e_one()));
  return acc;
}
// VecOps::horner: rfold acc * x + c (utils.rs:124-127)
inline kb::E4 horner(const kb::E4 *c, size_t n, const kb::E4 &x) {
  using namespace kb;
  E4 acc = e_zero();
  for (size_t i = n; i-- > 0;) acc = e_add(e_mul(acc, x), c[i]);
  return acc;
}
// the same at a base-field point (an extension times base product is four
// base products)
inline kb::E4 horner_base(const kb::E4 *c, size_t n, uint32_t x) {
  using namespace kb;
  E4 acc = e_zero();
  for (size_t i = n; i-- > 0;) acc = e_add(e_scale(acc, x), c[i]);
  return acc;
}
// Point::expand: (v, v^2, v^4, ...) (point.rs:115-124)
inline void expand(kb::E4 *out, int k, kb::E4 v) {
  for (int i = 0; i < k; i++) {
    out[i] = v;
    v = kb::e_sq(v);
  }
}
// <eq, poly> with an eq table already built (eq_host): n entries
inline kb::E4 dot_eq_ext(const kb::E4 *eq, const kb::E4 *poly, size_t n) {
  using namespace kb;
  E4 acc = e_zero();
  for (size_t i = 0; i < n; i++) acc = e_add(acc, e_mul(eq[i], poly[i]));
  return acc;
}
inline kb::E4 dot_eq_base(const kb::E4 *eq, const uint32_t *poly, size_t n) {
  using namespace kb;
  E4 acc = e_zero();
  for (size_t i = 0; i < n; i++) acc = e_add(acc, e_scale(eq[i], poly[i]));
  return acc;
}
// <eq(z), poly> for a short extension poly of 2^k entries
inline kb::E4 eval_ext_small(const kb::E4 *poly, int k, const kb::E4 *z) {
  using namespace kb;
  std::vector<E4> eq((size_t)1 << k);
  eq_host(z, k, e_one(), eq.data());
  E4 acc = e_zero();
  for (size_t i = 0; i < eq.size(); i++) acc = e_add(acc, e_mul(eq[i], poly[i]));
  return acc;
}
// <eq(z), poly> for a short base poly of 2^k entries
inline kb::E4 eval_base_small(const uint32_t *poly, int k, const kb::E4 *z) {
  using namespace kb;
  std::vector<E4> eq((size_t)1 << k);
  eq_host(z, k, e_one(), eq.data());
  E4 acc = e_zero();
  for (size_t i = 0; i < eq.size(); i++) acc = e_add(acc, e_scale(eq[i], poly[i]));
  return acc;
}

}  // namespace whir
