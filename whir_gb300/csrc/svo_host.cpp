// Host side of the SVO claims and rounds (see svo_host.h).
#include "svo_host.h"

#include "host_math.h"

namespace whir {

using kb::E4;
using namespace kb;

size_t ipow3(int r) {
  size_t v = 1;
  while (r--) v *= 3;
  return v;
}
E4 reduce_acc(const unsigned long long *a) {
  E4 r;
  for (int c = 0; c < 4; c++) r.c[c] = (uint32_t)(a[c] % P);
  return r;
}
size_t svo_acc_size(int ks) {
  size_t s = 0;
  for (int r = 0; r < ks; r++) s += 2 * ipow3(r);
  return s;
}

void svo_finish(SvoClaim &c, int ks, const unsigned long long *sums) {
  const E4 *point = c.point.data();
  size_t n = (size_t)1 << ks;
  c.compressed.resize(n);
  for (size_t j = 0; j < n; j++) c.compressed[j] = reduce_acc(sums + 4 * j);
  std::vector<E4> eq(n);
  eq_host(point, ks, e_one(), eq.data());
  c.eval = e_zero();
  for (size_t j = 0; j < n; j++) c.eval = e_add(c.eval, e_mul(eq[j], c.compressed[j]));
  c.partial.assign(partial_off(ks + 1), e_zero());
  for (int l = 1; l <= ks; l++) {  // svo_partial_evals (svo.rs:18-38)
    size_t na2 = (size_t)1 << l, nr = (size_t)1 << (ks - l);
    std::vector<E4> er(nr);
    eq_host(point + l, ks - l, e_one(), er.data());
    E4 *out = c.partial.data() + partial_off(l);
    for (size_t x = 0; x < na2; x++) {
      E4 s = e_zero();
      for (size_t r = 0; r < nr; r++) s = e_add(s, e_mul(c.compressed[x + na2 * r], er[r]));
      out[x] = s;
    }
  }
}

// Svo::calculate_accumulators for one claim weighted by `w` (svo.rs:225-278);
// accumulators are linear in the weighted partial evals, so summing per
// claim equals the reference's per-point grouping.  For each round r and
// grid point u in {0,1,2}^r x {0 or 2}: acc += eq(u, svo[..r+1]) * <w pe_r, eq_u>.
// The eq tables eq_u have base-field entries and do not depend on the claim
// (Svo::new, svo.rs:158-222), so they are built once per prover.  Table r
// depends on r alone: a prover reused with a larger folding only adds the
// missing rounds.
void SvoTables::build(int ks) {
  const int have = (int)eq_.size();
  if (have >= ks) return;
  eq_.resize(ks);
  const uint32_t vals[3][2] = {{ONE, 0}, {0, ONE}, {neg(ONE), dbl(ONE)}};  // (1-u, u)
  for (int r = have; r < ks; r++) {
    int l = r + 1;
    size_t n = ipow3(r), na = (size_t)1 << l;
    std::vector<uint32_t> &tab = eq_[r];
    tab.assign(2 * n * na, 0);
    for (int which = 0; which < 2; which++)
      for (size_t t = 0; t < n; t++) {
        int dig[16];
        size_t tt = t;
        for (int i = 0; i < r; i++) {
          dig[i] = (int)(tt % 3);
          tt /= 3;
        }
        dig[r] = which ? 2 : 0;
        uint32_t *e = tab.data() + (which * n + t) * na;
        for (size_t a = 0; a < na; a++) {
          uint32_t v = ONE;
          for (int i = 0; i < l; i++) v = mul(v, vals[dig[i]][(a >> i) & 1]);
          e[a] = v;
        }
      }
  }
}
void SvoTables::accumulate(std::vector<E4> &accv, const SvoClaim &c, const E4 &w, int ks) {
  build(ks);
  size_t off = 0;
  std::vector<E4> wpe, fac, nxt;
  for (int r = 0; r < ks; r++) {
    int l = r + 1;
    size_t n = ipow3(r), na = (size_t)1 << l;
    const E4 *pe = c.partial.data() + partial_off(l);
    wpe.resize(na);
    for (size_t a = 0; a < na; a++) wpe[a] = e_mul(w, pe[a]);
    // eval_eq_xy(u, y) = prod_i f(u_i, y_i) with f(0,y) = 1-y, f(1,y) = y,
    // f(2,y) = 3y-1; the 3^r prefix products in base-3 digit order
    fac.assign(1, e_one());
    for (int i = 0; i < r; i++) {
      const E4 &y = c.point[i];
      E4 f3[3] = {e_sub(e_one(), y), y, e_sub(e_add(e_dbl(y), y), e_one())};
      nxt.resize(fac.size() * 3);
      for (int d = 0; d < 3; d++)
        for (size_t t = 0; t < fac.size(); t++) nxt[d * fac.size() + t] = e_mul(fac[t], f3[d]);
      fac.swap(nxt);
    }
    const E4 &yl = c.point[r];
    E4 last[2] = {e_sub(e_one(), yl), e_sub(e_add(e_dbl(yl), yl), e_one())};
    const uint32_t *tab = eq_[r].data();
    for (int which = 0; which < 2; which++)
      for (size_t t = 0; t < n; t++) {
        const uint32_t *eq = tab + (which * n + t) * na;
        uint64_t s4[4] = {0, 0, 0, 0};
        for (size_t a = 0; a < na; a++)
          for (int q = 0; q < 4; q++) s4[q] += (uint64_t)mul(wpe[a].c[q], eq[a]);
        E4 dot;
        for (int q = 0; q < 4; q++) dot.c[q] = (uint32_t)(s4[q] % kb::P);
        E4 v = e_mul(e_mul(fac[t], last[which]), dot);
        accv[off + which * n + t] = e_add(accv[off + which * n + t], v);
      }
    off += 2 * n;
  }
}


void svo_rounds(Transcript &ts, const std::vector<E4> &accv, int ks, E4 &sum,
                std::vector<E4> &rs) {
  size_t off = 0;
  for (int r = 0; r < ks; r++) {
    size_t nw = ipow3(r);
    std::vector<E4> wts(1, e_one());
    for (int i = 0; i < r; i++) {  // lagrange_weights_012_multi (svo.rs:7-16)
      E4 l3[3];
      lagrange012(rs[i], l3);
      std::vector<E4> nx(wts.size() * 3);
      for (int d = 0; d < 3; d++)
        for (size_t t = 0; t < wts.size(); t++) nx[d * wts.size() + t] = e_mul(wts[t], l3[d]);
      wts.swap(nx);
    }
    E4 c0 = e_zero(), c2 = e_zero();
    for (size_t t = 0; t < nw; t++) {
      c0 = e_add(c0, e_mul(accv[off + t], wts[t]));
      c2 = e_add(c2, e_mul(accv[off + nw + t], wts[t]));
    }
    off += 2 * nw;
    ts.write_ext(c0);
    ts.write_ext(c2);
    E4 r_ = ts.draw_ext();
    sum = extrapolate012(c0, e_sub(sum, c0), c2, r_);
    rs.push_back(r_);
  }
}

}  // namespace whir
