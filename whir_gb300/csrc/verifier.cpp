// WHIR verifier on the host (see verifier.h).
#include "verifier.h"

#include <string.h>

#include <algorithm>

#include "host_math.h"
#include "poseidon2_host.h"
#include "transcript.h"

namespace whir {
namespace {

using kb::E4;

// PaddingFreeSponge<Poseidon2<24>, 24, 16, 8> over one row
// (crates/merkle/src/poseidon.rs:33-59): overwrite the rate lanes, permute.
void hash_leaf(const uint32_t *row, size_t n, uint32_t out[8]) {
  const Poseidon2Constants &c = poseidon2_constants(24);
  uint32_t s[24] = {0};
  size_t pos = 0;
  while (pos < n) {
    size_t take = std::min<size_t>(16, n - pos);
    for (size_t j = 0; j < take; j++) s[j] = row[pos + j];
    pos += take;
    poseidon2_permute_host(c, s);
  }
  memcpy(out, s, 32);
}
// TruncatedPermutation<Poseidon2<16>, 2, 8, 16> (poseidon.rs:61-74)
void compress(const uint32_t a[8], const uint32_t b[8], uint32_t out[8]) {
  uint32_t s[16];
  memcpy(s, a, 32);
  memcpy(s + 8, b, 32);
  poseidon2_permute_host(poseidon2_constants(16), s);
  memcpy(out, s, 32);
}

// MerkleTree::verify (crates/merkle/src/poseidon_packed.rs:235-257, path
// check :22-41): the leaf words, then the siblings bottom to top (halves
// pairing: the sibling of index i at a level of 2m nodes is i ^ m).
// With defer, the path is recorded (as read) instead of hashed.
bool open_path(TranscriptReader &ts, const uint32_t root[8], size_t index, size_t row_len,
               int log_h, std::vector<uint32_t> &row, DeferredPaths *defer) {
  const size_t word = ts.offset() / 4;
  row.resize(row_len);
  ts.hint_words(row.data(), row_len);
  if (defer) {
    if (log_h < 0 || log_h > 40 || index >= ((size_t)1 << log_h)) return false;
    ts.hint_words(nullptr, 8 * (size_t)log_h);  // read (and range-checked) only
    if (ts.failed()) return false;  // ran out mid-path: the transcript failure comes first
    PathCheck c;
    c.word = word;
    c.index = (uint64_t)index;
    c.log_h = log_h;
    c.row_len = (int)row_len;
    memcpy(c.root, root, 32);
    defer->checks.push_back(c);
    return true;
  }
  uint32_t acc[8];
  hash_leaf(row.data(), row_len, acc);
  if (log_h < 0 || log_h > 40 || index >= ((size_t)1 << log_h)) return false;
  size_t idx = index;
  for (int l = 0; l < log_h; l++) {
    uint32_t w[8], nxt[8];
    ts.hint_digest(w);
    size_t mid = (size_t)1 << (log_h - l - 1);
    if (idx >= mid) compress(w, acc, nxt);
    else compress(acc, w, nxt);
    memcpy(acc, nxt, 32);
    idx &= mid - 1;
  }
  return !ts.failed() && memcmp(acc, root, 32) == 0;
}

}  // namespace

bool merkle_path_ok(const uint32_t root[8], size_t index, const uint32_t *row, size_t row_len,
                    const uint32_t *siblings, int log_h) {
  if (log_h < 0 || log_h > 40 || index >= ((size_t)1 << log_h)) return false;
  uint32_t acc[8];
  hash_leaf(row, row_len, acc);
  size_t idx = index;
  for (int l = 0; l < log_h; l++) {
    uint32_t nxt[8];
    const size_t mid = (size_t)1 << (log_h - l - 1);
    if (idx >= mid) compress(siblings + 8 * l, acc, nxt);
    else compress(acc, siblings + 8 * l, nxt);
    memcpy(acc, nxt, 32);
    idx &= mid - 1;
  }
  return memcmp(acc, root, 32) == 0;
}

namespace {

// whir.rs:64-77: n sample_bits draws, sorted and deduplicated
std::vector<size_t> stir_indexes(TranscriptReader &ts, int bits, int n) {
  std::vector<size_t> v(n);
  for (int i = 0; i < n; i++) v[i] = ts.draw_bits(bits);
  std::sort(v.begin(), v.end());
  v.erase(std::unique(v.begin(), v.end()), v.end());
  return v;
}

// The claims of one folding round as SumcheckVerifier keeps them
// (verifier.rs:199-306): eq points over kfull variables, pow variables, the
// challenges drawn since, and the combination randomness.
struct FoldingRound {
  int kfull = 0;
  std::vector<E4> eq_pts;  // n_eq * kfull
  std::vector<uint32_t> pow_vars;
  std::vector<E4> rs;
  E4 alpha = kb::e_zero();
};

// the round's claims evaluated against the final polynomial (verifier.rs:308-323)
E4 final_value(const FoldingRound &f, const std::vector<E4> &fp, int kp) {
  using namespace kb;
  size_t n_eq = f.eq_pts.size() / (f.kfull ? f.kfull : 1);
  int nr = (int)f.rs.size();
  std::vector<E4> w;
  for (size_t i = 0; i < n_eq; i++) {
    const E4 *z = f.eq_pts.data() + i * f.kfull;
    w.push_back(e_mul(eval_eq_xy(z, f.rs.data(), nr), eval_ext_small(fp.data(), kp, z + nr)));
  }
  std::vector<uint32_t> pt(f.kfull);
  for (uint32_t v : f.pow_vars) {
    for (int j = 0; j < f.kfull; j++) {
      pt[j] = v;
      v = mul(v, v);
    }
    E4 e = horner_base(fp.data(), fp.size(), pt[nr]);  // eval_univariate
    w.push_back(e_mul(eval_pow_xy(pt.data(), f.rs.data(), nr), e));
  }
  return horner(w.data(), w.size(), f.alpha);
}

// one sumcheck round: read (c0, c2), draw r, extrapolate the claimed sum
E4 reduce_round(TranscriptReader &ts, E4 *sum) {
  E4 v0 = ts.read_ext(), v2 = ts.read_ext();
  E4 r = ts.draw_ext();
  *sum = extrapolate012(v0, kb::e_sub(*sum, v0), v2, r);
  return r;
}

}  // namespace

VerifyResult verify(const Params &p, const std::vector<int> &poly_k,
                    const std::vector<std::vector<int>> &groups, const uint8_t *proof, size_t len,
                    uint32_t *checkpoint, DeferredPaths *defer) {
  using namespace kb;
  if (!proof && len) throw WhirError(-1, "null proof");
  Prover::workspace_bytes(p);  // validates the parameters
  const int f = p.folding, k = p.k;
  std::vector<LayEntry> lay = stack_layout(poly_k, k, f);
  const int n_polys = (int)poly_k.size();
  for (auto &g : groups) {
    if (g.empty()) throw WhirError(-1, "empty claim group");
    for (int id : g)
      if (id < 0 || id >= n_polys || poly_k[id] != poly_k[g[0]])
        throw WhirError(-1, "bad claim group");
  }
  TranscriptReader ts(proof, len);
  const size_t row_base = (size_t)1 << f, row_ext = row_base * 4;
  uint32_t comm[8];
  ts.read_digest(comm);
  // claims (harness test.rs:218-235): one drawn point per group
  struct Claim {
    int poly;
    std::vector<E4> point;
    E4 eval;
  };
  std::vector<Claim> claims;
  for (auto &g : groups) {
    int kg = poly_k[g[0]];
    E4 z = ts.draw_ext();
    for (int id : g) {
      Claim c;
      c.poly = id;
      c.point.resize(kg);
      expand(c.point.data(), kg, z);
      c.eval = ts.read_ext();
      claims.push_back(std::move(c));
    }
  }
  // the claims in layout order, lifted by their selector bits, then the
  // virtual (out-of-domain) claims over all k variables (verifier.rs:199-246)
  std::vector<FoldingRound> fr(1);
  FoldingRound &f0 = fr[0];
  f0.kfull = k;
  std::vector<E4> evals;
  for (auto &e : lay)
    for (auto &c : claims)
      if (c.poly == e.poly) {
        int kp = poly_k[e.poly];
        for (int i = 0; i < kp; i++) f0.eq_pts.push_back(c.point[i]);
        for (int b = 0; b < e.nbits; b++) f0.eq_pts.push_back(e.bits[b] ? e_one() : e_zero());
        evals.push_back(c.eval);
      }
  int n_ood = n_ood_queries(p.soundness, p.security_level, k, p.rate, EXT_BITS);
  for (int i = 0; i < n_ood; i++) {
    std::vector<E4> z(k);
    expand(z.data(), k, ts.draw_ext());
    f0.eq_pts.insert(f0.eq_pts.end(), z.begin(), z.end());
    evals.push_back(ts.read_ext());
  }
  f0.alpha = ts.draw_ext();
  E4 sum = horner(evals.data(), evals.size(), f0.alpha);
  for (int i = 0; i < f; i++) f0.rs.push_back(reduce_round(ts, &sum));
  int kcur = k - f;
  std::vector<E4> round_point(f0.rs.begin(), f0.rs.end());
  int n_rounds, final_rounds;
  number_of_rounds(f, k, &n_rounds, &final_rounds);
  uint32_t round_comm[8];
  bool have_round_comm = false;
  std::vector<uint32_t> row;
  std::vector<E4> eqr((size_t)1 << f);
  for (int round = 0; round < n_rounds; round++) {
    int kfd, this_rate, prev_rate;
    round_params(p, round, &kfd, &this_rate, &prev_rate);
    uint32_t rcomm[8];
    ts.read_digest(rcomm);
    FoldingRound fn;
    fn.kfull = kcur;
    std::vector<E4> oev;
    int n_o = n_ood_queries(p.soundness, p.security_level, kcur, this_rate, EXT_BITS);
    for (int i = 0; i < n_o; i++) {
      E4 z = ts.draw_ext();
      oev.push_back(ts.read_ext());
      std::vector<E4> pt(kcur);
      expand(pt.data(), kcur, z);
      fn.eq_pts.insert(fn.eq_pts.end(), pt.begin(), pt.end());
    }
    int n_s = n_stir_queries(p.soundness, p.security_level, prev_rate);
    std::vector<size_t> idx = stir_indexes(ts, kfd, n_s);
    uint32_t omega = two_adic_generator(kfd);
    // eq(round point), shared by every opening of the round
    eq_host(round_point.data(), f, e_one(), eqr.data());
    for (size_t q : idx) {
      E4 e;
      if (round == 0) {
        if (!open_path(ts, comm, q, row_base, kfd, row, defer)) return ts.failed() ? V_TRANSCRIPT : V_MERKLE;
        e = dot_eq_base(eqr.data(), row.data(), eqr.size());
      } else {
        if (!open_path(ts, round_comm, q, row_ext, kfd, row, defer))
          return ts.failed() ? V_TRANSCRIPT : V_MERKLE;
        e = dot_eq_ext(eqr.data(), reinterpret_cast<const E4 *>(row.data()), eqr.size());
      }
      fn.pow_vars.push_back(kb::pow(omega, q));
      oev.push_back(e);
    }
    memcpy(round_comm, rcomm, 32);
    have_round_comm = true;
    // SumcheckVerifier::fold (verifier.rs:262-306)
    fn.alpha = ts.draw_ext();
    sum = e_add(sum, horner(oev.data(), oev.size(), fn.alpha));
    std::vector<E4> rsn;
    for (int i = 0; i < f; i++) rsn.push_back(reduce_round(ts, &sum));
    for (auto &g : fr) g.rs.insert(g.rs.end(), rsn.begin(), rsn.end());
    fn.rs = rsn;
    fr.push_back(std::move(fn));
    kcur -= f;
    round_point = rsn;
  }
  if (kcur != final_rounds) return V_SHAPE;
  std::vector<E4> fp((size_t)1 << kcur);
  for (auto &e : fp) e = ts.read_ext();
  {
    int kfd, this_rate, prev_rate;
    round_params(p, n_rounds, &kfd, &this_rate, &prev_rate);
    int n_s = n_stir_queries(p.soundness, p.security_level, prev_rate);
    std::vector<size_t> idx = stir_indexes(ts, kfd, n_s);
    uint32_t omega = two_adic_generator(kfd);
    eq_host(round_point.data(), f, e_one(), eqr.data());
    for (size_t q : idx) {
      E4 e;
      if (have_round_comm) {
        if (!open_path(ts, round_comm, q, row_ext, kfd, row, defer))
          return ts.failed() ? V_TRANSCRIPT : V_MERKLE;
        e = dot_eq_ext(eqr.data(), reinterpret_cast<const E4 *>(row.data()), eqr.size());
      } else {
        if (!open_path(ts, comm, q, row_base, kfd, row, defer)) return ts.failed() ? V_TRANSCRIPT : V_MERKLE;
        e = dot_eq_base(eqr.data(), row.data(), eqr.size());
      }
      E4 want = horner_base(fp.data(), fp.size(), kb::pow(omega, q));
      if (!e_eq(e, want)) return V_STIR;
    }
  }
  // SumcheckVerifier::finalize (verifier.rs:308-323)
  E4 tot = e_zero();
  for (auto &g : fr) tot = e_add(tot, final_value(g, fp, kcur));
  if (!e_eq(tot, sum)) return V_SUMCHECK;
  uint32_t cp = ts.draw_fe();
  if (ts.failed()) return V_TRANSCRIPT;
  if (checkpoint) *checkpoint = cp;
  return V_OK;
}

std::vector<uint8_t> deferred_paths_ok(const uint8_t *proof, size_t len, const DeferredPaths &d) {
  std::vector<uint8_t> ok(d.checks.size());
  std::vector<uint32_t> w;
  for (size_t i = 0; i < d.checks.size(); i++) {
    const PathCheck &c = d.checks[i];
    const size_t n = (size_t)c.row_len + 8 * (size_t)c.log_h;
    if (4 * (c.word + n) > len) throw WhirError(-1, "path outside the proof");
    w.resize(n);
    memcpy(w.data(), proof + 4 * c.word, 4 * n);  // little-endian words, as bincode writes them
    ok[i] = merkle_path_ok(c.root, c.index, w.data(), c.row_len, w.data() + c.row_len, c.log_h);
  }
  return ok;
}

VerifyResult verify_resolve(VerifyResult deferred, const DeferredPaths &d, const uint8_t *path_ok) {
  for (size_t i = 0; i < d.checks.size(); i++)
    if (!path_ok[i]) return V_MERKLE;
  return deferred;
}

}  // namespace whir
