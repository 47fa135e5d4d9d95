// Batched verification (see verify_batch.h).
//
// Staging layout (pinned host, copied to the device in one go): the proofs,
// each from a 16-byte boundary, then one PathDesc per path, then the paths'
// roots (8 words each); the device writes one flag per path after them.
// Paths are ordered by (row_len, log_h) so that the threads of a warp do the
// same number of permutations.
#include "verify_batch.h"

#include <string.h>

#include <algorithm>

namespace whir {

BatchVerifier::BatchVerifier(Context *ctx, int host_threads) : ctx_(ctx), pool_(host_threads) {}

namespace {
size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }
struct PathRef {
  int proof;
  int check;
};
}  // namespace

void BatchVerifier::verify(const Params &p, const std::vector<int> &poly_k,
                           const std::vector<std::vector<int>> &groups, int n,
                           const uint8_t *const *proofs, const size_t *lens, int32_t *results,
                           uint32_t *checkpoints) {
  if (n < 0 || (n > 0 && (!proofs || !lens || !results || !checkpoints)))
    throw WhirError(-1, "bad proof list");
  last_paths_ = 0;
  if (n == 0) return;
  for (int b = 0; b < n; b++)
    if (!proofs[b] && lens[b]) throw WhirError(-1, "null proof");
  // 1. every proof's transcript pass, paths deferred
  std::vector<DeferredPaths> dp(n);
  std::vector<VerifyResult> res(n);
  std::vector<uint32_t> cp(n, 0);
  pool_.run(n, [&](int b) {
    res[b] = whir::verify(p, poly_k, groups, proofs[b], lens[b], &cp[b], &dp[b]);
  }, pool_.threads());

  // 2. staging: proofs, descriptors, roots
  std::vector<size_t> base(n);  // first word of proof b in the staging area
  size_t proof_bytes = 0, n_paths = 0;
  for (int b = 0; b < n; b++) {
    base[b] = proof_bytes / 4;
    if (!dp[b].checks.empty()) proof_bytes += align16(lens[b]);
    n_paths += dp[b].checks.size();
  }
  std::vector<PathRef> order;
  order.reserve(n_paths);
  for (int b = 0; b < n; b++)
    for (int j = 0; j < (int)dp[b].checks.size(); j++) order.push_back({b, j});
  std::stable_sort(order.begin(), order.end(), [&](const PathRef &x, const PathRef &y) {
    const PathCheck &a = dp[x.proof].checks[x.check], &c = dp[y.proof].checks[y.check];
    return a.row_len != c.row_len ? a.row_len < c.row_len : a.log_h < c.log_h;
  });
  const size_t desc_off = proof_bytes, root_off = align16(desc_off + sizeof(gpu::PathDesc) * n_paths),
               ok_off = align16(root_off + 32 * n_paths), total = align16(ok_off + n_paths);
  std::vector<uint8_t> ok(n_paths, 0);
  if (n_paths) {
    if (n_paths > (size_t)0x7fffffff) throw WhirError(-1, "too many paths in one batch");
    stage_.reserve(total);
    dev_.reserve(total);
    uint8_t *st = stage_.data();
    pool_.run(n, [&](int b) {
      if (!dp[b].checks.empty()) memcpy(st + 4 * base[b], proofs[b], lens[b]);
    }, pool_.threads());
    gpu::PathDesc *desc = reinterpret_cast<gpu::PathDesc *>(st + desc_off);
    uint32_t *roots = reinterpret_cast<uint32_t *>(st + root_off);
    for (size_t i = 0; i < n_paths; i++) {
      const PathCheck &c = dp[order[i].proof].checks[order[i].check];
      // the opening was read from the proof, so its words lie inside it
      if (4 * (c.word + (size_t)c.row_len + 8 * (size_t)c.log_h) > lens[order[i].proof])
        throw WhirError(-1, "path outside its proof");
      desc[i].off = base[order[i].proof] + c.word;
      desc[i].index = c.index;
      desc[i].log_h = c.log_h;
      desc[i].row_len = c.row_len;
      memcpy(roots + 8 * i, c.root, 32);
    }
    // 3. one copy in, one launch, the flags back
    uint8_t *d = dev_.as<uint8_t>();
    cuda_check(copy_async(*ctx_, d, st, ok_off, cudaMemcpyHostToDevice), "h2d");
    cuda_check(gpu::verify_paths(reinterpret_cast<const gpu::PathDesc *>(d + desc_off),
                                 reinterpret_cast<const uint32_t *>(d),
                                 reinterpret_cast<const uint32_t *>(d + root_off), (int)n_paths,
                                 d + ok_off, ctx_->stream()),
               "verify_paths");
    cuda_check(copy_async(*ctx_, st + ok_off, d + ok_off, n_paths, cudaMemcpyDeviceToHost), "d2h");
    ctx_->sync();
    for (size_t i = 0; i < n_paths; i++) ok[i] = st[ok_off + i];
  }
  last_paths_ = n_paths;

  // 4. each proof's first failure in verify()'s order
  std::vector<std::vector<uint8_t>> per(n);
  for (int b = 0; b < n; b++) per[b].assign(dp[b].checks.size(), 0);
  for (size_t i = 0; i < n_paths; i++) per[order[i].proof][order[i].check] = ok[i];
  for (int b = 0; b < n; b++) {
    VerifyResult r = verify_resolve(res[b], dp[b], per[b].data());
    results[b] = (int32_t)r;
    checkpoints[b] = r == V_OK ? cp[b] : 0;
  }
}

}  // namespace whir
