/*
 * whir_gb300.h -- C ABI of the GB300 (sm_103a) WHIR commit-and-open prover.
 *
 * This is the drop-in boundary for the reference's prover hot path
 * (kilic/whir, Rust): plain pointers and sizes, no C++ or torch types.  Each
 * group below names the reference interface it replaces.
 *
 * Conventions
 *  - A field element is a uint32_t holding the Montgomery word of a KoalaBear
 *    element (x * 2^32 mod p, p = 2^31 - 2^24 + 1): the in-memory layout of
 *    Plonky3's KoalaBear, so a Rust &[KoalaBear] can be passed as is.  An
 *    extension element is 4 such words (BinomialExtensionField<_, 4>), a
 *    digest 8 ([KoalaBear; 8]).  Every input word must be < p.
 *  - Pointers documented "device" point to memory of the context's GPU
 *    (whir_device_alloc or any cudaMalloc'd memory); all others are host.
 *  - Every function returns WHIR_OK (0) or a negative WHIR_ERR_* code;
 *    whir_last_error() then describes the failure (per calling thread).
 *    No C++ exception crosses this boundary.
 *  - Entry points that take a whir_ctx run on the context's stream and
 *    return after their results are complete.  A context, and every object
 *    made from it, must be used by one host thread at a time.
 */
#ifndef WHIR_GB300_H
#define WHIR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define WHIR_API __attribute__((visibility("default")))
#else
#define WHIR_API
#endif

#define WHIR_OK 0
#define WHIR_ERR_ARG (-1)      /* invalid argument or parameters */
#define WHIR_ERR_CUDA (-2)     /* CUDA runtime error */
#define WHIR_ERR_NOMEM (-3)    /* device or host allocation failed */
#define WHIR_ERR_CAPACITY (-4) /* caller buffer too small, or a job beyond the device budget */
#define WHIR_ERR_INTERNAL (-5)

typedef struct whir_ctx whir_ctx;
typedef struct whir_transcript whir_transcript;
typedef struct whir_prover whir_prover;
typedef struct whir_tree whir_tree;

/* Whir::new arguments (crates/whir/src/whir.rs:104-125).  soundness:
 * 0 UniqueDecoding, 1 JohnsonBound, 2 CapacityBound (params.rs:6-21). */
typedef struct {
  int32_t k;
  int32_t folding;
  int32_t rate; /* log_inv_rate */
  int32_t initial_reduction;
  int32_t soundness;
  int32_t security_level;
} whir_params;

WHIR_API const char *whir_last_error(void);

/* ---- context: one GPU, one stream, constant tables, staging ---- */
WHIR_API int whir_ctx_create(int device, whir_ctx **out);
WHIR_API int whir_ctx_destroy(whir_ctx *ctx);
WHIR_API int whir_ctx_stream(whir_ctx *ctx, void **cuda_stream);
WHIR_API int whir_device_alloc(whir_ctx *ctx, size_t bytes, void **out);
WHIR_API int whir_device_free(whir_ctx *ctx, void *ptr);
WHIR_API int whir_copy_to_device(whir_ctx *ctx, void *dst_device, const void *src, size_t bytes);
WHIR_API int whir_copy_to_host(whir_ctx *ctx, void *dst, const void *src_device, size_t bytes);

/* ---- Reed-Solomon encoding.  Replaces TwoAdicSubgroupDft::dft_batch and
 * dft_algebra_batch as called by commit_base / commit_ext
 * (crates/whir/src/whir.rs:31-34, 56-59).  in: h_in rows of `width` words
 * (device), zero-padded to 2^log_h rows; out: 2^log_h rows (device).  An
 * extension matrix of w columns is the word matrix of 4w columns. ---- */
WHIR_API int whir_dft_batch(whir_ctx *ctx, const uint32_t *in, size_t h_in, size_t width, int log_h,
                   uint32_t *out);

/* ---- Merkle commitment.  Replaces MerkleTree / MerkleTreeExt ::commit and
 * ::query of PackedPoseidonMerkleTree (crates/merkle/src/lib.rs:19-83,
 * crates/merkle/src/poseidon_packed.rs:145-233,259-384): leaves hashed by
 * PaddingFreeSponge<Poseidon2<24>,24,16,8>, nodes by
 * TruncatedPermutation<Poseidon2<16>,2,8,16>, node i of a level paired with
 * node i + n/2.  rows (device) must outlive the tree. ---- */
WHIR_API int whir_merkle_commit(whir_ctx *ctx, const uint32_t *rows, int log_h, size_t row_len,
                       whir_tree **out, uint32_t root[8]);
/* all levels, leaves first: (2^(log_h+1) - 1) digests */
WHIR_API int whir_merkle_levels(whir_tree *tree, uint32_t *out);
/* per index: the leaf row (row_len words) then log_h sibling digests
 * bottom-up, i.e. the hints query() writes */
WHIR_API int whir_merkle_open(whir_tree *tree, const size_t *idx, size_t n, uint32_t *out);
WHIR_API int whir_merkle_free(whir_tree *tree);

/* ---- polynomial and sumcheck passes (crates/poly/src/{point,eq,poly}.rs,
 * crates/whir/src/sumcheck/{svo,expr,combine}.rs) ---- */
/* Point::eq (point.rs:110-126): 2^k extension words at out (device) */
WHIR_API int whir_eq_table(whir_ctx *ctx, const uint32_t *point, int k, const uint32_t scale[4],
                  uint32_t *out);
/* SplitEq::compress_hi (eq.rs:290-398): fix the high kz variables of a base
 * poly (device, 2^k words) to point (kz ext); out: 2^(k-kz) ext (host) */
WHIR_API int whir_compress_hi(whir_ctx *ctx, const uint32_t *poly, int k, const uint32_t *point, int kz,
                     uint32_t *out);
/* SplitEq::compress_lo (eq.rs:400-489): fix the low kz variables; out (device) */
WHIR_API int whir_compress_lo(whir_ctx *ctx, const uint32_t *poly, int k, const uint32_t *point, int kz,
                     uint32_t *out);
/* Poly::eval_ext (poly.rs:89-95) of an extension poly (device) */
WHIR_API int whir_eval_ext(whir_ctx *ctx, const uint32_t *poly, int k, const uint32_t *point,
                  uint32_t out[4]);
/* coeffs (expr.rs:14-27) of extension poly and weights (device, 2^k each) */
WHIR_API int whir_sumcheck_coeffs(whir_ctx *ctx, const uint32_t *poly, const uint32_t *weights, int k,
                         uint32_t c0[4], uint32_t c2[4]);
/* fix_lo_var_mut (poly.rs:131-142) of both arrays into poly_out/w_out
 * (device, 2^(k-1) each; must not alias the inputs) */
WHIR_API int whir_sumcheck_fold(whir_ctx *ctx, const uint32_t *poly, const uint32_t *weights, int k,
                       const uint32_t r[4], uint32_t *poly_out, uint32_t *weights_out);
/* eq::combine_eqs (combine.rs:179-203): w += sum_i alpha^i eq(z_i) */
WHIR_API int whir_combine_eqs(whir_ctx *ctx, uint32_t *weights, int k, const uint32_t *points, int n,
                     const uint32_t alpha[4]);
/* pow::combine_pows (combine.rs:408-438): w[j] += sum_i alpha^(shift+i) var_i^j */
WHIR_API int whir_combine_pows(whir_ctx *ctx, uint32_t *weights, int k, const uint32_t *vars, int n,
                      const uint32_t alpha[4], int shift);
/* pow::combine_pows_scaled (combine.rs:441-468): w[j] += sum_i s_i var_i^j */
WHIR_API int whir_combine_pows_scaled(whir_ctx *ctx, uint32_t *weights, int k, const uint32_t *vars,
                             int n, const uint32_t *scales);

/* The code part of SumcheckProver::fold_with_code (sumcheck/prover.rs:400-561)
 * on its own, as the reference's test_fold_with_code (prover.rs:598-768)
 * exercises it: for queries idx[0..n) of a base codeword (device, 2^k_data
 * rows of 2^folding words) with scales s_i (n ext), the per-query recursion
 * g from the rows' evaluations at eq(rs) (rs: folding ext), folded round by
 * round with r[0..folding-1) (ext); out[8 j .. 8 j + 8) = round j's (c0, c2)
 * of the pow claims, out[8 folding .. + 4) = sum_i s_i g(0, idx_i) (the
 * round-0 sum term). */
WHIR_API int whir_fold_code_rounds(whir_ctx *ctx, const uint32_t *codeword, int k_data,
                                   int folding, const size_t *idx, int n,
                                   const uint32_t *scales, const uint32_t *rs, const uint32_t *r,
                                   uint32_t *out);

/* Debug mode of the single-instance prover, process-wide, off by default.
 * Bit 0: the reference's debug-build invariants, checked on the device's
 * results: after the expression build, every sumcheck round of fold and
 * fold_with_code, <poly, weights> equals the claimed sum
 * (crates/whir/src/sumcheck/prover.rs:346,558, expr.rs:68), every opened
 * Merkle path hashes to its root (crates/merkle/src/poseidon_packed.rs:158-230),
 * and every opened row folded at the round point equals the current
 * polynomial at its domain point (crates/whir/src/whir.rs:263-264, 287-288,
 * 331-352; the polynomial is read back once per round, so keep k small),
 * and each out-of-domain claim combined over a stacked layout equals the
 * claim made on the stacked polynomial (sumcheck/prover.rs:257-266);
 * a failure ends the proof with WHIR_ERR_ARG and a "debug check" message.
 * The checks add a reduction per round; proofs are unchanged.  Bit 1: NVTX
 * ranges around the prover's phases, named like the reference's tracing
 * spans (whir.rs:19-314, sumcheck/prover.rs:184-497).  Bit 2: whir_verify
 * hashes each Merkle opening where it reads it (Whir::verify's order,
 * whir.rs:361-522) instead of after reading the whole proof (the order
 * whir_verify_batch uses); the results are the same either way. */
WHIR_API int whir_debug_set(unsigned flags);

/* Poseidon2KoalaBear<width>::permute_mut on the host (width 16 or 24), with
 * the constants of new_from_rng_128(&mut rng(1000)) used by the harness
 * (crates/whir/src/test.rs:195-196). */
WHIR_API int whir_poseidon2_permute(int width, uint32_t *state);

/* n field elements as Poly::rand(&mut rng(seed), ..) draws them (StdRng
 * seed_from_u64 + StandardUniform<KoalaBear>, crates/poly/src/utils.rs:6-11):
 * the reference harness's seeded polynomial (crates/whir/src/test.rs:213,219). */
WHIR_API int whir_random_field(uint64_t seed, uint32_t *out, size_t n);

/* ---- Fiat-Shamir transcript.  Replaces PoseidonWriter<Vec<u8>, KoalaBear,
 * DuplexChallenger<_, Poseidon2<16>, 16, 8>> (crates/transcript/src/poseidon.rs:13-87)
 * with the challenger permutation of the harness (test.rs:195-200). ---- */
WHIR_API int whir_transcript_new(whir_transcript **out);
WHIR_API int whir_transcript_free(whir_transcript *t);
WHIR_API int whir_transcript_write(whir_transcript *t, const uint32_t e[4]);   /* Writer<Ext>::write */
WHIR_API int whir_transcript_write_base(whir_transcript *t, uint32_t v);       /* Writer<F>::write */
WHIR_API int whir_transcript_draw(whir_transcript *t, uint32_t out[4]);        /* Challenge<F,Ext>::draw */
WHIR_API int whir_transcript_draw_base(whir_transcript *t, uint32_t *out);     /* Challenge<F,F>::draw */
WHIR_API int whir_transcript_draw_bits(whir_transcript *t, int bits, size_t *out); /* ChallengeBits */
WHIR_API int whir_transcript_size(whir_transcript *t, size_t *len);
WHIR_API int whir_transcript_bytes(whir_transcript *t, uint8_t *out, size_t cap);  /* finalize() */

/* ---- protocol.  Replaces Whir::new / Whir::commit / ProverStack /
 * Whir::open (crates/whir/src/whir.rs:104-359, sumcheck/prover.rs:32-125) ---- */
WHIR_API int whir_prover_new(whir_ctx *ctx, const whir_params *params, whir_prover **out);
WHIR_API int whir_prover_free(whir_prover *p);
/* commit the stacked layout of n_polys polys given back to back (sizes
 * 2^poly_k[i]; host, or device when on_device != 0); the stacked size must
 * equal 2^params.k.  Writes the root.  Each later whir_stack_eval refers to
 * a poly by its index here. */
WHIR_API int whir_commit(whir_prover *p, whir_transcript *t, const uint32_t *polys, int on_device,
                const int32_t *poly_k, int n_polys);
/* ProverStack::eval: claim on poly id at point (2^0.. poly_k[id] ext), writes eval */
WHIR_API int whir_stack_eval(whir_prover *p, whir_transcript *t, int id, const uint32_t *point,
                    uint32_t eval[4]);
/* Whir::open over the committed layout and the claims made so far */
WHIR_API int whir_open(whir_prover *p, whir_transcript *t);
/* The reference harness in one call (crates/whir/src/test.rs:218-235 up to
 * the checkpoint draw): commit, then for each claim group g draw one point,
 * expand it to k_g variables and evaluate it on group_ids[off_g ..
 * off_g + group_n[g]), then open. */
WHIR_API int whir_prove(whir_prover *p, whir_transcript *t, const uint32_t *polys, int on_device,
               const int32_t *poly_k, int n_polys, const int32_t *group_n, int n_groups,
               const int32_t *group_ids);

/* Lock-step proving of `batch` polynomials of one shape: the reference
 * harness (crates/whir/src/test.rs:218-235) on each polynomial (commit, then
 * n_claims claims at transcript-drawn points, then Whir::open; or the
 * commitment alone), with every device pass of all instances in one launch
 * and every transcript round trip waited for once.  No counterpart in the
 * reference, whose harness proves one polynomial per call; each instance's
 * proof bytes equal whir_prove's on the same polynomial.  polys[b]: 2^k
 * words each (host, or device when on_device != 0).  Proof b is copied to
 * proofs + b * proof_cap (up to proof_cap bytes; proof_len[b] is its full
 * length) and checkpoints[b] is the base element drawn after it
 * (test.rs:236).  1 <= batch <= whir_batch_max(params). */
WHIR_API int whir_prove_batch(whir_ctx *ctx, const whir_params *params,
                              const uint32_t *const *polys, int on_device, int batch,
                              int n_claims, int commit_only, uint8_t *proofs, size_t proof_cap,
                              size_t *proof_len, uint32_t *checkpoints);
/* the largest batch whir_prove_batch takes for these parameters (the batched
 * codewords must fit the DFT's 32-bit indexing) */
WHIR_API int whir_batch_max(const whir_params *params, int32_t *max_batch);

/* Whir::verify (crates/whir/src/whir.rs:361-522, sumcheck/verifier.rs) on the
 * host: checks a proof of whir_prove with the same parameters, polynomial
 * sizes and claim groups.  The Merkle openings (hints, which no challenge
 * depends on) are hashed after the rest of the proof is read; the result is
 * the first failure in Whir::verify's order all the same.  *result: 0 accepted; 1 the bytes ran out or held a
 * non-canonical word; 2 a Merkle opening failed; 3 a final opening disagrees
 * with the final polynomial; 4 the sumcheck's final claim failed; 5 the round
 * structure does not match.  On acceptance *checkpoint (may be NULL) is the
 * base element the harness draws after the proof.  Needs no GPU. */
WHIR_API int whir_verify(const whir_params *params, const int32_t *poly_k, int n_polys,
                         const int32_t *group_n, int n_groups, const int32_t *group_ids,
                         const uint8_t *proof, size_t len, int32_t *result,
                         uint32_t *checkpoint);
/* Many proofs of one shape (the same parameters, polynomial sizes and claim
 * groups) checked together: results[b] and checkpoints[b] equal whir_verify's
 * on proofs[b] (lens[b] bytes) alone.  Each proof's transcript pass runs on
 * host threads with its Merkle openings deferred (they are hints: no
 * challenge depends on them), then every opening of every proof is hashed
 * in one GPU launch on ctx's stream, and a proof's result is its first
 * failure in whir_verify's order.  No counterpart in the reference, whose
 * Whir::verify (crates/whir/src/whir.rs:361-522) checks one proof per call.
 * n_proofs >= 0; the call returns when all results are written. */
WHIR_API int whir_verify_batch(whir_ctx *ctx, const whir_params *params, const int32_t *poly_k,
                               int n_polys, const int32_t *group_n, int n_groups,
                               const int32_t *group_ids, int n_proofs,
                               const uint8_t *const *proofs, const size_t *lens, int32_t *results,
                               uint32_t *checkpoints);

/* ---- many proofs on one GPU (batched and served proving).  No
 * counterpart in the reference, whose harness proves one polynomial per call
 * (crates/whir/src/test.rs:218-235); each job here is that harness on one
 * polynomial, with n_claims claim groups of that polynomial, or the
 * commitment alone.  n_workers host threads each own a stream and a prover
 * (device buffers are reused from job to job and only grow), so the kernels
 * of concurrent jobs overlap on the GPU.  Jobs start in arrival order; a job
 * starts once it has arrived (whir_serve; whir_batch_prove releases all at
 * once), a worker is free and the device bytes held by all workers
 * (whir_workspace_bytes per job, buffers never shrink) stay within
 * device_budget.  A job's proof bytes are the same whichever worker runs it
 * and whatever runs beside it.  The call returns when every job is done;
 * per-job failures are reported in job->status, argument errors in the
 * return value.  Replicas on several GPUs are separate calls. ---- */
typedef struct whir_job {
  whir_params params;
  const uint32_t *poly;   /* 2^params.k words, Montgomery form */
  int32_t poly_on_device; /* nonzero: poly is device memory of this process */
  int32_t n_claims;       /* evaluation claims at transcript-drawn points */
  int32_t commit_only;    /* nonzero: commit only; the proof is the root */
  double arrival_s;       /* whir_serve: release time after the start of the call */
  uint8_t *proof;         /* out: caller buffer of proof_cap bytes (NULL with cap 0) */
  size_t proof_cap;
  size_t proof_len;       /* out: full proof length (copied up to proof_cap) */
  uint32_t checkpoint;    /* out: base element drawn after the proof (test.rs:236) */
  int32_t status;         /* out: WHIR_OK or an error code */
  int32_t worker;         /* out: the worker that ran it */
  double start_s, done_s; /* out: seconds after the start of the call */
} whir_job;
typedef struct whir_run_stats {
  double seconds;             /* wall time of the whole call */
  uint64_t peak_device_bytes; /* largest total held by the workers */
} whir_run_stats;
/* A persistent worker pool: workers keep their streams, pinned staging and
 * prover buffers between runs (the first run on a worker creates them).  One
 * run at a time per server; honor_arrival as whir_serve. */
typedef struct whir_server whir_server;
WHIR_API int whir_server_new(int device, int n_workers, uint64_t device_budget,
                             whir_server **out);
WHIR_API int whir_server_run(whir_server *s, whir_job *jobs, int n_jobs, int honor_arrival,
                             whir_run_stats *stats);
/* Lock-step groups: a worker that takes a job also takes the jobs of the
 * same shape (parameters, claim count, commit-only, input memory) that have
 * arrived, and proves them together as whir_prove_batch does, every pass of
 * the group in one launch.  max_group bounds a group (1: every job alone;
 * 0: the default, 64); a group also holds at most 2^26 evaluations in all
 * and shrinks to fit the device budget.  Proof bytes do not change. */
WHIR_API int whir_server_set_lockstep(whir_server *s, int max_group);
WHIR_API int whir_server_free(whir_server *s);
/* one-shot forms on a temporary pool */
WHIR_API int whir_batch_prove(int device, whir_job *jobs, int n_jobs, int n_workers,
                              uint64_t device_budget, whir_run_stats *stats);
WHIR_API int whir_serve(int device, whir_job *jobs, int n_jobs, int n_workers,
                        uint64_t device_budget, whir_run_stats *stats);
/* device bytes one worker holds while proving with these parameters */
WHIR_API int whir_workspace_bytes(const whir_params *params, uint64_t *bytes);
/* an upper bound of the proof length with n_claims claims (sizes job->proof) */
WHIR_API int whir_proof_bytes_max(const whir_params *params, int n_claims, uint64_t *bytes);
/* The admission order of whir_serve with a stand-in for the GPU: job j
 * occupies a worker for duration_s[j] seconds (a host sleep) and holds
 * need[j] bytes.  A negative duration injects a failure: the job fails
 * (status WHIR_ERR_INTERNAL) after |duration_s[j]| seconds with its worker's
 * buffers grown for it, as a proof that hits a transcript or I/O error
 * would; the worker goes on with later jobs.  Host only, for testing the
 * scheduling. */
WHIR_API int whir_serve_simulate(const double *arrival_s, const uint64_t *need,
                                 const double *duration_s, int n_jobs, int n_workers,
                                 uint64_t device_budget, double *start_s, double *done_s,
                                 int32_t *worker, int32_t *status);
/* The same with lock-step groups (whir_server_set_lockstep): jobs of equal
 * shape[j] that have arrived are taken together, up to max_group; a group
 * holds its size times its first job's need and takes its first job's
 * duration.  Host only. */
WHIR_API int whir_serve_simulate_groups(const double *arrival_s, const uint64_t *need,
                                        const double *duration_s, const int32_t *shape,
                                        int max_group, int n_jobs, int n_workers,
                                        uint64_t device_budget, double *start_s, double *done_s,
                                        int32_t *worker, int32_t *status);

/* ---- allocation-free SVO compression.  No counterpart in the reference:
 * an extra entry point for callers that must not allocate device memory (a
 * host whose GPU memory is all owned by its own pool, or code that cannot
 * afford the device-wide synchronisation cudaMalloc/cudaFree may cause
 * mid-proof).  Same result as whir_compress_hi, but it allocates nothing:
 * its scratch is one fixed 40 KiB device array inside the library, held by
 * every GPU that loads it until exit.  Limits: kz <= 20 fixed variables and
 * k - kz <= 8 kept ones; larger sizes return WHIR_ERR_ARG.  Runs on
 * cuda_stream (NULL: the default stream) of the current device and returns
 * once out (host, 2^(k-kz) extension elements) is written.  The first call
 * on a device looks up the array's device address; make it before any
 * stream capture, and do not call it after a cudaDeviceReset in the same
 * process (the address is kept; a reset may move the array).  All calls share
 * the array, so calls must be serialised: issued to one stream from one host
 * thread, or under the caller's own lock.  Calls that overlap on the GPU
 * (other streams), or that two host threads queue on one stream at the same
 * time, race. ---- */
WHIR_API int whir_compress_hi_noalloc(void *cuda_stream, const uint32_t *poly, int k,
                                      const uint32_t *point, int kz, uint32_t *out);

/* ---- launch-split autotuning (no counterpart in the reference).  How a
 * Merkle tree of height log_h and a two-pass DFT of 2^log_h rows are split
 * into launches is chosen per size; every choice gives the same result.
 * whir_autotune times the candidates for log_h in [lo, hi] on the context's
 * stream (a few hundred ms, up to ~1.5 GB of temporary device memory),
 * installs the fastest process-wide and writes a text report (one line per
 * size) into report.  whir_tune_tree / whir_tune_dft set one choice (tree:
 * levels making >= 2^wide_log nodes run one thread per node, the rest as
 * 2^((S + split) / 2) subtrees, split in -1..1; DFT: first pass of 2^L1
 * rows, L1 = (log_h + 1) / 2 + l1_bias); whir_tune_reset restores the
 * defaults. ---- */
WHIR_API int whir_autotune(whir_ctx *ctx, int log_h_lo, int log_h_hi, char *report, size_t cap);
WHIR_API int whir_tune_tree(int log_h, int wide_log, int split);
WHIR_API int whir_tune_dft(int log_h, size_t width, int l1_bias);
WHIR_API int whir_tune_reset(void);

/* ---- per-kernel-class timing with CUDA events on the context stream:
 * klass 0 DFT, 1 leaf hash, 2 tree, 3 sumcheck passes; klass 4 is host time
 * blocked waiting for the stream (ms and number of waits).  read returns and
 * clears total ms, launches and algorithmic bytes since enabling. ---- */
WHIR_API int whir_prof_enable(whir_ctx *ctx, int on);
/* time only the classes whose bit (1 << klass) is set: fewer events on the
 * stream while the rest runs untimed */
WHIR_API int whir_prof_enable_classes(whir_ctx *ctx, unsigned mask);
WHIR_API int whir_prof_read(whir_ctx *ctx, int klass, double *ms, long *launches, double *bytes);
/* kernels launched by this library in this process, and the bytes the
 * prover of this context copied host->device / device->host, since start */
WHIR_API int whir_counters(whir_ctx *ctx, uint64_t *kernel_launches, uint64_t *h2d_bytes,
                           uint64_t *d2h_bytes);

#ifdef __cplusplus
}
#endif
#endif
