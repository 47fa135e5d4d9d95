/*
 * whir_oracle.h -- CPU restatement of the kilic/whir commit-and-open prover
 * and its verifier, written in plain C.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the correctness oracle for the
 * CUDA prover in whir_gb300/ and the timed CPU baseline.  Only tests/,
 * __graft_entry__.smoke() and bench.py (cpu_baseline leg and the reference
 * arm) load it.  The product never links, loads or calls it.
 *
 * Parity status: UNPINNED against the Rust reference.  The reference cannot
 * be compiled here (no cargo/rustc; Plonky3, rand and bincode are not
 * vendored) and its tests hold no golden vectors.  Every constant that lives
 * in those absent crates (Poseidon2 round numbers and internal diagonals,
 * the ChaCha12/PCG32 seeding of StdRng, the rejection sampler for KoalaBear,
 * Montgomery-form serialization) is restated from the published algorithms
 * and marked at its definition.
 *
 * Field elements are uint32_t in Montgomery form (value * 2^32 mod p), the
 * in-memory representation of Plonky3's MontyField31, so buffers can be
 * shared with the reference's Rust slices and with the CUDA prover as-is.
 * An extension element is 4 consecutive field elements (coefficients of
 * 1, x, x^2, x^3 in F[x]/(x^4 - 3)).  A digest is 8 field elements.
 */
#ifndef WHIR_ORACLE_H
#define WHIR_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Only the wo_* API is exported; internal helpers are hidden so that they
 * cannot be interposed by same-named symbols of other loaded libraries. */
#pragma GCC visibility push(default)

/* ---- field (crates/common/src/field.rs re-exports p3 KoalaBear) ---- */
uint32_t wo_fe_from_u32(uint32_t canonical);
uint32_t wo_fe_to_u32(uint32_t mont);
uint32_t wo_fe_mul(uint32_t a, uint32_t b);
uint32_t wo_fe_add(uint32_t a, uint32_t b);
uint32_t wo_fe_inv(uint32_t a);
void wo_ext_mul(const uint32_t *a, const uint32_t *b, uint32_t *out);
uint32_t wo_two_adic_generator(int bits); /* Montgomery form */

/* ---- randomness: StdRng::seed_from_u64 + StandardUniform<KoalaBear> ---- */
void wo_chacha_block(const uint32_t key[8], uint64_t counter, uint64_t stream,
                     int rounds, uint32_t out[16]);
/* n field elements drawn the way Poly::rand(&mut rng(seed), ..) draws them */
void wo_rand_fe(uint64_t seed, uint32_t *out, size_t n);

/* ---- Poseidon2 (p3-koala-bear Poseidon2KoalaBear<16|24>::new_from_rng_128(rng(1000))) ---- */
int wo_p2_permute(int width, uint32_t *state);
/* export the constants: ext[8*width] (4 initial rounds then 4 terminal), internal[rounds_p], diag[width] */
int wo_p2_constants(int width, uint32_t *ext_rc, uint32_t *int_rc, uint32_t *diag,
                    int *rounds_p);
/* PaddingFreeSponge<P24,24,16,8>::hash_iter over n elements */
void wo_hash_leaf(const uint32_t *in, size_t n, uint32_t out[8]);
/* TruncatedPermutation<P16,2,8,16>::compress */
void wo_compress(const uint32_t left[8], const uint32_t right[8], uint32_t out[8]);

/* ---- DFT (p3 TwoAdicSubgroupDft::dft_batch / dft_algebra_batch) ---- */
/* in: h_in rows x width elems (row-major); zero-padded to 2^log_h_out rows. */
void wo_dft_batch(const uint32_t *in, size_t h_in, size_t width, int log_h_out,
                  uint32_t *out);

/* ---- Merkle (crates/merkle/src/poseidon.rs, poseidon_packed.rs) ---- */
/* rows: 2^log_h rows of row_len field elements; levels: (2^(log_h+1)-1)*8 */
void wo_merkle_tree(const uint32_t *rows, int log_h, size_t row_len, uint32_t *levels);

/* ---- poly kernels (crates/poly/src/{point,eq,poly}.rs) ---- */
void wo_eq_table(const uint32_t *point, int k, const uint32_t *scale, uint32_t *out);
void wo_compress_hi(const uint32_t *poly, int k, const uint32_t *point, int kz,
                    uint32_t *out);
void wo_compress_lo(const uint32_t *poly, int k, const uint32_t *point, int kz,
                    uint32_t *out);
void wo_eval_ext(const uint32_t *poly, int k, const uint32_t *point, uint32_t *out);
void wo_coeffs(const uint32_t *poly, const uint32_t *weights, int k, uint32_t *c0,
               uint32_t *c2);
void wo_fix_lo(uint32_t *poly, int k, const uint32_t *r);
void wo_combine_eqs(uint32_t *weights, int k, const uint32_t *points, int n,
                    const uint32_t *alpha);
void wo_combine_pows(uint32_t *weights, int k, const uint32_t *vars, int n,
                     const uint32_t *alpha, int shift);
void wo_combine_pows_scaled(uint32_t *weights, int k, const uint32_t *vars, int n,
                            const uint32_t *scales);

/* ---- SVO (crates/whir/src/sumcheck/svo.rs): one claim's value and its
 * accumulators with weight 1, per round r < l0 3^r entries at u_r = 0 then
 * 3^r at u_r = 2 (u_0..u_{r-1} the base-3 digits of the entry, lowest first) ---- */
void wo_svo_accumulators(const uint32_t *poly, int k, const uint32_t *point, int l0,
                         uint32_t *out);

/* ---- params (crates/whir/src/params.rs) ---- */
int wo_n_ood_queries(int soundness, int security, int log_degree, int log_inv_rate,
                     int field_bits);
int wo_n_stir_queries(int soundness, int security, int log_inv_rate);
void wo_number_of_rounds(int folding, int k, int *n_rounds, int *final_rounds);

/* ---- full protocol (crates/whir/src/whir.rs, harness test.rs:174-254) ---- */
typedef struct {
  int k;                 /* variables of the stacked layout (single poly: its k) */
  int folding;
  int rate;              /* log_inv_rate */
  int initial_reduction;
  int soundness;         /* 0 UniqueDecoding, 1 JohnsonBound, 2 CapacityBound */
  int security_level;
} wo_params;

/* Claims script shared by prover and verifier: claim group g draws one
 * point expand(k_g, draw()) and evaluates it on ids[off_g .. off_g+n_g). */
typedef struct {
  int n_polys;
  const int *poly_k;        /* [n_polys] */
  int n_groups;
  const int *group_n;       /* [n_groups] */
  const int *group_ids;     /* concatenated ids */
} wo_claims;

/* Prove: polys concatenated in registration order.  Writes the proof bytes
 * (caller buffer of cap bytes), the checkpoint draw (1 field element) and
 * returns 0, or a negative error. *len receives the proof size. */
int wo_prove(const wo_params *prm, const wo_claims *cl, const uint32_t *polys,
             uint8_t *proof, size_t cap, size_t *len, uint32_t *checkpoint);
/* Verify proof bytes; returns 0 when accepted and writes the checkpoint. */
int wo_verify(const wo_params *prm, const wo_claims *cl, const uint8_t *proof,
              size_t len, uint32_t *checkpoint);

/* threads used by the hot loops (OpenMP); 1 when built without OpenMP */
int wo_threads(void);
void wo_set_threads(int n);
/* nonzero: Merkle trees hash WO_LANES leaves / nodes per call through the
 * lane-packed permutation (the timed baseline); 0 (default): the scalar
 * permutation.  Same results either way. */
void wo_set_packed(int on);

#pragma GCC visibility pop

#ifdef __cplusplus
}
#endif
#endif
