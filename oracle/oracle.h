/*
 * CPU oracle for the vkhel hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * This is a plain-C restatement of the reference's algorithms (lolzballs/vkhel):
 * its host number theory (src/numbers.c), its twiddle-table builder
 * (src/ntt_tables.c), the arithmetic of its eight compute shaders
 * (src/kernels/shaders/ *.comp) and the host stage loops that drive them
 * (src/vector.c).  Each function cites the reference lines it follows.
 *
 * Only the test suite, the smoke check and the CPU-baseline leg of the
 * benchmark may call into this code, and only to compare against.  The product
 * library (libvkhel.so) never links or loads it.
 *
 * Parity pin: the oracle is checked against every golden vector of the
 * reference's own tests (test/vector.c, test/numbers.c, test/ntt.c) by running
 * those test programs against it (oracle/Makefile, targets ref-tests), and its
 * tables are compared with the reference's own ntt_tables.c built from source.
 */
#ifndef VKHEL_ORACLE_H
#define VKHEL_ORACLE_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- number theory (src/numbers.c, include/priv/numbers.h) ---- */
uint64_t orc_bitlen(uint64_t v);
uint64_t orc_shoup_factor(uint64_t factor, uint64_t mod);
uint64_t orc_barrett_mu(uint64_t mod);
uint64_t orc_mulmod(uint64_t a, uint64_t b, uint64_t mod);
uint64_t orc_powmod(uint64_t base, uint64_t exp, uint64_t mod);
bool orc_is_primitive_root(uint64_t root, uint64_t degree, uint64_t mod);
uint64_t orc_invmod(uint64_t a, uint64_t mod);

/* ---- twiddle tables (src/ntt_tables.c) ---- */
void orc_ntt_tables(uint64_t n, uint64_t q, uint64_t w,
		uint64_t *roots, uint64_t *inv_roots,
		uint64_t *roots_shoup, uint64_t *inv_roots_shoup);

/* ---- element-wise shader math (src/kernels/shaders) ---- */
void orc_elemmul(const uint64_t *a, const uint64_t *b, uint64_t *res,
		size_t len, uint64_t mod);
void orc_elemmulconst(const uint64_t *a, uint64_t *res, size_t len,
		uint64_t b, uint64_t mod);
void orc_elemfma(const uint64_t *a, const uint64_t *b, uint64_t *res,
		size_t len, uint64_t multiplier, uint64_t mod);
void orc_elemfma_canonical(const uint64_t *a, const uint64_t *b,
		uint64_t *res, size_t len, uint64_t multiplier, uint64_t mod);
void orc_elemgtsub(const uint64_t *a, uint64_t *res, size_t len,
		uint64_t bound, uint64_t diff, uint64_t mod);
void orc_elemgtadd(const uint64_t *a, uint64_t *res, size_t len,
		uint64_t bound, uint64_t diff);
void orc_elemmodbytwo(const uint64_t *a, uint64_t *res, size_t len,
		uint64_t signed_bound);
void orc_elemmod(const uint64_t *a, uint64_t *res, size_t len,
		uint64_t mod, uint64_t q);

/* ---- transforms (src/vector.c stage loops + butterfly shaders) ----
 * Tables are the four arrays built by orc_ntt_tables.  `data` is transformed
 * in place (the reference reads `operand` in the first stage and `result`
 * afterwards, which is the same function of the input).  Returns 0, or -1
 * when the reference's `while (x < y) x += q` loop would wrap around 2^64
 * (the reference does not terminate usefully there). */
int orc_ntt_forward(uint64_t *data, uint64_t n, uint64_t q,
		const uint64_t *roots, const uint64_t *roots_shoup);
int orc_ntt_inverse(uint64_t *data, uint64_t n, uint64_t q,
		const uint64_t *inv_roots, const uint64_t *inv_roots_shoup);

/* Negacyclic product by the reference's own composition:
 * forward(a), forward(b), elemmul, inverse.  a and b are not modified. */
int orc_polymul(const uint64_t *a, const uint64_t *b, uint64_t *c,
		uint64_t n, uint64_t q, uint64_t w);

/* Schoolbook negacyclic product mod (X^n + 1, q), for cross-checking. */
void orc_negacyclic_schoolbook(const uint64_t *a, const uint64_t *b,
		uint64_t *c, uint64_t n, uint64_t q);

/* Batched polymul for the CPU baseline: `count` independent limb-polymuls,
 * job j uses prime index prime_idx[j] into (ns, qs, ws) and operands at
 * a + j*stride etc.  Runs on `threads` OpenMP threads (0 = all).
 * Returns the number of threads used. */
int orc_polymul_batch(const uint64_t *a, const uint64_t *b, uint64_t *c,
		size_t count, size_t stride, uint64_t n,
		const uint64_t *qs, const uint64_t *ws, const uint32_t *prime_idx,
		size_t n_primes, int threads);

/* The same with the primes' tables built beforehand (a caller of the
 * reference builds one vkhel_ntt_tables per (n, q, w) and reuses it):
 * tabs = n_primes consecutive sets of the four orc_ntt_tables arrays
 * (roots, inv_roots, roots_shoup, inv_roots_shoup; 4 n words per prime). */
int orc_polymul_batch_tables(const uint64_t *a, const uint64_t *b, uint64_t *c,
		size_t count, size_t stride, uint64_t n,
		const uint64_t *qs, const uint64_t *tabs, const uint32_t *prime_idx,
		int threads);

#ifdef __cplusplus
}
#endif

#endif
