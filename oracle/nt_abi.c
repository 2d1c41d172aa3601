/*
 * The reference's host number-theory entry points (include/priv/numbers.h:16-22)
 * defined over the CPU oracle -- TEST INFRASTRUCTURE ONLY.  Linking the
 * reference's own test/numbers.c against this file runs its known-answer
 * tests (test/numbers.c:20-94) on the oracle's arithmetic.
 */
#include <stdbool.h>
#include <stdint.h>

#include "oracle.h"

uint64_t nt_compute_barrett_factor(uint64_t factor, uint64_t mod, uint64_t n) {
	(void) n;
	return orc_shoup_factor(factor, mod);
}

uint64_t nt_multiply_mod(const uint64_t a, const uint64_t b,
		const uint64_t mod, const uint64_t barrett_factor) {
	(void) barrett_factor; /* src/numbers.c:36-40 ignores it as well */
	return orc_mulmod(a, b, mod);
}

uint64_t nt_power_mod(uint64_t base, uint64_t exp, const uint64_t mod) {
	return orc_powmod(base, exp, mod);
}

bool nt_is_primitive_root(const uint64_t root, const uint64_t degree,
		const uint64_t mod) {
	return orc_is_primitive_root(root, degree, mod);
}

uint64_t nt_inverse_mod(const uint64_t a, const uint64_t mod) {
	return orc_invmod(a, mod);
}
