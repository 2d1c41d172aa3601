/*
 * Host number theory of libvkhel.  The formulas are the reference's
 * (src/numbers.c, include/priv/numbers.h) so that every table and every
 * constant pushed to a kernel has the value the reference computes:
 *   - Barrett with alpha = 62, beta = -2 (numbers.h:7-9, numbers.c:5-28);
 *   - factor floor(f * 2^64 / q), truncated to 64 bits (numbers.c:30-34);
 *   - inverse by signed extended Euclid on int64 (numbers.c:71-99).
 */
#include "internal.h"

typedef unsigned __int128 u128;

uint64_t vkh_bitlen(uint64_t v) {
	return v == 0 ? 0 : (uint64_t) (64 - __builtin_clzll(v));
}

uint64_t vkh_shoup(uint64_t factor, uint64_t mod) {
	return (uint64_t) ((((u128) factor) << 64) / mod);
}

uint64_t vkh_barrett_mu(uint64_t mod) {
	return vkh_shoup((uint64_t) 1 << (vkh_bitlen(mod) - 2), mod);
}

uint64_t vkh_ref_reduce64(uint64_t x, uint64_t mod, uint64_t mu) {
	const uint64_t n = vkh_bitlen(mod);
	const uint64_t qh = (uint64_t) (((u128) (x >> (n - 2)) * mu) >> 64);
	const uint64_t z = x - qh * mod;
	return z >= mod ? z - mod : z;
}

/* nt_multiply_mod: Barrett reduction of the 128-bit product. */
uint64_t vkh_mulmod(uint64_t a, uint64_t b, uint64_t mod) {
	const uint64_t n = vkh_bitlen(mod);
	const u128 p = (u128) a * b;
	const uint64_t hi = (uint64_t) (p >> 64), lo = (uint64_t) p;
	const uint64_t sh = 66 - n;
	const uint64_t num = (sh >= 64 ? 0 : hi << sh) + (lo >> (n - 2));
	const uint64_t qh = (uint64_t) (((u128) num * vkh_barrett_mu(mod)) >> 64);
	const uint64_t z = lo - qh * mod;
	return z >= mod ? z - mod : z;
}

uint64_t vkh_powmod(uint64_t base, uint64_t exp, uint64_t mod) {
	uint64_t acc = 1;
	base %= mod;
	while (exp) {
		if (exp & 1)
			acc = vkh_mulmod(acc, base, mod);
		base = vkh_mulmod(base, base, mod);
		exp >>= 1;
	}
	return acc;
}

uint64_t vkh_invmod(uint64_t input, uint64_t mod) {
	if (mod == 1)
		return 0;
	int64_t a = (int64_t) input, b = (int64_t) mod, x = 1, y = 0;
	while (a > 1) {
		if (b == 0)
			return 0; /* not invertible; the reference divides by zero */
		const int64_t q = a / b, r = a % b;
		a = b;
		b = r;
		const int64_t t = y;
		y = x - q * y;
		x = t;
	}
	if (x < 0)
		x += (int64_t) mod;
	return (uint64_t) x;
}
