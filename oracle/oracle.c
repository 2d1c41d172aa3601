/*
 * CPU oracle for the vkhel hot path -- TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * Restates, in plain C, the arithmetic of the reference (lolzballs/vkhel):
 *   - Barrett constants alpha = 62, beta = -2      include/priv/numbers.h:7-9
 *   - Barrett multiply-mod                         src/numbers.c:5-28
 *   - Shoup/Barrett factor floor(f * 2^64 / q)     src/numbers.c:30-34
 *   - power, primitive-root test, inverse          src/numbers.c:36-99
 *   - bit-reversed twiddle tables                  src/ntt_tables.c:8-44
 *   - shader arithmetic                            src/kernels/shaders/ *.comp
 *   - forward / inverse stage loops                src/vector.c:536-566, 599-649
 * The GLSL helper mul64 (e.g. elemmul.comp:24-34) forms an exact 64x64->128
 * product from 32-bit halves; here that is a plain unsigned __int128 product.
 */
#include "oracle.h"

#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef unsigned __int128 u128;

static const int64_t kAlpha = 62; /* include/priv/numbers.h:8 */
static const int64_t kBeta = -2;  /* include/priv/numbers.h:9 */

static inline uint64_t hi64(uint64_t a, uint64_t b) {
	return (uint64_t) (((u128) a * b) >> 64);
}

/* A left shift by 64 or more yields 0.  The only place a shader shifts that far
 * is reduce128 with a 2-bit modulus (elemmul.comp:50), where the shifted high
 * word is 0 because both factors are already reduced below 4. */
static inline uint64_t shl_sat(uint64_t x, uint64_t s) {
	return s >= 64 ? 0 : x << s;
}

/* nt_ceil_log2 (include/priv/numbers.h:11-13): the bit length of v. */
uint64_t orc_bitlen(uint64_t v) {
	return v == 0 ? 0 : (uint64_t) (64 - __builtin_clzll(v));
}

/* nt_compute_barrett_factor (src/numbers.c:30-34): floor(factor * 2^64 / mod),
 * truncated to 64 bits.  With factor = a twiddle this is the Shoup factor. */
uint64_t orc_shoup_factor(uint64_t factor, uint64_t mod) {
	return (uint64_t) ((((u128) factor) << 64) / mod);
}

/* The Barrett constant mu = floor(2^(n + alpha) / mod) that every caller passes
 * (e.g. src/kernels/elemmul.c:159-162).  Needs n + alpha >= 64, i.e. mod >= 2. */
uint64_t orc_barrett_mu(uint64_t mod) {
	const uint64_t n = orc_bitlen(mod);
	return orc_shoup_factor((uint64_t) 1 << (n + kAlpha - 64), mod);
}

/* compute_mod (src/numbers.c:5-28) applied to a 128-bit value hi:lo. */
static uint64_t barrett128(uint64_t hi, uint64_t lo, uint64_t mod, uint64_t mu) {
	const uint64_t n = orc_bitlen(mod);
	const uint64_t num_c = shl_sat(hi, 64 - (n + kBeta)) + (lo >> (n + kBeta));
	const uint64_t q_hat = hi64(num_c, mu);
	uint64_t z = lo - q_hat * mod;
	if (z >= mod)
		z -= mod;
	return z;
}

/* reduce64 (elemmul.comp:36-47, elemgtsub.comp:36-47). */
static uint64_t barrett64(uint64_t x, uint64_t mod, uint64_t mu) {
	const uint64_t n = orc_bitlen(mod);
	const uint64_t q_hat = hi64(x >> (n + kBeta), mu);
	uint64_t z = x - q_hat * mod;
	if (z >= mod)
		z -= mod;
	return z;
}

/* nt_multiply_mod (src/numbers.c:36-40). */
uint64_t orc_mulmod(uint64_t a, uint64_t b, uint64_t mod) {
	const u128 p = (u128) a * b;
	return barrett128((uint64_t) (p >> 64), (uint64_t) p, mod, orc_barrett_mu(mod));
}

/* nt_power_mod (src/numbers.c:42-59): right-to-left square and multiply. */
uint64_t orc_powmod(uint64_t base, uint64_t exp, uint64_t mod) {
	uint64_t acc = 1;
	base %= mod;
	for (; exp > 0; exp >>= 1) {
		if (exp & 1)
			acc = orc_mulmod(acc, base, mod);
		base = orc_mulmod(base, base, mod);
	}
	return acc;
}

/* nt_is_primitive_root (src/numbers.c:61-69): root^(degree/2) == -1. */
bool orc_is_primitive_root(uint64_t root, uint64_t degree, uint64_t mod) {
	if (root == 0)
		return false;
	return orc_powmod(root, degree / 2, mod) == mod - 1;
}

/* nt_inverse_mod (src/numbers.c:71-99): signed extended Euclid on int64.
 * A zero divisor (input not coprime to mod) returns 0 here; the reference
 * divides by zero in that case. */
uint64_t orc_invmod(uint64_t input, uint64_t mod) {
	if (mod == 1)
		return 0;
	int64_t a = (int64_t) input, b = (int64_t) mod, x = 1, y = 0;
	while (a > 1) {
		if (b == 0)
			return 0;
		const int64_t quot = a / b, rem = a % b;
		a = b;
		b = rem;
		const int64_t prev_y = y;
		y = x - quot * y;
		x = prev_y;
	}
	if (x < 0)
		x += (int64_t) mod;
	return (uint64_t) x;
}

/* reverse_bits (src/ntt_tables.c:8-15). */
static uint64_t bit_reverse(uint64_t v, uint64_t width) {
	uint64_t r = 0;
	for (uint64_t k = 0; k < width; k++) {
		r = (r << 1) | (v & 1);
		v >>= 1;
	}
	return r;
}

/* compute_roots_of_unity_powers (src/ntt_tables.c:17-44): roots[bitrev(i)] =
 * w^i by repeated multiplication, inverses by extended Euclid, and the Shoup
 * factor of every entry. */
void orc_ntt_tables(uint64_t n, uint64_t q, uint64_t w,
		uint64_t *roots, uint64_t *inv_roots,
		uint64_t *roots_shoup, uint64_t *inv_roots_shoup) {
	const uint64_t width = orc_bitlen(n) - 1;
	roots[0] = 1;
	inv_roots[0] = orc_invmod(1, q);
	uint64_t power = 1;
	for (uint64_t i = 1; i < n; i++) {
		const uint64_t slot = bit_reverse(i, width);
		power = orc_mulmod(power, w, q);
		roots[slot] = power;
		inv_roots[slot] = orc_invmod(power, q);
	}
	for (uint64_t i = 0; i < n; i++) {
		roots_shoup[i] = orc_shoup_factor(roots[i], q);
		inv_roots_shoup[i] = orc_shoup_factor(inv_roots[i], q);
	}
}

/* ------------------------------------------------------------------ */
/* element-wise shaders                                                */
/* ------------------------------------------------------------------ */

/* elemmul.comp:62-73 with constants from src/kernels/elemmul.c:159-168. */
void orc_elemmul(const uint64_t *a, const uint64_t *b, uint64_t *res,
		size_t len, uint64_t mod) {
	const uint64_t mu = orc_barrett_mu(mod);
	for (size_t i = 0; i < len; i++) {
		const uint64_t x = barrett64(a[i], mod, mu);
		const uint64_t y = barrett64(b[i], mod, mu);
		const u128 p = (u128) x * y;
		res[i] = barrett128((uint64_t) (p >> 64), (uint64_t) p, mod, mu);
	}
}

/* Shoup product x*b mod q with one conditional subtraction
 * (elemmulconst.comp:42-46, nttfwdbutterfly.comp:44-48). */
static inline uint64_t shoup_mul(uint64_t x, uint64_t b, uint64_t b_shoup,
		uint64_t mod) {
	uint64_t r = x * b - hi64(x, b_shoup) * mod;
	if (r >= mod)
		r -= mod;
	return r;
}

/* elemmulconst.comp:35-49 with constants from elemmulconst.c:154-163. */
void orc_elemmulconst(const uint64_t *a, uint64_t *res, size_t len,
		uint64_t b, uint64_t mod) {
	const uint64_t bs = orc_shoup_factor(b, mod);
	for (size_t i = 0; i < len; i++)
		res[i] = shoup_mul(a[i], b, bs, mod);
}

/* elemfma.comp:36-55 as written, with constants from elemfma.c:159-169.  The
 * two "reductions" compute mod - x instead of x - mod (elemfma.comp:47-48 and
 * 51-52), so results differ from (a*m + b) mod q whenever the Shoup estimate
 * is one short or the sum reaches q. */
void orc_elemfma(const uint64_t *a, const uint64_t *b, uint64_t *res,
		size_t len, uint64_t multiplier, uint64_t mod) {
	const uint64_t ms = orc_shoup_factor(multiplier, mod);
	for (size_t i = 0; i < len; i++) {
		uint64_t p = a[i] * multiplier - hi64(a[i], ms) * mod;
		if (p >= mod)
			p = mod - p;
		const uint64_t s = p + b[i];
		res[i] = s >= mod ? mod - s : s;
	}
}

/* (a*m + b) mod q: what elemfma is meant to compute (the golden vectors of
 * test/vector.c:39-83 agree with both formulas). */
void orc_elemfma_canonical(const uint64_t *a, const uint64_t *b,
		uint64_t *res, size_t len, uint64_t multiplier, uint64_t mod) {
	for (size_t i = 0; i < len; i++)
		res[i] = (uint64_t) (((u128) a[i] * multiplier + b[i]) % mod);
}

/* elemgtsub.comp:49-67 with constants from elemgtsub.c:154-168. */
void orc_elemgtsub(const uint64_t *a, uint64_t *res, size_t len,
		uint64_t bound, uint64_t diff, uint64_t mod) {
	const uint64_t mu = orc_barrett_mu(mod);
	const uint64_t d = barrett64(diff, mod, mu);
	for (size_t i = 0; i < len; i++) {
		const uint64_t r = barrett64(a[i], mod, mu);
		if (a[i] > bound) {
			const uint64_t z = r + mod - d;
			res[i] = z >= mod ? z - mod : z;
		} else {
			res[i] = r;
		}
	}
}

/* elemgtadd.comp:20-30 (plain wrapping add). */
void orc_elemgtadd(const uint64_t *a, uint64_t *res, size_t len,
		uint64_t bound, uint64_t diff) {
	for (size_t i = 0; i < len; i++)
		res[i] = a[i] > bound ? a[i] + diff : a[i];
}

/* elemmodbytwo.comp:19-27. */
void orc_elemmodbytwo(const uint64_t *a, uint64_t *res, size_t len,
		uint64_t signed_bound) {
	for (size_t i = 0; i < len; i++) {
		const uint64_t bit = a[i] & 1;
		res[i] = a[i] > signed_bound ? 1 - bit : bit;
	}
}

/* vkhel_vector_elemmod dispatch (src/vector.c:360-368). */
void orc_elemmod(const uint64_t *a, uint64_t *res, size_t len,
		uint64_t mod, uint64_t q) {
	if (mod == 2)
		orc_elemmodbytwo(a, res, len, q / 2);
	else
		orc_elemgtsub(a, res, len, q / 2, q, mod);
}

/* ------------------------------------------------------------------ */
/* transforms                                                          */
/* ------------------------------------------------------------------ */

/* `x = X; while (x < y) x += q; x -= y;` (nttfwdbutterfly.comp:50-54,
 * nttrevbutterfly.comp:44-48) in closed form.  Returns -1 if the loop would
 * wrap past 2^64 before reaching y. */
static inline int sub_loop(uint64_t x, uint64_t y, uint64_t q, uint64_t *out) {
	if (x >= y) {
		*out = x - y;
		return 0;
	}
	const uint64_t k = (y - x + q - 1) / q;
	const u128 top = (u128) x + (u128) k * q;
	if (top >> 64)
		return -1;
	*out = (uint64_t) top - y;
	return 0;
}

/* vkhel_vector_forward_transform: the stage loop of src/vector.c:536-566 with
 * the Cooley-Tukey butterfly of nttfwdbutterfly.comp:41-57. */
int orc_ntt_forward(uint64_t *d, uint64_t n, uint64_t q,
		const uint64_t *roots, const uint64_t *roots_shoup) {
	int status = 0;
	uint64_t t = n / 2;
	for (uint64_t m = 1; m < n; m *= 2, t /= 2) {
		for (uint64_t blk = 0; blk < m; blk++) {
			const uint64_t w = roots[m + blk], ws = roots_shoup[m + blk];
			uint64_t *x = d + 2 * t * blk, *y = x + t;
			for (uint64_t j = 0; j < t; j++) {
				const uint64_t wy = shoup_mul(y[j], w, ws, q);
				uint64_t diff = 0;
				if (sub_loop(x[j], wy, q, &diff))
					status = -1;
				const uint64_t sum = x[j] + wy;
				x[j] = sum % q;
				y[j] = diff % q;
			}
		}
	}
	return status;
}

/* vkhel_vector_inverse_transform: the stage loop of src/vector.c:599-630 with
 * the Gentleman-Sande butterfly of nttrevbutterfly.comp:41-57, then the
 * elemmulconst pass by n^-1 (src/vector.c:632-638). */
int orc_ntt_inverse(uint64_t *d, uint64_t n, uint64_t q,
		const uint64_t *inv_roots, const uint64_t *inv_roots_shoup) {
	int status = 0;
	uint64_t t = 1;
	for (uint64_t m = n / 2; m >= 1; m /= 2, t *= 2) {
		for (uint64_t blk = 0; blk < m; blk++) {
			const uint64_t w = inv_roots[m + blk], ws = inv_roots_shoup[m + blk];
			uint64_t *x = d + 2 * t * blk, *y = x + t;
			for (uint64_t j = 0; j < t; j++) {
				uint64_t diff = 0;
				if (sub_loop(x[j], y[j], q, &diff))
					status = -1;
				const uint64_t sum = x[j] + y[j];
				x[j] = sum % q;
				y[j] = shoup_mul(diff, w, ws, q);
			}
		}
	}
	orc_elemmulconst(d, d, n, orc_invmod(n, q), q);
	return status;
}

int orc_polymul(const uint64_t *a, const uint64_t *b, uint64_t *c,
		uint64_t n, uint64_t q, uint64_t w) {
	uint64_t *tab = malloc(sizeof(uint64_t) * 4 * n);
	uint64_t *tb = malloc(sizeof(uint64_t) * n);
	orc_ntt_tables(n, q, w, tab, tab + n, tab + 2 * n, tab + 3 * n);
	memcpy(c, a, sizeof(uint64_t) * n);
	memcpy(tb, b, sizeof(uint64_t) * n);
	int st = orc_ntt_forward(c, n, q, tab, tab + 2 * n);
	st |= orc_ntt_forward(tb, n, q, tab, tab + 2 * n);
	orc_elemmul(c, tb, c, n, q);
	st |= orc_ntt_inverse(c, n, q, tab + n, tab + 3 * n);
	free(tb);
	free(tab);
	return st;
}

void orc_negacyclic_schoolbook(const uint64_t *a, const uint64_t *b,
		uint64_t *c, uint64_t n, uint64_t q) {
	for (uint64_t k = 0; k < n; k++)
		c[k] = 0;
	for (uint64_t i = 0; i < n; i++) {
		for (uint64_t j = 0; j < n; j++) {
			const uint64_t p = (uint64_t) (((u128) (a[i] % q) * (b[j] % q)) % q);
			const uint64_t k = i + j;
			if (k < n)
				c[k] = (uint64_t) (((u128) c[k] + p) % q);
			else
				c[k - n] = (uint64_t) (((u128) c[k - n] + q - p) % q);
		}
	}
}

int orc_polymul_batch_tables(const uint64_t *a, const uint64_t *b, uint64_t *c,
		size_t count, size_t stride, uint64_t n,
		const uint64_t *qs, const uint64_t *tabs, const uint32_t *prime_idx,
		int threads) {
	int used = 1;
#ifdef _OPENMP
	if (threads <= 0)
		threads = omp_get_max_threads();
	used = threads;
#pragma omp parallel num_threads(threads)
#endif
	{
		uint64_t *tb = malloc(sizeof(uint64_t) * n);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
		for (size_t j = 0; j < count; j++) {
			const uint64_t *t = tabs + 4 * n * prime_idx[j];
			const uint64_t q = qs[prime_idx[j]];
			uint64_t *cj = c + j * stride;
			memcpy(cj, a + j * stride, sizeof(uint64_t) * n);
			memcpy(tb, b + j * stride, sizeof(uint64_t) * n);
			orc_ntt_forward(cj, n, q, t, t + 2 * n);
			orc_ntt_forward(tb, n, q, t, t + 2 * n);
			orc_elemmul(cj, tb, cj, n, q);
			orc_ntt_inverse(cj, n, q, t + n, t + 3 * n);
		}
		free(tb);
	}
	return used;
}

int orc_polymul_batch(const uint64_t *a, const uint64_t *b, uint64_t *c,
		size_t count, size_t stride, uint64_t n,
		const uint64_t *qs, const uint64_t *ws, const uint32_t *prime_idx,
		size_t n_primes, int threads) {
	/* One table set per prime, built once like a caller of the reference
	 * builds one vkhel_ntt_tables per (n, q, w). */
	uint64_t *tabs = malloc(sizeof(uint64_t) * 4 * n * n_primes);
	for (size_t p = 0; p < n_primes; p++) {
		uint64_t *t = tabs + 4 * n * p;
		orc_ntt_tables(n, qs[p], ws[p], t, t + n, t + 2 * n, t + 3 * n);
	}
	const int used = orc_polymul_batch_tables(a, b, c, count, stride, n, qs, tabs, prime_idx, threads);
	free(tabs);
	return used;
}
