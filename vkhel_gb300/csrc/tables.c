/*
 * NTT twiddle tables: host construction (values identical to the reference's
 * src/ntt_tables.c:17-44) and the per-context device cache.
 *
 * Host side.  roots[bitrev(i)] = w^i by repeated Barrett multiplication
 * (ntt_tables.c:25-34).  The reference inverts every root with extended
 * Euclid; when w^n = -1 (a primitive 2n-th root, the case every caller uses)
 * the same canonical values follow by index, w^-i = -w^(n-i), at no cost, and
 * Euclid is kept for any other w.  Shoup factors floor(r 2^64 / q) as in
 * ntt_tables.c:36-43.  The host arrays are built on first use only.
 *
 * Device side.  One pool allocation per (n, q, w) holds a vkcu_twset header
 * and the forward and inverse tables as interleaved (root, shoup) pairs so a
 * butterfly fetches its twiddle with one 16-byte load.  When q < 2^61 and
 * w^n = -1 the device generates the tables itself (vkcu_twiddles): the host
 * computes only 2 sqrt(n) powers and uploads 16 sqrt(n) bytes instead of
 * 32 n; the values equal the host arrays (Barrett products are exact below
 * 2^61, so every power is canonical whatever the order of the products).
 * Otherwise the host arrays are uploaded.  Contexts cache these by value, so
 * separately created table objects with equal parameters share one copy.
 */
#include <inttypes.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "internal.h"

typedef unsigned __int128 u128;

static uint64_t bit_reverse(uint64_t v, uint32_t width) {
	uint64_t r = 0;
	for (uint32_t k = 0; k < width; k++) {
		r = (r << 1) | (v & 1);
		v >>= 1;
	}
	return r;
}

/* The reference's table builder (src/ntt_tables.c:17-44): roots[bitrev(i)] =
 * w^i by repeated Barrett products, inverses by index when w^n = -1 and by
 * extended Euclid otherwise, Shoup factors of every entry. */
static void compute_host_arrays(struct vkhel_ntt_tables *t) {
	const uint64_t n = t->n, q = t->q, w = t->w;
	t->roots[0] = 1;
	uint64_t power = 1;
	int canonical = 1;
	for (uint64_t i = 1; i < n; i++) {
		power = vkh_mulmod(power, w, q);
		t->roots[bit_reverse(i, t->log_n)] = power;
		canonical &= power < q && power != 0;
	}
	/* The index rule needs true powers of w: canonical Barrett products are
	 * (their estimate never overflows below 2^62); at 63 bits the reference's
	 * product can wrap, so there every entry is inverted as it does. */
	const int negacyclic = canonical && t->qbits <= 62 && n > 1 && vkh_mulmod(power, w, q) == q - 1;
	t->inv_roots[0] = vkh_invmod(1, q);
	for (uint64_t i = 1; i < n; i++) {
		const uint64_t slot = bit_reverse(i, t->log_n);
		if (negacyclic)
			t->inv_roots[slot] = q - t->roots[bit_reverse(n - i, t->log_n)];
		else
			t->inv_roots[slot] = vkh_invmod(t->roots[slot], q);
	}
	for (uint64_t i = 0; i < n; i++) {
		t->roots_shoup[i] = vkh_shoup(t->roots[i], q);
		t->inv_roots_shoup[i] = vkh_shoup(t->inv_roots[i], q);
		t->unreduced |= t->roots[i] >= q || t->inv_roots[i] >= q;
	}
}

static pthread_mutex_t g_host_mu = PTHREAD_MUTEX_INITIALIZER;

/* Host arrays on demand (table copy-out, debug print, host upload path). */
static int ensure_host(struct vkhel_ntt_tables *t) {
	pthread_mutex_lock(&g_host_mu);
	int st = VKHEL_OK;
	if (!t->host_ready) {
		uint64_t *mem = malloc(sizeof(uint64_t) * 4 * t->n);
		if (!mem) {
			st = vkh_fail(NULL, VKHEL_ERR_OUT_OF_MEMORY, "ntt tables: host allocation failed");
		} else {
			t->roots = mem;
			t->inv_roots = mem + t->n;
			t->roots_shoup = mem + 2 * t->n;
			t->inv_roots_shoup = mem + 3 * t->n;
			compute_host_arrays(t);
			t->host_ready = 1;
		}
	}
	pthread_mutex_unlock(&g_host_mu);
	return st;
}

struct vkhel_ntt_tables *vkhel_ntt_tables_create(uint64_t n, uint64_t q, uint64_t w) {
	if (n == 0 || (n & (n - 1)) != 0) {
		vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT,
				"ntt tables: n=%" PRIu64 " is not a power of two", n);
		return NULL;
	}
	if (q < 2 || n >= ((uint64_t) 1 << 31)) {
		vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT,
				"ntt tables: unsupported n=%" PRIu64 " q=%" PRIu64, n, q);
		return NULL;
	}
	struct vkhel_ntt_tables *t = calloc(1, sizeof(*t));
	if (!t) {
		vkh_fail(NULL, VKHEL_ERR_OUT_OF_MEMORY, "ntt tables: host allocation failed");
		return NULL;
	}
	t->n = n;
	t->q = q;
	t->w = w;
	t->log_n = (uint32_t) vkh_bitlen(n) - 1;
	t->qbits = (uint32_t) vkh_bitlen(q);
	t->mu = t->qbits >= 2 ? vkh_barrett_mu(q) : 0;
	t->ninv = vkh_invmod(n, q); /* src/vector.c:633 */
	t->ninv_s = vkh_shoup(t->ninv, q);
	/* Barrett products are exact below 2^61, so every power is canonical and
	 * the device can form them in any order; w^n = -1 makes the inverses
	 * follow by index. */
	t->w_red = t->qbits >= 2 ? vkh_mulmod(1, w, q) : 0;
	t->device_gen = n >= 2 && t->qbits >= 3 && t->qbits <= 61 && w < q && w != 0 &&
			vkh_powmod(t->w_red, n, q) == q - 1;
	uint64_t w1 = 1; /* inv_roots[1] = (w^(n/2))^-1 */
	if (t->device_gen) {
		w1 = q - vkh_powmod(t->w_red, n / 2, q);
	} else {
		if (ensure_host(t) != VKHEL_OK) {
			free(t);
			return NULL;
		}
		if (n > 1)
			w1 = t->inv_roots[1];
	}
	t->w1ninv = (uint64_t) (((u128) w1 * t->ninv) % q);
	t->w1ninv_s = vkh_shoup(t->w1ninv, q);
	return t;
}

void vkhel_ntt_tables_destroy(struct vkhel_ntt_tables *t) {
	if (!t)
		return;
	free(t->roots);
	free(t);
}

int vkhel_ntt_tables_copy(const struct vkhel_ntt_tables *ct, uint64_t *roots,
		uint64_t *inv_roots, uint64_t *roots_shoup, uint64_t *inv_roots_shoup) {
	if (!ct)
		return vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "ntt tables: NULL");
	struct vkhel_ntt_tables *t = (struct vkhel_ntt_tables *) ct;
	const int st = ensure_host(t);
	if (st)
		return st;
	const size_t bytes = sizeof(uint64_t) * t->n;
	if (roots)
		memcpy(roots, t->roots, bytes);
	if (inv_roots)
		memcpy(inv_roots, t->inv_roots, bytes);
	if (roots_shoup)
		memcpy(roots_shoup, t->roots_shoup, bytes);
	if (inv_roots_shoup)
		memcpy(inv_roots_shoup, t->inv_roots_shoup, bytes);
	return VKHEL_OK;
}

void vkhel_ntt_tables_dbgprint(struct vkhel_ntt_tables *t) {
	if (!t || ensure_host(t) != VKHEL_OK)
		return;
	printf("ntt_tables: (n=%" PRIu64 " q=%" PRIu64 " w=%" PRIu64 ")\n", t->n, t->q, t->w);
	printf("\troots_of_unity: ");
	for (uint64_t i = 0; i < t->n; i++)
		printf(i + 1 == t->n ? "%" PRIu64 : "%" PRIu64 ", ", t->roots[i]);
	printf("\n\tinv_roots_of_unity: ");
	for (uint64_t i = 0; i < t->n; i++)
		printf(i + 1 == t->n ? "%" PRIu64 : "%" PRIu64 ", ", t->inv_roots[i]);
	printf("\n");
}

int vkh_devtab_get(struct vkhel_ctx *ctx, const struct vkhel_ntt_tables *t,
		const struct vkh_devtab **out) {
	for (struct vkh_devtab *d = ctx->tabs; d; d = d->next) {
		if (d->n == t->n && d->q == t->q && d->w == t->w) {
			*out = d;
			return VKHEL_OK;
		}
	}
	const uint64_t n = t->n;
	const uint64_t head = 256; /* vkcu_twset, padded to keep the tables aligned */
	const uint32_t lb = (t->log_n + 1) / 2; /* power table split: w^i = w^(hi 2^lb) w^lo */
	const uint64_t nlo = (uint64_t) 1 << lb, nhi = n >> lb;
	const uint64_t table_bytes = head + 2 * 16 * n;
	const uint64_t bytes = table_bytes + (t->device_gen ? 8 * (nlo + nhi) : 0);
	const uint64_t staged = t->device_gen ? head + 8 * (nlo + nhi) : bytes;
	if (!t->device_gen && ensure_host((struct vkhel_ntt_tables *) t) != VKHEL_OK)
		return vkh_fail(ctx, VKHEL_ERR_OUT_OF_MEMORY, "tables: host arrays");
	uint64_t *host = malloc(staged);
	struct vkh_devtab *d = calloc(1, sizeof(*d));
	if (!host || !d) {
		free(host);
		free(d);
		return vkh_fail(ctx, VKHEL_ERR_OUT_OF_MEMORY, "tables: host staging failed");
	}
	void *mem = NULL;
	int st = vkh_dev_alloc(ctx, bytes, &mem);
	if (st != VKHEL_OK) {
		free(host);
		free(d);
		return st;
	}
	vkcu_twset s;
	memset(&s, 0, sizeof s);
	s.q = t->q;
	s.q2 = 2 * t->q;
	s.mu = t->mu;
	s.ninv = t->ninv;
	s.ninv_s = t->ninv_s;
	s.w1ninv = t->w1ninv;
	s.w1ninv_s = t->w1ninv_s;
	s.qbits = t->qbits;
	s.log_n = t->log_n;
	s.fwd = (const uint64_t *) ((char *) mem + head);
	s.inv = s.fwd + 2 * n;
	memcpy(host, &s, sizeof s);
	if (t->device_gen) {
		/* header + the two short power tables; the kernel fills the rest */
		uint64_t *plo = host + head / 8, *phi = plo + nlo;
		plo[0] = 1;
		for (uint64_t k = 1; k < nlo; k++)
			plo[k] = vkh_mulmod(plo[k - 1], t->w_red, t->q);
		const uint64_t wb = vkh_mulmod(plo[nlo - 1], t->w_red, t->q); /* w^(2^lb) */
		phi[0] = 1;
		for (uint64_t j = 1; j < nhi; j++)
			phi[j] = vkh_mulmod(phi[j - 1], wb, t->q);
		uint64_t *dev_pow = (uint64_t *) ((char *) mem + table_bytes);
		st = vkcu_h2d(ctx->stream, mem, host, head);
		if (!st)
			st = vkcu_h2d(ctx->stream, dev_pow, plo, 8 * (nlo + nhi));
		if (!st)
			st = vkcu_twiddles(ctx->stream, (uint64_t *) s.fwd, (uint64_t *) s.inv, dev_pow + nlo, dev_pow,
					t->log_n, lb, t->q, t->mu, t->qbits);
	} else {
		uint64_t *fwd = host + head / 8, *inv = fwd + 2 * n;
		for (uint64_t i = 0; i < n; i++) {
			fwd[2 * i] = t->roots[i];
			fwd[2 * i + 1] = t->roots_shoup[i];
			inv[2 * i] = t->inv_roots[i];
			inv[2 * i + 1] = t->inv_roots_shoup[i];
		}
		st = vkcu_h2d(ctx->stream, mem, host, bytes);
	}
	if (st == 0)
		st = vkcu_sync(ctx->stream);
	free(host);
	if (st != 0) {
		vkh_dev_free(ctx, mem, bytes);
		free(d);
		return vkh_cuda(ctx, st, "tables upload");
	}
	d->n = t->n;
	d->q = t->q;
	d->w = t->w;
	d->mem = mem;
	d->bytes = bytes;
	d->dev_set = (const vkcu_twset *) mem;
	d->host_set = s;
	d->next = ctx->tabs;
	ctx->tabs = d;
	*out = d;
	return VKHEL_OK;
}

int vkhel_ntt_tables_device_copy(struct vkhel_ctx *ctx, const struct vkhel_ntt_tables *t, uint64_t *roots,
		uint64_t *inv_roots, uint64_t *roots_shoup, uint64_t *inv_roots_shoup) {
	if (!ctx || !t)
		return vkh_fail(ctx, VKHEL_ERR_INVALID_ARGUMENT, "tables_device_copy: NULL argument");
	const struct vkh_devtab *d = NULL;
	int st = vkh_devtab_get(ctx, t, &d);
	if (st)
		return st;
	const uint64_t n = t->n;
	uint64_t *h = malloc(2 * 16 * n);
	if (!h)
		return vkh_fail(ctx, VKHEL_ERR_OUT_OF_MEMORY, "tables_device_copy: host allocation failed");
	int e = vkcu_d2h(ctx->stream, h, d->host_set.fwd, 2 * 16 * n);
	if (!e)
		e = vkcu_sync(ctx->stream);
	if (!e) {
		for (uint64_t i = 0; i < n; i++) {
			if (roots)
				roots[i] = h[2 * i];
			if (roots_shoup)
				roots_shoup[i] = h[2 * i + 1];
			if (inv_roots)
				inv_roots[i] = h[2 * n + 2 * i];
			if (inv_roots_shoup)
				inv_roots_shoup[i] = h[2 * n + 2 * i + 1];
		}
	}
	free(h);
	return vkh_cuda(ctx, e, "tables_device_copy");
}

const struct vkh_devtab *vkh_devtab_find(const struct vkhel_ctx *ctx, const struct vkhel_ntt_tables *t) {
	for (const struct vkh_devtab *d = ctx->tabs; d; d = d->next)
		if (d->n == t->n && d->q == t->q && d->w == t->w)
			return d;
	return NULL;
}

void vkh_devtab_release_all(struct vkhel_ctx *ctx) {
	struct vkh_devtab *d = ctx->tabs;
	while (d) {
		struct vkh_devtab *next = d->next;
		vkh_dev_free(ctx, d->mem, d->bytes);
		free(d);
		d = next;
	}
	ctx->tabs = NULL;
}
