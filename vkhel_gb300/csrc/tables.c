/*
 * NTT twiddle tables: host construction (values identical to the reference's
 * src/ntt_tables.c:17-44) and the per-context device cache.
 *
 * Host side.  roots[bitrev(i)] = w^i by repeated Barrett multiplication
 * (ntt_tables.c:25-34).  The reference inverts every root with extended
 * Euclid; when w^n = -1 (a primitive 2n-th root, the case every caller uses)
 * the same canonical values follow by index, w^-i = -w^(n-i), at no cost, and
 * Euclid is kept for any other w.  Shoup factors floor(r 2^64 / q) as in
 * ntt_tables.c:36-43.
 *
 * Device side.  One pool allocation per (n, q, w) holds a vkcu_twset header
 * and the forward and inverse tables as interleaved (root, shoup) pairs so a
 * butterfly fetches its twiddle with one 16-byte load.  Contexts cache these
 * by value, so separately created table objects with equal parameters share
 * one device copy.
 */
#include <inttypes.h>
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

struct vkhel_ntt_tables *vkhel_ntt_tables_create(uint64_t n, uint64_t q, uint64_t w) {
	if (n == 0 || (n & (n - 1)) != 0) {
		vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT,
				"ntt tables: n=%" PRIu64 " is not a power of two", n);
		return NULL;
	}
	if (q < 2 || n >= ((uint64_t) 1 << 40)) {
		vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT,
				"ntt tables: unsupported n=%" PRIu64 " q=%" PRIu64, n, q);
		return NULL;
	}
	struct vkhel_ntt_tables *t = calloc(1, sizeof(*t));
	uint64_t *mem = malloc(sizeof(uint64_t) * 4 * n);
	if (!t || !mem) {
		free(t);
		free(mem);
		vkh_fail(NULL, VKHEL_ERR_OUT_OF_MEMORY, "ntt tables: host allocation failed");
		return NULL;
	}
	t->n = n;
	t->q = q;
	t->w = w;
	t->log_n = (uint32_t) vkh_bitlen(n) - 1;
	t->roots = mem;
	t->inv_roots = mem + n;
	t->roots_shoup = mem + 2 * n;
	t->inv_roots_shoup = mem + 3 * n;

	t->roots[0] = 1;
	uint64_t power = 1;
	bool canonical = true;
	for (uint64_t i = 1; i < n; i++) {
		power = vkh_mulmod(power, w, q);
		t->roots[bit_reverse(i, t->log_n)] = power;
		canonical &= power < q && power != 0;
	}
	const bool negacyclic = canonical && n > 1 && vkh_mulmod(power, w, q) == q - 1;
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
	}

	t->qbits = (uint32_t) vkh_bitlen(q);
	t->mu = t->qbits >= 2 ? vkh_barrett_mu(q) : 0;
	t->ninv = vkh_invmod(n, q); /* src/vector.c:633 */
	t->ninv_s = vkh_shoup(t->ninv, q);
	const uint64_t w1 = n > 1 ? t->inv_roots[1] : 1;
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

int vkhel_ntt_tables_copy(const struct vkhel_ntt_tables *t, uint64_t *roots,
		uint64_t *inv_roots, uint64_t *roots_shoup, uint64_t *inv_roots_shoup) {
	if (!t)
		return vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "ntt tables: NULL");
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
	const uint64_t bytes = head + 2 * 16 * n;
	uint64_t *host = malloc(bytes);
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
	uint64_t *fwd = host + head / 8, *inv = fwd + 2 * n;
	for (uint64_t i = 0; i < n; i++) {
		fwd[2 * i] = t->roots[i];
		fwd[2 * i + 1] = t->roots_shoup[i];
		inv[2 * i] = t->inv_roots[i];
		inv[2 * i + 1] = t->inv_roots_shoup[i];
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
	st = vkcu_h2d(ctx->stream, mem, host, bytes);
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
