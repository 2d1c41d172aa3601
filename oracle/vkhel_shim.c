/*
 * Host-memory implementation of the public vkhel API over the CPU oracle --
 * TEST INFRASTRUCTURE ONLY.
 *
 * Purpose: the reference's own GPU test program (test/vector.c) includes only
 * the public header, so it can be compiled unmodified against this file.  When
 * its assertions pass, every golden vector in that program has been reproduced
 * by the oracle.  With VKHEL_SHIM_LOG=<path> set, every operation is appended
 * to <path> as one JSON line (operation, parameters, inputs, output), which is
 * how tests/golden/reference_vectors.json is produced.
 *
 * Semantics follow src/vector.c: create zero-fills unless create2(.., false)
 * (vector.c:211-229), map returns a host window of the device contents
 * (vector.c:270-283), unmap writes `length` elements back (vector.c:285-296),
 * element-wise ops take their length from `result` (e.g. elemmul.c:164),
 * forward/inverse transform work on the first n elements and the inverse then
 * scales all `result->length` elements by n^-1 (vector.c:632-638).
 */
#include <inttypes.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "vkhel.h"
#include "oracle.h"

struct vkhel_ctx {
	int unused;
};

struct vkhel_vector {
	struct vkhel_ctx *ctx;
	uint64_t length;
	uint64_t *data;
	uint64_t *window;
};

struct vkhel_ntt_tables {
	uint64_t n, q, w;
	uint64_t *roots, *inv_roots, *roots_shoup, *inv_roots_shoup;
};

static FILE *log_file(void) {
	static FILE *f;
	static int opened;
	if (!opened) {
		opened = 1;
		const char *p = getenv("VKHEL_SHIM_LOG");
		if (p && *p)
			f = fopen(p, "a");
	}
	return f;
}

static void log_array(FILE *f, const char *key, const uint64_t *v, uint64_t n) {
	fprintf(f, "\"%s\": [", key);
	for (uint64_t i = 0; i < n; i++)
		fprintf(f, i ? ", \"%" PRIu64 "\"" : "\"%" PRIu64 "\"", v[i]);
	fprintf(f, "]");
}

/* One JSON object per operation; numbers are written as decimal strings so
 * that 64-bit values survive any JSON reader. */
static void log_op(const char *op, const char *params,
		const uint64_t *a, const uint64_t *b, uint64_t in_len,
		const uint64_t *out, uint64_t out_len) {
	FILE *f = log_file();
	if (!f)
		return;
	fprintf(f, "{\"op\": \"%s\", \"params\": {%s}, ", op, params);
	if (a) {
		log_array(f, "a", a, in_len);
		fprintf(f, ", ");
	}
	if (b) {
		log_array(f, "b", b, in_len);
		fprintf(f, ", ");
	}
	log_array(f, "expected", out, out_len);
	fprintf(f, "}\n");
	fflush(f);
}

struct vkhel_ctx *vkhel_ctx_create() {
	return calloc(1, sizeof(struct vkhel_ctx));
}

void vkhel_ctx_destroy(struct vkhel_ctx *ctx) {
	free(ctx);
}

struct vkhel_ntt_tables *vkhel_ntt_tables_create(uint64_t n, uint64_t q,
		uint64_t w) {
	struct vkhel_ntt_tables *t = calloc(1, sizeof(*t));
	t->n = n;
	t->q = q;
	t->w = w;
	t->roots = malloc(sizeof(uint64_t) * n);
	t->inv_roots = malloc(sizeof(uint64_t) * n);
	t->roots_shoup = malloc(sizeof(uint64_t) * n);
	t->inv_roots_shoup = malloc(sizeof(uint64_t) * n);
	orc_ntt_tables(n, q, w, t->roots, t->inv_roots, t->roots_shoup,
			t->inv_roots_shoup);
	return t;
}

void vkhel_ntt_tables_destroy(struct vkhel_ntt_tables *t) {
	free(t->roots);
	free(t->inv_roots);
	free(t->roots_shoup);
	free(t->inv_roots_shoup);
	free(t);
}

struct vkhel_vector *vkhel_vector_create(struct vkhel_ctx *ctx, uint64_t length) {
	return vkhel_vector_create2(ctx, length, true);
}

struct vkhel_vector *vkhel_vector_create2(struct vkhel_ctx *ctx,
		uint64_t length, bool zero) {
	struct vkhel_vector *v = calloc(1, sizeof(*v));
	v->ctx = ctx;
	v->length = length;
	v->data = malloc(sizeof(uint64_t) * (length ? length : 1));
	if (zero)
		memset(v->data, 0, sizeof(uint64_t) * length);
	return v;
}

void vkhel_vector_destroy(struct vkhel_vector *v) {
	free(v->window);
	free(v->data);
	free(v);
}

struct vkhel_vector *vkhel_vector_dup(struct vkhel_vector *src) {
	struct vkhel_vector *v = vkhel_vector_create2(src->ctx, src->length, false);
	memcpy(v->data, src->data, sizeof(uint64_t) * src->length);
	log_op("dup", "", src->data, NULL, src->length, v->data, v->length);
	return v;
}

void vkhel_vector_copy_from_host(struct vkhel_vector *v, const uint64_t *e) {
	memcpy(v->data, e, sizeof(uint64_t) * v->length);
	log_op("copy_from_host", "", e, NULL, v->length, v->data, v->length);
}

void vkhel_vector_map(struct vkhel_vector *v, void **mem, size_t size) {
	const size_t bytes = sizeof(uint64_t) * v->length;
	v->window = calloc(1, size > bytes ? size : bytes);
	memcpy(v->window, v->data, bytes);
	*mem = v->window;
}

void vkhel_vector_unmap(struct vkhel_vector *v) {
	memcpy(v->data, v->window, sizeof(uint64_t) * v->length);
	free(v->window);
	v->window = NULL;
}

void vkhel_vector_elemfma(const struct vkhel_vector *a,
		const struct vkhel_vector *b, struct vkhel_vector *res,
		uint64_t multiplier, uint64_t mod) {
	uint64_t *in_a = malloc(sizeof(uint64_t) * res->length);
	uint64_t *in_b = malloc(sizeof(uint64_t) * res->length);
	memcpy(in_a, a->data, sizeof(uint64_t) * res->length);
	memcpy(in_b, b->data, sizeof(uint64_t) * res->length);
	orc_elemfma(in_a, in_b, res->data, res->length, multiplier, mod);
	char params[128];
	snprintf(params, sizeof params,
			"\"multiplier\": \"%" PRIu64 "\", \"mod\": \"%" PRIu64 "\"",
			multiplier, mod);
	log_op("elemfma", params, in_a, in_b, res->length, res->data, res->length);
	free(in_a);
	free(in_b);
}

void vkhel_vector_elemmod(const struct vkhel_vector *a,
		struct vkhel_vector *res, uint64_t mod, uint64_t q) {
	uint64_t *in_a = malloc(sizeof(uint64_t) * res->length);
	memcpy(in_a, a->data, sizeof(uint64_t) * res->length);
	orc_elemmod(in_a, res->data, res->length, mod, q);
	char params[128];
	snprintf(params, sizeof params,
			"\"mod\": \"%" PRIu64 "\", \"q\": \"%" PRIu64 "\"", mod, q);
	log_op("elemmod", params, in_a, NULL, res->length, res->data, res->length);
	free(in_a);
}

void vkhel_vector_elemmul(const struct vkhel_vector *a,
		const struct vkhel_vector *b, struct vkhel_vector *res, uint64_t mod) {
	uint64_t *in_a = malloc(sizeof(uint64_t) * res->length);
	uint64_t *in_b = malloc(sizeof(uint64_t) * res->length);
	memcpy(in_a, a->data, sizeof(uint64_t) * res->length);
	memcpy(in_b, b->data, sizeof(uint64_t) * res->length);
	orc_elemmul(in_a, in_b, res->data, res->length, mod);
	char params[64];
	snprintf(params, sizeof params, "\"mod\": \"%" PRIu64 "\"", mod);
	log_op("elemmul", params, in_a, in_b, res->length, res->data, res->length);
	free(in_a);
	free(in_b);
}

void vkhel_vector_elemgtadd(const struct vkhel_vector *a,
		struct vkhel_vector *res, uint64_t bound, uint64_t diff) {
	uint64_t *in_a = malloc(sizeof(uint64_t) * res->length);
	memcpy(in_a, a->data, sizeof(uint64_t) * res->length);
	orc_elemgtadd(in_a, res->data, res->length, bound, diff);
	char params[128];
	snprintf(params, sizeof params,
			"\"bound\": \"%" PRIu64 "\", \"diff\": \"%" PRIu64 "\"", bound, diff);
	log_op("elemgtadd", params, in_a, NULL, res->length, res->data, res->length);
	free(in_a);
}

void vkhel_vector_elemgtsub(const struct vkhel_vector *a,
		struct vkhel_vector *res, uint64_t bound, uint64_t diff, uint64_t mod) {
	uint64_t *in_a = malloc(sizeof(uint64_t) * res->length);
	memcpy(in_a, a->data, sizeof(uint64_t) * res->length);
	orc_elemgtsub(in_a, res->data, res->length, bound, diff, mod);
	char params[160];
	snprintf(params, sizeof params,
			"\"bound\": \"%" PRIu64 "\", \"diff\": \"%" PRIu64
			"\", \"mod\": \"%" PRIu64 "\"", bound, diff, mod);
	log_op("elemgtsub", params, in_a, NULL, res->length, res->data, res->length);
	free(in_a);
}

static void transform(const char *op, const struct vkhel_vector *operand,
		struct vkhel_vector *res, struct vkhel_ntt_tables *t, int inverse) {
	const uint64_t n = t->n;
	uint64_t *in = malloc(sizeof(uint64_t) * n);
	memcpy(in, operand->data, sizeof(uint64_t) * n);
	if (!inverse) {
		if (n > 1) {
			memcpy(res->data, in, sizeof(uint64_t) * n);
			orc_ntt_forward(res->data, n, t->q, t->roots, t->roots_shoup);
		}
	} else {
		if (n > 1) {
			memcpy(res->data, in, sizeof(uint64_t) * n);
			orc_ntt_inverse(res->data, n, t->q, t->inv_roots, t->inv_roots_shoup);
		} else {
			orc_elemmulconst(res->data, res->data, n, orc_invmod(n, t->q), t->q);
		}
		/* vector.c:635-638 scales result->length elements, not n. */
		if (res->length > n)
			orc_elemmulconst(res->data + n, res->data + n, res->length - n,
					orc_invmod(n, t->q), t->q);
	}
	char params[160];
	snprintf(params, sizeof params,
			"\"n\": \"%" PRIu64 "\", \"q\": \"%" PRIu64 "\", \"w\": \"%" PRIu64 "\"",
			t->n, t->q, t->w);
	log_op(op, params, in, NULL, n, res->data, n);
	free(in);
}

void vkhel_vector_forward_transform(const struct vkhel_vector *operand,
		struct vkhel_vector *res, struct vkhel_ntt_tables *t) {
	transform("forward_transform", operand, res, t, 0);
}

void vkhel_vector_inverse_transform(const struct vkhel_vector *operand,
		struct vkhel_vector *res, struct vkhel_ntt_tables *t) {
	transform("inverse_transform", operand, res, t, 1);
}
