/*
 * The extension API (include/vkhel/vkhel_ext.h) as a C program sees it.
 *
 * Checks, against a schoolbook negacyclic product and plain C modular
 * arithmetic computed here (unsigned __int128):
 *   - vkhel_vector_polymul and vkhel_vector_polymul_lift (centred elemmod);
 *   - vkhel_vector_polymul_ntt with NTT(b) from vkhel_vector_forward_transform;
 *   - a committed batch (CUDA graph) of three RNS limb products with a lift;
 *   - an element-wise batch (elemmul, elemgtadd, elemfma_canonical);
 *   - one server request with host operands, and one on a resident operand;
 *   - status reporting (vkhel_ctx_last_error) for a bad argument.
 *
 *   test_vkhel_ext N Q0 W0 Q1 W1 Q2 W2
 *
 * N is a power of two in [256, 16384]; (Qk, Wk) are NTT-friendly primes with
 * primitive 2N-th roots.  Exit status: 0 all checks passed, 1 a mismatch,
 * 77 no CUDA device.
 */
#include <inttypes.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vkhel.h>
#include <vkhel_ext.h>

typedef unsigned __int128 u128;

static uint64_t rng_state = 0x9e3779b97f4a7c15ull;
static uint64_t next_rand(void) { /* splitmix64 */
	uint64_t z = (rng_state += 0x9e3779b97f4a7c15ull);
	z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
	z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
	return z ^ (z >> 31);
}

/* c = a * b mod (X^n + 1, q), schoolbook */
static void negacyclic(const uint64_t *a, const uint64_t *b, uint64_t *c, uint64_t n, uint64_t q) {
	memset(c, 0, n * sizeof(uint64_t));
	for (uint64_t i = 0; i < n; i++)
		for (uint64_t j = 0; j < n; j++) {
			const uint64_t p = (uint64_t) (((u128) a[i] * b[j]) % q);
			const uint64_t k = i + j;
			if (k < n)
				c[k] = (uint64_t) (((u128) c[k] + p) % q);
			else
				c[k - n] = (uint64_t) (((u128) c[k - n] + q - p) % q);
		}
}

/* the reference's elemmod with mod != 2 on canonical x: x > q/2 ? (x - q) mod t : x mod t */
static uint64_t centred_mod(uint64_t x, uint64_t t, uint64_t q) {
	const uint64_t r = x % t;
	if (x <= q / 2)
		return r;
	const uint64_t d = q % t;
	return (r + t - d) % t;
}

static int failures = 0;
static void check(int ok, const char *what) {
	printf("%-40s %s\n", what, ok ? "ok" : "MISMATCH");
	failures += !ok;
}

static int equal(const uint64_t *x, const uint64_t *y, uint64_t n) {
	for (uint64_t i = 0; i < n; i++)
		if (x[i] != y[i])
			return 0;
	return 1;
}

int main(int argc, char **argv) {
	if (argc != 8) {
		fprintf(stderr, "usage: %s N Q0 W0 Q1 W1 Q2 W2\n", argv[0]);
		return 2;
	}
	const uint64_t n = strtoull(argv[1], NULL, 10);
	uint64_t qs[3], ws[3];
	for (int k = 0; k < 3; k++) {
		qs[k] = strtoull(argv[2 + 2 * k], NULL, 10);
		ws[k] = strtoull(argv[3 + 2 * k], NULL, 10);
	}
	struct vkhel_ctx *ctx = vkhel_ctx_create();
	if (!ctx) {
		printf("no CUDA device\n");
		return 77;
	}
	const uint64_t t_plain = 65537;
	struct vkhel_ntt_tables *tab[3];
	for (int k = 0; k < 3; k++)
		tab[k] = vkhel_ntt_tables_create(n, qs[k], ws[k]);

	uint64_t *a = malloc(3 * n * 8), *b = malloc(3 * n * 8), *c = malloc(3 * n * 8), *ref = malloc(3 * n * 8);
	for (int k = 0; k < 3; k++)
		for (uint64_t i = 0; i < n; i++) {
			a[k * n + i] = next_rand() % qs[k];
			b[k * n + i] = next_rand() % qs[k];
		}
	for (int k = 0; k < 3; k++)
		negacyclic(a + k * n, b + k * n, ref + k * n, n, qs[k]);

	/* single polymul and lifted polymul on limb 0 */
	struct vkhel_vector *va = vkhel_vector_create(ctx, n), *vb = vkhel_vector_create(ctx, n),
			*vc = vkhel_vector_create(ctx, n);
	vkhel_vector_upload(va, a, n);
	vkhel_vector_upload(vb, b, n);
	int st = vkhel_vector_polymul(va, vb, vc, tab[0]);
	vkhel_vector_download(vc, c, n);
	check(st == VKHEL_OK && equal(c, ref, n), "vkhel_vector_polymul");
	const struct vkhel_lift_step lift = {VKHEL_LIFT_ELEMMOD, t_plain, 0, 0};
	st = vkhel_vector_polymul_lift(va, vb, vc, tab[0], &lift, 1);
	vkhel_vector_download(vc, c, n);
	int ok = st == VKHEL_OK;
	for (uint64_t i = 0; ok && i < n; i++)
		ok = c[i] == centred_mod(ref[i], t_plain, qs[0]);
	check(ok, "vkhel_vector_polymul_lift (elemmod)");
	struct vkhel_vector *vbh = vkhel_vector_create(ctx, n);
	vkhel_vector_forward_transform(vb, vbh, tab[0]);
	st = vkhel_vector_polymul_ntt(va, vbh, vc, tab[0]);
	vkhel_vector_download(vc, c, n);
	check(st == VKHEL_OK && equal(c, ref, n), "vkhel_vector_polymul_ntt (NTT(b) kept)");
	vkhel_vector_destroy(vbh);

	/* batch of three RNS limbs with the lift, replayed from a CUDA graph */
	struct vkhel_vector *ba = vkhel_vector_create(ctx, 3 * n), *bb = vkhel_vector_create(ctx, 3 * n),
			*bc = vkhel_vector_create(ctx, 3 * n);
	vkhel_vector_upload(ba, a, 3 * n);
	vkhel_vector_upload(bb, b, 3 * n);
	struct vkhel_batch *bt = vkhel_batch_create(ctx);
	st = vkhel_batch_add_polymul_lift(bt, tab, 3, ba, bb, bc, &lift, 1);
	if (!st)
		st = vkhel_batch_commit(bt, VKHEL_BATCH_GRAPH);
	if (!st)
		st = vkhel_batch_run(bt);
	vkhel_vector_download(bc, c, 3 * n);
	ok = st == VKHEL_OK;
	for (int k = 0; ok && k < 3; k++)
		for (uint64_t i = 0; ok && i < n; i++)
			ok = c[k * n + i] == centred_mod(ref[k * n + i], t_plain, qs[k]);
	check(ok, "vkhel_batch (3 limbs, lift, graph)");
	vkhel_batch_destroy(bt);

	/* element-wise batch over the three limbs */
	struct vkhel_vector *e1 = vkhel_vector_create(ctx, n), *e2 = vkhel_vector_create(ctx, n),
			*e3 = vkhel_vector_create(ctx, n);
	struct vkhel_elem_batch *eb = vkhel_elem_batch_create(ctx);
	st = vkhel_elem_batch_add(eb, VKHEL_ELEM_MUL, qs[0], 0, 0, va, vb, e1);
	if (!st)
		st = vkhel_elem_batch_add(eb, VKHEL_ELEM_GTADD, qs[0] / 2, 7, 0, va, NULL, e2);
	if (!st)
		st = vkhel_elem_batch_add(eb, VKHEL_ELEM_FMA_CANONICAL, 12345, qs[0], 0, va, vb, e3);
	if (!st)
		st = vkhel_elem_batch_commit(eb, 0);
	if (!st)
		st = vkhel_elem_batch_run(eb);
	uint64_t *r1 = malloc(n * 8), *r2 = malloc(n * 8), *r3 = malloc(n * 8);
	vkhel_vector_download(e1, r1, n);
	vkhel_vector_download(e2, r2, n);
	vkhel_vector_download(e3, r3, n);
	ok = st == VKHEL_OK;
	for (uint64_t i = 0; ok && i < n; i++) {
		const uint64_t x = a[i], y = b[i];
		ok = r1[i] == (uint64_t) (((u128) x * y) % qs[0]) && r2[i] == (x > qs[0] / 2 ? x + 7 : x) &&
				r3[i] == (uint64_t) (((u128) x * 12345 + y) % qs[0]);
	}
	check(ok, "vkhel_elem_batch (mul, gtadd, fma)");
	vkhel_elem_batch_destroy(eb);

	/* one server request with host operands */
	struct vkhel_server_config cfg = {0, 0, 0};
	struct vkhel_server *srv = vkhel_server_create(&cfg);
	ok = srv != NULL;
	if (ok) {
		memset(c, 0, 3 * n * 8);
		const int64_t id = vkhel_server_submit(srv, tab, 3, a, b, c);
		ok = id > 0 && vkhel_server_wait(srv, id, 10000) == VKHEL_OK && equal(c, ref, 3 * n);
		const int64_t op = vkhel_server_add_operand(srv, tab, 3, b, 0);
		memset(c, 0, 3 * n * 8);
		const int64_t id2 = op > 0 ? vkhel_server_submit_operand(srv, tab, 3, a, op, c) : -1;
		ok = ok && id2 > 0 && vkhel_server_wait(srv, id2, 10000) == VKHEL_OK && equal(c, ref, 3 * n) &&
				vkhel_server_remove_operand(srv, op) == VKHEL_OK;
		vkhel_server_destroy(srv);
	}
	check(ok, "vkhel_server (one 3-limb request, then one on a resident operand)");

	/* status reporting */
	struct vkhel_vector *small = vkhel_vector_create(ctx, n / 2);
	st = vkhel_vector_polymul(va, vb, small, tab[0]);
	char msg[128];
	check(st == VKHEL_ERR_INVALID_ARGUMENT && vkhel_ctx_last_error(ctx, msg, sizeof msg) == st,
			"status for a short result vector");
	vkhel_ctx_clear_error(ctx);

	vkhel_vector_destroy(small);
	vkhel_vector_destroy(e1);
	vkhel_vector_destroy(e2);
	vkhel_vector_destroy(e3);
	vkhel_vector_destroy(ba);
	vkhel_vector_destroy(bb);
	vkhel_vector_destroy(bc);
	vkhel_vector_destroy(va);
	vkhel_vector_destroy(vb);
	vkhel_vector_destroy(vc);
	for (int k = 0; k < 3; k++)
		vkhel_ntt_tables_destroy(tab[k]);
	vkhel_ctx_destroy(ctx);
	free(a);
	free(b);
	free(c);
	free(ref);
	free(r1);
	free(r2);
	free(r3);
	printf("%d checks failed\n", failures);
	return failures ? 1 : 0;
}
