/*
 * Drop-in check through the public C header only (include/vkhel/vkhel.h).
 *
 * Replays recorded golden operations with the call pattern of the reference's
 * own test program (test/vector.c:13-21 and its tests): vkhel_vector_create,
 * vkhel_vector_copy_from_host, the operation, then vkhel_vector_map /
 * vkhel_vector_unmap to read the result.  The cases come from a text file
 * written by tests/test_c_api.py from tests/golden/reference_vectors.json:
 *
 *   <op> <p0> <p1> <p2>      operation name and up to three parameters
 *   a <len> <words...>
 *   b <len> <words...>       (binary operations only)
 *   e <len> <words...>       expected result
 *
 * Exit status: 0 all cases matched, 1 a mismatch, 77 no CUDA device.
 */
#include <inttypes.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vkhel.h>

static int read_words(FILE *f, const char *tag, uint64_t **out, size_t *len) {
	char t[8];
	if (fscanf(f, "%7s %zu", t, len) != 2 || strcmp(t, tag) != 0)
		return -1;
	*out = malloc(sizeof(uint64_t) * (*len ? *len : 1));
	for (size_t i = 0; i < *len; i++)
		if (fscanf(f, "%" SCNu64, &(*out)[i]) != 1)
			return -1;
	return 0;
}

static int matches(struct vkhel_vector *v, const uint64_t *expect, size_t len) {
	uint64_t *mapped = NULL;
	vkhel_vector_map(v, (void **) &mapped, sizeof(uint64_t) * len);
	if (!mapped)
		return 0;
	int ok = 1;
	for (size_t i = 0; i < len; i++)
		ok &= mapped[i] == expect[i];
	vkhel_vector_unmap(v);
	return ok;
}

int main(int argc, char **argv) {
	if (argc != 2) {
		fprintf(stderr, "usage: %s cases.txt\n", argv[0]);
		return 2;
	}
	struct vkhel_ctx *ctx = vkhel_ctx_create();
	if (!ctx) {
		printf("no CUDA device\n");
		return 77;
	}
	FILE *f = fopen(argv[1], "r");
	if (!f)
		return 2;
	char op[64];
	uint64_t p[3];
	int cases = 0, failed = 0;
	while (fscanf(f, "%63s %" SCNu64 " %" SCNu64 " %" SCNu64, op, &p[0], &p[1], &p[2]) == 4) {
		uint64_t *a = NULL, *b = NULL, *e = NULL;
		size_t la = 0, lb = 0, le = 0;
		const int binary = !strcmp(op, "elemfma") || !strcmp(op, "elemmul");
		if (read_words(f, "a", &a, &la) || (binary && read_words(f, "b", &b, &lb)) || read_words(f, "e", &e, &le)) {
			fprintf(stderr, "bad case file near case %d\n", cases);
			return 2;
		}
		struct vkhel_vector *va = vkhel_vector_create(ctx, la);
		vkhel_vector_copy_from_host(va, a);
		struct vkhel_vector *vb = NULL, *res = NULL;
		struct vkhel_ntt_tables *t = NULL;
		if (binary) {
			vb = vkhel_vector_create(ctx, lb);
			vkhel_vector_copy_from_host(vb, b);
		}
		if (!strcmp(op, "copy_from_host")) {
			res = va;
		} else if (!strcmp(op, "dup")) {
			res = vkhel_vector_dup(va);
		} else if (!strcmp(op, "forward_transform") || !strcmp(op, "inverse_transform")) {
			t = vkhel_ntt_tables_create(p[0], p[1], p[2]);
			res = vkhel_vector_create(ctx, p[0]);
			if (op[0] == 'f')
				vkhel_vector_forward_transform(va, res, t);
			else
				vkhel_vector_inverse_transform(va, res, t);
		} else {
			res = vkhel_vector_create(ctx, le);
			if (!strcmp(op, "elemfma"))
				vkhel_vector_elemfma(va, vb, res, p[0], p[1]);
			else if (!strcmp(op, "elemmul"))
				vkhel_vector_elemmul(va, vb, res, p[0]);
			else if (!strcmp(op, "elemmod"))
				vkhel_vector_elemmod(va, res, p[0], p[1]);
			else if (!strcmp(op, "elemgtadd"))
				vkhel_vector_elemgtadd(va, res, p[0], p[1]);
			else if (!strcmp(op, "elemgtsub"))
				vkhel_vector_elemgtsub(va, res, p[0], p[1], p[2]);
		}
		const int ok = matches(res, e, le);
		printf("%-18s %s\n", op, ok ? "ok" : "MISMATCH");
		failed += !ok;
		cases++;
		if (res != va)
			vkhel_vector_destroy(res);
		vkhel_vector_destroy(va);
		if (vb)
			vkhel_vector_destroy(vb);
		if (t)
			vkhel_ntt_tables_destroy(t);
		free(a);
		free(b);
		free(e);
	}
	fclose(f);
	vkhel_ctx_destroy(ctx);
	printf("%d cases, %d failed\n", cases, failed);
	return failed ? 1 : 0;
}
