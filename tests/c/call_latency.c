/*
 * Per-call latency of the public C API, as a C caller of the reference sees
 * it: each call is timed with a monotonic host clock around `reps` calls
 * (best of 5 such loops), with the calls blocking as the reference's do, and
 * again on a stream-ordered context (vkhel_ctx_set_async) where the loop
 * ends with one vkhel_ctx_sync.
 *
 *   call_latency N_PRIME_16384 W_16384 Q_4096 W_4096 Q_65536 W_65536 [reps]
 *
 * The NTT-friendly primes and roots come from the caller.  Prints one JSON
 * object; exit status 0, or 77 without a CUDA device.
 */
#include <inttypes.h>
#include <stdio.h>
#include <stdlib.h>
#include <time.h>

#include <vkhel.h>
#include <vkhel_ext.h>

static double now_us(void) {
	struct timespec ts;
	clock_gettime(CLOCK_MONOTONIC, &ts);
	return 1e6 * (double) ts.tv_sec + 1e-3 * (double) ts.tv_nsec;
}

enum { OP_GTADD1, OP_FWD, OP_INV, OP_MUL };

struct op_case {
	const char *name;
	int op;
	int table; /* index into tabs (-1: none) */
};

static void run(int op, struct vkhel_vector *a, struct vkhel_vector *b, struct vkhel_vector *c,
		struct vkhel_vector *w1, struct vkhel_ntt_tables *t) {
	switch (op) {
	case OP_GTADD1:
		vkhel_vector_elemgtadd(w1, w1, 3, 1);
		break;
	case OP_FWD:
		vkhel_vector_forward_transform(a, c, t);
		break;
	case OP_INV:
		vkhel_vector_inverse_transform(c, c, t);
		break;
	default:
		vkhel_vector_polymul(a, b, c, t);
		break;
	}
}

int main(int argc, char **argv) {
	if (argc < 7) {
		fprintf(stderr, "usage: %s Q16384 W16384 Q4096 W4096 Q65536 W65536 [reps]\n", argv[0]);
		return 2;
	}
	const int reps = argc > 7 ? atoi(argv[7]) : 2000;
	struct vkhel_ctx *ctx = vkhel_ctx_create();
	if (!ctx)
		return 77;
	const uint64_t ns[3] = {16384, 4096, 65536};
	struct vkhel_ntt_tables *tabs[3];
	struct vkhel_vector *va[3], *vb[3], *vc[3];
	for (int k = 0; k < 3; k++) {
		tabs[k] = vkhel_ntt_tables_create(ns[k], strtoull(argv[1 + 2 * k], NULL, 10),
				strtoull(argv[2 + 2 * k], NULL, 10));
		va[k] = vkhel_vector_create(ctx, ns[k]);
		vb[k] = vkhel_vector_create(ctx, ns[k]);
		vc[k] = vkhel_vector_create(ctx, ns[k]);
		if (!tabs[k] || !va[k] || !vb[k] || !vc[k])
			return 1;
	}
	struct vkhel_vector *w1 = vkhel_vector_create(ctx, 1);
	const struct op_case cases[] = {
			{"elemgtadd_1_word", OP_GTADD1, -1}, {"forward_4096", OP_FWD, 1},
			{"forward_16384", OP_FWD, 0},        {"inverse_16384", OP_INV, 0},
			{"polymul_16384", OP_MUL, 0},        {"forward_65536", OP_FWD, 2},
			{"polymul_65536", OP_MUL, 2},
	};
	const int ncases = (int) (sizeof cases / sizeof cases[0]);
	printf("{\"reps\": %d", reps);
	for (int mode = 0; mode < 2; mode++) {
		vkhel_ctx_set_async(ctx, mode);
		printf(", \"%s\": {", mode ? "stream_ordered_us" : "blocking_us");
		for (int i = 0; i < ncases; i++) {
			const int k = cases[i].table < 0 ? 0 : cases[i].table;
			for (int r = 0; r < 20; r++)
				run(cases[i].op, va[k], vb[k], vc[k], w1, tabs[k]);
			vkhel_ctx_sync(ctx);
			double best = 1e30;
			for (int loop = 0; loop < 5; loop++) {
				const double t0 = now_us();
				for (int r = 0; r < reps; r++)
					run(cases[i].op, va[k], vb[k], vc[k], w1, tabs[k]);
				vkhel_ctx_sync(ctx);
				const double per = (now_us() - t0) / reps;
				if (per < best)
					best = per;
			}
			printf("%s\"%s\": %.2f", i ? ", " : "", cases[i].name, best);
		}
		printf("}");
	}
	printf("}\n");
	const int err = vkhel_ctx_last_error(ctx, NULL, 0);
	vkhel_ctx_set_async(ctx, 0);
	for (int k = 0; k < 3; k++) {
		vkhel_vector_destroy(va[k]);
		vkhel_vector_destroy(vb[k]);
		vkhel_vector_destroy(vc[k]);
		vkhel_ntt_tables_destroy(tabs[k]);
	}
	vkhel_vector_destroy(w1);
	vkhel_ctx_destroy(ctx);
	return err ? 1 : 0;
}
