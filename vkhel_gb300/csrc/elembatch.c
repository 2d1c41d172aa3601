/*
 * Element-wise batch (no counterpart in the reference, whose callers issue
 * one blocking element-wise call per vector): many independent element-wise
 * jobs of ragged lengths -- each one of the reference's element-wise ops on
 * its own operands -- recorded once, committed to one device job table, and
 * run as a single kernel launch (optionally replayed from a CUDA graph).
 *
 * Every job computes exactly what the single-vector call computes: the op's
 * constants are derived here the way src/vector.c's wrappers derive them
 * (and as api.c does for the single calls), and the device applies the same
 * per-word functions.  Jobs run concurrently, so a job may not write memory
 * that another job of the batch reads or writes; commit() rejects such
 * batches.  A job may work in place (res equal to one of its operands).
 */
#include <inttypes.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "internal.h"

struct vkhel_elem_batch {
	struct vkhel_ctx *ctx;
	vkcu_elem_job *jobs;
	uint32_t njobs, cap;
	int committed;
	void *dev;              /* unit table: the jobs cut into VKCU_ELEM_CHUNK-word pieces */
	uint64_t dev_bytes;
	uint64_t chunks;
	void *graph;
};

struct vkhel_elem_batch *vkhel_elem_batch_create(struct vkhel_ctx *ctx) {
	if (!ctx) {
		vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "elem_batch_create: NULL context");
		return NULL;
	}
	struct vkhel_elem_batch *b = calloc(1, sizeof(*b));
	if (!b)
		vkh_fail(ctx, VKHEL_ERR_OUT_OF_MEMORY, "elem_batch_create: host allocation failed");
	else
		b->ctx = ctx;
	return b;
}

/* The op's device constants, derived as the single-vector calls derive them. */
static int compile_op(struct vkhel_ctx *ctx, uint32_t op, uint64_t p0, uint64_t p1, uint64_t p2, vkcu_elem_job *j) {
	int st = VKHEL_OK;
	switch (op) {
	case VKHEL_ELEM_FMA: /* elemfma.c:159-161: multiplier as given, truncated Shoup factor */
		if ((st = vkh_check_mod(ctx, "elem_batch fma", p1)))
			return st;
		*j = (vkcu_elem_job){.op = VKCU_ELEM_FMA, .c0 = p0, .c1 = vkh_shoup(p0, p1), .c2 = p1};
		return VKHEL_OK;
	case VKHEL_ELEM_FMA_CANONICAL: {
		if ((st = vkh_check_mod(ctx, "elem_batch fma_canonical", p1)))
			return st;
		const uint64_t m = p0 % p1;
		*j = (vkcu_elem_job){.op = VKCU_ELEM_FMA_CANON, .bits = (uint32_t) vkh_bitlen(p1), .c0 = m,
				.c1 = vkh_shoup(m, p1), .c2 = p1, .c3 = vkh_barrett_mu(p1)};
		return VKHEL_OK;
	}
	case VKHEL_ELEM_MUL:
		if ((st = vkh_check_mod(ctx, "elem_batch mul", p0)))
			return st;
		*j = (vkcu_elem_job){.op = VKCU_ELEM_MUL, .bits = (uint32_t) vkh_bitlen(p0), .c0 = p0,
				.c1 = vkh_barrett_mu(p0)};
		return VKHEL_OK;
	case VKHEL_ELEM_MULCONST: /* elemmulconst.c:154-163 */
		if ((st = vkh_check_mod(ctx, "elem_batch mulconst", p1)))
			return st;
		*j = (vkcu_elem_job){.op = VKCU_ELEM_MULCONST, .c0 = p0, .c1 = vkh_shoup(p0, p1), .c2 = p1};
		return VKHEL_OK;
	case VKHEL_ELEM_MOD: /* src/vector.c:360-368 */
		if (p0 == 2) {
			*j = (vkcu_elem_job){.op = VKCU_ELEM_MODTWO, .c0 = p1 / 2};
			return VKHEL_OK;
		}
		if ((st = vkh_check_mod(ctx, "elem_batch mod", p0)))
			return st;
		p2 = p0;
		p0 = p1 / 2;
		/* elemgtsub(bound = q / 2, diff = q, mod) */
		/* fall through */
	case VKHEL_ELEM_GTSUB: {
		if ((st = vkh_check_mod(ctx, "elem_batch gtsub", p2)))
			return st;
		const uint64_t mu = vkh_barrett_mu(p2);
		*j = (vkcu_elem_job){.op = VKCU_ELEM_GTSUB, .bits = (uint32_t) vkh_bitlen(p2), .c0 = p0,
				.c1 = vkh_ref_reduce64(p1, p2, mu), .c2 = p2, .c3 = mu};
		return VKHEL_OK;
	}
	case VKHEL_ELEM_GTADD:
		*j = (vkcu_elem_job){.op = VKCU_ELEM_GTADD, .c0 = p0, .c1 = p1};
		return VKHEL_OK;
	default:
		return vkh_fail(ctx, VKHEL_ERR_INVALID_ARGUMENT, "elem_batch: unknown op %u", op);
	}
}

static int is_binary(uint32_t op) {
	return op == VKHEL_ELEM_FMA || op == VKHEL_ELEM_FMA_CANONICAL || op == VKHEL_ELEM_MUL;
}

static int add_job(struct vkhel_elem_batch *b, uint32_t op, uint64_t p0, uint64_t p1, uint64_t p2, const uint64_t *a,
		const uint64_t *bb, uint64_t *res, uint64_t len) {
	struct vkhel_ctx *ctx = b->ctx;
	if (b->committed)
		return vkh_fail(ctx, VKHEL_ERR_INVALID_ARGUMENT, "elem_batch: already committed");
	if (len && (!a || !res || (is_binary(op) && !bb)))
		return vkh_fail(ctx, VKHEL_ERR_INVALID_ARGUMENT, "elem_batch_add: NULL operand");
	if (((uintptr_t) a | (uintptr_t) bb | (uintptr_t) res) & 7)
		return vkh_fail(ctx, VKHEL_ERR_INVALID_ARGUMENT, "elem_batch_add: pointers must be 8-byte aligned");
	vkcu_elem_job j;
	int st = compile_op(ctx, op, p0, p1, p2, &j);
	if (st)
		return st;
	j.a = a;
	j.b = is_binary(op) ? bb : NULL;
	j.res = res;
	j.len = len;
	if (b->njobs == b->cap) {
		const uint32_t cap = b->cap ? 2 * b->cap : 64;
		vkcu_elem_job *t = realloc(b->jobs, sizeof(*t) * cap);
		if (!t)
			return vkh_fail(ctx, VKHEL_ERR_OUT_OF_MEMORY, "elem_batch_add: host allocation failed");
		b->jobs = t;
		b->cap = cap;
	}
	b->jobs[b->njobs++] = j;
	return VKHEL_OK;
}

int vkhel_elem_batch_add(struct vkhel_elem_batch *b, uint32_t op, uint64_t p0, uint64_t p1, uint64_t p2,
		const struct vkhel_vector *a, const struct vkhel_vector *bb, struct vkhel_vector *res) {
	if (!b)
		return vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "elem_batch_add: NULL batch");
	if (!a || !res || (is_binary(op) && !bb))
		return vkh_fail(b->ctx, VKHEL_ERR_INVALID_ARGUMENT, "elem_batch_add: NULL vector");
	if (a->ctx != b->ctx || res->ctx != b->ctx || (is_binary(op) && bb->ctx != b->ctx))
		return vkh_fail(b->ctx, VKHEL_ERR_INVALID_ARGUMENT, "elem_batch_add: vectors of another context");
	/* as the single calls: result->length words of every operand */
	if (a->length < res->length || (is_binary(op) && bb->length < res->length))
		return vkh_fail(b->ctx, VKHEL_ERR_INVALID_ARGUMENT,
				"elem_batch_add: operand shorter than result (%" PRIu64 ")", res->length);
	return add_job(b, op, p0, p1, p2, a->dev, is_binary(op) ? bb->dev : NULL, res->dev, res->length);
}

int vkhel_elem_batch_add_raw(struct vkhel_elem_batch *b, uint32_t op, uint64_t p0, uint64_t p1, uint64_t p2,
		const uint64_t *a, const uint64_t *bb, uint64_t *res, uint64_t len) {
	if (!b)
		return vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "elem_batch_add: NULL batch");
	return add_job(b, op, p0, p1, p2, a, bb, res, len);
}

struct span {
	uintptr_t lo, hi;
	uint32_t job;
};

static int cmp_span(const void *x, const void *y) {
	const struct span *a = x, *b = y;
	return (a->lo > b->lo) - (a->lo < b->lo);
}

/* 0 when no job writes memory that another job reads or writes. */
static int jobs_independent(const vkcu_elem_job *jobs, uint32_t njobs, uint32_t *bad) {
	struct span *w = malloc(sizeof(*w) * (njobs ? njobs : 1));
	if (!w)
		return -1;
	uint32_t nw = 0;
	for (uint32_t i = 0; i < njobs; i++)
		if (jobs[i].len)
			w[nw++] = (struct span){(uintptr_t) jobs[i].res, (uintptr_t) (jobs[i].res + jobs[i].len), i};
	qsort(w, nw, sizeof(*w), cmp_span);
	int rc = 0;
	for (uint32_t k = 1; k < nw && !rc; k++)
		if (w[k].lo < w[k - 1].hi) {
			*bad = w[k].job;
			rc = 1;
		}
	/* writes are now disjoint and sorted: a read [lo, hi) meets another
	 * job's write iff one of the last two writes starting below hi does */
	for (uint32_t i = 0; i < njobs && !rc; i++) {
		const uint64_t *ops[2] = {jobs[i].a, jobs[i].b};
		for (int o = 0; o < 2 && !rc && jobs[i].len; o++) {
			if (!ops[o])
				continue;
			const uintptr_t lo = (uintptr_t) ops[o], hi = (uintptr_t) (ops[o] + jobs[i].len);
			uint32_t l = 0, h = nw; /* first write with lo >= hi */
			while (l < h) {
				const uint32_t m = (l + h) / 2;
				if (w[m].lo < hi)
					l = m + 1;
				else
					h = m;
			}
			for (uint32_t k = l; k > 0 && k + 2 > l && !rc; k--) {
				const struct span *s = &w[k - 1];
				if (s->job != i && s->hi > lo) {
					*bad = i;
					rc = 1;
				}
			}
		}
	}
	free(w);
	return rc;
}

int vkhel_elem_batch_commit(struct vkhel_elem_batch *b, uint32_t flags) {
	if (!b)
		return vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "elem_batch_commit: NULL batch");
	struct vkhel_ctx *ctx = b->ctx;
	if (b->committed)
		return vkh_fail(ctx, VKHEL_ERR_INVALID_ARGUMENT, "elem_batch_commit: already committed");
	if (b->njobs == 0)
		return vkh_fail(ctx, VKHEL_ERR_INVALID_ARGUMENT, "elem_batch_commit: empty batch");
	uint32_t bad = 0;
	const int dep = jobs_independent(b->jobs, b->njobs, &bad);
	if (dep < 0)
		return vkh_fail(ctx, VKHEL_ERR_OUT_OF_MEMORY, "elem_batch_commit: host allocation failed");
	if (dep)
		return vkh_fail(ctx, VKHEL_ERR_INVALID_ARGUMENT,
				"elem_batch_commit: job %u overlaps memory another job writes", bad);
	/* what a commit that failed part-way left behind (retried commit) */
	vkcu_graph_destroy(b->graph);
	b->graph = NULL;
	vkh_dev_free(ctx, b->dev, b->dev_bytes);
	b->dev = NULL;
	b->dev_bytes = 0;
	uint64_t chunks = 0;
	for (uint32_t i = 0; i < b->njobs; i++) {
		const uint64_t unit = b->jobs[i].b ? VKCU_ELEM_CHUNK : VKCU_ELEM_CHUNK_UNARY;
		chunks += (b->jobs[i].len + unit - 1) / unit;
	}
	const uint64_t dev_bytes = sizeof(vkcu_elem_job) * (chunks ? chunks : 1);
	vkcu_elem_job *host = malloc(dev_bytes);
	if (!host)
		return vkh_fail(ctx, VKHEL_ERR_OUT_OF_MEMORY, "elem_batch_commit: host allocation failed");
	uint64_t k = 0;
	for (uint32_t i = 0; i < b->njobs; i++) {
		const vkcu_elem_job *j = &b->jobs[i];
		const uint64_t unit = j->b ? VKCU_ELEM_CHUNK : VKCU_ELEM_CHUNK_UNARY;
		for (uint64_t w = 0; w < j->len; w += unit) {
			vkcu_elem_job u = *j;
			u.a = j->a + w;
			u.b = j->b ? j->b + w : NULL;
			u.res = j->res + w;
			u.len = j->len - w < unit ? j->len - w : unit;
			host[k++] = u;
		}
	}
	b->chunks = chunks;
	int st = vkh_dev_alloc(ctx, dev_bytes, &b->dev);
	if (st) {
		free(host);
		return st;
	}
	b->dev_bytes = dev_bytes;
	int e = vkcu_h2d(ctx->stream, b->dev, host, b->dev_bytes);
	if (!e)
		e = vkcu_sync(ctx->stream);
	free(host);
	if (e)
		return vkh_cuda(ctx, e, "elem_batch_commit: unit table upload");
	if ((flags & VKHEL_BATCH_GRAPH) && b->chunks) {
		e = vkcu_capture_begin(ctx->stream);
		if (!e) {
			const int ie = vkcu_elem_batch(ctx->stream, b->dev, b->chunks, ctx->sms);
			void *exec = NULL;
			e = vkcu_capture_end(ctx->stream, &exec);
			if (!e)
				e = ie;
			b->graph = exec;
			if (!ie)
				vkcu_count_launches((uint64_t) 0 - 1); /* capture executes nothing */
		}
		if (e)
			return vkh_cuda(ctx, e, "elem_batch_commit: capture");
	}
	b->committed = 1;
	return VKHEL_OK;
}

int vkhel_elem_batch_launch(struct vkhel_elem_batch *b) {
	if (!b || !b->committed)
		return vkh_fail(b ? b->ctx : NULL, VKHEL_ERR_INVALID_ARGUMENT, "elem_batch_launch: not committed");
	vkcu_range_push("vkhel_elem_batch_launch");
	int e = 0;
	if (b->graph) {
		e = vkcu_graph_launch(b->graph, b->ctx->stream);
		if (!e)
			vkcu_count_launches(1);
	} else if (b->chunks) {
		e = vkcu_elem_batch(b->ctx->stream, b->dev, b->chunks, b->ctx->sms);
	}
	vkcu_range_pop();
	return vkh_cuda(b->ctx, e, "elem_batch_launch");
}

int vkhel_elem_batch_run(struct vkhel_elem_batch *b) {
	const int st = vkhel_elem_batch_launch(b);
	if (st)
		return st;
	return vkh_cuda(b->ctx, vkcu_sync(b->ctx->stream), "elem_batch_run");
}

uint32_t vkhel_elem_batch_jobs(const struct vkhel_elem_batch *b) { return b ? b->njobs : 0; }

void vkhel_elem_batch_destroy(struct vkhel_elem_batch *b) {
	if (!b)
		return;
	vkcu_sync(b->ctx->stream);
	vkcu_graph_destroy(b->graph);
	vkh_dev_free(b->ctx, b->dev, b->dev_bytes);
	free(b->jobs);
	free(b);
}
