/*
 * Batched polynomial multiply (no counterpart in the reference, whose callers
 * compose forward(a), forward(b), elemmul, inverse one blocking call at a
 * time: 3 log2(n) + 2 submits per limb product).
 *
 * A batch records limb jobs, then commit():
 *   - sorts the jobs by degree into classes and uploads one device job table;
 *   - gives every job that needs it an n-word scratch slice (NTT(b) parking
 *     when c aliases a, or the composed path for n outside the fused range);
 *   - optionally captures the class launches into a CUDA graph (one fused
 *     persistent kernel per class for 256 <= n <= 16384; forward, forward,
 *     pointwise, inverse kernels over the whole class otherwise).
 * launch() replays the graph (or re-issues the launches) on the context
 * stream without waiting.
 */
#include <stdlib.h>
#include <string.h>

#include "internal.h"

#define MAX_CLASSES 64

struct job_rec {
	uint32_t kind;         /* VKH_JOB_* */
	uint32_t log_n;
	uint32_t needs_scratch;
	uint32_t lift;         /* index into the batch's lift table, 0 = none */
	uint32_t wide;         /* modulus class: 2^62 <= q < 2^63 */
	uint32_t b_ntt;        /* b holds NTT(b) (VKCU_JOB_B_NTT) */
	uint32_t order;        /* insertion order, keeps the sort stable */
	vkcu_poly_job job;
};

struct vkhel_batch {
	struct vkhel_ctx *ctx;
	struct job_rec *recs;
	uint32_t njobs, cap;
	int committed;
	vkcu_lift *lifts;      /* [0] unused (no epilogue) */
	uint32_t nlifts;
	uint32_t flags;
	struct vkh_job_class classes[MAX_CLASSES];
	uint32_t nclasses;
	void *dev;             /* poly jobs, then 3 ntt-job arrays per composed class */
	uint64_t dev_bytes;
	void *scratch;
	uint64_t scratch_bytes;
	vkcu_poly_job *dev_poly;
	vkcu_ntt_job *dev_ntt; /* [3 * njobs]: b->scratch, a->c, c->c */
	void *graph;
	uint32_t kernels;
	/* a ragged batch as one launch (tuning family 3, log_n 2): item table,
	 * job copies (plus a dummy copy for an odd pair), two counters and the
	 * dummy products' output, in one device allocation */
	int ragged;
	uint32_t n_cluster_items, n_items;
	void *ragged_dev;
	uint64_t ragged_bytes;
	/* concurrent degree classes: one stream and one join event per class
	 * after the first, one fork event */
	uint32_t naux;
	void *aux[MAX_CLASSES];
	void *join[MAX_CLASSES];
	void *fork;
};

struct vkhel_batch *vkhel_batch_create(struct vkhel_ctx *ctx) {
	if (!ctx) {
		vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "batch_create: NULL context");
		return NULL;
	}
	struct vkhel_batch *b = calloc(1, sizeof(*b));
	if (!b)
		vkh_fail(ctx, VKHEL_ERR_OUT_OF_MEMORY, "batch_create: host allocation failed");
	else
		b->ctx = ctx;
	return b;
}

/* Index of `l` in the batch's lift table (added when new); 0 for none. */
static int lift_index(struct vkhel_batch *b, const vkcu_lift *l, uint32_t *idx) {
	*idx = 0;
	if (!l || l->count == 0)
		return VKHEL_OK;
	for (uint32_t i = 1; i < b->nlifts; i++) {
		if (!memcmp(&b->lifts[i], l, sizeof *l)) {
			*idx = i;
			return VKHEL_OK;
		}
	}
	const uint32_t n = b->nlifts ? b->nlifts : 1;
	vkcu_lift *t = realloc(b->lifts, sizeof(*t) * (n + 1));
	if (!t)
		return vkh_fail(b->ctx, VKHEL_ERR_OUT_OF_MEMORY, "batch_add: host allocation failed");
	memset(&t[0], 0, sizeof t[0]);
	t[n] = *l;
	b->lifts = t;
	b->nlifts = n + 1;
	*idx = n;
	return VKHEL_OK;
}

/* Limb jobs of one call: a polymul (a, bb -> c; bb holding NTT(b) when
 * b_ntt) or a transform (a -> c, bb unused). */
static int add_jobs(struct vkhel_batch *b, struct vkhel_ntt_tables *const *tables, uint32_t limbs,
		const uint64_t *a, const uint64_t *bb, uint64_t *c, const vkcu_lift *lift, uint32_t kind, int b_ntt) {
	struct vkhel_ctx *ctx = b->ctx;
	if (b->committed)
		return vkh_fail(ctx, VKHEL_ERR_INVALID_ARGUMENT, "batch: already committed");
	if (!tables || limbs == 0 || !a || (kind == VKH_JOB_POLYMUL && !bb) || !c)
		return vkh_fail(ctx, VKHEL_ERR_INVALID_ARGUMENT, "batch_add: bad arguments");
	if (((uintptr_t) a | (uintptr_t) bb | (uintptr_t) c) & 31)
		return vkh_fail(ctx, VKHEL_ERR_INVALID_ARGUMENT, "batch_add: pointers must be 32-byte aligned");
	const uint64_t n = tables[0] ? tables[0]->n : 0;
	/* the composed path (n outside the fused range) writes c before it reads NTT(b) */
	if (b_ntt && bb < c + (uint64_t) limbs * n && c < bb + (uint64_t) limbs * n)
		return vkh_fail(ctx, VKHEL_ERR_INVALID_ARGUMENT, "batch_add: c overlaps NTT(b)");
	for (uint32_t k = 0; k < limbs; k++) {
		const struct vkhel_ntt_tables *t = tables[k];
		if (!t || t->n != n || n < 2)
			return vkh_fail(ctx, VKHEL_ERR_INVALID_ARGUMENT, "batch_add: limb %u tables invalid", k);
		if (t->q >= ((uint64_t) 1 << 63) || t->q < 3 || t->unreduced || t->log_n > vkcu_max_log_n())
			return vkh_fail(ctx, VKHEL_ERR_UNSUPPORTED, "batch_add: limb %u (n, q) unsupported", k);
	}
	uint32_t lift_id = 0;
	const int lst = lift_index(b, lift, &lift_id);
	if (lst)
		return lst;
	if (b->njobs + limbs > b->cap) {
		uint32_t cap = b->cap ? b->cap : 64;
		while (cap < b->njobs + limbs)
			cap *= 2;
		struct job_rec *r = realloc(b->recs, sizeof(*r) * cap);
		if (!r)
			return vkh_fail(ctx, VKHEL_ERR_OUT_OF_MEMORY, "batch_add: host allocation failed");
		b->recs = r;
		b->cap = cap;
	}
	/* every limb's tables resident before any job is recorded, so a failed
	 * add leaves the batch as it was (the lookups below are then hits) */
	for (uint32_t k = 0; k < limbs; k++) {
		const struct vkh_devtab *d = NULL;
		const int st = vkh_devtab_get(ctx, tables[k], &d);
		if (st)
			return st;
	}
	for (uint32_t k = 0; k < limbs; k++) {
		const struct vkh_devtab *d = NULL;
		const int st = vkh_devtab_get(ctx, tables[k], &d);
		if (st)
			return st;
		struct job_rec *r = &b->recs[b->njobs++];
		const uint32_t log_n = tables[k]->log_n;
		const int fused = log_n >= 8 && log_n <= vkcu_max_fused_log_n();
		const uint64_t *ak = a + (uint64_t) k * n, *bk = bb ? bb + (uint64_t) k * n : NULL;
		uint64_t *ck = c + (uint64_t) k * n;
		/* the fused kernel parks NTT(b) in c, which must not hold a */
		const int overlap = ak < ck + n && ck < ak + n;
		r->kind = kind;
		r->log_n = log_n;
		r->needs_scratch = kind == VKH_JOB_POLYMUL && !b_ntt && (!fused || overlap);
		r->lift = lift_id;
		r->wide = (uint32_t) vkcu_wide(tables[k]->q);
		r->b_ntt = (uint32_t) (b_ntt != 0);
		r->order = b->njobs - 1;
		r->job.a = ak;
		r->job.b = kind == VKH_JOB_POLYMUL ? bk : NULL;
		r->job.c = ck;
		/* NTT(b) given: the composed path's pointwise step reads it as the scratch */
		r->job.scratch = b_ntt ? (uint64_t *) bk : ck;
		r->job.tw = d->dev_set;
		r->job.flags = b_ntt ? VKCU_JOB_B_NTT : 0;
	}
	return VKHEL_OK;
}

int vkhel_batch_add_polymul(struct vkhel_batch *b, struct vkhel_ntt_tables *const *tables, uint32_t limbs,
		const struct vkhel_vector *a, const struct vkhel_vector *bb, struct vkhel_vector *c) {
	if (!b)
		return vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "batch_add: NULL batch");
	if (!a || !bb || !c || !tables || !tables[0])
		return vkh_fail(b->ctx, VKHEL_ERR_INVALID_ARGUMENT, "batch_add: NULL argument");
	if (a->ctx != b->ctx || bb->ctx != b->ctx || c->ctx != b->ctx)
		return vkh_fail(b->ctx, VKHEL_ERR_INVALID_ARGUMENT, "batch_add: vectors of another context");
	const uint64_t need = (uint64_t) limbs * tables[0]->n;
	if (a->length < need || bb->length < need || c->length < need)
		return vkh_fail(b->ctx, VKHEL_ERR_INVALID_ARGUMENT, "batch_add: vectors shorter than limbs * n");
	return add_jobs(b, tables, limbs, a->dev, bb->dev, c->dev, NULL, VKH_JOB_POLYMUL, 0);
}

int vkhel_batch_add_polymul_ntt(struct vkhel_batch *b, struct vkhel_ntt_tables *const *tables, uint32_t limbs,
		const struct vkhel_vector *a, const struct vkhel_vector *b_ntt, struct vkhel_vector *c) {
	if (!b)
		return vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "batch_add: NULL batch");
	if (!a || !b_ntt || !c || !tables || !tables[0])
		return vkh_fail(b->ctx, VKHEL_ERR_INVALID_ARGUMENT, "batch_add: NULL argument");
	if (a->ctx != b->ctx || b_ntt->ctx != b->ctx || c->ctx != b->ctx)
		return vkh_fail(b->ctx, VKHEL_ERR_INVALID_ARGUMENT, "batch_add: vectors of another context");
	const uint64_t need = (uint64_t) limbs * tables[0]->n;
	if (a->length < need || b_ntt->length < need || c->length < need)
		return vkh_fail(b->ctx, VKHEL_ERR_INVALID_ARGUMENT, "batch_add: vectors shorter than limbs * n");
	return add_jobs(b, tables, limbs, a->dev, b_ntt->dev, c->dev, NULL, VKH_JOB_POLYMUL, 1);
}

int vkhel_batch_add_polymul_ntt_raw(struct vkhel_batch *b, struct vkhel_ntt_tables *const *tables, uint32_t limbs,
		const uint64_t *a, const uint64_t *b_ntt, uint64_t *c) {
	if (!b)
		return vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "batch_add: NULL batch");
	return add_jobs(b, tables, limbs, a, b_ntt, c, NULL, VKH_JOB_POLYMUL, 1);
}

int vkhel_batch_add_polymul_lift(struct vkhel_batch *b, struct vkhel_ntt_tables *const *tables, uint32_t limbs,
		const struct vkhel_vector *a, const struct vkhel_vector *bb, struct vkhel_vector *c,
		const struct vkhel_lift_step *steps, uint32_t nsteps) {
	if (!b)
		return vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "batch_add: NULL batch");
	if (!a || !bb || !c || !tables || !tables[0])
		return vkh_fail(b->ctx, VKHEL_ERR_INVALID_ARGUMENT, "batch_add: NULL argument");
	if (a->ctx != b->ctx || bb->ctx != b->ctx || c->ctx != b->ctx)
		return vkh_fail(b->ctx, VKHEL_ERR_INVALID_ARGUMENT, "batch_add: vectors of another context");
	const uint64_t need = (uint64_t) limbs * tables[0]->n;
	if (a->length < need || bb->length < need || c->length < need)
		return vkh_fail(b->ctx, VKHEL_ERR_INVALID_ARGUMENT, "batch_add: vectors shorter than limbs * n");
	/* ELEMMOD with q = 0 resolves each limb's modulus on the device */
	vkcu_lift lift;
	const int st = vkh_lift_compile(b->ctx, steps, nsteps, 0, &lift);
	if (st)
		return st;
	return add_jobs(b, tables, limbs, a->dev, bb->dev, c->dev, &lift, VKH_JOB_POLYMUL, 0);
}

int vkhel_batch_add_transform(struct vkhel_batch *b, struct vkhel_ntt_tables *const *tables, uint32_t limbs,
		const struct vkhel_vector *in, struct vkhel_vector *out, uint32_t direction,
		const struct vkhel_lift_step *steps, uint32_t nsteps) {
	if (!b)
		return vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "batch_add_transform: NULL batch");
	if (!in || !out || !tables || !tables[0])
		return vkh_fail(b->ctx, VKHEL_ERR_INVALID_ARGUMENT, "batch_add_transform: NULL argument");
	if (in->ctx != b->ctx || out->ctx != b->ctx)
		return vkh_fail(b->ctx, VKHEL_ERR_INVALID_ARGUMENT, "batch_add_transform: vectors of another context");
	if (direction != VKHEL_TRANSFORM_FORWARD && direction != VKHEL_TRANSFORM_INVERSE)
		return vkh_fail(b->ctx, VKHEL_ERR_INVALID_ARGUMENT, "batch_add_transform: unknown direction %u", direction);
	if (nsteps && direction != VKHEL_TRANSFORM_INVERSE)
		return vkh_fail(b->ctx, VKHEL_ERR_INVALID_ARGUMENT, "batch_add_transform: an epilogue needs the inverse");
	const uint64_t need = (uint64_t) limbs * tables[0]->n;
	if (in->length < need || out->length < need)
		return vkh_fail(b->ctx, VKHEL_ERR_INVALID_ARGUMENT, "batch_add_transform: vectors shorter than limbs * n");
	vkcu_lift lift;
	const int st = vkh_lift_compile(b->ctx, steps, nsteps, 0, &lift);
	if (st)
		return st;
	return add_jobs(b, tables, limbs, in->dev, NULL, out->dev, &lift,
			direction == VKHEL_TRANSFORM_FORWARD ? VKH_JOB_FORWARD : VKH_JOB_INVERSE, 0);
}

int vkhel_batch_add_polymul_raw(struct vkhel_batch *b, struct vkhel_ntt_tables *const *tables, uint32_t limbs,
		const uint64_t *a, const uint64_t *bb, uint64_t *c) {
	if (!b)
		return vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "batch_add: NULL batch");
	return add_jobs(b, tables, limbs, a, bb, c, NULL, VKH_JOB_POLYMUL, 0);
}

/* Words of one job's scratch slice: n rounded up to 32 words (256 bytes). */
static uint64_t slice_words(uint32_t log_n) { return (((uint64_t) 1 << log_n) + 31) & ~(uint64_t) 31; }

static int cmp_rec(const void *x, const void *y) {
	const struct job_rec *a = x, *b = y;
	if (a->kind != b->kind)
		return (a->kind > b->kind) - (a->kind < b->kind);
	if (a->log_n != b->log_n)
		return (a->log_n > b->log_n) - (a->log_n < b->log_n);
	if (a->wide != b->wide)
		return (a->wide > b->wide) - (a->wide < b->wide);
	if (a->lift != b->lift)
		return (a->lift > b->lift) - (a->lift < b->lift);
	if (a->b_ntt != b->b_ntt)
		return (a->b_ntt > b->b_ntt) - (a->b_ntt < b->b_ntt);
	return (a->order > b->order) - (a->order < b->order);
}

/* Launch the kernels of `nclasses` degree classes on `stream`: one fused
 * polymul launch per class with 2^8 <= n <= 2^17, otherwise forward(b ->
 * scratch), forward(a -> c), pointwise, inverse(c) over the class's slice of
 * the ntt-job array (laid out at 3 * first: b jobs, a jobs, c jobs).  A
 * class's epilogue rides on its last launch. */
int vkh_issue_classes(void *stream, int sms, const vkcu_poly_job *dev_poly, const vkcu_ntt_job *dev_ntt,
		const struct vkh_job_class *classes, uint32_t nclasses, const vkcu_lift *lifts) {
	for (uint32_t k = 0; k < nclasses; k++) {
		const struct vkh_job_class *cl = &classes[k];
		const vkcu_lift *lift = lifts && cl->lift ? &lifts[cl->lift] : NULL;
		const vkcu_ntt_job *tj = dev_ntt + 3 * (size_t) cl->first;
		int e;
		if (cl->kind == VKH_JOB_FORWARD) {
			e = vkcu_ntt_forward(stream, tj, (int) cl->count, NULL, cl->log_n, cl->wide, sms);
		} else if (cl->kind == VKH_JOB_INVERSE) {
			e = vkcu_ntt_inverse_lift(stream, tj, (int) cl->count, NULL, cl->log_n, cl->wide, sms, lift);
		} else if (cl->fused) {
			e = vkcu_polymul_lift(stream, dev_poly + cl->first, (int) cl->count, NULL, cl->log_n, cl->wide, sms,
					lift, (int) cl->b_ntt);
		} else {
			const vkcu_ntt_job *nj = dev_ntt + 3 * (size_t) cl->first;
			e = cl->b_ntt ? 0 : vkcu_ntt_forward(stream, nj, (int) cl->count, NULL, cl->log_n, cl->wide, sms);
			if (!e)
				e = vkcu_ntt_forward(stream, nj + cl->count, (int) cl->count, NULL, cl->log_n, cl->wide, sms);
			if (!e)
				e = vkcu_pointwise(stream, dev_poly + cl->first, (int) cl->count, cl->log_n, cl->wide, sms);
			if (!e)
				e = vkcu_ntt_inverse_lift(stream, nj + 2 * (size_t) cl->count, (int) cl->count, NULL, cl->log_n,
						cl->wide, sms, lift);
		}
		if (e)
			return e;
	}
	return 0;
}

/* Fill the ntt-job arrays from the recorded jobs: three per job of a composed
 * polymul class, one per job of a transform class. */
void vkh_fill_ntt_jobs(const vkcu_poly_job *poly, vkcu_ntt_job *ntt, const struct vkh_job_class *classes,
		uint32_t nclasses) {
	for (uint32_t k = 0; k < nclasses; k++) {
		const struct vkh_job_class *cl = &classes[k];
		vkcu_ntt_job *nj = ntt + 3 * (size_t) cl->first;
		if (cl->kind != VKH_JOB_POLYMUL) { /* one transform job each: in -> out */
			for (uint32_t i = 0; i < cl->count; i++) {
				const vkcu_poly_job *j = &poly[cl->first + i];
				nj[i] = (vkcu_ntt_job){j->a, j->c, j->tw};
			}
			continue;
		}
		if (cl->fused)
			continue;
		for (uint32_t i = 0; i < cl->count; i++) {
			const vkcu_poly_job *j = &poly[cl->first + i];
			nj[i] = (vkcu_ntt_job){j->b, j->scratch, j->tw};
			nj[cl->count + i] = (vkcu_ntt_job){j->a, j->c, j->tw};
			nj[2 * cl->count + i] = (vkcu_ntt_job){j->c, j->c, j->tw};
		}
	}
}

/* Same, with class k > 0 on aux[k - 1]: the auxiliary streams wait for
 * `fork` recorded on `stream`, and `stream` waits for each join[k - 1], so
 * the classes run concurrently and the whole still ends on `stream` (this is
 * also how a CUDA graph capture picks up the parallel branches). */
int vkh_issue_classes_forked(void *stream, void *const *aux, void *fork, void *const *join, int sms,
		const vkcu_poly_job *dev_poly, const vkcu_ntt_job *dev_ntt, const struct vkh_job_class *classes,
		uint32_t nclasses, const vkcu_lift *lifts) {
	if (nclasses < 2)
		return vkh_issue_classes(stream, sms, dev_poly, dev_ntt, classes, nclasses, lifts);
	int e = vkcu_event_record(fork, stream);
	for (uint32_t k = 1; !e && k < nclasses; k++)
		e = vkcu_stream_wait(aux[k - 1], fork);
	for (uint32_t k = 0; !e && k < nclasses; k++)
		e = vkh_issue_classes(k ? aux[k - 1] : stream, sms, dev_poly, dev_ntt, &classes[k], 1, lifts);
	for (uint32_t k = 1; !e && k < nclasses; k++) {
		e = vkcu_event_record(join[k - 1], aux[k - 1]);
		if (!e)
			e = vkcu_stream_wait(stream, join[k - 1]);
	}
	return e;
}

static int issue(struct vkhel_batch *b) {
	if (b->ragged) {
		const char *base = b->ragged_dev;
		const uint64_t items_bytes = (sizeof(vkcu_ragged_item) * b->n_items + 255) & ~(uint64_t) 255;
		const uint64_t jobs_bytes = (sizeof(vkcu_poly_job) * (b->njobs + 2) + 255) & ~(uint64_t) 255;
		return vkcu_polymul_ragged(b->ctx->stream, (const vkcu_ragged_item *) base, (int) b->n_cluster_items,
				(int) b->n_items, (const vkcu_poly_job *) (base + items_bytes),
				(unsigned *) (base + items_bytes + jobs_bytes), b->ctx->sms);
	}
	if (b->naux)
		return vkh_issue_classes_forked(b->ctx->stream, b->aux, b->fork, b->join, b->ctx->sms, b->dev_poly,
				b->dev_ntt, b->classes, b->nclasses, b->lifts);
	return vkh_issue_classes(b->ctx->stream, b->ctx->sms, b->dev_poly, b->dev_ntt, b->classes, b->nclasses,
			b->lifts);
}

/* The single-launch form of a ragged batch (ntt_ragged.cu) when the tuning
 * table asks for it and every class is a fused product of degree 2^12 ..
 * 2^16 with q < 2^62 and no epilogue: items in decreasing size, 2^15 and
 * 2^12 products in pairs, an odd pair completed by a copy of its product
 * that writes a dummy buffer. */
static int ragged_setup(struct vkhel_batch *b) {
	b->ragged = 0;
	if (b->ragged_dev) { /* a commit that failed after this step is being retried */
		vkh_dev_free(b->ctx, b->ragged_dev, b->ragged_bytes);
		b->ragged_dev = NULL;
		b->ragged_bytes = 0;
	}
	if (b->nclasses < 2 || vkh_variant(3, 2) != 1)
		return VKHEL_OK;
	uint32_t first[17] = {0}, count[17] = {0};
	for (uint32_t k = 0; k < b->nclasses; k++) {
		const struct vkh_job_class *cl = &b->classes[k];
		if (cl->kind != VKH_JOB_POLYMUL || !cl->fused || cl->wide || cl->lift || cl->b_ntt || cl->log_n < 12 ||
				cl->log_n > 16 || count[cl->log_n])
			return VKHEL_OK;
		first[cl->log_n] = cl->first;
		count[cl->log_n] = cl->count;
	}
	const uint32_t dummy15 = b->njobs, dummy12 = b->njobs + 1; /* job indices of the dummy copies */
	const uint32_t n_cluster = count[16] + (count[15] + 1) / 2;
	const uint32_t n_items = n_cluster + count[14] + count[13] + (count[12] + 1) / 2;
	const uint64_t items_bytes = (sizeof(vkcu_ragged_item) * n_items + 255) & ~(uint64_t) 255;
	const uint64_t jobs_bytes = (sizeof(vkcu_poly_job) * (b->njobs + 2) + 255) & ~(uint64_t) 255;
	const uint64_t dummy_off = items_bytes + jobs_bytes + 256;
	const uint64_t bytes = dummy_off + sizeof(uint64_t) * (((uint64_t) 1 << 15) + ((uint64_t) 1 << 12));
	char *host = calloc(1, dummy_off);
	if (!host)
		return vkh_fail(b->ctx, VKHEL_ERR_OUT_OF_MEMORY, "batch_commit: host allocation failed");
	int st = vkh_dev_alloc(b->ctx, bytes, &b->ragged_dev);
	if (st) {
		free(host);
		return st;
	}
	b->ragged_bytes = bytes;
	vkcu_ragged_item *items = (vkcu_ragged_item *) host;
	vkcu_poly_job *jobs = (vkcu_poly_job *) (host + items_bytes);
	uint64_t *dummy = (uint64_t *) ((char *) b->ragged_dev + dummy_off);
	for (uint32_t i = 0; i < b->njobs; i++)
		jobs[i] = b->recs[i].job;
	uint32_t m = 0;
	for (uint32_t i = 0; i < count[16]; i++)
		items[m++] = (vkcu_ragged_item){16, first[16] + i, 0};
	for (uint32_t i = 0; i < count[15]; i += 2) {
		const uint32_t j = first[15] + i;
		uint32_t j1 = j + 1;
		if (i + 1 == count[15]) { /* odd: the second pair runs a copy into the dummy buffer */
			jobs[dummy15] = jobs[j];
			jobs[dummy15].c = jobs[dummy15].scratch = dummy;
			j1 = dummy15;
		}
		items[m++] = (vkcu_ragged_item){15, j, j1};
	}
	for (uint32_t i = 0; i < count[14]; i++)
		items[m++] = (vkcu_ragged_item){14, first[14] + i, 0};
	for (uint32_t i = 0; i < count[13]; i++)
		items[m++] = (vkcu_ragged_item){13, first[13] + i, 0};
	for (uint32_t i = 0; i < count[12]; i += 2) {
		const uint32_t j = first[12] + i;
		uint32_t j1 = j + 1;
		if (i + 1 == count[12]) {
			jobs[dummy12] = jobs[j];
			jobs[dummy12].c = jobs[dummy12].scratch = dummy + ((uint64_t) 1 << 15);
			j1 = dummy12;
		}
		items[m++] = (vkcu_ragged_item){12, j, j1};
	}
	int e = vkcu_h2d(b->ctx->stream, b->ragged_dev, host, items_bytes + jobs_bytes);
	if (!e)
		e = vkcu_sync(b->ctx->stream);
	free(host);
	if (e)
		return vkh_cuda(b->ctx, e, "batch_commit: ragged item table upload");
	b->n_cluster_items = n_cluster;
	b->n_items = n_items;
	b->ragged = 1;
	return VKHEL_OK;
}

int vkhel_batch_commit(struct vkhel_batch *b, uint32_t flags) {
	if (!b)
		return vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "batch_commit: NULL batch");
	struct vkhel_ctx *ctx = b->ctx;
	if (b->committed)
		return vkh_fail(ctx, VKHEL_ERR_INVALID_ARGUMENT, "batch_commit: already committed");
	if (b->njobs == 0)
		return vkh_fail(ctx, VKHEL_ERR_INVALID_ARGUMENT, "batch_commit: empty batch");
	/* what a commit that failed part-way left behind (retried commit) */
	vkcu_graph_destroy(b->graph);
	b->graph = NULL;
	for (uint32_t k = 0; k < b->naux; k++) {
		vkcu_stream_destroy(b->aux[k]);
		vkcu_event_destroy(b->join[k]);
	}
	b->naux = 0;
	vkcu_event_destroy(b->fork);
	b->fork = NULL;
	vkh_dev_free(ctx, b->dev, b->dev_bytes);
	vkh_dev_free(ctx, b->scratch, b->scratch_bytes);
	b->dev = b->scratch = NULL;
	b->dev_bytes = b->scratch_bytes = 0;
	qsort(b->recs, b->njobs, sizeof(*b->recs), cmp_rec);

	/* classes and scratch slices; every slice starts on a 256-byte boundary:
	 * the kernels of n >= 2^8 move 16 consecutive words with 32-byte vector
	 * accesses, and slices of n = 1 or 2 words would shift the ones after them */
	uint64_t scratch_words = 0;
	b->nclasses = 0;
	for (uint32_t i = 0; i < b->njobs; i++) {
		struct job_rec *r = &b->recs[i];
		if (b->nclasses == 0 || b->classes[b->nclasses - 1].kind != r->kind ||
				b->classes[b->nclasses - 1].log_n != r->log_n || b->classes[b->nclasses - 1].wide != (int) r->wide ||
				b->classes[b->nclasses - 1].lift != r->lift || b->classes[b->nclasses - 1].b_ntt != r->b_ntt) {
			if (b->nclasses == MAX_CLASSES)
				return vkh_fail(ctx, VKHEL_ERR_UNSUPPORTED, "batch_commit: too many degree classes");
			struct vkh_job_class *cl = &b->classes[b->nclasses++];
			cl->kind = r->kind;
			cl->log_n = r->log_n;
			cl->wide = (int) r->wide;
			cl->lift = r->lift;
			cl->b_ntt = r->b_ntt;
			cl->first = i;
			cl->count = 0;
			cl->fused = r->log_n >= 8 && r->log_n <= vkcu_max_fused_log_n();
		}
		b->classes[b->nclasses - 1].count++;
		if (r->needs_scratch)
			scratch_words += slice_words(r->log_n);
	}
	if (scratch_words) {
		b->scratch_bytes = scratch_words * sizeof(uint64_t);
		int st = vkh_dev_alloc(ctx, b->scratch_bytes, &b->scratch);
		if (st)
			return st;
		uint64_t off = 0;
		for (uint32_t i = 0; i < b->njobs; i++) {
			struct job_rec *r = &b->recs[i];
			if (r->needs_scratch) {
				r->job.scratch = (uint64_t *) b->scratch + off;
				off += slice_words(r->log_n);
			}
		}
	}

	/* device job table: poly jobs, then per composed class 3 ntt-job arrays
	 * laid out at 3 * first (so every class indexes its own slice) */
	const uint64_t poly_bytes = sizeof(vkcu_poly_job) * b->njobs;
	const uint64_t ntt_off = (poly_bytes + 255) & ~(uint64_t) 255;
	b->dev_bytes = ntt_off + sizeof(vkcu_ntt_job) * 3 * (uint64_t) b->njobs;
	void *host = calloc(1, b->dev_bytes);
	if (!host)
		return vkh_fail(ctx, VKHEL_ERR_OUT_OF_MEMORY, "batch_commit: host allocation failed");
	vkcu_poly_job *hp = host;
	vkcu_ntt_job *hn = (vkcu_ntt_job *) ((char *) host + ntt_off);
	for (uint32_t i = 0; i < b->njobs; i++)
		hp[i] = b->recs[i].job;
	vkh_fill_ntt_jobs(hp, hn, b->classes, b->nclasses);
	int st = vkh_dev_alloc(ctx, b->dev_bytes, &b->dev);
	if (st) {
		free(host);
		return st;
	}
	int e = vkcu_h2d(ctx->stream, b->dev, host, b->dev_bytes);
	if (!e)
		e = vkcu_sync(ctx->stream);
	free(host);
	if (e)
		return vkh_cuda(ctx, e, "batch_commit: job table upload");
	b->dev_poly = b->dev;
	b->dev_ntt = (vkcu_ntt_job *) ((char *) b->dev + ntt_off);

	if ((st = ragged_setup(b)))
		return st;
	if (!b->ragged && b->nclasses > 1 && vkh_variant(3, 0) == 1) {
		e = vkcu_event_create(&b->fork);
		for (uint32_t k = 0; !e && k + 1 < b->nclasses; k++) {
			e = vkcu_stream_create(&b->aux[k]);
			if (!e)
				e = vkcu_event_create(&b->join[k]);
			if (!e)
				b->naux = k + 1;
		}
		if (e)
			return vkh_cuda(ctx, e, "batch_commit: class streams");
	}
	const uint64_t before = vkcu_launch_count();
	if (flags & VKHEL_BATCH_GRAPH) {
		e = vkcu_capture_begin(ctx->stream);
		if (!e) {
			const int ie = issue(b);
			void *exec = NULL;
			e = vkcu_capture_end(ctx->stream, &exec);
			if (!e)
				e = ie;
			b->graph = exec;
		}
	}
	/* eager batches run nothing here (a job may work in place, so a trial run
	 * would change its data); their first launch counts the kernels */
	b->kernels = (uint32_t) (vkcu_launch_count() - before);
	if (flags & VKHEL_BATCH_GRAPH)
		vkcu_count_launches((uint64_t) 0 - b->kernels); /* capture executes nothing */
	if (e)
		return vkh_cuda(ctx, e, "batch_commit: launch");
	b->flags = flags;
	b->committed = 1;
	return VKHEL_OK;
}

int vkhel_batch_launch(struct vkhel_batch *b) {
	if (!b || !b->committed)
		return vkh_fail(b ? b->ctx : NULL, VKHEL_ERR_INVALID_ARGUMENT, "batch_launch: not committed");
	vkcu_range_push("vkhel_batch_launch");
	int e;
	if (b->graph) {
		e = vkcu_graph_launch(b->graph, b->ctx->stream);
		if (!e)
			vkcu_count_launches(b->kernels);
	} else {
		const uint64_t before = vkcu_launch_count();
		e = issue(b);
		if (!e && !b->kernels)
			b->kernels = (uint32_t) (vkcu_launch_count() - before);
	}
	vkcu_range_pop();
	return vkh_cuda(b->ctx, e, "batch_launch");
}

int vkhel_batch_run(struct vkhel_batch *b) {
	int st = vkhel_batch_launch(b);
	if (st)
		return st;
	return vkh_cuda(b->ctx, vkcu_sync(b->ctx->stream), "batch_run");
}

uint32_t vkhel_batch_jobs(const struct vkhel_batch *b) { return b ? b->njobs : 0; }
uint32_t vkhel_batch_kernels(const struct vkhel_batch *b) { return b ? b->kernels : 0; }

void vkhel_batch_destroy(struct vkhel_batch *b) {
	if (!b)
		return;
	struct vkhel_ctx *ctx = b->ctx;
	vkcu_sync(ctx->stream);
	vkcu_graph_destroy(b->graph);
	for (uint32_t k = 0; k < b->naux; k++) {
		vkcu_stream_destroy(b->aux[k]);
		vkcu_event_destroy(b->join[k]);
	}
	vkcu_event_destroy(b->fork);
	vkh_dev_free(ctx, b->dev, b->dev_bytes);
	vkh_dev_free(ctx, b->scratch, b->scratch_bytes);
	vkh_dev_free(ctx, b->ragged_dev, b->ragged_bytes);
	free(b->recs);
	free(b->lifts);
	free(b);
}
