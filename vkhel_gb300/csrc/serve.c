/*
 * Serving loop: continuous batching of polynomial-multiply requests (no
 * counterpart in the reference, whose calls block one at a time).
 *
 * Callers submit requests -- `limbs` limb products of degree n with host
 * operands and a host result buffer -- from any thread and wait for them.  A
 * scheduler thread owned by the server:
 *   - admits requests in arrival order while the device-memory budget and a
 *     free micro-batch slot allow (a request waits at the head of the queue
 *     until enough in-flight memory is released);
 *   - forms a micro-batch of up to max_batch_limbs limb products of any mix
 *     of degrees, uploads its operands (each request as soon as its buffer
 *     is allocated) and job table on the input stream, runs one kernel per
 *     degree class on the compute stream (the fused polymul for 2^8 <= n <=
 *     2^14, the composed transforms otherwise) and downloads results on the
 *     output stream; the streams are chained by events, so while one
 *     micro-batch computes the next is uploaded and the previous one
 *     downloaded;
 *   - at low load splits a large micro-batch into chunks of limbs that
 *     pipeline the same way within the micro-batch (SRV_CHUNKS below);
 *   - a stream callback after each micro-batch's downloads completes its
 *     requests, releases their memory and wakes waiters and the scheduler
 *     (slower event polls catch a failed stream); requests that arrive while
 *     others run join the next micro-batch.
 * Resident operands: a polynomial that many requests multiply by (a key, a
 * plaintext) can be uploaded once and kept in the transform domain; its
 * requests then upload only a, and their products skip NTT(b).  The upload
 * runs on the scheduler thread, in queue order (all use of the server's
 * context stays on that thread).
 * Every limb product is computed exactly as in the plain API, so a request's
 * result is the same alone and in any mix.  Latency = completion - submission
 * (monotonic clock), recorded per request.  All device work happens on the
 * server's own context and streams.
 */
#include <errno.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "internal.h"

/* classes of one micro-batch: one per (degree, modulus class, resident
 * operand or not) present, at most 4 per degree 2^1 .. 2^26; the first
 * SRV_AUX + 1 of them can run on concurrent streams */
#define SRV_MAX_CLASSES 104
#define SRV_AUX 32
/* At low load (the micro-batch took every queued request) a micro-batch of
 * at most SRV_CHUNKS requests and at least 2 SRV_CHUNK_MIN bytes of operands
 * is issued in up to SRV_CHUNKS chunks of limbs: chunk c computes (on its
 * own stream) as soon as its operands are up, while later chunks upload,
 * and its results download while later chunks compute.  Under load the
 * micro-batches run whole, their degree classes on concurrent streams, and
 * overlap with the micro-batches before and after them instead (measured:
 * chunking under load cost 6-19 % of the throughput of an overloaded
 * server). */
#define SRV_CHUNKS 4
#define SRV_CHUNK_MIN ((uint64_t) 4 << 20)

/* A resident operand: `limbs` limb polynomials kept on the device in the
 * transform domain for the requests that multiply by them. */
struct srv_operand {
	uint32_t limbs, log_n;
	uint64_t n;
	struct vkhel_ntt_tables **tables; /* per limb; a request's (n, q, w) must match */
	const uint64_t *host;             /* b or NTT(b), read by the upload */
	int is_ntt;
	void *dev;                        /* NTT(b), limbs * n words */
	uint64_t bytes;
	uint32_t users;                   /* queued and running requests that read it */
};

struct srv_req {
	struct srv_req *next;
	int64_t id;
	uint32_t limbs, log_n;
	uint64_t n;
	const uint64_t *a, *b;
	uint64_t *c;
	struct vkhel_ntt_tables **tables;
	struct srv_operand *op; /* b is this resident operand (b unused) */
	int upload;             /* a queue entry that uploads `op` (no product) */
	int state; /* 0 queued, 1 running, 2 finished */
	int status;
	double t_submit, t_done;
	void *dev;
	uint64_t dev_bytes;
};

struct vkhel_server;

struct srv_slot {
	struct vkhel_server *srv;
	int busy;
	int done;                 /* finished (by its callback or, on error, by a poll) */
	uint64_t launches;        /* micro-batches enqueued on this slot */
	uint64_t callbacks;       /* completion callbacks run (stream order = launch order) */
	void *ev_in[SRV_CHUNKS], *ev_comp[SRV_CHUNKS], *ev_done;
	vkcu_poly_job *host_poly; /* pinned */
	vkcu_ntt_job *host_ntt;   /* pinned, 3 per job */
	void *dev_jobs;           /* poly jobs then ntt jobs */
	struct srv_req **reqs;
	uint32_t nreqs;
	int chunkable; /* formed at low load: the queue was empty after it */
};

struct vkhel_server {
	struct vkhel_ctx *ctx; /* private context: tables cache, pool, SM count */
	void *s_in, *s_comp, *s_out;
	void *s_chunk[SRV_CHUNKS - 1]; /* compute streams of chunks 1 .. SRV_CHUNKS-1 (chunk 0: s_comp) */
	/* concurrent degree classes of a micro-batch (tuning flag) */
	int forked;
	void *aux[SRV_AUX], *join[SRV_AUX], *fork;
	uint64_t budget, bytes;
	uint32_t max_limbs, nslots;
	struct srv_slot *slots;
	pthread_t thread;
	pthread_mutex_t mu;
	pthread_cond_t cv_work, cv_done;
	int stop;
	struct srv_req *q_head, *q_tail;
	struct srv_req **by_id; /* index id - 1 */
	int64_t next_id, cap_id;
	struct srv_operand **ops; /* resident operands, index id - 1 (NULL: removed) */
	int64_t nops, cap_ops;
	double *lat_ms;
	uint64_t nlat, cap_lat;
	uint64_t submitted, completed, failed, batches, limbs_done;
	double t_first, t_last;
};

static double now_s(void) {
	struct timespec ts;
	clock_gettime(CLOCK_MONOTONIC, &ts);
	return (double) ts.tv_sec + 1e-9 * (double) ts.tv_nsec;
}

static int fused_log_n(uint32_t log_n) {
	return log_n >= 8 && log_n <= vkcu_max_fused_log_n();
}

/* Device words of a request: a, b, c (+ an NTT(b) scratch off the fused
 * range); a and c only with a resident operand. */
static uint64_t req_bytes(const struct srv_req *r) {
	const uint64_t words = (uint64_t) r->limbs * r->n;
	return 8 * words * (r->op ? 2 : fused_log_n(r->log_n) ? 3 : 4);
}

/* Host bytes a request uploads per limb word: a and b, or a alone. */
static uint64_t up_per_word(const struct srv_req *r) { return r->op ? 8 : 16; }

static int cmp_job_log_n(const void *x, const void *y) {
	const uint64_t a = *(const uint64_t *) x, b = *(const uint64_t *) y;
	return (a > b) - (a < b);
}

static void finish_slot(struct vkhel_server *s, struct srv_slot *sl, int status);

/* Stream callback after a micro-batch's downloads: completes its requests at
 * once (no CUDA calls here) and wakes the scheduler for the freed slot.  If
 * the stream failed, the callback may never run; the scheduler's slower
 * event polls then finish the slot with an error. */
static void slot_done_cb(void *arg) {
	struct srv_slot *sl = arg;
	struct vkhel_server *s = sl->srv;
	pthread_mutex_lock(&s->mu);
	/* only the callback of the slot's current launch finishes it */
	if (++sl->callbacks == sl->launches && sl->busy && !sl->done) {
		sl->done = 1;
		finish_slot(s, sl, 0);
	}
	pthread_cond_broadcast(&s->cv_work);
	pthread_mutex_unlock(&s->mu);
}

/* limbs [k0, k1) of request `req` of a micro-batch */
struct srv_seg {
	uint32_t req, k0, k1;
};

/* The chunk plan: chunk c ends at the limb where the running upload bytes
 * reach (c + 1) / nchunks of the micro-batch's. */
static uint32_t chunk_count(const struct vkhel_server *s, const struct srv_slot *sl, uint64_t *up_bytes) {
	uint64_t b = 0;
	for (uint32_t i = 0; i < sl->nreqs; i++)
		b += up_per_word(sl->reqs[i]) * sl->reqs[i]->limbs * sl->reqs[i]->n;
	*up_bytes = b;
	if (!sl->chunkable || sl->nreqs > SRV_CHUNKS || b < 2 * SRV_CHUNK_MIN)
		return 1;
	return b / SRV_CHUNK_MIN < SRV_CHUNKS ? (uint32_t) (b / SRV_CHUNK_MIN) : SRV_CHUNKS;
}

/* Enqueue one chunk whose operand uploads are issued: its job-table slice
 * (jobs [j0, j1) sorted by degree, one class per degree) on the input
 * stream, its kernels on its compute stream after the uploads, its result
 * downloads (segs) on the output stream after the kernels. */
static int issue_chunk(struct vkhel_server *s, struct srv_slot *sl, uint32_t c, uint32_t nchunks, uint64_t *keys,
		const vkcu_poly_job *tmp, uint32_t j0, uint32_t j1, const struct srv_seg *segs, uint32_t nsegs) {
	struct vkhel_ctx *ctx = s->ctx;
	const uint64_t cap = ((uint64_t) s->max_limbs + 64) * 2;
	struct vkh_job_class classes[SRV_MAX_CLASSES];
	uint32_t nclasses = 0;
	qsort(keys + j0, j1 - j0, sizeof(uint64_t), cmp_job_log_n);
	for (uint32_t i = j0; i < j1; i++) {
		const uint32_t log_n = (uint32_t) (keys[i] >> 40);
		const int wide = (int) ((keys[i] >> 39) & 1);
		const uint32_t b_ntt = (uint32_t) ((keys[i] >> 38) & 1);
		sl->host_poly[i] = tmp[keys[i] & 0x3fffffffffull];
		if (nclasses == 0 || classes[nclasses - 1].log_n != log_n || classes[nclasses - 1].wide != wide ||
				classes[nclasses - 1].b_ntt != b_ntt) {
			if (nclasses == SRV_MAX_CLASSES)
				return VKHEL_ERR_UNSUPPORTED;
			struct vkh_job_class *cl = &classes[nclasses++];
			cl->kind = VKH_JOB_POLYMUL;
			cl->log_n = log_n;
			cl->wide = wide;
			cl->lift = 0;
			cl->b_ntt = b_ntt;
			cl->first = i;
			cl->count = 0;
			cl->fused = fused_log_n(log_n);
		}
		classes[nclasses - 1].count++;
	}
	vkh_fill_ntt_jobs(sl->host_poly, sl->host_ntt, classes, nclasses);
	vkcu_poly_job *dpoly = sl->dev_jobs;
	vkcu_ntt_job *dntt = (vkcu_ntt_job *) ((char *) sl->dev_jobs + sizeof(vkcu_poly_job) * cap);
	int e = vkcu_h2d(s->s_in, dpoly + j0, sl->host_poly + j0, sizeof(vkcu_poly_job) * (j1 - j0));
	if (!e)
		e = vkcu_h2d(s->s_in, dntt + 3 * (size_t) j0, sl->host_ntt + 3 * (size_t) j0,
				sizeof(vkcu_ntt_job) * 3 * (j1 - j0));
	void *cs = c == 0 ? s->s_comp : s->s_chunk[c - 1];
	if (!e)
		e = vkcu_event_record(sl->ev_in[c], s->s_in);
	if (!e)
		e = vkcu_stream_wait(cs, sl->ev_in[c]);
	if (!e) /* a whole micro-batch: its classes on concurrent streams when tuned so */
		e = s->forked && nchunks == 1 && nclasses <= SRV_AUX + 1
				? vkh_issue_classes_forked(cs, s->aux, s->fork, s->join, ctx->sms, dpoly, dntt, classes, nclasses, NULL)
				: vkh_issue_classes(cs, ctx->sms, dpoly, dntt, classes, nclasses, NULL);
	if (!e)
		e = vkcu_event_record(sl->ev_comp[c], cs);
	if (!e)
		e = vkcu_stream_wait(s->s_out, sl->ev_comp[c]);
	for (uint32_t g = 0; !e && g < nsegs; g++) {
		struct srv_req *r = sl->reqs[segs[g].req];
		const uint64_t words = (uint64_t) r->limbs * r->n, off = (uint64_t) segs[g].k0 * r->n;
		e = vkcu_d2h(s->s_out, r->c + off, (uint64_t *) r->dev + (r->op ? 1 : 2) * words + off,
				8 * (size_t) (segs[g].k1 - segs[g].k0) * r->n);
	}
	return e;
}

/* Enqueue one micro-batch on the server streams (called without the lock).
 * Each request's device buffer is allocated and its operands uploaded at
 * once (the copy engine starts on the first request while the host prepares
 * the rest); each chunk is enqueued as soon as its last limb is uploaded. */
static void launch_slot(struct vkhel_server *s, struct srv_slot *sl) {
	struct vkhel_ctx *ctx = s->ctx;
	vkcu_range_push("vkhel_server micro-batch");
	const uint64_t cap = ((uint64_t) s->max_limbs + 64) * 2;
	/* keys: log_n in the high bits, then the modulus class, running index in
	 * the low bits -> stable sort into classes of one degree and class */
	uint64_t *keys = malloc(sizeof(uint64_t) * cap);
	vkcu_poly_job *tmp = malloc(sizeof(vkcu_poly_job) * cap);
	struct srv_seg *segs = malloc(sizeof(struct srv_seg) * (sl->nreqs + SRV_CHUNKS));
	int err = !keys || !tmp || !segs ? VKHEL_ERR_OUT_OF_MEMORY : 0;
	uint64_t up_bytes = 0, acc = 0;
	const uint32_t nchunks = chunk_count(s, sl, &up_bytes);
	uint32_t njobs = 0, c = 0, chunk_j0 = 0, chunk_s0 = 0, nsegs = 0;
	int issued = 0; /* device work of this micro-batch enqueued (uploads at least) */
	for (uint32_t i = 0; !err && i < sl->nreqs; i++) {
		struct srv_req *r = sl->reqs[i];
		const uint64_t words = (uint64_t) r->limbs * r->n;
		const int fused = fused_log_n(r->log_n);
		int e = vkh_inject_alloc_failure() ? VKHEL_ERR_OUT_OF_MEMORY
		                                   : vkcu_alloc(ctx->pool, s->s_in, r->dev_bytes, &r->dev);
		uint32_t k0 = 0;
		for (uint32_t k = 0; !e && k < r->limbs; k++) {
			const struct vkh_devtab *d = NULL;
			e = vkh_devtab_get(ctx, r->tables[k], &d);
			if (e)
				break;
			uint64_t *base = r->dev;
			vkcu_poly_job j = {0};
			j.a = base + (uint64_t) k * r->n;
			if (r->op) { /* device layout a, c; b is the resident NTT(b) */
				j.b = (const uint64_t *) r->op->dev + (uint64_t) k * r->n;
				j.c = base + words + (uint64_t) k * r->n;
				j.scratch = (uint64_t *) j.b; /* read by the composed path's pointwise step */
				j.flags = VKCU_JOB_B_NTT;
			} else { /* a, b, c (+ scratch) */
				j.b = base + words + (uint64_t) k * r->n;
				j.c = base + 2 * words + (uint64_t) k * r->n;
				j.scratch = fused ? j.c : base + 3 * words + (uint64_t) k * r->n;
			}
			j.tw = d->dev_set;
			keys[njobs] = ((uint64_t) r->log_n << 40) | ((uint64_t) vkcu_wide(r->tables[k]->q) << 39) |
					((uint64_t) (r->op != NULL) << 38) | njobs;
			tmp[njobs++] = j;
			acc += up_per_word(r) * r->n;
			const int last = i + 1 == sl->nreqs && k + 1 == r->limbs;
			const int close = last || (c + 1 < nchunks && acc * nchunks >= up_bytes * (c + 1));
			if (close || k + 1 == r->limbs) { /* a segment ends: upload it */
				const uint64_t off = (uint64_t) k0 * r->n;
				const size_t len = 8 * (size_t) (k + 1 - k0) * r->n;
				segs[nsegs++] = (struct srv_seg){i, k0, k + 1};
				k0 = k + 1;
				issued = 1;
				e = vkcu_h2d(s->s_in, (uint64_t *) r->dev + off, r->a + off, len);
				if (!e && !r->op)
					e = vkcu_h2d(s->s_in, (uint64_t *) r->dev + words + off, r->b + off, len);
			}
			if (!e && close) {
				e = issue_chunk(s, sl, c, nchunks, keys, tmp, chunk_j0, njobs, segs + chunk_s0, nsegs - chunk_s0);
				c++;
				chunk_j0 = njobs;
				chunk_s0 = nsegs;
			}
		}
		if (e)
			err = e == 2 /* cudaErrorMemoryAllocation */ || e == VKHEL_ERR_BUDGET || e == VKHEL_ERR_OUT_OF_MEMORY
					? VKHEL_ERR_OUT_OF_MEMORY
					: VKHEL_ERR_DEVICE;
	}
	if (err) { /* the micro-batch's requests fail; what was enqueued still drains */
		for (uint32_t i = 0; i < sl->nreqs; i++)
			sl->reqs[i]->status = err;
		if (issued) { /* frees below: after every upload and kernel enqueued so far */
			vkcu_event_record(sl->ev_done, s->s_in);
			vkcu_stream_wait(s->s_out, sl->ev_done);
			for (uint32_t cc = 0; cc <= c && cc < nchunks; cc++) {
				void *cs = cc == 0 ? s->s_comp : s->s_chunk[cc - 1];
				vkcu_event_record(sl->ev_comp[cc], cs);
				vkcu_stream_wait(s->s_out, sl->ev_comp[cc]);
			}
		}
	}
	for (uint32_t i = 0; i < sl->nreqs; i++) {
		struct srv_req *r = sl->reqs[i];
		if (r->dev)
			vkcu_free(s->s_out, r->dev); /* stream-ordered: after the downloads */
		r->dev = NULL;
	}
	vkcu_event_record(sl->ev_done, s->s_out);
	vkcu_launch_host_func(s->s_out, slot_done_cb, sl);
	free(keys);
	free(tmp);
	free(segs);
	vkcu_range_pop();
}

/* Mark a finished slot's requests done (lock held). */
static void finish_slot(struct vkhel_server *s, struct srv_slot *sl, int status) {
	const double t = now_s();
	for (uint32_t i = 0; i < sl->nreqs; i++) {
		struct srv_req *r = sl->reqs[i];
		if (r->status == 0 && status)
			r->status = status;
		r->state = 2;
		r->t_done = t;
		s->bytes -= r->dev_bytes;
		if (r->op)
			r->op->users--;
		if (r->status == 0) {
			s->completed++;
			s->limbs_done += r->limbs;
			if (s->nlat == s->cap_lat) {
				s->cap_lat = s->cap_lat ? 2 * s->cap_lat : 4096;
				s->lat_ms = realloc(s->lat_ms, sizeof(double) * s->cap_lat);
			}
			s->lat_ms[s->nlat++] = 1e3 * (t - r->t_submit);
			s->t_last = t;
		} else {
			s->failed++;
		}
	}
	sl->nreqs = 0;
	sl->busy = 0;
	s->batches++;
	pthread_cond_broadcast(&s->cv_done);
}

/* Upload a resident operand (scheduler thread, no lock): b or NTT(b) into a
 * pool buffer on the input stream, then, for b, a forward transform of every
 * limb in place; returns a status. */
static int upload_operand(struct vkhel_server *s, struct srv_operand *op) {
	struct vkhel_ctx *ctx = s->ctx;
	op->bytes = 8 * (uint64_t) op->limbs * op->n;
	if (vkh_inject_alloc_failure() || vkcu_alloc(ctx->pool, s->s_in, op->bytes, &op->dev)) {
		op->dev = NULL;
		return VKHEL_ERR_OUT_OF_MEMORY;
	}
	int st = VKHEL_OK;
	int e = vkcu_h2d(s->s_in, op->dev, op->host, op->bytes);
	for (uint32_t k = 0; !e && !st && !op->is_ntt && k < op->limbs; k++) {
		const struct vkh_devtab *d = NULL;
		st = vkh_devtab_get(ctx, op->tables[k], &d);
		if (st)
			break;
		uint64_t *p = (uint64_t *) op->dev + (uint64_t) k * op->n;
		const vkcu_ntt_job j = {p, p, d->dev_set};
		e = vkcu_ntt_forward(s->s_in, NULL, 1, &j, op->log_n, vkcu_wide(op->tables[k]->q), ctx->sms);
	}
	const int se = vkcu_sync(s->s_in);
	if (!e)
		e = se;
	if (!st && e)
		st = VKHEL_ERR_DEVICE;
	if (st) {
		vkcu_free(s->s_in, op->dev);
		op->dev = NULL;
	}
	return st;
}

static void *scheduler(void *arg) {
	struct vkhel_server *s = arg;
	vkcu_set_device(s->ctx->device);
	for (;;) {
		int progressed = 0;
		/* micro-batches complete through their stream callbacks; these polls
		 * only catch a failed stream, whose callback may never run */
		for (uint32_t k = 0; k < s->nslots; k++) {
			struct srv_slot *sl = &s->slots[k];
			pthread_mutex_lock(&s->mu);
			const int live = sl->busy && !sl->done;
			pthread_mutex_unlock(&s->mu);
			if (!live)
				continue;
			const int q = vkcu_event_query(sl->ev_done);
			if (q == 0 || q == 1) /* done (its callback finishes it) or still running */
				continue;
			pthread_mutex_lock(&s->mu);
			if (sl->busy && !sl->done) {
				sl->done = 1;
				finish_slot(s, sl, VKHEL_ERR_DEVICE);
				progressed = 1;
			}
			pthread_mutex_unlock(&s->mu);
		}
		/* admission */
		pthread_mutex_lock(&s->mu);
		struct srv_slot *free_slot = NULL;
		int inflight = 0;
		for (uint32_t k = 0; k < s->nslots; k++) {
			if (s->slots[k].busy)
				inflight++;
			else if (!free_slot)
				free_slot = &s->slots[k];
		}
		if (s->stop && !s->q_head && inflight == 0) {
			pthread_mutex_unlock(&s->mu);
			break;
		}
		/* an operand upload at the head of the queue runs before anything
		 * queued after it (requests that read it come later) */
		if (s->q_head && s->q_head->upload) {
			struct srv_req *r = s->q_head;
			s->q_head = r->next;
			if (!s->q_head)
				s->q_tail = NULL;
			r->state = 1;
			pthread_mutex_unlock(&s->mu);
			const int st = upload_operand(s, r->op);
			pthread_mutex_lock(&s->mu);
			r->status = st;
			r->state = 2;
			r->t_done = now_s();
			pthread_cond_broadcast(&s->cv_done);
			pthread_mutex_unlock(&s->mu);
			continue;
		}
		uint32_t limbs = 0;
		if (free_slot) {
			while (s->q_head) {
				struct srv_req *r = s->q_head;
				if (r->upload) /* runs once this micro-batch is launched */
					break;
				if (free_slot->nreqs > 0 && limbs + r->limbs > s->max_limbs)
					break;
				if (s->budget && s->bytes + r->dev_bytes > s->budget && (inflight > 0 || free_slot->nreqs > 0))
					break; /* wait for memory held by running requests */
				s->q_head = r->next;
				if (!s->q_head)
					s->q_tail = NULL;
				r->state = 1;
				s->bytes += r->dev_bytes;
				limbs += r->limbs;
				free_slot->reqs[free_slot->nreqs++] = r;
			}
		}
		if (free_slot && free_slot->nreqs) {
			free_slot->chunkable = s->q_head == NULL;
			free_slot->busy = 1;
			free_slot->done = 0;
			free_slot->launches++;
			pthread_mutex_unlock(&s->mu);
			launch_slot(s, free_slot);
			progressed = 1;
			continue;
		}
		if (!progressed) {
			if (inflight == 0) {
				while (!s->q_head && !s->stop)
					pthread_cond_wait(&s->cv_work, &s->mu);
			} else {
				/* woken by a completion callback or a submission; the timeout
				 * bounds how late a failed stream is noticed */
				struct timespec dl;
				clock_gettime(CLOCK_REALTIME, &dl);
				dl.tv_nsec += 200000;
				if (dl.tv_nsec >= 1000000000L) {
					dl.tv_sec++;
					dl.tv_nsec -= 1000000000L;
				}
				pthread_cond_timedwait(&s->cv_work, &s->mu, &dl);
			}
		}
		pthread_mutex_unlock(&s->mu);
	}
	return NULL;
}

struct vkhel_server *vkhel_server_create(const struct vkhel_server_config *cfg) {
	struct vkhel_server *s = calloc(1, sizeof(*s));
	if (!s) {
		vkh_fail(NULL, VKHEL_ERR_OUT_OF_MEMORY, "server: host allocation failed");
		return NULL;
	}
	s->ctx = vkhel_ctx_create();
	if (!s->ctx) {
		free(s);
		return NULL;
	}
	s->budget = cfg && cfg->device_budget ? cfg->device_budget : ((uint64_t) 40 << 30);
	s->max_limbs = cfg && cfg->max_batch_limbs ? cfg->max_batch_limbs : 1024;
	s->nslots = cfg && cfg->max_inflight_batches ? cfg->max_inflight_batches : 3;
	s->slots = calloc(s->nslots, sizeof(*s->slots));
	int e = !s->slots;
	/* request buffers are allocated on the input stream and freed on the
	 * output stream: without this the pool may make an upload wait for an
	 * earlier micro-batch's download, serializing the two copy directions */
	if (!e)
		e = vkcu_pool_independent_streams(s->ctx->pool);
	if (!e)
		e = vkcu_stream_create(&s->s_in);
	if (!e)
		e = vkcu_stream_create(&s->s_comp);
	if (!e)
		e = vkcu_stream_create(&s->s_out);
	for (int c = 0; !e && c < SRV_CHUNKS - 1; c++)
		e = vkcu_stream_create(&s->s_chunk[c]);
	s->forked = vkh_variant(3, 0) == 1;
	if (!e && s->forked)
		e = vkcu_event_create(&s->fork);
	for (uint32_t k = 0; !e && s->forked && k < SRV_AUX; k++) {
		e = vkcu_stream_create(&s->aux[k]);
		if (!e)
			e = vkcu_event_create(&s->join[k]);
	}
	const uint64_t cap = (uint64_t) s->max_limbs + 64;
	for (uint32_t k = 0; !e && k < s->nslots; k++) {
		struct srv_slot *sl = &s->slots[k];
		sl->srv = s;
		sl->reqs = calloc(2 * cap, sizeof(*sl->reqs));
		e = !sl->reqs;
		for (int c = 0; !e && c < SRV_CHUNKS; c++) {
			e = vkcu_event_create(&sl->ev_in[c]);
			if (!e)
				e = vkcu_event_create(&sl->ev_comp[c]);
		}
		if (!e)
			e = vkcu_event_create(&sl->ev_done);
		if (!e)
			e = vkcu_host_alloc((void **) &sl->host_poly, sizeof(vkcu_poly_job) * 2 * cap);
		if (!e)
			e = vkcu_host_alloc((void **) &sl->host_ntt, sizeof(vkcu_ntt_job) * 6 * cap);
		if (!e)
			e = vkh_dev_alloc(s->ctx, (sizeof(vkcu_poly_job) + 3 * sizeof(vkcu_ntt_job)) * 2 * cap, &sl->dev_jobs);
	}
	if (!e)
		e = vkcu_sync(s->ctx->stream);
	if (e) {
		vkh_fail(NULL, VKHEL_ERR_DEVICE, "server: set-up failed (%d)", e);
		vkhel_server_destroy(s);
		return NULL;
	}
	pthread_mutex_init(&s->mu, NULL);
	pthread_cond_init(&s->cv_work, NULL);
	pthread_cond_init(&s->cv_done, NULL);
	s->next_id = 1;
	if (pthread_create(&s->thread, NULL, scheduler, s) != 0) {
		vkh_fail(NULL, VKHEL_ERR_DEVICE, "server: thread creation failed");
		s->thread = 0;
		vkhel_server_destroy(s);
		return NULL;
	}
	return s;
}

/* The tables of one submission: every limb of one degree n >= 2 and a
 * modulus the kernels take. */
static int check_tables(struct vkhel_ntt_tables *const *tables, uint32_t limbs, const char *fn) {
	const uint64_t n = tables[0]->n;
	for (uint32_t k = 0; k < limbs; k++) {
		const struct vkhel_ntt_tables *t = tables[k];
		if (!t || t->n != n || n < 2)
			return vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "%s: limb %u tables invalid", fn, k);
		if (t->q >= ((uint64_t) 1 << 63) || t->q < 3 || t->unreduced || t->log_n > vkcu_max_log_n())
			return vkh_fail(NULL, VKHEL_ERR_UNSUPPORTED, "%s: limb %u (n, q) unsupported", fn, k);
	}
	return VKHEL_OK;
}

/* A request (or operand upload) for the given limbs, tables copied. */
static struct srv_req *new_req(struct vkhel_ntt_tables *const *tables, uint32_t limbs) {
	struct srv_req *r = calloc(1, sizeof(*r));
	struct vkhel_ntt_tables **tcopy = malloc(sizeof(*tcopy) * limbs);
	if (!r || !tcopy) {
		free(r);
		free(tcopy);
		vkh_fail(NULL, VKHEL_ERR_OUT_OF_MEMORY, "server: host allocation failed");
		return NULL;
	}
	memcpy(tcopy, tables, sizeof(*tcopy) * limbs);
	r->tables = tcopy;
	r->limbs = limbs;
	r->n = tables[0]->n;
	r->log_n = tables[0]->log_n;
	return r;
}

/* Queue `r` (id assigned); with operand > 0 the request reads that resident
 * operand, whose limbs must have the request's (n, q, w).  Returns the id or
 * -status (r freed). */
static int64_t enqueue(struct vkhel_server *s, struct srv_req *r, int64_t operand, const char *fn) {
	int st = VKHEL_OK;
	pthread_mutex_lock(&s->mu);
	if (s->stop) {
		st = vkh_fail(NULL, VKHEL_ERR_CANCELLED, "%s: server is stopping", fn);
	} else if (operand) {
		struct srv_operand *op = operand > 0 && operand <= s->nops ? s->ops[operand - 1] : NULL;
		if (!op) {
			st = vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "%s: unknown or removed operand %lld", fn,
					(long long) operand);
		} else if (op->limbs != r->limbs || op->n != r->n) {
			st = vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "%s: operand %lld has %u limbs of degree %llu", fn,
					(long long) operand, op->limbs, (unsigned long long) op->n);
		} else {
			for (uint32_t k = 0; k < r->limbs && !st; k++)
				if (op->tables[k]->q != r->tables[k]->q || op->tables[k]->w != r->tables[k]->w)
					st = vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "%s: limb %u tables differ from operand %lld's",
							fn, k, (long long) operand);
		}
		if (!st) {
			r->op = op;
			r->dev_bytes = req_bytes(r);
		}
	}
	if (!st && s->next_id > s->cap_id) {
		const int64_t cap = s->cap_id ? 2 * s->cap_id : 4096;
		struct srv_req **m = realloc(s->by_id, sizeof(*m) * (size_t) cap);
		if (!m) {
			st = vkh_fail(NULL, VKHEL_ERR_OUT_OF_MEMORY, "%s: host allocation failed", fn);
		} else {
			s->by_id = m;
			s->cap_id = cap;
		}
	}
	if (st) {
		pthread_mutex_unlock(&s->mu);
		free(r->tables);
		free(r);
		return -st;
	}
	if (r->op && !r->upload)
		r->op->users++;
	r->id = s->next_id++;
	s->by_id[r->id - 1] = r;
	r->t_submit = now_s();
	if (!r->upload && s->submitted++ == 0)
		s->t_first = r->t_submit;
	if (s->q_tail)
		s->q_tail->next = r;
	else
		s->q_head = r;
	s->q_tail = r;
	pthread_cond_signal(&s->cv_work);
	pthread_mutex_unlock(&s->mu);
	return r->id;
}

static int64_t submit_impl(struct vkhel_server *s, struct vkhel_ntt_tables *const *tables, uint32_t limbs,
		const uint64_t *a, const uint64_t *b, int64_t operand, uint64_t *c, const char *fn) {
	if (!s || !tables || !limbs || !a || (!b && !operand) || !c || !tables[0])
		return -vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "%s: bad arguments", fn);
	if (limbs > s->max_limbs)
		return -vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "%s: %u limbs exceed the micro-batch size %u", fn, limbs,
				s->max_limbs);
	int st = check_tables(tables, limbs, fn);
	if (st)
		return -st;
	struct srv_req *r = new_req(tables, limbs);
	if (!r)
		return -VKHEL_ERR_OUT_OF_MEMORY;
	r->a = a;
	r->b = b;
	r->c = c;
	r->dev_bytes = req_bytes(r);
	return enqueue(s, r, operand, fn);
}

int64_t vkhel_server_submit(struct vkhel_server *s, struct vkhel_ntt_tables *const *tables, uint32_t limbs,
		const uint64_t *a, const uint64_t *b, uint64_t *c) {
	return submit_impl(s, tables, limbs, a, b, 0, c, "server_submit");
}

int64_t vkhel_server_submit_operand(struct vkhel_server *s, struct vkhel_ntt_tables *const *tables, uint32_t limbs,
		const uint64_t *a, int64_t operand, uint64_t *c) {
	if (operand < 1)
		return -vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "server_submit_operand: bad operand id");
	return submit_impl(s, tables, limbs, a, NULL, operand, c, "server_submit_operand");
}

int64_t vkhel_server_add_operand(struct vkhel_server *s, struct vkhel_ntt_tables *const *tables, uint32_t limbs,
		const uint64_t *b, int is_ntt) {
	const char *fn = "server_add_operand";
	if (!s || !tables || !limbs || !b || !tables[0])
		return -vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "%s: bad arguments", fn);
	int st = check_tables(tables, limbs, fn);
	if (st)
		return -st;
	struct srv_operand *op = calloc(1, sizeof(*op));
	struct srv_req *r = new_req(tables, limbs);
	if (!op || !r) {
		free(op);
		if (r) {
			free(r->tables);
			free(r);
		}
		return -vkh_fail(NULL, VKHEL_ERR_OUT_OF_MEMORY, "%s: host allocation failed", fn);
	}
	op->tables = r->tables; /* kept by the operand; the queue entry's copy is not freed twice */
	r->tables = NULL;
	op->limbs = limbs;
	op->n = r->n;
	op->log_n = r->log_n;
	op->host = b;
	op->is_ntt = is_ntt != 0;
	r->upload = 1;
	r->op = op;
	const int64_t id = enqueue(s, r, 0, fn);
	if (id < 0) {
		free(op->tables);
		free(op);
		return id;
	}
	/* the scheduler runs the upload in queue order; wait for it */
	while ((st = vkhel_server_wait(s, id, 60000)) == VKHEL_ERR_TIMEOUT)
		;
	if (st) {
		free(op->tables);
		free(op);
		return -vkh_fail(NULL, st, "%s: upload failed", fn);
	}
	op->host = NULL;
	pthread_mutex_lock(&s->mu);
	if (s->nops == s->cap_ops) {
		const int64_t cap = s->cap_ops ? 2 * s->cap_ops : 64;
		struct srv_operand **m = realloc(s->ops, sizeof(*m) * (size_t) cap);
		if (!m) {
			pthread_mutex_unlock(&s->mu);
			vkcu_free(s->ctx->stream, op->dev);
			free(op->tables);
			free(op);
			return -vkh_fail(NULL, VKHEL_ERR_OUT_OF_MEMORY, "%s: host allocation failed", fn);
		}
		s->ops = m;
		s->cap_ops = cap;
	}
	s->ops[s->nops++] = op;
	const int64_t oid = s->nops;
	pthread_mutex_unlock(&s->mu);
	return oid;
}

int vkhel_server_remove_operand(struct vkhel_server *s, int64_t operand) {
	if (!s)
		return vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "server_remove_operand: NULL server");
	pthread_mutex_lock(&s->mu);
	struct srv_operand *op = operand > 0 && operand <= s->nops ? s->ops[operand - 1] : NULL;
	if (!op || op->users) {
		const uint32_t users = op ? op->users : 0;
		pthread_mutex_unlock(&s->mu);
		return op ? vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT,
		                     "server_remove_operand: operand %lld is read by %u queued or running requests",
		                     (long long) operand, users)
		          : vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "server_remove_operand: unknown or removed operand %lld",
		                     (long long) operand);
	}
	s->ops[operand - 1] = NULL;
	pthread_mutex_unlock(&s->mu);
	/* no request reads it any more: every one that did has finished, kernels included */
	vkcu_free(s->ctx->stream, op->dev);
	free(op->tables);
	free(op);
	return VKHEL_OK;
}

int vkhel_server_wait(struct vkhel_server *s, int64_t id, uint32_t timeout_ms) {
	if (!s || id < 1)
		return vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "server_wait: bad arguments");
	struct timespec dl;
	clock_gettime(CLOCK_REALTIME, &dl);
	dl.tv_sec += timeout_ms / 1000;
	dl.tv_nsec += (long) (timeout_ms % 1000) * 1000000L;
	if (dl.tv_nsec >= 1000000000L) {
		dl.tv_sec++;
		dl.tv_nsec -= 1000000000L;
	}
	pthread_mutex_lock(&s->mu);
	if (id >= s->next_id || !s->by_id[id - 1]) {
		pthread_mutex_unlock(&s->mu);
		return vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "server_wait: unknown or already collected id %lld",
				(long long) id);
	}
	struct srv_req *r = s->by_id[id - 1];
	while (r->state != 2) {
		if (pthread_cond_timedwait(&s->cv_done, &s->mu, &dl) == ETIMEDOUT && r->state != 2) {
			pthread_mutex_unlock(&s->mu);
			return VKHEL_ERR_TIMEOUT;
		}
	}
	const int st = r->status;
	s->by_id[id - 1] = NULL;
	pthread_mutex_unlock(&s->mu);
	free(r->tables);
	free(r);
	return st;
}

int vkhel_server_cancel(struct vkhel_server *s, int64_t id) {
	if (!s || id < 1)
		return vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "server_cancel: bad arguments");
	pthread_mutex_lock(&s->mu);
	if (id >= s->next_id || !s->by_id[id - 1]) {
		pthread_mutex_unlock(&s->mu);
		return vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "server_cancel: unknown or already collected id %lld",
				(long long) id);
	}
	struct srv_req *r = s->by_id[id - 1];
	if (r->state != 0) {
		pthread_mutex_unlock(&s->mu);
		return vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "server_cancel: request %lld is already %s",
				(long long) id, r->state == 1 ? "running" : "finished");
	}
	/* unlink from the queue */
	struct srv_req *prev = NULL;
	for (struct srv_req *q = s->q_head; q && q != r; q = q->next)
		prev = q;
	if (prev)
		prev->next = r->next;
	else
		s->q_head = r->next;
	if (s->q_tail == r)
		s->q_tail = prev;
	r->next = NULL;
	r->state = 2;
	r->status = VKHEL_ERR_CANCELLED;
	r->t_done = now_s();
	if (r->op && !r->upload)
		r->op->users--;
	if (!r->upload)
		s->failed++;
	pthread_cond_broadcast(&s->cv_done);
	pthread_mutex_unlock(&s->mu);
	return VKHEL_OK;
}

static int cmp_double(const void *x, const void *y) {
	const double a = *(const double *) x, b = *(const double *) y;
	return (a > b) - (a < b);
}

int vkhel_server_stats(struct vkhel_server *s, struct vkhel_server_stats *out) {
	if (!s || !out)
		return vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "server_stats: NULL argument");
	memset(out, 0, sizeof(*out));
	pthread_mutex_lock(&s->mu);
	out->submitted = s->submitted;
	out->completed = s->completed;
	out->failed = s->failed;
	out->batches = s->batches;
	out->limbs = s->limbs_done;
	out->span_s = s->completed ? s->t_last - s->t_first : 0;
	const uint64_t n = s->nlat;
	double *v = n ? malloc(sizeof(double) * n) : NULL;
	if (v)
		memcpy(v, s->lat_ms, sizeof(double) * n);
	pthread_mutex_unlock(&s->mu);
	if (v) {
		qsort(v, n, sizeof(double), cmp_double);
		double sum = 0;
		for (uint64_t i = 0; i < n; i++)
			sum += v[i];
		out->mean_ms = sum / (double) n;
		out->p50_ms = v[n / 2];
		out->p99_ms = v[(uint64_t) (0.99 * (double) (n - 1))];
		out->max_ms = v[n - 1];
		free(v);
	}
	return VKHEL_OK;
}

int vkhel_server_reset_stats(struct vkhel_server *s) {
	if (!s)
		return vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "server_reset_stats: NULL server");
	pthread_mutex_lock(&s->mu);
	s->nlat = 0;
	s->submitted = s->completed = s->failed = s->batches = s->limbs_done = 0;
	s->t_first = s->t_last = 0;
	pthread_mutex_unlock(&s->mu);
	return VKHEL_OK;
}

/* Drains: queued requests still run; then every resource is released.
 * Requests never waited for are freed here. */
void vkhel_server_destroy(struct vkhel_server *s) {
	if (!s)
		return;
	if (s->thread) {
		pthread_mutex_lock(&s->mu);
		s->stop = 1;
		pthread_cond_broadcast(&s->cv_work);
		pthread_mutex_unlock(&s->mu);
		pthread_join(s->thread, NULL);
		pthread_mutex_destroy(&s->mu);
		pthread_cond_destroy(&s->cv_work);
		pthread_cond_destroy(&s->cv_done);
	}
	void *streams[3] = {s->s_in, s->s_comp, s->s_out};
	for (int i = 0; i < 3; i++)
		if (streams[i])
			vkcu_sync(streams[i]);
	for (int c = 0; c < SRV_CHUNKS - 1; c++)
		if (s->s_chunk[c]) {
			vkcu_sync(s->s_chunk[c]);
			vkcu_stream_destroy(s->s_chunk[c]);
		}
	for (uint32_t k = 0; s->slots && k < s->nslots; k++) {
		struct srv_slot *sl = &s->slots[k];
		for (int c = 0; c < SRV_CHUNKS; c++) {
			vkcu_event_destroy(sl->ev_in[c]);
			vkcu_event_destroy(sl->ev_comp[c]);
		}
		vkcu_event_destroy(sl->ev_done);
		vkcu_host_free(sl->host_poly);
		vkcu_host_free(sl->host_ntt);
		if (sl->dev_jobs)
			vkh_dev_free(s->ctx, sl->dev_jobs,
					(sizeof(vkcu_poly_job) + 3 * sizeof(vkcu_ntt_job)) * 2 * ((uint64_t) s->max_limbs + 64));
		free(sl->reqs);
	}
	for (int i = 0; i < 3; i++)
		if (streams[i])
			vkcu_stream_destroy(streams[i]);
	for (int k = 0; k < SRV_AUX; k++) {
		if (s->aux[k]) {
			vkcu_sync(s->aux[k]);
			vkcu_stream_destroy(s->aux[k]);
		}
		vkcu_event_destroy(s->join[k]);
	}
	vkcu_event_destroy(s->fork);
	for (int64_t i = 0; i + 1 < s->next_id; i++) {
		if (s->by_id[i]) {
			free(s->by_id[i]->tables);
			free(s->by_id[i]);
		}
	}
	for (int64_t i = 0; i < s->nops; i++) {
		if (s->ops[i]) {
			vkcu_free(s->ctx->stream, s->ops[i]->dev);
			free(s->ops[i]->tables);
			free(s->ops[i]);
		}
	}
	if (s->ctx && s->nops)
		vkcu_sync(s->ctx->stream);
	free(s->ops);
	if (s->ctx)
		vkhel_ctx_destroy(s->ctx);
	free(s->slots);
	free(s->by_id);
	free(s->lat_ms);
	free(s);
}
