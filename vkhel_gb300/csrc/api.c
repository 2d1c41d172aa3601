/*
 * libvkhel public API on CUDA (C host layer).
 *
 * Replaces the reference's src/vkhel.c (context), src/vector.c (vectors,
 * transfers, op dispatch, transform stage loops) and the src/kernels/ wrappers (push
 * constants): each call validates its arguments, computes the same constants
 * the reference pushes, launches one kernel through the vkcu_* C ABI on the
 * context stream and waits for it, exactly as the reference waits on its
 * fence after every submit.
 */
#include <inttypes.h>
#include <stdatomic.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "internal.h"

static _Thread_local int tls_error;
static _Thread_local char tls_msg[256];

static int env_flag(const char *name) {
	const char *v = getenv(name);
	return v && *v && strcmp(v, "0") != 0;
}

int vkh_fail(struct vkhel_ctx *ctx, int code, const char *fmt, ...) {
	char buf[256];
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(buf, sizeof buf, fmt, ap);
	va_end(ap);
	if (ctx) {
		ctx->last_error = code;
		memcpy(ctx->last_msg, buf, sizeof buf);
	}
	tls_error = code;
	memcpy(tls_msg, buf, sizeof buf);
	if (env_flag("VKHEL_DEBUG") || (ctx && ctx->strict) || (!ctx && env_flag("VKHEL_STRICT")))
		fprintf(stderr, "vkhel: %s\n", buf);
	if ((ctx && ctx->strict) || (!ctx && env_flag("VKHEL_STRICT")))
		abort();
	return code;
}

int vkh_cuda(struct vkhel_ctx *ctx, int err, const char *what) {
	if (err == 0)
		return VKHEL_OK;
	const int code = (err == 2 /* cudaErrorMemoryAllocation */) ? VKHEL_ERR_OUT_OF_MEMORY : VKHEL_ERR_DEVICE;
	return vkh_fail(ctx, code, "%s: CUDA error %d (%s)", what, err, vkcu_error_string(err));
}

/* Host-side fault injection for tests: after `skip` more device allocations,
 * the next `count` fail as if the device were out of memory. */
static _Atomic uint64_t g_fail_skip, g_fail_count;

int vkhel_debug_fail_allocations(uint64_t skip, uint64_t count) {
	g_fail_count = 0;
	g_fail_skip = skip;
	g_fail_count = count;
	return VKHEL_OK;
}

int vkh_inject_alloc_failure(void) {
	for (;;) {
		uint64_t c = g_fail_count;
		if (c == 0)
			return 0;
		uint64_t k = g_fail_skip;
		if (k > 0) {
			if (atomic_compare_exchange_weak(&g_fail_skip, &k, k - 1))
				return 0;
			continue;
		}
		if (atomic_compare_exchange_weak(&g_fail_count, &c, c - 1))
			return 1;
	}
}

int vkh_dev_alloc(struct vkhel_ctx *ctx, uint64_t bytes, void **ptr) {
	if (vkh_inject_alloc_failure())
		return vkh_fail(ctx, VKHEL_ERR_OUT_OF_MEMORY, "device allocation of %" PRIu64 " bytes failed (injected)",
				bytes);
	if (ctx->budget && ctx->in_use + bytes > ctx->budget)
		return vkh_fail(ctx, VKHEL_ERR_BUDGET,
				"device budget: %" PRIu64 " + %" PRIu64 " bytes exceeds %" PRIu64,
				ctx->in_use, bytes, ctx->budget);
	const int e = vkcu_alloc(ctx->pool, ctx->stream, bytes, ptr);
	if (e != 0)
		return vkh_cuda(ctx, e, "device allocation");
	ctx->in_use += bytes;
	return VKHEL_OK;
}

void vkh_dev_free(struct vkhel_ctx *ctx, void *ptr, uint64_t bytes) {
	if (!ptr)
		return;
	vkcu_free(ctx->stream, ptr);
	ctx->in_use -= bytes;
}

/* ------------------------------------------------------------------ */
/* context                                                             */
/* ------------------------------------------------------------------ */

struct vkhel_ctx *vkhel_ctx_create() {
	struct vkhel_ctx *ctx = calloc(1, sizeof(*ctx));
	if (!ctx) {
		vkh_fail(NULL, VKHEL_ERR_OUT_OF_MEMORY, "context: host allocation failed");
		return NULL;
	}
	ctx->strict = env_flag("VKHEL_STRICT");
	ctx->async = env_flag("VKHEL_ASYNC");
	const char *dev = getenv("VKHEL_DEVICE");
	ctx->device = dev ? atoi(dev) : 0;
	const char *budget = getenv("VKHEL_DEVICE_BUDGET");
	ctx->budget = budget ? strtoull(budget, NULL, 10) : 0;
	int count = 0;
	int e = vkcu_device_count(&count);
	if (e != 0 || count <= ctx->device) {
		vkh_fail(NULL, VKHEL_ERR_NO_DEVICE, "context: no CUDA device %d (count %d, error %d)",
				ctx->device, count, e);
		free(ctx);
		return NULL;
	}
	if ((e = vkcu_set_device(ctx->device)) || (e = vkcu_sm_count(ctx->device, &ctx->sms)) ||
			(e = vkcu_stream_create(&ctx->stream)) || (e = vkcu_pool_create(ctx->device, &ctx->pool))) {
		vkh_cuda(NULL, e, "context creation");
		if (ctx->stream)
			vkcu_stream_destroy(ctx->stream);
		free(ctx);
		return NULL;
	}
	return ctx;
}

void vkhel_ctx_destroy(struct vkhel_ctx *ctx) {
	if (!ctx)
		return;
	vkcu_sync(ctx->stream);
	vkh_devtab_release_all(ctx);
	vkcu_sync(ctx->stream);
	vkcu_pool_destroy(ctx->pool);
	vkcu_stream_destroy(ctx->stream);
	free(ctx);
}

int vkhel_ctx_last_error(const struct vkhel_ctx *ctx, char *msg, size_t len) {
	const int code = ctx ? ctx->last_error : tls_error;
	if (msg && len) {
		snprintf(msg, len, "%s", ctx ? ctx->last_msg : tls_msg);
	}
	return code;
}

void vkhel_ctx_clear_error(struct vkhel_ctx *ctx) {
	if (ctx) {
		ctx->last_error = 0;
		ctx->last_msg[0] = 0;
	}
	tls_error = 0;
	tls_msg[0] = 0;
}

int vkhel_ctx_set_async(struct vkhel_ctx *ctx, int on) {
	if (!ctx)
		return vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "set_async: NULL context");
	if (ctx->async && !on) { /* back to blocking calls: nothing may still be queued */
		const int e = vkcu_sync(ctx->stream);
		ctx->async = 0;
		return vkh_cuda(ctx, e, "set_async: synchronize");
	}
	ctx->async = on != 0;
	return VKHEL_OK;
}

int vkhel_ctx_set_budget(struct vkhel_ctx *ctx, uint64_t bytes) {
	if (!ctx)
		return vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "set_budget: NULL context");
	ctx->budget = bytes;
	return VKHEL_OK;
}

uint64_t vkhel_ctx_bytes_in_use(const struct vkhel_ctx *ctx) { return ctx ? ctx->in_use : 0; }
void *vkhel_ctx_stream(struct vkhel_ctx *ctx) { return ctx ? ctx->stream : NULL; }
int vkhel_ctx_sm_count(const struct vkhel_ctx *ctx) { return ctx ? ctx->sms : 0; }
uint64_t vkhel_launch_count(void) { return vkcu_launch_count(); }

int vkhel_measure_int_peak(struct vkhel_ctx *ctx, double *bfly, double *imad) {
	if (!ctx || !bfly || !imad)
		return vkh_fail(ctx, VKHEL_ERR_INVALID_ARGUMENT, "measure_int_peak: NULL argument");
	return vkh_cuda(ctx, vkcu_measure_int_peak(ctx->stream, ctx->sms, bfly, imad), "measure_int_peak");
}

int vkhel_ctx_sync(struct vkhel_ctx *ctx) {
	if (!ctx)
		return vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "sync: NULL context");
	return vkh_cuda(ctx, vkcu_sync(ctx->stream), "stream synchronize");
}

/* ------------------------------------------------------------------ */
/* vectors                                                             */
/* ------------------------------------------------------------------ */

struct vkhel_vector *vkhel_vector_create(struct vkhel_ctx *ctx, uint64_t length) {
	return vkhel_vector_create2(ctx, length, true);
}

struct vkhel_vector *vkhel_vector_create2(struct vkhel_ctx *ctx, uint64_t length, bool zero) {
	if (!ctx) {
		vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "vector_create: NULL context");
		return NULL;
	}
	if (length > ((uint64_t) 1 << 40)) {
		vkh_fail(ctx, VKHEL_ERR_INVALID_ARGUMENT, "vector_create: length %" PRIu64 " too large", length);
		return NULL;
	}
	struct vkhel_vector *v = calloc(1, sizeof(*v));
	if (!v) {
		vkh_fail(ctx, VKHEL_ERR_OUT_OF_MEMORY, "vector_create: host allocation failed");
		return NULL;
	}
	v->ctx = ctx;
	v->length = length;
	v->bytes = (length ? length : 1) * sizeof(uint64_t);
	if (vkh_dev_alloc(ctx, v->bytes, (void **) &v->dev) != VKHEL_OK) {
		free(v);
		return NULL;
	}
	if (zero) {
		const int e = vkcu_memset0(ctx->stream, v->dev, v->bytes);
		if (e) {
			vkh_cuda(ctx, e, "vector_create: zero fill");
			vkh_dev_free(ctx, v->dev, v->bytes);
			free(v);
			return NULL;
		}
	}
	return v;
}

void vkhel_vector_destroy(struct vkhel_vector *v) {
	if (!v)
		return;
	vkh_dev_free(v->ctx, v->dev, v->bytes);
	if (v->window) {
		vkcu_sync(v->ctx->stream);
		vkcu_host_free(v->window);
	}
	free(v);
}

struct vkhel_vector *vkhel_vector_dup(struct vkhel_vector *src) {
	if (!src) {
		vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "vector_dup: NULL vector");
		return NULL;
	}
	struct vkhel_vector *v = vkhel_vector_create2(src->ctx, src->length, false);
	if (!v)
		return NULL;
	int e = vkcu_d2d(src->ctx->stream, v->dev, src->dev, src->length * sizeof(uint64_t));
	if (!e)
		e = vkcu_sync(src->ctx->stream);
	if (e) {
		vkh_cuda(src->ctx, e, "vector_dup");
		vkhel_vector_destroy(v);
		return NULL;
	}
	return v;
}

uint64_t vkhel_vector_length(const struct vkhel_vector *v) { return v ? v->length : 0; }
uint64_t *vkhel_vector_device_ptr(struct vkhel_vector *v) { return v ? v->dev : NULL; }

int vkhel_vector_upload(struct vkhel_vector *v, const uint64_t *src, uint64_t count) {
	if (!v || (!src && count))
		return vkh_fail(v ? v->ctx : NULL, VKHEL_ERR_INVALID_ARGUMENT, "upload: NULL argument");
	if (count > v->length)
		return vkh_fail(v->ctx, VKHEL_ERR_INVALID_ARGUMENT,
				"upload: %" PRIu64 " words into a vector of %" PRIu64, count, v->length);
	int e = vkcu_h2d(v->ctx->stream, v->dev, src, count * sizeof(uint64_t));
	if (!e)
		e = vkcu_sync(v->ctx->stream);
	return vkh_cuda(v->ctx, e, "upload");
}

int vkhel_vector_download(const struct vkhel_vector *v, uint64_t *dst, uint64_t count) {
	if (!v || (!dst && count))
		return vkh_fail(v ? v->ctx : NULL, VKHEL_ERR_INVALID_ARGUMENT, "download: NULL argument");
	if (count > v->length)
		return vkh_fail(v->ctx, VKHEL_ERR_INVALID_ARGUMENT,
				"download: %" PRIu64 " words from a vector of %" PRIu64, count, v->length);
	int e = vkcu_d2h(v->ctx->stream, dst, v->dev, count * sizeof(uint64_t));
	if (!e)
		e = vkcu_sync(v->ctx->stream);
	return vkh_cuda(v->ctx, e, "download");
}

int vkhel_vector_upload_async(struct vkhel_vector *v, const uint64_t *src, uint64_t count) {
	if (!v || (!src && count) || count > v->length)
		return vkh_fail(v ? v->ctx : NULL, VKHEL_ERR_INVALID_ARGUMENT, "upload_async: bad argument");
	return vkh_cuda(v->ctx, vkcu_h2d(v->ctx->stream, v->dev, src, count * sizeof(uint64_t)), "upload_async");
}

int vkhel_vector_download_async(const struct vkhel_vector *v, uint64_t *dst, uint64_t count) {
	if (!v || (!dst && count) || count > v->length)
		return vkh_fail(v ? v->ctx : NULL, VKHEL_ERR_INVALID_ARGUMENT, "download_async: bad argument");
	return vkh_cuda(v->ctx, vkcu_d2h(v->ctx->stream, dst, v->dev, count * sizeof(uint64_t)), "download_async");
}

/* Reference: map + memcpy + unmap (src/vector.c:262-268); one direct copy here. */
void vkhel_vector_copy_from_host(struct vkhel_vector *v, const uint64_t *e) {
	if (!v)
		return (void) vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "copy_from_host: NULL vector");
	vkhel_vector_upload(v, e, v->length);
}

/* Reference: src/vector.c:270-283 (staging buffer of `size` bytes, filled
 * from the device).  The window here is at least length * 8 bytes and holds
 * the whole vector, so unmap's write-back of length words is always defined. */
void vkhel_vector_map(struct vkhel_vector *v, void **mem, size_t size) {
	if (!v || !mem)
		return (void) vkh_fail(v ? v->ctx : NULL, VKHEL_ERR_INVALID_ARGUMENT, "map: NULL argument");
	*mem = NULL;
	const size_t need = size > v->length * sizeof(uint64_t) ? size : v->length * sizeof(uint64_t);
	if (v->window_bytes < need) {
		if (v->window) {
			vkcu_sync(v->ctx->stream);
			vkcu_host_free(v->window);
			v->window = NULL;
			v->window_bytes = 0;
		}
		const int e = vkcu_host_alloc(&v->window, need);
		if (e) {
			v->window = NULL;
			return (void) vkh_cuda(v->ctx, e, "map: pinned window");
		}
		v->window_bytes = need;
	}
	int e = vkcu_d2h(v->ctx->stream, v->window, v->dev, v->length * sizeof(uint64_t));
	if (!e)
		e = vkcu_sync(v->ctx->stream);
	if (e)
		return (void) vkh_cuda(v->ctx, e, "map: download");
	if (size > v->length * sizeof(uint64_t))
		memset((char *) v->window + v->length * sizeof(uint64_t), 0, size - v->length * sizeof(uint64_t));
	v->mapped = true;
	*mem = v->window;
}

/* Reference: src/vector.c:285-296 (writes length words back). */
void vkhel_vector_unmap(struct vkhel_vector *v) {
	if (!v || !v->mapped)
		return (void) vkh_fail(v ? v->ctx : NULL, VKHEL_ERR_INVALID_ARGUMENT, "unmap: vector not mapped");
	int e = vkcu_h2d(v->ctx->stream, v->dev, v->window, v->length * sizeof(uint64_t));
	if (!e)
		e = vkcu_sync(v->ctx->stream);
	v->mapped = false;
	vkh_cuda(v->ctx, e, "unmap: upload");
}

void vkhel_vector_dbgprint(const struct vkhel_vector *v) {
	if (!v)
		return;
	uint64_t *h = malloc(sizeof(uint64_t) * (v->length ? v->length : 1));
	if (!h || vkhel_vector_download(v, h, v->length) != VKHEL_OK) {
		free(h);
		return;
	}
	for (uint64_t i = 0; i < v->length; i++)
		printf(i + 1 == v->length ? "%" PRIu64 : "%" PRIu64 ", ", h[i]);
	printf("\n");
	free(h);
}

/* ------------------------------------------------------------------ */
/* element-wise operations                                             */
/* ------------------------------------------------------------------ */

static int check_ops(const char *op, const struct vkhel_vector *a, const struct vkhel_vector *b,
		const struct vkhel_vector *res, bool binary) {
	if (!a || !res || (binary && !b))
		return vkh_fail(res ? res->ctx : (a ? a->ctx : NULL), VKHEL_ERR_INVALID_ARGUMENT, "%s: NULL vector", op);
	/* src/vector.c:302 asserts one context for all operands */
	if (a->ctx != res->ctx || (b && b->ctx != res->ctx))
		return vkh_fail(res->ctx, VKHEL_ERR_INVALID_ARGUMENT, "%s: vectors belong to different contexts", op);
	/* the reference reads result->length words of every operand */
	if (a->length < res->length || (b && b->length < res->length))
		return vkh_fail(res->ctx, VKHEL_ERR_INVALID_ARGUMENT,
				"%s: operand shorter than result (%" PRIu64 ")", op, res->length);
	return VKHEL_OK;
}

int vkh_check_mod(struct vkhel_ctx *ctx, const char *op, uint64_t mod) {
	/* Barrett needs bitlen(mod) + 62 >= 64 (include/priv/numbers.h:7-9) */
	if (mod < 2)
		return vkh_fail(ctx, VKHEL_ERR_INVALID_ARGUMENT, "%s: modulus %" PRIu64 " < 2", op, mod);
	return VKHEL_OK;
}

/* End of a single call: wait for its kernels as the reference waits on its
 * fence (src/vector.c:326), unless the context is stream-ordered. */
static int finish(struct vkhel_ctx *ctx, int launch_err, const char *op) {
	int e = launch_err;
	if (!e && !ctx->async)
		e = vkcu_sync(ctx->stream);
	return vkh_cuda(ctx, e, op);
}

void vkhel_vector_elemfma(const struct vkhel_vector *a, const struct vkhel_vector *b,
		struct vkhel_vector *res, uint64_t multiplier, uint64_t mod) {
	if (check_ops("elemfma", a, b, res, true) || vkh_check_mod(res->ctx, "elemfma", mod))
		return;
	/* elemfma.c:159-161: Shoup factor of the multiplier, truncated */
	const uint64_t ms = vkh_shoup(multiplier, mod);
	finish(res->ctx, vkcu_elemfma(res->ctx->stream, res->dev, a->dev, b->dev, res->length, multiplier, ms, mod),
			"elemfma");
}

void vkhel_vector_elemfma_canonical(const struct vkhel_vector *a, const struct vkhel_vector *b,
		struct vkhel_vector *res, uint64_t multiplier, uint64_t mod) {
	if (check_ops("elemfma_canonical", a, b, res, true) || vkh_check_mod(res->ctx, "elemfma_canonical", mod))
		return;
	const uint64_t m = multiplier % mod;
	finish(res->ctx,
			vkcu_elemfma_canonical(res->ctx->stream, res->dev, a->dev, b->dev, res->length, m,
					vkh_shoup(m, mod), mod, vkh_barrett_mu(mod), (uint32_t) vkh_bitlen(mod)),
			"elemfma_canonical");
}

static void elemgtsub(struct vkhel_vector *res, const struct vkhel_vector *a, uint64_t bound,
		uint64_t diff, uint64_t mod) {
	const uint64_t mu = vkh_barrett_mu(mod);
	/* elemgtsub.comp:57 reduces diff in every invocation; it is uniform */
	const uint64_t d = vkh_ref_reduce64(diff, mod, mu);
	finish(res->ctx,
			vkcu_elemgtsub(res->ctx->stream, res->dev, a->dev, res->length, bound, d, mod, mu,
					(uint32_t) vkh_bitlen(mod)),
			"elemgtsub");
}

/* src/vector.c:360-368: mod 2 is the centred parity, others elemgtsub. */
void vkhel_vector_elemmod(const struct vkhel_vector *a, struct vkhel_vector *res, uint64_t mod, uint64_t q) {
	if (check_ops("elemmod", a, NULL, res, false))
		return;
	if (mod == 2) {
		finish(res->ctx, vkcu_elemmodbytwo(res->ctx->stream, res->dev, a->dev, res->length, q / 2), "elemmod");
		return;
	}
	if (vkh_check_mod(res->ctx, "elemmod", mod))
		return;
	elemgtsub(res, a, q / 2, q, mod);
}

void vkhel_vector_elemmul(const struct vkhel_vector *a, const struct vkhel_vector *b,
		struct vkhel_vector *res, uint64_t mod) {
	if (check_ops("elemmul", a, b, res, true) || vkh_check_mod(res->ctx, "elemmul", mod))
		return;
	finish(res->ctx,
			vkcu_elemmul(res->ctx->stream, res->dev, a->dev, b->dev, res->length, mod, vkh_barrett_mu(mod),
					(uint32_t) vkh_bitlen(mod)),
			"elemmul");
}

void vkhel_vector_elemgtadd(const struct vkhel_vector *a, struct vkhel_vector *res, uint64_t bound, uint64_t diff) {
	if (check_ops("elemgtadd", a, NULL, res, false))
		return;
	finish(res->ctx, vkcu_elemgtadd(res->ctx->stream, res->dev, a->dev, res->length, bound, diff), "elemgtadd");
}

void vkhel_vector_elemgtsub(const struct vkhel_vector *a, struct vkhel_vector *res, uint64_t bound, uint64_t diff,
		uint64_t mod) {
	if (check_ops("elemgtsub", a, NULL, res, false) || vkh_check_mod(res->ctx, "elemgtsub", mod))
		return;
	elemgtsub(res, a, bound, diff, mod);
}

/* ------------------------------------------------------------------ */
/* transforms                                                          */
/* ------------------------------------------------------------------ */

static int check_transform(const char *op, const struct vkhel_vector *a, const struct vkhel_vector *res,
		const struct vkhel_ntt_tables *t, const struct vkh_devtab **d) {
	if (!a || !res || !t)
		return vkh_fail(res ? res->ctx : (a ? a->ctx : NULL), VKHEL_ERR_INVALID_ARGUMENT, "%s: NULL argument", op);
	if (a->ctx != res->ctx)
		return vkh_fail(res->ctx, VKHEL_ERR_INVALID_ARGUMENT, "%s: vectors belong to different contexts", op);
	if (a->length < t->n || res->length < t->n)
		return vkh_fail(res->ctx, VKHEL_ERR_INVALID_ARGUMENT,
				"%s: vectors of %" PRIu64 "/%" PRIu64 " words for n=%" PRIu64, op, a->length, res->length, t->n);
	/* the reference's inverse-mod and butterfly sums hold below 2^63
	 * (src/numbers.c:71-99, nttfwdbutterfly.comp:44-57) */
	if (t->q >= ((uint64_t) 1 << 63) || t->q < 3)
		return vkh_fail(res->ctx, VKHEL_ERR_UNSUPPORTED, "%s: q=%" PRIu64 " outside [3, 2^63)", op, t->q);
	if (t->unreduced)
		return vkh_fail(res->ctx, VKHEL_ERR_UNSUPPORTED, "%s: a table entry is not below q=%" PRIu64, op, t->q);
	if (t->log_n > vkcu_max_log_n())
		return vkh_fail(res->ctx, VKHEL_ERR_UNSUPPORTED, "%s: n=%" PRIu64 " above 2^%u", op, t->n,
				vkcu_max_log_n());
	if (t->n == 1)
		return VKHEL_OK;
	return vkh_devtab_get(res->ctx, t, d);
}

static void forward_impl(const struct vkhel_vector *a, struct vkhel_vector *res, struct vkhel_ntt_tables *t) {
	const struct vkh_devtab *d = NULL;
	if (check_transform("forward_transform", a, res, t, &d))
		return;
	if (t->n == 1)
		return; /* the stage loop of src/vector.c:537 runs zero times */
	const vkcu_ntt_job job = {a->dev, res->dev, d->dev_set};
	finish(res->ctx, vkcu_ntt_forward(res->ctx->stream, NULL, 1, &job, t->log_n, vkcu_wide(t->q), res->ctx->sms),
			"forward_transform");
}

void vkhel_vector_forward_transform(const struct vkhel_vector *a, struct vkhel_vector *res,
		struct vkhel_ntt_tables *t) {
	vkcu_range_push("vkhel_vector_forward_transform");
	forward_impl(a, res, t);
	vkcu_range_pop();
}

static int inverse_impl(const struct vkhel_vector *a, struct vkhel_vector *res, struct vkhel_ntt_tables *t,
		const struct vkhel_lift_step *steps, uint32_t nsteps) {
	const struct vkh_devtab *d = NULL;
	int st = check_transform("inverse_transform", a, res, t, &d);
	if (st)
		return st;
	struct vkhel_ctx *ctx = res->ctx;
	vkcu_lift lift;
	if ((st = vkh_lift_compile(ctx, steps, nsteps, t->q, &lift)))
		return st;
	const vkcu_lift *lp = lift.count ? &lift : NULL;
	int e = 0;
	if (t->n > 1) {
		const vkcu_ntt_job job = {a->dev, res->dev, d->dev_set};
		e = vkcu_ntt_inverse_lift(ctx->stream, NULL, 1, &job, t->log_n, vkcu_wide(t->q), ctx->sms, lp);
	}
	/* src/vector.c:635-638 scales result->length words by n^-1: words past n
	 * (and, for n == 1, the untouched result) are scaled here. */
	const uint64_t from = t->n > 1 ? t->n : 0;
	if (!e && res->length > from)
		e = vkcu_elemmulconst(ctx->stream, res->dev + from, res->dev + from, res->length - from, t->ninv, t->ninv_s,
				t->q);
	if (!e && res->length > from)
		e = vkcu_lift_range(ctx->stream, res->dev + from, res->length - from, t->q, ctx->sms, lp);
	return finish(ctx, e, "inverse_transform");
}

void vkhel_vector_inverse_transform(const struct vkhel_vector *a, struct vkhel_vector *res,
		struct vkhel_ntt_tables *t) {
	vkcu_range_push("vkhel_vector_inverse_transform");
	inverse_impl(a, res, t, NULL, 0);
	vkcu_range_pop();
}

int vkhel_vector_inverse_transform_lift(const struct vkhel_vector *a, struct vkhel_vector *res,
		struct vkhel_ntt_tables *t, const struct vkhel_lift_step *steps, uint32_t nsteps) {
	vkcu_range_push("vkhel_vector_inverse_transform_lift");
	const int st = inverse_impl(a, res, t, steps, nsteps);
	vkcu_range_pop();
	return st;
}

/* The reference's element-wise ops as epilogue steps, with the constants its
 * host wrappers derive (src/vector.c:342-386, 429-511; the same derivations
 * as vkhel_vector_elemmod / elemgtsub / elemgtadd above). */
int vkh_lift_compile(struct vkhel_ctx *ctx, const struct vkhel_lift_step *steps, uint32_t nsteps, uint64_t q,
		vkcu_lift *out) {
	memset(out, 0, sizeof *out);
	if (nsteps == 0)
		return VKHEL_OK;
	if (!steps || nsteps > VKCU_MAX_LIFT)
		return vkh_fail(ctx, VKHEL_ERR_INVALID_ARGUMENT, "lift: %u steps (1..%d)", nsteps, VKCU_MAX_LIFT);
	for (uint32_t i = 0; i < nsteps; i++) {
		const struct vkhel_lift_step *s = &steps[i];
		vkcu_lift_step *d = &out->step[i];
		switch (s->op) {
		case VKHEL_LIFT_ELEMMOD: {
			const uint64_t qq = s->p1 ? s->p1 : q;
			const uint32_t tq = qq ? 0 : VKCU_LIFT_TABLE_Q;
			if (s->p0 == 2) {
				d->kind = VKCU_LIFT_MODTWO | tq;
				d->bound = qq / 2;
				break;
			}
			const int st = vkh_check_mod(ctx, "lift elemmod", s->p0);
			if (st)
				return st;
			d->kind = VKCU_LIFT_GTSUB | tq;
			d->mod = s->p0;
			d->mu = vkh_barrett_mu(s->p0);
			d->bits = (uint32_t) vkh_bitlen(s->p0);
			d->bound = qq / 2;
			d->d = vkh_ref_reduce64(qq, d->mod, d->mu);
			break;
		}
		case VKHEL_LIFT_ELEMGTSUB: {
			const int st = vkh_check_mod(ctx, "lift elemgtsub", s->p2);
			if (st)
				return st;
			d->kind = VKCU_LIFT_GTSUB;
			d->mod = s->p2;
			d->mu = vkh_barrett_mu(s->p2);
			d->bits = (uint32_t) vkh_bitlen(s->p2);
			d->bound = s->p0;
			d->d = vkh_ref_reduce64(s->p1, d->mod, d->mu);
			break;
		}
		case VKHEL_LIFT_ELEMGTADD:
			d->kind = VKCU_LIFT_GTADD;
			d->bound = s->p0;
			d->d = s->p1;
			break;
		default:
			return vkh_fail(ctx, VKHEL_ERR_INVALID_ARGUMENT, "lift: step %u has unknown op %u", i, s->op);
		}
	}
	out->count = nsteps;
	return VKHEL_OK;
}

static int polymul_impl(const struct vkhel_vector *a, const struct vkhel_vector *b, struct vkhel_vector *res,
		struct vkhel_ntt_tables *t, const struct vkhel_lift_step *steps, uint32_t nsteps, int b_ntt);

int vkhel_vector_polymul(const struct vkhel_vector *a, const struct vkhel_vector *b, struct vkhel_vector *res,
		struct vkhel_ntt_tables *t) {
	vkcu_range_push("vkhel_vector_polymul");
	const int st = polymul_impl(a, b, res, t, NULL, 0, 0);
	vkcu_range_pop();
	return st;
}

/* The reference's call pattern forward(a), elemmul(., NTT(b)), inverse with
 * NTT(b) kept from an earlier forward transform, in one call. */
int vkhel_vector_polymul_ntt(const struct vkhel_vector *a, const struct vkhel_vector *b_ntt,
		struct vkhel_vector *res, struct vkhel_ntt_tables *t) {
	vkcu_range_push("vkhel_vector_polymul_ntt");
	const int st = polymul_impl(a, b_ntt, res, t, NULL, 0, 1);
	vkcu_range_pop();
	return st;
}

int vkhel_vector_polymul_lift(const struct vkhel_vector *a, const struct vkhel_vector *b, struct vkhel_vector *res,
		struct vkhel_ntt_tables *t, const struct vkhel_lift_step *steps, uint32_t nsteps) {
	vkcu_range_push("vkhel_vector_polymul_lift");
	const int st = polymul_impl(a, b, res, t, steps, nsteps, 0);
	vkcu_range_pop();
	return st;
}

static int polymul_impl(const struct vkhel_vector *a, const struct vkhel_vector *b, struct vkhel_vector *res,
		struct vkhel_ntt_tables *t, const struct vkhel_lift_step *steps, uint32_t nsteps, int b_ntt) {
	const struct vkh_devtab *d = NULL;
	int st = check_transform("polymul", a, res, t, &d);
	if (st)
		return st;
	if (!b || b->ctx != res->ctx || b->length < t->n)
		return vkh_fail(res->ctx, VKHEL_ERR_INVALID_ARGUMENT, "polymul: bad operand b");
	/* the composed path writes the result before it reads NTT(b) */
	if (b_ntt && b->dev == res->dev)
		return vkh_fail(res->ctx, VKHEL_ERR_INVALID_ARGUMENT, "polymul_ntt: result aliases NTT(b)");
	struct vkhel_ctx *ctx = res->ctx;
	vkcu_lift lift;
	if ((st = vkh_lift_compile(ctx, steps, nsteps, t->q, &lift)))
		return st;
	const vkcu_lift *lp = lift.count ? &lift : NULL;
	const uint64_t bytes = t->n * sizeof(uint64_t);
	if (t->n == 1) {
		/* forward is a no-op at n = 1 and inverse scales by 1 */
		int e = vkcu_elemmul(ctx->stream, res->dev, a->dev, b->dev, 1, t->q, t->mu, t->qbits);
		if (!e)
			e = vkcu_lift_range(ctx->stream, res->dev, 1, t->q, ctx->sms, lp);
		return finish(ctx, e, "polymul");
	}
	uint64_t *scratch = b_ntt ? b->dev : res->dev;
	void *tmp = NULL;
	const int fused = t->log_n >= 8 && t->log_n <= vkcu_max_fused_log_n();
	/* NTT(b) is parked in the result vector unless that would overwrite a
	 * before it is read (the fused kernel reads a after writing NTT(b)), or
	 * the transform needs its own output buffer; a given NTT(b) needs none. */
	if (!b_ntt && (!fused || res->dev == a->dev)) {
		if ((st = vkh_dev_alloc(ctx, bytes, &tmp)))
			return st;
		scratch = tmp;
	}
	int e;
	if (fused) {
		const vkcu_poly_job job = {a->dev, b->dev, res->dev, scratch, d->dev_set, b_ntt ? VKCU_JOB_B_NTT : 0};
		e = vkcu_polymul_lift(ctx->stream, NULL, 1, &job, t->log_n, vkcu_wide(t->q), ctx->sms, lp, b_ntt);
	} else {
		const vkcu_ntt_job jb = {b->dev, scratch, d->dev_set};
		const vkcu_ntt_job ja = {a->dev, res->dev, d->dev_set};
		const vkcu_ntt_job jc = {res->dev, res->dev, d->dev_set};
		e = b_ntt ? 0 : vkcu_ntt_forward(ctx->stream, NULL, 1, &jb, t->log_n, vkcu_wide(t->q), ctx->sms);
		if (!e)
			e = vkcu_ntt_forward(ctx->stream, NULL, 1, &ja, t->log_n, vkcu_wide(t->q), ctx->sms);
		if (!e)
			e = vkcu_elemmul(ctx->stream, res->dev, res->dev, scratch, t->n, t->q, t->mu, t->qbits);
		if (!e)
			e = vkcu_ntt_inverse_lift(ctx->stream, NULL, 1, &jc, t->log_n, vkcu_wide(t->q), ctx->sms, lp);
	}
	st = finish(ctx, e, "polymul");
	if (tmp)
		vkh_dev_free(ctx, tmp, bytes);
	return st;
}
