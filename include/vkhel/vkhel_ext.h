/*
 * vkhel extensions for GB300 -- declared beside the reference API.
 *
 * Everything here is exported by the same version script as the reference
 * API (every vkhel_* symbol is global).  None of it has a counterpart in the
 * reference's public header except where a line says so; the reference
 * reports failures through assert() only and has no batched or asynchronous
 * entry points.
 */
#ifndef VKHEL_EXT_H
#define VKHEL_EXT_H

#include "vkhel.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
enum vkhel_status {
	VKHEL_OK = 0,
	VKHEL_ERR_INVALID_ARGUMENT = 1, /* bad size, modulus, length or mismatched context */
	VKHEL_ERR_OUT_OF_MEMORY = 2,    /* device or pinned allocation failed */
	VKHEL_ERR_BUDGET = 3,           /* allocation would exceed the context budget */
	VKHEL_ERR_DEVICE = 4,           /* a CUDA call failed */
	VKHEL_ERR_NO_DEVICE = 5,        /* no CUDA device */
	VKHEL_ERR_TIMEOUT = 6,          /* a bounded wait ran out */
	VKHEL_ERR_CANCELLED = 7,        /* request cancelled before it ran */
	VKHEL_ERR_UNSUPPORTED = 8       /* valid request this library does not support */
};

/* ---- context ---- */
/* Status of the most recent failed call on this context (VKHEL_OK if none)
 * and its message (copied into msg[0..len)).  Calls made with a NULL context,
 * such as vkhel_ntt_tables_create, record into a per-thread slot read with
 * ctx == NULL. */
int vkhel_ctx_last_error(const struct vkhel_ctx *ctx, char *msg, size_t len);
void vkhel_ctx_clear_error(struct vkhel_ctx *ctx);
/* Device-memory budget in bytes for vectors and tables of this context
 * (0 = unlimited, the default; VKHEL_DEVICE_BUDGET sets it at creation). */
int vkhel_ctx_set_budget(struct vkhel_ctx *ctx, uint64_t bytes);
uint64_t vkhel_ctx_bytes_in_use(const struct vkhel_ctx *ctx);
/* The context's cudaStream_t, for interop and event timing. */
void *vkhel_ctx_stream(struct vkhel_ctx *ctx);
int vkhel_ctx_sync(struct vkhel_ctx *ctx);
int vkhel_ctx_sm_count(const struct vkhel_ctx *ctx);
/* Stream-ordered single calls (off by default; VKHEL_ASYNC=1 turns them on
 * for new contexts).  On, the transform, element-wise and polymul calls of
 * this context return once their kernels are enqueued on the context stream,
 * instead of after they finish as the reference's fence wait makes them:
 * consecutive calls then run back to back on the GPU.  Results are the same:
 * every call runs in order on one stream, and the calls that move data to
 * or from the host (copy_from_host, map, upload, download, dbgprint, dup)
 * and vkhel_ctx_sync wait for the work before them.  A kernel's device
 * error is reported by the next call that waits.  Turning it off waits for
 * the queued work. */
int vkhel_ctx_set_async(struct vkhel_ctx *ctx, int on);
/* Kernels launched by this library in this process (graph replays count
 * each kernel node once per replay). */
uint64_t vkhel_launch_count(void);
/* Integer-pipe peak of the context's GPU, measured now: independent lazy
 * Cooley-Tukey butterflies per second with all operands in registers (the
 * roofline denominator of the transform kernels) and 32-bit IMADs per
 * second.  Allocates and frees a few KB of device memory. */
int vkhel_measure_int_peak(struct vkhel_ctx *ctx, double *butterflies_per_s,
		double *imad_per_s);
/* Fault injection for tests (host side, process-wide): after `skip` more
 * device allocations by this library, the next `count` fail with
 * VKHEL_ERR_OUT_OF_MEMORY as if the device had run out of memory.
 * count = 0 switches it off. */
int vkhel_debug_fail_allocations(uint64_t skip, uint64_t count);

/* ---- vectors ---- */
uint64_t vkhel_vector_length(const struct vkhel_vector *v);
/* Device address of the vector's words (CUDA device pointer). */
uint64_t *vkhel_vector_device_ptr(struct vkhel_vector *v);
/* Synchronous copies of `count` words between host memory and the start of
 * the vector (count <= length). */
int vkhel_vector_upload(struct vkhel_vector *v, const uint64_t *src, uint64_t count);
int vkhel_vector_download(const struct vkhel_vector *v, uint64_t *dst, uint64_t count);
/* Stream-ordered variants: enqueue the copy on the context stream and return.
 * The host buffer must stay valid (and should be pinned for the copy to be
 * truly asynchronous) until vkhel_ctx_sync returns. */
int vkhel_vector_upload_async(struct vkhel_vector *v, const uint64_t *src, uint64_t count);
int vkhel_vector_download_async(const struct vkhel_vector *v, uint64_t *dst, uint64_t count);
/* Print the vector (reference: src/vector.c:237-247, exported there through
 * the vkhel_* glob of vkhel.syms). */
void vkhel_vector_dbgprint(const struct vkhel_vector *v);

/* ---- tables ---- */
/* Copy the host tables out (n words each; any pointer may be NULL). */
int vkhel_ntt_tables_copy(const struct vkhel_ntt_tables *t, uint64_t *roots,
		uint64_t *inv_roots, uint64_t *roots_shoup, uint64_t *inv_roots_shoup);
/* Reference: src/ntt_tables.c:46-63. */
void vkhel_ntt_tables_dbgprint(struct vkhel_ntt_tables *t);
/* Copy the context's device copy of the tables out (making it resident
 * first); equal to vkhel_ntt_tables_copy word for word. */
int vkhel_ntt_tables_device_copy(struct vkhel_ctx *ctx,
		const struct vkhel_ntt_tables *t, uint64_t *roots, uint64_t *inv_roots,
		uint64_t *roots_shoup, uint64_t *inv_roots_shoup);

/* ---- arithmetic ---- */
/* (a * multiplier + b) mod `mod`, canonical, for every 64-bit input: what
 * vkhel_vector_elemfma computes whenever the reference shader's wrap-around
 * (elemfma.comp:47-52) does not trigger. */
void vkhel_vector_elemfma_canonical(const struct vkhel_vector *a,
		const struct vkhel_vector *b, struct vkhel_vector *result,
		uint64_t multiplier, uint64_t mod);
/* Negacyclic product result = a * b mod (X^n + 1, q) of the first n words,
 * equal to the reference composition forward(a), forward(b), elemmul,
 * inverse.  One fused launch for 256 <= n <= 131072 (one CTA, or a cluster
 * of CTAs sharing the polynomial through distributed shared memory).
 * Returns a status. */
int vkhel_vector_polymul(const struct vkhel_vector *a,
		const struct vkhel_vector *b, struct vkhel_vector *result,
		struct vkhel_ntt_tables *ntt);
/* The same product with b given in the transform domain: b_ntt holds NTT(b)
 * as vkhel_vector_forward_transform writes it (bit-reversed order), e.g. a
 * key or plaintext transformed once and reused.  Equal to the reference
 * composition forward(a), elemmul(., b_ntt), inverse, so b_ntt's words need
 * not be reduced (elemmul reduces its operands).  One transform fewer per
 * product.  result may alias a, not b_ntt.  Returns a status. */
int vkhel_vector_polymul_ntt(const struct vkhel_vector *a,
		const struct vkhel_vector *b_ntt, struct vkhel_vector *result,
		struct vkhel_ntt_tables *ntt);

/* ---- centred-lift epilogues ----
 * Up to VKHEL_MAX_LIFT_STEPS of the reference's element-wise ops applied, in
 * order, to the output of an inverse transform or polymul, inside the same
 * kernel for 256 <= n <= 131072 (a separate element-wise launch otherwise).
 * Results equal calling the reference functions one after another on the
 * result vector (src/vector.c:342-386, 429-511):
 *   VKHEL_LIFT_ELEMMOD    p0 = mod, p1 = q          vkhel_vector_elemmod
 *   VKHEL_LIFT_ELEMGTSUB  p0 = bound, p1 = diff, p2 = mod   vkhel_vector_elemgtsub
 *   VKHEL_LIFT_ELEMGTADD  p0 = bound, p1 = diff     vkhel_vector_elemgtadd
 * ELEMMOD with p1 = 0 takes q from the transform's tables (in a batch, from
 * each limb's tables): the BFV-style centred reduction of every limb. */
enum vkhel_lift_op {
	VKHEL_LIFT_ELEMMOD = 1,
	VKHEL_LIFT_ELEMGTSUB = 2,
	VKHEL_LIFT_ELEMGTADD = 3
};
#define VKHEL_MAX_LIFT_STEPS 4
struct vkhel_lift_step {
	uint32_t op;
	uint64_t p0, p1, p2;
};
/* vkhel_vector_polymul, then the steps on the n result words. */
int vkhel_vector_polymul_lift(const struct vkhel_vector *a,
		const struct vkhel_vector *b, struct vkhel_vector *result,
		struct vkhel_ntt_tables *ntt, const struct vkhel_lift_step *steps,
		uint32_t nsteps);
/* vkhel_vector_inverse_transform, then the steps on every result word (the
 * reference's element-wise ops cover the whole result vector). */
int vkhel_vector_inverse_transform_lift(const struct vkhel_vector *a,
		struct vkhel_vector *result, struct vkhel_ntt_tables *ntt,
		const struct vkhel_lift_step *steps, uint32_t nsteps);

/* Same product as vkhel_vector_polymul without allocating any device memory
 * (no counterpart in the reference).  For callers that cannot let the library
 * allocate where they multiply -- a program whose device memory is all held
 * by its own allocator or a fixed per-tenant reservation, or a latency-
 * critical loop that must not call cudaMalloc / cudaFree, which can wait for
 * queued device work -- the kernel's NTT(b) scratch is a static device array
 * of 16384 words (128 KiB per device, kept until exit) instead of a pool
 * buffer.  Needs 256 <= n <= 16384 (other sizes: VKHEL_ERR_UNSUPPORTED) and
 * the tables already resident on the context through an earlier transform,
 * polymul or batch call with them (otherwise VKHEL_ERR_INVALID_ARGUMENT).
 * All calls share the array: calls that overlap on the GPU race.  The first
 * call on a device looks up the array's address and first launches the
 * kernel for its degree; make it during set-up, before any stream capture.
 * Synchronous; returns a status. */
int vkhel_vector_polymul_noalloc(const struct vkhel_vector *a,
		const struct vkhel_vector *b, struct vkhel_vector *result,
		const struct vkhel_ntt_tables *ntt);

/* ---- batched polynomial multiply and transforms ----
 * A batch is a fixed list of limb products, built once, committed (the job
 * table is uploaded and, with VKHEL_BATCH_GRAPH, the launch sequence is
 * captured in a CUDA graph), then launched any number of times.  Jobs of
 * different degrees may be mixed; each degree class runs in its own kernel
 * inside the same graph.  Operand memory is read at launch time, so new data
 * in the same vectors is picked up by every launch; the vectors must outlive
 * the batch (it keeps their device addresses, not references). */
struct vkhel_batch;
enum vkhel_batch_flags {
	VKHEL_BATCH_GRAPH = 1   /* capture and replay a CUDA graph */
};
struct vkhel_batch *vkhel_batch_create(struct vkhel_ctx *ctx);
/* Add `limbs` limb products of one RNS polynomial: limb k uses tables[k] and
 * the n words at offset k * n of a, b and c (vectors of >= limbs * n words). */
int vkhel_batch_add_polymul(struct vkhel_batch *batch,
		struct vkhel_ntt_tables *const *tables, uint32_t limbs,
		const struct vkhel_vector *a, const struct vkhel_vector *b,
		struct vkhel_vector *c);
/* Same with raw device pointers (32-byte aligned, limb-major). */
int vkhel_batch_add_polymul_raw(struct vkhel_batch *batch,
		struct vkhel_ntt_tables *const *tables, uint32_t limbs,
		const uint64_t *a, const uint64_t *b, uint64_t *c);
/* Limb products with b in the transform domain (vkhel_vector_polymul_ntt):
 * limb k of b_ntt holds NTT(b_k) for tables[k]; c must not overlap b_ntt. */
int vkhel_batch_add_polymul_ntt(struct vkhel_batch *batch,
		struct vkhel_ntt_tables *const *tables, uint32_t limbs,
		const struct vkhel_vector *a, const struct vkhel_vector *b_ntt,
		struct vkhel_vector *c);
int vkhel_batch_add_polymul_ntt_raw(struct vkhel_batch *batch,
		struct vkhel_ntt_tables *const *tables, uint32_t limbs,
		const uint64_t *a, const uint64_t *b_ntt, uint64_t *c);
/* Transforms of `limbs` limbs: limb k of `out` (n words at offset k n) =
 * the forward or inverse transform of limb k of `in` with tables[k], equal
 * to vkhel_vector_forward_transform / vkhel_vector_inverse_transform of that
 * limb (in place when in == out).  An inverse may carry a centred-lift
 * epilogue (steps, as vkhel_batch_add_polymul_lift; nsteps 0 for none). */
enum vkhel_transform_direction {
	VKHEL_TRANSFORM_FORWARD = 0,
	VKHEL_TRANSFORM_INVERSE = 1
};
int vkhel_batch_add_transform(struct vkhel_batch *batch,
		struct vkhel_ntt_tables *const *tables, uint32_t limbs,
		const struct vkhel_vector *in, struct vkhel_vector *out,
		uint32_t direction, const struct vkhel_lift_step *steps,
		uint32_t nsteps);
/* vkhel_batch_add_polymul with a centred-lift epilogue on every limb. */
int vkhel_batch_add_polymul_lift(struct vkhel_batch *batch,
		struct vkhel_ntt_tables *const *tables, uint32_t limbs,
		const struct vkhel_vector *a, const struct vkhel_vector *b,
		struct vkhel_vector *c, const struct vkhel_lift_step *steps,
		uint32_t nsteps);
int vkhel_batch_commit(struct vkhel_batch *batch, uint32_t flags);
/* Enqueue one run on the context stream and return (asynchronous). */
int vkhel_batch_launch(struct vkhel_batch *batch);
/* Launch and wait. */
int vkhel_batch_run(struct vkhel_batch *batch);
uint32_t vkhel_batch_jobs(const struct vkhel_batch *batch);
/* Kernels one launch of the batch issues (known after commit for a graph
 * batch, after the first launch otherwise: commit itself runs nothing). */
uint32_t vkhel_batch_kernels(const struct vkhel_batch *batch);
void vkhel_batch_destroy(struct vkhel_batch *batch);

/* ---- element-wise batch ----
 * Many independent element-wise jobs of ragged lengths, each one of the
 * reference's element-wise ops on its own vectors, run as one kernel launch
 * (optionally replayed from a CUDA graph).  Each job gives exactly what the
 * matching single call gives; jobs run concurrently, so commit rejects a
 * batch in which a job writes memory that another job reads or writes (a job
 * may work in place).  No counterpart in the reference. */
enum vkhel_elem_op {
	VKHEL_ELEM_FMA = 1,           /* p0 multiplier, p1 mod: vkhel_vector_elemfma */
	VKHEL_ELEM_FMA_CANONICAL = 2, /* p0 multiplier, p1 mod: vkhel_vector_elemfma_canonical */
	VKHEL_ELEM_MUL = 3,           /* p0 mod: vkhel_vector_elemmul */
	VKHEL_ELEM_MULCONST = 4,      /* p0 multiplier, p1 mod: the inverse transform's
	                               * n^-1 scaling kernel (src/vector.c:635-638) */
	VKHEL_ELEM_MOD = 5,           /* p0 mod, p1 q: vkhel_vector_elemmod */
	VKHEL_ELEM_GTADD = 6,         /* p0 bound, p1 diff: vkhel_vector_elemgtadd */
	VKHEL_ELEM_GTSUB = 7          /* p0 bound, p1 diff, p2 mod: vkhel_vector_elemgtsub */
};
struct vkhel_elem_batch;
struct vkhel_elem_batch *vkhel_elem_batch_create(struct vkhel_ctx *ctx);
/* result->length words, as the single call; b is ignored by unary ops. */
int vkhel_elem_batch_add(struct vkhel_elem_batch *batch, uint32_t op,
		uint64_t p0, uint64_t p1, uint64_t p2, const struct vkhel_vector *a,
		const struct vkhel_vector *b, struct vkhel_vector *result);
/* Same on raw device pointers (8-byte aligned) of `len` words. */
int vkhel_elem_batch_add_raw(struct vkhel_elem_batch *batch, uint32_t op,
		uint64_t p0, uint64_t p1, uint64_t p2, const uint64_t *a,
		const uint64_t *b, uint64_t *result, uint64_t len);
/* flags: VKHEL_BATCH_GRAPH to capture the launch into a CUDA graph. */
int vkhel_elem_batch_commit(struct vkhel_elem_batch *batch, uint32_t flags);
int vkhel_elem_batch_launch(struct vkhel_elem_batch *batch);
int vkhel_elem_batch_run(struct vkhel_elem_batch *batch);
uint32_t vkhel_elem_batch_jobs(const struct vkhel_elem_batch *batch);
void vkhel_elem_batch_destroy(struct vkhel_elem_batch *batch);

/* ---- kernel variants (autotuning) ----
 * Each fused kernel family has, per degree 2^log_n, a few compiled variants
 * (threads per polynomial, radix-16 groups in flight per thread); the table
 * of which one to launch is read once per process from $VKHEL_TUNE_TABLE or
 * from tuning/gb300.txt beside the package (written by vkhel_gb300.autotune).
 * Family VKHEL_TUNE_BATCH, log_n 0: 1 = run the degree classes of a batch on
 * concurrent streams; log_n 1: 1 = never split a few n = 2^12 .. 2^16 jobs
 * (at most one per 8 SMs, e.g. a single call) over clusters (the default, 0,
 * splits them: over 16 CTAs for n >= 2^14 with at most one job per 16 SMs,
 * otherwise over 8); log_n 2: 1 = run a ragged batch of fused products of
 * 2^12 .. 2^16 as one persistent launch; log_n 3: 1 = split over 8 CTAs
 * only. */
enum vkhel_tune_family {
	VKHEL_TUNE_POLYMUL = 0,
	VKHEL_TUNE_FORWARD = 1,
	VKHEL_TUNE_INVERSE = 2,
	VKHEL_TUNE_BATCH = 3
};
int vkhel_tune_set(uint32_t family, uint32_t log_n, int32_t variant);
int vkhel_tune_get(uint32_t family, uint32_t log_n);
int vkhel_tune_load(const char *path);

/* ---- serving: continuous batching of polynomial-multiply requests ----
 * A server owns a private context (device VKHEL_DEVICE), three streams and a
 * scheduler thread.  Requests (limbs limb products of one degree with host
 * operands a, b and host result c, limb-major, limbs * n words each) can be
 * submitted from any thread; they are admitted in arrival order while the
 * device budget allows, grouped into micro-batches of mixed degrees, and run
 * with uploads, compute and downloads of consecutive micro-batches
 * overlapping.  Host buffers must stay valid until the request is waited for;
 * pinned host memory makes the copies asynchronous.  Each result equals the
 * plain API's (forward, forward, elemmul, inverse per limb). */
struct vkhel_server;
struct vkhel_server_config {
	uint64_t device_budget;        /* bytes for in-flight requests (0: 40 GiB) */
	uint32_t max_batch_limbs;      /* limb products per micro-batch (0: 1024) */
	uint32_t max_inflight_batches; /* micro-batches on the device at once (0: 3) */
};
struct vkhel_server_stats {
	uint64_t submitted, completed, failed, batches, limbs;
	double span_s;                 /* first submission to last completion */
	double mean_ms, p50_ms, p99_ms, max_ms; /* request latency, submit -> done */
};
struct vkhel_server *vkhel_server_create(const struct vkhel_server_config *cfg);
/* Returns a request id > 0, or -status. */
int64_t vkhel_server_submit(struct vkhel_server *s,
		struct vkhel_ntt_tables *const *tables, uint32_t limbs,
		const uint64_t *a, const uint64_t *b, uint64_t *c);
/* Cancels request `id` if it is still queued (not yet in a micro-batch): its
 * wait then returns VKHEL_ERR_CANCELLED.  Fails with INVALID_ARGUMENT for a
 * request that is running, finished, collected or unknown. */
int vkhel_server_cancel(struct vkhel_server *s, int64_t id);
/* Waits up to timeout_ms for request `id`; returns its status, or
 * VKHEL_ERR_TIMEOUT (the request stays pending and can be waited for again).
 * After a non-timeout return the id is collected and cannot be waited again. */
int vkhel_server_wait(struct vkhel_server *s, int64_t id, uint32_t timeout_ms);
/* Resident operands: `limbs` limb polynomials that many requests multiply by
 * (a key, a plaintext), uploaded once and kept on the server's device in the
 * transform domain.  b holds b (is_ntt 0: transformed on the device) or
 * NTT(b) as vkhel_vector_forward_transform writes it (is_ntt 1), limb-major;
 * it is read before the call returns.  Returns an operand id > 0, or
 * -status.  The upload runs in queue order on the scheduler. */
int64_t vkhel_server_add_operand(struct vkhel_server *s,
		struct vkhel_ntt_tables *const *tables, uint32_t limbs,
		const uint64_t *b, int is_ntt);
/* A request c = a * b with b the resident operand `operand`, whose limbs must
 * have these tables' (n, q, w): only a is uploaded.  Returns a request id,
 * or -status; wait for it as for vkhel_server_submit. */
int64_t vkhel_server_submit_operand(struct vkhel_server *s,
		struct vkhel_ntt_tables *const *tables, uint32_t limbs,
		const uint64_t *a, int64_t operand, uint64_t *c);
/* Frees a resident operand; INVALID_ARGUMENT while queued or running
 * requests still read it (wait for them first) or for an unknown id. */
int vkhel_server_remove_operand(struct vkhel_server *s, int64_t operand);
int vkhel_server_stats(struct vkhel_server *s, struct vkhel_server_stats *out);
int vkhel_server_reset_stats(struct vkhel_server *s);
/* Runs the remaining queue to completion, then frees everything. */
void vkhel_server_destroy(struct vkhel_server *s);

#ifdef __cplusplus
}
#endif

#endif
