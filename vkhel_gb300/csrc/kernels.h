/*
 * C ABI between the C host library (api.c, tables.c) and the CUDA side
 * (runtime.cu, elem.cu, ntt.cu).  Plain pointers and sizes only.  These
 * symbols are internal to libvkhel.so (the version script exports vkhel_*
 * only).
 */
#ifndef VKHEL_GB300_KERNELS_H
#define VKHEL_GB300_KERNELS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Device-resident constants of one (n, q, w) twiddle set.  `fwd` and `inv`
 * point to n interleaved (root, shoup(root)) pairs in the reference's
 * bit-reversed order (src/ntt_tables.c:25-43). */
typedef struct vkcu_twset {
	uint64_t q, q2, mu;          /* q, 2q, floor(2^(bits+62)/q) */
	uint64_t ninv, ninv_s;       /* n^-1 mod q and its Shoup factor */
	uint64_t w1ninv, w1ninv_s;   /* inv_roots[1] * n^-1 mod q and Shoup factor */
	uint32_t qbits, log_n;
	const uint64_t *fwd;
	const uint64_t *inv;
} vkcu_twset;

/* One transform of one vector.  The transform reads n words at `in` and
 * writes n words at `out` (which may equal `in`). */
typedef struct vkcu_ntt_job {
	const uint64_t *in;
	uint64_t *out;
	const vkcu_twset *tw;        /* device pointer */
} vkcu_ntt_job;

/* One negacyclic limb product c = a * b mod (X^n + 1, q).  `scratch` holds n
 * words for NTT(b) during the kernel; it may be `c` unless c overlaps a.
 * With VKCU_JOB_B_NTT in `flags`, b already holds NTT(b) (bit-reversed, as
 * the forward transform writes it; words reduced as elemmul reduces its
 * operands) and `scratch` is unused: c = INTT(NTT(a) . b). */
#define VKCU_JOB_B_NTT 1u
typedef struct vkcu_poly_job {
	const uint64_t *a;
	const uint64_t *b;
	uint64_t *c;
	uint64_t *scratch;
	const vkcu_twset *tw;        /* device pointer */
	uint64_t flags;              /* VKCU_JOB_* */
} vkcu_poly_job;

/* ---- runtime (runtime.cu) ---- */
int vkcu_device_count(int *count);
int vkcu_set_device(int device);
int vkcu_sm_count(int device, int *sms);
int vkcu_stream_create(void **stream);
int vkcu_stream_destroy(void *stream);
int vkcu_pool_create(int device, void **pool);
int vkcu_pool_destroy(void *pool);
int vkcu_pool_independent_streams(void *pool);
/* fn(arg) on a driver thread after the stream's earlier work (no CUDA calls in fn). */
int vkcu_launch_host_func(void *stream, void (*fn)(void *), void *arg);
/* Profiler ranges (NVTX) around entry points. */
void vkcu_range_push(const char *name);
void vkcu_range_pop(void);
int vkcu_alloc(void *pool, void *stream, size_t bytes, void **ptr);
int vkcu_free(void *stream, void *ptr);
int vkcu_memset0(void *stream, void *ptr, size_t bytes);
int vkcu_h2d(void *stream, void *dst, const void *src, size_t bytes);
int vkcu_d2h(void *stream, void *dst, const void *src, size_t bytes);
int vkcu_d2d(void *stream, void *dst, const void *src, size_t bytes);
int vkcu_sync(void *stream);
int vkcu_host_alloc(void **ptr, size_t bytes);
int vkcu_host_free(void *ptr);
const char *vkcu_error_string(int code);
uint64_t vkcu_launch_count(void);
void vkcu_count_launches(uint64_t n);
int vkcu_capture_begin(void *stream);
int vkcu_capture_end(void *stream, void **exec);
int vkcu_graph_launch(void *exec, void *stream);
int vkcu_graph_destroy(void *exec);
int vkcu_event_create(void **ev);
int vkcu_event_destroy(void *ev);
int vkcu_event_record(void *ev, void *stream);
int vkcu_stream_wait(void *stream, void *ev);
int vkcu_event_query(void *ev);
int vkcu_host_is_pinned(const void *p);

/* ---- element-wise kernels (elem.cu); `len` elements of `res` ---- */
int vkcu_elemmul(void *stream, uint64_t *res, const uint64_t *a,
		const uint64_t *b, uint64_t len, uint64_t mod, uint64_t mu, uint32_t bits);
int vkcu_elemmulconst(void *stream, uint64_t *res, const uint64_t *a,
		uint64_t len, uint64_t c, uint64_t c_shoup, uint64_t mod);
int vkcu_elemfma(void *stream, uint64_t *res, const uint64_t *a,
		const uint64_t *b, uint64_t len, uint64_t m, uint64_t m_shoup,
		uint64_t mod);
int vkcu_elemfma_canonical(void *stream, uint64_t *res, const uint64_t *a,
		const uint64_t *b, uint64_t len, uint64_t m_red, uint64_t m_shoup,
		uint64_t mod, uint64_t mu, uint32_t bits);
int vkcu_elemgtsub(void *stream, uint64_t *res, const uint64_t *a,
		uint64_t len, uint64_t bound, uint64_t diff_red, uint64_t mod,
		uint64_t mu, uint32_t bits);
int vkcu_elemgtadd(void *stream, uint64_t *res, const uint64_t *a,
		uint64_t len, uint64_t bound, uint64_t diff);
int vkcu_elemmodbytwo(void *stream, uint64_t *res, const uint64_t *a,
		uint64_t len, uint64_t signed_bound);

/* One job of an element-wise batch: res[i] = op(a[i], b[i]) for i < len,
 * with the op's constants as the single-vector launchers take them. */
enum {
	VKCU_ELEM_MUL = 1,        /* c0 mod, c1 mu, bits */
	VKCU_ELEM_MULCONST = 2,   /* c0 c, c1 c_shoup, c2 mod */
	VKCU_ELEM_FMA = 3,        /* c0 m, c1 m_shoup, c2 mod (reference wrap) */
	VKCU_ELEM_FMA_CANON = 4,  /* c0 m mod q, c1 m_shoup, c2 mod, c3 mu, bits */
	VKCU_ELEM_GTSUB = 5,      /* c0 bound, c1 reduced diff, c2 mod, c3 mu, bits */
	VKCU_ELEM_GTADD = 6,      /* c0 bound, c1 diff */
	VKCU_ELEM_MODTWO = 7      /* c0 signed bound */
};
typedef struct vkcu_elem_job {
	uint32_t op, bits;
	const uint64_t *a, *b;       /* b NULL for unary ops */
	uint64_t *res;
	uint64_t len;
	uint64_t c0, c1, c2, c3;
} vkcu_elem_job;
/* Words per work unit of the element-wise batch kernel: a batch is launched
 * as a table of units, each a vkcu_elem_job of at most this many words (the
 * jobs cut into pieces, pointers offset to each piece); unary ops take units
 * twice as long, so that every unit moves the same bytes. */
#define VKCU_ELEM_CHUNK 2048
#define VKCU_ELEM_CHUNK_UNARY 4096
int vkcu_elem_batch(void *stream, const vkcu_elem_job *units, uint64_t nunits, int sms);

/* Device twiddle generation (q < 2^61, w^n = -1): fwd/inv are n interleaved
 * (root, shoup) pairs; phi[j] = w^(j 2^lb), plo[k] = w^k for k < 2^lb. */
int vkcu_twiddles(void *stream, uint64_t *fwd, uint64_t *inv, const uint64_t *phi,
		const uint64_t *plo, uint32_t log_n, uint32_t lb, uint64_t q, uint64_t mu, uint32_t qbits);

/* Epilogue of an inverse transform or polymul: the reference's elemmod /
 * elemgtsub / elemgtadd applied in order to every output word.  With
 * VKCU_LIFT_TABLE_Q the step takes bound = q / 2 (and, for GTSUB, d = q
 * reduced mod `mod`) from the job's own modulus. */
enum { VKCU_LIFT_MODTWO = 1, VKCU_LIFT_GTSUB = 2, VKCU_LIFT_GTADD = 3 };
#define VKCU_LIFT_TABLE_Q 0x100u
#define VKCU_MAX_LIFT 4
typedef struct vkcu_lift_step {
	uint32_t kind, bits;         /* kind | VKCU_LIFT_TABLE_Q; bits = bitlen(mod) */
	uint64_t bound, d, mod, mu;  /* d: reduced diff (GTSUB) or diff (GTADD) */
} vkcu_lift_step;
typedef struct vkcu_lift {
	uint32_t count, pad;
	vkcu_lift_step step[VKCU_MAX_LIFT];
} vkcu_lift;

/* ---- transforms (ntt.cu) ----
 * `jobs` is a device array of `njobs` jobs that all share log_n and the
 * modulus class, or NULL to launch the single job `one` passed by value.
 * `wide` selects the class: 0 for q < 2^62 (lazy [0, 4q) butterflies), 1 for
 * 2^62 <= q < 2^63 ([0, 2q) butterflies). */
#define VKCU_WIDE_Q ((uint64_t) 1 << 62)
static inline int vkcu_wide(uint64_t q) { return q >= VKCU_WIDE_Q; }
int vkcu_ntt_forward(void *stream, const vkcu_ntt_job *jobs, int njobs,
		const vkcu_ntt_job *one, uint32_t log_n, int wide, int sms);
int vkcu_ntt_inverse(void *stream, const vkcu_ntt_job *jobs, int njobs,
		const vkcu_ntt_job *one, uint32_t log_n, int wide, int sms);
int vkcu_polymul(void *stream, const vkcu_poly_job *jobs, int njobs,
		const vkcu_poly_job *one, uint32_t log_n, int wide, int sms);
/* The same with an epilogue (`lift` NULL or count 0: none); fused into the
 * last pass for 2^8 <= n <= 2^17, a separate element-wise launch otherwise.
 * b_ntt: the jobs carry VKCU_JOB_B_NTT; only the epilogue instantiations of
 * the fused kernels read that flag, so such jobs run those (with no steps
 * when `lift` has none) and the plain kernels stay as lean as before. */
int vkcu_ntt_inverse_lift(void *stream, const vkcu_ntt_job *jobs, int njobs,
		const vkcu_ntt_job *one, uint32_t log_n, int wide, int sms, const vkcu_lift *lift);
int vkcu_polymul_lift(void *stream, const vkcu_poly_job *jobs, int njobs,
		const vkcu_poly_job *one, uint32_t log_n, int wide, int sms, const vkcu_lift *lift, int b_ntt);
/* The epilogue alone, in place on `len` words at p (modulus q for TABLE_Q
 * steps), or on the n output words of every job. */
int vkcu_lift_range(void *stream, uint64_t *p, uint64_t len, uint64_t q, int sms, const vkcu_lift *lift);
int vkcu_lift_jobs(void *stream, const vkcu_ntt_job *jobs, int njobs, const vkcu_ntt_job *one,
		uint32_t log_n, int sms, const vkcu_lift *lift);
/* c = c * scratch mod q for every job (both canonical forward-transform
 * outputs; the word the reference's elemmul stores): the pointwise step of a
 * polymul that is not fused. */
int vkcu_pointwise(void *stream, const vkcu_poly_job *jobs, int njobs,
		uint32_t log_n, int wide, int sms);
/* A ragged batch of fused limb products of degrees 2^12 .. 2^16 as one
 * persistent launch (ntt_ragged.cu): items in decreasing size, the first
 * n_cluster_items of kind 16 (one product of 2^16 on a cluster of four CTAs)
 * or 15 (two products of 2^15, one per CTA pair), then kinds 14 and 13 (one
 * product per CTA) and 12 (two products per CTA); job0 / job1 index `jobs`.
 * `counters` is two words of device memory the launch resets first. */
typedef struct vkcu_ragged_item {
	uint32_t kind;
	uint32_t job0, job1;
} vkcu_ragged_item;
int vkcu_polymul_ragged(void *stream, const vkcu_ragged_item *items, int n_cluster_items,
		int n_items, const vkcu_poly_job *jobs, unsigned *counters, int sms);

/* Kernel variant table (tuning.c): family 0 = fused polymul, 1 = forward,
 * 2 = inverse, 3 = batch options (log_n 0: concurrent degree classes, 1:
 * no split of single jobs over 8 CTAs, 2: ragged batches as one launch);
 * per degree and, for a launch of njobs jobs
 * on sms SMs, per job-count bucket (vkh_variant: the many-jobs entry). */
int vkh_variant(int family, int log_n);
int vkh_variant_jobs(int family, int log_n, long njobs, int sms);
/* Integer-pipe microbenchmarks (peak.cu). */
int vkcu_measure_int_peak(void *stream, int sms, double *bfly_per_s, double *imad_per_s);
/* Largest log_n of the single-launch kernels (one CTA up to 2^14, one
 * cluster up to 2^17), and the largest log_n handled at all (2^26: passes
 * over HBM plus 2^14-word sub-blocks). */
uint32_t vkcu_max_fused_log_n(void);
uint32_t vkcu_max_log_n(void);

#ifdef __cplusplus
}
#endif

#endif
