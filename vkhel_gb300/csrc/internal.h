/*
 * Internal types of libvkhel's C host layer.
 */
#ifndef VKHEL_GB300_INTERNAL_H
#define VKHEL_GB300_INTERNAL_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#include "../../include/vkhel/vkhel_ext.h"
#include "kernels.h"

#ifdef __cplusplus
extern "C" {
#endif

/* CUDA translation units compile with hidden visibility; public entry points
 * defined there are marked with this (the version script then keeps only
 * vkhel_* symbols). */
#define VKHEL_EXPORT __attribute__((visibility("default")))

/* Device copy of one (n, q, w) table set, cached in a context. */
struct vkh_devtab {
	struct vkh_devtab *next;
	uint64_t n, q, w;
	void *mem;                 /* pool allocation: twset struct + 2 tables */
	uint64_t bytes;
	const vkcu_twset *dev_set; /* device address of the twset struct */
	vkcu_twset host_set;       /* same values, device pointers */
};

struct vkhel_ctx {
	int device;
	int sms;
	void *stream;
	void *pool;
	uint64_t budget;           /* 0 = unlimited */
	uint64_t in_use;
	int strict;                /* abort on error like the reference's asserts */
	int async;                 /* single calls return once enqueued (vkhel_ctx_set_async) */
	int last_error;
	char last_msg[256];
	struct vkh_devtab *tabs;
};

struct vkhel_vector {
	struct vkhel_ctx *ctx;
	uint64_t length;
	uint64_t *dev;
	uint64_t bytes;            /* bytes charged to the context */
	void *window;              /* pinned host window of map/unmap */
	size_t window_bytes;
	bool mapped;
};

struct vkhel_ntt_tables {
	uint64_t n, q, w;
	uint32_t log_n;
	/* host arrays, the reference's layout (include/priv/ntt_tables.h:6-15);
	 * computed on first use when the device can generate the tables */
	uint64_t *roots, *inv_roots, *roots_shoup, *inv_roots_shoup;
	int host_ready;
	/* q < 2^61, n >= 2 and w^n = -1: generated on the device */
	int device_gen;
	/* some root or inverse root is not below q (only 63-bit moduli, whose
	 * Barrett products in the reference's table builder can overflow): the
	 * transforms refuse these tables */
	int unreduced;
	uint64_t w_red; /* w mod q */
	/* derived constants for the device twiddle set */
	uint64_t mu, ninv, ninv_s, w1ninv, w1ninv_s;
	uint32_t qbits;
};

/* numbers.c -- host number theory with the reference's formulas */
uint64_t vkh_bitlen(uint64_t v);
uint64_t vkh_shoup(uint64_t factor, uint64_t mod);
uint64_t vkh_barrett_mu(uint64_t mod);
uint64_t vkh_ref_reduce64(uint64_t x, uint64_t mod, uint64_t mu);
uint64_t vkh_mulmod(uint64_t a, uint64_t b, uint64_t mod);
uint64_t vkh_powmod(uint64_t base, uint64_t exp, uint64_t mod);
uint64_t vkh_invmod(uint64_t a, uint64_t mod);

/* api.c -- error reporting; returns `code` */
int vkh_fail(struct vkhel_ctx *ctx, int code, const char *fmt, ...);
int vkh_cuda(struct vkhel_ctx *ctx, int cuda_err, const char *what);
int vkh_dev_alloc(struct vkhel_ctx *ctx, uint64_t bytes, void **ptr);
void vkh_dev_free(struct vkhel_ctx *ctx, void *ptr, uint64_t bytes);
/* tables.c -- device table cache */
int vkh_devtab_get(struct vkhel_ctx *ctx, const struct vkhel_ntt_tables *t,
		const struct vkh_devtab **out);
void vkh_devtab_release_all(struct vkhel_ctx *ctx);
/* api.c -- 1 when the test fault injector fails this device allocation */
int vkh_inject_alloc_failure(void);
/* api.c -- modulus check of the element-wise ops (mod >= 2) */
int vkh_check_mod(struct vkhel_ctx *ctx, const char *op, uint64_t mod);
/* api.c -- centred-lift steps to the device form; q = 0 leaves ELEMMOD's
 * modulus to each job's tables */
int vkh_lift_compile(struct vkhel_ctx *ctx, const struct vkhel_lift_step *steps, uint32_t nsteps, uint64_t q,
		vkcu_lift *out);
/* batch.c -- degree classes of a sorted job list, shared with the server */
enum { VKH_JOB_POLYMUL = 0, VKH_JOB_FORWARD = 1, VKH_JOB_INVERSE = 2 };
struct vkh_job_class {
	uint32_t kind;         /* VKH_JOB_*; transform jobs keep in / out / tables in a, c, tw */
	uint32_t log_n;
	uint32_t first, count;
	int fused;
	int wide;              /* modulus class of every job: 2^62 <= q < 2^63 */
	uint32_t lift;         /* index into the lift table, 0 = none */
	uint32_t b_ntt;        /* polymul jobs whose b holds NTT(b) (VKCU_JOB_B_NTT) */
};
/* lifts: table indexed by vkh_job_class.lift (NULL when no class has one) */
int vkh_issue_classes(void *stream, int sms, const vkcu_poly_job *dev_poly, const vkcu_ntt_job *dev_ntt,
		const struct vkh_job_class *classes, uint32_t nclasses, const vkcu_lift *lifts);
int vkh_issue_classes_forked(void *stream, void *const *aux, void *fork, void *const *join, int sms,
		const vkcu_poly_job *dev_poly, const vkcu_ntt_job *dev_ntt, const struct vkh_job_class *classes,
		uint32_t nclasses, const vkcu_lift *lifts);
void vkh_fill_ntt_jobs(const vkcu_poly_job *poly, vkcu_ntt_job *ntt, const struct vkh_job_class *classes,
		uint32_t nclasses);
/* tuning.c -- variant of kernel family (VKHEL_TUNE_*) for degree 2^log_n */
int vkh_variant(int family, int log_n);
int vkh_variant_jobs(int family, int log_n, long njobs, int sms);
/* Lookup only: NULL when (n, q, w) has no device copy in ctx yet. */
const struct vkh_devtab *vkh_devtab_find(const struct vkhel_ctx *ctx, const struct vkhel_ntt_tables *t);

#ifdef __cplusplus
}
#endif

#endif
