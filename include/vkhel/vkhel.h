/*
 * vkhel public C API -- GB300 (sm_103a) implementation.
 *
 * Drop-in for the reference's include/vkhel/vkhel.h (lolzballs/vkhel,
 * include/vkhel/vkhel.h:1-55): the same types and the same 18 functions with
 * the same signatures and argument meanings, exported from libvkhel.so under
 * the same version script (every vkhel_* symbol global, vkhel.syms:1-6).
 *
 * Semantics kept from the reference:
 *   - every call is synchronous: it returns after the device work finished
 *     (src/vector.c:326 and the other fence waits);
 *   - vectors are device-resident arrays of `length` uint64 words, zeroed by
 *     vkhel_vector_create (src/vector.c:206-229);
 *   - element-wise operations take their length from `result`
 *     (src/kernels/elemmul.c:164) and may run in place;
 *   - transforms are negacyclic: `w` is a primitive 2n-th root of unity mod q,
 *     the forward transform maps natural order to bit-reversed order, the
 *     inverse maps back and multiplies by n^-1 (src/vector.c:513-657);
 *   - results are bit-identical to the reference's shader arithmetic for every
 *     input it defines, including elemfma's wrap-around (vkhel_ext.h declares
 *     a canonical variant).
 *
 * Differences: failures that the reference turns into assert() aborts are
 * reported instead (NULL from constructors, a recorded error that
 * vkhel_ctx_last_error() returns); set VKHEL_STRICT=1 to abort like the
 * reference.  Unsupported transform parameters are rejected rather than
 * computed with undefined behaviour: n not a power of two or above 2^26,
 * q >= 2^63 (where the reference's inverse-mod and butterfly sums overflow,
 * src/numbers.c:71-99), and the rare 63-bit (n, q, w) whose table the
 * reference's builder leaves with an entry not below q.
 */
#ifndef VKHEL_H
#define VKHEL_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Context: one CUDA device (VKHEL_DEVICE, default 0), one stream, one device
 * memory pool.  Reference: vkhel.h:8-10, src/vkhel.c:4-13. */
struct vkhel_ctx;
struct vkhel_ctx *vkhel_ctx_create();
void vkhel_ctx_destroy(struct vkhel_ctx *);

/* Twiddle tables for degree n, modulus q and primitive 2n-th root w.  Built on
 * the host with the reference's arithmetic (src/ntt_tables.c:17-80); uploaded
 * once per context on first use and cached there per (n, q, w).
 * Reference: vkhel.h:12-15. */
struct vkhel_ntt_tables;
struct vkhel_ntt_tables *vkhel_ntt_tables_create(
		uint64_t n, uint64_t q, uint64_t w);
void vkhel_ntt_tables_destroy(struct vkhel_ntt_tables *);

/* Device vectors.  Reference: vkhel.h:17-25, src/vector.c:206-296.
 * map(v, &p, size) downloads the vector into a host window of at least
 * `size` bytes (and at least length * 8); unmap writes length words back. */
struct vkhel_vector;
struct vkhel_vector *vkhel_vector_create(struct vkhel_ctx *, uint64_t length);
struct vkhel_vector *vkhel_vector_create2(struct vkhel_ctx *, uint64_t length,
		bool zero);
void vkhel_vector_destroy(struct vkhel_vector *);
struct vkhel_vector *vkhel_vector_dup(struct vkhel_vector *);
void vkhel_vector_copy_from_host(struct vkhel_vector *, const uint64_t *);
void vkhel_vector_map(struct vkhel_vector *, void **, size_t);
void vkhel_vector_unmap(struct vkhel_vector *);

/* Element-wise operations.  Reference: vkhel.h:27-45, src/vector.c:298-511. */
void vkhel_vector_elemfma(
		const struct vkhel_vector *a,
		const struct vkhel_vector *b,
		struct vkhel_vector *result,
		uint64_t multiplier, uint64_t mod);
void vkhel_vector_elemmod(
		const struct vkhel_vector *a,
		struct vkhel_vector *result, uint64_t mod, uint64_t q);
void vkhel_vector_elemmul(
		const struct vkhel_vector *a,
		const struct vkhel_vector *b,
		struct vkhel_vector *result, uint64_t mod);
void vkhel_vector_elemgtadd(const struct vkhel_vector *operand,
		struct vkhel_vector *result,
		uint64_t bound, uint64_t diff);
void vkhel_vector_elemgtsub(
		const struct vkhel_vector *operand,
		struct vkhel_vector *result,
		uint64_t bound, uint64_t diff, uint64_t mod);

/* Transforms.  Reference: vkhel.h:46-53, src/vector.c:513-657. */
void vkhel_vector_forward_transform(
		const struct vkhel_vector *operand,
		struct vkhel_vector *result,
		struct vkhel_ntt_tables *ntt);
void vkhel_vector_inverse_transform(
		const struct vkhel_vector *operand,
		struct vkhel_vector *result,
		struct vkhel_ntt_tables *ntt);

#ifdef __cplusplus
}
#endif

#endif
