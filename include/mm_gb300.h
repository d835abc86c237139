/*
 * mm_gb300.h -- C ABI of the GB300-native Gaussian->Fock hot path.
 *
 * The library computes MrMustard's renormalised multidimensional Hermite
 * recurrence (Bargmann triple (A, b, c) -> Fock amplitudes G, complex128,
 * row-major), its closed-form vector-Jacobian product, and the Fock-space
 * contraction that follows it, with hand-written sm_103a CUDA kernels.
 *
 * Conventions (every entry point):
 *  - complex128 values are mm_c128 {re, im}: the layout of numpy complex128,
 *    C99 double _Complex and std::complex<double>.
 *  - Arrays named A, b, c, G, dLdG, dA, db, dc, U, X, Y are DEVICE pointers;
 *    `shape`, `D`, `shapes` are HOST arrays.  Tensors are C-contiguous.
 *  - Calls are asynchronous on `stream` (a cudaStream_t; NULL = legacy default).
 *  - `ws` is caller-owned device scratch of at least the size the matching
 *    *_workspace_bytes query returns, 256-byte aligned.  Its first 4 bytes
 *    are a sticky device status word: kernels that give up a bounded wait
 *    record MM_ERR_WAIT_TIMEOUT there.  Zero it once with mm_workspace_init and
 *    read it with mm_workspace_status.
 *  - Return value: MM_OK or an mm_status code; nothing aborts or traps.
 *  - There is no CPU fallback: without a CUDA device every compute entry
 *    point returns MM_ERR_NO_DEVICE.
 */
#ifndef MM_GB300_H
#define MM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define MM_API __attribute__((visibility("default")))
#else
#define MM_API
#endif

typedef struct {
  double re, im;
} mm_c128;

typedef struct CUstream_st *mm_stream_t; /* identical to cudaStream_t */

enum mm_status {
  MM_OK = 0,
  MM_ERR_INVALID_ARG = 1,   /* bad pointer, shape entry < 1, D < 1, ... */
  MM_ERR_UNSUPPORTED = 2,   /* D > mm_max_modes() */
  MM_ERR_TOO_LARGE = 3,     /* a slab of the recurrence exceeds 2^31 - 1 amplitudes, or (only from
                               mm_hermite_vjp_noalloc) its scratch exceeds MM_NOALLOC_SCRATCH_BYTES */
  MM_ERR_CUDA = 4,          /* a CUDA runtime call failed */
  MM_ERR_WAIT_TIMEOUT = 5,  /* a bounded inter-CTA wait gave up (device status word) */
  MM_ERR_WORKSPACE = 6,     /* workspace missing, misaligned or too small */
  MM_ERR_NO_DEVICE = 7      /* no CUDA device */
};

/* Human-readable text of a status code (static storage). */
MM_API const char *mm_status_string(int status);
/* Largest number of modes (tensor rank) an instance may have. */
MM_API int mm_max_modes(void);
/* Text of the last CUDA error seen by this thread (static storage, "" if none). */
MM_API const char *mm_last_cuda_error(void);

/* Zero the workspace status word (async on stream). */
MM_API int mm_workspace_init(void *ws, size_t ws_bytes, mm_stream_t stream);
/* Synchronise `stream`, read the workspace status word into *status and clear it. */
MM_API int mm_workspace_status(void *ws, mm_stream_t stream, int *status);

/* ------------------------------------------------------------------ forward */

/*
 * Workspace bytes for mm_hermite_fwd / _batched / mm_hermite_vjp / _batched
 * on `batch` instances of one shape (batch = 1 for the unbatched calls).
 */
MM_API size_t mm_hermite_workspace_bytes(int D, const int64_t *shape, int64_t batch);

/*
 * G = vanilla_numba(shape, A, b, c)            (stable = 0)
 * G = stable_numba(shape, A, b, c)             (stable != 0)
 * Replaces mrmustard/math/lattice/strategies/vanilla/core.py:25-124 (vanilla_numba)
 * and core.py:127-213 (stable_numba), reached from
 * mrmustard/math/backend_numpy.py:381-392 (BackendNumpy.hermite_renormalized).
 * A: D x D row-major, b: D, c: 1 element, G: prod(shape) elements (every one written).
 */
MM_API int mm_hermite_fwd(int D, const int64_t *shape, const mm_c128 *A, const mm_c128 *b, const mm_c128 *c, int stable,
                   mm_c128 *G, void *ws, size_t ws_bytes, mm_stream_t stream);

/*
 * G[k] = vanilla_numba / stable_numba(shape, A[k], b[k], c[k]) for k < B.
 * Replaces mrmustard/math/lattice/strategies/vanilla/batch.py:27-61 (vanilla_batch_numba),
 * reached from mrmustard/math/backend_numpy.py:394-403 (hermite_renormalized_batched).
 * A: B x D x D, b: B x D, c: B, G: B x prod(shape).
 */
MM_API int mm_hermite_fwd_batched(int64_t B, int D, const int64_t *shape, const mm_c128 *A, const mm_c128 *b,
                           const mm_c128 *c, int stable, mm_c128 *G, void *ws, size_t ws_bytes, mm_stream_t stream);

/*
 * vanilla_numba / stable_numba with HOST buffers in and out -- the call the reference's
 * numpy-in / numpy-out strategy makes (core.py:25-213): A (D x D), b (D), c (1) and G
 * (prod(shape)) are ordinary host memory.  The library stages them through a pinned buffer and a
 * device buffer of its own (allocated on first use per device, grown as needed, reused), runs
 * mm_hermite_fwd on `stream`, and returns after G has been copied back (one synchronisation,
 * which also reads the device status word).  Calls on one device are serialised.
 */
MM_API int mm_hermite_fwd_host(int D, const int64_t *shape, const mm_c128 *A, const mm_c128 *b, const mm_c128 *c,
                               int stable, mm_c128 *G, mm_stream_t stream);

/* ---------------------------------------------------------------------- VJP */

/*
 * (dA, db, dc) = vanilla_vjp_numba(G, c, dLdG): holomorphic VJP (no conjugation),
 * dA symmetrised as (dLdA + dLdA^T) / 2.
 * Replaces mrmustard/math/lattice/strategies/vanilla/gradients.py:25-82, reached from
 * mrmustard/math/jax_vjps/hermite.py:86-102 (hermite_renormalized_jax_bwd).
 * dA: D x D, db: D, dc: 1.
 */
MM_API int mm_hermite_vjp(int D, const int64_t *shape, const mm_c128 *G, const mm_c128 *c, const mm_c128 *dLdG, mm_c128 *dA,
                   mm_c128 *db, mm_c128 *dc, void *ws, size_t ws_bytes, mm_stream_t stream);

/*
 * Batched VJP over B instances of one shape.
 * Replaces mrmustard/math/lattice/strategies/vanilla/gradients.py:85-116
 * (vanilla_batch_vjp_numba), reached from mrmustard/math/jax_vjps/hermite.py:158-175.
 * dA: B x D x D, db: B x D, dc: B.
 */
MM_API int mm_hermite_vjp_batched(int64_t B, int D, const int64_t *shape, const mm_c128 *G, const mm_c128 *c,
                           const mm_c128 *dLdG, mm_c128 *dA, mm_c128 *db, mm_c128 *dc, void *ws, size_t ws_bytes,
                           mm_stream_t stream);

/*
 * Checkpointed VJP: vanilla_vjp_numba(G, c, dLdG) without G.  The JAX custom VJP keeps the
 * whole tensor G as its residual (mrmustard/math/jax_vjps/hermite.py:80-81); here the forward
 * keeps only checkpoint slabs along axis 0 and the backward recomputes the rest, segment by
 * segment, before running the stencil of gradients.py:25-82 on it.
 *  - Segments of K >= 2 slabs (slab m = every amplitude with k_0 = m, strides[0] of them);
 *    the checkpoint buffer holds slab 0, then slabs jK - 2 and jK - 1 for j = 1 .. nseg - 1
 *    (nseg = ceil(shape[0] / K)): mm_hermite_checkpoint_elems(D, shape, K) complex values,
 *    about 2 / K of G.
 *  - mm_hermite_checkpoint_save copies those slabs out of a forward's G (device to device).
 *  - mm_hermite_vjp_checkpointed takes A, b, c (for the recomputation), the checkpoints and
 *    the full cotangent; its workspace (mm_hermite_vjp_checkpointed_workspace_bytes) holds
 *    a window of K + 2 slabs, never all of G.  Vanilla recurrence only.
 * Results equal mm_hermite_vjp on the forward's G to rounding (the recomputed slabs follow
 * the forward's terms; the per-fiber sums are split at segment boundaries).
 * mm_hermite_checkpoint_elems returns -1 for a bad shape or K < 2.
 */
MM_API int64_t mm_hermite_checkpoint_elems(int D, const int64_t *shape, int K);
MM_API int mm_hermite_checkpoint_save(int D, const int64_t *shape, int K, const mm_c128 *G, mm_c128 *ckpt,
                                      mm_stream_t stream);
MM_API size_t mm_hermite_vjp_checkpointed_workspace_bytes(int D, const int64_t *shape, int K);
MM_API int mm_hermite_vjp_checkpointed(int D, const int64_t *shape, int K, const mm_c128 *A, const mm_c128 *b,
                                       const mm_c128 *c, const mm_c128 *ckpt, const mm_c128 *dLdG, mm_c128 *dA,
                                       mm_c128 *db, mm_c128 *dc, void *ws, size_t ws_bytes, mm_stream_t stream);

/*
 * mm_hermite_vjp without a workspace argument: the same kernels and results,
 * for callers that cannot allocate device memory when they call (for example a
 * custom-call handler inside another framework's runtime, which owns all
 * device memory and the stream, so a cudaMalloc there would synchronise the
 * device or escape the framework's memory accounting).  No counterpart in the
 * reference.
 *  - Scratch is an array of MM_NOALLOC_SCRATCH_BYTES (2 MiB) in the library's
 *    device memory, held by every GPU that loads the library until the process
 *    exits; shapes whose scratch (512-byte header, three sqrt tables of
 *    max(shape) + 1 doubles, 720 bytes of partial sums per work item) does not
 *    fit return MM_ERR_TOO_LARGE, which mm_hermite_vjp with a workspace would
 *    not.  Sufficient test before calling:
 *    mm_hermite_workspace_bytes(D, shape, 1) <= MM_NOALLOC_SCRATCH_BYTES.
 *    Nothing is allocated by the call.  Every argument is checked before the
 *    array is touched, so a rejected call changes nothing on the device.
 *  - The first call on a device looks up the array's device address
 *    (cudaGetSymbolAddress, with that device current) and keeps it for the
 *    life of the process; make that first call before any stream capture.
 *    cudaDeviceReset ends the context that address belongs to: do not call
 *    this entry point on a device after resetting it.
 *  - Every call uses the same array, so calls whose work overlaps on the GPU
 *    (other streams, other host threads) race: issue them in order on one
 *    stream.  The status word of the array is zeroed by each call.
 */
#define MM_NOALLOC_SCRATCH_BYTES (2u << 20)
MM_API int mm_hermite_vjp_noalloc(int D, const int64_t *shape, const mm_c128 *G, const mm_c128 *c,
                                  const mm_c128 *dLdG, mm_c128 *dA, mm_c128 *db, mm_c128 *dc, mm_stream_t stream);

/*
 * vanilla_vjp_numba(G, c, dLdG) with HOST buffers (G, dLdG: prod(shape); c: 1; dA: D x D; db: D;
 * dc: 1), staged like mm_hermite_fwd_host; returns after the gradients are back on the host.
 */
MM_API int mm_hermite_vjp_host(int D, const int64_t *shape, const mm_c128 *G, const mm_c128 *c, const mm_c128 *dLdG,
                               mm_c128 *dA, mm_c128 *db, mm_c128 *dc, mm_stream_t stream);

/* ------------------------------------------------------------ ragged batches */

/*
 * A ragged batch holds B instances with their own mode count D[k] and shape
 * (shapes[] concatenates the B shapes).  The reference has no ragged entry
 * point: its batch API (batch.py:27-61, backend_manager.py:683-720) needs one
 * shape, so a ragged batch there is a Python loop of vanilla_numba /
 * vanilla_vjp_numba calls; these entry points replace that loop with
 * persistent launches over a cost-sorted work queue.
 *
 * Packing (host offsets from mm_ragged_plan_offsets): instance k's tensor G_k
 * starts at element g_off[k] of G (and of dLdG), A_k at element a_off[k] of A
 * (D_k^2 entries), b_k at b_off[k] of b (D_k entries), c_k = c[k]; dA/db use
 * the a_off/b_off packing, dc[k] is one element per instance.
 */
typedef struct mm_ragged_plan mm_ragged_plan;

MM_API int mm_ragged_plan_create(int64_t B, const int32_t *D, const int64_t *shapes, mm_ragged_plan **plan);
MM_API void mm_ragged_plan_destroy(mm_ragged_plan *plan);
MM_API size_t mm_ragged_plan_workspace_bytes(const mm_ragged_plan *plan);
MM_API int64_t mm_ragged_plan_amplitudes(const mm_ragged_plan *plan);
/* Host arrays of B entries each (any may be NULL). */
MM_API int mm_ragged_plan_offsets(const mm_ragged_plan *plan, int64_t *g_off, int64_t *a_off, int64_t *b_off);
/*
 * Tuning knobs of the plan (set before mm_ragged_plan_upload):
 *   team_min_amps:  instances with at least this many amplitudes run their forward on a
 *                   cluster of CTAs instead of one CTA (0 = never);
 *   vjp_item_amps:  target amplitudes per VJP work item.
 */
MM_API int mm_ragged_plan_set_tuning(mm_ragged_plan *plan, int64_t team_min_amps, int64_t vjp_item_amps);
/* CTAs per cluster team for the large instances: 1 (no teams), 2, 4, 8 (default) or 16. */
MM_API int mm_ragged_plan_set_team_size(mm_ragged_plan *plan, int cluster_ctas);
/* Split of a host copy of G between mm_ragged_fwd_copy_g and mm_ragged_vjp_copy_g: instances k
 * with (k mod 8) < eighths get it from the forward, the others from the VJP (0..8, default 0).
 * A host-buffer step uses it to drive the host link during the forward too. */
MM_API int mm_ragged_plan_set_copy_split(mm_ragged_plan *plan, int eighths);
/* Copy the plan's descriptors and work queues into ws (blocks the host until copied). */
MM_API int mm_ragged_plan_upload(const mm_ragged_plan *plan, void *ws, size_t ws_bytes, mm_stream_t stream);

/* Forward of every instance of an uploaded plan (vanilla or stable). */
MM_API int mm_ragged_fwd(const mm_ragged_plan *plan, const mm_c128 *A, const mm_c128 *b, const mm_c128 *c, int stable,
                  mm_c128 *G, void *ws, size_t ws_bytes, mm_stream_t stream);
/* mm_ragged_fwd that also writes the forward's share (mm_ragged_plan_set_copy_split) of a copy
 * of G to G_copy, which may be pinned host memory; G_copy = NULL is mm_ragged_fwd.  (No
 * counterpart in the reference.) */
MM_API int mm_ragged_fwd_copy_g(const mm_ragged_plan *plan, const mm_c128 *A, const mm_c128 *b, const mm_c128 *c,
                                int stable, mm_c128 *G, mm_c128 *G_copy, void *ws, size_t ws_bytes,
                                mm_stream_t stream);
/* VJP of every instance of an uploaded plan.  G and dLdG may be any device-accessible
 * addresses, including pinned host memory (read by the kernels over the host link). */
MM_API int mm_ragged_vjp(const mm_ragged_plan *plan, const mm_c128 *G, const mm_c128 *c, const mm_c128 *dLdG, mm_c128 *dA,
                  mm_c128 *db, mm_c128 *dc, void *ws, size_t ws_bytes, mm_stream_t stream);
/* mm_ragged_vjp that also writes a copy of G to G_copy, which may be pinned host memory: the
 * VJP kernels store the G values they load anyway, so a host-buffer step gets G back over the
 * host link while the VJP runs, without a copy-engine transfer.  Every amplitude of the
 * instances outside the forward's share (mm_ragged_plan_set_copy_split; all of them by
 * default) is written once.  G_copy = NULL is mm_ragged_vjp.  (No counterpart in the reference.) */
MM_API int mm_ragged_vjp_copy_g(const mm_ragged_plan *plan, const mm_c128 *G, const mm_c128 *c, const mm_c128 *dLdG,
                                mm_c128 *dA, mm_c128 *db, mm_c128 *dc, mm_c128 *G_copy, void *ws, size_t ws_bytes,
                                mm_stream_t stream);

/* ------------------------------------------------------- Fock contraction */

/*
 * Y = U X for complex128 row-major U (M x K), X (K x N), Y (M x N): the dense
 * Fock-space contraction after the recurrence, e.g. a 2-mode gate's Fock tensor
 * reshaped to (c^2 x c^2) applied to a batch of kets stacked as columns.
 * Replaces ArrayAnsatz.contract -> math.einsum -> opt_einsum -> numpy
 * tensordot / BLAS zgemm (mrmustard/physics/ansatz/array_ansatz.py:159-226,
 * mrmustard/math/backend_manager.py:526-548).
 * mode MM_GEMM_FP64: native FP64 (DFMA).  mode MM_GEMM_FP64_DMMA: native FP64 on the
 * FP64 matrix-multiply instruction (mma.sync .f64).  mode MM_GEMM_OZAKI_BF16: FP64 values
 * split into `slices` (2..7) balanced 8-bit digits (each in [-128, 128]) per row
 * of U / column of X, digit products on the BF16 tensor cores with exact FP32
 * accumulation, recombined through integer sums and one FP64 scaling per slice
 * order; `slices` = 7 keeps 55 bits per operand.  ws: mm_fock_gemm_workspace_bytes
 * (256 bytes for the two FP64 modes).
 */
enum mm_gemm_mode { MM_GEMM_FP64 = 0, MM_GEMM_OZAKI_BF16 = 1, MM_GEMM_FP64_DMMA = 2 };
MM_API size_t mm_fock_gemm_workspace_bytes(int mode, int64_t M, int64_t N, int64_t K, int slices);
MM_API int mm_fock_gemm(int mode, int64_t M, int64_t N, int64_t K, const mm_c128 *U, const mm_c128 *X, mm_c128 *Y,
                        int slices, void *ws, size_t ws_bytes, mm_stream_t stream);

/* ------------------------------------------------------------- binomial fill */

/*
 * Fock tensor of one triple filled by total photon number with an L2 early
 * stop.  Replaces binomial(local_cutoffs, A, b, c, max_l2, global_cutoff)
 * (mrmustard/math/lattice/strategies/binomial.py:30-70), reached through
 * math.hermite_renormalized_binomial (mrmustard/math/backend_manager.py:790-814,
 * backend_numpy.py:405-421, which default max_l2 to AUTOSHAPE_PROBABILITY and
 * global_cutoff to sum(shape) - D + 1).
 * G (shape, C order) receives every amplitude of total photon number up to the
 * first weight w < global_cutoff after which the running sum of |G|^2 exceeds
 * max_l2 (or up to global_cutoff - 1), zeros elsewhere; *norm_out (device,
 * optional) that sum.  Pass max_l2 = +inf for no early stop.  Amplitudes equal
 * the vanilla recurrence's (same pivot rule).  ws: mm_binomial_workspace_bytes.
 * With a finite max_l2 only the weights up to the stop are computed, weight by
 * weight (one CTA, one thread-block cluster or a cooperative grid per weight,
 * picked from the weight's size); with max_l2 = +inf the vanilla forward fills
 * the tensor and the weights above global_cutoff - 1 are zeroed.
 */
MM_API size_t mm_binomial_workspace_bytes(int D, const int64_t *shape);
MM_API int mm_binomial(int D, const int64_t *shape, const mm_c128 *A, const mm_c128 *b, const mm_c128 *c,
                       double max_l2, int64_t global_cutoff, mm_c128 *G, double *norm_out, void *ws,
                       size_t ws_bytes, mm_stream_t stream);

/* ------------------------------------------------------------- autoshape */

/*
 * Per-mode Fock cutoffs of B Gaussian density-matrix triples with M modes each.
 * Replaces autoshape_numba(A, b, c, max_prob, max_shape, min_shape)
 * (mrmustard/math/lattice/autoshape.py:23-154), which State.auto_shape
 * (mrmustard/lab/states/base.py:383-430) calls on the triple of
 * `ansatz.conj & ansatz` with the settings AUTOSHAPE_PROBABILITY (0.99999),
 * AUTOSHAPE_MAX (50) and AUTOSHAPE_MIN (1).
 * A (B, 2M, 2M), b (B, 2M), c (B,): device complex128, variables ordered bra
 * copy then ket copy, as the reference reshapes them ((2, M, 2, M)).
 * shapes (B, M): device int64 output, shapes[s * M + m] = clip(k, min_shape,
 * max_shape) where k is the number of recurrence steps taken for mode m; a
 * state whose reduction is singular (the reference raises LinAlgError) gets -1
 * in every mode.  1 <= M <= 8; max_shape <= 99998 (the reference's sqrt table
 * ends at 99999; larger values return MM_ERR_TOO_LARGE).  No workspace;
 * asynchronous on `stream`.
 */
MM_API int mm_autoshape_batched(int64_t B, int M, const mm_c128 *A, const mm_c128 *b, const mm_c128 *c,
                                double max_prob, int64_t max_shape, int64_t min_shape, int64_t *shapes,
                                mm_stream_t stream);

/* ------------------------------------------------------------- diagonal strategies */

/*
 * Number of "slot" arrays of the diagonal strategy for M modes: the reference's
 * arr0 (1), arr2 (M), arr1010 (M (M-1)), arr1001 (M (M-1)) and arr1 (2M), stored back
 * to back in that order, each of P * nb values (P = prod cutoffs, params in C order,
 * batch index last) -- each one exactly the layout of the reference's array.
 */
MM_API int64_t mm_diagonal_slots(int M);
MM_API size_t mm_diagonal_workspace_bytes(int M, const int64_t *cutoffs, int64_t nb);

/*
 * Diagonal of the Fock representation (PNR amplitudes): replaces
 * fock_representation_diagonal_amps(A, B, G0, M, cutoffs)
 * (mrmustard/math/lattice/strategies/compactFock/diagonal_amps.py:217-248), reached
 * through hermite_multidimensional_diagonal (compactFock/inputValidation.py:61-79) and
 * math.hermite_renormalized_diagonal (mrmustard/math/backend_manager.py:729-757,
 * backend_numpy.py:423-432).  A (2M, 2M) and B (2M, nb) in the interleaved mode order
 * (mode0, mode0', mode1, ...), G0 (nb,): device complex128.  W receives
 * mm_diagonal_slots(M) * P * nb values; W[0 .. P*nb) is arr0 = G[k0,k0,k1,k1,...].
 * 1 <= M <= 8.  Asynchronous on `stream`; ws from mm_diagonal_workspace_bytes.
 */
MM_API int mm_diagonal_amps(int M, const int64_t *cutoffs, int64_t nb, const mm_c128 *A, const mm_c128 *B,
                            const mm_c128 *G0, mm_c128 *W, void *ws, size_t ws_bytes, mm_stream_t stream);

/*
 * Jacobians of every slot w.r.t. A and B: replaces fock_representation_diagonal_grad
 * (compactFock/diagonal_grad.py:261-378) behind grad_hermite_multidimensional_diagonal
 * (compactFock/inputValidation.py:82-100).  W: the slots of mm_diagonal_amps with nb = 1.
 * J receives mm_diagonal_slots(M) * P * (4M^2 + 2M) values, J[slot][point][d/dA (2M x 2M
 * row-major), then d/dB (2M)]; J[0 .. P*(4M^2+2M)) are arr0_dA and arr0_dB.  ws as for
 * mm_diagonal_workspace_bytes(M, cutoffs, 1).
 */
MM_API int mm_diagonal_jacobian(int M, const int64_t *cutoffs, const mm_c128 *A, const mm_c128 *B, const mm_c128 *W,
                                mm_c128 *J, void *ws, size_t ws_bytes, mm_stream_t stream);

/*
 * Vector-Jacobian product of the diagonal: dA = sum_k g_k arr0_dA[k], dB = sum_k g_k
 * arr0_dB[k], dG0 = sum_k g_k arr0[k] / G0 -- the contraction of
 * hermite_renormalized_diagonal_jax_bwd (mrmustard/math/jax_vjps/hermite.py:292-329).
 * J, W from the two calls above; g (P,) upstream; dA (2M, 2M), dB (2M,), dG0 (1,).
 */
MM_API int mm_diagonal_vjp(int M, const int64_t *cutoffs, const mm_c128 *J, const mm_c128 *W, const mm_c128 *G0,
                           const mm_c128 *g, mm_c128 *dA, mm_c128 *dB, mm_c128 *dG0, mm_stream_t stream);

/*
 * Leftover-mode strategy (M modes: mode 0 left over with cutoff q = cutoffs[0], modes
 * 1..M-1 photon-number resolved with cutoffs[1..]): replaces
 * fock_representation_1leftoverMode_amps (compactFock/singleLeftoverMode_amps.py:385-421) and
 * fock_representation_1leftoverMode_grad (singleLeftoverMode_grad.py:571-724), reached through
 * hermite_multidimensional_1leftoverMode / grad_hermite_multidimensional_1leftoverMode
 * (compactFock/inputValidation.py:103-142) and hermite_renormalized_1leftoverMode_jax
 * (mrmustard/math/jax_vjps/hermite.py:339-430, the JAX backend's path).
 * A (2M, 2M), B (2M) interleaved, G0 (1): device complex128.  W receives mm_leftover_slots(M)
 * slots (the diagonal strategy's slots over the M-1 detected modes) of q*q*P' values each,
 * [slot][m][n][params]; W[0 .. q*q*P') is arr0 (q, q, *cutoffs[1..]).  J receives
 * mm_leftover_slots(M) * q*q*P' * (4M^2 + 2M) values (Jacobian rows as for the diagonal).
 * 2 <= M <= 8, q <= 1000 (the reference's sqrt table).
 */
MM_API int64_t mm_leftover_slots(int M);
MM_API size_t mm_leftover_workspace_bytes(int M, const int64_t *cutoffs);
MM_API int mm_leftover_amps(int M, const int64_t *cutoffs, const mm_c128 *A, const mm_c128 *B, const mm_c128 *G0,
                            mm_c128 *W, void *ws, size_t ws_bytes, mm_stream_t stream);
MM_API int mm_leftover_jacobian(int M, const int64_t *cutoffs, const mm_c128 *A, const mm_c128 *B, const mm_c128 *W,
                                mm_c128 *J, void *ws, size_t ws_bytes, mm_stream_t stream);
/* dA = sum g * arr0_dA, dB = sum g * arr0_dB, dG0 = sum g * arr0 / G0 over the q*q*P' entries of arr0
 * (the contraction of hermite_renormalized_1leftoverMode_jax_bwd, jax_vjps/hermite.py:389-430). */
MM_API int mm_leftover_vjp(int M, const int64_t *cutoffs, const mm_c128 *J, const mm_c128 *W, const mm_c128 *G0,
                           const mm_c128 *g, mm_c128 *dA, mm_c128 *dB, mm_c128 *dG0, mm_stream_t stream);

MM_API size_t mm_fast_diagonal_workspace_bytes(int L, const int64_t *pnr_cutoffs, int64_t output_cutoff);

/*
 * Conditional density matrices of mode 0 with modes 1..L-1 photon-number resolved:
 * replaces fast_diagonal(A, b, c, output_cutoff, pnr_cutoffs, stable)
 * (mrmustard/math/lattice/strategies/fast_diagonal.py:32-77), which
 * backend_numpy.hermite_renormalized_1leftoverMode calls (backend_numpy.py:434-446).
 * A (2L, 2L), b (2L,), c (1,) in the caller's order (all first copies, then all second
 * copies); out: (pnr_1+1, ..., pnr_{L-1}+1, oc+1, oc+1) complex128, the layout
 * fast_diagonal returns (the backend transposes the last two axes to the front).
 * stable != 0 fills the first block with stable_numba instead of vanilla_numba.
 * Entries whose weight the reference's loop (range(1, 2 oc + 2 sum(pnr) - L)) never
 * reaches stay zero, as there.  2 <= L <= 8 (L = 1 returns MM_ERR_UNSUPPORTED).
 */
MM_API int mm_fast_diagonal(int L, const int64_t *pnr_cutoffs, int64_t output_cutoff, const mm_c128 *A,
                            const mm_c128 *b, const mm_c128 *c, int stable, mm_c128 *out, void *ws, size_t ws_bytes,
                            mm_stream_t stream);

/* ------------------------------------------------------------- Fock einsum building blocks */

/*
 * The pieces of a general pairwise Fock-space contraction, replacing what
 * ArrayAnsatz.contract (mrmustard/physics/ansatz/array_ansatz.py:159-226) reaches through
 * math.einsum (mrmustard/math/backend_manager.py:526-548) and opt_einsum: the slicing of the
 * contracted labels to a common dimension, the permutations, and the BLAS matrix product.
 * All complex128 device pointers, asynchronous on `stream`, no workspace.
 *
 * mm_tensor_permute: out (C order over out_shape, rank <= 16) gets
 *   out[i_0, ..., i_{r-1}] = in[in_offset + sum_k i_k * in_strides[k]]
 * -- any strided view (a permutation, a slice, the diagonal of a repeated label) made contiguous.
 */
MM_API int mm_tensor_permute(int rank, const int64_t *out_shape, const int64_t *in_strides, int64_t in_offset,
                             const mm_c128 *in, mm_c128 *out, mm_stream_t stream);
/* out[r] = sum_j in[r * inner + j] (a label summed inside one operand). */
MM_API int mm_tensor_sum_inner(int64_t rows, int64_t inner, const mm_c128 *in, mm_c128 *out, mm_stream_t stream);
/*
 * C[z] = A[z] @ B[z] for z < batch, row-major M x K, K x N, M x N blocks at element strides
 * strideA / strideB / strideC; FP64 arithmetic (GEMV kernels when N == 1 or M == 1; zeros when K == 0).
 */
MM_API int mm_zgemm_batched(int64_t batch, int64_t M, int64_t N, int64_t K, const mm_c128 *A, int64_t strideA,
                            const mm_c128 *B, int64_t strideB, mm_c128 *C, int64_t strideC, mm_stream_t stream);

/* ------------------------------------------------------------- diagnostics */

/*
 * Device self-test of the kernels' instance views: builds the per-instance
 * view of a one-shape batch and of a ragged batch on the device exactly as the
 * compute kernels do and compares every field with the host's values; *nbad
 * receives the number of mismatching fields (0 = pass).  Reads and writes only
 * the first 8 KiB of ws (at least that many bytes are required); synchronises
 * `stream`.  The Python layer runs it once per device before any compute call.
 * (No counterpart in the reference.)
 */
MM_API int mm_selftest(void *ws, size_t ws_bytes, mm_stream_t stream, int *nbad);

/*
 * Launch a two-CTA cooperative kernel whose grid barrier can never complete,
 * so that its bounded wait gives up after budget_ns and records
 * MM_ERR_WAIT_TIMEOUT in the workspace status word.  Used by the tests of the
 * timeout path; no GPU fault is involved.
 */
MM_API int mm_test_wait_timeout(void *ws, size_t ws_bytes, uint64_t budget_ns, mm_stream_t stream);

/*
 * FP64 pipe probe: `blocks` CTAs of 256 threads, each thread running 8 independent
 * DFMA chains of `iters` steps (2 * 8 * iters * blocks * 256 FLOP per launch); `out`
 * receives blocks * 256 doubles.  Gives the measured FP64 peak that the recurrence's
 * FP64 roofline is quoted against (no counterpart in the reference).
 */
MM_API int mm_probe_dfma(double *out, int blocks, int iters, mm_stream_t stream);

/*
 * Self-check of the division used by autoshape's recurrence (a / sqrt(k) as three
 * FP64 operations from a correctly rounded reciprocal, Markstein's theorem): n
 * pseudo-random quotients (seeded) are compared bit for bit with the correctly
 * rounded division; *bad (device, caller-zeroed) receives the number that differ.
 * Test infrastructure for the kernels' arithmetic; not a compute entry point.
 */
MM_API int mm_probe_division(int64_t n, uint64_t seed, unsigned long long *bad, mm_stream_t stream);

/* Number of kernel launches issued by this library since load (all threads). */
MM_API int64_t mm_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif /* MM_GB300_H */
