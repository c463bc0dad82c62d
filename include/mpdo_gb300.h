/*
 * mpdo_gb300.h -- C ABI of the GB300-native MPDO noisy-circuit engine.
 *
 * Plain C: opaque handles, host pointers to small parameter arrays, sizes.
 * No torch or CUDA-runtime types appear in the signatures (streams are passed
 * as void*).  Every call returns an mpdo_status; mpdo_last_error() gives the
 * message of the last failing call on the calling thread.
 *
 * Each entry point replaces one operation of the reference's MPDO path
 * (paths relative to the WeiguoMa/Tomography-assisted-MPDO-QCircuit root):
 *
 *   mpdo_chain_create      Tools.py:110-198 create_ket*Series (product state)
 *   mpdo_apply_1q          Circuit.py:138-178 _apply_single_qubit_gate
 *   mpdo_apply_2q          Circuit.py:74-136  _apply_two_qubits_gate
 *   mpdo_truncate          Circuit.py:476-481 truncate layer =
 *                          TNNOptimizer.py:72-84 bondTruncate (qr_left2right
 *                          87-108 + svd_right2left 111-134) and
 *                          TNNOptimizer.py:164-197 svdKappa_left2right
 *   mpdo_kappa_truncate    TNNOptimizer.py:164-197 (the final pass of
 *                          Circuit.py:487-489)
 *   mpdo_reduced_dm        Circuit.py:226-295 cal_dm / _contract_dm
 *   mpdo_probs             Tools.py:242-273 density2prob (diagonal of cal_dm)
 *   mpdo_expect_ops        dmOperations.py:135-201 expect / pauli_expect
 *                          (single-site operator products)
 *   mpdo_expect_pauli_batch  many pauli_expect terms sharing one pass
 *   mpdo_trace_rho_rho     dmOperations.py:51-132 trace_rho_rho / purities
 *   mpdo_sample            Circuit.py:297-446 sample (conditional sampling)
 *   mpdo_sample_schemes    Circuit.py:448-466 randomSample (many schemes)
 *
 * Layout of a site tensor in device memory: complex, row-major
 * A[l][s][a][r] (l left bond, s physical = 2, a Kraus leg I_k, r right bond).
 * Complex numbers crossing the ABI are interleaved (re, im) doubles.
 */
#ifndef MPDO_GB300_H
#define MPDO_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MPDO_ABI_VERSION 1

typedef enum {
  MPDO_OK = 0,
  MPDO_ERR_INVALID = 1,        /* bad argument (reference: ValueError) */
  MPDO_ERR_BAD_SHAPE = 2,      /* inconsistent tensor shapes */
  MPDO_ERR_OOM = 3,            /* device allocation failed */
  MPDO_ERR_CUDA = 4,           /* a CUDA runtime call failed */
  MPDO_ERR_NOT_CONVERGED = 5,  /* Jacobi hit its sweep limit (reference: LinAlgError) */
  MPDO_ERR_NONFINITE = 6,      /* NaN/Inf met in a factorisation (reference: LinAlgError) */
  MPDO_ERR_NO_DEVICE = 7       /* no usable CUDA device */
} mpdo_status;

typedef enum { MPDO_C64 = 0, MPDO_C128 = 1 } mpdo_dtype;

typedef struct mpdo_engine_s *mpdo_engine_t;
typedef struct mpdo_chain_s *mpdo_chain_t;

int mpdo_abi_version(void);
const char *mpdo_status_string(mpdo_status s);
const char *mpdo_last_error(void);

/* One engine per device: owns the stream, the stream-ordered memory pool and
 * the workspaces.  Not thread-safe per handle. */
mpdo_status mpdo_engine_create(int device, mpdo_engine_t *out);
mpdo_status mpdo_engine_destroy(mpdo_engine_t eng);
/* stream: a cudaStream_t, or NULL for the engine's own stream. */
mpdo_status mpdo_engine_set_stream(mpdo_engine_t eng, void *stream);
/* Engine options (no counterpart in the reference; they select between
 * equivalent evaluation orders):
 *   "fuse_2q"    1 (default): a 2q gate followed by truncate() is fused into
 *                the QR sweep; 0: always split theta by SVD first (the
 *                reference's exact sequence, including its split cutoff).
 *   "defer_1q"   1 (default): a trace-preserving 1q Kraus map (sum K^H K = I)
 *                is kept pending on its site (composed with later ones while
 *                K <= 16) and applied when the site is next read; a truncate
 *                sweeps the pre-gate sites, which gives the same R factors and
 *                left singular vectors.  0: applied at once.
 *   "wide_range" on bonds too wide for one CTA, first try a verified
 *                randomized range finder (accepted only when the residual
 *                outside its span is at rounding level, so the triplets are
 *                those of an exact SVD): 1 always, 0 never (Gram +
 *                block-Jacobi path only), -1 (default) complex128 only.
 *   "wide_range_tol" acceptance factor of the range finder: the residual must
 *                be <= factor * eps * sqrt(p) * |Y|_F (default 8, rounding level).
 *   "wide_eig"   the exact wide-bond path diagonalises the Gram matrix by
 *                Householder tridiagonalisation on a thread-block cluster +
 *                bisection / inverse iteration (1), or by block Jacobi (0);
 *                -1 (default): tridiagonal for complex128; in complex64
 *                block Jacobi below "wide_eig_from" columns (default 257)
 *                and tridiagonal from there.  Both are followed by a
 *                Rayleigh-Ritz refinement in the leading
 *                (want + wide_oversample) directions.
 *   "bjacobi_bs" block width (columns per block) of the wide-bond block
 *                Jacobi, capped by shared memory; 0 (default) picks
 *                max(8, n / 16) up to 32.
 *   "bjacobi_fused" 1 (default): the block Jacobi runs as one launch on a
 *                thread-block cluster (one CTA per block pair, at most 16)
 *                that stops on the device after the first sweep without a
 *                rotation (at most 40 sweeps); 0, or where the cluster does
 *                not fit: one launch per tournament round and a host read of
 *                the rotation flag after every sweep.  Same columns either way.
 *   "tsqr_ratio" TSQR chunks hold at least this many times the column count
 *                in rows (shared memory when they fit, else global memory);
 *                default 3, so every level shrinks the stacked R threefold.
 *   "wide_oversample" extra Rayleigh-Ritz directions of a wide bond beyond
 *                the kept count (default 16).
 *   "max_sweeps" Jacobi sweep limit (default 60). */
mpdo_status mpdo_engine_set_option(mpdo_engine_t eng, const char *name, double value);
/* Wait for all queued work; returns the first deferred device status
 * (NOT_CONVERGED / NONFINITE) raised since the last sync. */
mpdo_status mpdo_engine_sync(mpdo_engine_t eng);
/* Per-kernel-class timing (no counterpart in the reference).  While enabled,
 * every launch is bracketed by CUDA events on the engine stream and its
 * algorithmic flop and byte counts are accumulated.  Classes: 0 GEMM,
 * 1 Householder QR factor, 2 QR explicit-Q apply, 3 one-sided Jacobi,
 * 4 Kraus 1q apply, 5 two-site gate mix, 6 other, 8 block Jacobi of wide
 * bonds (one launch per eigen-solve; one per round with bjacobi_fused = 0;
 * class 3 is the single-CTA Jacobi).  Class 7 returns counters
 * instead: launches = wide bonds solved by the range finder, flops = wide
 * bonds solved by the exact block Jacobi, bytes = the largest accepted relative
 * residual |Y - Q Q^H Y|_F / |Y|_F, ms = wide bonds whose exact path used the
 * tridiagonal eigensolver.  Classes 9-12 are phases (launches = count, ms =
 * summed span): 9 QR sweep, 10 SVD sweep, 11 kappa pass, 12 the wide-bond
 * SVDs inside the SVD sweep.  Class 13: cluster tridiagonalisation of
 * wide-bond Gram matrices.  Enabling resets the sums. */
mpdo_status mpdo_engine_profile(mpdo_engine_t eng, int enable);
mpdo_status mpdo_engine_profile_read(mpdo_engine_t eng, int kclass, long long *launches, double *ms,
                                     double *flops, double *bytes);
/* Number of kernels this library launched so far (all engines). */
mpdo_status mpdo_engine_launch_count(mpdo_engine_t eng, uint64_t *count);
/* Launches so far per launcher function, as text lines "name count\n"
 * (truncated to len-1 characters). */
mpdo_status mpdo_launch_histogram(char *buf, int len);

/* Product state.  vectors: n x 2 complex (4n doubles).  connected != 0 adds
 * dimension-1 bonds between all neighbours (the reference's check_connected
 * is then true from the start); otherwise bonds appear with the first 2q gate
 * on each pair, as in the reference. */
mpdo_status mpdo_chain_create(mpdo_engine_t eng, int n, int dtype, const double *vectors,
                              int connected, mpdo_chain_t *out);
mpdo_status mpdo_chain_destroy(mpdo_chain_t ch);
mpdo_status mpdo_chain_clone(mpdo_chain_t src, mpdo_chain_t *out);
mpdo_status mpdo_chain_num_sites(mpdo_chain_t ch, int *n);
/* dims = {l, s, a, r} of one site (after any deferred work is applied). */
mpdo_status mpdo_chain_site_dims(mpdo_chain_t ch, int site, int dims[4]);
mpdo_status mpdo_chain_bond_present(mpdo_chain_t ch, int bond, int *present);
/* Copy a site tensor to host: l*2*a*r complex (interleaved doubles). */
mpdo_status mpdo_chain_read_site(mpdo_chain_t ch, int site, double *host_out);
/* Replace a site tensor from host (dims = {l, 2, a, r}). */
mpdo_status mpdo_chain_write_site(mpdo_chain_t ch, int site, const int dims[4],
                                  const double *host_in);
/* The same two copies with a caller's DEVICE buffer, so that a site crosses
 * the boundary without a host round trip.  They replace the reads and writes
 * of Node.tensor on the reference's state nodes (AbstractCircuit.py:115-116
 * hands them out, Tools.py:44-72 names their legs), which hold torch tensors
 * on the circuit's device.  The buffer holds l*2*a*r complex values in the
 * chain's own precision, row-major [l][s][a][r]: interleaved floats for
 * complex64 chains, interleaved doubles for complex128 chains.  It must be
 * device or managed memory of the engine's device.  A host pointer or
 * another device's memory is rejected with MPDO_ERR_INVALID.  The copy runs
 * on the engine's stream.  The call returns once it has completed, so the
 * caller may reuse its buffer at once.  Work on other streams that produces
 * dev_in must be complete before the call. */
mpdo_status mpdo_chain_read_site_device(mpdo_chain_t ch, int site, void *dev_out);
mpdo_status mpdo_chain_write_site_device(mpdo_chain_t ch, int site, const int dims[4],
                                         const void *dev_in);

/* Gate (K = 1) or noisy gate (K Kraus operators) on one qubit.
 * kraus: [out][in][k] complex, 2*2*K entries.  The Kraus leg is flattened
 * into I_site after the existing one (Circuit.py:174-178). */
mpdo_status mpdo_apply_1q(mpdo_chain_t ch, int site, const double *kraus, int K);

/* Gate on the nearest-neighbour pair (site_min, site_min + 1).
 * kraus: [o_min][o_max][i_min][i_max][k] complex, 16*K entries; the Kraus leg
 * goes to I_{site_min+1} (Circuit.py:109-114).  abs_cutoff: the absolute
 * singular-value cutoff of the split (GLOBAL_MINIMUM in the reference). */
mpdo_status mpdo_apply_2q(mpdo_chain_t ch, int site_min, const double *kraus, int K,
                          double abs_cutoff);

/* truncate() layer.  chi <= 0: no bond cap; kappa <= 0: no Kraus cap;
 * max_err < 0: no error rule; noisy != 0 runs the kappa pass.  Skipped
 * entirely while the chain is not connected (TNNOptimizer.py:51-61).
 * discarded_out (nullable, n-1 doubles): per-bond discarded weight
 * sum(s_rest^2)/sum(s^2) of the SVD sweep. */
mpdo_status mpdo_truncate(mpdo_chain_t ch, int chi, int kappa, double max_err, int noisy,
                          double *discarded_out);
mpdo_status mpdo_kappa_truncate(mpdo_chain_t ch, int kappa, double max_err);

/* The reference's sweeps one at a time on a connected chain:
 *   mpdo_qr_left2right   TNNOptimizer.py:87-108 (reduced QR per site, R absorbed
 *                        into the next site; no truncation)
 *   mpdo_svd_right2left  TNNOptimizer.py:111-134 and
 *   mpdo_svd_left2right  TNNOptimizer.py:137-161: per bond, the SVD of the
 *                        contracted pair keeping <= chi values (chi <= 0: no
 *                        cap) and the relative error rule (max_err < 0: none),
 *                        sqrt(S) on both factors.  The pair is decomposed
 *                        exactly without forming it (QR / LQ of the other
 *                        site first).  discarded_out (nullable, n-1 doubles):
 *                        per-bond discarded weight. */
mpdo_status mpdo_qr_left2right(mpdo_chain_t ch);
mpdo_status mpdo_svd_right2left(mpdo_chain_t ch, int chi, double max_err, double *discarded_out);
mpdo_status mpdo_svd_left2right(mpdo_chain_t ch, int chi, double max_err, double *discarded_out);

/* Reduced density matrix on `keep` (m ascending qubit indices; m <= 14):
 * 2^m x 2^m complex, rows = ket (qubit keep[0] most significant). */
mpdo_status mpdo_reduced_dm(mpdo_chain_t ch, const int *keep, int m, double *host_out);
/* dmOperations.py:51-66 trace_rho_rho: Re Tr(rho_a rho_b), both states traced
 * over the qubits not in `keep` (m ascending indices, any m <= n), without
 * forming either density matrix (four-layer environment sweep; the largest
 * intermediate holds bond^4 x 2 x Kraus-leg elements).  a and b may be the
 * same chain; they need the same n and precision. */
mpdo_status mpdo_trace_rho_rho(mpdo_chain_t a, mpdo_chain_t b, const int *keep, int m, double *out);
/* Diagonal of the reduced density matrix (real parts), 2^m doubles (m <= 24). */
mpdo_status mpdo_probs(mpdo_chain_t ch, const int *keep, int m, double *host_out);
/* Re Tr(rho . prod_j O_j): ops is m x (2x2 complex) [row][col], on distinct
 * sites; identity elsewhere.  Not normalised by Tr(rho). */
mpdo_status mpdo_expect_ops(mpdo_chain_t ch, const int *sites, const double *ops, int m,
                            double *out);
/* nterms Pauli strings, paulis[t*n + q] in {0:I, 1:X, 2:Y, 3:Z}; out[t] = Re Tr(rho P_t). */
mpdo_status mpdo_expect_pauli_batch(mpdo_chain_t ch, const int8_t *paulis, int nterms,
                                    double *out);

/* Circuit.py:297-446 sample (conditional, grouped by measured prefix): L
 * ascending qubits `order` are sampled, the others traced; bits_out is
 * shots x L (row-major, 0/1).  pfloor is added to both conditional
 * probabilities (GLOBAL_MINIMUM in the reference); seed drives the host
 * binomial splits.  Right environments are built once and every group's
 * left environment advances in one batched step per measured qubit. */
mpdo_status mpdo_sample(mpdo_chain_t ch, const int *order, int L, int64_t shots, uint64_t seed, double pfloor,
                        int8_t *bits_out);

/* Circuit.py:448-466 randomSample: the same sampling in S measurement schemes
 * in one call.  schemes is S x L (0: X, 1: Y, 2: Z per measured qubit), rot
 * the MeasureX and MeasureY gates as two 2 x 2 complex matrices (8 doubles
 * each, row-major (out, in); may be NULL when every basis is Z), seeds one
 * per scheme, bits_out S x shots x L.  Scheme s gives the bits mpdo_sample
 * gives with seeds[s] on a copy of the chain rotated by mpdo_apply_1q.  The
 * right environments are built once for all schemes (a basis change on a
 * traced leg leaves it unchanged). */
mpdo_status mpdo_sample_schemes(mpdo_chain_t ch, const int *order, int L, const int *schemes, int S,
                                int64_t shots, const uint64_t *seeds, double pfloor, const double *rot,
                                int8_t *bits_out);

/* ---- Batched evolution of independent circuits ----------------------------
 * A batch runner owns `workers` host threads, each with its own engine (its
 * own non-blocking stream and memory pool) on `device`.  mpdo_batch_run hands
 * whole circuits to the workers, longest first, so that the small
 * factorisation launches of many circuits overlap on the GPU.  Each circuit
 * runs the same path as mpdo_chain_create + mpdo_apply_* + mpdo_truncate, so
 * its result does not depend on the worker or on the other circuits.  There
 * is no counterpart in the reference (its callers loop over circuits). */
typedef struct mpdo_batch_s *mpdo_batch_t;

enum { MPDO_OP_1Q = 1, MPDO_OP_2Q = 2, MPDO_OP_TRUNCATE = 3, MPDO_OP_KAPPA = 4 };

typedef struct {
  int n;                     /* qubits */
  int dtype;                 /* MPDO_C64 / MPDO_C128 */
  int connected;             /* as mpdo_chain_create */
  const double *vectors;     /* n x 2 complex initial product state */
  int chi, kappa;            /* truncate(): <= 0 means no cap */
  double max_err;            /* < 0: no error rule */
  int noisy;                 /* truncate() runs the kappa pass */
  double abs_cutoff;         /* 2q split cutoff (GLOBAL_MINIMUM in the reference) */
  int nops;
  const int *op_kind;        /* MPDO_OP_* per op */
  const int *op_site;        /* 1q: site; 2q: the smaller site of the pair */
  const int *op_k;           /* Kraus count (1q: 4K doubles, 2q: 16K complex) */
  const int64_t *op_offset;  /* start of each op's tensor in `kraus`, in doubles */
  const double *kraus;       /* interleaved complex, layouts as mpdo_apply_1q / _2q */
  double *z;                 /* out (nullable): n values <Z_i> */
  double *zz;                /* out (nullable): n-1 values <Z_i Z_{i+1}> */
  double *discarded;         /* out (nullable): (number of truncate ops) x (n-1) weights */
} mpdo_program;

mpdo_status mpdo_batch_create(int device, int workers, mpdo_batch_t *out);
mpdo_status mpdo_batch_destroy(mpdo_batch_t b);
/* Applies mpdo_engine_set_option to every worker's engine. */
mpdo_status mpdo_batch_set_option(mpdo_batch_t b, const char *name, double value);
mpdo_status mpdo_batch_num_workers(mpdo_batch_t b, int *workers);
/* The engine of one worker (for readouts of chains returned by a run). */
mpdo_status mpdo_batch_engine(mpdo_batch_t b, int worker, mpdo_engine_t *out);
/* Runs every program to completion.  chains_out (nullable, ncirc): the final
 * states, owned by the caller afterwards (mpdo_chain_destroy), each living on
 * the engine of worker_out[i] (nullable).  status_out (nullable, ncirc): each
 * circuit's status.  Returns the first failing circuit's status (all circuits
 * are attempted); mpdo_batch_error gives each failure's message. */
mpdo_status mpdo_batch_run(mpdo_batch_t b, int ncirc, const mpdo_program *progs, mpdo_chain_t *chains_out,
                           int *worker_out, int *status_out);
const char *mpdo_batch_error(mpdo_batch_t b, int circuit);

/* ---- Reverse-mode gradient ------------------------------------------------
 * No counterpart in the reference (its gate tensors detach the angles,
 * SingleGates.py:181-185, YGates.py:66-68); it differentiates the evolution
 * the reference defines (Circuit.py:469-491, TNNOptimizer.py:87-197).
 * Evolves `prog` (connected = 1, max_err < 0; z / zz / discarded ignored),
 * evaluates loss = Re Tr(rho H) for a Hermitian H given as a matrix-product
 * operator and writes dloss/d(every gate tensor) into grad_out, laid out like
 * prog->kraus (interleaved complex, cotangent = dL/dRe + i dL/dIm).
 * mpo_dims: n + 1 bond dimensions D_0 = 1 .. D_n = 1 (each <= 64); mpo: per
 * site k, W_k[D_k][D_k+1][out][in] complex, concatenated.  Every split keeps
 * at most the numerical rank (singular values above rank_tol * s_0) and
 * pending 2q gates are materialised by QR (no absolute cutoff); the
 * 1/(lam_j - lam_i) terms of the split adjoints are broadened to
 * d / (d^2 + (broadening lam_0)^2).  The chain is checkpointed per truncate
 * segment and each segment is recomputed once in the reverse sweep.
 * phase_ms (nullable, 3 doubles): CUDA-event spans of the forward pass, the
 * readout with its adjoint, and the reverse sweep. */
mpdo_status mpdo_program_grad(mpdo_engine_t eng, const mpdo_program *prog, const int *mpo_dims, const double *mpo,
                              double rank_tol, double broadening, double *loss_out, double *grad_out,
                              double *phase_ms);

/* Kernel-level test hooks (no counterpart in the reference).  Host in/out,
 * row-major complex (interleaved doubles).
 * mpdo_debug_qr:  A (m x n) = Q (m x k) R (k x n), k = min(m, n), Householder
 *                 (TSQR for tall inputs).
 * mpdo_debug_svd: right singular vectors of A (m x n): W (n x n, column-major,
 *                 columns sorted by singular value, descending) and sigma (n).
 * mpdo_debug_split: Y (m x n) ~= L (m x keep) R (keep x n), L = U_k sqrt(S_k),
 *                 R = sqrt(S_k) V_k^H (the split used by every SVD step). */
mpdo_status mpdo_debug_split(mpdo_engine_t eng, int dtype, int m, int n, int keep, const double *y,
                             double *l, double *r);
mpdo_status mpdo_debug_qr(mpdo_engine_t eng, int dtype, int m, int n, const double *a, double *q,
                          double *r);
mpdo_status mpdo_debug_svd(mpdo_engine_t eng, int dtype, int m, int n, const double *a, double *w,
                           double *sigma);

/* The truncation rule every SVD step applies to its singular values
 * (decompositions.py:121-140; the split's absolute cutoff, Circuit.py:123,
 * and the sweeps' relative error, TNNOptimizer.py:124-129): how many of the
 * descending values s[0..len) of a matrix with nsv singular values (entries
 * len..nsv-1 are zero) are kept under the cap max_sv and the error rule
 * (err < 0: no error rule; relative != 0: threshold err * s[0]).  Host code
 * only; needs no device. */
mpdo_status mpdo_keep_count(const double *s, int len, int nsv, int max_sv, double err, int relative, int *keep);

/* Allocation-free SVD step (no counterpart in the reference).  For callers
 * that cannot allocate device memory -- a process whose device memory is
 * pre-partitioned by its own allocator, or code under an allocation hook that
 * forbids cudaMalloc -- this computes what the engine's SVD step computes
 * (Householder TSQR of A, one-sided Jacobi on R with accumulated rotations)
 * using only a fixed 8 MiB static device array as scratch; it calls no
 * cudaMalloc/cudaFree.  complex64 only, 1 <= m <= 8192, 1 <= n <= 64; larger
 * sizes are rejected with MPDO_ERR_INVALID.  Inputs/outputs are DEVICE
 * pointers on the current device: a (m x n row-major), w (n x n column-major:
 * right singular vectors sorted by singular value, descending), sigma (n
 * floats), status (nullable: a device int receiving 0 ok, 1 sweep limit,
 * 2 non-finite).  stream: a cudaStream_t or NULL.  The first call on a device
 * resolves the array's device address; make it before any stream capture.
 * All calls share the array (it keeps the last call's contents), so calls
 * that overlap on the GPU race and must be serialised by the caller. */
mpdo_status mpdo_right_svd_noalloc(int m, int n, const void *a, void *w, void *sigma, int *status,
                                   void *stream);

#ifdef __cplusplus
}
#endif
#endif /* MPDO_GB300_H */
