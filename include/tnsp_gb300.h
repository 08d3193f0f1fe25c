/*
 * tnsp_gb300: GB300-native sampling-lattice Monte Carlo over a PEPS (sweep sampling, local
 * energy and energy gradient with boundary-MPS contraction truncated to Dcut).
 *
 * C ABI.  Every function returns 0 on success or a negative TNSP_E_* code; the message of the
 * last failure of a context is returned by tnsp_last_error.  No C++ exception crosses this
 * boundary.  One host thread per context; all device work is enqueued on the context stream.
 *
 * Each entry point names the reference interface it replaces (path:line in USTC-TNS/TNSP).
 */
#ifndef TNSP_GB300_H
#define TNSP_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TNSP_OK 0
#define TNSP_E_ARG (-1)        /* invalid argument or unsupported model shape */
#define TNSP_E_CUDA (-2)       /* a CUDA runtime call failed */
#define TNSP_E_STATE (-3)      /* call out of order (no lattice, no chains, ...) */
#define TNSP_E_DEVICE (-4)     /* a kernel reported a failure (see the status word) */
#define TNSP_E_NOMEM (-5)      /* device allocation failed */
#define TNSP_E_TOO_LARGE (-6)  /* problem exceeds the fixed arena of tnsp_amplitude_noalloc */

/* device status word bits (tnsp_device_status) */
#define TNSP_ST_SVD_NOCONV 1   /* one-sided Jacobi hit its sweep limit */
#define TNSP_ST_NONFINITE 2    /* a NaN/Inf amplitude or ratio appeared */
#define TNSP_ST_UNSUPPORTED 4  /* a Hamiltonian element changes one site only */
#define TNSP_ST_ZERO_WS 8      /* a chain's amplitude is exactly zero */

typedef struct tnsp_ctx tnsp_ctx;

/* precision of the tensor arithmetic inside the sampler (ratios, exponents and every accumulator
 * are float64 in all modes):
 *   TNSP_FP64  float64 (the reference's arithmetic)
 *   TNSP_FP32  float32; too coarse where amplitudes cancel strongly (large lattices)
 *   TNSP_DD    double-float: each value is a pair of floats (hi + lo, about 2^-46 relative
 *              precision) computed on the FP32 pipe, which GB300 runs at 64x its FP64 rate
 *   TNSP_MIXED the factorisations (per-sector QR and truncated SVD) in double-float, the tensors
 *              (boundaries, compression tensors, strips) stored and contracted in float32; amplitudes
 *              and E_loc carry float32-level rounding (~1e-5 relative on an 8x8 D=6 Dcut=36 lattice)
 *              while the truncation decisions keep double-float precision */
#define TNSP_FP64 0
#define TNSP_FP32 1
#define TNSP_DD 2
#define TNSP_MIXED 3

/*
 * Creates a context on CUDA device `device` using stream `stream` (a cudaStream_t, or NULL for
 * the legacy default stream).
 * Replaces: the per-process state of TAT/PyTAT (PyTAT/PyTAT.hpp:87, the global mt19937_64) and
 * the Configuration object graph (tetragono/tetragono/sampling_lattice/lattice.py:58-79).
 */
int tnsp_ctx_create(tnsp_ctx** out, int device, void* stream);
int tnsp_ctx_destroy(tnsp_ctx* ctx);
/* The message of the context's last failure; with ctx == NULL, the message of the calling thread's
 * last failed context-free call (tnsp_amplitude_noalloc). */
const char* tnsp_last_error(tnsp_ctx* ctx);

/*
 * Uploads the lattice: L1 x L2 sites, physical dimension P, the four virtual bond extents of
 * every site (dims[(l1*L2+l2)*4 + {0:U,1:D,2:L,3:R}], 1 where the bond is absent) and the dense
 * site tensors A[p][u][d][l][r] (float64, concatenated in row-major site order).  A block-sparse
 * (Bose U(1)/Z2) tensor is passed densely with zeros outside its blocks; the host package
 * converts the reference's block storage (TAT/include/TAT/structure/core.hpp:152-191).
 * Replaces: SamplingLattice.__init__/__setitem__ (tetragono/tetragono/sampling_lattice/lattice.py:746-796)
 * and the shrinker projection set-up (lattice.py:291-339).
 */
int tnsp_lattice_upload(tnsp_ctx* ctx, int L1, int L2, int P, const int* dims, const double* tensors, int cut);

/*
 * Declares the U(1)/Z-graded block structure of the uploaded lattice (optional; without it every
 * charge is zero and every matrix is one block).  leg_charges[(site*4 + leg)*Dmax + i] is the charge
 * of index i of leg U, D, L, R (Dmax = largest bond extent), phys_charges[p] the charge of physical
 * index p, site_flux[site] the conserved sum: every nonzero A[p][u][d][l][r] must satisfy
 * phys[p] + U[u] + D[d] + L[l] + R[r] == site_flux (checked; connected legs must carry opposite
 * charges).  With charges, every QR and SVD of the boundary compression runs per charge sector and
 * the truncation keeps the largest singular values over all sectors.
 * Replaces: the Symmetry/Edge segment structure of TAT (TAT/include/TAT/structure/symmetry.hpp:94-239,
 * edge.hpp:212-292) and its per-sector QR/SVD (TAT/include/TAT/implement/qr.hpp:310-510, svd.hpp:259-532).
 */
int tnsp_lattice_charges(tnsp_ctx* ctx, const int* leg_charges, const int* phys_charges, const int* site_flux);

/*
 * Makes the uploaded lattice fermionic (Fermi U(1), spinless: physical slices 0 = empty, 1 = occupied;
 * call after tnsp_lattice_upload with P = 2 and tnsp_lattice_charges; a new upload makes it bosonic
 * again).  slices holds per site, in site order, 8 arrays shaped like the site's (u, d, l, r) slice:
 * [family][n][prefix parity], family 0 read by the row boundaries and strips, 1 by the column ones,
 * each the stored slice of occupation n times its static sign and, for prefix parity 1, the parity of
 * its D (row) or R (column) index.  total_charge is the charge of the T leg of site (0, 0).  The
 * sampler then evaluates the reference's graded amplitudes: E_loc terms carry the hop's sign (and on
 * column strips the configuration signs), holes the prefix parity; gradient and natural-gradient rows
 * stay in the two-slice layout of the upload and take the static per-element sign on the host.
 * Replaces: TAT's fermionic edge operations and contraction signs (TAT/include/TAT/implement/
 * edge_operator.hpp:497-612, contract.hpp:381-580, conjugate.hpp:30-122) on this path.
 */
int tnsp_lattice_fermion(tnsp_ctx* ctx, const double* slices, int total_charge);

/*
 * Uploads the Hamiltonian: n_terms two-site terms in the reference's dictionary order.
 * sites[t*4 + {0,1,2,3}] = (l1, l2) of positions[0] then positions[1] of term t (nearest
 * neighbours).  For term t and input pair index i = s0*P + s1 (s0 at positions[0]) the outputs
 * are entries [offsets[t*P*P + i], offsets[t*P*P + i] + counts[t*P*P + i]) of out_index (o0*P + o1)
 * and value, in the order tensor_element lists them (counts = -1: input not in the table).
 * Replaces: tensor_element/calculate_element (tetragono/tetragono/tensor_element.py:20-108) and
 * SweepSampling._get_proper_position_order (tetragono/tetragono/sampling_lattice/sampling.py:156-190).
 */
int tnsp_model_upload(tnsp_ctx* ctx, int n_terms, const int* sites, const int* offsets, const int* counts,
                      int n_entries, const int* out_index, const double* values);

/*
 * The sweep's proposal tables, laid out as in tnsp_model_upload (no values: only which outputs an input
 * can hop to, and how many), and per-entry allow flags (NULL: all allowed).  A proposal whose picked
 * entry is not allowed is rejected before its amplitude ratio and before its uniform draw, as the
 * reference's restricted subspace rejects it.  n_terms == 0 keeps the energy tables as the proposal
 * tables and applies `allowed` (one flag per energy-table entry) to them.  A later tnsp_model_upload
 * drops these tables.
 * Replaces: SweepSampling's hopping_hamiltonians and restrict_subspace
 * (tetragono/tetragono/sampling_lattice/sampling.py:81-91, 117-143).
 */
int tnsp_model_hopping(tnsp_ctx* ctx, int n_terms, const int* sites, const int* offsets, const int* counts,
                       int n_entries, const int* out_index, const unsigned char* allowed);

/*
 * Per-entry allow flags of the energy tables for the observation (NULL: all allowed): an E_loc term whose
 * entry is not allowed contributes nothing.
 * Replaces: Observer's restrict_subspace (tetragono/tetragono/sampling_lattice/observer.py:224-233, 364-367).
 */
int tnsp_model_energy_restrict(tnsp_ctx* ctx, const unsigned char* allowed);

/*
 * Sets up B independent chains: configs[b*L1*L2 + l1*L2 + l2] are physical indices, seeds[b]
 * seeds chain b's mt19937_64 exactly as TAT.random.seed does, and `discard` uniform_real draws
 * are skipped first (SeedDiffer draws one, tetragono/tetragono/utility.py:146-150).
 * Replaces: Configuration.import_configuration (lattice.py:181-206) + TAT.random.seed (PyTAT/PyTAT.hpp:89-94).
 * TNSP_DD and TNSP_MIXED are refused (TNSP_E_ARG) for a lattice uploaded without charges whose site tensors are more
 * than a quarter exact zeros: such block-sparse tensors stored densely make rank-deficient boundaries
 * whose structural zeros double-float cannot resolve (errors up to 1e-3); declare the charges
 * (tnsp_lattice_charges) or use TNSP_FP64.
 */
int tnsp_chains_init(tnsp_ctx* ctx, int B, const int32_t* configs, const uint64_t* seeds, int discard,
                     int precision);

/* options of tnsp_set_option */
#define TNSP_OPT_JACOBI_SWEEPS 1  /* sweep limit of the one-sided Jacobi SVD (default 60, range 1..1000);
                                     a factorisation that does not converge within it sets
                                     TNSP_ST_SVD_NOCONV and the call returns TNSP_E_DEVICE */
#define TNSP_OPT_BLOCKS_PER_SM 2  /* resident sampler blocks per SM (0 = the most the occupancy
                                     calculator allows, the default); fewer blocks give each chain's
                                     block more shared memory for its factorisations */

/*
 * Number of chains one launch advances at once (the resident thread blocks, one chain each, planned for
 * this lattice, cut, precision and TNSP_OPT_BLOCKS_PER_SM): a batch of B chains runs in ceil(B / n)
 * waves.  Needs tnsp_chains_init.  No reference counterpart (one chain per reference process).
 */
int tnsp_resident_chains(tnsp_ctx* ctx, int* n);

/*
 * Sets a context option (TNSP_OPT_*).  Takes effect at the next tnsp_chains_init / tnsp_sweep.  A new
 * TNSP_OPT_BLOCKS_PER_SM re-plans the per-block scratch, which drops the gradient sums accumulated since
 * the last tnsp_observer_reset: set it before observing.
 * Replaces: the reference's LAPACK error branch of the SVD (TAT/include/TAT/implement/svd.hpp:114-122,
 * `what_if_lapack_error`), whose iteration limit is LAPACK's own; no counterpart for the block count.
 */
int tnsp_set_option(tnsp_ctx* ctx, int option, int value);

/*
 * Runs `nsweeps` sweeps of every chain.  When `observe` is non-zero every sweep is followed by
 * the observation of its configuration: E_loc, the gradient holes and the reweighted
 * accumulators (energy, Delta, E*Delta), and per-sample E_loc and log|ws| are recorded.
 * nsweeps == 0 with observe != 0 observes the chains' current configurations once (sampling
 * weight |ws|^2 of the configuration itself), e.g. to re-evaluate configurations in another precision.
 * Replaces: SweepSampling.__call__ (sampling.py:145-154, with _single_term :117-143) and
 * Observer.__call__ (tetragono/tetragono/sampling_lattice/observer.py:313-415).
 */
int tnsp_sweep(tnsp_ctx* ctx, int nsweeps, int observe);

/*
 * tnsp_sweep for n contexts (different lattices, bond dimensions, cuts, precisions; one device) as
 * one CUDA graph launch: their sweep kernels run concurrently and fill each other's idle SMs.  Every
 * context's results are those of tnsp_sweep; tnsp_last_timing of each reports the whole graph.  A
 * failure status is reported through the first context that has one.
 * No reference counterpart: the reference runs one lattice per process.
 */
int tnsp_sweep_batch(tnsp_ctx* const* ctxs, int n, int nsweeps, int observe);

/*
 * Replaces the configurations of all chains (configs as in tnsp_chains_init), keeping each chain's
 * random-number stream: the next tnsp_sweep starts from them (e.g. after accepted proposals of a
 * learned sampler).  No reference counterpart (the reference's chains only move by local sweeps).
 */
int tnsp_chains_write(tnsp_ctx* ctx, const int32_t* configs);

/* Zeroes the observer accumulators and the per-sample record (Observer.__enter__, observer.py:41-81). */
int tnsp_observer_reset(tnsp_ctx* ctx);

/*
 * Reads the reduced accumulators (Observer.__exit__ + estimators, observer.py:83-126, 433-555):
 * scalars[0..7] = count, total_weight, total_weight_square, total_log_ws, sum E*w, sum E*w^2,
 * sum E^2*w^2, number of proposals accepted; delta / edelta (may be NULL) receive sum hole*w and
 * sum E*hole*w in the dense site layout of tnsp_lattice_upload.
 */
int tnsp_observer_read(tnsp_ctx* ctx, double* scalars, double* delta, double* edelta);

/*
 * Copies the per-sample record of the last tnsp_sweep(observe=1) call: eloc[s*B + b],
 * log_ws[s*B + b] (natural log of |ws|) and reweight[s*B + b] for s < nsweeps.
 */
int tnsp_samples_read(tnsp_ctx* ctx, double* eloc, double* log_ws, double* reweight);

/*
 * Natural gradient support.  tnsp_holes_keep(ctx, 1) makes every observed sweep append, per sample,
 * the row <psi|s|dpsi/dA>/<psi|s|psi> over all parameters (dense A[p][u][d][l][r] order of the
 * upload, zero outside the sampled physical slices; row order: sweep-major, then chain, following
 * tnsp_samples_read) until the next tnsp_observer_reset; 0 releases the rows.  tnsp_holes_count gives
 * the number of rows kept.  tnsp_holes_gemv computes y = H x (transpose == 0: x has n_params
 * entries, y one per row) or y = H^T x (transpose != 0) on the device, x and y in host memory.
 * Replaces: the per-sample deltas Observer.__call__ keeps with enable_natural_gradient
 * (tetragono/tetragono/sampling_lattice/observer.py:403-409) and the D / DT products of
 * natural_gradient_by_conjugate_gradient (observer.py:612-641).
 */
int tnsp_holes_keep(tnsp_ctx* ctx, int enable);
int tnsp_holes_count(tnsp_ctx* ctx, int64_t* rows);
int tnsp_holes_gemv(tnsp_ctx* ctx, int transpose, const double* x, double* y);

/*
 * gram (rows x rows, row-major, rows = tnsp_holes_count) = H H^T over the kept hole rows, float64, one
 * launch: the sample-space matrix of the pseudo-inverse natural gradient, whose T = D D^T follows on the
 * host from it, H delta and delta.delta (D = the rows minus their weighted mean delta).
 * Replaces: the D D^T product of natural_gradient_by_direct_pseudo_inverse
 * (tetragono/tetragono/sampling_lattice/observer.py:697-907, single-process form :902-907).
 */
int tnsp_holes_gram(tnsp_ctx* ctx, double* gram);

/* Copies the chains' current configurations (export_configuration, lattice.py:208-229) and, if
 * not NULL, the sampling weight log|ws|^2 of their last sweep (log of `possibility`). */
int tnsp_chains_read(tnsp_ctx* ctx, int32_t* configs, double* log_possibility);

/*
 * Amplitude ws = hole(()) of B arbitrary configurations (row-0 strip of the truncated boundary
 * MPS, tetragono/tetragono/auxiliaries/single_layer_auxiliaries.py:710-720); results as
 * mantissa * 2^exponent.
 */
int tnsp_amplitude(tnsp_ctx* ctx, int B, const int32_t* configs, double* mantissa, int32_t* exponent);

/* Returns and clears the device status word (TNSP_ST_* bits). */
int tnsp_device_status(tnsp_ctx* ctx, int32_t* status);

/* Milliseconds spent in the last tnsp_sweep's kernels (CUDA events on the context stream), and the
 * number of kernel launches it made. */
int tnsp_last_timing(tnsp_ctx* ctx, double* ms, int64_t* launches);

/*
 * Algorithmic work done by tnsp_sweep since the last reset (flops must hold 16 doubles), summed
 * over blocks: flops[0] block contractions (2mnk per product), flops[1] Householder QR (with
 * explicit Q), flops[2] truncated SVD (Golub-Van Loan count 4m^2n + 8mn^2 + 9n^3), flops[3] strip
 * environments and holes; flops[4..15] SM clock cycles spent by the blocks in the phases two-line
 * contraction, sector analysis, QR, R absorption, Jacobi, SVD output, U*S absorption, strip steps,
 * (reserved), observation holes, (reserved), (reserved).  `reset` non-zero zeroes the counters.
 * No reference counterpart: instrumentation for the roofline of the sampler kernel.
 */
int tnsp_counters_read(tnsp_ctx* ctx, double* flops, int reset);

/*
 * Allocation-free variant of tnsp_amplitude.  No counterpart in the reference.  It is for callers that
 * must not allocate device memory after start-up: a host application whose device memory is all
 * reserved by its own pool or caching allocator (a cudaMalloc behind its back fails or fragments that
 * pool), and latency-bound or real-time hosts, where cudaMalloc/cudaFree can synchronise the device
 * and take unbounded time.  It needs no context: tensors (dense A[p][u][d][l][r], float64), configs
 * (B x L1*L2 int32), mantissa (B doubles) and exponent (B int32) are caller-owned DEVICE pointers;
 * dims (L1*L2*4 ints, as in tnsp_lattice_upload) is a host pointer; stream is a cudaStream_t or NULL.
 * Configuration entries must lie in [0, P): they are not checked on the device.  The call returns
 * after the stream has finished its work (it reads the device status word back).
 * Every matrix is factorised as one block (no charge sectors are declared): for block-sparse tensors
 * passed densely the amplitudes equal tnsp_amplitude's in float64 to rounding, at a higher cost.
 * Scratch comes from a 64 MiB array compiled into the library (held by every device that loads
 * it, until the process exits); cut * max bond extent above 1024, or a lattice/cut whose one-chain
 * scratch does not fit in it, returns TNSP_E_TOO_LARGE before any device work.  The first call on a
 * device resolves the array's device address (cudaGetSymbolAddress) with that device current.  No
 * call can be captured into a CUDA graph: each copies host arrays to the device and waits for its
 * stream.  All calls share the array, which keeps the last
 * call's contents (each call rewrites what must start at a known value): calls that overlap on the
 * GPU race and must be serialised.  On failure tnsp_last_error(NULL) gives the reason.
 */
int tnsp_amplitude_noalloc(int L1, int L2, int P, const int* dims, const double* tensors, int cut, int B,
                           const int32_t* configs, double* mantissa, int32_t* exponent, void* stream);

/*
 * Learned proposal (no reference counterpart): an autoregressive masked MLP (MADE) over n_sites binary
 * sites, x -> relu(W1 x + b1) -> relu(W2 h1 + b2) -> logits W3 h2 + b3 with p(x_i = 1 | x_<i) =
 * sigmoid(logit_i); weights float32 (Adam), used as bfloat16, float32 accumulation; hand-written
 * training and sampling kernels.  configs are 0/1 per site, [B][n_sites], B <= batch_capacity.
 *   tnsp_made_train: one Adam step (learning rate lr) on the mean negative log-likelihood of the
 *     batch; *loss = that mean before the step.
 *   tnsp_made_gradient: the gradient of that loss (float32, parameter order of tnsp_made_params).
 *   tnsp_made_logq: log q(x) per configuration.
 *   tnsp_made_sample: B independent configurations drawn site by site, with their log q.
 *   tnsp_made_params: read (write == 0) or replace the float32 parameters, in the order
 *     W1 [hidden][n], b1 [hidden], W2 [hidden][hidden], b2 [hidden], W3 [n][hidden], b3 [n].
 */
typedef struct tnsp_made tnsp_made;
int tnsp_made_create(tnsp_made** out, int device, int n_sites, int hidden, uint64_t seed, int batch_capacity);
int tnsp_made_destroy(tnsp_made* made);
const char* tnsp_made_error(tnsp_made* made);
int tnsp_made_params(tnsp_made* made, float* params, int write);
int tnsp_made_train(tnsp_made* made, const int32_t* configs, int B, double lr, double* loss);
int tnsp_made_gradient(tnsp_made* made, const int32_t* configs, int B, float* grad);
int tnsp_made_logq(tnsp_made* made, const int32_t* configs, int B, double* logq);
int tnsp_made_sample(tnsp_made* made, int B, int32_t* configs, double* logq);

#ifdef __cplusplus
}
#endif

#endif
