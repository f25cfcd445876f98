/*
 * sep_gb300.h -- C ABI of libsep_gb300.so, the GB300 (sm_103a) implementation
 * of the filter-diagonalisation path of the semi-empirical pseudopotential
 * method (the reference's filter/ program).
 *
 * Plain C types only: host or device pointers plus sizes.  All functions
 * return an int status (SEP_OK = 0, negative on error) and leave a message for
 * sep_last_error().  Arrays follow the reference's layouts:
 *   grids        x fastest, jxyz = nx (ny jz + jy) + jx   (filter/init.c:139-141)
 *   complex      interleaved {re, im} doubles, as zomplex  (filter/fd.h:17-19)
 *   state blocks state-major psitot[state * ngrid + g]     (filter/main.c:86)
 * Host-pointer entry points copy in and out; the *_dev variants take device
 * pointers and run on the context's stream.
 *
 * The fd.h-compatible entry points (same names and arguments as the
 * reference's filter/fd.h:81-145) are declared in sep_fd_compat.h.
 */
#ifndef SEP_GB300_H
#define SEP_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum sep_status {
  SEP_OK = 0,
  SEP_ERR_ARG = -1,          /* bad argument or unsupported size */
  SEP_ERR_CUDA = -2,         /* CUDA runtime / device error */
  SEP_ERR_NOMEM = -3,        /* device allocation failed */
  SEP_ERR_SOLVER = -4,       /* dense eigensolver failed (reference: dsyev/dgesvd info) */
  SEP_ERR_NO_DEVICE = -5,    /* no CUDA device / library built without one */
  SEP_ERR_NUMERIC = -6,      /* non-finite values, empty subspace */
  SEP_ERR_IO = -7            /* a file could not be read or written */
};

enum sep_precision {
  SEP_PREC_F64 = 0,    /* complex128 filter, FP64 subspace */
  SEP_PREC_MIXED = 1   /* complex64 filter with FP32 accumulation, FP64 subspace */
};

typedef struct sep_ctx sep_ctx;

/* Stage wall times of sep_pipeline, seconds (CUDA events on the context stream). */
typedef struct {
  double energy_range_s, filter_s, ortho_s, rayleigh_ritz_s, sigma_s, total_s;
  long power_iterations, mkept, h_applies;
  double emax, dE, dt;
  double polish_s;  /* the FP64 polish of sep_ctx_set_polish (0 when off) */
} sep_timing;

/* ---- library ------------------------------------------------------------ */
const char *sep_last_error(void);
int sep_version(void);                      /* 10000*major + 100*minor + patch */
int sep_device_count(int *count);

/* ---- context: one grid + one local potential -----------------------------
 * Replaces the grid / ksqr / potl set-up of filter/init.c:90-199 and the FFT
 * plans of filter/main.c:58-59.  steps = (dx, dy, dz) in bohr; ekinmax = the
 * kinetic cap in hartree (10.0 in filter/init.c:31; k^2 is pre-scaled by
 * 1/N and capped at ekinmax/N as filter/init.c:125-143).  potl: N doubles or
 * NULL (set later).  Supported axis lengths: 14 16 18 20 24 32 36 40 48 56 64
 * 72 80 96 112 128 160 192 256. */
int sep_ctx_create(const long dims[3], const double steps[3], double ekinmax,
                   const double *potl, int precision, sep_ctx **out);
int sep_ctx_destroy(sep_ctx *ctx);
int sep_ctx_set_potential(sep_ctx *ctx, const double *potl);      /* host */
int sep_ctx_set_potential_dev(sep_ctx *ctx, const double *potl);  /* device */
/* Vmin, Vmax of the potential (filter/init.c:196-199) and dv = dx dy dz */
int sep_ctx_info(sep_ctx *ctx, double *vmin, double *vmax, double *dv, long *ngrid);
int sep_ctx_stream(sep_ctx *ctx, void **cuda_stream);             /* cudaStream_t */
/* Capture the Newton loop of sep_filter* in a CUDA graph (default 1). */
int sep_ctx_set_graphs(sep_ctx *ctx, int enable);
/* Newton steps accumulated per pass over the step history, 1 <= k <= 128
 * (default 32; the history holds k grids per pair of states). */
int sep_ctx_set_block_steps(sep_ctx *ctx, int k);
/* Complex64 Newton steps take two grid passes instead of four.  On cubic
 * grids with nx in {96, 112, 128, 160, 192, 256}: a z pass that also does the
 * y transform's R-point stage (R = 4 or 8), and a fused pass per sub-plane of
 * L / R rows for the rest of the y transform, the x transforms and the
 * epilogue (same transforms with y and z split differently: equal to the line
 * passes within FP32 rounding).  On other grids with nx = ny in {40, 48, 56,
 * 64, 72, 80, 96, 112, 128}: the z line pass and one fused pass per z-plane
 * for the x and y transforms and the epilogue (same arithmetic per line as
 * the line passes).  enable = 0 selects the four line passes.  Default 1. */
int sep_ctx_set_fusion(sep_ctx *ctx, int enable);
/* FP64 refinement steps (0..8, default 0) that sep_pipeline runs after
 * Rayleigh-Ritz (filter/Hmat.c:11-86).  Each step extends the subspace with
 * the residuals H psi - E psi of the Ritz pairs (preconditioned with
 * (T + 1 Ha)^-1 in complex64 contexts), made orthogonal to them and
 * orthonormal (directions of negligible residuals dropped), and repeats the
 * Rayleigh-Ritz diagonalisation in FP64: about squaring the eigenvalue error
 * of each pair; the lowest mkept pairs of the extended space are kept.  No
 * counterpart in the reference.  A step needs a second block of 2 mkept
 * states on the device and is skipped when it does not fit.  The refinement
 * time is counted in rayleigh_ritz_s. */
int sep_ctx_set_refine(sep_ctx *ctx, int steps);
/* FP64 polish that sep_pipeline runs after sigma (default off, nc = 0): the
 * Ritz pairs whose values lie in [el_min - guard, el_max + guard] are
 * filtered once more in FP64 by one wide Gaussian at the window's centre
 * (filter/filter.c:59-83 with nc Newton steps, dt = (nc / 2.5 dE)^2 as
 * filter/main.c:70), then orthonormalised (filter/ortho.c:11-52),
 * diagonalised (filter/Hmat.c:11-86) and their sigma recomputed
 * (filter/energy.c:88-119); the block replaces its rows of psi, eval and
 * sige.  Meant for complex64 filters: their Ritz vectors carry broadband
 * single-precision rounding noise that holds sigma near 1e-4 Ha while their
 * Ritz values already match the FP64 path; the wide Gaussian damps the noise
 * far from the window.  No counterpart in the reference.  nc in {0} or
 * [2, 8192]; guard >= 0 (hartree, default 0.01).  Its time is
 * sep_timing.polish_s (also in total_s). */
int sep_ctx_set_polish(sep_ctx *ctx, long nc, double guard);

/* Arithmetic of the FP64-class work inside sep_pipeline: the H applies of
 * Rayleigh-Ritz (filter/Hmat.c:11-86), of sigma (filter/energy.c:88-119) and
 * of the residual refinement, and the Newton filter of the polish.
 * mode 0: IEEE FP64 line passes (bound by the FP64 pipe on GB300).
 * mode 1: double-float line passes, each value the unevaluated sum of two
 * floats (about 48 significant bits; TwoSum / TwoProd with fused multiply-
 * adds) on the FP32 pipe: an H apply about 3.7x faster at 128^3, within
 * 2e-14 relative of the FP64 result.  States stay FP64 in memory between the
 * stages.  Default 1 for complex64 contexts, 0 for FP64 contexts (whose
 * pipeline is the FP64 reference).  In an FP64 context mode 1 also runs the
 * Newton filter of sep_filter* and sep_pipeline in double-float (an FP64-
 * class filter about 3.7x faster at 128^3).  The energy range,
 * sep_hamiltonian and sep_energy_all always use FP64. */
int sep_ctx_set_arith(sep_ctx *ctx, int mode);

/* ---- Hamiltonian: filter/hamiltonian.c:11-44 -----------------------------
 * hpsi = T psi + V psi for nstates complex grids (interleaved complex128). */
int sep_hamiltonian(sep_ctx *ctx, const double *psi, double *hpsi, long nstates);
int sep_hamiltonian_dev(sep_ctx *ctx, const double *psi, double *hpsi, long nstates);

/* ---- general apply: out = alpha (T x + V y) + beta y ----------------------
 * Covers kinetic (y = NULL: out = alpha T x, filter/hamiltonian.c:27-44),
 * hamiltonian_norm (T phi + V psi, filter/hnorm.c:29-39) and hnorm. */
int sep_apply(sep_ctx *ctx, const double *x, const double *y, double *out, long nstates,
              double alpha, double beta);
/* Override the kinetic cap with an already 1/N-scaled value (the reference's
 * par.Ekinmax after filter/init.c:137). */
int sep_ctx_set_kcap(sep_ctx *ctx, double kcap_scaled);
/* out[r] = sum_g x[r][g]^2 for m rows of len doubles, without a context. */
int sep_row_sumsq(const double *x, long m, long len, double *out);
/* The context's k^2 grid (ngrid doubles) with its current cap. */
int sep_ctx_ksqr(sep_ctx *ctx, double *out);
/* filter/norm.c:40-54 without a context (any ngrid). */
int sep_normalize_states(double *psi, long m, long ngrid, double dv);
/* filter/rand.c:28-66 ran_nrc with its process-wide shuffle state, and
 * filter/init.c:236-251 init_psi drawing from it (real parts; *idum advances). */
double sep_ran_nrc(long *idum);
int sep_init_psi(long *idum, long ngrid, double dv, double *psi_re);

/* ---- filter/hnorm.c:11-39 ------------------------------------------------
 * psin = dE_1 H psim1 - (2 + zm1 + vmin dE_1) psim1 (complex grids). */
int sep_hnorm(sep_ctx *ctx, const double *psim1, double *psin, long nstates, double dE_1,
              double vmin, double zm1);

/* ---- Newton filter: filter/filter.c:59-83 (filter) for ns start states ---
 * start: ns x N real states; an_re: ms x nc (real parts of the reference's
 * zomplex an[nc*e + j]); zn: nc points; out: ns x ms x N, block s holding
 * psi0[e][g] = sum_j an_re[e][j] Re psi_j[g] as filter.c computes it.
 * In SEP_PREC_MIXED the recursion and the sums run in complex64 / FP32. */
int sep_filter(sep_ctx *ctx, const double *start, long ns, const double *an_re,
               const double *zn, long ms, long nc, double dE_1, double vmin, double *out);
int sep_filter_dev(sep_ctx *ctx, const double *start, long ns, const double *an_re,
                   const double *zn, long ms, long nc, double dE_1, double vmin, double *out);

/* ---- filter/norm.c:40-54 normalize_all, filter/energy.c:28-49 energy_all --- */
int sep_normalize_all(sep_ctx *ctx, double *psi, long m);
int sep_energy_all(sep_ctx *ctx, const double *psi, long m, double *ene);

/* ---- filter/energy.c:53-83 get_energy_range ------------------------------
 * Power iteration from the fixed seed -874917403 until |dE/E| <= 1e-4 or 500
 * iterations; dE = 1.1 (emax - vmin). */
int sep_energy_range(sep_ctx *ctx, double vmin, double *emax, double *dE, long *iters);

/* ---- subspace: filter/ortho.c:11-52, filter/Hmat.c:11-86, energy.c:88-119 --
 * sep_ortho: orthonormalise the m real states in place (dv metric) and keep
 * the directions whose singular value ratio S_i/S_0 >= 1e-10 as portho does;
 * *mkept = kept count (the first *mkept rows of psi).
 * sep_rayleigh_ritz: Hmatreal -- project H, diagonalise, rotate psi in place,
 * eval ascending.  sep_sigma: sqrt(|<H^2> - <H>^2|) per state. */
int sep_ortho(sep_ctx *ctx, double *psi, long m, long *mkept);
int sep_rayleigh_ritz(sep_ctx *ctx, double *psi, long m, double *eval);
int sep_sigma(sep_ctx *ctx, const double *psi, long m, double *sige);

/* ---- whole path: filter/main.c:64-142 ------------------------------------
 * start: ns x N real start states (host).  el: ms target energies.  vmin:
 * minimum of the potential.  dE <= 0: computed by the power iteration.
 * psi_out (optional, host, ns*ms x N): Ritz vectors, first *mkept rows.
 * eval / sige: ns*ms entries, first *mkept valid. */
int sep_pipeline(sep_ctx *ctx, const double *start, long ns, const double *el, long ms,
                 long nc, double vmin, double dE, double *psi_out, double *eval,
                 double *sige, long *mkept, sep_timing *timing);

/* ---- the filter's chunk plan (no counterpart in the reference) -----------
 * How sep_filter splits `pairs` pairs of states (ceil(ns / 2)) into chunks of
 * at most max_pairs (the pairs whose workspaces fit the device).  With host
 * buffers (host_buffers != 0) each chunk's output copy runs under the next
 * chunk's filter, so the last chunk splits off a tail: with a measured
 * copy_ratio >= 0 (output copy time over filter time; a context measures it
 * on each host-buffer call and uses it on the next) the smallest tail t >= 4
 * with copy_ratio (c - t) <= t, at most half of it; with copy_ratio < 0 (not
 * measured) the last chunk halves while it has 8 pairs or more.  counts: the
 * chunks' pair counts in order (cap entries); *nchunks: their number. */
int sep_filter_chunk_plan(long pairs, long max_pairs, int host_buffers, double copy_ratio,
                          long *counts, long cap, long *nchunks);

/* ---- host helpers, bit-identical to the reference -----------------------
 * filter/coeff.c:16-134: Newton coefficients of the Gaussian filters.
 * an_re, an_im: ms x nc; zn: nc. */
int sep_coefficients(long ms, long nc, double dE, double vmin, double dt, const double *el,
                     double *an_re, double *an_im, double *zn);
/* filter/init.c:236-251 + filter/rand.c:28-66: ns consecutive start states
 * from one seed (idum <= 0), each normalised with dv; out: ns x ngrid. */
int sep_start_states(long idum, long ns, long ngrid, double dv, double *out);
/* filter/init.c:124-144: the capped, 1/N-scaled k^2 grid. */
int sep_ksqr(const long dims[3], const double steps[3], double ekinmax, double *ksqr);
/* pseudopotFitting/pot.c:35-63 with hamiltonian.c:91-94: 1024-point
 * real-space table (r, v) of one species' form factor. */
int sep_form_factor_table(const double params[4], double vol_per_atom, double *r, double *v);

/* ---- local potential: filter/init.c:157-182 + filter/interpolate.c:11-23 --
 * potl[g] = sum_a scale_a * table_{type_a}(|r_g - R_a|) on the context grid.
 * xyz: natom x 3 (centred, bohr); types: natom ints in [0, ntype); scale:
 * natom (filterStrainCube/interpolate.c:11-25 strain factor) or NULL;
 * tab_r / tab_v: ntype x tab_stride (shifted tables, filter/read.c:105-108);
 * tab_n: ntype lengths.  mins = (xmin, ymin, zmin).  The result also becomes
 * the context's potential when `install` is non-zero. */
int sep_vbuild(sep_ctx *ctx, long natom, const double *xyz, const int *types,
               const double *scale, long ntype, const double *tab_r, const double *tab_v,
               const long *tab_n, long tab_stride, const double mins[3], double *potl,
               int install);
/* Backward of sep_vbuild: given dL/dpotl (N doubles), accumulate
 * dL/dtab_v (ntype x tab_stride) and, when dscale != NULL, dL/dscale (natom). */
int sep_vbuild_backward(sep_ctx *ctx, long natom, const double *xyz, const int *types,
                        const double *scale, long ntype, const double *tab_r,
                        const double *tab_v, const long *tab_n, long tab_stride,
                        const double mins[3], const double *dpotl, double *dtab_v,
                        double *dscale);

/* Hellmann-Feynman: rho[g] = dv sum_k w[k] psi[k][g]^2 for m real states
 * (host arrays).  For normalised eigenstates, dE_k/dV(r_g) = psi_k(r_g)^2 dv,
 * so with w = dL/dE this is dL/dpotl for sep_vbuild_backward.  No
 * counterpart in the reference (it has no gradients). */
int sep_hf_density(sep_ctx *ctx, const double *psi, long m, const double *w, double *rho);

/* ---- band-edge adjoint: forward and backward ------------------------------
 * theta = a0..a3 per type (ntype x 4, pseudopotFitting/hamiltonian.c:91-94).
 * No counterpart in the reference, which fits theta by a derivative-free
 * Monte Carlo search (pseudopotFitting/fit.c:29-50).
 *
 * Forward, step 1: the 1024-point table of each type (pot.c:35-63), minus its
 * last value (filter/read.c:105-108), then V(r) on the context grid
 * (filter/init.c:157-182), installed as the context's potential (potl: host
 * copy, may be NULL).  Step 2 is sep_pipeline on that potential. */
int sep_potential_from_params(sep_ctx *ctx, long natom, const double *xyz, const int *types,
                              const double *scale, long ntype, const double *params,
                              double vol_per_atom, const double mins[3], double *potl);
/* Backward: dparams (ntype x 4) = dL/dtheta for Ritz pairs (psi: m x ngrid
 * normalised states of the last forward, host) and dL_dE (m).  Chain:
 * Hellmann-Feynman density, V(r) backward, adjoint of the table shift,
 * transpose of the sine-transform Jacobian. */
int sep_band_edge_backward(sep_ctx *ctx, long natom, const double *xyz, const int *types,
                           const double *scale, long ntype, const double *params,
                           double vol_per_atom, const double mins[3], const double *psi, long m,
                           const double *dL_dE, double *dparams);
/* The table part of the backward for one type: dparams[4] from dL/d(shifted
 * table) (1024 values).  Host only. */
int sep_form_factor_backward(const double params[4], double vol_per_atom, const double *dtab,
                             double *dparams);

/* ---- many nanocrystals in one launch ---------------------------------------
 * A batch holds one job per context (grids may differ): job j filters ns[j]
 * start states with ms targets and nc Newton steps.  sep_batch_create
 * captures every job's whole Newton filter as a parallel branch of ONE CUDA
 * graph; sep_batch_run launches it once.  sep_batch_io returns each job's
 * device start (ns x N) and output (ns x ms x N, float64) arrays; the
 * coefficients of each job are uploaded before a run.  Each job needs its own
 * context; while the batch exists, a context's filter workspace cannot grow
 * (filters that fit it still run).  No counterpart in the reference (one
 * program run per crystal). */
typedef struct sep_batch sep_batch;
int sep_batch_create(int njobs, sep_ctx *const *ctxs, const long *ns, long ms, long nc,
                     sep_batch **out);
int sep_batch_io(sep_batch *b, int job, double **start_dev, double **out_dev);
int sep_batch_set_coefficients(sep_batch *b, int job, const double *an_re, const double *zn,
                               double dE_1, double vmin);
int sep_batch_run(sep_batch *b);
/* host copies into / out of a job's device arrays */
int sep_batch_load_start(sep_batch *b, int job, const double *host);
int sep_batch_read_out(sep_batch *b, int job, double *host);
int sep_batch_destroy(sep_batch *b);
/* Tile-shape autotuner: times both compiled tile shapes of each of the 5
 * Newton-step passes on npairs grids and keeps the faster per pass for this
 * context; choices (5 ints, may be NULL) receives the picks. */
int sep_ctx_autotune(sep_ctx *ctx, long npairs, int reps, int *choices);
/* Set the 5 tile shapes (0 or 1) by hand. */
int sep_ctx_set_tiles(sep_ctx *ctx, const int *choices);

/* ---- subspace contractions ------------------------------------------------
 * The Gram, projection and rotation products of sep_ortho (filter/ortho.c:11-52)
 * and sep_rayleigh_ritz (filter/Hmat.c:11-86).  mode 1 (default): on the
 * tcgen05 tensor cores by exact splitting into bf16 digits with exact integer
 * accumulation, FP64-accurate; mode 0: on the FP64 pipe. */
int sep_ctx_set_subspace(sep_ctx *ctx, int mode);
/* C (m x n) = alpha A B^T, A m x k, B n x k (host, row-major); sym: B = A
 * (B may be NULL) and C is symmetric.  Uses the context's mode. */
int sep_subspace_gemm(sep_ctx *ctx, const double *A, const double *B, long m, long n, long k,
                      double alpha, int sym, double *C);
/* The same on device pointers, on the context's stream; in mode 1 it waits
 * for the stream before returning (it reads the kernel's status word). */
int sep_subspace_gemm_dev(sep_ctx *ctx, const double *A, const double *B, long m, long n,
                          long k, double alpha, int sym, double *C);
/* out (m x w) = W (m x k) X (k x w), host row-major.  Uses the context's mode. */
int sep_subspace_rotate(sep_ctx *ctx, const double *W, const double *X, long m, long k, long w,
                        double *out);

/* ---- dense symmetric eigensolver -------------------------------------------
 * The eigen-decompositions of ortho (filter/ortho.c:11-52, where the reference
 * calls dgesvd) and Rayleigh-Ritz (filter/Hmat.c:11-86, dsyev) run on the
 * library's own FP64 solver or on cuSOLVER's syevd.  The library's solver:
 * Householder tridiagonalisation in one cooperative kernel, divide and
 * conquer on the tridiagonal (QL leaves of 8 rows, deflation, secular roots
 * by bisection, Loewner-corrected vectors), back-transformation; no library
 * call.  mode 1 (default): the library's solver, 0: cuSOLVER's syevd. */
int sep_ctx_set_eigensolver(sep_ctx *ctx, int mode);
/* w (n) ascending and v (n x n, column-major: v[i + j n] is component i of
 * eigenvector j) of the symmetric n x n matrix a (host arrays, n <= 16384),
 * on the calling thread's current device with the library's solver. */
int sep_eigh(const double *a, long n, double *w, double *v);
/* The same on device arrays: a_dev (n x n) becomes the eigenvectors, w_dev
 * the eigenvalues; work_dev holds sep_eigh_work_bytes(n) bytes.  Returns
 * after the stream has reached its end (the merges sort on the host).
 * stage_ms (3 doubles, may be NULL): device times of the tridiagonalisation,
 * the divide and conquer and the back-transformation. */
size_t sep_eigh_work_bytes(long n);
int sep_eigh_dev(double *a_dev, long n, double *w_dev, double *work_dev, void *cuda_stream,
                 double *stage_ms);

/* ---- measurement --------------------------------------------------------
 * Average device time (ms, CUDA events on the context stream) of one launch
 * of each Newton-step kernel on npairs complex grids in the context's
 * precision, over reps launches each: ms_out[0..6] = x forward, y forward,
 * z forward*k^2*inverse, y inverse, x inverse+epilogue+forward, accumulate
 * (block_steps history grids into ms = 8 state pairs), and the fused step's
 * xy pass (y/x inverse + epilogue + x/y forward, on planes or sub-planes; 0
 * when the context has no fused step; sep_time_fused_step also times its z
 * pass).  No counterpart in the reference; used for the roofline report. */
int sep_time_passes(sep_ctx *ctx, long npairs, int reps, double *ms_out);
/* The two passes of the fused complex64 Newton step (sep_ctx_set_fusion) on
 * npairs grids, average device ms per launch over reps launches: ms_out[0]
 * the xy pass (plane or sub-plane form, with the epilogue and the forward
 * transforms), ms_out[1] the z pass of that step (the z line pass, or the zy
 * pass of the sub-plane form).  Both 0 when the context has no fused step.
 * No counterpart in the reference; used for the roofline report. */
int sep_time_fused_step(sep_ctx *ctx, long npairs, int reps, double *ms_out);

/* ---- normalisation that allocates nothing ------------------------------
 * filter/norm.c:40-54 (psi_m <- psi_m / sqrt(dv sum_g psi_m(g)^2)) on m real
 * states of ngrid doubles already on the device, psi_dev state-major.  No
 * counterpart in the reference (which normalises host arrays, and whose
 * drop-in here, sep_normalize_states, copies them to the device and
 * allocates on each call).  This one calls no cudaMalloc/cudaFree or any
 * other allocating routine, for callers that cannot allocate at that point:
 * code running while another allocator (a framework's caching pool) holds
 * the device's memory, and loops that must not wait on cudaMalloc/cudaFree.
 *  - Scratch: a fixed 2,105,344-byte array in the library's device image (one
 *    per device); nothing in it needs to start at zero.
 *  - Limit: m <= 1024 states per call (SEP_ERR_ARG above that; split the
 *    block).  ngrid is not limited.
 *  - Device: the calling thread's current device; psi_dev must live there.
 *    Each call made outside stream capture looks up the scratch address in
 *    the current context (cudaGetSymbolAddress), so it stays valid after
 *    cudaDeviceReset and in non-primary contexts; a call made while
 *    cuda_stream captures reuses the last address found on that device, so
 *    make the first call on each device before any stream capture begins
 *    (a first call during capture returns SEP_ERR_ARG).
 *  - Asynchronous on cuda_stream (a cudaStream_t; NULL = the legacy default
 *    stream): the states are normalised when the stream reaches the call.
 *  - Calls that overlap on one device (other streams or threads, not
 *    ordered by the caller) share the scratch and race: serialise them. */
int sep_normalize_states_noalloc(double *psi_dev, long m, long ngrid, double dv,
                                 void *cuda_stream);

/* ---- output files ---------------------------------------------------------
 * Byte for byte what the reference's stdio calls write; no device needed.
 * sep_write_states: m raw FP64 state blocks of ngrid values, no header
 *   (psi.dat, filter/main.c:129-131; psi-filt-<tid>-<jns>.dat,
 *   filter/filter.c:44-47).  Large files are written by a team of threads.
 * sep_write_eval: "%ld %.16g %g\n" = index, E, sigma per line (eval.dat,
 *   filter/main.c:138-142).
 * sep_write_filter_eval: "%ld %.16g %.16g\n" = index, E, target per line
 *   (eval-filt-<tid>-<jns>.dat, filter/filter.c:37-41).
 * SEP_ERR_IO when a file cannot be created or written. */
int sep_write_states(const char *path, const double *psi, long m, long ngrid);
int sep_write_eval(const char *path, const double *eval, const double *sige, long m);
int sep_write_filter_eval(const char *path, const double *eval, const double *el, long ms);

/* ---- merge of several filter runs (combine_filter_outputs.py) -------------
 * The step between the filter and bse/: reads eval_name (default eval.dat)
 * and psi_name (default psi.dat) in each of the ndatasets directories, sorts
 * every state by (E, sigma, run, index in run) and writes into output_dir
 * (default merged_filter, created with its parents):
 *   eval.par             "%d %.16g %.16g\n" with the new indices;
 *   psi.par              the state blocks in the new order;
 *   merge_manifest.txt   ngrid, nstates, the sources and the mapping;
 *   conf.par             a copy of the first run's, when copy_conf != 0.
 * The checks and messages are the script's (combine_filter_outputs.py:
 * 125-214, 250-263): a missing file, a line with fewer than 3 columns or a
 * field that Python's int()/float() rejects, an empty eval file, an
 * input.par whose nx ny nz disagree with ngrid, a psi file whose size is not
 * nstates x ngrid doubles, indices not 0..n-1, conf.par files that differ,
 * copy_conf without a first conf.par.  Those return SEP_ERR_ARG with the
 * script's message in sep_last_error(); a file that cannot be opened, read
 * or written returns SEP_ERR_IO.  nstates (ndatasets entries) and total may
 * be NULL.  The state blocks are copied by a team of threads. */
int sep_combine_outputs(int ndatasets, const char *const *dirs, const char *eval_name,
                        const char *psi_name, long ngrid, const char *output_dir,
                        int copy_conf, long *nstates, long *total);
/* nx*ny*nz from the first three integers of an input.par (filter or bse),
 * combine_filter_outputs.py:125-145; SEP_ERR_ARG with the script's message
 * when they are missing, not integers or not positive. */
int sep_read_grid_source(const char *path, long *ngrid);

/* ---- bulk band structures and their gradient (pseudopotFitting/) ---------
 * The empirical-pseudopotential fit to bulk band structures.  No device work
 * in sep_bulk_basis.
 * sep_bulk_basis: the plane waves G = i b0 + j b1 + k b2 with |G|^2 / 2 <
 *   max_ke for the cell rows a0, a1, a2 (bohr; init.c:21-45,
 *   states.c:10-61), ordered by |G|.  g == NULL: *nbv only; else g holds
 *   cap >= *nbv vectors (x, y, z).
 * sep_bulk_create: one crystal on the calling thread's device: nbv plane
 *   waves g, natom atoms tau (bohr) with types[a] in [0, ntype), ntype <= 8,
 *   nk k-points (bohr^-1), the kinetic scale s of H = s |k+G|^2 / 2 + V
 *   (input.par kineticEnergyScaling) and nev <= nbv bands kept per k-point.
 * sep_bulk_bands: params = ntype x {a0, a1, a2, a3} of
 *   v(q) = a0 (q^2 - a1) / (a2 exp(a3 q^2) + 1) (hamiltonian.c:91-94);
 *   bands = nk x nev lowest eigenvalues in eV (fit.c:71-97: V once, H_k for
 *   all k-points, one batched Hermitian eigensolve of the lowest nev + 16
 *   eigenpairs).
 * sep_bulk_bands_backward: given dL/dE (nk x nev, per eV), writes
 *   dL/dparams (ntype x 4) by Hellmann-Feynman (no reference counterpart:
 *   the reference fits by Monte Carlo, fit.c:9-69), and the bands when
 *   bands != NULL.  Where a k-point has degenerate bands (equal to 1e-10
 *   relative) with unequal dL/dE, the sorted bands are not differentiable;
 *   per parameter the result is then the limit of central differences,
 *   from degenerate perturbation theory on each cluster (the eigenvalues of
 *   U_c^H dV/dtheta U_c, up to 16 bands per cluster; bands past nev in a
 *   cluster count with dL/dE = 0).
 * sep_bulk_solver_path: 2 when the library's batched solver ran, 1 when
 *   cuSOLVER's batched eigensolver ran, 0 when the matrices went to cuSOLVER
 *   one per call, -1 before the first solve.
 * sep_bulk_set_eigensolver: 1 (default) = the library's batched solver (one
 *   CTA per k-point, up to 512 plane waves; larger bases use cuSOLVER);
 *   0 = cuSOLVER.
 * sep_bulk_set_solver: for cuSOLVER, 1 (default) = its batched eigensolver,
 *   one matrix per call where it declines the size; 0 = one matrix per call. */
typedef struct sep_bulk sep_bulk;
int sep_bulk_basis(const double cell[9], double max_ke, long cap, long *nbv, double *g);
int sep_bulk_create(long nbv, const double *g, long natom, const double *tau, const int *types,
                    long ntype, long nk, const double *kpts, double ke_scale, long nev,
                    sep_bulk **out);
int sep_bulk_bands(sep_bulk *b, const double *params, double *bands);
/* sep_bulk_bands that also keeps the eigenvectors: a following
 * sep_bulk_bands_backward with the same params reuses this solve. */
int sep_bulk_bands_keep(sep_bulk *b, const double *params, double *bands);
int sep_bulk_bands_backward(sep_bulk *b, const double *params, const double *dl_de,
                            double *bands, double *dl_dparams);
int sep_bulk_solver_path(sep_bulk *b, int *batched);
int sep_bulk_set_solver(sep_bulk *b, int batched);
int sep_bulk_set_eigensolver(sep_bulk *b, int mode);
/* The library's batched Hermitian solver on host arrays: a = nmat matrices
 * of order n (2 <= n <= 512), complex interleaved (re, im), column-major,
 * both triangles; w = nmat x nw lowest eigenvalues ascending (nw <= 64);
 * with vectors, v = nmat x nw unit eigenvectors of n complex each (the
 * matrix's first nw columns).  Replaces one zheev per k-point
 * (pseudopotFitting/diag.c:12-48) keeping the lowest bands (fit.c:86-88). */
int sep_hermitian_lowest(const double *a, long n, long nmat, long nw, int vectors, double *w,
                         double *v);
int sep_bulk_destroy(sep_bulk *b);

/* ---- spin-orbit operator of the spinor filter (spinors/filterSpinors/) ----
 * One neighbour-list entry, laid out as the reference's nlc_st
 * (spinors/filterSpinors/fd.h:55-60), so its nlc arrays pass unchanged:
 * grid index, the l = 1 harmonics Y10, Y11, Y1-1 (re, im), the
 * Kleinman-Bylander radial factors, r, 1/r^2, r^2 and Vso(r). */
typedef struct {
  long jxyz;
  double y10[2], y11[2], y1_1[2];
  double Vs0G1, Vs0G_2;
  double r, r2_1, r2, Vr;
} sep_nlc;
/* psinl = Vso psi for spinors of 2 ngrid complex values (interleaved re, im;
 * the spin-up grid, then the spin-down grid).  natom atoms, each with nl[a]
 * entries at nlc[a * nnlc].  flagkb = 0: the Gaussian form of
 * filterSpinors/hamiltonian.c:81-190 with delta width sigma (sigma_1 =
 * sqrt(1/2)/sigma as filterSpinors/init.c:96-97); flagkb = 1: the
 * Kleinman-Bylander form of hamiltonian.c:193-401 with elkb = 2 natom
 * energies (G1 block, then G_2).  dv = the volume element.  psinl is
 * overwritten.  sep_spinor_vso takes host arrays and checks that every
 * jxyz lies on the grid; sep_spinor_vso_dev takes device arrays (already
 * checked) and runs on cuda_stream (a cudaStream_t; NULL = the legacy
 * default stream). */
int sep_spinor_vso(const double *psi, long ngrid, long natom, long nnlc, const sep_nlc *nlc,
                   const long *nl, double sigma, double dv, int flagkb, const double *elkb,
                   double *psinl);
int sep_spinor_vso_dev(const double *psi, long ngrid, long natom, long nnlc,
                       const sep_nlc *nlc, const long *nl, double sigma, double dv, int flagkb,
                       const double *elkb, double *psinl, void *cuda_stream);
/* The neighbour lists of filterSpinors/init.c:114-181 (init_list), entry
 * for entry: for atom a at rxyz[3a..3a+2] (bohr) the points of the grid
 * vx[nx] x vy[ny] x vz[nz] (x fastest) with squared distance below rnlcut2,
 * Vr = vso[a] exp(-r^2 / 0.49), the harmonics and r, 1/r^2, r^2; Vs0G1 and
 * Vs0G_2 are left 0 (filterSpinors/init.c:183+ fills them for the
 * Kleinman-Bylander form).  nl[a] receives the count.  nlc == NULL: counts
 * only (to size nnlc); else nlc holds natom x nnlc entries and a count above
 * nnlc is SEP_ERR_ARG (the reference would write past its array).  Host
 * only; each atom visits only the box of grid lines within its radius. */
int sep_spinor_neighbour_lists(long nx, long ny, long nz, const double *vx, const double *vy,
                               const double *vz, long natom, const double *rxyz,
                               const double *vso, double rnlcut2, long nnlc, sep_nlc *nlc,
                               long *nl);

/* ---- the spinor filter program (spinors/filterSpinors/) -------------------
 * Spinors: 2 ngrid complex values (interleaved re, im doubles), the spin-up
 * grid then the spin-down grid; H = T + V on each component grid plus the
 * spin-orbit operator Vso of sep_spinor_vso.  All in FP64, on the context's
 * grid and local potential.
 * sep_spinor_set_operator: the neighbour lists (natom x nnlc sep_nlc, nl[a]
 *   used per atom, every jxyz on the grid), sigma (Gaussian form) or
 *   flagkb = 1 with elkb (2 natom energies); copied to the device, kept by
 *   the context until set again.
 * sep_spinor_hamiltonian: hpsi = H psi for nspinors spinors
 *   (filterSpinors/hamiltonian.c:8-46).
 * sep_spinor_energy_range: filterSpinors/energy.c:49-109 from four
 *   component grids that init_psi draws from the seed -874917403: Emin by
 *   phi <- normalise(psi - 0.025 H psi), Emax by power iteration, each to a
 *   relative change of 1e-6 or 500 steps; *vmin = Emin - 0.2 |Emin|,
 *   *dE = 1.2 Emax - *vmin.
 * sep_spinor_filter: filterSpinors/filter.c:48-80 for ns start spinors:
 *   out[s][e] = sum_j (an_re + i an_im)[e][j] psi_j, psi_0 = start[s],
 *   psi_j = dE_1 H psi_{j-1} - (2 + zn[j-1] + vmin dE_1) psi_{j-1};
 *   an_re, an_im: ms x nc (ms <= 16); out: ns x ms spinors.
 * sep_spinor_pipeline: filterSpinors/main.c:84-175 from given start spinors
 *   (ns x 2 ngrid complex): energy range (dE <= 0: computed, vmin then
 *   comes from it), coefficients, filter, normalisation, ortho (the Gram
 *   scheme of sep_ortho on the Hermitian Gram matrix, keeping singular-value
 *   ratios >= 1e-10 like filterSpinors/ortho.c's zgesvd), Rayleigh-Ritz
 *   (filterSpinors/Hmat.c), sigma = |H psi - E psi| (energy.c:114-145).
 *   psi_out (optional): the *mkept Ritz spinors; eval, sige: ns ms entries. */
int sep_spinor_set_operator(sep_ctx *ctx, long natom, long nnlc, const sep_nlc *nlc,
                            const long *nl, double sigma, int flagkb, const double *elkb);
int sep_spinor_hamiltonian(sep_ctx *ctx, const double *psi, double *hpsi, long nspinors);
int sep_spinor_energy_range(sep_ctx *ctx, double *vmin, double *dE, long *iters);
int sep_spinor_filter(sep_ctx *ctx, const double *start, long ns, const double *an_re,
                      const double *an_im, const double *zn, long ms, long nc, double dE_1,
                      double vmin, double *out);
int sep_spinor_pipeline(sep_ctx *ctx, const double *start, long ns, const double *el, long ms,
                        long nc, double vmin, double dE, double *psi_out, double *eval,
                        double *sige, long *mkept, sep_timing *timing);

#ifdef __cplusplus
}
#endif
#endif
