/*
 * nmgpu.h -- C-ABI of the GB300 (sm_103a) eigensolver for planetary normal
 * modes: the drop-in for the operator callbacks and the eigensolve driver of
 * js1019/NormalModes.
 *
 * The reference hands pEVSL three callbacks with the Fortran signature
 * (v, w, mymv) -- v, w real*8(n_loc) by reference, mymv the opaque
 * `type(mvparameters)` context (src/mod_cg_datatype.f90:88-115):
 *
 *   sparseAV   src/mod_matvec.f90:445-458   w = D A D v            (solid only)
 *   sparsefsAV src/mod_matvec.f90:498-520   w = D(Ad D v + E D_p Cheb_Ap(D_p ET D v))
 *   sparseBV   src/mod_matvec.f90:461-472   w = B_s v
 *   solveBV    src/mod_matvec.f90:475-483   w = Cheb_B(v)   (pEVSL chebiter type 2)
 *
 * registered at src/mod_pevsl.f90:69-80, and runs the whole solve in
 * `pnm_apply_pevsl` (src/mod_pevsl.f90:16-222).  Here one opaque nm_ctx owns
 * the operators on one GPU; nm_amv / nm_bmv / nm_bsolve are the callbacks
 * (host vectors, or device vectors with the *_dev variants) and nm_solve is
 * the whole filtered-Lanczos solve, so the Krylov basis never leaves the GPU.
 *
 * Conventions: 0-based int32 CSR (`col - 1` of src/mod_matvec.f90:59), float64
 * values, the caller keeps ownership of every array it passes (the library
 * copies), every entry point returns an NM_* status, nm_last_error() explains
 * the last failure of a context.  Calls on one context are not thread-safe;
 * distinct contexts are independent.  There is no CPU fallback: without a
 * usable GPU nm_create fails with NM_ERR_CUDA.
 */
#ifndef NMGPU_H
#define NMGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NM_OK 0
#define NM_ERR_ARG (-1)     /* bad argument / inconsistent sizes            */
#define NM_ERR_CUDA (-2)    /* CUDA runtime error or no usable device        */
#define NM_ERR_OOM (-3)     /* device allocation failed                      */
#define NM_ERR_NOCONV (-4)  /* Lanczos hit MAXIT before the trace converged  */
#define NM_ERR_TIMEOUT (-5) /* a bounded device-side wait gave up            */
#define NM_ERR_NUMERIC (-6) /* non-positive diagonal, NaN/Inf, breakdown     */

/* One CSR matrix, 0-based. */
typedef struct {
  int nrows, ncols;
  const int* rowptr; /* nrows + 1 */
  const int* col;    /* rowptr[nrows] */
  const double* val; /* rowptr[nrows] */
} nm_csr;

typedef struct {
  int porder;        /* pOrder of global_conf: 1 or 2 (selects Chebyshev degrees) */
  int device;        /* CUDA device ordinal                                      */
  int b_cheb_deg;    /* 0: 45 (P2) / 25 (P1), src/mod_matvec.f90:88-92           */
  int ap_cheb_deg;   /* 0: max(min(int(cond),15)*3,100) (P2) / 25 (P1), :167-171  */
  double b_bounds[2];  /* if b_bounds[1] > 0: use instead of Lanczos bounds of B_s */
  double ap_bounds[2]; /* idem for Ap_s                                           */
  int precision;     /* NM_PREC_FP64 or NM_PREC_MIXED (FP32 filter SpMVs)        */
  int verbose;       /* print the reference's progress lines                      */
  /* Mixed-precision block path; 0 everywhere gives the measured defaults.      */
  int filter_form;   /* 0: range form W = p(0) Z + A B~^-1 Y (last A-op in FP64,
                        no FP32 rounding in the zero-frequency modes); 1: the
                        plain FP32 filter                                        */
  int orth;          /* block Gram-Schmidt of the mixed path against the FP32
                        basis copies: 0 the projection V^T W on the tensor cores
                        (tcgen05, 3xTF32) where the GPU has them, else cuBLAS
                        SGEMM; 1 FP64 (DGEMM on the FP64 basis); 2 SGEMM     */
  double inner_tol;  /* relative accuracy of the FP32 filter's inner B~^-1
                        Chebyshev solve, which sets its degree (0: 2^-24, FP32;
                        < 0: the reference's degree)                           */
  int autotune;      /* 0: time the gather kernels' launch shapes on the first
                        block use; -1: keep the default shapes                  */
} nm_opts;

#define NM_PREC_FP64 0
#define NM_PREC_MIXED 1

/* Progress of nm_solve: called on the calling thread with the context's
 * stream synchronised, at the end of each phase and after every Lanczos step
 * (single vector) or block step (block path) and every refined block of Ritz
 * vectors; `done` of `total` units of the phase (total -1 when open-ended).
 * The reference prints the same milestones (src/mod_pevsl.f90:84-134). */
typedef void (*nm_progress_fn)(void* data, int phase, int done, int total);
#define NM_PHASE_BOUNDS 0  /* bounds of B^-1 A (LANBOUNDS) known                */
#define NM_PHASE_LANCZOS 1 /* one more Lanczos step / block step; total = MAXIT */
#define NM_PHASE_RITZ 2    /* Ritz vectors formed (first Rayleigh-Ritz done)     */
#define NM_PHASE_REFINE 3  /* one more block of Ritz vectors refined / checked  */
#define NM_PHASE_DONE 4    /* residual check done, results copied                */

typedef struct {
  int maxit;          /* 0: 3*max(4*802,2000) = 9624 (src/mod_pevsl.f90:116-119) */
  double tol;         /* 0: 1e-5 (src/mod_pevsl.f90:52)                            */
  double thresh_int;  /* 0: 0.8 (src/mod_pevsl.f90:108)                            */
  double thresh_ext;  /* 0: 0.7 (src/mod_pevsl.f90:109)                            */
  int mlan_bounds;    /* 0: 3000 (src/mod_pevsl.f90:49)                            */
  double ab_bounds[2];/* if ab_bounds[1] > 0: skip LANBOUNDS(B^-1 A), use these    */
  int damping;        /* 0/1: Jackson, 2: Lanczos sigma                            */
  int want_vectors;   /* copy eigenvectors to the result                           */
  int unscale;        /* vectors as x = y .* D (src/mod_pevsl.f90:199) not y       */
  int use_graph;      /* capture the filter in a CUDA graph (default on)           */
  int block;          /* 0/1: single-vector ChebLanNr (the reference's algorithm);
                         32: block filtered Lanczos, 32 vectors per filter pass  */
  int polish;         /* mixed block path, refinement of the Ritz vectors towards
                         FP64 residuals: 0 adaptive (degree per block of 32 Ritz
                         vectors from their measured FP64 residuals, until
                         err_ref <= resid_tol); > 0 a fixed plan of that degree
                         for the lowest block (capped at 2 sqrt(lmax / (b - a)));
                         < 0 off                                               */
  double resid_tol;   /* adaptive refinement target for err_ref (0: 1e-10)        */
  int refine_sweeps;  /* adaptive refinement: at most this many passes, each
                         closed by an FP64 Rayleigh-Ritz (0: until the wanted
                         Ritz vectors meet resid_tol, at most 6, stopping when
                         a pass no longer halves their largest residual)     */
  int refine_maxdeg;  /* adaptive refinement: degree cap per block (0: 4000)      */
  double refine_band; /* adaptive refinement: the damped band starts at this
                         multiple of the block's largest Ritz value (0: 8)     */
  int refine_purge;   /* adaptive refinement polynomial: 0 or 1 with the factor
                         x / theta, which removes the Ritz vectors' content in
                         the null space of A (the zero-frequency fluid modes);
                         -1 without it                                          */
  nm_progress_fn progress; /* host callback at phase boundaries (NULL: none)      */
  void* progress_data;     /* first argument of progress                          */
  double refine_guard; /* adaptive refinement: the Ritz vectors with Rayleigh
                          quotients in (b, g b] and [a / g, a) join the
                          refinement and every Rayleigh-Ritz pass as guards
                          (then dropped), g = this (0: 1.5; <= 1: no guards)  */
  double refine_near;  /* adaptive refinement passes after the first: the damped
                          band starts at this multiple of the largest guarded
                          Ritz value, or higher where the polynomial would grow
                          by more than refine_growth below a block's Ritz
                          values (0: 1.05; < 0: every pass uses refine_band)  */
  double refine_growth; /* see refine_near (0: 1e3)                             */
} nm_solve_opts;

typedef struct {
  int nev;            /* eigenpairs found in [a, b]                                */
  int n;              /* vector length                                              */
  double* lam;        /* nev, ascending                                             */
  double* vec;        /* n * nev column-major (if want_vectors), else NULL          */
  double* err_ref;    /* sqrt(sum (Ay - lam By)^2 / N) / |lam|, src/mod_pevsl.f90:158 */
  double* res2;       /* ||Ay - lam By||_2 / |lam| with ||y||_B = 1                  */
  double xintv[4];    /* [a, b, lmin, lmax] of src/mod_pevsl.f90:93-103              */
  int pol_deg;        /* filter degree                                               */
  double pol_gam, pol_bar;
  int lanczos_steps;
  int nritz_above_bar;
  double t_bounds, t_filter_design, t_lanczos, t_ritz, t_total; /* seconds        */
  long long n_amv, n_bsolve, n_spmv; /* operator applications / SpMV launches       */
  long long n_kernels;   /* kernels of this library launched by the solve            */
  double t_filter;       /* block path: seconds in the filter applications (CUDA events) */
  double t_orth;         /* block path: seconds in the block Gram-Schmidt (CUDA events)  */
  double t_eig;          /* block path: seconds in the projected (block-tridiagonal) eigensolves */
  int refine_passes;     /* mixed block path, adaptive refinement: passes run (each
                            closed by an FP64 Rayleigh-Ritz)                        */
  int refine_blocks;     /* blocks of 32 Ritz vectors refined, over all passes      */
  int refine_maxdeg;     /* largest refinement degree                               */
  long long refine_steps;      /* block degree steps spent refining                 */
  double res2_before_refine;   /* largest res2 of the Ritz vectors before refining  */
  int refine_guards;     /* guard Ritz vectors (quotients just outside [a, b]) that
                            took part in the refinement                          */
} nm_result;

typedef struct nm_ctx nm_ctx;

/* Operator construction: replaces setupmatvec (src/mod_matvec.f90:24-250).
 * Solid-only model: A = stiffness, Ap = E = ET = NULL.  Fluid-solid model:
 * A = Ad, plus Ap (reference sign, negative definite), E, ET.  The library
 * computes D = diag(B)^-1/2, D_p = diag(-Ap)^-1/2, the scaled operators, the
 * Lanczos bounds of B_s and Ap_s and the Chebyshev set-ups itself.
 * *out is set in every case but a NULL out: on failure it holds the context
 * with the error message (nm_last_error), and the caller calls nm_destroy. */
int nm_create(nm_ctx** out, const nm_csr* A, const nm_csr* B, const nm_csr* Ap, const nm_csr* E,
              const nm_csr* ET, const nm_opts* opts);
void nm_destroy(nm_ctx* ctx);
void nm_default_opts(nm_opts* o);
void nm_default_solve_opts(nm_solve_opts* o);

/* Callbacks, host vectors of length n (copies in and out). */
int nm_amv(nm_ctx* ctx, const double* x, double* y);    /* sparseAV / sparsefsAV */
int nm_bmv(nm_ctx* ctx, const double* x, double* y);    /* sparseBV              */
int nm_bsolve(nm_ctx* ctx, const double* x, double* y); /* solveBV               */
/* Same on device pointers, enqueued on the context's stream (no sync). */
int nm_amv_dev(nm_ctx* ctx, const double* x, double* y);
int nm_bmv_dev(nm_ctx* ctx, const double* x, double* y);
int nm_bsolve_dev(nm_ctx* ctx, const double* x, double* y);
/* nm_bsolve_dev that allocates nothing.  No counterpart in the reference: it
 * is an addition of this library for callers that must not allocate device
 * memory (cudaMalloc/cudaFree can synchronize the device, and a context
 * sized for the largest models leaves no headroom).  Same arithmetic and
 * the same result bits as nm_bsolve_dev, enqueued on the context's stream
 * (no sync); its Chebyshev work vectors live in one scratch array compiled
 * into the library (4 x NM_NOALLOC_MAX_ROWS doubles = 40 MiB per device),
 * not in the context.
 *  - Rejects n > NM_NOALLOC_MAX_ROWS with NM_ERR_ARG (see nm_last_error).
 *  - The first call on a device looks the scratch address up
 *    (cudaGetSymbolAddress with the context's device current); make that
 *    first call before any stream capture.  The address is kept for the
 *    life of the process: after cudaDeviceReset of that device it is stale,
 *    so do not call this entry point on a device that was reset.
 *  - Nothing in the scratch has to start at zero: each call writes every
 *    row of its work vectors before reading it.
 *  - All calls on a device share the scratch, across contexts: calls that
 *    overlap on the GPU race and give undefined results. */
#define NM_NOALLOC_MAX_ROWS 1310720
int nm_bsolve_dev_noalloc(nm_ctx* ctx, const double* x, double* y);
/* Blocks of ncols column vectors with leading dimension ld (host memory). */
int nm_amv_block(nm_ctx* ctx, const double* X, double* Y, int ncols, int ld);
int nm_bmv_block(nm_ctx* ctx, const double* X, double* Y, int ncols, int ld);
int nm_bsolve_block(nm_ctx* ctx, const double* X, double* Y, int ncols, int ld);

/* The whole solve of pnm_apply_pevsl for [f_lo, f_hi] mHz. */
int nm_solve(nm_ctx* ctx, double f_lo_mhz, double f_hi_mhz, const nm_solve_opts* opts, nm_result* res);
void nm_result_free(nm_result* res);

/* Spectrum slicing (the reference runs one interval per job): solves every
 * slice [f_lo_mhz, f_hi_mhz] on the same context, one after another, with the
 * same options, into results[i] (nslices results, each freed with
 * nm_result_free).  Returns NM_OK, the first NM_ERR_NOCONV after finishing
 * the other slices, or the first other error (results of the slices before
 * it stay valid). */
typedef struct {
  double f_lo_mhz, f_hi_mhz;
} nm_slice;
int nm_solve_batched(nm_ctx* ctx, const nm_slice* slices, int nslices, const nm_solve_opts* opts,
                     nm_result* results);

/* Spectrum slicing by a kernel-polynomial (KPM) estimate of the eigenvalue
 * density of B^-1 A.  No counterpart in the reference (one interval per
 * job); the method is pEVSL's kpmdos + spslicer (Lin, Saad & Yang, SIAM
 * Review 58, 2016), on the lambda-weighted density so that the zero modes of
 * a fluid-solid pencil do not leak into the count:
 *   mu_k = tr(T_k(S) B^-1 A) / n,  S = (B^-1 A - c) / e,  c, e the centre and
 *   half-width of [lmin, lmax],
 * estimated with nvec Rademacher vectors.  The count of (a, b] is the
 * integral of the Jackson-damped expansion divided by lambda. */
typedef int (*nm_block_op)(void* data, const double* X, double* Y, int ncols, int ld); /* Y = B^-1 A X */
typedef struct {
  int degree;              /* 0: nm_kpm_degree for the interval and slice count       */
  int nvec;                /* random vectors (0: 16)                                  */
  unsigned long long seed;
  double ab_bounds[2];     /* bounds of B^-1 A; ab_bounds[1] <= 0: Lanczos bounds as in nm_solve */
} nm_kpm_opts;
void nm_default_kpm_opts(nm_kpm_opts* o);
/* Degree whose Jackson kernel (about pi / d wide in theta = acos(t),
 * t = (lambda - c) / e) is a quarter of the mean slice width in theta:
 * 4 pi nslices / (theta(lam_lo) - theta(lam_hi)), clamped to [50, 4000];
 * 0 for bad arguments. */
int nm_kpm_degree(double lmin, double lmax, double lam_lo, double lam_hi, int nslices);
/* Moments mu[0..degree] through a block operator (host arrays, n x ncols,
 * leading dimension ld); runs on the host, so any operator will do. */
int nm_kpm_moments(nm_block_op op, void* data, int n, double lmin, double lmax, int degree, int nvec,
                   unsigned long long seed, double* mu);
/* The same moments (same Rademacher vectors and estimator) on the device:
 * B^-1 A applied to 32-column blocks with the context's block operators (in
 * FP32 for a mixed-precision context, FP64 otherwise), one on-device dot per
 * degree and no host round trip until the end.  NM_ERR_ARG if the context has
 * no block operators (then use nm_kpm_moments with nm_amv_block +
 * nm_bsolve_block). */
int nm_kpm_moments_ctx(nm_ctx* ctx, double lmin, double lmax, int degree, int nvec, unsigned long long seed,
                       double* mu);
/* Estimated number of eigenvalues in (lam_lo, lam_hi], lam_lo > 0. */
int nm_kpm_count(const double* mu, int degree, int n, double lmin, double lmax, double lam_lo, double lam_hi,
                 double* count);
/* nslices slices of [f_lo_mhz, f_hi_mhz] (f_lo_mhz > 0) with equal estimated
 * counts; counts (nullable) receives the estimate per slice.  Frequencies
 * map to eigenvalues as in nm_solve (src/mod_pevsl.f90:93-99). */
int nm_kpm_slices(const double* mu, int degree, int n, double lmin, double lmax, double f_lo_mhz, double f_hi_mhz,
                  int nslices, nm_slice* out, double* counts);
/* All of the above on a context: Lanczos bounds (unless given), moments
 * (nm_kpm_moments_ctx, or through nm_amv_block + nm_bsolve_block when the
 * context has no block operators), slices for nm_solve_batched. */
int nm_slice_spectrum(nm_ctx* ctx, double f_lo_mhz, double f_hi_mhz, int nslices, const nm_kpm_opts* opts,
                      nm_slice* out, double* counts);

/* Adjoint sensitivities.  No counterpart in the reference (it has no
 * gradients); the element model is the mesh, DOF map and nodal material of
 * the assembly behind the context's operators (nmm_mesh_arrays and
 * nmm_reference return exactly these arrays).  All host arrays, borrowed for
 * the call.  With g0 set (operators assembled with the reference gravity,
 * JOB = 2) the gravity terms are differentiated too, the field held fixed
 * (nm_adjoint_gravity). */
typedef struct {
  int ntet, pnp, nnode;
  int fluid_solid;                  /* 1: fluid-solid (general) model              */
  const int* tets;                  /* pnp*ntet, reference-element local order     */
  const double* xyz;                /* 3*nnode                                      */
  const unsigned char* fluid;       /* ntet                                         */
  const int* vstt;                  /* nnode: first displacement DOF (solid copy)   */
  const int* rnum;                  /* nnode: 3, or 6 at fluid-solid nodes          */
  const int* pstt;                  /* nnode: pressure DOF, -1 if none              */
  const double *vp, *vs, *rho;      /* pnp*ntet nodal material                      */
  const double* ref_mass;           /* pnp*pnp, row-major                           */
  const double* ref_drst;           /* 3*pnp*pnp, d/dr, d/ds, d/dt                  */
  const double* g0;                 /* 3*pnp*ntet reference gravity (m/s^2) or NULL  */
  const double* ref_massf;          /* 4*nfp*nfp face masses (needed with g0)        */
  const int* ref_fmask;             /* 4*nfp face node lists, 0-based (with g0)      */
} nm_elem_model;

/* The reference-gravity terms of the sensitivities (JOB = 2,
 * src/mod_cg_create_matrix.f90:192-265, 329-377, 492-705, 866-920): ADDS
 * them to grad (k x ntet x 3, per pair) for unscaled eigenvectors X
 * (n x k, leading dimension ldx) and their pressures P (np x k, ldp; NULL
 * for a solid model).  Host code, no GPU; nm_adjoint calls it when em->g0
 * is set. */
int nm_adjoint_gravity(const nm_elem_model* em, int k, const double* X, int ldx, const double* P, int ldp,
                       double* grad);

#define NM_ADJ_PAIR 0      /* one gradient per eigenpair                          */
#define NM_ADJ_MULTIPLET 1 /* one per group of eigenvalues within tol (relative) */

/* dlam/dm_e = x^T (dA/dm_e - lam dB/dm_e) x for every element e and
 * m = (density, bulk modulus, shear modulus), where dm_e shifts all nodal
 * values of m in element e by the same amount and the other two parameters
 * stay fixed.  For a fluid-solid model x is completed by its pressure
 * p = -Ap^-1 ET x (the context's Chebyshev approximation of Ap^-1, the same
 * one its A-operator applies), and the pressure block enters through the
 * fluid elements' bulk modulus; fluid elements have no shear gradient (0).
 * The element matrices are recomputed on the GPU, not stored.
 *   lam : k eigenvalues (ascending), X : n x k unscaled eigenvectors with
 *         x^T B x = 1 (nm_solve with unscale = 1), column-major, ld ldx.
 *   grad: (k or ngroups) x ntet x 3 doubles, [.][e][0:rho, 1:kappa, 2:mu].
 *   group (k ints, may be NULL) receives each pair's group, *ngroups their
 *   count (a group is a run of consecutive eigenvalues closer than tol,
 *   relative); NM_ADJ_MULTIPLET sums the pairs of a group (basis-independent for
 *   a degenerate multiplet). */
int nm_adjoint(nm_ctx* ctx, const nm_elem_model* em, int k, const double* lam, const double* X, int ldx, int mode,
               double tol, double* grad, int* group, int* ngroups);

/* Element-level assembly of the JOB = 1 operators on the GPU (no gravity):
 * the element matrices of CGE3D_ISO / CGFSE3D_ISO (src/mod_cg_create_matrix.f90:
 * 103-1266: solid elements, fluid elements, fluid-solid interface faces)
 * computed per tetrahedron on the device and added into the given CSR
 * structures (:1269-2033).  em: the mesh, DOF map, nodal material and
 * reference element (as for nm_adjoint; g0 must be NULL).  Each nm_csr_fill
 * gives a structure (host rowptr/col, 0-based, sorted columns) and receives
 * its values (host val, overwritten); solid model: A and B (Ap, E, ET NULL),
 * fluid-solid model: Ad (as A), B, Ap, E, ET.  seconds (nullable) receives
 * the device time of the assembly kernel.  NM_ERR_ARG if a structure lacks
 * an entry an element needs, NM_ERR_NUMERIC for a flat tetrahedron. */
typedef struct {
  int nrows;
  const int* rowptr; /* nrows + 1 */
  const int* col;    /* rowptr[nrows], ascending within each row */
  double* val;       /* rowptr[nrows], written */
} nm_csr_fill;
int nm_assemble(const nm_elem_model* em, nm_csr_fill* A, nm_csr_fill* B, nm_csr_fill* Ap, nm_csr_fill* E,
                nm_csr_fill* ET, double* seconds);


/* Introspection. */
typedef struct {
  int n, np, fs, porder, precision;
  long long nnz_a, nnz_b, nnz_ap, nnz_e, nnz_et;
  double b_bounds[2], ap_bounds[2];
  int b_cheb_deg, ap_cheb_deg;
  double t_setup;        /* seconds spent in nm_create                        */
  long long h2d_bytes;   /* bytes copied host -> device by nm_create          */
  size_t device_bytes;   /* device memory held by the context                 */
  /* launch shape of the block filter's mass and Ap Chebyshev gathers picked
   * by the autotuner (vec 1: 16-byte gathers; -1 before the first block use) */
  int mass_vec, mass_threads, ap_vec, ap_threads;
  /* row schedule of those (1: one contiguous row range per CTA, 0: a few
   * rows per CTA) and the CTA size / schedule of the block A-op kernels */
  int mass_sweep, ap_sweep, aop_threads, aop_sweep;
} nm_info;
int nm_get_info(nm_ctx* ctx, nm_info* info);
void* nm_get_stream(nm_ctx* ctx); /* cudaStream_t of the context */
const char* nm_last_error(nm_ctx* ctx);
int nm_sync(nm_ctx* ctx);

/* Kernel-level timing of the dominant operators (CUDA events on the
 * context's stream), for roofline reporting: runs `reps` back-to-back
 * applications of the selected operator on device vectors and returns the
 * mean time per application in milliseconds and the algorithmic bytes one
 * application moves.  which: 0 = A-op, 1 = B SpMV, 2 = B Chebyshev solve,
 * 3 = one filter degree step (B-solve + A-op + recurrence); block (32-column,
 * in the context's precision): 4 = mass Chebyshev solve, 5 = A-op, 6 = one
 * filter degree step. */
int nm_time_op(nm_ctx* ctx, int which, int reps, double* ms_per_op, double* bytes_per_op, int* launches_per_op);

#ifdef __cplusplus
}
#endif
#endif
