/*
 * bdda.h -- C ABI of the GB300 block-DDA solve path.
 *
 * Drop-in boundary for the reference's fast operator and block solvers
 * (nmoteki/block-DDA).  Plain C types only: complex numbers are interleaved
 * {re, im} doubles (or floats for FP32 device buffers); matrices are
 * column-major with an explicit leading dimension, exactly like the Eigen
 * MatrixXcd the reference passes around (column l = right-hand side l,
 * row 3*m + c = component c of occupied dipole m).
 *
 * Every function returns BDDA_OK (0) or an error code; bdda_last_error()
 * gives the message of the calling thread's last failure.  Nothing in this
 * library calls exit(); a CUDA error is reported, not fatal.
 *
 * Thread safety: calls on one bdda_op are serialised by a lock inside the
 * operator, so host threads may call bdda_mbt_fft_mvp concurrently on a shared
 * operator (the reference calls MBT_fft_mvp from OpenMP threads on shared
 * plans, bl_krylov_mvp_fft/bl_cocg_rq_mvp_fft.cpp:38-51).
 */
#ifndef BDDA_H
#define BDDA_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define BDDA_OK 0
#define BDDA_ERR_INVALID 1      /* bad argument (size, f, pointer, box too large) */
#define BDDA_ERR_CUDA 2         /* CUDA runtime error */
#define BDDA_ERR_NOMEM 3        /* device allocation failed */
#define BDDA_ERR_BREAKDOWN 4    /* singular L x L system, failed Cholesky or NaN in a solve */
#define BDDA_ERR_NOT_CONVERGED 5 /* itermax / refinement limit reached before the tolerance */

/* ---- precision bits of an operator ----------------------------------- */
#define BDDA_PREC_FP64 1        /* complex FP64 tables (plain FP64 path, true residuals) */
#define BDDA_PREC_FP32 2        /* complex FP32 tables (mixed-precision inner solves)   */
#define BDDA_PREC_DF64 4        /* complex double-float tables: FP32 pairs hi+lo, ~48-bit significand;
                                   the mixed solve's true residuals run on them when present */

/* ---- solvers (bl_*_mvp_fft in bl_krylov_mvp_fft/DDA_linear_solvers.hpp:1-6) */
#define BDDA_SOLVER_COCG_RQ 0   /* block COCG-RQ, complex-symmetric systems  */
#define BDDA_SOLVER_BICGSTAB 1  /* block BiCGSTAB                            */
#define BDDA_SOLVER_BICGGR 2    /* block BiCGGR                              */

/* ---- solve precision -------------------------------------------------- */
#define BDDA_SOLVE_FP64 0       /* everything in complex FP64                                  */
#define BDDA_SOLVE_MIXED 1      /* complex FP32 Krylov + FFT-MVP inside FP64 iterative refinement */

typedef struct bdda_op bdda_op;

/*
 * Operator creation.  Replaces MBT_fft_init (mvp_fft/MBT_fft_init.cpp:10-42,
 * declared in MBT_utils.hpp:5): instead of returning the FFT of the 1-D MBT
 * projection Au_til, the Green-tensor spectrum on the 2x-padded 5-smooth grid
 * is built on the device and kept in the handle.
 *   n[3]        lattice box (nx, ny, nz), each 1..600 (padded FFT lines up to 1200 points)
 *   f           3 (electric dipoles, the reference's CED) or 6 (electric and
 *               magnetic dipoles, its default CEMD mode): rows f*m + c of every
 *               vector, c < 3 electric, c >= 3 magnetic
 *   lf          lattice spacing (physical length)
 *   k_re, k_im  wavenumber in the medium
 *   prec        any of BDDA_PREC_FP64, BDDA_PREC_FP32, BDDA_PREC_DF64
 */
int bdda_op_create(bdda_op** op, const int n[3], int f, double lf, double k_re, double k_im, int prec);

/* Release an operator (null is accepted). */
int bdda_op_destroy(bdda_op* op);

/*
 * Rebuild the Green spectra for a new wavenumber (the next wavelength of a
 * sweep) and keep everything else: plans, twiddles, dipoles, workspaces.  No
 * counterpart in the reference, which re-creates its Solver per wavelength and
 * target (block_DDA_main.cpp:138-163).  Waits for the operator's stream; MVPs
 * or solves the caller runs on other streams must be finished.
 */
int bdda_op_set_wavenumber(bdda_op* op, double k_re, double k_im);

/*
 * Occupied lattice sites (host array of 0-based addresses
 * ny*nz*ix + nz*iy + iz, Target_manager.cpp:98,167-169, in the caller's dipole
 * order).  Required before bdda_op_mvp_device / bdda_solve*.
 */
int bdda_op_set_dipoles(bdda_op* op, const int* address, int nocc);

/* Padded grid, dipole count and number of occupied (y, 8-wide z) lattice tiles. */
int bdda_op_info(const bdda_op* op, int P[3], int* nocc, int* ntiles);

/*
 * Reference MBT_fft_mvp (mvp_fft/MBT_fft_mvp.cpp:8-43, MBT_utils.hpp:6):
 * q_hat = A_off p_hat on the full cuboid vector of length f*nx*ny*nz (host
 * buffers, interleaved complex FP64, site-major xyz).  No diagonal.
 */
int bdda_mbt_fft_mvp(bdda_op* op, const double* p_hat, double* q_hat);

/*
 * Block MVP over the dipoles set with bdda_op_set_dipoles, device buffers,
 * all L right-hand sides in one pass:
 *   y = [diag o x +] A_off x [o jpre]
 * This is the inline block-MVP wrapper of every reference solver
 * (e.g. bl_krylov_mvp_fft/bl_cocg_rq_jacobi_mvp_fft.cpp:43-60).
 *   prec      BDDA_PREC_FP64 (double2 buffers), BDDA_PREC_FP32 (float2 buffers) or
 *             BDDA_PREC_DF64 (buffers of {re_hi, re_lo, im_hi, im_lo} floats)
 *   x, y      f*nocc x L column-major, leading dimensions ldx, ldy (>= f*nocc)
 *   diag      f*nocc complex or null (off-diagonal part only)
 *   jpre      f*nocc complex or null (no Jacobi scaling)
 *   stream    cudaStream_t or null (the operator's stream)
 */
int bdda_op_mvp_device(bdda_op* op, int prec, const void* x, int ldx, void* y, int ldy, int L,
                       const void* diag, const void* jpre, void* stream);

/*
 * Block MVP that allocates no device memory.  No counterpart in the
 * reference: it exists for callers that cannot let a library call cudaMalloc
 * -- frameworks that own all device memory through their own pool, and
 * serving loops that must never enter the CUDA allocator (which can
 * synchronise the device).  Same arguments and result as bdda_op_mvp_device
 * for prec BDDA_PREC_FP64 and BDDA_PREC_FP32 (BDDA_PREC_DF64 is rejected with
 * BDDA_ERR_INVALID), but the two FFT workspaces come from a fixed 64 MiB
 * __device__ array; boxes and nrhs whose workspace exceeds it are rejected with
 * BDDA_ERR_INVALID and a message.  The array is reserved on a device when the
 * library's code holding it is loaded there -- with CUDA's default lazy module
 * loading, at the first call of this entry point on that device -- and kept
 * until the process exits; that first call also looks up the array's device
 * address.  Make the first call at set-up, before any stream capture and
 * while the device still has 64 MiB free.  The address is kept for the life
 * of the process: a cudaDeviceReset after the first call is not supported.
 * All calls share the array: calls that overlap on the GPU race and must be
 * ordered by the caller.
 */
int bdda_op_mvp_device_noalloc(bdda_op* op, int prec, const void* x, int ldx, void* y, int ldy, int L,
                               const void* diag, const void* jpre, void* stream);

/* ---- block solvers ----------------------------------------------------- */
typedef struct {
  int solver;         /* BDDA_SOLVER_* */
  int jacobi;         /* 1: left Jacobi scaling by 1/DIAG_A (the *_jacobi_mvp_fft variants) */
  int precision;      /* BDDA_SOLVE_FP64 or BDDA_SOLVE_MIXED (a mixed refinement whose FP32 inner step breaks
                         down or gains less than a digit continues with FP64 inner solves when the
                         operator holds FP64 tables; stats->fp64_inner_steps counts them) */
  double tol;         /* reference stopping test on the recurrence error (Solver.hpp:27 default 1e-2) */
  int itermax;        /* reference iteration limit per Krylov solve (Solver.hpp:28 default 300) */
  double true_tol;    /* >0: iterate until every column's true residual ||b-Ax||/||b|| <= true_tol
                         (FP64 residuals, iterative refinement); <=0: one reference-semantics solve */
  double inner_tol;   /* refinement mode: tolerance of the first inner Krylov solve; later ones aim at the
                         reduction still needed, no tighter than min(inner_tol, 2e-5) for mixed solves
                         (0 -> automatic: 5e-5 mixed, 0.3 true_tol FP64) */
  int max_refine;     /* refinement steps limit (0 -> 8) */
  int check_every;    /* host convergence poll period in iterations (0 -> 4) */
  int warm_start;     /* 1: X holds an initial guess on entry (e.g. the solution at a neighbouring
                         wavelength) and refinement starts from B - A X; needs true_tol > 0 */
} bdda_solve_opts;

typedef struct {
  int status;             /* BDDA_OK / BDDA_ERR_BREAKDOWN / BDDA_ERR_NOT_CONVERGED */
  int iterations;         /* Krylov iterations, summed over refinement steps */
  int refinements;        /* inner solves performed */
  int mvps;               /* block MVPs performed (all precisions) */
  double final_err;       /* last recurrence error (the reference's printed value) */
  double true_res_max;    /* max over columns of ||b_l - A x_l|| / ||b_l|| (FP64), -1 if not computed */
  double ms_solve;        /* device time of the whole solve (CUDA events) */
  int fp64_inner_steps;   /* mixed solves: refinement steps run with FP64 inner solves after FP32 Krylov
                             stagnated or broke down on the system (0 normally) */
} bdda_solve_stats;

/* Fill opts with the reference defaults (COCG-RQ-Jacobi, FP64, tol 1e-2, itermax 300). */
void bdda_solve_opts_default(bdda_solve_opts* opts);

/*
 * Solve (DIAG_A + A_off) X = B for L right-hand sides.  Replaces
 * bl_cocg_rq_mvp_fft, bl_cocg_rq_jacobi_mvp_fft, bl_bicgstab_mvp_fft,
 * bl_bicgstab_jacobi_mvp_fft, bl_bicggr_mvp_fft, bl_bicggr_jacobi_mvp_fft
 * (bl_krylov_mvp_fft/DDA_linear_solvers.hpp:1-6).
 * Device buffers, complex FP64: diag[f*nocc], B (ldb), X (ldx), X is overwritten
 * (f = the operator's 3 or 6 components per dipole).
 */
int bdda_solve_device(bdda_op* op, const bdda_solve_opts* opts, const double* diag, const double* B, int ldb,
                      double* X, int ldx, int L, bdda_solve_stats* stats, void* stream);

/* Same with host buffers (copies in and out inside the call). */
int bdda_solve(bdda_op* op, const bdda_solve_opts* opts, const double* diag, const double* B, int ldb,
               double* X, int ldx, int L, bdda_solve_stats* stats);

/*
 * Thin QR with R real-positive on the diagonal (qr_reduced,
 * bl_krylov_mvp_fft/qr_reduced.cpp:9-31, linear_algebra_addon.hpp:1), complex
 * FP64 host buffers: A (m x n, lda) -> Q (m x n, ldq), R (n x n, column-major).
 * Computed on the device by CholQR2.  n <= 32.
 */
int bdda_qr_reduced(const double* A, int m, int n, int lda, double* Q, int ldq, double* R);

/* ---- batched solves and the request server ------------------------------- */
/*
 * Replace the reference's sequential wavelength x target loop
 * (block_DDA_main.cpp:138-163) with concurrent solves on one GPU.  A request
 * is one target: its box, spacing, wavenumber, dipole addresses, DIAG_A and
 * right-hand sides (host buffers that must stay valid until the request is
 * done; X receives the solution).
 */
typedef struct {
  int n[3];
  double lf;
  double k_re, k_im;
  const int* address;
  int nocc;
  const double* diag;   /* f*nocc complex */
  const double* B;      /* f*nocc x L complex, column-major, ld f*nocc */
  int L;                /* 1..32 */
  double* X;            /* f*nocc x L complex output */
  int f;                /* 3 (electric dipoles; 0 means 3) or 6 (electric + magnetic, CEMD) */
} bdda_request;

typedef struct {
  int status;             /* BDDA_OK or the solve's error code */
  int iterations;
  int refinements;
  double true_res_max;
  double t_submit, t_start, t_done;   /* seconds since the server started (steady clock) */
  double footprint_bytes;             /* device memory reserved for the request */
  int retried_fp64;                   /* 1: the mixed solve broke down or stagnated and was solved again in
                                         FP64, starting from the mixed solve's iterate */
} bdda_request_result;

/* Device-memory footprint the server reserves for one f = 3 request (bytes). */
double bdda_request_footprint(const int n[3], int nocc, int L, int precision);
/* The same for f = 3 or 6 components per dipole. */
double bdda_request_footprint_f(const int n[3], int nocc, int L, int precision, int f);

typedef struct bdda_server bdda_server;

/*
 * Start a server with `slots` concurrent solves and a device-memory budget.
 * Requests are admitted in arrival order when their footprint fits the
 * budget; a later request that fits may overtake a waiting head at most 8
 * times.  opts must ask for a true residual (true_tol > 0).  dry_run != 0
 * runs no device work (each request just holds its slot and memory for a
 * time proportional to its footprint) -- for testing admission and queueing.
 */
int bdda_server_create(bdda_server** s, int slots, double mem_budget_bytes, const bdda_solve_opts* opts, int dry_run);
/* Queue a request; BDDA_ERR_NOMEM if its footprint exceeds the whole budget. */
int bdda_server_submit(bdda_server* s, const bdda_request* r, long long* ticket);
/* Block until the request is done; returns its status and fills res. */
int bdda_server_wait(bdda_server* s, long long ticket, bdda_request_result* res);
/* Peak reserved memory, peak concurrent requests, completed requests. */
int bdda_server_stats(bdda_server* s, double* peak_inflight_bytes, int* peak_running, long long* completed);
/*
 * Spectrum cache: a finished request's operator (Green spectra, plans and
 * workspaces, resident in HBM) is kept idle, and a later request with the same
 * box, f, lattice spacing, wavenumber and precision takes it instead of
 * rebuilding the spectrum.  Idle operators count against the memory budget
 * and against max_bytes (default: a quarter of the budget; 0 disables the
 * cache); the least recently used go first when an admission needs memory.
 * No counterpart in the reference, which rebuilds everything per target and
 * wavelength (block_DDA_main.cpp:138-163).
 */
int bdda_server_set_spectrum_cache(bdda_server* s, double max_bytes);
/* Requests that reused a cached operator, operators built, device bytes held idle. */
int bdda_server_cache_stats(bdda_server* s, long long* spectra_reused, long long* spectra_built, double* cached_bytes);
/* Drain the queue, join the workers, free the server (and its idle operators). */
int bdda_server_destroy(bdda_server* s);
/* Solve `count` requests concurrently (a server submitted all at once). */
int bdda_batch_solve(const bdda_request* reqs, int count, int slots, double mem_budget_bytes,
                     const bdda_solve_opts* opts, bdda_request_result* results);

/* ---- target, fields and cross sections (host) --------------------------- */

/*
 * Polarizability alpha = 3 i a1 / (2 k^3) of a sphere of radius r_p
 * (Target_manager.cpp:215-233), a1 the first Mie coefficient (BH83).  Also
 * returns b1 (for magnetic dipoles).  eps/mu as {re, im}.
 */
int bdda_mie_a1b1(double wl0, double r_p, const double eps_p[2], const double mu_p[2], const double eps_m[2],
                  const double mu_m[2], double a1[2], double b1[2]);

/*
 * Seeded lattice particle-cluster aggregate of exactly nocc sites with
 * radius of gyration Rg(N) = a (N/kf)^(1/Df) (a = 1 lattice spacing).
 * Output: box n[3] and 0-based addresses (address must hold nocc ints).
 */
int bdda_aggregate(int nocc, double kf, double Df, unsigned long long seed, int n[3], int* address);

/*
 * Incident fields for f=3 (Target_manager.cpp:262-279): B[3m+c, l] =
 * e_l[c] exp(i k u_l . r_m), r_m = (ix, iy, iz) lf.  uinc, einc: L x 3
 * (einc complex interleaved).  B has leading dimension ldb.
 */
int bdda_incident_fields(const int n[3], double lf, const int* address, int nocc, double k, int L,
                         const double* uinc, const double* einc, double* B, int ldb);

/*
 * Cext, Cabs, Csca per column (Result_manager.cpp:132-143): out[3*l + {0,1,2}].
 * Host buffers.  alpha0 = polarizability of dipole 0 (the reference uses it
 * for every dipole).
 */
int bdda_cross_sections(double k, const double alpha0[2], const double* E, int lde, const double* P, int ldp,
                        int nrows, int L, double* out);

/*
 * Incident fields for f=6 (Target_manager.cpp:280-291): rows 6m..6m+2 =
 * e_l exp(i k u_l . r_m), rows 6m+3..6m+5 = h_l exp(i k u_l . r_m).  hinc:
 * L x 3 complex interleaved (the H amplitude of each wave).  ldb >= 6*nocc.
 */
int bdda_incident_fields_eh(const int n[3], double lf, const int* address, int nocc, double k, int L,
                            const double* uinc, const double* einc, const double* hinc, double* B, int ldb);

/*
 * Cext, Cabs, Csca per column for f=6 (Result_manager.cpp:90-115):
 * out[3*l + {0,1,2}].  Cext over all 6*nocc rows; Cabs weighs the electric
 * rows (6m..6m+2) with alpha_E of dipole 0 and the magnetic rows with
 * alpha_H of dipole 0, as the reference does for every dipole.
 */
int bdda_cross_sections_eh(double k, const double alpha_e0[2], const double alpha_h0[2], const double* EH, int lde,
                           const double* PM, int ldp, int nocc, int L, double* out);

/* ---- target ingestion ------------------------------------------------------ */

/*
 * Read a target file DDA_target_*.out (Target_manager.cpp:114-202): header
 * lines pp radius, aggregate volume, coating volume, "nx ny nz", lf; then rows
 * "address vol material_index" (index 0 or 1).  lf and vol are multiplied by
 * scale_factor and scale_factor^3 (:157,172).  *nocc receives the row count;
 * address, vol, material (each may be null) receive up to capacity rows.
 * Call with capacity 0 to size the arrays; capacity > 0 and smaller than the
 * row count is an error.  Blank and '#' lines are skipped.
 */
int bdda_read_target_file(const char* path, double scale_factor, int n[3], double* lf, int* nocc, int capacity,
                          int* address, double* vol, int* material);

/* Shapes of Target_manager::is_in_target_volume (Shape_Name.hpp). */
#define BDDA_SHAPE_SPHERE 0
#define BDDA_SHAPE_CUBE 1
#define BDDA_SHAPE_ELLIPSOID 2
#define BDDA_SHAPE_CUBOID 3
#define BDDA_SHAPE_CYLINDER 4
#define BDDA_SHAPE_ROUNDED_CYLINDER 5  /* as the reference: only the lower cap is rounded */

/*
 * Shape target (Target_manager.cpp:84-112): lf = max side / nmax, n_i =
 * ceil(nmax side_i / max side), every site (ix, iy, iz) lf inside the shape is
 * occupied (element volume lf^3).  Sizing as bdda_read_target_file.
 */
int bdda_shape_target(int shape, int nmax, const double side_lengths[3], int n[3], double* lf, int* nocc,
                      int capacity, int* address);

/*
 * Materials (Material.cpp:10-124): a table file (rows "wl0 (re,im) (re,im)"
 * of eper and mper against ascending free-space wavelength, '##' comments)
 * interpolated linearly in wl0, or a constant.  Evaluating outside the table
 * is an error (the reference exits).  bdda_material_eval with eper and mper
 * both null returns only the density (g/cm^3, may be null).
 */
typedef struct bdda_material bdda_material;
int bdda_material_load(const char* path, double density, bdda_material** out);
int bdda_material_constant(const double eper[2], const double mper[2], double density, bdda_material** out);
int bdda_material_eval(const bdda_material* m, double wl0, double eper[2], double mper[2], double* density);
int bdda_material_destroy(bdda_material* m);

/*
 * alpha_E (and alpha_H if not null) of every dipole in vacuum
 * (Target_manager.cpp:215-260): 3 i a1 / (2 k^3), 3 i b1 / (2 k^3), k = 2 pi /
 * wl0, Mie a1, b1 of the volume-equivalent sphere (Target.cpp:13-19) of the
 * dipole's element volume and material mats[material[i]] (material may be
 * null: all 0).  The Mie coefficients are computed once per distinct
 * (volume, material); *mie_evaluations (may be null) receives that count.
 */
int bdda_polarizabilities(double wl0, int nocc, const double* vol, const int* material,
                          const bdda_material* const* mats, int nmat, double* alpha_e, double* alpha_h,
                          int* mie_evaluations);

/* DIAG_A (Solver.cpp:28-56): 1/alpha_E on rows f*m + 0..2, 1/alpha_H on rows 6m + 3..5 (f = 6). */
int bdda_diag_a(int f, int nocc, const double* alpha_e, const double* alpha_h, double* diag);

/*
 * Mie efficiencies {Qsca, Qabs, Qext} of a sphere of radius r_p in a
 * non-absorbing medium (what the reference's gmie returns first,
 * gmie/gmie.cpp:9-152, for its volume-equivalent Mie comparison).
 */
int bdda_mie_q(double wl0, double r_p, const double eps_p[2], const double mu_p[2], const double eps_m[2],
               const double mu_m[2], double q[3]);

/* ---- result files ---------------------------------------------------------- */

typedef struct {
  int wl0_index, target_index;
  double wl0;
  int N_inc;
  double eper_medium[2], mper_medium[2];
  const char* target_fname;
  int is_homogeneous;                  /* 1: one material ("particle"); 0: core + coat */
  double eper_core[2], mper_core[2];   /* the particle's material when homogeneous */
  double volume_core;                  /* um^3 (the particle's when homogeneous) */
  double density_core;                 /* g/cm^3 */
  double eper_coat[2], mper_coat[2];
  double volume_coat;
  int L;
  const double* cext;                  /* L values, um^2 */
  const double* cabs;
  int f, nx, ny, nz, num_element_occupy;
  double solver_time;                  /* seconds */
  int append_mac_mie;                  /* add the volume-equivalent Mie MAC line (block_DDA_main.cpp:169-183) */
} bdda_result_record;

/*
 * One result section in the reference's DDA_result.dat format
 * (Result_manager.cpp:10-133 and :178-245, Basic_Stats.hpp; MAC_mie line of
 * block_DDA_main.cpp:169-183).  *len receives the text length; buf (cap bytes,
 * may be null) receives the text, NUL-terminated.
 */
int bdda_format_result(const bdda_result_record* r, char* buf, int cap, int* len);

/* ---- wavelength x target sweep ------------------------------------------- */

typedef struct {
  int n[3];               /* lattice box */
  double lf;              /* physical lattice spacing (um) */
  int nocc;
  const int* address;     /* occupied sites */
  const double* vol;      /* element volumes (um^3) */
  const int* material;    /* index into bdda_sweep_spec.materials, or null: all 0 */
} bdda_sweep_target;

typedef struct {
  int f;                                   /* 3 or 6 */
  int n_wl;
  const double* wl0;                       /* free-space wavelengths (um), vacuum medium */
  int n_targets;
  const bdda_sweep_target* targets;
  int nmat;
  const bdda_material* const* materials;
  int L;                                   /* incident waves, 1..32 */
  const double* uinc;                      /* L x 3 propagation directions */
  const double* einc;                      /* L x 3 complex E amplitudes */
  const double* hinc;                      /* L x 3 complex H amplitudes (f = 6) */
  bdda_solve_opts opts;                    /* per solve (opts.warm_start is set by the sweep) */
  int warm_start;                          /* refine each wavelength from the previous one's solution */
  int prec;                                /* operator tables (0: FP64 | FP32 | DF64) */
} bdda_sweep_spec;

typedef struct {
  int status;                  /* BDDA_OK or the first error of this (wavelength, target) */
  int iterations;
  int refinements;
  int mie_evaluations;         /* distinct (volume, material) Mie evaluations */
  double true_res_max;
  double final_err;
  double ms_solve;
  double alpha_e0[2], alpha_h0[2];   /* polarizabilities of dipole 0 (the cross sections use them) */
} bdda_sweep_result;

/*
 * The reference's experiment loop (block_DDA_main.cpp:138-163) as one call:
 * for every wavelength and target, material constants, polarizabilities,
 * DIAG_A, incident fields, solve and cross sections.  One operator per target
 * is reused across wavelengths (only its spectrum is rebuilt).
 * cross[((w * n_targets + t) * L + l) * 3 + {0,1,2}] = Cext, Cabs, Csca;
 * res[w * n_targets + t].  Returns BDDA_OK or the first error.
 */
int bdda_sweep(const bdda_sweep_spec* spec, double* cross, bdda_sweep_result* res);

/* ---- instrumentation ------------------------------------------------------ */

/*
 * Algorithmic HBM bytes of one block MVP over the operator's dipoles with L
 * right-hand sides (prec BDDA_PREC_FP64 / BDDA_PREC_FP32), per kernel pass:
 * bytes[0..4] = passes A..E (the minimum reads + writes each pass must do).
 * with_diag / with_jpre add the diagonal and Jacobi reads.  Returns BDDA_OK.
 */
int bdda_op_mvp_bytes(const bdda_op* op, int prec, int L, int with_diag, int with_jpre, double bytes[5]);

/* Per-kernel CUDA-event timing on the operator: 0 off, 1 every kernel class,
 * 2 the fused z pass (pass C) of each precision only (two events per block
 * MVP, for timing a whole solve with little overhead). */
int bdda_op_set_timing(bdda_op* op, int enable);

/* Block Krylov solves on op run every poll cycle after the first (the
 * check_every iterations between two reads of the control block) as one
 * launch of a captured CUDA graph (on = 1, the default) or launch by launch
 * (on = 0; results are bitwise the same).  Graphs pay where one solve's
 * launches leave the GPU idle (small systems); with many solves in flight on
 * other streams they only add their capture, and the request scheduler
 * (bdda_batch_solve, bdda_server_*) turns them off for its operators. */
int bdda_op_set_graphs(bdda_op* op, int on);

/* FFT schedule autotuner (no counterpart in the reference, whose FFTW plans
 * are FFTW_ESTIMATE).  With on = 1 (the default) the first complex FP32 block
 * MVP of an nrhs whose FFT workspace is at least 64 MiB times, with CUDA
 * events on the operator's own buffers, the candidates of each tile pass's
 * launch schedule -- y passes double- or single-buffered with a grid of 2, 4,
 * 8 or 16 waves of the resident CTAs, the scalar, packed-pair or pipelined z
 * pass where they run the geometry, x passes aiming at 5, 10 or 20 CTAs per
 * SM -- and keeps the fastest (also for later operators of the same box,
 * occupancy and nrhs in this process).  Not inside stream capture.  The
 * schedules only reorder work: results equal the default schedule's bitwise
 * (the pipelined and scalar z passes too), except that the packed z pass
 * rounds differently (FP32 MVP tolerance).  on = 0 restores the defaults and
 * forgets the choices. */
int bdda_op_set_autotune(bdda_op* op, int on);
/* The schedule in use for nrhs L: schedule = {y waves, y buffers, z pass (-1
 * default rule, 0 scalar, 1 packed, 2 pipelined), x CTAs per SM, inverse y
 * (pass D) waves, inverse y buffers}; candidate_ms (may be null): measured ms
 * of pass B with 1 then 2 buffers x waves 2, 4, 8, 16 ([0..7]), pass C
 * scalar / packed ([8..9]), pass A at 5, 10, 20 CTAs per SM ([10..12]), pass
 * C pipelined ([13]), pass D as pass B ([14..21]), -1 where not measured.
 * BDDA_ERR_NOT_CONVERGED when L was not tuned (defaults returned). */
int bdda_op_get_tuning(bdda_op* op, int L, int schedule[6], float candidate_ms[22]);
/* Forces the complex FP32 pass C kernel for every nrhs: -1 the autotuned /
 * default choice, 0 scalar, 1 packed-pair, 2 pipelined.  Where the forced
 * kernel cannot run the operator's z plan (packed: radices above 16 or a fused
 * last radix above 5, or more shared memory than two CTAs per SM; pipelined:
 * f = 6 or more shared memory than a CTA may take) the scalar kernel runs.
 * The kernels compute the same transform; the packed one rounds its pair
 * arithmetic differently (FP32 MVP tolerance). */
int bdda_op_set_z_kernel(bdda_op* op, int kind);
/* Reads and clears the operator's kernel status word.  The pipelined z pass
 * (complex FP32) waits on its bulk copies for at most 2 s; a wait that gives
 * up (never expected) sets the word and the MVP's results are invalid.
 * bdda_solve / bdda_solve_device read it at their end; after
 * bdda_op_mvp_device, synchronise its stream and call this.  BDDA_OK, or
 * BDDA_ERR_CUDA with a message. */
int bdda_op_check_status(bdda_op* op);
/* Test hook of that path: while on, warp 0 of the first CTA of every
 * pipelined z pass first waits on a barrier that nothing arrives on, gives up
 * after the 2 s limit and sets the status word; the launch's results are then
 * invalid, the context stays usable. */
int bdda_op_test_z_stall(bdda_op* op, int on);

/*
 * Per-kernel totals since the last reset: ms[i], launches[i] for
 * i = 0..n-1 in the order passA..passE of the complex FP32 MVP, passA..passE
 * of the complex FP64 MVP, gram (Gram / dot / norm reductions), update (row
 * transforms), small (one-CTA L x L steps), other (conversions, residuals).  Returns the number of entries written (<= n).  reset=1 zeroes
 * the counters after reading.
 */
int bdda_op_kernel_stats(bdda_op* op, double* ms, long long* launches, int n, int reset);

/* Message of the calling thread's last error (empty string if none). */
const char* bdda_last_error(void);

/*
 * Test hook: run the device FFT core (the same source the kernels inline) on
 * the CPU for one line of length N (5-smooth, <= 512).  inverse = 0: natural
 * order in, digit-reversed spectrum out; inverse = 1: digit-reversed in,
 * natural out, unnormalised.  prec 1 = FP64, 2 = FP32, 3 = double-float
 * arithmetic.  nvalid in
 * (0, N) makes the forward transform read only the first nvalid inputs (the
 * rest count as zero); 0 reads all.  data holds N interleaved complex doubles,
 * overwritten.  The schedule is the one the operator gives an axis of that
 * length for the element width of prec: radix[0] on input > 8 selects the z
 * axis (fused three-line pass), otherwise the x / y axes (tile passes);
 * radix[1] = 1 on input selects the complex FP32 schedule whatever prec (the
 * one its Green spectrum is transformed with in FP64).  Radices are written
 * to radix[0..16) on return.  Returns the number of radix stages or -1 for
 * an unsupported N.
 */
int bdda_host_fft_line(int N, int inverse, int prec, int nvalid, double* data, int* radix);

#ifdef __cplusplus
}
#endif

#endif /* BDDA_H */
