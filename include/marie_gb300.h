/*
 * marie_gb300.h -- C ABI of the GB300 FFT-VIE operator and GMRES solver.
 *
 * Drop-in boundary for MARIE's pure-VIE hot path.  In the reference the path
 * is reached through the MATLAB function-handle table built by
 * src/src_utils/src_loaders/parse_inputs.m:6-37 (func.mvp_N, func.mvp_K,
 * func.mvp_herm_adj_N/K, func.mvp_G, func.mvp_invG) and through
 *   [x,iter,resvec] = is_gmres_vie(A,b,restart,tol,maxit,x0)
 * (src/src_solver/src_iterative_solvers/is_gmres_vie.m:1).  A MEX gateway or
 * any FFI binds the functions below; no C++ or torch type crosses the ABI.
 *
 * Conventions
 *  - Complex numbers are interleaved (re, im) pairs: double for MARIE_C128,
 *    float for MARIE_C64 (MATLAB R2018a mxComplexDouble / mxComplexSingle).
 *  - Grids are column-major (n1, n2, n3, C) per right-hand side; body vectors
 *    have length N_b = C * N_s in component-major blocks, exactly the order
 *    of idx_solution (src/src_geometry/body_geometry/geo_body_domain.m:22-34).
 *  - Several right-hand sides are contiguous: rhs r starts at r * len.
 *  - All vector pointers passed to apply/solve calls are DEVICE pointers
 *    unless a comment says otherwise; descriptor arrays are HOST pointers.
 *  - Work is enqueued on the caller's stream (cudaStream_t passed as void*;
 *    NULL = legacy default stream).  A handle is not thread-safe; distinct
 *    handles are independent.  No call throws; every call returns a status.
 */
#ifndef MARIE_GB300_H
#define MARIE_GB300_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  MARIE_OK = 0,
  MARIE_ERR_BAD_ARG = 1,        /* invalid argument (message via marie_last_error) */
  MARIE_ERR_OOM = 2,            /* device allocation failed or cap exceeded */
  MARIE_ERR_NONFINITE = 3,      /* NaN/Inf in an input or an iterate */
  MARIE_ERR_NOT_CONVERGED = 4,  /* maxit reached; report holds the residual */
  MARIE_ERR_DEVICE_TIMEOUT = 5, /* a bounded device wait expired */
  MARIE_ERR_CUDA = 6,           /* CUDA runtime error (code via marie_last_error) */
  MARIE_ERR_NOT_SUPPORTED = 7   /* valid but unsupported configuration */
} marie_status;

typedef enum { MARIE_C128 = 0, MARIE_C64 = 1 } marie_precision;
typedef enum { MARIE_PWC = 0, MARIE_PWL = 1 } marie_basis;

typedef struct marie_vie marie_vie; /* opaque handle */

/* One Tucker block as produced by assembly_fft_circ_tucker_{pwc,pwl}.m:
 * G is r1 x r2 x r3 (column-major); U1 is r1 x 2*n1, U2 r2 x 2*n2, U3 r3 x 2*n3
 * (already circulant-extended, FFT'd and transposed). Host pointers. */
typedef struct {
  int32_t r1, r2, r3;
  const double* G;   /* interleaved complex, r1*r2*r3 */
  const double* U1;  /* interleaved complex, r1*2*n1 */
  const double* U2;
  const double* U3;
} marie_tucker_block;

typedef struct {
  int32_t n1, n2, n3;        /* grid edges */
  int32_t basis;             /* MARIE_PWC (C=3) or MARIE_PWL (C=12) */
  double res;                /* voxel edge [m] */
  double freq;               /* frequency [Hz] (ce = i*2*pi*freq*eps0) */
  int64_t n_b;               /* length of idx_solution (= C * N_s) */
  const int64_t* idx_solution; /* host, 0-based, component-major blocks */
  const double* Mr;          /* host, n1*n2*n3 interleaved complex (em_assembly.m:14) */
  /* N operator: either Tucker blocks (count 6 PWC / 60 PWL, index j*6+k for
   * T(j+1,k+1)) or a dense I_V (n1,n2,n3,pwx,6) column-major; one must be set. */
  const marie_tucker_block* tucker_N;
  const double* dense_N;
  /* K operator (optional): Tucker (3 PWC / 30 PWL, index j*3+k) or dense (n1,n2,n3,pwx,3). */
  const marie_tucker_block* tucker_K;
  const double* dense_K;
  int32_t precisions;        /* bit mask: 1 = build the native C128 path, 2 = the C64 path, 4 = C128 in
                                float-float arithmetic (edges 16*NB; exclusive with 1), 8 = keep the
                                Tucker factors of tucker_N and re-expand the C64 spectrum at the start of
                                every C64 application of N / N^H, as mvp_N_pwl_tucker.m:31 re-expands
                                its blocks in every product (needs bit 2, tucker_N, edges 16*NB) */
  int32_t max_rhs;           /* largest nrhs per apply/solve call (workspace sizing) */
  int64_t mem_cap_bytes;     /* 0 = no cap; otherwise create/solve fail with OOM above it */
} marie_vie_desc;

/* Build an operator handle: uploads the body map, contrast and Green's-tensor
 * spectra and sizes the workspaces.  Replaces the operator set-up of
 * ie_solver_vie.m:14 (fN = to_GPU(MREDM.operators.N,1)) together with the
 * per-product Tucker re-expansion of mvp_N_pwl_tucker.m:31 (done once here).
 * Any grid edge up to 1024 is accepted, as MATLAB's fftn accepts any length:
 * a grid with an edge whose prime factors exceed 31 (e.g. 73) is embedded in
 * a larger grid the FFT passes cover (all edges rounded up to multiples of 16
 * when every edge is <= 128, else that edge to the next 31-smooth length),
 * with the operator zero-padded, which leaves mvp_vie, the solves and the
 * field maps on the caller's body unchanged; the full-grid operators below
 * then return MARIE_ERR_NOT_SUPPORTED.  Environment MARIE_EMBED=1 embeds
 * smooth grids with edges <= 128 the same way (four-step passes). */
marie_status marie_vie_create(marie_vie** h, const marie_vie_desc* d);
marie_status marie_vie_destroy(marie_vie* h);

/* y = mvp_vie(x): src/src_solver/src_mvp/mvp_vie/mvp_vie.m:1-19
 * (x, y: nrhs x N_b, precision prec). */
marie_status marie_vie_apply(marie_vie* h, int32_t prec, const void* x, void* y, int32_t nrhs, void* stream);
/* y = A^H x for A = mvp_vie: y = x - N^H(invG .* conj(Mc./Mr) .* x), with N^H
 * from mvp_N_herm_adj_{pwc,pwl}_tucker.m. */
marie_status marie_vie_apply_adjoint(marie_vie* h, int32_t prec, const void* x, void* y, int32_t nrhs, void* stream);
/* Raw operators on full grids (nrhs x n1*n2*n3*C; not on embedded grids):
 * mvp_N_{pwc,pwl}_tucker.m:1-33/43, mvp_N_herm_adj_{pwc,pwl}_tucker.m,
 * mvp_K_{pwc,pwl}_tucker.m:1-36/45, mvp_K_herm_adj_{pwc,pwl}_tucker.m. */
marie_status marie_vie_apply_N(marie_vie* h, int32_t prec, const void* x, void* y, int32_t nrhs, void* stream);
marie_status marie_vie_apply_N_adj(marie_vie* h, int32_t prec, const void* x, void* y, int32_t nrhs, void* stream);
marie_status marie_vie_apply_K(marie_vie* h, int32_t prec, const void* x, void* y, int32_t nrhs, void* stream);
marie_status marie_vie_apply_K_adj(marie_vie* h, int32_t prec, const void* x, void* y, int32_t nrhs, void* stream);

/* Allocation-free y = mvp_N(x) for ONE complex64 right-hand side, without a
 * handle.  No counterpart in the reference: it is for callers that must not
 * allocate device memory (an allocator-free region of a host framework, a
 * real-time loop, a process that reserved all device memory up front) and so
 * cannot call marie_vie_create.  The caller passes device pointers: the N
 * octant spectrum green_octant (complex64, layout [blk][n2+1][n1+1][n3+1],
 * blk = j*6+k for block T(j+1,k+1), scaled by 1/(8 n1 n2 n3)), x and y (grids,
 * n1*n2*n3*C, column-major).  The FFT work arrays live in a fixed 64 MiB
 * file-scope device array, so 6*n1*n2*n3*C*8 bytes must not exceed 64 MiB
 * (larger grids return MARIE_ERR_BAD_ARG).  That array is held by every GPU
 * that loads the library until exit and is shared by all calls: calls that
 * overlap on the GPU race.  The first call on a device looks up the array's
 * device address; make it before any stream capture.  Never calls cudaMalloc
 * or cudaFree. */
marie_status marie_vie_apply_N_noalloc(int32_t n1, int32_t n2, int32_t n3, int32_t basis,
                                       const void* green_octant, const void* x, void* y, void* stream);

typedef enum {
  MARIE_SOLVE_FP64 = 0,   /* complex128 GMRES, faithful to is_gmres_vie.m */
  MARIE_SOLVE_MIXED = 1,  /* complex64 GMRES inside an FP64 iterative-refinement loop */
  MARIE_SOLVE_MIXED_BLOCK = 2  /* MIXED with one block Krylov space shared by the right-hand
                                  sides of each refinement step (block GMRES, block_steps
                                  block Arnoldi steps per cycle, maxit cycles) */
} marie_solve_mode;

typedef struct {
  int32_t restart;        /* is_gmres_vie restart (reference: 50), 1..128 */
  int32_t maxit;          /* max restart cycles (reference: 200) */
  double tol;             /* relative residual target */
  int32_t mode;           /* marie_solve_mode */
  int32_t x0_present;     /* 1: x holds the initial guess; 0: start from zero */
  double inner_tol;       /* MIXED: floor of the inner c64 GMRES relative tolerance (0 = 1e-7) */
  int32_t max_refine;     /* MIXED: max refinement steps (0 = 10) */
  double inner_safety;    /* MIXED: each inner solve asks for
                             clamp(inner_safety*tol/current residual, inner_tol, 0.5) (0 = 0.9);
                             the FP64 true residual decides convergence either way */
  int32_t adjoint;        /* 1: solve A^H x = b (A^H as marie_vie_apply_adjoint), for adjoint
                             sensitivities; 0: A x = b */
  int32_t block_steps;    /* MIXED_BLOCK: block Arnoldi steps per cycle (0 = 30); the block
                             basis holds (block_steps+1) x nrhs complex64 vectors */
} marie_gmres_opts;

typedef struct {
  int32_t* iters;         /* host, per rhs: total inner iterations (may be NULL) */
  int32_t* outer;         /* host, per rhs: restart cycles (iter(2) of is_gmres_vie) */
  int32_t* last_inner;    /* host, per rhs: iterations in the last cycle (iter(1)) */
  double* true_resid;     /* host, per rhs: ||b - A x|| / ||b|| recomputed in FP64 */
  double* resvec;         /* host, per rhs x resvec_cap: relative residual history (may be NULL) */
  int32_t resvec_cap;
  int32_t* resvec_len;    /* host, per rhs */
  int32_t* status;        /* host, per rhs: marie_status */
  int32_t matvecs_c128;   /* out: FP64 operator applications per rhs batch */
  int32_t matvecs_c64;    /* out: complex64 operator applications */
} marie_gmres_report;

/* [x,iter,resvec] = is_gmres_vie(A,b,restart,tol,maxit,x0) with A = mvp_vie,
 * for nrhs independent right-hand sides in one batched launch sequence
 * (src/src_solver/src_iterative_solvers/is_gmres_vie.m:1-30,
 *  is_iter_gmres_vie.m:1-38; the serial port loop of ie_solver_vie.m:16-21).
 * b and x are device complex128 (nrhs x N_b). */
marie_status marie_gmres_vie(marie_vie* h, const void* b, void* x, int32_t nrhs,
                             const marie_gmres_opts* opts, marie_gmres_report* report, void* stream);

/* marie_gmres_vie with b and x in host memory (nrhs x N_b complex128; x
 * holds x0 on entry when opts->x0_present).  The right-hand sides are solved
 * in chunks of at most the matvec chunk size; copies of the next chunk in and
 * the previous chunk out run on a second stream while a chunk is solved, so
 * with page-locked host buffers only the first copy in and the last copy out
 * are exposed, and the first and last chunks are a quarter chunk.  The MATLAB
 * host-array path of is_gmres_vie (to_GPU.m:8-51). */
marie_status marie_gmres_vie_host(marie_vie* h, const void* b_host, void* x_host, int32_t nrhs,
                                  const marie_gmres_opts* opts, marie_gmres_report* report, void* stream);

/* Replaces the body's materials: Mr_body (host, N_s complex128, body voxels
 * in idx_solution order) = eps_r + sigma/ce per voxel (em_assembly.m:14).
 * Recomputes the contrast (1./Mr).*Mc of every built precision and the
 * absorbed-power weights; the Green's tensor, body map and workspaces stay.
 * Waits for the device to be idle first.  No counterpart in the reference
 * (which rebuilds EP); used by material sweeps and finite-difference checks
 * of the adjoint gradient. */
marie_status marie_vie_set_materials(marie_vie* h, const double* Mr_body);

/* H (M x p complex64, column-major, leading dimension ldh) = V^H W for
 * complex64 device arrays V (K x M, column a at V + a*ldv) and W (K x p,
 * p <= 64), on the tensor cores (tcgen05, TF32 with three split products);
 * the block GMRES solver's projection and Gram-matrix kernel.  ldv and ldw
 * even, V and W 16-byte aligned; part: device scratch of
 * marie_block_gemm_part_floats(K, M) floats; err: device int, set to 1 if a
 * bounded device wait expired.  Enqueued on stream.  No counterpart in the
 * reference (MATLAB's V'*W). */
marie_status marie_block_gemm_cn(const void* V, int64_t ldv, const void* W, int64_t ldw, int64_t K, int32_t M,
                                 int32_t p, void* H, int64_t ldh, void* part, int64_t part_floats, void* err,
                                 void* stream);
int64_t marie_block_gemm_part_floats(int64_t K, int32_t M);

/* Frees the GMRES workspace the handle keeps between solves (Krylov basis,
 * residual vectors; reused by the next solve of the same or smaller shape).
 * No counterpart in the reference (MATLAB frees its arrays itself). */
marie_status marie_vie_release_workspace(marie_vie* h);

/* Operator-generation helpers (producers of the hot path's operands). */
/* I_V of assembly_N.m / assembly_K.m (far and medium zones by 6D Gauss rules,
 * near zone {0,1}^3 by the staggered stand-in rule); out: host, dense
 * (n1,n2,n3,pwx,6|3) interleaved complex.  kernel: 0 = N, 1 = K. */
marie_status marie_assemble_green(int32_t n1, int32_t n2, int32_t n3, double res, double freq,
                                  int32_t basis, int32_t kernel, double* out_host);

/* marie_assemble_green with options.  flags: MARIE_GREEN_SELF_POINT_TERM adds
 * to the self offset I_V(0,0,0) of N the point term of its kernel, (2/3)
 * Gram_ll' on the xx, yy, zz components (Gram = diag(res^3, res^3/12 x 3)):
 * the six N components are those of curl curl (g I), whose distributional
 * part (2/3) delta_pq delta(r) the surface-surface near zone of assembly_N.m
 * (:56-81) contains and the stand-in cubature does not.  Without it the
 * field inside a quasi-static dielectric sphere comes out ~3x too small. */
#define MARIE_GREEN_SELF_POINT_TERM 1
/* MARIE_GREEN_NEAR_EXACT replaces the near offsets {0,1}^3 (N or K) with an
 * accurate host cubature of the same integrals (relative coordinate
 * u = r - r', the box split so that u = 0 is a corner of its pieces, Duffy
 * pyramids there, the static N singularity as a principal value over the
 * cube plus the point term above; converged to ~1e-14), instead of the
 * staggered 8^3 x 7^3 stand-in, which is off by 13% on face neighbours. */
#define MARIE_GREEN_NEAR_EXACT 2
marie_status marie_assemble_green_ex(int32_t n1, int32_t n2, int32_t n3, double res, double freq,
                                     int32_t basis, int32_t kernel, int32_t flags, double* out_host);
/* Incident field of closed loops with unit current, tested onto the PWC/PWL
 * basis (coef_l = int E.f_l / int f_l^2): the loop/wire RHS generator.
 * loops: host, nloop x 6 doubles (centre xyz, normal xyz); out: device
 * complex128, nloop x N_b.  voxel centres: centre of voxel (0,0,0) = origin. */
marie_status marie_incident_loops(marie_vie* h, const double* origin, const double* loops, int32_t nloop,
                                  double radius, int32_t nseg, void* out_dev, void* stream);
/* Incident field of wire currents in the reference's wire-basis convention,
 * as coefficients on the body: invG(Zbw * coef) restricted to the body, with
 * Zbw the voxel-wire coupling of Assemble_tri_coupling_matrix_N_* (kind 0,
 * electric field) or _K_* (kind 1, magnetic field) times res^3
 * (src_wvie/Cpp_Assembly/src/Assemble_tri_coupling_matrix_N_x.cpp:21-205,
 * wvie_mrgf_assembly.m:26-49; the tested fields of em_efield_wvie.m:43-47 and
 * em_hfield_wvie.m:38).  Wire basis t spans r_p -> r_2 -> r_n (host, n_tri x 3
 * doubles each); both halves carry a current ramping up from the half's start
 * point, as the reference places its source points.  coef: host, nrhs x n_tri
 * complex128 wire currents, or NULL for all ones (a closed loop of unit
 * coefficients).  q_wire / q_vox: Gauss points per half / per voxel axis
 * (the reference's Quad_order_wie_coup = 4, Quad_order_vie = 2).  out: device
 * complex128, nrhs x N_b. */
marie_status marie_incident_wire(marie_vie* h, int32_t kind, const double* origin, const double* r_p,
                                 const double* r_n, const double* r_2, int32_t n_tri, const double* coef,
                                 int32_t nrhs, int32_t q_wire, int32_t q_vox, void* out_dev, void* stream);
/* Unit x-polarised plane wave exp(-i k0 z) tested onto the basis. */
marie_status marie_incident_plane_wave(marie_vie* h, const double* origin, void* out_dev, void* stream);

/* Field post-processing of solved body currents J (device, nrhs x N_b, the
 * handle's body-vector layout) in precision prec.
 * E = Ue + mask.*invG((1/ce)(N J - G J))  (em_efield_vie_excitation.m:21)
 * H = Ub + mask.*invG(K J)                (em_hfield_vie_excitation.m:20)
 * restricted to the body; Ue / Ub (incident fields, same layout) may be NULL
 * (zero); E or H may be NULL (not computed).  H needs the K operator. */
marie_status marie_vie_fields(marie_vie* h, int32_t prec, const void* J, const void* Ue, const void* Ub, void* E,
                              void* H, int32_t nrhs, void* stream);
/* Absorbed-power / noise-covariance matrix of em_ehfield_vie.m:44-52:
 * phi = conj(J^H (real(Mpow) .* (G J))), Mpow = Mc_inv/ce per body voxel
 * (0 where Mc = 0).  J: device complex128, nrhs x N_b (nrhs <= 64);
 * phi_host: host, nrhs x nrhs complex128 (row p, column q), FP64 sums in a
 * fixed order. */
marie_status marie_vie_absorbed_power(marie_vie* h, const void* J, int32_t nrhs, double* phi_host, void* stream);
/* Adjoint of the H-field map of marie_vie_fields: y = K^H(invG x) on the
 * body (x, y: body vectors, nrhs x N_b).  Needs the K operator.  Used for
 * the adjoint source of B1+ objectives. */
marie_status marie_vie_apply_hfield_adjoint(marie_vie* h, int32_t prec, const void* x, void* y, int32_t nrhs,
                                            void* stream);
/* Adjoint sensitivities of J_obj = M/P with M = mean_ROI |B1+|^2 and P the
 * absorbed power (1/2) phi(1,1) of one solved current J (device complex128
 * body vectors, one right-hand side):
 *   marie_vie_gradient_source: g = gM/P - (M/P^2)(1/2) D J, gM = dM/dconj(J),
 *     D = G real(Mc_inv/ce) (the adjoint equation A^H lam = g follows, GMRES
 *     with opts.adjoint = 1);
 *   marie_vie_gradient: dJ_obj/d eps_r and dJ_obj/d sigma per body voxel
 *     (device double, N_s each) from J, lam and the total field E of
 *     marie_vie_fields.
 * No counterpart in the reference: the derivation is in csrc/fields.cu. */
marie_status marie_vie_gradient_source(marie_vie* h, const void* J, const void* gM, double M, double P, void* g,
                                       void* stream);
marie_status marie_vie_gradient(marie_vie* h, const void* J, const void* lam, const void* E, double M, double P,
                                double* d_eps, double* d_sigma, void* stream);
/* B1+ = mu0 (H_x + i H_y) on the constant moment of each body voxel
 * (em_ehfield_vie.m:68).  H: device complex128, nrhs x N_b; out: device
 * complex128, nrhs x N_s. */
marie_status marie_vie_b1_plus(marie_vie* h, const void* H, int32_t nrhs, void* out, void* stream);

/* Coupled coil/body matvec of the pFFT formulation: Vout =
 * mvp_svie_pfft(Jcb, pfft_PS, pfft_Z_cc, pfft_Z_bc_N, ext_Mc_inv, func, fN,
 * Multiplier_1, Multiplier_2, emc, N_sie, res, pfft_dims)
 * (src/src_solver/src_mvp/mvp_svie/mvp_svie_pfft.m:1-19; its caller
 * ie_solver_svie_pfft.m:25-27).  Unknowns [Jc; Jb]: n_sie coil currents
 * then n_b body currents.  grid_op is a marie_vie handle on the extended
 * (pFFT) grid pfft_n1 x pfft_n2 x pfft_n3 holding its N operator (the
 * reference's MREDM.operators.pfft_N); it must outlive this handle and not
 * be an embedded grid.  Sparse matrices are host CSR with 0-based indices
 * and interleaved complex128 values, copied at create:
 *   PS     (pfft_n1*pfft_n2*pfft_n3*ql) x (n_sie + n_b)  (pfft_PS)
 *   Z_cc   n_sie x n_sie                                 (pfft_Z_cc)
 *   Z_bc_N n_b x n_sie                                   (pfft_Z_bc_N)
 * ext_Mc_inv: host, pfft_n1*pfft_n2*pfft_n3 complex128 (EP.ext_Mc_inv,
 * em_assembly.m:35-37).  M1 / M2: host, n_sie + n_b doubles, or NULL for
 * ie_solver_svie_pfft.m's [ones(N_sie); -ones(N_b)] and [zeros(N_sie);
 * ones(N_b)]. */
typedef struct {
  int64_t rows, cols, nnz;
  const int64_t* row_ptr;   /* rows + 1 */
  const int64_t* col_idx;   /* nnz */
  const double* val;        /* 2 * nnz (re, im) */
} marie_csr;

typedef struct marie_svie_pfft marie_svie_pfft; /* opaque handle */

typedef struct {
  marie_vie* grid_op;
  int64_t n_sie;
  int64_t n_b;
  marie_csr PS;
  marie_csr Z_cc;
  marie_csr Z_bc_N;
  const double* ext_Mc_inv;
  const double* M1;
  const double* M2;
} marie_svie_pfft_desc;

marie_status marie_svie_pfft_create(marie_svie_pfft** h, const marie_svie_pfft_desc* d);
/* y = mvp_svie_pfft(x) for nrhs right-hand sides (device, nrhs x (n_sie +
 * n_b), precision prec; complex64 needs the grid handle's complex64 state,
 * complex128 its complex128 or float-float state), on `stream`. */
marie_status marie_svie_pfft_apply(marie_svie_pfft* h, int32_t prec, const void* x, void* y, int32_t nrhs,
                                   void* stream);
marie_status marie_svie_pfft_destroy(marie_svie_pfft* h);

/* Diagnostics. */
/* Average device time [ms] of each matvec pass over `reps` repetitions of
 * one mvp_vie application of nrhs right-hand sides (x/y: device, precision
 * prec), timed with CUDA events on `stream`:
 * ms[0] x-forward, ms[1] y-forward, ms[2] z (FFT, Green multiply, iFFT),
 * ms[3] y-inverse, ms[4] x-inverse + epilogue.  ms[5] = whole application. */
marie_status marie_vie_profile(marie_vie* h, int32_t prec, const void* x, void* y, int32_t nrhs, int32_t reps,
                               double* ms, void* stream);
/* Shape of a handle: out[0..2] = the caller's grid edges n1, n2, n3,
 * out[3] = ql (3 PWC, 12 PWL), out[4] = N_s body voxels, out[5] = N_b body
 * unknowns (dims.N_b of geo_assembly.m). */
marie_status marie_vie_info(marie_vie* h, int64_t* out);
/* Autotuner of the FFT tiles: times `reps` applications of mvp_vie in
 * precision prec on x (device, nrhs x N_b; y receives the results) for every
 * z-pass tile width (a power of two <= 16: pencils x interleaved right-hand
 * sides) whose shared memory fits one CTA and whose bundles fit the handle's
 * work arrays, and keeps the fastest for later calls.  widths / ms (host,
 * cap entries) receive the widths tried and their mean times; *count the
 * number tried.  No counterpart in the reference (MATLAB's fftn plans its
 * own transforms). */
marie_status marie_vie_autotune(marie_vie* h, int32_t prec, const void* x, void* y, int32_t nrhs, int32_t reps,
                                int32_t* widths, double* ms, int32_t cap, int32_t* count, void* stream);
/* Workspace right-hand sides per matvec chunk and the z-pass tile width:
 * out[0] = chunk, out[1] = tile width (pencils x interleaved right-hand
 * sides), out[2..3] reserved (0). */
marie_status marie_vie_tiles(marie_vie* h, int32_t prec, int32_t* out);
const char* marie_last_error(void);
const char* marie_version(void);
/* Number of kernel launches issued by this library since load. */
int64_t marie_launch_count(void);

#ifdef __cplusplus
}
#endif

#endif /* MARIE_GB300_H */
