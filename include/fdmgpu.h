/*
 * fdmgpu.h - C-ABI of the GB300 FDM assembly + solve (drop-in for FDMNES mat_solve).
 *
 * The reference solves, for one photon energy, the finite-difference system
 * assembled row by row by calcMatRow (source/mat.f90:1034-1727) with either the
 * Gaussian profile solver (source/mat_solve_gaussian.f90:5-372) or MUMPS
 * (source/mat_solve_mumps.f90:5-261).  Both backends share the 86-argument
 * Fortran interface `mat_solve` (source/mat_solve_gaussian.f90:5-12,
 * source/mat_solve_mumps.f90:5-12) called from `mat` (source/mat.f90:186-194).
 *
 * This header restates that argument list as two plain structs:
 *   fdmgpu_grid    - energy-independent arguments (grid, stencil, boundary
 *                    tables, harmonics, representation tables); uploaded once
 *                    per handle;
 *   fdmgpu_energy  - arguments that change from one call to the next (row
 *                    numbering from newind, potential, atomic boundary
 *                    functions, outer Bessel/Neumann, energy, flags).
 * Every array keeps the reference's Fortran layout: column-major, and index
 * VALUES are 1-based exactly as the Fortran caller holds them.  No pointer is
 * retained after a call returns.
 *
 * All entry points return an fdmgpu_status code; none of them aborts the
 * process (the reference `stop`s on a zero pivot, source/mat_solve_gaussian.f90:265-302).
 * Handles are not thread-safe: use one handle per host thread.
 */
#ifndef FDMGPU_H
#define FDMGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
typedef enum {
  FDMGPU_OK = 0,
  FDMGPU_ERR_ARG = 1,          /* invalid argument / inconsistent sizes          */
  FDMGPU_ERR_UNSUPPORTED = 2,  /* flag combination the library does not provide   */
  FDMGPU_ERR_CUDA = 3,         /* CUDA runtime error (message via fdmgpu_last_error) */
  FDMGPU_ERR_ZERO_PIVOT = 4,   /* |pivot| below threshold: the reference stops here */
  FDMGPU_ERR_NOT_CONVERGED = 5,/* mixed precision refinement did not converge      */
  FDMGPU_ERR_NOMEM = 6         /* device allocation failed                         */
} fdmgpu_status;

/* Arithmetic of the factorisation. */
typedef enum {
  FDMGPU_PREC_FP64 = 0,        /* plain FP64 profile LU: the correctness path          */
  FDMGPU_PREC_MIXED = 1        /* FP32 profile LU + FP64 residual and refinement       */
} fdmgpu_precision;

/* Arithmetic of the refinement residual b - A x in the mixed precision path. */
typedef enum {
  FDMGPU_RESIDUAL_FP64 = 0,    /* native FP64                                          */
  FDMGPU_RESIDUAL_DF64 = 1     /* double-float (hi + lo float pairs, ~48 bits) on the
                                  FP32 pipes: the default, GB300 FP64 is ~60x slower    */
} fdmgpu_residual_mode;

/* Refinement of the mixed precision path. */
typedef enum {
  FDMGPU_REFINE_CLASSIC = 0,   /* x += LU32^-1 r, r in double-float every step (default) */
  FDMGPU_REFINE_GMRES = 1,     /* GMRES-IR: GMRES(m) on LU32^-1 A per correction        */
  FDMGPU_REFINE_RECURRENCE = 2 /* classical, with r updated by r -= A dx in FP32 between
                                  double-float residuals that start and confirm it      */
} fdmgpu_refinement;

/* Re-solve of an energy whose mixed precision refinement missed its tolerance. */
typedef enum {
  FDMGPU_ESCALATE_FP64 = 0,    /* FP64 profile LU (no pivoting, as the reference)       */
  FDMGPU_ESCALATE_DF64 = 1,    /* double-float LU of the equilibrated matrix with
                                  tile-local pivoting + double-float refinement steps,
                                  after the FP32 refinement of every energy has ended   */
  FDMGPU_ESCALATE_DF64_OVERLAP = 2, /* the same, started on a second stream as soon as an
                                  energy stalls, while the others keep refining         */
  FDMGPU_ESCALATE_WIDE_DF64 = 3, /* first the FP32 factor again with double-float sums in
                                  every trailing update and FP32 refinement, then
                                  double-float for the energies still stalled            */
  FDMGPU_ESCALATE_DF64_F32 = 4 /* (default) double-float LU and solve, the factors then
                                  rounded to FP32 in place of the stalled FP32 factors
                                  and FP32 refinement steps confirm the double-float
                                  solution: the rounded factors of an accurate LU
                                  contract the error by about 1e-3 per step where the
                                  FP32-computed ones stall, so no double-float
                                  refinement step is needed; double-float steps only
                                  for energies still above the accepted level, and
                                  in a real batch the FP64 assembly and elimination
                                  for those the double-float steps leave above it
                                  (a complex batch reports them not converged)          */
} fdmgpu_escalation;

/* Energy-independent arguments of mat_solve (source/mat_solve_gaussian.f90:17-67). */
typedef struct fdmgpu_grid {
  int32_t npoint;     /* grid points inside the FDM sphere                                   */
  int32_t npsom;      /* grid points including the outer shell (leading dim of ivois/numia)  */
  int32_t nvois;      /* neighbours per point (12 for iord = 4, cubic)                       */
  int32_t natome;     /* atoms of the calculation cluster                                    */
  int32_t nbm;        /* leading dim of poidsa                                               */
  int32_t nbtm;       /* leading dim of ibord, isbord, Ylmato                                */
  int32_t nim;        /* size of rvol                                                        */
  int32_t nsm;        /* size of poidso                                                      */
  int32_t nsort;      /* outer-boundary points (rows of Ylmso, Bessel)                       */
  int32_t nsortf;     /* the first nsortf of them are inside the sphere                      */
  int32_t nstm;       /* size of isrt                                                        */
  int32_t nspin;      /* second dim of Vr                                                    */
  int32_t nlmmax;     /* second dim of Ylmato                                                */
  int32_t nlmomax;    /* second dim of Ylmso                                                 */
  int32_t nlmsam;     /* leading dim of lato/mato/iato                                       */
  int32_t nso1;       /* leading dim of lso/mso/iso                                          */
  int32_t ngrph;      /* number of representations (1 for C1)                                */
  int32_t nspino;     /* 1, or 2 with spin-orbit                                             */
  const int32_t* ivois;   /* (npsom, nvois) neighbour point, 1-based                        */
  const int32_t* isvois;  /* (npsom, nvois) symmetry operation of the neighbour             */
  const int32_t* numia;   /* (npsom) 0 interstitial, ia>0 inside atom ia, -2 outside        */
  const int32_t* nbord;   /* (natome) boundary points of each atom                          */
  const int32_t* nbordf;  /* (natome) the first nbordf of them are outside the atom         */
  const int32_t* ibord;   /* (nbtm, natome) boundary point, 1-based                         */
  const int32_t* isbord;  /* (nbtm, natome) symmetry operation                              */
  const int32_t* isrt;    /* (nstm) outer-boundary point, 1-based                           */
  const int32_t* lato;    /* (nlmsam, natome, ngrph) L of atom harmonics                    */
  const int32_t* mato;    /* (nlmsam, natome, ngrph) m                                      */
  const int32_t* iato;    /* (nlmsam, natome, ngrph) spin of the solution                   */
  const int32_t* lso;     /* (nso1, ngrph) L of outer harmonics                             */
  const int32_t* mso;     /* (nso1, ngrph) m                                                */
  const int32_t* iso;     /* (nso1, ngrph) spin                                             */
  const double* clapl;    /* (0:nvois) Laplacian coefficients                               */
  const double* cgrad;    /* (nvois) gradient coefficients                                  */
  const double* rvol;     /* (nim) relative point volumes                                   */
  const double* poidsa;   /* (nbm, natome) atom boundary weights                            */
  const double* poidso;   /* (nsm) outer boundary weights                                   */
  const double* Ylmato;   /* (nbtm, nlmmax, natome) real harmonics at atom boundary points  */
  const double* Ylmso;    /* (nsort, nlmomax) real harmonics at outer boundary points       */
  const double* Kar;      /* (64, nspino) characters, real part                             */
  const double* Kari;     /* (64, nspino) characters, imaginary part                        */
} fdmgpu_grid;

/* Per-call arguments of mat_solve. */
typedef struct fdmgpu_energy {
  int32_t nligne;     /* matrix order                                                        */
  int32_t nligneso;   /* rows before the outer-sphere rows (nligne - nlmso when regular)     */
  int32_t nlmso;      /* outer harmonics = number of right-hand sides                        */
  int32_t lmaxso;     /* outer l cut-off (Bessel second dim is 0:lmaxso)                     */
  int32_t nlmagm;     /* second dim of phiato                                                */
  int32_t nphiato1;   /* leading dim of phiato                                               */
  int32_t nphiato7;   /* last dim of phiato (2 when phiato is complex)                       */
  int32_t nspinp;     /* spin dim of phiato                                                  */
  int32_t n_RI;       /* regular (1) or regular+irregular (2)                                */
  int32_t n_ato_RI;   /* atomic solutions per harmonic                                       */
  int32_t nspinr;     /* spin dim of the Bessel arrays                                       */
  int32_t nsort_r;    /* leading dim of Besselr/Neumanr (nsort for real energies, else 0)    */
  int32_t nsort_c;    /* leading dim of complex Bessel/Neuman                                */
  int32_t igrph;      /* representation (1-based)                                            */
  int32_t ispin;      /* spin block (1-based)                                                */
  int32_t nicm;       /* leading dim of gradvr                                               */
  /* flags (logical in the reference) */
  int32_t Cal_comp, E_comp, Basereel, Base_hexa, irregular, Relativiste, Spinorbite,
          Repres_comp, Ylm_comp, Test_reg;
  double Enervide;    /* energy relative to vacuum (Ry)                                      */
  double Eimag;       /* imaginary part of the energy (Ry)                                   */
  const int32_t* new_;    /* (0:npoint) row of each point, 1-based, 0 for atom points       */
  const int32_t* newinv;  /* (nligne) point of each row, 0 outer, -ia atom                  */
  const int32_t* lb1;     /* (nligne) first column of each row                              */
  const int32_t* lb2;     /* (nligne) last column of each row                               */
  const int32_t* ianew;   /* (natome) row before the first harmonic row of each atom        */
  const int32_t* nlmsa;   /* (natome) harmonics per atom                                    */
  const double* Vr;       /* (npoint, nspin) potential at the grid points (Ry)              */
  const double* gradvr;   /* (nicm, 3, nspin) potential gradient (relativistic / SO)        */
  const double* phiato;   /* (nphiato1, nlmagm, nspinp, nspino, n_RI, natome, nphiato7)     */
  const double* Besselr;  /* (nsort_r, 0:lmaxso, nspinr) real j_l * sqrt(k/pi)              */
  const double* Neumanr;  /* (nsort_r, 0:lmaxso, nspinr) real n_l * sqrt(k/pi)              */
  const double* Bessel;   /* (2, nsort_c, 0:lmaxso, nspinr) complex, interleaved re/im      */
  const double* Neuman;   /* (2, nsort_c, 0:lmaxso, nspinr)                                 */
} fdmgpu_energy;

typedef struct fdmgpu_handle fdmgpu_handle;

/* Per-call diagnostics. */
typedef struct fdmgpu_info {
  int64_t nnz_profile;      /* stored entries of the profile factor                          */
  double flops_factor;      /* algorithmic flops of the factorisation (profile count)        */
  double flops_solve;       /* algorithmic flops of one forward+backward solve               */
  int32_t refine_iters;     /* refinement iterations used (mixed precision)                  */
  double residual;          /* final max_k ||b_k - A x_k|| / ||b_k||                          */
  double ms_assemble, ms_factor, ms_solve, ms_refine;   /* device time per phase             */
  int32_t n_fallback;       /* problems solved again in FP64 after the mixed path missed its
                               tolerance (precision escalation)                               */
  int64_t n_kernels;        /* kernels launched by the call (graph kernel nodes included)     */
  /* mixed precision only: the first refinement residual (all problems active)
   * and the escalation's factorisation, each with its algorithmic flops       */
  double ms_residual_first, flops_residual;
  double ms_escalate_factor, flops_escalate_factor;
  /* mixed precision with FDMGPU_ESCALATE_WIDE_DF64: problems factorised again
   * with double-float sums in every trailing update, and that factorisation's
   * device time and algorithmic flops                                         */
  int32_t n_wide_refactor;
  double ms_wide_refactor, flops_wide_refactor;
  /* mixed precision: device time of the classical refinement loop alone (from
   * the first residual until every problem has stopped; ms_refine less this
   * is the escalation), and the refinement steps summed over the problems     */
  double ms_refine_loop;
  int64_t refine_steps;
} fdmgpu_info;

/* Accumulation of the FP32 factor of the mixed path. */
typedef enum {
  FDMGPU_FACTOR_FP32 = 0,      /* FP32 sums throughout (default)                          */
  FDMGPU_FACTOR_WIDE_ATOM = 1, /* double-float sums in the trailing update of the steps
                                  whose tile row holds atom-harmonic rows; those steps'
                                  multipliers are large, and FP32 sums next to them cost
                                  the factor the accuracy that keeps the refinement from
                                  escalating                                              */
  FDMGPU_FACTOR_WIDE_ALL = 2   /* double-float sums in the trailing update of every step */
} fdmgpu_factor_mode;

/* Arithmetic units of the FP32 tile updates of the mixed path (the trailing
 * update of the factor, source/mat_solve_gaussian.f90:231-262 in tile form,
 * and the forward / backward updates of the refinement solves). */
typedef enum {
  FDMGPU_ENGINE_SIMT = 0,      /* FP32 FMA pipes, one register-blocked 64x64x64 product
                                  per CTA                                                */
  FDMGPU_ENGINE_TCGEN05 = 1,   /* tensor cores (tcgen05.mma kind::tf32), operands split
                                  hi + lo into TF32 pairs, three products per tile pair:
                                  the accuracy of FP32 products, FP32 accumulation       */
  FDMGPU_ENGINE_TCGEN05_FACTOR = 2, /* tensor cores for the factor's trailing update only;
                                  the refinement solves on the FP32 pipes                */
  FDMGPU_ENGINE_SIMT_STREAM = 3 /* (default) FP32 pipes, one operand tile per CTA held in shared
                                  memory while the tiles it multiplies stream through
                                  a two-stage ring filled by bulk copies (cp.async.bulk,
                                  mbarrier completion); also the double-float updates
                                  of the escalation                                     */
} fdmgpu_tile_engine;

/* Order of the triangular solves of the mixed path's refinement (the
 * resolution loop of source/mat_solve_gaussian.f90:348-358 and its forward
 * counterpart, in tile form). */
typedef enum {
  FDMGPU_SOLVE_COLUMNS = 0,    /* step by step: the diagonal tile, then the update of every
                                  row below (above) it, two launches per tile step       */
  FDMGPU_SOLVE_ROWS = 1        /* row by row: each row's strip of products summed in
                                  registers, then its diagonal tile, one launch per tile
                                  row; every right-hand-side tile written once           */
} fdmgpu_solve_order;

/* Arithmetic units of the double-float trailing update of the escalation
 * factor (the energies whose FP32 refinement stalls). */
typedef enum {
  FDMGPU_DF64_SIMT = 0,        /* FP32 pipes, about 12 instructions per multiply-add      */
  FDMGPU_DF64_TCGEN05 = 1      /* (default) tensor cores: rows of L and columns of U scaled by powers
                                  of two and cut into seven 7-bit integer slices (exact
                                  bf16), the 34 slice pairs of orders <= 9 multiplied by
                                  tcgen05.mma kind::f16 into one FP32 accumulator per
                                  order, exact (sums below 2^24), combined in double-float */
} fdmgpu_df64_engine;

/* Library version string. */
const char* fdmgpu_version(void);

/* Message of the last error on this thread. */
const char* fdmgpu_last_error(void);

/* Create a handle on the current CUDA device and upload the energy-independent
 * arguments (the grid, stencil, boundary and harmonic tables that mat_solve
 * receives on every call, source/mat_solve_gaussian.f90:30-67). */
fdmgpu_status fdmgpu_create(const fdmgpu_grid* grid, fdmgpu_handle** out);

/* Release every device resource held by the handle. */
void fdmgpu_destroy(fdmgpu_handle* h);

/* Drop-in for mat_solve (source/mat_solve_gaussian.f90:5-372 and
 * source/mat_solve_mumps.f90:5-261): assemble the FDM matrix and the right-hand
 * sides of one energy on the GPU, factorise, solve, and write the solution into
 * smr (nlmso, nligne) column-major (and smi when Cal_comp).  Synchronous.
 * smr/smi are host pointers.  info may be NULL.
 * Complex problems (Cal_comp: complex harmonics, spin-orbit with nspino = 2,
 * relativistic terms; real or complex energies (E_comp), complex basis, C1
 * characters; the regular solution, or FDM_comp's irregular one with both
 * atomic solutions: irregular = 1, n_RI = n_ato_RI = 2, Test_reg = 0,
 * nligneso = nligne) are solved as their real-equivalent system with
 * tile-local pivoting, in FP64 or in mixed precision (FP32 factor,
 * double-float residual refinement); smi must be given. */
fdmgpu_status fdmgpu_mat_solve(fdmgpu_handle* h, const fdmgpu_energy* e, int32_t precision,
                               double* smr, double* smi, fdmgpu_info* info);

/* Residual arithmetic of the mixed precision refinement (default DF64).
 * No counterpart in the reference, which solves in FP64 only. */
fdmgpu_status fdmgpu_set_residual_mode(fdmgpu_handle* h, int32_t mode);

/* Refinement scheme of the mixed precision path and the Krylov dimension of
 * one GMRES cycle (1..16, default 12).  No counterpart in the reference. */
fdmgpu_status fdmgpu_set_refinement(fdmgpu_handle* h, int32_t mode, int32_t krylov_dim);

/* Escalation arithmetic for energies the FP32 factors cannot refine.  No
 * counterpart in the reference. */
fdmgpu_status fdmgpu_set_escalation(fdmgpu_handle* h, int32_t mode);

/* Stopping rule of the mixed precision refinement: an energy stops when the
 * correction max|dx|/max|x| falls to tol (default 1e-10); when it stalls
 * above tol it is accepted if at most tol_accept (default 1e-7 with the df64
 * residual, 1e-9 with FP64), else solved again by escalation.  0 selects the
 * default.  No counterpart in the reference. */
fdmgpu_status fdmgpu_set_tolerance(fdmgpu_handle* h, double tol, double tol_accept);

/* Accumulation mode of the FP32 factor (fdmgpu_factor_mode), for the
 * batches planned after the call.  No counterpart in the reference. */
fdmgpu_status fdmgpu_set_factor_mode(fdmgpu_handle* h, int32_t mode);

/*
 * Radial tables for per-energy inputs generated on the device (real path).
 * With them, an energy whose phiato, Besselr and Neumanr are all NULL has
 * those inputs computed on the GPU: the regular radial solution of each atom
 * type by the three-point recursion of Sch_radial (source/sphere.f90:324-396,
 * :519-523 start, :583-695 recursion), interpolated onto the atom's boundary
 * points and multiplied by Ylmato as cal_phiato does (source/sphere.f90:
 * 3225-3370, f_interp2 source/tools.f90:504-522), and the outer Bessel and
 * Neumann values of phiso (source/mat.f90:739-1028, cbessneur
 * source/sphere.f90:7356-7384) at k = sqrt(Enervide - v0bd - dv_spin(ispin)).
 * The energy's nlmsa give each atom's l cut-off and nlmagm the layout.
 * No counterpart in the reference, which computes them on the host per energy.
 */
typedef struct fdmgpu_radial {
  int32_t ntype;          /* atom types (<= 8)                                              */
  int32_t nr_max;         /* leading dimension of r and V                                    */
  int32_t nspin;          /* spin blocks of dv_spin                                          */
  const int32_t* nr;      /* (ntype) mesh points of each type                               */
  const double* r;        /* (nr_max, ntype) radial mesh (bohr), increasing                 */
  const double* V;        /* (nr_max, ntype) spherical potential of each type (Ry)          */
  const double* dv_spin;  /* (nspin) spin shift of the potential (Ry)                       */
  const double* z_origin; /* (ntype) charge of the expansion of u_L at the origin           */
  const int32_t* itype;   /* (natome) type of each atom, 1-based                            */
  const double* rrel;     /* (nbtm, natome) distance of each boundary point to its atom     */
  const double* rsort;    /* (nsort) distance of each outer point to the absorber (bohr)    */
  double v0bd;            /* interstitial level: kinetic energy = Enervide - v0bd - dv (Ry) */
} fdmgpu_radial;
fdmgpu_status fdmgpu_set_radial(fdmgpu_handle* h, const fdmgpu_radial* radial);

/* Engine of the double-float trailing update (fdmgpu_df64_engine) for the
 * mixed batches planned after the call.  No counterpart in the reference. */
fdmgpu_status fdmgpu_set_df64_engine(fdmgpu_handle* h, int32_t engine);

/* Solve order of the mixed batches planned after the call (fdmgpu_solve_order).
 * No counterpart in the reference. */
fdmgpu_status fdmgpu_set_solve_order(fdmgpu_handle* h, int32_t order);

/* Tile engine of the FP32 updates (fdmgpu_tile_engine) for the real mixed
 * batches planned after the call; steps that accumulate wide
 * (FDMGPU_FACTOR_WIDE_ATOM) stay on the FP32 pipes.  No counterpart in the
 * reference. */
fdmgpu_status fdmgpu_set_tile_engine(fdmgpu_handle* h, int32_t engine);

/* Autotuner (on by default): when a batch needs a new plan, the trailing
 * update of the factor is timed on this batch with 64 threads per 64x64 tile
 * pair (8x8 accumulators per thread) and with 128 (8x4), over eight steps
 * from the middle of the band, and the faster layout is used for the plan.
 * fdmgpu_get_tuning reports the layout chosen for a precision (0 before the
 * first plan) and the two trial times.  No counterpart in the reference. */
fdmgpu_status fdmgpu_set_autotune(fdmgpu_handle* h, int32_t on);
fdmgpu_status fdmgpu_get_tuning(fdmgpu_handle* h, int32_t precision, int32_t* trailing_threads, double* ms64,
                                double* ms128);

/* Measured FMA rates of the current GPU's FP32 and FP64 pipes (TFLOP/s, 2
 * flops per FMA), the roofline peaks of the kernels that run on them.
 * Allocates a few bytes of device memory; takes ~0.1 s.  No counterpart in
 * the reference. */
fdmgpu_status fdmgpu_measure_pipe_peaks(double* fp32_tflops, double* fp64_tflops);

/* Counterpart of getSolverParams (source/mat_solve_gaussian.f90:376-389,
 * source/mat_solve_mumps.f90:705-736): solver name "GPU" and group size 1. */
void fdmgpu_get_solver_params(int32_t* mpi_host_num_for_mumps, char solver[6]);

/*
 * Batched spectrum: every energy of a spectrum (and every spin block) solved
 * in one captured launch sequence, with the Taull contraction of `mat`
 * (source/mat.f90:306-405) and its symmetrisation (source/mat.f90:598-644) on
 * the device.  The caller adds the per-energy arguments, runs, then reads the
 * absorber scattering amplitude Taull(nlm, nlm) (complex, interleaved re/im,
 * column-major, nlm = nlmsa(iaabs)) of each energy.
 */
fdmgpu_status fdmgpu_batch_begin(fdmgpu_handle* h, int32_t precision, int32_t max_energies);
fdmgpu_status fdmgpu_batch_add(fdmgpu_handle* h, const fdmgpu_energy* e, int32_t iaabs);
/* Add an energy of another absorbing site: e refers to the grid of the handle
 * `site` (its own fdmgpu_create), and the problem joins h's batch, so the
 * energies of several sites with different grids and orders run in one
 * launch sequence.  fdmgpu_batch_add(h, e, iaabs) is the case site = h.  The
 * site handle must outlive the batch's runs.  vjp and adjoint_dot need a
 * single-site batch. */
fdmgpu_status fdmgpu_batch_add_site(fdmgpu_handle* h, fdmgpu_handle* site, const fdmgpu_energy* e, int32_t iaabs);
fdmgpu_status fdmgpu_batch_run(fdmgpu_handle* h, fdmgpu_info* info);
/* Device memory a batch's pools may take (bytes; 0, the default, selects 85%
 * of the device's memory).  A batch above it runs in consecutive chunks of
 * energies, each planned and launched like a batch of its own; Taull and the
 * statistics of every energy are kept (on the host), while solutions,
 * cross-sections, inputs and the adjoint (which need the pools) return
 * FDMGPU_ERR_UNSUPPORTED.  fdmgpu_batch_rerun of a chunked batch runs every
 * chunk again.  No counterpart in the reference, whose energies each hold
 * their own matrix. */
fdmgpu_status fdmgpu_set_memory_budget(fdmgpu_handle* h, double bytes);
/* Run the last batch again on the inputs already in device memory (no host
 * copies): the device-resident timing of a spectrum.  No counterpart in the
 * reference. */
fdmgpu_status fdmgpu_batch_rerun(fdmgpu_handle* h, fdmgpu_info* info);
/* Taull of energy k (0-based, in add order): writes nlm*nlm complex values,
 * column-major, indexed by Lm0 - 1 = L^2 + L + m on both sides.  For a complex
 * batch nlm = nspino * (lmax + 1)^2 and the index is (Lm0 - 1) + (lmax + 1)^2
 * (spin - 1), the reference's Taull(Lm0, spin, Lm0', spin'). */
fdmgpu_status fdmgpu_batch_taull(fdmgpu_handle* h, int32_t k, double* taull, int32_t* nlm);
/* Tau_RI of FDM_comp (source/mat.f90:219-292, the complex-energy mode with
 * the irregular solution, source/fdm.f90:1734-1738) from the batch's regular
 * solution k_reg and irregular solution k_irr (irregular = 1, n_ato_RI = 2) of
 * the same energy, site and absorber: writes 2*nlm*nlm complex values, the
 * Taull layout of fdmgpu_batch_taull for i_RI = 1 (amplitudes of the
 * irregular problem's regular atomic solution) then i_RI = 2 (irregular
 * atomic solution).  Computed on the device from the two solutions.  Returns
 * the pair's solve status (FDMGPU_ERR_NOT_CONVERGED if either did not
 * converge); refuses a batch that ran in chunks. */
fdmgpu_status fdmgpu_batch_tau_ri(fdmgpu_handle* h, int32_t k_reg, int32_t k_irr, double* tau_ri, int32_t* nlm);
/* Taull of every energy in one copy: nlm_k*nlm_k complex values per energy,
 * concatenated in add order (capacity counts doubles). */
fdmgpu_status fdmgpu_batch_taull_all(fdmgpu_handle* h, double* taull, int64_t capacity);
/* Solution of energy k (nlmso, nligne) column-major into smr (host).  For a
 * complex batch (nlmso, 2 nligne): column 2ii-1 holds Re x(ii), 2ii Im x(ii). */
fdmgpu_status fdmgpu_batch_solution(fdmgpu_handle* h, int32_t k, double* smr);
/* Per-energy diagnostics of the last run: refinement (outer) iterations,
 * final relative correction max|dx|/max|x|, whether the energy was solved
 * again in FP64, and the GMRES steps summed over the refinement.  Returns the
 * energy's status (FDMGPU_OK when it converged).  Any pointer may be NULL. */
fdmgpu_status fdmgpu_batch_stats(fdmgpu_handle* h, int32_t k, int32_t* iters, double* residual,
                                 int32_t* fallback, int32_t* inner_iters);

/* The per-energy inputs energy k of the last run was assembled from, as the
 * device holds them: phiato (nbtm, nlmagm, natome) of its spin block and
 * Besselr, Neumanr (nsort, 0:lmaxso), column-major.  Real problems; any
 * pointer may be NULL.  For checking inputs generated on the device
 * (fdmgpu_set_radial).  No counterpart in the reference. */
fdmgpu_status fdmgpu_batch_inputs(fdmgpu_handle* h, int32_t k, double* phiato, double* besselr, double* neumanr);

/*
 * Dipole absorption of the last batch, in FP64 on the device, from the Taull
 * already in device memory: the K-edge E1E1 channel of tens_ab
 * (source/tensor.f90:1218-1264) and the Lorentzian convolution of the
 * spectrum (source/convolution.f90:1612-1680).  One problem per energy, added
 * in increasing energy order.
 *   energies_ev (n)   photon energies of the batch's problems (add order);
 *   half_width  (n)   Lorentzian half width per energy (the reference's bb);
 *   width_per_input   0: the width of the output energy (bb(ie)), 1: of the
 *                     input bin (Gamma_var);
 *   weight      (n)   |radial integral|^2 per energy, or NULL for 1;
 *   sigma       (n)   out: sigma(E) = -Im sum over the L = 1 block of w Taull
 *                     (both spin blocks for a complex batch);
 *   sigma_conv  (n)   out or NULL: the convolved spectrum;
 *   tensor      (9n)  out or NULL (real batches): S(a, b) = -Im w (T(a,b) +
 *                     T(b,a)) / 2 for a, b in x, y, z, row-major per energy.
 * Host pointers.  Synchronous.
 */
fdmgpu_status fdmgpu_batch_xanes(fdmgpu_handle* h, const double* energies_ev, const double* half_width,
                                 int32_t width_per_input, const double* weight, double* sigma, double* sigma_conv,
                                 double* tensor);

/*
 * Vector-Jacobian product of the last batch: given the cotangent
 * gtaull = dL/d(Im Taull) of every energy (nlm*nlm reals per energy,
 * column-major, concatenated in add order), writes dL/dVr into grad_vr
 * (npoint, nspin), column-major like Vr.  It reuses the batch's factors
 * (transposed solves A^T Lambda = dL/dX) and its solutions; Vr enters the FDM
 * matrix on the diagonal of the grid rows (source/mat.f90:1151-1156).  After
 * an FP64 batch the FP64 factors solve A^T directly; after a mixed batch the
 * FP32 (or, for escalated energies, double-float) factors of the equilibrated
 * matrix are refined with a double-float transposed residual (classical or
 * recurrence refinement with double-float escalation).  Points inside atoms
 * get 0.  ms (may be NULL) receives the device time.  Real-basis batches only
 * (a complex batch returns FDMGPU_ERR_UNSUPPORTED).  No counterpart in the
 * reference.
 */
fdmgpu_status fdmgpu_batch_vjp(fdmgpu_handle* h, const double* gtaull, double* grad_vr, double* ms);

/*
 * Parameter gradients through the adjoint.  For a parameter theta that moves
 * matrix values but not the grid structure (a shell distance: atom positions,
 * the potential and the atomic boundary functions change, grid membership and
 * row numbering do not), dL/dtheta = Lambda^T (dB/dtheta - dA/dtheta X).
 * fdmgpu_batch_adjoint_dot assembles A' and B' from the energy arguments e[k]
 * (same row structure as the batch's energy k) and writes, per energy,
 * out[k] = sum_c Lambda_c^T (B'_c - A' X_c) with the X and Lambda of the last
 * fdmgpu_batch_run + fdmgpu_batch_vjp.  Central differences of out over
 * theta +- h give dL/dtheta with O(h^2) error in the assembly only.  The
 * batch's factors are overwritten: run the batch again before another vjp.
 *
 * fdmgpu_update_grid_values replaces the real-valued tables of the handle's
 * grid (rvol, poidsa, poidso, Ylmato, Ylmso, Kar, clapl) by those of g, whose
 * integer structure must equal the handle's (else FDMGPU_ERR_ARG).
 * No counterparts in the reference.
 */
fdmgpu_status fdmgpu_update_grid_values(fdmgpu_handle* h, const fdmgpu_grid* g);
fdmgpu_status fdmgpu_batch_adjoint_dot(fdmgpu_handle* h, const fdmgpu_energy* const* e, int32_t n, double* out);

/*
 * Taull of one energy from a solution that is already in device memory,
 * without allocating any device memory.  No counterpart in the reference,
 * where mat forms Taull on the host right after mat_solve
 * (source/mat.f90:306-405, symmetrised at :598-644).
 *
 * Who needs it: a caller that keeps smr on the GPU but may not allocate
 * there.  Examples are a host code whose own memory pool already holds nearly
 * all device memory, so a cudaMalloc here would fail, and a per-energy loop
 * that shares the GPU with work on other streams, where cudaFree would stall
 * all of it (cudaFree synchronises the whole device).  fdmgpu_batch_* allocate
 * their pools on first use and are no use to such a caller.
 *
 * d_smr     device, (nlmso, nligne) column-major FP64: the layout
 *           fdmgpu_mat_solve writes smr in.
 * ianew_abs row offset of the absorber's rows, as ianew(iaabs) of mat_solve;
 *           the absorber rows are ianew_abs + 1 .. ianew_abs + nlm_abs.
 * d_taull   device, nlm_abs * nlm_abs complex values: interleaved re/im,
 *           column-major, 16-byte aligned.  Same layout as
 *           fdmgpu_batch_taull.
 * d_status  device int32 or NULL.  The kernel sets it to FDMGPU_OK, or to
 *           FDMGPU_ERR_ZERO_PIVOT when norm is singular.
 * stream    a cudaStream_t, NULL for the default stream.  The call only
 *           enqueues one kernel on it and returns.
 *
 * Limits: nlmso <= FDMGPU_TAULL_NOALLOC_MAX_NLMSO, and the working matrix,
 * nlmso * (nlmso + nlm_abs) * 16 bytes, must fit in the fixed
 * FDMGPU_TAULL_NOALLOC_SCRATCH_BYTES (2 MiB) array that the library's device
 * image holds for it.  Larger sizes return FDMGPU_ERR_ARG and enqueue nothing.
 * Nothing has to start at zero: the kernel writes every element of that array
 * before reading it, and writes *d_status itself.
 *
 * Ordering: there is one such array per device, shared by all calls on that
 * device.  Calls that can overlap on the GPU race on it: calls from several
 * host threads, or on more than one stream.  The caller must order them, for
 * example by issuing them all on one stream.
 *
 * The first call on each device looks up the array's address, with that
 * device current, and so does the first call after the device's context was
 * replaced (cudaDeviceReset): the address is kept per CUDA context.  That
 * lookup can load the library's device code.  A caller that captures streams
 * should make one call on each device before capture.
 */
#define FDMGPU_TAULL_NOALLOC_SCRATCH_BYTES (2 * 1024 * 1024)
#define FDMGPU_TAULL_NOALLOC_MAX_NLMSO 512
fdmgpu_status fdmgpu_taull_noalloc(const double* d_smr, int32_t nlmso, int32_t nligne, int32_t ianew_abs,
                                   int32_t nlm_abs, double* d_taull, int32_t* d_status, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* FDMGPU_H */
