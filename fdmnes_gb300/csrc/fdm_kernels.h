// fdm_kernels.h - host-side launch interface shared by the CUDA translation units.
#pragma once

#include <vector>
#include <cuda_runtime.h>

#include "fdm_internal.cuh"

namespace fdm {

// Largest number of work items per step over the problems of a batch.
struct StepPlan {
  int ntmax = 0;
  int nrtmax = 0;
  std::vector<int> panel, panel_rhs;   // L + U tiles (+ RHS tiles) of step K
  std::vector<int> trail, trail_rhs;   // trailing tiles (+ RHS tiles) of step K
  std::vector<int> fwd, bwd;           // forward / backward update tiles of step K
  std::vector<int> tfwd, tbwd;         // the same for the transposed solves (U^T, then L^T)
  std::vector<int> wide_any;           // step K of some problem accumulates wide (FP32 factor)
  // FP32 tile updates on the tensor cores (tc_update.cu): work items (two tile
  // rows x up to four tile columns) of the trailing update with the fused
  // right-hand sides, and of the forward / backward solve updates
  int tc = 0;        // trailing update of the FP32 factor on the tensor cores
  int tc_solve = 0;  // forward / backward updates of the FP32 solves on the tensor cores
  std::vector<int> trail_tc, fwd_tc, bwd_tc;
  int* tc_err = nullptr;               // per-problem status word of the solve updates (mbarrier timeout)
  int row_solve = 0;                   // forward / backward solves row by row (one launch per tile row)
  // double-float trailing update on the tensor cores through integer slices
  // (oz_update.cu): per step the operand tiles (max over problems) and the
  // CTAs; per problem a scratch slot of oz_capI + oz_capC tiles of images
  int oz = 0;
  std::vector<int> oz_nI, oz_nC, oz_items;
  // FP32 / double-float tile updates as bulk-copy-staged strips
  // (strip_update.cu): CTAs per step of the trailing update (without and with
  // the right-hand-side columns) and of the forward / backward solve updates
  int strip = 0;
  std::vector<int> strip_trail, strip_trail_rhs, strip_fwd, strip_bwd;
  // double-float panel as products with the inverted diagonal triangles (with
  // the strips): CTAs per step for the L tiles and the U (+ RHS) tiles, and the
  // per-problem inverse scratch (U^-1, L^-1)
  std::vector<int> strip_panel_l, strip_panel_u, strip_panel_u_rhs;
  dfl* dfl_inv = nullptr;
  // U^-1 of every step of the last double-float factorisation (ntmax tiles a
  // problem), when the caller keeps them for a backward solve
  dfl* dfl_uinv_keep = nullptr;
  int oz_capI = 0, oz_capC = 0;
  unsigned char* oz_img = nullptr;
  int* oz_exp = nullptr;
};

void setup_strip_kernels();
int strip_items(int nI, int nC, int G);
int strip_rows(int mode);
// mode 0: factor trailing update (fuse_rhs: with the right-hand-side columns;
// wide: the FP32 problems whose step is marked wide, with double-float sums);
// 1: forward solve update; 2: backward solve update
template <typename T>
void launch_strip(int mode, int items, int nprob, T* env, T* rhs, const Prob* probs, Tables tb, int K, int fuse_rhs,
                  const int* active, int* err, cudaStream_t s, bool wide);

int launch_dfl_backward_inv(const StepPlan& sp, dfl* env, dfl* rhs, const Prob* probs, Tables tb, int nprob,
                            const int* active, int* err, cudaStream_t s);
int launch_dfl_panel_inv(const StepPlan& sp, dfl* env, dfl* rhs, const Prob* probs, Tables tb, int nprob, int K,
                         int fuse_rhs, const int* active, int* err, double piv_thr, int* piv, dfl* inv,
                         cudaStream_t s);

void setup_oz_kernels();
int64_t oz_tile_bytes();
int launch_oz_update(const StepPlan& sp, dfl* env, dfl* rhs, const Prob* probs, Tables tb, int nprob, int K,
                     const int* active, int* err, cudaStream_t s);

// Split-TF32 tcgen05 tile updates (tc_update.cu).  mode 0: factor trailing
// update C -= L U with the fused right-hand sides; 1: forward solve update
// Y(I) -= L(I,K) Y(K); 2: backward solve update Y(I) -= U(I,K) Y(K).
void setup_tc_kernels();
void launch_tc_update(int mode, int items, int nprob, float* env, float* rhs, const Prob* probs, Tables tb, int K,
                      const int* active, int* err, cudaStream_t s);
int tc_items(int nI, int nC);

template <typename T> void setup_factor_kernels();
template <typename T>
int launch_factor(const StepPlan& sp, T* env, T* rhs, const Prob* probs, Tables tb, int nprob, int fuse_rhs,
                  const int* active, int* err, double piv_thr, int* piv, cudaStream_t s, int trail_threads = 0,
                  int k_begin = 0, int k_end = -1);
template <typename T>
int launch_forward(const StepPlan& sp, const T* env, T* rhs, const Prob* probs, Tables tb, int nprob,
                    const int* active, const int* piv, cudaStream_t s);
template <typename T>
int launch_backward(const StepPlan& sp, const T* env, T* rhs, const Prob* probs, Tables tb, int nprob,
                     const int* active, cudaStream_t s);

// Transposed solves with the factors of launch_factor: U^T w = g (forward over
// K), then the block-lower factor M of A = M U transposed (backward over K,
// tile-local row orders undone).  Together they solve A^T x = g.
template <typename T>
void launch_forward_t(const StepPlan& sp, const T* env, T* rhs, const Prob* probs, Tables tb, int nprob,
                      const int* active, cudaStream_t s);
template <typename T>
void launch_backward_t(const StepPlan& sp, const T* env, T* rhs, const Prob* probs, Tables tb, int nprob,
                       const int* active, const int* piv, cudaStream_t s);

// Device pools of one batch (pointers into device memory).
struct Pools {
  const int* ipool = nullptr;      // per-problem integer inputs
  const double* dpool = nullptr;   // per-problem double inputs
  double* env64 = nullptr;         // FP64 band tiles
  float* env32 = nullptr;          // FP32 band tiles (mixed precision)
  double* B64 = nullptr;           // FP64 right-hand sides (tiles)
  double* X64 = nullptr;           // FP64 solution (tiles)
  float* Y32 = nullptr;            // FP32 work right-hand sides (tiles)
  double* rs = nullptr;            // row scales (per row, stride npad + 1)
  double* cs = nullptr;            // column scales
  int* rowptr = nullptr;           // CSR row pointers (stride npad + 1)
  int* piv = nullptr;              // tile-local row order of the FP32 factor (stride npad + 1)
  int* col = nullptr;              // CSR columns
  double* val = nullptr;           // CSR values
  float2* val2 = nullptr;          // CSR values as double-float (hi, lo)
  float2* Xs = nullptr;            // solution as double-float (hi, lo), RHS tile layout
  double* taull = nullptr;         // complex Taull (interleaved)
  double* tscratch = nullptr;      // complex Taull scratch
  unsigned long long* dmax = nullptr;  // per problem max |correction| (double bits)
  unsigned long long* xmax = nullptr;  // per problem max |x| (double bits)
  unsigned long long* amax = nullptr;  // per problem scratch
  int* err = nullptr;
  int* active = nullptr;
  float* R32 = nullptr;            // residual of the scaled system, updated by recurrence
  int* act_df = nullptr;           // active problems that take a true (double-float) residual
  int* act_rec = nullptr;          // active problems that take the recurrence residual
  // GMRES-IR
  float* valS = nullptr;           // equilibrated FP32 CSR values
  float* V = nullptr;              // Krylov basis, (m+1) vectors of vstride floats
  int64_t vstride = 0;
  float* W = nullptr;              // work vector
  void* gstate = nullptr;          // per-column GMRES state
  int* active_gm = nullptr;        // problems refined by GMRES cycles (subset of active)
  int* inner_active = nullptr;
  int* jdone = nullptr;
  int* notconv = nullptr;
};

struct LaunchDims {
  int nprob = 0;
  int max_rows = 0;        // max npad
  int max_tiles = 0;       // max band tiles of one problem
  int max_rhs_tiles = 0;   // max nt * nrt
  int max_nlmso = 0;
  int max_atom_rows = 0;   // natome * max nlmsa
  int npr = 0;             // max interstitial points over the batch's sites
  int max_nsortf = 0;      // max outer-boundary points inside the sphere over the sites
  int max_natome = 0;      // max atoms over the sites
  int max_nlmsa = 0;       // max harmonics of one atom over the batch
  int64_t rowv_total = 0;  // entries of the per-row vectors (sum of npad + 1)
};

// Device-side stopping rule of the classical refinement (refine.cu).
struct RefineState {   // per problem
  int active, slow, iters, pad;
  double prev, resid;
};
struct RefineCtl {     // per batch
  int it;              // refinement steps done
  int max_iter;
  double tol;
  int nact;            // problems still active after the last step
  int pad;
};
void launch_refine_init(RefineState* rs, int* active, int np, cudaStream_t s);
void launch_refine_check(RefineState* rs, int* active, const Pools& pl, RefineCtl* ctl, int np,
                         cudaGraphConditionalHandle cond, int use_cond, cudaStream_t s);

// Generated per-energy inputs (radial.cu).
struct GenDims {
  int nprob_gen = 0;   // problems with generated inputs
  int ntype_max = 0;
  int lmax1 = 1;       // max l cut-off + 1 over the generated problems and types
  int natome_max = 0;
  int nsort_max = 0;
  int nr_max = 0;
};
void launch_generate_inputs(const Prob* probs, const RadialDev* rads, const StaticDev* sites, const int* ipool,
                            const LaunchDims& d, const GenDims& g, double* U, double* dpool, cudaStream_t s);

// Dipole absorption and tensor per energy, Lorentzian convolution (xsection.cu).
void launch_dipole(const Prob* probs, const double* taull, const double* weight, int nprob, double* sigma,
                   double* tensor, cudaStream_t s);
void launch_lorentz(const double* E, const double* x, const double* width, int width_per_input, int n, double* out,
                    cudaStream_t s);

void launch_assemble(const StaticDev* sites, const Prob* probs, const Pools& pl, Tables tb, const LaunchDims& d,
                     cudaStream_t s);
// Complex problems in their real-equivalent form (complex.cu).
void launch_assemble_c(const StaticDev* sites, const Prob* probs, const Pools& pl, Tables tb, const LaunchDims& d,
                       int basereel, cudaStream_t s);
void launch_taull_c(const StaticDev* sites, const Prob* probs, const Pools& pl, const LaunchDims& d, int max_nlm,
                    cudaStream_t s);
// Tau_RI of FDM_comp from a regular problem (*preg) and an irregular one
// (*pirr) of the same site and absorber: (nlm, nlm, 2) complex into out.
void launch_tau_ri(const StaticDev* sites, const Prob* preg, const Prob* pirr, const double* X, int nlm, double2* out,
                   cudaStream_t s);
void launch_equilibrate_convert(const Prob* probs, const Pools& pl, Tables tb, const LaunchDims& d, cudaStream_t s);
void launch_csr(const Prob* probs, const Pools& pl, Tables tb, const LaunchDims& d, cudaStream_t s);
void launch_convert_masked(const Prob* probs, const Pools& pl, Tables tb, const LaunchDims& d, cudaStream_t s);
// X64 = cs * Y32 (first solve) or X64 += cs * Y32 (refinement), with max reductions.
void launch_update_x(const Prob* probs, const Pools& pl, const LaunchDims& d, int first, cudaStream_t s);
// Y32 = rs * (B64 - A X64) using the CSR copy of A, in FP64 or in double-float.
void launch_residual(const Prob* probs, const Pools& pl, const LaunchDims& d, int df64, cudaStream_t s);
void launch_csr_scale(const Prob* probs, const Pools& pl, const LaunchDims& d, cudaStream_t s);
void launch_gmres_cycle(const StepPlan& sp, const Prob* probs, const Pools& pl, Tables tb, const LaunchDims& d, int m,
                        float tol, cudaStream_t s);
size_t gmres_state_bytes();
int gmres_max_dim();
void launch_copy_rhs(const Prob* probs, const Pools& pl, const LaunchDims& d, cudaStream_t s);
int launch_dfl_escalation(const StepPlan& sp, const Prob* probs, const Pools& pl, Tables tb, const LaunchDims& d,
                           dfl* D, cudaStream_t s, cudaEvent_t ev_f0 = nullptr, cudaEvent_t ev_f1 = nullptr);
void launch_gather_probs(const Prob* probs, const int* list, int n, Prob* out, cudaStream_t s);
void launch_scatter_err(const int* list, int n, const int* err_c, int* err, cudaStream_t s);
int launch_dfl_factor_f32(const StepPlan& sp, const Prob* probs, const Pools& pl, Tables tb, const LaunchDims& d,
                          dfl* D, cudaStream_t s, cudaEvent_t ev_f0, cudaEvent_t ev_f1);
int launch_dfl_refine_step(const StepPlan& sp, const Prob* probs, const Pools& pl, Tables tb, const LaunchDims& d,
                           dfl* D, cudaStream_t s);
void launch_resid_update(const Prob* probs, const Pools& pl, const LaunchDims& d, cudaStream_t s);
void launch_copy_rhs32(const Prob* probs, const LaunchDims& d, const float* src, float* dst, const int* mask,
                       cudaStream_t s);
void launch_csr_nnz(const Prob* probs, const int* rowptr, const LaunchDims& d, int* nnz, cudaStream_t s);
cudaError_t taull_noalloc_scratch(double2** out);
cudaError_t launch_taull_noalloc(const double* smr, int nlmso, int nligne, int ianew_abs, int nlm_abs,
                                 double2* scratch, double* taull, int* status, cudaStream_t s);
void launch_taull_vjp(const Prob* probs, const LaunchDims& d, const double* X, const double* gT, double* scratch,
                      double* G, int* err, cudaStream_t s);
void launch_grad_vr(const StaticDev& S, const Prob* probs, const int* ipool, const LaunchDims& d, int nspin,
                    const double* X, const double* Lam, double* part, double* grad, cudaStream_t s);
void launch_csr_scan(const Prob* probs, int* ptr, const LaunchDims& d, cudaStream_t s);
void launch_rhs_to_dfl(const Prob* probs, const LaunchDims& d, const double* B, const float* Y, const double* scale,
                       dfl* D, int from_b, const int* mask, cudaStream_t s);
void launch_dfl_to_x(const Prob* probs, const LaunchDims& d, const dfl* D, double* X, float2* Xs, const double* scale,
                     int first, unsigned long long* dmax, unsigned long long* xmax, const int* mask, cudaStream_t s);
void launch_csc_build(const Prob* probs, const Pools& pl, const LaunchDims& d, int* colptr, int* cursor, int* cscrow,
                      float2* cscval2, cudaStream_t s);
void launch_lambda_dot(const Prob* probs, const Pools& pl, const LaunchDims& d, const double* Lam, double* rowpart,
                       double* out, cudaStream_t s);
void launch_taull(const Prob* probs, const Pools& pl, const LaunchDims& d, const double* X, cudaStream_t s);
void launch_solution_out(const Prob& P, const double* X, double* smr_dev, cudaStream_t s);

}  // namespace fdm
