// capi.cu - the C-ABI of include/fdmgpu.h: handle, static upload, per-problem
// planning of the band tiles, device pools and the launch sequences.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/fdmgpu.h"
#include "fdm_internal.cuh"
#include "fdm_kernels.h"

using namespace fdm;

namespace {

thread_local std::string g_last_error;

fdmgpu_status fail(fdmgpu_status st, const std::string& msg) {
  g_last_error = msg;
  return st;
}

#define CK(call)                                                                                   \
  do {                                                                                             \
    cudaError_t _e = (call);                                                                       \
    if (_e != cudaSuccess)                                                                         \
      return fail(FDMGPU_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e));            \
  } while (0)

template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t cap = 0;  // elements
  cudaError_t reserve(size_t n) {
    if (n <= cap && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t m = std::max<size_t>(n, 1);
    cudaError_t e = cudaMalloc(&p, m * sizeof(T));
    if (e == cudaSuccess) cap = m;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
};

template <typename T>
cudaError_t upload(DevBuf<T>& b, const std::vector<T>& h, cudaStream_t s) {
  cudaError_t e = b.reserve(h.size());
  if (e != cudaSuccess) return e;
  if (h.empty()) return cudaSuccess;
  return cudaMemcpyAsync(b.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s);
}

// One problem (one energy / spin block) of a batch, host side.
struct HostProb {
  Prob P;
  std::vector<int> J0, J1, Imax, Imin;  // nt + 1
  std::vector<int64_t> strip;           // nt + 1
  std::vector<unsigned char> wide;      // nt + 1: tile row holds atom-harmonic rows
  int64_t ntiles = 0;
  int64_t nnz_cap = 0;
  int64_t nnz_profile = 0;
  double flops_factor = 0, flops_solve = 0;
  std::vector<int> in_i;
  std::vector<double> in_d;
  // offsets inside in_d of the Vr, gradvr, phiato, Bessel and Neumann blocks
  int64_t rel_grad = 0, rel_phi = 0, rel_bes = 0, rel_neu = 0;
  int64_t gen_phi = 0, gen_bes = 0;   // generated inputs: doubles of phiato and of one Bessel table
  int nlmsa_max = 0;
  uint64_t sig = 0;
};

struct Batch {
  int precision = FDMGPU_PREC_FP64;
  int cplx = -1;   // complex (1) or real (0) problems; -1 before the first energy
  int max_energies = 0;
  std::vector<HostProb> probs;
  // results
  std::vector<int> iters;
  std::vector<int> fallback;   // solved again in FP64 after the mixed path missed its tolerance
  std::vector<int> wide;       // factorised again with double-float sums in every trailing update
  std::vector<int> res64;      // assembled again and solved by the FP64 elimination (last resort)
  std::vector<int> inner;      // GMRES steps summed over the refinement
  std::vector<double> resid;
  std::vector<int> err;
  bool ran = false;
  bool lam_valid = false;  // the adjoint Lambda of the last vjp matches the batch's factors
  // a batch larger than the memory budget runs in consecutive chunks; its
  // Taull then lives on the host (concatenated in add order)
  bool chunked = false;
  int nchunks = 0;
  std::vector<double> taull_host;
  std::vector<int64_t> taull_off;   // per problem, in doubles
  std::vector<fdmgpu_handle*> sites;  // grids of the batch's problems; sites[0] is the batch's own handle
};

}  // namespace

struct fdmgpu_handle {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t stream2 = nullptr;  // escalation overlapped with the refinement of the other problems
  int overlap_escalation = 0;  // measured slower on the 401-energy Cu spectrum: off by default
  cudaEvent_t ev_join = nullptr;
  cudaEvent_t ev_esc[2 * 16] = {};  // factor start / end of up to 16 overlapped escalation batches
  DevBuf<int> d_esc_mask;
  DevBuf<int> d_esc_list, d_err_esc;  // the escalated problems and their status words (compact launches)
  DevBuf<Prob> d_probs_esc;
  DevBuf<float2> d_uinv_keep;  // U^-1 of every step of the escalation factor (strip engine)
  int* h_esc_mask = nullptr;  // pinned, 16 slots of nprob ints
  size_t h_esc_mask_cap = 0;
  DevBuf<unsigned long long> d_red_esc, d_red_tmp;
  // static structure
  fdmgpu_grid g{};
  StaticDev S{};
  std::vector<int> inter_pt_h, nb_kind_h, nb_idx_h;
  std::vector<double> nb_coef_h;
  std::vector<int> n_inter_h, has_outer_h;       // per interstitial point
  std::vector<std::vector<int>> nb_atoms_h;      // distinct atoms touched per interstitial point
  std::vector<int> numia_h, isrt_h, ibord_h, nbordf_h;
  std::vector<int> lato_h, mato_h;
  DevBuf<int> d_inter_pt, d_nb_kind, d_nb_idx, d_numia, d_nbord, d_nbordf, d_ibord, d_isbord, d_isrt, d_lato, d_mato,
      d_lso, d_mso, d_iato, d_iso;
  DevBuf<double> d_nb_coef, d_rvol, d_clapl, d_poidsa, d_poidso, d_Kar, d_YsoT, d_Ylmato, d_cgrad;
  bool chars_c1 = false;  // every character the grid uses is 1 (Kar) with Kari = 0: what the complex path needs
  // batch pools
  Batch batch;
  DevBuf<Prob> d_probs;
  DevBuf<int> d_J0, d_J1, d_Imax, d_Imin;
  DevBuf<int64_t> d_strip;
  DevBuf<int> d_ipool;
  DevBuf<double> d_dpool;
  DevBuf<double> d_env64, d_B64, d_X64, d_rs, d_cs, d_val, d_taull, d_tscratch, d_smr;
  DevBuf<double> d_gT, d_lam, d_gpart, d_grad;  // adjoint
  DevBuf<double> d_G;                            // adjoint of a mixed batch: cotangent of X
  DevBuf<float2> d_lams, d_cscval2;              // Lambda as double-float pairs; A^T values
  DevBuf<int> d_colptr, d_cursor, d_cscrow;      // CSR of A^T
  DevBuf<float> d_env32, d_Y32, d_R32;
  DevBuf<float2> d_dfl_inv;  // inverted diagonal triangles of the double-float factor (strip engine)
  DevBuf<int> d_act_df, d_act_rec;
  DevBuf<float2> d_val2, d_Xs;
  DevBuf<float> d_valS, d_V, d_W;
  DevBuf<unsigned char> d_gstate;
  DevBuf<int> d_inner, d_jdone, d_notconv, d_active_gm;
  int residual_df64 = 1;
  int refine_gmres = 0;   // GMRES-IR (1) or classical refinement (0)
  int refine_recur = 0;   // classical refinement with the residual updated by recurrence (1)
  int escalate_dfl = 1;   // escalation by a double-float (1) or an FP64 (0) factorisation
  int escalate_wide = 0;  // first a wide-accumulation FP32 re-factorisation of the stalled energies
  int escalate_f32 = 1;   // double-float factors rounded to FP32, then FP32 refinement (default)
  double mem_budget = 0;  // device bytes a batch's pools may take before it runs in chunks (0: 85% of the device)
  DevBuf<unsigned char> d_wide_all;  // every step wide (the re-factorisation's table)
  int gmres_m = 12;       // Krylov dimension of one GMRES cycle
  int autotune = 1;         // time the trailing-update layouts on each new plan
  int factor_mode = 0;      // FDMGPU_FACTOR_*: wide accumulation at the atom-harmonic steps of the FP32 factor
  int tile_engine = FDMGPU_ENGINE_SIMT_STREAM;  // FDMGPU_ENGINE_*: FP32 tile updates (default: streamed strips)
  int solve_order = FDMGPU_SOLVE_COLUMNS;  // FDMGPU_SOLVE_*: refinement solves step by step or row by row
  int df64_engine = FDMGPU_DF64_TCGEN05;   // FDMGPU_DF64_*: double-float trailing update (default: tensor cores)
  DevBuf<unsigned char> d_oz_img;          // integer-slice images of one factor step
  DevBuf<int> d_oz_exp;
  DevBuf<unsigned char> d_wide;
  int trail_threads[2] = {0, 0};        // chosen layout per precision (FP64, FP32); 0: built-in default
  double trail_ms[2][2] = {{0, 0}, {0, 0}};  // trial device ms [precision][64 | 128 threads]
  double tol = 0.0;         // refinement stop: max|dx|/max|x| (0: the default of the residual mode)
  double tol_accept = 0.0;  // accepted without escalation when refinement stalls (0: default)
  int64_t ncols = 0;      // right-hand-side columns of the batch (sum of nrt * TS)
  int64_t ncols_tmp = 0;
  DevBuf<int> d_rowptr, d_col, d_err, d_active, d_piv;
  DevBuf<unsigned long long> d_red;  // dmax | xmax | amax
  int* h_pinned_i = nullptr;
  size_t h_pinned_i_cap = 0;
  double* h_pinned_d = nullptr;
  size_t h_pinned_d_cap = 0;
  // graphs of the last plan
  uint64_t plan_sig = 0;
  uint64_t ptr_sig = 0;
  int plan_prec = -1;
  cudaGraphExec_t g_asm = nullptr, g_fac = nullptr, g_sol = nullptr, g_res = nullptr, g_iter = nullptr;
  int64_t nk_asm = 0, nk_fac = 0, nk_sol = 0, nk_res = 0, nk_iter = 0;  // kernel nodes per graph
  // classical refinement driven on the device: the stopping rule of every
  // step is evaluated by k_refine_check and a while node repeats the step
  cudaGraphExec_t g_loop = nullptr;
  int64_t nk_loop_body = 0;
  DevBuf<double> d_xs;  // cross-section inputs and outputs of fdmgpu_batch_xanes
  // radial tables of this grid's atom types (fdmgpu_set_radial) for inputs
  // generated on the device
  bool has_radial = false;
  RadialDev rad{};
  int rad_ntype = 0, rad_nr_max = 0;
  double rad_v0bd = 0.0, rad_dv_max = 0.0;
  std::vector<int> rad_itype;           // host copy, 0-based
  DevBuf<int> d_rad_i;                  // nr | itype | iidx
  DevBuf<double> d_rad_d;               // r | mcl0 | gm | gp | f2 | V | dv | z | rrel | rsort
  DevBuf<RadialDev> d_rads;             // per batch site
  DevBuf<double> d_radU;                // radial solutions of a batch
  GenDims gdims;
  DevBuf<RefineState> d_rstate;
  DevBuf<RefineCtl> d_rctl;
  StepPlan sp;
  LaunchDims dims;
  Tables tb{};
  Pools pl{};
  cudaEvent_t ev[11] = {};
  DevBuf<StaticDev> d_sites;  // static tables of every site of the batch, indexed by Prob::site
  DevBuf<int> d_nnz;  // CSR nonzeros per problem (algorithmic work of the residual)
};

namespace {

inline int32_t F2(const int32_t* a, int64_t ld, int64_t i, int64_t j) { return a[(i - 1) + (j - 1) * ld]; }

uint64_t mix(uint64_t h, uint64_t v) {
  h ^= v + 0x9e3779b97f4a7c15ULL + (h << 6) + (h >> 2);
  return h;
}

// Complex problems (Cal_comp): the complex outgoing basis with real energies,
// complex or real harmonics, optionally spin-orbit (nspino = 2, two spin
// blocks) and the relativistic terms; C1 characters; the regular solution,
// or FDM_comp's irregular one with both atomic solutions (Test_reg = 0).
fdmgpu_status check_energy_c(const fdmgpu_handle* h, const fdmgpu_energy* e) {
  const fdmgpu_grid& g = h->g;
  if (e->Repres_comp || e->Base_hexa || e->Basereel || e->nphiato7 != 2 ||
      (e->irregular ? (e->n_RI != 2 || e->n_ato_RI != 2 || e->Test_reg != 0 || !e->E_comp)
                    : (e->n_ato_RI != 1 || e->n_RI < 1 || e->n_RI > 2)))
    return fail(FDMGPU_ERR_UNSUPPORTED,
                "the library's complex path: Cal_comp, real or complex energies (E_comp), the complex basis "
                "(Basereel false), complex phiato (nphiato7 = 2); the regular solution (n_ato_RI = 1) or, with "
                "E_comp, the irregular one with both atomic solutions (n_RI = n_ato_RI = 2, Test_reg = 0)");
  if (!h->chars_c1) return fail(FDMGPU_ERR_UNSUPPORTED, "the complex path needs the C1 characters (Kar = 1, Kari = 0)");
  if (e->Spinorbite != (g.nspino == 2)) return fail(FDMGPU_ERR_ARG, "Spinorbite must match the grid's nspino");
  if (e->Spinorbite && (g.nspin != 2 || e->nspinp != 2 || e->nspinr != 2))
    return fail(FDMGPU_ERR_UNSUPPORTED, "spin-orbit needs two spin blocks (nspin = nspinp = nspinr = 2)");
  if (!e->Spinorbite && e->nspinr != 1) return fail(FDMGPU_ERR_ARG, "nspinr must be 1 without spin-orbit");
  if (e->nligne <= 0 || e->nlmso <= 0 || e->nligneso != (e->irregular ? e->nligne : e->nligne - e->nlmso))
    return fail(FDMGPU_ERR_ARG, "inconsistent nligne / nlmso / nligneso");
  if ((int64_t)2 * e->nligne > (int64_t)1 << 30) return fail(FDMGPU_ERR_ARG, "nligne too large");
  if (e->lmaxso < 0 || g.nspino * (e->lmaxso + 1) * (e->lmaxso + 1) < e->nlmso ||
      (e->E_comp ? e->nsort_c : e->nsort_r) < g.nsort)
    return fail(FDMGPU_ERR_ARG, "Bessel arrays too small for nlmso");
  if (e->nlmso > g.nso1) return fail(FDMGPU_ERR_ARG, "nlmso exceeds the outer harmonic tables");
  if (e->ispin < 1 || e->nspinp < std::min(e->ispin, g.nspin) || e->nphiato1 < g.nbtm)
    return fail(FDMGPU_ERR_ARG, "phiato too small (nspinp or nphiato1)");
  if (!e->new_ || !e->newinv || !e->lb1 || !e->lb2 || !e->ianew || !e->nlmsa || !e->Vr || !e->phiato ||
      (e->E_comp ? (!e->Bessel || !e->Neuman) : (!e->Besselr || !e->Neumanr)) ||
      ((e->Relativiste || e->Spinorbite) && !e->gradvr))
    return fail(FDMGPU_ERR_ARG, "null array argument");
  if ((e->Relativiste || e->Spinorbite) && e->nicm < g.npoint) return fail(FDMGPU_ERR_ARG, "gradvr too small (nicm)");
  for (int Lm = 1; Lm <= e->nlmso; ++Lm)
    if (F2(g.lso, g.nso1, Lm, 1) > e->lmaxso) return fail(FDMGPU_ERR_ARG, "outer harmonic above lmaxso");
  return FDMGPU_OK;
}

fdmgpu_status check_energy(const fdmgpu_handle* h, const fdmgpu_energy* e) {
  if (!e) return fail(FDMGPU_ERR_ARG, "null energy arguments");
  if (e->Cal_comp) return check_energy_c(h, e);
  if (e->Cal_comp || e->E_comp || e->Spinorbite || e->Relativiste || e->Repres_comp || e->Ylm_comp || e->irregular ||
      e->Base_hexa || e->n_RI != 1 || e->n_ato_RI != 1 || e->nphiato7 != 1 || h->g.nspino != 1 || !e->Basereel)
    return fail(FDMGPU_ERR_UNSUPPORTED,
                "the library provides the real-arithmetic regular solution (Cal_comp = E_comp = Spinorbite = "
                "Relativiste = irregular = false, Basereel = true, nspino = 1)");
  if (e->nligne <= 0 || e->nlmso <= 0 || e->nligneso != e->nligne - e->nlmso)
    return fail(FDMGPU_ERR_ARG, "inconsistent nligne / nlmso / nligneso");
  if (e->lmaxso < 0 || (e->lmaxso + 1) * (e->lmaxso + 1) < e->nlmso || e->nsort_r < h->g.nsort)
    return fail(FDMGPU_ERR_ARG, "Bessel arrays too small for nlmso");
  if (e->nlmso > h->g.nso1) return fail(FDMGPU_ERR_ARG, "nlmso exceeds the outer harmonic tables");
  const bool gen = !e->phiato && !e->Besselr && !e->Neumanr;
  if (gen && !h->has_radial)
    return fail(FDMGPU_ERR_ARG, "phiato / Besselr / Neumanr are NULL but the grid has no radial tables "
                                "(fdmgpu_set_radial)");
  if (e->ispin < 1 || (!gen && e->nspinp < std::min(e->ispin, h->g.nspin)))
    return fail(FDMGPU_ERR_ARG, "phiato must hold spin block min(ispin, nspin) (nspinp too small)");
  if (!e->new_ || !e->newinv || !e->lb1 || !e->lb2 || !e->ianew || !e->nlmsa || !e->Vr ||
      (!gen && (!e->phiato || !e->Besselr || !e->Neumanr)))
    return fail(FDMGPU_ERR_ARG, "null array argument");
  if (gen) {
    // the generated phiato holds the atoms' harmonics up to their type's cut-off
    for (int ia = 0; ia < h->g.natome; ++ia) {
      const int l = (int)std::lround(std::sqrt((double)e->nlmsa[ia])) - 1;
      if ((l + 1) * (l + 1) != e->nlmsa[ia] || e->nlmsa[ia] > e->nlmagm)
        return fail(FDMGPU_ERR_ARG, "nlmsa must be (lmax + 1)^2 <= nlmagm with generated inputs");
    }
    if (e->Enervide - h->rad_v0bd - h->rad_dv_max <= 0.0)
      return fail(FDMGPU_ERR_ARG, "generated inputs need a positive kinetic energy");
  }
  return FDMGPU_OK;
}

// Band tile plan of one problem from newind's lb1/lb2.
fdmgpu_status plan_problem(fdmgpu_handle* h, const fdmgpu_energy* e, HostProb& hp) {
  // a complex problem is planned as its real-equivalent system: complex row ii
  // becomes rows 2ii-1 and 2ii, each spanning the columns 2 lb1 - 1 .. 2 lb2
  const bool cplx = e->Cal_comp != 0;
  const int n = cplx ? 2 * e->nligne : e->nligne;
  auto lb1 = [&](int ii) { return cplx ? 2 * e->lb1[(ii + 1) / 2 - 1] - 1 : e->lb1[ii - 1]; };
  auto lb2 = [&](int ii) { return cplx ? 2 * e->lb2[(ii + 1) / 2 - 1] : e->lb2[ii - 1]; };
  const int nt = (n + TS - 1) / TS;
  const int npad = nt * TS;
  std::vector<int> fl(npad), lu(npad);
  for (int p = 0; p < npad; ++p) {
    if (p < n) {
      const int ii = n - p;
      const int l1 = lb1(ii), l2 = lb2(ii);
      if (l1 < 1 || l2 > n || l1 > ii || l2 < ii) return fail(FDMGPU_ERR_ARG, "lb1/lb2 do not bracket the diagonal");
      fl[p] = n - l2;
      lu[p] = n - l1;
    } else {
      fl[p] = lu[p] = p;
    }
    if (p > 0 && lu[p] < lu[p - 1]) return fail(FDMGPU_ERR_ARG, "lb1 is not monotone");
  }
  hp.J0.assign(nt + 1, 0);
  hp.J1.assign(nt + 1, 0);
  hp.Imax.assign(nt + 1, 0);
  hp.Imin.assign(nt + 1, 0);
  hp.strip.assign(nt + 1, 0);
  for (int I = 0; I < nt; ++I) {
    int a = npad, b = 0;
    for (int p = I * TS; p < (I + 1) * TS; ++p) {
      a = std::min(a, fl[p]);
      b = std::max(b, lu[p]);
    }
    hp.J0[I] = a / TS;
    hp.J1[I] = b / TS;
  }
  for (int I = nt - 2; I >= 0; --I) hp.J0[I] = std::min(hp.J0[I], hp.J0[I + 1]);
  for (int I = 1; I < nt; ++I) hp.J1[I] = std::max(hp.J1[I], hp.J1[I - 1]);
  int64_t off = 0;
  for (int I = 0; I < nt; ++I) {
    hp.strip[I] = off;
    off += hp.J1[I] - hp.J0[I] + 1;
  }
  hp.strip[nt] = off;
  hp.ntiles = off;
  // tile rows holding atom-harmonic rows (newind marks them with -ia)
  hp.wide.assign(nt + 1, 0);
  for (int p = 0; p < n; ++p) {
    const int ii = n - p;
    const int ic = cplx ? (ii + 1) / 2 : ii;
    if (e->newinv[ic - 1] < 0) hp.wide[p / TS] = 1;
  }
  for (int K = 0; K < nt; ++K) {
    int im = K;
    while (im + 1 < nt && hp.J0[im + 1] <= K) ++im;
    hp.Imax[K] = im;
    int mn = K;
    while (mn - 1 >= 0 && hp.J1[mn - 1] >= K) --mn;
    hp.Imin[K] = mn;
  }
  // algorithmic work of the profile: sum_k 2 l_k u_k and the two solves
  std::vector<int64_t> cnt(npad + 1, 0);
  for (int p = 0; p < n; ++p) cnt[fl[p]]++;
  int64_t cum = 0, nnzL = 0, nnzU = 0;
  double ff = 0;
  for (int k = 0; k < n; ++k) {
    cum += cnt[k];
    const int64_t lk = cum - (k + 1);
    const int64_t uk = lu[k] - k;
    nnzL += lk;
    nnzU += uk;
    ff += 2.0 * (double)lk * (double)uk + (double)lk;
  }
  hp.flops_factor = ff;
  hp.flops_solve = 2.0 * e->nlmso * (double)(nnzL + nnzU + n);
  hp.nnz_profile = nnzL + nnzU + n;
  // CSR capacity: structural nonzeros of calcMatRow (a grid point has nspino
  // rows, each reaching both spin rows of its interstitial neighbours); in the
  // real-equivalent form every complex entry is a 2x2 block
  const fdmgpu_grid& g = h->g;
  const int nso = g.nspino;
  // (the irregular solution: two amplitude columns and rows per atom harmonic)
  const int nato = (cplx && e->irregular) ? 2 : 1;
  int64_t cap = 0;
  for (size_t k = 0; k < h->inter_pt_h.size(); ++k) {
    int64_t row = 1 + (int64_t)nso * h->n_inter_h[k] + (h->has_outer_h[k] ? e->nlmso : 0);
    for (int ia : h->nb_atoms_h[k]) row += (int64_t)nato * e->nlmsa[ia - 1];
    cap += nso * row;
  }
  cap += (int64_t)e->nlmso * (e->nlmso + g.nsortf);
  for (int ia = 1; ia <= g.natome; ++ia)
    cap += (int64_t)nato * e->nlmsa[ia - 1] * (h->nbordf_h[ia - 1] + (int64_t)nato * e->nlmsa[ia - 1]);
  if (cplx) cap *= 4;
  hp.nnz_cap = cap + (npad - n);
  // descriptor (offsets filled later)
  Prob& P = hp.P;
  memset(&P, 0, sizeof(P));
  P.n = n;
  P.nt = nt;
  P.nlmso = e->nlmso;
  P.nrt = (e->nlmso + TS - 1) / TS;
  P.nligneso = e->nligneso;
  P.lmaxso = e->lmaxso;
  P.nlmagm = e->nlmagm;
  P.ispin = e->ispin;
  P.enervide = e->Enervide;
  P.cplx = cplx ? 1 : 0;
  P.ecomp = (cplx && e->E_comp) ? 1 : 0;
  P.eimag = P.ecomp ? e->Eimag : 0.0;
  P.nligne_c = e->nligne;
  P.so = e->Spinorbite ? 1 : 0;
  P.rel = e->Relativiste ? 1 : 0;
  P.ylmc = e->Ylm_comp ? 1 : 0;
  P.nspinp = e->nspinp;
  P.nspinr = std::max(1, e->nspinr);
  P.nspin = g.nspin;
  P.irr = (cplx && e->irregular) ? 1 : 0;
  P.nri = P.irr ? 2 : 1;
  // signature of the plan
  uint64_t s = mix(0, (uint64_t)n);
  s = mix(s, (uint64_t)e->nlmso);
  s = mix(s, (uint64_t)(P.irr * 16 + P.cplx * 8 + P.so * 4 + P.rel * 2 + P.ylmc));
  for (int i = 0; i < e->nligne; i += 7) s = mix(s, (uint64_t)e->lb1[i] * 131 + (uint64_t)e->lb2[i]);
  for (int ia = 0; ia < g.natome; ++ia) s = mix(s, (uint64_t)e->nlmsa[ia] * 1000003u + (uint64_t)e->ianew[ia]);
  hp.sig = s;
  return FDMGPU_OK;
}

// Pack the per-energy inputs (selected spin) into flat host vectors.
void pack_inputs(fdmgpu_handle* h, const fdmgpu_energy* e, HostProb& hp) {
  const fdmgpu_grid& g = h->g;
  hp.in_i.clear();
  hp.in_d.clear();
  // ints: new_(0:npoint), ianew, nlmsa
  hp.in_i.insert(hp.in_i.end(), e->new_, e->new_ + g.npoint + 1);
  hp.in_i.insert(hp.in_i.end(), e->ianew, e->ianew + g.natome);
  hp.in_i.insert(hp.in_i.end(), e->nlmsa, e->nlmsa + g.natome);
  // atom rows per atom: nlmsa, 2 nlmsa for the irregular solution
  hp.nlmsa_max = 0;
  for (int ia = 0; ia < g.natome; ++ia) hp.nlmsa_max = std::max(hp.nlmsa_max, e->nlmsa[ia]);
  if (e->Cal_comp && e->irregular) hp.nlmsa_max *= 2;
  if (e->Cal_comp) {
    // Vr (npoint, nspin) | gradvr (npoint, 3, nspin) | phiato real part, imaginary part
    // (nbtm, nlmagm, nspinp, nspino, nri, natome), nri = 2 (regular, irregular
    // atomic solution) for the irregular solution, else the regular one alone |
    // Bessel, Neumann [nspinr][nsort][lmaxso+1]
    hp.in_d.insert(hp.in_d.end(), e->Vr, e->Vr + (int64_t)g.npoint * g.nspin);
    hp.rel_grad = (int64_t)hp.in_d.size();
    for (int isp = 1; isp <= g.nspin; ++isp)
      for (int k = 1; k <= 3; ++k)
        for (int i = 1; i <= g.npoint; ++i)
          hp.in_d.push_back(e->gradvr ? e->gradvr[(i - 1) + (int64_t)e->nicm * ((k - 1) + 3 * (int64_t)(isp - 1))]
                                      : 0.0);
    hp.rel_phi = (int64_t)hp.in_d.size();
    const int64_t d1 = e->nphiato1, d2 = e->nlmagm, d3 = e->nspinp, d4 = g.nspino, d5 = e->n_RI, d6 = g.natome;
    const int nri = e->irregular ? 2 : 1;
    for (int part = 0; part < 2; ++part)
      for (int ia = 1; ia <= g.natome; ++ia)
        for (int iri = 1; iri <= nri; ++iri)
          for (int isol = 1; isol <= g.nspino; ++isol)
            for (int isp = 1; isp <= e->nspinp; ++isp)
              for (int lm = 1; lm <= e->nlmagm; ++lm) {
                const double* src = e->phiato + d1 * ((lm - 1) + d2 * ((isp - 1) + d3 * ((isol - 1) + d4 * ((iri - 1) +
                                                  d5 * ((ia - 1) + d6 * part)))));
                hp.in_d.insert(hp.in_d.end(), src, src + g.nbtm);
              }
    const int nl = e->lmaxso + 1;
    for (int which = 0; which < 2; ++which) {
      (which == 0 ? hp.rel_bes : hp.rel_neu) = (int64_t)hp.in_d.size();
      if (e->E_comp) {
        // complex (2, nsort_c, 0:lmaxso, nspinr): the real block, then the imaginary block
        const double* a = which == 0 ? e->Bessel : e->Neuman;
        for (int part = 0; part < 2; ++part)
          for (int isp = 1; isp <= std::max(1, e->nspinr); ++isp)
            for (int ib = 0; ib < g.nsort; ++ib)
              for (int L = 0; L < nl; ++L)
                hp.in_d.push_back(a[2 * (ib + (int64_t)e->nsort_c * (L + (int64_t)nl * (isp - 1))) + part]);
      } else {
        const double* a = which == 0 ? e->Besselr : e->Neumanr;
        for (int isp = 1; isp <= std::max(1, e->nspinr); ++isp)
          for (int ib = 0; ib < g.nsort; ++ib)
            for (int L = 0; L < nl; ++L)
              hp.in_d.push_back(a[ib + (int64_t)e->nsort_r * (L + (int64_t)nl * (isp - 1))]);
      }
    }
    return;
  }
  // doubles: Vr(:, ispp)
  const int ispp = std::min(e->ispin, g.nspin);
  hp.in_d.insert(hp.in_d.end(), e->Vr + (int64_t)g.npoint * (ispp - 1), e->Vr + (int64_t)g.npoint * ispp);
  if (!e->phiato) {
    // generated on the device: only their sizes here; upload_inputs places
    // them after every uploaded block
    hp.P.gen = 1;
    for (int t = 0; t < MAX_GEN_TYPES; ++t) hp.P.gen_lmax[t] = -1;
    for (int ia = 0; ia < g.natome; ++ia) {
      const int t = h->rad_itype[ia];
      const int l = (int)std::lround(std::sqrt((double)e->nlmsa[ia])) - 1;
      hp.P.gen_lmax[t] = std::max(hp.P.gen_lmax[t], l);
    }
    hp.gen_phi = (int64_t)g.nbtm * e->nlmagm * g.natome;
    hp.gen_bes = (int64_t)g.nsort * (e->lmaxso + 1);
    hp.rel_grad = g.npoint;
    hp.rel_phi = hp.rel_bes = hp.rel_neu = -1;
    return;
  }
  hp.P.gen = 0;
  // phiato(ib, Lm, isp, isol=1, iRI=1, ia, 1) -> (nbtm, nlmagm, natome)
  const int isp = std::min(e->ispin, g.nspin);  // calcMatRow reads phiato at min(ispin, nspin)
  const int64_t d1 = e->nphiato1, d2 = e->nlmagm, d3 = e->nspinp, d4 = g.nspino, d5 = e->n_RI;
  const size_t base = hp.in_d.size();
  hp.in_d.resize(base + (size_t)g.nbtm * e->nlmagm * g.natome, 0.0);
  const int nb = std::min<int>(e->nphiato1, g.nbtm);
  for (int ia = 1; ia <= g.natome; ++ia)
    for (int lm = 1; lm <= e->nlmagm; ++lm) {
      const double* src = e->phiato + d1 * ((lm - 1) + d2 * ((isp - 1) + d3 * (0 + d4 * (0 + d5 * (int64_t)(ia - 1)))));
      double* dst = hp.in_d.data() + base + (size_t)g.nbtm * ((lm - 1) + (size_t)e->nlmagm * (ia - 1));
      memcpy(dst, src, sizeof(double) * nb);
    }
  // Bessel / Neumann (nsort_r, 0:lmaxso, ispq = 1) -> [ib][L]
  const int nl = e->lmaxso + 1;
  hp.rel_grad = g.npoint;
  hp.rel_phi = g.npoint;
  for (int which = 0; which < 2; ++which) {
    const double* a = which == 0 ? e->Besselr : e->Neumanr;
    const size_t b0 = hp.in_d.size();
    (which == 0 ? hp.rel_bes : hp.rel_neu) = (int64_t)b0;
    hp.in_d.resize(b0 + (size_t)g.nsort * nl);
    for (int ib = 0; ib < g.nsort; ++ib)
      for (int L = 0; L < nl; ++L) hp.in_d[b0 + (size_t)ib * nl + L] = a[ib + (int64_t)e->nsort_r * L];
  }
}

void build_step_plan(fdmgpu_handle* h) {
  StepPlan& sp = h->sp;
  auto& pr = h->batch.probs;
  sp.ntmax = 0;
  sp.nrtmax = 0;
  for (auto& hp : pr) {
    sp.ntmax = std::max(sp.ntmax, hp.P.nt);
    sp.nrtmax = std::max(sp.nrtmax, hp.P.nrt);
  }
  const int N = sp.ntmax;
  sp.panel.assign(N, 0);
  sp.panel_rhs.assign(N, 0);
  sp.trail.assign(N, 0);
  sp.trail_rhs.assign(N, 0);
  sp.fwd.assign(N, 0);
  sp.bwd.assign(N, 0);
  sp.tfwd.assign(N, 0);
  sp.tbwd.assign(N, 0);
  sp.wide_any.assign(N, 0);
  if (h->tb.wide)
    for (auto& hp : pr)
      for (int K = 0; K < hp.P.nt; ++K) sp.wide_any[K] |= (h->factor_mode == FDMGPU_FACTOR_WIDE_ALL) ? 1 : hp.wide[K];
  sp.trail_tc.assign(N, 0);
  sp.fwd_tc.assign(N, 0);
  sp.bwd_tc.assign(N, 0);
  sp.oz_nI.assign(N, 0);
  sp.oz_nC.assign(N, 0);
  sp.oz_items.assign(N, 0);
  sp.oz_capI = sp.oz_capC = 0;
  sp.strip_trail.assign(N, 0);
  sp.strip_trail_rhs.assign(N, 0);
  sp.strip_fwd.assign(N, 0);
  sp.strip_bwd.assign(N, 0);
  sp.strip_panel_l.assign(N, 0);
  sp.strip_panel_u.assign(N, 0);
  sp.strip_panel_u_rhs.assign(N, 0);
  for (auto& hp : pr) {
    for (int K = 0; K < hp.P.nt; ++K) {
      const int nI = hp.Imax[K] - K, nJ = hp.J1[K] - K, nR = hp.P.nrt;
      sp.trail_tc[K] = std::max(sp.trail_tc[K], tc_items(nI, nJ + nR));
      sp.oz_nI[K] = std::max(sp.oz_nI[K], nI);
      sp.oz_nC[K] = std::max(sp.oz_nC[K], nJ + nR);
      sp.oz_items[K] = std::max(sp.oz_items[K], nI > 0 ? ((nI + 1) / 2) * (nJ + nR) : 0);
      sp.oz_capI = std::max(sp.oz_capI, nI);
      sp.oz_capC = std::max(sp.oz_capC, nJ + nR);
      sp.strip_trail[K] = std::max(sp.strip_trail[K], strip_items(nI, nJ, strip_rows(0)));
      sp.strip_trail_rhs[K] = std::max(sp.strip_trail_rhs[K], strip_items(nI, nJ + nR, strip_rows(0)));
      sp.strip_fwd[K] = std::max(sp.strip_fwd[K], strip_items(nI, nR, strip_rows(1)));
      sp.strip_bwd[K] = std::max(sp.strip_bwd[K], strip_items(K - hp.Imin[K], nR, strip_rows(2)));
      sp.strip_panel_l[K] = std::max(sp.strip_panel_l[K], strip_items(nI, 1, strip_rows(0)));
      sp.strip_panel_u[K] = std::max(sp.strip_panel_u[K], strip_items(nJ, 1, strip_rows(0)));
      sp.strip_panel_u_rhs[K] = std::max(sp.strip_panel_u_rhs[K], strip_items(nJ + nR, 1, strip_rows(0)));
      sp.fwd_tc[K] = std::max(sp.fwd_tc[K], tc_items(nI, nR));
      sp.bwd_tc[K] = std::max(sp.bwd_tc[K], tc_items(K - hp.Imin[K], nR));
      sp.panel[K] = std::max(sp.panel[K], nI + nJ);
      sp.panel_rhs[K] = std::max(sp.panel_rhs[K], nI + nJ + nR);
      sp.trail[K] = std::max(sp.trail[K], nI * nJ);
      sp.trail_rhs[K] = std::max(sp.trail_rhs[K], nI * (nJ + nR));
      sp.fwd[K] = std::max(sp.fwd[K], nI * nR);
      sp.bwd[K] = std::max(sp.bwd[K], (K - hp.Imin[K]) * nR);
      sp.tfwd[K] = std::max(sp.tfwd[K], nJ * nR);
      sp.tbwd[K] = std::max(sp.tbwd[K], (K - hp.J0[K]) * nR);
    }
  }
}

// Pool offsets of every problem and the launch dimensions of the batch.
// Runs on every batch (the descriptors are rebuilt by fdmgpu_batch_add);
// allocate_and_upload_plan() below runs only when the plan changes.
struct Layout {
  int64_t env = 0, rhs = 0, rowv = 0, csr = 0, taull = 0, scratch = 0;
  std::vector<int> J0, J1, Imax, Imin;
  std::vector<unsigned char> wide;
  std::vector<int64_t> strip;
};

void layout_batch(fdmgpu_handle* h, Layout& L) {
  auto& pr = h->batch.probs;
  const int np = (int)pr.size();
  const bool mixed = h->batch.precision == FDMGPU_PREC_MIXED;
  int64_t& env = L.env; int64_t& rhs = L.rhs; int64_t& rowv = L.rowv;
  int64_t& csr = L.csr; int64_t& taull = L.taull; int64_t& scratch = L.scratch;
  int trow = 0;
  LaunchDims& d = h->dims;
  d = LaunchDims();
  d.nprob = np;
  h->ncols_tmp = 0;
  for (auto* sh : h->batch.sites) {
    d.npr = std::max(d.npr, sh->S.npr);
    d.max_nsortf = std::max(d.max_nsortf, sh->S.nsortf);
    d.max_natome = std::max(d.max_natome, sh->S.natome);
  }
  std::vector<int>& J0 = L.J0; std::vector<int>& J1 = L.J1;
  std::vector<int>& Imax = L.Imax; std::vector<int>& Imin = L.Imin;
  std::vector<int64_t>& strip = L.strip;
  for (auto& hp : pr) {
    Prob& P = hp.P;
    P.trow = trow;
    P.env = env * TS2;
    P.rhs = rhs;
    P.rowv = rowv;
    P.csr = csr;
    P.csr_cap = mixed ? hp.nnz_cap : 0;
    P.csr_col = h->ncols_tmp;
    h->ncols_tmp += (int64_t)P.nrt * TS;
    P.taull = taull;
    P.scratch = scratch;
    trow += P.nt + 1;
    env += hp.ntiles;
    rhs += (int64_t)P.nt * P.nrt * TS2;
    rowv += (int64_t)P.nt * TS + 1;
    csr += mixed ? hp.nnz_cap : 0;
    taull += (int64_t)P.nlm_abs * P.nlm_abs;
    scratch += (int64_t)P.nlmso * (P.nlmso + 2 * P.nlm_abs);  // N | Xa, then the adjoint's Q
    J0.insert(J0.end(), hp.J0.begin(), hp.J0.end());
    J1.insert(J1.end(), hp.J1.begin(), hp.J1.end());
    Imax.insert(Imax.end(), hp.Imax.begin(), hp.Imax.end());
    Imin.insert(Imin.end(), hp.Imin.begin(), hp.Imin.end());
    strip.insert(strip.end(), hp.strip.begin(), hp.strip.end());
    if (h->factor_mode == FDMGPU_FACTOR_WIDE_ALL)
      L.wide.insert(L.wide.end(), hp.wide.size(), (unsigned char)1);
    else
      L.wide.insert(L.wide.end(), hp.wide.begin(), hp.wide.end());
    d.max_rows = std::max(d.max_rows, P.nt * TS);
    d.max_tiles = std::max<int>(d.max_tiles, (int)hp.ntiles);
    d.max_rhs_tiles = std::max(d.max_rhs_tiles, P.nt * P.nrt);
    d.max_nlmso = std::max(d.max_nlmso, P.nlmso);
    d.max_atom_rows = std::max(d.max_atom_rows, h->batch.sites[P.site]->g.natome * hp.nlmsa_max);
    d.max_nlmsa = std::max(d.max_nlmsa, hp.nlmsa_max);
  }
  d.rowv_total = rowv;
  h->ncols = h->ncols_tmp;
}

// Allocate the device pools of the batch and upload the plan tables.
fdmgpu_status allocate_and_upload_plan(fdmgpu_handle* h, const Layout& L) {
  const int np = (int)h->batch.probs.size();
  const bool mixed = h->batch.precision == FDMGPU_PREC_MIXED;
  const int64_t env = L.env, rhs = L.rhs, rowv = L.rowv, csr = L.csr, taull = L.taull, scratch = L.scratch;
  const std::vector<int>& J0 = L.J0; const std::vector<int>& J1 = L.J1;
  const std::vector<int>& Imax = L.Imax; const std::vector<int>& Imin = L.Imin;
  const std::vector<int64_t>& strip = L.strip;
  cudaStream_t s = h->stream;
  CK(upload(h->d_J0, J0, s));
  CK(upload(h->d_J1, J1, s));
  CK(upload(h->d_Imax, Imax, s));
  CK(upload(h->d_Imin, Imin, s));
  CK(upload(h->d_strip, strip, s));
  CK(upload(h->d_wide, L.wide, s));
  CK(upload(h->d_wide_all, std::vector<unsigned char>(L.wide.size(), 1), s));
  if (h->d_env64.reserve((size_t)env * TS2) != cudaSuccess || h->d_B64.reserve(rhs) != cudaSuccess ||
      h->d_X64.reserve(rhs) != cudaSuccess || h->d_err.reserve(np) != cudaSuccess ||
      h->d_active.reserve(np) != cudaSuccess || h->d_red.reserve(3 * (size_t)np) != cudaSuccess ||
      h->d_taull.reserve(2 * (size_t)std::max<int64_t>(taull, 1)) != cudaSuccess ||
      h->d_tscratch.reserve(2 * (size_t)std::max<int64_t>(scratch, 1)) != cudaSuccess)
    return fail(FDMGPU_ERR_NOMEM, "device allocation of the batch pools failed");
  const bool cplx = h->batch.cplx == 1;
  if (cplx && h->d_piv.reserve(rowv) != cudaSuccess) return fail(FDMGPU_ERR_NOMEM, "device allocation of the pivots");
  if (mixed) {
    if (h->d_env32.reserve((size_t)env * TS2) != cudaSuccess || h->d_Y32.reserve(rhs) != cudaSuccess ||
        h->d_rs.reserve(rowv) != cudaSuccess || h->d_cs.reserve(rowv) != cudaSuccess ||
        h->d_rowptr.reserve(rowv) != cudaSuccess || h->d_col.reserve(csr) != cudaSuccess ||
        h->d_piv.reserve(rowv) != cudaSuccess || h->d_val2.reserve(csr) != cudaSuccess ||
        h->d_Xs.reserve(rhs) != cudaSuccess || h->d_valS.reserve(csr) != cudaSuccess ||
        h->d_V.reserve((size_t)(h->refine_gmres ? h->gmres_m + 1 : 2) * rhs) != cudaSuccess ||
        h->d_W.reserve(rhs) != cudaSuccess || h->d_R32.reserve(rhs) != cudaSuccess ||
        h->d_act_df.reserve(np) != cudaSuccess || h->d_act_rec.reserve(np) != cudaSuccess ||
        h->d_gstate.reserve(gmres_state_bytes() * (size_t)std::max<int64_t>(h->ncols, 1)) != cudaSuccess ||
        h->d_inner.reserve(np) != cudaSuccess || h->d_jdone.reserve(np) != cudaSuccess ||
        h->d_notconv.reserve(np) != cudaSuccess || h->d_active_gm.reserve(np) != cudaSuccess ||
        h->d_val.reserve(csr) != cudaSuccess)
      return fail(FDMGPU_ERR_NOMEM, "device allocation of the mixed precision pools failed");
  }
  h->tb.J0 = h->d_J0.p;
  h->tb.J1 = h->d_J1.p;
  h->tb.Imax = h->d_Imax.p;
  h->tb.Imin = h->d_Imin.p;
  h->tb.strip = h->d_strip.p;
  h->tb.wide = (mixed && h->factor_mode != FDMGPU_FACTOR_FP32) ? h->d_wide.p : nullptr;
  // real mixed batches may run their FP32 tile updates on the tensor cores
  h->sp.tc = (mixed && !cplx && (h->tile_engine == FDMGPU_ENGINE_TCGEN05 ||
                                  h->tile_engine == FDMGPU_ENGINE_TCGEN05_FACTOR)) ? 1 : 0;
  h->sp.tc_solve = (mixed && !cplx && h->tile_engine == FDMGPU_ENGINE_TCGEN05) ? 1 : 0;
  h->sp.row_solve = (mixed && h->solve_order == FDMGPU_SOLVE_ROWS) ? 1 : 0;
  h->sp.strip = (mixed && !cplx && h->tile_engine == FDMGPU_ENGINE_SIMT_STREAM) ? 1 : 0;
  h->sp.tc_err = h->d_err.p;
  Pools& pl = h->pl;
  pl = Pools();
  pl.env64 = h->d_env64.p;
  pl.B64 = h->d_B64.p;
  pl.X64 = h->d_X64.p;
  pl.err = h->d_err.p;
  pl.active = h->d_active.p;
  pl.dmax = h->d_red.p;
  pl.xmax = h->d_red.p + np;
  pl.amax = h->d_red.p + 2 * np;
  pl.taull = h->d_taull.p;
  pl.tscratch = h->d_tscratch.p;
  if (cplx) pl.piv = h->d_piv.p;
  if (mixed) {
    pl.env32 = h->d_env32.p;
    pl.Y32 = h->d_Y32.p;
    pl.R32 = h->d_R32.p;
    pl.act_df = h->d_act_df.p;
    pl.act_rec = h->d_act_rec.p;
    pl.rs = h->d_rs.p;
    pl.cs = h->d_cs.p;
    pl.rowptr = h->d_rowptr.p;
    pl.piv = h->d_piv.p;
    pl.val2 = h->d_val2.p;
    pl.Xs = h->d_Xs.p;
    pl.valS = h->d_valS.p;
    pl.V = h->d_V.p;
    pl.vstride = rhs;
    pl.W = h->d_W.p;
    pl.gstate = h->d_gstate.p;
    pl.inner_active = h->d_inner.p;
    pl.active_gm = h->d_active_gm.p;
    pl.jdone = h->d_jdone.p;
    pl.notconv = h->d_notconv.p;
    pl.col = h->d_col.p;
    pl.val = h->d_val.p;
  }
  build_step_plan(h);
  h->sp.dfl_inv = nullptr;
  if (h->sp.strip) {
    if (h->d_dfl_inv.reserve((size_t)np * 2 * TS2) != cudaSuccess)
      return fail(FDMGPU_ERR_NOMEM, "inverse scratch of the double-float panel");
    h->sp.dfl_inv = reinterpret_cast<dfl*>(h->d_dfl_inv.p);
  }
  h->sp.oz = 0;
  h->sp.oz_img = nullptr;
  h->sp.oz_exp = nullptr;
  if (mixed && h->df64_engine == FDMGPU_DF64_TCGEN05 && h->sp.oz_capI > 0) {
    const size_t slot = (size_t)(h->sp.oz_capI + h->sp.oz_capC);
    if (h->d_oz_img.reserve((size_t)np * slot * (size_t)oz_tile_bytes()) != cudaSuccess ||
        h->d_oz_exp.reserve((size_t)np * slot * TS) != cudaSuccess)
      return fail(FDMGPU_ERR_NOMEM, "integer-slice scratch of the double-float update");
    h->sp.oz = 1;
    h->sp.oz_img = h->d_oz_img.p;
    h->sp.oz_exp = h->d_oz_exp.p;
  }
  return FDMGPU_OK;
}

// Upload the per-problem inputs and descriptors (every run).
fdmgpu_status upload_inputs(fdmgpu_handle* h) {
  auto& pr = h->batch.probs;
  size_t ni = 0, nd = 0;
  for (auto& hp : pr) {
    const fdmgpu_grid& g = h->batch.sites[hp.P.site]->g;
    hp.P.in_new = ni;
    hp.P.in_ianew = ni + g.npoint + 1;
    hp.P.in_nlmsa = hp.P.in_ianew + g.natome;
    ni += hp.in_i.size();
    hp.P.in_vr = nd;
    hp.P.in_grad = nd + hp.rel_grad;
    hp.P.in_phi = nd + hp.rel_phi;
    hp.P.in_bes = nd + hp.rel_bes;
    hp.P.in_neu = nd + hp.rel_neu;
    nd += hp.in_d.size();
  }
  // device-generated phiato / Bessel / Neumann after the uploaded doubles
  const size_t nd_up = nd;
  GenDims& gd = h->gdims;
  gd = GenDims();
  for (auto& hp : pr) {
    if (!hp.P.gen) continue;
    const fdmgpu_handle* sh = h->batch.sites[hp.P.site];
    hp.P.in_phi = nd;
    hp.P.in_bes = nd + hp.gen_phi;
    hp.P.in_neu = nd + hp.gen_phi + hp.gen_bes;
    nd += hp.gen_phi + 2 * hp.gen_bes;
    ++gd.nprob_gen;
    gd.ntype_max = std::max(gd.ntype_max, sh->rad_ntype);
    for (int t = 0; t < MAX_GEN_TYPES; ++t) gd.lmax1 = std::max(gd.lmax1, hp.P.gen_lmax[t] + 1);
    gd.natome_max = std::max(gd.natome_max, sh->g.natome);
    gd.nsort_max = std::max(gd.nsort_max, sh->g.nsort);
    gd.nr_max = std::max(gd.nr_max, sh->rad_nr_max);
  }
  if (ni > h->h_pinned_i_cap) {
    if (h->h_pinned_i) cudaFreeHost(h->h_pinned_i);
    CK(cudaMallocHost(&h->h_pinned_i, ni * sizeof(int)));
    h->h_pinned_i_cap = ni;
  }
  if (nd_up > h->h_pinned_d_cap) {
    if (h->h_pinned_d) cudaFreeHost(h->h_pinned_d);
    CK(cudaMallocHost(&h->h_pinned_d, nd_up * sizeof(double)));
    h->h_pinned_d_cap = nd_up;
  }
  CK(cudaStreamSynchronize(h->stream));  // the pinned buffers may still feed a previous copy
  size_t oi = 0, od = 0;
  std::vector<Prob> P;
  for (auto& hp : pr) {
    memcpy(h->h_pinned_i + oi, hp.in_i.data(), hp.in_i.size() * sizeof(int));
    memcpy(h->h_pinned_d + od, hp.in_d.data(), hp.in_d.size() * sizeof(double));
    oi += hp.in_i.size();
    od += hp.in_d.size();
    P.push_back(hp.P);
  }
  if (h->d_ipool.reserve(ni) != cudaSuccess || h->d_dpool.reserve(nd) != cudaSuccess)
    return fail(FDMGPU_ERR_NOMEM, "device allocation of the input pools failed");
  CK(cudaMemcpyAsync(h->d_ipool.p, h->h_pinned_i, ni * sizeof(int), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->d_dpool.p, h->h_pinned_d, nd_up * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CK(upload(h->d_probs, P, h->stream));
  std::vector<StaticDev> sites;
  for (auto* sh : h->batch.sites) sites.push_back(sh->S);
  CK(upload(h->d_sites, sites, h->stream));
  std::vector<RadialDev> rads;
  for (auto* sh : h->batch.sites) rads.push_back(sh->rad);
  CK(upload(h->d_rads, rads, h->stream));
  if (gd.nprob_gen > 0 &&
      h->d_radU.reserve((size_t)h->batch.probs.size() * gd.ntype_max * gd.lmax1 * gd.nr_max) != cudaSuccess)
    return fail(FDMGPU_ERR_NOMEM, "radial solution scratch");
  h->pl.ipool = h->d_ipool.p;
  h->pl.dpool = h->d_dpool.p;
  return FDMGPU_OK;
}

// Main sequence in three captured parts, timed by events recorded between
// the graph launches: (1) assemble (+ CSR copy and FP32 conversion when
// mixed), (2) factor with the fused forward substitution, (3) backward
// substitution (+ first update of x when mixed).
void record_asm(fdmgpu_handle* h) {
  cudaStream_t s = h->stream;
  const Pools& pl = h->pl;
  const Prob* probs = h->d_probs.p;
  const int np = h->dims.nprob;
  int64_t env = 0, rhs = 0;
  for (auto& hp : h->batch.probs) {
    env += hp.ntiles * TS2;
    rhs += (int64_t)hp.P.nt * hp.P.nrt * TS2;
  }
  cudaMemsetAsync(pl.env64, 0, env * sizeof(double), s);
  cudaMemsetAsync(pl.B64, 0, rhs * sizeof(double), s);
  cudaMemsetAsync(pl.err, 0, np * sizeof(int), s);
  if (h->batch.cplx == 1) {
    launch_assemble_c(h->d_sites.p, probs, pl, h->tb, h->dims, 0, s);
  } else {
    launch_generate_inputs(probs, h->d_rads.p, h->d_sites.p, h->d_ipool.p, h->dims, h->gdims, h->d_radU.p,
                           h->d_dpool.p, s);
    launch_assemble(h->d_sites.p, probs, pl, h->tb, h->dims, s);
  }
  if (h->batch.precision == FDMGPU_PREC_FP64) {
    cudaMemcpyAsync(pl.X64, pl.B64, rhs * sizeof(double), cudaMemcpyDeviceToDevice, s);
  } else {
    launch_csr(probs, pl, h->tb, h->dims, s);
    launch_equilibrate_convert(probs, pl, h->tb, h->dims, s);
    launch_csr_scale(probs, pl, h->dims, s);
    cudaMemsetAsync(pl.notconv, 0, np * sizeof(int), s);
  }
}

void record_factor_window(fdmgpu_handle* h, int threads, int k_begin, int k_end) {
  cudaStream_t s = h->stream;
  const Pools& pl = h->pl;
  const int np = h->dims.nprob;
  // the real-equivalent form of a complex problem pivots inside the diagonal
  // tiles (the real part of a complex pivot can vanish); real problems keep
  // the reference's elimination order
  if (h->batch.precision == FDMGPU_PREC_FP64)
    launch_factor<double>(h->sp, pl.env64, pl.X64, h->d_probs.p, h->tb, np, 1, nullptr, pl.err, 1e-10,
                          h->batch.cplx == 1 ? pl.piv : nullptr, s, threads, k_begin, k_end);
  else
    launch_factor<float>(h->sp, pl.env32, pl.Y32, h->d_probs.p, h->tb, np, 1, nullptr, pl.err, 1e-30, pl.piv, s,
                         threads, k_begin, k_end);
}

void record_factor(fdmgpu_handle* h) {
  record_factor_window(h, h->trail_threads[h->batch.precision == FDMGPU_PREC_FP64 ? 0 : 1], 0, -1);
}

void record_asm(fdmgpu_handle* h);

// Autotuner: on a new plan, time the trailing update of the factor with 64
// threads per tile pair (8x8 accumulators each) and with 128 (8x4) on eight
// factorisation steps from the middle of the band of this batch, and keep the
// faster.  The trial overwrites the band, which the run assembles again.
fdmgpu_status tune_trailing(fdmgpu_handle* h) {
  const int pi = h->batch.precision == FDMGPU_PREC_FP64 ? 0 : 1;
  const int k0 = h->sp.ntmax / 3, k1 = std::min(h->sp.ntmax, k0 + 8);
  const int variants[2] = {64, 128};
  h->trail_ms[pi][0] = h->trail_ms[pi][1] = 1e30;
  // two rounds in alternating order, minimum kept: the first launch of each
  // kernel carries one-off costs (module loading)
  for (int round = 0; round < 2; ++round)
    for (int v = 0; v < 2; ++v) {
      record_asm(h);
      CK(cudaEventRecord(h->ev[0], h->stream));
      record_factor_window(h, variants[v], k0, k1);
      CK(cudaEventRecord(h->ev[1], h->stream));
      CK(cudaStreamSynchronize(h->stream));
      float t = 0;
      CK(cudaEventElapsedTime(&t, h->ev[0], h->ev[1]));
      h->trail_ms[pi][v] = std::min(h->trail_ms[pi][v], (double)t);
    }
  CK(cudaGetLastError());
  h->trail_threads[pi] = h->trail_ms[pi][1] < h->trail_ms[pi][0] ? 128 : 64;
  return FDMGPU_OK;
}

void record_solve(fdmgpu_handle* h) {
  cudaStream_t s = h->stream;
  const Pools& pl = h->pl;
  const int np = h->dims.nprob;
  if (h->batch.precision == FDMGPU_PREC_FP64) {
    launch_backward<double>(h->sp, pl.env64, pl.X64, h->d_probs.p, h->tb, np, nullptr, s);
  } else {
    launch_backward<float>(h->sp, pl.env32, pl.Y32, h->d_probs.p, h->tb, np, nullptr, s);
    cudaMemsetAsync(pl.dmax, 0, 3 * np * sizeof(unsigned long long), s);
    launch_update_x(h->d_probs.p, pl, h->dims, 1, s);
  }
}

// One refinement step in two graphs: the residual, then the correction (so
// that the first residual of a run can be timed on its own).
void record_residual(fdmgpu_handle* h) {
  cudaStream_t s = h->stream;
  const Pools& pl = h->pl;
  cudaMemsetAsync(pl.dmax, 0, 3 * h->dims.nprob * sizeof(unsigned long long), s);
  if (h->refine_recur) {
    // true residual where act_df is set (then restart the recurrence from it),
    // the recurrence residual R32 elsewhere
    Pools pd = pl;
    pd.active = pl.act_df;
    launch_residual(h->d_probs.p, pd, h->dims, h->residual_df64, s);
    launch_copy_rhs32(h->d_probs.p, h->dims, pl.Y32, pl.R32, pl.act_df, s);
    launch_copy_rhs32(h->d_probs.p, h->dims, pl.R32, pl.Y32, pl.act_rec, s);
  } else {
    launch_residual(h->d_probs.p, pl, h->dims, h->residual_df64, s);
  }
}

void record_iter(fdmgpu_handle* h) {
  cudaStream_t s = h->stream;
  const Pools& pl = h->pl;
  const Prob* probs = h->d_probs.p;
  const int np = h->dims.nprob;
  if (h->refine_gmres) {
    launch_gmres_cycle(h->sp, probs, pl, h->tb, h->dims, h->gmres_m, 1e-6f, s);
  } else {
    launch_forward<float>(h->sp, pl.env32, pl.Y32, probs, h->tb, np, pl.active, pl.piv, s);
    launch_backward<float>(h->sp, pl.env32, pl.Y32, probs, h->tb, np, pl.active, s);
  }
  launch_update_x(probs, pl, h->dims, 0, s);
  if (h->refine_recur) launch_resid_update(probs, pl, h->dims, s);
}

size_t count_kernel_nodes(cudaGraph_t graph) {
  size_t nn = 0;
  if (cudaGraphGetNodes(graph, nullptr, &nn) != cudaSuccess) return 0;
  std::vector<cudaGraphNode_t> nodes(nn);
  if (nn && cudaGraphGetNodes(graph, nodes.data(), &nn) != cudaSuccess) return 0;
  size_t nk = 0;
  for (auto nd : nodes) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++nk;
  }
  return nk;
}

// The refinement loop as one graph: the stopping rule of the first step (whose
// residual and solves the caller launches, so the first residual can be timed)
// followed by a while node whose body is one more step plus its stopping rule.
fdmgpu_status capture_refine_loop(fdmgpu_handle* h) {
  if (h->g_loop) {
    cudaGraphExecDestroy(h->g_loop);
    h->g_loop = nullptr;
  }
  const int np = h->dims.nprob;
  cudaGraph_t g = nullptr;
  CK(cudaGraphCreate(&g, 0));
  cudaGraphConditionalHandle cond;
  fdmgpu_status st = FDMGPU_OK;
  cudaError_t e = cudaGraphConditionalHandleCreate(&cond, g, 0, 0);
  cudaGraphNode_t first = nullptr, loop = nullptr;
  size_t nn = 1;
  cudaGraphNodeParams cp = {};
  if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(h->stream, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    launch_refine_check(h->d_rstate.p, h->d_active.p, h->pl, h->d_rctl.p, np, cond, 1, h->stream);
    e = cudaStreamEndCapture(h->stream, &g);
  }
  if (e == cudaSuccess) e = cudaGraphGetNodes(g, &first, &nn);
  if (e == cudaSuccess) {
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = cond;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    e = cudaGraphAddNode(&loop, g, &first, nullptr, 1, &cp);
  }
  if (e == cudaSuccess) {
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    e = cudaStreamBeginCaptureToGraph(h->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      record_residual(h);
      record_iter(h);
      launch_refine_check(h->d_rstate.p, h->d_active.p, h->pl, h->d_rctl.p, np, cond, 1, h->stream);
      e = cudaStreamEndCapture(h->stream, &body);
    }
    if (e == cudaSuccess) h->nk_loop_body = (int64_t)count_kernel_nodes(body);
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&h->g_loop, g, 0);
  if (e != cudaSuccess) st = fail(FDMGPU_ERR_CUDA, std::string("refinement loop graph: ") + cudaGetErrorString(e));
  cudaGraphDestroy(g);
  return st;
}

fdmgpu_status capture(fdmgpu_handle* h, void (*rec)(fdmgpu_handle*), cudaGraphExec_t* out, int64_t* nkernels) {
  if (*out) {
    cudaGraphExecDestroy(*out);
    *out = nullptr;
  }
  cudaGraph_t graph;
  CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  rec(h);
  CK(cudaStreamEndCapture(h->stream, &graph));
  size_t nn = 0;
  CK(cudaGraphGetNodes(graph, nullptr, &nn));
  std::vector<cudaGraphNode_t> nodes(nn);
  if (nn) CK(cudaGraphGetNodes(graph, nodes.data(), &nn));
  int64_t nk = 0;
  for (auto nd : nodes) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++nk;
  }
  *nkernels = nk;
  cudaError_t e = cudaGraphInstantiate(out, graph, 0);
  cudaGraphDestroy(graph);
  CK(e);
  return FDMGPU_OK;
}

// Last resort of the mixed path for real batches: the listed problems (whose
// FP64 bands the double-float escalation has overwritten) are assembled again
// in FP64 and solved by the FP64 elimination, as the FP64 path solves them;
// one grid row per listed problem.  Returns the launches.
int64_t solve_fp64_subset(fdmgpu_handle* h, const std::vector<int>& list) {
  cudaStream_t s = h->stream;
  Batch& b = h->batch;
  const int ne = (int)list.size();
  if (ne == 0) return 0;
  if (h->d_esc_list.reserve(ne) != cudaSuccess || h->d_err_esc.reserve(ne) != cudaSuccess ||
      h->d_probs_esc.reserve(ne) != cudaSuccess)
    return -1;
  for (int k : list) {
    const HostProb& hp = b.probs[k];
    cudaMemsetAsync(h->pl.env64 + hp.P.env, 0, (size_t)hp.ntiles * TS2 * sizeof(double), s);
    cudaMemsetAsync(h->pl.B64 + hp.P.rhs, 0, (size_t)hp.P.nt * hp.P.nrt * TS2 * sizeof(double), s);
  }
  cudaMemcpyAsync(h->d_esc_list.p, list.data(), ne * sizeof(int), cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(h->d_err_esc.p, 0, ne * sizeof(int), s);
  launch_gather_probs(h->d_probs.p, h->d_esc_list.p, ne, h->d_probs_esc.p, s);
  Pools pf = h->pl;
  pf.err = h->d_err_esc.p;
  pf.active = nullptr;
  LaunchDims df = h->dims;
  df.nprob = ne;
  launch_assemble(h->d_sites.p, h->d_probs_esc.p, pf, h->tb, df, s);
  launch_copy_rhs(h->d_probs_esc.p, pf, df, s);
  int64_t nk = 8;
  nk += launch_factor<double>(h->sp, h->pl.env64, h->pl.X64, h->d_probs_esc.p, h->tb, ne, 1, nullptr,
                              h->d_err_esc.p, 1e-10, nullptr, s);
  nk += launch_backward<double>(h->sp, h->pl.env64, h->pl.X64, h->d_probs_esc.p, h->tb, ne, nullptr, s);
  launch_scatter_err(h->d_esc_list.p, ne, h->d_err_esc.p, h->pl.err, s);
  cudaStreamSynchronize(s);  // the host list lives until here
  return nk;
}

fdmgpu_status run_batch(fdmgpu_handle* h, fdmgpu_info* info, bool resident) {
  Batch& b = h->batch;
  const int np = (int)b.probs.size();
  if (np == 0) return fail(FDMGPU_ERR_ARG, "empty batch");
  uint64_t sig = mix(0, (uint64_t)np);
  for (auto& hp : b.probs) sig = mix(sig, hp.sig);
  // the launch dimensions depend on the sites' grids
  for (auto* sh : b.sites) {
    sig = mix(sig, (uint64_t)(uintptr_t)sh);
    sig = mix(sig, ((uint64_t)sh->S.npr << 32) ^ ((uint64_t)sh->S.nsortf << 16) ^ (uint64_t)sh->S.natome);
  }
  fdmgpu_status st;
  cudaGetLastError();  // clear a stale error of an earlier call on this thread
  sig = mix(sig, (uint64_t)h->residual_df64);
  sig = mix(sig, (uint64_t)(h->refine_gmres * 1000 + h->gmres_m));
  sig = mix(sig, (uint64_t)h->factor_mode + 77u);
  sig = mix(sig, (uint64_t)h->tile_engine + 191u);
  sig = mix(sig, (uint64_t)h->solve_order + 733u);
  sig = mix(sig, (uint64_t)h->df64_engine + 919u);
  for (auto& hp : b.probs) {
    sig = mix(sig, (uint64_t)hp.P.gen * 31u);
    if (hp.P.gen)
      for (int t = 0; t < MAX_GEN_TYPES; ++t) sig = mix(sig, (uint64_t)(hp.P.gen_lmax[t] + 2) * 7u + t);
  }
  const bool replan = sig != h->plan_sig || b.precision != h->plan_prec || !h->g_asm;
  Layout lay;
  layout_batch(h, lay);
  if (replan) {
    st = allocate_and_upload_plan(h, lay);
    if (st) return st;
  }
  if (resident) {
    if (replan || !b.ran) return fail(FDMGPU_ERR_ARG, "rerun needs an unchanged batch that has run once");
  } else {
    st = upload_inputs(h);
    if (st) return st;
  }
  // the graphs hold device pointers: capture again whenever one moved
  uint64_t ps = 0;
  const void* ptrs[] = {h->d_probs.p, h->d_ipool.p, h->d_dpool.p, h->d_env64.p, h->d_env32.p, h->d_B64.p,
                        h->d_X64.p,   h->d_Y32.p,   h->d_rs.p,    h->d_cs.p,    h->d_rowptr.p, h->d_col.p,
                        h->d_val.p,   h->d_err.p,   h->d_active.p, h->d_red.p,  h->d_J0.p,   h->d_strip.p,
                        h->d_piv.p,   h->d_val2.p,  h->d_Xs.p,    h->d_valS.p,  h->d_V.p,    h->d_W.p,
                        h->d_gstate.p, h->d_inner.p, h->d_jdone.p, h->d_notconv.p, h->d_active_gm.p,
                        h->d_nb_coef.p, h->d_rvol.p, h->d_poidsa.p, h->d_poidso.p, h->d_Kar.p, h->d_YsoT.p,
                        h->d_Ylmato.p, h->d_R32.p, h->d_act_df.p, h->d_act_rec.p, h->d_sites.p, h->d_wide.p,
                        h->d_rads.p,  h->d_radU.p,  h->d_oz_img.p, h->d_oz_exp.p, h->d_dfl_inv.p};
  for (const void* q : ptrs) ps = mix(ps, (uint64_t)(uintptr_t)q);
  if (replan && h->autotune) {
    st = tune_trailing(h);
    if (st) return st;
  }
  if (replan || ps != h->ptr_sig) {
    h->ptr_sig = ps;
    st = capture(h, record_asm, &h->g_asm, &h->nk_asm);
    if (st) return st;
    st = capture(h, record_factor, &h->g_fac, &h->nk_fac);
    if (st) return st;
    st = capture(h, record_solve, &h->g_sol, &h->nk_sol);
    if (st) return st;
    if (b.precision == FDMGPU_PREC_MIXED) {
      st = capture(h, record_residual, &h->g_res, &h->nk_res);
      if (st) return st;
      st = capture(h, record_iter, &h->g_iter, &h->nk_iter);
      if (st) return st;
      if (h->d_rstate.reserve(np) != cudaSuccess || h->d_rctl.reserve(1) != cudaSuccess)
        return fail(FDMGPU_ERR_NOMEM, "refinement state");
      st = capture_refine_loop(h);
      if (st) return st;
    }
    h->plan_sig = sig;
    h->plan_prec = b.precision;
  }
  CK(cudaEventRecord(h->ev[0], h->stream));
  CK(cudaGraphLaunch(h->g_asm, h->stream));
  CK(cudaEventRecord(h->ev[1], h->stream));
  CK(cudaGraphLaunch(h->g_fac, h->stream));
  CK(cudaEventRecord(h->ev[2], h->stream));
  CK(cudaGraphLaunch(h->g_sol, h->stream));
  CK(cudaEventRecord(h->ev[3], h->stream));
  int64_t nkern = h->nk_asm + h->nk_fac + h->nk_sol;
  b.iters.assign(np, 0);
  b.fallback.assign(np, 0);
  b.wide.assign(np, 0);
  b.res64.assign(np, 0);
  b.inner.assign(np, 0);
  b.resid.assign(np, 0.0);
  b.err.assign(np, 0);
  float ms_refine = 0;
  float wide_ms = 0;
  double wide_flops = 0.0;
  std::vector<int> wide_esc(np, 0);
  bool esc_timed = false;
  double esc_ms_overlap = -1.0, esc_flops_overlap = 0.0;
  if (b.precision == FDMGPU_PREC_MIXED) {
    // Per problem: classical refinement x += LU^-1 r while it contracts (a step
    // counts as slow when the correction does not halve); after two slow steps
    // the problem switches to GMRES-IR cycles (when enabled) or stops; two
    // slow GMRES cycles stop it.  A batched classical step costs a few percent
    // of a re-factorisation per problem, so slow convergence is preferred to
    // escalation.  Stop at max|dx|/max|x| <= tol; problems that stop above
    // tol_accept go to the escalation below (double-float by default).
    const int max_iter = 40;
    const double tol = h->tol > 0 ? h->tol : 1e-10;
    const double tol_accept = h->tol_accept > 0 ? h->tol_accept : (h->residual_df64 ? 1e-7 : 1e-9);
    std::vector<int> active(np, 1), slow(np, 0), gm(np, 0);
    std::vector<double> prev(np, 1e300);
    // recurrence mode: which problems take a true residual next, the last
    // correction measured against a true residual
    std::vector<int> use_df(np, 1), act_df(np, 1), act_rec(np, 0);
    std::vector<double> prev_true(np, 1e300);
    if (h->refine_recur) {
      CK(cudaMemcpyAsync(h->d_act_df.p, act_df.data(), np * sizeof(int), cudaMemcpyHostToDevice, h->stream));
      CK(cudaMemcpyAsync(h->d_act_rec.p, act_rec.data(), np * sizeof(int), cudaMemcpyHostToDevice, h->stream));
    }
    std::vector<unsigned long long> red(3 * np);
    std::vector<int> jd(np, 0);
    // Overlapped escalation: a problem whose refinement stalls above
    // tol_accept is factorised again in double-float arithmetic on stream2
    // at once, while the others keep refining on the main stream.  Each such
    // batch has its own mask; its refinement maxima go to d_red_esc (zeroed
    // once per run: every problem escalates at most once), the initial
    // solve's to d_red_tmp.
    const bool overlap = h->overlap_escalation && h->escalate_dfl && !h->refine_gmres && !h->refine_recur;
    std::vector<int> escalated(np, 0);
    int n_esc_batches = 0;
    double esc_flops_timed = 0.0;
    auto escalate_now = [&](const std::vector<int>& which) -> fdmgpu_status {
      // one pinned + device mask slot per batch, so that the upload does not
      // wait for the previous batch; from the 16th batch on, slot 15 is
      // reused after stream2 has drained
      const int slot = std::min(n_esc_batches, 15);
      if (n_esc_batches >= 15) CK(cudaStreamSynchronize(h->stream2));
      int* hmask = h->h_esc_mask + (size_t)np * slot;
      int* mask = h->d_esc_mask.p + (size_t)np * slot;
      std::copy(which.begin(), which.end(), hmask);
      CK(cudaEventRecord(h->ev_join, h->stream));
      CK(cudaStreamWaitEvent(h->stream2, h->ev_join, 0));
      CK(cudaMemcpyAsync(mask, hmask, np * sizeof(int), cudaMemcpyHostToDevice, h->stream2));
      Pools pe = h->pl;
      pe.active = mask;
      pe.dmax = h->d_red_tmp.p;
      pe.xmax = h->d_red_tmp.p + np;
      pe.amax = h->d_red_tmp.p + 2 * np;
      dfl* D = reinterpret_cast<dfl*>(h->pl.V);
      const bool timed = n_esc_batches < 16;
      nkern += launch_dfl_escalation(h->sp, h->d_probs.p, pe, h->tb, h->dims, D, h->stream2,
                                     timed ? h->ev_esc[2 * n_esc_batches] : nullptr,
                                     timed ? h->ev_esc[2 * n_esc_batches + 1] : nullptr);
      pe.dmax = h->d_red_esc.p;
      pe.xmax = h->d_red_esc.p + np;
      pe.amax = h->d_red_esc.p + 2 * np;
      nkern += launch_dfl_refine_step(h->sp, h->d_probs.p, pe, h->tb, h->dims, D, h->stream2);
      for (int k = 0; k < np; ++k)
        if (which[k]) {
          escalated[k] = 1;
          if (timed) esc_flops_timed += b.probs[k].flops_factor;
        }
      ++n_esc_batches;
      return FDMGPU_OK;
    };
    if (overlap) {
      if (h->d_red_esc.reserve(3 * (size_t)np) != cudaSuccess || h->d_red_tmp.reserve(3 * (size_t)np) != cudaSuccess ||
          h->d_esc_mask.reserve(16 * (size_t)np) != cudaSuccess)
        return fail(FDMGPU_ERR_NOMEM, "escalation buffers");
      if (h->h_esc_mask_cap < 16 * (size_t)np) {
        CK(cudaStreamSynchronize(h->stream2));
        if (h->h_esc_mask) cudaFreeHost(h->h_esc_mask);
        h->h_esc_mask = nullptr;
        CK(cudaMallocHost(&h->h_esc_mask, 16 * (size_t)np * sizeof(int)));
        h->h_esc_mask_cap = 16 * (size_t)np;
      }
      CK(cudaMemsetAsync(h->d_red_esc.p, 0, 3 * np * sizeof(unsigned long long), h->stream));
    }
    CK(cudaMemcpyAsync(h->d_active.p, active.data(), np * sizeof(int), cudaMemcpyHostToDevice, h->stream));
    if (h->refine_gmres)
      CK(cudaMemsetAsync(h->d_active_gm.p, 0, np * sizeof(int), h->stream));
    CK(cudaEventRecord(h->ev[4], h->stream));
    // Classical refinement: the whole loop runs on the device (one graph with
    // a while node, k_refine_check deciding after every step); the host reads
    // the per-problem outcome once at the end.
    const bool dev_loop = !h->refine_gmres && !h->refine_recur && !overlap;
    if (dev_loop) {
      const RefineCtl c0{0, max_iter, tol, np, 0};
      CK(cudaMemcpyAsync(h->d_rctl.p, &c0, sizeof c0, cudaMemcpyHostToDevice, h->stream));
      launch_refine_init(h->d_rstate.p, h->d_active.p, np, h->stream);
      CK(cudaEventRecord(h->ev[6], h->stream));
      CK(cudaGraphLaunch(h->g_res, h->stream));
      CK(cudaEventRecord(h->ev[7], h->stream));
      CK(cudaGraphLaunch(h->g_iter, h->stream));
      CK(cudaGraphLaunch(h->g_loop, h->stream));
      std::vector<RefineState> rs(np);
      RefineCtl c1;
      CK(cudaMemcpyAsync(rs.data(), h->d_rstate.p, np * sizeof(RefineState), cudaMemcpyDeviceToHost, h->stream));
      CK(cudaMemcpyAsync(&c1, h->d_rctl.p, sizeof c1, cudaMemcpyDeviceToHost, h->stream));
      CK(cudaStreamSynchronize(h->stream));
      nkern += 2 + h->nk_res + h->nk_iter + (int64_t)std::max(c1.it - 1, 0) * h->nk_loop_body;
      for (int k = 0; k < np; ++k) {
        b.iters[k] = rs[k].iters;
        b.resid[k] = rs[k].resid;
        active[k] = rs[k].active;
      }
    }
    for (int it = 1; it <= max_iter && !dev_loop; ++it) {
      if (it == 1) CK(cudaEventRecord(h->ev[6], h->stream));
      CK(cudaGraphLaunch(h->g_res, h->stream));
      if (it == 1) CK(cudaEventRecord(h->ev[7], h->stream));
      CK(cudaGraphLaunch(h->g_iter, h->stream));
      nkern += h->nk_res + h->nk_iter;
      CK(cudaMemcpyAsync(red.data(), h->d_red.p, 3 * np * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                         h->stream));
      if (h->refine_gmres)
        CK(cudaMemcpyAsync(jd.data(), h->d_jdone.p, np * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
      CK(cudaStreamSynchronize(h->stream));
      int nact = 0;
      bool gm_changed = false;
      for (int k = 0; k < np; ++k) {
        if (!active[k]) continue;
        if (gm[k]) b.inner[k] += jd[k];
        double dm, xm;
        memcpy(&dm, &red[k], 8);
        memcpy(&xm, &red[np + k], 8);
        const double r = xm > 0 ? dm / xm : dm;
        b.iters[k] = it;
        if (h->refine_recur) {
          // Only a step that started from a true residual can accept or stop a
          // problem; recurrence steps that look converged or stall call for one.
          if (use_df[k]) {
            b.resid[k] = r;
            if (!std::isfinite(r) || r <= tol || (prev_true[k] < 1e299 && r > 0.5 * prev_true[k])) {
              active[k] = 0;
            } else {
              prev_true[k] = r;
              use_df[k] = 0;
              slow[k] = 0;
              ++nact;
            }
          } else {
            slow[k] = (r > 0.5 * prev[k]) ? slow[k] + 1 : 0;
            use_df[k] = (!std::isfinite(r) || r <= tol || slow[k] >= 2) ? 1 : 0;
            ++nact;
          }
          prev[k] = r;
          continue;
        }
        b.resid[k] = r;
        if (!std::isfinite(r) || r <= tol) {
          active[k] = 0;
        } else {
          slow[k] = (it > 1 && r > 0.5 * prev[k]) ? slow[k] + 1 : 0;
          if (slow[k] >= 2) {
            if (h->refine_gmres && !gm[k] && r > tol_accept * 1e-2) {
              gm[k] = 1;
              slow[k] = 0;
              gm_changed = true;
              ++nact;
            } else {
              active[k] = 0;
            }
          } else {
            ++nact;
          }
        }
        prev[k] = r;
      }
      if (overlap) {
        std::vector<int> which(np, 0);
        int nw = 0;
        for (int k = 0; k < np; ++k)
          if (!active[k] && !escalated[k] && b.iters[k] == it && !(b.resid[k] <= tol_accept)) {
            which[k] = 1;
            ++nw;
          }
        if (nw) {
          st = escalate_now(which);
          if (st) return st;
        }
      }
      if (nact == 0) break;
      CK(cudaMemcpyAsync(h->d_active.p, active.data(), np * sizeof(int), cudaMemcpyHostToDevice, h->stream));
      if (h->refine_recur) {
        for (int k = 0; k < np; ++k) {
          act_df[k] = active[k] && use_df[k];
          act_rec[k] = active[k] && !use_df[k];
        }
        CK(cudaMemcpyAsync(h->d_act_df.p, act_df.data(), np * sizeof(int), cudaMemcpyHostToDevice, h->stream));
        CK(cudaMemcpyAsync(h->d_act_rec.p, act_rec.data(), np * sizeof(int), cudaMemcpyHostToDevice, h->stream));
        CK(cudaStreamSynchronize(h->stream));  // the host vectors are reused next step
      }
      if (gm_changed || h->refine_gmres) {
        std::vector<int> agm(np);
        for (int k = 0; k < np; ++k) agm[k] = active[k] && gm[k];
        CK(cudaMemcpyAsync(h->d_active_gm.p, agm.data(), np * sizeof(int), cudaMemcpyHostToDevice, h->stream));
        CK(cudaStreamSynchronize(h->stream));
      }
    }
    CK(cudaEventRecord(h->ev[10], h->stream));  // end of the classical refinement loop
    // First escalation stage (FDMGPU_ESCALATE_WIDE_DF64): the stalled
    // problems are factorised again in FP32 with double-float sums in every
    // trailing update (the FP32 band converted again from the FP64 one), and
    // the device refinement loop continues from their current solution.
    int n_wide = 0;
    if (dev_loop && h->escalate_wide) {
      std::vector<RefineState> rs(np);
      for (int k = 0; k < np; ++k) {
        const bool w = !(b.resid[k] <= tol_accept);
        n_wide += w;
        rs[k].active = w ? 1 : 0;
        rs[k].slow = 0;
        rs[k].iters = 0;
        rs[k].pad = 0;
        rs[k].prev = 1e300;
        rs[k].resid = b.resid[k];
        active[k] = w ? 1 : 0;
      }
      if (n_wide > 0) {
        CK(cudaEventRecord(h->ev[8], h->stream));
        CK(cudaMemcpyAsync(h->d_active.p, active.data(), np * sizeof(int), cudaMemcpyHostToDevice, h->stream));
        CK(cudaMemcpyAsync(h->d_rstate.p, rs.data(), np * sizeof(RefineState), cudaMemcpyHostToDevice, h->stream));
        const RefineCtl c0{0, max_iter, tol, n_wide, 0};
        CK(cudaMemcpyAsync(h->d_rctl.p, &c0, sizeof c0, cudaMemcpyHostToDevice, h->stream));
        launch_convert_masked(h->d_probs.p, h->pl, h->tb, h->dims, h->stream);
        Tables tw = h->tb;
        tw.wide = h->d_wide_all.p;
        StepPlan sw = h->sp;
        sw.wide_any.assign(sw.ntmax, 1);
        nkern += 1 + launch_factor<float>(sw, h->pl.env32, h->pl.Y32, h->d_probs.p, tw, np, 0, h->d_active.p,
                                          h->pl.err, 1e-30, h->pl.piv, h->stream,
                                          h->trail_threads[1]);
        CK(cudaEventRecord(h->ev[9], h->stream));
        CK(cudaGraphLaunch(h->g_res, h->stream));
        CK(cudaGraphLaunch(h->g_iter, h->stream));
        CK(cudaGraphLaunch(h->g_loop, h->stream));
        std::vector<RefineState> rs2(np);
        RefineCtl c1;
        CK(cudaMemcpyAsync(rs2.data(), h->d_rstate.p, np * sizeof(RefineState), cudaMemcpyDeviceToHost, h->stream));
        CK(cudaMemcpyAsync(&c1, h->d_rctl.p, sizeof c1, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        CK(cudaGetLastError());
        nkern += h->nk_res + h->nk_iter + 1 + (int64_t)std::max(c1.it - 1, 0) * h->nk_loop_body;
        for (int k = 0; k < np; ++k)
          if (rs[k].active) {
            b.iters[k] += rs2[k].iters;
            b.resid[k] = rs2[k].resid;
            wide_esc[k] = 1;
          }
        float t = 0;
        CK(cudaEventElapsedTime(&t, h->ev[8], h->ev[9]));
        wide_ms = t;
        for (int k = 0; k < np; ++k)
          if (rs[k].active) wide_flops += b.probs[k].flops_factor;
      }
    }
    // Precision escalation: problems whose refinement missed tol_accept are
    // factorised again in double-float (or FP64) arithmetic and solved.
    int nfail = 0;
    for (int k = 0; k < np; ++k) {
      active[k] = !(b.resid[k] <= tol_accept);
      nfail += active[k];
    }
    if (overlap) {
      std::vector<int> which(np, 0);
      int nw = 0;
      for (int k = 0; k < np; ++k)
        if (active[k] && !escalated[k]) {
          which[k] = 1;
          ++nw;
        }
      if (nw) {
        st = escalate_now(which);
        if (st) return st;
      }
      if (n_esc_batches > 0) {
        CK(cudaEventRecord(h->ev_join, h->stream2));
        CK(cudaStreamWaitEvent(h->stream, h->ev_join, 0));
        std::vector<unsigned long long> red2(3 * np);
        CK(cudaMemcpyAsync(red2.data(), h->d_red_esc.p, 3 * np * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                           h->stream));
        CK(cudaStreamSynchronize(h->stream));
        std::vector<int> act2(np, 0);
        int more = 0;
        for (int k = 0; k < np; ++k)
          if (escalated[k]) {
            double dm, xm;
            memcpy(&dm, &red2[k], 8);
            memcpy(&xm, &red2[np + k], 8);
            b.resid[k] = xm > 0 ? dm / xm : dm;
            act2[k] = !(b.resid[k] <= tol_accept);
            more += act2[k];
          }
        // rare: further double-float steps on the main stream
        dfl* D = reinterpret_cast<dfl*>(h->pl.V);
        for (int step = 1; step < 3 && more; ++step) {
          CK(cudaMemcpyAsync(h->d_active.p, act2.data(), np * sizeof(int), cudaMemcpyHostToDevice, h->stream));
          CK(cudaMemsetAsync(h->pl.dmax, 0, 3 * np * sizeof(unsigned long long), h->stream));
          nkern += launch_dfl_refine_step(h->sp, h->d_probs.p, h->pl, h->tb, h->dims, D, h->stream);
          CK(cudaMemcpyAsync(red2.data(), h->d_red.p, 3 * np * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                             h->stream));
          CK(cudaStreamSynchronize(h->stream));
          more = 0;
          for (int k = 0; k < np; ++k)
            if (act2[k]) {
              double dm, xm;
              memcpy(&dm, &red2[k], 8);
              memcpy(&xm, &red2[np + k], 8);
              b.resid[k] = xm > 0 ? dm / xm : dm;
              act2[k] = !(b.resid[k] <= tol_accept);
              more += act2[k];
            }
        }
        for (int k = 0; k < np; ++k) b.fallback[k] = escalated[k];
        // the escalation factor time of the timed batches (they overlap the refinement)
        float tsum = 0;
        for (int i = 0; i < std::min(n_esc_batches, 16); ++i) {
          float t = 0;
          CK(cudaEventElapsedTime(&t, h->ev_esc[2 * i], h->ev_esc[2 * i + 1]));
          tsum += t;
        }
        esc_ms_overlap = tsum;
        esc_flops_overlap = esc_flops_timed;
        esc_timed = true;
      }
      nfail = 0;  // handled above
    }
    if (nfail > 0) {
      CK(cudaMemcpyAsync(h->d_active.p, active.data(), np * sizeof(int), cudaMemcpyHostToDevice, h->stream));
      if (h->escalate_dfl) {
        // double-float factorisation of the equilibrated matrix, then
        // double-float refinement steps.  The double-float factors contract
        // the error by orders of magnitude per step, so the solution after a
        // step whose correction is within tol_accept is far more accurate than
        // that correction: stop there (one step is the rule, three at most).
        dfl* D = reinterpret_cast<dfl*>(h->pl.V);
        std::vector<int> act2 = active;
        std::vector<unsigned long long> red2(3 * np);
        int dfl_steps = 3;
        if (h->escalate_f32 && dev_loop) {
          // double-float factors rounded to FP32, then the device FP32
          // refinement loop from the current solution; the energies it leaves
          // above the accepted level take double-float steps below
          // the factor runs over the escalated problems only (one grid row each)
          std::vector<int> list;
          for (int k = 0; k < np; ++k)
            if (active[k]) list.push_back(k);
          const int ne = (int)list.size();
          if (h->d_esc_list.reserve(ne) != cudaSuccess || h->d_err_esc.reserve(ne) != cudaSuccess ||
              h->d_probs_esc.reserve(ne) != cudaSuccess)
            return fail(FDMGPU_ERR_NOMEM, "escalation descriptors");
          CK(cudaMemcpyAsync(h->d_esc_list.p, list.data(), ne * sizeof(int), cudaMemcpyHostToDevice, h->stream));
          CK(cudaMemsetAsync(h->d_err_esc.p, 0, ne * sizeof(int), h->stream));
          launch_gather_probs(h->d_probs.p, h->d_esc_list.p, ne, h->d_probs_esc.p, h->stream);
          Pools pe = h->pl;
          pe.active = nullptr;
          pe.err = h->d_err_esc.p;
          LaunchDims de = h->dims;
          de.nprob = ne;
          // with the strips, the factor keeps every step's U^-1 and the
          // double-float solve multiplies by them (compact problem order)
          if (h->sp.strip && h->sp.dfl_inv &&
              h->d_uinv_keep.reserve((size_t)ne * h->sp.ntmax * TS2) == cudaSuccess)
            h->sp.dfl_uinv_keep = reinterpret_cast<dfl*>(h->d_uinv_keep.p);
          nkern += 2 + launch_dfl_factor_f32(h->sp, h->d_probs_esc.p, pe, h->tb, de, D, h->stream, h->ev[8],
                                             h->ev[9]);
          h->sp.dfl_uinv_keep = nullptr;
          launch_scatter_err(h->d_esc_list.p, ne, h->d_err_esc.p, h->pl.err, h->stream);
          CK(cudaStreamSynchronize(h->stream));  // the host list lives until here
          esc_timed = true;
          std::vector<RefineState> rs(np);
          for (int k = 0; k < np; ++k) {
            rs[k].active = active[k];
            rs[k].slow = 0;
            rs[k].iters = 0;
            rs[k].pad = 0;
            rs[k].prev = 1e300;
            rs[k].resid = b.resid[k];
          }
          CK(cudaMemcpyAsync(h->d_rstate.p, rs.data(), np * sizeof(RefineState), cudaMemcpyHostToDevice, h->stream));
          const RefineCtl c0{0, max_iter, tol, nfail, 0};
          CK(cudaMemcpyAsync(h->d_rctl.p, &c0, sizeof c0, cudaMemcpyHostToDevice, h->stream));
          CK(cudaGraphLaunch(h->g_res, h->stream));
          CK(cudaGraphLaunch(h->g_iter, h->stream));
          CK(cudaGraphLaunch(h->g_loop, h->stream));
          std::vector<RefineState> rs2(np);
          RefineCtl c1;
          CK(cudaMemcpyAsync(rs2.data(), h->d_rstate.p, np * sizeof(RefineState), cudaMemcpyDeviceToHost, h->stream));
          CK(cudaMemcpyAsync(&c1, h->d_rctl.p, sizeof c1, cudaMemcpyDeviceToHost, h->stream));
          CK(cudaStreamSynchronize(h->stream));
          CK(cudaGetLastError());
          nkern += h->nk_res + h->nk_iter + (int64_t)std::max(c1.it - 1, 0) * h->nk_loop_body;
          int more = 0;
          for (int k = 0; k < np; ++k)
            if (active[k]) {
              b.iters[k] += rs2[k].iters;
              b.resid[k] = rs2[k].resid;
              act2[k] = !(b.resid[k] <= tol_accept);
              more += act2[k];
            } else {
              act2[k] = 0;
            }
          if (more) CK(cudaMemcpyAsync(h->d_active.p, act2.data(), np * sizeof(int), cudaMemcpyHostToDevice, h->stream));
          else dfl_steps = 0;
        } else {
          nkern += launch_dfl_escalation(h->sp, h->d_probs.p, h->pl, h->tb, h->dims, D, h->stream, h->ev[8], h->ev[9]);
          esc_timed = true;
        }
        for (int step = 0; step < dfl_steps; ++step) {
          CK(cudaMemsetAsync(h->pl.dmax, 0, 3 * np * sizeof(unsigned long long), h->stream));
          nkern += launch_dfl_refine_step(h->sp, h->d_probs.p, h->pl, h->tb, h->dims, D, h->stream);
          CK(cudaMemcpyAsync(red2.data(), h->d_red.p, 3 * np * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                             h->stream));
          CK(cudaStreamSynchronize(h->stream));
          int more = 0;
          for (int k = 0; k < np; ++k)
            if (act2[k]) {
              double dm, xm;
              memcpy(&dm, &red2[k], 8);
              memcpy(&xm, &red2[np + k], 8);
              b.resid[k] = xm > 0 ? dm / xm : dm;
              act2[k] = !(b.resid[k] <= tol_accept);
              more += act2[k];
            }
          if (!more) break;
          CK(cudaMemcpyAsync(h->d_active.p, act2.data(), np * sizeof(int), cudaMemcpyHostToDevice, h->stream));
        }
        // default escalation: energies still above the accepted level get the
        // FP64 assembly and elimination (FDMGPU_ESCALATE_DF64 reports them)
        std::vector<int> last;
        for (int k = 0; k < np; ++k)
          if (act2[k]) last.push_back(k);
        // (real batches only: a complex energy left above the level is
        // reported not converged with its double-float solution)
        if (h->escalate_f32 && !last.empty() && b.cplx != 1) {
          const int64_t nk64 = solve_fp64_subset(h, last);
          if (nk64 < 0) return fail(FDMGPU_ERR_NOMEM, "FP64 re-solve descriptors");
          CK(cudaGetLastError());
          nkern += nk64;
          for (int k : last) {
            b.resid[k] = 0.0;  // direct FP64 solve, no correction measured
            b.res64[k] = 1;
          }
        }
      } else {
        launch_copy_rhs(h->d_probs.p, h->pl, h->dims, h->stream);
        nkern += 1;
        nkern += launch_factor<double>(h->sp, h->pl.env64, h->pl.X64, h->d_probs.p, h->tb, np, 1,
                                       h->d_active.p, h->pl.err, 1e-10, b.cplx == 1 ? h->pl.piv : nullptr,
                                       h->stream);
        nkern += launch_backward<double>(h->sp, h->pl.env64, h->pl.X64, h->d_probs.p, h->tb, np,
                                         h->d_active.p, h->stream);
      }
      CK(cudaGetLastError());
      for (int k = 0; k < np; ++k) {
        b.fallback[k] = active[k];
        if (active[k] && !h->escalate_dfl) b.resid[k] = 0.0;  // direct FP64 solve, no correction measured
      }
    }
    CK(cudaEventRecord(h->ev[5], h->stream));
    for (int k = 0; k < np; ++k)
      if (!(b.resid[k] <= tol_accept)) b.err[k] = FDMGPU_ERR_NOT_CONVERGED;
    for (int k = 0; k < np; ++k) b.wide[k] = wide_esc[k];
  }
  if (b.probs[0].P.nlm_abs > 0) {
    if (b.cplx == 1) {
      int mx = 0;
      for (auto& hp : b.probs) mx = std::max(mx, hp.P.nlm_abs);
      launch_taull_c(h->d_sites.p, h->d_probs.p, h->pl, h->dims, mx, h->stream);
      nkern += 2;
    } else {
      launch_taull(h->d_probs.p, h->pl, h->dims, h->pl.X64, h->stream);
      nkern += 1;
    }
  }
  std::vector<int> err(np);
  CK(cudaMemcpyAsync(err.data(), h->d_err.p, np * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaGetLastError());
  for (int k = 0; k < np; ++k)
    if (err[k]) b.err[k] = err[k];
  b.ran = true;
  b.lam_valid = false;
  if (info) {
    memset(info, 0, sizeof(*info));
    info->n_kernels = nkern;
    for (auto& hp : b.probs) {
      info->nnz_profile += hp.nnz_profile;
      info->flops_factor += hp.flops_factor;
      info->flops_solve += hp.flops_solve;
    }
    float t = 0;
    CK(cudaEventElapsedTime(&t, h->ev[0], h->ev[1]));
    info->ms_assemble = t;
    CK(cudaEventElapsedTime(&t, h->ev[1], h->ev[2]));
    info->ms_factor = t;
    CK(cudaEventElapsedTime(&t, h->ev[2], h->ev[3]));
    info->ms_solve = t;
    if (b.precision == FDMGPU_PREC_MIXED) {
      CK(cudaEventElapsedTime(&ms_refine, h->ev[4], h->ev[5]));
      info->ms_refine = ms_refine;
      CK(cudaEventElapsedTime(&t, h->ev[6], h->ev[7]));
      info->ms_residual_first = t;
      // algorithmic work of that residual: 2 flops per nonzero per right-hand side
      if (h->d_nnz.reserve(np) != cudaSuccess) return fail(FDMGPU_ERR_NOMEM, "nnz buffer");
      launch_csr_nnz(h->d_probs.p, h->pl.rowptr, h->dims, h->d_nnz.p, h->stream);
      std::vector<int> nnz(np);
      CK(cudaMemcpyAsync(nnz.data(), h->d_nnz.p, np * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
      CK(cudaStreamSynchronize(h->stream));
      for (int k = 0; k < np; ++k) info->flops_residual += 2.0 * nnz[k] * b.probs[k].P.nlmso;
      if (esc_timed && esc_ms_overlap >= 0) {
        info->ms_escalate_factor = esc_ms_overlap;
        info->flops_escalate_factor = esc_flops_overlap;
      } else if (esc_timed) {
        CK(cudaEventElapsedTime(&t, h->ev[8], h->ev[9]));
        info->ms_escalate_factor = t;
        for (int k = 0; k < np; ++k)
          if (b.fallback[k]) info->flops_escalate_factor += b.probs[k].flops_factor;
      }
      int mi = 0;
      double mr = 0;
      for (int k = 0; k < np; ++k) {
        mi = std::max(mi, b.iters[k]);
        mr = std::max(mr, b.resid[k]);
      }
      info->refine_iters = mi;
      info->residual = mr;
      for (int k = 0; k < np; ++k) info->n_fallback += b.fallback[k];
      for (int k = 0; k < np; ++k) info->n_wide_refactor += b.wide[k];
      info->ms_wide_refactor = wide_ms;
      info->flops_wide_refactor = wide_flops;
      CK(cudaEventElapsedTime(&t, h->ev[4], h->ev[10]));
      info->ms_refine_loop = t;
      for (int k = 0; k < np; ++k) info->refine_steps += b.iters[k];
    }
  }
  // hard errors first; a refinement that did not reach its tolerance still
  // leaves a usable solution and is reported per problem (fdmgpu_batch_stats)
  fdmgpu_status worst = FDMGPU_OK;
  for (int k = 0; k < np; ++k)
    if (b.err[k] && (worst == FDMGPU_OK || worst == FDMGPU_ERR_NOT_CONVERGED)) {
      char buf[160];
      snprintf(buf, sizeof buf, "problem %d: status %d (%s)", k, b.err[k],
               b.err[k] == FDMGPU_ERR_NOT_CONVERGED ? "refinement did not converge" : "zero pivot or bad input");
      g_last_error = buf;
      worst = (fdmgpu_status)b.err[k];
    }
  return worst;
}

}  // namespace

extern "C" {

const char* fdmgpu_version(void) { return "fdmgpu 0.1 (sm_103a)"; }

const char* fdmgpu_last_error(void) { return g_last_error.c_str(); }

void fdmgpu_get_solver_params(int32_t* mpi_host_num_for_mumps, char solver[6]) {
  if (mpi_host_num_for_mumps) *mpi_host_num_for_mumps = 1;
  if (solver) memcpy(solver, "GPU  ", 6);
}

fdmgpu_status fdmgpu_create(const fdmgpu_grid* g, fdmgpu_handle** out) {
  if (!g || !out) return fail(FDMGPU_ERR_ARG, "null argument");
  *out = nullptr;
  if ((g->nspino != 1 && g->nspino != 2) || g->ngrph < 1) return fail(FDMGPU_ERR_ARG, "nspino must be 1 or 2");
  if (g->npoint <= 0 || g->npsom < g->npoint || g->nvois <= 0 || g->natome < 0)
    return fail(FDMGPU_ERR_ARG, "inconsistent grid sizes");
  fdmgpu_handle* h = new fdmgpu_handle();
  h->g = *g;
  CK(cudaGetDevice(&h->device));
  CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&h->stream2, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming));
  for (auto& e : h->ev_esc) CK(cudaEventCreate(&e));
  for (auto& e : h->ev) CK(cudaEventCreate(&e));
  // derived neighbour descriptors of the interstitial points
  const int nv = g->nvois;
  std::vector<std::unordered_map<int, int>> atom_ib(g->natome + 1);
  for (int ia = 1; ia <= g->natome; ++ia)
    for (int ib = g->nbordf[ia - 1] + 1; ib <= g->nbord[ia - 1]; ++ib)
      atom_ib[ia][F2(g->ibord, g->nbtm, ib, ia)] = ib;
  std::unordered_map<int, int> outer_ib;
  for (int ib = g->nsortf + 1; ib <= g->nsort; ++ib) outer_ib[g->isrt[ib - 1]] = ib;
  for (int i = 1; i <= g->npoint; ++i) {
    if (g->numia[i - 1] != 0) continue;
    h->inter_pt_h.push_back(i);
    int nint = 0, hout = 0;
    std::vector<int> atoms;
    for (int iv = 1; iv <= nv; ++iv) {
      const int j = F2(g->ivois, g->npsom, i, iv);
      if (j < 1 || j > g->npsom) {
        fdmgpu_destroy(h);
        return fail(FDMGPU_ERR_ARG, "neighbour table points outside the grid");
      }
      const int ia = g->numia[j - 1];
      const double charac = g->Kar[std::abs(F2(g->isvois, g->npsom, i, iv)) - 1];
      double cf = -g->clapl[iv];
      cf = charac * cf;
      cf = cf * g->rvol[i - 1];
      int kind = 0, idx = j;
      if (ia == 0) {
        ++nint;
      } else if (ia > 0) {
        auto it = atom_ib[ia].find(j);
        if (it == atom_ib[ia].end()) {
          fdmgpu_destroy(h);
          return fail(FDMGPU_ERR_ARG, "atom neighbour missing from the interior boundary list");
        }
        idx = it->second;
        const int isym = std::abs(F2(g->isbord, g->nbtm, idx, ia));
        if (isym != 1) cf = g->Kar[isym - 1] * cf;
        kind = ia;
        if (std::find(atoms.begin(), atoms.end(), ia) == atoms.end()) atoms.push_back(ia);
      } else if (ia == -2) {
        auto it = outer_ib.find(j);
        if (it == outer_ib.end()) {
          fdmgpu_destroy(h);
          return fail(FDMGPU_ERR_ARG, "outer neighbour missing from isrt");
        }
        idx = it->second;
        kind = -2;
        hout = 1;
      } else {
        fdmgpu_destroy(h);
        return fail(FDMGPU_ERR_ARG, "unexpected numia value");
      }
      h->nb_kind_h.push_back(kind);
      h->nb_idx_h.push_back(idx);
      h->nb_coef_h.push_back(cf);
    }
    h->n_inter_h.push_back(nint);
    h->has_outer_h.push_back(hout);
    h->nb_atoms_h.push_back(atoms);
  }
  h->nbordf_h.assign(g->nbordf, g->nbordf + g->natome);
  // the complex path folds no characters: every one the grid uses must be 1
  h->chars_c1 = g->ngrph == 1 && g->Kar && g->Kari;
  for (int i = 1; h->chars_c1 && i <= g->npoint; ++i)
    for (int iv = 1; iv <= nv && h->chars_c1; ++iv) {
      const int is = std::abs(F2(g->isvois, g->npsom, i, iv));
      for (int sp = 0; sp < g->nspino; ++sp)
        if (is < 1 || is > 64 || g->Kar[is - 1 + 64 * sp] != 1.0 || g->Kari[is - 1 + 64 * sp] != 0.0) h->chars_c1 = false;
    }
  for (int ia = 1; h->chars_c1 && ia <= g->natome; ++ia)
    for (int ib = 1; ib <= g->nbord[ia - 1] && h->chars_c1; ++ib) {
      const int is = std::abs(F2(g->isbord, g->nbtm, ib, ia));
      for (int sp = 0; sp < g->nspino; ++sp)
        if (is < 1 || is > 64 || g->Kar[is - 1 + 64 * sp] != 1.0 || g->Kari[is - 1 + 64 * sp] != 0.0) h->chars_c1 = false;
    }
  cudaStream_t s = h->stream;
  auto up_i = [&](DevBuf<int>& b, const int32_t* p, size_t n) {
    return upload(b, std::vector<int>(p, p + n), s);
  };
  auto up_d = [&](DevBuf<double>& b, const double* p, size_t n) {
    return upload(b, std::vector<double>(p, p + n), s);
  };
  cudaError_t e = cudaSuccess;
  e = e ? e : upload(h->d_inter_pt, h->inter_pt_h, s);
  e = e ? e : upload(h->d_nb_kind, h->nb_kind_h, s);
  e = e ? e : upload(h->d_nb_idx, h->nb_idx_h, s);
  e = e ? e : upload(h->d_nb_coef, h->nb_coef_h, s);
  e = e ? e : up_i(h->d_numia, g->numia, g->npsom);
  e = e ? e : up_i(h->d_nbord, g->nbord, g->natome);
  e = e ? e : up_i(h->d_nbordf, g->nbordf, g->natome);
  e = e ? e : up_i(h->d_ibord, g->ibord, (size_t)g->nbtm * g->natome);
  e = e ? e : up_i(h->d_isbord, g->isbord, (size_t)g->nbtm * g->natome);
  e = e ? e : up_i(h->d_isrt, g->isrt, g->nstm);
  e = e ? e : up_i(h->d_lato, g->lato, (size_t)g->nlmsam * g->natome);
  e = e ? e : up_i(h->d_mato, g->mato, (size_t)g->nlmsam * g->natome);
  e = e ? e : up_i(h->d_lso, g->lso, g->nso1);
  e = e ? e : up_i(h->d_mso, g->mso, g->nso1);
  // spin and gradient tables are read by the complex path only; absent ones read as 1 and 0
  e = e ? e : (g->iato ? up_i(h->d_iato, g->iato, (size_t)g->nlmsam * g->natome)
                       : upload(h->d_iato, std::vector<int>((size_t)g->nlmsam * g->natome, 1), s));
  e = e ? e : (g->iso ? up_i(h->d_iso, g->iso, g->nso1) : upload(h->d_iso, std::vector<int>(g->nso1, 1), s));
  e = e ? e : (g->cgrad ? up_d(h->d_cgrad, g->cgrad, g->nvois)
                        : upload(h->d_cgrad, std::vector<double>(g->nvois, 0.0), s));
  e = e ? e : up_d(h->d_rvol, g->rvol, g->nim);
  e = e ? e : up_d(h->d_clapl, g->clapl, g->nvois + 1);
  e = e ? e : up_d(h->d_poidsa, g->poidsa, (size_t)g->nbm * g->natome);
  e = e ? e : up_d(h->d_poidso, g->poidso, g->nsm);
  e = e ? e : up_d(h->d_Kar, g->Kar, 64);
  e = e ? e : up_d(h->d_Ylmato, g->Ylmato, (size_t)g->nbtm * g->nlmmax * g->natome);
  std::vector<double> ysot((size_t)g->nsort * g->nlmomax);
  for (int ib = 0; ib < g->nsort; ++ib)
    for (int lm = 0; lm < g->nlmomax; ++lm) ysot[(size_t)ib * g->nlmomax + lm] = g->Ylmso[ib + (int64_t)g->nsort * lm];
  e = e ? e : upload(h->d_YsoT, ysot, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    fdmgpu_destroy(h);
    return fail(FDMGPU_ERR_CUDA, std::string("static upload: ") + cudaGetErrorString(e));
  }
  StaticDev& S = h->S;
  S.npoint = g->npoint;
  S.npsom = g->npsom;
  S.nvois = g->nvois;
  S.natome = g->natome;
  S.nbtm = g->nbtm;
  S.nbm = g->nbm;
  S.nsort = g->nsort;
  S.nsortf = g->nsortf;
  S.nlmmax = g->nlmmax;
  S.nlmomax = g->nlmomax;
  S.nlmsam = g->nlmsam;
  S.nso1 = g->nso1;
  S.npr = (int)h->inter_pt_h.size();
  S.inter_pt = h->d_inter_pt.p;
  S.nb_kind = h->d_nb_kind.p;
  S.nb_idx = h->d_nb_idx.p;
  S.nb_coef = h->d_nb_coef.p;
  S.rvol = h->d_rvol.p;
  S.clapl = h->d_clapl.p;
  S.numia = h->d_numia.p;
  S.nbord = h->d_nbord.p;
  S.nbordf = h->d_nbordf.p;
  S.ibord = h->d_ibord.p;
  S.isrt = h->d_isrt.p;
  S.poidsa = h->d_poidsa.p;
  S.poidso = h->d_poidso.p;
  S.Kar = h->d_Kar.p;
  S.isbord = h->d_isbord.p;
  S.YsoT = h->d_YsoT.p;
  S.Ylmato = h->d_Ylmato.p;
  S.lato = h->d_lato.p;
  S.mato = h->d_mato.p;
  S.lso = h->d_lso.p;
  S.mso = h->d_mso.p;
  S.iato = h->d_iato.p;
  S.iso = h->d_iso.p;
  S.cgrad = h->d_cgrad.p;
  S.nspino = g->nspino;
  S.nspin = g->nspin;
  setup_factor_kernels<float>();
  setup_factor_kernels<double>();
  setup_factor_kernels<dfl>();
  setup_tc_kernels();
  setup_oz_kernels();
  setup_strip_kernels();
  *out = h;
  return FDMGPU_OK;
}

void fdmgpu_destroy(fdmgpu_handle* h) {
  if (!h) return;
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->g_asm) cudaGraphExecDestroy(h->g_asm);
  if (h->g_fac) cudaGraphExecDestroy(h->g_fac);
  if (h->g_sol) cudaGraphExecDestroy(h->g_sol);
  if (h->g_iter) cudaGraphExecDestroy(h->g_iter);
  if (h->g_loop) cudaGraphExecDestroy(h->g_loop);
  h->d_rstate.release();
  h->d_rctl.release();
  h->d_xs.release();
  h->d_rad_i.release();
  h->d_rad_d.release();
  h->d_rads.release();
  h->d_radU.release();
  if (h->g_res) cudaGraphExecDestroy(h->g_res);
  h->d_nnz.release();
  DevBuf<int>* ib[] = {&h->d_inter_pt, &h->d_nb_kind, &h->d_nb_idx, &h->d_numia, &h->d_nbord, &h->d_nbordf,
                       &h->d_ibord,    &h->d_isbord,  &h->d_isrt,   &h->d_lato,  &h->d_mato,  &h->d_lso,
                       &h->d_mso,      &h->d_J0,      &h->d_J1,     &h->d_Imax,  &h->d_Imin,  &h->d_ipool,
                       &h->d_rowptr,   &h->d_col,     &h->d_err,    &h->d_active, &h->d_piv,   &h->d_iato,
                       &h->d_iso};
  for (auto* b : ib) b->release();
  DevBuf<double>* db[] = {&h->d_nb_coef, &h->d_rvol, &h->d_clapl, &h->d_poidsa, &h->d_poidso, &h->d_Kar,
                          &h->d_YsoT,    &h->d_Ylmato, &h->d_dpool, &h->d_env64, &h->d_B64,  &h->d_X64,
                          &h->d_rs,      &h->d_cs,   &h->d_val,   &h->d_taull,  &h->d_tscratch, &h->d_smr,
                          &h->d_gT,      &h->d_lam,  &h->d_gpart, &h->d_grad,  &h->d_cgrad};
  for (auto* b : db) b->release();
  h->d_env32.release();
  h->d_val2.release();
  h->d_Xs.release();
  h->d_valS.release();
  h->d_V.release();
  h->d_W.release();
  h->d_gstate.release();
  h->d_inner.release();
  h->d_jdone.release();
  h->d_notconv.release();
  h->d_active_gm.release();
  h->d_Y32.release();
  h->d_sites.release();
  h->d_R32.release();
  h->d_act_df.release();
  h->d_act_rec.release();
  h->d_strip.release();
  h->d_wide.release();
  h->d_wide_all.release();
  h->d_oz_img.release();
  h->d_oz_exp.release();
  h->d_dfl_inv.release();
  h->d_esc_list.release();
  h->d_err_esc.release();
  h->d_probs_esc.release();
  h->d_uinv_keep.release();
  h->d_probs.release();
  h->d_red.release();
  if (h->h_pinned_i) cudaFreeHost(h->h_pinned_i);
  if (h->h_pinned_d) cudaFreeHost(h->h_pinned_d);
  for (auto& e : h->ev)
    if (e) cudaEventDestroy(e);
  if (h->stream) cudaStreamDestroy(h->stream);
  if (h->stream2) cudaStreamDestroy(h->stream2);
  if (h->ev_join) cudaEventDestroy(h->ev_join);
  for (auto& e : h->ev_esc)
    if (e) cudaEventDestroy(e);
  h->d_esc_mask.release();
  h->d_G.release();
  h->d_lams.release();
  h->d_colptr.release();
  h->d_cursor.release();
  h->d_cscrow.release();
  h->d_cscval2.release();
  if (h->h_esc_mask) cudaFreeHost(h->h_esc_mask);
  h->d_red_esc.release();
  h->d_red_tmp.release();
  delete h;
}

fdmgpu_status fdmgpu_set_residual_mode(fdmgpu_handle* h, int32_t mode) {
  if (!h || (mode != FDMGPU_RESIDUAL_FP64 && mode != FDMGPU_RESIDUAL_DF64))
    return fail(FDMGPU_ERR_ARG, "unknown residual mode");
  h->residual_df64 = mode == FDMGPU_RESIDUAL_DF64;
  return FDMGPU_OK;
}

fdmgpu_status fdmgpu_set_refinement(fdmgpu_handle* h, int32_t mode, int32_t krylov_dim) {
  if (!h || (mode != FDMGPU_REFINE_CLASSIC && mode != FDMGPU_REFINE_GMRES && mode != FDMGPU_REFINE_RECURRENCE) ||
      krylov_dim < 1 || krylov_dim > gmres_max_dim())
    return fail(FDMGPU_ERR_ARG, "unknown refinement mode or Krylov dimension out of range");
  h->refine_gmres = mode == FDMGPU_REFINE_GMRES;
  h->refine_recur = mode == FDMGPU_REFINE_RECURRENCE;
  h->gmres_m = krylov_dim;
  h->plan_sig = 0;  // pool sizes and graphs depend on the mode: plan again
  return FDMGPU_OK;
}

fdmgpu_status fdmgpu_set_tolerance(fdmgpu_handle* h, double tol, double tol_accept) {
  if (!h || !(tol >= 0) || !(tol_accept >= 0) || tol >= 1 || tol_accept >= 1 || (tol > 0 && tol_accept > 0 && tol_accept < tol))
    return fail(FDMGPU_ERR_ARG, "tolerances must satisfy 0 <= tol <= tol_accept < 1 (0 selects the default)");
  h->tol = tol;
  h->tol_accept = tol_accept;
  return FDMGPU_OK;
}

fdmgpu_status fdmgpu_set_factor_mode(fdmgpu_handle* h, int32_t mode) {
  if (!h) return fail(FDMGPU_ERR_ARG, "null handle");
  if (mode != FDMGPU_FACTOR_FP32 && mode != FDMGPU_FACTOR_WIDE_ATOM && mode != FDMGPU_FACTOR_WIDE_ALL)
    return fail(FDMGPU_ERR_ARG, "unknown factor mode");
  h->factor_mode = mode;
  return FDMGPU_OK;
}

fdmgpu_status fdmgpu_set_radial(fdmgpu_handle* h, const fdmgpu_radial* rd) {
  if (!h || !rd) return fail(FDMGPU_ERR_ARG, "null argument");
  const fdmgpu_grid& g = h->g;
  if (g.nspino != 1) return fail(FDMGPU_ERR_UNSUPPORTED, "generated inputs are provided for the real path (nspino = 1)");
  if (rd->ntype < 1 || rd->ntype > MAX_GEN_TYPES || rd->nr_max < 4 || rd->nspin < 1 || !rd->nr || !rd->r || !rd->V ||
      !rd->dv_spin || !rd->z_origin || !rd->itype || !rd->rrel || !rd->rsort)
    return fail(FDMGPU_ERR_ARG, "radial tables: bad sizes or null arrays (1 <= ntype <= 8)");
  const int T = rd->ntype, NR = rd->nr_max, nb = g.nbtm, na = g.natome;
  std::vector<int> ih(T + na + (size_t)nb * na, 0);
  std::vector<double> dh((size_t)6 * NR * T + rd->nspin + T + (size_t)nb * na + g.nsort, 0.0);
  double* r = dh.data();
  double* mcl0 = r + (size_t)NR * T;
  double* gm = mcl0 + (size_t)NR * T;
  double* gp = gm + (size_t)NR * T;
  double* f2 = gp + (size_t)NR * T;
  double* V = f2 + (size_t)NR * T;
  double* dv = V + (size_t)NR * T;
  double* z = dv + rd->nspin;
  double* rrel = z + T;
  double* rsort = rrel + (size_t)nb * na;
  h->rad_dv_max = -1e300;
  for (int i = 0; i < rd->nspin; ++i) {
    dv[i] = rd->dv_spin[i];
    h->rad_dv_max = std::max(h->rad_dv_max, dv[i]);
  }
  for (int t = 0; t < T; ++t) {
    const int n = rd->nr[t];
    if (n < 4 || n > NR) return fail(FDMGPU_ERR_ARG, "radial mesh size out of range");
    ih[t] = n;
    z[t] = rd->z_origin[t];
    const double* rt = rd->r + (size_t)NR * t;
    for (int i = 0; i < n; ++i) {
      if (!(rt[i] > 0.0) || (i > 0 && !(rt[i] > rt[i - 1]))) return fail(FDMGPU_ERR_ARG, "radial mesh must increase");
      r[(size_t)NR * t + i] = rt[i];
      V[(size_t)NR * t + i] = rd->V[(size_t)NR * t + i];
    }
    // three-point Laplacian coefficients of the mesh (coef_sch_rad,
    // source/sphere.f90:324-396), with the mesh extended geometrically past
    // both ends
    for (int i = 0; i < n; ++i) {
      const double rp = i + 1 < n ? rt[i + 1] : rt[n - 1] * rt[n - 1] / rt[n - 2];
      const double rm = i > 0 ? rt[i - 1] : rt[0] * rt[0] / rt[1];
      const double drr = 0.5 * (rp - rm);
      const double cm = 1.0 / ((rt[i] - rm) * drr), cp = 1.0 / ((rp - rt[i]) * drr);
      const double c0 = -cm - cp;
      mcl0[(size_t)NR * t + i] = -c0;
      gm[(size_t)NR * t + i] = -cm;
      gp[(size_t)NR * t + i] = -cp;
      f2[(size_t)NR * t + i] = 1.0 / (rt[i] * rt[i]);
    }
  }
  h->rad_itype.assign(na, 0);
  for (int ia = 0; ia < na; ++ia) {
    const int t = rd->itype[ia] - 1;
    if (t < 0 || t >= T) return fail(FDMGPU_ERR_ARG, "itype out of range");
    ih[T + ia] = t;
    h->rad_itype[ia] = t;
    const double* rt = rd->r + (size_t)NR * t;
    const int n = rd->nr[t];
    for (int ib = 0; ib < g.nbord[ia] && ib < nb; ++ib) {
      const double x = rd->rrel[ib + (size_t)nb * ia];
      rrel[ib + (size_t)nb * ia] = x;
      // first mesh point beyond x, kept inside [2, n - 1] (cal_phiato's stencil)
      int k = (int)(std::upper_bound(rt, rt + n, x) - rt);
      k = std::min(std::max(k, 2), n - 1);
      ih[T + na + ib + (size_t)nb * ia] = k;
    }
  }
  for (int ib = 0; ib < g.nsort; ++ib) rsort[ib] = rd->rsort[ib];
  cudaStream_t s = h->stream;
  CK(upload(h->d_rad_i, ih, s));
  CK(upload(h->d_rad_d, dh, s));
  CK(cudaStreamSynchronize(s));
  RadialDev R{};
  R.ntype = T;
  R.nr_max = NR;
  R.nspin = rd->nspin;
  R.nr = h->d_rad_i.p;
  R.itype = h->d_rad_i.p + T;
  R.iidx = h->d_rad_i.p + T + na;
  const double* b = h->d_rad_d.p;
  R.r = b;
  R.mcl0 = b + (size_t)NR * T;
  R.gm = b + (size_t)2 * NR * T;
  R.gp = b + (size_t)3 * NR * T;
  R.f2 = b + (size_t)4 * NR * T;
  R.V = b + (size_t)5 * NR * T;
  R.dv_spin = b + (size_t)6 * NR * T;
  R.z_origin = R.dv_spin + rd->nspin;
  R.rrel = R.z_origin + T;
  R.rsort = R.rrel + (size_t)nb * na;
  R.v0bd = rd->v0bd;
  h->rad = R;
  h->rad_ntype = T;
  h->rad_nr_max = NR;
  h->rad_v0bd = rd->v0bd;
  h->has_radial = true;
  h->plan_sig = 0;
  return FDMGPU_OK;
}

fdmgpu_status fdmgpu_set_solve_order(fdmgpu_handle* h, int32_t order) {
  if (!h) return fail(FDMGPU_ERR_ARG, "null handle");
  if (order != FDMGPU_SOLVE_COLUMNS && order != FDMGPU_SOLVE_ROWS) return fail(FDMGPU_ERR_ARG, "unknown solve order");
  h->solve_order = order;
  return FDMGPU_OK;
}

fdmgpu_status fdmgpu_set_df64_engine(fdmgpu_handle* h, int32_t engine) {
  if (!h) return fail(FDMGPU_ERR_ARG, "null handle");
  if (engine != FDMGPU_DF64_SIMT && engine != FDMGPU_DF64_TCGEN05) return fail(FDMGPU_ERR_ARG, "unknown engine");
  h->df64_engine = engine;
  return FDMGPU_OK;
}

fdmgpu_status fdmgpu_set_tile_engine(fdmgpu_handle* h, int32_t engine) {
  if (!h) return fail(FDMGPU_ERR_ARG, "null handle");
  if (engine != FDMGPU_ENGINE_SIMT && engine != FDMGPU_ENGINE_TCGEN05 && engine != FDMGPU_ENGINE_TCGEN05_FACTOR &&
      engine != FDMGPU_ENGINE_SIMT_STREAM)
    return fail(FDMGPU_ERR_ARG, "unknown tile engine");
  h->tile_engine = engine;
  return FDMGPU_OK;
}

fdmgpu_status fdmgpu_set_autotune(fdmgpu_handle* h, int32_t on) {
  if (!h) return fail(FDMGPU_ERR_ARG, "null handle");
  h->autotune = on != 0;
  if (!h->autotune) h->trail_threads[0] = h->trail_threads[1] = 0;
  h->plan_sig = 0;
  return FDMGPU_OK;
}

fdmgpu_status fdmgpu_get_tuning(fdmgpu_handle* h, int32_t precision, int32_t* trailing_threads, double* ms64,
                                double* ms128) {
  if (!h || (precision != FDMGPU_PREC_FP64 && precision != FDMGPU_PREC_MIXED))
    return fail(FDMGPU_ERR_ARG, "null handle or unknown precision");
  const int pi = precision == FDMGPU_PREC_FP64 ? 0 : 1;
  if (trailing_threads) *trailing_threads = h->trail_threads[pi];
  if (ms64) *ms64 = h->trail_ms[pi][0];
  if (ms128) *ms128 = h->trail_ms[pi][1];
  return FDMGPU_OK;
}

fdmgpu_status fdmgpu_set_escalation(fdmgpu_handle* h, int32_t mode) {
  if (!h || (mode != FDMGPU_ESCALATE_FP64 && mode != FDMGPU_ESCALATE_DF64 && mode != FDMGPU_ESCALATE_DF64_OVERLAP &&
             mode != FDMGPU_ESCALATE_WIDE_DF64 && mode != FDMGPU_ESCALATE_DF64_F32))
    return fail(FDMGPU_ERR_ARG, "unknown escalation mode");
  h->escalate_dfl = mode != FDMGPU_ESCALATE_FP64;
  h->overlap_escalation = mode == FDMGPU_ESCALATE_DF64_OVERLAP;
  h->escalate_wide = mode == FDMGPU_ESCALATE_WIDE_DF64;
  h->escalate_f32 = mode == FDMGPU_ESCALATE_DF64_F32;
  h->plan_sig = 0;
  return FDMGPU_OK;
}

fdmgpu_status fdmgpu_batch_begin(fdmgpu_handle* h, int32_t precision, int32_t max_energies) {
  if (!h) return fail(FDMGPU_ERR_ARG, "null handle");
  if (precision != FDMGPU_PREC_FP64 && precision != FDMGPU_PREC_MIXED)
    return fail(FDMGPU_ERR_ARG, "unknown precision");
  h->batch.probs.clear();
  h->batch.cplx = -1;
  h->batch.sites.assign(1, h);
  h->batch.precision = precision;
  h->batch.max_energies = max_energies;
  h->batch.ran = false;
  h->batch.probs.reserve(std::max(0, (int)max_energies));
  return FDMGPU_OK;
}

fdmgpu_status fdmgpu_batch_add_site(fdmgpu_handle* h, fdmgpu_handle* site, const fdmgpu_energy* e, int32_t iaabs) {
  if (!h || !site) return fail(FDMGPU_ERR_ARG, "null handle");
  if (site->device != h->device) return fail(FDMGPU_ERR_ARG, "the site handle lives on another device");
  Batch& b = h->batch;
  if (b.sites.empty()) b.sites.assign(1, h);
  fdmgpu_status st = check_energy(site, e);
  if (st) return st;
  if (b.max_energies > 0 && (int)b.probs.size() >= b.max_energies) return fail(FDMGPU_ERR_ARG, "batch is full");
  int si = (int)(std::find(b.sites.begin(), b.sites.end(), site) - b.sites.begin());
  if (si == (int)b.sites.size()) b.sites.push_back(site);
  const int cplx = e->Cal_comp ? 1 : 0;
  if (b.cplx >= 0 && b.cplx != cplx) return fail(FDMGPU_ERR_ARG, "a batch holds either real or complex problems");
  if (cplx && b.sites.size() > 1) return fail(FDMGPU_ERR_UNSUPPORTED, "complex problems of several sites in one batch");
  HostProb hp;
  st = plan_problem(site, e, hp);
  if (st) return st;
  hp.P.site = si;
  const fdmgpu_grid& g = site->g;
  if (iaabs >= 1 && iaabs <= g.natome) {
    hp.P.iaabs = iaabs;
    hp.P.nlm_abs = e->nlmsa[iaabs - 1];
    hp.P.ianew_abs = e->ianew[iaabs - 1];
    if (cplx) {
      // every (L, m, spin) up to the absorber's lmax once, so that Taull is dense
      // in (L^2 + L + m, spin) on both sides
      const int nsp = g.nspino;
      int lmax = 0;
      std::vector<int> seen;
      for (int lm = 1; lm <= hp.P.nlm_abs; ++lm) lmax = std::max(lmax, F2(g.lato, g.nlmsam, lm, iaabs));
      const int nlmq = (lmax + 1) * (lmax + 1);
      if (hp.P.nlm_abs != nsp * nlmq) return fail(FDMGPU_ERR_UNSUPPORTED, "Taull needs complete absorber harmonic tables");
      seen.assign(nsp * nlmq, 0);
      for (int lm = 1; lm <= hp.P.nlm_abs; ++lm) {
        const int L = F2(g.lato, g.nlmsam, lm, iaabs), m = F2(g.mato, g.nlmsam, lm, iaabs);
        const int is = nsp == 2 ? F2(g.iato, g.nlmsam, lm, iaabs) : 1;
        if (m < -L || m > L || is < 1 || is > nsp || seen[(L * L + L + m) + nlmq * (is - 1)]++)
          return fail(FDMGPU_ERR_UNSUPPORTED, "Taull needs complete absorber harmonic tables");
      }
      if ((int64_t)hp.P.nlm_abs * hp.P.nlm_abs > (int64_t)e->nlmso * (e->nlmso + 2 * hp.P.nlm_abs))
        return fail(FDMGPU_ERR_UNSUPPORTED, "absorber harmonics exceed the Taull scratch");
    } else {
      for (int lm = 1; lm <= hp.P.nlm_abs; ++lm) {
        const int L = F2(g.lato, g.nlmsam, lm, iaabs), m = F2(g.mato, g.nlmsam, lm, iaabs);
        if (L * L + L + 1 + m != lm) return fail(FDMGPU_ERR_UNSUPPORTED, "Taull needs the C1 harmonic order");
      }
    }
  }
  b.cplx = cplx;
  hp.sig = mix(hp.sig, (uint64_t)hp.P.nlm_abs * 7919u + (uint64_t)hp.P.ianew_abs);
  hp.sig = mix(hp.sig, (uint64_t)si * 104729u + 1u);
  pack_inputs(site, e, hp);
  b.probs.push_back(std::move(hp));
  b.ran = false;
  return FDMGPU_OK;
}

fdmgpu_status fdmgpu_batch_add(fdmgpu_handle* h, const fdmgpu_energy* e, int32_t iaabs) {
  return fdmgpu_batch_add_site(h, h, e, iaabs);
}

// Device bytes of one problem's pools (band FP64 + FP32, right-hand-side
// tiles, CSR copy, per-row vectors), the quantities allocate_and_upload_plan
// reserves per problem.
static double problem_bytes(const HostProb& hp, bool mixed) {
  const double tiles = (double)hp.ntiles * TS2, rhs = (double)hp.P.nt * hp.P.nrt * TS2;
  const double rowv = (double)hp.P.nt * TS + 1;
  if (!mixed) return tiles * 8 + rhs * 16 + rowv * 4;
  // + the integer-slice images of one step's L and U / RHS tiles (7 bf16 images a tile)
  const double slices = (double)(hp.P.nt + hp.P.nrt) * 7 * TS2 * 2;
  return tiles * 12 + rhs * 44 + (double)hp.nnz_cap * 24 + rowv * 28 + slices;
}

// A batch whose pools exceed the budget runs in consecutive chunks of
// problems (add order), each planned, captured and run like a batch of its
// own; Taull, refinement statistics and statuses are gathered per problem.
static fdmgpu_status run_chunked(fdmgpu_handle* h, fdmgpu_info* info, double budget) {
  Batch& b = h->batch;
  std::vector<HostProb> all = std::move(b.probs);
  const int np = (int)all.size();
  const bool mixed = b.precision == FDMGPU_PREC_MIXED;
  std::vector<int> iters(np), fallback(np), wide(np), inner(np), err(np);
  std::vector<double> resid(np);
  b.taull_off.assign(np + 1, 0);
  for (int k = 0; k < np; ++k) b.taull_off[k + 1] = b.taull_off[k] + 2 * (int64_t)all[k].P.nlm_abs * all[k].P.nlm_abs;
  b.taull_host.assign(b.taull_off[np], 0.0);
  fdmgpu_info acc;
  memset(&acc, 0, sizeof(acc));
  fdmgpu_status worst = FDMGPU_OK;
  int k0 = 0, nchunks = 0;
  while (k0 < np) {
    int k1 = k0;
    double bytes = 0;
    while (k1 < np && (k1 == k0 || bytes + problem_bytes(all[k1], mixed) <= budget)) bytes += problem_bytes(all[k1++], mixed);
    b.probs.clear();
    for (int k = k0; k < k1; ++k) b.probs.push_back(all[k]);
    fdmgpu_info ci;
    fdmgpu_status st = run_batch(h, &ci, false);
    if (st && st != FDMGPU_ERR_NOT_CONVERGED) {
      b.probs = std::move(all);
      b.ran = false;
      return st;
    }
    if (st) worst = st;
    // Taull of the chunk (contiguous in its pool)
    if (b.taull_off[k1] > b.taull_off[k0])
      CK(cudaMemcpy(b.taull_host.data() + b.taull_off[k0], h->d_taull.p + 2 * b.probs[0].P.taull,
                    sizeof(double) * (b.taull_off[k1] - b.taull_off[k0]), cudaMemcpyDeviceToHost));
    for (int k = k0; k < k1; ++k) {
      const int j = k - k0;
      iters[k] = b.iters.empty() ? 0 : b.iters[j];
      resid[k] = b.resid.empty() ? 0.0 : b.resid[j];
      fallback[k] = b.fallback.empty() ? 0 : b.fallback[j];
      wide[k] = b.wide.empty() ? 0 : b.wide[j];
      inner[k] = b.inner.empty() ? 0 : b.inner[j];
      err[k] = b.err.empty() ? 0 : b.err[j];
    }
    acc.nnz_profile += ci.nnz_profile;
    acc.flops_factor += ci.flops_factor;
    acc.flops_solve += ci.flops_solve;
    acc.refine_iters = std::max(acc.refine_iters, ci.refine_iters);
    acc.residual = std::max(acc.residual, ci.residual);
    acc.ms_assemble += ci.ms_assemble;
    acc.ms_factor += ci.ms_factor;
    acc.ms_solve += ci.ms_solve;
    acc.ms_refine += ci.ms_refine;
    acc.n_fallback += ci.n_fallback;
    acc.n_kernels += ci.n_kernels;
    acc.ms_residual_first += ci.ms_residual_first;
    acc.flops_residual += ci.flops_residual;
    acc.ms_escalate_factor += ci.ms_escalate_factor;
    acc.flops_escalate_factor += ci.flops_escalate_factor;
    acc.n_wide_refactor += ci.n_wide_refactor;
    acc.ms_wide_refactor += ci.ms_wide_refactor;
    acc.flops_wide_refactor += ci.flops_wide_refactor;
    ++nchunks;
    k0 = k1;
  }
  b.probs = std::move(all);
  b.iters = iters;
  b.resid = resid;
  b.fallback = fallback;
  b.wide = wide;
  b.inner = inner;
  b.err = err;
  b.ran = true;
  b.chunked = true;
  b.nchunks = nchunks;
  h->plan_sig = 0;  // the pools hold the last chunk only
  if (info) *info = acc;
  return worst;
}

static double batch_budget(fdmgpu_handle* h) {
  if (h->mem_budget > 0) return h->mem_budget;
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return 1e300;
  return 0.85 * (double)tot;
}

fdmgpu_status fdmgpu_batch_run(fdmgpu_handle* h, fdmgpu_info* info) {
  if (!h) return fail(FDMGPU_ERR_ARG, "null handle");
  Batch& b = h->batch;
  b.chunked = false;
  b.taull_host.clear();
  const bool mixed = b.precision == FDMGPU_PREC_MIXED;
  double total = 0;
  for (auto& hp : b.probs) total += problem_bytes(hp, mixed);
  const double budget = batch_budget(h);
  if (total > budget && b.probs.size() > 1) return run_chunked(h, info, budget);
  return run_batch(h, info, false);
}

fdmgpu_status fdmgpu_batch_rerun(fdmgpu_handle* h, fdmgpu_info* info) {
  if (!h) return fail(FDMGPU_ERR_ARG, "null handle");
  if (h->batch.chunked) return run_chunked(h, info, batch_budget(h));
  return run_batch(h, info, true);
}

fdmgpu_status fdmgpu_set_memory_budget(fdmgpu_handle* h, double bytes) {
  if (!h || !(bytes >= 0)) return fail(FDMGPU_ERR_ARG, "bad memory budget");
  h->mem_budget = bytes;
  return FDMGPU_OK;
}

fdmgpu_status fdmgpu_batch_taull(fdmgpu_handle* h, int32_t k, double* taull, int32_t* nlm) {
  if (!h || !h->batch.ran || k < 0 || k >= (int)h->batch.probs.size())
    return fail(FDMGPU_ERR_ARG, "no such batch result");
  const Prob& P = h->batch.probs[k].P;
  if (nlm) *nlm = P.nlm_abs;
  if (!taull) return FDMGPU_OK;
  if (h->batch.chunked) {
    memcpy(taull, h->batch.taull_host.data() + h->batch.taull_off[k], sizeof(double) * 2 * P.nlm_abs * P.nlm_abs);
    return FDMGPU_OK;
  }
  CK(cudaMemcpy(taull, h->d_taull.p + 2 * P.taull, sizeof(double) * 2 * P.nlm_abs * P.nlm_abs,
                cudaMemcpyDeviceToHost));
  return FDMGPU_OK;
}

fdmgpu_status fdmgpu_batch_tau_ri(fdmgpu_handle* h, int32_t k_reg, int32_t k_irr, double* tau_ri, int32_t* nlm) {
  if (!h || !h->batch.ran) return fail(FDMGPU_ERR_ARG, "run a batch first");
  Batch& b = h->batch;
  const int np = (int)b.probs.size();
  if (k_reg < 0 || k_reg >= np || k_irr < 0 || k_irr >= np) return fail(FDMGPU_ERR_ARG, "no such batch result");
  if (b.chunked) return fail(FDMGPU_ERR_UNSUPPORTED, "Tau_RI of a batch that ran in chunks (its solutions are gone)");
  const Prob& P = b.probs[k_reg].P;
  const Prob& Q = b.probs[k_irr].P;
  if (!P.cplx || P.irr || !Q.irr)
    return fail(FDMGPU_ERR_ARG, "k_reg must be a regular and k_irr an irregular complex solution");
  if (P.site != Q.site || P.iaabs < 1 || P.iaabs != Q.iaabs || P.nlm_abs != Q.nlm_abs || P.nlmso != Q.nlmso)
    return fail(FDMGPU_ERR_ARG, "the pair must share the site, the absorber and the outer harmonics");
  if (P.enervide != Q.enervide || P.eimag != Q.eimag || P.ispin != Q.ispin)
    return fail(FDMGPU_ERR_ARG, "the pair must be one energy and spin block");
  if (nlm) *nlm = P.nlm_abs;
  if (!tau_ri) return FDMGPU_OK;
  const size_t n = 2 * (size_t)P.nlm_abs * P.nlm_abs;   // complex values
  if (h->d_smr.reserve(2 * n) != cudaSuccess) return fail(FDMGPU_ERR_NOMEM, "Tau_RI buffer");
  launch_tau_ri(h->d_sites.p, h->d_probs.p + k_reg, h->d_probs.p + k_irr, h->d_X64.p, P.nlm_abs,
                reinterpret_cast<double2*>(h->d_smr.p), h->stream);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(tau_ri, h->d_smr.p, 2 * n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return (fdmgpu_status)(b.err[k_reg] ? b.err[k_reg] : b.err[k_irr]);
}

fdmgpu_status fdmgpu_batch_taull_all(fdmgpu_handle* h, double* taull, int64_t capacity) {
  if (!h || !h->batch.ran || h->batch.probs.empty()) return fail(FDMGPU_ERR_ARG, "no batch result");
  int64_t n = 0;
  for (auto& hp : h->batch.probs) n += (int64_t)hp.P.nlm_abs * hp.P.nlm_abs;
  if (!taull || capacity < 2 * n) return fail(FDMGPU_ERR_ARG, "Taull buffer too small");
  if (h->batch.chunked) {
    memcpy(taull, h->batch.taull_host.data(), sizeof(double) * 2 * n);
    return FDMGPU_OK;
  }
  // the pool holds the energies' Taull contiguously in add order
  CK(cudaMemcpy(taull, h->d_taull.p + 2 * h->batch.probs[0].P.taull, sizeof(double) * 2 * n,
                cudaMemcpyDeviceToHost));
  return FDMGPU_OK;
}

fdmgpu_status fdmgpu_batch_solution(fdmgpu_handle* h, int32_t k, double* smr) {
  if (h && h->batch.chunked) return fail(FDMGPU_ERR_UNSUPPORTED, "a batch that ran in chunks keeps only its Taull (solutions of the last chunk are gone)");
  if (!h || !h->batch.ran || k < 0 || k >= (int)h->batch.probs.size())
    return fail(FDMGPU_ERR_ARG, "no such batch result");
  const Prob& P = h->batch.probs[k].P;
  const size_t n = (size_t)P.n * P.nlmso;
  if (h->d_smr.reserve(n) != cudaSuccess) return fail(FDMGPU_ERR_NOMEM, "solution buffer");
  launch_solution_out(P, h->d_X64.p, h->d_smr.p, h->stream);
  CK(cudaMemcpyAsync(smr, h->d_smr.p, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return FDMGPU_OK;
}

fdmgpu_status fdmgpu_batch_stats(fdmgpu_handle* h, int32_t k, int32_t* iters, double* residual,
                                 int32_t* fallback, int32_t* inner_iters) {
  if (!h || !h->batch.ran || k < 0 || k >= (int)h->batch.probs.size())
    return fail(FDMGPU_ERR_ARG, "no such batch result");
  if (iters) *iters = h->batch.iters[k];
  if (inner_iters) *inner_iters = h->batch.inner.empty() ? 0 : h->batch.inner[k];
  if (residual) *residual = h->batch.resid[k];
  if (fallback) *fallback = h->batch.fallback.empty() ? 0 : h->batch.fallback[k];
  return (fdmgpu_status)h->batch.err[k];
}

fdmgpu_status fdmgpu_mat_solve(fdmgpu_handle* h, const fdmgpu_energy* e, int32_t precision, double* smr, double* smi,
                               fdmgpu_info* info) {
  if (!h || !smr || !e) return fail(FDMGPU_ERR_ARG, "null argument");
  if (e->Cal_comp && !smi) return fail(FDMGPU_ERR_ARG, "a complex problem needs smi");
  fdmgpu_status st = fdmgpu_batch_begin(h, precision, 1);
  if (st) return st;
  st = fdmgpu_batch_add(h, e, 0);
  if (st) return st;
  st = fdmgpu_batch_run(h, info);
  if (st && st != FDMGPU_ERR_NOT_CONVERGED) return st;
  if (!e->Cal_comp) {
    fdmgpu_status st2 = fdmgpu_batch_solution(h, 0, smr);
    return st2 ? st2 : st;
  }
  // real-equivalent solution: row 2ii-1 holds Re x(ii), row 2ii Im x(ii)
  const int64_t n = e->nligne, m = e->nlmso;
  std::vector<double> xe((size_t)(2 * n * m));
  fdmgpu_status st2 = fdmgpu_batch_solution(h, 0, xe.data());
  if (st2) return st2;
  for (int64_t ii = 0; ii < n; ++ii)
    for (int64_t l = 0; l < m; ++l) {
      smr[l + m * ii] = xe[(size_t)(l + m * (2 * ii))];
      smi[l + m * ii] = xe[(size_t)(l + m * (2 * ii + 1))];
    }
  return st;
}

// Adjoint solve of a mixed batch: A^T Lambda = G with the batch's factors of the
// equilibrated matrix Ah = R A C (FP32 with tile-local pivots, or the
// double-float factors of the escalated problems):  Ah^T mu = C G, Lambda = R mu,
// refined with the transposed double-float residual C (G - A^T Lambda) from the
// CSR of A^T.  With Lambda = 0 the first residual is C G itself.
static fdmgpu_status vjp_mixed(fdmgpu_handle* h, int64_t nrhs) {
  Batch& b = h->batch;
  const int np = h->dims.nprob;
  cudaStream_t s = h->stream;
  int64_t csr = 0;
  for (auto& hp : b.probs) csr = std::max<int64_t>(csr, hp.P.csr + hp.P.csr_cap);
  const int64_t rowv = h->dims.rowv_total;
  if (h->d_G.reserve(nrhs) != cudaSuccess || h->d_lams.reserve(nrhs) != cudaSuccess ||
      h->d_colptr.reserve(rowv) != cudaSuccess || h->d_cursor.reserve(rowv) != cudaSuccess ||
      h->d_cscrow.reserve(csr) != cudaSuccess || h->d_cscval2.reserve(csr) != cudaSuccess)
    return fail(FDMGPU_ERR_NOMEM, "device allocation of the mixed adjoint pools failed");
  CK(cudaMemsetAsync(h->d_G.p, 0, nrhs * sizeof(double), s));
  CK(cudaMemsetAsync(h->d_lams.p, 0, nrhs * sizeof(float2), s));
  launch_taull_vjp(h->d_probs.p, h->dims, h->pl.X64, h->d_gT.p, h->pl.tscratch, h->d_G.p, h->pl.err, s);
  launch_csc_build(h->d_probs.p, h->pl, h->dims, h->d_colptr.p, h->d_cursor.p, h->d_cscrow.p, h->d_cscval2.p, s);
  // residual: rows of A^T, scaled by C; update: Lambda += R * correction
  Pools pa = h->pl;
  pa.rowptr = h->d_colptr.p;
  pa.col = h->d_cscrow.p;
  pa.val2 = h->d_cscval2.p;
  pa.B64 = h->d_G.p;
  pa.rs = h->pl.cs;
  pa.X64 = h->d_lam.p;
  pa.Xs = h->d_lams.p;
  pa.cs = h->pl.rs;
  pa.active = h->d_active.p;
  dfl* D = reinterpret_cast<dfl*>(h->pl.V);
  dfl* envd = reinterpret_cast<dfl*>(h->pl.env64);
  const double tol = h->tol > 0 ? h->tol : 1e-10;
  std::vector<int> active(np, 1), slow(np, 0), m32(np), mdf(np);
  std::vector<double> prev(np, 1e300);
  std::vector<unsigned long long> red(3 * np);
  for (int it = 1; it <= 30; ++it) {
    int n32 = 0, ndf = 0;
    for (int k = 0; k < np; ++k) {
      m32[k] = active[k] && !b.fallback[k];
      mdf[k] = active[k] && b.fallback[k];
      n32 += m32[k];
      ndf += mdf[k];
    }
    if (!n32 && !ndf) break;
    CK(cudaMemcpyAsync(h->d_active.p, active.data(), np * sizeof(int), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(h->d_act_rec.p, m32.data(), np * sizeof(int), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(h->d_act_df.p, mdf.data(), np * sizeof(int), cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(h->pl.dmax, 0, 3 * np * sizeof(unsigned long long), s));
    launch_residual(h->d_probs.p, pa, h->dims, 1, s);
    // FP32 factors (the step launches of a factor kind none of the active
    // problems use are skipped)
    if (n32) {
      launch_forward_t<float>(h->sp, h->pl.env32, h->pl.Y32, h->d_probs.p, h->tb, np, h->d_act_rec.p, s);
      launch_backward_t<float>(h->sp, h->pl.env32, h->pl.Y32, h->d_probs.p, h->tb, np, h->d_act_rec.p, h->pl.piv,
                               s);
      Pools pu = pa;
      pu.active = h->d_act_rec.p;
      launch_update_x(h->d_probs.p, pu, h->dims, 0, s);
    }
    // double-float factors of the escalated problems
    if (ndf) {
      launch_rhs_to_dfl(h->d_probs.p, h->dims, nullptr, h->pl.Y32, h->pl.cs, D, 0, h->d_act_df.p, s);
      launch_forward_t<dfl>(h->sp, envd, D, h->d_probs.p, h->tb, np, h->d_act_df.p, s);
      launch_backward_t<dfl>(h->sp, envd, D, h->d_probs.p, h->tb, np, h->d_act_df.p, h->pl.piv, s);
      launch_dfl_to_x(h->d_probs.p, h->dims, D, h->d_lam.p, h->d_lams.p, h->pl.rs, 0, h->pl.dmax, h->pl.xmax,
                      h->d_act_df.p, s);
    }
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(red.data(), h->d_red.p, 3 * np * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    for (int k = 0; k < np; ++k) {
      if (!active[k]) continue;
      double dm, xm;
      memcpy(&dm, &red[k], 8);
      memcpy(&xm, &red[np + k], 8);
      const double r = xm > 0 ? dm / xm : dm;
      if (!std::isfinite(r) || r <= tol) {
        active[k] = 0;
      } else {
        slow[k] = (it > 1 && r > 0.5 * prev[k]) ? slow[k] + 1 : 0;
        if (slow[k] >= 2) active[k] = 0;
      }
      prev[k] = r;
    }
  }
  return FDMGPU_OK;
}

fdmgpu_status fdmgpu_batch_vjp(fdmgpu_handle* h, const double* gtaull, double* grad_vr, double* ms) {
  if (h && h->batch.chunked) return fail(FDMGPU_ERR_UNSUPPORTED, "vjp of a batch that ran in chunks");
  if (!h || !gtaull || !grad_vr) return fail(FDMGPU_ERR_ARG, "null argument");
  Batch& b = h->batch;
  if (!b.ran) return fail(FDMGPU_ERR_ARG, "vjp needs a batch that has run");
  if (b.cplx == 1) return fail(FDMGPU_ERR_UNSUPPORTED, "vjp of a complex batch (the adjoint is the real-basis one)");
  if (b.sites.size() > 1) return fail(FDMGPU_ERR_UNSUPPORTED, "vjp of a batch over several sites");
  if (b.precision == FDMGPU_PREC_MIXED && (h->refine_gmres || !h->escalate_dfl))
    return fail(FDMGPU_ERR_UNSUPPORTED, "vjp of a mixed batch needs classical or recurrence refinement and "
                                        "double-float escalation");
  const int np = h->dims.nprob;
  for (int k = 0; k < np; ++k) {
    if (b.probs[k].P.nlm_abs <= 0) return fail(FDMGPU_ERR_ARG, "vjp needs an absorber (iaabs > 0) in every energy");
    if (b.err[k]) return fail((fdmgpu_status)b.err[k], "vjp of a batch with a failed energy");
    if (b.precision == FDMGPU_PREC_MIXED && k < (int)b.res64.size() && b.res64[k])
      return fail(FDMGPU_ERR_UNSUPPORTED, "vjp of a mixed batch with an energy re-solved in FP64 (run it in FP64)");
  }
  cudaStream_t s = h->stream;
  int64_t ntaull = 0, nrhs = 0;
  for (auto& hp : b.probs) {
    ntaull = std::max<int64_t>(ntaull, hp.P.taull + (int64_t)hp.P.nlm_abs * hp.P.nlm_abs);
    nrhs = std::max<int64_t>(nrhs, hp.P.rhs + (int64_t)hp.P.nt * hp.P.nrt * TS2);
  }
  const int nspin = std::max(h->g.nspin, 1);
  if (h->d_gT.reserve(ntaull) != cudaSuccess || h->d_lam.reserve(nrhs) != cudaSuccess ||
      h->d_gpart.reserve((size_t)np * std::max(h->S.npr, 1)) != cudaSuccess ||
      h->d_grad.reserve((size_t)h->g.npoint * nspin) != cudaSuccess)
    return fail(FDMGPU_ERR_NOMEM, "device allocation of the adjoint pools failed");
  // per-energy cotangents, concatenated in add order, placed at the Taull offsets
  std::vector<double> gT(ntaull, 0.0);
  int64_t off = 0;
  for (auto& hp : b.probs) {
    const int64_t mm = (int64_t)hp.P.nlm_abs * hp.P.nlm_abs;
    std::copy(gtaull + off, gtaull + off + mm, gT.begin() + hp.P.taull);
    off += mm;
  }
  CK(cudaGetLastError());
  CK(cudaEventRecord(h->ev[0], s));
  CK(cudaMemcpyAsync(h->d_gT.p, gT.data(), ntaull * sizeof(double), cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(h->d_lam.p, 0, nrhs * sizeof(double), s));
  CK(cudaMemsetAsync(h->d_grad.p, 0, (size_t)h->g.npoint * nspin * sizeof(double), s));
  if (b.precision == FDMGPU_PREC_FP64) {
    launch_taull_vjp(h->d_probs.p, h->dims, h->pl.X64, h->d_gT.p, h->pl.tscratch, h->d_lam.p, h->pl.err, s);
    launch_forward_t<double>(h->sp, h->pl.env64, h->d_lam.p, h->d_probs.p, h->tb, np, nullptr, s);
    launch_backward_t<double>(h->sp, h->pl.env64, h->d_lam.p, h->d_probs.p, h->tb, np, nullptr, nullptr, s);
  } else {
    fdmgpu_status st = vjp_mixed(h, nrhs);
    if (st) return st;
  }
  launch_grad_vr(h->S, h->d_probs.p, h->pl.ipool, h->dims, nspin, h->pl.X64, h->d_lam.p, h->d_gpart.p,
                 h->d_grad.p, s);
  CK(cudaGetLastError());
  CK(cudaEventRecord(h->ev[1], s));
  CK(cudaMemcpyAsync(grad_vr, h->d_grad.p, (size_t)h->g.npoint * nspin * sizeof(double), cudaMemcpyDeviceToHost, s));
  std::vector<int> err(np);
  CK(cudaMemcpyAsync(err.data(), h->pl.err, np * sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  float t = 0;
  CK(cudaEventElapsedTime(&t, h->ev[0], h->ev[1]));
  if (ms) *ms = t;
  for (int k = 0; k < np; ++k)
    if (err[k]) return fail((fdmgpu_status)err[k], "singular normalisation matrix in the Taull adjoint");
  b.lam_valid = true;
  return FDMGPU_OK;
}

fdmgpu_status fdmgpu_update_grid_values(fdmgpu_handle* h, const fdmgpu_grid* g) {
  if (!h || !g) return fail(FDMGPU_ERR_ARG, "null argument");
  const fdmgpu_grid& a = h->g;
  if (g->npoint != a.npoint || g->npsom != a.npsom || g->nvois != a.nvois || g->natome != a.natome ||
      g->nbm != a.nbm || g->nbtm != a.nbtm || g->nim != a.nim || g->nsm != a.nsm || g->nsort != a.nsort ||
      g->nsortf != a.nsortf || g->nstm != a.nstm || g->nspin != a.nspin || g->nlmmax != a.nlmmax ||
      g->nlmomax != a.nlmomax || g->nlmsam != a.nlmsam || g->nso1 != a.nso1 || g->ngrph != a.ngrph ||
      g->nspino != a.nspino)
    return fail(FDMGPU_ERR_ARG, "grid sizes differ from the handle's");
  fdmgpu_handle* t = nullptr;
  fdmgpu_status st = fdmgpu_create(g, &t);
  if (st) return st;
  // the integer structure must be the handle's: neighbour kinds and indices,
  // boundary and outer-point tables
  bool same = t->inter_pt_h == h->inter_pt_h && t->nb_kind_h == h->nb_kind_h && t->nb_idx_h == h->nb_idx_h &&
              t->nbordf_h == h->nbordf_h;
  auto same_dev = [&](const DevBuf<int>& x, const DevBuf<int>& y, size_t n) {
    std::vector<int> u(n), v(n);
    if (n == 0) return true;
    if (cudaMemcpy(u.data(), x.p, n * sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(v.data(), y.p, n * sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
      return false;
    return u == v;
  };
  same = same && same_dev(t->d_numia, h->d_numia, a.npsom) && same_dev(t->d_nbord, h->d_nbord, a.natome) &&
         same_dev(t->d_ibord, h->d_ibord, (size_t)a.nbtm * a.natome) && same_dev(t->d_isrt, h->d_isrt, a.nstm) &&
         same_dev(t->d_lato, h->d_lato, (size_t)a.nlmsam * a.natome) &&
         same_dev(t->d_mato, h->d_mato, (size_t)a.nlmsam * a.natome);
  if (!same) {
    fdmgpu_destroy(t);
    return fail(FDMGPU_ERR_ARG, "the grid's integer structure (membership, boundary, neighbours) changed");
  }
  CK(cudaStreamSynchronize(h->stream));
  std::swap(h->d_nb_coef, t->d_nb_coef);
  std::swap(h->d_rvol, t->d_rvol);
  std::swap(h->d_clapl, t->d_clapl);
  std::swap(h->d_poidsa, t->d_poidsa);
  std::swap(h->d_poidso, t->d_poidso);
  std::swap(h->d_Kar, t->d_Kar);
  std::swap(h->d_YsoT, t->d_YsoT);
  std::swap(h->d_Ylmato, t->d_Ylmato);
  h->S.nb_coef = t->S.nb_coef;
  h->S.rvol = t->S.rvol;
  h->S.clapl = t->S.clapl;
  h->S.poidsa = t->S.poidsa;
  h->S.poidso = t->S.poidso;
  h->S.Kar = t->S.Kar;
  h->S.YsoT = t->S.YsoT;
  h->S.Ylmato = t->S.Ylmato;
  h->nb_coef_h.swap(t->nb_coef_h);
  fdmgpu_destroy(t);  // frees the previous value tables
  h->batch.ran = false;  // the batch's factors belong to the previous values
  return FDMGPU_OK;
}

fdmgpu_status fdmgpu_batch_adjoint_dot(fdmgpu_handle* h, const fdmgpu_energy* const* e, int32_t n, double* out) {
  if (h && h->batch.chunked) return fail(FDMGPU_ERR_UNSUPPORTED, "adjoint of a batch that ran in chunks");
  if (!h || !e || !out) return fail(FDMGPU_ERR_ARG, "null argument");
  Batch& b = h->batch;
  const int np = (int)b.probs.size();
  if (!b.lam_valid) return fail(FDMGPU_ERR_ARG, "adjoint_dot needs a vjp of the batch that has run");
  if (b.sites.size() > 1) return fail(FDMGPU_ERR_UNSUPPORTED, "adjoint_dot of a batch over several sites");
  if (n != np) return fail(FDMGPU_ERR_ARG, "one energy argument per batch energy is needed");
  for (int k = 0; k < np; ++k) {
    fdmgpu_status st = check_energy(h, e[k]);
    if (st) return st;
    HostProb hp;
    st = plan_problem(h, e[k], hp);
    if (st) return st;
    const Prob& P0 = b.probs[k].P;
    if (hp.P.n != P0.n || hp.P.nlmso != P0.nlmso || hp.ntiles != b.probs[k].ntiles ||
        hp.J0 != b.probs[k].J0 || hp.J1 != b.probs[k].J1 ||
        (P0.iaabs > 0 && e[k]->ianew[P0.iaabs - 1] != P0.ianew_abs))
      return fail(FDMGPU_ERR_ARG, "energy " + std::to_string(k) + ": row structure differs from the batch's");
  }
  // the new inputs replace the batch's; the solutions X and Lambda stay
  for (int k = 0; k < np; ++k) {
    HostProb hp;
    hp.P = b.probs[k].P;
    pack_inputs(h, e[k], hp);
    if (hp.in_i.size() != b.probs[k].in_i.size() || hp.in_d.size() != b.probs[k].in_d.size() ||
        hp.P.gen != b.probs[k].P.gen)
      return fail(FDMGPU_ERR_ARG, "energy " + std::to_string(k) + ": input sizes differ from the batch's");
    b.probs[k].in_i.swap(hp.in_i);
    b.probs[k].in_d.swap(hp.in_d);
    b.probs[k].P = hp.P;
    b.probs[k].rel_grad = hp.rel_grad;
    b.probs[k].rel_phi = hp.rel_phi;
    b.probs[k].rel_bes = hp.rel_bes;
    b.probs[k].rel_neu = hp.rel_neu;
    b.probs[k].gen_phi = hp.gen_phi;
    b.probs[k].gen_bes = hp.gen_bes;
  }
  b.ran = false;  // the factors are overwritten below; X and Lambda stay valid
  // CSR copy of the new matrices: an FP64 batch plans no CSR, so place it here
  int64_t csr_off = 0;
  for (auto& hp : b.probs) {
    hp.P.csr = csr_off;
    hp.P.csr_cap = hp.nnz_cap;
    csr_off += hp.nnz_cap;
  }
  fdmgpu_status st = upload_inputs(h);
  if (st) return st;
  int64_t env = 0, rhs = 0, rowv = 0, csr = 0;
  for (auto& hp : b.probs) {
    env = std::max<int64_t>(env, (hp.P.env / TS2 + hp.ntiles) * TS2);
    rhs = std::max<int64_t>(rhs, hp.P.rhs + (int64_t)hp.P.nt * hp.P.nrt * TS2);
    rowv = std::max<int64_t>(rowv, hp.P.rowv + (int64_t)hp.P.nt * TS + 1);
    csr = std::max<int64_t>(csr, hp.P.csr + hp.P.csr_cap);
  }
  if (h->d_rowptr.reserve(rowv) != cudaSuccess || h->d_col.reserve(csr) != cudaSuccess ||
      h->d_val.reserve(csr) != cudaSuccess || h->d_val2.reserve(csr) != cudaSuccess ||
      h->d_gpart.reserve((size_t)rowv + np) != cudaSuccess)
    return fail(FDMGPU_ERR_NOMEM, "device allocation of the CSR pools failed");
  Pools pl = h->pl;
  pl.rowptr = h->d_rowptr.p;
  pl.col = h->d_col.p;
  pl.val = h->d_val.p;
  pl.val2 = h->d_val2.p;
  cudaStream_t s = h->stream;
  CK(cudaGetLastError());
  CK(cudaMemsetAsync(pl.env64, 0, env * sizeof(double), s));
  CK(cudaMemsetAsync(pl.B64, 0, rhs * sizeof(double), s));
  CK(cudaMemsetAsync(pl.err, 0, np * sizeof(int), s));
  launch_generate_inputs(h->d_probs.p, h->d_rads.p, h->d_sites.p, h->d_ipool.p, h->dims, h->gdims, h->d_radU.p,
                         h->d_dpool.p, s);
  launch_assemble(h->d_sites.p, h->d_probs.p, pl, h->tb, h->dims, s);
  launch_csr(h->d_probs.p, pl, h->tb, h->dims, s);
  launch_lambda_dot(h->d_probs.p, pl, h->dims, h->d_lam.p, h->d_gpart.p, h->d_gpart.p + rowv, s);
  CK(cudaGetLastError());
  std::vector<int> err(np);
  CK(cudaMemcpyAsync(out, h->d_gpart.p + rowv, np * sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(err.data(), pl.err, np * sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  for (int k = 0; k < np; ++k)
    if (err[k]) return fail((fdmgpu_status)err[k], "assembly of energy " + std::to_string(k) + " failed");
  return FDMGPU_OK;
}

fdmgpu_status fdmgpu_batch_inputs(fdmgpu_handle* h, int32_t k, double* phiato, double* besselr, double* neumanr) {
  if (h && h->batch.chunked) return fail(FDMGPU_ERR_UNSUPPORTED, "a batch that ran in chunks keeps only its Taull (inputs of the last chunk are gone)");
  if (!h) return fail(FDMGPU_ERR_ARG, "null handle");
  Batch& b = h->batch;
  if (k < 0 || k >= (int)b.probs.size() || !b.ran) return fail(FDMGPU_ERR_ARG, "no such energy in the last run");
  const HostProb& hp = b.probs[k];
  if (hp.P.cplx) return fail(FDMGPU_ERR_UNSUPPORTED, "real problems only");
  const fdmgpu_grid& g = b.sites[hp.P.site]->g;
  const size_t nphi = (size_t)g.nbtm * hp.P.nlmagm * g.natome, nb = (size_t)g.nsort * (hp.P.lmaxso + 1);
  cudaStream_t s = h->stream;
  if (phiato) CK(cudaMemcpyAsync(phiato, h->d_dpool.p + hp.P.in_phi, nphi * sizeof(double), cudaMemcpyDeviceToHost, s));
  // [ib][L] on the device -> (nsort, 0:lmaxso) column-major
  std::vector<double> t(nb);
  for (int w = 0; w < 2; ++w) {
    double* out = w == 0 ? besselr : neumanr;
    if (!out) continue;
    CK(cudaMemcpyAsync(t.data(), h->d_dpool.p + (w == 0 ? hp.P.in_bes : hp.P.in_neu), nb * sizeof(double),
                       cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    const int nl = hp.P.lmaxso + 1;
    for (int ib = 0; ib < g.nsort; ++ib)
      for (int L = 0; L < nl; ++L) out[ib + (size_t)g.nsort * L] = t[(size_t)ib * nl + L];
  }
  CK(cudaStreamSynchronize(s));
  return FDMGPU_OK;
}

fdmgpu_status fdmgpu_batch_xanes(fdmgpu_handle* h, const double* energies_ev, const double* half_width,
                                 int32_t width_per_input, const double* weight, double* sigma, double* sigma_conv,
                                 double* tensor) {
  if (!h || !energies_ev || !half_width || !sigma) return fail(FDMGPU_ERR_ARG, "null argument");
  Batch& b = h->batch;
  if (b.chunked) return fail(FDMGPU_ERR_UNSUPPORTED, "cross-section of a batch that ran in chunks");
  const int n = (int)b.probs.size();
  if (!b.ran || n == 0) return fail(FDMGPU_ERR_ARG, "run a batch first");
  if (b.probs[0].P.nlm_abs < 4) return fail(FDMGPU_ERR_ARG, "the absorber needs its p harmonics (lmax >= 1)");
  if (b.cplx == 1 && tensor) return fail(FDMGPU_ERR_UNSUPPORTED, "the Cartesian tensor is formed for real batches only");
  for (auto& hp : b.probs)
    if (hp.P.irr) return fail(FDMGPU_ERR_UNSUPPORTED, "an irregular solution has no Taull (its pair forms Tau_RI)");
  for (int k = 1; k < n; ++k)
    if (!(energies_ev[k] > energies_ev[k - 1])) return fail(FDMGPU_ERR_ARG, "energies must increase, one problem each");
  if (sigma_conv && n < 2) return fail(FDMGPU_ERR_ARG, "the convolution needs two energies");
  // E | width | weight | sigma | conv | tensor
  if (h->d_xs.reserve((size_t)n * 14) != cudaSuccess) return fail(FDMGPU_ERR_NOMEM, "cross-section buffers");
  double* dE = h->d_xs.p;
  double* dW = dE + n;
  double* dw = dW + n;
  double* dS = dw + n;
  double* dC = dS + n;
  double* dT = dC + n;
  cudaStream_t s = h->stream;
  CK(cudaMemcpyAsync(dE, energies_ev, n * sizeof(double), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(dW, half_width, n * sizeof(double), cudaMemcpyHostToDevice, s));
  if (weight) CK(cudaMemcpyAsync(dw, weight, n * sizeof(double), cudaMemcpyHostToDevice, s));
  launch_dipole(h->d_probs.p, h->pl.taull, weight ? dw : nullptr, n, dS, tensor ? dT : nullptr, s);
  if (sigma_conv) launch_lorentz(dE, dS, dW, width_per_input != 0, n, dC, s);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(sigma, dS, n * sizeof(double), cudaMemcpyDeviceToHost, s));
  if (sigma_conv) CK(cudaMemcpyAsync(sigma_conv, dC, n * sizeof(double), cudaMemcpyDeviceToHost, s));
  if (tensor) CK(cudaMemcpyAsync(tensor, dT, 9 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return FDMGPU_OK;
}

fdmgpu_status fdmgpu_taull_noalloc(const double* d_smr, int32_t nlmso, int32_t nligne, int32_t ianew_abs,
                                   int32_t nlm_abs, double* d_taull, int32_t* d_status, void* stream) {
  if (!d_smr || !d_taull) return fail(FDMGPU_ERR_ARG, "null device pointer");
  if (nlmso < 1 || nlm_abs < 1 || nligne < nlmso || ianew_abs < 0 || (int64_t)ianew_abs + nlm_abs > nligne)
    return fail(FDMGPU_ERR_ARG, "inconsistent nlmso / nligne / ianew_abs / nlm_abs");
  if (nlmso > FDMGPU_TAULL_NOALLOC_MAX_NLMSO)
    return fail(FDMGPU_ERR_ARG, "nlmso = " + std::to_string(nlmso) + " exceeds FDMGPU_TAULL_NOALLOC_MAX_NLMSO = " +
                                    std::to_string(FDMGPU_TAULL_NOALLOC_MAX_NLMSO));
  const int64_t need = (int64_t)nlmso * (nlmso + nlm_abs) * 16;
  if (need > FDMGPU_TAULL_NOALLOC_SCRATCH_BYTES)
    return fail(FDMGPU_ERR_ARG, "working matrix of " + std::to_string(need) + " bytes exceeds the " +
                                    std::to_string(FDMGPU_TAULL_NOALLOC_SCRATCH_BYTES) + "-byte static scratch");
  if (reinterpret_cast<uintptr_t>(d_taull) % 16 || reinterpret_cast<uintptr_t>(d_smr) % 8 ||
      reinterpret_cast<uintptr_t>(d_status) % 4)
    return fail(FDMGPU_ERR_ARG, "misaligned device pointer");
  double2* scratch = nullptr;
  CK(taull_noalloc_scratch(&scratch));
  CK(launch_taull_noalloc(d_smr, nlmso, nligne, ianew_abs, nlm_abs, scratch, d_taull, d_status,
                          static_cast<cudaStream_t>(stream)));
  return FDMGPU_OK;
}

}  // extern "C"
