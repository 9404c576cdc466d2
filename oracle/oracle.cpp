// oracle.cpp - CPU restatement of the FDMNES FDM assembly + Gaussian solve.
//
// TEST INFRASTRUCTURE ONLY.  This file is the CPU model that the GPU path is
// compared against; nothing in the product links, imports or calls it.  Only
// tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
//
// Parity status: the reference is Fortran and no Fortran compiler exists on
// either machine, and the reference ships no tests or golden outputs, so this
// restatement could not be compared with reference-produced numbers ("parity
// unpinned" against the reference binary).  It is pinned instead by
// known-answer tests: closed-form Bessel functions and harmonics, the exact
// stencil coefficients, a dense LU solve of the same assembled matrix, and
// the free-space answer of the whole system (a transparent absorber - flat
// potential, free-space j_l as its boundary functions - scatters nothing, up
// to the fourth-order stencil's error).
//
// Restated routines (real-arithmetic path: Cal_comp = E_comp = Spinorbite =
// Relativiste = Repres_comp = Ylm_comp = irregular = false, nspino = 1):
//   calcMatRow           source/mat.f90:1034-1632
//   mat_solve (Gaussian) source/mat_solve_gaussian.f90:5-372, operation order kept
//   newind               source/mat.f90:1761-1921
//   cbessneur            source/sphere.f90:7356-7384
//   invcomp -> zgetrf/zgetri  source/mat.f90:1927-1992, source/sub_util.f:11149,11382
//   Taull assembly       source/mat.f90:306-405 and symmetrisation :598-644
// The arguments are the mat_solve argument structs of include/fdmgpu.h, which
// restate the reference's Fortran argument list (column-major, 1-based values).

#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <chrono>

#include "../include/fdmgpu.h"

#include "oracle_ctx.h"

namespace {

using namespace oracle;

// One row of the matrix (abvr over lb1..lb2, stored at abvr[k - lb1]) and the
// right-hand side smr(:, ii).  Real path of calcMatRow, source/mat.f90:1034-1632.
void calc_mat_row(const Ctx& c, int ii, double* abvr, int lb1, double* smr_col) {
  const fdmgpu_grid* g = c.g;
  const fdmgpu_energy* e = c.e;
  const int nspino = c.nspino;
  const int i = e->newinv[ii - 1];
  const int nspin = g->nspin;
  const int ispin = c.ispin;
  auto A = [&](int col) -> double& { return abvr[col - lb1]; };
  if (i > 0) {
    // grid point rows (mat.f90:1142-1402)
    const int ispp = std::min(ispin, nspin);
    const int isp = std::min(ispin, nspino);
    const double VmE = e->Vr[(i - 1) + (int64_t)g->npoint * (ispp - 1)] - e->Enervide;
    A(ii) = VmE - g->clapl[0];
    for (int iv = 1; iv <= g->nvois; ++iv) {
      const int j = c.ivois(i, iv);
      const int ia = g->numia[j - 1];
      double cfvs_r = -g->clapl[iv];
      const double charac_r = c.Kar(std::abs(c.isvois(i, iv)), 1);
      cfvs_r = charac_r * cfvs_r;
      cfvs_r = cfvs_r * g->rvol[i - 1];
      if (ia == 0) {
        const int jj = e->new_[j] - nspino + isp;
        A(jj) = A(jj) + cfvs_r / g->rvol[j - 1];
      } else if (ia > 0) {
        int ib;
        for (ib = g->nbordf[ia - 1] + 1; ib <= g->nbord[ia - 1]; ++ib)
          if (j == c.ibord(ib, ia)) break;
        const int isym = std::abs(c.isbord(ib, ia));
        if (isym != 1) cfvs_r = c.Kar(isym, 1) * cfvs_r;
        for (int Lm = 1; Lm <= e->nlmsa[ia - 1]; ++Lm) {
          const int jjj = e->ianew[ia - 1] + Lm;
          const int L = Lato(c, Lm, ia);
          const int isol = Iato(c, Lm, ia);
          for (int ispo = 1; ispo <= nspino; ++ispo) {
            const int m = Mato(c, Lm, ia) + ispo - isol;
            if (m > L || m < -L) continue;
            const int Lm0 = L * L + L + 1 + m;
            A(jjj) = A(jjj) + cfvs_r * Phiato(c, ib, Lm0, ispp, isol, 1, ia);
          }
        }
      } else if (ia == -2) {
        int ib;
        for (ib = g->nsortf + 1; ib <= g->nsort; ++ib)
          if (j == g->isrt[ib - 1]) break;
        for (int Lm = 1; Lm <= e->nlmso; ++Lm) {
          const int L = Lso(c, Lm), m = Mso(c, Lm);
          const int Lm0 = L * L + L + 1 + m;
          const int ispq = std::min(Iso(c, Lm), e->nspinr);
          const int jjj = e->nligneso + Lm;
          const double fr = c.Ylmso(ib, Lm0) * Bes(c, e->Neumanr, ib, L, ispq);
          A(jjj) = A(jjj) + cfvs_r * fr;
        }
        for (int Lm = 1; Lm <= e->nlmso; ++Lm) {
          const int L = Lso(c, Lm), m = Mso(c, Lm);
          const int Lm0 = L * L + L + 1 + m;
          const int ispq = std::min(Iso(c, Lm), e->nspinr);
          const double fr = c.Ylmso(ib, Lm0) * Bes(c, e->Besselr, ib, L, ispq);
          smr_col[Lm - 1] = smr_col[Lm - 1] - cfvs_r * fr;
        }
      }
    }
  } else if (i == 0) {
    // outer sphere rows (mat.f90:1405-1511)
    const int Lm = ii - e->nligneso;
    const int m = Mso(c, Lm);
    const int Lm0 = Lso(c, Lm) * Lso(c, Lm) + Lso(c, Lm) + 1 + m;
    const int isp = Iso(c, Lm);
    for (int Lmp = 1; Lmp <= e->nlmso; ++Lmp) {
      if (Iso(c, Lmp) != isp) continue;
      const int L = Lso(c, Lmp);
      const int mp = Mso(c, Lmp);
      const int lmp0 = L * L + L + 1 + mp;
      const int ispq = std::min(Iso(c, Lmp), e->nspinr);
      const int ljj = e->nligneso + Lmp;
      double charmr = 0.0;
      for (int ib = 1; ib <= g->nsortf; ++ib) {
        const double fac = g->poidso[ib - 1] * c.Ylmso(ib, Lm0) * c.Ylmso(ib, lmp0);
        charmr = charmr + fac * Bes(c, e->Neumanr, ib, L, ispq);
      }
      A(ljj) = A(ljj) + charmr;
    }
    for (int ib = 1; ib <= g->nsortf; ++ib) {
      const int j = g->isrt[ib - 1];
      const int jj = e->new_[j] - nspino + isp;
      const double fac = g->poidso[ib - 1] * c.Ylmso(ib, Lm0);
      A(jj) = A(jj) - fac / g->rvol[j - 1];
      for (int Lmf = 1; Lmf <= e->nlmso; ++Lmf) {
        const int ispq = std::min(Iso(c, Lmf), e->nspinr);
        if (isp != Iso(c, Lmf)) continue;
        const int L = Lso(c, Lmf);
        const int mf = Mso(c, Lmf);
        const int lmf0 = L * L + L + 1 + mf;
        const double fad = fac * c.Ylmso(ib, lmf0);
        smr_col[Lmf - 1] = smr_col[Lmf - 1] - fad * Bes(c, e->Besselr, ib, L, ispq);
      }
    }
  } else {
    // atom expansion rows (mat.f90:1515-1632), regular solution only
    const int ia = -i;
    const int Lm = ii - e->ianew[ia - 1];
    const int L = Lato(c, Lm, ia);
    const int ispt = Iato(c, Lm, ia);
    const int m = Mato(c, Lm, ia);
    const int Lm0 = L * L + L + 1 + m;
    for (int ib = 1; ib <= g->nbordf[ia - 1]; ++ib) {
      const int j = c.ibord(ib, ia);
      const int isym = std::abs(c.isbord(ib, ia));
      const int jj = e->new_[j] - nspino + ispt;
      const double f = c.poidsa(ib, ia) * c.Kar(isym, ispt) / g->rvol[j - 1];
      A(jj) = A(jj) - f * Ylmato(c, ib, Lm0, ia);
    }
    for (int Lmp = 1; Lmp <= e->nlmsa[ia - 1]; ++Lmp) {
      const int Lp = Lato(c, Lmp, ia);
      const int isol = Iato(c, Lmp, ia);
      const int mp = Mato(c, Lmp, ia) + ispt - isol;
      if (mp > Lp || mp < -Lp) continue;
      const int Lmp0 = Lp * Lp + Lp + 1 + mp;
      const int ispint = std::min(ispin, e->nspinp);
      double charmr = 0.0;
      for (int ib = 1; ib <= g->nbordf[ia - 1]; ++ib)
        charmr = charmr + c.poidsa(ib, ia) * Ylmato(c, ib, Lm0, ia) * Phiato(c, ib, Lmp0, ispint, isol, 1, ia);
      const int ljj = e->ianew[ia - 1] + Lmp;
      A(ljj) = A(ljj) + charmr;
    }
  }
}

int check_supported(const fdmgpu_grid* g, const fdmgpu_energy* e) {
  if (e->Cal_comp || e->E_comp || e->Spinorbite || e->Relativiste || e->Repres_comp || e->Ylm_comp ||
      e->irregular || e->Base_hexa || g->nspino != 1 || e->n_ato_RI != 1 || e->nphiato7 != 1)
    return FDMGPU_ERR_UNSUPPORTED;
  return FDMGPU_OK;
}

}  // namespace

namespace oracle {

int64_t symbolic_profile(const Ctx& c, std::vector<int32_t>& ind, std::vector<int32_t>& nb_not_zero,
                         std::vector<int64_t>& lbz) {
  const fdmgpu_grid* g = c.g;
  const fdmgpu_energy* e = c.e;
  const int nligne = e->nligne, nlmso = e->nlmso, nspino = g->nspino;
  const int nligneso = e->nligneso;
  const int* newinv = e->newinv;
  const int* new_ = e->new_;
  std::vector<char> colnz(nligne + 1, 0);
  nb_not_zero.assign(nligne + 1, 0);
  lbz.assign(nligne + 1, 0);
  std::vector<int32_t> ind_inv;
  int64_t nb_tot = 0;
  for (int pass = 1; pass <= 2; ++pass) {
    const bool second = pass == 2;
    if (second) ind_inv.assign(nb_tot, 0);
    nb_tot = 0;
    std::fill(colnz.begin(), colnz.end(), 0);
    std::fill(nb_not_zero.begin(), nb_not_zero.end(), 0);
    for (int ii = nligne; ii >= 1; --ii) {
      const int i = newinv[ii - 1];
      if (i > 0) {
        for (int iv = 1; iv <= g->nvois; ++iv) {
          const int j = c.ivois(i, iv);
          const int ia = g->numia[j - 1];
          if (ia == 0) {
            for (int k = new_[j] - nspino + 1; k <= new_[j]; ++k) colnz[k] = 1;
          } else if (ia > 0) {
            for (int k = e->ianew[ia - 1] + 1; k <= e->ianew[ia - 1] + e->n_ato_RI * e->nlmsa[ia - 1]; ++k) colnz[k] = 1;
          } else if (ia == -2 && !e->irregular) {
            for (int k = nligneso + 1; k <= nligneso + nlmso; ++k) colnz[k] = 1;
          }
        }
      } else if (i == 0) {
        if (!e->irregular) {
          for (int k = nligneso + 1; k <= nligneso + nlmso; ++k) colnz[k] = 1;
          const int lm = ii - nligneso;
          const int isp = Iso(c, lm);
          for (int ib = 1; ib <= g->nsortf; ++ib) {
            const int j = g->isrt[ib - 1];
            colnz[new_[j] - nspino + isp] = 1;
          }
        }
      } else {
        const int ia = -i;
        for (int k = e->ianew[ia - 1] + 1; k <= e->ianew[ia - 1] + e->n_ato_RI * e->nlmsa[ia - 1]; ++k) colnz[k] = 1;
        int lm = ii - e->ianew[ia - 1];
        if (lm > e->nlmsa[ia - 1]) lm -= e->nlmsa[ia - 1];
        const int isp = Iato(c, lm, ia);
        for (int ib = 1; ib <= g->nbordf[ia - 1]; ++ib) {
          const int j = c.ibord(ib, ia);
          colnz[new_[j] - nspino + isp] = 1;
        }
      }
      for (int j = ii - 1; j >= 1; --j) {
        if (!colnz[j]) continue;
        ++nb_tot;
        if (second) {
          nb_not_zero[ii] += 1;
          ind_inv[nb_tot - 1] = j;
        }
      }
    }
  }
  ind.assign(nb_tot, 0);
  for (int64_t lk = 1; lk <= nb_tot; ++lk) ind[lk - 1] = ind_inv[nb_tot + 1 - lk - 1];
  ind_inv.clear();
  lbz[1] = 0;
  for (int ii = 2; ii <= nligne; ++ii) lbz[ii] = lbz[ii - 1] + nb_not_zero[ii - 1];
  return nb_tot;
}

}  // namespace oracle

extern "C" {

// Dense assembly of A (nligne x nligne, column-major) and B = smr (nlmso x nligne),
// row by row with calcMatRow.  Used by the dense-LU known-answer test.
int oracle_assemble_dense(const fdmgpu_grid* g, const fdmgpu_energy* e, double* A, double* smr) {
  int st = check_supported(g, e);
  if (st) return st;
  Ctx c = make_ctx(g, e);
  const int n = e->nligne;
  std::vector<double> row;
  for (int ii = 1; ii <= n; ++ii) {
    const int l1 = e->lb1[ii - 1], l2 = e->lb2[ii - 1];
    row.assign(l2 - l1 + 1, 0.0);
    calc_mat_row(c, ii, row.data(), l1, smr + (int64_t)(ii - 1) * e->nlmso);
    for (int k = l1; k <= l2; ++k) A[(int64_t)(ii - 1) + (int64_t)(k - 1) * n] = row[k - l1];
  }
  return 0;
}

// Sparse assembly: the nonzeros of A in CSR form (rows ii = 1..nligne in
// order, 0-based columns) and B = smr (nlmso x nligne), with calcMatRow.  With
// colidx == nullptr only the row pointers are written (rowptr[nligne] = nnz),
// so the caller can size the arrays.  Used by the backward-error checks of
// problems too large for a dense copy.
int oracle_assemble_csr(const fdmgpu_grid* g, const fdmgpu_energy* e, int64_t* rowptr, int32_t* colidx, double* val,
                        double* smr) {
  int st = check_supported(g, e);
  if (st) return st;
  Ctx c = make_ctx(g, e);
  const int n = e->nligne;
  std::vector<double> row;
  std::vector<double> brow(e->nlmso);
  rowptr[0] = 0;
  for (int ii = 1; ii <= n; ++ii) {
    const int l1 = e->lb1[ii - 1], l2 = e->lb2[ii - 1];
    row.assign(l2 - l1 + 1, 0.0);
    double* b = smr ? smr + (int64_t)(ii - 1) * e->nlmso : brow.data();
    calc_mat_row(c, ii, row.data(), l1, b);
    int64_t q = rowptr[ii - 1];
    for (int k = l1; k <= l2; ++k) {
      if (row[k - l1] == 0.0) continue;
      if (colidx) {
        colidx[q] = k - 1;
        val[q] = row[k - l1];
      }
      ++q;
    }
    rowptr[ii] = q;
  }
  return 0;
}

// Gaussian profile solve, source/mat_solve_gaussian.f90:5-372 (real branch).
// smr (nlmso, nligne) is zero on entry and holds the solution on return.
int oracle_mat_solve(const fdmgpu_grid* g, const fdmgpu_energy* e, double* smr, int64_t* nnz_out,
                     double* time_fill, double* time_tria, int32_t* bad_row) {
  int st = check_supported(g, e);
  if (st) return st;
  Ctx c = make_ctx(g, e);
  const int nligne = e->nligne, nlmso = e->nlmso;
  std::vector<int32_t> ind, nb_not_zero;
  std::vector<int64_t> lbz;
  const int64_t nb_tot = symbolic_profile(c, ind, nb_not_zero, lbz);
  if (nnz_out) *nnz_out = nb_tot;

  // Filling, elimination and normalisation (:177-317).
  std::vector<double> abr(nb_tot, 0.0);
  std::vector<double> abvr;
  const double eps15 = 1e-15;
  double tfill = 0, ttria = 0;
  for (int ii = nligne; ii >= 1; --ii) {
    auto t0 = std::chrono::steady_clock::now();
    const int lb1r = e->lb1[ii - 1], lb2r = e->lb2[ii - 1];
    abvr.assign(lb2r - lb1r + 1, 0.0);
    double* smr_ii = smr + (int64_t)(ii - 1) * nlmso;
    calc_mat_row(c, ii, abvr.data(), lb1r, smr_ii);
    auto t1 = std::chrono::steady_clock::now();
    for (int j = lb2r; j >= ii + 1; --j) {
      const double fac = abvr[j - lb1r];
      if (std::fabs(fac) > eps15) {
        const int64_t b = lbz[j], nz = nb_not_zero[j];
        for (int64_t lk = b; lk < b + nz; ++lk) {
          const int k = ind[lk];
          abvr[k - lb1r] = abvr[k - lb1r] - fac * abr[lk];
        }
        const double* smr_j = smr + (int64_t)(j - 1) * nlmso;
        for (int l = 0; l < nlmso; ++l) smr_ii[l] = smr_ii[l] - fac * smr_j[l];
      }
    }
    if (std::fabs(abvr[ii - lb1r]) < 1e-10) {
      if (bad_row) *bad_row = ii;
      return FDMGPU_ERR_ZERO_PIVOT;
    }
    const double vnormalr = 1.0 / abvr[ii - lb1r];
    {
      const int64_t b = lbz[ii], nz = nb_not_zero[ii];
      for (int64_t lk = b; lk < b + nz; ++lk) abr[lk] = abvr[ind[lk] - lb1r] * vnormalr;
    }
    for (int l = 0; l < nlmso; ++l) smr_ii[l] = smr_ii[l] * vnormalr;
    auto t2 = std::chrono::steady_clock::now();
    tfill += std::chrono::duration<double>(t1 - t0).count();
    ttria += std::chrono::duration<double>(t2 - t1).count();
  }
  // Resolution (:348-358).
  for (int ii = 2; ii <= nligne; ++ii) {
    double* smr_ii = smr + (int64_t)(ii - 1) * nlmso;
    const int64_t b = lbz[ii], nz = nb_not_zero[ii];
    for (int64_t lk = b; lk < b + nz; ++lk) {
      const int j = ind[lk];
      const double a = abr[lk];
      const double* smr_j = smr + (int64_t)(j - 1) * nlmso;
      for (int l = 0; l < nlmso; ++l) smr_ii[l] = smr_ii[l] - a * smr_j[l];
    }
  }
  if (time_fill) *time_fill += tfill;
  if (time_tria) *time_tria += ttria;
  return 0;
}

// newind, source/mat.f90:1761-1921, nspino 1 or 2: the regular solution
// (n_ato_RI = 1), or with irregular != 0 FDM_comp's irregular one with both
// atomic solutions (n_ato_RI = 2, no outer-sphere rows, :1862).
// xyz4: (npsom) distance of each point; new_ has npoint+1 entries (index 0..npoint).
static int newind_rows(const fdmgpu_grid* g, const double* xyz4, const double* distai, const int32_t* nlmsa,
                       int nlmso, int32_t nligne, int irregular, int32_t* new_, int32_t* newinv, int32_t* ianew,
                       int32_t* lb1, int32_t* lb2) {
  const int npoint = g->npoint, natome = g->natome, nspino = g->nspino, n_ato_RI = irregular ? 2 : 1;
  int ii = 0;
  new_[0] = 0;
  for (int i = 1; i <= npoint; ++i) {
    if (g->numia[i - 1] == 0) { ii += nspino; new_[i] = ii; } else new_[i] = 0;
  }
  int npf = 1, npf1 = 0;
  for (int ia = 1; ia <= natome; ++ia) {
    int i;
    for (i = npf; i <= npoint; ++i)
      if (g->numia[i - 1] == 0 && xyz4[i - 1] >= distai[ia - 1]) break;
    npf = i;
    if (npf1 == npf) ianew[ia - 1] = ianew[ia - 2] + n_ato_RI * nlmsa[ia - 2];
    else ianew[ia - 1] = new_[npf] - nspino;
    npf1 = npf;
    for (i = npf; i <= npoint; ++i)
      if (g->numia[i - 1] == 0) new_[i] += n_ato_RI * nlmsa[ia - 1];
  }
  for (int r = 1; r <= nligne; ++r) { lb1[r - 1] = r; lb2[r - 1] = r; }
  const int n = nspino - 1;
  I2 ivois{g->ivois, g->npsom};
  for (int i = 1; i <= npoint; ++i) {
    if (g->numia[i - 1] != 0) continue;
    const int r = new_[i];
    for (int iv = 1; iv <= g->nvois; ++iv) {
      const int j = ivois(i, iv);
      if (j == 0) return FDMGPU_ERR_ARG;
      const int ia = g->numia[j - 1];
      if (ia == 0) {
        lb1[r - 1] = std::min(lb1[r - 1], new_[j] - n);
        lb2[r - 1] = std::max(lb2[r - 1], new_[j]);
      } else if (ia > 0) {
        lb1[r - 1] = std::min(lb1[r - 1], ianew[ia - 1] + 1);
        lb2[r - 1] = std::max(lb2[r - 1], ianew[ia - 1] + n_ato_RI * nlmsa[ia - 1]);
      } else if (ia == -2) {
        lb2[r - 1] = nligne;
      }
    }
    if (nspino == 2) {  // the point's spin-1 row has the same span (mat.f90:1841-1844)
      lb1[r - 2] = lb1[r - 1];
      lb2[r - 2] = lb2[r - 1];
    }
  }
  I2 ibord{g->ibord, g->nbtm};
  for (int ia = 1; ia <= natome; ++ia) {
    int lb11 = ianew[ia - 1] + 1, lb22 = ianew[ia - 1] + n_ato_RI * nlmsa[ia - 1];
    for (int ib = 1; ib <= g->nbordf[ia - 1]; ++ib) {
      lb11 = std::min(lb11, new_[ibord(ib, ia)] - n);
      lb22 = std::max(lb22, new_[ibord(ib, ia)]);
    }
    for (int L = 1; L <= n_ato_RI * nlmsa[ia - 1]; ++L) {
      lb1[ianew[ia - 1] + L - 1] = lb11;
      lb2[ianew[ia - 1] + L - 1] = lb22;
    }
  }
  if (!irregular) {
    int lb11 = nligne - nlmso + 1;
    for (int ib = 1; ib <= g->nsortf; ++ib) lb11 = std::min(lb11, new_[g->isrt[ib - 1]] - n);
    for (int r = nligne - nlmso + 1; r <= nligne; ++r) { lb1[r - 1] = lb11; lb2[r - 1] = nligne; }
  }
  for (int r = nligne - 1; r >= 1; --r) lb1[r - 1] = std::min(lb1[r - 1], lb1[r]);
  for (int r = 0; r < nligne; ++r) newinv[r] = 0;
  for (int i = 1; i <= npoint; ++i) {
    const int r = new_[i];
    if (r != 0) {
      newinv[r - 1] = i;
      if (nspino == 2) newinv[r - 2] = i;
    }
  }
  for (int ia = 1; ia <= natome; ++ia)
    for (int Lm = 1; Lm <= n_ato_RI * nlmsa[ia - 1]; ++Lm) newinv[ianew[ia - 1] + Lm - 1] = -ia;
  return 0;
}

int oracle_newind(const fdmgpu_grid* g, const double* xyz4, const double* distai, const int32_t* nlmsa, int nlmso,
                  int32_t nligne, int32_t* new_, int32_t* newinv, int32_t* ianew, int32_t* lb1, int32_t* lb2) {
  return newind_rows(g, xyz4, distai, nlmsa, nlmso, nligne, 0, new_, newinv, ianew, lb1, lb2);
}

int oracle_newind_irregular(const fdmgpu_grid* g, const double* xyz4, const double* distai, const int32_t* nlmsa,
                            int32_t nligne, int32_t* new_, int32_t* newinv, int32_t* ianew, int32_t* lb1,
                            int32_t* lb2) {
  return newind_rows(g, xyz4, distai, nlmsa, 0, nligne, 1, new_, newinv, ianew, lb1, lb2);
}

// cbessneur, source/sphere.f90:7356-7384: fnorm*j_l(z), fnorm*n_l(z), l = 0..lmax.
void oracle_cbessneur(double fnorm, double z, int lmax, double* bessel, double* neuman) {
  neuman[0] = -fnorm * std::cos(z) / z;
  bessel[0] = fnorm * std::sin(z) / z;
  if (lmax == 0) return;
  neuman[1] = neuman[0] / z - bessel[0];
  bessel[1] = bessel[0] / z + neuman[0];
  for (int L = 2; L <= lmax; ++L) {
    const int L1 = 2 * L - 1;
    neuman[L] = L1 * neuman[L - 1] / z - neuman[L - 2];
    bessel[L] = L1 * bessel[L - 1] / z - bessel[L - 2];
  }
}

// invcomp with is = 0 (source/mat.f90:1927-1992): zgetrf (partial pivoting on
// |re|+|im|, source/sub_util.f:11149) followed by the inverse (zgetri,
// source/sub_util.f:11382), restated as an LU solve against the identity.
// a: (n, n) complex column-major, interleaved; overwritten by its inverse.
int oracle_invcomp(int n, double* a_ri) {
  cdouble* a = reinterpret_cast<cdouble*>(a_ri);
  std::vector<int> piv(n);
  auto A = [&](int i, int j) -> cdouble& { return a[i + (int64_t)j * n]; };
  for (int k = 0; k < n; ++k) {
    int p = k;
    double best = -1;
    for (int i = k; i < n; ++i) {
      const double v = std::fabs(A(i, k).real()) + std::fabs(A(i, k).imag());
      if (v > best) { best = v; p = i; }
    }
    piv[k] = p;
    if (best == 0.0) return FDMGPU_ERR_ZERO_PIVOT;
    if (p != k)
      for (int j = 0; j < n; ++j) std::swap(A(k, j), A(p, j));
    const cdouble inv = 1.0 / A(k, k);
    for (int i = k + 1; i < n; ++i) A(i, k) *= inv;
    for (int j = k + 1; j < n; ++j) {
      const cdouble u = A(k, j);
      if (u == 0.0) continue;
      for (int i = k + 1; i < n; ++i) A(i, j) -= A(i, k) * u;
    }
  }
  std::vector<cdouble> inv((size_t)n * n);
  std::vector<cdouble> x(n);
  for (int col = 0; col < n; ++col) {
    for (int i = 0; i < n; ++i) x[i] = 0.0;
    x[col] = 1.0;
    for (int k = 0; k < n; ++k) std::swap(x[k], x[piv[k]]);
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < i; ++k) x[i] -= A(i, k) * x[k];
    for (int i = n - 1; i >= 0; --i) {
      for (int k = i + 1; k < n; ++k) x[i] -= A(i, k) * x[k];
      x[i] /= A(i, i);
    }
    for (int i = 0; i < n; ++i) inv[i + (int64_t)col * n] = x[i];
  }
  for (size_t q = 0; q < inv.size(); ++q) a[q] = inv[q];
  return 0;
}

// Taull of the absorbing atom from the solution, real-basis case
// (source/mat.f90:306-405, FDM_comp false) followed by the symmetrisation
// Taull = i*Im(Taull) of the non spin-orbit real-harmonics case (:598-644).
// smr: (nlmso, nligne) solution.  taull: (nlm, nlm) complex interleaved,
// indexed by Lm0 = L^2+L+1+m of each harmonic.  Returns nlm in *nlm_out.
int oracle_taull(const fdmgpu_grid* g, const fdmgpu_energy* e, int iaabs, const double* smr, double* taull,
                 int32_t* nlm_out) {
  Ctx c = make_ctx(g, e);
  const int nlmso = e->nlmso, nligneso = e->nligneso;
  std::vector<cdouble> norm((size_t)nlmso * nlmso);
  for (int Lm = 1; Lm <= nlmso; ++Lm) {
    const int ii = nligneso + Lm;
    for (int Lm2 = 1; Lm2 <= nlmso; ++Lm2)
      norm[(Lm2 - 1) + (int64_t)(Lm - 1) * nlmso] = cdouble(0.0, smr[(Lm2 - 1) + (int64_t)(ii - 1) * nlmso]);
  }
  for (int Lm = 1; Lm <= nlmso; ++Lm) norm[(Lm - 1) + (int64_t)(Lm - 1) * nlmso] += 1.0;
  int st = oracle_invcomp(nlmso, reinterpret_cast<double*>(norm.data()));
  if (st) return st;
  // norm_t = transpose(norm): ampl(Lmf) = sum_k norm_t(k, Lmf) * smr(k, ii) = sum_k norm(Lmf, k) smr(k, ii)
  const int ia = iaabs;
  const int nlm = e->nlmsa[ia - 1];
  int lmax = 0;
  for (int Lm = 1; Lm <= nlm; ++Lm) lmax = std::max(lmax, Lato(c, Lm, ia));
  const int nlmq = (lmax + 1) * (lmax + 1);
  std::vector<cdouble> T((size_t)nlmq * nlmq, 0.0);
  std::vector<cdouble> ampl((size_t)nlmso * nlm);
  for (int Lm1 = 1; Lm1 <= nlm; ++Lm1) {
    const int ii = e->ianew[ia - 1] + Lm1;
    for (int Lmf = 1; Lmf <= nlmso; ++Lmf) {
      cdouble s = 0.0;
      for (int k = 1; k <= nlmso; ++k)
        s += norm[(Lmf - 1) + (int64_t)(k - 1) * nlmso] * smr[(k - 1) + (int64_t)(ii - 1) * nlmso];
      ampl[(Lmf - 1) + (int64_t)(Lm1 - 1) * nlmso] = s;
    }
  }
  const cdouble img(0.0, 1.0);
  for (int Lm1 = 1; Lm1 <= nlm; ++Lm1) {
    const int L1 = Lato(c, Lm1, ia), m1 = Mato(c, Lm1, ia);
    const int Lm01 = L1 * L1 + L1 + 1 + m1;
    for (int Lm2 = 1; Lm2 <= nlm; ++Lm2) {
      const int L2 = Lato(c, Lm2, ia), m2 = Mato(c, Lm2, ia);
      const int Lm02 = L2 * L2 + L2 + 1 + m2;
      cdouble cfac = 0.0;
      for (int Lmf = 1; Lmf <= nlmso; ++Lmf) {
        const cdouble a1 = ampl[(Lmf - 1) + (int64_t)(Lm1 - 1) * nlmso];
        const cdouble a2 = ampl[(Lmf - 1) + (int64_t)(Lm2 - 1) * nlmso];
        cfac = cfac - img * a1 * std::conj(a2);
      }
      T[(Lm01 - 1) + (int64_t)(Lm02 - 1) * nlmq] += cfac;
    }
  }
  for (auto& t : T) t = cdouble(0.0, t.imag());
  std::memcpy(taull, T.data(), sizeof(cdouble) * T.size());
  if (nlm_out) *nlm_out = nlmq;
  return 0;
}

}  // extern "C"
