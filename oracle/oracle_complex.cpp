// oracle_complex.cpp - CPU restatement of the complex (Cal_comp) branch of the
// FDMNES FDM assembly and Gaussian solve.
//
// TEST INFRASTRUCTURE ONLY, like oracle.cpp: compared against, never part of the product.
//
// Parity status: unpinned against the reference binary (no Fortran compiler
// on either machine); pinned by known-answer tests instead: a dense complex
// LU solve of the same assembled matrix, the reduction of the complex
// machinery to the real branch, the equality of the complex-basis Taull with
// the renormalised real-basis Taull, the decoupling of the spin-orbit system
// into two spin copies when the coupling vanishes, and the unitary relation
// between the complex- and real-harmonic Taull.
//
// Restated (Cal_comp = true; Repres_comp = Base_hexa = false; the regular
// solution, and the irregular solution of FDM_comp with Test_reg = 0, i.e.
// n_RI = n_ato_RI = 2):
//   calcMatRow, complex branch        source/mat.f90:1034-1632
//     grid rows with the relativistic and spin-orbit gradient terms :1142-1402
//       (irregular: both atom-solution columns, no outer-sphere columns,
//       right-hand side from -i j_l + n_l, :1266-1369)
//     outer-sphere rows (regular solution only)                     :1405-1511
//     atom rows (irregular: the boundary points split in halves)    :1515-1632
//   Tau_RI, the regular x irregular amplitude products   source/mat.f90:219-292
//   Yc (complex harmonic from two real ones)  source/mat.f90:1733-1754
//   cbessneu (complex-argument j_l, n_l)       source/sphere.f90:7226-7254
//   mat_solve (Gaussian), complex branch       source/mat_solve_gaussian.f90:196-358
//   Taull of the complex basis                 source/mat.f90:354-405 (Basereel false)
//     and the symmetrisation                   source/mat.f90:594-644
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "oracle_ctx.h"

namespace {

using namespace oracle;

const cdouble img(0.0, 1.0);
// Physical constants of source/main.f90:58,76.
const double alfa_sf = 0.0072973525664;   // fine-structure constant (CODATA 2014)
const double sqrt_1o2 = 1.0 / std::sqrt(2.0);

// Yc, source/mat.f90:1733-1754: complex harmonic of order m from the real
// harmonics of orders m (y1) and -m (y2).
cdouble Yc(int m, double y1, double y2) {
  if (m == 0) return cdouble(y1, 0.0);
  if (m < 0) return cdouble(y2, -y1) * sqrt_1o2;
  const double sgn = (m % 2 == 0) ? 1.0 : -1.0;
  return cdouble(y1, y2) * sgn * sqrt_1o2;
}

// phiato(ib, Lm, isp, isol, i_RI, ia, 1 + part): part 0 real, 1 imaginary;
// i_RI 1 the regular, 2 the irregular atomic solution.
double PhiatoPart(const Ctx& c, int ib, int lm, int isp, int isol, int ia, int part, int iri = 1) {
  const fdmgpu_energy* e = c.e;
  const int64_t d1 = e->nphiato1, d2 = e->nlmagm, d3 = e->nspinp, d4 = c.nspino, d5 = e->n_RI;
  const int64_t d6 = c.g->natome;
  const int64_t off = (ib - 1) + d1 * ((lm - 1) + d2 * ((isp - 1) + d3 * ((isol - 1) + d4 * ((iri - 1) + d5 * ((ia - 1) +
                      d6 * part)))));
  return e->phiato[off];
}
cdouble PhiatoC(const Ctx& c, int ib, int lm, int isp, int isol, int ia, int iri = 1) {
  if (c.e->nphiato7 == 2)
    return cdouble(PhiatoPart(c, ib, lm, isp, isol, ia, 0, iri), PhiatoPart(c, ib, lm, isp, isol, ia, 1, iri));
  return cdouble(PhiatoPart(c, ib, lm, isp, isol, ia, 0, iri), 0.0);
}
// Complex Bessel / Neuman (2, nsort_c, 0:lmaxso, nspinr), interleaved.
cdouble BesC(const Ctx& c, const double* a, int ib, int L, int isp) {
  const fdmgpu_energy* e = c.e;
  const int64_t off = (ib - 1) + (int64_t)e->nsort_c * (L + (int64_t)(e->lmaxso + 1) * (isp - 1));
  return cdouble(a[2 * off], a[2 * off + 1]);
}
double Kari(const Ctx& c, int isym, int isp) { return c.g->Kari[(isym - 1) + 64 * (int64_t)(isp - 1)]; }
double Gradvr(const Ctx& c, int i, int k, int isp) {
  const fdmgpu_energy* e = c.e;
  return e->gradvr[(i - 1) + (int64_t)e->nicm * ((k - 1) + 3 * (int64_t)(isp - 1))];
}
double Ylmso(const Ctx& c, int ib, int lm) { return c.Ylmso(ib, lm); }

// Complex harmonic of the outer sphere at boundary point ib (Ycomp of the reference).
cdouble Yso(const Ctx& c, int ib, int m, int Lm0) {
  if (c.e->Ylm_comp && m != 0) return Yc(m, Ylmso(c, ib, Lm0), Ylmso(c, ib, Lm0 - 2 * m));
  return cdouble(Ylmso(c, ib, Lm0), 0.0);
}
cdouble Yato(const Ctx& c, int ib, int m, int Lm0, int ia) {
  if (c.e->Ylm_comp && m != 0) return Yc(m, Ylmato(c, ib, Lm0, ia), Ylmato(c, ib, Lm0 - 2 * m, ia));
  return cdouble(Ylmato(c, ib, Lm0, ia), 0.0);
}

// Outer-sphere radial factor of a column (the outgoing or real basis function).
cdouble outer_column_factor(const Ctx& c, int ib, int L, int ispq) {
  const fdmgpu_energy* e = c.e;
  if (e->Basereel) {
    if (e->E_comp) return BesC(c, e->Neuman, ib, L, ispq);
    return cdouble(Bes(c, e->Neumanr, ib, L, ispq), 0.0);
  }
  if (e->E_comp) return BesC(c, e->Bessel, ib, L, ispq) + img * BesC(c, e->Neuman, ib, L, ispq);
  return cdouble(Bes(c, e->Besselr, ib, L, ispq), Bes(c, e->Neumanr, ib, L, ispq));
}
// Radial factor of the right-hand side: the incoming j_l of the regular
// solution, -i j_l + n_l of the irregular one (complex energies only).
cdouble outer_rhs_factor(const Ctx& c, int ib, int L, int ispq) {
  const fdmgpu_energy* e = c.e;
  if (e->irregular) return -img * BesC(c, e->Bessel, ib, L, ispq) + BesC(c, e->Neuman, ib, L, ispq);
  if (e->E_comp) return BesC(c, e->Bessel, ib, L, ispq);
  return cdouble(Bes(c, e->Besselr, ib, L, ispq), 0.0);
}

// One complex row: A(col) for col in lb1..lb2 (stored at row[col - lb1]) and the
// right-hand side rhs(Lm) = smr(Lm, ii) + i smi(Lm, ii).
void calc_mat_row_c(const Ctx& c, int ii, cdouble* row, int lb1, cdouble* rhs) {
  const fdmgpu_grid* g = c.g;
  const fdmgpu_energy* e = c.e;
  const int nspino = c.nspino;
  const int nspin = g->nspin;
  const int natome = g->natome;
  const int i = e->newinv[ii - 1];
  auto A = [&](int col) -> cdouble& { return row[col - lb1]; };
  int ispin = c.ispin;
  const double a2s4 = 0.25 * alfa_sf * alfa_sf;

  if (e->Spinorbite && i > 0) {
    // spin of a grid row: rows of a point alternate spin 1, spin 2 (mat.f90:1128-1134)
    int ia = natome;
    for (; ia >= 1; --ia)
      if (ii > e->ianew[ia - 1]) break;
    const int base = ia >= 1 ? e->ianew[ia - 1] + e->n_ato_RI * e->nlmsa[ia - 1] : 0;
    const int ii1 = ii - base;
    ispin = 2 - (((ii1 % 2) + 2) % 2);
  }

  if (i > 0) {
    const int ispp = std::min(ispin, nspin);
    const int indg = 3 - ispin;
    // ispq is one variable of the row in the reference: the outer-neighbour
    // case below reassigns it, and later neighbours' spin-orbit terms see the
    // reassigned value.  Kept as one variable here for the same arithmetic.
    int ispq = std::min(indg, nspin);
    const int isp = std::min(ispin, nspino);
    const double VmE = e->Vr[(i - 1) + (int64_t)g->npoint * (ispp - 1)] - e->Enervide;
    A(ii) = cdouble(VmE - g->clapl[0], e->E_comp ? -e->Eimag : 0.0);
    if (e->Relativiste) A(ii) -= a2s4 * (VmE * VmE);   // a2s4 * VmE**2
    double bder = 0.0;
    if (e->Relativiste || e->Spinorbite) bder = -a2s4 / (1.0 - a2s4 * VmE);
    double cfvs_r[2] = {0.0, 0.0}, cfvs_i[2] = {0.0, 0.0};
    for (int iv = 1; iv <= g->nvois; ++iv) {
      const int j = c.ivois(i, iv);
      const int ia = g->numia[j - 1];
      cfvs_r[isp - 1] = -g->clapl[iv];
      cfvs_i[isp - 1] = 0.0;
      double charac_r[2], charac_i[2];
      for (int s = 1; s <= nspino; ++s) {
        charac_r[s - 1] = c.Kar(std::abs(c.isvois(i, iv)), s);
        charac_i[s - 1] = Kari(c, std::abs(c.isvois(i, iv)), s);
      }
      (void)charac_i;  // Repres_comp only
      const int k = 1 + ((iv - 1) / 2) % 3;   // axis of the neighbour (cubic grid)
      if (e->Relativiste) cfvs_r[isp - 1] += bder * g->cgrad[iv - 1] * Gradvr(c, i, k, ispp);
      if (e->Spinorbite) {
        double csor[2] = {0.0, 0.0}, csoi[2] = {0.0, 0.0};
        switch (k) {
          case 1:
            csoi[isp - 1] = -Gradvr(c, i, 2, ispp);
            csor[indg - 1] = Gradvr(c, i, 3, ispq);
            break;
          case 2:
            csoi[isp - 1] = Gradvr(c, i, 1, ispp);
            csoi[indg - 1] = -Gradvr(c, i, 3, ispq);
            break;
          default:
            csor[indg - 1] = -Gradvr(c, i, 1, ispq) + Gradvr(c, i, 2, ispq);
            break;
        }
        for (int s = 0; s < 2; ++s) {
          csor[s] = bder * g->cgrad[iv - 1] * csor[s];
          csoi[s] = bder * g->cgrad[iv - 1] * csoi[s];
        }
        cfvs_r[isp - 1] = cfvs_r[isp - 1] + csor[isp - 1];
        cfvs_r[indg - 1] = csor[indg - 1];
        cfvs_i[0] = csoi[0];
        cfvs_i[1] = csoi[1];
        for (int s = 0; s < 2; ++s) {
          cfvs_i[s] = charac_r[s] * cfvs_i[s];
          cfvs_r[s] = charac_r[s] * cfvs_r[s];
        }
      } else {
        cfvs_r[isp - 1] = charac_r[isp - 1] * cfvs_r[isp - 1];
      }
      for (int s = 0; s < nspino; ++s) {
        cfvs_r[s] = cfvs_r[s] * g->rvol[i - 1];
        cfvs_i[s] = cfvs_i[s] * g->rvol[i - 1];
      }

      if (ia == 0) {
        const int jj = e->new_[j] - nspino + isp;
        for (int ispo = 1; ispo <= nspino; ++ispo) {
          const int jj1 = jj + ispo - isp;
          A(jj1) += cdouble(cfvs_r[ispo - 1] / g->rvol[j - 1], cfvs_i[ispo - 1] / g->rvol[j - 1]);
        }
      } else if (ia > 0) {
        int ib;
        for (ib = g->nbordf[ia - 1] + 1; ib <= g->nbord[ia - 1]; ++ib)
          if (j == c.ibord(ib, ia)) break;
        const int isym = std::abs(c.isbord(ib, ia));
        if (isym != 1)
          for (int s = 1; s <= nspino; ++s) {
            cfvs_r[s - 1] = c.Kar(isym, s) * cfvs_r[s - 1];
            cfvs_i[s - 1] = c.Kar(isym, s) * cfvs_i[s - 1];
          }
        // one column block per atomic solution: the regular amplitudes, and
        // with the irregular solution the irregular ones after them
        for (int jri = 1; jri <= e->n_ato_RI; ++jri) {
          const int iri = e->irregular ? jri : 1;
          for (int Lm = 1; Lm <= e->nlmsa[ia - 1]; ++Lm) {
            int jjj = e->ianew[ia - 1] + Lm;
            if (iri == 2 && e->n_ato_RI == 2) jjj += e->nlmsa[ia - 1];
            const int L = Lato(c, Lm, ia);
            const int isol = Iato(c, Lm, ia);
            for (int ispo = 1; ispo <= nspino; ++ispo) {
              const int m = Mato(c, Lm, ia) + ispo - isol;
              if (m > L || m < -L) continue;
              const int Lm0 = L * L + L + 1 + m;
              if (e->Spinorbite) {
                A(jjj) += cdouble(cfvs_r[ispo - 1], cfvs_i[ispo - 1]) * PhiatoC(c, ib, Lm0, ispo, isol, ia, iri);
              } else if (e->nphiato7 == 2) {
                A(jjj) += cdouble(cfvs_r[isp - 1], cfvs_i[isp - 1]) * PhiatoC(c, ib, Lm0, ispp, isol, ia, iri);
              } else {
                const double ph = PhiatoPart(c, ib, Lm0, ispp, isol, ia, 0, iri);
                A(jjj) += cdouble(cfvs_r[isp - 1] * ph, cfvs_i[isp - 1] * ph);
              }
            }
          }
        }
      } else if (ia == -2) {
        int ib;
        for (ib = g->nsortf + 1; ib <= g->nsort; ++ib)
          if (j == g->isrt[ib - 1]) break;
        // the irregular solution has no scattered wave in the outer sphere
        for (int Lm = 1; Lm <= (e->irregular ? 0 : e->nlmso); ++Lm) {
          const int L = Lso(c, Lm), m = Mso(c, Lm);
          const int Lm0 = L * L + L + 1 + m;
          ispq = std::min(Iso(c, Lm), e->nspinr);
          const int jjj = e->nligneso + Lm;
          const cdouble f = outer_column_factor(c, ib, L, ispq) * Yso(c, ib, m, Lm0);
          const int s = (isp == Iso(c, Lm)) ? isp : indg;
          A(jjj) += f * cdouble(cfvs_r[s - 1], cfvs_i[s - 1]);
        }
        for (int Lm = 1; Lm <= e->nlmso; ++Lm) {
          const int L = Lso(c, Lm), m = Mso(c, Lm);
          const int Lm0 = L * L + L + 1 + m;
          ispq = std::min(Iso(c, Lm), e->nspinr);
          const cdouble f = Yso(c, ib, m, Lm0) * outer_rhs_factor(c, ib, L, ispq);
          const int s = (isp == Iso(c, Lm)) ? isp : indg;
          rhs[Lm - 1] -= f * cdouble(cfvs_r[s - 1], cfvs_i[s - 1]);
        }
      }
    }
  } else if (i == 0) {
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
      cdouble charmc = 0.0;
      for (int ib = 1; ib <= g->nsortf; ++ib) {
        cdouble cfac;
        if (e->Ylm_comp && m != 0 && mp != 0)
          cfac = std::conj(Yc(m, Ylmso(c, ib, Lm0), Ylmso(c, ib, Lm0 - 2 * m))) *
                 Yc(mp, Ylmso(c, ib, lmp0), Ylmso(c, ib, lmp0 - 2 * mp));
        else if (e->Ylm_comp && m != 0)
          cfac = std::conj(Yc(m, Ylmso(c, ib, Lm0), Ylmso(c, ib, Lm0 - 2 * m))) * Ylmso(c, ib, lmp0);
        else if (e->Ylm_comp && mp != 0)
          cfac = Ylmso(c, ib, Lm0) * Yc(mp, Ylmso(c, ib, lmp0), Ylmso(c, ib, lmp0 - 2 * mp));
        else
          cfac = cdouble(Ylmso(c, ib, Lm0) * Ylmso(c, ib, lmp0), 0.0);
        cfac = g->poidso[ib - 1] * cfac;
        charmc += cfac * outer_column_factor(c, ib, L, ispq);
      }
      A(e->nligneso + Lmp) += charmc;
    }
    for (int ib = 1; ib <= g->nsortf; ++ib) {
      const int j = g->isrt[ib - 1];
      const int jj = e->new_[j] - nspino + isp;
      cdouble cfac;
      if (e->Ylm_comp && m != 0) {
        cfac = g->poidso[ib - 1] * std::conj(Yc(m, Ylmso(c, ib, Lm0), Ylmso(c, ib, Lm0 - 2 * m)));
        A(jj) -= cfac / g->rvol[j - 1];
      } else {
        const double fac = g->poidso[ib - 1] * Ylmso(c, ib, Lm0);
        cfac = cdouble(fac, 0.0);
        A(jj) -= fac / g->rvol[j - 1];
      }
      for (int Lmf = 1; Lmf <= e->nlmso; ++Lmf) {
        const int ispq = std::min(Iso(c, Lmf), e->nspinr);
        if (isp != Iso(c, Lmf)) continue;
        const int L = Lso(c, Lmf);
        const int mf = Mso(c, Lmf);
        const int lmf0 = L * L + L + 1 + mf;
        cdouble cfad = cfac * Yso(c, ib, mf, lmf0);
        cfad = cfad * outer_rhs_factor(c, ib, L, ispq);
        rhs[Lmf - 1] -= cfad;
      }
    }
  } else {
    const int ia = -i;
    const int nl = e->nlmsa[ia - 1];
    const int Ln = ii - e->ianew[ia - 1];
    // with both atomic solutions the rows of the irregular amplitudes follow
    // those of the regular ones
    const int iri = (e->n_ato_RI == 2 && Ln > nl) ? 2 : 1;
    const int Lm = iri == 2 ? Ln - nl : Ln;
    const int L = Lato(c, Lm, ia);
    const int ispt = Iato(c, Lm, ia);
    const int m = Mato(c, Lm, ia);
    const int Lm0 = L * L + L + 1 + m;
    // irregular solution: the first half of the boundary points carries the
    // regular, the second half the irregular matching
    const int nhalf = g->nbordf[ia - 1] / 2;
    const bool split = e->irregular && e->n_ato_RI == 2;
    for (int ib = 1; ib <= g->nbordf[ia - 1]; ++ib) {
      if (split && iri == 1 && ib > nhalf) break;
      if (split && iri == 2 && ib <= nhalf) continue;
      const int j = c.ibord(ib, ia);
      const int isym = std::abs(c.isbord(ib, ia));
      const int jj = e->new_[j] - nspino + ispt;
      const cdouble yc = Yato(c, ib, m, Lm0, ia);
      cdouble cfac;
      if (std::fabs(Kari(c, isym, ispt)) < 1e-10)
        cfac = c.poidsa(ib, ia) * std::conj(yc) * c.Kar(isym, ispt) / g->rvol[j - 1];
      else
        cfac = c.poidsa(ib, ia) * std::conj(yc) * cdouble(c.Kar(isym, ispt), -Kari(c, isym, ispt)) / g->rvol[j - 1];
      A(jj) -= cfac;
    }
    for (int jri = 1; jri <= (e->irregular ? 2 : 1); ++jri) {
      for (int Lmp = 1; Lmp <= nl; ++Lmp) {
        const int Lp = Lato(c, Lmp, ia);
        const int isol = Iato(c, Lmp, ia);
        const int mp = Mato(c, Lmp, ia) + ispt - isol;
        if (mp > Lp || mp < -Lp) continue;
        const int Lmp0 = Lp * Lp + Lp + 1 + mp;
        const int ispint = e->Spinorbite ? std::min(ispt, e->nspinp) : std::min(ispin, e->nspinp);
        double charmr = 0.0, charmi = 0.0;
        for (int ib = 1; ib <= g->nbordf[ia - 1]; ++ib) {
          if (e->irregular && jri == 1 && ib > nhalf) break;
          if (e->irregular && jri == 2 && ib <= nhalf) continue;
          cdouble cfac = PhiatoC(c, ib, Lmp0, ispint, isol, ia, jri);
          if (e->Ylm_comp && m != 0)
            cfac = cfac * std::conj(Yc(m, Ylmato(c, ib, Lm0, ia), Ylmato(c, ib, Lm0 - 2 * m, ia)));
          else
            cfac = cfac * Ylmato(c, ib, Lm0, ia);
          charmr = charmr + c.poidsa(ib, ia) * cfac.real();
          charmi = charmi + c.poidsa(ib, ia) * cfac.imag();
        }
        int ljj = e->ianew[ia - 1] + Lmp;
        if (jri == 2 && e->n_ato_RI == 2) ljj += nl;
        A(ljj) += cdouble(charmr, charmi);
      }
    }
  }
}

int check_supported_c(const fdmgpu_grid* g, const fdmgpu_energy* e) {
  if (!e->Cal_comp || e->Repres_comp || e->Base_hexa) return FDMGPU_ERR_UNSUPPORTED;
  if (e->irregular) {
    // FDM_comp's irregular solution with both atomic solutions (Test_reg = 0)
    if (e->n_RI != 2 || e->n_ato_RI != 2 || e->Test_reg != 0 || !e->E_comp || e->Basereel)
      return FDMGPU_ERR_UNSUPPORTED;
    if (e->nligneso != e->nligne) return FDMGPU_ERR_ARG;
  } else if (e->n_ato_RI != 1 || e->n_RI < 1 || e->n_RI > 2) {
    return FDMGPU_ERR_UNSUPPORTED;
  }
  if (e->Spinorbite != (g->nspino == 2)) return FDMGPU_ERR_ARG;
  if (e->Spinorbite && g->nspin != 2) return FDMGPU_ERR_UNSUPPORTED;
  if ((e->Relativiste || e->Spinorbite) && !e->gradvr) return FDMGPU_ERR_ARG;
  if (e->E_comp && (!e->Bessel || !e->Neuman)) return FDMGPU_ERR_ARG;
  if (!e->E_comp && (!e->Besselr || !e->Neumanr)) return FDMGPU_ERR_ARG;
  return FDMGPU_OK;
}

}  // namespace

extern "C" {

// cbessneu, source/sphere.f90:7226-7254: fnorm*j_l(z), fnorm*n_l(z) for complex
// z and fnorm by upward recursion, l = 0..lmax; outputs interleaved re/im.
void oracle_cbessneu(double fnorm_re, double fnorm_im, double z_re, double z_im, int lmax, double* bessel_ri,
                     double* neuman_ri) {
  const cdouble fnorm(fnorm_re, fnorm_im), z(z_re, z_im);
  cdouble* bs = reinterpret_cast<cdouble*>(bessel_ri);
  cdouble* nm = reinterpret_cast<cdouble*>(neuman_ri);
  nm[0] = -fnorm * std::cos(z) / z;
  bs[0] = fnorm * std::sin(z) / z;
  if (lmax == 0) return;
  nm[1] = nm[0] / z - bs[0];
  bs[1] = bs[0] / z + nm[0];
  for (int L = 2; L <= lmax; ++L) {
    const double L1 = 2 * L - 1;
    nm[L] = L1 * nm[L - 1] / z - nm[L - 2];
    bs[L] = L1 * bs[L - 1] / z - bs[L - 2];
  }
}

// Dense complex assembly: A (nligne x nligne) and B = smr + i smi (nlmso x
// nligne), both column-major complex interleaved.
int oracle_assemble_dense_c(const fdmgpu_grid* g, const fdmgpu_energy* e, double* A_ri, double* B_ri) {
  int st = check_supported_c(g, e);
  if (st) return st;
  Ctx c = make_ctx(g, e);
  cdouble* A = reinterpret_cast<cdouble*>(A_ri);
  cdouble* B = reinterpret_cast<cdouble*>(B_ri);
  const int n = e->nligne;
  std::vector<cdouble> row;
  for (int ii = 1; ii <= n; ++ii) {
    const int l1 = e->lb1[ii - 1], l2 = e->lb2[ii - 1];
    row.assign(l2 - l1 + 1, 0.0);
    calc_mat_row_c(c, ii, row.data(), l1, B + (int64_t)(ii - 1) * e->nlmso);
    for (int k = l1; k <= l2; ++k) A[(int64_t)(ii - 1) + (int64_t)(k - 1) * n] = row[k - l1];
  }
  return 0;
}

// Sparse complex assembly in CSR form (see oracle_assemble_csr); values and
// B complex interleaved.
int oracle_assemble_csr_c(const fdmgpu_grid* g, const fdmgpu_energy* e, int64_t* rowptr, int32_t* colidx,
                          double* val_ri, double* B_ri) {
  int st = check_supported_c(g, e);
  if (st) return st;
  Ctx c = make_ctx(g, e);
  cdouble* val = reinterpret_cast<cdouble*>(val_ri);
  cdouble* B = reinterpret_cast<cdouble*>(B_ri);
  const int n = e->nligne;
  std::vector<cdouble> row;
  std::vector<cdouble> brow(e->nlmso);
  rowptr[0] = 0;
  for (int ii = 1; ii <= n; ++ii) {
    const int l1 = e->lb1[ii - 1], l2 = e->lb2[ii - 1];
    row.assign(l2 - l1 + 1, 0.0);
    cdouble* b = B ? B + (int64_t)(ii - 1) * e->nlmso : brow.data();
    std::fill(brow.begin(), brow.end(), cdouble(0.0));
    calc_mat_row_c(c, ii, row.data(), l1, b);
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

// Gaussian profile solve, complex branch (source/mat_solve_gaussian.f90:196-358):
// the row elimination of the real branch with the complex products written out
// as the reference writes them, the division by the pivot through its
// conjugate over |a|^2 (:265-290), zero-pivot test |a|^2 < 1e-20.
// smr, smi (nlmso, nligne) are zero on entry and hold the solution on return.
int oracle_mat_solve_c(const fdmgpu_grid* g, const fdmgpu_energy* e, double* smr, double* smi, int64_t* nnz_out,
                       double* time_fill, double* time_tria, int32_t* bad_row) {
  int st = check_supported_c(g, e);
  if (st) return st;
  Ctx c = make_ctx(g, e);
  const int nligne = e->nligne, nlmso = e->nlmso;
  std::vector<int32_t> ind, nb_not_zero;
  std::vector<int64_t> lbz;
  const int64_t nb_tot = symbolic_profile(c, ind, nb_not_zero, lbz);
  if (nnz_out) *nnz_out = nb_tot;
  std::vector<double> abr(nb_tot, 0.0), abi(nb_tot, 0.0);
  std::vector<cdouble> row, rhs(nlmso);
  std::vector<double> abvr, abvi;
  const double eps15 = 1e-15;
  double tfill = 0, ttria = 0;
  for (int ii = nligne; ii >= 1; --ii) {
    auto t0 = std::chrono::steady_clock::now();
    const int lb1 = e->lb1[ii - 1], lb2 = e->lb2[ii - 1];
    row.assign(lb2 - lb1 + 1, 0.0);
    std::fill(rhs.begin(), rhs.end(), cdouble(0.0));
    calc_mat_row_c(c, ii, row.data(), lb1, rhs.data());
    double* sr = smr + (int64_t)(ii - 1) * nlmso;
    double* si = smi + (int64_t)(ii - 1) * nlmso;
    for (int l = 0; l < nlmso; ++l) {
      sr[l] += rhs[l].real();
      si[l] += rhs[l].imag();
    }
    abvr.resize(row.size());
    abvi.resize(row.size());
    for (size_t q = 0; q < row.size(); ++q) {
      abvr[q] = row[q].real();
      abvi[q] = row[q].imag();
    }
    auto t1 = std::chrono::steady_clock::now();
    for (int j = lb2; j >= ii + 1; --j) {
      const double facr = abvr[j - lb1], faci = abvi[j - lb1];
      if (std::fabs(facr) > eps15 || std::fabs(faci) > eps15) {
        const int64_t b = lbz[j], nz = nb_not_zero[j];
        for (int64_t lk = b; lk < b + nz; ++lk) {
          const int k = ind[lk] - lb1;
          abvr[k] = abvr[k] - facr * abr[lk] + faci * abi[lk];
          abvi[k] = abvi[k] - facr * abi[lk] - faci * abr[lk];
        }
        const double* srj = smr + (int64_t)(j - 1) * nlmso;
        const double* sij = smi + (int64_t)(j - 1) * nlmso;
        for (int l = 0; l < nlmso; ++l) {
          const double r = sr[l] - facr * srj[l] + faci * sij[l];
          const double q = si[l] - facr * sij[l] - faci * srj[l];
          sr[l] = r;
          si[l] = q;
        }
      }
    }
    const double pr = abvr[ii - lb1], pi = abvi[ii - lb1];
    const double den = pr * pr + pi * pi;
    if (den < 1e-20) {
      if (bad_row) *bad_row = ii;
      return FDMGPU_ERR_ZERO_PIVOT;
    }
    const double vr = pr / den, vi = -pi / den;
    {
      const int64_t b = lbz[ii], nz = nb_not_zero[ii];
      for (int64_t lk = b; lk < b + nz; ++lk) {
        const int k = ind[lk] - lb1;
        abr[lk] = abvr[k] * vr - abvi[k] * vi;
        abi[lk] = abvi[k] * vr + abvr[k] * vi;
      }
    }
    for (int l = 0; l < nlmso; ++l) {
      const double fr = sr[l] * vr - si[l] * vi;
      const double fi = sr[l] * vi + si[l] * vr;
      sr[l] = fr;
      si[l] = fi;
    }
    auto t2 = std::chrono::steady_clock::now();
    tfill += std::chrono::duration<double>(t1 - t0).count();
    ttria += std::chrono::duration<double>(t2 - t1).count();
  }
  for (int ii = 2; ii <= nligne; ++ii) {
    double* sr = smr + (int64_t)(ii - 1) * nlmso;
    double* si = smi + (int64_t)(ii - 1) * nlmso;
    const int64_t b = lbz[ii], nz = nb_not_zero[ii];
    for (int64_t lk = b; lk < b + nz; ++lk) {
      const int j = ind[lk];
      const double ar = abr[lk], ai = abi[lk];
      const double* srj = smr + (int64_t)(j - 1) * nlmso;
      const double* sij = smi + (int64_t)(j - 1) * nlmso;
      for (int l = 0; l < nlmso; ++l) {
        const double r = sr[l] - ar * srj[l] + ai * sij[l];
        const double q = si[l] - ar * sij[l] - ai * srj[l];
        sr[l] = r;
        si[l] = q;
      }
    }
  }
  if (time_fill) *time_fill += tfill;
  if (time_tria) *time_tria += ttria;
  return 0;
}

// Taull of atom iaabs from a complex-basis solution (Basereel false,
// FDM_comp false; source/mat.f90:354-405): Taull(Lm1 s1, Lm2 s2) +=
// -i sum_f ampl1(f) conj(ampl2(f)) with ampl = smr + i smi on the atom's rows,
// s = iato with spin-orbit, else 1.  With symmetrise != 0 the symmetrisation of
// source/mat.f90:594-644 follows (none with spin-orbit and nspin = 2; the
// (-1)^(m1+m2) pairing with complex harmonics; i Im(Taull) otherwise).
// taull: (nlmq, nsp, nlmq, nsp) complex interleaved, nlmq = (lmax+1)^2,
// nsp = nspino; *nlm_out = nlmq.
int oracle_taull_c(const fdmgpu_grid* g, const fdmgpu_energy* e, int iaabs, const double* smr, const double* smi,
                   int symmetrise, double* taull, int32_t* nlm_out) {
  Ctx c = make_ctx(g, e);
  const int nlmso = e->nlmso;
  const int ia = iaabs;
  const int nlm = e->nlmsa[ia - 1];
  const int nsp = c.nspino;
  int lmax = 0;
  for (int Lm = 1; Lm <= nlm; ++Lm) lmax = std::max(lmax, Lato(c, Lm, ia));
  const int nlmq = (lmax + 1) * (lmax + 1);
  const int64_t dim = (int64_t)nlmq * nsp;
  std::vector<cdouble> T((size_t)(dim * dim), 0.0);
  auto Tix = [&](int lm0, int s1, int lm02, int s2) -> cdouble& {
    return T[(size_t)((lm0 - 1) + (int64_t)nlmq * (s1 - 1) + dim * ((lm02 - 1) + (int64_t)nlmq * (s2 - 1)))];
  };
  for (int Lm1 = 1; Lm1 <= nlm; ++Lm1) {
    const int L1 = Lato(c, Lm1, ia), m1 = Mato(c, Lm1, ia);
    const int is1 = e->Spinorbite ? Iato(c, Lm1, ia) : 1;
    const int Lm01 = L1 * L1 + L1 + 1 + m1;
    const int ii = e->ianew[ia - 1] + Lm1;
    for (int Lm2 = 1; Lm2 <= nlm; ++Lm2) {
      const int L2 = Lato(c, Lm2, ia), m2 = Mato(c, Lm2, ia);
      const int is2 = (nsp == 2) ? Iato(c, Lm2, ia) : 1;
      const int Lm02 = L2 * L2 + L2 + 1 + m2;
      const int jj = e->ianew[ia - 1] + Lm2;
      cdouble cfac = 0.0;
      for (int f = 0; f < nlmso; ++f) {
        const cdouble a1(smr[f + (int64_t)(ii - 1) * nlmso], smi[f + (int64_t)(ii - 1) * nlmso]);
        const cdouble a2(smr[f + (int64_t)(jj - 1) * nlmso], smi[f + (int64_t)(jj - 1) * nlmso]);
        cfac = cfac - img * a1 * std::conj(a2);
      }
      Tix(Lm01, is1, Lm02, is2) += cfac;
    }
  }
  if (symmetrise && !(e->Spinorbite && g->nspin == 2)) {
    for (int Lm1 = 1; Lm1 <= nlm; ++Lm1) {
      const int L1 = Lato(c, Lm1, ia), m1 = Mato(c, Lm1, ia);
      const int Lm01 = L1 * L1 + L1 + 1 + m1;
      const int is1 = e->Spinorbite ? Iato(c, Lm1, ia) : 1;
      for (int Lm2 = 1; Lm2 <= nlm; ++Lm2) {
        const int L2 = Lato(c, Lm2, ia), m2 = Mato(c, Lm2, ia);
        const int Lm02 = L2 * L2 + L2 + 1 + m2;
        const int is2 = (nsp == 2) ? Iato(c, Lm2, ia) : 1;
        if (e->Spinorbite) {
          const double isg = ((m1 - m2 - is1 + is2) % 2 == 0) ? 1.0 : -1.0;
          const cdouble cf = 0.5 * (Tix(Lm01, is1, Lm02, is2) + isg * Tix(Lm02 - 2 * m2, 3 - is2, Lm01 - 2 * m1, 3 - is1));
          Tix(Lm01, is1, Lm02, is2) = cf;
          Tix(Lm02 - 2 * m2, 3 - is2, Lm01 - 2 * m1, 3 - is1) = isg * cf;
        } else if (e->Ylm_comp) {
          const double isg = ((m1 + m2) % 2 == 0) ? 1.0 : -1.0;
          const cdouble cf = 0.5 * (Tix(Lm01, is1, Lm02, is2) + isg * Tix(Lm02 - 2 * m2, is2, Lm01 - 2 * m1, is1));
          Tix(Lm01, is1, Lm02, is2) = cf;
          Tix(Lm02 - 2 * m2, is2, Lm01 - 2 * m1, is1) = isg * cf;
        } else {
          Tix(Lm01, is1, Lm02, is2) = cdouble(0.0, Tix(Lm01, is1, Lm02, is2).imag());
        }
      }
    }
  }
  std::memcpy(taull, T.data(), sizeof(cdouble) * T.size());
  if (nlm_out) *nlm_out = nlmq;
  return 0;
}

// Tau_RI of atom iaabs (FDM_comp, source/mat.f90:219-292): from the regular
// solution (problem e_reg, smr_reg + i smi_reg) and the irregular one (e_irr),
// Tau_RI(Lm1 s1, Lm2 s2, i_RI) = sum_f Ampl(f, Lm1) Ampl_I(f, (i_RI - 1) nlmsa + Lm2)
// with Ampl the regular amplitudes of the atom's rows and Ampl_I the
// irregular problem's amplitudes (regular atomic solution, then irregular);
// no conjugate, no symmetrisation (the reference skips it with FDM_comp).
// s = iato with spin-orbit, else 1.  tau_ri: (nlmq, nsp, nlmq, nsp, 2) complex
// interleaved; *nlm_out = nlmq.
int oracle_tau_ri(const fdmgpu_grid* g, const fdmgpu_energy* e_reg, const double* smr_reg, const double* smi_reg,
                  const fdmgpu_energy* e_irr, const double* smr_irr, const double* smi_irr, int iaabs, double* tau_ri,
                  int32_t* nlm_out) {
  if (e_reg->irregular || !e_irr->irregular || e_irr->n_ato_RI != 2 || e_reg->nlmso != e_irr->nlmso ||
      e_reg->nlmsa[iaabs - 1] != e_irr->nlmsa[iaabs - 1])
    return FDMGPU_ERR_ARG;
  Ctx c = make_ctx(g, e_reg);
  const int nlmso = e_reg->nlmso;
  const int ia = iaabs;
  const int nlm = e_reg->nlmsa[ia - 1];
  const int nsp = c.nspino;
  int lmax = 0;
  for (int Lm = 1; Lm <= nlm; ++Lm) lmax = std::max(lmax, Lato(c, Lm, ia));
  const int nlmq = (lmax + 1) * (lmax + 1);
  const int64_t dim = (int64_t)nlmq * nsp;
  std::vector<cdouble> T((size_t)(2 * dim * dim), 0.0);
  for (int Lm1 = 1; Lm1 <= nlm; ++Lm1) {
    const int L1 = Lato(c, Lm1, ia), m1 = Mato(c, Lm1, ia);
    const int is1 = e_reg->Spinorbite ? Iato(c, Lm1, ia) : 1;
    const int64_t row = (L1 * L1 + L1 + m1) + (int64_t)nlmq * (is1 - 1);
    const int64_t ii = e_reg->ianew[ia - 1] + Lm1;
    for (int iri = 1; iri <= 2; ++iri)
      for (int Lm2 = 1; Lm2 <= nlm; ++Lm2) {
        const int L2 = Lato(c, Lm2, ia), m2 = Mato(c, Lm2, ia);
        const int is2 = e_reg->Spinorbite ? Iato(c, Lm2, ia) : 1;
        const int64_t col = (L2 * L2 + L2 + m2) + (int64_t)nlmq * (is2 - 1);
        const int64_t jj = e_irr->ianew[ia - 1] + (iri - 1) * nlm + Lm2;
        cdouble& t = T[(size_t)(row + dim * col + dim * dim * (iri - 1))];
        for (int f = 0; f < nlmso; ++f) {
          const cdouble a(smr_reg[f + (ii - 1) * nlmso], smi_reg[f + (ii - 1) * nlmso]);
          const cdouble b(smr_irr[f + (jj - 1) * nlmso], smi_irr[f + (jj - 1) * nlmso]);
          t = t + a * b;
        }
      }
  }
  std::memcpy(tau_ri, T.data(), sizeof(cdouble) * T.size());
  if (nlm_out) *nlm_out = nlmq;
  return 0;
}

}  // extern "C"
