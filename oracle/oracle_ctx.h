// oracle_ctx.h - argument accessors shared by the real and complex branches of
// the CPU restatement (test infrastructure only).
#pragma once

#include <complex>
#include <cstdint>
#include <vector>

#include "../include/fdmgpu.h"

namespace oracle {

typedef std::complex<double> cdouble;

// Fortran-style accessors (1-based indices).
struct I2 {
  const int32_t* p; int64_t ld;
  int32_t operator()(int64_t i, int64_t j) const { return p[(i - 1) + (j - 1) * ld]; }
};
struct D2 {
  const double* p; int64_t ld;
  double operator()(int64_t i, int64_t j) const { return p[(i - 1) + (j - 1) * ld]; }
};

struct Ctx {
  const fdmgpu_grid* g;
  const fdmgpu_energy* e;
  I2 ivois, isvois, ibord, isbord;
  D2 poidsa, Ylmso, Kar;
  int64_t ld_ylmato1, ld_ylmato2;
  int nspino;
  int ispin;
};

inline double Ylmato(const Ctx& c, int ib, int lm, int ia) {
  return c.g->Ylmato[(ib - 1) + (int64_t)(lm - 1) * c.g->nbtm + (int64_t)(ia - 1) * c.g->nbtm * c.g->nlmmax];
}
// phiato(ib, Lm, isp, isol, i_RI, ia, 1), dims (nphiato1, nlmagm, nspinp, nspino, n_RI, natome, nphiato7)
inline double Phiato(const Ctx& c, int ib, int lm, int isp, int isol, int iri, int ia) {
  const fdmgpu_energy* e = c.e;
  int64_t d1 = e->nphiato1, d2 = e->nlmagm, d3 = e->nspinp, d4 = c.nspino, d5 = e->n_RI;
  int64_t off = (ib - 1) + d1 * ((lm - 1) + d2 * ((isp - 1) + d3 * ((isol - 1) + d4 * ((iri - 1) + d5 * (ia - 1)))));
  return e->phiato[off];
}
// Besselr / Neumanr (nsort_r, 0:lmaxso, nspinr)
inline double Bes(const Ctx& c, const double* a, int ib, int L, int isp) {
  const fdmgpu_energy* e = c.e;
  return a[(ib - 1) + (int64_t)e->nsort_r * (L + (int64_t)(e->lmaxso + 1) * (isp - 1))];
}
inline int Lato(const Ctx& c, int lm, int ia) { return c.g->lato[(lm - 1) + (int64_t)c.g->nlmsam * (ia - 1 + (int64_t)c.g->natome * (c.e->igrph - 1))]; }
inline int Mato(const Ctx& c, int lm, int ia) { return c.g->mato[(lm - 1) + (int64_t)c.g->nlmsam * (ia - 1 + (int64_t)c.g->natome * (c.e->igrph - 1))]; }
inline int Iato(const Ctx& c, int lm, int ia) { return c.g->iato[(lm - 1) + (int64_t)c.g->nlmsam * (ia - 1 + (int64_t)c.g->natome * (c.e->igrph - 1))]; }
inline int Lso(const Ctx& c, int lm) { return c.g->lso[(lm - 1) + (int64_t)c.g->nso1 * (c.e->igrph - 1)]; }
inline int Mso(const Ctx& c, int lm) { return c.g->mso[(lm - 1) + (int64_t)c.g->nso1 * (c.e->igrph - 1)]; }
inline int Iso(const Ctx& c, int lm) { return c.g->iso[(lm - 1) + (int64_t)c.g->nso1 * (c.e->igrph - 1)]; }

inline Ctx make_ctx(const fdmgpu_grid* g, const fdmgpu_energy* e) {
  Ctx c;
  c.g = g; c.e = e;
  c.ivois = {g->ivois, g->npsom};
  c.isvois = {g->isvois, g->npsom};
  c.ibord = {g->ibord, g->nbtm};
  c.isbord = {g->isbord, g->nbtm};
  c.poidsa = {g->poidsa, g->nbm};
  c.Ylmso = {g->Ylmso, g->nsort};
  c.Kar = {g->Kar, 64};
  c.nspino = g->nspino;
  c.ispin = e->ispin;
  return c;
}

// Symbolic phase of the Gaussian profile solve (source/mat_solve_gaussian.f90:67-165):
// the columns left of the diagonal that each row holds after elimination.
// ind[lbz[ii] .. lbz[ii] + nb_not_zero[ii] - 1] are row ii's columns in
// ascending order (arrays indexed 1..nligne).  Returns the total count.
int64_t symbolic_profile(const Ctx& c, std::vector<int32_t>& ind, std::vector<int32_t>& nb_not_zero,
                         std::vector<int64_t>& lbz);

}  // namespace oracle
