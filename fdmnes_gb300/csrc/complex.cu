// complex.cu - complex (Cal_comp) assembly and Taull on the GPU.
//
// A complex problem is stored as its real-equivalent system: complex row ii
// (1-based, the reference's numbering) becomes rows 2ii-1 (real part) and 2ii
// (imaginary part), each complex entry a the 2x2 block [Re a, -Im a; Im a,
// Re a], each complex right-hand side one real column [Re b; Im b].  The band
// factorisation, the tile-local pivoting and the solves of the real path then
// run unchanged on an order-2n system whose profile is the complex one with
// every row and column doubled.  Pivoting inside the 64-row diagonal tiles
// keeps the 2x2 blocks stable where the real part of a pivot is small (the
// two rows of a block always share a tile).
//
// Restates the complex branch of calcMatRow (source/mat.f90:1034-1632) for
// Cal_comp = true, Repres_comp = false, C1 characters (Kar = 1, Kari = 0), real
// energies or complex ones (E_comp: -i Eimag on the grid diagonal,
// mat.f90:1151-1152, and the complex Bessel / Neumann of phiso), the regular
// solution and FDM_comp's irregular one with both atomic solutions (Test_reg
// = 0: amplitude columns of the regular then the irregular atomic solution,
// no outer-sphere rows or columns, right-hand side from -i j_l + n_l):
//   k_asmc_grid       grid rows with the relativistic and spin-orbit gradient
//                     terms (mat.f90:1142-1402), one warp per point, both spin
//                     rows of a point in turn
//   k_asmc_outer      outer-sphere rows, outer columns and right-hand sides
//                     (mat.f90:1405-1469, 1486-1510; regular solution only)
//   k_asmc_outer_bnd  outer rows, boundary-point columns (mat.f90:1471-1484)
//   k_asmc_atom       atom rows (mat.f90:1515-1632; irregular solution: the
//                     first half of the boundary points matches the regular,
//                     the second half the irregular atomic solution)
// the Taull of the complex basis (Basereel false, mat.f90:354-405) with its
// symmetrisation (mat.f90:594-644), and FDM_comp's Tau_RI from a regular and
// an irregular solution (mat.f90:219-292).  Within an entry, contributions are
// summed in the reference's order (neighbours iv ascending, boundary points
// ascending).
#include "fdm_internal.cuh"
#include "fdm_kernels.h"

namespace fdm {
namespace {

constexpr double kAlfaSf = 0.0072973525664;   // fine-structure constant, source/main.f90:58

__device__ __forceinline__ double2 c_mul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 c_conj(double2 a) { return make_double2(a.x, -a.y); }

// Yc (source/mat.f90:1733-1754): complex harmonic of order m from the real
// harmonics of orders m (y1) and -m (y2).
__device__ __forceinline__ double2 yc(int m, double y1, double y2) {
  const double s = 0x1.6a09e667f3bccp-1;   // 1 / sqrt(2) rounded as the reference computes it
  if (m == 0) return make_double2(y1, 0.0);
  if (m < 0) return make_double2(y2 * s, -y1 * s);
  const double sg = (m & 1) ? -1.0 : 1.0;
  return make_double2(y1 * sg * s, y2 * sg * s);
}

// Band entry (p, q) of the real-equivalent system; nullptr (and an error
// flag) outside the stored strip of row p.
__device__ __forceinline__ double* envc_at(double* env, const Prob& P, const Tables& tb, int p, int q, int* err,
                                           int e) {
  const int I = p / TS, J = q / TS;
  if (p < 0 || p >= P.nt * TS || q < 0 || q >= P.nt * TS || J < tb.J0[P.trow + I] || J > tb.J1[P.trow + I]) {
    atomicExch(&err[e], (int)FDMGPU_ERR_ARG);
    return nullptr;
  }
  return tile_ptr(env, P, tb, I, J) + (p % TS) * TS + (q % TS);
}

// A(ii, col) += v for complex 1-based indices.
__device__ __forceinline__ void add_c(double* env, const Prob& P, const Tables& tb, int ii, int col, double2 v,
                                      int* err, int e) {
  const int pr = P.n - (2 * ii - 1), pi = P.n - 2 * ii;
  const int qr = P.n - (2 * col - 1), qi = P.n - 2 * col;
  double* a;
  if ((a = envc_at(env, P, tb, pr, qr, err, e))) *a += v.x;
  if ((a = envc_at(env, P, tb, pr, qi, err, e))) *a -= v.y;
  if ((a = envc_at(env, P, tb, pi, qr, err, e))) *a += v.y;
  if ((a = envc_at(env, P, tb, pi, qi, err, e))) *a += v.x;
}

// B(lm, ii) += v (right-hand side lm, complex row ii).
__device__ __forceinline__ void add_rhs_c(double* B, const Prob& P, int ii, int lm, double2 v) {
  const int pr = P.n - (2 * ii - 1), pi = P.n - 2 * ii;
  const int r = lm - 1;
  rhs_ptr(B, P, pr / TS, r / TS)[(pr % TS) * TS + (r % TS)] += v.x;
  rhs_ptr(B, P, pi / TS, r / TS)[(pi % TS) * TS + (r % TS)] += v.y;
}

// Per-problem packed inputs of a complex problem (see pack_inputs):
//   Vr (npoint, nspin) | gradvr (npoint, 3, nspin) | phiato re, im
//   (nbtm, nlmagm, nspinp, nspino, nri, natome) | Bessel [nspinr][nsort][lmaxso+1] | Neumann (same)
struct CIn {
  const double* vr;
  const double* grad;
  const double* phi;
  const double* bes;
  const double* neu;
  int64_t phi_im;   // offset of the imaginary part
  int nl;
};
__device__ __forceinline__ CIn cin(const Prob& P, const StaticDev& S, const double* dpool) {
  CIn c;
  c.vr = dpool + P.in_vr;
  c.grad = dpool + P.in_grad;
  c.phi = dpool + P.in_phi;
  c.bes = dpool + P.in_bes;
  c.neu = dpool + P.in_neu;
  c.phi_im = (int64_t)S.nbtm * P.nlmagm * P.nspinp * S.nspino * P.nri * S.natome;
  c.nl = P.lmaxso + 1;
  return c;
}
// phiato of atomic solution iri (1 regular, 2 irregular)
__device__ __forceinline__ double2 phic(const CIn& c, const Prob& P, const StaticDev& S, int ib, int lm0, int isp,
                                        int isol, int ia, int iri = 1) {
  const int64_t off =
      (ib - 1) + (int64_t)S.nbtm * ((lm0 - 1) + (int64_t)P.nlmagm * ((isp - 1) + (int64_t)P.nspinp *
                                    ((isol - 1) + (int64_t)S.nspino * ((iri - 1) + (int64_t)P.nri * (ia - 1)))));
  return make_double2(c.phi[off], c.phi[off + c.phi_im]);
}
// Complex Bessel / Neumann value: the imaginary block follows the real one
// (complex energies); zero imaginary part for real energies.
__device__ __forceinline__ double2 besc(const CIn& c, const Prob& P, const double* a, const StaticDev& S, int ib, int L,
                                        int isp) {
  const int64_t o = ((int64_t)(isp - 1) * S.nsort + (ib - 1)) * c.nl + L;
  return make_double2(a[o], P.ecomp ? a[o + (int64_t)P.nspinr * S.nsort * c.nl] : 0.0);
}
__device__ __forceinline__ double ysot(const StaticDev& S, int ib, int lm0) {
  return S.YsoT[(int64_t)(ib - 1) * S.nlmomax + (lm0 - 1)];
}
__device__ __forceinline__ double2 yso(const Prob& P, const StaticDev& S, int ib, int m, int lm0) {
  if (P.ylmc && m != 0) return yc(m, ysot(S, ib, lm0), ysot(S, ib, lm0 - 2 * m));
  return make_double2(ysot(S, ib, lm0), 0.0);
}
__device__ __forceinline__ double ylmato(const StaticDev& S, int ib, int lm0, int ia) {
  return S.Ylmato[(ib - 1) + (int64_t)S.nbtm * ((lm0 - 1) + (int64_t)S.nlmmax * (ia - 1))];
}
// Outer radial factor of a column: the outgoing Besselr + i Neumanr, or
// Neumanr in the real basis (Basereel, kept for completeness).
__device__ __forceinline__ double2 colfac(const CIn& c, const Prob& P, const StaticDev& S, int basereel, int ib, int L,
                                          int ispq) {
  const double2 n = besc(c, P, c.neu, S, ib, L, ispq);
  if (basereel) return n;
  const double2 j = besc(c, P, c.bes, S, ib, L, ispq);
  return make_double2(j.x - n.y, j.y + n.x);  // j + i n
}

__global__ void k_asmc_pad(const Prob* probs, double* env, Tables tb, int* err) {
  const Prob P = probs[blockIdx.y];
  const int p = P.n + threadIdx.x;
  if (p < P.nt * TS) {
    double* a = envc_at(env, P, tb, p, p, err, blockIdx.y);
    if (a) *a = 1.0;
  }
}

// Grid rows: one warp per interstitial point, its spin rows in turn.
__global__ void __launch_bounds__(256) k_asmc_grid(const StaticDev* sites, const Prob* probs, const int* ipool,
                                                   const double* dpool, double* env, double* B, Tables tb,
                                                   int basereel, int* err) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  const StaticDev& S = sites[P.site];
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int k = blockIdx.x * 8 + warp;
  if (k >= S.npr) return;
  const int i = S.inter_pt[k];
  const int* new_ = ipool + P.in_new;
  const int* ianew = ipool + P.in_ianew;
  const int* nlmsa = ipool + P.in_nlmsa;
  const CIn c = cin(P, S, dpool);
  const int nspino = S.nspino;
  const double a2s4 = 0.25 * kAlfaSf * kAlfaSf;
  const double rvi = S.rvol[i - 1];
  auto grad = [&](int kax, int isp) { return c.grad[(i - 1) + (int64_t)S.npoint * ((kax - 1) + 3 * (isp - 1))]; };
  for (int srow = 1; srow <= nspino; ++srow) {
    const int ii = new_[i] - nspino + srow;
    const int ispin = P.so ? srow : P.ispin;
    const int ispp = min(ispin, P.nspin);
    const int indg = 3 - ispin;
    int ispq = min(indg, P.nspin);   // reassigned by an outer neighbour, as in the reference
    const int isp = min(ispin, nspino);
    const double VmE = c.vr[(i - 1) + (int64_t)S.npoint * (ispp - 1)] - P.enervide;
    double dr = VmE - S.clapl[0];
    if (P.rel) dr = dr - a2s4 * (VmE * VmE);
    if (lane == 0) add_c(env, P, tb, ii, ii, make_double2(dr, P.ecomp ? -P.eimag : 0.0), err, e);
    const double bder = (P.rel || P.so) ? -a2s4 / (1.0 - a2s4 * VmE) : 0.0;
    double cr[2] = {0.0, 0.0}, ci[2] = {0.0, 0.0};
    for (int iv = 0; iv < S.nvois; ++iv) {
      const int kind = S.nb_kind[(int64_t)k * S.nvois + iv];
      const int idx = S.nb_idx[(int64_t)k * S.nvois + iv];
      cr[isp - 1] = -S.clapl[iv + 1];
      ci[isp - 1] = 0.0;
      const int kax = 1 + (iv / 2) % 3;   // axis of the neighbour on the cubic grid
      if (P.rel) cr[isp - 1] = cr[isp - 1] + bder * S.cgrad[iv] * grad(kax, ispp);
      if (P.so) {
        double sr[2] = {0.0, 0.0}, si[2] = {0.0, 0.0};
        if (kax == 1) {
          si[isp - 1] = -grad(2, ispp);
          sr[indg - 1] = grad(3, ispq);
        } else if (kax == 2) {
          si[isp - 1] = grad(1, ispp);
          si[indg - 1] = -grad(3, ispq);
        } else {
          sr[indg - 1] = -grad(1, ispq) + grad(2, ispq);
        }
        for (int q = 0; q < 2; ++q) {
          sr[q] = bder * S.cgrad[iv] * sr[q];
          si[q] = bder * S.cgrad[iv] * si[q];
        }
        cr[isp - 1] = cr[isp - 1] + sr[isp - 1];
        cr[indg - 1] = sr[indg - 1];
        ci[0] = si[0];
        ci[1] = si[1];
      }
      for (int q = 0; q < nspino; ++q) {
        cr[q] = cr[q] * rvi;
        ci[q] = ci[q] * rvi;
      }
      if (kind == 0) {
        if (lane == 0) {
          const double rvj = S.rvol[idx - 1];
          for (int ispo = 1; ispo <= nspino; ++ispo)
            add_c(env, P, tb, ii, new_[idx] - nspino + ispo, make_double2(cr[ispo - 1] / rvj, ci[ispo - 1] / rvj),
                  err, e);
        }
      } else if (kind > 0) {
        const int ia = kind, ib = idx;
        const int nl = nlmsa[ia - 1];
        // the irregular solution's second column block: the irregular atomic solution
        for (int q = lane; q < P.nri * nl; q += 32) {
          const int iri = q / nl + 1, Lm = q % nl + 1;
          const int64_t t = (Lm - 1) + (int64_t)S.nlmsam * (ia - 1);
          const int L = S.lato[t], isol = S.iato[t], mb = S.mato[t];
          const int jjj = ianew[ia - 1] + Lm + (iri - 1) * nl;
          for (int ispo = 1; ispo <= nspino; ++ispo) {
            const int m = mb + ispo - isol;
            if (m > L || m < -L) continue;
            const int lm0 = L * L + L + 1 + m;
            const double2 v =
                P.so ? c_mul(make_double2(cr[ispo - 1], ci[ispo - 1]), phic(c, P, S, ib, lm0, ispo, isol, ia, iri))
                     : c_mul(make_double2(cr[isp - 1], ci[isp - 1]), phic(c, P, S, ib, lm0, ispp, isol, ia, iri));
            add_c(env, P, tb, ii, jjj, v, err, e);
          }
        }
      } else if (kind == -2) {
        const int ib = idx;
        for (int Lm = lane + 1; Lm <= P.nlmso; Lm += 32) {
          const int L = S.lso[Lm - 1], m = S.mso[Lm - 1], so_ = S.iso[Lm - 1];
          const int lm0 = L * L + L + 1 + m;
          const int iq = min(so_, P.nspinr);
          const int s = (isp == so_) ? isp : indg;
          const double2 cf = make_double2(cr[s - 1], ci[s - 1]);
          const double2 y = yso(P, S, ib, m, lm0);
          const double2 jv = besc(c, P, c.bes, S, ib, L, iq);
          if (!P.irr) {
            add_c(env, P, tb, ii, P.nligneso + Lm, c_mul(c_mul(colfac(c, P, S, basereel, ib, L, iq), y), cf), err, e);
          }
          // regular solution: the incoming j_l; irregular: -i j_l + n_l (no
          // scattered wave in the outer sphere)
          double2 rf = jv;
          if (P.irr) {
            const double2 nv = besc(c, P, c.neu, S, ib, L, iq);
            rf = make_double2(jv.y + nv.x, -jv.x + nv.y);
          }
          const double2 g = c_mul(c_mul(y, rf), cf);
          add_rhs_c(B, P, ii, Lm, make_double2(-g.x, -g.y));
        }
        ispq = min(S.iso[P.nlmso - 1], P.nspinr);
      }
    }
  }
}

// Outer rows x outer columns and their right-hand sides: one thread per (Lm, Lmp).
__global__ void __launch_bounds__(256) k_asmc_outer(const StaticDev* sites, const Prob* probs, const double* dpool,
                                                    double* env, double* B, Tables tb, int basereel, int* err) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  if (P.irr) return;   // the irregular solution has no outer-sphere rows
  const StaticDev& S = sites[P.site];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nlmso = P.nlmso;
  if (t >= nlmso * nlmso) return;
  const int Lm = t / nlmso + 1, Lmp = t % nlmso + 1;
  const int isp = S.iso[Lm - 1];
  if (S.iso[Lmp - 1] != isp) return;
  const CIn c = cin(P, S, dpool);
  const int m = S.mso[Lm - 1];
  const int lm0 = S.lso[Lm - 1] * S.lso[Lm - 1] + S.lso[Lm - 1] + 1 + m;
  const int L = S.lso[Lmp - 1], mp = S.mso[Lmp - 1];
  const int lmp0 = L * L + L + 1 + mp;
  const int iq = min(S.iso[Lmp - 1], P.nspinr);
  double2 charm = make_double2(0.0, 0.0), sm = make_double2(0.0, 0.0);
  for (int ib = 1; ib <= S.nsortf; ++ib) {
    const double po = S.poidso[ib - 1];
    // column factor: conj(Y_m) Y_mp (mat.f90:1428-1440)
    double2 cf;
    if (P.ylmc && m != 0 && mp != 0)
      cf = c_mul(c_conj(yc(m, ysot(S, ib, lm0), ysot(S, ib, lm0 - 2 * m))), yc(mp, ysot(S, ib, lmp0), ysot(S, ib, lmp0 - 2 * mp)));
    else if (P.ylmc && m != 0) {
      const double2 a = c_conj(yc(m, ysot(S, ib, lm0), ysot(S, ib, lm0 - 2 * m)));
      const double y = ysot(S, ib, lmp0);
      cf = make_double2(a.x * y, a.y * y);
    } else if (P.ylmc && mp != 0) {
      const double2 b = yc(mp, ysot(S, ib, lmp0), ysot(S, ib, lmp0 - 2 * mp));
      const double y = ysot(S, ib, lm0);
      cf = make_double2(y * b.x, y * b.y);
    } else {
      cf = make_double2(ysot(S, ib, lm0) * ysot(S, ib, lmp0), 0.0);
    }
    cf = make_double2(po * cf.x, po * cf.y);
    const double2 w = c_mul(cf, colfac(c, P, S, basereel, ib, L, iq));
    charm = make_double2(charm.x + w.x, charm.y + w.y);
    // right-hand side: poidso conj(Y_m) Y_mp j_L (mat.f90:1473-1508)
    double2 cb;
    if (P.ylmc && m != 0) {
      const double2 a = c_conj(yc(m, ysot(S, ib, lm0), ysot(S, ib, lm0 - 2 * m)));
      cb = make_double2(po * a.x, po * a.y);
    } else {
      cb = make_double2(po * ysot(S, ib, lm0), 0.0);
    }
    double2 cd;
    if (P.ylmc && mp != 0)
      cd = c_mul(cb, yc(mp, ysot(S, ib, lmp0), ysot(S, ib, lmp0 - 2 * mp)));
    else
      cd = c_mul(cb, make_double2(ysot(S, ib, lmp0), 0.0));
    cd = c_mul(cd, besc(c, P, c.bes, S, ib, L, iq));
    sm = make_double2(sm.x - cd.x, sm.y - cd.y);
  }
  const int ii = P.nligneso + Lm;
  add_c(env, P, tb, ii, P.nligneso + Lmp, charm, err, e);
  add_rhs_c(B, P, ii, Lmp, sm);
}

// Outer rows, boundary-point columns: one thread per (Lm, ib).
__global__ void __launch_bounds__(256) k_asmc_outer_bnd(const StaticDev* sites, const Prob* probs, const int* ipool,
                                                        double* env, Tables tb, int* err) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  if (P.irr) return;   // the irregular solution has no outer-sphere rows
  const StaticDev& S = sites[P.site];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= P.nlmso * S.nsortf) return;
  const int Lm = t / S.nsortf + 1, ib = t % S.nsortf + 1;
  const int* new_ = ipool + P.in_new;
  const int m = S.mso[Lm - 1];
  const int lm0 = S.lso[Lm - 1] * S.lso[Lm - 1] + S.lso[Lm - 1] + 1 + m;
  const int isp = S.iso[Lm - 1];
  const int j = S.isrt[ib - 1];
  const double rvj = S.rvol[j - 1];
  double2 v;
  if (P.ylmc && m != 0) {
    const double2 a = c_conj(yc(m, ysot(S, ib, lm0), ysot(S, ib, lm0 - 2 * m)));
    const double po = S.poidso[ib - 1];
    v = make_double2(-(po * a.x) / rvj, -(po * a.y) / rvj);
  } else {
    v = make_double2(-(S.poidso[ib - 1] * ysot(S, ib, lm0)) / rvj, 0.0);
  }
  add_c(env, P, tb, P.nligneso + Lm, new_[j] - S.nspino + isp, v, err, e);
}

// Atom rows: block per (atom, amplitude row).  The irregular solution has
// 2 nlmsa rows per atom (regular, then irregular amplitudes); its boundary
// points split in halves: a row's grid columns come from the half of its own
// atomic solution, each amplitude column block sums over the half of its
// atomic solution (mat.f90:1528-1627 with Test_reg = 0).
__global__ void __launch_bounds__(128) k_asmc_atom(const StaticDev* sites, const Prob* probs, const int* ipool,
                                                   const double* dpool, double* env, Tables tb, int max_nlm,
                                                   int* err) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  const StaticDev& S = sites[P.site];
  const int ia = blockIdx.x / max_nlm + 1;
  const int Ln = blockIdx.x % max_nlm + 1;
  const int* new_ = ipool + P.in_new;
  const int* ianew = ipool + P.in_ianew;
  const int* nlmsa = ipool + P.in_nlmsa;
  if (ia > S.natome) return;
  const int nl = nlmsa[ia - 1];
  if (Ln > P.nri * nl) return;
  const int iri = Ln > nl ? 2 : 1;
  const int Lm = Ln - (iri - 1) * nl;
  const CIn c = cin(P, S, dpool);
  const int64_t t0 = (Lm - 1) + (int64_t)S.nlmsam * (ia - 1);
  const int L = S.lato[t0], ispt = S.iato[t0], m = S.mato[t0];
  const int lm0 = L * L + L + 1 + m;
  const int ii = ianew[ia - 1] + Ln;
  const int nbf = S.nbordf[ia - 1];
  const int nhalf = nbf / 2;
  // boundary points of atomic solution r: all of them, or its half
  auto ib_lo = [&](int r) { return P.irr ? (r == 1 ? 1 : nhalf + 1) : 1; };
  auto ib_hi = [&](int r) { return P.irr ? (r == 1 ? nhalf : nbf) : nbf; };
  auto ycon = [&](int ib) -> double2 {   // conj of the row's harmonic at boundary point ib
    if (P.ylmc && m != 0) return c_conj(yc(m, ylmato(S, ib, lm0, ia), ylmato(S, ib, lm0 - 2 * m, ia)));
    return make_double2(ylmato(S, ib, lm0, ia), 0.0);
  };
  for (int ib = ib_lo(iri) + threadIdx.x; ib <= ib_hi(iri); ib += blockDim.x) {
    const int j = S.ibord[(ib - 1) + (int64_t)S.nbtm * (ia - 1)];
    const double po = S.poidsa[(ib - 1) + (int64_t)S.nbm * (ia - 1)];
    const double2 y = ycon(ib);
    const double rvj = S.rvol[j - 1];
    add_c(env, P, tb, ii, new_[j] - S.nspino + ispt, make_double2(-((po * y.x) / rvj), -((po * y.y) / rvj)), err, e);
  }
  const int ispint = P.so ? min(ispt, P.nspinp) : min(P.ispin, P.nspinp);
  for (int q = threadIdx.x; q < P.nri * nl; q += blockDim.x) {
    const int jri = q / nl + 1, Lmp = q % nl + 1;
    const int64_t t = (Lmp - 1) + (int64_t)S.nlmsam * (ia - 1);
    const int Lp = S.lato[t], isol = S.iato[t];
    const int mp = S.mato[t] + ispt - isol;
    if (mp > Lp || mp < -Lp) continue;
    const int lmp0 = Lp * Lp + Lp + 1 + mp;
    double sr = 0.0, si = 0.0;
    for (int ib = ib_lo(jri); ib <= ib_hi(jri); ++ib) {
      const double po = S.poidsa[(ib - 1) + (int64_t)S.nbm * (ia - 1)];
      const double2 f = c_mul(phic(c, P, S, ib, lmp0, ispint, isol, ia, jri), ycon(ib));
      sr = sr + po * f.x;
      si = si + po * f.y;
    }
    add_c(env, P, tb, ii, ianew[ia - 1] + Lmp + (jri - 1) * nl, make_double2(sr, si), err, e);
  }
}

// Taull of the absorber, unsymmetrised, into the scratch: T(a, b) = -i sum_f
// x(a, f) conj(x(b, f)), indexed (Lm0 - 1) + nlmq (s - 1) on both sides.
__global__ void k_taullc_raw(const StaticDev* sites, const Prob* probs, const double* X, double2* scratch) {
  const Prob P = probs[blockIdx.y];
  const StaticDev& S = sites[P.site];
  const int nlm = P.nlm_abs;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nlm * nlm) return;
  const int a = t / nlm + 1, b = t % nlm + 1;
  const int nsp = S.nspino, nlmq = nlm / nsp;
  const int64_t ta = (a - 1) + (int64_t)S.nlmsam * (P.iaabs - 1), tbi = (b - 1) + (int64_t)S.nlmsam * (P.iaabs - 1);
  const int L1 = S.lato[ta], m1 = S.mato[ta], is1 = P.so ? S.iato[ta] : 1;
  const int L2 = S.lato[tbi], m2 = S.mato[tbi], is2 = nsp == 2 ? S.iato[tbi] : 1;
  const int row = (L1 * L1 + L1 + m1) + nlmq * (is1 - 1), col = (L2 * L2 + L2 + m2) + nlmq * (is2 - 1);
  const int ii = P.ianew_abs + a, jj = P.ianew_abs + b;
  const int p1r = P.n - (2 * ii - 1), p1i = P.n - 2 * ii, p2r = P.n - (2 * jj - 1), p2i = P.n - 2 * jj;
  auto xv = [&](int p, int f) {
    return X[P.rhs + ((int64_t)(p / TS) * P.nrt + f / TS) * TS2 + (p % TS) * TS + (f % TS)];
  };
  double2 cf = make_double2(0.0, 0.0);
  for (int f = 0; f < P.nlmso; ++f) {
    const double2 a1 = make_double2(xv(p1r, f), xv(p1i, f));
    const double2 a2 = make_double2(xv(p2r, f), -xv(p2i, f));
    const double2 ia1 = make_double2(-a1.y, a1.x);   // i * a1
    const double2 z = c_mul(ia1, a2);
    cf = make_double2(cf.x - z.x, cf.y - z.y);
  }
  scratch[P.scratch + row + (int64_t)nlm * col] = cf;
}

// Symmetrisation (mat.f90:594-644): none with spin-orbit and two spin blocks;
// with complex harmonics T(a, b) and (-1)^(m1+m2) T(b~, a~) (m -> -m) averaged;
// otherwise i Im(T).
__global__ void k_taullc_sym(const StaticDev* sites, const Prob* probs, const double2* scratch, double2* taull) {
  const Prob P = probs[blockIdx.y];
  const StaticDev& S = sites[P.site];
  const int nlm = P.nlm_abs;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nlm * nlm) return;
  const int nsp = S.nspino, nlmq = nlm / nsp;
  const int row = t % nlm, col = t / nlm;
  const double2 v = scratch[P.scratch + t];
  double2 out;
  if (P.so && P.nspin == 2) {
    out = v;
  } else if (P.ylmc) {
    // row = lm0 - 1 with lm0 = L^2 + L + 1 + m (nsp = 1 here)
    int L1 = 0;
    while ((L1 + 1) * (L1 + 1) <= row) ++L1;
    int L2 = 0;
    while ((L2 + 1) * (L2 + 1) <= col) ++L2;
    const int m1 = row - (L1 * L1 + L1), m2 = col - (L2 * L2 + L2);
    const int prow = col - 2 * m2, pcol = row - 2 * m1;
    const double sg = ((m1 + m2) & 1) ? -1.0 : 1.0;
    const double2 w = scratch[P.scratch + prow + (int64_t)nlm * pcol];
    out = make_double2(0.5 * (v.x + sg * w.x), 0.5 * (v.y + sg * w.y));
  } else {
    out = make_double2(0.0, v.y);
  }
  (void)nlmq;
  taull[P.taull + t] = out;
}

// Tau_RI of FDM_comp (mat.f90:219-292): one thread per (Lm1, Lm2, i_RI) of
// the absorber, Tau_RI(Lm1 s1, Lm2 s2, i_RI) = sum_f Ampl(f, Lm1)
// Ampl_I(f, (i_RI - 1) nlmsa + Lm2): the regular problem's amplitudes times
// the irregular problem's (regular atomic solution, then irregular); no
// conjugate and no symmetrisation.  Indexed like Taull, i_RI outermost.
__global__ void k_tau_ri(const StaticDev* sites, const Prob* preg, const Prob* pirr, const double* X,
                         double2* out) {
  const Prob P = *preg, Q = *pirr;
  const StaticDev& S = sites[P.site];
  const int nlm = P.nlm_abs;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 2 * nlm * nlm) return;
  const int iri = t / (nlm * nlm) + 1, r = t % (nlm * nlm);
  const int a = r / nlm + 1, b = r % nlm + 1;
  const int nsp = S.nspino, nlmq = nlm / nsp;
  const int64_t ta = (a - 1) + (int64_t)S.nlmsam * (P.iaabs - 1), tbi = (b - 1) + (int64_t)S.nlmsam * (P.iaabs - 1);
  const int L1 = S.lato[ta], m1 = S.mato[ta], is1 = P.so ? S.iato[ta] : 1;
  const int L2 = S.lato[tbi], m2 = S.mato[tbi], is2 = P.so ? S.iato[tbi] : 1;
  const int row = (L1 * L1 + L1 + m1) + nlmq * (is1 - 1), col = (L2 * L2 + L2 + m2) + nlmq * (is2 - 1);
  const int ii = P.ianew_abs + a, jj = Q.ianew_abs + (iri - 1) * nlm + b;
  const int pr = P.n - (2 * ii - 1), pi = P.n - 2 * ii, qr = Q.n - (2 * jj - 1), qi = Q.n - 2 * jj;
  auto xv = [&](const Prob& R, int p, int f) {
    return X[R.rhs + ((int64_t)(p / TS) * R.nrt + f / TS) * TS2 + (p % TS) * TS + (f % TS)];
  };
  double2 cf = make_double2(0.0, 0.0);
  for (int f = 0; f < P.nlmso; ++f) {
    const double2 z = c_mul(make_double2(xv(P, pr, f), xv(P, pi, f)), make_double2(xv(Q, qr, f), xv(Q, qi, f)));
    cf = make_double2(cf.x + z.x, cf.y + z.y);
  }
  out[row + (int64_t)nlm * col + (int64_t)nlm * nlm * (iri - 1)] = cf;
}

}  // namespace

void launch_tau_ri(const StaticDev* sites, const Prob* preg, const Prob* pirr, const double* X, int nlm, double2* out,
                   cudaStream_t s) {
  const int n = 2 * nlm * nlm;
  if (n <= 0) return;
  k_tau_ri<<<(n + 127) / 128, 128, 0, s>>>(sites, preg, pirr, X, out);
}

void launch_assemble_c(const StaticDev* sites, const Prob* probs, const Pools& pl, Tables tb, const LaunchDims& d,
                       int basereel, cudaStream_t s) {
  const int np = d.nprob;
  k_asmc_pad<<<dim3(1, np), TS, 0, s>>>(probs, pl.env64, tb, pl.err);
  if (d.npr > 0)
    k_asmc_grid<<<dim3((d.npr + 7) / 8, np), 256, 0, s>>>(sites, probs, pl.ipool, pl.dpool, pl.env64, pl.B64, tb,
                                                          basereel, pl.err);
  const int nsq = d.max_nlmso * d.max_nlmso;
  k_asmc_outer<<<dim3((nsq + 255) / 256, np), 256, 0, s>>>(sites, probs, pl.dpool, pl.env64, pl.B64, tb, basereel,
                                                           pl.err);
  const int nb = d.max_nlmso * d.max_nsortf;
  if (nb > 0)
    k_asmc_outer_bnd<<<dim3((nb + 255) / 256, np), 256, 0, s>>>(sites, probs, pl.ipool, pl.env64, tb, pl.err);
  if (d.max_natome > 0 && d.max_nlmsa > 0)
    k_asmc_atom<<<dim3(d.max_natome * d.max_nlmsa, np), 128, 0, s>>>(sites, probs, pl.ipool, pl.dpool, pl.env64, tb,
                                                                     d.max_nlmsa, pl.err);
}

void launch_taull_c(const StaticDev* sites, const Prob* probs, const Pools& pl, const LaunchDims& d, int max_nlm,
                    cudaStream_t s) {
  const int n2 = max_nlm * max_nlm;
  if (n2 <= 0) return;
  double2* scratch = reinterpret_cast<double2*>(pl.tscratch);
  k_taullc_raw<<<dim3((n2 + 127) / 128, d.nprob), 128, 0, s>>>(sites, probs, pl.X64, scratch);
  k_taullc_sym<<<dim3((n2 + 127) / 128, d.nprob), 128, 0, s>>>(sites, probs, scratch,
                                                               reinterpret_cast<double2*>(pl.taull));
}

}  // namespace fdm
