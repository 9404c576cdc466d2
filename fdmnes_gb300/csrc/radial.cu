// radial.cu - the per-energy inputs of the real path generated on the device:
// the atomic boundary functions phiato (Sphere -> Sch_radial -> cal_phiato,
// source/sphere.f90:8,324-733,3186-3370) and the outer-sphere Bessel and
// Neumann values (phiso's real branch, source/mat.f90:739-1028, with
// cbessneur, source/sphere.f90:7356-7384).  All in FP64.
//
// Radial solution.  For every problem, atom type t and L <= lmax, the regular
// solution u_L of the radial Schroedinger equation is integrated outwards on
// the type's radial mesh by the three-point recursion of coef_sch_rad /
// Sch_radial (source/sphere.f90:324-396 coefficients, :583-695 recursion):
//   u(i+1) = -((c0(i) - E + L(L+1)/r_i^2) u(i) + gm(i) u(i-1)) / gp(i),
// where c0 = -clapl0 + V(r) + dV(spin) holds the energy-independent part,
// started from the expansion at the origin (:519-523)
//   u = (1 + br r + cr r^2) r^(L+1),  br = -Z/(L+1),  cr = -(2 Z br + Ekin)/(4L+6),
// and R_L = u / r.  One thread per (type, L) of a problem: the recursion is
// sequential in r.
//
// cal_phiato (source/sphere.f90:3225-3370): R_L at each boundary point of an
// atom by quadratic interpolation through the three mesh points around its
// distance (f_interp2, source/tools.f90:504-522), times the real harmonic
// Ylmato of the point.  The interpolation indices are static (host tables).
#include <cuda_runtime.h>

#include "fdm_internal.cuh"
#include "fdm_kernels.h"

namespace fdm {

namespace {

// Products and sums without contraction into FMA, in the order the host
// restatement (numpy) evaluates them, so both give the same FP64 values.
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }

// R_L(r_i) of problem e, type t, degree L at U[((e * ntype + t) * lmax1 + L) * nr_max + i].
__global__ void k_radial(const Prob* probs, const RadialDev* rads, int nprob, int lmax1, double* U) {
  const int e = blockIdx.y;
  if (e >= nprob) return;
  const Prob P = probs[e];
  if (!P.gen) return;
  const RadialDev& R = rads[P.site];
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int t = q / lmax1, L = q % lmax1;
  if (t >= R.ntype || t >= MAX_GEN_TYPES || L > P.gen_lmax[t]) return;
  const int nr = R.nr[t];
  const double* r = R.r + (int64_t)t * R.nr_max;
  const double* mcl0 = R.mcl0 + (int64_t)t * R.nr_max;
  const double* V = R.V + (int64_t)t * R.nr_max;
  const double* gm = R.gm + (int64_t)t * R.nr_max;
  const double* gp = R.gp + (int64_t)t * R.nr_max;
  const double* f2 = R.f2 + (int64_t)t * R.nr_max;
  const int isp = min(P.ispin, R.nspin);
  const double dvs = R.dv_spin[isp - 1];
  const double ecs = sub(P.enervide, add(R.v0bd, dvs));
  const double Z = R.z_origin[t];
  const double br = -Z / (L + 1.0);
  const double cr = -add(mul(mul(2.0, Z), br), ecs) / (4.0 * L + 6.0);
  const double p = L + 1.0;
  double* u = U + (((int64_t)e * R.ntype + t) * lmax1 + L) * R.nr_max;
  double uv[2];
  for (int i = 0; i < 2; ++i) {
    const double x = r[i];
    uv[i] = mul(add(add(1.0, mul(br, x)), mul(cr, mul(x, x))), pow(x, p));
    u[i] = uv[i] / x;
  }
  double um = uv[0], u0 = uv[1];
  const double L2 = (double)(L * (L + 1));
  for (int i = 1; i < nr - 1; ++i) {
    const double g0 = add(mcl0[i], sub(add(V[i], dvs), P.enervide));
    const double td = add(g0, mul(L2, f2[i]));
    const double up = -add(mul(td, u0), mul(gm[i], um)) / gp[i];
    um = u0;
    u0 = up;
    u[i + 1] = up / r[i + 1];
  }
}

// phiato(ib, lm, ia) of problem e, written at dpool + P.in_phi as (nbtm, nlmagm, natome).
__global__ void k_phiato(const Prob* probs, const RadialDev* rads, const StaticDev* sites, const int* ipool,
                         int nprob, int lmax1, const double* U, double* dpool) {
  const int e = blockIdx.z;
  if (e >= nprob) return;
  const Prob P = probs[e];
  if (!P.gen) return;
  const RadialDev& R = rads[P.site];
  const StaticDev& S = sites[P.site];
  const int ia = blockIdx.y;
  if (ia >= S.natome) return;
  const int t = R.itype[ia];
  const int nlmsa = ipool[P.in_nlmsa + ia];
  double* phi = dpool + P.in_phi + (int64_t)S.nbtm * P.nlmagm * ia;
  const int nb = S.nbord[ia];
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < S.nbtm * P.nlmagm; idx += gridDim.x * blockDim.x) {
    const int ib = idx % S.nbtm, lm = idx / S.nbtm;
    double v = 0.0;
    if (ib < nb && lm < nlmsa) {
      int L = 0;
      while ((L + 1) * (L + 1) <= lm) ++L;
      const int k = R.iidx[ib + (int64_t)S.nbtm * ia];  // first mesh point beyond rrel, 0-based, >= 2
      const double* r = R.r + (int64_t)t * R.nr_max;
      const double* u = U + (((int64_t)e * R.ntype + t) * lmax1 + L) * R.nr_max;
      const double x = R.rrel[ib + (int64_t)S.nbtm * ia];
      const double rm = r[k - 2], r0 = r[k - 1], rp = r[k];
      const double fm = u[k - 2], f0 = u[k - 1], fp = u[k];
      // f_interp2: the parabola through the three points, evaluated at x
      const double dp0 = sub(rp, r0), dpm = sub(rp, rm), d0m = sub(r0, rm);
      const double a = add(sub(mul(fm, dp0), mul(f0, dpm)), mul(fp, d0m)) / mul(mul(d0m, dp0), dpm);
      const double b = sub(sub(f0, fm) / d0m, mul(a, add(r0, rm)));
      const double c = sub(sub(f0, mul(a, mul(r0, r0))), mul(b, r0));
      const double f = add(add(mul(a, mul(x, x)), mul(b, x)), c);
      v = mul(f, S.Ylmato[ib + (int64_t)S.nbtm * (lm + (int64_t)S.nlmmax * ia)]);
    }
    phi[ib + (int64_t)S.nbtm * lm] = v;
  }
}

// fnorm j_l(k r_b), fnorm n_l(k r_b) for l <= lmaxso at every outer point, as
// [ib][l] at dpool + P.in_bes / P.in_neu; k = sqrt(Ekin), fnorm = sqrt(k/pi).
__global__ void k_bessel(const Prob* probs, const RadialDev* rads, const StaticDev* sites, int nprob, double* dpool) {
  const int e = blockIdx.y;
  if (e >= nprob) return;
  const Prob P = probs[e];
  if (!P.gen) return;
  const RadialDev& R = rads[P.site];
  const StaticDev& S = sites[P.site];
  const int ib = blockIdx.x * blockDim.x + threadIdx.x;
  if (ib >= S.nsort) return;
  const int isp = min(P.ispin, R.nspin);
  const double ecin = sub(P.enervide, add(R.v0bd, R.dv_spin[isp - 1]));
  const double konder = sqrt(ecin);
  const double fnorm = sqrt(konder / 3.14159265358979323846);
  const double z = mul(konder, R.rsort[ib]);
  const int nl = P.lmaxso + 1;
  double* bs = dpool + P.in_bes + (int64_t)ib * nl;
  double* nm = dpool + P.in_neu + (int64_t)ib * nl;
  double s, c;
  sincos(z, &s, &c);
  double n0 = mul(-fnorm, c) / z, b0 = mul(fnorm, s) / z;
  nm[0] = n0;
  bs[0] = b0;
  if (nl == 1) return;
  double n1 = sub(n0 / z, b0), b1 = add(b0 / z, n0);
  nm[1] = n1;
  bs[1] = b1;
  for (int L = 2; L < nl; ++L) {
    const double L1 = 2 * L - 1;
    const double n2 = sub(mul(L1, n1) / z, n0), b2 = sub(mul(L1, b1) / z, b0);
    nm[L] = n2;
    bs[L] = b2;
    n0 = n1;
    n1 = n2;
    b0 = b1;
    b1 = b2;
  }
}

}  // namespace

void launch_generate_inputs(const Prob* probs, const RadialDev* rads, const StaticDev* sites, const int* ipool,
                            const LaunchDims& d, const GenDims& g, double* U, double* dpool, cudaStream_t s) {
  if (g.nprob_gen == 0) return;
  const int nq = g.ntype_max * g.lmax1;
  k_radial<<<dim3((nq + 31) / 32, d.nprob), 32, 0, s>>>(probs, rads, d.nprob, g.lmax1, U);
  k_phiato<<<dim3(8, g.natome_max, d.nprob), 256, 0, s>>>(probs, rads, sites, ipool, d.nprob, g.lmax1, U, dpool);
  k_bessel<<<dim3((g.nsort_max + 127) / 128, d.nprob), 128, 0, s>>>(probs, rads, sites, d.nprob, dpool);
}

}  // namespace fdm
