// assemble.cu - FP64 assembly of the FDM matrix and right-hand sides on the GPU.
//
// Restates calcMatRow (source/mat.f90:1034-1632), real-arithmetic branch, for
// all rows of all problems of a batch at once, writing directly into the
// reversed-order band tiles (see fdm_internal.cuh) and the RHS tiles:
//   k_asm_grid   grid-point rows  (mat.f90:1142-1402), one warp per point
//   k_asm_outer_tiled, k_asm_outer_bnd  outer-sphere rows (mat.f90:1405-1511)
//   k_asm_atom   atom-expansion rows (mat.f90:1515-1632)
// Within every matrix entry the contributions are summed in the reference's
// order (neighbours iv = 1..nvois; boundary points ib ascending).
#include "fdm_internal.cuh"
#include "fdm_kernels.h"

namespace fdm {

// Address of band entry (p, q); nullptr (and an error flag) when (p, q) lies
// outside the stored strip of row p, i.e. when the caller's lb1/lb2 do not
// cover a column that calcMatRow writes.
__device__ __forceinline__ double* env_at(double* env, const Prob& P, const Tables& tb, int p, int q, int* err,
                                          int e) {
  const int I = p / TS, J = q / TS;
  if (p < 0 || p >= P.nt * TS || q < 0 || J < tb.J0[P.trow + I] || J > tb.J1[P.trow + I]) {
    atomicExch(&err[e], (int)FDMGPU_ERR_ARG);
    return nullptr;
  }
  return tile_ptr(env, P, tb, I, J) + (p % TS) * TS + (q % TS);
}
__device__ __forceinline__ double* rhs_at(double* rhs, const Prob& P, int p, int r) {
  return rhs_ptr(rhs, P, p / TS, r / TS) + (p % TS) * TS + (r % TS);
}

// Identity on the padding rows n..npad-1.
__global__ void k_asm_pad(const Prob* probs, double* env, Tables tb, int* err) {
  const Prob P = probs[blockIdx.y];
  const int p = P.n + threadIdx.x;
  if (p < P.nt * TS) {
    double* a = env_at(env, P, tb, p, p, err, blockIdx.y);
    if (a) *a = 1.0;
  }
}

// Grid-point rows: one warp per interstitial point.
__global__ void __launch_bounds__(256) k_asm_grid(const StaticDev* sites, const Prob* probs, const int* ipool,
                                                  const double* dpool, double* env, double* B, Tables tb, int* err) {
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
  const double* Vr = dpool + P.in_vr;
  const double* phi = dpool + P.in_phi;
  const double* bes = dpool + P.in_bes;
  const double* neu = dpool + P.in_neu;
  const int ii = new_[i];
  const int p = P.n - ii;
  if (lane == 0) {
    double* a = env_at(env, P, tb, p, p, err, e);
    if (a) *a = (Vr[i - 1] - P.enervide) - S.clapl[0];
  }
  for (int iv = 0; iv < S.nvois; ++iv) {
    const int kind = S.nb_kind[(int64_t)k * S.nvois + iv];
    const int idx = S.nb_idx[(int64_t)k * S.nvois + iv];
    const double cf = S.nb_coef[(int64_t)k * S.nvois + iv];
    if (kind == 0) {
      if (lane == 0) {
        double* a = env_at(env, P, tb, p, P.n - new_[idx], err, e);
        if (a) *a = *a + cf / S.rvol[idx - 1];
      }
    } else if (kind > 0) {
      const int ia = kind, ib = idx;
      const int nlm = nlmsa[ia - 1];
      for (int Lm = lane + 1; Lm <= nlm; Lm += 32) {
        const int L = S.lato[(Lm - 1) + (int64_t)S.nlmsam * (ia - 1)];
        const int m = S.mato[(Lm - 1) + (int64_t)S.nlmsam * (ia - 1)];
        const int Lm0 = L * L + L + 1 + m;
        const double ph = phi[(ib - 1) + (int64_t)S.nbtm * ((Lm0 - 1) + (int64_t)P.nlmagm * (ia - 1))];
        double* a = env_at(env, P, tb, p, P.n - (ianew[ia - 1] + Lm), err, e);
        if (a) *a = *a + cf * ph;
      }
    } else if (kind == -2) {
      const int ib = idx;
      const int nl = P.lmaxso + 1;
      for (int Lm = lane + 1; Lm <= P.nlmso; Lm += 32) {
        const int L = S.lso[Lm - 1], m = S.mso[Lm - 1];
        const int Lm0 = L * L + L + 1 + m;
        const double y = S.YsoT[(int64_t)(ib - 1) * S.nlmomax + (Lm0 - 1)];
        double* a = env_at(env, P, tb, p, P.n - (P.nligneso + Lm), err, e);
        const double fr = y * neu[(int64_t)(ib - 1) * nl + L];
        if (a) *a = *a + cf * fr;
        double* b = rhs_at(B, P, p, Lm - 1);
        const double fb = y * bes[(int64_t)(ib - 1) * nl + L];
        *b = *b - cf * fb;
      }
    }
  }
}

// Outer-sphere rows (mat.f90:1405-1511): the outer block and the right-hand
// side are sums over the outer boundary points ib,
//   A(Lm, Lmp) = sum_ib W(ib, Lm) N(ib, Lmp),  B(Lm, Lmp) = -sum_ib W(ib, Lm) J(ib, Lmp)
// with W = poidso(ib) Y(ib, Lm), N = Y(ib, Lmp) neumann(ib, l(Lmp)) and
// J = Y(ib, Lmp) bessel(ib, l(Lmp)): a product of two (nsortf x nlmso) panels,
// run as a tiled FP64 product (32 x 32 outputs per block, 2 x 2 per thread,
// the panels' 32-point chunks computed once per block into shared memory), two
// FMAs per term; ib ascending as in the reference, the product grouped as
// W (Y n) where the reference forms (W Y) n.
__global__ void __launch_bounds__(256) k_asm_outer_tiled(const StaticDev* sites, const Prob* probs, const double* dpool,
                                                         double* env, double* B, Tables tb, int* err) {
  const int e = blockIdx.z;
  const Prob P = probs[e];
  const StaticDev& S = sites[P.site];
  const int nlmso = P.nlmso;
  const int m0 = blockIdx.y * 32, q0 = blockIdx.x * 32;
  if (m0 >= nlmso || q0 >= nlmso) return;
  const int nl = P.lmaxso + 1;
  const double* bes = dpool + P.in_bes;
  const double* neu = dpool + P.in_neu;
  __shared__ double W[32][33], Nn[32][33], Jb[32][33];
  const int t = threadIdx.x, tx = t % 16, ty = t / 16;
  double an[2][2] = {{0.0, 0.0}, {0.0, 0.0}}, ab[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
  for (int ib0 = 0; ib0 < S.nsortf; ib0 += 32) {
    for (int q = t; q < 32 * 32; q += 256) {
      const int i = q / 32, c = q % 32, ib = ib0 + i;
      double w = 0.0, vn = 0.0, vb = 0.0;
      if (ib < S.nsortf) {
        const double* yrow = S.YsoT + (int64_t)ib * S.nlmomax;
        const int Lm = m0 + c;
        if (Lm < nlmso) {
          const int l = S.lso[Lm];
          w = S.poidso[ib] * yrow[l * l + l + S.mso[Lm]];
        }
        const int Lmp = q0 + c;
        if (Lmp < nlmso) {
          const int l = S.lso[Lmp];
          const double y = yrow[l * l + l + S.mso[Lmp]];
          vn = y * neu[(int64_t)ib * nl + l];
          vb = y * bes[(int64_t)ib * nl + l];
        }
      }
      W[i][c] = w;
      Nn[i][c] = vn;
      Jb[i][c] = vb;
    }
    __syncthreads();
    const int ni = min(32, S.nsortf - ib0);
    for (int i = 0; i < ni; ++i) {
      const double w0 = W[i][2 * ty], w1 = W[i][2 * ty + 1];
      const double n0 = Nn[i][2 * tx], n1 = Nn[i][2 * tx + 1];
      const double b0 = Jb[i][2 * tx], b1 = Jb[i][2 * tx + 1];
      an[0][0] = fma(w0, n0, an[0][0]);
      an[0][1] = fma(w0, n1, an[0][1]);
      an[1][0] = fma(w1, n0, an[1][0]);
      an[1][1] = fma(w1, n1, an[1][1]);
      ab[0][0] = fma(-w0, b0, ab[0][0]);
      ab[0][1] = fma(-w0, b1, ab[0][1]);
      ab[1][0] = fma(-w1, b0, ab[1][0]);
      ab[1][1] = fma(-w1, b1, ab[1][1]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 2; ++b) {
      const int Lm = m0 + 2 * ty + a + 1, Lmp = q0 + 2 * tx + b + 1;
      if (Lm > nlmso || Lmp > nlmso) continue;
      const int p = P.n - (P.nligneso + Lm);
      double* ap = env_at(env, P, tb, p, P.n - (P.nligneso + Lmp), err, e);
      if (ap) *ap = an[a][b];
      *rhs_at(B, P, p, Lmp - 1) = ab[a][b];
    }
}

// The boundary-point columns of the outer-sphere rows.
__global__ void __launch_bounds__(256) k_asm_outer_bnd(const StaticDev* sites, const Prob* probs, const int* ipool, double* env,
                                                       Tables tb, int* err) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  const StaticDev& S = sites[P.site];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= P.nlmso * S.nsortf) return;
  const int Lm = t / S.nsortf + 1, ib = t % S.nsortf + 1;
  const int* new_ = ipool + P.in_new;
  const int Lm0 = S.lso[Lm - 1] * S.lso[Lm - 1] + S.lso[Lm - 1] + 1 + S.mso[Lm - 1];
  const int j = S.isrt[ib - 1];
  const double fac = S.poidso[ib - 1] * S.YsoT[(int64_t)(ib - 1) * S.nlmomax + (Lm0 - 1)];
  const int p = P.n - (P.nligneso + Lm);
  double* a = env_at(env, P, tb, p, P.n - new_[j], err, e);
  if (a) *a = *a - fac / S.rvol[j - 1];
}

// Atom rows: block per (atom, harmonic row); threads over the own-block
// columns and then over the boundary points.
__global__ void __launch_bounds__(128) k_asm_atom(const StaticDev* sites, const Prob* probs, const int* ipool, const double* dpool,
                                                  double* env, Tables tb, int max_nlm, int* err) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  const StaticDev& S = sites[P.site];
  const int ia = blockIdx.x / max_nlm + 1;
  const int Lm = blockIdx.x % max_nlm + 1;
  const int* new_ = ipool + P.in_new;
  const int* ianew = ipool + P.in_ianew;
  const int* nlmsa = ipool + P.in_nlmsa;
  if (ia > S.natome || Lm > nlmsa[ia - 1]) return;
  const double* phi = dpool + P.in_phi;
  const int L = S.lato[(Lm - 1) + (int64_t)S.nlmsam * (ia - 1)];
  const int m = S.mato[(Lm - 1) + (int64_t)S.nlmsam * (ia - 1)];
  const int Lm0 = L * L + L + 1 + m;
  const int ii = ianew[ia - 1] + Lm;
  const int p = P.n - ii;
  const int nbf = S.nbordf[ia - 1];
  const double* ya = S.Ylmato + (int64_t)S.nbtm * ((Lm0 - 1) + (int64_t)S.nlmmax * (ia - 1));
  for (int ib = 1 + threadIdx.x; ib <= nbf; ib += blockDim.x) {
    const int j = S.ibord[(ib - 1) + (int64_t)S.nbtm * (ia - 1)];
    const int isym = abs(S.isbord[(ib - 1) + (int64_t)S.nbtm * (ia - 1)]);
    const double f = S.poidsa[(ib - 1) + (int64_t)S.nbm * (ia - 1)] * S.Kar[isym - 1] / S.rvol[j - 1];
    double* a = env_at(env, P, tb, p, P.n - new_[j], err, e);
    if (a) *a = *a - f * ya[ib - 1];
  }
  for (int Lmp = 1 + threadIdx.x; Lmp <= nlmsa[ia - 1]; Lmp += blockDim.x) {
    const int Lp = S.lato[(Lmp - 1) + (int64_t)S.nlmsam * (ia - 1)];
    const int mp = S.mato[(Lmp - 1) + (int64_t)S.nlmsam * (ia - 1)];
    const int Lmp0 = Lp * Lp + Lp + 1 + mp;
    const double* ph = phi + (int64_t)S.nbtm * ((Lmp0 - 1) + (int64_t)P.nlmagm * (ia - 1));
    double charm = 0.0;
    for (int ib = 1; ib <= nbf; ++ib)
      charm = charm + S.poidsa[(ib - 1) + (int64_t)S.nbm * (ia - 1)] * ya[ib - 1] * ph[ib - 1];
    double* a = env_at(env, P, tb, p, P.n - (ianew[ia - 1] + Lmp), err, e);
    if (a) *a = *a + charm;
  }
}

void launch_assemble(const StaticDev* sites, const Prob* probs, const Pools& pl, Tables tb, const LaunchDims& d,
                     cudaStream_t s) {
  const int np = d.nprob;
  k_asm_pad<<<dim3(1, np), TS, 0, s>>>(probs, pl.env64, tb, pl.err);
  if (d.npr > 0)
    k_asm_grid<<<dim3((d.npr + 7) / 8, np), 256, 0, s>>>(sites, probs, pl.ipool, pl.dpool, pl.env64, pl.B64, tb,
                                                         pl.err);
  const int nb32 = (d.max_nlmso + 31) / 32;
  if (nb32 > 0)
    k_asm_outer_tiled<<<dim3(nb32, nb32, np), 256, 0, s>>>(sites, probs, pl.dpool, pl.env64, pl.B64, tb, pl.err);
  const int nb = d.max_nlmso * d.max_nsortf;
  if (nb > 0)
    k_asm_outer_bnd<<<dim3((nb + 255) / 256, np), 256, 0, s>>>(sites, probs, pl.ipool, pl.env64, tb, pl.err);
  if (d.max_natome > 0 && d.max_nlmsa > 0)
    k_asm_atom<<<dim3(d.max_natome * d.max_nlmsa, np), 128, 0, s>>>(sites, probs, pl.ipool, pl.dpool, pl.env64, tb,
                                                                    d.max_nlmsa, pl.err);
}

}  // namespace fdm
