// gmres.cu - GMRES-based iterative refinement (GMRES-IR) of the mixed path.
//
// Classical refinement x <- x + LU^-1 r stalls or diverges when the FP32
// factors of the indefinite FDM matrix are poor (small pivots in the atomic
// harmonic blocks at some energies).  GMRES-IR (Carson & Higham, SIAM J. Sci.
// Comput. 40, 2018) instead solves each correction equation A d = r with
// GMRES on the left-preconditioned operator (LU)^-1 A, which converges even
// when ||I - (LU)^-1 A|| is near or above one.
//
// Everything below runs on the equilibrated system  Dr A Dc  (FP32 CSR copy
// "valS") with the tile-pivoted FP32 LU as preconditioner, independently for
// every problem and every right-hand-side column.  Vectors use the RHS tile
// layout of fdm_internal.cuh.  Per column, GMRES(m) keeps the Hessenberg
// matrix in Givens-reduced form (H, cs, sn, g).  A problem leaves the inner
// loop (inner_active = 0) once all its columns reach |g_{j+1}| <= tol * beta.
#include "fdm_internal.cuh"
#include "fdm_kernels.h"

namespace fdm {

constexpr int GM_MAX = 16;  // largest Krylov dimension supported

struct GmresState {          // per right-hand-side column
  float H[GM_MAX * (GM_MAX + 1)];  // column-major, H[i + j*(GM_MAX+1)]
  float cs[GM_MAX], sn[GM_MAX];
  float g[GM_MAX + 1];
  float beta;
  int done;                  // column converged or empty
  int nsteps;                // Arnoldi steps taken while the column was open
};

__device__ __forceinline__ int64_t vidx(const Prob& P, int p, int R, int c) {
  return P.rhs + ((int64_t)(p / TS) * P.nrt + R) * TS2 + (p % TS) * TS + c;
}

// valS = float(rs(p) * a(p,q) * cs(q)): the equilibrated FP32 matrix in CSR.
__global__ void k_csr_scale(const Prob* probs, const int* rowptr, const int* col, const double* val, const double* rs,
                            const double* cs, float* valS) {
  const Prob P = probs[blockIdx.y];
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P.nt * TS) return;
  const double r = rs[P.rowv + p];
  const int k1 = min(rowptr[P.rowv + p + 1], (int)P.csr_cap);
  for (int k = rowptr[P.rowv + p]; k < k1; ++k)
    valS[P.csr + k] = (float)(r * val[P.csr + k] * cs[P.rowv + col[P.csr + k]]);
}

// W = (Dr A Dc) V for active problems: warp per row, lanes over columns.
__global__ void k_spmv32(const Prob* probs, const int* rowptr, const int* col, const float* valS, const float* V,
                         float* W, const int* active) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  if (!active[e]) return;
  const int p = blockIdx.x * 8 + threadIdx.x / 32, lane = threadIdx.x % 32;
  if (p >= P.nt * TS) return;
  const int k0 = rowptr[P.rowv + p], k1 = min(rowptr[P.rowv + p + 1], (int)P.csr_cap);
  const int nrhs = P.nrt * TS;
  for (int r0 = 0; r0 < nrhs; r0 += 256) {
    float acc[8];
#pragma unroll
    for (int t = 0; t < 8; ++t) acc[t] = 0.f;
    for (int k = k0; k < k1; ++k) {
      const int q = col[P.csr + k];
      const float a = valS[P.csr + k];
      const float* vr = V + P.rhs + ((int64_t)(q / TS) * P.nrt) * TS2 + (q % TS) * TS;
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const int r = r0 + lane + 32 * t;
        if (r < nrhs) acc[t] = fmaf(a, vr[(int64_t)(r / TS) * TS2 + (r % TS)], acc[t]);
      }
    }
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const int r = r0 + lane + 32 * t;
      if (r < nrhs) W[vidx(P, p, r / TS, r % TS)] = acc[t];
    }
  }
}

// Block per (problem, RHS tile R): 64 columns x 4 row groups.
// Start of a GMRES cycle: Z holds z0 = LU^-1 r; beta = ||z0||, V0 = z0 / beta.
__global__ void k_gmres_start(const Prob* probs, const float* Z, float* V0, GmresState* st, const int* active,
                              int* inner_active, int* jdone, int* notconv) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  const int R = blockIdx.x;
  if (threadIdx.x == 0 && R == 0) {
    inner_active[e] = active[e];
    jdone[e] = 0;
    notconv[e] = 0;
  }
  if (!active[e] || R >= P.nrt) return;
  const int c = threadIdx.x % TS, rg = threadIdx.x / TS;
  const int npad = P.nt * TS;
  __shared__ float part[4][TS];
  float s = 0.f;
  for (int p = rg; p < npad; p += 4) {
    const float z = Z[vidx(P, p, R, c)];
    s = fmaf(z, z, s);
  }
  part[rg][c] = s;
  __syncthreads();
  const float beta = sqrtf(part[0][c] + part[1][c] + part[2][c] + part[3][c]);
  const bool empty = !(beta > 0.f) || !isfinite(beta);
  const float inv = empty ? 0.f : 1.f / beta;
  for (int p = rg; p < npad; p += 4) V0[vidx(P, p, R, c)] = Z[vidx(P, p, R, c)] * inv;
  if (rg == 0) {
    GmresState& S = st[P.csr_col + R * TS + c];
    S.beta = empty ? 0.f : beta;
    S.done = empty ? 1 : 0;
    S.nsteps = 0;
    for (int i = 0; i <= GM_MAX; ++i) S.g[i] = 0.f;
    S.g[0] = S.beta;
  }
}

// Arnoldi step j with classical Gram-Schmidt applied twice, then the Givens
// update of the column.  W holds w = LU^-1 A V_j; V_{j+1} = w / ||w||.
__global__ void __launch_bounds__(256) k_gmres_arnoldi(const Prob* probs, float* V, int64_t vstride, const float* W,
                                                       GmresState* st, const int* inner_active, int* notconv, int j,
                                                       float tol) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  const int R = blockIdx.x;
  if (!inner_active[e] || R >= P.nrt) return;
  const int c = threadIdx.x % TS, rg = threadIdx.x / TS;
  const int npad = P.nt * TS;
  __shared__ float part[4][TS][GM_MAX + 1];
  __shared__ float h[TS][GM_MAX + 2];
  float* Wm = const_cast<float*>(W);
  for (int pass = 0; pass < 2; ++pass) {
    float acc[GM_MAX];
#pragma unroll
    for (int i = 0; i < GM_MAX; ++i) acc[i] = 0.f;
    for (int p = rg; p < npad; p += 4) {
      const int64_t o = vidx(P, p, R, c);
      const float w = Wm[o];
#pragma unroll
      for (int i = 0; i < GM_MAX; ++i)
        if (i <= j) acc[i] = fmaf(V[i * vstride + o], w, acc[i]);
    }
#pragma unroll
    for (int i = 0; i < GM_MAX; ++i) part[rg][c][i] = acc[i];
    __syncthreads();
    if (rg == 0)
      for (int i = 0; i <= j; ++i) {
        const float d = part[0][c][i] + part[1][c][i] + part[2][c][i] + part[3][c][i];
        h[c][i] = pass == 0 ? d : h[c][i] + d;
        part[0][c][i] = d;  // coefficients of this pass
      }
    __syncthreads();
    float nrm2 = 0.f;
    for (int p = rg; p < npad; p += 4) {
      const int64_t o = vidx(P, p, R, c);
      float w = Wm[o];
      for (int i = 0; i <= j; ++i) w = fmaf(-part[0][c][i], V[i * vstride + o], w);
      Wm[o] = w;
      nrm2 = fmaf(w, w, nrm2);
    }
    __syncthreads();
    if (pass == 1) part[rg][c][GM_MAX] = nrm2;
    __syncthreads();
  }
  const float nrm = sqrtf(part[0][c][GM_MAX] + part[1][c][GM_MAX] + part[2][c][GM_MAX] + part[3][c][GM_MAX]);
  GmresState& S = st[P.csr_col + R * TS + c];
  const bool colDone = S.done != 0;
  const float inv = (nrm > 0.f && !colDone) ? 1.f / nrm : 0.f;
  for (int p = rg; p < npad; p += 4) {
    const int64_t o = vidx(P, p, R, c);
    V[(j + 1) * vstride + o] = Wm[o] * inv;
  }
  if (rg == 0) {
    if (!colDone) {
      float hh[GM_MAX + 1];
      for (int i = 0; i <= j; ++i) hh[i] = h[c][i];
      hh[j + 1] = nrm;
      for (int i = 0; i < j; ++i) {
        const float a = hh[i], b = hh[i + 1];
        hh[i] = S.cs[i] * a + S.sn[i] * b;
        hh[i + 1] = -S.sn[i] * a + S.cs[i] * b;
      }
      const float r = hypotf(hh[j], hh[j + 1]);
      const float cj = r > 0.f ? hh[j] / r : 1.f, sj = r > 0.f ? hh[j + 1] / r : 0.f;
      hh[j] = r;
      S.cs[j] = cj;
      S.sn[j] = sj;
      S.g[j + 1] = -sj * S.g[j];
      S.g[j] = cj * S.g[j];
      for (int i = 0; i <= j; ++i) S.H[i + j * (GM_MAX + 1)] = hh[i];
      S.nsteps = j + 1;
      if (fabsf(S.g[j + 1]) <= tol * S.beta || !(nrm > 0.f)) S.done = 1;
      else atomicAdd(&notconv[e], 1);
    }
  }
}

// Close an Arnoldi step: count it and drop problems whose columns all converged.
__global__ void k_gmres_flags(const Prob* probs, int nprob, int* inner_active, int* jdone, int* notconv) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nprob || !inner_active[e]) return;
  jdone[e] += 1;
  if (notconv[e] == 0) inner_active[e] = 0;
  notconv[e] = 0;
}

// Correction d = V y with H y = g (upper triangular, size jdone) per column,
// written into D in the RHS tile layout.
__global__ void k_gmres_finish(const Prob* probs, const float* V, int64_t vstride, const GmresState* st,
                               const int* active, const int* jdone, float* D) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  const int R = blockIdx.x;
  if (!active[e] || R >= P.nrt) return;
  const int c = threadIdx.x % TS, rg = threadIdx.x / TS;
  const GmresState& S = st[P.csr_col + R * TS + c];
  const int m = min(S.nsteps, jdone[e]);  // steps taken by this column
  __shared__ float y[TS][GM_MAX];
  if (rg == 0) {
    for (int i = m - 1; i >= 0; --i) {
      float s = S.g[i];
      for (int k = i + 1; k < m; ++k) s -= S.H[i + k * (GM_MAX + 1)] * y[c][k];
      const float d = S.H[i + i * (GM_MAX + 1)];
      y[c][i] = (d != 0.f && S.beta > 0.f) ? s / d : 0.f;
    }
  }
  __syncthreads();
  const int npad = P.nt * TS;
  for (int p = rg; p < npad; p += 4) {
    const int64_t o = vidx(P, p, R, c);
    float d = 0.f;
    for (int i = 0; i < m; ++i) d = fmaf(y[c][i], V[i * vstride + o], d);
    D[o] = d;
  }
}

void launch_csr_scale(const Prob* probs, const Pools& pl, const LaunchDims& d, cudaStream_t s) {
  k_csr_scale<<<dim3((d.max_rows + 255) / 256, d.nprob), 256, 0, s>>>(probs, pl.rowptr, pl.col, pl.val, pl.rs, pl.cs,
                                                                      pl.valS);
}

// One refinement step after the residual r (scaled, FP32) sits in Y32:
//   Y32 <- LU^-1 Y32 for every active problem (the classical correction), then,
//   for the problems in active_gm, GMRES(m) on LU^-1 (Dr A Dc) started from
//   that vector replaces Y32 by the GMRES correction.
void launch_gmres_cycle(const StepPlan& sp, const Prob* probs, const Pools& pl, Tables tb, const LaunchDims& d, int m,
                        float tol, cudaStream_t s) {
  const int np = d.nprob;
  launch_forward<float>(sp, pl.env32, pl.Y32, probs, tb, np, pl.active, pl.piv, s);
  launch_backward<float>(sp, pl.env32, pl.Y32, probs, tb, np, pl.active, s);
  GmresState* st = reinterpret_cast<GmresState*>(pl.gstate);
  k_gmres_start<<<dim3(sp.nrtmax, np), 256, 0, s>>>(probs, pl.Y32, pl.V, st, pl.active_gm, pl.inner_active,
                                                    pl.jdone, pl.notconv);
  for (int j = 0; j < m; ++j) {
    const float* Vj = pl.V + (int64_t)j * pl.vstride;
    k_spmv32<<<dim3((d.max_rows + 7) / 8, np), 256, 0, s>>>(probs, pl.rowptr, pl.col, pl.valS, Vj, pl.W,
                                                           pl.inner_active);
    launch_forward<float>(sp, pl.env32, pl.W, probs, tb, np, pl.inner_active, pl.piv, s);
    launch_backward<float>(sp, pl.env32, pl.W, probs, tb, np, pl.inner_active, s);
    k_gmres_arnoldi<<<dim3(sp.nrtmax, np), 256, 0, s>>>(probs, pl.V, pl.vstride, pl.W, st, pl.inner_active,
                                                        pl.notconv, j, tol);
    k_gmres_flags<<<(np + 127) / 128, 128, 0, s>>>(probs, np, pl.inner_active, pl.jdone, pl.notconv);
  }
  k_gmres_finish<<<dim3(sp.nrtmax, np), 256, 0, s>>>(probs, pl.V, pl.vstride, st, pl.active_gm, pl.jdone, pl.Y32);
}

size_t gmres_state_bytes() { return sizeof(GmresState); }
int gmres_max_dim() { return GM_MAX; }

}  // namespace fdm
