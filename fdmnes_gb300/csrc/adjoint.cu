// adjoint.cu - reverse mode of the batched spectrum: gradient of a scalar
// loss L(Taull(E_1), ..., Taull(E_n)) with respect to the grid potential Vr.
//
// Forward: A(Vr) X = B per energy (mat_solve, source/mat_solve_gaussian.f90),
// then Taull from X (source/mat.f90:306-405,598-644):
//   N = I + i S,  S(f, g) = X(outer row g, rhs f),  Xa(f, a) = X(absorber row a, rhs f)
//   Amp = N^-1 Xa,  T(a, b) = Im Taull(a, b) = -Re sum_f Amp(f, a) conj(Amp(f, b)).
// Reverse, given Gt(a, b) = dL/dT(a, b):
//   Q = Amp (Gt + Gt^T),  W = N^-H Q,
//   dL/dXa(f, a) = -Re W(f, a),  dL/dS(f, g) = -Im sum_a conj(W(f, a)) Amp(g, a),
// which is the cotangent G of X on the outer and absorber rows.  Then
// Lambda = A^-T G with the factors already in HBM (transposed tile solves),
// and since Vr(i) enters only the diagonal of grid row new(i)
// (calcMatRow, source/mat.f90:1151-1156),
//   dL/dVr(i) = -sum_E sum_k Lambda_E(new(i), k) X_E(new(i), k).
#include "fdm_internal.cuh"
#include "fdm_kernels.h"

namespace fdm {

namespace {

__device__ __forceinline__ double2 cmulz(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double2 cdivz(double2 a, double2 b) {
  const double d = b.x * b.x + b.y * b.y;
  return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
__device__ __forceinline__ double xat(const double* X, const Prob& P, int p, int r) {
  return X[P.rhs + ((int64_t)(p / TS) * P.nrt + r / TS) * TS2 + (p % TS) * TS + (r % TS)];
}
__device__ __forceinline__ double* gat(double* G, const Prob& P, int p, int r) {
  return G + P.rhs + ((int64_t)(p / TS) * P.nrt + r / TS) * TS2 + (p % TS) * TS + (r % TS);
}

constexpr int VJP_THREADS = 512;

}  // namespace

// One CTA per energy.  scratch: n x (n + 2m) complex at P.scratch (column-major
// N | Xa, then Q).  gT: m x m real at P.taull.  G: RHS tiles, zero on entry.
__global__ void __launch_bounds__(VJP_THREADS) k_taull_vjp(const Prob* probs, const double* X, const double* gT,
                                                           double2* scratch, double* G, int* err) {
  const int e = blockIdx.x;
  const Prob P = probs[e];
  const int n = P.nlmso, m = P.nlm_abs, W = n + m;
  if (m <= 0) return;
  double2* M = scratch + P.scratch;
  double2* Q = M + (int64_t)n * W;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* lcol = reinterpret_cast<double2*>(smem_raw);  // n
  int* pv = reinterpret_cast<int*>(lcol + n);             // n
  __shared__ double bestv[VJP_THREADS / 32];
  __shared__ int besti[VJP_THREADS / 32];
  __shared__ int piv_s;
  const int tid = threadIdx.x;
  for (int idx = tid; idx < n * W; idx += blockDim.x) {
    const int i = idx % n, j = idx / n;
    M[idx] = j < n ? make_double2(i == j ? 1.0 : 0.0, xat(X, P, P.nlmso - (j + 1), i))
                   : make_double2(xat(X, P, P.n - P.ianew_abs - (j - n + 1), i), 0.0);
  }
  __syncthreads();
  // P N = L U with partial pivoting on |re| + |im|; whole rows are swapped so
  // that the stored L matches P.
  for (int k = 0; k < n; ++k) {
    double bv = -1.0;
    int bi = n;
    for (int i = k + tid; i < n; i += blockDim.x) {
      const double2 a = M[i + (int64_t)k * n];
      const double v = fabs(a.x) + fabs(a.y);
      if (v > bv) { bv = v; bi = i; }
    }
    for (int o = 16; o; o >>= 1) {
      const double ov = __shfl_xor_sync(0xffffffffu, bv, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
    }
    if ((tid & 31) == 0) { bestv[tid / 32] = bv; besti[tid / 32] = bi; }
    __syncthreads();
    if (tid == 0) {
      double v = bestv[0];
      int ix = besti[0];
      for (int w = 1; w < VJP_THREADS / 32; ++w)
        if (bestv[w] > v || (bestv[w] == v && besti[w] < ix)) { v = bestv[w]; ix = besti[w]; }
      if (!(v > 0.0) || ix >= n) {
        atomicExch(&err[e], (int)FDMGPU_ERR_ZERO_PIVOT);
        ix = k;
      }
      piv_s = ix;
      pv[k] = ix;
    }
    __syncthreads();
    const int pr = piv_s;
    if (pr != k)
      for (int j = tid; j < W; j += blockDim.x) {
        const double2 t = M[k + (int64_t)j * n];
        M[k + (int64_t)j * n] = M[pr + (int64_t)j * n];
        M[pr + (int64_t)j * n] = t;
      }
    __syncthreads();
    const double2 d = M[k + (int64_t)k * n];
    for (int i = k + 1 + tid; i < n; i += blockDim.x) {
      const double2 l = cdivz(M[i + (int64_t)k * n], d);
      lcol[i] = l;
      M[i + (int64_t)k * n] = l;
    }
    __syncthreads();
    const int nr = n - k - 1, nc = W - k - 1;
    for (int idx = tid; idx < nr * nc; idx += blockDim.x) {
      const int i = k + 1 + idx % nr, j = k + 1 + idx / nr;
      const double2 u = M[k + (int64_t)j * n];
      double2 c = M[i + (int64_t)j * n];
      const double2 t = cmulz(lcol[i], u);
      c.x -= t.x;
      c.y -= t.y;
      M[i + (int64_t)j * n] = c;
    }
    __syncthreads();
  }
  // Amp = U^-1 (L^-1 P Xa), already L^-1 P Xa in the right columns
  for (int k = n - 1; k >= 0; --k) {
    const double2 d = M[k + (int64_t)k * n];
    for (int a = tid; a < m; a += blockDim.x) M[k + (int64_t)(n + a) * n] = cdivz(M[k + (int64_t)(n + a) * n], d);
    __syncthreads();
    for (int idx = tid; idx < k * m; idx += blockDim.x) {
      const int i = idx % k, a = idx / k;
      const double2 t = cmulz(M[i + (int64_t)k * n], M[k + (int64_t)(n + a) * n]);
      double2 c = M[i + (int64_t)(n + a) * n];
      c.x -= t.x;
      c.y -= t.y;
      M[i + (int64_t)(n + a) * n] = c;
    }
    __syncthreads();
  }
  const double2* Amp = M + (int64_t)n * n;
  const double* g = gT + P.taull;
  // Q = Amp (Gt + Gt^T)
  for (int idx = tid; idx < n * m; idx += blockDim.x) {
    const int f = idx % n, a = idx / n;
    double2 q = make_double2(0.0, 0.0);
    for (int b = 0; b < m; ++b) {
      const double s = g[b + (int64_t)a * m] + g[a + (int64_t)b * m];
      q.x += Amp[f + (int64_t)b * n].x * s;
      q.y += Amp[f + (int64_t)b * n].y * s;
    }
    Q[idx] = q;
  }
  __syncthreads();
  // U^H y = Q (forward)
  for (int k = 0; k < n; ++k) {
    const double2 dk = cconj(M[k + (int64_t)k * n]);
    for (int a = tid; a < m; a += blockDim.x) Q[k + (int64_t)a * n] = cdivz(Q[k + (int64_t)a * n], dk);
    __syncthreads();
    const int nr = n - k - 1;
    for (int idx = tid; idx < nr * m; idx += blockDim.x) {
      const int i = k + 1 + idx % nr, a = idx / nr;
      const double2 t = cmulz(cconj(M[k + (int64_t)i * n]), Q[k + (int64_t)a * n]);
      Q[i + (int64_t)a * n].x -= t.x;
      Q[i + (int64_t)a * n].y -= t.y;
    }
    __syncthreads();
  }
  // L^H z = y (backward, unit diagonal)
  for (int k = n - 1; k > 0; --k) {
    for (int idx = tid; idx < k * m; idx += blockDim.x) {
      const int i = idx % k, a = idx / k;
      const double2 t = cmulz(cconj(M[k + (int64_t)i * n]), Q[k + (int64_t)a * n]);
      Q[i + (int64_t)a * n].x -= t.x;
      Q[i + (int64_t)a * n].y -= t.y;
    }
    __syncthreads();
  }
  // W = P^T z: undo the row swaps, last first
  for (int k = n - 1; k >= 0; --k) {
    const int pr = pv[k];
    if (pr != k)
      for (int a = tid; a < m; a += blockDim.x) {
        const double2 t = Q[k + (int64_t)a * n];
        Q[k + (int64_t)a * n] = Q[pr + (int64_t)a * n];
        Q[pr + (int64_t)a * n] = t;
      }
    __syncthreads();
  }
  // cotangent of X: absorber rows, then outer rows
  for (int idx = tid; idx < n * m; idx += blockDim.x) {
    const int f = idx % n, a = idx / n;
    *gat(G, P, P.n - (P.ianew_abs + a + 1), f) = -Q[idx].x;
  }
  for (int idx = tid; idx < n * n; idx += blockDim.x) {
    const int f = idx % n, gg = idx / n;
    double im = 0.0;
    for (int a = 0; a < m; ++a) {
      const double2 w = Q[f + (int64_t)a * n], am = Amp[gg + (int64_t)a * n];
      im += w.x * am.y - w.y * am.x;  // Im(conj(w) am)
    }
    *gat(G, P, P.nlmso - (gg + 1), f) = -im;
  }
}

// part[e * npr + k] = -sum_c Lambda(p, c) X(p, c), p the row of interstitial
// point k in energy e.  One warp per point.
__global__ void __launch_bounds__(256) k_grad_points(StaticDev S, const Prob* probs, const int* ipool,
                                                     const double* X, const double* Lam, double* part) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int k = blockIdx.x * 8 + warp;
  if (k >= S.npr) return;
  const int i = S.inter_pt[k];
  const int p = P.n - ipool[P.in_new + i];
  double s = 0.0;
  for (int c = lane; c < P.nlmso; c += 32) s += xat(Lam, P, p, c) * xat(X, P, p, c);
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) part[(int64_t)e * S.npr + k] = -s;
}

// grad(i, spin) = sum over the energies of that spin block, in batch order.
__global__ void k_grad_reduce(StaticDev S, const Prob* probs, int np, int nspin, const double* part, double* grad) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= S.npr * nspin) return;
  const int k = t % S.npr, isp = t / S.npr;
  double s = 0.0;
  for (int e = 0; e < np; ++e)
    if (probs[e].ispin == isp + 1) s += part[(int64_t)e * S.npr + k];
  grad[(S.inter_pt[k] - 1) + (int64_t)S.npoint * isp] = s;
}

// rowpart[rowv + p] = sum_c Lambda(p, c) (B(p, c) - sum_q A(p, q) X(q, c)), warp per
// row p, from the CSR copy of the band.
__global__ void k_lambda_rows(const Prob* probs, const int* rowptr, const int* col, const double* val, const double* B,
                              const double* X, const double* Lam, double* rowpart) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  const int p = blockIdx.x * 8 + threadIdx.x / 32, lane = threadIdx.x % 32;
  if (p >= P.nt * TS) return;
  const int k0 = rowptr[P.rowv + p], k1 = min(rowptr[P.rowv + p + 1], (int)P.csr_cap);
  double dot = 0.0;
  for (int c = lane; c < P.nlmso; c += 32) {
    double r = xat(B, P, p, c);
    for (int k = k0; k < k1; ++k) r -= val[P.csr + k] * xat(X, P, col[P.csr + k], c);
    dot += xat(Lam, P, p, c) * r;
  }
  for (int o = 16; o; o >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, o);
  if (lane == 0) rowpart[P.rowv + p] = dot;
}

// out[e] = sum of the row partials of problem e in a fixed order.
__global__ void k_lambda_sum(const Prob* probs, const double* rowpart, double* out) {
  const int e = blockIdx.x;
  const Prob P = probs[e];
  const int npad = P.nt * TS;
  __shared__ double red[256];
  double s = 0.0;
  for (int p = threadIdx.x; p < npad; p += blockDim.x) s += rowpart[P.rowv + p];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[e] = red[0];
}

void launch_lambda_dot(const Prob* probs, const Pools& pl, const LaunchDims& d, const double* Lam, double* rowpart,
                       double* out, cudaStream_t s) {
  k_lambda_rows<<<dim3((d.max_rows + 7) / 8, d.nprob), 256, 0, s>>>(probs, pl.rowptr, pl.col, pl.val, pl.B64, pl.X64,
                                                                   Lam, rowpart);
  k_lambda_sum<<<d.nprob, 256, 0, s>>>(probs, rowpart, out);
}

// Transposed CSR (the CSR of A^T) of every problem, for the transposed
// residual of a mixed batch's adjoint.  Counts per column, then one warp per
// problem fills the rows in order, so each column lists its rows ascending
// (deterministic sums).  Within one row the columns are distinct, so the
// lanes of a warp never share a cursor.
__global__ void k_csc_count(const Prob* probs, const int* rowptr, const int* col, int* colcnt) {
  const Prob P = probs[blockIdx.y];
  const int p = blockIdx.x * 8 + threadIdx.x / 32, lane = threadIdx.x % 32;
  if (p >= P.nt * TS) return;
  const int k0 = rowptr[P.rowv + p], k1 = min(rowptr[P.rowv + p + 1], (int)P.csr_cap);
  for (int k = k0 + lane; k < k1; k += 32) atomicAdd(&colcnt[P.rowv + col[P.csr + k] + 1], 1);
}

__global__ void k_csc_fill(const Prob* probs, int np, const int* rowptr, const int* col, const float2* val2,
                           int* cursor, int* cscrow, float2* cscval2) {
  const int e = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32, lane = threadIdx.x % 32;
  if (e >= np) return;
  const Prob P = probs[e];
  for (int p = 0; p < P.nt * TS; ++p) {
    const int k0 = rowptr[P.rowv + p], k1 = min(rowptr[P.rowv + p + 1], (int)P.csr_cap);
    for (int k = k0 + lane; k < k1; k += 32) {
      const int c = col[P.csr + k];
      const int pos = cursor[P.rowv + c]++;
      if (pos < P.csr_cap) {
        cscrow[P.csr + pos] = p;
        cscval2[P.csr + pos] = val2[P.csr + k];
      }
    }
    __syncwarp();
  }
}

void launch_csc_build(const Prob* probs, const Pools& pl, const LaunchDims& d, int* colptr, int* cursor, int* cscrow,
                      float2* cscval2, cudaStream_t s) {
  cudaMemsetAsync(colptr, 0, d.rowv_total * sizeof(int), s);
  k_csc_count<<<dim3((d.max_rows + 7) / 8, d.nprob), 256, 0, s>>>(probs, pl.rowptr, pl.col, colptr);
  launch_csr_scan(probs, colptr, d, s);
  cudaMemcpyAsync(cursor, colptr, d.rowv_total * sizeof(int), cudaMemcpyDeviceToDevice, s);
  k_csc_fill<<<(d.nprob + 3) / 4, 128, 0, s>>>(probs, d.nprob, pl.rowptr, pl.col, pl.val2, cursor, cscrow, cscval2);
}

void launch_taull_vjp(const Prob* probs, const LaunchDims& d, const double* X, const double* gT, double* scratch,
                      double* G, int* err, cudaStream_t s) {
  const size_t sm = (size_t)d.max_nlmso * (sizeof(double2) + sizeof(int));
  if (sm > 48 * 1024) cudaFuncSetAttribute(k_taull_vjp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_taull_vjp<<<d.nprob, VJP_THREADS, sm, s>>>(probs, X, gT, reinterpret_cast<double2*>(scratch), G, err);
}

void launch_grad_vr(const StaticDev& S, const Prob* probs, const int* ipool, const LaunchDims& d, int nspin,
                    const double* X, const double* Lam, double* part, double* grad, cudaStream_t s) {
  k_grad_points<<<dim3((S.npr + 7) / 8, d.nprob), 256, 0, s>>>(S, probs, ipool, X, Lam, part);
  const int n = S.npr * nspin;
  k_grad_reduce<<<(n + 255) / 256, 256, 0, s>>>(S, probs, d.nprob, nspin, part, grad);
}

}  // namespace fdm
