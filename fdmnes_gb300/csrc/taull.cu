// taull.cu - absorber scattering amplitude Taull from the FDM solution.
//
// Real-basis case of `mat` (source/mat.f90:306-405, FDM_comp false):
//   norm = I + i S,  S(Lm2, Lm) = x(outer row Lm, rhs Lm2)       (:312-330)
//   norm^-1 by zgetrf/zgetri (invcomp, :339, :1927-1992)
//   ampl(f, a) = sum_k norm^-1(f, k) x(absorber row a, rhs k)    (:370-378)
//   Taull(a, b) = -i sum_f ampl(f, a) conj(ampl(f, b))            (:385-390)
// followed by the symmetrisation of the real-harmonics case,
// Taull = i Im(Taull) (:598-644).  Instead of forming norm^-1, the kernel
// solves norm * ampl = x_abs with Gaussian elimination and partial pivoting on
// |re| + |im| (the pivot rule of zgetrf), one block per problem, in FP64.
#include "fdm_internal.cuh"
#include "fdm_kernels.h"

namespace fdm {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
  const double d = b.x * b.x + b.y * b.y;
  return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}

__device__ __forceinline__ double xval(const double* X, const Prob& P, int p, int r) {
  return X[P.rhs + ((int64_t)(p / TS) * P.nrt + r / TS) * TS2 + (p % TS) * TS + (r % TS)];
}

constexpr int TAULL_THREADS = 512;

__global__ void __launch_bounds__(TAULL_THREADS) k_taull(const Prob* probs, const double* X, double2* scratch,
                                                         double2* taull, int* err) {
  const int e = blockIdx.x;
  const Prob P = probs[e];
  const int n = P.nlmso, m = P.nlm_abs, W = n + m;
  double2* M = scratch + P.scratch;  // n x W, column-major
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* lcol = reinterpret_cast<double2*>(smem_raw);  // n
  __shared__ double bestv[TAULL_THREADS / 32];
  __shared__ int besti[TAULL_THREADS / 32];
  __shared__ int piv_s;
  const int tid = threadIdx.x;
  for (int idx = tid; idx < n * W; idx += blockDim.x) {
    const int i = idx % n, j = idx / n;
    double2 v;
    if (j < n) {
      const int Lm = j + 1;
      v = make_double2(i == j ? 1.0 : 0.0, xval(X, P, P.nlmso - Lm, i));
    } else {
      const int a = j - n + 1;
      v = make_double2(xval(X, P, P.n - P.ianew_abs - a, i), 0.0);
    }
    M[idx] = v;
  }
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    // pivot: first row of largest |re| + |im| in column k
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
      for (int w = 1; w < (int)blockDim.x / 32; ++w)
        if (bestv[w] > v || (bestv[w] == v && besti[w] < ix)) { v = bestv[w]; ix = besti[w]; }
      piv_s = ix;
      if (!(v > 0.0)) atomicExch(&err[e], (int)FDMGPU_ERR_ZERO_PIVOT);
    }
    __syncthreads();
    const int pr = piv_s;
    if (pr != k && pr < n)
      for (int j = k + tid; j < W; j += blockDim.x) {
        const double2 t = M[k + (int64_t)j * n];
        M[k + (int64_t)j * n] = M[pr + (int64_t)j * n];
        M[pr + (int64_t)j * n] = t;
      }
    __syncthreads();
    const double2 pv = M[k + (int64_t)k * n];
    for (int i = k + 1 + tid; i < n; i += blockDim.x) lcol[i] = cdiv(M[i + (int64_t)k * n], pv);
    __syncthreads();
    const int nr = n - k - 1;
    const int ncols = W - k - 1;
    for (int idx = tid; idx < nr * ncols; idx += blockDim.x) {
      const int i = k + 1 + idx % nr, j = k + 1 + idx / nr;
      const double2 u = M[k + (int64_t)j * n];
      const double2 l = lcol[i];
      double2 c = M[i + (int64_t)j * n];
      c.x -= l.x * u.x - l.y * u.y;
      c.y -= l.x * u.y + l.y * u.x;
      M[i + (int64_t)j * n] = c;
    }
    __syncthreads();
  }
  // back substitution on the m right-hand columns
  for (int k = n - 1; k >= 0; --k) {
    const double2 d = M[k + (int64_t)k * n];
    for (int j = tid; j < m; j += blockDim.x) M[k + (int64_t)(n + j) * n] = cdiv(M[k + (int64_t)(n + j) * n], d);
    __syncthreads();
    for (int idx = tid; idx < k * m; idx += blockDim.x) {
      const int i = idx % k, j = n + idx / k;
      const double2 u = M[i + (int64_t)k * n];
      const double2 x = M[k + (int64_t)j * n];
      double2 c = M[i + (int64_t)j * n];
      c.x -= u.x * x.x - u.y * x.y;
      c.y -= u.x * x.y + u.y * x.x;
      M[i + (int64_t)j * n] = c;
    }
    __syncthreads();
  }
  // Taull(a, b) = i * Im(-i sum_f ampl(f,a) conj(ampl(f,b))) = (0, -Re(sum))
  double2* T = taull + P.taull;
  for (int idx = tid; idx < m * m; idx += blockDim.x) {
    const int a = idx % m, b = idx / m;
    const double2* A1 = M + (int64_t)(n + a) * n;
    const double2* A2 = M + (int64_t)(n + b) * n;
    double s = 0.0;
    for (int f = 0; f < n; ++f) s += A1[f].x * A2[f].x + A1[f].y * A2[f].y;
    T[a + (int64_t)b * m] = make_double2(0.0, -s);
  }
}

void launch_taull(const Prob* probs, const Pools& pl, const LaunchDims& d, const double* X, cudaStream_t s) {
  const size_t sm = (size_t)d.max_nlmso * sizeof(double2);
  if (sm > 48 * 1024) cudaFuncSetAttribute(k_taull, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_taull<<<d.nprob, TAULL_THREADS, sm, s>>>(probs, X, reinterpret_cast<double2*>(pl.tscratch),
                                             reinterpret_cast<double2*>(pl.taull), pl.err);
}

}  // namespace fdm
