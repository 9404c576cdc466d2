// taull_noalloc.cu - Taull of one energy from a device-resident solution smr,
// with its working matrix in a fixed array of this library's device image
// instead of memory allocated at run time.
//
// Same contraction as k_taull (source/mat.f90:306-405 and the real-harmonics
// symmetrisation at :598-644): norm = I + i S with S(Lm2, Lm) = smr(Lm2, outer
// row Lm), solve norm * ampl = smr(:, absorber rows) by Gaussian elimination
// with |re| + |im| partial pivoting, Taull(a, b) = (0, -Re sum_f ampl(f, a)
// conj(ampl(f, b))).  The input here is smr in mat_solve's own layout
// (nlmso, nligne) column-major, so a caller that keeps smr on the device can
// call it directly.
#include <mutex>

#include "fdm_internal.cuh"
#include "fdm_kernels.h"

namespace fdm {

namespace {

constexpr int NOALLOC_THREADS = 512;
constexpr int64_t NOALLOC_ELEMS = FDMGPU_TAULL_NOALLOC_SCRATCH_BYTES / (int64_t)sizeof(double2);

// The working matrix norm | smr(:, absorber rows): nlmso x (nlmso + nlm_abs)
// complex, column-major.  One array per device, shared by every call.
static __device__ __align__(256) double2 g_taull_scratch[NOALLOC_ELEMS];

__device__ __forceinline__ double2 cdiv_na(double2 a, double2 b) {
  const double d = b.x * b.x + b.y * b.y;
  return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}

__global__ void __launch_bounds__(NOALLOC_THREADS)
    k_taull_static(const double* __restrict__ smr, int n, int nligne, int ianew_abs, int m,
                   double2* __restrict__ M, double2* __restrict__ taull, int* status) {
  const int W = n + m;
  __shared__ double2 lcol[FDMGPU_TAULL_NOALLOC_MAX_NLMSO];
  __shared__ double bestv[NOALLOC_THREADS / 32];
  __shared__ int besti[NOALLOC_THREADS / 32];
  __shared__ int piv_s, bad_s;
  const int tid = threadIdx.x;
  if (tid == 0) bad_s = 0;
  // smr(lm, ii) sits at smr[lm + (ii - 1) * n]; outer row Lm is ii = nligne - n + Lm,
  // absorber harmonic a is ii = ianew_abs + a.
  for (int idx = tid; idx < n * W; idx += blockDim.x) {
    const int i = idx % n, j = idx / n;
    double2 v;
    if (j < n)
      v = make_double2(i == j ? 1.0 : 0.0, smr[i + (int64_t)(nligne - n + j) * n]);
    else
      v = make_double2(smr[i + (int64_t)(ianew_abs + j - n) * n], 0.0);
    M[idx] = v;
  }
  __syncthreads();
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
      for (int w = 1; w < NOALLOC_THREADS / 32; ++w)
        if (bestv[w] > v || (bestv[w] == v && besti[w] < ix)) { v = bestv[w]; ix = besti[w]; }
      piv_s = ix;
      if (!(v > 0.0)) bad_s = 1;
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
    for (int i = k + 1 + tid; i < n; i += blockDim.x) lcol[i] = cdiv_na(M[i + (int64_t)k * n], pv);
    __syncthreads();
    const int nr = n - k - 1, ncols = W - k - 1;
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
  for (int k = n - 1; k >= 0; --k) {
    const double2 d = M[k + (int64_t)k * n];
    for (int j = tid; j < m; j += blockDim.x) M[k + (int64_t)(n + j) * n] = cdiv_na(M[k + (int64_t)(n + j) * n], d);
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
  for (int idx = tid; idx < m * m; idx += blockDim.x) {
    const int a = idx % m, b = idx / m;
    const double2* A1 = M + (int64_t)(n + a) * n;
    const double2* A2 = M + (int64_t)(n + b) * n;
    double s = 0.0;
    for (int f = 0; f < n; ++f) s += A1[f].x * A2[f].x + A1[f].y * A2[f].y;
    taull[a + (int64_t)b * m] = make_double2(0.0, -s);
  }
  if (tid == 0 && status) *status = bad_s ? (int)FDMGPU_ERR_ZERO_PIVOT : (int)FDMGPU_OK;
}

constexpr int MAX_DEVICES = 64;
std::mutex g_scratch_mu;
double2* g_scratch_addr[MAX_DEVICES] = {};
unsigned long long g_scratch_ctx[MAX_DEVICES] = {};  // context the address belongs to

// Unique id of the calling thread's current CUDA context (0 when it cannot be
// read).  A device reset destroys the primary context and the next one may
// load this library's device image at another address; the id tells the two
// apart (a context's address can be reused, its id is not).
typedef int (*ctx_get_current_fn)(void**);
typedef int (*ctx_get_id_fn)(void*, unsigned long long*);
unsigned long long current_context_id() {
  static ctx_get_current_fn get_current = nullptr;
  static ctx_get_id_fn get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    void* f1 = nullptr;
    void* f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
        q1 == cudaDriverEntryPointSuccess &&
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
        q2 == cudaDriverEntryPointSuccess) {
      get_current = reinterpret_cast<ctx_get_current_fn>(f1);
      get_id = reinterpret_cast<ctx_get_id_fn>(f2);
    }
    looked_up = true;
  }
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
  return id;
}

}  // namespace

// Address of this device's scratch array, looked up with that device current
// once per device and CUDA context (the lookup may load this library's device
// code).  After a device reset the new context's address is looked up again.
cudaError_t taull_noalloc_scratch(double2** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= MAX_DEVICES) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  const unsigned long long ctx = current_context_id();
  if (!g_scratch_addr[dev] || ctx == 0 || ctx != g_scratch_ctx[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_taull_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[dev] = static_cast<double2*>(p);
    // the id is read after the lookup: the lookup makes the context current
    g_scratch_ctx[dev] = current_context_id();
  }
  *out = g_scratch_addr[dev];
  return cudaSuccess;
}

cudaError_t launch_taull_noalloc(const double* smr, int nlmso, int nligne, int ianew_abs, int nlm_abs,
                                 double2* scratch, double* taull, int* status, cudaStream_t s) {
  k_taull_static<<<1, NOALLOC_THREADS, 0, s>>>(smr, nlmso, nligne, ianew_abs, nlm_abs, scratch,
                                               reinterpret_cast<double2*>(taull), status);
  return cudaGetLastError();
}

}  // namespace fdm
