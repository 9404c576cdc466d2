// factor.cu - batched tile LU of the FDM band and the triangular solves.
//
// One launch handles one panel step K for every problem of a batch
// (blockIdx.y = problem).  The elimination is the reference's no-pivot
// Gaussian elimination (source/mat_solve_gaussian.f90:196-317) carried out in
// reversed order as a right-looking LU on TS x TS tiles:
//   k_panel     factor tile (K,K); L tiles (I,K) <- A(I,K) U(K,K)^-1;
//               U tiles (K,J) and RHS tiles (K,R) <- L(K,K)^-1 A(K,.)
//               (the RHS columns ride along, so the forward substitution of the
//               reference's elimination loop, :231-262, is fused here);
//   k_trailing  A(I,J) -= L(I,K) U(K,J) and Y(I,R) -= L(I,K) Y(K,R).
// The backward substitution (the reference's resolution loop, :348-358) is
// k_bwd_diag + k_bwd_update; k_fwd_* are used by the refinement solves.
#include <algorithm>
#include <type_traits>

#include "fdm_internal.cuh"
#include "fdm_kernels.h"

namespace fdm {

// Factor the diagonal tile (K,K) in place (one CTA per problem).  With piv,
// partial pivoting among the tile's rows; the row order is stored in
// piv[rowv + K*TS + r] and applied to the U and RHS tiles of block K when they
// are loaded (the L tiles left of the diagonal keep the order in which the
// earlier steps updated them, and the forward substitution permutes Y(K) at
// step K, so P A = L U holds block by block).
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_diag(T* env, const Prob* probs, Tables tb, int K,
                                                   const int* active, int* err, double piv_thr, int* piv) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  if (K >= P.nt || (active && !active[e])) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* D = reinterpret_cast<T*>(smem_raw);
  __shared__ double mp;
  __shared__ int perm[TS];
  if (threadIdx.x < TS) perm[threadIdx.x] = threadIdx.x;
  T* dtile = tile_ptr(env, P, tb, K, K);
  load_tile(D, dtile);
  __syncthreads();
  tile_lu(D, &mp, piv ? perm : nullptr);
  __syncthreads();
  store_tile(dtile, D);
  if (piv && threadIdx.x < TS) piv[P.rowv + (int64_t)K * TS + threadIdx.x] = perm[threadIdx.x];
  // smallest |pivot| of the tile (padding rows carry 1); NaN also trips the test
  if (threadIdx.x == 0 && !(mp >= piv_thr)) atomicExch(&err[e], (int)FDMGPU_ERR_ZERO_PIVOT);
}

// Panel of step K with the factored diagonal tile: L tiles (I,K), U tiles
// (K,J) and, when fused, the RHS tiles (K,R).
// Separate register allocation for the two branches of the panel.
template <typename T>
__device__ __noinline__ void panel_row_solve(T* g, const T* D, T* Ws) { row_solve_upper(g, D, Ws); }
template <typename T>
__device__ __noinline__ void panel_col_solve(T* g, const T* D, const int* perm) { col_solve_lower_unit(g, D, perm); }

template <typename T>
__global__ void __launch_bounds__(GEMM_THREADS) k_panel(T* env, T* rhs, const Prob* probs, Tables tb, int K,
                                                    int fuse_rhs, const int* active, const int* piv) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  if (K >= P.nt || (active && !active[e])) return;
  const int nI = tb.Imax[P.trow + K] - K;
  const int nJ = tb.J1[P.trow + K] - K;
  const int nR = fuse_rhs ? P.nrt : 0;
  const int w = blockIdx.x;
  if (w >= nI + nJ + nR) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* D = reinterpret_cast<T*>(smem_raw);
  T* Ws = D + TS * SP;
  load_tile_n(D, tile_ptr(env, P, tb, K, K), GEMM_THREADS);
  __syncthreads();
  if (w < nI) {
    // L(I,K) = A(I,K) U_KK^-1
    panel_row_solve(tile_ptr(env, P, tb, K + 1 + w, K), D, Ws);
  } else {
    // U(K,J) = L_KK^-1 P A(K,J) and Y(K,R) = L_KK^-1 P Y(K,R)
    T* g = w < nI + nJ ? tile_ptr(env, P, tb, K, K + 1 + (w - nI)) : rhs_ptr(rhs, P, K, w - nI - nJ);
    panel_col_solve(g, D, piv ? piv + P.rowv + (int64_t)K * TS : (const int*)nullptr);
  }
}

// NT: threads per tile pair (64: 8x8 accumulators per thread; 128: 8x4),
// chosen per batch plan by the autotuner in the host code.  WIDE (FP32 only):
// double-float accumulation of the products; each FP32 problem's step runs in
// exactly one of the two instantiations, as tb.wide marks it.
template <typename T, int NT, bool WIDE = false>
__global__ void __launch_bounds__(NT) k_trailing(T* env, T* rhs, const Prob* probs, Tables tb, int K,
                                                       int fuse_rhs, const int* active) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  if (K >= P.nt || (active && !active[e])) return;
  if (std::is_same<T, float>::value) {
    const bool w = tb.wide && tb.wide[P.trow + K];
    if (w != WIDE) return;
  }
  const int nI = tb.Imax[P.trow + K] - K;
  const int nJ = tb.J1[P.trow + K] - K;
  const int nC = nJ + (fuse_rhs ? P.nrt : 0);
  const int w = blockIdx.x;
  if (w >= nI * nC) return;
  const int I = K + 1 + w / nC;
  const int c = w % nC;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* As = reinterpret_cast<T*>(smem_raw);
  T* Bs = As + TS * SP;
  const T* A = tile_ptr(env, P, tb, I, K);
  const T* B;
  T* C;
  if (c < nJ) {
    B = tile_ptr(env, P, tb, K, K + 1 + c);
    C = tile_ptr(env, P, tb, I, K + 1 + c);
  } else {
    B = rhs_ptr(rhs, P, K, c - nJ);
    C = rhs_ptr(rhs, P, I, c - nJ);
  }
  if constexpr (WIDE)
    tile_mm64<T, true, false, NT, facc>(C, A, B, (const int*)nullptr, As, Bs);
  else
    tile_mm64<T, true, false, NT>(C, A, B, (const int*)nullptr, As, Bs);
}

// Forward substitution, unit lower L: Y(K,R) <- L(K,K)^-1 P Y(K,R).
template <typename T>
__global__ void __launch_bounds__(GEMM_THREADS) k_fwd_diag(const T* env, T* rhs, const Prob* probs,
                                                           Tables tb, int K, const int* active, const int* piv) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  if (K >= P.nt || (active && !active[e])) return;
  const int R = blockIdx.x;
  if (R >= P.nrt) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* D = reinterpret_cast<T*>(smem_raw);
  load_tile_n(D, tile_ptr(const_cast<T*>(env), P, tb, K, K), GEMM_THREADS);
  __syncthreads();
  col_solve_lower_unit(rhs_ptr(rhs, P, K, R), D, piv ? piv + P.rowv + (int64_t)K * TS : (const int*)nullptr);
}

// Y(I,R) -= L(I,K) Y(K,R) for I in (K, Imax(K)].
template <typename T>
__global__ void __launch_bounds__(MMThreads<T>::value) k_fwd_update(const T* env, T* rhs, const Prob* probs, Tables tb, int K,
                                                         const int* active) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  if (K >= P.nt || (active && !active[e])) return;
  const int nI = tb.Imax[P.trow + K] - K;
  const int w = blockIdx.x;
  if (w >= nI * P.nrt) return;
  const int I = K + 1 + w / P.nrt, R = w % P.nrt;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* As = reinterpret_cast<T*>(smem_raw);
  T* Bs = As + TS * SP;
  tile_mm64<T, true>(rhs_ptr(rhs, P, I, R), tile_ptr(const_cast<T*>(env), P, tb, I, K), rhs_ptr(rhs, P, K, R),
                     (const int*)nullptr, As, Bs);
}

// Backward substitution, upper U: Y(K,R) <- U(K,K)^-1 Y(K,R).
template <typename T>
__global__ void __launch_bounds__(GEMM_THREADS) k_bwd_diag(const T* env, T* rhs, const Prob* probs,
                                                           Tables tb, int K, const int* active) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  if (K >= P.nt || (active && !active[e])) return;
  const int R = blockIdx.x;
  if (R >= P.nrt) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* D = reinterpret_cast<T*>(smem_raw);
  load_tile_n(D, tile_ptr(const_cast<T*>(env), P, tb, K, K), GEMM_THREADS);
  __syncthreads();
  col_solve_upper(rhs_ptr(rhs, P, K, R), D);
}

// Y(I,R) -= U(I,K) Y(K,R) for I in [Imin(K), K).
template <typename T>
__global__ void __launch_bounds__(MMThreads<T>::value) k_bwd_update(const T* env, T* rhs, const Prob* probs, Tables tb, int K,
                                                         const int* active) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  if (K >= P.nt || (active && !active[e])) return;
  const int i0 = tb.Imin[P.trow + K];
  const int nI = K - i0;
  const int w = blockIdx.x;
  if (w >= nI * P.nrt) return;
  const int I = i0 + w / P.nrt, R = w % P.nrt;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* As = reinterpret_cast<T*>(smem_raw);
  T* Bs = As + TS * SP;
  tile_mm64<T, true>(rhs_ptr(rhs, P, I, R), tile_ptr(const_cast<T*>(env), P, tb, I, K), rhs_ptr(rhs, P, K, R),
                     (const int*)nullptr, As, Bs);
}

// Transposed forward step K: W(K,R) <- U(K,K)^-T W(K,R).
template <typename T>
__global__ void __launch_bounds__(GEMM_THREADS) k_tfwd_diag(const T* env, T* rhs, const Prob* probs, Tables tb,
                                                            int K, const int* active) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  if (K >= P.nt || (active && !active[e])) return;
  const int R = blockIdx.x;
  if (R >= P.nrt) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* D = reinterpret_cast<T*>(smem_raw);
  load_tile_trans_n(D, tile_ptr(const_cast<T*>(env), P, tb, K, K), GEMM_THREADS);
  __syncthreads();
  col_solve_lower_trans(rhs_ptr(rhs, P, K, R), D);
}

// W(J,R) -= U(K,J)^T W(K,R) for J in (K, J1(K)].
template <typename T>
__global__ void __launch_bounds__(MMThreads<T>::value) k_tfwd_update(const T* env, T* rhs, const Prob* probs, Tables tb,
                                                              int K, const int* active) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  if (K >= P.nt || (active && !active[e])) return;
  const int nJ = tb.J1[P.trow + K] - K;
  const int w = blockIdx.x;
  if (w >= nJ * P.nrt) return;
  const int J = K + 1 + w / P.nrt, R = w % P.nrt;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* As = reinterpret_cast<T*>(smem_raw);
  T* Bs = As + TS * SP;
  tile_mm64<T, true, true>(rhs_ptr(rhs, P, J, R), tile_ptr(const_cast<T*>(env), P, tb, K, J), rhs_ptr(rhs, P, K, R),
                           (const int*)nullptr, As, Bs);
}

// Transposed backward step K: W(K,R) <- P_K^T L(K,K)^-T W(K,R).
template <typename T>
__global__ void __launch_bounds__(GEMM_THREADS) k_tbwd_diag(const T* env, T* rhs, const Prob* probs, Tables tb,
                                                            int K, const int* active, const int* piv) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  if (K >= P.nt || (active && !active[e])) return;
  const int R = blockIdx.x;
  if (R >= P.nrt) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* D = reinterpret_cast<T*>(smem_raw);
  load_tile_trans_n(D, tile_ptr(const_cast<T*>(env), P, tb, K, K), GEMM_THREADS);
  __syncthreads();
  col_solve_upper_unit_trans(rhs_ptr(rhs, P, K, R), D, piv ? piv + P.rowv + (int64_t)K * TS : (const int*)nullptr);
}

// W(I,R) -= L(K,I)^T W(K,R) for I in [J0(K), K).
template <typename T>
__global__ void __launch_bounds__(MMThreads<T>::value) k_tbwd_update(const T* env, T* rhs, const Prob* probs, Tables tb,
                                                              int K, const int* active) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  if (K >= P.nt || (active && !active[e])) return;
  const int i0 = tb.J0[P.trow + K];
  const int nI = K - i0;
  const int w = blockIdx.x;
  if (w >= nI * P.nrt) return;
  const int I = i0 + w / P.nrt, R = w % P.nrt;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* As = reinterpret_cast<T*>(smem_raw);
  T* Bs = As + TS * SP;
  tile_mm64<T, true, true>(rhs_ptr(rhs, P, I, R), tile_ptr(const_cast<T*>(env), P, tb, K, I), rhs_ptr(rhs, P, K, R),
                           (const int*)nullptr, As, Bs);
}

// Row-oriented (left-looking) solves: one launch per tile row, one CTA per
// (right-hand-side tile, problem).  The CTA accumulates the products of its
// row's strip in registers and finishes with the diagonal tile, so Y(I,R) is
// written once per solve instead of at every step of the right-looking form,
// and the forward step needs one launch instead of two:
//   forward  Y(I) <- L(I,I)^-1 P_I (Y(I) - sum_{K in [J0(I), I)} L(I,K) Y(K))
//   backward Y(I) <- U(I,I)^-1     (Y(I) - sum_{K in (I, J1(I)]} U(I,K) Y(K))
// (the same eliminations as the reference's, source/mat_solve_gaussian.f90:
// 231-262 and 348-358, summed per row instead of per column).
template <typename T, bool FWD>
__global__ void __launch_bounds__(MMThreads<T>::value) k_solve_row(const T* env, T* rhs, const Prob* probs, Tables tb,
                                                                   int I, const int* active, const int* piv) {
  constexpr int NT = MMThreads<T>::value;
  constexpr int CW = NT == 128 ? 4 : 8;
  const int e = blockIdx.y;
  const Prob P = probs[e];
  if (I >= P.nt || (active && !active[e])) return;
  const int R = blockIdx.x;
  if (R >= P.nrt) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* As = reinterpret_cast<T*>(smem_raw);
  T* Bs = As + TS * SPA;
  T* D = Bs + TS * SP;
  const int k0 = FWD ? tb.J0[P.trow + I] : I + 1;
  const int k1 = FWD ? I : tb.J1[P.trow + I] + 1;
  const int t = threadIdx.x;
  const int tx = t % (NT / 8), ty = t / (NT / 8);
  T acc[8][CW];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < CW; ++j) acc[i][j] = T(0);
  for (int K = k0; K < k1; ++K) {
    const T* A = tile_ptr(const_cast<T*>(env), P, tb, I, K);
    const T* B = rhs_ptr(rhs, P, K, R);
    for (int idx = t; idx < TS2 / 4; idx += NT) {
      const int r = idx / (TS / 4), c4 = (idx % (TS / 4)) * 4;
      T a[4], b[4];
      ld4(A + r * TS + c4, a);
      ld4(B + r * TS + c4, b);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        As[r * SPA + c4 + q] = a[q];
        Bs[r * SP + c4 + q] = b[q];
      }
    }
    __syncthreads();
#pragma unroll 2
    for (int k = 0; k < TS; ++k) {
      T a[8], b[CW];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        a[i] = As[(4 * ty + i) * SPA + k];
        a[4 + i] = As[(32 + 4 * ty + i) * SPA + k];
      }
      ld4(Bs + k * SP + 4 * tx, b);
      if (CW == 8) ld4(Bs + k * SP + 32 + 4 * tx, b + 4);
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < CW; ++j) mac(acc[i][j], a[i], b[j]);
    }
    // renormalise the double-float sums once per tile (no-op for float and double)
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < CW; ++j) acc[i][j] = mac_finish(acc[i][j]);
    __syncthreads();
  }
  // Y(I,R) - acc, then the diagonal tile's triangular solve
  T* y = rhs_ptr(rhs, P, I, R);
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int row = (i < 4 ? 4 * ty + i : 32 + 4 * ty + (i - 4));
#pragma unroll
    for (int h = 0; h < CW / 4; ++h) {
      T* cp = y + row * TS + 32 * h + 4 * tx;
#pragma unroll
      for (int j = 0; j < 4; ++j) cp[j] = acc_apply<T, T>(cp[j], acc[i][4 * h + j], true);
    }
  }
  load_tile_n(D, tile_ptr(const_cast<T*>(env), P, tb, I, I), NT);
  __syncthreads();  // the block's writes of Y(I,R) and D are visible to every thread
  if (FWD)
    col_solve_lower_unit(y, D, piv ? piv + P.rowv + (int64_t)I * TS : (const int*)nullptr);
  else
    col_solve_upper(y, D);
}

template <typename T>
static size_t smem_bytes() { return 2 * TS * SP * sizeof(T); }
// the row solve holds the left operand (stride SPA), the right one and the diagonal tile
template <typename T>
static size_t smem_bytes_row() { return (TS * SPA + 2 * TS * SP) * sizeof(T); }
// the panel holds the diagonal tile plus one SPA-strided work tile (two for
// FP64, whose row solve also stages the transposed diagonal tile)
template <typename T>
static size_t smem_bytes_panel() {
  return (TS * SP + (std::is_same<T, double>::value ? 2 : 1) * TS * SPA) * sizeof(T);
}

template <typename T>
void setup_factor_kernels() {
  const int bytes = (int)smem_bytes<T>();
  cudaFuncSetAttribute(k_diag<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  cudaFuncSetAttribute(k_panel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes_panel<T>());
  cudaFuncSetAttribute(k_trailing<T, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  cudaFuncSetAttribute(k_trailing<T, 128>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if constexpr (std::is_same<T, float>::value) {
    cudaFuncSetAttribute(k_trailing<T, 64, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(k_trailing<T, 128, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  }
  cudaFuncSetAttribute(k_fwd_diag<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  cudaFuncSetAttribute(k_fwd_update<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  cudaFuncSetAttribute(k_bwd_diag<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  cudaFuncSetAttribute(k_bwd_update<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  cudaFuncSetAttribute(k_tfwd_diag<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  cudaFuncSetAttribute(k_tfwd_update<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  cudaFuncSetAttribute(k_tbwd_diag<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  cudaFuncSetAttribute(k_tbwd_update<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  cudaFuncSetAttribute(k_solve_row<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes_row<T>());
  cudaFuncSetAttribute(k_solve_row<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes_row<T>());
}

// The solve updates as strips (FP32 and double-float only; the FP64 path keeps
// the one-tile kernels).
template <typename T>
static void launch_strip_t(int mode, int items, int nprob, T* env, T* rhs, const Prob* probs, Tables tb, int K,
                           int fuse_rhs, const int* active, int* err, cudaStream_t s, bool wide) {
  if constexpr (!std::is_same<T, double>::value)
    launch_strip<T>(mode, items, nprob, env, rhs, probs, tb, K, fuse_rhs, active, err, s, wide);
}

template <typename T>
int launch_factor(const StepPlan& sp, T* env, T* rhs, const Prob* probs, Tables tb, int nprob, int fuse_rhs,
                  const int* active, int* err, double piv_thr, int* piv, cudaStream_t s, int trail_threads,
                  int k_begin, int k_end) {
  if (trail_threads != 64 && trail_threads != 128) trail_threads = MMThreads<T>::value;
  const size_t sm = smem_bytes<T>();
  int nk = 0;
  if (k_end < 0 || k_end > sp.ntmax) k_end = sp.ntmax;
  for (int K = std::max(k_begin, 0); K < k_end; ++K) {
    const int np = fuse_rhs ? sp.panel_rhs[K] : sp.panel[K];
    if (std::is_same<T, dfl>::value && sp.strip && sp.dfl_inv && piv) {
      // double-float diagonal tile with its inverted triangles, the panel as products
      nk += launch_dfl_panel_inv(sp, reinterpret_cast<dfl*>(env), reinterpret_cast<dfl*>(rhs), probs, tb, nprob, K,
                                 fuse_rhs, active, err, piv_thr, piv, sp.dfl_inv, s);
    } else {
      k_diag<T><<<dim3(1, nprob), NTHREADS, sm, s>>>(env, probs, tb, K, active, err, piv_thr, piv);
      ++nk;
    }
    if (np > 0 && !(std::is_same<T, dfl>::value && sp.strip && sp.dfl_inv && piv)) {
      k_panel<T><<<dim3(np, nprob), GEMM_THREADS, smem_bytes_panel<T>(), s>>>(env, rhs, probs, tb, K, fuse_rhs,
                                                                             active, piv);
      ++nk;
    }
    const int nt = fuse_rhs ? sp.trail_rhs[K] : sp.trail[K];
    if (nt > 0) {
      if (std::is_same<T, float>::value && sp.tc && fuse_rhs)
        launch_tc_update(0, sp.trail_tc[K], nprob, reinterpret_cast<float*>(env), reinterpret_cast<float*>(rhs),
                         probs, tb, K, active, err, s);
      else if (std::is_same<T, dfl>::value && sp.oz && fuse_rhs && sp.oz_img)
        nk += launch_oz_update(sp, reinterpret_cast<dfl*>(env), reinterpret_cast<dfl*>(rhs), probs, tb, nprob, K,
                               active, err, s) - 1;
      else if (!std::is_same<T, double>::value && sp.strip)
        launch_strip_t(0, fuse_rhs ? sp.strip_trail_rhs[K] : sp.strip_trail[K], nprob, env, rhs, probs, tb, K,
                       fuse_rhs, active, err, s, false);
      else if (trail_threads == 128)
        k_trailing<T, 128><<<dim3(nt, nprob), 128, sm, s>>>(env, rhs, probs, tb, K, fuse_rhs, active);
      else
        k_trailing<T, 64><<<dim3(nt, nprob), 64, sm, s>>>(env, rhs, probs, tb, K, fuse_rhs, active);
      ++nk;
      // the problems whose step K is marked wide run in the wide instantiation
      if constexpr (std::is_same<T, float>::value) {
        if (tb.wide && K < (int)sp.wide_any.size() && sp.wide_any[K]) {
          if (sp.strip)
            launch_strip_t(0, fuse_rhs ? sp.strip_trail_rhs[K] : sp.strip_trail[K], nprob, env, rhs, probs, tb, K,
                           fuse_rhs, active, err, s, true);
          else if (trail_threads == 128)
            k_trailing<T, 128, true><<<dim3(nt, nprob), 128, sm, s>>>(env, rhs, probs, tb, K, fuse_rhs, active);
          else
            k_trailing<T, 64, true><<<dim3(nt, nprob), 64, sm, s>>>(env, rhs, probs, tb, K, fuse_rhs, active);
          ++nk;
        }
      }
    }
  }
  return nk;
}

template <typename T>
int launch_forward(const StepPlan& sp, const T* env, T* rhs, const Prob* probs, Tables tb, int nprob,
                   const int* active, const int* piv, cudaStream_t s) {
  const size_t sm = smem_bytes<T>();
  int nk = 0;
  if (sp.row_solve) {
    for (int I = 0; I < sp.ntmax; ++I) {
      k_solve_row<T, true><<<dim3(sp.nrtmax, nprob), MMThreads<T>::value, smem_bytes_row<T>(), s>>>(
          env, rhs, probs, tb, I, active, piv);
      ++nk;
    }
    return nk;
  }
  for (int K = 0; K < sp.ntmax; ++K) {
    k_fwd_diag<T><<<dim3(sp.nrtmax, nprob), GEMM_THREADS, sm, s>>>(env, rhs, probs, tb, K, active, piv);
    ++nk;
    if (sp.fwd[K] > 0) {
      if (std::is_same<T, float>::value && sp.tc_solve)
        launch_tc_update(1, sp.fwd_tc[K], nprob, reinterpret_cast<float*>(const_cast<T*>(env)),
                         reinterpret_cast<float*>(rhs), probs, tb, K, active, sp.tc_err, s);
      else if (!std::is_same<T, double>::value && sp.strip)
        launch_strip_t(1, sp.strip_fwd[K], nprob, const_cast<T*>(env), rhs, probs, tb, K, 0, active, sp.tc_err, s,
                       false);
      else
        k_fwd_update<T><<<dim3(sp.fwd[K], nprob), MMThreads<T>::value, sm, s>>>(env, rhs, probs, tb, K, active);
      ++nk;
    }
  }
  return nk;
}

template <typename T>
int launch_backward(const StepPlan& sp, const T* env, T* rhs, const Prob* probs, Tables tb, int nprob,
                    const int* active, cudaStream_t s) {
  const size_t sm = smem_bytes<T>();
  int nk = 0;
  if (sp.row_solve) {
    for (int I = sp.ntmax - 1; I >= 0; --I) {
      k_solve_row<T, false><<<dim3(sp.nrtmax, nprob), MMThreads<T>::value, smem_bytes_row<T>(), s>>>(
          env, rhs, probs, tb, I, active, nullptr);
      ++nk;
    }
    return nk;
  }
  for (int K = sp.ntmax - 1; K >= 0; --K) {
    k_bwd_diag<T><<<dim3(sp.nrtmax, nprob), GEMM_THREADS, sm, s>>>(env, rhs, probs, tb, K, active);
    ++nk;
    if (sp.bwd[K] > 0) {
      if (std::is_same<T, float>::value && sp.tc_solve)
        launch_tc_update(2, sp.bwd_tc[K], nprob, reinterpret_cast<float*>(const_cast<T*>(env)),
                         reinterpret_cast<float*>(rhs), probs, tb, K, active, sp.tc_err, s);
      else if (!std::is_same<T, double>::value && sp.strip)
        launch_strip_t(2, sp.strip_bwd[K], nprob, const_cast<T*>(env), rhs, probs, tb, K, 0, active, sp.tc_err, s,
                       false);
      else
        k_bwd_update<T><<<dim3(sp.bwd[K], nprob), MMThreads<T>::value, sm, s>>>(env, rhs, probs, tb, K, active);
      ++nk;
    }
  }
  return nk;
}

template <typename T>
void launch_forward_t(const StepPlan& sp, const T* env, T* rhs, const Prob* probs, Tables tb, int nprob,
                      const int* active, cudaStream_t s) {
  const size_t sm = smem_bytes<T>();
  for (int K = 0; K < sp.ntmax; ++K) {
    k_tfwd_diag<T><<<dim3(sp.nrtmax, nprob), GEMM_THREADS, sm, s>>>(env, rhs, probs, tb, K, active);
    if (sp.tfwd[K] > 0)
      k_tfwd_update<T><<<dim3(sp.tfwd[K], nprob), MMThreads<T>::value, sm, s>>>(env, rhs, probs, tb, K, active);
  }
}

template <typename T>
void launch_backward_t(const StepPlan& sp, const T* env, T* rhs, const Prob* probs, Tables tb, int nprob,
                       const int* active, const int* piv, cudaStream_t s) {
  const size_t sm = smem_bytes<T>();
  for (int K = sp.ntmax - 1; K >= 0; --K) {
    k_tbwd_diag<T><<<dim3(sp.nrtmax, nprob), GEMM_THREADS, sm, s>>>(env, rhs, probs, tb, K, active, piv);
    if (sp.tbwd[K] > 0)
      k_tbwd_update<T><<<dim3(sp.tbwd[K], nprob), MMThreads<T>::value, sm, s>>>(env, rhs, probs, tb, K, active);
  }
}

template void launch_forward_t<double>(const StepPlan&, const double*, double*, const Prob*, Tables, int, const int*,
                                       cudaStream_t);
template void launch_backward_t<double>(const StepPlan&, const double*, double*, const Prob*, Tables, int,
                                        const int*, const int*, cudaStream_t);
template void launch_forward_t<dfl>(const StepPlan&, const dfl*, dfl*, const Prob*, Tables, int, const int*,
                                    cudaStream_t);
template void launch_backward_t<dfl>(const StepPlan&, const dfl*, dfl*, const Prob*, Tables, int, const int*,
                                     const int*, cudaStream_t);
template void launch_forward_t<float>(const StepPlan&, const float*, float*, const Prob*, Tables, int, const int*,
                                      cudaStream_t);
template void launch_backward_t<float>(const StepPlan&, const float*, float*, const Prob*, Tables, int, const int*,
                                       const int*, cudaStream_t);

template void setup_factor_kernels<float>();
template void setup_factor_kernels<dfl>();
template int launch_factor<dfl>(const StepPlan&, dfl*, dfl*, const Prob*, Tables, int, int, const int*, int*,
                                 double, int*, cudaStream_t, int, int, int);
template int launch_forward<dfl>(const StepPlan&, const dfl*, dfl*, const Prob*, Tables, int, const int*,
                                  const int*, cudaStream_t);
template int launch_backward<dfl>(const StepPlan&, const dfl*, dfl*, const Prob*, Tables, int, const int*,
                                   cudaStream_t);
template void setup_factor_kernels<double>();
template int launch_factor<float>(const StepPlan&, float*, float*, const Prob*, Tables, int, int, const int*,
                                   int*, double, int*, cudaStream_t, int, int, int);
template int launch_factor<double>(const StepPlan&, double*, double*, const Prob*, Tables, int, int,
                                    const int*, int*, double, int*, cudaStream_t, int, int, int);
template int launch_forward<float>(const StepPlan&, const float*, float*, const Prob*, Tables, int,
                                    const int*, const int*, cudaStream_t);
template int launch_forward<double>(const StepPlan&, const double*, double*, const Prob*, Tables, int,
                                     const int*, const int*, cudaStream_t);
template int launch_backward<float>(const StepPlan&, const float*, float*, const Prob*, Tables, int,
                                     const int*, cudaStream_t);
template int launch_backward<double>(const StepPlan&, const double*, double*, const Prob*, Tables, int,
                                      const int*, cudaStream_t);

}  // namespace fdm
