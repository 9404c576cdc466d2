// strip_update.cu - tile updates of the factor and of the refinement solves on
// the FP32 pipes, with the streamed operand tiles staged by bulk copies.
//
// Every update of the band LU has the form  C(I) -= A(I) B  for a run of tile
// rows I sharing one operand tile B:
//   factor trailing update (source/mat_solve_gaussian.f90:231-262 in tile
//   form): A(I) = L(I,K), B = U(K,J) or the right-hand-side tile Y(K,R),
//   C(I) = A(I,J) or Y(I,R), I in (K, Imax(K)];
//   forward solve update: A(I) = L(I,K), B = Y(K,R), C(I) = Y(I,R);
//   backward solve update (:348-358): A(I) = U(I,K), I in [Imin(K), K).
// One CTA takes one B tile and up to G consecutive tile rows: B is staged once
// (plain coalesced loads), the A tiles stream through a two-stage shared ring
// filled by cp.async.bulk row copies that complete on an mbarrier, so the
// next A tile is in flight while the current one is multiplied (a second
// mbarrier per stage collects the threads' releases before warp 0 refills
// it; no CTA-wide barrier inside the loop); C is read,
// updated and written with 16-byte accesses (FP32: loaded into registers
// before the product).  The product is register-blocked like the one-tile
// kernels (128 threads, 8 rows x 4 columns per thread) but reads A along k
// with 16-byte loads (row-major A, padded stride), three 16-byte shared loads
// per 32 multiply-adds for FP32.
//
// The double-float factor's panel uses the same kernel on the inverted
// triangles of the factored diagonal tile (k_diag_inv below):
//   mode 3: L(I,K) = A(I,K) U(K,K)^-1, streamed A(I,K), fixed U^-1, in place;
//   mode 4: U(K,J) = L(K,K)^-1 P A(K,J) (and Y(K,R) alike when the right-hand
//           sides ride along): fixed left operand L^-1, streamed right operand
//           whose rows the copies take in the pivot order P, in place.
// These replace the 64-step triangular substitutions (one dependent chain per
// thread, two warps per tile) by tile products.
//
// Waits are bounded: a stage whose copy does not land within the limit sets
// the problem's status word and the CTA stops after waiting (bounded) for the
// copies it issued.
#include <cstdint>
#include <type_traits>

#include "fdm_internal.cuh"
#include "fdm_kernels.h"

namespace fdm {
namespace strip {

constexpr int NT = 128;
constexpr int NS = 2;  // A stages
constexpr long long WAIT_LIMIT = 1ll << 22;

// padded shared stride (elements): rows stay 16-byte aligned and the two row
// groups a warp reads in one k step fall on different bank groups
template <typename T> struct Stride { static constexpr int value = 68; };
template <> struct Stride<dfl> { static constexpr int value = 66; };

template <typename T>
constexpr int smem_bytes() {
  return (1 + NS) * TS * Stride<T>::value * (int)sizeof(T) + 16 * NS + 16;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (long long i = 0; i < WAIT_LIMIT; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

// 16 bytes of consecutive elements: 4 floats or 2 double-floats
template <typename T> struct KVec { static constexpr int value = 16 / (int)sizeof(T); };
template <typename T>
__device__ __forceinline__ void ldv(const T* p, T* v);
template <>
__device__ __forceinline__ void ldv<float>(const float* p, float* v) {
  const float4 q = *reinterpret_cast<const float4*>(p);
  v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
}
template <>
__device__ __forceinline__ void ldv<dfl>(const dfl* p, dfl* v) {
  const float4 q = *reinterpret_cast<const float4*>(p);
  v[0] = dfl(q.x, q.y); v[1] = dfl(q.z, q.w);
}

// Copy tile A (TS x TS, row-major in global memory) into a padded stage: warp
// 0 only; lane 0 announces the byte count, every lane copies two rows.
template <typename T>
__device__ __forceinline__ void issue_tile(T* stage, const T* A, uint32_t bar, const int* perm = nullptr) {
  constexpr int SPS = Stride<T>::value;
  const int lane = threadIdx.x & 31;
  if (lane == 0) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"((uint32_t)(TS2 * sizeof(T)))
                 : "memory");
  }
  __syncwarp();
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int r = lane + 32 * h;
    bulk_g2s(smem_u32(stage + r * SPS), A + (perm ? perm[r] : r) * TS, TS * sizeof(T), bar);
  }
}

// MODE 0: factor trailing update (with the fused right-hand-side columns when
// aux != 0); 1: forward solve update; 2: backward solve update; 3 and 4: the
// double-float panel from the inverted diagonal triangles (inv: U^-1 then
// L^-1 of every problem, piv: the diagonal tile's row order; MODE 4 with the
// right-hand sides when aux != 0); 5: Y(K,R) = U(K,K)^-1 Y(K,R) with the kept
// inverses (inv: aux tiles a problem, one per step).  Acc is the
// accumulator type (facc: double-float sums of FP32 products); WIDE selects
// the FP32 problems whose step K is marked for wide accumulation.
template <typename T, int MODE, typename Acc, bool WIDE>
__global__ void __launch_bounds__(NT) k_strip(T* env, T* rhs, const Prob* probs, Tables tb, int K, int aux,
                                              int G, const int* active, int* err, const T* inv, const int* piv) {
  constexpr int SPS = Stride<T>::value;
  constexpr int KV = KVec<T>::value;
  constexpr bool STREAM_B = MODE >= 4;  // the streamed tiles are the right operand
  constexpr bool SUB = MODE <= 2;       // C -= A B, else C = A B
  const int e = blockIdx.y;
  const Prob P = probs[e];
  if (K >= P.nt || (active && !active[e])) return;
  if (MODE == 0 && std::is_same<T, float>::value) {
    const bool w = tb.wide && tb.wide[P.trow + K];
    if (w != WIDE) return;
  }
  // n: streamed tiles of the step; nC: fixed-operand tiles (B columns, or one)
  int i0 = 0, n, nC, nJ = 0;
  if (MODE == 2) {
    i0 = tb.Imin[P.trow + K];
    n = K - i0;
  } else if (MODE == 4) {
    nJ = tb.J1[P.trow + K] - K;
    n = nJ + (aux ? P.nrt : 0);
  } else if (MODE == 5) {
    n = P.nrt;
  } else {
    i0 = K + 1;
    n = tb.Imax[P.trow + K] - K;
  }
  if (MODE == 0) {
    nJ = tb.J1[P.trow + K] - K;
    nC = nJ + (aux ? P.nrt : 0);
  } else if (MODE >= 3) {
    nC = 1;
  } else {
    nC = P.nrt;
  }
  if (n <= 0) return;
  const int nch = (n + G - 1) / G;
  if ((int)blockIdx.x >= nC * nch) return;
  const int c = blockIdx.x / nch, ch = blockIdx.x % nch;
  const int ia = ch * G;  // first streamed tile (index into the step's run)
  const int nt = min(G, n - ia);
  const int* prow = (MODE == 4 && piv) ? piv + P.rowv + (int64_t)K * TS : nullptr;
  // fixed operand, streamed tile q, output tile q
  const T* F;
  if (MODE == 3)
    F = inv + (int64_t)e * 2 * TS2;
  else if (MODE == 4)
    F = inv + (int64_t)e * 2 * TS2 + TS2;
  else if (MODE == 5)
    F = inv + ((int64_t)e * aux + K) * TS2;
  else if (MODE == 0 && c < nJ)
    F = tile_ptr(env, P, tb, K, K + 1 + c);
  else
    F = rhs_ptr(rhs, P, K, MODE == 0 ? c - nJ : c);
  auto streamed = [&](int q) -> T* {
    if (MODE == 5) return rhs_ptr(rhs, P, K, q);
    if (MODE == 4) return q < nJ ? tile_ptr(env, P, tb, K, K + 1 + q) : rhs_ptr(rhs, P, K, q - nJ);
    return tile_ptr(env, P, tb, i0 + q, K);
  };
  auto output = [&](int q) -> T* {
    if (MODE >= 3) return streamed(q);
    const int I = i0 + q;
    if (MODE == 0 && c < nJ) return tile_ptr(env, P, tb, I, K + 1 + c);
    return rhs_ptr(rhs, P, I, MODE == 0 ? c - nJ : c);
  };

  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* Fs = reinterpret_cast<T*>(smem_raw);
  T* Ring = Fs + TS * SPS;
  // bars[s]: stage s filled (the copies' bytes); bars[NS + s]: stage s read
  // by every thread (NT arrivals), after which warp 0 refills it
  uint64_t* bars = reinterpret_cast<uint64_t*>(Ring + NS * TS * SPS);
  const int t = threadIdx.x;
  if (t == 0) {
    for (int s = 0; s < NS; ++s) {
      mbar_init(smem_u32(&bars[s]), 1);
      mbar_init(smem_u32(&bars[NS + s]), NT);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (t < 32)
    for (int s = 0; s < NS && s < nt; ++s) issue_tile(Ring + s * TS * SPS, streamed(ia + s), smem_u32(&bars[s]), prow);
  // the fixed operand while the first streamed tiles are in flight
  for (int idx = t; idx < TS2 / 4; idx += NT) {
    const int r = idx / (TS / 4), c4 = (idx % (TS / 4)) * 4;
    T b[4];
    ld4(F + r * TS + c4, b);
    st4(Fs + r * SPS + c4, b);
  }
  __syncthreads();

  // No CTA barrier inside the loop: every thread waits on the stage it reads
  // and releases it; warp 0 waits for the release before refilling, so the
  // other warps run ahead into the next (already filled) stage.
  const int tx = t % 16, ty = t / 16;
  int issued = min(NS, nt), done = 0;
  bool ok = true;
  for (int it = 0; it < nt; ++it) {
    const int s = it % NS;
    const uint32_t parity = (uint32_t)((it / NS) & 1);
    ok = mbar_wait(smem_u32(&bars[s]), parity);
    if (!ok) break;
    done = it + 1;
    T* C = output(ia + it);
    // FP32 updates: this tile's C rows in registers before the product
    constexpr bool PF = std::is_same<T, float>::value && SUB;
    T cv[8][4];
    if (PF) {
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int row = i < 4 ? 4 * ty + i : 32 + 4 * ty + (i - 4);
        ld4(C + row * TS + 4 * tx, cv[i]);
      }
    }
    const T* As = STREAM_B ? Fs : Ring + s * TS * SPS;
    const T* Bs = STREAM_B ? Ring + s * TS * SPS : Fs;
    Acc acc[8][4];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = acc_zero<Acc>();
#pragma unroll 2
    for (int k0 = 0; k0 < TS; k0 += KV) {
      T a[8][KV], b[KV][4];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int row = i < 4 ? 4 * ty + i : 32 + 4 * ty + (i - 4);
        ldv(As + row * SPS + k0, a[i]);
      }
#pragma unroll
      for (int kk = 0; kk < KV; ++kk) ld4(Bs + (k0 + kk) * SPS + 4 * tx, b[kk]);
#pragma unroll
      for (int kk = 0; kk < KV; ++kk)
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) mac(acc[i][j], a[i][kk], b[kk][j]);
    }
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&bars[NS + s])) : "memory");
    if (t < 32 && issued < nt) {
      bool rel = true;
      if (t == 0) rel = mbar_wait(smem_u32(&bars[NS + s]), parity);
      rel = __shfl_sync(0xffffffffu, rel ? 1 : 0, 0) != 0;
      if (!rel) {
        ok = false;
        break;
      }
      issue_tile(Ring + s * TS * SPS, streamed(ia + issued), smem_u32(&bars[s]), prow);
      ++issued;
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int row = i < 4 ? 4 * ty + i : 32 + 4 * ty + (i - 4);
      T* cp = C + row * TS + 4 * tx;
      T v[4];
      if (PF) {
#pragma unroll
        for (int j = 0; j < 4; ++j) v[j] = cv[i][j];
      } else if (SUB) {
        ld4(cp, v);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) v[j] = acc_apply<T, Acc>(v[j], acc[i][j], SUB);
      st4(cp, v);
    }
  }
  if (!ok) {
    atomicExch(&err[e], (int)FDMGPU_ERR_CUDA);
    // the copies warp 0 issued but no thread consumed must land before the
    // CTA leaves (issued is exact in warp 0)
    if (t == 0)
      for (int it = done; it < issued; ++it) mbar_wait(smem_u32(&bars[it % NS]), (uint32_t)((it / NS) & 1));
  }
}

// Factor the diagonal tile (K,K) of every active problem as k_diag does
// (tile-local partial pivoting, smallest pivot checked) and write the inverses
// of its triangles to inv (per problem U^-1, then L^-1 of the unit lower
// triangle): column j of each inverse solves a triangular system with the
// unit vector e_j (the substitutions of the solves), threads 0-63 for U,
// 64-127 for L.
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_diag_inv(T* env, const Prob* probs, Tables tb, int K, const int* active,
                                                       int* err, double piv_thr, int* piv, T* inv, T* keep,
                                                       int keep_slots) {
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
  tile_lu(D, &mp, perm);
  __syncthreads();
  store_tile(dtile, D);
  if (threadIdx.x < TS) piv[P.rowv + (int64_t)K * TS + threadIdx.x] = perm[threadIdx.x];
  if (threadIdx.x == 0 && !(mp >= piv_thr)) atomicExch(&err[e], (int)FDMGPU_ERR_ZERO_PIVOT);
  T* Ui = inv + (int64_t)e * 2 * TS2;
  T* Li = Ui + TS2;
  // each thread starts its column of the identity and solves it in place
  const int j = threadIdx.x % TS;
  if (threadIdx.x < 2 * TS) {
    T* g = threadIdx.x < TS ? Ui : Li;
    for (int r = 0; r < TS; ++r) g[r * TS + j] = T(r == j ? 1.0f : 0.0f, 0.0f);
    if (threadIdx.x < TS)
      col_solve_upper(Ui, D, j);
    else
      col_solve_lower_unit(Li, D, (const int*)nullptr, j);
  }
  if (keep) {
    // U^-1 of every step, for the backward solve with these factors
    __syncthreads();
    T* k = keep + ((int64_t)e * keep_slots + K) * TS2;
    for (int idx = threadIdx.x; idx < TS2; idx += blockDim.x) k[idx] = Ui[idx];
  }
}

template <typename T, int MODE, typename Acc, bool WIDE>
void set_smem() {
  cudaFuncSetAttribute(k_strip<T, MODE, Acc, WIDE>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes<T>());
}

}  // namespace strip

// Tile rows per CTA: the trailing update has ~25 rows per B tile and many B
// tiles; the solves have few B tiles (the right-hand-side columns), so they
// take shorter runs for more CTAs.
constexpr int STRIP_G_TRAIL = 8;
constexpr int STRIP_G_SOLVE = 4;

int strip_items(int nI, int nC, int G) { return nI > 0 ? nC * ((nI + G - 1) / G) : 0; }
int strip_rows(int mode) { return mode == 0 ? STRIP_G_TRAIL : STRIP_G_SOLVE; }

void setup_strip_kernels() {
  using namespace strip;
  cudaFuncSetAttribute(k_diag_inv<dfl>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(TS * SP * sizeof(dfl)));
  set_smem<dfl, 3, dfl, false>();
  set_smem<dfl, 4, dfl, false>();
  set_smem<dfl, 5, dfl, false>();
  set_smem<float, 0, float, false>();
  set_smem<float, 0, facc, true>();
  set_smem<float, 1, float, false>();
  set_smem<float, 2, float, false>();
  set_smem<dfl, 0, dfl, false>();
  set_smem<dfl, 1, dfl, false>();
  set_smem<dfl, 2, dfl, false>();
}

template <typename T>
void launch_strip(int mode, int items, int nprob, T* env, T* rhs, const Prob* probs, Tables tb, int K, int fuse_rhs,
                  const int* active, int* err, cudaStream_t s, bool wide) {
  using namespace strip;
  if (items <= 0) return;
  const dim3 grid(items, nprob);
  const int G = strip_rows(mode);
  const size_t sm = smem_bytes<T>();
  if constexpr (std::is_same<T, float>::value) {
    if (mode == 0 && wide)
      k_strip<float, 0, facc, true><<<grid, NT, sm, s>>>(env, rhs, probs, tb, K, fuse_rhs, G, active, err, nullptr,
                                                         nullptr);
    else if (mode == 0)
      k_strip<float, 0, float, false><<<grid, NT, sm, s>>>(env, rhs, probs, tb, K, fuse_rhs, G, active, err, nullptr, nullptr);
    else if (mode == 1)
      k_strip<float, 1, float, false><<<grid, NT, sm, s>>>(env, rhs, probs, tb, K, 0, G, active, err, nullptr, nullptr);
    else
      k_strip<float, 2, float, false><<<grid, NT, sm, s>>>(env, rhs, probs, tb, K, 0, G, active, err, nullptr, nullptr);
  } else {
    if (mode == 0)
      k_strip<dfl, 0, dfl, false><<<grid, NT, sm, s>>>(env, rhs, probs, tb, K, fuse_rhs, G, active, err, nullptr, nullptr);
    else if (mode == 1)
      k_strip<dfl, 1, dfl, false><<<grid, NT, sm, s>>>(env, rhs, probs, tb, K, 0, G, active, err, nullptr, nullptr);
    else
      k_strip<dfl, 2, dfl, false><<<grid, NT, sm, s>>>(env, rhs, probs, tb, K, 0, G, active, err, nullptr, nullptr);
  }
}

// Step K of the double-float factor's diagonal tile and panel with the
// inverted triangles: k_diag_inv, then the L tiles (mode 3) and the U and
// right-hand-side tiles (mode 4) as products; returns the launches.
int launch_dfl_panel_inv(const StepPlan& sp, dfl* env, dfl* rhs, const Prob* probs, Tables tb, int nprob, int K,
                         int fuse_rhs, const int* active, int* err, double piv_thr, int* piv, dfl* inv,
                         cudaStream_t s) {
  using namespace strip;
  k_diag_inv<dfl><<<dim3(1, nprob), NTHREADS, TS * SP * sizeof(dfl), s>>>(env, probs, tb, K, active, err, piv_thr,
                                                                          piv, inv, sp.dfl_uinv_keep, sp.ntmax);
  int nk = 1;
  const size_t sm = smem_bytes<dfl>();
  const int G = strip_rows(0);
  const int nL = sp.strip_panel_l[K], nU = fuse_rhs ? sp.strip_panel_u_rhs[K] : sp.strip_panel_u[K];
  if (nL > 0) {
    k_strip<dfl, 3, dfl, false><<<dim3(nL, nprob), NT, sm, s>>>(env, rhs, probs, tb, K, fuse_rhs, G, active, err,
                                                                inv, piv);
    ++nk;
  }
  if (nU > 0) {
    k_strip<dfl, 4, dfl, false><<<dim3(nU, nprob), NT, sm, s>>>(env, rhs, probs, tb, K, fuse_rhs, G, active, err,
                                                                inv, piv);
    ++nk;
  }
  return nk;
}

// Backward solve with the double-float factors of the last factorisation,
// whose U^-1 tiles were kept (sp.dfl_uinv_keep, the same problem order):
// per step K from the last, Y(K,R) = U(K,K)^-1 Y(K,R) as products (mode 5),
// then the update strips Y(I,R) -= U(I,K) Y(K,R).
int launch_dfl_backward_inv(const StepPlan& sp, dfl* env, dfl* rhs, const Prob* probs, Tables tb, int nprob,
                            const int* active, int* err, cudaStream_t s) {
  using namespace strip;
  const size_t sm = smem_bytes<dfl>();
  int nk = 0;
  for (int K = sp.ntmax - 1; K >= 0; --K) {
    k_strip<dfl, 5, dfl, false><<<dim3(strip_items(sp.nrtmax, 1, strip_rows(1)), nprob), NT, sm, s>>>(
        env, rhs, probs, tb, K, sp.ntmax, strip_rows(1), active, err, sp.dfl_uinv_keep, nullptr);
    ++nk;
    if (sp.strip_bwd[K] > 0) {
      launch_strip<dfl>(2, sp.strip_bwd[K], nprob, env, rhs, probs, tb, K, 0, active, err, s, false);
      ++nk;
    }
  }
  return nk;
}

template void launch_strip<float>(int, int, int, float*, float*, const Prob*, Tables, int, int, const int*, int*,
                                  cudaStream_t, bool);
template void launch_strip<dfl>(int, int, int, dfl*, dfl*, const Prob*, Tables, int, int, const int*, int*,
                                cudaStream_t, bool);

}  // namespace fdm
