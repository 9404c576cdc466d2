// oz_update.cu - the double-float trailing update of the escalation factor on
// the 5th-generation tensor cores, through exact integer slices.
//
// The escalation re-factorises, in double-float arithmetic (hi + lo floats,
// about 48 significand bits), the energies whose FP32 refinement stalls; its
// trailing update C(I,J) -= L(I,K) U(K,J) (the elimination of
// source/mat_solve_gaussian.f90:231-262 in tile form) is the dominant kernel
// of the mixed path.  Tensor cores add in FP32, so products of rounded pieces
// would lose the double-float accuracy in the sums.  Instead every operand
// row of L (column of U) is scaled by a power of two 2^E so that its largest
// element is below 1 in magnitude, and each element is cut into seven signed
// 7-bit integers:  x = 2^E sum_{i=1..7} a_i 2^(-7 i),  |a_i| <= 128,
// exact as bf16 values.  A product of two slices is an integer below 2^14;
// the sum over the 64 columns of a tile and over the (at most seven) slice
// pairs of one order s = i + j stays below 2^24, so one FP32 tensor-memory
// accumulator per order holds it EXACTLY.  The 34 slice pairs with s <= 9
// (dropped terms are ~2^-50 of the row and column maxima) run as bf16 MMAs
// (tcgen05.mma kind::f16, M = 128, N = 64, K = 16) into eight accumulators;
// the epilogue scales each order by 2^(E_m + F_n - 7 s), adds them from the
// smallest in double-float arithmetic and subtracts the sum from C.
//
// k_oz_slice   per step: each L tile (A operand, exponents per row) and each
//              U / right-hand-side tile (B operand, exponents per column,
//              transposed to K-major) cut into seven 8 KB bf16 images in the
//              K-major no-swizzle operand layout, written to a scratch pool.
// k_oz_mma     one CTA per (two tile rows, one tile column): the 14 + 7 images
//              are fetched with bulk copies (cp.async.bulk, completion on an
//              mbarrier), one thread issues 34 x 4 MMAs into a 512-column TMEM
//              allocation, the epilogue reads it with tcgen05.ld.
#include <cstdint>

#include "fdm_internal.cuh"
#include "fdm_kernels.h"

namespace fdm {
namespace oz {

constexpr int NSL = 7;                        // slices per operand
constexpr int SMAX = NSL + 2;                 // highest slice order kept (8 accumulators of 64 columns)
constexpr int IMG = TS * TS * 2;              // one bf16 image of a 64x64 tile: 8 KB
constexpr int TILE_IMGS = NSL * IMG;          // 56 KB per tile
constexpr int MMA_THREADS = 128;
constexpr int SMEM_MMA = 2 * TILE_IMGS + TILE_IMGS + (2 * TS + TS) * 4 + 1024 + 64;
constexpr int SMEM_SLICE = TS * TS * 8 + TILE_IMGS + TS * 4 + 64;
constexpr uint32_t TMEM_COLS = 512;
constexpr long long WAIT_LIMIT = 1ll << 20;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// K-major no-swizzle image of bf16: core matrix (r / 8, k / 8) of 8 rows x
// 16 bytes at 128-byte slots, eight per 8-row group.
__device__ __forceinline__ uint32_t img_off(int r, int k) {
  return (uint32_t)((((r >> 3) * (TS / 8) + (k >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1));
}
constexpr uint32_t LBO = 128;
constexpr uint32_t SBO = (TS / 8) * 128;

__device__ __forceinline__ uint64_t sdesc(uint32_t addr) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(LBO >> 4) << 16) | ((uint64_t)(SBO >> 4) << 32) |
         (1ull << 46);
}
// kind::f16 with bf16 operands (bits 7-9, 10-12 = 1), FP32 accumulator
// (bits 4-5 = 1), both K-major, N = 64 (bits 17-22), M = 128 (bits 24-28).
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(64 >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);

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
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %3, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %4, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(acc), "r"(IDESC)
      : "memory");
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
      "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// 16 columns of one TMEM lane quarter; the caller waits (tcgen05.wait::ld) once
// for a batch of such loads.
__device__ __forceinline__ void tmem_ld16_nowait(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

// Operand tiles of step K: A tile a is L(K+1+a, K); B tile c is U(K, K+1+c)
// for c < nJ, then the right-hand-side tiles Y(K, c - nJ).
struct StepShape {
  int nI, nJ, nC;
};
__device__ __forceinline__ StepShape shape(const Prob& P, const Tables& tb, int K) {
  StepShape s;
  s.nI = tb.Imax[P.trow + K] - K;
  s.nJ = tb.J1[P.trow + K] - K;
  s.nC = s.nJ + P.nrt;
  return s;
}

// Slices of one tile.  IS_A: the exponent is per row of the tile and image
// row r = tile row; else per column and image row = tile column (transposed).
template <bool IS_A>
__global__ void __launch_bounds__(256) k_oz_slice(const dfl* env, const dfl* rhs, const Prob* probs, Tables tb, int K,
                                                  const int* active, unsigned char* img, int* ex, int64_t slot_tiles,
                                                  int capI) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  if (K >= P.nt || (active && !active[e])) return;
  const StepShape sh = shape(P, tb, K);
  const int w = blockIdx.x;
  const dfl* src;
  int slot;
  if (IS_A) {
    if (w >= sh.nI) return;
    src = tile_ptr(const_cast<dfl*>(env), P, tb, K + 1 + w, K);
    slot = w;
  } else {
    if (w >= sh.nC) return;
    src = w < sh.nJ ? tile_ptr(const_cast<dfl*>(env), P, tb, K, K + 1 + w) : rhs_ptr(const_cast<dfl*>(rhs), P, K, w - sh.nJ);
    slot = capI + w;
  }
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* T = reinterpret_cast<float2*>(smem_raw);                 // the tile, 32 KB
  unsigned char* S = smem_raw + TS * TS * 8;                       // seven images, 56 KB
  int* E = reinterpret_cast<int*>(S + TILE_IMGS);                  // 64 exponents
  const int t = threadIdx.x;
  for (int idx = t; idx < TS * TS; idx += 256) T[idx] = reinterpret_cast<const float2*>(src)[idx];
  __syncthreads();
  // exponent of the row (A) or column (B): 2^E > max |hi| (frexp), 0 for an all-zero line
  if (t < TS) {
    float m = 0.f;
    for (int k = 0; k < TS; ++k) m = fmaxf(m, fabsf(IS_A ? T[t * TS + k].x : T[k * TS + t].x));
    int ex2 = 0;
    if (m > 0.f) frexpf(m, &ex2);
    E[t] = ex2;
  }
  __syncthreads();
  for (int idx = t; idx < TS * TS; idx += 256) {
    const int r = idx / TS, k = idx % TS;      // image row r, image column (K index) k
    const float2 v = IS_A ? T[r * TS + k] : T[k * TS + r];
    float yh = ldexpf(v.x, -E[r]), yl = ldexpf(v.y, -E[r]);
#pragma unroll
    for (int i = 0; i < NSL; ++i) {
      const float th = yh * 128.f, tl = yl * 128.f;   // exact (power of two)
      const float q = truncf(th);
      const float d = th - q;                           // exact
      const float s = d + tl;                           // renormalised remainder
      const float bb = s - d;
      yl = (d - (s - bb)) + (tl - bb);
      yh = s;
      // |q| <= 128 has at most 8 significant bits: its bf16 pattern is the
      // float's upper half, exactly
      *reinterpret_cast<unsigned short*>(S + i * IMG + img_off(r, k)) = (unsigned short)(__float_as_uint(q) >> 16);
    }
  }
  __syncthreads();
  unsigned char* dst = img + ((int64_t)e * slot_tiles + slot) * TILE_IMGS;
  for (int idx = t; idx < TILE_IMGS / 16; idx += 256)
    reinterpret_cast<uint4*>(dst)[idx] = reinterpret_cast<const uint4*>(S)[idx];
  if (t < TS) ex[((int64_t)e * slot_tiles + slot) * TS + t] = E[t];
}

__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float x) {
  const float s = hi + x;
  const float bb = s - hi;
  lo += (hi - (s - bb)) + (x - bb);
  hi = s;
}

__global__ void __launch_bounds__(MMA_THREADS, 1) k_oz_mma(dfl* env, dfl* rhs, const Prob* probs, Tables tb, int K,
                                                           const int* active, int* err, const unsigned char* img,
                                                           const int* ex, int64_t slot_tiles, int capI) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  if (K >= P.nt || (active && !active[e])) return;
  const StepShape sh = shape(P, tb, K);
  const int npair = (sh.nI + 1) >> 1;
  if (sh.nI <= 0 || sh.nC <= 0 || (int)blockIdx.x >= npair * sh.nC) return;
  const int pr = blockIdx.x / sh.nC, c = blockIdx.x % sh.nC;
  const int a0 = 2 * pr, a1 = 2 * pr + 1;
  const bool has1 = a1 < sh.nI;

  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char* base =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* SA = base;                     // slice i of the two A tiles at i * 16 KB (tile a1 at +8 KB)
  unsigned char* SB = SA + 2 * TILE_IMGS;       // slice j of the B tile at j * 8 KB
  int* EA = reinterpret_cast<int*>(SB + TILE_IMGS);
  int* EB = EA + 2 * TS;
  uint64_t* bars = reinterpret_cast<uint64_t*>(EB + TS);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 3);
  const uint32_t bar_ld = smem_u32(&bars[0]), bar_mma = smem_u32(&bars[1]), bar_c = smem_u32(&bars[2]);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned char* ia0 = img + ((int64_t)e * slot_tiles + a0) * TILE_IMGS;
  const unsigned char* ia1 = img + ((int64_t)e * slot_tiles + a1) * TILE_IMGS;
  const unsigned char* ib = img + ((int64_t)e * slot_tiles + capI + c) * TILE_IMGS;

  if (threadIdx.x == 0) {
    mbar_init(bar_ld, 1);
    mbar_init(bar_mma, 1);
    mbar_init(bar_c, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t bytes = (uint32_t)((has1 ? 2 : 1) * TILE_IMGS + TILE_IMGS);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_ld), "r"(bytes) : "memory");
    for (int i = 0; i < NSL; ++i) {
      bulk_g2s(smem_u32(SA + i * 2 * IMG), ia0 + i * IMG, IMG, bar_ld);
      if (has1) bulk_g2s(smem_u32(SA + i * 2 * IMG + IMG), ia1 + i * IMG, IMG, bar_ld);
      bulk_g2s(smem_u32(SB + i * IMG), ib + i * IMG, IMG, bar_ld);
    }
  }
  if (threadIdx.x < TS) {
    EA[threadIdx.x] = ex[((int64_t)e * slot_tiles + a0) * TS + threadIdx.x];
    EA[TS + threadIdx.x] = has1 ? ex[((int64_t)e * slot_tiles + a1) * TS + threadIdx.x] : 0;
    EB[threadIdx.x] = ex[((int64_t)e * slot_tiles + capI + c) * TS + threadIdx.x];
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  bool ok = __syncthreads_and(mbar_wait(bar_ld, 0u)) != 0;
  if (ok && threadIdx.x == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // order s = i + j (2..SMAX) accumulates in TMEM columns (s - 2) * 64
    for (int s = 2; s <= SMAX; ++s) {
      bool first = true;
      for (int i = 1; i <= NSL; ++i) {
        const int j = s - i;
        if (j < 1 || j > NSL) continue;
        const uint32_t a = smem_u32(SA + (i - 1) * 2 * IMG), b = smem_u32(SB + (j - 1) * IMG);
#pragma unroll
        for (int kk = 0; kk < TS / 16; ++kk) {
          mma_bf16(tmem + (uint32_t)((s - 2) * TS), sdesc(a + kk * 256), sdesc(b + kk * 256), first ? 0u : 1u);
          first = false;
        }
      }
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar_mma)
                 : "memory");
  }
  if (ok) ok = __syncthreads_and(mbar_wait(bar_mma, 0u)) != 0;
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  // Epilogue.  The operand images are no longer read: their shared memory
  // receives the C tiles (bulk copies issued at once, in flight while the
  // products are formed) and the 128 x 64 double-float products, written row
  // per thread from the TMEM lanes; then C -= products with coalesced 16-byte
  // stores.
  constexpr int SXS = TS + 1;  // staging stride in float2 (odd: conflict-free row writes)
  float2* Sx = reinterpret_cast<float2*>(base);
  float4* Cs = reinterpret_cast<float4*>(base + 80 * 1024);  // two C tiles, 32 KB each
  const int ntile = has1 ? 2 : 1;
  auto c_tile = [&](int h) -> dfl* {
    const int I = K + 1 + (h == 0 ? a0 : a1);
    return c < sh.nJ ? tile_ptr(env, P, tb, I, K + 1 + c) : rhs_ptr(rhs, P, I, c - sh.nJ);
  };
  const bool c_armed = ok;
  if (ok && threadIdx.x == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_c),
                 "r"((uint32_t)(ntile * TS2 * 8))
                 : "memory");
    for (int h = 0; h < ntile; ++h) bulk_g2s(smem_u32(Cs + h * (TS2 / 2)), c_tile(h), TS2 * 8, bar_c);
  }
  if (ok) {
    // thread (warp, lane): accumulator row r = 32 warp + lane
    const int r = 32 * warp + lane;
    const int er = EA[r];
    for (int q0 = 0; q0 < TS; q0 += 16) {
      uint32_t v[SMAX - 1][16];
#pragma unroll
      for (int s = 2; s <= SMAX; ++s)
        tmem_ld16_nowait(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)((s - 2) * TS + q0), v[s - 2]);
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        // sum of the orders in units of 2^(-7 SMAX), smallest first: each order
        // scaled by 2^(7 (SMAX - s)) (exact), then one scaling to the row and
        // column exponents
        float hi = 0.f, lo = 0.f;
#pragma unroll
        for (int s = SMAX; s >= 2; --s)
          two_sum_acc(hi, lo, __uint_as_float(v[s - 2][q]) * __int_as_float((127 + 7 * (SMAX - s)) << 23));
        const int sc = er + EB[q0 + q] - 7 * SMAX;
        Sx[r * SXS + q0 + q] = make_float2(ldexpf(hi, sc), ldexpf(lo, sc));
      }
    }
  }
  if (ok) ok = __syncthreads_and(mbar_wait(bar_c, 0u)) != 0;
  if (ok) {
    for (int idx = threadIdx.x; idx < ntile * TS2 / 2; idx += MMA_THREADS) {
      const int h = idx / (TS2 / 2), w2 = idx % (TS2 / 2);
      const int row = w2 / (TS / 2), col = (w2 % (TS / 2)) * 2;
      const float4 x = Cs[idx];
      const float2 p0 = Sx[(64 * h + row) * SXS + col], p1 = Sx[(64 * h + row) * SXS + col + 1];
      float2 o[2];
      const float xh[2] = {x.x, x.z}, xl[2] = {x.y, x.w}, ph[2] = {p0.x, p1.x}, pl[2] = {p0.y, p1.y};
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        // (xh + xl) - (ph + pl) in double-float
        const float s1 = xh[u] - ph[u];
        const float bb = s1 - xh[u];
        const float err1 = (xh[u] - (s1 - bb)) + (-ph[u] - bb);
        const float l = err1 + (xl[u] - pl[u]);
        const float sh2 = s1 + l;
        o[u] = make_float2(sh2, l - (sh2 - s1));
      }
      reinterpret_cast<float4*>(c_tile(h))[w2] = make_float4(o[0].x, o[0].y, o[1].x, o[1].y);
    }
  } else if (threadIdx.x == 0) {
    atomicExch(&err[e], (int)FDMGPU_ERR_CUDA);
    // the copies this CTA started must land before its shared memory is reused
    mbar_wait(bar_ld, 0u);
    if (c_armed) mbar_wait(bar_c, 0u);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
}

}  // namespace oz

void setup_oz_kernels() {
  cudaFuncSetAttribute(oz::k_oz_slice<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, oz::SMEM_SLICE);
  cudaFuncSetAttribute(oz::k_oz_slice<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, oz::SMEM_SLICE);
  cudaFuncSetAttribute(oz::k_oz_mma, cudaFuncAttributeMaxDynamicSharedMemorySize, oz::SMEM_MMA);
}

int64_t oz_tile_bytes() { return oz::TILE_IMGS; }

int launch_oz_update(const StepPlan& sp, dfl* env, dfl* rhs, const Prob* probs, Tables tb, int nprob, int K,
                     const int* active, int* err, cudaStream_t s) {
  const int nI = sp.oz_nI[K], nC = sp.oz_nC[K], items = sp.oz_items[K];
  if (items <= 0) return 0;
  const int64_t slot = sp.oz_capI + sp.oz_capC;
  oz::k_oz_slice<true><<<dim3(nI, nprob), 256, oz::SMEM_SLICE, s>>>(env, rhs, probs, tb, K, active, sp.oz_img,
                                                                     sp.oz_exp, slot, sp.oz_capI);
  oz::k_oz_slice<false><<<dim3(nC, nprob), 256, oz::SMEM_SLICE, s>>>(env, rhs, probs, tb, K, active, sp.oz_img,
                                                                      sp.oz_exp, slot, sp.oz_capI);
  oz::k_oz_mma<<<dim3(items, nprob), oz::MMA_THREADS, oz::SMEM_MMA, s>>>(env, rhs, probs, tb, K, active, err,
                                                                         sp.oz_img, sp.oz_exp, slot, sp.oz_capI);
  return 3;
}

}  // namespace fdm
