// tc_update.cu - the FP32 tile updates of the mixed precision path on the
// 5th-generation tensor cores (tcgen05.mma, kind::tf32), split-TF32.
//
// The elimination of the reference (source/mat_solve_gaussian.f90:231-262:
// row_ii -= a_ij * L_j over the profile) is, in the reversed tile order of this
// library, the right-looking update C(I,J) -= L(I,K) U(K,J) of every tile pair
// inside the band at panel step K, with the right-hand-side tiles riding along
// (Y(I,R) -= L(I,K) Y(K,R), the fused forward substitution).  The refinement
// solves apply the same tile product: Y(I,R) -= L(I,K) Y(K,R) (forward) and
// Y(I,R) -= U(I,K) Y(K,R) (backward).  These are the dense GEMMs of the band.
//
// Precision.  TF32 keeps 10 mantissa bits, far too few for these matrices
// (equilibrated condition numbers 1e6..4e7), so every FP32 operand x is split
// as x = hi + lo with hi = rna_tf32(x) and lo = rna_tf32(x - hi), and a
// product is formed as A_lo B_hi + A_hi B_lo + A_hi B_hi (three MMAs, FP32
// accumulation in tensor memory).  The dropped lo*lo term and the rounding of
// lo are ~2^-22 relative: the products are as accurate as FP32 products.
//
// One CTA (128 threads, two per SM) computes a 128 x (64 nc) block of C: two
// tile rows (I, I') times nc <= 4 tile columns, K = 64 in two halves of 32.
// Per half, the 128 threads read the FP32 tiles from global memory, split them
// and write the hi and lo parts into shared memory in the K-major, no-swizzle
// operand layout of tcgen05 (8-row x 16-byte core matrices, 128 contiguous
// bytes each); one thread issues 4 k-steps x 3 MMAs (M = 128, N = 64 nc,
// K = 8) into a TMEM accumulator of 256 columns and commits them to an
// mbarrier.  The epilogue reads the accumulator with tcgen05.ld (one TMEM lane
// = one row per thread) and writes C - acc over the C tiles.
#include <cstdint>

#include "fdm_internal.cuh"
#include "fdm_kernels.h"

namespace fdm {
namespace tc {

constexpr int THREADS = 128;
constexpr int NG = 4;                        // tile columns per CTA (N <= 256)
constexpr int KH = 32;                       // K staged per pass
constexpr int IMG_A = 128 * KH * 4;          // one operand image of A: 16 KB
constexpr int IMG_B = NG * TS * KH * 4;      // one operand image of B: 32 KB
constexpr int SMEM_BYTES = 2 * IMG_A + 2 * IMG_B + 1024 + 64;
constexpr uint32_t TMEM_COLS = 256;
constexpr long long WAIT_LIMIT = 1ll << 20;  // mbarrier polls before a CTA gives up

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor of tcgen05: start address, leading byte
// offset (between core matrices adjacent in K), stride byte offset (between
// 8-row groups), version 1 at bits 46-47, no swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
         (1ull << 46);
}

// Instruction descriptor of kind::tf32: D FP32 (bits 4-5 = 1), A and B TF32
// (bits 7-9, 10-12 = 2), both K-major, N >> 3 at bits 17-22, M >> 4 at 24-28.
__device__ __forceinline__ uint32_t idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ uint32_t rna_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}
// x = hi + lo, both TF32 values (their low 13 mantissa bits are zero)
__device__ __forceinline__ void split(float x, uint32_t& hi, uint32_t& lo) {
  hi = rna_tf32(x);
  lo = rna_tf32(x - __uint_as_float(hi));
}

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
// Bounded wait: false when the phase did not complete within WAIT_LIMIT polls.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (long long i = 0; i < WAIT_LIMIT; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

#define TC_LD32_OUT(r)                                                                                              \
  "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),     \
      "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),      \
      "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),     \
      "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])

// 32 consecutive accumulator columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
      "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : TC_LD32_OUT(r)
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Byte offset of element (r, k) (r: row of the operand, M or N; k < KH) in a
// K-major no-swizzle image: core matrix (r / 8, k / 4) at 128-byte slots, eight
// per 8-row group; inside it row r % 8 at 16 bytes, k % 4 at 4 bytes.
__device__ __forceinline__ uint32_t img_off(int r, int k) {
  return (uint32_t)((((r >> 3) * (KH / 4) + (k >> 2)) << 7) + ((r & 7) << 4) + ((k & 3) << 2));
}
constexpr uint32_t LBO = 128;                // next core matrix along K
constexpr uint32_t SBO = (KH / 4) * 128;     // next 8-row group

// Work of one CTA.  MODE 0: factor trailing update at step K, C(I,J) and the
// fused right-hand sides Y(I,R); MODE 1: forward solve update; MODE 2:
// backward solve update.
struct Work {
  const float* A[2];     // A tiles of the two rows (nullptr: absent row)
  const float* B[NG];    // B tiles of the nc columns
  float* C[2][NG];       // C tiles
  int nc;
};

template <int MODE>
__device__ __forceinline__ bool decode(float* env, float* rhs, const Prob& P, const Tables& tb, int K, int item,
                                       Work& w) {
  int nI, i0, nJ, nC;
  if (MODE == 0) {
    nI = tb.Imax[P.trow + K] - K;
    i0 = K + 1;
    nJ = tb.J1[P.trow + K] - K;
    nC = nJ + P.nrt;
  } else if (MODE == 1) {
    nI = tb.Imax[P.trow + K] - K;
    i0 = K + 1;
    nJ = 0;
    nC = P.nrt;
  } else {
    i0 = tb.Imin[P.trow + K];
    nI = K - i0;
    nJ = 0;
    nC = P.nrt;
  }
  const int npair = (nI + 1) >> 1, ngrp = (nC + NG - 1) / NG;
  if (nI <= 0 || nC <= 0 || item >= npair * ngrp) return false;
  const int pr = item / ngrp, g = item % ngrp;
  const int c0 = g * NG;
  w.nc = min(NG, nC - c0);
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int i = 2 * pr + h;
    if (i < nI) {
      const int I = i0 + i;
      w.A[h] = tile_ptr(env, P, tb, I, K);
#pragma unroll
      for (int c = 0; c < NG; ++c) {
        const int cc = c0 + c;
        w.C[h][c] = c >= w.nc ? nullptr : (cc < nJ ? tile_ptr(env, P, tb, I, K + 1 + cc) : rhs_ptr(rhs, P, I, cc - nJ));
      }
    } else {
      w.A[h] = nullptr;
#pragma unroll
      for (int c = 0; c < NG; ++c) w.C[h][c] = nullptr;
    }
  }
#pragma unroll
  for (int c = 0; c < NG; ++c) {
    const int cc = c0 + c;
    w.B[c] = c >= w.nc ? nullptr : (cc < nJ ? tile_ptr(env, P, tb, K, K + 1 + cc) : rhs_ptr(rhs, P, K, cc - nJ));
  }
  return true;
}

// Operands of one K half in registers: thread t holds the A chunks
// q = t + 128 i (i < 8: row r, four consecutive k) and the B units
// q = t + 128 j (j < 16: column n, four consecutive k), read from global
// memory before any of them is written to shared memory, so that all the
// loads of a half are in flight together.
struct Regs {
  float4 a[8];
  float b[16][4];
};

__device__ __forceinline__ void load_half(const Work& w, int kh, Regs& R) {
  const int t = threadIdx.x;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int q = t + THREADS * i;
    const int kq = (q >> 3) & 7, r = ((q >> 6) << 3) | (q & 7);
    const float* a = w.A[r >> 6];
    R.a[i] = a ? __ldg(reinterpret_cast<const float4*>(a + (r & 63) * TS + kh * KH + 4 * kq))
               : make_float4(0.f, 0.f, 0.f, 0.f);
  }
  const int nn = w.nc * TS;
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    const int q = t + THREADS * j;
    if (q < nn * (KH / 4)) {
      const int n = q % nn, kq = q / nn;
      const float* b = w.B[n >> 6] + (kh * KH + 4 * kq) * TS + (n & 63);
      R.b[j][0] = __ldg(b);
      R.b[j][1] = __ldg(b + TS);
      R.b[j][2] = __ldg(b + 2 * TS);
      R.b[j][3] = __ldg(b + 3 * TS);
    }
  }
}

// Split the registers into hi and lo TF32 parts and write the K-major images.
// A: lanes 0-7 of a quarter warp fill one 128-byte core matrix; B: one thread
// writes one 16-byte core-matrix row (4 consecutive k of column n), lanes with
// consecutive n hit distinct bank groups.
__device__ __forceinline__ void store_half(const Work& w, const Regs& R, unsigned char* sAhi, unsigned char* sAlo,
                                           unsigned char* sBhi, unsigned char* sBlo) {
  const int t = threadIdx.x;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int q = t + THREADS * i;
    const int kq = (q >> 3) & 7, r = ((q >> 6) << 3) | (q & 7);
    uint4 hi, lo;
    split(R.a[i].x, hi.x, lo.x);
    split(R.a[i].y, hi.y, lo.y);
    split(R.a[i].z, hi.z, lo.z);
    split(R.a[i].w, hi.w, lo.w);
    const uint32_t off = img_off(r, 4 * kq);
    *reinterpret_cast<uint4*>(sAhi + off) = hi;
    *reinterpret_cast<uint4*>(sAlo + off) = lo;
  }
  const int nn = w.nc * TS;
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    const int q = t + THREADS * j;
    if (q < nn * (KH / 4)) {
      const int n = q % nn, kq = q / nn;
      uint4 hi, lo;
      split(R.b[j][0], hi.x, lo.x);
      split(R.b[j][1], hi.y, lo.y);
      split(R.b[j][2], hi.z, lo.z);
      split(R.b[j][3], hi.w, lo.w);
      const uint32_t off = img_off(n, 4 * kq);
      *reinterpret_cast<uint4*>(sBhi + off) = hi;
      *reinterpret_cast<uint4*>(sBlo + off) = lo;
    }
  }
}

// One thread issues the 4 k-steps x 3 products of a half and commits them.
__device__ __forceinline__ void issue_half(uint32_t tmem, uint32_t idesc, int kh, const unsigned char* sAhi,
                                           const unsigned char* sAlo, const unsigned char* sBhi,
                                           const unsigned char* sBlo, uint32_t bar) {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t ahi = smem_u32(sAhi), alo = smem_u32(sAlo), bhi = smem_u32(sBhi), blo = smem_u32(sBlo);
#pragma unroll
  for (int s = 0; s < KH / 8; ++s) {
    const uint32_t ko = s * 2 * 128;  // 8 TF32 = two core matrices along K
    mma_tf32(tmem, sdesc(alo + ko, LBO, SBO), sdesc(bhi + ko, LBO, SBO), idesc, (kh | s) ? 1u : 0u);
    mma_tf32(tmem, sdesc(ahi + ko, LBO, SBO), sdesc(blo + ko, LBO, SBO), idesc, 1u);
    mma_tf32(tmem, sdesc(ahi + ko, LBO, SBO), sdesc(bhi + ko, LBO, SBO), idesc, 1u);
  }
  mma_commit(bar);
}

template <int MODE>
__global__ void __launch_bounds__(THREADS, 2) k_tc_update(float* env, float* rhs, const Prob* probs, Tables tb,
                                                          int K, const int* active, int* err) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  if (K >= P.nt || (active && !active[e])) return;
  if (MODE == 0 && tb.wide && tb.wide[P.trow + K]) return;  // the double-float instantiation takes this step
  Work w;
  if (!decode<MODE>(env, rhs, P, tb, K, blockIdx.x, w)) return;

  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* sAhi = base;
  unsigned char* sAlo = sAhi + IMG_A;
  unsigned char* sBhi = sAlo + IMG_A;
  unsigned char* sBlo = sBhi + IMG_B;
  uint64_t* bar = reinterpret_cast<uint64_t*>(sBlo + IMG_B);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar + 1);
  const uint32_t bar_a = smem_u32(bar);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  Regs R;
  load_half(w, 0, R);  // in flight while the barrier and TMEM are set up
  if (threadIdx.x == 0) {
    mbar_init(bar_a, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
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
  const uint32_t idesc = idesc_tf32(128, TS * w.nc);

  // half 0: images, MMAs; half 1's loads are in flight while they run
  store_half(w, R, sAhi, sAlo, sBhi, sBlo);
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // generic-proxy writes -> tensor core
  __syncthreads();
  if (threadIdx.x == 0) issue_half(tmem, idesc, 0, sAhi, sAlo, sBhi, sBlo, bar_a);
  load_half(w, 1, R);
  // the images are overwritten only once the half-0 MMAs have read them (a
  // uniform decision: every thread sees the same outcome)
  bool ok = __syncthreads_and(mbar_wait(bar_a, 0u)) != 0;
  if (ok) {
    store_half(w, R, sAhi, sAlo, sBhi, sBlo);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0) issue_half(tmem, idesc, 1, sAhi, sAlo, sBhi, sBlo, bar_a);
  }
  // epilogue: thread (warp, lane) owns accumulator row r = 32 warp + lane,
  // row r % 64 of tile row r / 64; the first C tile is read while the last
  // MMAs run
  const int r = 32 * warp + lane;
  const int h = r >> 6, row = r & 63;
  float4 c4[16];
  {
    float* cp = w.C[h][0];
    if (cp) {
#pragma unroll
      for (int j = 0; j < 16; ++j) c4[j] = __ldcs(reinterpret_cast<const float4*>(cp + row * TS) + j);
    }
  }
  if (ok) ok = __syncthreads_and(mbar_wait(bar_a, 1u)) != 0;
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok) {
    for (int c = 0; c < w.nc; ++c) {
      uint32_t v[64];
      tmem_ld32(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(c * TS), v);
      tmem_ld32(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(c * TS + 32), v + 32);
      float* cp = w.C[h][c];
      if (cp) {
        float4* q = reinterpret_cast<float4*>(cp + row * TS);
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          float4 x = c4[j];
          x.x -= __uint_as_float(v[4 * j + 0]);
          x.y -= __uint_as_float(v[4 * j + 1]);
          x.z -= __uint_as_float(v[4 * j + 2]);
          x.w -= __uint_as_float(v[4 * j + 3]);
          __stcs(q + j, x);
        }
      }
      // next C tile of this row
      if (c + 1 < w.nc) {
        float* cn = w.C[h][c + 1];
        if (cn) {
#pragma unroll
          for (int j = 0; j < 16; ++j) c4[j] = __ldcs(reinterpret_cast<const float4*>(cn + row * TS) + j);
        }
      }
    }
  } else if (threadIdx.x == 0) {
    atomicExch(&err[e], (int)FDMGPU_ERR_CUDA);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
}

}  // namespace tc

void setup_tc_kernels() {
  cudaFuncSetAttribute(tc::k_tc_update<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::SMEM_BYTES);
  cudaFuncSetAttribute(tc::k_tc_update<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::SMEM_BYTES);
  cudaFuncSetAttribute(tc::k_tc_update<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::SMEM_BYTES);
}

void launch_tc_update(int mode, int items, int nprob, float* env, float* rhs, const Prob* probs, Tables tb, int K,
                      const int* active, int* err, cudaStream_t s) {
  if (items <= 0) return;
  const dim3 grid(items, nprob);
  if (mode == 0)
    tc::k_tc_update<0><<<grid, tc::THREADS, tc::SMEM_BYTES, s>>>(env, rhs, probs, tb, K, active, err);
  else if (mode == 1)
    tc::k_tc_update<1><<<grid, tc::THREADS, tc::SMEM_BYTES, s>>>(env, rhs, probs, tb, K, active, err);
  else
    tc::k_tc_update<2><<<grid, tc::THREADS, tc::SMEM_BYTES, s>>>(env, rhs, probs, tb, K, active, err);
}

int tc_items(int nI, int nC) { return nI <= 0 || nC <= 0 ? 0 : ((nI + 1) / 2) * ((nC + tc::NG - 1) / tc::NG); }

}  // namespace fdm
