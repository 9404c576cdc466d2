// fdm_internal.cuh - shared declarations of the GB300 FDM solver.
//
// Storage model.  One FDM system of order n (one energy, one spin block) is
// held in REVERSED order: row p = n - ii and column q = n - jj, where ii/jj are
// the reference's 1-based rows and columns.  The reference eliminates rows
// bottom-up (UL, source/mat_solve_gaussian.f90:196-317); in reversed order the
// same elimination is a top-down LU without pivoting, so the profile of the
// reference (lb1 made monotone by newind, source/mat.f90:1874-1876) becomes a
// variable band whose right edge lu(p) = n - lb1(ii) never decreases.
//
// The band is stored as dense TS x TS tiles (row-major inside a tile).  Row
// block I keeps the contiguous run of tiles J0(I)..J1(I) that covers every
// row's columns [n - lb2, n - lb1]; J0 is replaced by its suffix minimum so
// that the rows touched by panel K form one range (K, Imax(K)].  Right-hand
// sides are TS x TS tiles too: tile (I, R) holds rows I*TS.. and RHS columns
// R*TS.. of one system.  Rows n..npad-1 are identity padding.
#pragma once

#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>

#include "../../include/fdmgpu.h"
#include "dfloat.cuh"

namespace fdm {

constexpr int TS = 64;            // tile edge
constexpr int TS2 = TS * TS;
constexpr int NTHREADS = 256;     // threads of every tile kernel

// Per-problem descriptor (device and host copy).
struct Prob {
  int n;          // order (nligne)
  int nt;         // tiles per edge (ceil(n / TS))
  int nlmso;      // right-hand sides
  int nrt;        // RHS tiles (ceil(nlmso / TS))
  int nligneso;   // rows before the outer-sphere rows
  int lmaxso;
  int nlmagm;
  int ispin;      // 1-based spin block (selects the Vr column)
  int iaabs;      // 1-based absorbing atom (Taull)
  int nlm_abs;    // harmonics of the absorber
  int ianew_abs;  // row offset of the absorber harmonics (1-based rows ianew+1..)
  int trow;       // offset into J0 / J1 / strip arrays (per tile row)
  int site;       // index of the problem's grid (absorbing site) in the batch's site table
  double enervide;
  int64_t env;    // element offset of the band tiles
  int64_t rhs;    // element offset of the RHS tiles (nt * nrt * TS2)
  int64_t rowv;   // offset into per-row vectors (npad entries): scales, csr row_ptr
  int64_t csr;    // offset into CSR columns/values
  int64_t csr_cap;    // CSR capacity of this problem (structural nonzeros of calcMatRow)
  int64_t csr_col;    // offset of this problem's per-column refinement state
  int64_t in_new;     // offset of new_(0:npoint) in the int pool
  int64_t in_ianew;   // offset of ianew(natome)
  int64_t in_nlmsa;   // offset of nlmsa(natome)
  int64_t in_vr;      // offset of Vr(npoint) (the selected spin) in the double pool
  int64_t in_phi;     // offset of phiato(nphiato1, nlmagm, natome) (spin-selected)
  int64_t in_bes;     // offset of Bessel j(ib, L) in the double pool, [nsort][lmaxso+1]
  int64_t in_neu;     // offset of Neumann n(ib, L), [nsort][lmaxso+1]
  int64_t taull;      // offset of Taull (complex) for this problem
  int64_t scratch;    // offset of the complex nlmso x (nlmso + nlm_abs) Taull scratch
  // complex (Cal_comp) problems, stored as the real-equivalent system: complex
  // row ii (1-based) becomes rows 2ii-1 (real part) and 2ii (imaginary part)
  // of an order-2n real system, each complex entry a the 2x2 block
  // [Re a, -Im a; Im a, Re a]; n above is then 2 nligne.
  int cplx;           // 0 real, 1 complex
  int nligne_c;       // complex order (nligne)
  int so, rel, ylmc;  // Spinorbite, Relativiste, Ylm_comp
  int nspinp, nspinr, nspin;
  int64_t in_grad;    // offset of gradvr(npoint, 3, nspin) in the double pool
  // inputs generated on the device (radial.cu) instead of uploaded: phiato,
  // Bessel and Neumann of the real path, from the site's radial tables
  int gen;
  int gen_lmax[8];    // l cut-off per atom type at this energy
  // complex energy (E_comp, regular solution): -i Eimag on the grid
  // diagonal, complex Bessel / Neumann stored as real blocks then imaginary
  // blocks, each [nspinr][nsort][lmaxso+1]
  int ecomp;
  double eimag;
  // FDM_comp: irr = 1 for the irregular cluster solution (2 nlmsa amplitude
  // rows per atom, no outer-sphere rows); nri = atomic solutions packed per
  // harmonic in the phiato block (1, or 2 with irr)
  int irr, nri;
};
constexpr int MAX_GEN_TYPES = 8;

// Energy-independent radial tables of a site for the generated inputs
// (device pointers; per atom type t the mesh and coefficients at t * nr_max).
struct RadialDev {
  int ntype, nr_max, nspin;
  const int* nr;           // (ntype) mesh points
  const double* r;         // (nr_max, ntype) radial mesh (bohr)
  const double* mcl0;      // -clapl0 of the three-point Laplacian on the mesh
  const double* gm;        // -claplm
  const double* gp;        // -claplp
  const double* f2;        // 1 / r^2
  const double* V;         // spherical potential of the type (Ry), spin-independent part
  const double* dv_spin;   // (nspin) spin shift of the potential (Ry)
  const double* z_origin;  // (ntype) charge of the expansion at the origin
  const int* itype;        // (natome) type of each atom, 0-based
  const double* rrel;      // (nbtm, natome) distance of each boundary point to its atom
  const int* iidx;         // (nbtm, natome) first mesh index with r > rrel (clipped to [2, nr-1])
  const double* rsort;     // (nsort) radius of each outer point (bohr)
  double v0bd;             // interstitial level subtracted from the energy for the kinetic energy
};

// Per tile-row / tile-column tables of a problem, at Prob::trow.
struct Tables {
  const int* J0;      // first stored tile of row block I (suffix-min hull)
  const int* J1;      // last stored tile of row block I
  const int64_t* strip;  // tile offset of row block I's strip
  const int* Imax;    // last row block with a stored tile in column K
  const int* Imin;    // first row block whose strip reaches column K
  const unsigned char* wide;  // per tile row: the FP32 factor accumulates step K's trailing
                              // update in double-float (nullptr: never)
};

template <typename T>
__device__ __forceinline__ T* tile_ptr(T* env, const Prob& P, const Tables& tb, int I, int J) {
  return env + P.env + (tb.strip[P.trow + I] + (J - tb.J0[P.trow + I])) * (int64_t)TS2;
}
template <typename T>
__device__ __forceinline__ T* rhs_ptr(T* rhs, const Prob& P, int I, int R) {
  return rhs + P.rhs + ((int64_t)I * P.nrt + R) * (int64_t)TS2;
}

// Static structure on the device (energy independent).
struct StaticDev {
  int npoint, npsom, nvois, natome, nbtm, nbm, nsort, nsortf, nlmmax, nlmomax, nlmsam, nso1;
  int npr;                 // interstitial points
  const int* inter_pt;     // (npr) interstitial point indices, 1-based
  const int* nb_kind;      // (npr, nvois): 0 interstitial, ia>0 atom, -2 outer
  const int* nb_idx;       // (npr, nvois): neighbour point j (1-based) or boundary index ib (1-based)
  const double* nb_coef;   // (npr, nvois): (Kar * -clapl(iv)) * rvol(i) [* Kar(isbord)]
  const double* rvol;      // (npoint)
  const double* clapl;     // (0:nvois)
  const int* numia;
  const int* nbord;
  const int* nbordf;
  const int* ibord;        // (nbtm, natome)
  const int* isrt;         // (nsort)
  const double* poidsa;    // (nbm, natome)
  const double* poidso;    // (nsortf)
  const double* Kar;       // (64)
  const int* isbord;       // (nbtm, natome)
  const double* YsoT;      // (nsort, nlmomax) row-major: YsoT[ib * nlmomax + lm]
  const double* Ylmato;    // (nbtm, nlmmax, natome) Fortran
  const int* lato;         // (nlmsam, natome) for igrph = 1
  const int* mato;
  const int* lso;          // (nso1)
  const int* mso;
  const int* iato;         // (nlmsam, natome) spin of each atom harmonic (spin-orbit)
  const int* iso;          // (nso1) spin of each outer harmonic
  const double* cgrad;     // (nvois) gradient coefficients
  int nspino, nspin;
};

// -------------------------------------------------------------------------
// Tile routines (256 threads, TS = 64).  Shared tiles are row-major with a
// padded stride.
// -------------------------------------------------------------------------
constexpr int SP = TS + 4;  // shared stride (keeps 16-byte alignment for float4/double2)

template <typename T>
__device__ __forceinline__ void load_tile(T* __restrict__ s, const T* __restrict__ g) {
  for (int idx = threadIdx.x; idx < TS2; idx += NTHREADS) {
    const int r = idx / TS, c = idx % TS;
    s[r * SP + c] = g[idx];
  }
}
template <typename T>
__device__ __forceinline__ void load_tile_n(T* __restrict__ s, const T* __restrict__ g, int nthreads) {
  for (int idx = threadIdx.x; idx < TS2; idx += nthreads) s[(idx / TS) * SP + idx % TS] = g[idx];
}
template <typename T>
__device__ __forceinline__ void store_tile(T* __restrict__ g, const T* __restrict__ s) {
  for (int idx = threadIdx.x; idx < TS2; idx += NTHREADS) {
    const int r = idx / TS, c = idx % TS;
    g[idx] = s[r * SP + c];
  }
}

// In-place LU of the shared tile D (Doolittle: unit L below, U on and above
// the diagonal).  With perm != nullptr, partial pivoting among the rows of the
// tile: perm[r] is the original tile row now at row r (perm must hold the
// identity on entry).  Records the smallest |pivot| in *minpiv.
template <typename T>
__device__ void tile_lu(T* D, double* minpiv, int* perm) {
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  __shared__ int prow;
  double mp = 1e300;
  for (int k = 0; k < TS; ++k) {
    if (perm) {
      if (threadIdx.x < 32) {
        const int i1 = k + threadIdx.x, i2 = k + threadIdx.x + 32;
        double v = i1 < TS ? fabs((double)D[i1 * SP + k]) : -1.0;
        int bi = i1;
        if (i2 < TS) {
          const double v2 = fabs((double)D[i2 * SP + k]);
          if (v2 > v) { v = v2; bi = i2; }
        }
        for (int o = 16; o; o >>= 1) {
          const double ov = __shfl_xor_sync(0xffffffffu, v, o);
          const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
          if (ov > v || (ov == v && oi < bi)) { v = ov; bi = oi; }
        }
        if (threadIdx.x == 0) prow = bi;
      }
      __syncthreads();
      const int pr = prow;
      if (pr != k) {
        if (threadIdx.x < TS) {
          const T t = D[k * SP + threadIdx.x];
          D[k * SP + threadIdx.x] = D[pr * SP + threadIdx.x];
          D[pr * SP + threadIdx.x] = t;
        }
        if (threadIdx.x == 0) {
          const int t = perm[k];
          perm[k] = perm[pr];
          perm[pr] = t;
        }
      }
      __syncthreads();
    }
    const T piv = D[k * SP + k];
    if (threadIdx.x == 0) mp = fmin(mp, fabs((double)piv));
    if (threadIdx.x > k && threadIdx.x < TS) D[threadIdx.x * SP + k] = D[threadIdx.x * SP + k] / piv;
    __syncthreads();
    for (int i = k + 1 + ty; i < TS; i += 16) {
      const T l = D[i * SP + k];
      for (int j = k + 1 + tx; j < TS; j += 16) D[i * SP + j] -= l * D[k * SP + j];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *minpiv = mp;
}

// Shared tile <- global tile with its rows permuted: s[r] = g[perm[r]].
template <typename T>
__device__ __forceinline__ void load_tile_perm(T* __restrict__ s, const T* __restrict__ g, const int* perm) {
  for (int idx = threadIdx.x; idx < TS2; idx += NTHREADS) {
    const int r = idx / TS, c = idx % TS;
    s[r * SP + c] = g[perm[r] * TS + c];
  }
}

// W <- W * inv(U), U = upper triangle (with diagonal) of D.
template <typename T>
__device__ void tile_right_upper_solve(T* W, const T* D) {
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  for (int k = 0; k < TS; ++k) {
    if (threadIdx.x < TS) W[threadIdx.x * SP + k] = W[threadIdx.x * SP + k] / D[k * SP + k];
    __syncthreads();
    for (int i = ty; i < TS; i += 16) {
      const T x = W[i * SP + k];
      for (int j = k + 1 + tx; j < TS; j += 16) W[i * SP + j] -= x * D[k * SP + j];
    }
    __syncthreads();
  }
}

// W <- inv(L) * W, L = unit lower triangle of D.
template <typename T>
__device__ void tile_left_lower_unit_solve(T* W, const T* D) {
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  for (int k = 0; k < TS - 1; ++k) {
    for (int i = k + 1 + ty; i < TS; i += 16) {
      const T l = D[i * SP + k];
      for (int j = tx; j < TS; j += 16) W[i * SP + j] -= l * W[k * SP + j];
    }
    __syncthreads();
  }
}

// W <- inv(U) * W, U = upper triangle (with diagonal) of D.
template <typename T>
__device__ void tile_left_upper_solve(T* W, const T* D) {
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  for (int k = TS - 1; k >= 0; --k) {
    if (threadIdx.x < TS) W[k * SP + threadIdx.x] = W[k * SP + threadIdx.x] / D[k * SP + k];
    __syncthreads();
    for (int i = ty; i < k; i += 16) {
      const T u = D[i * SP + k];
      for (int j = tx; j < TS; j += 16) W[i * SP + j] -= u * W[k * SP + j];
    }
    __syncthreads();
  }
}

// C(global, row-major TS x TS) -= A(global) * B(global), all TS x TS tiles.
// Shared use: As (TS x SP, A transposed) + Bs (TS x SP).
template <typename T>
__device__ void tile_gemm_sub(T* __restrict__ C, const T* __restrict__ A, const T* __restrict__ B, T* As, T* Bs) {
  // stage A transposed: As[k * SP + r] = A[r * TS + k]
  for (int idx = threadIdx.x; idx < TS2; idx += NTHREADS) {
    const int r = idx / TS, k = idx % TS;
    As[k * SP + r] = A[idx];
    Bs[r * SP + k] = B[idx];
  }
  __syncthreads();
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  T acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
#pragma unroll 4
  for (int k = 0; k < TS; ++k) {
    T a[4], b[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) a[i] = As[k * SP + ty * 4 + i];
#pragma unroll
    for (int j = 0; j < 4; ++j) b[j] = Bs[k * SP + tx * 4 + j];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] += a[i] * b[j];
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    T* crow = C + (ty * 4 + i) * TS + tx * 4;
#pragma unroll
    for (int j = 0; j < 4; ++j) crow[j] -= acc[i][j];
  }
}

// C = A * P B (C, A, B global TS x TS tiles; P the row order perm, nullable).
// C may alias A or B: both are staged in shared memory first.
template <typename T>
__device__ void tile_gemm_assign(T* C, const T* A, const T* B, const int* perm, T* As, T* Bs) {
  for (int idx = threadIdx.x; idx < TS2; idx += NTHREADS) {
    const int r = idx / TS, k = idx % TS;
    As[k * SP + r] = A[idx];
    Bs[r * SP + k] = perm ? B[perm[r] * TS + k] : B[idx];
  }
  __syncthreads();
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  T acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
#pragma unroll 4
  for (int k = 0; k < TS; ++k) {
    T a[4], b[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) a[i] = As[k * SP + ty * 4 + i];
#pragma unroll
    for (int j = 0; j < 4; ++j) b[j] = Bs[k * SP + tx * 4 + j];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] += a[i] * b[j];
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    T* crow = C + (ty * 4 + i) * TS + tx * 4;
#pragma unroll
    for (int j = 0; j < 4; ++j) crow[j] = acc[i][j];
  }
}

// -------------------------------------------------------------------------
// 64-thread tile product: C (-)= A * P B with every operand a TS x TS tile.
// Thread (tx, ty) of the 8 x 8 thread grid owns rows {4ty + i, 32 + 4ty + i}
// and columns {4tx + j, 32 + 4tx + j} (i, j < 4): an 8 x 8 register tile, fed
// per k by eight scalar reads of A (row-major, odd stride: no bank conflicts)
// and two 16-byte reads of B.  Shared use: As, Bs of TS x SP each.
// -------------------------------------------------------------------------
constexpr int GEMM_THREADS = 64;

template <typename T> struct Vec4;
template <> struct Vec4<float> { typedef float4 type; };

template <typename T>
__device__ __forceinline__ void ld4(const T* p, T* v) {
  v[0] = p[0]; v[1] = p[1]; v[2] = p[2]; v[3] = p[3];
}
template <>
__device__ __forceinline__ void ld4<float>(const float* p, float* v) {
  const float4 q = *reinterpret_cast<const float4*>(p);
  v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
}
template <>
__device__ __forceinline__ void ld4<dfl>(const dfl* p, dfl* v) {
  const float4 a = *reinterpret_cast<const float4*>(p);
  const float4 b = *reinterpret_cast<const float4*>(p + 2);
  v[0] = dfl(a.x, a.y); v[1] = dfl(a.z, a.w); v[2] = dfl(b.x, b.y); v[3] = dfl(b.z, b.w);
}
template <>
__device__ __forceinline__ void ld4<double>(const double* p, double* v) {
  const double2 a = *reinterpret_cast<const double2*>(p);
  const double2 b = *reinterpret_cast<const double2*>(p + 2);
  v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}

constexpr int SPA = TS + 1;  // odd stride: conflict-free reads of a row per thread

// acc += a * b inside a dot product.  For double-float the accumulator is
// kept unnormalised: the high parts are summed with Knuth's two-sum, the
// rounding errors and the cross terms collect in lo, and mac_finish
// renormalises once per dot product (about 12 FP32 operations per step
// instead of 18 for a renormalised multiply and add).
template <typename T>
__device__ __forceinline__ void mac(T& acc, T a, T b) { acc += a * b; }
template <>
__device__ __forceinline__ void mac<dfl>(dfl& acc, dfl a, dfl b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
  const float s = acc.hi + p;
  const float bb = s - acc.hi;
  const float err = (acc.hi - (s - bb)) + (p - bb);
  acc.hi = s;
  acc.lo += err + e;
}
template <typename T>
__device__ __forceinline__ T mac_finish(T acc) { return acc; }
template <>
__device__ __forceinline__ dfl mac_finish<dfl>(dfl acc) { return df_fast_two_sum(acc.hi, acc.lo); }

// Wide accumulation of FP32 products: the exact product (p + e, e by FMA) is
// added to an unnormalised double-float sum with Knuth's two-sum (about 8
// FP32 operations per multiply-add).  Used by the FP32 factor at the steps
// whose multipliers are large (the atom-harmonic tiles), where FP32 sums
// next to them lose the factor's accuracy.
struct facc {
  float hi, lo;
};
template <typename A>
__device__ __forceinline__ A acc_zero() { return A(0); }
template <>
__device__ __forceinline__ facc acc_zero<facc>() { return facc{0.0f, 0.0f}; }
__device__ __forceinline__ void mac(facc& acc, float a, float b) {
  const float p = a * b;
  const float e = fmaf(a, b, -p);
  const float s = acc.hi + p;
  const float bb = s - acc.hi;
  const float err = (acc.hi - (s - bb)) + (p - bb);
  acc.hi = s;
  acc.lo += err + e;
}
// c - acc (sub) or acc, rounded once more to the storage type.
template <typename T, typename A>
__device__ __forceinline__ T acc_apply(T c, A acc, bool sub) {
  const T v = mac_finish(acc);
  return sub ? c - v : v;
}
template <>
__device__ __forceinline__ float acc_apply<float, facc>(float c, facc a, bool sub) {
  if (!sub) return a.hi + a.lo;
  const float s = c - a.hi;            // two-sum of c and -hi
  const float t = s - c;
  const float err = (c - (s - t)) + (-a.hi - t);
  return s + (err - a.lo);
}

// Threads of the tile-product kernels: 64 threads with 8 x 8 accumulators per
// thread (FP64), or 128 threads with 8 x 4 (FP32 and double-float: twice the
// warps per tile for the same registers, which hides the latency of the
// staging loads and of the dependent double-float operations).
template <typename T> struct MMThreads { static constexpr int value = GEMM_THREADS; };
template <> struct MMThreads<dfl> { static constexpr int value = 128; };
template <> struct MMThreads<float> { static constexpr int value = 128; };

template <typename T>
__device__ __forceinline__ void st4(T* p, const T* v) {
  p[0] = v[0]; p[1] = v[1]; p[2] = v[2]; p[3] = v[3];
}
template <>
__device__ __forceinline__ void st4<float>(float* p, const float* v) {
  *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
template <>
__device__ __forceinline__ void st4<double>(double* p, const double* v) {
  *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
  *reinterpret_cast<double2*>(p + 2) = make_double2(v[2], v[3]);
}
template <>
__device__ __forceinline__ void st4<dfl>(dfl* p, const dfl* v) {
  *reinterpret_cast<float4*>(p) = make_float4(v[0].hi, v[0].lo, v[1].hi, v[1].lo);
  *reinterpret_cast<float4*>(p + 2) = make_float4(v[2].hi, v[2].lo, v[3].hi, v[3].lo);
}

// TA: use the transpose of A (C (-)= A^T * P B).  Thread (tx, ty) owns rows
// {4ty + i, 32 + 4ty + i} (i < 4) and columns {4tx + j, 32 + 4tx + j} (64
// threads) or {4tx + j} (128 threads), j < 4.
template <typename T, bool SUB, bool TA = false, int NT = MMThreads<T>::value, typename Acc = T>
__device__ __forceinline__ void tile_mm64(T* C, const T* A, const T* B, const int* perm, T* As, T* Bs) {
  static_assert(NT == 64 || NT == 128, "tile_mm64 runs on 64 or 128 threads");
  constexpr int CW = NT == 128 ? 4 : 8;  // columns per thread
  const int t = threadIdx.x;
  // stage: As[r][k] = A[r][k] (A[k][r] when TA; stride SPA), Bs[r][c] = B[perm ? perm[r] : r][c] (stride SP)
  for (int idx = t; idx < TS2 / 4; idx += NT) {
    const int r = idx / (TS / 4), c4 = (idx % (TS / 4)) * 4;
    T a[4], b[4];
    ld4(A + r * TS + c4, a);
    ld4(B + (perm ? perm[r] : r) * TS + c4, b);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if (TA)
        As[(c4 + q) * SPA + r] = a[q];
      else
        As[r * SPA + c4 + q] = a[q];
      Bs[r * SP + c4 + q] = b[q];
    }
  }
  __syncthreads();
  const int tx = t % (NT / 8), ty = t / (NT / 8);
  Acc acc[8][CW];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < CW; ++j) acc[i][j] = acc_zero<Acc>();
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
  __syncthreads();  // C may alias A or B, which are no longer read
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int row = (i < 4 ? 4 * ty + i : 32 + 4 * ty + (i - 4));
#pragma unroll
    for (int h = 0; h < CW / 4; ++h) {
      T* cp = C + row * TS + 32 * h + 4 * tx;
#pragma unroll
      for (int j = 0; j < 4; ++j) cp[j] = acc_apply<T, Acc>(cp[j], acc[i][4 * h + j], SUB);
    }
  }
}

// -------------------------------------------------------------------------
// Triangular substitution by 64 independent threads (no barriers inside).
// The factored diagonal tile sits in shared memory with stride SP.
// -------------------------------------------------------------------------

// g <- L^-1 P g (L unit lower): thread c (threadIdx.x unless given) owns
// column c of the tile.  Column
// (axpy) order: once x[k] is final it is subtracted from every later row, so
// the 63 - k updates of step k are independent (instruction-level parallelism
// for the dependent double-float operations) instead of one dot-product chain.
template <typename T>
__device__ __forceinline__ void col_solve_lower_unit(T* g, const T* Ls, const int* perm, int c = -1) {
  if (c < 0) c = threadIdx.x;
  if (c >= TS) return;
  T x[TS];
#pragma unroll
  for (int r = 0; r < TS; ++r) x[r] = g[(perm ? perm[r] : r) * TS + c];
  if constexpr (std::is_same<T, double>::value) {
    // FP64 (the reference's arithmetic): dot-product order
#pragma unroll
    for (int k = 1; k < TS; ++k) {
      T acc = x[k];
#pragma unroll
      for (int i = 0; i < k; ++i) acc -= Ls[k * SP + i] * x[i];
      x[k] = acc;
    }
  } else {
#pragma unroll
    for (int k = 0; k < TS - 1; ++k) {
      const T xk = x[k];
#pragma unroll
      for (int i = k + 1; i < TS; ++i) x[i] -= Ls[i * SP + k] * xk;
    }
  }
#pragma unroll
  for (int r = 0; r < TS; ++r) g[r * TS + c] = x[r];
}

// g <- U^-1 g (U upper with diagonal): thread c owns column c.  Dot-product
// order from the last row up; for FP32 and double-float each dot product runs
// as four interleaved partial sums (independent dependency chains), combined
// before the division.
template <typename T>
__device__ __forceinline__ void col_solve_upper(T* g, const T* Us, int c = -1) {
  if (c < 0) c = threadIdx.x;
  if (c >= TS) return;
  T x[TS];
#pragma unroll
  for (int r = 0; r < TS; ++r) x[r] = g[r * TS + c];
  if constexpr (std::is_same<T, double>::value) {
#pragma unroll
    for (int k = TS - 1; k >= 0; --k) {
      T acc = x[k];
#pragma unroll
      for (int i = k + 1; i < TS; ++i) acc -= Us[k * SP + i] * x[i];
      x[k] = acc / Us[k * SP + k];
    }
  } else {
#pragma unroll
    for (int k = TS - 1; k >= 0; --k) {
      T acc[4] = {x[k], T(0), T(0), T(0)};
#pragma unroll
      for (int i = k + 1; i < TS; ++i) acc[(i - k - 1) & 3] -= Us[k * SP + i] * x[i];
      x[k] = ((acc[0] + acc[2]) + (acc[1] + acc[3])) / Us[k * SP + k];
    }
  }
#pragma unroll
  for (int r = 0; r < TS; ++r) g[r * TS + c] = x[r];
}

// Transposed substitutions.  The caller stages the TRANSPOSE of the factored
// diagonal tile (Dt[r][c] = D[c][r]) so that the inner loops read rows.

// g <- U^-T g: with Ut = U^T (lower, diagonal of U), forward substitution.
template <typename T>
__device__ __forceinline__ void col_solve_lower_trans(T* g, const T* Ut) {
  const int c = threadIdx.x;
  if (c >= TS) return;
  T x[TS];
#pragma unroll
  for (int r = 0; r < TS; ++r) x[r] = g[r * TS + c];
#pragma unroll
  for (int k = 0; k < TS; ++k) {
    T acc = x[k];
#pragma unroll
    for (int i = 0; i < k; ++i) acc -= Ut[k * SP + i] * x[i];
    x[k] = acc / Ut[k * SP + k];
  }
#pragma unroll
  for (int r = 0; r < TS; ++r) g[r * TS + c] = x[r];
}

// g <- P^T L^-T g: with Lt = L^T (unit upper), backward substitution; perm[r]
// is the original tile row at row r, so result row r goes to row perm[r].
template <typename T>
__device__ __forceinline__ void col_solve_upper_unit_trans(T* g, const T* Lt, const int* perm) {
  const int c = threadIdx.x;
  if (c >= TS) return;
  T x[TS];
#pragma unroll
  for (int r = 0; r < TS; ++r) x[r] = g[r * TS + c];
#pragma unroll
  for (int k = TS - 2; k >= 0; --k) {
    T acc = x[k];
#pragma unroll
    for (int i = k + 1; i < TS; ++i) acc -= Lt[k * SP + i] * x[i];
    x[k] = acc;
  }
  if (perm) {
    int pr[TS];
#pragma unroll
    for (int r = 0; r < TS; ++r) pr[r] = perm[r];
#pragma unroll
    for (int r = 0; r < TS; ++r) g[pr[r] * TS + c] = x[r];
  } else {
#pragma unroll
    for (int r = 0; r < TS; ++r) g[r * TS + c] = x[r];
  }
}

// Shared tile <- transpose of a global tile.
template <typename T>
__device__ __forceinline__ void load_tile_trans_n(T* __restrict__ s, const T* __restrict__ g, int nthreads) {
  for (int idx = threadIdx.x; idx < TS2; idx += nthreads) s[(idx % TS) * SP + idx / TS] = g[idx];
}

// g <- g U^-1 (U upper with diagonal): thread r owns row r.  The rows pass
// through shared memory Ws (stride SPA) so that the global accesses stay
// coalesced and the row reads conflict-free.  FP32 and double-float eliminate
// in column order: x[k] /= U(k,k), then x[j] -= x[k] U(k,j) for every j > k
// (independent updates, U's row k read as a broadcast; Ws holds TS x SPA
// elements).  FP64 solves U^T x = a by forward substitution in dot-product
// order, with U^T staged into Ws's tail (2 TS x SPA elements in all).
template <typename T>
__device__ __forceinline__ void row_solve_upper(T* g, const T* Us, T* Ws) {
  constexpr bool F64 = std::is_same<T, double>::value;
  T* Ut = Ws + TS * SPA;  // FP64 only: Ut[k][i] = U[i][k], stride SPA
  for (int idx = threadIdx.x; idx < TS2; idx += blockDim.x) {
    const int a = idx / TS, b = idx % TS;
    Ws[a * SPA + b] = g[idx];
    if (F64) Ut[b * SPA + a] = Us[a * SP + b];
  }
  __syncthreads();
  const int r = threadIdx.x;
  if (r < TS) {
    T x[TS];
#pragma unroll
    for (int k = 0; k < TS; ++k) x[k] = Ws[r * SPA + k];
    if constexpr (F64) {
#pragma unroll
      for (int k = 0; k < TS; ++k) {
        T acc = x[k];
#pragma unroll
        for (int i = 0; i < k; ++i) acc -= Ut[k * SPA + i] * x[i];
        x[k] = acc / Ut[k * SPA + k];
      }
    } else {
#pragma unroll
      for (int k = 0; k < TS; ++k) {
        const T xk = x[k] / Us[k * SP + k];
        x[k] = xk;
#pragma unroll
        for (int j = k + 1; j < TS; ++j) x[j] -= xk * Us[k * SP + j];
      }
    }
#pragma unroll
    for (int k = 0; k < TS; ++k) Ws[r * SPA + k] = x[k];
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < TS2; idx += blockDim.x) g[idx] = Ws[(idx / TS) * SPA + idx % TS];
}

}  // namespace fdm
