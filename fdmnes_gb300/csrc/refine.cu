// refine.cu - mixed precision support: equilibration, FP64 -> FP32 band
// conversion, FP64 residual in CSR form and the refinement update.
//
// The FP32 factor is of the equilibrated matrix Dr A Dc, with Dr and Dc powers
// of two (exact in FP64), so only the conversion to FP32 rounds.  The residual
// b - A x is taken in FP64 from the assembled matrix (CSR copy of the nonzeros
// of the FP64 band) and the correction is solved with the FP32 factors:
//   x <- x + Dc * solve32(Dr * (b - A x)).
#include <cfloat>
#include "fdm_internal.cuh"
#include "fdm_kernels.h"

namespace fdm {

__device__ __forceinline__ double pow2_inv_scale(double m) {
  if (!(m > 0.0) || !isfinite(m)) return 1.0;
  int ex;
  frexp(m, &ex);           // m = f * 2^ex, f in [0.5, 1)
  return ldexp(1.0, -ex);  // m * scale in [0.5, 1)
}

__device__ __forceinline__ void atomic_max_abs(unsigned long long* a, double v) {
  atomicMax(a, (unsigned long long)__double_as_longlong(fabs(v)));
}

// The equilibration and conversion passes read the whole FP64 band; GB300's
// FP64 pipe is 1/64 of its FP32 rate, so they work on the bit patterns with
// integer instructions where the result is exact: the bits of a non-negative
// double order like its value, and scaling by a power of two 2^k is an add to
// the exponent field while the input and the result are normal numbers (the
// other cases take the FP64 expression, with the same result as before).
__device__ __forceinline__ unsigned long long abs_bits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
}
// the exponent k of a normal power of two 2^k
__device__ __forceinline__ int pow2_exp(double s) { return (int)((__double_as_longlong(s) >> 52) & 0x7FF) - 1023; }
// bits of |s x| for s = 2^k
__device__ __forceinline__ unsigned long long scaled_abs_bits(double x, double s, int k) {
  const unsigned long long b = abs_bits(x);
  if (b == 0) return 0;
  const int E = (int)(b >> 52);
  if (E >= 1 && E + k >= 1 && E + k <= 2046) return b + ((unsigned long long)(long long)k << 52);
  return abs_bits(s * x);
}
// float(sr sc x) rounded to nearest even, for sr sc = 2^k
__device__ __forceinline__ float scaled_to_float(double x, double sr, double sc, int k) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned long long a = u & 0x7FFFFFFFFFFFFFFFull;
  const unsigned sign = (unsigned)(u >> 63) << 31;
  if (a == 0) return __uint_as_float(sign);
  const int E = (int)(a >> 52);
  const int e32 = E + k - 1023 + 127;
  if (E >= 1 && e32 >= 1 && e32 <= 254) {
    const unsigned long long M = a & 0xFFFFFFFFFFFFFull;
    unsigned bits = ((unsigned)e32 << 23) | (unsigned)(M >> 29);
    const unsigned long long rem = M & 0x1FFFFFFFull;
    if (rem > 0x10000000ull || (rem == 0x10000000ull && (bits & 1u))) bits += 1u;  // a carry may reach inf
    return __uint_as_float(bits | sign);
  }
  return (float)(sr * sc * x);
}
// dfl(sr sc x) (high part rounded to nearest, low part the rounded remainder)
// for sr sc = 2^k: the remainder is the low 29 mantissa bits less the rounding
// step, an integer below 2^28 in units of the double's last place
__device__ __forceinline__ dfl scaled_to_dfl(double x, double sr, double sc, int k) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned long long a = u & 0x7FFFFFFFFFFFFFFFull;
  const unsigned neg = (unsigned)(u >> 63);
  if (a == 0) return dfl(__uint_as_float(neg << 31), 0.f);
  const int E = (int)(a >> 52);
  const int e32 = E + k - 1023 + 127, sh = E + k - 1075;
  if (E >= 1 && e32 >= 1 && e32 <= 253 && sh >= -126 && sh <= 127) {
    const unsigned long long M = a & 0xFFFFFFFFFFFFFull;
    const unsigned top = (unsigned)(M >> 29);
    const int rem = (int)(M & 0x1FFFFFFFull);
    const int up = (rem > 0x10000000 || (rem == 0x10000000 && (top & 1u))) ? 1 : 0;
    const float hi = __uint_as_float((((unsigned)e32 << 23) | top) + (unsigned)up | (neg << 31));
    const int r = rem - (up << 29);
    float lo = 0.f;
    if (r != 0) {
      lo = __int2float_rn(r) * __uint_as_float((unsigned)(sh + 127) << 23);
      if (neg) lo = -lo;
    }
    return dfl(hi, lo);
  }
  return dfl(sr * sc * x);
}

// Locate the row block of band tile w of a problem (strip has nt+1 entries).
__device__ __forceinline__ int tile_row_of(const Tables& tb, const Prob& P, int64_t w) {
  int lo = 0, hi = P.nt - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) / 2;
    if (tb.strip[P.trow + mid] <= w) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Row scales: warp per row.
__global__ void k_rowscale(const Prob* probs, const double* env, double* rs, Tables tb) {
  const Prob P = probs[blockIdx.y];
  const int p = blockIdx.x * 8 + threadIdx.x / 32, lane = threadIdx.x % 32;
  const int npad = P.nt * TS;
  if (p >= npad) return;
  const int I = p / TS;
  const int j0 = tb.J0[P.trow + I], j1 = tb.J1[P.trow + I];
  unsigned long long m = 0;
  for (int J = j0; J <= j1; ++J) {
    const double* t = tile_ptr(const_cast<double*>(env), P, tb, I, J) + (p % TS) * TS;
    m = max(m, max(abs_bits(t[lane]), abs_bits(t[lane + 32])));
  }
  for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (lane == 0) rs[P.rowv + p] = pow2_inv_scale(__longlong_as_double((long long)m));
}

// Column maxima of |rs(p) a(p,q)|: block per band tile, into colmax (double bits).
__global__ void k_colmax(const Prob* probs, const double* env, const double* rs, unsigned long long* colmax,
                         Tables tb) {
  const Prob P = probs[blockIdx.y];
  const int64_t w = blockIdx.x;
  const int64_t ntiles = tb.strip[P.trow + P.nt];
  if (w >= ntiles) return;
  const int I = tile_row_of(tb, P, w);
  const int J = tb.J0[P.trow + I] + (int)(w - tb.strip[P.trow + I]);
  const double* t = env + P.env + w * TS2;
  __shared__ unsigned long long cm[4][TS];
  const int c = threadIdx.x % TS, r0 = threadIdx.x / TS;
  unsigned long long m = 0;
  for (int r = r0; r < TS; r += 4) {
    const double sr = rs[P.rowv + I * TS + r];
    m = max(m, scaled_abs_bits(t[r * TS + c], sr, pow2_exp(sr)));
  }
  cm[r0][c] = m;
  __syncthreads();
  if (threadIdx.x < TS) {
    m = max(max(cm[0][c], cm[1][c]), max(cm[2][c], cm[3][c]));
    atomicMax(&colmax[P.rowv + J * TS + c], m);
  }
}

__global__ void k_colscale_finish(const Prob* probs, double* cs) {
  const Prob P = probs[blockIdx.y];
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P.nt * TS) return;
  unsigned long long* bits = reinterpret_cast<unsigned long long*>(cs);
  const double m = __longlong_as_double((long long)bits[P.rowv + q]);
  cs[P.rowv + q] = pow2_inv_scale(m);
}

// E32 = float(rs * cs * E64), tile by tile.
__global__ void k_convert(const Prob* probs, const double* env64, float* env32, const double* rs, const double* cs,
                          Tables tb, const int* active) {
  if (active && !active[blockIdx.y]) return;
  const Prob P = probs[blockIdx.y];
  const int64_t w = blockIdx.x;
  const int64_t ntiles = tb.strip[P.trow + P.nt];
  if (w >= ntiles) return;
  const int I = tile_row_of(tb, P, w);
  const int J = tb.J0[P.trow + I] + (int)(w - tb.strip[P.trow + I]);
  const double* t = env64 + P.env + w * TS2;
  float* o = env32 + P.env + w * TS2;
  for (int idx = threadIdx.x; idx < TS2; idx += blockDim.x) {
    const int r = idx / TS, c = idx % TS;
    const double sr = rs[P.rowv + I * TS + r], sc = cs[P.rowv + J * TS + c];
    o[idx] = scaled_to_float(t[idx], sr, sc, pow2_exp(sr) + pow2_exp(sc));
  }
}

// Y32 = float(rs * B64) for every RHS tile.
__global__ void k_rhs_scale(const Prob* probs, const double* B, float* Y, const double* rs) {
  const Prob P = probs[blockIdx.y];
  const int64_t w = blockIdx.x;
  if (w >= (int64_t)P.nt * P.nrt) return;
  const int I = (int)(w / P.nrt);
  const double* b = B + P.rhs + w * TS2;
  float* y = Y + P.rhs + w * TS2;
  for (int idx = threadIdx.x; idx < TS2; idx += blockDim.x) y[idx] = (float)(rs[P.rowv + I * TS + idx / TS] * b[idx]);
}

// CSR of the nonzeros of the FP64 band: count per row (warp per row).
__global__ void k_csr_count(const Prob* probs, const double* env, int* rowptr, Tables tb) {
  const Prob P = probs[blockIdx.y];
  const int p = blockIdx.x * 8 + threadIdx.x / 32, lane = threadIdx.x % 32;
  if (p >= P.nt * TS) return;
  const int I = p / TS;
  int cnt = 0;
  for (int J = tb.J0[P.trow + I]; J <= tb.J1[P.trow + I]; ++J) {
    const double* t = tile_ptr(const_cast<double*>(env), P, tb, I, J) + (p % TS) * TS;
    cnt += __popc(__ballot_sync(0xffffffffu, abs_bits(t[lane]) != 0)) +
           __popc(__ballot_sync(0xffffffffu, abs_bits(t[lane + 32]) != 0));
  }
  if (lane == 0) rowptr[P.rowv + p + 1] = cnt;
}

// Exclusive scan of the row counts of one problem (one block per problem).
__global__ void k_csr_scan(const Prob* probs, int* rowptr) {
  const Prob P = probs[blockIdx.y];
  const int npad = P.nt * TS;
  int* rp = rowptr + P.rowv;
  __shared__ int part[1024];
  const int per = (npad + blockDim.x - 1) / blockDim.x;
  const int a = threadIdx.x * per, b = min(npad, a + per);
  int s = 0;
  for (int p = a; p < b; ++p) s += rp[p + 1];
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int k = 0; k < (int)blockDim.x; ++k) { const int v = part[k]; part[k] = acc; acc += v; }
  }
  __syncthreads();
  int acc = part[threadIdx.x];
  for (int p = a; p < b; ++p) { acc += rp[p + 1]; rp[p + 1] = acc; }
  if (threadIdx.x == 0) rp[0] = 0;
}

__global__ void k_csr_fill(const Prob* probs, const double* env, const int* rowptr, int* col, double* val, float2* val2,
                           Tables tb, int* err) {
  const Prob P = probs[blockIdx.y];
  const int p = blockIdx.x * 8 + threadIdx.x / 32, lane = threadIdx.x % 32;
  if (p >= P.nt * TS) return;
  const int I = p / TS;
  int pos = rowptr[P.rowv + p];
  const unsigned lower = (1u << lane) - 1u;
  for (int J = tb.J0[P.trow + I]; J <= tb.J1[P.trow + I]; ++J) {
    const double* t = tile_ptr(const_cast<double*>(env), P, tb, I, J) + (p % TS) * TS;
    for (int h = 0; h < 2; ++h) {
      const double v = t[lane + 32 * h];
      const bool nz = abs_bits(v) != 0;
      const unsigned bal = __ballot_sync(0xffffffffu, nz);
      if (nz) {
        const int o = pos + __popc(bal & lower);
        if (o < P.csr_cap) {
          col[P.csr + o] = J * TS + lane + 32 * h;
          val[P.csr + o] = v;
          const float hi = (float)v;
          val2[P.csr + o] = make_float2(hi, (float)(v - (double)hi));
        } else {
          atomicExch(&err[blockIdx.y], (int)FDMGPU_ERR_ARG);
        }
      }
      pos += __popc(bal);
    }
  }
}

// Y32 = float(rs * (B64 - A X64)), warp per row, lanes over RHS columns.
__global__ void k_residual(const Prob* probs, const int* rowptr, const int* col, const double* val, const double* B,
                           const double* X, float* Y, const double* rs, unsigned long long* rmax, const int* active) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  if (active && !active[e]) return;
  const int p = blockIdx.x * 8 + threadIdx.x / 32, lane = threadIdx.x % 32;
  if (p >= P.nt * TS) return;
  const int k0 = rowptr[P.rowv + p], k1 = min(rowptr[P.rowv + p + 1], (int)P.csr_cap);
  const int nrhs = P.nrt * TS;
  const double sc = rs[P.rowv + p];
  double rm = 0.0;
  for (int r0 = 0; r0 < nrhs; r0 += 256) {
    double acc[8];
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const int r = r0 + lane + 32 * t;
      acc[t] = (r < nrhs) ? B[P.rhs + ((int64_t)(p / TS) * P.nrt + r / TS) * TS2 + (p % TS) * TS + (r % TS)] : 0.0;
    }
    for (int k = k0; k < k1; ++k) {
      const int q = col[P.csr + k];
      const double a = val[P.csr + k];
      const double* xr = X + P.rhs + ((int64_t)(q / TS) * P.nrt) * TS2 + (q % TS) * TS;
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const int r = r0 + lane + 32 * t;
        if (r < nrhs) acc[t] -= a * xr[(int64_t)(r / TS) * TS2 + (r % TS)];
      }
    }
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const int r = r0 + lane + 32 * t;
      if (r < nrhs) {
        rm = fmax(rm, fabs(acc[t]));
        Y[P.rhs + ((int64_t)(p / TS) * P.nrt + r / TS) * TS2 + (p % TS) * TS + (r % TS)] = (float)(sc * acc[t]);
      }
    }
  }
  for (int o = 16; o; o >>= 1) rm = fmax(rm, __shfl_xor_sync(0xffffffffu, rm, o));
  if (lane == 0) atomic_max_abs(&rmax[e], rm);
}

// Double-float arithmetic (an FP64 stand-in on the FP32 pipes): a value is the
// unevaluated sum hi + lo of two floats, about 48 significand bits.
struct df {
  float hi, lo;
};
// acc -= a * x with a = (ah, al), x = (xh, xl): the product ah*xh is split
// exactly with an FMA, the cross terms are added at float precision, and the
// high parts are summed with Knuth's two-sum.
__device__ __forceinline__ void df_sub_prod(df& acc, float2 a, float2 x) {
  const float p = a.x * x.x;
  const float e = fmaf(a.x, x.x, -p);
  const float t = fmaf(a.x, x.y, fmaf(a.y, x.x, e));
  const float s = acc.hi - p;
  const float bb = s - acc.hi;
  const float err = (acc.hi - (s - bb)) + (-p - bb);
  acc.hi = s;
  acc.lo = acc.lo + (err - t);
}
__device__ __forceinline__ df df_norm(df a) {
  const float s = a.hi + a.lo;
  return df{s, a.lo - (s - a.hi)};
}

// Y32 = float(rs * (B - A X)) with A and X in double-float form.
__global__ void k_residual_df(const Prob* probs, const int* rowptr, const int* col, const float2* val2, const double* B,
                              const float2* Xs, float* Y, const double* rs, unsigned long long* rmax,
                              const int* active) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  if (active && !active[e]) return;
  const int p = blockIdx.x * 8 + threadIdx.x / 32, lane = threadIdx.x % 32;
  if (p >= P.nt * TS) return;
  const int k0 = rowptr[P.rowv + p], k1 = min(rowptr[P.rowv + p + 1], (int)P.csr_cap);
  const int nrhs = P.nrt * TS;
  const float sc = (float)rs[P.rowv + p];  // a power of two
  double rm = 0.0;
  for (int r0 = 0; r0 < nrhs; r0 += 256) {
    df acc[8];
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const int r = r0 + lane + 32 * t;
      const double b = (r < nrhs) ? B[P.rhs + ((int64_t)(p / TS) * P.nrt + r / TS) * TS2 + (p % TS) * TS + (r % TS)] : 0.0;
      acc[t].hi = (float)b;
      acc[t].lo = (float)(b - (double)acc[t].hi);
    }
    // the row's nonzeros in chunks of 32: lane j fetches the column and value
    // of nonzero j (one coalesced load each), broadcast by shuffles; two
    // nonzeros per step keep 16 X loads in flight per lane
    for (int kb = k0; kb < k1; kb += 32) {
      const int nk = min(32, k1 - kb);
      int qv = 0;
      float2 av = make_float2(0.f, 0.f);
      if (lane < nk) {
        qv = col[P.csr + kb + lane];
        av = val2[P.csr + kb + lane];
      }
      for (int j = 0; j < nk; j += 2) {
        const int q0 = __shfl_sync(0xffffffffu, qv, j);
        const float2 a0 = make_float2(__shfl_sync(0xffffffffu, av.x, j), __shfl_sync(0xffffffffu, av.y, j));
        const bool two = j + 1 < nk;
        const int q1 = __shfl_sync(0xffffffffu, qv, two ? j + 1 : j);
        const float2 a1 = two ? make_float2(__shfl_sync(0xffffffffu, av.x, j + 1), __shfl_sync(0xffffffffu, av.y, j + 1))
                              : make_float2(0.f, 0.f);
        const float2* xr0 = Xs + P.rhs + ((int64_t)(q0 / TS) * P.nrt) * TS2 + (q0 % TS) * TS;
        const float2* xr1 = Xs + P.rhs + ((int64_t)(q1 / TS) * P.nrt) * TS2 + (q1 % TS) * TS;
        float2 x0[8], x1[8];
#pragma unroll
        for (int t = 0; t < 8; ++t) {
          const int r = r0 + lane + 32 * t;
          const int64_t o = (int64_t)(r / TS) * TS2 + (r % TS);
          x0[t] = r < nrhs ? xr0[o] : make_float2(0.f, 0.f);
          x1[t] = (r < nrhs && two) ? xr1[o] : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int t = 0; t < 8; ++t) {
          df_sub_prod(acc[t], a0, x0[t]);
          df_sub_prod(acc[t], a1, x1[t]);
        }
      }
#pragma unroll
      for (int t = 0; t < 8; ++t) acc[t] = df_norm(acc[t]);
    }
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const int r = r0 + lane + 32 * t;
      if (r < nrhs) {
        const float v = acc[t].hi + acc[t].lo;
        rm = fmax(rm, fabs((double)v));
        Y[P.rhs + ((int64_t)(p / TS) * P.nrt + r / TS) * TS2 + (p % TS) * TS + (r % TS)] = sc * v;
      }
    }
  }
  for (int o = 16; o; o >>= 1) rm = fmax(rm, __shfl_xor_sync(0xffffffffu, rm, o));
  if (lane == 0) atomic_max_abs(&rmax[e], rm);
}

// Residual by recurrence: R32 -= (Dr A Dc) Y32, the equilibrated FP32 matrix
// times the correction just solved for, for the active problems.  Because the
// corrections shrink geometrically, the FP32 rounding of this update is second
// order in the FP32 unit roundoff relative to |A||x|; a true (double-float)
// residual confirms convergence.  Warp per row, nonzeros in chunks of 32.
__global__ void k_resid_update(const Prob* probs, const int* rowptr, const int* col, const float* valS, const float* Y,
                               float* R, const int* active) {
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
    for (int kb = k0; kb < k1; kb += 32) {
      const int nk = min(32, k1 - kb);
      int qv = 0;
      float av = 0.f;
      if (lane < nk) {
        qv = col[P.csr + kb + lane];
        av = valS[P.csr + kb + lane];
      }
      for (int j = 0; j < nk; j += 2) {
        const bool two = j + 1 < nk;
        const int q0 = __shfl_sync(0xffffffffu, qv, j), q1 = __shfl_sync(0xffffffffu, qv, two ? j + 1 : j);
        const float a0 = __shfl_sync(0xffffffffu, av, j);
        const float a1 = two ? __shfl_sync(0xffffffffu, av, j + 1) : 0.f;
        const float* y0 = Y + P.rhs + ((int64_t)(q0 / TS) * P.nrt) * TS2 + (q0 % TS) * TS;
        const float* y1 = Y + P.rhs + ((int64_t)(q1 / TS) * P.nrt) * TS2 + (q1 % TS) * TS;
        float v0[8], v1[8];
#pragma unroll
        for (int t = 0; t < 8; ++t) {
          const int r = r0 + lane + 32 * t;
          const int64_t o = (int64_t)(r / TS) * TS2 + (r % TS);
          v0[t] = r < nrhs ? y0[o] : 0.f;
          v1[t] = (r < nrhs && two) ? y1[o] : 0.f;
        }
#pragma unroll
        for (int t = 0; t < 8; ++t) acc[t] = fmaf(a1, v1[t], fmaf(a0, v0[t], acc[t]));
      }
    }
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const int r = r0 + lane + 32 * t;
      if (r < nrhs) R[P.rhs + ((int64_t)(p / TS) * P.nrt + r / TS) * TS2 + (p % TS) * TS + (r % TS)] -= acc[t];
    }
  }
}

// dst = src over the RHS tiles of the problems whose mask is set.
__global__ void k_copy_rhs32(const Prob* probs, const float* src, float* dst, const int* mask) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  if (!mask[e]) return;
  const int64_t w = blockIdx.x;
  if (w >= (int64_t)P.nt * P.nrt) return;
  const float4* a = reinterpret_cast<const float4*>(src + P.rhs + w * TS2);
  float4* b = reinterpret_cast<float4*>(dst + P.rhs + w * TS2);
  for (int idx = threadIdx.x; idx < TS2 / 4; idx += blockDim.x) b[idx] = a[idx];
}

void launch_resid_update(const Prob* probs, const Pools& pl, const LaunchDims& d, cudaStream_t s) {
  k_resid_update<<<dim3((d.max_rows + 7) / 8, d.nprob), 256, 0, s>>>(probs, pl.rowptr, pl.col, pl.valS, pl.Y32, pl.R32,
                                                                    pl.active);
}

void launch_copy_rhs32(const Prob* probs, const LaunchDims& d, const float* src, float* dst, const int* mask,
                       cudaStream_t s) {
  k_copy_rhs32<<<dim3(d.max_rhs_tiles, d.nprob), 256, 0, s>>>(probs, src, dst, mask);
}

// X64 (+)= cs * Y32 over RHS tiles, with per-problem maxima of |d| and |x|.
__global__ void k_update_x(const Prob* probs, const float* Y, double* X, float2* Xs, const double* cs, int first,
                           unsigned long long* dmax, unsigned long long* xmax, const int* active) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  if (active && !active[e]) return;
  const int64_t w = blockIdx.x;
  if (w >= (int64_t)P.nt * P.nrt) return;
  const int I = (int)(w / P.nrt);
  const float* y = Y + P.rhs + w * TS2;
  double* x = X + P.rhs + w * TS2;
  float2* xs = Xs + P.rhs + w * TS2;
  double dm = 0.0, xm = 0.0;
  for (int idx = threadIdx.x; idx < TS2; idx += blockDim.x) {
    const double d = cs[P.rowv + I * TS + idx / TS] * (double)y[idx];
    const double xn = first ? d : x[idx] + d;
    x[idx] = xn;
    const float hi = (float)xn;
    xs[idx] = make_float2(hi, (float)(xn - (double)hi));
    dm = fmax(dm, fabs(d));
    xm = fmax(xm, fabs(xn));
  }
  for (int o = 16; o; o >>= 1) {
    dm = fmax(dm, __shfl_xor_sync(0xffffffffu, dm, o));
    xm = fmax(xm, __shfl_xor_sync(0xffffffffu, xm, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomic_max_abs(&dmax[e], dm);
    atomic_max_abs(&xmax[e], xm);
  }
}

// smr(Lm, ii) = X(n - ii, Lm) (Fortran layout, nlmso x nligne).
__global__ void k_solution_out(Prob P, const double* X, double* smr) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)P.n * P.nlmso) return;
  const int lm = (int)(t % P.nlmso);
  const int ii = (int)(t / P.nlmso) + 1;
  const int p = P.n - ii;
  smr[t] = X[P.rhs + ((int64_t)(p / TS) * P.nrt + lm / TS) * TS2 + (p % TS) * TS + (lm % TS)];
}

void launch_equilibrate_convert(const Prob* probs, const Pools& pl, Tables tb, const LaunchDims& d, cudaStream_t s) {
  const int np = d.nprob;
  k_rowscale<<<dim3((d.max_rows + 7) / 8, np), 256, 0, s>>>(probs, pl.env64, pl.rs, tb);
  // cs first serves as the atomic column-max accumulator: it must start at 0
  cudaMemsetAsync(pl.cs, 0, d.rowv_total * sizeof(double), s);
  k_colmax<<<dim3(d.max_tiles, np), 256, 0, s>>>(probs, pl.env64, pl.rs, reinterpret_cast<unsigned long long*>(pl.cs),
                                                 tb);
  k_colscale_finish<<<dim3((d.max_rows + 255) / 256, np), 256, 0, s>>>(probs, pl.cs);
  k_convert<<<dim3(d.max_tiles, np), 256, 0, s>>>(probs, pl.env64, pl.env32, pl.rs, pl.cs, tb, nullptr);
  k_rhs_scale<<<dim3(d.max_rhs_tiles, np), 256, 0, s>>>(probs, pl.B64, pl.Y32, pl.rs);
}

// FP32 band of the problems marked in pl.active converted again from the FP64
// band with the batch's equilibration scales (before a re-factorisation).
void launch_convert_masked(const Prob* probs, const Pools& pl, Tables tb, const LaunchDims& d, cudaStream_t s) {
  k_convert<<<dim3(d.max_tiles, d.nprob), 256, 0, s>>>(probs, pl.env64, pl.env32, pl.rs, pl.cs, tb, pl.active);
}

void launch_csr(const Prob* probs, const Pools& pl, Tables tb, const LaunchDims& d, cudaStream_t s) {
  const int np = d.nprob;
  k_csr_count<<<dim3((d.max_rows + 7) / 8, np), 256, 0, s>>>(probs, pl.env64, pl.rowptr, tb);
  k_csr_scan<<<dim3(1, np), 1024, 0, s>>>(probs, pl.rowptr);
  k_csr_fill<<<dim3((d.max_rows + 7) / 8, np), 256, 0, s>>>(probs, pl.env64, pl.rowptr, pl.col, pl.val, pl.val2, tb,
                                                             pl.err);
}

void launch_csr_scan(const Prob* probs, int* ptr, const LaunchDims& d, cudaStream_t s) {
  k_csr_scan<<<dim3(1, d.nprob), 1024, 0, s>>>(probs, ptr);
}

void launch_residual(const Prob* probs, const Pools& pl, const LaunchDims& d, int df64, cudaStream_t s) {
  if (df64)
    k_residual_df<<<dim3((d.max_rows + 7) / 8, d.nprob), 256, 0, s>>>(probs, pl.rowptr, pl.col, pl.val2, pl.B64,
                                                                      pl.Xs, pl.Y32, pl.rs, pl.amax, pl.active);
  else
    k_residual<<<dim3((d.max_rows + 7) / 8, d.nprob), 256, 0, s>>>(probs, pl.rowptr, pl.col, pl.val, pl.B64, pl.X64,
                                                                   pl.Y32, pl.rs, pl.amax, pl.active);
}

void launch_update_x(const Prob* probs, const Pools& pl, const LaunchDims& d, int first, cudaStream_t s) {
  k_update_x<<<dim3(d.max_rhs_tiles, d.nprob), 256, 0, s>>>(probs, pl.Y32, pl.X64, pl.Xs, pl.cs, first, pl.dmax,
                                                            pl.xmax, first ? nullptr : pl.active);
}

// X64 = B64 for the active problems (start of an FP64 re-solve).
__global__ void k_copy_rhs(const Prob* probs, const double* B, double* X, const int* active) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  if (active && !active[e]) return;
  const int64_t w = blockIdx.x;
  if (w >= (int64_t)P.nt * P.nrt) return;
  for (int idx = threadIdx.x; idx < TS2; idx += blockDim.x) X[P.rhs + w * TS2 + idx] = B[P.rhs + w * TS2 + idx];
}

// Escalation to a double-float factorisation of the equilibrated matrix:
// envd = dfl(rs * cs * E64) in place over the FP64 band of the active problems.
__global__ void k_env_to_dfl(const Prob* probs, double* env, const double* rs, const double* cs, Tables tb,
                             const int* active) {
  const Prob P = probs[blockIdx.y];
  if (active && !active[blockIdx.y]) return;
  const int64_t w = blockIdx.x;
  if (w >= tb.strip[P.trow + P.nt]) return;
  const int I = tile_row_of(tb, P, w);
  const int J = tb.J0[P.trow + I] + (int)(w - tb.strip[P.trow + I]);
  double* t = env + P.env + w * TS2;
  dfl* o = reinterpret_cast<dfl*>(t);
  for (int idx = threadIdx.x; idx < TS2; idx += blockDim.x) {
    const double sr = rs[P.rowv + I * TS + idx / TS], sc = cs[P.rowv + J * TS + idx % TS];
    o[idx] = scaled_to_dfl(t[idx], sr, sc, pow2_exp(sr) + pow2_exp(sc));
  }
}

// D = dfl(rs * B64) (from_b) or dfl(Y32) (already scaled) for the active problems.
__global__ void k_rhs_to_dfl(const Prob* probs, const double* B, const float* Y, const double* rs, dfl* D, int from_b,
                             const int* active) {
  const Prob P = probs[blockIdx.y];
  if (active && !active[blockIdx.y]) return;
  const int64_t w = blockIdx.x;
  if (w >= (int64_t)P.nt * P.nrt) return;
  const int I = (int)(w / P.nrt);
  for (int idx = threadIdx.x; idx < TS2; idx += blockDim.x) {
    const int64_t o = P.rhs + w * TS2 + idx;
    D[o] = from_b ? dfl(rs[P.rowv + I * TS + idx / TS] * B[o]) : dfl((double)Y[o]);
  }
}

// X64 (+)= cs * D for the active problems, with the split copy and maxima.
__global__ void k_dfl_to_x(const Prob* probs, const dfl* D, double* X, float2* Xs, const double* cs, int first,
                           unsigned long long* dmax, unsigned long long* xmax, const int* active) {
  const int e = blockIdx.y;
  const Prob P = probs[e];
  if (active && !active[e]) return;
  const int64_t w = blockIdx.x;
  if (w >= (int64_t)P.nt * P.nrt) return;
  const int I = (int)(w / P.nrt);
  double dm = 0.0, xm = 0.0;
  for (int idx = threadIdx.x; idx < TS2; idx += blockDim.x) {
    const int64_t o = P.rhs + w * TS2 + idx;
    const double d = cs[P.rowv + I * TS + idx / TS] * (double)D[o];
    const double xn = first ? d : X[o] + d;
    X[o] = xn;
    const float hi = (float)xn;
    Xs[o] = make_float2(hi, (float)(xn - (double)hi));
    dm = fmax(dm, fabs(d));
    xm = fmax(xm, fabs(xn));
  }
  for (int o = 16; o; o >>= 1) {
    dm = fmax(dm, __shfl_xor_sync(0xffffffffu, dm, o));
    xm = fmax(xm, __shfl_xor_sync(0xffffffffu, xm, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomic_max_abs(&dmax[e], dm);
    atomic_max_abs(&xmax[e], xm);
  }
}

// Double-float re-solve of the active problems: factorisation of Dr A Dc,
// solve, then `iters` refinement steps with the double-float residual and the
// double-float factors.  Scratch D (dfl, RHS layout) must hold rhs elements.
// Number of CSR nonzeros of every problem.
__global__ void k_csr_nnz(const Prob* probs, int np, const int* rowptr, int* nnz) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= np) return;
  const Prob P = probs[e];
  nnz[e] = min(rowptr[P.rowv + P.nt * TS], (int)P.csr_cap);
}

void launch_csr_nnz(const Prob* probs, const int* rowptr, const LaunchDims& d, int* nnz, cudaStream_t s) {
  k_csr_nnz<<<(d.nprob + 127) / 128, 128, 0, s>>>(probs, d.nprob, rowptr, nnz);
}

int launch_dfl_escalation(const StepPlan& sp, const Prob* probs, const Pools& pl, Tables tb, const LaunchDims& d,
                          dfl* D, cudaStream_t s, cudaEvent_t ev_f0, cudaEvent_t ev_f1) {
  const int np = d.nprob;
  dfl* envd = reinterpret_cast<dfl*>(pl.env64);
  int nk = 0;
  k_env_to_dfl<<<dim3(d.max_tiles, np), 256, 0, s>>>(probs, pl.env64, pl.rs, pl.cs, tb, pl.active);
  k_rhs_to_dfl<<<dim3(d.max_rhs_tiles, np), 256, 0, s>>>(probs, pl.B64, pl.Y32, pl.rs, D, 1, pl.active);
  nk += 2;
  if (ev_f0) cudaEventRecord(ev_f0, s);
  nk += launch_factor<dfl>(sp, envd, D, probs, tb, np, 1, pl.active, pl.err, 1e-30, pl.piv, s);
  if (ev_f1) cudaEventRecord(ev_f1, s);
  nk += launch_backward<dfl>(sp, envd, D, probs, tb, np, pl.active, s);
  k_dfl_to_x<<<dim3(d.max_rhs_tiles, np), 256, 0, s>>>(probs, D, pl.X64, pl.Xs, pl.cs, 1, pl.dmax, pl.xmax, pl.active);
  return nk + 1;
}

// The FP32 band <- the high parts of the double-float band (the high part of a
// normalised double-float is its value rounded to FP32), active problems.
__global__ void k_dfl_to_f32(const Prob* probs, const double* env, float* env32, Tables tb, const int* active) {
  if (active && !active[blockIdx.y]) return;
  const Prob P = probs[blockIdx.y];
  const int64_t w = blockIdx.x;
  if (w >= tb.strip[P.trow + P.nt]) return;
  const float2* t = reinterpret_cast<const float2*>(env + P.env + w * TS2);
  float* o = env32 + P.env + w * TS2;
  for (int idx = threadIdx.x; idx < TS2; idx += blockDim.x) o[idx] = t[idx].x;
}

// The descriptors of the listed problems, contiguous: launches over an
// escalated subset then have one grid row per escalated problem instead of
// one per problem of the batch.
__global__ void k_gather_probs(const Prob* probs, const int* list, int n, Prob* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = probs[list[i]];
}
// Status words of a compact launch back to the batch's problems.
__global__ void k_scatter_err(const int* list, int n, const int* err_c, int* err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && err_c[i]) atomicExch(&err[list[i]], err_c[i]);
}
void launch_gather_probs(const Prob* probs, const int* list, int n, Prob* out, cudaStream_t s) {
  k_gather_probs<<<(n + 127) / 128, 128, 0, s>>>(probs, list, n, out);
}
void launch_scatter_err(const int* list, int n, const int* err_c, int* err, cudaStream_t s) {
  k_scatter_err<<<(n + 127) / 128, 128, 0, s>>>(list, n, err_c, err);
}

// Double-float factorisation of the active problems' equilibrated bands (in
// place of their FP64 bands) with the right-hand sides riding along, the
// double-float backward solve (X = the double-float solution, accurate to
// about the acceptance level of the refinement), and the factors rounded into
// the FP32 band for the FP32 refinement steps that confirm it; the
// double-float refinement steps that may follow read the double-float
// factors, which stay in place.
int launch_dfl_factor_f32(const StepPlan& sp, const Prob* probs, const Pools& pl, Tables tb, const LaunchDims& d,
                          dfl* D, cudaStream_t s, cudaEvent_t ev_f0, cudaEvent_t ev_f1) {
  const int np = d.nprob;
  dfl* envd = reinterpret_cast<dfl*>(pl.env64);
  int nk = 0;
  k_env_to_dfl<<<dim3(d.max_tiles, np), 256, 0, s>>>(probs, pl.env64, pl.rs, pl.cs, tb, pl.active);
  k_rhs_to_dfl<<<dim3(d.max_rhs_tiles, np), 256, 0, s>>>(probs, pl.B64, pl.Y32, pl.rs, D, 1, pl.active);
  nk += 2;
  if (ev_f0) cudaEventRecord(ev_f0, s);
  nk += launch_factor<dfl>(sp, envd, D, probs, tb, np, 1, pl.active, pl.err, 1e-30, pl.piv, s);
  if (ev_f1) cudaEventRecord(ev_f1, s);
  if (sp.strip && sp.dfl_uinv_keep)
    nk += launch_dfl_backward_inv(sp, envd, D, probs, tb, np, pl.active, pl.err, s);
  else
    nk += launch_backward<dfl>(sp, envd, D, probs, tb, np, pl.active, s);
  k_dfl_to_x<<<dim3(d.max_rhs_tiles, np), 256, 0, s>>>(probs, D, pl.X64, pl.Xs, pl.cs, 1, pl.dmax, pl.xmax, pl.active);
  k_dfl_to_f32<<<dim3(d.max_tiles, np), 256, 0, s>>>(probs, pl.env64, pl.env32, tb, pl.active);
  return nk + 2;
}

// One refinement step with the double-float factors: residual, solve, x += d;
// dmax / xmax receive max|d| and max|x| of each active problem.
int launch_dfl_refine_step(const StepPlan& sp, const Prob* probs, const Pools& pl, Tables tb, const LaunchDims& d,
                           dfl* D, cudaStream_t s) {
  const int np = d.nprob;
  dfl* envd = reinterpret_cast<dfl*>(pl.env64);
  int nk = 0;
  launch_residual(probs, pl, d, 1, s);
  k_rhs_to_dfl<<<dim3(d.max_rhs_tiles, np), 256, 0, s>>>(probs, pl.B64, pl.Y32, pl.rs, D, 0, pl.active);
  nk += 2;
  nk += launch_forward<dfl>(sp, envd, D, probs, tb, np, pl.active, pl.piv, s);
  nk += launch_backward<dfl>(sp, envd, D, probs, tb, np, pl.active, s);
  k_dfl_to_x<<<dim3(d.max_rhs_tiles, np), 256, 0, s>>>(probs, D, pl.X64, pl.Xs, pl.cs, 0, pl.dmax, pl.xmax, pl.active);
  return nk + 1;
}

void launch_rhs_to_dfl(const Prob* probs, const LaunchDims& d, const double* B, const float* Y, const double* scale,
                       dfl* D, int from_b, const int* mask, cudaStream_t s) {
  k_rhs_to_dfl<<<dim3(d.max_rhs_tiles, d.nprob), 256, 0, s>>>(probs, B, Y, scale, D, from_b, mask);
}

void launch_dfl_to_x(const Prob* probs, const LaunchDims& d, const dfl* D, double* X, float2* Xs, const double* scale,
                     int first, unsigned long long* dmax, unsigned long long* xmax, const int* mask, cudaStream_t s) {
  k_dfl_to_x<<<dim3(d.max_rhs_tiles, d.nprob), 256, 0, s>>>(probs, D, X, Xs, scale, first, dmax, xmax, mask);
}

void launch_copy_rhs(const Prob* probs, const Pools& pl, const LaunchDims& d, cudaStream_t s) {
  k_copy_rhs<<<dim3(d.max_rhs_tiles, d.nprob), 256, 0, s>>>(probs, pl.B64, pl.X64, pl.active);
}

void launch_solution_out(const Prob& P, const double* X, double* smr_dev, cudaStream_t s) {
  const int64_t n = (int64_t)P.n * P.nlmso;
  k_solution_out<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(P, X, smr_dev);
}

}  // namespace fdm

namespace fdm {

// Stopping rule of the classical refinement, evaluated on the device after
// every step (one block): problem k stops when r = max|dx|/max|x| <= tol or r
// is not finite, or after two consecutive steps that do not halve r; the loop
// ends when no problem is active or ctl->it reaches ctl->max_iter.  With a
// conditional handle, the while node of the refinement graph reads the
// decision, so no step needs the host.
__global__ void __launch_bounds__(1024) k_refine_check(RefineState* rs, int* active, const unsigned long long* dmax,
                                                       const unsigned long long* xmax, RefineCtl* ctl, int np,
                                                       cudaGraphConditionalHandle cond, int use_cond) {
  __shared__ int nact;
  if (threadIdx.x == 0) nact = 0;
  __syncthreads();
  const int it = ctl->it + 1;
  const double tol = ctl->tol;
  for (int k = threadIdx.x; k < np; k += blockDim.x) {
    RefineState s = rs[k];
    if (!s.active) continue;
    const double dm = __longlong_as_double((long long)dmax[k]);
    const double xm = __longlong_as_double((long long)xmax[k]);
    const double r = xm > 0 ? dm / xm : dm;
    s.iters = it;
    s.resid = r;
    if (!isfinite(r) || r <= tol) {
      s.active = 0;
    } else {
      s.slow = (it > 1 && r > 0.5 * s.prev) ? s.slow + 1 : 0;
      if (s.slow >= 2)
        s.active = 0;
      else
        atomicAdd(&nact, 1);
    }
    s.prev = r;
    rs[k] = s;
    active[k] = s.active;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    ctl->it = it;
    ctl->nact = nact;
    if (use_cond) cudaGraphSetConditional(cond, (nact > 0 && it < ctl->max_iter) ? 1u : 0u);
  }
}

__global__ void k_refine_init(RefineState* rs, int* active, int np) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= np) return;
  RefineState s;
  s.active = 1;
  s.slow = 0;
  s.iters = 0;
  s.pad = 0;
  s.prev = 1e300;
  s.resid = __longlong_as_double(0x7ff8000000000000ll);
  rs[k] = s;
  active[k] = 1;
}

void launch_refine_init(RefineState* rs, int* active, int np, cudaStream_t s) {
  k_refine_init<<<(np + 255) / 256, 256, 0, s>>>(rs, active, np);
}

void launch_refine_check(RefineState* rs, int* active, const Pools& pl, RefineCtl* ctl, int np,
                         cudaGraphConditionalHandle cond, int use_cond, cudaStream_t s) {
  k_refine_check<<<1, 1024, 0, s>>>(rs, active, pl.dmax, pl.xmax, ctl, np, cond, use_cond);
}

}  // namespace fdm
