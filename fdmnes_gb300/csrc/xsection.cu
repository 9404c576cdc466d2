// xsection.cu - dipole absorption of every energy of a batch from its Taull,
// and the Lorentzian convolution of the spectrum, in FP64 on the device.
//
// Cross-section.  For a K edge the dipole (E1E1) channel reaches the p
// harmonics of the absorber, and tens_ab (source/tensor.f90:1218-1264) forms
// the tensor from Taull(L=1 block) times the radial integrals of the two
// transitions.  With the real harmonics of the real path, the L = 1 rows
// Lm0 - 1 = 1, 2, 3 (m = -1, 0, 1) are the Cartesian components y, z, x, so
// the polarisation tensor is
//   S(a, b) = -Im( w(E) * (T(m_a, m_b) + T(m_b, m_a)) / 2 ),   a, b in {x, y, z},
// with w(E) = |rof(E)|^2 the radial weight (1 when the caller gives none), and
// the isotropic absorption sigma(E) = S(x,x) + S(y,y) + S(z,z).  For complex
// batches (spin-orbit, complex harmonics) only sigma is formed: the trace of
// the L = 1 block summed over both spin blocks, a basis-independent quantity.
//
// Convolution (source/convolution.f90:1612-1680).  Sample j stands for the bin
// [e1_j, e2_j] between the mid-points to its neighbours (the outer edges
// extrapolated by half a step) and the Lorentzian of half width b is integrated
// exactly over every bin:
//   out(E_i) = -(1/pi) sum_j [atan((e1_j - E_i)/b) - atan((e2_j - E_i)/b)] x_j,
// with b = width(E_i) (the reference's bb(ie)), or width(E_j) per input bin
// (Gamma_var); widths are clamped below at 1e-8 as the reference does.
#include <cuda_runtime.h>

#include "fdm_internal.cuh"
#include "fdm_kernels.h"

namespace fdm {

namespace {

// one warp per energy
__global__ void k_dipole(const Prob* probs, const double* taull, const double* weight, int nprob, double* sigma,
                         double* tensor) {
  const int k = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  if (k >= nprob) return;
  const Prob P = probs[k];
  const double2* T = reinterpret_cast<const double2*>(taull + 2 * P.taull);
  const int nlm = P.nlm_abs;
  const double w = weight ? weight[k] : 1.0;
  if (P.cplx) {
    // trace of the L = 1 block of every spin block
    const int nsp = P.so ? 2 : 1, nlmq = nlm / nsp;
    double s = 0.0;
    if (lane < 3 * nsp) {
      const int m = lane % 3, sp = lane / 3;
      const int i = 1 + m + nlmq * sp;
      s = -w * T[i + (int64_t)nlm * i].y;
    }
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) sigma[k] = s;
    return;
  }
  // Cartesian a = x, y, z -> 0-based harmonic 3, 1, 2
  double v = 0.0;
  if (lane < 9) {
    const int a = lane / 3, b = lane % 3;
    const int ia = a == 0 ? 3 : a, ib = b == 0 ? 3 : b;
    v = -w * 0.5 * (T[ia + (int64_t)nlm * ib].y + T[ib + (int64_t)nlm * ia].y);
    if (tensor) tensor[9 * (int64_t)k + lane] = v;
  }
  double s = (lane == 0 || lane == 4 || lane == 8) ? v : 0.0;
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) sigma[k] = s;
}

// one thread per output energy; the bins are recomputed from the energies
__global__ void k_lorentz(const double* E, const double* x, const double* width, int width_per_input, int n,
                          double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double Ei = E[i];
  double acc = 0.0;
  for (int j = 0; j < n; ++j) {
    const double e1 = j == 0 ? 1.5 * E[0] - 0.5 * E[1] : 0.5 * (E[j] + E[j - 1]);
    const double e2 = j == n - 1 ? 1.5 * E[n - 1] - 0.5 * E[n - 2] : 0.5 * (E[j] + E[j + 1]);
    const double bw = width[width_per_input ? j : i];
    const double b = bw >= 0.0 ? fmax(bw, 1e-8) : bw;
    acc += (atan((e1 - Ei) / b) - atan((e2 - Ei) / b)) * x[j];
  }
  out[i] = -acc / 3.14159265358979323846;
}

}  // namespace

void launch_dipole(const Prob* probs, const double* taull, const double* weight, int nprob, double* sigma,
                   double* tensor, cudaStream_t s) {
  k_dipole<<<(nprob + 3) / 4, 128, 0, s>>>(probs, taull, weight, nprob, sigma, tensor);
}

void launch_lorentz(const double* E, const double* x, const double* width, int width_per_input, int n, double* out,
                    cudaStream_t s) {
  k_lorentz<<<(n + 127) / 128, 128, 0, s>>>(E, x, width, width_per_input, n, out);
}

}  // namespace fdm
