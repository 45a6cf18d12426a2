// reconstruct.cu — FP64 reconstruction of spectral functions from Chebyshev
// moments on the device.
//   kernel_seq                TB/numerical.h:393-447 (Dirichlet, Fejer, Lorentz,
//                             Jackson, Lanczos, Wang-Zunger)
//   expn_coef_alpha_seq       TB/numerical.h:304-316 (resolvent coefficients)
//   GreenFunctionImag::()     TB/lattice.h:618-624
//   GreenFunctionImag::fft    TB/lattice.h:625-640 (FFTW REDFT01 = DCT-III)
//   density_of_states_seq     TB/functions.h:26-30
#include <cuda_runtime.h>

#include <complex>
#include <vector>

#include "tbk_internal.h"

namespace tbk {

__device__ double kernel_value(int kind, int N, int n, double p0, double p1) {
  const double pi = 3.14159265358979323846;
  switch (kind) {
    case TBK_KERNEL_DIRICHLET: return 1.0;
    case TBK_KERNEL_FEJER: return 1.0 - (double)n / N;
    case TBK_KERNEL_LORENTZ: return sinh(p0 * (1.0 - (double)n / N)) / sinh(p0);
    case TBK_KERNEL_JACKSON: {
      int N1 = N + 1;
      double s1 = pi / N1, s2 = n * s1;
      return ((N1 - n) * cos(s2) + sin(s2) / tan(s1)) / N1;
    }
    case TBK_KERNEL_LANCZOS: {
      double piN = pi / N;
      return pow(sin(n * piN) / piN, p0);
    }
    case TBK_KERNEL_WANG_ZUNGER: return exp(-pow(n * (p0 / N), p1));
  }
  return 1.0;
}

__global__ void kernel_seq_kernel(int kind, int N, double p0, double p1, double* g) {
  int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n < N) g[n] = kernel_value(kind, N, n, p0, p1);
}

struct dc { double r, i; };
__device__ __forceinline__ dc cmul(dc a, dc b) { return {a.r * b.r - a.i * b.i, a.r * b.i + a.i * b.r}; }
__device__ __forceinline__ dc cdiv(dc a, dc b) {
  double d = b.r * b.r + b.i * b.i;
  return {(a.r * b.r + a.i * b.i) / d, (a.i * b.r - a.r * b.i) / d};
}
__device__ __forceinline__ dc csqrt_p(dc z) {  // principal branch, as std::sqrt(complex)
  double m = hypot(z.r, z.i);
  double s = sqrt(0.5 * (m + fabs(z.r)));
  if (s == 0.0) return {0.0, 0.0};
  if (z.r >= 0.0) return {s, z.i / (2.0 * s)};
  return {fabs(z.i) / (2.0 * s), signbit(z.i) ? -s : s};
}

// f(z) = sum_n g_n Im(alpha_n(z)) mu_n with the reference's recurrence for alpha_n.
__global__ void green_imag_kernel(int n, const double* __restrict__ g, const double* __restrict__ mu, int nz,
                                  const double* __restrict__ z, double scale, double* __restrict__ out) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nz) return;
  dc zz = {z[2 * k], z[2 * k + 1]};
  dc z2 = cmul(zz, zz);
  dc s1 = csqrt_p({1.0 - z2.r, 0.0 - z2.i});
  dc s2 = {zz.r + s1.i, zz.i - s1.r};              // z - i s1
  dc sn = cdiv({0.0, -2.0}, s1);
  dc a0 = cdiv({0.0, -1.0}, s1);
  double sum = g[0] * a0.i * mu[0];
  for (int m = 1; m < n; ++m) {
    sn = cmul(sn, s2);
    sum += g[m] * sn.i * mu[m];
  }
  out[k] = scale * sum;
}

// DCT-III (REDFT01) of g*mu at x_k = cos((k+1/2) pi / N), times 1/sqrt(1-x^2).
__global__ void green_fft_kernel(int n, const double* __restrict__ g, const double* __restrict__ mu, int N,
                                 double* __restrict__ E, double* __restrict__ val) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= N) return;
  const double pi = 3.14159265358979323846;
  double th = 0.5 * pi / N + k * (pi / N);
  double x = cos(th);
  // T_m(x) by the three-term recurrence
  double t0 = 1.0, t1 = x;
  double y = g[0] * mu[0];
  for (int m = 1; m < n; ++m) {
    y += 2.0 * (g[m] * mu[m]) * t1;
    double t2 = 2.0 * x * t1 - t0;
    t0 = t1;
    t1 = t2;
  }
  E[k] = x;
  val[k] = y * (1.0 / sqrt(1.0 - x * x));
}

template <typename T>
static int upload(DevBuf& b, const T* h, size_t n, cudaStream_t st) {
  TBK_TRY(b.alloc(sizeof(T) * (n ? n : 1)));
  if (n) TBK_CUDA(cudaMemcpyAsync(b.p, h, sizeof(T) * n, cudaMemcpyHostToDevice, st));
  return TBK_OK;
}

}  // namespace tbk

using namespace tbk;

extern "C" {

int tbk_expn_coef_alpha_seq(double z_re, double z_im, int32_t n, double* alpha) {
  if (n < 1 || !alpha) return fail(TBK_ERR_INVALID, "tbk_expn_coef_alpha_seq: bad argument");
  // 1/(z - x) = sum_k alpha_k(z) T_k(x), TB/numerical.h:304-316: s1 = sqrt(1 - z^2)
  // (principal branch), alpha_0 = -i / s1, alpha_k = -2i (z - i s1)^k / s1
  const std::complex<double> z(z_re, z_im), I(0.0, 1.0);
  const std::complex<double> s1 = std::sqrt(1.0 - z * z);
  const std::complex<double> s2 = z - I * s1;
  std::complex<double> sn = -2.0 * I / s1;
  const std::complex<double> a0 = -I / s1;
  alpha[0] = a0.real();
  alpha[1] = a0.imag();
  for (int32_t k = 1; k < n; ++k) {
    sn *= s2;
    alpha[2 * k] = sn.real();
    alpha[2 * k + 1] = sn.imag();
  }
  return TBK_OK;
}

int tbk_kernel_seq(int32_t kind, int32_t N, double p0, double p1, double* g_out) {
  if (N < 1 || !g_out) return fail(TBK_ERR_INVALID, "tbk_kernel_seq: bad argument");
  if (kind < 0 || kind > 5) return fail(TBK_ERR_INVALID, "unknown kernel %d", kind);
  DevBuf g;
  TBK_TRY(g.alloc(sizeof(double) * N));
  kernel_seq_kernel<<<(N + 255) / 256, 256>>>(kind, N, p0, p1, g.as<double>());
  TBK_CHECK_LAUNCH();
  TBK_CUDA(cudaMemcpy(g_out, g.p, sizeof(double) * N, cudaMemcpyDeviceToHost));
  return TBK_OK;
}

int tbk_green_imag_eval(int32_t n, const double* g, const double* mu, int32_t n_z, const double* z, double* out,
                        void* stream) {
  if (n < 1 || n_z < 0 || !g || !mu || (n_z && (!z || !out))) return fail(TBK_ERR_INVALID, "tbk_green_imag_eval: bad argument");
  if (n_z == 0) return TBK_OK;
  cudaStream_t st = as_stream(stream);
  DevBuf dg, dm, dz, dout;
  TBK_TRY(upload(dg, g, n, st));
  TBK_TRY(upload(dm, mu, n, st));
  TBK_TRY(upload(dz, z, 2 * (size_t)n_z, st));
  TBK_TRY(dout.alloc(sizeof(double) * n_z));
  green_imag_kernel<<<(n_z + 127) / 128, 128, 0, st>>>(n, dg.as<double>(), dm.as<double>(), n_z, dz.as<double>(),
                                                       1.0, dout.as<double>());
  TBK_CHECK_LAUNCH();
  TBK_CUDA(cudaMemcpyAsync(out, dout.p, sizeof(double) * n_z, cudaMemcpyDeviceToHost, st));
  TBK_CUDA(cudaStreamSynchronize(st));
  return TBK_OK;
}

int tbk_green_imag_fft(int32_t n, const double* g, const double* mu, int32_t upsample, double* E_out,
                       double* val_out, void* stream) {
  if (n < 1 || !g || !mu || !E_out || !val_out) return fail(TBK_ERR_INVALID, "tbk_green_imag_fft: bad argument");
  if (upsample < 1) upsample = 1;
  cudaStream_t st = as_stream(stream);
  const int32_t N = n * upsample;
  DevBuf dg, dm, dE, dv;
  TBK_TRY(upload(dg, g, n, st));
  TBK_TRY(upload(dm, mu, n, st));
  TBK_TRY(dE.alloc(sizeof(double) * N));
  TBK_TRY(dv.alloc(sizeof(double) * N));
  green_fft_kernel<<<(N + 127) / 128, 128, 0, st>>>(n, dg.as<double>(), dm.as<double>(), N, dE.as<double>(),
                                                    dv.as<double>());
  TBK_CHECK_LAUNCH();
  TBK_CUDA(cudaMemcpyAsync(E_out, dE.p, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
  TBK_CUDA(cudaMemcpyAsync(val_out, dv.p, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
  TBK_CUDA(cudaStreamSynchronize(st));
  return TBK_OK;
}

int tbk_dos_from_moments(int32_t n, const double* mu, int32_t kind, double p0, double p1, double R, int32_t n_e,
                         const double* e, double* rho, void* stream) {
  if (n < 1 || !mu || n_e < 0 || (n_e && (!e || !rho)) || !(R > 0.0))
    return fail(TBK_ERR_INVALID, "tbk_dos_from_moments: bad argument");
  if (kind < 0 || kind > 5) return fail(TBK_ERR_INVALID, "unknown kernel %d", kind);
  if (n_e == 0) return TBK_OK;
  cudaStream_t st = as_stream(stream);
  DevBuf dg, dm, dz, dout;
  TBK_TRY(dg.alloc(sizeof(double) * n));
  kernel_seq_kernel<<<(n + 255) / 256, 256, 0, st>>>(kind, n, p0, p1, dg.as<double>());
  TBK_CHECK_LAUNCH();
  TBK_TRY(upload(dm, mu, n, st));
  std::vector<double> z(2 * (size_t)n_e);
  for (int32_t k = 0; k < n_e; ++k) { z[2 * k] = e[k]; z[2 * k + 1] = 0.0; }
  TBK_TRY(upload(dz, z.data(), z.size(), st));
  TBK_TRY(dout.alloc(sizeof(double) * n_e));
  const double pi = 3.14159265358979323846;
  // rho = -1/R/pi * f(e), TB/functions.h:28
  green_imag_kernel<<<(n_e + 127) / 128, 128, 0, st>>>(n, dg.as<double>(), dm.as<double>(), n_e, dz.as<double>(),
                                                       -1.0 / R / pi, dout.as<double>());
  TBK_CHECK_LAUNCH();
  TBK_CUDA(cudaMemcpyAsync(rho, dout.p, sizeof(double) * n_e, cudaMemcpyDeviceToHost, st));
  TBK_CUDA(cudaStreamSynchronize(st));
  return TBK_OK;
}

}  // extern "C"
