// deb_observables.cu -- observables on top of the perturbations: redshift-
// space multipoles and Kaiser P(k, mu), Savitzky-Golay smoothing of ln P, and
// the phase factors of the FFTLog transform to the correlation function.
// C ABI in include/discoeb_gb300.h.  Reference: src/discoeb/perturbations.py
// get_xi_from_P :1065-1098, get_power_smoothed :1126-1159, power_Kaiser
// :1162-1199, power_multipoles :1202-1224; util.py lngamma_complex_e :12-44.

#include <cuda_runtime.h>

#include <cmath>

#include "deb_core.cuh"
#include "discoeb_gb300.h"

namespace {

// sqrt of the primordial factor 2 pi^2 A_s (k / k_p)^(n_s - 1) k^-3 of
// get_power (perturbations.py:1123): the amplitude that turns y[idx] into
// sqrt(P)
__device__ double amplitude(const double* tables, int blob_len, int ci, double k) {
  const double* b = tables + (long)ci * blob_len;
  const double As = b[deb::H_AS], ns = b[deb::H_NS], kp = b[deb::H_KP];
  return sqrt(2.0 * M_PI * M_PI * As * pow(k / kp, ns - 1.0) * pow(k, -3.0));
}

// one thread per (mode, output): P0, P2, P4 (perturbations.py:1217-1224)
__global__ void multipoles_kernel(const double* tables, int ncosmo, int blob_len, const double* k, const int* cosmo,
                                  int nmode, int nout, const double* y, int stride, double b, double* P0, double* P2,
                                  double* P4) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)nmode * nout) return;
  const int m = (int)(t / nout);
  const int ci = cosmo ? cosmo[m] : 0;
  if (ci < 0 || ci >= ncosmo) {
    P0[t] = P2[t] = P4[t] = __longlong_as_double(0x7ff8000000000000LL);
    return;
  }
  const double A = amplitude(tables, blob_len, ci, k[m]);
  const double d = A * y[t * stride + 4], th = A * y[t * stride + 5];
  P0[t] = b * b * d * d - 2.0 * b / 3.0 * d * th + th * th / 5.0;
  P2[t] = -4.0 * b / 3.0 * d * th + 4.0 / 7.0 * th * th;
  P4[t] = 8.0 / 35.0 * th * th;
}

// one thread per (mode, mu): (b delta - mu^2 theta)^2 (perturbations.py:1198)
__global__ void kaiser_kernel(const double* delta, const double* theta, int nmode, const double* mu, int nmu, double b,
                              double* out) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)nmode * nmu) return;
  const int m = (int)(t / nmu), j = (int)(t - (long)m * nmu);
  const double v = b * delta[m] - mu[j] * mu[j] * theta[m];
  out[t] = v * v;
}

// delta and theta amplitudes sqrt(fac) y[4], sqrt(fac) y[5] (perturbations.py:1188-1190)
__global__ void fields_kernel(const double* tables, int ncosmo, int blob_len, const double* k, const int* cosmo,
                              int nmode, const double* y, int stride, double* delta, double* theta) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nmode) return;
  const int ci = cosmo ? cosmo[m] : 0;
  if (ci < 0 || ci >= ncosmo) {
    delta[m] = theta[m] = __longlong_as_double(0x7ff8000000000000LL);
    return;
  }
  const double A = amplitude(tables, blob_len, ci, k[m]);
  delta[m] = A * y[(long)m * stride + 4];
  theta[m] = A * y[(long)m * stride + 5];
}

// Savitzky-Golay smoothing of ln P along k for nrow independent rows of n
// points: 'same' convolution with the window coefficients (zero outside the
// row), exp, and the first window/2 and the last window/2 + 1 points
// replaced by the input, as the reference's slices [:w//2] and [-w//2:] do
// for odd w (perturbations.py:1148-1159, util.py:407-444).  One thread per point.
__global__ void savgol_log_kernel(const double* P, int nrow, int n, const double* c, int w, double* out) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)nrow * n) return;
  const int r = (int)(t / n), i = (int)(t - (long)r * n);
  const double* row = P + (long)r * n;
  const int h = w / 2;
  if (i < h || i >= n - h - 1) {
    out[t] = row[i];
    return;
  }
  double s = 0.0;
  for (int j = 0; j < w; ++j) s += c[w - 1 - j] * log(row[i + j - h]);   // convolution flips the window
  out[t] = exp(s);
}

// complex helpers for the Lanczos series
struct C { double re, im; };
__device__ C cmul(C a, C b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__device__ C cadd(C a, C b) { return {a.re + b.re, a.im + b.im}; }
__device__ C clog(C a) { return {log(hypot(a.re, a.im)), atan2(a.im, a.re)}; }

// ln Gamma(z) for Re z > 1/2 by the published Lanczos series (g = 7, nine
// coefficients), the method of util.py:23-39; FFTLog only needs
// z = (1.5 + ell) / 2 + i t with ell >= 0.
__device__ C lngamma_lanczos(C z) {
  const double c[9] = {0.99999999999980993227684700473478, 676.520368121885098567009190444019,
                       -1259.13921672240287047156078755283, 771.3234287776530788486528258894,
                       -176.61502916214059906584551354, 12.507343278686904814458936853,
                       -0.13857109526572011689554707, 9.984369578019570859563e-6, 1.50563273514931155834e-7};
  const C zm = {z.re - 1.0, z.im};
  C ag = {c[0], 0.0};
  for (int j = 1; j < 9; ++j) {
    const double dr = zm.re + j, di = zm.im, d2 = dr * dr + di * di;
    ag = cadd(ag, C{c[j] * dr / d2, -c[j] * di / d2});   // c_j / (z - 1 + j)
  }
  const C t = {zm.re + 7.5, zm.im};
  const C lt = clog(t);
  const C a = cmul(C{zm.re + 0.5, zm.im}, lt);
  const C la = clog(ag);
  return {a.re - t.re + 0.91893853320467274178 + la.re, a.im - t.im + la.im};
}

// FFTLog phase factors exp(2 i (arg Gamma(z_p) - ln(pi) t_p)), z_p = (1.5 + ell)/2 + i t_p,
// t_p = pi p / L, p = 0 .. nfreq-1 (perturbations.py:1088-1094); interleaved (re, im)
__global__ void fftlog_phase_kernel(int nfreq, double L, int ell, double* phase) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nfreq) return;
  const double t = M_PI * p / L;
  const C lg = lngamma_lanczos(C{(1.5 + ell) / 2.0, t});
  const double ang = 2.0 * (lg.im - log(M_PI) * t);
  phase[2 * p] = cos(ang);
  phase[2 * p + 1] = sin(ang);
}

int grid_of(long n, int block) { return (int)((n + block - 1) / block); }

}  // namespace

extern "C" {

int deb_power_multipoles(const double* d_tables, int ncosmo, int blob_len, const double* d_k, const int* d_cosmo_of_mode,
                         int nmode, int nout, const double* d_y, int stride, double bias, double* d_P0, double* d_P2,
                         double* d_P4, void* stream) {
  if (nmode < 0 || nout <= 0 || stride < 6 || ncosmo <= 0 || blob_len <= deb::HDR_LEN) return DEB_ERR_INVALID;
  if (nmode == 0) return DEB_OK;
  if (!d_tables || !d_k || !d_y || !d_P0 || !d_P2 || !d_P4) return DEB_ERR_INVALID;
  const long n = (long)nmode * nout;
  multipoles_kernel<<<grid_of(n, 128), 128, 0, (cudaStream_t)stream>>>(d_tables, ncosmo, blob_len, d_k, d_cosmo_of_mode,
                                                                        nmode, nout, d_y, stride, bias, d_P0, d_P2, d_P4);
  return cudaGetLastError() == cudaSuccess ? DEB_OK : DEB_ERR_CUDA;
}

int deb_density_velocity(const double* d_tables, int ncosmo, int blob_len, const double* d_k, const int* d_cosmo_of_mode,
                         int nmode, const double* d_y, int stride, double* d_delta, double* d_theta, void* stream) {
  if (nmode < 0 || stride < 6 || ncosmo <= 0 || blob_len <= deb::HDR_LEN) return DEB_ERR_INVALID;
  if (nmode == 0) return DEB_OK;
  if (!d_tables || !d_k || !d_y || !d_delta || !d_theta) return DEB_ERR_INVALID;
  fields_kernel<<<grid_of(nmode, 128), 128, 0, (cudaStream_t)stream>>>(d_tables, ncosmo, blob_len, d_k, d_cosmo_of_mode,
                                                                        nmode, d_y, stride, d_delta, d_theta);
  return cudaGetLastError() == cudaSuccess ? DEB_OK : DEB_ERR_CUDA;
}

int deb_power_kaiser(const double* d_delta, const double* d_theta, int nmode, const double* d_mu, int nmu, double bias,
                     double* d_Pkmu, void* stream) {
  if (nmode < 0 || nmu <= 0) return DEB_ERR_INVALID;
  if (nmode == 0) return DEB_OK;
  if (!d_delta || !d_theta || !d_mu || !d_Pkmu) return DEB_ERR_INVALID;
  const long n = (long)nmode * nmu;
  kaiser_kernel<<<grid_of(n, 128), 128, 0, (cudaStream_t)stream>>>(d_delta, d_theta, nmode, d_mu, nmu, bias, d_Pkmu);
  return cudaGetLastError() == cudaSuccess ? DEB_OK : DEB_ERR_CUDA;
}

int deb_savgol_log(const double* d_P, int nrow, int n, const double* d_coeffs, int window, double* d_out, void* stream) {
  if (nrow < 0 || n <= 0 || window <= 0 || (window & 1) == 0 || window > n) return DEB_ERR_INVALID;
  if (nrow == 0) return DEB_OK;
  if (!d_P || !d_coeffs || !d_out) return DEB_ERR_INVALID;
  const long t = (long)nrow * n;
  savgol_log_kernel<<<grid_of(t, 128), 128, 0, (cudaStream_t)stream>>>(d_P, nrow, n, d_coeffs, window, d_out);
  return cudaGetLastError() == cudaSuccess ? DEB_OK : DEB_ERR_CUDA;
}

int deb_fftlog_phase(int nfreq, double log_kmax_over_kmin, int ell, double* d_phase, void* stream) {
  if (nfreq <= 0 || !(log_kmax_over_kmin > 0.0) || ell < 0 || !d_phase) return DEB_ERR_INVALID;
  fftlog_phase_kernel<<<grid_of(nfreq, 128), 128, 0, (cudaStream_t)stream>>>(nfreq, log_kmax_over_kmin, ell, d_phase);
  return cudaGetLastError() == cudaSuccess ? DEB_OK : DEB_ERR_CUDA;
}

}  // extern "C"
