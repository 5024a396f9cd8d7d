// lombscargle.cu -- generalised Lomb-Scargle periodogram on top of the adjoint
// NFFT (the use the reference library was written for, its README).
//
// Floating-mean periodogram (Zechmeister & Kuerster 2009) with weights
// w_j = 1/dy_j^2 normalised to sum 1 (uniform without dy), at frequencies
// f_k = (k + 1) df, k = 0 .. nfreq-1:
//   A_k = sum_j w_j (y_j - ybar) e^{i w t_j},  B_k = sum_j w_j e^{i w t_j},
//   YC = Re A, YS = Im A, C = Re B_k, S = Im B_k, C2 = Re B_2k, S2 = Im B_2k,
//   CC = (1 + C2)/2 - C^2, SS = (1 - C2)/2 - S^2, CS = S2/2 - C S,
//   P = (SS YC^2 + CC YS^2 - 2 CS YC YS) / (YY (CC SS - CS^2)),
//   YY = sum_j w_j (y_j - ybar)^2.
// A and B come from one two-channel adjoint NFFT (cuna2_adjoint_multi: shared
// binning and gridding) of an accurate plan with period T = 1/df, so output
// bin k is frequency k df; the common phase factor of the
// x = (t - t0)/T - 1/2 origin multiplies A_k, B_k by (-1)^k and B_2k by 1,
// which leaves P unchanged.
#include <math.h>
#include <map>
#include <mutex>
#include <tuple>
#include "common.cuh"
#include "runtime.h"

namespace cuna {
namespace {

// sums[0] = sum w, sums[1] = sum w y, sums[2] = sum w y^2 (double)
template <typename T>
__global__ void k_ls_sums(const T *__restrict__ y, const T *__restrict__ dy, int64_t n, double *sums) {
  double a = 0, b = 0, c = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double w = dy ? 1.0 / ((double)dy[i] * (double)dy[i]) : 1.0;
    const double v = (double)y[i];
    a += w;
    b += w * v;
    c += w * v * v;
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
    c += __shfl_down_sync(0xffffffffu, c, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&sums[0], a);
    atomicAdd(&sums[1], b);
    atomicAdd(&sums[2], c);
  }
}

// w_j / sum w and w_j (y_j - ybar) / sum w
template <typename T>
__global__ void k_ls_weights(const T *__restrict__ y, const T *__restrict__ dy, int64_t n,
                             const double *__restrict__ sums, T *__restrict__ w, T *__restrict__ wy) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double W = sums[0], ybar = sums[1] / sums[0];
  const double wi = (dy ? 1.0 / ((double)dy[i] * (double)dy[i]) : 1.0) / W;
  w[i] = (T)wi;
  wy[i] = (T)(wi * ((double)y[i] - ybar));
}

template <typename T>
__global__ void k_ls_power(const typename CxOf<T>::type *__restrict__ A, const typename CxOf<T>::type *__restrict__ B,
                           int64_t K, int64_t nfreq, const double *__restrict__ sums, T *__restrict__ P) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;  // frequency (k + 1) df
  if (k >= nfreq) return;
  const int64_t q = k + 1;
  const double W = sums[0], ybar = sums[1] / W;
  const double YY = sums[2] / W - ybar * ybar;
  const double YC = A[K + q].x, YS = A[K + q].y;
  const double C = B[K + q].x, S = B[K + q].y;
  const double C2 = B[K + 2 * q].x, S2 = B[K + 2 * q].y;
  const double CC = 0.5 * (1.0 + C2) - C * C;
  const double SS = 0.5 * (1.0 - C2) - S * S;
  const double CS = 0.5 * S2 - C * S;
  const double D = CC * SS - CS * CS;
  const double num = SS * YC * YC + CC * YS * YS - 2.0 * CS * YC * YS;
  P[k] = (YY > 0 && D > 0) ? (T)(num / (YY * D)) : (T)0;
}

std::mutex g_ls_mu;
std::map<std::tuple<int, int, int64_t, int, int>, cuna2_plan> *g_ls_plans =
    new std::map<std::tuple<int, int, int64_t, int, int>, cuna2_plan>();

template <typename T>
int ls_run(int dtype, const double *t, const T *y, const T *dy, int64_t n, int64_t nfreq, double df, double t0,
           int R, int m, T *P, cudaStream_t st) {
  typedef typename CxOf<T>::type C;
  if (n < 2 || !t || !y || !P || nfreq < 1 || !(df > 0) || !std::isfinite(df) || !std::isfinite(t0))
    return fail(CUNA2_ERROR_INVALID_VALUE, "invalid argument (n=%lld nfreq=%lld df=%g)", (long long)n,
                (long long)nfreq, df);
  // outputs up to 2 (nfreq) df are needed: nf / 2 > 2 nfreq, nf a power of two
  int64_t nf = 2;
  while (nf / 2 <= 2 * nfreq) nf *= 2;
  int dev = 0;
  CUNA_CK(cudaGetDevice(&dev));
  cuna2_plan plan = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_ls_mu);
    auto key = std::make_tuple(dev, dtype, nf, R, m);
    auto it = g_ls_plans->find(key);
    if (it == g_ls_plans->end()) {
      CUNA_TRY(cuna2_plan_create(&plan, dtype, nf, R, m));
      (*g_ls_plans)[key] = plan;
    } else {
      plan = it->second;
    }
  }
  // workspace: sums (3 doubles) | channels [wy; w] | outputs [A; B]
  const size_t o_ch = 256, o_A = o_ch + ((2 * sizeof(T) * n + 255) & ~(size_t)255);
  void *ws = nullptr;
  CUNA_TRY(stream_workspace(st, o_A + 2 * sizeof(C) * nf, &ws));
  char *w8 = (char *)ws;
  double *sums = (double *)w8;
  T *wy = (T *)(w8 + o_ch), *w = wy + n;
  C *A = (C *)(w8 + o_A), *B = A + nf;
  CUNA_CK(cudaMemsetAsync(sums, 0, 3 * sizeof(double), st));
  k_ls_sums<T><<<std::min<int64_t>(4 * device_sm_count(), (n + 255) / 256), 256, 0, st>>>(y, dy, n, sums);
  CUNA_CK(cudaGetLastError());
  k_ls_weights<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(y, dy, n, sums, w, wy);
  CUNA_CK(cudaGetLastError());
  const double T_ = 1.0 / df;
  // both channels in one fused transform (shared binning and gridding)
  CUNA_TRY(cuna2_adjoint_multi(plan, t, wy, A, n, 2, t0, T_, st));
  k_ls_power<T><<<(unsigned)((nfreq + 255) / 256), 256, 0, st>>>(A, B, nf / 2, nfreq, sums, P);
  CUNA_CK(cudaGetLastError());
  return CUNA2_SUCCESS;
}

}  // namespace
}  // namespace cuna

using namespace cuna;

extern "C" int cuna2_lomb_scargle(int dtype, const double *t, const void *y, const void *dy, int64_t n,
                                  int64_t nfreq, double df, double t0, int R, int m, void *power,
                                  cudaStream_t stream) {
  clear_error();
  if (dtype == CUNA2_F32)
    return ls_run<float>(dtype, t, (const float *)y, (const float *)dy, n, nfreq, df, t0, R, m, (float *)power,
                         stream);
  if (dtype == CUNA2_F64)
    return ls_run<double>(dtype, t, (const double *)y, (const double *)dy, n, nfreq, df, t0, R, m, (double *)power,
                          stream);
  return fail(CUNA2_ERROR_INVALID_VALUE, "dtype %d", dtype);
}
