// Initial conditions (21cmpy's Programs/initialize.py:33-111, initialize.cu:58-95, 133-190): the
// k-space pieces around the engine's inverse FFT.
//
//  * ic_spectrum: the Gaussian random field's half spectrum in numpy rfftn layout,
//    H(k) = sqrt(P(|k|) V) (n_re + i n_im) / sqrt(2) for 0 < k_z < N/2 and the Hermitian part
//    sqrt(P V) ((n_re(k) + n_re(-k)) + i (n_im(k) - n_im(-k))) / 2 on the k_z = 0 and N/2 planes, P
//    linearly interpolated in a table (init_kernel, initialize.cu:58-95).  The reference fills a
//    full complex box with independent normals and keeps the real part of its inverse FFT; that
//    real part is the inverse FFT of the Hermitian part of the box, whose modes have exactly this
//    distribution (variance P V per mode), so the half spectrum is drawn directly.
//  * ic_shape: H(k) times the smoothing window W(kR) (HII_filter, initialize.cu:12-40) and, for a
//    velocity component c, the factor i k_c / k^2 (set_velocity, initialize.cu:148-190), zero at
//    the component's Nyquist index (an odd derivative has no real value there; the reference's
//    real part drops it the same way).
//  * ic_subsample: nearest-cell subsample of a DIM^3 box onto HII_DIM^3 with a scale factor
//    (subsample, initialize.cu:133-146, and the 1 / scale^3 normalisation of initialize.py:89-109).
#include <cuda_runtime.h>
#include <stdint.h>

#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <string>

#include "es_engine.h"
#include "es_kernels.cuh"

namespace ic {

__device__ __forceinline__ int wrapk(int m, int n) { return m > n / 2 ? m - n : m; }

// first index i in [1, tn) with K[i] >= k (K[0] < k holds for every k > 0 of the box)
__device__ __forceinline__ int upper(const float* K, int tn, float k) {
  int lo = 1, hi = tn - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (K[mid] >= k) hi = mid; else lo = mid + 1;
  }
  return lo;
}

__global__ void spectrum_kernel(int n, float dk, const float* __restrict__ nre, const float* __restrict__ nim,
                                const float* __restrict__ K, const float* __restrict__ P, int tn, float vol,
                                float2* __restrict__ out) {
  const int h = n / 2 + 1;
  const long total = (long)n * n * h;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (long)gridDim.x * blockDim.x) {
    const int k2 = (int)(idx % h);
    const long t = idx / h;
    const int k1 = (int)(t % n), k0 = (int)(t / n);
    const float kx = __fmul_rn((float)wrapk(k0, n), dk), ky = __fmul_rn((float)wrapk(k1, n), dk),
                kz = __fmul_rn((float)k2, dk);
    const float ksq = __fadd_rn(__fadd_rn(__fmul_rn(kx, kx), __fmul_rn(ky, ky)), __fmul_rn(kz, kz));
    if (ksq == 0.0f) {
      out[idx] = make_float2(0.f, 0.f);
      continue;
    }
    const float kmag = __fsqrt_rn(ksq);
    const int i = upper(K, tn, kmag);
    // P[i-1] + (P[i] - P[i-1]) (k - K[i-1]) / (K[i] - K[i-1])   (initialize.cu:90)
    const float ps = __fadd_rn(P[i - 1], __fdiv_rn(__fmul_rn(__fsub_rn(P[i], P[i - 1]), __fsub_rn(kmag, K[i - 1])),
                                                 __fsub_rn(K[i], K[i - 1])));
    const float amp = __fsqrt_rn(__fmul_rn(ps, vol));
    if (k2 != 0 && k2 != n / 2) {
      const float a = __fmul_rn(amp, 0.70710678118654752f);
      out[idx] = make_float2(__fmul_rn(a, nre[idx]), __fmul_rn(a, nim[idx]));
    } else {
      // the k_z = 0 and N/2 planes hold both k and -k: their Hermitian part (X_k + conj X_-k) / 2,
      // real at the self-conjugate modes
      const long mid = ((long)((n - k0) % n) * n + (n - k1) % n) * h + k2;
      const float re = __fmul_rn(__fadd_rn(nre[idx], nre[mid]), 0.5f);
      const float im = __fmul_rn(__fsub_rn(nim[idx], nim[mid]), 0.5f);
      out[idx] = make_float2(__fmul_rn(amp, re), __fmul_rn(amp, im));
    }
  }
}

__global__ void shape_kernel(int n, float dk, const float2* __restrict__ in, int comp, int filter, float R,
                             int k2cut, int ref_compat, float2* __restrict__ out) {
  const int h = n / 2 + 1;
  const long total = (long)n * n * h;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (long)gridDim.x * blockDim.x) {
    const int k2 = (int)(idx % h);
    const long t = idx / h;
    const int k1 = (int)(t % n), k0 = (int)(t / n);
    const int m0 = wrapk(k0, n), m1 = wrapk(k1, n);
    const int kk = m0 * m0 + m1 * m1 + k2 * k2;
    float2 v = in[idx];
    const float W = filter >= 0 ? es::filter_weight(kk, dk, R, k2cut, filter, ref_compat) : 1.0f;
    v = make_float2(v.x * W, v.y * W);
    if (comp >= 0) {
      const int mc = comp == 0 ? m0 : (comp == 1 ? m1 : k2);
      if (kk == 0 || mc == n / 2) {           // no odd derivative at the component's Nyquist index
        v = make_float2(0.f, 0.f);
      } else {
        const float kc = (float)(comp == 0 ? m0 : (comp == 1 ? m1 : k2)) * dk;
        const float f = kc / ((float)kk * dk * dk);           // k_c / k^2
        v = make_float2(-f * v.y, f * v.x);                   // i f (a + i b)
      }
    }
    out[idx] = v;
  }
}

__global__ void subsample_kernel(int dim, int sw, float pf, float scale, const float* __restrict__ large,
                                 float* __restrict__ small) {
  const long total = (long)sw * sw * sw;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (long)gridDim.x * blockDim.x) {
    const int a2 = (int)(idx % sw);
    const long t = idx / sw;
    const int a1 = (int)(t % sw), a0 = (int)(t / sw);
    int l[3];
    const int a[3] = {a0, a1, a2};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      int li = (int)floorf(__fadd_rn(__fmul_rn((float)a[d], pf), 0.5f));
      l[d] = li < 0 ? 0 : (li >= dim ? dim - 1 : li);
    }
    small[idx] = __fmul_rn(large[((size_t)l[0] * dim + l[1]) * dim + l[2]], scale);
  }
}

}  // namespace ic

namespace {
thread_local std::string g_ic_error;
int icfail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_ic_error = buf;
  return code;
}
unsigned grid_for(long total) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  long b = (total + 255) / 256;
  const long cap = (long)sms * 8;
  return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}
}  // namespace

extern "C" {

int ic_spectrum(int n, float box_len, const float* normals_re, const float* normals_im, const float* k_table,
                const float* p_table, int table_n, void* out_half, void* stream) {
  if (n < 2 || n > 2048 || !(box_len > 0.f) || !normals_re || !normals_im || !k_table || !p_table || !out_half ||
      table_n < 2)
    return icfail(ES_E_ARG, "ic_spectrum: bad arguments");
  const float dk = (float)(2.0 * M_PI / (double)box_len);
  const float vol = box_len * box_len * box_len;
  const long total = (long)n * n * (n / 2 + 1);
  ic::spectrum_kernel<<<grid_for(total), 256, 0, (cudaStream_t)stream>>>(
      n, dk, normals_re, normals_im, k_table, p_table, table_n, vol, (float2*)out_half);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? ES_OK : icfail(ES_E_CUDA, "ic_spectrum launch: %s", cudaGetErrorString(e));
}

int ic_shape(int n, float box_len, const void* in_half, int component, int filter_type, float R, int ref_compat,
             void* out_half, void* stream) {
  if (n < 2 || n > 2048 || !(box_len > 0.f) || !in_half || !out_half || component < -1 || component > 2 ||
      filter_type < -1 || filter_type > 2)
    return icfail(ES_E_ARG, "ic_shape: bad arguments");
  const float dk = (float)(2.0 * M_PI / (double)box_len);
  // k-space top-hat keeps modes with (dk |k| R) 0.413566994 <= 1 (initialize.cu:31-34)
  int k2cut = INT_MAX;
  if (filter_type == 1 || (ref_compat && filter_type == 0)) {
    const double d = dk, r = R;
    long m = (long)std::floor(std::pow(1.0 / (0.413566994 * d * r), 2)) + 2;
    while (m >= 0 && (d * std::sqrt((double)m) * r) * 0.413566994 > 1.0) --m;
    k2cut = (int)(m < (long)INT_MAX ? m : (long)INT_MAX);
  }
  const long total = (long)n * n * (n / 2 + 1);
  ic::shape_kernel<<<grid_for(total), 256, 0, (cudaStream_t)stream>>>(n, dk, (const float2*)in_half, component,
                                                                       filter_type, R, k2cut, ref_compat,
                                                                       (float2*)out_half);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? ES_OK : icfail(ES_E_CUDA, "ic_shape launch: %s", cudaGetErrorString(e));
}

int ic_subsample(int dim, int hii_dim, float pixel_factor, float scale, const float* large, float* small,
                 void* stream) {
  if (dim < 1 || hii_dim < 1 || hii_dim > dim || !(pixel_factor > 0.f) || !large || !small)
    return icfail(ES_E_ARG, "ic_subsample: bad arguments");
  const long total = (long)hii_dim * hii_dim * hii_dim;
  ic::subsample_kernel<<<grid_for(total), 256, 0, (cudaStream_t)stream>>>(dim, hii_dim, pixel_factor, scale, large,
                                                                           small);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? ES_OK : icfail(ES_E_CUDA, "ic_subsample launch: %s", cudaGetErrorString(e));
}

int ic_last_error(char* buf, int len) {
  if (!buf || len <= 0) return ES_E_ARG;
  std::snprintf(buf, (size_t)len, "%s", g_ic_error.c_str());
  return ES_OK;
}

}  // extern "C"
