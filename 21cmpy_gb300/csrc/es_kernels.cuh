// Excursion-set engine kernels, templated on the box size N (sm_103a).
//
// Spectrum layout in HBM (per box): the half spectrum of an N^3 real box is split into
//   main[k][j][i], i in [0, N/2)   (N * N * N/2 complex64, rows of N/2 elements)
//   nyq[k][j]                       (the i = N/2 plane, N * N complex64)
// where k and j are the z and y wavenumber indices (natural FFT order) and i the x one.
// Real boxes are C-order [z][y][x] float32, the reference's INDEX(k,j,i) (find_bubbles.cu:6).
//
// Passes (each one HBM read + one write of the data it touches):
//   rows  : length-N real <-> half-complex transform along x (N/2-point complex FFT + split)
//   col-y : length-N complex FFT along y within each z plane
//   col-z : length-N complex FFT along z
// The i = 0 and i = N/2 columns are Hermitian in (j, k); along y they are transformed together
// as one complex sequence (packed as re + i*im) and split again on the forward side.
#pragma once
#include <cuda.h>
#include "es_fft.cuh"

namespace es {

enum ColMode { COL_Z_FWD = 0, COL_Y_FWD = 1, COL_Z_INV_FILTER = 2, COL_Y_INV = 3, COL_Z_FWD_PK = 4, COL_Z_INV = 5 };
enum RowPro { PRO_SCALE = 0, PRO_PK = 1 };
enum RowEpi { EPI_STORE = 0, EPI_IONIZE = 1 };
// L2 policies of the TMA copies
enum { ES_HINT_NORMAL = 0, ES_HINT_EVICT_FIRST = 1, ES_HINT_EVICT_LAST = 2 };

constexpr int PK_MAX_BINS = 128;

struct OpArgs {
  // TMA descriptors of the column passes' input / output spectra (main array, Nyquist plane)
  CUtensorMap tm_in, tm_out, tm_in_nyq, tm_out_nyq;
  unsigned* err;                  // device error word (bounded waits that timed out)
  int variant;                    // passes: 0 synchronous tiles, 1 TMA double-buffered
  int col_tile, row_tile;         // TMA tile-shape variants (chosen by the autotuner)
  int col_radix, row_radix;       // radix schedules of the per-radius passes (0: up to 16, 1: up to 8)
  int hint_in, hint_out;          // L2 policies of the TMA loads / stores (ES_HINT_*)
  int discard_in;                 // row pass: drop the consumed input lines from L2
  int grid;                       // CTAs to launch (persistent grid-stride)
  int wait_log2;                  // TMA passes: 2^wait_log2 mbarrier polls before a wait times out (0: default)
  int stall;                      // TMA passes: debug stall of CTA 0's first tile (the wait times out)
  // real boxes viewed as float2 pairs of consecutive x
  const float2* rin;
  float2* rout;
  // spectra
  const float2* cin;
  const float2* cin_nyq;
  float2* cout;
  float2* cout_nyq;
  const float2* tw;               // w_N^m = exp(-2 pi i m / N), m < N
  // row R2C prologue
  float scale;                    // PRO_SCALE: multiply input by scale
  const float* ave;               // PRO_PK: device mean of the input
  float pk_norm;                  // PRO_PK: V / N^3
  int dimensional;                // PRO_PK: multiply by the mean (DIMENSIONAL_T_POWER_SPEC)
  // col-z inverse filter (times scale, the growth rescale)
  const float* wtab;              // W(k^2) / N^3 for this radius
  float fR;                       // filter radius [Mpc] (TMA variant computes W inline)
  int fk2cut;                     // k-space top-hat cut
  int filter, ref_compat;
  float inv_n3;
  // row C2R ionisation epilogue
  const float2* prev;             // delta_R of the previous radius (pairs)
  uint32_t* flags;                // ionisation bitmap, pair-major: voxel v = 2p + h is bit
                                  // (p % 32) + 32 h of 64-bit word p / 32
  int has_prev;
  float dc;                       // delta_c(z) (float32, find_bubbles.cu:54)
  float denom;                    // this radius
  float denom_prev;               // previous radius
  const float* stats_prev;        // {sum, mean, norm} of the previous radius
  float inv_zeta;                 // float32(1/zeta)
  int update;                     // 0 centre pixel, 1 sphere painting
  int marker;                     // centre pixel: carry the flag in delta_R's lowest mantissa bit
                                  // instead of the bitmap (TMA row pass)
  uint32_t* centers;              // sphere mode: centres passing at the previous radius
  unsigned* center_count;
  // reductions
  float* partials;
  unsigned* counter;
  float* stats_out;               // {sum, mean, norm}
  float fc_mean;                  // mean collapse fraction (normalisation target)
  int normalize;                  // rescale fcoll by fc_mean / <fcoll>
  // P(k)
  const int* thr;                 // integer k^2 thresholds per bin
  int nbins;
  float dk;
  float volume;
  float* pk_out;                  // [3 * nbins]: ps_ave, k_ave, count
};

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block sum; the result is valid in every thread.  sred holds T/32 floats.
template <int T>
__device__ __forceinline__ float block_sum(float v, float* sred) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) sred[warp] = v;
  __syncthreads();
  float s = 0.f;
#pragma unroll
  for (int w = 0; w < T / 32; ++w) s += sred[w];
  return s;
}

// Deterministic grid-wide sum: every CTA publishes its partial, the last CTA to arrive adds
// all partials in a fixed order.  Returns true in the last CTA, with *total set there.
template <int T>
__device__ __forceinline__ bool grid_sum(float mine, float* partials, unsigned* counter,
                                         float* sred, float* total) {
  __shared__ unsigned s_last;
  float s = block_sum<T>(mine, sred);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = s;
    __threadfence();
    unsigned t = atomicAdd(counter, 1u);
    s_last = (t == gridDim.x - 1) ? 1u : 0u;
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  float acc = 0.f;
  for (int i = threadIdx.x; i < (int)gridDim.x; i += T) acc += __ldcg(partials + i);
  acc = block_sum<T>(acc, sred);
  if (threadIdx.x == 0) *counter = 0u;
  *total = acc;
  return true;
}

// erfc for the per-radius sum of fcoll, after Numerical Recipes' erfcc (Press et al. 1992, sec.
// 6.2): erfc(z) = t exp(-z^2 - 1.26551223 + t P(t)), t = 1 / (1 + z/2), fractional error below
// 1.2e-7 for z >= 0, erfc(-z) = 2 - erfc(z).  z^2 is split exactly (hi + lo, with an FMA) so
// its rounding does not reach the exponential.  Only the sum over cells uses it; per-cell
// values (final partial ionisation) use the library erfcf.
__device__ __forceinline__ float erfc_sum_term(float x) {
  const float z = fabsf(x);
  const float t = __fdividef(1.0f, fmaf(0.5f, z, 1.0f));   // divisor in [1, 11]: within 2 ulp
  float p = 0.17087277f;
  p = fmaf(p, t, -0.82215223f);
  p = fmaf(p, t, 1.48851587f);
  p = fmaf(p, t, -1.13520398f);
  p = fmaf(p, t, 0.27886807f);
  p = fmaf(p, t, -0.18628806f);
  p = fmaf(p, t, 0.09678418f);
  p = fmaf(p, t, 0.37409196f);
  p = fmaf(p, t, 1.00002368f);
  const float hi = z * z;
  const float lo = fmaf(z, z, -hi);                    // z^2 = hi + lo exactly
  // __expf is accurate to a few units of the last place for the arguments (|x| < 20) where
  // erfc contributes to the sum
  const float r = t * __expf(fmaf(t, p, -1.26551223f) - hi) * (1.0f - lo);
  return x >= 0.0f ? r : 2.0f - r;
}

// ------------------------------------------------------------ packed FP32 pairs (sm_100 and later)
// A pair (lo, hi) of floats in one 64-bit register; fma/mul/add/sub.rn.f32x2 work on both halves
// with one instruction.
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 pk2(float lo, float hi) {
  f32x2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ f32x2 bc2(float v) { return pk2(v, v); }
__device__ __forceinline__ float2 upk2(f32x2 v) {
  float2 r;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
  return r;
}
__device__ __forceinline__ f32x2 fma2(f32x2 a, f32x2 b, f32x2 c) {
  f32x2 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ f32x2 mul2(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f32x2 add2(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f32x2 sub2(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// erfc_sum_term for two arguments at once on packed pairs (the same Numerical Recipes erfcc).
// log2(e) is folded into the polynomial and the constant so the exponential is one ex2 of
// (t P(t) - 1.26551223 - z^2) log2(e); z^2 = hi + lo is split exactly as above.  For x < 0 the
// term is 2 - r, written as s r + (1 - s) with s = copysign(1, x) so both halves stay packed.
__device__ __forceinline__ f32x2 erfc_sum_pair(f32x2 xv) {
  constexpr float L2E = 1.4426950408889634f;
  const float2 x = upk2(xv);
  const float z0 = fabsf(x.x), z1 = fabsf(x.y);
  const f32x2 Z = pk2(z0, z1), NZ = pk2(-z0, -z1);
  const float2 d = upk2(fma2(Z, bc2(0.5f), bc2(1.0f)));
  const f32x2 T = pk2(__fdividef(1.0f, d.x), __fdividef(1.0f, d.y));
  f32x2 P = bc2(0.17087277f * L2E);
  P = fma2(P, T, bc2(-0.82215223f * L2E));
  P = fma2(P, T, bc2(1.48851587f * L2E));
  P = fma2(P, T, bc2(-1.13520398f * L2E));
  P = fma2(P, T, bc2(0.27886807f * L2E));
  P = fma2(P, T, bc2(-0.18628806f * L2E));
  P = fma2(P, T, bc2(0.09678418f * L2E));
  P = fma2(P, T, bc2(0.37409196f * L2E));
  P = fma2(P, T, bc2(1.00002368f * L2E));
  const f32x2 H = mul2(Z, Z);                        // hi = z^2 rounded
  const f32x2 NLO = fma2(NZ, Z, H);                  // hi - z^2 = -lo exactly
  f32x2 E = fma2(T, P, bc2(-1.26551223f * L2E));
  E = fma2(H, bc2(-L2E), E);
  const float2 e = upk2(E);
  f32x2 R = mul2(T, pk2(ex2_approx(e.x), ex2_approx(e.y)));
  R = fma2(R, NLO, R);                               // r (1 - lo)
  const f32x2 S = pk2(copysignf(1.0f, x.x), copysignf(1.0f, x.y));
  return fma2(S, R, fma2(S, bc2(-1.0f), bc2(1.0f)));
}

// Real-space top-hat W(x) = 3 (sin x - x cos x) / x^3; below x = 1 its Taylor series
// sum_n 3 (-1)^n (2n+2) x^(2n) / (2n+3)! avoids the cancellation of the closed form.  Above it the
// hardware sine / cosine and division are used: for the arguments of a box (kR below ~150) their
// error is ~1e-5 relative on weights that are already below 1e-3 there, far under the float32
// rounding of the filtered field.
__device__ __forceinline__ float rtophat_f(float x) {
  if (x < 1.0f) {
    const float y = x * x;
    return 1.0f + y * (-0.1f + y * (1.0f / 280.0f + y * (-1.0f / 15120.0f +
           y * (1.0f / 1330560.0f + y * (-1.0f / 172972800.0f)))));
  }
  float s, c;
  __sincosf(x, &s, &c);
  return __fdividef(3.0f * (s - x * c), x * x * x);
}

// HII_filter's window (find_bubbles.cu:26-41) for a mode of integer |k/dk|^2 = k2.  k2cut is the
// host-computed k-space top-hat cut; ref_compat reproduces the switch fall-through 0 -> 1 -> 2.
__device__ __forceinline__ float filter_weight(int k2, float dk, float R, int k2cut, int filter, int ref_compat) {
  const float kR = dk * sqrtf((float)k2) * R;
  float W;
  if (!ref_compat) {
    if (filter == 0) W = rtophat_f(kR);
    else if (filter == 1) W = k2 <= k2cut ? 1.0f : 0.0f;
    else { const float x = 0.643f * kR; W = expf(-0.5f * x * x); }
  } else {
    W = 1.0f;
    float x = kR;
    if (filter == 0 && kR > 1e-4f) W = rtophat_f(kR);
    if (filter <= 1) { x *= 0.413566994f; if (k2 > k2cut) W = 0.0f; }
    x *= 0.643f;
    W *= expf(-0.5f * x * x);
  }
  return W;
}

__device__ __forceinline__ int isqrt_dev(int v) {
  int r = (int)sqrtf((float)v);
  while (r * r > v) --r;
  while ((r + 1) * (r + 1) <= v) ++r;
  return r;
}

__device__ __forceinline__ unsigned long long bit_range(long lo, long hi, long q) {
  // bits lo - 32q .. hi - 32q of a 32-bit half, clipped to [0, 31]; 0 when empty
  if (lo < 32 * q) lo = 32 * q;
  if (hi > 32 * q + 31) hi = 32 * q + 31;
  if (lo > hi) return 0ull;
  const int l = (int)(lo - 32 * q), h = (int)(hi - 32 * q);
  const unsigned long long top = h == 31 ? 0xffffffffull : ((1ull << (h + 1)) - 1ull);
  return top & ~((1ull << l) - 1ull);
}

// set voxels a..b (inclusive) in the pair-major bitmap: voxel v = 2p + h is bit (p % 32) + 32 h
// of 64-bit word p / 32
__device__ __forceinline__ void set_bits(uint32_t* flags, long a, long b) {
  unsigned long long* f = reinterpret_cast<unsigned long long*>(flags);
  const long e_lo = (a + 1) >> 1, e_hi = b >> 1;          // even voxels 2p in [a, b]
  const long o_lo = a >> 1, o_hi = (b - 1) >> 1;          // odd voxels 2p + 1 in [a, b]
  for (long q = (a >> 1) / 32; q <= (b >> 1) / 32; ++q) {
    const unsigned long long m = bit_range(e_lo, e_hi, q) | (bit_range(o_lo, o_hi, q) << 32);
    if (m) atomicOr(f + q, m);
  }
}


// Sphere painting (update_sphere_kernel, find_bubbles.cu:73-102), one warp per centre: every cell
// within integer |d|^2 <= r2max of voxel v (linear index, x fastest) is set in the pair-major
// bitmap; lanes split the (dz, dy) rows of the ball; periodic wraps, otherwise clips to the box.
__device__ __forceinline__ void paint_ball(uint32_t v, int n, int r2max, int periodic, uint32_t* flags) {
  const int lane = threadIdx.x & 31;
  const int r = isqrt_dev(r2max), side = 2 * r + 1;
  const int cx = (int)(v % n), cy = (int)((v / n) % n), cz = (int)(v / ((uint32_t)n * n));
  for (int idx = lane; idx < side * side; idx += 32) {
    const int dz = idx / side - r, dy = idx % side - r;
    const int rem = r2max - dz * dz - dy * dy;
    if (rem < 0) continue;
    const int w = isqrt_dev(rem);
    int z = cz + dz, y = cy + dy;
    if (periodic) { z = ((z % n) + n) % n; y = ((y % n) + n) % n; }
    else if (z < 0 || z >= n || y < 0 || y >= n) continue;
    const long rb = ((long)z * n + y) * n;
    int x0 = cx - w, x1 = cx + w;
    if (periodic) {
      if (x1 - x0 + 1 >= n) { set_bits(flags, rb, rb + n - 1); continue; }
      if (x0 < 0) { set_bits(flags, rb + x0 + n, rb + n - 1); x0 = 0; }
      if (x1 >= n) { set_bits(flags, rb, rb + x1 - n); x1 = n - 1; }
    } else {
      if (x0 < 0) x0 = 0;
      if (x1 > n - 1) x1 = n - 1;
    }
    set_bits(flags, rb + x0, rb + x1);
  }
}

template <int N> __device__ __forceinline__ int wrap2(int k) {
  const int w = (k > N / 2) ? k - N : k;
  return w * w;
}

// P(k) bins are kept per warp in shared memory as [3][PK_MAX_BINS]: the sums of k^3 |G|^2 / (2 pi^2 V)
// and of |k| as float, and the mode counts (weights 1 or 2) as exact unsigned integers in the
// third row (a bin of a 512^3 box holds more than 2^24 modes, beyond float32's exact integers).
__device__ __forceinline__ unsigned* pk_counts(float* bins) { return reinterpret_cast<unsigned*>(bins) + 2 * PK_MAX_BINS; }

// Per-CTA bins (fixed warp order) -> partials -> the last CTA to arrive adds the partials in a
// fixed order and writes ps_ave, k_ave and the count (rounded to float32 once, at the end).
template <int T>
__device__ __forceinline__ void pk_finish(float* bins, const OpArgs& a) {
  __syncthreads();
  const int nb3 = 3 * a.nbins;
  for (int idx = threadIdx.x; idx < nb3; idx += T) {
    const int q = idx / a.nbins, bin = idx % a.nbins;
    if (q < 2) {
      float s = 0.f;
      for (int w = 0; w < T / 32; ++w) s += bins[w * PK_MAX_BINS * 3 + q * PK_MAX_BINS + bin];
      a.partials[(size_t)blockIdx.x * nb3 + idx] = s;
    } else {
      unsigned s = 0u;
      for (int w = 0; w < T / 32; ++w) s += pk_counts(bins + w * PK_MAX_BINS * 3)[bin];
      a.partials[(size_t)blockIdx.x * nb3 + idx] = __uint_as_float(s);
    }
  }
  __shared__ unsigned s_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = (atomicAdd(a.counter, 1u) == gridDim.x - 1) ? 1u : 0u;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  // One warp per value: lanes stride over the CTAs' partials (32 loads in flight instead of one
  // dependent chain per thread), then a fixed butterfly: deterministic
  float* tot = bins;                                  // reuse: [3 * nbins]
  const int lane = threadIdx.x & 31;
  for (int idx = threadIdx.x >> 5; idx < nb3; idx += T / 32) {
    if (idx < 2 * a.nbins) {
      float s = 0.f;
      for (int b = lane; b < (int)gridDim.x; b += 32) s += __ldcg(a.partials + (size_t)b * nb3 + idx);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) tot[idx] = s;
    } else {
      unsigned long long s = 0ull;
      for (int b = lane; b < (int)gridDim.x; b += 32) s += __float_as_uint(__ldcg(a.partials + (size_t)b * nb3 + idx));
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) tot[idx] = __ull2float_rn(s);
    }
  }
  __syncthreads();
  for (int bin = threadIdx.x; bin < a.nbins; bin += T) {
    const float n = tot[2 * a.nbins + bin];
    a.pk_out[bin] = n > 0.f ? tot[bin] / n : 0.f;                        // ps_ave
    a.pk_out[a.nbins + bin] = n > 0.f ? tot[a.nbins + bin] / n : 0.f;    // k_ave
    a.pk_out[2 * a.nbins + bin] = n;                                     // count
  }
  if (threadIdx.x == 0) *a.counter = 0u;
}

// ------------------------------------------------------------------ column passes (y or z)
template <int N> struct ColCfg;
template <> struct ColCfg<16>  { static constexpr int TI = 8,  T = 64; };
template <> struct ColCfg<32>  { static constexpr int TI = 16, T = 128; };
template <> struct ColCfg<48>  { static constexpr int TI = 8,  T = 128; };
template <> struct ColCfg<64>  { static constexpr int TI = 16, T = 128; };
template <> struct ColCfg<96>  { static constexpr int TI = 16, T = 256; };
template <> struct ColCfg<128> { static constexpr int TI = 16, T = 256; };
template <> struct ColCfg<160> { static constexpr int TI = 16, T = 256; };
template <> struct ColCfg<256> { static constexpr int TI = 16, T = 256; };
template <> struct ColCfg<512> { static constexpr int TI = 8,  T = 256; };
template <> struct ColCfg<1024> { static constexpr int TI = 4, T = 256; };

template <int N, int MODE> struct ColSmem {
  static constexpr int TI = ColCfg<N>::TI, T = ColCfg<N>::T;
  static constexpr int fft_bytes = (N + 2 * N * TI) * 8;
  static constexpr int pk_bytes = (MODE == COL_Z_FWD_PK)
      ? ((T / 32) * PK_MAX_BINS * 3 + (T / 32) * 32 * 4 + PK_MAX_BINS) * 4 : 0;
  static constexpr int bytes = fft_bytes + pk_bytes;
};

template <int N, int MODE>
__global__ void __launch_bounds__(ColCfg<N>::T) col_pass(OpArgs a) {
  constexpr int M = N / 2;
  constexpr int TI = ColCfg<N>::TI, T = ColCfg<N>::T;
  constexpr bool INV = (MODE == COL_Z_INV_FILTER || MODE == COL_Y_INV || MODE == COL_Z_INV);
  constexpr bool ZPASS = (MODE == COL_Z_FWD || MODE == COL_Z_INV_FILTER || MODE == COL_Z_FWD_PK || MODE == COL_Z_INV);
  constexpr int CPR = M / TI;
  static_assert(M % TI == 0 && N % TI == 0, "tile width must divide N/2");
  const int nmain = N * CPR;
  const int ntiles = ZPASS ? nmain + N / TI : nmain;

  extern __shared__ float4 smem4[];
  float2* tw = reinterpret_cast<float2*>(smem4);
  float2* A = tw + N;
  float2* B = A + N * TI;
  float* bins = reinterpret_cast<float*>(B + N * TI);          // [warps][3][PK_MAX_BINS]
  float* scratch = bins + (T / 32) * PK_MAX_BINS * 3;          // [warps][32][4]
  int* sthr = reinterpret_cast<int*>(scratch + (T / 32) * 32 * 4);
  __shared__ float sred[T / 32];

  for (int i = threadIdx.x; i < N; i += T) tw[i] = a.tw[i];
  if (MODE == COL_Z_FWD_PK) {
    for (int i = threadIdx.x; i < (T / 32) * PK_MAX_BINS * 3; i += T) bins[i] = 0.f;
    for (int i = threadIdx.x; i < a.nbins; i += T) sthr[i] = a.thr[i];
  }
  __syncthreads();

  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    // ---- addressing of this tile: TI columns, N elements along the transform axis
    bool nyq_tile = false;
    int c = 0, plane = 0;
    size_t off;
    size_t es_g;
    if (ZPASS) {
      if (tile < nmain) { plane = tile / CPR; c = tile % CPR; off = (size_t)plane * M + c * TI; es_g = (size_t)N * M; }
      else { nyq_tile = true; c = tile - nmain; off = (size_t)c * TI; es_g = N; }
    } else {
      plane = tile / CPR; c = tile % CPR; off = (size_t)plane * N * M + c * TI; es_g = M;
    }
    const float2* src = nyq_tile ? a.cin_nyq : a.cin;
    // ---- load (+ filter)
    for (int e = threadIdx.x; e < N * TI; e += T) {
      const int row = e / TI, col = e % TI;
      float2 v = src[off + row * es_g + col];
      if (MODE == COL_Z_INV_FILTER) {
        int k2;
        if (!nyq_tile) { const int kx = c * TI + col; k2 = wrap2<N>(row) + wrap2<N>(plane) + kx * kx; }
        else { k2 = wrap2<N>(row) + wrap2<N>(c * TI + col) + M * M; }
        v = cscale(v, __ldg(a.wtab + k2) * a.scale);
      }
      A[e] = v;
    }
    if (MODE == COL_Y_INV && c == 0) {
      // pack the Hermitian columns i = 0 and i = N/2: u = y0 + i * yM
      __syncthreads();
      for (int j = threadIdx.x; j < N; j += T) {
        const float2 y0 = A[j * TI];
        const float2 ym = a.cin_nyq[(size_t)plane * N + j];
        A[j * TI] = make_float2(y0.x - ym.y, y0.y + ym.x);
      }
    }
    __syncthreads();
    float2* Rr = fft_lines<N, INV, TI, T, true, TI, 1, N>(A, B, tw);

    if (MODE == COL_Z_FWD_PK) {
      // ---- spherical binning of k^3 |G|^2 / (2 pi^2 V), |k| and counts, warp-aggregated
      const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
      float* wb = bins + warp * PK_MAX_BINS * 3;
      float* ws = scratch + warp * 32 * 4;
      const float inv = 1.0f / (2.0f * 9.8696044010893586f * a.volume);
      for (int e = threadIdx.x; e < N * TI; e += T) {      // whole warps iterate together
        const int row = e / TI, col = e % TI;
        int k2;
        float wgt;
        if (!nyq_tile) { const int kx = c * TI + col; k2 = wrap2<N>(row) + wrap2<N>(plane) + kx * kx; wgt = kx == 0 ? 1.f : 2.f; }
        else { k2 = wrap2<N>(row) + wrap2<N>(c * TI + col) + M * M; wgt = 1.f; }
        int lo = 0, hi = a.nbins;                           // first bin with k2 <= thr[bin]
        while (lo < hi) { const int mid = (lo + hi) >> 1; if (k2 <= sthr[mid]) hi = mid; else lo = mid + 1; }
        int bin = lo;
        if (k2 == 0) bin = a.nbins;                           // the mean (k = 0) is excluded
        const float2 g = Rr[e];
        const float km = a.dk * sqrtf((float)k2);
        ws[lane * 4 + 0] = wgt * km * km * km * (g.x * g.x + g.y * g.y) * inv;
        ws[lane * 4 + 1] = wgt * km;
        reinterpret_cast<unsigned*>(ws)[lane * 4 + 2] = (unsigned)wgt;
        const unsigned peers = __match_any_sync(0xffffffffu, bin);
        __syncwarp();
        if (bin < a.nbins && lane == __ffs(peers) - 1) {
          float p = 0.f, k = 0.f;
          unsigned n = 0u;
          unsigned m = peers;
          while (m) {
            const int l = __ffs(m) - 1;
            m &= m - 1;
            p += ws[l * 4 + 0]; k += ws[l * 4 + 1]; n += reinterpret_cast<const unsigned*>(ws)[l * 4 + 2];
          }
          wb[bin] += p; wb[PK_MAX_BINS + bin] += k; pk_counts(wb)[bin] += n;
        }
        __syncwarp();
      }
    } else if (MODE == COL_Y_FWD && c == 0) {
      // split the packed column 0: A = FFT(x0) -> main column 0, B = FFT(xM) -> nyq plane
      for (int e = threadIdx.x; e < N * TI; e += T) {
        const int row = e / TI, col = e % TI;
        if (col == 0) {
          const float2 v = Rr[row * TI];
          const float2 w = Rr[((N - row) % N) * TI];
          a.cout[off + row * es_g] = make_float2(0.5f * (v.x + w.x), 0.5f * (v.y - w.y));
          a.cout_nyq[(size_t)plane * N + row] = make_float2(0.5f * (v.y + w.y), -0.5f * (v.x - w.x));
        } else {
          a.cout[off + row * es_g + col] = Rr[e];
        }
      }
    } else {
      float2* dst = nyq_tile ? a.cout_nyq : a.cout;
      for (int e = threadIdx.x; e < N * TI; e += T) {
        const int row = e / TI, col = e % TI;
        dst[off + row * es_g + col] = Rr[e];
      }
    }
    __syncthreads();
  }

  if (MODE == COL_Z_FWD_PK) pk_finish<T>(bins, a);
  (void)sred;
}

// ------------------------------------------------------------------ row passes (x)
template <int N> struct RowCfg;
template <> struct RowCfg<16>  { static constexpr int RL = 16, T = 64; };
template <> struct RowCfg<32>  { static constexpr int RL = 16, T = 128; };
template <> struct RowCfg<48>  { static constexpr int RL = 8,  T = 128; };
template <> struct RowCfg<64>  { static constexpr int RL = 8,  T = 128; };
template <> struct RowCfg<96>  { static constexpr int RL = 8,  T = 128; };
template <> struct RowCfg<128> { static constexpr int RL = 8,  T = 256; };
template <> struct RowCfg<160> { static constexpr int RL = 8,  T = 256; };
template <> struct RowCfg<256> { static constexpr int RL = 8,  T = 256; };
template <> struct RowCfg<512> { static constexpr int RL = 4,  T = 256; };
template <> struct RowCfg<1024> { static constexpr int RL = 2, T = 256; };

template <int N> struct RowSmem {
  static constexpr int bytes = (N + 2 * RowCfg<N>::RL * (N / 2)) * 8;
};

// Real rows -> half spectrum rows (main layout; slot 0 holds (X[0], X[N/2]), both real).
template <int N, int PRO>
__global__ void __launch_bounds__(RowCfg<N>::T) row_r2c(OpArgs a) {
  constexpr int M = N / 2, RL = RowCfg<N>::RL, T = RowCfg<N>::T;
  static_assert((RL * N) % 64 == 0, "row tile must cover whole 64-voxel flag pairs");
  extern __shared__ float4 smem4[];
  float2* tw = reinterpret_cast<float2*>(smem4);
  float2* A = tw + N;
  float2* B = A + RL * M;
  for (int i = threadIdx.x; i < N; i += T) tw[i] = a.tw[i];
  float s = a.scale, sh = 0.f;
  if (PRO == PRO_PK) {
    const float ave = *a.ave;
    // g = (x / ave - 1) V / N^3  (delta_T.py:80-82), optionally times ave
    s = a.pk_norm / ave;
    sh = -a.pk_norm;
    if (a.dimensional) { s *= ave; sh *= ave; }
  }
  __syncthreads();
  const int ntiles = N * N / RL;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const size_t base = (size_t)tile * RL * M;
    for (int e = threadIdx.x; e < RL * M; e += T) {
      float2 v = a.rin[base + e];
      if (PRO == PRO_PK) v = make_float2(fmaf(v.x, s, sh), fmaf(v.y, s, sh));
      else v = cscale(v, s);
      A[e] = v;
    }
    __syncthreads();
    float2* Z = fft_lines<M, false, RL, T, false, 1, M, N>(A, B, tw);
    for (int q = threadIdx.x; q < RL * (M / 2 + 1); q += T) {
      const int row = q / (M / 2 + 1), m = q % (M / 2 + 1);
      const float2* z = Z + row * M;
      float2* out = a.cout + base + (size_t)row * M;
      if (m == 0) {
        const float2 z0 = z[0];
        out[0] = make_float2(z0.x + z0.y, z0.x - z0.y);
      } else {
        const int m2 = M - m;
        const float2 zm = z[m], zc = z[m2];
        {
          const float2 t = cmul(tw[m], make_float2(zm.x - zc.x, zm.y + zc.y));   // w^m (Zm - conj Zc)
          out[m] = make_float2(0.5f * (zm.x + zc.x + t.y), 0.5f * (zm.y - zc.y - t.x));
        }
        if (m2 != m) {
          const float2 t = cmul(tw[m2], make_float2(zc.x - zm.x, zc.y + zm.y));
          out[m2] = make_float2(0.5f * (zc.x + zm.x + t.y), 0.5f * (zc.y - zm.y - t.x));
        }
      }
    }
    __syncthreads();
  }
}

// Half spectrum rows -> real rows, with the excursion-set epilogue.
template <int N, int EPI>
__global__ void __launch_bounds__(RowCfg<N>::T) row_c2r(OpArgs a) {
  constexpr int M = N / 2, RL = RowCfg<N>::RL, T = RowCfg<N>::T;
  static_assert((RL * N) % 64 == 0, "row tile must cover whole 64-voxel flag pairs");
  static_assert((RL * M) % 32 == 0 && T % 32 == 0, "whole warps per row tile");
  extern __shared__ float4 smem4[];
  float2* tw = reinterpret_cast<float2*>(smem4);
  float2* A = tw + N;
  float2* B = A + RL * M;
  __shared__ float sred[T / 32];
  for (int i = threadIdx.x; i < N; i += T) tw[i] = a.tw[i];
  // The previous radius' test erfc((dc - d) / denom_prev) * norm_prev >= 1/zeta is monotone in d:
  // it holds exactly when d >= dc - denom_prev * erfcinv(1 / (zeta * norm_prev)), one scalar per
  // radius instead of an erfc per cell.
  float thr_prev = __int_as_float(0x7f800000);          // +inf: nothing passes
  if (EPI == EPI_IONIZE && a.has_prev) {
    const float y = a.inv_zeta / a.stats_prev[2];
    if (y < 2.0f) thr_prev = a.dc - a.denom_prev * erfcinvf(y);
  }
  const float dc = a.dc, inv_denom = 1.0f / a.denom;
  float acc = 0.f;
  const int lane = threadIdx.x & 31;
  __syncthreads();
  const int ntiles = N * N / RL;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const size_t base = (size_t)tile * RL * M;
    for (int e = threadIdx.x; e < RL * M; e += T) A[e] = a.cin[base + e];
    __syncthreads();
    for (int q = threadIdx.x; q < RL * (M / 2 + 1); q += T) {
      const int row = q / (M / 2 + 1), m = q % (M / 2 + 1);
      float2* x = A + row * M;
      if (m == 0) {
        const float2 x0 = x[0];                       // (X[0], X[N/2]), both real
        x[0] = make_float2(x0.x + x0.y, x0.x - x0.y);
      } else {
        const int m2 = M - m;
        const float2 xm = x[m], xc = x[m2];
        // Z[m] = (Xm + conj Xc) + i w^-m (Xm - conj Xc)
        const float2 t1 = cmul(cconj(tw[m]), make_float2(xm.x - xc.x, xm.y + xc.y));
        x[m] = make_float2(xm.x + xc.x - t1.y, xm.y - xc.y + t1.x);
        if (m2 != m) {
          const float2 t2 = cmul(cconj(tw[m2]), make_float2(xc.x - xm.x, xc.y + xm.y));
          x[m2] = make_float2(xc.x + xm.x - t2.y, xc.y - xm.y + t2.x);
        }
      }
    }
    __syncthreads();
    float2* Zr = fft_lines<M, true, RL, T, false, 1, M, N>(A, B, tw);
    if (EPI == EPI_STORE) {
      for (int e = threadIdx.x; e < RL * M; e += T) a.rout[base + e] = Zr[e];
    } else {
      for (int e = threadIdx.x; e < RL * M; e += T) {   // whole warps: 64 consecutive voxels
        const float2 d = Zr[e];
        acc += erfcf((dc - d.x) * inv_denom) + erfcf((dc - d.y) * inv_denom);
        if (a.has_prev) {
          const float2 p = a.prev[base + e];
          const bool px = p.x >= thr_prev;
          const bool py = p.y >= thr_prev;
          const unsigned bx = __ballot_sync(0xffffffffu, px);
          const unsigned by = __ballot_sync(0xffffffffu, py);
          if (a.update == 0) {
            if (lane == 0 && (bx | by))
              atomicOr(reinterpret_cast<unsigned long long*>(a.flags) + (base + e) / 32,
                       ((unsigned long long)by << 32) | bx);
          } else if (bx | by) {
            const unsigned cnt = __popc(bx) + __popc(by);
            unsigned first = 0;
            if (lane == 0) first = atomicAdd(a.center_count, cnt);
            first = __shfl_sync(0xffffffffu, first, 0);
            const unsigned lt = (1u << lane) - 1u;
            const unsigned v0 = (unsigned)((base + e) * 2);
            unsigned pos = first + __popc(bx & lt) + __popc(by & lt);
            if (px) a.centers[pos++] = v0;
            if (py) a.centers[pos] = v0 + 1;
          }
        }
        a.rout[base + e] = d;
      }
    }
    __syncthreads();
  }
  if (EPI == EPI_IONIZE) {
    float total;
    if (grid_sum<T>(acc, a.partials, a.counter, sred, &total) && threadIdx.x == 0) {
      const float mean = total / ((float)N * (float)N * (float)N);
      a.stats_out[0] = total;
      a.stats_out[1] = mean;
      a.stats_out[2] = a.normalize ? a.fc_mean / mean : 1.f;
    }
  }
}

}  // namespace es
