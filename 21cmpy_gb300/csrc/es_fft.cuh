// Shared-memory FFT building blocks for the excursion-set engine (sm_103a).
//
// Line transforms are mixed-radix Stockham (autosort) FFTs over lines held in shared memory:
// stage s with radix R reads x[j + r n/R], twiddles by w_{Ns R}^{(j mod Ns) r}, applies an
// R-point DFT in registers and writes to ((j / Ns) Ns R + j mod Ns) + r Ns.  Twiddles come from a
// table of w_n^m = exp(-2 pi i m / n) computed in float64 on the host, so no device
// trigonometry is involved in the transforms.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace es {

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// multiply by -i for a forward transform, +i for an inverse one
template <bool INV> __device__ __forceinline__ float2 rot(float2 a) {
  return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}
// multiply by w = (c, s) for the forward sign convention, conj(w) for the inverse one
template <bool INV> __device__ __forceinline__ float2 twid(float2 a, float c, float s) {
  return INV ? make_float2(a.x * c + a.y * s, a.y * c - a.x * s)
             : make_float2(a.x * c - a.y * s, a.y * c + a.x * s);
}

// ---------------------------------------------------------------- R-point DFTs in registers
template <int R, bool INV> struct Dft;

template <bool INV> struct Dft<2, INV> {
  static __device__ __forceinline__ void run(float2* v) {
    float2 a = v[0], b = v[1];
    v[0] = cadd(a, b); v[1] = csub(a, b);
  }
};

template <bool INV> struct Dft<3, INV> {
  static __device__ __forceinline__ void run(float2* v) {
    const float h = 0.86602540378443865f;            // sin(2 pi / 3)
    float2 t = cadd(v[1], v[2]);
    float2 d = csub(v[1], v[2]);
    float2 a = make_float2(v[0].x - 0.5f * t.x, v[0].y - 0.5f * t.y);
    float2 b = rot<INV>(cscale(d, h));
    v[0] = cadd(v[0], t);
    v[1] = cadd(a, b);
    v[2] = csub(a, b);
  }
};

template <bool INV> struct Dft<4, INV> {
  static __device__ __forceinline__ void run(float2* v) {
    float2 s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
    float2 s13 = cadd(v[1], v[3]), d13 = rot<INV>(csub(v[1], v[3]));
    v[0] = cadd(s02, s13); v[2] = csub(s02, s13);
    v[1] = cadd(d02, d13); v[3] = csub(d02, d13);
  }
};

template <bool INV> struct Dft<5, INV> {
  static __device__ __forceinline__ void run(float2* v) {
    const float c1 = 0.30901699437494745f, c2 = -0.80901699437494734f;   // cos(2pi/5), cos(4pi/5)
    const float s1 = 0.95105651629515353f, s2 = 0.58778525229247325f;    // sin(2pi/5), sin(4pi/5)
    float2 t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
    float2 d1 = csub(v[1], v[4]), d2 = csub(v[2], v[3]);
    float2 a1 = make_float2(v[0].x + c1 * t1.x + c2 * t2.x, v[0].y + c1 * t1.y + c2 * t2.y);
    float2 a2 = make_float2(v[0].x + c2 * t1.x + c1 * t2.x, v[0].y + c2 * t1.y + c1 * t2.y);
    float2 b1 = rot<INV>(make_float2(s1 * d1.x + s2 * d2.x, s1 * d1.y + s2 * d2.y));
    float2 b2 = rot<INV>(make_float2(s2 * d1.x - s1 * d2.x, s2 * d1.y - s1 * d2.y));
    v[0] = cadd(v[0], cadd(t1, t2));
    v[1] = cadd(a1, b1); v[4] = csub(a1, b1);
    v[2] = cadd(a2, b2); v[3] = csub(a2, b2);
  }
};

// radix-8 = two radix-4 DFTs of the even/odd samples combined with w_8^k
template <bool INV> struct Dft<8, INV> {
  static __device__ __forceinline__ void run(float2* v) {
    const float r = 0.70710678118654752f;
    float2 e[4] = {v[0], v[2], v[4], v[6]};
    float2 o[4] = {v[1], v[3], v[5], v[7]};
    Dft<4, INV>::run(e);
    Dft<4, INV>::run(o);
    o[1] = twid<INV>(o[1], r, -r);
    o[2] = rot<INV>(o[2]);
    o[3] = twid<INV>(o[3], -r, -r);
#pragma unroll
    for (int k = 0; k < 4; ++k) { v[k] = cadd(e[k], o[k]); v[k + 4] = csub(e[k], o[k]); }
  }
};

// radix-16 = two radix-8 DFTs combined with w_16^k
template <bool INV> struct Dft<16, INV> {
  static __device__ __forceinline__ void run(float2* v) {
    const float c1 = 0.92387953251128674f, s1 = 0.38268343236508978f;   // cos, sin(pi/8)
    const float r = 0.70710678118654752f;
    float2 e[8], o[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) { e[k] = v[2 * k]; o[k] = v[2 * k + 1]; }
    Dft<8, INV>::run(e);
    Dft<8, INV>::run(o);
    o[1] = twid<INV>(o[1], c1, -s1);
    o[2] = twid<INV>(o[2], r, -r);
    o[3] = twid<INV>(o[3], s1, -c1);
    o[4] = rot<INV>(o[4]);
    o[5] = twid<INV>(o[5], -s1, -c1);
    o[6] = twid<INV>(o[6], -r, -r);
    o[7] = twid<INV>(o[7], -c1, -s1);
#pragma unroll
    for (int k = 0; k < 8; ++k) { v[k] = cadd(e[k], o[k]); v[k + 8] = csub(e[k], o[k]); }
  }
};

// ---------------------------------------------------------------- radix plans per line length
// RS selects the radix schedule: 0 = fewest stages (radix up to 16), 1 = radices up to 8 (one more
// stage where that differs; smaller butterflies, fewer registers per thread).
template <int N, int RS = 0> struct Plan;
#define ES_PLAN(NN, RSV, ...)                                              \
  template <> struct Plan<NN, RSV> {                                       \
    static constexpr int radix[] = {__VA_ARGS__};                          \
    static constexpr int stages = sizeof(radix) / sizeof(int);             \
  };
ES_PLAN(8, 0, 8)
ES_PLAN(16, 0, 16)
ES_PLAN(24, 0, 8, 3)
ES_PLAN(32, 0, 8, 4)
ES_PLAN(48, 0, 16, 3)
ES_PLAN(64, 0, 8, 8)
ES_PLAN(80, 0, 16, 5)
ES_PLAN(96, 0, 8, 4, 3)
ES_PLAN(128, 0, 16, 8)
ES_PLAN(160, 0, 8, 4, 5)
ES_PLAN(256, 0, 16, 16)
ES_PLAN(512, 0, 8, 8, 8)
ES_PLAN(1024, 0, 16, 8, 8)
ES_PLAN(8, 1, 4, 2)
ES_PLAN(16, 1, 4, 4)
ES_PLAN(24, 1, 8, 3)
ES_PLAN(32, 1, 4, 8)
ES_PLAN(48, 1, 4, 4, 3)
ES_PLAN(64, 1, 4, 4, 4)
ES_PLAN(80, 1, 4, 4, 5)
ES_PLAN(96, 1, 8, 4, 3)
ES_PLAN(128, 1, 8, 4, 4)
ES_PLAN(160, 1, 8, 4, 5)
ES_PLAN(256, 1, 8, 8, 4)
ES_PLAN(512, 1, 8, 8, 8)
ES_PLAN(1024, 1, 8, 8, 4, 4)
#undef ES_PLAN

template <int N, int S, int RS = 0> struct StageNs {      // product of the radices before stage S
  static constexpr int value = StageNs<N, S - 1, RS>::value * Plan<N, RS>::radix[S - 1];
};
template <int N, int RS> struct StageNs<N, 0, RS> { static constexpr int value = 1; };

// Lines of length N in shared memory: element e of line l at buf[l * LS + e * ES].
// LINE_FAST maps consecutive threads to consecutive lines (column tiles), otherwise to
// consecutive butterflies of one line (row tiles).  tw[m] = w_TWN^m with TWN a multiple of N.
template <int N, int S, bool INV, int NL, int T, bool LINE_FAST, int ES, int LS, int TWN, int RS = 0>
__device__ __forceinline__ void stockham_stage(const float2* __restrict__ in, float2* __restrict__ out,
                                               const float2* __restrict__ tw) {
  constexpr int R = Plan<N, RS>::radix[S];
  constexpr int Ns = StageNs<N, S, RS>::value;
  constexpr int NB = NL * (N / R);
  for (int b = threadIdx.x; b < NB; b += T) {
    int l, j;
    if (LINE_FAST) { l = b % NL; j = b / NL; } else { j = b % (N / R); l = b / (N / R); }
    const float2* src = in + l * LS;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = src[(j + r * (N / R)) * ES];
    if (Ns > 1) {
      const int k = j % Ns;
#pragma unroll
      for (int r = 1; r < R; ++r) {
        float2 w = tw[k * r * (TWN / (Ns * R))];
        v[r] = twid<INV>(v[r], w.x, w.y);
      }
    }
    Dft<R, INV>::run(v);
    float2* dst = out + l * LS;
    const int idxD = (j / Ns) * Ns * R + (j % Ns);
#pragma unroll
    for (int r = 0; r < R; ++r) dst[(idxD + r * Ns) * ES] = v[r];
  }
}

template <int N, int S, bool INV, int NL, int T, bool LINE_FAST, int ES, int LS, int TWN, int RS = 0,
          bool LAST = (S == Plan<N, RS>::stages)>
struct Stages {
  // runs stages S.. and returns the buffer that holds the result
  static __device__ __forceinline__ float2* run(float2* a, float2* b, const float2* tw) {
    stockham_stage<N, S, INV, NL, T, LINE_FAST, ES, LS, TWN, RS>(a, b, tw);
    __syncthreads();
    return Stages<N, S + 1, INV, NL, T, LINE_FAST, ES, LS, TWN, RS>::run(b, a, tw);
  }
};
template <int N, int S, bool INV, int NL, int T, bool LINE_FAST, int ES, int LS, int TWN, int RS>
struct Stages<N, S, INV, NL, T, LINE_FAST, ES, LS, TWN, RS, true> {
  static __device__ __forceinline__ float2* run(float2* a, float2*, const float2*) { return a; }
};

// Full line FFT, ping-ponging between a and b; the caller synchronises before it.
template <int N, bool INV, int NL, int T, bool LINE_FAST, int ES, int LS, int TWN, int RS = 0>
__device__ __forceinline__ float2* fft_lines(float2* a, float2* b, const float2* tw) {
  return Stages<N, 0, INV, NL, T, LINE_FAST, ES, LS, TWN, RS>::run(a, b, tw);
}

// bit spread: 16-bit x -> 32-bit word with x's bits at the even positions
__device__ __forceinline__ uint32_t spread16(uint32_t x) {
  x &= 0xFFFFu;
  x = (x | (x << 8)) & 0x00FF00FFu;
  x = (x | (x << 4)) & 0x0F0F0F0Fu;
  x = (x | (x << 2)) & 0x33333333u;
  x = (x | (x << 1)) & 0x55555555u;
  return x;
}

}  // namespace es
