// Batched excursion-set engine: many boxes of uneven HII_DIM (and their own zeta, R_mfp, T_vir,
// z) run in ONE persistent launch.  The host lists every box's passes (forward transform, three
// passes per radius, final step) level by level, interleaving the boxes; CTAs take tiles from a
// global ticket counter in that order.  A pass of a box starts once the box's previous pass has
// counted all its tiles done, so tiles only ever wait on tiles with smaller tickets, all held by
// resident CTAs: the queue cannot deadlock.  Every wait is bounded; a timeout raises the batch's
// error word and an abort flag that makes every CTA leave.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "es_engine.h"
#include "es_kernels.cuh"

namespace esb {
using namespace es;

constexpr int BT = 256;              // threads per CTA
constexpr int FINAL_PAIRS = 2048;    // voxel pairs per final-step tile
constexpr long kSpinLimit = 1L << 24;          // polls of 100 ns before a wait is declared hung
constexpr unsigned ES_DEV_ERR_BATCH_TIMEOUT = 2u;

enum BOp { B_ROW_R2C = 0, B_COL_Y_FWD = 1, B_COL_Z_FWD = 2, B_COL_Z_INV = 3, B_COL_Y_INV = 4, B_ROW_C2R = 5, B_FINAL = 6 };

struct RadB { float R, denom; int k2cut, pad; };

struct BoxDev {
  int n, n_radii, normalize, filter, ref_compat, output;
  float dk, dc, fc_mean, zeta, inv_zeta, growth, inv_n3, pad0;
  const float* delta;
  float* out;
  float* nf;
  float2 *X, *Xnyq, *T, *Tnyq;
  float *dR0, *dR1;
  unsigned long long* flags;
  const float2* tw;
  const RadB* rad;
  float* stats;          // [n_radii][4]: sum, mean, norm
  float* partials;       // per-tile partial sums of the reducing passes
  unsigned* arrive;      // [n_radii + 1] arrival counters
};

struct PassDesc { int box, op, radius, tiles, first, dep, need, pad; };   // need: done count awaited on dep

struct BatchArgs {
  const BoxDev* boxes;
  const PassDesc* passes;
  int npasses;
  unsigned total;
  unsigned* ticket;
  unsigned* done;
  unsigned* err;
  unsigned* abort;
  long spin_limit;
};

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

template <int N> struct BCol { static constexpr int TI = ColCfg<N>::TI; };
template <int N> struct BRow { static constexpr int RL = N >= 256 ? 8 : 16; };

template <int N> __host__ __device__ constexpr int col_tiles_z() { return N * ((N / 2) / BCol<N>::TI) + N / BCol<N>::TI; }
template <int N> __host__ __device__ constexpr int col_tiles_y() { return N * ((N / 2) / BCol<N>::TI); }
template <int N> __host__ __device__ constexpr int row_tiles() { return N * N / BRow<N>::RL; }
template <int N> __host__ __device__ constexpr int final_tiles() { return (N * N * (N / 2) + FINAL_PAIRS - 1) / FINAL_PAIRS; }
template <int N> __host__ __device__ constexpr int smem_bytes() {
  constexpr int col = (N + 2 * N * BCol<N>::TI) * 8;
  constexpr int row = (N + 2 * (N / 2) * (BRow<N>::RL + 1)) * 8;
  return col > row ? col : row;
}

__device__ float block_sum_b(float v, float* sred) { return block_sum<BT>(v, sred); }

// Deterministic per-box reduction: every tile publishes its partial, the last one sums them.
__device__ bool tile_reduce(float mine, float* partials, unsigned* arrive, int tile, int tiles, float* sred,
                            float* total) {
  __shared__ unsigned s_last;
  const float s = block_sum_b(mine, sred);
  if (threadIdx.x == 0) {
    partials[tile] = s;
    __threadfence();
    s_last = (atomicAdd(arrive, 1u) == (unsigned)tiles - 1) ? 1u : 0u;
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  float acc = 0.f;
  for (int i = threadIdx.x; i < tiles; i += BT) acc += __ldcg(partials + i);
  *total = block_sum_b(acc, sred);
  return true;
}

// ---------------------------------------------------------------- column tiles (y or z)
template <int N, int OP>
__device__ __noinline__ void b_col(const BoxDev& b, int radius, int tile, float2* sm) {
  constexpr int M = N / 2, TI = BCol<N>::TI, CPR = M / TI;
  constexpr bool INV = OP == B_COL_Z_INV || OP == B_COL_Y_INV;
  constexpr bool Z = OP == B_COL_Z_FWD || OP == B_COL_Z_INV;
  float2* tw = sm;
  float2* A = tw + N;
  float2* B = A + N * TI;
  for (int i = threadIdx.x; i < N; i += BT) tw[i] = __ldg(b.tw + i);
  bool nyq = false;
  int c, plane;
  size_t off, es_g;
  if (Z) {
    if (tile < N * CPR) { plane = tile / CPR; c = tile % CPR; off = (size_t)plane * M + c * TI; es_g = (size_t)N * M; }
    else { nyq = true; plane = 0; c = tile - N * CPR; off = (size_t)c * TI; es_g = N; }
  } else {
    plane = tile / CPR; c = tile % CPR; off = (size_t)plane * N * M + c * TI; es_g = M;
  }
  const float2* src = OP == B_COL_Z_INV ? (nyq ? b.Xnyq : b.X) : (nyq ? b.Tnyq : b.T);
  if (OP == B_COL_Y_FWD || OP == B_COL_Z_FWD) src = nyq ? b.Xnyq : b.X;
  float2* dst = OP == B_COL_Y_FWD || OP == B_COL_Z_FWD ? (nyq ? b.Xnyq : b.X) : (nyq ? b.Tnyq : b.T);
  // z inverse: W depends on |k|^2 = kz^2 + (the column's ky^2 + kx^2), N/2 + 1 distinct values per
  // column; they go into B (free until the transform) before the tile is loaded
  float* wcol = reinterpret_cast<float*>(B);
  if (OP == B_COL_Z_INV) {
    const RadB rd = b.rad[radius];
    const float sc = b.growth * b.inv_n3;
    for (int q = threadIdx.x; q < TI * (M + 1); q += BT) {
      const int col = q / (M + 1), kz = q % (M + 1);
      const int ck2 = !nyq ? wrap2<N>(plane) + (c * TI + col) * (c * TI + col) : wrap2<N>(c * TI + col) + M * M;
      wcol[q] = filter_weight(kz * kz + ck2, b.dk, rd.R, rd.k2cut, b.filter, b.ref_compat) * sc;
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < N * TI; e += BT) {
    const int row = e / TI, col = e % TI;
    float2 v = __ldcg(src + off + row * es_g + col);
    if (OP == B_COL_Z_INV) v = cscale(v, wcol[col * (M + 1) + (row > M ? N - row : row)]);
    A[e] = v;
  }
  if (OP == B_COL_Y_INV && c == 0) {
    __syncthreads();
    for (int j = threadIdx.x; j < N; j += BT) {
      const float2 y0 = A[j * TI];
      const float2 ym = __ldcg(b.Tnyq + (size_t)plane * N + j);
      A[j * TI] = make_float2(y0.x - ym.y, y0.y + ym.x);
    }
  }
  __syncthreads();
  float2* Rr = fft_lines<N, INV, TI, BT, true, TI, 1, N>(A, B, tw);
  if (OP == B_COL_Y_FWD && c == 0) {
    for (int e = threadIdx.x; e < N * TI; e += BT) {
      const int row = e / TI, col = e % TI;
      if (col == 0) {
        const float2 v = Rr[row * TI];
        const float2 w = Rr[((N - row) % N) * TI];
        dst[off + row * es_g] = make_float2(0.5f * (v.x + w.x), 0.5f * (v.y - w.y));
        b.Xnyq[(size_t)plane * N + row] = make_float2(0.5f * (v.y + w.y), -0.5f * (v.x - w.x));
      } else {
        dst[off + row * es_g + col] = Rr[e];
      }
    }
  } else {
    for (int e = threadIdx.x; e < N * TI; e += BT) {
      const int row = e / TI, col = e % TI;
      dst[off + row * es_g + col] = Rr[e];
    }
  }
}

// ---------------------------------------------------------------- row tiles (x), transposed layout
template <int N>
__device__ __noinline__ void b_row_r2c(const BoxDev& b, int tile, float2* sm) {
  constexpr int M = N / 2, RL = BRow<N>::RL, ES = RL + 1;
  float2* tw = sm;
  float2* A = tw + N;
  float2* B = A + M * ES;
  for (int i = threadIdx.x; i < N; i += BT) tw[i] = __ldg(b.tw + i);
  const size_t pair0 = (size_t)tile * RL * M;
  const float2* in = reinterpret_cast<const float2*>(b.delta) + pair0;
  for (int e = threadIdx.x; e < RL * M; e += BT) {
    const int row = e / M, p = e % M;
    A[p * ES + row] = __ldg(in + e);
  }
  __syncthreads();
  float2* Z = fft_lines<M, false, RL, BT, true, ES, 1, N>(A, B, tw);
  // item t of row l makes X[t] and X[M-t] (item 0: the packed (X[0], X[N/2]) and X[M/2])
  for (int q = threadIdx.x; q < RL * (M / 2); q += BT) {
    const int t = q % (M / 2), l = q / (M / 2);
    float2* out = b.X + pair0 + (size_t)l * M;
    if (t == 0) {
      const float2 z0 = Z[l];
      out[0] = make_float2(z0.x + z0.y, z0.x - z0.y);
      const float2 zh = Z[(M / 2) * ES + l];
      const float2 th = cmul(tw[M / 2], make_float2(0.f, zh.y + zh.y));
      out[M / 2] = make_float2(0.5f * (zh.x + zh.x + th.y), -0.5f * th.x);
    } else {
      const int m2 = M - t;
      const float2 zm = Z[t * ES + l], zc = Z[m2 * ES + l], w = tw[t];
      const float2 t1 = cmul(w, make_float2(zm.x - zc.x, zm.y + zc.y));
      out[t] = make_float2(0.5f * (zm.x + zc.x + t1.y), 0.5f * (zm.y - zc.y - t1.x));
      const float2 t2 = cmul(make_float2(-w.x, w.y), make_float2(zc.x - zm.x, zc.y + zm.y));   // w^(M-t)
      out[m2] = make_float2(0.5f * (zc.x + zm.x + t2.y), 0.5f * (zc.y - zm.y - t2.x));
    }
  }
}

template <int N>
__device__ __noinline__ void b_row_c2r(const BoxDev& b, int radius, int tile, float2* sm, float* sred) {
  constexpr int M = N / 2, RL = BRow<N>::RL, ES = RL + 1;
  float2* tw = sm;
  float2* A = tw + N;
  float2* B = A + M * ES;
  for (int i = threadIdx.x; i < N; i += BT) tw[i] = __ldg(b.tw + i);
  __syncthreads();                                        // the split below reads the twiddles
  const size_t pair0 = (size_t)tile * RL * M;
  const float2* src = b.T + pair0;
  // item t of row l makes Z[t] and Z[M-t] (item 0: Z[0] from (X[0], X[N/2]) and Z[M/2])
  for (int q = threadIdx.x; q < RL * (M / 2); q += BT) {
    const int t = q % (M / 2), l = q / (M / 2);
    const float2* x = src + (size_t)l * M;
    if (t == 0) {
      const float2 x0 = __ldcg(x), xh = __ldcg(x + M / 2);
      A[l] = make_float2(x0.x + x0.y, x0.x - x0.y);
      const float2 th = cmul(cconj(tw[M / 2]), make_float2(0.f, xh.y + xh.y));
      A[(M / 2) * ES + l] = make_float2(xh.x + xh.x - th.y, th.x);
    } else {
      const int m2 = M - t;
      const float2 xm = __ldcg(x + t), xc = __ldcg(x + m2), w = tw[t];
      const float2 t1 = cmul(cconj(w), make_float2(xm.x - xc.x, xm.y + xc.y));
      A[t * ES + l] = make_float2(xm.x + xc.x - t1.y, xm.y - xc.y + t1.x);
      const float2 t2 = cmul(make_float2(-w.x, -w.y), make_float2(xc.x - xm.x, xc.y + xm.y));   // conj w^(M-t)
      A[m2 * ES + l] = make_float2(xc.x + xm.x - t2.y, xc.y - xm.y + t2.x);
    }
  }
  __syncthreads();
  float2* Zr = fft_lines<M, true, RL, BT, true, ES, 1, N>(A, B, tw);
  const bool has_prev = radius > 0;
  float2* cur = reinterpret_cast<float2*>((radius & 1) ? b.dR1 : b.dR0);
  const float2* prv = reinterpret_cast<const float2*>((radius & 1) ? b.dR0 : b.dR1);
  float thr = __int_as_float(0x7f800000);
  if (has_prev) {
    const float y = b.inv_zeta / __ldcg(b.stats + 4 * (radius - 1) + 2);
    if (y < 2.0f) thr = b.dc - b.rad[radius - 1].denom * erfcinvf(y);
  }
  const float inv_denom = 1.0f / b.rad[radius].denom, dc = b.dc;
  const int lane = threadIdx.x & 31;
  float acc = 0.f;
  for (int e = threadIdx.x; e < RL * M; e += BT) {       // whole warps: 64 consecutive voxels
    const int row = e / M, p = e % M;
    const float2 d = Zr[p * ES + row];
    acc += erfc_sum_term((dc - d.x) * inv_denom) + erfc_sum_term((dc - d.y) * inv_denom);
    if (has_prev) {
      const float2 pp = __ldcg(prv + pair0 + e);
      const unsigned bx = __ballot_sync(0xffffffffu, pp.x >= thr);
      const unsigned by = __ballot_sync(0xffffffffu, pp.y >= thr);
      if (lane == 0 && (bx | by)) atomicOr(b.flags + (pair0 + e) / 32, ((unsigned long long)by << 32) | bx);
    }
    cur[pair0 + e] = d;
  }
  float total;
  if (tile_reduce(acc, b.partials, b.arrive + radius, tile, row_tiles<N>(), sred, &total) && threadIdx.x == 0) {
    const float mean = total * b.inv_n3;
    b.stats[4 * radius + 0] = total;
    b.stats[4 * radius + 1] = mean;
    b.stats[4 * radius + 2] = b.normalize ? b.fc_mean / mean : 1.f;
  }
}

template <int N>
__device__ __noinline__ void b_final(const BoxDev& b, int tile, float* sred) {
  const int last = b.n_radii - 1;
  const float2* dR = reinterpret_cast<const float2*>((last & 1) ? b.dR1 : b.dR0);
  const float norm = __ldcg(b.stats + 4 * last + 2), denom = b.rad[last].denom;
  const long pairs = (long)N * N * (N / 2);
  const long p0 = (long)tile * FINAL_PAIRS;
  float acc = 0.f;
  for (long p = p0 + threadIdx.x; p < p0 + FINAL_PAIRS && p < pairs; p += BT) {
    const float2 d = __ldcg(dR + p);
    const unsigned long long w = __ldcg(b.flags + p / 32);
    const int bit = (int)(p % 32);
    float ion[2];
    const float dv[2] = {d.x, d.y};
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      if ((w >> (bit + 32 * h)) & 1ull) { ion[h] = 1.0f; continue; }
      const float f = erfcf((b.dc - dv[h]) / denom) * norm;
      ion[h] = f >= b.inv_zeta ? 1.0f : f * b.zeta;
    }
    acc += (1.0f - ion[0]) + (1.0f - ion[1]);
    reinterpret_cast<float2*>(b.out)[p] =
        b.output == 0 ? make_float2(1.0f - ion[0], 1.0f - ion[1]) : make_float2(ion[0], ion[1]);
  }
  float total;
  if (tile_reduce(acc, b.partials, b.arrive + b.n_radii, tile, final_tiles<N>(), sred, &total) && threadIdx.x == 0)
    *b.nf = total * b.inv_n3;
}

template <int N>
__device__ __forceinline__ void run_item(const BoxDev& b, const PassDesc& pd, int tile, float2* sm, float* sred) {
  switch (pd.op) {
    case B_ROW_R2C: b_row_r2c<N>(b, tile, sm); break;
    case B_COL_Y_FWD: b_col<N, B_COL_Y_FWD>(b, 0, tile, sm); break;
    case B_COL_Z_FWD: b_col<N, B_COL_Z_FWD>(b, 0, tile, sm); break;
    case B_COL_Z_INV: b_col<N, B_COL_Z_INV>(b, pd.radius, tile, sm); break;
    case B_COL_Y_INV: b_col<N, B_COL_Y_INV>(b, pd.radius, tile, sm); break;
    case B_ROW_C2R: b_row_c2r<N>(b, pd.radius, tile, sm, sred); break;
    case B_FINAL: b_final<N>(b, tile, sred); break;
  }
}

#define ESB_SIZES(X) X(32) X(48) X(64) X(96) X(128) X(160) X(256)

__global__ void __launch_bounds__(BT) batch_kernel(BatchArgs g) {
  extern __shared__ float4 smem4[];
  float2* sm = reinterpret_cast<float2*>(smem4);
  __shared__ float sred[BT / 32];
  __shared__ unsigned s_t;
  __shared__ int s_go;
  for (;;) {
    if (threadIdx.x == 0) {
      s_t = *(volatile unsigned*)g.abort ? g.total : atomicAdd(g.ticket, 1u);
    }
    __syncthreads();
    const unsigned t = s_t;
    if (t >= g.total) break;
    int lo = 0, hi = g.npasses - 1;                       // pass holding ticket t
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if ((unsigned)g.passes[mid].first <= t) lo = mid; else hi = mid - 1;
    }
    const PassDesc pd = g.passes[lo];
    if (threadIdx.x == 0) {
      int go = 1;
      if (pd.dep >= 0) {
        const unsigned need = (unsigned)pd.need;
        long it = 0;
        while (ld_acquire(g.done + pd.dep) < need) {
          if (++it > g.spin_limit || *(volatile unsigned*)g.abort) { go = 0; break; }
          __nanosleep(100);
        }
        if (!go) { atomicOr(g.err, ES_DEV_ERR_BATCH_TIMEOUT); atomicExch(g.abort, 1u); }
      }
      s_go = go;
    }
    __syncthreads();
    if (!s_go) break;
    const BoxDev& b = g.boxes[pd.box];
    const int tile = (int)(t - (unsigned)pd.first);
    switch (b.n) {
#define ESB_CASE(NN) case NN: run_item<NN>(b, pd, tile, sm, sred); break;
      ESB_SIZES(ESB_CASE)
#undef ESB_CASE
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(g.done + lo, 1u);
  }
}

}  // namespace esb

// ------------------------------------------------------------------ host side
namespace {

thread_local std::string g_batch_error;

int bfail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_batch_error = buf;
  return code;
}

#define ESB_CUDA(call)                                                                         \
  do {                                                                                         \
    cudaError_t err__ = (call);                                                                \
    if (err__ != cudaSuccess) return bfail(ES_E_CUDA, "%s failed: %s", #call, cudaGetErrorString(err__)); \
  } while (0)

size_t a256(size_t x) { return (x + 255) / 256 * 256; }

template <int N> struct SizeInfo {
  static void get(int* ct_z, int* ct_y, int* rt, int* ft, int* smem) {
    *ct_z = esb::col_tiles_z<N>();
    *ct_y = esb::col_tiles_y<N>();
    *rt = esb::row_tiles<N>();
    *ft = esb::final_tiles<N>();
    *smem = esb::smem_bytes<N>();
  }
};

bool size_info(int n, int* ct_z, int* ct_y, int* rt, int* ft, int* smem) {
  switch (n) {
#define ESB_INFO(NN) case NN: SizeInfo<NN>::get(ct_z, ct_y, rt, ft, smem); return true;
    ESB_SIZES(ESB_INFO)
#undef ESB_INFO
    default: return false;
  }
}

}  // namespace

struct es_batch {
  int device = 0, count = 0, grid = 0, smem = 0;
  void* base = nullptr;
  esb::BoxDev* d_boxes = nullptr;
  esb::PassDesc* d_passes = nullptr;
  unsigned* ctrl = nullptr;          // [0] ticket, [1] err, [2] abort, then done[npasses]
  int npasses = 0;
  unsigned total = 0;
  size_t zero_bytes = 0;             // counters + arrive + flags cleared before every run
  void* zero_base = nullptr;
  cudaGraphExec_t graph = nullptr;
  long spin_limit = esb::kSpinLimit;
  std::vector<esb::PassDesc> h_passes;
};

extern "C" {

int es_batch_create(const es_batch_box* boxes, int count, es_batch** out) {
  if (!boxes || count <= 0 || !out) return bfail(ES_E_ARG, "es_batch_create: bad arguments");
  *out = nullptr;
  es_batch* bt = new es_batch();
  auto cleanup = [&](int code) { es_batch_destroy(bt); return code; };
  if (cudaGetDevice(&bt->device) != cudaSuccess) return cleanup(bfail(ES_E_CUDA, "no CUDA device"));
  bt->count = count;
  std::vector<esb::BoxDev> hb(count);
  std::vector<esb::PassDesc> passes;
  // sizes of every box's workspace
  struct Sz { size_t X, Xn, T, Tn, dR, flags, stats, partials, arrive, rad, tw; };
  std::vector<Sz> sz(count);
  size_t total_bytes = 0;
  int smem = 0;
  std::vector<std::vector<int>> levels(count);
  for (int i = 0; i < count; ++i) {
    const es_batch_box& bx = boxes[i];
    int ctz, cty, rt, ft, sm;
    if (!size_info(bx.n, &ctz, &cty, &rt, &ft, &sm))
      return cleanup(bfail(ES_E_UNSUPPORTED, "es_batch_create: box %d has HII_DIM=%d (batched sizes: 32..256)", i, bx.n));
    const es_ionize_params& p = bx.params;
    if (!bx.delta || !bx.out || !bx.nf || !p.radii || p.n_radii < 1 || p.n_radii > 4096)
      return cleanup(bfail(ES_E_ARG, "es_batch_create: box %d has a NULL buffer or bad radius count", i));
    if (p.update != 0) return cleanup(bfail(ES_E_ARG, "es_batch_create: box %d: the batched engine paints centres only (update=0)", i));
    if (!(p.zeta > 0) || p.filter_type < 0 || p.filter_type > 2)
      return cleanup(bfail(ES_E_ARG, "es_batch_create: box %d has bad parameters", i));
    smem = sm > smem ? sm : smem;
    const size_t N = bx.n, M = N / 2;
    Sz& s = sz[i];
    s.X = a256(N * N * M * 8); s.Xn = a256(N * N * 8); s.T = s.X; s.Tn = s.Xn;
    s.dR = a256(N * N * N * 4); s.flags = a256(N * N * N / 8); s.stats = a256((size_t)p.n_radii * 16);
    s.partials = a256((size_t)(rt > ft ? rt : ft) * 4); s.arrive = a256((size_t)(p.n_radii + 1) * 4);
    s.rad = a256((size_t)p.n_radii * sizeof(esb::RadB)); s.tw = a256(N * 8);
    total_bytes += s.X + s.Xn + s.T + s.Tn + 2 * s.dR + s.flags + s.stats + s.partials + s.arrive + s.rad + s.tw;
  }
  // passes, interleaved by level: forward (3), 3 per radius, final
  std::vector<std::vector<esb::PassDesc>> per_box(count);
  for (int i = 0; i < count; ++i) {
    int ctz, cty, rt, ft, sm;
    size_info(boxes[i].n, &ctz, &cty, &rt, &ft, &sm);
    auto& v = per_box[i];
    v.push_back({i, esb::B_ROW_R2C, 0, rt, 0, -1, 0, 0});
    v.push_back({i, esb::B_COL_Y_FWD, 0, cty, 0, -1, 0, 0});
    v.push_back({i, esb::B_COL_Z_FWD, 0, ctz, 0, -1, 0, 0});
    for (int r = 0; r < boxes[i].params.n_radii; ++r) {
      v.push_back({i, esb::B_COL_Z_INV, r, ctz, 0, -1, 0, 0});
      v.push_back({i, esb::B_COL_Y_INV, r, cty, 0, -1, 0, 0});
      v.push_back({i, esb::B_ROW_C2R, r, rt, 0, -1, 0, 0});
    }
    v.push_back({i, esb::B_FINAL, 0, ft, 0, -1, 0, 0});
  }
  size_t max_levels = 0;
  for (auto& v : per_box) max_levels = v.size() > max_levels ? v.size() : max_levels;
  std::vector<int> last(count, -1);
  unsigned first = 0;
  for (size_t l = 0; l < max_levels; ++l)
    for (int i = 0; i < count; ++i) {
      if (l >= per_box[i].size()) continue;
      esb::PassDesc d = per_box[i][l];
      d.first = (int)first;
      d.dep = last[i];
      d.need = last[i] >= 0 ? passes[last[i]].tiles : 0;
      first += d.tiles;
      last[i] = (int)passes.size();
      passes.push_back(d);
    }
  bt->npasses = (int)passes.size();
  bt->h_passes = passes;
  bt->total = first;
  bt->smem = smem;
  const size_t ctrl_bytes = a256((3 + passes.size()) * 4);
  const size_t box_bytes = a256(count * sizeof(esb::BoxDev)), pass_bytes = a256(passes.size() * sizeof(esb::PassDesc));
  total_bytes += ctrl_bytes + box_bytes + pass_bytes;
  if (cudaMalloc(&bt->base, total_bytes) != cudaSuccess) {
    cudaGetLastError();
    return cleanup(bfail(ES_E_NOMEM, "es_batch_create: cannot allocate %zu bytes", total_bytes));
  }
  // layout: control block first, then per-box zero-initialised parts, then the rest
  char* b = static_cast<char*>(bt->base);
  size_t off = 0;
  bt->ctrl = reinterpret_cast<unsigned*>(b);
  off += ctrl_bytes;
  bt->zero_base = b;
  std::vector<size_t> flags_off(count), arrive_off(count);
  for (int i = 0; i < count; ++i) { flags_off[i] = off; off += sz[i].flags; arrive_off[i] = off; off += sz[i].arrive; }
  bt->zero_bytes = off;
  bt->d_boxes = reinterpret_cast<esb::BoxDev*>(b + off); off += box_bytes;
  bt->d_passes = reinterpret_cast<esb::PassDesc*>(b + off); off += pass_bytes;
  for (int i = 0; i < count; ++i) {
    const es_batch_box& bx = boxes[i];
    const es_ionize_params& p = bx.params;
    const Sz& s = sz[i];
    esb::BoxDev& d = hb[i];
    std::memset(&d, 0, sizeof(d));
    d.n = bx.n; d.n_radii = p.n_radii; d.normalize = p.normalize_mean; d.filter = p.filter_type;
    d.ref_compat = p.ref_compat; d.output = p.output;
    d.dk = (float)(2.0 * M_PI / (double)(float)bx.box_len);
    d.dc = p.delta_c; d.fc_mean = p.fc_mean_ps; d.zeta = p.zeta; d.inv_zeta = (float)(1.0 / (double)p.zeta);
    d.growth = p.growth_scale; d.inv_n3 = (float)(1.0 / ((double)bx.n * bx.n * bx.n));
    d.delta = bx.delta; d.out = bx.out; d.nf = bx.nf;
    d.X = reinterpret_cast<float2*>(b + off); off += s.X;
    d.Xnyq = reinterpret_cast<float2*>(b + off); off += s.Xn;
    d.T = reinterpret_cast<float2*>(b + off); off += s.T;
    d.Tnyq = reinterpret_cast<float2*>(b + off); off += s.Tn;
    d.dR0 = reinterpret_cast<float*>(b + off); off += s.dR;
    d.dR1 = reinterpret_cast<float*>(b + off); off += s.dR;
    d.flags = reinterpret_cast<unsigned long long*>(b + flags_off[i]);
    d.arrive = reinterpret_cast<unsigned*>(b + arrive_off[i]);
    d.stats = reinterpret_cast<float*>(b + off); off += s.stats;
    d.partials = reinterpret_cast<float*>(b + off); off += s.partials;
    esb::RadB* rad = reinterpret_cast<esb::RadB*>(b + off); off += s.rad;
    float2* tw = reinterpret_cast<float2*>(b + off); off += s.tw;
    d.rad = rad; d.tw = tw;
    std::vector<esb::RadB> hr(p.n_radii);
    for (int r = 0; r < p.n_radii; ++r) {
      const float R = p.radii[r].R, den = p.radii[r].denom;
      if (!(R > 0) || !(den > 0)) return cleanup(bfail(ES_E_ARG, "es_batch_create: box %d radius %d invalid", i, r));
      hr[r].R = R; hr[r].denom = den; hr[r].pad = 0;
      hr[r].k2cut = 0x7fffffff;
      if (p.filter_type == 1 || (p.ref_compat && p.filter_type == 0)) {
        const double dk = d.dk;
        const long k2n = 3L * (bx.n / 2) * (bx.n / 2) + 1;
        long m = (long)std::floor(std::pow(1.0 / (0.413566994 * dk * R), 2)) + 2;
        while (m >= 0 && (dk * std::sqrt((double)m) * R) * 0.413566994 > 1.0) --m;
        hr[r].k2cut = (int)(m < k2n ? m : k2n);
      }
    }
    std::vector<float2> htw(bx.n);
    for (int m = 0; m < bx.n; ++m) {
      const double ang = -2.0 * M_PI * (double)m / (double)bx.n;
      htw[m] = make_float2((float)std::cos(ang), (float)std::sin(ang));
    }
    if (cudaMemcpy(rad, hr.data(), sizeof(esb::RadB) * p.n_radii, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(tw, htw.data(), sizeof(float2) * bx.n, cudaMemcpyHostToDevice) != cudaSuccess)
      return cleanup(bfail(ES_E_CUDA, "es_batch_create: upload failed"));
  }
  if (cudaMemcpy(bt->d_boxes, hb.data(), sizeof(esb::BoxDev) * count, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(bt->d_passes, passes.data(), sizeof(esb::PassDesc) * passes.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return cleanup(bfail(ES_E_CUDA, "es_batch_create: upload failed"));
  // persistent grid: exactly the co-resident CTAs (the queue relies on all CTAs being resident)
  if (cudaFuncSetAttribute(esb::batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
    return cleanup(bfail(ES_E_CUDA, "es_batch_create: shared memory opt-in failed"));
  int per_sm = 0, sms = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, esb::batch_kernel, esb::BT, smem) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, bt->device) != cudaSuccess || per_sm < 1)
    return cleanup(bfail(ES_E_CUDA, "es_batch_create: occupancy query failed"));
  bt->grid = per_sm * sms;
  *out = bt;
  return ES_OK;
}

static int batch_enqueue(es_batch* bt, cudaStream_t s) {
  ESB_CUDA(cudaMemsetAsync(bt->zero_base, 0, bt->zero_bytes, s));
  esb::BatchArgs g;
  g.boxes = bt->d_boxes;
  g.passes = bt->d_passes;
  g.npasses = bt->npasses;
  g.total = bt->total;
  g.ticket = bt->ctrl;
  g.err = bt->ctrl + 1;
  g.abort = bt->ctrl + 2;
  g.done = bt->ctrl + 3;
  g.spin_limit = bt->spin_limit;
  esb::batch_kernel<<<bt->grid, esb::BT, bt->smem, s>>>(g);
  ESB_CUDA(cudaGetLastError());
  return ES_OK;
}

int es_batch_run(es_batch* bt, int use_graph, void* stream) {
  if (!bt) return bfail(ES_E_ARG, "es_batch_run: NULL batch");
  int cur = -1;
  cudaGetDevice(&cur);
  if (cur != bt->device) return bfail(ES_E_ARG, "es_batch_run: call with the batch's device current");
  cudaStream_t s = (cudaStream_t)stream;
  if (!use_graph) return batch_enqueue(bt, s);
  if (!bt->graph) {
    // capture the clear + launch once; replays reuse the same buffers
    cudaStream_t cap;
    ESB_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaGraph_t graph;
    ESB_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
    int rc = batch_enqueue(bt, cap);
    cudaError_t e = cudaStreamEndCapture(cap, &graph);
    cudaStreamDestroy(cap);
    if (rc) return rc;
    if (e != cudaSuccess) return bfail(ES_E_CUDA, "stream capture failed: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(&bt->graph, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) { bt->graph = nullptr; return bfail(ES_E_CUDA, "graph instantiation failed: %s", cudaGetErrorString(e)); }
  }
  ESB_CUDA(cudaGraphLaunch(bt->graph, s));
  return ES_OK;
}

int es_batch_debug_stall(es_batch* bt, int pass, long spin_limit) {
  if (!bt || pass < 0 || pass >= bt->npasses || bt->h_passes[pass].dep < 0 || spin_limit < 1)
    return bfail(ES_E_ARG, "es_batch_debug_stall: bad arguments");
  // the pass now waits for one tile more than its dependency has: its wait must run out
  esb::PassDesc d = bt->h_passes[pass];
  d.need += 1;
  ESB_CUDA(cudaMemcpy(bt->d_passes + pass, &d, sizeof(d), cudaMemcpyHostToDevice));
  bt->spin_limit = spin_limit;
  if (bt->graph) { cudaGraphExecDestroy(bt->graph); bt->graph = nullptr; }
  return ES_OK;
}

int es_batch_check(es_batch* bt, void* stream) {
  if (!bt) return bfail(ES_E_ARG, "es_batch_check: NULL batch");
  unsigned w[2] = {0, 0};
  ESB_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  ESB_CUDA(cudaMemcpy(w, bt->ctrl + 1, sizeof(w), cudaMemcpyDeviceToHost));
  if (w[0] || w[1]) return bfail(ES_E_DEVICE, "batched launch aborted: a pass waited too long (error word 0x%x)", w[0]);
  return ES_OK;
}

int es_batch_info(const es_batch* bt, int* grid, int* passes, unsigned* tiles, int* smem) {
  if (!bt) return bfail(ES_E_ARG, "es_batch_info: NULL batch");
  if (grid) *grid = bt->grid;
  if (passes) *passes = bt->npasses;
  if (tiles) *tiles = bt->total;
  if (smem) *smem = bt->smem;
  return ES_OK;
}

int es_batch_destroy(es_batch* bt) {
  if (!bt) return ES_OK;
  if (bt->graph) cudaGraphExecDestroy(bt->graph);
  if (bt->base) cudaFree(bt->base);
  delete bt;
  return ES_OK;
}

int es_batch_last_error(char* buf, int len) {
  if (!buf || len <= 0) return ES_E_ARG;
  std::snprintf(buf, (size_t)len, "%s", g_batch_error.c_str());
  return ES_OK;
}

}  // extern "C"
