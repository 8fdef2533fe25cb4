// Batched excursion-set engine: many boxes of uneven HII_DIM (and their own zeta, R_mfp, T_vir,
// z) run in ONE persistent launch.  The host lists every box's passes (forward transform, three
// passes per radius, final step) and merges them into one work queue: the boxes are dealt to
// `lanes` lanes (balanced by N^3 * N_R), a lane runs its boxes one after the other, and the lanes
// advance side by side, each in proportion to its own total work so that they finish together;
// only `lanes` boxes' workspaces are live at a time.  CTAs take tickets of `chunk` tiles from a global counter
// in queue order.  A pass waits until its dependencies (at most two earlier passes of its box)
// have counted all their tickets done.  The filtered spectrum alternates between two buffers by
// radius parity, so the z inverse of radius r + 1 depends only on the row pass of radius r - 1 and
// overlaps radius r's y and row passes.  Dependencies always point to earlier tickets, all held by
// resident CTAs: the queue cannot deadlock.  Every wait is bounded; a timeout raises the batch's
// error word and an abort flag that makes every CTA leave.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <algorithm>
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

enum BOp { B_ROW_R2C = 0, B_COL_Y_FWD = 1, B_COL_Z_FWD = 2, B_COL_Z_INV = 3, B_COL_Y_INV = 4, B_ROW_C2R = 5, B_FINAL = 6,
           B_WTAB = 7, B_PAINT = 8, B_PK_R2C = 9, B_COL_Z_FWD_PK = 10 };
constexpr int WTAB_TILE = 2048;      // filter-table entries per tile
constexpr int PROF_OPS = 16;         // per-op counters of the optional profile
constexpr int PAINT_TILES = 64;      // tiles of a painting pass (8 warps each, one centre per warp at a time)
// P(k) binning's shared memory after a column tile's buffers: per-warp bins [8][3][nbins],
// per-warp scratch [8][32][4], the bin thresholds
__host__ __device__ constexpr int pk_smem(int nbins) { return (8 * 3 * nbins + 8 * 32 * 4 + nbins) * 4; }

struct RadB { float R, denom; int k2cut, r2max; };   // r2max: sphere painting's largest |d|^2 (-1: none)

struct BoxDev {
  int n, n_radii, normalize, filter, ref_compat, output;
  float dk, dc, fc_mean, zeta, inv_zeta, growth, inv_n3, pad0;
  const float* delta;
  float* out;
  float* nf;
  float2 *X, *Xnyq, *T[2], *Tnyq[2];  // filtered spectrum: one buffer per radius parity
  float* wtab;           // [n_radii][k2n]: W(k^2) * growth / N^3 of every radius, k^2 = 0 .. 3 (N/2)^2
  int k2n, update;       // table row length; 1: sphere painting
  uint32_t* centers;     // sphere mode: centres found by the current row pass
  unsigned* ccount;      // [n_radii]: centres found by the row pass of each radius
  float *dR0, *dR1;
  unsigned long long* flags;
  const float2* tw;
  const RadB* rad;
  float* stats;          // [n_radii][4]: sum, mean, norm
  float* partials;       // per-tile partial sums of the reducing passes
  unsigned* arrive;      // [n_radii + 3] arrival counters: row passes, final step, delta_T mean, P(k)
  // delta_T and P(k) (delta_T.py:73-98): tfac = 0 skips both, nbins = 0 skips P(k)
  float tfac, pk_norm, volume;
  int nbins, dimensional, pad1;
  float* dT;
  float* ave;
  const int* thr;        // [nbins] k^2 thresholds
  float* pk_out;         // [3 nbins]
  float* pk_part;        // [z tiles][3 nbins] per-tile bins (counts as unsigned)
  float* partials2;      // per-tile partial sums of delta_T
};

// first: first ticket; dep/dep2: passes awaited (-1: none), need/need2: their ticket counts
struct PassDesc { int box, op, radius, tiles, first, tickets, dep, need, dep2, need2, pad0, pad1; };

struct BatchArgs {
  const BoxDev* boxes;
  const PassDesc* passes;
  const int* first;    // first ticket of every pass (a compact copy for the search)
  int npasses;
  unsigned total;
  unsigned* ticket;
  unsigned* done;
  unsigned* err;
  unsigned* abort;
  long spin_limit;
  int chunk;           // tiles per ticket
  unsigned long long* prof;   // NULL, or [PROF_OPS][4]: cycles in tiles, tiles, cycles finding and awaiting tickets, tickets
};

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Column tiles: TI columns x N rows; row tiles: RL rows of N/2 complex pairs; RS picks the radix
// schedule (es_fft.cuh Plan<N, RS>).  Chosen so that every stage of the line transforms has
// close to one butterfly per thread of the CTA or more: a tile's time is its slowest stage's
// latency, and a radix-16 stage over 8 rows of 80 points keeps only 40 of 256 threads busy.
template <int N> struct BCol;
template <> struct BCol<32>  { static constexpr int TI = 16, RS = 0; };
template <> struct BCol<48>  { static constexpr int TI = 8,  RS = 1; };
template <> struct BCol<64>  { static constexpr int TI = 16, RS = 1; };
template <> struct BCol<96>  { static constexpr int TI = 16, RS = 0; };
template <> struct BCol<128> { static constexpr int TI = 8,  RS = 1; };
template <> struct BCol<160> { static constexpr int TI = 8,  RS = 0; };
template <> struct BCol<256> { static constexpr int TI = 8,  RS = 1; };
template <int N> struct BRow;
template <> struct BRow<32>  { static constexpr int RL = 32, RS = 1; };
template <> struct BRow<48>  { static constexpr int RL = 16, RS = 1; };
template <> struct BRow<64>  { static constexpr int RL = 32, RS = 1; };
template <> struct BRow<96>  { static constexpr int RL = 16, RS = 1; };
template <> struct BRow<128> { static constexpr int RL = 16, RS = 1; };
template <> struct BRow<160> { static constexpr int RL = 16, RS = 1; };
template <> struct BRow<256> { static constexpr int RL = 8,  RS = 1; };

template <int N> __host__ __device__ constexpr int col_tiles_z() { return N * ((N / 2) / BCol<N>::TI) + N / BCol<N>::TI; }
template <int N> __host__ __device__ constexpr int col_tiles_y() { return N * ((N / 2) / BCol<N>::TI); }
template <int N> __host__ __device__ constexpr int row_tiles() { return N * N / BRow<N>::RL; }
template <int N> __host__ __device__ constexpr int final_tiles() { return (N * N * (N / 2) + FINAL_PAIRS - 1) / FINAL_PAIRS; }
// column passes: twiddles, three tile buffers (two landing while one is transformed) and the
// transform's second buffer; row passes: twiddles, the transform's two
// buffers, two raw-row buffers and the previous radius's delta_R tile
template <int N> __host__ __device__ constexpr int smem_bytes(int pk_bins) {
  constexpr int TI = BCol<N>::TI, RL = BRow<N>::RL, M = N / 2;
  constexpr int col = (N + 4 * N * TI) * 8;
  constexpr int row = (N + 2 * M * (RL + 1) + 3 * RL * M) * 8;
  const int colp = col + (pk_bins ? pk_smem(pk_bins) : 0);   // P(k) bins follow a column tile's buffers
  return colp > row ? colp : row;
}

__device__ __forceinline__ void cp16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;"
               ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(__cvta_generic_to_global(src)) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int K> __device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(K) : "memory"); }
__device__ __forceinline__ void cp8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;"
               ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(__cvta_generic_to_global(src)) : "memory");
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

// ---------------------------------------------------------------- P(k) (delta_T.py:84-98)
// Spherical binning of one z-forward tile of g's spectrum: k^3 |G|^2 / (2 pi^2 V), |k| and the mode
// count (1, or 2 for kx > 0 of the half spectrum) into per-warp bins, warp-aggregated per bin;
// arithmetic as the per-box plan's binning.
template <int N, int TI>
__device__ __forceinline__ void pk_bin_tile(const BoxDev& b, int plane, int c, bool nyq, const float2* Rr, float* bins,
                                            float* scratch, const int* sthr) {
  constexpr int M = N / 2;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int NB = b.nbins;
  float* wb = bins + warp * NB * 3;
  float* ws = scratch + warp * 32 * 4;
  const float inv = 1.0f / (2.0f * 9.8696044010893586f * b.volume);
  for (int e = threadIdx.x; e < N * TI; e += BT) {       // whole warps iterate together
    const int row = e / TI, col = e % TI;
    int k2;
    float wgt;
    if (!nyq) { const int kx = c * TI + col; k2 = wrap2<N>(row) + wrap2<N>(plane) + kx * kx; wgt = kx == 0 ? 1.f : 2.f; }
    else { k2 = wrap2<N>(row) + wrap2<N>(c * TI + col) + M * M; wgt = 1.f; }
    int lo = 0, hi = b.nbins;                            // first bin with k2 <= thr[bin]
    while (lo < hi) { const int mid = (lo + hi) >> 1; if (k2 <= sthr[mid]) hi = mid; else lo = mid + 1; }
    int bin = lo;
    if (k2 == 0) bin = b.nbins;                          // the mean (k = 0) is excluded
    const float2 gk = Rr[e];
    const float km = b.dk * sqrtf((float)k2);
    ws[lane * 4 + 0] = wgt * km * km * km * (gk.x * gk.x + gk.y * gk.y) * inv;
    ws[lane * 4 + 1] = wgt * km;
    reinterpret_cast<unsigned*>(ws)[lane * 4 + 2] = (unsigned)wgt;
    const unsigned peers = __match_any_sync(0xffffffffu, bin);
    __syncwarp();
    if (bin < b.nbins && lane == __ffs(peers) - 1) {
      float p = 0.f, k = 0.f;
      unsigned n = 0u;
      unsigned m = peers;
      while (m) {
        const int l = __ffs(m) - 1;
        m &= m - 1;
        p += ws[l * 4 + 0]; k += ws[l * 4 + 1]; n += reinterpret_cast<const unsigned*>(ws)[l * 4 + 2];
      }
      wb[bin] += p; wb[NB + bin] += k; reinterpret_cast<unsigned*>(wb)[2 * NB + bin] += n;
    }
    __syncwarp();
  }
}

// The tile's bins (warps summed in a fixed order) go to its slot of the per-tile partials; the
// last tile of the pass to arrive sums the slots in tile order (lanes over tiles, a fixed
// butterfly), so P(k) does not depend on which CTA ran which tile, and writes the bin means.
template <int N>
__device__ __forceinline__ void pk_tile_done(const BoxDev& b, int tile, float* bins, float* scratch) {
  __shared__ unsigned s_last;
  const int nb = b.nbins, nb3 = 3 * nb, tiles = col_tiles_z<N>();
  __syncthreads();
  for (int idx = threadIdx.x; idx < nb3; idx += BT) {
    const int q = idx / nb, bin = idx % nb;
    if (q < 2) {
      float acc = 0.f;
      for (int w = 0; w < 8; ++w) acc += bins[w * nb3 + q * nb + bin];
      b.pk_part[(size_t)tile * nb3 + idx] = acc;
    } else {
      unsigned acc = 0u;
      for (int w = 0; w < 8; ++w) acc += reinterpret_cast<const unsigned*>(bins + w * nb3)[2 * nb + bin];
      reinterpret_cast<unsigned*>(b.pk_part)[(size_t)tile * nb3 + idx] = acc;
    }
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = (atomicAdd(b.arrive + b.n_radii + 2, 1u) == (unsigned)tiles - 1) ? 1u : 0u;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float* tot = scratch;                                  // [3 nb] <= 384 floats, inside the scratch
  for (int idx = warp; idx < nb3; idx += BT / 32) {
    if (idx < 2 * nb) {
      float acc = 0.f;
      for (int t = lane; t < tiles; t += 32) acc += __ldcg(b.pk_part + (size_t)t * nb3 + idx);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (lane == 0) tot[idx] = acc;
    } else {
      unsigned acc = 0u;
      for (int t = lane; t < tiles; t += 32) acc += __ldcg(reinterpret_cast<const unsigned*>(b.pk_part) + (size_t)t * nb3 + idx);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (lane == 0) tot[idx] = __uint2float_rn(acc);
    }
  }
  __syncthreads();
  for (int bin = threadIdx.x; bin < nb; bin += BT) {
    const float n = tot[2 * nb + bin];
    b.pk_out[bin] = n > 0.f ? tot[bin] / n : 0.f;                 // ps_ave
    b.pk_out[nb + bin] = n > 0.f ? tot[nb + bin] / n : 0.f;       // k_ave
    b.pk_out[2 * nb + bin] = n;                                   // count
  }
}

// The tiles [t0, t1) of one column pass, software-pipelined: tile t + 1's columns land in shared
// memory (cp.async, 16 bytes per copy) while tile t is transformed.
template <int N, int OP>
__device__ __noinline__ void b_col_chunk(const BoxDev& b, int radius, int t0, int t1, float2* sm) {
  constexpr int M = N / 2, TI = BCol<N>::TI, CPR = M / TI;
  constexpr bool INV = OP == B_COL_Z_INV || OP == B_COL_Y_INV;
  constexpr bool PK = OP == B_COL_Z_FWD_PK;
  constexpr bool Z = OP == B_COL_Z_FWD || OP == B_COL_Z_INV || PK;
  constexpr bool FWD = OP == B_COL_Y_FWD || OP == B_COL_Z_FWD || PK;
  float2* tw = sm;
  float2* const abuf = tw + N;                                 // three tile buffers
  float2* B = abuf + 3 * N * TI;
  float* bins = reinterpret_cast<float*>(B + N * TI);          // P(k): [8][3][nbins]
  float* scratch = bins + 8 * 3 * b.nbins;                      // [8][32][4]
  int* sthr = reinterpret_cast<int*>(scratch + 8 * 32 * 4);     // [nbins]
  if (PK)
    for (int i = threadIdx.x; i < b.nbins; i += BT) sthr[i] = __ldg(b.thr + i);
  for (int i = threadIdx.x; i < N; i += BT) tw[i] = __ldg(b.tw + i);
  float2* const T = b.T[radius & 1];
  float2* const Tnyq = b.Tnyq[radius & 1];
  struct Geo { int plane, c; size_t off, es_g; bool nyq; };
  auto geom = [&](int tile) {
    Geo g;
    g.nyq = false;
    if (Z) {
      if (tile < N * CPR) { g.plane = tile / CPR; g.c = tile % CPR; g.off = (size_t)g.plane * M + g.c * TI; g.es_g = (size_t)N * M; }
      else { g.nyq = true; g.plane = 0; g.c = tile - N * CPR; g.off = (size_t)g.c * TI; g.es_g = N; }
    } else {
      g.plane = tile / CPR; g.c = tile % CPR; g.off = (size_t)g.plane * N * M + g.c * TI; g.es_g = M;
    }
    return g;
  };
  auto source = [&](const Geo& g) -> const float2* {
    if (OP == B_COL_Z_INV || FWD) return g.nyq ? b.Xnyq : b.X;
    return g.nyq ? Tnyq : T;
  };
  auto issue = [&](int tile, float2* buf) {
    const Geo g = geom(tile);
    const float2* src = source(g) + g.off;
    for (int q = threadIdx.x; q < N * TI / 2; q += BT) {
      const int row = q / (TI / 2), col = 2 * (q % (TI / 2));
      cp16(buf + row * TI + col, src + row * g.es_g + col);
    }
    cp_commit();
  };
  // Three tile buffers: two tiles' copies are in flight while one is transformed.  Barriers per
  // tile: one after the copies land (each thread first fixes up the 16-byte pieces it copied
  // itself, which cp.async.wait_group makes visible to it) and the transform's own.  Tile t + 2's
  // copies are issued after that first barrier, when every thread has finished storing tile t - 1
  // out of the buffer they overwrite.
  issue(t0, abuf);
  if (t0 + 1 < t1) issue(t0 + 1, abuf + N * TI);
  for (int tile = t0; tile < t1; ++tile) {
    float2* A = abuf + ((tile - t0) % 3) * N * TI;
    const bool more = tile + 1 < t1;
    const Geo g = geom(tile);
    float2* dst = FWD ? (g.nyq ? b.Xnyq : b.X) : (g.nyq ? Tnyq : T);
    if (PK)
      for (int i = threadIdx.x; i < 8 * 3 * b.nbins; i += BT) bins[i] = 0.f;
    if (more) cp_wait<1>(); else cp_wait<0>();          // tile + 1 may stay in flight
    if (OP == B_COL_Z_INV) {
      // W depends on |k|^2 = kz^2 + (the column's ky^2 + kx^2) only: the radius's table row
      const float* wt = b.wtab + (size_t)radius * b.k2n;
      for (int q = threadIdx.x; q < N * TI / 2; q += BT) {
        const int row = q / (TI / 2), col = 2 * (q % (TI / 2));
        const int kz2 = (row > M ? N - row : row) * (row > M ? N - row : row);
        int ck0, ck1;
        if (!g.nyq) {
          const int w = wrap2<N>(g.plane), kx = g.c * TI + col;
          ck0 = w + kx * kx; ck1 = w + (kx + 1) * (kx + 1);
        } else {
          ck0 = wrap2<N>(g.c * TI + col) + M * M; ck1 = wrap2<N>(g.c * TI + col + 1) + M * M;
        }
        float2* a = A + row * TI + col;
        a[0] = cscale(a[0], __ldg(wt + kz2 + ck0));
        a[1] = cscale(a[1], __ldg(wt + kz2 + ck1));
      }
    }
    if (OP == B_COL_Y_INV && g.c == 0) {
      for (int q = threadIdx.x; q < N * TI / 2; q += BT) {
        if (q % (TI / 2) != 0) continue;                 // the piece holding column 0 of row j
        const int j = q / (TI / 2);
        const float2 y0 = A[j * TI];
        const float2 ym = __ldcg(Tnyq + (size_t)g.plane * N + j);
        A[j * TI] = make_float2(y0.x - ym.y, y0.y + ym.x);
      }
    }
    __syncthreads();
    if (tile + 2 < t1) issue(tile + 2, abuf + ((tile - t0 + 2) % 3) * N * TI);   // tile - 1's buffer
    float2* Rr = fft_lines<N, INV, TI, BT, true, TI, 1, N, BCol<N>::RS>(A, B, tw);
    if (PK) {
      pk_bin_tile<N, TI>(b, g.plane, g.c, g.nyq, Rr, bins, scratch, sthr);
      pk_tile_done<N>(b, tile, bins, scratch);
    } else if (OP == B_COL_Y_FWD && g.c == 0) {
      for (int e = threadIdx.x; e < N * TI; e += BT) {
        const int row = e / TI, col = e % TI;
        if (col == 0) {
          const float2 v = Rr[row * TI];
          const float2 w = Rr[((N - row) % N) * TI];
          dst[g.off + row * g.es_g] = make_float2(0.5f * (v.x + w.x), 0.5f * (v.y - w.y));
          b.Xnyq[(size_t)g.plane * N + row] = make_float2(0.5f * (v.y + w.y), -0.5f * (v.x - w.x));
        } else {
          dst[g.off + row * g.es_g + col] = Rr[e];
        }
      }
    } else {
      for (int q = threadIdx.x; q < N * TI / 2; q += BT) {        // 16-byte stores
        const int row = q / (TI / 2), col = 2 * (q % (TI / 2));
        const float2 v0 = Rr[row * TI + col], v1 = Rr[row * TI + col + 1];
        *reinterpret_cast<float4*>(dst + g.off + row * g.es_g + col) = make_float4(v0.x, v0.y, v1.x, v1.y);
      }
    }
    if (PK) __syncthreads();             // the bins and scratch are reused by the next tile
  }
}

// ---------------------------------------------------------------- row tiles (x), transposed layout
// x R2C of the density, or (PK) of g = (delta_T / ave - 1) V / N^3 (times ave when dimensional),
// the per-box plan's P(k) prologue (delta_T.py:80-82)
template <int N, bool PK>
__device__ __noinline__ void b_row_r2c(const BoxDev& b, int tile, float2* sm) {
  constexpr int M = N / 2, RL = BRow<N>::RL, ES = RL + 1;
  float2* tw = sm;
  float2* A = tw + N;
  float2* B = A + M * ES;
  for (int i = threadIdx.x; i < N; i += BT) tw[i] = __ldg(b.tw + i);
  const size_t pair0 = (size_t)tile * RL * M;
  const float2* in = reinterpret_cast<const float2*>(PK ? b.dT : b.delta) + pair0;
  float sc = 1.f, sh = 0.f;
  if (PK) {
    const float ave = __ldcg(b.ave);
    sc = b.pk_norm / ave;
    sh = -b.pk_norm;
    if (b.dimensional) { sc *= ave; sh *= ave; }
  }
  for (int e = threadIdx.x; e < RL * M; e += BT) {
    const int row = e / M, p = e % M;
    float2 v = PK ? __ldcg(in + e) : __ldg(in + e);
    if (PK) v = make_float2(fmaf(v.x, sc, sh), fmaf(v.y, sc, sh));
    A[p * ES + row] = v;
  }
  __syncthreads();
  float2* Z = fft_lines<M, false, RL, BT, true, ES, 1, N, BRow<N>::RS>(A, B, tw);
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

// The tiles [t0, t1) of one row pass (x C2R + ionisation epilogue), software-pipelined: tile
// t + 1's rows and tile t's previous-radius delta_R land in shared memory (cp.async) while tile t
// is split and transformed.  Arithmetic as b_row_c2r.
template <int N>
__device__ __noinline__ void b_row_c2r_chunk(const BoxDev& b, int radius, int t0, int t1, float2* sm, float* sred) {
  constexpr int M = N / 2, RL = BRow<N>::RL, ES = RL + 1;
  float2* tw = sm;
  float2* A = tw + N;
  float2* B = A + M * ES;
  float2* const raw0 = B + M * ES;
  float2* const raw1 = raw0 + RL * M;
  float2* const P = raw1 + RL * M;
  for (int i = threadIdx.x; i < N; i += BT) tw[i] = __ldg(b.tw + i);
  const bool has_prev = radius > 0;
  float2* cur = reinterpret_cast<float2*>((radius & 1) ? b.dR1 : b.dR0);
  const float2* prv = reinterpret_cast<const float2*>((radius & 1) ? b.dR0 : b.dR1);
  const float2* srcT = b.T[radius & 1];
  float thr = __int_as_float(0x7f800000);
  if (has_prev) {
    const float y = b.inv_zeta / __ldcg(b.stats + 4 * (radius - 1) + 2);
    if (y < 2.0f) thr = b.dc - b.rad[radius - 1].denom * erfcinvf(y);
  }
  const float inv_denom = 1.0f / b.rad[radius].denom, dc = b.dc;
  const int lane = threadIdx.x & 31;
  const f32x2 DC2 = bc2(dc), INV2 = bc2(inv_denom);
  auto issue_rows = [&](const float2* src, size_t pair0, float2* buf) {
    for (int q = threadIdx.x; q < RL * M / 2; q += BT) cp16(buf + 2 * q, src + pair0 + 2 * q);
    cp_commit();
  };
  // the previous radius's delta_R: each thread copies exactly the pairs its epilogue reads, so
  // the epilogue needs no barrier after the copies land
  auto issue_prev = [&](size_t pair0) {
    for (int e = threadIdx.x; e < RL * M; e += BT) cp8(P + e, prv + pair0 + e);
    cp_commit();
  };
  // Barriers per tile: after the rows land, after the split, the transform's own and one at the
  // end.  The buffers the next tile's copies overwrite were last read before one of them.
  issue_rows(srcT, (size_t)t0 * RL * M, raw0);
  for (int tile = t0; tile < t1; ++tile) {
    const size_t pair0 = (size_t)tile * RL * M;
    const float2* raw = ((tile - t0) & 1) ? raw1 : raw0;
    const bool more = tile + 1 < t1;
    if (has_prev) issue_prev(pair0); else cp_commit();
    if (more) issue_rows(srcT, pair0 + RL * M, ((tile - t0) & 1) ? raw0 : raw1);
    if (more) cp_wait<2>(); else cp_wait<1>();
    __syncthreads();
    // item t of row l makes Z[t] and Z[M-t] (item 0: Z[0] from (X[0], X[N/2]) and Z[M/2])
    for (int q = threadIdx.x; q < RL * (M / 2); q += BT) {
      const int t = q % (M / 2), l = q / (M / 2);
      const float2* x = raw + l * M;
      if (t == 0) {
        const float2 x0 = x[0], xh = x[M / 2];
        A[l] = make_float2(x0.x + x0.y, x0.x - x0.y);
        const float2 th = cmul(cconj(tw[M / 2]), make_float2(0.f, xh.y + xh.y));
        A[(M / 2) * ES + l] = make_float2(xh.x + xh.x - th.y, th.x);
      } else {
        const int m2 = M - t;
        const float2 xm = x[t], xc = x[m2], w = tw[t];
        const float2 t1v = cmul(cconj(w), make_float2(xm.x - xc.x, xm.y + xc.y));
        A[t * ES + l] = make_float2(xm.x + xc.x - t1v.y, xm.y - xc.y + t1v.x);
        const float2 t2v = cmul(make_float2(-w.x, -w.y), make_float2(xc.x - xm.x, xc.y + xm.y));   // conj w^(M-t)
        A[m2 * ES + l] = make_float2(xc.x + xm.x - t2v.y, xc.y - xm.y + t2v.x);
      }
    }
    __syncthreads();
    float2* Zr = fft_lines<M, true, RL, BT, true, ES, 1, N, BRow<N>::RS>(A, B, tw);
    if (more) cp_wait<1>(); else cp_wait<0>();
    f32x2 acc2 = bc2(0.f);
    for (int e = threadIdx.x; e < RL * M; e += BT) {     // whole warps: 64 consecutive voxels
      const int row = e / M, p = e % M;
      const float2 d = Zr[p * ES + row];
      acc2 = add2(acc2, erfc_sum_pair(mul2(sub2(DC2, pk2(d.x, d.y)), INV2)));
      if (!b.update) {
        // centre mode: a cell's "ionised by an earlier radius" flag rides in the lowest mantissa
        // bit of its delta_R (as in the per-box plans): the previous radius's bit, or its test
        unsigned fx = 0u, fy = 0u;
        if (has_prev) {
          const float2 pp = P[e];
          fx = (__float_as_uint(pp.x) & 1u) | (pp.x >= thr ? 1u : 0u);
          fy = (__float_as_uint(pp.y) & 1u) | (pp.y >= thr ? 1u : 0u);
        }
        cur[pair0 + e] = make_float2(__uint_as_float((__float_as_uint(d.x) & ~1u) | fx),
                                     __uint_as_float((__float_as_uint(d.y) & ~1u) | fy));
        continue;
      }
      if (has_prev) {
        const float2 pp = P[e];
        const bool px = pp.x >= thr, py = pp.y >= thr;
        const unsigned bx = __ballot_sync(0xffffffffu, px);
        const unsigned by = __ballot_sync(0xffffffffu, py);
        if (bx | by) {                     // sphere mode: list the centres for the painting pass
          unsigned first = 0;
          if (lane == 0) first = atomicAdd(b.ccount + radius, __popc(bx) + __popc(by));
          first = __shfl_sync(0xffffffffu, first, 0);
          const unsigned lt = (1u << lane) - 1u;
          const uint32_t v0 = (uint32_t)((pair0 + e) * 2);
          unsigned pos = first + __popc(bx & lt) + __popc(by & lt);
          if (px) b.centers[pos++] = v0;
          if (py) b.centers[pos] = v0 + 1;
        }
      }
      cur[pair0 + e] = d;
    }
    // the tile's sum as one partial per warp (a fixed lane order), so the radius's total does not
    // depend on which CTA ran which tiles
    const float2 a2 = upk2(acc2);
    float acc = a2.x + a2.y;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) b.partials[(size_t)tile * (BT / 32) + (threadIdx.x >> 5)] = acc;
    __syncthreads();                     // ends every thread's reads of A, B, the raw rows and P
  }
  // one arrival per ticket; the CTA that completes the pass sums every tile's partials in order
  __shared__ unsigned s_last;
  const int tiles = row_tiles<N>();
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = (atomicAdd(b.arrive + radius, (unsigned)(t1 - t0)) + (unsigned)(t1 - t0) == (unsigned)tiles) ? 1u : 0u;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  float part = 0.f;
  for (int i = threadIdx.x; i < tiles * (BT / 32); i += BT) part += __ldcg(b.partials + i);
  const float total = block_sum_b(part, sred);
  if (threadIdx.x == 0) {
    const float mean = total * b.inv_n3;
    b.stats[4 * radius + 0] = total;
    b.stats[4 * radius + 1] = mean;
    b.stats[4 * radius + 2] = b.normalize ? b.fc_mean / mean : 1.f;
  }
}

// Filter table of every radius: W(k^2) * growth / N^3 for k^2 = 0 .. 3 (N/2)^2, the same product
// the per-box plans form per column (filter_weight, find_bubbles.cu:14-41).
__device__ __noinline__ void b_wtab(const BoxDev& b, int tile) {
  const long total = (long)b.n_radii * b.k2n;
  const float sc = b.growth * b.inv_n3;
  for (long i = (long)tile * WTAB_TILE + threadIdx.x; i < (long)(tile + 1) * WTAB_TILE && i < total; i += BT) {
    const int r = (int)(i / b.k2n), k2 = (int)(i % b.k2n);
    const RadB rd = b.rad[r];
    b.wtab[i] = filter_weight(k2, b.dk, rd.R, rd.k2cut, b.filter, b.ref_compat) * sc;
  }
}

// Sphere painting of the centres the row pass of `radius` found (they passed at radius - 1, so
// the ball has radius - 1's size); periodic, or clipped to the box in the reference's mode.
__device__ __noinline__ void b_paint(const BoxDev& b, int radius, int tile) {
  const unsigned cnt = __ldcg(b.ccount + radius);
  const int r2max = b.rad[radius - 1].r2max;
  if (r2max < 0) return;
  const int warp = threadIdx.x >> 5;
  for (unsigned ci = tile * (BT / 32) + warp; ci < cnt; ci += PAINT_TILES * (BT / 32))
    paint_ball(__ldcg(b.centers + ci), b.n, r2max, b.ref_compat ? 0 : 1, reinterpret_cast<uint32_t*>(b.flags));
}

template <int N>
__device__ __noinline__ void b_final(const BoxDev& b, int tile, float* sred) {
  const int last = b.n_radii - 1;
  const float2* dR = reinterpret_cast<const float2*>((last & 1) ? b.dR1 : b.dR0);
  const float norm = __ldcg(b.stats + 4 * last + 2), denom = b.rad[last].denom;
  const f32x2 NORM = bc2(norm), DC = bc2(b.dc), INV = bc2(1.0f / denom);   // as the per-box plans' final step
  const long pairs = (long)N * N * (N / 2);
  const long p0 = (long)tile * FINAL_PAIRS;
  const bool dt = b.tfac != 0.f;
  float acc = 0.f, acc_t = 0.f;
  for (long p = p0 + threadIdx.x; p < p0 + FINAL_PAIRS && p < pairs; p += BT) {
    const float2 d = __ldcg(dR + p);
    unsigned fl[2];
    if (!b.update) {                                   // centre mode: the flag in delta_R's lowest bit
      fl[0] = __float_as_uint(d.x) & 1u;
      fl[1] = __float_as_uint(d.y) & 1u;
    } else {                                           // sphere mode: the painted bitmap
      const unsigned long long w = __ldcg(b.flags + p / 32);
      const int bit = (int)(p % 32);
      fl[0] = (unsigned)(w >> bit) & 1u;
      fl[1] = (unsigned)(w >> (bit + 32)) & 1u;
    }
    float ion[2];
    const float2 f = upk2(mul2(erfc_sum_pair(mul2(sub2(DC, pk2(d.x, d.y)), INV)), NORM));
    const float fv[2] = {f.x, f.y};
#pragma unroll
    for (int h = 0; h < 2; ++h)
      ion[h] = fl[h] ? 1.0f : (fv[h] >= b.inv_zeta ? 1.0f : fv[h] * b.zeta);
    acc += (1.0f - ion[0]) + (1.0f - ion[1]);
    reinterpret_cast<float2*>(b.out)[p] =
        b.output == 0 ? make_float2(1.0f - ion[0], 1.0f - ion[1]) : make_float2(ion[0], ion[1]);
    if (dt) {                                          // delta_T.py:75: c x_HI (1 + delta)
      const float2 dd = __ldg(reinterpret_cast<const float2*>(b.delta) + p);
      const float2 t = make_float2(b.tfac * (1.0f - ion[0]) * (1.0f + dd.x), b.tfac * (1.0f - ion[1]) * (1.0f + dd.y));
      acc_t += t.x + t.y;
      reinterpret_cast<float2*>(b.dT)[p] = t;
    }
  }
  float total;
  if (tile_reduce(acc, b.partials, b.arrive + b.n_radii, tile, final_tiles<N>(), sred, &total) && threadIdx.x == 0)
    *b.nf = total * b.inv_n3;
  if (dt) {
    __syncthreads();
    if (tile_reduce(acc_t, b.partials2, b.arrive + b.n_radii + 1, tile, final_tiles<N>(), sred, &total) &&
        threadIdx.x == 0)
      *b.ave = total * b.inv_n3;
  }
}

template <int N>
__device__ __forceinline__ void run_item(const BoxDev& b, const PassDesc& pd, int tile, float2* sm, float* sred) {
  switch (pd.op) {
    case B_ROW_R2C: b_row_r2c<N, false>(b, tile, sm); break;
    case B_PK_R2C: b_row_r2c<N, true>(b, tile, sm); break;
    case B_FINAL: b_final<N>(b, tile, sred); break;
    case B_WTAB: b_wtab(b, tile); break;
    case B_PAINT: b_paint(b, pd.radius, tile); break;
  }
}

template <int N>
__device__ __forceinline__ void run_chunk(const BoxDev& b, const PassDesc& pd, int t0, int t1, float2* sm, float* sred) {
  switch (pd.op) {
    case B_COL_Y_FWD: b_col_chunk<N, B_COL_Y_FWD>(b, 0, t0, t1, sm); return;
    case B_COL_Z_FWD: b_col_chunk<N, B_COL_Z_FWD>(b, 0, t0, t1, sm); return;
    case B_COL_Z_INV: b_col_chunk<N, B_COL_Z_INV>(b, pd.radius, t0, t1, sm); return;
    case B_COL_Y_INV: b_col_chunk<N, B_COL_Y_INV>(b, pd.radius, t0, t1, sm); return;
    case B_COL_Z_FWD_PK: b_col_chunk<N, B_COL_Z_FWD_PK>(b, 0, t0, t1, sm); return;
    case B_ROW_C2R: b_row_c2r_chunk<N>(b, pd.radius, t0, t1, sm, sred); return;
    default:
      for (int tile = t0; tile < t1; ++tile) {
        run_item<N>(b, pd, tile, sm, sred);
        __syncthreads();                                 // shared memory is reused by the next tile
      }
  }
}

#define ESB_SIZES(X) X(32) X(48) X(64) X(96) X(128) X(160) X(256)

__global__ void __launch_bounds__(BT, 4) batch_kernel(BatchArgs g) {
  extern __shared__ float4 smem4[];
  float2* sm = reinterpret_cast<float2*>(smem4);
  __shared__ float sred[BT / 32];
  __shared__ unsigned s_t, s_next;
  __shared__ int s_pass, s_go;
  const int lane = threadIdx.x & 31;
  int cursor = 0;                                       // pass of this CTA's previous ticket
  if (threadIdx.x == 0) s_t = atomicAdd(g.ticket, 1u);
  __syncthreads();
  for (;;) {
    const unsigned t = s_t;
    if (t >= g.total) break;
    const long long c_start = clock64();
    if (threadIdx.x < 32) {
      // the next ticket is taken now, so its latency hides behind this one's work; tickets only
      // grow, so the pass holding t is at or after the previous ticket's (32-ary search)
      unsigned nxt = 0;
      if (lane == 0) nxt = atomicAdd(g.ticket, 1u);
      int lo = cursor, hi = g.npasses;
      while (hi - lo > 1) {
        const int step = (hi - lo + 31) / 32;
        const int idx = lo + lane * step;
        const bool le = idx < hi && (unsigned)__ldg(g.first + idx) <= t;
        const unsigned m = __ballot_sync(0xffffffffu, le);   // bit 0 set: first[lo] <= t
        lo += (31 - __clz(m)) * step;
        hi = min(lo + step, hi);
      }
      cursor = lo;
      if (lane == 0) {
        const PassDesc& pd = g.passes[lo];
        int go = 1;
        long it = 0;
        for (int k = 0; k < 2 && go; ++k) {
          const int dep = k ? pd.dep2 : pd.dep;
          if (dep < 0) continue;
          const unsigned need = (unsigned)(k ? pd.need2 : pd.need);
          while (ld_acquire(g.done + dep) < need) {
            if (++it > g.spin_limit || *(volatile unsigned*)g.abort) { go = 0; break; }
            __nanosleep(100);
          }
        }
        if (!go) { atomicOr(g.err, ES_DEV_ERR_BATCH_TIMEOUT); atomicExch(g.abort, 1u); }
        s_pass = lo;
        s_go = go;
        s_next = nxt;
      }
    }
    __syncthreads();
    const long long c_ready = clock64();
    if (!s_go) break;
    const PassDesc pd = g.passes[s_pass];
    const BoxDev& b = g.boxes[pd.box];
    const int t0 = (int)(t - (unsigned)pd.first) * g.chunk;
    const int t1 = min(t0 + g.chunk, pd.tiles);
    switch (b.n) {
#define ESB_CASE(NN) case NN: run_chunk<NN>(b, pd, t0, t1, sm, sred); break;
      ESB_SIZES(ESB_CASE)
#undef ESB_CASE
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
      if (g.prof) {                                      // SM clock cycles of this CTA
        unsigned long long* c = g.prof + 4 * pd.op;
        atomicAdd(c + 0, (unsigned long long)(clock64() - c_ready));
        atomicAdd(c + 1, (unsigned long long)(t1 - t0));
        atomicAdd(c + 2, (unsigned long long)(c_ready - c_start));
        atomicAdd(c + 3, 1ull);
      }
      atomicAdd(g.done + s_pass, 1u);
      s_t = *(volatile unsigned*)g.abort ? g.total : s_next;
    }
    __syncthreads();
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
  static void get(int* ct_z, int* ct_y, int* rt, int* ft, int* smem, int pk_bins) {
    *ct_z = esb::col_tiles_z<N>();
    *ct_y = esb::col_tiles_y<N>();
    *rt = esb::row_tiles<N>();
    *ft = esb::final_tiles<N>();
    *smem = esb::smem_bytes<N>(pk_bins);
  }
};

bool size_info(int n, int* ct_z, int* ct_y, int* rt, int* ft, int* smem, int pk_bins = 0) {
  switch (n) {
#define ESB_INFO(NN) case NN: SizeInfo<NN>::get(ct_z, ct_y, rt, ft, smem, pk_bins); return true;
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
  int* d_first = nullptr;
  unsigned* ctrl = nullptr;          // [0] ticket, [1] err, [2] abort, then done[npasses]
  int npasses = 0;
  unsigned total = 0;
  size_t zero_bytes = 0;             // counters + arrive + flags cleared before every run
  void* zero_base = nullptr;
  cudaGraphExec_t graph = nullptr;
  long spin_limit = esb::kSpinLimit;
  int lanes = 0, chunk = 1;          // queue schedule (lanes 0: every box its own lane)
  unsigned long long* prof = nullptr;  // per-op cycle counters while profiling
  std::vector<esb::PassDesc> h_passes;
  std::vector<std::vector<esb::PassDesc>> per_box;   // dep / dep2: indices within the box's list
  std::vector<int> h_n, h_nr;                        // HII_DIM and radius count per box
};

namespace {

using PassList = std::vector<esb::PassDesc>;

// One box's passes, dependencies as indices in the list: the filter table of every radius, the
// forward transform (3 passes), per radius the z inverse, y inverse and row pass (and in sphere
// mode, from radius 1 on, the painting of the centres its row pass found), the final step (with
// delta_T), and with P(k) the forward transform of delta_T ending in the binning z pass.
PassList box_passes(int box, int n, int nr, int update, int pk) {
  int ctz, cty, rt, ft, sm;
  size_info(n, &ctz, &cty, &rt, &ft, &sm);
  const long k2n = 3L * (n / 2) * (n / 2) + 1;
  PassList v;
  auto add = [&](int op, int r, int tiles, int dep, int dep2) {
    esb::PassDesc d;
    std::memset(&d, 0, sizeof(d));
    d.box = box; d.op = op; d.radius = r; d.tiles = tiles; d.dep = dep; d.dep2 = dep2;
    v.push_back(d);
    return (int)v.size() - 1;
  };
  const int iw = add(esb::B_WTAB, 0, (int)((nr * k2n + esb::WTAB_TILE - 1) / esb::WTAB_TILE), -1, -1);
  const int ir2c = add(esb::B_ROW_R2C, 0, rt, -1, -1);
  const int iyf = add(esb::B_COL_Y_FWD, 0, cty, ir2c, -1);
  const int izf = add(esb::B_COL_Z_FWD, 0, ctz, iyf, -1);
  std::vector<int> irow(nr), ipaint(nr, -1);
  for (int r = 0; r < nr; ++r) {
    // the z inverse writes the spectrum buffer of its parity, last read by radius r - 2's row pass
    const int iz = add(esb::B_COL_Z_INV, r, ctz, r < 2 ? izf : irow[r - 2], r < 2 ? iw : -1);
    const int iy = add(esb::B_COL_Y_INV, r, cty, iz, -1);
    // the row pass needs its spectrum and radius r - 1's statistics and delta_R; in sphere mode
    // it refills the centre list, which radius r - 1's painting must have finished reading
    irow[r] = add(esb::B_ROW_C2R, r, rt, iy, r == 0 ? -1 : (ipaint[r - 1] >= 0 ? ipaint[r - 1] : irow[r - 1]));
    if (update && r >= 1) ipaint[r] = add(esb::B_PAINT, r, esb::PAINT_TILES, irow[r], -1);
  }
  const int ifin = add(esb::B_FINAL, 0, ft, ipaint[nr - 1] >= 0 ? ipaint[nr - 1] : irow[nr - 1], -1);
  if (pk) {
    // P(k) of delta_T (written by the final step) through the forward spectrum's buffers
    const int ipr = add(esb::B_PK_R2C, 0, rt, ifin, -1);
    const int ipy = add(esb::B_COL_Y_FWD, 0, cty, ipr, -1);
    add(esb::B_COL_Z_FWD_PK, 0, ctz, ipy, -1);
  }
  return v;
}

// Merge the boxes' pass lists into the work queue (see the top of the file) and fill in tickets
// and global dependency indices; returns the number of tickets.
unsigned make_queue(const std::vector<PassList>& per_box, const std::vector<int>& n, const std::vector<int>& nr,
                    int lanes, int chunk, PassList* out) {
  const int count = (int)per_box.size();
  const int L = lanes <= 0 || lanes > count ? count : lanes;
  // deal boxes to lanes, heaviest (N^3 * N_R) first onto the lightest lane
  std::vector<double> cost(count);
  for (int i = 0; i < count; ++i) cost[i] = std::pow((double)n[i], 3) * nr[i];
  std::vector<int> order(count);
  for (int i = 0; i < count; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
  std::vector<std::vector<int>> lane_boxes(L);
  std::vector<double> load(L, 0.0);
  for (int i : order) {
    int best = 0;
    for (int l = 1; l < L; ++l) if (load[l] < load[best]) best = l;
    lane_boxes[best].push_back(i);
    load[best] += cost[i];
  }
  // lanes advance in proportion to their own total work (passes x N^3), so they all finish together
  // and the end of the queue still holds many independent passes: always extend the lane that
  // has queued the smallest fraction of its work
  std::vector<double> lane_work(L, 0.0);
  for (int l = 0; l < L; ++l)
    for (int i : lane_boxes[l]) lane_work[l] += (double)per_box[i].size() * std::pow((double)n[i], 3);
  struct Cursor { size_t box = 0, pass = 0; double work = 0.0; };
  std::vector<Cursor> cur(L);
  std::vector<std::vector<int>> gidx(count);
  for (int i = 0; i < count; ++i) gidx[i].assign(per_box[i].size(), -1);
  PassList& q = *out;
  q.clear();
  unsigned first = 0;
  for (;;) {
    int pick = -1;
    for (int l = 0; l < L; ++l)
      if (cur[l].box < lane_boxes[l].size() && (pick < 0 || cur[l].work < cur[pick].work)) pick = l;
    if (pick < 0) break;
    Cursor& c = cur[pick];
    const int box = lane_boxes[pick][c.box];
    esb::PassDesc d = per_box[box][c.pass];
    const int ld = d.dep, ld2 = d.dep2;
    d.dep = ld >= 0 ? gidx[box][ld] : -1;
    d.dep2 = ld2 >= 0 ? gidx[box][ld2] : -1;
    d.need = d.dep >= 0 ? q[d.dep].tickets : 0;
    d.need2 = d.dep2 >= 0 ? q[d.dep2].tickets : 0;
    d.tickets = (d.tiles + chunk - 1) / chunk;
    d.first = (int)first;
    first += (unsigned)d.tickets;
    gidx[box][c.pass] = (int)q.size();
    q.push_back(d);
    c.work += std::pow((double)n[box], 3) / lane_work[pick];
    if (++c.pass == per_box[box].size()) { c.pass = 0; ++c.box; }
  }
  return first;
}

cudaError_t upload_queue(es_batch* bt) {
  std::vector<int> first(bt->h_passes.size());
  for (size_t k = 0; k < first.size(); ++k) first[k] = bt->h_passes[k].first;
  cudaError_t e = cudaMemcpy(bt->d_passes, bt->h_passes.data(), sizeof(esb::PassDesc) * bt->h_passes.size(),
                             cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(bt->d_first, first.data(), sizeof(int) * first.size(), cudaMemcpyHostToDevice);
  return e;
}

void build_queue(es_batch* bt, int lanes, int chunk) {
  bt->total = make_queue(bt->per_box, bt->h_n, bt->h_nr, lanes, chunk, &bt->h_passes);
  bt->lanes = lanes <= 0 || lanes > bt->count ? 0 : lanes;
  bt->chunk = chunk;
}

}  // namespace

extern "C" {

int es_batch_create(const es_batch_box* boxes, int count, es_batch** out) {
  if (!boxes || count <= 0 || !out) return bfail(ES_E_ARG, "es_batch_create: bad arguments");
  *out = nullptr;
  es_batch* bt = new es_batch();
  auto cleanup = [&](int code) { es_batch_destroy(bt); return code; };
  if (cudaGetDevice(&bt->device) != cudaSuccess) return cleanup(bfail(ES_E_CUDA, "no CUDA device"));
  bt->count = count;
  std::vector<esb::BoxDev> hb(count);
  // sizes of every box's workspace
  struct Sz { size_t X, Xn, T, Tn, dR, flags, stats, partials, arrive, rad, tw, wtab, centers, ccount, pk_part,
               partials2, thr; };
  std::vector<Sz> sz(count);
  size_t total_bytes = 0;
  int smem = 0;
  for (int i = 0; i < count; ++i) {
    const es_batch_box& bx = boxes[i];
    int ctz, cty, rt, ft, sm;
    if (!size_info(bx.n, &ctz, &cty, &rt, &ft, &sm))
      return cleanup(bfail(ES_E_UNSUPPORTED, "es_batch_create: box %d has HII_DIM=%d (batched sizes: 32..256)", i, bx.n));
    const es_ionize_params& p = bx.params;
    if (!bx.delta || !bx.out || !bx.nf || !p.radii || p.n_radii < 1 || p.n_radii > 4096)
      return cleanup(bfail(ES_E_ARG, "es_batch_create: box %d has a NULL buffer or bad radius count", i));
    if (!(p.zeta > 0) || p.filter_type < 0 || p.filter_type > 2 || p.update < 0 || p.update > 1)
      return cleanup(bfail(ES_E_ARG, "es_batch_create: box %d has bad parameters", i));
    const bool want_dt = bx.t_factor != 0.f, want_pk = want_dt && bx.k2_thresholds;
    if (want_dt && (!bx.dT || !bx.ave))
      return cleanup(bfail(ES_E_ARG, "es_batch_create: box %d: delta_T needs dT and ave buffers", i));
    if (want_pk) {
      if (!bx.pk || bx.nbins < 1 || bx.nbins > es::PK_MAX_BINS)
        return cleanup(bfail(ES_E_ARG, "es_batch_create: box %d: P(k) needs pk and 1..%d bins", i, es::PK_MAX_BINS));
      for (int k = 1; k < bx.nbins; ++k)
        if (bx.k2_thresholds[k] < bx.k2_thresholds[k - 1])
          return cleanup(bfail(ES_E_ARG, "es_batch_create: box %d: k^2 thresholds must be non-decreasing", i));
    }
    if (want_pk) size_info(bx.n, &ctz, &cty, &rt, &ft, &sm, bx.nbins);
    smem = sm > smem ? sm : smem;
    const size_t N = bx.n, M = N / 2;
    Sz& s = sz[i];
    s.X = a256(N * N * M * 8); s.Xn = a256(N * N * 8); s.T = 2 * s.X; s.Tn = 2 * s.Xn;
    s.dR = a256(N * N * N * 4); s.flags = a256(N * N * N / 8); s.stats = a256((size_t)p.n_radii * 16);
    s.partials = a256((size_t)(rt * (esb::BT / 32) > ft ? rt * (esb::BT / 32) : ft) * 4); s.arrive = a256((size_t)(p.n_radii + 3) * 4);
    s.rad = a256((size_t)p.n_radii * sizeof(esb::RadB)); s.tw = a256(N * 8);
    s.wtab = a256((size_t)p.n_radii * (3 * M * M + 1) * 4);
    s.centers = p.update ? a256(N * N * N * 4) : 0;
    s.ccount = a256((size_t)p.n_radii * 4);
    s.pk_part = want_pk ? a256((size_t)ctz * 3 * bx.nbins * 4) : 0;
    s.thr = want_pk ? a256((size_t)bx.nbins * 4) : 0;
    s.partials2 = want_dt ? a256((size_t)ft * 4) : 0;
    total_bytes += s.X + s.Xn + s.T + s.Tn + 2 * s.dR + s.flags + s.stats + s.partials + s.arrive + s.rad + s.tw +
                   s.wtab + s.centers + s.ccount + s.pk_part + s.thr + s.partials2;
  }
  bt->per_box.assign(count, {});
  bt->h_n.assign(count, 0);
  bt->h_nr.assign(count, 0);
  for (int i = 0; i < count; ++i) {
    bt->h_n[i] = boxes[i].n;
    bt->h_nr[i] = boxes[i].params.n_radii;
    bt->per_box[i] = box_passes(i, boxes[i].n, boxes[i].params.n_radii, boxes[i].params.update,
                                boxes[i].t_factor != 0.f && boxes[i].k2_thresholds ? 1 : 0);
  }
  build_queue(bt, 0, 16);
  bt->npasses = (int)bt->h_passes.size();
  bt->smem = smem;
  const size_t ctrl_bytes = a256((3 + bt->h_passes.size()) * 4);
  const size_t box_bytes = a256(count * sizeof(esb::BoxDev)), pass_bytes = a256(bt->h_passes.size() * sizeof(esb::PassDesc));
  const size_t first_bytes = a256(bt->h_passes.size() * sizeof(int));
  total_bytes += ctrl_bytes + box_bytes + pass_bytes + first_bytes;
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
  std::vector<size_t> flags_off(count), arrive_off(count), ccount_off(count);
  for (int i = 0; i < count; ++i) {
    flags_off[i] = off; off += sz[i].flags;
    arrive_off[i] = off; off += sz[i].arrive;
    ccount_off[i] = off; off += sz[i].ccount;
  }
  bt->zero_bytes = off;
  bt->d_boxes = reinterpret_cast<esb::BoxDev*>(b + off); off += box_bytes;
  bt->d_passes = reinterpret_cast<esb::PassDesc*>(b + off); off += pass_bytes;
  bt->d_first = reinterpret_cast<int*>(b + off); off += first_bytes;
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
    for (int h = 0; h < 2; ++h) {
      d.T[h] = reinterpret_cast<float2*>(b + off); off += s.T / 2;
      d.Tnyq[h] = reinterpret_cast<float2*>(b + off); off += s.Tn / 2;
    }
    d.dR0 = reinterpret_cast<float*>(b + off); off += s.dR;
    d.dR1 = reinterpret_cast<float*>(b + off); off += s.dR;
    d.flags = reinterpret_cast<unsigned long long*>(b + flags_off[i]);
    d.arrive = reinterpret_cast<unsigned*>(b + arrive_off[i]);
    d.ccount = reinterpret_cast<unsigned*>(b + ccount_off[i]);
    d.update = p.update;
    d.k2n = 3 * (bx.n / 2) * (bx.n / 2) + 1;
    d.wtab = reinterpret_cast<float*>(b + off); off += s.wtab;
    d.centers = s.centers ? reinterpret_cast<uint32_t*>(b + off) : nullptr; off += s.centers;
    d.tfac = bx.t_factor;
    d.dT = bx.dT; d.ave = bx.ave;
    d.pk_norm = (float)(bx.box_len * bx.box_len * bx.box_len / ((double)bx.n * bx.n * bx.n));
    d.volume = (float)(bx.box_len * bx.box_len * bx.box_len);
    d.dimensional = bx.dimensional;
    d.nbins = s.thr ? bx.nbins : 0;
    d.pk_out = s.thr ? bx.pk : nullptr;
    d.pk_part = s.pk_part ? reinterpret_cast<float*>(b + off) : nullptr; off += s.pk_part;
    d.partials2 = s.partials2 ? reinterpret_cast<float*>(b + off) : nullptr; off += s.partials2;
    int* thr = s.thr ? reinterpret_cast<int*>(b + off) : nullptr; off += s.thr;
    d.thr = thr;
    if (thr && cudaMemcpy(thr, bx.k2_thresholds, sizeof(int) * bx.nbins, cudaMemcpyHostToDevice) != cudaSuccess)
      return cleanup(bfail(ES_E_CUDA, "es_batch_create: upload failed"));
    d.stats = reinterpret_cast<float*>(b + off); off += s.stats;
    d.partials = reinterpret_cast<float*>(b + off); off += s.partials;
    esb::RadB* rad = reinterpret_cast<esb::RadB*>(b + off); off += s.rad;
    float2* tw = reinterpret_cast<float2*>(b + off); off += s.tw;
    d.rad = rad; d.tw = tw;
    std::vector<esb::RadB> hr(p.n_radii);
    for (int r = 0; r < p.n_radii; ++r) {
      const float R = p.radii[r].R, den = p.radii[r].denom;
      if (!(R > 0) || !(den > 0)) return cleanup(bfail(ES_E_ARG, "es_batch_create: box %d radius %d invalid", i, r));
      hr[r].R = R; hr[r].denom = den;
      // sphere: cells with integer |d|^2 < R_cells^2 (find_bubbles.cu:97-98); in the reference's
      // mode R in Mpc is used as cells with a float32 compare
      if (p.ref_compat) {
        const float r2 = R * R;
        long m = (long)std::floor((double)r2);
        while (m >= 0 && (float)m >= r2) --m;
        hr[r].r2max = (int)m;
      } else {
        const double rc2 = std::pow((double)R / (bx.box_len / bx.n), 2);
        long m = (long)std::floor(rc2);
        while (m >= 0 && (double)m >= rc2) --m;
        hr[r].r2max = (int)m;
      }
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
      upload_queue(bt) != cudaSuccess)
    return cleanup(bfail(ES_E_CUDA, "es_batch_create: upload failed"));
  // persistent grid: exactly the co-resident CTAs (the queue relies on all CTAs being resident)
  if (cudaFuncSetAttribute(esb::batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
    return cleanup(bfail(ES_E_CUDA, "es_batch_create: shared memory opt-in failed"));
  int per_sm = 0, sms = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, esb::batch_kernel, esb::BT, smem) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, bt->device) != cudaSuccess || per_sm < 1)
    return cleanup(bfail(ES_E_CUDA, "es_batch_create: occupancy query failed"));
  bt->grid = per_sm * sms;
  // default schedule: every box in flight; 16 tiles per ticket when each CTA has thousands of
  // tiles to take (the uneven 64-box batch: 16 beat 8 by 6%), fewer for smaller batches (16
  // boxes: 8 per ticket beat 16 by 18%), so short passes still spread over the grid
  unsigned long long tiles = 0;
  for (const auto& d : bt->h_passes) tiles += (unsigned)d.tiles;
  const double per_cta = (double)tiles / bt->grid;
  const int chunk = per_cta >= 4000.0 ? 16 : (per_cta >= 1000.0 ? 8 : 4);
  if (chunk != bt->chunk) {
    build_queue(bt, 0, chunk);
    if (upload_queue(bt) != cudaSuccess) return cleanup(bfail(ES_E_CUDA, "es_batch_create: upload failed"));
  }
  *out = bt;
  return ES_OK;
}

static int batch_enqueue(es_batch* bt, cudaStream_t s) {
  ESB_CUDA(cudaMemsetAsync(bt->zero_base, 0, bt->zero_bytes, s));
  esb::BatchArgs g;
  g.boxes = bt->d_boxes;
  g.passes = bt->d_passes;
  g.first = bt->d_first;
  g.npasses = bt->npasses;
  g.total = bt->total;
  g.ticket = bt->ctrl;
  g.err = bt->ctrl + 1;
  g.abort = bt->ctrl + 2;
  g.done = bt->ctrl + 3;
  g.spin_limit = bt->spin_limit;
  g.chunk = bt->chunk;
  g.prof = bt->prof;
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

int es_batch_queue(const int* n, const int* n_radii, const int* update, const int* pk, int count, int lanes,
                   int chunk, int* out, int cap) {
  if (!n || !n_radii || count <= 0 || lanes < 0 || chunk < 1 || chunk > 64 || (!out && cap > 0))
    return bfail(ES_E_ARG, "es_batch_queue: bad arguments");
  std::vector<PassList> per_box(count);
  std::vector<int> vn(n, n + count), vr(n_radii, n_radii + count);
  for (int i = 0; i < count; ++i) {
    int a, b2, c, d, e;
    if (!size_info(n[i], &a, &b2, &c, &d, &e)) return bfail(ES_E_UNSUPPORTED, "es_batch_queue: HII_DIM=%d", n[i]);
    if (n_radii[i] < 1 || n_radii[i] > 4096) return bfail(ES_E_ARG, "es_batch_queue: bad radius count");
    per_box[i] = box_passes(i, n[i], n_radii[i], update ? update[i] : 0, pk ? pk[i] : 0);
  }
  PassList q;
  make_queue(per_box, vn, vr, lanes, chunk, &q);
  for (size_t k = 0; k < q.size() && (int)k < cap; ++k) {
    const esb::PassDesc& d = q[k];
    const int row[8] = {d.box, d.op, d.radius, d.tiles, d.first, d.tickets, d.dep, d.dep2};
    std::memcpy(out + 8 * k, row, sizeof(row));
  }
  return (int)q.size();
}

int es_batch_set_schedule(es_batch* bt, int lanes, int chunk) {
  if (!bt || lanes < 0 || chunk < 1 || chunk > 64) return bfail(ES_E_ARG, "es_batch_set_schedule: bad arguments");
  build_queue(bt, lanes, chunk);
  ESB_CUDA(upload_queue(bt));
  bt->spin_limit = esb::kSpinLimit;
  if (bt->graph) { cudaGraphExecDestroy(bt->graph); bt->graph = nullptr; }
  return ES_OK;
}

int es_batch_profile(es_batch* bt, int enable) {
  if (!bt) return bfail(ES_E_ARG, "es_batch_profile: NULL batch");
  const size_t bytes = sizeof(unsigned long long) * esb::PROF_OPS * 4;
  if (enable) {
    if (!bt->prof) ESB_CUDA(cudaMalloc(&bt->prof, bytes));
    ESB_CUDA(cudaMemset(bt->prof, 0, bytes));
  } else if (bt->prof) {
    cudaFree(bt->prof);
    bt->prof = nullptr;
  }
  if (bt->graph) { cudaGraphExecDestroy(bt->graph); bt->graph = nullptr; }
  return ES_OK;
}

int es_batch_profile_read(es_batch* bt, unsigned long long* out, int nops) {
  if (!bt || !out || nops < 1) return bfail(ES_E_ARG, "es_batch_profile_read: bad arguments");
  if (!bt->prof) return bfail(ES_E_ARG, "es_batch_profile_read: profiling is off");
  const int n = nops < esb::PROF_OPS ? nops : esb::PROF_OPS;
  ESB_CUDA(cudaDeviceSynchronize());
  ESB_CUDA(cudaMemcpy(out, bt->prof, sizeof(unsigned long long) * 4 * n, cudaMemcpyDeviceToHost));
  return ES_OK;
}

int es_batch_get_schedule(const es_batch* bt, int* lanes, int* chunk, unsigned* tickets) {
  if (!bt) return bfail(ES_E_ARG, "es_batch_get_schedule: NULL batch");
  if (lanes) *lanes = bt->lanes;
  if (chunk) *chunk = bt->chunk;
  if (tickets) *tickets = bt->total;
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
  if (tiles) {
    unsigned long long t = 0;
    for (const auto& d : bt->h_passes) t += (unsigned)d.tiles;
    *tiles = (unsigned)t;
  }
  if (smem) *smem = bt->smem;
  return ES_OK;
}

int es_batch_destroy(es_batch* bt) {
  if (!bt) return ES_OK;
  if (bt->graph) cudaGraphExecDestroy(bt->graph);
  if (bt->base) cudaFree(bt->base);
  if (bt->prof) cudaFree(bt->prof);
  delete bt;
  return ES_OK;
}

int es_batch_last_error(char* buf, int len) {
  if (!buf || len <= 0) return ES_E_ARG;
  std::snprintf(buf, (size_t)len, "%s", g_batch_error.c_str());
  return ES_OK;
}

}  // extern "C"
