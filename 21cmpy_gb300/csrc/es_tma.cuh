// TMA-fed column passes (sm_103a): tiles of TI spectrum columns x N elements move between HBM and
// shared memory with cp.async.bulk.tensor, two tiles in flight per CTA, completion tracked by
// mbarriers.  Every wait is bounded; a timeout sets the plan's error word and the CTA leaves.
#pragma once
#include <cuda.h>
#include "es_kernels.cuh"

namespace es {

constexpr unsigned ES_DEV_ERR_TIMEOUT = 1u;
constexpr int kWaitLog2 = 26;             // default: 2^26 mbarrier polls before a wait is declared hung

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int wait_log2) {
  const long limit = 1L << (wait_log2 > 0 ? wait_log2 : kWaitLog2);
  for (long it = 0; it < limit; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
// After a timed-out wait at tile `it`, the loads issued for tiles it and it + 1 (two in flight)
// may still be landing in this CTA's shared memory.  Thread 0 waits for them, bounded like every
// other wait, before the CTA leaves, so no copy outlives the CTA that owns its destination.
__device__ __forceinline__ void drain_tile_loads(uint64_t* bars, int it, int count, int wait_log2) {
  for (int j = it; j < it + 2 && j < count; ++j) mbar_wait(&bars[j & 1], (uint32_t)((j >> 1) & 1), wait_log2);
}
// Debug stall: CTA 0 announces 16 bytes more than its first tile brings, so that tile's wait can
// only end by timing out (the copies themselves complete normally).
__device__ __forceinline__ uint32_t stall_bytes(int stall, int it) {
  return (stall && it == 0 && blockIdx.x == 0) ? 16u : 0u;
}
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// L2 eviction-priority policies for the copies (ES_HINT_*): the intermediate spectrum is kept
// (evict_last) while streamed inputs and outputs go first.
__device__ __forceinline__ uint64_t l2_policy(int hint) {
  uint64_t pol;
  if (hint == ES_HINT_EVICT_LAST)
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
  else if (hint == ES_HINT_EVICT_FIRST)
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  else
    asm volatile("createpolicy.fractional.L2::evict_normal.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}
__device__ __forceinline__ void tma_load3(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2,
                                          uint64_t pol) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1, {%2, %3, %4}], [%5], %6;"
      ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar)), "l"(pol)
      : "memory");
}
__device__ __forceinline__ void tma_load2(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, uint64_t pol) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1, {%2, %3}], [%4], %5;"
      ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(smem_u32(bar)), "l"(pol)
      : "memory");
}
__device__ __forceinline__ void tma_store3(const CUtensorMap* map, const void* src, int c0, int c1, int c2, uint64_t pol) {
  asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group.L2::cache_hint [%0, {%2, %3, %4}], [%1], %5;"
               ::"l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(src)), "r"(c0), "r"(c1), "r"(c2), "l"(pol)
               : "memory");
}
__device__ __forceinline__ void tma_store2(const CUtensorMap* map, const void* src, int c0, int c1, uint64_t pol) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.tile.bulk_group.L2::cache_hint [%0, {%2, %3}], [%1], %4;"
               ::"l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(src)), "r"(c0), "r"(c1), "l"(pol)
               : "memory");
}
// drop a dead 128-byte line from L2 without writing it back
__device__ __forceinline__ void l2_discard(const void* p) {
  asm volatile("discard.global.L2 [%0], 128;" ::"l"(p) : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read0() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait0() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// Stage 0 of a line FFT with a hook applied to every loaded element (filter, column packing).
template <int N, bool INV, int NL, int T, int ES, int TWN, int RS, class Pre>
__device__ __forceinline__ void stockham_stage0_pre(const float2* __restrict__ in, float2* __restrict__ out,
                                                    const float2* __restrict__ tw, Pre pre) {
  constexpr int R = Plan<N, RS>::radix[0];
  constexpr int NB = NL * (N / R);
  for (int b = threadIdx.x; b < NB; b += T) {
    const int l = b % NL, j = b / NL;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = pre(l, j + r * (N / R), in[l + (j + r * (N / R)) * ES]);
    Dft<R, INV>::run(v);                      // Ns = 1: no twiddles in the first stage
#pragma unroll
    for (int r = 0; r < R; ++r) out[l + (j * R + r) * ES] = v[r];
  }
}

template <int N, bool INV, int NL, int T, int ES, int TWN, int RS, class Pre>
__device__ __forceinline__ float2* fft_columns_pre(float2* a, float2* b, const float2* tw, Pre pre) {
  stockham_stage0_pre<N, INV, NL, T, ES, TWN, RS>(a, b, tw, pre);
  __syncthreads();
  return Stages<N, 1, INV, NL, T, true, ES, 1, TWN, RS>::run(b, a, tw);
}

// TMA column-pass tile shapes: variant 0 = (TI columns, T threads) of the synchronous pass,
// 1 = half as wide with half the threads (smaller shared memory, more CTAs per SM),
// 2 = TI columns with twice the threads (more warps to hide latency).
template <int N, int V> struct ColTile {
  static constexpr int TI = V == 1 ? ColCfg<N>::TI / 2 : ColCfg<N>::TI;
  static constexpr int T = V == 1 ? ColCfg<N>::T / 2 : (V == 2 ? 2 * ColCfg<N>::T : ColCfg<N>::T);
  static constexpr int MINB = T >= 512 ? 2 : 1;       // keep two 512-thread CTAs resident
};

struct TileCoord { int plane, c; bool nyq; };

template <int N, int MODE, int V>
__device__ __forceinline__ TileCoord tile_coord(int tile) {
  constexpr int CPR = (N / 2) / ColTile<N, V>::TI;
  constexpr bool ZPASS = (MODE == COL_Z_FWD || MODE == COL_Z_INV_FILTER || MODE == COL_Z_FWD_PK || MODE == COL_Z_INV);
  TileCoord t;
  const int nmain = N * CPR;
  if (ZPASS && tile >= nmain) { t.nyq = true; t.plane = 0; t.c = tile - nmain; }
  else { t.nyq = false; t.plane = tile / CPR; t.c = tile % CPR; }
  return t;
}

// The tiles one CTA takes, in order.  Plain passes: tiles blockIdx.x + k gridDim.x.  The z inverse +
// filter pass: first its share of the mirror-plane pairs (planes j and N - j of one column block,
// back to back: the same |k|^2 column by column, so the filter weights of the first serve the
// second), then its share of the remaining tiles (planes 0 and N/2, and the Nyquist plane).
template <int N, int MODE, int V> struct TileSeq {
  static constexpr int TI = ColTile<N, V>::TI, CPR = (N / 2) / TI;
  static constexpr bool PAIRS = MODE == COL_Z_INV_FILTER;
  static constexpr int NPAIR = PAIRS ? (N / 2 - 1) * CPR : 0;     // pair units
  static constexpr int NREST = PAIRS ? 2 * CPR + N / TI : 0;      // single tiles after them
  int npair_mine = 0, count = 0;
  __device__ __forceinline__ explicit TileSeq(int ntiles) {
    const int b = blockIdx.x, G = gridDim.x;
    if (PAIRS) {
      npair_mine = b < NPAIR ? (NPAIR - 1 - b) / G + 1 : 0;
      count = 2 * npair_mine + (b < NREST ? (NREST - 1 - b) / G + 1 : 0);
    } else {
      count = b < ntiles ? (ntiles - 1 - b) / G + 1 : 0;
    }
  }
  // the it-th tile; *reuse: the filter weights of the previous tile apply unchanged
  __device__ __forceinline__ TileCoord at(int it, bool* reuse) const {
    *reuse = false;
    if (!PAIRS) return tile_coord<N, MODE, V>(blockIdx.x + it * gridDim.x);
    TileCoord t;
    t.nyq = false;
    if (it < 2 * npair_mine) {
      const int unit = blockIdx.x + (it >> 1) * gridDim.x;
      const int jj = unit / CPR + 1;
      t.c = unit % CPR;
      t.plane = (it & 1) ? N - jj : jj;
      *reuse = (it & 1) != 0;
      return t;
    }
    const int k = blockIdx.x + (it - 2 * npair_mine) * gridDim.x;
    if (k < 2 * CPR) { t.plane = k < CPR ? 0 : N / 2; t.c = k % CPR; }
    else { t.nyq = true; t.plane = 0; t.c = k - 2 * CPR; }
    return t;
  }
};

// Tile load: z-pass boxes are (TI, 1, BOX) at (c TI, j, k0); y-pass boxes (TI, BOX, 1) at (c TI, j0, k);
// Nyquist-plane boxes (TI, BOX) at (c TI, k0).  BOX = min(N, 256) (a TMA box side is <= 256).
template <int N, int MODE, int V>
__device__ __forceinline__ void issue_tile_load(const OpArgs& a, const TileCoord& t, float2* dst, uint64_t* bar,
                                                uint32_t extra = 0) {
  constexpr int TI = ColTile<N, V>::TI;
  constexpr int BOX = N < 256 ? N : 256;
  constexpr bool ZPASS = (MODE == COL_Z_FWD || MODE == COL_Z_INV_FILTER || MODE == COL_Z_FWD_PK || MODE == COL_Z_INV);
  mbar_expect_tx(bar, (uint32_t)(N * TI * 8) + extra);
  const uint64_t pol = l2_policy(a.hint_in);
#pragma unroll
  for (int h = 0; h < N / BOX; ++h) {
    float2* d = dst + h * BOX * TI;
    if (t.nyq) tma_load2(d, &a.tm_in_nyq, bar, t.c * TI, h * BOX, pol);
    else if (ZPASS) tma_load3(d, &a.tm_in, bar, t.c * TI, t.plane, h * BOX, pol);
    else tma_load3(d, &a.tm_in, bar, t.c * TI, h * BOX, t.plane, pol);
  }
}

template <int N, int MODE, int V>
__device__ __forceinline__ void issue_tile_store(const OpArgs& a, const TileCoord& t, const float2* src) {
  constexpr int TI = ColTile<N, V>::TI;
  constexpr int BOX = N < 256 ? N : 256;
  constexpr bool ZPASS = (MODE == COL_Z_FWD || MODE == COL_Z_INV_FILTER || MODE == COL_Z_FWD_PK || MODE == COL_Z_INV);
  const uint64_t pol = l2_policy(a.hint_out);
#pragma unroll
  for (int h = 0; h < N / BOX; ++h) {
    const float2* s = src + h * BOX * TI;
    if (t.nyq) tma_store2(&a.tm_out_nyq, s, t.c * TI, h * BOX, pol);
    else if (ZPASS) tma_store3(&a.tm_out, s, t.c * TI, t.plane, h * BOX, pol);
    else tma_store3(&a.tm_out, s, t.c * TI, h * BOX, t.plane, pol);
  }
  bulk_commit();
}

template <int N, int MODE, int V> struct TmaSmem {
  static constexpr int TI = ColTile<N, V>::TI, T = ColTile<N, V>::T;
  static constexpr int tile = N * TI * 8;
  static constexpr int pk = (MODE == COL_Z_FWD_PK)
      ? ((T / 32) * PK_MAX_BINS * 3 + PK_MAX_BINS) * 4
      : (MODE == COL_Z_INV_FILTER ? TI * (N / 2 + 1) * 4 : 0);    // per-tile filter weights
  // [S0 | S1 | W | twiddles | pk bins or filter weights | 2 mbarriers] after aligning the base
  static constexpr int bytes = 3 * tile + N * 8 + pk + 16 + 128;
};

template <int N, int MODE, int V, int RS = 0>
__global__ void __launch_bounds__(ColTile<N, V>::T, ColTile<N, V>::MINB) col_tma(const __grid_constant__ OpArgs a) {
  constexpr int M = N / 2;
  constexpr int TI = ColTile<N, V>::TI, T = ColTile<N, V>::T;
  constexpr bool INV = (MODE == COL_Z_INV_FILTER || MODE == COL_Y_INV || MODE == COL_Z_INV);
  constexpr bool ZPASS = (MODE == COL_Z_FWD || MODE == COL_Z_INV_FILTER || MODE == COL_Z_FWD_PK || MODE == COL_Z_INV);
  constexpr int CPR = M / TI;
  constexpr bool RESULT_IN_W = (Plan<N, RS>::stages % 2) == 1;
  const int ntiles = ZPASS ? N * CPR + N / TI : N * CPR;

  extern __shared__ __align__(128) unsigned char smem_raw[];
  // TMA destinations must be 128-byte aligned: align the base explicitly (128 bytes of slack)
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  float2* S0 = reinterpret_cast<float2*>(base);
  float2* S1 = S0 + N * TI;
  float2* W = S1 + N * TI;
  float2* tw = W + N * TI;
  float* bins = reinterpret_cast<float*>(tw + N);
  float* wcol = bins;                         // COL_Z_INV_FILTER: W[col][|kz|], TI x (N/2 + 1)
  int* sthr = reinterpret_cast<int*>(bins + (T / 32) * PK_MAX_BINS * 3);
  uint64_t* bars = reinterpret_cast<uint64_t*>(base + 3 * TmaSmem<N, MODE, V>::tile + N * 8 + TmaSmem<N, MODE, V>::pk);
  __shared__ int s_abort;

  const TileSeq<N, MODE, V> seq(ntiles);
  const int my_count = seq.count;
  bool reuse_w;
  if (threadIdx.x == 0) {
    s_abort = 0;
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_mbar_init();
    fence_async_smem();
    for (int s = 0; s < 2 && s < my_count; ++s)
      issue_tile_load<N, MODE, V>(a, seq.at(s, &reuse_w), s ? S1 : S0, &bars[s], stall_bytes(a.stall, s));
  }
  for (int i = threadIdx.x; i < N; i += T) tw[i] = a.tw[i];
  if (MODE == COL_Z_FWD_PK) {
    for (int i = threadIdx.x; i < (T / 32) * PK_MAX_BINS * 3; i += T) bins[i] = 0.f;
    for (int i = threadIdx.x; i < a.nbins; i += T) sthr[i] = a.thr[i];
  }
  __syncthreads();

  for (int it = 0; it < my_count; ++it) {
    const int s = it & 1;
    float2* S = s ? S1 : S0;
    const TileCoord t = seq.at(it, &reuse_w);
    if (threadIdx.x == 0 && it >= 1) {
      // The store of tile it - 1 must have read its result out of shared memory before that
      // buffer (or W) is written again; waiting here, beside the tile wait below, keeps the rest
      // of the CTA from idling at a barrier behind it.  Tile it + 1 then goes into the buffer
      // tile it - 1 arrived in.
      bulk_wait_read0();
      if (it + 1 < my_count) {
        fence_async_smem();
        bool unused;
        issue_tile_load<N, MODE, V>(a, seq.at(it + 1, &unused), s ? S0 : S1, &bars[s ^ 1]);
      }
    }
    if (MODE == COL_Z_INV_FILTER && !reuse_w) {
      // W depends on |k|^2 = kz^2 + (ky^2 + kx^2 of the column): N/2 + 1 distinct values per
      // column.  Computed before waiting for the tile, so the arithmetic overlaps the copy; the
      // mirror plane N - j that follows plane j uses the same values.
      const float scale = a.scale * a.inv_n3;
      for (int q = threadIdx.x; q < TI * (M + 1); q += T) {
        const int col = q / (M + 1), kz = q % (M + 1);
        const int ck2 = !t.nyq ? wrap2<N>(t.plane) + (t.c * TI + col) * (t.c * TI + col)
                               : wrap2<N>(t.c * TI + col) + M * M;
        wcol[q] = filter_weight(kz * kz + ck2, a.dk, a.fR, a.fk2cut, a.filter, a.ref_compat) * scale;
      }
    }
    if (!mbar_wait(&bars[s], (uint32_t)((it >> 1) & 1), a.wait_log2)) {
      atomicOr(a.err, ES_DEV_ERR_TIMEOUT);
      s_abort = 1;
    }
    __syncthreads();
    if (s_abort) {
      if (threadIdx.x == 0) drain_tile_loads(bars, it, my_count, a.wait_log2);
      break;
    }

    float2* out;
    if (MODE == COL_Z_INV_FILTER) {
      out = fft_columns_pre<N, INV, TI, T, TI, N, RS>(S, W, tw, [&](int col, int k, float2 v) {
        return cscale(v, wcol[col * (M + 1) + (k > M ? N - k : k)]);
      });
    } else if (MODE == COL_Y_INV) {
      const float2* nyq = a.cin_nyq + (size_t)t.plane * N;
      const bool pack = t.c == 0;
      out = fft_columns_pre<N, INV, TI, T, TI, N, RS>(S, W, tw, [&](int col, int j, float2 v) {
        if (pack && col == 0) {                      // u = y0 + i yM (both Hermitian columns)
          const float2 ym = nyq[j];
          v = make_float2(v.x - ym.y, v.y + ym.x);
        }
        return v;
      });
    } else {
      out = fft_columns_pre<N, INV, TI, T, TI, N, RS>(S, W, tw, [](int, int, float2 v) { return v; });
    }
    (void)RESULT_IN_W;

    if (MODE == COL_Z_FWD_PK) {
      // Each thread runs down KR consecutive kz of one column, where |k| changes slowly, and
      // accumulates one bin at a time; when a lane's bin changes, the warp merges the finished
      // runs of all lanes that changed (grouped by bin, summed in lane order: deterministic).
      constexpr int NSEG = T / TI;                          // k segments per column
      constexpr int KR = (N + NSEG - 1) / NSEG;             // kz per segment (last may be short)
      static_assert(NSEG * TI == T, "threads must cover whole columns");
      const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
      float* wb = bins + warp * PK_MAX_BINS * 3;
      // the warps' merge scratch [warps][32][4] lives in whichever of S / W the transform left free
      // (this tile's input buffer is loaded again only after the barrier that ends the tile), so
      // the P(k) pass needs no shared memory of its own beyond the bins and fits two CTAs per SM
      float* ws = reinterpret_cast<float*>(out == W ? S : W) + warp * 32 * 4;
      const float inv = 1.0f / (2.0f * 9.8696044010893586f * a.volume);
      const int col = threadIdx.x % TI, k0 = (threadIdx.x / TI) * KR;
      int ck2;
      float wgt;
      if (!t.nyq) { const int kx = t.c * TI + col; ck2 = wrap2<N>(t.plane) + kx * kx; wgt = kx == 0 ? 1.f : 2.f; }
      else { ck2 = wrap2<N>(t.c * TI + col) + M * M; wgt = 1.f; }
      int cur = -1;
      int pos = -1;                                          // bin of the previous k in this run
      float ap = 0.f, ak = 0.f;
      unsigned an = 0u;                                      // mode count: exact integer
      const unsigned wgt_u = (unsigned)wgt;
      auto flush = [&](bool mine) {
        const int key = mine ? cur : -1;
        const unsigned peers = __match_any_sync(0xffffffffu, key);
        ws[lane * 4 + 0] = ap; ws[lane * 4 + 1] = ak; reinterpret_cast<unsigned*>(ws)[lane * 4 + 2] = an;
        __syncwarp();
        if (mine && lane == __ffs(peers) - 1) {
          float p = 0.f, k = 0.f;
          unsigned n = 0u;
          unsigned m = peers;
          while (m) {
            const int l = __ffs(m) - 1;
            m &= m - 1;
            p += ws[l * 4 + 0]; k += ws[l * 4 + 1]; n += reinterpret_cast<const unsigned*>(ws)[l * 4 + 2];
          }
          wb[cur] += p; wb[PK_MAX_BINS + cur] += k; pk_counts(wb)[cur] += n;
        }
        __syncwarp();
      };
      for (int q = 0; q < KR; ++q) {                         // warp-uniform trip count
        const int k = k0 + q;
        const bool valid = k < N;
        const int k2 = wrap2<N>(valid ? k : 0) + ck2;
        // first bin with k2 <= thr[bin]: a binary search for the run's first k, then a walk from the
        // previous k's bin (|k|^2 rises, then falls past N/2, so the bin moves by a step or two)
        int lo = pos;
        if (lo < 0) {
          int hi = a.nbins;
          lo = 0;
          while (lo < hi) { const int mid = (lo + hi) >> 1; if (k2 <= sthr[mid]) hi = mid; else lo = mid + 1; }
        } else {
          while (lo < a.nbins && k2 > sthr[lo]) ++lo;
          while (lo > 0 && k2 <= sthr[lo - 1]) --lo;
        }
        pos = lo;
        const int bin = (k2 == 0 || !valid) ? a.nbins : lo;    // the mean (k = 0) is excluded
        const bool change = bin != cur;
        if (__any_sync(0xffffffffu, change && cur >= 0 && cur < a.nbins))
          flush(change && cur >= 0 && cur < a.nbins);
        if (change) { cur = bin; ap = ak = 0.f; an = 0u; }
        if (!valid) continue;
        const float2 g = out[k * TI + col];
        const float km = a.dk * sqrtf((float)k2);
        ap += wgt * km * km * km * (g.x * g.x + g.y * g.y) * inv;
        ak += wgt * km;
        an += wgt_u;
      }
      flush(cur >= 0 && cur < a.nbins);
      __syncthreads();
    } else {
      if (MODE == COL_Y_FWD && t.c == 0) {
        // split the packed column 0: FFT(x0) stays in column 0, FFT(xM) goes to the nyq plane
        constexpr int Q = (N + T - 1) / T;
        float2 av[Q], bv[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) {
          const int j = threadIdx.x + q * T;
          if (j < N) {
            const float2 v = out[j * TI];
            const float2 w = out[((N - j) % N) * TI];
            av[q] = make_float2(0.5f * (v.x + w.x), 0.5f * (v.y - w.y));
            bv[q] = make_float2(0.5f * (v.y + w.y), -0.5f * (v.x - w.x));
          }
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < Q; ++q) {
          const int j = threadIdx.x + q * T;
          if (j < N) {
            out[j * TI] = av[q];
            a.cout_nyq[(size_t)t.plane * N + j] = bv[q];
          }
        }
      }
      fence_async_smem();
      __syncthreads();
      if (threadIdx.x == 0) issue_tile_store<N, MODE, V>(a, t, out);
    }
  }
  if (threadIdx.x == 0) bulk_wait0();

  if (MODE == COL_Z_FWD_PK) pk_finish<T>(bins, a);
}

}  // namespace es
