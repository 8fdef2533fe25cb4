// TMA-fed row passes (x axis): RL contiguous rows per tile arrive by 1-D bulk copies
// (cp.async.bulk, two tiles in flight, completion on mbarriers), are transposed into a padded
// [element][row] layout (pitch RL + 1, so every Stockham stage reads and writes shared memory
// without bank conflicts) and leave through coalesced stores.
#pragma once
#include <type_traits>
#include "es_tma.cuh"

namespace es {

template <int N> struct Row2Cfg;
template <> struct Row2Cfg<16>  { static constexpr int RL = 16, T = 128; };
template <> struct Row2Cfg<32>  { static constexpr int RL = 16, T = 128; };
template <> struct Row2Cfg<48>  { static constexpr int RL = 16, T = 128; };
template <> struct Row2Cfg<64>  { static constexpr int RL = 16, T = 256; };
template <> struct Row2Cfg<96>  { static constexpr int RL = 16, T = 256; };
template <> struct Row2Cfg<128> { static constexpr int RL = 16, T = 256; };
template <> struct Row2Cfg<160> { static constexpr int RL = 16, T = 256; };
template <> struct Row2Cfg<256> { static constexpr int RL = 16, T = 256; };
template <> struct Row2Cfg<512> { static constexpr int RL = 8,  T = 256; };
template <> struct Row2Cfg<1024> { static constexpr int RL = 4, T = 256; };

// Row-pass tile shapes: variant 0 = (RL rows, T threads) above, 1 = RL/2 rows with T/2 threads,
// 2 = RL rows with T/2 threads, 3 = RL rows with 2T threads.
template <int N, int V> struct RowTile {
  static constexpr int RL = V == 1 ? Row2Cfg<N>::RL / 2 : Row2Cfg<N>::RL;
  static constexpr int T = V == 0 ? Row2Cfg<N>::T : (V == 3 ? 2 * Row2Cfg<N>::T : Row2Cfg<N>::T / 2);
};

template <int N, bool PREV, int V> struct Row2Smem {
  static constexpr int RL = RowTile<N, V>::RL, M = N / 2;
  static constexpr int stage = RL * M * 8;                 // one tile of rows, as loaded
  static constexpr int work = M * (RL + 1) * 8;            // transposed, padded
  // [S0 | S1 | A | B | twiddles | 4 mbarriers] after aligning the base to 128 bytes.  With the
  // ionisation epilogue the previous radius' tile lands in S[s] once the split has read the
  // spectrum there, so it needs no buffers of its own.
  static constexpr int bytes = 2 * stage + 2 * work + N * 8 + 32 + 128;
};

// Resident CTAs per SM that the shared memory of a row tile allows (227 KB per SM, 1 KB reserved
// per CTA) and the threads (2048 per SM); registers are capped to match (__launch_bounds__).
template <int N, int V> struct RowOcc {
  static constexpr int by_smem = (227 * 1024) / (Row2Smem<N, true, V>::bytes + 1024);
  static constexpr int by_threads = 2048 / RowTile<N, V>::T;
  static constexpr int m = by_smem < by_threads ? by_smem : by_threads;
  static constexpr int MINB = m < 1 ? 1 : (m > 8 ? 8 : m);
};

__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar, uint64_t pol) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;"
               ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(pol)
               : "memory");
}

// Stockham stages S.. STOP - 1 of a line FFT (line-fast thread mapping); returns the buffer that
// holds the input of stage STOP.
template <int N, int S, int STOP, bool INV, int NL, int T, int ES, int TWN, int RS, bool DONE = (S == STOP)>
struct StagesTo {
  static __device__ __forceinline__ float2* run(float2* a, float2* b, const float2* tw) {
    stockham_stage<N, S, INV, NL, T, true, ES, 1, TWN, RS>(a, b, tw);
    __syncthreads();
    return StagesTo<N, S + 1, STOP, INV, NL, T, ES, TWN, RS>::run(b, a, tw);
  }
};
template <int N, int S, int STOP, bool INV, int NL, int T, int ES, int TWN, int RS>
struct StagesTo<N, S, STOP, INV, NL, T, ES, TWN, RS, true> {
  static __device__ __forceinline__ float2* run(float2* a, float2*, const float2*) { return a; }
};

// The last Stockham stage of NL lines of length N held as [element][line] (pitch ES), with the
// results handed to `out` in registers instead of written back.  Thread b takes butterfly
// j = b % Ns of line l = b / Ns (consecutive threads: consecutive butterflies of one line), whose
// outputs are the elements j + r Ns, r < R: for every r the threads of a line hold a run of Ns
// consecutive elements.  out(l, j, v) receives the R outputs.
template <int N, bool INV, int NL, int T, int ES, int TWN, int RS, class Out>
__device__ __forceinline__ void last_stage_to_regs(const float2* __restrict__ in, const float2* __restrict__ tw, Out out) {
  constexpr int S = Plan<N, RS>::stages - 1;
  constexpr int R = Plan<N, RS>::radix[S];
  constexpr int Ns = StageNs<N, S, RS>::value;
  static_assert(Ns * R == N, "the last stage spans the line");
  for (int b = threadIdx.x; b < NL * Ns; b += T) {
    const int j = b % Ns, l = b / Ns;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = in[l + (j + r * Ns) * ES];
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) {
        const float2 w = tw[j * r * (TWN / N)];
        v[r] = twid<INV>(v[r], w.x, w.y);
      }
    }
    Dft<R, INV>::run(v);
    out(l, j, v);
  }
}

// Half-spectrum rows -> real rows with the excursion-set epilogue (EPI_IONIZE) or a plain store.
template <int N, int EPI, int V, int RS = 0>
__global__ void __launch_bounds__(RowTile<N, V>::T, RowOcc<N, V>::MINB) row2_c2r(const __grid_constant__ OpArgs a) {
  constexpr int M = N / 2, RL = RowTile<N, V>::RL, T = RowTile<N, V>::T, ES = RL + 1;
  constexpr bool PREV = EPI == EPI_IONIZE;
  using SM = Row2Smem<N, PREV, V>;
  // last FFT stage: radix RLAST with NSL butterflies per line; its outputs go straight to the
  // epilogue when every warp of it is full (ballots need whole warps)
  constexpr int LAST = Plan<M, RS>::stages - 1;
  constexpr int RLAST = Plan<M, RS>::radix[LAST];
  constexpr int NSL = StageNs<M, LAST, RS>::value;
  constexpr bool FUSED = (RL * NSL) % 32 == 0 && (NSL & (NSL - 1)) == 0;
  constexpr int G = NSL < 32 ? NSL : 32;                 // lanes per run of consecutive pairs
  constexpr unsigned GMASK = G == 32 ? 0xffffffffu : ((1u << G) - 1u);
  static_assert((RL * N) % 64 == 0 && (RL * M) % 32 == 0, "row tiles must hold whole 64-voxel flag pairs");
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  float2* const S0 = reinterpret_cast<float2*>(base);
  float2* const S1 = reinterpret_cast<float2*>(base + SM::stage);
  float2* A = reinterpret_cast<float2*>(base + 2 * SM::stage);
  float2* B = A + M * ES;
  float2* tw = B + M * ES;
  uint64_t* bars = reinterpret_cast<uint64_t*>(tw + N);     // [0, 1] spectrum tiles, [2, 3] previous radius
  __shared__ float sred[T / 32];
  __shared__ int s_abort;

  const int ntiles = N * N / RL;
  const int my_count = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
  const bool has_prev = PREV && a.has_prev;
  const uint32_t tile_bytes = RL * M * 8;
  const uint64_t pol_in = l2_policy(a.hint_in), pol_prev = l2_policy(ES_HINT_EVICT_FIRST);
  auto issue = [&](int it, int s) {
    const size_t pair0 = (size_t)(blockIdx.x + it * gridDim.x) * RL * M;
    mbar_expect_tx(&bars[s], tile_bytes + stall_bytes(a.stall, it));
    bulk_load(s ? S1 : S0, a.cin + pair0, tile_bytes, &bars[s], pol_in);
  };
  // delta_R of the previous radius for tile `it`, into the stage its spectrum has left
  auto issue_prev = [&](int it, int s) {
    const size_t pair0 = (size_t)(blockIdx.x + it * gridDim.x) * RL * M;
    mbar_expect_tx(&bars[2 + s], tile_bytes);
    bulk_load(s ? S1 : S0, a.prev + pair0, tile_bytes, &bars[2 + s], pol_prev);
  };
  if (threadIdx.x == 0) {
    s_abort = 0;
    for (int b = 0; b < 4; ++b) mbar_init(&bars[b], 1);
    fence_mbar_init();
    fence_async_smem();
    for (int s = 0; s < 2 && s < my_count; ++s) issue(s, s);
  }
  for (int i = threadIdx.x; i < N; i += T) tw[i] = a.tw[i];
  // previous radius: erfc((dc - d) / denom_prev) * norm_prev >= 1/zeta  <=>  d >= thr_prev
  float thr_prev = __int_as_float(0x7f800000);
  if (has_prev) {
    const float y = a.inv_zeta / a.stats_prev[2];
    if (y < 2.0f) thr_prev = a.dc - a.denom_prev * erfcinvf(y);
  }
  const float inv_denom = PREV ? 1.0f / a.denom : 0.f;
  const f32x2 DC = bc2(a.dc), INV = bc2(inv_denom);
  const int lane = threadIdx.x & 31;
  f32x2 acc = bc2(0.0f);                              // two running sums (even, odd voxels)
  __syncthreads();

  for (int it = 0; it < my_count; ++it) {
    const int s = it & 1;
    const size_t pair0 = (size_t)(blockIdx.x + it * gridDim.x) * RL * M;
    if (!mbar_wait(&bars[s], (uint32_t)((it >> 1) & 1), a.wait_log2)) {
      atomicOr(a.err, ES_DEV_ERR_TIMEOUT);
      s_abort = 1;
    }
    __syncthreads();
    if (s_abort) {
      if (threadIdx.x == 0) drain_tile_loads(bars, it, my_count, a.wait_log2);
      break;
    }
    // C2R split + transpose: Z[m] = (X[m] + conj X[M-m]) + i w^-m (X[m] - conj X[M-m]).  Item t of
    // row l makes Z[t] and Z[M-t]; item 0 makes Z[0] from the packed (X[0], X[N/2]) and the
    // self-paired Z[M/2].  RL * M/2 items: every thread has whole items, no division when M/2 is a
    // power of two.  w^-(M-t) = -w^t, so one twiddle serves both outputs.
    const float2* src = s ? S1 : S0;
    for (int q = threadIdx.x; q < RL * (M / 2); q += T) {
      const int t = q % (M / 2), l = q / (M / 2);
      const float2* x = src + l * M;
      if (t == 0) {
        const float2 x0 = x[0];                       // (X[0], X[N/2]), both real
        A[l] = make_float2(x0.x + x0.y, x0.x - x0.y);
        const float2 xh = x[M / 2];
        const float2 th = cmul(cconj(tw[M / 2]), make_float2(0.f, xh.y + xh.y));
        A[(M / 2) * ES + l] = make_float2(xh.x + xh.x - th.y, th.x);
      } else {
        const int m2 = M - t;
        const float2 xm = x[t], xc = x[m2], w = tw[t];
        const float2 t1 = cmul(cconj(w), make_float2(xm.x - xc.x, xm.y + xc.y));
        A[t * ES + l] = make_float2(xm.x + xc.x - t1.y, xm.y - xc.y + t1.x);
        const float2 t2 = cmul(make_float2(-w.x, -w.y), make_float2(xc.x - xm.x, xc.y + xm.y));
        A[m2 * ES + l] = make_float2(xc.x + xm.x - t2.y, xc.y - xm.y + t2.x);
      }
    }
    if (a.discard_in) {
      // the intermediate spectrum is dead once copied: drop its lines from L2 unwritten
      const char* g = reinterpret_cast<const char*>(a.cin + pair0);
      for (int l = threadIdx.x; l < (int)(tile_bytes / 128); l += T) l2_discard(g + 128 * l);
    }
    __syncthreads();                                   // the split has read S[s]
    if (has_prev && threadIdx.x == 0) {
      fence_async_smem();
      issue_prev(it, s);
    }
    // every thread waits for the previous radius' tile before its epilogue reads it; a timeout
    // marks the CTA, which finishes the tile (on stale data) and leaves at the end of it
    auto wait_prev = [&]() {
      if (has_prev && !mbar_wait(&bars[2 + s], (uint32_t)((it >> 1) & 1), a.wait_log2)) {
        atomicOr(a.err, ES_DEV_ERR_TIMEOUT);
        s_abort = 1;
      }
    };
    const float2* pv = s ? S1 : S0;                    // the previous radius' tile, row-major
    if constexpr (FUSED) {
      // all stages but the last in shared memory; the last one hands its outputs to the
      // epilogue in registers (element p = j + r Ns of line l)
      const float2* Y = StagesTo<M, 0, LAST, true, RL, T, ES, N, RS>::run(A, B, tw);
      if (EPI == EPI_STORE) {
        last_stage_to_regs<M, true, RL, T, ES, N, RS>(Y, tw, [&](int l, int j, const float2* v) {
#pragma unroll
          for (int r = 0; r < RLAST; ++r) a.rout[pair0 + (size_t)l * M + j + r * NSL] = v[r];
        });
      } else {
        // one instantiation per (previous radius present, update mode): tests that are uniform
        // over the launch stay out of the loop body
        auto epilogue = [&](auto hp, auto upd) {
          constexpr bool HP = decltype(hp)::value;
          constexpr int UPD = decltype(upd)::value;
          last_stage_to_regs<M, true, RL, T, ES, N, RS>(Y, tw, [&](int l, int j, const float2* v) {
            const size_t row0 = pair0 + (size_t)l * M;
            // the erfc sum first: the RLAST chains are independent and overlap
            f32x2 e[RLAST];
#pragma unroll
            for (int r = 0; r < RLAST; ++r) e[r] = erfc_sum_pair(mul2(sub2(DC, pk2(v[r].x, v[r].y)), INV));
#pragma unroll
            for (int r = 0; r < RLAST; ++r) acc = add2(acc, e[r]);
            if (UPD == 2) {
              // centre mode: whether a cell passed at an earlier radius travels in the lowest
              // mantissa bit of delta_R (a change of at most one unit in the last place), so the
              // next radius carries it forward with no bitmap and no atomics
              if (HP) wait_prev();
#pragma unroll
              for (int r = 0; r < RLAST; ++r) {
                const int p = j + r * NSL;
                unsigned fx = 0u, fy = 0u;
                if (HP) {
                  const float2 pp = pv[l * M + p];
                  fx = (__float_as_uint(pp.x) & 1u) | (pp.x >= thr_prev ? 1u : 0u);
                  fy = (__float_as_uint(pp.y) & 1u) | (pp.y >= thr_prev ? 1u : 0u);
                }
                __stcs(a.rout + row0 + p, make_float2(__uint_as_float((__float_as_uint(v[r].x) & ~1u) | fx),
                                                      __uint_as_float((__float_as_uint(v[r].y) & ~1u) | fy)));
              }
              return;
            }
#pragma unroll
            for (int r = 0; r < RLAST; ++r)
              __stcs(a.rout + row0 + j + r * NSL, v[r]);  // streamed: read again only next radius
            if (HP) {
              // then the previous radius' test on its tile, which has had all of the above to land
              wait_prev();
#pragma unroll
              for (int r = 0; r < RLAST; ++r) {
                const int p = j + r * NSL;
                const float2 pp = pv[l * M + p];
                const bool px = pp.x >= thr_prev, py = pp.y >= thr_prev;
                const unsigned bx = __ballot_sync(0xffffffffu, px);
                const unsigned by = __ballot_sync(0xffffffffu, py);
                if (UPD == 0) {
                  // pair-major bitmap: one 64-bit word per 32 pairs, even voxels in the low half.
                  // The G lanes of a run hold G consecutive pairs starting at a multiple of G, so
                  // the run lies in one word; its first lane ORs the run's bits in (fire and forget)
                  const unsigned gx = (bx >> (lane & ~(G - 1))) & GMASK;
                  const unsigned gy = (by >> (lane & ~(G - 1))) & GMASK;
                  if ((lane & (G - 1)) == 0 && (gx | gy)) {
                    const size_t pr = row0 + p;
                    const int off = (int)(pr & 31);
                    atomicOr(reinterpret_cast<unsigned long long*>(a.flags) + pr / 32,
                             ((unsigned long long)gy << (32 + off)) | ((unsigned long long)gx << off));
                  }
                } else if (bx | by) {
                  const unsigned cnt = __popc(bx) + __popc(by);
                  unsigned first = 0;
                  if (lane == 0) first = atomicAdd(a.center_count, cnt);
                  first = __shfl_sync(0xffffffffu, first, 0);
                  const unsigned lt = (1u << lane) - 1u;
                  const unsigned v0 = (unsigned)((row0 + p) * 2);
                  unsigned pos = first + __popc(bx & lt) + __popc(by & lt);
                  if (px) a.centers[pos++] = v0;
                  if (py) a.centers[pos] = v0 + 1;
                }
              }
            }
          });
        };
        // update modes: 0 centre pixel with the bitmap, 1 sphere painting (centre list),
        // 2 centre pixel with the flag carried in delta_R
        if (!has_prev) {
          if (a.marker) epilogue(std::false_type{}, std::integral_constant<int, 2>{});
          else epilogue(std::false_type{}, std::integral_constant<int, 0>{});
        } else if (a.update == 1) epilogue(std::true_type{}, std::integral_constant<int, 1>{});
        else if (a.marker) epilogue(std::true_type{}, std::integral_constant<int, 2>{});
        else epilogue(std::true_type{}, std::integral_constant<int, 0>{});
      }
    } else {
      float2* Zr = fft_lines<M, true, RL, T, true, ES, 1, N, RS>(A, B, tw);
      wait_prev();
      if (EPI == EPI_STORE) {
        for (int e = threadIdx.x; e < RL * M; e += T) {
          const int row = e / M, p = e % M;
          a.rout[pair0 + e] = Zr[p * ES + row];
        }
      } else {
        // one loop per (previous radius present, update mode): tests that are uniform over the
        // launch stay out of the loop body
        auto epilogue = [&](auto hp, auto upd) {
          constexpr bool HP = decltype(hp)::value;
          constexpr int UPD = decltype(upd)::value;
          for (int e = threadIdx.x; e < RL * M; e += T) {     // whole warps: 64 consecutive voxels
            const int row = e / M, p = e % M;
            const float2 d = Zr[p * ES + row];
            acc = add2(acc, erfc_sum_pair(mul2(sub2(DC, pk2(d.x, d.y)), INV)));
            if (UPD == 2) {                                 // flag carried in delta_R (as above)
              unsigned fx = 0u, fy = 0u;
              if (HP) {
                const float2 pp = pv[e];
                fx = (__float_as_uint(pp.x) & 1u) | (pp.x >= thr_prev ? 1u : 0u);
                fy = (__float_as_uint(pp.y) & 1u) | (pp.y >= thr_prev ? 1u : 0u);
              }
              __stcs(a.rout + pair0 + e, make_float2(__uint_as_float((__float_as_uint(d.x) & ~1u) | fx),
                                                     __uint_as_float((__float_as_uint(d.y) & ~1u) | fy)));
              continue;
            }
            if (HP) {
              const float2 pp = pv[e];
              const bool px = pp.x >= thr_prev, py = pp.y >= thr_prev;
              const unsigned bx = __ballot_sync(0xffffffffu, px);
              const unsigned by = __ballot_sync(0xffffffffu, py);
              if (UPD == 0) {
                // pair-major bitmap: one 64-bit word per 32 pairs, even voxels in the low half;
                // a fire-and-forget OR, so nothing on the warp's path waits for memory
                if (lane == 0 && (bx | by))
                  atomicOr(reinterpret_cast<unsigned long long*>(a.flags) + (pair0 + e) / 32,
                           ((unsigned long long)by << 32) | bx);
              } else if (bx | by) {
                const unsigned cnt = __popc(bx) + __popc(by);
                unsigned first = 0;
                if (lane == 0) first = atomicAdd(a.center_count, cnt);
                first = __shfl_sync(0xffffffffu, first, 0);
                const unsigned lt = (1u << lane) - 1u;
                const unsigned v0 = (unsigned)((pair0 + e) * 2);
                unsigned pos = first + __popc(bx & lt) + __popc(by & lt);
                if (px) a.centers[pos++] = v0;
                if (py) a.centers[pos] = v0 + 1;
              }
            }
            __stcs(a.rout + pair0 + e, d);                 // streamed: read again only next radius
          }
        };
        if (!has_prev) {
          if (a.marker) epilogue(std::false_type{}, std::integral_constant<int, 2>{});
          else epilogue(std::false_type{}, std::integral_constant<int, 0>{});
        } else if (a.update == 1) epilogue(std::true_type{}, std::integral_constant<int, 1>{});
        else if (a.marker) epilogue(std::true_type{}, std::integral_constant<int, 2>{});
        else epilogue(std::true_type{}, std::integral_constant<int, 0>{});
      }
    }
    __syncthreads();                                   // S[s], A, B free again
    if (s_abort) {
      // the previous radius' tile of this tile and the spectrum of the next may still be landing
      if (threadIdx.x == 0) {
        if (has_prev) mbar_wait(&bars[2 + s], (uint32_t)((it >> 1) & 1), a.wait_log2);
        if (it + 1 < my_count) mbar_wait(&bars[s ^ 1], (uint32_t)(((it + 1) >> 1) & 1), a.wait_log2);
      }
      break;
    }
    if (threadIdx.x == 0 && it + 2 < my_count) {
      fence_async_smem();
      issue(it + 2, s);
    }
  }
  if (EPI == EPI_IONIZE) {
    float total;
    const float2 acc2 = upk2(acc);
    if (grid_sum<T>(acc2.x + acc2.y, a.partials, a.counter, sred, &total) && threadIdx.x == 0) {
      const float mean = total / ((float)N * (float)N * (float)N);
      a.stats_out[0] = total;
      a.stats_out[1] = mean;
      a.stats_out[2] = a.normalize ? a.fc_mean / mean : 1.f;
    }
  }
}

// Real rows -> half-spectrum rows (slot 0 holds (X[0], X[N/2])), with a scale or P(k) prologue.
template <int N, int PRO, int V>
__global__ void __launch_bounds__(RowTile<N, V>::T, RowOcc<N, V>::MINB) row2_r2c(const __grid_constant__ OpArgs a) {
  constexpr int M = N / 2, RL = RowTile<N, V>::RL, T = RowTile<N, V>::T, ES = RL + 1;
  using SM = Row2Smem<N, false, V>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  float2* const S0 = reinterpret_cast<float2*>(base);
  float2* const S1 = reinterpret_cast<float2*>(base + SM::stage);
  float2* A = reinterpret_cast<float2*>(base + 2 * SM::stage);
  float2* B = A + M * ES;
  float2* tw = B + M * ES;
  uint64_t* bars = reinterpret_cast<uint64_t*>(tw + N);
  __shared__ int s_abort;

  const int ntiles = N * N / RL;
  const int my_count = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
  const uint32_t tile_bytes = RL * M * 8;
  auto issue = [&](int it, int s) {
    const size_t pair0 = (size_t)(blockIdx.x + it * gridDim.x) * RL * M;
    mbar_expect_tx(&bars[s], tile_bytes + stall_bytes(a.stall, it));
    bulk_load(s ? S1 : S0, a.rin + pair0, tile_bytes, &bars[s], l2_policy(a.hint_in));
  };
  if (threadIdx.x == 0) {
    s_abort = 0;
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_mbar_init();
    fence_async_smem();
    for (int s = 0; s < 2 && s < my_count; ++s) issue(s, s);
  }
  for (int i = threadIdx.x; i < N; i += T) tw[i] = a.tw[i];
  float sc = a.scale, sh = 0.f;
  if (PRO == PRO_PK) {
    const float ave = *a.ave;
    // g = (x / ave - 1) V / N^3  (delta_T.py:80-82), optionally times ave
    sc = a.pk_norm / ave;
    sh = -a.pk_norm;
    if (a.dimensional) { sc *= ave; sh *= ave; }
  }
  __syncthreads();

  for (int it = 0; it < my_count; ++it) {
    const int s = it & 1;
    const size_t pair0 = (size_t)(blockIdx.x + it * gridDim.x) * RL * M;
    if (!mbar_wait(&bars[s], (uint32_t)((it >> 1) & 1), a.wait_log2)) {
      atomicOr(a.err, ES_DEV_ERR_TIMEOUT);
      s_abort = 1;
    }
    __syncthreads();
    if (s_abort) {
      if (threadIdx.x == 0) drain_tile_loads(bars, it, my_count, a.wait_log2);
      break;
    }
    const float2* src = s ? S1 : S0;
    for (int e = threadIdx.x; e < RL * M; e += T) {
      const int row = e / M, p = e % M;
      float2 v = src[e];
      v = PRO == PRO_PK ? make_float2(fmaf(v.x, sc, sh), fmaf(v.y, sc, sh)) : cscale(v, sc);
      A[p * ES + row] = v;
    }
    __syncthreads();
    float2* Z = fft_lines<M, false, RL, T, true, ES, 1, N>(A, B, tw);
    // X[m] = (Z[m] + conj Z[M-m]) / 2 - i w^m (Z[m] - conj Z[M-m]) / 2; item t of row l makes X[t]
    // and X[M-t], item 0 the packed (X[0], X[N/2]) and the self-paired X[M/2]; w^(M-t) = -conj w^t
    for (int q = threadIdx.x; q < RL * (M / 2); q += T) {
      const int t = q % (M / 2), l = q / (M / 2);
      float2* out = a.cout + pair0 + (size_t)l * M;
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
        const float2 t2 = cmul(make_float2(-w.x, w.y), make_float2(zc.x - zm.x, zc.y + zm.y));
        out[m2] = make_float2(0.5f * (zc.x + zm.x + t2.y), 0.5f * (zc.y - zm.y - t2.x));
      }
    }
    __syncthreads();
    if (threadIdx.x == 0 && it + 2 < my_count) {
      fence_async_smem();
      issue(it + 2, s);
    }
  }
}

}  // namespace es
