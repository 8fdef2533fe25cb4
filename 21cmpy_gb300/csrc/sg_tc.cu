// Surrogate convolutions on the 5th-generation tensor cores (tcgen05, sm_103a) for 128^3 boxes.
//
// The 3x3x3 circular convolution of a channels-last BF16 box [z][y][x][CIN] with weights
// [27][COUT][CIN] (tap (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1)) is computed input-stationary.  One
// CTA per SM walks a contiguous range of output rows (z, y) of one z-plane at a time.  For each
// input row Y of the plane's three neighbours (z + dz) and each shift dx, one
// `tcgen05.mma.kind::f16` (BF16 x BF16 -> FP32, M = 128 voxels, K = 16 channels) multiplies the
// shifted row by the weights of the three taps (dz, dy = -1, 0, +1, dx) side by side in N:
// N = 3 * COUT columns land in the tensor-memory accumulators of output rows Y + 1, Y and Y - 1.
// Sharing the A operand (the shifted input row) between three output rows cuts the MMAs per output
// row from 27 * CIN / 16 with N = COUT to 9 * CIN / 16 with N = 3 * COUT; an N = COUT MMA pays
// for the whole 128 x 16 A tile from shared memory.
//
// Tensor memory holds S = 512 / COUT accumulators of COUT columns; output row o (the CTA's o-th)
// owns slot S - 1 - (o mod S), so rows Y + 1, Y, Y - 1 sit in ascending columns and one MMA covers
// them (two where the slot ring wraps).  Every MMA accumulates: the epilogue zeroes a slot after
// reading it, and all slots start zeroed.
//
// Shared memory holds every weight, per (dz, dx) as [ci / 8][dy, co][ci % 8] (K-major, no swizzle),
// and a ring of YS input-row groups; a group is the three rows (z - 1, z, z + 1) at one y, each
// stored per 8-channel chunk as 130 16-byte positions, position p holding voxel x = (p - 1) mod 128,
// so shift dx reads the 128 rows starting at position 1 + dx: the circular wrap in x costs nothing.
// A group is used by exactly one round of MMAs and released right after it.  The copies are
// 16-byte cp.async by four producer warps (each warp reads 512 contiguous bytes per instruction);
// a producer keeps three groups in flight and publishes a group with a proxy fence and an mbarrier
// arrive once its own copies have landed.
//
// Roles: warps 0..3 copy; warp 4 issues the MMAs (one elected lane) and commits completion to mbarriers;
// warps 5..8 read finished accumulators (tcgen05.ld, one TMEM lane = one voxel per thread), zero
// them, add the bias and apply ReLU / sigmoid / the input-gradient mask, and store BF16 (or FP32)
// rows.  Every wait is bounded; on a timeout the CTA records the error, drains its copies and
// MMAs, frees its TMEM and leaves.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <string>
#include <type_traits>

#include "es_engine.h"

namespace sgtc {

constexpr int N = 128;                 // box side: one x-row is one M = 128 tile
constexpr int POS = N + 2;             // 16-byte positions per 8-channel chunk of a staged row
constexpr int XOFF = 1;                // position of x = 0
constexpr int CHUNK = POS * 16;        // 2080: distance between the K core matrices of A
constexpr int YS = 6;                  // input-row groups in the ring
constexpr int INFLIGHT = 3;            // groups a producer thread keeps in flight (<= YS - 2)
constexpr int PRODUCERS = 128;         // warps 0..3
constexpr int MMA_WARP = 4;
constexpr int EPI_GROUPS = 1;          // epilogue warpgroups, taking output rows in turn
constexpr int THREADS = 32 * (MMA_WARP + 1 + 4 * EPI_GROUPS);   // + warp 4 (MMA) + warps 5..8 (epilogue)
constexpr uint32_t TMEM_COLS = 512;
constexpr long kSpin = 1L << 24;       // mbarrier polls before a wait is declared hung
constexpr unsigned ERR_TIMEOUT = 1u;

enum Mode { FWD_RELU = 0, FWD_SIGMOID = 1, DGRAD_MASK = 2 };

__device__ unsigned g_err;

template <int CIN, int COUT> struct Layout {
  static constexpr int KC = CIN / 8;                  // 8-channel chunks
  static constexpr int S = TMEM_COLS / COUT;          // accumulator slots
  static constexpr int LBO_B = 3 * COUT * 16;         // B: K core matrices 3 * COUT rows apart
  static constexpr int PAIR_B = KC * LBO_B;           // B of one (dz, dx): 3 taps
  static constexpr int W_BYTES = 9 * PAIR_B;
  static constexpr int ROW_BYTES = KC * CHUNK;
  static constexpr int RING_BYTES = YS * 3 * ROW_BYTES;
  static constexpr int BAR_OFF = W_BYTES + RING_BYTES;
  static constexpr int NBARS = 2 * YS + 2 * S + 1;    // full[YS], sfree[YS], done[S], tfree[S], drain
  static constexpr int BYTES = BAR_OFF + NBARS * 8 + 16 + 128;   // + tmem slot, abort, alignment
  static_assert(W_BYTES % 16 == 0 && ROW_BYTES % 16 == 0, "16-byte aligned regions");
  static_assert(3 * COUT <= 256 && COUT % 16 == 0, "N = 3 COUT must be a valid M = 128 MMA width");
  static_assert(INFLIGHT <= YS - 2, "a producer must not wait on a slot its own pending groups hold");
  static_assert(BYTES <= 232448, "shared memory per CTA");
};

// ------------------------------------------------------------------ PTX wrappers
__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void bar_init(uint64_t* b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void bar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(saddr(b)) : "memory");
}
__device__ __forceinline__ bool bar_try(uint64_t* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(saddr(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait; gives up (and raises the CTA's abort flag) after kSpin polls or once another role
// has aborted
__device__ __forceinline__ bool bar_wait(uint64_t* b, uint32_t parity, volatile int* abort) {
  for (long i = 0; i < kSpin; ++i) {
    if (bar_try(b, parity)) return true;
    if ((i & 255) == 255 && *abort) return false;
  }
  *abort = 1;
  atomicOr(&g_err, ERR_TIMEOUT);
  return false;
}
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(saddr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int K> __device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(K) : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_bar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void tc_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t cols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(slot)), "r"(cols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t cols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols) : "memory");
}

// Shared-memory matrix descriptor, K-major without swizzle: core matrices of 8 rows x 16 bytes,
// `lbo` between core matrices along K, `sbo` between 8-row groups along M / N.
__device__ __forceinline__ uint64_t mdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}
// D += A B; every MMA of this kernel accumulates into a zeroed or partly summed slot.  The whole
// warp runs the issue loop (its operands stay warp-uniform) and one elected lane issues.
__device__ __forceinline__ void mma_acc(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc) {
  asm volatile(
      "{\n .reg .pred p, e;\n setp.ne.b32 p, 1, 0;\n elect.sync _|e, 0xffffffff;\n"
      " @e tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
      ::"r"(d), "l"(a), "l"(b), "r"(idesc)
      : "memory");
}
// completion of every MMA issued so far arrives once on `b` (one elected lane of a converged warp)
__device__ __forceinline__ void mma_commit(uint64_t* b) {
  asm volatile(
      "{\n .reg .pred e;\n elect.sync _|e, 0xffffffff;\n"
      " @e tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n}\n" ::"r"(saddr(b))
      : "memory");
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
// zero 16 columns of this warp's 32 lanes
__device__ __forceinline__ void tmem_zero16(uint32_t taddr) {
  const uint32_t z = 0;
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, "
      "%1};" ::"r"(taddr), "r"(z)
      : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// Output rows [r0, r1) of this CTA, walked in segments of one z-plane each.
struct Range {
  int r0, r1;
};
__device__ __forceinline__ Range my_rows() {
  const int rows = N * N;
  return {(int)((long)rows * blockIdx.x / gridDim.x), (int)((long)rows * (blockIdx.x + 1) / gridDim.x)};
}

template <int CIN, int COUT, int MODE>
__global__ void __launch_bounds__(THREADS, 1) conv_tc_kernel(const __nv_bfloat16* __restrict__ in,
                                                             const __nv_bfloat16* __restrict__ w,
                                                             const float* __restrict__ bias, void* out,
                                                             const __nv_bfloat16* __restrict__ mask) {
  using L = Layout<CIN, COUT>;
  constexpr int KC = L::KC, S = L::S;
  constexpr int KSTEPS = CIN / 16;                    // MMA K steps per (dz, dx)
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  unsigned char* sw = sm;
  unsigned char* ring = sm + L::W_BYTES;
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + L::BAR_OFF);
  uint64_t* full = bars;
  uint64_t* sfree = bars + YS;
  uint64_t* done = bars + 2 * YS;
  uint64_t* tfree = bars + 2 * YS + S;
  uint64_t* drain = bars + 2 * YS + 2 * S;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + L::NBARS);
  volatile int* abort = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int i = 0; i < YS; ++i) {
      bar_init(&full[i], PRODUCERS);
      bar_init(&sfree[i], 1);
    }
    for (int i = 0; i < S; ++i) {
      bar_init(&done[i], 1);
      bar_init(&tfree[i], 128);
    }
    bar_init(drain, 1);
    *abort = 0;
    fence_bar_init();
  }
  if (warp == 0) {
    tmem_alloc(tmem_slot, TMEM_COLS);
    tmem_relinquish();
  }
  // weights -> per (dz, dx): [ci / 8][dy, co][ci % 8], 16-byte chunks
  for (int c = threadIdx.x; c < 27 * COUT * KC; c += THREADS) {
    const int kc = c % KC, co = (c / KC) % COUT, t = c / (KC * COUT);
    const int dz = t / 9, dy = (t / 3) % 3, dx = t % 3;
    const uint4 v = __ldg(reinterpret_cast<const uint4*>(w + ((size_t)(t * COUT + co) * CIN + kc * 8)));
    *reinterpret_cast<uint4*>(sw + (dz * 3 + dx) * L::PAIR_B + kc * L::LBO_B + (dy * COUT + co) * 16) = v;
  }
  fence_proxy_async();                                // generic writes -> tensor-core reads
  tc_before();
  __syncthreads();
  tc_after();
  const uint32_t tmem = *tmem_slot;
  if (warp > MMA_WARP && warp <= MMA_WARP + 4) {
    // every accumulator slot starts at zero
    const uint32_t lanes = (uint32_t)(32 * (warp & 3)) << 16;
    for (int c = 0; c < (int)TMEM_COLS; c += 16) tmem_zero16(tmem + lanes + (uint32_t)c);
    tmem_wait_st();
  }
  tc_before();
  __syncthreads();
  tc_after();
  const Range rg = my_rows();

  if (warp < MMA_WARP) {
    // ------------------------------------------------------------------ copies
    // Copy j of a row: position p, chunk kc with kc fastest, so a warp reads 8 whole voxels; the
    // offsets depend only on the thread and j, so they are computed once.
    constexpr int PER_ROW = KC * POS, JR = (PER_ROW + PRODUCERS - 1) / PRODUCERS;
    const int pt = threadIdx.x;
    uint32_t soff[JR], goff[JR];
#pragma unroll
    for (int j = 0; j < JR; ++j) {
      const int c = pt + j * PRODUCERS, p = c / KC, kc = c % KC;
      soff[j] = (uint32_t)(kc * CHUNK + p * 16);
      goff[j] = (uint32_t)(((p + N - 1) % N) * CIN + kc * 8);
    }
    int g = 0, published = 0;
    for (int r = rg.r0; r < rg.r1 && !*abort;) {
      const int z = r / N, yb = r % N;
      const int ye = (z + 1) * N < rg.r1 ? N : rg.r1 - z * N;
      for (int yy = yb - 1; yy <= ye && !*abort; ++yy) {
        const int slot = g % YS;
        if (g >= YS && !bar_wait(&sfree[slot], (uint32_t)((g / YS - 1) & 1), abort)) break;
        const int yw = (yy + N) % N;
        unsigned char* gb = ring + slot * 3 * L::ROW_BYTES;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const __nv_bfloat16* src = in + (size_t)(((z + d + N - 1) % N) * N + yw) * N * CIN;
          unsigned char* dst = gb + d * L::ROW_BYTES;
#pragma unroll
          for (int j = 0; j < JR; ++j)
            if (PER_ROW % PRODUCERS == 0 || pt + j * PRODUCERS < PER_ROW) cp_async16(dst + soff[j], src + goff[j]);
        }
        cp_async_commit();
        ++g;
        if (g - published >= INFLIGHT) {
          cp_async_wait<INFLIGHT - 1>();             // the oldest pending group has landed
          fence_proxy_async();
          bar_arrive(&full[published % YS]);
          ++published;
        }
      }
      r = z * N + ye;
    }
    cp_async_wait<0>();
    fence_proxy_async();
    if (!*abort)
      for (; published < g; ++published) bar_arrive(&full[published % YS]);
  } else if (warp == MMA_WARP) {
    {
      // ---------------------------------------------------------------- MMA issue
      // Descriptors are a base descriptor plus (byte offset >> 4) in the 14-bit address field.
      const uint64_t a_base = mdesc(saddr(ring), CHUNK, 128);
      const uint64_t b_base = mdesc(saddr(sw), L::LBO_B, 128);
      int g = 0, o0 = 0;
      for (int r = rg.r0; r < rg.r1 && !__any_sync(0xFFFFFFFFu, *abort);) {
        const int z = r / N, yb = r % N;
        const int ye = (z + 1) * N < rg.r1 ? N : rg.r1 - z * N;
        bool ok = true;
        for (int Y = yb - 1; Y <= ye && ok; ++Y, ++g) {
          ok = __all_sync(0xFFFFFFFFu, bar_wait(&full[g % YS], (uint32_t)((g / YS) & 1), abort));
          // output rows this input row feeds: y in [ylo, yhi], tap dy = Y - y
          const int ylo = Y - 1 > yb ? Y - 1 : yb, yhi = Y + 1 < ye - 1 ? Y + 1 : ye - 1;
          const int ohi = o0 + (yhi - yb);
          if (ok && yhi == Y + 1 && ohi >= S)          // first touch of row Y + 1's slot
            ok = __all_sync(0xFFFFFFFFu, bar_wait(&tfree[(S - 1) - ohi % S], (uint32_t)((ohi / S - 1) & 1), abort));
          if (!ok) break;
          tc_after();
          const int nrows = yhi - ylo + 1;
          const int s0 = (S - 1) - ohi % S;            // slot of row yhi; rows below follow upward
          const int n1 = nrows < S - s0 ? nrows : S - s0, n2 = nrows - n1;
          const uint32_t id1 = idesc_bf16(128, n1 * COUT), id2 = idesc_bf16(128, (n2 > 0 ? n2 : 1) * COUT);
          const uint32_t d1 = tmem + (uint32_t)(s0 * COUT);
          const uint64_t a_g = a_base + (uint64_t)((g % YS) * (3 * L::ROW_BYTES / 16));
          const uint64_t b_blk = b_base + (uint64_t)((Y - yhi + 1) * COUT);   // first dy block, 16-byte units
// One straight run of MMAs per case: a test between the MMAs (whether the slot ring wraps)
          // would put a branch around every elected issue and slow the issue to ~90 cycles per MMA;
          // without it the issue keeps pace with the tensor pipe (~56 cycles at N = 96).
          auto issue = [&](auto two) {
            constexpr bool TWO = decltype(two)::value;
#pragma unroll
            for (int dz = 0; dz < 3; ++dz) {
#pragma unroll
              for (int dx = 0; dx < 3; ++dx) {
                const uint64_t ad = a_g + (uint64_t)((dz * L::ROW_BYTES + (XOFF + dx - 1) * 16) / 16);
                const uint64_t bd = b_blk + (uint64_t)((dz * 3 + dx) * L::PAIR_B / 16);
#pragma unroll
                for (int k = 0; k < KSTEPS; ++k) {
                  const uint64_t ak = ad + (uint64_t)(2 * k * CHUNK / 16);
                  const uint64_t bk = bd + (uint64_t)(2 * k * L::LBO_B / 16);
                  mma_acc(d1, ak, bk, id1);
                  if (TWO) mma_acc(tmem, ak, bk + (uint64_t)(n1 * COUT), id2);
                }
              }
            }
          };
          if (n2 > 0) issue(std::true_type{}); else issue(std::false_type{});
          mma_commit(&sfree[g % YS]);                 // this input group is not read again
          if (Y - 1 >= yb && Y - 1 < ye) {
            const int od = o0 + (Y - 1 - yb);          // output row Y - 1 has all 27 taps
            mma_commit(&done[(S - 1) - od % S]);
          }
        }
        if (!ok) break;
        o0 += ye - yb;
        r = z * N + ye;
      }
      // every MMA this CTA issued has completed before its accumulators are freed
      __syncwarp();
      mma_commit(drain);
      for (long i = 0; i < kSpin && !bar_try(drain, 0); ++i) {
      }
    }
  } else {
    // ------------------------------------------------------------------ epilogue
    const int q = warp & 3;                            // TMEM lanes 32 q .. 32 q + 31
    const int x = 32 * q + lane;
    const uint32_t lanes = (uint32_t)(32 * q) << 16;
    float bv[COUT];
#pragma unroll
    for (int c = 0; c < COUT; ++c) bv[c] = bias ? bias[c] : 0.f;
    const int eg = (warp - MMA_WARP - 1) / 4;         // this warpgroup takes rows o = eg mod EPI_GROUPS
    for (int o = eg; o < rg.r1 - rg.r0; o += EPI_GROUPS) {
      const int r = rg.r0 + o;
      const int slot = (S - 1) - o % S;
      const bool ok = bar_wait(&done[slot], (uint32_t)((o / S) & 1), abort);
      if (!__all_sync(0xFFFFFFFFu, ok)) break;        // tcgen05.ld / st need the whole warp
      tc_after();
      float v[COUT];
      const uint32_t ta = tmem + lanes + (uint32_t)(slot * COUT);
      if (COUT == 32) tmem_ld32(ta, v); else tmem_ld16(ta, v);
#pragma unroll
      for (int c = 0; c < COUT; c += 16) tmem_zero16(ta + (uint32_t)c);
      tmem_wait_st();
      tc_before();
      bar_arrive(&tfree[slot]);
      const size_t vox = (size_t)r * N + x;
      if (MODE == FWD_SIGMOID) {
        reinterpret_cast<float*>(out)[vox] = 1.0f / (1.0f + __expf(-(v[0] + bv[0])));
      } else {
        uint32_t mbits = 0xFFFFFFFFu;
        if (MODE == DGRAD_MASK) {
          const uint4* mp = reinterpret_cast<const uint4*>(mask + vox * COUT);
          mbits = 0;
#pragma unroll
          for (int j = 0; j < COUT / 8; ++j) {
            const uint4 m = __ldg(mp + j);
            const uint32_t wds[4] = {m.x, m.y, m.z, m.w};
#pragma unroll
            for (int h = 0; h < 8; ++h) {
              const __nv_bfloat16 e = __ushort_as_bfloat16((unsigned short)(wds[h / 2] >> (16 * (h & 1))));
              if (__bfloat162float(e) > 0.f) mbits |= 1u << (8 * j + h);
            }
          }
        }
        uint4* op = reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(out) + vox * COUT);
#pragma unroll
        for (int j = 0; j < COUT / 8; ++j) {
          uint32_t pk[4];
#pragma unroll
          for (int h = 0; h < 4; ++h) {
            const int c = 8 * j + 2 * h;
            float a0 = v[c] + bv[c], a1 = v[c + 1] + bv[c + 1];
            if (MODE == FWD_RELU) {
              a0 = fmaxf(a0, 0.f);
              a1 = fmaxf(a1, 0.f);
            } else {
              if (!((mbits >> c) & 1u)) a0 = 0.f;
              if (!((mbits >> (c + 1)) & 1u)) a1 = 0.f;
            }
            const __nv_bfloat162 p2 = __floats2bfloat162_rn(a0, a1);
            pk[h] = *reinterpret_cast<const uint32_t*>(&p2);
          }
          op[j] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
        }
      }
    }
  }

  tc_before();
  __syncthreads();
  if (warp == 0) {
    __syncwarp();
    tc_after();
    tmem_dealloc(tmem, TMEM_COLS);
  }
}

// ------------------------------------------------------------------ weight gradient
// dW[t][co][ci] = sum_v dZ[v][co] X[v + (dz, dy, dx)][ci] and db[co] = sum_v dZ[v][co] at 128^3.
// With u = v + (0, 0, dx): dW = sum_u dZ[u - dx][co] X[u + (dz, dy, 0)][ci], so for one output row
// (z, y) of dZ and one dy, one MMA per 16 voxels covers every (dz, ci) x (dx, co):
//   A (M = 128, MN-major): the input rows z - 1, z, z + 1 at y + dy with 32 channel slots each, then
//     a constant row of ones, whose products are the bias gradient;
//   B (N = 3 COUT, MN-major): the dZ row (z, y) staged three times, shifted by dx = -1, 0, +1 (the
//     circular wrap in x is applied while staging);
//   D: one accumulator per dy (3 COUT columns of tensor memory), summed over all of the CTA's rows.
// Staged rows hold, per 8-channel chunk, 128 voxel positions of 16 bytes: in MN-major terms the
// core matrices (8 voxels x 8 channels) are 128 bytes apart along K and one chunk (2048 bytes)
// apart along M / N, the same stride from a row's last chunk to the next row's first.  For
// CIN = 16 the chunk slots 2 and 3 of a row are never written; they feed accumulator rows that are
// not read.  Per-CTA partials [3][128][3 COUT] are summed in a fixed order by wgrad_tc_reduce.
namespace wg {
constexpr int CH = N * 16;                 // 2048 bytes per 8-channel chunk of a staged row
constexpr int KCS = 4;                     // channel-chunk slots per staged input row
constexpr int XROW = KCS * CH;             // 8192
constexpr int XGROUP = 4 * XROW;           // rows z - 1, z, z + 1 and the ones row
constexpr int XS = 4;                      // input-row groups: y - 1, y, y + 1 in use, y + 2 landing
constexpr int DSL = 2;                     // dZ row slots
constexpr int WINFLIGHT = 3;               // items (groups or dZ rows) a producer keeps in flight
}  // namespace wg

template <int CIN, int COUT> struct WLayout {
  static constexpr int KC = CIN / 8, KCD = COUT / 8;
  static constexpr int DCOPY = KCD * wg::CH;           // one shifted copy of a dZ row
  static constexpr int DSLOT = 3 * DCOPY;
  static constexpr int NCOLS = 3 * COUT;               // N of one MMA
  static constexpr uint32_t TCOLS = 3 * NCOLS <= 256 ? 256u : 512u;
  static constexpr int XRING = wg::XS * wg::XGROUP;
  static constexpr int BAR_OFF = XRING + wg::DSL * DSLOT;
  static constexpr int NBARS = 2 * wg::XS + 2 * wg::DSL + 1;    // xfull, xfree, dfull, dfree, done
  static constexpr int BYTES = BAR_OFF + NBARS * 8 + 16 + 128;
  static_assert(NCOLS % 16 == 0 && NCOLS <= 256, "N = 3 COUT must be a valid M = 128 MMA width");
  static_assert(KC <= wg::KCS, "at most 32 input channels");
  static_assert(BYTES <= 232448, "shared memory per CTA");
};

// Where a weight-gradient wait gave up: {tag, sequence number, CTA, progress of the MMA warp};
// the first record wins.  Tags: 1 producer xfree, 2 producer dfree, 3 MMA xfull at a segment start,
// 4 MMA xfull per row, 5 MMA dfull, 6 partials-out done.
__device__ int g_wdiag[4];
constexpr long kWSpin = 1L << 20;
__device__ __forceinline__ bool wbar_wait(uint64_t* b, uint32_t parity, volatile int* abort, int tag, int seq, int prog) {
  for (long i = 0; i < kWSpin; ++i) {
    if (bar_try(b, parity)) return true;
    if ((i & 255) == 255 && *abort) return false;
  }
  *abort = 1;
  atomicOr(&g_err, ERR_TIMEOUT);
  if (atomicCAS(&g_wdiag[0], 0, tag) == 0) {
    g_wdiag[1] = seq;
    g_wdiag[2] = (int)blockIdx.x;
    g_wdiag[3] = prog;
  }
  return false;
}

// Shared-memory matrix descriptor, MN-major without swizzle: core matrices of 8 K-rows x 16 bytes
// (8 elements along M or N), `lbo` between core matrices along K, `sbo` along M / N.
__device__ __forceinline__ uint64_t mdesc_mn(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// kind::f16 instruction descriptor with both operands MN-major (transpose bits 15 and 16)
__host__ __device__ constexpr uint32_t idesc_bf16_mn(int m, int n) { return idesc_bf16(m, n) | (1u << 15) | (1u << 16); }

template <int CIN, int COUT>
__global__ void __launch_bounds__(THREADS, 1) wgrad_tc_kernel(const __nv_bfloat16* __restrict__ x,
                                                              const __nv_bfloat16* __restrict__ dz,
                                                              float* __restrict__ partials) {
  using L = WLayout<CIN, COUT>;
  constexpr int KC = L::KC, KCD = L::KCD;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  unsigned char* xring = sm;
  unsigned char* dring = sm + L::XRING;
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + L::BAR_OFF);
  uint64_t* xfull = bars;
  uint64_t* xfree = bars + wg::XS;
  uint64_t* dfull = bars + 2 * wg::XS;
  uint64_t* dfree = bars + 2 * wg::XS + wg::DSL;
  uint64_t* done = bars + 2 * wg::XS + 2 * wg::DSL;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + L::NBARS);
  volatile int* abort = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int i = 0; i < wg::XS; ++i) {
      bar_init(&xfull[i], PRODUCERS);
      bar_init(&xfree[i], 1);
    }
    for (int i = 0; i < wg::DSL; ++i) {
      bar_init(&dfull[i], PRODUCERS);
      bar_init(&dfree[i], 1);
    }
    bar_init(done, 1);
    *abort = 0;
    fence_bar_init();
  }
  if (warp == 0) {
    tmem_alloc(tmem_slot, L::TCOLS);
    tmem_relinquish();
  }
  // the ones row of every input-group slot (bf16 1.0 = 0x3F80), written once
  {
    const uint4 ones = make_uint4(0x3F803F80u, 0x3F803F80u, 0x3F803F80u, 0x3F803F80u);
    for (int i = threadIdx.x; i < wg::XS * (wg::XROW / 16); i += THREADS) {
      const int slot = i / (wg::XROW / 16), j = i % (wg::XROW / 16);
      *reinterpret_cast<uint4*>(xring + slot * wg::XGROUP + 3 * wg::XROW + 16 * j) = ones;
    }
  }
  fence_proxy_async();
  tc_before();
  __syncthreads();
  tc_after();
  const uint32_t tmem = *tmem_slot;
  if (warp > MMA_WARP && warp <= MMA_WARP + 4) {
    const uint32_t lanes = (uint32_t)(32 * (warp & 3)) << 16;
    for (int c = 0; c < (int)L::TCOLS; c += 16) tmem_zero16(tmem + lanes + (uint32_t)c);
    tmem_wait_st();
  }
  tc_before();
  __syncthreads();
  tc_after();
  const Range rg = my_rows();

  if (warp < MMA_WARP) {
    // ------------------------------------------------------------------ copies
    // Items in order, per z-plane segment [yb, ye) of the CTA's rows: X(yb - 1), X(yb), then per
    // output row y: X(y + 1), dZ(y).  An item is published (proxy fence + arrive) once WINFLIGHT - 1
    // newer ones are in flight, or at the end.
    const int pt = threadIdx.x;
    int nx = 0, nd = 0;                           // items issued of each kind
    int kinds = 0;                                // bit i of the in-flight FIFO: 1 = dZ row
    int pending = 0;                              // items issued but not yet published
    int pub_x = 0, pub_d = 0;
    auto publish_oldest = [&]() {
      const bool isd = (kinds >> (pending - 1)) & 1;    // oldest at the highest bit
      fence_proxy_async();
      if (isd) bar_arrive(&dfull[pub_d++ % wg::DSL]);
      else bar_arrive(&xfull[pub_x++ % wg::XS]);
      --pending;
      kinds &= (1 << pending) - 1;
    };
    auto after_issue = [&](bool isd) {
      cp_async_commit();
      kinds = (kinds << 1) | (isd ? 1 : 0);
      ++pending;
      if (pending >= wg::WINFLIGHT) {
        cp_async_wait<wg::WINFLIGHT - 1>();       // the oldest pending item has landed
        publish_oldest();
      }
    };
    auto issue_x = [&](int z, int yw) -> bool {
      const int slot = nx % wg::XS;
      if (nx >= wg::XS && !wbar_wait(&xfree[slot], (uint32_t)((nx / wg::XS - 1) & 1), abort, 1, nx, nd)) return false;
      unsigned char* gb = xring + slot * wg::XGROUP;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const __nv_bfloat16* src = x + (size_t)(((z + d + N - 1) % N) * N + yw) * N * CIN;
        unsigned char* dst = gb + d * wg::XROW;
        for (int c = pt; c < KC * N; c += PRODUCERS) {
          const int kc = c % KC, v = c / KC;
          cp_async16(dst + kc * wg::CH + v * 16, src + (size_t)v * CIN + kc * 8);
        }
      }
      ++nx;
      after_issue(false);
      return true;
    };
    auto issue_d = [&](int r) -> bool {
      const int slot = nd % wg::DSL;
      if (nd >= wg::DSL && !wbar_wait(&dfree[slot], (uint32_t)((nd / wg::DSL - 1) & 1), abort, 2, nd, nx)) return false;
      const __nv_bfloat16* src = dz + (size_t)r * N * COUT;
      unsigned char* db = dring + slot * L::DSLOT;
#pragma unroll
      for (int sh = 0; sh < 3; ++sh) {               // copy sh holds dZ[(u - dx) mod N] at u, dx = sh - 1
        unsigned char* dst = db + sh * L::DCOPY;
        for (int c = pt; c < KCD * N; c += PRODUCERS) {
          const int kc = c % KCD, u = c / KCD;
          const int v = (u - (sh - 1) + N) % N;
          cp_async16(dst + kc * wg::CH + u * 16, src + (size_t)v * COUT + kc * 8);
        }
      }
      ++nd;
      after_issue(true);
      return true;
    };
    bool ok = true;
    for (int r = rg.r0; r < rg.r1 && ok && !*abort;) {
      const int z = r / N, yb = r % N;
      const int ye = (z + 1) * N < rg.r1 ? N : rg.r1 - z * N;
      ok = issue_x(z, (yb - 1 + N) % N) && issue_x(z, yb);
      for (int y = yb; y < ye && ok && !*abort; ++y)
        ok = issue_x(z, (y + 1) % N) && issue_d(z * N + y);
      // The segment's last items are published now: the next segment opens with two input groups,
      // and the second waits for the slot of a group that this segment's last row still reads.
      cp_async_wait<0>();
      if (ok && !*abort)
        while (pending > 0) publish_oldest();
      r = z * N + ye;
    }
    cp_async_wait<0>();
    if (!*abort)
      while (pending > 0) publish_oldest();
  } else if (warp == MMA_WARP) {
    // ---------------------------------------------------------------- MMA issue
    const uint64_t a_base = mdesc_mn(saddr(xring), 128, wg::CH);
    const uint64_t b_base = mdesc_mn(saddr(dring), 128, wg::CH);
    constexpr uint32_t idesc = idesc_bf16_mn(128, L::NCOLS);
    int gx = 0, gd = 0;
    bool ok = true;
    for (int r = rg.r0; r < rg.r1 && ok;) {
      const int z = r / N, yb = r % N;
      const int ye = (z + 1) * N < rg.r1 ? N : rg.r1 - z * N;
      const int nrows = ye - yb;
      ok = __all_sync(0xFFFFFFFFu, wbar_wait(&xfull[gx % wg::XS], (uint32_t)((gx / wg::XS) & 1), abort, 3, gx, gd)) &&
           __all_sync(0xFFFFFFFFu, wbar_wait(&xfull[(gx + 1) % wg::XS], (uint32_t)(((gx + 1) / wg::XS) & 1), abort, 3, gx + 1, gd));
      for (int i = 0; i < nrows && ok; ++i) {
        const int gn = gx + i + 2;
        ok = __all_sync(0xFFFFFFFFu, wbar_wait(&xfull[gn % wg::XS], (uint32_t)((gn / wg::XS) & 1), abort, 4, gn, gd)) &&
             __all_sync(0xFFFFFFFFu, wbar_wait(&dfull[gd % wg::DSL], (uint32_t)((gd / wg::DSL) & 1), abort, 5, gd, gn));
        if (!ok) break;
        tc_after();
        const uint64_t bd = b_base + (uint64_t)((gd % wg::DSL) * (L::DSLOT / 16));
#pragma unroll
        for (int dyi = 0; dyi < 3; ++dyi) {
          const uint64_t ad = a_base + (uint64_t)(((gx + i + dyi) % wg::XS) * (wg::XGROUP / 16));
          const uint32_t dcol = tmem + (uint32_t)(dyi * L::NCOLS);
#pragma unroll
          for (int ks = 0; ks < N / 16; ++ks) mma_acc(dcol, ad + (uint64_t)(ks * 16), bd + (uint64_t)(ks * 16), idesc);
        }
        mma_commit(&dfree[gd % wg::DSL]);           // this dZ row is not read again
        mma_commit(&xfree[(gx + i) % wg::XS]);      // nor is input group y - 1
        ++gd;
      }
      if (!ok) break;
      mma_commit(&xfree[(gx + nrows) % wg::XS]);    // groups ye - 1 and ye end with the segment
      mma_commit(&xfree[(gx + nrows + 1) % wg::XS]);
      gx += nrows + 2;
      r = z * N + ye;
    }
    __syncwarp();
    mma_commit(done);                               // every MMA of this CTA, also after an abort
    // the accumulators are freed only once every MMA issued has completed (bounded)
    for (long i = 0; i < kWSpin && !bar_try(done, 0); ++i) {
    }
  } else {
    // ------------------------------------------------------------------ partials out
    const int q = warp & 3;
    const uint32_t lanes = (uint32_t)(32 * q) << 16;
    const bool ok = wbar_wait(done, 0, abort, 6, 0, 0);
    if (__all_sync(0xFFFFFFFFu, ok)) {
      tc_after();
      const int m = 32 * q + lane;
      float* dst = partials + (size_t)blockIdx.x * 3 * 128 * L::NCOLS;
#pragma unroll
      for (int dyi = 0; dyi < 3; ++dyi) {
#pragma unroll
        for (int c0 = 0; c0 < L::NCOLS; c0 += COUT) {
          float v[COUT];
          const uint32_t ta = tmem + lanes + (uint32_t)(dyi * L::NCOLS + c0);
          if (COUT == 32) tmem_ld32(ta, v); else tmem_ld16(ta, v);
          float* row = dst + ((size_t)dyi * 128 + m) * L::NCOLS + c0;
#pragma unroll
          for (int c = 0; c < COUT; c += 4) *reinterpret_cast<float4*>(row + c) = make_float4(v[c], v[c + 1], v[c + 2], v[c + 3]);
        }
      }
    }
  }

  tc_before();
  __syncthreads();
  if (warp == 0) {
    __syncwarp();
    tc_after();
    tmem_dealloc(tmem, L::TCOLS);
  }
}

// dW[27][COUT][CIN] and db[COUT] from the per-CTA partials [cta][dy][(dz, ci) | ones][(dx, co)],
// summed over CTAs in a fixed order.
template <int CIN, int COUT>
__global__ void wgrad_tc_reduce(const float* __restrict__ partials, int ctas, float* __restrict__ dw,
                                float* __restrict__ db) {
  constexpr int NCOLS = 3 * COUT, PER = 3 * 128 * NCOLS, NW = 27 * COUT * CIN;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NW + COUT; i += gridDim.x * blockDim.x) {
    int dyi, m, n;
    if (i < NW) {
      const int t = i / (COUT * CIN), co = (i / CIN) % COUT, ci = i % CIN;
      dyi = (t / 3) % 3;
      m = (t / 9) * 32 + ci;
      n = (t % 3) * COUT + co;
    } else {
      dyi = 1;
      m = 96;                                      // the ones row
      n = COUT + (i - NW);                         // the unshifted dZ copy
    }
    float s = 0.f;
    for (int c = 0; c < ctas; ++c) s += partials[(size_t)c * PER + ((size_t)dyi * 128 + m) * NCOLS + n];
    if (i < NW) dw[i] = s; else db[i - NW] = s;
  }
}

template <int CIN, int COUT>
int launch_wgrad(const void* x, const void* dz, float* dw, float* db, float* ws, size_t ws_bytes, cudaStream_t s,
                 std::string* err) {
  using L = WLayout<CIN, COUT>;
  auto kern = wgrad_tc_kernel<CIN, COUT>;
  static unsigned configured = 0u;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  if (!(configured & (1u << (dev & 31)))) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, L::BYTES) != cudaSuccess) {
      *err = "tcgen05 wgrad: shared memory opt-in failed";
      return ES_E_CUDA;
    }
    configured |= 1u << (dev & 31);
  }
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t need = (size_t)sms * 3 * 128 * L::NCOLS * sizeof(float);
  if (!ws || ws_bytes < need) {
    *err = "tcgen05 wgrad: workspace needs " + std::to_string(need) + " bytes";
    return ES_E_ARG;
  }
  kern<<<sms, THREADS, L::BYTES, s>>>((const __nv_bfloat16*)x, (const __nv_bfloat16*)dz, ws);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    wgrad_tc_reduce<CIN, COUT><<<64, 256, 0, s>>>(ws, sms, dw, db);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    *err = std::string("tcgen05 wgrad launch: ") + cudaGetErrorString(e);
    return ES_E_CUDA;
  }
  return ES_OK;
}

// ------------------------------------------------------------------ host side
template <int CIN, int COUT, int MODE>
int launch(const void* in, const void* w, const float* bias, void* out, const void* mask, cudaStream_t s,
           std::string* err) {
  using L = Layout<CIN, COUT>;
  auto kern = conv_tc_kernel<CIN, COUT, MODE>;
  static unsigned configured = 0u;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  if (!(configured & (1u << (dev & 31)))) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, L::BYTES) != cudaSuccess) {
      *err = "tcgen05 conv: shared memory opt-in failed";
      return ES_E_CUDA;
    }
    configured |= 1u << (dev & 31);
  }
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  kern<<<sms, THREADS, L::BYTES, s>>>((const __nv_bfloat16*)in, (const __nv_bfloat16*)w, bias, out,
                                      (const __nv_bfloat16*)mask);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    *err = std::string("tcgen05 conv launch: ") + cudaGetErrorString(e);
    return ES_E_CUDA;
  }
  return ES_OK;
}

}  // namespace sgtc

// Dispatch for 128^3 boxes; returns ES_E_UNSUPPORTED for a combination that is not compiled.
__attribute__((visibility("hidden"))) int sg_tc_conv_fwd(int cin, int cout, int mode, const void* in, const void* w,
                                                         const float* bias, void* out, const void* mask,
                                                         cudaStream_t s, std::string* err) {
  using namespace sgtc;
  if ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(w) | reinterpret_cast<uintptr_t>(out) |
       reinterpret_cast<uintptr_t>(mask)) & 15u) {
    *err = "tcgen05 conv: tensors must be 16-byte aligned";
    return ES_E_ARG;
  }
  if (mode == FWD_RELU) {
    if (cin == 16 && cout == 32) return launch<16, 32, FWD_RELU>(in, w, bias, out, mask, s, err);
    if (cin == 32 && cout == 32) return launch<32, 32, FWD_RELU>(in, w, bias, out, mask, s, err);
  } else if (mode == FWD_SIGMOID) {
    if (cin == 32 && cout == 16) return launch<32, 16, FWD_SIGMOID>(in, w, bias, out, mask, s, err);
  } else if (mode == DGRAD_MASK) {
    if (cin == 32 && cout == 32) return launch<32, 32, DGRAD_MASK>(in, w, bias, out, mask, s, err);
    if (cin == 16 && cout == 32) return launch<16, 32, DGRAD_MASK>(in, w, bias, out, mask, s, err);
  }
  *err = "tcgen05 conv: combination not compiled";
  return ES_E_UNSUPPORTED;
}

// Device-side status of the tcgen05 convolutions: nonzero once a wait gave up; reading clears it.
__attribute__((visibility("hidden"))) int sg_tc_status(unsigned* status) {
  unsigned zero = 0;
  cudaError_t e = cudaMemcpyFromSymbol(status, sgtc::g_err, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(sgtc::g_err, &zero, sizeof(unsigned));
  return e == cudaSuccess ? ES_OK : ES_E_CUDA;
}

// Weight gradient at 128^3 on the tensor cores; ES_E_UNSUPPORTED for a combination not compiled.
__attribute__((visibility("hidden"))) int sg_tc_conv_wgrad(int cin, int cout, const void* x, const void* dz, float* dw,
                                                           float* db, float* ws, size_t ws_bytes, cudaStream_t s,
                                                           std::string* err) {
  using namespace sgtc;
  if ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(dz) | reinterpret_cast<uintptr_t>(ws)) & 15u) {
    *err = "tcgen05 wgrad: tensors must be 16-byte aligned";
    return ES_E_ARG;
  }
  if (cin == 16 && cout == 32) return launch_wgrad<16, 32>(x, dz, dw, db, ws, ws_bytes, s, err);
  if (cin == 32 && cout == 32) return launch_wgrad<32, 32>(x, dz, dw, db, ws, ws_bytes, s, err);
  if (cin == 32 && cout == 16) return launch_wgrad<32, 16>(x, dz, dw, db, ws, ws_bytes, s, err);
  *err = "tcgen05 wgrad: combination not compiled";
  return ES_E_UNSUPPORTED;
}

// Workspace of the tensor-core weight gradient (per-CTA partials).
__attribute__((visibility("hidden"))) size_t sg_tc_wgrad_workspace(int cout) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return (size_t)sms * 3 * 128 * 3 * cout * sizeof(float);
}

// The weight gradient's wait record (see g_wdiag); reading clears it.
__attribute__((visibility("hidden"))) int sg_tc_wgrad_diag(int* out4) {
  int zero[4] = {0, 0, 0, 0};
  cudaError_t e = cudaMemcpyFromSymbol(out4, sgtc::g_wdiag, sizeof(zero));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(sgtc::g_wdiag, zero, sizeof(zero));
  return e == cudaSuccess ? ES_OK : ES_E_CUDA;
}
