// Host engine and C ABI of the excursion-set path (declared in include/es_engine.h), plus the
// size-independent kernels: filter tables, final partial ionisation, sphere painting, delta_T
// and layout conversions for the FFT self-tests.
#include <cudaTypedefs.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <algorithm>
#include <vector>

#include "es_engine.h"
#include "es_kernels.cuh"
#include "es_ops.h"

namespace {

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

#define ES_CUDA(call)                                                                   \
  do {                                                                                  \
    cudaError_t err__ = (call);                                                         \
    if (err__ != cudaSuccess)                                                           \
      return fail(ES_E_CUDA, "%s failed: %s", #call, cudaGetErrorString(err__));         \
  } while (0)

struct DeviceGuard {
  int prev = -1;
  cudaError_t err = cudaSuccess;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev) err = cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};

typedef cudaError_t (*launch_fn)(int, const es::OpArgs*, cudaStream_t);
typedef void (*geom_fn)(es::OpGeometry*);

struct SizeEntry { int n; launch_fn launch; geom_fn geom; };
#define ES_SIZE_ENTRY(N) {N, es_launch_##N, es_geometry_##N},
const SizeEntry kSizes[] = {ES_FOR_EACH_SIZE(ES_SIZE_ENTRY)};
#undef ES_SIZE_ENTRY

const SizeEntry* find_size(int n) {
  for (const auto& s : kSizes)
    if (s.n == n) return &s;
  return nullptr;
}

}  // namespace

// per-radius constants derived on the host in double precision
struct RadDev {
  float R;
  float denom;
  int k2cut;      // largest integer k^2 kept by the k-space top-hat (INT_MAX: no cut)
  int r2max;      // largest integer squared cell distance painted by a sphere (-1: none)
};

struct es_plan {
  int n = 0, m = 0, device = 0, sms = 0, max_radii = 0, k2n = 0;
  double box_len = 0;
  float dk = 0;
  const SizeEntry* size = nullptr;
  es::OpGeometry geo{};
  // workspace
  void* base = nullptr;
  size_t bytes = 0;
  float2 *X = nullptr, *Xnyq = nullptr, *T = nullptr, *Tnyq = nullptr, *tw = nullptr;
  float* dR[2] = {nullptr, nullptr};
  uint32_t* flags = nullptr;
  uint32_t* centers = nullptr;
  float* wtab = nullptr;
  float* partials = nullptr;
  unsigned* counters = nullptr;     // [0] reductions, [1] centre count, [2] error word
  float* stats = nullptr;           // [max_radii + 2][4]
  RadDev* rad = nullptr;
  int* thr = nullptr;
  // pinned host staging for per-call parameter uploads
  RadDev* h_rad = nullptr;
  int* h_thr = nullptr;
  std::vector<RadDev> hr;           // this call's per-radius parameters (kernel arguments by value)
  cudaEvent_t staged = nullptr;     // last upload from the staging buffers
  size_t partial_floats = 0;
  // optional per-launch timing: event pairs around every kernel while enabled
  std::vector<cudaEvent_t> prof_events;
  std::vector<int> prof_ops;
  int prof_used = 0;
  int prof_dropped = 0;
  // TMA descriptors: main arrays with z-pass and y-pass boxes, Nyquist planes with z-pass boxes
  CUtensorMap tmX_z, tmX_y, tmXn, tmT_z, tmT_y, tmTn;
  // overlapped radii: a second intermediate spectrum so the column passes of radius r + 1 run on
  // the plan's own stream while the row pass of radius r runs on the caller's
  float2* T2 = nullptr;
  float2* Tnyq2 = nullptr;
  CUtensorMap tmT2_z, tmT2_y, tmT2n;
  cudaStream_t aux = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_col[2] = {nullptr, nullptr}, ev_row[2] = {nullptr, nullptr};
  int overlap = 0;                  // ES_OPT_OVERLAP
  int row_per_sm = 0, col_per_sm = 0;   // ES_OPT_ROW_CTAS / ES_OPT_COL_CTAS caps (0 = by occupancy)
  int col_variant = 1;              // passes: 1 TMA double-buffered (default), 0 synchronous
  int col_tile = 0, row_tile = 0;   // TMA tile-shape variants
  int col_radix = 0, row_radix = 0; // radix schedules of the per-radius passes
  int l2_hints = 1;                 // keep the intermediate spectrum in L2 when it fits
  long l2_bytes = 0;                // device L2 size
  unsigned* err = nullptr;          // device error word (timed-out waits)
  int wait_log2 = 0;                // ES_OPT_WAIT_LOG2 (0: the kernels' default limit)
  int stall = 0;                    // ES_OPT_DEBUG_STALL: pass whose first tile of CTA 0 times out
};

namespace {

constexpr int kStatsStride = 4;

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

struct Layout {
  size_t X, Xnyq, T, Tnyq, T2, Tnyq2, tw, dR0, dR1, flags, centers, wtab, partials, counters, stats, rad, thr, total;
};

Layout layout(int n, int max_radii, size_t partial_floats) {
  const size_t N = n, M = n / 2;
  const size_t k2n = 3 * M * M + 1;
  Layout L{};
  size_t off = 0;
  auto take = [&](size_t bytes) { size_t o = off; off = align_up(off + bytes, 256); return o; };
  L.X = take(N * N * M * 8);
  L.Xnyq = take(N * N * 8);
  L.T = take(N * N * M * 8);
  L.Tnyq = take(N * N * 8);
  L.T2 = take(N * N * M * 8);
  L.Tnyq2 = take(N * N * 8);
  L.tw = take(N * 8);
  L.dR0 = take(N * N * N * 4);
  L.dR1 = take(N * N * N * 4);
  L.flags = take(N * N * N / 8);
  L.centers = take(N * N * N * 4);
  L.wtab = take((size_t)max_radii * k2n * 4);
  L.partials = take(partial_floats * 4);
  L.counters = take(64);
  L.stats = take((size_t)(max_radii + 2) * kStatsStride * 4);
  L.rad = take((size_t)max_radii * sizeof(RadDev));
  L.thr = take(es::PK_MAX_BINS * 4);
  L.total = off;
  return L;
}

int occupancy_grid(const es_plan* p, int tiles, int threads, int smem) {
  // resident CTAs per SM from the thread and shared-memory budgets of sm_103a
  int by_threads = 2048 / threads;
  int by_smem = (227 * 1024) / (smem + 1024);
  int per_sm = by_threads < by_smem ? by_threads : by_smem;
  if (per_sm < 1) per_sm = 1;
  long g = (long)p->sms * per_sm;
  return (int)(tiles < g ? tiles : g);
}

size_t partial_floats_for(int sms, const es::OpGeometry& g) {
  size_t row = (size_t)sms * 16, col = (size_t)sms * 16;
  size_t pk = col * 3 * es::PK_MAX_BINS;
  size_t el = (size_t)sms * 16;
  size_t m = row > pk ? row : pk;
  return m > el ? m : el;
}

// ------------------------------------------------------------------ size-independent kernels

__global__ void filter_table_kernel(float* wtab, int k2n, const RadDev* rad, int nr, float dk,
                                    int filter, int ref_compat, float inv_n3) {
  const long total = (long)nr * k2n;
  for (long idx = blockIdx.x * (long)blockDim.x + threadIdx.x; idx < total;
       idx += (long)gridDim.x * blockDim.x) {
    const int r = (int)(idx / k2n), k2 = (int)(idx % k2n);
    const RadDev rd = rad[r];
    const float W = es::filter_weight(k2, dk, rd.R, rd.k2cut, filter, ref_compat);
    wtab[idx] = W * inv_n3;
  }
}

// Final radius (find_bubbles.cu:142-158): cells flagged at a loop radius stay ionised, the others
// take zeta f, or 1 where f >= 1/zeta.  The flags come from the bitmap or, with `marker`, from
// the lowest mantissa bit of the final delta_R (centre mode of the TMA row pass).  f uses the same
// erfcc as the per-radius sums (relative error ~1e-7; the result is continuous at the threshold).
template <int T>
__global__ void __launch_bounds__(T) final_kernel(const float2* dR, const uint32_t* flags, int marker, long pairs,
                                                  float dc, float denom, const float* stats,
                                                  float zeta, float inv_zeta, int output,
                                                  float2* out, float* partials, unsigned* counter,
                                                  float* nf, float inv_n3) {
  __shared__ float sred[T / 32];
  const es::f32x2 NORM = es::bc2(stats[2]), DC = es::bc2(dc), INV = es::bc2(1.0f / denom);
  float acc = 0.f;
  for (long p = blockIdx.x * (long)T + threadIdx.x; p < pairs; p += (long)gridDim.x * T) {
    const float2 d = dR[p];
    unsigned fx, fy;
    if (marker) {
      fx = __float_as_uint(d.x) & 1u;
      fy = __float_as_uint(d.y) & 1u;
    } else {
      const unsigned long long w = __ldg(reinterpret_cast<const unsigned long long*>(flags) + p / 32);
      const int bit = (int)(p % 32);
      fx = (unsigned)(w >> bit) & 1u;
      fy = (unsigned)(w >> (bit + 32)) & 1u;
    }
    const float2 f = es::upk2(es::mul2(es::erfc_sum_pair(es::mul2(es::sub2(DC, es::pk2(d.x, d.y)), INV)), NORM));
    const float ix = fx ? 1.0f : (f.x >= inv_zeta ? 1.0f : f.x * zeta);
    const float iy = fy ? 1.0f : (f.y >= inv_zeta ? 1.0f : f.y * zeta);
    acc += (1.0f - ix) + (1.0f - iy);
    out[p] = output == 0 ? make_float2(1.0f - ix, 1.0f - iy) : make_float2(ix, iy);
  }
  float total;
  if (es::grid_sum<T>(acc, partials, counter, sred, &total) && threadIdx.x == 0) *nf = total * inv_n3;
}

template <int T>
__global__ void __launch_bounds__(T) delta_T_kernel(const float2* xH, const float2* delta, long pairs,
                                                    float c, float2* dT, float* partials,
                                                    unsigned* counter, float* ave, float inv_n3) {
  __shared__ float sred[T / 32];
  float acc = 0.f;
  for (long p = blockIdx.x * (long)T + threadIdx.x; p < pairs; p += (long)gridDim.x * T) {
    const float2 x = xH[p], d = delta[p];
    const float2 t = make_float2(c * x.x * (1.0f + d.x), c * x.y * (1.0f + d.y));  // delta_T.py:75
    acc += t.x + t.y;
    dT[p] = t;
  }
  float total;
  if (es::grid_sum<T>(acc, partials, counter, sred, &total) && threadIdx.x == 0) *ave = total * inv_n3;
}

// update_sphere_kernel (find_bubbles.cu:73-102): every cell within |d|^2 <= r2max of a centre
// is ionised.  One warp per centre; lanes split the (dz, dy) rows of the ball.
__global__ void paint_kernel(const uint32_t* centers, const unsigned* count, uint32_t* flags, int n,
                             int r2max, int periodic) {
  const unsigned cnt = *count;
  if (r2max < 0) return;
  const long warp = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5;
  const long nwarps = ((long)gridDim.x * blockDim.x) >> 5;
  for (long ci = warp; ci < (long)cnt; ci += nwarps) es::paint_ball(centers[ci], n, r2max, periodic, flags);
}

__global__ void erfc_selftest_kernel(const float* x, float* fast, float* lib, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    // the packed two-argument form the row pass uses (the second argument is a mirror image)
    fast[i] = es::upk2(es::erfc_sum_pair(es::pk2(x[i], -x[i]))).x;
    lib[i] = erfcf(x[i]);
  }
}

// numpy rfftn layout (n, n, n/2+1)  <->  main (n, n, n/2) + nyq (n, n)
__global__ void to_std_kernel(const float2* mainp, const float2* nyq, float2* out, int n) {
  const int m = n / 2;
  const long total = (long)n * n * (m + 1);
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const long row = i / (m + 1);
    const int x = (int)(i % (m + 1));
    out[i] = x < m ? mainp[row * m + x] : nyq[row];
  }
}

__global__ void from_std_kernel(const float2* in, float2* mainp, float2* nyq, int n) {
  const int m = n / 2;
  const long total = (long)n * n * (m + 1);
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const long row = i / (m + 1);
    const int x = (int)(i % (m + 1));
    if (x < m) mainp[row * m + x] = in[i]; else nyq[row] = in[i];
  }
}

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  });
  return fn;
}

// main spectrum [k][j][i < n/2] as 8-byte elements; z-pass box (ti, 1, box), y-pass box (ti, box, 1)
int make_main_map(CUtensorMap* m, void* base, int n, int ti, bool zbox) {
  auto enc = tensor_map_encoder();
  if (!enc) return fail(ES_E_CUDA, "cuTensorMapEncodeTiled is unavailable");
  const cuuint64_t M = n / 2;
  const cuuint32_t box = n < 256 ? n : 256;
  cuuint64_t dims[3] = {M, (cuuint64_t)n, (cuuint64_t)n};
  cuuint64_t strides[2] = {M * 8, (cuuint64_t)n * M * 8};
  cuuint32_t bdim[3] = {(cuuint32_t)ti, zbox ? 1u : box, zbox ? box : 1u};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, base, dims, strides, bdim, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(ES_E_CUDA, "cuTensorMapEncodeTiled (main, n=%d) failed: %d", n, (int)r);
  return ES_OK;
}

// Nyquist plane [k][j] as 8-byte elements; box (ti, box)
int make_nyq_map(CUtensorMap* m, void* base, int n, int ti) {
  auto enc = tensor_map_encoder();
  if (!enc) return fail(ES_E_CUDA, "cuTensorMapEncodeTiled is unavailable");
  const cuuint32_t box = n < 256 ? n : 256;
  cuuint64_t dims[2] = {(cuuint64_t)n, (cuuint64_t)n};
  cuuint64_t strides[1] = {(cuuint64_t)n * 8};
  cuuint32_t bdim[2] = {(cuuint32_t)ti, box};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, base, dims, strides, bdim, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(ES_E_CUDA, "cuTensorMapEncodeTiled (nyq, n=%d) failed: %d", n, (int)r);
  return ES_OK;
}

// TMA descriptors of the plan's spectra for the current column tile width
int encode_maps(es_plan* p) {
  int rc = 0;
  const int n = p->n, ti = p->geo.tcol_ti[p->col_tile];
  if ((rc = make_main_map(&p->tmX_z, p->X, n, ti, true)) || (rc = make_main_map(&p->tmX_y, p->X, n, ti, false)) ||
      (rc = make_main_map(&p->tmT_z, p->T, n, ti, true)) || (rc = make_main_map(&p->tmT_y, p->T, n, ti, false)) ||
      (rc = make_nyq_map(&p->tmXn, p->Xnyq, n, ti)) || (rc = make_nyq_map(&p->tmTn, p->Tnyq, n, ti)) ||
      (rc = make_main_map(&p->tmT2_z, p->T2, n, ti, true)) || (rc = make_main_map(&p->tmT2_y, p->T2, n, ti, false)) ||
      (rc = make_nyq_map(&p->tmT2n, p->Tnyq2, n, ti)))
    return rc;
  return ES_OK;
}

es::OpArgs base_args(const es_plan* p) {
  es::OpArgs a;
  std::memset(&a, 0, sizeof(a));
  a.tw = p->tw;
  a.partials = p->partials;
  a.counter = p->counters;
  a.err = p->err;
  a.variant = p->col_variant;
  a.col_tile = p->col_tile;
  a.row_tile = p->row_tile;
  a.col_radix = p->col_radix;
  a.row_radix = p->row_radix;
  a.scale = 1.0f;
  a.wait_log2 = p->wait_log2;
  return a;
}

// column-pass descriptors: input / output spectra, Nyquist planes, for a z or a y pass
void set_maps(es::OpArgs& a, const CUtensorMap& in, const CUtensorMap& out, const CUtensorMap* in_nyq,
              const CUtensorMap* out_nyq) {
  a.tm_in = in;
  a.tm_out = out;
  if (in_nyq) a.tm_in_nyq = *in_nyq;
  if (out_nyq) a.tm_out_nyq = *out_nyq;
}

// Records the start event of a timed launch; returns the slot or -1 when timing is off/full.
int prof_begin(es_plan* p, int op, cudaStream_t s) {
  if (p->prof_events.empty()) return -1;
  if (2 * (p->prof_used + 1) > (int)p->prof_events.size()) { ++p->prof_dropped; return -1; }
  const int slot = p->prof_used++;
  p->prof_ops[slot] = op;
  cudaEventRecord(p->prof_events[2 * slot], s);
  return slot;
}
void prof_end(es_plan* p, int slot, cudaStream_t s) {
  if (slot >= 0) cudaEventRecord(p->prof_events[2 * slot + 1], s);
}

int run_op(es_plan* p, int op, es::OpArgs a, int grid, cudaStream_t s) {
  a.grid = grid;
  a.stall = (p->stall == ES_STALL_COL_Z_INV && op == es::OP_COL_Z_INV_FILTER) ||
            (p->stall == ES_STALL_ROW_C2R && op == es::OP_ROW_C2R_IONIZE) ||
            (p->stall == ES_STALL_ROW_R2C && op == es::OP_ROW_R2C_SCALE);
  const int slot = prof_begin(p, op, s);
  cudaError_t e = p->size->launch(op, &a, s);
  prof_end(p, slot, s);
  if (e != cudaSuccess) return fail(ES_E_CUDA, "kernel op %d (n=%d) launch failed: %s", op, p->n, cudaGetErrorString(e));
  return ES_OK;
}

int grid_col_z(const es_plan* p, bool pk) {
  if (p->col_variant == 1) {
    const int v = p->col_tile;
    return occupancy_grid(p, p->geo.tcol_tiles_z[v], p->geo.tcol_threads[v],
                          pk ? p->geo.tcol_smem_pk[v] : p->geo.tcol_smem[v]);
  }
  return occupancy_grid(p, p->geo.col_tiles_z, p->geo.col_threads, pk ? p->geo.col_smem_pk : p->geo.col_smem);
}
int grid_col_y(const es_plan* p) {
  if (p->col_variant == 1) {
    const int v = p->col_tile;
    return occupancy_grid(p, p->geo.tcol_tiles_y[v], p->geo.tcol_threads[v], p->geo.tcol_smem[v]);
  }
  return occupancy_grid(p, p->geo.col_tiles_y, p->geo.col_threads, p->geo.col_smem);
}
int grid_row(const es_plan* p, bool prev = false) {
  if (p->col_variant == 1) {
    const int v = p->row_tile;
    return occupancy_grid(p, p->geo.trow_tiles[v], p->geo.trow_threads[v],
                          prev ? p->geo.trow_smem_prev[v] : p->geo.trow_smem[v]);
  }
  return occupancy_grid(p, p->geo.row_tiles, p->geo.row_threads, p->geo.row_smem);
}
int grid_elem(const es_plan* p) { return p->sms * 8; }

// wait until the previous upload from the staging buffers has been consumed
int reuse_staging(es_plan* p) {
  cudaError_t e = cudaEventSynchronize(p->staged);
  if (e != cudaSuccess) return fail(ES_E_CUDA, "cudaEventSynchronize: %s", cudaGetErrorString(e));
  return ES_OK;
}

// forward transform of a real box into the X (into_T = false) or T spectrum; rows -> y -> z
int forward_into(es_plan* p, const float* in, float scale, bool into_T, cudaStream_t s) {
  float2* mainp = into_T ? p->T : p->X;
  float2* nyq = into_T ? p->Tnyq : p->Xnyq;
  const CUtensorMap& mz = into_T ? p->tmT_z : p->tmX_z;
  const CUtensorMap& my = into_T ? p->tmT_y : p->tmX_y;
  const CUtensorMap& mn = into_T ? p->tmTn : p->tmXn;
  es::OpArgs a = base_args(p);
  a.rin = reinterpret_cast<const float2*>(in);
  a.cout = mainp;
  a.scale = scale;
  int rc = run_op(p, es::OP_ROW_R2C_SCALE, a, grid_row(p), s);
  if (rc) return rc;
  a = base_args(p);
  a.cin = mainp; a.cout = mainp; a.cout_nyq = nyq;
  set_maps(a, my, my, nullptr, nullptr);
  if ((rc = run_op(p, es::OP_COL_Y_FWD, a, grid_col_y(p), s))) return rc;
  a = base_args(p);
  a.cin = mainp; a.cin_nyq = nyq; a.cout = mainp; a.cout_nyq = nyq;
  set_maps(a, mz, mz, &mn, &mn);
  return run_op(p, es::OP_COL_Z_FWD, a, grid_col_z(p, false), s);
}

}  // namespace

extern "C" {

int es_version(void) { return 3; }

int es_last_error(char* buf, int len) {
  if (!buf || len <= 0) return ES_E_ARG;
  std::snprintf(buf, (size_t)len, "%s", g_last_error.c_str());
  return ES_OK;
}

int es_supported_sizes(int* sizes, int cap) {
  int c = 0;
  for (const auto& s : kSizes) {
    if (sizes && c < cap) sizes[c] = s.n;
    ++c;
  }
  return c;
}

size_t es_plan_workspace_bytes(int n, int max_radii) {
  const SizeEntry* se = find_size(n);
  if (!se || max_radii <= 0) return 0;
  es::OpGeometry g{};
  se->geom(&g);
  // partial-sum space is sized for the largest GB300 part (152 SMs) when no device is queried
  return layout(n, max_radii, partial_floats_for(152, g)).total;
}

int es_plan_create(int n, double box_len, int max_radii, es_plan** out) {
  if (!out) return fail(ES_E_ARG, "es_plan_create: plan pointer is NULL");
  *out = nullptr;
  const SizeEntry* se = find_size(n);
  if (!se) return fail(ES_E_UNSUPPORTED, "es_plan_create: HII_DIM=%d has no compiled kernels", n);
  if (!(box_len > 0)) return fail(ES_E_ARG, "es_plan_create: BOX_LEN must be positive");
  if (max_radii <= 0 || max_radii > 4096) return fail(ES_E_ARG, "es_plan_create: max_radii out of range");
  es_plan* p = new es_plan();
  p->n = n; p->m = n / 2; p->box_len = box_len; p->max_radii = max_radii; p->size = se;
  p->k2n = 3 * p->m * p->m + 1;
  p->hr.reserve(max_radii);         // es_ionize fills it without reallocating
  // DELTA_K = float32(2 pi / float32(BOX_LEN)) (delta_T.py:52)
  p->dk = (float)(2.0 * M_PI / (double)(float)box_len);
  se->geom(&p->geo);
  auto cleanup = [&](int code) { es_plan_destroy(p); return code; };
  if (cudaGetDevice(&p->device) != cudaSuccess) return cleanup(fail(ES_E_CUDA, "no CUDA device"));
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, p->device) != cudaSuccess) return cleanup(fail(ES_E_CUDA, "cudaGetDeviceProperties failed"));
  p->sms = prop.multiProcessorCount;
  p->l2_bytes = prop.l2CacheSize;
  p->partial_floats = partial_floats_for(p->sms, p->geo);
  Layout L = layout(n, max_radii, p->partial_floats);
  if (cudaMalloc(&p->base, L.total) != cudaSuccess) {
    cudaGetLastError();
    return cleanup(fail(ES_E_NOMEM, "es_plan_create: cannot allocate %zu bytes of workspace", L.total));
  }
  p->bytes = L.total;
  char* b = static_cast<char*>(p->base);
  p->X = (float2*)(b + L.X); p->Xnyq = (float2*)(b + L.Xnyq);
  p->T = (float2*)(b + L.T); p->Tnyq = (float2*)(b + L.Tnyq);
  p->T2 = (float2*)(b + L.T2); p->Tnyq2 = (float2*)(b + L.Tnyq2);
  p->tw = (float2*)(b + L.tw);
  p->dR[0] = (float*)(b + L.dR0); p->dR[1] = (float*)(b + L.dR1);
  p->flags = (uint32_t*)(b + L.flags);
  p->centers = (uint32_t*)(b + L.centers);
  p->wtab = (float*)(b + L.wtab);
  p->partials = (float*)(b + L.partials);
  p->counters = (unsigned*)(b + L.counters);
  p->stats = (float*)(b + L.stats);
  p->rad = (RadDev*)(b + L.rad);
  p->thr = (int*)(b + L.thr);
  p->err = p->counters + 2;
  if (int rc = encode_maps(p)) return cleanup(rc);
  if (cudaMallocHost(&p->h_rad, sizeof(RadDev) * max_radii) != cudaSuccess ||
      cudaMallocHost(&p->h_thr, sizeof(int) * es::PK_MAX_BINS) != cudaSuccess)
    return cleanup(fail(ES_E_NOMEM, "es_plan_create: pinned staging allocation failed"));
  if (cudaEventCreateWithFlags(&p->staged, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&p->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&p->ev_col[0], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&p->ev_col[1], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&p->ev_row[0], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&p->ev_row[1], cudaEventDisableTiming) != cudaSuccess)
    return cleanup(fail(ES_E_CUDA, "es_plan_create: cudaEventCreate failed"));
  if (cudaStreamCreateWithFlags(&p->aux, cudaStreamNonBlocking) != cudaSuccess)
    return cleanup(fail(ES_E_CUDA, "es_plan_create: cudaStreamCreate failed"));
  // twiddles w_n^m = exp(-2 pi i m / n) in double, rounded once
  std::vector<float2> tw(n);
  for (int m = 0; m < n; ++m) {
    const double ang = -2.0 * M_PI * (double)m / (double)n;
    tw[m] = make_float2((float)std::cos(ang), (float)std::sin(ang));
  }
  if (cudaMemcpy(p->tw, tw.data(), n * sizeof(float2), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(p->counters, 0, 64) != cudaSuccess || cudaMemset(p->stats, 0, (size_t)(max_radii + 2) * kStatsStride * 4) != cudaSuccess)
    return cleanup(fail(ES_E_CUDA, "es_plan_create: initial upload failed"));
  if (cudaEventRecord(p->staged, 0) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess)
    return cleanup(fail(ES_E_CUDA, "es_plan_create: synchronisation failed"));
  *out = p;
  return ES_OK;
}

int es_plan_destroy(es_plan* p) {
  if (!p) return ES_OK;
  DeviceGuard g(p->device);
  if (p->staged) cudaEventSynchronize(p->staged);
  if (p->aux) cudaStreamSynchronize(p->aux);
  if (p->base) cudaFree(p->base);
  if (p->h_rad) cudaFreeHost(p->h_rad);
  if (p->h_thr) cudaFreeHost(p->h_thr);
  if (p->staged) cudaEventDestroy(p->staged);
  for (cudaEvent_t e : {p->ev_fork, p->ev_col[0], p->ev_col[1], p->ev_row[0], p->ev_row[1]})
    if (e) cudaEventDestroy(e);
  if (p->aux) cudaStreamDestroy(p->aux);
  for (cudaEvent_t e : p->prof_events) cudaEventDestroy(e);
  delete p;
  return ES_OK;
}

int es_forward(es_plan* p, const float* delta, void* stream) {
  if (!p || !delta) return fail(ES_E_ARG, "es_forward: NULL argument");
  DeviceGuard g(p->device);
  return forward_into(p, delta, 1.0f, false, (cudaStream_t)stream);
}

int es_ionize(es_plan* p, const es_ionize_params* prm, float* out, float* nf, void* stream) {
  if (!p || !prm || !out || !nf) return fail(ES_E_ARG, "es_ionize: NULL argument");
  const int nr = prm->n_radii;
  if (nr < 1 || nr > p->max_radii || !prm->radii)
    return fail(ES_E_ARG, "es_ionize: n_radii=%d outside [1, %d]", nr, p->max_radii);
  if (prm->filter_type < 0 || prm->filter_type > 2) return fail(ES_E_ARG, "es_ionize: filter_type must be 0, 1 or 2");
  if (prm->update < 0 || prm->update > 1) return fail(ES_E_ARG, "es_ionize: update must be 0 or 1");
  if (!(prm->zeta > 0)) return fail(ES_E_ARG, "es_ionize: zeta must be positive");
  for (int r = 0; r < nr; ++r)
    if (!(prm->radii[r].R > 0) || !(prm->radii[r].denom > 0) || !std::isfinite(prm->radii[r].denom))
      return fail(ES_E_ARG, "es_ionize: radius %d has R=%g denom=%g", r, prm->radii[r].R, prm->radii[r].denom);
  DeviceGuard g(p->device);
  cudaStream_t s = (cudaStream_t)stream;
  int rc = 0;
  const double scale = p->box_len / p->n;
  p->hr.resize(nr);
  for (int r = 0; r < nr; ++r) {
    RadDev rd;
    rd.R = prm->radii[r].R;
    rd.denom = prm->radii[r].denom;
    // k-space top-hat keeps modes with (dk |k| R) * 0.413566994 <= 1 (find_bubbles.cu:34-37)
    rd.k2cut = 0x7fffffff;
    if (prm->filter_type == 1 || (prm->ref_compat && prm->filter_type == 0)) {
      const double R = rd.R, dk = p->dk;
      long m = (long)std::floor(std::pow(1.0 / (0.413566994 * dk * R), 2)) + 2;
      while (m >= 0 && (dk * std::sqrt((double)m) * R) * 0.413566994 > 1.0) --m;
      rd.k2cut = (int)(m < p->k2n ? m : p->k2n);
    }
    // sphere: cells with integer |d|^2 < R_cells^2 (find_bubbles.cu:97-98)
    if (prm->ref_compat) {
      const float r2 = rd.R * rd.R;                  // R in Mpc used as cells, float32 compare
      long m = (long)std::floor((double)r2);
      while (m >= 0 && (float)m >= r2) --m;
      rd.r2max = (int)m;
    } else {
      const double rc2 = std::pow((double)rd.R / scale, 2);
      long m = (long)std::floor(rc2);
      while (m >= 0 && (double)m >= rc2) --m;
      rd.r2max = (int)m;
    }
    p->hr[r] = rd;
  }
  // Only the synchronous column pass reads the radii from device memory (its filter tables); the
  // TMA passes take them as kernel arguments, so with those the call does no host-to-device copy
  // and no host wait, and can be captured in a CUDA graph.
  if (p->col_variant == 0) {
    if ((rc = reuse_staging(p))) return rc;
    std::copy(p->hr.begin(), p->hr.end(), p->h_rad);
    ES_CUDA(cudaMemcpyAsync(p->rad, p->h_rad, sizeof(RadDev) * nr, cudaMemcpyHostToDevice, s));
    ES_CUDA(cudaEventRecord(p->staged, s));
  }
  const float inv_n3 = (float)(1.0 / ((double)p->n * p->n * p->n));
  int slot = -1;
  if (p->col_variant == 0) {        // the synchronous column pass gathers W from per-radius tables
    slot = prof_begin(p, ES_PROF_FILTER_TABLE, s);
    filter_table_kernel<<<p->sms * 4, 256, 0, s>>>(p->wtab, p->k2n, p->rad, nr, p->dk, prm->filter_type,
                                                     prm->ref_compat, inv_n3);
    prof_end(p, slot, s);
    ES_CUDA(cudaGetLastError());
  }
  const size_t N3 = (size_t)p->n * p->n * p->n;
  // centre mode on the TMA row pass carries the flags in delta_R itself; the bitmap serves the
  // synchronous row pass and sphere painting
  const int marker = (p->col_variant == 1 && prm->update == 0) ? 1 : 0;
  if (!marker) ES_CUDA(cudaMemsetAsync(p->flags, 0, N3 / 8, s));
  const float inv_zeta = (float)(1.0 / (double)prm->zeta);
  // The intermediate spectrum T is written by the z pass, rewritten by the y pass and read by the
  // row pass; when it fits comfortably in L2 it is kept there (evict_last) while the input
  // spectrum and the delta_R boxes stream (evict_first), and the row pass drops T's consumed
  // lines so the dead data is never written back.
  const size_t t_bytes = (size_t)p->n * p->n * (p->m + 1) * sizeof(float2);
  const bool keep_T = p->l2_hints && (double)t_bytes <= 0.6 * (double)p->l2_bytes;
  const int keep = keep_T ? es::ES_HINT_EVICT_LAST : es::ES_HINT_NORMAL;
  // Intermediate spectra: T for every radius, or T / T2 alternating when radii overlap.
  struct TBuf { float2* main; float2* nyq; const CUtensorMap* mz; const CUtensorMap* my; const CUtensorMap* mn; };
  const TBuf tb[2] = {{p->T, p->Tnyq, &p->tmT_z, &p->tmT_y, &p->tmTn},
                      {p->T2, p->Tnyq2, &p->tmT2_z, &p->tmT2_y, &p->tmT2n}};
  const bool ovl = p->overlap != 0 && nr > 1;
  auto capped = [&](int grid, int per_sm) { return (ovl && per_sm > 0 && grid > p->sms * per_sm) ? p->sms * per_sm : grid; };
  const int g_z = capped(grid_col_z(p, false), p->col_per_sm), g_y = capped(grid_col_y(p), p->col_per_sm);
  const int g_row = capped(grid_row(p, true), p->row_per_sm);
  // z inverse with the filter of radius r, then y inverse, into the radius' intermediate spectrum
  auto col_passes = [&](int r, cudaStream_t cs) -> int {
    const TBuf& t = tb[ovl ? (r & 1) : 0];
    es::OpArgs a = base_args(p);
    a.cin = p->X; a.cin_nyq = p->Xnyq; a.cout = t.main; a.cout_nyq = t.nyq;
    a.wtab = p->wtab + (size_t)r * p->k2n;
    a.scale = prm->growth_scale;
    a.fR = p->hr[r].R;
    a.fk2cut = p->hr[r].k2cut;
    a.filter = prm->filter_type;
    a.ref_compat = prm->ref_compat;
    a.dk = p->dk;
    a.inv_n3 = inv_n3;
    a.hint_in = p->l2_hints ? es::ES_HINT_EVICT_FIRST : es::ES_HINT_NORMAL;
    a.hint_out = keep;
    set_maps(a, p->tmX_z, *t.mz, &p->tmXn, t.mn);
    if (int e = run_op(p, es::OP_COL_Z_INV_FILTER, a, g_z, cs)) return e;
    a = base_args(p);
    a.cin = t.main; a.cin_nyq = t.nyq; a.cout = t.main;
    a.hint_in = keep;
    a.hint_out = keep;
    set_maps(a, *t.my, *t.my, nullptr, nullptr);
    return run_op(p, es::OP_COL_Y_INV, a, g_y, cs);
  };
  // x C2R with the excursion-set epilogue of radius r (and the sphere painting of radius r - 1)
  auto row_pass = [&](int r) -> int {
    const TBuf& t = tb[ovl ? (r & 1) : 0];
    if (prm->update == 1 && r > 0) ES_CUDA(cudaMemsetAsync(p->counters + 1, 0, sizeof(unsigned), s));
    es::OpArgs a = base_args(p);
    a.cin = t.main;
    a.rout = reinterpret_cast<float2*>(p->dR[r & 1]);
    a.prev = reinterpret_cast<const float2*>(p->dR[(r + 1) & 1]);
    a.has_prev = r > 0;
    a.flags = p->flags;
    a.dc = prm->delta_c;
    a.denom = prm->radii[r].denom;
    a.denom_prev = r > 0 ? prm->radii[r - 1].denom : 1.0f;
    a.stats_prev = p->stats + (size_t)(r > 0 ? r - 1 : 0) * kStatsStride;
    a.stats_out = p->stats + (size_t)r * kStatsStride;
    a.inv_zeta = inv_zeta;
    a.update = prm->update;
    a.marker = marker;
    a.centers = p->centers;
    a.center_count = p->counters + 1;
    a.fc_mean = prm->fc_mean_ps;
    a.normalize = prm->normalize_mean;
    a.hint_in = p->l2_hints ? es::ES_HINT_EVICT_FIRST : es::ES_HINT_NORMAL;
    a.discard_in = p->l2_hints;
    if (int e = run_op(p, es::OP_ROW_C2R_IONIZE, a, g_row, s)) return e;
    if (prm->update == 1 && r > 0) {
      const int ps = prof_begin(p, ES_PROF_PAINT, s);
      paint_kernel<<<p->sms * 4, 256, 0, s>>>(p->centers, p->counters + 1, p->flags, p->n,
                                              p->hr[r - 1].r2max, prm->ref_compat ? 0 : 1);
      prof_end(p, ps, s);
      ES_CUDA(cudaGetLastError());
    }
    return ES_OK;
  };
  if (!ovl) {
    for (int r = 0; r < nr; ++r)
      if ((rc = col_passes(r, s)) || (rc = row_pass(r))) return rc;
  } else {
    // Software pipeline over two streams: the column passes of radius r + 1 (plan stream) run
    // while the row pass of radius r (caller's stream) runs.  Radius r + 1 writes the spectrum
    // that radius r - 1 read, so it waits for that row pass; each row pass waits for its own
    // column passes.  Everything the plan stream does is joined back before the last row pass.
    // On a failed launch, whatever the plan stream holds is still joined to the caller's stream.
    auto joined = [&](int code) {
      if (cudaEventRecord(p->ev_fork, p->aux) == cudaSuccess) cudaStreamWaitEvent(s, p->ev_fork, 0);
      return code;
    };
    ES_CUDA(cudaEventRecord(p->ev_fork, s));
    ES_CUDA(cudaStreamWaitEvent(p->aux, p->ev_fork, 0));
    if ((rc = col_passes(0, p->aux))) return joined(rc);
    if (cudaEventRecord(p->ev_col[0], p->aux) != cudaSuccess) return joined(fail(ES_E_CUDA, "es_ionize: event record failed"));
    for (int r = 0; r < nr; ++r) {
      if (r + 1 < nr) {
        if (r >= 1 && cudaStreamWaitEvent(p->aux, p->ev_row[(r + 1) & 1], 0) != cudaSuccess)
          return joined(fail(ES_E_CUDA, "es_ionize: stream wait failed"));
        if ((rc = col_passes(r + 1, p->aux))) return joined(rc);
        if (cudaEventRecord(p->ev_col[(r + 1) & 1], p->aux) != cudaSuccess)
          return joined(fail(ES_E_CUDA, "es_ionize: event record failed"));
      }
      if (cudaStreamWaitEvent(s, p->ev_col[r & 1], 0) != cudaSuccess)
        return joined(fail(ES_E_CUDA, "es_ionize: stream wait failed"));
      if ((rc = row_pass(r))) return joined(rc);
      if (cudaEventRecord(p->ev_row[r & 1], s) != cudaSuccess)
        return joined(fail(ES_E_CUDA, "es_ionize: event record failed"));
    }
  }
  slot = prof_begin(p, ES_PROF_FINAL, s);
  final_kernel<256><<<grid_elem(p), 256, 0, s>>>(
      reinterpret_cast<const float2*>(p->dR[(nr - 1) & 1]), p->flags, marker, (long)(N3 / 2), prm->delta_c,
      prm->radii[nr - 1].denom, p->stats + (size_t)(nr - 1) * kStatsStride, prm->zeta, inv_zeta,
      prm->output, reinterpret_cast<float2*>(out), p->partials, p->counters, nf, inv_n3);
  prof_end(p, slot, s);
  ES_CUDA(cudaGetLastError());
  return ES_OK;
}

int es_delta_T(es_plan* p, const float* xH, const float* delta, float c, float* dT, float* ave, void* stream) {
  if (!p || !xH || !delta || !dT || !ave) return fail(ES_E_ARG, "es_delta_T: NULL argument");
  DeviceGuard g(p->device);
  const size_t N3 = (size_t)p->n * p->n * p->n;
  const int slot = prof_begin(p, ES_PROF_DELTA_T, (cudaStream_t)stream);
  delta_T_kernel<256><<<grid_elem(p), 256, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<const float2*>(xH), reinterpret_cast<const float2*>(delta), (long)(N3 / 2), c,
      reinterpret_cast<float2*>(dT), p->partials, p->counters, ave, (float)(1.0 / (double)N3));
  prof_end(p, slot, (cudaStream_t)stream);
  ES_CUDA(cudaGetLastError());
  return ES_OK;
}

int es_power_spectrum(es_plan* p, const float* dT, const float* ave, const int* thr, int nbins,
                      int dimensional, float* out, void* stream) {
  if (!p || !dT || !ave || !thr || !out) return fail(ES_E_ARG, "es_power_spectrum: NULL argument");
  if (nbins < 1 || nbins > es::PK_MAX_BINS) return fail(ES_E_ARG, "es_power_spectrum: nbins=%d outside [1, %d]", nbins, es::PK_MAX_BINS);
  for (int b = 1; b < nbins; ++b)
    if (thr[b] < thr[b - 1]) return fail(ES_E_ARG, "es_power_spectrum: k^2 thresholds must be non-decreasing");
  DeviceGuard g(p->device);
  cudaStream_t s = (cudaStream_t)stream;
  int rc = reuse_staging(p);
  if (rc) return rc;
  std::memcpy(p->h_thr, thr, sizeof(int) * nbins);
  ES_CUDA(cudaMemcpyAsync(p->thr, p->h_thr, sizeof(int) * nbins, cudaMemcpyHostToDevice, s));
  ES_CUDA(cudaEventRecord(p->staged, s));
  const double L = (double)(float)p->box_len;
  es::OpArgs a = base_args(p);
  a.rin = reinterpret_cast<const float2*>(dT);
  a.cout = p->T;
  a.ave = ave;
  a.pk_norm = (float)(L * L * L / ((double)p->n * p->n * p->n));
  a.dimensional = dimensional;
  if ((rc = run_op(p, es::OP_ROW_R2C_PK, a, grid_row(p), s))) return rc;
  a = base_args(p);
  a.cin = p->T; a.cout = p->T; a.cout_nyq = p->Tnyq;
  set_maps(a, p->tmT_y, p->tmT_y, nullptr, nullptr);
  if ((rc = run_op(p, es::OP_COL_Y_FWD, a, grid_col_y(p), s))) return rc;
  a = base_args(p);
  a.cin = p->T; a.cin_nyq = p->Tnyq;
  set_maps(a, p->tmT_z, p->tmT_z, &p->tmTn, &p->tmTn);
  a.thr = p->thr; a.nbins = nbins; a.dk = p->dk; a.volume = (float)(L * L * L);
  a.pk_out = out;
  return run_op(p, es::OP_COL_Z_FWD_PK, a, grid_col_z(p, true), s);
}

int es_fft_r2c(es_plan* p, const float* in, void* out, void* stream) {
  if (!p || !in || !out) return fail(ES_E_ARG, "es_fft_r2c: NULL argument");
  DeviceGuard g(p->device);
  cudaStream_t s = (cudaStream_t)stream;
  int rc = forward_into(p, in, 1.0f, true, s);
  if (rc) return rc;
  to_std_kernel<<<p->sms * 8, 256, 0, s>>>(p->T, p->Tnyq, (float2*)out, p->n);
  ES_CUDA(cudaGetLastError());
  return ES_OK;
}

int es_fft_c2r(es_plan* p, const void* in, float* out, void* stream) {
  if (!p || !in || !out) return fail(ES_E_ARG, "es_fft_c2r: NULL argument");
  DeviceGuard g(p->device);
  cudaStream_t s = (cudaStream_t)stream;
  from_std_kernel<<<p->sms * 8, 256, 0, s>>>((const float2*)in, p->T, p->Tnyq, p->n);
  ES_CUDA(cudaGetLastError());
  es::OpArgs a = base_args(p);
  a.cin = p->T; a.cin_nyq = p->Tnyq; a.cout = p->T; a.cout_nyq = p->Tnyq;
  set_maps(a, p->tmT_z, p->tmT_z, &p->tmTn, &p->tmTn);
  int rc = run_op(p, es::OP_COL_Z_INV, a, grid_col_z(p, false), s);
  if (rc) return rc;
  a = base_args(p);
  a.cin = p->T; a.cin_nyq = p->Tnyq; a.cout = p->T;
  set_maps(a, p->tmT_y, p->tmT_y, nullptr, nullptr);
  if ((rc = run_op(p, es::OP_COL_Y_INV, a, grid_col_y(p), s))) return rc;
  a = base_args(p);
  a.cin = p->T;
  a.rout = reinterpret_cast<float2*>(out);
  return run_op(p, es::OP_ROW_C2R_STORE, a, grid_row(p), s);
}

// ------------------------------------------------------------------ allocation-free delta_T
// Scratch of es_delta_T_noalloc: one partial sum per CTA (at most ES_NOALLOC_MAX_CTAS) and, in
// the word after them, the CTAs' arrival counter.  It is a static device array, so every GPU that
// loads this library holds these 16.25 KiB until the process exits, and every call shares it.
static __device__ __align__(256) float g_noalloc_scratch[ES_NOALLOC_MAX_CTAS + 64];

namespace {
std::mutex g_noalloc_mu;
constexpr int kNoallocMaxDevices = 64;
void* g_noalloc_ptr[kNoallocMaxDevices] = {};
int g_noalloc_grid[kNoallocMaxDevices] = {};
}  // namespace

int es_delta_T_noalloc(int n, const float* xH, const float* delta, float c, float* dT, float* ave, void* stream) {
  if (!xH || !delta || !dT || !ave) return fail(ES_E_ARG, "es_delta_T_noalloc: NULL argument");
  if (n < 2 || n % 2 || n > ES_NOALLOC_MAX_N)
    return fail(ES_E_ARG, "es_delta_T_noalloc: HII_DIM=%d must be even and at most %d", n, ES_NOALLOC_MAX_N);
  int dev = 0;
  ES_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoallocMaxDevices) return fail(ES_E_ARG, "es_delta_T_noalloc: device %d out of range", dev);
  void* base = nullptr;
  int grid = 0;
  {
    // first call on this device: resolve the device address of the static scratch (host code
    // cannot use the array's name as a device pointer) and size the grid to the device
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
      void* ptr = nullptr;
      ES_CUDA(cudaGetSymbolAddress(&ptr, g_noalloc_scratch));
      int sms = 0;
      ES_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
      g_noalloc_grid[dev] = sms * 8 < ES_NOALLOC_MAX_CTAS ? sms * 8 : ES_NOALLOC_MAX_CTAS;
      g_noalloc_ptr[dev] = ptr;
    }
    base = g_noalloc_ptr[dev];
    grid = g_noalloc_grid[dev];
  }
  float* partials = static_cast<float*>(base);
  unsigned* counter = reinterpret_cast<unsigned*>(partials + ES_NOALLOC_MAX_CTAS);
  cudaStream_t s = (cudaStream_t)stream;
  // the counter must start at zero; a call that never finished would have left it elsewhere
  ES_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned), s));
  const size_t N3 = (size_t)n * n * n;
  delta_T_kernel<256><<<grid, 256, 0, s>>>(
      reinterpret_cast<const float2*>(xH), reinterpret_cast<const float2*>(delta), (long)(N3 / 2), c,
      reinterpret_cast<float2*>(dT), partials, counter, ave, (float)(1.0 / (double)N3));
  ES_CUDA(cudaGetLastError());
  return ES_OK;
}

int es_selftest_erfc(const float* x, float* fast, float* lib, int n, void* stream) {
  if (!x || !fast || !lib || n < 0) return fail(ES_E_ARG, "es_selftest_erfc: bad arguments");
  if (n == 0) return ES_OK;
  erfc_selftest_kernel<<<(n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024, 256, 0, (cudaStream_t)stream>>>(x, fast, lib, n);
  ES_CUDA(cudaGetLastError());
  return ES_OK;
}

int es_plan_set_option(es_plan* p, int option, int value) {
  if (!p) return fail(ES_E_ARG, "es_plan_set_option: NULL plan");
  switch (option) {
    case ES_OPT_COL_VARIANT:
      if (value != 0 && value != 1) return fail(ES_E_ARG, "es_plan_set_option: column variant must be 0 or 1");
      p->col_variant = value;
      return ES_OK;
    case ES_OPT_COL_TILE: {
      if (value < 0 || value >= es::kColTileVariants) return fail(ES_E_ARG, "es_plan_set_option: column tile variant out of range");
      const int old = p->col_tile;
      p->col_tile = value;
      if (int rc = encode_maps(p)) { p->col_tile = old; encode_maps(p); return rc; }
      return ES_OK;
    }
    case ES_OPT_ROW_TILE:
      if (value < 0 || value >= es::kRowTileVariants) return fail(ES_E_ARG, "es_plan_set_option: row tile variant out of range");
      p->row_tile = value;
      return ES_OK;
    case ES_OPT_L2_HINTS:
      if (value != 0 && value != 1) return fail(ES_E_ARG, "es_plan_set_option: L2 hints must be 0 or 1");
      p->l2_hints = value;
      return ES_OK;
    case ES_OPT_COL_RADIX:
    case ES_OPT_ROW_RADIX:
      if (value != 0 && value != 1) return fail(ES_E_ARG, "es_plan_set_option: radix schedule must be 0 or 1");
      (option == ES_OPT_COL_RADIX ? p->col_radix : p->row_radix) = value;
      return ES_OK;
    case ES_OPT_OVERLAP:
      if (value != 0 && value != 1) return fail(ES_E_ARG, "es_plan_set_option: overlap must be 0 or 1");
      p->overlap = value;
      return ES_OK;
    case ES_OPT_ROW_CTAS:
    case ES_OPT_COL_CTAS:
      if (value < 0 || value > 16) return fail(ES_E_ARG, "es_plan_set_option: CTAs per SM must be in [0, 16]");
      (option == ES_OPT_ROW_CTAS ? p->row_per_sm : p->col_per_sm) = value;
      return ES_OK;
    case ES_OPT_WAIT_LOG2:
      if (value != 0 && (value < 8 || value > 30)) return fail(ES_E_ARG, "es_plan_set_option: wait limit must be 0 or 8..30");
      p->wait_log2 = value;
      return ES_OK;
    case ES_OPT_DEBUG_STALL:
      if (value < 0 || value > ES_STALL_ROW_R2C) return fail(ES_E_ARG, "es_plan_set_option: unknown debug stall %d", value);
      p->stall = value;
      return ES_OK;
    default:
      return fail(ES_E_ARG, "es_plan_set_option: unknown option %d", option);
  }
}

int es_plan_get_option(es_plan* p, int option, int* value) {
  if (!p || !value) return fail(ES_E_ARG, "es_plan_get_option: NULL argument");
  switch (option) {
    case ES_OPT_COL_VARIANT: *value = p->col_variant; return ES_OK;
    case ES_OPT_COL_TILE: *value = p->col_tile; return ES_OK;
    case ES_OPT_ROW_TILE: *value = p->row_tile; return ES_OK;
    case ES_OPT_L2_HINTS: *value = p->l2_hints; return ES_OK;
    case ES_OPT_COL_RADIX: *value = p->col_radix; return ES_OK;
    case ES_OPT_ROW_RADIX: *value = p->row_radix; return ES_OK;
    case ES_OPT_OVERLAP: *value = p->overlap; return ES_OK;
    case ES_OPT_ROW_CTAS: *value = p->row_per_sm; return ES_OK;
    case ES_OPT_COL_CTAS: *value = p->col_per_sm; return ES_OK;
    case ES_OPT_WAIT_LOG2: *value = p->wait_log2; return ES_OK;
    case ES_OPT_DEBUG_STALL: *value = p->stall; return ES_OK;
    default: return fail(ES_E_ARG, "es_plan_get_option: unknown option %d", option);
  }
}

int es_plan_check(es_plan* p, void* stream) {
  if (!p) return fail(ES_E_ARG, "es_plan_check: NULL plan");
  DeviceGuard g(p->device);
  unsigned word = 0;
  ES_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  ES_CUDA(cudaMemcpy(&word, p->err, sizeof(unsigned), cudaMemcpyDeviceToHost));
  if (word) {
    ES_CUDA(cudaMemset(p->err, 0, sizeof(unsigned)));
    return fail(ES_E_DEVICE, "a device-side wait timed out (error word 0x%x); results of the affected calls are invalid", word);
  }
  return ES_OK;
}

int es_profile_enable(es_plan* p, int max_launches) {
  if (!p || max_launches < 0 || max_launches > (1 << 22)) return fail(ES_E_ARG, "es_profile_enable: bad arguments");
  DeviceGuard g(p->device);
  ES_CUDA(cudaDeviceSynchronize());
  for (cudaEvent_t e : p->prof_events) cudaEventDestroy(e);
  p->prof_events.clear();
  p->prof_ops.assign(max_launches, -1);
  p->prof_used = 0;
  p->prof_dropped = 0;
  for (int i = 0; i < 2 * max_launches; ++i) {
    cudaEvent_t e;
    ES_CUDA(cudaEventCreate(&e));
    p->prof_events.push_back(e);
  }
  return ES_OK;
}

int es_profile_reset(es_plan* p) {
  if (!p) return fail(ES_E_ARG, "es_profile_reset: NULL plan");
  p->prof_used = 0;
  p->prof_dropped = 0;
  return ES_OK;
}

int es_profile_read(es_plan* p, float* total_ms, int* counts, int nops) {
  if (!p || !total_ms || !counts || nops < ES_PROF_COUNT) return fail(ES_E_ARG, "es_profile_read: bad arguments");
  DeviceGuard g(p->device);
  for (int i = 0; i < nops; ++i) { total_ms[i] = 0.f; counts[i] = 0; }
  for (int k = 0; k < p->prof_used; ++k) {
    float ms = 0.f;
    ES_CUDA(cudaEventSynchronize(p->prof_events[2 * k + 1]));
    ES_CUDA(cudaEventElapsedTime(&ms, p->prof_events[2 * k], p->prof_events[2 * k + 1]));
    const int op = p->prof_ops[k];
    if (op >= 0 && op < nops) { total_ms[op] += ms; counts[op] += 1; }
  }
  return p->prof_dropped;
}

}  // extern "C"
