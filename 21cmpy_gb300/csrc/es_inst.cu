// Per-box-size instantiation of the FFT pass kernels.  Compiled once per supported N with
// -DES_N=<N>; each object exports es_launch_<N>(), which es_engine.cu dispatches to.
#include "es_kernels.cuh"
#include "es_tma.cuh"
#include "es_rows.cuh"
#include "es_ops.h"

#ifndef ES_N
#error "compile with -DES_N=<box size>"
#endif

namespace es {

// One static record per kernel (the template argument is the kernel itself) and device: opt in to
// more than 48 KB of dynamic shared memory once, and remember how many CTAs of it fit on the
// device at once (registers included), so a persistent grid never exceeds one resident wave.
template <auto Kernel>
static cudaError_t launch(int smem, const OpArgs& a, int threads, cudaStream_t s) {
  static unsigned configured = 0u;
  static int resident[32];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned bit = 1u << (dev & 31);
  if (!(configured & bit)) {
    e = cudaFuncSetAttribute(Kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0, sms = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, Kernel, threads, smem);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    resident[dev & 31] = (per_sm > 0 ? per_sm : 1) * sms;
    configured |= bit;
  }
  const int grid = a.grid < resident[dev & 31] ? a.grid : resident[dev & 31];
  Kernel<<<grid, threads, smem, s>>>(a);
  return cudaGetLastError();
}

template <int N, int MODE, int RS>
static cudaError_t launch_col_tma(const OpArgs& a, cudaStream_t s) {
  if (a.col_tile == 1) return launch<col_tma<N, MODE, 1, RS>>(TmaSmem<N, MODE, 1>::bytes, a, ColTile<N, 1>::T, s);
  if (a.col_tile == 2) return launch<col_tma<N, MODE, 2, RS>>(TmaSmem<N, MODE, 2>::bytes, a, ColTile<N, 2>::T, s);
  return launch<col_tma<N, MODE, 0, RS>>(TmaSmem<N, MODE, 0>::bytes, a, ColTile<N, 0>::T, s);
}

// The per-radius column passes also come with the small-radix schedule (ES_OPT_COL_RADIX).
template <int N, int MODE>
static cudaError_t launch_col(const OpArgs& a, cudaStream_t s) {
  if (a.variant == 0) return launch<col_pass<N, MODE>>(ColSmem<N, MODE>::bytes, a, ColCfg<N>::T, s);
  if constexpr (MODE == COL_Z_INV_FILTER || MODE == COL_Y_INV) {
    if (a.col_radix == 1) return launch_col_tma<N, MODE, 1>(a, s);
  }
  return launch_col_tma<N, MODE, 0>(a, s);
}

template <int N, int PRO>
static cudaError_t launch_r2c(const OpArgs& a, cudaStream_t s) {
  if (a.variant == 0) return launch<row_r2c<N, PRO>>(RowSmem<N>::bytes, a, RowCfg<N>::T, s);
  switch (a.row_tile) {
    case 1: return launch<row2_r2c<N, PRO, 1>>(Row2Smem<N, false, 1>::bytes, a, RowTile<N, 1>::T, s);
    case 2: return launch<row2_r2c<N, PRO, 2>>(Row2Smem<N, false, 2>::bytes, a, RowTile<N, 2>::T, s);
    case 3: return launch<row2_r2c<N, PRO, 3>>(Row2Smem<N, false, 3>::bytes, a, RowTile<N, 3>::T, s);
    default: return launch<row2_r2c<N, PRO, 0>>(Row2Smem<N, false, 0>::bytes, a, RowTile<N, 0>::T, s);
  }
}

template <int N, int EPI, int RS>
static cudaError_t launch_c2r_tma(const OpArgs& a, cudaStream_t s) {
  constexpr bool P = EPI == EPI_IONIZE;
  switch (a.row_tile) {
    case 1: return launch<row2_c2r<N, EPI, 1, RS>>(Row2Smem<N, P, 1>::bytes, a, RowTile<N, 1>::T, s);
    case 2: return launch<row2_c2r<N, EPI, 2, RS>>(Row2Smem<N, P, 2>::bytes, a, RowTile<N, 2>::T, s);
    case 3: return launch<row2_c2r<N, EPI, 3, RS>>(Row2Smem<N, P, 3>::bytes, a, RowTile<N, 3>::T, s);
    default: return launch<row2_c2r<N, EPI, 0, RS>>(Row2Smem<N, P, 0>::bytes, a, RowTile<N, 0>::T, s);
  }
}

// The per-radius row pass also comes with the small-radix schedule (ES_OPT_ROW_RADIX).
template <int N, int EPI>
static cudaError_t launch_c2r(const OpArgs& a, cudaStream_t s) {
  if (a.variant == 0) return launch<row_c2r<N, EPI>>(RowSmem<N>::bytes, a, RowCfg<N>::T, s);
  if constexpr (EPI == EPI_IONIZE) {
    if (a.row_radix == 1) return launch_c2r_tma<N, EPI, 1>(a, s);
  }
  return launch_c2r_tma<N, EPI, 0>(a, s);
}

template <int N>
static cudaError_t launch_op(int op, const OpArgs& a, cudaStream_t s) {
  switch (op) {
    case OP_COL_Z_FWD: return launch_col<N, COL_Z_FWD>(a, s);
    case OP_COL_Y_FWD: return launch_col<N, COL_Y_FWD>(a, s);
    case OP_COL_Z_INV_FILTER: return launch_col<N, COL_Z_INV_FILTER>(a, s);
    case OP_COL_Z_INV: return launch_col<N, COL_Z_INV>(a, s);
    case OP_COL_Y_INV: return launch_col<N, COL_Y_INV>(a, s);
    case OP_COL_Z_FWD_PK: return launch_col<N, COL_Z_FWD_PK>(a, s);
    case OP_ROW_R2C_SCALE: return launch_r2c<N, PRO_SCALE>(a, s);
    case OP_ROW_R2C_PK: return launch_r2c<N, PRO_PK>(a, s);
    case OP_ROW_C2R_STORE: return launch_c2r<N, EPI_STORE>(a, s);
    case OP_ROW_C2R_IONIZE: return launch_c2r<N, EPI_IONIZE>(a, s);
    default: return cudaErrorInvalidValue;
  }
}

template <int N, int V>
static void col_geometry(OpGeometry* g) {
  constexpr int TI = ColTile<N, V>::TI;
  g->tcol_ti[V] = TI;
  g->tcol_threads[V] = ColTile<N, V>::T;
  g->tcol_tiles_z[V] = N * ((N / 2) / TI) + N / TI;
  g->tcol_tiles_y[V] = N * ((N / 2) / TI);
  g->tcol_smem[V] = TmaSmem<N, COL_Z_INV_FILTER, V>::bytes;
  g->tcol_smem_pk[V] = TmaSmem<N, COL_Z_FWD_PK, V>::bytes;
}

template <int N, int V>
static void row_geometry(OpGeometry* g) {
  g->trow_tiles[V] = N * N / RowTile<N, V>::RL;
  g->trow_threads[V] = RowTile<N, V>::T;
  g->trow_smem[V] = Row2Smem<N, false, V>::bytes;
  g->trow_smem_prev[V] = Row2Smem<N, true, V>::bytes;
}

template <int N>
static void geometry(OpGeometry* g) {
  constexpr int M = N / 2;
  g->col_tiles_z = N * (M / ColCfg<N>::TI) + N / ColCfg<N>::TI;
  g->col_tiles_y = N * (M / ColCfg<N>::TI);
  g->row_tiles = N * N / RowCfg<N>::RL;
  g->col_threads = ColCfg<N>::T;
  g->row_threads = RowCfg<N>::T;
  g->col_smem = ColSmem<N, COL_Z_INV_FILTER>::bytes;
  g->col_smem_pk = ColSmem<N, COL_Z_FWD_PK>::bytes;
  g->row_smem = RowSmem<N>::bytes;
  col_geometry<N, 0>(g);
  col_geometry<N, 1>(g);
  col_geometry<N, 2>(g);
  row_geometry<N, 0>(g);
  row_geometry<N, 1>(g);
  row_geometry<N, 2>(g);
  row_geometry<N, 3>(g);
}

}  // namespace es

#define ES_CAT2(a, b) a##b
#define ES_CAT(a, b) ES_CAT2(a, b)

extern "C" ES_HIDDEN cudaError_t ES_CAT(es_launch_, ES_N)(int op, const es::OpArgs* a, cudaStream_t s) {
  return es::launch_op<ES_N>(op, *a, s);
}
extern "C" ES_HIDDEN void ES_CAT(es_geometry_, ES_N)(es::OpGeometry* g) { es::geometry<ES_N>(g); }
