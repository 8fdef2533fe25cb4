// Per-box-size instantiation of the FFT pass kernels.  Compiled once per supported N with
// -DES_N=<N>; each object exports es_launch_<N>(), which es_engine.cu dispatches to.
#include "es_kernels.cuh"
#include "es_ops.h"

#ifndef ES_N
#error "compile with -DES_N=<box size>"
#endif

namespace es {

// One static flag per kernel (the template argument is the kernel itself): opt in to more than
// 48 KB of dynamic shared memory once per kernel and device.
template <auto Kernel>
static cudaError_t launch(int smem, const OpArgs& a, int threads, cudaStream_t s) {
  static unsigned configured = 0u;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned bit = 1u << (dev & 31);
  if (!(configured & bit)) {
    e = cudaFuncSetAttribute(Kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    configured |= bit;
  }
  Kernel<<<a.grid, threads, smem, s>>>(a);
  return cudaGetLastError();
}

template <int N>
static cudaError_t launch_op(int op, const OpArgs& a, cudaStream_t s) {
  switch (op) {
    case OP_COL_Z_FWD:
      return launch<col_pass<N, COL_Z_FWD>>(ColSmem<N, COL_Z_FWD>::bytes, a, ColCfg<N>::T, s);
    case OP_COL_Y_FWD:
      return launch<col_pass<N, COL_Y_FWD>>(ColSmem<N, COL_Y_FWD>::bytes, a, ColCfg<N>::T, s);
    case OP_COL_Z_INV_FILTER:
      return launch<col_pass<N, COL_Z_INV_FILTER>>(ColSmem<N, COL_Z_INV_FILTER>::bytes, a, ColCfg<N>::T, s);
    case OP_COL_Z_INV:
      return launch<col_pass<N, COL_Z_INV>>(ColSmem<N, COL_Z_INV>::bytes, a, ColCfg<N>::T, s);
    case OP_COL_Y_INV:
      return launch<col_pass<N, COL_Y_INV>>(ColSmem<N, COL_Y_INV>::bytes, a, ColCfg<N>::T, s);
    case OP_COL_Z_FWD_PK:
      return launch<col_pass<N, COL_Z_FWD_PK>>(ColSmem<N, COL_Z_FWD_PK>::bytes, a, ColCfg<N>::T, s);
    case OP_ROW_R2C_SCALE:
      return launch<row_r2c<N, PRO_SCALE>>(RowSmem<N>::bytes, a, RowCfg<N>::T, s);
    case OP_ROW_R2C_PK:
      return launch<row_r2c<N, PRO_PK>>(RowSmem<N>::bytes, a, RowCfg<N>::T, s);
    case OP_ROW_C2R_STORE:
      return launch<row_c2r<N, EPI_STORE>>(RowSmem<N>::bytes, a, RowCfg<N>::T, s);
    case OP_ROW_C2R_IONIZE:
      return launch<row_c2r<N, EPI_IONIZE>>(RowSmem<N>::bytes, a, RowCfg<N>::T, s);
    default:
      return cudaErrorInvalidValue;
  }
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
}

}  // namespace es

#define ES_CAT2(a, b) a##b
#define ES_CAT(a, b) ES_CAT2(a, b)

extern "C" ES_HIDDEN cudaError_t ES_CAT(es_launch_, ES_N)(int op, const es::OpArgs* a, cudaStream_t s) {
  return es::launch_op<ES_N>(op, *a, s);
}
extern "C" ES_HIDDEN void ES_CAT(es_geometry_, ES_N)(es::OpGeometry* g) { es::geometry<ES_N>(g); }
