// Internal interface between the host engine (es_engine.cu) and the per-size kernel objects.
#pragma once
#include <cuda_runtime.h>

namespace es {

struct OpArgs;

enum Op {
  OP_COL_Z_FWD = 0,
  OP_COL_Y_FWD = 1,
  OP_COL_Z_INV_FILTER = 2,
  OP_COL_Y_INV = 3,
  OP_COL_Z_FWD_PK = 4,
  OP_ROW_R2C_SCALE = 5,
  OP_ROW_R2C_PK = 6,
  OP_ROW_C2R_STORE = 7,
  OP_ROW_C2R_IONIZE = 8,
  OP_COL_Z_INV = 9,
};

constexpr int kColTileVariants = 3;
constexpr int kRowTileVariants = 4;

struct OpGeometry {
  int col_tiles_z, col_tiles_y, row_tiles;
  int col_threads, row_threads;
  int col_smem, col_smem_pk, row_smem;
  // TMA column passes, per tile variant (ES_OPT_COL_TILE)
  int tcol_ti[kColTileVariants], tcol_threads[kColTileVariants], tcol_tiles_z[kColTileVariants];
  int tcol_tiles_y[kColTileVariants], tcol_smem[kColTileVariants], tcol_smem_pk[kColTileVariants];
  // TMA row passes, per tile variant (ES_OPT_ROW_TILE)
  int trow_tiles[kRowTileVariants], trow_threads[kRowTileVariants], trow_smem[kRowTileVariants];
  int trow_smem_prev[kRowTileVariants];
};

}  // namespace es

#define ES_FOR_EACH_SIZE(X) X(16) X(32) X(48) X(64) X(96) X(128) X(160) X(256) X(512) X(1024)

#define ES_HIDDEN __attribute__((visibility("hidden")))
#define ES_DECLARE_SIZE(N)                                                                      \
  extern "C" ES_HIDDEN cudaError_t es_launch_##N(int op, const es::OpArgs* a, cudaStream_t s);   \
  extern "C" ES_HIDDEN void es_geometry_##N(es::OpGeometry* g);
ES_FOR_EACH_SIZE(ES_DECLARE_SIZE)
