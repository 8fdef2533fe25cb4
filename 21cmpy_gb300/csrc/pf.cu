// Density evolution that produces the excursion-set input boxes (perturb_field):
//
//  * linear: updated = delta * D(z), one FP32 multiply per voxel (perturb_field.py:39-50);
//  * Zel'dovich: every cell (a0, a1, a2) of the DIM^3 initial-conditions box moves by the
//    displacement of the HII_DIM^3 cell it lies in, (v_a * (D(z) - D(z_init)) / L) per axis, and
//    adds its mass 1 + D(z_init) delta to the HII_DIM^3 cell it lands in; the result is
//    mass / MASS_FACTOR - 1 (perturb_field.cu:90-132, perturb_field.py:76-101).
//
// The reference scatters with float atomicAdd, so its sums depend on the order the atomics land
// in.  Here each cell's mass (the same float32 value the reference adds) is converted to a signed
// 64-bit fixed-point number with 32 fraction bits (round to nearest even) and summed with integer
// atomics: the sum is exact, so the result does not depend on the order and a CPU restatement
// reproduces it bit for bit.  Per-axis positions (a + 0.5) / DIM and the HII_DIM cell of every
// DIM index are computed on the host (in double and in float32 respectively, as the reference's
// device code does) and passed as tables, so the device arithmetic is FP32 only.
//
// The scatter runs a grid-stride loop of warps over bricks of 8 x 4 x 8 cells; cells of a lane's
// run that land in one cell share a 64-bit integer atomic; the accumulator (8 bytes per HII cell)
// stays in L2.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

#include "es_engine.h"

namespace pf {

constexpr float kFix = 4294967296.0f;         // 2^32: fixed-point scale of a cell's mass
constexpr float kInvFix = 2.3283064365386963e-10f;   // 2^-32
constexpr int kWrapLimit = 64;                // box lengths a displacement may span

// HII cell index along one axis for a cell at fractional position p (in box lengths) displaced by
// vel * ds box lengths (perturb_field.cu:111-127; the reference's unbounded wrap loops stop after
// kWrapLimit box lengths here, and non-finite positions land in cell 0)
__device__ __forceinline__ int target(float p, float vel, float ds, float swf, int sw) {
  float f = __fadd_rn(p, __fmul_rn(vel, ds));
  f = __fmul_rn(f, swf);
  if (f >= 0.0f && f < swf) {                 // no wrap: the common case
    const int i = (int)f;
    return i < sw ? i : sw - 1;
  }
  if (!isfinite(f)) return 0;
  for (int it = 0; it < kWrapLimit && f >= swf; ++it) f = __fsub_rn(f, swf);
  for (int it = 0; it < kWrapLimit && f < 0.0f; ++it) f = __fadd_rn(f, swf);
  int i = (int)f;
  if (i >= sw) i -= sw;
  if (i < 0) i += sw;
  return i < 0 ? 0 : (i >= sw ? sw - 1 : i);
}

// Warps walk bricks of 8 x 4 x 8 cells (axes 0, 1, 2): a lane owns a run of 8 cells along axis 0
// at one (a1, a2), and every 8 lanes read 32 contiguous bytes of deltax per cell of the run.  The
// run's cells share a1 and a2, so their axis-1 and axis-2 positions, and while they stay in one
// HII cell also the displacement gathers and the axis-1 / axis-2 targets, are computed once per
// run (the HII cell along axis 0 is the same for the whole warp, so the test does not diverge).
// Consecutive cells of a run that land in the same cell add their fixed-point masses in a register
// first; each group then takes one 64-bit atomic (the accumulator is L2-resident).  The brick
// index advances by the grid's warp count as a mixed-radix (axis 0, 1, 2) counter, so the loop
// needs no integer division.
constexpr int kRun = 8;                         // cells per lane along axis 0
__global__ void __launch_bounds__(256) move_mass_kernel(int dim, int sw, const float* __restrict__ delta,
                                                        const float* __restrict__ vx, const float* __restrict__ vy,
                                                        const float* __restrict__ vz, const float* __restrict__ pos,
                                                        const int* __restrict__ hidx, float g0, float ds,
                                                        unsigned long long* __restrict__ acc) {
  const int nb0 = (dim + kRun - 1) / kRun, nb1 = (dim + 3) / 4, nb2 = (dim + 7) / 8;
  const int warps = (int)(gridDim.x * (blockDim.x / 32));
  const int w2 = warps % nb2, w1 = (warps / nb2) % nb1, w0 = warps / (nb2 * nb1);
  const int id = (int)(blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5));
  int c2 = id % nb2, c1 = (id / nb2) % nb1, c0 = id / (nb2 * nb1);
  const float swf = (float)sw;
  const unsigned usw = (unsigned)sw;
  const int lane = threadIdx.x & 31;
  const int l1 = lane >> 3, l2 = lane & 7;
  while (c0 < nb0) {
    const int a1 = c1 * 4 + l1, a2 = c2 * 8 + l2;
    if (a1 < dim && a2 < dim) {
      const unsigned h1 = (unsigned)__ldg(hidx + a1), h2 = (unsigned)__ldg(hidx + a2);
      const float p1 = __ldg(pos + a1), p2 = __ldg(pos + a2);
      int hprev = -1, t1 = 0, t2 = 0;
      float vxv = 0.0f;
      unsigned run_t = 0xffffffffu;              // the run's cells that land in one cell add up first
      unsigned long long run_q = 0ull;
#pragma unroll
      for (int k = 0; k < kRun; ++k) {
        const int a0 = c0 * kRun + k;
        if (a0 < dim) {
          const int h0 = __ldg(hidx + a0);
          if (h0 != hprev) {
            // HII grids up to 1024^3 index in 32 bits
            const unsigned sc = ((unsigned)h0 * usw + h1) * usw + h2;
            vxv = __ldg(vx + sc);
            t1 = target(p1, __ldg(vy + sc), ds, swf, sw);
            t2 = target(p2, __ldg(vz + sc), ds, swf, sw);
            hprev = h0;
          }
          const int t0 = target(__ldg(pos + a0), vxv, ds, swf, sw);
          const float* row = delta + ((size_t)a0 * dim + a1) * dim;   // 64-bit row base
          const float mass = __fadd_rn(1.0f, __fmul_rn(g0, __ldg(row + a2)));
          const long long q = __float2ll_rn(mass * kFix);   // exact scaling by a power of two, then rounding
          const unsigned t = ((unsigned)t0 * usw + (unsigned)t1) * usw + (unsigned)t2;
          if (t != run_t) {                      // integer sums: the grouping does not change the result
            if (run_t != 0xffffffffu) atomicAdd(acc + run_t, run_q);
            run_t = t;
            run_q = 0ull;
          }
          run_q += (unsigned long long)q;
        }
      }
      if (run_t != 0xffffffffu) atomicAdd(acc + run_t, run_q);
    }
    c2 += w2;
    if (c2 >= nb2) { c2 -= nb2; ++c1; }
    c1 += w1;
    if (c1 >= nb1) { c1 -= nb1; ++c0; }
    c0 += w0;
  }
}

__global__ void finalize_kernel(long n, const unsigned long long* __restrict__ acc, float mass_factor,
                                float* __restrict__ out) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const float mass = __ll2float_rn((long long)acc[i]) * kInvFix;
    out[i] = __fsub_rn(__fdiv_rn(mass, mass_factor), 1.0f);
  }
}

__global__ void scale_kernel(long n, const float* __restrict__ in, float g, float* __restrict__ out) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    out[i] = __fmul_rn(in[i], g);
}

}  // namespace pf

struct pf_plan {
  int dim = 0, hii = 0, device = 0, sms = 0;
  float* pos = nullptr;            // [dim] (a + 0.5) / dim
  int* hidx = nullptr;             // [dim] HII cell of index a
  unsigned long long* acc = nullptr;   // [hii^3] fixed-point masses
};

namespace {
thread_local std::string g_pf_error;
int pffail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_pf_error = buf;
  return code;
}
#define PF_CUDA(x)                                                                        \
  do {                                                                                    \
    cudaError_t e_ = (x);                                                                 \
    if (e_ != cudaSuccess) return pffail(ES_E_CUDA, "%s: %s", #x, cudaGetErrorString(e_)); \
  } while (0)
}  // namespace

extern "C" {

int pf_plan_create(int dim, int hii_dim, float pixel_factor, pf_plan** out) {
  if (!out) return pffail(ES_E_ARG, "pf_plan_create: NULL output");
  *out = nullptr;
  if (dim < 1 || dim > 2048 || hii_dim < 1 || hii_dim > dim || hii_dim > 1024)
    return pffail(ES_E_ARG, "pf_plan_create: need 1 <= HII_DIM (%d) <= min(DIM (%d), 1024), DIM <= 2048", hii_dim,
                  dim);
  if (!(pixel_factor > 0.0f)) return pffail(ES_E_ARG, "pf_plan_create: pixel factor must be positive");
  std::vector<float> pos(dim);
  std::vector<int> hidx(dim);
  for (int a = 0; a < dim; ++a) {
    pos[a] = (float)(((double)a + 0.5) / (double)dim);
    const float h = std::floor((float)a / pixel_factor);
    if (!(h >= 0.0f) || h >= (float)hii_dim)
      return pffail(ES_E_ARG, "pf_plan_create: index %d / pixel factor %g leaves the %d^3 grid", a,
                    (double)pixel_factor, hii_dim);
    hidx[a] = (int)h;
  }
  pf_plan* p = new pf_plan;
  p->dim = dim;
  p->hii = hii_dim;
  cudaGetDevice(&p->device);
  cudaDeviceGetAttribute(&p->sms, cudaDevAttrMultiProcessorCount, p->device);
  const size_t cells = (size_t)hii_dim * hii_dim * hii_dim;
  if (cudaMalloc(&p->pos, dim * sizeof(float)) != cudaSuccess || cudaMalloc(&p->hidx, dim * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&p->acc, cells * sizeof(unsigned long long)) != cudaSuccess) {
    cudaFree(p->pos);
    cudaFree(p->hidx);
    cudaFree(p->acc);
    delete p;
    return pffail(ES_E_NOMEM, "pf_plan_create: device allocation failed");
  }
  if (cudaMemcpy(p->pos, pos.data(), dim * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(p->hidx, hidx.data(), dim * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(p->pos);
    cudaFree(p->hidx);
    cudaFree(p->acc);
    delete p;
    return pffail(ES_E_CUDA, "pf_plan_create: table upload failed");
  }
  *out = p;
  return ES_OK;
}

int pf_plan_destroy(pf_plan* p) {
  if (!p) return ES_OK;
  cudaFree(p->pos);
  cudaFree(p->hidx);
  cudaFree(p->acc);
  delete p;
  return ES_OK;
}

int pf_move_mass(pf_plan* p, const float* delta, const float* vx, const float* vy, const float* vz,
                 float init_growth, float disp_scale, float mass_factor, float* updated, void* stream) {
  if (!p || !delta || !vx || !vy || !vz || !updated) return pffail(ES_E_ARG, "pf_move_mass: NULL argument");
  if (!(mass_factor > 0.0f)) return pffail(ES_E_ARG, "pf_move_mass: mass factor must be positive");
  cudaStream_t s = (cudaStream_t)stream;
  const long cells = (long)p->hii * p->hii * p->hii;
  PF_CUDA(cudaMemsetAsync(p->acc, 0, cells * sizeof(unsigned long long), s));
  const long bricks = (long)((p->dim + pf::kRun - 1) / pf::kRun) * ((p->dim + 3) / 4) * ((p->dim + 7) / 8);
  long blocks = (bricks + 7) / 8;                 // 8 warps per block
  const long cap = (long)p->sms * 8;
  if (blocks > cap) blocks = cap;
  pf::move_mass_kernel<<<(unsigned)blocks, 256, 0, s>>>(p->dim, p->hii, delta, vx, vy, vz, p->pos, p->hidx,
                                                        init_growth, disp_scale, p->acc);
  PF_CUDA(cudaGetLastError());
  long fb = (cells + 255) / 256;
  if (fb > cap) fb = cap;
  pf::finalize_kernel<<<(unsigned)fb, 256, 0, s>>>(cells, p->acc, mass_factor, updated);
  PF_CUDA(cudaGetLastError());
  return ES_OK;
}

int pf_evolve_linear(long long n, const float* delta, float growth, float* out, void* stream) {
  if (n < 0 || (n > 0 && (!delta || !out))) return pffail(ES_E_ARG, "pf_evolve_linear: bad arguments");
  if (n == 0) return ES_OK;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  long blocks = (long)((n + 255) / 256);
  if (blocks > (long)sms * 8) blocks = (long)sms * 8;
  pf::scale_kernel<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>((long)n, delta, growth, out);
  PF_CUDA(cudaGetLastError());
  return ES_OK;
}

int pf_last_error(char* buf, int len) {
  if (!buf || len <= 0) return ES_E_ARG;
  std::snprintf(buf, (size_t)len, "%s", g_pf_error.c_str());
  return ES_OK;
}

}  // extern "C"
