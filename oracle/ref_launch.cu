// C launchers for the reference's own excursion-set kernels (Programs/find_bubbles.cu), compiled
// from the reference source after the reference's own %-templating (find_HII_bubbles.py:63-69) --
// TEST INFRASTRUCTURE ONLY: the second oracle of the parity tests.  The product never builds,
// loads or calls this.
//
// REF_SOURCE names the templated copy of find_bubbles.cu (oracle/_ref/...); the build recipe
// (oracle/build_ref.py) passes it with -DREF_SOURCE and puts oracle/ref_shim on the include path.
// Launch shape: the reference's 8x8x8 blocks (INIT_PARAMS.py:49); the grid covers the box (the
// reference launches (DIM/8)^3 blocks whatever HII_DIM is, INIT_PARAMS.py:51-53; the extra threads
// return at the kernels' bounds tests, so the results are the same).
#include <cuda_runtime.h>
#include REF_SOURCE

namespace {
dim3 box_grid(int w) { const int g = (w + 7) / 8; return dim3(g, g, g); }
const dim3 kBlock(8, 8, 8);
int status() { return (int)cudaGetLastError(); }
}  // namespace

extern "C" {

// HII_filter(fourierbox, w, filter_type, R): find_bubbles.cu:12-42, launched as find_HII_bubbles.py:147
int ref_hii_filter(void* box, int w, int filter_type, float R, void* stream) {
  HII_filter<<<box_grid(w), kBlock, 0, (cudaStream_t)stream>>>(static_cast<pycuda::complex<float>*>(box), w,
                                                                filter_type, R);
  return status();
}

// fcoll_kernel(fcollapse, smoothed, w, denom): find_bubbles.cu:43-58, launched as find_HII_bubbles.py:156,169
int ref_fcoll(float* fcoll, float* smoothed, int w, float denom, void* stream) {
  fcoll_kernel<<<box_grid(w), kBlock, 0, (cudaStream_t)stream>>>(fcoll, smoothed, w, denom);
  return status();
}

// update_kernel(ionized, fcollapse, w): find_bubbles.cu:59-71, launched as find_HII_bubbles.py:163
int ref_update(float* ionized, float* fcoll, int w, void* stream) {
  update_kernel<<<box_grid(w), kBlock, 0, (cudaStream_t)stream>>>(ionized, fcoll, w);
  return status();
}

// update_sphere_kernel(ionized, fcollapse, w, R): find_bubbles.cu:73-140, launched as
// find_HII_bubbles.py:165 (R in Mpc)
int ref_update_sphere(float* ionized, float* fcoll, int w, float R, void* stream) {
  update_sphere_kernel<<<box_grid(w), kBlock, 0, (cudaStream_t)stream>>>(ionized, fcoll, w, R);
  return status();
}

// final_kernel(ionized, fcollapse, w, denom): find_bubbles.cu:142-158.  find_HII_bubbles.py:175
// launches it with three arguments; the fourth (denom) is never read by the kernel, so 0 is passed.
int ref_final(float* ionized, float* fcoll, int w, void* stream) {
  final_kernel<<<box_grid(w), kBlock, 0, (cudaStream_t)stream>>>(ionized, fcoll, w, 0.0f);
  return status();
}

}  // extern "C"
