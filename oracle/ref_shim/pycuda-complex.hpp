// Stand-in for PyCUDA's <pycuda-complex.hpp> so the reference's Programs/find_bubbles.cu compiles
// with nvcc 13 as it is -- TEST INFRASTRUCTURE ONLY (the second oracle; nothing in the product
// includes this).
//
// * pycuda::complex<float> is a float pair with complex arithmetic; cuda::std::complex<float>
//   has the same layout (re, im) and operators, which is all HII_filter uses (find_bubbles.cu:12-42:
//   `*=` by a real scalar and assignment of 0).
// * Line 9 of find_bubbles.cu declares a legacy texture reference (`texture<float,3> img;`) that
//   no kernel reads; CUDA 12 removed texture references, so an empty class template of that name
//   lets the declaration stand as an unused host object.
#pragma once
#include <cuda/std/complex>

namespace pycuda {
template <class T>
using complex = cuda::std::complex<T>;
}

template <class T, int Dim>
struct texture {};
