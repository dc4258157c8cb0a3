// Compatibility header for compiling the reference's GPU programs (written for sm_35 / sm_61
// and CUDA 10-era thrust) with CUDA 13 for sm_103a.  TEST INFRASTRUCTURE ONLY: passed with
// `nvcc -include` by oracle/Makefile's ref-gpu target; the reference sources themselves are
// not modified.  Nothing in the product includes it.
//   - cudaDeviceProp::clockRate was removed in CUDA 13; the programs only print it.
//   - thrust::unary_function was removed in CCCL 3; the programs derive functors from it.
//   - thrust/remove.h and thrust/unique.h are no longer pulled in by the headers they include.
//   - __shfl_down (no mask) was removed; every call site in the programs runs with all 32
//     lanes of the warp active, so the full mask is the same operation.
#pragma once
#include <cstdint>
#include <cstring>
#include <thrust/functional.h>
#include <thrust/remove.h>
#include <thrust/unique.h>
namespace thrust {
template <class Arg, class Result>
struct unary_function {
  typedef Arg argument_type;
  typedef Result result_type;
};
}  // namespace thrust
#define clockRate multiProcessorCount
#define __shfl_down(v, d) __shfl_down_sync(0xffffffffu, (v), (d))
