/* Host shim for compiling the reference's Siddon device functions as plain C++.
 *
 * Test infrastructure only: this header lets g++ compile the functions that precede the first
 * __global__ in srfnef/cc/siddon/siddon.cu.cc and srfnef/cc/siddon_tof/siddon_tof.cu.cc
 * (project_device / backproject_device) on the CPU, so that the CPU restatement in
 * oracle/siddon_oracle.c can be pinned against the reference's own arithmetic.
 *
 * - __device__ / __global__ become nothing;
 * - atomicAdd(p, v) becomes a sequential *p += v, counted in ref_atomic_count so the oracle can
 *   report backprojection pair visits;
 * - floor / sqrt / exp resolve to the <cmath> overloads (float stays float, double stays double),
 *   the same overload set CUDA's device headers expose.
 */
#pragma once
#include <cmath>
#include <cstdint>

#define __device__
#define __global__
#define __host__

using std::exp;
using std::floor;
using std::sqrt;

extern "C" int64_t ref_atomic_count;

static inline float atomicAdd(float *addr, float val) {
    float old = *addr;
    *addr = old + val;
    ++ref_atomic_count;
    return old;
}
