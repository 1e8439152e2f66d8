/*
 * Host-only stand-in for the CUDA runtime, used to compile the reference's
 * own sources (src/simFDTD.cu, src/simulation.h, src/gpu.h) with g++ so
 * that they run on the CPU.  TEST INFRASTRUCTURE ONLY (oracle pinning).
 *
 * - __global__ functions become plain functions; blockIdx/threadIdx/
 *   blockDim/gridDim are globals set by the launch emulator.
 * - A launch `k<<<g, b, sh, st>>>(args)` is rewritten by oracle/ref_build.sh
 *   into `REF_LAUNCH(k, g, b, sh, st)(args)`, which runs every block and
 *   every thread in sequence.  None of the reference kernels reads a value
 *   that another thread of the same launch writes (each thread owns the
 *   cells it stores), so sequential emulation equals the parallel launch.
 * - Device memory is host memory; all copies are synchronous memcpy.
 */
#ifndef REF_SHIM_CUDA_RUNTIME_H
#define REF_SHIM_CUDA_RUNTIME_H

#include <algorithm>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline

struct uint3 {
  unsigned int x, y, z;
};
struct dim3 {
  unsigned int x, y, z;
  dim3(unsigned long long a = 1, unsigned long long b = 1,
       unsigned long long c = 1)
      : x((unsigned int)a), y((unsigned int)b), z((unsigned int)c) {}
};

inline uint3 threadIdx, blockIdx;
inline dim3 blockDim, gridDim;

typedef int cudaError_t;
typedef struct ref_stream *cudaStream_t;
enum { cudaSuccess = 0 };
enum cudaMemcpyKind {
  cudaMemcpyHostToHost = 0,
  cudaMemcpyHostToDevice = 1,
  cudaMemcpyDeviceToHost = 2,
  cudaMemcpyDeviceToDevice = 3,
  cudaMemcpyDefault = 4
};

template <class T> inline cudaError_t cudaMalloc(T **p, size_t n) {
  *p = (T *)std::calloc(n ? n : 1, 1);
  return 0;
}
template <class T> inline cudaError_t cudaMallocHost(T **p, size_t n) {
  *p = (T *)std::calloc(n ? n : 1, 1);
  return 0;
}
inline cudaError_t cudaFree(void *p) {
  std::free(p);
  return 0;
}
inline cudaError_t cudaFreeHost(void *p) {
  std::free(p);
  return 0;
}
inline cudaError_t cudaMemcpyAsync(void *d, const void *s, size_t n,
                                   cudaMemcpyKind, cudaStream_t = nullptr) {
  std::memmove(d, s, n);
  return 0;
}
inline cudaError_t cudaMemsetAsync(void *d, int v, size_t n,
                                   cudaStream_t = nullptr) {
  std::memset(d, v, n);
  return 0;
}
inline cudaError_t cudaStreamCreate(cudaStream_t *s) {
  *s = nullptr;
  return 0;
}
inline cudaError_t cudaStreamDestroy(cudaStream_t) { return 0; }
inline cudaError_t cudaStreamSynchronize(cudaStream_t) { return 0; }

using std::max;
using std::min;

template <class F> struct ref_launcher {
  F f;
  dim3 g, b;
  template <class... A> void operator()(A &&...args) {
    gridDim = g;
    blockDim = b;
    for (unsigned bz = 0; bz < g.z; ++bz)
      for (unsigned by = 0; by < g.y; ++by)
        for (unsigned bx = 0; bx < g.x; ++bx) {
          blockIdx = uint3{bx, by, bz};
          for (unsigned tz = 0; tz < b.z; ++tz)
            for (unsigned ty = 0; ty < b.y; ++ty)
              for (unsigned tx = 0; tx < b.x; ++tx) {
                threadIdx = uint3{tx, ty, tz};
                f(args...);
              }
        }
  }
};

template <class F>
inline ref_launcher<F> ref_make_launcher(F f, dim3 g, dim3 b, size_t = 0,
                                         cudaStream_t = nullptr) {
  return ref_launcher<F>{f, g, b};
}

#define REF_LAUNCH(K, ...) \
  ref_make_launcher([](auto &&...a) { K(a...); }, __VA_ARGS__)

#endif
