// CUDA emulation header for compiling the reference's device code as host
// C++ (test infrastructure only: it pins the oracle against the reference's
// own kernels, and times that code on the host cores as the CPU baseline).
// "Device" memory is host memory.  Block-level primitives (__syncthreads,
// warp shuffles) are not emulated: the recipe only runs kernels whose result
// is defined without them, and replaces Utility/ParallelScan.h with a
// prefix offset handed out one thread at a time.
//
// Two launch modes:
//  * serial (default): every (block, thread) of the grid in order, one
//    emulated thread at a time; atomics are plain read-modify-writes.  The
//    golden fixtures come from this mode, so allocation and list orders are
//    those of one thread.
//  * SHIM_OMP: an OpenMP parallel loop over the grid's blocks, each block's
//    threads in order on one host thread (block-shared variables are
//    per-host-thread statics); atomics are real atomics.  Results are then
//    as racy as on the GPU (list orders, the bucket lock's skipped
//    allocations), which is the reference's own behaviour; this mode times
//    the reference's code on the host cores.
#ifndef REF_SHIM_CUDA_RUNTIME_H_
#define REF_SHIM_CUDA_RUNTIME_H_

#include <sys/types.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#define __device__
#define __host__
#define __global__
#define __forceinline__ inline
#define __inline__ inline
#ifdef SHIM_OMP
#define __shared__ static thread_local
#else
#define __shared__ static
#endif
#define __constant__
#define __launch_bounds__(...)
#define __align__(n) alignas(n)

using std::ceil;
using std::exp;
using std::fabs;
using std::floor;
using std::fmax;
using std::fmin;
using std::isinf;
using std::isnan;
using std::pow;
using std::sqrt;

// ------------------------------------------------------------ vector types
struct alignas(8) float2 { float x, y; };
struct float3 { float x, y, z; };
struct alignas(16) float4 { float x, y, z, w; };
struct alignas(8) int2 { int x, y; };
struct int3 { int x, y, z; };
struct alignas(16) int4 { int x, y, z, w; };
struct alignas(8) uint2 { unsigned x, y; };
struct uint3 { unsigned x, y, z; };
struct alignas(2) uchar2 { unsigned char x, y; };
struct uchar3 { unsigned char x, y, z; };
struct alignas(4) uchar4 { unsigned char x, y, z, w; };
struct alignas(4) short2 { short x, y; };
struct alignas(16) double2 { double x, y; };
struct alignas(16) double4 { double x, y, z, w; };
struct dim3 {
  unsigned x, y, z;
  dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};

inline float2 make_float2(float x, float y) { return {x, y}; }
inline float3 make_float3(float x, float y, float z) { return {x, y, z}; }
inline float4 make_float4(float x, float y, float z, float w) { return {x, y, z, w}; }
inline int2 make_int2(int x, int y) { return {x, y}; }
inline int3 make_int3(int x, int y, int z) { return {x, y, z}; }
inline int4 make_int4(int x, int y, int z, int w) { return {x, y, z, w}; }
inline uint2 make_uint2(unsigned x, unsigned y) { return {x, y}; }
inline uint3 make_uint3(unsigned x, unsigned y, unsigned z) { return {x, y, z}; }
inline uchar3 make_uchar3(unsigned char x, unsigned char y, unsigned char z) { return {x, y, z}; }
inline uchar4 make_uchar4(unsigned char x, unsigned char y, unsigned char z, unsigned char w) {
  return {x, y, z, w};
}
inline short2 make_short2(short x, short y) { return {x, y}; }
inline double4 make_double4(double x, double y, double z, double w) { return {x, y, z, w}; }

// --------------------------------------------------------- thread indices
extern thread_local uint3 threadIdx;
extern thread_local uint3 blockIdx;
extern thread_local dim3 blockDim;
extern thread_local dim3 gridDim;
static const int warpSize = 32;

inline void __syncthreads() {}
template <class T>
inline T __shfl_down_sync(unsigned, T v, int) { return v; }

// -------------------------------------------------------------- intrinsics
inline float __int_as_float(int i) { float f; memcpy(&f, &i, 4); return f; }
inline int __float_as_int(float f) { int i; memcpy(&i, &f, 4); return i; }
inline int shim_f2i(double v) {  // cvt.rzi semantics: NaN -> 0, saturating
  if (std::isnan(v)) return 0;
  if (v >= 2147483647.0) return 2147483647;
  if (v <= -2147483648.0) return (-2147483647 - 1);
  return (int)v;
}
inline float __saturatef(float v) { return v < 0.f ? 0.f : (v > 1.f ? 1.f : (v == v ? v : 0.f)); }
inline int __float2int_rd(float v) { return shim_f2i(std::floor(v)); }
inline int __float2int_rn(float v) { return shim_f2i(std::nearbyint(v)); }
inline float __powf(float a, float b) { return std::pow(a, b); }
inline int __float2int_ru(float v) { return shim_f2i(std::ceil(v)); }

inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
inline unsigned min(unsigned a, unsigned b) { return a < b ? a : b; }
inline unsigned max(unsigned a, unsigned b) { return a > b ? a : b; }
inline float min(float a, float b) { return std::fmin(a, b); }
inline float max(float a, float b) { return std::fmax(a, b); }
inline double min(double a, double b) { return std::fmin(a, b); }
inline double max(double a, double b) { return std::fmax(a, b); }

#ifdef SHIM_OMP
// real atomics (blocks run concurrently on the host threads)
inline int atomicAdd(int *p, int v) { return __atomic_fetch_add(p, v, __ATOMIC_RELAXED); }
inline unsigned atomicAdd(unsigned *p, unsigned v) { return __atomic_fetch_add(p, v, __ATOMIC_RELAXED); }
inline float atomicAdd(float *p, float v) {
  unsigned *u = (unsigned *)p;
  unsigned o = __atomic_load_n(u, __ATOMIC_RELAXED), n;
  do {
    float f;
    memcpy(&f, &o, 4);
    f += v;
    memcpy(&n, &f, 4);
  } while (!__atomic_compare_exchange_n(u, &o, n, false, __ATOMIC_RELAXED, __ATOMIC_RELAXED));
  float r;
  memcpy(&r, &o, 4);
  return r;
}
inline int atomicSub(int *p, int v) { return __atomic_fetch_sub(p, v, __ATOMIC_RELAXED); }
inline unsigned atomicSub(unsigned *p, unsigned v) { return __atomic_fetch_sub(p, v, __ATOMIC_RELAXED); }
inline int atomicExch(int *p, int v) { return __atomic_exchange_n(p, v, __ATOMIC_ACQ_REL); }
inline unsigned atomicExch(unsigned *p, unsigned v) { return __atomic_exchange_n(p, v, __ATOMIC_ACQ_REL); }
inline int atomicCAS(int *p, int c, int v) {
  __atomic_compare_exchange_n(p, &c, v, false, __ATOMIC_ACQ_REL, __ATOMIC_RELAXED);
  return c;  // the old value on success and failure alike
}
inline int atomicMin(int *p, int v) {
  int o = __atomic_load_n(p, __ATOMIC_RELAXED);
  while (v < o && !__atomic_compare_exchange_n(p, &o, v, false, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
  }
  return o;
}
inline int atomicMax(int *p, int v) {
  int o = __atomic_load_n(p, __ATOMIC_RELAXED);
  while (v > o && !__atomic_compare_exchange_n(p, &o, v, false, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
  }
  return o;
}
#else
// serial atomics (one emulated thread at a time)
inline int atomicAdd(int *p, int v) { int o = *p; *p = o + v; return o; }
inline unsigned atomicAdd(unsigned *p, unsigned v) { unsigned o = *p; *p = o + v; return o; }
inline float atomicAdd(float *p, float v) { float o = *p; *p = o + v; return o; }
inline int atomicSub(int *p, int v) { int o = *p; *p = o - v; return o; }
inline unsigned atomicSub(unsigned *p, unsigned v) { unsigned o = *p; *p = o - v; return o; }
inline int atomicExch(int *p, int v) { int o = *p; *p = v; return o; }
inline unsigned atomicExch(unsigned *p, unsigned v) { unsigned o = *p; *p = v; return o; }
inline int atomicCAS(int *p, int c, int v) { int o = *p; if (o == c) *p = v; return o; }
inline int atomicMin(int *p, int v) { int o = *p; if (v < o) *p = v; return o; }
inline int atomicMax(int *p, int v) { int o = *p; if (v > o) *p = v; return o; }
#endif

// ------------------------------------------------------------ runtime API
typedef int cudaError_t;
enum { cudaSuccess = 0, cudaErrorMemoryAllocation = 2 };
enum cudaMemcpyKind {
  cudaMemcpyHostToHost = 0,
  cudaMemcpyHostToDevice = 1,
  cudaMemcpyDeviceToHost = 2,
  cudaMemcpyDeviceToDevice = 3,
  cudaMemcpyDefault = 4
};
inline const char *cudaGetErrorString(cudaError_t e) { return e ? "shim error" : "no error"; }
inline cudaError_t cudaGetLastError() { return cudaSuccess; }
inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
inline cudaError_t cudaMalloc(void **p, size_t n) {
  *p = std::calloc(1, n ? n : 1);
  return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
template <class T>
inline cudaError_t cudaMalloc(T **p, size_t n) { return cudaMalloc((void **)p, n); }
inline cudaError_t cudaMallocPitch(void **p, size_t *pitch, size_t w, size_t h) {
  *pitch = (w + 255) / 256 * 256;  // pitched rows, as cudaMallocPitch gives
  return cudaMalloc(p, *pitch * h);
}
inline cudaError_t cudaFree(void *p) { std::free(p); return cudaSuccess; }
inline cudaError_t cudaMemcpy(void *d, const void *s, size_t n, cudaMemcpyKind) {
  if (n) memmove(d, s, n);
  return cudaSuccess;
}
inline cudaError_t cudaMemcpy2D(void *d, size_t dp, const void *s, size_t sp, size_t w, size_t h,
                                cudaMemcpyKind) {
  for (size_t r = 0; r < h; ++r) memmove((char *)d + r * dp, (const char *)s + r * sp, w);
  return cudaSuccess;
}
inline cudaError_t cudaMemset(void *d, int v, size_t n) { memset(d, v, n); return cudaSuccess; }
inline cudaError_t cudaMemset2D(void *d, size_t dp, int v, size_t w, size_t h) {
  for (size_t r = 0; r < h; ++r) memset((char *)d + r * dp, v, w);
  return cudaSuccess;
}
inline cudaError_t cudaMemGetInfo(size_t *f, size_t *t) { *f = *t = 0; return cudaSuccess; }

// Launch: every (block, thread) of the grid, blocks in order (serial) or
// spread over the host threads (SHIM_OMP), each block's threads in order.
template <class F>
inline void shim_launch(dim3 grid, dim3 block, F &&f) {
#ifdef SHIM_OMP
  const long long nb = (long long)grid.x * grid.y * grid.z;
#pragma omp parallel for schedule(dynamic, 4)
  for (long long b = 0; b < nb; ++b) {
    gridDim = grid;
    blockDim = block;
    blockIdx = {(unsigned)(b % grid.x), (unsigned)((b / grid.x) % grid.y), (unsigned)(b / ((long long)grid.x * grid.y))};
    for (unsigned tz = 0; tz < block.z; ++tz)
      for (unsigned ty = 0; ty < block.y; ++ty)
        for (unsigned tx = 0; tx < block.x; ++tx) {
          threadIdx = {tx, ty, tz};
          f();
        }
  }
  return;
#endif
  gridDim = grid;
  blockDim = block;
  for (unsigned bz = 0; bz < grid.z; ++bz)
    for (unsigned by = 0; by < grid.y; ++by)
      for (unsigned bx = 0; bx < grid.x; ++bx) {
        blockIdx = {bx, by, bz};
        for (unsigned tz = 0; tz < block.z; ++tz)
          for (unsigned ty = 0; ty < block.y; ++ty)
            for (unsigned tx = 0; tx < block.x; ++tx) {
              threadIdx = {tx, ty, tz};
              f();
            }
      }
}
template <class G, class B, class F>
inline void shim_launch_any(G g, B b, F &&f) {
  shim_launch(dim3(g), dim3(b), f);
}

// Double buffer around the UnifyNeighbor launch: the pass writes each
// voxel's label fields into a copy of the voxel array taken at the launch
// while its neighbour lookups read the array itself, and the copy replaces
// the array after the launch.  Every voxel then updates from the pass-start
// state, the deterministic form of the in-place GPU pass.
struct ShimUnifyBuffer {
  std::vector<unsigned char> copy;
  void *src = nullptr;
};
inline ShimUnifyBuffer &shim_unify_buffer() {
  static ShimUnifyBuffer b;
  return b;
}
inline void shim_unify_begin(void *voxels, size_t bytes) {
  ShimUnifyBuffer &b = shim_unify_buffer();
  b.src = voxels;
  b.copy.assign((const unsigned char *)voxels, (const unsigned char *)voxels + bytes);
}
inline void shim_unify_end() {
  ShimUnifyBuffer &b = shim_unify_buffer();
  memcpy(b.src, b.copy.data(), b.copy.size());
}
#define shim_unify_dst ((void *)shim_unify_buffer().copy.data())

#endif
