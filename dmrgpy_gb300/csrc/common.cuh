// Shared definitions for the GB300 DMRG/TDVP sweep library.
#pragma once

#include <cuda_runtime.h>
#include <cuComplex.h>
#include <atomic>
#include <cstdint>
#include <cstddef>

#include "../../include/dmrg_gb300.h"

namespace dmrg {

// ---------------------------------------------------------------- scalars
// Two element types: real double and interleaved complex double (the
// layout of numpy complex128 / torch.complex128).
typedef cuDoubleComplex cplx;

template <typename T> struct Sc;

template <> struct Sc<double> {
  static __host__ __device__ __forceinline__ double zero() { return 0.0; }
  static __host__ __device__ __forceinline__ double one() { return 1.0; }
  static __host__ __device__ __forceinline__ double make(double re, double) { return re; }
  static __host__ __device__ __forceinline__ double conj(double a) { return a; }
  static __host__ __device__ __forceinline__ double re(double a) { return a; }
  static __host__ __device__ __forceinline__ double im(double) { return 0.0; }
  static __host__ __device__ __forceinline__ double abs2(double a) { return a * a; }
  static __host__ __device__ __forceinline__ double mul(double a, double b) { return a * b; }
  static __host__ __device__ __forceinline__ double add(double a, double b) { return a + b; }
  static __host__ __device__ __forceinline__ double sub(double a, double b) { return a - b; }
  static __host__ __device__ __forceinline__ double fma(double a, double b, double c) { return ::fma(a, b, c); }
  static __host__ __device__ __forceinline__ double scale(double a, double s) { return a * s; }
};

template <> struct Sc<cplx> {
  static __host__ __device__ __forceinline__ cplx zero() { return make_cuDoubleComplex(0.0, 0.0); }
  static __host__ __device__ __forceinline__ cplx one() { return make_cuDoubleComplex(1.0, 0.0); }
  static __host__ __device__ __forceinline__ cplx make(double re, double im) { return make_cuDoubleComplex(re, im); }
  static __host__ __device__ __forceinline__ cplx conj(cplx a) { return make_cuDoubleComplex(a.x, -a.y); }
  static __host__ __device__ __forceinline__ double re(cplx a) { return a.x; }
  static __host__ __device__ __forceinline__ double im(cplx a) { return a.y; }
  static __host__ __device__ __forceinline__ double abs2(cplx a) { return a.x * a.x + a.y * a.y; }
  static __host__ __device__ __forceinline__ cplx mul(cplx a, cplx b) {
    return make_cuDoubleComplex(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
  }
  static __host__ __device__ __forceinline__ cplx add(cplx a, cplx b) { return make_cuDoubleComplex(a.x + b.x, a.y + b.y); }
  static __host__ __device__ __forceinline__ cplx sub(cplx a, cplx b) { return make_cuDoubleComplex(a.x - b.x, a.y - b.y); }
  // c + a*b
  static __host__ __device__ __forceinline__ cplx fma(cplx a, cplx b, cplx c) {
    return make_cuDoubleComplex(::fma(a.x, b.x, ::fma(-a.y, b.y, c.x)), ::fma(a.x, b.y, ::fma(a.y, b.x, c.y)));
  }
  static __host__ __device__ __forceinline__ cplx scale(cplx a, double s) { return make_cuDoubleComplex(a.x * s, a.y * s); }
};

template <typename T> __device__ __forceinline__ T cond_conj(T a, bool c) { return c ? Sc<T>::conj(a) : a; }

// ---------------------------------------------------------------- reductions
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---------------------------------------------------------------- launch checks
// Every kernel launch of the library is followed by this check, which also
// counts the launch (dmrg_kernel_launches()).
void count_launch();
void count_launches(unsigned long long n);    // kernels of a replayed graph
void uncount_launches(unsigned long long n);  // launches made during a graph capture
#define DMRG_CHECK_LAUNCH()                                      \
  do {                                                           \
    cudaError_t _e = cudaGetLastError();                         \
    if (_e != cudaSuccess) return DMRG_ERR_CUDA;                 \
    ::dmrg::count_launch();                                      \
  } while (0)

#define DMRG_CUDA_TRY(x)                                         \
  do {                                                           \
    cudaError_t _e = (x);                                        \
    if (_e != cudaSuccess) return DMRG_ERR_CUDA;                 \
  } while (0)

#define DMRG_TRY(x)                                              \
  do {                                                           \
    int _s = (x);                                                \
    if (_s != DMRG_OK) return _s;                                \
  } while (0)

// Raises a kernel's dynamic shared-memory limit once per device: the
// attribute belongs to the device, and a process may drive several.  `done`
// (one per kernel and size) records the devices already set.
inline int smem_attr_once(const void* fn, int bytes, std::atomic<unsigned long long>& done) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return DMRG_ERR_CUDA;
  const unsigned long long bit = 1ull << (dev & 63);
  if (done.load(std::memory_order_acquire) & bit) return DMRG_OK;
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess) return DMRG_ERR_CUDA;
  done.fetch_or(bit, std::memory_order_release);
  return DMRG_OK;
}

inline size_t align_up(size_t x, size_t a = 256) { return (x + a - 1) / a * a; }

// Bump allocator over a caller-provided workspace.
struct Arena {
  char* base;
  size_t size;
  size_t used;
  Arena(void* b, size_t s) : base(static_cast<char*>(b)), size(s), used(0) {}
  template <typename T> T* take(size_t count) {
    size_t bytes = align_up(count * sizeof(T));
    if (base == nullptr) {  // sizing pass
      used += bytes;
      return nullptr;
    }
    if (used + bytes > size) return nullptr;
    T* p = reinterpret_cast<T*>(base + used);
    used += bytes;
    return p;
  }
  bool sizing() const { return base == nullptr; }
};

// ---------------------------------------------------------------- strided contraction
// C[b] = alpha * opA(A[b]) * opB(B[b]) + beta * C[b], where every logical
// dimension (batch, M, N, K) is a pair of sub-indices (outer, inner) with
// independent element strides in each operand.  This covers every
// transpose/permutation the FP64 sweep needs without copies.
struct Ax2 {
  int n1, n2;          // extents (outer, inner); logical size n1*n2
};
struct St2 {
  long long s1, s2;    // element strides (outer, inner)
};
struct TGemm {
  Ax2 B, M, N, K;
  St2 a_b, a_m, a_k;
  St2 b_b, b_k, b_n;
  St2 c_b, c_m, c_n;
  int conjA, conjB;
};

inline Ax2 ax(int n1, int n2 = 1) { Ax2 a; a.n1 = n1; a.n2 = n2; return a; }
inline St2 st(long long s1, long long s2 = 0) { St2 s; s.s1 = s1; s.s2 = s2; return s; }

template <typename T>
int tgemm(const TGemm& g, T alpha, const T* A, const T* B, T beta, T* C, cudaStream_t stream);
// Many strided contractions of different shapes in one launch.  desc_host
// (pageable, tgemm_grouped_desc_bytes(nprob)) stages the problem table that
// is copied to desc_dev (device, same size) on the stream.
// G (k x k) = X^T X for X (m x k, row stride ld), FP64: only the upper
// triangle of output tiles is computed, each off-diagonal tile written twice.
int tgemm_gram(const double* X, long long ld, int m, int k, double* G, cudaStream_t stream);
size_t tgemm_grouped_desc_bytes(int nprob);
// the same split in two: the problem table built on the host (desc_host),
// then -- after the caller has copied it to device memory -- the launch
int tgemm_grouped_build(int nprob, const TGemm* g, const void* const* A, const void* const* B, void* const* C,
                        void* desc_host, int* nout, long long* tiles_out);
template <typename T>
int tgemm_grouped_launch(const void* desc_dev, int n, long long tiles, T alpha, T beta, cudaStream_t stream);
template <typename T>
int tgemm_grouped(int nprob, const TGemm* g, const void* const* A, const void* const* B, void* const* C, T alpha,
                  T beta, void* desc_dev, void* desc_host, cudaStream_t stream);

// ---------------------------------------------------------------- vector ops (device scalars)
template <typename T> int vdot(const T* x, const T* y, long long n, T* out, double* scratch, cudaStream_t s);
template <typename T> int vnorm(const T* x, long long n, double* out, double* scratch, cudaStream_t s);
template <typename T> int vscale_dev_inv(T* y, const T* x, const double* denom, long long n, cudaStream_t s);
template <typename T> int vscale(T* x, T a, long long n, cudaStream_t s);
// CTAs per vector of the block dot products h = Q^H w (two per SM); the
// caller's partial scratch holds 2 * MULTIDOT_MAX_GRID doubles per vector
constexpr int MULTIDOT_MAX_GRID = 2 * 152;
template <typename T> int vcopy(T* y, const T* x, long long n, cudaStream_t s);
template <typename T> int vfill_random(T* x, long long n, unsigned long long seed, cudaStream_t s);
// w = w - Q h (or w = Q h when overwrite); Q column-major n x k, leading dim ldq
template <typename T> int gemv_sub(const T* Q, long long ldq, int k, const T* h, T* w, long long n, int overwrite, cudaStream_t s);
int nan_check(const void* x, long long n_doubles, int* flag, cudaStream_t s);

// FP64 value of an FP32 one from its bit pattern (exact; zero, subnormal,
// inf and nan take the conversion), keeping the FP64 pipe free in the
// epilogues that widen FP32 accumulators
__device__ __forceinline__ double widen(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t ef = (u >> 23) & 0xffu;
  if (ef == 0u || ef == 0xffu) return static_cast<double>(f);
  return __hiloint2double(static_cast<int>((u & 0x80000000u) | ((ef + 896u) << 20) | ((u & 0x7fffffu) >> 3)),
                          static_cast<int>(u << 29));
}

// FP32 value of an FP64 one (round half away from zero at 24 bits) from its
// bit pattern; values outside the FP32 normal range take the conversion
__device__ __forceinline__ float narrow(double x) {
  const uint32_t xh = static_cast<uint32_t>(__double2hiint(x));
  const uint32_t xl = static_cast<uint32_t>(__double2loint(x));
  const int e = static_cast<int>((xh >> 20) & 0x7ffu);
  if (e < 897 || e > 1150) return static_cast<float>(x);
  const uint32_t frac = ((xh & 0xfffffu) << 3) | (xl >> 29);   // 23 fraction bits
  // a carry out of the fraction moves into the exponent field (to inf past the top)
  return __uint_as_float((xh & 0x80000000u) | ((static_cast<uint32_t>(e - 896) << 23) + frac + ((xl >> 28) & 1u)));
}

}  // namespace dmrg
