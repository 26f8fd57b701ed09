// FP64 vector kernels of the Krylov loops: dot products and norms with a
// deterministic single-launch two-level reduction (warp shuffles, then the
// last CTA folds the per-CTA partials in a fixed order), fused axpy /
// scaling with scalars that stay in device memory, and the block
// reorthogonalisation h = Q^H w, w -= Q h.  All HBM-bound; grids are sized in
// multiples of the 152 SMs.
#include "common.cuh"

namespace dmrg {

namespace {

constexpr int RT = 256;          // threads per reduction CTA
constexpr int RB = 2 * 152;      // reduction CTAs (two per SM)

template <typename T>
__device__ __forceinline__ void acc_dot(const T& a, const T& b, double& re, double& im);
template <>
__device__ __forceinline__ void acc_dot<double>(const double& a, const double& b, double& re, double& im) {
  re = ::fma(a, b, re);
}
template <>
__device__ __forceinline__ void acc_dot<cplx>(const cplx& a, const cplx& b, double& re, double& im) {
  // conj(a) * b
  re = ::fma(a.x, b.x, ::fma(a.y, b.y, re));
  im = ::fma(a.x, b.y, ::fma(-a.y, b.x, im));
}

__device__ __forceinline__ void block_sum2(double& re, double& im, double* sh) {
  re = warp_sum(re);
  im = warp_sum(im);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) { sh[2 * wid] = re; sh[2 * wid + 1] = im; }
  __syncthreads();
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    re = lane < nw ? sh[2 * lane] : 0.0;
    im = lane < nw ? sh[2 * lane + 1] : 0.0;
    re = warp_sum(re);
    im = warp_sum(im);
  }
  __syncthreads();
}

// MODE 0: out = sum conj(x) y ; MODE 1: out = sqrt(sum |x|^2)
template <typename T, int MODE>
__global__ void __launch_bounds__(RT) reduce_kernel(const T* __restrict__ x, const T* __restrict__ y, long long n,
                                                    double* __restrict__ partials, unsigned* __restrict__ counter,
                                                    double* __restrict__ out) {
  __shared__ double sh[64];
  __shared__ bool last;
  double re = 0.0, im = 0.0;
  const long long stride = (long long)gridDim.x * blockDim.x;
#pragma unroll 4
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    if (MODE == 0) acc_dot<T>(x[i], y[i], re, im);
    else acc_dot<T>(x[i], x[i], re, im);
  }
  block_sum2(re, im, sh);
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = re;
    partials[2 * blockIdx.x + 1] = im;
    __threadfence();
    unsigned prev = atomicAdd(counter, 1u);
    last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  re = 0.0;
  im = 0.0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
    re += ((volatile double*)partials)[2 * b];
    im += ((volatile double*)partials)[2 * b + 1];
  }
  block_sum2(re, im, sh);
  if (threadIdx.x == 0) {
    if (MODE == 0) { out[0] = re; out[1] = im; }
    else { out[0] = sqrt(re); out[1] = 0.0; }
    *counter = 0u;  // leave the counter ready for the next reduction
  }
}

inline int grid_for(long long n) {
  long long g = (n + RT - 1) / RT;
  if (g > RB) g = RB;
  if (g < 1) g = 1;
  return (int)g;
}

// y -= a1*x1 + a2*x2 with a1, a2 device doubles (NULL => skip that term)
template <typename T>
__global__ void axpy2_kernel(T* __restrict__ y, const T* __restrict__ x1, const double* __restrict__ a1,
                             const T* __restrict__ x2, const double* __restrict__ a2, long long n) {
  const double c1 = a1 ? *a1 : 0.0;
  const double c2 = (a2 && x2) ? *a2 : 0.0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    T v = y[i];
    if (a1) v = Sc<T>::sub(v, Sc<T>::scale(x1[i], c1));
    if (a2 && x2) v = Sc<T>::sub(v, Sc<T>::scale(x2[i], c2));
    y[i] = v;
  }
}

template <typename T>
__global__ void scale_inv_kernel(T* __restrict__ y, const T* __restrict__ x, const double* __restrict__ den, long long n) {
  const double s = 1.0 / *den;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) y[i] = Sc<T>::scale(x[i], s);
}

template <typename T>
__global__ void scale_kernel(T* __restrict__ x, T a, long long n) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) x[i] = Sc<T>::mul(a, x[i]);
}

template <typename T>
__global__ void copy_kernel(T* __restrict__ y, const T* __restrict__ x, long long n) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) y[i] = x[i];
}

__device__ __forceinline__ double hash_normal(unsigned long long seed, long long i) {
  // splitmix64 pair -> Box-Muller
  auto mix = [](unsigned long long z) {
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
  };
  unsigned long long a = mix(seed ^ (2ull * (unsigned long long)i));
  unsigned long long b = mix(seed ^ (2ull * (unsigned long long)i + 1ull));
  double u1 = ((a >> 11) + 1.0) * (1.0 / 9007199254740993.0);
  double u2 = (b >> 11) * (1.0 / 9007199254740992.0);
  return sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
}

template <typename T>
__global__ void random_kernel(T* __restrict__ x, long long n, unsigned long long seed) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    x[i] = Sc<T>::make(hash_normal(seed, i), 0.0);
}

// partial[j * G + g] = sum over the g-th slice of conj(q_j) w
template <typename T>
__global__ void __launch_bounds__(RT) multidot_partial(const T* __restrict__ Q, long long ldq, const T* __restrict__ w,
                                                       long long n, double* __restrict__ partial) {
  __shared__ double sh[64];
  const int j = blockIdx.y;
  const T* q = Q + (long long)j * ldq;
  double re = 0.0, im = 0.0;
  const long long stride = (long long)gridDim.x * blockDim.x;
#pragma unroll 4
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) acc_dot<T>(q[i], w[i], re, im);
  block_sum2(re, im, sh);
  if (threadIdx.x == 0) {
    partial[2 * ((long long)j * gridDim.x + blockIdx.x)] = re;
    partial[2 * ((long long)j * gridDim.x + blockIdx.x) + 1] = im;
  }
}

template <typename T>
__global__ void multidot_final(const double* __restrict__ partial, int G, T* __restrict__ h) {
  __shared__ double sh[64];
  const int j = blockIdx.x;
  double re = 0.0, im = 0.0;
  for (int g = threadIdx.x; g < G; g += blockDim.x) {
    re += partial[2 * ((long long)j * G + g)];
    im += partial[2 * ((long long)j * G + g) + 1];
  }
  block_sum2(re, im, sh);
  if (threadIdx.x == 0) h[j] = Sc<T>::make(re, im);
}

// w = (overwrite ? 0 : w) - sign * Q h   (sign = +1 subtract, overwrite => w = Q h)
template <typename T>
__global__ void gemv_kernel(const T* __restrict__ Q, long long ldq, int k, const T* __restrict__ h, T* __restrict__ w,
                            long long n, int overwrite) {
  extern __shared__ unsigned char smem_raw[];
  T* hs = reinterpret_cast<T*>(smem_raw);
  for (int j = threadIdx.x; j < k; j += blockDim.x) hs[j] = h[j];
  __syncthreads();
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    T acc = Sc<T>::zero();
    for (int j = 0; j < k; ++j) acc = Sc<T>::fma(Q[i + (long long)j * ldq], hs[j], acc);
    w[i] = overwrite ? acc : Sc<T>::sub(w[i], acc);
  }
}

__global__ void nan_kernel(const double* __restrict__ x, long long n, int* __restrict__ flag) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  int bad = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    if (!isfinite(x[i])) bad = 1;
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flag, 1);
}

inline int egrid(long long n) {
  long long g = (n + 255) / 256;
  long long cap = 152 * 8;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

}  // namespace

// scratch layout for the reductions: [0]: counter (as unsigned), [8..]: partials
template <typename T>
int vdot(const T* x, const T* y, long long n, T* out, double* scratch, cudaStream_t s) {
  int g = grid_for(n);
  reduce_kernel<T, 0><<<g, RT, 0, s>>>(x, y, n, scratch + 8, reinterpret_cast<unsigned*>(scratch),
                                       reinterpret_cast<double*>(out));
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

template <typename T>
int vnorm(const T* x, long long n, double* out, double* scratch, cudaStream_t s) {
  int g = grid_for(n);
  reduce_kernel<T, 1><<<g, RT, 0, s>>>(x, x, n, scratch + 8, reinterpret_cast<unsigned*>(scratch), out);
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

template <typename T>
int vaxpy2(T* y, const T* x1, const double* a1, const T* x2, const double* a2, long long n, cudaStream_t s) {
  axpy2_kernel<T><<<egrid(n), 256, 0, s>>>(y, x1, a1, x2, a2, n);
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

template <typename T>
int vscale_dev_inv(T* y, const T* x, const double* den, long long n, cudaStream_t s) {
  scale_inv_kernel<T><<<egrid(n), 256, 0, s>>>(y, x, den, n);
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

template <typename T>
int vscale(T* x, T a, long long n, cudaStream_t s) {
  scale_kernel<T><<<egrid(n), 256, 0, s>>>(x, a, n);
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

template <typename T>
int vcopy(T* y, const T* x, long long n, cudaStream_t s) {
  copy_kernel<T><<<egrid(n), 256, 0, s>>>(y, x, n);
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

template <typename T>
int vfill_random(T* x, long long n, unsigned long long seed, cudaStream_t s) {
  random_kernel<T><<<egrid(n), 256, 0, s>>>(x, n, seed);
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

// partial scratch needs 2*k*G doubles with G = min(grid_for(n), MULTIDOT_MAX_GRID)
template <typename T>
int multidot_ws(const T* Q, long long ldq, int k, const T* w, long long n, T* h, double* partial, cudaStream_t s) {
  if (k <= 0) return DMRG_OK;
  int g = grid_for(n);
  if (g > MULTIDOT_MAX_GRID) g = MULTIDOT_MAX_GRID;
  dim3 grid(g, k);
  multidot_partial<T><<<grid, RT, 0, s>>>(Q, ldq, w, n, partial);
  DMRG_CHECK_LAUNCH();
  multidot_final<T><<<k, 64, 0, s>>>(partial, g, h);
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

template <typename T>
int gemv_sub(const T* Q, long long ldq, int k, const T* h, T* w, long long n, int overwrite, cudaStream_t s) {
  if (k <= 0 && !overwrite) return DMRG_OK;
  size_t sm = sizeof(T) * (size_t)(k > 0 ? k : 1);
  gemv_kernel<T><<<egrid(n), 256, sm, s>>>(Q, ldq, k, h, w, n, overwrite);
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

int nan_check(const void* x, long long n_doubles, int* flag, cudaStream_t s) {
  nan_kernel<<<egrid(n_doubles), 256, 0, s>>>(static_cast<const double*>(x), n_doubles, flag);
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

#define INST(T)                                                                                  \
  template int vdot<T>(const T*, const T*, long long, T*, double*, cudaStream_t);               \
  template int vnorm<T>(const T*, long long, double*, double*, cudaStream_t);                   \
  template int vaxpy2<T>(T*, const T*, const double*, const T*, const double*, long long, cudaStream_t); \
  template int vscale_dev_inv<T>(T*, const T*, const double*, long long, cudaStream_t);         \
  template int vscale<T>(T*, T, long long, cudaStream_t);                                       \
  template int vcopy<T>(T*, const T*, long long, cudaStream_t);                                 \
  template int vfill_random<T>(T*, long long, unsigned long long, cudaStream_t);                \
  template int multidot_ws<T>(const T*, long long, int, const T*, long long, T*, double*, cudaStream_t); \
  template int gemv_sub<T>(const T*, long long, int, const T*, T*, long long, int, cudaStream_t);
INST(double)
INST(cplx)
#undef INST

}  // namespace dmrg
