// Generic strided batched contraction C = alpha*opA(A)*opB(B) + beta*C in
// FP64 / complex FP64 on the CUDA cores.  This is the FP64 reference path of
// the sweep: on GB300 the FP64 pipe (about 1 TFLOP/s) is the bound, so the
// kernel only has to keep that pipe fed: 64x64 output tile per 256-thread
// CTA, 4x4 register block per thread, K staged through shared memory in
// slices of 16.  Every logical dimension is an (outer, inner) index pair
// with its own element strides, which expresses all the permuted views the
// H_eff / environment / Gram contractions need without copies.
#include "common.cuh"

namespace dmrg {

namespace {

constexpr int BM = 64;
constexpr int BN = 64;
constexpr int BK = 16;
constexpr int NT = 256;

struct Dev {
  int B2, M, M2, N, N2, K, K2;
  long long ab1, ab2, am1, am2, ak1, ak2;
  long long bb1, bb2, bk1, bk2, bn1, bn2;
  long long cb1, cb2, cm1, cm2, cn1, cn2;
  int conjA, conjB;
  int a_kfast, b_kfast;
};

__device__ __forceinline__ long long off2(int i, int n2, long long s1, long long s2) {
  int q = i / n2;
  int r = i - q * n2;
  return (long long)q * s1 + (long long)r * s2;
}

// one BM x BN output tile (m0, n0) of batch entry bz
// MIRROR: C is square with equal M and N layouts and the product is
// symmetric (C = X^T X); an off-diagonal tile also writes its transpose.
template <typename T, bool MIRROR = false>
__device__ __forceinline__ void tgemm_tile(const Dev& d, T alpha, const T* __restrict__ A, const T* __restrict__ B,
                                           T beta, T* __restrict__ C, int m0, int n0, int bz) {
  __shared__ T As[BK][BM + 1];
  __shared__ T Bs[BK][BN + 1];
  const int tid = threadIdx.x;
  const int tx = tid & 15;
  const int ty = tid >> 4;
  const int bq = bz / d.B2, br = bz - bq * d.B2;
  const T* Ab = A + (long long)bq * d.ab1 + (long long)br * d.ab2;
  const T* Bb = B + (long long)bq * d.bb1 + (long long)br * d.bb2;
  T* Cb = C + (long long)bq * d.cb1 + (long long)br * d.cb2;

  T acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = Sc<T>::zero();

  for (int k0 = 0; k0 < d.K; k0 += BK) {
#pragma unroll
    for (int r = 0; r < (BM * BK) / NT; ++r) {
      int e = tid + r * NT;
      int mm, kk;
      if (d.a_kfast) { kk = e % BK; mm = e / BK; } else { mm = e % BM; kk = e / BM; }
      int gm = m0 + mm, gk = k0 + kk;
      T v = Sc<T>::zero();
      if (gm < d.M && gk < d.K) {
        v = Ab[off2(gm, d.M2, d.am1, d.am2) + off2(gk, d.K2, d.ak1, d.ak2)];
        v = cond_conj(v, d.conjA);
      }
      As[kk][mm] = v;
    }
#pragma unroll
    for (int r = 0; r < (BN * BK) / NT; ++r) {
      int e = tid + r * NT;
      int nn, kk;
      if (d.b_kfast) { kk = e % BK; nn = e / BK; } else { nn = e % BN; kk = e / BN; }
      int gn = n0 + nn, gk = k0 + kk;
      T v = Sc<T>::zero();
      if (gn < d.N && gk < d.K) {
        v = Bb[off2(gk, d.K2, d.bk1, d.bk2) + off2(gn, d.N2, d.bn1, d.bn2)];
        v = cond_conj(v, d.conjB);
      }
      Bs[kk][nn] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      T a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = Sc<T>::fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  const bool use_beta = (Sc<T>::re(beta) != 0.0) || (Sc<T>::im(beta) != 0.0);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    int gm = m0 + ty + 16 * i;
    if (gm >= d.M) continue;
    long long om = off2(gm, d.M2, d.cm1, d.cm2);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int gn = n0 + tx + 16 * j;
      if (gn >= d.N) continue;
      long long o = om + off2(gn, d.N2, d.cn1, d.cn2);
      T v = Sc<T>::mul(alpha, acc[i][j]);
      if (use_beta) v = Sc<T>::fma(beta, Cb[o], v);
      Cb[o] = v;
      if (MIRROR && m0 != n0) Cb[off2(gn, d.M2, d.cm1, d.cm2) + off2(gm, d.N2, d.cn1, d.cn2)] = v;
    }
  }
}

// Symmetric product: only the tiles with tile row <= tile column, numbered
// row by row over the upper triangle of a tiles x tiles grid.
template <typename T>
__global__ void __launch_bounds__(NT) tgemm_sym_kernel(Dev d, T alpha, const T* __restrict__ A,
                                                       const T* __restrict__ B, T* __restrict__ C, int tiles) {
  int rem = blockIdx.x, tm = 0;
  while (tm < tiles && rem >= tiles - tm) {
    rem -= tiles - tm;
    ++tm;
  }
  if (tm >= tiles) return;
  tgemm_tile<T, true>(d, alpha, A, B, Sc<T>::zero(), C, tm * BM, (tm + rem) * BN, 0);
}

template <typename T>
__global__ void __launch_bounds__(NT) tgemm_kernel(Dev d, T alpha, const T* __restrict__ A,
                                                   const T* __restrict__ B, T beta, T* __restrict__ C) {
  tgemm_tile<T>(d, alpha, A, B, beta, C, blockIdx.x * BM, blockIdx.y * BN, blockIdx.z);
}

// Grouped launch: problem p owns the flat tile range [start, start + tiles)
// (tiles = batch * tiles_m * tiles_n); each CTA finds its problem by binary
// search over the starts and runs one tile of it.
struct GProb {
  Dev d;
  const void* A;
  const void* B;
  void* C;
  int tiles_m, tiles_n;
  long long start;
};

template <typename T>
__global__ void __launch_bounds__(NT) tgemm_grouped_kernel(const GProb* __restrict__ probs, int nprob, T alpha,
                                                           T beta) {
  const long long t = blockIdx.x;
  int lo = 0, hi = nprob - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (probs[mid].start <= t) lo = mid; else hi = mid - 1;
  }
  const GProb& g = probs[lo];
  const long long local = t - g.start;
  const long long per_b = (long long)g.tiles_m * g.tiles_n;
  const int bz = (int)(local / per_b);
  const int rem = (int)(local - (long long)bz * per_b);
  const int tm = rem % g.tiles_m, tn = rem / g.tiles_m;
  tgemm_tile<T>(g.d, alpha, static_cast<const T*>(g.A), static_cast<const T*>(g.B), beta, static_cast<T*>(g.C),
                tm * BM, tn * BN, bz);
}

// Dev from a TGemm; returns false when there is nothing to do, *err on bad input
bool make_dev(const TGemm& g, Dev* out, int* err) {
  Dev& d = *out;
  *err = DMRG_OK;
  const long long nb = (long long)g.B.n1 * g.B.n2;
  d.B2 = g.B.n2 > 0 ? g.B.n2 : 1;
  d.M = g.M.n1 * g.M.n2;
  d.M2 = g.M.n2;
  d.N = g.N.n1 * g.N.n2;
  d.N2 = g.N.n2;
  d.K = g.K.n1 * g.K.n2;
  d.K2 = g.K.n2;
  if (d.M <= 0 || d.N <= 0 || nb <= 0) return false;
  if (d.M2 <= 0 || d.N2 <= 0 || d.K2 <= 0 || nb > 65535) {
    *err = DMRG_ERR_ARG;
    return false;
  }
  d.ab1 = g.a_b.s1; d.ab2 = g.a_b.s2; d.am1 = g.a_m.s1; d.am2 = g.a_m.s2; d.ak1 = g.a_k.s1; d.ak2 = g.a_k.s2;
  d.bb1 = g.b_b.s1; d.bb2 = g.b_b.s2; d.bk1 = g.b_k.s1; d.bk2 = g.b_k.s2; d.bn1 = g.b_n.s1; d.bn2 = g.b_n.s2;
  d.cb1 = g.c_b.s1; d.cb2 = g.c_b.s2; d.cm1 = g.c_m.s1; d.cm2 = g.c_m.s2; d.cn1 = g.c_n.s1; d.cn2 = g.c_n.s2;
  d.conjA = g.conjA;
  d.conjB = g.conjB;
  // pick the load mapping whose fast thread index walks unit stride
  const long long ak_in = g.K.n2 == 1 ? g.a_k.s1 : g.a_k.s2;
  const long long am_in = g.M.n2 == 1 ? g.a_m.s1 : g.a_m.s2;
  const long long bk_in = g.K.n2 == 1 ? g.b_k.s1 : g.b_k.s2;
  const long long bn_in = g.N.n2 == 1 ? g.b_n.s1 : g.b_n.s2;
  d.a_kfast = (ak_in == 1 && am_in != 1) ? 1 : 0;
  d.b_kfast = (bk_in == 1 && bn_in != 1) ? 1 : 0;
  return true;
}

}  // namespace

template <typename T>
int tgemm(const TGemm& g, T alpha, const T* A, const T* B, T beta, T* C, cudaStream_t stream) {
  Dev d;
  int err = DMRG_OK;
  if (!make_dev(g, &d, &err)) return err;
  const long long nb = (long long)g.B.n1 * g.B.n2;
  dim3 grid((d.M + BM - 1) / BM, (d.N + BN - 1) / BN, (unsigned)nb);
  if (grid.y > 65535) return DMRG_ERR_ARG;
  tgemm_kernel<T><<<grid, NT, 0, stream>>>(d, alpha, A, B, beta, C);
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

int tgemm_gram(const double* X, long long ld, int m, int k, double* G, cudaStream_t stream) {
  if (m < 1 || k < 1) return DMRG_ERR_ARG;
  TGemm g{};
  g.B = ax(1); g.M = ax(k); g.K = ax(m); g.N = ax(k);
  g.a_m = st(1); g.a_k = st(ld);
  g.b_k = st(ld); g.b_n = st(1);
  g.c_m = st(k); g.c_n = st(1);
  Dev d;
  int err = DMRG_OK;
  if (!make_dev(g, &d, &err)) return err;
  const int tiles = (k + BM - 1) / BM;
  const long long ntri = (long long)tiles * (tiles + 1) / 2;
  if (ntri > 0x7fffffffLL) return DMRG_ERR_ARG;
  tgemm_sym_kernel<double><<<(unsigned)ntri, NT, 0, stream>>>(d, 1.0, X, X, G, tiles);
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

size_t tgemm_grouped_desc_bytes(int nprob) { return align_up(sizeof(GProb) * (size_t)(nprob > 0 ? nprob : 1)); }

int tgemm_grouped_build(int nprob, const TGemm* g, const void* const* A, const void* const* B, void* const* C,
                        void* desc_host, int* nout, long long* tiles_out) {
  GProb* h = static_cast<GProb*>(desc_host);
  int n = 0;
  long long tiles = 0;
  for (int p = 0; p < nprob; ++p) {
    Dev d;
    int err = DMRG_OK;
    if (!make_dev(g[p], &d, &err)) {
      if (err != DMRG_OK) return err;
      continue;
    }
    GProb& q = h[n++];
    q.d = d;
    q.A = A[p];
    q.B = B[p];
    q.C = C[p];
    q.tiles_m = (d.M + BM - 1) / BM;
    q.tiles_n = (d.N + BN - 1) / BN;
    q.start = tiles;
    tiles += (long long)g[p].B.n1 * g[p].B.n2 * q.tiles_m * q.tiles_n;
  }
  if (tiles > 0x7fffffffLL) return DMRG_ERR_ARG;
  *nout = n;
  *tiles_out = tiles;
  return DMRG_OK;
}

template <typename T>
int tgemm_grouped_launch(const void* desc_dev, int n, long long tiles, T alpha, T beta, cudaStream_t stream) {
  if (n == 0 || tiles == 0) return DMRG_OK;
  tgemm_grouped_kernel<T><<<(unsigned)tiles, NT, 0, stream>>>(static_cast<const GProb*>(desc_dev), n, alpha, beta);
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

template <typename T>
int tgemm_grouped(int nprob, const TGemm* g, const void* const* A, const void* const* B, void* const* C, T alpha,
                  T beta, void* desc_dev, void* desc_host, cudaStream_t stream) {
  int n = 0;
  long long tiles = 0;
  DMRG_TRY(tgemm_grouped_build(nprob, g, A, B, C, desc_host, &n, &tiles));
  if (n == 0) return DMRG_OK;
  DMRG_CUDA_TRY(cudaMemcpyAsync(desc_dev, desc_host, sizeof(GProb) * (size_t)n, cudaMemcpyHostToDevice, stream));
  return tgemm_grouped_launch<T>(desc_dev, n, tiles, alpha, beta, stream);
}

template int tgemm<double>(const TGemm&, double, const double*, const double*, double, double*, cudaStream_t);
template int tgemm<cplx>(const TGemm&, cplx, const cplx*, const cplx*, cplx, cplx*, cudaStream_t);
template int tgemm_grouped_launch<double>(const void*, int, long long, double, double, cudaStream_t);
template int tgemm_grouped_launch<cplx>(const void*, int, long long, cplx, cplx, cudaStream_t);
template int tgemm_grouped<double>(int, const TGemm*, const void* const*, const void* const*, void* const*, double,
                                   double, void*, void*, cudaStream_t);
template int tgemm_grouped<cplx>(int, const TGemm*, const void* const*, const void* const*, void* const*, cplx, cplx,
                                 void*, void*, cudaStream_t);

}  // namespace dmrg
