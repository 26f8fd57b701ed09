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

template <typename T>
__global__ void __launch_bounds__(NT) tgemm_kernel(Dev d, T alpha, const T* __restrict__ A,
                                                   const T* __restrict__ B, T beta, T* __restrict__ C) {
  __shared__ T As[BK][BM + 1];
  __shared__ T Bs[BK][BN + 1];
  const int tid = threadIdx.x;
  const int tx = tid & 15;
  const int ty = tid >> 4;
  const int m0 = blockIdx.x * BM;
  const int n0 = blockIdx.y * BN;
  const int bz = blockIdx.z;
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
    }
  }
}

}  // namespace

template <typename T>
int tgemm(const TGemm& g, T alpha, const T* A, const T* B, T beta, T* C, cudaStream_t stream) {
  Dev d;
  const long long nb = (long long)g.B.n1 * g.B.n2;
  d.B2 = g.B.n2 > 0 ? g.B.n2 : 1;
  d.M = g.M.n1 * g.M.n2;
  d.M2 = g.M.n2;
  d.N = g.N.n1 * g.N.n2;
  d.N2 = g.N.n2;
  d.K = g.K.n1 * g.K.n2;
  d.K2 = g.K.n2;
  if (d.M <= 0 || d.N <= 0 || nb <= 0) return DMRG_OK;
  if (d.M2 <= 0 || d.N2 <= 0 || d.K2 <= 0 || nb > 65535) return DMRG_ERR_ARG;
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
  dim3 grid((d.M + BM - 1) / BM, (d.N + BN - 1) / BN, (unsigned)nb);
  if (grid.y > 65535) return DMRG_ERR_ARG;
  tgemm_kernel<T><<<grid, NT, 0, stream>>>(d, alpha, A, B, beta, C);
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

template int tgemm<double>(const TGemm&, double, const double*, const double*, double, double*, cudaStream_t);
template int tgemm<cplx>(const TGemm&, cplx, const cplx*, const cplx*, cplx, cplx*, cudaStream_t);

}  // namespace dmrg
