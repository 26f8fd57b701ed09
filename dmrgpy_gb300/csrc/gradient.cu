// Adjoint of the environment chain: the derivative of <psi|H|psi> with
// respect to one MPO tensor,
//
//   G[k][s][s'][m] = sum_{a,a',b,b'} L[a'][k][a] A[a][s][b] conj(A)[a'][s'][b'] R[b'][m][b],
//
// L (chil, wl, chil) = contraction of the sites left of the tensor, R (chir,
// wr, chir) of the sites right of it, A (chil, d, chir) the site tensor and
// W (wl, d, d, wr) with d_in (ket) before d_out (bra), the layouts of the
// environment updates.  Because <psi|H|psi> is linear in every single W_i,
// sum_{k,s,s',m} G W_i = <psi|H|psi> for every site i: the reverse pass of
// the energy with respect to all MPO couplings costs one extra environment
// sweep plus one of these per site.
//
// Steps (FP64 / complex FP64):
//   Y1[(a',k)][(s,b)]     = L[(a',k)][a] A[a][(s,b)]                 (GEMM, chi^3 d w)
//   Y2[a'][b'][(k,s)][m]  = Y1[(a',k,s)][b] R[(b',m)][b]              (GEMM, chi^3 d w^2)
//   G[(k,s)][s'][m]       = sum_{(a',b')} Y2[(a',b')][(k,s,m)] conj(A)[a'][s'][b']
//                           (tall-skinny reduction over chi^2 rows, split into
//                            row chunks, deterministic two-pass sum)
#include "common.cuh"

namespace dmrg {
namespace {

constexpr int kRowsPerBlock = 512;
constexpr int kThreads = 256;

// part[blk][o], o = (p, q) with p = (k,s,m) flattened and q = s'.
template <typename T>
__global__ void __launch_bounds__(kThreads)
grad_partial_kernel(const T* __restrict__ Y2, const T* __restrict__ A, long long rows, int P, int d, long long cr,
                    T* __restrict__ part) {
  const long long r0 = (long long)blockIdx.x * kRowsPerBlock;
  const long long r1 = r0 + kRowsPerBlock < rows ? r0 + kRowsPerBlock : rows;
  const int outs = P * d;
  for (int o = threadIdx.x; o < outs; o += blockDim.x) {
    const int p = o / d, q = o % d;
    T acc = Sc<T>::zero();
    for (long long r = r0; r < r1; ++r) {
      const long long ap = r / cr, bp = r % cr;
      const T a = Sc<T>::conj(A[(ap * d + q) * cr + bp]);
      acc = Sc<T>::fma(Y2[r * P + p], a, acc);
    }
    part[(long long)blockIdx.x * outs + o] = acc;
  }
}

// G[k][s][s'][m] = sum_blk part[blk][((k,s,m), s')]
template <typename T>
__global__ void grad_final_kernel(const T* __restrict__ part, int nblk, int wl, int d, int wr, T* __restrict__ G) {
  const int P = wl * d * wr;
  const int outs = P * d;
  for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < outs; o += gridDim.x * blockDim.x) {
    T acc = Sc<T>::zero();
    for (int b = 0; b < nblk; ++b) acc = Sc<T>::add(acc, part[(long long)b * outs + o]);
    const int p = o / d, q = o % d;
    const int k = p / (d * wr), s = (p / wr) % d, m = p % wr;
    G[(((long long)k * d + s) * d + q) * wr + m] = acc;
  }
}

long long nblocks(long long rows) { return (rows + kRowsPerBlock - 1) / kRowsPerBlock; }

template <typename T>
size_t grad_ws(long long cl, long long d, long long cr, long long wl, long long wr) {
  const size_t y1 = sizeof(T) * (size_t)(cl * wl * d * cr);
  const size_t y2 = sizeof(T) * (size_t)(cl * cr * wl * d * wr);
  const size_t pt = sizeof(T) * (size_t)(nblocks(cl * cr) * wl * d * wr * d);
  return align_up(y1, 1024) + align_up(y2, 1024) + align_up(pt, 1024);
}

template <typename T>
int env_gradient(long long cl, long long d, long long cr, long long wl, long long wr, const T* L, const T* A,
                 const T* R, T* G, void* work, size_t work_bytes, cudaStream_t s) {
  if (grad_ws<T>(cl, d, cr, wl, wr) > work_bytes) return DMRG_ERR_WORKSPACE;
  char* p = static_cast<char*>(work);
  T* Y1 = reinterpret_cast<T*>(p); p += align_up(sizeof(T) * (size_t)(cl * wl * d * cr), 1024);
  T* Y2 = reinterpret_cast<T*>(p); p += align_up(sizeof(T) * (size_t)(cl * cr * wl * d * wr), 1024);
  T* part = reinterpret_cast<T*>(p);
  const T one = Sc<T>::one(), zero = Sc<T>::zero();
  TGemm g{};
  g.B = ax(1); g.M = ax((int)(cl * wl)); g.K = ax((int)cl); g.N = ax((int)(d * cr));
  g.a_m = st(cl); g.a_k = st(1);
  g.b_k = st(d * cr); g.b_n = st(1);
  g.c_m = st(d * cr); g.c_n = st(1);
  DMRG_TRY(tgemm<T>(g, one, L, A, zero, Y1, s));
  // rows (a', (k,s)), columns (b', m), reduction over b
  g = TGemm{};
  g.B = ax(1);
  g.M = ax((int)cl, (int)(wl * d));
  g.K = ax((int)cr);
  g.N = ax((int)cr, (int)wr);
  g.a_m = st(wl * d * cr, cr); g.a_k = st(1);
  g.b_k = st(1); g.b_n = st(wr * cr, cr);
  g.c_m = st(cr * wl * d * wr, wr); g.c_n = st(wl * d * wr, 1);
  DMRG_TRY(tgemm<T>(g, one, Y1, R, zero, Y2, s));
  const long long rows = cl * cr;
  const int P = (int)(wl * d * wr);
  const long long nb = nblocks(rows);
  grad_partial_kernel<T><<<(unsigned)nb, kThreads, 0, s>>>(Y2, A, rows, P, (int)d, cr, part);
  DMRG_CHECK_LAUNCH();
  const int outs = P * (int)d;
  grad_final_kernel<T><<<(outs + 255) / 256, 256, 0, s>>>(part, (int)nb, (int)wl, (int)d, (int)wr, G);
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

// ---- transition (bra != ket) forms, for <chi|H|psi> with two different MPS
// bra B (clb, d, crb), ket A (clk, d, crk); environments (chi_bra, w, chi_ket).

template <typename T>
size_t mixed_grad_ws(long long clb, long long crb, long long clk, long long crk, long long d, long long wl,
                     long long wr) {
  const size_t y1 = sizeof(T) * (size_t)(clb * wl * d * crk);
  const size_t y2 = sizeof(T) * (size_t)(clb * crb * wl * d * wr);
  const size_t pt = sizeof(T) * (size_t)(nblocks(clb * crb) * wl * d * wr * d);
  return align_up(y1, 1024) + align_up(y2, 1024) + align_up(pt, 1024);
}

// G[k][s][s'][m] = sum L[a'][k][a] A[a][s][b] conj(B)[a'][s'][b'] R[b'][m][b]
template <typename T>
int env_gradient_mixed(long long clb, long long crb, long long clk, long long crk, long long d, long long wl,
                       long long wr, const T* L, const T* B, const T* A, const T* R, T* G, void* work,
                       size_t work_bytes, cudaStream_t s) {
  if (mixed_grad_ws<T>(clb, crb, clk, crk, d, wl, wr) > work_bytes) return DMRG_ERR_WORKSPACE;
  char* p = static_cast<char*>(work);
  T* Y1 = reinterpret_cast<T*>(p); p += align_up(sizeof(T) * (size_t)(clb * wl * d * crk), 1024);
  T* Y2 = reinterpret_cast<T*>(p); p += align_up(sizeof(T) * (size_t)(clb * crb * wl * d * wr), 1024);
  T* part = reinterpret_cast<T*>(p);
  const T one = Sc<T>::one(), zero = Sc<T>::zero();
  // Y1[(a',k)][(s,b)] = L[(a',k)][a] A[a][(s,b)]
  TGemm g{};
  g.B = ax(1); g.M = ax((int)(clb * wl)); g.K = ax((int)clk); g.N = ax((int)(d * crk));
  g.a_m = st(clk); g.a_k = st(1);
  g.b_k = st(d * crk); g.b_n = st(1);
  g.c_m = st(d * crk); g.c_n = st(1);
  DMRG_TRY(tgemm<T>(g, one, L, A, zero, Y1, s));
  // Y2[a'][b'][(k,s)][m] = Y1[(a',k,s)][b] R[(b',m)][b]
  g = TGemm{};
  g.B = ax(1);
  g.M = ax((int)clb, (int)(wl * d));
  g.K = ax((int)crk);
  g.N = ax((int)crb, (int)wr);
  g.a_m = st(wl * d * crk, crk); g.a_k = st(1);
  g.b_k = st(1); g.b_n = st(wr * crk, crk);
  g.c_m = st(crb * wl * d * wr, wr); g.c_n = st(wl * d * wr, 1);
  DMRG_TRY(tgemm<T>(g, one, Y1, R, zero, Y2, s));
  const long long rows = clb * crb;
  const int P = (int)(wl * d * wr);
  const long long nb = nblocks(rows);
  grad_partial_kernel<T><<<(unsigned)nb, kThreads, 0, s>>>(Y2, B, rows, P, (int)d, crb, part);
  DMRG_CHECK_LAUNCH();
  const int outs = P * (int)d;
  grad_final_kernel<T><<<(outs + 255) / 256, 256, 0, s>>>(part, (int)nb, (int)wl, (int)d, (int)wr, G);
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

template <typename T>
size_t mixed_env_ws(int side, long long clb, long long crb, long long clk, long long crk, long long d, long long wl,
                    long long wr) {
  if (side == 0) return align_up(sizeof(T) * (size_t)(clb * wl * d * crk + clb * d * wr * crk), 1024);
  return align_up(sizeof(T) * (size_t)(crb * wr * clk * d + crb * wl * d * clk), 1024);
}

// side 0: Lnew (crb, wr, crk) = L (clb, wl, clk) . conj(B) . W . A
// side 1: Rnew (clb, wl, clk) = R (crb, wr, crk) . conj(B) . W . A
template <typename T>
int env_mixed(int side, long long clb, long long crb, long long clk, long long crk, long long d, long long wl,
              long long wr, const T* E, const T* W, const T* B, const T* A, T* Enew, void* work, size_t work_bytes,
              cudaStream_t s) {
  if (mixed_env_ws<T>(side, clb, crb, clk, crk, d, wl, wr) > work_bytes) return DMRG_ERR_WORKSPACE;
  const T one = Sc<T>::one(), zero = Sc<T>::zero();
  T* P1 = static_cast<T*>(work);
  TGemm g{};
  if (side == 0) {
    T* Y2 = P1 + clb * wl * d * crk;
    // Y1[(a',k)][(s,b)] = L[(a',k)][a] A[a][(s,b)]
    g.B = ax(1); g.M = ax((int)(clb * wl)); g.K = ax((int)clk); g.N = ax((int)(d * crk));
    g.a_m = st(clk); g.a_k = st(1);
    g.b_k = st(d * crk); g.b_n = st(1);
    g.c_m = st(d * crk); g.c_n = st(1);
    DMRG_TRY(tgemm<T>(g, one, E, A, zero, P1, s));
    // Y2[a'][(s',m)][b] = W[(k,s)][(s',m)] Y1[a'][(k,s)][b]
    g = TGemm{};
    g.B = ax((int)clb); g.M = ax((int)(d * wr)); g.K = ax((int)(wl * d)); g.N = ax((int)crk);
    g.a_b = st(0); g.a_m = st(1); g.a_k = st(d * wr);
    g.b_b = st(wl * d * crk); g.b_k = st(crk); g.b_n = st(1);
    g.c_b = st(d * wr * crk); g.c_m = st(crk); g.c_n = st(1);
    DMRG_TRY(tgemm<T>(g, one, W, P1, zero, Y2, s));
    // Lnew[b'][(m,b)] = conj(B)[(a',s')][b'] Y2[(a',s')][(m,b)]
    g = TGemm{};
    g.B = ax(1); g.M = ax((int)crb); g.K = ax((int)(clb * d)); g.N = ax((int)(wr * crk));
    g.a_m = st(1); g.a_k = st(crb); g.conjA = 1;
    g.b_k = st(wr * crk); g.b_n = st(1);
    g.c_m = st(wr * crk); g.c_n = st(1);
    DMRG_TRY(tgemm<T>(g, one, B, Y2, zero, Enew, s));
  } else {
    T* Z2 = P1 + crb * wr * clk * d;
    // Z1[(b',m)][(a,s)] = R[(b',m)][b] A[(a,s)][b]
    g.B = ax(1); g.M = ax((int)(crb * wr)); g.K = ax((int)crk); g.N = ax((int)(clk * d));
    g.a_m = st(crk); g.a_k = st(1);
    g.b_k = st(1); g.b_n = st(crk);
    g.c_m = st(clk * d); g.c_n = st(1);
    DMRG_TRY(tgemm<T>(g, one, E, A, zero, P1, s));
    // Z2[b'][(k,s')][a] = W[k][s][s'][m] Z1[b'][m][a][s]   (K = (m, s))
    g = TGemm{};
    g.B = ax((int)crb);
    g.M = ax((int)wl, (int)d);
    g.K = ax((int)wr, (int)d);
    g.N = ax((int)clk);
    g.a_b = st(0); g.a_m = st(d * d * wr, wr); g.a_k = st(1, d * wr);
    g.b_b = st(wr * clk * d); g.b_k = st(clk * d, 1); g.b_n = st(d);
    g.c_b = st(wl * d * clk); g.c_m = st(d * clk, clk); g.c_n = st(1);
    DMRG_TRY(tgemm<T>(g, one, W, P1, zero, Z2, s));
    // Rnew[a'][(k,a)] = conj(B)[a'][(b',s')] Z2[(b',s')][(k,a)]
    g = TGemm{};
    g.B = ax(1);
    g.M = ax((int)clb);
    g.K = ax((int)crb, (int)d);
    g.N = ax((int)wl, (int)clk);
    g.a_m = st(d * crb); g.a_k = st(1, crb); g.conjA = 1;
    g.b_k = st(wl * d * clk, clk); g.b_n = st(d * clk, 1);
    g.c_m = st(wl * clk); g.c_n = st(clk, 1);
    DMRG_TRY(tgemm<T>(g, one, B, Z2, zero, Enew, s));
  }
  return DMRG_OK;
}

bool mixed_dims_ok(int clb, int crb, int clk, int crk, int d, int wl, int wr) {
  if (clb < 1 || crb < 1 || clk < 1 || crk < 1 || d < 1 || wl < 1 || wr < 1) return false;
  const long long y2 = (long long)clb * crb * wl * d * wr;
  return y2 < (1LL << 40) && (long long)clb * wl < (1LL << 31) && (long long)d * crk < (1LL << 31) &&
         (long long)crb * wr < (1LL << 31) && (long long)clk * d < (1LL << 31) && (long long)wr * crk < (1LL << 31);
}

bool dims_ok(int cl, int d, int cr, int wl, int wr) {
  if (cl < 1 || d < 1 || cr < 1 || wl < 1 || wr < 1) return false;
  const long long y2 = (long long)cl * cr * wl * d * wr;
  return y2 < (1LL << 40) && (long long)cl * wl < (1LL << 31) && (long long)d * cr < (1LL << 31);
}

}  // namespace
}  // namespace dmrg

using namespace dmrg;

extern "C" size_t dmrg_env_gradient_workspace_bytes(int dtype, int chil, int d, int chir, int wl, int wr) {
  if (!dims_ok(chil, d, chir, wl, wr)) return 0;
  return dtype == DMRG_COMPLEX128 ? grad_ws<cplx>(chil, d, chir, wl, wr) : grad_ws<double>(chil, d, chir, wl, wr);
}

extern "C" int dmrg_env_gradient(int dtype, int chil, int d, int chir, int wl, int wr, const void* L, const void* A,
                                 const void* R, void* G, void* work, size_t work_bytes, void* stream) {
  if (!dims_ok(chil, d, chir, wl, wr) || !L || !A || !R || !G || !work) return DMRG_ERR_ARG;
  if (dtype != DMRG_REAL64 && dtype != DMRG_COMPLEX128) return DMRG_ERR_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (dtype == DMRG_COMPLEX128)
    return env_gradient<cplx>(chil, d, chir, wl, wr, static_cast<const cplx*>(L), static_cast<const cplx*>(A),
                              static_cast<const cplx*>(R), static_cast<cplx*>(G), work, work_bytes, s);
  return env_gradient<double>(chil, d, chir, wl, wr, static_cast<const double*>(L), static_cast<const double*>(A),
                              static_cast<const double*>(R), static_cast<double*>(G), work, work_bytes, s);
}

extern "C" size_t dmrg_env_mixed_workspace_bytes(int side, int dtype, int clb, int crb, int clk, int crk, int d, int wl,
                                                 int wr) {
  if ((side != 0 && side != 1) || !mixed_dims_ok(clb, crb, clk, crk, d, wl, wr)) return 0;
  return dtype == DMRG_COMPLEX128 ? mixed_env_ws<cplx>(side, clb, crb, clk, crk, d, wl, wr)
                                  : mixed_env_ws<double>(side, clb, crb, clk, crk, d, wl, wr);
}

extern "C" int dmrg_env_extend_mixed(int side, int dtype, int clb, int crb, int clk, int crk, int d, int wl, int wr,
                                     const void* E, const void* W, const void* B, const void* A, void* Enew,
                                     void* work, size_t work_bytes, void* stream) {
  if ((side != 0 && side != 1) || !mixed_dims_ok(clb, crb, clk, crk, d, wl, wr) || !E || !W || !B || !A || !Enew ||
      !work)
    return DMRG_ERR_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (dtype == DMRG_COMPLEX128)
    return env_mixed<cplx>(side, clb, crb, clk, crk, d, wl, wr, static_cast<const cplx*>(E),
                           static_cast<const cplx*>(W), static_cast<const cplx*>(B), static_cast<const cplx*>(A),
                           static_cast<cplx*>(Enew), work, work_bytes, s);
  if (dtype != DMRG_REAL64) return DMRG_ERR_ARG;
  return env_mixed<double>(side, clb, crb, clk, crk, d, wl, wr, static_cast<const double*>(E),
                           static_cast<const double*>(W), static_cast<const double*>(B), static_cast<const double*>(A),
                           static_cast<double*>(Enew), work, work_bytes, s);
}

extern "C" size_t dmrg_env_gradient_mixed_workspace_bytes(int dtype, int clb, int crb, int clk, int crk, int d, int wl,
                                                          int wr) {
  if (!mixed_dims_ok(clb, crb, clk, crk, d, wl, wr)) return 0;
  return dtype == DMRG_COMPLEX128 ? mixed_grad_ws<cplx>(clb, crb, clk, crk, d, wl, wr)
                                  : mixed_grad_ws<double>(clb, crb, clk, crk, d, wl, wr);
}

extern "C" int dmrg_env_gradient_mixed(int dtype, int clb, int crb, int clk, int crk, int d, int wl, int wr,
                                       const void* L, const void* B, const void* A, const void* R, void* G, void* work,
                                       size_t work_bytes, void* stream) {
  if (!mixed_dims_ok(clb, crb, clk, crk, d, wl, wr) || !L || !B || !A || !R || !G || !work) return DMRG_ERR_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (dtype == DMRG_COMPLEX128)
    return env_gradient_mixed<cplx>(clb, crb, clk, crk, d, wl, wr, static_cast<const cplx*>(L),
                                    static_cast<const cplx*>(B), static_cast<const cplx*>(A),
                                    static_cast<const cplx*>(R), static_cast<cplx*>(G), work, work_bytes, s);
  if (dtype != DMRG_REAL64) return DMRG_ERR_ARG;
  return env_gradient_mixed<double>(clb, crb, clk, crk, d, wl, wr, static_cast<const double*>(L),
                                    static_cast<const double*>(B), static_cast<const double*>(A),
                                    static_cast<const double*>(R), static_cast<double*>(G), work, work_bytes, s);
}
