// Symmetric eigendecomposition A = V diag(w) V^T by the parallel cyclic
// block-Jacobi method (two-sided), the eigensolver of the Gram-matrix
// truncation route (pyitensor/svd.py:108-151 diagonalises M M^dag with
// np.linalg.eigh; this kernel set stands in for that call).
//
// The matrix is padded to np = a multiple of 32 (zero rows and columns,
// which no rotation ever touches) and cut into nb = np/16 blocks of 16
// indices.  One sweep visits every pair of blocks once, in nb-1 rounds of
// nb/2 disjoint pairs (round-robin tournament).  A round is two launches:
//   solve  one CTA per pair: one cyclic scalar Jacobi sweep over the 32 x 32
//          subproblem [G_II G_IJ; G_JI G_JJ] in shared memory (16 disjoint
//          rotations at a time, one 2 x 2 block of the matrix per thread,
//          Golub & Van Loan's symmetric Schur rotation), writing the
//          accumulated rotation out;
//   apply  G <- P^T G P and V <- V P with P = the pairs' rotations: one CTA
//          per 32 x 32 block (X, Y) of pair rows/columns (upper triangle,
//          mirrored) and one per 32-row panel of V and pair X.
// The rotation of a pair is kept as D = R - I and applied as a correction,
// G_XY + D_X^T G_XY + (...) D_Y and V + V D_X: a nearly converged (small)
// rotation then adds rounding only at the size of its own effect, instead
// of eps |G| to every entry of the blocks it touches, which would let the
// eigenvalues drift over the hundreds of rounds a large matrix takes and
// keep re-creating off-diagonal noise above the stop threshold.  A pair
// whose subproblem is already diagonal to the threshold records D = 0 and
// its blocks are skipped by the apply.  The sweep loop stops when a full
// sweep rotated nothing.
//
// Two element types: FP64 (the Gram route and the FP64 subspace route) and
// FP32 (the Ritz values of the split-TF32 truncation, whose inputs are
// FP32-accurate anyway; FP32 runs at 64x the FP64 rate on GB300, where FP64
// is ~2 FMA per clock per SM and bounds the FP64 apply at 8 n^3 FLOP per
// sweep).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "heff.cuh"

namespace dmrg {

namespace {

constexpr int JB = 16;        // indices per block
constexpr int JP = 2 * JB;    // subproblem size (one pair of blocks)
constexpr int JLD = JP + 1;   // padded shared-memory row

// Relative (x sqrt|a_pp a_qq|) and absolute (x max|a_ii|) thresholds below
// which an off-diagonal element counts as zero, per element type.  One inner
// sweep per round: a NumPy model of the block method (same tournament, same
// thresholds) needs as many outer sweeps with one inner sweep as with the
// subproblem diagonalised in full, at a fraction of the solve time.
template <typename T> struct JacTol;
template <> struct JacTol<double> {
  static constexpr double rel = 1e-14, abs = 1e-15;
};
template <> struct JacTol<float> {
  static constexpr double rel = 2e-6, abs = 1e-13;
};
constexpr int JAC_MAX_INNER = 1;

struct SyevWs {
  int np, nb, npair;
  double* G;                 // np x np (FP32 runs use the first half)
  double* V;                 // np x np
  double* T;                 // np x np (FP64 runs with an FP32 presolve)
  double* R;                 // npair x 32 x 32: D = R - I of each pair
  int* ident;                // npair
  int* pairs;                // (nb-1) x npair x 2
  int* flag;                 // [0] rotating subproblems in the sweep
  unsigned long long* scale; // max |a_ii| as ordered bits
  double* diag;              // np
  int* perm;                 // np
};

size_t syev_layout(int n, SyevWs* w, void* base) {
  const int np = (n + JP - 1) / JP * JP;
  const int nb = np / JB, npair = nb / 2;
  char* p = static_cast<char*>(base);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    void* q = p ? p + off : nullptr;
    off += align_up(bytes);
    return q;
  };
  SyevWs s;
  s.np = np; s.nb = nb; s.npair = npair;
  s.G = static_cast<double*>(take(sizeof(double) * (size_t)np * np));
  s.V = static_cast<double*>(take(sizeof(double) * (size_t)np * np));
  s.T = static_cast<double*>(take(sizeof(double) * (size_t)np * np));
  s.R = static_cast<double*>(take(sizeof(double) * (size_t)npair * JP * JP));
  s.ident = static_cast<int*>(take(sizeof(int) * npair));
  s.pairs = static_cast<int*>(take(sizeof(int) * 2 * (size_t)(nb - 1 > 0 ? nb - 1 : 1) * npair));
  s.flag = static_cast<int*>(take(sizeof(int) * 4));
  s.scale = static_cast<unsigned long long*>(take(sizeof(unsigned long long)));
  s.diag = static_cast<double*>(take(sizeof(double) * np));
  s.perm = static_cast<int*>(take(sizeof(int) * np));
  if (w) *w = s;
  return off;
}

template <typename T>
__global__ void syev_init_kernel(const double* __restrict__ A, long long lda, int n, int np, T* __restrict__ G,
                                 T* __restrict__ V, unsigned long long* __restrict__ scale) {
  const long long total = (long long)np * np;
  unsigned long long mx = 0;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e / np), j = (int)(e - (long long)i * np);
    double v = 0.0;
    if (i < n && j < n) v = A[(long long)i * lda + j];
    G[e] = (T)v;
    V[e] = i == j ? (T)1 : (T)0;
    if (i == j) {
      // |v| as bits: the order of non-negative doubles is that of their bits
      const double a = fabs(v);
      unsigned long long b;
      memcpy(&b, &a, sizeof(b));
      if (a == a && b > mx) mx = b;
    }
  }
  if (mx) atomicMax(scale, mx);
}

// index at tournament position pos (0..31) in inner round ir
__device__ __forceinline__ int tour(int pos, int ir) { return pos == 0 ? 0 : 1 + (pos - 1 + ir) % (JP - 1); }

template <typename T>
__global__ void __launch_bounds__(256) syev_solve_kernel(const T* __restrict__ G, int np,
                                                         const int* __restrict__ pr, T* __restrict__ R,
                                                         int* __restrict__ ident, int* __restrict__ flag,
                                                         const unsigned long long* __restrict__ scale) {
  __shared__ T a[JP][JLD];
  __shared__ T r[JP][JLD];
  __shared__ T cs[JB], sn[JB], cm[JB];
  __shared__ int pp[JB], qq[JB];
  const int pair = blockIdx.x;
  const int bi = pr[2 * pair], bj = pr[2 * pair + 1];
  const int tid = threadIdx.x;
  double sc;
  {
    const unsigned long long b = *scale;
    memcpy(&sc, &b, sizeof(sc));
  }
  const T floor_ = (T)(JacTol<T>::abs * sc);
  const T rtol = (T)JacTol<T>::rel;
  for (int e = tid; e < JP * JP; e += blockDim.x) {
    const int i = e / JP, j = e - (e / JP) * JP;
    const int gi = i < JB ? bi * JB + i : bj * JB + i - JB;
    const int gj = j < JB ? bi * JB + j : bj * JB + j - JB;
    a[i][j] = G[(long long)gi * np + gj];
    r[i][j] = (T)0;
  }
  __syncthreads();
  int any = 0;
  for (int sw = 0; sw < JAC_MAX_INNER; ++sw) {
    int rotated = 0;
    for (int ir = 0; ir < JP - 1; ++ir) {
      if (tid < JB) {
        const int p = tour(tid, ir), q = tour(JP - 1 - tid, ir);
        const T apq = a[p][q], app = a[p][p], aqq = a[q][q];
        T c = (T)1, s = (T)0, cm1 = (T)0;
        if (fabs(apq) > fmax(rtol * sqrt(fabs(app * aqq)), floor_)) {
          // symmetric Schur rotation (Golub & Van Loan, Alg. 8.4.1)
          const T tau = (aqq - app) / ((T)2 * apq);
          const T at = fabs(tau);
          const T big = sizeof(T) == 8 ? (T)1e150 : (T)1e18;
          T t = at < big ? (T)1 / (at + sqrt((T)1 + at * at)) : (T)0.5 / at;
          t = copysign(t, tau);
          const T u = sqrt((T)1 + t * t);
          c = (T)1 / u;
          cm1 = -t * t / (u * ((T)1 + u));   // c - 1 without cancellation
          s = t * c;
          if (s != (T)0) rotated = 1;
        }
        pp[tid] = p; qq[tid] = q; cs[tid] = c; sn[tid] = s; cm[tid] = cm1;
      }
      __syncthreads();
      {
        const int ti = tid >> 4, tj = tid & 15;
        if (ti <= tj) {
          const int pi = pp[ti], qi = qq[ti], pj = pp[tj], qj = qq[tj];
          const T ci = cs[ti], si = sn[ti], cj = cs[tj], sj = sn[tj];
          if (ti == tj) {
            if (si != (T)0) {
              const T t = si / ci;
              const T apq = a[pi][qi];
              a[pi][pi] -= t * apq;
              a[qi][qi] += t * apq;
              a[pi][qi] = (T)0;
              a[qi][pi] = (T)0;
            }
          } else if (si != (T)0 || sj != (T)0) {
            const T x00 = a[pi][pj], x01 = a[pi][qj], x10 = a[qi][pj], x11 = a[qi][qj];
            const T y00 = ci * x00 - si * x10, y01 = ci * x01 - si * x11;
            const T y10 = si * x00 + ci * x10, y11 = si * x01 + ci * x11;
            const T z00 = cj * y00 - sj * y01, z01 = sj * y00 + cj * y01;
            const T z10 = cj * y10 - sj * y11, z11 = sj * y10 + cj * y11;
            a[pi][pj] = z00; a[pi][qj] = z01; a[qi][pj] = z10; a[qi][qj] = z11;
            a[pj][pi] = z00; a[qj][pi] = z01; a[pj][qi] = z10; a[qj][qi] = z11;
          }
        }
        // D <- (D + I) J - I = D J + (J - I) on columns p, q of pair
        // (tid & 15), rows tid >> 4 and +16
        const int pj = tid & 15;
        const T s = sn[pj], cm1 = cm[pj];
        if (s != (T)0) {
          const int p = pp[pj], q = qq[pj];
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int rr = (tid >> 4) + 16 * h;
            const T u = r[rr][p], v = r[rr][q];
            T np_ = fma(cm1, u, u) - s * v;
            T nq_ = fma(s, u, fma(cm1, v, v));
            if (rr == p) { np_ += cm1; nq_ += s; }
            if (rr == q) { np_ -= s; nq_ += cm1; }
            r[rr][p] = np_;
            r[rr][q] = nq_;
          }
        }
      }
      __syncthreads();
    }
    if (!__syncthreads_or(rotated)) break;
    any = 1;
  }
  T* Rp = R + (size_t)pair * JP * JP;
  for (int e = tid; e < JP * JP; e += blockDim.x) Rp[e] = r[e / JP][e % JP];
  if (tid == 0) {
    ident[pair] = any ? 0 : 1;
    if (any) atomicAdd(flag, 1);
  }
}

__device__ __forceinline__ int pair_index(int b0, int b1, int l) { return l < JB ? b0 * JB + l : b1 * JB + l - JB; }

// G <- P^T G P on blocks (X, Y), X <= Y (grid part 1, npair^2 CTAs, the
// lower triangle exits) and V <- V P on 32-row panels (grid part 2)
template <typename T>
__global__ void __launch_bounds__(256) syev_apply_kernel(T* __restrict__ G, T* __restrict__ V, int np,
                                                         const int* __restrict__ pr, const T* __restrict__ R,
                                                         const int* __restrict__ ident, int npair) {
  __shared__ T x[JP][JLD];
  __shared__ T rx[JP][JLD];
  __shared__ T ry[JP][JLD];
  __shared__ T t[JP][JLD];
  const int tid = threadIdx.x;
  const int i = tid >> 3, j0 = (tid & 7) * 4;
  int b = blockIdx.x;
  const int nG = npair * npair;
  if (b < nG) {
    const int X = b / npair, Y = b - (b / npair) * npair;
    if (X > Y) return;
    const int idX = ident[X], idY = ident[Y];
    if (idX && idY) return;
    const int xb0 = pr[2 * X], xb1 = pr[2 * X + 1], yb0 = pr[2 * Y], yb1 = pr[2 * Y + 1];
    for (int e = tid; e < JP * JP; e += blockDim.x) {
      const int r0 = e / JP, c0 = e - (e / JP) * JP;
      x[r0][c0] = G[(long long)pair_index(xb0, xb1, r0) * np + pair_index(yb0, yb1, c0)];
      rx[r0][c0] = R[(size_t)X * JP * JP + e];
      ry[r0][c0] = R[(size_t)Y * JP * JP + e];
    }
    __syncthreads();
    T o[4];
    // t = x + D_X^T x
#pragma unroll
    for (int q = 0; q < 4; ++q) o[q] = (T)0;
    if (!idX) {
#pragma unroll 8
      for (int k = 0; k < JP; ++k) {
        const T rk = rx[k][i];
#pragma unroll
        for (int q = 0; q < 4; ++q) o[q] = fma(rk, x[k][j0 + q], o[q]);
      }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      o[q] += x[i][j0 + q];
      t[i][j0 + q] = o[q];
    }
    __syncthreads();
    // out = t + t D_Y
    if (!idY) {
      T d[4] = {(T)0, (T)0, (T)0, (T)0};
#pragma unroll 8
      for (int k = 0; k < JP; ++k) {
        const T tk = t[i][k];
#pragma unroll
        for (int q = 0; q < 4; ++q) d[q] = fma(tk, ry[k][j0 + q], d[q]);
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) o[q] += d[q];
    }
    const long long gi = pair_index(xb0, xb1, i);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const long long gj = pair_index(yb0, yb1, j0 + q);
      G[gi * np + gj] = o[q];
      if (X != Y) G[gj * np + gi] = o[q];
    }
    return;
  }
  b -= nG;
  const int X = b % npair, rt = b / npair;
  if (ident[X]) return;
  const int xb0 = pr[2 * X], xb1 = pr[2 * X + 1];
  for (int e = tid; e < JP * JP; e += blockDim.x) {
    const int r0 = e / JP, c0 = e - (e / JP) * JP;
    x[r0][c0] = V[(long long)(rt * JP + r0) * np + pair_index(xb0, xb1, c0)];
    rx[r0][c0] = R[(size_t)X * JP * JP + e];
  }
  __syncthreads();
  // V <- V + V D_X
  T o[4] = {(T)0, (T)0, (T)0, (T)0};
#pragma unroll 8
  for (int k = 0; k < JP; ++k) {
    const T v = x[i][k];
#pragma unroll
    for (int q = 0; q < 4; ++q) o[q] = fma(v, rx[k][j0 + q], o[q]);
  }
#pragma unroll
  for (int q = 0; q < 4; ++q)
    V[(long long)(rt * JP + i) * np + pair_index(xb0, xb1, j0 + q)] = x[i][j0 + q] + o[q];
}

// out (double, np x np) = in (float, np x np)
__global__ void syev_widen_kernel(const float* __restrict__ in, double* __restrict__ out, long long total) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x)
    out[e] = (double)in[e];
}

// B = 1.5 I - 0.5 B in place (the Newton-Schulz factor from B = Q^T Q)
__global__ void syev_ns_kernel(double* __restrict__ B, int np) {
  const long long total = (long long)np * np;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e / np), j = (int)(e - (long long)i * np);
    B[e] = (i == j ? 1.5 : 0.0) - 0.5 * B[e];
  }
}

// *scale = max_i |G_ii| as ordered bits
__global__ void syev_scale_kernel(const double* __restrict__ G, int np, unsigned long long* __restrict__ scale) {
  unsigned long long mx = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
    const double a = fabs(G[(long long)i * np + i]);
    unsigned long long b;
    memcpy(&b, &a, sizeof(b));
    if (a == a && b > mx) mx = b;
  }
  if (mx) atomicMax(scale, mx);
}

template <typename T>
__global__ void syev_diag_kernel(const T* __restrict__ G, int np, double* __restrict__ d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < np) d[i] = (double)G[(long long)i * np + i];
}

// out[r * ldo + c] = V[r * np + perm[c]] for r < n, c < ncols (transposed:
// out[c * ldo + r])
template <typename T>
__global__ void syev_gather_kernel(const T* __restrict__ V, int np, const int* __restrict__ perm, int n, int ncols,
                                   double* __restrict__ out, long long ldo, int transposed) {
  const long long total = (long long)n * ncols;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    if (!transposed) {
      const int r = (int)(e / ncols), c = (int)(e - (long long)r * ncols);
      out[(long long)r * ldo + c] = (double)V[(long long)r * np + perm[c]];
    } else {
      const int c = (int)(e / n), r = (int)(e - (long long)c * n);
      out[(long long)c * ldo + r] = (double)V[(long long)r * np + perm[c]];
    }
  }
}

inline int grid_for(long long n) {
  long long g = (n + 255) / 256;
  if (g > 152 * 8) g = 152 * 8;
  return (int)(g < 1 ? 1 : g);
}

// round-robin tournament of nb blocks: round r pairs positions (i, nb-1-i)
void tournament(int nb, std::vector<int>& out) {
  const int npair = nb / 2, rounds = nb - 1;
  out.assign((size_t)2 * (rounds > 0 ? rounds : 1) * npair, 0);
  auto at = [&](int pos, int r) { return pos == 0 ? 0 : 1 + (pos - 1 + r) % (nb - 1); };
  for (int r = 0; r < rounds; ++r)
    for (int i = 0; i < npair; ++i) {
      out[(size_t)2 * (r * npair + i)] = at(i, r);
      out[(size_t)2 * (r * npair + i) + 1] = at(nb - 1 - i, r);
    }
}

// sweeps over (G, V) until one rotates nothing (at most max_sweeps)
template <typename T>
int syev_sweeps(SyevWs& ws, T* G, T* V, int max_sweeps, int* done, int* converged, cudaStream_t s) {
  const int np = ws.np, npair = ws.npair, rounds = ws.nb - 1;
  T* R = reinterpret_cast<T*>(ws.R);
  const int apply_grid = npair * npair + (np / JP) * npair;
  int sw = 0, conv = 0;
  for (; sw < max_sweeps && !conv; ++sw) {
    DMRG_CUDA_TRY(cudaMemsetAsync(ws.flag, 0, sizeof(int), s));
    for (int r = 0; r < rounds; ++r) {
      const int* pr = ws.pairs + (size_t)2 * r * npair;
      syev_solve_kernel<T><<<npair, 256, 0, s>>>(G, np, pr, R, ws.ident, ws.flag, ws.scale);
      DMRG_CHECK_LAUNCH();
      syev_apply_kernel<T><<<apply_grid, 256, 0, s>>>(G, V, np, pr, R, ws.ident, npair);
      DMRG_CHECK_LAUNCH();
    }
    int h = 0;
    DMRG_CUDA_TRY(cudaMemcpyAsync(&h, ws.flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    DMRG_CUDA_TRY(cudaStreamSynchronize(s));
    conv = h == 0;
  }
  *done += sw;
  *converged = conv;
  return DMRG_OK;
}

// C (np x np) = A B, all np x np row-major FP64
int syev_gemm(int np, const double* A, const double* B, double* C, cudaStream_t s) {
  TGemm g{};
  g.B = ax(1); g.M = ax(np); g.K = ax(np); g.N = ax(np);
  g.a_m = st(np); g.a_k = st(1);
  g.b_k = st(np); g.b_n = st(1);
  g.c_m = st(np); g.c_n = st(1);
  return tgemm<double>(g, 1.0, A, B, 0.0, C, s);
}

// Sorted eigenvalues to the host and the permutation to the workspace.
template <typename T>
int syev_finish(int n, SyevWs& ws, const T* G, double* w, cudaStream_t s) {
  const int np = ws.np;
  syev_diag_kernel<T><<<(np + 255) / 256, 256, 0, s>>>(G, np, ws.diag);
  DMRG_CHECK_LAUNCH();
  std::vector<double> d(n);
  DMRG_CUDA_TRY(cudaMemcpyAsync(d.data(), ws.diag, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  DMRG_CUDA_TRY(cudaStreamSynchronize(s));
  for (int i = 0; i < n; ++i)
    if (!(d[i] == d[i])) return DMRG_ERR_NAN;
  std::vector<int> perm(n);
  std::iota(perm.begin(), perm.end(), 0);
  std::stable_sort(perm.begin(), perm.end(), [&](int x, int y) { return d[x] > d[y]; });
  for (int i = 0; i < n; ++i) w[i] = d[perm[i]];
  DMRG_CUDA_TRY(cudaMemcpyAsync(ws.perm, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
  // the host vector perm must outlive the copy
  DMRG_CUDA_TRY(cudaStreamSynchronize(s));
  return DMRG_OK;
}

// Eigenvectors of an FP64 matrix from n = 256 on come from an FP32 presolve
// and an FP64 polish: the FP32 sweeps (64x the FP64 rate on GB300) take the
// matrix from cold to off-diagonals ~1e-6 of the diagonal; their rotation Q
// is made orthonormal in FP64 by two Newton-Schulz steps
// (Q <- Q (3 I - Q^T Q) / 2), the matrix transformed as Q^T A Q in FP64, and
// the FP64 sweeps, starting from V = Q, converge quadratically from there
// (two or three sweeps instead of the ten to fifteen of a cold start).
constexpr int PRESOLVE_MIN_N = 256;

template <typename T>
int syev_impl(int n, const double* A, long long lda, double* w, int max_sweeps, int* sweeps, void* work,
              cudaStream_t s) {
  SyevWs ws;
  syev_layout(n, &ws, work);
  const int np = ws.np, nb = ws.nb;
  std::vector<int> tab;
  tournament(nb, tab);
  DMRG_CUDA_TRY(cudaMemcpyAsync(ws.pairs, tab.data(), sizeof(int) * tab.size(), cudaMemcpyHostToDevice, s));
  DMRG_CUDA_TRY(cudaMemsetAsync(ws.scale, 0, sizeof(unsigned long long), s));
  int done = 0, conv = 0;
  const bool presolve = sizeof(T) == 8 && n >= PRESOLVE_MIN_N;
  if (!presolve) {
    T* G = reinterpret_cast<T*>(ws.G);
    T* V = reinterpret_cast<T*>(ws.V);
    syev_init_kernel<T><<<grid_for((long long)np * np), 256, 0, s>>>(A, lda, n, np, G, V, ws.scale);
    DMRG_CHECK_LAUNCH();
    DMRG_TRY(syev_sweeps<T>(ws, G, V, max_sweeps, &done, &conv, s));
    if (sweeps) *sweeps = done;
    DMRG_TRY(syev_finish<T>(n, ws, G, w, s));
    return conv ? DMRG_OK : DMRG_ERR_NOCONV;
  }
  // FP32 presolve: G32 in ws.G, V32 in ws.T
  float* G32 = reinterpret_cast<float*>(ws.G);
  float* V32 = reinterpret_cast<float*>(ws.T);
  syev_init_kernel<float><<<grid_for((long long)np * np), 256, 0, s>>>(A, lda, n, np, G32, V32, ws.scale);
  DMRG_CHECK_LAUNCH();
  int done32 = 0;
  DMRG_TRY(syev_sweeps<float>(ws, G32, V32, 15, &done32, &conv, s));
  const long long nn = (long long)np * np;
  syev_widen_kernel<<<grid_for(nn), 256, 0, s>>>(V32, ws.V, nn);    // Q0 (ws.V)
  DMRG_CHECK_LAUNCH();
  // two Newton-Schulz steps: ws.V -> ws.T -> ws.V
  double* src = ws.V;
  double* dst = ws.T;
  for (int it = 0; it < 2; ++it) {
    DMRG_TRY(tgemm_gram(src, np, np, np, ws.G, s));                  // B = Q^T Q
    syev_ns_kernel<<<grid_for(nn), 256, 0, s>>>(ws.G, np);            // B = 1.5 I - 0.5 B
    DMRG_CHECK_LAUNCH();
    DMRG_TRY(syev_gemm(np, src, ws.G, dst, s));                      // Q B
    std::swap(src, dst);
  }
  // G = Q^T A Q (the padded rows and columns of A are zero): P = A Q[:n] in
  // ws.T, then Q^T P in ws.G
  {
    TGemm g{};
    g.B = ax(1); g.M = ax(n); g.K = ax(n); g.N = ax(np);
    g.a_m = st(lda); g.a_k = st(1);
    g.b_k = st(np); g.b_n = st(1);
    g.c_m = st(np); g.c_n = st(1);
    DMRG_TRY(tgemm<double>(g, 1.0, A, ws.V, 0.0, ws.T, s));
    TGemm h{};
    h.B = ax(1); h.M = ax(np); h.K = ax(n); h.N = ax(np);
    h.a_m = st(1); h.a_k = st(np);
    h.b_k = st(np); h.b_n = st(1);
    h.c_m = st(np); h.c_n = st(1);
    DMRG_TRY(tgemm<double>(h, 1.0, ws.V, ws.T, 0.0, ws.G, s));
  }
  DMRG_CUDA_TRY(cudaMemsetAsync(ws.scale, 0, sizeof(unsigned long long), s));
  syev_scale_kernel<<<(np + 255) / 256, 256, 0, s>>>(ws.G, np, ws.scale);
  DMRG_CHECK_LAUNCH();
  DMRG_TRY(syev_sweeps<double>(ws, ws.G, ws.V, max_sweeps, &done, &conv, s));
  if (sweeps) *sweeps = done;
  DMRG_TRY(syev_finish<double>(n, ws, ws.G, w, s));
  return conv ? DMRG_OK : DMRG_ERR_NOCONV;
}

}  // namespace

size_t syev_jacobi_workspace_bytes(int n) { return n > 0 ? syev_layout(n, nullptr, nullptr) : 0; }

// Eigenvalues (host w, descending) of the symmetric n x n matrix A (ld lda);
// the eigenvectors stay in the workspace for syev_vectors.  fp32 != 0 runs
// the sweeps in FP32 (input rounded to FP32).  At most max_sweeps sweeps;
// DMRG_ERR_NOCONV when the last one still rotated.
int syev_jacobi(int n, const double* A, long long lda, double* w, int max_sweeps, int* sweeps, void* work,
                size_t work_bytes, cudaStream_t s, int fp32) {
  if (n <= 0 || !A || lda < n || !w || max_sweeps < 1) return DMRG_ERR_ARG;
  if (!work || syev_jacobi_workspace_bytes(n) > work_bytes) return DMRG_ERR_WORKSPACE;
  return fp32 ? syev_impl<float>(n, A, lda, w, max_sweeps, sweeps, work, s)
              : syev_impl<double>(n, A, lda, w, max_sweeps, sweeps, work, s);
}

// The eigenvectors of the ncols largest eigenvalues of the last syev_jacobi
// on this workspace (same fp32 flag): out[r * ldo + j] (transposed:
// out[j * ldo + r]).
int syev_vectors(int n, int ncols, double* out, long long ldo, int transposed, void* work, cudaStream_t s, int fp32) {
  if (n <= 0 || ncols < 0 || ncols > n || (ncols > 0 && !out) || !work) return DMRG_ERR_ARG;
  if (ncols == 0) return DMRG_OK;
  if (ldo < (transposed ? n : ncols)) return DMRG_ERR_ARG;
  SyevWs ws;
  syev_layout(n, &ws, work);
  if (fp32)
    syev_gather_kernel<float><<<grid_for((long long)n * ncols), 256, 0, s>>>(
        reinterpret_cast<const float*>(ws.V), ws.np, ws.perm, n, ncols, out, ldo, transposed);
  else
    syev_gather_kernel<double><<<grid_for((long long)n * ncols), 256, 0, s>>>(ws.V, ws.np, ws.perm, n, ncols, out,
                                                                               ldo, transposed);
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

}  // namespace dmrg
