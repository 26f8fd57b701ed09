// Truncated SVD on the device: one-sided (Hestenes) cyclic Jacobi in FP64.
//
// The columns of a working copy X (r x c, column-major, c = min(m, n)) are
// orthogonalised pairwise with the round-robin (tournament) ordering, so the
// c/2 pairs of a round touch disjoint columns and run concurrently, one warp
// per pair: the warp reduces the 2x2 Gram block (|x_p|^2, |x_q|^2,
// x_p^H x_q) with shuffles, builds the Hermitian Jacobi rotation and applies
// it to the two columns of X and of the accumulated V.  Rounds are separated
// by a barrier: __syncthreads() for the single-CTA variant (small matrices,
// the common case at the chain edges and at small chi) or a bounded grid
// barrier for the cooperative multi-CTA variant.  A sweep with no rotation
// above tol*sqrt(|x_p|^2 |x_q|^2) ends the iteration.  The singular values
// are the column norms of X; the singular vectors are X/sigma and V.  Unlike
// the Gram-matrix route this keeps small singular values to high relative
// accuracy, so no exact-SVD fallback is needed.
#include <vector>

#include "common.cuh"

namespace dmrg {

namespace {

constexpr long long kBarrierSpinLimit = 1ll << 26;  // ~seconds: far beyond any real wait

struct GridBar {
  unsigned* count;
  unsigned* gen;
  int* err;
};

// Bounded grid-wide barrier for cooperatively launched grids (all CTAs
// co-resident).  Gives up after kBarrierSpinLimit polls, records
// DMRG_ERR_TIMEOUT and lets every CTA fall through.
__device__ __forceinline__ bool grid_barrier(const GridBar& b) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* vgen = b.gen;
    unsigned g = *vgen;
    __threadfence();
    unsigned arrived = atomicAdd(b.count, 1u);
    if (arrived == gridDim.x - 1) {
      *b.count = 0u;
      __threadfence();
      atomicAdd(b.gen, 1u);
    } else {
      long long it = 0;
      while (*vgen == g) {
        if (++it > kBarrierSpinLimit) {
          atomicExch(b.err, DMRG_ERR_TIMEOUT);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return *((volatile int*)b.err) == 0;
}

template <typename T>
struct HArgs {
  T* X;          // r x c, column-major (ld = r)
  T* V;          // c x c, column-major (ld = c)
  int r, c, cp;  // cp = c rounded up to even
  int max_sweeps;
  double tol;
  const double* frob;  // |M|_F (device): absolute floor of the rotation test
  GridBar bar;
  unsigned* rotcnt;  // [3], used cyclically: sweep k counts into slot k%3
  int* sweeps_out;
  int X_in_smem;
  int abs_floor;  // 1: skip couplings below 1e-16 |M|_F^2 (the divided factor is not returned)
};

template <typename T>
__device__ __forceinline__ void gram2(const T* xp, const T* xq, int r, int lane, double& al, double& be, double& gre,
                                      double& gim);
template <>
__device__ __forceinline__ void gram2<double>(const double* xp, const double* xq, int r, int lane, double& al,
                                              double& be, double& gre, double& gim) {
  al = be = gre = gim = 0.0;
  for (int i = lane; i < r; i += 32) {
    double a = xp[i], b = xq[i];
    al = ::fma(a, a, al);
    be = ::fma(b, b, be);
    gre = ::fma(a, b, gre);
  }
}
template <>
__device__ __forceinline__ void gram2<cplx>(const cplx* xp, const cplx* xq, int r, int lane, double& al, double& be,
                                            double& gre, double& gim) {
  al = be = gre = gim = 0.0;
  for (int i = lane; i < r; i += 32) {
    cplx a = xp[i], b = xq[i];
    al = ::fma(a.x, a.x, ::fma(a.y, a.y, al));
    be = ::fma(b.x, b.x, ::fma(b.y, b.y, be));
    gre = ::fma(a.x, b.x, ::fma(a.y, b.y, gre));   // Re conj(a) b
    gim = ::fma(a.x, b.y, ::fma(-a.y, b.x, gim));  // Im conj(a) b
  }
}

// apply X <- X J on columns (p, q): J = [[c, s e], [-s conj(e), c]]
template <typename T>
__device__ __forceinline__ void rot_cols(T* xp, T* xq, int r, int lane, double c, double s, T e) {
  const T se = Sc<T>::scale(e, s);
  const T sce = Sc<T>::scale(Sc<T>::conj(e), s);
  for (int i = lane; i < r; i += 32) {
    T a = xp[i], b = xq[i];
    xp[i] = Sc<T>::sub(Sc<T>::scale(a, c), Sc<T>::mul(sce, b));
    xq[i] = Sc<T>::add(Sc<T>::mul(se, a), Sc<T>::scale(b, c));
  }
}

__device__ __forceinline__ int player(int pos, int round, int cp) {
  return pos == 0 ? 0 : 1 + (pos - 1 + round) % (cp - 1);
}

template <typename T, bool COOP>
__global__ void __launch_bounds__(1024) hestenes_kernel(HArgs<T> a) {
  extern __shared__ unsigned char hsm[];
  // single-CTA variant: work on a shared-memory copy of X when it fits
  T* const Xg = a.X;
  if (!COOP && a.X_in_smem) {
    T* xs = reinterpret_cast<T*>(hsm);
    for (long long i = threadIdx.x; i < (long long)a.r * a.c; i += blockDim.x) xs[i] = Xg[i];
    a.X = xs;
    __syncthreads();
  }
  const double fro = *a.frob;
  const double abs_floor = a.abs_floor ? 1e-16 * fro * fro : 0.0;
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  const int half = a.cp / 2;
  const long long gtid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long gthreads = (long long)gridDim.x * blockDim.x;

  // V = identity
  for (long long idx = gtid; idx < (long long)a.c * a.c; idx += gthreads) {
    int col = (int)(idx / a.c), row = (int)(idx - (long long)col * a.c);
    a.V[idx] = row == col ? Sc<T>::one() : Sc<T>::zero();
  }
  if (gtid == 0) { a.rotcnt[0] = 0u; a.rotcnt[1] = 0u; a.rotcnt[2] = 0u; }
  if (COOP) { if (!grid_barrier(a.bar)) return; } else { __syncthreads(); }

  int sweep = 0;
  bool converged = a.cp < 2;
  for (; sweep < a.max_sweeps && !converged; ++sweep) {
    // slot (sweep+1)%3 was last read at the end of sweep-2, before at least
    // one barrier of sweep-1, so no CTA can still be reading it
    if (gtid == 0) a.rotcnt[(sweep + 1) % 3] = 0u;
    for (int round = 0; round < a.cp - 1; ++round) {
      for (int i = gw; i < half; i += nw) {
        int p = player(i, round, a.cp), q = player(a.cp - 1 - i, round, a.cp);
        if (p > q) { int t = p; p = q; q = t; }
        if (q >= a.c) continue;  // dummy column of an odd count
        T* xp = a.X + (long long)p * a.r;
        T* xq = a.X + (long long)q * a.r;
        double al, be, gre, gim;
        gram2<T>(xp, xq, a.r, lane, al, be, gre, gim);
        al = warp_sum(al);
        be = warp_sum(be);
        gre = warp_sum(gre);
        gim = warp_sum(gim);
        double ag = sqrt(gre * gre + gim * gim);
        double scale = sqrt(al) * sqrt(be);  // no overflow of the product
        // rotate only couplings above tol relative to the pair and above an
        // absolute floor (1e-16 |M|_F^2): singular values come out to the
        // absolute accuracy of a standard SVD without chasing the relative
        // accuracy of negligible ones, which costs many extra sweeps on the
        // steeply graded spectra of DMRG bonds
        if (!(ag > a.tol * scale) || !(ag > abs_floor) || !(ag > 1e-300)) continue;
        double tau = (be - al) / (2.0 * ag);
        double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
        double cs = 1.0 / sqrt(1.0 + t * t);
        double sn = t * cs;
        T e = Sc<T>::make(gre / ag, gim / ag);
        rot_cols<T>(xp, xq, a.r, lane, cs, sn, e);
        rot_cols<T>(a.V + (long long)p * a.c, a.V + (long long)q * a.c, a.c, lane, cs, sn, e);
        if (lane == 0) atomicAdd(&a.rotcnt[sweep % 3], 1u);
      }
      if (COOP) { if (!grid_barrier(a.bar)) return; } else { __syncthreads(); }
    }
    converged = (((volatile unsigned*)a.rotcnt)[sweep % 3] == 0u);
  }
  if (gtid == 0) *a.sweeps_out = converged ? sweep : -sweep;
  if (!COOP && a.X_in_smem) {
    __syncthreads();
    for (long long i = threadIdx.x; i < (long long)a.r * a.c; i += blockDim.x) Xg[i] = a.X[i];
  }
}

// sigma_j = |X_j|, one warp per column
template <typename T>
__global__ void colnorm_kernel(const T* __restrict__ X, int r, int c, double* __restrict__ sig) {
  const int lane = threadIdx.x & 31;
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= c) return;
  const T* x = X + (long long)w * r;
  double s = 0.0;
  for (int i = lane; i < r; i += 32) s += Sc<T>::abs2(x[i]);
  s = warp_sum(s);
  if (lane == 0) sig[w] = sqrt(s);
}

// perm[k] = index of the k-th largest sigma (stable), sorted[k] = its value
__global__ void rank_kernel(const double* __restrict__ sig, int c, int* __restrict__ perm, double* __restrict__ sorted) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c) return;
  double v = sig[i];
  int rank = 0;
  for (int j = 0; j < c; ++j) {
    double u = sig[j];
    rank += (u > v) || (u == v && j < i);
  }
  perm[rank] = i;
  sorted[rank] = v;
}

// copy M (row-major m x n) into X (column-major r x c):
//   left = (m <= n): X = M^H  (r = n, c = m): X[j*n + i] = conj(M[j*n + i])
//   else           : X = M    (r = m, c = n): X[j*m + i] = M[i*n + j]
template <typename T>
__global__ void load_x_kernel(const T* __restrict__ M, int m, int n, int left, T* __restrict__ X) {
  long long total = (long long)m * n;
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += stride) {
    if (left) {
      X[idx] = Sc<T>::conj(M[idx]);
    } else {
      int j = (int)(idx / m), i = (int)(idx - (long long)j * m);
      X[idx] = M[(long long)i * n + j];
    }
  }
}

// Outputs.  left case (X = M^H V = Y, U = V, S.Vh = Y^H):
//   lo[i,k] = V[i, perm k] * (absorb==1 ? sigma_k : 1)           (m x keep)
//   ro[k,j] = conj(Y[j, perm k]) / (absorb==0 ? 1 : sigma_k)     (keep x n)
// right case (X = M V = Y, U = Y/sigma, Vh = V^H):
//   lo[i,k] = Y[i, perm k] / (absorb==1 ? 1 : sigma_k)
//   ro[k,j] = conj(V[j, perm k]) * (absorb==0 ? sigma_k : 1)
template <typename T>
__global__ void out_kernel(const T* __restrict__ X, const T* __restrict__ V, const int* __restrict__ perm,
                           const double* __restrict__ sorted, int m, int n, int left, int keep, int absorb,
                           T* __restrict__ lo, T* __restrict__ ro) {
  long long nl = (long long)m * keep, nr = (long long)keep * n;
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < nl + nr; idx += stride) {
    if (idx < nl) {
      int i = (int)(idx / keep), k = (int)(idx - (long long)i * keep);
      int pk = perm[k];
      double sg = sorted[k];
      T v;
      if (left) {
        v = V[(long long)pk * m + i];
        if (absorb == 1) v = Sc<T>::scale(v, sg);
      } else {
        v = X[(long long)pk * m + i];
        if (absorb != 1) v = Sc<T>::scale(v, sg > 0.0 ? 1.0 / sg : 0.0);
      }
      lo[idx] = v;
    } else {
      long long o = idx - nl;
      int k = (int)(o / n), j = (int)(o - (long long)k * n);
      int pk = perm[k];
      double sg = sorted[k];
      T v;
      if (left) {
        v = Sc<T>::conj(X[(long long)pk * n + j]);
        if (absorb != 0) v = Sc<T>::scale(v, sg > 0.0 ? 1.0 / sg : 0.0);
      } else {
        v = Sc<T>::conj(V[(long long)pk * n + j]);
        if (absorb == 0) v = Sc<T>::scale(v, sg);
      }
      ro[o] = v;
    }
  }
}

// ---------------------------------------------------------------- batched
// Many small SVDs at once (one CTA per problem, X and V in global memory):
// the same one-sided Jacobi with the same tolerances as the single-problem
// kernel, rounds separated by __syncthreads().  Used by the batched sweep of
// many independent chains.
template <typename T>
struct BSvd {
  const T* M;
  int m, n, left, r, c;
  T* X;
  T* V;
  double* sig;
  double* sorted;
  int* perm;
  int* info;  // [0] sweeps (negative: sweep limit reached)
  int abs_floor;
};

template <typename T>
__global__ void __launch_bounds__(1024) hestenes_batch_kernel(const BSvd<T>* __restrict__ tab, int max_sweeps) {
  const BSvd<T> a = tab[blockIdx.x];
  __shared__ double red[32];
  __shared__ unsigned rot;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int r = a.r, c = a.c, cp = c + (c & 1), half = cp / 2;
  T* X = a.X;
  T* V = a.V;
  const long long mn = (long long)a.m * a.n;
  double part = 0.0;
  for (long long idx = threadIdx.x; idx < mn; idx += blockDim.x) {
    T v;
    if (a.left) {
      v = Sc<T>::conj(a.M[idx]);
    } else {
      const int j = (int)(idx / a.m), i = (int)(idx - (long long)j * a.m);
      v = a.M[(long long)i * a.n + j];
    }
    X[idx] = v;
    part += Sc<T>::abs2(v);
  }
  for (long long idx = threadIdx.x; idx < (long long)c * c; idx += blockDim.x) {
    const int col = (int)(idx / c), row = (int)(idx - (long long)col * c);
    V[idx] = row == col ? Sc<T>::one() : Sc<T>::zero();
  }
  part = warp_sum(part);
  if (lane == 0) red[wid] = part;
  __syncthreads();
  double fro2 = 0.0;
  for (int w = 0; w < nw; ++w) fro2 += red[w];
  const double abs_floor = a.abs_floor ? 1e-16 * fro2 : 0.0;
  double tol = 2.2e-16 * sqrt((double)r);
  tol = tol > 1e-15 ? tol : 1e-15;
  int sweep = 0;
  bool converged = cp < 2;
  for (; sweep < max_sweeps && !converged; ++sweep) {
    if (threadIdx.x == 0) rot = 0u;
    __syncthreads();
    for (int round = 0; round < cp - 1; ++round) {
      for (int i = wid; i < half; i += nw) {
        int p = player(i, round, cp), q = player(cp - 1 - i, round, cp);
        if (p > q) { const int t = p; p = q; q = t; }
        if (q >= c) continue;
        T* xp = X + (long long)p * r;
        T* xq = X + (long long)q * r;
        double al, be, gre, gim;
        gram2<T>(xp, xq, r, lane, al, be, gre, gim);
        al = warp_sum(al);
        be = warp_sum(be);
        gre = warp_sum(gre);
        gim = warp_sum(gim);
        const double ag = sqrt(gre * gre + gim * gim);
        const double scale = sqrt(al) * sqrt(be);
        if (!(ag > tol * scale) || !(ag > abs_floor) || !(ag > 1e-300)) continue;
        const double tau = (be - al) / (2.0 * ag);
        const double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
        const double cs = 1.0 / sqrt(1.0 + t * t);
        const double sn = t * cs;
        const T e = Sc<T>::make(gre / ag, gim / ag);
        rot_cols<T>(xp, xq, r, lane, cs, sn, e);
        rot_cols<T>(V + (long long)p * c, V + (long long)q * c, c, lane, cs, sn, e);
        if (lane == 0) atomicAdd(&rot, 1u);
      }
      __syncthreads();
    }
    converged = (*(volatile unsigned*)&rot == 0u);
    __syncthreads();
  }
  // singular values, then their descending (stable) order
  for (int col = wid; col < c; col += nw) {
    const T* x = X + (long long)col * r;
    double s2 = 0.0;
    for (int i = lane; i < r; i += 32) s2 += Sc<T>::abs2(x[i]);
    s2 = warp_sum(s2);
    if (lane == 0) a.sig[col] = sqrt(s2);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < c; i += blockDim.x) {
    const double v = a.sig[i];
    int rank = 0;
    for (int j = 0; j < c; ++j) {
      const double u = a.sig[j];
      rank += (u > v) || (u == v && j < i);
    }
    a.perm[rank] = i;
    a.sorted[rank] = v;
  }
  if (threadIdx.x == 0) a.info[0] = converged ? sweep : -sweep;
}

template <typename T>
struct BOut {
  const T* X;
  const T* V;
  const int* perm;
  const double* sorted;
  int m, n, left, keep;
  T* lo;
  T* ro;
};

// grid (blocks, nprob): the single-problem out_kernel per problem
template <typename T>
__global__ void out_batch_kernel(const BOut<T>* __restrict__ tab, int absorb) {
  const BOut<T> o = tab[blockIdx.y];
  const int m = o.m, n = o.n, keep = o.keep;
  const long long nl = (long long)m * keep, nr = (long long)keep * n;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < nl + nr; idx += stride) {
    if (idx < nl) {
      const int i = (int)(idx / keep), k = (int)(idx - (long long)i * keep);
      const int pk = o.perm[k];
      const double sg = o.sorted[k];
      T v;
      if (o.left) {
        v = o.V[(long long)pk * m + i];
        if (absorb == 1) v = Sc<T>::scale(v, sg);
      } else {
        v = o.X[(long long)pk * m + i];
        if (absorb != 1) v = Sc<T>::scale(v, sg > 0.0 ? 1.0 / sg : 0.0);
      }
      o.lo[idx] = v;
    } else {
      const long long q = idx - nl;
      const int k = (int)(q / n), j = (int)(q - (long long)k * n);
      const int pk = o.perm[k];
      const double sg = o.sorted[k];
      T v;
      if (o.left) {
        v = Sc<T>::conj(o.X[(long long)pk * n + j]);
        if (absorb != 0) v = Sc<T>::scale(v, sg > 0.0 ? 1.0 / sg : 0.0);
      } else {
        v = Sc<T>::conj(o.V[(long long)pk * n + j]);
        if (absorb == 0) v = Sc<T>::scale(v, sg);
      }
      o.ro[q] = v;
    }
  }
}

inline int egrid(long long n) {
  long long g = (n + 255) / 256;
  if (g > 152 * 8) g = 152 * 8;
  if (g < 1) g = 1;
  return (int)g;
}

}  // namespace

struct SvdWork {
  void* X;
  void* V;
  double* sig;
  double* sorted;
  int* perm;
  unsigned* ctrl;  // [0..1] barrier, [2..4] rotation counters, [5] err, [6] sweeps, [8..9] |M|_F
  double* red;     // reduction scratch
};

size_t svd_work_bytes(int dtype, int m, int n) {
  size_t es = dtype == DMRG_COMPLEX128 ? 16 : 8;
  size_t c = (size_t)(m < n ? m : n);
  size_t r = (size_t)(m < n ? n : m);
  return align_up(r * c * es) + align_up(c * c * es) + 2 * align_up(c * 8) + align_up(c * 4) + align_up(64) +
         align_up((8 + 2 * 2 * 152) * 8);
}

static SvdWork carve(void* work, int dtype, int m, int n) {
  size_t es = dtype == DMRG_COMPLEX128 ? 16 : 8;
  size_t c = (size_t)(m < n ? m : n);
  size_t r = (size_t)(m < n ? n : m);
  char* p = static_cast<char*>(work);
  SvdWork w;
  w.X = p; p += align_up(r * c * es);
  w.V = p; p += align_up(c * c * es);
  w.sig = reinterpret_cast<double*>(p); p += align_up(c * 8);
  w.sorted = reinterpret_cast<double*>(p); p += align_up(c * 8);
  w.perm = reinterpret_cast<int*>(p); p += align_up(c * 4);
  w.ctrl = reinterpret_cast<unsigned*>(p); p += align_up(64);
  w.red = reinterpret_cast<double*>(p);
  return w;
}

// Phase 1: factorise.  abs_floor = 1 stops on couplings below 1e-16 |M|_F^2
// (fewer sweeps on graded spectra): the accumulated rotations stay exactly
// orthonormal, but the factor formed as X/sigma is then orthonormal only to
// ~1e-16 |M|^2 / (sigma_p sigma_q); callers enable it only when that factor
// is not the one that must be orthonormal.
// Leaves sorted singular values in w.sorted (device)
// and copies them to host_s.  Returns DMRG_ERR_NOCONV if the sweep limit was
// reached (the factorisation is still usable).
template <typename T>
int hestenes_factor(const T* M, int m, int n, int left, void* work, double* host_s, int* sweeps, int abs_floor,
                    cudaStream_t s) {
  const int r = left ? n : m;
  const int c = left ? m : n;
  SvdWork w = carve(work, sizeof(T) == 16 ? DMRG_COMPLEX128 : DMRG_REAL64, m, n);
  DMRG_CUDA_TRY(cudaMemsetAsync(w.ctrl, 0, 64, s));
  load_x_kernel<T><<<egrid((long long)m * n), 256, 0, s>>>(M, m, n, left, static_cast<T*>(w.X));
  DMRG_CHECK_LAUNCH();
  double* frob = reinterpret_cast<double*>(w.ctrl + 8);
  DMRG_CUDA_TRY(cudaMemsetAsync(w.red, 0, 64, s));
  DMRG_TRY(vnorm<T>(static_cast<const T*>(w.X), (long long)m * n, frob, w.red, s));
  HArgs<T> a;
  a.X = static_cast<T*>(w.X);
  a.V = static_cast<T*>(w.V);
  a.r = r;
  a.c = c;
  a.cp = c + (c & 1);
  a.max_sweeps = 60;
  double tol = 2.2e-16 * sqrt((double)r);
  a.tol = tol > 1e-15 ? tol : 1e-15;
  a.bar.count = w.ctrl + 0;
  a.bar.gen = w.ctrl + 1;
  a.rotcnt = w.ctrl + 2;
  a.bar.err = reinterpret_cast<int*>(w.ctrl + 5);
  a.sweeps_out = reinterpret_cast<int*>(w.ctrl + 6);
  a.frob = frob;
  a.X_in_smem = 0;
  a.abs_floor = abs_floor;
  const int half = a.cp / 2;
  // one CTA while the pairs of a round fit in 32 warps of one CTA and the
  // columns are short; otherwise a cooperative grid with one warp per pair
  if ((half <= 64 && (long long)r * c <= (1ll << 20)) || half <= 8) {
    int threads = 32 * (half < 32 ? (half > 0 ? half : 1) : 32);
    const size_t xbytes = sizeof(T) * (size_t)r * c;
    size_t smem = 0;
    if (xbytes <= 160 * 1024) {
      a.X_in_smem = 1;
      smem = xbytes;
      static std::atomic<unsigned long long> attr_d{0}, attr_z{0};
      DMRG_TRY(smem_attr_once(reinterpret_cast<const void*>(hestenes_kernel<double, false>), 160 * 1024, attr_d));
      DMRG_TRY(smem_attr_once(reinterpret_cast<const void*>(hestenes_kernel<cplx, false>), 160 * 1024, attr_z));
    }
    hestenes_kernel<T, false><<<1, threads, smem, s>>>(a);
    DMRG_CHECK_LAUNCH();
  } else {
    int dev = 0;
    DMRG_CUDA_TRY(cudaGetDevice(&dev));
    int nsm = 0;
    DMRG_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    int per_sm = 0;
    const int threads = 256;
    DMRG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, hestenes_kernel<T, true>, threads, 0));
    if (per_sm < 1) return DMRG_ERR_CUDA;
    int want = (half + (threads / 32) - 1) / (threads / 32);
    int maxb = per_sm * nsm;
    int blocks = want < maxb ? want : maxb;
    if (blocks < 1) blocks = 1;
    void* args[] = {&a};
    DMRG_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)hestenes_kernel<T, true>, blocks, threads, args, 0, s));
    count_launch();
  }
  colnorm_kernel<T><<<(c * 32 + 255) / 256, 256, 0, s>>>(a.X, r, c, w.sig);
  DMRG_CHECK_LAUNCH();
  rank_kernel<<<(c + 255) / 256, 256, 0, s>>>(w.sig, c, w.perm, w.sorted);
  DMRG_CHECK_LAUNCH();
  int ctrl_host[2] = {0, 0};
  DMRG_CUDA_TRY(cudaMemcpyAsync(host_s, w.sorted, sizeof(double) * c, cudaMemcpyDeviceToHost, s));
  DMRG_CUDA_TRY(cudaMemcpyAsync(ctrl_host, w.ctrl + 5, sizeof(int) * 2, cudaMemcpyDeviceToHost, s));
  DMRG_CUDA_TRY(cudaStreamSynchronize(s));
  if (ctrl_host[0] != 0) return ctrl_host[0];
  if (sweeps) *sweeps = ctrl_host[1];
  for (int k = 0; k < c; ++k)
    if (!(host_s[k] == host_s[k]) || host_s[k] > 1e300) return DMRG_ERR_NAN;
  return ctrl_host[1] < 0 ? DMRG_ERR_NOCONV : DMRG_OK;
}

template <typename T>
int hestenes_output(int m, int n, int left, int keep, int absorb, void* work, T* lo, T* ro, cudaStream_t s) {
  SvdWork w = carve(work, sizeof(T) == 16 ? DMRG_COMPLEX128 : DMRG_REAL64, m, n);
  long long tot = (long long)m * keep + (long long)keep * n;
  out_kernel<T><<<egrid(tot), 256, 0, s>>>(static_cast<const T*>(w.X), static_cast<const T*>(w.V), w.perm, w.sorted,
                                           m, n, left, keep, absorb, lo, ro);
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

// Which side Jacobi rotates: left (X = M^H, the accumulated rotations are U)
// when m < n, right (X = M, rotations are V) when m > n; a square matrix
// takes the side whose accumulated, exactly orthonormal, factor is the one
// the caller keeps orthonormal (absorb 0: U, absorb 1: V).
int svd_orientation_left(int m, int n, int absorb) { return m != n ? (m < n) : (absorb != 1); }
// The absolute stop floor (couplings below 1e-16 |M|_F^2 are not rotated)
// leaves the divided factor X/sigma orthonormal only to ~1e-16 |M|^2 /
// (sigma_p sigma_q); it is safe when that factor is not the kept-orthonormal one.
int svd_abs_floor(int left, int absorb) { return (left && absorb == 0) || (!left && absorb == 1); }

// ---- batched host drivers
namespace {
struct BLayout {
  size_t total;
  std::vector<size_t> X, V, sig, sorted, perm, info;
  size_t tab, otab;
};

BLayout batch_layout(size_t es, int nprob, const int* m, const int* n, size_t tab_es, size_t otab_es) {
  BLayout L;
  size_t off = 0;
  L.tab = off; off += align_up(tab_es * (size_t)nprob);
  L.otab = off; off += align_up(otab_es * (size_t)nprob);
  L.X.resize(nprob); L.V.resize(nprob); L.sig.resize(nprob); L.sorted.resize(nprob); L.perm.resize(nprob);
  L.info.resize(nprob);
  for (int p = 0; p < nprob; ++p) {
    const size_t c = (size_t)(m[p] < n[p] ? m[p] : n[p]);
    const size_t r = (size_t)(m[p] < n[p] ? n[p] : m[p]);
    L.X[p] = off; off += align_up(r * c * es);
    L.V[p] = off; off += align_up(c * c * es);
    L.sig[p] = off; off += align_up(c * 8);
    L.sorted[p] = off; off += align_up(c * 8);
    L.perm[p] = off; off += align_up(c * 4);
    L.info[p] = off; off += align_up(8);
  }
  L.total = off;
  return L;
}
}  // namespace

size_t svd_batch_work_bytes(int dtype, int nprob, const int* m, const int* n) {
  const size_t es = dtype == DMRG_COMPLEX128 ? 16 : 8;
  return batch_layout(es, nprob, m, n, sizeof(BSvd<cplx>), sizeof(BOut<cplx>)).total;
}

// Phase 1 for every problem; the sorted singular values of problem p go to
// host_s + p * ld_s.
template <typename T>
int hestenes_batch_factor(int nprob, const int* m, const int* n, const T* const* M, void* work, double* host_s,
                          int ld_s, int absorb, cudaStream_t s) {
  const BLayout L = batch_layout(sizeof(T), nprob, m, n, sizeof(BSvd<cplx>), sizeof(BOut<cplx>));
  char* base = static_cast<char*>(work);
  std::vector<BSvd<T>> tab(nprob);
  for (int p = 0; p < nprob; ++p) {
    BSvd<T>& a = tab[p];
    a.M = M[p];
    a.m = m[p];
    a.n = n[p];
    a.left = svd_orientation_left(m[p], n[p], absorb);
    a.r = a.left ? n[p] : m[p];
    a.c = a.left ? m[p] : n[p];
    a.X = reinterpret_cast<T*>(base + L.X[p]);
    a.V = reinterpret_cast<T*>(base + L.V[p]);
    a.sig = reinterpret_cast<double*>(base + L.sig[p]);
    a.sorted = reinterpret_cast<double*>(base + L.sorted[p]);
    a.perm = reinterpret_cast<int*>(base + L.perm[p]);
    a.info = reinterpret_cast<int*>(base + L.info[p]);
    a.abs_floor = svd_abs_floor(a.left, absorb);
  }
  DMRG_CUDA_TRY(cudaMemcpyAsync(base + L.tab, tab.data(), sizeof(BSvd<T>) * nprob, cudaMemcpyHostToDevice, s));
  hestenes_batch_kernel<T><<<nprob, 1024, 0, s>>>(reinterpret_cast<const BSvd<T>*>(base + L.tab), 60);
  DMRG_CHECK_LAUNCH();
  std::vector<int> info(nprob);
  for (int p = 0; p < nprob; ++p) {
    const int c = tab[p].c;
    DMRG_CUDA_TRY(cudaMemcpyAsync(host_s + (size_t)p * ld_s, tab[p].sorted, sizeof(double) * c,
                                  cudaMemcpyDeviceToHost, s));
    DMRG_CUDA_TRY(cudaMemcpyAsync(&info[p], tab[p].info, sizeof(int), cudaMemcpyDeviceToHost, s));
  }
  DMRG_CUDA_TRY(cudaStreamSynchronize(s));
  int st = DMRG_OK;
  for (int p = 0; p < nprob; ++p) {
    for (int k = 0; k < tab[p].c; ++k) {
      const double v = host_s[(size_t)p * ld_s + k];
      if (!(v == v) || v > 1e300) return DMRG_ERR_NAN;
    }
    if (info[p] < 0) st = DMRG_ERR_NOCONV;
  }
  return st;
}

template <typename T>
int hestenes_batch_output(int nprob, const int* m, const int* n, const int* keep, int absorb, void* work,
                          T* const* lo, T* const* ro, cudaStream_t s) {
  const BLayout L = batch_layout(sizeof(T), nprob, m, n, sizeof(BSvd<cplx>), sizeof(BOut<cplx>));
  char* base = static_cast<char*>(work);
  std::vector<BOut<T>> tab(nprob);
  long long most = 1;
  for (int p = 0; p < nprob; ++p) {
    BOut<T>& o = tab[p];
    o.X = reinterpret_cast<const T*>(base + L.X[p]);
    o.V = reinterpret_cast<const T*>(base + L.V[p]);
    o.perm = reinterpret_cast<const int*>(base + L.perm[p]);
    o.sorted = reinterpret_cast<const double*>(base + L.sorted[p]);
    o.m = m[p];
    o.n = n[p];
    o.left = svd_orientation_left(m[p], n[p], absorb);
    o.keep = keep[p];
    o.lo = lo[p];
    o.ro = ro[p];
    const long long tot = (long long)m[p] * keep[p] + (long long)keep[p] * n[p];
    if (tot > most) most = tot;
  }
  DMRG_CUDA_TRY(cudaMemcpyAsync(base + L.otab, tab.data(), sizeof(BOut<T>) * nprob, cudaMemcpyHostToDevice, s));
  long long gx = (most + 255) / 256;
  if (gx > 64) gx = 64;
  if (nprob > 65535) return DMRG_ERR_ARG;
  out_batch_kernel<T><<<dim3((unsigned)gx, (unsigned)nprob), 256, 0, s>>>(
      reinterpret_cast<const BOut<T>*>(base + L.otab), absorb);
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

template int hestenes_batch_factor<double>(int, const int*, const int*, const double* const*, void*, double*, int,
                                           int, cudaStream_t);
template int hestenes_batch_factor<cplx>(int, const int*, const int*, const cplx* const*, void*, double*, int, int,
                                         cudaStream_t);
template int hestenes_batch_output<double>(int, const int*, const int*, const int*, int, void*, double* const*,
                                           double* const*, cudaStream_t);
template int hestenes_batch_output<cplx>(int, const int*, const int*, const int*, int, void*, cplx* const*,
                                         cplx* const*, cudaStream_t);

template int hestenes_factor<double>(const double*, int, int, int, void*, double*, int*, int, cudaStream_t);
template int hestenes_factor<cplx>(const cplx*, int, int, int, void*, double*, int*, int, cudaStream_t);
template int hestenes_output<double>(int, int, int, int, int, void*, double*, double*, cudaStream_t);
template int hestenes_output<cplx>(int, int, int, int, int, void*, cplx*, cplx*, cudaStream_t);

}  // namespace dmrg
