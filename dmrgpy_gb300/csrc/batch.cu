// Batched sweeps of many independent chains: every step of a bond update
// (two-site merge, Lanczos, truncated SVD, environment extension) runs for
// all chains at once, with problems of different bond dimensions in the same
// launch.
//
//   * contractions: one grouped launch per contraction step
//     (tgemm_grouped: each CTA finds its problem by binary search over a
//     tile table), built from the same step plans as the single-chain path;
//   * Lanczos: the recurrence runs for all chains in lock step; the vector
//     kernels (dot, fused axpy, reorthogonalisation, norm + normalise) run one
//     CTA per chain; blocks of kBlock steps are captured once as a CUDA graph
//     and replayed (the graph is cached per shape signature, so the same bond
//     of the next sweep replays it); only alpha/beta of all chains cross to
//     the host after each block, where each chain's tridiagonal problem and
//     stop test are evaluated exactly as in the single-chain driver;
//   * truncation: one CTA per chain one-sided Jacobi (jacobi.cu), the
//     reference's truncation rule per chain on the host.
// FP64 / complex FP64 throughout (the bond dimensions of such batches are
// small enough that the FP64 pipe is not the limit).
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "heff.cuh"

namespace dmrg {
namespace {

constexpr int kBlock = 8;      // Lanczos steps per captured graph
constexpr int kVecThreads = 512;

template <typename T>
struct LSeg {
  T* x;          // caller's vector (start in, Ritz vector out)
  T* Q;          // (kmax + 1) x n, row j = q_j
  T* w;          // n
  T* v;          // n: input of the matvec (= current q_j)
  double* alpha; // kmax
  double* beta;  // kmax
  T* h;          // kmax + 1: reorthogonalisation coefficients
  const T* y;    // kmax: Ritz coefficients (uploaded by the host)
  long long n;
  int* dead;     // 1 after a breakdown (beta < tol)
};

template <typename T>
__device__ __forceinline__ double block_sum(double v, double* red) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double s = 0.0;
  for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[i];
  return s;
}

template <typename T>
__device__ __forceinline__ double re_dot(T a, T b);
template <>
__device__ __forceinline__ double re_dot<double>(double a, double b) { return a * b; }
template <>
__device__ __forceinline__ double re_dot<cplx>(cplx a, cplx b) { return a.x * b.x + a.y * b.y; }

// q0 = x / |x| (a zero start becomes a fixed pseudo-random vector), into Q[0] and v
template <typename T>
__global__ void __launch_bounds__(kVecThreads) lz_init_kernel(const LSeg<T>* __restrict__ tab) {
  __shared__ double red[32];
  const LSeg<T> a = tab[blockIdx.x];
  double s = 0.0;
  for (long long i = threadIdx.x; i < a.n; i += blockDim.x) s += Sc<T>::abs2(a.x[i]);
  s = block_sum<T>(s, red);
  const bool zero = !(s > 0.0);
  if (zero) {
    double r2 = 0.0;
    for (long long i = threadIdx.x; i < a.n; i += blockDim.x) {
      unsigned long long z = 0x5eedULL ^ (0x9e3779b97f4a7c15ull * (unsigned long long)(i + 1));
      z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
      z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
      z ^= z >> 31;
      const double u = (double)(z >> 11) * (1.0 / 9007199254740992.0) - 0.5;
      a.v[i] = Sc<T>::make(u, 0.0);
      r2 += u * u;
    }
    s = block_sum<T>(r2, red);
  }
  const double inv = 1.0 / sqrt(s);
  for (long long i = threadIdx.x; i < a.n; i += blockDim.x) {
    const T q = Sc<T>::scale(zero ? a.v[i] : a.x[i], inv);
    a.Q[i] = q;
    a.v[i] = q;
  }
  if (threadIdx.x == 0) *a.dead = 0;
}

// alpha_j = Re <q_j, w>;  w -= alpha_j q_j + beta_{j-1} q_{j-1}
template <typename T>
__global__ void __launch_bounds__(kVecThreads) lz_alpha_axpy_kernel(const LSeg<T>* __restrict__ tab, int j) {
  __shared__ double red[32];
  const LSeg<T> a = tab[blockIdx.x];
  const T* qj = a.Q + (long long)j * a.n;
  double s = 0.0;
  for (long long i = threadIdx.x; i < a.n; i += blockDim.x) s += re_dot<T>(qj[i], a.w[i]);
  const double al = block_sum<T>(s, red);
  const double bp = j > 0 ? a.beta[j - 1] : 0.0;
  const T* qm = j > 0 ? a.Q + (long long)(j - 1) * a.n : qj;
  for (long long i = threadIdx.x; i < a.n; i += blockDim.x) {
    T w = a.w[i];
    w = Sc<T>::sub(w, Sc<T>::scale(qj[i], al));
    if (j > 0) w = Sc<T>::sub(w, Sc<T>::scale(qm[i], bp));
    a.w[i] = w;
  }
  if (threadIdx.x == 0) a.alpha[j] = al;
}

// h_i = <q_i, w> for i < j; grid (j, nprob)
template <typename T>
__global__ void __launch_bounds__(kVecThreads) lz_multidot_kernel(const LSeg<T>* __restrict__ tab) {
  __shared__ double red[32];
  const LSeg<T> a = tab[blockIdx.y];
  const int i = blockIdx.x;
  const T* q = a.Q + (long long)i * a.n;
  double sr = 0.0, si = 0.0;
  for (long long e = threadIdx.x; e < a.n; e += blockDim.x) {
    const T c = Sc<T>::mul(Sc<T>::conj(q[e]), a.w[e]);
    sr += Sc<T>::re(c);
    si += Sc<T>::im(c);
  }
  sr = block_sum<T>(sr, red);
  si = block_sum<T>(si, red);
  if (threadIdx.x == 0) a.h[i] = Sc<T>::make(sr, si);
}

// w -= sum_{i<j} h_i q_i; grid (blocks, nprob)
template <typename T>
__global__ void lz_gemv_kernel(const LSeg<T>* __restrict__ tab, int j) {
  const LSeg<T> a = tab[blockIdx.y];
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < a.n; e += (long long)gridDim.x * blockDim.x) {
    T w = a.w[e];
    for (int i = 0; i < j; ++i) w = Sc<T>::sub(w, Sc<T>::mul(a.h[i], a.Q[(long long)i * a.n + e]));
    a.w[e] = w;
  }
}

// beta_j = |w|; q_{j+1} = w / beta_j into Q[j+1] and v (zero after a breakdown)
template <typename T>
__global__ void __launch_bounds__(kVecThreads) lz_beta_kernel(const LSeg<T>* __restrict__ tab, int j, double tol) {
  __shared__ double red[32];
  const LSeg<T> a = tab[blockIdx.x];
  double s = 0.0;
  for (long long i = threadIdx.x; i < a.n; i += blockDim.x) s += Sc<T>::abs2(a.w[i]);
  const double be = sqrt(block_sum<T>(s, red));
  const bool dead = *((volatile int*)a.dead) != 0 || !(be >= tol);
  const double inv = dead ? 0.0 : 1.0 / be;
  T* qn = a.Q + (long long)(j + 1) * a.n;
  for (long long i = threadIdx.x; i < a.n; i += blockDim.x) {
    const T q = Sc<T>::scale(a.w[i], inv);
    qn[i] = q;
    a.v[i] = q;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    a.beta[j] = be;
    if (dead) *a.dead = 1;
  }
}

// x = sum_{i<kused} y_i q_i over the kused rows every problem has computed
// (the host pads y with zeros past each problem's own dimension); grid
// (blocks, nprob)
template <typename T>
__global__ void lz_ritz_kernel(const LSeg<T>* __restrict__ tab, int kused) {
  const LSeg<T> a = tab[blockIdx.y];
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < a.n; e += (long long)gridDim.x * blockDim.x) {
    T s = Sc<T>::zero();
    for (int i = 0; i < kused; ++i) s = Sc<T>::fma(a.y[i], a.Q[(long long)i * a.n + e], s);
    a.x[e] = s;
  }
}


// ---------------------------------------------------------------- Lanczos driver
struct LzLayout {
  size_t total = 0;
  size_t seg_tab = 0, gemm_tab[4] = {0, 0, 0, 0}, alpha = 0, beta = 0, y = 0, dead = 0;
  std::vector<size_t> Q, w, v, h, P, Pq;
};

template <typename T>
bool lz_layout(int nprob, const dmrg_heff_t* ops, int kmax, LzLayout* L) {
  size_t off = 0;
  L->seg_tab = off; off += align_up(sizeof(LSeg<T>) * (size_t)nprob);
  for (int k = 0; k < 4; ++k) { L->gemm_tab[k] = off; off += align_up(tgemm_grouped_desc_bytes(nprob)); }
  L->alpha = off; off += align_up(sizeof(double) * (size_t)nprob * kmax);
  L->beta = off; off += align_up(sizeof(double) * (size_t)nprob * kmax);
  L->y = off; off += align_up(sizeof(T) * (size_t)nprob * kmax);
  L->dead = off; off += align_up(sizeof(int) * (size_t)nprob);
  L->Q.resize(nprob); L->w.resize(nprob); L->v.resize(nprob); L->h.resize(nprob); L->P.resize(nprob);
  L->Pq.resize(nprob);
  for (int p = 0; p < nprob; ++p) {
    const dmrg_heff_t& o = ops[p];
    if (o.kind != 2 || o.precision != DMRG_PREC_FP64 || o.chil < 1 || o.chir < 1 || o.d1 < 1 || o.d2 < 1 ||
        o.wl < 1 || o.wm < 1 || o.wr < 1 || !o.L || !o.R || !o.W1 || !o.W2)
      return false;
    const size_t n = (size_t)o.chil * o.d1 * o.d2 * o.chir;
    size_t P = 0, Q = 0;
    heff_fp64_elems<T>(o, &P, &Q);
    L->Q[p] = off; off += align_up(sizeof(T) * n * (size_t)(kmax + 1));
    L->w[p] = off; off += align_up(sizeof(T) * n);
    L->v[p] = off; off += align_up(sizeof(T) * n);
    L->h[p] = off; off += align_up(sizeof(T) * (size_t)(kmax + 1));
    L->P[p] = off; off += align_up(sizeof(T) * P);
    L->Pq[p] = off; off += align_up(sizeof(T) * (Q > 0 ? Q : 1));
  }
  L->total = off;
  return true;
}

struct GraphEntry {
  cudaGraphExec_t exec = nullptr;
  unsigned long long kernels = 0;
};
std::mutex g_graph_mu;
std::map<std::string, GraphEntry> g_graphs;
cudaStream_t g_capture_stream[64] = {};

int capture_stream(cudaStream_t* out) {
  int dev = 0;
  DMRG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return DMRG_ERR_UNSUPPORTED;
  if (!g_capture_stream[dev]) DMRG_CUDA_TRY(cudaStreamCreateWithFlags(&g_capture_stream[dev], cudaStreamNonBlocking));
  *out = g_capture_stream[dev];
  return DMRG_OK;
}

template <typename T>
struct LzPlan {
  const LSeg<T>* seg;
  const void* gtab[4];
  int gn[4];
  long long gtiles[4];
  int nprob;
  long long nmax;
  double tol;
};

// steps j0 .. j1-1 of the recurrence for every problem
template <typename T>
int lz_steps(const LzPlan<T>& pl, int j0, int j1, unsigned long long* kernels, cudaStream_t s) {
  long long gx = (pl.nmax + 255) / 256;
  if (gx > 64) gx = 64;
  unsigned long long before = dmrg_kernel_launches();
  for (int j = j0; j < j1; ++j) {
    for (int k = 0; k < 4; ++k)
      DMRG_TRY(tgemm_grouped_launch<T>(pl.gtab[k], pl.gn[k], pl.gtiles[k], Sc<T>::one(), Sc<T>::zero(), s));
    lz_alpha_axpy_kernel<T><<<pl.nprob, kVecThreads, 0, s>>>(pl.seg, j);
    DMRG_CHECK_LAUNCH();
    if (j > 0) {
      lz_multidot_kernel<T><<<dim3((unsigned)j, (unsigned)pl.nprob), kVecThreads, 0, s>>>(pl.seg);
      DMRG_CHECK_LAUNCH();
      lz_gemv_kernel<T><<<dim3((unsigned)gx, (unsigned)pl.nprob), 256, 0, s>>>(pl.seg, j);
      DMRG_CHECK_LAUNCH();
    }
    lz_beta_kernel<T><<<pl.nprob, kVecThreads, 0, s>>>(pl.seg, j, pl.tol);
    DMRG_CHECK_LAUNCH();
  }
  if (kernels) *kernels = dmrg_kernel_launches() - before;
  return DMRG_OK;
}

template <typename T>
int lz_block(const LzPlan<T>& pl, const std::string& key, int j0, int j1, bool use_graph, cudaStream_t s) {
  if (!use_graph) return lz_steps<T>(pl, j0, j1, nullptr, s);
  GraphEntry e;
  {
    std::lock_guard<std::mutex> lock(g_graph_mu);
    auto it = g_graphs.find(key);
    if (it != g_graphs.end()) e = it->second;
  }
  if (!e.exec) {
    cudaStream_t cs;
    DMRG_TRY(capture_stream(&cs));
    DMRG_CUDA_TRY(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    unsigned long long nk = 0;
    const int st = lz_steps<T>(pl, j0, j1, &nk, cs);
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(cs, &g);
    if (st != DMRG_OK) {
      if (g) cudaGraphDestroy(g);
      return st;
    }
    if (ce != cudaSuccess || !g) return DMRG_ERR_CUDA;
    cudaGraphExec_t ex = nullptr;
    const cudaError_t ie = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) return DMRG_ERR_CUDA;
    e.exec = ex;
    e.kernels = nk;
    uncount_launches(nk);  // captured launches execute on replay, counted there
    std::lock_guard<std::mutex> lock(g_graph_mu);
    if (g_graphs.size() > 4096) {
      for (auto& kv : g_graphs) cudaGraphExecDestroy(kv.second.exec);
      g_graphs.clear();
    }
    g_graphs[key] = e;
  }
  DMRG_CUDA_TRY(cudaGraphLaunch(e.exec, s));
  count_launches(e.kernels);
  return DMRG_OK;
}

template <typename T>
int batch_lanczos(int nprob, const dmrg_heff_t* ops, void* const* x, int kmax, double tol, int use_graph,
                  double* energies, int* iters, void* work, size_t work_bytes, cudaStream_t s) {
  LzLayout L;
  if (!lz_layout<T>(nprob, ops, kmax, &L)) return DMRG_ERR_ARG;
  if (L.total > work_bytes) return DMRG_ERR_WORKSPACE;
  char* base = static_cast<char*>(work);
  std::vector<LSeg<T>> seg(nprob);
  std::vector<long long> n(nprob);
  long long nmax = 1;
  std::vector<GStep> steps((size_t)nprob * 4);
  for (int p = 0; p < nprob; ++p) {
    const dmrg_heff_t& o = ops[p];
    n[p] = (long long)o.chil * o.d1 * o.d2 * o.chir;
    nmax = n[p] > nmax ? n[p] : nmax;
    LSeg<T>& a = seg[p];
    a.x = static_cast<T*>(x[p]);
    a.Q = reinterpret_cast<T*>(base + L.Q[p]);
    a.w = reinterpret_cast<T*>(base + L.w[p]);
    a.v = reinterpret_cast<T*>(base + L.v[p]);
    a.h = reinterpret_cast<T*>(base + L.h[p]);
    a.alpha = reinterpret_cast<double*>(base + L.alpha) + (size_t)p * kmax;
    a.beta = reinterpret_cast<double*>(base + L.beta) + (size_t)p * kmax;
    a.y = reinterpret_cast<const T*>(base + L.y) + (size_t)p * kmax;
    a.n = n[p];
    a.dead = reinterpret_cast<int*>(base + L.dead) + p;
    const int ns = heff_fp64_plan<T>(o, a.v, a.w, reinterpret_cast<T*>(base + L.P[p]),
                                     reinterpret_cast<T*>(base + L.Pq[p]), &steps[(size_t)p * 4]);
    if (ns != 4) return DMRG_ERR_ARG;
  }
  LzPlan<T> pl;
  pl.seg = reinterpret_cast<const LSeg<T>*>(base + L.seg_tab);
  pl.nprob = nprob;
  pl.nmax = nmax;
  pl.tol = tol;
  std::vector<char> hdesc(tgemm_grouped_desc_bytes(nprob));
  std::vector<TGemm> g(nprob);
  std::vector<const void*> A(nprob), B(nprob);
  std::vector<void*> C(nprob);
  std::string key = std::to_string((unsigned long long)(size_t)work) + ":" + std::to_string(nprob) + ":" +
                    std::to_string(kmax) + ":" + std::to_string(sizeof(T));
  for (int k = 0; k < 4; ++k) {
    for (int p = 0; p < nprob; ++p) {
      const GStep& st = steps[(size_t)p * 4 + k];
      g[p] = st.g;
      A[p] = st.A;
      B[p] = st.B;
      C[p] = st.C;
    }
    DMRG_TRY(tgemm_grouped_build(nprob, g.data(), A.data(), B.data(), C.data(), hdesc.data(), &pl.gn[k],
                                 &pl.gtiles[k]));
    DMRG_CUDA_TRY(cudaMemcpyAsync(base + L.gemm_tab[k], hdesc.data(), tgemm_grouped_desc_bytes(nprob),
                                  cudaMemcpyHostToDevice, s));
    pl.gtab[k] = base + L.gemm_tab[k];
    key += ":" + std::to_string(pl.gn[k]) + "/" + std::to_string(pl.gtiles[k]);
  }
  key += ":" + std::to_string(nmax);
  DMRG_CUDA_TRY(cudaMemcpyAsync(base + L.seg_tab, seg.data(), sizeof(LSeg<T>) * nprob, cudaMemcpyHostToDevice, s));
  lz_init_kernel<T><<<nprob, kVecThreads, 0, s>>>(pl.seg);
  DMRG_CHECK_LAUNCH();

  // host replay of the single-chain stop logic, per problem
  std::vector<int> done(nprob, 0), kfin(nprob, 1), last(nprob, -1);
  std::vector<double> prev(nprob, 0.0);
  std::vector<double> al((size_t)nprob * kmax), be((size_t)nprob * kmax);
  int j = 0;
  while (j < kmax) {
    const int j1 = j + kBlock < kmax ? j + kBlock : kmax;
    DMRG_TRY(lz_block<T>(pl, key + ":" + std::to_string(j) + "-" + std::to_string(j1), j, j1, use_graph != 0, s));
    DMRG_CUDA_TRY(cudaMemcpyAsync(al.data(), base + L.alpha, sizeof(double) * al.size(), cudaMemcpyDeviceToHost, s));
    DMRG_CUDA_TRY(cudaMemcpyAsync(be.data(), base + L.beta, sizeof(double) * be.size(), cudaMemcpyDeviceToHost, s));
    DMRG_CUDA_TRY(cudaStreamSynchronize(s));
    bool all = true;
    for (int p = 0; p < nprob; ++p) {
      if (done[p]) continue;
      const double* a = &al[(size_t)p * kmax];
      const double* b = &be[(size_t)p * kmax];
      const int jmax = (int)((n[p] < (long long)j1) ? n[p] : (long long)j1);
      for (int jj = last[p] + 1; jj < jmax && !done[p]; ++jj) {
        if (!(a[jj] == a[jj]) || !(b[jj] == b[jj])) return DMRG_ERR_NAN;
        if (jj == 0) {
          prev[p] = a[0];
          kfin[p] = 1;
        } else if (b[jj - 1] < tol) {
          done[p] = 1;
        } else {
          std::vector<double> av(a, a + jj + 1), bv(b, b + jj);
          double cur = 0.0;
          DMRG_TRY(lowest_ritz(av, bv, &cur, nullptr));
          kfin[p] = jj + 1;
          if (std::fabs(cur - prev[p]) < tol * std::max(1.0, std::fabs(cur))) done[p] = 1;
          prev[p] = cur;
        }
        last[p] = jj;
      }
      if (jmax >= n[p] || last[p] + 1 >= kmax) done[p] = 1;
      all = all && done[p];
    }
    j = j1;
    if (all) break;
  }
  // Ritz vectors
  std::vector<T> y((size_t)nprob * kmax, Sc<T>::zero());
  for (int p = 0; p < nprob; ++p) {
    const int k = kfin[p];
    std::vector<double> av(&al[(size_t)p * kmax], &al[(size_t)p * kmax] + k);
    std::vector<double> bv(&be[(size_t)p * kmax], &be[(size_t)p * kmax] + (k - 1));
    double ev = 0.0;
    std::vector<double> yv;
    DMRG_TRY(lowest_ritz(av, bv, &ev, &yv));
    for (int i = 0; i < k; ++i) y[(size_t)p * kmax + i] = Sc<T>::make(yv[i], 0.0);
    if (energies) energies[p] = ev;
    if (iters) iters[p] = k;
  }
  DMRG_CUDA_TRY(cudaMemcpyAsync(base + L.y, y.data(), sizeof(T) * y.size(), cudaMemcpyHostToDevice, s));
  long long gx = (nmax + 255) / 256;
  if (gx > 64) gx = 64;
  // rows 0..j of every problem hold q_0..q_j (zeros after a breakdown)
  const int kused = j + 1 < kmax ? j + 1 : kmax;
  lz_ritz_kernel<T><<<dim3((unsigned)gx, (unsigned)nprob), 256, 0, s>>>(pl.seg, kused);
  DMRG_CHECK_LAUNCH();
  DMRG_CUDA_TRY(cudaStreamSynchronize(s));
  return DMRG_OK;
}

}  // namespace
}  // namespace dmrg

// ---------------------------------------------------------------- grouped contractions
namespace dmrg {
namespace {

size_t env_scratch_bytes(int side, size_t es, int cl, int d, int cr, int wl, int wr) {
  return align_up(es * env_fp64_elems(side, cl, d, cr, wl, wr));
}

bool env_dims_ok(int nprob, const int* cl, const int* d, const int* cr, const int* wl, const int* wr) {
  if (nprob < 1 || !cl || !d || !cr || !wl || !wr) return false;
  for (int p = 0; p < nprob; ++p)
    if (cl[p] < 1 || d[p] < 1 || cr[p] < 1 || wl[p] < 1 || wr[p] < 1) return false;
  return true;
}

template <typename T>
int batch_env(int side, int nprob, const int* cl, const int* d, const int* cr, const int* wl, const int* wr,
              const void* const* E, const void* const* W, const void* const* A, void* const* Enew, void* work,
              cudaStream_t s) {
  char* base = static_cast<char*>(work);
  const size_t tab = tgemm_grouped_desc_bytes(nprob);
  char* scratch = base + 3 * tab;
  std::vector<GStep> steps((size_t)nprob * 3);
  for (int p = 0; p < nprob; ++p) {
    T* P = reinterpret_cast<T*>(scratch);
    scratch += env_scratch_bytes(side, sizeof(T), cl[p], d[p], cr[p], wl[p], wr[p]);
    const int ns = side == 0
        ? env_left_plan<T>(cl[p], d[p], cr[p], wl[p], wr[p], static_cast<const T*>(E[p]),
                           static_cast<const T*>(W[p]), static_cast<const T*>(A[p]), static_cast<T*>(Enew[p]), P,
                           &steps[(size_t)p * 3])
        : env_right_plan<T>(cl[p], d[p], cr[p], wl[p], wr[p], static_cast<const T*>(E[p]),
                            static_cast<const T*>(W[p]), static_cast<const T*>(A[p]), static_cast<T*>(Enew[p]), P,
                            &steps[(size_t)p * 3]);
    if (ns != 3) return DMRG_ERR_ARG;
  }
  std::vector<char> hdesc(tab);
  std::vector<TGemm> g(nprob);
  std::vector<const void*> a(nprob), b(nprob);
  std::vector<void*> c(nprob);
  for (int k = 0; k < 3; ++k) {
    for (int p = 0; p < nprob; ++p) {
      const GStep& st = steps[(size_t)p * 3 + k];
      g[p] = st.g; a[p] = st.A; b[p] = st.B; c[p] = st.C;
    }
    DMRG_TRY(tgemm_grouped<T>(nprob, g.data(), a.data(), b.data(), c.data(), Sc<T>::one(), Sc<T>::zero(),
                              base + (size_t)k * tab, hdesc.data(), s));
  }
  return DMRG_OK;
}

}  // namespace
}  // namespace dmrg

using namespace dmrg;

extern "C" {

size_t dmrg_batch_lanczos_workspace_bytes(int nprob, const dmrg_heff_t* ops, int niter) {
  if (nprob < 1 || !ops || niter < 1) return 0;
  LzLayout L;
  const bool ok = ops[0].dtype == DMRG_COMPLEX128 ? lz_layout<cplx>(nprob, ops, niter, &L)
                                                  : lz_layout<double>(nprob, ops, niter, &L);
  return ok ? L.total : 0;
}

int dmrg_batch_lanczos_ground(int nprob, const dmrg_heff_t* ops, void* const* x, int niter, double tol, int use_graph,
                              double* energies, int* iters, void* work, size_t work_bytes, void* stream) {
  if (nprob < 1 || nprob > 65535 || !ops || !x || niter < 1 || niter > 4096 || !work) return DMRG_ERR_ARG;
  const int dt = ops[0].dtype;
  for (int p = 0; p < nprob; ++p)
    if (ops[p].dtype != dt || !x[p]) return DMRG_ERR_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (dt == DMRG_COMPLEX128)
    return batch_lanczos<cplx>(nprob, ops, x, niter, tol, use_graph, energies, iters, work, work_bytes, s);
  if (dt != DMRG_REAL64) return DMRG_ERR_ARG;
  return batch_lanczos<double>(nprob, ops, x, niter, tol, use_graph, energies, iters, work, work_bytes, s);
}

size_t dmrg_batch_gemm_workspace_bytes(int nprob) { return nprob < 1 ? 0 : tgemm_grouped_desc_bytes(nprob); }

int dmrg_batch_gemm(int dtype, int nprob, const int* m, const int* k, const int* n, const void* const* A,
                    const void* const* B, void* const* C, void* work, size_t work_bytes, void* stream) {
  if (nprob < 1 || !m || !k || !n || !A || !B || !C || !work) return DMRG_ERR_ARG;
  if (tgemm_grouped_desc_bytes(nprob) > work_bytes) return DMRG_ERR_WORKSPACE;
  std::vector<TGemm> g(nprob);
  for (int p = 0; p < nprob; ++p) {
    if (m[p] < 1 || k[p] < 1 || n[p] < 1 || !A[p] || !B[p] || !C[p]) return DMRG_ERR_ARG;
    TGemm& t = g[p];
    t = TGemm{};
    t.B = ax(1); t.M = ax(m[p]); t.K = ax(k[p]); t.N = ax(n[p]);
    t.a_m = st(k[p]); t.a_k = st(1);
    t.b_k = st(n[p]); t.b_n = st(1);
    t.c_m = st(n[p]); t.c_n = st(1);
  }
  std::vector<char> hdesc(tgemm_grouped_desc_bytes(nprob));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (dtype == DMRG_COMPLEX128)
    return tgemm_grouped<cplx>(nprob, g.data(), A, B, C, Sc<cplx>::one(), Sc<cplx>::zero(), work, hdesc.data(), s);
  if (dtype != DMRG_REAL64) return DMRG_ERR_ARG;
  return tgemm_grouped<double>(nprob, g.data(), A, B, C, 1.0, 0.0, work, hdesc.data(), s);
}

size_t dmrg_batch_env_workspace_bytes(int side, int dtype, int nprob, const int* chil, const int* d, const int* chir,
                                      const int* wl, const int* wr) {
  if ((side != 0 && side != 1) || !env_dims_ok(nprob, chil, d, chir, wl, wr)) return 0;
  const size_t es = dtype == DMRG_COMPLEX128 ? 16 : 8;
  size_t tot = 3 * tgemm_grouped_desc_bytes(nprob);
  for (int p = 0; p < nprob; ++p) tot += env_scratch_bytes(side, es, chil[p], d[p], chir[p], wl[p], wr[p]);
  return tot;
}

int dmrg_batch_env_extend(int side, int dtype, int nprob, const int* chil, const int* d, const int* chir,
                          const int* wl, const int* wr, const void* const* E, const void* const* W,
                          const void* const* A, void* const* Enew, void* work, size_t work_bytes, void* stream) {
  if ((side != 0 && side != 1) || !env_dims_ok(nprob, chil, d, chir, wl, wr) || !E || !W || !A || !Enew || !work)
    return DMRG_ERR_ARG;
  if (dmrg_batch_env_workspace_bytes(side, dtype, nprob, chil, d, chir, wl, wr) > work_bytes)
    return DMRG_ERR_WORKSPACE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (dtype == DMRG_COMPLEX128) return batch_env<cplx>(side, nprob, chil, d, chir, wl, wr, E, W, A, Enew, work, s);
  if (dtype != DMRG_REAL64) return DMRG_ERR_ARG;
  return batch_env<double>(side, nprob, chil, d, chir, wl, wr, E, W, A, Enew, work, s);
}

size_t dmrg_batch_svd_workspace_bytes(int dtype, int nprob, const int* m, const int* n) {
  if (nprob < 1 || !m || !n) return 0;
  for (int p = 0; p < nprob; ++p)
    if (m[p] < 1 || n[p] < 1) return 0;
  return svd_batch_work_bytes(dtype, nprob, m, n);
}

int dmrg_batch_svd_factor(int dtype, int nprob, const int* m, const int* n, const void* const* M, double cutoff,
                          const int* maxdim, int mindim, int absorb, int* keep, double* discarded, double* svals,
                          int ld_svals, void* work, size_t work_bytes, void* stream) {
  if (nprob < 1 || nprob > 65535 || !m || !n || !M || !maxdim || !keep || !work || (absorb < 0 || absorb > 2))
    return DMRG_ERR_ARG;
  int cmax = 1;
  for (int p = 0; p < nprob; ++p) {
    if (m[p] < 1 || n[p] < 1 || !M[p]) return DMRG_ERR_ARG;
    const int c = m[p] < n[p] ? m[p] : n[p];
    cmax = c > cmax ? c : cmax;
  }
  if (svals && ld_svals < cmax) return DMRG_ERR_ARG;
  if (svd_batch_work_bytes(dtype, nprob, m, n) > work_bytes) return DMRG_ERR_WORKSPACE;
  std::vector<double> sv((size_t)nprob * cmax, 0.0);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int st;
  if (dtype == DMRG_COMPLEX128)
    st = hestenes_batch_factor<cplx>(nprob, m, n, reinterpret_cast<const cplx* const*>(M), work, sv.data(), cmax,
                                     absorb, s);
  else if (dtype == DMRG_REAL64)
    st = hestenes_batch_factor<double>(nprob, m, n, reinterpret_cast<const double* const*>(M), work, sv.data(), cmax,
                                       absorb, s);
  else
    return DMRG_ERR_ARG;
  if (st != DMRG_OK && st != DMRG_ERR_NOCONV) return st;
  for (int p = 0; p < nprob; ++p) {
    const int c = m[p] < n[p] ? m[p] : n[p];
    int kp = 1;
    double dc = 0.0;
    keep_rule(&sv[(size_t)p * cmax], c, cutoff, maxdim[p], mindim > 1 ? mindim : 1, &kp, &dc);
    keep[p] = kp > c ? c : kp;
    if (discarded) discarded[p] = dc;
    if (svals) std::memcpy(svals + (size_t)p * ld_svals, &sv[(size_t)p * cmax], sizeof(double) * c);
  }
  return st;
}

int dmrg_batch_svd_output(int dtype, int nprob, const int* m, const int* n, const int* keep, int absorb,
                          void* const* left, void* const* right, void* work, size_t work_bytes, void* stream) {
  if (nprob < 1 || nprob > 65535 || !m || !n || !keep || !left || !right || !work || (absorb < 0 || absorb > 2))
    return DMRG_ERR_ARG;
  for (int p = 0; p < nprob; ++p) {
    const int c = m[p] < n[p] ? m[p] : n[p];
    if (m[p] < 1 || n[p] < 1 || keep[p] < 1 || keep[p] > c || !left[p] || !right[p]) return DMRG_ERR_ARG;
  }
  if (svd_batch_work_bytes(dtype, nprob, m, n) > work_bytes) return DMRG_ERR_WORKSPACE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (dtype == DMRG_COMPLEX128)
    return hestenes_batch_output<cplx>(nprob, m, n, keep, absorb, work, reinterpret_cast<cplx* const*>(left),
                                       reinterpret_cast<cplx* const*>(right), s);
  if (dtype != DMRG_REAL64) return DMRG_ERR_ARG;
  return hestenes_batch_output<double>(nprob, m, n, keep, absorb, work, reinterpret_cast<double* const*>(left),
                                       reinterpret_cast<double* const*>(right), s);
}

}  // extern "C"
