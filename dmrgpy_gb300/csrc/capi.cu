// extern "C" entry points (include/dmrg_gb300.h) and the host-side drivers
// of the Krylov loops.  Vectors, Krylov bases and every reduction stay on the
// device; per iteration only the two Lanczos scalars (alpha, beta) cross to
// the host, where the k x k tridiagonal problem is solved (k <= niter).
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#include "heff.cuh"
#include "tf32x3.cuh"

#include <atomic>

namespace dmrg {

static std::atomic<unsigned long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void count_launches(unsigned long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
void uncount_launches(unsigned long long n) { g_launches.fetch_sub(n, std::memory_order_relaxed); }

namespace {

inline size_t esize(int dtype) { return dtype == DMRG_COMPLEX128 ? 16 : 8; }

bool heff_valid(const dmrg_heff_t* o) {
  if (!o) return false;
  if (o->dtype != DMRG_REAL64 && o->dtype != DMRG_COMPLEX128) return false;
  if (o->precision != DMRG_PREC_FP64 && o->precision != DMRG_PREC_TF32X3) return false;
  if (o->chil <= 0 || o->chir <= 0 || o->wl <= 0 || o->wr <= 0) return false;
  if (!o->L || !o->R) return false;
  if (o->kind == 2) return o->d1 > 0 && o->d2 > 0 && o->wm > 0 && o->W1 && o->W2;
  if (o->kind == 1) return o->d1 > 0 && o->W1;
  if (o->kind == 0) return o->wl == o->wr;
  return false;
}

long long heff_n(const dmrg_heff_t* o) {
  long long n = (long long)o->chil * o->chir;
  if (o->kind >= 1) n *= o->d1;
  if (o->kind == 2) n *= o->d2;
  return n;
}

// ---- workspace of one H_eff application
size_t heff_ws(const dmrg_heff_t* o) {
  if (o->precision == DMRG_PREC_TF32X3) return tf32x3_heff_workspace_bytes(*o);
  size_t P, Q;
  if (o->dtype == DMRG_COMPLEX128) heff_fp64_elems<cplx>(*o, &P, &Q);
  else heff_fp64_elems<double>(*o, &P, &Q);
  return align_up(P * esize(o->dtype)) + align_up(Q * esize(o->dtype));
}

// One-off preparation of an operator (split-TF32: operand splitting of L, R
// and the two-site MPO), then heff_run per Krylov iteration.
template <typename T>
int heff_prepare(const dmrg_heff_t* o, void* work, cudaStream_t s) {
  if (o->precision != DMRG_PREC_TF32X3) return DMRG_OK;
  if (o->dtype != DMRG_REAL64) return DMRG_ERR_UNSUPPORTED;
  return tf32x3_heff_prepare(*o, work, s);
}

template <typename T>
int heff_finish(const dmrg_heff_t* o, void* work, cudaStream_t s) {
  if (o->precision != DMRG_PREC_TF32X3) return DMRG_OK;
  return tf32x3_heff_status(*o, work, s);
}

template <typename T>
int heff_run(const dmrg_heff_t* o, const T* x, T* y, void* work, cudaStream_t s) {
  if (o->precision == DMRG_PREC_TF32X3) {
    if (o->dtype != DMRG_REAL64) return DMRG_ERR_UNSUPPORTED;
    return tf32x3_heff_apply_prepared(*o, reinterpret_cast<const double*>(x), reinterpret_cast<double*>(y), work, s);
  }
  size_t P, Q;
  heff_fp64_elems<T>(*o, &P, &Q);
  T* Pp = static_cast<T*>(work);
  T* Qp = reinterpret_cast<T*>(static_cast<char*>(work) + align_up(P * sizeof(T)));
  return heff_apply_fp64<T>(*o, x, y, Pp, Qp, s);
}

}  // namespace

// ---- symmetric tridiagonal eigenproblem (implicit QL with Wilkinson-type
// shifts, Golub & Van Loan sec. 8.3 / the EISPACK tql2 scheme).  d: diagonal
// (overwritten by eigenvalues), e: off-diagonal e[0..n-2]; z (n x n,
// z[i*n + j] = component i of eigenvector j) if wantz.
bool tridiag_eig(int n, std::vector<double>& d, std::vector<double> e, std::vector<double>* z) {
  e.resize(n, 0.0);
  if (n > 0) e[n - 1] = 0.0;
  if (z) {
    z->assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) (*z)[(size_t)i * n + i] = 1.0;
  }
  const double eps = 2.220446049250313e-16;
  for (int l = 0; l < n; ++l) {
    int iter = 0;
    int m;
    do {
      for (m = l; m < n - 1; ++m) {
        double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
        if (std::fabs(e[m]) <= eps * dd) break;
      }
      if (m != l) {
        if (iter++ == 100) return false;
        double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
        double r = std::hypot(g, 1.0);
        g = d[m] - d[l] + e[l] / (g + std::copysign(r, g));
        double s = 1.0, c = 1.0, p = 0.0;
        int i;
        bool deflated = false;
        for (i = m - 1; i >= l; --i) {
          double f = s * e[i];
          double b = c * e[i];
          r = std::hypot(f, g);
          e[i + 1] = r;
          if (r == 0.0) {
            d[i + 1] -= p;
            e[m] = 0.0;
            deflated = true;
            break;
          }
          s = f / r;
          c = g / r;
          g = d[i + 1] - p;
          r = (d[i] - g) * s + 2.0 * c * b;
          p = s * r;
          d[i + 1] = g + p;
          g = c * r - b;
          if (z) {
            for (int k = 0; k < n; ++k) {
              double* zk = &(*z)[(size_t)k * n];
              f = zk[i + 1];
              zk[i + 1] = s * zk[i] + c * f;
              zk[i] = c * zk[i] - s * f;
            }
          }
        }
        if (deflated) continue;
        d[l] -= p;
        e[l] = g;
        e[m] = 0.0;
      }
    } while (m != l);
  }
  return true;
}

int lowest_ritz(const std::vector<double>& al, const std::vector<double>& be, double* ev, std::vector<double>* vec) {
  const int k = (int)al.size();
  std::vector<double> d(al), e(be);
  std::vector<double> z;
  if (!tridiag_eig(k, d, e, vec ? &z : nullptr)) return DMRG_ERR_NOCONV;
  int imin = 0;
  for (int i = 1; i < k; ++i)
    if (d[i] < d[imin]) imin = i;
  *ev = d[imin];
  if (vec) {
    vec->resize(k);
    for (int i = 0; i < k; ++i) (*vec)[i] = z[(size_t)i * k + imin];
  }
  return DMRG_OK;
}

namespace {


// ---- workspace layout of the Krylov drivers
struct KrylovWs {
  void* Q;        // kcap x n
  void* w;        // n
  void* hdev;     // kcap (T)
  double* sc;     // scalars: [0] alpha (T: 2 doubles) [2] beta [3] beta_prev [4] norm
  double* part;   // multidot partials 2 * MULTIDOT_MAX_GRID * kcap
  double* red;    // reduction scratch: 8 + 2*RB
  void* hw;       // heff workspace
};

size_t krylov_ws(const dmrg_heff_t* o, int kcap, KrylovWs* out, void* base) {
  const size_t es = esize(o->dtype);
  const size_t n = (size_t)heff_n(o);
  char* p = static_cast<char*>(base);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    void* q = p ? p + off : nullptr;
    off += align_up(bytes);
    return q;
  };
  KrylovWs w;
  w.Q = take((size_t)kcap * n * es);
  w.w = take(n * es);
  w.hdev = take((size_t)kcap * es);
  w.sc = static_cast<double*>(take(16 * sizeof(double)));
  w.part = static_cast<double*>(take(2 * (size_t)MULTIDOT_MAX_GRID * kcap * sizeof(double)));
  w.red = static_cast<double*>(take((8 + 2 * 2 * 152) * sizeof(double)));
  w.hw = take(heff_ws(o));
  if (out) *out = w;
  return off;
}

template <typename T>
int copy_scalar_to_host(const void* dev, double* host, int count, cudaStream_t s) {
  DMRG_CUDA_TRY(cudaMemcpyAsync(host, dev, sizeof(double) * count, cudaMemcpyDeviceToHost, s));
  return DMRG_OK;
}

template <typename T>
int lanczos_impl(const dmrg_heff_t* o, T* x, int niter, double tol, double* energy, int* iters, void* work,
                 size_t work_bytes, cudaStream_t s) {
  const long long n = heff_n(o);
  const int m = (int)std::min<long long>(niter, n);
  if (m < 1) return DMRG_ERR_ARG;
  KrylovWs ws;
  size_t need = krylov_ws(o, m, &ws, work);
  if (need > work_bytes) return DMRG_ERR_WORKSPACE;
  T* Q = static_cast<T*>(ws.Q);
  T* w = static_cast<T*>(ws.w);
  T* h = static_cast<T*>(ws.hdev);
  double* alpha_d = ws.sc + 0;  // T-sized (2 doubles)
  double* beta_d = ws.sc + 2;
  double* bprev_d = ws.sc + 4;
  double* nrm_d = ws.sc + 6;
  DMRG_CUDA_TRY(cudaMemsetAsync(ws.red, 0, 64, s));
  DMRG_CUDA_TRY(cudaMemsetAsync(ws.sc, 0, 16 * sizeof(double), s));

  double hbuf[4];
  DMRG_TRY(vnorm<T>(x, n, nrm_d, ws.red, s));
  DMRG_CUDA_TRY(cudaMemcpyAsync(hbuf, nrm_d, sizeof(double), cudaMemcpyDeviceToHost, s));
  DMRG_CUDA_TRY(cudaStreamSynchronize(s));
  if (!(hbuf[0] == hbuf[0])) return DMRG_ERR_NAN;
  if (hbuf[0] == 0.0) {
    DMRG_TRY(vfill_random<T>(x, n, 0x5eedULL, s));
    DMRG_TRY(vnorm<T>(x, n, nrm_d, ws.red, s));
  }
  DMRG_TRY(vscale_dev_inv<T>(Q, x, nrm_d, n, s));  // q0
  DMRG_TRY(heff_prepare<T>(o, ws.hw, s));
  DMRG_TRY(heff_run<T>(o, Q, w, ws.hw, s));
  DMRG_TRY(vdot<T>(Q, w, n, reinterpret_cast<T*>(alpha_d), ws.red, s));
  DMRG_TRY(vaxpy2<T>(w, Q, alpha_d, nullptr, nullptr, n, s));
  DMRG_TRY(vnorm<T>(w, n, beta_d, ws.red, s));
  DMRG_CUDA_TRY(cudaMemcpyAsync(hbuf, ws.sc, 4 * sizeof(double), cudaMemcpyDeviceToHost, s));
  DMRG_CUDA_TRY(cudaStreamSynchronize(s));
  std::vector<double> al{hbuf[0]}, be;
  double beta = hbuf[2];
  if (!(hbuf[0] == hbuf[0]) || !(beta == beta)) return DMRG_ERR_NAN;
  double prev = al[0];
  int k = 1;
  for (int j = 1; j < m; ++j) {
    if (beta < tol) break;
    be.push_back(beta);
    T* qj = Q + (long long)j * n;
    T* qjm = Q + (long long)(j - 1) * n;
    DMRG_TRY(vscale_dev_inv<T>(qj, w, beta_d, n, s));
    DMRG_CUDA_TRY(cudaMemcpyAsync(bprev_d, beta_d, sizeof(double), cudaMemcpyDeviceToDevice, s));
    DMRG_TRY(heff_run<T>(o, qj, w, ws.hw, s));
    DMRG_TRY(vdot<T>(qj, w, n, reinterpret_cast<T*>(alpha_d), ws.red, s));
    DMRG_TRY(vaxpy2<T>(w, qj, alpha_d, qjm, bprev_d, n, s));
    // full reorthogonalisation against q_0 .. q_{j-1}
    DMRG_TRY(multidot_ws<T>(Q, n, j, w, n, h, ws.part, s));
    DMRG_TRY(gemv_sub<T>(Q, n, j, h, w, n, 0, s));
    DMRG_TRY(vnorm<T>(w, n, beta_d, ws.red, s));
    DMRG_CUDA_TRY(cudaMemcpyAsync(hbuf, ws.sc, 4 * sizeof(double), cudaMemcpyDeviceToHost, s));
    DMRG_CUDA_TRY(cudaStreamSynchronize(s));
    if (!(hbuf[0] == hbuf[0]) || !(hbuf[2] == hbuf[2])) return DMRG_ERR_NAN;
    al.push_back(hbuf[0]);
    beta = hbuf[2];
    k = j + 1;
    double cur;
    DMRG_TRY(lowest_ritz(al, be, &cur, nullptr));
    if (std::fabs(cur - prev) < tol * std::max(1.0, std::fabs(cur))) break;
    prev = cur;
  }
  double ev;
  std::vector<double> y;
  DMRG_TRY(lowest_ritz(al, be, &ev, &y));
  std::vector<T> yt(k);
  for (int i = 0; i < k; ++i) yt[i] = Sc<T>::make(y[i], 0.0);
  DMRG_CUDA_TRY(cudaMemcpyAsync(h, yt.data(), sizeof(T) * k, cudaMemcpyHostToDevice, s));
  DMRG_TRY(gemv_sub<T>(Q, n, k, h, x, n, 1, s));
  DMRG_CUDA_TRY(cudaStreamSynchronize(s));
  DMRG_TRY(heff_finish<T>(o, ws.hw, s));
  if (energy) *energy = ev;
  if (iters) *iters = k;
  return DMRG_OK;
}

template <typename T>
int expm_impl(const dmrg_heff_t* o, T* x, std::complex<double> coeff, int niter, double tol, double errgoal,
              int* iters, void* work, size_t work_bytes, cudaStream_t s) {
  const long long n = heff_n(o);
  const int m = (int)std::min<long long>(niter, n);
  if (m < 1) return DMRG_ERR_ARG;
  if (sizeof(T) == 8 && coeff.imag() != 0.0) return DMRG_ERR_UNSUPPORTED;
  KrylovWs ws;
  size_t need = krylov_ws(o, m, &ws, work);
  if (need > work_bytes) return DMRG_ERR_WORKSPACE;
  T* Q = static_cast<T*>(ws.Q);
  T* w = static_cast<T*>(ws.w);
  T* h = static_cast<T*>(ws.hdev);
  double* alpha_d = ws.sc + 0;
  double* beta_d = ws.sc + 2;
  double* bprev_d = ws.sc + 4;
  double* nrm_d = ws.sc + 6;
  DMRG_CUDA_TRY(cudaMemsetAsync(ws.red, 0, 64, s));
  DMRG_CUDA_TRY(cudaMemsetAsync(ws.sc, 0, 16 * sizeof(double), s));
  double hbuf[4];
  DMRG_TRY(vnorm<T>(x, n, nrm_d, ws.red, s));
  DMRG_CUDA_TRY(cudaMemcpyAsync(hbuf, nrm_d, sizeof(double), cudaMemcpyDeviceToHost, s));
  DMRG_CUDA_TRY(cudaStreamSynchronize(s));
  const double beta0 = hbuf[0];
  if (!(beta0 == beta0)) return DMRG_ERR_NAN;
  if (beta0 == 0.0) {
    if (iters) *iters = 0;
    return DMRG_OK;
  }
  DMRG_TRY(vscale_dev_inv<T>(Q, x, nrm_d, n, s));
  DMRG_TRY(heff_prepare<T>(o, ws.hw, s));
  std::vector<double> al, be;
  for (int it = 0; it < m; ++it) {
    T* qi = Q + (long long)it * n;
    DMRG_TRY(heff_run<T>(o, qi, w, ws.hw, s));
    DMRG_TRY(vdot<T>(qi, w, n, reinterpret_cast<T*>(alpha_d), ws.red, s));
    DMRG_TRY(vaxpy2<T>(w, qi, alpha_d, it > 0 ? Q + (long long)(it - 1) * n : nullptr, it > 0 ? bprev_d : nullptr,
                       n, s));
    DMRG_TRY(multidot_ws<T>(Q, n, it + 1, w, n, h, ws.part, s));
    DMRG_TRY(gemv_sub<T>(Q, n, it + 1, h, w, n, 0, s));
    DMRG_TRY(vnorm<T>(w, n, beta_d, ws.red, s));
    DMRG_CUDA_TRY(cudaMemcpyAsync(hbuf, ws.sc, 4 * sizeof(double), cudaMemcpyDeviceToHost, s));
    DMRG_CUDA_TRY(cudaStreamSynchronize(s));
    if (!(hbuf[0] == hbuf[0]) || !(hbuf[2] == hbuf[2])) return DMRG_ERR_NAN;
    al.push_back(hbuf[0]);
    const double beta = hbuf[2];
    const int k = it + 1;
    // first column of exp(coeff T_k)
    std::vector<std::complex<double>> c(k);
    if (k == 1) {
      c[0] = std::exp(coeff * al[0]);
    } else {
      std::vector<double> d(al), z;
      std::vector<double> e(be.begin(), be.begin() + (k - 1));
      if (!tridiag_eig(k, d, e, &z)) return DMRG_ERR_NOCONV;
      for (int i = 0; i < k; ++i) {
        std::complex<double> acc = 0.0;
        for (int j = 0; j < k; ++j) acc += z[(size_t)i * k + j] * std::exp(coeff * d[j]) * z[(size_t)0 * k + j];
        c[i] = acc;
      }
    }
    if (beta < tol || it == m - 1 || beta0 * beta * std::abs(c[k - 1]) < errgoal) {
      std::vector<T> ct(k);
      for (int i = 0; i < k; ++i) ct[i] = Sc<T>::make(beta0 * c[i].real(), beta0 * c[i].imag());
      DMRG_CUDA_TRY(cudaMemcpyAsync(h, ct.data(), sizeof(T) * k, cudaMemcpyHostToDevice, s));
      DMRG_TRY(gemv_sub<T>(Q, n, k, h, x, n, 1, s));
      DMRG_CUDA_TRY(cudaStreamSynchronize(s));
      DMRG_TRY(heff_finish<T>(o, ws.hw, s));
      if (iters) *iters = k;
      return DMRG_OK;
    }
    be.push_back(beta);
    DMRG_CUDA_TRY(cudaMemcpyAsync(bprev_d, beta_d, sizeof(double), cudaMemcpyDeviceToDevice, s));
    DMRG_TRY(vscale_dev_inv<T>(Q + (long long)(it + 1) * n, w, beta_d, n, s));
  }
  return DMRG_ERR_ARG;  // unreachable: the it == m-1 branch returns
}

}  // namespace

// cutoff/maxdim/mindim rule of pyitensor/svd.py:32-68 on descending s
void keep_rule(const double* s, int n, double cutoff, int maxdim, int mindim, int* keep, double* disc) {
  std::vector<double> p(n);
  double total = 0.0;
  for (int i = 0; i < n; ++i) {
    p[i] = s[i] * s[i];
    total += p[i];
  }
  if (!(total > 0.0)) {
    *keep = std::max(1, mindim);
    *disc = 0.0;
    return;
  }
  for (int i = 0; i < n; ++i) p[i] /= total;
  const int hi = maxdim > 0 ? std::min(maxdim, n) : n;
  const int j_upper = std::max(0, n - mindim);
  const int j_forced = std::min(std::max(0, n - hi), j_upper);
  int j;
  if (j_upper <= j_forced) {
    j = j_forced;
  } else {
    // ascending tail sums beyond the forced drops
    double forced = 0.0;
    for (int t = 0; t < j_forced; ++t) forced += p[n - 1 - t];
    int best = -1;
    double run = 0.0;
    if (forced + 0.0 <= cutoff) best = 0;
    for (int t = 1; t <= j_upper - j_forced; ++t) {
      run += p[n - 1 - (j_forced + t - 1)];
      if (forced + run <= cutoff) best = t;
    }
    j = j_forced + (best >= 0 ? best : 0);
  }
  *keep = n - j;
  double d = 0.0;
  for (int i = *keep; i < n; ++i) d += p[i];
  *disc = d;
}

namespace {

// Real matrices with min(m, n) >= 16 take the Gram-matrix route of
// pyitensor/svd.py:108-151 (gramtrunc.cu) when the Gram matrix of the kept
// side is at most twice the smaller side and at most 4096; everything else
// (the reference's exact-SVD cases, complex matrices, strongly rectangular
// shapes) the one-sided Jacobi SVD.
bool gram_route(int dtype, int m, int n, int absorb) {
  if (dtype != DMRG_REAL64) return false;
  const int c = std::min(m, n);
  if (c < 16) return false;
  const int ck = absorb == 0 ? m : absorb == 1 ? n : c;
  return ck <= 2 * c && ck <= 4096;
}

size_t svd_total_bytes(int dtype, int m, int n, int absorb) {
  size_t b = svd_work_bytes(dtype, m, n);
  if (gram_route(dtype, m, n, absorb)) b = std::max(b, gram_truncate_workspace_bytes(m, n, absorb));
  return b;
}

template <typename T>
int svd_impl(int m, int n, const T* M, double cutoff, int maxdim, int mindim, int absorb, T* lo, T* ro, double* svals,
             int* keep, double* disc, void* work, size_t work_bytes, cudaStream_t s) {
  const int dtype = sizeof(T) == 16 ? DMRG_COMPLEX128 : DMRG_REAL64;
  if (svd_total_bytes(dtype, m, n, absorb) > work_bytes) return DMRG_ERR_WORKSPACE;
  if (gram_route(dtype, m, n, absorb)) {
    const int st = gram_truncate(m, n, reinterpret_cast<const double*>(M), cutoff, maxdim, mindim, absorb,
                                 reinterpret_cast<double*>(lo), reinterpret_cast<double*>(ro), svals, keep, disc,
                                 nullptr, work, work_bytes, s);
    if (st != GRAM_FALLBACK) return st;
  }
  const int c = std::min(m, n);
  std::vector<double> sv(c);
  int sweeps = 0;
  const int left = svd_orientation_left(m, n, absorb);
  int st = hestenes_factor<T>(M, m, n, left, work, sv.data(), &sweeps, svd_abs_floor(left, absorb), s);
  if (st != DMRG_OK && st != DMRG_ERR_NOCONV) return st;
  int kp;
  double dc;
  keep_rule(sv.data(), c, cutoff, maxdim, std::max(1, mindim), &kp, &dc);
  if (kp > c) kp = c;
  DMRG_TRY(hestenes_output<T>(m, n, left, kp, absorb, work, lo, ro, s));
  if (svals) std::memcpy(svals, sv.data(), sizeof(double) * c);
  if (keep) *keep = kp;
  if (disc) *disc = dc;
  return st;
}

}  // namespace
}  // namespace dmrg

using namespace dmrg;

extern "C" {

int dmrg_version(void) { return 100; }

unsigned long long dmrg_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

const char* dmrg_status_string(int status) {
  switch (status) {
    case DMRG_OK: return "ok";
    case DMRG_ERR_ARG: return "invalid argument";
    case DMRG_ERR_WORKSPACE: return "workspace too small";
    case DMRG_ERR_CUDA: return "CUDA error";
    case DMRG_ERR_NAN: return "non-finite value";
    case DMRG_ERR_NOCONV: return "iterative solver did not converge";
    case DMRG_ERR_TIMEOUT: return "bounded device wait timed out";
    case DMRG_ERR_UNSUPPORTED: return "unsupported combination";
    case DMRG_ERR_PRECISION: return "split-TF32 weights cannot resolve the cutoff; use the FP64 route";
    default: return "unknown status";
  }
}

size_t dmrg_heff_workspace_bytes(const dmrg_heff_t* op) {
  if (!heff_valid(op)) return 0;
  return heff_ws(op);
}

int dmrg_heff_apply(const dmrg_heff_t* op, const void* x, void* y, void* work, size_t work_bytes, void* stream) {
  if (!heff_valid(op) || !x || !y || x == y) return DMRG_ERR_ARG;
  if (heff_ws(op) > work_bytes || (!work && heff_ws(op) > 0)) return DMRG_ERR_WORKSPACE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (op->dtype == DMRG_COMPLEX128) return heff_run<cplx>(op, static_cast<const cplx*>(x), static_cast<cplx*>(y), work, s);
  DMRG_TRY(heff_prepare<double>(op, work, s));
  DMRG_TRY(heff_run<double>(op, static_cast<const double*>(x), static_cast<double*>(y), work, s));
  return heff_finish<double>(op, work, s);
}

int dmrg_heff_prepare(const dmrg_heff_t* op, void* work, size_t work_bytes, void* stream) {
  if (!heff_valid(op)) return DMRG_ERR_ARG;
  if (heff_ws(op) > work_bytes || (!work && heff_ws(op) > 0)) return DMRG_ERR_WORKSPACE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (op->dtype == DMRG_COMPLEX128) return heff_prepare<cplx>(op, work, s);
  return heff_prepare<double>(op, work, s);
}

int dmrg_heff_apply_prepared(const dmrg_heff_t* op, const void* x, void* y, void* work, size_t work_bytes,
                             void* stream) {
  if (!heff_valid(op) || !x || !y || x == y) return DMRG_ERR_ARG;
  if (heff_ws(op) > work_bytes || (!work && heff_ws(op) > 0)) return DMRG_ERR_WORKSPACE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (op->dtype == DMRG_COMPLEX128) return heff_run<cplx>(op, static_cast<const cplx*>(x), static_cast<cplx*>(y), work, s);
  return heff_run<double>(op, static_cast<const double*>(x), static_cast<double*>(y), work, s);
}

int dmrg_heff_status(const dmrg_heff_t* op, void* work, size_t work_bytes, void* stream) {
  if (!heff_valid(op)) return DMRG_ERR_ARG;
  if (heff_ws(op) > work_bytes) return DMRG_ERR_WORKSPACE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  DMRG_CUDA_TRY(cudaStreamSynchronize(s));
  return heff_finish<double>(op, work, s);
}

size_t dmrg_env_workspace_bytes(int dtype, int precision, int chil, int d, int chir, int wl, int wr) {
  if (precision == DMRG_PREC_TF32X3) return tf32x3_env_workspace_bytes(chil, d, chir, wl, wr);
  size_t a = env_fp64_elems(0, chil, d, chir, wl, wr), b = env_fp64_elems(1, chil, d, chir, wl, wr);
  return align_up((a > b ? a : b) * esize(dtype));
}

static int env_common(int side, int dtype, int precision, int chil, int d, int chir, int wl, int wr, const void* E,
                      const void* W, const void* A, void* Enew, void* work, size_t work_bytes, void* stream) {
  if ((dtype != DMRG_REAL64 && dtype != DMRG_COMPLEX128) || chil <= 0 || chir <= 0 || d <= 0 || wl <= 0 || wr <= 0)
    return DMRG_ERR_ARG;
  if (!E || !W || !A || !Enew) return DMRG_ERR_ARG;
  if (dmrg_env_workspace_bytes(dtype, precision, chil, d, chir, wl, wr) > work_bytes) return DMRG_ERR_WORKSPACE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (precision == DMRG_PREC_TF32X3) {
    if (dtype != DMRG_REAL64) return DMRG_ERR_UNSUPPORTED;
    return tf32x3_env(side, chil, d, chir, wl, wr, static_cast<const double*>(E), static_cast<const double*>(W),
                      static_cast<const double*>(A), static_cast<double*>(Enew), work, s);
  }
  if (dtype == DMRG_COMPLEX128) {
    if (side == 0)
      return env_left_fp64<cplx>(chil, d, chir, wl, wr, (const cplx*)E, (const cplx*)W, (const cplx*)A, (cplx*)Enew,
                                 (cplx*)work, s);
    return env_right_fp64<cplx>(chil, d, chir, wl, wr, (const cplx*)E, (const cplx*)W, (const cplx*)A, (cplx*)Enew,
                                (cplx*)work, s);
  }
  if (side == 0)
    return env_left_fp64<double>(chil, d, chir, wl, wr, (const double*)E, (const double*)W, (const double*)A,
                                 (double*)Enew, (double*)work, s);
  return env_right_fp64<double>(chil, d, chir, wl, wr, (const double*)E, (const double*)W, (const double*)A,
                                (double*)Enew, (double*)work, s);
}

int dmrg_env_extend_left(int dtype, int precision, int chil, int d, int chir, int wl, int wr, const void* L,
                         const void* W, const void* A, void* Lnew, void* work, size_t work_bytes, void* stream) {
  return env_common(0, dtype, precision, chil, d, chir, wl, wr, L, W, A, Lnew, work, work_bytes, stream);
}

int dmrg_env_extend_right(int dtype, int precision, int chil, int d, int chir, int wl, int wr, const void* R,
                          const void* W, const void* B, void* Rnew, void* work, size_t work_bytes, void* stream) {
  return env_common(1, dtype, precision, chil, d, chir, wl, wr, R, W, B, Rnew, work, work_bytes, stream);
}

size_t dmrg_lanczos_workspace_bytes(const dmrg_heff_t* op, int niter) {
  if (!heff_valid(op) || niter < 1) return 0;
  int kcap = (int)std::min<long long>(niter, heff_n(op));
  return krylov_ws(op, kcap, nullptr, nullptr);
}

int dmrg_lanczos_ground(const dmrg_heff_t* op, void* x, int niter, double tol, double* energy, int* iters, void* work,
                        size_t work_bytes, void* stream) {
  if (!heff_valid(op) || !x || niter < 1) return DMRG_ERR_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (op->dtype == DMRG_COMPLEX128)
    return lanczos_impl<cplx>(op, static_cast<cplx*>(x), niter, tol, energy, iters, work, work_bytes, s);
  return lanczos_impl<double>(op, static_cast<double*>(x), niter, tol, energy, iters, work, work_bytes, s);
}

size_t dmrg_expm_workspace_bytes(const dmrg_heff_t* op, int niter) { return dmrg_lanczos_workspace_bytes(op, niter); }

int dmrg_krylov_expm(const dmrg_heff_t* op, void* x, double coeff_re, double coeff_im, int niter, double tol,
                     double errgoal, int* iters, void* work, size_t work_bytes, void* stream) {
  if (!heff_valid(op) || !x || niter < 1) return DMRG_ERR_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  std::complex<double> c(coeff_re, coeff_im);
  if (op->dtype == DMRG_COMPLEX128)
    return expm_impl<cplx>(op, static_cast<cplx*>(x), c, niter, tol, errgoal, iters, work, work_bytes, s);
  return expm_impl<double>(op, static_cast<double*>(x), c, niter, tol, errgoal, iters, work, work_bytes, s);
}

size_t dmrg_svd_workspace_bytes(int dtype, int m, int n) {
  if (m <= 0 || n <= 0) return 0;
  size_t b = 0;
  for (int absorb = 0; absorb < 3; ++absorb) b = std::max(b, svd_total_bytes(dtype, m, n, absorb));
  return b;
}

int dmrg_svd_truncate(int dtype, int m, int n, const void* M, double cutoff, int maxdim, int mindim, int absorb,
                      void* left_out, void* right_out, double* svals, int* keep, double* discarded, void* work,
                      size_t work_bytes, void* stream) {
  if (m <= 0 || n <= 0 || !M || !left_out || !right_out || absorb < 0 || absorb > 2) return DMRG_ERR_ARG;
  if (dtype != DMRG_REAL64 && dtype != DMRG_COMPLEX128) return DMRG_ERR_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (dtype == DMRG_COMPLEX128)
    return svd_impl<cplx>(m, n, static_cast<const cplx*>(M), cutoff, maxdim, mindim, absorb, static_cast<cplx*>(left_out),
                          static_cast<cplx*>(right_out), svals, keep, discarded, work, work_bytes, s);
  return svd_impl<double>(m, n, static_cast<const double*>(M), cutoff, maxdim, mindim, absorb,
                          static_cast<double*>(left_out), static_cast<double*>(right_out), svals, keep, discarded, work,
                          work_bytes, s);
}

size_t dmrg_gemm_workspace_bytes(int dtype, int precision, int m, int k, int n) {
  if (precision == DMRG_PREC_TF32X3) return tf32x3_gemm_workspace_bytes(m, k, n);
  return 0;
}

int dmrg_gemm(int dtype, int precision, int m, int k, int n, const void* A, const void* B, void* C, void* work,
              size_t work_bytes, void* stream) {
  if (m <= 0 || k <= 0 || n <= 0 || !A || !B || !C) return DMRG_ERR_ARG;
  if (dtype != DMRG_REAL64 && dtype != DMRG_COMPLEX128) return DMRG_ERR_ARG;
  if (dmrg_gemm_workspace_bytes(dtype, precision, m, k, n) > work_bytes) return DMRG_ERR_WORKSPACE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (precision == DMRG_PREC_TF32X3) {
    if (dtype != DMRG_REAL64) return DMRG_ERR_UNSUPPORTED;
    return tf32x3_gemm(m, k, n, static_cast<const double*>(A), static_cast<const double*>(B), static_cast<double*>(C),
                       work, s);
  }
  TGemm g{};
  g.B = ax(1); g.M = ax(m); g.K = ax(k); g.N = ax(n);
  g.a_m = st(k); g.a_k = st(1);
  g.b_k = st(n); g.b_n = st(1);
  g.c_m = st(n); g.c_n = st(1);
  if (dtype == DMRG_COMPLEX128)
    return tgemm<cplx>(g, Sc<cplx>::one(), static_cast<const cplx*>(A), static_cast<const cplx*>(B), Sc<cplx>::zero(),
                       static_cast<cplx*>(C), s);
  return tgemm<double>(g, 1.0, static_cast<const double*>(A), static_cast<const double*>(B), 0.0,
                       static_cast<double*>(C), s);
}

size_t dmrg_gram_workspace_bytes(int method, int m, int k) {
  if (m <= 0 || k <= 0) return 0;
  return method == DMRG_GRAM_DIGITS ? gram_digits_workspace_bytes(m, k) : 0;
}

int dmrg_gram(int method, int m, int k, const void* X, long long ld, void* G, void* work, size_t work_bytes,
              void* stream) {
  if (m <= 0 || k <= 0 || ld < k || !X || !G) return DMRG_ERR_ARG;
  if (method != DMRG_GRAM_FP64 && method != DMRG_GRAM_DIGITS) return DMRG_ERR_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const double* x = static_cast<const double*>(X);
  double* g = static_cast<double*>(G);
  if (method == DMRG_GRAM_FP64) {
    DMRG_TRY(tgemm_gram(x, ld, m, k, g, s));
    DMRG_CUDA_TRY(cudaStreamSynchronize(s));
    return DMRG_OK;
  }
  if (!work || dmrg_gram_workspace_bytes(method, m, k) > work_bytes) return DMRG_ERR_WORKSPACE;
  int* err = static_cast<int*>(work);   // the workspace head is reserved for the status word
  DMRG_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), s));
  DMRG_TRY(gram_digits(x, ld, m, k, g, work, work_bytes, err, s));
  int h = 0;
  DMRG_CUDA_TRY(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  DMRG_CUDA_TRY(cudaStreamSynchronize(s));
  return h;
}

size_t dmrg_subspace_workspace_bytes(int m, int n, int k) {
  if (m <= 0 || n <= 0 || k <= 0) return 0;
  return subspace_workspace_bytes(m, n, k);
}

int dmrg_subspace_truncate(int m, int n, int k, const void* theta, const void* start, int kstart, int absorb,
                           int iters, void* left_out, void* right_out, double* discarded, void* work,
                           size_t work_bytes, void* stream) {
  if (m <= 0 || n <= 0 || k <= 0 || !theta || !left_out || !right_out || (kstart > 0 && !start)) return DMRG_ERR_ARG;
  if (absorb != 0 && absorb != 1) return DMRG_ERR_ARG;
  return subspace_truncate(m, n, k, static_cast<const double*>(theta), static_cast<const double*>(start), kstart,
                           absorb, iters, static_cast<double*>(left_out), static_cast<double*>(right_out), discarded,
                           work, work_bytes, static_cast<cudaStream_t>(stream));
}

size_t dmrg_syev_workspace_bytes(int n) { return n > 0 ? syev_jacobi_workspace_bytes(n) : 0; }

int dmrg_syev(int n, const void* A, long long lda, double* w, void* V, long long ldv, int* sweeps, void* work,
              size_t work_bytes, void* stream) {
  if (n <= 0 || !A || lda < n || !w || (V && ldv < n)) return DMRG_ERR_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  DMRG_TRY(syev_jacobi(n, static_cast<const double*>(A), lda, w, 40, sweeps, work, work_bytes, s));
  if (V) {
    DMRG_TRY(syev_vectors(n, n, static_cast<double*>(V), ldv, 0, work, s));
    DMRG_CUDA_TRY(cudaStreamSynchronize(s));
  }
  return DMRG_OK;
}

size_t dmrg_subspace_truncate_ex_workspace_bytes(int precision, int m, int n, int k) {
  if (m <= 0 || n <= 0 || k <= 0) return 0;
  if (precision == DMRG_PREC_FP64) return rr_truncate_workspace_bytes(m, n, k);
  // the residual check of a positive cutoff reuses the Ritz scratch:
  // theta - lo ro (m x n) plus the split operands of that product
  const size_t ritz = std::max(subspace_ritz_workspace_bytes(m, n, k),
                               align_up(sizeof(double) * (size_t)m * n) + tf32x3_gemm_ex_workspace_bytes(m, n, k));
  return subspace_workspace_bytes(m, n, k) + ritz + align_up(64);
}

int dmrg_subspace_truncate_ex(int precision, int m, int n, int k, const void* theta, const void* start, int kstart,
                              int absorb, int iters, double cutoff, int mindim, void* left_out, void* right_out,
                              double* svals, int* keep, double* discarded, void* work, size_t work_bytes,
                              void* stream) {
  if (m <= 0 || n <= 0 || k <= 0 || k > std::min(m, n) || !theta || !left_out || !right_out || !keep ||
      (kstart > 0 && !start) || (absorb != 0 && absorb != 1) || (precision == DMRG_PREC_FP64 && !svals))
    return DMRG_ERR_ARG;
  if (precision != DMRG_PREC_FP64 && precision != DMRG_PREC_TF32X3) return DMRG_ERR_ARG;
  if (!work || dmrg_subspace_truncate_ex_workspace_bytes(precision, m, n, k) > work_bytes) return DMRG_ERR_WORKSPACE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const double* th = static_cast<const double*>(theta);
  double* lo = static_cast<double*>(left_out);
  double* ro = static_cast<double*>(right_out);
  double disc = 0.0;
  if (precision == DMRG_PREC_FP64) {
    int nv = 0;
    DMRG_TRY(rr_truncate(m, n, k, th, static_cast<const double*>(start), kstart, absorb, iters, cutoff, mindim, lo,
                         ro, svals, &nv, keep, &disc, work, work_bytes, s));
    for (int i = nv; i < k; ++i) svals[i] = 0.0;
  } else {
    const size_t sb = subspace_workspace_bytes(m, n, k);
    char* base = static_cast<char*>(work);
    double* tot = reinterpret_cast<double*>(base + sb);
    void* rw = base + sb + align_up(64);
    DMRG_TRY(subspace_truncate(m, n, k, th, static_cast<const double*>(start), kstart, absorb, iters, lo, ro, &disc,
                               work, sb, s));
    if (cutoff > 0.0) {
      // the weight outside the kept space as |theta - lo ro|^2: the
      // split-TF32 error of the factors (~5e-7 |theta|) enters it squared
      // plus a cross term, whereas |theta|^2 - |C|^2 carries it linearly
      double* res = static_cast<double*>(rw);
      int* err = reinterpret_cast<int*>(tot + 2);
      DMRG_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), s));
      DMRG_CUDA_TRY(cudaMemcpyAsync(res, th, sizeof(double) * (size_t)m * n, cudaMemcpyDeviceToDevice, s));
      DMRG_TRY(tf32x3_gemm_ex(0, 0, m, n, k, -1.f, lo, k, ro, n, 1, res, n,
                              static_cast<char*>(rw) + align_up(sizeof(double) * (size_t)m * n), err, s));
      DMRG_TRY(sumsq_dev(th, (long long)m * n, tot, s));
      DMRG_TRY(sumsq_dev(res, (long long)m * n, tot + 1, s));
      int e = 0;
      double h[2] = {0.0, 0.0};
      DMRG_CUDA_TRY(cudaMemcpyAsync(&e, err, sizeof(int), cudaMemcpyDeviceToHost, s));
      DMRG_CUDA_TRY(cudaMemcpyAsync(h, tot, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
      DMRG_CUDA_TRY(cudaStreamSynchronize(s));
      if (e != 0) return e;
      const double rem = h[0] > 0.0 ? h[1] / h[0] : 0.0;
      // keep = k is the rule's answer when the weight beyond the kept space
      // exceeds the cutoff (no kept direction may then be dropped); decide it
      // only when that holds beyond the estimate's own error and beyond the
      // few 1e-12 by which one product with the previous basis may miss the
      // optimal subspace, else leave the bond to the FP64 route
      if (!(rem - (1e-12 + 2e-6 * std::sqrt(rem)) > cutoff) || rem < 10.0 * cutoff + 1e-11)
        return DMRG_ERR_PRECISION;
      disc = rem;
    }
    *keep = k;
    if (svals) DMRG_TRY(subspace_ritz(m, n, k, absorb, lo, ro, svals, rw, work_bytes - sb - align_up(64), s));
  }
  if (discarded) *discarded = disc;
  return DMRG_OK;
}

}  // extern "C"
