// Effective-Hamiltonian matvecs and environment updates as chains of strided
// contractions (FP64 / complex FP64 path).  Contraction order follows the
// reference plan (theta.L, .W_i, .W_j, .R), with the two small MPO steps
// run as batched GEMMs; the index permutations are expressed through strides
// so no transpose copies are made.
#include "heff.cuh"

namespace dmrg {

template <typename T>
size_t heff_fp64_elems(const dmrg_heff_t& o, size_t* p_elems, size_t* q_elems) {
  size_t P = 0, Q = 0;
  const size_t cl = o.chil, cr = o.chir, d1 = o.d1, d2 = o.d2, wl = o.wl, wm = o.wm, wr = o.wr;
  if (o.kind == 2) {
    size_t x1 = cl * wl * d1 * d2 * cr, x2 = cl * d1 * wm * d2 * cr, x3 = cl * d1 * d2 * wr * cr;
    P = x1 > x3 ? x1 : x3;
    Q = x2;
  } else if (o.kind == 1) {
    P = cl * wl * d1 * cr;
    Q = cl * d1 * wr * cr;
  } else {
    P = cl * wl * cr;
    Q = 0;
  }
  if (p_elems) *p_elems = P;
  if (q_elems) *q_elems = Q;
  return P + Q;
}

// The contraction steps of one matvec (all with alpha 1, beta 0), in order.
template <typename T>
int heff_fp64_plan(const dmrg_heff_t& o, const T* x, T* y, T* P, T* Q, GStep* steps) {
  int n = 0;
  const long long cl = o.chil, cr = o.chir, d1 = o.d1, d2 = o.d2, wl = o.wl, wm = o.wm, wr = o.wr;
  const T* L = static_cast<const T*>(o.L);
  const T* R = static_cast<const T*>(o.R);
  const T* W1 = static_cast<const T*>(o.W1);
  const T* W2 = static_cast<const T*>(o.W2);
  TGemm g;
  if (o.kind == 2) {
    // X1[(a',k)][(s,t,b)] = L[(a',k)][a] x[a][(s,t,b)]
    g = TGemm{};
    g.B = ax(1); g.M = ax((int)(cl * wl)); g.K = ax((int)cl); g.N = ax((int)(d1 * d2 * cr));
    g.a_m = st(cl); g.a_k = st(1);
    g.b_k = st(d1 * d2 * cr); g.b_n = st(1);
    g.c_m = st(d1 * d2 * cr); g.c_n = st(1);
    steps[n++] = GStep{g, L, x, P};
    // X2[a'][(s',m)][(t,b)] = W1[(k,s)][(s',m)] X1[a'][(k,s)][(t,b)]
    g = TGemm{};
    g.B = ax((int)cl); g.M = ax((int)(d1 * wm)); g.K = ax((int)(wl * d1)); g.N = ax((int)(d2 * cr));
    g.a_b = st(0); g.a_m = st(1); g.a_k = st(d1 * wm);
    g.b_b = st(wl * d1 * d2 * cr); g.b_k = st(d2 * cr); g.b_n = st(1);
    g.c_b = st(d1 * wm * d2 * cr); g.c_m = st(d2 * cr); g.c_n = st(1);
    steps[n++] = GStep{g, W1, P, Q};
    // X3[(a',s')][(t',n)][b] = W2[(m,t)][(t',n)] X2[(a',s')][(m,t)][b]
    g = TGemm{};
    g.B = ax((int)(cl * d1)); g.M = ax((int)(d2 * wr)); g.K = ax((int)(wm * d2)); g.N = ax((int)cr);
    g.a_b = st(0); g.a_m = st(1); g.a_k = st(d2 * wr);
    g.b_b = st(wm * d2 * cr); g.b_k = st(cr); g.b_n = st(1);
    g.c_b = st(d2 * wr * cr); g.c_m = st(cr); g.c_n = st(1);
    steps[n++] = GStep{g, W2, Q, P};
    // y[(a',s',t')][b'] = X3[(a',s',t')][(n,b)] R[b'][(n,b)]
    g = TGemm{};
    g.B = ax(1); g.M = ax((int)(cl * d1 * d2)); g.K = ax((int)(wr * cr)); g.N = ax((int)cr);
    g.a_m = st(wr * cr); g.a_k = st(1);
    g.b_k = st(1); g.b_n = st(wr * cr);
    g.c_m = st(cr); g.c_n = st(1);
    steps[n++] = GStep{g, P, R, y};
  } else if (o.kind == 1) {
    g = TGemm{};
    g.B = ax(1); g.M = ax((int)(cl * wl)); g.K = ax((int)cl); g.N = ax((int)(d1 * cr));
    g.a_m = st(cl); g.a_k = st(1);
    g.b_k = st(d1 * cr); g.b_n = st(1);
    g.c_m = st(d1 * cr); g.c_n = st(1);
    steps[n++] = GStep{g, L, x, P};
    // X2[a'][(s',m)][b] = W[(k,s)][(s',m)] X1[a'][(k,s)][b]
    g = TGemm{};
    g.B = ax((int)cl); g.M = ax((int)(d1 * wr)); g.K = ax((int)(wl * d1)); g.N = ax((int)cr);
    g.a_b = st(0); g.a_m = st(1); g.a_k = st(d1 * wr);
    g.b_b = st(wl * d1 * cr); g.b_k = st(cr); g.b_n = st(1);
    g.c_b = st(d1 * wr * cr); g.c_m = st(cr); g.c_n = st(1);
    steps[n++] = GStep{g, W1, P, Q};
    // y[(a',s')][b'] = X2[(a',s')][(m,b)] R[b'][(m,b)]
    g = TGemm{};
    g.B = ax(1); g.M = ax((int)(cl * d1)); g.K = ax((int)(wr * cr)); g.N = ax((int)cr);
    g.a_m = st(wr * cr); g.a_k = st(1);
    g.b_k = st(1); g.b_n = st(wr * cr);
    g.c_m = st(cr); g.c_n = st(1);
    steps[n++] = GStep{g, Q, R, y};
  } else {
    g = TGemm{};
    g.B = ax(1); g.M = ax((int)(cl * wl)); g.K = ax((int)cl); g.N = ax((int)cr);
    g.a_m = st(cl); g.a_k = st(1);
    g.b_k = st(cr); g.b_n = st(1);
    g.c_m = st(cr); g.c_n = st(1);
    steps[n++] = GStep{g, L, x, P};
    g = TGemm{};
    g.B = ax(1); g.M = ax((int)cl); g.K = ax((int)(wl * cr)); g.N = ax((int)cr);
    g.a_m = st(wl * cr); g.a_k = st(1);
    g.b_k = st(1); g.b_n = st(wl * cr);
    g.c_m = st(cr); g.c_n = st(1);
    steps[n++] = GStep{g, P, R, y};
  }
  return n;
}

template <typename T>
int heff_apply_fp64(const dmrg_heff_t& o, const T* x, T* y, T* P, T* Q, cudaStream_t s) {
  GStep steps[4];
  const int n = heff_fp64_plan<T>(o, x, y, P, Q, steps);
  for (int i = 0; i < n; ++i)
    DMRG_TRY(tgemm<T>(steps[i].g, Sc<T>::one(), static_cast<const T*>(steps[i].A), static_cast<const T*>(steps[i].B),
                      Sc<T>::zero(), static_cast<T*>(steps[i].C), s));
  return DMRG_OK;
}

size_t env_fp64_elems(int side, long long cl, long long d, long long cr, long long wl, long long wr) {
  if (side == 0) return (size_t)(cl * wl * d * cr + cl * d * wr * cr);
  return (size_t)(cr * wr * cl * d + cr * wl * d * cl);
}

template <typename T>
int env_left_plan(long long cl, long long d, long long cr, long long wl, long long wr, const T* L, const T* W,
                  const T* A, T* Lnew, T* P, GStep* steps) {
  int n = 0;
  T* Y1 = P;
  T* Y2 = P + cl * wl * d * cr;
  TGemm g{};
  g.B = ax(1); g.M = ax((int)(cl * wl)); g.K = ax((int)cl); g.N = ax((int)(d * cr));
  g.a_m = st(cl); g.a_k = st(1);
  g.b_k = st(d * cr); g.b_n = st(1);
  g.c_m = st(d * cr); g.c_n = st(1);
  steps[n++] = GStep{g, L, A, Y1};
  g = TGemm{};
  g.B = ax((int)cl); g.M = ax((int)(d * wr)); g.K = ax((int)(wl * d)); g.N = ax((int)cr);
  g.a_b = st(0); g.a_m = st(1); g.a_k = st(d * wr);
  g.b_b = st(wl * d * cr); g.b_k = st(cr); g.b_n = st(1);
  g.c_b = st(d * wr * cr); g.c_m = st(cr); g.c_n = st(1);
  steps[n++] = GStep{g, W, Y1, Y2};
  // Lnew[b'][(m,b)] = conj(A)[(a',s')][b'] Y2[(a',s')][(m,b)]
  g = TGemm{};
  g.B = ax(1); g.M = ax((int)cr); g.K = ax((int)(cl * d)); g.N = ax((int)(wr * cr));
  g.a_m = st(1); g.a_k = st(cr); g.conjA = 1;
  g.b_k = st(wr * cr); g.b_n = st(1);
  g.c_m = st(wr * cr); g.c_n = st(1);
  steps[n++] = GStep{g, A, Y2, Lnew};
  return n;
}

template <typename T>
int env_left_fp64(long long cl, long long d, long long cr, long long wl, long long wr, const T* L, const T* W,
                  const T* A, T* Lnew, T* P, cudaStream_t s) {
  GStep steps[3];
  const int n = env_left_plan<T>(cl, d, cr, wl, wr, L, W, A, Lnew, P, steps);
  for (int i = 0; i < n; ++i)
    DMRG_TRY(tgemm<T>(steps[i].g, Sc<T>::one(), static_cast<const T*>(steps[i].A), static_cast<const T*>(steps[i].B),
                      Sc<T>::zero(), static_cast<T*>(steps[i].C), s));
  return DMRG_OK;
}

template <typename T>
int env_right_plan(long long cl, long long d, long long cr, long long wl, long long wr, const T* R, const T* W,
                   const T* B, T* Rnew, T* P, GStep* steps) {
  int n = 0;
  T* Z1 = P;
  T* Z2 = P + cr * wr * cl * d;
  // Z1[(b',m)][(a,s)] = R[(b',m)][b] B[(a,s)][b]
  TGemm g{};
  g.B = ax(1); g.M = ax((int)(cr * wr)); g.K = ax((int)cr); g.N = ax((int)(cl * d));
  g.a_m = st(cr); g.a_k = st(1);
  g.b_k = st(1); g.b_n = st(cr);
  g.c_m = st(cl * d); g.c_n = st(1);
  steps[n++] = GStep{g, R, B, Z1};
  // Z2[b'][(k,s')][a] = W[k][s][s'][m] Z1[b'][m][a][s]   (K = (m, s))
  g = TGemm{};
  g.B = ax((int)cr);
  g.M = ax((int)wl, (int)d);
  g.K = ax((int)wr, (int)d);
  g.N = ax((int)cl);
  g.a_b = st(0); g.a_m = st(d * d * wr, wr); g.a_k = st(1, d * wr);
  g.b_b = st(wr * cl * d); g.b_k = st(cl * d, 1); g.b_n = st(d);
  g.c_b = st(wl * d * cl); g.c_m = st(d * cl, cl); g.c_n = st(1);
  steps[n++] = GStep{g, W, Z1, Z2};
  // Rnew[a'][(k,a)] = conj(B)[a'][(b',s')] Z2[(b',s')][(k,a)]
  g = TGemm{};
  g.B = ax(1);
  g.M = ax((int)cl);
  g.K = ax((int)cr, (int)d);
  g.N = ax((int)wl, (int)cl);
  g.a_m = st(d * cr); g.a_k = st(1, cr); g.conjA = 1;
  g.b_k = st(wl * d * cl, cl); g.b_n = st(d * cl, 1);
  g.c_m = st(wl * cl); g.c_n = st(cl, 1);
  steps[n++] = GStep{g, B, Z2, Rnew};
  return n;
}

template <typename T>
int env_right_fp64(long long cl, long long d, long long cr, long long wl, long long wr, const T* R, const T* W,
                   const T* B, T* Rnew, T* P, cudaStream_t s) {
  GStep steps[3];
  const int n = env_right_plan<T>(cl, d, cr, wl, wr, R, W, B, Rnew, P, steps);
  for (int i = 0; i < n; ++i)
    DMRG_TRY(tgemm<T>(steps[i].g, Sc<T>::one(), static_cast<const T*>(steps[i].A), static_cast<const T*>(steps[i].B),
                      Sc<T>::zero(), static_cast<T*>(steps[i].C), s));
  return DMRG_OK;
}

template size_t heff_fp64_elems<double>(const dmrg_heff_t&, size_t*, size_t*);
template size_t heff_fp64_elems<cplx>(const dmrg_heff_t&, size_t*, size_t*);
template int heff_apply_fp64<double>(const dmrg_heff_t&, const double*, double*, double*, double*, cudaStream_t);
template int heff_apply_fp64<cplx>(const dmrg_heff_t&, const cplx*, cplx*, cplx*, cplx*, cudaStream_t);
template int heff_fp64_plan<double>(const dmrg_heff_t&, const double*, double*, double*, double*, GStep*);
template int heff_fp64_plan<cplx>(const dmrg_heff_t&, const cplx*, cplx*, cplx*, cplx*, GStep*);
template int env_left_plan<double>(long long, long long, long long, long long, long long, const double*,
                                   const double*, const double*, double*, double*, GStep*);
template int env_left_plan<cplx>(long long, long long, long long, long long, long long, const cplx*, const cplx*,
                                 const cplx*, cplx*, cplx*, GStep*);
template int env_right_plan<double>(long long, long long, long long, long long, long long, const double*,
                                    const double*, const double*, double*, double*, GStep*);
template int env_right_plan<cplx>(long long, long long, long long, long long, long long, const cplx*, const cplx*,
                                  const cplx*, cplx*, cplx*, GStep*);
template int env_left_fp64<double>(long long, long long, long long, long long, long long, const double*, const double*,
                                   const double*, double*, double*, cudaStream_t);
template int env_left_fp64<cplx>(long long, long long, long long, long long, long long, const cplx*, const cplx*,
                                 const cplx*, cplx*, cplx*, cudaStream_t);
template int env_right_fp64<double>(long long, long long, long long, long long, long long, const double*, const double*,
                                    const double*, double*, double*, cudaStream_t);
template int env_right_fp64<cplx>(long long, long long, long long, long long, long long, const cplx*, const cplx*,
                                  const cplx*, cplx*, cplx*, cudaStream_t);

}  // namespace dmrg
