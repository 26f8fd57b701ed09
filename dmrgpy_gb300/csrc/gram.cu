// Gram matrix G = X^T X of an FP64 block X (m x k, row-major) on the
// tensor cores with near-FP64 accuracy, by exact digit products (an
// Ozaki-type splitting).
//
// Each column a of X is scaled by a power of two sigma_a >= max_i |X_ia|,
// so y = X / sigma lies in [-1, 1], and cut into three 8-bit digits and a
// tail:
//   y = D0 + D1 + D2 + T,  D0 = d0 2^-7, D1 = d1 2^-15, D2 = d2 2^-23,
//   |d0|, |d1|, |d2| <= 128 (integers),  |T| <= 1.5 2^-24,  T = Th + Tl (TF32)
// (the digits are those of y rounded to FP32, T holds the rest of y).
// Every digit is exact in TF32 and every digit product is exact in FP32.
// Per K-slice of 32 the products of one order are summed in their own TMEM
// accumulator:
//   P0 = sum D0 D0                          (a multiple of 2^-14)
//   P1 = sum (D0 D1 + D1 D0)                (a multiple of 2^-22)
//   P2 = sum (D1 D1 + D0 D2 + D2 D0)        (a multiple of 2^-30)
// each below 2^21 units, so the tensor core adds them without rounding
// whatever its accumulation rounding; the epilogue adds them over the
// slices as int32 counts of their unit.  The tail
//   P3 = sum over (D1 D2, D2 D1, D0 Th, Th D0, D0 Tl, Tl D0, D2 D2, D1 Th,
//                  Th D1, D2 Th, Th D2, D1 Tl, Tl D1)
// (products <= 1.5 2^-24) is summed in FP32; the pairs left out are below
// 2^-46 per product.  Then
//   G_ab = sigma_a sigma_b (P0 2^-14 + P1 2^-22 + P2 2^-30 + P3)
// with the first three terms exact (45 bits, added exactly in FP64).
// Against an extended-precision Gram the error is ~1e-13 relative to
// |x_a| |x_b| (an FP64 product: ~1e-15), where a split-TF32 Gram gives
// ~1e-7; the FP64 CUDA-core Gram it replaces is 15-20x slower.
//
// Only tiles touching the upper triangle are computed; each element with
// column >= row is written to G[r][c] and G[c][r], so G is exactly
// symmetric.
//
// Kernel layout (one CTA per 128 x 32 tile, 320 threads):
//   warp 0     TMA producer: per K-slice the five digit operands of the
//              128-row A panel and of the 32-row B panel (100 KB per
//              stage, two stages);
//   warp 1     TMEM allocation and the single MMA-issuing thread
//              (tcgen05.mma kind::tf32, 19 digit pairs x 4 K-steps);
//   warps 2-9  epilogue: warp w reads TMEM lane quarter w % 4, columns
//              16 * ((w - 2) / 4) .. +15, of the four accumulators.
// All mbarrier waits are bounded (DMRG_ERR_TIMEOUT is recorded on expiry).
#include "tcgen05.cuh"
#include "tf32x3.cuh"

namespace dmrg {

namespace {

constexpr int GM = 128;                 // tile rows = TMEM lanes
constexpr int GN = 32;                  // tile columns
constexpr int GK = 32;                  // fp32 per K-slice = one SW128 row
constexpr int GSTAGES = 2;
constexpr int NOPS = 5;                 // digit operands D0, D1, D2, Th, Tl
constexpr int GA_BYTES = GM * GK * 4;   // 16 KB
constexpr int GB_BYTES = GN * GK * 4;   // 4 KB
constexpr int GST_BYTES = NOPS * (GA_BYTES + GB_BYTES);   // 100 KB
constexpr int GRAM_SMEM = GSTAGES * GST_BYTES + 1024 + 256;
constexpr int GRAM_THREADS = 320;
constexpr int NBUF = 4;                 // P0, P1, P2 (exact), P3 (tail)
constexpr int GACC = 2;                 // K-slices in flight in TMEM
constexpr int TMEM_COLS = 256;          // = NBUF * GACC * GN (power of two)
// per K-slice |P2| <= 3 * 32 * 2^14 units, so the int32 running sums stay
// below 2^31 for up to 1024 K-slices (m <= 32768)
constexpr int MAX_KT = 1024;

constexpr int TPR = GM / GN;            // column tiles per row tile
static_assert(GM % GN == 0, "tile rows a multiple of tile columns");
constexpr int ECOLS = GN / 2;           // columns per epilogue thread
static_assert(NBUF * GACC * GN <= TMEM_COLS, "TMEM accumulators");

__global__ void colmax_kernel(const double* __restrict__ X, long long ld, int m, int k,
                              unsigned long long* __restrict__ mx, int* __restrict__ err) {
  __shared__ double sh[8][33];
  const int lane = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int c = blockIdx.x * 32 + lane;
  // |x| and its maximum on the bit patterns (integer compares order
  // non-negative doubles like their values; no FP64 arithmetic)
  unsigned long long v = 0ull;
  bool bad = false;
  if (c < k) {
    for (int r = blockIdx.y * 8 + ty; r < m; r += gridDim.y * 8) {
      const unsigned long long a =
          static_cast<unsigned long long>(__double_as_longlong(X[(long long)r * ld + c])) & 0x7FFFFFFFFFFFFFFFull;
      if (a >= 0x7FF0000000000000ull) bad = true;   // inf or nan
      v = a > v ? a : v;
    }
  }
  if (bad) atomicExch(err, DMRG_ERR_NAN);
  sh[ty][lane] = v;
  __syncthreads();
  if (ty == 0 && c < k) {
#pragma unroll
    for (int j = 1; j < 8; ++j) v = sh[j][lane] > v ? sh[j][lane] : v;
    atomicMax(&mx[c], v);
  }
}

// power of two >= x (x >= 0 finite); 1 for x = 0
__device__ __forceinline__ double pow2_ceil(double x) {
  if (!(x > 0.0)) return 1.0;
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
  int e = (int)((b >> 52) & 0x7FF);             // biased exponent, x in [2^(e-1023), 2^(e-1022))
  const bool exact = (b & 0xFFFFFFFFFFFFFull) == 0 && e != 0;
  if (e == 0) e = 1;                            // subnormal: 2^-1022 bounds it
  else if (!exact) e += 1;
  if (e > 2046) e = 2046;
  return __longlong_as_double(static_cast<long long>(static_cast<unsigned long long>(e) << 52));
}

// Digit operands, transposed: out[a][i] (a < k, i < Kp) from X[i][a];
// rows i >= m are zero.  sigma[a] = pow2_ceil(max_i |X_ia|).
__global__ void digits_kernel(const double* __restrict__ X, long long ld, int m, int k, int Kp,
                              const unsigned long long* __restrict__ mx, double* __restrict__ sigma,
                              float* __restrict__ D0, float* __restrict__ D1, float* __restrict__ D2,
                              float* __restrict__ Th, float* __restrict__ Tl) {
  __shared__ double t[32][33];
  const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int j = ty; j < 32; j += 8) {
    const int r = r0 + j, c = c0 + tx;
    t[j][tx] = (r < m && c < k) ? X[(long long)r * ld + c] : 0.0;
  }
  __syncthreads();
  for (int j = ty; j < 32; j += 8) {
    const int c = c0 + j, r = r0 + tx;
    if (c >= k || r >= Kp) continue;
    const double sg = pow2_ceil(__longlong_as_double(static_cast<long long>(mx[c])));
    if (r == 0) sigma[c] = sg;
    // y = x / sg (|y| <= 1) as an FP32 pair yh + yl (48 bits; one FP64
    // product and one subtraction, the rest bit operations and FP32
    // arithmetic: GB300's FP64 pipe bounded the all-FP64 form).  The digits come from yh: every FP32
    // step below is exact (power-of-two scalings, integer rounding, and the
    // difference of a number and its rounding), so Z = yh 2^23 =
    // d0 2^16 + d1 2^8 + d2 + rem exactly with |d*| <= 128, |rem| <= 1/2.
    // 1/sg from the exponent bits (sg = 2^(e - 1023), 1 <= e <= 2045 after
    // pow2_ceil: 1/sg = 2^(1023 - e), biased exponent 2046 - e)
    const int e = (int)((static_cast<unsigned long long>(__double_as_longlong(sg)) >> 52) & 0x7FF);
    const double inv = (e >= 1 && e <= 2045)
                           ? __longlong_as_double(static_cast<long long>(static_cast<unsigned long long>(2046 - e) << 52))
                           : 1.0 / sg;
    const double y = t[tx][j] * inv;      // exact: a power-of-two scaling
    const float yh = narrow(y);
    const float yl = narrow(y - widen(yh));   // exact difference
    const float d0 = rintf(yh * 128.0f);
    const float r1 = yh * 128.0f - d0;
    const float d1 = rintf(r1 * 256.0f);
    const float r2 = r1 * 256.0f - d1;
    const float d2 = rintf(r2 * 256.0f);
    const float tt = fmaf(r2 * 256.0f - d2, 0x1p-23f, yl);   // tail of y beyond the digits, |tt| <= 1.5 2^-24
    const float th = to_tf32(tt);
    const float tl = to_tf32(tt - th);
    const long long o = (long long)c * Kp + r;
    D0[o] = d0 * 0x1p-7f;
    D1[o] = d1 * 0x1p-15f;
    D2[o] = d2 * 0x1p-23f;
    Th[o] = th;
    Tl[o] = tl;
  }
}

__global__ void __launch_bounds__(GRAM_THREADS, 1)
    gram_digits_kernel(const __grid_constant__ CUtensorMap mA0, const __grid_constant__ CUtensorMap mA1,
                       const __grid_constant__ CUtensorMap mA2, const __grid_constant__ CUtensorMap mA3,
                       const __grid_constant__ CUtensorMap mA4, const __grid_constant__ CUtensorMap mB0,
                       const __grid_constant__ CUtensorMap mB1, const __grid_constant__ CUtensorMap mB2,
                       const __grid_constant__ CUtensorMap mB3, const __grid_constant__ CUtensorMap mB4, int KT,
                       int tiles_m, int tiles_n, int k, const double* __restrict__ sigma, double* __restrict__ G,
                       int* err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + GSTAGES * GST_BYTES);
  uint64_t* empty = full + GSTAGES;
  uint64_t* acc_full = empty + GSTAGES;
  uint64_t* acc_empty = acc_full + GACC;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(acc_empty + GACC);

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  // upper-triangle tile list, row-tile by row-tile: row tile mi keeps the
  // column tiles nj >= TPR mi (the first one whose last column reaches row
  // GM mi)
  int t = (int)blockIdx.x, mi = 0;
  for (; mi < tiles_m; ++mi) {
    const int cnt = tiles_n - TPR * mi;
    if (cnt <= 0) { mi = tiles_m; break; }
    if (t < cnt) break;
    t -= cnt;
  }
  if (mi >= tiles_m) return;   // (grid sized to the tile count: not reached)
  const int m0 = mi * GM;
  const int n0 = (TPR * mi + t) * GN;

  if (threadIdx.x == 0) {
    for (int s = 0; s < GSTAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < GACC; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], 8);   // one arrival per epilogue warp
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      for (int kt = 0; kt < KT; ++kt) {
        const int s = kt % GSTAGES;
        const int it = kt / GSTAGES;
        if (kt >= GSTAGES && !mbar_wait(&empty[s], (it - 1) & 1, err)) break;
        unsigned char* st = smem + s * GST_BYTES;
        mbar_expect_tx(&full[s], GST_BYTES);
        const int x = kt * GK;
        tma_load_2d(st + 0 * GA_BYTES, &mA0, &full[s], x, m0);
        tma_load_2d(st + 1 * GA_BYTES, &mA1, &full[s], x, m0);
        tma_load_2d(st + 2 * GA_BYTES, &mA2, &full[s], x, m0);
        tma_load_2d(st + 3 * GA_BYTES, &mA3, &full[s], x, m0);
        tma_load_2d(st + 4 * GA_BYTES, &mA4, &full[s], x, m0);
        unsigned char* sb = st + NOPS * GA_BYTES;
        tma_load_2d(sb + 0 * GB_BYTES, &mB0, &full[s], x, n0);
        tma_load_2d(sb + 1 * GB_BYTES, &mB1, &full[s], x, n0);
        tma_load_2d(sb + 2 * GB_BYTES, &mB2, &full[s], x, n0);
        tma_load_2d(sb + 3 * GB_BYTES, &mB3, &full[s], x, n0);
        tma_load_2d(sb + 4 * GB_BYTES, &mB4, &full[s], x, n0);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_tf32(GM, GN);
      for (int kt = 0; kt < KT; ++kt) {
        const int s = kt % GSTAGES;
        const int it = kt / GSTAGES;
        const int b = kt % GACC;
        const int u = kt / GACC;
        if (!mbar_wait(&full[s], it & 1, err)) break;
        if (kt >= GACC && !mbar_wait(&acc_empty[b], (u - 1) & 1, err)) break;
        tc_fence_after();
        const uint32_t acc = tmem + b * NBUF * GN;
        const uint32_t p0 = acc, p1 = acc + GN, p2 = acc + 2 * GN, p3 = acc + 3 * GN;
        const uint32_t base = smem_u32(smem + s * GST_BYTES);
        const uint32_t bbase = base + NOPS * GA_BYTES;
#pragma unroll
        for (int kk = 0; kk < GK / 8; ++kk) {
          const uint32_t o = kk * 32;   // 8 tf32 = 32 bytes along K inside the swizzle row
          uint64_t a[NOPS], bb[NOPS];
#pragma unroll
          for (int i = 0; i < NOPS; ++i) {
            a[i] = sdesc_sw128(base + i * GA_BYTES + o);
            bb[i] = sdesc_sw128(bbase + i * GB_BYTES + o);
          }
          const uint32_t first = kk != 0;
          // operand index: 0 D0, 1 D1, 2 D2, 3 Th, 4 Tl
          mma_tf32(p0, a[0], bb[0], idesc, first);
          mma_tf32(p1, a[0], bb[1], idesc, first);
          mma_tf32(p1, a[1], bb[0], idesc, 1u);
          mma_tf32(p2, a[1], bb[1], idesc, first);
          mma_tf32(p2, a[0], bb[2], idesc, 1u);
          mma_tf32(p2, a[2], bb[0], idesc, 1u);
          mma_tf32(p3, a[1], bb[2], idesc, first);
          mma_tf32(p3, a[2], bb[1], idesc, 1u);
          mma_tf32(p3, a[0], bb[3], idesc, 1u);
          mma_tf32(p3, a[3], bb[0], idesc, 1u);
          mma_tf32(p3, a[0], bb[4], idesc, 1u);
          mma_tf32(p3, a[4], bb[0], idesc, 1u);
          mma_tf32(p3, a[2], bb[2], idesc, 1u);
          mma_tf32(p3, a[1], bb[3], idesc, 1u);
          mma_tf32(p3, a[3], bb[1], idesc, 1u);
          mma_tf32(p3, a[2], bb[3], idesc, 1u);
          mma_tf32(p3, a[3], bb[2], idesc, 1u);
          mma_tf32(p3, a[1], bb[4], idesc, 1u);
          mma_tf32(p3, a[4], bb[1], idesc, 1u);
        }
        mma_commit(&empty[s]);
        mma_commit(&acc_full[b]);
      }
    }
  } else {
    const int q = warp & 3;                 // TMEM lane quarter accessible to this warp
    const int h = (warp - 2) >> 2;          // column half
    const int row = q * 32 + lane;
    const uint32_t lane_addr = static_cast<uint32_t>(q * 32) << 16;
    int i0[ECOLS], i1[ECOLS], i2[ECOLS];
    float f3[ECOLS];
#pragma unroll
    for (int c = 0; c < ECOLS; ++c) {
      i0[c] = 0;
      i1[c] = 0;
      i2[c] = 0;
      f3[c] = 0.f;
    }
    bool ok = true;
    for (int kt = 0; kt < KT && ok; ++kt) {
      const int b = kt % GACC;
      const int u = kt / GACC;
      ok = mbar_wait(&acc_full[b], u & 1, err);
      tc_fence_after();
      if (ok) {
        const uint32_t t0 = tmem + lane_addr + b * NBUF * GN + h * ECOLS;
        float v[16];
        // P0..P2 are exact multiples of 2^-14, 2^-22, 2^-30 below 2^21 units
        tmem_ld16(t0, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) i0[j] += __float2int_rn(v[j] * 0x1p14f);
        tmem_ld16(t0 + GN, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) i1[j] += __float2int_rn(v[j] * 0x1p22f);
        tmem_ld16(t0 + 2 * GN, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) i2[j] += __float2int_rn(v[j] * 0x1p30f);
        tmem_ld16(t0 + 3 * GN, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) f3[j] += v[j];
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&acc_empty[b])) : "memory");
    }
    const int r = m0 + row;
    if (ok && r < k) {
      const double sr = sigma[r];
#pragma unroll
      for (int c = 0; c < ECOLS; ++c) {
        const int cc = n0 + h * ECOLS + c;
        if (cc >= r && cc < k) {
          const double exact = static_cast<double>(i0[c]) * 0x1p-14 + static_cast<double>(i1[c]) * 0x1p-22 +
                               static_cast<double>(i2[c]) * 0x1p-30;
          const double g = (exact + static_cast<double>(f3[c])) * (sr * sigma[cc]);
          G[(long long)r * k + cc] = g;
          G[(long long)cc * k + r] = g;
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
  }
}

inline int pad32i(long long x) { return (int)((x + 31) / 32 * 32); }

}  // namespace

size_t gram_digits_workspace_bytes(int m, int k) {
  if (m < 1 || k < 1) return 0;
  const size_t Kp = (size_t)pad32i(m);
  return align_up(256, 1024) + 2 * align_up(sizeof(double) * (size_t)k, 1024) +
         NOPS * align_up(sizeof(float) * (size_t)k * Kp, 1024);
}

int gram_digits(const double* X, long long ld, int m, int k, double* G, void* work, size_t work_bytes, int* err,
                cudaStream_t s) {
  if (m < 1 || k < 1 || ld < k || !X || !G) return DMRG_ERR_ARG;
  const int Kp = pad32i(m);
  if (Kp / GK > MAX_KT) return DMRG_ERR_ARG;
  if (gram_digits_workspace_bytes(m, k) > work_bytes) return DMRG_ERR_WORKSPACE;
  char* p = static_cast<char*>(work) + align_up(256, 1024);
  unsigned long long* mx = reinterpret_cast<unsigned long long*>(p); p += align_up(sizeof(double) * (size_t)k, 1024);
  double* sigma = reinterpret_cast<double*>(p); p += align_up(sizeof(double) * (size_t)k, 1024);
  float* ops[NOPS];
  for (int i = 0; i < NOPS; ++i) {
    ops[i] = reinterpret_cast<float*>(p);
    p += align_up(sizeof(float) * (size_t)k * Kp, 1024);
  }
  DMRG_CUDA_TRY(cudaMemsetAsync(mx, 0, sizeof(double) * (size_t)k, s));
  const int gy = (m + 7) / 8 < 64 ? (m + 7) / 8 : 64;
  colmax_kernel<<<dim3((k + 31) / 32, gy), 256, 0, s>>>(X, ld, m, k, mx, err);
  DMRG_CHECK_LAUNCH();
  const dim3 dg((k + 31) / 32, Kp / 32);
  if (dg.y > 65535) return DMRG_ERR_ARG;
  digits_kernel<<<dg, 256, 0, s>>>(X, ld, m, k, Kp, mx, sigma, ops[0], ops[1], ops[2], ops[3], ops[4]);
  DMRG_CHECK_LAUNCH();
  CUtensorMap ma[NOPS], mb[NOPS];
  for (int i = 0; i < NOPS; ++i) {
    DMRG_TRY(tma_map_k32(&ma[i], ops[i], k, Kp, GM));
    DMRG_TRY(tma_map_k32(&mb[i], ops[i], k, Kp, GN));
  }
  static std::atomic<unsigned long long> attr{0};
  DMRG_TRY(smem_attr_once(reinterpret_cast<const void*>(gram_digits_kernel), GRAM_SMEM, attr));
  const int tiles_m = (k + GM - 1) / GM, tiles_n = (k + GN - 1) / GN;
  long long tiles = 0;
  for (int mi = 0; mi < tiles_m; ++mi) tiles += tiles_n - TPR * mi > 0 ? tiles_n - TPR * mi : 0;
  if (tiles < 1 || tiles > 0x7fffffffLL) return DMRG_ERR_ARG;
  gram_digits_kernel<<<(unsigned)tiles, GRAM_THREADS, GRAM_SMEM, s>>>(ma[0], ma[1], ma[2], ma[3], ma[4], mb[0], mb[1],
                                                                      mb[2], mb[3], mb[4], Kp / GK, tiles_m, tiles_n,
                                                                      k, sigma, G, err);
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

}  // namespace dmrg
