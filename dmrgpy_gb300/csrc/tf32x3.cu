// Split-TF32 contraction path on the 5th-generation tensor cores (sm_103a).
//
// Every FP64 operand x is split into two TF32 values, hi = tf32(x) and
// lo = tf32(x - hi); a product is formed from three TF32 MMAs,
// A_hi.B_hi + A_hi.B_lo + A_lo.B_hi, accumulated in FP32 in TMEM (the
// lo.lo term is below FP32 resolution and dropped).  That gives FP32-level
// accuracy (~1e-7 relative) at tensor-core rate.  The same kernel runs FP16
// pairs of power-of-two scaled operands (kind::f16, the same 22-bit split),
// used by the polar iteration of the subspace truncation.
//
// GEMM kernel (C[M,N] = sum_k A[M,k] B[N,k], both operands K-major),
// persistent: one CTA per SM walks the output tiles b, b + gridDim.x, ...
//   warp 0   TMA producer: per stage (one 128-byte swizzle row of K: 32 tf32
//            or 64 fp16) loads the A_hi, A_lo, B_hi, B_lo tiles into a
//            shared-memory ring (SWIZZLE_128B), signalling an mbarrier with
//            the transaction byte count;
//   warp 1   allocates TMEM, then one thread issues tcgen05.mma.cta_group::1
//            (kind::tf32 K=8 or kind::f16 K=16; M=128, N=BNT or, merged,
//            one N=2 BNT MMA for A_hi.[B_hi; B_lo]) into a ring of TMEM
//            buffers, one per 32-wide K run, and tcgen05.commit's the stage
//            back to the producer and each buffer to the epilogue;
//   warps 2-5 epilogue: each thread owns one output row (its warp's 32-lane
//            TMEM quarter), adds every K run's buffer into FP32 registers,
//            and after the tile's last run stores FP32/FP64 with arbitrary
//            strides, or (polar iteration) FP64 plus the TF32/FP16 operand
//            pairs of the next GEMM.
// The stage and TMEM rings run on across tiles, so a tile's stores overlap
// the next tile's loads and MMAs.  All mbarrier waits are bounded
// (DMRG_ERR_TIMEOUT is recorded on expiry).
//
// Around the GEMMs: split kernels that produce the K-padded hi/lo operand
// arrays (optionally transposing), and the MPO-step kernel that contracts
// the two site MPO tensors into the GEMM1 output in one pass.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <atomic>
#include <map>
#include <mutex>

#include <cuda_fp16.h>

#include "tcgen05.cuh"
#include "tf32x3.cuh"

namespace dmrg {

namespace {

constexpr int BM = 128;     // accumulator rows = TMEM lanes
constexpr int BK = 32;      // fp32 per K-slice = 128 bytes = one SW128 row
// shared-memory stages: 3 x 64 KB for 128-wide tiles, 4 x 48 KB for
// 64-wide (a stage's TMA round trip is ~2 us under load, so the bytes in
// flight bound the K-slice rate)
template <int BNT> __host__ __device__ constexpr int stages_of() { return BNT == 64 ? 4 : 3; }
constexpr int TILE_A_BYTES = BM * BK * 4;   // 16 KB
// dynamic shared memory of the GEMM for an N-tile width of bnt columns
constexpr int gemm_smem_bytes(int bnt) {
  return (bnt == 64 ? 4 : 3) * (2 * TILE_A_BYTES + 2 * bnt * BK * 4) + 1024 + 256;
}
constexpr int GEMM_THREADS = 320;           // 10 warps: TMA producer, MMA issuer, 8 epilogue

// TF32 pair of an FP64 value: hi = x rounded to 11 significant bits, lo =
// (x - hi) rounded to 11 bits.  Built from the bit pattern with integer and
// FP32 operations: GB300 issues FP64 arithmetic and FP64 <-> FP32
// conversions at a small fraction of the FP32 rate, and the split of a
// chi=1024 two-site tensor (9.4M values) through them took ~70 us.  Values
// whose parts leave the FP32 normal range (|x| < 2^-126 or |x| >= 2^115,
// zero, inf, nan) take the conversion route.
__device__ __forceinline__ void split2(double x, float& hi, float& lo) {
  const uint32_t xh = static_cast<uint32_t>(__double2hiint(x));
  const uint32_t xl = static_cast<uint32_t>(__double2loint(x));
  const int e = static_cast<int>((xh >> 20) & 0x7ffu);   // biased FP64 exponent
  if (e < 897 || e > 1138) {
    hi = to_tf32(static_cast<float>(x));
    lo = to_tf32(static_cast<float>(x - static_cast<double>(hi)));
    return;
  }
  const uint32_t sgn = xh & 0x80000000u;
  const uint32_t mh = xh & 0xfffffu;        // fraction bits 51..32
  const uint32_t up = (mh >> 9) & 1u;       // round half away at fraction bit 41
  // a carry out of the 10 fraction bits moves into the exponent field
  hi = __uint_as_float(sgn | ((static_cast<uint32_t>(e - 896) << 23) + (((mh >> 10) + up) << 13)));
  // x - hi = (rh 2^32 + xl) 2^(e - 1075) with |rh 2^32 + xl| <= 2^41
  const int rh = static_cast<int>(mh & 0x3ffu) - static_cast<int>(up << 10);
  const float r = fmaf(static_cast<float>(rh), 4294967296.0f, static_cast<float>(xl));
  const float v = r * 5.42101086242752217e-20f * __uint_as_float(static_cast<uint32_t>(e - 884) << 23);
  lo = to_tf32(sgn ? -v : v);
}

// FP16 pair of x * scale (scale a power of two chosen so that |x * scale|
// stays below the FP16 maximum): hi = fp16(x s), lo = fp16(x s - hi)
__device__ __forceinline__ void split2h(double x, double scale, __half& hi, __half& lo) {
  const double v = x * scale;
  hi = __double2half(v);
  lo = __double2half(v - static_cast<double>(__half2float(hi)));
}

// the same pairs of an FP32 value (scale a power of two): x s - hi is exact
// in FP32, so the pair matches the FP64 route up to ties
__device__ __forceinline__ void split2h(float x, float scale, __half& hi, __half& lo) {
  const float v = x * scale;
  hi = __float2half_rn(v);
  lo = __float2half_rn(v - __half2float(hi));
}

__device__ __forceinline__ void split2(float x, float& hi, float& lo) {
  hi = to_tf32(x);
  lo = to_tf32(x - hi);
}

// Epilogue of the polar-iteration GEMMs (GemmOut with split outputs, a
// diagonal term or no C): v = alpha*acc + diag*[row == col] (+ C if
// accumulate), stored to C (FP64) if present and as TF32 hi/lo pairs,
// row-major and/or transposed.  It only stores (no loads unless it
// accumulates), so the stores of one tile overlap the next tile's MMAs; the
// transposed pairs are written by consecutive lanes (= consecutive rows)
// and so coalesce; the row-major ones use 16-byte stores where aligned.
template <int BNT, bool F16>
__device__ __forceinline__ void store_extra(const float* acc, const GemmOut& out, int gm, int n0) {
  double* C = static_cast<double*>(out.C);
  const long long crow = (long long)gm * out.ldm;
  const bool full = n0 + BNT <= out.N;
  const bool cvec = full && C && out.ldn == 1 && ((reinterpret_cast<uintptr_t>(C) & 15) == 0) && out.ldm % 2 == 0;
  // 4 split values per store: 16 bytes (tf32 pairs) or 8 bytes (fp16)
  const bool rvec = full && out.rhi && ((reinterpret_cast<uintptr_t>(out.rhi) & 15) == 0) &&
                    ((reinterpret_cast<uintptr_t>(out.rlo) & 15) == 0) && out.rld % 4 == 0;
  // FP64 values only where they carry more than the FP32 accumulator: an
  // accumulated C, or a diagonal term added to a stored C.  Otherwise the
  // value, its C copy and its splits come from FP32 arithmetic (the FP64
  // pipe of GB300 would otherwise bound this epilogue).
  const bool wide = out.accumulate || (C && out.diag != 0.0);
  const float diagf = static_cast<float>(out.diag);
  const float scalef = static_cast<float>(out.split_scale);
#pragma unroll
  for (int c = 0; c < BNT; c += 4) {
    double v[4];
    float vf[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (wide) {
        v[j] = static_cast<double>(out.alpha * acc[c + j]) + (n0 + c + j == gm ? out.diag : 0.0);
      } else {
        vf[j] = out.alpha * acc[c + j] + (n0 + c + j == gm ? diagf : 0.f);
        v[j] = widen(vf[j]);
      }
    }
    if (C) {
      if (cvec) {
        double2* p = reinterpret_cast<double2*>(C + crow + n0 + c);
        if (out.accumulate) {
          const double2 a = p[0], b = p[1];
          v[0] += a.x; v[1] += a.y; v[2] += b.x; v[3] += b.y;
        }
        p[0] = make_double2(v[0], v[1]);
        p[1] = make_double2(v[2], v[3]);
      } else {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int gn = n0 + c + j;
          if (gn < out.N) {
            const long long o = crow + (long long)gn * out.ldn;
            if (out.accumulate) v[j] += C[o];
            C[o] = v[j];
          }
        }
      }
    }
    if (out.rhi || out.thi) {
      if constexpr (F16) {
        __half h[4], l[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          if (wide) split2h(v[j], out.split_scale, h[j], l[j]);
          else split2h(vf[j], scalef, h[j], l[j]);
        }
        if (out.rhi) {
          __half* ph = static_cast<__half*>(out.rhi) + (long long)gm * out.rld + n0 + c;
          __half* pl = static_cast<__half*>(out.rlo) + (long long)gm * out.rld + n0 + c;
          if (rvec) {
            __half2 h01 = __halves2half2(h[0], h[1]), h23 = __halves2half2(h[2], h[3]);
            __half2 l01 = __halves2half2(l[0], l[1]), l23 = __halves2half2(l[2], l[3]);
            uint2 uh, ul;
            uh.x = *reinterpret_cast<uint32_t*>(&h01); uh.y = *reinterpret_cast<uint32_t*>(&h23);
            ul.x = *reinterpret_cast<uint32_t*>(&l01); ul.y = *reinterpret_cast<uint32_t*>(&l23);
            *reinterpret_cast<uint2*>(ph) = uh;
            *reinterpret_cast<uint2*>(pl) = ul;
          } else {
#pragma unroll
            for (int j = 0; j < 4; ++j)
              if (n0 + c + j < out.N) {
                ph[j] = h[j];
                pl[j] = l[j];
              }
          }
        }
        if (out.thi) {
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int gn = n0 + c + j;
            if (gn < out.N) {
              static_cast<__half*>(out.thi)[(long long)gn * out.tld + gm] = h[j];
              static_cast<__half*>(out.tlo)[(long long)gn * out.tld + gm] = l[j];
            }
          }
        }
      } else {
        float h[4], l[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          if (wide) split2(v[j], h[j], l[j]);
          else split2(vf[j], h[j], l[j]);
        }
        if (out.rhi) {
          float* ph = static_cast<float*>(out.rhi) + (long long)gm * out.rld + n0 + c;
          float* pl = static_cast<float*>(out.rlo) + (long long)gm * out.rld + n0 + c;
          if (rvec) {
            *reinterpret_cast<float4*>(ph) = make_float4(h[0], h[1], h[2], h[3]);
            *reinterpret_cast<float4*>(pl) = make_float4(l[0], l[1], l[2], l[3]);
          } else {
#pragma unroll
            for (int j = 0; j < 4; ++j)
              if (n0 + c + j < out.N) {
                ph[j] = h[j];
                pl[j] = l[j];
              }
          }
        }
        if (out.thi) {
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int gn = n0 + c + j;
            if (gn < out.N) {
              static_cast<float*>(out.thi)[(long long)gn * out.tld + gm] = h[j];
              static_cast<float*>(out.tlo)[(long long)gn * out.tld + gm] = l[j];
            }
          }
        }
      }
    }
  }
}

// The tensor-core FP32 accumulation is not round-to-nearest: summed over a
// long K its error grows linearly.  Each K-slice of 32 is therefore
// accumulated into its own TMEM buffer (a ring of NACC buffers) and
// the slice results are summed by the epilogue warps in FP32 registers with
// ordinary rounding, so the biased part spans at most 32 products.
// tile index -> origin in the grouped order: consecutive tile indices walk
// `group` M-tiles for each N-tile, so the tiles in flight at one time share
// their operand panels in L2 (group = tiles_m is plain M-fastest order)
__device__ __forceinline__ void tile_origin(int t, int tiles_m, int tiles_n, int group, int bnt, int& m0, int& n0) {
  const int per_group = group * tiles_n;
  const int gid = t / per_group;
  const int first_m = gid * group;
  const int gsz = min(tiles_m - first_m, group);
  const int local = t - gid * per_group;
  m0 = (first_m + local % gsz) * BM;
  n0 = (local / gsz) * bnt;
}

// Persistent: CTA b computes tiles b, b + gridDim.x, ...  The producer and
// MMA warps run through the K-slices of consecutive tiles without a break
// (the stage and TMEM rings continue across tiles), so loading and MMAs of
// the next tile overlap the epilogue's stores of the current one.
template <int BNT, bool EXTRA, bool F16, bool MERGE>
__global__ void __launch_bounds__(GEMM_THREADS, 1)
    tf32x3_gemm_kernel(const __grid_constant__ CUtensorMap mAhi, const __grid_constant__ CUtensorMap mAlo,
                       const __grid_constant__ CUtensorMap mBhi, const __grid_constant__ CUtensorMap mBlo, int KT,
                       int tiles_m, int tiles_n, int group, GemmOut out, int* err) {
  constexpr int TB_BYTES = BNT * BK * 4;                       // B tile
  constexpr int ST_BYTES = 2 * TILE_A_BYTES + 2 * TB_BYTES;    // one stage
  constexpr int STAGES = stages_of<BNT>();
  // fp16 operands: one 128-byte swizzle row is 64 K-elements, split into two
  // TMEM sub-slices of 32 so that the FP32 accumulation runs stay 32 long
  constexpr int KE = F16 ? 64 : 32;      // K-elements per stage
  constexpr int SUB = F16 ? 2 : 1;       // TMEM sub-slices per stage
  constexpr int KK_SUB = (BK / 8) / SUB; // MMA K-steps per sub-slice
  // MERGE issues A_hi.[B_hi; B_lo] as one N = 2 BNT MMA (two MMAs per
  // K-step instead of three: a single thread issues ~25 ns per MMA, about
  // as long as 12 MMAs of a stage take to execute); its TMEM buffers are
  // 2 BNT columns wide, so a 128-wide tile keeps two of them, not four
  constexpr int ACC_COLS = MERGE ? 2 * BNT : BNT;
  constexpr int NACC = (512 / ACC_COLS) < 4 ? (512 / ACC_COLS) : 4;   // TMEM ring of K-slice buffers
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * ST_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* acc_full = empty + STAGES;
  uint64_t* acc_empty = acc_full + NACC;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(acc_empty + NACC);

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int ntiles = tiles_m * tiles_n;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < NACC; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], 8);  // one arrival per epilogue warp
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(NACC * ACC_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      long long g = 0;   // K-slice counter over all tiles of this CTA
      bool ok = true;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        int m0, n0;
        tile_origin(t, tiles_m, tiles_n, group, BNT, m0, n0);
        for (int kt = 0; kt < KT; ++kt, ++g) {
          const int s = (int)(g % STAGES);
          const long long it = g / STAGES;
          if (g >= STAGES && !mbar_wait(&empty[s], (uint32_t)((it - 1) & 1), err)) {
            ok = false;
            break;
          }
          unsigned char* st = smem + s * ST_BYTES;
          mbar_expect_tx(&full[s], ST_BYTES);
          const int x = kt * KE;
          tma_load_2d(st, &mAhi, &full[s], x, m0);
          tma_load_2d(st + TILE_A_BYTES, &mAlo, &full[s], x, m0);
          tma_load_2d(st + 2 * TILE_A_BYTES, &mBhi, &full[s], x, n0);
          tma_load_2d(st + 2 * TILE_A_BYTES + TB_BYTES, &mBlo, &full[s], x, n0);
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = F16 ? idesc_f16(BM, BNT) : idesc_tf32(BM, BNT);
      constexpr uint32_t idesc2 = F16 ? idesc_f16(BM, 2 * BNT) : idesc_tf32(BM, 2 * BNT);
      long long g = 0;    // stage counter
      long long gs = 0;   // TMEM sub-slice counter
      bool ok = true;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        for (int kt = 0; kt < KT && ok; ++kt, ++g) {
          const int s = (int)(g % STAGES);
          const long long it = g / STAGES;
          if (!mbar_wait(&full[s], (uint32_t)(it & 1), err)) {
            ok = false;
            break;
          }
          // descriptors of the stage's four tiles at K-step 0; a K-step of 32
          // bytes adds 2 to the start-address field (address >> 4)
          const uint32_t base = smem_u32(smem + s * ST_BYTES);
          const uint64_t dah0 = sdesc_sw128(base), dal0 = sdesc_sw128(base + TILE_A_BYTES);
          const uint64_t dbh0 = sdesc_sw128(base + 2 * TILE_A_BYTES);
          const uint64_t dbl0 = sdesc_sw128(base + 2 * TILE_A_BYTES + TB_BYTES);
#pragma unroll
          for (int j = 0; j < SUB; ++j, ++gs) {
            const int b = (int)(gs % NACC);
            const long long u = gs / NACC;
            if (gs >= NACC && !mbar_wait(&acc_empty[b], (uint32_t)((u - 1) & 1), err)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t d = tmem + b * ACC_COLS;
#pragma unroll
            for (int kq = 0; kq < KK_SUB; ++kq) {
              // 32 bytes along K inside the swizzle row: 8 tf32 or 16 fp16
              const uint64_t o = (uint64_t)((j * KK_SUB + kq) * 2);
              if constexpr (MERGE) {
                // A_hi . [B_hi; B_lo] (N = 2 BNT: the two B tiles are adjacent
                // rows of one operand) into columns [0, 2 BNT), then A_lo . B_hi
                // into columns [0, BNT); the epilogue adds the two halves
                if constexpr (F16) {
                  mma_f16(d, dah0 + o, dbh0 + o, idesc2, kq != 0);
                  mma_f16(d, dal0 + o, dbh0 + o, idesc, 1u);
                } else {
                  mma_tf32(d, dah0 + o, dbh0 + o, idesc2, kq != 0);
                  mma_tf32(d, dal0 + o, dbh0 + o, idesc, 1u);
                }
              } else {
                if constexpr (F16) {
                  mma_f16(d, dah0 + o, dbh0 + o, idesc, kq != 0);
                  mma_f16(d, dah0 + o, dbl0 + o, idesc, 1u);
                  mma_f16(d, dal0 + o, dbh0 + o, idesc, 1u);
                } else {
                  mma_tf32(d, dah0 + o, dbh0 + o, idesc, kq != 0);
                  mma_tf32(d, dah0 + o, dbl0 + o, idesc, 1u);
                  mma_tf32(d, dal0 + o, dbh0 + o, idesc, 1u);
                }
              }
            }
            mma_commit(&acc_full[b]);
          }
          if (ok) mma_commit(&empty[s]);
        }
      }
    }
  } else {
    // epilogue: warps 2..9.  A warp reaches only the TMEM lane quarter
    // warp % 4, so two warps share each quarter (one row per thread) and
    // split the tile's columns: warps 2..5 the first BNT / 2, warps 6..9 the
    // rest.  Each K-slice buffer is thus drained by two warps in parallel,
    // and each warp stores half of the tile.
    constexpr int HB = BNT / 2;
    const int q = warp & 3;
    const int half = (warp - 2) >> 2;
    const int row = q * 32 + lane;
    long long g = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
      int m0, n0t;
      tile_origin(t, tiles_m, tiles_n, group, BNT, m0, n0t);
      const int n0 = n0t + half * HB;   // first output column of this warp
      // column pairs in 64-bit registers, summed with packed FP32 adds
      // (round to nearest per lane, as the scalar add): half the add
      // instructions, which share their issue slots with the MMA warp on one
      // SM sub-partition
      uint64_t acc2[HB / 2];
#pragma unroll
      for (int c = 0; c < HB / 2; ++c) acc2[c] = 0ull;
      for (int kt = 0; kt < KT * SUB && ok; ++kt, ++g) {
        const int b = (int)(g % NACC);
        const long long u = g / NACC;
        ok = mbar_wait(&acc_full[b], (uint32_t)(u & 1), err);
        tc_fence_after();
        if (ok) {
          // MERGE buffers hold A_hi.B_hi (+ A_lo.B_hi) in columns [0, BNT)
          // and A_hi.B_lo in [BNT, 2 BNT): both halves add into acc
#pragma unroll
          for (int grp = 0; grp < ACC_COLS / BNT; ++grp) {
            uint32_t v[HB];
            tmem_ld_cols<HB>(tmem + (static_cast<uint32_t>(q * 32) << 16) + b * ACC_COLS + grp * BNT + half * HB, v);
#pragma unroll
            for (int j = 0; j < HB; j += 2) add_f32x2(acc2[j / 2], v[j], v[j + 1]);
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&acc_empty[b])) : "memory");
      }
      float acc[HB];
#pragma unroll
      for (int c = 0; c < HB / 2; ++c) unpack_f32x2(acc2[c], acc[2 * c], acc[2 * c + 1]);
      if (!ok) break;
      const int gm = m0 + row;
      if constexpr (EXTRA) {
        if (gm < out.M) store_extra<HB, F16>(acc, out, gm, n0);
      } else {
      // full-width tiles of row-contiguous outputs are written with 16-byte
      // stores (4 floats / 2+2 doubles per step) instead of one element
      const bool inrow = ok && gm < out.M;
      // transposed FP32 overwrite (the matvec's X1): one coalesced 4-byte
      // store per element across the warp's consecutive rows, no branches
      const bool tstore = inrow && out.ldm == 1 && !out.out_f64 && !out.accumulate;
      if (tstore) {
        float* pc = static_cast<float*>(out.C) + gm + (long long)n0 * out.ldn;
        if (n0 + HB <= out.N) {
#pragma unroll
          for (int c = 0; c < HB; ++c) pc[(long long)c * out.ldn] = out.alpha * acc[c];
        } else {
#pragma unroll
          for (int c = 0; c < HB; ++c)
            if (n0 + c < out.N) pc[(long long)c * out.ldn] = out.alpha * acc[c];
        }
      }
      const bool vec = inrow && out.ldn == 1 && n0 + HB <= out.N &&
                       ((reinterpret_cast<uintptr_t>(out.C) & 15) == 0) &&
                       (out.out_f64 ? (out.ldm % 2 == 0) : (out.ldm % 4 == 0));
      if (inrow && !tstore) {
        const long long rowoff = (long long)gm * out.ldm;
#pragma unroll
        for (int c = 0; c < HB; c += 4) {
          const float r0 = out.alpha * acc[c], r1 = out.alpha * acc[c + 1];
          const float r2 = out.alpha * acc[c + 2], r3 = out.alpha * acc[c + 3];
          if (vec) {
            if (out.out_f64) {
              double2* p = reinterpret_cast<double2*>(static_cast<double*>(out.C) + rowoff + n0 + c);
              double2 u = make_double2(widen(r0), widen(r1)), v = make_double2(widen(r2), widen(r3));
              if (out.accumulate) {
                const double2 pu = p[0], pv = p[1];
                u.x += pu.x; u.y += pu.y; v.x += pv.x; v.y += pv.y;
              }
              p[0] = u;
              p[1] = v;
            } else {
              float4* p = reinterpret_cast<float4*>(static_cast<float*>(out.C) + rowoff + n0 + c);
              float4 u = make_float4(r0, r1, r2, r3);
              if (out.accumulate) {
                const float4 o = *p;
                u.x += o.x; u.y += o.y; u.z += o.z; u.w += o.w;
              }
              *p = u;
            }
          } else {
            const float rr[4] = {r0, r1, r2, r3};
#pragma unroll
            for (int j = 0; j < 4; ++j) {
              const int gn = n0 + c + j;
              if (gn < out.N) {
                const long long o = rowoff + (long long)gn * out.ldn;
                if (out.out_f64) {
                  double* C = static_cast<double*>(out.C);
                  C[o] = out.accumulate ? C[o] + widen(rr[j]) : widen(rr[j]);
                } else {
                  float* C = static_cast<float*>(out.C);
                  C[o] = out.accumulate ? C[o] + rr[j] : rr[j];
                }
              }
            }
          }
        }
      }
    }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(NACC * ACC_COLS));
  }
}

// ---------------------------------------------------------------- splitting

// out[r][k] (r < R, k < Kp) = split(in[r*ldr + k*ldk]) for k < K, 0 beyond.
template <typename Tin>
__global__ void split_kernel(const Tin* __restrict__ in, long long ldr, long long ldk, int R, int K, int Kp,
                             float* __restrict__ hi, float* __restrict__ lo) {
  const long long total = (long long)R * Kp;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
    const int r = (int)(i / Kp);
    const int k = (int)(i - (long long)r * Kp);
    float h = 0.f, l = 0.f;
    if (k < K) split2(static_cast<double>(in[(long long)r * ldr + (long long)k * ldk]), h, l);
    hi[i] = h;
    lo[i] = l;
  }
}

// Transposing split through a 32x33 shared tile:
// out[c][r] (c < C, r < Rp) = split(in[r*ld + c]) for r < R, 0 beyond.
__global__ void split_transpose_kernel(const double* __restrict__ in, long long ld, int R, int C, int Rp,
                                       float* __restrict__ hi, float* __restrict__ lo) {
  __shared__ double t[32][33];
  const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  for (int j = ty; j < 32; j += 8) {
    const int r = r0 + j, c = c0 + tx;
    t[j][tx] = (r < R && c < C) ? in[(long long)r * ld + c] : 0.0;
  }
  __syncthreads();
  for (int j = ty; j < 32; j += 8) {
    const int c = c0 + j, r = r0 + tx;
    if (c < C && r < Rp) {
      float h, l;
      split2(t[tx][j], h, l);
      hi[(long long)c * Rp + r] = h;
      lo[(long long)c * Rp + r] = l;
    }
  }
}

// Combined two-site MPO W2[(s',t',n)][(s,t,k)] = sum_m Wi[k,s,s',m] Wj[m,t,t',n]
__global__ void w2_kernel(const double* __restrict__ Wi, const double* __restrict__ Wj, int d1, int d2, int wl, int wm,
                          int wr, float* __restrict__ W2) {
  const int rows = d1 * d2 * wr, cols = d1 * d2 * wl;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < rows * cols; i += gridDim.x * blockDim.x) {
    const int r = i / cols, c = i - r * cols;
    const int sp = r / (d2 * wr), tp = (r / wr) % d2, n = r % wr;
    const int s = c / (d2 * wl), t = (c / wl) % d2, k = c % wl;
    double acc = 0.0;
    for (int m = 0; m < wm; ++m)
      acc += Wi[((k * d1 + s) * d1 + sp) * wm + m] * Wj[((m * d2 + t) * d2 + tp) * wr + n];
    W2[i] = static_cast<float>(acc);
  }
}

// MPO step of the two-site matvec:
//   X3[(a',s',t')][n*chir + b] = sum_{s,t,k} W2[(s',t',n)][(s,t,k)] X1[(s,t,b)][(a',k)]
// written as split TF32 (hi, lo) rows of padded length Kp.  A CTA takes 32
// consecutive b and AT consecutive a'; a warp's lanes walk b so the stores
// of a row are 128-byte coalesced.
constexpr int MID_AT = 4;
__global__ void __launch_bounds__(256) mpo_step_kernel(const float* __restrict__ X1, const float* __restrict__ W2,
                                                       int chil, int d1, int d2, int chir, int wl, int wr, int Kp,
                                                       float* __restrict__ hi, float* __restrict__ lo) {
  extern __shared__ float sm[];
  const int nst = d1 * d2;
  const int in_cols = nst * wl;   // (s,t,k)
  const int out_rows = nst * wr;  // (s',t',n)
  float* sW = sm;                              // out_rows x in_cols
  float* sX = sW + out_rows * in_cols;         // [a_local][(s,t,k)][b_local 32]
  const int b0 = blockIdx.x * 32;
  const int a0 = blockIdx.y * MID_AT;
  const long long ldx = (long long)chil * wl;
  for (int i = threadIdx.x; i < out_rows * in_cols; i += blockDim.x) sW[i] = W2[i];
  // load X1 rows (s,t,b) for the b tile, columns (a',k) for the a' tile
  const int ncolx = MID_AT * wl;
  for (int i = threadIdx.x; i < nst * 32 * ncolx; i += blockDim.x) {
    const int col = i % ncolx;
    const int bl = (i / ncolx) % 32;
    const int st = i / (ncolx * 32);
    const int al = col / wl, k = col % wl;
    const int b = b0 + bl, a = a0 + al;
    float v = 0.f;
    if (b < chir && a < chil) v = X1[((long long)st * chir + b) * ldx + (long long)a * wl + k];
    sX[(al * in_cols + st * wl + k) * 32 + bl] = v;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int b = b0 + lane;
  for (int row = warp; row < MID_AT * out_rows; row += 8) {
    const int al = row / out_rows, r = row % out_rows;
    const int a = a0 + al;
    if (a >= chil) continue;
    const float* w = sW + r * in_cols;
    const float* x = sX + (al * in_cols) * 32 + lane;
    float acc = 0.f;
    for (int c = 0; c < in_cols; ++c) acc = fmaf(w[c], x[c * 32], acc);
    if (b < chir) {
      const int sp_tp = r / wr, n = r % wr;
      const long long o = ((long long)a * nst + sp_tp) * Kp + (long long)n * chir + b;
      float h = to_tf32(acc);
      hi[o] = h;
      lo[o] = to_tf32(acc - h);
    }
  }
}

// Register-tiled form of the same step (d1 d2 wl <= 96): warp al of the CTA
// owns a' = a0+al, lane owns b = b0+lane; the thread keeps its (s,t,k) input
// column in registers and reads each MPO row as broadcast float4s from
// shared memory, so the loop is FMA-bound instead of shared-load-bound (one
// shared load per four FMAs).  MAXC >= (d1 d2 wl) rounded up to 4.
constexpr int RT_A = 8;

// It reads X1 transposed, X1T[(a',k)][(s,t,b)] (leading
// dimension d1 d2 chir), as GEMM1 stores it: a warp covers 32 consecutive b
// of one a', so each of its d1 d2 wl input loads is one coalesced 128-byte
// segment and the inputs go straight to registers, without the
// shared-memory staging that an untransposed X1 needs (it held such a kernel
// to 3 CTAs per SM, with loads and FMAs in separate phases).  W2 and the
// input offsets are in shared memory (broadcast reads).
template <int MAXC>
__global__ void __launch_bounds__(256) mpo_step_t_kernel(const float* __restrict__ X1T, const float* __restrict__ W2,
                                                         int chil, int d1, int d2, int chir, int wl, int wr, int Kp,
                                                         float* __restrict__ hi, float* __restrict__ lo) {
  extern __shared__ float4 sm4[];
  float* sW = reinterpret_cast<float*>(sm4);
  const int nst = d1 * d2;
  const int in_cols = nst * wl;
  const int out_rows = nst * wr;
  const int cpad = (in_cols + 3) & ~3;
  int* sOff = reinterpret_cast<int*>(sW + out_rows * cpad);   // MAXC input offsets
  const long long ldt = (long long)nst * chir;
  for (int i = threadIdx.x; i < out_rows * cpad; i += blockDim.x) {
    const int r = i / cpad, c = i - r * cpad;
    sW[i] = c < in_cols ? W2[r * in_cols + c] : 0.f;
  }
  for (int c = threadIdx.x; c < MAXC; c += blockDim.x) {
    const int st = c / wl, k = c - (c / wl) * wl;
    sOff[c] = c < in_cols ? (int)(k * ldt + (long long)st * chir) : -1;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int a = blockIdx.y * RT_A + (threadIdx.x >> 5), b = blockIdx.x * 32 + lane;
  if (a >= chil || b >= chir) return;
  const float* base = X1T + (long long)a * wl * ldt + b;
  float x[MAXC];
#pragma unroll
  for (int c = 0; c < MAXC; ++c) {
    const int off = sOff[c];
    x[c] = off >= 0 ? base[off] : 0.f;
  }
  for (int r = 0; r < out_rows; ++r) {
    const float4* w4 = reinterpret_cast<const float4*>(sW + r * cpad);
    float acc = 0.f;
#pragma unroll
    for (int c4 = 0; c4 < MAXC / 4; ++c4) {
      if (c4 * 4 < cpad) {
        const float4 w = w4[c4];
        acc = fmaf(w.x, x[4 * c4 + 0], acc);
        acc = fmaf(w.y, x[4 * c4 + 1], acc);
        acc = fmaf(w.z, x[4 * c4 + 2], acc);
        acc = fmaf(w.w, x[4 * c4 + 3], acc);
      }
    }
    const int sp_tp = r / wr, n = r - sp_tp * wr;
    const long long o = ((long long)a * nst + sp_tp) * Kp + (long long)n * chir + b;
    const float h = to_tf32(acc);
    hi[o] = h;
    lo[o] = to_tf32(acc - h);
  }
}

// Tensor-core form of the same step for d1 d2 wl <= 48 and d1 d2 wr <= 48
// (the S=1 bond: 45 x 45): per a' the step is the small GEMM
// X3_a (out x b) = W2 (out x in) X1_a (in x b), run on legacy mma.sync
// m16n8k8 TF32 tiles with the three split products (W2_hi X_hi + W2_hi X_lo
// + W2_lo X_hi) accumulated in FP32.  The CUDA-core form above issues
// 2025 FMAs and 506 shared loads per output column and sits at ~80% of the
// SM's issue rate with the HBM at a quarter of its bandwidth; here a warp
// covers one a' and 32 columns b (3 x 4 output tiles, 6 K steps, 216 MMAs),
// W2 split once per CTA into shared memory.  Fragment layouts (PTX ISA,
// mma.m16n8k8 .tf32): A a0 (g, t) a1 (g+8, t) a2 (g, t+4) a3 (g+8, t+4);
// B b0 (t, g) b1 (t+4, g); C c0 (g, 2t) c1 (g, 2t+1) c2 (g+8, 2t)
// c3 (g+8, 2t+1), with g = lane / 4 and t = lane % 4.
constexpr int MMA_K = 48;            // padded in/out width

__device__ __forceinline__ void mma_tf32_16x8x8(float* c, const uint32_t* a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__global__ void __launch_bounds__(256, 3) mpo_step_mma_kernel(const float* __restrict__ X1T,
                                                          const float* __restrict__ W2, int chil, int d1, int d2,
                                                          int chir, int wl, int wr, int Kp, int pair_stores,
                                                          float* __restrict__ hi, float* __restrict__ lo) {
  // W2 hi/lo in fragment order: entry (mt * 6 + kt) * 32 + lane holds that
  // lane's a0..a3 of m-tile mt, k-tile kt, so one 16-byte load per fragment
  __shared__ float4 sAh[3 * 6 * 32];
  __shared__ float4 sAl[3 * 6 * 32];
  __shared__ int sOff[MMA_K];   // input column -> offset in X1T (-1: padding)
  __shared__ int sOut[MMA_K];   // output row -> offset in the X3 row of a' (-1: padding)
  const int nst = d1 * d2;
  const int in_cols = nst * wl;
  const int out_rows = nst * wr;
  const long long ldt = (long long)nst * chir;
  for (int i = threadIdx.x; i < 3 * 6 * 32; i += blockDim.x) {
    const int f = i >> 5, l = i & 31;
    const int mt = f / 6, kt = f - (f / 6) * 6;
    const int r0 = 16 * mt + (l >> 2), c0 = 8 * kt + (l & 3);
    float w[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int r = r0 + (j & 1) * 8, c = c0 + (j >> 1) * 4;
      w[j] = (r < out_rows && c < in_cols) ? W2[r * in_cols + c] : 0.f;
    }
    float4 h, q;
    h.x = to_tf32(w[0]); q.x = to_tf32(w[0] - h.x);
    h.y = to_tf32(w[1]); q.y = to_tf32(w[1] - h.y);
    h.z = to_tf32(w[2]); q.z = to_tf32(w[2] - h.z);
    h.w = to_tf32(w[3]); q.w = to_tf32(w[3] - h.w);
    sAh[i] = h;
    sAl[i] = q;
  }
  for (int c = threadIdx.x; c < MMA_K; c += blockDim.x) {
    const int st = c / wl, k = c - (c / wl) * wl;
    sOff[c] = c < in_cols ? (int)(k * ldt + (long long)st * chir) : -1;
    const int sp_tp = c / wr, n = c - (c / wr) * wr;
    sOut[c] = c < out_rows ? sp_tp * Kp + n * chir : -1;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int g = lane >> 2, t = lane & 3;
  const int a = blockIdx.y * RT_A + (threadIdx.x >> 5);
  const int b0 = blockIdx.x * 32;
  if (a >= chil) return;
  const float* base = X1T + (long long)a * wl * ldt + b0;
  float acc[3][4][4];
#pragma unroll
  for (int mt = 0; mt < 3; ++mt)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[mt][nt][q] = 0.f;
#pragma unroll 1
  for (int kt = 0; kt < MMA_K / 8; ++kt) {
    const int off0 = sOff[8 * kt + t], off1 = sOff[8 * kt + t + 4];
    uint32_t bh[4][2], bl[4][2];
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
      const int col = 8 * nt + g;
      const bool ok = b0 + col < chir;
      const float x0 = (ok && off0 >= 0) ? base[off0 + col] : 0.f;
      const float x1 = (ok && off1 >= 0) ? base[off1 + col] : 0.f;
      const float h0 = to_tf32(x0), h1 = to_tf32(x1);
      bh[nt][0] = __float_as_uint(h0);
      bh[nt][1] = __float_as_uint(h1);
      bl[nt][0] = __float_as_uint(to_tf32(x0 - h0));
      bl[nt][1] = __float_as_uint(to_tf32(x1 - h1));
    }
#pragma unroll
    for (int mt = 0; mt < 3; ++mt) {
      const float4 fh = sAh[(mt * 6 + kt) * 32 + lane];
      const float4 fl = sAl[(mt * 6 + kt) * 32 + lane];
      const uint32_t ah[4] = {__float_as_uint(fh.x), __float_as_uint(fh.y), __float_as_uint(fh.z),
                              __float_as_uint(fh.w)};
      const uint32_t al[4] = {__float_as_uint(fl.x), __float_as_uint(fl.y), __float_as_uint(fl.z),
                              __float_as_uint(fl.w)};
#pragma unroll
      for (int nt = 0; nt < 4; ++nt) {
        mma_tf32_16x8x8(acc[mt][nt], ah, bh[nt][0], bh[nt][1]);
        mma_tf32_16x8x8(acc[mt][nt], ah, bl[nt][0], bl[nt][1]);
        mma_tf32_16x8x8(acc[mt][nt], al, bh[nt][0], bh[nt][1]);
      }
    }
  }
  // c0/c1 (and c2/c3) are neighbouring columns b, b + 1 of one output row
  const long long arow = (long long)a * nst * Kp;
#pragma unroll
  for (int mt = 0; mt < 3; ++mt)
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int ro = sOut[16 * mt + g + 8 * half];
      if (ro < 0) continue;
#pragma unroll
      for (int nt = 0; nt < 4; ++nt) {
        const int b = b0 + 8 * nt + 2 * t;
        if (b >= chir) continue;
        const long long o = arow + ro + b;
        const float v0 = acc[mt][nt][2 * half], v1 = acc[mt][nt][2 * half + 1];
        const float h0 = to_tf32(v0), h1 = to_tf32(v1);
        if (pair_stores && b + 1 < chir) {
          *reinterpret_cast<float2*>(hi + o) = make_float2(h0, h1);
          *reinterpret_cast<float2*>(lo + o) = make_float2(to_tf32(v0 - h0), to_tf32(v1 - h1));
        } else {
          hi[o] = h0;
          lo[o] = to_tf32(v0 - h0);
          if (b + 1 < chir) {
            hi[o + 1] = h1;
            lo[o + 1] = to_tf32(v1 - h1);
          }
        }
      }
    }
}

inline int egrid(long long n) {
  long long g = (n + 255) / 256;
  if (g > 152 * 16) g = 152 * 16;
  if (g < 1) g = 1;
  return (int)g;
}

inline int pad32(long long x) { return (int)((x + 31) / 32 * 32); }

// ---------------------------------------------------------------- host side
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

int get_encoder() {
  if (g_encode) return DMRG_OK;
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || fn == nullptr)
    return DMRG_ERR_CUDA;
  g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  return DMRG_OK;
}

// 2D row-major [rows][Kp] operand, box = (one 128-byte row, box_rows),
// SWIZZLE_128B: fp32 (32 per row, Kp % 32 == 0) or fp16 (64 per row,
// Kp % 64 == 0)
int make_map(CUtensorMap* m, const void* base, int rows, int Kp, int box_rows, bool f16 = false) {
  const int ke = f16 ? 64 : BK, es = f16 ? 2 : 4;
  if ((reinterpret_cast<uintptr_t>(base) & 15) != 0 || (Kp % ke) != 0) return DMRG_ERR_ARG;
  cuuint64_t dims[2] = {(cuuint64_t)Kp, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)Kp * es};
  cuuint32_t box[2] = {(cuuint32_t)ke, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(m, f16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                        const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? DMRG_OK : DMRG_ERR_ARG;
}


// C (M x N) = A (M x Kp) . B (N x Kp)^T from split operands.
// ---------------------------------------------------------------- tile-order tuner
// Decisions per (device, M, N, Kp) of the split GEMM: the shapes of one
// sweep are functions of (chi_l, chi_r, d, w), so a sweep tunes each of its
// few shapes once.
struct TuneKey {
  int dev, M, N, K, f16;
  bool operator<(const TuneKey& o) const {
    if (dev != o.dev) return dev < o.dev;
    if (f16 != o.f16) return f16 < o.f16;
    if (M != o.M) return M < o.M;
    if (N != o.N) return N < o.N;
    return K < o.K;
  }
};
struct TuneVal {
  int bnt;
  int merge;
  int group;
  float ms;
};
std::mutex g_tune_mu;
std::map<TuneKey, TuneVal> g_tune;
std::atomic<int> g_tune_on{1};

TuneKey tune_key(int M, int N, int K, bool f16) {
  int dev = 0;
  cudaGetDevice(&dev);
  return TuneKey{dev, M, N, K, f16 ? 1 : 0};
}
bool tune_enabled() { return g_tune_on.load() != 0; }
struct GemmCfg;
bool tune_lookup(const TuneKey& k, GemmCfg* cfg);
void tune_store(const TuneKey& k, const GemmCfg& cfg, float ms);

// Launch configuration of one split GEMM: N-tile width (128 or 64 columns),
// whether the two B splits go into one MMA, and grouped tile order.
struct GemmCfg {
  int bnt;
  int merge;
  int group;
};

bool tune_lookup(const TuneKey& k, GemmCfg* cfg) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  auto it = g_tune.find(k);
  if (it == g_tune.end()) return false;
  *cfg = GemmCfg{it->second.bnt, it->second.merge, it->second.group};
  return true;
}
void tune_store(const TuneKey& k, const GemmCfg& cfg, float ms) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune[k] = TuneVal{cfg.bnt, cfg.merge, cfg.group, ms};
}

// multiprocessor count of the current device (cached per device)
int sm_count() {
  static std::atomic<int> cache[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return 0;
  if (dev < 64) {
    const int c = cache[dev].load();
    if (c > 0) return c;
  }
  int n = 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  if (dev < 64) cache[dev].store(n);
  return n;
}

template <int BNT, bool EXTRA, bool F16, bool MERGE>
int gemm_launch_t(const CUtensorMap& mah, const CUtensorMap& mal, const void* Bhi, const void* Blo, int M, int N,
                  int Kp, int group, const GemmOut& out, int* err, cudaStream_t s) {
  static std::atomic<unsigned long long> attr{0};
  DMRG_TRY(smem_attr_once(reinterpret_cast<const void*>(tf32x3_gemm_kernel<BNT, EXTRA, F16, MERGE>),
                          gemm_smem_bytes(BNT), attr));
  CUtensorMap mbh, mbl;
  DMRG_TRY(make_map(&mbh, Bhi, N, Kp, BNT, F16));
  DMRG_TRY(make_map(&mbl, Blo, N, Kp, BNT, F16));
  const int tiles_m = (M + BM - 1) / BM, tiles_n = (N + BNT - 1) / BNT;
  const long long tiles = (long long)tiles_m * tiles_n;
  if (tiles > 0x7fffffffLL) return DMRG_ERR_ARG;
  const int g = group < 1 ? 1 : (group > tiles_m ? tiles_m : group);
  // persistent CTAs: one per SM (the shared-memory stages allow no second)
  const int nsm = sm_count();
  if (nsm < 1) return DMRG_ERR_CUDA;
  const long long grid = tiles < nsm ? tiles : nsm;
  tf32x3_gemm_kernel<BNT, EXTRA, F16, MERGE><<<(unsigned)grid, GEMM_THREADS, gemm_smem_bytes(BNT), s>>>(
      mah, mal, mbh, mbl, Kp / (F16 ? 64 : BK), tiles_m, tiles_n, g, out, err);
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

template <bool F16>
int gemm_launch_cfg(int bnt, int merge, bool extra, const CUtensorMap& mah, const CUtensorMap& mal, const void* Bhi,
                    const void* Blo, int M, int N, int Kp, int group, const GemmOut& out, int* err, cudaStream_t s) {
  // 64-wide tiles always merge; 128-wide tiles either way (tuned)
  if (bnt == 64)
    return extra ? gemm_launch_t<64, true, F16, true>(mah, mal, Bhi, Blo, M, N, Kp, group, out, err, s)
                 : gemm_launch_t<64, false, F16, true>(mah, mal, Bhi, Blo, M, N, Kp, group, out, err, s);
  if (merge)
    return extra ? gemm_launch_t<128, true, F16, true>(mah, mal, Bhi, Blo, M, N, Kp, group, out, err, s)
                 : gemm_launch_t<128, false, F16, true>(mah, mal, Bhi, Blo, M, N, Kp, group, out, err, s);
  return extra ? gemm_launch_t<128, true, F16, false>(mah, mal, Bhi, Blo, M, N, Kp, group, out, err, s)
               : gemm_launch_t<128, false, F16, false>(mah, mal, Bhi, Blo, M, N, Kp, group, out, err, s);
}

int gemm_split(const void* Ahi, const void* Alo, const void* Bhi, const void* Blo, int M, int N, int Kp,
               const GemmOut& out, int* err, cudaStream_t s, bool f16 = false) {
  DMRG_TRY(get_encoder());
  CUtensorMap mah, mal;
  DMRG_TRY(make_map(&mah, Ahi, M, Kp, BM, f16));
  DMRG_TRY(make_map(&mal, Alo, M, Kp, BM, f16));
  const bool extra = out.rhi || out.thi || !out.C || out.diag != 0.0;
  if (extra && !out.out_f64) return DMRG_ERR_ARG;
  auto launch = [&](const GemmCfg& c) -> int {
    return f16 ? gemm_launch_cfg<true>(c.bnt, c.merge, extra, mah, mal, Bhi, Blo, M, N, Kp, c.group, out, err, s)
               : gemm_launch_cfg<false>(c.bnt, c.merge, extra, mah, mal, Bhi, Blo, M, N, Kp, c.group, out, err, s);
  };
  const int tiles_m = (M + BM - 1) / BM;
  GemmCfg cfg{128, 0, tiles_m};
  // Tile width and order are tuned per GEMM shape on its first
  // overwrite-mode call (re-running an overwrite GEMM reproduces its output
  // bit for bit: every output element sums the same K slices in the same
  // order whatever the tiling); accumulate-mode calls use the decision for
  // their shape if one exists, else 128-wide tiles in plain order.
  const TuneKey key = tune_key(M, N, Kp, f16);
  if (!tune_lookup(key, &cfg)) {
    cfg = GemmCfg{128, 0, tiles_m};
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    DMRG_CUDA_TRY(cudaStreamIsCapturing(s, &cap));
    const long long tiles128 = (long long)tiles_m * ((N + 127) / 128);
    if (tune_enabled() && !out.accumulate && cap == cudaStreamCaptureStatusNone && tiles128 >= 48) {
      const GemmCfg cand[9] = {{128, 0, tiles_m}, {128, 0, 16}, {128, 0, 8}, {128, 1, tiles_m}, {128, 1, 16},
                               {128, 1, 8},       {64, 1, tiles_m}, {64, 1, 16}, {64, 1, 8}};
      float best = 0.f;
      bool have = false;
      cudaEvent_t e0, e1;
      DMRG_CUDA_TRY(cudaEventCreate(&e0));
      DMRG_CUDA_TRY(cudaEventCreate(&e1));
      for (int i = 0; i < 9; ++i) {
        GemmCfg c = cand[i];
        if (c.group > tiles_m) c.group = tiles_m;
        if (i % 3 != 0 && c.group == tiles_m) continue;   // same as the plain order
        DMRG_TRY(launch(c));  // warm
        DMRG_CUDA_TRY(cudaEventRecord(e0, s));
        DMRG_TRY(launch(c));
        DMRG_CUDA_TRY(cudaEventRecord(e1, s));
        DMRG_CUDA_TRY(cudaEventSynchronize(e1));
        float ms = 0.f;
        DMRG_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
        if (!have || ms < best) {
          best = ms;
          cfg = c;
          have = true;
        }
      }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      tune_store(key, cfg, best);
    }
  }
  return launch(cfg);
}

int split_rows(const double* in, long long ldr, long long ldk, int R, int K, int Kp, float* hi, float* lo,
               cudaStream_t s) {
  split_kernel<double><<<egrid((long long)R * Kp), 256, 0, s>>>(in, ldr, ldk, R, K, Kp, hi, lo);
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

int split_transpose(const double* in, long long ld, int R, int C, int Rp, float* hi, float* lo, cudaStream_t s) {
  dim3 grid((C + 31) / 32, (Rp + 31) / 32);
  if (grid.y > 65535) return DMRG_ERR_ARG;
  split_transpose_kernel<<<grid, 256, 0, s>>>(in, ld, R, C, Rp, hi, lo);
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

// ---------------------------------------------------------------- two-site matvec plan
struct Heff2Plan {
  int cl, d1, d2, cr, wl, wm, wr;
  int Kp1, Kp4;
  long long M1, N1, M4;
  float *thT_hi, *thT_lo, *L_hi, *L_lo, *X1, *X3_hi, *X3_lo, *R_hi, *R_lo, *W2;
  int* err;
  size_t bytes;
};

Heff2Plan plan2(const dmrg_heff_t& o, void* work) {
  Heff2Plan p;
  p.cl = o.chil; p.d1 = o.d1; p.d2 = o.d2; p.cr = o.chir; p.wl = o.wl; p.wm = o.wm; p.wr = o.wr;
  p.Kp1 = pad32(p.cl);
  p.Kp4 = pad32((long long)p.wr * p.cr);
  p.M1 = (long long)p.d1 * p.d2 * p.cr;
  p.N1 = (long long)p.cl * p.wl;
  p.M4 = (long long)p.cl * p.d1 * p.d2;
  char* b = static_cast<char*>(work);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    void* q = b ? b + off : nullptr;
    off += align_up(bytes, 1024);
    return q;
  };
  p.err = static_cast<int*>(take(256));
  p.W2 = static_cast<float*>(take(sizeof(float) * (size_t)p.d1 * p.d2 * p.wr * p.d1 * p.d2 * p.wl));
  p.L_hi = static_cast<float*>(take(sizeof(float) * p.N1 * p.Kp1));
  p.L_lo = static_cast<float*>(take(sizeof(float) * p.N1 * p.Kp1));
  p.R_hi = static_cast<float*>(take(sizeof(float) * (size_t)p.cr * p.Kp4));
  p.R_lo = static_cast<float*>(take(sizeof(float) * (size_t)p.cr * p.Kp4));
  p.thT_hi = static_cast<float*>(take(sizeof(float) * p.M1 * p.Kp1));
  p.thT_lo = static_cast<float*>(take(sizeof(float) * p.M1 * p.Kp1));
  p.X1 = static_cast<float*>(take(sizeof(float) * p.M1 * p.N1));
  p.X3_hi = static_cast<float*>(take(sizeof(float) * p.M4 * p.Kp4));
  p.X3_lo = static_cast<float*>(take(sizeof(float) * p.M4 * p.Kp4));
  p.bytes = off;
  return p;
}

template <int MAXC>
int launch_mpo_step_t(const Heff2Plan& p, cudaStream_t s) {
  const int nst = p.d1 * p.d2;
  const int cpad = (nst * p.wl + 3) & ~3;
  const size_t smem = sizeof(float) * (size_t)nst * p.wr * cpad + sizeof(int) * MAXC;
  if (smem > 200 * 1024) return DMRG_ERR_UNSUPPORTED;
  static std::atomic<unsigned long long> attr{0};
  DMRG_TRY(smem_attr_once(reinterpret_cast<const void*>(mpo_step_t_kernel<MAXC>), 200 * 1024, attr));
  dim3 grid((p.cr + 31) / 32, (p.cl + RT_A - 1) / RT_A);
  if (grid.y > 65535) return DMRG_ERR_ARG;
  mpo_step_t_kernel<MAXC><<<grid, 256, smem, s>>>(p.X1, p.W2, p.cl, p.d1, p.d2, p.cr, p.wl, p.wr, p.Kp4, p.X3_hi,
                                                  p.X3_lo);
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

int launch_mpo_step_mma(const Heff2Plan& p, cudaStream_t s) {
  dim3 grid((p.cr + 31) / 32, (p.cl + RT_A - 1) / RT_A);
  if (grid.y > 65535) return DMRG_ERR_ARG;
  // paired 8-byte stores need even offsets: chir, Kp even and 8-byte aligned bases
  const int pair = ((p.cr | p.Kp4) & 1) == 0 && (reinterpret_cast<uintptr_t>(p.X3_hi) & 7) == 0 &&
                   (reinterpret_cast<uintptr_t>(p.X3_lo) & 7) == 0;
  mpo_step_mma_kernel<<<grid, 256, 0, s>>>(p.X1, p.W2, p.cl, p.d1, p.d2, p.cr, p.wl, p.wr, p.Kp4, pair, p.X3_hi,
                                           p.X3_lo);
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

}  // namespace

int tf32x3_gemm_split(const float* Ahi, const float* Alo, const float* Bhi, const float* Blo, int M, int N, int Kp,
                      const GemmOut& out, int* err, cudaStream_t s) {
  return gemm_split(Ahi, Alo, Bhi, Blo, M, N, Kp, out, err, s, false);
}

int f16x3_gemm_split(const void* Ahi, const void* Alo, const void* Bhi, const void* Blo, int M, int N, int Kp,
                     const GemmOut& out, int* err, cudaStream_t s) {
  return gemm_split(Ahi, Alo, Bhi, Blo, M, N, Kp, out, err, s, true);
}

int tma_map_k64h(CUtensorMap* m, const void* base, int rows, int Kp, int box_rows) {
  DMRG_TRY(get_encoder());
  return make_map(m, base, rows, Kp, box_rows, true);
}

int tf32x3_split_rows(const double* in, long long ld, int R, int K, int Kp, float* hi, float* lo, cudaStream_t s) {
  return split_rows(in, ld, 1, R, K, Kp, hi, lo, s);
}

int tf32x3_split_transpose(const double* in, long long ld, int R, int C, int Rp, float* hi, float* lo,
                           cudaStream_t s) {
  return split_transpose(in, ld, R, C, Rp, hi, lo, s);
}

int tma_map_k32(CUtensorMap* m, const float* base, int rows, int Kp, int box_rows) {
  DMRG_TRY(get_encoder());
  return make_map(m, base, rows, Kp, box_rows);
}

size_t tf32x3_heff_workspace_bytes(const dmrg_heff_t& o) {
  if (o.kind != 2) return 0;
  return plan2(o, nullptr).bytes;
}

int tf32x3_heff_prepare(const dmrg_heff_t& o, void* work, cudaStream_t s) {
  if (o.kind != 2 || o.dtype != DMRG_REAL64) return DMRG_ERR_UNSUPPORTED;
  Heff2Plan p = plan2(o, work);
  DMRG_CUDA_TRY(cudaMemsetAsync(p.err, 0, 256, s));
  const int w2n = p.d1 * p.d2 * p.wr * p.d1 * p.d2 * p.wl;
  w2_kernel<<<(w2n + 255) / 256, 256, 0, s>>>(static_cast<const double*>(o.W1), static_cast<const double*>(o.W2),
                                              p.d1, p.d2, p.wl, p.wm, p.wr, p.W2);
  DMRG_CHECK_LAUNCH();
  // L (cl, wl, cl) as rows (a',k), K = a
  DMRG_TRY(split_rows(static_cast<const double*>(o.L), p.cl, 1, (int)p.N1, p.cl, p.Kp1, p.L_hi, p.L_lo, s));
  // R (cr, wr, cr) as rows b', K = (n, b)
  DMRG_TRY(split_rows(static_cast<const double*>(o.R), (long long)p.wr * p.cr, 1, p.cr, p.wr * p.cr, p.Kp4, p.R_hi,
                      p.R_lo, s));
  // padding columns of X3 stay zero for every later matvec
  DMRG_CUDA_TRY(cudaMemsetAsync(p.X3_hi, 0, sizeof(float) * p.M4 * p.Kp4, s));
  DMRG_CUDA_TRY(cudaMemsetAsync(p.X3_lo, 0, sizeof(float) * p.M4 * p.Kp4, s));
  return DMRG_OK;
}

int mpo_step_generic(const Heff2Plan& p, cudaStream_t s);

int tf32x3_heff_apply_prepared(const dmrg_heff_t& o, const double* x, double* y, void* work, cudaStream_t s) {
  Heff2Plan p = plan2(o, work);
  // theta (cl, d1 d2 cr) -> thetaT rows (s,t,b), K = a
  DMRG_TRY(split_transpose(x, p.M1, p.cl, (int)p.M1, p.Kp1, p.thT_hi, p.thT_lo, s));
  const int nst = p.d1 * p.d2;
  const int in_cols = nst * p.wl;
  if (in_cols <= 96) {
    // X1 stored transposed, X1T[(a',k)][(s,t,b)]: the epilogue's stores
    // coalesce across lanes (consecutive rows) and so do the MPO step's loads
    GemmOut g1{p.X1, 1, p.M1, (int)p.M1, (int)p.N1, 0, 0, 1.f};
    DMRG_TRY(gemm_split(p.thT_hi, p.thT_lo, p.L_hi, p.L_lo, (int)p.M1, (int)p.N1, p.Kp1, g1, p.err, s));
    if (in_cols <= MMA_K && nst * p.wr <= MMA_K) DMRG_TRY(launch_mpo_step_mma(p, s));
    else if (in_cols <= 48) DMRG_TRY(launch_mpo_step_t<48>(p, s));
    else DMRG_TRY(launch_mpo_step_t<96>(p, s));
  } else {
    GemmOut g1{p.X1, p.N1, 1, (int)p.M1, (int)p.N1, 0, 0, 1.f};
    DMRG_TRY(gemm_split(p.thT_hi, p.thT_lo, p.L_hi, p.L_lo, (int)p.M1, (int)p.N1, p.Kp1, g1, p.err, s));
    DMRG_TRY(mpo_step_generic(p, s));
  }
  GemmOut g4{y, p.cr, 1, (int)p.M4, p.cr, 1, 0, 1.f};
  DMRG_TRY(gemm_split(p.X3_hi, p.X3_lo, p.R_hi, p.R_lo, (int)p.M4, p.cr, p.Kp4, g4, p.err, s));
  return DMRG_OK;
}

// the shared-memory form for wide MPO steps (d1 d2 wl > 96)
int mpo_step_generic(const Heff2Plan& p, cudaStream_t s) {
  const int nst = p.d1 * p.d2;
  const size_t smem = sizeof(float) * ((size_t)nst * p.wr * nst * p.wl + (size_t)MID_AT * nst * p.wl * 32);
  if (smem > 200 * 1024) return DMRG_ERR_UNSUPPORTED;
  static std::atomic<unsigned long long> attr{0};
  DMRG_TRY(smem_attr_once(reinterpret_cast<const void*>(mpo_step_kernel), 200 * 1024, attr));
  dim3 grid((p.cr + 31) / 32, (p.cl + MID_AT - 1) / MID_AT);
  if (grid.y > 65535) return DMRG_ERR_ARG;
  mpo_step_kernel<<<grid, 256, smem, s>>>(p.X1, p.W2, p.cl, p.d1, p.d2, p.cr, p.wl, p.wr, p.Kp4, p.X3_hi, p.X3_lo);
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

int tf32x3_heff_status(const dmrg_heff_t& o, void* work, cudaStream_t s) {
  Heff2Plan p = plan2(o, work);
  int h = 0;
  DMRG_CUDA_TRY(cudaMemcpyAsync(&h, p.err, sizeof(int), cudaMemcpyDeviceToHost, s));
  DMRG_CUDA_TRY(cudaStreamSynchronize(s));
  return h;
}

int tf32x3_heff_apply(const dmrg_heff_t& o, const double* x, double* y, void* work, cudaStream_t s) {
  DMRG_TRY(tf32x3_heff_prepare(o, work, s));
  DMRG_TRY(tf32x3_heff_apply_prepared(o, x, y, work, s));
  return tf32x3_heff_status(o, work, s);
}

// ---------------------------------------------------------------- general GEMM
// C (m x n, ldc) (+)= alpha * op(A) op(B); op(A) is m x k, op(B) is k x n.
// A stored row-major with leading dim lda: transA=0 -> A[i*lda + kk],
// transA=1 -> A[kk*lda + i].  B likewise: transB=0 -> B[kk*ldb + j],
// transB=1 -> B[j*ldb + kk].
size_t tf32x3_gemm_ex_workspace_bytes(int m, int n, int k) {
  const size_t Kp = pad32(k);
  return align_up(256, 1024) + 2 * align_up(sizeof(float) * (size_t)m * Kp, 1024) +
         2 * align_up(sizeof(float) * (size_t)n * Kp, 1024);
}

int tf32x3_gemm_ex(int transA, int transB, int m, int n, int k, float alpha, const double* A, long long lda,
                   const double* B, long long ldb, int accumulate, double* C, long long ldc, void* work, int* err,
                   cudaStream_t s) {
  const int Kp = pad32(k);
  char* b = static_cast<char*>(work) + align_up(256, 1024);
  float* ahi = reinterpret_cast<float*>(b); b += align_up(sizeof(float) * (size_t)m * Kp, 1024);
  float* alo = reinterpret_cast<float*>(b); b += align_up(sizeof(float) * (size_t)m * Kp, 1024);
  float* bhi = reinterpret_cast<float*>(b); b += align_up(sizeof(float) * (size_t)n * Kp, 1024);
  float* blo = reinterpret_cast<float*>(b);
  if (!transA) DMRG_TRY(split_rows(A, lda, 1, m, k, Kp, ahi, alo, s));
  else DMRG_TRY(split_transpose(A, lda, k, m, Kp, ahi, alo, s));
  if (transB) DMRG_TRY(split_rows(B, ldb, 1, n, k, Kp, bhi, blo, s));
  else DMRG_TRY(split_transpose(B, ldb, k, n, Kp, bhi, blo, s));
  GemmOut g{C, ldc, 1, m, n, 1, accumulate, alpha};
  return gemm_split(ahi, alo, bhi, blo, m, n, Kp, g, err, s);
}

// ---------------------------------------------------------------- plain GEMM (merges)
size_t tf32x3_gemm_workspace_bytes(int m, int k, int n) {
  const size_t Kp = pad32(k);
  return align_up(256, 1024) + 2 * align_up(sizeof(float) * (size_t)m * Kp, 1024) +
         2 * align_up(sizeof(float) * (size_t)n * Kp, 1024);
}

int tf32x3_gemm(int m, int k, int n, const double* A, const double* B, double* C, void* work, cudaStream_t s) {
  const int Kp = pad32(k);
  char* b = static_cast<char*>(work);
  int* err = reinterpret_cast<int*>(b);
  b += align_up(256, 1024);
  float* ahi = reinterpret_cast<float*>(b); b += align_up(sizeof(float) * (size_t)m * Kp, 1024);
  float* alo = reinterpret_cast<float*>(b); b += align_up(sizeof(float) * (size_t)m * Kp, 1024);
  float* bhi = reinterpret_cast<float*>(b); b += align_up(sizeof(float) * (size_t)n * Kp, 1024);
  float* blo = reinterpret_cast<float*>(b);
  DMRG_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), s));
  DMRG_TRY(split_rows(A, k, 1, m, k, Kp, ahi, alo, s));
  DMRG_TRY(split_transpose(B, n, k, n, Kp, bhi, blo, s));
  GemmOut g{C, n, 1, m, n, 1, 0, 1.f};
  DMRG_TRY(gemm_split(ahi, alo, bhi, blo, m, n, Kp, g, err, s));
  int h = 0;
  DMRG_CUDA_TRY(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  DMRG_CUDA_TRY(cudaStreamSynchronize(s));
  return h;
}

// ---------------------------------------------------------------- environments
// Left:  Y1[(s,b)][(a',k)]  = sum_a   A^T[(s,b)][a] L[(a',k)][a]            (GEMM)
//        Y2[(m,b)][(a',s')] = sum_{k,s} W[k,s,s',m] Y1[(s,b)][(a',k)]        (MPO step)
//        Lnew[b'][(m,b)]    = sum_{(a',s')} A^T[b'][(a',s')] Y2[(m,b)][(a',s')]  (GEMM)
// Right: Z1[(a,s)][(b',m)]  = sum_b   B[(a,s)][b] R[(b',m)][b]              (GEMM)
//        Z2[(k,a)][(s',b')] = sum_{s,m} W[k,s,s',m] Z1[(a,s)][(b',m)]        (MPO step)
//        Rnew[a'][(k,a)]    = sum_{(s',b')} B[a'][(s',b')] Z2[(k,a)][(s',b')]    (GEMM)
namespace {

// Y2 (left): CTA = 32 consecutive a' (lanes) x EB consecutive b.
constexpr int EB = 8;
__global__ void __launch_bounds__(256) env_left_mpo_kernel(const float* __restrict__ Y1, const double* __restrict__ W,
                                                           int chil, int d, int chir, int wl, int wr, int Kp,
                                                           float* __restrict__ hi, float* __restrict__ lo) {
  extern __shared__ float sm[];
  const int nin = d * wl, nout = d * wr;
  float* sW = sm;                    // [(s',m)][(s,k)]
  float* sX = sW + nout * nin;       // [b_local][(s,k)][a_local 32]
  const int a0 = blockIdx.x * 32, b0 = blockIdx.y * EB;
  for (int i = threadIdx.x; i < nout * nin; i += blockDim.x) {
    const int r = i / nin, c = i % nin;
    const int sp = r / wr, m = r % wr, s = c / wl, k = c % wl;
    sW[i] = static_cast<float>(W[((k * d + s) * d + sp) * wr + m]);
  }
  const long long ldy = (long long)chil * wl;
  for (int i = threadIdx.x; i < EB * d * 32 * wl; i += blockDim.x) {
    const int col = i % (32 * wl);            // (a_local, k) contiguous in Y1
    const int s = (i / (32 * wl)) % d;
    const int bl = i / (32 * wl * d);
    const int al = col / wl, k = col % wl;
    const int a = a0 + al, b = b0 + bl;
    float v = 0.f;
    if (a < chil && b < chir) v = Y1[((long long)s * chir + b) * ldy + (long long)a * wl + k];
    sX[(bl * nin + s * wl + k) * 32 + al] = v;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int a = a0 + lane;
  for (int row = warp; row < EB * nout; row += 8) {
    const int bl = row / nout, r = row % nout;
    const int b = b0 + bl;
    if (b >= chir) continue;
    const float* w = sW + r * nin;
    const float* x = sX + (bl * nin) * 32 + lane;
    float acc = 0.f;
    for (int c = 0; c < nin; ++c) acc = fmaf(w[c], x[c * 32], acc);
    if (a < chil) {
      const int sp = r / wr, m = r % wr;
      const long long o = ((long long)m * chir + b) * Kp + (long long)a * d + sp;
      const float h = to_tf32(acc);
      hi[o] = h;
      lo[o] = to_tf32(acc - h);
    }
  }
}

// Z2 (right): CTA = 32 consecutive b' (lanes) x EB consecutive a.
__global__ void __launch_bounds__(256) env_right_mpo_kernel(const float* __restrict__ Z1, const double* __restrict__ W,
                                                            int chil, int d, int chir, int wl, int wr, int Kp,
                                                            float* __restrict__ hi, float* __restrict__ lo) {
  extern __shared__ float sm[];
  const int nin = d * wr, nout = wl * d;
  float* sW = sm;                    // [(k,s')][(s,m)]
  float* sX = sW + nout * nin;       // [a_local][(s,m)][b_local 32]
  const int b0 = blockIdx.x * 32, a0 = blockIdx.y * EB;
  for (int i = threadIdx.x; i < nout * nin; i += blockDim.x) {
    const int r = i / nin, c = i % nin;
    const int k = r / d, sp = r % d, s = c / wr, m = c % wr;
    sW[i] = static_cast<float>(W[((k * d + s) * d + sp) * wr + m]);
  }
  const long long ldz = (long long)chir * wr;
  for (int i = threadIdx.x; i < EB * d * 32 * wr; i += blockDim.x) {
    const int col = i % (32 * wr);            // (b_local, m) contiguous in Z1
    const int s = (i / (32 * wr)) % d;
    const int al = i / (32 * wr * d);
    const int bl = col / wr, m = col % wr;
    const int a = a0 + al, b = b0 + bl;
    float v = 0.f;
    if (a < chil && b < chir) v = Z1[((long long)a * d + s) * ldz + (long long)b * wr + m];
    sX[(al * nin + s * wr + m) * 32 + bl] = v;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int b = b0 + lane;
  for (int row = warp; row < EB * nout; row += 8) {
    const int al = row / nout, r = row % nout;
    const int a = a0 + al;
    if (a >= chil) continue;
    const float* w = sW + r * nin;
    const float* x = sX + (al * nin) * 32 + lane;
    float acc = 0.f;
    for (int c = 0; c < nin; ++c) acc = fmaf(w[c], x[c * 32], acc);
    if (b < chir) {
      const int k = r / d, sp = r % d;
      const long long o = ((long long)k * chil + a) * Kp + (long long)sp * chir + b;
      const float h = to_tf32(acc);
      hi[o] = h;
      lo[o] = to_tf32(acc - h);
    }
  }
}

struct EnvPlan {
  int Kp1, Kp2;
  float *A1hi, *A1lo, *E1hi, *E1lo, *Y1, *Y2hi, *Y2lo, *A2hi, *A2lo;
  int* err;
  size_t bytes;
};

EnvPlan env_plan(int side, int cl, int d, int cr, int wl, int wr, void* work) {
  EnvPlan p;
  char* b = static_cast<char*>(work);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    void* q = b ? b + off : nullptr;
    off += align_up(bytes, 1024);
    return q;
  };
  const size_t f = sizeof(float);
  p.err = static_cast<int*>(take(256));
  if (side == 0) {
    p.Kp1 = pad32(cl);
    p.Kp2 = pad32((long long)cl * d);
    p.A1hi = static_cast<float*>(take(f * (size_t)d * cr * p.Kp1));
    p.A1lo = static_cast<float*>(take(f * (size_t)d * cr * p.Kp1));
    p.E1hi = static_cast<float*>(take(f * (size_t)cl * wl * p.Kp1));
    p.E1lo = static_cast<float*>(take(f * (size_t)cl * wl * p.Kp1));
    p.Y1 = static_cast<float*>(take(f * (size_t)d * cr * cl * wl));
    p.Y2hi = static_cast<float*>(take(f * (size_t)wr * cr * p.Kp2));
    p.Y2lo = static_cast<float*>(take(f * (size_t)wr * cr * p.Kp2));
    p.A2hi = static_cast<float*>(take(f * (size_t)cr * p.Kp2));
    p.A2lo = static_cast<float*>(take(f * (size_t)cr * p.Kp2));
  } else {
    p.Kp1 = pad32(cr);
    p.Kp2 = pad32((long long)cr * d);
    p.A1hi = static_cast<float*>(take(f * (size_t)cl * d * p.Kp1));
    p.A1lo = static_cast<float*>(take(f * (size_t)cl * d * p.Kp1));
    p.E1hi = static_cast<float*>(take(f * (size_t)cr * wr * p.Kp1));
    p.E1lo = static_cast<float*>(take(f * (size_t)cr * wr * p.Kp1));
    p.Y1 = static_cast<float*>(take(f * (size_t)cl * d * cr * wr));
    p.Y2hi = static_cast<float*>(take(f * (size_t)wl * cl * p.Kp2));
    p.Y2lo = static_cast<float*>(take(f * (size_t)wl * cl * p.Kp2));
    p.A2hi = static_cast<float*>(take(f * (size_t)cl * p.Kp2));
    p.A2lo = static_cast<float*>(take(f * (size_t)cl * p.Kp2));
  }
  p.bytes = off;
  return p;
}

}  // namespace

size_t tf32x3_env_workspace_bytes(int chil, int d, int chir, int wl, int wr) {
  size_t a = env_plan(0, chil, d, chir, wl, wr, nullptr).bytes;
  size_t b = env_plan(1, chil, d, chir, wl, wr, nullptr).bytes;
  return a > b ? a : b;
}

int tf32x3_env(int side, int cl, int d, int cr, int wl, int wr, const double* E, const double* W, const double* A,
               double* Enew, void* work, cudaStream_t s) {
  EnvPlan p = env_plan(side, cl, d, cr, wl, wr, work);
  DMRG_CUDA_TRY(cudaMemsetAsync(p.err, 0, 256, s));
  static std::atomic<unsigned long long> attr_l{0}, attr_r{0};
  DMRG_TRY(smem_attr_once(reinterpret_cast<const void*>(env_left_mpo_kernel), 200 * 1024, attr_l));
  DMRG_TRY(smem_attr_once(reinterpret_cast<const void*>(env_right_mpo_kernel), 200 * 1024, attr_r));
  if (side == 0) {
    // GEMM 1: rows (s,b) of A^T, cols (a',k) of L, K = a
    DMRG_TRY(split_transpose(A, (long long)d * cr, cl, d * cr, p.Kp1, p.A1hi, p.A1lo, s));
    DMRG_TRY(split_rows(E, cl, 1, cl * wl, cl, p.Kp1, p.E1hi, p.E1lo, s));
    GemmOut g1{p.Y1, (long long)cl * wl, 1, d * cr, cl * wl, 0, 0, 1.f};
    DMRG_TRY(gemm_split(p.A1hi, p.A1lo, p.E1hi, p.E1lo, d * cr, cl * wl, p.Kp1, g1, p.err, s));
    // MPO step -> Y2 rows (m,b), K = (a',s')
    DMRG_CUDA_TRY(cudaMemsetAsync(p.Y2hi, 0, sizeof(float) * (size_t)wr * cr * p.Kp2, s));
    DMRG_CUDA_TRY(cudaMemsetAsync(p.Y2lo, 0, sizeof(float) * (size_t)wr * cr * p.Kp2, s));
    const size_t smem = sizeof(float) * ((size_t)d * wr * d * wl + (size_t)EB * d * wl * 32);
    if (smem > 200 * 1024) return DMRG_ERR_UNSUPPORTED;
    dim3 grid((cl + 31) / 32, (cr + EB - 1) / EB);
    if (grid.y > 65535) return DMRG_ERR_ARG;
    env_left_mpo_kernel<<<grid, 256, smem, s>>>(p.Y1, W, cl, d, cr, wl, wr, p.Kp2, p.Y2hi, p.Y2lo);
    DMRG_CHECK_LAUNCH();
    // GEMM 2: rows b' of A^T (K = (a',s')), cols (m,b)
    DMRG_TRY(split_transpose(A, cr, cl * d, cr, p.Kp2, p.A2hi, p.A2lo, s));
    GemmOut g2{Enew, (long long)wr * cr, 1, cr, wr * cr, 1, 0, 1.f};
    DMRG_TRY(gemm_split(p.A2hi, p.A2lo, p.Y2hi, p.Y2lo, cr, wr * cr, p.Kp2, g2, p.err, s));
  } else {
    // GEMM 1: rows (a,s) of B, cols (b',m) of R, K = b
    DMRG_TRY(split_rows(A, cr, 1, cl * d, cr, p.Kp1, p.A1hi, p.A1lo, s));
    DMRG_TRY(split_rows(E, cr, 1, cr * wr, cr, p.Kp1, p.E1hi, p.E1lo, s));
    GemmOut g1{p.Y1, (long long)cr * wr, 1, cl * d, cr * wr, 0, 0, 1.f};
    DMRG_TRY(gemm_split(p.A1hi, p.A1lo, p.E1hi, p.E1lo, cl * d, cr * wr, p.Kp1, g1, p.err, s));
    DMRG_CUDA_TRY(cudaMemsetAsync(p.Y2hi, 0, sizeof(float) * (size_t)wl * cl * p.Kp2, s));
    DMRG_CUDA_TRY(cudaMemsetAsync(p.Y2lo, 0, sizeof(float) * (size_t)wl * cl * p.Kp2, s));
    const size_t smem = sizeof(float) * ((size_t)wl * d * d * wr + (size_t)EB * d * wr * 32);
    if (smem > 200 * 1024) return DMRG_ERR_UNSUPPORTED;
    dim3 grid((cr + 31) / 32, (cl + EB - 1) / EB);
    if (grid.y > 65535) return DMRG_ERR_ARG;
    env_right_mpo_kernel<<<grid, 256, smem, s>>>(p.Y1, W, cl, d, cr, wl, wr, p.Kp2, p.Y2hi, p.Y2lo);
    DMRG_CHECK_LAUNCH();
    // GEMM 2: rows a' of B (K = (s',b')), cols (k,a)
    DMRG_TRY(split_rows(A, (long long)d * cr, 1, cl, d * cr, p.Kp2, p.A2hi, p.A2lo, s));
    GemmOut g2{Enew, (long long)wl * cl, 1, cl, wl * cl, 1, 0, 1.f};
    DMRG_TRY(gemm_split(p.A2hi, p.A2lo, p.Y2hi, p.Y2lo, cl, wl * cl, p.Kp2, g2, p.err, s));
  }
  int h = 0;
  DMRG_CUDA_TRY(cudaMemcpyAsync(&h, p.err, sizeof(int), cudaMemcpyDeviceToHost, s));
  DMRG_CUDA_TRY(cudaStreamSynchronize(s));
  return h;
}

}  // namespace dmrg

// ---------------------------------------------------------------- C ABI of the tuner
extern "C" int dmrg_autotune_enable(int enable) { return dmrg::g_tune_on.exchange(enable ? 1 : 0); }

extern "C" int dmrg_autotune_entries(int* out, int max_entries) {
  std::lock_guard<std::mutex> lock(dmrg::g_tune_mu);
  int n = 0;
  for (const auto& kv : dmrg::g_tune) {
    if (out && n < max_entries) {
      int* e = out + 7 * n;
      e[0] = kv.first.M;
      e[1] = kv.first.N;
      e[2] = kv.first.K;
      e[3] = kv.second.bnt;
      e[4] = kv.second.merge;
      e[5] = kv.second.group;
      e[6] = (int)(kv.second.ms * 1000.f);
    }
    ++n;
  }
  return n;
}
