// Fast form of the two-photon luminosity: the per-cell quadrature of
// calcTwoPhotonLumi (src/UpcCrossSection.cpp:221-271) as a tensor-core
// contraction.
//
// The reference's 120-bin midpoint rule differs from the converged integral
// by 2e-4 .. 6e-2 (relative), so a fast form on fixed radial grids cannot match
// it to 1e-4.  This form keeps the reference's nodes exactly and changes only
// the survival kernel's representation and the arithmetic:
//
//   L/(2 pi^2 M) = sum_ij a1_i G(b1_i, b2_j) a2_j,   a_i = N(b_i, k) b_i (bh-bl)_i
//
// * nodes with b > 250 fm see G = c exactly (every azimuth gives b >= 20 fm),
//   so their part is c (S1far S2 + S1near S2far) in FP64;
// * for the near nodes G is interpolated on a fixed log grid r_p (P = 1024
//   points, 0.1 .. 256 fm) with 4-point Lagrange weights phi_p in ln r:
//   sum_ij a1_i G_ij a2_j ~= A1 . Gfix . A2,  A_p = sum_i a_i phi_p(b_i);
// * A1 . Gfix runs on tcgen05 tensor cores as a three-term BF16 split
//   (hi*hi + hi*lo + lo*hi, FP32 accumulation in TMEM); the row-dot with A2
//   is fused into the TMEM epilogue, so the cells x P product never reaches HBM.
//
// Kernel k_contract: one CTA per 128-cell x 256-column tile, warp-specialised:
// warp 0 issues TMA (SWIZZLE_128B boxes of 64 bf16), warp 1 allocates TMEM and
// issues tcgen05.mma (M=128, N=256, K=16) from one thread, warps 2-5 drain the
// accumulator with tcgen05.ld.  Two 96 KB pipeline stages.  Every mbarrier
// wait is bounded by a 2 s timer and reports through an error word.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include "upcg_internal.h"

namespace upcg {

namespace {

constexpr int BM = 128, BN = 256, BK = 64;
static_assert(BK == kContractBK, "K tile of the work items");
constexpr int kStages = 2;
constexpr int kATile = BM * BK * 2;  // 16 KB
constexpr int kBTile = BN * BK * 2;  // 32 KB
constexpr int kStageBytes = 2 * kATile + 2 * kBTile;
constexpr int kContractSmem = kStages * kStageBytes + 1024;  // + alignment slack
constexpr int kTmemCols = 256;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t gtimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: gives up after ~2 s, records `code` in *err and returns false.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, unsigned* err,
                                          unsigned code) {
  const uint64_t t0 = gtimer();
  for (uint32_t i = 0;; ++i) {
    if (mbar_try(bar, parity)) return true;
    if ((i & 255u) == 255u && gtimer() - t0 > 2000000000ull) {
      atomicOr(err, code);
      return false;
    }
  }
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar,
                                            int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4}], [%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y)
      : "memory");
}

// Shared-memory matrix descriptor: K-major, SWIZZLE_128B (8 rows x 128 bytes
// per 1024-byte atom, atoms stacked at 1024 bytes), descriptor version 1.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;            // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;  // stride byte offset between 8-row atoms
  d |= (uint64_t)1 << 46;            // version
  d |= (uint64_t)2 << 61;            // SWIZZLE_128B
  return d;
}

// Instruction descriptor, kind::f16: D = F32, A = B = BF16, both K-major.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                            ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void umma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(kIdesc), "r"(acc));
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

struct ContractArgs {
  int ktiles, ncells, P, ntiles;
  const float* a2;  // [cells_pad][P]
  float* partial;   // [cells][ntiles]
  unsigned* err;
  // store epilogue (general product D = A B^T): when out_f32 or out_hi is set
  // the D tile goes to memory instead of the row-dot with a2 -- FP32, or as a
  // bf16 hi/lo pair that feeds a following product; rows < ncells, ld = ldo
  float* out_f32;
  __nv_bfloat16* out_hi;
  __nv_bfloat16* out_lo;
  int ldo;
};

__global__ void __launch_bounds__(192, 1) k_contract(const __grid_constant__ CUtensorMap tAh,
                                                     const __grid_constant__ CUtensorMap tAl,
                                                     const __grid_constant__ CUtensorMap tBh,
                                                     const __grid_constant__ CUtensorMap tBl,
                                                     ContractArgs args) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[kStages], empty_bar[kStages], done_bar;
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // the N tiles of one 128-cell row block are adjacent in launch order, so
  // the row block's A tiles come from DRAM once and from L2 for the others
  const int nt = blockIdx.x, mt = blockIdx.y;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    mbar_init(&done_bar, 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_slot)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

  if (warp == 0 && lane == 0) {
    // ---------------- TMA producer
    int issued = 0;
    for (int kt = 0; kt < args.ktiles; ++kt) {
      const int s = kt % kStages;
      const uint32_t ph = (kt / kStages) & 1;
      if (kt >= kStages && !mbar_wait(&empty_bar[s], ph ^ 1, args.err, 1u)) {
        abort_flag = 1;
        break;
      }
      if (abort_flag) break;
      uint8_t* st = smem + s * kStageBytes;
      mbar_expect_tx(&full_bar[s], kStageBytes);
      const int x = kt * BK;
      tma_load_2d(st, &tAh, &full_bar[s], x, mt * BM);
      tma_load_2d(st + kATile, &tAl, &full_bar[s], x, mt * BM);
      tma_load_2d(st + 2 * kATile, &tBh, &full_bar[s], x, nt * BN);
      tma_load_2d(st + 2 * kATile + kBTile, &tBl, &full_bar[s], x, nt * BN);
      issued = kt + 1;
    }
    // our own copies in flight must land before the CTA can exit
    for (int kt = (issued > kStages ? issued - kStages : 0); kt < issued; ++kt)
      mbar_wait(&full_bar[kt % kStages], (kt / kStages) & 1, args.err, 8u);
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer (single thread)
    bool ok = true;
    for (int kt = 0; kt < args.ktiles && ok; ++kt) {
      const int s = kt % kStages;
      if (!mbar_wait(&full_bar[s], (kt / kStages) & 1, args.err, 2u)) {
        ok = false;
        abort_flag = 1;
        break;
      }
      tc_fence_after();
      const uint32_t base = smem_u32(smem + s * kStageBytes);
      const uint32_t ah = base, al = base + kATile, bh = base + 2 * kATile,
                     bl = base + 2 * kATile + kBTile;
#pragma unroll
      for (int kk = 0; kk < BK / 16; ++kk) {
        const uint32_t off = kk * 32;  // 16 bf16 along K inside the 128-byte swizzled row
        const uint64_t dah = sw128_desc(ah + off), dal = sw128_desc(al + off);
        const uint64_t dbh = sw128_desc(bh + off), dbl = sw128_desc(bl + off);
        umma(tmem, dah, dbh, (kt > 0 || kk > 0) ? 1u : 0u);
        umma(tmem, dah, dbl, 1u);
        umma(tmem, dal, dbh, 1u);
      }
      umma_commit(&empty_bar[s]);  // frees the stage once these MMAs have read it
    }
    umma_commit(&done_bar);
  } else if (warp >= 2) {
    // ---------------- epilogue: TMEM -> registers, row-dot with A2
    const bool ok = mbar_wait(&done_bar, 0, args.err, 4u);
    tc_fence_after();
    const int quad = warp & 3;  // TMEM lanes 32*quad .. 32*quad+31
    const int row = quad * 32 + lane;
    const int cell = mt * BM + row;
    float acc = 0.f;
    if (args.out_f32 || args.out_hi) {
      for (int c0 = 0; c0 < BN; c0 += 16) {
        float v[16];
        if (ok) tmem_ld16(tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)c0, v);
        if (!ok || cell >= args.ncells) continue;
        const size_t o = (size_t)cell * args.ldo + nt * BN + c0;
        if (args.out_f32) {
          float4* d = reinterpret_cast<float4*>(args.out_f32 + o);
#pragma unroll
          for (int q = 0; q < 4; ++q) d[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
        } else {
          uint32_t hw[8], lw[8];
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * q], v[2 * q + 1]);
            const float2 f = __bfloat1622float2(h);
            const __nv_bfloat162 l = __floats2bfloat162_rn(v[2 * q] - f.x, v[2 * q + 1] - f.y);
            hw[q] = *reinterpret_cast<const uint32_t*>(&h);
            lw[q] = *reinterpret_cast<const uint32_t*>(&l);
          }
          uint4* dh = reinterpret_cast<uint4*>(args.out_hi + o);
          uint4* dl = reinterpret_cast<uint4*>(args.out_lo + o);
          dh[0] = make_uint4(hw[0], hw[1], hw[2], hw[3]);
          dh[1] = make_uint4(hw[4], hw[5], hw[6], hw[7]);
          dl[0] = make_uint4(lw[0], lw[1], lw[2], lw[3]);
          dl[1] = make_uint4(lw[4], lw[5], lw[6], lw[7]);
        }
      }
    } else if (ok) {
      const float* a2 = args.a2 + (size_t)cell * args.P + nt * BN;
      for (int c0 = 0; c0 < BN; c0 += 16) {
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)c0, v);
        if (cell < args.ncells) {
          const float4* a4 = reinterpret_cast<const float4*>(a2 + c0);
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const float4 w = __ldg(a4 + q);
            acc += v[4 * q] * w.x + v[4 * q + 1] * w.y + v[4 * q + 2] * w.z + v[4 * q + 3] * w.w;
          }
        }
      }
    }
    if (!args.out_f32 && !args.out_hi && cell < args.ncells)
      args.partial[(size_t)cell * args.ntiles + nt] = ok ? acc : 0.f;
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemCols));
  }
}

// ------------------------------------------------------------ TF32 product --
// k_gemm_tf32: D = A B^T on tcgen05 kind::tf32, one product per k step (no
// hi / lo split: TF32 keeps 10 mantissa bits of each FP32 operand), FP32
// accumulation in TMEM, FP32 store epilogue.  A [Mpad][K], B [N][K] FP32 with
// K contiguous; 128-byte rows of 32 elements in SWIZZLE_128B boxes, so the
// shared-memory layout, the descriptors and the 32-byte step per MMA (K = 8)
// are those of the bf16 kernels.  One CTA per 128 x 256 tile, 4 stages;
// warps 0 (TMA), 1 (MMA), 2-5 (epilogue), every wait bounded.
constexpr int kT32K = 32;                 // elements per 128-byte row
constexpr int kT32A = BM * 128;           // 16 KB
constexpr int kT32B = BN * 128;           // 32 KB
constexpr int kT32Stages = 4;
constexpr int kT32Smem = kT32Stages * (kT32A + kT32B) + 1024;
// instruction descriptor, kind::tf32: D = F32, A = B = TF32, both K-major
constexpr uint32_t kIdescTf32 = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BN >> 3) << 17) |
                                ((uint32_t)(BM >> 4) << 24);

__global__ void __launch_bounds__(192, 1) k_gemm_tf32(const __grid_constant__ CUtensorMap tA,
                                                      const __grid_constant__ CUtensorMap tB,
                                                      int ktiles, int M, int ldo, float* out,
                                                      unsigned* err) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[kT32Stages], empty_bar[kT32Stages], done_bar;
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nt = blockIdx.x, mt = blockIdx.y;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kT32Stages; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    mbar_init(&done_bar, 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_slot)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  if (warp == 0 && lane == 0) {
    int issued = 0;
    for (int kt = 0; kt < ktiles; ++kt) {
      const int s = kt % kT32Stages;
      const uint32_t ph = (kt / kT32Stages) & 1;
      if (kt >= kT32Stages && !mbar_wait(&empty_bar[s], ph ^ 1, err, 1u)) {
        abort_flag = 1;
        break;
      }
      if (abort_flag) break;
      uint8_t* st = smem + s * (kT32A + kT32B);
      mbar_expect_tx(&full_bar[s], kT32A + kT32B);
      const int x = kt * kT32K;
      tma_load_2d(st, &tA, &full_bar[s], x, mt * BM);
      tma_load_2d(st + kT32A, &tB, &full_bar[s], x, nt * BN);
      issued = kt + 1;
    }
    for (int kt = (issued > kT32Stages ? issued - kT32Stages : 0); kt < issued; ++kt)
      mbar_wait(&full_bar[kt % kT32Stages], (kt / kT32Stages) & 1, err, 8u);
  } else if (warp == 1 && lane == 0) {
    for (int kt = 0; kt < ktiles; ++kt) {
      const int s = kt % kT32Stages;
      if (!mbar_wait(&full_bar[s], (kt / kT32Stages) & 1, err, 2u)) {
        abort_flag = 1;
        break;
      }
      tc_fence_after();
      const uint32_t a = smem_u32(smem + s * (kT32A + kT32B)), b = a + kT32A;
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {  // 8 TF32 (32 bytes) along K per MMA
        const uint64_t da = sw128_desc(a + kk * 32), db = sw128_desc(b + kk * 32);
        const uint32_t acc = (kt > 0 || kk > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(da), "l"(db), "r"(kIdescTf32), "r"(acc));
      }
      umma_commit(&empty_bar[s]);
    }
    umma_commit(&done_bar);
  } else if (warp >= 2) {
    const bool ok = mbar_wait(&done_bar, 0, err, 4u);
    tc_fence_after();
    const int quad = warp & 3;
    const int row = mt * BM + quad * 32 + lane;
    for (int c0 = 0; c0 < BN; c0 += 16) {
      float v[16];
      if (ok) tmem_ld16(tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)c0, v);
      if (!ok || row >= M) continue;
      float4* d = reinterpret_cast<float4*>(out + (size_t)row * ldo + nt * BN + c0);
#pragma unroll
      for (int q = 0; q < 4; ++q) d[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemCols));
  }
}

// FP32 value of a bf16 hi / lo pair (the operands of the TF32 products)
__global__ void k_pair_to_f32(const __nv_bfloat16* __restrict__ hi, const __nv_bfloat16* __restrict__ lo,
                              size_t n, float* __restrict__ out) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = __bfloat162float(hi[i]) + __bfloat162float(lo[i]);
}

// --------------------------------------------------------------- grids ---
struct FastGrid {
  int P;
  double u0, h, inv_h;  // r_p = exp(u0 + p h)
  double r_near;        // nodes up to here are projected
  // per-cell constants of the projection, in logs (set by launch_fast_project)
  const double* lnm2;   // ln(m_im / 2)
  double ln5ghc1, ln5ghc2, ln5R, lnbmin, ln2R, ln_rnear, lnghc, lnc_pt, lnc_ff;
  double c_far;         // G where every azimuth has b >= 20 fm: P(20) sum_k w_k
  // rows -> cells: null, row = cell; else row r is cell (m0 + r / n_rep_y,
  // rep_y[r % n_rep_y]) -- one cell of each pair of mirror rapidities
  // (L(m, -y) = L(m, y): the two photons swap and G is symmetric)
  const int* rep_y;
  int n_rep_y, m0;
};

__device__ __forceinline__ int fast_cell(const FastGrid& fg, int ny, int row) {
  if (!fg.rep_y) return row;
  const int q = row / fg.n_rep_y;
  return (fg.m0 + q) * ny + __ldg(fg.rep_y + (row - q * fg.n_rep_y));
}

struct GParams {
  SplineF gaa, brk;
  int has_brk;
  float P20, cosk[5], wk[5];
  float u0, h;
  const double* P20d;  // when set: P20 from the device (k_far_consts)
  // when far_out is set, each block takes P20 from the FP64 breakup spline
  // itself, and block (0, 0) writes k_far_consts' pair (P20, P20 sum_k w_k)
  // to far_out and resets the contraction's error word err0
  SplineU brk64;
  double wkd[5];
  double* far_out;
  unsigned* err0;
  // delta: store G - P20 sum_k w_k (zero wherever all five azimuths reach
  // b >= 20 fm); k_fast_finish adds the constant's share back in FP64
  int delta;
};

// G_pq = sum_k w_k P(min(b,20)) (b<20 ? G_AA(b) : 1), b^2 = r_p^2 + r_q^2 +
// 2 r_p r_q cos phi_k (the azimuthal sum of src/UpcCrossSection.cpp:250-262)
// in FP32 -- the bf16 hi/lo pair it is stored as keeps 2^-16 of it.
__global__ void k_fast_G(GParams gp, int P, __nv_bfloat16* __restrict__ gh,
                         __nv_bfloat16* __restrict__ gl) {
  __shared__ float4 sg[200];
  __shared__ float sP20;
  for (int i = threadIdx.x; i < gp.gaa.n - 1 && i < 200; i += blockDim.x) sg[i] = gp.gaa.coef[i];
  if (gp.far_out && threadIdx.x == 0) {  // k_far_consts' arithmetic
    const double P20 = gp.has_brk ? spline_eval(gp.brk64, 20.) : 1.;
    sP20 = (float)P20;
    if (blockIdx.x == 0 && blockIdx.y == 0) {
      double c = 0.;
      for (int k = 0; k < 5; ++k) c += P20 * 1. * gp.wkd[k];
      gp.far_out[0] = P20;
      gp.far_out[1] = c;
      if (gp.err0) *gp.err0 = 0u;
    }
  }
  __syncthreads();
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int pp = blockIdx.y;
  if (q >= P) return;
  const float rp = expf(gp.u0 + pp * gp.h), rq = expf(gp.u0 + q * gp.h);
  const float P20 = gp.far_out ? sP20 : (gp.P20d ? (float)__ldg(gp.P20d) : gp.P20);
  float g = 0.f;
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const float bsq = rp * rp + rq * rq + 2.f * rp * rq * gp.cosk[k];
    float v = P20;
    if (bsq < 400.f) {
      const float b = sqrtf(bsq);
      if (b < 20.f)
        v = (gp.has_brk ? spline_eval_f(gp.brk, gp.brk.coef, b) : 1.f) * spline_eval_f(gp.gaa, sg, b);
    }
    g += (gp.delta ? v - P20 : v) * gp.wk[k];
  }
  const __nv_bfloat16 hi = __float2bfloat16(g);
  const __nv_bfloat16 lo = __float2bfloat16(g - __bfloat162float(hi));
  gh[(size_t)pp * P + q] = hi;
  gl[(size_t)pp * P + q] = lo;
}

// ------------------------------------------------------- flux tables ----
// Point flux: N = factor k/g^2 (K1(x)^2 + K0(x)^2/g^2), x = b k/(g hc).  The
// table holds S(ln x) = ln(K1^2 + K0^2/g^2) + 2x (smooth, O(1)) on a uniform
// grid in ln x, in FP64 and as an FP32 copy; ln N = ln(factor k/g^2) + S - 2x.
constexpr int kKTabN = 8192;
constexpr double kKTabU0 = -16.11809565095832;  // ln(1e-7)
constexpr double kKTabU1 = 5.703782474656201;   // ln(300): beyond it the flux is below 1e-250 and
                                                // is taken as zero (exp(-2x) underflows near x = 354)

__global__ void k_ktab(double g, double* __restrict__ t1, float* __restrict__ t32) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kKTabN) return;
  const double h = (kKTabU1 - kKTabU0) / (kKTabN - 1);
  const double x = exp(kKTabU0 + i * h);
  double K0, K1;
  bessel_k01(x, K0, K1);
  const double v = log(K1 * K1 + K0 * K0 / g / g) + 2. * x;
  t1[i] = v;
  t32[i] = (float)v;
}

// The same table from cached Bessel logs: lk = ln K + x on the fixed x grid
// (independent of g), S = 2 lk1 + ln(1 + e^{2 (lk0 - lk1)} / g^2).
__global__ void k_k01_logs(double2* __restrict__ lk) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kKTabN) return;
  const double h = (kKTabU1 - kKTabU0) / (kKTabN - 1);
  const double x = exp(kKTabU0 + i * h);
  double K0, K1;
  bessel_k01(x, K0, K1);
  lk[i] = make_double2(log(K0) + x, log(K1) + x);
}

__global__ void k_ktab_logs(double g, const double2* __restrict__ lk, double* __restrict__ t1,
                            float* __restrict__ t32) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kKTabN) return;
  const double2 l = lk[i];
  const double v = 2. * l.y + log1p(exp(2. * (l.x - l.y)) / (g * g));
  t1[i] = v;
  t32[i] = (float)v;
}

// Form-factor flux amplitude Q(w, b) = int_0^10 q^2 F(q^2 + w^2/g^2)/(q^2 + w^2/g^2)
// J1(b q / hc) dq (the integrand of src/UpcCrossSection.cpp:181-191, clamp at
// Q2max - dQ2 included): composite Gauss-Legendre on q in [0, kQNodeMax] as
// the product H[w][n] J[n][b] (k_qtab_product, double-float), the rest in
// closed form (k_dgemm_reduce).
__global__ void k_qtab_H(LumiParams p, const double* __restrict__ qn, const double* __restrict__ wn,
                         int nq, double lw0, double hw, double* __restrict__ H, double lb0,
                         double hb, int nb, double* __restrict__ tail) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  const int iw = blockIdx.y;
  // q in [kQNodeMax, 10]: q^2 + w^2/g^2 > Q2max, so the reference's integrand
  // is F(Q2max - dQ2) q^2 / (q^2 + w^2/g^2) J1(b q / hc); with the
  // q^2 / (q^2 + w^2/g^2) factor taken as 1 its integral is
  // F_c hc / b (J0(b qc / hc) - J0(10 b / hc)).  The factor's departure,
  // (w/g)^2 / qc^2 at most, is below 1e-2 for w < 0.2 g, where this part is
  // itself ~1e-6 of Q; at larger w the flux is below 1e-10 of its peak.
  if (blockIdx.x == 0 && iw == 0) {
    const double fc = spline_eval(p.ff, p.q2clamp) * kHc;
    for (int j = threadIdx.x; j < nb; j += blockDim.x) {
      const double b = exp(lb0 + j * hb);
      tail[j] = fc / b * (j0(b * kQNodeMax / kHc) - j0(b * 10. / kHc));
    }
  }
  // (w / g)^2 of the block's row, once per block: an FP64 exp and two
  // divisions cost a warp the same for one lane as for 32
  __shared__ double s_e2;
  if (threadIdx.x == 0) {
    const double w = exp(lw0 + iw * hw);
    s_e2 = w * w / p.g1 / p.g1;
  }
  __syncthreads();
  if (n >= nq) return;
  const double q = qn[n];
  const double t = q * q + s_e2;
  const double ffv = spline_eval(p.ff, t < p.q2max ? t : p.q2clamp);
  const double h = wn[n] * (q * q * ffv / t);
  // stored as a double-float pair (hi, lo) for k_qtab_product
  const float hh = (float)h;
  reinterpret_cast<float2*>(H)[(size_t)iw * nq + n] = make_float2(hh, (float)(h - (double)hh));
}

// J1(b q_n / hc) on the table's (node, b) grid: it needs no form factor, so
// it can run before the form-factor chain is done
__global__ void k_qtab_J(const double* __restrict__ qn, int nq, double lb0, double hb, int nb,
                         double* __restrict__ J) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = blockIdx.y;
  if (j >= nb) return;
  const double b = exp(lb0 + j * hb);
  const double jv = j1(b * qn[n] / kHc);
  const float jh = (float)jv;  // a double-float pair (hi, lo) for k_qtab_product
  reinterpret_cast<float2*>(J)[(size_t)n * nb + j] = make_float2(jh, (float)(jv - (double)jh));
}

// Split-K product Cp[s][M][N] = A[M][Ks] B[Ks][N] over the s-th slice of K
// (kslice columns; M, N multiples of 64, kslice of 16), 64 x 64 tiles, in
// double-float arithmetic: the operands come as float pairs (hi + lo, written
// so by k_qtab_H / k_qtab_J), each product is split exactly (hi = a_h b_h, its rounding
// error by an FMA, plus the cross terms), and the sum is a compensated
// (hi, lo) pair.  About 2^-44 relative to the terms' size -- FP64-grade for a
// Hankel sum whose terms cancel -- on the FP32 pipe, which this part runs at
// 64x its FP64 rate.  The 512 x 256 table is 32 tiles, a fifth of the SMs;
// the K slices give the rest of the machine work.
__global__ void __launch_bounds__(256) k_qtab_product(const float2* __restrict__ A,
                                                      const float2* __restrict__ B,
                                                      double* __restrict__ Cp, int M, int N, int K,
                                                      int kslice) {
  __shared__ float sah[16][64 + 1], sal[16][64 + 1], sbh[16][64 + 1], sbl[16][64 + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
  const int kb = blockIdx.z * kslice, ke = kb + kslice;
  double* C = Cp + (size_t)blockIdx.z * M * N;
  float sh[4][4] = {}, sl[4][4] = {};  // the sums as (hi, lo) pairs
  for (int k0 = kb; k0 < ke; k0 += 16) {
    for (int e = threadIdx.x; e < 16 * 64; e += 256) {
      const int r = e >> 4, c = e & 15;  // A tile: 64 rows x 16 cols
      const float2 a = A[(size_t)(m0 + r) * K + k0 + c];
      sah[c][r] = a.x;
      sal[c][r] = a.y;
      const int rb = e >> 6, cb = e & 63;  // B tile: 16 rows x 64 cols
      const float2 b = B[(size_t)(k0 + rb) * N + n0 + cb];
      sbh[rb][cb] = b.x;
      sbl[rb][cb] = b.y;
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < 16; ++kk) {
      float ah[4], al[4], bh[4], bl[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        ah[i] = sah[kk][ty * 4 + i];
        al[i] = sal[kk][ty * 4 + i];
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        bh[j] = sbh[kk][tx * 4 + j];
        bl[j] = sbl[kk][tx * 4 + j];
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          // __fmul_rn / __fadd_rn / __fsub_rn: no contraction into FMAs, which
          // would break the error-free transformations
          const float p = __fmul_rn(ah[i], bh[j]);
          float e = fmaf(ah[i], bh[j], -p);  // the exact rounding error of p
          e = fmaf(ah[i], bl[j], fmaf(al[i], bh[j], e));
          // two-sum of the running hi part and p; the errors gather in lo
          const float t = __fadd_rn(sh[i][j], p);
          const float v = __fsub_rn(t, sh[i][j]);
          const float err = __fadd_rn(__fsub_rn(sh[i][j], __fsub_rn(t, v)), __fsub_rn(p, v));
          sl[i][j] = __fadd_rn(sl[i][j], __fadd_rn(err, e));
          sh[i][j] = t;
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
      C[(size_t)(m0 + ty * 4 + i) * N + n0 + tx * 4 + j] = (double)sh[i][j] + (double)sl[i][j];
}

// C = sum over the slices in order (FP64), and its FP32 copy
// Sums the K slices and adds the closed-form part beyond kQNodeMax (k_qtab_J).
__global__ void k_dgemm_reduce(const double* __restrict__ Cp, int nslice, size_t mn, int nb,
                               const double* __restrict__ tail, double* __restrict__ C,
                               float* __restrict__ C32) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= mn) return;
  double v = 0.;
  for (int z = 0; z < nslice; ++z) v += Cp[(size_t)z * mn + i];
  v += __ldg(tail + (int)(i % (size_t)nb));
  C[i] = v;
  C32[i] = (float)v;
}

// 4-point Lagrange weights at fractional position t of a uniform table of n
// points (first point p0, clamped so that the stencil stays inside).
__device__ __forceinline__ int lag4f(float t, int n, float w[4]) {
  int p0 = (int)floorf(t) - 1;
  p0 = p0 < 0 ? 0 : (p0 > n - 4 ? n - 4 : p0);
  const float s = t - (float)p0;
  const float s1 = s - 1.f, s2 = s - 2.f, s3 = s - 3.f;
  w[0] = -s1 * s2 * s3 * (1.f / 6.f);
  w[1] = s * s2 * s3 * 0.5f;
  w[2] = -s * s1 * s3 * 0.5f;
  w[3] = s * s1 * s2 * (1.f / 6.f);
  return p0;
}

struct FluxTabs {
  const float* s32;  // S(ln x), kKTabN points
  const float* q32;  // Q[nw][nb]
  int nw, nb;
  double lw0, inv_hw, lb0, inv_hb;
};

// ------------------------------------------------------------ projection --
// One CTA per cell.  Per side (photon), everything that decides which
// formula or which part a node belongs to is taken in FP64 from the
// reference's own node positions ((bl + bh)/2, src/UpcCrossSection.cpp:
// 232-262); the per-node work runs in FP32 in log space: ln a_i with
// a_i = N(b_i, k) b_i (bh - bl)_i.  Each side is normalised by its largest
// near-node weight, so cells whose luminosity lies far below FP32's range
// keep full precision; the scale returns in FP64 in k_fast_finish.
constexpr int kMaxP = 1024;  // radial grid points (the projection's shared-memory row)
constexpr int kNodeStride = 128;  // floats per (row, side) of a node list: header [4], weights [120], pad

struct __align__(16) SideC {  // 80 bytes: five 16-byte loads
  float lnb0, ld;   // ln b_i = lnb0 + i ld
  float tg0, tgd;   // radial-grid coordinate of node i: tg0 + i tgd
  float inv_tgd;
  float lnw0;       // ln(b_i (bh - bl)_i) = 2 ln b_i + lnw0
  float tk0, tkd;   // point-flux table coordinate of node i: tk0 + i tkd
  float lnxk;       // ln x_i = ln b_i + lnxk
  float lnc_pt;     // ln(factor k / g^2)
  float lnc_ff;     // ln(factor / (A^2 k))
  float tb0, tbd;   // Q-table b coordinate of node i: tb0 + i tbd
  int n_form;       // nodes 0 .. n_form-1 take the form-factor flux (b <= 2R)
  int n_near;       // nodes 0 .. n_near-1 lie at b <= r_near
  int iw;           // Q-table w row of the photon energy
  float ww[4];
};

// ln((1 + e^d)/2) - d/2 = ln cosh(d/2), by its Taylor series in z = d/2
// (|z| <= 0.1 here: the truncation is below 1e-16).  With it the reference's
// node midpoints b_i = (bl + bh)/2 (src/UpcCrossSection.cpp:236-238) are
// ln b_i = ln bmin + (i + 1/2) d + ln cosh(d/2) without an FP64 exp, which
// this part's FP64 pipe (1/64 of the FP32 rate) cannot afford per cell.
__device__ __forceinline__ double ln_cosh_half(double d) {
  const double z2 = 0.25 * d * d;
  // ln cosh z = z^2/2 - z^4/12 + z^6/45 - 17 z^8/2520 + 31 z^10/14175 - 691 z^12/935550
  double r = -691. / 935550.;
  r = fma(r, z2, 31. / 14175.);
  r = fma(r, z2, -17. / 2520.);
  r = fma(r, z2, 1. / 45.);
  r = fma(r, z2, -1. / 12.);
  r = fma(r, z2, 0.5);
  return r * z2;
}

// Side constants of every (cell, photon): one thread each, so that the few
// FP64 operations they need run on full warps (an FP64 warp instruction
// costs the same with 2 active lanes as with 32 on this part).
__global__ void k_fast_sides(LumiParams p, FastGrid fg, FluxTabs ft, int cell0, int ncells,
                             SideC* __restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 2 * ncells) return;
  const int lc = t >> 1, side = t & 1;
  const int cell = fast_cell(fg, p.ny, cell0 + lc);
  const int im = cell / p.ny, iy = cell - (cell / p.ny) * p.ny;
  const double Y = p.ymin + p.dy * iy;
  const double lnk = fg.lnm2[im] + (side ? -Y : Y);  // k = m/2 e^{+-y} (:224-225)
  // bmax = max(5 g hc / k, 5R) (:229-230); g = g2 for the second photon
  const double lnbmax = fmax((side ? fg.ln5ghc2 : fg.ln5ghc1) - lnk, fg.ln5R);
  const double d = (lnbmax - fg.lnbmin) * (1. / kNb);
  const double inv_d = 1. / d;  // the one FP64 division per side
  const double lnb0 = fg.lnbmin + 0.5 * d + ln_cosh_half(d);
  constexpr double inv_hK = (kKTabN - 1) / (kKTabU1 - kKTabU0);
  const double lnxk = lnk - fg.lnghc;  // x = b k / (g1 hc): fluxPoint and the form
                                       // integrand use g1 (:169, :198)
  SideC c;
  c.lnb0 = (float)lnb0;
  c.ld = (float)d;
  c.tg0 = (float)((lnb0 - fg.u0) * fg.inv_h);
  c.tgd = (float)(d * fg.inv_h);
  c.inv_tgd = (float)(inv_d * fg.h);
  c.lnw0 = logf(2.f * tanhf(0.5f * (float)d));  // b (bh - bl) = b^2 2 tanh(d/2)
  c.tk0 = (float)((lnb0 + lnxk - kKTabU0) * inv_hK);
  c.tkd = (float)(d * inv_hK);
  c.lnxk = (float)lnxk;
  c.lnc_pt = (float)(fg.lnc_pt + lnk);
  c.lnc_ff = (float)(fg.lnc_ff - lnk);
  // node counts below 2R and r_near: ln b_i <= ln X for i < floor((ln X - lnb0)/d) + 1
  auto count_le = [&](double lnX) {
    const double t = floor((lnX - lnb0) * inv_d) + 1.;
    return t < 0. ? 0 : (t > kNb ? kNb : (int)t);
  };
  c.n_form = p.isPoint ? 0 : count_le(fg.ln2R);
  c.n_near = count_le(fg.ln_rnear);
  c.tb0 = 0.f;
  c.tbd = 0.f;
  c.iw = 0;
  c.ww[0] = c.ww[1] = c.ww[2] = c.ww[3] = 0.f;
  if (!p.isPoint && ft.q32) {
    c.tb0 = (float)((lnb0 - ft.lb0) * ft.inv_hb);
    c.tbd = (float)(d * ft.inv_hb);
    const double tw = (lnk - ft.lw0) * ft.inv_hw;
    int p0 = (int)floor(tw) - 1;
    p0 = p0 < 0 ? 0 : (p0 > ft.nw - 4 ? ft.nw - 4 : p0);
    c.iw = p0;
    const float sw = (float)(tw - p0);
    const float s1 = sw - 1.f, s2 = sw - 2.f, s3 = sw - 3.f;
    c.ww[0] = -s1 * s2 * s3 * (1.f / 6.f);
    c.ww[1] = sw * s2 * s3 * 0.5f;
    c.ww[2] = -sw * s1 * s3 * 0.5f;
    c.ww[3] = sw * s1 * s2 * (1.f / 6.f);
  }
  out[t] = c;
}

// One warp per (row, side): the side's 120 nodes, lane l taking nodes l,
// l + 32, l + 64, l + 96.  Per node ln a_i in FP32 log space (point flux from
// the S(ln x) table; form-factor flux from the Q(w, b) table read at the node,
// 4 x 4 Lagrange weights in ln w and ln b; or the plain path's node fluxes),
// then the side's largest near-node ln a (warp maximum), the normalised
// weights an_i = a_i / max near a and the near / far sums (warp sums).  Per
// side the warp writes either its node list (kNodeStride floats: [0] tg0, [1]
// tgd, [2] the near count as int bits, [4 + i] an_i of the near nodes) or its
// dense row on the radial grid (A_side[p0_i + m] += an_i phi_m(s_i); side 0 as
// a bf16 hi / lo pair, side 1 in FP32), and side_part[row][side] = (ln scale,
// near sum, far sum).  No block barrier: rows are independent warps.
constexpr int kWeightWarps = 8;

__global__ void __launch_bounds__(kWeightWarps * 32) k_fast_weights(
    LumiParams p, FastGrid fg, FluxTabs ft, int cell0, int ncells, int nrows_pad,
    const SideC* __restrict__ sides, const double* __restrict__ flux_nodes, int dense_mask,
    __nv_bfloat16* __restrict__ ah, __nv_bfloat16* __restrict__ al, float* __restrict__ a2,
    float* __restrict__ nodes, float4* __restrict__ side_part) {
  __shared__ __align__(16) float s_row[kWeightWarps][kMaxP];  // a dense row per warp
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gw = blockIdx.x * kWeightWarps + warp;
  const int lc = gw >> 1, side = gw & 1;
  if (lc >= nrows_pad) return;  // whole warps leave; nothing below waits for others
  const bool dense = (dense_mask >> side) & 1;
  const int P = fg.P;
  if (lc >= ncells) {  // padding rows of the last 128-row tile
    if (lane == 0) side_part[2 * lc + side] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (!dense) {
      if (lane == 0)
        *reinterpret_cast<float4*>(nodes + ((size_t)lc * 2 + side) * kNodeStride) =
            make_float4(0.f, 1.f, 0.f, 0.f);
    } else {
      const size_t row = (size_t)lc * P;
      for (int q = 4 * lane; q < P; q += 128) {
        if (side == 0) {
          *reinterpret_cast<uint2*>(ah + row + q) = make_uint2(0u, 0u);
          *reinterpret_cast<uint2*>(al + row + q) = make_uint2(0u, 0u);
        } else {
          *reinterpret_cast<float4*>(a2 + row + q) = make_float4(0.f, 0.f, 0.f, 0.f);
        }
      }
    }
    return;
  }
  const int cell = fast_cell(fg, p.ny, cell0 + lc);
  const int iy = cell - (cell / p.ny) * p.ny;
  const SideC c = sides[2 * lc + side];
  // ln a_i of this lane's nodes
  float la[4];
  bool nr[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int i = lane + 32 * j;
    la[j] = -INFINITY;
    nr[j] = false;
    if (i >= kNb) continue;
    const float lnb = fmaf((float)i, c.ld, c.lnb0);
    nr[j] = i < c.n_near;
    if (flux_nodes) {  // the plain path's node fluxes (QAGS / K0, K1)
      const bool mir = side == 1 && p.mirror != nullptr && p.mirror[iy] >= 0;
      const double f = mir ? flux_nodes[((size_t)(lc + p.mirror[iy] - iy) * 2) * kNb + i]
                           : flux_nodes[((size_t)lc * 2 + side) * kNb + i];
      if (f > 0.) la[j] = (float)log(f) + 2.f * lnb + c.lnw0;
    } else if (i >= c.n_form) {  // point flux: ln N = ln(factor k/g^2) + S - 2x
      const float tk = fmaf((float)i, c.tkd, c.tk0);
      if (tk <= (float)(kKTabN - 1)) {  // x <= 300; beyond, the flux is taken as zero
        float w[4];
        const int i0 = lag4f(tk, kKTabN, w);
        const float S = w[0] * __ldg(ft.s32 + i0) + w[1] * __ldg(ft.s32 + i0 + 1) +
                        w[2] * __ldg(ft.s32 + i0 + 2) + w[3] * __ldg(ft.s32 + i0 + 3);
        // x up to 300 enters as e^{-2x}: its relative error is multiplied by
        // 2x, so x takes the accurate expf (not the approximate __expf)
        const float x = expf(lnb + c.lnxk);
        la[j] = c.lnc_pt + S - 2.f * x + 2.f * lnb + c.lnw0;
      }
    } else {  // form-factor flux: N = factor Q^2 / (A^2 k), Q from the table at (k, b_i)
      float wb[4];
      const int j0 = lag4f(fmaf((float)i, c.tbd, c.tb0), ft.nb, wb);
      const float* q = ft.q32 + (size_t)c.iw * ft.nb + j0;
      float Q = 0.f;
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const float* qr = q + (size_t)r * ft.nb;
        Q = fmaf(c.ww[r],
                 wb[0] * __ldg(qr) + wb[1] * __ldg(qr + 1) + wb[2] * __ldg(qr + 2) +
                     wb[3] * __ldg(qr + 3),
                 Q);
      }
      if (Q != 0.f) la[j] = c.lnc_ff + 2.f * __logf(fabsf(Q)) + 2.f * lnb + c.lnw0;
    }
  }
  // the side's largest near-node ln a
  float m = -INFINITY;
#pragma unroll
  for (int j = 0; j < 4; ++j)
    if (nr[j]) m = fmaxf(m, la[j]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (m == -INFINITY) m = 0.f;  // a side without flux: all weights 0
  float an[4], sn = 0.f, sf = 0.f;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    an[j] = la[j] == -INFINITY ? 0.f : __expf(la[j] - m);
    if (nr[j]) sn += an[j];
    else sf += an[j];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sn += __shfl_xor_sync(0xffffffffu, sn, o);
    sf += __shfl_xor_sync(0xffffffffu, sf, o);
  }
  if (lane == 0) side_part[2 * lc + side] = make_float4(m, sn, sf, 0.f);
  if (!dense) {
    float* out = nodes + ((size_t)lc * 2 + side) * kNodeStride;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int i = lane + 32 * j;
      if (i < kNb) out[4 + i] = nr[j] ? an[j] : 0.f;
    }
    if (lane == 0)
      *reinterpret_cast<float4*>(out) = make_float4(c.tg0, c.tgd, __int_as_float(c.n_near), 0.f);
    return;
  }
  // dense row: A_side[p0_i + m] += an_i phi_m(s_i).  Nodes i = r (mod np) go
  // in pass r, np = ceil(4.5 / spacing): within a pass the 4-point stencils
  // are disjoint, so no atomics and a fixed summation order.
  float* row = s_row[warp];
  for (int q = 4 * lane; q < P; q += 128)
    *reinterpret_cast<float4*>(row + q) = make_float4(0.f, 0.f, 0.f, 0.f);
  __syncwarp();
  const int np = (int)ceilf(4.5f * c.inv_tgd);
  if (np == 1) {
    // stencils 4.5 or more points apart (always so for the form-factor flux):
    // each column takes at most one node's value, stored without a read
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int i = lane + 32 * j;
      if (i < kNb && nr[j]) {
        const float t = fmaf((float)i, c.tgd, c.tg0);
        const int p0 = (int)floorf(t) - 1;  // in [0, P-4]: the host checks the grid's span
        const float s = t - (float)p0;
        const float s1 = s - 1.f, s2 = s - 2.f, s3 = s - 3.f;
        const float a = an[j];
        float* r = row + p0;
        r[0] = a * (-s1 * s2 * s3 * (1.f / 6.f));
        r[1] = a * (s * s2 * s3 * 0.5f);
        r[2] = a * (-s * s1 * s3 * 0.5f);
        r[3] = a * (s * s1 * s2 * (1.f / 6.f));
      }
    }
    __syncwarp();
  } else {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int i = lane + 32 * j;
      for (int pass = 0; pass < np; ++pass) {
        if (i < kNb && nr[j] && i % np == pass) {
          const float t = fmaf((float)i, c.tgd, c.tg0);
          const int p0 = (int)floorf(t) - 1;  // in [0, P-4]: the host checks the grid's span
          const float s = t - (float)p0;
          const float s1 = s - 1.f, s2 = s - 2.f, s3 = s - 3.f;
          const float a = an[j];
          float* r = row + p0;
          r[0] = fmaf(a, -s1 * s2 * s3 * (1.f / 6.f), r[0]);
          r[1] = fmaf(a, s * s2 * s3 * 0.5f, r[1]);
          r[2] = fmaf(a, -s * s1 * s3 * 0.5f, r[2]);
          r[3] = fmaf(a, s * s1 * s2 * (1.f / 6.f), r[3]);
        }
        __syncwarp();
      }
    }
  }
  const size_t base = (size_t)lc * P;
  for (int q = 4 * lane; q < P; q += 128) {
    const float4 x = *reinterpret_cast<const float4*>(row + q);
    if (side == 1) {
      *reinterpret_cast<float4*>(a2 + base + q) = x;
      continue;
    }
    const __nv_bfloat162 h01 = __floats2bfloat162_rn(x.x, x.y);
    const __nv_bfloat162 h23 = __floats2bfloat162_rn(x.z, x.w);
    const float2 f01 = __bfloat1622float2(h01), f23 = __bfloat1622float2(h23);
    const __nv_bfloat162 l01 = __floats2bfloat162_rn(x.x - f01.x, x.y - f01.y);
    const __nv_bfloat162 l23 = __floats2bfloat162_rn(x.z - f23.x, x.w - f23.y);
    uint2 hv, lv;
    hv.x = *reinterpret_cast<const uint32_t*>(&h01);
    hv.y = *reinterpret_cast<const uint32_t*>(&h23);
    lv.x = *reinterpret_cast<const uint32_t*>(&l01);
    lv.y = *reinterpret_cast<const uint32_t*>(&l23);
    *reinterpret_cast<uint2*>(ah + base + q) = hv;
    *reinterpret_cast<uint2*>(al + base + q) = lv;
  }
}

// P(20 fm) and c = P(20) sum_k w_k into out[0], out[1] (device-side, for
// captured scans that may not read them back to the host)
__global__ void k_far_consts(SplineU brk, int has_brk, LumiParams p, double* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const double P20 = has_brk ? spline_eval(brk, 20.) : 1.;
  double c = 0.;
  for (int q = 0; q < 5; ++q) c += P20 * 1. * p.wk[q];
  out[0] = P20;
  out[1] = c;
}

// L = 2 pi^2 M dm dy e^{ln scale0 + ln scale1} (c (S0far S1 + S0near S1far) +
// sum over the N tiles of the contraction's partial row-dots), per row; the
// side sums and scales come from k_fast_weights (side_part[row][side]).
__global__ void k_fast_finish(LumiParams p, int cell0, int ncells, int ntiles, double c_far,
                              const double* __restrict__ c_far_d,
                              const float* __restrict__ partial, const float4* __restrict__ side_part,
                              double* __restrict__ lumi, FastGrid fg, const int* __restrict__ rep_mir,
                              int delta) {
  const int lc = blockIdx.x * blockDim.x + threadIdx.x;
  if (lc >= ncells) return;
  const int cell = fast_cell(fg, p.ny, cell0 + lc);
  const int im = cell / p.ny;
  const double M = p.mmin + p.dm * im;
  double t2 = 0.;
  for (int t = 0; t < ntiles; ++t) t2 += (double)partial[(size_t)lc * ntiles + t];
  const float4 s0 = side_part[2 * lc], s1 = side_part[2 * lc + 1];  // (ln scale, near, far)
  // the constant part of the survival kernel, c (S0 S1 - S0near S1near) --
  // or, when the contraction took G - c (delta), c S0 S1
  double far;
  if (delta)
    far = ((double)s0.y + (double)s0.z) * ((double)s1.y + (double)s1.z);
  else
    far = (double)(s0.z * (s1.y + s1.z) + s0.y * s1.z);
  const double cf = c_far_d ? c_far_d[1] : c_far;
  const double s = exp((double)s0.x + (double)s1.x) * (cf * far + t2);
  const double v = 2 * kPi * kPi * M * s * p.dm * p.dy;
  lumi[cell] = v;
  if (fg.rep_y) {  // the mirror rapidity's cell
    const int j = (cell0 + lc) % fg.n_rep_y, iym = __ldg(rep_mir + j);
    if (iym >= 0) lumi[im * p.ny + iym] = v;
  }
}

// reference contraction in FP64 for the self-test
__global__ void k_contract_ref(const __nv_bfloat16* __restrict__ ah, const __nv_bfloat16* __restrict__ al,
                               const __nv_bfloat16* __restrict__ gh, const __nv_bfloat16* __restrict__ gl,
                               const float* __restrict__ a2, int ncells, int P, double* __restrict__ out) {
  const int c = blockIdx.x;
  double acc = 0.;
  for (int q = threadIdx.x; q < P; q += blockDim.x) {
    double t = 0.;
    for (int pp = 0; pp < P; ++pp) {
      const double a = (double)__bfloat162float(ah[(size_t)c * P + pp]) +
                       (double)__bfloat162float(al[(size_t)c * P + pp]);
      const double g = (double)__bfloat162float(gh[(size_t)q * P + pp]) +
                       (double)__bfloat162float(gl[(size_t)q * P + pp]);
      t += a * g;
    }
    acc += t * a2[(size_t)c * P + q];
  }
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[c] = red[0];
}

__global__ void k_fill_random(__nv_bfloat16* h, __nv_bfloat16* l, float* f, size_t n, uint64_t seed,
                              int signed_vals) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t x = (i + 1) * 0x9E3779B97F4A7C15ull ^ seed;
  x ^= x >> 31; x *= 0xBF58476D1CE4E5B9ull; x ^= x >> 27; x *= 0x94D049BB133111EBull; x ^= x >> 33;
  double v = (double)(x >> 11) * (1.0 / 9007199254740992.0);
  if (signed_vals) v = 2. * v - 1.;
  if (h) {
    const __nv_bfloat16 hi = __double2bfloat16(v);
    h[i] = hi;
    l[i] = __double2bfloat16(v - (double)__bfloat162float(hi));
  }
  if (f) f[i] = (float)v;
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* ptr = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ptr);
  }
  return fn;
}

// 2-D bf16 tensor map, rows x cols (cols contiguous), box = box_rows x 64.
cudaError_t make_map(CUtensorMap* m, const void* base, uint64_t rows, uint64_t cols,
                     uint32_t box_rows) {
  auto fn = encode_fn();
  if (!fn) return cudaErrorNotSupported;
  cuuint64_t dims[2] = {cols, rows};
  cuuint64_t strides[1] = {cols * 2};
  cuuint32_t box[2] = {(cuuint32_t)BK, box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides,
                  box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// 3-D bf16 tensor map over [planes][rows][cols] (cols contiguous), box =
// box_rows x 64 x 1: the stacked survival kernels of several configurations.
cudaError_t make_map3(CUtensorMap* m, const void* base, uint64_t planes, uint64_t rows,
                      uint64_t cols, uint32_t box_rows) {
  auto fn = encode_fn();
  if (!fn) return cudaErrorNotSupported;
  cuuint64_t dims[3] = {cols, rows, planes};
  cuuint64_t strides[2] = {cols * 2, rows * cols * 2};
  cuuint32_t box[3] = {(cuuint32_t)BK, box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides,
                  box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// 2-D FP32 tensor map, rows x cols (cols contiguous), box = box_rows x 32
// (128-byte rows, SWIZZLE_128B as the bf16 maps).
cudaError_t make_map_f32(CUtensorMap* m, const void* base, uint64_t rows, uint64_t cols,
                         uint32_t box_rows) {
  auto fn = encode_fn();
  if (!fn) return cudaErrorNotSupported;
  cuuint64_t dims[2] = {cols, rows};
  cuuint64_t strides[1] = {cols * 4};
  cuuint32_t box[2] = {(cuuint32_t)kT32K, box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base), dims, strides,
                  box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar,
                                            int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y), "r"(z)
      : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Work item of the persistent contraction: a 128-row tile of the stacked
// operands, one N tile of the survival kernel, and the configuration whose
// kernel plane it uses.
// One work item: an M tile of rows x an N tile of the radial grid.  pack:
// bits 0-7 the tile's valid rows (<= 128); bits 8-15 / 16-23 the item's K
// tiles [lo, hi), hi = 0 for all of them -- the K tiles where the survival
// kernel's N tile is nonzero (the delta form, G - c, is zero on the others).
struct PersItem {
  int mtile, ntile, config, pack;
};

__device__ __forceinline__ int item_rows(const PersItem& w) { return w.pack & 0xff; }

// The K tiles an item multiplies: its own range within [kt0, ktiles) (kt0:
// the first K tile with a nonzero A1 column in any row).  An empty range keeps
// the single tile kt0, whose product is zero -- its A1 or its survival tile
// is -- so that every item has an accumulator to read.
struct KRange {
  int lo, hi;
};
__device__ __forceinline__ KRange item_krange(const PersItem& w, int kt0, int ktiles) {
  const int e = (w.pack >> 16) & 0xff;
  if (e == 0) return {kt0, ktiles};
  const int a = (w.pack >> 8) & 0xff;
  KRange r{a > kt0 ? a : kt0, e < ktiles ? e : ktiles};
  if (r.lo >= r.hi) r = {kt0, kt0 + 1};
  return r;
}

struct PersArgs {
  const PersItem* items;
  int nitems, ktiles, P, ntiles;
  int kt0;  // first K tile with a nonzero A1 column in any row (the earlier ones are skipped)
  const float* a2;     // [rows of all tiles][P], or nullptr:
  const float* nodes;  // side 1's node lists [rows][2][kNodeStride] (k_fast_weights)
  float* partial;      // [rows][ntiles]
  unsigned* err;
};

// The epilogue's row-dot of one 16-column accumulator chunk v (columns lo ..
// lo + 15 of the radial grid) with side 1's dense row, gathered at its node
// stencils: sum_i an_i sum_m phi_m(s_i) v[p0_i + m - lo].  `cur` walks the
// nodes forward across the chunks of a row; scr is the thread's own 16-float
// scratch for the dynamically indexed reads.
__device__ __forceinline__ float gather_dot16(const float* v, int lo, float tg0, float tgd,
                                              int nn, const float* __restrict__ an, int& cur,
                                              float* scr, float acc) {
  const int hi = lo + 15;
  while (cur < nn && (int)floorf(fmaf((float)cur, tgd, tg0)) - 1 + 3 < lo) ++cur;
  if (cur >= nn || (int)floorf(fmaf((float)cur, tgd, tg0)) - 1 > hi) return acc;
#pragma unroll
  for (int j = 0; j < 16; ++j) scr[j] = v[j];
  for (int i = cur; i < nn; ++i) {
    const float t = fmaf((float)i, tgd, tg0);
    const int p0 = (int)floorf(t) - 1;
    if (p0 > hi) break;
    const float s = t - (float)p0;
    const float s1 = s - 1.f, s2 = s - 2.f, s3 = s - 3.f;
    const float w[4] = {-s1 * s2 * s3 * (1.f / 6.f), s * s2 * s3 * 0.5f, -s * s1 * s3 * 0.5f,
                        s * s1 * s2 * (1.f / 6.f)};
    const float a = __ldg(an + i);
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const int c = p0 + m - lo;
      if ((unsigned)c < 16u) acc = fmaf(a * w[m], scr[c], acc);
    }
  }
  return acc;
}

// Persistent form of k_contract: each CTA walks the work list (item
// blockIdx.x, + gridDim.x, ...).  The k-stage ring and its phases run on
// across items; the accumulator is double-buffered in TMEM (2 x TBN columns),
// so the MMAs of one item overlap the epilogue of the previous one.
// Template: TBN = N tile (256 or 128), TST = stages (2 or 3): the shapes the
// autotuner picks from.
template <int TBN, int TST>
__global__ void __launch_bounds__(192, 1) k_contract_pers(const __grid_constant__ CUtensorMap tAh,
                                                          const __grid_constant__ CUtensorMap tAl,
                                                          const __grid_constant__ CUtensorMap tBh,
                                                          const __grid_constant__ CUtensorMap tBl,
                                                          PersArgs args) {
  constexpr int kA = BM * BK * 2, kB = TBN * BK * 2, kStage = 2 * kA + 2 * kB;
  constexpr uint32_t kCols = 2 * TBN;
  constexpr uint32_t kId = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TBN >> 3) << 17) |
                           ((uint32_t)(BM >> 4) << 24);
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[TST], empty_bar[TST], accf[2], acce[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  __shared__ float ep_scr[4][32][17];  // gathered row-dot: one accumulator chunk per thread
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < TST; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], 4);  // one arrival per epilogue warp
    }
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_slot)),
                 "r"(kCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  // this CTA's items: blockIdx.x, + gridDim.x, ... (nmine of them)
  const int i0 = blockIdx.x, istep = gridDim.x;
  const int nmine = args.nitems > (int)blockIdx.x
                        ? (args.nitems - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x
                        : 0;

  if (warp == 0 && lane == 0) {
    // ---------------- TMA producer
    int g = 0;  // k tiles issued by this CTA
    bool ok = true;
    for (int it = 0; it < nmine && ok; ++it) {
      const PersItem w = args.items[i0 + it * istep];
      const KRange kr = item_krange(w, args.kt0, args.ktiles);
      for (int kt = kr.lo; kt < kr.hi; ++kt, ++g) {
        const int s = g % TST;
        if (g >= TST && !mbar_wait(&empty_bar[s], ((g / TST) & 1) ^ 1, args.err, 1u)) {
          ok = false;
          abort_flag = 1;
          break;
        }
        if (abort_flag) {
          ok = false;
          break;
        }
        uint8_t* st = smem + s * kStage;
        mbar_expect_tx(&full_bar[s], kStage);
        const int x = kt * BK;
        tma_load_2d(st, &tAh, &full_bar[s], x, w.mtile * BM);
        tma_load_2d(st + kA, &tAl, &full_bar[s], x, w.mtile * BM);
        tma_load_3d(st + 2 * kA, &tBh, &full_bar[s], x, w.ntile * TBN, w.config);
        tma_load_3d(st + 2 * kA + kB, &tBl, &full_bar[s], x, w.ntile * TBN, w.config);
      }
    }
    // the copies in flight land before the CTA exits
    for (int q = (g > TST ? g - TST : 0); q < g; ++q)
      mbar_wait(&full_bar[q % TST], (q / TST) & 1, args.err, 8u);
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer
    int g = 0;
    bool ok = true;
    for (int it = 0; it < nmine && ok; ++it) {
      const int b = it & 1;
      if (it >= 2 && !mbar_wait(&acce[b], ((it >> 1) & 1) ^ 1, args.err, 16u)) {
        ok = false;
        abort_flag = 1;
        break;
      }
      tc_fence_after();
      const uint32_t acc = tmem + (uint32_t)(b * TBN);
      const PersItem w = args.items[i0 + it * istep];
      const KRange kr = item_krange(w, args.kt0, args.ktiles);
      for (int kt = kr.lo; kt < kr.hi; ++kt, ++g) {
        const int s = g % TST;
        if (!mbar_wait(&full_bar[s], (g / TST) & 1, args.err, 2u)) {
          ok = false;
          abort_flag = 1;
          break;
        }
        tc_fence_after();
        const uint32_t base = smem_u32(smem + s * kStage);
        const uint32_t ah = base, al = base + kA, bh = base + 2 * kA, bl = base + 2 * kA + kB;
#pragma unroll
        for (int kk = 0; kk < BK / 16; ++kk) {
          const uint32_t off = kk * 32;
          const uint64_t dah = sw128_desc(ah + off), dal = sw128_desc(al + off);
          const uint64_t dbh = sw128_desc(bh + off), dbl = sw128_desc(bl + off);
          const uint32_t first = (kt > kr.lo || kk > 0) ? 1u : 0u;
          asm volatile(
              "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
              " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(acc),
              "l"(dah), "l"(dbh), "r"(kId), "r"(first));
          asm volatile(
              "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
              " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(acc),
              "l"(dah), "l"(dbl), "r"(kId), "r"(1u));
          asm volatile(
              "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
              " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(acc),
              "l"(dal), "l"(dbh), "r"(kId), "r"(1u));
        }
        umma_commit(&empty_bar[s]);
      }
      if (ok) umma_commit(&accf[b]);
    }
  } else if (warp >= 2) {
    // ---------------- epilogue: TMEM -> registers, row-dot with A2
    const int quad = warp & 3;
    constexpr int kPf = 4;  // A2 chunks (16 floats) in flight ahead of the row-dot
    for (int it = 0; it < nmine; ++it) {
      const PersItem w = args.items[i0 + it * istep];
      const int b = it & 1;
      const int row = quad * 32 + lane;
      const size_t grow = (size_t)w.mtile * BM + row;
      const bool vrow = row < item_rows(w);
      // the row's first A2 chunks are requested before the accumulator is
      // ready (they do not depend on it), the later ones kPf chunks ahead
      const float4* a4 =
          args.a2 ? reinterpret_cast<const float4*>(args.a2 + grow * args.P + w.ntile * TBN)
                  : nullptr;
      float4 xq[kPf][4];
      if (a4 && vrow) {
#pragma unroll
        for (int c = 0; c < kPf; ++c)
#pragma unroll
          for (int q = 0; q < 4; ++q) xq[c][q] = __ldg(a4 + 4 * c + q);
      }
      const bool ok = mbar_wait(&accf[b], (it >> 1) & 1, args.err, 4u);
      tc_fence_after();
      float acc = 0.f;
      if (ok && !args.a2) {  // side 1 from its node list
        const float* nd = args.nodes + (grow * 2 + 1) * kNodeStride;
        float tg0 = 0.f, tgd = 1.f;
        int nn = 0;
        if (row < item_rows(w)) {
          const float4 hd = __ldg(reinterpret_cast<const float4*>(nd));
          tg0 = hd.x;
          tgd = hd.y;
          nn = __float_as_int(hd.z);
        }
        int cur = 0;
        float* scr = &ep_scr[warp - 2][lane][0];
        for (int c0 = 0; c0 < TBN; c0 += 16) {
          float v[16];
          tmem_ld16(tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(b * TBN + c0), v);
          acc = gather_dot16(v, w.ntile * TBN + c0, tg0, tgd, nn, nd + 4, cur, scr, acc);
        }
      } else if (ok) {
#pragma unroll
        for (int c = 0; c < TBN / 16; ++c) {
          float v[16];
          tmem_ld16(tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(b * TBN + 16 * c), v);
          if (vrow) {
            const int sl = c % kPf;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              const float4 x = xq[sl][q];
              acc += v[4 * q] * x.x + v[4 * q + 1] * x.y + v[4 * q + 2] * x.z + v[4 * q + 3] * x.w;
            }
            if (c + kPf < TBN / 16) {
#pragma unroll
              for (int q = 0; q < 4; ++q) xq[sl][q] = __ldg(a4 + 4 * (c + kPf) + q);
            }
          }
        }
      }
      if (vrow) args.partial[grow * args.ntiles + w.ntile] = ok ? acc : 0.f;
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&acce[b]);
      if (!ok) break;
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols));
  }
}

// ---------------------------------------------------- fused contraction --
// k_contract_fused: the persistent contraction with the projection folded in.
// The A1 operand (side 0 on the radial grid, bf16 hi / lo) is built in shared
// memory by builder warps from the row's node list, stage by stage, instead
// of being read by TMA from an 8 KB-per-row array; the A2 row-dot of the
// epilogue gathers the accumulator at side 1's node stencils instead of
// reading a dense A2 row.  Only the survival kernel G still comes by TMA.
// Per CTA (448 threads):
//   warp 0       TMA producer of the G tiles (B operand);
//   warp 1       TMEM allocation and the single-thread tcgen05.mma issuer;
//   warps 2-5    epilogue: TMEM -> registers -> the gathered row-dot;
//   warps 6-13   A1 builders: two threads per row, 32 columns of a stage each.
// A stage is complete when the TMA transaction bytes have landed and the 8
// builder warps have arrived (full barrier of count 9); the builders write
// generic-proxy shared memory and fence it to the async proxy before they
// arrive.  A builder stages its 32 FP32 values in its own row of the stage's
// hi (first half) or lo (second half) tile, reads them back after the
// partner thread has read its half, and overwrites both rows with the bf16
// pair in the SWIZZLE_128B K-major layout the MMA descriptors expect.
constexpr int kBuildWarps = 8;
constexpr int kFusedThreads = (6 + kBuildWarps) * 32;

__device__ __forceinline__ int node_p0(float tg0, float tgd, int i) {
  return (int)floorf(fmaf((float)i, tgd, tg0)) - 1;
}

// 4-point Lagrange weights of a node at fractional offset s from its first
// stencil point (the projection's formula)
__device__ __forceinline__ void lag4_weights(float s, float w[4]) {
  const float s1 = s - 1.f, s2 = s - 2.f, s3 = s - 3.f;
  w[0] = -s1 * s2 * s3 * (1.f / 6.f);
  w[1] = s * s2 * s3 * 0.5f;
  w[2] = -s * s1 * s3 * 0.5f;
  w[3] = s * s1 * s2 * (1.f / 6.f);
}

__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

struct FusedArgs {
  const PersItem* items;
  int nitems, ktiles, P, ntiles;
  int kt0;  // first K tile with a nonzero A1 column in any row (the earlier ones are skipped)
  const float* nodes;  // [rows][2][kNodeStride] (k_fast_nodes)
  float* partial;      // [rows][ntiles]
  unsigned* err;
};

template <int TBN, int TST>
__global__ void __launch_bounds__(kFusedThreads, 1) k_contract_fused(
    const __grid_constant__ CUtensorMap tBh, const __grid_constant__ CUtensorMap tBl,
    FusedArgs args) {
  constexpr int kA = BM * BK * 2, kB = TBN * BK * 2, kStage = 2 * kA + 2 * kB;
  constexpr uint32_t kCols = 2 * TBN;
  constexpr uint32_t kId = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TBN >> 3) << 17) |
                           ((uint32_t)(BM >> 4) << 24);
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[TST], empty_bar[TST], accf[2], acce[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  __shared__ float ep_scr[4][32][17];  // epilogue: one 16-column accumulator chunk per thread
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < TST; ++s) {
      mbar_init(&full_bar[s], 1 + kBuildWarps);
      mbar_init(&empty_bar[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], 4);  // one arrival per epilogue warp
    }
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_slot)),
                 "r"(kCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  // this CTA's items: blockIdx.x, + gridDim.x, ... (nmine of them)
  const int i0 = blockIdx.x, istep = gridDim.x;
  const int nmine = args.nitems > (int)blockIdx.x
                        ? (args.nitems - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x
                        : 0;

  if (warp == 0) {
    if (lane == 0) {
      // ---------------- TMA producer: the G tiles
      int g = 0;
      bool ok = true;
      for (int it = 0; it < nmine && ok; ++it) {
        const PersItem w = args.items[i0 + it * istep];
        const KRange kr = item_krange(w, args.kt0, args.ktiles);
        for (int kt = kr.lo; kt < kr.hi; ++kt, ++g) {
          const int s = g % TST;
          if (g >= TST && !mbar_wait(&empty_bar[s], ((g / TST) & 1) ^ 1, args.err, 1u)) {
            ok = false;
            abort_flag = 1;
            break;
          }
          if (abort_flag) {
            ok = false;
            break;
          }
          uint8_t* st = smem + s * kStage;
          mbar_expect_tx(&full_bar[s], 2 * kB);
          const int x = kt * BK;
          tma_load_3d(st + 2 * kA, &tBh, &full_bar[s], x, w.ntile * TBN, w.config);
          tma_load_3d(st + 2 * kA + kB, &tBl, &full_bar[s], x, w.ntile * TBN, w.config);
        }
      }
      // the copies in flight land before the CTA exits
      for (int q = (g > TST ? g - TST : 0); q < g; ++q)
        mbar_wait(&full_bar[q % TST], (q / TST) & 1, args.err, 8u);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---------------- MMA issuer
      int g = 0;
      bool ok = true;
      for (int it = 0; it < nmine && ok; ++it) {
        const int b = it & 1;
        if (it >= 2 && !mbar_wait(&acce[b], ((it >> 1) & 1) ^ 1, args.err, 16u)) {
          ok = false;
          abort_flag = 1;
          break;
        }
        tc_fence_after();
        const uint32_t acc = tmem + (uint32_t)(b * TBN);
        const PersItem w = args.items[i0 + it * istep];
        const KRange kr = item_krange(w, args.kt0, args.ktiles);
        for (int kt = kr.lo; kt < kr.hi; ++kt, ++g) {
          const int s = g % TST;
          if (!mbar_wait(&full_bar[s], (g / TST) & 1, args.err, 2u)) {
            ok = false;
            abort_flag = 1;
            break;
          }
          tc_fence_after();
          const uint32_t base = smem_u32(smem + s * kStage);
          const uint32_t ah = base, al = base + kA, bh = base + 2 * kA, bl = base + 2 * kA + kB;
#pragma unroll
          for (int kk = 0; kk < BK / 16; ++kk) {
            const uint32_t off = kk * 32;
            const uint64_t dah = sw128_desc(ah + off), dal = sw128_desc(al + off);
            const uint64_t dbh = sw128_desc(bh + off), dbl = sw128_desc(bl + off);
            const uint32_t first = (kt > kr.lo || kk > 0) ? 1u : 0u;
            asm volatile(
                "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(acc),
                "l"(dah), "l"(dbh), "r"(kId), "r"(first));
            asm volatile(
                "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(acc),
                "l"(dah), "l"(dbl), "r"(kId), "r"(1u));
            asm volatile(
                "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(acc),
                "l"(dal), "l"(dbh), "r"(kId), "r"(1u));
          }
          umma_commit(&empty_bar[s]);
        }
        if (ok) umma_commit(&accf[b]);
      }
    }
  } else if (warp < 6) {
    // ---------------- epilogue: TMEM -> registers, row-dot gathered at side 1's nodes
    const int quad = warp & 3;
    const int row = quad * 32 + lane;
    float* scr = &ep_scr[warp - 2][lane][0];
    for (int it = 0; it < nmine; ++it) {
      const PersItem w = args.items[i0 + it * istep];
      const int b = it & 1;
      const bool ok = mbar_wait(&accf[b], (it >> 1) & 1, args.err, 4u);
      tc_fence_after();
      const size_t grow = (size_t)w.mtile * BM + row;
      const float* nd = args.nodes + (grow * 2 + 1) * kNodeStride;
      float tg0 = 0.f, tgd = 1.f;
      int nn = 0;
      if (row < item_rows(w)) {
        const float4 hd = __ldg(reinterpret_cast<const float4*>(nd));
        tg0 = hd.x;
        tgd = hd.y;
        nn = __float_as_int(hd.z);
      }
      int cur = 0;  // first node whose stencil may reach the current columns
      float acc = 0.f;
      if (ok) {
        for (int c0 = 0; c0 < TBN; c0 += 16) {
          float v[16];
          tmem_ld16(tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(b * TBN + c0), v);
          acc = gather_dot16(v, w.ntile * TBN + c0, tg0, tgd, nn, nd + 4, cur, scr, acc);
        }
      }
      if (row < item_rows(w)) args.partial[grow * args.ntiles + w.ntile] = ok ? acc : 0.f;
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&acce[b]);
      if (!ok) break;
    }
  } else {
    // ---------------- A1 builders: row r, columns 32h .. 32h+31 of each stage
    const int r = (warp - 6) * 16 + (lane >> 1);
    const int h = lane & 1;
    const uint32_t roff = (uint32_t)((r >> 3) * 1024 + (r & 7) * 128);
    const int sw = r & 7;
    int g = 0;
    bool ok = true;
    for (int it = 0; it < nmine && ok; ++it) {
      const PersItem w = args.items[i0 + it * istep];
      const size_t grow = (size_t)w.mtile * BM + r;
      const float* nd = args.nodes + grow * 2 * kNodeStride;  // side 0
      float tg0 = 0.f, tgd = 1.f;
      int nn = 0;
      if (r < item_rows(w)) {
        const float4 hd = __ldg(reinterpret_cast<const float4*>(nd));
        tg0 = hd.x;
        tgd = hd.y;
        nn = __float_as_int(hd.z);
      }
      int cur = 0;
      // node stencils 4.5 or more grid points apart never share a column
      // (first points floor(t_i) - 1 at least 4 apart after rounding; always
      // so for the form-factor flux, where b_max / b_min >= 100 gives >= 5)
      const bool disjoint = tgd >= 4.5f;
      const KRange kr = item_krange(w, args.kt0, args.ktiles);
      for (int kt = kr.lo; kt < kr.hi; ++kt, ++g) {
        const int s = g % TST;
        if (g >= TST && !mbar_wait(&empty_bar[s], ((g / TST) & 1) ^ 1, args.err, 32u)) {
          ok = false;
          abort_flag = 1;
        }
        ok = __all_sync(0xffffffffu, ok && !abort_flag);  // the warp leaves together
        if (!ok) break;
        uint8_t* st = smem + s * kStage;
        float* stg = reinterpret_cast<float*>(st + (h ? kA : 0) + roff);  // own 32 floats
        const int c_lo = kt * BK + 32 * h, c_hi = c_lo + 31;
        while (cur < nn && node_p0(tg0, tgd, cur) + 3 < c_lo) ++cur;
        float v[32];
        if (cur < nn && node_p0(tg0, tgd, cur) <= c_hi) {
          // FP32 staging in the own row, 16-byte chunks XOR-swizzled by row
#pragma unroll
          for (int q = 0; q < 8; ++q)
            *reinterpret_cast<float4*>(stg + ((q ^ sw) << 2)) = make_float4(0.f, 0.f, 0.f, 0.f);
          if (disjoint) {
            // stencils at least 4 points apart: every column gets at most one
            // node's value, stored without reading the staging back; two
            // nodes per iteration (independent loads and stores)
            for (int i = cur; i < nn; i += 2) {
              const float t0 = fmaf((float)i, tgd, tg0);
              const int q0 = (int)floorf(t0) - 1;
              if (q0 > c_hi) break;
              const bool two = i + 1 < nn;
              const float t1 = fmaf((float)(i + 1), tgd, tg0);
              const int q1 = (int)floorf(t1) - 1;
              const float a0 = __ldg(nd + 4 + i);
              const float a1 = two ? __ldg(nd + 5 + i) : 0.f;
              float w0[4], w1[4];
              lag4_weights(t0 - (float)q0, w0);
              lag4_weights(t1 - (float)q1, w1);
#pragma unroll
              for (int m = 0; m < 4; ++m) {
                const int c = q0 + m - c_lo;
                if ((unsigned)c < 32u) stg[(((c >> 2) ^ sw) << 2) | (c & 3)] = a0 * w0[m];
              }
              if (!two || q1 > c_hi) break;
#pragma unroll
              for (int m = 0; m < 4; ++m) {
                const int c = q1 + m - c_lo;
                if ((unsigned)c < 32u) stg[(((c >> 2) ^ sw) << 2) | (c & 3)] = a1 * w1[m];
              }
            }
          } else {
            for (int i = cur; i < nn; ++i) {
              const float t = fmaf((float)i, tgd, tg0);
              const int p0 = (int)floorf(t) - 1;
              if (p0 > c_hi) break;
              float wl[4];
              lag4_weights(t - (float)p0, wl);
              const float a = __ldg(nd + 4 + i);
#pragma unroll
              for (int m = 0; m < 4; ++m) {
                const int c = p0 + m - c_lo;
                if ((unsigned)c < 32u) {
                  float* e = stg + ((((c >> 2) ^ sw) << 2) | (c & 3));
                  *e = fmaf(a, wl[m], *e);
                }
              }
            }
          }
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const float4 x = *reinterpret_cast<const float4*>(stg + ((q ^ sw) << 2));
            v[4 * q] = x.x;
            v[4 * q + 1] = x.y;
            v[4 * q + 2] = x.z;
            v[4 * q + 3] = x.w;
          }
        } else {
#pragma unroll
          for (int j = 0; j < 32; ++j) v[j] = 0.f;
        }
        __syncwarp();  // the partner thread has read its staging (in this row's other half)
        // bf16 hi / lo of the 32 values: chunks 4h .. 4h+3 of the 128-byte row
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          uint32_t hw[4], lw[4];
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const float x0 = v[8 * q + 2 * e], x1 = v[8 * q + 2 * e + 1];
            const __nv_bfloat162 hh = __floats2bfloat162_rn(x0, x1);
            const float2 f = __bfloat1622float2(hh);
            const __nv_bfloat162 ll = __floats2bfloat162_rn(x0 - f.x, x1 - f.y);
            hw[e] = *reinterpret_cast<const uint32_t*>(&hh);
            lw[e] = *reinterpret_cast<const uint32_t*>(&ll);
          }
          const uint32_t ch = (uint32_t)(((4 * h + q) ^ sw) << 4);
          *reinterpret_cast<uint4*>(st + roff + ch) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
          *reinterpret_cast<uint4*>(st + kA + roff + ch) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
        }
        fence_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(&full_bar[s]);
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols));
  }
}

// Synthetic node lists for the autotuner: every row and side with 120 near
// nodes spread like a form-factor row (spacing 5 - 5.6 grid points from 157).
__global__ void k_fill_nodes_synthetic(float* __restrict__ nodes, int rows) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= rows * 2) return;
  float* o = nodes + (size_t)t * kNodeStride;
  o[0] = 157.f + (float)(t % 61) * 0.5f;
  o[1] = 5.f + (float)(t % 7) * 0.1f;
  o[2] = __int_as_float(kNb);
  o[3] = 0.f;
  for (int i = 0; i < kNb; ++i) o[4 + i] = 1.f / (1.f + (float)i);
}

template <int TBN, int TST>
constexpr int pers_smem() {
  return TST * (2 * BM * BK * 2 + 2 * TBN * BK * 2) + 1024;
}

}  // namespace

int fast_grid_points() { return 1024; }

// The first K tile (64 radial points) that can hold a near node's stencil:
// nodes lie at b >= b_min, their stencils start at floor(t) - 1 with t the
// node's grid coordinate, so the columns below floor((ln b_min - u0)/h) - 1
// are zero in every row (one more column of margin here).
int fast_first_ktile(double b_min, double u0, double h) {
  const int p0 = (int)std::floor((std::log(b_min) - u0) / h) - 2;
  return p0 < 0 ? 0 : p0 / BK;
}

// For azimuth cosine c, b^2 = rp^2 + rq^2 + 2 rp rq c < T holds for rq in
// (-rp c - d, -rp c + d), d = sqrt(T - rp^2 (1 - c^2)): per grid row p the
// columns q of that interval (one column of margin each side), per tile pair
// the union over p and the azimuths.  T = 400 (1 + 1e-3) covers the FP32
// radii and b^2 of k_fast_G.
void delta_tile_ranges(int P, double u0, double h, const double* cosk, int ncos, int tbn, int bk,
                       std::vector<std::pair<int, int>>& out) {
  const int nt = P / tbn;
  std::vector<int> lo(nt, 1 << 30), hi(nt, -1);
  const double T = 400. * (1. + 1e-3);
  for (int p = 0; p < P; ++p) {
    const double rp = std::exp(u0 + p * h);
    for (int k = 0; k < ncos; ++k) {
      const double c = cosk[k];
      const double disc = T - rp * rp * (1. - c * c);
      if (disc < 0.) continue;
      const double d = std::sqrt(disc), rm = -rp * c - d, rpl = -rp * c + d;
      if (rpl <= 0.) continue;
      int q0 = rm > 0. ? (int)std::floor((std::log(rm) - u0) / h) - 1 : 0;
      int q1 = (int)std::ceil((std::log(rpl) - u0) / h) + 1;
      q0 = std::max(q0, 0);
      q1 = std::min(q1, P - 1);
      for (int t = q0 / tbn; q0 <= q1 && t <= q1 / tbn; ++t) {
        lo[t] = std::min(lo[t], p / bk);
        hi[t] = std::max(hi[t], p / bk + 1);
      }
    }
  }
  out.resize(nt);
  for (int t = 0; t < nt; ++t)
    out[t] = hi[t] < 0 ? std::make_pair(P / bk, P / bk) : std::make_pair(lo[t], hi[t]);
}

// CTA b takes items b, b + grid, ...: the grid items of one round run side by
// side, and the list keeps the N tiles of a row tile adjacent, so that a
// round's CTAs share their row tiles' A reads in L2.  With items of unequal
// work (their K ranges per N tile) a CTA would meet the same N tile in every
// round; rotating round r by r positions deals each CTA every N tile in turn.
void rotate_rounds(std::vector<int4>& items, int grid) {
  const int n = (int)items.size();
  if (grid < 2 || n < 2) return;
  std::vector<int4> out(items.size());
  for (int r0 = 0, r = 0; r0 < n; r0 += grid, ++r) {
    const int m = std::min(grid, n - r0);
    for (int b = 0; b < m; ++b) out[r0 + b] = items[r0 + (b + r) % m];
  }
  items.swap(out);
}

cudaError_t launch_contract(const void* ah, const void* al, const void* gh, const void* gl,
                            const float* a2, int ncells_pad, int ncells, int P, float* partial,
                            unsigned* d_err, cudaStream_t st) {
  if (ncells_pad % BM != 0 || P % BN != 0 || P % BK != 0) return cudaErrorInvalidValue;
  CUtensorMap tAh, tAl, tBh, tBl;
  cudaError_t e;
  if ((e = make_map(&tAh, ah, ncells_pad, P, BM)) != cudaSuccess) return e;
  if ((e = make_map(&tAl, al, ncells_pad, P, BM)) != cudaSuccess) return e;
  if ((e = make_map(&tBh, gh, P, P, BN)) != cudaSuccess) return e;
  if ((e = make_map(&tBl, gl, P, P, BN)) != cudaSuccess) return e;
  static std::atomic<uint64_t> attr{0};  // devices with the limit raised
  {
    const cudaError_t ea = smem_attr_once(attr, k_contract, kContractSmem);
    if (ea != cudaSuccess) return ea;
  }
  ContractArgs args{P / BK, ncells, P, P / BN, a2, partial, d_err, nullptr, nullptr, nullptr, 0};
  dim3 grid(P / BN, ncells_pad / BM);
  note_launch();
  k_contract<<<grid, 192, kContractSmem, st>>>(tAh, tAl, tBh, tBl, args);
  return cudaGetLastError();
}

cudaError_t launch_contract_pers(const void* ah, const void* al, const void* gh, const void* gl,
                                 int nconf, int rows_total, int P, const void* items, int nitems,
                                 const float* a2, float* partial, unsigned* d_err, int shape,
                                 int grid, cudaStream_t st, const float* nodes, int kt0) {
  // shape 0: N tile 256, 2 stages; shape 1: N tile 128, 3 stages
  const int tbn = shape == 0 ? 256 : 128;
  if (P % tbn != 0 || P % BK != 0 || rows_total % BM != 0 || nitems <= 0 || grid <= 0 ||
      (!a2 && !nodes))
    return cudaErrorInvalidValue;
  CUtensorMap tAh, tAl, tBh, tBl;
  cudaError_t e;
  if ((e = make_map(&tAh, ah, rows_total, P, BM)) != cudaSuccess) return e;
  if ((e = make_map(&tAl, al, rows_total, P, BM)) != cudaSuccess) return e;
  if ((e = make_map3(&tBh, gh, nconf, P, P, tbn)) != cudaSuccess) return e;
  if ((e = make_map3(&tBl, gl, nconf, P, P, tbn)) != cudaSuccess) return e;
  if (kt0 < 0 || kt0 >= P / BK) return cudaErrorInvalidValue;
  PersArgs args{static_cast<const PersItem*>(items), nitems, P / BK, P, P / tbn, kt0, a2, nodes,
                partial, d_err};
  if (grid > nitems) grid = nitems;
  if (shape == 0) {
    static std::atomic<uint64_t> attr{0};  // devices with the limit raised
    constexpr int sm = pers_smem<256, 2>();
    {
      const cudaError_t ea = smem_attr_once(attr, k_contract_pers<256, 2>, sm);
      if (ea != cudaSuccess) return ea;
    }
    note_launch();
    k_contract_pers<256, 2><<<grid, 192, sm, st>>>(tAh, tAl, tBh, tBl, args);
  } else {
    static std::atomic<uint64_t> attr{0};  // devices with the limit raised
    constexpr int sm = pers_smem<128, 3>();
    {
      const cudaError_t ea = smem_attr_once(attr, k_contract_pers<128, 3>, sm);
      if (ea != cudaSuccess) return ea;
    }
    note_launch();
    k_contract_pers<128, 3><<<grid, 192, sm, st>>>(tAh, tAl, tBh, tBl, args);
  }
  return cudaGetLastError();
}

int contract_item_bytes() { return (int)sizeof(PersItem); }

cudaError_t launch_contract_fused(const void* gh, const void* gl, int nconf, int rows_total, int P,
                                  const void* items, int nitems, const float* nodes,
                                  float* partial, unsigned* d_err, int shape, int grid,
                                  cudaStream_t st, int kt0) {
  // shape 0: N tile 256, 2 stages; shape 1: N tile 128, 3 stages
  const int tbn = shape == 0 ? 256 : 128;
  if (P % tbn != 0 || P % BK != 0 || P > kMaxP || rows_total % BM != 0 || nitems <= 0 ||
      grid <= 0 || !nodes)
    return cudaErrorInvalidValue;
  CUtensorMap tBh, tBl;
  cudaError_t e;
  if ((e = make_map3(&tBh, gh, nconf, P, P, tbn)) != cudaSuccess) return e;
  if ((e = make_map3(&tBl, gl, nconf, P, P, tbn)) != cudaSuccess) return e;
  if (kt0 < 0 || kt0 >= P / BK) return cudaErrorInvalidValue;
  FusedArgs args{static_cast<const PersItem*>(items), nitems, P / BK, P, P / tbn, kt0, nodes,
                 partial, d_err};
  if (grid > nitems) grid = nitems;
  if (shape == 0) {
    static std::atomic<uint64_t> attr{0};  // devices with the limit raised
    constexpr int sm = pers_smem<256, 2>();
    {
      const cudaError_t ea = smem_attr_once(attr, k_contract_fused<256, 2>, sm);
      if (ea != cudaSuccess) return ea;
    }
    note_launch();
    k_contract_fused<256, 2><<<grid, kFusedThreads, sm, st>>>(tBh, tBl, args);
  } else {
    static std::atomic<uint64_t> attr{0};  // devices with the limit raised
    constexpr int sm = pers_smem<128, 3>();
    {
      const cudaError_t ea = smem_attr_once(attr, k_contract_fused<128, 3>, sm);
      if (ea != cudaSuccess) return ea;
    }
    note_launch();
    k_contract_fused<128, 3><<<grid, kFusedThreads, sm, st>>>(tBh, tBl, args);
  }
  return cudaGetLastError();
}

int fast_node_floats_per_row() { return 2 * kNodeStride; }

cudaError_t launch_fill_nodes_synthetic(float* nodes, int rows, cudaStream_t st) {
  note_launch();
  k_fill_nodes_synthetic<<<(2 * rows + 255) / 256, 256, 0, st>>>(nodes, rows);
  return cudaGetLastError();
}

cudaError_t launch_gemm_bf16x3(const void* ah, const void* al, const void* bh, const void* bl,
                               int M, int N, int K, float* out_f32, void* out_hi, void* out_lo,
                               unsigned* d_err, cudaStream_t st) {
  // A [M_pad][K], B [N][K] (K contiguous, bf16 hi/lo); D = A B^T, M_pad = M
  // rounded up to 128 rows of A (the rows beyond M are read, not stored)
  if (M <= 0 || N % BN != 0 || K % BK != 0 || (!out_f32 && !(out_hi && out_lo)))
    return cudaErrorInvalidValue;
  const int Mpad = (M + BM - 1) / BM * BM;
  CUtensorMap tAh, tAl, tBh, tBl;
  cudaError_t e;
  if ((e = make_map(&tAh, ah, Mpad, K, BM)) != cudaSuccess) return e;
  if ((e = make_map(&tAl, al, Mpad, K, BM)) != cudaSuccess) return e;
  if ((e = make_map(&tBh, bh, N, K, BN)) != cudaSuccess) return e;
  if ((e = make_map(&tBl, bl, N, K, BN)) != cudaSuccess) return e;
  static std::atomic<uint64_t> attr{0};  // devices with the limit raised
  {
    const cudaError_t ea = smem_attr_once(attr, k_contract, kContractSmem);
    if (ea != cudaSuccess) return ea;
  }
  ContractArgs args{K / BK, M, K, N / BN, nullptr, nullptr, d_err, out_f32,
                    static_cast<__nv_bfloat16*>(out_hi), static_cast<__nv_bfloat16*>(out_lo), N};
  dim3 grid(N / BN, Mpad / BM);
  note_launch();
  k_contract<<<grid, 192, kContractSmem, st>>>(tAh, tAl, tBh, tBl, args);
  return cudaGetLastError();
}

cudaError_t launch_gemm_tf32(const float* a, const float* b, int M, int N, int K, float* out,
                             unsigned* d_err, cudaStream_t st) {
  // A [M_pad][K], B [N][K] FP32 (K contiguous); D = A B^T into out [M][N]
  if (M <= 0 || N % BN != 0 || K % kT32K != 0 || !out) return cudaErrorInvalidValue;
  const int Mpad = (M + BM - 1) / BM * BM;
  CUtensorMap tA, tB;
  cudaError_t e;
  if ((e = make_map_f32(&tA, a, Mpad, K, BM)) != cudaSuccess) return e;
  if ((e = make_map_f32(&tB, b, N, K, BN)) != cudaSuccess) return e;
  static std::atomic<uint64_t> attr{0};  // devices with the limit raised
  {
    const cudaError_t ea = smem_attr_once(attr, k_gemm_tf32, kT32Smem);
    if (ea != cudaSuccess) return ea;
  }
  dim3 grid(N / BN, Mpad / BM);
  note_launch();
  k_gemm_tf32<<<grid, 192, kT32Smem, st>>>(tA, tB, K / kT32K, M, N, out, d_err);
  return cudaGetLastError();
}

cudaError_t launch_pair_to_f32(const void* hi, const void* lo, size_t n, float* out,
                               cudaStream_t st) {
  note_launch();
  k_pair_to_f32<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
      static_cast<const __nv_bfloat16*>(hi), static_cast<const __nv_bfloat16*>(lo), n, out);
  return cudaGetLastError();
}

cudaError_t launch_fast_G(const LumiParams& p, double u0, double h, int P, double P20,
                          float4* d_gaa32, float4* d_brk32, void* gh, void* gl, cudaStream_t st,
                          const double* P20d, int convert, double* far_out, unsigned* err0,
                          int delta) {
  if (p.gaa.n - 1 > 200) return cudaErrorInvalidValue;
  GParams gp{};
  if (convert) {
    note_launch();
    k_coef_f32<<<(p.gaa.n - 1 + 255) / 256, 256, 0, st>>>(p.gaa.coef, d_gaa32, p.gaa.n - 1);
  }
  gp.gaa = SplineF{d_gaa32, (float)p.gaa.x0, (float)p.gaa.h, (float)p.gaa.inv_h, p.gaa.n};
  gp.has_brk = p.breakupMode != 1;
  if (gp.has_brk) {
    if (convert) {
      note_launch();
      k_coef_f32<<<(p.brk.n - 1 + 255) / 256, 256, 0, st>>>(p.brk.coef, d_brk32, p.brk.n - 1);
    }
    gp.brk = SplineF{d_brk32, (float)p.brk.x0, (float)p.brk.h, (float)p.brk.inv_h, p.brk.n};
  }
  gp.brk64 = p.brk;
  for (int k = 0; k < 5; ++k) gp.wkd[k] = p.wk[k];
  gp.far_out = far_out;
  gp.err0 = err0;
  gp.delta = delta;
  gp.P20 = (float)P20;
  for (int k = 0; k < 5; ++k) {
    gp.cosk[k] = (float)p.cosk[k];
    gp.wk[k] = (float)p.wk[k];
  }
  gp.u0 = (float)u0;
  gp.h = (float)h;
  gp.P20d = P20d;
  dim3 grid((P + 255) / 256, P);
  note_launch();
  k_fast_G<<<grid, 256, 0, st>>>(gp, P, (__nv_bfloat16*)gh, (__nv_bfloat16*)gl);
  return cudaGetLastError();
}

cudaError_t launch_fast_project(const LumiParams& p, double u0, double h, int P, int cell0,
                                int ncells, int ncells_pad, const double* lnm2, double c_far,
                                const double* flux_nodes, const FastFluxTables* t, void* d_sides,
                                void* ah, void* al, float* a2, void* side_part, cudaStream_t st,
                                const int* rep_y, int n_rep_y, int m0, float* nodes, int part) {
  if (rep_y && (flux_nodes || n_rep_y <= 0)) return cudaErrorInvalidValue;
  if (part < 0 || part > 2) return cudaErrorInvalidValue;
  // side 0: dense A1 (bf16 hi / lo) when ah and al are given, side 1: dense A2
  // (FP32) when a2 is; a side without a dense row writes its node list
  const int dense_mask = ((ah && al) ? 1 : 0) | (a2 ? 2 : 0);
  if (dense_mask != 3 && !nodes) return cudaErrorInvalidValue;
  if ((ah != nullptr) != (al != nullptr)) return cudaErrorInvalidValue;
  FastGrid fg{P, u0, h, 1.0 / h, 250.};
  fg.rep_y = rep_y;
  fg.n_rep_y = n_rep_y;
  fg.m0 = m0;
  fg.lnm2 = lnm2;
  fg.ln5ghc1 = std::log(5. * p.g1 * kHc);
  fg.ln5ghc2 = std::log(5. * p.g2 * kHc);
  fg.ln5R = std::log(5. * p.R);
  fg.lnbmin = std::log(p.isPoint ? p.R : 0.05 * p.R);
  fg.ln2R = std::log(2. * p.R);
  fg.ln_rnear = std::log(fg.r_near);
  fg.lnghc = std::log(p.g1 * kHc);
  fg.lnc_pt = std::log(p.factor / p.g1 / p.g1);
  fg.lnc_ff = std::log(p.factor / ((double)p.A * p.A));
  fg.c_far = c_far;
  FluxTabs ft{};
  if (P != kMaxP || P % 128 != 0 || ncells_pad % kWeightWarps != 0) return cudaErrorInvalidValue;
  // every near node's 4-point stencil inside the grid: b_min >= r_1, b <= r_near < r_{P-3}
  if (std::log(p.isPoint ? p.R : 0.05 * p.R) < u0 + h || std::log(250.) > u0 + (P - 4) * h)
    return cudaErrorInvalidValue;
  if (t) {
    ft = FluxTabs{t->st32, t->qt32, t->nw, t->nb, t->lw0, 1. / t->hw, t->lb0, 1. / t->hb};
  }
  SideC* sides = static_cast<SideC*>(d_sides);
  if (part != 2) {
    note_launch();
    k_fast_sides<<<(2 * ncells + 255) / 256, 256, 0, st>>>(p, fg, ft, cell0, ncells, sides);
  }
  if (part == 1) return cudaGetLastError();
  note_launch();
  k_fast_weights<<<2 * ncells_pad / kWeightWarps, kWeightWarps * 32, 0, st>>>(
      p, fg, ft, cell0, ncells, ncells_pad, sides, flux_nodes, dense_mask, (__nv_bfloat16*)ah,
      (__nv_bfloat16*)al, a2, nodes, static_cast<float4*>(side_part));
  return cudaGetLastError();
}

size_t fast_side_bytes() { return sizeof(SideC); }

int flux_table_part_doubles(int nw, int nb) { return 8 * nw * nb + nb; }  // slices + tail

cudaError_t launch_ktab(double g1, double* st, float* st32, cudaStream_t stream, void* d_lk,
                        int lk_ready) {
  if (!d_lk) {
    note_launch();
    k_ktab<<<(kKTabN + 255) / 256, 256, 0, stream>>>(g1, st, st32);
    return cudaGetLastError();
  }
  double2* lk = static_cast<double2*>(d_lk);
  if (!lk_ready) {
    note_launch();
    k_k01_logs<<<(kKTabN + 255) / 256, 256, 0, stream>>>(lk);
  }
  note_launch();
  k_ktab_logs<<<(kKTabN + 255) / 256, 256, 0, stream>>>(g1, lk, st, st32);
  return cudaGetLastError();
}

cudaError_t build_flux_tables(const LumiParams& p, FastFluxTables* t, double* d_qn, double* d_wn,
                              int nq, double* d_H, double* d_J, double* d_part, cudaStream_t st,
                              int w_lo, int with_ktab, cudaStream_t js, cudaEvent_t ev_j) {
  if (with_ktab) {
    note_launch();
    k_ktab<<<(kKTabN + 255) / 256, 256, 0, st>>>(p.g1, t->st, t->st32);
  }
  // Q rows [w_lo, nw) by the quadrature (w_lo a multiple of 64; the rows below
  // come from elsewhere)
  const int rows = t->nw - w_lo;
  if (!p.isPoint && rows > 0) {
    if (w_lo % 64 != 0) return cudaErrorInvalidValue;
    const double lw = t->lw0 + w_lo * t->hw;
    // J on js when given (ev_j recorded there, joined before H), else on st
    dim3 gj((t->nb + 255) / 256, nq);
    note_launch();
    k_qtab_J<<<gj, 256, 0, js ? js : st>>>(d_qn, nq, t->lb0, t->hb, t->nb, d_J);
    if (js) {
      cudaError_t e = cudaEventRecord(ev_j, js);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(st, ev_j, 0);
      if (e != cudaSuccess) return e;
    }
    dim3 gh((nq + 255) / 256, rows);
    double* d_tail = d_part + (size_t)8 * t->nw * t->nb;
    note_launch();
    k_qtab_H<<<gh, 256, 0, st>>>(p, d_qn, d_wn, nq, lw, t->hw, d_H, t->lb0, t->hb, t->nb,
                                 d_tail);
    // K = nq split into nq / kslice slices; d_part holds them
    const int nslice = nq % (8 * 16) == 0 ? 8 : 1;
    const int kslice = nq / nslice;
    dim3 gg(t->nb / 64, rows / 64, nslice);
    note_launch();
    k_qtab_product<<<gg, 256, 0, st>>>(reinterpret_cast<const float2*>(d_H),
                                       reinterpret_cast<const float2*>(d_J), d_part, rows, t->nb,
                                       nq, kslice);
    const size_t mn = (size_t)rows * t->nb;
    const size_t off = (size_t)w_lo * t->nb;
    note_launch();
    k_dgemm_reduce<<<(unsigned)((mn + 255) / 256), 256, 0, st>>>(d_part, nslice, mn, t->nb, d_tail,
                                                                 t->qt + off, t->qt32 + off);
  }
  return cudaGetLastError();
}

int flux_table_ktab_n() { return kKTabN; }
void flux_table_ktab_range(double* u0, double* u1) {
  *u0 = kKTabU0;
  *u1 = kKTabU1;
}

cudaError_t launch_far_consts(const LumiParams& p, int has_brk, double* d_out, cudaStream_t st) {
  note_launch();
  k_far_consts<<<1, 32, 0, st>>>(p.brk, has_brk, p, d_out);
  return cudaGetLastError();
}

cudaError_t launch_fast_finish(const LumiParams& p, int cell0, int ncells, int ntiles,
                               double c_far, const float* partial, const void* side_part,
                               double* lumi, cudaStream_t st, const double* c_far_d,
                               const int* rep_y, const int* rep_mir, int n_rep_y, int m0,
                               int delta) {
  FastGrid fg{};
  fg.rep_y = rep_y;
  fg.n_rep_y = n_rep_y;
  fg.m0 = m0;
  if (rep_y && (!rep_mir || n_rep_y <= 0)) return cudaErrorInvalidValue;
  note_launch();
  k_fast_finish<<<(ncells + 255) / 256, 256, 0, st>>>(p, cell0, ncells, ntiles, c_far, c_far_d,
                                                      partial, static_cast<const float4*>(side_part),
                                                      lumi, fg, rep_mir, delta);
  return cudaGetLastError();
}

cudaError_t contract_selftest(int ncells, int P, uint64_t seed, double* max_rel, double* ms) {
  const int pad = (ncells + BM - 1) / BM * BM;
  __nv_bfloat16 *ah, *al, *gh, *gl;
  float *a2, *partial;
  double *ref;
  unsigned* err;
  cudaMalloc(&ah, (size_t)pad * P * 2);
  cudaMalloc(&al, (size_t)pad * P * 2);
  cudaMalloc(&gh, (size_t)P * P * 2);
  cudaMalloc(&gl, (size_t)P * P * 2);
  cudaMalloc(&a2, (size_t)pad * P * 4);
  cudaMalloc(&partial, (size_t)ncells * (P / BN) * 4);
  cudaMalloc(&ref, (size_t)ncells * 8);
  cudaMalloc(&err, 4);
  cudaMemset(err, 0, 4);
  const size_t na = (size_t)pad * P, ng = (size_t)P * P;
  note_launch();
  k_fill_random<<<(unsigned)((na + 255) / 256), 256>>>(ah, al, nullptr, na, seed, 0);
  note_launch();
  k_fill_random<<<(unsigned)((ng + 255) / 256), 256>>>(gh, gl, nullptr, ng, seed ^ 0x1234, 0);
  note_launch();
  k_fill_random<<<(unsigned)((na + 255) / 256), 256>>>(nullptr, nullptr, a2, na, seed ^ 0x777, 0);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0);
  cudaError_t e = launch_contract(ah, al, gh, gl, a2, pad, ncells, P, partial, err, 0);
  cudaEventRecord(e1);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  float t = 0;
  cudaEventElapsedTime(&t, e0, e1);
  *ms = t;
  note_launch();
  k_contract_ref<<<ncells, 256>>>(ah, al, gh, gl, a2, ncells, P, ref);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  unsigned herr = 0;
  cudaMemcpy(&herr, err, 4, cudaMemcpyDeviceToHost);
  double worst = 0;
  if (e == cudaSuccess) {
    const int nt = P / BN;
    float* hp = new float[(size_t)ncells * nt];
    double* hr = new double[ncells];
    cudaMemcpy(hp, partial, (size_t)ncells * nt * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(hr, ref, (size_t)ncells * 8, cudaMemcpyDeviceToHost);
    for (int c = 0; c < ncells; ++c) {
      double s = 0;
      for (int t2 = 0; t2 < nt; ++t2) s += hp[(size_t)c * nt + t2];
      const double r = std::fabs(s - hr[c]) / std::fabs(hr[c]);
      if (!(r <= worst)) worst = r;
    }
    delete[] hp;
    delete[] hr;
  }
  *max_rel = herr ? -(double)herr : worst;
  cudaFree(ah); cudaFree(al); cudaFree(gh); cudaFree(gl); cudaFree(a2); cudaFree(partial);
  cudaFree(ref); cudaFree(err);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return e;
}

}  // namespace upcg
