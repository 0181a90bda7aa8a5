// Complex GEMM on the 5th-generation tensor cores (tcgen05) for sm_103a:
// C (M x N, complex64, column-major) = alpha op(A) op(B) + beta C with
// FP32-level accuracy from split-TF32x3 products accumulated in FP32.
//
// Each complex operand element x is split as x = hi + lo with hi = tf32(x),
// lo = tf32(x - hi).  The 4M complex product becomes one real GEMM
// D (M x 2N) = sum_seg A_seg . B_seg^T over six K-segments:
//   seg  A plane     B plane rows (2n | 2n+1)
//   0    hi(re A)    hi(re B) | hi(im B)
//   1    hi(re A)    lo(re B) | lo(im B)
//   2    lo(re A)    hi(re B) | hi(im B)
//   3    hi(im A)   -hi(im B) | hi(re B)
//   4    hi(im A)   -lo(im B) | lo(re B)
//   5    lo(im A)   -hi(im B) | hi(re B)
// so D[:, 2n] = re C[:, n] and D[:, 2n+1] = im C[:, n] (the lo*lo terms are
// dropped).  The gather kernels write the planes K-major (row-major M x K),
// TMA (128B swizzle) stages 128x32 / 256x32 FP32 tiles through a 4-deep
// mbarrier ring, and one elected thread issues tcgen05.mma kind::tf32 into
// TMEM.  The tensor core's FP32 accumulation loses about one ulp of the
// running sum per MMA step (measured: a relative error growing linearly with
// K, ~1e-7 per step), so the K loop is cut into chunks of CK k-blocks (8 MMA
// steps) accumulated alternately in two TMEM buffers (2 x 256 columns); eight
// epilogue warps drain each finished chunk with tcgen05.ld into FP32
// registers (round-to-nearest adds) while the next chunk accumulates in the
// other buffer, then write interleaved complex64 directly.
// Every mbarrier wait is bounded by a %globaltimer limit; on expiry the CTA
// records QT_FLAG_TIMEOUT-style status, drains its copies (bounded), frees
// TMEM and returns.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstring>
#include <mutex>

#include "qt_internal.cuh"

namespace {

constexpr int BM = 128, BN = 256, BK = 32;  // FP32 elements; BK * 4 B = one 128 B swizzle row
constexpr int STAGES = 4;
constexpr int A_TILE = BM * BK * 4;          // 16 KiB
constexpr int B_TILE = BN * BK * 4;          // 32 KiB
constexpr int STAGE_BYTES = A_TILE + B_TILE;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 256;
constexpr int NTHREADS = 320;                // warp 0 TMA, warp 1 MMA, warps 2-9 epilogue
constexpr int NEPI = 8;                      // epilogue warps: two per TMEM sub-partition
constexpr int CK = 2;                        // k-blocks per accumulation chunk
constexpr uint32_t TMEM_COLS = 512;          // two 256-column accumulator buffers
constexpr unsigned long long WAIT_NS = 2000000000ull;  // 2 s per wait
constexpr int NSEG = 6;
__constant__ int kSegA[NSEG] = {0, 0, 2, 1, 1, 3};
__constant__ int kSegB[NSEG] = {0, 1, 0, 2, 3, 2};

struct TcParams {
  int M, N, Kp, Mp, N2p;  // true complex M, N; padded K, M, 2N
  float2 alpha, beta;
  float2* C;
  int64_t ldc;
  int* status;            // nonzero on a timed-out wait
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait on an mbarrier phase; false when the time limit passed.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = now_ns();
  while (!mbar_try_wait(bar, parity))
    if (now_ns() - t0 > WAIT_NS) return false;
  return true;
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], [%2];" ::
          "r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}

// Shared-memory matrix descriptor: K-major, 128B swizzle, 8-row groups 1024 B apart.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)1 << 16;             // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;   // stride byte offset
  d |= (uint64_t)1 << 46;             // descriptor version for sm_100 family
  d |= (uint64_t)2 << 61;             // SWIZZLE_128B
  return d;
}

// Instruction descriptor: D FP32, A/B TF32, both K-major, M = 128, N = 256.
constexpr uint32_t IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void umma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          d_tmem),
      "l"(a), "l"(b), "r"(IDESC), "r"(accumulate));
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__global__ void __launch_bounds__(NTHREADS, 1)
tc_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, TcParams p) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* accf = empty + STAGES;  // chunk accumulated in buffer b (MMA -> epilogue)
  uint64_t* acce = accf + 2;        // buffer b drained (epilogue -> MMA)
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(acce + 2);
  int* fail = reinterpret_cast<int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const int nkb_seg = p.Kp / BK, nkb = nkb_seg * NSEG;
  const int nch = (nkb + CK - 1) / CK;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], NEPI);
    }
    *fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      int issued = 0;
      for (int kb = 0; kb < nkb; kb++) {
        const int s = kb % STAGES;
        if (kb >= STAGES && !mbar_wait(&empty[s], ((kb / STAGES) & 1) ^ 1)) { *fail = 1; break; }
        if (*(volatile int*)fail) break;
        mbar_expect_tx(&full[s], STAGE_BYTES);
        const int seg = kb / nkb_seg, kk = (kb % nkb_seg) * BK;
        tma_load_3d(smem + s * STAGE_BYTES, &tmA, &full[s], kk, m0, kSegA[seg]);
        tma_load_3d(smem + s * STAGE_BYTES + A_TILE, &tmB, &full[s], kk, n0, kSegB[seg]);
        issued = kb + 1;
      }
      // drain: every issued stage must have landed before the CTA may exit
      for (int kb = (issued > STAGES ? issued - STAGES : 0); kb < issued; kb++)
        mbar_wait(&full[kb % STAGES], (kb / STAGES) & 1);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      bool ok = true;
      for (int c = 0; c < nch && ok; c++) {
        const int b = c & 1;
        // buffer b is free once the epilogue drained chunk c - 2
        if (c >= 2 && !mbar_wait(&acce[b], ((c >> 1) - 1) & 1)) { *fail = 1; break; }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t dt = tmem + (uint32_t)(b * 256);
        const int kb_end = min(nkb, (c + 1) * CK);
        for (int kb = c * CK; kb < kb_end; kb++) {
          const int s = kb % STAGES;
          if (!mbar_wait(&full[s], (kb / STAGES) & 1)) { *fail = 1; ok = false; break; }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t a0 = smem_u32(smem + s * STAGE_BYTES), b0 = smem_u32(smem + s * STAGE_BYTES + A_TILE);
#pragma unroll
          for (int k = 0; k < BK / 8; k++)  // kind::tf32 consumes K = 8 (32 bytes) per instruction
            umma_tf32(dt, sdesc(a0 + 32 * k), sdesc(b0 + 32 * k), (kb != c * CK || k != 0) ? 1u : 0u);
          umma_commit(&empty[s]);
        }
        if (ok) umma_commit(&accf[b]);
      }
    }
  } else {
    // epilogue: warp w drains TMEM lanes 32*(w % 4) .. +31 (its sub-partition),
    // columns 128*h .. +127 of the buffer, h = (w - 2) / 4
    const int quarter = warp & 3, half = (warp - 2) >> 2;
    float acc[128];
#pragma unroll
    for (int i = 0; i < 128; i++) acc[i] = 0.f;
    bool ok = true;
#pragma unroll 1
    for (int c = 0; c < nch; c++) {
      const int b = c & 1;
      if (!mbar_wait(&accf[b], (c >> 1) & 1)) { *fail = 1; ok = false; break; }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t base = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(b * 256 + half * 128);
#pragma unroll
      for (int q = 0; q < 4; q++) {
        uint32_t r[32];
        tmem_ld32(base + (uint32_t)(q * 32), r);
#pragma unroll
        for (int i = 0; i < 32; i++) acc[q * 32 + i] += __uint_as_float(r[i]);
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(&acce[b]);
    }
    if (ok && !*(volatile int*)fail) {
      const int m = m0 + quarter * 32 + lane;
      const bool use_beta = (p.beta.x != 0.f || p.beta.y != 0.f);
      if (m < p.M) {
#pragma unroll
        for (int j = 0; j < 64; j++) {
          const int n = (n0 + half * 128) / 2 + j;
          if (n < p.N) {
            const float re = acc[2 * j], im = acc[2 * j + 1];
            float2 v = make_float2(p.alpha.x * re - p.alpha.y * im, p.alpha.x * im + p.alpha.y * re);
            float2* dst = p.C + m + p.ldc * (int64_t)n;
            if (use_beta) {
              const float2 o = *dst;
              v.x += p.beta.x * o.x - p.beta.y * o.y;
              v.y += p.beta.x * o.y + p.beta.y * o.x;
            }
            *dst = v;
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (threadIdx.x == 0 && *fail) atomicExch(p.status, 1);
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

__device__ __forceinline__ float tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// A planes (4 x Mp x Kp, row-major per plane): hi re, hi im, lo re, lo im of op(A).
__global__ void gather_a_kernel(const float2* __restrict__ src, int64_t lda, int opC, int M, int K, int Mp, int Kp,
                                float* __restrict__ planes) {
  __shared__ float2 tile[32][33];
  const int m0 = blockIdx.y * 32, k0 = blockIdx.x * 32;
  for (int r = threadIdx.y; r < 32; r += 8) {
    if (!opC) {  // op(A)(m, k) = src[m + lda k]; threads along m
      const int m = m0 + threadIdx.x, k = k0 + r;
      tile[threadIdx.x][r] = (m < M && k < K) ? src[m + lda * (int64_t)k] : make_float2(0.f, 0.f);
    } else {     // op(A)(m, k) = conj(src[k + lda m]); threads along k
      const int m = m0 + r, k = k0 + threadIdx.x;
      float2 v = (m < M && k < K) ? src[k + lda * (int64_t)m] : make_float2(0.f, 0.f);
      v.y = -v.y;
      tile[r][threadIdx.x] = v;
    }
  }
  __syncthreads();
  const size_t plane = (size_t)Mp * Kp;
  for (int r = threadIdx.y; r < 32; r += 8) {
    const int m = m0 + r, k = k0 + threadIdx.x;
    if (m >= Mp || k >= Kp) continue;
    const float2 v = tile[r][threadIdx.x];
    const float hr = tf32_rna(v.x), hi = tf32_rna(v.y);
    const size_t o = (size_t)m * Kp + k;
    planes[o] = hr;
    planes[o + plane] = hi;
    planes[o + 2 * plane] = tf32_rna(v.x - hr);
    planes[o + 3 * plane] = tf32_rna(v.y - hi);
  }
}

// B planes (4 x N2p x Kp): rows 2n, 2n+1 of plane 0 = hi re, hi im; plane 1 =
// lo re, lo im; plane 2 = -hi im, hi re; plane 3 = -lo im, lo re of op(B)(k, n).
__global__ void gather_b_kernel(const float2* __restrict__ src, int64_t ldb, int opC, int K, int N, int N2p, int Kp,
                                float* __restrict__ planes) {
  __shared__ float2 tile[32][33];  // [n][k]
  const int n0 = blockIdx.y * 32, k0 = blockIdx.x * 32;
  for (int r = threadIdx.y; r < 32; r += 8) {
    if (!opC) {  // op(B)(k, n) = src[k + ldb n]; threads along k
      const int n = n0 + r, k = k0 + threadIdx.x;
      tile[r][threadIdx.x] = (n < N && k < K) ? src[k + ldb * (int64_t)n] : make_float2(0.f, 0.f);
    } else {     // op(B)(k, n) = conj(src[n + ldb k]); threads along n
      const int n = n0 + threadIdx.x, k = k0 + r;
      float2 v = (n < N && k < K) ? src[n + ldb * (int64_t)k] : make_float2(0.f, 0.f);
      v.y = -v.y;
      tile[threadIdx.x][r] = v;
    }
  }
  __syncthreads();
  const size_t plane = (size_t)N2p * Kp;
  for (int r = threadIdx.y; r < 32; r += 8) {
    const int n = n0 + r, k = k0 + threadIdx.x;
    if (2 * n >= N2p || k >= Kp) continue;
    const float2 v = tile[r][threadIdx.x];
    const float hr = tf32_rna(v.x), hi = tf32_rna(v.y);
    const float lr = tf32_rna(v.x - hr), li = tf32_rna(v.y - hi);
    const size_t o0 = (size_t)(2 * n) * Kp + k, o1 = o0 + Kp;
    planes[o0] = hr;               planes[o1] = hi;
    planes[o0 + plane] = lr;       planes[o1 + plane] = li;
    planes[o0 + 2 * plane] = -hi;  planes[o1 + 2 * plane] = hr;
    planes[o0 + 3 * plane] = -li;  planes[o1 + 3 * plane] = lr;
  }
}

// The same planes from a permuted view of an N-d tensor: op(A)(m, k) =
// src[rowoff[m] + coloff[k]] (rowoff over A's free legs, coloff over its
// contracted legs, both in element strides of the source).  This is the ncon
// permute folded into the operand gather: no permuted copy of A is written.
// rows_fast: the source's unit-stride leg is a row leg (threads load along
// m), otherwise a column leg (threads load along k).
__global__ void gather_a_map_kernel(const float2* __restrict__ src, const int64_t* __restrict__ rowoff,
                                    const int64_t* __restrict__ coloff, int rows_fast, int M, int K, int Mp, int Kp,
                                    float* __restrict__ planes) {
  __shared__ float2 tile[32][33];
  const int m0 = blockIdx.y * 32, k0 = blockIdx.x * 32;
  for (int r = threadIdx.y; r < 32; r += 8) {
    if (rows_fast) {
      const int m = m0 + threadIdx.x, k = k0 + r;
      tile[threadIdx.x][r] = (m < M && k < K) ? src[rowoff[m] + coloff[k]] : make_float2(0.f, 0.f);
    } else {
      const int m = m0 + r, k = k0 + threadIdx.x;
      tile[r][threadIdx.x] = (m < M && k < K) ? src[rowoff[m] + coloff[k]] : make_float2(0.f, 0.f);
    }
  }
  __syncthreads();
  const size_t plane = (size_t)Mp * Kp;
  for (int r = threadIdx.y; r < 32; r += 8) {
    const int m = m0 + r, k = k0 + threadIdx.x;
    if (m >= Mp || k >= Kp) continue;
    const float2 v = tile[r][threadIdx.x];
    const float hr = tf32_rna(v.x), hi = tf32_rna(v.y);
    const size_t o = (size_t)m * Kp + k;
    planes[o] = hr;
    planes[o + plane] = hi;
    planes[o + 2 * plane] = tf32_rna(v.x - hr);
    planes[o + 3 * plane] = tf32_rna(v.y - hi);
  }
}

// B planes from op(B)(k, n) = src[rowoff[k] + coloff[n]] (rowoff over B's
// contracted legs, coloff over its free legs); rows_fast: unit stride in k.
__global__ void gather_b_map_kernel(const float2* __restrict__ src, const int64_t* __restrict__ rowoff,
                                    const int64_t* __restrict__ coloff, int rows_fast, int K, int N, int N2p, int Kp,
                                    float* __restrict__ planes) {
  __shared__ float2 tile[32][33];  // [n][k]
  const int n0 = blockIdx.y * 32, k0 = blockIdx.x * 32;
  for (int r = threadIdx.y; r < 32; r += 8) {
    if (rows_fast) {
      const int n = n0 + r, k = k0 + threadIdx.x;
      tile[r][threadIdx.x] = (n < N && k < K) ? src[rowoff[k] + coloff[n]] : make_float2(0.f, 0.f);
    } else {
      const int n = n0 + threadIdx.x, k = k0 + r;
      tile[threadIdx.x][r] = (n < N && k < K) ? src[rowoff[k] + coloff[n]] : make_float2(0.f, 0.f);
    }
  }
  __syncthreads();
  const size_t plane = (size_t)N2p * Kp;
  for (int r = threadIdx.y; r < 32; r += 8) {
    const int n = n0 + r, k = k0 + threadIdx.x;
    if (2 * n >= N2p || k >= Kp) continue;
    const float2 v = tile[r][threadIdx.x];
    const float hr = tf32_rna(v.x), hi = tf32_rna(v.y);
    const float lr = tf32_rna(v.x - hr), li = tf32_rna(v.y - hi);
    const size_t o0 = (size_t)(2 * n) * Kp + k, o1 = o0 + Kp;
    planes[o0] = hr;               planes[o1] = hi;
    planes[o0 + plane] = lr;       planes[o1 + plane] = li;
    planes[o0 + 2 * plane] = -hi;  planes[o1 + 2 * plane] = hr;
    planes[o0 + 3 * plane] = -li;  planes[o1 + 3 * plane] = lr;
  }
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_encode_once;

bool encode_fn() {
  std::call_once(g_encode_once, [] {
    cudaDriverEntryPointQueryResult q;
    void* fn = nullptr;
    if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &fn, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  });
  return g_encode != nullptr;
}

bool make_map(CUtensorMap* map, float* base, int K, int rows, int box_rows) {
  cuuint64_t dims[3] = {(cuuint64_t)K, (cuuint64_t)rows, 4};
  cuuint64_t strides[2] = {(cuuint64_t)K * 4, (cuuint64_t)K * rows * 4};
  cuuint32_t box[3] = {BK, (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  return g_encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

inline int64_t round_up(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

}  // namespace

int qt_cgemm_c64(qt_handle* h, int opA, int opB, int64_t M, int64_t N, int64_t K, float2 alpha, const float2* A,
                 int64_t lda, const float2* B, int64_t ldb, float2 beta, float2* C, int64_t ldc) {
  if (h->cfg.tc_gemm && opA != QT_OP_T && opB != QT_OP_T && M >= 64 && N >= 32 && K >= 32)
    return qt_cgemm_tc(h, opA, opB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
  return qt_cgemm<float2>(h, opA, opB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
}

namespace {

// The tensor-core GEMM on planes already gathered (pa: 4 x Mp x Kp, pb: 4 x
// N2p x Kp); C (M x N) = alpha A B + beta C.
int tc_gemm_planes(qt_handle* h, float* pa, float* pb, int64_t M, int64_t N, int64_t K, int64_t Mp, int64_t N2p,
                   int64_t Kp, float2 alpha, float2 beta, float2* C, int64_t ldc, int* status) {
  CUtensorMap ma, mb;
  if (!make_map(&ma, pa, (int)Kp, (int)Mp, BM) || !make_map(&mb, pb, (int)Kp, (int)N2p, BN))
    return qt_fail(h, QT_ECUDA, "tc gemm: tensor map encoding failed");
  static bool attr_set = false;
  if (!attr_set) {
    QT_CHECK_CUDA(h, cudaFuncSetAttribute(tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
    attr_set = true;
  }
  TcParams p;
  p.M = (int)M; p.N = (int)N; p.Kp = (int)Kp; p.Mp = (int)Mp; p.N2p = (int)N2p;
  p.alpha = alpha; p.beta = beta; p.C = C; p.ldc = ldc; p.status = status;
  dim3 grid((unsigned)(Mp / BM), (unsigned)(N2p / BN));
  QT_LAUNCH(h, tc_gemm_kernel, grid, NTHREADS, SMEM_BYTES, ma, mb, p);
  h->work_tc_flops += 24.0 * (double)M * (double)N * (double)K;
  h->work_tc_launches += 1;
  if (status != h->d_status) {  // a handle without a status word: check here
    int hs = 0;
    QT_CHECK_CUDA(h, cudaMemcpyAsync(&hs, status, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
    if (hs) return qt_fail(h, QT_ETIMEOUT, "tc gemm: a pipeline wait timed out");
  }
  return QT_OK;
}

}  // namespace

// C (M x N) = alpha op(A) op(B) + beta C on the tensor cores; op in {N, C}.
int qt_cgemm_tc(qt_handle* h, int opA, int opB, int64_t M, int64_t N, int64_t K, float2 alpha, const float2* A,
                int64_t lda, const float2* B, int64_t ldb, float2 beta, float2* C, int64_t ldc) {
  if (M <= 0 || N <= 0) return QT_OK;
  if (opA == QT_OP_T || opB == QT_OP_T) return qt_fail(h, QT_ENOTSUP, "tc gemm: plain transpose not supported");
  if (!encode_fn()) return qt_fail(h, QT_ENOTSUP, "tc gemm: cuTensorMapEncodeTiled unavailable");
  const int64_t Mp = round_up(M, BM), N2p = round_up(2 * N, BN), Kp = round_up(std::max<int64_t>(K, 1), BK);
  qt_scratch s(h);
  float *pa, *pb;
  int* status = h->d_status;  // sticky: checked by qt_check_status where the caller synchronises
  QT_TRY(s.get(&pa, (size_t)4 * Mp * Kp));
  QT_TRY(s.get(&pb, (size_t)4 * N2p * Kp));
  if (!status) {
    QT_TRY(s.get(&status, 1));
    QT_CHECK_CUDA(h, cudaMemsetAsync(status, 0, sizeof(int), h->stream));
  }
  {
    dim3 grid((unsigned)(Kp / 32), (unsigned)(Mp / 32));
    QT_LAUNCH(h, gather_a_kernel, grid, dim3(32, 8), 0, A, lda, opA == QT_OP_C ? 1 : 0, (int)M, (int)K, (int)Mp,
              (int)Kp, pa);
  }
  {
    dim3 grid((unsigned)(Kp / 32), (unsigned)(N2p / 2 / 32 + ((N2p / 2) % 32 ? 1 : 0)));
    QT_LAUNCH(h, gather_b_kernel, grid, dim3(32, 8), 0, B, ldb, opB == QT_OP_C ? 1 : 0, (int)K, (int)N, (int)N2p,
              (int)Kp, pb);
  }
  return tc_gemm_planes(h, pa, pb, M, N, K, Mp, N2p, Kp, alpha, beta, C, ldc, status);
}

// C (M x N, ld M) = A_view B_view on the tensor cores, the operands read
// through offset tables (device arrays): A_view(m, k) = A[a_row[m] +
// a_col[k]], B_view(k, n) = B[b_row[k] + b_col[n]] -- the pairwise ncon
// contraction with its permutes folded into the operand gathers.
int qt_cgemm_tc_mapped(qt_handle* h, int64_t M, int64_t N, int64_t K, const float2* A, const int64_t* a_row,
                       const int64_t* a_col, int a_rows_fast, const float2* B, const int64_t* b_row,
                       const int64_t* b_col, int b_rows_fast, float2* C) {
  if (M <= 0 || N <= 0) return QT_OK;
  if (!encode_fn()) return qt_fail(h, QT_ENOTSUP, "tc gemm: cuTensorMapEncodeTiled unavailable");
  const int64_t Mp = round_up(M, BM), N2p = round_up(2 * N, BN), Kp = round_up(std::max<int64_t>(K, 1), BK);
  qt_scratch s(h);
  float *pa, *pb;
  int* status = h->d_status;
  QT_TRY(s.get(&pa, (size_t)4 * Mp * Kp));
  QT_TRY(s.get(&pb, (size_t)4 * N2p * Kp));
  if (!status) {
    QT_TRY(s.get(&status, 1));
    QT_CHECK_CUDA(h, cudaMemsetAsync(status, 0, sizeof(int), h->stream));
  }
  {
    dim3 grid((unsigned)(Kp / 32), (unsigned)(Mp / 32));
    QT_LAUNCH(h, gather_a_map_kernel, grid, dim3(32, 8), 0, A, a_row, a_col, a_rows_fast, (int)M, (int)K, (int)Mp,
              (int)Kp, pa);
  }
  {
    dim3 grid((unsigned)(Kp / 32), (unsigned)(N2p / 2 / 32 + ((N2p / 2) % 32 ? 1 : 0)));
    QT_LAUNCH(h, gather_b_map_kernel, grid, dim3(32, 8), 0, B, b_row, b_col, b_rows_fast, (int)K, (int)N,
              (int)N2p, (int)Kp, pb);
  }
  return tc_gemm_planes(h, pa, pb, M, N, K, Mp, N2p, Kp, make_float2(1.f, 0.f), make_float2(0.f, 0.f), C, M,
                        status);
}
