// Tensor-core Walsh-Hadamard sub-blocks (5th-generation tensor cores).
//
// One FWHT bit group of width 4 (a 16-point Hadamard H16 along the element
// index bits [s, s + 4) of every vector in a shared-memory tile) is a dense
// 16 x 16 contraction: with rows m enumerating every (vector, other bits)
// combination, Y[m, :] = X[m, :] H16.  Each 128-row chunk of X is staged in
// shared memory as BF16 in the canonical K-major layout (8-row x 16-byte
// core matrices, no swizzle), split exactly into three BF16 terms
// x = hi + mid + lo (8 + 8 + 8 significand bits cover float32's 24), and
// `tcgen05.mma.kind::f16` multiplies every term by H16 (entries +-1, exact
// in BF16) accumulating in FP32 in tensor memory (TMEM).  `tcgen05.ld` brings
// each row back to the thread that staged it, which writes it into the
// tile.  Up to four chunks (512 rows, one per thread of a 512-thread CTA)
// are in flight per round, each in its own 16 TMEM columns.
//
// The MMA issue is a single thread; completion is signalled through an
// mbarrier by `tcgen05.commit` and waited for with a bounded poll.
#pragma once

#include <cuda_bf16.h>

namespace fmk {

// shared memory the tensor-core state needs beyond the tile ring
constexpr int kTcStageBytes = 4096;  // one 128 x 16 BF16 operand
constexpr int kTcSplits = 3;
constexpr int kTcChunks = 4;
constexpr int kTcBytes = kTcSplits * kTcChunks * kTcStageBytes + 512 + 64;
constexpr int kTcCols = 64;  // TMEM columns: 16 per chunk

struct TcState {
  unsigned char *stage;  // [split][chunk][4096 B]
  unsigned char *hmat;   // H16 as a 16 x 16 K-major BF16 operand
  unsigned long long *bar;
  unsigned *slot;        // TMEM base address written by tcgen05.alloc
  unsigned tmem;
  unsigned phase;
  int *err;
  bool failed;
};

__device__ __forceinline__ unsigned tc_smem(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

// byte offset of element (row i, column k) of a K-major no-swizzle operand
// with 8 x 16-byte core matrices: core (i / 8, k / 8) at 256 (i / 8) +
// 128 (k / 8), row i % 8 at 16 (i % 8)
__device__ __forceinline__ int tc_core_off(int i, int k) {
  return (i >> 3) * 256 + (k >> 3) * 128 + (i & 7) * 16 + (k & 7) * 2;
}

// shared-memory matrix descriptor: start address, leading-dimension byte
// offset (K direction, 128 B), stride byte offset (M/N direction, 256 B),
// descriptor version 1, no swizzle
__device__ __forceinline__ unsigned long long tc_desc(const void *p) {
  const unsigned long long a = (tc_smem(p) & 0x3FFFFu) >> 4;
  return a | ((unsigned long long)(128 >> 4) << 16) |
         ((unsigned long long)(256 >> 4) << 32) | (1ull << 46);
}

// instruction descriptor, kind::f16: D F32, A and B BF16, both K-major,
// N = 16, M = 128
constexpr unsigned kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) |
                              ((16u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// allocation by warp 0 (all 32 lanes), then H16 and the mbarrier
__device__ __forceinline__ void tc_init(TcState &tc, unsigned char *base,
                                        int *err, int tid) {
  tc.stage = base;
  tc.hmat = base + kTcSplits * kTcChunks * kTcStageBytes;
  tc.bar = reinterpret_cast<unsigned long long *>(tc.hmat + 512);
  tc.slot = reinterpret_cast<unsigned *>(tc.hmat + 512 + 8);
  tc.phase = 0;
  tc.err = err;
  tc.failed = false;
  if (tid < 32) {
    asm volatile(
        "tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
        ::"r"(tc_smem(tc.slot)), "r"(kTcCols)
        : "memory");
    asm volatile(
        "tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::
            : "memory");
  }
  // H16[n][k] = (-1)^popcount(n & k), BF16 +-1 (0x3F80 / 0xBF80)
  for (int e = tid; e < 256; e += blockDim.x) {
    const int n = e >> 4, k = e & 15;
    const unsigned short v = (__popc(n & k) & 1) ? 0xBF80u : 0x3F80u;
    *reinterpret_cast<unsigned short *>(tc.hmat + tc_core_off(n, k)) = v;
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(
                     tc_smem(tc.bar))
                 : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  tc.tmem = *tc.slot;
}

__device__ __forceinline__ void tc_release(TcState &tc, int tid) {
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (tid < 32)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::
                     "r"(tc.tmem),
                 "r"(kTcCols)
                 : "memory");
}

__device__ __forceinline__ void tc_mma(unsigned d, unsigned long long a,
                                       unsigned long long b, int accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(kTcIdesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void tc_commit(unsigned long long *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 "
      "[%0];" ::"r"(tc_smem(bar))
      : "memory");
}

__device__ __forceinline__ bool tc_wait(unsigned long long *bar,
                                        unsigned parity) {
  const unsigned a = tc_smem(bar);
  for (long long it = 0; it < (1LL << 22); ++it) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, "
        "[%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tc_ld16(unsigned taddr, float *v) {
  unsigned r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, "
      "%7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]),
        "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
        "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
        "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ unsigned short bf16_bits(__nv_bfloat16 h) {
  return *reinterpret_cast<unsigned short *>(&h);
}

// H16 along bits [s, s + 4) of every vector of a float tile (layout LAY,
// Lf elements per vector, B vectors).  Requires blockDim.x to be a
// multiple of 128 and at most 512.
template <int LAY>
__device__ void run_h16tc(float *sm, int Lp, int B, int Lf, int s,
                          TcState &tc, int tid, int T) {
  const int S = 1 << s;
  const int lgR = __ffs(Lf >> 4) - 1;  // rows per vector = Lf / 16
  const int lgB = __ffs(B) - 1;
  const int rows = B << lgR;
  const int chunk = tid >> 7, i = tid & 127;
  const int nchunks = T >> 7;
  const int warp = tid >> 5;
  for (int r0 = 0; r0 < rows; r0 += T) {
    const int m = r0 + tid;
    float *vec = nullptr;
    int j0 = 0;
    const bool live = m < rows;
    if (live) {
      int b, r;
      if constexpr (LAY == 1) {
        b = m & (B - 1);
        r = m >> lgB;
      } else {
        b = m >> lgR;
        r = m & ((1 << lgR) - 1);
      }
      const int lo = r & (S - 1), hi = r >> s;
      j0 = (hi << (s + 4)) | lo;
      vec = vbase<float, LAY>(sm, b, Lp);
    }
    // stage the three BF16 terms of this row
    unsigned short t[kTcSplits][16];
#pragma unroll
    for (int d = 0; d < 16; ++d) {
      const float x = live ? vec[jx<float, LAY>(j0 + d * S, B)] : 0.f;
      const __nv_bfloat16 h = __float2bfloat16_rn(x);
      const float r1 = x - __bfloat162float(h);
      const __nv_bfloat16 mh = __float2bfloat16_rn(r1);
      const __nv_bfloat16 lh = __float2bfloat16_rn(r1 - __bfloat162float(mh));
      t[0][d] = bf16_bits(h);
      t[1][d] = bf16_bits(mh);
      t[2][d] = bf16_bits(lh);
    }
#pragma unroll
    for (int sp = 0; sp < kTcSplits; ++sp) {
      unsigned char *a = tc.stage + (sp * kTcChunks + chunk) * kTcStageBytes;
#pragma unroll
      for (int h8 = 0; h8 < 2; ++h8) {
        uint4 w;
        w.x = t[sp][8 * h8 + 0] | ((unsigned)t[sp][8 * h8 + 1] << 16);
        w.y = t[sp][8 * h8 + 2] | ((unsigned)t[sp][8 * h8 + 3] << 16);
        w.z = t[sp][8 * h8 + 4] | ((unsigned)t[sp][8 * h8 + 5] << 16);
        w.w = t[sp][8 * h8 + 6] | ((unsigned)t[sp][8 * h8 + 7] << 16);
        *reinterpret_cast<uint4 *>(a + tc_core_off(i, 8 * h8)) = w;
      }
    }
    // generic-proxy writes -> visible to the tensor core (async proxy)
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (!tc.failed) {
      if (tid == 0) {
        const unsigned long long bd = tc_desc(tc.hmat);
        for (int q = 0; q < nchunks; ++q)
          for (int sp = 0; sp < kTcSplits; ++sp)
            tc_mma(tc.tmem + 16 * q,
                   tc_desc(tc.stage + (sp * kTcChunks + q) * kTcStageBytes),
                   bd, sp > 0);
        tc_commit(tc.bar);
      }
      const bool ok = tc_wait(tc.bar, tc.phase);
      tc.phase ^= 1u;
      // block-wide vote keeps tc.failed uniform across the CTA
      if (__syncthreads_or(!ok)) {
        tc.failed = true;
        if (tid == 0 && tc.err) atomicExch(tc.err, FM_ERR_TIMEOUT);
      }
    }
    tc_fence_after();
    // warp w reads TMEM lanes 32 (w % 4) .. + 31, columns of chunk w / 4
    float y[16];
    tc_ld16(tc.tmem + ((unsigned)(32 * (warp & 3)) << 16) + 16 * chunk, y);
    if (live) {
#pragma unroll
      for (int n = 0; n < 16; ++n) vec[jx<float, LAY>(j0 + n * S, B)] = y[n];
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
  }
}

}  // namespace fmk
