// Dense factors on the tensor cores (kernel class 6, float32 data).
//
// A square dense operator D (n x n, n <= 64; a dense Kron factor, fastmat's
// Matrix, applied mode-wise by fastmat/Kron.pyx:284-300) applied to the B
// vectors of a tile is a matrix product: with one row per vector,
// Y (B x n) = X (B x n) D^T.  n is padded with zeros to Kp, a multiple of
// 16.  Per CTA the factor is staged once in shared memory as three BF16
// terms d = d1 + d2 + d3 (8 + 8 + 8 significand bits: exact for float32),
// each in the canonical K-major no-swizzle layout (rows = output index,
// K = input index; 8-row x 16-byte core matrices).  Per round every thread
// stages its vector's row the same way (three terms), one thread issues
// `tcgen05.mma.kind::f16` for the six products x_a d_b with a + b <= 4
// (the rest lie below 2^-24 relative) over the K chunks of 16, accumulating
// in FP32 in tensor memory, `tcgen05.commit` signals an mbarrier (bounded
// wait), and `tcgen05.ld` brings each row back to the thread that staged
// it.  The MMA shape is M = 128 rows (vectors), N = Kp, K = 16, the same
// BF16 instruction kind and descriptor format as the Hadamard groups
// (fm_tc.cuh).
#pragma once

#include <cuda_bf16.h>

namespace fmk {

constexpr int kTdMaxN = 64;                       // largest factor order
constexpr int kTdStageBytes = 96 * 1024;          // row staging, all rounds
constexpr int kTdMatBytes = 3 * kTdMaxN * kTdMaxN * 2;
constexpr int kTdBytes = kTdMatBytes + kTdStageBytes + 64;
constexpr int kTdCols = 128;  // TMEM columns: chunks x Kp <= 128

struct TdState {
  unsigned char *mat;    // [3][Kp x Kp] BF16, K-major core layout
  unsigned char *stage;  // [3][chunk][128 x Kp] BF16
  unsigned long long *bar;
  unsigned *slot;
  unsigned tmem;
  unsigned phase;
  int *err;
  int n, Kp, chunks;  // order, padded order, 128-row chunks per round
  bool failed;
};

// byte offset of (row i, column k) in a K-major no-swizzle operand whose
// rows hold Kp BF16: core (i / 8, k / 8) at (i / 8) Kp 16 + (k / 8) 128,
// row i % 8 at 16 (i % 8)
__device__ __forceinline__ int td_off(int i, int k, int Kp) {
  return (i >> 3) * (Kp * 16) + (k >> 3) * 128 + (i & 7) * 16 + (k & 7) * 2;
}

// shared-memory matrix descriptor: leading (K) byte offset 128, stride
// (row-group) byte offset Kp * 16, version 1, no swizzle
__device__ __forceinline__ unsigned long long td_desc(const void *p, int Kp) {
  const unsigned long long a = (tc_smem(p) & 0x3FFFFu) >> 4;
  return a | ((unsigned long long)(128 >> 4) << 16) |
         ((unsigned long long)((Kp * 16) >> 4) << 32) | (1ull << 46);
}

// instruction descriptor, kind::f16: D F32, A and B BF16, both K-major,
// N = Kp, M = 128
__device__ __forceinline__ unsigned td_idesc(int Kp) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (((unsigned)Kp >> 3) << 17) |
         ((128u >> 4) << 24);
}

__device__ __forceinline__ void td_mma(unsigned d, unsigned long long a,
                                       unsigned long long b, unsigned idesc,
                                       int accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

// float -> three BF16 terms whose sum is exact
__device__ __forceinline__ void td_split(float x, unsigned short &a,
                                         unsigned short &b,
                                         unsigned short &c) {
  const __nv_bfloat16 h = __float2bfloat16_rn(x);
  const float r1 = x - __bfloat162float(h);
  const __nv_bfloat16 m = __float2bfloat16_rn(r1);
  const __nv_bfloat16 l = __float2bfloat16_rn(r1 - __bfloat162float(m));
  a = bf16_bits(h);
  b = bf16_bits(m);
  c = bf16_bits(l);
}

// TMEM allocation (warp 0), the factor's three terms, the mbarrier.
// dmat: the factor, column-major n x n floats (element (i, j) at i + j n).
__device__ __forceinline__ void td_init(TdState &td, unsigned char *base,
                                        const float *dmat, int n, int T,
                                        int *err, int tid) {
  td.n = n;
  td.Kp = (n + 15) & ~15;
  int ch = kTdStageBytes / (3 * 128 * td.Kp * 2);
  if (ch > 4) ch = 4;
  if (ch > T / 128) ch = T / 128;
  if (ch * td.Kp > kTdCols) ch = kTdCols / td.Kp;
  td.chunks = ch < 1 ? 1 : ch;
  td.mat = base;
  td.stage = base + kTdMatBytes;
  td.bar = reinterpret_cast<unsigned long long *>(base + kTdMatBytes +
                                                  kTdStageBytes);
  td.slot = reinterpret_cast<unsigned *>(base + kTdMatBytes + kTdStageBytes +
                                         8);
  td.phase = 0;
  td.err = err;
  td.failed = false;
  if (tid < 32) {
    asm volatile(
        "tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
        ::"r"(tc_smem(td.slot)), "r"(kTdCols)
        : "memory");
    asm volatile(
        "tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::
            : "memory");
  }
  const int Kp = td.Kp;
  const int msz = Kp * Kp * 2;
  for (int e = tid; e < Kp * Kp; e += blockDim.x) {
    const int i = e / Kp, k = e % Kp;  // output i, input k
    const float v = (i < n && k < n) ? dmat[i + k * n] : 0.f;
    unsigned short a, b, c;
    td_split(v, a, b, c);
    const int o = td_off(i, k, Kp);
    *reinterpret_cast<unsigned short *>(td.mat + o) = a;
    *reinterpret_cast<unsigned short *>(td.mat + msz + o) = b;
    *reinterpret_cast<unsigned short *>(td.mat + 2 * msz + o) = c;
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(
                     tc_smem(td.bar))
                 : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  td.tmem = *td.slot;
}

__device__ __forceinline__ void td_release(TdState &td, int tid) {
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (tid < 32)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::
                     "r"(td.tmem),
                 "r"(kTdCols)
                 : "memory");
}

// Y = X D^T on the B vectors of a float tile (layout LAY, n points each).
// Requires blockDim.x to be a multiple of 128.
template <int LAY>
__device__ void run_densetc(float *sm, int Lp, int B, TdState &td, int tid,
                            int T) {
  const int n = td.n, Kp = td.Kp, CH = td.chunks;
  const int per = CH * 128;  // rows per round
  const int chunk = tid >> 7, i = tid & 127;
  const int warp = tid >> 5;
  const int ssz = 128 * Kp * 2;  // one term of one chunk
  const int msz = Kp * Kp * 2;
  const unsigned idesc = td_idesc(Kp);
  for (int r0 = 0; r0 < B; r0 += per) {
    const int b = r0 + tid;
    const bool stager = tid < per;
    const bool live = stager && b < B;
    float *vec = live ? vbase<float, LAY>(sm, b, Lp) : nullptr;
    if (stager) {
      unsigned char *a0 = td.stage + (0 * CH + chunk) * ssz;
      unsigned char *a1 = td.stage + (1 * CH + chunk) * ssz;
      unsigned char *a2 = td.stage + (2 * CH + chunk) * ssz;
      for (int k0 = 0; k0 < Kp; k0 += 8) {
        unsigned short t0[8], t1[8], t2[8];
#pragma unroll
        for (int d = 0; d < 8; ++d) {
          const int k = k0 + d;
          const float x = (live && k < n) ? vec[jx<float, LAY>(k, B)] : 0.f;
          td_split(x, t0[d], t1[d], t2[d]);
        }
        const int o = td_off(i, k0, Kp);
        uint4 w;
        w.x = t0[0] | ((unsigned)t0[1] << 16);
        w.y = t0[2] | ((unsigned)t0[3] << 16);
        w.z = t0[4] | ((unsigned)t0[5] << 16);
        w.w = t0[6] | ((unsigned)t0[7] << 16);
        *reinterpret_cast<uint4 *>(a0 + o) = w;
        w.x = t1[0] | ((unsigned)t1[1] << 16);
        w.y = t1[2] | ((unsigned)t1[3] << 16);
        w.z = t1[4] | ((unsigned)t1[5] << 16);
        w.w = t1[6] | ((unsigned)t1[7] << 16);
        *reinterpret_cast<uint4 *>(a1 + o) = w;
        w.x = t2[0] | ((unsigned)t2[1] << 16);
        w.y = t2[2] | ((unsigned)t2[3] << 16);
        w.z = t2[4] | ((unsigned)t2[5] << 16);
        w.w = t2[6] | ((unsigned)t2[7] << 16);
        *reinterpret_cast<uint4 *>(a2 + o) = w;
      }
    }
    // generic-proxy writes -> visible to the tensor core (async proxy)
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (!td.failed) {
      if (tid == 0) {
        // x_a d_b for a + b <= 4 (terms numbered 1..3)
        const int pa[6] = {0, 0, 1, 0, 1, 2};
        const int pb[6] = {0, 1, 0, 2, 1, 0};
        for (int q = 0; q < CH; ++q) {
          int acc = 0;
          for (int kc = 0; kc < Kp; kc += 16) {
            for (int t = 0; t < 6; ++t) {
              const unsigned char *a =
                  td.stage + (pa[t] * CH + q) * ssz + kc * 16;
              const unsigned char *bm = td.mat + pb[t] * msz + kc * 16;
              td_mma(td.tmem + q * Kp, td_desc(a, Kp), td_desc(bm, Kp),
                     idesc, acc);
              acc = 1;
            }
          }
        }
        tc_commit(td.bar);
      }
      const bool ok = tc_wait(td.bar, td.phase);
      td.phase ^= 1u;
      // block-wide vote keeps td.failed uniform across the CTA
      if (__syncthreads_or(!ok)) {
        td.failed = true;
        if (tid == 0 && td.err) atomicExch(td.err, FM_ERR_TIMEOUT);
      }
    }
    tc_fence_after();
    // warp w reads TMEM lanes 32 (w % 4) .. + 31 of chunk w / 4
    if (stager) {
      for (int c0 = 0; c0 < Kp; c0 += 16) {
        float y[16];
        tc_ld16(td.tmem + ((unsigned)(32 * (warp & 3)) << 16) + chunk * Kp +
                    c0,
                y);
        if (live) {
#pragma unroll
          for (int d = 0; d < 16; ++d)
            if (c0 + d < n) vec[jx<float, LAY>(c0 + d, B)] = y[d];
        }
      }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
  }
}

}  // namespace fmk
