// Two adjacent Kron modes in one launch, block by block: a circulant mode
// on contiguous vectors (the register convolution, fm_rconv.cuh) followed
// by a Hadamard mode on vectors at a stride that is a multiple of the
// convolution's length (the strided register FWHT, fm_rfwht.cuh), applied
// in place (fastmat/Kron.pyx:284-300 applies the factors mode by mode).
// The FWHT's vectors live in blocks of L2 S rows that the convolution's
// vectors tile exactly, so the second mode of a block needs only that
// block's first mode: a cooperative persistent launch hands out work items
// in order with an atomic counter -- the convolution items of block k (32
// vectors each), then the FWHT items of block k - lag (NV adjacent real
// vectors each; lag about twice the resident CTAs over a block's items, so
// the awaited items have mostly finished and a few MB of blocks are in
// flight) -- and an FWHT item waits (bounded, acquire) until its
// block's convolution items have all raised its counter (release after
// their stores).  A block is 256 KiB (complex64) to 512 KiB, so it is still
// in L2 when its second mode reads it: two modes for one HBM round trip.
// Every awaited item was handed out earlier to a resident CTA and never
// waits itself, so the waits end.
#pragma once

#include "fm_rconv.cuh"
#include "fm_rfwht.cuh"

namespace fmk {

struct RchPair {
  RcStep c;        // convolution mode, x -> y (plain: no pre/post products)
  RfStep h;        // FWHT mode, y -> y in place (real view)
  unsigned *ctr;   // [0] items handed out, [1 + k] convolution items done
  int *err;
  long long wait_limit;
  i64 blocks;      // blocks over all columns
  int n1, n2;      // convolution / FWHT items per block
  int lag;         // blocks between a block's first and second mode
};

#define FM_RCH_THREADS 256
// real element type of a complex compute type
template <class E> struct RealOf {
  typedef typename std::conditional<Emu<E>::v, df, float>::type type;
};

template <class E, int L1, int L2> struct RchShape {
  typedef typename RealOf<E>::type R;
  static constexpr int P = RcLane<E>::P;
  static constexpr int G = L1 / P;
  static constexpr int VPW = 32 / G;
  static constexpr int VPC = (FM_RCH_THREADS / 32) * VPW;  // per item
  static constexpr int S1 = rc_stages(L1, P);
  static constexpr int TWN = rc_twlen<E, L1, S1>();
  static constexpr int W2 = L2 / RfLane<R>::P;
  static constexpr int NV2 = FM_RCH_THREADS / W2;  // real vectors per item
  static constexpr size_t cbuf =
      (size_t)(FM_RCH_THREADS / 32) * VPW * RcBuf<E, L1>::Lp * sizeof(E);
  static constexpr size_t hbuf =
      (size_t)NV2 * RsShape<R, L2>::Lx * sizeof(R) + 4 * NV2;
  static constexpr size_t region = ((cbuf > hbuf ? cbuf : hbuf) + 15) / 16 *
                                   16;
  static constexpr size_t bytes =
      16 + ((size_t)(TWN + L1) * sizeof(E) + 15) / 16 * 16 + region;
};
template <class E> struct RchOcc {
  static constexpr int v = Emu<E>::v ? 2 : 3;
};

template <class E, int L1, int L2>
__global__ void __launch_bounds__(FM_RCH_THREADS, (RchOcc<E>::v))
    rkch_kernel(const __grid_constant__ RchPair p) {
  typedef RchShape<E, L1, L2> Sh;
  typedef typename Sh::R R;
  constexpr int P = Sh::P, G = Sh::G, VPW = Sh::VPW, VPC = Sh::VPC;
  constexpr int S1 = Sh::S1;
  constexpr int NV2 = Sh::NV2;
  static_assert(G >= 1 && G <= 32 && NV2 >= 1, "layout");
  typedef typename std::conditional<Emu<E>::v, double2, E>::type Raw;
  extern __shared__ __align__(128) unsigned char fm_smem[];
  unsigned *sitem = reinterpret_cast<unsigned *>(fm_smem);
  E *stw = reinterpret_cast<E *>(fm_smem + 16);
  E *sspec = stw + Sh::TWN;
  unsigned char *region =
      fm_smem + 16 + ((size_t)(Sh::TWN + L1) * sizeof(E) + 15) / 16 * 16;
  const int tid = threadIdx.x;
  rc_fill_tw<E, L1, 0>(stw, (const E *)p.c.tw);
  // the spectrum in lane-major order (as the register convolution keeps it)
  for (int i = tid; i < L1; i += FM_RCH_THREADS) {
    const int j = i / G, gg = i % G;
    sspec[i] = ((const E *)p.c.spec)[rc_base<E, L1, S1 - 1>(gg) +
                                      rc_off<E, L1, S1 - 1>(j)];
  }
  __syncthreads();
  const int lane = tid & 31, wib = tid >> 5;
  const int q = lane / G, g = lane % G;
  const unsigned n1 = (unsigned)p.n1, n2 = (unsigned)p.n2;
  const unsigned per = n1 + n2;
  const unsigned NB = (unsigned)p.blocks;
  const unsigned total = NB * per;
  const unsigned lag = (unsigned)p.lag;
  const unsigned na = NB < lag ? NB : lag;
  const unsigned nb = NB > lag ? NB - lag : 0u;
  const FDiv dAc((unsigned)p.c.A), dAh((unsigned)p.h.A),
      dSh((unsigned)p.h.es);
  for (;;) {
    if (tid == 0) sitem[0] = atomicAdd(p.ctr, 1u);
    __syncthreads();
    const unsigned item = sitem[0];
    __syncthreads();  // (sitem is rewritten by the next item)
    if (item >= total) break;
    // block k's convolution items, then block k - lag's FWHT items (the
    // first lag blocks' convolutions alone, the last lag blocks' FWHTs at
    // the end)
    bool first;
    unsigned blk, idx;
    if (item < na * n1) {
      first = true;
      blk = item / n1;
      idx = item % n1;
    } else if (item - na * n1 < nb * per) {
      const unsigned i = item - na * n1;
      const unsigned k = lag + i / per, r = i % per;
      first = r < n1;
      blk = first ? k : k - lag;
      idx = first ? r : r - n1;
    } else {
      const unsigned i = item - na * n1 - nb * per;
      first = false;
      blk = nb + i / n2;
      idx = i % n2;
    }
    if (first) {
      // VPC contiguous vectors; warp wib takes VPW of them, lane g of
      // vector q its points g + G r
      E *buf = reinterpret_cast<E *>(region) +
               (wib * VPW + q) * RcBuf<E, L1>::Lp;
      const i64 v = ((i64)blk * n1 + idx) * VPC + wib * VPW + q;
      const unsigned m = dAc.div((unsigned)v);
      const unsigned a = (unsigned)v - m * (unsigned)p.c.A;
      const Raw *src = (const Raw *)p.c.src + (i64)m * p.c.ld_src +
                       (i64)a * p.c.in_stride;
      Raw d[P];
#pragma unroll
      for (int r = 0; r < P; ++r) d[r] = src[g + G * r];
      E x[P];
      int s = 0;
      if constexpr (Emu<E>::v) {
        int emax = 0;
#pragma unroll
        for (int r = 0; r < P; ++r)
          emax = max(emax, max(dexp(d[r].x), dexp(d[r].y)));
#pragma unroll
        for (int o = G / 2; o >= 1; o /= 2)
          emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o, G));
        s = emax > 0 ? emax - 1023 : 0;
#pragma unroll
        for (int r = 0; r < P; ++r)
          x[r] = dfc{d2df_scaled(d[r].x, s), d2df_scaled(d[r].y, s)};
      } else {
#pragma unroll
        for (int r = 0; r < P; ++r) x[r] = d[r];
      }
      rc_forward<E, L1, 0>(x, buf, g, stw);
#pragma unroll
      for (int j = 0; j < P; ++j)
        x[j] = mulv(x[j], sspec[j * G + g], p.c.spec_conj != 0);
      rc_inverse<E, L1, S1 - 1>(x, buf, g, stw);
      Raw *dst = (Raw *)p.c.dst + (i64)m * p.c.ld_dst +
                 (i64)a * p.c.out_stride;
#pragma unroll
      for (int r = 0; r < P; ++r) {
        if constexpr (Emu<E>::v)
          dst[g + G * r] = make_double2(df2d_scaled(x[r].x, s),
                                        df2d_scaled(x[r].y, s));
        else
          dst[g + G * r] = x[r];
      }
      // this item's stores, then its count (release)
      __syncthreads();
      if (tid == 0) {
        __threadfence();
        atomicAdd(p.ctr + 1 + blk, 1u);
      }
    } else {
      // wait for the block's convolution items (acquire), bounded
      if (tid == 0) {
        long long polls = 0;
        unsigned done;
        for (;;) {
          asm volatile("ld.acquire.gpu.global.u32 %0, [%1];"
                       : "=r"(done)
                       : "l"(p.ctr + 1 + blk)
                       : "memory");
          if (done >= n1) break;
          if (++polls > p.wait_limit) {
            atomicExch(p.err, FM_ERR_TIMEOUT);
            break;
          }
          __nanosleep(64);
        }
        sitem[1] = done >= n1 ? 1u : 0u;
      }
      __syncthreads();
      const bool ready = sitem[1] != 0;
      __syncthreads();
      if (ready) {
        R *xb = reinterpret_cast<R *>(region);
        int *sexp = reinterpret_cast<int *>(xb + NV2 * RsShape<R, L2>::Lx);
        rs_batch<R, L2, NV2>(p.h, (i64)blk * n2 + idx, xb, sexp, dAh, dSh);
      }
    }
    __syncthreads();  // shared memory is reused by the next item
  }
}

}  // namespace fmk
