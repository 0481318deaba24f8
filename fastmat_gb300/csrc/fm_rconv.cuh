// Register-resident circular convolution of contiguous power-of-two vectors:
//
//     y = post . conj_out(scale * IFFT(S . FFT(zpad(pre . conj_in(x)))))
//
// the program a Circulant / Toeplitz / Bluestein apply lowers to when its
// length fits one warp (fastmat applies it as fft, product, ifft:
// fastmat/Circulant.pyx:127-133, fastmat/Toeplitz.pyx:255-268).  The generic
// vector-program kernel runs every FFT stage as a pass through a shared-
// memory tile with run-time index arithmetic; here the whole transform pair
// lives in registers:
//
//   * a vector of L points is held by G = L / P lanes of one warp, P points
//     per lane (16 complex64 or 8 double-float complex), loaded straight
//     from global memory in natural order (lane g holds points g + G r), so
//     a warp covers 32 / G vectors;
//   * the forward FFT is an in-place decimation-in-frequency over the radix
//     sequence (P, P, ..., rest): every stage is P / R radix-R butterflies
//     per lane in registers, with the twiddles of its butterflies (which
//     depend only on the lane) from a table in shared memory; between stages
//     the lanes of a vector exchange points through a per-warp shared-memory
//     buffer (warp barriers only);
//   * after the last forward stage each lane holds its points in digit-
//     reversed order; they are multiplied by the spectrum stored in that
//     order, and the inverse transform (decimation in time, the stages in
//     reverse) starts on the same registers: the last forward and the first
//     inverse stage share their butterflies, so no exchange between them;
//   * the inverse leaves lane g with points g + G r again, stored straight
//     to global memory.
//
// Positions follow the in-place DIF of the vector-program kernel
// (fm_vprog.cuh): stage i with radix R, Mprev = L / (R_0 ... R_{i-1}) and
// M = Mprev / R takes, for block K and t < M, the points K Mprev + t + M r.
// Lane g's butterflies at stage i are w = g + G u (u < P / R); because M
// divides G, t = g mod M and the position is a per-lane base plus a
// compile-time offset u G R + M r.
#pragma once

#include <type_traits>

#include "fm_vprog.cuh"

namespace fmk {

// One launch of the register convolution (built by the planner from a
// vector-program step whose program is [zero pad] FFT, product, inverse FFT
// on contiguous vectors).
struct RcStep {
  const void *src;
  void *dst;
  i64 ld_src, ld_dst;
  int src_type, dst_type;
  i64 A;                      // vectors per column
  i64 in_stride, out_stride;  // rows from one vector of a column to the next
  i64 in_rows, out_rows;      // rows of a column that exist / are written
  int in_len, out_len;        // points of a vector read (rest: zero) / stored
  i64 num_cols;
  const void *spec;  // spectrum / L in the forward stages' output order
  const void *tw;    // tw[j] = exp(-2 pi i j / L), j < L
  const void *pre, *post;  // loader / storer products indexed by row
  int *err;
  int spec_conj, conj_in, conj_out, has_scale, accumulate;
  int L;
  double scale_re, scale_im;
};

// ---- compile-time plan: P points per lane, radices (P, P, ..., rest)
// (rc_stages / rc_radix / rc_mprev / rc_log2 in fm_rtile.cuh)
template <class E> struct RcLane {
  static constexpr int P = sizeof(E) == 8 ? 16 : 8;
};

// Shared-memory layout of a vector's exchange buffer: point p at
// p + (p >> SH), vectors Lp points apart; its input slot: natural order,
// vectors Ls points apart.  (SH, Lp, Ls) per element size and length were
// chosen by enumerating the bank pattern of every access the kernel makes
// (the stage layouts' exchange writes and reads and the slot reads, per
// half- or quarter-warp phase): all are conflict-free except the exchange
// of L = 32 (4 wavefronts where 3 would do, on average); the twiddle and
// spectrum tables are read lane-major (consecutive lanes, consecutive
// entries) and broadcast across the vectors of a warp.
template <class E, int L> struct RcBuf {
  static constexpr bool C64 = sizeof(E) == 8;
  static constexpr int SH =
      C64 ? (L == 64 ? 2 : L == 128 ? 3 : 4) : (L == 32 ? 2 : 3);
  static constexpr int Lp =
      C64 ? (L == 16 ? 17 : L == 32 ? 34 : L == 64 ? 84 : L == 128 ? 152
             : L + (L >> 4))
          : (L == 8 ? 9 : L == 32 ? 44 : L + (L >> 3));
  // input slot stride (natural order, read at g + G r): conflict-free
  static constexpr int Ls = C64 ? (L <= 128 ? L + L / 16 : L)
                                : (L <= 32 ? L + L / 8 : L);
};
template <class E, int L> __device__ __forceinline__ int rc_pad(int p) {
  return p + (p >> RcBuf<E, L>::SH);
}

// Offset of stage I's lane-major twiddle table (R_I x G entries, stages
// with M > 1 only) within the twiddle area of shared memory.
template <class E, int L, int I>
__host__ __device__ constexpr int rc_twoff() {
  constexpr int P = RcLane<E>::P;
  if constexpr (I == 0) {
    return 0;
  } else {
    constexpr int R = rc_radix(I - 1, L, P);
    constexpr int M = rc_mprev(I - 1, L, P) / R;
    return rc_twoff<E, L, I - 1>() + (M > 1 ? R * (L / P) : 0);
  }
}
template <class E, int L, int I>
__host__ __device__ constexpr int rc_twlen() {  // entries of stages < I
  return rc_twoff<E, L, I>();
}

// Stage `I` of the forward (INV = false: DFT, then twiddles of the outputs)
// or inverse (INV = true: conjugate twiddles of the inputs, then DFT with
// sign +1) transform on the lane's P registers, in place: register
// u R + r holds position base + u G R + M r before and after.
template <class E, int L, int I, bool INV, int FSG = -1>
__device__ __forceinline__ void rc_stage(E (&x)[RcLane<E>::P], int g,
                                         const E *__restrict__ stw) {
  constexpr int P = RcLane<E>::P;
  constexpr int R = rc_radix(I, L, P);
  constexpr int Mprev = rc_mprev(I, L, P);
  constexpr int M = Mprev / R;
  constexpr int NB = P / R;
  constexpr int TS = L / Mprev;  // table stride of w_Mprev
  constexpr int SG = INV ? +1 : FSG;  // FSG: sign of a forward-order DIF
  typedef typename Lazy<E>::type LC;
  constexpr int G = L / P;
  // the twiddles w_Mprev^(t k), t = g mod M, k < R, are the same for all
  // u: lane-major table of this stage (entry k G + g), conflict-free reads
  E w[R];
  if constexpr (M > 1) {
    const E *tab = stw + rc_twoff<E, L, I>();
#pragma unroll
    for (int k = 1; k < R; ++k) w[k] = tab[k * G + g];
  }
  (void)TS;
#pragma unroll
  for (int u = 0; u < NB; ++u) {
    LC v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = to_lazy(x[u * R + r]);
    if constexpr (INV && M > 1) {
#pragma unroll
      for (int k = 1; k < R; ++k) v[k] = cmul_lazy<+1>(v[k], w[k]);
    }
    dif_stages<R, R / 2>(v, SG);  // v[i] = output brev(i)
#pragma unroll
    for (int i = 0; i < R; ++i) {
      LC y = v[i];
      const int k = brev<R>(i);
      if constexpr (!INV && M > 1) {
        if (k != 0) y = cmul_lazy<FSG>(y, w[k]);
      }
      x[u * R + k] = from_lazy(y);
    }
  }
}

// position base of lane g at stage I (see the file comment)
template <class E, int L, int I>
__device__ __forceinline__ int rc_base(int g) {
  constexpr int P = RcLane<E>::P;
  constexpr int Mprev = rc_mprev(I, L, P);
  constexpr int M = Mprev / rc_radix(I, L, P);
  constexpr int LM = rc_log2(M);
  return (g >> LM) * Mprev + (g & (M - 1));
}
template <class E, int L, int I>
__device__ __forceinline__ int rc_off(int j) {  // register j = u R + r
  constexpr int P = RcLane<E>::P;
  constexpr int R = rc_radix(I, L, P);
  constexpr int G = L / P;
  constexpr int M = rc_mprev(I, L, P) / R;
  return (j / R) * G * R + M * (j % R);
}

// Registers laid out for stage IA -> shared buffer -> registers laid out
// for stage IB (warp barriers: the lanes of a vector are in one warp).
// (CTA: the threads of a vector span several warps, CTA barriers)
template <class E, int L, int IA, int IB, bool CTA = false>
__device__ __forceinline__ void rc_exchange(E (&x)[RcLane<E>::P], E *buf,
                                            int g) {
  constexpr int P = RcLane<E>::P;
  const int ba = rc_base<E, L, IA>(g), bb = rc_base<E, L, IB>(g);
#pragma unroll
  for (int j = 0; j < P; ++j)
    buf[rc_pad<E, L>(ba + rc_off<E, L, IA>(j))] = x[j];
  if constexpr (CTA)
    __syncthreads();
  else
    __syncwarp();
#pragma unroll
  for (int j = 0; j < P; ++j)
    x[j] = buf[rc_pad<E, L>(bb + rc_off<E, L, IB>(j))];
  if constexpr (CTA)
    __syncthreads();
  else
    __syncwarp();
}

template <class E, int L, int I, int FSG = -1, bool CTA = false>
__device__ __forceinline__ void rc_forward(E (&x)[RcLane<E>::P], E *buf, int g,
                                           const E *stw) {
  rc_stage<E, L, I, false, FSG>(x, g, stw);
  constexpr int S = rc_stages(L, RcLane<E>::P);
  if constexpr (I + 1 < S) {
    rc_exchange<E, L, I, I + 1, CTA>(x, buf, g);
    rc_forward<E, L, I + 1, FSG, CTA>(x, buf, g, stw);
  }
}

// natural index of the forward transform's output position p (radices
// (P, ..., rest), R_0 most significant in the position): its digits in
// reverse
template <class E, int L, int I>
__host__ __device__ constexpr int rc_below() {  // bits of the digits > I
  constexpr int P = RcLane<E>::P;
  if constexpr (I + 1 >= rc_stages(L, P))
    return 0;
  else
    return rc_log2(rc_radix(I + 1, L, P)) + rc_below<E, L, I + 1>();
}
template <class E, int L, int I>
__device__ __forceinline__ int rc_nat_from(int p, int sh) {
  constexpr int P = RcLane<E>::P;
  if constexpr (I >= rc_stages(L, P)) {
    return 0;
  } else {
    constexpr int BI = rc_log2(rc_radix(I, L, P));
    constexpr int BELOW = rc_below<E, L, I>();
    return (((p >> BELOW) & ((1 << BI) - 1)) << sh) |
           rc_nat_from<E, L, I + 1>(p, sh + BI);
  }
}
template <class E, int L>
__device__ __forceinline__ int rc_nat(int p) {
  return rc_nat_from<E, L, 0>(p, 0);
}
template <class E, int L, int I>
__device__ __forceinline__ void rc_inverse(E (&x)[RcLane<E>::P], E *buf, int g,
                                           const E *stw) {
  rc_stage<E, L, I, true>(x, g, stw);
  if constexpr (I > 0) {
    rc_exchange<E, L, I, I - 1>(x, buf, g);
    rc_inverse<E, L, I - 1>(x, buf, g, stw);
  }
}

// threads per CTA and CTAs per SM of the register convolution
#define FM_RC_THREADS 256
template <class E, int L> struct RcOcc {
  static constexpr int v = sizeof(E) == 8 && L < 512 ? 3 : 2;
};

// shared memory: twiddle and spectrum tables, then per warp an input slot
// (the next vectors, copied in ahead) and an exchange buffer
template <class E, int L>
__host__ __device__ constexpr size_t rc_smem() {
  return (size_t)(rc_twlen<E, L, rc_stages(L, RcLane<E>::P)>() + L +
                  (FM_RC_THREADS / 32) * (32 / (L / RcLane<E>::P)) *
                      (RcBuf<E, L>::Lp + RcBuf<E, L>::Ls)) *
         sizeof(E);
}

// Fill the lane-major twiddle tables of stages I.. from the natural table
// tw[j] = exp(-2 pi i j / L): entry k G + g of stage I is w_Mprev^(t k),
// t = g mod M (the stage's table stride L / Mprev in tw).
template <class E, int L, int I>
__device__ __forceinline__ void rc_fill_tw(E *stw, const E *tw) {
  constexpr int P = RcLane<E>::P;
  constexpr int S = rc_stages(L, P);
  if constexpr (I < S) {
    constexpr int R = rc_radix(I, L, P);
    constexpr int Mprev = rc_mprev(I, L, P);
    constexpr int M = Mprev / R;
    constexpr int G = L / P;
    if constexpr (M > 1) {
      E *tab = stw + rc_twoff<E, L, I>();
      for (int i = threadIdx.x; i < R * G; i += blockDim.x) {
        const int k = i / G, g = i % G;
        tab[i] = tw[(g & (M - 1)) * k * (L / Mprev)];
      }
    }
    rc_fill_tw<E, L, I + 1>(stw, tw);
  }
}

template <class E, int L>
__global__ void __launch_bounds__(FM_RC_THREADS, (RcOcc<E, L>::v))
    rconv_kernel(const __grid_constant__ RcStep p) {
  constexpr int P = RcLane<E>::P;
  constexpr int G = L / P;
  static_assert(G >= 1 && G <= 32 && (G & (G - 1)) == 0, "lanes per vector");
  constexpr int VPW = 32 / G;
  constexpr int S = rc_stages(L, P);
  constexpr int Lp = RcBuf<E, L>::Lp;
  extern __shared__ __align__(128) unsigned char fm_smem[];
  constexpr int TWN = rc_twlen<E, L, S>();
  E *stw = reinterpret_cast<E *>(fm_smem);
  E *sspec = stw + TWN;
  E *sx = sspec + L;
  rc_fill_tw<E, L, 0>(stw, (const E *)p.tw);
  // spectrum in lane-major order: entry j G + g is the point lane g holds
  // in register j after the last forward stage
  for (int i = threadIdx.x; i < L; i += blockDim.x) {
    const int j = i / G, gg = i % G;
    sspec[i] = ((const E *)p.spec)[rc_base<E, L, S - 1>(gg) +
                                    rc_off<E, L, S - 1>(j)];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int q = lane / G, g = lane % G;
  E *buf = sx + (wib * VPW + q) * Lp;  // exchange buffer of this vector
  // input slot of this vector: the raw bits of its points, natural order
  E *slot = sx + (FM_RC_THREADS / 32) * VPW * Lp +
            (wib * VPW + q) * RcBuf<E, L>::Ls;
  const i64 NV = p.A * p.num_cols;
  const FDiv dA((unsigned)p.A);
  const i64 nwarps = (i64)gridDim.x * (blockDim.x >> 5);
  // inputs already in the buffers' type are copied in one batch ahead by
  // cp.async (zero-filled beyond the vector / the column); others are
  // converted by synchronous loads
  const bool raw_in = p.src_type == Tr<E>::code;
  const bool raw_out = p.dst_type == Tr<E>::code && !p.accumulate;
  const bool plain_out =
      raw_out && !p.post && !p.has_scale && !p.conj_out;
  const E cs = scalar_of<E>(p.scale_re, p.scale_im);
  typedef typename std::conditional<Emu<E>::v, double2, E>::type Raw;
  static_assert(sizeof(Raw) == sizeof(E), "raw element size");
  auto prefetch = [&](i64 vn) {
    const i64 v = vn + q;
    unsigned m = 0, a = 0;
    const bool act = v < NV;
    if (act) {
      m = dA.div((unsigned)v);
      a = (unsigned)v - m * (unsigned)p.A;
    }
    const Raw *src = (const Raw *)p.src + (i64)m * p.ld_src +
                     (i64)a * p.in_stride;
    const i64 left = p.in_rows - (i64)a * p.in_stride;
    if (act && p.in_len == L && left >= L) {  // whole vector: no masks
#pragma unroll
      for (int r = 0; r < P; ++r)
        cp_async<sizeof(E)>(slot + g + G * r, src + g + G * r, true);
    } else {
#pragma unroll
      for (int r = 0; r < P; ++r) {
        const int j = g + G * r;
        const bool ok = act && j < p.in_len && j < left;
        cp_async<sizeof(E)>(slot + j, ok ? (const void *)(src + j)
                                         : (const void *)p.src, ok);
      }
    }
    cp_async_commit();
  };
  const i64 v0 = ((i64)blockIdx.x * (blockDim.x >> 5) + wib) * VPW;
  if (raw_in && v0 < NV) prefetch(v0);
  for (i64 vb = v0; vb < NV; vb += nwarps * VPW) {
    const i64 v = vb + q;
    const bool act = v < NV;
    unsigned m = 0, a = 0;
    if (act) {
      m = dA.div((unsigned)v);
      a = (unsigned)v - m * (unsigned)p.A;
    }
    const i64 rin0 = (i64)a * p.in_stride;   // row of point 0 in the column
    const i64 rout0 = (i64)a * p.out_stride;
    E x[P];
    Raw d[P];
    if (raw_in) {
      cp_async_wait<0>();
      __syncwarp();
#pragma unroll
      for (int r = 0; r < P; ++r)
        d[r] = reinterpret_cast<const Raw *>(slot)[g + G * r];
      __syncwarp();
      if (vb + nwarps * VPW < NV) prefetch(vb + nwarps * VPW);
    } else {
#pragma unroll
      for (int r = 0; r < P; ++r) {
        const int j = g + G * r;
        const i64 row = rin0 + j;
        Raw val;
        if constexpr (Emu<E>::v) {
          val = make_double2(0., 0.);
          if (act && j < p.in_len && row < p.in_rows) {
            double re, im;
            split(load_as<double2>(p.src, p.src_type,
                                   (i64)m * p.ld_src + row),
                  re, im);
            val = make_double2(re, im);
          }
        } else {
          val = zero<E>();
          if (act && j < p.in_len && row < p.in_rows)
            val = load_as<E>(p.src, p.src_type, (i64)m * p.ld_src + row);
        }
        d[r] = val;
      }
    }
    int sexp = 0;
    if constexpr (Emu<E>::v) {
      // float64 / complex128 bits, scaled per vector by the power of two of
      // its largest exponent (the double-float exponent range is float's)
      int emax = 0;
#pragma unroll
      for (int r = 0; r < P; ++r)
        emax = max(emax, max(dexp(d[r].x), dexp(d[r].y)));
#pragma unroll
      for (int o = G / 2; o >= 1; o /= 2)
        emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o, G));
      sexp = emax > 0 ? emax - 1023 : 0;
#pragma unroll
      for (int r = 0; r < P; ++r)
        x[r] = dfc{d2df_scaled(d[r].x, sexp), d2df_scaled(d[r].y, sexp)};
    } else {
#pragma unroll
      for (int r = 0; r < P; ++r) x[r] = d[r];
    }
    if (p.conj_in || p.pre) {
#pragma unroll
      for (int r = 0; r < P; ++r) {
        const i64 row = rin0 + g + G * r;
        if (p.conj_in) x[r] = conjv(x[r]);
        if (p.pre && g + G * r < p.in_len && row < p.in_rows)
          x[r] = mulv(x[r], ((const E *)p.pre)[row], false);
      }
    }
    // ---- forward transform, spectrum product, inverse transform
    rc_forward<E, L, 0>(x, buf, g, stw);
#pragma unroll
    for (int j = 0; j < P; ++j)
      x[j] = mulv(x[j], sspec[j * G + g], p.spec_conj != 0);
    rc_inverse<E, L, S - 1>(x, buf, g, stw);
    // ---- store points g + G r
    if (act && plain_out && p.out_len == L && rout0 + L <= p.out_rows) {
      // whole vector in the buffer's type, nothing applied on the way out
      const i64 base = (i64)m * p.ld_dst + rout0;
#pragma unroll
      for (int r = 0; r < P; ++r) {
        if constexpr (Emu<E>::v)
          ((double2 *)p.dst)[base + g + G * r] = make_double2(
              df2d_scaled(x[r].x, sexp), df2d_scaled(x[r].y, sexp));
        else
          ((E *)p.dst)[base + g + G * r] = x[r];
      }
    } else if (act) {
#pragma unroll
      for (int r = 0; r < P; ++r) {
        const int j = g + G * r;
        const i64 row = rout0 + j;
        if (j >= p.out_len || row >= p.out_rows) continue;
        E val = x[r];
        if (p.post) val = mulv(val, ((const E *)p.post)[row], false);
        if (p.has_scale) val = mulv(val, cs, false);
        if (p.conj_out) val = conjv(val);
        const i64 idx = (i64)m * p.ld_dst + row;
        if constexpr (Emu<E>::v) {
          if (raw_out)
            ((double2 *)p.dst)[idx] = make_double2(
                df2d_scaled(val.x, sexp), df2d_scaled(val.y, sexp));
          else
            store_as<E>(p.dst, p.dst_type, idx, val, p.accumulate != 0,
                        sexp);
        } else {
          if (raw_out)
            ((E *)p.dst)[idx] = val;
          else
            store_as<E>(p.dst, p.dst_type, idx, val, p.accumulate != 0);
        }
      }
    }
  }
}

}  // namespace fmk
