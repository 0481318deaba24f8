// Register-resident Walsh-Hadamard transform of contiguous power-of-two
// vectors (fastmat's Hadamard, fastmat/Hadamard.pyx:164-230: a + b / a - b
// butterflies at distance 1, 2, 4, ...), for real float32 and double-float
// data.
//
//   * a vector of L points is held by G = L / P threads of a CTA, P points
//     per thread (32 float or 16 double-float); the CTA works on
//     max(1, 256 / G) vectors at a time;
//   * the index bits are taken in passes of log2(P) bits from the least
//     significant one, so the butterflies run in fastmat's order and float32
//     results are bit-identical to its float32 transform; within a pass every
//     thread's groups of points (the points that differ only in the pass's
//     bits) are in its registers, and the levels of the pass are plain
//     register butterflies (double-float: unnormalised inside the pass, one
//     renormalisation at its end);
//   * the first pass takes thread t's P consecutive points (t P .. t P + P-1)
//     from a shared-memory slot that cp.async filled one batch ahead; between
//     passes the points go through a shared-memory exchange buffer (CTA
//     barriers: a long vector spans several warps); the last pass stores
//     straight to global memory, consecutive threads on consecutive points.
//
// Thread t's groups at a pass with bit offset s and width w are
// h = t + G u (u < P / 2^w); point r of group h sits at
// ((h >> s) << (s + w)) | (r << s) | (h mod 2^s).  The exchange buffer puts
// point e at e + (e >> 5) (float) or e + (e >> 4) (double-float), the slot
// holds raw float32 / float64 words with a 16-byte pad per 128 bytes: every
// access pattern of the kernel is then free of bank conflicts (checked by
// enumerating them for the lengths instantiated).
#pragma once

#include <type_traits>

#include "fm_vprog.cuh"

namespace fmk {

// One launch of the register FWHT (built by the planner from a vector
// program that is one FWHT over contiguous whole vectors).
struct RfStep {
  const void *src;
  void *dst;
  i64 ld_src, ld_dst;
  i64 A;       // vectors per column
  i64 stride;  // contiguous vectors: rows from one vector to the next
  i64 es;      // element stride: 1 contiguous vectors; S > 1: vector
               // v = a S + c has point j at row a L S + c + j S
  i64 num_cols;
  int *err;
  int L;
};

#define FM_RF_THREADS 256
template <class E> struct RfLane {
  static constexpr int P = std::is_same<E, float>::value ? 32 : 16;
  static constexpr int PB = std::is_same<E, float>::value ? 5 : 4;
  // raw word of the global buffers: float32 or float64
  typedef typename std::conditional<std::is_same<E, float>::value, float,
                                    double>::type Raw;
  static constexpr int XSH = std::is_same<E, float>::value ? 5 : 4;
};
template <class E, int L> struct RfShape {
  static constexpr int P = RfLane<E>::P;
  static constexpr int G = L / P;
  static constexpr int T = G > FM_RF_THREADS ? G : FM_RF_THREADS;
  static constexpr int VPC = T / G;  // vectors per CTA batch
  typedef typename RfLane<E>::Raw Raw;
  static constexpr int CH = 16 / (int)sizeof(Raw);   // raw words per chunk
  static constexpr int ROW = 128 / (int)sizeof(Raw);  // raw words per 128 B
  static constexpr int Ls = L + (L / ROW) * CH;        // slot stride
  static constexpr int Lx = L + (L >> RfLane<E>::XSH);  // exchange stride
};
__host__ __device__ constexpr int rf_log2(int n) {
  return n <= 1 ? 0 : 1 + rf_log2(n / 2);
}
template <class E, int L>
__host__ __device__ constexpr size_t rf_smem() {
  typedef RfShape<E, L> S;
  return (size_t)S::VPC * S::Ls * sizeof(typename S::Raw) +
         (size_t)S::VPC * S::Lx * sizeof(E) + 64;
}
template <class E, int L> struct RfOcc {
  static constexpr int v = RfShape<E, L>::T > 256 ? 1 : 2;
};

template <class E>
__device__ __forceinline__ int rf_xpad(int e) {
  return e + (e >> RfLane<E>::XSH);
}
__device__ __forceinline__ int rf_pos(int h, int s, int r, int w) {
  return ((h >> s) << (s + w)) | (r << s) | (h & ((1 << s) - 1));
}

// the levels of one pass (w bits) on the thread's P registers, in place:
// register u 2^w + r is point r of group u
template <class LE, int P, int W>
__device__ __forceinline__ void rf_levels(LE (&v)[P]) {
  constexpr int R = 1 << W;
#pragma unroll
  for (int u = 0; u < P / R; ++u) {
#pragma unroll
    for (int h = 1; h < R; h <<= 1) {
#pragma unroll
      for (int r = 0; r < R; ++r) {
        if ((r & h) == 0) {
          const LE a = v[u * R + r], c = v[u * R + r + h];
          v[u * R + r] = addv(a, c);
          v[u * R + r + h] = subv(a, c);
        }
      }
    }
  }
}

template <class E, int L, int S0>
__device__ __forceinline__ void rf_pass(E (&x)[RfLane<E>::P]) {
  constexpr int P = RfLane<E>::P, PB = RfLane<E>::PB, K = rf_log2(L);
  constexpr int W = K - S0 < PB ? K - S0 : PB;
  typedef typename Lazy<E>::type LE;
  LE v[P];
#pragma unroll
  for (int j = 0; j < P; ++j) v[j] = to_lazy(x[j]);
  rf_levels<LE, P, W>(v);
#pragma unroll
  for (int j = 0; j < P; ++j) x[j] = from_lazy(v[j]);
}

// registers laid out for the pass at bit offset SA -> exchange buffer ->
// registers for the pass at SB (CTA barriers)
template <class E, int L, int SA, int SB>
__device__ __forceinline__ void rf_exchange(E (&x)[RfLane<E>::P], E *buf,
                                            int t) {
  constexpr int P = RfLane<E>::P, PB = RfLane<E>::PB, K = rf_log2(L);
  constexpr int G = L / P;
  constexpr int WA = K - SA < PB ? K - SA : PB;
  constexpr int WB = K - SB < PB ? K - SB : PB;
#pragma unroll
  for (int j = 0; j < P; ++j) {
    const int u = j >> WA, r = j & ((1 << WA) - 1);
    buf[rf_xpad<E>(rf_pos(t + G * u, SA, r, WA))] = x[j];
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < P; ++j) {
    const int u = j >> WB, r = j & ((1 << WB) - 1);
    x[j] = buf[rf_xpad<E>(rf_pos(t + G * u, SB, r, WB))];
  }
  __syncthreads();
}

template <class E, int L, int S0>
__device__ __forceinline__ void rf_passes(E (&x)[RfLane<E>::P], E *buf,
                                          int t) {
  constexpr int PB = RfLane<E>::PB, K = rf_log2(L);
  rf_pass<E, L, S0>(x);
  if constexpr (S0 + PB < K) {
    rf_exchange<E, L, S0, S0 + PB>(x, buf, t);
    rf_passes<E, L, S0 + PB>(x, buf, t);
  }
}
// bit offset of the last pass
template <class E, int L> __host__ __device__ constexpr int rf_last() {
  return ((rf_log2(L) - 1) / RfLane<E>::PB) * RfLane<E>::PB;
}

// The rest of a contiguous batch once thread t of vector vl holds its
// first-pass points d (raw words): double-float scaling, the passes, the
// stores of the last pass.
template <class E, int L>
__device__ __forceinline__ void rf_finish(
    typename RfShape<E, L>::Raw (&d)[RfLane<E>::P], const RfStep &p, i64 gv,
    bool act, E *buf, int *sexp, int vl, int t, const FDiv &dA) {
  typedef RfShape<E, L> Sh;
  constexpr int P = Sh::P, G = Sh::G, VPC = Sh::VPC;
  constexpr int SL = rf_last<E, L>();
  constexpr int WL = rf_log2(L) - SL;
  typedef typename Sh::Raw Raw;
  E x[P];
  int s = 0;
  if constexpr (Emu<E>::v) {
    // double-float: every vector scaled by the power of two of its
    // largest exponent (float's exponent range), restored on store
    // (reduced over the vector's lanes within each warp, then across its
    // warps in shared memory)
    constexpr int WV = G < 32 ? G : 32;
    int emax = 0;
#pragma unroll
    for (int r = 0; r < P; ++r) emax = max(emax, dexp(d[r]));
#pragma unroll
    for (int o = WV / 2; o >= 1; o /= 2)
      emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o, WV));
    if (threadIdx.x < VPC) sexp[threadIdx.x] = 0;
    __syncthreads();
    if (t % WV == 0 && emax > 0) atomicMax(sexp + vl, emax);
    __syncthreads();
    s = sexp[vl] > 0 ? sexp[vl] - 1023 : 0;
#pragma unroll
    for (int r = 0; r < P; ++r) x[r] = d2df_scaled(d[r], s);
  } else {
#pragma unroll
    for (int r = 0; r < P; ++r) x[r] = d[r];
  }
  rf_passes<E, L, 0>(x, buf, t);
  // last pass's points, straight to global memory
  if (act) {
    const unsigned m = dA.div((unsigned)gv);
    const unsigned a = (unsigned)gv - m * (unsigned)p.A;
    Raw *dst = (Raw *)p.dst + (i64)m * p.ld_dst + (i64)a * p.stride;
#pragma unroll
    for (int j = 0; j < P; ++j) {
      const int u = j >> WL, r = j & ((1 << WL) - 1);
      const int e = rf_pos(t + G * u, SL, r, WL);
      if constexpr (Emu<E>::v)
        dst[e] = df2d_scaled(x[j], s);
      else
        dst[e] = x[j];
    }
  }
}

template <class E, int L>
__global__ void __launch_bounds__(RfShape<E, L>::T, (RfOcc<E, L>::v))
    rfwht_kernel(const __grid_constant__ RfStep p) {
  typedef RfShape<E, L> Sh;
  typedef typename Sh::Raw Raw;
  constexpr int P = Sh::P, G = Sh::G, VPC = Sh::VPC;
  extern __shared__ __align__(128) unsigned char fm_smem[];
  Raw *slot = reinterpret_cast<Raw *>(fm_smem);
  E *xb = reinterpret_cast<E *>(fm_smem + (size_t)VPC * Sh::Ls * sizeof(Raw));
  int *sexp = reinterpret_cast<int *>(xb + (size_t)VPC * Sh::Lx);
  const int vl = threadIdx.x / G, t = threadIdx.x % G;
  Raw *vslot = slot + vl * Sh::Ls;
  E *buf = xb + vl * Sh::Lx;
  const i64 NV = p.A * p.num_cols;
  const FDiv dA((unsigned)p.A);
  const i64 step = (i64)gridDim.x * VPC;
  // cp.async of a batch of VPC vectors into the slot, 16-byte chunks
  auto prefetch = [&](i64 vb) {
    constexpr int NCH = VPC * L / Sh::CH;
    for (int c = threadIdx.x; c < NCH; c += Sh::T) {
      const int v = c / (L / Sh::CH), ch = c % (L / Sh::CH);
      const i64 gv = vb + v;
      const bool ok = gv < NV;
      const Raw *src = (const Raw *)p.src;
      if (ok) {
        const unsigned m = dA.div((unsigned)gv);
        const unsigned a = (unsigned)gv - m * (unsigned)p.A;
        src += (i64)m * p.ld_src + (i64)a * p.stride + (i64)ch * Sh::CH;
      }
      const int e = ch * Sh::CH;
      cp_async<16>(slot + v * Sh::Ls + e + (e / Sh::ROW) * Sh::CH, src, ok);
    }
    cp_async_commit();
  };
  const i64 v0 = (i64)blockIdx.x * VPC;
  if (v0 < NV) prefetch(v0);
  for (i64 vb = v0; vb < NV; vb += step) {
    const i64 gv = vb + vl;
    const bool act = gv < NV;
    cp_async_wait<0>();
    __syncthreads();
    // first pass: points t P .. t P + P - 1 of the vector
    // (P raw words = 128 bytes per thread, one 16-byte pad after them)
    Raw d[P];
    {
      typedef typename std::conditional<std::is_same<Raw, float>::value,
                                        float4, double2>::type V;
      const V *src = reinterpret_cast<const V *>(vslot + t * (P + Sh::CH));
#pragma unroll
      for (int c = 0; c < P / Sh::CH; ++c)
        *reinterpret_cast<V *>(d + c * Sh::CH) = src[c];
    }
    __syncthreads();
    if (vb + step < NV) prefetch(vb + step);
    rf_finish<E, L>(d, p, gv, act, buf, sexp, vl, t, dA);
  }
  cp_async_wait<0>();
}

// ---- strided vectors (the high index bits of a long transform: vectors
// of L points at element stride S, S a multiple of 32, adjacent vectors
// adjacent in memory).  The lanes of a warp take NV = 32 (or, for vectors
// of more than 32 P points, 16) adjacent vectors, so every load and store of
// a warp is one or two contiguous row segments; the CTA's threads share the
// vectors' points, thread t = tid / NV of vector v = tid % NV holding points
// t P .. t P + P - 1 as thread t of the contiguous kernel,
// and the passes run as there (the exchanges go through a buffer per vector
// whose odd stride keeps the lanes of each half-warp on distinct banks).
// The first pass loads straight from global memory (P independent loads per
// thread), the last stores straight to it.
template <class E, int L> struct RsShape {
  static constexpr int P = RfLane<E>::P;
  static constexpr int W = L / P;             // threads per vector
  static constexpr int NV = W > 32 ? 16 : 32;  // vectors per CTA batch
  static constexpr int T = NV * W;
  static constexpr int Lx = (L + (L >> RfLane<E>::XSH)) | 1;
};
template <class E, int L>
__host__ __device__ constexpr size_t rs_smem() {
  return (size_t)RsShape<E, L>::NV * RsShape<E, L>::Lx * sizeof(E) +
         32 * sizeof(int);
}
template <class E, int L> struct RsOcc {
  static constexpr int v =
      RsShape<E, L>::T >= 1024 ? 1 : 1024 / RsShape<E, L>::T;
};

// One batch bt of NV adjacent strided vectors (NV = 32, 16, ..., the
// launch's threads / (L / P)): thread t = tid / NV of vector v = tid % NV.
template <class E, int L, int NV>
__device__ __forceinline__ void rs_batch(const RfStep &p, i64 bt, E *xb,
                                         int *sexp, const FDiv &dA,
                                         const FDiv &dS) {
  typedef typename RfLane<E>::Raw Raw;
  constexpr int P = RfLane<E>::P, W = L / P;
  constexpr int Lx = RsShape<E, L>::Lx;
  constexpr int SL = rf_last<E, L>();
  constexpr int WL = rf_log2(L) - SL;
  const int v = threadIdx.x % NV, t = threadIdx.x / NV;
  E *buf = xb + v * Lx;
  const i64 S = p.es;
  const unsigned gv = (unsigned)(bt * NV);
  const unsigned m = dA.div(gv), v0 = gv - m * (unsigned)p.A;
  const unsigned a = dS.div(v0), c0 = v0 - a * (unsigned)S;
  const i64 row0 = (i64)a * L * S + c0 + v;
  const Raw *src = (const Raw *)p.src + (i64)m * p.ld_src + row0;
  Raw d[P];
#pragma unroll
  for (int r = 0; r < P; ++r) d[r] = src[(i64)(t * P + r) * S];
  E x[P];
  int s = 0;
  if constexpr (Emu<E>::v) {
    // double-float: each vector scaled by the power of two of its largest
    // exponent (float's exponent range), restored on store
    int emax = 0;
#pragma unroll
    for (int r = 0; r < P; ++r) emax = max(emax, dexp(d[r]));
    if (threadIdx.x < NV) sexp[threadIdx.x] = 0;
    __syncthreads();
    if (emax > 0) atomicMax(sexp + v, emax);
    __syncthreads();
    s = sexp[v] > 0 ? sexp[v] - 1023 : 0;
#pragma unroll
    for (int r = 0; r < P; ++r) x[r] = d2df_scaled(d[r], s);
  } else {
#pragma unroll
    for (int r = 0; r < P; ++r) x[r] = d[r];
  }
  // (W >= 2: the passes hold at least one exchange, whose barriers also
  // separate this batch's reads of sexp from the next batch's reset)
  static_assert(W >= 2, "threads per vector");
  rf_passes<E, L, 0>(x, buf, t);
  Raw *dst = (Raw *)p.dst + (i64)m * p.ld_dst + row0;
#pragma unroll
  for (int j = 0; j < P; ++j) {
    const int u = j >> WL, r = j & ((1 << WL) - 1);
    const int e = rf_pos(t + W * u, SL, r, WL);
    if constexpr (Emu<E>::v)
      dst[(i64)e * S] = df2d_scaled(x[j], s);
    else
      dst[(i64)e * S] = x[j];
  }
}

template <class E, int L>
__global__ void __launch_bounds__(RsShape<E, L>::T, (RsOcc<E, L>::v))
    rsfwht_kernel(const __grid_constant__ RfStep p) {
  typedef RsShape<E, L> Sh;
  static_assert(Sh::T <= 1024, "threads per CTA");
  extern __shared__ __align__(128) unsigned char fm_smem[];
  E *xb = reinterpret_cast<E *>(fm_smem);
  int *sexp = reinterpret_cast<int *>(xb + Sh::NV * Sh::Lx);
  const i64 nb = p.A * p.num_cols / Sh::NV;  // batches of NV vectors
  const FDiv dA((unsigned)p.A), dS((unsigned)p.es);
  for (i64 bt = blockIdx.x; bt < nb; bt += gridDim.x)
    rs_batch<E, L, Sh::NV>(p, bt, xb, sexp, dA, dS);
}

// ---- both passes of a two-pass FWHT (fastmat/Hadamard.pyx:164-230 for
// 2^n > one tile: the low bits on contiguous vectors of L1 points, then the
// high bits on vectors of L2 points at stride L1) in one cooperative
// persistent launch that works column by column, so that a column's
// intermediate result (written to y by the first pass, transformed in place
// by the second) is still in L2 when the second pass reads it.  Work items
// are handed out in order by an atomic counter: the first-pass items of
// column k (one vector each), then the second-pass items of column k - lag
// (NV2 strided vectors each; the planner uses lag 1).  A second-pass item of column m waits until
// all first-pass items of column m have finished (their count in ctr[1 +
// m], raised with release semantics after each item's stores; read with
// acquire semantics, polls bounded by wait_limit).  Every awaited item was
// handed out earlier to a resident CTA (the launch is cooperative) and never
// waits itself, so the waits end.
struct RfPair {
  RfStep a;        // contiguous pass, x -> y
  RfStep b;        // strided pass, y -> y in place
  unsigned *ctr;   // [0] items handed out, [1 + m] first-pass items done
  int *err;
  long long wait_limit;
  int lag;         // columns between a column's first and second pass
};
#define FM_RF2_THREADS 256

// shared memory: the item index, one region for the first pass's copy slot
// and exchange buffer (the slot is read into registers before the first
// exchange writes) or the second pass's exchange buffers, the exponents.
// (A second region to copy the next item in while one runs costs a CTA per
// SM and measured slower: 0.81 against 0.67 ms for Hadamard(22) float32.)
template <class E, int L1, int L2> struct Rf2Mem {
  typedef RfShape<E, L1> S1;
  static constexpr int NV2 = FM_RF2_THREADS / (L2 / RfLane<E>::P);
  static constexpr size_t slot = (size_t)S1::Ls * sizeof(typename S1::Raw);
  static constexpr size_t x1 = (size_t)S1::Lx * sizeof(E);
  static constexpr size_t x2 = (size_t)NV2 * RsShape<E, L2>::Lx * sizeof(E);
  static constexpr size_t m01 = slot > x1 ? slot : x1;
  static constexpr size_t region = ((m01 > x2 ? m01 : x2) + 15) / 16 * 16;
  static constexpr size_t bytes = 16 + region + 4 * (NV2 > 1 ? NV2 : 1);
};
template <class E, int L1, int L2>
__host__ __device__ constexpr size_t rf2_smem() {
  return Rf2Mem<E, L1, L2>::bytes;
}
// CTAs per SM: float32 fits four (64 registers a thread), double-float three
template <class E> struct Rf2Occ {
  static constexpr int v = std::is_same<E, float>::value ? 4 : 3;
};

template <class E, int L1, int L2>
__global__ void __launch_bounds__(FM_RF2_THREADS, (Rf2Occ<E>::v))
    rfwht2_kernel(const __grid_constant__ RfPair p) {
  typedef RfShape<E, L1> S1;
  typedef typename S1::Raw Raw;
  typedef Rf2Mem<E, L1, L2> Mem;
  static_assert(S1::T == FM_RF2_THREADS && S1::VPC == 1,
                "one first-pass vector per CTA item");
  constexpr int P = S1::P;
  constexpr int NV2 = Mem::NV2;
  static_assert(NV2 >= 1, "second-pass vectors per item");
  extern __shared__ __align__(128) unsigned char fm_smem[];
  unsigned *sitem = reinterpret_cast<unsigned *>(fm_smem);
  unsigned char *base = fm_smem + 16;
  int *sexp = reinterpret_cast<int *>(base + Mem::region);
  const int tid = threadIdx.x;
  const i64 M = p.a.num_cols;
  const unsigned n1 = (unsigned)p.a.A;        // first-pass items per column
  const unsigned n2 = (unsigned)(p.b.A / NV2);  // second-pass items
  const unsigned per = n1 + n2;
  const unsigned total = (unsigned)M * per;
  const unsigned lag = (unsigned)p.lag;
  const unsigned na = (unsigned)M < lag ? (unsigned)M : lag;
  const unsigned nb = (unsigned)M > lag ? (unsigned)M - lag : 0u;
  const FDiv dA1((unsigned)p.a.A), dA2((unsigned)p.b.A),
      dS2((unsigned)p.b.es);
  for (;;) {
    if (tid == 0) sitem[0] = atomicAdd(p.ctr, 1u);
    __syncthreads();
    const unsigned item = sitem[0];
    __syncthreads();  // (sitem is rewritten by the next item)
    if (item >= total) break;
    // decode: column k's first pass, then column k - lag's second pass
    // (the first lag columns' first passes alone, the last lag columns'
    // second passes at the end)
    bool first;
    unsigned col, idx;
    if (item < na * n1) {
      first = true;
      col = item / n1;
      idx = item % n1;
    } else if (item - na * n1 < nb * per) {
      const unsigned i = item - na * n1;
      const unsigned k = lag + i / per, r = i % per;
      first = r < n1;
      col = first ? k : k - lag;
      idx = first ? r : r - n1;
    } else {
      const unsigned i = item - na * n1 - nb * per;
      first = false;
      col = nb + i / n2;
      idx = i % n2;
    }
    if (first) {
      // one contiguous vector: 16-byte cp.async into the padded slot
      Raw *slot = reinterpret_cast<Raw *>(base);
      const Raw *src = (const Raw *)p.a.src + (i64)col * p.a.ld_src +
                       (i64)idx * p.a.stride;
      for (int c = tid; c < L1 / S1::CH; c += FM_RF2_THREADS) {
        const int e = c * S1::CH;
        cp_async<16>(slot + e + (e / S1::ROW) * S1::CH, src + e, true);
      }
      cp_async_commit();
      cp_async_wait<0>();
      __syncthreads();
      Raw d[P];
      {
        typedef typename std::conditional<std::is_same<Raw, float>::value,
                                          float4, double2>::type V;
        const V *sv = reinterpret_cast<const V *>(slot + tid * (P + S1::CH));
#pragma unroll
        for (int c = 0; c < P / S1::CH; ++c)
          *reinterpret_cast<V *>(d + c * S1::CH) = sv[c];
      }
      __syncthreads();
      // the exchange buffer takes the slot's place
      rf_finish<E, L1>(d, p.a, (i64)col * n1 + idx, true,
                       reinterpret_cast<E *>(base), sexp, 0, tid, dA1);
      // this item's stores, then its count (release)
      __syncthreads();
      if (tid == 0) {
        __threadfence();
        atomicAdd(p.ctr + 1 + col, 1u);
      }
    } else {
      // wait for the column's first pass (acquire), bounded
      if (tid == 0) {
        long long polls = 0;
        unsigned done;
        for (;;) {
          asm volatile("ld.acquire.gpu.global.u32 %0, [%1];"
                       : "=r"(done)
                       : "l"(p.ctr + 1 + col)
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
      if (ready)
        rs_batch<E, L2, NV2>(p.b, (i64)col * n2 + idx,
                             reinterpret_cast<E *>(base), sexp, dA2, dS2);
    }
    __syncthreads();  // shared memory is reused by the next item
  }
}

}  // namespace fmk
