// Register-resident FFT programs on vector-major tiles (complex64), for the
// batched kernel: the passes of long transforms (fastmat/Fourier.pyx and the
// convolutions of fastmat/Circulant.pyx:127-133 split four-step as
// N = N1 N2) and short convolutions, whose vector programs are
//
//   RT_FFT:   [zero pad] DIF(L) [twiddle] -> natural order
//   RT_CONV:  [zero pad] DIF(L) spectrum product DIT(L) [twiddle]
//
// for power-of-two L = 64 .. 512 with the planner's radix sequence
// (8, 8, ..., rest).  The generic tile program runs each FFT stage and each
// product as a pass over the shared-memory tile with run-time index
// arithmetic; here a vector's L points sit in the registers of G = L / 8
// threads (8 points each, natural order g + G r after the load), the
// radix-8 / 4 / 2 stages run in registers with compile-time positions and
// exchange through the vector's own storage in the tile, the twiddle and
// spectrum products are applied on the registers, and the results go back
// to the tile in natural order (the storer's digit-reversal table is then
// not used).  The arithmetic is the generic program's, operation for
// operation (same stage order, twiddle tables and products) except for the
// four-step twiddle product, which takes its factor from a two-level table
// (one more rounding; see RtTw).
//
// Positions follow the in-place DIF of the generic program: stage i with
// radix R, Mprev = L / (R_0 ... R_{i-1}) and M = Mprev / R takes, for block K
// and t < M, the points K Mprev + t + M r.  Thread g's butterflies at stage
// i are w = g + G u (u < 8 / R); M divides G, so t = g mod M and the position
// is a per-thread base plus a compile-time offset u G R + M r.
#pragma once

namespace fmk {

// ---- compile-time radix plan: P points per thread, radices (P, ..., rest)
__host__ __device__ constexpr int rc_stages(int L, int P) {
  return L <= P ? 1 : 1 + rc_stages(L / P, P);
}
__host__ __device__ constexpr int rc_radix(int i, int L, int P) {
  return i == 0 ? (L < P ? L : P) : rc_radix(i - 1, L / P, P);
}
// L / (R_0 ... R_{i-1})
__host__ __device__ constexpr int rc_mprev(int i, int L, int P) {
  return i == 0 ? L : rc_mprev(i - 1, L, P) / rc_radix(i - 1, L, P);
}
__host__ __device__ constexpr int rc_log2(int n) {
  return n <= 1 ? 0 : 1 + rc_log2(n / 2);
}

// Step::rprog: program shape (bits 0-1) and flags
enum {
  RT_NONE = 0,
  RT_FFT = 1,
  RT_CONV = 2,
  RT_ZPAD = 4,  // ops[0] is a zero pad
  RT_TW = 8,    // the last op is a twiddle product
  RT_INV = 16,  // RT_FFT: the transform has sign +1
  RT_DIRECT = 32  // RT_CONV: results stored from registers (contiguous
                  // complex64 output, plain store): no storer pass
};
constexpr int kRtP = 8;  // points per thread

template <int L, int I>
__device__ __forceinline__ int rt_base(int g) {
  constexpr int Mprev = rc_mprev(I, L, kRtP);
  constexpr int M = Mprev / rc_radix(I, L, kRtP);
  constexpr int LM = rc_log2(M);
  return (g >> LM) * Mprev + (g & (M - 1));
}
template <int L, int I>
__host__ __device__ constexpr int rt_off(int j) {  // register j = u R + r
  constexpr int R = rc_radix(I, L, kRtP);
  constexpr int M = rc_mprev(I, L, kRtP) / R;
  return (j / R) * (L / kRtP) * R + M * (j % R);
}
// natural index of DIF output position p: the position's digits (radix
// R_0 most significant) read in reverse
template <int L, int I>
__host__ __device__ constexpr int rt_below() {  // bits of the digits > I
  if constexpr (I + 1 >= rc_stages(L, kRtP))
    return 0;
  else
    return rc_log2(rc_radix(I + 1, L, kRtP)) + rt_below<L, I + 1>();
}
template <int L, int I>
__device__ __forceinline__ int rt_nat_from(int p, int sh) {
  constexpr int S = rc_stages(L, kRtP);
  if constexpr (I >= S) {
    return 0;
  } else {
    constexpr int BI = rc_log2(rc_radix(I, L, kRtP));
    constexpr int BELOW = rt_below<L, I>();
    return (((p >> BELOW) & ((1 << BI) - 1)) << sh) |
           rt_nat_from<L, I + 1>(p, sh + BI);
  }
}
template <int L>
__device__ __forceinline__ int rt_nat(int p) {
  return rt_nat_from<L, 0>(p, 0);
}

// barrier of the threads of one vector: the warp, or for L = 512 the pair
// of warps (named barrier 1 + pair index; the CTA has 16 warps, so ids
// 1..8), or the CTA beyond
template <int L>
__device__ __forceinline__ void rt_sync() {
  constexpr int G = L / kRtP;
  if constexpr (G <= 32)
    __syncwarp();
  else if constexpr (G == 64)
    asm volatile("bar.sync %0, 64;" ::"r"(1 + (int)(threadIdx.x >> 6))
                 : "memory");
  else
    __syncthreads();
}

// stage I: DIF (DFT, then twiddles of the outputs) or DIT (twiddles of the
// inputs, then DFT), transform sign SG; register u R + r holds position
// base + u G R + M r before and after
template <int L, int I, bool DIT, int SG>
__device__ __forceinline__ void rt_stage(float2 (&x)[kRtP], int g,
                                         const float2 *__restrict__ tw) {
  constexpr int R = rc_radix(I, L, kRtP);
  constexpr int Mprev = rc_mprev(I, L, kRtP);
  constexpr int M = Mprev / R;
  constexpr int NB = kRtP / R;
  constexpr int TS = L / Mprev;  // table stride of w_Mprev in tw (length L)
  float2 w[R];
  if constexpr (M > 1) {
    const int t = g & (M - 1);
#pragma unroll
    for (int k = 1; k < R; ++k) w[k] = __ldg(tw + t * k * TS);
  }
#pragma unroll
  for (int u = 0; u < NB; ++u) {
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = x[u * R + r];
    if constexpr (DIT && M > 1) {
#pragma unroll
      for (int k = 1; k < R; ++k) v[k] = cmul_lazy<SG>(v[k], w[k]);
    }
    dif_stages<R, R / 2>(v, SG);  // v[i] = output brev(i)
#pragma unroll
    for (int i = 0; i < R; ++i) {
      float2 y = v[i];
      const int k = brev<R>(i);
      if constexpr (!DIT && M > 1) {
        if (k != 0) y = cmul_lazy<SG>(y, w[k]);
      }
      x[u * R + k] = y;
    }
  }
}

// registers laid out for stage IA -> the vector's tile storage ->
// registers laid out for stage IB
template <int L, int IA, int IB>
__device__ __forceinline__ void rt_exchange(float2 (&x)[kRtP], float2 *vec,
                                            int g, bool act) {
  const int ba = rt_base<L, IA>(g), bb = rt_base<L, IB>(g);
  if (act) {
#pragma unroll
    for (int j = 0; j < kRtP; ++j)
      vec[pidx<float2>(ba + rt_off<L, IA>(j))] = x[j];
  }
  rt_sync<L>();
  if (act) {
#pragma unroll
    for (int j = 0; j < kRtP; ++j)
      x[j] = vec[pidx<float2>(bb + rt_off<L, IB>(j))];
  }
  rt_sync<L>();
}

template <int L, int I, int SG>
__device__ __forceinline__ void rt_forward(float2 (&x)[kRtP], float2 *vec,
                                           int g, bool act,
                                           const float2 *tw) {
  rt_stage<L, I, false, SG>(x, g, tw);
  constexpr int S = rc_stages(L, kRtP);
  if constexpr (I + 1 < S) {
    rt_exchange<L, I, I + 1>(x, vec, g, act);
    rt_forward<L, I + 1, SG>(x, vec, g, act, tw);
  }
}
template <int L, int I, int SG>
__device__ __forceinline__ void rt_inverse(float2 (&x)[kRtP], float2 *vec,
                                           int g, bool act,
                                           const float2 *tw) {
  rt_stage<L, I, true, SG>(x, g, tw);
  if constexpr (I > 0) {
    rt_exchange<L, I, I - 1>(x, vec, g, act);
    rt_inverse<L, I - 1, SG>(x, vec, g, act, tw);
  }
}

// twiddle product (OP_TW): e *= w_N^(+-q nat), w = exp(-2 pi i / N), from
// the op's two-level table (ptr3: w^e = T1[e >> s] T0[e & (2^s - 1)],
// s = ceil(log2(N) / 2)), whose two factors stay in the L1 cache where the
// N-entry table of the generic program is read from L2 at random; one more
// rounding than the full table
struct RtTw {
  const float2 *t0, *t1;
  i64 N;
  int s;
  bool neg;
  unsigned q;
  __device__ __forceinline__ float2 apply(float2 e, int nat) const {
    i64 t = (i64)q * nat;
    if (t >= N) t %= N;
    const float2 a = __ldg(t1 + (t >> s));
    const float2 b = __ldg(t0 + (t & ((1 << s) - 1)));
    const float2 wv = make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
    return neg ? cmul(e, wv) : cmulc(e, wv);
  }
};
__device__ __forceinline__ RtTw rt_tw(const Op &op, unsigned vcol) {
  RtTw t;
  const i64 N = op.N;
  int b = 0;
  while ((1LL << b) < N) ++b;
  t.s = (b + 1) / 2;
  t.t0 = (const float2 *)op.ptr3;
  t.t1 = t.t0 + (1 << t.s);
  t.N = N;
  t.neg = op.sign < 0;
  t.q = (op.div == 1 && op.mod == 1)
            ? 0u
            : (vcol / (unsigned)op.div) % (unsigned)op.mod;
  return t;
}

// The whole tile program of a step with rprog != 0 on the B vectors of a
// vector-major tile; leaves the results in natural order.  All threads of
// the CTA take part (barriers for L = 512).
template <int L, int SHAPE, int SG>
__device__ __noinline__ void rt_program_l(const Step &p, float2 *sm,
                                          const VInfo *vi, int tid, int T) {
  constexpr int G = L / kRtP;
  constexpr int S = rc_stages(L, kRtP);
  // (the launch record lives in shared memory like the tile: the fields a
  // loop over points uses are read into registers first, each where it is
  // needed, to keep the registers of the transforms free)
  const int B = p.B, Lp = p.Lp;
  const int nvr = T / G;
  const int f = p.rprog;
  const int o0 = (f & RT_ZPAD) ? 1 : 0;
  const int zfrom = o0 ? p.ops[0].len : L;
  const bool has_tw = (f & RT_TW) != 0;
  for (int b0 = 0; b0 < B; b0 += nvr) {
    const int b = b0 + tid / G, g = tid % G;
    const bool act = b < B;
    float2 *vec = sm + (act ? b : 0) * Lp;
    const unsigned vcol = act ? (unsigned)vi[b].vcol : 0u;
    const float2 *const twf = (const float2 *)p.ops[o0].ptr;
    float2 x[kRtP];
#pragma unroll
    for (int r = 0; r < kRtP; ++r) {
      const int j = g + G * r;
      x[r] = (act && j < zfrom) ? vec[pidx<float2>(j)] : make_float2(0.f, 0.f);
    }
    // (stage 0 writes each thread's exchange values to the positions it has
    // just read, so no barrier is needed before the first exchange)
    if constexpr (SHAPE == RT_CONV) {
      rt_forward<L, 0, -1>(x, vec, g, act, twf);
      {
        const Op &mul = p.ops[o0 + 1];
        const unsigned mdiv = (unsigned)mul.div, mmod = (unsigned)mul.mod;
        const unsigned q =
            (mdiv == 1 && mmod == 1) ? 0u : (vcol / mdiv) % mmod;
        const float2 *P = (const float2 *)mul.ptr + (int)q * (int)mul.stride;
        const bool mconj = mul.sign != 0;
        const int bl = rt_base<L, S - 1>(g);
#pragma unroll
        for (int j = 0; j < kRtP; ++j)
          x[j] = mulv(x[j], __ldg(P + bl + rt_off<L, S - 1>(j)), mconj);
      }
      rt_inverse<L, S - 1, +1>(x, vec, g, act,
                               (const float2 *)p.ops[o0 + 2].ptr);
      // natural order: register r holds point g + G r
      if (has_tw) {
        const RtTw tw = rt_tw(p.ops[p.nops - 1], vcol);
#pragma unroll
        for (int r = 0; r < kRtP; ++r) x[r] = tw.apply(x[r], g + G * r);
      }
      if (f & RT_DIRECT) {
        // consecutive threads hold consecutive points: coalesced stores;
        // post-product, scale and conjugation in the storer's order
        const i64 rb = act ? vi[b].rb_out : -1;
        if (rb >= 0) {
          float2 *dst = (float2 *)p.dst + vi[b].col_dst + rb;
          const int out_len = p.out_len;
          const i64 lim = p.out_rows - rb;
          const float2 *post = (const float2 *)p.post;
          const bool has_scale = p.has_scale != 0, conj_out = p.conj_out != 0;
          const float2 c = scalar_of<float2>(p.scale_re, p.scale_im);
#pragma unroll
          for (int r = 0; r < kRtP; ++r) {
            const int j = g + G * r;
            if (j < out_len && j < lim) {
              float2 val = x[r];
              if (post) val = mulv(val, post[rb + j], false);
              if (has_scale) val = mulv(val, c, false);
              if (conj_out) val = conjv(val);
              dst[j] = val;
            }
          }
        }
      } else if (act) {
#pragma unroll
        for (int r = 0; r < kRtP; ++r) vec[pidx<float2>(g + G * r)] = x[r];
      }
    } else {
      rt_forward<L, 0, SG>(x, vec, g, act, twf);
      const int bl = rt_base<L, S - 1>(g);
      RtTw tw;
      if (has_tw) tw = rt_tw(p.ops[p.nops - 1], vcol);
#pragma unroll
      for (int j = 0; j < kRtP; ++j) {
        const int nat = rt_nat<L>(bl + rt_off<L, S - 1>(j));
        float2 y = x[j];
        if (has_tw) y = tw.apply(y, nat);
        if (act) vec[pidx<float2>(nat)] = y;
      }
    }
    rt_sync<L>();
  }
  __syncthreads();
}

template <int SHAPE, int SG>
__device__ __forceinline__ void rt_program_s(const Step &p, float2 *sm,
                                             const VInfo *vi, int tid,
                                             int T) {
  switch (p.L) {
    case 64: rt_program_l<64, SHAPE, SG>(p, sm, vi, tid, T); break;
    case 128: rt_program_l<128, SHAPE, SG>(p, sm, vi, tid, T); break;
    case 256: rt_program_l<256, SHAPE, SG>(p, sm, vi, tid, T); break;
    default: rt_program_l<512, SHAPE, SG>(p, sm, vi, tid, T); break;
  }
}

__device__ __forceinline__ void rt_program(const Step &p, float2 *sm,
                                           const VInfo *vi, int tid, int T) {
  if ((p.rprog & 3) == RT_CONV)
    rt_program_s<RT_CONV, -1>(p, sm, vi, tid, T);
  else if (p.rprog & RT_INV)
    rt_program_s<RT_FFT, +1>(p, sm, vi, tid, T);
  else
    rt_program_s<RT_FFT, -1>(p, sm, vi, tid, T);
}

}  // namespace fmk
