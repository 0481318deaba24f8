// The vector-program kernel: one fused launch of a lowered operator stage.
//
// Data model.  Every column of the operand is viewed as a 3-D array
// (A, n, Cc): element j of vector (a, c) sits at row r = (a * n + j) * Cc + c.
// A whole column is the view (1, n, 1); mode k of a Kronecker product
// (fastmat/Kron.pyx:267-341) is the view (prod of the sizes before k, n_k,
// prod of the sizes after k); the passes of a four-step FFT are the views
// (1, N1, N2) and (N1, N2, 1).  A launch loads a tile of B vectors through
// the input view into shared memory, runs a short straight-line program on
// them (Stockham FFT passes, pointwise multiplies, Walsh-Hadamard passes,
// gathers, dense products, four-step twiddles) and stores the tile through
// the output view, so a whole chain such as Partial * Circulant * Diag reads
// and writes HBM once.
#pragma once

#include <cuda.h>

#include <type_traits>

#include "fm_types.cuh"

namespace fmk {

enum OpKind {
  OP_FFT = 1,     // Stockham FFT of size len, sign -1 (forward) / +1
  OP_MUL = 2,     // v[j] *= P[q * stride + j] (conj if sign), j < len
  OP_ZPAD = 3,    // v[j] = 0 for len <= j < len2
  OP_GATHER = 4,  // v'[i] = map[i] < 0 ? 0 : v[map[i]], i < len
  OP_FWHT = 5,    // Sylvester-ordered Walsh-Hadamard transform of size len
  OP_DENSE = 6,   // v'[i] = sum_j M[i + j * len] v[j], i < len, j < len2
  OP_SCALE = 7,   // v[j] *= (sre + i sim), j < len
  OP_CONJ = 8,    // v[j] = conj(v[j]), j < len
  OP_TW = 9,      // v[j] *= exp(sign 2 pi i ((q * nat(j)) mod N) / N),
                  // nat = perm table (ptr2) or identity, j < len
  OP_DIF = 10,    // in-place FFT, natural order in, digit-reversed out
  OP_DIT = 11     // in-place FFT, digit-reversed in, natural order out
};

#define FM_MAX_OPS 14

struct Op {
  int kind;
  int len;
  int len2;
  int sign;
  int nrad;
  unsigned char rad[16];  // FFT radices / FWHT bit-group widths
  const void *ptr;        // twiddles, vector, map, matrix
  const int *ptr2;        // TW: storage position -> natural index
  const void *ptr3;       // TW (complex64): two-level table, see
                          // twiddle2 in the planner
  i64 div, mod, stride;   // q = (v / div) % mod for MUL / TW
  i64 N;
  double sre, sim;
};

struct View {
  i64 A, n, Cc;
};

struct Step {
  // TMA descriptors of the input / output views (element-major tiles only;
  // encoded on the host per call because they hold the buffer address)
  alignas(64) CUtensorMap tm_in;
  alignas(64) CUtensorMap tm_out;
  const void *src;
  void *dst;
  i64 ld_src, ld_dst;
  int src_type, dst_type;
  View vin, vout;
  i64 in_rows;   // loader: rows >= in_rows read as zero (map: map length)
  i64 out_rows;  // storer: rows >= out_rows are not written
  const i64 *map_in;
  const i64 *map_out;
  int out_mode;  // 0 plain, 1 gather (whole column), 2 scatter (inverse map)
  int n_out;     // gather mode: rows written per column
  const void *pre;
  const void *post;
  const int *out_pos;  // storer: natural element j sits at position out_pos[j]
  int *err;            // device status word (bounded waits that gave up)
  int conj_in, conj_out, accumulate, has_scale;
  double scale_re, scale_im;
  int L, Lp, B;
  int nbuf;      // tile buffers of the copy ring (2..4)
  int tma_in, tma_out;  // element-major tiles moved by TMA boxes
  int box_rows;  // rows per TMA box (<= 256)
  int elem_k;    // TMA elements per E (2 for 16-byte E)
  int in_len, out_len;
  i64 V;         // vectors per column
  i64 num_cols;
  long long wait_limit;  // polls of a bounded copy wait before it gives up
  int nops;
  int rprog;  // register tile program of the batched kernel (RT_*)
  Op ops[FM_MAX_OPS];
};

// elements each thread holds in registers per pass
// (a launch uses at most FM_MAX_THREADS threads, so a tile holds at most
// FM_MAX_THREADS * Ept elements)
#define FM_MAX_THREADS 512
template <class E> struct Ept {
  static constexpr int v = sizeof(E) == 4 ? 16 : 8;
};

// ------------------------------------------------------------ small DFTs
// y_k = sum_r x_r exp(sign * 2 pi i r k / R), in place.
template <class C> __device__ __forceinline__ C rot90(C a, int sign) {
  // a * (i * sign)
  C r;
  r.x = smul(-sign, a.y);
  r.y = smul(sign, a.x);
  return r;
}

template <class C> __device__ __forceinline__ void dft2(C *v) {
  C a = v[0], b = v[1];
  v[0] = a + b;
  v[1] = a - b;
}

template <class C> __device__ __forceinline__ void dft4(C *v, int sign) {
  C s0 = v[0] + v[2], d0 = v[0] - v[2];
  C s1 = v[1] + v[3], d1 = rot90(v[1] - v[3], sign);
  v[0] = s0 + s1;
  v[2] = s0 - s1;
  v[1] = d0 + d1;
  v[3] = d0 - d1;
}

template <class C> __device__ __forceinline__ void dft8(C *v, int sign) {
  typedef typename Tr<C>::R R;
  const R h = (R)0.7071067811865476;
  C a[4], b[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    a[k] = v[k] + v[k + 4];
    b[k] = v[k] - v[k + 4];
  }
  // b_k *= exp(sign 2 pi i k / 8)
  C t;
  t.x = h * (b[1].x - smul(sign, b[1].y));
  t.y = h * (b[1].y + smul(sign, b[1].x));
  b[1] = t;
  b[2] = rot90(b[2], sign);
  t.x = h * (-b[3].x - smul(sign, b[3].y));
  t.y = h * (-b[3].y + smul(sign, b[3].x));
  b[3] = t;
  dft4(a, sign);
  dft4(b, sign);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    v[2 * k] = a[k];
    v[2 * k + 1] = b[k];
  }
}

template <class C> __device__ __forceinline__ void dft16(C *v, int sign) {
  typedef typename Tr<C>::R R;
  // cos / sin of k pi / 8, k = 0..7
  const R cs[8] = {(R)1.0, (R)0.9238795325112867, (R)0.7071067811865476,
                   (R)0.3826834323650898, (R)0.0, (R)-0.3826834323650898,
                   (R)-0.7071067811865476, (R)-0.9238795325112867};
  const R sn[8] = {(R)0.0, (R)0.3826834323650898, (R)0.7071067811865476,
                   (R)0.9238795325112867, (R)1.0, (R)0.9238795325112867,
                   (R)0.7071067811865476, (R)0.3826834323650898};
  C a[8], b[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    a[k] = v[k] + v[k + 8];
    C d = v[k] - v[k + 8];
    const R c = cs[k], s = smul(sign, sn[k]);
    b[k].x = d.x * c - d.y * s;
    b[k].y = d.x * s + d.y * c;
  }
  dft8(a, sign);
  dft8(b, sign);
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    v[2 * k] = a[k];
    v[2 * k + 1] = b[k];
  }
}

template <class C> __device__ __forceinline__ void dft3(C *v, int sign) {
  typedef typename Tr<C>::R R;
  const R c = (R)-0.5, s0 = (R)0.8660254037844386;
  const R s = sign < 0 ? -s0 : s0;
  C t = v[1] + v[2], d = v[1] - v[2];
  C y0 = v[0] + t;
  C m;
  m.x = v[0].x + c * t.x;
  m.y = v[0].y + c * t.y;
  C r;
  r.x = -(s * d.y);
  r.y = s * d.x;
  v[0] = y0;
  v[1] = m + r;
  v[2] = m - r;
}

// odd prime radices via symmetric pairs t_m = x_m + x_{R-m},
// d_m = x_m - x_{R-m}:  y_k = x0 + sum_m t_m cos(2 pi m k / R)
//                             + i sign sum_m d_m sin(2 pi m k / R)
template <class C>
__device__ __forceinline__ C pair_out(C a, C b, int sign, bool plus) {
  // a + i*sign*b  (plus) or  a - i*sign*b
  C r;
  const int sb = plus ? sign : -sign;
  r.x = a.x - smul(sb, b.y);
  r.y = a.y + smul(sb, b.x);
  return r;
}

template <class C> __device__ __forceinline__ void dft5(C *v, int sign) {
  typedef typename Tr<C>::R R;
  const R c1 = (R)0.30901699437494745, c2 = (R)-0.8090169943749473;
  const R s1 = (R)0.9510565162951535, s2 = (R)0.5877852522924732;
  const C x0 = v[0];
  const C t1 = v[1] + v[4], t2 = v[2] + v[3];
  const C d1 = v[1] - v[4], d2 = v[2] - v[3];
  C a1, a2, b1, b2;
  a1.x = x0.x + c1 * t1.x + c2 * t2.x;
  a1.y = x0.y + c1 * t1.y + c2 * t2.y;
  a2.x = x0.x + c2 * t1.x + c1 * t2.x;
  a2.y = x0.y + c2 * t1.y + c1 * t2.y;
  b1.x = s1 * d1.x + s2 * d2.x;
  b1.y = s1 * d1.y + s2 * d2.y;
  b2.x = s2 * d1.x - s1 * d2.x;
  b2.y = s2 * d1.y - s1 * d2.y;
  v[0] = x0 + t1 + t2;
  v[1] = pair_out(a1, b1, sign, true);
  v[4] = pair_out(a1, b1, sign, false);
  v[2] = pair_out(a2, b2, sign, true);
  v[3] = pair_out(a2, b2, sign, false);
}

template <class C> __device__ __forceinline__ void dft7(C *v, int sign) {
  typedef typename Tr<C>::R R;
  const R c1 = (R)0.6234898018587336, c2 = (R)-0.22252093395631434,
          c3 = (R)-0.900968867902419;
  const R s1 = (R)0.7818314824680298, s2 = (R)0.9749279121818236,
          s3 = (R)0.43388373911755823;
  const C x0 = v[0];
  const C t1 = v[1] + v[6], t2 = v[2] + v[5], t3 = v[3] + v[4];
  const C d1 = v[1] - v[6], d2 = v[2] - v[5], d3 = v[3] - v[4];
  C a, b;
  v[0] = x0 + t1 + t2 + t3;
  a.x = x0.x + c1 * t1.x + c2 * t2.x + c3 * t3.x;
  a.y = x0.y + c1 * t1.y + c2 * t2.y + c3 * t3.y;
  b.x = s1 * d1.x + s2 * d2.x + s3 * d3.x;
  b.y = s1 * d1.y + s2 * d2.y + s3 * d3.y;
  v[1] = pair_out(a, b, sign, true);
  v[6] = pair_out(a, b, sign, false);
  a.x = x0.x + c2 * t1.x + c3 * t2.x + c1 * t3.x;
  a.y = x0.y + c2 * t1.y + c3 * t2.y + c1 * t3.y;
  b.x = s2 * d1.x - s3 * d2.x - s1 * d3.x;
  b.y = s2 * d1.y - s3 * d2.y - s1 * d3.y;
  v[2] = pair_out(a, b, sign, true);
  v[5] = pair_out(a, b, sign, false);
  a.x = x0.x + c3 * t1.x + c1 * t2.x + c2 * t3.x;
  a.y = x0.y + c3 * t1.y + c1 * t2.y + c2 * t3.y;
  b.x = s3 * d1.x - s1 * d2.x + s2 * d3.x;
  b.y = s3 * d1.y - s1 * d2.y + s2 * d3.y;
  v[3] = pair_out(a, b, sign, true);
  v[4] = pair_out(a, b, sign, false);
}

template <int R, class C> __device__ __forceinline__ void dft(C *v, int sign) {
  if constexpr (R == 2) dft2(v);
  else if constexpr (R == 3) dft3(v, sign);
  else if constexpr (R == 4) dft4(v, sign);
  else if constexpr (R == 5) dft5(v, sign);
  else if constexpr (R == 7) dft7(v, sign);
  else if constexpr (R == 8) dft8(v, sign);
  else if constexpr (R == 16) dft16(v, sign);
}

// ------------------------------------------------------------ in-place pow2 DFT
// Decimation-in-frequency radix-2 network over R registers, in place: after
// it, v[i] holds output bitrev(i).  Twiddles are compile-time constants
// exp(sign 2 pi i k / M), taken from cos/sin of multiples of pi / 8.
__host__ __device__ constexpr double kCos16(int i) {
  // cos(2 pi i / 16), i = 0..15
  return i == 0 ? 1.0 : i == 1 ? 0.9238795325112867 : i == 2 ? 0.7071067811865476
       : i == 3 ? 0.3826834323650898 : i == 4 ? 0.0 : i == 5 ? -0.3826834323650898
       : i == 6 ? -0.7071067811865476 : i == 7 ? -0.9238795325112867
       : i == 8 ? -1.0 : i == 9 ? -0.9238795325112867 : i == 10 ? -0.7071067811865476
       : i == 11 ? -0.3826834323650898 : i == 12 ? 0.0 : i == 13 ? 0.3826834323650898
       : i == 14 ? 0.7071067811865476 : 0.9238795325112867;
}
__host__ __device__ constexpr double kSin16(int i) { return kCos16((i + 12) & 15); }

template <int M, int K, class C>
__device__ __forceinline__ C twc(C x, int sign) {
  typedef typename Tr<C>::R R;
  constexpr int idx = (16 / M) * K;  // angle 2 pi idx / 16
  if constexpr (idx == 0) {
    return x;
  } else if constexpr (idx == 4) {
    return rot90(x, sign);  // * (i sign)
  } else {
    const R c = (R)kCos16(idx), sp = (R)kSin16(idx);
    const R sn = sign < 0 ? -sp : sp;
    C r;
    r.x = x.x * c - x.y * sn;
    r.y = x.x * sn + x.y * c;
    return r;
  }
}

template <int R, int H, int K, class C>
__device__ __forceinline__ void dif_stage_k(C *v, int sign) {
  if constexpr (K < H) {
#pragma unroll
    for (int blk = 0; blk < R; blk += 2 * H) {
      const C a = v[blk + K], b = v[blk + K + H];
      v[blk + K] = a + b;
      v[blk + K + H] = twc<2 * H, K>(a - b, sign);
    }
    dif_stage_k<R, H, K + 1>(v, sign);
  }
}

template <int R, int H, class C>
__device__ __forceinline__ void dif_stages(C *v, int sign) {
  if constexpr (H >= 1) {
    dif_stage_k<R, H, 0>(v, sign);
    dif_stages<R, H / 2>(v, sign);
  }
}

template <int R> __host__ __device__ constexpr int brev(int i) {
  int r = 0;
  for (int b = 1; b < R; b <<= 1) r = (r << 1) | ((i & b) ? 1 : 0);
  return r;
}

// ------------------------------------------------------------ index helpers
// Unsigned division by a runtime divisor 1 <= d < 2^31 for dividends below
// 2^31 with one multiply-high: q = (umulhi(n, m) + n) >> s,
// s = ceil(log2 d), m = 2^32 (2^s - d) / d + 1 (round-up multiplier).
// Powers of two (the common case: built per FFT stage of every tile) skip
// the 64-bit division: m = 1, and umulhi(n, 1) = 0 leaves n >> s.
struct FDiv {
  unsigned d, m, s;
  __device__ __forceinline__ explicit FDiv(unsigned d_) : d(d_) {
    s = d > 1 ? 32 - __clz(d - 1) : 0;  // ceil(log2 d)
    m = (d & (d - 1)) == 0
            ? 1u
            : (unsigned)(((1ull << 32) * ((1ull << s) - d)) / d + 1);
  }
  __device__ __forceinline__ unsigned div(unsigned n) const {
    return (__umulhi(n, m) + n) >> s;
  }
};

// Walks the flat index f = tid, tid + T, ... of a tile of vectors of length
// len, keeping (b, j) = (f / len, f % len) without dividing per step.
struct Walk {
  int b, j, tb, tj, len;
  __device__ __forceinline__ Walk(int f0, int len_, int T) : len(len_) {
    if (len > 0 && (len & (len - 1)) == 0) {  // shifts for powers of two
      const int lg = __ffs(len) - 1;
      b = f0 >> lg;
      j = f0 & (len - 1);
      tb = T >> lg;
      tj = T & (len - 1);
    } else {
      b = f0 / len;
      j = f0 - b * len;
      tb = T / len;
      tj = T - tb * len;
    }
  }
  __device__ __forceinline__ void next() {
    j += tj;
    b += tb;
    if (j >= len) {
      j -= len;
      ++b;
    }
  }
};

// Per-vector addressing of a tile, computed once per launch: column offsets
// of source and destination, the row of element 0 in the input and output
// views (-1: vector beyond the operand) and the vector's index within its
// column.
struct VInfo {
  i64 col_src, rb_in, col_dst, rb_out, vcol;
};

// ------------------------------------------------------------ layouts
// LAY 0: vector-major tile, vector b at b * Lp with one pad element per 128
//        bytes (pidx), threads walk the elements of a vector.
// LAY 1: element-major tile, element j of vector b at j * B + b (dense),
//        threads walk the vectors first; filled and drained by TMA boxes.
// LAY 2: vector-major tile without padding (vector b at b * L): contiguous
//        vectors then move as one bulk copy per run of vectors, at the cost
//        of bank conflicts for some strided FFT stages (the autotuner picks
//        between LAY 0 and LAY 2).
template <class E, int LAY>
__device__ __forceinline__ int jx(int j, int B) {
  if constexpr (LAY == 1) return j * B;
  else if constexpr (LAY == 2) return j;
  else return pidx<E>(j);
}
// position of element j inside a vector-major vector (LAY 0 or 2)
template <class E, int LAY>
__device__ __forceinline__ int vx(int j) {
  if constexpr (LAY == 2) return j;
  else return pidx<E>(j);
}
template <class E, int LAY>
__device__ __forceinline__ E *vbase(E *sm, int b, int Lp) {
  if constexpr (LAY == 1) return sm + b;
  else return sm + b * Lp;
}

}  // namespace fmk
#include "fm_tc.cuh"
#include "fm_tcdense.cuh"
namespace fmk {

// ------------------------------------------------------------ FFT stages
// In-place mixed-radix stages.  With L = R_1 ... R_S and M_0 = L,
// M_s = M_{s-1} / R_s, stage s of the DIF transform takes, for every block
// K (offset K M_{s-1}) and t < M_s, the R_s elements at K M_{s-1} + t + M_s n,
// applies the radix-R_s DFT over n, multiplies output k by
// w_{M_{s-1}}^{t k} and writes it back to K M_{s-1} + t + M_s k.  After all
// stages position ((k_1 R_2 + k_2) R_3 + ...) holds output
// k_1 + R_1 (k_2 + R_2 (...)).  The DIT transform runs the stages in reverse
// (twiddle first, then the DFT over k), taking that digit-reversed order to
// natural order; with opposite signs the two are inverse up to the factor L.
// Each work item reads and writes the same R positions, so a stage needs one
// barrier and holds only R values per thread.
// Barrier of the threads that run one tile program together: the whole CTA,
// or a single warp when the tile's vectors are divided among warps (T == 32;
// a 32-thread CTA is one warp too).
__device__ __forceinline__ void group_sync(int T) {
  if (T <= 32)
    __syncwarp();
  else
    __syncthreads();
}

// A pointwise product applied by the last stage of a forward transform as
// it stores its outputs (the spectrum product of a circular convolution,
// kernel class 5): output j is multiplied by p[j] (conj: by conj(p[j])).
struct Post {
  const void *p;
  int conj;
};

// a * w (SG < 0) or a * conj(w) (SG > 0) for a butterfly value a in the
// butterfly's computing type and a twiddle w (unnormalised products and
// sums for double-float; the plain complex product otherwise)
template <int SG, class LC, class C>
__device__ __forceinline__ LC cmul_lazy(LC a, C w) {
  if constexpr (std::is_same<LC, C>::value) {
    return SG < 0 ? cmul(a, w) : cmulc(a, w);
  } else {
    const LC b = to_lazy(w);
    LC r;
    if constexpr (SG < 0) {
      r.x = a.x * b.x - a.y * b.y;
      r.y = a.x * b.y + a.y * b.x;
    } else {
      r.x = a.x * b.x + a.y * b.y;
      r.y = a.y * b.x - a.x * b.y;
    }
    return r;
  }
}

// UT: every twiddle of the stage is 1 (M = 1: the last DIF stage and the
// first DIT stage, where t = 0 for every butterfly), so the products are
// left out
template <int R, bool DIT, int LAY, int SG, bool UT, class C>
__device__ __forceinline__ void fft_stage_body(C *sm, int Lp, int B, int Lf,
                                               int Mprev,
                                               const C *__restrict__ tw,
                                               int tid, int T, Post post) {
  constexpr int sign = SG;
  const int M = Mprev / R;
  const int nw = Lf / R;
  const int total = B * nw;
  const FDiv dnw((unsigned)nw), dM((unsigned)M);
  const int lgB = __ffs(B) - 1;
  const int tscale = (Mprev & (Mprev - 1)) == 0 ? Lf >> (__ffs(Mprev) - 1)
                                                 : Lf / Mprev;
  for (int g = tid; g < total; g += T) {
    int b, w;
    if constexpr (LAY == 1) {
      b = g & (B - 1);
      w = g >> lgB;
    } else {
      b = (int)dnw.div((unsigned)g);
      w = g - b * nw;
    }
    const int K = (int)dM.div((unsigned)w), t = w - K * M;
    C *vec = vbase<C, LAY>(sm, b, Lp);
    const int base = K * Mprev + t;
    // twiddle w^(t k) is tw[k * tstep]; for t = 0 it is tw[0] = 1 exactly,
    // so the products run unconditionally (straight-line code)
    const C *twt = tw;
    const int tstep = t * tscale;
    C v[R];
#pragma unroll
    for (int n = 0; n < R; ++n) v[n] = vec[jx<C, LAY>(base + M * n, B)];
    if constexpr ((R & (R - 1)) == 0) {
      // twiddles and butterflies run in the unnormalised form of
      // double-float (one renormalisation per output element)
      typedef typename Lazy<C>::type LC;
      LC u[R];
#pragma unroll
      for (int n = 0; n < R; ++n) u[n] = to_lazy(v[n]);
      if constexpr (DIT && !UT) {
#pragma unroll
        for (int k = 1; k < R; ++k)
          u[k] = cmul_lazy<sign>(u[k], twt[k * tstep]);
      }
      dif_stages<R, R / 2>(u, sign);  // u[i] = output brev(i)
#pragma unroll
      for (int i = 0; i < R; ++i) {
        LC y = u[i];
        if constexpr (!DIT && !UT) {
          if (brev<R>(i) != 0)  // folded by the unrolled loop
            y = cmul_lazy<sign>(y, twt[brev<R>(i) * tstep]);
        }
        if constexpr (!DIT && UT) {
          if (post.p) {
            const C pw = ((const C *)post.p)[base + M * brev<R>(i)];
            y = post.conj ? cmul_lazy<+1>(y, pw) : cmul_lazy<-1>(y, pw);
          }
        }
        vec[jx<C, LAY>(base + M * brev<R>(i), B)] = from_lazy(y);
      }
    } else {
      if constexpr (DIT) {
#pragma unroll
        for (int k = 1; k < R; ++k) {
          const C w = twt[k * tstep];
          v[k] = sign < 0 ? cmul(v[k], w) : cmulc(v[k], w);
        }
      }
      dft<R>(v, sign);
#pragma unroll
      for (int k = 0; k < R; ++k) {
        C y = v[k];
        if constexpr (!DIT) {
          if (k != 0) {
            const C w = twt[k * tstep];
            y = sign < 0 ? cmul(y, w) : cmulc(y, w);
          }
        }
        vec[jx<C, LAY>(base + M * k, B)] = y;
      }
    }
  }
}

template <int R, bool DIT, int LAY, int SG, class C>
__device__ __forceinline__ void fft_stage(C *sm, int Lp, int B, int Lf,
                                          int Mprev,
                                          const C *__restrict__ tw, int tid,
                                          int T, Post post) {
  if constexpr ((R & (R - 1)) == 0) {
    if (Mprev == R)
      fft_stage_body<R, DIT, LAY, SG, true>(sm, Lp, B, Lf, Mprev, tw, tid, T,
                                            post);
    else
      fft_stage_body<R, DIT, LAY, SG, false>(sm, Lp, B, Lf, Mprev, tw, tid,
                                             T, post);
  } else {
    fft_stage_body<R, DIT, LAY, SG, false>(sm, Lp, B, Lf, Mprev, tw, tid, T,
                                           post);
  }
  group_sync(T);
}

// Register budget per element type: the single-precision kernels run two
// 512-thread CTAs per SM (64 registers per thread) to hide more latency,
// which leaves no room for radix-16 butterflies; the wider types keep one
// CTA per SM and radix 16 (double-float tops out at radix 8).  The planner
// picks radices with the same rule (max_radix_for in fm_launch.cuh).
template <class E, int CLS> struct MinBlocks {
  static constexpr int v = ((std::is_same<E, float>::value ||
                             std::is_same<E, float2>::value) &&
                            CLS != 4 && CLS != 6)
                               ? 2
                               : 1;
};
template <class C> struct Radix16 {
  static constexpr bool v =
      !Emu<C>::v && !std::is_same<C, float2>::value &&
      !std::is_same<C, float>::value;
};

template <bool DIT, int CLS, int LAY, int SG, class C>
__device__ __forceinline__ void fft_stage_s(int R, C *sm, int Lp, int B,
                                            int Lf, int Mprev, const C *tw,
                                            int tid, int T, Post post) {
  switch (R) {
    case 2: fft_stage<2, DIT, LAY, SG>(sm, Lp, B, Lf, Mprev, tw, tid, T, post); break;
    case 4: fft_stage<4, DIT, LAY, SG>(sm, Lp, B, Lf, Mprev, tw, tid, T, post); break;
    case 8: fft_stage<8, DIT, LAY, SG>(sm, Lp, B, Lf, Mprev, tw, tid, T, post); break;
    case 16:
      // double-float vectors of 16 elements do not fit the register budget
      if constexpr (Radix16<C>::v)
        fft_stage<16, DIT, LAY, SG>(sm, Lp, B, Lf, Mprev, tw, tid, T, post);
      break;
    case 3:
      if constexpr (CLS != 1 && CLS != 5)
        fft_stage<3, DIT, LAY, SG>(sm, Lp, B, Lf, Mprev, tw, tid, T, post);
      break;
    case 5:
      if constexpr (CLS != 1 && CLS != 5)
        fft_stage<5, DIT, LAY, SG>(sm, Lp, B, Lf, Mprev, tw, tid, T, post);
      break;
    case 7:
      if constexpr (CLS != 1 && CLS != 5)
        fft_stage<7, DIT, LAY, SG>(sm, Lp, B, Lf, Mprev, tw, tid, T, post);
      break;
    default: break;
  }
}

// the transform sign is a template parameter of the stages, so rotations
// by +-i and conjugated twiddles cost no run-time selects
template <bool DIT, int CLS, int LAY, class C>
__device__ __forceinline__ void fft_stage_r(int R, C *sm, int Lp, int B,
                                            int Lf, int Mprev, int sign,
                                            const C *tw, int tid, int T,
                                            Post post) {
  if (sign < 0)
    fft_stage_s<DIT, CLS, LAY, -1>(R, sm, Lp, B, Lf, Mprev, tw, tid, T, post);
  else
    fft_stage_s<DIT, CLS, LAY, +1>(R, sm, Lp, B, Lf, Mprev, tw, tid, T, post);
}

// post: a pointwise product for the last DIF stage (class 5 only; its radix
// is a power of two), otherwise none
template <class C, int CLS, int LAY>
__device__ void run_fft(const Op &op, C *sm, int Lp, int B, int tid, int T,
                        Post post) {
  const C *tw = (const C *)op.ptr;
  if (op.kind == OP_DIF) {
    int Mprev = op.len;
    for (int p = 0; p < op.nrad; ++p) {
      const int R = op.rad[p];
      Post pp = Post{nullptr, 0};
      if constexpr (CLS == 5)
        if (p + 1 == op.nrad) pp = post;
      fft_stage_r<false, CLS, LAY>(R, sm, Lp, B, op.len, Mprev, op.sign, tw,
                                   tid, T, pp);
      Mprev /= R;
    }
  } else {
    int Mprev = 1;
    for (int p = op.nrad - 1; p >= 0; --p) {
      Mprev *= op.rad[p];
      fft_stage_r<true, CLS, LAY>(op.rad[p], sm, Lp, B, op.len, Mprev,
                                  op.sign, tw, tid, T, Post{nullptr, 0});
    }
  }
}

// ------------------------------------------------------------ FWHT pass
// In-place butterflies over the bit group [s, s + K) of every element index.
template <int K, int LAY, class E>
__device__ __forceinline__ void fwht_pass(E *sm, int Lp, int B, int Lf, int s,
                                          int tid, int T) {
  constexpr int R = 1 << K;
  constexpr int MB = (Ept<E>::v + R - 1) / R;
  const int nb = Lf >> K;
  const int lg = __ffs(nb) - 1;
  const int lgB = __ffs(B) - 1;
  const int total = B * nb;
  const int lomask = (1 << s) - 1;
#pragma unroll
  for (int i = 0; i < MB; ++i) {
    const int g = tid + i * T;
    if (g < total) {
      int b, q;
      if constexpr (LAY == 1) {
        b = g & (B - 1);
        q = g >> lgB;
      } else {
        b = g >> lg;
        q = g & (nb - 1);
      }
      const int base = ((q >> s) << (s + K)) | (q & lomask);
      E *vec = vbase<E, LAY>(sm, b, Lp);
      // unnormalised double-float inside the group (see dfu)
      typedef typename Lazy<E>::type LE;
      LE v[R];
#pragma unroll
      for (int r = 0; r < R; ++r)
        v[r] = to_lazy(vec[jx<E, LAY>(base + (r << s), B)]);
#pragma unroll
      for (int h = 1; h < R; h <<= 1) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
          if ((r & h) == 0) {
            const LE a = v[r], c = v[r + h];
            v[r] = addv(a, c);
            v[r + h] = subv(a, c);
          }
        }
      }
#pragma unroll
      for (int r = 0; r < R; ++r)
        vec[jx<E, LAY>(base + (r << s), B)] = from_lazy(v[r]);
    }
  }
  group_sync(T);
}

template <class E, int LAY>
__device__ void run_fwht(const Op &op, E *sm, int Lp, int B, int tid, int T,
                         TcState *tc = nullptr) {
  int s = 0;
  for (int p = 0; p < op.nrad; ++p) {
    const int K = op.rad[p];
    if constexpr (std::is_same<E, float>::value) {
      // 16-point groups on the tensor cores (op.sign marks the form)
      if (tc && op.sign && K == 4 && !tc->failed) {
        run_h16tc<LAY>(sm, Lp, B, op.len, s, *tc, tid, T);
        s += K;
        continue;
      }
    }
    switch (K) {
      case 1: fwht_pass<1, LAY>(sm, Lp, B, op.len, s, tid, T); break;
      case 2: fwht_pass<2, LAY>(sm, Lp, B, op.len, s, tid, T); break;
      case 3: fwht_pass<3, LAY>(sm, Lp, B, op.len, s, tid, T); break;
      default: fwht_pass<4, LAY>(sm, Lp, B, op.len, s, tid, T); break;
    }
    s += K;
  }
}

// ------------------------------------------------------------ other ops
// (gathers and dense products run on vector-major tiles only)
template <class E, int LAY>
__device__ void run_gather(const Op &op, E *sm, int Lp, int B, int tid,
                           int T) {
  constexpr int MB = Ept<E>::v;
  const i64 *map = (const i64 *)op.ptr;
  const int total = B * op.len;
  E v[MB];
  {
    Walk w(tid, op.len, T);
#pragma unroll
    for (int i = 0; i < MB; ++i, w.next()) {
      if (tid + i * T < total) {
        const i64 src = map[w.j];
        v[i] = src < 0 ? zero<E>() : sm[w.b * Lp + vx<E, LAY>((int)src)];
      }
    }
  }
  group_sync(T);
  {
    Walk w(tid, op.len, T);
#pragma unroll
    for (int i = 0; i < MB; ++i, w.next())
      if (tid + i * T < total) sm[w.b * Lp + vx<E, LAY>(w.j)] = v[i];
  }
  group_sync(T);
}

template <class E, int LAY>
__device__ void run_dense(const Op &op, E *sm, int Lp, int B, int tid,
                          int T) {
  constexpr int MB = Ept<E>::v;
  const E *M = (const E *)op.ptr;
  const int rows = op.len, cols = op.len2;
  const int total = B * rows;
  E v[MB];
  {
    Walk w(tid, rows, T);
#pragma unroll
    for (int i = 0; i < MB; ++i, w.next()) {
      if (tid + i * T < total) {
        const E *vec = sm + w.b * Lp;
        E acc = zero<E>();
        for (int j = 0; j < cols; ++j)
          acc = addv(acc, mulv(M[w.j + (i64)j * rows], vec[vx<E, LAY>(j)],
                               false));
        v[i] = acc;
      }
    }
  }
  group_sync(T);
  {
    Walk w(tid, rows, T);
#pragma unroll
    for (int i = 0; i < MB; ++i, w.next())
      if (tid + i * T < total) sm[w.b * Lp + vx<E, LAY>(w.j)] = v[i];
  }
  group_sync(T);
}

// one pass over the B x len elements of a tile applying f(element, b, j)
template <class E, int LAY, class F>
__device__ __forceinline__ void ew_loop(E *sm, int Lp, int B, int len,
                                        int tid, int T, F f) {
  const int total = B * len;
  if constexpr (LAY == 1) {
    const int lgB = __ffs(B) - 1;
    for (int g = tid; g < total; g += T) {
      const int b = g & (B - 1), j = g >> lgB;
      f(sm[j * B + b], b, j);
    }
  } else {
    Walk w(tid, len, T);
    for (int g = tid; g < total; g += T, w.next())
      f(sm[w.b * Lp + vx<E, LAY>(w.j)], w.b, w.j);
  }
}

template <class E, int LAY>
__device__ void run_elementwise(const Op &op, E *sm, int Lp, int B,
                                const VInfo *vi, i64 *sq, int tid, int T) {
  const int kind = op.kind;
  if (kind == OP_MUL || kind == OP_TW) {
    // vcol < 2^31: 32-bit arithmetic, nothing to do for the common
    // div = mod = 1 (sq = 0)
    if (op.div == 1 && op.mod == 1) {
      for (int b = tid; b < B; b += T) sq[b] = 0;
    } else {
      for (int b = tid; b < B; b += T)
        sq[b] = ((unsigned)vi[b].vcol / (unsigned)op.div) % (unsigned)op.mod;
    }
    group_sync(T);
  }
  const int len = op.len;
  switch (kind) {
    case OP_MUL: {
      // the table holds mod * stride < 2^31 entries: 32-bit indices
      const E *P = (const E *)op.ptr;
      const int stride = op.stride;
      if (op.sign)
        ew_loop<E, LAY>(sm, Lp, B, len, tid, T, [&](E &e, int b, int j) {
          e = mulv(e, P[(int)sq[b] * stride + j], true);
        });
      else
        ew_loop<E, LAY>(sm, Lp, B, len, tid, T, [&](E &e, int b, int j) {
          e = mulv(e, P[(int)sq[b] * stride + j], false);
        });
      break;
    }
    case OP_SCALE: {
      const E c = scalar_of<E>(op.sre, op.sim);
      ew_loop<E, LAY>(sm, Lp, B, len, tid, T,
                      [&](E &e, int, int) { e = mulv(e, c, false); });
      break;
    }
    case OP_CONJ:
      ew_loop<E, LAY>(sm, Lp, B, len, tid, T,
                      [&](E &e, int, int) { e = conjv(e); });
      break;
    case OP_TW:
      if constexpr (Tr<E>::cplx) {
        const E *tw = (const E *)op.ptr;
        const int *perm = op.ptr2;
        const i64 N = op.N;
        const bool neg = op.sign < 0;
        ew_loop<E, LAY>(sm, Lp, B, len, tid, T, [&](E &e, int b, int j) {
          const int nat = perm ? perm[j] : j;
          // q * nat < N in the four-step passes (q < N / len,
          // nat < len): reduce only when a product reaches N
          i64 t = sq[b] * (i64)nat;
          if (t >= N) t %= N;
          const E wv = tw[t];
          e = neg ? cmul(e, wv) : cmulc(e, wv);
        });
      }
      break;
    default: break;
  }
  group_sync(T);
}

template <class E, int LAY>
__device__ void run_zpad(const Op &op, E *sm, int Lp, int B, int tid, int T) {
  const int cnt = op.len2 - op.len;
  const int total = B * cnt;
  const int lgB = __ffs(B) - 1;
  Walk w(tid, cnt, T);
  for (int f = tid; f < total; f += T, w.next()) {
    int b, j;
    if constexpr (LAY == 1) {
      b = f & (B - 1);
      j = f >> lgB;
    } else {
      b = w.b;
      j = w.j;
    }
    vbase<E, LAY>(sm, b, Lp)[jx<E, LAY>(op.len + j, B)] = zero<E>();
  }
  group_sync(T);
}

// ------------------------------------------------------------ async copies
// cp.async: per-thread global -> shared copies that complete in the
// background; src_bytes = 0 writes zeros without reading global memory.
template <int N>
__device__ __forceinline__ void cp_async(void *smem, const void *gmem,
                                         bool valid) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  const int n = valid ? N : 0;
  if constexpr (N == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s),
                 "l"(gmem), "r"(n));
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;\n" ::"r"(s),
                 "l"(gmem), "n"(N), "r"(n));
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::);
}
template <int N> __device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}
// wait until at most n groups are pending (n = 0..3)
__device__ __forceinline__ void cp_async_wait_n(int n) {
  switch (n) {
    case 0: cp_async_wait<0>(); break;
    case 1: cp_async_wait<1>(); break;
    case 2: cp_async_wait<2>(); break;
    default: cp_async_wait<3>(); break;
  }
}

// ---- TMA (cp.async.bulk.tensor) with mbarrier completion
__device__ __forceinline__ unsigned smem_addr(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar));
}
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes) {
  asm volatile(
      "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar),
      "r"(bytes)
      : "memory");
}
// one poll; the thread may be suspended inside it for up to ~1 us while the
// phase is incomplete (it resumes as soon as the phase completes)
__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned phase) {
  unsigned done;
  asm volatile(
      "{\n .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, 1000;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(bar), "r"(phase)
      : "memory");
  return done != 0;
}
// bounded wait: gives up after `limit` polls (each poll may suspend the
// thread for a while) and reports false
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned phase,
                                          long long limit) {
  for (long long it = 0; it < limit; ++it)
    if (mbar_try_wait(bar, phase)) return true;
  return false;
}
__device__ __forceinline__ void tma_load_4d(unsigned dst, const CUtensorMap *tm,
                                            int c0, int c1, int c2, int c3,
                                            unsigned bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::"
      "complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];\n" ::"r"(dst),
      "l"(tm), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void tma_store_4d(const CUtensorMap *tm,
                                             unsigned src, int c0, int c1,
                                             int c2, int c3) {
  asm volatile(
      "cp.async.bulk.tensor.4d.global.shared::cta.tile.bulk_group "
      "[%0, {%1, %2, %3, %4}], [%5];\n" ::"l"(tm),
      "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(src)
      : "memory");
}
__device__ __forceinline__ void bulk_commit() {
  asm volatile("cp.async.bulk.commit_group;\n" ::: "memory");
}
template <int N> __device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read %0;\n" ::"n"(N) : "memory");
}
__device__ __forceinline__ void bulk_wait_all() {
  asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory");
}
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}
// 1-D bulk copies (cp.async.bulk): 16-byte aligned, multiple of 16 bytes
__device__ __forceinline__ void bulk_load(unsigned dst, const void *src,
                                          unsigned bytes, unsigned bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1], %2, [%3];\n" ::"r"(dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void bulk_store(void *dst, unsigned src,
                                           unsigned bytes) {
  asm volatile(
      "cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;\n" ::"l"(
          dst),
      "r"(src), "r"(bytes)
      : "memory");
}

// bytes of one tile buffer (B vectors of Lp elements), 128-byte aligned
__host__ __device__ __forceinline__ size_t tile_bytes(int B, int Lp,
                                                      int esz) {
  return ((size_t)B * Lp * esz + 127) / 128 * 128;
}

// dynamic shared memory of a launch: nbuf tile buffers, nbuf mbarriers,
// nbuf sets of per-vector records and one per-vector scalar array
__host__ __device__ __forceinline__ size_t launch_smem(int B, int Lp, int esz,
                                                       int nbuf) {
  return nbuf * tile_bytes(B, Lp, esz) + 8 * (size_t)nbuf +
         (size_t)B * (nbuf * sizeof(VInfo) + 8 + 4);
}

// per-vector addressing of tile `tile` (vector indices below 2^31)
__device__ __forceinline__ void setup_tile(const Step &p, VInfo *vi,
                                           i64 tile, const FDiv &dV,
                                           const FDiv &dci, const FDiv &dco,
                                           i64 nvec, int tid, int T) {
  for (int b = tid; b < p.B; b += T) {
    const i64 gv = tile * p.B + b;
    VInfo x;
    if (gv < nvec) {
      const unsigned g = (unsigned)gv;
      const unsigned m = dV.div(g), v = g - m * (unsigned)p.V;
      const unsigned a = dci.div(v), c = v - a * (unsigned)p.vin.Cc;
      const unsigned a2 = dco.div(v), c2 = v - a2 * (unsigned)p.vout.Cc;
      x.col_src = (i64)m * p.ld_src;
      x.rb_in = (i64)a * p.vin.n * p.vin.Cc + c;
      x.col_dst = (i64)m * p.ld_dst;
      x.rb_out = (i64)a2 * p.vout.n * p.vout.Cc + c2;
      x.vcol = v;
    } else {
      x.col_src = x.col_dst = x.vcol = 0;
      x.rb_in = x.rb_out = -1;
    }
    vi[b] = x;
  }
}

// TMA coordinates of an element-major tile: all B vectors share column m and
// outer index a (the planner makes B divide Cc), inner offset c0.
__device__ __forceinline__ void tile_coords(const Step &p, i64 tile,
                                            const View &vw, int &c0, int &a,
                                            int &m) {
  const i64 gv = tile * p.B;
  const i64 mm = gv / p.V, v = gv - mm * p.V;
  const i64 aa = v / vw.Cc;
  c0 = (int)(v - aa * vw.Cc);
  a = (int)aa;
  m = (int)mm;
}

template <class E>
__device__ __forceinline__ void tma_issue_load(const Step &p, E *sm,
                                               unsigned bar, i64 tile) {
  int c0, a, m;
  tile_coords(p, tile, p.vin, c0, a, m);
  const unsigned bytes = (unsigned)((size_t)p.B * p.L * sizeof(E));
  mbar_expect_tx(bar, bytes);
  for (int j0 = 0; j0 < p.L; j0 += p.box_rows)
    tma_load_4d(smem_addr(sm + (size_t)j0 * p.B), &p.tm_in, c0 * p.elem_k,
                j0, a, m, bar);
}

template <class E>
__device__ __forceinline__ void tma_issue_store(const Step &p, const E *sm,
                                                i64 tile) {
  int c0, a, m;
  tile_coords(p, tile, p.vout, c0, a, m);
  fence_async_smem();
  for (int j0 = 0; j0 < p.out_len; j0 += p.box_rows)
    tma_store_4d(&p.tm_out, smem_addr(sm + (size_t)j0 * p.B), c0 * p.elem_k,
                 j0, a, m);
  bulk_commit();
}

// Hardware copies of a whole tile.  Element-major tiles: TMA boxes issued by
// one thread.  Vector-major tiles of contiguous vectors: one 1-D bulk copy
// per 128-byte chunk of every vector, spread over the threads, into the
// padded layout (each chunk is contiguous and 16-byte aligned there).
template <class E, int LAY>
__device__ __forceinline__ void issue_load(const Step &p, E *sm, unsigned bar,
                                           i64 tile, const FDiv &dV, i64 nvec,
                                           int tid, int T) {
  if constexpr (LAY == 1) {
    if (tid == 0) tma_issue_load<E>(p, sm, bar, tile);
  } else if constexpr (LAY == 2) {
    // dense tile: every run of consecutive vectors within one column is a
    // single bulk copy (vector b at b * L, L = in_len)
    if (tid != 0) return;
    const i64 gv0 = tile * p.B;
    const int nv = (int)(nvec - gv0 < p.B ? nvec - gv0 : p.B);
    const int L = p.in_len;
    mbar_expect_tx(bar, (unsigned)((size_t)nv * L * sizeof(E)));
    const E *src = (const E *)p.src;
    for (int b = 0; b < nv;) {
      const unsigned g = (unsigned)(gv0 + b);
      const unsigned m = dV.div(g), v = g - m * (unsigned)p.V;
      int cnt = (int)((unsigned)p.V - v);
      if (cnt > nv - b) cnt = nv - b;
      bulk_load(smem_addr(sm + (i64)b * L),
                src + (i64)m * p.ld_src + (i64)v * p.vin.n,
                (unsigned)((size_t)cnt * L * sizeof(E)), bar);
      b += cnt;
    }
  } else {
    constexpr int CH = 128 / (int)sizeof(E);
    const int nch = (p.in_len + CH - 1) / CH;
    const i64 gv0 = tile * p.B;
    const i64 nv = nvec - gv0 < p.B ? nvec - gv0 : p.B;
    if (tid == 0)
      mbar_expect_tx(bar, (unsigned)((size_t)nv * p.in_len * sizeof(E)));
    const E *src = (const E *)p.src;
    const FDiv dch((unsigned)nch);
    for (int c = tid; c < nv * nch; c += T) {
      const int b = (int)dch.div((unsigned)c), k = c - b * nch;
      const unsigned g = (unsigned)(gv0 + b);
      const unsigned m = dV.div(g), v = g - m * (unsigned)p.V;
      const i64 off = (i64)m * p.ld_src + (i64)v * p.vin.n + (i64)k * CH;
      const int cnt = p.in_len - k * CH < CH ? p.in_len - k * CH : CH;
      bulk_load(smem_addr(sm + b * p.Lp + pidx<E>(k * CH)), src + off,
                (unsigned)(cnt * sizeof(E)), bar);
    }
  }
}

template <class E, int LAY>
__device__ __forceinline__ void issue_store(const Step &p, const E *sm,
                                            i64 tile, const FDiv &dV,
                                            i64 nvec, int tid, int T) {
  if constexpr (LAY == 1) {
    if (tid == 0) tma_issue_store<E>(p, sm, tile);
  } else if constexpr (LAY == 2) {
    if (tid != 0) return;
    const i64 gv0 = tile * p.B;
    const int nv = (int)(nvec - gv0 < p.B ? nvec - gv0 : p.B);
    const int L = p.out_len;
    E *dst = (E *)p.dst;
    for (int b = 0; b < nv;) {
      const unsigned g = (unsigned)(gv0 + b);
      const unsigned m = dV.div(g), v = g - m * (unsigned)p.V;
      int cnt = (int)((unsigned)p.V - v);
      if (cnt > nv - b) cnt = nv - b;
      bulk_store(dst + (i64)m * p.ld_dst + (i64)v * p.vout.n,
                 smem_addr(sm + (i64)b * L),
                 (unsigned)((size_t)cnt * L * sizeof(E)));
      b += cnt;
    }
    bulk_commit();
  } else {
    constexpr int CH = 128 / (int)sizeof(E);
    const int nch = (p.out_len + CH - 1) / CH;
    const i64 gv0 = tile * p.B;
    const i64 nv = nvec - gv0 < p.B ? nvec - gv0 : p.B;
    E *dst = (E *)p.dst;
    fence_async_smem();
    bool any = false;
    const FDiv dch((unsigned)nch);
    for (int c = tid; c < nv * nch; c += T) {
      const int b = (int)dch.div((unsigned)c), k = c - b * nch;
      const unsigned g = (unsigned)(gv0 + b);
      const unsigned m = dV.div(g), v = g - m * (unsigned)p.V;
      const i64 off = (i64)m * p.ld_dst + (i64)v * p.vout.n + (i64)k * CH;
      const int cnt = p.out_len - k * CH < CH ? p.out_len - k * CH : CH;
      bulk_store(dst + off, smem_addr(sm + b * p.Lp + pidx<E>(k * CH)),
                 (unsigned)(cnt * sizeof(E)));
      any = true;
    }
    if (any) bulk_commit();
  }
}

// vector-major tiles before a bulk store: reorder (out_pos), post-multiply,
// scale, conjugate and (double-float) convert in shared memory
template <class E, int LAY>
__device__ __forceinline__ void store_fixup_vm(const Step &p, E *sm,
                                               const VInfo *vi,
                                               const int *sexp, int tid,
                                               int T, bool natural = false) {
  const int B = p.B, Lp = p.Lp, n = p.out_len;
  const int total = B * n;
  if (p.out_pos && !natural) {
    constexpr int MB = Ept<E>::v;
    E v[MB];
    {
      Walk w(tid, n, T);
#pragma unroll
      for (int i = 0; i < MB; ++i, w.next())
        if (tid + i * T < total)
          v[i] = sm[w.b * Lp + vx<E, LAY>(p.out_pos[w.j])];
    }
    __syncthreads();
    {
      Walk w(tid, n, T);
#pragma unroll
      for (int i = 0; i < MB; ++i, w.next())
        if (tid + i * T < total) sm[w.b * Lp + vx<E, LAY>(w.j)] = v[i];
    }
    __syncthreads();
  }
  const bool any = p.post || p.has_scale || p.conj_out || Emu<E>::v;
  if (!any) return;
  const E *post = (const E *)p.post;
  const bool has_scale = p.has_scale != 0, cj = p.conj_out != 0;
  const E c = scalar_of<E>(p.scale_re, p.scale_im);
  Walk w(tid, n, T);
  for (int f = tid; f < total; f += T, w.next()) {
    const int b = w.b, j = w.j;
    E *e = sm + b * Lp + vx<E, LAY>(j);
    E val = *e;
    if (post && vi[b].rb_out >= 0)
      val = mulv(val, post[vi[b].rb_out + j], false);
    if (has_scale) val = mulv(val, c, false);
    if (cj) val = conjv(val);
    if constexpr (Emu<E>::v) val = to_bits(val, sexp[b]);
    *e = val;
  }
  __syncthreads();
}

// asynchronous per-thread load of a tile whose source already has the
// compute type and needs no gather: every element (zero padding included)
// is one cp.async
template <class E, int LAY>
__device__ __forceinline__ void load_async(const Step &p, E *sm,
                                           const VInfo *vi, int tid, int T) {
  // (the launch record may sit in shared memory: its fields are read once,
  // so the copies below need not reload them)
  const int B = p.B, L = p.L, Lp = p.Lp;
  const int total = B * L;
  const E *src = (const E *)p.src;
  const i64 cc = p.vin.Cc;
  const int in_len = p.in_len;
  const i64 in_rows = p.in_rows;
  const int lgB = __ffs(B) - 1;
  if constexpr (LAY == 0 && sizeof(E) == 8) {
    if (cc == 1 && (Lp & 1) == 0 && (L & (L - 1)) == 0 &&
        ((size_t)src & 15) == 0) {
      // contiguous vectors of a power-of-two length: pairs of points as one
      // 16-byte copy where both exist and the source pair is aligned
      const int lgh = __ffs(L) - 2;  // log2(L / 2)
      for (int f = tid; f < total / 2; f += T) {
        const int b = f >> lgh, j = (f & ((L >> 1) - 1)) << 1;
        const i64 rb = vi[b].rb_in;
        const i64 r = rb + j;
        E *d = sm + b * Lp + pidx<E>(j);
        const E *s = src + vi[b].col_src + r;
        if (rb >= 0 && j + 1 < in_len && r + 1 < in_rows &&
            (((size_t)s & 15) == 0)) {
          cp_async<16>(d, s, true);
        } else {
          const bool ok0 = rb >= 0 && j < in_len && r < in_rows;
          const bool ok1 = rb >= 0 && j + 1 < in_len && r + 1 < in_rows;
          cp_async<8>(d, ok0 ? (const void *)s : (const void *)src, ok0);
          cp_async<8>(d + 1, ok1 ? (const void *)(s + 1) : (const void *)src,
                      ok1);
        }
      }
      return;
    }
  }
  if (LAY == 0 && cc > 1 && B <= T) {
    // vectors strided across rows: consecutive threads take consecutive
    // vectors, so (T a multiple of B) each thread keeps one vector and
    // walks its points
    const int b = tid & (B - 1);
    const i64 rb = vi[b].rb_in;
    const E *s = src + vi[b].col_src + rb;
    E *d = sm + b * Lp;
    const int js = T >> lgB;
    const i64 lim = rb >= 0 ? in_rows - rb : 0;
    for (int j = tid >> lgB; j < L; j += js) {
      const i64 off = (i64)j * cc;
      const bool ok = j < in_len && off < lim;
      cp_async<sizeof(E)>(d + pidx<E>(j), ok ? (const void *)(s + off)
                                             : (const void *)src,
                          ok);
    }
    return;
  }
  Walk w(tid, L, T);
  for (int f = tid; f < total; f += T, w.next()) {
    int b, j;
    if (cc > 1 || LAY == 1) {
      j = f >> lgB;
      b = f & (B - 1);
    } else {
      b = w.b;
      j = w.j;
    }
    const i64 rb = vi[b].rb_in;
    const i64 r = rb + (i64)j * cc;
    const bool ok = rb >= 0 && j < in_len && r < in_rows;
    cp_async<sizeof(E)>(vbase<E, LAY>(sm, b, Lp) + jx<E, LAY>(j, B),
                        ok ? (const void *)(src + vi[b].col_src + r)
                           : (const void *)src,
                        ok);
  }
}

// synchronous load with type conversion, gather map, conjugation and
// pre-multiplication
template <class E, int LAY>
__device__ __forceinline__ void load_general(const Step &p, E *sm,
                                             const VInfo *vi, int tid,
                                             int T) {
  const int B = p.B, L = p.L, Lp = p.Lp;
  const int total = B * L;
  const i64 cc = p.vin.Cc;
  const int lgB = __ffs(B) - 1;
  Walk w(tid, L, T);
  for (int f = tid; f < total; f += T, w.next()) {
    int b, j;
    if (cc > 1 || LAY == 1) {
      j = f >> lgB;
      b = f & (B - 1);
    } else {
      b = w.b;
      j = w.j;
    }
    E val = zero<E>();
    const i64 rb = vi[b].rb_in;
    if (rb >= 0 && j < p.in_len) {
      const i64 r = rb + (i64)j * cc;
      if (r < p.in_rows) {
        const i64 srow = p.map_in ? p.map_in[r] : r;
        if (srow >= 0) {
          val = load_as<E>(p.src, p.src_type, vi[b].col_src + srow);
          if (p.conj_in) val = conjv(val);
          if (p.pre) val = mulv(val, ((const E *)p.pre)[r], false);
        }
      }
    }
    vbase<E, LAY>(sm, b, Lp)[jx<E, LAY>(j, B)] = val;
  }
}

// conjugation / pre-multiplication applied in shared memory after an
// asynchronous load
template <class E, int LAY>
__device__ __forceinline__ void load_fixup(const Step &p, E *sm,
                                           const VInfo *vi, int tid, int T) {
  const int B = p.B, L = p.L, Lp = p.Lp;
  const int total = B * L;
  const i64 cc = p.vin.Cc;
  const int in_len = p.in_len;
  const i64 in_rows = p.in_rows;
  const bool conj_in = p.conj_in != 0;
  const E *const pre = (const E *)p.pre;
  const int lgB = __ffs(B) - 1;
  Walk w(tid, L, T);
  for (int f = tid; f < total; f += T, w.next()) {
    int b, j;
    if constexpr (LAY == 1) {
      b = f & (B - 1);
      j = f >> lgB;
    } else {
      b = w.b;
      j = w.j;
    }
    const i64 rb = vi[b].rb_in;
    if (rb < 0 || j >= in_len) continue;
    const i64 r = rb + (i64)j * cc;
    if (r >= in_rows) continue;
    E *e = vbase<E, LAY>(sm, b, Lp) + jx<E, LAY>(j, B);
    E val = *e;
    if (conj_in) val = conjv(val);
    if (pre) val = mulv(val, pre[r], false);
    *e = val;
  }
}

// element-major tiles before a TMA store: reorder (out_pos), post-multiply,
// scale and conjugate in shared memory
template <class E>
__device__ __forceinline__ void store_fixup_em(const Step &p, E *sm,
                                               const VInfo *vi, int tid,
                                               int T) {
  const int B = p.B;
  const int total = B * p.out_len;
  const int lgB = __ffs(B) - 1;
  const i64 cc = p.vout.Cc;
  if (p.out_pos) {
    // permute through registers: gather, barrier, write back
    constexpr int MB = Ept<E>::v;
    E v[MB];
#pragma unroll
    for (int i = 0; i < MB; ++i) {
      const int f = tid + i * T;
      if (f < total)
        v[i] = sm[p.out_pos[f >> lgB] * B + (f & (B - 1))];
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < MB; ++i) {
      const int f = tid + i * T;
      if (f < total) sm[f] = v[i];
    }
    __syncthreads();
  }
  if (!p.post && !p.has_scale && !p.conj_out) return;
  const E c = scalar_of<E>(p.scale_re, p.scale_im);
  for (int f = tid; f < total; f += T) {
    const int b = f & (B - 1), j = f >> lgB;
    E val = sm[f];
    if (p.post) {
      const i64 rb = vi[b].rb_out;
      if (rb >= 0) val = mulv(val, ((const E *)p.post)[rb + (i64)j * cc], false);
    }
    if (p.has_scale) val = mulv(val, c, false);
    if (p.conj_out) val = conjv(val);
    sm[f] = val;
  }
  __syncthreads();
}

template <class E, int LAY>
__device__ __forceinline__ void store_tile(const Step &p, const E *sm,
                                           const VInfo *vi, const int *sexp,
                                           int tid, int T,
                                           bool natural = false) {
  const int B = p.B, Lp = p.Lp;
  const bool acc = p.accumulate != 0;
  const E c = scalar_of<E>(p.scale_re, p.scale_im);
  if constexpr (LAY != 1) {
    if (p.out_mode == 1) {
      // gather: out row i of column m takes vector element map_out[i]
      Walk w(tid, p.n_out, T);
      for (int f = tid; f < B * p.n_out; f += T, w.next()) {
        const int b = w.b, i = w.j;
        if (vi[b].rb_out < 0) continue;
        const i64 j = p.map_out[i];
        E val = j < 0 ? zero<E>() : sm[b * Lp + vx<E, LAY>((int)j)];
        if (j >= 0 && p.post) val = mulv(val, ((const E *)p.post)[j], false);
        if (p.has_scale) val = mulv(val, c, false);
        if (p.conj_out) val = conjv(val);
        store_as<E>(p.dst, p.dst_type, vi[b].col_dst + i, val, acc,
                    Emu<E>::v ? sexp[b] : 0);
      }
      return;
    }
  }
  // (the launch record may sit in shared memory, and the compiler cannot
  // rule out that the global stores below alias it: its fields are read
  // into registers once)
  const i64 ccout = p.vout.Cc;
  const int out_len = p.out_len;
  const int total = B * out_len;
  const int lgB = __ffs(B) - 1;
  const i64 out_rows = p.out_rows;
  const i64 *const map_out = p.out_mode == 2 ? p.map_out : nullptr;
  const int *const out_pos = natural ? nullptr : p.out_pos;
  const E *const post = (const E *)p.post;
  const bool has_scale = p.has_scale != 0, conj_out = p.conj_out != 0;
  const bool raw = p.dst_type == Tr<E>::code && !acc;
  void *const dst = p.dst;
  const int dst_type = p.dst_type;
  if (LAY == 0 && ccout > 1 && B <= T && !map_out) {
    // one vector per thread (T a multiple of B), its points j, j + T / B, ..
    const int b = tid & (B - 1);
    const i64 rb = vi[b].rb_out;
    if (rb < 0) return;
    const E *vsm = sm + b * Lp;
    const i64 lim = out_rows - rb;
    const i64 base = vi[b].col_dst + rb;
    const int js = T >> lgB;
    for (int j = tid >> lgB; j < out_len; j += js) {
      const i64 off = (i64)j * ccout;
      if (off >= lim) break;
      E val = vsm[pidx<E>(out_pos ? out_pos[j] : j)];
      if (post) val = mulv(val, post[rb + off], false);
      if (has_scale) val = mulv(val, c, false);
      if (conj_out) val = conjv(val);
      if constexpr (Emu<E>::v) {
        if (raw)
          ((E *)dst)[base + off] = to_bits(val, sexp[b]);
        else
          store_as<E>(dst, dst_type, base + off, val, acc, sexp[b]);
      } else {
        if (raw)
          ((E *)dst)[base + off] = val;
        else
          store_as<E>(dst, dst_type, base + off, val, acc);
      }
    }
    return;
  }
  Walk w(tid, out_len, T);
  for (int f = tid; f < total; f += T, w.next()) {
    int b, j;
    if (ccout > 1 || LAY == 1) {
      j = f >> lgB;
      b = f & (B - 1);
    } else {
      b = w.b;
      j = w.j;
    }
    const i64 rb = vi[b].rb_out;
    if (rb < 0) continue;
    const i64 r = rb + (i64)j * ccout;
    if (r >= out_rows) continue;
    const i64 drow = map_out ? map_out[r] : r;
    if (drow < 0) continue;
    E val = vbase<E, LAY>(const_cast<E *>(sm), b, Lp)
        [jx<E, LAY>(out_pos ? out_pos[j] : j, B)];
    if (post) val = mulv(val, post[r], false);
    if (has_scale) val = mulv(val, c, false);
    if (conj_out) val = conjv(val);
    if constexpr (Emu<E>::v) {
      if (raw)
        ((E *)dst)[vi[b].col_dst + drow] = to_bits(val, sexp[b]);
      else
        store_as<E>(dst, dst_type, vi[b].col_dst + drow, val, acc, sexp[b]);
    } else {
      if (raw)
        ((E *)dst)[vi[b].col_dst + drow] = val;
      else
        store_as<E>(dst, dst_type, vi[b].col_dst + drow, val, acc);
    }
  }
}

// ---- double-float tiles: the tile arrives as float64 / complex128 bits;
// each vector is normalised by the power of two of its largest exponent
// (exact) and split into double-floats in place; the store path reverses it
template <class E, int LAY>
__device__ __forceinline__ void emu_in(const Step &p, E *sm, const VInfo *vi,
                                       int *sexp, int tid, int T) {
  const int B = p.B, L = p.L, Lp = p.Lp;
  const int total = B * L;
  const int lgB = __ffs(B) - 1;
  for (int b = tid; b < B; b += T) sexp[b] = 0;
  __syncthreads();
  {
    // per-thread maximum over the run of elements of one vector, one
    // shared-memory atomic per run
    Walk w(tid, L, T);
    int cb = -1, cmax = 0;
    for (int f = tid; f < total; f += T, w.next()) {
      int b, j;
      if constexpr (LAY == 1) {
        b = f & (B - 1);
        j = f >> lgB;
      } else {
        b = w.b;
        j = w.j;
      }
      if (b != cb) {
        if (cb >= 0 && cmax > 0) atomicMax(sexp + cb, cmax);
        cb = b;
        cmax = 0;
      }
      const int e = raw_exp(vbase<E, LAY>(sm, b, Lp)[jx<E, LAY>(j, B)]);
      cmax = e > cmax ? e : cmax;
    }
    if (cb >= 0 && cmax > 0) atomicMax(sexp + cb, cmax);
  }
  __syncthreads();
  for (int b = tid; b < B; b += T) sexp[b] = sexp[b] > 0 ? sexp[b] - 1023 : 0;
  __syncthreads();
  Walk w(tid, L, T);
  for (int f = tid; f < total; f += T, w.next()) {
    int b, j;
    if constexpr (LAY == 1) {
      b = f & (B - 1);
      j = f >> lgB;
    } else {
      b = w.b;
      j = w.j;
    }
    E *e = vbase<E, LAY>(sm, b, Lp) + jx<E, LAY>(j, B);
    *e = from_bits(*e, sexp[b]);
  }
}

template <class E>
__device__ __forceinline__ void emu_out_em(const Step &p, E *sm,
                                          const int *sexp, int tid, int T) {
  const int total = p.B * p.L;
  for (int f = tid; f < total; f += T) sm[f] = to_bits(sm[f], sexp[f & (p.B - 1)]);
}

template <class E, int CLS, int LAY>
__device__ __forceinline__ void run_program(const Step &p, E *sm, int Lp,
                                            int B, const VInfo *vi, i64 *sq,
                                            int tid, int T,
                                            TcState *tc = nullptr,
                                            TdState *td = nullptr) {
  for (int o = 0; o < p.nops; ++o) {
    const Op &op = p.ops[o];
    switch (op.kind) {
      case OP_DIF:
      case OP_DIT:
        if constexpr (Tr<E>::cplx && CLS == 5) {
          // a whole-vector product with one table right after a forward
          // transform (a convolution's spectrum) is applied by the
          // transform's last stage as it stores its outputs
          const Op *nx = o + 1 < p.nops ? &p.ops[o + 1] : nullptr;
          const int last = op.nrad > 0 ? op.rad[op.nrad - 1] : 0;
          const bool fuse = op.kind == OP_DIF && nx && nx->kind == OP_MUL &&
                            nx->div == 1 && nx->mod == 1 &&
                            nx->len == op.len && last > 1 &&
                            (last & (last - 1)) == 0;
          run_fft<E, CLS, LAY>(op, sm, Lp, B, tid, T,
                               fuse ? Post{nx->ptr, nx->sign}
                                    : Post{nullptr, 0});
          if (fuse) ++o;
        } else if constexpr (Tr<E>::cplx && CLS != 3) {
          run_fft<E, CLS, LAY>(op, sm, Lp, B, tid, T, Post{nullptr, 0});
        }
        break;
      case OP_FWHT:
        if constexpr (CLS == 0 || CLS == 3 || CLS == 4)
          run_fwht<E, LAY>(op, sm, Lp, B, tid, T, tc);
        break;
      case OP_GATHER:
        if constexpr (CLS == 0 && LAY != 1)
          run_gather<E, LAY>(op, sm, Lp, B, tid, T);
        break;
      case OP_DENSE:
        if constexpr (CLS == 0 && LAY != 1)
          run_dense<E, LAY>(op, sm, Lp, B, tid, T);
        if constexpr (CLS == 6 && std::is_same<E, float>::value)
          run_densetc<LAY>(sm, Lp, B, *td, tid, T);
        break;
      case OP_ZPAD: run_zpad<E, LAY>(op, sm, Lp, B, tid, T); break;
      default:
        run_elementwise<E, LAY>(op, sm, Lp, B, vi, sq, tid, T);
        break;
    }
  }
}

}  // namespace fmk
#include "fm_rtile.cuh"
namespace fmk {

// polls of a bounded mbarrier wait before a launch reports FM_ERR_TIMEOUT
// (the default of Step::wait_limit; fm_plan_set_wait_limit changes it)
#define FM_WAIT_LIMIT (1LL << 22)

// ------------------------------------------------------------ the kernel
// CLS selects the op subset compiled into an instantiation, so the hot
// programs (power-of-two FFT, FWHT) do not carry the register pressure of
// the rarely used ops: 1 = pow2 FFT + pointwise, 2 = FFT with radices 3/5/7,
// 3 = FWHT + pointwise, 4 = FWHT with 16-point groups on the tensor cores
// (float only) + pointwise, 5 = as 1 with a convolution's spectrum product
// applied by the last stage of the forward transform, 0 = everything.  LAY
// is the tile layout.
//
// Persistent CTAs: each CTA walks tiles blockIdx.x, blockIdx.x + gridDim.x,
// ...  Tiles are copied into a ring of p.nbuf shared-memory buffers
// nbuf - 1 tiles ahead of the one being transformed and stored, so several
// tiles of HBM reads are in flight per SM while the butterflies run: by TMA
// boxes (one instruction per box, completion counted on an mbarrier) for
// element-major tiles, by per-thread cp.async otherwise.  Element-major
// results leave by TMA box stores.  Dynamic shared memory (launch_smem):
// nbuf tile buffers, nbuf mbarriers, nbuf sets of VInfo records, per-vector
// scalars.
// Whether the warps of a CTA can run the tile program on disjoint sets of
// vectors (vector-major tiles whose B vectors divide evenly among the warps,
// few enough elements per warp for the register-staged ops), so that the
// program's stages need warp barriers only.
template <class E, int CLS, int LAY>
__device__ __forceinline__ bool warp_mode(int B, int L, int nwarps) {
  return LAY != 1 && CLS != 4 && CLS != 6 && nwarps > 1 && B % nwarps == 0 &&
         (B / nwarps) * L <= 32 * Ept<E>::v;
}

template <class E, int CLS, int LAY>
__global__ void __launch_bounds__(FM_MAX_THREADS, (MinBlocks<E, CLS>::v))
    vprog_kernel(const __grid_constant__ Step p) {
  extern __shared__ __align__(128) unsigned char fm_smem[];
  const int tid = threadIdx.x, T = blockDim.x;
  const int B = p.B, Lp = p.Lp;
  const int NB = p.nbuf;
  const size_t tb = tile_bytes(B, Lp, sizeof(E));
  unsigned long long *bars =
      reinterpret_cast<unsigned long long *>(fm_smem + NB * tb);
  VInfo *const vi0 = reinterpret_cast<VInfo *>(bars + NB);
  i64 *sq = reinterpret_cast<i64 *>(vi0 + NB * B);
  int *sexp = reinterpret_cast<int *>(sq + B);  // per-vector scale (emu)
  auto buf = [&](int k) { return reinterpret_cast<E *>(fm_smem + k * tb); };
  auto vis = [&](int k) { return vi0 + k * B; };
  const i64 nvec = p.V * p.num_cols;
  const i64 ntiles = (nvec + B - 1) / B;
  const FDiv dV((unsigned)p.V), dci((unsigned)p.vin.Cc),
      dco((unsigned)p.vout.Cc);
  const bool tma_in = p.tma_in != 0;    // hardware copies into the ring
  const bool tma_out = p.tma_out != 0;  // hardware copies out of the tile
  const bool async_in = tma_in || (p.src_type == Tr<E>::code && !p.map_in);
  const bool fixup = p.conj_in || p.pre;
  const i64 G = gridDim.x;
  const int nwarps = T >> 5;
  const bool wmode = warp_mode<E, CLS, LAY>(B, p.L, nwarps);

  if (tma_in) {
    if (tid == 0) {
      for (int k = 0; k < NB; ++k) mbar_init(smem_addr(bars + k));
      mbar_init_fence();
    }
    __syncthreads();
  }
  TcState tcs;
  TcState *tc = nullptr;
  if constexpr (CLS == 4) {
    const size_t off =
        (launch_smem(B, Lp, sizeof(E), NB) + 1023) & ~(size_t)1023;
    tc_init(tcs, fm_smem + off, p.err, tid);
    tc = &tcs;
  }
  // class 6: the program's one dense factor, staged for the tensor cores
  TdState tds;
  if constexpr (CLS == 6 && std::is_same<E, float>::value) {
    const size_t off =
        (launch_smem(B, Lp, sizeof(E), NB) + 1023) & ~(size_t)1023;
    const Op *dop = nullptr;
    for (int o = 0; o < p.nops; ++o)
      if (p.ops[o].kind == OP_DENSE) dop = &p.ops[o];
    td_init(tds, fm_smem + off, (const float *)dop->ptr, dop->len, T, p.err,
            tid);
  }

  i64 tile = blockIdx.x;
  // prologue: the first nbuf - 1 tiles
  if (async_in) {
    for (int k = 0; k < NB - 1; ++k) {
      const i64 t = tile + k * G;
      if (t < ntiles) {
        setup_tile(p, vis(k), t, dV, dci, dco, nvec, tid, T);
        if (tma_in) {
          issue_load<E, LAY>(p, buf(k), smem_addr(bars + k), t, dV, nvec, tid,
                             T);
        } else {
          __syncthreads();
          load_async<E, LAY>(p, buf(k), vis(k), tid, T);
        }
      }
      if (!tma_in) cp_async_commit();
    }
  }
  int cur = 0;
  unsigned phase_bits = 0;  // bit k: parity of the next completion of bar k
  bool failed = false;
  while (tile < ntiles) {
    E *sm = buf(cur);
    VInfo *vi = vis(cur);
    // per-thread loads refill buffers that a bulk store may still be
    // reading: wait for those reads (a barrier follows before any refill)
    if (tma_out && !tma_in) bulk_wait_read<0>();
    if (async_in) {
      if (!tma_in) {
        const i64 ahead = tile + (NB - 1) * G;
        int slot = cur + NB - 1;
        if (slot >= NB) slot -= NB;
        if (ahead < ntiles) {
          setup_tile(p, vis(slot), ahead, dV, dci, dco, nvec, tid, T);
          __syncthreads();
          load_async<E, LAY>(p, buf(slot), vis(slot), tid, T);
        }
        cp_async_commit();
        cp_async_wait_n(NB - 1);
      } else {
        // one warp polls the barrier, the others wait at the block barrier
        // (which issues no instructions); the vote then tells every thread
        // whether the copy landed, so all leave the loop together
        bool ok = true;
        if (tid < 32)
          ok = mbar_wait(smem_addr(bars + cur), (phase_bits >> cur) & 1u,
                         p.wait_limit);
        if (__syncthreads_or(!ok)) {
          failed = true;
          break;
        }
        phase_bits ^= 1u << cur;
      }
      __syncthreads();
      if constexpr (Emu<E>::v) {
        emu_in<E, LAY>(p, sm, vi, sexp, tid, T);
        __syncthreads();
      }
      if (fixup) {
        load_fixup<E, LAY>(p, sm, vi, tid, T);
        __syncthreads();
      }
    } else {
      setup_tile(p, vi, tile, dV, dci, dco, nvec, tid, T);
      if constexpr (Emu<E>::v)
        for (int b = tid; b < B; b += T) sexp[b] = 0;
      __syncthreads();
      load_general<E, LAY>(p, sm, vi, tid, T);
      __syncthreads();
    }

    bool natural = false, stored = false;
    if constexpr (std::is_same<E, float2>::value && LAY == 0) {
      if (p.rprog) {
        // the program on registers (fm_rtile.cuh); results in natural
        // order, or already stored
        rt_program(p, sm, vi, tid, T);
        natural = true;
        stored = (p.rprog & RT_DIRECT) != 0;
      }
    }
    if (natural) {
    } else if (wmode) {
      // each warp runs the program on its own B / nwarps vectors
      const int w = tid >> 5, vw = B / nwarps;
      run_program<E, CLS, LAY>(p, sm + w * vw * Lp, Lp, vw, vi + w * vw,
                               sq + w * vw, tid & 31, 32, tc, &tds);
      __syncthreads();
    } else {
      run_program<E, CLS, LAY>(p, sm, Lp, B, vi, sq, tid, T, tc, &tds);
    }

    if (stored) {
    } else if (tma_out) {
      if constexpr (LAY == 1) {
        store_fixup_em<E>(p, sm, vi, tid, T);
        if constexpr (Emu<E>::v) {
          emu_out_em<E>(p, sm, sexp, tid, T);
          __syncthreads();
        }
      } else {
        store_fixup_vm<E, LAY>(p, sm, vi, sexp, tid, T, natural);
      }
      // every writer orders its shared-memory writes before the bulk /
      // TMA reads of the store, then the issuing threads start it
      fence_async_smem();
      __syncthreads();
      issue_store<E, LAY>(p, sm, tile, dV, nvec, tid, T);
    } else {
      store_tile<E, LAY>(p, sm, vi, sexp, tid, T, natural);
    }
    if (tma_in) {
      // refill the buffer freed one iteration ago (tile - G) with the tile
      // nbuf - 1 ahead, once its TMA store has finished reading it
      const i64 ahead = tile + (NB - 1) * G;
      int slot = cur + NB - 1;
      if (slot >= NB) slot -= NB;
      // every thread that issued bulk stores waits until the older ones
      // have been read out of shared memory
      if (tma_out) bulk_wait_read<1>();
      fence_async_smem();
      __syncthreads();
      if (ahead < ntiles) {
        setup_tile(p, vis(slot), ahead, dV, dci, dco, nvec, tid, T);
        issue_load<E, LAY>(p, buf(slot), smem_addr(bars + slot), ahead, dV,
                           nvec, tid, T);
      }
    }
    __syncthreads();
    if (++cur == NB) cur = 0;
    tile += G;
  }
  if (failed) {
    if (tid == 0 && p.err) atomicExch(p.err, FM_ERR_TIMEOUT);
    // let the loads still in flight (this tile and up to nbuf - 2 ahead)
    // land before the CTA exits, again with bounded waits (of the default
    // length, whatever limit made the first wait give up)
    for (int d = 0; d < NB - 1; ++d) {
      int k = cur + d;
      if (k >= NB) k -= NB;
      if (tile + d * G < ntiles)
        mbar_wait(smem_addr(bars + k), (phase_bits >> k) & 1u, FM_WAIT_LIMIT);
    }
  }
  if (tma_out) bulk_wait_all();
  if (!tma_in) cp_async_wait<0>();
  if constexpr (CLS == 4) tc_release(tcs, tid);
  if constexpr (CLS == 6 && std::is_same<E, float>::value)
    td_release(tds, tid);
}


// ------------------------------------------------------------ batches
// Many operators in one persistent launch.  The launches of every operator's
// plan are grouped into levels (level k holds the k-th launch of every plan);
// level k + 1 reads what level k wrote, so the CTAs of the (cooperative)
// launch meet at a grid barrier between levels.  Within a level the tiles of
// all its steps form one index range, start[] holding each step's first
// tile; every CTA walks it with stride gridDim.x.  Tiles are vector-major and
// moved by plain loads and stores (one buffer), the step parameters are read
// from global memory.

// Bounded grid barrier: thread 0 of every CTA arrives on a counter and waits
// until all gridDim.x CTAs of this phase have arrived.  Returns false (and
// records FM_ERR_TIMEOUT) if the wait gives up; the caller then returns.
__device__ __forceinline__ bool grid_barrier(unsigned *bar, unsigned target,
                                             int *err, long long limit) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(bar, 1u);
    unsigned v = 0;
    long long it = 0;
    for (;;) {
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];"
                   : "=r"(v)
                   : "l"(bar)
                   : "memory");
      if (v >= target || ++it > limit) break;
      __nanosleep(64);
    }
    ok = v >= target;
    if (!ok && err) atomicExch(err, FM_ERR_TIMEOUT);
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

// shared memory of the batch kernel: two slots of launch records, the
// per-vector scalars, two slots of (per-vector records, per-vector
// exponents) and two tile buffers
__host__ __device__ __forceinline__ size_t batch_steps_bytes() {
  return (2 * sizeof(Step) + 127) / 128 * 128;
}
__host__ __device__ __forceinline__ size_t batch_head_bytes(int max_B) {
  return batch_steps_bytes() +
         ((size_t)max_B * (8 + 2 * (sizeof(VInfo) + 4)) + 127) / 128 * 128;
}
__host__ __device__ __forceinline__ size_t batch_smem(int max_B,
                                                      size_t max_tile) {
  return batch_head_bytes(max_B) + 2 * max_tile;
}


// Loads of one batch tile into a slot: cp.async when the source already
// has the compute type and needs no gather (completion is awaited later,
// so the copy overlaps the previous tile's program), synchronous loads with
// conversion and gather otherwise.
// The launch record is first copied into shared memory (read there by
// every op of the tile program instead of from global memory).
template <class E>
__device__ __forceinline__ void batch_issue_load(const Step *gp, Step *slot,
                                                 E *sm, VInfo *vi, i64 tile,
                                                 int tid, int T) {
  {
    static_assert(sizeof(Step) % 16 == 0, "launch record size");
    const int4 *src = reinterpret_cast<const int4 *>(gp);
    int4 *dst = reinterpret_cast<int4 *>(slot);
    for (int i = tid; i < (int)(sizeof(Step) / 16); i += T) dst[i] = src[i];
  }
  __syncthreads();
  const Step &p = *slot;
  const i64 nvec = p.V * p.num_cols;
  const FDiv dV((unsigned)p.V), dci((unsigned)p.vin.Cc),
      dco((unsigned)p.vout.Cc);
  setup_tile(p, vi, tile, dV, dci, dco, nvec, tid, T);
  __syncthreads();
  if (p.src_type == Tr<E>::code && !p.map_in)
    load_async<E, 0>(p, sm, vi, tid, T);
  else
    load_general<E, 0>(p, sm, vi, tid, T);
  cp_async_commit();
}

template <class E, int CLS>
__global__ void __launch_bounds__(FM_MAX_THREADS, (MinBlocks<E, CLS>::v))
    batch_kernel(const Step *__restrict__ steps, const i64 *__restrict__ start,
                 const int *__restrict__ level, int nlev, unsigned *bar,
                 int *err, int max_B, size_t max_tile, long long wait_limit) {
  extern __shared__ __align__(128) unsigned char fm_smem[];
  const int tid = threadIdx.x, T = blockDim.x;
  Step *const sst = reinterpret_cast<Step *>(fm_smem);
  unsigned char *const h = fm_smem + batch_steps_bytes();
  i64 *sq = reinterpret_cast<i64 *>(h);
  // slot k: launch record, per-vector records, exponents and tile buffer
  // (addresses recomputed on use to keep registers free)
  const unsigned rec = (unsigned)((sizeof(VInfo) + 4) * max_B);
  auto vis = [&](int k) {
    return reinterpret_cast<VInfo *>(h + 8 * max_B + k * rec);
  };
  auto sexps = [&](int k) {
    return reinterpret_cast<int *>(h + 8 * max_B + k * rec +
                                   sizeof(VInfo) * max_B);
  };
  auto bufs = [&](int k) {
    return reinterpret_cast<E *>(fm_smem + batch_head_bytes(max_B) +
                                 k * max_tile);
  };
  const i64 G = gridDim.x;
  for (int l = 0; l < nlev; ++l) {
    const int s0 = level[l], s1 = level[l + 1];
    const i64 t1 = start[s1];
    // two-slot pipeline: the loads of tile g + G are issued before tile g
    // is transformed and stored
    i64 g = start[s0] + blockIdx.x;
    int kc = s0, cur = 0;
    if (g < t1) {
      while (start[kc + 1] <= g) ++kc;
      batch_issue_load<E>(steps + kc, sst, bufs(0), vis(0), g - start[kc],
                          tid, T);
    }
    for (; g < t1; g += G) {
      const i64 gn = g + G;
      int kn = kc;
      if (gn < t1) {
        while (start[kn + 1] <= gn) ++kn;
        batch_issue_load<E>(steps + kn, sst + (cur ^ 1), bufs(cur ^ 1),
                            vis(cur ^ 1), gn - start[kn], tid, T);
        cp_async_wait<1>();
      } else {
        cp_async_wait<0>();
      }
      __syncthreads();
      const Step &p = sst[cur];
      E *sm = bufs(cur);
      VInfo *vi = vis(cur);
      int *sexp = sexps(cur);
      const bool async = p.src_type == Tr<E>::code && !p.map_in;
      if constexpr (Emu<E>::v) {
        if (async) {
          emu_in<E, 0>(p, sm, vi, sexp, tid, T);
        } else {
          for (int b = tid; b < p.B; b += T) sexp[b] = 0;
        }
        __syncthreads();
      }
      if (async && (p.conj_in || p.pre)) {
        load_fixup<E, 0>(p, sm, vi, tid, T);
        __syncthreads();
      }
      const int nwarps = T >> 5;
      bool natural = false, stored = false;
      if constexpr (std::is_same<E, float2>::value) {
        if (p.rprog) {
          // the program on registers; results in natural order (or already
          // stored)
          rt_program(p, sm, vi, tid, T);
          natural = true;
          stored = (p.rprog & RT_DIRECT) != 0;
        }
      }
      if (natural) {
      } else if (warp_mode<E, CLS, 0>(p.B, p.L, nwarps)) {
        const int w = tid >> 5, vw = p.B / nwarps;
        run_program<E, CLS, 0>(p, sm + w * vw * p.Lp, p.Lp, vw, vi + w * vw,
                               sq + w * vw, tid & 31, 32);
        __syncthreads();
      } else {
        run_program<E, CLS, 0>(p, sm, p.Lp, p.B, vi, sq, tid, T);
      }
      if (!stored) store_tile<E, 0>(p, sm, vi, sexp, tid, T, natural);
      __syncthreads();
      cur ^= 1;
      kc = kn;
    }
    if (l + 1 < nlev &&
        !grid_barrier(bar, (unsigned)(l + 1) * gridDim.x, err, wait_limit))
      return;
  }
}

}  // namespace fmk
