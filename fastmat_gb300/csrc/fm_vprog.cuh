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
  OP_TW = 9       // v[j] *= exp(sign 2 pi i ((q * j) mod N) / N), j < len
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
  i64 div, mod, stride;   // q = (v / div) % mod for MUL / TW
  i64 N;
  double sre, sim;
};

struct View {
  i64 A, n, Cc;
};

struct Step {
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
  int conj_in, conj_out, accumulate, has_scale;
  double scale_re, scale_im;
  int L, Lp, B;
  int in_len, out_len;
  i64 V;         // vectors per column
  i64 num_cols;
  int nops;
  int pad_;
  Op ops[FM_MAX_OPS];
};

// elements each thread holds in registers per pass
// (a launch uses at most FM_MAX_THREADS threads, so a tile holds at most
// FM_MAX_THREADS * Ept elements)
#define FM_MAX_THREADS 512
template <class E> struct Ept {
  static constexpr int v = sizeof(E) >= 16 ? 8 : 16;
};

// ------------------------------------------------------------ small DFTs
// y_k = sum_r x_r exp(sign * 2 pi i r k / R), in place.
template <class C> __device__ __forceinline__ C rot90(C a, int sign) {
  // a * (i * sign)
  C r;
  r.x = -sign * a.y;
  r.y = sign * a.x;
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
  t.x = h * (b[1].x - sign * b[1].y);
  t.y = h * (b[1].y + sign * b[1].x);
  b[1] = t;
  b[2] = rot90(b[2], sign);
  t.x = h * (-b[3].x - sign * b[3].y);
  t.y = h * (-b[3].y + sign * b[3].x);
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
    const R c = cs[k], s = sign * sn[k];
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
  const R c = (R)-0.5, s = (R)(sign * 0.8660254037844386);
  C t = v[1] + v[2], d = v[1] - v[2];
  C y0 = v[0] + t;
  C m;
  m.x = v[0].x + c * t.x;
  m.y = v[0].y + c * t.y;
  C r;
  r.x = -s * d.y;
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
  const typename Tr<C>::R sb = plus ? sign : -sign;
  r.x = a.x - sb * b.y;
  r.y = a.y + sb * b.x;
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

// ------------------------------------------------------------ FFT pass
// One Stockham autosort pass of radix R over all B vectors of the tile
// (decimation in time; output of the last pass is in natural order).
template <int R, class C>
__device__ __forceinline__ void fft_pass(C *sm, int Lp, int B, int Lf, int Ns,
                                         int sign, const C *__restrict__ tw,
                                         int tid, int T) {
  // odd radices hold half as many elements per thread (the planner gives
  // programs with odd radices twice the threads)
  constexpr int EP = (R & 1) ? Ept<C>::v / 2 : Ept<C>::v;
  constexpr int MB = (EP + R - 1) / R;
  const int nb = Lf / R;
  const int total = B * nb;
  C v[MB][R];
#pragma unroll
  for (int i = 0; i < MB; ++i) {
    const int g = tid + i * T;
    if (g < total) {
      const int b = g / nb, q = g - b * nb;
      const C *vec = sm + b * Lp;
#pragma unroll
      for (int r = 0; r < R; ++r) v[i][r] = vec[pidx<C>(q + r * nb)];
    }
  }
  __syncthreads();
  const int tstep = Lf / (Ns * R);
#pragma unroll
  for (int i = 0; i < MB; ++i) {
    const int g = tid + i * T;
    if (g < total) {
      const int b = g / nb, q = g - b * nb;
      const int k = q % Ns;
      if (Ns > 1) {
#pragma unroll
        for (int r = 1; r < R; ++r) {
          const C w = tw[r * k * tstep];
          v[i][r] = sign < 0 ? cmul(v[i][r], w) : cmulc(v[i][r], w);
        }
      }
      dft<R>(v[i], sign);
      C *vec = sm + b * Lp;
      const int base = (q - k) * R + k;
#pragma unroll
      for (int r = 0; r < R; ++r) vec[pidx<C>(base + r * Ns)] = v[i][r];
    }
  }
  __syncthreads();
}

template <class C, int CLS>
__device__ void run_fft(const Op &op, C *sm, int Lp, int B, int tid, int T) {
  const C *tw = (const C *)op.ptr;
  int Ns = 1;
  for (int p = 0; p < op.nrad; ++p) {
    const int R = op.rad[p];
    switch (R) {
      case 2: fft_pass<2>(sm, Lp, B, op.len, Ns, op.sign, tw, tid, T); break;
      case 3: if constexpr (CLS != 1) fft_pass<3>(sm, Lp, B, op.len, Ns, op.sign, tw, tid, T); break;
      case 4: fft_pass<4>(sm, Lp, B, op.len, Ns, op.sign, tw, tid, T); break;
      case 5: if constexpr (CLS != 1) fft_pass<5>(sm, Lp, B, op.len, Ns, op.sign, tw, tid, T); break;
      case 7: if constexpr (CLS != 1) fft_pass<7>(sm, Lp, B, op.len, Ns, op.sign, tw, tid, T); break;
      case 8: fft_pass<8>(sm, Lp, B, op.len, Ns, op.sign, tw, tid, T); break;
      default:
        if constexpr (Ept<C>::v >= 16)
          fft_pass<16>(sm, Lp, B, op.len, Ns, op.sign, tw, tid, T);
        break;
    }
    Ns *= R;
  }
}

// ------------------------------------------------------------ FWHT pass
// In-place butterflies over the bit group [s, s + K) of every element index.
template <int K, class E>
__device__ __forceinline__ void fwht_pass(E *sm, int Lp, int B, int Lf, int s,
                                          int tid, int T) {
  constexpr int R = 1 << K;
  constexpr int MB = (Ept<E>::v + R - 1) / R;
  const int nb = Lf >> K;
  const int total = B * nb;
  const int lomask = (1 << s) - 1;
#pragma unroll
  for (int i = 0; i < MB; ++i) {
    const int g = tid + i * T;
    if (g < total) {
      const int b = g / nb, q = g - b * nb;
      const int base = ((q >> s) << (s + K)) | (q & lomask);
      E *vec = sm + b * Lp;
      E v[R];
#pragma unroll
      for (int r = 0; r < R; ++r) v[r] = vec[pidx<E>(base + (r << s))];
#pragma unroll
      for (int h = 1; h < R; h <<= 1) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
          if ((r & h) == 0) {
            const E a = v[r], c = v[r + h];
            v[r] = addv(a, c);
            v[r + h] = subv(a, c);
          }
        }
      }
#pragma unroll
      for (int r = 0; r < R; ++r) vec[pidx<E>(base + (r << s))] = v[r];
    }
  }
  __syncthreads();
}

template <class E>
__device__ void run_fwht(const Op &op, E *sm, int Lp, int B, int tid, int T) {
  int s = 0;
  for (int p = 0; p < op.nrad; ++p) {
    const int K = op.rad[p];
    switch (K) {
      case 1: fwht_pass<1>(sm, Lp, B, op.len, s, tid, T); break;
      case 2: fwht_pass<2>(sm, Lp, B, op.len, s, tid, T); break;
      case 3: fwht_pass<3>(sm, Lp, B, op.len, s, tid, T); break;
      default:
        if constexpr (Ept<E>::v >= 16) fwht_pass<4>(sm, Lp, B, op.len, s, tid, T);
        break;
    }
    s += K;
  }
}

// ------------------------------------------------------------ other ops
template <class E>
__device__ void run_gather(const Op &op, E *sm, int Lp, int B, int tid,
                           int T) {
  constexpr int MB = Ept<E>::v;
  const i64 *map = (const i64 *)op.ptr;
  const int total = B * op.len;
  E v[MB];
#pragma unroll
  for (int i = 0; i < MB; ++i) {
    const int f = tid + i * T;
    if (f < total) {
      const int b = f / op.len, j = f - b * op.len;
      const i64 src = map[j];
      v[i] = src < 0 ? zero<E>() : sm[b * Lp + pidx<E>((int)src)];
    }
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < MB; ++i) {
    const int f = tid + i * T;
    if (f < total) {
      const int b = f / op.len, j = f - b * op.len;
      sm[b * Lp + pidx<E>(j)] = v[i];
    }
  }
  __syncthreads();
}

template <class E>
__device__ void run_dense(const Op &op, E *sm, int Lp, int B, int tid,
                          int T) {
  constexpr int MB = Ept<E>::v;
  const E *M = (const E *)op.ptr;
  const int rows = op.len, cols = op.len2;
  const int total = B * rows;
  E v[MB];
#pragma unroll
  for (int i = 0; i < MB; ++i) {
    const int f = tid + i * T;
    if (f < total) {
      const int b = f / rows, r = f - b * rows;
      const E *vec = sm + b * Lp;
      E acc = zero<E>();
      for (int j = 0; j < cols; ++j)
        acc = addv(acc, mulv(M[r + (i64)j * rows], vec[pidx<E>(j)], false));
      v[i] = acc;
    }
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < MB; ++i) {
    const int f = tid + i * T;
    if (f < total) {
      const int b = f / rows, r = f - b * rows;
      sm[b * Lp + pidx<E>(r)] = v[i];
    }
  }
  __syncthreads();
}

template <class E>
__device__ void run_elementwise(const Op &op, E *sm, int Lp, int B, i64 gv0,
                                i64 V, int tid, int T) {
  const int len = op.len;
  const int total = B * len;
  for (int f = tid; f < total; f += T) {
    const int b = f / len, j = f - b * len;
    E *e = sm + b * Lp + pidx<E>(j);
    switch (op.kind) {
      case OP_MUL: {
        const i64 v = (gv0 + b) % V;
        const i64 q = (v / op.div) % op.mod;
        const E m = ((const E *)op.ptr)[q * op.stride + j];
        *e = mulv(*e, m, op.sign != 0);
        break;
      }
      case OP_SCALE: *e = scalev(*e, op.sre, op.sim); break;
      case OP_CONJ: *e = conjv(*e); break;
      case OP_TW: {
        if constexpr (Tr<E>::cplx) {
          const i64 v = (gv0 + b) % V;
          const i64 q = (v / op.div) % op.mod;
          const i64 t = (q * (i64)j) % op.N;
          const E w = ((const E *)op.ptr)[t];
          *e = op.sign < 0 ? cmul(*e, w) : cmulc(*e, w);
        }
        break;
      }
      default: break;
    }
  }
  __syncthreads();
}

template <class E>
__device__ void run_zpad(const Op &op, E *sm, int Lp, int B, int tid, int T) {
  const int cnt = op.len2 - op.len;
  const int total = B * cnt;
  for (int f = tid; f < total; f += T) {
    const int b = f / cnt, j = op.len + (f - b * cnt);
    sm[b * Lp + pidx<E>(j)] = zero<E>();
  }
  __syncthreads();
}

// ------------------------------------------------------------ the kernel
// CLS selects the op subset compiled into an instantiation, so the hot
// programs (power-of-two FFT, FWHT) do not carry the register pressure of
// the rarely used ops: 1 = pow2 FFT + pointwise, 2 = FFT with radices 3/5/7,
// 3 = FWHT + pointwise, 0 = everything.
template <class E, int CLS>
__global__ void __launch_bounds__(FM_MAX_THREADS)
    vprog_kernel(const __grid_constant__ Step p) {
  extern __shared__ __align__(16) unsigned char fm_smem[];
  E *sm = reinterpret_cast<E *>(fm_smem);
  const int tid = threadIdx.x, T = blockDim.x;
  const int B = p.B, L = p.L, Lp = p.Lp;
  const i64 gv0 = (i64)blockIdx.x * B;
  const i64 nvec = p.V * p.num_cols;

  // ---- load: tile of B vectors, converted to E, zero padded to L
  {
    const bool strided = p.vin.Cc > 1;
    const int total = B * L;
    for (int f = tid; f < total; f += T) {
      int b, j;
      if (strided) {
        j = f / B;
        b = f - j * B;
      } else {
        b = f / L;
        j = f - b * L;
      }
      const i64 gv = gv0 + b;
      E val = zero<E>();
      if (gv < nvec && j < p.in_len) {
        const i64 m = gv / p.V, v = gv - m * p.V;
        const i64 a = v / p.vin.Cc, c = v - a * p.vin.Cc;
        const i64 r = (a * p.vin.n + j) * p.vin.Cc + c;
        if (r < p.in_rows) {
          const i64 srow = p.map_in ? p.map_in[r] : r;
          if (srow >= 0) {
            val = load_as<E>(p.src, p.src_type, m * p.ld_src + srow);
            if (p.conj_in) val = conjv(val);
            if (p.pre) val = mulv(val, ((const E *)p.pre)[r], false);
          }
        }
      }
      sm[b * Lp + pidx<E>(j)] = val;
    }
  }
  __syncthreads();

  // ---- program
  for (int o = 0; o < p.nops; ++o) {
    const Op &op = p.ops[o];
    switch (op.kind) {
      case OP_FFT:
        if constexpr (Tr<E>::cplx && CLS != 3) run_fft<E, CLS>(op, sm, Lp, B, tid, T);
        break;
      case OP_FWHT:
        if constexpr (CLS == 0 || CLS == 3) run_fwht<E>(op, sm, Lp, B, tid, T);
        break;
      case OP_GATHER:
        if constexpr (CLS == 0) run_gather<E>(op, sm, Lp, B, tid, T);
        break;
      case OP_DENSE:
        if constexpr (CLS == 0) run_dense<E>(op, sm, Lp, B, tid, T);
        break;
      case OP_ZPAD: run_zpad<E>(op, sm, Lp, B, tid, T); break;
      default: run_elementwise<E>(op, sm, Lp, B, gv0, p.V, tid, T); break;
    }
  }

  // ---- store
  const bool acc = p.accumulate != 0;
  if (p.out_mode == 1) {
    // gather: out row i of column m takes vector element map_out[i]
    for (int f = tid; f < B * p.n_out; f += T) {
      const int b = f / p.n_out, i = f - b * p.n_out;
      const i64 gv = gv0 + b;
      if (gv >= nvec) continue;
      const i64 m = gv / p.V;
      const i64 j = p.map_out[i];
      E val = j < 0 ? zero<E>() : sm[b * Lp + pidx<E>((int)j)];
      if (j >= 0 && p.post) val = mulv(val, ((const E *)p.post)[j], false);
      if (p.has_scale) val = scalev(val, p.scale_re, p.scale_im);
      if (p.conj_out) val = conjv(val);
      store_as<E>(p.dst, p.dst_type, m * p.ld_dst + i, val, acc);
    }
    return;
  }
  const bool strided = p.vout.Cc > 1;
  const int total = B * p.out_len;
  for (int f = tid; f < total; f += T) {
    int b, j;
    if (strided) {
      j = f / B;
      b = f - j * B;
    } else {
      b = f / p.out_len;
      j = f - b * p.out_len;
    }
    const i64 gv = gv0 + b;
    if (gv >= nvec) continue;
    const i64 m = gv / p.V, v = gv - m * p.V;
    const i64 a = v / p.vout.Cc, c = v - a * p.vout.Cc;
    const i64 r = (a * p.vout.n + j) * p.vout.Cc + c;
    if (r >= p.out_rows) continue;
    const i64 drow = p.out_mode == 2 ? p.map_out[r] : r;
    if (drow < 0) continue;
    E val = sm[b * Lp + pidx<E>(j)];
    if (p.post) val = mulv(val, ((const E *)p.post)[r], false);
    if (p.has_scale) val = scalev(val, p.scale_re, p.scale_im);
    if (p.conj_out) val = conjv(val);
    store_as<E>(p.dst, p.dst_type, m * p.ld_dst + drow, val, acc);
  }
}

}  // namespace fmk
