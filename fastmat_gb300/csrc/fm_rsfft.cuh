// Register-resident FFT of strided complex vectors: a Fourier factor of a
// Kron applied mode-wise (fastmat/Kron.pyx:284-300 with the transform of
// fastmat/Fourier.pyx), i.e. vectors of L points at an element stride S
// that is a multiple of 32, adjacent vectors adjacent in memory.
//
//   * the lanes take NV adjacent vectors (NV = 32, or fewer for long
//     vectors: NV G <= 256 threads), so each load and store of a warp covers
//     contiguous row segments of 128 bytes or more;
//   * vector v's L points are held by G = L / P threads (P = 16 complex64 or
//     8 double-float complex per thread), thread t of the vector holding
//     points t + G r, exactly the natural-order layout of the register
//     convolution (fm_rconv.cuh), whose radix stages run here unchanged:
//     the in-place DIF over the radices (P, P, ..., rest), twiddles from
//     lane-major tables in shared memory, exchanges between the stages
//     through a buffer per vector (odd stride: the lanes of each wavefront
//     on distinct banks; CTA barriers, the threads of a vector sit in
//     different warps);
//   * the results leave in natural order: each register's digit-reversed
//     position is mapped back at compile time, and the store of a point
//     goes to its row for all NV vectors at once.
// Double-float vectors are scaled by the power of two of their largest
// exponent on the way in (float's exponent range) and back on the way out.
#pragma once

#include "fm_rconv.cuh"

namespace fmk {

struct RsfStep {
  const void *src;
  void *dst;
  i64 ld_src, ld_dst;
  i64 A;   // vectors per column (a S + c: block a, offset c < S)
  i64 es;  // element stride S
  i64 num_cols;
  const void *tw;  // tw[j] = exp(-2 pi i j / L), j < L
  int *err;
  int L;
  int sign;  // -1 forward, +1 inverse (unscaled)
};

#define FM_RSF_THREADS 256
template <class E, int L> struct RsfShape {
  static constexpr int P = RcLane<E>::P;
  static constexpr int G = L / P;  // threads per vector
  static constexpr int NV = FM_RSF_THREADS / G > 32 ? 32
                                                    : FM_RSF_THREADS / G;
  static constexpr int T = NV * G;
  static constexpr int Lx = (L + (L >> RcBuf<E, L>::SH)) | 1;
};
template <class E> struct RsfOcc {
  static constexpr int v = sizeof(E) == 8 ? 3 : 2;
};
template <class E, int L>
__host__ __device__ constexpr size_t rsf_smem() {
  return (size_t)(rc_twlen<E, L, rc_stages(L, RcLane<E>::P)>() +
                  RsfShape<E, L>::NV * RsfShape<E, L>::Lx) *
             sizeof(E) +
         32 * sizeof(int);
}

template <class E, int L, int SG>
__global__ void __launch_bounds__(RsfShape<E, L>::T, (RsfOcc<E>::v))
    rsfft_kernel(const __grid_constant__ RsfStep p) {
  typedef RsfShape<E, L> Sh;
  constexpr int P = Sh::P, G = Sh::G, NV = Sh::NV;
  constexpr int S = rc_stages(L, P);
  static_assert(G >= 2 && NV >= 1 && NV <= 32, "vector layout");
  typedef typename std::conditional<Emu<E>::v, double2, E>::type Raw;
  extern __shared__ __align__(128) unsigned char fm_smem[];
  constexpr int TWN = rc_twlen<E, L, S>();
  E *stw = reinterpret_cast<E *>(fm_smem);
  E *xb = stw + TWN;
  int *sexp = reinterpret_cast<int *>(xb + NV * Sh::Lx);
  rc_fill_tw<E, L, 0>(stw, (const E *)p.tw);
  __syncthreads();
  const int v = threadIdx.x % NV, t = threadIdx.x / NV;
  E *buf = xb + v * Sh::Lx;
  const i64 Sx = p.es;
  const i64 nb = p.A * p.num_cols / NV;  // batches of NV adjacent vectors
  const FDiv dA((unsigned)p.A), dS((unsigned)Sx);
  for (i64 bt = blockIdx.x; bt < nb; bt += gridDim.x) {
    const unsigned gv = (unsigned)(bt * NV);
    const unsigned m = dA.div(gv), v0 = gv - m * (unsigned)p.A;
    const unsigned a = dS.div(v0), c0 = v0 - a * (unsigned)Sx;
    const i64 row0 = (i64)a * L * Sx + c0 + v;
    const Raw *src = (const Raw *)p.src + (i64)m * p.ld_src + row0;
    Raw d[P];
#pragma unroll
    for (int r = 0; r < P; ++r) d[r] = src[(i64)(t + G * r) * Sx];
    E x[P];
    int s = 0;
    if constexpr (Emu<E>::v) {
      int emax = 0;
#pragma unroll
      for (int r = 0; r < P; ++r)
        emax = max(emax, max(dexp(d[r].x), dexp(d[r].y)));
      if (threadIdx.x < NV) sexp[threadIdx.x] = 0;
      __syncthreads();
      if (emax > 0) atomicMax(sexp + v, emax);
      __syncthreads();
      s = sexp[v] > 0 ? sexp[v] - 1023 : 0;
#pragma unroll
      for (int r = 0; r < P; ++r)
        x[r] = dfc{d2df_scaled(d[r].x, s), d2df_scaled(d[r].y, s)};
    } else {
#pragma unroll
      for (int r = 0; r < P; ++r) x[r] = d[r];
    }
    // (S >= 2: the stages hold at least one exchange, whose barriers also
    // separate this batch's reads of sexp from the next batch's reset)
    rc_forward<E, L, 0, SG, true>(x, buf, t, stw);
    Raw *dst = (Raw *)p.dst + (i64)m * p.ld_dst + row0;
    const int bl = rc_base<E, L, S - 1>(t);
#pragma unroll
    for (int j = 0; j < P; ++j) {
      const int nat = rc_nat<E, L>(bl + rc_off<E, L, S - 1>(j));
      if constexpr (Emu<E>::v)
        dst[(i64)nat * Sx] = make_double2(df2d_scaled(x[j].x, s),
                                          df2d_scaled(x[j].y, s));
      else
        dst[(i64)nat * Sx] = x[j];
    }
  }
}

}  // namespace fmk
