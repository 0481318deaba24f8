// Planner and C ABI of the matvec engine.
//
// fm_plan_create lowers an operator tree (fm_node array, see fmgpu.h) into a
// list of vector-program launches per direction:
//   * every operator whose working vector fits in shared memory becomes a
//     straight-line program over whole columns (Fourier: Stockham FFT;
//     Circulant/Toeplitz: zero pad, FFT, spectrum multiply, inverse FFT,
//     truncate; Bluestein Fourier: chirp, convolution, chirp; Hadamard: FWHT;
//     Diag: multiply; Partial/Permutation: gathers), and adjacent programs
//     of a Product chain are merged into one launch;
//   * long transforms use the four-step decomposition N = N1 * N2 as two
//     (FFT) or three (convolution) launches over strided views;
//   * Kron applies each factor's program along its mode, in place;
//   * Sum accumulates its terms into the output.
// Device constants (twiddles, spectra, chirps, index maps) are computed on
// the GPU in double precision and stored in the plan's compute type.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <atomic>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/fmgpu.h"
#include "fm_launch.cuh"

#include <cuda.h>

using fmk::i64;
typedef std::complex<double> cd;

namespace {

thread_local std::string g_err;

struct Error {
  int code;
  std::string msg;
};

[[noreturn]] void fail(int code, const std::string &m) { throw Error{code, m}; }

#define CUDA_TRY(x)                                                         \
  do {                                                                      \
    cudaError_t e_ = (x);                                                   \
    if (e_ != cudaSuccess)                                                  \
      fail(e_ == cudaErrorMemoryAllocation ? FM_ERR_NOMEM : FM_ERR_CUDA,    \
           std::string(#x) + ": " + cudaGetErrorString(e_));                \
  } while (0)

// One-shot allocation failure for tests of the out-of-memory path
// (fm_debug_fail_allocation): after g_alloc_skip more successful device
// allocations the next one fails as if the device were full; -1 = disarmed.
std::atomic<long long> g_alloc_skip{-1};

template <class T> cudaError_t dev_malloc(T **p, size_t bytes) {
  long long k = g_alloc_skip.load();
  while (k >= 0) {
    if (g_alloc_skip.compare_exchange_weak(k, k - 1)) {
      if (k == 0) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
      }
      break;
    }
  }
  return cudaMalloc((void **)p, bytes);
}

// a device buffer freed when it goes out of scope (planner temporaries)
struct DevTemp {
  void *p = nullptr;
  DevTemp() = default;
  DevTemp(const DevTemp &) = delete;
  DevTemp &operator=(const DevTemp &) = delete;
  ~DevTemp() {
    if (p) cudaFree(p);
  }
};

int esize(int t) {
  switch (t) {
    case FM_F64_DF: return 8;
    case FM_C128_DF: return 16;
    case FM_F32_TC: return 4;
    case FM_I8: return 1;
    case FM_I16: return 2;
    case FM_I32: return 4;
    case FM_I64: return 8;
    case FM_F32: return 4;
    case FM_F64: return 8;
    case FM_C64: return 8;
    case FM_C128: return 16;
    default: return 0;
  }
}
bool is_cplx(int t) {
  return t == FM_C64 || t == FM_C128 || t == FM_C128_DF;
}
// element type of the buffers a plan of compute type t reads and writes
int io_of(int t) {
  return t == FM_F64_DF    ? FM_F64
         : t == FM_C128_DF ? FM_C128
         : t == FM_F32_TC  ? FM_F32
                           : t;
}
bool valid_type(int t) { return t >= FM_I8 && t <= FM_C128; }

cd host_get(const void *p, int t, i64 i) {
  switch (t) {
    case FM_I8: return cd(((const int8_t *)p)[i], 0);
    case FM_I16: return cd(((const int16_t *)p)[i], 0);
    case FM_I32: return cd(((const int32_t *)p)[i], 0);
    case FM_I64: return cd((double)((const int64_t *)p)[i], 0);
    case FM_F32: return cd(((const float *)p)[i], 0);
    case FM_F64: return cd(((const double *)p)[i], 0);
    case FM_C64: {
      const float *f = (const float *)p + 2 * i;
      return cd(f[0], f[1]);
    }
    case FM_C128: {
      const double *f = (const double *)p + 2 * i;
      return cd(f[0], f[1]);
    }
  }
  fail(FM_ERR_TYPE, "unsupported element type");
}

i64 host_get_int(const void *p, int t, i64 i) {
  switch (t) {
    case FM_I8: return ((const int8_t *)p)[i];
    case FM_I16: return ((const int16_t *)p)[i];
    case FM_I32: return ((const int32_t *)p)[i];
    case FM_I64: return ((const int64_t *)p)[i];
    default: return (i64)host_get(p, t, i).real();
  }
}

bool smooth(i64 n) {
  if (n < 1) return false;
  for (int p : {2, 3, 5, 7})
    while (n % p == 0) n /= p;
  return n == 1;
}
i64 next_pow2(i64 n) {
  i64 p = 1;
  while (p < n) p <<= 1;
  return p;
}
bool is_pow2(i64 n) { return n > 0 && (n & (n - 1)) == 0; }

// ------------------------------------------------------------ helper kernels
template <class E> __device__ E mk(double re, double im);
template <> __device__ float mk<float>(double re, double) { return (float)re; }
template <> __device__ double mk<double>(double re, double) { return re; }
template <> __device__ i64 mk<i64>(double re, double) { return (i64)llrint(re); }
template <> __device__ float2 mk<float2>(double re, double im) {
  return make_float2((float)re, (float)im);
}
template <> __device__ double2 mk<double2>(double re, double im) {
  return make_double2(re, im);
}
template <> __device__ fmk::df mk<fmk::df>(double re, double) {
  return fmk::d2df(re);
}
template <> __device__ fmk::dfc mk<fmk::dfc>(double re, double im) {
  return fmk::dfc{fmk::d2df(re), fmk::d2df(im)};
}

// tw[t] = exp(-2 pi i t / N); the phase t/N is exact in integers and the
// only rounding is in double-precision sincospi.
template <class E>
__global__ void k_twiddle(E *tw, i64 N) {
  for (i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x; t < N;
       t += (i64)gridDim.x * blockDim.x) {
    double s, c;
    sincospi(-2.0 * (double)t / (double)N, &s, &c);
    tw[t] = mk<E>(c, s);
  }
}

// Two-level twiddle table of length-N transforms: w^e = T1[e >> s] T0[e & (2^s - 1)],
// T0[j] = w^j (j < 2^s) at tw[j], T1[m] = w^(m 2^s) (m <= (N - 1) >> s) at
// tw[2^s + m], w = exp(-2 pi i / N); both factors small enough to stay in
// the L1 cache.
template <class E>
__global__ void k_twiddle2(E *tw, i64 N, int s) {
  const i64 n0 = 1LL << s, n1 = ((N - 1) >> s) + 1;
  for (i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x; t < n0 + n1;
       t += (i64)gridDim.x * blockDim.x) {
    const i64 e = t < n0 ? t : (t - n0) << s;
    double sn, c;
    sincospi(-2.0 * (double)e / (double)N, &sn, &c);
    tw[t] = mk<E>(c, sn);
  }
}

// Bluestein chirp a[n] = exp(-i pi n^2 / N) with n^2 reduced mod 2N exactly
__global__ void k_chirp(double2 *a, i64 N) {
  for (i64 n = blockIdx.x * (i64)blockDim.x + threadIdx.x; n < N;
       n += (i64)gridDim.x * blockDim.x) {
    const i64 m = (n * n) % (2 * N);
    double s, c;
    sincospi(-(double)m / (double)N, &s, &c);
    a[n] = make_double2(c, s);
  }
}

// Bluestein filter h[m] = conj(a[|m|]) on the circle of length Lb
__global__ void k_bluestein_filter(double2 *h, const double2 *a, i64 N,
                                   i64 Lb) {
  for (i64 m = blockIdx.x * (i64)blockDim.x + threadIdx.x; m < Lb;
       m += (i64)gridDim.x * blockDim.x) {
    double2 v = make_double2(0., 0.);
    if (m < N) v = make_double2(a[m].x, -a[m].y);
    else if (Lb - m < N) v = make_double2(a[Lb - m].x, -a[Lb - m].y);
    h[m] = v;
  }
}

// out[o] = scale * in[perm(o)] converted to E; perm for the four-step
// layout: o = k1 * L2 + k2  <-  k1 + L1 * k2   (L1 == 0: identity)
template <class E>
__global__ void k_convert(E *out, const double2 *in, i64 n, double scale,
                          i64 L1, i64 L2) {
  for (i64 o = blockIdx.x * (i64)blockDim.x + threadIdx.x; o < n;
       o += (i64)gridDim.x * blockDim.x) {
    i64 src = o;
    if (L1 > 0) {
      const i64 k1 = o / L2, k2 = o - k1 * L2;
      src = k1 + L1 * k2;
    }
    const double2 v = in[src];
    out[o] = mk<E>(v.x * scale, v.y * scale);
  }
}

int grid_for(i64 n) { return (int)std::min<i64>((n + 255) / 256, 4096); }

// ------------------------------------------------------------ plan state
struct LStep {
  fmk::Step st;
  int src, dst;  // 0 = x, 1 = y, >= 2 scratch
  // first row of the launch's operand inside its buffer (Blocks segments)
  i64 src_off = 0, dst_off = 0;
  // 0: vector program (vprog_kernel); 1: CSR sparse product (spmv_kernel);
  // 2: register-resident convolution (rconv_kernel), 3: register-resident
  // FWHT (rfwht_kernel / rsfwht_kernel / rfwht2_kernel), 4: register FFT of
  // strided vectors (rsfft_kernel); for 2..4 `st` still holds the
  // equivalent vector program (run by batches, and when the buffers do not
  // suit the register kernel)
  int kind = 0;
  int rc_L = 0;
  // kind 3: the real type the FWHT kernel runs in (complex data as pairs
  // of real vectors), and for strided vectors their element stride and
  // count per column in real words (rc_es 0: contiguous kernel); kind 4:
  // the same stride and count in elements
  int rc_ct = 0;
  i64 rc_es = 0, rc_A = 0;
  // two-pass FWHT run as one launch (rfwht2_kernel): 1 on the contiguous
  // pass, which then also runs the strided pass that follows it (its length,
  // element stride and vectors per column in rc2_*), 2 on that strided pass
  int pair = 0;
  int rc2_L = 0;
  int rc_sign = 0;  // kind 4: transform sign
  i64 rc2_es = 0, rc2_A = 0;
  // pair 3: a circulant mode (this step, kind 2) and the strided FWHT mode
  // after it in one launch (rkch_kernel): FWHT blocks per column, items
  int rc2_blocks = 0, rc2_n1 = 0, rc2_n2 = 0;
  const void *rc_spec = nullptr, *rc_tw = nullptr;  // spectrum in rconv order
  const void *rc_pre = nullptr, *rc_post = nullptr;
  int rc_conj_in = 0, rc_conj_out = 0, rc_spec_conj = 0;
  const i64 *sp_ptr = nullptr, *sp_idx = nullptr;
  const void *sp_val = nullptr;
  i64 sp_rows = 0;
  int sp_group = 32;
  int cls = 0, threads = 0;
  size_t smem = 0;
  int lay = 0;                     // tile layout (1: element-major)
  int ept = 8;                     // elements per thread of its class
  int tma_in_ok = 0, tma_out_ok = 0;  // views allow TMA boxes
  // last encoded tensor maps and the (address, ld, columns) they describe
  const void *tm_in_key = nullptr, *tm_out_key = nullptr;
  i64 tm_in_ld = -1, tm_out_ld = -1, tm_in_m = -1, tm_out_m = -1;
  CUtensorMap tm_in, tm_out;
};

}  // namespace

struct fm_plan {
  int ctype = FM_C128;  // compute type (FM_* or FM_*_DF)
  int io_type = FM_C128;  // element type of scratch buffers
  int esz = 16;
  int device = 0;
  i64 rows = 0, cols = 0;
  std::vector<void *> allocs;
  i64 const_bytes = 0;
  std::map<i64, void *> twiddles;
  std::vector<LStep> steps[2];
  std::vector<i64> scratch_rows;  // rows per scratch buffer (id - 2)
  // execution state
  void *scratch = nullptr;
  size_t scratch_cap = 0;
  int *err = nullptr;  // device status word written by bounded waits
  long long wait_limit = FM_WAIT_LIMIT;  // polls of a bounded copy wait
  // counters of the fused two-pass FWHT (1 + columns), allocated with the
  // plan; pair_done: the last launch ran a pair, so its second pass is done
  unsigned *pair_ctr = nullptr;
  i64 pair_cap = 0;  // counters in pair_ctr
  bool pair_done = false;
  bool no_pair = false;  // run pairs as separate launches (host pipeline)
  ~fm_plan();
};

fm_plan::~fm_plan() {
  for (void *p : allocs) cudaFree(p);
  if (scratch) cudaFree(scratch);
}

struct fm_batch {
  int device = 0;
  std::vector<void *> allocs;
  fmk::BatchLaunch launch;
  i64 num_steps = 0, total_tiles = 0;
  int *status = nullptr;  // [0] grid-barrier counter, [1] error word
  cudaStream_t gstream = nullptr;
  cudaGraphExec_t exec = nullptr;
  ~fm_batch();
};

fm_batch::~fm_batch() {
  if (exec) cudaGraphExecDestroy(exec);
  if (gstream) cudaStreamDestroy(gstream);
  for (void *p : allocs) cudaFree(p);
}

namespace {

int run_plan(fm_plan *P, int dir, const void *x, int x_type, i64 ld_x,
             void *y, int y_type, i64 ld_y, i64 M, cudaStream_t s,
             std::vector<cudaEvent_t> *events = nullptr);

// ------------------------------------------------------------ planner IR
struct SStep {
  fmk::View vin{1, 1, 1}, vout{1, 1, 1};
  i64 in_rows = 0, out_rows = 0;
  int L = 0, in_len = 0, out_len = 0;
  std::vector<fmk::Op> ops;
  int src = -1, dst = -2;  // -1 unit input, -2 unit output, k >= 0 temp k
  const void *pre = nullptr, *post = nullptr;
  const i64 *map_in = nullptr, *map_out = nullptr;  // gather / scatter
  int out_mode = 0;
  int conj_in = 0, conj_out = 0;
};

struct Unit;
typedef std::vector<Unit> Chain;

struct Unit {
  enum Kind { PROG, STEPS, SUM, BLOCKS, SPARSE } kind = PROG;
  i64 n_in = 0, n_out = 0;
  // PROG
  std::vector<fmk::Op> ops;
  i64 L = 0;
  // STEPS
  std::vector<SStep> steps;
  std::vector<i64> tmp_rows;
  // SUM
  std::vector<Chain> terms;
  // BLOCKS: grid[o][q] maps input segment q to output segment o (has = 0:
  // zero block); segment lengths in rows
  std::vector<std::vector<Chain>> grid;
  std::vector<std::vector<int>> has;
  std::vector<i64> seg_in, seg_out;
  // SPARSE: CSR of the operator (or of its adjoint) on the device
  const i64 *sp_ptr = nullptr, *sp_idx = nullptr;
  const void *sp_val = nullptr;
  int sp_group = 32;
};

struct NodeRec {
  fm_node d;
  std::vector<int> ch;
};

fmk::Op mkop(int kind, int len) {
  fmk::Op o;
  memset(&o, 0, sizeof(o));
  o.kind = kind;
  o.len = len;
  o.div = 1;
  o.mod = 1;
  o.stride = 0;
  o.N = 1;
  o.sre = 1.0;
  return o;
}

// Tile configuration of one launch: layout, vectors per tile (B), threads,
// copy-ring depth and shared memory.  want_B / want_nbuf = 0 picks the
// heuristic choice; explicit values (the autotuner's candidates) are
// accepted when feasible.  Returns false if the request cannot be met.
bool configure(int esz, LStep &ls, int want_B, int want_nbuf,
               bool allow_em = true, int want_lay = -1,
               bool allow_dense = true) {
  fmk::Step &st = ls.st;
  const int L = std::max(st.L, 1);
  const int ept = ls.ept;
  // the tensor-core FWHT (class 4) works on whole warpgroups and needs
  // its staging area and TMEM bookkeeping beyond the tile ring
  // (class 6: the tensor-core dense factor, the same granularity and its
  // factor and row staging)
  const bool tcg = ls.cls == 4 || ls.cls == 6;
  const int tgran = tcg ? 128 : 32;
  const size_t extra = ls.cls == 4   ? (size_t)fmk::kTcBytes + 1024
                       : ls.cls == 6 ? (size_t)fmk::kTdBytes + 1024
                                     : 0;
  auto threads_for = [&](int b) {
    i64 t = ((i64)b * L + ept - 1) / ept;
    t = (t + tgran - 1) / tgran * tgran;
    return (int)std::max<i64>(t, tgran);
  };
  auto lsmem = [&](int B, int Lp, int nb) {
    return fmk::launch_smem(B, Lp, esz, nb) + extra;
  };
  // the deepest ring (4 .. 2 buffers) that still lets two CTAs share an SM
  auto pick_nbuf = [&](int B, int Lp) {
    if (want_nbuf) return want_nbuf;
    int nb = 4;
    while (nb > 2 && lsmem(B, Lp, nb) > (size_t)112 * 1024)
      --nb;
    return nb;
  };
  const bool pow2 = want_B == 0 || (want_B & (want_B - 1)) == 0;
  if (!pow2 || want_nbuf < 0 || want_nbuf == 1 || want_nbuf > 4) return false;

  // element-major tiles: strided input and output views whose inner extent
  // holds whole tiles (B | Cc); rows of B * esz bytes (128 B when the thread
  // budget allows, never below 16 B), moved by TMA boxes
  const bool em_class = ls.cls == 1 || ls.cls == 3 || ls.cls == 4 ||
                        ls.cls == 5 || ls.cls == 6;
  if (want_lay == 1 && !(allow_em && em_class)) return false;
  if (allow_em && (want_lay == -1 || want_lay == 1) && em_class &&
      st.vin.Cc > 1 &&
      st.vout.Cc > 1) {
    // (the tensor-core dense factor fills 128-row MMA chunks: 128 vectors)
    int B = want_B ? want_B : (ls.cls == 6 ? 128 : 128 / esz);
    if (!want_B) {
      while (B > 1 && (st.vin.Cc % B || st.vout.Cc % B)) B /= 2;
      while (B * esz > 16 && threads_for(B) > FM_MAX_THREADS) B /= 2;
    }
    if (B * esz >= 16 && threads_for(B) <= FM_MAX_THREADS &&
        st.V % B == 0 && st.vin.Cc % B == 0 && st.vout.Cc % B == 0) {
      const int nbuf = pick_nbuf(B, L);
      const size_t smem = lsmem(B, L, nbuf);
      if (smem <= (size_t)fmk::kMaxSmem) {
        ls.lay = 1;
        st.B = B;
        st.Lp = L;
        st.nbuf = nbuf;
        st.box_rows = std::min(L, 256);
        st.elem_k = esz == 16 ? 2 : 1;
        const bool rows_ok = L % st.box_rows == 0;
        ls.tma_in_ok = rows_ok && st.in_len == st.vin.n && !st.map_in &&
                       st.in_rows == st.vin.A * st.vin.n * st.vin.Cc;
        ls.tma_out_ok = rows_ok && st.out_len == st.vout.n &&
                        st.out_mode == 0 && !st.accumulate &&
                        st.out_rows == st.vout.A * st.vout.n * st.vout.Cc;
        ls.threads = threads_for(B);
        ls.smem = smem;
        return true;
      }
    }
    if (want_B || want_lay == 1) return false;
  }
  if (want_lay == 1) return false;

  // vector-major tiles.  Padded (layout 0): one 16-byte granule per 128
  // bytes (pidx), rounded to whole granules, with an odd granule count so
  // that consecutive vectors start on different banks.  Dense (layout 2):
  // vectors back to back, so that runs of contiguous vectors move as single
  // bulk copies; chosen for contiguous vectors whose program has no
  // butterfly stages (bank conflicts only matter there), or when asked.
  const bool strided = st.vin.Cc > 1 || st.vout.Cc > 1;
  bool stages = false;
  for (int o = 0; o < st.nops; ++o)
    if (st.ops[o].kind == fmk::OP_DIF || st.ops[o].kind == fmk::OP_DIT ||
        st.ops[o].kind == fmk::OP_FWHT)
      stages = true;
  const bool dense_ok = allow_dense && !strided && want_lay != 0;
  if (want_lay == 2 && !dense_ok) return false;
  if (want_lay > 2) return false;
  const bool dense = dense_ok && (want_lay == 2 || !stages);
  const int shift = esz >= 16 ? 3 : (esz == 8 ? 4 : 5);
  const int gran = 16 / esz;
  int Lp = (L - 1) + gran * ((L - 1) >> shift) + 1;
  Lp = (Lp + gran - 1) / gran * gran;
  if (((Lp / gran) & 1) == 0) Lp += gran;
  if (dense) Lp = L;
  auto smem_for = [&](int b, int nb) {
    return lsmem(b, Lp, nb);
  };
  int B;
  if (want_B) {
    B = want_B;
  } else {
    B = strided ? std::max(1, 128 / esz) : 1;
    const size_t budget = 110 * 1024;
    while (B > 1 && (threads_for(B) > FM_MAX_THREADS ||
                     smem_for(B, 2) > (size_t)fmk::kMaxSmem))
      B /= 2;
    while (threads_for(B) < 128 && threads_for(2 * B) <= FM_MAX_THREADS &&
           smem_for(2 * B, 2) <= budget && (i64)B < st.V * 64 && B < 1024)
      B *= 2;
  }
  if (threads_for(B) > FM_MAX_THREADS) return false;
  const int nbuf = pick_nbuf(B, Lp);
  const size_t smem = smem_for(B, nbuf);
  if (smem > (size_t)fmk::kMaxSmem) return false;
  ls.lay = dense ? 2 : 0;
  st.B = B;
  st.Lp = Lp;
  st.nbuf = nbuf;
  ls.threads = threads_for(B);
  ls.smem = smem;
  // contiguous vectors move by 1-D bulk copies of their 128-byte chunks
#ifndef FM_VM_BULK
#define FM_VM_BULK 1
#endif
  ls.tma_in_ok = FM_VM_BULK && st.vin.Cc == 1 && st.in_len == L && st.in_len == st.vin.n &&
                 !st.map_in && st.in_rows == st.vin.A * st.vin.n &&
                 ((i64)st.in_len * esz) % 16 == 0;
  ls.tma_out_ok = FM_VM_BULK && st.vout.Cc == 1 &&
                  st.out_len == st.vout.n && (!dense || st.out_len == L) &&
                  st.out_mode == 0 && !st.accumulate &&
                  st.out_rows == st.vout.A * st.vout.n &&
                  ((i64)st.out_len * esz) % 16 == 0;
  return true;
}

// The register tile program (fm_rtile.cuh) a complex64 batch step runs, or
// 0 when its vector program is not one of the shapes it covers:
// [zero pad] DIF(L) [twiddle] or [zero pad] DIF(L) product DIT(L) [twiddle],
// L = 64 .. 512 with the radix sequence (8, 8, ..., rest).
static int rtile_shape(const fmk::Step &st);
// the launch's threads cover whole vectors of the register tile program
static bool rtile_threads_ok(const LStep &ls) {
  const int G = ls.st.L / fmk::kRtP;
  return ls.lay == 0 && G >= 1 && ls.threads >= G && ls.threads % G == 0 &&
         ls.threads <= FM_MAX_THREADS;
}
static int rtile_shape(const fmk::Step &st) {
  const int L = st.L;
  if (L != 64 && L != 128 && L != 256 && L != 512) return 0;
  if (st.out_mode == 1 || st.nops < 1) return 0;
  auto radices_ok = [&](const fmk::Op &op) {
    if (op.len != L || op.nrad != fmk::rc_stages(L, fmk::kRtP)) return false;
    for (int i = 0; i < op.nrad; ++i)
      if (op.rad[i] != fmk::rc_radix(i, L, fmk::kRtP)) return false;
    return true;
  };
  int f = 0, o = 0, end = st.nops;
  if (st.ops[0].kind == fmk::OP_ZPAD) {
    if (st.ops[0].len2 != L || st.ops[0].len > L) return 0;
    f |= fmk::RT_ZPAD;
    o = 1;
  }
  if (end > o + 1 && st.ops[end - 1].kind == fmk::OP_TW) {
    const fmk::Op &t = st.ops[end - 1];
    if (t.len != L || t.N <= 0 || t.div < 1 || t.mod < 1 || !t.ptr3)
      return 0;
    f |= fmk::RT_TW;
    --end;
  }
  if (o >= end) return 0;
  const fmk::Op &d = st.ops[o];
  if (d.kind != fmk::OP_DIF || !radices_ok(d)) return 0;
  if (end == o + 1) {
    if ((f & fmk::RT_TW) && !st.ops[st.nops - 1].ptr2) return 0;
    return f | fmk::RT_FFT | (d.sign > 0 ? fmk::RT_INV : 0);
  }
  if (end == o + 3 && st.ops[o + 1].kind == fmk::OP_MUL &&
      st.ops[o + 1].len == L && st.ops[o + 1].div >= 1 &&
      st.ops[o + 1].mod >= 1 && st.ops[o + 2].kind == fmk::OP_DIT &&
      radices_ok(st.ops[o + 2]) && d.sign < 0 && st.ops[o + 2].sign > 0) {
    if ((f & fmk::RT_TW) && st.ops[st.nops - 1].ptr2) return 0;
    f |= fmk::RT_CONV;
    if (st.vout.Cc == 1 && st.out_mode == 0 && st.dst_type == FM_C64 &&
        !st.accumulate)
      f |= fmk::RT_DIRECT;
    return f;
  }
  return 0;
}

class Planner {
 public:
  Planner(fm_plan *P, const std::vector<NodeRec> &nodes)
      : P_(P), nodes_(nodes) {
    cplx_ = is_cplx(P->ctype);
    ept_ = P->esz == 4 ? 16 : 8;
    lmax_ = (i64)ept_ * FM_MAX_THREADS;
  }

  void build(int root) {
    for (int dir = 0; dir < 2; ++dir) {
      Chain c = compile(root, dir == FM_FORWARD);
      const NodeRec &r = nodes_[root];
      const i64 n_in = dir == FM_FORWARD ? r.d.cols : r.d.rows;
      const i64 n_out = dir == FM_FORWARD ? r.d.rows : r.d.cols;
      std::vector<LStep> &out = P_->steps[dir];
      lower(c, 0, n_in, 1, n_out, out);
      if (out.empty()) emit_copy(0, 1, n_in, out);
      pair_fwht(out);
    }
  }

  // the plan's counters of fused launches, at least n of them
  void counters(i64 n) {
    if (P_->pair_cap >= n) return;
    P_->pair_ctr = (unsigned *)dalloc((size_t)n * 4);
    P_->pair_cap = n;
  }

  // A plain register convolution on contiguous vectors followed by a
  // strided register FWHT in place on its output whose blocks (L2 S rows)
  // the convolution's vectors tile (a circulant Kron mode and the Hadamard
  // mode before it) become one launch that keeps each block in L2.
  // (complex64 only: the double-float pair measured slower than its two
  // launches, 3.00 against 2.70 ms for the Kron workload, the arithmetic
  // being the bound there)
  bool pair_conv_fwht(LStep &a, LStep &b) {
    if (P_->ctype != FM_C64) return false;
    if (a.kind != 2 || b.kind != 3 || b.rc_es <= 1 || a.pair || b.pair)
      return false;
    if (a.dst != b.src || b.src != b.dst || a.src == a.dst || a.dst_off ||
        b.src_off || b.dst_off)
      return false;
    const fmk::Step &sa = a.st, &sb = b.st;
    const i64 L1 = a.rc_L;
    if (a.rc_pre || a.rc_post || a.rc_conj_in || a.rc_conj_out || sa.pre ||
        sa.post || sa.conj_in || sa.conj_out || sa.has_scale ||
        sa.accumulate || sa.map_in || sa.map_out || sa.out_mode)
      return false;
    if (sa.vin.Cc != 1 || sa.vout.Cc != 1 || sa.vin.n != L1 ||
        sa.vout.n != L1 || sa.vin.A != sa.vout.A || sa.in_len != L1 ||
        sa.out_len != L1 || sa.in_rows != sa.vin.A * L1 ||
        sa.out_rows != sa.vout.A * L1)
      return false;
    const i64 S = sb.vin.Cc, L2 = b.rc_L;
    const i64 block_rows = L2 * S;
    if (sb.vin.A * block_rows != sa.vin.A * L1) return false;
    int n1 = 0, n2 = 0;
    const i64 k = b.rc_es / S;  // real words per element
    if (!fmk::rkch_supported(P_->ctype, (int)L1, (int)L2, block_rows,
                             S * k, &n1, &n2))
      return false;
    counters(1 + 4096 * sb.vin.A);
    a.pair = 3;
    b.pair = 2;
    a.rc2_L = b.rc_L;
    a.rc2_es = b.rc_es;
    a.rc2_A = b.rc_A;
    a.rc2_blocks = (int)sb.vin.A;
    a.rc2_n1 = n1;
    a.rc2_n2 = n2;
    return true;
  }

  // A contiguous register FWHT followed by the strided one that finishes
  // the same transform in place (the two passes of a long Hadamard) become
  // one launch that keeps each column's intermediate in L2.
  void pair_fwht(std::vector<LStep> &out) {
    for (size_t i = 0; i + 1 < out.size(); ++i) {
      LStep &a = out[i], &b = out[i + 1];
      if (pair_conv_fwht(a, b)) {
        ++i;
        continue;
      }
      if (a.kind != 3 || b.kind != 3 || a.rc_es != 0 || b.rc_es <= 1 ||
          a.pair || b.pair || a.rc_ct != b.rc_ct)
        continue;
      if (a.dst != b.src || b.src != b.dst || a.src == a.dst ||
          a.dst_off || b.src_off || b.dst_off)
        continue;
      const fmk::Step &sa = a.st, &sb = b.st;
      // a: vectors of N2 points; b: vectors of N1 points at stride N2,
      // over the same N1 N2 rows
      const i64 N2 = a.rc_L, N1 = b.rc_L;
      if (sa.vin.Cc != 1 || sa.vin.n != N2 || sa.vin.A != N1 ||
          sb.vin.A != 1 || sb.vin.n != N1 || sb.vin.Cc != N2 ||
          b.rc_es != N2)
        continue;
      if (!fmk::rfwht2_supported(a.rc_ct, a.rc_L, b.rc_L)) continue;
      counters(1 + 4096);
      a.pair = 1;
      b.pair = 2;
      a.rc2_L = b.rc_L;
      a.rc2_es = b.rc_es;
      a.rc2_A = b.rc_A;
      ++i;
    }
  }

 private:
  fm_plan *P_;
  const std::vector<NodeRec> &nodes_;
  bool cplx_;
  int ept_;
  i64 lmax_;
  std::map<const void *, std::vector<cd>> host_vec_;  // host copies of MUL
  std::map<const void *, std::vector<i64>> host_map_;  // and GATHER data

  // ---------------------------------------------------------- device data
  void *dalloc(size_t bytes) {
    void *p = nullptr;
    CUDA_TRY(dev_malloc(&p, std::max<size_t>(bytes, 16)));
    P_->allocs.push_back(p);
    P_->const_bytes += (i64)bytes;
    return p;
  }

  const void *twiddle(i64 N) {
    auto it = P_->twiddles.find(N);
    if (it != P_->twiddles.end()) return it->second;
    void *p = dalloc((size_t)N * P_->esz);
    if (P_->ctype == FM_C64)
      k_twiddle<float2><<<grid_for(N), 256>>>((float2 *)p, N);
    else if (P_->ctype == FM_C128_DF)
      k_twiddle<fmk::dfc><<<grid_for(N), 256>>>((fmk::dfc *)p, N);
    else
      k_twiddle<double2><<<grid_for(N), 256>>>((double2 *)p, N);
    CUDA_TRY(cudaGetLastError());
    P_->twiddles[N] = p;
    return p;
  }

  // split of the two-level twiddle table of length N (complex64 only)
  static int twiddle2_bits(i64 N) {
    int b = 0;
    while ((1LL << b) < N) ++b;
    return (b + 1) / 2;
  }
  const void *twiddle2(i64 N) {
    if (P_->ctype != FM_C64) return nullptr;
    auto it = P_->twiddles.find(-N);
    if (it != P_->twiddles.end()) return it->second;
    const int s = twiddle2_bits(N);
    const i64 n = (1LL << s) + ((N - 1) >> s) + 1;
    void *p = dalloc((size_t)n * P_->esz);
    k_twiddle2<float2><<<grid_for(n), 256>>>((float2 *)p, N, s);
    CUDA_TRY(cudaGetLastError());
    P_->twiddles[-N] = p;
    return p;
  }

  // upload a host vector in the compute type
  const void *upload(const std::vector<cd> &v) {
    const size_t n = v.size();
    std::vector<unsigned char> buf(n * P_->esz);
    for (size_t i = 0; i < n; ++i) {
      auto hi = [](double d) { return (float)d; };
      auto lo = [](double d) { return (float)(d - (double)(float)d); };
      switch (P_->ctype) {
        case FM_F64_DF:
          ((float *)buf.data())[2 * i] = hi(v[i].real());
          ((float *)buf.data())[2 * i + 1] = lo(v[i].real());
          break;
        case FM_C128_DF:
          ((float *)buf.data())[4 * i] = hi(v[i].real());
          ((float *)buf.data())[4 * i + 1] = lo(v[i].real());
          ((float *)buf.data())[4 * i + 2] = hi(v[i].imag());
          ((float *)buf.data())[4 * i + 3] = lo(v[i].imag());
          break;
        case FM_F32:
        case FM_F32_TC: ((float *)buf.data())[i] = (float)v[i].real(); break;
        case FM_F64: ((double *)buf.data())[i] = v[i].real(); break;
        case FM_I64:
          ((int64_t *)buf.data())[i] = (int64_t)llround(v[i].real());
          break;
        case FM_C64:
          ((float *)buf.data())[2 * i] = (float)v[i].real();
          ((float *)buf.data())[2 * i + 1] = (float)v[i].imag();
          break;
        default:
          ((double *)buf.data())[2 * i] = v[i].real();
          ((double *)buf.data())[2 * i + 1] = v[i].imag();
          break;
      }
      if (!cplx_ && v[i].imag() != 0.0)
        fail(FM_ERR_TYPE, "complex operator data in a real-valued plan");
    }
    void *p = dalloc(buf.size());
    CUDA_TRY(cudaMemcpy(p, buf.data(), buf.size(), cudaMemcpyHostToDevice));
    host_vec_[p] = v;
    return p;
  }

  const i64 *upload_map(const std::vector<i64> &m) {
    void *p = dalloc(m.size() * sizeof(i64));
    CUDA_TRY(cudaMemcpy(p, m.data(), m.size() * sizeof(i64),
                        cudaMemcpyHostToDevice));
    host_map_[p] = m;
    return (const i64 *)p;
  }

  std::vector<cd> node_vec(const fm_node &d, int which) {
    const void *p = which == 0 ? d.vec0 : d.vec1;
    const i64 n = which == 0 ? d.len0 : d.len1;
    const int t = which == 0 ? d.type0 : d.type1;
    std::vector<cd> v((size_t)n);
    if (n > 0 && !p) fail(FM_ERR_VALUE, "missing operator data");
    for (i64 i = 0; i < n; ++i) v[i] = host_get(p, t, i);
    return v;
  }
  std::vector<i64> node_idx(const fm_node &d, int which) {
    const void *p = which == 0 ? d.vec0 : d.vec1;
    const i64 n = which == 0 ? d.len0 : d.len1;
    const int t = which == 0 ? d.type0 : d.type1;
    std::vector<i64> v((size_t)n);
    for (i64 i = 0; i < n; ++i) v[i] = host_get_int(p, t, i);
    return v;
  }

  // FFT of a length-L device c128 vector (L smooth), forward, in double,
  // through a nested plan of this engine.
  void fft_f64_device(const double2 *in, double2 *out, i64 L) {
    fm_node nd;
    memset(&nd, 0, sizeof(nd));
    nd.kind = FM_NODE_FOURIER;
    nd.dtype = FM_C128;
    nd.rows = nd.cols = L;
    nd.n = L;
    std::vector<NodeRec> sub(1);
    sub[0].d = nd;
    fm_plan Q;
    Q.ctype = FM_C128;
    Q.io_type = FM_C128;
    Q.esz = 16;
    Q.device = P_->device;
    Q.rows = Q.cols = L;
    Planner(&Q, sub).build(0);
    const int st = run_plan(&Q, FM_FORWARD, in, FM_C128, L, out, FM_C128, L,
                            1, 0);
    if (st != FM_OK) fail(st, "nested FFT failed: " + g_err);
    CUDA_TRY(cudaDeviceSynchronize());
  }

  // spectrum fft(v)/L of a host vector (length L), in the compute type,
  // optionally in the four-step (L1, L2) layout
  const void *spectrum(const std::vector<cd> &v, i64 L1 = 0, i64 L2 = 0) {
    const i64 L = (i64)v.size();
    DevTemp tin, tout;
    CUDA_TRY(dev_malloc(&tin.p, L * sizeof(double2)));
    CUDA_TRY(dev_malloc(&tout.p, L * sizeof(double2)));
    double2 *din = (double2 *)tin.p, *dout = (double2 *)tout.p;
    CUDA_TRY(cudaMemcpy(din, v.data(), L * sizeof(double2),
                        cudaMemcpyHostToDevice));
    fft_f64_device(din, dout, L);
    return convert_dev(dout, L, 1.0 / (double)L, L1, L2);
  }

  const void *convert_dev(const double2 *src, i64 n, double scale, i64 L1,
                          i64 L2) {
    void *p = dalloc((size_t)n * P_->esz);
    if (P_->ctype == FM_C64)
      k_convert<float2><<<grid_for(n), 256>>>((float2 *)p, src, n, scale, L1,
                                               L2);
    else if (P_->ctype == FM_C128_DF)
      k_convert<fmk::dfc><<<grid_for(n), 256>>>((fmk::dfc *)p, src, n, scale,
                                                 L1, L2);
    else
      k_convert<double2><<<grid_for(n), 256>>>((double2 *)p, src, n, scale,
                                                L1, L2);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaDeviceSynchronize());
    // host copy for chunked-step normalisation
    std::vector<cd> h((size_t)n);
    std::vector<double2> raw((size_t)n);
    CUDA_TRY(cudaMemcpy(raw.data(), src, n * sizeof(double2),
                        cudaMemcpyDeviceToHost));
    for (i64 o = 0; o < n; ++o) {
      i64 s = o;
      if (L1 > 0) s = (o / L2) + L1 * (o % L2);
      h[o] = cd(raw[s].x, raw[s].y) * scale;
    }
    host_vec_[p] = h;
    return p;
  }

  // ---------------------------------------------------------- FFT order
  // The device FFT runs in place: DIF leaves the spectrum in digit-reversed
  // order for its radix sequence, DIT takes that order back to natural.
  // nat[P] is the natural index stored at position P, pos its inverse.
  struct Perm {
    std::vector<int> nat, pos;
    const int *nat_dev = nullptr, *pos_dev = nullptr;
  };
  std::map<std::vector<int>, Perm> perms_;

  const Perm &perm_for(const std::vector<int> &rad) {
    auto it = perms_.find(rad);
    if (it != perms_.end()) return it->second;
    int L = 1;
    for (int r : rad) L *= r;
    Perm pm;
    pm.nat.assign(L, 0);
    pm.pos.assign(L, 0);
    std::vector<int> k(rad.size(), 0);
    for (int c = 0; c < L; ++c) {
      // digits k (k[0] most significant in the position)
      int posv = 0, natv = 0, mul = 1;
      for (size_t i = 0; i < rad.size(); ++i) posv = posv * rad[i] + k[i];
      for (size_t i = 0; i < rad.size(); ++i) {
        natv += k[i] * mul;
        mul *= rad[i];
      }
      pm.nat[posv] = natv;
      pm.pos[natv] = posv;
      for (int i = (int)rad.size() - 1; i >= 0; --i) {
        if (++k[i] < rad[i]) break;
        k[i] = 0;
      }
    }
    void *a = dalloc(L * sizeof(int));
    void *b = dalloc(L * sizeof(int));
    CUDA_TRY(cudaMemcpy(a, pm.nat.data(), L * sizeof(int),
                        cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(b, pm.pos.data(), L * sizeof(int),
                        cudaMemcpyHostToDevice));
    pm.nat_dev = (const int *)a;
    pm.pos_dev = (const int *)b;
    return perms_.emplace(rad, pm).first->second;
  }

  std::vector<int> op_radices(const fmk::Op &o) {
    return std::vector<int>(o.rad, o.rad + o.nrad);
  }

  // Lower abstract FFT ops of a program to DIF/DIT, keeping track of the
  // element order; returns the storer's position table if the program ends
  // in digit-reversed order (nullptr otherwise).
  const int *finalize(std::vector<fmk::Op> &ops) {
    std::vector<fmk::Op> out;
    bool permuted = false;
    std::vector<int> cur;
    auto to_natural = [&]() {
      const Perm &pm = perm_for(cur);
      std::vector<i64> m(pm.pos.begin(), pm.pos.end());
      out.push_back(gather_op(m));
      permuted = false;
    };
    for (fmk::Op o : ops) {
      switch (o.kind) {
        case fmk::OP_FFT: {
          std::vector<int> rad = op_radices(o);
          if (permuted && rad != cur) to_natural();
          if (!permuted) {
            o.kind = fmk::OP_DIF;
            permuted = true;
            cur = rad;
          } else {
            o.kind = fmk::OP_DIT;
            permuted = false;
          }
          out.push_back(o);
          break;
        }
        case fmk::OP_MUL: {
          if (permuted) {
            const Perm &pm = perm_for(cur);
            const std::vector<cd> &v = host_vec_.at(o.ptr);
            std::vector<cd> w(v);
            const i64 len = o.len;
            const i64 rows = o.stride > 0 ? (i64)v.size() / o.stride : 1;
            const i64 rs = o.stride > 0 ? o.stride : 0;
            for (i64 r = 0; r < rows; ++r)
              for (i64 P = 0; P < len; ++P)
                w[r * rs + P] = v[r * rs + pm.nat[P]];
            o.ptr = upload(w);
          }
          out.push_back(o);
          break;
        }
        case fmk::OP_GATHER: {
          if (permuted) {
            const Perm &pm = perm_for(cur);
            const std::vector<i64> &m = host_map_.at(o.ptr);
            std::vector<i64> c(m.size());
            for (size_t i = 0; i < m.size(); ++i)
              c[i] = m[i] < 0 ? -1 : pm.pos[m[i]];
            o.ptr = upload_map(c);
            permuted = false;
          }
          out.push_back(o);
          break;
        }
        case fmk::OP_TW:
          if (permuted) o.ptr2 = perm_for(cur).nat_dev;
          out.push_back(o);
          break;
        case fmk::OP_CONJ:
        case fmk::OP_SCALE: out.push_back(o); break;
        default:
          if (permuted) to_natural();
          out.push_back(o);
          break;
      }
    }
    ops.swap(out);
    return permuted ? perm_for(cur).pos_dev : nullptr;
  }

  // ---------------------------------------------------------- FFT helpers
  std::vector<int> radices(i64 n) {
    std::vector<int> r;
    for (int p : {7, 5, 3})
      while (n % p == 0) {
        r.push_back(p);
        n /= p;
      }
    // largest radix the kernels of this compute type are built with
    const int big = fmk::max_radix_for(P_->ctype);
    while (n % big == 0) {
      r.push_back(big);
      n /= big;
    }
    for (int p : {8, 4, 2})
      while (n % p == 0) {
        r.push_back(p);
        n /= p;
      }
    if (n != 1) fail(FM_ERR_UNSUPPORTED, "FFT length is not 2,3,5,7-smooth");
    return r;
  }

  fmk::Op fft_op(i64 n, int sign) {
    if (!cplx_) fail(FM_ERR_TYPE, "Fourier-type operator in a real plan");
    fmk::Op o = mkop(fmk::OP_FFT, (int)n);
    o.sign = sign;
    std::vector<int> r = radices(n);
    if (r.size() > sizeof(o.rad)) fail(FM_ERR_UNSUPPORTED, "FFT too long");
    o.nrad = (int)r.size();
    for (size_t i = 0; i < r.size(); ++i) o.rad[i] = (unsigned char)r[i];
    o.ptr = twiddle(n);
    return o;
  }

  fmk::Op fwht_op(i64 n) {
    fmk::Op o = mkop(fmk::OP_FWHT, (int)n);
    o.sign = P_->ctype == FM_F32_TC ? 1 : 0;  // 16-point groups on MMA
    int bits = 0;
    while ((1LL << bits) < n) ++bits;
    const int g = 4;
    while (bits > 0) {
      const int k = std::min(g, bits);
      o.rad[o.nrad++] = (unsigned char)k;
      bits -= k;
    }
    return o;
  }

  fmk::Op mul_op(const void *v, i64 len, bool conj) {
    fmk::Op o = mkop(fmk::OP_MUL, (int)len);
    o.ptr = v;
    o.sign = conj ? 1 : 0;
    return o;
  }

  fmk::Op zpad_op(i64 from, i64 to) {
    fmk::Op o = mkop(fmk::OP_ZPAD, (int)from);
    o.len2 = (int)to;
    return o;
  }

  fmk::Op gather_op(const std::vector<i64> &map) {
    fmk::Op o = mkop(fmk::OP_GATHER, (int)map.size());
    o.ptr = upload_map(map);
    return o;
  }

  // split N = N1 * N2 with both factors <= limit, N1 as close to sqrt(N)
  void split2(i64 N, i64 limit, i64 &N1, i64 &N2) {
    N1 = 0;
    const double r = std::sqrt((double)N);
    double best = 1e300;
    for (i64 d = 2; d <= limit && d < N; ++d) {
      if (N % d) continue;
      const i64 e = N / d;
      if (e > limit || !smooth(d) || !smooth(e)) continue;
      // prefer power-of-two factors and balanced splits
      const double score = std::fabs(std::log((double)d / r)) +
                           (is_pow2(d) && is_pow2(e) ? 0 : 0.5);
      if (score < best) {
        best = score;
        N1 = d;
      }
    }
    if (!N1)
      fail(FM_ERR_UNSUPPORTED,
           "transform length " + std::to_string(N) +
               " exceeds the two-pass limit");
    N2 = N / N1;
  }

  // ---------------------------------------------------------- units
  Unit prog(std::vector<fmk::Op> ops, i64 n_in, i64 n_out, i64 L) {
    Unit u;
    u.kind = Unit::PROG;
    u.ops = std::move(ops);
    u.n_in = n_in;
    u.n_out = n_out;
    u.L = L;
    return u;
  }

  // circular convolution of length L with a device spectrum (natural
  // layout for the in-smem program, four-step layout for long L)
  Chain conv(i64 L, i64 n_in, i64 n_out, const std::vector<cd> &filt,
             bool conj, const void *pre = nullptr, const void *post = nullptr,
             bool conj_io = false) {
    Chain c;
    const i64 lim = has_odd(L) ? lmax_ / 2 : lmax_;
    if (L <= lim) {
      const void *S = spectrum(filt);
      std::vector<fmk::Op> ops;
      if (conj_io) ops.push_back(mkop(fmk::OP_CONJ, (int)n_in));
      if (pre) ops.push_back(mul_op(pre, n_in, false));
      if (n_in < L) ops.push_back(zpad_op(n_in, L));
      ops.push_back(fft_op(L, -1));
      ops.push_back(mul_op(S, L, conj));
      ops.push_back(fft_op(L, +1));
      if (post) ops.push_back(mul_op(post, n_out, false));
      if (conj_io) ops.push_back(mkop(fmk::OP_CONJ, (int)n_out));
      c.push_back(prog(ops, n_in, n_out, L));
      return c;
    }
    i64 L1, L2;
    split2(L, has_odd(L) ? lmax_ / 2 : lmax_, L1, L2);
    const void *S = spectrum(filt, L1, L2);
    Unit u;
    u.kind = Unit::STEPS;
    u.n_in = n_in;
    u.n_out = n_out;
    u.tmp_rows.push_back(L);
    SStep a;
    a.vin = a.vout = fmk::View{1, L1, L2};
    a.in_rows = n_in;
    a.out_rows = L;
    a.L = a.in_len = a.out_len = (int)L1;
    a.src = -1;
    a.dst = 0;
    a.pre = pre;
    a.conj_in = conj_io;
    a.ops.push_back(fft_op(L1, -1));
    fmk::Op tw = mkop(fmk::OP_TW, (int)L1);
    tw.ptr = twiddle(L);
    tw.ptr3 = twiddle2(L);
    tw.N = L;
    tw.sign = -1;
    tw.div = 1;
    tw.mod = L2;
    a.ops.push_back(tw);
    SStep b;
    b.vin = b.vout = fmk::View{L1, L2, 1};
    b.in_rows = b.out_rows = L;
    b.L = b.in_len = b.out_len = (int)L2;
    b.src = 0;
    b.dst = 0;
    b.ops.push_back(fft_op(L2, -1));
    fmk::Op m = mul_op(S, L2, conj);
    m.div = 1;
    m.mod = L1;
    m.stride = L2;
    b.ops.push_back(m);
    b.ops.push_back(fft_op(L2, +1));
    fmk::Op tw2 = mkop(fmk::OP_TW, (int)L2);
    tw2.ptr = twiddle(L);
    tw2.ptr3 = twiddle2(L);
    tw2.N = L;
    tw2.sign = +1;
    tw2.div = 1;
    tw2.mod = L1;
    b.ops.push_back(tw2);
    SStep cc;
    cc.vin = cc.vout = fmk::View{1, L1, L2};
    cc.in_rows = L;
    cc.out_rows = n_out;
    cc.L = cc.in_len = cc.out_len = (int)L1;
    cc.src = 0;
    cc.dst = -2;
    cc.post = post;
    cc.conj_out = conj_io;
    cc.ops.push_back(fft_op(L1, +1));
    u.steps = {a, b, cc};
    c.push_back(u);
    return c;
  }

  bool has_odd(i64 L) { return L % 3 == 0 || L % 5 == 0 || L % 7 == 0; }

  Chain fourier(i64 N, bool fwd) {
    const int sign = fwd ? -1 : +1;
    Chain c;
    if (smooth(N)) {
      const i64 lim = has_odd(N) ? lmax_ / 2 : lmax_;
      if (N <= lim) {
        c.push_back(prog({fft_op(N, sign)}, N, N, N));
        return c;
      }
      i64 N1, N2;
      split2(N, lim, N1, N2);
      Unit u;
      u.kind = Unit::STEPS;
      u.n_in = u.n_out = N;
      u.tmp_rows.push_back(N);
      SStep a;
      a.vin = a.vout = fmk::View{1, N1, N2};
      a.in_rows = a.out_rows = N;
      a.L = a.in_len = a.out_len = (int)N1;
      a.src = -1;
      a.dst = 0;
      a.ops.push_back(fft_op(N1, sign));
      fmk::Op tw = mkop(fmk::OP_TW, (int)N1);
      tw.ptr = twiddle(N);
      tw.ptr3 = twiddle2(N);
      tw.N = N;
      tw.sign = sign;
      tw.div = 1;
      tw.mod = N2;
      a.ops.push_back(tw);
      SStep b;
      b.vin = fmk::View{N1, N2, 1};
      b.vout = fmk::View{1, N2, N1};
      b.in_rows = b.out_rows = N;
      b.L = b.in_len = b.out_len = (int)N2;
      b.src = 0;
      b.dst = -2;
      b.ops.push_back(fft_op(N2, sign));
      u.steps = {a, b};
      c.push_back(u);
      return c;
    }
    // Bluestein: x -> a . x -> (*) h -> a . (first N)
    const i64 Lb = next_pow2(2 * N - 1);
    DevTemp ta, th;
    CUDA_TRY(dev_malloc(&ta.p, N * sizeof(double2)));
    CUDA_TRY(dev_malloc(&th.p, Lb * sizeof(double2)));
    double2 *da = (double2 *)ta.p, *dh = (double2 *)th.p;
    k_chirp<<<grid_for(N), 256>>>(da, N);
    k_bluestein_filter<<<grid_for(Lb), 256>>>(dh, da, N, Lb);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaDeviceSynchronize());
    const void *chirp = convert_dev(da, N, 1.0, 0, 0);
    std::vector<double2> hh((size_t)Lb);
    CUDA_TRY(cudaMemcpy(hh.data(), dh, Lb * sizeof(double2),
                        cudaMemcpyDeviceToHost));
    std::vector<cd> filt((size_t)Lb);
    for (i64 i = 0; i < Lb; ++i) filt[i] = cd(hh[i].x, hh[i].y);
    return conv(Lb, N, N, filt, false, chirp, chirp, !fwd);
  }

  Chain compile(int id, bool fwd) {
    const NodeRec &r = nodes_[id];
    const fm_node &d = r.d;
    const i64 n_in = fwd ? d.cols : d.rows;
    const i64 n_out = fwd ? d.rows : d.cols;
    Chain c;
    switch (d.kind) {
      case FM_NODE_FOURIER: return fourier(d.n, fwd);
      case FM_NODE_CIRCULANT: {
        const i64 n = d.len0;
        std::vector<cd> cv = node_vec(d, 0);
        i64 L = n;
        if (!smooth(n)) L = next_pow2(2 * n - 1);
        std::vector<cd> filt((size_t)L, cd(0, 0));
        for (i64 i = 0; i < n; ++i) filt[i] = cv[i];
        if (L != n)
          for (i64 i = 1; i < n; ++i) filt[L - n + i] = cv[i];
        return conv(L, n, n, filt, !fwd);
      }
      case FM_NODE_TOEPLITZ: {
        const i64 nr = d.len0, nc = d.len1 + 1;
        std::vector<cd> vc = node_vec(d, 0), vr = node_vec(d, 1);
        const i64 dd = nr + nc - 1;
        const i64 L = smooth(dd) && is_pow2(dd) ? dd : next_pow2(dd);
        std::vector<cd> filt((size_t)L, cd(0, 0));
        for (i64 i = 0; i < nr; ++i) filt[i] = vc[i];
        for (i64 i = 0; i < nc - 1; ++i) filt[L - (nc - 1) + i] = vr[i];
        return fwd ? conv(L, nc, nr, filt, false) : conv(L, nr, nc, filt, true);
      }
      case FM_NODE_HADAMARD: {
        const i64 N = 1LL << d.n;
        if (N <= lmax_) {
          c.push_back(prog({fwht_op(N)}, N, N, N));
          return c;
        }
        // widest contiguous pass that fits one tile, the rest strided (so
        // the strided pass keeps wide TMA rows)
        int p2 = 0;
        while ((2LL << p2) <= lmax_ && p2 + 1 < d.n) ++p2;
        int p1 = (int)(d.n - p2);
        if ((1LL << p1) > lmax_) {
          p1 = (int)(d.n / 2);
          p2 = (int)(d.n - p1);
        }
        const i64 N1 = 1LL << p1, N2 = 1LL << p2;
        Unit u;
        u.kind = Unit::STEPS;
        u.n_in = u.n_out = N;
        // the low index bits first (contiguous vectors of N2), then the
        // high bits (vectors of N1 at stride N2): the butterflies then run
        // in fastmat's order, distance 1, 2, 4, ... (fastmat/Hadamard.pyx:
        // 182-228), so single-precision results are bit-identical to it
        SStep b;
        b.vin = b.vout = fmk::View{N1, N2, 1};
        b.in_rows = b.out_rows = N;
        b.L = b.in_len = b.out_len = (int)N2;
        b.src = -1;
        b.dst = -2;
        b.ops.push_back(fwht_op(N2));
        SStep a;
        a.vin = a.vout = fmk::View{1, N1, N2};
        a.in_rows = a.out_rows = N;
        a.L = a.in_len = a.out_len = (int)N1;
        a.src = -2;
        a.dst = -2;
        a.ops.push_back(fwht_op(N1));
        u.steps = {b, a};
        c.push_back(u);
        return c;
      }
      case FM_NODE_DIAG: {
        const void *dv = upload(node_vec(d, 0));
        c.push_back(prog({mul_op(dv, d.len0, !fwd)}, d.len0, d.len0, d.len0));
        return c;
      }
      case FM_NODE_PERMUTATION: {
        std::vector<i64> s = node_idx(d, 0);
        const i64 n = (i64)s.size();
        std::vector<i64> t((size_t)n, -1);
        for (i64 i = 0; i < n; ++i) {
          if (s[i] < 0 || s[i] >= n || t[s[i]] >= 0)
            fail(FM_ERR_VALUE, "Not a permutation.");
          t[s[i]] = i;
        }
        c.push_back(prog({gather_op(fwd ? s : t)}, n, n, n));
        return c;
      }
      case FM_NODE_PARTIAL: {
        const NodeRec &ch = nodes_[r.ch.at(0)];
        const i64 crow = ch.d.rows, ccol = ch.d.cols;
        std::vector<i64> rows, cols;
        if (d.vec0) rows = node_idx(d, 0);
        if (d.vec1) cols = node_idx(d, 1);
        auto check = [](const std::vector<i64> &v, i64 n) {
          for (i64 x : v)
            if (x < 0 || x >= n)
              fail(FM_ERR_VALUE, "Partial: index exceeds matrix dimensions.");
        };
        check(rows, crow);
        check(cols, ccol);
        auto inverse = [](const std::vector<i64> &sel, i64 n) {
          std::vector<i64> inv((size_t)n, -1);
          for (size_t k = 0; k < sel.size(); ++k) inv[sel[k]] = (i64)k;
          return inv;
        };
        const std::vector<i64> &sel_in = fwd ? cols : rows;
        const std::vector<i64> &sel_out = fwd ? rows : cols;
        const bool has_in = fwd ? d.vec1 != nullptr : d.vec0 != nullptr;
        const bool has_out = fwd ? d.vec0 != nullptr : d.vec1 != nullptr;
        const i64 full_in = fwd ? ccol : crow;
        if (has_in) {
          std::vector<i64> inv = inverse(sel_in, full_in);
          c.push_back(prog({gather_op(inv)}, (i64)sel_in.size(), full_in,
                           std::max<i64>(full_in, (i64)sel_in.size())));
        }
        Chain inner = compile(r.ch.at(0), fwd);
        c.insert(c.end(), inner.begin(), inner.end());
        if (has_out) {
          const i64 full_out = fwd ? crow : ccol;
          c.push_back(prog({gather_op(sel_out)}, full_out,
                           (i64)sel_out.size(),
                           std::max<i64>(full_out, (i64)sel_out.size())));
        }
        return c;
      }
      case FM_NODE_PRODUCT: {
        const bool scaled = d.scalar_re != 1.0 || d.scalar_im != 0.0;
        if (scaled) {
          fmk::Op s = mkop(fmk::OP_SCALE, (int)n_in);
          s.sre = d.scalar_re;
          s.sim = fwd ? d.scalar_im : -d.scalar_im;
          if (!cplx_ && s.sim != 0.0)
            fail(FM_ERR_TYPE, "complex scalar in a real plan");
          c.push_back(prog({s}, n_in, n_in, n_in));
        }
        const int k = (int)r.ch.size();
        for (int i = 0; i < k; ++i) {
          const int idx = fwd ? r.ch[k - 1 - i] : r.ch[i];
          Chain t = compile(idx, fwd);
          c.insert(c.end(), t.begin(), t.end());
        }
        return c;
      }
      case FM_NODE_SUM: {
        Unit u;
        u.kind = Unit::SUM;
        u.n_in = n_in;
        u.n_out = n_out;
        for (int ch : r.ch) u.terms.push_back(compile(ch, fwd));
        c.push_back(u);
        return c;
      }
      case FM_NODE_KRON: return kron(r, fwd);
      case FM_NODE_BLOCKS: {
        const i64 R = d.n, k = (i64)r.ch.size();
        if (R < 1 || k < 1 || k % R)
          fail(FM_ERR_VALUE, "Blocks: children do not form a grid");
        const i64 C = k / R;
        std::vector<i64> hr((size_t)R, -1), wc((size_t)C, -1);
        for (i64 i = 0; i < R; ++i)
          for (i64 j = 0; j < C; ++j) {
            const int ch = r.ch[(size_t)(i * C + j)];
            if (ch < 0) continue;
            const fm_node &b = nodes_[ch].d;
            if ((hr[i] >= 0 && hr[i] != b.rows) ||
                (wc[j] >= 0 && wc[j] != b.cols))
              fail(FM_ERR_VALUE, "Blocks: block shapes do not form a grid");
            hr[i] = b.rows;
            wc[j] = b.cols;
          }
        i64 sr = 0, sc = 0;
        for (i64 v : hr) {
          if (v < 0) fail(FM_ERR_VALUE, "Blocks: a block row holds no block");
          sr += v;
        }
        for (i64 v : wc) {
          if (v < 0)
            fail(FM_ERR_VALUE, "Blocks: a block column holds no block");
          sc += v;
        }
        if (sr != d.rows || sc != d.cols)
          fail(FM_ERR_VALUE, "Blocks: blocks do not add up to the shape");
        Unit u;
        u.kind = Unit::BLOCKS;
        u.n_in = n_in;
        u.n_out = n_out;
        // forward: output segments are the block rows; the adjoint swaps
        // rows and columns and takes every block's adjoint
        u.seg_out = fwd ? hr : wc;
        u.seg_in = fwd ? wc : hr;
        u.grid.assign(u.seg_out.size(), std::vector<Chain>(u.seg_in.size()));
        u.has.assign(u.seg_out.size(), std::vector<int>(u.seg_in.size(), 0));
        for (i64 i = 0; i < R; ++i)
          for (i64 j = 0; j < C; ++j) {
            const int ch = r.ch[(size_t)(i * C + j)];
            if (ch < 0) continue;
            const size_t o = (size_t)(fwd ? i : j), q = (size_t)(fwd ? j : i);
            u.grid[o][q] = compile(ch, fwd);
            u.has[o][q] = 1;
          }
        c.push_back(u);
        return c;
      }
      case FM_NODE_SPARSE: return sparse(d, fwd);
      case FM_NODE_HERMITIAN: return compile(r.ch.at(0), !fwd);
      case FM_NODE_CONJUGATE: {
        c.push_back(prog({mkop(fmk::OP_CONJ, (int)n_in)}, n_in, n_in, n_in));
        Chain t = compile(r.ch.at(0), fwd);
        c.insert(c.end(), t.begin(), t.end());
        c.push_back(
            prog({mkop(fmk::OP_CONJ, (int)n_out)}, n_out, n_out, n_out));
        return c;
      }
      case FM_NODE_EYE: return c;
      case FM_NODE_DENSE: {
        const i64 R = d.rows, C = d.cols;
        std::vector<cd> a = node_vec(d, 0);
        if ((i64)a.size() != R * C) fail(FM_ERR_VALUE, "dense data size");
        std::vector<cd> m((size_t)(R * C));
        if (fwd) m = a;
        else
          for (i64 i = 0; i < R; ++i)
            for (i64 j = 0; j < C; ++j) m[j + i * C] = std::conj(a[i + j * R]);
        fmk::Op o = mkop(fmk::OP_DENSE, (int)n_out);
        o.len2 = (int)n_in;
        o.ptr = upload(m);
        // square factors of order <= 64 on float32 data in the tensor-core
        // form run as MMA tiles (kernel class 6)
        o.sign = P_->ctype == FM_F32_TC && R == C && R <= fmk::kTdMaxN;
        c.push_back(prog({o}, n_in, n_out, std::max(n_in, n_out)));
        return c;
      }
      default: fail(FM_ERR_UNSUPPORTED, "unknown node kind");
    }
  }

  // merge consecutive PROG units of a chain (when the result fits)
  Chain merged(const Chain &in) {
    Chain out;
    for (const Unit &u : in) {
      if (u.kind == Unit::PROG && !out.empty() &&
          out.back().kind == Unit::PROG) {
        Unit &p = out.back();
        const i64 L = std::max(p.L, u.L);
        std::vector<fmk::Op> cat = p.ops;
        cat.insert(cat.end(), u.ops.begin(), u.ops.end());
        if (L <= limit_for(cat) && cat.size() <= (size_t)FM_MAX_OPS) {
          p.ops.insert(p.ops.end(), u.ops.begin(), u.ops.end());
          p.n_out = u.n_out;
          p.L = L;
          continue;
        }
      }
      out.push_back(u);
    }
    // fold pointwise programs into neighbouring multi-launch units
    Chain fused;
    for (size_t i = 0; i < out.size(); ++i) {
      if (i + 1 < out.size() && out[i + 1].kind == Unit::STEPS) {
        Unit next = out[i + 1];
        if (fold_before(out[i], next)) {
          out[i + 1] = next;
          continue;
        }
      }
      if (!fused.empty() && fused.back().kind == Unit::STEPS) {
        Unit prev = fused.back();
        if (fold_after(prev, out[i])) {
          fused.back() = prev;
          continue;
        }
      }
      fused.push_back(out[i]);
    }
    return fused;
  }

  // CSR product (fastmat/Sparse.pyx): forward uses the node's CSR, the
  // adjoint its conjugate transpose, built here as a second CSR (entries of
  // a row in ascending source-row order)
  Chain sparse(const fm_node &d, bool fwd) {
    const i64 R = d.rows, C = d.cols, nnz = d.n;
    if (nnz < 0 || d.len0 != nnz || d.len1 != R + 1 + nnz)
      fail(FM_ERR_VALUE, "Sparse: inconsistent CSR arrays");
    const std::vector<cd> val = nnz ? node_vec(d, 0) : std::vector<cd>();
    const std::vector<i64> iv = node_idx(d, 1);
    if (iv[0] != 0 || iv[(size_t)R] != nnz)
      fail(FM_ERR_VALUE, "Sparse: row pointers must run from 0 to nnz");
    for (i64 r = 0; r < R; ++r)
      if (iv[(size_t)r + 1] < iv[(size_t)r])
        fail(FM_ERR_VALUE, "Sparse: row pointers must not decrease");
    for (i64 k = 0; k < nnz; ++k) {
      const i64 c = iv[(size_t)(R + 1 + k)];
      if (c < 0 || c >= C) fail(FM_ERR_VALUE, "Sparse: column index out of range");
    }
    std::vector<i64> ptr, idx;
    std::vector<cd> v;
    if (fwd) {
      ptr.assign(iv.begin(), iv.begin() + (R + 1));
      idx.assign(iv.begin() + (R + 1), iv.end());
      v = val;
    } else {
      ptr.assign((size_t)C + 1, 0);
      for (i64 k = 0; k < nnz; ++k) ++ptr[(size_t)iv[(size_t)(R + 1 + k)] + 1];
      for (i64 c = 0; c < C; ++c) ptr[(size_t)c + 1] += ptr[(size_t)c];
      std::vector<i64> fill(ptr.begin(), ptr.end() - 1);
      idx.assign((size_t)nnz, 0);
      v.assign((size_t)nnz, cd(0.0, 0.0));
      for (i64 r = 0; r < R; ++r)
        for (i64 k = iv[(size_t)r]; k < iv[(size_t)r + 1]; ++k) {
          const i64 c = iv[(size_t)(R + 1 + k)];
          const i64 at = fill[(size_t)c]++;
          idx[(size_t)at] = r;
          v[(size_t)at] = std::conj(val[(size_t)k]);
        }
    }
    const i64 rows = fwd ? R : C;
    if (idx.empty()) {  // keep the device arrays non-empty
      idx.push_back(0);
      v.push_back(cd(0.0, 0.0));
    }
    Unit u;
    u.kind = Unit::SPARSE;
    u.n_in = fwd ? C : R;
    u.n_out = rows;
    u.sp_ptr = upload_map(ptr);
    u.sp_idx = upload_map(idx);
    u.sp_val = upload(v);
    // lanes per row: the mean row length rounded up to a power of two
    const i64 mean = rows > 0 ? (nnz + rows - 1) / rows : 1;
    int g = 1;
    while (g < 32 && g < mean) g *= 2;
    u.sp_group = g;
    return Chain{u};
  }

  Chain kron(const NodeRec &r, bool fwd) {
    std::vector<i64> dims;
    for (int ch : r.ch) dims.push_back(nodes_[ch].d.rows);
    i64 N = 1;
    for (i64 x : dims) N *= x;
    Unit u;
    u.kind = Unit::STEPS;
    u.n_in = u.n_out = N;
    const int K = (int)dims.size();
    // apply the contiguous (last) mode first, then outward
    for (int step = 0; step < K; ++step) {
      const int k = K - 1 - step;
      Chain fc = merged(compile(r.ch[k], fwd));
      if (fc.empty()) continue;  // identity factor
      if (fc.size() != 1 || fc[0].kind != Unit::PROG)
        fail(FM_ERR_UNSUPPORTED,
             "Kron factor too large for a single shared-memory program");
      const Unit &p = fc[0];
      if (p.L > limit_for(p.ops))
        fail(FM_ERR_UNSUPPORTED, "Kron factor too large");
      i64 A = 1, Cc = 1;
      for (int i = 0; i < k; ++i) A *= dims[i];
      for (int i = k + 1; i < K; ++i) Cc *= dims[i];
      SStep s;
      s.vin = s.vout = fmk::View{A, dims[k], Cc};
      s.in_rows = s.out_rows = N;
      s.L = (int)p.L;
      s.in_len = s.out_len = (int)dims[k];
      s.ops = p.ops;
      s.src = u.steps.empty() ? -1 : -2;
      s.dst = -2;
      u.steps.push_back(s);
    }
    Chain c;
    if (!u.steps.empty()) c.push_back(u);
    return c;
  }

  // ---------------------------------------------------------- lowering
  int new_scratch(i64 rows) {
    P_->scratch_rows.push_back(rows);
    return 1 + (int)P_->scratch_rows.size();
  }

  int kernel_class(const std::vector<fmk::Op> &ops) {
    bool fft = false, odd = false, fwht = false, gen = false;
    int dense = 0, dense_tc = 0;
    for (const fmk::Op &o : ops) {
      if (o.kind == fmk::OP_DENSE) {
        ++dense;
        if (o.sign) ++dense_tc;
      }
      if (o.kind == fmk::OP_FFT || o.kind == fmk::OP_DIF ||
          o.kind == fmk::OP_DIT) {
        fft = true;
        for (int i = 0; i < o.nrad; ++i)
          if (o.rad[i] & 1) odd = true;
      }
      if (o.kind == fmk::OP_FWHT) fwht = true;
      if (o.kind == fmk::OP_GATHER || o.kind == fmk::OP_DENSE) gen = true;
    }
    // one tensor-core dense factor with pointwise work around it
    bool other = false;
    for (const fmk::Op &o : ops)
      if (o.kind == fmk::OP_GATHER || o.kind == fmk::OP_FFT ||
          o.kind == fmk::OP_DIF || o.kind == fmk::OP_DIT ||
          o.kind == fmk::OP_FWHT || o.kind == fmk::OP_ZPAD)
        other = true;
    if (dense == 1 && dense_tc == 1 && !other) return 6;
    if (gen || (fft && fwht)) return 0;
    if (fwht) return P_->ctype == FM_F32_TC ? 4 : 3;
    if (fft) return odd ? 2 : 1;
    return 3;
  }

  // a forward (DIF) transform followed by a product with one table over
  // the whole vector: kernel class 5 applies the product in the transform's
  // last stage (its radix a power of two)
  static bool spectrum_fusable(const std::vector<fmk::Op> &ops) {
    for (size_t i = 0; i + 1 < ops.size(); ++i) {
      const fmk::Op &a = ops[i], &m = ops[i + 1];
      if (a.kind != fmk::OP_DIF || a.nrad < 1) continue;
      const int last = a.rad[a.nrad - 1];
      if (m.kind == fmk::OP_MUL && m.div == 1 && m.mod == 1 &&
          m.len == a.len && last > 1 && (last & (last - 1)) == 0)
        return true;
    }
    return false;
  }

  // whether lowering the FFTs of a program to DIF/DIT needs an explicit
  // reordering gather (an order-sensitive op follows a digit-reversed FFT)
  static bool needs_gather(const std::vector<fmk::Op> &ops) {
    bool permuted = false;
    std::vector<int> cur;
    for (const fmk::Op &o : ops) {
      switch (o.kind) {
        case fmk::OP_FFT: {
          std::vector<int> rad(o.rad, o.rad + o.nrad);
          if (permuted && rad != cur) return true;
          permuted = !permuted;
          cur = rad;
          break;
        }
        case fmk::OP_GATHER: permuted = false; break;
        case fmk::OP_MUL:
        case fmk::OP_TW:
        case fmk::OP_CONJ:
        case fmk::OP_SCALE: break;
        default:
          if (permuted) return true;
          break;
      }
    }
    return false;
  }

  // longest working length a program of this op mix may use in one tile
  i64 limit_for(const std::vector<fmk::Op> &ops) {
    const int cls = needs_gather(ops) ? 0 : kernel_class(ops);
    return (cls == 0 || cls == 2) ? lmax_ / 2 : lmax_;
  }

  // A program that is one circular convolution of contiguous vectors,
  // [conj] [pre] [zero pad] FFT(-1), spectrum product, FFT(+1) [post]
  // [conj], with a length the register kernel is built for, runs there
  // (kind 2); its spectrum is stored in that kernel's digit order.
  void try_rconv(LStep &ls, const std::vector<fmk::Op> &ops) {
    const int ct = P_->ctype;
    const int lmax = fmk::rconv_max_len(ct), lmin = fmk::rconv_min_len(ct);
    const fmk::Step &st = ls.st;
    if (!lmax || st.vin.Cc != 1 || st.vout.Cc != 1 || st.map_in ||
        st.map_out || st.out_mode != 0)
      return;
    auto whole = [](const fmk::Op &o) {
      return o.kind == fmk::OP_MUL && o.div == 1 && o.mod == 1 &&
             o.stride == 0;
    };
    auto is = [&](size_t i, int kind) {
      return i < ops.size() && ops[i].kind == kind;
    };
    size_t i = 0;
    bool cj_in = false, cj_out = false;
    const void *pre = nullptr, *post = nullptr;
    if (is(i, fmk::OP_CONJ)) cj_in = true, ++i;
    if (i < ops.size() && whole(ops[i]) && ops[i].sign == 0 &&
        (is(i + 1, fmk::OP_ZPAD) || is(i + 1, fmk::OP_FFT)))
      pre = ops[i++].ptr;
    if (is(i, fmk::OP_ZPAD)) {
      if (ops[i].len != st.in_len) return;
      ++i;
    }
    if (!is(i, fmk::OP_FFT) || ops[i].sign != -1) return;
    const int L = ops[i].len;
    ++i;
    if (i >= ops.size() || !whole(ops[i]) || ops[i].len != L) return;
    const fmk::Op &sm = ops[i++];
    if (!is(i, fmk::OP_FFT) || ops[i].sign != 1 || ops[i].len != L) return;
    ++i;
    if (i < ops.size() && whole(ops[i]) && ops[i].sign == 0)
      post = ops[i++].ptr;
    if (is(i, fmk::OP_CONJ)) cj_out = true, ++i;
    if (i != ops.size()) return;
    if (!is_pow2(L) || L < lmin || L > lmax || st.L != L ||
        st.in_len > L || st.out_len > L)
      return;
    // products in the program index points of a vector, the launch's by
    // rows: the same when a column holds one vector
    if ((pre && (st.pre || st.vin.A != 1)) ||
        (post && (st.post || st.vout.A != 1)) || (cj_in && st.conj_in) ||
        (cj_out && st.conj_out))
      return;
    const int P = fmk::rconv_min_len(ct);
    std::vector<int> rad;
    for (int rest = L; rest > 1;) {
      const int r = std::min(rest, P);
      rad.push_back(r);
      rest /= r;
    }
    const Perm &pm = perm_for(rad);
    const std::vector<cd> &S = host_vec_.at(sm.ptr);
    std::vector<cd> w((size_t)L);
    for (int q = 0; q < L; ++q) w[(size_t)q] = S[(size_t)pm.nat[q]];
    ls.rc_spec = upload(w);
    ls.rc_tw = twiddle(L);
    ls.rc_L = L;
    ls.rc_pre = pre;
    ls.rc_post = post;
    ls.rc_conj_in = cj_in;
    ls.rc_conj_out = cj_out;
    ls.rc_spec_conj = sm.sign;
    ls.kind = 2;
  }

  // A program that is one FWHT over whole vectors, with a length the
  // register FWHTs are built for, runs there (kind 3): contiguous vectors
  // of real data (rfwht_kernel), or vectors at an element stride that is a
  // multiple of 32 (rsfwht_kernel), real or complex (the real and imaginary
  // parts of complex vectors at stride S are real vectors at stride 2 S).
  // The tensor-core form of the FWHT (FM_F32_TC) runs in these kernels as
  // well: the transform is bound by HBM traffic, which they reach on the
  // FP32 pipes.
  void try_rfwht(LStep &ls, const std::vector<fmk::Op> &ops) {
    const int ct0 = P_->ctype;
    const bool cx = ct0 == FM_C64 || ct0 == FM_C128_DF;
    const int ct = (ct0 == FM_C64 || ct0 == FM_F32_TC)
                       ? FM_F32
                       : ct0 == FM_C128_DF ? FM_F64_DF : ct0;
    const fmk::Step &st = ls.st;
    if (ops.size() != 1 || ops[0].kind != fmk::OP_FWHT ||
        (ops[0].sign != 0 && ct0 != FM_F32_TC))
      return;
    const int L = ops[0].len;
    if (!is_pow2(L) || st.L != L) return;
    if (st.vin.A != st.vout.A || st.vin.n != L || st.vout.n != L ||
        st.vin.Cc != st.vout.Cc || st.in_len != L || st.out_len != L ||
        st.in_rows != st.vin.A * L * st.vin.Cc ||
        st.out_rows != st.vout.A * L * st.vout.Cc || st.map_in ||
        st.map_out || st.out_mode || st.pre || st.post || st.conj_in ||
        st.conj_out || st.has_scale || st.accumulate)
      return;
    const i64 S = st.vin.Cc;
    if (S == 1) {
      if (cx || L < fmk::rfwht_min_len(ct) || L > fmk::rfwht_max_len(ct))
        return;
      ls.rc_es = 0;
    } else {
      if (S % 32 || L < fmk::rsfwht_min_len(ct) ||
          L > fmk::rsfwht_max_len(ct))
        return;
      const int k = cx ? 2 : 1;  // real words per element
      ls.rc_es = S * k;
      ls.rc_A = st.vin.A * S * k;
    }
    ls.rc_ct = ct;
    ls.rc_L = L;
    ls.kind = 3;
  }

  // A program that is one FFT over whole vectors at an element stride that
  // is a multiple of 32 (a Fourier mode of a Kron), complex64 or
  // double-float complex, with a length the strided register FFT is built
  // for, runs there (kind 4).
  void try_rsfft(LStep &ls, const std::vector<fmk::Op> &ops) {
    const int ct = P_->ctype;
    const fmk::Step &st = ls.st;
    const int lmin = fmk::rsfft_min_len(ct), lmax = fmk::rsfft_max_len(ct);
    if (!lmax || ops.size() != 1 || ops[0].kind != fmk::OP_FFT) return;
    const int L = ops[0].len;
    const i64 S = st.vin.Cc;
    if (!is_pow2(L) || L < lmin || L > lmax || st.L != L || S % 32) return;
    if (st.vin.A != st.vout.A || st.vin.n != L || st.vout.n != L ||
        st.vout.Cc != S || st.in_len != L || st.out_len != L ||
        st.in_rows != st.vin.A * L * S || st.out_rows != st.vout.A * L * S ||
        st.map_in || st.map_out || st.out_mode || st.pre || st.post ||
        st.conj_in || st.conj_out || st.has_scale || st.accumulate)
      return;
    ls.rc_L = L;
    ls.rc_es = S;
    ls.rc_A = st.vin.A * S;
    ls.rc_tw = twiddle(L);
    ls.rc_sign = ops[0].sign;
    ls.kind = 4;
  }

  void finish(LStep &ls, const std::vector<fmk::Op> &ops_in) {
    fmk::Step &st = ls.st;
    try_rconv(ls, ops_in);
    if (ls.kind == 0) try_rfwht(ls, ops_in);
    if (ls.kind == 0) try_rsfft(ls, ops_in);
    std::vector<fmk::Op> ops = ops_in;
    st.out_pos = finalize(ops);
    if ((int)ops.size() > FM_MAX_OPS)
      fail(FM_ERR_UNSUPPORTED, "operator chain too long for one launch");
    st.nops = (int)ops.size();
    for (size_t i = 0; i < ops.size(); ++i) st.ops[i] = ops[i];
    ls.cls = kernel_class(ops);
    if (ls.cls == 1 && spectrum_fusable(ops)) ls.cls = 5;
    const bool odd = ls.cls == 2 || ls.cls == 0;
    ls.ept = odd ? ept_ / 2 : ept_;
    if (!configure(P_->esz, ls, 0, 0))
      fail(FM_ERR_UNSUPPORTED, "working length too large for one tile");
    if (P_->ctype == FM_C64 && ls.kind == 0 && rtile_shape(ls.st)) {
      // a register tile program (fm_rtile.cuh) runs on vector-major tiles
      // that give every thread its 8 points (the autotuner may still pick
      // another layout, which then runs the stage program)
      int wantB = 0;
      for (int b = 1; b <= 1024; b *= 2) {
        LStep t = ls;
        if (!configure(P_->esz, t, b, 0, false, 0, false)) continue;
        if (t.threads > FM_MAX_THREADS ||
            fmk::tile_bytes(b, t.st.Lp, P_->esz) > (size_t)48 * 1024)
          break;
        wantB = b;
      }
      LStep t = ls;
      if (wantB && configure(P_->esz, t, wantB, 0, false, 0, false) &&
          rtile_threads_ok(t))
        ls = t;
    }
  }

  fmk::Step base_step() {
    fmk::Step st;
    memset(&st, 0, sizeof(st));
    st.scale_re = 1.0;
    return st;
  }

  void emit_copy(int src, int dst, i64 n, std::vector<LStep> &out) {
    Unit u = prog({}, n, n, n);
    emit_prog(u, src, dst, out);
  }

  // whole-column program, or a chunked pointwise/gather program
  void emit_prog(const Unit &u, int src, int dst, std::vector<LStep> &out) {
    if (u.L <= limit_for(u.ops)) {
      LStep ls;
      ls.src = src;
      ls.dst = dst;
      fmk::Step &st = ls.st;
      st = base_step();
      st.vin = fmk::View{1, u.n_in, 1};
      st.vout = fmk::View{1, u.n_out, 1};
      st.in_rows = u.n_in;
      st.out_rows = u.n_out;
      st.in_len = (int)u.n_in;
      st.out_len = (int)u.n_out;
      st.L = (int)std::max<i64>(u.L, 1);
      st.V = 1;
      finish(ls, u.ops);
      out.push_back(ls);
      return;
    }
    emit_chunked(u, src, dst, out);
  }

  // A program made only of pointwise operations and gathers, composed into
  // y[i] = s * d[i] * cx(x[map[i]]) (map empty: identity, d empty: ones).
  struct Pointwise {
    std::vector<i64> map;
    std::vector<cd> dv;
    cd s{1, 0};
    bool cx = false;
    i64 len = 0;
  };

  bool pointwise(const Unit &u, Pointwise &pw) {
    if (u.kind != Unit::PROG) return false;
    i64 len = u.n_in;
    std::vector<i64> &map = pw.map;
    std::vector<cd> &dv = pw.dv;
    for (const fmk::Op &o : u.ops) {
      switch (o.kind) {
        case fmk::OP_GATHER: {
          const std::vector<i64> &m = host_map_.at(o.ptr);
          std::vector<i64> nm(m.size());
          std::vector<cd> nd;
          if (!dv.empty()) nd.resize(m.size());
          for (size_t i = 0; i < m.size(); ++i) {
            const i64 j = m[i];
            nm[i] = j < 0 ? -1 : (map.empty() ? j : map[j]);
            if (!dv.empty()) nd[i] = j < 0 ? cd(0, 0) : dv[j];
          }
          map.swap(nm);
          if (!dv.empty()) dv.swap(nd);
          len = (i64)m.size();
          break;
        }
        case fmk::OP_MUL: {
          if (o.div != 1 || o.mod != 1 || o.stride != 0) return false;
          const std::vector<cd> &v = host_vec_.at(o.ptr);
          if (dv.empty()) dv.assign((size_t)len, cd(1, 0));
          for (i64 i = 0; i < len; ++i)
            dv[i] *= o.sign ? std::conj(v[i]) : v[i];
          break;
        }
        case fmk::OP_SCALE: pw.s *= cd(o.sre, o.sim); break;
        case fmk::OP_CONJ:
          pw.s = std::conj(pw.s);
          for (cd &x : dv) x = std::conj(x);
          pw.cx = !pw.cx;
          break;
        default: return false;
      }
    }
    pw.len = len;
    return true;
  }

  // Fold a pointwise program that feeds a multi-launch unit into the
  // loader of its first launch (gather map, conjugation and
  // pre-multiplication).
  bool fold_before(const Unit &p, Unit &u) {
    Pointwise pw;
    if (!pointwise(p, pw) || u.kind != Unit::STEPS || u.steps.empty())
      return false;
    SStep &a = u.steps[0];
    if (a.src != -1 || a.pre || a.map_in || a.conj_in) return false;
    for (size_t k = 1; k < u.steps.size(); ++k)
      if (u.steps[k].src == -1) return false;  // input read again later
    if (pw.len != u.n_in || a.in_rows != u.n_in) return false;
    if (pw.s != cd(1, 0)) {
      if (pw.dv.empty()) pw.dv.assign((size_t)pw.len, cd(1, 0));
      for (cd &x : pw.dv) x *= pw.s;
    }
    if (!pw.map.empty()) a.map_in = upload_map(pw.map);
    if (!pw.dv.empty()) a.pre = upload(pw.dv);
    a.conj_in = pw.cx;
    u.n_in = p.n_in;
    return true;
  }

  // Fold a pointwise program that consumes a multi-launch unit's result
  // into the storer of its last launch (post-multiplication, conjugation,
  // and a row selection as a scatter through the inverse map).  Only
  // selections that pick every row at most once can be inverted.
  bool fold_after(Unit &u, const Unit &p) {
    Pointwise pw;
    if (u.kind != Unit::STEPS || u.steps.empty() || !pointwise(p, pw))
      return false;
    SStep &c = u.steps.back();
    if (c.dst != -2 || c.post || c.map_out || c.conj_out) return false;
    for (size_t k = 0; k + 1 < u.steps.size(); ++k)
      if (u.steps[k].dst == -2 || u.steps[k].src == -2)
        return false;  // output buffer also used as working storage
    if (p.n_in != u.n_out || c.out_rows != u.n_out) return false;
    std::vector<i64> inv;
    if (!pw.map.empty()) {
      inv.assign((size_t)u.n_out, -1);
      for (size_t i = 0; i < pw.map.size(); ++i) {
        const i64 j = pw.map[i];
        if (j < 0 || j >= u.n_out || inv[j] >= 0) return false;
        inv[j] = (i64)i;
      }
    }
    std::vector<cd> post;
    if (!pw.dv.empty() || pw.s != cd(1, 0)) {
      post.assign((size_t)u.n_out, cd(0, 0));
      for (i64 r = 0; r < u.n_out; ++r) {
        const i64 i = inv.empty() ? r : inv[r];
        if (i < 0) continue;
        cd v = (pw.dv.empty() ? cd(1, 0) : pw.dv[i]) * pw.s;
        // stored value: conj_out(post * x) = d * cx(x)
        post[r] = pw.cx ? std::conj(v) : v;
      }
    }
    if (!inv.empty()) {
      c.map_out = upload_map(inv);
      c.out_mode = 2;
    }
    if (!post.empty()) c.post = upload(post);
    c.conj_out = pw.cx;
    u.n_out = pw.len;
    return true;
  }

  // y[i] = s * d[i] * cx(x[map[i]]) over chunks of the column
  void emit_chunked(const Unit &u, int src, int dst, std::vector<LStep> &out) {
    Pointwise pw;
    if (!pointwise(u, pw))
      fail(FM_ERR_UNSUPPORTED,
           "long vector program with non-pointwise operations");
    const std::vector<i64> &map = pw.map;
    std::vector<cd> &dv = pw.dv;
    const cd s = pw.s;
    const bool cx = pw.cx;
    const i64 len = pw.len;
    const i64 n_out = len;
    const i64 Lc = std::min<i64>(2048, std::max<i64>(n_out, 1));
    const i64 nch = (n_out + Lc - 1) / Lc;
    LStep ls;
    ls.src = src;
    ls.dst = dst;
    fmk::Step &st = ls.st;
    st = base_step();
    st.vin = st.vout = fmk::View{nch, Lc, 1};
    st.in_rows = map.empty() ? u.n_in : n_out;
    st.out_rows = n_out;
    st.in_len = st.out_len = (int)Lc;
    st.L = (int)Lc;
    st.V = nch;
    if (!map.empty()) st.map_in = upload_map(map);
    st.conj_in = cx;
    std::vector<fmk::Op> ops;
    if (!dv.empty()) {
      dv.resize((size_t)(nch * Lc), cd(0, 0));
      fmk::Op m = mul_op(upload(dv), Lc, false);
      m.div = 1;
      m.mod = nch;
      m.stride = Lc;
      ops.push_back(m);
    }
    if (s != cd(1, 0)) {
      st.has_scale = 1;
      st.scale_re = s.real();
      st.scale_im = s.imag();
    }
    finish(ls, ops);
    out.push_back(ls);
  }

  void emit_steps(const Unit &u, int src, int dst, std::vector<LStep> &out) {
    std::vector<int> tmp;
    for (i64 rows : u.tmp_rows) tmp.push_back(new_scratch(rows));
    auto resolve = [&](int id) {
      if (id == -1) return src;
      if (id == -2) return dst;
      return tmp.at(id);
    };
    for (const SStep &s : u.steps) {
      LStep ls;
      ls.src = resolve(s.src);
      ls.dst = resolve(s.dst);
      fmk::Step &st = ls.st;
      st = base_step();
      st.vin = s.vin;
      st.vout = s.vout;
      st.in_rows = s.in_rows;
      st.out_rows = s.out_rows;
      st.in_len = s.in_len;
      st.out_len = s.out_len;
      st.L = s.L;
      st.V = s.vin.A * s.vin.Cc;
      st.pre = s.pre;
      st.post = s.post;
      st.map_in = s.map_in;
      st.map_out = s.map_out;
      st.out_mode = s.out_mode;
      st.conj_in = s.conj_in;
      st.conj_out = s.conj_out;
      finish(ls, s.ops);
      out.push_back(ls);
    }
  }

  void lower(const Chain &chain_in, int in_id, i64 in_rows, int out_id,
             i64 out_rows, std::vector<LStep> &out) {
    const Chain chain = merged(chain_in);
    if (chain.empty()) {
      emit_copy(in_id, out_id, in_rows, out);
      return;
    }
    int cur = in_id;
    for (size_t i = 0; i < chain.size(); ++i) {
      const Unit &u = chain[i];
      const bool last = i + 1 == chain.size();
      const int dst = last ? out_id : new_scratch(u.n_out);
      switch (u.kind) {
        case Unit::PROG: emit_prog(u, cur, dst, out); break;
        case Unit::STEPS: emit_steps(u, cur, dst, out); break;
        case Unit::SUM: {
          for (size_t t = 0; t < u.terms.size(); ++t) {
            if (t == 0) {
              lower(u.terms[t], cur, u.n_in, dst, u.n_out, out);
              continue;
            }
            // later terms: evaluate into scratch, then accumulate
            const int tmp = new_scratch(u.n_out);
            lower(u.terms[t], cur, u.n_in, tmp, u.n_out, out);
            Unit cp = prog({}, u.n_out, u.n_out, u.n_out);
            std::vector<LStep> acc;
            emit_prog(cp, tmp, dst, acc);
            for (LStep &a : acc) {
              a.st.accumulate = 1;
              a.tma_out_ok = 0;  // accumulation reads the destination
            }
            out.insert(out.end(), acc.begin(), acc.end());
          }
          break;
        }
        case Unit::SPARSE: {
          LStep ls;
          ls.kind = 1;
          ls.src = cur;
          ls.dst = dst;
          ls.st = base_step();
          ls.sp_ptr = u.sp_ptr;
          ls.sp_idx = u.sp_idx;
          ls.sp_val = u.sp_val;
          ls.sp_rows = u.n_out;
          ls.sp_group = u.sp_group;
          out.push_back(ls);
          break;
        }
        case Unit::BLOCKS: {
          // output segment o = sum over q of block (o, q) applied to input
          // segment q: the first block writes, later ones go through
          // scratch and accumulate
          i64 oo = 0;
          for (size_t o = 0; o < u.grid.size(); ++o) {
            const i64 m = u.seg_out[o];
            bool first = true;
            i64 io = 0;
            for (size_t q = 0; q < u.grid[o].size(); ++q) {
              const i64 nq = u.seg_in[q];
              if (u.has[o][q]) {
                if (first) {
                  lower_at(u.grid[o][q], cur, io, nq, dst, oo, m, out);
                  first = false;
                } else {
                  const int tmp = new_scratch(m);
                  lower_at(u.grid[o][q], cur, io, nq, tmp, 0, m, out);
                  Unit cp = prog({}, m, m, m);
                  std::vector<LStep> acc;
                  emit_prog(cp, tmp, dst, acc);
                  for (LStep &a : acc) {
                    a.st.accumulate = 1;
                    a.tma_out_ok = 0;
                    a.dst_off += oo;
                  }
                  out.insert(out.end(), acc.begin(), acc.end());
                }
              }
              io += nq;
            }
            oo += m;
          }
          break;
        }
      }
      cur = dst;
    }
    (void)out_rows;
  }

  // lower a chain that reads rows [in_off, in_off + in_rows) of buffer in_id
  // and writes rows [out_off, out_off + out_rows) of buffer out_id
  void lower_at(const Chain &ch, int in_id, i64 in_off, i64 in_rows,
                int out_id, i64 out_off, i64 out_rows,
                std::vector<LStep> &out) {
    std::vector<LStep> part;
    lower(ch, in_id, in_rows, out_id, out_rows, part);
    for (LStep &ls : part) {
      if (ls.src == in_id) ls.src_off += in_off;
      else if (ls.src == out_id) ls.src_off += out_off;
      if (ls.dst == out_id) ls.dst_off += out_off;
      else if (ls.dst == in_id) ls.dst_off += in_off;
    }
    out.insert(out.end(), part.begin(), part.end());
  }
};

// ------------------------------------------------------------ TMA descriptors
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType,
                                  cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion,
                                  CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static std::mutex mu;
  static EncodeTiledFn fn = nullptr;
  static bool tried = false;
  std::lock_guard<std::mutex> lock(mu);
  if (!tried) {
    tried = true;
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                         cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  }
  return fn;
}

// Describe the view (A, n, Cc) of `num_cols` columns at `base` (leading
// dimension ld) as a 4-D tensor {Cc, n, A, columns} read in boxes of
// {B, box_rows, 1, 1} elements.  Returns false when the buffer does not meet
// TMA's alignment rules (the launch then uses per-thread copies).
bool encode_view(CUtensorMap *tm, const void *base, const fmk::View &vw,
                 i64 ld, i64 num_cols, int B, int box_rows, int esz) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  const int k = esz == 16 ? 2 : 1;
  const int tsz = esz / k;
  if (((uintptr_t)base & 15) || (ld * esz) % 16 || (vw.Cc * esz) % 16)
    return false;
  const cuuint64_t dims[4] = {(cuuint64_t)(vw.Cc * k), (cuuint64_t)vw.n,
                              (cuuint64_t)vw.A, (cuuint64_t)num_cols};
  for (cuuint64_t d : dims)
    if (d == 0 || d > (1ull << 32)) return false;
  const cuuint64_t strides[3] = {(cuuint64_t)(vw.Cc * esz),
                                 (cuuint64_t)(vw.n * vw.Cc * esz),
                                 (cuuint64_t)(ld * esz)};
  for (cuuint64_t st : strides)
    if (st >= (1ull << 40)) return false;
  const cuuint32_t box[4] = {(cuuint32_t)(B * k), (cuuint32_t)box_rows, 1, 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  const CUtensorMapDataType dt =
      tsz == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_INT64;
  return fn(tm, dt, 4, const_cast<void *>(base), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Finish a bound launch (TMA descriptors, status word) and issue it.
void launch_step(fm_plan *P, LStep &ls, fmk::Step &st, cudaStream_t s) {
  if (ls.pair == 2 && P->pair_done && !P->no_pair) {
    // the fused launch of the previous step ran this pass
    P->pair_done = false;
    return;
  }
  P->pair_done = false;
  st.rprog = 0;
  if (ls.kind == 0 && P->ctype == FM_C64 && rtile_threads_ok(ls))
    st.rprog = rtile_shape(st);
  if (ls.kind == 3) {
    // raw buffers of the I/O type; the contiguous kernel also wants
    // 16-byte aligned columns and vectors
    const int esz = esize(P->io_type);
    const bool strided = ls.rc_es > 1;
    const bool fit = st.src_type == P->io_type && st.dst_type == P->io_type &&
                     !st.accumulate &&
                     (strided || (((uintptr_t)st.src & 15) == 0 &&
                                  ((uintptr_t)st.dst & 15) == 0 &&
                                  (st.ld_src * esz) % 16 == 0 &&
                                  (st.ld_dst * esz) % 16 == 0));
    if (fit) {
      fmk::RfStep rf;
      const int k = strided ? (int)(ls.rc_es / st.vin.Cc) : 1;
      rf.src = st.src;
      rf.dst = st.dst;
      rf.ld_src = st.ld_src * k;
      rf.ld_dst = st.ld_dst * k;
      rf.A = strided ? ls.rc_A : st.vin.A;
      rf.stride = st.vin.n;
      rf.es = strided ? ls.rc_es : 1;
      rf.num_cols = st.num_cols;
      rf.err = P->err;
      rf.L = ls.rc_L;
      if (rf.A * rf.num_cols >= 0x7fffffffLL || rf.es >= 0x7fffffffLL)
        fail(FM_ERR_UNSUPPORTED, "more than 2^31 vectors in one launch");
      if (ls.pair == 1 && !P->no_pair && 1 + st.num_cols <= P->pair_cap &&
          (i64)st.num_cols * (rf.A + ls.rc2_A) < 0xffffffffLL) {
        // both passes, column by column; the second runs in place on dst
        fmk::RfPair pr;
        pr.a = rf;
        pr.b = rf;
        pr.b.src = st.dst;
        pr.b.ld_src = st.ld_dst;
        pr.b.A = ls.rc2_A;
        pr.b.es = ls.rc2_es;
        pr.b.L = ls.rc2_L;
        pr.ctr = P->pair_ctr;
        pr.err = P->err;
        pr.wait_limit = P->wait_limit;
        pr.lag = 1;  // (2 for float32 measured slower: 0.72 vs 0.67 ms)
        CUDA_TRY(cudaMemsetAsync(P->pair_ctr, 0,
                                 (size_t)(1 + st.num_cols) * 4, s));
        CUDA_TRY(fmk::launch_rfwht2(ls.rc_ct, pr, s));
        P->pair_done = true;
        return;
      }
      CUDA_TRY(fmk::launch_rfwht(ls.rc_ct, rf, s));
      return;
    }
    // otherwise the equivalent vector program below
  }
  if (ls.kind == 4) {
    // raw buffers of the I/O type
    if (st.src_type == P->io_type && st.dst_type == P->io_type &&
        !st.accumulate) {
      fmk::RsfStep rs;
      rs.src = st.src;
      rs.dst = st.dst;
      rs.ld_src = st.ld_src;
      rs.ld_dst = st.ld_dst;
      rs.A = ls.rc_A;
      rs.es = ls.rc_es;
      rs.num_cols = st.num_cols;
      rs.tw = ls.rc_tw;
      rs.err = P->err;
      rs.L = ls.rc_L;
      rs.sign = ls.rc_sign;
      if (rs.A * rs.num_cols >= 0x7fffffffLL || rs.es >= 0x7fffffffLL)
        fail(FM_ERR_UNSUPPORTED, "more than 2^31 vectors in one launch");
      CUDA_TRY(fmk::launch_rsfft(P->ctype, rs, s));
      return;
    }
    // otherwise the equivalent vector program below
  }
  if (ls.kind == 2) {
    fmk::RcStep rc;
    memset(&rc, 0, sizeof(rc));
    rc.src = st.src;
    rc.dst = st.dst;
    rc.ld_src = st.ld_src;
    rc.ld_dst = st.ld_dst;
    rc.src_type = st.src_type;
    rc.dst_type = st.dst_type;
    rc.A = st.vin.A;
    rc.in_stride = st.vin.n;
    rc.out_stride = st.vout.n;
    rc.in_rows = st.in_rows;
    rc.out_rows = st.out_rows;
    rc.in_len = st.in_len;
    rc.out_len = st.out_len;
    rc.num_cols = st.num_cols;
    rc.spec = ls.rc_spec;
    rc.tw = ls.rc_tw;
    rc.pre = st.pre ? st.pre : ls.rc_pre;
    rc.post = st.post ? st.post : ls.rc_post;
    rc.err = P->err;
    rc.spec_conj = ls.rc_spec_conj;
    rc.conj_in = st.conj_in || ls.rc_conj_in;
    rc.conj_out = st.conj_out || ls.rc_conj_out;
    rc.has_scale = st.has_scale;
    rc.accumulate = st.accumulate;
    rc.L = ls.rc_L;
    rc.scale_re = st.scale_re;
    rc.scale_im = st.scale_im;
    if (rc.A * rc.num_cols >= 0x7fffffffLL)
      fail(FM_ERR_UNSUPPORTED, "more than 2^31 vectors in one launch");
    const i64 blocks = (i64)ls.rc2_blocks * st.num_cols;
    if (ls.pair == 3 && !P->no_pair && st.src_type == P->io_type &&
        st.dst_type == P->io_type && 1 + blocks <= P->pair_cap &&
        blocks * (ls.rc2_n1 + ls.rc2_n2) < 0xffffffffLL &&
        ls.rc2_A * st.num_cols < 0x7fffffffLL) {
      // this circulant mode and the Hadamard mode after it, block by block;
      // the FWHT runs in place on dst, in its real view (two real words
      // per complex element)
      fmk::RchPair pr;
      pr.c = rc;
      fmk::RfStep &h = pr.h;
      const int kw = 2;
      h.src = st.dst;
      h.dst = st.dst;
      h.ld_src = h.ld_dst = st.ld_dst * kw;
      h.A = ls.rc2_A;
      h.stride = 0;
      h.es = ls.rc2_es;
      h.num_cols = st.num_cols;
      h.err = P->err;
      h.L = ls.rc2_L;
      pr.ctr = P->pair_ctr;
      pr.err = P->err;
      pr.wait_limit = P->wait_limit;
      pr.blocks = blocks;
      pr.n1 = ls.rc2_n1;
      pr.n2 = ls.rc2_n2;
      pr.lag = 1;  // set by the launcher from the resident grid
      CUDA_TRY(cudaMemsetAsync(P->pair_ctr, 0, (size_t)(1 + blocks) * 4, s));
      CUDA_TRY(fmk::launch_rkch(P->ctype, pr, s));
      P->pair_done = true;
      return;
    }
    CUDA_TRY(fmk::launch_rconv(P->ctype, rc, s));
    return;
  }
  if (ls.kind == 1) {
    fmk::SpStep sp;
    sp.ptr = ls.sp_ptr;
    sp.idx = ls.sp_idx;
    sp.val = ls.sp_val;
    sp.src = st.src;
    sp.dst = st.dst;
    sp.src_type = st.src_type;
    sp.dst_type = st.dst_type;
    sp.ld_src = st.ld_src;
    sp.ld_dst = st.ld_dst;
    sp.rows = ls.sp_rows;
    sp.num_cols = st.num_cols;
    CUDA_TRY(fmk::launch_spmv(P->ctype, sp, ls.sp_group, s));
    return;
  }
  st.err = P->err;
  st.wait_limit = P->wait_limit;
  st.tma_in = st.tma_out = 0;
  if (ls.lay == 0 || ls.lay == 2) {
    const int esz = P->esz;
    auto aligned = [&](const void *ptr, i64 ld, i64 n) {
      return ((uintptr_t)ptr & 15) == 0 && (ld * esz) % 16 == 0 &&
             (n * esz) % 16 == 0;
    };
    st.tma_in = ls.tma_in_ok && st.src_type == P->io_type &&
                aligned(st.src, st.ld_src, st.vin.n);
    st.tma_out = ls.tma_out_ok && !st.accumulate &&
                 st.dst_type == P->io_type &&
                 aligned(st.dst, st.ld_dst, st.vout.n);
  }
  if (ls.lay == 1) {
    if (ls.tma_in_ok && st.src_type == P->io_type) {
      if (ls.tm_in_key != st.src || ls.tm_in_ld != st.ld_src ||
          ls.tm_in_m != st.num_cols) {
        ls.tm_in_key = nullptr;
        if (encode_view(&ls.tm_in, st.src, st.vin, st.ld_src, st.num_cols,
                        st.B, st.box_rows, P->esz)) {
          ls.tm_in_key = st.src;
          ls.tm_in_ld = st.ld_src;
          ls.tm_in_m = st.num_cols;
        }
      }
      if (ls.tm_in_key) {
        st.tm_in = ls.tm_in;
        st.tma_in = 1;
      }
    }
    if (ls.tma_out_ok && !st.accumulate && st.dst_type == P->io_type) {
      if (ls.tm_out_key != st.dst || ls.tm_out_ld != st.ld_dst ||
          ls.tm_out_m != st.num_cols) {
        ls.tm_out_key = nullptr;
        if (encode_view(&ls.tm_out, st.dst, st.vout, st.ld_dst, st.num_cols,
                        st.B, st.box_rows, P->esz)) {
          ls.tm_out_key = st.dst;
          ls.tm_out_ld = st.ld_dst;
          ls.tm_out_m = st.num_cols;
        }
      }
      if (ls.tm_out_key) {
        st.tm_out = ls.tm_out;
        st.tma_out = 1;
      }
    }
  }
  const i64 grid = (st.V * st.num_cols + st.B - 1) / st.B;
  if (st.V * st.num_cols >= 0x7fffffffLL)
    fail(FM_ERR_UNSUPPORTED, "more than 2^31 vectors in one launch");
  cudaError_t e;
  switch (P->ctype) {
    case FM_F32:
    case FM_F32_TC: e = fmk::launch_f32(st, ls.cls, ls.lay, ls.threads, ls.smem, grid, s); break;
    case FM_F64: e = fmk::launch_f64(st, ls.cls, ls.lay, ls.threads, ls.smem, grid, s); break;
    case FM_C64: e = fmk::launch_c64(st, ls.cls, ls.lay, ls.threads, ls.smem, grid, s); break;
    case FM_I64: e = fmk::launch_i64(st, ls.cls, ls.lay, ls.threads, ls.smem, grid, s); break;
    case FM_F64_DF: e = fmk::launch_df(st, ls.cls, ls.lay, ls.threads, ls.smem, grid, s); break;
    case FM_C128_DF: e = fmk::launch_dfc(st, ls.cls, ls.lay, ls.threads, ls.smem, grid, s); break;
    default: e = fmk::launch_c128(st, ls.cls, ls.lay, ls.threads, ls.smem, grid, s); break;
  }
  CUDA_TRY(e);
}

// ------------------------------------------------------------ execution
int run_plan(fm_plan *P, int dir, const void *x, int x_type, i64 ld_x,
             void *y, int y_type, i64 ld_y, i64 M, cudaStream_t s,
             std::vector<cudaEvent_t> *events) {
  if (M <= 0) return FM_OK;
  // scratch
  const size_t align = 256;
  std::vector<size_t> offs(P->scratch_rows.size());
  size_t total = 0;
  for (size_t k = 0; k < P->scratch_rows.size(); ++k) {
    offs[k] = total;
    total += ((size_t)P->scratch_rows[k] * M * P->esz + align - 1) / align *
             align;
  }
  if (total > P->scratch_cap) {
    if (P->scratch) {
      cudaStreamSynchronize(s);
      cudaFree(P->scratch);
      P->scratch = nullptr;
      P->scratch_cap = 0;
    }
    CUDA_TRY(dev_malloc(&P->scratch, total));
    P->scratch_cap = total;
  }
  size_t li = 0;
  if (events) CUDA_TRY(cudaEventRecord((*events)[li++], s));
  for (LStep &ls : P->steps[dir]) {
    fmk::Step st = ls.st;
    auto bind = [&](int id, const void *&ptr, int &type, i64 &ld) {
      if (id == 0) {
        ptr = x;
        type = x_type;
        ld = ld_x;
      } else if (id == 1) {
        ptr = y;
        type = y_type;
        ld = ld_y;
      } else {
        ptr = (char *)P->scratch + offs[id - 2];
        type = P->io_type;
        ld = P->scratch_rows[id - 2];
      }
    };
    const void *sp;
    const void *dp;
    bind(ls.src, sp, st.src_type, st.ld_src);
    bind(ls.dst, dp, st.dst_type, st.ld_dst);
    st.src = (const char *)sp + ls.src_off * esize(st.src_type);
    st.dst = (char *)const_cast<void *>(dp) + ls.dst_off * esize(st.dst_type);
    st.num_cols = M;
    launch_step(P, ls, st, s);
    if (events) CUDA_TRY(cudaEventRecord((*events)[li++], s));
  }
  return FM_OK;
}

// ------------------------------------------------------------ static scratch
// Scratch for fm_execute_static: a fixed array in device memory, reserved by
// every GPU that loads this library for as long as the process lives, so that
// callers which must not allocate device memory during a call can still run
// the multi-launch plans (long four-step transforms, Sum) that keep
// intermediates between launches.
static __device__ __align__(256) unsigned char
    g_static_scratch[FM_STATIC_SCRATCH_BYTES];

// Device address of g_static_scratch, looked up once per device (host code
// cannot use the symbol's name as an address).
void *static_scratch_address() {
  static std::mutex mu;
  static std::map<int, void *> addr;
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  auto it = addr.find(dev);
  if (it != addr.end()) return it->second;
  void *p = nullptr;
  CUDA_TRY(cudaGetSymbolAddress(&p, g_static_scratch));
  addr[dev] = p;
  return p;
}

// The launch loop of run_plan with every scratch buffer placed in the static
// array; returns FM_ERR_VALUE before launching anything if the plan needs
// more scratch than the array holds.
int run_plan_static(fm_plan *P, int dir, const void *x, int x_type, i64 ld_x,
                    void *y, int y_type, i64 ld_y, i64 M, cudaStream_t s) {
  if (M <= 0) return FM_OK;
  const size_t align = 256;
  std::vector<size_t> offs(P->scratch_rows.size());
  size_t total = 0;
  for (size_t k = 0; k < P->scratch_rows.size(); ++k) {
    offs[k] = total;
    total += ((size_t)P->scratch_rows[k] * M * P->esz + align - 1) / align *
             align;
  }
  if (total > (size_t)FM_STATIC_SCRATCH_BYTES)
    fail(FM_ERR_VALUE,
         "fm_execute_static: this call needs " + std::to_string(total) +
             " bytes of scratch, more than the " +
             std::to_string((size_t)FM_STATIC_SCRATCH_BYTES) +
             "-byte static array; use fewer columns or fm_execute");
  char *base = total ? (char *)static_scratch_address() : nullptr;
  for (LStep &ls : P->steps[dir]) {
    fmk::Step st = ls.st;
    auto bind = [&](int id, const void *&ptr, int &type, i64 &ld) {
      if (id == 0) {
        ptr = x;
        type = x_type;
        ld = ld_x;
      } else if (id == 1) {
        ptr = y;
        type = y_type;
        ld = ld_y;
      } else {
        ptr = base + offs[id - 2];
        type = P->io_type;
        ld = P->scratch_rows[id - 2];
      }
    };
    const void *sp;
    const void *dp;
    bind(ls.src, sp, st.src_type, st.ld_src);
    bind(ls.dst, dp, st.dst_type, st.ld_dst);
    st.src = (const char *)sp + ls.src_off * esize(st.src_type);
    st.dst = (char *)const_cast<void *>(dp) + ls.dst_off * esize(st.dst_type);
    st.num_cols = M;
    launch_step(P, ls, st, s);
  }
  return FM_OK;
}

const char *kind_name(int k) {
  switch (k) {
    case fmk::OP_FFT: return "fft";
    case fmk::OP_MUL: return "mul";
    case fmk::OP_ZPAD: return "zpad";
    case fmk::OP_GATHER: return "gather";
    case fmk::OP_FWHT: return "fwht";
    case fmk::OP_DENSE: return "dense";
    case fmk::OP_SCALE: return "scale";
    case fmk::OP_CONJ: return "conj";
    case fmk::OP_TW: return "twiddle";
    case fmk::OP_DIF: return "fft-dif";
    case fmk::OP_DIT: return "fft-dit";
  }
  return "?";
}

// Whether the subtree at `id` only moves data: gathers, scatters, zero
// fills and conjugation (Permutation, Partial, Eye, Hermitian, Conjugate),
// scalars +-1 / +-i, and Sum / Kron / Blocks / Product of such subtrees.
// Such trees run in the I/O element type itself rather than double-float, so
// every output element is an input element (or an IEEE sum of them, in
// fastmat's order for Sum), bit for bit as in fastmat's gathers
// (fastmat/Permutation.pyx:120-124, fastmat/Partial.pyx:268-294).
bool moves_data_only(const std::vector<NodeRec> &recs, int id, int depth = 0) {
  if (id < 0) return true;  // zero block of a Blocks node
  if (depth > 256 || id >= (int)recs.size()) return false;
  const NodeRec &r = recs[(size_t)id];
  auto children = [&]() {
    for (int c : r.ch)
      if (!moves_data_only(recs, c, depth + 1)) return false;
    return true;
  };
  switch (r.d.kind) {
    case FM_NODE_PERMUTATION:
    case FM_NODE_EYE: return true;
    case FM_NODE_PARTIAL:
    case FM_NODE_HERMITIAN:
    case FM_NODE_CONJUGATE:
    case FM_NODE_SUM:
    case FM_NODE_KRON:
    case FM_NODE_BLOCKS: return children();
    case FM_NODE_PRODUCT: {
      const double re = r.d.scalar_re, im = r.d.scalar_im;
      const bool unit = (im == 0.0 && (re == 1.0 || re == -1.0)) ||
                        (re == 0.0 && (im == 1.0 || im == -1.0));
      return unit && children();
    }
    default: return false;
  }
}

template <class F> int guarded(F f) {
  try {
    g_err.clear();
    return f();
  } catch (const Error &e) {
    g_err = e.msg;
    return e.code;
  } catch (const std::bad_alloc &) {
    g_err = "host allocation failed";
    return FM_ERR_NOMEM;
  } catch (const std::exception &e) {
    g_err = e.what();
    return FM_ERR_VALUE;
  }
}

void check_device(int want, const char *what) {
  int dev = -1;
  CUDA_TRY(cudaGetDevice(&dev));
  if (dev != want)
    fail(FM_ERR_VALUE, std::string(what) + " was built on device " +
                           std::to_string(want) + " but device " +
                           std::to_string(dev) + " is current");
}

// Arguments common to the execute entry points; the plan must run on the
// device it was built on (its constants and scratch live there).
void check_call(const fm_plan *plan, int direction, const void *x, int x_type,
                i64 ld_x, const void *y, int y_type, i64 ld_y, i64 num_cols) {
  if (!plan) fail(FM_ERR_VALUE, "plan is NULL");
  if (direction != FM_FORWARD && direction != FM_BACKWARD)
    fail(FM_ERR_VALUE, "invalid direction");
  if (!valid_type(x_type) || !valid_type(y_type))
    fail(FM_ERR_TYPE, "unsupported element type");
  const i64 n_in = direction == FM_FORWARD ? plan->cols : plan->rows;
  const i64 n_out = direction == FM_FORWARD ? plan->rows : plan->cols;
  if (num_cols < 0) fail(FM_ERR_VALUE, "negative column count");
  if (num_cols > 0 && (!x || !y)) fail(FM_ERR_VALUE, "NULL data pointer");
  if (ld_x < n_in || ld_y < n_out)
    fail(FM_ERR_VALUE, "leading dimension smaller than the vector size");
  check_device(plan->device, "the plan");
}

// Report and clear a failure kernels of the plan recorded on the device.
int check_status(fm_plan *plan) {
  if (!plan->err) return FM_OK;
  int e = 0;
  CUDA_TRY(cudaMemcpy(&e, plan->err, sizeof(int), cudaMemcpyDeviceToHost));
  if (e != 0) {
    CUDA_TRY(cudaMemset(plan->err, 0, sizeof(int)));
    fail(FM_ERR_TIMEOUT,
         "a bounded wait for a tile copy gave up; results of the affected "
         "call are incomplete");
  }
  return FM_OK;
}

// Device staging of fm_execute_host, one per device and shared by every
// plan (calls on one device take turns): the operand buffers, sized by the
// largest call so far, and the copy-in / compute / copy-out streams.  Kept
// until the process exits.
struct HostStage {
  std::mutex mu;
  void *dx = nullptr, *dy = nullptr;
  size_t dx_cap = 0, dy_cap = 0;
  cudaStream_t comp = nullptr, in = nullptr, out = nullptr;
  std::vector<cudaEvent_t> ev;  // chunk hand-over events
  void reserve(size_t bx, size_t by) {
    if (bx > dx_cap) {
      if (dx) cudaFree(dx);
      dx = nullptr;
      dx_cap = 0;
      CUDA_TRY(dev_malloc(&dx, bx));
      dx_cap = bx;
    }
    if (by > dy_cap) {
      if (dy) cudaFree(dy);
      dy = nullptr;
      dy_cap = 0;
      CUDA_TRY(dev_malloc(&dy, by));
      dy_cap = by;
    }
  }
};

HostStage &host_stage(int dev) {
  static std::mutex mu;
  static std::map<int, HostStage *> stages;
  std::lock_guard<std::mutex> lock(mu);
  HostStage *&h = stages[dev];
  if (!h) h = new HostStage();
  return *h;
}

}  // namespace

// ------------------------------------------------------------ C ABI
namespace fmk {
void set_last_error(const char *msg) { g_err = msg ? msg : ""; }
}  // namespace fmk

extern "C" {

int fm_plan_create(const fm_node *nodes, int32_t num_nodes,
                   const int32_t *children, int32_t num_children, int32_t root,
                   int32_t compute_type, fm_plan **out_plan) {
  return guarded([&]() {
    if (!out_plan) fail(FM_ERR_VALUE, "out_plan is NULL");
    *out_plan = nullptr;
    if (!nodes || num_nodes <= 0 || root < 0 || root >= num_nodes)
      fail(FM_ERR_VALUE, "invalid node array");
    if (compute_type != FM_F32 && compute_type != FM_F64 &&
        compute_type != FM_C64 && compute_type != FM_C128 &&
        compute_type != FM_I64 && compute_type != FM_F64_DF &&
        compute_type != FM_C128_DF && compute_type != FM_F32_TC)
      fail(FM_ERR_TYPE, "unsupported compute type");
    std::vector<NodeRec> recs((size_t)num_nodes);
    for (int i = 0; i < num_nodes; ++i) {
      recs[i].d = nodes[i];
      const fm_node &d = nodes[i];
      if (d.num_children < 0 ||
          (d.num_children > 0 &&
           (!children || d.first_child < 0 ||
            d.first_child + d.num_children > num_children)))
        fail(FM_ERR_VALUE, "invalid child range");
      for (int k = 0; k < d.num_children; ++k) {
        const int c = children[d.first_child + k];
        // -1 marks a zero block of a Blocks node
        if (c < -1 || c >= num_nodes || (c == -1 && d.kind != FM_NODE_BLOCKS))
          fail(FM_ERR_VALUE, "invalid child");
        recs[i].ch.push_back(c);
      }
      if (d.rows < 0 || d.cols < 0) fail(FM_ERR_VALUE, "negative shape");
    }
    // data movement computes in the buffers' own type: bit-exact
    int ctype = compute_type;
    if ((ctype == FM_F64_DF || ctype == FM_C128_DF || ctype == FM_F32_TC) &&
        moves_data_only(recs, root))
      ctype = io_of(ctype);
    std::unique_ptr<fm_plan> P(new fm_plan);
    P->ctype = ctype;
    P->io_type = io_of(ctype);
    P->esz = esize(ctype);
    CUDA_TRY(cudaGetDevice(&P->device));
    P->rows = nodes[root].rows;
    P->cols = nodes[root].cols;
    Planner(P.get(), recs).build(root);
    CUDA_TRY(dev_malloc(&P->err, sizeof(int)));
    P->allocs.push_back(P->err);
    CUDA_TRY(cudaMemset(P->err, 0, sizeof(int)));
    CUDA_TRY(cudaDeviceSynchronize());
    *out_plan = P.release();
    return FM_OK;
  });
}

int fm_execute(fm_plan *plan, int32_t direction, const void *x, int32_t x_type,
               int64_t ld_x, void *y, int32_t y_type, int64_t ld_y,
               int64_t num_cols, void *stream) {
  return guarded([&]() {
    check_call(plan, direction, x, x_type, ld_x, y, y_type, ld_y, num_cols);
    return run_plan(plan, direction, x, x_type, ld_x, y, y_type, ld_y,
                    num_cols, (cudaStream_t)stream);
  });
}

int fm_execute_profiled(fm_plan *plan, int32_t direction, const void *x,
                        int32_t x_type, int64_t ld_x, void *y, int32_t y_type,
                        int64_t ld_y, int64_t num_cols, void *stream,
                        float *ms, int32_t *num_launches) {
  return guarded([&]() {
    if (!ms || !num_launches) fail(FM_ERR_VALUE, "NULL argument");
    check_call(plan, direction, x, x_type, ld_x, y, y_type, ld_y, num_cols);
    const size_t n = plan->steps[direction].size();
    if ((size_t)*num_launches < n) fail(FM_ERR_VALUE, "ms array too short");
    std::vector<cudaEvent_t> ev(n + 1, nullptr);
    for (auto &e : ev) CUDA_TRY(cudaEventCreate(&e));
    const cudaStream_t s = (cudaStream_t)stream;
    int st = FM_OK;
    try {
      st = run_plan(plan, direction, x, x_type, ld_x, y, y_type, ld_y,
                    num_cols, s, &ev);
      if (st == FM_OK) {
        CUDA_TRY(cudaEventSynchronize(ev[n]));
        for (size_t i = 0; i < n; ++i)
          CUDA_TRY(cudaEventElapsedTime(&ms[i], ev[i], ev[i + 1]));
        *num_launches = (int32_t)n;
      }
    } catch (...) {
      for (auto &e : ev) cudaEventDestroy(e);
      throw;
    }
    for (auto &e : ev) cudaEventDestroy(e);
    return st;
  });
}

int fm_execute_static(fm_plan *plan, int32_t direction, const void *x,
                      int32_t x_type, int64_t ld_x, void *y, int32_t y_type,
                      int64_t ld_y, int64_t num_cols, void *stream) {
  return guarded([&]() {
    check_call(plan, direction, x, x_type, ld_x, y, y_type, ld_y, num_cols);
    return run_plan_static(plan, direction, x, x_type, ld_x, y, y_type, ld_y,
                           num_cols, (cudaStream_t)stream);
  });
}

int fm_execute_host(fm_plan *plan, int32_t direction, const void *x,
                    int32_t x_type, int64_t ld_x, void *y, int32_t y_type,
                    int64_t ld_y, int64_t num_cols) {
  if (!plan) return guarded([]() -> int { fail(FM_ERR_VALUE, "plan is NULL"); });
  // the call runs on the plan's device and leaves the caller's current
  // device as it was
  int prev = -1;
  if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
  const bool switched = prev != plan->device;
  if (switched && cudaSetDevice(plan->device) != cudaSuccess)
    return guarded([&]() -> int {
      fail(FM_ERR_CUDA, "cannot make the plan's device current");
    });
  HostStage &hs = host_stage(plan->device);
  std::lock_guard<std::mutex> lock(hs.mu);
  const int st = guarded([&]() {
    if (num_cols > 0 && (!x || !y)) fail(FM_ERR_VALUE, "x or y is NULL");
    check_call(plan, direction, x, x_type, ld_x, y, y_type, ld_y, num_cols);
    if (num_cols <= 0) return FM_OK;
    const size_t cx = (size_t)ld_x * esize(x_type);  // bytes per column
    const size_t cy = (size_t)ld_y * esize(y_type);
    const size_t bx = cx * (size_t)num_cols, by = cy * (size_t)num_cols;
    for (cudaStream_t *sp : {&hs.comp, &hs.in, &hs.out})
      if (!*sp) CUDA_TRY(cudaStreamCreateWithFlags(sp, cudaStreamNonBlocking));
    hs.reserve(bx, by);
    // column chunks of at least ~64 MiB of operands, at most 8
    const i64 want = (i64)std::min<size_t>(
        8, std::max<size_t>(1, (bx + by) / ((size_t)64 << 20)));
    const i64 per = (num_cols + std::min<i64>(want, num_cols) - 1) /
                    std::min<i64>(want, num_cols);
    const i64 nch = (num_cols + per - 1) / per;
    while ((i64)hs.ev.size() < 2 * nch) {
      cudaEvent_t e;
      CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      hs.ev.push_back(e);
    }
    for (i64 k = 0; k < nch; ++k) {
      const i64 c0 = k * per, m = std::min(per, num_cols - c0);
      cudaEvent_t ev_in = hs.ev[(size_t)(2 * k)];
      cudaEvent_t ev_done = hs.ev[(size_t)(2 * k + 1)];
      char *dxk = (char *)hs.dx + c0 * cx;
      char *dyk = (char *)hs.dy + c0 * cy;
      CUDA_TRY(cudaMemcpyAsync(dxk, (const char *)x + c0 * cx, m * cx,
                               cudaMemcpyHostToDevice, hs.in));
      CUDA_TRY(cudaEventRecord(ev_in, hs.in));
      CUDA_TRY(cudaStreamWaitEvent(hs.comp, ev_in, 0));
      // (the chunks run their fused pairs as separate launches: with the
      // fused launches inside this pipeline the Kron call measured 19.8
      // against 7.4 ms)
      struct NoPair {  // reset also when run_plan throws
        fm_plan *p;
        explicit NoPair(fm_plan *q) : p(q) { p->no_pair = true; }
        ~NoPair() { p->no_pair = false; }
      } no_pair(plan);
      const int s2 = run_plan(plan, direction, dxk, x_type, ld_x, dyk, y_type,
                              ld_y, m, hs.comp);
      if (s2 != FM_OK) return s2;
      CUDA_TRY(cudaEventRecord(ev_done, hs.comp));
      CUDA_TRY(cudaStreamWaitEvent(hs.out, ev_done, 0));
      CUDA_TRY(cudaMemcpyAsync((char *)y + c0 * cy, dyk, m * cy,
                               cudaMemcpyDeviceToHost, hs.out));
    }
    CUDA_TRY(cudaStreamSynchronize(hs.out));
    CUDA_TRY(cudaStreamSynchronize(hs.comp));
    CUDA_TRY(cudaStreamSynchronize(hs.in));
    return check_status(plan);
  });
  // streams that may still hold copies into the caller's buffers are
  // drained before any return
  if (st != FM_OK)
    for (cudaStream_t q : {hs.in, hs.comp, hs.out})
      if (q) cudaStreamSynchronize(q);
  if (switched && prev >= 0) cudaSetDevice(prev);
  return st;
}

int fm_plan_set_tile(fm_plan *plan, int32_t direction, int32_t launch,
                     int32_t vectors_per_tile, int32_t nbuf) {
  return guarded([&]() {
    if (!plan) fail(FM_ERR_VALUE, "plan is NULL");
    if (direction != FM_FORWARD && direction != FM_BACKWARD)
      fail(FM_ERR_VALUE, "invalid direction");
    std::vector<LStep> &steps = plan->steps[direction];
    if (launch < 0 || launch >= (int)steps.size())
      fail(FM_ERR_VALUE, "launch index out of range");
    LStep &ls = steps[launch];
    if (ls.kind != 0) return FM_OK;  // no tile shape to set
    const LStep keep = ls;
    if (!configure(plan->esz, ls, vectors_per_tile, nbuf, true, ls.lay)) {
      ls = keep;
      fail(FM_ERR_VALUE, "tile configuration not feasible for this launch");
    }
    ls.tm_in_key = ls.tm_out_key = nullptr;  // boxes follow the tile shape
    return FM_OK;
  });
}

int fm_plan_set_tile_layout(fm_plan *plan, int32_t direction, int32_t launch,
                            int32_t vectors_per_tile, int32_t nbuf,
                            int32_t layout) {
  return guarded([&]() {
    if (!plan) fail(FM_ERR_VALUE, "plan is NULL");
    if (direction != FM_FORWARD && direction != FM_BACKWARD)
      fail(FM_ERR_VALUE, "invalid direction");
    std::vector<LStep> &steps = plan->steps[direction];
    if (launch < 0 || launch >= (int)steps.size())
      fail(FM_ERR_VALUE, "launch index out of range");
    if (layout < 0 || layout > 2) fail(FM_ERR_VALUE, "invalid layout");
    LStep &ls = steps[launch];
    if (ls.kind != 0) return FM_OK;  // no tile shape to set
    const LStep keep = ls;
    if (!configure(plan->esz, ls, vectors_per_tile, nbuf, true, layout)) {
      ls = keep;
      fail(FM_ERR_VALUE, "tile configuration not feasible for this launch");
    }
    ls.tm_in_key = ls.tm_out_key = nullptr;
    return FM_OK;
  });
}

int fm_plan_get_tile(const fm_plan *plan, int32_t direction, int32_t launch,
                     int32_t *vectors_per_tile, int32_t *nbuf,
                     int32_t *layout) {
  return guarded([&]() {
    if (!plan || !vectors_per_tile || !nbuf || !layout)
      fail(FM_ERR_VALUE, "NULL argument");
    if (direction != FM_FORWARD && direction != FM_BACKWARD)
      fail(FM_ERR_VALUE, "invalid direction");
    const std::vector<LStep> &steps = plan->steps[direction];
    if (launch < 0 || launch >= (int)steps.size())
      fail(FM_ERR_VALUE, "launch index out of range");
    *vectors_per_tile = steps[launch].st.B;
    *nbuf = steps[launch].st.nbuf;
    *layout = steps[launch].lay;
    return FM_OK;
  });
}

int fm_plan_autotune(fm_plan *plan, int32_t direction, int64_t num_cols,
                     void *stream) {
  return guarded([&]() {
    if (!plan) fail(FM_ERR_VALUE, "plan is NULL");
    if (direction != FM_FORWARD && direction != FM_BACKWARD)
      fail(FM_ERR_VALUE, "invalid direction");
    if (num_cols <= 0) fail(FM_ERR_VALUE, "num_cols must be positive");
    check_device(plan->device, "the plan");
    const cudaStream_t s = (cudaStream_t)stream;
    const i64 n_in = direction == FM_FORWARD ? plan->cols : plan->rows;
    const i64 n_out = direction == FM_FORWARD ? plan->rows : plan->cols;
    auto rows_of = [&](int id) {
      return id == 0 ? n_in : id == 1 ? n_out : plan->scratch_rows[id - 2];
    };
    cudaEvent_t e0, e1;
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    void *tsrc = nullptr, *tdst = nullptr;
    try {
      for (LStep &ls : plan->steps[direction]) {
        if (ls.kind != 0) continue;  // sparse products have no tile shape
        const i64 rs = rows_of(ls.src), rd = rows_of(ls.dst);
        // a sample of the columns, at most ~512 MiB per operand
        const i64 cap = std::max<i64>(
            1, (512ll << 20) / (std::max(rs, rd) * plan->esz));
        const i64 M = std::min<i64>(num_cols, cap);
        CUDA_TRY(dev_malloc(&tsrc, (size_t)(rs * M * plan->esz)));
        CUDA_TRY(dev_malloc(&tdst, (size_t)(rd * M * plan->esz)));
        // normal numbers (0x3F bytes) so that no fast path for zeros runs
        CUDA_TRY(cudaMemsetAsync(tsrc, 0x3F, (size_t)(rs * M * plan->esz), s));
        CUDA_TRY(cudaMemsetAsync(tdst, 0x3F, (size_t)(rd * M * plan->esz), s));
        const LStep base = ls;
        float best = 1e30f;
        int bestB = base.st.B, bestN = base.st.nbuf, bestL = base.lay;
        for (int lay : {1, 0, 2})
        for (int B = 1; B <= 1024; B *= 2) {
          for (int nb = 2; nb <= 4; ++nb) {
            ls = base;
            if (!configure(plan->esz, ls, B, nb, true, lay)) continue;
            fmk::Step st = ls.st;
            st.src = tsrc;
            st.dst = tdst;
            st.src_type = st.dst_type = plan->io_type;
            st.ld_src = rs;
            st.ld_dst = rd;
            st.num_cols = M;
            launch_step(plan, ls, st, s);  // warm-up
            float t = 1e30f;
            for (int rep = 0; rep < 3; ++rep) {
              CUDA_TRY(cudaEventRecord(e0, s));
              launch_step(plan, ls, st, s);
              CUDA_TRY(cudaEventRecord(e1, s));
              CUDA_TRY(cudaEventSynchronize(e1));
              float ms = 0.f;
              CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
              t = std::min(t, ms);
            }
            if (t < best) {
              best = t;
              bestB = B;
              bestN = nb;
              bestL = lay;
            }
          }
        }
        ls = base;
        if (!configure(plan->esz, ls, bestB, bestN, true, bestL)) ls = base;
        ls.tm_in_key = ls.tm_out_key = nullptr;  // descriptors of the temps
        cudaFree(tsrc);
        cudaFree(tdst);
        tsrc = tdst = nullptr;
      }
    } catch (...) {
      if (tsrc) cudaFree(tsrc);
      if (tdst) cudaFree(tdst);
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return fm_plan_check(plan);
  });
}

int fm_plan_check(fm_plan *plan) {
  return guarded([&]() {
    if (!plan) fail(FM_ERR_VALUE, "plan is NULL");
    return check_status(plan);
  });
}

int fm_plan_set_wait_limit(fm_plan *plan, int64_t polls) {
  return guarded([&]() {
    if (!plan) fail(FM_ERR_VALUE, "plan is NULL");
    if (polls < 0) fail(FM_ERR_VALUE, "negative wait limit");
    plan->wait_limit = polls;
    return FM_OK;
  });
}

int fm_release_host_staging(void) {
  return guarded([&]() {
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    HostStage &hs = host_stage(dev);
    std::lock_guard<std::mutex> lock(hs.mu);
    for (cudaStream_t q : {hs.in, hs.comp, hs.out})
      if (q) CUDA_TRY(cudaStreamSynchronize(q));
    if (hs.dx) cudaFree(hs.dx);
    if (hs.dy) cudaFree(hs.dy);
    hs.dx = hs.dy = nullptr;
    hs.dx_cap = hs.dy_cap = 0;
    return FM_OK;
  });
}

int fm_debug_fail_allocation(int32_t after) {
  g_alloc_skip.store(after < 0 ? -1 : (long long)after);
  return FM_OK;
}

int fm_plan_destroy(fm_plan *plan) {
  return guarded([&]() {
    delete plan;
    return FM_OK;
  });
}

int fm_plan_get_info(const fm_plan *plan, fm_plan_info *info) {
  return guarded([&]() {
    if (!plan || !info) fail(FM_ERR_VALUE, "NULL argument");
    memset(info, 0, sizeof(*info));
    info->rows = plan->rows;
    info->cols = plan->cols;
    info->num_launches_fwd = (int32_t)plan->steps[0].size();
    info->num_launches_bwd = (int32_t)plan->steps[1].size();
    i64 sc = 0;
    for (i64 r : plan->scratch_rows) sc += r * plan->esz;
    info->scratch_bytes_per_col = sc;
    info->const_bytes = plan->const_bytes;
    info->compute_type = plan->ctype;
    return FM_OK;
  });
}

int fm_plan_describe(const fm_plan *plan, int32_t direction, char *buf,
                     int64_t buf_len) {
  return guarded([&]() {
    if (!plan || !buf || buf_len <= 0) fail(FM_ERR_VALUE, "NULL argument");
    if (direction != FM_FORWARD && direction != FM_BACKWARD)
      fail(FM_ERR_VALUE, "invalid direction");
    std::string s;
    char line[512];
    for (const LStep &ls : plan->steps[direction]) {
      const fmk::Step &st = ls.st;
      if (ls.kind == 1) {
        snprintf(line, sizeof(line),
                 "launch src=%d dst=%d sparse rows=%lld lanes_per_row=%d\n",
                 ls.src, ls.dst, ls.sp_rows, ls.sp_group);
        s += line;
        continue;
      }
      if (ls.kind == 3) {
        snprintf(line, sizeof(line),
                 "launch src=%d dst=%d in=(%lld,%lld,%lld) out=(%lld,%lld,"
                 "%lld) rfwht L=%d stride=%lld %sacc=%d: fwht(%d)\n",
                 ls.src, ls.dst, st.vin.A, st.vin.n, st.vin.Cc, st.vout.A,
                 st.vout.n, st.vout.Cc, ls.rc_L,
                 (long long)(ls.rc_es > 1 ? ls.rc_es : 1),
                 ls.pair == 1   ? "fused-with-next "
                 : ls.pair == 2 ? "fused-with-previous "
                                : "",
                 st.accumulate, ls.rc_L);
        s += line;
        continue;
      }
      if (ls.kind == 4) {
        snprintf(line, sizeof(line),
                 "launch src=%d dst=%d in=(%lld,%lld,%lld) out=(%lld,%lld,"
                 "%lld) rsfft L=%d stride=%lld acc=%d: fft(%d, sign %d)\n",
                 ls.src, ls.dst, st.vin.A, st.vin.n, st.vin.Cc, st.vout.A,
                 st.vout.n, st.vout.Cc, ls.rc_L, (long long)ls.rc_es,
                 st.accumulate, ls.rc_L, ls.rc_sign);
        s += line;
        continue;
      }
      if (ls.kind == 2) {
        snprintf(line, sizeof(line),
                 "launch src=%d dst=%d in=(%lld,%lld,%lld) out=(%lld,%lld,"
                 "%lld) rconv L=%d acc=%d:",
                 ls.src, ls.dst, st.vin.A, st.vin.n, st.vin.Cc, st.vout.A,
                 st.vout.n, st.vout.Cc, ls.rc_L, st.accumulate);
        s += line;
        s += ls.rc_conj_in || st.conj_in ? " conj" : "";
        s += ls.rc_pre || st.pre ? " pre" : "";
        s += " fft-conv";
        s += ls.rc_post || st.post ? " post" : "";
        s += ls.rc_conj_out || st.conj_out ? " conj" : "";
        s += ls.pair == 3 ? " fused-with-next" : "";
        s += "\n";
        continue;
      }
      snprintf(line, sizeof(line),
               "launch src=%d dst=%d in=(%lld,%lld,%lld) out=(%lld,%lld,%lld) "
               "L=%d B=%d threads=%d smem=%zu cls=%d acc=%d:",
               ls.src, ls.dst, st.vin.A, st.vin.n, st.vin.Cc, st.vout.A,
               st.vout.n, st.vout.Cc, st.L, st.B, ls.threads, ls.smem, ls.cls,
               st.accumulate);
      s += line;
      for (int i = 0; i < st.nops; ++i) {
        snprintf(line, sizeof(line), " %s(%d)", kind_name(st.ops[i].kind),
                 st.ops[i].len);
        s += line;
      }
      if (st.map_in) s += " map_in";
      if (st.pre) s += " pre";
      if (st.post) s += " post";
      if (st.out_pos) s += " out_perm";
      s += "\n";
    }
    const size_t n = std::min<size_t>(s.size(), (size_t)buf_len - 1);
    memcpy(buf, s.data(), n);
    buf[n] = 0;
    return FM_OK;
  });
}

int fm_batch_create(int32_t num_ops, fm_plan *const *plans,
                    const int32_t *directions, const void *const *x,
                    const int32_t *x_types, const int64_t *ld_x,
                    void *const *y, const int32_t *y_types,
                    const int64_t *ld_y, const int64_t *num_cols,
                    fm_batch **batch) {
  return guarded([&]() {
    if (!batch || num_ops < 1 || !plans || !directions || !x || !x_types ||
        !ld_x || !y || !y_types || !ld_y || !num_cols)
      fail(FM_ERR_VALUE, "fm_batch_create: NULL argument or no operators");
    *batch = nullptr;
    const int ctype = plans[0] ? plans[0]->ctype : -1;
    if (ctype != FM_C64 && ctype != FM_C128_DF)
      fail(FM_ERR_UNSUPPORTED, "batches compute in complex64 or complex128 "
                               "(double-float) only");
    const int esz = plans[0]->esz;
    std::unique_ptr<fm_batch> B(new fm_batch());
    CUDA_TRY(cudaGetDevice(&B->device));
    struct Item {
      int level;
      fmk::Step st;
      int cls;
      i64 tiles;
    };
    std::vector<Item> items;
    std::vector<std::pair<int, size_t>> scratch_of;  // (op, bytes)
    // scratch: one allocation for all operators
    std::vector<size_t> op_off((size_t)num_ops + 1, 0);
    const size_t align = 256;
    for (int i = 0; i < num_ops; ++i) {
      fm_plan *P = plans[i];
      if (!P || P->ctype != ctype)
        fail(FM_ERR_VALUE, "fm_batch_create: plans must share one compute "
                           "type");
      check_device(P->device, "a plan of the batch");
      size_t bytes = 0;
      if (num_cols[i] > 0)
        for (i64 r : P->scratch_rows)
          bytes += ((size_t)r * num_cols[i] * esz + align - 1) / align *
                   align;
      op_off[i + 1] = op_off[i] + bytes;
    }
    char *scratch = nullptr;
    if (op_off[num_ops]) {
      CUDA_TRY(dev_malloc(&scratch, op_off[num_ops]));
      B->allocs.push_back(scratch);
    }
    CUDA_TRY(dev_malloc(&B->status, 2 * sizeof(int)));
    B->allocs.push_back(B->status);
    CUDA_TRY(cudaMemset(B->status, 0, 2 * sizeof(int)));
    for (int i = 0; i < num_ops; ++i) {
      fm_plan *P = plans[i];
      const int dir = directions[i];
      if (dir != FM_FORWARD && dir != FM_BACKWARD)
        fail(FM_ERR_VALUE, "fm_batch_create: invalid direction");
      const i64 M = num_cols[i];
      if (M < 0) fail(FM_ERR_VALUE, "fm_batch_create: negative num_cols");
      if (M == 0) continue;
      const i64 n_in = dir == FM_FORWARD ? P->cols : P->rows;
      const i64 n_out = dir == FM_FORWARD ? P->rows : P->cols;
      if (!x[i] || !y[i] || (M > 1 && (ld_x[i] < n_in || ld_y[i] < n_out)))
        fail(FM_ERR_VALUE, "fm_batch_create: bad operand of operator " +
                               std::to_string(i));
      if (!valid_type(x_types[i]) || !valid_type(y_types[i]))
        fail(FM_ERR_TYPE, "fm_batch_create: unsupported element type");
      std::vector<size_t> offs(P->scratch_rows.size());
      size_t o = op_off[i];
      for (size_t k = 0; k < P->scratch_rows.size(); ++k) {
        offs[k] = o;
        o += ((size_t)P->scratch_rows[k] * M * esz + align - 1) / align *
             align;
      }
      int level = 0;
      for (const LStep &ls0 : P->steps[dir]) {
        if (ls0.kind == 1)
          fail(FM_ERR_UNSUPPORTED, "fm_batch_create: sparse operators run "
                                   "outside batches");
        // (register convolutions and FWHTs run as their vector program)
        LStep ls = ls0;
        // vectors per tile: as many as keep the batch's 512-thread CTA busy
        // (up to one work item per thread) within a 48 KB tile slot
        int wantB = 0;
        for (int b = 1; b <= 1024; b *= 2) {
          LStep t = ls0;
          if (!configure(esz, t, b, 2, false, 0, false)) continue;
          if (t.threads > FM_MAX_THREADS ||
              fmk::tile_bytes(b, t.st.Lp, esz) > (size_t)48 * 1024)
            break;
          wantB = b;
        }
        if (!configure(esz, ls, wantB, 0, false, 0, false))
          fail(FM_ERR_UNSUPPORTED, "fm_batch_create: a launch has no "
                                   "vector-major tile shape");
        fmk::Step st = ls.st;
        auto bind = [&](int id, const void *&ptr, int &type, i64 &ld) {
          if (id == 0) {
            ptr = x[i];
            type = x_types[i];
            ld = M > 1 ? ld_x[i] : n_in;
          } else if (id == 1) {
            ptr = y[i];
            type = y_types[i];
            ld = M > 1 ? ld_y[i] : n_out;
          } else {
            ptr = scratch + offs[id - 2];
            type = P->io_type;
            ld = P->scratch_rows[id - 2];
          }
        };
        const void *sp, *dp;
        bind(ls.src, sp, st.src_type, st.ld_src);
        bind(ls.dst, dp, st.dst_type, st.ld_dst);
        st.src = (const char *)sp + ls.src_off * esize(st.src_type);
        st.dst =
            (char *)const_cast<void *>(dp) + ls.dst_off * esize(st.dst_type);
        st.num_cols = M;
        st.err = B->status + 1;
        st.tma_in = st.tma_out = 0;
        st.rprog = ctype == FM_C64 ? rtile_shape(st) : 0;
        const i64 tiles = (st.V * M + st.B - 1) / st.B;
        if (st.V * M >= 0x7fffffffLL)
          fail(FM_ERR_UNSUPPORTED, "more than 2^31 vectors in one launch");
        // the batch kernel has no class 5: its class 1 runs the same
        // program with the spectrum product as a separate op
        items.push_back(Item{level++, st, ls.cls == 5 ? 1 : ls.cls, tiles});
      }
    }
    if (items.empty()) fail(FM_ERR_VALUE, "fm_batch_create: no work");
    std::stable_sort(items.begin(), items.end(),
                     [](const Item &a, const Item &b) {
                       return a.level < b.level;
                     });
    // one kernel class that covers every program of the batch
    int cls = items[0].cls;
    for (const Item &it : items) {
      const int c = it.cls;
      if (c == cls) continue;
      if (c == 0 || cls == 0 || c == 3 || cls == 3) cls = 0;
      else cls = 2;  // mixed power-of-two and odd-radix FFTs
    }
    if (ctype == FM_C128_DF) cls = 0;
    std::vector<fmk::Step> steps;
    std::vector<i64> start(1, 0);
    std::vector<int> level(1, 0);
    int max_B = 1;
    size_t max_tile = 0;
    i64 level_tiles = 0, max_level_tiles = 1;
    for (size_t k = 0; k < items.size(); ++k) {
      if (k > 0 && items[k].level != items[k - 1].level) {
        level.push_back((int)k);
        max_level_tiles = std::max(max_level_tiles, level_tiles);
        level_tiles = 0;
      }
      steps.push_back(items[k].st);
      start.push_back(start.back() + items[k].tiles);
      level_tiles += items[k].tiles;
      max_B = std::max(max_B, items[k].st.B);
      max_tile = std::max(max_tile, fmk::tile_bytes(items[k].st.B,
                                                   items[k].st.Lp, esz));
    }
    max_level_tiles = std::max(max_level_tiles, level_tiles);
    level.push_back((int)items.size());
    // two slots: the next tile loads while the current one is transformed
    const size_t smem = fmk::batch_smem(max_B, max_tile);
    if (smem > (size_t)fmk::kMaxSmem)
      fail(FM_ERR_UNSUPPORTED, "fm_batch_create: tile too large");
    fmk::Step *dsteps = nullptr;
    i64 *dstart = nullptr;
    int *dlevel = nullptr;
    CUDA_TRY(dev_malloc(&dsteps, steps.size() * sizeof(fmk::Step)));
    B->allocs.push_back(dsteps);
    CUDA_TRY(dev_malloc(&dstart, start.size() * sizeof(i64)));
    B->allocs.push_back(dstart);
    CUDA_TRY(dev_malloc(&dlevel, level.size() * sizeof(int)));
    B->allocs.push_back(dlevel);
    CUDA_TRY(cudaMemcpy(dsteps, steps.data(),
                        steps.size() * sizeof(fmk::Step),
                        cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(dstart, start.data(), start.size() * sizeof(i64),
                        cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(dlevel, level.data(), level.size() * sizeof(int),
                        cudaMemcpyHostToDevice));
    fmk::BatchLaunch &L = B->launch;
    L.ctype = ctype;
    L.cls = cls;
    L.steps = dsteps;
    L.start = dstart;
    L.level = dlevel;
    L.nlev = (int)level.size() - 1;
    L.bar = reinterpret_cast<unsigned *>(B->status);
    L.err = B->status + 1;
    L.max_B = max_B;
    L.max_tile = max_tile;
    L.smem = smem;
    L.max_level_tiles = max_level_tiles;
    B->num_steps = (i64)steps.size();
    B->total_tiles = start.back();
    *batch = B.release();
    return FM_OK;
  });
}

int fm_batch_execute(fm_batch *batch, void *stream) {
  return guarded([&]() {
    if (!batch) fail(FM_ERR_VALUE, "batch is NULL");
    check_device(batch->device, "the batch");
    const cudaStream_t s = (cudaStream_t)stream;
    CUDA_TRY(cudaMemsetAsync(batch->status, 0, sizeof(int), s));
    CUDA_TRY(fmk::launch_batch(batch->launch, s));
    return FM_OK;
  });
}

int fm_batch_execute_graph(fm_batch *batch, void *stream) {
  return guarded([&]() {
    if (!batch) fail(FM_ERR_VALUE, "batch is NULL");
    check_device(batch->device, "the batch");
    if (!batch->exec) {
      if (!batch->gstream)
        CUDA_TRY(cudaStreamCreateWithFlags(&batch->gstream,
                                           cudaStreamNonBlocking));
      cudaGraph_t g = nullptr;
      CUDA_TRY(cudaStreamBeginCapture(batch->gstream,
                                      cudaStreamCaptureModeThreadLocal));
      cudaError_t e1 =
          cudaMemsetAsync(batch->status, 0, sizeof(int), batch->gstream);
      cudaError_t e2 = e1 == cudaSuccess
                           ? fmk::launch_batch(batch->launch, batch->gstream)
                           : e1;
      cudaError_t e3 = cudaStreamEndCapture(batch->gstream, &g);
      CUDA_TRY(e2);
      CUDA_TRY(e3);
      cudaError_t e4 = cudaGraphInstantiate(&batch->exec, g, 0);
      cudaGraphDestroy(g);
      CUDA_TRY(e4);
    }
    CUDA_TRY(cudaGraphLaunch(batch->exec, (cudaStream_t)stream));
    return FM_OK;
  });
}

int fm_batch_set_wait_limit(fm_batch *batch, int64_t polls) {
  return guarded([&]() {
    if (!batch) fail(FM_ERR_VALUE, "batch is NULL");
    if (polls < 0) fail(FM_ERR_VALUE, "negative wait limit");
    if (batch->exec)
      fail(FM_ERR_VALUE, "the batch's graph is already captured with its "
                         "wait limit");
    batch->launch.wait_limit = polls;
    return FM_OK;
  });
}

int fm_batch_check(fm_batch *batch) {
  return guarded([&]() {
    if (!batch) fail(FM_ERR_VALUE, "batch is NULL");
    CUDA_TRY(cudaDeviceSynchronize());
    int v = 0;
    CUDA_TRY(cudaMemcpy(&v, batch->status + 1, sizeof(int),
                        cudaMemcpyDeviceToHost));
    if (v) {
      CUDA_TRY(cudaMemset(batch->status + 1, 0, sizeof(int)));
      fail(v, "a bounded device wait of the batch gave up");
    }
    return FM_OK;
  });
}

int fm_batch_get_info(const fm_batch *batch, int64_t *num_launches,
                      int64_t *num_levels, int64_t *num_tiles) {
  return guarded([&]() {
    if (!batch) fail(FM_ERR_VALUE, "batch is NULL");
    if (num_launches) *num_launches = batch->num_steps;
    if (num_levels) *num_levels = batch->launch.nlev;
    if (num_tiles) *num_tiles = batch->total_tiles;
    return FM_OK;
  });
}

int fm_batch_destroy(fm_batch *batch) {
  delete batch;
  return FM_OK;
}

const char *fm_last_error(void) { return g_err.c_str(); }

int32_t fm_version(void) { return 102; }

}  // extern "C"
