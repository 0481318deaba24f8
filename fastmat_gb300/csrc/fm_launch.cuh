// Host-side launch entry points of the vector-program kernel, one per
// compute element type (each defined in its own translation unit so the
// five instantiations compile in parallel).
#pragma once

#include <cuda_runtime.h>

#include "fm_rconv.cuh"
#include "fm_rfwht.cuh"
#include "fm_rsfft.cuh"
#include "fm_rpair.cuh"
#include "fm_vprog.cuh"

namespace fmk {

cudaError_t launch_f32(const Step &st, int cls, int lay, int threads,
                       size_t smem, i64 grid, cudaStream_t s);
cudaError_t launch_f64(const Step &st, int cls, int lay, int threads,
                       size_t smem, i64 grid, cudaStream_t s);
cudaError_t launch_c64(const Step &st, int cls, int lay, int threads,
                       size_t smem, i64 grid, cudaStream_t s);
cudaError_t launch_c128(const Step &st, int cls, int lay, int threads,
                       size_t smem, i64 grid, cudaStream_t s);
cudaError_t launch_df(const Step &st, int cls, int lay, int threads,
                      size_t smem, i64 grid, cudaStream_t s);
cudaError_t launch_dfc(const Step &st, int cls, int lay, int threads,
                       size_t smem, i64 grid, cudaStream_t s);
cudaError_t launch_i64(const Step &st, int cls, int lay, int threads,
                       size_t smem, i64 grid, cudaStream_t s);

// one batched persistent launch (batch_kernel)
struct BatchLaunch {
  int ctype = 0, cls = 0;
  const Step *steps = nullptr;  // device array, grouped by level
  const i64 *start = nullptr;   // first tile of every step (+ total)
  const int *level = nullptr;   // first step of every level (+ count)
  int nlev = 0;
  unsigned *bar = nullptr;      // grid-barrier counter, zero at launch
  int *err = nullptr;
  int max_B = 1;
  size_t max_tile = 0;  // bytes of the largest tile (one of two slots)
  size_t smem = 0;
  long long max_level_tiles = 1;
  long long wait_limit = 1LL << 22;  // polls of a grid-barrier wait
};
cudaError_t launch_batch(const BatchLaunch &b, cudaStream_t s);

// one CSR sparse-times-columns launch (fm_sparse.cu): y[:, m] = S x[:, m]
// for m < num_cols, S given by row pointers, column indices and values in
// the compute element type; group = lanes per row (1, 2, ..., 32)
struct SpStep {
  const i64 *ptr = nullptr, *idx = nullptr;
  const void *val = nullptr;
  const void *src = nullptr;
  void *dst = nullptr;
  int src_type = 0, dst_type = 0;
  i64 ld_src = 0, ld_dst = 0, rows = 0, num_cols = 0;
};
cudaError_t launch_spmv(int ctype, const SpStep &p, int group,
                        cudaStream_t s);

// register-resident convolution (fm_rconv.cuh): lengths it is built for
// (powers of two from rconv_min_len to rconv_max_len; 0: not for this type)
// and one launch
int rconv_max_len(int ctype);
int rconv_min_len(int ctype);
cudaError_t launch_rconv(int ctype, const RcStep &p, cudaStream_t s);

// register-resident FWHT of contiguous real vectors (fm_rfwht.cuh):
// lengths it is built for (powers of two; 0: not for this type), one launch
int rfwht_min_len(int ctype);
int rfwht_max_len(int ctype);
int rsfwht_min_len(int ctype);  // strided vectors (element stride % 32 == 0)
int rsfwht_max_len(int ctype);
// FFT of strided complex vectors (rsfft_kernel)
int rsfft_min_len(int ctype);
int rsfft_max_len(int ctype);
cudaError_t launch_rsfft(int ctype, const RsfStep &p, cudaStream_t s);
// a circulant Kron mode and the Hadamard mode after it in one launch
// (rkch_kernel): whether it is built for the lengths and a block's items
// divide evenly (n1 / n2: convolution / FWHT items per block)
bool rkch_supported(int ctype, int L1, int L2, i64 block_rows,
                    i64 real_per_block, int *n1, int *n2);
cudaError_t launch_rkch(int ctype, const RchPair &p, cudaStream_t s);
// both passes of a two-pass FWHT in one launch (rfwht2_kernel)
bool rfwht2_supported(int ctype, int L1, int L2);
cudaError_t launch_rfwht2(int ctype, const RfPair &p, cudaStream_t s);
cudaError_t launch_rfwht(int ctype, const RfStep &p, cudaStream_t s);

// largest FFT radix the kernels of a compute type are built with (see
// MinBlocks / Radix16 in fm_vprog.cuh): 8 for single precision and
// double-float, 16 otherwise
inline int max_radix_for(int ctype) {
  return (ctype == 4 /* FM_F32 */ || ctype == 6 /* FM_C64 */ ||
          ctype == 16 /* FM_F64_DF */ || ctype == 17 /* FM_C128_DF */ ||
          ctype == 18 /* FM_F32_TC */)
             ? 8
             : 16;
}

// records the message fm_last_error() returns on the calling thread
void set_last_error(const char *msg);

// maximum dynamic shared memory a launch may request (GB300: 227 KB / CTA)
constexpr int kMaxSmem = 227 * 1024;

}  // namespace fmk
