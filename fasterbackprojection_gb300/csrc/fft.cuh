// Batched power-of-two FFTs along one axis of a complex 3-D array, computed
// in shared memory (radix-2, decimation in time, bit-reversed load).
//
// A CTA transforms C lines at once.  Element j of line i of a CTA's group sits
// at  base + i * line_step + j * elem_stride  with
//     base = blockIdx.y * outer_stride + blockIdx.x * C * line_step,
// so for the contiguous axis the C lines are consecutive rows and for the
// strided axes they are C adjacent columns (coalesced loads either way).
// Launch grids may cover only part of the array: LCT and the LoG-FFT filter
// skip lines that are known to be zero or are not needed.
#pragma once

#include "fbp_internal.cuh"

namespace fbp {

enum FftMode { FFT_FORWARD = 0, FFT_INVERSE = 1, FFT_FWD_MUL_INV = 2 };
enum FftLoad { LOAD_COMPLEX = 0, LOAD_REAL = 1, LOAD_RESAMPLE = 2 };
enum FftStore { STORE_COMPLEX = 0, STORE_REAL = 1 };
enum FftMul { MUL_NONE = 0, MUL_ARRAY = 1, MUL_LOG = 2 };

struct FftLineParams {
    float2* data;            // complex array (in place for LOAD_COMPLEX / STORE_COMPLEX)
    const float* real_in;    // LOAD_REAL: real input with the same indexing
    float* real_out;         // STORE_REAL: real part written here
    const float2* tw;        // n/2 twiddles exp(-2 pi i k / n)
    const float2* mul;       // MUL_ARRAY: multiplier with the same indexing as data
    int log2n;
    int lines;               // lines per CTA (C, a power of two)
    int log2c;               // log2(lines), set by the launcher
    long long elem_stride, line_step, outer_stride;
    float scale;             // applied on store
    // LOAD_RESAMPLE (LCT): element j < n_valid of row (z', y) is
    //   sum_k val[k] * src[col[k]*rs_sz + y*rs_sy + j*rs_sx] * gscale(col[k], y),
    // j >= n_valid is zero; rows are indexed by blockIdx.y = z' and the line
    // index within the CTA group is y.
    const int* rs_rowptr;
    const int* rs_col;
    const float* rs_val;
    const float* rs_src;
    long long rs_sz, rs_sy, rs_sx;  // source strides of (bin, row, column)
    int rs_ns;               // N (source row length and row count)
    int rs_m;                // M (bins)
    int rs_power;            // radiometric exponent (2 or 4; 0 for none)
    int rs_grid_tiled;       // 1: python/lct.py tiling grid[(z*N + y) % M], 0: grid[z]
    const float* rs_gtab;    // [M] grid^power per grid index (rs_power > 0)
    int n_valid;             // elements j >= n_valid are zero and not read (<= 0: n)
    int n_store;             // elements j >= n_store are not written (<= 0: n)
    // MUL_LOG: frequency response of buildLoGKernel3D over an nx*ny*nz grid
    int nx, ny, nz;
    float sigma;
};

fbp_status fft_twiddles(fbp_context* ctx, int log2n, cudaStream_t stream, const float2** out);
// Launches fft_lines over grid (inner_blocks, outer_count).
fbp_status fft_launch(fbp_context* ctx, const FftLineParams& p, int mode, int load, int store, int mul,
                      unsigned inner_blocks, unsigned outer_count, cudaStream_t stream);
// Lines per CTA for a transform of length 2^log2n (shared memory budget).
int fft_lines_per_cta(int log2n);

// The LCT of lct_fused.cu (scan grids N x N with 8 <= N <= 1024,
// 16 <= M <= 2048 bins; both powers of two).
struct LctFusedInputs {
    const float* data;            // capture: [M][N][N] (time_major) or [N][N][M]
    int time_major;
    int log2n, log2m;
    const int *rp, *ci, *rpt, *cit;  // resampling operator and its transpose (CSR)
    const float *v, *vt;
    const float* gtab;            // [M] radiometric scale per grid index
    int power, tiled;
    const float2* wiener;         // [2M][2N][2N]
    float* volume;                // [M][N][N]
    int magnitude;                // 1: |vol| (lct_2.py), 0: max(real(vol), 0) (lct.py)
};
// The LoG-FFT filter on the half spectrum (log_fft.cu): every axis a power of
// two in [32, 1024].
bool log_fft_half_supported(uint32_t nx, uint32_t ny, uint32_t nz);
fbp_status launch_log_fft_half(fbp_context* ctx, const float* in, float* out, uint32_t nx, uint32_t ny, uint32_t nz,
                               float sigma, cudaStream_t stream);
bool lct_fused_supported(uint32_t N, uint32_t M);
fbp_status lct_fused_run(fbp_context* ctx, const LctFusedInputs& in, cudaStream_t stream);

}  // namespace fbp
