// Confocal light-cone transform (LCT) on the GPU.
//
// Implements the LCT the reference only has in NumPy (python/lct.py:97-211,
// define_psf :295-347, resampling_operator :350-419); its C++ entry point
// LCT::reconstructAABB (LCT.cpp:16-18) is an empty stub.  Steps:
//   1. radiometric scale by grid_z^4 (diffuse) or grid_z^2, resample the time
//      axis with mtx, pad to (2M, 2N, 2N)          -> fused into the x-FFT load
//   2. 3-D FFT, multiply by the Wiener filter conj(F)/(|F|^2 + 1/snr) of the
//      PSF, inverse 3-D FFT                           -> 5 line-FFT passes, the
//      z pass doing forward * filter * inverse at once; lines that are zero
//      padding or not needed in the output are skipped
//   3. unpad, inverse resample with mtxi = mtx^T, max(real, 0) (lct.py) or
//      the magnitude (lct_2.py).
// The PSF's Wiener filter and the resampling operator depend only on
// (N, M, slope, snr) and stay cached in the context.  FP64 is used for the
// PSF construction and the Wiener normalisation; the transforms are FP32.
#include "fft.cuh"

#include <cmath>
#include <vector>

namespace fbp {

// define_psf (python/lct.py:295-347) on the (2M, 2N, 2N) grid, FP64 with the
// same operation order as NumPy.  Writes 1 where |c (x^2 + y^2) - z| is the
// column minimum (0 elsewhere) at the rolled position (0, +U, +U), and counts
// the ones.  gx: 2U coordinates, gz: 2V coordinates (numpy.linspace values).
__global__ void lct_psf_kernel(float2* __restrict__ psf, const double* __restrict__ gx, const double* __restrict__ gz,
                               int U, int V, double c, unsigned long long* __restrict__ count) {
    const int X = 2 * U, Z = 2 * V;
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= X * X) return;
    const int y = col / X, x = col % X;
    const double r = __dadd_rn(__dmul_rn(gx[x], gx[x]), __dmul_rn(gx[y], gx[y]));
    const double a = __dmul_rn(c, r);
    double best = INFINITY;
    for (int z = 0; z < Z; ++z) best = fmin(best, fabs(__dsub_rn(a, gz[z])));
    const int yr = (y + U) % X, xr = (x + U) % X;
    unsigned long long ones = 0;
    for (int z = 0; z < Z; ++z) {
        const bool hit = fabs(__dsub_rn(a, gz[z])) == best;
        psf[((size_t)z * X + yr) * X + xr] = make_float2(hit ? 1.f : 0.f, 0.f);
        ones += hit;
    }
    atomicAdd(count, ones);
}

// invpsf = conj(F) / (|F|^2 + 1/snr) with F = FFT(psf) / sqrt(#ones), in FP64
// (the indicator normalised by its column sum and then its L2 norm reduces to
// 1/sqrt(#ones) exactly).
__global__ void lct_wiener_kernel(float2* __restrict__ f, size_t n, const unsigned long long* __restrict__ count,
                                  double inv_snr) {
    const double scale = 1.0 / sqrt((double)*count);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double re = (double)f[i].x * scale, im = (double)f[i].y * scale;
        const double den = re * re + im * im + inv_snr;
        f[i] = make_float2((float)(re / den), (float)(-im / den));
    }
}

// Step 3: with c = sum_k val[k] * buf[col[k], y, x] * scale (mtxi is real),
// vol[z', y, x] = max(Re c, 0) (lct.py) or |c| (magnitude, lct_2.py).
__global__ void lct_unresample_kernel(const float2* __restrict__ buf, const int* __restrict__ rowptr,
                                      const int* __restrict__ colidx, const float* __restrict__ val, int N, int M,
                                      int X, float scale, int magnitude, float* __restrict__ vol) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= (size_t)M * N * N) return;
    const int zp = (int)(i / ((size_t)N * N));
    const int y = (int)((i / N) % N), x = (int)(i % N);
    float re = 0.f, im = 0.f;
    for (int k = rowptr[zp]; k < rowptr[zp + 1]; ++k) {
        const float2 b = buf[((size_t)colidx[k] * X + y) * X + x];
        re = fmaf(val[k], b.x, re);
        im = fmaf(val[k], b.y, im);
    }
    vol[i] = magnitude ? sqrtf(re * re + im * im) * scale : fmaxf(re * scale, 0.f);
}

namespace {

int ilog2_pow2(uint32_t v) {
    if (v == 0 || (v & (v - 1))) return -1;
    int l = 0;
    while ((1u << l) < v) ++l;
    return l;
}

// numpy.linspace(start, stop, num): i * step + start, last = stop.
std::vector<double> np_linspace(double start, double stop, int num) {
    std::vector<double> y(num);
    const double step = (stop - start) / (double)(num - 1);
    for (int i = 0; i < num; ++i) {
        volatile double t = (double)i * step;  // no contraction: multiply, then add
        y[i] = t + start;
    }
    if (num > 1) y[num - 1] = stop;
    return y;
}

// resampling_operator(M) as CSR of the pooled M x M matrix and its transpose:
// row r averages base rows [rM, (r+1)M), base row i has 1/sqrt(i+1) at column
// ceil(sqrt(i+1)) - 1.
void build_resampling(uint32_t M, std::vector<int>& rp, std::vector<int>& ci, std::vector<float>& v,
                      std::vector<int>& rpt, std::vector<int>& cit, std::vector<float>& vt) {
    std::vector<std::vector<std::pair<int, double>>> rows(M), cols(M);
    for (uint32_t r = 0; r < M; ++r) {
        std::vector<double> acc;
        int c0 = -1;
        for (uint64_t i = (uint64_t)r * M; i < (uint64_t)(r + 1) * M; ++i) {
            int c = (int)std::ceil(std::sqrt((double)(i + 1))) - 1;
            c = std::min<int>(std::max(c, 0), (int)M - 1);
            if (c0 < 0) c0 = c;
            if ((int)acc.size() <= c - c0) acc.resize(c - c0 + 1, 0.0);
            acc[c - c0] += 1.0 / std::sqrt((double)(i + 1));
        }
        for (size_t k = 0; k < acc.size(); ++k)
            if (acc[k] != 0.0) {
                rows[r].push_back({c0 + (int)k, acc[k] / (double)M});
                cols[c0 + k].push_back({(int)r, acc[k] / (double)M});
            }
    }
    auto pack = [](const std::vector<std::vector<std::pair<int, double>>>& a, std::vector<int>& p, std::vector<int>& c,
                   std::vector<float>& w) {
        p.assign(1, 0);
        c.clear();
        w.clear();
        for (const auto& row : a) {
            for (const auto& e : row) {
                c.push_back(e.first);
                w.push_back((float)e.second);
            }
            p.push_back((int)c.size());
        }
    };
    pack(rows, rp, ci, v);
    pack(cols, rpt, cit, vt);
}

struct LctOperator {
    const int *rp, *ci, *rpt, *cit;
    const float *v, *vt;
    const float *g2, *g4;  // [M] radiometric scales grid^2, grid^4 (grid = linspace(0, 1, M))
};

}  // namespace

static fbp_status lct_plan(fbp_context* ctx, uint32_t N, uint32_t M, double slope, double snr, cudaStream_t s,
                           float2** invpsf, LctOperator* op) {
    const int X = 2 * N, Z = 2 * M;
    const size_t nfull = (size_t)Z * X * X;
    void* b = nullptr;
    void* o = nullptr;
    FBP_TRY(workspace(ctx, WS_FFT_B, nfull * sizeof(float2), s, &b));
    const bool same = ctx->lct_key_valid && ctx->lct_N == N && ctx->lct_M == M && ctx->lct_slope == slope &&
                      ctx->lct_snr == snr;
    // Operator layout in WS_LCT_OPERATOR: rp[M+1] ci[nnz] rpt[M+1] cit[nnz] v[nnz] vt[nnz], then the
    // PSF's one-count and the numpy.linspace coordinate tables.
    std::vector<int> rp, ci, rpt, cit;
    std::vector<float> v, vt;
    if (!same) {
        build_resampling(M, rp, ci, v, rpt, cit, vt);
        ctx->lct_nnz = ci.size();
    }
    const size_t nnz = ctx->lct_nnz;
    const size_t hdr = 256;
    const size_t bytes_ops = hdr + (2 * (M + 1) + 2 * nnz) * sizeof(int) + 2 * nnz * sizeof(float);
    const size_t bytes_aux = 256 + (X + Z) * sizeof(double) + 2 * (size_t)M * sizeof(float);
    const size_t aux_at = (bytes_ops + 255) & ~size_t(255);  // the aux tables start 256-aligned
    FBP_TRY(workspace(ctx, WS_LCT_OPERATOR, aux_at + bytes_aux, s, &o));
    char* base = static_cast<char*>(o);
    int* d_rp = reinterpret_cast<int*>(base + hdr);
    int* d_ci = d_rp + (M + 1);
    int* d_rpt = d_ci + nnz;
    int* d_cit = d_rpt + (M + 1);
    float* d_v = reinterpret_cast<float*>(d_cit + nnz);
    float* d_vt = d_v + nnz;
    char* aux = base + aux_at;
    unsigned long long* d_count = reinterpret_cast<unsigned long long*>(aux);
    double* d_gx = reinterpret_cast<double*>(aux + 256);
    double* d_gz = d_gx + X;
    float* d_g2 = reinterpret_cast<float*>(d_gz + Z);
    float* d_g4 = d_g2 + M;
    op->rp = d_rp; op->ci = d_ci; op->rpt = d_rpt; op->cit = d_cit; op->v = d_v; op->vt = d_vt;
    op->g2 = d_g2; op->g4 = d_g4;
    *invpsf = static_cast<float2*>(b);
    if (same) return FBP_OK;

    ctx->lct_key_valid = false;
    FBP_TRY_CUDA(cudaMemcpyAsync(d_rp, rp.data(), rp.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    FBP_TRY_CUDA(cudaMemcpyAsync(d_ci, ci.data(), nnz * sizeof(int), cudaMemcpyHostToDevice, s));
    FBP_TRY_CUDA(cudaMemcpyAsync(d_rpt, rpt.data(), rpt.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    FBP_TRY_CUDA(cudaMemcpyAsync(d_cit, cit.data(), nnz * sizeof(int), cudaMemcpyHostToDevice, s));
    FBP_TRY_CUDA(cudaMemcpyAsync(d_v, v.data(), nnz * sizeof(float), cudaMemcpyHostToDevice, s));
    FBP_TRY_CUDA(cudaMemcpyAsync(d_vt, vt.data(), nnz * sizeof(float), cudaMemcpyHostToDevice, s));
    // Radiometric scales: lin = gi / (M - 1) rounded to float, then squared
    // (and squared again) in float.
    std::vector<float> g2(M), g4(M);
    for (uint32_t gi = 0; gi < M; ++gi) {
        const float lin = M > 1 ? (float)((double)gi / (double)(M - 1)) : 0.f;
        const float l2 = lin * lin;
        g2[gi] = l2;
        g4[gi] = l2 * l2;
    }
    FBP_TRY_CUDA(cudaMemcpyAsync(d_g2, g2.data(), M * sizeof(float), cudaMemcpyHostToDevice, s));
    FBP_TRY_CUDA(cudaMemcpyAsync(d_g4, g4.data(), M * sizeof(float), cudaMemcpyHostToDevice, s));
    const std::vector<double> gx = np_linspace(-1.0, 1.0, X), gz = np_linspace(0.0, 2.0, Z);
    FBP_TRY_CUDA(cudaMemcpyAsync(d_gx, gx.data(), X * sizeof(double), cudaMemcpyHostToDevice, s));
    FBP_TRY_CUDA(cudaMemcpyAsync(d_gz, gz.data(), Z * sizeof(double), cudaMemcpyHostToDevice, s));
    FBP_TRY_CUDA(cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), s));
    const double c4 = 4.0 * slope;
    lct_psf_kernel<<<cdiv((size_t)X * X, 128), 128, 0, s>>>(*invpsf, d_gx, d_gz, (int)N, (int)M, c4 * c4, d_count);
    FBP_CHECK_LAUNCH(ctx, "lct_psf_kernel");

    // Forward 3-D FFT of the PSF, all lines.
    const int lx = ilog2_pow2(X), lz = ilog2_pow2(Z);
    FftLineParams p{};
    p.data = *invpsf;
    p.scale = 1.f;
    p.log2n = lx;
    p.lines = std::min(fft_lines_per_cta(lx), X);
    FBP_TRY(fft_twiddles(ctx, lx, s, &p.tw));
    p.elem_stride = 1; p.line_step = X; p.outer_stride = (long long)X * X;
    FBP_TRY(fft_launch(ctx, p, FFT_FORWARD, LOAD_COMPLEX, STORE_COMPLEX, MUL_NONE, cdiv(X, p.lines), Z, s));
    p.elem_stride = X; p.line_step = 1; p.outer_stride = (long long)X * X;
    FBP_TRY(fft_launch(ctx, p, FFT_FORWARD, LOAD_COMPLEX, STORE_COMPLEX, MUL_NONE, cdiv(X, p.lines), Z, s));
    p.log2n = lz;
    p.lines = std::min(fft_lines_per_cta(lz), X);
    FBP_TRY(fft_twiddles(ctx, lz, s, &p.tw));
    p.elem_stride = (long long)X * X; p.line_step = 1; p.outer_stride = X;
    FBP_TRY(fft_launch(ctx, p, FFT_FORWARD, LOAD_COMPLEX, STORE_COMPLEX, MUL_NONE, cdiv(X, p.lines), X, s));
    const unsigned wb = (unsigned)std::min<size_t>(cdiv(nfull, 256), (size_t)ctx->sm_count * 16);
    lct_wiener_kernel<<<wb, 256, 0, s>>>(*invpsf, nfull, d_count, 1.0 / snr);
    FBP_CHECK_LAUNCH(ctx, "lct_wiener_kernel");
    ctx->lct_key_valid = true;
    ctx->lct_N = N;
    ctx->lct_M = M;
    ctx->lct_slope = slope;
    ctx->lct_snr = snr;
    return FBP_OK;
}

fbp_status lct_run(fbp_context* ctx, const float* data, int layout, uint32_t N, uint32_t M, const fbp_lct_params& prm,
                   float* volume, cudaStream_t s) {
    const int ln = ilog2_pow2(N), lm = ilog2_pow2(M);
    if (ln < 0 || lm < 0 || N > 2048 || M > 2048 || N < 2 || M < 2)
        return set_error(FBP_ERR_UNSUPPORTED, "fbp_lct: N and M must be powers of two in [2, 2048]");
    if (!(prm.bin_length > 0.f) || !(prm.snr > 0.f) || !(prm.width > 0.f))
        return set_error(FBP_ERR_INVALID_ARG, "fbp_lct: width, bin_length and snr must be > 0");
    const int X = 2 * N, Z = 2 * M;
    const double range = (double)M * (double)prm.bin_length;
    const double slope = (double)prm.width / range;
    float2* invpsf = nullptr;
    LctOperator op{};
    FBP_TRY(lct_plan(ctx, N, M, slope, (double)prm.snr, s, &invpsf, &op));

    if (lct_fused_supported(N, M)) {
        LctFusedInputs fi{};
        fi.data = data;
        fi.time_major = layout == FBP_LAYOUT_TIME_MAJOR;
        fi.log2n = ln;
        fi.log2m = lm;
        fi.rp = op.rp; fi.ci = op.ci; fi.v = op.v;
        fi.rpt = op.rpt; fi.cit = op.cit; fi.vt = op.vt;
        fi.power = prm.diffuse ? 4 : 2;
        fi.gtab = prm.diffuse ? op.g4 : op.g2;
        fi.tiled = prm.grid_mode == FBP_LCT_GRID_REFERENCE;
        fi.wiener = invpsf;
        fi.volume = volume;
        fi.magnitude = prm.output == FBP_LCT_OUTPUT_MAGNITUDE;
        return lct_fused_run(ctx, fi, s);
    }
    void* a = nullptr;
    const size_t nfull = (size_t)Z * X * X;
    FBP_TRY(workspace(ctx, WS_FFT_A, nfull * sizeof(float2), s, &a));
    float2* buf = static_cast<float2*>(a);
    // Rows (z' < M, y >= N) and planes z' >= M are zero padding: never
    // written, and every pass treats them as zero instead of reading them
    // (n_valid); passes store only what later passes read (n_store).

    const int lx = ln + 1, lz = lm + 1;
    FftLineParams p{};
    p.data = buf;
    p.scale = 1.f;
    // 1. resample + radiometric scale + x-FFT of rows (z' < M, y < N).
    p.log2n = lx;
    p.lines = std::min(fft_lines_per_cta(lx), (int)N);
    FBP_TRY(fft_twiddles(ctx, lx, s, &p.tw));
    p.elem_stride = 1; p.line_step = X; p.outer_stride = (long long)X * X;
    p.rs_rowptr = op.rp; p.rs_col = op.ci; p.rs_val = op.v; p.rs_src = data;
    if (layout == FBP_LAYOUT_TIME_MAJOR) {
        p.rs_sz = (long long)N * N; p.rs_sy = N; p.rs_sx = 1;
    } else {
        p.rs_sz = 1; p.rs_sy = (long long)N * M; p.rs_sx = M;
    }
    p.rs_ns = (int)N; p.rs_m = (int)M;
    p.rs_power = prm.diffuse ? 4 : 2;
    p.rs_gtab = prm.diffuse ? op.g4 : op.g2;
    p.rs_grid_tiled = prm.grid_mode == FBP_LCT_GRID_REFERENCE;
    p.n_valid = (int)N;
    p.n_store = X;
    FBP_TRY(fft_launch(ctx, p, FFT_FORWARD, LOAD_RESAMPLE, STORE_COMPLEX, MUL_NONE, cdiv(N, p.lines), M, s));
    // 2. y-FFT of planes z' < M (rows y >= N are zero).
    p.lines = std::min(fft_lines_per_cta(lx), X);
    p.elem_stride = X; p.line_step = 1; p.outer_stride = (long long)X * X;
    p.n_valid = (int)N;
    p.n_store = X;
    FBP_TRY(fft_launch(ctx, p, FFT_FORWARD, LOAD_COMPLEX, STORE_COMPLEX, MUL_NONE, cdiv(X, p.lines), M, s));
    // 3. z: forward (planes z' >= M are zero), Wiener filter, inverse, every
    //    (y, x) line; only z < M is kept.
    p.log2n = lz;
    p.lines = std::min(fft_lines_per_cta(lz), X);
    FBP_TRY(fft_twiddles(ctx, lz, s, &p.tw));
    p.elem_stride = (long long)X * X; p.line_step = 1; p.outer_stride = X;
    p.mul = invpsf;
    p.n_valid = (int)M;
    p.n_store = (int)M;
    FBP_TRY(fft_launch(ctx, p, FFT_FWD_MUL_INV, LOAD_COMPLEX, STORE_COMPLEX, MUL_ARRAY, cdiv(X, p.lines), X, s));
    // 4. inverse y-FFT of planes z < M; only rows y < N are kept.
    p.log2n = lx;
    p.lines = std::min(fft_lines_per_cta(lx), X);
    FBP_TRY(fft_twiddles(ctx, lx, s, &p.tw));
    p.elem_stride = X; p.line_step = 1; p.outer_stride = (long long)X * X;
    p.n_valid = X;
    p.n_store = (int)N;
    FBP_TRY(fft_launch(ctx, p, FFT_INVERSE, LOAD_COMPLEX, STORE_COMPLEX, MUL_NONE, cdiv(X, p.lines), M, s));
    // 5. inverse x-FFT of rows (z < M, y < N); only x < N is kept.
    p.lines = std::min(fft_lines_per_cta(lx), (int)N);
    p.elem_stride = 1; p.line_step = X; p.outer_stride = (long long)X * X;
    p.n_valid = X;
    p.n_store = (int)N;
    FBP_TRY(fft_launch(ctx, p, FFT_INVERSE, LOAD_COMPLEX, STORE_COMPLEX, MUL_NONE, cdiv(N, p.lines), M, s));
    // 6. unpad, inverse resample (mtxi = mtx^T), normalise the inverse FFT, clamp.
    const size_t nout = (size_t)M * N * N;
    lct_unresample_kernel<<<cdiv(nout, 256), 256, 0, s>>>(buf, op.rpt, op.cit, op.vt, (int)N, (int)M, X,
                                                          (float)(1.0 / (double)nfull),
                                                          prm.output == FBP_LCT_OUTPUT_MAGNITUDE, volume);
    FBP_CHECK_LAUNCH(ctx, "lct_unresample_kernel");
    return FBP_OK;
}

}  // namespace fbp

using namespace fbp;

extern "C" fbp_status fbp_lct(fbp_context* ctx, const float* data, int layout, uint32_t N, uint32_t M,
                              const fbp_lct_params* params, float* volume, void* stream) {
    return guarded("fbp_lct", [&]() -> fbp_status {
        clear_error();
        FBP_TRY(check_ctx(ctx));
        if (!data || !params || !volume) return set_error(FBP_ERR_INVALID_ARG, "fbp_lct: null argument");
        if (layout != FBP_LAYOUT_TIME_MAJOR && layout != FBP_LAYOUT_TIME_INNER)
            return set_error(FBP_ERR_INVALID_ARG, "fbp_lct: unknown layout");
        if (params->grid_mode != FBP_LCT_GRID_REFERENCE && params->grid_mode != FBP_LCT_GRID_DEPTH)
            return set_error(FBP_ERR_INVALID_ARG, "fbp_lct: unknown grid mode");
        if (params->output != FBP_LCT_OUTPUT_CLAMPED_REAL && params->output != FBP_LCT_OUTPUT_MAGNITUDE)
            return set_error(FBP_ERR_INVALID_ARG, "fbp_lct: unknown output mode");
        return lct_run(ctx, data, layout, N, M, *params, volume, (cudaStream_t)stream);
    });
}
