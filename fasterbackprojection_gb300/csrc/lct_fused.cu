// Confocal LCT in three passes for scan grids up to 64 x 64 (padded planes
// of at most 128 x 128 complex values fit one CTA's shared memory), five for
// larger grids (the plane pass split into row and column passes).
//
// The LCT of lct.cu (python/lct.py:97-211) pads the resampled capture to
// (2M, 2N, 2N), takes a 3-D FFT, multiplies by the PSF's Wiener filter and
// inverse-transforms.  The 3-D transform is separable, so here the axes run
// in the order z, (y, x) forward, filter, (y, x), z inverse, and only what is
// not padding is ever stored.  The capture and the PSF are real, so every
// z-line's spectrum is Hermitian (X[2M - kz] = conj(X[kz])) before and after
// the (y, x) filtering: only the planes kz = 0..M are computed and stored.
//   1. lct_zfwd_kernel: per scan point (y, x), radiometric scale, resample
//      the time axis with mtx, 2M-point FFT along z (the upper M inputs are
//      zero padding), two real lines per complex transform; stores
//      buf[kz][y][x] for kz <= M (an N x N plane per frequency kz).
//   2. lct_plane_kernel: per kz <= M, the 2N x 2N plane in shared memory (rows and
//      columns >= N are zero padding, never materialised: the first pass of
//      each forward transform skips them, the last pass of each inverse
//      transform skips outputs that are cut), forward row and column FFTs, times the Wiener
//      filter, inverse column and row FFTs; stores the N x N corner back.
//   3. lct_zinv_kernel: per (y, x), the whole z spectrum from the stored half,
//      inverse 2M-point FFT along z (two lines per complex transform: the
//      results are real), then rows z < M of mtx^T (the inverse resample), the
//      1/(2M 2N 2N) normalisation and max(real, 0) (lct.py) or the magnitude
//      (lct_2.py); stores vol[z][y][x].
// The FFTs are Stockham passes (radix 16 or 8, then 4 or 2) with compile-time
// sizes; each pass reads its twiddles from a per-stage table
// exp(-2 pi i r jm / (Ns R)) built in double precision on the host.
#include "fft.cuh"
#include "fft_lean.cuh"

#include <cmath>
#include <vector>

namespace fbp {
namespace {

struct LctFusedParams {
    const float* src;             // capture, strides (bin, row, column)
    long long sz, sy, sx;
    int N;                        // scan side
    const int *rp, *ci;           // mtx rows (z' -> source bins)
    const float* v;
    const int *rpt, *cit;         // mtx^T rows (z -> z')
    const float* vt;
    const float* gtab;            // [M] radiometric scale per grid index
    int power, tiled;
    const float2* tw_z;           // stage tables, n = 2M and n = 2N
    const float2* tw_x;
    const float2* wiener;         // [2M][2N][2N], planes kz <= M read
    float2* buf;                  // [M + 1][N][N]
    float2* pad;                  // [M + 1][N][2N]: rows of the padded planes (N > 64 only)
    float* vol;                   // [M][N][N]
    float scale;                  // 1 / (2M * 2N * 2N)
    int magnitude;                // 1: |vol| (lct_2.py), 0: max(real(vol), 0) (lct.py)
};

constexpr int kZThreads = 512;

// Real lines per CTA of the z kernels (even: lines j and j + C/2 share one
// complex transform): 64 KiB of line buffers at most, at most 8.
constexpr int z_lines(int log2z) { return log2z <= 10 ? 8 : (log2z == 11 ? 4 : 2); }

template <int LOG2Z>
constexpr size_t zfwd_smem() {
    constexpr int Z = 1 << LOG2Z, C = z_lines(LOG2Z);
    return ((size_t)(C / 2) * line_stride(Z) + stage_table_size(LOG2Z)) * sizeof(float2) +
           (size_t)C * (Z / 2) * sizeof(float);
}
template <int LOG2Z>
constexpr size_t zinv_smem() {
    constexpr int Z = 1 << LOG2Z, C = z_lines(LOG2Z);
    return ((size_t)C * line_stride(Z) + stage_table_size(LOG2Z)) * sizeof(float2);
}
template <int LOG2X>
constexpr size_t plane_smem() {
    constexpr int X = 1 << LOG2X;
    return ((size_t)X * line_stride(X) + stage_table_size(LOG2X)) * sizeof(float2);
}
template <int LOG2X>
constexpr int plane_threads() { return LOG2X >= 7 ? 512 : 256; }

template <int LOG2Z>
__global__ void __launch_bounds__(kZThreads, 2) lct_zfwd_kernel(LctFusedParams p) {
    constexpr int Z = 1 << LOG2Z, M = Z / 2, C = z_lines(LOG2Z), H = C / 2, LS = line_stride(Z),
                  TWN = stage_table_size(LOG2Z);
    extern __shared__ __align__(16) float2 sm[];
    float2* lines = sm;  // [H] complex lines: line j in the real part, line j + H in the imaginary part
    float2* tw = lines + H * LS;
    float* raw = reinterpret_cast<float*>(tw + TWN);  // [C][M], scaled capture
    for (int i = threadIdx.x; i < TWN; i += kZThreads) tw[i] = p.tw_z[i];
    const int N = p.N, y = blockIdx.y, x0 = blockIdx.x * C;
    const bool time_inner = p.sz == 1;
    {
        // All of a thread's loads in flight together; consecutive threads read
        // consecutive addresses in either layout.
        constexpr int PL = (C * M + kZThreads - 1) / kZThreads;
        float val[PL];
#pragma unroll
        for (int u = 0; u < PL; ++u) {
            const int e = threadIdx.x + u * kZThreads;
            const int i = time_inner ? e / M : e % C, z = time_inner ? e % M : e / C;
            val[u] = (e < C * M && x0 + i < N) ? p.src[z * p.sz + y * p.sy + (long long)(x0 + i) * p.sx] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < PL; ++u) {
            const int e = threadIdx.x + u * kZThreads;
            if (e >= C * M) break;
            const int i = time_inner ? e / M : e % C, z = time_inner ? e % M : e / C;
            float g = 1.f;
            if (p.power > 0) g = p.gtab[p.tiled ? (z * N + y) % M : z];
            raw[i * M + z] = val[u] * g;
        }
    }
    __syncthreads();
    // z' < M only: the first FFT pass treats z' >= M as zero without reading it.
    for (int e = threadIdx.x; e < C * M; e += kZThreads) {
        const int i = e / M, zp = e % M;
        float acc = 0.f;
        for (int k = p.rp[zp]; k < p.rp[zp + 1]; ++k) acc = fmaf(p.v[k], raw[i * M + p.ci[k]], acc);
        reinterpret_cast<float*>(lines + (i % H) * LS + pidx(zp))[i / H] = acc;
    }
    __syncthreads();
    lean_fft<LOG2Z, 0, H, kZThreads, false, false, true, false>(lines, tw, LS);  // inputs z' >= M are zero
    // P = FFT(a + i b) of two real lines: A[k] = (P[k] + conj(P[Z - k])) / 2,
    // B[k] = (P[k] - conj(P[Z - k])) / 2i; kz = 0..M stored.
    for (int e = threadIdx.x; e < C * (M + 1); e += kZThreads) {
        const int i = e % C, kz = e / C;
        if (x0 + i >= N) continue;
        const float2* l = lines + (i % H) * LS;
        const float2 pk = l[pidx(kz)], pm = l[pidx((Z - kz) & (Z - 1))];
        p.buf[((size_t)kz * N + y) * N + x0 + i] = i < H ? make_float2(0.5f * (pk.x + pm.x), 0.5f * (pk.y - pm.y))
                                                          : make_float2(0.5f * (pk.y + pm.y), 0.5f * (pm.x - pk.x));
    }
}

template <int LOG2X>
__global__ void __launch_bounds__(plane_threads<LOG2X>()) lct_plane_kernel(LctFusedParams p) {
    constexpr int X = 1 << LOG2X, N = X / 2, RS = line_stride(X), TWN = stage_table_size(LOG2X);
    constexpr int NT = plane_threads<LOG2X>();
    extern __shared__ __align__(16) float2 sm[];
    float2* plane = sm;
    float2* tw = plane + X * RS;
    for (int i = threadIdx.x; i < TWN; i += NT) tw[i] = p.tw_x[i];
    const size_t kz = blockIdx.x;
    float2* g = p.buf + kz * N * N;
    // The N x N corner only: the first passes of the forward row and column
    // transforms treat x >= N and y >= N as zero without reading them.
    {
        constexpr int PL = (N * N + NT - 1) / NT;
        float2 t[PL];
#pragma unroll
        for (int u = 0; u < PL; ++u) {
            const int e = threadIdx.x + u * NT;
            t[u] = e < N * N ? g[e] : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < PL; ++u) {
            const int e = threadIdx.x + u * NT;
            if (e < N * N) plane[(e / N) * RS + pidx(e % N)] = t[u];
        }
    }
    __syncthreads();
    lean_fft<LOG2X, 0, N, NT, false, false, true, false>(plane, tw, RS);  // rows y < N (the rest are zero), x >= N zero
    lean_fft<LOG2X, 0, X, NT, false, true, true, false>(plane, tw, RS);   // every column, rows y >= N zero
    {
        // The plane's Wiener filter, all of a thread's loads in flight together.
        // Rounds of 16 loads per thread keep the register count in bounds.
        const float2* w = p.wiener + kz * X * X;
        constexpr int PW = (X * X + NT - 1) / NT, RW = PW < 16 ? PW : 16;
#pragma unroll
        for (int c = 0; c < PW; c += RW) {
            float2 t[RW];
#pragma unroll
            for (int u = 0; u < RW; ++u) {
                const int e = threadIdx.x + (c + u) * NT;
                t[u] = e < X * X ? w[e] : make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int u = 0; u < RW; ++u) {
                const int e = threadIdx.x + (c + u) * NT;
                if (e < X * X) {
                    const int a = (e / X) * RS + pidx(e % X);
                    plane[a] = cmul(plane[a], t[u]);
                }
            }
        }
    }
    __syncthreads();
    lean_fft<LOG2X, 0, X, NT, true, true, false, true>(plane, tw, RS);    // every column, rows y < N kept
    lean_fft<LOG2X, 0, N, NT, true, false, false, true>(plane, tw, RS);   // rows y < N, x < N kept
    for (int e = threadIdx.x; e < N * N; e += NT) {
        const int y = e / N, x = e % N;
        g[e] = plane[y * RS + pidx(x)];
    }
}

// The plane pass for 2N = 128 with the 128-point transforms in registers
// (8 x 16, the four-step factorisation): a line's 8 threads hold 16 values
// each (n = n1 + 8 n2), take a 16-point DFT, multiply by w128^(n1 k1) (the
// second stage table of n = 128), trade values once through shared memory,
// and take two 8-point DFTs (k1 = n1 and n1 + 8); the thread then holds
// X[n1 + 8 j], the same distribution as its input.  Rows (y < 64) go to a
// 64 x 130 plane in shared memory; the columns run in rounds (forward, times
// the Wiener filter, whose loads are issued before the forward transform,
// inverse, rows y < 64 kept) and go back to the plane; the inverse rows keep
// x < 64 and store to global memory.  Rows: 8 adjacent threads per row;
// columns: a warp holds one n1 of 32 adjacent columns, so the Wiener and
// plane accesses of a warp are 256 contiguous bytes.  256 threads (32 lines
// at a time) keep a CTA near 105 KB, so two share an SM.
constexpr int kP128Threads = 256;
constexpr int kP128Lines = kP128Threads / 8;
constexpr int kP128Ps = 136;                  // plane row stride (8 mod 16: conflict-free row pairs)
constexpr int kP128RowLine = 16 * 9 + 8;      // a row's exchange scratch (8 mod 16 between the rows of a half-warp)
constexpr int kP128ColLine = 16 * 9 + 9;      // a column's (odd: the 16 columns of a half-warp)
constexpr int kP128Tw = 16 + 128;             // the stage tables of n = 128 (radix 16, 8)
constexpr size_t kP128Smem = ((size_t)64 * kP128Ps + (size_t)kP128Lines * kP128ColLine + kP128Tw) * sizeof(float2);

template <bool INV>
__device__ __forceinline__ void fs128(float2 (&v)[16], float2* s, int n1, const float2* tw) {
    dft16<INV>(v);
#pragma unroll
    for (int k1 = 1; k1 < 16; ++k1) {
        float2 w = tw[16 + k1 * 8 + n1];  // second stage table: entry jm * 8 + k = w128^(jm k)
        if (INV) w.y = -w.y;
        v[k1] = cmul(v[k1], w);
    }
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) s[k1 * 9 + n1] = v[k1];
    __syncthreads();
    float2 a[8], b[8];
#pragma unroll
    for (int m = 0; m < 8; ++m) {
        a[m] = s[n1 * 9 + m];
        b[m] = s[(n1 + 8) * 9 + m];
    }
    __syncthreads();  // the scratch is free again
    dft8<INV>(a);     // X[n1 + 16 k2]
    dft8<INV>(b);     // X[n1 + 8 + 16 k2]
#pragma unroll
    for (int k2 = 0; k2 < 8; ++k2) {
        v[2 * k2] = a[k2];
        v[2 * k2 + 1] = b[k2];
    }
}

__global__ void __launch_bounds__(kP128Threads, 2) lct_plane128_kernel(LctFusedParams p) {
    constexpr int X = 128, N = 64;
    extern __shared__ __align__(16) float2 sm[];
    float2* plane = sm;                              // [64][kP128Ps]
    float2* scratch = plane + 64 * kP128Ps;          // [kP128Lines][kP128ColLine]
    float2* tw = scratch + kP128Lines * kP128ColLine;
    for (int i = threadIdx.x; i < kP128Tw; i += kP128Threads) tw[i] = p.tw_x[i];
    const size_t kz = blockIdx.x;
    float2* g = p.buf + kz * N * N;
    const int line = threadIdx.x >> 3, n1 = threadIdx.x & 7;
    float2* s = scratch + line * kP128RowLine;
    float2 v[16];
    __syncthreads();  // tw
    // Forward rows y < 64 (inputs x >= 64 are zero).
#pragma unroll 1
    for (int r0 = 0; r0 < N; r0 += kP128Lines) {
        const int y = r0 + line;
#pragma unroll
        for (int n2 = 0; n2 < 8; ++n2) v[n2] = g[y * N + n1 + 8 * n2];
#pragma unroll
        for (int n2 = 8; n2 < 16; ++n2) v[n2] = make_float2(0.f, 0.f);
        fs128<false>(v, s, n1, tw);
#pragma unroll
        for (int j = 0; j < 16; ++j) plane[y * kP128Ps + n1 + 8 * j] = v[j];
    }
    __syncthreads();
    // Columns: forward (rows y >= 64 are zero), the Wiener filter, inverse keeping y < 64.
    const float2* wz = p.wiener + kz * X * X;
    const int cl = threadIdx.x & 31, u = threadIdx.x >> 5;  // column of the round, its n1
    float2* sc = scratch + cl * kP128ColLine;
#pragma unroll 1
    for (int c0 = 0; c0 < X; c0 += kP128Lines) {
        const int kx = c0 + cl;
        float2 wf[16];  // the column's Wiener values, in flight during the forward transform
#pragma unroll
        for (int j = 0; j < 16; ++j) wf[j] = wz[(u + 8 * j) * X + kx];
#pragma unroll
        for (int m2 = 0; m2 < 8; ++m2) v[m2] = plane[(u + 8 * m2) * kP128Ps + kx];
#pragma unroll
        for (int m2 = 8; m2 < 16; ++m2) v[m2] = make_float2(0.f, 0.f);
        fs128<false>(v, sc, u, tw);
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = cmul(v[j], wf[j]);
        fs128<true>(v, sc, u, tw);
#pragma unroll
        for (int j = 0; j < 8; ++j) plane[(u + 8 * j) * kP128Ps + kx] = v[j];
    }
    __syncthreads();
    // Inverse rows y < 64, x < 64 kept.
#pragma unroll 1
    for (int r0 = 0; r0 < N; r0 += kP128Lines) {
        const int y = r0 + line;
#pragma unroll
        for (int n2 = 0; n2 < 16; ++n2) v[n2] = plane[y * kP128Ps + n1 + 8 * n2];
        fs128<true>(v, s, n1, tw);
#pragma unroll
        for (int j = 0; j < 8; ++j) g[y * N + n1 + 8 * j] = v[j];
    }
}

template <int LOG2Z>
__global__ void __launch_bounds__(kZThreads, 2) lct_zinv_kernel(LctFusedParams p) {
    constexpr int Z = 1 << LOG2Z, M = Z / 2, C = z_lines(LOG2Z), H = C / 2, LS = line_stride(Z),
                  TWN = stage_table_size(LOG2Z);
    extern __shared__ __align__(16) float2 sm[];
    float2* lines = sm;
    float2* tw = lines + C * LS;
    for (int i = threadIdx.x; i < TWN; i += kZThreads) tw[i] = p.tw_z[i];
    const int N = p.N, y = blockIdx.y, x0 = blockIdx.x * C;
    {
        constexpr int PL = (C * (M + 1) + kZThreads - 1) / kZThreads;
        float2 t[PL];
#pragma unroll
        for (int u = 0; u < PL; ++u) {
            const int e = threadIdx.x + u * kZThreads;
            const int i = e % C, kz = e / C;
            t[u] = (e < C * (M + 1) && x0 + i < N) ? p.buf[((size_t)kz * N + y) * N + x0 + i] : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < PL; ++u) {
            const int e = threadIdx.x + u * kZThreads;
            if (e < C * (M + 1)) lines[(e % C) * LS + pidx(e / C)] = t[u];
        }
    }
    __syncthreads();
    // Q = A + i B over the whole period for the line pair (j, j + H), with
    // A[Z - k] = conj(A[k]) and B[Z - k] = conj(B[k]) (and the real parts at
    // k = 0 and M): IFFT(Q) = Re IFFT(A) + i Re IFFT(B).
    for (int e = threadIdx.x; e < H * (M + 1); e += kZThreads) {
        const int j = e / (M + 1), k = e % (M + 1);
        const float2 a = lines[j * LS + pidx(k)], b = lines[(j + H) * LS + pidx(k)];
        if (k == 0 || k == M) {
            lines[j * LS + pidx(k)] = make_float2(a.x, b.x);
        } else {
            lines[j * LS + pidx(k)] = make_float2(a.x - b.y, a.y + b.x);
            lines[j * LS + pidx(Z - k)] = make_float2(a.x + b.y, b.x - a.y);
        }
    }
    __syncthreads();
    lean_fft<LOG2Z, 0, H, kZThreads, true, false, false, true>(lines, tw, LS);  // z < M kept
    for (int e = threadIdx.x; e < C * M; e += kZThreads) {
        const int i = e % C, z = e / C;
        if (x0 + i >= N) continue;
        const float* l = reinterpret_cast<const float*>(lines + (i % H) * LS) + i / H;  // a: real, b: imaginary
        float re = 0.f;
        for (int k = p.rpt[z]; k < p.rpt[z + 1]; ++k) re = fmaf(p.vt[k], l[2 * pidx(p.cit[k])], re);
        p.vol[((size_t)z * N + y) * N + x0 + i] = p.magnitude ? fabsf(re) * p.scale : fmaxf(re * p.scale, 0.f);
    }
}

// Planes wider than one CTA's shared memory (N > 64): the (y, x) transform
// as passes over rows y < N of the padded planes in global memory.
//   lct_rows_kernel<.., false>: compact rows (x < N; the rest is zero padding,
//     skipped by the first pass) -> forward 2N-point FFT -> pad[kz][y][.]
//   lct_cols_kernel: columns of pad (rows y >= N are zero, skipped), forward
//     FFT, times the Wiener filter, inverse FFT keeping rows y < N
//   lct_rows_kernel<.., true>: inverse FFT of pad rows, x < N kept -> buf.
constexpr int kRowThreads = 256;
constexpr int row_lines(int log2x) { return (8192 >> log2x) < 32 ? (8192 >> log2x) : 32; }
template <int LOG2X>
constexpr size_t rows_smem() {
    return ((size_t)row_lines(LOG2X) * line_stride(1 << LOG2X) + stage_table_size(LOG2X)) * sizeof(float2);
}

template <int LOG2X, bool INV>
__global__ void __launch_bounds__(kRowThreads) lct_rows_kernel(LctFusedParams p) {
    constexpr int X = 1 << LOG2X, N = X / 2, C = row_lines(LOG2X), LS = line_stride(X), TWN = stage_table_size(LOG2X);
    constexpr int NIN = INV ? X : N, PL = (C * NIN + kRowThreads - 1) / kRowThreads;
    extern __shared__ __align__(16) float2 sm[];
    float2* lines = sm;
    float2* tw = lines + C * LS;
    for (int i = threadIdx.x; i < TWN; i += kRowThreads) tw[i] = p.tw_x[i];
    const size_t kz = blockIdx.y;
    const int y0 = blockIdx.x * C;
    {
        float2 v[PL];
#pragma unroll
        for (int u = 0; u < PL; ++u) {
            const int e = threadIdx.x + u * kRowThreads, i = e / NIN, x = e % NIN;
            v[u] = make_float2(0.f, 0.f);
            if (e < C * NIN && y0 + i < N)
                v[u] = INV ? p.pad[(kz * N + y0 + i) * X + x] : p.buf[(kz * N + y0 + i) * N + x];
        }
#pragma unroll
        for (int u = 0; u < PL; ++u) {
            const int e = threadIdx.x + u * kRowThreads;
            if (e < C * NIN) lines[(e / NIN) * LS + pidx(e % NIN)] = v[u];
        }
    }
    __syncthreads();
    lean_fft<LOG2X, 0, C, kRowThreads, INV, false, !INV, INV>(lines, tw, LS);
    constexpr int NOUT = INV ? N : X;
    for (int e = threadIdx.x; e < C * NOUT; e += kRowThreads) {
        const int i = e / NOUT, x = e % NOUT;
        if (y0 + i >= N) continue;
        const float2 c = lines[i * LS + pidx(x)];
        if (INV) p.buf[(kz * N + y0 + i) * N + x] = c;
        else p.pad[(kz * N + y0 + i) * X + x] = c;
    }
}

template <int LOG2X>
__global__ void __launch_bounds__(kRowThreads) lct_cols_kernel(LctFusedParams p) {
    constexpr int X = 1 << LOG2X, N = X / 2, C = row_lines(LOG2X), LS = line_stride(X), TWN = stage_table_size(LOG2X);
    constexpr int PL = (C * N + kRowThreads - 1) / kRowThreads;
    extern __shared__ __align__(16) float2 sm[];
    float2* lines = sm;
    float2* tw = lines + C * LS;
    for (int i = threadIdx.x; i < TWN; i += kRowThreads) tw[i] = p.tw_x[i];
    const size_t kz = blockIdx.y;
    const int x0 = blockIdx.x * C;
    float2* plane = p.pad + kz * N * X;
    {
        float2 v[PL];
#pragma unroll
        for (int u = 0; u < PL; ++u) {
            const int e = threadIdx.x + u * kRowThreads, i = e % C, y = e / C;
            v[u] = e < C * N ? plane[(size_t)y * X + x0 + i] : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < PL; ++u) {
            const int e = threadIdx.x + u * kRowThreads;
            if (e < C * N) lines[(e % C) * LS + pidx(e / C)] = v[u];
        }
    }
    __syncthreads();
    lean_fft<LOG2X, 0, C, kRowThreads, false, false, true, false>(lines, tw, LS);  // rows y >= N are zero
    {
        const float2* w = p.wiener + kz * X * X;
        constexpr int PW = (C * X + kRowThreads - 1) / kRowThreads, RW = PW < 16 ? PW : 16;
#pragma unroll
        for (int c = 0; c < PW; c += RW) {
            float2 t[RW];
#pragma unroll
            for (int u = 0; u < RW; ++u) {
                const int e = threadIdx.x + (c + u) * kRowThreads;
                t[u] = e < C * X ? w[(size_t)(e / C) * X + x0 + e % C] : make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int u = 0; u < RW; ++u) {
                const int e = threadIdx.x + (c + u) * kRowThreads;
                if (e < C * X) {
                    const int a = (e % C) * LS + pidx(e / C);
                    lines[a] = cmul(lines[a], t[u]);
                }
            }
        }
    }
    __syncthreads();
    lean_fft<LOG2X, 0, C, kRowThreads, true, false, false, true>(lines, tw, LS);  // rows y < N kept
    for (int e = threadIdx.x; e < C * N; e += kRowThreads) {
        const int i = e % C, y = e / C;
        plane[(size_t)y * X + x0 + i] = lines[i * LS + pidx(y)];
    }
}

template <int LOG2X>
fbp_status launch_rows_cols(fbp_context* ctx, const LctFusedParams& p, unsigned planes, cudaStream_t s) {
    constexpr int X = 1 << LOG2X, N = X / 2, C = row_lines(LOG2X);
    constexpr size_t smem = rows_smem<LOG2X>();
    static_assert(smem <= 200 * 1024, "row tile too large");
    auto kf = lct_rows_kernel<LOG2X, false>;
    auto kc = lct_cols_kernel<LOG2X>;
    auto ki = lct_rows_kernel<LOG2X, true>;
    FBP_TRY_CUDA(cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    FBP_TRY_CUDA(cudaFuncSetAttribute(kc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    FBP_TRY_CUDA(cudaFuncSetAttribute(ki, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kf<<<dim3(cdiv(N, C), planes), kRowThreads, smem, s>>>(p);
    FBP_CHECK_LAUNCH(ctx, "lct_rows_kernel");
    kc<<<dim3(X / C, planes), kRowThreads, smem, s>>>(p);
    FBP_CHECK_LAUNCH(ctx, "lct_cols_kernel");
    ki<<<dim3(cdiv(N, C), planes), kRowThreads, smem, s>>>(p);
    FBP_CHECK_LAUNCH(ctx, "lct_rows_kernel");
    return FBP_OK;
}

template <int LOG2Z>
fbp_status launch_z(fbp_context* ctx, const LctFusedParams& p, bool forward, cudaStream_t s) {
    constexpr int C = z_lines(LOG2Z);
    const dim3 grid(cdiv(p.N, C), p.N);
    if (forward) {
        constexpr size_t smem = zfwd_smem<LOG2Z>();
        static_assert(smem <= 200 * 1024, "z-forward tile too large");
        auto k = lct_zfwd_kernel<LOG2Z>;
        FBP_TRY_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k<<<grid, kZThreads, smem, s>>>(p);
        FBP_CHECK_LAUNCH(ctx, "lct_zfwd_kernel");
    } else {
        constexpr size_t smem = zinv_smem<LOG2Z>();
        auto k = lct_zinv_kernel<LOG2Z>;
        FBP_TRY_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k<<<grid, kZThreads, smem, s>>>(p);
        FBP_CHECK_LAUNCH(ctx, "lct_zinv_kernel");
    }
    return FBP_OK;
}

template <int LOG2X>
fbp_status launch_plane(fbp_context* ctx, const LctFusedParams& p, unsigned planes, cudaStream_t s) {
    constexpr size_t smem = plane_smem<LOG2X>();
    static_assert(smem <= 200 * 1024, "plane tile too large");
    auto k = lct_plane_kernel<LOG2X>;
    FBP_TRY_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k<<<planes, plane_threads<LOG2X>(), smem, s>>>(p);
    FBP_CHECK_LAUNCH(ctx, "lct_plane_kernel");
    return FBP_OK;
}

fbp_status dispatch_z(fbp_context* ctx, int log2z, const LctFusedParams& p, bool forward, cudaStream_t s) {
    switch (log2z) {
        case 5: return launch_z<5>(ctx, p, forward, s);
        case 6: return launch_z<6>(ctx, p, forward, s);
        case 7: return launch_z<7>(ctx, p, forward, s);
        case 8: return launch_z<8>(ctx, p, forward, s);
        case 9: return launch_z<9>(ctx, p, forward, s);
        case 10: return launch_z<10>(ctx, p, forward, s);
        case 11: return launch_z<11>(ctx, p, forward, s);
        case 12: return launch_z<12>(ctx, p, forward, s);
        default: return set_error(FBP_ERR_UNSUPPORTED, "fbp_lct: fused path needs 16 <= M <= 2048");
    }
}

fbp_status launch_plane128(fbp_context* ctx, const LctFusedParams& p, unsigned planes, cudaStream_t s) {
    static_assert(stage_table_size(7) == kP128Tw && stage_radix_bits(7, 0) == 4 && stage_radix_bits(7, 4) == 3,
                  "the register path reads the radix-16, radix-8 stage tables of n = 128");
    FBP_TRY_CUDA(cudaFuncSetAttribute(lct_plane128_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kP128Smem));
    lct_plane128_kernel<<<planes, kP128Threads, kP128Smem, s>>>(p);
    FBP_CHECK_LAUNCH(ctx, "lct_plane128_kernel");
    return FBP_OK;
}

fbp_status dispatch_plane(fbp_context* ctx, int log2x, const LctFusedParams& p, unsigned planes, cudaStream_t s) {
    switch (log2x) {
        case 4: return launch_plane<4>(ctx, p, planes, s);
        case 5: return launch_plane<5>(ctx, p, planes, s);
        case 6: return launch_plane<6>(ctx, p, planes, s);
        case 7: return launch_plane128(ctx, p, planes, s);
        case 8: return launch_rows_cols<8>(ctx, p, planes, s);
        case 9: return launch_rows_cols<9>(ctx, p, planes, s);
        case 10: return launch_rows_cols<10>(ctx, p, planes, s);
        case 11: return launch_rows_cols<11>(ctx, p, planes, s);
        default: return set_error(FBP_ERR_UNSUPPORTED, "fbp_lct: fused path needs 8 <= N <= 1024");
    }
}

}  // namespace

fbp_status stage_twiddles(fbp_context* ctx, int log2n, cudaStream_t s, const float2** out) {
    if (log2n < 1 || log2n > 15) return set_error(FBP_ERR_UNSUPPORTED, "FFT length must be 2..32768");
    if (!ctx->stage_twiddles[log2n]) {
        std::vector<float2> h;
        for (int done = 0; done < log2n;) {
            const int rb = stage_radix_bits(log2n, done);
            const int ns = 1 << done, r = 1 << rb;
            for (int jm = 0; jm < ns; ++jm)
                for (int k = 0; k < r; ++k) {
                    const double a = -2.0 * M_PI * (double)k * (double)jm / (double)(ns * r);
                    h.push_back(make_float2((float)std::cos(a), (float)std::sin(a)));
                }
            done += rb;
        }
        void* d = nullptr;
        FBP_TRY_CUDA(cudaMalloc(&d, h.size() * sizeof(float2)));
        FBP_TRY_CUDA(cudaMemcpyAsync(d, h.data(), h.size() * sizeof(float2), cudaMemcpyHostToDevice, s));
        FBP_TRY_CUDA(cudaStreamSynchronize(s));  // h is a host temporary
        ctx->stage_twiddles[log2n] = d;
    }
    *out = static_cast<const float2*>(ctx->stage_twiddles[log2n]);
    return FBP_OK;
}

bool lct_fused_supported(uint32_t N, uint32_t M) { return N >= 8 && N <= 1024 && M >= 16 && M <= 2048; }

fbp_status lct_fused_run(fbp_context* ctx, const LctFusedInputs& in, cudaStream_t s) {
    const int log2x = in.log2n + 1, log2z = in.log2m + 1;
    const uint32_t N = 1u << in.log2n, M = 1u << in.log2m;
    LctFusedParams p{};
    p.src = in.data;
    if (in.time_major) {
        p.sz = (long long)N * N; p.sy = N; p.sx = 1;
    } else {
        p.sz = 1; p.sy = (long long)N * M; p.sx = M;
    }
    p.N = (int)N;
    p.rp = in.rp; p.ci = in.ci; p.v = in.v;
    p.rpt = in.rpt; p.cit = in.cit; p.vt = in.vt;
    p.gtab = in.gtab;
    p.power = in.power;
    p.tiled = in.tiled;
    p.wiener = in.wiener;
    p.vol = in.volume;
    p.magnitude = in.magnitude;
    p.scale = (float)(1.0 / ((double)(2 * M) * (double)(2 * N) * (double)(2 * N)));
    FBP_TRY(stage_twiddles(ctx, log2z, s, &p.tw_z));
    FBP_TRY(stage_twiddles(ctx, log2x, s, &p.tw_x));
    void* b = nullptr;
    FBP_TRY(workspace(ctx, WS_FFT_A, (size_t)(M + 1) * N * N * sizeof(float2), s, &b));
    p.buf = static_cast<float2*>(b);
    if (N > 64) {
        void* pd = nullptr;
        FBP_TRY(workspace(ctx, WS_FFT_C, (size_t)(M + 1) * N * (2 * N) * sizeof(float2), s, &pd));
        p.pad = static_cast<float2*>(pd);
    }
    FBP_TRY(dispatch_z(ctx, log2z, p, true, s));
    FBP_TRY(dispatch_plane(ctx, log2x, p, M + 1, s));  // planes kz > M are conjugates
    FBP_TRY(dispatch_z(ctx, log2z, p, false, s));
    return FBP_OK;
}

}  // namespace fbp
