// Stockham FFT passes with compile-time sizes over lines held in shared
// memory (rows: line i at i * rs + pidx(j); columns: element j at
// j * rs + pidx(i)), and their per-stage twiddle tables.  Used by the LCT
// (lct_fused.cu) and the LoG-FFT filter (log_fft.cu).
#pragma once

#include "fbp_internal.cuh"
#include "fft_codelets.cuh"

namespace fbp {


// Entries of the stage tables of an n = 2^LOG2N transform: pass p starting at
// 2^done covers Ns * R = 2^(done + bits) entries (jm < Ns, r < R).  Radices:
// the fewest passes, radix 16 where it saves one (4 bits), else 8, then 4 or 2.
constexpr int stage_radix_bits(int log2n, int done) {
    const int rem = log2n - done;
    return (rem == 4 || rem == 7 || rem == 8 || rem >= 10) ? 4 : (rem >= 3 ? 3 : rem);
}
constexpr int stage_offset(int log2n, int done) {
    int off = 0;
    for (int d = 0; d < done; d += stage_radix_bits(log2n, d)) off += 1 << (d + stage_radix_bits(log2n, d));
    return off;
}
constexpr int stage_table_size(int log2n) { return stage_offset(log2n, log2n); }

// Element e of line `line`: rows are contiguous lines, columns are strided.
template <bool COLS>
__device__ __forceinline__ int lean_addr(int line, int e, int rs) {
    return COLS ? e * rs + pidx(line) : line * rs + pidx(e);
}

template <int R, bool INV>
__device__ __forceinline__ void lean_dft(float2 (&v)[R]) {
    if constexpr (R == 16) dft16<INV>(v);
    else if constexpr (R == 8) dft8<INV>(v);
    else if constexpr (R == 4) dft4<INV>(v[0], v[1], v[2], v[3]);
    else dft2<INV>(v[0], v[1]);
}

// One Stockham pass over NLINES lines of N = 2^LOG2N points (see fft.cu for
// the formulation), NT threads, butterflies spread over the threads.
// HALF_IN (first pass only): inputs N/2 .. N-1 are zero, i.e. the inputs
// r >= R/2 of every butterfly, and are not read.  HALF_OUT (last pass only):
// outputs N/2 .. N-1, the outputs k >= R/2 of every butterfly, are not
// stored.  Stage tables hold R entries per jm (64-byte aligned for R >= 8).
template <int LOG2N, int DONE, int NLINES, int NT, bool INV, bool COLS, bool HALF_IN, bool HALF_OUT>
__device__ __forceinline__ void lean_pass(float2* x, const float2* tw, int rs) {
    constexpr int RB = stage_radix_bits(LOG2N, DONE), R = 1 << RB;
    constexpr int N = 1 << LOG2N, NB = N / R, TOTAL = NLINES * NB, NS = 1 << DONE;
    constexpr int PER = (TOTAL + NT - 1) / NT;
    constexpr int RIN = HALF_IN ? R / 2 : R, ROUT = HALF_OUT ? R / 2 : R;
    static_assert(!HALF_IN || DONE == 0, "zero inputs are a first-pass property");
    static_assert(!HALF_OUT || DONE + RB == LOG2N, "dropped outputs are a last-pass property");
    const float2* tws = tw + stage_offset(LOG2N, DONE);
    float2 v[PER][R];
#pragma unroll
    for (int u = 0; u < PER; ++u) {
        const int b = threadIdx.x + u * NT;
        if (TOTAL % NT == 0 || b < TOTAL) {
            const int line = COLS ? b % NLINES : b / NB, j = COLS ? b / NLINES : b % NB;
#pragma unroll
            for (int r = 0; r < R; ++r)
                v[u][r] = r < RIN ? x[lean_addr<COLS>(line, j + r * NB, rs)] : make_float2(0.f, 0.f);
            if constexpr (DONE > 0) {
                float2 w[R];
                if constexpr (R >= 4) {
                    const float4* t4 = reinterpret_cast<const float4*>(tws + (j & (NS - 1)) * R);
#pragma unroll
                    for (int q = 0; q < R / 2; ++q) {
                        const float4 t = t4[q];
                        w[2 * q] = make_float2(t.x, t.y);
                        w[2 * q + 1] = make_float2(t.z, t.w);
                    }
                } else {
                    w[1] = tws[(j & (NS - 1)) * R + 1];
                }
#pragma unroll
                for (int r = 1; r < R; ++r) {
                    if (INV) w[r].y = -w[r].y;
                    v[u][r] = cmul(v[u][r], w[r]);
                }
            }
            lean_dft<R, INV>(v[u]);
        }
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < PER; ++u) {
        const int b = threadIdx.x + u * NT;
        if (TOTAL % NT == 0 || b < TOTAL) {
            const int line = COLS ? b % NLINES : b / NB, j = COLS ? b / NLINES : b % NB;
            const int d = (j >> DONE) * NS * R + (j & (NS - 1));
#pragma unroll
            for (int k = 0; k < ROUT; ++k) x[lean_addr<COLS>(line, d + k * NS, rs)] = v[u][k];
        }
    }
    __syncthreads();
}

// A full transform; HALF_IN / HALF_OUT as in lean_pass, for the first and
// the last pass.
template <int LOG2N, int DONE, int NLINES, int NT, bool INV, bool COLS, bool HALF_IN = false, bool HALF_OUT = false>
__device__ __forceinline__ void lean_fft(float2* x, const float2* tw, int rs) {
    if constexpr (DONE < LOG2N) {
        constexpr int NEXT = DONE + stage_radix_bits(LOG2N, DONE);
        lean_pass<LOG2N, DONE, NLINES, NT, INV, COLS, HALF_IN && DONE == 0, HALF_OUT && NEXT == LOG2N>(x, tw, rs);
        lean_fft<LOG2N, NEXT, NLINES, NT, INV, COLS, HALF_IN, HALF_OUT>(x, tw, rs);
    }
}

// Stage tables for n = 2^log2n in pass order (see stage_offset), built in
// double precision and cached in the context.
fbp_status stage_twiddles(fbp_context* ctx, int log2n, cudaStream_t s, const float2** out);

}  // namespace fbp
