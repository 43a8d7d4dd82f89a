// regfft.cuh -- two-level register FFT for lines of length N = P*Q.
//
// Q threads cooperate on a line; thread t holds element t + Q*j in v[j],
// j in [0, P), both on entry and on exit.  With n = Q a + b, k = c + P d:
//   X[c + P d] = sum_b W_Q^{bd} W_N^{bc} sum_a x[Q a + b] W_P^{ac}
// so thread t (= b) does one P-point DFT over its own registers, multiplies by
// W_N^{tc}, one shared-memory transpose hands column c to thread c mod Q, and
// Q-point DFTs finish the line.  Global loads and stores move directly
// between registers and memory in the t + Q j pattern, which is coalesced
// across the threads of neighbouring lines (columns) or within a row.
#pragma once
#include "fft_core.cuh"

namespace xpfc {

template <int N> struct RP {
    static constexpr bool ok = false, three = false;
    static constexpr int P = 1, Q = 1;
};
template <> struct RP<24> { static constexpr bool ok = true, three = false; static constexpr int P = 12, Q = 2; };
template <> struct RP<48> { static constexpr bool ok = true, three = false; static constexpr int P = 12, Q = 4; };
template <> struct RP<64> { static constexpr bool ok = true, three = false; static constexpr int P = 8, Q = 8; };
template <> struct RP<96> { static constexpr bool ok = true, three = false; static constexpr int P = 24, Q = 4; };
template <> struct RP<192> { static constexpr bool ok = true, three = false; static constexpr int P = 24, Q = 8; };
// 512 = 8 x 8 x 8 and 4096 = 16 x 16 x 16: three levels (reg_fft3), R values
// per thread, R^2 threads per line
template <> struct RP<512> {
    static constexpr bool ok = true, three = true;
    static constexpr int P = 8, Q = 64;
};
template <> struct RP<4096> {
    static constexpr bool ok = true, three = true;
    static constexpr int P = 16, Q = 256;
};
template <> struct RP<128> { static constexpr bool ok = true, three = false; static constexpr int P = 16, Q = 8; };
template <> struct RP<256> { static constexpr bool ok = true, three = false; static constexpr int P = 16, Q = 16; };

// Which lengths take the register kernels.  The pencil kernel holds two
// lines (P values each) per thread: FP64 keeps the shared-memory kernel for
// P above 16 there, FP32 for P above 24 (the 32-value plan of 512 spilled
// about 400 bytes per thread).  The one-line row and column passes keep it
// for the 32-value plan too, whose 167 registers leave one block per SM and
// ran slower than the shared-memory kernel (594 against 405 us at 512^3).
template <typename T, int N> __host__ __device__ constexpr bool reg_pen_ok() {
    return RP<N>::ok && (sizeof(T) == 4 ? RP<N>::P <= 24 : (RP<N>::P <= 16 && RP<N>::Q <= 64));
}
template <typename T, int N> constexpr bool reg_line_ok() {
    return RP<N>::ok && RP<N>::P <= 24;
}
// the row pass pairs k with N - k through warp shuffles: a row must sit in
// one warp
template <typename T, int N> constexpr bool reg_row_ok() {
    return reg_line_ok<T, N>() && RP<N>::Q <= 32;
}

// Transpose scratch of one line: P rows of QP slots (QP odd: conflict-free
// column reads), lines LPITCH apart.
template <int N> struct RPad {
    static constexpr int P = RP<N>::P, Q = RP<N>::Q;
    static constexpr int QP = Q + 1;
    // scratch of one line: P rows of QP (two levels); for three levels the
    // larger of R rows of Q + 2 (first transpose) and Q rows of R + 1 (second)
    static constexpr int BASE = RP<N>::three ? (P * (Q + 2) > Q * (P + 1) ? P * (Q + 2) : Q * (P + 1)) : P * QP;
    // line pitch (complex elements) for lines that sit side by side in a warp:
    // FP32 column kernels want pitch = 2 mod 16, FP32 row kernels 8 mod 16,
    // FP64 an odd pitch.
    template <int MOD, int REM> static constexpr int pitch() {
        int p = BASE;
        while (p % MOD != REM) p++;
        return p;
    }
};

// Three-level transform for N = R^3 (Q = R^2 threads, R values each), the
// same layout on entry and exit (thread t holds element t + Q j).  With
// n = t + Q j, t = s + R u and k = c + R e + Q f:
//   X[k] = sum_s W_R^{sf} W_Q^{se} sum_u W_R^{ue} [W_N^{tc} sum_j x[t + Qj] W_R^{jc}]
// so thread t does an R-point DFT over j and twiddles by W_N^{tc}; after one
// transpose thread c + R s does the R-point DFT over u and twiddles by
// W_Q^{se}; after a second, thread c + R e does the R-point DFT over s, which
// leaves X[c + R e + Q f] in its register f.  Four __syncthreads inside.
template <typename T, int N, int DIR>
__device__ __forceinline__ void reg_fft3(cplx<T> *v, int t, cplx<T> *buf, const cplx<T> *__restrict__ tw) {
    constexpr int R = RP<N>::P, Q = RP<N>::Q, L1 = Q + 2, L2 = R + 1;
    static_assert(R * Q == N && R * R == Q, "three-level plans are cubes");
    dftR<R, DIR, T>(v);
#pragma unroll
    for (int c = 1; c < R; c++) v[c] = twmul<DIR>(v[c], XS(&tw[t * c], 209) ? tw[t * c] : mk<T>((T)1, (T)0));
    __syncthreads();
#pragma unroll
    for (int c = 0; c < R; c++)
        if (XS(&buf[c * L1 + t], 210)) buf[c * L1 + t] = v[c];
    __syncthreads();
    const int c = t % R, s = t / R;
#pragma unroll
    for (int u = 0; u < R; u++)
        v[u] = XS(&buf[c * L1 + s + R * u], 211) ? buf[c * L1 + s + R * u] : mk<T>((T)0, (T)0);
    dftR<R, DIR, T>(v);
#pragma unroll
    for (int e = 1; e < R; e++) v[e] = twmul<DIR>(v[e], XS(&tw[R * s * e], 212) ? tw[R * s * e] : mk<T>((T)1, (T)0));
    __syncthreads();
#pragma unroll
    for (int e = 0; e < R; e++)
        if (XS(&buf[(e * R + c) * L2 + s], 213)) buf[(e * R + c) * L2 + s] = v[e];
    __syncthreads();
    const int e = t / R;
#pragma unroll
    for (int q = 0; q < R; q++)
        v[q] = XS(&buf[(e * R + c) * L2 + q], 214) ? buf[(e * R + c) * L2 + q] : mk<T>((T)0, (T)0);
    dftR<R, DIR, T>(v);
}

// v: P registers (element t + Q j).  buf: this line's scratch.  tw: W_N^k.
// Every thread of the block must call it (two __syncthreads inside, four
// for the three-level plans).  WARP: the Q threads of every line sit in one
// warp and the scratch is the line's own (the row pass), so the transposes
// only need the warp to agree (__syncwarp) instead of the whole block.
template <bool WARP> __device__ __forceinline__ void line_sync() {
    if constexpr (WARP) __syncwarp();
    else __syncthreads();
}

template <typename T, int N, int DIR, bool WARP = false>
__device__ __forceinline__ void reg_fft(cplx<T> *v, int t, cplx<T> *buf, const cplx<T> *__restrict__ tw) {
    static_assert(!WARP || (!RP<N>::three && RP<N>::Q <= 32), "a warp-synchronised line fits one warp");
    if constexpr (RP<N>::three) {
        reg_fft3<T, N, DIR>(v, t, buf, tw);
    } else {
        constexpr int P = RP<N>::P, Q = RP<N>::Q, M = (P / Q > 0 ? P / Q : 1), QP = RPad<N>::QP;
        static_assert(P % Q == 0, "P must be a multiple of Q");
        dftR<P, DIR, T>(v);
#pragma unroll
        for (int c = 1; c < P; c++) v[c] = twmul<DIR>(v[c], XS(&tw[t * c], 207) ? tw[t * c] : mk<T>((T)1, (T)0));
        line_sync<WARP>();
#pragma unroll
        for (int c = 0; c < P; c++)
            if (XS(&buf[c * QP + t], 201)) buf[c * QP + t] = v[c];
        line_sync<WARP>();
        cplx<T> u[P];
#pragma unroll
        for (int m = 0; m < M; m++)
#pragma unroll
            for (int b = 0; b < Q; b++)
                u[m * Q + b] = XS(&buf[(t + Q * m) * QP + b], 202) ? buf[(t + Q * m) * QP + b] : mk<T>((T)0, (T)0);
#pragma unroll
        for (int m = 0; m < M; m++) dftR<Q, DIR, T>(u + m * Q);
#pragma unroll
        for (int m = 0; m < M; m++)
#pragma unroll
            for (int d = 0; d < Q; d++) v[m + M * d] = u[m * Q + d];
    }
}

// Two lines (e.g. the state and the nonlinear term of one pencil) through
// the same pattern, sharing the two barriers.
template <typename T, int N, int DIR>
__device__ __forceinline__ void reg_fft2(cplx<T> *v, cplx<T> *w, int t, cplx<T> *bufv, cplx<T> *bufw,
                                         const cplx<T> *__restrict__ tw) {
    if constexpr (RP<N>::three) {
        reg_fft3<T, N, DIR>(v, t, bufv, tw);
        reg_fft3<T, N, DIR>(w, t, bufw, tw);
    } else {
        constexpr int P = RP<N>::P, Q = RP<N>::Q, M = (P / Q > 0 ? P / Q : 1), QP = RPad<N>::QP;
        dftR<P, DIR, T>(v);
        dftR<P, DIR, T>(w);
#pragma unroll
        for (int c = 1; c < P; c++) {
            const cplx<T> tc = XS(&tw[t * c], 208) ? tw[t * c] : mk<T>((T)1, (T)0);
            v[c] = twmul<DIR>(v[c], tc);
            w[c] = twmul<DIR>(w[c], tc);
        }
        __syncthreads();
#pragma unroll
        for (int c = 0; c < P; c++) {
            if (XS(&bufv[c * QP + t], 203) && XS(&bufw[c * QP + t], 204)) {
                bufv[c * QP + t] = v[c];
                bufw[c * QP + t] = w[c];
            }
        }
        __syncthreads();
        cplx<T> u[P];
#pragma unroll
        for (int m = 0; m < M; m++)
#pragma unroll
            for (int b = 0; b < Q; b++)
                u[m * Q + b] = XS(&bufv[(t + Q * m) * QP + b], 205) ? bufv[(t + Q * m) * QP + b] : mk<T>((T)0, (T)0);
#pragma unroll
        for (int m = 0; m < M; m++) dftR<Q, DIR, T>(u + m * Q);
#pragma unroll
        for (int m = 0; m < M; m++)
#pragma unroll
            for (int d = 0; d < Q; d++) v[m + M * d] = u[m * Q + d];
#pragma unroll
        for (int m = 0; m < M; m++)
#pragma unroll
            for (int b = 0; b < Q; b++)
                u[m * Q + b] = XS(&bufw[(t + Q * m) * QP + b], 206) ? bufw[(t + Q * m) * QP + b] : mk<T>((T)0, (T)0);
#pragma unroll
        for (int m = 0; m < M; m++) dftR<Q, DIR, T>(u + m * Q);
#pragma unroll
        for (int m = 0; m < M; m++)
#pragma unroll
            for (int d = 0; d < Q; d++) w[m + M * d] = u[m * Q + d];
    }
}

}  // namespace xpfc
