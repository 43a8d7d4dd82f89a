// xpfc_regkernels.cuh -- the step's passes built on the two-level register
// FFT (regfft.cuh) for line lengths with a register plan (64, 128, 256).
// Same arguments, layouts and results as the shared-memory Stockham passes
// of xpfc_kernels.cuh, which serve every other length.
#pragma once
#include "regfft.cuh"
#include "xpfc_kernels.cuh"

namespace xpfc {

constexpr unsigned FULLMASK = 0xffffffffu;

template <typename T>
__device__ __forceinline__ cplx<T> shfl_c(cplx<T> v, int src) {
    return mk<T>(__shfl_sync(FULLMASK, v.x, src), __shfl_sync(FULLMASK, v.y, src));
}

// Diagnostics sums: FP64 on the FP64 path; on the FP32 path compensated
// (Kahan) FP32 within a thread and FP64 across threads, which keeps the sample
// steps off GB300's narrow FP64 pipe.
template <typename T, int NQ> struct DSum {
    double v[NQ];
    __device__ DSum() {
#pragma unroll
        for (int q = 0; q < NQ; q++) v[q] = 0.0;
    }
    __device__ __forceinline__ void add(int q, double x) { v[q] += x; }
    __device__ __forceinline__ double get(int q) const { return v[q]; }
};
template <int NQ> struct DSum<float, NQ> {
    float s[NQ], c[NQ];
    __device__ DSum() {
#pragma unroll
        for (int q = 0; q < NQ; q++) s[q] = c[q] = 0.f;
    }
    __device__ __forceinline__ void add(int q, float x) {
        const float y = x - c[q];
        const float t = s[q] + y;
        c[q] = (t - s[q]) - y;
        s[q] = t;
    }
    __device__ __forceinline__ double get(int q) const { return (double)s[q] - (double)c[q]; }
};

// Pitch (complex elements) between the transpose scratch of lines that sit
// side by side in a warp.  Shared memory serves a 64-bit access per half-warp
// (FP32 complex) and a 128-bit access per quarter-warp (FP64) in one
// wavefront when those G lanes (G = 16 or 8) touch the 32 banks once.  In the
// column and pencil passes the G lanes are TX columns times G/TX consecutive
// threads of a line, whose slots are consecutive, so line l must start G/TX
// slots (mod G) after line l - 1; in the row pass the G lanes are G/Q rows
// times Q consecutive threads, so rows start Q slots (mod G) apart.  (A pitch
// of 2 mod 16 served the 8-column pencils but made every 16-column column
// pass take two wavefronts per access.)
template <typename T, int N, int TX> constexpr int line_pitch() {
    constexpr int G = sizeof(T) == 4 ? 16 : 8;
    return RPad<N>::template pitch<G, TX >= G ? 1 : (G / TX) % G>();
}
template <typename T, int N> constexpr int row_pitch() {
    constexpr int G = sizeof(T) == 4 ? 16 : 8;
    return RPad<N>::template pitch<G, RP<N>::Q % G>();
}

// ---------------------------------------------------------------------------
// column pass (C2C along a strided axis), TX columns per block
// ---------------------------------------------------------------------------
template <typename T, int N> struct RColShape {
    static constexpr int Q = RP<N>::Q, P = RP<N>::P;
    // 16 (FP32) / 8 (FP64) columns, fewer for long lines (at most 1024 FP32
    // or 512 FP64 threads, so that the lines stay in registers)
    static constexpr int TXd = sizeof(T) == 4 ? 16 : 8, MAXT = sizeof(T) == 4 ? 1024 : 512;
    static constexpr int TX = TXd * Q > MAXT ? MAXT / Q : TXd;
    static constexpr int THREADS = TX * Q;
    static constexpr int LP = line_pitch<T, N, TX>();
    static constexpr size_t SMEM = sizeof(cplx<T>) * (N + (size_t)TX * LP);
};

template <typename T, int N, int DIR>
__global__ void __launch_bounds__(RColShape<T, N>::THREADS)
col_kernel_reg(ColArgs args, const cplx<T> *__restrict__ twN) {
    using S = RColShape<T, N>;
    constexpr int TX = S::TX, Q = S::Q, P = S::P;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *stw = reinterpret_cast<cplx<T> *>(smem_raw);
    cplx<T> *buf = stw + N;
    const int tid = threadIdx.x;
    for (int i = tid; i < N; i += S::THREADS)
        if (XG(&twN[i], 401) && XS(&stw[i], 402)) stw[i] = twN[i];
    pdl_wait();
    const int c = tid % TX, t = tid / TX;
    const bool cvalid = (int)blockIdx.x * TX + c < args.ncols;
    const long long base = (long long)blockIdx.x * TX + (long long)blockIdx.y * args.ostride +
                           (long long)blockIdx.z * args.zstride + c;
    const cplx<T> *gin = reinterpret_cast<const cplx<T> *>(args.in) + base;
    cplx<T> v[P];
#pragma unroll
    for (int j = 0; j < P; j++)
        v[j] = (cvalid && XG(&gin[(long long)(t + Q * j) * args.es], 403)) ? gin[(long long)(t + Q * j) * args.es]
                                                                           : mk<T>((T)0, (T)0);
    __syncthreads();
    reg_fft<T, N, DIR>(v, t, buf + c * S::LP, stw);
    if (!cvalid) return;
    cplx<T> *gout = reinterpret_cast<cplx<T> *>(args.out) + base;
    const T sc = (T)args.scale;
#pragma unroll
    for (int j = 0; j < P; j++)
        if (XG(&gout[(long long)(t + Q * j) * args.es], 404))
            gout[(long long)(t + Q * j) * args.es] = (args.scale != 1.0) ? cscale(v[j], sc) : v[j];
}

// ---------------------------------------------------------------------------
// row pass: C2R unpack, inverse FFT, real-space op, forward FFT, R2C pack.
// Q threads per row; the pairing of k with L - k uses warp shuffles.
// ---------------------------------------------------------------------------
template <typename T, int N> struct RRowShape {
    static constexpr int Q = RP<N>::Q, P = RP<N>::P;
    static constexpr int ROWS = 256 / Q;
    static constexpr int THREADS = ROWS * Q;
    static constexpr int LP = row_pitch<T, N>();
    static constexpr size_t SMEM = sizeof(cplx<T>) * (2 * N + (size_t)ROWS * LP) + sizeof(double) * 32 * NQ_ROW;
};

// Z[k] = (Xk + conj Xc) + i (Xk - conj Xc) W_{2N}^{-k} for this thread's k = t + Q j
template <typename T, int N>
__device__ __forceinline__ void reg_unpack(cplx<T> *v, int t, int lane, const cplx<T> *__restrict__ tw2) {
    constexpr int Q = RP<N>::Q, P = RP<N>::P;
    const int partner = (t == 0) ? lane : lane + Q - 2 * t;
    cplx<T> z[P];
#pragma unroll
    for (int j = 0; j < P; j++) {
        const cplx<T> sh = shfl_c<T>(v[P - 1 - j], partner);
        const int k = t + Q * j;
        if (k == 0) {
            const cplx<T> p = v[0];
            z[0] = mk<T>(p.x + p.y, p.x - p.y);
            continue;
        }
        const cplx<T> xc = (t == 0) ? v[P - j] : sh;   // X[N - k]
        const cplx<T> xk = v[j];
        const cplx<T> e = cadd(xk, cconj(xc));
        const cplx<T> o = cmulc(csub(xk, cconj(xc)), tw2[k]);
        z[j] = cadd(e, cmuli<1>(o));
    }
#pragma unroll
    for (int j = 0; j < P; j++) v[j] = z[j];
}

// X[k] = ((Zk + conj Zc) - i W_{2N}^k (Zk - conj Zc))/2, slot 0 = (X0, XN)
template <typename T, int N>
__device__ __forceinline__ void reg_pack(cplx<T> *v, int t, int lane, const cplx<T> *__restrict__ tw2) {
    constexpr int Q = RP<N>::Q, P = RP<N>::P;
    const int partner = (t == 0) ? lane : lane + Q - 2 * t;
    const T h = (T)0.5;
    cplx<T> z[P];
#pragma unroll
    for (int j = 0; j < P; j++) {
        const cplx<T> sh = shfl_c<T>(v[P - 1 - j], partner);
        const int k = t + Q * j;
        if (k == 0) {
            const cplx<T> p = v[0];
            z[0] = mk<T>(p.x + p.y, p.x - p.y);
            continue;
        }
        const cplx<T> zc = (t == 0) ? v[P - j] : sh;   // Z[N - k]
        const cplx<T> zk = v[j];
        const cplx<T> e = cadd(zk, cconj(zc));
        const cplx<T> o = cmul(csub(zk, cconj(zc)), tw2[k]);
        z[j] = cscale(csub(e, cmuli<1>(o)), h);
    }
#pragma unroll
    for (int j = 0; j < P; j++) v[j] = z[j];
}

// RED: this launch also produces the real-space sums (diagnostics steps); a
// separate instance keeps that code out of the hot loop of the other steps.
template <typename T, int N, int MODE, bool RED>
__global__ void __launch_bounds__(RRowShape<T, N>::THREADS,
                                  sizeof(T) == 4 ? (RP<N>::P <= 16 ? 4 : RP<N>::P <= 24 ? 2 : 1) : 1)
row_kernel_reg(RowArgs args, const cplx<T> *__restrict__ twN, const cplx<T> *__restrict__ tw2N) {
    using S = RRowShape<T, N>;
    constexpr int Q = S::Q, P = S::P;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *stw = reinterpret_cast<cplx<T> *>(smem_raw);
    cplx<T> *stw2 = stw + N;
    cplx<T> *buf = stw2 + N;
    double *sred = reinterpret_cast<double *>(buf + S::ROWS * S::LP);
    const int tid = threadIdx.x;
    for (int i = tid; i < N; i += S::THREADS) {
        if (XG(&twN[i], 411) && XG(&tw2N[i], 412) && XS(&stw[i], 413) && XS(&stw2[i], 414)) {
            stw[i] = twN[i];
            stw2[i] = tw2N[i];
        }
    }
    pdl_wait();
    const int r = tid / Q, t = tid % Q, lane = tid & 31;
    const long long row = (long long)blockIdx.x * S::ROWS + r;
    const bool valid = row < args.nrows;
    const long long zoff = (long long)blockIdx.z * args.zstride;
    const cplx<T> *gin = reinterpret_cast<const cplx<T> *>(args.in) + zoff + row * N + t;
    cplx<T> v[P];
#pragma unroll
    for (int j = 0; j < P; j++) v[j] = (valid && XG(&gin[Q * j], 415)) ? gin[Q * j] : mk<T>((T)0, (T)0);
    __syncthreads();
    cplx<T> *line = buf + r * S::LP;

    if (MODE == ROW_INV || MODE == ROW_FUSED) {
        reg_unpack<T, N>(v, t, lane, stw2);
        reg_fft<T, N, +1, true>(v, t, line, stw);
    }
    if (MODE == ROW_INV) {
        const T sc = (T)args.scale;
#pragma unroll
        for (int j = 0; j < P; j++) v[j] = cscale(v[j], sc);
    } else if (MODE == ROW_FUSED || MODE == ROW_NL_FWD) {
        DSum<T, NQ_ROW> acc;
        const T sc = (T)args.scale;
        const T a = (T)args.a, b = (T)args.b;
        T *rout = args.real_out ? reinterpret_cast<T *>(args.real_out) + 2 * zoff + row * (2 * N) : nullptr;
#pragma unroll
        for (int j = 0; j < P; j++) {
            T x0 = v[j].x, x1 = v[j].y;
            if (MODE == ROW_FUSED) { x0 *= sc; x1 *= sc; }
            const int m = t + Q * j;
            if (rout && valid && XG(&rout[2 * m + 1], 416)) { rout[2 * m] = x0; rout[2 * m + 1] = x1; }
            const T p20 = powi(x0, 2, args.ref_compat), p21 = powi(x1, 2, args.ref_compat);
            const T p30 = powi(x0, 3, args.ref_compat), p31 = powi(x1, 3, args.ref_compat);
            if (RED && valid) {
                acc.add(0, x0);
                acc.add(0, x1);
                acc.add(1, p20);
                acc.add(1, p21);
                acc.add(2, p30);
                acc.add(2, p31);
                acc.add(3, powi(x0, 4, args.ref_compat));
                acc.add(3, powi(x1, 4, args.ref_compat));
            }
            v[j] = mk<T>(-a * p20 + b * p30, -a * p21 + b * p31);
        }
        if (RED) {
            double tot[NQ_ROW];
#pragma unroll
            for (int q = 0; q < NQ_ROW; q++) tot[q] = acc.get(q);
            block_reduce_store<NQ_ROW>(tot, args.partials + block_slot() * NQ_ROW, sred);
        }
    }
    if (MODE != ROW_INV) {
        reg_fft<T, N, -1, true>(v, t, line, stw);
        reg_pack<T, N>(v, t, lane, stw2);
    }
    if (!valid) return;
    cplx<T> *gout = reinterpret_cast<cplx<T> *>(args.out) + zoff + row * N + t;
#pragma unroll
    for (int j = 0; j < P; j++)
        if (XG(&gout[Q * j], 417)) gout[Q * j] = v[j];
}

// ---------------------------------------------------------------------------
// pencil pass (last axis): forward FFT of S and W, semi-implicit update in
// registers, k-space sums, inverse FFT of S.  3-D blocks pair rows p and
// n1 - p (NG = 2) so that slot 0 finds its mirror mode in the block.
// ---------------------------------------------------------------------------
template <typename T, int N, int NG> struct RPenShape {
    static constexpr int Q = RP<N>::Q, P = RP<N>::P;
    // columns per block: 8 (FP32) for the 16-thread lines; the 4-thread lines
    // of 96 take 16, so that a block still holds four warps
    // (the three-level plans: 4 columns of 64-thread lines, 2 for FP64 pairs
    // of groups; 2 columns of the 256-thread lines of 4096)
    static constexpr int TX = RP<N>::three ? (Q >= 256 ? 2 : (sizeof(T) == 4 || NG == 1) ? 4 : 2)
                                           : (sizeof(T) == 4 ? 8 : 4) * ((Q == 4 && N >= 96) ? 2 : 1);
    static constexpr int THREADS = TX * Q * NG;
    static constexpr int LP = line_pitch<T, N, TX>();
    static constexpr int LINES = TX * NG;
    static constexpr size_t BASE_SMEM = sizeof(cplx<T>) * (N + 2 * (size_t)LINES * LP) + sizeof(double) * 32 * NQ_PEN;
    // the slot-0 pass publishes the [group][kz] pencils at the start of bufS
    // and bufW and writes its results after them in bufS (2 NG N values)
    static_assert(!RP<N>::ok || 2 * NG * N <= LINES * LP, "bufS must hold the slot-0 areas");
    // two resident blocks per SM (128 registers per thread) for the FP32
    // instances of 256 threads; three (168 registers) for the 24-value lines
    // (four for the 128-thread FP32 blocks of 64 and 128, capped at 128
    // registers: 128^3 56.9 -> 59.1 Gpt-steps/s against 166 registers and
    // three blocks)
    static constexpr int MINB = (sizeof(T) == 4 && THREADS == 64 && P <= 16)    ? 8
                                : (sizeof(T) == 4 && THREADS == 128 && P <= 16) ? 4
                                : (sizeof(T) == 4 && THREADS == 256 && P <= 16) ? 2
                                : (sizeof(T) == 4 && P > 16)                  ? 3
                                                                              : 1;
    // FP32 shell tables: the coefficients of the block's TX columns for every
    // shell along the pencil (|kz| = 0 .. N/2: the two mirror rows of a block
    // share them, and so do kz and N - kz) are staged in shared memory after
    // the block sums, CP entries per column (odd, so that the 16-byte reads
    // of a quarter-warp's columns are conflict-free), where that keeps MINB
    // blocks resident per SM (228 KB, 1 KB reserved per block)
    static constexpr int CP = N / 2 + 1;
    static constexpr size_t CSMEM = (size_t)TX * CP * 16;
    static constexpr bool CSM = sizeof(T) == 4 && N <= 512 && (BASE_SMEM + CSMEM + 1024) * MINB <= 233472;
    static constexpr size_t SMEM = BASE_SMEM + (CSM ? CSMEM : 0);
    static_assert(BASE_SMEM % 16 == 0, "the staged coefficients need 16-byte alignment");
};

// Coefficients of mode (i0, kz of the pencil): from the block's staged
// shell entries when there are some (column c of the block), else from the
// table in global memory or computed (kcoef).
template <typename T, int N>
__device__ __forceinline__ Coef<T> pen_coef(const KSpace &ks, const void *table, const float4 *scoef, int c, int i0,
                                            int i1, int i2, int kz) {
    if constexpr (sizeof(T) == 4) {
        if (scoef) {
            const int s = kz <= N / 2 ? kz : N - kz;
            const float4 e = XS(&scoef[c * (N / 2 + 1) + s], 449) ? scoef[c * (N / 2 + 1) + s] : make_float4(0.f, 0.f, 0.f, 0.f);
            Coef<T> r;
            r.A = e.x; r.B = e.y; r.c2 = e.z; r.k2 = e.w;
            return r;
        }
    }
    return kcoef<T>(ks, table, i0, i1, i2);
}

// k-space sums of one updated mode: weight c2 |X|^2 (free energy) and
// weight |res|^2 (sse_calculation.cu:133-140).  On the FP32 path, with
// Mo_res = Mo, the residual comes from the update itself,
//   res = xi/dt + Mo k^2 ((1 - c2)(X - X') + eps X'),
// where X - X' of two nearby FP32 values is exact; otherwise the general form
// in FP64.
template <typename T>
__device__ __forceinline__ void diag_mode(const KSpace &ks, const Coef<T> &cf, cplx<T> xs, cplx<T> xw, cplx<T> noise,
                                          cplx<T> xn, DSum<T, NQ_PEN> &acc, T weight) {
    if constexpr (sizeof(T) == 4) {
        if (ks.Mo_res == ks.Mo) {
            const float m = ks.f_Mo * cf.k2, omc = 1.f - cf.c2, idt = 1.f / ks.f_dt;
            const float rr = noise.x * idt + m * (omc * (xs.x - xn.x) + ks.f_eps * xn.x);
            const float ri = noise.y * idt + m * (omc * (xs.y - xn.y) + ks.f_eps * xn.y);
            acc.add(0, weight * cf.c2 * (xs.x * xs.x + xs.y * xs.y));
            acc.add(1, weight * (rr * rr + ri * ri));
            return;
        }
    }
    const double xr = xs.x, xi = xs.y, k2 = cf.k2, c2 = cf.c2, w = weight;
    const double rr = ((double)xn.x - xr) / ks.dt + ks.Mo_res * k2 * ((1.0 - c2) * xr + (double)xw.x);
    const double ri = ((double)xn.y - xi) / ks.dt + ks.Mo_res * k2 * ((1.0 - c2) * xi + (double)xw.y);
    acc.add(0, (T)(w * c2 * (xr * xr + xi * xi)));
    acc.add(1, (T)(w * (rr * rr + ri * ri)));
}

// The update of one mode given its coefficients and noise (zero when off).
// (interior modes: never k = 0, so no pinning)
template <typename T, bool RED>
__device__ __forceinline__ cplx<T> update_coef(const KSpace &ks, const Coef<T> &cf, cplx<T> xs, cplx<T> xw,
                                               cplx<T> noise, DSum<T, NQ_PEN> &acc, T weight) {
    const cplx<T> num = cadd(xs, noise);
    cplx<T> xn = mk<T>(cf.A * num.x + cf.B * xw.x, cf.A * num.y + cf.B * xw.y);
    if (RED) diag_mode<T>(ks, cf, xs, xw, noise, xn, acc, weight);
    return xn;
}

template <typename T>
__device__ __forceinline__ cplx<T> update_mode(const KSpace &ks, const Inst &in, const PenArgs &args, int i0, int i1,
                                               int i2, cplx<T> xs, cplx<T> xw, DSum<T, NQ_PEN> &acc, T weight) {
    const Coef<T> cf = kcoef<T>(ks, in.table, i0, i1, i2);
    cplx<T> noise = mk<T>((T)0, (T)0);
    if (ks.noise_on) noise = noise_at<T>(ks, in.seed, in.nstream, i0, i1, i2, cf.k2);
    const cplx<T> num = cadd(xs, noise);
    cplx<T> xn = mk<T>(cf.A * num.x + cf.B * xw.x, cf.A * num.y + cf.B * xw.y);
    if (args.pin && i0 == 0 && i1 == 0 && i2 == 0) xn = mk<T>((T)in.pin, (T)0);
    if (args.want_red) diag_mode<T>(ks, cf, xs, xw, noise, xn, acc, weight);
    return xn;
}

// SPEC (args.Shat set): the pencil-axis spectrum of S is kept from one step
// to the next in its own array (Shat), so the pass reads Shat instead of
// transforming S forward, and writes the updated spectrum to Shat beside the
// inverse-transformed S that the xy passes read: one array more of HBM
// traffic (read and written) for one transform less (of three) in an
// issue-bound pass.  The 3-D slot-0 pass needs room for its unscaled results
// too (3 NG N values in bufS).
// Measured on GB300 (pencil per launch): 256^3 116 against 120 us (step
// 0.174 against 0.176 ms), 128^3 41.2 against 40.0 us, 512^3 1.212 against
// 1.181 ms, 64^3 no change; the 24-value plans, which park W in the scratch,
// spilled with it.  So lines of 256 only.  (Copying the spectrum into bufS
// with cp.async instead, which frees its registers through W's transform and
// keeps three blocks per SM resident at 80 registers, was slower: 130 against
// 120 us at 256^3.)
template <typename T, int N, int NG> __host__ __device__ constexpr bool spec_ok() {
    return reg_pen_ok<T, N>() && RP<N>::P <= 16 && N == 256 && NG == 2 &&
           3 * NG * N <= RPenShape<T, N, NG>::LINES * RPenShape<T, N, NG>::LP;
}

template <typename T, int N, int NG, bool RED, bool SPEC = false>
__global__ void __launch_bounds__(RPenShape<T, N, NG>::THREADS, RPenShape<T, N, NG>::MINB)
pencil_kernel_reg(PenArgs args, KSpace ks, const cplx<T> *__restrict__ twN) {
    static_assert(!SPEC || spec_ok<T, N, NG>(), "no room for the kept spectrum's slot-0 results");
    Inst in = inst_of<T>(ks);
    in.pin = pin_of(args);
    using S = RPenShape<T, N, NG>;
    constexpr int TX = S::TX, Q = S::Q, P = S::P;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *stw = reinterpret_cast<cplx<T> *>(smem_raw);
    cplx<T> *bufS = stw + N;
    cplx<T> *bufW = bufS + S::LINES * S::LP;
    double *sred = reinterpret_cast<double *>(bufW + S::LINES * S::LP);
    const int tid = threadIdx.x;
    for (int i = tid; i < N; i += S::THREADS)
        if (XG(&twN[i], 421) && XS(&stw[i], 422)) stw[i] = twN[i];
    // the shell coefficients of the block's columns, copied before the wait
    // on the previous pass (the tables do not change during a solve), so
    // that the update reads shared memory instead of one scattered L2 line
    // per mode; row |s1| of the block in 3-D (both mirror rows), 0 in 2-D
    const float4 *scoef = nullptr;
    if constexpr (S::CSM) {
        if (in.table) {
            float4 *sc = reinterpret_cast<float4 *>(sred + 32 * NQ_PEN);
            const float4 *tab = reinterpret_cast<const float4 *>(in.table);
            const int s1 = args.three_d ? signed_idx((int)blockIdx.y, ks.n1) : 0;
            const int kxb = blockIdx.x * TX;
            for (int e = tid; e < TX * S::CP; e += S::THREADS) {
                const int cc = e / S::CP, sz = e - cc * S::CP, ix = kxb + cc;
                const int m = ix * ix + s1 * s1 + sz * sz;
                if (ix < args.L0 && XS(&sc[e], 447) && XG(&tab[m], 448)) cp_async16(&sc[e], &tab[m]);
            }
            cp_async_commit();
            scoef = sc;
        }
    }
    pdl_wait();

    const int c = tid % TX, t = (tid / TX) % Q, g = tid / (TX * Q);
    const int p = blockIdx.y;
    const int y1 = p, y2 = (NG == 2) ? (ks.n1 - p) % ks.n1 : p;
    const int G = (NG == 2 && y2 != y1) ? 2 : 1;
    const int yg = (g == 0) ? y1 : y2;
    const int kx0 = blockIdx.x * TX;
    const bool valid = (g < G) && (kx0 + c < args.L0);
    const long long off = (long long)blockIdx.z * args.zstride + (long long)yg * args.gstride + kx0 + c;
    cplx<T> *gS = reinterpret_cast<cplx<T> *>(args.S) + off;
    const cplx<T> *gW = reinterpret_cast<const cplx<T> *>(args.W) + off;
    // SPEC: the state is read from (and its update written to) the kept
    // spectrum instead
    cplx<T> *gH = SPEC ? reinterpret_cast<cplx<T> *>(args.Shat) + off : gS;
    // Plans of 24 values per thread would hold 48 values of S and W through
    // both transforms (over 255 registers, with spills).  They load and
    // transform W first and keep it in its line's scratch of bufW, in natural
    // order (element kz at ln LP + kz), until the update; S is loaded and
    // transformed after.
    constexpr bool STASH = P > 16;
    // distance between the two groups' kx = 0 pencils of W in bufW
    constexpr int WG = STASH ? TX * S::LP : N;
    static_assert(!STASH || (N <= S::LP && (NG - 1) * WG + N <= S::LINES * S::LP),
                  "a line's scratch must hold its parked W pencil");
    cplx<T> vs[P], vw[P];
#pragma unroll
    for (int j = 0; j < P; j++) {
        const long long e = (long long)(t + Q * j) * args.es;
        if constexpr (!STASH) vs[j] = (valid && XG(&gH[e], 423)) ? gH[e] : mk<T>((T)0, (T)0);
        vw[j] = (valid && XG(&gW[e], 424)) ? gW[e] : mk<T>((T)0, (T)0);
    }
    __syncthreads();
    // this thread's coefficient copies are complete; the transform's first
    // barrier publishes every thread's
    if constexpr (S::CSM) cp_async_wait_all();
    const int ln = g * TX + c;
    if constexpr (STASH) {
        reg_fft<T, N, -1>(vw, t, bufW + ln * S::LP, stw);
        __syncthreads();   // every thread of the line is done reading its scratch
#pragma unroll
        for (int j = 0; j < P; j++)
            if (XS(&bufW[ln * S::LP + t + Q * j], 433)) bufW[ln * S::LP + t + Q * j] = vw[j];
#pragma unroll
        for (int j = 0; j < P; j++) {
            const long long e = (long long)(t + Q * j) * args.es;
            vs[j] = (valid && XG(&gH[e], 423)) ? gH[e] : mk<T>((T)0, (T)0);
        }
        if constexpr (!SPEC) reg_fft<T, N, -1>(vs, t, bufS + ln * S::LP, stw);
    } else if constexpr (SPEC) {
        reg_fft<T, N, -1>(vw, t, bufW + ln * S::LP, stw);
    } else {
        reg_fft2<T, N, -1>(vs, vw, t, bufS + ln * S::LP, bufW + ln * S::LP, stw);
    }
    const bool keep = SPEC && args.update;   // write the updated spectrum to Shat

    DSum<T, NQ_PEN> acc;
    const T sc = (T)args.scale;
    const int nh = args.L0;
    const cplx<T> zero = mk<T>((T)0, (T)0);

    // slot 0 (only in the block holding kx' = 0): the kx = 0 and kx = n0/2
    // planes separate with the mirror mode (-k1, -k2).  Those pencils go
    // through shared memory and every thread of the block takes a share,
    // which keeps this rare path small in the instruction stream.  The
    // pencils of S are published as [group][kz] at the start of bufS; those
    // of W as [group][kz] at the start of bufW, or where the stash already
    // holds them (group gg at gg WG).
    if (kx0 == 0) {
        cplx<T> *outS = bufS + G * N;                  // after the [group][kz] publish area of S
        cplx<T> *outU = bufS + 2 * G * N;              // SPEC: the unscaled results, for Shat
        __syncthreads();
        if (c == 0 && g < G) {
#pragma unroll
            for (int j = 0; j < P; j++) {
                if (XS(&bufS[g * N + t + Q * j], 425)) bufS[g * N + t + Q * j] = vs[j];
                if constexpr (!STASH)
                    if (XS(&bufW[g * N + t + Q * j], 426)) bufW[g * N + t + Q * j] = vw[j];
            }
        }
        __syncthreads();
#pragma unroll 1
        for (int idx = tid; idx < G * N; idx += S::THREADS) {
            const int gg = idx / N, kz = idx % N;
            const int yy = (gg == 0) ? y1 : y2;
            const int i1 = args.three_d ? yy : kz;
            const int i2 = args.three_d ? kz : 0;
            const int gm = (G == 2) ? 1 - gg : gg;
            const int kzm = (N - kz) % N;
            if (!XS(&bufW[gg * WG + kz], 427) || !XS(&bufW[gm * WG + kzm], 428) || !XS(&outS[gg * N + kz], 429)) continue;
            const cplx<T> xs = bufS[gg * N + kz], xw = bufW[gg * WG + kz];
            const cplx<T> ps = bufS[gm * N + kzm], pw = bufW[gm * WG + kzm];
            const T h = (T)0.5;
            const cplx<T> s0 = cscale(cadd(xs, cconj(ps)), h), sN = cscale(cmuli<-1>(csub(xs, cconj(ps))), h);
            const cplx<T> w0 = cscale(cadd(xw, cconj(pw)), h), wN = cscale(cmuli<-1>(csub(xw, cconj(pw))), h);
            const cplx<T> x0 = update_mode<T>(ks, in, args, 0, i1, i2, s0, w0, acc, (T)1);
            const cplx<T> xN = update_mode<T>(ks, in, args, nh, i1, i2, sN, wN, acc, (T)1);
            const cplx<T> packed = cadd(x0, cmuli<1>(xN));
            outS[gg * N + kz] = cscale(packed, sc);
            if constexpr (SPEC)
                if (XS(&outU[gg * N + kz], 437)) outU[gg * N + kz] = packed;
        }
        __syncthreads();
        if (c == 0 && g < G) {
#pragma unroll
            for (int j = 0; j < P; j++) {
                if (XS(&outS[g * N + t + Q * j], 430)) vs[j] = outS[g * N + t + Q * j];
                if constexpr (SPEC) {
                    const long long e = (long long)(t + Q * j) * args.es;
                    if (keep && XS(&outU[g * N + t + Q * j], 438) && XG(&gH[e], 439)) gH[e] = outU[g * N + t + Q * j];
                }
            }
        }
    }
    // interior columns: modes j and j + P/2 sit at kz and kz + N/2 and share
    // one Philox draw.  The draws are made first, in a rolled loop, into
    // shared memory (bufS is free between the two transforms; each thread
    // reads back only its own entries), so that the Philox and Box-Muller code
    // appears once in the instruction stream instead of P/2 times.
    const bool interior = valid && kx0 + c != 0;
    const int i0 = kx0 + c;
    cplx<T> *snoise = bufS;
    static_assert(P * S::THREADS <= S::LINES * S::LP, "noise staging must fit in bufS");
    if (ks.noise_on) {
        __syncthreads();   // the forward transform and the slot-0 pass are done with bufS
        if (interior) {
            // two draws per trip (two independent Philox chains in flight:
            // 256^3 pencil 104.6 -> 103.3 us against one per trip), one for
            // the 24-value plans, whose registers are spent
            auto draw = [&](int j) {
                const int kza = t + Q * j;
                const int i1a = args.three_d ? yg : kza, i2a = args.three_d ? kza : 0;
                cplx<T> ga, gb;
                noise_pair_unit<T>(ks, in.seed, in.nstream, i0, i1a, i2a, ga, gb);
                if (XS(&snoise[(j + P / 2) * S::THREADS + tid], 431)) {
                    snoise[j * S::THREADS + tid] = ga;
                    snoise[(j + P / 2) * S::THREADS + tid] = gb;
                }
            };
            if constexpr (P <= 16) {
#pragma unroll 2
                for (int j = 0; j < P / 2; j++) draw(j);
            } else {
#pragma unroll 1
                for (int j = 0; j < P / 2; j++) draw(j);
            }
        }
    }
    if (interior) {
#pragma unroll
        for (int j = 0; j < P / 2; j++) {
            const int kza = t + Q * j, kzb = kza + N / 2;
            const int i1a = args.three_d ? yg : kza, i2a = args.three_d ? kza : 0;
            const int i1b = args.three_d ? yg : kzb, i2b = args.three_d ? kzb : 0;
            const Coef<T> ca = pen_coef<T, N>(ks, in.table, scoef, c, i0, i1a, i2a, kza);
            const Coef<T> cb = pen_coef<T, N>(ks, in.table, scoef, c, i0, i1b, i2b, kzb);
            cplx<T> na = zero, nb = zero;
            if (ks.noise_on) {
                na = cscale(snoise[j * S::THREADS + tid], noise_amp_of<T>(ks, ca.k2));
                nb = cscale(snoise[(j + P / 2) * S::THREADS + tid], noise_amp_of<T>(ks, cb.k2));
            }
            cplx<T> wa = vw[j], wb = vw[j + P / 2];
            if constexpr (STASH) {
                wa = XS(&bufW[ln * S::LP + kza], 434) ? bufW[ln * S::LP + kza] : zero;
                wb = XS(&bufW[ln * S::LP + kzb], 435) ? bufW[ln * S::LP + kzb] : zero;
            }
            const cplx<T> xa = update_coef<T, RED>(ks, ca, vs[j], wa, na, acc, (T)2);
            const cplx<T> xb = update_coef<T, RED>(ks, cb, vs[j + P / 2], wb, nb, acc, (T)2);
            if constexpr (SPEC) {
                if (keep && XG(&gH[(long long)kza * args.es], 440) && XG(&gH[(long long)kzb * args.es], 441)) {
                    gH[(long long)kza * args.es] = xa;
                    gH[(long long)kzb * args.es] = xb;
                }
            }
            vs[j] = cscale(xa, sc);
            vs[j + P / 2] = cscale(xb, sc);
        }
    }
    if (RED) {
        double tot[NQ_PEN] = {acc.get(0), acc.get(1)};
        block_reduce_store<NQ_PEN>(tot, args.partials + block_slot() * NQ_PEN, sred);
    }
    if (!args.update) return;
    // The twiddles and the global addresses are taken afresh from opaque
    // copies of their base pointers: otherwise the compiler keeps the forward
    // transform's twiddles and the loads' addresses in registers through the
    // whole update (158 instead of 194 registers at N = 128).
    reg_fft<T, N, +1>(vs, t, bufS + ln * S::LP, opaque(stw));
    if (!valid) return;
    cplx<T> *o = opaque(gS) + (long long)t * args.es;
    const long long step = (long long)Q * args.es;
#pragma unroll
    for (int j = 0; j < P; j++, o += step)
        if (XG(o, 432)) *o = vs[j];
}

// ---------------------------------------------------------------------------
// Persistent kept-spectrum pencil (FP32, the two mirror rows of pencil_kernel_reg
// per tile).  Each block loops over tiles: while one tile is transformed and
// updated, W of the block's next tile is copied into a stage (cp.async, each
// thread its own elements, so the stage needs no barrier of its own) and the
// next tile's shell coefficients into the other half of a double buffer, so
// that only a block's first tile waits for W.  The kept spectrum of a tile is
// loaded into registers at its start and is first needed after W's
// transform.  One transpose scratch serves W's forward transform, the slot-0
// areas, the noise staging and S's inverse transform in turn.  Per mode the
// arithmetic is pencil_kernel_reg's; the block sums go to the slot of the tile
// (the same layout as one block per tile).
// ---------------------------------------------------------------------------
template <int N> struct PPenShape {
    using R = RPenShape<float, N, 2>;
    static constexpr int TX = R::TX, Q = R::Q, P = R::P, THREADS = R::THREADS, LINES = R::LINES, LP = R::LP;
    static constexpr int CP = R::CP;
    static constexpr size_t SCR = (size_t)LINES * LP;       // complex slots
    static constexpr size_t STAGE = (size_t)P * THREADS;    // complex slots
    static constexpr size_t OFF_SCR = sizeof(cplx<float>) * N;
    static constexpr size_t OFF_STAGE = OFF_SCR + sizeof(cplx<float>) * SCR;
    static constexpr size_t OFF_RED = OFF_STAGE + sizeof(cplx<float>) * STAGE;
    static constexpr size_t OFF_COEF = OFF_RED + sizeof(double) * 32 * NQ_PEN;
    static constexpr size_t SMEM = OFF_COEF + 2 * (size_t)TX * CP * sizeof(float4);
    static_assert(OFF_COEF % 16 == 0, "16-byte coefficient copies");
    // the scratch holds a line's transpose, the slot-0 areas (published S
    // and W pencils of both rows and the results: 6 N) and the noise staging
    static_assert(6 * N <= SCR && STAGE <= SCR, "scratch areas");
    static_assert(2 * (SMEM + 1024) <= 233472, "two blocks per SM");
};

template <int N, bool RED>
__global__ void __launch_bounds__(PPenShape<N>::THREADS, 2)
pencil_kernel_pst(PenArgs args, KSpace ks, const cplx<float> *__restrict__ twN, int nkx, int npairs, int ntiles) {
    using T = float;
    using S = PPenShape<N>;
    constexpr int TX = S::TX, Q = S::Q, P = S::P, THREADS = S::THREADS, CP = S::CP;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *stw = reinterpret_cast<cplx<T> *>(smem_raw);
    cplx<T> *scr = reinterpret_cast<cplx<T> *>(smem_raw + S::OFF_SCR);
    cplx<T> *stage = reinterpret_cast<cplx<T> *>(smem_raw + S::OFF_STAGE);
    double *sred = reinterpret_cast<double *>(smem_raw + S::OFF_RED);
    float4 *coefs = reinterpret_cast<float4 *>(smem_raw + S::OFF_COEF);
    const int tid = threadIdx.x;
    const int c = tid % TX, t = (tid / TX) % Q, g = tid / (TX * Q);
    const int ln = g * TX + c;
    const cplx<T> zero = mk<T>((T)0, (T)0);
    for (int i = tid; i < N; i += THREADS)
        if (XG(&twN[i], 451) && XS(&stw[i], 452)) stw[i] = twN[i];

    // this thread's share of tile tt's shell coefficients, into buffer dst
    auto coef_copy = [&](int tt, float4 *dst) {
        const int kx0 = (tt % nkx) * TX, rest = tt / nkx, pp = rest % npairs;
        const float4 *tab = reinterpret_cast<const float4 *>(inst_at<T>(ks, rest / npairs).table);
        if (!tab) return;
        const int s1 = signed_idx(pp, ks.n1);
        for (int e = tid; e < TX * CP; e += THREADS) {
            const int cc = e / CP, sz = e - cc * CP, ix = kx0 + cc;
            const int m = ix * ix + s1 * s1 + sz * sz;
            if (ix < args.L0 && XS(&dst[e], 453) && XG(&tab[m], 454)) cp_async16(&dst[e], &tab[m]);
        }
    };
    // this thread's elements of W of tile tt, into its own stage slots
    auto w_copy = [&](int tt) {
        const int kx0 = (tt % nkx) * TX, rest = tt / nkx, pp = rest % npairs, zi = rest / npairs;
        const int yy1 = pp, yy2 = (ks.n1 - pp) % ks.n1;
        const bool ok = (g == 0 || yy2 != yy1) && (kx0 + c < args.L0);
        const cplx<T> *gw = reinterpret_cast<const cplx<T> *>(args.W) + (long long)zi * args.zstride +
                            (long long)(g == 0 ? yy1 : yy2) * args.gstride + kx0 + c;
#pragma unroll
        for (int j = 0; j < P; j++) {
            cplx<T> *d = &stage[j * THREADS + tid];
            const long long e = (long long)(t + Q * j) * args.es;
            if (!XS(d, 455)) continue;
            if (ok && XG(&gw[e], 456)) cp_async8(d, &gw[e]);
            else *d = zero;
        }
    };

    int tile = blockIdx.x;
    if (tile < ntiles) coef_copy(tile, coefs);   // the tables do not change during a solve
    pdl_wait();
    if (tile < ntiles) w_copy(tile);
    cp_async_commit();
    int buf = 0;
    for (; tile < ntiles; tile += gridDim.x, buf ^= 1) {
        const int kxb = tile % nkx, rest = tile / nkx, p = rest % npairs, zi = rest / npairs;
        const int y1 = p, y2 = (ks.n1 - p) % ks.n1;
        const int G = (y2 != y1) ? 2 : 1;
        const int yg = (g == 0) ? y1 : y2;
        const int kx0 = kxb * TX;
        const bool valid = (g < G) && (kx0 + c < args.L0);
        Inst in = inst_at<T>(ks, zi);
        in.pin = args.pin_values ? args.pin_values[zi] : args.pin_value;
        const long long off = (long long)zi * args.zstride + (long long)yg * args.gstride + kx0 + c;
        cplx<T> *gH = reinterpret_cast<cplx<T> *>(args.Shat) + off;
        const float4 *scoef = in.table ? coefs + buf * TX * CP : nullptr;

        // W and the coefficients of this tile have landed (every thread's
        // copies, after the barrier), and every thread is done with the last tile
        cp_async_wait_all();
        __syncthreads();
        cplx<T> vs[P], vw[P];
#pragma unroll
        for (int j = 0; j < P; j++) vw[j] = XS(&stage[j * THREADS + tid], 457) ? stage[j * THREADS + tid] : zero;
        const int nt = tile + (int)gridDim.x;
        if (nt < ntiles) {
            w_copy(nt);
            coef_copy(nt, coefs + (buf ^ 1) * TX * CP);
        }
        cp_async_commit();
#pragma unroll
        for (int j = 0; j < P; j++) {
            const long long e = (long long)(t + Q * j) * args.es;
            vs[j] = (valid && XG(&gH[e], 458)) ? gH[e] : zero;
        }
        reg_fft<T, N, -1>(vw, t, scr + ln * S::LP, stw);
        const bool keep = args.update;   // write the updated spectrum to Shat
        DSum<T, NQ_PEN> acc;
        const T sc = (T)args.scale;
        const int nh = args.L0;

        // slot 0 (tiles holding kx' = 0), as pencil_kernel_reg: published S
        // and W pencils of both rows, the results for the kx = 0 threads, the
        // unscaled results straight to Shat
        if (kx0 == 0) {
            cplx<T> *pubS = scr, *pubW = scr + 2 * N, *outS = scr + 4 * N;
            __syncthreads();
            if (c == 0 && g < G) {
#pragma unroll
                for (int j = 0; j < P; j++) {
                    if (XS(&pubS[g * N + t + Q * j], 459) && XS(&pubW[g * N + t + Q * j], 460)) {
                        pubS[g * N + t + Q * j] = vs[j];
                        pubW[g * N + t + Q * j] = vw[j];
                    }
                }
            }
            __syncthreads();
#pragma unroll 1
            for (int idx = tid; idx < G * N; idx += THREADS) {
                const int gg = idx / N, kz = idx % N;
                const int yy = (gg == 0) ? y1 : y2;
                const int gm = (G == 2) ? 1 - gg : gg;
                const int kzm = (N - kz) % N;
                if (!XS(&pubW[gm * N + kzm], 461) || !XS(&outS[gg * N + kz], 462)) continue;
                const cplx<T> xs = pubS[gg * N + kz], xw = pubW[gg * N + kz];
                const cplx<T> ps = pubS[gm * N + kzm], pw = pubW[gm * N + kzm];
                const T h = (T)0.5;
                const cplx<T> s0 = cscale(cadd(xs, cconj(ps)), h), sN = cscale(cmuli<-1>(csub(xs, cconj(ps))), h);
                const cplx<T> w0 = cscale(cadd(xw, cconj(pw)), h), wN = cscale(cmuli<-1>(csub(xw, cconj(pw))), h);
                const cplx<T> x0 = update_mode<T>(ks, in, args, 0, yy, kz, s0, w0, acc, (T)1);
                const cplx<T> xN = update_mode<T>(ks, in, args, nh, yy, kz, sN, wN, acc, (T)1);
                const cplx<T> packed = cadd(x0, cmuli<1>(xN));
                outS[gg * N + kz] = cscale(packed, sc);
                cplx<T> *h0 = reinterpret_cast<cplx<T> *>(args.Shat) + (long long)zi * args.zstride +
                              (long long)yy * args.gstride + (long long)kz * args.es;
                if (keep && XG(h0, 463)) *h0 = packed;
            }
            __syncthreads();
            if (c == 0 && g < G) {
#pragma unroll
                for (int j = 0; j < P; j++)
                    if (XS(&outS[g * N + t + Q * j], 464)) vs[j] = outS[g * N + t + Q * j];
            }
        }
        // interior columns: the noise draws first, two per trip, into the
        // scratch (each thread reads back only its own entries)
        const bool interior = valid && kx0 + c != 0;
        const int i0 = kx0 + c;
        cplx<T> *snoise = scr;
        if (ks.noise_on) {
            __syncthreads();   // the transform and the slot-0 pass are done with the scratch
            if (interior) {
#pragma unroll 2
                for (int j = 0; j < P / 2; j++) {
                    cplx<T> ga, gb;
                    noise_pair_unit<T>(ks, in.seed, in.nstream, i0, yg, t + Q * j, ga, gb);
                    if (XS(&snoise[(j + P / 2) * THREADS + tid], 465)) {
                        snoise[j * THREADS + tid] = ga;
                        snoise[(j + P / 2) * THREADS + tid] = gb;
                    }
                }
            }
        }
        if (interior) {
#pragma unroll
            for (int j = 0; j < P / 2; j++) {
                const int kza = t + Q * j, kzb = kza + N / 2;
                const Coef<T> ca = pen_coef<T, N>(ks, in.table, scoef, c, i0, yg, kza, kza);
                const Coef<T> cb = pen_coef<T, N>(ks, in.table, scoef, c, i0, yg, kzb, kzb);
                cplx<T> na = zero, nb = zero;
                if (ks.noise_on) {
                    na = cscale(snoise[j * THREADS + tid], noise_amp_of<T>(ks, ca.k2));
                    nb = cscale(snoise[(j + P / 2) * THREADS + tid], noise_amp_of<T>(ks, cb.k2));
                }
                const cplx<T> xa = update_coef<T, RED>(ks, ca, vs[j], vw[j], na, acc, (T)2);
                const cplx<T> xb = update_coef<T, RED>(ks, cb, vs[j + P / 2], vw[j + P / 2], nb, acc, (T)2);
                if (keep && XG(&gH[(long long)kza * args.es], 466) && XG(&gH[(long long)kzb * args.es], 467)) {
                    gH[(long long)kza * args.es] = xa;
                    gH[(long long)kzb * args.es] = xb;
                }
                vs[j] = cscale(xa, sc);
                vs[j + P / 2] = cscale(xb, sc);
            }
        }
        if (RED) {
            double tot[NQ_PEN] = {acc.get(0), acc.get(1)};
            block_reduce_store<NQ_PEN>(tot, args.partials + (size_t)tile * NQ_PEN, sred);
        }
        if (!args.update) continue;
        reg_fft<T, N, +1>(vs, t, scr + ln * S::LP, opaque(stw));
        if (valid) {
            cplx<T> *o = opaque(reinterpret_cast<cplx<T> *>(args.S)) + off + (long long)t * args.es;
            const long long step = (long long)Q * args.es;
#pragma unroll
            for (int j = 0; j < P; j++, o += step)
                if (XG(o, 468)) *o = vs[j];
        }
    }
    cp_async_wait_all();   // no copy outstanding when the block exits
}

}  // namespace xpfc
