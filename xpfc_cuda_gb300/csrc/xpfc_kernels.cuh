// xpfc_kernels.cuh -- the passes of the XPFC step on sm_103a.
//
// Device layout (n0 = fastest axis, the real-FFT axis; n2 = 1 in 2-D):
//   real field      T      [n2][n1][n0]
//   packed spectrum cplx<T>[n2][n1][n0/2]   (same bytes as the real field)
// Row transform of a real row x (length n0 = 2 L): z[m] = x[2m] + i x[2m+1],
// Z = FFT_L(z), X[k] = E[k] + W_{2L}^k O[k] with E = (Z[k] + conj Z[L-k])/2,
// O = -i (Z[k] - conj Z[L-k])/2; slot 0 stores X[0] + i X[L] (both real).
// The other axes are full complex FFTs of the packed rows, so after them
// slot 0 holds X0 + i XN, X0 and XN the Hermitian (k1,k2)-planes of kx = 0 and
// kx = n0/2; they separate with the mirror (-k1,-k2):
//   X0 = (P + conj Pm)/2,  XN = (P - conj Pm)/(2i).
#pragma once
#include "fft_core.cuh"

namespace xpfc {

constexpr int NQ_ROW = 4;   // sum x, sum P2(x), sum P3(x), sum P4(x)
constexpr int NQ_PEN = 2;   // sum w c2 |X|^2, sum w |res|^2

// ---------------------------------------------------------------------------
// shapes chosen at compile time from the line length
// ---------------------------------------------------------------------------
template <int L> struct RowShape {
    static constexpr int TPL = L >= 32 ? L / 16 : (L >= 16 ? 2 : 1);
    static constexpr int ROWS = (TPL >= 128) ? 1 : (128 / TPL > 32 ? 32 : 128 / TPL);
    static constexpr int THREADS = ROWS * TPL;
};

template <typename T, int L> struct ColShape {
    // tile width: keep the [L][TX] tile near 64 KB
    static constexpr int BYTES = 65536;
    static constexpr int TXc = BYTES / (L * (int)sizeof(cplx<T>));
    static constexpr int TX = TXc >= 16 ? 16 : TXc >= 8 ? 8 : TXc >= 4 ? 4 : TXc >= 2 ? 2 : 1;
    static constexpr int TPLc = L >= 32 ? L / 16 : 1;
    static constexpr int TPL = (TPLc * TX > 1024) ? 1024 / TX : TPLc;
    static constexpr int THREADS = TX * TPL;
};

template <typename T, int L, int NG> struct PenShape {
    // 2*NG [L][TX] tiles (S and W; pencil and, in 3-D, its mirror) near 128 KB;
    // long 2-D pencils (L >= 256; a 2-D grid has only n0/2 of them) keep
    // their tiles 32 bytes wide (four FP32 or two FP64 columns) to give the
    // grid enough blocks; every block stays a whole number of warps
    static constexpr int BYTES = 131072;
    static constexpr int TXc0 = BYTES / (2 * NG * L * (int)sizeof(cplx<T>));
    static constexpr int TXc =
        (NG == 1 && L >= 256 && TXc0 * (int)sizeof(cplx<T>) > 32) ? 32 / (int)sizeof(cplx<T>) : TXc0;
    static constexpr int TX = TXc >= 16 ? 16 : TXc >= 8 ? 8 : TXc >= 4 ? 4 : TXc >= 2 ? 2 : 1;
    static constexpr int TPLc = L >= 32 ? L / 16 : 1;
    static constexpr int TPL = (2 * NG * TX * TPLc > 1024) ? 1024 / (2 * NG * TX) : TPLc;
    static constexpr int THREADS = 2 * NG * TX * TPL;
    static_assert(THREADS % 32 == 0, "the reductions use full-warp shuffles");
};

// ---------------------------------------------------------------------------
// real-space op
// ---------------------------------------------------------------------------
// The reference's float power (power_functions.cu:47), kept out of line: it
// runs only in reference-compatible mode and would otherwise be inlined at
// every call site of the unrolled loops.
static __device__ __noinline__ float ref_powf(float x, float p) { return powf(x, p); }

template <typename T> __device__ __forceinline__ T powi(T x, int p, int ref_compat) {
    if (ref_compat) return (T)ref_powf((float)x, (float)p);
    if (p == 2) return x * x;
    if (p == 3) return x * x * x;
    T s = x * x;
    return s * s;
}

// Programmatic dependent launch.  The step's passes are launched with
// programmatic stream serialisation, so a pass's blocks may be scheduled while
// the previous pass drains; each pass reads only constant tables (twiddles)
// before pdl_wait(), which blocks until the previous grid has completed and
// its writes are visible, and then lets the next pass start launching.
// Without the launch attribute both instructions are no-ops.
__device__ __forceinline__ void pdl_wait() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// The same pointer, with its value hidden from the compiler: addresses (and
// shared-memory loads) derived from it are recomputed at the new use instead
// of being kept in registers from an earlier use of the same expressions.
template <typename P> __device__ __forceinline__ P *opaque(P *p) {
    asm volatile("" : "+l"(p));
    return p;
}

// Batched launches: grid z indexes the instance; instance z's field starts
// z * zstride complex elements after the base pointers and its partial sums
// follow the other instances' (block_slot).  One field: zstride = 0, nz = 1.
__device__ __forceinline__ size_t block_slot() {
    return ((size_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
}
__host__ __device__ inline unsigned grid_z(int nz) { return nz > 1 ? (unsigned)nz : 1u; }

struct RowArgs {
    const void *in;
    void *out;
    void *real_out;       // optional copy of the real field (type T), may be null
    long long nrows;
    double a, b;
    double scale;         // multiplies the inverse-transform output
    double *partials;     // [instance][gridDim.x][NQ_ROW] when want_red
    int want_red;
    int ref_compat;
    long long zstride;    // complex elements between batched instances
    int nz;               // batched instances (0 or 1: one field)
};

enum { ROW_FWD = 0, ROW_INV = 1, ROW_FUSED = 2, ROW_NL_FWD = 3 };

// C2R pre-processing of one row (thread t of TPL handles pairs k, L-k)
template <typename T, int L, int TPL>
__device__ __forceinline__ void row_unpack(cplx<T> *line, int t, const cplx<T> *__restrict__ tw2) {
    using I = LineIdx<T, ROW_LAYOUT>;
    for (int k = t; k <= L / 2; k += TPL) {
        if (k == 0) {
            cplx<T> p = line[I::at(0)];
            // Z0 = (X0 + XL) + i (X0 - XL)
            line[I::at(0)] = mk<T>(p.x + p.y, p.x - p.y);
            continue;
        }
        const int kk = L - k;
        if (!XS(&line[I::at(k)], 301) || !XS(&line[I::at(kk)], 302) || !XS(&tw2[k], 303)) continue;
        cplx<T> xk = line[I::at(k)], xc = line[I::at(kk)];
        // Z[k] = (Xk + conj X[L-k]) + i (Xk - conj X[L-k]) W^{-k}
        cplx<T> e = cadd(xk, cconj(xc));
        cplx<T> o = cmulc(csub(xk, cconj(xc)), tw2[k]);
        cplx<T> zk = cadd(e, cmuli<1>(o));
        if (kk != k) {
            // Z[L-k] from X[L-k] and conj X[k]; W_{2L}^{-(L-k)} = -W_{2L}^{k}
            cplx<T> e2 = cadd(xc, cconj(xk));
            cplx<T> o2 = cmul(csub(xc, cconj(xk)), tw2[k]);
            o2 = mk<T>(-o2.x, -o2.y);
            line[I::at(kk)] = cadd(e2, cmuli<1>(o2));
        }
        line[I::at(k)] = zk;
    }
}

// R2C post-processing of one row, packing X[L] into slot 0
template <typename T, int L, int TPL>
__device__ __forceinline__ void row_pack(cplx<T> *line, int t, const cplx<T> *__restrict__ tw2) {
    using I = LineIdx<T, ROW_LAYOUT>;
    const T h = (T)0.5;
    for (int k = t; k <= L / 2; k += TPL) {
        if (k == 0) {
            cplx<T> z = line[I::at(0)];
            line[I::at(0)] = mk<T>(z.x + z.y, z.x - z.y);
            continue;
        }
        const int kk = L - k;
        cplx<T> zk = line[I::at(k)], zc = line[I::at(kk)];
        // X[k] = (Zk + conj Zc)/2 - i W^k (Zk - conj Zc)/2
        cplx<T> e = cadd(zk, cconj(zc));
        cplx<T> o = cmul(csub(zk, cconj(zc)), tw2[k]);
        cplx<T> xk = cscale(csub(e, cmuli<1>(o)), h);
        if (kk != k) {
            // W_{2L}^{L-k} = -conj(W_{2L}^k)
            cplx<T> e2 = cadd(zc, cconj(zk));
            cplx<T> o2 = cmulc(csub(zc, cconj(zk)), tw2[k]);
            o2 = mk<T>(-o2.x, -o2.y);
            line[I::at(kk)] = cscale(csub(e2, cmuli<1>(o2)), h);
        }
        line[I::at(k)] = xk;
    }
}

// Row pass over rows of n0 = 2L reals.  One block handles ROWS rows.
template <typename T, int L, int MODE>
__global__ void __launch_bounds__(RowShape<L>::THREADS)
row_kernel(RowArgs args, const cplx<T> *__restrict__ twL, const cplx<T> *__restrict__ tw2L) {
    using S = RowShape<L>;
    using I = LineIdx<T, ROW_LAYOUT>;
    constexpr int SPAN = I::span(L);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *stw = reinterpret_cast<cplx<T> *>(smem_raw);          // L
    cplx<T> *stw2 = stw + L;                                        // L
    cplx<T> *lines = stw2 + L;                                      // ROWS * SPAN
    double *sred = reinterpret_cast<double *>(lines + S::ROWS * SPAN);

    const int tid = threadIdx.x;
    for (int i = tid; i < L; i += S::THREADS) {
        if (XG(&twL[i], 311) && XG(&tw2L[i], 312) && XS(&stw[i], 313) && XS(&stw2[i], 314)) {
            stw[i] = twL[i];
            stw2[i] = tw2L[i];
        }
    }
    pdl_wait();
    const long long row0 = (long long)blockIdx.x * S::ROWS;
    const int nvalid = (int)min((long long)S::ROWS, args.nrows - row0);
    const long long zoff = (long long)blockIdx.z * args.zstride;
    const cplx<T> *gin = reinterpret_cast<const cplx<T> *>(args.in) + zoff + row0 * L;
    for (int e = tid; e < nvalid * L; e += S::THREADS) {
        const int r = e / L, c = e - r * L;
        if (XG(&gin[e], 315) && XS(&lines[r * SPAN + I::at(c)], 316)) lines[r * SPAN + I::at(c)] = gin[e];
    }
    __syncthreads();

    const int r = tid / S::TPL, t = tid - r * S::TPL;
    cplx<T> *line = lines + r * SPAN;

    if (MODE == ROW_INV || MODE == ROW_FUSED) {
        row_unpack<T, L, S::TPL>(line, t, stw2);
        __syncthreads();
        line_fft<T, L, +1, S::TPL, ROW_LAYOUT>(line, t, stw);
    }

    if (MODE == ROW_INV) {
        const T sc = (T)args.scale;
        for (int m = t; m < L; m += S::TPL) line[I::at(m)] = cscale(line[I::at(m)], sc);
        __syncthreads();
    } else if (MODE == ROW_FUSED || MODE == ROW_NL_FWD) {
        // real-space op: n -> N(n) = -a n^2 + b n^3, with FP64 sums
        double v[NQ_ROW] = {0.0, 0.0, 0.0, 0.0};
        const T sc = (T)args.scale;
        const T a = (T)args.a, b = (T)args.b;
        const bool valid = r < nvalid;
        T *rout = args.real_out ? reinterpret_cast<T *>(args.real_out) + 2 * zoff + (row0 + r) * (2 * L) : nullptr;
        for (int m = t; m < L; m += S::TPL) {
            cplx<T> z = line[I::at(m)];
            T x0 = z.x, x1 = z.y;
            if (MODE == ROW_FUSED) { x0 *= sc; x1 *= sc; }
            if (rout && valid && XG(&rout[2 * m + 1], 317)) { rout[2 * m] = x0; rout[2 * m + 1] = x1; }
            T p20 = powi(x0, 2, args.ref_compat), p21 = powi(x1, 2, args.ref_compat);
            T p30 = powi(x0, 3, args.ref_compat), p31 = powi(x1, 3, args.ref_compat);
            if (args.want_red && valid) {
                v[0] += (double)x0 + (double)x1;
                v[1] += (double)p20 + (double)p21;
                v[2] += (double)p30 + (double)p31;
                v[3] += (double)powi(x0, 4, args.ref_compat) + (double)powi(x1, 4, args.ref_compat);
            }
            line[I::at(m)] = mk<T>(-a * p20 + b * p30, -a * p21 + b * p31);
        }
        if (args.want_red) block_reduce_store<NQ_ROW>(v, args.partials + block_slot() * NQ_ROW, sred);
        __syncthreads();
    }

    if (MODE != ROW_INV) {
        line_fft<T, L, -1, S::TPL, ROW_LAYOUT>(line, t, stw);
        row_pack<T, L, S::TPL>(line, t, stw2);
        __syncthreads();
    }

    cplx<T> *gout = reinterpret_cast<cplx<T> *>(args.out) + zoff + row0 * L;
    for (int e = tid; e < nvalid * L; e += S::THREADS) {
        const int rr = e / L, c = e - rr * L;
        if (XG(&gout[e], 318) && XS(&lines[rr * SPAN + I::at(c)], 319)) gout[e] = lines[rr * SPAN + I::at(c)];
    }
}

template <typename T, int L> constexpr size_t row_smem_bytes() {
    using S = RowShape<L>;
    return sizeof(cplx<T>) * (2 * L + S::ROWS * LineIdx<T, ROW_LAYOUT>::span(L)) + sizeof(double) * 32 * NQ_ROW;
}

// ---------------------------------------------------------------------------
// Column pass: C2C FFT along a strided axis for tiles of TX adjacent columns.
// Block (x = column tile, y = outer index); element e of column c of the tile
// lives at base + e*es + c with base = x*TX + y*ostride.
// ---------------------------------------------------------------------------
struct ColArgs {
    const void *in;
    void *out;
    long long es;         // element stride (complex units)
    long long ostride;    // stride per blockIdx.y
    double scale;
    int ncols;            // columns in a row (n0/2); the last tile may be partial
    long long zstride;    // complex elements between batched instances
    int nz;               // batched instances (0 or 1: one field)
};

template <typename T, int L, int DIR>
__global__ void __launch_bounds__(ColShape<T, L>::THREADS)
col_kernel(ColArgs args, const cplx<T> *__restrict__ twL) {
    using S = ColShape<T, L>;
    constexpr int TX = S::TX;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *stw = reinterpret_cast<cplx<T> *>(smem_raw);
    cplx<T> *tile = stw + L;
    const int tid = threadIdx.x;
    for (int i = tid; i < L; i += S::THREADS)
        if (XG(&twL[i], 321) && XS(&stw[i], 322)) stw[i] = twL[i];
    pdl_wait();
    const long long base =
        (long long)blockIdx.x * TX + (long long)blockIdx.y * args.ostride + (long long)blockIdx.z * args.zstride;
    const cplx<T> *gin = reinterpret_cast<const cplx<T> *>(args.in) + base;
    const int c = tid % TX, t = tid / TX;
    const bool cvalid = (int)blockIdx.x * TX + c < args.ncols;
    if (cvalid)
        for (int e = t; e < L; e += S::TPL)
            if (XG(&gin[e * args.es + c], 323) && XS(&tile[e * TX + c], 324)) tile[e * TX + c] = gin[e * args.es + c];
    __syncthreads();
    line_fft<T, L, DIR, S::TPL, TX>(tile + c, t, stw);
    cplx<T> *gout = reinterpret_cast<cplx<T> *>(args.out) + base;
    const T sc = (T)args.scale;
    if (!cvalid) return;
    if (args.scale != 1.0)
        for (int e = t; e < L; e += S::TPL) {
            if (XG(&gout[e * args.es + c], 325)) gout[e * args.es + c] = cscale(tile[e * TX + c], sc);
        }
    else
        for (int e = t; e < L; e += S::TPL) {
            if (XG(&gout[e * args.es + c], 326)) gout[e * args.es + c] = tile[e * TX + c];
        }
}

template <typename T, int L> constexpr size_t col_smem_bytes() {
    using S = ColShape<T, L>;
    return sizeof(cplx<T>) * (L + L * S::TX);
}

// ---------------------------------------------------------------------------
// k-space coefficients
// ---------------------------------------------------------------------------
struct KSpace {
    int n0, n1, n2;                 // grid (n0 real axis)
    double dk0sq, dk1sq, dk2sq;     // (2 pi/L_d)^2
    const void *table;              // per shell m: {A, B, c2, k2} in T, or null
    long long tstride;              // table entries between batched instances
    int mmax;
    // on-the-fly coefficients (no table)
    double dt, Mo, Mo_res, eps;
    int npeaks, envelope;
    double pk_k[8], pk_inv2a2[8], pk_dw[8];
    // noise
    int noise_on;
    double noise_scale;             // amp * sqrt(cells)
    unsigned long long noise_seed;
    const unsigned long long *seeds; // per batched instance (null: noise_seed)
    long long step;
    // a step call replayed from a captured graph reads its first iteration
    // from this device word and adds step (null: step alone)
    const long long *step_base;
    // the same constants in FP32 for the mixed path (no FP64 work per mode)
    float f_dk0sq, f_dk1sq, f_dk2sq, f_dt, f_Mo, f_eps, f_noise_scale;
    float f_pk_k[8], f_pk_inv2a2[8], f_pk_dw[8];
};

template <typename T> struct Coef { T A, B, c2, k2; };

// This block's instance (grid z) of a batched launch: its coefficient table
// and noise seed, resolved once per block so that the per-mode code does not
// see the batch.
struct Inst {
    const void *table;
    unsigned long long seed;
    unsigned long long nstream;   // Philox stream word of this iteration's noise: 1 + iteration
    double pin;   // the pinned k = 0 value (pencil passes; set by the kernel)
};
// instance z of a batched launch
template <typename T>
__device__ __forceinline__ Inst inst_at(const KSpace &k, int z) {
    Inst r;
    r.table = k.table;
    r.seed = k.noise_seed;
    r.pin = 0.0;
    r.nstream = 1ull + (unsigned long long)(k.step + (k.step_base ? *k.step_base : 0ll));
    if (k.tstride && k.table)
        r.table = reinterpret_cast<const char *>(k.table) + (size_t)z * k.tstride * 4 * sizeof(T);
    if (k.seeds) r.seed = k.seeds[z];
    return r;
}
template <typename T>
__device__ __forceinline__ Inst inst_of(const KSpace &k) {
    return inst_at<T>(k, blockIdx.z);
}

__device__ __forceinline__ int signed_idx(int i, int n) { return 2 * i <= n ? i : i - n; }

template <typename T>
__device__ __forceinline__ Coef<T> kcoef(const KSpace &ks, const void *table, int i0, int i1, int i2) {
    const int s1 = signed_idx(i1, ks.n1), s2 = signed_idx(i2, ks.n2);
    Coef<T> r;
    if (table) {
        const int m = i0 * i0 + s1 * s1 + s2 * s2;
        if constexpr (sizeof(T) == 4) {
            const float4 e = __ldg(reinterpret_cast<const float4 *>(table) + m);
            r.A = e.x; r.B = e.y; r.c2 = e.z; r.k2 = e.w;
        } else {
            const double2 e0 = __ldg(reinterpret_cast<const double2 *>(table) + 2 * (size_t)m);
            const double2 e1 = __ldg(reinterpret_cast<const double2 *>(table) + 2 * (size_t)m + 1);
            r.A = e0.x; r.B = e0.y; r.c2 = e1.x; r.k2 = e1.y;
        }
        return r;
    }
    const bool f = sizeof(T) == 4;
    const T k2 = (f ? (T)ks.f_dk0sq : (T)ks.dk0sq) * (T)(i0 * i0) + (f ? (T)ks.f_dk1sq : (T)ks.dk1sq) * (T)(s1 * s1) +
                 (f ? (T)ks.f_dk2sq : (T)ks.dk2sq) * (T)(s2 * s2);
    const T kk = sqrt(k2);
    T c2 = (T)0;
    for (int p = 0; p < ks.npeaks; p++) {
        const T d = kk - (f ? (T)ks.f_pk_k[p] : (T)ks.pk_k[p]);
        const T v = (f ? (T)ks.f_pk_dw[p] : (T)ks.pk_dw[p]) * exp(-(d * d) * (f ? (T)ks.f_pk_inv2a2[p] : (T)ks.pk_inv2a2[p]));
        c2 = ks.envelope == 0 ? c2 + v : (p == 0 || v > c2 ? v : c2);
    }
    const T dt = f ? (T)ks.f_dt : (T)ks.dt, Mo = f ? (T)ks.f_Mo : (T)ks.Mo, eps = f ? (T)ks.f_eps : (T)ks.eps;
    const T den = ((T)1 + k2 * dt * Mo * ((T)1 - eps) - k2 * Mo * dt * c2);
    r.A = (T)1 / den;
    r.B = -(k2 * Mo * dt) / den;
    r.c2 = c2;
    r.k2 = k2;
    return r;
}

// Square root through the hardware approximation (relative error about
// 2^-23): enough for noise amplitudes, one instruction instead of the
// correctly rounded sequence.
__device__ __forceinline__ float sqrt_approx(float x) {
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ float lg2_approx(float x) {
    float r;
    asm("lg2.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Box-Muller of two 32-bit draws: u1 = (a+1) 2^-32 in (0,1], u2 = b 2^-32.
// FP32 uses the hardware log/sqrt/sin/cos approximations (the noise only
// needs its distribution); FP64 the accurate functions.
template <typename T>
__device__ __forceinline__ void box_muller(uint32_t a, uint32_t b, T &g0, T &g1) {
    if (sizeof(T) == 8) {
        const double u1 = ((double)a + 1.0) * 2.3283064365386963e-10;
        const double u2 = (double)b * 2.3283064365386963e-10;
        const double rr = sqrt(-2.0 * log(u1));
        double sn, cs;
        sincospi(2.0 * u2, &sn, &cs);
        g0 = (T)(rr * cs);
        g1 = (T)(rr * sn);
    } else {
        const float u1 = ((float)a + 1.0f) * 2.3283064365386963e-10f;
        const float rr = sqrt_approx(fmaxf(0.0f, -1.38629436111989061883f * lg2_approx(u1)));   // -2 ln u1
        float sn, cs;
        __sincosf((float)b * 1.46291807926715968e-09f, &sn, &cs);   // 2 pi b 2^-32
        g0 = (T)(rr * cs);
        g1 = (T)(rr * sn);
    }
}

// The same pair scaled by 1/sqrt 2 (the Hermitian split of a complex mode):
// sqrt(-2 ln u1)/sqrt 2 = sqrt(-ln u1), folded into the radius.
__device__ __forceinline__ void box_muller_half(uint32_t a, uint32_t b, float &g0, float &g1) {
    const float u1 = ((float)a + 1.0f) * 2.3283064365386963e-10f;
    const float rr = sqrt_approx(fmaxf(0.0f, -0.69314718055994530942f * lg2_approx(u1)));   // -ln u1
    float sn, cs;
    __sincosf((float)b * 1.46291807926715968e-09f, &sn, &cs);
    g0 = rr * cs;
    g1 = rr * sn;
}

// Philox draw for a canonical mode (c0, c1, c2): the slowest axis (z in 3-D,
// y in 2-D) is folded in half; the lower half takes outputs 0,1, the upper 2,3.
template <bool ROLLED = true>
__device__ __forceinline__ uint4 noise_draw(const KSpace &ks, unsigned long long seed, unsigned long long stream,
                                            int c0, int c1, int c2, bool &upper) {
    // the counter is below n0 n1 n2 / 2, which fits in 32 bits for every
    // supported grid (at most 2^27 cells), so its upper word is 0
    uint32_t ctr;
    if (ks.n2 > 1) {
        upper = 2 * c2 >= ks.n2;
        const int f2 = upper ? c2 - ks.n2 / 2 : c2;
        ctr = ((uint32_t)f2 * (uint32_t)ks.n1 + (uint32_t)c1) * (uint32_t)ks.n0 + (uint32_t)c0;
    } else {
        upper = 2 * c1 >= ks.n1;
        const int f1 = upper ? c1 - ks.n1 / 2 : c1;
        ctr = (uint32_t)f1 * (uint32_t)ks.n0 + (uint32_t)c0;
    }
    return philox4x32_10<ROLLED>(make_uint4(ctr, 0u, (uint32_t)stream, (uint32_t)(stream >> 32)),
                                 make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
}

template <typename T> __device__ __forceinline__ T noise_amp_of(const KSpace &ks, T k2) {
    if constexpr (sizeof(T) == 4) return ks.f_noise_scale * sqrt_approx(k2);
    else return (T)ks.noise_scale * sqrt(k2);
}

// conserved noise xi_k = amp sqrt(cells) |k| g_k at full-grid mode (i0,i1,i2),
// i0 in [0, n0/2]; Hermitian pairing as the oracle defines it
template <typename T>
__device__ __forceinline__ cplx<T> noise_at(const KSpace &ks, unsigned long long seed, unsigned long long stream, int i0,
                                            int i1, int i2, T k2) {
    const int j1 = (ks.n1 - i1) % ks.n1, j2 = (ks.n2 - i2) % ks.n2;
    const bool edge = (i0 == 0) || (2 * i0 == ks.n0);
    const bool selfc = edge && j1 == i1 && j2 == i2;
    bool canon = true;
    if (edge) canon = (long long)i2 * ks.n1 + i1 <= (long long)j2 * ks.n1 + j1;
    bool upper;
    const uint4 o =
        canon ? noise_draw(ks, seed, stream, i0, i1, i2, upper) : noise_draw(ks, seed, stream, i0, j1, j2, upper);
    T g0, g1;
    box_muller<T>(upper ? o.z : o.x, upper ? o.w : o.y, g0, g1);
    const T amp = noise_amp_of<T>(ks, k2);
    if (selfc) return mk<T>(amp * g0, (T)0);
    const T h = (T)0.70710678118654752440;
    return mk<T>(amp * g0 * h, (canon ? amp : -amp) * g1 * h);
}

// Unit-amplitude noise of two interior modes (0 < i0 < n0/2) whose slow
// coordinates are s and s + n_slow/2: one Philox call, both halves of its
// output, each complex Gaussian scaled by 1/sqrt 2 (the mode amplitude
// noise_amp_of(k^2) multiplies it where the coefficients are at hand).
template <typename T>
__device__ __forceinline__ void noise_pair_unit(const KSpace &ks, unsigned long long seed, unsigned long long stream,
                                                int i0, int i1, int i2, cplx<T> &ga, cplx<T> &gb) {
    bool upper;
    const uint4 o = noise_draw<false>(ks, seed, stream, i0, i1, i2, upper);
    if constexpr (sizeof(T) == 4) {
        float g0, g1, g2, g3;
        box_muller_half(o.x, o.y, g0, g1);
        box_muller_half(o.z, o.w, g2, g3);
        ga = mk<T>(g0, g1);
        gb = mk<T>(g2, g3);
    } else {
        T g0, g1, g2, g3;
        box_muller<T>(o.x, o.y, g0, g1);
        box_muller<T>(o.z, o.w, g2, g3);
        const T h = (T)0.70710678118654752440;
        ga = mk<T>(h * g0, h * g1);
        gb = mk<T>(h * g2, h * g3);
    }
}

// ---------------------------------------------------------------------------
// Pencil pass: along the last axis (z in 3-D, y in 2-D), fused
//   forward FFT of S (state) and W (nonlinear term), the semi-implicit update,
//   k-space diagnostics, inverse FFT of S.
// 3-D: block (x = column tile, y = pair index p in [0, n1/2]) handles rows
//   y1 = p and y2 = (n1 - p) % n1 of every z.  2-D: one group, y = pencil.
// ---------------------------------------------------------------------------
struct PenArgs {
    void *S;
    const void *W;
    void *Shat;          // kept pencil-axis spectrum of S (null: transform S each step)
    long long es;        // pencil element stride (complex)
    long long gstride;   // stride of the paired axis (3-D: L0), 0 in 2-D
    int three_d;
    int L0;              // packed row length n0/2
    double scale;        // folds the pencil-axis inverse normalisation
    int update;          // 0: diagnostics only (no update, no store)
    int want_red;
    double *partials;
    int pin;             // overwrite the k = 0 mode with pin_value (unscaled)
    double pin_value;
    const double *pin_values;   // per batched instance (null: pin_value)
    long long zstride;   // complex elements between batched instances
    int nz;              // batched instances (0 or 1: one field)
};
__device__ __forceinline__ double pin_of(const PenArgs &a) {
    return a.pin_values ? a.pin_values[blockIdx.z] : a.pin_value;
}

template <typename T, int L, int NG>
__global__ void __launch_bounds__(PenShape<T, L, NG>::THREADS)
pencil_kernel(PenArgs args, KSpace ks, const cplx<T> *__restrict__ twL) {
    const Inst in = inst_of<T>(ks);
    using S = PenShape<T, L, NG>;
    constexpr int TX = S::TX, TPL = S::TPL;
    constexpr int TILE = L * TX;
    constexpr int NT = 2 * NG;                      // tiles: [array][group]
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *stw = reinterpret_cast<cplx<T> *>(smem_raw);
    cplx<T> *tiles = stw + L;                        // [array 0..1][group 0..NG-1][L][TX]
    double *sred = reinterpret_cast<double *>(tiles + NT * TILE);

    const int tid = threadIdx.x;
    for (int i = tid; i < L; i += S::THREADS)
        if (XG(&twL[i], 331) && XS(&stw[i], 332)) stw[i] = twL[i];
    pdl_wait();

    const int p = blockIdx.y;
    int yg[2];
    yg[0] = p;
    yg[1] = (NG == 2) ? (ks.n1 - p) % ks.n1 : p;
    const int G = (NG == 2 && yg[1] != yg[0]) ? 2 : 1;
    const int kx0 = blockIdx.x * TX;
    cplx<T> *gS = reinterpret_cast<cplx<T> *>(args.S) + (long long)blockIdx.z * args.zstride;
    const cplx<T> *gW = reinterpret_cast<const cplx<T> *>(args.W) + (long long)blockIdx.z * args.zstride;

    // load
    {
        const int c = tid % TX, rest = tid / TX;   // rest in [0, NT TPL)
        if (kx0 + c < args.L0)
            for (int idx = rest; idx < 2 * G * L; idx += NT * TPL) {
                const int a = idx / (G * L), g = (idx / L) % G, e = idx % L;
                const long long off = (long long)yg[g] * args.gstride + kx0 + c + (long long)e * args.es;
                if (XS(&tiles[(a * NG + g) * TILE + e * TX + c], 333) && XG(&gS[off], 334) && XG(&gW[off], 335))
                    tiles[(a * NG + g) * TILE + e * TX + c] = (a == 0) ? gS[off] : gW[off];
            }
    }
    __syncthreads();
    // forward FFT of all (array, group, column) lines
    {
        const int c = tid % TX, t = (tid / TX) % TPL, ag = tid / (TX * TPL);
        line_fft<T, L, -1, TPL, TX>(tiles + ag * TILE + c, t, stw);
    }

    // update: every thread handles modes (g, kz, c) in group-major order
    double v[NQ_PEN] = {0.0, 0.0};
    constexpr int PER = cdiv(NG * TILE, S::THREADS);
    cplx<T> res[PER];
    const T sc = (T)args.scale;
    const int nh = args.L0;   // n0/2
#pragma unroll
    for (int q = 0; q < PER; q++) {
        const int idx = tid + q * S::THREADS;
        if (idx >= G * TILE) continue;
        const int g = idx / TILE, kz = (idx / TX) % L, c = idx % TX;
        const int slot = kx0 + c;
        if (slot >= args.L0) continue;
        const int i1 = args.three_d ? yg[g] : kz;
        const int i2 = args.three_d ? kz : 0;
        if (!XS(&tiles[(1 * NG + g) * TILE + kz * TX + c], 336)) continue;
        const cplx<T> xs = tiles[(0 * NG + g) * TILE + kz * TX + c];
        const cplx<T> xw = tiles[(1 * NG + g) * TILE + kz * TX + c];
        cplx<T> out;
        if (slot != 0) {
            Coef<T> cf = kcoef<T>(ks, in.table, slot, i1, i2);
            cplx<T> num = xs;
            if (ks.noise_on) num = cadd(num, noise_at<T>(ks, in.seed, in.nstream, slot, i1, i2, cf.k2));
            cplx<T> xn = mk<T>(cf.A * num.x + cf.B * xw.x, cf.A * num.y + cf.B * xw.y);
            if (args.want_red) {
                const double xr = xs.x, xi = xs.y;
                const double k2 = cf.k2, c2 = cf.c2;
                v[0] += 2.0 * c2 * (xr * xr + xi * xi);
                const double rr = ((double)xn.x - xr) / ks.dt + ks.Mo_res * k2 * ((1.0 - c2) * xr + (double)xw.x);
                const double ri = ((double)xn.y - xi) / ks.dt + ks.Mo_res * k2 * ((1.0 - c2) * xi + (double)xw.y);
                v[1] += 2.0 * (rr * rr + ri * ri);
            }
            out = cscale(xn, sc);
        } else {
            // slot 0: separate the kx = 0 and kx = n0/2 planes with the mirror mode
            const int gm = (G == 2) ? 1 - g : g;
            const int kzm = (L - kz) % L;
            const cplx<T> ps = XS(&tiles[(0 * NG + gm) * TILE + kzm * TX], 337) ? tiles[(0 * NG + gm) * TILE + kzm * TX]
                                                                                : mk<T>((T)0, (T)0);
            const cplx<T> pw = XS(&tiles[(1 * NG + gm) * TILE + kzm * TX], 338) ? tiles[(1 * NG + gm) * TILE + kzm * TX]
                                                                                : mk<T>((T)0, (T)0);
            const T h = (T)0.5;
            // X0 = (P + conj Pm)/2, XN = (P - conj Pm)/(2i) = -i (P - conj Pm)/2
            const cplx<T> s0 = cscale(cadd(xs, cconj(ps)), h), sN = cscale(cmuli<-1>(csub(xs, cconj(ps))), h);
            const cplx<T> w0 = cscale(cadd(xw, cconj(pw)), h), wN = cscale(cmuli<-1>(csub(xw, cconj(pw))), h);
            const Coef<T> c0 = kcoef<T>(ks, in.table, 0, i1, i2), cN = kcoef<T>(ks, in.table, nh, i1, i2);
            cplx<T> num0 = s0, numN = sN;
            if (ks.noise_on) {
                num0 = cadd(num0, noise_at<T>(ks, in.seed, in.nstream, 0, i1, i2, c0.k2));
                numN = cadd(numN, noise_at<T>(ks, in.seed, in.nstream, nh, i1, i2, cN.k2));
            }
            cplx<T> x0n = mk<T>(c0.A * num0.x + c0.B * w0.x, c0.A * num0.y + c0.B * w0.y);
            cplx<T> xNn = mk<T>(cN.A * numN.x + cN.B * wN.x, cN.A * numN.y + cN.B * wN.y);
            if (args.pin && i1 == 0 && i2 == 0) x0n = mk<T>((T)pin_of(args), (T)0);
            if (args.want_red) {
                const double k20 = c0.k2, c20 = c0.c2, k2N = cN.k2, c2N = cN.c2;
                v[0] += c20 * ((double)s0.x * s0.x + (double)s0.y * s0.y);
                v[0] += c2N * ((double)sN.x * sN.x + (double)sN.y * sN.y);
                double rr = ((double)x0n.x - s0.x) / ks.dt + ks.Mo_res * k20 * ((1.0 - c20) * s0.x + (double)w0.x);
                double ri = ((double)x0n.y - s0.y) / ks.dt + ks.Mo_res * k20 * ((1.0 - c20) * s0.y + (double)w0.y);
                v[1] += rr * rr + ri * ri;
                rr = ((double)xNn.x - sN.x) / ks.dt + ks.Mo_res * k2N * ((1.0 - c2N) * sN.x + (double)wN.x);
                ri = ((double)xNn.y - sN.y) / ks.dt + ks.Mo_res * k2N * ((1.0 - c2N) * sN.y + (double)wN.y);
                v[1] += rr * rr + ri * ri;
            }
            // repack P = X0 + i XN
            out = cscale(cadd(x0n, cmuli<1>(xNn)), sc);
        }
        res[q] = out;
    }
    if (args.want_red)
        block_reduce_store<NQ_PEN>(v, args.partials + block_slot() * NQ_PEN, sred);
    if (!args.update) return;
    __syncthreads();
#pragma unroll
    for (int q = 0; q < PER; q++) {
        const int idx = tid + q * S::THREADS;
        if (idx >= G * TILE) continue;
        const int g = idx / TILE, kz = (idx / TX) % L, c = idx % TX;
        if (kx0 + c >= args.L0) continue;
        if (XS(&tiles[(0 * NG + g) * TILE + kz * TX + c], 339)) tiles[(0 * NG + g) * TILE + kz * TX + c] = res[q];
    }
    __syncthreads();
    // inverse FFT of the state lines: NG TX lines, 2 TPL threads each
    {
        const int c = tid % TX, t = (tid / TX) % (2 * TPL), g = tid / (TX * 2 * TPL);
        line_fft<T, L, +1, 2 * TPL, TX>(tiles + g * TILE + c, t, stw);
    }
    {
        const int c = tid % TX, rest = tid / TX;
        if (kx0 + c < args.L0)
            for (int idx = rest; idx < G * L; idx += NT * TPL) {
                const int g = idx / L, e = idx % L;
                const long long off = (long long)yg[g] * args.gstride + kx0 + c + (long long)e * args.es;
                if (XG(&gS[off], 340) && XS(&tiles[g * TILE + e * TX + c], 341)) gS[off] = tiles[g * TILE + e * TX + c];
            }
    }
}

template <typename T, int L, int NG> constexpr size_t pen_smem_bytes() {
    using S = PenShape<T, L, NG>;
    return sizeof(cplx<T>) * (L + 2 * NG * L * S::TX) + sizeof(double) * 32 * NQ_PEN;
}

// ---------------------------------------------------------------------------
// Deterministic final reduction of per-block partials: out[q] = sum_b part[b][q]
// (one block; fixed order for a fixed partial count).
// ---------------------------------------------------------------------------
// Batched: block z reduces instance z's partials into out + z * ostride.
template <int NQ>
__global__ void __launch_bounds__(256) finalize_kernel(const double *__restrict__ part, long long nparts,
                                                       double *__restrict__ out, long long ostride) {
    __shared__ double sred[32 * NQ];
    pdl_wait();
    part += (size_t)blockIdx.z * nparts * NQ;
    out += (size_t)blockIdx.z * ostride;
    double v[NQ];
#pragma unroll
    for (int q = 0; q < NQ; q++) v[q] = 0.0;
    for (long long b = threadIdx.x; b < nparts; b += blockDim.x)
#pragma unroll
        for (int q = 0; q < NQ; q++) v[q] += XG(&part[b * NQ + q], 351) ? part[b * NQ + q] : 0.0;
    block_reduce_store<NQ>(v, out, sred);
}

// ---------------------------------------------------------------------------
// Staged API kernels (the reference's per-stage wrappers, FP64)
// ---------------------------------------------------------------------------
// power_functions.cu:34-53: out = in^p
template <typename T>
__global__ void power_kernel(const T *__restrict__ in, T *__restrict__ out, long long n, int p, int ref_compat) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = powi(in[i], p, ref_compat);
}

// scaling_step.cu:34-53: f *= s
template <typename T>
__global__ void scale_kernel(T *__restrict__ f, long long n, T s) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        f[i] *= s;
}

// element type conversion (upload to / download from the mixed state)
template <typename A, typename B>
__global__ void convert_kernel(const A *__restrict__ in, B *__restrict__ out, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = (B)in[i];
}

// FE_calc.cu:54-68 density, summed per block: sum ff
// Avg_calc: sum x (p2 == nullptr); squares (square = 1) for the residual RMS
template <typename T>
__global__ void __launch_bounds__(256) density_partials(const T *__restrict__ psi, const T *__restrict__ p2,
                                                        const T *__restrict__ p3, const T *__restrict__ p4,
                                                        const T *__restrict__ convl, long long n, double a, double b,
                                                        int square, int ref_compat, double *__restrict__ partials) {
    __shared__ double sred[32];
    double v[1] = {0.0};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        if (p2)
            v[0] += 0.5 * (double)p2[i] - (a / 3.0) * (double)p3[i] + (b / 4.0) * (double)p4[i] -
                    0.5 * (double)psi[i] * (double)convl[i];
        else if (square)
            v[0] += (double)powi(psi[i], 2, ref_compat);
        else
            v[0] += (double)psi[i];
    }
    block_reduce_store<1>(v, partials + blockIdx.x, sred);
}

enum { KOP_EULER = 0, KOP_CONVOLVE = 1, KOP_RESIDUAL = 2 };

// k-space pointwise op on packed spectra at full-grid mode (i0, i1, i2)
template <typename T, int OP>
__device__ __forceinline__ cplx<T> kop(const KSpace &ks, double a, double b, int i0, int i1, int i2, cplx<T> x1,
                                        cplx<T> x2, cplx<T> x3, cplx<T> x4) {
    const Coef<T> cf = kcoef<T>(ks, ks.table, i0, i1, i2);
    const T k2 = cf.k2, c2 = cf.c2, dt = (T)ks.dt, Mo = (T)ks.Mo;
    if (OP == KOP_EULER) {
        // euler_step.cu:50-59
        const T ca = (T)a * k2 * Mo * dt, cb = (T)b * k2 * dt * Mo;
        const T den = ((T)1 + k2 * dt * Mo * ((T)1 - (T)ks.eps) - k2 * Mo * dt * c2);
        return mk<T>((x1.x + ca * x2.x - cb * x3.x) / den, (x1.y + ca * x2.y - cb * x3.y) / den);
    } else if (OP == KOP_CONVOLVE) {
        return cscale(x1, c2);   // convolve_fields.cu:41-42
    } else {
        // sse_calculation.cu:133-140 with x1 = psi_kp1, x2 = psi_k, x3 = psi2_k, x4 = psi3_k
        const T Mr = (T)ks.Mo_res;
        const T d2r = -Mr * k2 * (x2.x - (T)a * x3.x + (T)b * x4.x - c2 * x2.x);
        const T d2i = -Mr * k2 * (x2.y - (T)a * x3.y + (T)b * x4.y - c2 * x2.y);
        return mk<T>((x1.x - x2.x) / dt - d2r, (x1.y - x2.y) / dt - d2i);
    }
}

template <typename T, int OP>
__global__ void kspace_kernel(KSpace ks, double a, double b, cplx<T> *__restrict__ out, const cplx<T> *x1,
                              const cplx<T> *x2, const cplx<T> *x3, const cplx<T> *x4) {
    const int L0 = ks.n0 / 2;
    const long long total = (long long)L0 * ks.n1 * ks.n2;
    const cplx<T> z = mk<T>((T)0, (T)0);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int slot = (int)(i % L0);
        const long long rest = i / L0;
        const int i1 = (int)(rest % ks.n1), i2 = (int)(rest / ks.n1);
        cplx<T> a1 = x1[i], a2 = x2 ? x2[i] : z, a3 = x3 ? x3[i] : z, a4 = x4 ? x4[i] : z;
        if (slot != 0) {
            out[i] = kop<T, OP>(ks, a, b, slot, i1, i2, a1, a2, a3, a4);
            continue;
        }
        const int j1 = (ks.n1 - i1) % ks.n1, j2 = (ks.n2 - i2) % ks.n2;
        const long long im = ((long long)j2 * ks.n1 + j1) * L0;
        const cplx<T> m1 = x1[im], m2 = x2 ? x2[im] : z, m3 = x3 ? x3[im] : z, m4 = x4 ? x4[im] : z;
        const T h = (T)0.5;
        auto lo = [&](cplx<T> p, cplx<T> q) { return cscale(cadd(p, cconj(q)), h); };
        auto hi = [&](cplx<T> p, cplx<T> q) { return cscale(cmuli<-1>(csub(p, cconj(q))), h); };
        cplx<T> r0 = kop<T, OP>(ks, a, b, 0, i1, i2, lo(a1, m1), lo(a2, m2), lo(a3, m3), lo(a4, m4));
        cplx<T> rN = kop<T, OP>(ks, a, b, ks.n0 / 2, i1, i2, hi(a1, m1), hi(a2, m2), hi(a3, m3), hi(a4, m4));
        out[i] = cadd(r0, cmuli<1>(rN));
    }
}

}  // namespace xpfc
