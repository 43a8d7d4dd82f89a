// fft_core.cuh -- complex arithmetic, register DFTs and the shared-memory
// Stockham line FFT used by every pass of the XPFC step (sm_103a).
//
// A "line" is one 1-D transform of compile-time length L held in shared
// memory with element stride ES (ES = 1 for rows, the tile width for column
// tiles).  TPL threads cooperate on a line; every thread of the block runs the
// same pass sequence, so passes are separated by __syncthreads().
//
// The Stockham autosort formulation (natural order in, natural order out):
//   for each radix R (NS = product of earlier radices):
//     butterfly j in [0, L/R): v[r] = x[j + r L/R] * W_{NS R}^{(j mod NS) r}
//     DFT_R(v);  y[(j/NS) NS R + (j mod NS) + r NS] = v[r]
// Twiddles come from a table W_L^k (k < L) computed in FP64 on the host and
// rounded to the working type.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace xpfc {

// Self-checking build (-DXPFC_CHECKED, a diagnostics build only): every
// global access of the step kernels is checked against the device buffers
// the library registered, every shared-memory access against the block's
// dynamic shared memory; an access outside them is skipped and the first one
// recorded (site, address, block, thread) for the host to read.
#ifdef XPFC_CHECKED
struct XRange {
    unsigned long long lo, hi;
};
static __device__ XRange g_xranges[64];
static __device__ int g_xnranges;
static __device__ unsigned long long g_xfault[4];
static __device__ __noinline__ bool xchk_fail(int site, unsigned long long a) {
    if (atomicAdd(&g_xfault[0], 1ull) == 0) {
        g_xfault[1] = (unsigned long long)site;
        g_xfault[2] = a;
        g_xfault[3] = ((unsigned long long)blockIdx.x << 32) | ((unsigned long long)blockIdx.y << 16) | threadIdx.x;
    }
    return false;
}
__device__ __forceinline__ bool xchk_g(const void *p, int bytes, int site) {
    const unsigned long long a = (unsigned long long)p;
    for (int i = 0; i < g_xnranges; i++)
        if (a >= g_xranges[i].lo && a + bytes <= g_xranges[i].hi) return true;
    return xchk_fail(site, a);
}
__device__ __forceinline__ bool xchk_s(const void *p, int bytes, int site) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned int dyn;
    asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn));
    const long long off = (const unsigned char *)p - smem_raw;
    if (off >= 0 && off + bytes <= (long long)dyn) return true;
    return xchk_fail(site, (unsigned long long)off);
}
#define XG(p, site) xchk_g((p), (int)sizeof(*(p)), (site))
#define XS(p, site) xchk_s((p), (int)sizeof(*(p)), (site))
#else
#define XG(p, site) true
#define XS(p, site) true
#endif

template <typename T> struct ctype;
template <> struct ctype<float> { using type = float2; };
template <> struct ctype<double> { using type = double2; };
template <typename T> using cplx = typename ctype<T>::type;

template <typename T> __device__ __forceinline__ cplx<T> mk(T x, T y) { cplx<T> r; r.x = x; r.y = y; return r; }
// FP32 complex values travel as one 64-bit register pair, so additions,
// subtractions and real scalings use Blackwell's packed f32x2 arithmetic
// (one instruction per complex operation instead of two).
__device__ __forceinline__ unsigned long long f2pack(float2 a) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
    return r;
}
__device__ __forceinline__ float2 f2unpack(unsigned long long r) {
    float2 a;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
    return a;
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) {
    unsigned long long d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2pack(a)), "l"(f2pack(b)));
    return f2unpack(d);
}
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
    unsigned long long d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2pack(a)), "l"(f2pack(b)));
    return f2unpack(d);
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
    return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__device__ __forceinline__ double2 cmulc(double2 a, double2 b) {
    return make_double2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) {
    unsigned long long d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2pack(a)), "l"(f2pack(make_float2(s, s))));
    return f2unpack(d);
}
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
// multiply by +i (s = +1) or -i (s = -1)
template <int S> __device__ __forceinline__ float2 cmuli(float2 a) {
    return S > 0 ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}
template <int S> __device__ __forceinline__ double2 cmuli(double2 a) {
    return S > 0 ? make_double2(-a.y, a.x) : make_double2(a.y, -a.x);
}
// twiddle multiply: forward (DIR=-1) uses w, inverse its conjugate
template <int DIR, typename C> __device__ __forceinline__ C twmul(C a, C w) {
    return DIR < 0 ? cmul(a, w) : cmulc(a, w);
}

// cos(pi k/8), sin(pi k/8) for k = 0..8, from the exact angles
__host__ __device__ constexpr double c16c(int k) {
    return k == 0 ? 1.0 : k == 1 ? 0.92387953251128675613 : k == 2 ? 0.70710678118654752440
         : k == 3 ? 0.38268343236508977173 : k == 4 ? 0.0 : k == 5 ? -0.38268343236508977173
         : k == 6 ? -0.70710678118654752440 : k == 7 ? -0.92387953251128675613 : -1.0;
}
__host__ __device__ constexpr double c16s(int k) { return c16c(k <= 4 ? 4 - k : k - 4) * (k <= 4 ? 1.0 : 1.0); }

// ---------------------------------------------------------------------------
// Register DFTs.  DIR = -1: X_k = sum x_n e^{-2 pi i nk/R}; DIR = +1: e^{+...}.
// ---------------------------------------------------------------------------
template <int DIR, typename C> __device__ __forceinline__ void dft2(C &a, C &b) {
    C t = a;
    a = cadd(t, b);
    b = csub(t, b);
}

template <int DIR, typename C> __device__ __forceinline__ void dft4(C &x0, C &x1, C &x2, C &x3) {
    C a = cadd(x0, x2), b = csub(x0, x2), c = cadd(x1, x3), d = csub(x1, x3);
    // forward: X1 = b - i d, X3 = b + i d
    C id = cmuli<DIR>(d);
    x0 = cadd(a, c);
    x2 = csub(a, c);
    x1 = cadd(b, id);
    x3 = csub(b, id);
}

template <int DIR, typename C, typename T> __device__ __forceinline__ C rot16(C a, int k) {
    // a * W16^k for the forward direction (W16 = e^{-2 pi i/16}), conjugate for inverse
    const T c = (T)c16c(k), s = (T)c16s(k);
    return DIR < 0 ? mk<T>(a.x * c + a.y * s, a.y * c - a.x * s) : mk<T>(a.x * c - a.y * s, a.y * c + a.x * s);
}

// a * W16^E with the exact special cases spelled out (IEEE arithmetic may
// not drop a multiplication by 0, so W16^0, ^4, ^8 and the sqrt(1/2) pairs
// ^2, ^6 get their own short forms); E in [0, 9]
template <int E, int DIR, typename T> __device__ __forceinline__ cplx<T> tw16c(cplx<T> a) {
    const T r = (T)0.70710678118654752440;
    if constexpr (E == 0) return a;
    else if constexpr (E == 4) return cmuli<DIR>(a);                     // forward: -i
    else if constexpr (E == 8) return mk<T>(-a.x, -a.y);
    else if constexpr (E == 2)                                           // forward: (1 - i)/sqrt 2
        return DIR < 0 ? mk<T>((a.x + a.y) * r, (a.y - a.x) * r) : mk<T>((a.x - a.y) * r, (a.y + a.x) * r);
    else if constexpr (E == 6)                                           // forward: -(1 + i)/sqrt 2
        return DIR < 0 ? mk<T>((a.y - a.x) * r, -(a.x + a.y) * r) : mk<T>(-(a.x + a.y) * r, (a.x - a.y) * r);
    else if constexpr (E == 9) {
        const cplx<T> q = rot16<DIR, cplx<T>, T>(a, 1);
        return mk<T>(-q.x, -q.y);
    } else
        return rot16<DIR, cplx<T>, T>(a, E);
}

template <int DIR, typename T> __device__ __forceinline__ void dft8(cplx<T> *v) {
    // 8 = 2 x 4 (decimation in time): E = DFT4(even), O = DFT4(odd), X_k = E_k + W8^k O_k
    dft4<DIR>(v[0], v[2], v[4], v[6]);
    dft4<DIR>(v[1], v[3], v[5], v[7]);
    cplx<T> o1 = tw16c<2, DIR, T>(v[3]);
    cplx<T> o2 = cmuli<DIR>(v[5]);
    cplx<T> o3 = tw16c<6, DIR, T>(v[7]);
    cplx<T> e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    v[0] = cadd(e0, v[1]);
    v[4] = csub(e0, v[1]);
    v[1] = cadd(e1, o1);
    v[5] = csub(e1, o1);
    v[2] = cadd(e2, o2);
    v[6] = csub(e2, o2);
    v[3] = cadd(e3, o3);
    v[7] = csub(e3, o3);
}

template <int DIR, typename T, int N1> __device__ __forceinline__ void dft16_col(cplx<T> *v, cplx<T> *y) {
    cplx<T> a = v[N1], b = v[N1 + 4], c = v[N1 + 8], d = v[N1 + 12];
    dft4<DIR>(a, b, c, d);
    y[N1 * 4 + 0] = a;
    y[N1 * 4 + 1] = tw16c<N1, DIR, T>(b);
    y[N1 * 4 + 2] = tw16c<2 * N1, DIR, T>(c);
    y[N1 * 4 + 3] = tw16c<3 * N1, DIR, T>(d);
}

template <int DIR, typename T> __device__ __forceinline__ void dft16(cplx<T> *v) {
    // 16 = 4 x 4 with n = n1 + 4 n2, k = k2 + 4 k1:
    // Y[n1][k2] = DFT4_n2(x[n1 + 4 n2]) * W16^{n1 k2};  X[k2 + 4 k1] = DFT4_n1(Y[n1][k2])
    cplx<T> y[16];
    dft16_col<DIR, T, 0>(v, y);
    dft16_col<DIR, T, 1>(v, y);
    dft16_col<DIR, T, 2>(v, y);
    dft16_col<DIR, T, 3>(v, y);
#pragma unroll
    for (int k2 = 0; k2 < 4; k2++) {
        cplx<T> a = y[0 * 4 + k2], b = y[1 * 4 + k2], c = y[2 * 4 + k2], d = y[3 * 4 + k2];
        dft4<DIR>(a, b, c, d);
        v[k2] = a;
        v[k2 + 4] = b;
        v[k2 + 8] = c;
        v[k2 + 12] = d;
    }
}

template <int DIR, typename T> __device__ __forceinline__ void dft3(cplx<T> *v) {
    const T h = (T)0.86602540378443864676;  // sqrt(3)/2
    cplx<T> s = cadd(v[1], v[2]);
    cplx<T> d = csub(v[1], v[2]);
    cplx<T> m = mk<T>(v[0].x - (T)0.5 * s.x, v[0].y - (T)0.5 * s.y);
    // forward: X1 = m - i h d, X2 = m + i h d
    cplx<T> ihd = cmuli<DIR>(cscale(d, h));
    v[0] = cadd(v[0], s);
    v[1] = cadd(m, ihd);
    v[2] = csub(m, ihd);
}

// cos(2 pi m/24) from the exact angles (m any integer)
__host__ __device__ constexpr double c24(int m) {
    m = ((m % 24) + 24) % 24;
    if (m > 12) m = 24 - m;
    if (m > 6) return -c24(12 - m);
    return m == 0 ? 1.0 : m == 1 ? 0.96592582628906828675 : m == 2 ? 0.86602540378443864676
         : m == 3 ? 0.70710678118654752440 : m == 4 ? 0.5 : m == 5 ? 0.25881904510252076235 : 0.0;
}
// cos(2 pi m/32) from the exact angles (m any integer)
__host__ __device__ constexpr double c32(int m) {
    m = ((m % 32) + 32) % 32;
    if (m > 16) m = 32 - m;
    if (m > 8) return -c32(16 - m);
    return m == 0 ? 1.0 : m == 1 ? 0.98078528040323044913 : m == 2 ? 0.92387953251128675613
         : m == 3 ? 0.83146961230254523708 : m == 4 ? 0.70710678118654752440 : m == 5 ? 0.55557023301960222474
         : m == 6 ? 0.38268343236508977173 : m == 7 ? 0.19509032201612826785 : 0.0;
}
// cos and sin of 2 pi m/N for N dividing 24 or 32
__host__ __device__ constexpr double cos2pi(int N, int m) { return 24 % N == 0 ? c24(m * (24 / N)) : c32(m * (32 / N)); }
__host__ __device__ constexpr double sin2pi(int N, int m) {
    return 24 % N == 0 ? c24(6 - m * (24 / N)) : c32(8 - m * (32 / N));
}

// a * W_N^m (W_N = e^{-2 pi i/N} forward, its conjugate inverse) for N
// dividing 24 or 32; the quarter turns are exact
template <int N, int DIR, typename T> __device__ __forceinline__ cplx<T> twc(cplx<T> a, int m) {
    const int q = ((m % N) + N) % N;
    if (q == 0) return a;
    if (4 * q == N) return cmuli<DIR>(a);
    if (2 * q == N) return mk<T>(-a.x, -a.y);
    if (4 * q == 3 * N) return cmuli<-DIR>(a);
    const T c = (T)cos2pi(N, q), sn = (T)sin2pi(N, q);
    return DIR < 0 ? mk<T>(a.x * c + a.y * sn, a.y * c - a.x * sn) : mk<T>(a.x * c - a.y * sn, a.y * c + a.x * sn);
}

template <int R, int DIR, typename T> __device__ __forceinline__ void dftR(cplx<T> *v);

// DFT of length R1 R2 (dividing 24 or 32) from R2-point DFTs, twiddles W^{n1 k2} and
// R1-point DFTs: n = n1 + R1 n2, k = k2 + R2 k1.
template <int R1, int R2, int DIR, typename T> __device__ __forceinline__ void dft_mixed(cplx<T> *v) {
    constexpr int N = R1 * R2;
    cplx<T> y[N];
#pragma unroll
    for (int n1 = 0; n1 < R1; n1++) {
        cplx<T> c[R2];
#pragma unroll
        for (int n2 = 0; n2 < R2; n2++) c[n2] = v[n1 + R1 * n2];
        dftR<R2, DIR, T>(c);
#pragma unroll
        for (int k2 = 0; k2 < R2; k2++) y[n1 * R2 + k2] = twc<N, DIR, T>(c[k2], n1 * k2);
    }
#pragma unroll
    for (int k2 = 0; k2 < R2; k2++) {
        cplx<T> c[R1];
#pragma unroll
        for (int n1 = 0; n1 < R1; n1++) c[n1] = y[n1 * R2 + k2];
        dftR<R1, DIR, T>(c);
#pragma unroll
        for (int k1 = 0; k1 < R1; k1++) v[k2 + R2 * k1] = c[k1];
    }
}

// 32 = 2 x 16 by decimation in frequency, in place: X[2k] = DFT16(x[n] +
// x[n+16]), X[2k+1] = DFT16((x[n] - x[n+16]) W32^n); the final interleave is
// a renaming of registers
template <int DIR, typename T> __device__ __forceinline__ void dft32(cplx<T> *v) {
#pragma unroll
    for (int n = 0; n < 16; n++) {
        const cplx<T> a = v[n], b = v[n + 16];
        v[n] = cadd(a, b);
        v[n + 16] = twc<32, DIR, T>(csub(a, b), n);
    }
    dft16<DIR, T>(v);
    dft16<DIR, T>(v + 16);
    cplx<T> u[32];
#pragma unroll
    for (int k = 0; k < 16; k++) {
        u[2 * k] = v[k];
        u[2 * k + 1] = v[16 + k];
    }
#pragma unroll
    for (int k = 0; k < 32; k++) v[k] = u[k];
}

template <int R, int DIR, typename T> __device__ __forceinline__ void dftR(cplx<T> *v) {
    if constexpr (R == 2) dft2<DIR>(v[0], v[1]);
    else if constexpr (R == 3) dft3<DIR, T>(v);
    else if constexpr (R == 4) dft4<DIR>(v[0], v[1], v[2], v[3]);
    else if constexpr (R == 8) dft8<DIR, T>(v);
    else if constexpr (R == 12) dft_mixed<3, 4, DIR, T>(v);
    else if constexpr (R == 16) dft16<DIR, T>(v);
    else if constexpr (R == 24) dft_mixed<3, 8, DIR, T>(v);
    else if constexpr (R == 32) dft32<DIR, T>(v);
    else static_assert(R == 2, "unsupported radix");
}

// ---------------------------------------------------------------------------
// Radix plan: 3s first, then 16s, finishing the power of two with 8/4/2
// (2^(4q+1) uses 8*4 for its last 16*2).
// ---------------------------------------------------------------------------
__host__ __device__ constexpr int radix_at(int L, int p) {
    // radix of pass p for length L
    int rem = L;
    for (int q = 0;; q++) {
        int r = 1;
        if (rem % 3 == 0) r = 3;
        else if (rem == 32) r = 8;
        else if (rem % 16 == 0) r = 16;
        else if (rem % 8 == 0) r = 8;
        else if (rem % 4 == 0) r = 4;
        else if (rem % 2 == 0) r = 2;
        else r = 1;
        if (q == p) return r;
        if (r == 1) return 1;
        rem /= r;
    }
}
__host__ __device__ constexpr int num_passes(int L) {
    int n = 0;
    while (radix_at(L, n) != 1) n++;
    return n;
}
__host__ __device__ constexpr int ns_at(int L, int p) {
    int ns = 1;
    for (int q = 0; q < p; q++) ns *= radix_at(L, q);
    return ns;
}
__host__ __device__ constexpr int cdiv(int a, int b) { return (a + b - 1) / b; }
// registers (complex values) a thread needs for any pass of length L with TPL threads
__host__ __device__ constexpr int max_regs(int L, int TPL) {
    int m = 0;
    for (int p = 0; p < num_passes(L); p++) {
        int R = radix_at(L, p);
        int v = cdiv(L / R, TPL) * R;
        m = v > m ? v : m;
    }
    return m;
}

// Shared-memory index of element e of a line.  ES = ROW_LAYOUT: a row of
// the row pass, with a skew of one slot per 128 bytes so that stride-R
// Stockham writes hit distinct banks; ES >= 1: a column of a tile ES columns
// wide (a one-column tile is plain contiguous storage, without the skew).
constexpr int ROW_LAYOUT = 0;
template <typename T, int ES> struct LineIdx {
    static constexpr int SK = (sizeof(cplx<T>) == 8) ? 4 : 3;
    __device__ __forceinline__ static int at(int e) {
        if constexpr (ES == ROW_LAYOUT) return e + (e >> SK);
        else return e * ES;
    }
    __host__ __device__ static constexpr int span(int L) { return ES == ROW_LAYOUT ? L + (L >> SK) + 1 : L * ES; }
};

// One Stockham pass of radix R on every line of the block.
template <typename T, int L, int P, int DIR, int TPL, int ES>
__device__ __forceinline__ void stockham_pass(cplx<T> *line, int t, const cplx<T> *__restrict__ tw) {
    constexpr int R = radix_at(L, P);
    constexpr int NS = ns_at(L, P);
    constexpr int NB = L / R;
    constexpr int PER = cdiv(NB, TPL);
    constexpr int TWS = L / (NS * R);
    using I = LineIdx<T, ES>;
    cplx<T> v[PER][R];
#pragma unroll
    for (int b = 0; b < PER; b++) {
        const int j = t + b * TPL;
        if (PER * TPL == NB || j < NB) {
            const int k = j % NS;
#pragma unroll
            for (int r = 0; r < R; r++) {
                cplx<T> x = XS(&line[I::at(j + r * NB)], 101) ? line[I::at(j + r * NB)] : mk<T>((T)0, (T)0);
                if (NS > 1 && r > 0) x = twmul<DIR>(x, XS(&tw[k * r * TWS], 103) ? tw[k * r * TWS] : mk<T>((T)1, (T)0));
                v[b][r] = x;
            }
            dftR<R, DIR, T>(v[b]);
        }
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < PER; b++) {
        const int j = t + b * TPL;
        if (PER * TPL == NB || j < NB) {
            const int k = j % NS;
            const int d = (j / NS) * NS * R + k;
#pragma unroll
            for (int r = 0; r < R; r++)
                if (XS(&line[I::at(d + r * NS)], 102)) line[I::at(d + r * NS)] = v[b][r];
        }
    }
    __syncthreads();
}

template <typename T, int L, int P, int DIR, int TPL, int ES>
__device__ __forceinline__ void line_fft_from(cplx<T> *line, int t, const cplx<T> *__restrict__ tw) {
    if constexpr (P < num_passes(L)) {
        stockham_pass<T, L, P, DIR, TPL, ES>(line, t, tw);
        line_fft_from<T, L, P + 1, DIR, TPL, ES>(line, t, tw);
    }
}

// Full unnormalised L-point FFT of the line (natural order in and out).
// The caller must __syncthreads() before (data ready); returns synchronised.
template <typename T, int L, int DIR, int TPL, int ES>
__device__ __forceinline__ void line_fft(cplx<T> *line, int t, const cplx<T> *__restrict__ tw) {
    line_fft_from<T, L, 0, DIR, TPL, ES>(line, t, tw);
}

// ---------------------------------------------------------------------------
// FP64 block reduction (warp shuffles, then one value per warp in shared
// memory).  Deterministic for a fixed block size.
// ---------------------------------------------------------------------------
template <int NQ>
__device__ __forceinline__ void block_reduce_store(double (&v)[NQ], double *__restrict__ out, double *sred) {
#pragma unroll
    for (int q = 0; q < NQ; q++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_down_sync(0xffffffffu, v[q], o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = (blockDim.x + 31) >> 5;
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < NQ; q++) sred[warp * NQ + q] = v[q];
    __syncthreads();
    if (threadIdx.x < NQ) {
        double s = 0.0;
        for (int w = 0; w < nwarps; w++) s += sred[w * NQ + threadIdx.x];
        if (XG(&out[threadIdx.x], 104)) out[threadIdx.x] = s;
    }
}

// ---------------------------------------------------------------------------
// Asynchronous global -> shared copies (cp.async): they land without holding
// registers; a block's threads see them after each copying thread's
// cp_async_wait_all and a barrier.  16 bytes (L2 only) or 8 (through L1).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cp_async16(void *sdst, const void *gsrc) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((unsigned)__cvta_generic_to_shared(sdst)),
                 "l"(gsrc)
                 : "memory");
}
// 8-byte copy (cp.async through L1: the size that .cg does not take)
__device__ __forceinline__ void cp_async8(void *sdst, const void *gsrc) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"((unsigned)__cvta_generic_to_shared(sdst)),
                 "l"(gsrc)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) and Box-Muller.
// ---------------------------------------------------------------------------
// ROLLED keeps the round loop as a loop: code on rare paths stays small
// (the instruction cache is the limit of the pencil pass).
template <bool ROLLED = true>
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll(ROLLED ? 1 : 10)
    for (int r = 0; r < 10; r++) {
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += 0x9E3779B9u;
        k.y += 0xBB67AE85u;
    }
    return c;
}

}  // namespace xpfc
