// xpfc_tma.cuh -- the k-space pencil pass of 3-D FP32 grids as a persistent
// kernel whose input tiles are staged in shared memory by the tensor-memory
// accelerator (TMA, cp.async.bulk.tensor).
//
// Work unit (a "tile"): TX adjacent kx columns of the two mirror rows
// y1 = p and y2 = (n1 - p) % n1, every kz, of S and W (four boxes of
// [N][TX] complex values, 64 KB at N = 256) -- the same unit a block of
// pencil_kernel_reg handles.  Each CTA walks the tiles
// blockIdx.x, blockIdx.x + gridDim.x, ...; one stage in shared memory holds
// a tile.  Thread 0 issues the four box loads of the next tile as soon as the
// block has copied the current tile into registers, so the next tile's HBM
// reads overlap the current tile's transforms, update and stores (the
// register pencil waits on its global loads: long_scoreboard was its largest
// stall).  Per mode the arithmetic, the transforms and the order of every
// sum are those of pencil_kernel_reg, so both give the same bits.
//
// Waits on the stage's mbarrier are bounded (about one second of
// %globaltimer); a block that gives up records XPFC_DEV_ETIMEDOUT in
// args.err and returns with its whole block (the give-up is voted with
// __syncthreads_or, so no thread is left at a barrier).
#pragma once
#include <cuda.h>

#include "xpfc_regkernels.cuh"

namespace xpfc {

constexpr int XPFC_DEV_ETIMEDOUT = 1;

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    // make the initialised barrier visible to the async proxy (the TMA unit)
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t phase) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(phase)
        : "memory");
    return ok != 0;
}

// true once the barrier's phase `phase` completed; false after ~1 s
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t phase) {
    const uint32_t b = smem_addr(bar);
    if (mbar_try_wait(b, phase)) return true;
    const unsigned long long t0 = global_ns();
    for (;;) {
        if (mbar_try_wait(b, phase)) return true;
        if (global_ns() - t0 > 1000000000ull) return false;
    }
}

// one 3-D box of a tiled tensor map into shared memory, completing on bar
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(smem_addr(dst)), "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z),
        "r"(smem_addr(bar))
        : "memory");
}

// Lengths with a staged pencil: FP32 register plans of at most 16 values per
// thread (64, 128, 256) whose whole pencil fits one box (N <= 256).
template <typename T, int N> constexpr bool tma_pen_ok() {
    return sizeof(T) == 4 && RP<N>::ok && !RP<N>::three && RP<N>::P <= 16 && N <= 256;
}

template <typename T, int N> struct TPenShape {
    using R = RPenShape<T, N, 2>;
    static constexpr int TX = R::TX, Q = R::Q, P = R::P, THREADS = R::THREADS, LINES = R::LINES, LP = R::LP;
    static constexpr int BOXC = N * TX;                                    // complex values per box
    static constexpr size_t BOX = sizeof(cplx<T>) * BOXC;                  // 16 KB at N = 256
    // one transpose scratch, used by S and W in turn; it also holds the
    // slot-0 areas (published S and W pencils of both groups and the results)
    // and the noise staging
    static constexpr int SCRC0 = LINES * LP, SCRC1 = 6 * N, SCRC2 = P * THREADS;
    static constexpr int SCRC = SCRC0 > SCRC1 ? (SCRC0 > SCRC2 ? SCRC0 : SCRC2) : (SCRC1 > SCRC2 ? SCRC1 : SCRC2);
    // [barrier, padded to 128 B][stage: S g0, S g1, W g0, W g1][twiddles][scratch][block sums]
    static constexpr size_t OFF_STAGE = 128;
    static constexpr size_t OFF_TW = OFF_STAGE + 4 * BOX;
    static constexpr size_t OFF_SCR = OFF_TW + sizeof(cplx<T>) * N;
    static constexpr size_t OFF_RED = OFF_SCR + sizeof(cplx<T>) * SCRC;
    static constexpr size_t SMEM = OFF_RED + sizeof(double) * 32 * NQ_PEN + 128;   // + alignment slack
    static constexpr int MINB = R::MINB;
};

template <typename T, int N, bool RED>
__global__ void __launch_bounds__(TPenShape<T, N>::THREADS, TPenShape<T, N>::MINB)
pencil_kernel_tma(PenArgs args, KSpace ks, const cplx<T> *__restrict__ twN, const __grid_constant__ CUtensorMap mapS,
                  const __grid_constant__ CUtensorMap mapW, int nkx, int npairs, int ntiles, int *err) {
    using S = TPenShape<T, N>;
    constexpr int TX = S::TX, Q = S::Q, P = S::P;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // the TMA destination wants 128-byte alignment: align the carve-up base
    unsigned char *base = smem_raw + ((128 - (smem_addr(smem_raw) & 127)) & 127);
    uint64_t *bar = reinterpret_cast<uint64_t *>(base);
    cplx<T> *stage = reinterpret_cast<cplx<T> *>(base + S::OFF_STAGE);
    cplx<T> *stw = reinterpret_cast<cplx<T> *>(base + S::OFF_TW);
    cplx<T> *scr = reinterpret_cast<cplx<T> *>(base + S::OFF_SCR);
    double *sred = reinterpret_cast<double *>(base + S::OFF_RED);
    const int tid = threadIdx.x;
    for (int i = tid; i < N; i += S::THREADS) stw[i] = twN[i];
    if (tid == 0) mbar_init(bar, 1);
    __syncthreads();
    pdl_wait();

    const int n2 = ks.n2, n1 = ks.n1;
    // thread 0: the four (or, for a self-mirrored row, two) boxes of tile tt
    auto issue = [&](int tt) {
        const int kxb = tt % nkx, rest = tt / nkx;
        const int p = rest % npairs, z0 = (rest / npairs) * n2;
        const int y1 = p, y2 = (n1 - p) % n1;
        const int G = (y2 != y1) ? 2 : 1;
        // the box loads overwrite what the block read of the last tile with
        // ordinary loads (ordered before this thread by the block barrier)
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(bar, (uint32_t)(2 * G * S::BOX));
        const int x = 2 * kxb * TX;
        tma_load_3d(stage + 0 * S::BOXC, &mapS, x, y1, z0, bar);
        tma_load_3d(stage + 2 * S::BOXC, &mapW, x, y1, z0, bar);
        if (G == 2) {
            tma_load_3d(stage + 1 * S::BOXC, &mapS, x, y2, z0, bar);
            tma_load_3d(stage + 3 * S::BOXC, &mapW, x, y2, z0, bar);
        }
    };
    if (tid == 0 && (int)blockIdx.x < ntiles) issue(blockIdx.x);

    const int c = tid % TX, t = (tid / TX) % Q, g = tid / (TX * Q);
    const int ln = g * TX + c;
    const T sc = (T)args.scale;
    const int nh = args.L0;
    const cplx<T> zero = mk<T>((T)0, (T)0);
    uint32_t phase = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int kxb = tile % nkx, rest = tile / nkx;
        const int p = rest % npairs, inst = rest / npairs;
        const int y1 = p, y2 = (n1 - p) % n1;
        const int G = (y2 != y1) ? 2 : 1;
        const int yg = (g == 0) ? y1 : y2;
        const int kx0 = kxb * TX;
        const bool valid = (g < G) && (kx0 + c < args.L0);
        Inst in = inst_at<T>(ks, inst);
        in.pin = args.pin_values ? args.pin_values[inst] : args.pin_value;

        const bool ok = mbar_wait_bounded(bar, phase);
        phase ^= 1u;
        cplx<T> vs[P], vw[P];
        {
            const cplx<T> *bs = stage + g * S::BOXC + c, *bw = stage + (2 + g) * S::BOXC + c;
#pragma unroll
            for (int j = 0; j < P; j++) {
                vs[j] = valid ? bs[(t + Q * j) * TX] : zero;
                vw[j] = valid ? bw[(t + Q * j) * TX] : zero;
            }
        }
        // every thread holds its values (or gave up waiting): the stage is
        // free for the next tile
        if (__syncthreads_or(!ok)) {
            if (tid == 0) atomicExch(err, XPFC_DEV_ETIMEDOUT);
            return;
        }
        if (tid == 0 && tile + (int)gridDim.x < ntiles) issue(tile + gridDim.x);

        reg_fft<T, N, -1>(vw, t, scr + ln * S::LP, stw);
        reg_fft<T, N, -1>(vs, t, scr + ln * S::LP, stw);

        DSum<T, NQ_PEN> acc;
        // slot 0 (tiles holding kx' = 0): as pencil_kernel_reg, with the
        // published S and W pencils and the results in the scratch
        if (kx0 == 0) {
            cplx<T> *pubS = scr, *pubW = scr + 2 * N, *outS = scr + 4 * N;
            __syncthreads();
            if (c == 0 && g < G) {
#pragma unroll
                for (int j = 0; j < P; j++) {
                    pubS[g * N + t + Q * j] = vs[j];
                    pubW[g * N + t + Q * j] = vw[j];
                }
            }
            __syncthreads();
#pragma unroll 1
            for (int idx = tid; idx < G * N; idx += S::THREADS) {
                const int gg = idx / N, kz = idx % N;
                const int yy = (gg == 0) ? y1 : y2;
                const int gm = (G == 2) ? 1 - gg : gg;
                const int kzm = (N - kz) % N;
                const cplx<T> xs = pubS[gg * N + kz], xw = pubW[gg * N + kz];
                const cplx<T> ps = pubS[gm * N + kzm], pw = pubW[gm * N + kzm];
                const T h = (T)0.5;
                const cplx<T> s0 = cscale(cadd(xs, cconj(ps)), h), sN = cscale(cmuli<-1>(csub(xs, cconj(ps))), h);
                const cplx<T> w0 = cscale(cadd(xw, cconj(pw)), h), wN = cscale(cmuli<-1>(csub(xw, cconj(pw))), h);
                const cplx<T> x0 = update_mode<T>(ks, in, args, 0, yy, kz, s0, w0, acc, (T)1);
                const cplx<T> xN = update_mode<T>(ks, in, args, nh, yy, kz, sN, wN, acc, (T)1);
                outS[gg * N + kz] = cscale(cadd(x0, cmuli<1>(xN)), sc);
            }
            __syncthreads();
            if (c == 0 && g < G) {
#pragma unroll
                for (int j = 0; j < P; j++) vs[j] = outS[g * N + t + Q * j];
            }
        }
        // interior columns: the noise draws first, in a rolled loop, into the
        // scratch (each thread reads back only its own entries)
        const bool interior = valid && kx0 + c != 0;
        const int i0 = kx0 + c;
        cplx<T> *snoise = scr;
        if (ks.noise_on) {
            __syncthreads();   // the transforms and the slot-0 pass are done with the scratch
            if (interior) {
#pragma unroll 1
                for (int j = 0; j < P / 2; j++) {
                    cplx<T> ga, gb;
                    noise_pair_unit<T>(ks, in.seed, in.nstream, i0, yg, t + Q * j, ga, gb);
                    snoise[j * S::THREADS + tid] = ga;
                    snoise[(j + P / 2) * S::THREADS + tid] = gb;
                }
            }
        }
        if (interior) {
#pragma unroll
            for (int j = 0; j < P / 2; j++) {
                const int kza = t + Q * j, kzb = kza + N / 2;
                const Coef<T> ca = kcoef<T>(ks, in.table, i0, yg, kza), cb = kcoef<T>(ks, in.table, i0, yg, kzb);
                cplx<T> na = zero, nb = zero;
                if (ks.noise_on) {
                    na = cscale(snoise[j * S::THREADS + tid], noise_amp_of<T>(ks, ca.k2));
                    nb = cscale(snoise[(j + P / 2) * S::THREADS + tid], noise_amp_of<T>(ks, cb.k2));
                }
                vs[j] = cscale(update_coef<T, RED>(ks, ca, vs[j], vw[j], na, acc, (T)2), sc);
                vs[j + P / 2] = cscale(update_coef<T, RED>(ks, cb, vs[j + P / 2], vw[j + P / 2], nb, acc, (T)2), sc);
            }
        }
        if (RED) {
            double tot[NQ_PEN] = {acc.get(0), acc.get(1)};
            block_reduce_store<NQ_PEN>(tot, args.partials + (size_t)tile * NQ_PEN, sred);
        }
        if (!args.update) continue;
        // as in pencil_kernel_reg: twiddles and store addresses from opaque
        // copies of their bases, so that the forward transform's are not kept
        // live through the update
        reg_fft<T, N, +1>(vs, t, scr + ln * S::LP, opaque(stw));
        if (valid) {
            cplx<T> *o = opaque(reinterpret_cast<cplx<T> *>(args.S)) + (long long)inst * args.zstride +
                         (long long)yg * args.gstride + kx0 + c + (long long)t * args.es;
            const long long step = (long long)Q * args.es;
#pragma unroll
            for (int j = 0; j < P; j++, o += step) *o = vs[j];
        }
    }
}

}  // namespace xpfc
