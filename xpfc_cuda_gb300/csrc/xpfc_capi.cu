// xpfc_capi.cu -- the C ABI of libxpfc (include/xpfc.h): context, fused
// step driver and the staged per-stage entry points.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <vector>

#include "../../include/xpfc.h"
#include "xpfc_host.h"
#include "xpfc_launch.h"

using namespace xpfc;

#ifdef XPFC_CHECKED
// Diagnostics build: every device allocation of the library is registered
// with the launcher units' checker tables.
#define XPFC_XDECL(t, p)                                                 \
    extern "C" int xpfc_xcheck_set_##t##_p##p(const void *ranges, int n); \
    extern "C" int xpfc_xcheck_get_##t##_p##p(unsigned long long *out);
XPFC_XDECL(f32, 1)
XPFC_XDECL(f32, 2)
XPFC_XDECL(f64, 1)
XPFC_XDECL(f64, 2)
static std::vector<XRange> g_host_ranges;
static void xcheck_publish() {
    const int n = (int)std::min<size_t>(g_host_ranges.size(), 64);
    xpfc_xcheck_set_f32_p1(g_host_ranges.data(), n);
    xpfc_xcheck_set_f32_p2(g_host_ranges.data(), n);
    xpfc_xcheck_set_f64_p1(g_host_ranges.data(), n);
    xpfc_xcheck_set_f64_p2(g_host_ranges.data(), n);
}
static cudaError_t xchk_malloc(void **p, size_t b) {
    cudaError_t e = ::cudaMalloc(p, b);
    if (e == cudaSuccess) {
        g_host_ranges.push_back({(unsigned long long)*p, (unsigned long long)*p + b});
        xcheck_publish();
    }
    return e;
}
static cudaError_t xchk_malloc_async(void **p, size_t b, cudaStream_t s) {
    cudaError_t e = ::cudaMallocAsync(p, b, s);
    if (e == cudaSuccess) {
        cudaStreamSynchronize(s);
        g_host_ranges.push_back({(unsigned long long)*p, (unsigned long long)*p + b});
        xcheck_publish();
    }
    return e;
}
static cudaError_t xchk_free(void *p) {
    for (size_t i = 0; i < g_host_ranges.size(); i++)
        if (g_host_ranges[i].lo == (unsigned long long)p) {
            g_host_ranges.erase(g_host_ranges.begin() + i);
            break;
        }
    cudaDeviceSynchronize();
    xcheck_publish();
    return ::cudaFree(p);
}
extern "C" int xpfc_xcheck_fault(unsigned long long *out) {
    unsigned long long v[4];
    int (*get[4])(unsigned long long *) = {xpfc_xcheck_get_f32_p1, xpfc_xcheck_get_f32_p2, xpfc_xcheck_get_f64_p1,
                                          xpfc_xcheck_get_f64_p2};
    for (int k = 0; k < 4; k++) {
        out[4 * k] = out[4 * k + 1] = out[4 * k + 2] = out[4 * k + 3] = 0;
        if (get[k](v) == 0)
            for (int j = 0; j < 4; j++) out[4 * k + j] = v[j];
    }
    return 0;
}
static cudaError_t xchk_free_async(void *p, cudaStream_t s) {
    cudaStreamSynchronize(s);
    for (size_t i = 0; i < g_host_ranges.size(); i++)
        if (g_host_ranges[i].lo == (unsigned long long)p) {
            g_host_ranges.erase(g_host_ranges.begin() + i);
            break;
        }
    xcheck_publish();
    return ::cudaFreeAsync(p, s);
}
#define cudaFreeAsync(p, s) xchk_free_async((void *)(p), (s))
#define cudaMalloc(p, b) xchk_malloc((void **)(p), (b))
#define cudaMallocAsync(p, b, s) xchk_malloc_async((void **)(p), (b), (s))
#define cudaFree(p) xchk_free((void *)(p))
#endif

struct xpfc_ctx {
    xpfc_params p;
    int n0, n1, n2, L0, three_d;
    double Lax[3];
    long long ncells;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string err;
    // fused state (T = float for XPFC_MIXED, double for XPFC_FP64)
    void *S = nullptr, *W = nullptr, *X = nullptr;
    // 3-D FP32 grids with a register pencil plan keep S's pencil-axis
    // spectrum between steps (the pencil pass then transforms only W forward)
    void *Shat = nullptr;
    bool spec = false;
    size_t esz = 8;
    // twiddle tables W_L^k (k < L), keyed by (L, is_double), and the host
    // sources of their stream-ordered uploads
    std::map<long long, void *> tw;
    std::map<long long, std::vector<unsigned char>> tw_host;
    // host sources of the stream-ordered uploads of the coefficient tables
    // and of the batch arrays (kept until the next upload or destroy)
    std::vector<double> table_host_d;
    std::vector<float> table_host_f;
    std::vector<double> pin_host;
    std::vector<unsigned long long> seed_host;
    // per-shell coefficient tables
    void *table_f = nullptr, *table_d = nullptr;
    int mmax = 0;
    double *partials = nullptr;
    size_t partials_cap = 0;
    double *slots = nullptr;
    double *hslots = nullptr;
    int slots_cap = 0;
    double *init_red = nullptr;
    double *staged[XPFC_NBUF] = {nullptr};
    long long iteration = 0;
    bool initialized = false;
    long long launches = 0;
    void *hstage = nullptr;
    size_t hstage_bytes = 0;
    // diagnostics schedule of the last step call
    std::vector<long long> diag_its;
    std::map<long long, int> diag_slot;   // iteration -> slot
    long long diag_it0 = 0, diag_fin = 0;
    bool diag_final = false, diag_pending = false;
    // further iterations whose free energy the schedule takes (a merged
    // server group: the final iterations of its shorter solves)
    std::set<long long> diag_extra;
    // per-pass profiling with CUDA events
    bool profiling = false;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<std::pair<int, int>> ev_used;   // (pass, pool index of the start event)
    double prof_ms[8] = {0};
    long long prof_n[8] = {0};
    // batched instances (one field: nb = 1).  Instance i's field sits i
    // fields of ncells values after S (and W), its coefficient table i tables
    // of mmax + 1 shells after the first, its sums and slots after the other
    // instances'.  Per instance: params in inst[i] (psi0, peaks, seeds).
    int nb = 1;
    std::vector<xpfc_params> inst;
    double *pin_values = nullptr;          // psi0_i * ncells
    unsigned long long *seeds = nullptr;   // noise_seed_i
    long long zstride = 0;                 // complex elements between instances
    size_t part_per_inst = 0;              // partial-sum doubles per instance
    // the xy passes of a 3-D step in plane chunks on auxiliary streams
    int xy_chunks = -1;                    // -1: not chosen yet
    // pencil variant: 1 the staged (TMA) pass where it exists, 0 the register
    // pass; chosen with xy_chunks by the autotuner (or the defaults)
    int use_tma = 1;   // (the staged pass still needs XPFC_TMA=1, see tma_enabled)
    bool tuned = false;
    // captured step graph: GRAPH_STEPS plain iterations replayed by one graph
    // launch, the first iteration read from a device word (d_step_base)
    cudaGraphExec_t graph_exec = nullptr;
    long long *d_step_base = nullptr;
    const long long *cap_base = nullptr;   // set while a graph is being captured
    int graph_state = 0;                   // 0: not built, 1: ready, -1: not used
    bool graph_warm = false;               // a plain iteration ran pass by pass
    int graph_chunks = -1;                 // the chunk count it was captured with
    long long graph_kernels = 0;           // kernels in one replay
    cudaStream_t aux[4] = {nullptr, nullptr, nullptr, nullptr};
    cudaEvent_t ev_fork = nullptr, ev_join[4] = {nullptr, nullptr, nullptr, nullptr};
    // staged pencil pass of 3-D FP32 grids: tensor maps of S and W, the
    // device word its blocks set when they give up waiting for a tile, and a
    // pinned host copy of that word taken at the end of every step call
    CUtensorMap tmS{}, tmW{};
    // asynchronous read-back of the field (xpfc_get_field_async): a copy
    // stream, the events that order it after the transform to real space and
    // mark its end, a pinned host buffer and the iteration it holds
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_x_ready = nullptr, ev_copied = nullptr;
    void *hfield = nullptr;
    bool field_pending = false, copy_used = false;
    long long field_iter = 0;
    int tma_state = 0;                     // 0: not set up yet, 1: in use, -1: not used
    int *dev_err = nullptr;
    int *herr = nullptr;
};

enum { PASS_PENCIL = 0, PASS_COL_INV = 1, PASS_ROW = 2, PASS_COL_FWD = 3, PASS_RED = 4 };

// brackets one launch with a pair of pooled events when profiling is on
struct ProfScope {
    xpfc_ctx *c;
    int pass, idx = -1;
    ProfScope(xpfc_ctx *ctx, int ps) : c(ctx), pass(ps) {
        if (!c->profiling) return;
        const int used = (int)c->ev_used.size() * 2;
        if (used + 2 > (int)c->ev_pool.size()) return;
        idx = used;
        cudaEventRecord(c->ev_pool[idx], c->stream);
    }
    ~ProfScope() {
        if (idx < 0) return;
        cudaEventRecord(c->ev_pool[idx + 1], c->stream);
        c->ev_used.push_back({pass, idx});
    }
};

static void drain_profile(xpfc_ctx *c) {
    if (c->ev_used.empty()) return;
    cudaStreamSynchronize(c->stream);
    for (auto &u : c->ev_used) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, c->ev_pool[u.second], c->ev_pool[u.second + 1]) == cudaSuccess) {
            c->prof_ms[u.first] += ms;
            c->prof_n[u.first]++;
        }
    }
    c->ev_used.clear();
}

static const char *kVersion = "xpfc-gb300 0.1 (sm_103a)";

// (a failed call's error is also cleared from the thread's last-error state,
// so that a later cudaGetLastError does not report it a second time)
#define XPFC_CUDA(ctx, call)                                                                      \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) {                                                                  \
            cudaGetLastError();                                                                   \
            (ctx)->err = std::string(#call) + ": " + cudaGetErrorString(e_);                      \
            return XPFC_ECUDA;                                                                    \
        }                                                                                         \
    } while (0)

#define XPFC_LAUNCH(ctx, call)   \
    do {                         \
        (ctx)->launches++;       \
        XPFC_CUDA(ctx, call);    \
    } while (0)

// Host loops over whole fields (tens of millions of values) run in 16 fixed
// chunks on up to 16 threads; the fixed chunking keeps the mean below the
// same on every machine.
template <typename F>
static void par_chunks(size_t n, F fn) {
    constexpr int K = 16;
    if (n < ((size_t)1 << 20)) {
        for (int k = 0; k < K; k++) fn(k, n * k / K, n * (k + 1) / K);
        return;
    }
    std::vector<std::thread> th;
    th.reserve(K);
    for (int k = 0; k < K; k++) th.emplace_back(fn, k, n * k / K, n * (k + 1) / K);
    for (auto &t : th) t.join();
}

// Copies a caller's field and pins its mean to psi0 (Avg_calc.cu:21-43: the
// difference is added to every value when the mean is not psi0).  The 16
// chunks run on their own threads, or one after another when the caller
// stages several fields in parallel (the same sums either way).
static void stage_and_pin_chunks(double *dst, const double *src, size_t n, double psi0, bool threaded) {
    double part[16] = {0.0};
    auto sum_chunk = [&](int k, size_t b, size_t e) {
        double s = 0.0;
        for (size_t i = b; i < e; i++) {
            dst[i] = src[i];
            s += src[i];
        }
        part[k] = s;
    };
    if (threaded) {
        par_chunks(n, sum_chunk);
    } else {
        for (int k = 0; k < 16; k++) sum_chunk(k, n * k / 16, n * (k + 1) / 16);
    }
    double s = 0.0;
    for (int k = 0; k < 16; k++) s += part[k];
    const double m = s / (double)n;
    const double diff = (m != psi0) ? psi0 - m : 0.0;
    if (diff == 0.0) return;
    auto add_chunk = [&](int, size_t b, size_t e) {
        for (size_t i = b; i < e; i++) dst[i] += diff;
    };
    if (threaded) {
        par_chunks(n, add_chunk);
    } else {
        for (int k = 0; k < 16; k++) add_chunk(k, n * k / 16, n * (k + 1) / 16);
    }
}

// A solve in the reference's semantics (ic_kind XPFC_IC_REFERENCE: a
// pfc.input deck) pins its mean exactly as configure_avg_density does: one
// sum in index order from 0.0 (Avg_calc.cu:3-19).  The order matters on large
// fields that are nearly constant: over 16.7M values of about 0.05 the
// rounding of a running sum is systematic, and a sum in 16 chunks differs
// from the reference's by about 1e-10 of the mean, which shifts the free
// energy by about 5e-10 (measured on 4096^2).  Other solves take the chunked
// sum on host threads.
static void stage_and_pin(double *dst, const double *src, size_t n, const xpfc_params &p, bool threaded = true) {
    if (p.ic_kind == XPFC_IC_REFERENCE) {
        memcpy(dst, src, sizeof(double) * n);
        pin_mean(dst, n, p.psi0);
        return;
    }
    stage_and_pin_chunks(dst, src, n, p.psi0, threaded);
}

// Pinned host staging for the synchronous initial-field uploads
// (xpfc_initialize, xpfc_batch_initialize), shared by every context of the
// process and kept between calls, so that a solve started after another one
// does not pin fresh host memory (hundreds of MB for a batch) first.  Held
// under upload_mu from staging until the upload has completed.
static std::mutex upload_mu;
static void *upload_buf = nullptr;
static size_t upload_bytes = 0;
static void *upload_pool(size_t bytes) {
    if (bytes <= upload_bytes) return upload_buf;
    if (upload_buf) cudaFreeHost(upload_buf);
    upload_buf = nullptr;
    upload_bytes = 0;
    if (cudaHostAlloc(&upload_buf, bytes, cudaHostAllocPortable) != cudaSuccess) {
        upload_buf = nullptr;
        return nullptr;
    }
    upload_bytes = bytes;
    return upload_buf;
}

// Diagnostics switch XPFC_POISON=1: every state buffer is filled with
// all-one bytes (a NaN in FP32 and in FP64) when it is allocated, so that a
// kernel reading an element that nothing wrote makes the results non-finite
// instead of depending on what the allocator handed back.
static void poison(void *p, size_t bytes, cudaStream_t s) {
    static const bool on = [] {
        const char *e = getenv("XPFC_POISON");
        return e && e[0] == '1';
    }();
    if (on && p) cudaMemsetAsync(p, 0xFF, bytes, s);
}

static void widen(const float *f, double *d, size_t n) {
    par_chunks(n, [&](int, size_t b, size_t e) {
        for (size_t i = b; i < e; i++) d[i] = (double)f[i];
    });
}

static int fail(xpfc_ctx *ctx, int code, const std::string &m) {
    if (ctx) ctx->err = m;
    else set_thread_error(m);
    return code;
}

// ---------------------------------------------------------------------------
// parameters
// ---------------------------------------------------------------------------
extern "C" int xpfc_default_params(xpfc_params *p) {
    if (!p) return XPFC_EINVAL;
    memset(p, 0, sizeof(*p));
    p->Mx = p->My = p->Mz = 64;
    p->Lx = p->Ly = p->Lz = 8.0;
    p->psi0 = 0.05;
    p->sigma = 0.1;
    p->a = 1.0;           // eta = 2
    p->b = 1.0 / 3.0;     // chi = 1
    p->eps = 0.0;
    p->Mo = 1.0;
    p->dt = 1.0;
    p->nsteps = 2001;
    p->t_sample = 100;
    p->npeaks = 1;
    p->pk_k[0] = 2.0 * M_PI;
    p->pk_alpha[0] = 1.0;
    p->pk_rho[0] = 1.0;
    p->pk_beta[0] = 8.0;
    p->envelope = XPFC_ENVELOPE_MAX;
    p->precision = XPFC_FP64;
    p->ref_compat = 0;
    p->ff_factor = (8.0 / 64) * (8.0 / 64) * (8.0 / 64);
    p->ic_kind = XPFC_IC_NOISE;
    p->iconfig = 2;
    p->ic_amp = 0.1;
    p->ic_seed = 1;
    p->noise_seed = 1;
    p->device = 0;
    return XPFC_OK;
}

extern "C" int xpfc_read_input(const char *path, xpfc_params *p) {
    if (!path || !p) return fail(nullptr, XPFC_EINVAL, "null argument");
    return read_input(path, p);
}

extern "C" const char *xpfc_version(void) { return kVersion; }

extern "C" const char *xpfc_last_error(const xpfc_ctx *ctx) { return ctx ? ctx->err.c_str() : thread_error(); }

extern "C" int xpfc_get_params(const xpfc_ctx *ctx, xpfc_params *p) {
    if (!ctx || !p) return XPFC_EINVAL;
    *p = ctx->p;
    return XPFC_OK;
}

extern "C" void *xpfc_get_stream(const xpfc_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

extern "C" long long xpfc_launch_count(const xpfc_ctx *ctx) { return ctx ? ctx->launches : 0; }

extern "C" long long xpfc_pass_bytes(const xpfc_ctx *ctx, int pass) {
    if (!ctx) return -1;
    const long long arr = (long long)ctx->esz * ctx->ncells * ctx->nb;   // one field array
    switch (pass) {
        case 0: return (ctx->spec ? 4 : 3) * arr;           // pencil: S (or Shat), W in; S (and Shat) out
        case 1: case 3: return ctx->three_d ? 2 * arr : 0;   // column passes
        case 2: return 2 * arr;                              // row pass
        default: return -1;
    }
}

extern "C" long long xpfc_iteration(const xpfc_ctx *ctx) { return ctx ? ctx->iteration : -1; }

extern "C" int xpfc_build_initial_field(const xpfc_params *p, double *host_psi) {
    if (!p || !host_psi) return fail(nullptr, XPFC_EINVAL, "null argument");
    return build_initial_field(p, host_psi);
}

extern "C" int xpfc_write_vtk(const char *path, const double *psi, int Mx, int My, int Mz, double Lx, double Ly,
                              double Lz, int precision) {
    if (!path || !psi || Mx <= 0 || My <= 0 || Mz <= 0) return fail(nullptr, XPFC_EINVAL, "bad argument");
    return write_vtk(path, psi, Mx, My, Mz, Lx, Ly, Lz, precision);
}

extern "C" int xpfc_read_vtk(const char *path, double *psi, size_t cap, int dims[3], double L[3]) {
    if (!path) return fail(nullptr, XPFC_EINVAL, "null path");
    return read_vtk(path, psi, cap, dims, L);
}

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
static double c2_of(const xpfc_params &p, double kmag) {
    // initialize.cu:209-217 (sum) and its max envelope
    double acc = 0.0;
    for (int i = 0; i < p.npeaks; i++) {
        const double sk = p.sigma * p.pk_k[i];
        const double dw = std::exp(-(sk * sk) / (2.0 * p.pk_rho[i] * p.pk_beta[i]));
        const double d = kmag - p.pk_k[i];
        const double v = dw * std::exp(-(d * d) / (2.0 * p.pk_alpha[i] * p.pk_alpha[i]));
        if (p.envelope == XPFC_ENVELOPE_SUM) acc += v;
        else acc = (i == 0 || v > acc) ? v : acc;
    }
    return acc;
}

// Twiddle table W_L^k of one length and precision, built on first use.  The
// upload is ordered on the context's stream (every launch that reads the
// table comes after it on that stream, or on an auxiliary stream forked from
// it later), and its host source stays alive in the context until destroy,
// so no kernel can read a partly written table.
static void *twiddle(xpfc_ctx *ctx, int L, bool dbl) {
    const long long key = 2LL * L + (dbl ? 1 : 0);
    auto it = ctx->tw.find(key);
    if (it != ctx->tw.end()) return it->second;
    const size_t bytes = (dbl ? sizeof(double) : sizeof(float)) * 2 * (size_t)L;
    std::vector<unsigned char> &h = ctx->tw_host[key];
    h.resize(bytes);
    for (int k = 0; k < L; k++) {
        const double ang = 2.0 * M_PI * (double)k / (double)L;
        const double c = std::cos(ang), s = -std::sin(ang);
        if (dbl) {
            reinterpret_cast<double *>(h.data())[2 * k] = c;
            reinterpret_cast<double *>(h.data())[2 * k + 1] = s;
        } else {
            reinterpret_cast<float *>(h.data())[2 * k] = (float)c;
            reinterpret_cast<float *>(h.data())[2 * k + 1] = (float)s;
        }
    }
    void *d = nullptr;
    cudaError_t e = cudaMalloc(&d, bytes);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d, h.data(), bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) {
        if (d) cudaFree(d);
        ctx->err = std::string("twiddle table upload: ") + cudaGetErrorString(e);
        return nullptr;
    }
    ctx->tw[key] = d;
    return d;
}

static KSpace make_kspace(const xpfc_ctx *ctx, bool dbl) {
    const xpfc_params &p = ctx->p;
    KSpace ks;
    memset(&ks, 0, sizeof(ks));
    ks.n0 = ctx->n0;
    ks.n1 = ctx->n1;
    ks.n2 = ctx->n2;
    const double d0 = 2.0 * M_PI / ctx->Lax[0], d1 = 2.0 * M_PI / ctx->Lax[1], d2 = 2.0 * M_PI / ctx->Lax[2];
    ks.dk0sq = d0 * d0;
    ks.dk1sq = d1 * d1;
    ks.dk2sq = ctx->n2 > 1 ? d2 * d2 : 0.0;
    ks.table = dbl ? ctx->table_d : ctx->table_f;
    ks.tstride = ctx->nb > 1 ? (long long)ctx->mmax + 1 : 0;
    ks.seeds = ctx->nb > 1 ? ctx->seeds : nullptr;
    ks.mmax = ctx->mmax;
    ks.dt = p.dt;
    ks.Mo = p.Mo;
    ks.Mo_res = p.ref_compat ? (double)(int)p.Mo : p.Mo;   // sse_calculation.cu:120 takes int Mo
    ks.eps = p.eps;
    ks.npeaks = p.npeaks;
    ks.envelope = p.envelope;
    for (int i = 0; i < p.npeaks && i < 8; i++) {
        const double sk = p.sigma * p.pk_k[i];
        ks.pk_k[i] = p.pk_k[i];
        ks.pk_inv2a2[i] = 1.0 / (2.0 * p.pk_alpha[i] * p.pk_alpha[i]);
        ks.pk_dw[i] = std::exp(-(sk * sk) / (2.0 * p.pk_rho[i] * p.pk_beta[i]));
    }
    ks.noise_on = p.noise_amp != 0.0;
    ks.noise_scale = p.noise_amp * std::sqrt((double)ctx->ncells);
    ks.noise_seed = p.noise_seed;
    ks.f_dk0sq = (float)ks.dk0sq;
    ks.f_dk1sq = (float)ks.dk1sq;
    ks.f_dk2sq = (float)ks.dk2sq;
    ks.f_dt = (float)ks.dt;
    ks.f_Mo = (float)ks.Mo;
    ks.f_eps = (float)ks.eps;
    ks.f_noise_scale = (float)ks.noise_scale;
    for (int i = 0; i < 8; i++) {
        ks.f_pk_k[i] = (float)ks.pk_k[i];
        ks.f_pk_inv2a2[i] = (float)ks.pk_inv2a2[i];
        ks.f_pk_dw[i] = (float)ks.pk_dw[i];
    }
    return ks;
}

static int build_tables(xpfc_ctx *ctx) {
    // one coefficient set per shell m = i0^2 + i1^2 + i2^2 when the k-grid
    // spacing is the same on every axis (equal box lengths)
    const bool cubic = (ctx->Lax[0] == ctx->Lax[1]) && (ctx->n2 == 1 || ctx->Lax[0] == ctx->Lax[2]);
    if (!cubic) {
        // coefficients on the fly; a reused context drops the tables of its last params
        cudaFree(ctx->table_d);
        cudaFree(ctx->table_f);
        ctx->table_d = ctx->table_f = nullptr;
        return XPFC_OK;
    }
    const int h0 = ctx->n0 / 2, h1 = ctx->n1 / 2, h2 = ctx->n2 / 2;
    ctx->mmax = h0 * h0 + h1 * h1 + h2 * h2;
    const size_t nm = (size_t)ctx->mmax + 1;
    // the host sources of the last upload stay alive in the context; a new
    // upload (a pooled context taking new params) waits for the last one
    if (!ctx->table_host_d.empty()) XPFC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    std::vector<double> &td = ctx->table_host_d;
    std::vector<float> &tf = ctx->table_host_f;
    td.assign(4 * nm * ctx->nb, 0.0);
    tf.assign(4 * nm * ctx->nb, 0.f);
    const double dk = 2.0 * M_PI / ctx->Lax[0];
    for (int i = 0; i < ctx->nb; i++) {
        const xpfc_params &p = ctx->inst[i];
        double *d = td.data() + 4 * nm * i;
        for (size_t m = 0; m < nm; m++) {
            const double k2 = dk * dk * (double)m;
            const double c2 = c2_of(p, std::sqrt(k2));
            const double den = (1.0 + k2 * p.dt * p.Mo * (1.0 - p.eps) - k2 * p.Mo * p.dt * c2);
            d[4 * m + 0] = 1.0 / den;
            d[4 * m + 1] = -(k2 * p.Mo * p.dt) / den;
            d[4 * m + 2] = c2;
            d[4 * m + 3] = k2;
        }
    }
    for (size_t j = 0; j < td.size(); j++) tf[j] = (float)td[j];
    // the size depends only on the grid and nb, so a reused context keeps its buffers
    if (!ctx->table_d) XPFC_CUDA(ctx, cudaMalloc(&ctx->table_d, sizeof(double) * td.size()));
    if (!ctx->table_f) XPFC_CUDA(ctx, cudaMalloc(&ctx->table_f, sizeof(float) * tf.size()));
    // stream-ordered: every pass that reads the tables comes after these
    XPFC_CUDA(ctx, cudaMemcpyAsync(ctx->table_d, td.data(), sizeof(double) * td.size(), cudaMemcpyHostToDevice,
                                   ctx->stream));
    XPFC_CUDA(ctx, cudaMemcpyAsync(ctx->table_f, tf.data(), sizeof(float) * tf.size(), cudaMemcpyHostToDevice,
                                   ctx->stream));
    return XPFC_OK;
}

static int ensure_partials(xpfc_ctx *ctx, size_t n) {
    if (n <= ctx->partials_cap) return XPFC_OK;
    if (ctx->partials) cudaFree(ctx->partials);
    ctx->partials = nullptr;
    XPFC_CUDA(ctx, cudaMalloc(&ctx->partials, sizeof(double) * n));
    poison(ctx->partials, sizeof(double) * n, ctx->stream);
    ctx->partials_cap = n;
    return XPFC_OK;
}

// A context over nb instances that share everything but psi0, the peaks
// (sigma, envelope) and the seeds: ps[0..nb-1].  nb = 1 is xpfc_create.
// The checks that need no device: sizes, scheme constants, compiled lengths.
static int check_params(const xpfc_params *q) {
    if (q->Mx <= 0 || q->My <= 0 || q->Mz <= 0) return fail(nullptr, XPFC_EINVAL, "grid sizes must be positive");
    if (q->dt <= 0.0 || q->npeaks < 1 || q->npeaks > XPFC_MAX_PEAKS)
        return fail(nullptr, XPFC_EINVAL, "dt must be > 0 and 1 <= npeaks <= 8");
    if (q->precision != XPFC_FP64 && q->precision != XPFC_MIXED) return fail(nullptr, XPFC_EINVAL, "bad precision");
    if (q->device < 0 || q->device >= 64)
        return fail(nullptr, XPFC_EINVAL, "device ordinal must be in [0, 64) (per-device launch set-up flags)");
    const bool three = q->Mz > 1;
    const int n0 = three ? q->Mz : q->My, n1 = three ? q->My : q->Mx, n2 = three ? q->Mx : 1;
    if (n0 % 2 != 0 || n1 % 2 != 0 || (three && n2 % 2 != 0))
        return fail(nullptr, XPFC_EINVAL, "grid sizes must be even");
    if (!row_supported(n0 / 2))
        return fail(nullptr, XPFC_EINVAL, "unsupported size of the fastest axis: " + std::to_string(n0));
    if (!col_supported(n1)) return fail(nullptr, XPFC_EINVAL, "unsupported axis length " + std::to_string(n1));
    if (three && (!col_supported(n2) || !pen_supported(n2, 2)))
        return fail(nullptr, XPFC_EINVAL, "unsupported axis length " + std::to_string(n2));
    if (!three && !pen_supported(n1, 1))
        return fail(nullptr, XPFC_EINVAL, "unsupported axis length " + std::to_string(n1));
    return XPFC_OK;
}

// Whether a context keeps S's pencil-axis spectrum (Shat): 3-D FP32 grids
// whose pencil length has the kept-spectrum register pencil, unless
// XPFC_SPEC=0 (or XPFC_TMA=1, whose staged pencil transforms S each step).
static bool spec_for(const xpfc_params &p) {
    static const bool on = [] {
        const char *e = getenv("XPFC_SPEC");
        const char *t = getenv("XPFC_TMA");
        return !(e && e[0] == '0') && !(t && t[0] == '1');
    }();
    return on && p.Mz > 1 && p.precision == XPFC_MIXED && pen_spec_supported(p.Mx, 4);
}

static int create_group(const xpfc_params *ps, int nb, xpfc_ctx **out) {
    const xpfc_params *p = ps;
    for (int i = 0; i < nb; i++) {
        const int rc = check_params(ps + i);
        if (rc != XPFC_OK) return rc;
    }
    xpfc_ctx *ctx = new xpfc_ctx();
    ctx->p = *p;
    ctx->nb = nb;
    ctx->inst.assign(ps, ps + nb);
    ctx->three_d = p->Mz > 1;
    if (ctx->three_d) {
        ctx->n0 = p->Mz; ctx->n1 = p->My; ctx->n2 = p->Mx;
        ctx->Lax[0] = p->Lz; ctx->Lax[1] = p->Ly; ctx->Lax[2] = p->Lx;
    } else {
        ctx->n0 = p->My; ctx->n1 = p->Mx; ctx->n2 = 1;
        ctx->Lax[0] = p->Ly; ctx->Lax[1] = p->Lx; ctx->Lax[2] = 1.0;
    }
    ctx->L0 = ctx->n0 / 2;
    ctx->ncells = (long long)ctx->n0 * ctx->n1 * ctx->n2;
    ctx->zstride = nb > 1 ? ctx->ncells / 2 : 0;
    cudaError_t e = cudaSetDevice(p->device);
    if (e != cudaSuccess) {
        set_thread_error(std::string("cudaSetDevice: ") + cudaGetErrorString(e));
        delete ctx;
        return XPFC_ECUDA;
    }
    if (p->stream) {
        ctx->stream = (cudaStream_t)p->stream;
    } else {
        e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            set_thread_error(std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
            delete ctx;
            return XPFC_ECUDA;
        }
        ctx->own_stream = true;
    }
    ctx->esz = p->precision == XPFC_MIXED ? sizeof(float) : sizeof(double);
    const size_t bytes = ctx->esz * (size_t)ctx->ncells * nb;
    int rc = XPFC_OK;
    if (cudaMalloc(&ctx->S, bytes) != cudaSuccess || cudaMalloc(&ctx->W, bytes) != cudaSuccess) {
        set_thread_error("device allocation of the state failed");
        xpfc_destroy(ctx);
        return XPFC_ENOMEM;
    }
    poison(ctx->S, bytes, ctx->stream);
    poison(ctx->W, bytes, ctx->stream);
    if (spec_for(*p)) {
        if (cudaMalloc(&ctx->Shat, bytes) != cudaSuccess) {
            set_thread_error("device allocation of the kept spectrum failed");
            xpfc_destroy(ctx);
            return XPFC_ENOMEM;
        }
        poison(ctx->Shat, bytes, ctx->stream);
        ctx->spec = true;
    }
    rc = build_tables(ctx);
    if (rc == XPFC_OK) {
        const int L0 = ctx->L0;
        const size_t rowblk = (size_t)ctx->n1 * ctx->n2 / row_rows(L0) + 1;
        const int tx = ctx->esz == 4 ? (ctx->three_d ? pen_tx<float>(ctx->n2, 2) : pen_tx<float>(ctx->n1, 1))
                                     : (ctx->three_d ? pen_tx<double>(ctx->n2, 2) : pen_tx<double>(ctx->n1, 1));
        const size_t penblk = (size_t)(L0 / tx + 1) * (ctx->n1 / 2 + 1);
        ctx->part_per_inst = std::max(rowblk * NQ_ROW, penblk * NQ_PEN);
        const size_t need = std::max(ctx->part_per_inst * nb, (size_t)IC_SCRATCH);
        rc = ensure_partials(ctx, need);
    }
    if (rc == XPFC_OK && cudaMalloc(&ctx->init_red, sizeof(double) * 8 * nb) != cudaSuccess) rc = XPFC_ENOMEM;
    if (rc == XPFC_OK && nb > 1) {
        // per-instance pinned means and noise seeds, uploaded on the context's
        // stream (ordered before every pass) from host copies the context keeps
        std::vector<double> &pv = ctx->pin_host;
        std::vector<unsigned long long> &sd = ctx->seed_host;
        pv.resize(nb);
        sd.resize(nb);
        for (int i = 0; i < nb; i++) {
            pv[i] = ps[i].psi0 * (double)ctx->ncells;
            sd[i] = ps[i].noise_seed;
        }
        if (cudaMalloc(&ctx->pin_values, sizeof(double) * nb) != cudaSuccess ||
            cudaMalloc(&ctx->seeds, sizeof(unsigned long long) * nb) != cudaSuccess) {
            rc = XPFC_ENOMEM;
        } else {
            cudaError_t e2 = cudaMemcpyAsync(ctx->pin_values, pv.data(), sizeof(double) * nb,
                                             cudaMemcpyHostToDevice, ctx->stream);
            if (e2 == cudaSuccess)
                e2 = cudaMemcpyAsync(ctx->seeds, sd.data(), sizeof(unsigned long long) * nb,
                                     cudaMemcpyHostToDevice, ctx->stream);
            if (e2 != cudaSuccess) {
                ctx->err = std::string("batch array upload: ") + cudaGetErrorString(e2);
                rc = XPFC_ECUDA;
            }
        }
    }
    if (rc != XPFC_OK) {
        set_thread_error(ctx->err.empty() ? "context set-up failed" : ctx->err);
        xpfc_destroy(ctx);
        return rc;
    }
    *out = ctx;
    return XPFC_OK;
}

extern "C" int xpfc_create(const xpfc_params *p, xpfc_ctx **out) {
    if (!p || !out) return fail(nullptr, XPFC_EINVAL, "null argument");
    *out = nullptr;
    return create_group(p, 1, out);
}

extern "C" int xpfc_destroy(xpfc_ctx *ctx) {
    if (!ctx) return XPFC_OK;
    cudaSetDevice(ctx->p.device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    cudaFree(ctx->S);
    cudaFree(ctx->W);
    cudaFree(ctx->X);
    cudaFree(ctx->Shat);
    for (auto &kv : ctx->tw) cudaFree(kv.second);
    cudaFree(ctx->table_f);
    cudaFree(ctx->table_d);
    cudaFree(ctx->partials);
    cudaFree(ctx->slots);
    cudaFree(ctx->init_red);
    cudaFree(ctx->pin_values);
    cudaFree(ctx->seeds);
    for (int k = 0; k < 4; k++) {
        if (ctx->aux[k]) cudaStreamDestroy(ctx->aux[k]);
        if (ctx->ev_join[k]) cudaEventDestroy(ctx->ev_join[k]);
    }
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    if (ctx->hslots) cudaFreeHost(ctx->hslots);
    if (ctx->hstage) cudaFreeHost(ctx->hstage);
    cudaFree(ctx->dev_err);
    if (ctx->herr) cudaFreeHost(ctx->herr);
    if (ctx->copy_stream) {
        cudaStreamSynchronize(ctx->copy_stream);
        cudaStreamDestroy(ctx->copy_stream);
    }
    if (ctx->ev_x_ready) cudaEventDestroy(ctx->ev_x_ready);
    if (ctx->ev_copied) cudaEventDestroy(ctx->ev_copied);
    if (ctx->hfield) cudaFreeHost(ctx->hfield);
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
    cudaFree(ctx->d_step_base);
    for (int b = 0; b < XPFC_NBUF; b++) cudaFree(ctx->staged[b]);
    for (auto &e : ctx->ev_pool) cudaEventDestroy(e);
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return XPFC_OK;
}

static int host_stage(xpfc_ctx *ctx, size_t bytes) {
    if (bytes <= ctx->hstage_bytes) return XPFC_OK;
    if (ctx->hstage) cudaFreeHost(ctx->hstage);
    ctx->hstage = nullptr;
    XPFC_CUDA(ctx, cudaMallocHost(&ctx->hstage, bytes));
    ctx->hstage_bytes = bytes;
    return XPFC_OK;
}

static double *staged_buf(xpfc_ctx *ctx, int b) {
    if (b < 0 || b >= XPFC_NBUF) return nullptr;
    if (!ctx->staged[b]) {
        if (cudaMalloc(&ctx->staged[b], sizeof(double) * (size_t)ctx->ncells) != cudaSuccess) return nullptr;
        cudaMemsetAsync(ctx->staged[b], 0, sizeof(double) * (size_t)ctx->ncells, ctx->stream);
    }
    return ctx->staged[b];
}

// ---------------------------------------------------------------------------
// transforms on one field buffer of type T (packed spectrum <-> real)
// ---------------------------------------------------------------------------
// Forward transform of everything but the pencil axis: the rows (unless
// do_rows is false) and, in 3-D, the y columns.
template <typename T>
static int fft_forward_xy(xpfc_ctx *ctx, void *buf, bool do_rows) {
    const bool dbl = sizeof(T) == 8;
    void *tw0 = twiddle(ctx, ctx->L0, dbl), *tw2 = twiddle(ctx, ctx->n0, dbl), *tw1 = twiddle(ctx, ctx->n1, dbl);
    if (!tw0 || !tw2 || !tw1) return fail(ctx, XPFC_ENOMEM, "twiddle tables");
    if (do_rows) {
        RowArgs ra{};
        ra.in = buf;
        ra.out = buf;
        ra.nrows = (long long)ctx->n1 * ctx->n2;
        ra.scale = 1.0;
        ra.zstride = ctx->zstride;
        ra.nz = ctx->nb;
        XPFC_LAUNCH(ctx, launch_row<T>(ROW_FWD, ctx->L0, ra, tw0, tw2, ctx->stream, nullptr));
    }
    if (!ctx->three_d) return XPFC_OK;
    ColArgs ca{};
    ca.in = buf;
    ca.out = buf;
    ca.es = ctx->L0;
    ca.ostride = (long long)ctx->n1 * ctx->L0;
    ca.scale = 1.0;
    ca.ncols = ctx->L0;
    ca.zstride = ctx->zstride;
    ca.nz = ctx->nb;
    XPFC_LAUNCH(ctx, launch_col<T>(-1, ctx->n1, ca, ctx->n2, tw1, ctx->stream));
    return XPFC_OK;
}

template <typename T>
static int fft_full(xpfc_ctx *ctx, void *buf, int dir) {
    const bool dbl = sizeof(T) == 8;
    void *tw0 = twiddle(ctx, ctx->L0, dbl), *tw2 = twiddle(ctx, ctx->n0, dbl), *tw1 = twiddle(ctx, ctx->n1, dbl);
    void *twz = ctx->three_d ? twiddle(ctx, ctx->n2, dbl) : nullptr;
    if (!tw0 || !tw2 || !tw1 || (ctx->three_d && !twz)) return fail(ctx, XPFC_ENOMEM, "twiddle tables");
    RowArgs ra{};
    ra.in = buf;
    ra.out = buf;
    ra.nrows = (long long)ctx->n1 * ctx->n2;
    ra.scale = 1.0;
    ColArgs cy{};
    cy.in = buf;
    cy.out = buf;
    cy.es = ctx->L0;
    cy.ostride = (long long)ctx->n1 * ctx->L0;
    cy.scale = 1.0;
    cy.ncols = ctx->L0;
    ColArgs cz{};
    cz.in = buf;
    cz.out = buf;
    cz.es = (long long)ctx->n1 * ctx->L0;
    cz.ostride = ctx->L0;
    cz.scale = 1.0;
    cz.ncols = ctx->L0;
    if (dir < 0) {
        XPFC_LAUNCH(ctx, launch_row<T>(ROW_FWD, ctx->L0, ra, tw0, tw2, ctx->stream, nullptr));
        XPFC_LAUNCH(ctx, launch_col<T>(-1, ctx->n1, cy, ctx->n2, tw1, ctx->stream));
        if (ctx->three_d) XPFC_LAUNCH(ctx, launch_col<T>(-1, ctx->n2, cz, ctx->n1, twz, ctx->stream));
    } else {
        if (ctx->three_d) XPFC_LAUNCH(ctx, launch_col<T>(1, ctx->n2, cz, ctx->n1, twz, ctx->stream));
        XPFC_LAUNCH(ctx, launch_col<T>(1, ctx->n1, cy, ctx->n2, tw1, ctx->stream));
        XPFC_LAUNCH(ctx, launch_row<T>(ROW_INV, ctx->L0, ra, tw0, tw2, ctx->stream, nullptr));
    }
    return XPFC_OK;
}

// ---------------------------------------------------------------------------
// initialisation of both the staged buffers and the fused state
// ---------------------------------------------------------------------------
template <typename T>
static int init_fused(xpfc_ctx *ctx, const double *dpsi) {
    const bool dbl = sizeof(T) == 8;
    const long long n = ctx->ncells * ctx->nb;
    if (dbl) XPFC_CUDA(ctx, cudaMemcpyAsync(ctx->S, dpsi, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
    else XPFC_LAUNCH(ctx, launch_convert_d2f(dpsi, (float *)ctx->S, n, ctx->stream));
    void *tw0 = twiddle(ctx, ctx->L0, dbl), *tw2 = twiddle(ctx, ctx->n0, dbl);
    if (!tw0 || !tw2) return fail(ctx, XPFC_ENOMEM, "twiddle tables");
    // W = row transform of N(psi), with the iteration-0 real-space sums
    RowArgs ra{};
    ra.in = ctx->S;
    ra.out = ctx->W;
    ra.nrows = (long long)ctx->n1 * ctx->n2;
    ra.a = ctx->p.a;
    ra.b = ctx->p.b;
    ra.scale = 1.0;
    ra.partials = ctx->partials;
    ra.want_red = 1;
    ra.ref_compat = ctx->p.ref_compat;
    ra.zstride = ctx->zstride;
    ra.nz = ctx->nb;
    int nb = 0;
    XPFC_LAUNCH(ctx, launch_row<T>(ROW_NL_FWD, ctx->L0, ra, tw0, tw2, ctx->stream, &nb));
    XPFC_LAUNCH(ctx, launch_finalize(NQ_ROW, ctx->partials, nb, ctx->init_red, ctx->stream, ctx->nb, 8));
    int rc = fft_forward_xy<T>(ctx, ctx->S, true);
    if (rc != XPFC_OK) return rc;
    if (ctx->three_d) {
        rc = fft_forward_xy<T>(ctx, ctx->W, false);
        if (rc != XPFC_OK) return rc;
    }
    if (ctx->spec) {
        // the kept spectrum: S transformed forward along the pencil axis (the
        // n1 L0 columns of every plane are contiguous, planes n1 L0 apart)
        void *twz = twiddle(ctx, ctx->n2, dbl);
        if (!twz) return fail(ctx, XPFC_ENOMEM, "twiddle tables");
        ColArgs cz{};
        cz.in = ctx->S;
        cz.out = ctx->Shat;
        cz.es = (long long)ctx->n1 * ctx->L0;
        cz.ostride = 0;
        cz.scale = 1.0;
        cz.ncols = (long long)ctx->n1 * ctx->L0;
        cz.zstride = ctx->zstride;
        cz.nz = ctx->nb;
        XPFC_LAUNCH(ctx, launch_col<T>(-1, ctx->n2, cz, 1, twz, ctx->stream));
    }
    return XPFC_OK;
}

// ---------------------------------------------------------------------------
// initial fields on the device (every generator but the VTK restart)
// ---------------------------------------------------------------------------
// The reference's own initial conditions (its lattices, seeds and the VTK
// restart) are built on the host by the restatement of initialize.cu, whose
// mean pin keeps the reference's summation order (see stage_and_pin); the
// library's generators (noise liquid, fcc seed) run on the device.
static bool ic_on_device(const xpfc_params &p) { return p.ic_kind != XPFC_IC_REFERENCE; }

// Enqueues p's initial field (mean pinned to psi0) into dpsi on stream s;
// scratch: IC_SCRATCH device doubles.  Returns a status and sets *why.
static int enqueue_initial_field(const xpfc_params &p, double *dpsi, double *scratch, cudaStream_t s,
                                 std::string *why) {
    ICArgs a{};
    a.Mx = p.Mx; a.My = p.My; a.Mz = p.Mz;
    a.Lx = p.Lx; a.Ly = p.Ly; a.Lz = p.Lz;
    a.psi0 = p.psi0;
    a.amp = p.ic_amp;
    a.seed = p.ic_seed;
    a.seed_amp = p.ic_seed_amp;
    a.seed_radius = p.ic_seed_radius;
    a.iconfig = p.iconfig; a.iseed = p.iseed; a.ishape = p.ishape;
    a.A_10 = p.A_10; a.A_11 = p.A_11; a.A_tri = p.A_tri;
    a.h = p.h; a.k = p.k; a.roa = p.roa;
    double *coords = nullptr;
    switch (p.ic_kind) {
        case XPFC_IC_NOISE: a.kind = IC_DEV_NOISE; break;
        case XPFC_IC_FCC_SEED: a.kind = IC_DEV_FCC_SEED; break;
        case XPFC_IC_REFERENCE: {
            if (p.iconfig == 10) {
                *why = "the VTK restart is read on the host";
                return XPFC_EINVAL;
            }
            if (p.Mz != 1) {
                *why = "reference initial conditions are 2-D (Mz must be 1)";
                return XPFC_EINVAL;
            }
            a.kind = IC_DEV_REFERENCE;
            // linspace.cu:5-18: accumulated coordinates, du = L/(M-1), summed in order
            std::vector<double> c((size_t)p.Mx + p.My + 2);
            const double dux = p.Lx / ((double)p.Mx - 1), duy = p.Ly / ((double)p.My - 1);
            c[0] = 0.0;
            for (int i = 0; i < p.Mx; i++) c[i + 1] = c[i] + dux;
            double *cy = c.data() + p.Mx + 1;
            cy[0] = 0.0;
            for (int j = 0; j < p.My; j++) cy[j + 1] = cy[j] + duy;
            cudaError_t e = cudaMallocAsync((void **)&coords, sizeof(double) * c.size(), s);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(coords, c.data(), sizeof(double) * c.size(), cudaMemcpyHostToDevice, s);
            if (e != cudaSuccess) {
                *why = std::string("coordinates: ") + cudaGetErrorString(e);
                return XPFC_ECUDA;
            }
            a.xs = coords;
            a.ys = coords + p.Mx + 1;
            break;
        }
        default: *why = "unknown ic_kind"; return XPFC_EINVAL;
    }
    cudaError_t e = launch_initial_field(a, dpsi, scratch, s);
    if (coords) cudaFreeAsync(coords, s);
    if (e != cudaSuccess) {
        *why = std::string("initial field: ") + cudaGetErrorString(e);
        return XPFC_ECUDA;
    }
    return XPFC_OK;
}

extern "C" int xpfc_build_initial_field_device(const xpfc_params *p, double *dev_psi, void *stream) {
    if (!p || !dev_psi) return fail(nullptr, XPFC_EINVAL, "null argument");
    cudaStream_t s = (cudaStream_t)stream;
    double *scratch = nullptr;
    cudaError_t e = cudaSetDevice(p->device);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&scratch, sizeof(double) * IC_SCRATCH, s);
    if (e != cudaSuccess) return fail(nullptr, XPFC_ECUDA, std::string("scratch: ") + cudaGetErrorString(e));
    std::string why;
    const int rc = enqueue_initial_field(*p, dev_psi, scratch, s, &why);
    cudaFreeAsync(scratch, s);
    if (rc != XPFC_OK) return fail(nullptr, rc, why);
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(nullptr, XPFC_ECUDA, cudaGetErrorString(e));
    return XPFC_OK;
}

extern "C" int xpfc_initialize(xpfc_ctx *ctx, const double *host_psi) {
    if (!ctx) return fail(nullptr, XPFC_EINVAL, "null context");
    XPFC_CUDA(ctx, cudaSetDevice(ctx->p.device));
    const size_t n = (size_t)ctx->ncells;
    double *dpsi = staged_buf(ctx, XPFC_BUF_PSI);
    if (!dpsi) return fail(ctx, XPFC_ENOMEM, "staged buffer allocation failed");
    int rc = XPFC_OK;
    if (!host_psi && ic_on_device(ctx->p)) {
        std::string why;
        rc = enqueue_initial_field(ctx->p, dpsi, ctx->partials, ctx->stream, &why);
        if (rc != XPFC_OK) return fail(ctx, rc, why);
    } else {
        std::lock_guard<std::mutex> g(upload_mu);
        double *h = (double *)upload_pool(sizeof(double) * n);
        if (!h) return fail(ctx, XPFC_ENOMEM, "pinned upload staging");
        if (host_psi) {
            stage_and_pin(h, host_psi, n, ctx->p);   // configure_avg_density, Avg_calc.cu:21-43
        } else {
            rc = build_initial_field(&ctx->p, h);   // the reference's initial conditions
            if (rc != XPFC_OK) return fail(ctx, rc, thread_error());
        }
        XPFC_CUDA(ctx, cudaMemcpyAsync(dpsi, h, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
        XPFC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));   // the staging is free again
    }
    rc = ctx->esz == 4 ? init_fused<float>(ctx, dpsi) : init_fused<double>(ctx, dpsi);
    if (rc != XPFC_OK) return rc;
    XPFC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->iteration = 0;
    ctx->initialized = true;
    return XPFC_OK;
}

// ---------------------------------------------------------------------------
// fused step
// ---------------------------------------------------------------------------
// The staged (TMA) pencil pass (xpfc_tma.cuh) for 3-D FP32 grids whose pencil
// length has a staged instance, selected with XPFC_TMA=1 in the environment.
// It is not the default: on GB300 at 256^3 it ran 138 us per launch against
// the register pencil's 120 us, and the two kernels' results differ in the
// last bits (the compiler contracts multiply-adds differently in each), so
// they are not interchangeable within one solve.
static bool tma_enabled() {
    static const bool on = [] {
        const char *e = getenv("XPFC_TMA");
        return e && e[0] == '1';
    }();
    return on;
}

// cuTensorMapEncodeTiled from the driver, through the runtime's entry-point
// query (the library links no driver library itself)
static PFN_cuTensorMapEncodeTiled_v12000 tma_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    }();
    return fn;
}

// Tensor maps of S and W for boxes of tx complex columns x 1 row x the whole
// pencil (length Lp), set up once per context; false: use the register pencil.
static bool tma_ready(xpfc_ctx *ctx, int tx, int Lp) {
    if (ctx->tma_state != 0) return ctx->tma_state > 0;
    ctx->tma_state = -1;
    if (!tma_enabled()) return false;
    PFN_cuTensorMapEncodeTiled_v12000 enc = tma_encoder();
    if (!enc) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)2 * ctx->L0, (cuuint64_t)ctx->n1, (cuuint64_t)ctx->n2 * ctx->nb};
    const cuuint64_t strides[2] = {(cuuint64_t)2 * ctx->L0 * sizeof(float),
                                   (cuuint64_t)2 * ctx->L0 * ctx->n1 * sizeof(float)};
    const cuuint32_t box[3] = {(cuuint32_t)(2 * tx), 1u, (cuuint32_t)Lp};
    const cuuint32_t es[3] = {1u, 1u, 1u};
    for (int a = 0; a < 2; a++) {
        const CUresult r = enc(a == 0 ? &ctx->tmS : &ctx->tmW, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3,
                               a == 0 ? ctx->S : ctx->W, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return false;
    }
    if (cudaMalloc(&ctx->dev_err, sizeof(int)) != cudaSuccess) return false;
    if (cudaMallocHost(&ctx->herr, sizeof(int)) != cudaSuccess) {
        cudaFree(ctx->dev_err);
        ctx->dev_err = nullptr;
        return false;
    }
    *ctx->herr = 0;
    if (cudaMemsetAsync(ctx->dev_err, 0, sizeof(int), ctx->stream) != cudaSuccess) return false;
    ctx->tma_state = 1;
    return true;
}

template <typename T>
static int launch_pencil_pass(xpfc_ctx *ctx, long long step, int update, int want_red, int *nb) {
    const bool dbl = sizeof(T) == 8;
    const int Lp = ctx->three_d ? ctx->n2 : ctx->n1;
    void *twp = twiddle(ctx, Lp, dbl);
    if (!twp) return fail(ctx, XPFC_ENOMEM, "twiddle tables");
    KSpace ks = make_kspace(ctx, dbl);
    ks.step = step;
    ks.step_base = ctx->cap_base;
    PenArgs pa{};
    pa.S = ctx->S;
    pa.W = ctx->W;
    pa.Shat = ctx->spec ? ctx->Shat : nullptr;
    pa.es = ctx->three_d ? (long long)ctx->n1 * ctx->L0 : ctx->L0;
    pa.gstride = ctx->three_d ? ctx->L0 : 0;
    pa.three_d = ctx->three_d;
    pa.L0 = ctx->L0;
    pa.scale = 1.0 / Lp;
    pa.update = update;
    pa.want_red = want_red;
    pa.partials = ctx->partials;
    pa.pin = (!dbl) ? 1 : 0;
    pa.pin_value = ctx->p.psi0 * (double)ctx->ncells;
    pa.pin_values = ctx->nb > 1 ? ctx->pin_values : nullptr;
    pa.zstride = ctx->zstride;
    pa.nz = ctx->nb;
    const int npairs = ctx->three_d ? ctx->n1 / 2 + 1 : 1;
    ProfScope ps(ctx, PASS_PENCIL);
    const int ttx = (ctx->three_d && sizeof(T) == 4) ? pen_tma_tx(Lp, 4) : 0;
    if (ctx->use_tma && ttx > 0 && ctx->L0 % ttx == 0 && tma_ready(ctx, ttx, Lp)) {
        XPFC_LAUNCH(ctx, launch_pencil_tma<T>(Lp, pa, ks, npairs, twp, &ctx->tmS, &ctx->tmW, ctx->dev_err,
                                              ctx->stream, nb));
        return XPFC_OK;
    }
    XPFC_LAUNCH(ctx, launch_pencil<T>(Lp, ctx->three_d ? 2 : 1, pa, ks, npairs, twp, ctx->stream, nb));
    return XPFC_OK;
}

// How many plane chunks the 3-D xy passes take (1: one launch per pass).
// A chunk's slab of S and W stays in L2 from the y-inverse pass through the
// row pass to the y-forward pass, and the chunks run on four auxiliary
// streams, so the passes of neighbouring chunks overlap on the SMs.
// XPFC_XY_CHUNKS overrides the choice.
// Auxiliary streams and events of the chunked xy passes (created once).
static bool ensure_aux(xpfc_ctx *ctx) {
    if (ctx->ev_fork) return true;
    for (int k = 0; k < 4; k++)
        if (cudaStreamCreateWithFlags(&ctx->aux[k], cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&ctx->ev_join[k], cudaEventDisableTiming) != cudaSuccess)
            return false;
    return cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) == cudaSuccess;
}

// The default chunk count (before or without tuning): four chunks for 3-D
// states of at least 32 MB whose slow axis divides by four.
static int xy_default_chunks(const xpfc_ctx *ctx) {
    const size_t slab = ctx->esz * (size_t)ctx->ncells * ctx->nb;
    return (ctx->three_d && ctx->n2 % 4 == 0 && ctx->n2 >= 64 && slab >= ((size_t)32 << 20)) ? 4 : 1;
}

static int xy_chunk_count(xpfc_ctx *ctx) {
    if (ctx->xy_chunks >= 0) return ctx->xy_chunks;
    int c = xy_default_chunks(ctx);
    if (const char *e = getenv("XPFC_XY_CHUNKS")) {
        const int v = atoi(e);
        if (v >= 1 && ctx->n2 % v == 0) c = v;
    }
    if (c > 1 && !ensure_aux(ctx)) c = 1;
    ctx->xy_chunks = c;
    return c;
}

template <typename T>
static int launch_xy_pass(xpfc_ctx *ctx, int want_red, int *nb) {
    const bool dbl = sizeof(T) == 8;
    void *tw0 = twiddle(ctx, ctx->L0, dbl), *tw2 = twiddle(ctx, ctx->n0, dbl);
    if (!tw0 || !tw2) return fail(ctx, XPFC_ENOMEM, "twiddle tables");
    RowArgs ra{};
    ra.nrows = (long long)ctx->n1 * ctx->n2;
    ra.a = ctx->p.a;
    ra.b = ctx->p.b;
    ra.partials = ctx->partials;
    ra.want_red = want_red;
    ra.ref_compat = ctx->p.ref_compat;
    ra.zstride = ctx->zstride;
    ra.nz = ctx->nb;
    if (ctx->three_d) {
        void *tw1 = twiddle(ctx, ctx->n1, dbl);
        if (!tw1) return fail(ctx, XPFC_ENOMEM, "twiddle tables");
        ColArgs cy{};
        cy.in = ctx->S;
        cy.out = ctx->W;
        cy.es = ctx->L0;
        cy.ostride = (long long)ctx->n1 * ctx->L0;
        cy.scale = 1.0;
        cy.ncols = ctx->L0;
        cy.zstride = ctx->zstride;
        cy.nz = ctx->nb;
        const int nch = (want_red || ctx->profiling) ? 1 : xy_chunk_count(ctx);
        if (nch > 1) {
            // chunks of planes (slow index n2), round robin over the auxiliary
            // streams, between a fork and a join on the context's stream
            const int per = ctx->n2 / nch;
            const long long plane = (long long)ctx->n1 * ctx->L0;   // complex elements per plane
            XPFC_CUDA(ctx, cudaEventRecord(ctx->ev_fork, ctx->stream));
            for (int k = 0; k < 4; k++) XPFC_CUDA(ctx, cudaStreamWaitEvent(ctx->aux[k], ctx->ev_fork, 0));
            for (int c = 0; c < nch; c++) {
                cudaStream_t s = ctx->aux[c % 4];
                const long long off = (long long)c * per * plane;
                ColArgs cc = cy;
                cc.in = (const cplx<T> *)ctx->S + off;
                cc.out = (cplx<T> *)ctx->W + off;
                XPFC_LAUNCH(ctx, launch_col<T>(1, ctx->n1, cc, per, tw1, s));
                RowArgs rc = ra;
                rc.in = (const cplx<T> *)ctx->W + off;
                rc.out = (cplx<T> *)ctx->W + off;
                rc.nrows = (long long)ctx->n1 * per;
                rc.scale = 1.0 / ((double)ctx->n0 * ctx->n1);
                XPFC_LAUNCH(ctx, launch_row<T>(ROW_FUSED, ctx->L0, rc, tw0, tw2, s, nullptr));
                cc.in = (const cplx<T> *)ctx->W + off;
                XPFC_LAUNCH(ctx, launch_col<T>(-1, ctx->n1, cc, per, tw1, s));
            }
            for (int k = 0; k < 4; k++) {
                XPFC_CUDA(ctx, cudaEventRecord(ctx->ev_join[k], ctx->aux[k]));
                XPFC_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->ev_join[k], 0));
            }
            return XPFC_OK;
        }
        {
            ProfScope ps(ctx, PASS_COL_INV);
            XPFC_LAUNCH(ctx, launch_col<T>(1, ctx->n1, cy, ctx->n2, tw1, ctx->stream));
        }
        ra.in = ctx->W;
        ra.out = ctx->W;
        ra.scale = 1.0 / ((double)ctx->n0 * ctx->n1);
        {
            ProfScope ps(ctx, PASS_ROW);
            XPFC_LAUNCH(ctx, launch_row<T>(ROW_FUSED, ctx->L0, ra, tw0, tw2, ctx->stream, nb));
        }
        cy.in = ctx->W;
        {
            ProfScope ps(ctx, PASS_COL_FWD);
            XPFC_LAUNCH(ctx, launch_col<T>(-1, ctx->n1, cy, ctx->n2, tw1, ctx->stream));
        }
    } else {
        ra.in = ctx->S;
        ra.out = ctx->W;
        ra.scale = 1.0 / (double)ctx->n0;
        ProfScope ps(ctx, PASS_ROW);
        XPFC_LAUNCH(ctx, launch_row<T>(ROW_FUSED, ctx->L0, ra, tw0, tw2, ctx->stream, nb));
    }
    return XPFC_OK;
}

static bool diag_wantF(const xpfc_ctx *ctx, long long i) {
    const int ts = ctx->p.t_sample;
    if (i == ctx->diag_it0) return ctx->diag_it0 == 0;
    return (ctx->diag_final && i == ctx->diag_fin) || (ts > 0 && i % ts == 0) ||
           (i < ctx->diag_fin && ctx->diag_extra.count(i));
}
static bool diag_wantR(const xpfc_ctx *ctx, long long i) {
    const int ts = ctx->p.t_sample;
    return i < ctx->diag_fin && ts > 0 && i % ts == 0;
}

// A step call in three parts, so that a batch can interleave its groups:
// begin (diagnostics schedule and slots), the iterations [i0, i1), end
// (final free energy, copy of the slots to the host).
static int enqueue_begin(xpfc_ctx *ctx, long long nsteps, bool final_F) {
    const long long it0 = ctx->iteration, fin = it0 + nsteps;
    const int ts = ctx->p.t_sample;
    ctx->diag_it0 = it0;
    ctx->diag_fin = fin;
    ctx->diag_final = final_F;
    std::vector<long long> &its = ctx->diag_its;
    std::map<long long, int> &slot = ctx->diag_slot;
    slot.clear();
    std::set<long long> want;   // in increasing order
    if (diag_wantF(ctx, it0) || diag_wantR(ctx, it0)) want.insert(it0);
    if (ts > 0)
        for (long long i = ((it0 / ts) + 1) * ts; i <= fin; i += ts)
            if (diag_wantF(ctx, i) || diag_wantR(ctx, i)) want.insert(i);
    for (long long i : ctx->diag_extra)
        if (i > it0 && i < fin) want.insert(i);
    if (final_F) want.insert(fin);
    its.assign(want.begin(), want.end());
    for (size_t k = 0; k < its.size(); k++) slot[its[k]] = (int)k;
    // slots: [instance][diagnostics iteration][8]
    const int ns = (int)its.size();
    const int nbi = ctx->nb;
    const long long sstride = 8LL * ns;
    if (ns * nbi > ctx->slots_cap) {
        cudaFree(ctx->slots);
        if (ctx->hslots) cudaFreeHost(ctx->hslots);
        ctx->slots = nullptr;
        ctx->hslots = nullptr;
        ctx->slots_cap = 0;
        XPFC_CUDA(ctx, cudaMalloc(&ctx->slots, sizeof(double) * 8 * ns * nbi));
        XPFC_CUDA(ctx, cudaMallocHost(&ctx->hslots, sizeof(double) * 8 * ns * nbi));
        ctx->slots_cap = ns * nbi;
    }
    if (ns > 0) XPFC_CUDA(ctx, cudaMemsetAsync(ctx->slots, 0, sizeof(double) * 8 * ns * nbi, ctx->stream));
    if (it0 == 0 && slot.count(0))
        XPFC_CUDA(ctx, cudaMemcpy2DAsync(ctx->slots + 8 * slot[0], sizeof(double) * sstride, ctx->init_red,
                                         sizeof(double) * 8, sizeof(double) * NQ_ROW, nbi, cudaMemcpyDeviceToDevice,
                                         ctx->stream));
    return XPFC_OK;
}

// ---------------------------------------------------------------------------
// autotuner of the step's schedule
// ---------------------------------------------------------------------------
// The schedule of a 3-D step: the number of plane chunks of the xy passes
// (1, 2, 4 or 8; chunks run on four auxiliary streams and keep their slab in
// L2 between passes).  Every candidate runs the same kernels on the same
// data, so all give the same bits, and the tuner times them on the solve's
// own first plain iterations: each candidate runs one untimed and TUNE_STEPS
// timed iterations between CUDA events, the fastest is kept for the context
// and remembered for its shape (grid, instances, precision, device) in a
// process-wide table, so later contexts of that shape start with it.
// XPFC_AUTOTUNE=0 keeps the defaults; XPFC_XY_CHUNKS fixes the chunk count.
struct Sched {
    int chunks, tma;
};
static std::mutex g_sched_mu;
static std::map<std::string, Sched> g_sched;
constexpr int TUNE_STEPS = 6;

static std::string sched_key(const xpfc_ctx *ctx) {
    return std::to_string(ctx->n0) + "x" + std::to_string(ctx->n1) + "x" + std::to_string(ctx->n2) + "/" +
           std::to_string(ctx->nb) + "/" + std::to_string(ctx->esz) + "/" + std::to_string(ctx->p.device);
}

static bool autotune_on() {
    static const bool on = [] {
        const char *e = getenv("XPFC_AUTOTUNE");
        return !(e && e[0] == '0');
    }();
    return on;
}

// Chunk counts above one are candidates only for states of at least 32 MB
// (the threshold of the default): a smaller state stays in L2 through the
// xy passes whole, and timing candidates of a small grid amid other solves'
// work (a server) could remember a many-launch schedule for its shape.
static std::vector<Sched> sched_candidates(xpfc_ctx *ctx) {
    std::vector<Sched> out;
    std::vector<int> chunks = {1};
    const size_t slab = ctx->esz * (size_t)ctx->ncells * ctx->nb;
    if (!getenv("XPFC_XY_CHUNKS") && slab >= ((size_t)32 << 20) && ensure_aux(ctx))
        for (int c : {2, 4, 8})
            if (ctx->n2 % c == 0 && ctx->n2 / c >= 8) chunks.push_back(c);
    for (int c : chunks) out.push_back({c, ctx->use_tma});
    return out;
}

static void sched_apply(xpfc_ctx *ctx, Sched s) {
    // chunked xy passes need the auxiliary streams of this context
    ctx->xy_chunks = (s.chunks > 1 && !ensure_aux(ctx)) ? 1 : s.chunks;
    ctx->use_tma = s.tma;
}

// A plain iteration (no diagnostics produced by it or by the next one).
static bool plain_iter(const xpfc_ctx *ctx, long long i) {
    return !(diag_wantF(ctx, i) || diag_wantR(ctx, i) || diag_wantF(ctx, i + 1));
}

template <typename T>
static int plain_step(xpfc_ctx *ctx, long long i) {
    int nb = 0;
    int rc = launch_pencil_pass<T>(ctx, i, 1, 0, &nb);
    if (rc == XPFC_OK) rc = launch_xy_pass<T>(ctx, 0, &nb);
    return rc;
}

// Schedule of the context before its first step: the remembered one for its
// shape, or the defaults.  Returns true when the context still has to tune.
static bool sched_init(xpfc_ctx *ctx) {
    if (ctx->tuned) return false;
    if (!ctx->three_d || !autotune_on() || ctx->profiling || sched_candidates(ctx).size() < 2) {
        ctx->tuned = true;
        return false;
    }
    std::lock_guard<std::mutex> g(g_sched_mu);
    auto it = g_sched.find(sched_key(ctx));
    if (it != g_sched.end()) {
        sched_apply(ctx, it->second);
        ctx->tuned = true;
        return false;
    }
    return true;
}

// Runs the candidates on iterations [i, i + n) (all plain; n = candidates x
// (TUNE_STEPS + 1)) and keeps the fastest.  Returns the next iteration.
template <typename T>
static int autotune(xpfc_ctx *ctx, long long &i) {
    const std::vector<Sched> cand = sched_candidates(ctx);
    std::vector<cudaEvent_t> ev(2 * cand.size(), nullptr);
    for (auto &e : ev) XPFC_CUDA(ctx, cudaEventCreate(&e));
    int rc = XPFC_OK;
    for (size_t c = 0; c < cand.size() && rc == XPFC_OK; c++) {
        sched_apply(ctx, cand[c]);
        rc = plain_step<T>(ctx, i++);   // untimed: first launches, tables, tensor maps
        if (rc != XPFC_OK) break;
        XPFC_CUDA(ctx, cudaEventRecord(ev[2 * c], ctx->stream));
        for (int k = 0; k < TUNE_STEPS && rc == XPFC_OK; k++) rc = plain_step<T>(ctx, i++);
        XPFC_CUDA(ctx, cudaEventRecord(ev[2 * c + 1], ctx->stream));
    }
    if (rc == XPFC_OK) {
        XPFC_CUDA(ctx, cudaEventSynchronize(ev.back()));
        size_t best = 0;
        float best_ms = 0.f;
        for (size_t c = 0; c < cand.size(); c++) {
            float ms = 0.f;
            XPFC_CUDA(ctx, cudaEventElapsedTime(&ms, ev[2 * c], ev[2 * c + 1]));
            if (c == 0 || ms < best_ms) {
                best = c;
                best_ms = ms;
            }
        }
        sched_apply(ctx, cand[best]);
        ctx->tuned = true;
        std::lock_guard<std::mutex> g(g_sched_mu);
        g_sched[sched_key(ctx)] = cand[best];
    }
    for (auto &e : ev) cudaEventDestroy(e);
    return rc;
}

// ---------------------------------------------------------------------------
// step graphs
// ---------------------------------------------------------------------------
// Runs of GRAPH_STEPS plain iterations (after the schedule is tuned) are
// replayed from one captured CUDA graph: the passes of those iterations with
// their programmatic dependences and the fork/join of the chunked xy passes.
// The noise of an iteration depends on its index, which the pencil passes read
// as (device word) + (their position in the graph); a one-thread kernel sets
// the word before each replay.  The graph is built once per context and
// schedule, and dropped when the context takes new params.  XPFC_GRAPH=0
// launches every pass on its own.
constexpr int GRAPH_STEPS = 16;

static bool graphs_on() {
    static const bool on = [] {
        const char *e = getenv("XPFC_GRAPH");
        return !(e && e[0] == '0');
    }();
    return on;
}

__global__ void set_step_base_kernel(long long *p, long long v) { *p = v; }

static void drop_graph(xpfc_ctx *ctx) {
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
    ctx->graph_exec = nullptr;
    ctx->graph_state = 0;
}

// Captures GRAPH_STEPS plain iterations; on any failure the context keeps
// launching pass by pass (graph_state -1).
template <typename T>
static int graph_build(xpfc_ctx *ctx) {
    drop_graph(ctx);
    ctx->graph_state = -1;
    if (!ctx->d_step_base && cudaMalloc(&ctx->d_step_base, sizeof(long long)) != cudaSuccess) {
        ctx->d_step_base = nullptr;
        cudaGetLastError();
        return XPFC_OK;
    }
    const long long l0 = ctx->launches;
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
        cudaGetLastError();
        return XPFC_OK;
    }
    ctx->cap_base = ctx->d_step_base;
    int rc = XPFC_OK;
    for (int j = 0; j < GRAPH_STEPS && rc == XPFC_OK; j++) rc = plain_step<T>(ctx, j);
    ctx->cap_base = nullptr;
    const cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    const long long kernels = ctx->launches - l0;
    ctx->launches = l0;   // a capture launches nothing
    if (rc != XPFC_OK || e != cudaSuccess || !g) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        ctx->err.clear();
        return XPFC_OK;
    }
    const cudaError_t ei = cudaGraphInstantiate(&ctx->graph_exec, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) {
        ctx->graph_exec = nullptr;
        cudaGetLastError();
        return XPFC_OK;
    }
    ctx->graph_state = 1;
    ctx->graph_chunks = ctx->xy_chunks;
    ctx->graph_kernels = kernels;
    return XPFC_OK;
}

// Replays the graph for iterations [i, i + GRAPH_STEPS) when it can.
template <typename T>
static int graph_try(xpfc_ctx *ctx, long long i, long long i1, bool &done) {
    done = false;
    if (!graphs_on() || !ctx->tuned || ctx->profiling || i + GRAPH_STEPS > i1) return XPFC_OK;
    for (long long j = i; j < i + GRAPH_STEPS; j++)
        if (!plain_iter(ctx, j)) return XPFC_OK;
    if (ctx->graph_state == 1 && ctx->graph_chunks != ctx->xy_chunks) drop_graph(ctx);
    if (ctx->graph_state == 0) {
        // the first plain iteration of a context runs pass by pass: it makes
        // the tables, streams and kernel set-up a capture must not create
        if (!ctx->graph_warm) {
            ctx->graph_warm = true;
            return XPFC_OK;
        }
        int rc = graph_build<T>(ctx);
        if (rc != XPFC_OK) return rc;
    }
    if (ctx->graph_state != 1) return XPFC_OK;
    set_step_base_kernel<<<1, 1, 0, ctx->stream>>>(ctx->d_step_base, i);
    XPFC_CUDA(ctx, cudaGetLastError());
    XPFC_CUDA(ctx, cudaGraphLaunch(ctx->graph_exec, ctx->stream));
    ctx->launches += 1 + ctx->graph_kernels;
    done = true;
    return XPFC_OK;
}

template <typename T>
static int enqueue_steps(xpfc_ctx *ctx, long long i0, long long i1) {
    std::map<long long, int> &slot = ctx->diag_slot;
    const int nbi = ctx->nb;
    const long long sstride = 8LL * (long long)ctx->diag_its.size();
    bool tune = sched_init(ctx);
    for (long long i = i0; i < i1; i++) {
        if (tune) {
            // tune on the first run of enough plain iterations
            const long long need = (long long)sched_candidates(ctx).size() * (TUNE_STEPS + 1);
            bool ok = need > 1 && i + need <= i1;
            for (long long j = i; ok && j < i + need; j++) ok = plain_iter(ctx, j);
            if (ok) {
                long long j = i;
                const int rc = autotune<T>(ctx, j);
                if (rc != XPFC_OK) return rc;
                tune = false;
                i = j - 1;
                continue;
            }
        }
        {
            bool replayed = false;
            const int rc = graph_try<T>(ctx, i, i1, replayed);
            if (rc != XPFC_OK) return rc;
            if (replayed) {
                i += GRAPH_STEPS - 1;
                continue;
            }
        }
        const bool red = diag_wantF(ctx, i) || diag_wantR(ctx, i);
        int nb = 0;
        int rc = launch_pencil_pass<T>(ctx, i, 1, red ? 1 : 0, &nb);
        if (rc != XPFC_OK) return rc;
        if (red) {
            ProfScope ps(ctx, PASS_RED);
            XPFC_LAUNCH(ctx, launch_finalize(NQ_PEN, ctx->partials, nb, ctx->slots + 8 * slot[i] + 4, ctx->stream, nbi,
                                             sstride));
        }
        const bool redl = diag_wantF(ctx, i + 1);
        rc = launch_xy_pass<T>(ctx, redl ? 1 : 0, &nb);
        if (rc != XPFC_OK) return rc;
        if (redl) {
            ProfScope ps(ctx, PASS_RED);
            XPFC_LAUNCH(ctx, launch_finalize(NQ_ROW, ctx->partials, nb, ctx->slots + 8 * slot[i + 1], ctx->stream, nbi,
                                             sstride));
        }
    }
    return XPFC_OK;
}

template <typename T>
static int enqueue_end(xpfc_ctx *ctx) {
    std::map<long long, int> &slot = ctx->diag_slot;
    const long long fin = ctx->diag_fin;
    const int ns = (int)ctx->diag_its.size();
    const int nbi = ctx->nb;
    const long long sstride = 8LL * ns;
    if (ctx->diag_final && diag_wantF(ctx, fin)) {
        // the final state's nonlocal term needs its spectrum: diagnostics-only pencil pass
        int nb = 0;
        int rc = launch_pencil_pass<T>(ctx, fin, 0, 1, &nb);
        if (rc != XPFC_OK) return rc;
        XPFC_LAUNCH(ctx, launch_finalize(NQ_PEN, ctx->partials, nb, ctx->slots + 8 * slot[fin] + 4, ctx->stream, nbi,
                                         sstride));
    }
    if (ns > 0)
        XPFC_CUDA(ctx, cudaMemcpyAsync(ctx->hslots, ctx->slots, sizeof(double) * 8 * ns * nbi,
                                       cudaMemcpyDeviceToHost, ctx->stream));
    if (ctx->dev_err)
        XPFC_CUDA(ctx, cudaMemcpyAsync(ctx->herr, ctx->dev_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->iteration = fin;
    ctx->diag_pending = true;
    return XPFC_OK;
}

// Enqueues nsteps iterations with their diagnostics into device slots.
template <typename T>
static int fused_enqueue(xpfc_ctx *ctx, long long nsteps, bool final_F) {
    int rc = enqueue_begin(ctx, nsteps, final_F);
    if (rc == XPFC_OK) rc = enqueue_steps<T>(ctx, ctx->diag_it0, ctx->diag_fin);
    if (rc == XPFC_OK) rc = enqueue_end<T>(ctx);
    return rc;
}

// Diagnostics of instance k from the last step call (stream already synchronised).
static int collect_inst(xpfc_ctx *ctx, int k, xpfc_diag *out, int cap, int *count) {
    if (count) *count = 0;
    if (!ctx->diag_pending) return XPFC_OK;
    if (ctx->herr && *ctx->herr)
        return fail(ctx, XPFC_ETIMEDOUT, "a pencil block gave up waiting for its staged tile (bounded wait)");
    const xpfc_params &p = ctx->inst[k];
    const double N = (double)ctx->ncells;
    const size_t ns = ctx->diag_its.size();
    int produced = 0;
    bool nonfinite = false;
    for (size_t s = 0; s < ns; s++) {
        const long long i = ctx->diag_its[s];
        const double *v = ctx->hslots + 8 * (ns * k + s);
        xpfc_diag d;
        d.iteration = i;
        d.has = 0;
        d.F = d.mean = d.rms = NAN;
        if (diag_wantF(ctx, i)) {
            d.F = p.ff_factor * (0.5 * v[1] - (p.a / 3.0) * v[2] + (p.b / 4.0) * v[3] - 0.5 * v[4] / N);
            d.mean = v[0] / N;
            d.has |= 1;
            if (!std::isfinite(d.F) || !std::isfinite(d.mean)) nonfinite = true;
        }
        if (diag_wantR(ctx, i)) {
            d.rms = std::sqrt(v[5]) / N;
            d.has |= 2;
        }
        if (!d.has) continue;
        if (out && produced < cap) out[produced] = d;
        produced++;
    }
    if (count) *count = (!out || produced < cap) ? produced : cap;
    if (nonfinite) return fail(ctx, XPFC_ENONFINITE, "free energy or mean is not finite");
    return XPFC_OK;
}

extern "C" int xpfc_collect(xpfc_ctx *ctx, xpfc_diag *out, int cap, int *count) {
    if (!ctx) return fail(nullptr, XPFC_EINVAL, "null context");
    XPFC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return collect_inst(ctx, 0, out, cap, count);
}

extern "C" int xpfc_step(xpfc_ctx *ctx, long long nsteps, xpfc_diag *out, int cap, int *count) {
    if (!ctx) return fail(nullptr, XPFC_EINVAL, "null context");
    if (!ctx->initialized) return fail(ctx, XPFC_ESTATE, "xpfc_step before xpfc_initialize");
    if (nsteps < 0) return fail(ctx, XPFC_EINVAL, "nsteps < 0");
    XPFC_CUDA(ctx, cudaSetDevice(ctx->p.device));
    int rc = ctx->esz == 4 ? fused_enqueue<float>(ctx, nsteps, true) : fused_enqueue<double>(ctx, nsteps, true);
    if (rc != XPFC_OK) return rc;
    return xpfc_collect(ctx, out, cap, count);
}

extern "C" int xpfc_step_async(xpfc_ctx *ctx, long long nsteps) {
    if (!ctx) return fail(nullptr, XPFC_EINVAL, "null context");
    if (!ctx->initialized) return fail(ctx, XPFC_ESTATE, "xpfc_step_async before xpfc_initialize");
    if (nsteps < 0) return fail(ctx, XPFC_EINVAL, "nsteps < 0");
    XPFC_CUDA(ctx, cudaSetDevice(ctx->p.device));
    return ctx->esz == 4 ? fused_enqueue<float>(ctx, nsteps, false) : fused_enqueue<double>(ctx, nsteps, false);
}

extern "C" int xpfc_set_profiling(xpfc_ctx *ctx, int enable) {
    if (!ctx) return fail(nullptr, XPFC_EINVAL, "null context");
    drain_profile(ctx);
    ctx->profiling = enable != 0;
    for (int i = 0; i < 8; i++) {
        ctx->prof_ms[i] = 0.0;
        ctx->prof_n[i] = 0;
    }
    if (ctx->profiling && ctx->ev_pool.empty()) {
        ctx->ev_pool.resize(65536);
        for (auto &e : ctx->ev_pool) XPFC_CUDA(ctx, cudaEventCreate(&e));
    }
    return XPFC_OK;
}

extern "C" int xpfc_get_profile(xpfc_ctx *ctx, int pass, double *ms, long long *launches) {
    if (!ctx || pass < 0 || pass >= 8) return fail(ctx, XPFC_EINVAL, "bad argument");
    drain_profile(ctx);
    if (ms) *ms = ctx->prof_ms[pass];
    if (launches) *launches = ctx->prof_n[pass];
    return XPFC_OK;
}

template <typename T>
static int field_to_X(xpfc_ctx *ctx, int k = 0) {
    const bool dbl = sizeof(T) == 8;
    void *Sk = (char *)ctx->S + ctx->esz * (size_t)ctx->ncells * k;
    // an asynchronous read-back may still be copying X to the host
    if (ctx->copy_used) XPFC_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->ev_copied, 0));
    if (!ctx->X) {
        XPFC_CUDA(ctx, cudaMalloc(&ctx->X, ctx->esz * (size_t)ctx->ncells));
        poison(ctx->X, ctx->esz * (size_t)ctx->ncells, ctx->stream);
    }
    void *tw0 = twiddle(ctx, ctx->L0, dbl), *tw2 = twiddle(ctx, ctx->n0, dbl);
    if (!tw0 || !tw2) return fail(ctx, XPFC_ENOMEM, "twiddle tables");
    RowArgs ra{};
    ra.nrows = (long long)ctx->n1 * ctx->n2;
    ra.out = ctx->X;
    if (ctx->three_d) {
        void *tw1 = twiddle(ctx, ctx->n1, dbl);
        ColArgs cy{};
        cy.in = Sk;
        cy.out = ctx->X;
        cy.es = ctx->L0;
        cy.ostride = (long long)ctx->n1 * ctx->L0;
        cy.scale = 1.0;
        cy.ncols = ctx->L0;
        XPFC_LAUNCH(ctx, launch_col<T>(1, ctx->n1, cy, ctx->n2, tw1, ctx->stream));
        ra.in = ctx->X;
        ra.scale = 1.0 / ((double)ctx->n0 * ctx->n1);
    } else {
        ra.in = Sk;
        ra.scale = 1.0 / (double)ctx->n0;
    }
    XPFC_LAUNCH(ctx, launch_row<T>(ROW_INV, ctx->L0, ra, tw0, tw2, ctx->stream, nullptr));
    return XPFC_OK;
}

extern "C" int xpfc_get_field(xpfc_ctx *ctx, double *host_psi) {
    if (!ctx || !host_psi) return fail(ctx, XPFC_EINVAL, "null argument");
    if (!ctx->initialized) return fail(ctx, XPFC_ESTATE, "no field before xpfc_initialize");
    XPFC_CUDA(ctx, cudaSetDevice(ctx->p.device));
    int rc = ctx->esz == 4 ? field_to_X<float>(ctx) : field_to_X<double>(ctx);
    if (rc != XPFC_OK) return rc;
    const size_t n = (size_t)ctx->ncells;
    rc = host_stage(ctx, ctx->esz * n);
    if (rc != XPFC_OK) return rc;
    XPFC_CUDA(ctx, cudaMemcpyAsync(ctx->hstage, ctx->X, ctx->esz * n, cudaMemcpyDeviceToHost, ctx->stream));
    XPFC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (ctx->esz == 4) {
        widen((const float *)ctx->hstage, host_psi, n);
    } else {
        memcpy(host_psi, ctx->hstage, sizeof(double) * n);
    }
    return XPFC_OK;
}

extern "C" int xpfc_get_field_device_f32(xpfc_ctx *ctx, float *dev_out) {
    if (!ctx || !dev_out) return fail(ctx, XPFC_EINVAL, "null argument");
    if (!ctx->initialized) return fail(ctx, XPFC_ESTATE, "no field before xpfc_initialize");
    XPFC_CUDA(ctx, cudaSetDevice(ctx->p.device));
    int rc = ctx->esz == 4 ? field_to_X<float>(ctx) : field_to_X<double>(ctx);
    if (rc != XPFC_OK) return rc;
    const long long n = ctx->ncells;
    if (ctx->esz == 4)
        XPFC_CUDA(ctx, cudaMemcpyAsync(dev_out, ctx->X, sizeof(float) * n, cudaMemcpyDeviceToDevice, ctx->stream));
    else
        XPFC_LAUNCH(ctx, launch_convert_d2f((const double *)ctx->X, dev_out, n, ctx->stream));
    XPFC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return XPFC_OK;
}

extern "C" int xpfc_get_field_async(xpfc_ctx *ctx) {
    if (!ctx) return fail(nullptr, XPFC_EINVAL, "null context");
    if (!ctx->initialized) return fail(ctx, XPFC_ESTATE, "no field before xpfc_initialize");
    XPFC_CUDA(ctx, cudaSetDevice(ctx->p.device));
    if (!ctx->copy_stream) {
        XPFC_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
        XPFC_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_x_ready, cudaEventDisableTiming));
        XPFC_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_copied, cudaEventDisableTiming));
        XPFC_CUDA(ctx, cudaMallocHost(&ctx->hfield, ctx->esz * (size_t)ctx->ncells));
    }
    // a read-back that was never collected is dropped; its copy finishes first
    int rc = ctx->esz == 4 ? field_to_X<float>(ctx) : field_to_X<double>(ctx);
    if (rc != XPFC_OK) return rc;
    XPFC_CUDA(ctx, cudaEventRecord(ctx->ev_x_ready, ctx->stream));
    XPFC_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_x_ready, 0));
    XPFC_CUDA(ctx, cudaMemcpyAsync(ctx->hfield, ctx->X, ctx->esz * (size_t)ctx->ncells, cudaMemcpyDeviceToHost,
                                   ctx->copy_stream));
    XPFC_CUDA(ctx, cudaEventRecord(ctx->ev_copied, ctx->copy_stream));
    ctx->copy_used = true;
    ctx->field_pending = true;
    ctx->field_iter = ctx->iteration;
    return XPFC_OK;
}

extern "C" int xpfc_get_field_wait(xpfc_ctx *ctx, double *host_psi, long long *iteration) {
    if (!ctx || !host_psi) return fail(ctx, XPFC_EINVAL, "null argument");
    if (!ctx->field_pending) return fail(ctx, XPFC_ESTATE, "no read-back requested (xpfc_get_field_async)");
    XPFC_CUDA(ctx, cudaEventSynchronize(ctx->ev_copied));
    const size_t n = (size_t)ctx->ncells;
    if (ctx->esz == 4) widen((const float *)ctx->hfield, host_psi, n);
    else memcpy(host_psi, ctx->hfield, sizeof(double) * n);
    if (iteration) *iteration = ctx->field_iter;
    ctx->field_pending = false;
    return XPFC_OK;
}

// ---------------------------------------------------------------------------
// state snapshots: the fused state (S and W) at full precision
// ---------------------------------------------------------------------------
namespace {
struct SnapHeader {
    char magic[8];            // "XPFCSNP1"
    int32_t esz, nb, Mx, My, Mz, narrays;   // S, W (and the kept spectrum)
    int64_t iteration;
    int64_t bytes;            // bytes of S (and of W)
    double psi0;
};
}  // namespace

extern "C" int xpfc_save_state(xpfc_ctx *ctx, const char *path) {
    if (!ctx || !path) return fail(ctx, XPFC_EINVAL, "null argument");
    if (!ctx->initialized) return fail(ctx, XPFC_ESTATE, "no state before xpfc_initialize");
    XPFC_CUDA(ctx, cudaSetDevice(ctx->p.device));
    const size_t bytes = ctx->esz * (size_t)ctx->ncells * ctx->nb;
    const int narr = ctx->spec ? 3 : 2;
    int rc = host_stage(ctx, narr * bytes);
    if (rc != XPFC_OK) return rc;
    char *h = static_cast<char *>(ctx->hstage);
    XPFC_CUDA(ctx, cudaMemcpyAsync(h, ctx->S, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    XPFC_CUDA(ctx, cudaMemcpyAsync(h + bytes, ctx->W, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    if (ctx->spec)
        XPFC_CUDA(ctx, cudaMemcpyAsync(h + 2 * bytes, ctx->Shat, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    XPFC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    SnapHeader hd{};
    memcpy(hd.magic, "XPFCSNP1", 8);
    hd.esz = (int32_t)ctx->esz;
    hd.nb = ctx->nb;
    hd.Mx = ctx->p.Mx;
    hd.My = ctx->p.My;
    hd.Mz = ctx->p.Mz;
    hd.iteration = ctx->iteration;
    hd.bytes = (int64_t)bytes;
    hd.narrays = narr;
    hd.psi0 = ctx->p.psi0;
    FILE *f = fopen(path, "wb");
    if (!f) return fail(ctx, XPFC_EIO, std::string("cannot open ") + path);
    const bool ok = fwrite(&hd, sizeof(hd), 1, f) == 1 && fwrite(h, 1, narr * bytes, f) == narr * bytes;
    if (fclose(f) != 0 || !ok) return fail(ctx, XPFC_EIO, std::string("write failed: ") + path);
    return XPFC_OK;
}

extern "C" int xpfc_load_state(xpfc_ctx *ctx, const char *path) {
    if (!ctx || !path) return fail(ctx, XPFC_EINVAL, "null argument");
    XPFC_CUDA(ctx, cudaSetDevice(ctx->p.device));
    FILE *f = fopen(path, "rb");
    if (!f) return fail(ctx, XPFC_EIO, std::string("cannot open ") + path);
    SnapHeader hd{};
    const size_t bytes = ctx->esz * (size_t)ctx->ncells * ctx->nb;
    if (fread(&hd, sizeof(hd), 1, f) != 1 || memcmp(hd.magic, "XPFCSNP1", 8) != 0) {
        fclose(f);
        return fail(ctx, XPFC_EIO, std::string("not a state snapshot: ") + path);
    }
    const int narr = ctx->spec ? 3 : 2;
    if (hd.esz != (int32_t)ctx->esz || hd.nb != ctx->nb || hd.Mx != ctx->p.Mx || hd.My != ctx->p.My ||
        hd.Mz != ctx->p.Mz || hd.bytes != (int64_t)bytes || hd.narrays != narr) {
        fclose(f);
        return fail(ctx, XPFC_EINVAL, "the snapshot's grid, precision or instance count differs from the context's");
    }
    int rc = host_stage(ctx, narr * bytes);
    if (rc != XPFC_OK) {
        fclose(f);
        return rc;
    }
    char *h = static_cast<char *>(ctx->hstage);
    // the staging buffer may still feed an upload enqueued earlier
    XPFC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const bool ok = fread(h, 1, narr * bytes, f) == narr * bytes;
    fclose(f);
    if (!ok) return fail(ctx, XPFC_EIO, std::string("truncated snapshot: ") + path);
    XPFC_CUDA(ctx, cudaMemcpyAsync(ctx->S, h, bytes, cudaMemcpyHostToDevice, ctx->stream));
    XPFC_CUDA(ctx, cudaMemcpyAsync(ctx->W, h + bytes, bytes, cudaMemcpyHostToDevice, ctx->stream));
    if (ctx->spec)
        XPFC_CUDA(ctx, cudaMemcpyAsync(ctx->Shat, h + 2 * bytes, bytes, cudaMemcpyHostToDevice, ctx->stream));
    XPFC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->iteration = hd.iteration;
    ctx->initialized = true;
    ctx->diag_pending = false;
    return XPFC_OK;
}

// ---------------------------------------------------------------------------
// staged API (FP64, reference semantics)
// ---------------------------------------------------------------------------
#define XPFC_BUF(ctx, var, id)                                                           \
    double *var = staged_buf(ctx, id);                                                   \
    if (!var) return fail(ctx, (id) < 0 || (id) >= XPFC_NBUF ? XPFC_EINVAL : XPFC_ENOMEM, \
                          "bad or unallocatable buffer id " + std::to_string(id))

static int sync_or_fail(xpfc_ctx *ctx) {
    XPFC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return XPFC_OK;
}

extern "C" int xpfc_upload(xpfc_ctx *ctx, int buf, const double *host) {
    if (!ctx || !host) return fail(ctx, XPFC_EINVAL, "null argument");
    XPFC_BUF(ctx, d, buf);
    XPFC_CUDA(ctx, cudaMemcpyAsync(d, host, sizeof(double) * ctx->ncells, cudaMemcpyHostToDevice, ctx->stream));
    return sync_or_fail(ctx);
}

extern "C" int xpfc_download(xpfc_ctx *ctx, int buf, double *host) {
    if (!ctx || !host) return fail(ctx, XPFC_EINVAL, "null argument");
    XPFC_BUF(ctx, d, buf);
    XPFC_CUDA(ctx, cudaMemcpyAsync(host, d, sizeof(double) * ctx->ncells, cudaMemcpyDeviceToHost, ctx->stream));
    return sync_or_fail(ctx);
}

extern "C" int xpfc_download_spectrum(xpfc_ctx *ctx, int buf, double *host_half) {
    if (!ctx || !host_half) return fail(ctx, XPFC_EINVAL, "null argument");
    XPFC_BUF(ctx, d, buf);
    std::vector<double> pk(ctx->ncells);
    XPFC_CUDA(ctx, cudaMemcpyAsync(pk.data(), d, sizeof(double) * ctx->ncells, cudaMemcpyDeviceToHost, ctx->stream));
    int rc = sync_or_fail(ctx);
    if (rc != XPFC_OK) return rc;
    const int L0 = ctx->L0, n1 = ctx->n1, n2 = ctx->n2, H = L0 + 1;
    for (int i2 = 0; i2 < n2; i2++)
        for (int i1 = 0; i1 < n1; i1++) {
            const size_t row = ((size_t)i2 * n1 + i1);
            const double *pr = pk.data() + 2 * row * L0;
            double *o = host_half + 2 * row * H;
            for (int k = 1; k < L0; k++) {
                o[2 * k] = pr[2 * k];
                o[2 * k + 1] = pr[2 * k + 1];
            }
            const int j1 = (n1 - i1) % n1, j2 = (n2 - i2) % n2;
            const double *pm = pk.data() + 2 * ((size_t)j2 * n1 + j1) * L0;
            const double Pr = pr[0], Pi = pr[1], Mr = pm[0], Mi = pm[1];
            // X0 = (P + conj Pm)/2, XN = -i (P - conj Pm)/2
            o[0] = 0.5 * (Pr + Mr);
            o[1] = 0.5 * (Pi - Mi);
            o[2 * L0] = 0.5 * (Pi + Mi);
            o[2 * L0 + 1] = -0.5 * (Pr - Mr);
        }
    return XPFC_OK;
}

extern "C" int xpfc_copy(xpfc_ctx *ctx, int src, int dst) {
    if (!ctx) return fail(nullptr, XPFC_EINVAL, "null context");
    XPFC_BUF(ctx, s, src);
    XPFC_BUF(ctx, d, dst);
    if (s != d)
        XPFC_CUDA(ctx, cudaMemcpyAsync(d, s, sizeof(double) * ctx->ncells, cudaMemcpyDeviceToDevice, ctx->stream));
    return sync_or_fail(ctx);
}

extern "C" int xpfc_fft(xpfc_ctx *ctx, int buf, int direction) {
    if (!ctx || (direction != XPFC_FORWARD && direction != XPFC_INVERSE)) return fail(ctx, XPFC_EINVAL, "bad argument");
    XPFC_BUF(ctx, d, buf);
    int rc = fft_full<double>(ctx, d, direction);
    if (rc != XPFC_OK) return rc;
    return sync_or_fail(ctx);
}

extern "C" int xpfc_power_functions(xpfc_ctx *ctx, int in, int out, int pw) {
    if (!ctx || pw < 2 || pw > 4) return fail(ctx, XPFC_EINVAL, "power must be 2, 3 or 4");
    XPFC_BUF(ctx, s, in);
    XPFC_BUF(ctx, d, out);
    XPFC_LAUNCH(ctx, launch_power<double>(s, d, ctx->ncells, pw, ctx->p.ref_compat, ctx->stream));
    return sync_or_fail(ctx);
}

extern "C" int xpfc_scaling_step(xpfc_ctx *ctx, int buf) {
    if (!ctx) return fail(nullptr, XPFC_EINVAL, "null context");
    XPFC_BUF(ctx, d, buf);
    XPFC_LAUNCH(ctx, launch_scale<double>(d, ctx->ncells, 1.0 / (double)ctx->ncells, ctx->stream));
    return sync_or_fail(ctx);
}

extern "C" int xpfc_copy_matrix(xpfc_ctx *ctx, int in, int out) {
    // copy_matrix.cu:34-49 keeps the real part; the real buffers here hold only it
    return xpfc_copy(ctx, in, out);
}

static int kspace_op(xpfc_ctx *ctx, int op, int out, int a1, int a2, int a3, int a4) {
    if (out == a1 || out == a2 || out == a3 || out == a4)
        return fail(ctx, XPFC_EINVAL, "k-space stages need an output buffer distinct from their inputs");
    XPFC_BUF(ctx, o, out);
    XPFC_BUF(ctx, x1, a1);
    double *x2 = a2 >= 0 ? staged_buf(ctx, a2) : nullptr;
    double *x3 = a3 >= 0 ? staged_buf(ctx, a3) : nullptr;
    double *x4 = a4 >= 0 ? staged_buf(ctx, a4) : nullptr;
    if ((a2 >= 0 && !x2) || (a3 >= 0 && !x3) || (a4 >= 0 && !x4)) return fail(ctx, XPFC_EINVAL, "bad buffer id");
    KSpace ks = make_kspace(ctx, true);
    XPFC_LAUNCH(ctx, launch_kspace<double>(op, ks, ctx->p.a, ctx->p.b, o, x1, x2, x3, x4, ctx->stream));
    return sync_or_fail(ctx);
}

extern "C" int xpfc_convolve_fields(xpfc_ctx *ctx, int psi_k, int out) {
    if (!ctx) return fail(nullptr, XPFC_EINVAL, "null context");
    return kspace_op(ctx, KOP_CONVOLVE, out, psi_k, -1, -1, -1);
}

extern "C" int xpfc_euler_step(xpfc_ctx *ctx, int n, int psi_kp1, int psi_k, int psi2_k, int psi3_k) {
    (void)n;
    if (!ctx) return fail(nullptr, XPFC_EINVAL, "null context");
    return kspace_op(ctx, KOP_EULER, psi_kp1, psi_k, psi2_k, psi3_k, -1);
}

static int reduce_sum(xpfc_ctx *ctx, const double *psi, const double *p2, const double *p3, const double *p4,
                      const double *convl, int square, double *result) {
    int nb = 0;
    XPFC_LAUNCH(ctx, launch_density<double>(psi, p2, p3, p4, convl, ctx->ncells, ctx->p.a, ctx->p.b, square,
                                            ctx->p.ref_compat, ctx->partials, ctx->stream, &nb));
    XPFC_LAUNCH(ctx, launch_finalize(1, ctx->partials, nb, ctx->init_red + 4, ctx->stream));
    XPFC_CUDA(ctx, cudaMemcpyAsync(result, ctx->init_red + 4, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    return sync_or_fail(ctx);
}

extern "C" int xpfc_FE_calc(xpfc_ctx *ctx, int n, int psi, int psi2, int psi3, int psi4, int convl_r, double *F) {
    (void)n;
    if (!ctx || !F) return fail(ctx, XPFC_EINVAL, "null argument");
    XPFC_BUF(ctx, a, psi);
    XPFC_BUF(ctx, b2, psi2);
    XPFC_BUF(ctx, b3, psi3);
    XPFC_BUF(ctx, b4, psi4);
    XPFC_BUF(ctx, c, convl_r);
    double s = 0.0;
    int rc = reduce_sum(ctx, a, b2, b3, b4, c, 0, &s);
    if (rc != XPFC_OK) return rc;
    *F = s * ctx->p.ff_factor;
    if (!std::isfinite(*F)) return fail(ctx, XPFC_ENONFINITE, "free energy is not finite");
    return XPFC_OK;
}

extern "C" int xpfc_Avg_calc(xpfc_ctx *ctx, int buf, double *mean) {
    if (!ctx || !mean) return fail(ctx, XPFC_EINVAL, "null argument");
    XPFC_BUF(ctx, a, buf);
    double s = 0.0;
    int rc = reduce_sum(ctx, a, nullptr, nullptr, nullptr, nullptr, 0, &s);
    if (rc != XPFC_OK) return rc;
    *mean = s / (double)ctx->ncells;
    return XPFC_OK;
}

extern "C" int xpfc_sse_calculation(xpfc_ctx *ctx, int n, int psi_kp1, int psi_k, int psi2_k, int psi3_k,
                                    double *rms) {
    (void)n;
    if (!ctx || !rms) return fail(ctx, XPFC_EINVAL, "null argument");
    int rc = kspace_op(ctx, KOP_RESIDUAL, XPFC_BUF_RES, psi_kp1, psi_k, psi2_k, psi3_k);
    if (rc != XPFC_OK) return rc;
    double *res = staged_buf(ctx, XPFC_BUF_RES);
    rc = fft_full<double>(ctx, res, XPFC_INVERSE);
    if (rc != XPFC_OK) return rc;
    XPFC_LAUNCH(ctx, launch_scale<double>(res, ctx->ncells, 1.0 / (double)ctx->ncells, ctx->stream));
    double s = 0.0;
    rc = reduce_sum(ctx, res, nullptr, nullptr, nullptr, nullptr, 1, &s);
    if (rc != XPFC_OK) return rc;
    *rms = std::sqrt(s / (double)ctx->ncells);   // sum_reduction.cu:77
    return XPFC_OK;
}

// ---------------------------------------------------------------------------
// batched sweeps: groups of instances that differ only in psi0, peaks, seeds
// and initial fields share one context whose launches cover all of them
// ---------------------------------------------------------------------------
struct xpfc_batch {
    std::vector<xpfc_ctx *> groups;
    std::vector<std::pair<int, int>> where;   // instance -> (group, index in group)
    std::string err;
};

static int bfail(xpfc_batch *b, int code, const std::string &m) {
    if (b) b->err = m;
    else set_thread_error(m);
    return code;
}

// params that must agree within a group
static bool same_group(const xpfc_params &a, const xpfc_params &b) {
    return a.Mx == b.Mx && a.My == b.My && a.Mz == b.Mz && a.Lx == b.Lx && a.Ly == b.Ly && a.Lz == b.Lz &&
           a.a == b.a && a.b == b.b && a.eps == b.eps && a.Mo == b.Mo && a.dt == b.dt && a.t_sample == b.t_sample &&
           a.precision == b.precision && a.ref_compat == b.ref_compat && a.noise_amp == b.noise_amp &&
           a.device == b.device && a.stream == b.stream;
}

extern "C" int xpfc_batch_create(const xpfc_params *ps, int n, xpfc_batch **out) {
    if (!ps || !out || n < 1) return bfail(nullptr, XPFC_EINVAL, "null argument or n < 1");
    *out = nullptr;
    for (int i = 0; i < n; i++) {
        const xpfc_params &p = ps[i];
        const bool cubic = p.Lx == p.Ly && (p.Mz == 1 || p.Lx == p.Lz);
        if (!cubic) return bfail(nullptr, XPFC_EINVAL, "batched instances need equal box lengths on every axis");
        if (check_params(&p) != XPFC_OK)
            return bfail(nullptr, XPFC_EINVAL, "instance " + std::to_string(i) + ": " + thread_error());
    }
    // group by shared params, in order of first appearance
    std::vector<std::vector<int>> members;
    std::vector<int> gid(n, -1);
    for (int i = 0; i < n; i++) {
        for (size_t g = 0; g < members.size() && gid[i] < 0; g++)
            if (same_group(ps[members[g][0]], ps[i])) gid[i] = (int)g;
        if (gid[i] < 0) {
            gid[i] = (int)members.size();
            members.emplace_back();
        }
        members[gid[i]].push_back(i);
    }
    xpfc_batch *b = new xpfc_batch();
    b->where.resize(n);
    for (size_t g = 0; g < members.size(); g++) {
        std::vector<xpfc_params> gp;
        for (size_t k = 0; k < members[g].size(); k++) {
            gp.push_back(ps[members[g][k]]);
            b->where[members[g][k]] = {(int)g, (int)k};
        }
        xpfc_ctx *ctx = nullptr;
        const int rc = create_group(gp.data(), (int)gp.size(), &ctx);
        if (rc != XPFC_OK) {
            const std::string m = thread_error();
            xpfc_batch_destroy(b);
            return bfail(nullptr, rc, "group " + std::to_string(g) + ": " + m);
        }
        b->groups.push_back(ctx);
    }
    *out = b;
    return XPFC_OK;
}

extern "C" int xpfc_batch_destroy(xpfc_batch *b) {
    if (!b) return XPFC_OK;
    for (xpfc_ctx *c : b->groups) xpfc_destroy(c);
    delete b;
    return XPFC_OK;
}

extern "C" const char *xpfc_batch_last_error(const xpfc_batch *b) { return b ? b->err.c_str() : thread_error(); }
extern "C" int xpfc_batch_size(const xpfc_batch *b) { return b ? (int)b->where.size() : 0; }
extern "C" int xpfc_batch_groups(const xpfc_batch *b) { return b ? (int)b->groups.size() : 0; }
extern "C" int xpfc_batch_group_of(const xpfc_batch *b, int i) {
    return (b && i >= 0 && i < (int)b->where.size()) ? b->where[i].first : -1;
}

// sync: wait for the set-up on the context's stream before returning (the
// server's merged groups skip it; their steps are ordered after it anyway)
static int init_group(xpfc_ctx *ctx, const std::vector<const double *> &fields, bool sync = true) {
    XPFC_CUDA(ctx, cudaSetDevice(ctx->p.device));
    const size_t n = (size_t)ctx->ncells, nb = (size_t)ctx->nb;
    int rc = XPFC_OK;
    bool need_host = false;
    for (size_t k = 0; k < nb; k++) need_host |= fields[k] != nullptr || !ic_on_device(ctx->inst[k]);
    std::unique_lock<std::mutex> up(upload_mu, std::defer_lock);
    double *h = nullptr;
    if (need_host) {
        up.lock();
        h = (double *)upload_pool(sizeof(double) * n * nb);
        if (!h) return fail(ctx, XPFC_ENOMEM, "pinned upload staging");
    }
    // host fields (given, or the VTK restart) go up in one copy per run of
    // consecutive instances; the other generators run on the device.  Given
    // fields are staged on up to 16 threads, one field per thread.
    std::vector<char> on_dev(nb, 0);
    std::vector<size_t> given;
    for (size_t k = 0; k < nb; k++) {
        if (fields[k]) {
            given.push_back(k);
        } else if (ic_on_device(ctx->inst[k])) {
            on_dev[k] = 1;
        } else {
            rc = build_initial_field(&ctx->inst[k], h + k * n);
            if (rc != XPFC_OK) return fail(ctx, rc, thread_error());
        }
    }
    if (given.size() == 1) {
        stage_and_pin(h + given[0] * n, fields[given[0]], n, ctx->inst[given[0]]);
    } else if (!given.empty()) {
        std::atomic<size_t> next{0};
        auto work = [&] {
            for (size_t i; (i = next.fetch_add(1)) < given.size();) {
                const size_t k = given[i];
                stage_and_pin(h + k * n, fields[k], n, ctx->inst[k], false);
            }
        };
        std::vector<std::thread> th;
        const size_t nt = std::min<size_t>(16, given.size());
        for (size_t w = 0; w < nt; w++) th.emplace_back(work);
        for (auto &t : th) t.join();
    }
    double *dpsi = nullptr;
    XPFC_CUDA(ctx, cudaMallocAsync((void **)&dpsi, sizeof(double) * n * nb, ctx->stream));
    cudaError_t e = cudaSuccess;
    for (size_t k = 0; k < nb && e == cudaSuccess && rc == XPFC_OK;) {
        size_t k1 = k + 1;
        while (k1 < nb && on_dev[k1] == on_dev[k]) k1++;
        if (on_dev[k]) {
            for (size_t j = k; j < k1 && rc == XPFC_OK; j++) {
                std::string why;
                rc = enqueue_initial_field(ctx->inst[j], dpsi + j * n, ctx->partials, ctx->stream, &why);
                if (rc != XPFC_OK) fail(ctx, rc, why);
            }
        } else {
            e = cudaMemcpyAsync(dpsi + k * n, h + k * n, sizeof(double) * n * (k1 - k), cudaMemcpyHostToDevice,
                                ctx->stream);
        }
        k = k1;
    }
    if (e != cudaSuccess) rc = fail(ctx, XPFC_ECUDA, std::string("cudaMemcpyAsync: ") + cudaGetErrorString(e));
    if (need_host) {
        // the uploads from the shared staging are complete before it is released
        const cudaError_t se = cudaStreamSynchronize(ctx->stream);
        up.unlock();
        if (se != cudaSuccess && rc == XPFC_OK)
            rc = fail(ctx, XPFC_ECUDA, std::string("upload: ") + cudaGetErrorString(se));
    }
    if (rc == XPFC_OK) rc = ctx->esz == 4 ? init_fused<float>(ctx, dpsi) : init_fused<double>(ctx, dpsi);
    cudaFreeAsync(dpsi, ctx->stream);
    if (rc != XPFC_OK) return rc;
    if (sync) XPFC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->iteration = 0;
    ctx->initialized = true;
    ctx->diag_pending = false;
    return XPFC_OK;
}

extern "C" int xpfc_batch_initialize(xpfc_batch *b, const double *const *fields) {
    if (!b) return bfail(nullptr, XPFC_EINVAL, "null batch");
    for (size_t g = 0; g < b->groups.size(); g++) {
        xpfc_ctx *ctx = b->groups[g];
        std::vector<const double *> f(ctx->nb, nullptr);
        if (fields)
            for (size_t i = 0; i < b->where.size(); i++)
                if (b->where[i].first == (int)g) f[b->where[i].second] = fields[i];
        const int rc = init_group(ctx, f);
        if (rc != XPFC_OK) return bfail(b, rc, "group " + std::to_string(g) + ": " + ctx->err);
    }
    return XPFC_OK;
}

extern "C" int xpfc_batch_step_async(xpfc_batch *b, long long nsteps) {
    if (!b) return bfail(nullptr, XPFC_EINVAL, "null batch");
    if (nsteps < 0) return bfail(b, XPFC_EINVAL, "nsteps < 0");
    for (xpfc_ctx *ctx : b->groups)
        if (!ctx->initialized) return bfail(b, XPFC_ESTATE, "xpfc_batch_step before xpfc_batch_initialize");
    // the groups' iterations go out in rounds of kChunk, so that every
    // group's stream holds work while the host enqueues (a stream's queue of
    // pending launches is finite: filling one group's first would hold the
    // host there until that group has nearly finished)
    constexpr long long kChunk = 16;
    const size_t ng = b->groups.size();
    for (size_t g = 0; g < ng; g++) {
        xpfc_ctx *ctx = b->groups[g];
        XPFC_CUDA(b, cudaSetDevice(ctx->p.device));
        const int rc = enqueue_begin(ctx, nsteps, true);
        if (rc != XPFC_OK) return bfail(b, rc, "group " + std::to_string(g) + ": " + ctx->err);
    }
    for (long long c = 0; c < nsteps; c += kChunk) {
        for (size_t g = 0; g < ng; g++) {
            xpfc_ctx *ctx = b->groups[g];
            const long long i0 = ctx->diag_it0 + c, i1 = std::min(ctx->diag_it0 + c + kChunk, ctx->diag_fin);
            XPFC_CUDA(b, cudaSetDevice(ctx->p.device));
            const int rc = ctx->esz == 4 ? enqueue_steps<float>(ctx, i0, i1) : enqueue_steps<double>(ctx, i0, i1);
            if (rc != XPFC_OK) return bfail(b, rc, "group " + std::to_string(g) + ": " + ctx->err);
        }
    }
    for (size_t g = 0; g < ng; g++) {
        xpfc_ctx *ctx = b->groups[g];
        XPFC_CUDA(b, cudaSetDevice(ctx->p.device));
        const int rc = ctx->esz == 4 ? enqueue_end<float>(ctx) : enqueue_end<double>(ctx);
        if (rc != XPFC_OK) return bfail(b, rc, "group " + std::to_string(g) + ": " + ctx->err);
    }
    return XPFC_OK;
}

extern "C" int xpfc_batch_step(xpfc_batch *b, long long nsteps) {
    const int rc = xpfc_batch_step_async(b, nsteps);
    if (rc != XPFC_OK) return rc;
    for (xpfc_ctx *ctx : b->groups) XPFC_CUDA(b, cudaStreamSynchronize(ctx->stream));
    return XPFC_OK;
}

extern "C" int xpfc_batch_collect(xpfc_batch *b, int i, xpfc_diag *out, int cap, int *count) {
    if (!b) return bfail(nullptr, XPFC_EINVAL, "null batch");
    if (i < 0 || i >= (int)b->where.size()) return bfail(b, XPFC_EINVAL, "instance index out of range");
    xpfc_ctx *ctx = b->groups[b->where[i].first];
    XPFC_CUDA(b, cudaStreamSynchronize(ctx->stream));
    const int rc = collect_inst(ctx, b->where[i].second, out, cap, count);
    if (rc != XPFC_OK) b->err = "instance " + std::to_string(i) + ": " + ctx->err;
    return rc;
}

extern "C" int xpfc_batch_get_field(xpfc_batch *b, int i, double *host_psi) {
    if (!b || !host_psi) return bfail(b, XPFC_EINVAL, "null argument");
    if (i < 0 || i >= (int)b->where.size()) return bfail(b, XPFC_EINVAL, "instance index out of range");
    xpfc_ctx *ctx = b->groups[b->where[i].first];
    if (!ctx->initialized) return bfail(b, XPFC_ESTATE, "no field before xpfc_batch_initialize");
    const int k = b->where[i].second;
    XPFC_CUDA(b, cudaSetDevice(ctx->p.device));
    int rc = ctx->esz == 4 ? field_to_X<float>(ctx, k) : field_to_X<double>(ctx, k);
    if (rc != XPFC_OK) return bfail(b, rc, ctx->err);
    const size_t n = (size_t)ctx->ncells;
    rc = host_stage(ctx, ctx->esz * n);
    if (rc != XPFC_OK) return bfail(b, rc, ctx->err);
    XPFC_CUDA(b, cudaMemcpyAsync(ctx->hstage, ctx->X, ctx->esz * n, cudaMemcpyDeviceToHost, ctx->stream));
    XPFC_CUDA(b, cudaStreamSynchronize(ctx->stream));
    if (ctx->esz == 4) {
        widen((const float *)ctx->hstage, host_psi, n);
    } else {
        memcpy(host_psi, ctx->hstage, sizeof(double) * n);
    }
    return XPFC_OK;
}

#include "xpfc_server.inc"
