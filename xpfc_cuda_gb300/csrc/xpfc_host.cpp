// xpfc_host.cpp -- host-side boundary of libxpfc: the pfc.input deck, VTK
// files, initial conditions and mean pinning.  FP64, plain C++; compiled with
// -ffp-contract=off so x86 and aarch64 hosts produce identical fields.
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/xpfc.h"
#include "xpfc_host.h"

namespace xpfc {

static thread_local std::string g_err;
void set_thread_error(const std::string &m) { g_err = m; }
const char *thread_error() { return g_err.c_str(); }

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11) and Box-Muller, host side.  The same
// counters as the device noise: (index lo, index hi, stream lo, stream hi).
// ---------------------------------------------------------------------------
static void philox(const uint32_t c_in[4], const uint32_t k_in[2], uint32_t out[4]) {
    uint32_t c0 = c_in[0], c1 = c_in[1], c2 = c_in[2], c3 = c_in[3], k0 = k_in[0], k1 = k_in[1];
    for (int r = 0; r < 10; r++) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0, hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

void gauss_pair(uint64_t seed, uint64_t stream, uint64_t index, double *g0, double *g1) {
    const uint32_t c[4] = {(uint32_t)index, (uint32_t)(index >> 32), (uint32_t)stream, (uint32_t)(stream >> 32)};
    const uint32_t k[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t o[4];
    philox(c, k, o);
    const double u1 = ((double)o[0] + 1.0) * 2.3283064365386963e-10;
    const double u2 = (double)o[1] * 2.3283064365386963e-10;
    const double r = std::sqrt(-2.0 * std::log(u1));
    *g0 = r * std::cos(2.0 * M_PI * u2);
    *g1 = r * std::sin(2.0 * M_PI * u2);
}

// ---------------------------------------------------------------------------
// pfc.input (read_input.cu:8-121)
// ---------------------------------------------------------------------------
static bool read_line(FILE *f, std::string &out) {
    out.clear();
    int ch;
    bool any = false;
    while ((ch = fgetc(f)) != EOF) {
        any = true;
        if (ch == '\n') break;
        out.push_back((char)ch);
    }
    return any;
}

static bool parse_nums(const std::string &line, int n, double *v) {
    const char *p = line.c_str();
    for (int i = 0; i < n; i++) {
        char *end = nullptr;
        errno = 0;
        v[i] = strtod(p, &end);
        if (end == p || errno != 0) return false;
        p = end;
    }
    return true;
}

static bool parse_ints(const std::string &line, int n, int *v) {
    const char *p = line.c_str();
    for (int i = 0; i < n; i++) {
        char *end = nullptr;
        errno = 0;
        long x = strtol(p, &end, 10);
        if (end == p || errno != 0) return false;
        v[i] = (int)x;
        p = end;
    }
    return true;
}

static std::string trim(const std::string &s) {
    size_t a = s.find_first_not_of(" \t\r"), b = s.find_last_not_of(" \t\r");
    return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

void set_reference_peaks(xpfc_params *p) {
    // initialize.cu:10-17 (hard-coded two-peak DCF), :215-217 (sum envelope)
    p->npeaks = 2;
    p->pk_k[0] = 2.0 * M_PI;
    p->pk_k[1] = 2.0 * M_PI * std::sqrt(2.0);
    p->pk_rho[0] = 1.0;
    p->pk_rho[1] = 1.0 / std::sqrt(2.0);
    p->pk_beta[0] = 4.0;
    p->pk_beta[1] = 4.0;
    p->pk_alpha[0] = 1.0;
    p->pk_alpha[1] = 1.0;
    p->envelope = XPFC_ENVELOPE_SUM;
}

int read_input(const char *path, xpfc_params *p) {
    FILE *f = fopen(path, "r");
    if (!f) {
        set_thread_error(std::string("cannot open input deck: ") + path);
        return XPFC_EIO;
    }
    xpfc_default_params(p);
    std::string L[18];
    for (int i = 0; i < 18; i++) {
        if (!read_line(f, L[i])) {
            fclose(f);
            set_thread_error("pfc.input truncated before line " + std::to_string(i + 1));
            return XPFC_EIO;
        }
    }
    double d[4];
    int iv[3];
    bool ok = true;
    // line layout of read_input.cu:19-115 (blank lines 4, 7, 11, 15)
    ok = ok && parse_ints(L[0], 1, iv);                                       // no_val
    ok = ok && parse_nums(L[1], 2, d) && ((p->psi0 = d[0]), (p->sigma = d[1]), true);
    double a_in = 0, b_in = 0;
    ok = ok && parse_nums(L[2], 4, d) && ((a_in = d[0]), (b_in = d[1]), (p->eps = d[2]), (p->Mo = d[3]), true);
    int Lxi = 0, Lyi = 0, Mx = 0, My = 0, t = 0, ts = 0, iconfig = 0;
    ok = ok && parse_ints(L[4], 2, iv) && ((Lxi = iv[0]), (Lyi = iv[1]), true);
    ok = ok && parse_ints(L[5], 2, iv) && ((Mx = iv[0]), (My = iv[1]), true);
    ok = ok && parse_ints(L[7], 1, iv) && ((t = iv[0]), true);
    ok = ok && parse_nums(L[8], 1, d) && ((p->dt = d[0]), true);
    ok = ok && parse_ints(L[9], 1, iv) && ((ts = iv[0]), true);
    ok = ok && parse_ints(L[11], 1, iv) && ((iconfig = iv[0]), true);
    ok = ok && parse_nums(L[12], 2, d) && ((p->A_10 = d[0]), (p->A_11 = d[1]), true);
    ok = ok && parse_nums(L[13], 1, d) && ((p->A_tri = d[0]), true);
    ok = ok && parse_ints(L[15], 1, iv) && ((p->iseed = iv[0]), true);
    ok = ok && parse_ints(L[16], 1, iv) && ((p->ishape = iv[0]), true);
    ok = ok && parse_nums(L[17], 3, d) && ((p->h = d[0]), (p->k = d[1]), (p->roa = d[2]), true);
    if (!ok) {
        fclose(f);
        set_thread_error("pfc.input: malformed value on lines 1-18");
        return XPFC_EIO;
    }
    if (iconfig != 0 && iconfig != 1 && iconfig != 2 && iconfig != 10) {
        fclose(f);
        set_thread_error("pfc.input: invalid iconfig " + std::to_string(iconfig));   // read_input.cu:71-73
        return XPFC_EINVAL;
    }
    if ((p->iseed != 0 && p->iseed != 1) || (p->ishape != 0 && p->ishape != 1)) {
        fclose(f);
        set_thread_error("pfc.input: invalid iseed/ishape");   // read_input.cu:95-110
        return XPFC_EINVAL;
    }
    p->a = 1.0 / a_in;   // read_input.cu:28
    p->b = 1.0 / b_in;
    p->iconfig = iconfig;
    p->ic_kind = XPFC_IC_REFERENCE;
    p->t_sample = ts;
    set_reference_peaks(p);
    p->ref_compat = 1;
    p->precision = XPFC_FP64;
    // initialize.cu:23-33: lattice scaling of the (integer) box lengths
    const double a_tri = 2.0 / std::sqrt(3.0);
    if (iconfig == 0) { Lxi = (int)(Lxi * a_tri); Lyi = (int)(Lyi * a_tri); }
    p->Mx = Mx; p->My = My; p->Mz = 1;
    p->Lx = Lxi; p->Ly = Lyi; p->Lz = 1.0;
    // initialize.cu:60 N_t_steps = t/dt + 1; the loop runs n < N_t_steps
    const double nts = (double)t / p->dt + 1.0;
    p->nsteps = (long long)std::ceil(nts);
    // optional extension lines "key = value" after line 18
    std::string line;
    while (read_line(f, line)) {
        std::string s = trim(line);
        if (s.empty() || s[0] == '#') continue;
        size_t eq = s.find('=');
        if (eq == std::string::npos) continue;
        std::string key = trim(s.substr(0, eq)), val = trim(s.substr(eq + 1));
        double v = strtod(val.c_str(), nullptr);
        if (key == "Mz") p->Mz = (int)v;
        else if (key == "Lz") p->Lz = v;
        else if (key == "precision") p->precision = (val == "mixed" || v == 1.0) ? XPFC_MIXED : XPFC_FP64;
        else if (key == "ref_compat") p->ref_compat = (int)v;
        else if (key == "envelope") p->envelope = (val == "max" || v == 1.0) ? XPFC_ENVELOPE_MAX : XPFC_ENVELOPE_SUM;
        else if (key == "noise_amp") p->noise_amp = v;
        else if (key == "noise_seed") p->noise_seed = strtoull(val.c_str(), nullptr, 10);
        else if (key == "ic_kind") p->ic_kind = (int)v;
        else if (key == "ic_amp") p->ic_amp = v;
        else if (key == "ic_seed") p->ic_seed = strtoull(val.c_str(), nullptr, 10);
        else if (key == "ic_seed_amp") p->ic_seed_amp = v;
        else if (key == "ic_seed_radius") p->ic_seed_radius = v;
        else if (key == "nsteps") p->nsteps = (long long)v;
        else if (key == "peaks") {
            // peaks = k,alpha,rho,beta; k,alpha,rho,beta; ...
            int n = 0;
            const char *q = val.c_str();
            while (*q && n < XPFC_MAX_PEAKS) {
                double pk[4];
                char *end;
                bool good = true;
                for (int j = 0; j < 4; j++) {
                    while (*q == ' ' || *q == ',' || *q == ';') q++;
                    pk[j] = strtod(q, &end);
                    if (end == q) { good = false; break; }
                    q = end;
                }
                if (!good) break;
                p->pk_k[n] = pk[0]; p->pk_alpha[n] = pk[1]; p->pk_rho[n] = pk[2]; p->pk_beta[n] = pk[3];
                n++;
                while (*q == ' ' || *q == ',') q++;
                if (*q == ';') q++;
            }
            if (n > 0) p->npeaks = n;
        }
    }
    fclose(f);
    if (p->Mz > 1) {
        // the reference is 2-D; for 3-D decks F uses the same (M-1) volume rule
        p->ff_factor = (p->Lx * p->Ly * p->Lz) / ((double)(p->Mx - 1) * (p->My - 1) * (p->Mz - 1));
    } else {
        // initialize.cu:63: ff_factor = Lx*Ly/((Mx-1)(My-1))
        p->ff_factor = (double)(Lxi * Lyi) / (double)((Mx - 1) * (My - 1));
    }
    if (iconfig == 10) {
        // obtain_box_size (read_input.cu:124-155): L = round(M * spacing)
        snprintf(p->vtk_path, sizeof(p->vtk_path), "initial_density_field.vtk");
        const char *slash = strrchr(path, '/');
        if (slash) {
            std::string dir(path, slash - path + 1);
            snprintf(p->vtk_path, sizeof(p->vtk_path), "%sinitial_density_field.vtk", dir.c_str());
        }
        int dims[3];
        double Lb[3];
        int rc = read_vtk_header(p->vtk_path, dims, Lb);
        if (rc != XPFC_OK) return rc;
        p->Lx = std::round(Lb[0]);
        p->Ly = std::round(Lb[1]);
        p->ff_factor = (p->Lx * p->Ly) / (double)((Mx - 1) * (My - 1));
    }
    return XPFC_OK;
}

// ---------------------------------------------------------------------------
// VTK (write_vtk.cu:4-35, read_input.cu:124-241)
// ---------------------------------------------------------------------------
int write_vtk(const char *path, const double *psi, int Mx, int My, int Mz, double Lx, double Ly, double Lz, int prec) {
    FILE *f = fopen(path, "w");
    if (!f) {
        set_thread_error(std::string("cannot write ") + path);
        return XPFC_EIO;
    }
    if (prec <= 0) prec = 6;
    fprintf(f, "# vtk DataFile Version 3.0\nDensity Data\nASCII\nDATASET STRUCTURED_POINTS\n");
    fprintf(f, "DIMENSIONS %d %d %d\nORIGIN 0 0 0\n", Mx, My, Mz);
    // SPACING as the reference prints double(L)/double(M) with ostream defaults
    fprintf(f, "SPACING %.6g %.6g %.6g\n", Lx / Mx, Ly / My, Mz > 1 ? Lz / Mz : 1.0);
    fprintf(f, "POINT_DATA %lld\nSCALARS DensityData float\nLOOKUP_TABLE default\n", (long long)Mx * My * Mz);
    // x fastest in the file; memory is [Mx][My][Mz] with z fastest
    char fmt[16];
    snprintf(fmt, sizeof(fmt), "%%.%dg\n", prec);
    for (int iz = 0; iz < Mz; iz++)
        for (int iy = 0; iy < My; iy++)
            for (int ix = 0; ix < Mx; ix++) fprintf(f, fmt, psi[((size_t)ix * My + iy) * Mz + iz]);
    if (fclose(f) != 0) return XPFC_EIO;
    return XPFC_OK;
}

int read_vtk_header(const char *path, int dims[3], double L[3]) {
    FILE *f = fopen(path, "r");
    if (!f) {
        set_thread_error(std::string("cannot open ") + path);
        return XPFC_EIO;
    }
    std::string line;
    int got = 0;
    double sp[3] = {1, 1, 1};
    while (read_line(f, line)) {
        if (sscanf(line.c_str(), "DIMENSIONS %d %d %d", &dims[0], &dims[1], &dims[2]) == 3) got |= 1;
        if (sscanf(line.c_str(), "SPACING %lf %lf %lf", &sp[0], &sp[1], &sp[2]) == 3) got |= 2;
        if (line.rfind("LOOKUP_TABLE", 0) == 0) break;
    }
    fclose(f);
    if (got != 3) {
        set_thread_error(std::string("malformed VTK header: ") + path);
        return XPFC_EIO;
    }
    for (int i = 0; i < 3; i++) L[i] = dims[i] * sp[i];
    return XPFC_OK;
}

int read_vtk(const char *path, double *psi, size_t cap, int dims_out[3], double L_out[3]) {
    int dims[3];
    double Lb[3];
    int rc = read_vtk_header(path, dims, Lb);
    if (rc != XPFC_OK) return rc;
    const size_t n = (size_t)dims[0] * dims[1] * dims[2];
    if (dims_out) memcpy(dims_out, dims, sizeof(dims));
    if (L_out) memcpy(L_out, Lb, sizeof(Lb));
    if (!psi) return XPFC_OK;
    if (cap < n) {
        set_thread_error("read_vtk: buffer too small");
        return XPFC_EINVAL;
    }
    FILE *f = fopen(path, "r");
    if (!f) return XPFC_EIO;
    std::string line;
    while (read_line(f, line))
        if (line.rfind("LOOKUP_TABLE", 0) == 0) break;
    const int Mx = dims[0], My = dims[1], Mz = dims[2];
    size_t i = 0;
    for (; i < n; i++) {
        if (!read_line(f, line)) break;
        char *end;
        double v = strtod(line.c_str(), &end);
        if (end == line.c_str()) break;
        const size_t ix = i % Mx, iy = (i / Mx) % My, iz = i / ((size_t)Mx * My);
        psi[(ix * My + iy) * Mz + iz] = v;
    }
    fclose(f);
    if (i != n) {
        set_thread_error("VTK file ends early at value " + std::to_string(i));   // read_input.cu:210-213
        return XPFC_EIO;
    }
    return XPFC_OK;
}

// ---------------------------------------------------------------------------
// initial conditions (initialize.cu:95-197) and mean pinning (Avg_calc.cu)
// ---------------------------------------------------------------------------
void pin_mean(double *psi, size_t n, double psi0) {
    double s = 0.0;
    for (size_t i = 0; i < n; i++) s += psi[i];
    const double m = s / (double)n;
    double diff = 0.0;
    if (m != psi0) diff = psi0 - m;
    for (size_t i = 0; i < n; i++) psi[i] += diff;
}

static void ic_reference(const xpfc_params *p, double *psi) {
    const int Mx = p->Mx, My = p->My;
    const double a_tri = 2.0 / std::sqrt(3.0), a_sq = 1.0;
    const double k_sq = 2 * M_PI / a_sq, k_tri = 2 * M_PI / a_tri;
    // linspace.cu:5-18: accumulated coordinates, du = L/(M-1)
    std::vector<double> x(Mx + 1), y(My + 1);
    const double dux = p->Lx / ((double)Mx - 1), duy = p->Ly / ((double)My - 1);
    x[0] = 0.0;
    for (int i = 0; i < Mx; i++) x[i + 1] = x[i] + dux;
    y[0] = 0.0;
    for (int j = 0; j < My; j++) y[j + 1] = y[j] + duy;
    double r = 0.0;
    if (p->iconfig == 1) r = p->roa * a_sq;
    else if (p->iconfig == 0) r = p->roa * a_tri;
    for (int i = 0; i < Mx; i++)
        for (int j = 0; j < My; j++) {
            const double X = x[i], Y = y[j];
            double v;
            if (p->iconfig == 1)
                v = p->A_10 * ((3.0 * std::sqrt(2.0) - 2.0) * std::cos(k_sq * Y) - 2.0 * std::cos(k_sq * X)) -
                    p->A_11 * std::cos(k_sq * X) * std::cos(k_sq * Y);
            else if (p->iconfig == 0)
                v = p->A_tri * (std::cos(k_tri * X) / 2.0 + std::cos(k_tri * X / 2.0) * std::cos(std::sqrt(3.0) * k_tri * Y / 2.0));
            else
                v = 0.0;
            psi[(size_t)i * My + j] = v + p->psi0;
        }
    if (p->iseed == 1) {
        for (int i = 0; i < Mx; i++)
            for (int j = 0; j < My; j++) {
                const double X = x[i], Y = y[j];
                const size_t id = (size_t)i * My + j;
                if (p->ishape == 0) {
                    const double d = std::sqrt((X - p->h) * (X - p->h) + (Y - p->k) * (Y - p->k));
                    if (d > r) psi[id] = p->psi0;
                } else {
                    const double g = std::exp(-((X - p->h) * (X - p->h) + (Y - p->k) * (Y - p->k)) / p->roa);
                    const double v = psi[id] - p->psi0;
                    psi[id] = v * g + p->psi0 * (1 - g);
                }
            }
    }
}

// Gaussian noise per point (stream 0); the counter is the point index in the
// [Mx][My][Mz] layout.
static void ic_noise(const xpfc_params *p, double *psi) {
    const size_t n = (size_t)p->Mx * p->My * p->Mz;
    for (size_t i = 0; i < n; i++) {
        double g0, g1;
        gauss_pair(p->ic_seed, 0, i, &g0, &g1);
        psi[i] = p->psi0 + p->ic_amp * g0;
    }
}

// fcc (111) seed: sphere of ic_seed_radius grid points about the box centre,
// psi = psi0 + ic_seed_amp * sum_j cos(q_j . r), q_j = (2 pi/sqrt 3)(+-1,+-1,1)
static void ic_fcc(const xpfc_params *p, double *psi) {
    const int Mx = p->Mx, My = p->My, Mz = p->Mz;
    const double q = 2.0 * M_PI / std::sqrt(3.0);
    const double dx = p->Lx / Mx, dy = p->Ly / My, dz = p->Lz / Mz;
    const double cx = 0.5 * Mx, cy = 0.5 * My, cz = 0.5 * Mz;
    const double R = p->ic_seed_radius;
    for (int ix = 0; ix < Mx; ix++)
        for (int iy = 0; iy < My; iy++)
            for (int iz = 0; iz < Mz; iz++) {
                const double rx = ix - cx, ry = iy - cy, rz = iz - cz;
                if (rx * rx + ry * ry + rz * rz > R * R) continue;
                const double X = rx * dx, Y = ry * dy, Z = rz * dz;
                const double s = std::cos(q * (X + Y + Z)) + std::cos(q * (X - Y + Z)) + std::cos(q * (-X + Y + Z)) +
                                 std::cos(q * (-X - Y + Z));
                psi[((size_t)ix * My + iy) * Mz + iz] = p->psi0 + p->ic_seed_amp * s;
            }
}

int build_initial_field(const xpfc_params *p, double *psi) {
    const size_t n = (size_t)p->Mx * p->My * p->Mz;
    switch (p->ic_kind) {
        case XPFC_IC_REFERENCE:
            if (p->iconfig == 10) {
                int rc = read_vtk(p->vtk_path, psi, n, nullptr, nullptr);
                if (rc != XPFC_OK) return rc;
            } else {
                if (p->Mz != 1) {
                    set_thread_error("reference initial conditions are 2-D (Mz must be 1)");
                    return XPFC_EINVAL;
                }
                ic_reference(p, psi);
            }
            break;
        case XPFC_IC_NOISE: ic_noise(p, psi); break;
        case XPFC_IC_FCC_SEED:
            ic_noise(p, psi);
            ic_fcc(p, psi);
            break;
        default: set_thread_error("unknown ic_kind"); return XPFC_EINVAL;
    }
    pin_mean(psi, n, p->psi0);
    return XPFC_OK;
}

}  // namespace xpfc
