// xpfc_host.h -- host-side helpers of libxpfc (deck, VTK, initial fields).
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>

#include "../../include/xpfc.h"

namespace xpfc {
void set_thread_error(const std::string &m);
const char *thread_error();
void gauss_pair(uint64_t seed, uint64_t stream, uint64_t index, double *g0, double *g1);
void set_reference_peaks(xpfc_params *p);
int read_input(const char *path, xpfc_params *p);
int write_vtk(const char *path, const double *psi, int Mx, int My, int Mz, double Lx, double Ly, double Lz, int prec);
int read_vtk_header(const char *path, int dims[3], double L[3]);
int read_vtk(const char *path, double *psi, size_t cap, int dims_out[3], double L_out[3]);
void pin_mean(double *psi, size_t n, double psi0);
int build_initial_field(const xpfc_params *p, double *psi);
}  // namespace xpfc
