// omx_host.h -- host-side set-up arithmetic of the reference, restated in C++: constants with
// their literal precision, CPML grading tables, den_* arrays, Drude / Drude-Lorentz ADE
// coefficients, the voxel -> media_map rule, source and q-group kernels.  Compiled with
// -ffp-contract=off so that every value equals the reference's FP64 value.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/omx_gpu.h"

namespace omx {

struct Consts {
    double pi0, c0, eps0, mu0;
    double sec_to_au, C_to_au, kg_to_au, m_to_au, sig_to_au;
    double nm_to_au, au_to_nm, ev_to_au, fs_to_au;
    double alphaCPML, kappaCPML;
    double aBH[4];
};
const Consts &consts();

struct CpmlTables {
    std::vector<double> be, ce, bh, ch, kappae, kappah;   // 0-based: index kk-1
};
CpmlTables cpml_tables(int npml, double dr, double dt);

// den_e / den_h per axis with the reference's CPML rules; entries 0..n+1 (1-based use).
void den_arrays(int dims, const int n[3], int npml, const int boundaries[3], double dr,
                const CpmlTables &T, std::vector<double> den_e[3], std::vector<double> den_h[3]);

void medium_dielectric(double eps_r, omx_medium *m);
void medium_drude(double omegaD, double GammaD, double eps_r, double dt, omx_medium *m);
bool medium_dl_library(const std::string &name, double eps_r, double dt, omx_medium *m);
void medium_dl_custom(double eps_inf, double wp_ev, double gamma_ev, int n_poles, const double *pole_ev,
                      const double *strength, const double *width_ev, double dt, omx_medium *m);

int media_map_from_voxels(int dims, const int n[3], double dr, int n_media, const int *n_vox,
                          const double *vox, int32_t *map);

// Source kernel (compute_kernel, source_mod.f90:251-327), normalised; i fastest.
std::vector<double> source_kernel(int dims, int n_ker, double dr);
// q-group `single` kernel (q_group_mod.f90:165-239), not normalised.
std::vector<double> qgroup_kernel(int dims, int n_ker);

}  // namespace omx
