// omx_host.cpp -- set-up arithmetic of the reference restated in C++ (see omx_host.h).
#include "omx_host.h"

#include <cmath>
#include <cstring>

namespace omx {

// Correctly rounded x^3: gfortran folds real**integer constant expressions with MPFR.
static double cube_correctly_rounded(double x)
{
    const double p = x * x;
    const double pe = std::fma(x, x, -p);
    const double q = p * x;
    const double qe = std::fma(p, x, -q);
    return q + (qe + pe * x);
}

static Consts make_consts()
{
    Consts c;
    // constants_mod.f90:13-49; default-real literals are rounded to single precision.
    c.pi0 = 3.141592653589793;
    c.c0 = 137.0;
    c.eps0 = 1.0 / (4.0 * c.pi0);
    c.mu0 = 1.0 / (c.eps0 * (c.c0 * c.c0));
    c.alphaCPML = static_cast<double>(0.05f);
    c.kappaCPML = 5.0;
    c.aBH[0] = 0.353222222;
    c.aBH[1] = -0.488;
    c.aBH[2] = 0.145;
    c.aBH[3] = -0.010222222;
    c.sec_to_au = 1.0 / 2.4188843265864e-17;
    c.C_to_au = 1.0 / 1.602176634e-19;
    c.kg_to_au = 1.0 / 9.1093837139e-31;
    c.m_to_au = 1.0 / 5.29177210544e-11;
    c.nm_to_au = static_cast<double>(18.897261259077823f);
    c.au_to_nm = 1.0 / c.nm_to_au;
    c.ev_to_au = static_cast<double>(1.0f / 27.2114f);
    c.fs_to_au = 1.0 / 2.4188843265864e-2;
    // mxll_3D_mod.f90:88
    c.sig_to_au = (c.C_to_au * c.C_to_au) * c.sec_to_au / (c.kg_to_au * cube_correctly_rounded(c.m_to_au));
    return c;
}

const Consts &consts()
{
    static const Consts c = make_consts();
    return c;
}

CpmlTables cpml_tables(int npml, double dr, double dt)
{
    // mxll_3D_mod.f90:294-318: the grading ratios are integer/default-real, so they and their
    // cubes are single precision; 0.8*(m+1) is a single-precision product.
    const Consts &c = consts();
    CpmlTables T;
    T.be.resize(npml);
    T.ce.resize(npml);
    T.kappae.resize(npml);
    T.bh.resize(npml > 1 ? npml - 1 : 0);
    T.ch.resize(T.bh.size());
    T.kappah.resize(T.bh.size());
    const double sigma_max = static_cast<double>(0.8f * 4.0f) / (dr * std::sqrt(c.mu0 / c.eps0));
    const float den = static_cast<float>(npml) - 1.0f;
    for (int kk = 1; kk <= npml; ++kk) {
        const float r = static_cast<float>(npml - kk) / den;
        const float r3 = r * r * r;
        const float ra = static_cast<float>(kk - 1) / den;
        const double sig = sigma_max * static_cast<double>(r3);
        const double alpha = c.alphaCPML * c.sig_to_au * static_cast<double>(ra);
        const double kap = 1.0 + (c.kappaCPML - 1.0) * static_cast<double>(r3);
        const double b = std::exp(-(sig / kap + alpha) * dt / c.eps0);
        T.kappae[kk - 1] = kap;
        T.be[kk - 1] = b;
        T.ce[kk - 1] = (sig == 0.0 && alpha == 0.0 && kk == npml) ? 0.0
                                                                   : sig * (b - 1.0) / (sig + kap * alpha) / kap;
    }
    for (int kk = 1; kk <= npml - 1; ++kk) {
        const float r = (static_cast<float>(npml - kk) - 0.5f) / den;
        const float r3 = r * r * r;
        const float ra = (static_cast<float>(kk) - 0.5f) / den;
        const double sig = sigma_max * static_cast<double>(r3);
        const double alpha = c.alphaCPML * c.sig_to_au * static_cast<double>(ra);
        const double kap = 1.0 + (c.kappaCPML - 1.0) * static_cast<double>(r3);
        const double b = std::exp(-(sig / kap + alpha) * dt / c.eps0);
        T.kappah[kk - 1] = kap;
        T.bh[kk - 1] = b;
        T.ch[kk - 1] = sig * (b - 1.0) / (sig + kap * alpha) / kap;
    }
    return T;
}

void den_arrays(int dims, const int n[3], int npml, const int boundaries[3], double dr, const CpmlTables &T,
                std::vector<double> den_e[3], std::vector<double> den_h[3])
{
    for (int a = 0; a < 3; ++a) {
        den_e[a].assign(n[a] + 2, 1.0 / dr);
        den_h[a].assign(n[a] + 2, 1.0 / dr);
    }
    if (dims == 1) {
        // mxll_1D_mod.f90:178-200 (the single axis is stored as axis 0 here)
        if (boundaries[0] != OMX_CPML_BOUNDARIES) return;
        const int nz = n[0];
        int kk = npml;
        for (int k = 1; k <= nz - 1; ++k) {
            if (k <= npml) den_e[0][k] = 1.0 / (T.kappae[k - 1] * dr);
            else if (k >= nz + 1 - npml) { den_e[0][k] = 1.0 / (T.kappae[kk - 1] * dr); --kk; }
            else den_e[0][k] = 1.0 / dr;
        }
        kk = npml - 1;
        for (int k = 1; k <= nz - 1; ++k) {
            if (k <= npml - 1) den_h[0][k] = 1.0 / (T.kappah[k - 1] * dr);
            else if (k >= nz + 1 - npml) { den_h[0][k] = 1.0 / (T.kappah[kk - 1] * dr); --kk; }
            else den_h[0][k] = 1.0 / dr;
        }
        return;
    }
    // mxll_3D_mod.f90:320-420 (2D :306-371)
    for (int a = 0; a < dims; ++a) {
        if (boundaries[a] != OMX_CPML_BOUNDARIES) continue;
        const int na = n[a];
        for (int k = 1; k <= na; ++k)
            if (k <= npml) den_e[a][k] = 1.0 / (T.kappae[k - 1] * dr);
        for (int k = 1; k <= na; ++k)
            if (k <= npml - 1) den_h[a][k] = 1.0 / (T.kappah[k - 1] * dr);
        int kk = npml;
        for (int k = 1; k <= na - 1; ++k)
            if (k >= na + 1 - npml) { den_e[a][k] = 1.0 / (T.kappae[kk - 1] * dr); --kk; }
        kk = npml - 1;
        for (int k = 1; k <= na - 1; ++k)
            if (k >= na + 1 - npml) { den_h[a][k] = 1.0 / (T.kappah[kk - 1] * dr); --kk; }
    }
}

// ---- init_classical_medium (classical_medium_mod.f90:46-104) ------------------------------------

void medium_dielectric(double eps_r, omx_medium *m)
{
    std::memset(m, 0, sizeof(*m));
    m->medium_type = OMX_DIELECTRIC_MEDIUM;
    m->eps_r = eps_r;
}

void medium_drude(double omegaD, double GammaD, double eps_r, double dt, omx_medium *m)
{
    const double eps0 = consts().eps0;
    std::memset(m, 0, sizeof(*m));
    m->medium_type = OMX_DRUDE_MEDIUM;
    m->eps_r = eps_r;
    m->A1 = (2.0 - GammaD * dt) / (2.0 + GammaD * dt);
    m->A2 = eps0 * (omegaD * omegaD) * dt / (2.0 + GammaD * dt);
    m->C1 = (eps_r * eps0 / dt - 0.5 * m->A2) / (eps_r * eps0 / dt + 0.5 * m->A2);
    m->C3 = 1.0 / (eps_r * eps0 / dt + 0.5 * m->A2);
    m->C4 = 0.5 * (m->A1 + 1.0) / (eps_r * eps0 / dt + 0.5 * m->A2);
}

struct PoleSet {
    double omegaD, GammaD, omegaP;
    int np;
    double w[OMX_MAX_POLES], g[OMX_MAX_POLES], a[OMX_MAX_POLES];
};

static void dl_from_poles(const PoleSet &P, double eps_r, double dt, omx_medium *m)
{
    const double eps0 = consts().eps0;
    std::memset(m, 0, sizeof(*m));
    m->medium_type = OMX_DL_MEDIUM;
    m->eps_r = eps_r;
    m->n_poles = P.np;
    for (int i = 0; i < P.np; ++i) {
        m->alpha_k[i] = (2.0 - (P.w[i] * P.w[i]) * (dt * dt)) / (1.0 + 0.5 * P.g[i] * dt);
        m->beta_k[i] = (P.g[i] * dt - 2.0) / (P.g[i] * dt + 2.0);
        m->gamma_k[i] = eps0 * P.a[i] * dt / (P.g[i] * dt + 2.0);
    }
    m->A1 = (2.0 - P.GammaD * dt) / (2.0 + P.GammaD * dt);
    m->A2 = eps0 * (P.omegaD * P.omegaD) * dt / (2.0 + P.GammaD * dt);
    double sum = 0.0;
    for (int i = 0; i < P.np; ++i) sum = sum + m->gamma_k[i];
    const double den = eps_r * eps0 / dt + 0.5 * m->A2 + 0.5 * sum;
    m->C1 = (eps_r * eps0 / dt - 0.5 * m->A2) / den;
    m->C2 = 0.5 * sum / den;
    m->C3 = 1.0 / den;
    m->C4 = 0.5 * (m->A1 + 1.0) / den;
    for (int i = 0; i < P.np; ++i) {
        m->B1_k[i] = 0.5 * (1.0 + m->alpha_k[i]) / den;
        m->B2_k[i] = 0.5 * m->beta_k[i] / den;
    }
}

bool medium_dl_library(const std::string &name, double eps_r, double dt, omx_medium *m)
{
    // get_DL_library_data (classical_medium_mod.f90:125-199): default-real literals.
    const double ev = consts().ev_to_au;
    PoleSet P{};
    const float *w = nullptr, *g = nullptr, *a = nullptr;
    static const float agW[5] = {0.816f, 4.481f, 8.185f, 9.083f, 20.29f};
    static const float agG[5] = {3.886f, 0.452f, 0.065f, 0.916f, 2.419f};
    static const float agA[5] = {0.065f, 0.124f, 0.011f, 0.840f, 5.646f};
    static const float alW[4] = {0.162f, 1.544f, 1.808f, 3.473f};
    static const float alG[4] = {0.333f, 0.312f, 1.351f, 3.382f};
    static const float alA[4] = {0.227f, 0.050f, 0.166f, 0.030f};
    static const float auW[5] = {0.415f, 0.830f, 2.969f, 4.304f, 13.32f};
    static const float auG[5] = {0.241f, 0.345f, 0.870f, 2.494f, 2.214f};
    static const float auA[5] = {0.024f, 0.010f, 0.071f, 0.601f, 4.384f};
    if (name == "Ag") {
        P.np = 5;
        P.GammaD = static_cast<double>(0.048f) * ev;
        P.omegaP = static_cast<double>(9.01f) * ev;
        P.omegaD = static_cast<double>(9.01f * 0.919238815542512f) * ev;
        w = agW; g = agG; a = agA;
    } else if (name == "Al") {
        P.np = 4;
        P.GammaD = static_cast<double>(0.047f) * ev;
        P.omegaP = static_cast<double>(14.98f) * ev;
        P.omegaD = static_cast<double>(14.98f * 0.723187389270582f) * ev;
        w = alW; g = alG; a = alA;
    } else if (name == "Au") {
        P.np = 5;
        P.GammaD = static_cast<double>(0.053f) * ev;
        P.omegaP = static_cast<double>(9.03f) * ev;
        P.omegaD = static_cast<double>(9.03f * 0.871779788708135f) * ev;
        w = auW; g = auG; a = auA;
    } else {
        return false;
    }
    for (int i = 0; i < P.np; ++i) {
        P.w[i] = static_cast<double>(w[i]) * ev;
        P.g[i] = static_cast<double>(g[i]) * ev;
        P.a[i] = static_cast<double>(a[i]) * (P.omegaP * P.omegaP);
    }
    dl_from_poles(P, eps_r, dt, m);
    return true;
}

void medium_dl_custom(double eps_inf, double wp_ev, double gamma_ev, int n_poles, const double *pole_ev,
                      const double *strength, const double *width_ev, double dt, omx_medium *m)
{
    const double ev = consts().ev_to_au;
    PoleSet P{};
    P.np = n_poles;
    P.omegaP = wp_ev * ev;
    P.omegaD = P.omegaP;
    P.GammaD = gamma_ev * ev;
    for (int i = 0; i < n_poles; ++i) {
        P.w[i] = pole_ev[i] * ev;
        P.g[i] = width_ev[i] * ev;
        P.a[i] = strength[i] * (P.omegaP * P.omegaP);
    }
    dl_from_poles(P, eps_inf, dt, m);
}

// ---- read_init_media_{1D,2D,3D} voxel rule (classical_medium_mod.f90:203-769) ------------------
int media_map_from_voxels(int dims, const int n[3], double dr, int n_media, const int *n_vox, const double *vox,
                          int32_t *map)
{
    const double nm = consts().nm_to_au;
    const int nx = n[0], ny = dims >= 2 ? n[1] : 1, nz = dims == 3 ? n[2] : 1;
    const long long N = (long long)nx * ny * nz;
    const int comps = dims == 1 ? 1 : 3;
    std::memset(map, 0, sizeof(int32_t) * (size_t)(N * comps));
    std::vector<int32_t> aux((size_t)N, 0);
    auto A = [&](int i, int j, int k) -> int32_t {
        if (i < 1 || i > nx || j < 1 || j > ny || k < 1 || k > nz) return 0;
        return aux[(size_t)((i - 1) + (long long)nx * ((j - 1) + (long long)ny * (k - 1)))];
    };
    long long off = 0;
    for (int m = 1; m <= n_media; ++m) {
        for (int v = 0; v < n_vox[m - 1]; ++v, ++off) {
            int idx[3] = {1, 1, 1};
            for (int a = 0; a < dims; ++a) {
                const double x = vox[off * dims + a] * nm;
                idx[a] = static_cast<int>(x / dr) + n[a] / 2;
            }
            if (idx[0] < 1 || idx[0] > nx || idx[1] < 1 || idx[1] > ny || idx[2] < 1 || idx[2] > nz) continue;
            int32_t &cell = aux[(size_t)((idx[0] - 1) + (long long)nx * ((idx[1] - 1) + (long long)ny * (idx[2] - 1)))];
            if (cell == 0) cell = m;   // overlap: the reference reports and keeps the first medium
        }
    }
    if (dims == 1) {
        for (long long q = 0; q < N; ++q) map[q] = aux[(size_t)q];
        return 0;
    }
    auto M = [&](int i, int j, int k, int c) -> int32_t & {
        return map[(size_t)((i - 1) + (long long)nx * ((j - 1) + (long long)ny * ((k - 1) + (long long)nz * (c - 1))))];
    };
    for (int m = 1; m <= n_media; ++m)
        for (int k = 1; k <= nz; ++k)
            for (int j = 1; j <= ny; ++j)
                for (int i = 1; i <= nx; ++i) {
                    const int32_t a = A(i, j, k);
                    const bool last_plane = (i == nx) || (j == ny) || (dims == 3 && k == nz);
                    if (last_plane && a == m) {
                        M(i, j, k, 1) = m;   // the reference sets only component 1 there
                        continue;
                    }
                    if ((a == m && A(i + 1, j, k) == m) || (a != 0 && A(i + 1, j, k) == m)) M(i, j, k, 1) = m;
                    if ((a == m && A(i, j + 1, k) == m) || (a != 0 && A(i, j + 1, k) == m)) M(i, j, k, 2) = m;
                    if (dims == 3) {
                        if ((a == m && A(i, j, k + 1) == m) || (a != 0 && A(i, j, k + 1) == m)) M(i, j, k, 3) = m;
                    } else {
                        if (a == m) M(i, j, k, 3) = m;
                    }
                }
    return 0;
}

// ---- source / q-group kernels ---------------------------------------------------------------------
static double bh_window(double r, double r0, double r_max)
{
    const Consts &c = consts();
    const double tp = 2.0 * c.pi0;
    return c.aBH[0] + c.aBH[1] * std::cos(tp * (r - r0) / r_max) + c.aBH[2] * std::cos(tp * 2.0 * (r - r0) / r_max) +
           c.aBH[3] * std::cos(tp * 3.0 * (r - r0) / r_max);
}

std::vector<double> source_kernel(int dims, int n_ker, double dr)
{
    // compute_kernel (source_mod.f90:251-327), points ordered with i fastest.
    const int side = 2 * n_ker + 1;
    const int cnt = dims == 3 ? side * side * side : (dims == 2 ? side * side : side);
    std::vector<double> ker((size_t)cnt);
    const double r_max = (n_ker * 2 + 2) * dr;
    const double r0 = r_max / 2.0;
    double norm = 0.0;
    int q = 0;
    const int kl = dims == 3 ? n_ker : 0, jl = dims >= 2 ? n_ker : 0;
    for (int k = -kl; k <= kl; ++k)
        for (int j = -jl; j <= jl; ++j)
            for (int i = -n_ker; i <= n_ker; ++i, ++q) {
                const double x = i * dr, y = j * dr, z = k * dr;
                double r;
                if (dims == 1) r = x;
                else if (dims == 2) r = std::sqrt(x * x + y * y);
                else r = std::sqrt(x * x + y * y + z * z);
                double w = bh_window(r, r0, r_max);
                if (dims >= 2 && w < 0.0) w = 0.0;
                ker[(size_t)q] = w;
                norm = norm + w;
            }
    for (auto &w : ker) w = w / norm;
    return ker;
}

std::vector<double> qgroup_kernel(int dims, int n_ker)
{
    // q_group_mod.f90:165-239: grid units, r_max = 2*n_ker+4, the norm is never applied.
    const int side = 2 * n_ker + 1;
    const int cnt = dims == 3 ? side * side * side : (dims == 2 ? side * side : side);
    std::vector<double> ker((size_t)cnt);
    const double r_max = static_cast<double>(n_ker * 2 + 4);
    const double r0 = r_max / 2.0;
    int q = 0;
    const int kl = dims == 3 ? n_ker : 0, jl = dims >= 2 ? n_ker : 0;
    for (int k = -kl; k <= kl; ++k)
        for (int j = -jl; j <= jl; ++j)
            for (int i = -n_ker; i <= n_ker; ++i, ++q) {
                const double x = i, y = j, z = k;
                double r;
                if (dims == 1) r = x;
                else if (dims == 2) r = std::sqrt(x * x + y * y);
                else r = std::sqrt(x * x + y * y + z * z);
                double w = bh_window(r, r0, r_max);
                if (dims >= 2 && w < 0.0) w = 0.0;
                ker[(size_t)q] = w;
            }
    return ker;
}

}  // namespace omx
