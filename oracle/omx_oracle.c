/*
 * omx_oracle.c -- CPU FP64 restatement of the OMxRTA time-domain hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker; never the product).  See omx_oracle.h
 * for the parity statement ("parity unpinned" against the reference itself).
 *
 * Compile with -ffp-contract=off and without -ffast-math: the reference is
 * gfortran -O3 on generic targets, which emits no fused multiply-adds and
 * evaluates every expression left to right as written.  Each routine below
 * keeps the reference's operation order so that its FP64 results are the
 * reference's results bit for bit, up to the libm calls (exp, cos, sqrt).
 */
#include "omx_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ======================================================================================= */
/* constants_mod.f90                                                                        */
/* ======================================================================================= */

/* Correctly rounded x**3, as gfortran folds real**integer constants with MPFR. */
static double cube_rn(double x)
{
    double p = x * x;
    double e = fma(x, x, -p);
    double q = p * x;
    double f = fma(p, x, -q);
    return q + (f + e * x);
}

void orc_get_constants(orc_constants *c)
{
    /* constants_mod.f90:13-49 */
    c->pi0 = 3.141592653589793;
    c->c0 = 137.0;
    c->eps0 = 1.0 / (4.0 * c->pi0);
    c->mu0 = 1.0 / (c->eps0 * (137.0 * 137.0));
    c->alphaCPML = (double)0.05f;                   /* single literal (:27) */
    c->kappaCPML = 5.0;
    c->aBH[0] = 0.353222222;
    c->aBH[1] = -0.488;
    c->aBH[2] = 0.145;
    c->aBH[3] = -0.010222222;
    c->sec_to_au = 1.0 / 2.4188843265864e-17;
    c->C_to_au = 1.0 / 1.602176634e-19;
    c->kg_to_au = 1.0 / 9.1093837139e-31;
    c->m_to_au = 1.0 / 5.29177210544e-11;
    c->nm_to_au = (double)18.897261259077823f;      /* single literal (:37) */
    c->au_to_nm = 1.0 / c->nm_to_au;
    c->ev_to_au = (double)(1.0f / 27.2114f);        /* single divide (:40) */
    c->au_to_ev = (double)27.2114f;
    c->Debye_to_au = (double)(3.0f / 7.63f);
    c->fs_to_au = 1.0 / 2.4188843265864e-2;
    c->au_to_fs = 2.4188843265864e-2;
    /* mxll_3D_mod.f90:88  C_to_au**2*sec_to_au/(kg_to_au*m_to_au**3), folded at compile time */
    c->sig_to_au = (c->C_to_au * c->C_to_au) * c->sec_to_au / (c->kg_to_au * cube_rn(c->m_to_au));
}

static orc_constants K;
static int K_ready = 0;
static const orc_constants *KC(void)
{
    if (!K_ready) {
        orc_get_constants(&K);
        K_ready = 1;
    }
    return &K;
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ======================================================================================= */
/* classical_medium_mod.f90: coefficient precompute                                         */
/* ======================================================================================= */

void orc_medium_dielectric(double eps_r, orc_medium *m)
{
    memset(m, 0, sizeof(*m));
    m->medium_type = ORC_DIELECTRIC; /* :62-63 (eps_r kept: the evident intent, N6) */
    m->eps_r = eps_r;
}

void orc_medium_drude(double omegaD, double GammaD, double eps_r, double dt, orc_medium *m)
{
    const double eps0 = KC()->eps0;
    memset(m, 0, sizeof(*m));
    m->medium_type = ORC_DRUDE; /* :64-74 */
    m->omegaD = omegaD;
    m->GammaD = GammaD;
    m->eps_r = eps_r;
    m->A1 = (2.0 - m->GammaD * dt) / (2.0 + m->GammaD * dt);
    m->A2 = eps0 * (m->omegaD * m->omegaD) * dt / (2.0 + m->GammaD * dt);
    m->C1 = (m->eps_r * eps0 / dt - 0.5 * m->A2) / (m->eps_r * eps0 / dt + 0.5 * m->A2);
    m->C3 = 1.0 / (m->eps_r * eps0 / dt + 0.5 * m->A2);
    m->C4 = 0.5 * (m->A1 + 1.0) / (m->eps_r * eps0 / dt + 0.5 * m->A2);
}

/* Drude-Lorentz coefficients from (omegaD, GammaD, omegaP_i, GammaP_i, AP_i): :76-100 */
static void dl_coefficients(orc_medium *m, double dt)
{
    const double eps0 = KC()->eps0;
    int i;
    double sum_g;
    for (i = 0; i < m->n_poles; i++) {
        double w = m->omegaP_i[i], G = m->GammaP_i[i];
        m->alpha_k[i] = (2.0 - (w * w) * (dt * dt)) / (1.0 + 0.5 * G * dt);
        m->beta_k[i] = (G * dt - 2.0) / (G * dt + 2.0);
        m->gamma_k[i] = eps0 * m->AP_i[i] * dt / (G * dt + 2.0);
    }
    m->A1 = (2.0 - m->GammaD * dt) / (2.0 + m->GammaD * dt);
    m->A2 = eps0 * (m->omegaD * m->omegaD) * dt / (2.0 + m->GammaD * dt);
    sum_g = 0.0; /* SUM(gamma_k): sequential */
    for (i = 0; i < m->n_poles; i++)
        sum_g = sum_g + m->gamma_k[i];
    {
        double den = m->eps_r * eps0 / dt + 0.5 * m->A2 + 0.5 * sum_g;
        m->C1 = (m->eps_r * eps0 / dt - 0.5 * m->A2) / den;
        m->C2 = 0.5 * sum_g / den;
        m->C3 = 1.0 / den;
        m->C4 = 0.5 * (m->A1 + 1.0) / den;
        for (i = 0; i < m->n_poles; i++) {
            m->B1_k[i] = 0.5 * (1.0 + m->alpha_k[i]) / den;
            m->B2_k[i] = 0.5 * m->beta_k[i] / den;
        }
    }
}

/* get_DL_library_data (:125-199): literals are default-real (single) */
int orc_medium_dl_library(const char *material, double eps_r, double dt, orc_medium *m)
{
    const double ev = KC()->ev_to_au;
    memset(m, 0, sizeof(*m));
    m->medium_type = ORC_DL;
    m->eps_r = eps_r;
#define S(x) ((double)(x##f))
    if (strcmp(material, "Ag") == 0) {
        static const float wP[5] = {0.816f, 4.481f, 8.185f, 9.083f, 20.29f};
        static const float gP[5] = {3.886f, 0.452f, 0.065f, 0.916f, 2.419f};
        static const float aP[5] = {0.065f, 0.124f, 0.011f, 0.840f, 5.646f};
        int i;
        m->n_poles = 5;
        m->GammaD = S(0.048) * ev;
        m->omegaP = S(9.01) * ev;
        m->omegaD = (double)(9.01f * 0.919238815542512f) * ev;
        for (i = 0; i < 5; i++) {
            m->omegaP_i[i] = (double)wP[i] * ev;
            m->GammaP_i[i] = (double)gP[i] * ev;
            m->AP_i[i] = (double)aP[i] * (m->omegaP * m->omegaP);
        }
    } else if (strcmp(material, "Al") == 0) {
        static const float wP[4] = {0.162f, 1.544f, 1.808f, 3.473f};
        static const float gP[4] = {0.333f, 0.312f, 1.351f, 3.382f};
        static const float aP[4] = {0.227f, 0.050f, 0.166f, 0.030f};
        int i;
        m->n_poles = 4;
        m->GammaD = S(0.047) * ev;
        m->omegaP = S(14.98) * ev;
        m->omegaD = (double)(14.98f * 0.723187389270582f) * ev;
        for (i = 0; i < 4; i++) {
            m->omegaP_i[i] = (double)wP[i] * ev;
            m->GammaP_i[i] = (double)gP[i] * ev;
            m->AP_i[i] = (double)aP[i] * (m->omegaP * m->omegaP);
        }
    } else if (strcmp(material, "Au") == 0) {
        static const float wP[5] = {0.415f, 0.830f, 2.969f, 4.304f, 13.32f};
        static const float gP[5] = {0.241f, 0.345f, 0.870f, 2.494f, 2.214f};
        static const float aP[5] = {0.024f, 0.010f, 0.071f, 0.601f, 4.384f};
        int i;
        m->n_poles = 5;
        m->GammaD = S(0.053) * ev;
        m->omegaP = S(9.03) * ev;
        m->omegaD = (double)(9.03f * 0.871779788708135f) * ev;
        for (i = 0; i < 5; i++) {
            m->omegaP_i[i] = (double)wP[i] * ev;
            m->GammaP_i[i] = (double)gP[i] * ev;
            m->AP_i[i] = (double)aP[i] * (m->omegaP * m->omegaP);
        }
    } else {
        return -1;
    }
#undef S
    dl_coefficients(m, dt);
    return 0;
}

void orc_medium_dl_custom(double eps_inf, double wp_ev, double gamma_ev, int n_poles,
                          const double *pole_ev, const double *strength, const double *width_ev,
                          double dt, orc_medium *m)
{
    const double ev = KC()->ev_to_au;
    int i;
    memset(m, 0, sizeof(*m));
    m->medium_type = ORC_DL;
    m->eps_r = eps_inf;
    m->n_poles = n_poles;
    m->omegaP = wp_ev * ev;
    m->omegaD = m->omegaP;
    m->GammaD = gamma_ev * ev;
    for (i = 0; i < n_poles; i++) {
        m->omegaP_i[i] = pole_ev[i] * ev;
        m->GammaP_i[i] = width_ev[i] * ev;
        m->AP_i[i] = strength[i] * (m->omegaP * m->omegaP);
    }
    dl_coefficients(m, dt);
}

/* ======================================================================================= */
/* CPML tables: mxll_3D_mod.f90:294-318 (identical in 2D :280-304 and 1D :152-176)          */
/* ======================================================================================= */

void orc_cpml_tables(int npml, double dr, double dt, double *be, double *ce, double *bh,
                     double *ch, double *kappae, double *kappah)
{
    const orc_constants *c = KC();
    const double sigmaCPML = (double)(0.8f * 4.0f) / (dr * sqrt(c->mu0 / c->eps0));
    int kk;
    for (kk = 1; kk <= npml; kk++) {
        float r = (float)(npml - kk) / ((float)npml - 1.0f);
        float r3 = r * r * r;
        float ra = (float)(kk - 1) / ((float)npml - 1.0f);
        double sige = sigmaCPML * (double)r3;
        double alphae = c->alphaCPML * c->sig_to_au * (double)ra;
        double kap = 1.0 + (c->kappaCPML - 1.0) * (double)r3;
        double b = exp(-(sige / kap + alphae) * dt / c->eps0);
        kappae[kk - 1] = kap;
        be[kk - 1] = b;
        if (sige == 0.0 && alphae == 0.0 && kk == npml)
            ce[kk - 1] = 0.0;
        else
            ce[kk - 1] = sige * (b - 1.0) / (sige + kap * alphae) / kap;
    }
    for (kk = 1; kk <= npml - 1; kk++) {
        float r = ((float)(npml - kk) - 0.5f) / ((float)npml - 1.0f);
        float r3 = r * r * r;
        float ra = ((float)kk - 0.5f) / ((float)npml - 1.0f);
        double sigh = sigmaCPML * (double)r3;
        double alphah = c->alphaCPML * c->sig_to_au * (double)ra;
        double kap = 1.0 + (c->kappaCPML - 1.0) * (double)r3;
        double b = exp(-(sigh / kap + alphah) * dt / c->eps0);
        kappah[kk - 1] = kap;
        bh[kk - 1] = b;
        ch[kk - 1] = sigh * (b - 1.0) / (sigh + kap * alphah) / kap;
    }
}

/* ======================================================================================= */
/* Arrays with Fortran bounds                                                               */
/* ======================================================================================= */

typedef struct {
    double *p;
    int lo[3], hi[3];
    long n0, n01;
} arr;

static void arr_alloc(arr *a, int l0, int h0, int l1, int h1, int l2, int h2)
{
    a->lo[0] = l0; a->hi[0] = h0;
    a->lo[1] = l1; a->hi[1] = h1;
    a->lo[2] = l2; a->hi[2] = h2;
    a->n0 = h0 - l0 + 1;
    a->n01 = a->n0 * (h1 - l1 + 1);
    a->p = (double *)calloc((size_t)(a->n01 * (h2 - l2 + 1)), sizeof(double));
}
static void arr_free(arr *a)
{
    free(a->p);
    a->p = NULL;
}
static long arr_size(const arr *a)
{
    return a->p ? a->n01 * (a->hi[2] - a->lo[2] + 1) : 0;
}
#define AT(a, i, j, k) ((a).p[((i) - (a).lo[0]) + (a).n0 * ((j) - (a).lo[1]) + (a).n01 * ((k) - (a).lo[2])])

/* ======================================================================================= */
/* Grid                                                                                     */
/* ======================================================================================= */

struct orc_grid {
    int dims, nx, ny, nz, npml, boundaries[3], mode, n_sec;
    int cpml_pos[6];
    double dt, dr, dt_eps0, dt_mu0, time, t_skip;
    arr Ex, Ey, Ez, Ex_old, Ey_old, Ez_old, Hx, Hy, Hz;
    arr eps_x, eps_y, eps_z;
    arr Jx, Jy, Jz, Jx_old, Jy_old, Jz_old, dJx, dJy, dJz;
    arr PD[3];
    arr PL[3][ORC_MAX_POLES], PL_old[3][ORC_MAX_POLES];
    int n_max_poles;
    arr psix_Eyx, psix_Ezx, psiy_Exy, psiy_Ezy, psiz_Exz, psiz_Eyz;
    arr psix_Hyx, psix_Hzx, psiy_Hxy, psiy_Hzy, psiz_Hxz, psiz_Hyz;
    double *be, *ce, *bh, *ch;                  /* 1-based */
    double *den_e[3], *den_h[3];                /* 1-based */
    int n_media;
    orc_medium *media;                          /* 1-based (media[0] unused) */
    int32_t *media_map;                         /* Fortran (n..., comps) */
};

static int mm_index(const orc_grid *g, int i, int j, int k, int c)
{
    if (g->dims == 3)
        return (i - 1) + g->nx * ((j - 1) + g->ny * ((k - 1) + g->nz * (c - 1)));
    if (g->dims == 2)
        return (i - 1) + g->nx * ((j - 1) + g->ny * (c - 1));
    return i - 1;
}

orc_grid *orc_grid_create(int dims, int nx, int ny, int nz, int npml, const int boundaries[3],
                          int mode, double dt, double dr)
{
    const orc_constants *c = KC();
    orc_grid *g = (orc_grid *)calloc(1, sizeof(orc_grid));
    int a, kk, k;
    double *kappae, *kappah;
    int n[3];
    g->dims = dims;
    g->npml = npml;
    g->mode = mode;
    g->dt = dt;
    g->dr = dr;
    g->dt_eps0 = dt / c->eps0;
    g->dt_mu0 = dt / c->mu0;
    g->n_sec = 2;
    g->n_max_poles = 1;
    for (a = 0; a < 3; a++)
        g->boundaries[a] = boundaries[a];
    if (dims == 3) {
        g->nx = nx; g->ny = ny; g->nz = nz;
        /* mxll_3D_mod.f90:123-143 */
        arr_alloc(&g->Ex, 0, nx, 1, ny + 1, 1, nz + 1);
        arr_alloc(&g->Ey, 1, nx + 1, 0, ny, 1, nz + 1);
        arr_alloc(&g->Ez, 1, nx + 1, 1, ny + 1, 0, nz);
        arr_alloc(&g->Ex_old, 0, nx, 1, ny + 1, 1, nz + 1);
        arr_alloc(&g->Ey_old, 1, nx + 1, 0, ny, 1, nz + 1);
        arr_alloc(&g->Ez_old, 1, nx + 1, 1, ny + 1, 0, nz);
        arr_alloc(&g->Hx, 1, nx, 0, ny, 0, nz);
        arr_alloc(&g->Hy, 0, nx, 1, ny, 0, nz);
        arr_alloc(&g->Hz, 0, nx, 0, ny, 1, nz);
        arr_alloc(&g->eps_x, 1, nx, 1, ny, 1, nz);
        arr_alloc(&g->eps_y, 1, nx, 1, ny, 1, nz);
        arr_alloc(&g->eps_z, 1, nx, 1, ny, 1, nz);
        arr_alloc(&g->Jx, 1, nx + 1, 1, ny, 1, nz);
        arr_alloc(&g->Jy, 1, nx, 1, ny + 1, 1, nz);
        arr_alloc(&g->Jz, 1, nx, 1, ny, 1, nz + 1);
        arr_alloc(&g->Jx_old, 1, nx + 1, 1, ny, 1, nz);
        arr_alloc(&g->Jy_old, 1, nx, 1, ny + 1, 1, nz);
        arr_alloc(&g->Jz_old, 1, nx, 1, ny, 1, nz + 1);
        arr_alloc(&g->dJx, 1, nx + 1, 1, ny, 1, nz);
        arr_alloc(&g->dJy, 1, nx, 1, ny + 1, 1, nz);
        arr_alloc(&g->dJz, 1, nx, 1, ny, 1, nz + 1);
        n[0] = nx; n[1] = ny; n[2] = nz;
    } else if (dims == 2) {
        g->nx = nx; g->ny = ny; g->nz = 1;
        /* mxll_2D_mod.f90:113-161 (TEz or TMz sets; k index fixed at 0) */
        if (mode == ORC_TEZ) {
            arr_alloc(&g->Ex, 0, nx, 1, ny + 1, 0, 0);
            arr_alloc(&g->Ey, 1, nx + 1, 0, ny, 0, 0);
            arr_alloc(&g->Ex_old, 0, nx, 1, ny + 1, 0, 0);
            arr_alloc(&g->Ey_old, 1, nx + 1, 0, ny, 0, 0);
            arr_alloc(&g->Hz, 0, nx, 0, ny, 0, 0);
            arr_alloc(&g->eps_x, 1, nx, 1, ny, 0, 0);
            arr_alloc(&g->eps_y, 1, nx, 1, ny, 0, 0);
            arr_alloc(&g->Jx, 1, nx + 1, 1, ny, 0, 0);
            arr_alloc(&g->Jx_old, 1, nx + 1, 1, ny, 0, 0);
            arr_alloc(&g->dJx, 1, nx + 1, 1, ny, 0, 0);
            arr_alloc(&g->Jy, 1, nx, 1, ny + 1, 0, 0);
            arr_alloc(&g->Jy_old, 1, nx, 1, ny + 1, 0, 0);
            arr_alloc(&g->dJy, 1, nx, 1, ny + 1, 0, 0);
        } else {
            arr_alloc(&g->Ez, 1, nx + 1, 1, ny + 1, 0, 0);
            arr_alloc(&g->Ez_old, 1, nx + 1, 1, ny + 1, 0, 0);
            arr_alloc(&g->Hx, 1, nx, 0, ny, 0, 0);
            arr_alloc(&g->Hy, 0, nx, 1, ny, 0, 0);
            arr_alloc(&g->eps_z, 1, nx, 1, ny, 0, 0);
            arr_alloc(&g->Jz, 1, nx, 1, ny, 0, 0);
            arr_alloc(&g->Jz_old, 1, nx, 1, ny, 0, 0);
            arr_alloc(&g->dJz, 1, nx, 1, ny, 0, 0);
        }
        /* eps arrays exist for all three in the reference only per mode; keep full */
        if (!g->eps_x.p) arr_alloc(&g->eps_x, 1, nx, 1, ny, 0, 0);
        if (!g->eps_y.p) arr_alloc(&g->eps_y, 1, nx, 1, ny, 0, 0);
        if (!g->eps_z.p) arr_alloc(&g->eps_z, 1, nx, 1, ny, 0, 0);
        n[0] = nx; n[1] = ny; n[2] = 1;
    } else {
        /* 1D: mxll_1D_mod.f90:91-109; the only axis is nz = grid_Ndims(1) */
        g->nx = 1; g->ny = 1; g->nz = nx;
        arr_alloc(&g->Ex, 1, nx, 0, 0, 0, 0);
        arr_alloc(&g->Ex_old, 1, nx, 0, 0, 0, 0);
        arr_alloc(&g->Hy, 1, nx - 1, 0, 0, 0, 0);
        arr_alloc(&g->Jx, 1, nx, 0, 0, 0, 0);
        arr_alloc(&g->eps_x, 1, nx, 0, 0, 0, 0);
        arr_alloc(&g->Jx_old, 1, nx, 0, 0, 0, 0);
        arr_alloc(&g->dJx, 1, nx, 0, 0, 0, 0);
        n[0] = 1; n[1] = 1; n[2] = nx;
    }
    /* eps default 1.0 */
    {
        arr *e[3] = {&g->eps_x, &g->eps_y, &g->eps_z};
        for (a = 0; a < 3; a++) {
            long s = arr_size(e[a]), q;
            for (q = 0; q < s; q++)
                e[a]->p[q] = 1.0;
        }
    }
    /* den arrays: 1/dr (1-based, length n+1 to keep 1-based indexing) */
    for (a = 0; a < 3; a++) {
        int len = n[a] + 2;
        g->den_e[a] = (double *)malloc(sizeof(double) * len);
        g->den_h[a] = (double *)malloc(sizeof(double) * len);
        for (k = 0; k < len; k++) {
            g->den_e[a][k] = 1.0 / dr;
            g->den_h[a][k] = 1.0 / dr;
        }
    }
    g->be = (double *)calloc(npml + 2, sizeof(double));
    g->ce = (double *)calloc(npml + 2, sizeof(double));
    g->bh = (double *)calloc(npml + 2, sizeof(double));
    g->ch = (double *)calloc(npml + 2, sizeof(double));
    kappae = (double *)calloc(npml + 2, sizeof(double));
    kappah = (double *)calloc(npml + 2, sizeof(double));

    if (dims == 1) {
        g->cpml_pos[4] = g->cpml_pos[5] = (boundaries[0] == ORC_CPML);
        if (boundaries[0] == ORC_CPML) {
            orc_cpml_tables(npml, dr, dt, g->be + 1, g->ce + 1, g->bh + 1, g->ch + 1, kappae + 1,
                            kappah + 1);
            arr_alloc(&g->psiz_Exz, 1, 2 * npml, 0, 0, 0, 0);
            arr_alloc(&g->psiz_Hyz, 1, 2 * (npml - 1), 0, 0, 0, 0);
            /* mxll_1D_mod.f90:178-200 */
            kk = npml;
            for (k = 1; k <= nx - 1; k++) {
                if (k <= npml)
                    g->den_e[2][k] = 1.0 / (kappae[k] * dr);
                else if (k >= nx + 1 - npml) {
                    g->den_e[2][k] = 1.0 / (kappae[kk] * dr);
                    kk--;
                } else
                    g->den_e[2][k] = 1.0 / dr;
            }
            kk = npml - 1;
            for (k = 1; k <= nx - 1; k++) {
                if (k <= npml - 1)
                    g->den_h[2][k] = 1.0 / (kappah[k] * dr);
                else if (k >= nx + 1 - npml) {
                    g->den_h[2][k] = 1.0 / (kappah[kk] * dr);
                    kk--;
                } else
                    g->den_h[2][k] = 1.0 / dr;
            }
        }
    } else {
        int ax_n = (dims == 3) ? 3 : 2;
        int any = 0;
        for (a = 0; a < ax_n; a++) {
            g->cpml_pos[2 * a] = g->cpml_pos[2 * a + 1] = (boundaries[a] == ORC_CPML);
            any |= (boundaries[a] == ORC_CPML);
        }
        if (any) {
            orc_cpml_tables(npml, dr, dt, g->be + 1, g->ce + 1, g->bh + 1, g->ch + 1, kappae + 1,
                            kappah + 1);
            /* den_e/den_h within the CPML (mxll_3D_mod.f90:320-420) */
            for (a = 0; a < ax_n; a++) {
                int na = n[a];
                if (!g->cpml_pos[2 * a])
                    continue;
                for (k = 1; k <= na; k++)
                    if (k <= npml)
                        g->den_e[a][k] = 1.0 / (kappae[k] * dr);
                for (k = 1; k <= na; k++)
                    if (k <= npml - 1)
                        g->den_h[a][k] = 1.0 / (kappah[k] * dr);
                kk = npml;
                for (k = 1; k <= na - 1; k++)
                    if (k >= na + 1 - npml) {
                        g->den_e[a][k] = 1.0 / (kappae[kk] * dr);
                        kk--;
                    }
                kk = npml - 1;
                for (k = 1; k <= na - 1; k++)
                    if (k >= na + 1 - npml) {
                        g->den_h[a][k] = 1.0 / (kappah[kk] * dr);
                        kk--;
                    }
            }
        }
        if (dims == 3) {
            if (g->cpml_pos[0]) {
                arr_alloc(&g->psix_Eyx, 1, 2 * npml, 1, ny, 1, nz);
                arr_alloc(&g->psix_Ezx, 1, 2 * npml, 1, ny, 1, nz);
                arr_alloc(&g->psix_Hyx, 1, 2 * (npml - 1), 1, ny, 1, nz);
                arr_alloc(&g->psix_Hzx, 1, 2 * (npml - 1), 1, ny, 1, nz);
            }
            if (g->cpml_pos[2]) {
                arr_alloc(&g->psiy_Exy, 1, nx, 1, 2 * npml, 1, nz);
                arr_alloc(&g->psiy_Ezy, 1, nx, 1, 2 * npml, 1, nz);
                arr_alloc(&g->psiy_Hxy, 1, nx, 1, 2 * (npml - 1), 1, nz);
                arr_alloc(&g->psiy_Hzy, 1, nx, 1, 2 * (npml - 1), 1, nz);
            }
            if (g->cpml_pos[4]) {
                arr_alloc(&g->psiz_Exz, 1, nx, 1, ny, 1, 2 * npml);
                arr_alloc(&g->psiz_Eyz, 1, nx, 1, ny, 1, 2 * npml);
                arr_alloc(&g->psiz_Hxz, 1, nx, 1, ny, 1, 2 * (npml - 1));
                arr_alloc(&g->psiz_Hyz, 1, nx, 1, ny, 1, 2 * (npml - 1));
            }
        } else {
            if (g->cpml_pos[0]) {
                arr_alloc(&g->psix_Eyx, 1, 2 * npml, 1, ny, 0, 0);
                arr_alloc(&g->psix_Ezx, 1, 2 * npml, 1, ny, 0, 0);
                arr_alloc(&g->psix_Hyx, 1, 2 * (npml - 1), 1, ny, 0, 0);
                arr_alloc(&g->psix_Hzx, 1, 2 * (npml - 1), 1, ny, 0, 0);
            }
            if (g->cpml_pos[2]) {
                arr_alloc(&g->psiy_Exy, 1, nx, 1, 2 * npml, 0, 0);
                arr_alloc(&g->psiy_Ezy, 1, nx, 1, 2 * npml, 0, 0);
                arr_alloc(&g->psiy_Hxy, 1, nx, 1, 2 * (npml - 1), 0, 0);
                arr_alloc(&g->psiy_Hzy, 1, nx, 1, 2 * (npml - 1), 0, 0);
            }
        }
    }
    free(kappae);
    free(kappah);
    /* media defaults: none */
    g->n_media = 0;
    g->media = (orc_medium *)calloc(1, sizeof(orc_medium));
    {
        long cells = (long)g->nx * g->ny * g->nz;
        int comps = (dims == 1) ? 1 : 3;
        g->media_map = (int32_t *)calloc((size_t)(cells * comps), sizeof(int32_t));
    }
    return g;
}

static void alloc_polarization(orc_grid *g)
{
    int c, p;
    int l2 = (g->dims == 3) ? 1 : 0, h2 = (g->dims == 3) ? g->nz : 0;
    int comps = (g->dims == 1) ? 1 : 3;
    for (c = 0; c < 3; c++) {
        arr_free(&g->PD[c]);
        for (p = 0; p < ORC_MAX_POLES; p++) {
            arr_free(&g->PL[c][p]);
            arr_free(&g->PL_old[c][p]);
        }
    }
    for (c = 0; c < comps; c++) {
        if (g->dims == 1) {
            arr_alloc(&g->PD[c], 1, g->nz, 0, 0, 0, 0);
            for (p = 0; p < g->n_max_poles; p++) {
                arr_alloc(&g->PL[c][p], 1, g->nz, 0, 0, 0, 0);
                arr_alloc(&g->PL_old[c][p], 1, g->nz, 0, 0, 0, 0);
            }
        } else {
            arr_alloc(&g->PD[c], 1, g->nx, 1, g->ny, l2, h2);
            for (p = 0; p < g->n_max_poles; p++) {
                arr_alloc(&g->PL[c][p], 1, g->nx, 1, g->ny, l2, h2);
                arr_alloc(&g->PL_old[c][p], 1, g->nx, 1, g->ny, l2, h2);
            }
        }
    }
}

int orc_grid_set_media(orc_grid *g, int n_media, const orc_medium *media, const int32_t *media_map,
                       const double *eps_x, const double *eps_y, const double *eps_z)
{
    long cells = (long)g->nx * g->ny * g->nz;
    int comps = (g->dims == 1) ? 1 : 3;
    int n, i, j, k;
    free(g->media);
    g->n_media = n_media;
    g->media = (orc_medium *)calloc((size_t)n_media + 1, sizeof(orc_medium));
    g->n_max_poles = 1;
    for (n = 1; n <= n_media; n++) {
        g->media[n] = media[n - 1];
        if (media[n - 1].medium_type == ORC_DL && media[n - 1].n_poles > g->n_max_poles)
            g->n_max_poles = media[n - 1].n_poles;
    }
    memcpy(g->media_map, media_map, sizeof(int32_t) * (size_t)(cells * comps));
    alloc_polarization(g);
    /* eps: explicit arrays or the reference's rule */
    if (eps_x || eps_y || eps_z) {
        const double *src[3] = {eps_x, eps_y, eps_z};
        arr *dst[3] = {&g->eps_x, &g->eps_y, &g->eps_z};
        int c;
        for (c = 0; c < 3; c++)
            if (src[c] && dst[c]->p)
                memcpy(dst[c]->p, src[c], sizeof(double) * (size_t)arr_size(dst[c]));
        return 0;
    }
    for (n = 1; n <= n_media; n++) {
        if (g->media[n].medium_type != ORC_DIELECTRIC)
            continue;
        if (g->dims == 3) {
            /* classical_medium_mod.f90:747-765 (eps_r stored: N6 intent) */
            for (k = 1; k <= g->nz; k++)
                for (j = 1; j <= g->ny; j++)
                    for (i = 1; i <= g->nx; i++) {
                        if (g->media_map[mm_index(g, i, j, k, 1)] == n)
                            AT(g->eps_x, i, j, k) = 1.0 / g->media[n].eps_r;
                        if (g->media_map[mm_index(g, i, j, k, 2)] == n)
                            AT(g->eps_y, i, j, k) = 1.0 / g->media[n].eps_r;
                        if (g->media_map[mm_index(g, i, j, k, 3)] == n)
                            AT(g->eps_z, i, j, k) = 1.0 / g->media[n].eps_r;
                    }
        } else if (g->dims == 2) {
            /* :526-538: all three keyed on component 1 of the map */
            for (j = 1; j <= g->ny; j++)
                for (i = 1; i <= g->nx; i++)
                    if (g->media_map[mm_index(g, i, j, 0, 1)] == n) {
                        AT(g->eps_x, i, j, 0) = 1.0 / g->media[n].eps_r;
                        AT(g->eps_y, i, j, 0) = 1.0 / g->media[n].eps_r;
                        AT(g->eps_z, i, j, 0) = 1.0 / g->media[n].eps_r;
                    }
        } else {
            /* 1D (:260-278): eps set during the voxel read for every listed voxel */
            for (i = 1; i <= g->nz; i++)
                if (g->media_map[i - 1] == n)
                    AT(g->eps_x, i, 0, 0) = 1.0 / g->media[n].eps_r;
        }
    }
    (void)cells;
    return 0;
}

void orc_grid_destroy(orc_grid *g)
{
    int c, p;
    arr *all[] = {&g->Ex, &g->Ey, &g->Ez, &g->Ex_old, &g->Ey_old, &g->Ez_old, &g->Hx, &g->Hy,
                  &g->Hz, &g->eps_x, &g->eps_y, &g->eps_z, &g->Jx, &g->Jy, &g->Jz, &g->Jx_old,
                  &g->Jy_old, &g->Jz_old, &g->dJx, &g->dJy, &g->dJz, &g->psix_Eyx, &g->psix_Ezx,
                  &g->psiy_Exy, &g->psiy_Ezy, &g->psiz_Exz, &g->psiz_Eyz, &g->psix_Hyx,
                  &g->psix_Hzx, &g->psiy_Hxy, &g->psiy_Hzy, &g->psiz_Hxz, &g->psiz_Hyz};
    size_t q;
    if (!g)
        return;
    for (q = 0; q < sizeof(all) / sizeof(all[0]); q++)
        arr_free(all[q]);
    for (c = 0; c < 3; c++) {
        arr_free(&g->PD[c]);
        for (p = 0; p < ORC_MAX_POLES; p++) {
            arr_free(&g->PL[c][p]);
            arr_free(&g->PL_old[c][p]);
        }
        free(g->den_e[c]);
        free(g->den_h[c]);
    }
    free(g->be); free(g->ce); free(g->bh); free(g->ch);
    free(g->media);
    free(g->media_map);
    free(g);
}

void orc_grid_set_time(orc_grid *g, double time, double t_skip)
{
    g->time = time;
    g->t_skip = t_skip;
}

static arr *field_arr(const orc_grid *g, int field)
{
    orc_grid *m = (orc_grid *)g;
    switch (field) {
    case ORC_EX: return &m->Ex;
    case ORC_EY: return &m->Ey;
    case ORC_EZ: return &m->Ez;
    case ORC_HX: return &m->Hx;
    case ORC_HY: return &m->Hy;
    case ORC_HZ: return &m->Hz;
    }
    return NULL;
}

long orc_field_size(const orc_grid *g, int field)
{
    arr *a = field_arr(g, field);
    return a ? arr_size(a) : -1;
}
long orc_field_get(const orc_grid *g, int field, double *out)
{
    arr *a = field_arr(g, field);
    long s;
    if (!a || !a->p)
        return -1;
    s = arr_size(a);
    memcpy(out, a->p, sizeof(double) * (size_t)s);
    return s;
}
long orc_field_set(orc_grid *g, int field, const double *in)
{
    arr *a = field_arr(g, field);
    long s;
    if (!a || !a->p)
        return -1;
    s = arr_size(a);
    memcpy(a->p, in, sizeof(double) * (size_t)s);
    return s;
}
int orc_field_bounds(const orc_grid *g, int field, int lo[3], int hi[3])
{
    arr *a = field_arr(g, field);
    int q;
    if (!a || !a->p)
        return -1;
    for (q = 0; q < 3; q++) {
        lo[q] = a->lo[q];
        hi[q] = a->hi[q];
    }
    return 0;
}
void orc_get_den(const orc_grid *g, double *den_e, double *den_h)
{
    int n[3] = {g->nx, g->ny, g->nz};
    int a, k, off = 0;
    for (a = 0; a < 3; a++) {
        for (k = 1; k <= n[a]; k++) {
            den_e[off + k - 1] = g->den_e[a][k];
            den_h[off + k - 1] = g->den_h[a][k];
        }
        off += n[a];
    }
}

/* ======================================================================================= */
/* get_medium_polarization (classical_medium_mod.f90:773-833)                               */
/* ======================================================================================= */

static int medium_polarization(const orc_grid *g, int idx, double *PDi, double **PLi,
                               double **PLi_old, double *Ei, double *Ei_old, double rotH)
{
    const orc_medium *m;
    if (idx == 0)
        return 1; /* no_medium */
    m = &g->media[idx];
    if (m->medium_type == ORC_DRUDE) {
        double tmpE = m->C1 * *Ei + m->C3 * rotH - m->C4 * *PDi;
        *PDi = m->A1 * *PDi + m->A2 * (tmpE + *Ei);
        *Ei = tmpE;
        return 0;
    }
    if (m->medium_type == ORC_DL) {
        double tmpE = m->C1 * *Ei + m->C2 * *Ei_old + m->C3 * rotH - m->C4 * *PDi;
        double tmpPL[ORC_MAX_POLES];
        int i;
        for (i = 0; i < m->n_poles; i++)
            tmpE = tmpE - m->B1_k[i] * *PLi[i] - m->B2_k[i] * *PLi_old[i];
        *PDi = m->A1 * *PDi + m->A2 * (tmpE + *Ei);
        for (i = 0; i < m->n_poles; i++)
            tmpPL[i] = m->alpha_k[i] * *PLi[i] + m->beta_k[i] * *PLi_old[i] +
                       m->gamma_k[i] * (tmpE - *Ei_old);
        *Ei_old = *Ei;
        for (i = 0; i < m->n_poles; i++) {
            *PLi_old[i] = *PLi[i];
            *PLi[i] = tmpPL[i];
        }
        *Ei = tmpE;
        return 0;
    }
    return 1; /* dielectric */
}

/* ======================================================================================= */
/* 3D propagation (mxll_3D_mod.f90:505-923)                                                 */
/* ======================================================================================= */

static void propagate_H_3d(orc_grid *g)
{
    const int nx = g->nx, ny = g->ny, nz = g->nz, npml = g->npml, n_sec = g->n_sec;
    const int n_base = (n_sec == 1) ? 0 : npml - 1;
    const double dt_mu0 = g->dt_mu0, dr = g->dr;
    const double *den_hx = g->den_h[0], *den_hy = g->den_h[1], *den_hz = g->den_h[2];
    const double *bh = g->bh, *ch = g->ch;
    int i, j, k, ii, jj, kk;

    /* periodic wraps :528-541 */
    if (g->boundaries[0] == ORC_PERIODIC) {
        for (k = g->Ez.lo[2]; k <= g->Ez.hi[2]; k++)
            for (j = g->Ez.lo[1]; j <= g->Ez.hi[1]; j++)
                AT(g->Ez, nx + 1, j, k) = AT(g->Ez, 1, j, k);
        for (k = g->Ey.lo[2]; k <= g->Ey.hi[2]; k++)
            for (j = g->Ey.lo[1]; j <= g->Ey.hi[1]; j++)
                AT(g->Ey, nx + 1, j, k) = AT(g->Ey, 1, j, k);
    }
    if (g->boundaries[1] == ORC_PERIODIC) {
        for (k = g->Ex.lo[2]; k <= g->Ex.hi[2]; k++)
            for (i = g->Ex.lo[0]; i <= g->Ex.hi[0]; i++)
                AT(g->Ex, i, ny + 1, k) = AT(g->Ex, i, 1, k);
        for (k = g->Ez.lo[2]; k <= g->Ez.hi[2]; k++)
            for (i = g->Ez.lo[0]; i <= g->Ez.hi[0]; i++)
                AT(g->Ez, i, ny + 1, k) = AT(g->Ez, i, 1, k);
    }
    if (g->boundaries[2] == ORC_PERIODIC) {
        for (j = g->Ex.lo[1]; j <= g->Ex.hi[1]; j++)
            for (i = g->Ex.lo[0]; i <= g->Ex.hi[0]; i++)
                AT(g->Ex, i, j, nz + 1) = AT(g->Ex, i, j, 1);
        for (j = g->Ey.lo[1]; j <= g->Ey.hi[1]; j++)
            for (i = g->Ey.lo[0]; i <= g->Ey.hi[0]; i++)
                AT(g->Ey, i, j, nz + 1) = AT(g->Ey, i, j, 1);
    }

#pragma omp parallel for collapse(2) schedule(static) private(i)
    for (k = 1; k <= nz; k++)
        for (j = 1; j <= ny; j++)
            for (i = 1; i <= nx; i++) {
                double rotE;
                rotE = (AT(g->Ez, i, j, k) - AT(g->Ez, i, j + 1, k)) * den_hy[j] +
                       (AT(g->Ey, i, j, k + 1) - AT(g->Ey, i, j, k)) * den_hz[k];
                AT(g->Hx, i, j, k) = AT(g->Hx, i, j, k) + dt_mu0 * rotE;
                rotE = (AT(g->Ez, i + 1, j, k) - AT(g->Ez, i, j, k)) * den_hx[i] +
                       (AT(g->Ex, i, j, k) - AT(g->Ex, i, j, k + 1)) * den_hz[k];
                AT(g->Hy, i, j, k) = AT(g->Hy, i, j, k) + dt_mu0 * rotE;
                rotE = (AT(g->Ey, i, j, k) - AT(g->Ey, i + 1, j, k)) * den_hx[i] +
                       (AT(g->Ex, i, j + 1, k) - AT(g->Ex, i, j, k)) * den_hy[j];
                AT(g->Hz, i, j, k) = AT(g->Hz, i, j, k) + dt_mu0 * rotE;
            }

    if (g->cpml_pos[0]) /* :585-600 */
        for (j = 1; j <= ny; j++)
            for (k = 1; k <= nz; k++)
                for (i = 1; i <= npml - 1; i++) {
                    AT(g->psix_Hyx, i, j, k) = bh[i] * AT(g->psix_Hyx, i, j, k) +
                                               ch[i] * (AT(g->Ez, i + 1, j, k) - AT(g->Ez, i, j, k)) / dr;
                    AT(g->psix_Hzx, i, j, k) = bh[i] * AT(g->psix_Hzx, i, j, k) +
                                               ch[i] * (AT(g->Ey, i, j, k) - AT(g->Ey, i + 1, j, k)) / dr;
                    AT(g->Hy, i, j, k) = AT(g->Hy, i, j, k) + dt_mu0 * AT(g->psix_Hyx, i, j, k);
                    AT(g->Hz, i, j, k) = AT(g->Hz, i, j, k) + dt_mu0 * AT(g->psix_Hzx, i, j, k);
                }
    if (g->cpml_pos[1]) /* :602-620 */
        for (j = 1; j <= ny; j++)
            for (k = 1; k <= nz; k++) {
                ii = n_sec * (npml - 1);
                for (i = nx + 1 - npml; i <= nx - 1; i++) {
                    AT(g->psix_Hyx, ii, j, k) = bh[ii - n_base] * AT(g->psix_Hyx, ii, j, k) +
                                                ch[ii - n_base] * (AT(g->Ez, i + 1, j, k) - AT(g->Ez, i, j, k)) / dr;
                    AT(g->psix_Hzx, ii, j, k) = bh[ii - n_base] * AT(g->psix_Hzx, ii, j, k) +
                                                ch[ii - n_base] * (AT(g->Ey, i, j, k) - AT(g->Ey, i + 1, j, k)) / dr;
                    AT(g->Hy, i, j, k) = AT(g->Hy, i, j, k) + dt_mu0 * AT(g->psix_Hyx, ii, j, k);
                    AT(g->Hz, i, j, k) = AT(g->Hz, i, j, k) + dt_mu0 * AT(g->psix_Hzx, ii, j, k);
                    ii--;
                }
            }
    if (g->cpml_pos[2]) /* :622-637 */
        for (k = 1; k <= nz; k++)
            for (i = 1; i <= nx; i++)
                for (j = 1; j <= npml - 1; j++) {
                    AT(g->psiy_Hxy, i, j, k) = bh[j] * AT(g->psiy_Hxy, i, j, k) +
                                               ch[j] * (AT(g->Ez, i, j, k) - AT(g->Ez, i, j + 1, k)) / dr;
                    AT(g->psiy_Hzy, i, j, k) = bh[j] * AT(g->psiy_Hzy, i, j, k) +
                                               ch[j] * (AT(g->Ex, i, j + 1, k) - AT(g->Ex, i, j, k)) / dr;
                    AT(g->Hx, i, j, k) = AT(g->Hx, i, j, k) + dt_mu0 * AT(g->psiy_Hxy, i, j, k);
                    AT(g->Hz, i, j, k) = AT(g->Hz, i, j, k) + dt_mu0 * AT(g->psiy_Hzy, i, j, k);
                }
    if (g->cpml_pos[3]) /* :639-657 */
        for (k = 1; k <= nz; k++)
            for (i = 1; i <= nx; i++) {
                jj = n_sec * (npml - 1);
                for (j = ny + 1 - npml; j <= ny - 1; j++) {
                    AT(g->psiy_Hxy, i, jj, k) = bh[jj - n_base] * AT(g->psiy_Hxy, i, jj, k) +
                                                ch[jj - n_base] * (AT(g->Ez, i, j, k) - AT(g->Ez, i, j + 1, k)) / dr;
                    AT(g->psiy_Hzy, i, jj, k) = bh[jj - n_base] * AT(g->psiy_Hzy, i, jj, k) +
                                                ch[jj - n_base] * (AT(g->Ex, i, j + 1, k) - AT(g->Ex, i, j, k)) / dr;
                    AT(g->Hx, i, j, k) = AT(g->Hx, i, j, k) + dt_mu0 * AT(g->psiy_Hxy, i, jj, k);
                    AT(g->Hz, i, j, k) = AT(g->Hz, i, j, k) + dt_mu0 * AT(g->psiy_Hzy, i, jj, k);
                    jj--;
                }
            }
    if (g->cpml_pos[4]) /* :659-674 */
        for (i = 1; i <= nx; i++)
            for (j = 1; j <= ny; j++)
                for (k = 1; k <= npml - 1; k++) {
                    AT(g->psiz_Hxz, i, j, k) = bh[k] * AT(g->psiz_Hxz, i, j, k) +
                                               ch[k] * (AT(g->Ey, i, j, k + 1) - AT(g->Ey, i, j, k)) / dr;
                    AT(g->psiz_Hyz, i, j, k) = bh[k] * AT(g->psiz_Hyz, i, j, k) +
                                               ch[k] * (AT(g->Ex, i, j, k) - AT(g->Ex, i, j, k + 1)) / dr;
                    AT(g->Hx, i, j, k) = AT(g->Hx, i, j, k) + dt_mu0 * AT(g->psiz_Hxz, i, j, k);
                    AT(g->Hy, i, j, k) = AT(g->Hy, i, j, k) + dt_mu0 * AT(g->psiz_Hyz, i, j, k);
                }
    if (g->cpml_pos[5]) /* :676-694 */
        for (i = 1; i <= nx; i++)
            for (j = 1; j <= ny; j++) {
                kk = n_sec * (npml - 1);
                for (k = nz + 1 - npml; k <= nz - 1; k++) {
                    AT(g->psiz_Hxz, i, j, kk) = bh[kk - n_base] * AT(g->psiz_Hxz, i, j, kk) +
                                                ch[kk - n_base] * (AT(g->Ey, i, j, k + 1) - AT(g->Ey, i, j, k)) / dr;
                    AT(g->psiz_Hyz, i, j, kk) = bh[kk - n_base] * AT(g->psiz_Hyz, i, j, kk) +
                                                ch[kk - n_base] * (AT(g->Ex, i, j, k) - AT(g->Ex, i, j, k + 1)) / dr;
                    AT(g->Hx, i, j, k) = AT(g->Hx, i, j, k) + dt_mu0 * AT(g->psiz_Hxz, i, j, kk);
                    AT(g->Hy, i, j, k) = AT(g->Hy, i, j, k) + dt_mu0 * AT(g->psiz_Hyz, i, j, kk);
                    kk--;
                }
            }
}

static void pol_ptrs(orc_grid *g, int c, int i, int j, int k, double **pl, double **plo)
{
    int p;
    for (p = 0; p < g->n_max_poles; p++) {
        pl[p] = &AT(g->PL[c][p], i, j, k);
        plo[p] = &AT(g->PL_old[c][p], i, j, k);
    }
}

static void propagate_E_3d(orc_grid *g)
{
    const int nx = g->nx, ny = g->ny, nz = g->nz, npml = g->npml, n_sec = g->n_sec;
    const int n_base = (n_sec == 1) ? 0 : npml;
    const double dt_eps0 = g->dt_eps0, dr = g->dr;
    const double *den_ex = g->den_e[0], *den_ey = g->den_e[1], *den_ez = g->den_e[2];
    const double *be = g->be, *ce = g->ce;
    const double tt = g->time - g->t_skip;
    int i, j, k, ii, jj, kk;

    /* periodic wraps :725-738 */
    if (g->boundaries[0] == ORC_PERIODIC) {
        for (k = g->Hy.lo[2]; k <= g->Hy.hi[2]; k++)
            for (j = g->Hy.lo[1]; j <= g->Hy.hi[1]; j++)
                AT(g->Hy, 0, j, k) = AT(g->Hy, nx, j, k);
        for (k = g->Hz.lo[2]; k <= g->Hz.hi[2]; k++)
            for (j = g->Hz.lo[1]; j <= g->Hz.hi[1]; j++)
                AT(g->Hz, 0, j, k) = AT(g->Hz, nx, j, k);
    }
    if (g->boundaries[1] == ORC_PERIODIC) {
        for (k = g->Hx.lo[2]; k <= g->Hx.hi[2]; k++)
            for (i = g->Hx.lo[0]; i <= g->Hx.hi[0]; i++)
                AT(g->Hx, i, 0, k) = AT(g->Hx, i, ny, k);
        for (k = g->Hz.lo[2]; k <= g->Hz.hi[2]; k++)
            for (i = g->Hz.lo[0]; i <= g->Hz.hi[0]; i++)
                AT(g->Hz, i, 0, k) = AT(g->Hz, i, ny, k);
    }
    if (g->boundaries[2] == ORC_PERIODIC) {
        for (j = g->Hx.lo[1]; j <= g->Hx.hi[1]; j++)
            for (i = g->Hx.lo[0]; i <= g->Hx.hi[0]; i++)
                AT(g->Hx, i, j, 0) = AT(g->Hx, i, j, nz);
        for (j = g->Hy.lo[1]; j <= g->Hy.hi[1]; j++)
            for (i = g->Hy.lo[0]; i <= g->Hy.hi[0]; i++)
                AT(g->Hy, i, j, 0) = AT(g->Hy, i, j, nz);
    }

#pragma omp parallel for collapse(2) schedule(static) private(i)
    for (k = 1; k <= nz; k++)
        for (j = 1; j <= ny; j++)
            for (i = 1; i <= nx; i++) {
                double rotH, Jav;
                double *pl[ORC_MAX_POLES], *plo[ORC_MAX_POLES];
                /* Ex :745-764 */
                rotH = (AT(g->Hz, i, j, k) - AT(g->Hz, i, j - 1, k)) * den_ey[j] +
                       (AT(g->Hy, i, j, k - 1) - AT(g->Hy, i, j, k)) * den_ez[k];
                pol_ptrs(g, 0, i, j, k, pl, plo);
                if (medium_polarization(g, g->media_map[mm_index(g, i, j, k, 1)], &AT(g->PD[0], i, j, k),
                                        pl, plo, &AT(g->Ex, i, j, k), &AT(g->Ex_old, i, j, k), rotH)) {
                    Jav = 0.5 * (AT(g->Jx_old, i, j, k) + tt * AT(g->dJx, i, j, k) +
                                 AT(g->Jx_old, i + 1, j, k) + tt * AT(g->dJx, i + 1, j, k));
                    AT(g->Ex, i, j, k) = AT(g->Ex, i, j, k) + dt_eps0 * AT(g->eps_x, i, j, k) * rotH -
                                         dt_eps0 * Jav;
                }
                /* Ey :767-789 */
                rotH = (AT(g->Hz, i - 1, j, k) - AT(g->Hz, i, j, k)) * den_ex[i] +
                       (AT(g->Hx, i, j, k) - AT(g->Hx, i, j, k - 1)) * den_ez[k];
                pol_ptrs(g, 1, i, j, k, pl, plo);
                if (medium_polarization(g, g->media_map[mm_index(g, i, j, k, 2)], &AT(g->PD[1], i, j, k),
                                        pl, plo, &AT(g->Ey, i, j, k), &AT(g->Ey_old, i, j, k), rotH)) {
                    Jav = 0.5 * (AT(g->Jy_old, i, j, k) + tt * AT(g->dJy, i, j, k) +
                                 AT(g->Jy_old, i, j + 1, k) + tt * AT(g->dJy, i, j + 1, k));
                    AT(g->Ey, i, j, k) = AT(g->Ey, i, j, k) + dt_eps0 * AT(g->eps_y, i, j, k) * rotH -
                                         dt_eps0 * Jav;
                }
                /* Ez :791-812 */
                rotH = (AT(g->Hy, i, j, k) - AT(g->Hy, i - 1, j, k)) * den_ex[i] +
                       (AT(g->Hx, i, j - 1, k) - AT(g->Hx, i, j, k)) * den_ey[j];
                pol_ptrs(g, 2, i, j, k, pl, plo);
                if (medium_polarization(g, g->media_map[mm_index(g, i, j, k, 3)], &AT(g->PD[2], i, j, k),
                                        pl, plo, &AT(g->Ez, i, j, k), &AT(g->Ez_old, i, j, k), rotH)) {
                    Jav = 0.5 * (AT(g->Jz_old, i, j, k) + tt * AT(g->dJz, i, j, k) +
                                 AT(g->Jz_old, i, j, k + 1) + tt * AT(g->dJz, i, j, k + 1));
                    AT(g->Ez, i, j, k) = AT(g->Ez, i, j, k) + dt_eps0 * AT(g->eps_z, i, j, k) * rotH -
                                         dt_eps0 * Jav;
                }
            }

    if (g->cpml_pos[0]) /* :817-831 */
        for (j = 1; j <= ny; j++)
            for (k = 1; k <= nz; k++)
                for (i = 2; i <= npml; i++) {
                    AT(g->psix_Eyx, i, j, k) = be[i] * AT(g->psix_Eyx, i, j, k) +
                                               ce[i] * (AT(g->Hz, i - 1, j, k) - AT(g->Hz, i, j, k)) / dr;
                    AT(g->psix_Ezx, i, j, k) = be[i] * AT(g->psix_Ezx, i, j, k) +
                                               ce[i] * (AT(g->Hy, i, j, k) - AT(g->Hy, i - 1, j, k)) / dr;
                    AT(g->Ey, i, j, k) = AT(g->Ey, i, j, k) + dt_eps0 * AT(g->psix_Eyx, i, j, k);
                    AT(g->Ez, i, j, k) = AT(g->Ez, i, j, k) + dt_eps0 * AT(g->psix_Ezx, i, j, k);
                }
    if (g->cpml_pos[1]) /* :833-849 */
        for (j = 1; j <= ny; j++)
            for (k = 1; k <= nz; k++) {
                ii = n_sec * npml;
                for (i = nx + 1 - npml; i <= nx - 1; i++) {
                    AT(g->psix_Eyx, ii, j, k) = be[ii - n_base] * AT(g->psix_Eyx, ii, j, k) +
                                                ce[ii - n_base] * (AT(g->Hz, i - 1, j, k) - AT(g->Hz, i, j, k)) / dr;
                    AT(g->psix_Ezx, ii, j, k) = be[ii - n_base] * AT(g->psix_Ezx, ii, j, k) +
                                                ce[ii - n_base] * (AT(g->Hy, i, j, k) - AT(g->Hy, i - 1, j, k)) / dr;
                    AT(g->Ey, i, j, k) = AT(g->Ey, i, j, k) + dt_eps0 * AT(g->psix_Eyx, ii, j, k);
                    AT(g->Ez, i, j, k) = AT(g->Ez, i, j, k) + dt_eps0 * AT(g->psix_Ezx, ii, j, k);
                    ii--;
                }
            }
    if (g->cpml_pos[2]) /* :851-866 */
        for (k = 1; k <= nz; k++)
            for (i = 1; i <= nx; i++)
                for (j = 2; j <= npml; j++) {
                    AT(g->psiy_Exy, i, j, k) = be[j] * AT(g->psiy_Exy, i, j, k) +
                                               ce[j] * (AT(g->Hz, i, j, k) - AT(g->Hz, i, j - 1, k)) / dr;
                    AT(g->psiy_Ezy, i, j, k) = be[j] * AT(g->psiy_Ezy, i, j, k) +
                                               ce[j] * (AT(g->Hx, i, j - 1, k) - AT(g->Hx, i, j, k)) / dr;
                    AT(g->Ex, i, j, k) = AT(g->Ex, i, j, k) + dt_eps0 * AT(g->psiy_Exy, i, j, k);
                    AT(g->Ez, i, j, k) = AT(g->Ez, i, j, k) + dt_eps0 * AT(g->psiy_Ezy, i, j, k);
                }
    if (g->cpml_pos[3]) /* :868-885 */
        for (k = 1; k <= nz; k++)
            for (i = 1; i <= nx; i++) {
                jj = n_sec * npml;
                for (j = ny + 1 - npml; j <= ny - 1; j++) {
                    AT(g->psiy_Exy, i, jj, k) = be[jj - n_base] * AT(g->psiy_Exy, i, jj, k) +
                                                ce[jj - n_base] * (AT(g->Hz, i, j, k) - AT(g->Hz, i, j - 1, k)) / dr;
                    AT(g->psiy_Ezy, i, jj, k) = be[jj - n_base] * AT(g->psiy_Ezy, i, jj, k) +
                                                ce[jj - n_base] * (AT(g->Hx, i, j - 1, k) - AT(g->Hx, i, j, k)) / dr;
                    AT(g->Ex, i, j, k) = AT(g->Ex, i, j, k) + dt_eps0 * AT(g->psiy_Exy, i, jj, k);
                    AT(g->Ez, i, j, k) = AT(g->Ez, i, j, k) + dt_eps0 * AT(g->psiy_Ezy, i, jj, k);
                    jj--;
                }
            }
    if (g->cpml_pos[4]) /* :887-902 */
        for (i = 1; i <= nx; i++)
            for (j = 1; j <= ny; j++)
                for (k = 2; k <= npml; k++) {
                    AT(g->psiz_Exz, i, j, k) = be[k] * AT(g->psiz_Exz, i, j, k) +
                                               ce[k] * (AT(g->Hy, i, j, k - 1) - AT(g->Hy, i, j, k)) / dr;
                    AT(g->psiz_Eyz, i, j, k) = be[k] * AT(g->psiz_Eyz, i, j, k) +
                                               ce[k] * (AT(g->Hx, i, j, k) - AT(g->Hx, i, j, k - 1)) / dr;
                    AT(g->Ex, i, j, k) = AT(g->Ex, i, j, k) + dt_eps0 * AT(g->psiz_Exz, i, j, k);
                    AT(g->Ey, i, j, k) = AT(g->Ey, i, j, k) + dt_eps0 * AT(g->psiz_Eyz, i, j, k);
                }
    if (g->cpml_pos[5]) /* :904-921 */
        for (i = 1; i <= nx; i++)
            for (j = 1; j <= ny; j++) {
                kk = n_sec * npml;
                for (k = nz + 1 - npml; k <= nz - 1; k++) {
                    AT(g->psiz_Exz, i, j, kk) = be[kk - n_base] * AT(g->psiz_Exz, i, j, kk) +
                                                ce[kk - n_base] * (AT(g->Hy, i, j, k - 1) - AT(g->Hy, i, j, k)) / dr;
                    AT(g->psiz_Eyz, i, j, kk) = be[kk - n_base] * AT(g->psiz_Eyz, i, j, kk) +
                                                ce[kk - n_base] * (AT(g->Hx, i, j, k) - AT(g->Hx, i, j, k - 1)) / dr;
                    AT(g->Ex, i, j, k) = AT(g->Ex, i, j, k) + dt_eps0 * AT(g->psiz_Exz, i, j, kk);
                    AT(g->Ey, i, j, k) = AT(g->Ey, i, j, k) + dt_eps0 * AT(g->psiz_Eyz, i, j, kk);
                    kk--;
                }
            }
}

/* ======================================================================================= */
/* 2D propagation (mxll_2D_mod.f90:450-864); arrays carry k == 0                             */
/* ======================================================================================= */

static void propagate_H_2d(orc_grid *g)
{
    const int nx = g->nx, ny = g->ny, npml = g->npml, n_sec = g->n_sec;
    const int n_base = (n_sec == 1) ? 0 : npml - 1;
    const double dt_mu0 = g->dt_mu0, dr = g->dr;
    const double *den_hx = g->den_h[0], *den_hy = g->den_h[1];
    const double *bh = g->bh, *ch = g->ch;
    int i, j, ii, jj;
    double rotE;
    if (g->mode == ORC_TMZ) {
        if (g->boundaries[0] == ORC_PERIODIC) /* :475-481 */
            for (j = 1; j <= ny + 1; j++)
                AT(g->Ez, nx + 1, j, 0) = AT(g->Ez, 1, j, 0);
        if (g->boundaries[1] == ORC_PERIODIC)
            for (i = 1; i <= nx + 1; i++)
                AT(g->Ez, i, ny + 1, 0) = AT(g->Ez, i, 1, 0);
#pragma omp parallel for schedule(static) private(i)
        for (j = 1; j <= ny; j++)
            for (i = 1; i <= nx; i++) {
                double r;
                r = (AT(g->Ez, i, j, 0) - AT(g->Ez, i, j + 1, 0)) * den_hy[j];
                AT(g->Hx, i, j, 0) = AT(g->Hx, i, j, 0) + dt_mu0 * r;
                r = (AT(g->Ez, i + 1, j, 0) - AT(g->Ez, i, j, 0)) * den_hx[i];
                AT(g->Hy, i, j, 0) = AT(g->Hy, i, j, 0) + dt_mu0 * r;
            }
        if (g->cpml_pos[0]) /* :504-513 */
            for (j = 1; j <= ny; j++)
                for (i = 1; i <= npml - 1; i++) {
                    rotE = (AT(g->Ez, i + 1, j, 0) - AT(g->Ez, i, j, 0)) / dr;
                    AT(g->psix_Hyx, i, j, 0) = bh[i] * AT(g->psix_Hyx, i, j, 0) + ch[i] * rotE;
                    AT(g->Hy, i, j, 0) = AT(g->Hy, i, j, 0) + dt_mu0 * AT(g->psix_Hyx, i, j, 0);
                }
        if (g->cpml_pos[1]) /* :515-527 */
            for (j = 1; j <= ny; j++) {
                ii = n_sec * (npml - 1);
                for (i = nx + 1 - npml; i <= nx - 1; i++) {
                    rotE = (AT(g->Ez, i + 1, j, 0) - AT(g->Ez, i, j, 0)) / dr;
                    AT(g->psix_Hyx, ii, j, 0) = bh[ii - n_base] * AT(g->psix_Hyx, ii, j, 0) + ch[ii - n_base] * rotE;
                    AT(g->Hy, i, j, 0) = AT(g->Hy, i, j, 0) + dt_mu0 * AT(g->psix_Hyx, ii, j, 0);
                    ii--;
                }
            }
        if (g->cpml_pos[2]) /* :529-538 */
            for (i = 1; i <= nx; i++)
                for (j = 1; j <= npml - 1; j++) {
                    rotE = (AT(g->Ez, i, j, 0) - AT(g->Ez, i, j + 1, 0)) / dr;
                    AT(g->psiy_Hxy, i, j, 0) = bh[j] * AT(g->psiy_Hxy, i, j, 0) + ch[j] * rotE;
                    AT(g->Hx, i, j, 0) = AT(g->Hx, i, j, 0) + dt_mu0 * AT(g->psiy_Hxy, i, j, 0);
                }
        if (g->cpml_pos[3]) /* :540-552 */
            for (i = 1; i <= nx; i++) {
                jj = n_sec * (npml - 1);
                for (j = ny + 1 - npml; j <= ny - 1; j++) {
                    rotE = (AT(g->Ez, i, j, 0) - AT(g->Ez, i, j + 1, 0)) / dr;
                    AT(g->psiy_Hxy, i, jj, 0) = bh[jj - n_base] * AT(g->psiy_Hxy, i, jj, 0) + ch[jj - n_base] * rotE;
                    AT(g->Hx, i, j, 0) = AT(g->Hx, i, j, 0) + dt_mu0 * AT(g->psiy_Hxy, i, jj, 0);
                    jj--;
                }
            }
    } else {
        if (g->boundaries[0] == ORC_PERIODIC) /* :561-567 */
            for (j = 0; j <= ny; j++)
                AT(g->Ey, nx + 1, j, 0) = AT(g->Ey, 1, j, 0);
        if (g->boundaries[1] == ORC_PERIODIC)
            for (i = 0; i <= nx; i++)
                AT(g->Ex, i, ny + 1, 0) = AT(g->Ex, i, 1, 0);
#pragma omp parallel for schedule(static) private(i)
        for (j = 1; j <= ny; j++)
            for (i = 1; i <= nx; i++) {
                double r = (AT(g->Ey, i, j, 0) - AT(g->Ey, i + 1, j, 0)) * den_hx[i] +
                           (AT(g->Ex, i, j + 1, 0) - AT(g->Ex, i, j, 0)) * den_hy[j];
                AT(g->Hz, i, j, 0) = AT(g->Hz, i, j, 0) + dt_mu0 * r;
            }
        if (g->cpml_pos[0])
            for (j = 1; j <= ny; j++)
                for (i = 1; i <= npml - 1; i++) {
                    rotE = (AT(g->Ey, i, j, 0) - AT(g->Ey, i + 1, j, 0)) / dr;
                    AT(g->psix_Hzx, i, j, 0) = bh[i] * AT(g->psix_Hzx, i, j, 0) + ch[i] * rotE;
                    AT(g->Hz, i, j, 0) = AT(g->Hz, i, j, 0) + dt_mu0 * AT(g->psix_Hzx, i, j, 0);
                }
        if (g->cpml_pos[1])
            for (j = 1; j <= ny; j++) {
                ii = n_sec * (npml - 1);
                for (i = nx + 1 - npml; i <= nx - 1; i++) {
                    rotE = (AT(g->Ey, i, j, 0) - AT(g->Ey, i + 1, j, 0)) / dr;
                    AT(g->psix_Hzx, ii, j, 0) = bh[ii - n_base] * AT(g->psix_Hzx, ii, j, 0) + ch[ii - n_base] * rotE;
                    AT(g->Hz, i, j, 0) = AT(g->Hz, i, j, 0) + dt_mu0 * AT(g->psix_Hzx, ii, j, 0);
                    ii--;
                }
            }
        if (g->cpml_pos[2])
            for (i = 1; i <= nx; i++)
                for (j = 1; j <= npml - 1; j++) {
                    rotE = (AT(g->Ex, i, j + 1, 0) - AT(g->Ex, i, j, 0)) / dr;
                    AT(g->psiy_Hzy, i, j, 0) = bh[j] * AT(g->psiy_Hzy, i, j, 0) + ch[j] * rotE;
                    AT(g->Hz, i, j, 0) = AT(g->Hz, i, j, 0) + dt_mu0 * AT(g->psiy_Hzy, i, j, 0);
                }
        if (g->cpml_pos[3])
            for (i = 1; i <= nx; i++) {
                jj = n_sec * (npml - 1);
                for (j = ny + 1 - npml; j <= ny - 1; j++) {
                    rotE = (AT(g->Ex, i, j + 1, 0) - AT(g->Ex, i, j, 0)) / dr;
                    AT(g->psiy_Hzy, i, jj, 0) = bh[jj - n_base] * AT(g->psiy_Hzy, i, jj, 0) + ch[jj - n_base] * rotE;
                    AT(g->Hz, i, j, 0) = AT(g->Hz, i, j, 0) + dt_mu0 * AT(g->psiy_Hzy, i, jj, 0);
                    jj--;
                }
            }
    }
}

static void propagate_E_2d(orc_grid *g)
{
    const int nx = g->nx, ny = g->ny, npml = g->npml, n_sec = g->n_sec;
    const int n_base = (n_sec == 1) ? 0 : npml;
    const double dt_eps0 = g->dt_eps0, dr = g->dr;
    const double *den_ex = g->den_e[0], *den_ey = g->den_e[1];
    const double *be = g->be, *ce = g->ce;
    const double tt = g->time - g->t_skip;
    int i, j, ii, jj;
    double rotH;
    if (g->mode == ORC_TMZ) {
        if (g->boundaries[0] == ORC_PERIODIC) /* :666-672 */
            for (j = 1; j <= ny; j++)
                AT(g->Hy, 0, j, 0) = AT(g->Hy, nx, j, 0);
        if (g->boundaries[1] == ORC_PERIODIC)
            for (i = 1; i <= nx; i++)
                AT(g->Hx, i, 0, 0) = AT(g->Hx, i, ny, 0);
#pragma omp parallel for schedule(static) private(i)
        for (j = 1; j <= ny; j++)
            for (i = 1; i <= nx; i++) {
                double *pl[ORC_MAX_POLES], *plo[ORC_MAX_POLES];
                double r = (AT(g->Hy, i, j, 0) - AT(g->Hy, i - 1, j, 0)) * den_ex[i] +
                           (AT(g->Hx, i, j - 1, 0) - AT(g->Hx, i, j, 0)) * den_ey[j];
                pol_ptrs(g, 2, i, j, 0, pl, plo);
                if (medium_polarization(g, g->media_map[mm_index(g, i, j, 0, 3)], &AT(g->PD[2], i, j, 0),
                                        pl, plo, &AT(g->Ez, i, j, 0), &AT(g->Ez_old, i, j, 0), r)) {
                    double Jav = AT(g->Jz_old, i, j, 0) + tt * AT(g->dJz, i, j, 0);
                    AT(g->Ez, i, j, 0) = AT(g->Ez, i, j, 0) + dt_eps0 * AT(g->eps_z, i, j, 0) * r - dt_eps0 * Jav;
                }
            }
        if (g->cpml_pos[0]) /* :699-707 */
            for (j = 1; j <= ny; j++)
                for (i = 2; i <= npml; i++) {
                    rotH = (AT(g->Hy, i, j, 0) - AT(g->Hy, i - 1, j, 0)) / dr;
                    AT(g->psix_Ezx, i, j, 0) = be[i] * AT(g->psix_Ezx, i, j, 0) + ce[i] * rotH;
                    AT(g->Ez, i, j, 0) = AT(g->Ez, i, j, 0) + dt_eps0 * AT(g->psix_Ezx, i, j, 0);
                }
        if (g->cpml_pos[1]) /* :709-721 */
            for (j = 1; j <= ny; j++) {
                ii = n_sec * npml;
                for (i = nx + 1 - npml; i <= nx - 1; i++) {
                    rotH = (AT(g->Hy, i, j, 0) - AT(g->Hy, i - 1, j, 0)) / dr;
                    AT(g->psix_Ezx, ii, j, 0) = be[ii - n_base] * AT(g->psix_Ezx, ii, j, 0) + ce[ii - n_base] * rotH;
                    AT(g->Ez, i, j, 0) = AT(g->Ez, i, j, 0) + dt_eps0 * AT(g->psix_Ezx, ii, j, 0);
                    ii--;
                }
            }
        if (g->cpml_pos[2]) /* :723-733 */
            for (i = 1; i <= nx; i++)
                for (j = 2; j <= npml; j++) {
                    rotH = (AT(g->Hx, i, j - 1, 0) - AT(g->Hx, i, j, 0)) / dr;
                    AT(g->psiy_Ezy, i, j, 0) = be[j] * AT(g->psiy_Ezy, i, j, 0) + ce[j] * rotH;
                    AT(g->Ez, i, j, 0) = AT(g->Ez, i, j, 0) + dt_eps0 * AT(g->psiy_Ezy, i, j, 0);
                }
        if (g->cpml_pos[3]) /* :735-748 */
            for (i = 1; i <= nx; i++) {
                jj = n_sec * npml;
                for (j = ny + 1 - npml; j <= ny - 1; j++) {
                    rotH = (AT(g->Hx, i, j - 1, 0) - AT(g->Hx, i, j, 0)) / dr;
                    AT(g->psiy_Ezy, i, jj, 0) = be[jj - n_base] * AT(g->psiy_Ezy, i, jj, 0) + ce[jj - n_base] * rotH;
                    AT(g->Ez, i, j, 0) = AT(g->Ez, i, j, 0) + dt_eps0 * AT(g->psiy_Ezy, i, jj, 0);
                    jj--;
                }
            }
    } else {
        if (g->boundaries[0] == ORC_PERIODIC) /* :757-763 */
            for (j = 0; j <= ny; j++)
                AT(g->Hz, 0, j, 0) = AT(g->Hz, nx, j, 0);
        if (g->boundaries[1] == ORC_PERIODIC)
            for (i = 0; i <= nx; i++)
                AT(g->Hz, i, 0, 0) = AT(g->Hz, i, ny, 0);
#pragma omp parallel for schedule(static) private(i)
        for (j = 1; j <= ny; j++)
            for (i = 1; i <= nx; i++) {
                double *pl[ORC_MAX_POLES], *plo[ORC_MAX_POLES];
                double r = (AT(g->Hz, i, j, 0) - AT(g->Hz, i, j - 1, 0)) * den_ey[j];
                pol_ptrs(g, 0, i, j, 0, pl, plo);
                if (medium_polarization(g, g->media_map[mm_index(g, i, j, 0, 1)], &AT(g->PD[0], i, j, 0),
                                        pl, plo, &AT(g->Ex, i, j, 0), &AT(g->Ex_old, i, j, 0), r)) {
                    double Jav = 0.5 * (AT(g->Jx_old, i, j, 0) + tt * AT(g->dJx, i, j, 0) +
                                        AT(g->Jx_old, i + 1, j, 0) + tt * AT(g->dJx, i + 1, j, 0));
                    AT(g->Ex, i, j, 0) = AT(g->Ex, i, j, 0) + dt_eps0 * AT(g->eps_x, i, j, 0) * r - dt_eps0 * Jav;
                }
            }
#pragma omp parallel for schedule(static) private(i)
        for (j = 1; j <= ny; j++)
            for (i = 1; i <= nx; i++) {
                double *pl[ORC_MAX_POLES], *plo[ORC_MAX_POLES];
                double r = (AT(g->Hz, i - 1, j, 0) - AT(g->Hz, i, j, 0)) * den_ex[i];
                pol_ptrs(g, 1, i, j, 0, pl, plo);
                if (medium_polarization(g, g->media_map[mm_index(g, i, j, 0, 2)], &AT(g->PD[1], i, j, 0),
                                        pl, plo, &AT(g->Ey, i, j, 0), &AT(g->Ey_old, i, j, 0), r)) {
                    double Jav = 0.5 * (AT(g->Jy_old, i, j, 0) + tt * AT(g->dJy, i, j, 0) +
                                        AT(g->Jy_old, i, j + 1, 0) + tt * AT(g->dJy, i, j + 1, 0));
                    AT(g->Ey, i, j, 0) = AT(g->Ey, i, j, 0) + dt_eps0 * AT(g->eps_y, i, j, 0) * r - dt_eps0 * Jav;
                }
            }
        if (g->cpml_pos[0]) /* :808-818 */
            for (j = 1; j <= ny; j++)
                for (i = 2; i <= npml; i++) {
                    rotH = (AT(g->Hz, i - 1, j, 0) - AT(g->Hz, i, j, 0)) / dr;
                    AT(g->psix_Eyx, i, j, 0) = be[i] * AT(g->psix_Eyx, i, j, 0) + ce[i] * rotH;
                    AT(g->Ey, i, j, 0) = AT(g->Ey, i, j, 0) + dt_eps0 * AT(g->psix_Eyx, i, j, 0);
                }
        if (g->cpml_pos[1]) /* :820-833 */
            for (j = 1; j <= ny; j++) {
                ii = n_sec * npml;
                for (i = nx + 1 - npml; i <= nx - 1; i++) {
                    rotH = (AT(g->Hz, i - 1, j, 0) - AT(g->Hz, i, j, 0)) / dr;
                    AT(g->psix_Eyx, ii, j, 0) = be[ii - n_base] * AT(g->psix_Eyx, ii, j, 0) + ce[ii - n_base] * rotH;
                    AT(g->Ey, i, j, 0) = AT(g->Ey, i, j, 0) + dt_eps0 * AT(g->psix_Eyx, ii, j, 0);
                    ii--;
                }
            }
        if (g->cpml_pos[2]) /* :835-846 */
            for (i = 1; i <= nx; i++)
                for (j = 2; j <= npml; j++) {
                    rotH = (AT(g->Hz, i, j, 0) - AT(g->Hz, i, j - 1, 0)) / dr;
                    AT(g->psiy_Exy, i, j, 0) = be[j] * AT(g->psiy_Exy, i, j, 0) + ce[j] * rotH;
                    AT(g->Ex, i, j, 0) = AT(g->Ex, i, j, 0) + dt_eps0 * AT(g->psiy_Exy, i, j, 0);
                }
        if (g->cpml_pos[3]) /* :848-860: jj = 2*npml hard-coded (N8), same as n_sec*npml here */
            for (i = 1; i <= nx; i++) {
                jj = 2 * npml;
                for (j = ny + 1 - npml; j <= ny - 1; j++) {
                    rotH = (AT(g->Hz, i, j, 0) - AT(g->Hz, i, j - 1, 0)) / dr;
                    AT(g->psiy_Exy, i, jj, 0) = be[jj - n_base] * AT(g->psiy_Exy, i, jj, 0) + ce[jj - n_base] * rotH;
                    AT(g->Ex, i, j, 0) = AT(g->Ex, i, j, 0) + dt_eps0 * AT(g->psiy_Exy, i, jj, 0);
                    jj--;
                }
            }
    }
}

/* ======================================================================================= */
/* 1D propagation (mxll_1D_mod.f90:252-355); only axis is z, array extent nz                */
/* ======================================================================================= */

static void propagate_H_1d(orc_grid *g)
{
    const int nz = g->nz, npml = g->npml;
    const double dt_mu0 = g->dt_mu0, dr = g->dr;
    const double *den_hz = g->den_h[2];
    int i, kk;
    /* periodic 1D writes Ex(nz+1) out of bounds in the reference (:269-271, N8): not restated */
    for (i = 1; i <= nz - 1; i++)
        AT(g->Hy, i, 0, 0) = AT(g->Hy, i, 0, 0) + dt_mu0 * (AT(g->Ex, i, 0, 0) - AT(g->Ex, i + 1, 0, 0)) * den_hz[i];
    if (g->boundaries[0] == ORC_CPML) {
        for (i = 1; i <= npml - 1; i++) {
            AT(g->psiz_Hyz, i, 0, 0) = g->bh[i] * AT(g->psiz_Hyz, i, 0, 0) +
                                       g->ch[i] * (AT(g->Ex, i, 0, 0) - AT(g->Ex, i + 1, 0, 0)) / dr;
            AT(g->Hy, i, 0, 0) = AT(g->Hy, i, 0, 0) + dt_mu0 * AT(g->psiz_Hyz, i, 0, 0);
        }
        kk = 2 * (npml - 1);
        for (i = nz + 1 - npml; i <= nz - 1; i++) {
            AT(g->psiz_Hyz, kk, 0, 0) = g->bh[kk - (npml - 1)] * AT(g->psiz_Hyz, kk, 0, 0) +
                                        g->ch[kk - (npml - 1)] * (AT(g->Ex, i, 0, 0) - AT(g->Ex, i + 1, 0, 0)) / dr;
            AT(g->Hy, i, 0, 0) = AT(g->Hy, i, 0, 0) + dt_mu0 * AT(g->psiz_Hyz, kk, 0, 0);
            kk--;
        }
    }
}

static void propagate_E_1d(orc_grid *g)
{
    const int nz = g->nz, npml = g->npml;
    const double dt_eps0 = g->dt_eps0, dr = g->dr;
    const double *den_ez = g->den_e[2];
    const double tt = g->time - g->t_skip;
    int i, kk;
    for (i = 2; i <= nz - 1; i++) {
        double *pl[ORC_MAX_POLES], *plo[ORC_MAX_POLES];
        double rotH = (AT(g->Hy, i - 1, 0, 0) - AT(g->Hy, i, 0, 0)) * den_ez[i];
        pol_ptrs(g, 0, i, 0, 0, pl, plo);
        if (medium_polarization(g, g->media_map[i - 1], &AT(g->PD[0], i, 0, 0), pl, plo,
                                &AT(g->Ex, i, 0, 0), &AT(g->Ex_old, i, 0, 0), rotH)) {
            double Jx = AT(g->Jx_old, i, 0, 0) + tt * AT(g->dJx, i, 0, 0);
            AT(g->Ex, i, 0, 0) = AT(g->Ex, i, 0, 0) + dt_eps0 * AT(g->eps_x, i, 0, 0) * rotH - dt_eps0 * Jx;
        }
    }
    if (g->boundaries[0] == ORC_CPML) {
        double rotH;
        for (i = 2; i <= npml; i++) {
            rotH = (AT(g->Hy, i - 1, 0, 0) - AT(g->Hy, i, 0, 0)) / dr;
            AT(g->psiz_Exz, i, 0, 0) = g->be[i] * AT(g->psiz_Exz, i, 0, 0) + g->ce[i] * rotH;
            AT(g->Ex, i, 0, 0) = AT(g->Ex, i, 0, 0) + dt_eps0 * AT(g->psiz_Exz, i, 0, 0);
        }
        kk = 2 * npml;
        for (i = nz + 1 - npml; i <= nz - 1; i++) {
            rotH = (AT(g->Hy, i - 1, 0, 0) - AT(g->Hy, i, 0, 0)) / dr;
            AT(g->psiz_Exz, kk, 0, 0) = g->be[kk - npml] * AT(g->psiz_Exz, kk, 0, 0) + g->ce[kk - npml] * rotH;
            AT(g->Ex, i, 0, 0) = AT(g->Ex, i, 0, 0) + dt_eps0 * AT(g->psiz_Exz, kk, 0, 0);
            kk--;
        }
    }
}

void orc_propagate_H(orc_grid *g)
{
    if (g->dims == 3)
        propagate_H_3d(g);
    else if (g->dims == 2)
        propagate_H_2d(g);
    else
        propagate_H_1d(g);
}

void orc_propagate_E(orc_grid *g)
{
    if (g->dims == 3)
        propagate_E_3d(g);
    else if (g->dims == 2)
        propagate_E_2d(g);
    else
        propagate_E_1d(g);
}

/* ======================================================================================= */
/* Media maps from voxel lists (classical_medium_mod.f90:203-769)                           */
/* ======================================================================================= */

int orc_media_map_3d(int nx, int ny, int nz, double dr, int n_media, const int *n_vox,
                     const double *vox, int32_t *map)
{
    const double nm = KC()->nm_to_au;
    long N = (long)nx * ny * nz;
    int32_t *aux = (int32_t *)calloc((size_t)N, sizeof(int32_t));
    int n, i, j, k;
    long v, off = 0;
#define AUX(i, j, k) aux[((i) - 1) + (long)nx * (((j) - 1) + (long)ny * ((k) - 1))]
#define AUXS(i, j, k) (((i) >= 1 && (i) <= nx && (j) >= 1 && (j) <= ny && (k) >= 1 && (k) <= nz) ? AUX(i, j, k) : 0)
#define MAP(i, j, k, c) map[((i) - 1) + (long)nx * (((j) - 1) + (long)ny * (((k) - 1) + (long)nz * ((c) - 1)))]
    memset(map, 0, sizeof(int32_t) * (size_t)(N * 3));
    for (n = 1; n <= n_media; n++) {
        for (v = 0; v < n_vox[n - 1]; v++, off++) {
            double x = vox[3 * off] * nm, y = vox[3 * off + 1] * nm, z = vox[3 * off + 2] * nm;
            int ii = (int)(x / dr) + nx / 2, jj = (int)(y / dr) + ny / 2, kk = (int)(z / dr) + nz / 2;
            if (ii < 1 || ii > nx || jj < 1 || jj > ny || kk < 1 || kk > nz)
                continue; /* out-of-box voxels write out of bounds in the reference */
            if (AUX(ii, jj, kk) == 0)
                AUX(ii, jj, kk) = n;
        }
    }
    /* :694-745 (single rank); out-of-range neighbour reads treated as 0 */
    for (n = 1; n <= n_media; n++)
        for (k = 1; k <= nz; k++)
            for (j = 1; j <= ny; j++)
                for (i = 1; i <= nx; i++) {
                    int a = AUX(i, j, k);
                    if (i == nx && a == n)
                        MAP(i, j, k, 1) = n;
                    else if (j == ny && a == n)
                        MAP(i, j, k, 1) = n;
                    else if (k == nz && a == n)
                        MAP(i, j, k, 1) = n;
                    else {
                        if (a == n && AUXS(i + 1, j, k) == n)
                            MAP(i, j, k, 1) = n;
                        else if (a != 0 && AUXS(i + 1, j, k) == n)
                            MAP(i, j, k, 1) = n;
                        if (a == n && AUXS(i, j + 1, k) == n)
                            MAP(i, j, k, 2) = n;
                        else if (a != 0 && AUXS(i, j + 1, k) == n)
                            MAP(i, j, k, 2) = n;
                        if (a == n && AUXS(i, j, k + 1) == n)
                            MAP(i, j, k, 3) = n;
                        else if (a != 0 && AUXS(i, j, k + 1) == n)
                            MAP(i, j, k, 3) = n;
                    }
                }
#undef AUX
#undef AUXS
#undef MAP
    free(aux);
    return 0;
}

int orc_media_map_2d(int nx, int ny, double dr, int n_media, const int *n_vox, const double *vox,
                     int32_t *map)
{
    const double nm = KC()->nm_to_au;
    long N = (long)nx * ny;
    int32_t *aux = (int32_t *)calloc((size_t)N, sizeof(int32_t));
    int n, i, j;
    long v, off = 0;
#define AUX(i, j) aux[((i) - 1) + (long)nx * ((j) - 1)]
#define AUXS(i, j) (((i) >= 1 && (i) <= nx && (j) >= 1 && (j) <= ny) ? AUX(i, j) : 0)
#define MAP(i, j, c) map[((i) - 1) + (long)nx * (((j) - 1) + (long)ny * ((c) - 1))]
    memset(map, 0, sizeof(int32_t) * (size_t)(N * 3));
    for (n = 1; n <= n_media; n++) {
        for (v = 0; v < n_vox[n - 1]; v++, off++) {
            double x = vox[2 * off] * nm, y = vox[2 * off + 1] * nm;
            int ii = (int)(x / dr) + nx / 2, jj = (int)(y / dr) + ny / 2;
            if (ii < 1 || ii > nx || jj < 1 || jj > ny)
                continue;
            if (AUX(ii, jj) == 0)
                AUX(ii, jj) = n;
        }
    }
    /* :484-524 */
    for (n = 1; n <= n_media; n++)
        for (j = 1; j <= ny; j++)
            for (i = 1; i <= nx; i++) {
                int a = AUX(i, j);
                if (i == nx && a == n)
                    MAP(i, j, 1) = n;
                else if (j == ny && a == n)
                    MAP(i, j, 1) = n;
                else {
                    if (a == n && AUXS(i + 1, j) == n)
                        MAP(i, j, 1) = n;
                    else if (a != 0 && AUXS(i + 1, j) == n)
                        MAP(i, j, 1) = n;
                    if (a == n && AUXS(i, j + 1) == n)
                        MAP(i, j, 2) = n;
                    else if (a != 0 && AUXS(i, j + 1) == n)
                        MAP(i, j, 2) = n;
                    if (a == n)
                        MAP(i, j, 3) = n;
                }
            }
#undef AUX
#undef AUXS
#undef MAP
    free(aux);
    return 0;
}

int orc_media_map_1d(int nz, double dr, int n_media, const int *n_vox, const double *vox,
                     int32_t *map)
{
    const double nm = KC()->nm_to_au;
    int n;
    long v, off = 0;
    memset(map, 0, sizeof(int32_t) * (size_t)nz);
    for (n = 1; n <= n_media; n++)
        for (v = 0; v < n_vox[n - 1]; v++, off++) {
            double x = vox[off] * nm;
            int ii = (int)(x / dr) + nz / 2;
            if (ii < 1 || ii > nz)
                continue;
            if (map[ii - 1] == 0)
                map[ii - 1] = n;
        }
    return 0;
}

/* ======================================================================================= */
/* Sources (source_mod.f90, interactions_mod.f90:21-163)                                    */
/* ======================================================================================= */

struct orc_source {
    orc_source_desc d;
    int dim, n_ker, side;
    double *ker;      /* side^dim, i fastest, (i,j,k) from -n_ker */
    double *J;        /* same + 1 trailing zero slot for the beyond-the-end read */
    int *ind;         /* 3 per point */
    double c_src;
};

orc_source *orc_source_create(const orc_grid *g, const orc_source_desc *d)
{
    const orc_constants *c = KC();
    orc_source *s = (orc_source *)calloc(1, sizeof(orc_source));
    const double dr = g->dr;
    int n_ker, side, npts, i, j, k, q;
    double r_max, r0, norm = 0.0;
    int N[3];
    s->d = *d;
    s->dim = g->dims;
    n_ker = (int)(d->rad / dr); /* :71 */
    s->n_ker = n_ker;
    side = 2 * n_ker + 1;
    s->side = side;
    npts = (s->dim == 3) ? side * side * side : (s->dim == 2 ? side * side : side);
    s->ker = (double *)calloc((size_t)npts, sizeof(double));
    s->J = (double *)calloc((size_t)npts + 1, sizeof(double));
    s->ind = (int *)calloc((size_t)npts * 3, sizeof(int));
    r_max = (n_ker * 2 + 2) * dr; /* compute_kernel :264-265 */
    r0 = r_max / 2.0;
    q = 0;
    for (k = (s->dim == 3 ? -n_ker : 0); k <= (s->dim == 3 ? n_ker : 0); k++)
        for (j = (s->dim >= 2 ? -n_ker : 0); j <= (s->dim >= 2 ? n_ker : 0); j++)
            for (i = -n_ker; i <= n_ker; i++, q++) {
                double x = i * dr, y = j * dr, z = k * dr, r, w;
                const double tp = 2.0 * c->pi0;
                if (s->dim == 1)
                    r = x; /* 1D uses (x - r0) directly (:270-279) */
                else if (s->dim == 2)
                    r = sqrt(x * x + y * y);
                else
                    r = sqrt(x * x + y * y + z * z);
                w = c->aBH[0] + c->aBH[1] * cos(tp * (r - r0) / r_max) +
                    c->aBH[2] * cos(tp * 2.0 * (r - r0) / r_max) +
                    c->aBH[3] * cos(tp * 3.0 * (r - r0) / r_max);
                if (s->dim >= 2 && w < 0.0)
                    w = 0.0;
                s->ker[q] = w;
                norm = norm + w;
            }
    for (q = 0; q < npts; q++)
        s->ker[q] = s->ker[q] / norm;
    /* determine_indx_and_ranks :345-367 (single rank) */
    if (s->dim == 1) {
        N[0] = g->nz; N[1] = 1; N[2] = 1;
    } else {
        N[0] = g->nx; N[1] = g->ny; N[2] = g->nz;
    }
    q = 0;
    for (k = (s->dim == 3 ? -n_ker : 0); k <= (s->dim == 3 ? n_ker : 0); k++)
        for (j = (s->dim >= 2 ? -n_ker : 0); j <= (s->dim >= 2 ? n_ker : 0); j++)
            for (i = -n_ker; i <= n_ker; i++, q++) {
                s->ind[3 * q] = i + (int)(d->r0[0] / dr) + N[0] / 2;
                s->ind[3 * q + 1] = (s->dim >= 2) ? j + (int)(d->r0[1] / dr) + N[1] / 2 : 0;
                s->ind[3 * q + 2] = (s->dim == 3) ? k + (int)(d->r0[2] / dr) + N[2] / 2 : 0;
            }
    s->c_src = g->dt_eps0 / g->dr / c->c0 / 2.0; /* :32 */
    return s;
}

void orc_source_destroy(orc_source *s)
{
    if (!s)
        return;
    free(s->ker);
    free(s->J);
    free(s->ind);
    free(s);
}

int orc_source_kernel(const orc_source *s, double *ker, int *n_ker)
{
    int npts = (s->dim == 3) ? s->side * s->side * s->side : (s->dim == 2 ? s->side * s->side : s->side);
    if (ker)
        memcpy(ker, s->ker, sizeof(double) * (size_t)npts);
    if (n_ker)
        *n_ker = s->n_ker;
    return npts;
}

void orc_source_update(orc_source *s, double time)
{
    int npts = (s->dim == 3) ? s->side * s->side * s->side : (s->dim == 2 ? s->side * s->side : s->side);
    int q;
    if (time >= s->d.t_init && time <= s->d.t_final) { /* :114-130 */
        double a = (time - s->d.t0) / s->d.tau;
        double envelope = exp(-(a * a));
        double ph = s->d.w0 * (time - s->d.t0) + s->d.phase;
        double cos_t, amp;
        if (s->d.chirp != 0.0) /* extension: linear chirp */
            ph = ph + 0.5 * s->d.chirp * ((time - s->d.t0) * (time - s->d.t0));
        cos_t = cos(ph);
        amp = s->d.j_amp * envelope * cos_t;
        for (q = 0; q < npts; q++)
            s->J[q] = amp * s->ker[q];
    } else {
        for (q = 0; q < npts; q++)
            s->J[q] = 0.0;
    }
    s->J[npts] = 0.0;
}

void orc_source_interactions(orc_grid *g, orc_source **list, int n)
{
    int si;
    for (si = 0; si < n; si++) {
        orc_source *s = list[si];
        const int side = s->side, nk = s->n_ker;
        const int npts = (s->dim == 3) ? side * side * side : (s->dim == 2 ? side * side : side);
        int i, j, k;
        /* stride of the next point along the source direction in the Fortran layout;
         * the reference reads J_mat(n_ker+1, ...) which aliases the next row (N8);
         * reading past the array end is taken as zero. */
        int stride = (s->d.dir == 'x') ? 1 : (s->d.dir == 'y' ? side : side * side);
        for (i = -nk; i <= nk; i++)
            for (j = (s->dim >= 2 ? -nk : 0); j <= (s->dim >= 2 ? nk : 0); j++)
                for (k = (s->dim == 3 ? -nk : 0); k <= (s->dim == 3 ? nk : 0); k++) {
                    int q = (i + nk) + side * ((s->dim >= 2 ? j + nk : 0) + side * (s->dim == 3 ? k + nk : 0));
                    int ii = s->ind[3 * q], jj = s->ind[3 * q + 1], kk = s->ind[3 * q + 2];
                    double Jav;
                    if (s->dim == 1) {
                        Jav = s->J[q]; /* :45-49 */
                        AT(g->Ex, ii, 0, 0) = AT(g->Ex, ii, 0, 0) + s->c_src * Jav;
                        continue;
                    }
                    if (s->dim == 2 && s->d.dir == 'z') {
                        Jav = s->J[q];
                    } else {
                        int q2 = q + stride;
                        double Jn = (q2 < npts) ? s->J[q2] : 0.0;
                        Jav = 0.5 * (s->J[q] + Jn);
                    }
                    if (s->d.dir == 'x')
                        AT(g->Ex, ii, jj, kk) = AT(g->Ex, ii, jj, kk) + s->c_src * Jav;
                    else if (s->d.dir == 'y')
                        AT(g->Ey, ii, jj, kk) = AT(g->Ey, ii, jj, kk) + s->c_src * Jav;
                    else
                        AT(g->Ez, ii, jj, kk) = AT(g->Ez, ii, jj, kk) + s->c_src * Jav;
                }
    }
}

void orc_plane_source_apply(orc_grid *g, const orc_plane_source_desc *d, double time)
{
    const orc_constants *c = KC();
    double amp = 0.0;
    double c_src = g->dt_eps0 / g->dr / c->c0 / 2.0;
    arr *E = (d->comp == 1) ? &g->Ex : (d->comp == 2 ? &g->Ey : &g->Ez);
    int i, j, k;
    if (time >= d->t_init && time <= d->t_final) {
        double a = (time - d->t0) / d->tau;
        double ph = d->w0 * (time - d->t0) + d->phase;
        if (d->chirp != 0.0)
            ph = ph + 0.5 * d->chirp * ((time - d->t0) * (time - d->t0));
        amp = d->j_amp * exp(-(a * a)) * cos(ph);
    }
    if (amp == 0.0)
        return;
    for (k = 1; k <= (g->dims == 3 ? g->nz : 1); k++)
        for (j = 1; j <= (g->dims >= 2 ? g->ny : 1); j++)
            for (i = 1; i <= (g->dims == 1 ? g->nz : g->nx); i++) {
                int p[3] = {i, j, k};
                int kk2 = (g->dims == 3) ? k : 0, jj2 = (g->dims >= 2) ? j : 0;
                if (p[d->plane_axis - 1] != d->plane_idx)
                    continue;
                AT(*E, i, jj2, kk2) = AT(*E, i, jj2, kk2) + c_src * amp;
            }
}

/* ======================================================================================= */
/* Few-level density-matrix emitters (new; no reference arithmetic)                          */
/* ======================================================================================= */
/*
 * State layout (real, FP64):
 *   2-level: rho = [p_e, re(rho_eg), im(rho_eg)]                               (3 reals)
 *   3-level: rho = [p1, p2, re r10, im r10, re r20, im r20, re r21, im r21]     (8 reals)
 * Ground populations are 1 - sum of excited populations.
 * Equation: d rho/dt = -i[H0 - E_u V, rho] + relaxation, with V the dipole operator
 * (couplings ground<->excited), T1 population decay to the ground state and T2
 * coherence decay.  Integrated with classical RK4 over dt with E_u held constant; the
 * relaxation rates 1/T1, 1/T2 are formed once per step.
 */

static void rhs2(const double *pr, double E_u, double g1, double g2, const double *rho, double *d)
{
    const double w0 = pr[0], mu = pr[1];
    const double pe = rho[0], a = rho[1], b = rho[2];
    const double pg = 1.0 - pe;
    const double muE = mu * E_u;
    /* d pe/dt = 2 mu E Im(rho_eg) - pe/T1   (g1 = 1/T1, g2 = 1/T2) */
    d[0] = 2.0 * muE * b - pe * g1;
    /* d rho_eg/dt = -i w0 rho_eg + i mu E (pg - pe) - rho_eg/T2 */
    d[1] = w0 * b - a * g2;
    d[2] = -(w0 * a) + muE * (pg - pe) - b * g2;
}

static void rhs3(const double *pr, double E_u, double g1r, double g2r, const double *rho, double *d)
{
    const double e1 = pr[0], e2 = pr[1], mu1 = pr[2], mu2 = pr[3];
    const double p1 = rho[0], p2 = rho[1];
    const double a10 = rho[2], b10 = rho[3], a20 = rho[4], b20 = rho[5], a21 = rho[6], b21 = rho[7];
    const double p0 = 1.0 - p1 - p2;
    const double g1 = mu1 * E_u, g2 = mu2 * E_u;
    /* H = diag(0,e1,e2) - E_u (mu1 (|0><1|+|1><0|) + mu2 (|0><2|+|2><0|)).
     * d rho_kk = -i (H rho - rho H)_kk; with W = -E_u V:
     * d p1 = 2 g1 Im(rho_10) ... derived with rho_kl = a_kl + i b_kl (k>l). */
    d[0] = 2.0 * g1 * b10 - p1 * g1r;
    d[1] = 2.0 * g2 * b20 - p2 * g1r;
    {
        /* (H rho)_10 = e1 rho_10 - g1 rho_00 ; (rho H)_10 = -g1 rho_11 - g2 rho_12
         * -i[(H rho)_10 - (rho H)_10] = -i e1 rho_10 + i g1 (rho_00 - rho_11) - i g2 rho_12 */
        /* rho_12 = conj(rho_21) = a21 - i b21 ; -i g2 (a21 - i b21) = -g2 b21 - i g2 a21 */
        d[2] = e1 * b10 - g2 * b21 - a10 * g2r;
        d[3] = -(e1 * a10) + g1 * (p0 - p1) - g2 * a21 - b10 * g2r;
    }
    {
        /* (H rho)_20 = e2 rho_20 - g2 rho_00 ; (rho H)_20 = -g1 rho_21 - g2 rho_22
         * -i[...]_20 = -i e2 rho_20 + i g2 (rho_00 - rho_22) - i g1 rho_21 */
        d[4] = e2 * b20 + g1 * b21 - a20 * g2r;
        d[5] = -(e2 * a20) + g2 * (p0 - p2) - g1 * a21 - b20 * g2r;
    }
    {
        /* (H rho)_21 = e2 rho_21 - g2 rho_01 ; (rho H)_21 = e1 rho_21 - g1 rho_20
         * -i[...]_21 = -i (e2 - e1) rho_21 + i g2 rho_01 - i g1 rho_20,
         * rho_01 = conj(rho_10) = a10 - i b10, -i g1 rho_20 = g1 b20 - i g1 a20 */
        double de = e2 - e1;
        d[6] = de * b21 + g2 * b10 + g1 * b20 - a21 * g2r;
        d[7] = -(de * a21) + g2 * a10 - g1 * a20 - b21 * g2r;
    }
}

void orc_emitter_step(int model, const double *pr, double *rho, double E_u, double dt)
{
    const int n = (model == ORC_EMITTER_2LEVEL) ? 3 : 8;
    double k1[8], k2[8], k3[8], k4[8], t[8];
    const double h2 = 0.5 * dt, h6 = dt / 6.0;
    /* relaxation rates once per step (the 2-level params hold T1, T2 at 2, 3; 3-level at 4, 5) */
    const double g1 = 1.0 / pr[model == ORC_EMITTER_2LEVEL ? 2 : 4];
    const double g2 = 1.0 / pr[model == ORC_EMITTER_2LEVEL ? 3 : 5];
    int q;
    void (*f)(const double *, double, double, double, const double *, double *) =
        (model == ORC_EMITTER_2LEVEL) ? rhs2 : rhs3;
    f(pr, E_u, g1, g2, rho, k1);
    for (q = 0; q < n; q++)
        t[q] = rho[q] + h2 * k1[q];
    f(pr, E_u, g1, g2, t, k2);
    for (q = 0; q < n; q++)
        t[q] = rho[q] + h2 * k2[q];
    f(pr, E_u, g1, g2, t, k3);
    for (q = 0; q < n; q++)
        t[q] = rho[q] + dt * k3[q];
    f(pr, E_u, g1, g2, t, k4);
    for (q = 0; q < n; q++)
        rho[q] = rho[q] + h6 * (k1[q] + 2.0 * k2[q] + 2.0 * k3[q] + k4[q]);
}

/* scalar dipole along the emitter axis: Tr(rho V) */
static double emitter_dipole(int model, const double *pr, const double *rho)
{
    if (model == ORC_EMITTER_2LEVEL)
        return 2.0 * pr[1] * rho[1];
    return 2.0 * pr[2] * rho[2] + 2.0 * pr[3] * rho[4];
}

struct orc_qgroup {
    int dims, group_type, model, n, npar, nst, n_ker;
    int32_t *cell;       /* n x 3 (i,j,k), 1-based */
    double *par;         /* n x npar */
    double *rho;         /* n x nst */
    double *E;           /* n x 3 */
    double *dipole, *dip_old, *dPt_dt; /* n x 3 */
    double density, dt;
    double *mat_kernel;  /* side^dims */
    int mode;
};

orc_qgroup *orc_qgroup_create(const orc_grid *g, int group_type, int model, int n, const int32_t *cell,
                              const double *params, double density, double dt_q)
{
    orc_qgroup *q = (orc_qgroup *)calloc(1, sizeof(orc_qgroup));
    const orc_constants *c = KC();
    int e, a;
    q->dims = g->dims;
    q->mode = g->mode;
    q->group_type = group_type;
    q->model = model;
    q->n = n;
    q->npar = (model == ORC_EMITTER_2LEVEL) ? 7 : 9;
    q->nst = (model == ORC_EMITTER_2LEVEL) ? 3 : 8;
    q->density = density;
    q->dt = dt_q;
    q->n_ker = 3; /* hard-coded (q_group_mod.f90:19) */
    q->cell = (int32_t *)calloc((size_t)n * 3, sizeof(int32_t));
    q->par = (double *)malloc(sizeof(double) * (size_t)n * q->npar);
    q->rho = (double *)calloc((size_t)n * q->nst, sizeof(double));
    q->E = (double *)calloc((size_t)n * 3, sizeof(double));
    q->dipole = (double *)calloc((size_t)n * 3, sizeof(double));
    q->dip_old = (double *)calloc((size_t)n * 3, sizeof(double));
    q->dPt_dt = (double *)calloc((size_t)n * 3, sizeof(double));
    for (e = 0; e < n; e++)
        for (a = 0; a < 3; a++)
            q->cell[3 * e + a] = (a < g->dims) ? cell[g->dims * e + a] : 0;
    memcpy(q->par, params, sizeof(double) * (size_t)n * q->npar);
    if (group_type == ORC_Q_SINGLE) {
        /* q_group_mod.f90:165-239 (norm computed but never applied, N7) */
        int nk = q->n_ker, side = 2 * nk + 1, i, j, k, p = 0;
        double r_max = (double)(nk * 2 + 4), r0 = r_max / 2.0;
        const double tp = 2.0 * c->pi0;
        int cnt = (g->dims == 3) ? side * side * side : (g->dims == 2 ? side * side : side);
        q->mat_kernel = (double *)calloc((size_t)cnt, sizeof(double));
        for (k = (g->dims == 3 ? -nk : 0); k <= (g->dims == 3 ? nk : 0); k++)
            for (j = (g->dims >= 2 ? -nk : 0); j <= (g->dims >= 2 ? nk : 0); j++)
                for (i = -nk; i <= nk; i++, p++) {
                    double x = (double)i, y = (double)j, z = (double)k, r, w;
                    if (g->dims == 1)
                        r = x;
                    else if (g->dims == 2)
                        r = sqrt(x * x + y * y);
                    else
                        r = sqrt(x * x + y * y + z * z);
                    w = c->aBH[0] + c->aBH[1] * cos(tp * (r - r0) / r_max) +
                        c->aBH[2] * cos(tp * 2.0 * (r - r0) / r_max) +
                        c->aBH[3] * cos(tp * 3.0 * (r - r0) / r_max);
                    if (g->dims >= 2 && w < 0.0)
                        w = 0.0;
                    q->mat_kernel[p] = w;
                }
    }
    /* gs_calculate: ground state, dipole zero */
    return q;
}

void orc_qgroup_destroy(orc_qgroup *q)
{
    if (!q)
        return;
    free(q->cell); free(q->par); free(q->rho); free(q->E);
    free(q->dipole); free(q->dip_old); free(q->dPt_dt); free(q->mat_kernel);
    free(q);
}

int orc_qgroup_state_size(const orc_qgroup *q) { return q->nst; }

void orc_send_E_to_J(const orc_grid *g, orc_qgroup *q)
{
    int e;
    for (e = 0; e < q->n; e++) {
        int i = q->cell[3 * e], j = q->cell[3 * e + 1], k = q->cell[3 * e + 2];
        double *E = &q->E[3 * e];
        if (g->dims == 3) { /* interactions_mod.f90:656-691 */
            E[0] = 0.5 * (AT(g->Ex, i - 1, j, k) + AT(g->Ex, i, j, k));
            E[1] = 0.5 * (AT(g->Ey, i, j - 1, k) + AT(g->Ey, i, j, k));
            E[2] = 0.5 * (AT(g->Ez, i, j, k - 1) + AT(g->Ez, i, j, k));
        } else if (g->dims == 2) { /* :486-526 */
            if (g->mode == ORC_TEZ) {
                E[0] = 0.5 * (AT(g->Ex, i - 1, j, 0) + AT(g->Ex, i, j, 0));
                E[1] = 0.5 * (AT(g->Ey, i, j - 1, 0) + AT(g->Ey, i, j, 0));
            } else {
                E[2] = AT(g->Ez, i, j, 0);
            }
        } else { /* :329-346 */
            E[0] = AT(g->Ex, i, 0, 0);
        }
    }
}

void orc_td_propagate_q_group(orc_qgroup *q, int tq_step)
{
    int e;
    (void)tq_step;
    /* q_group_mod.f90:813-816; TQ_sys%td_propagate sets dipole and dPt_dt=(dipole-dip_old)/dt
     * as the only existing implementation does (q_sys_dftb_mod.f90:416-426). */
    for (e = 0; e < q->n; e++) {
        const double *pr = &q->par[(size_t)e * q->npar];
        double *rho = &q->rho[(size_t)e * q->nst];
        const double *u = pr + (q->npar - 3);
        const double *E = &q->E[3 * e];
        double E_u = u[0] * E[0] + u[1] * E[1] + u[2] * E[2];
        double d;
        int a;
        for (a = 0; a < 3; a++)
            q->dip_old[3 * e + a] = q->dipole[3 * e + a];
        orc_emitter_step(q->model, pr, rho, E_u, q->dt);
        d = emitter_dipole(q->model, pr, rho);
        for (a = 0; a < 3; a++) {
            q->dipole[3 * e + a] = d * u[a];
            q->dPt_dt[3 * e + a] = (q->dipole[3 * e + a] - q->dip_old[3 * e + a]) / q->dt;
        }
    }
}

void orc_send_J_to_E(orc_grid *g, orc_qgroup *q)
{
    int e;
    arr *J[3] = {&g->Jx, &g->Jy, &g->Jz}, *Jo[3] = {&g->Jx_old, &g->Jy_old, &g->Jz_old};
    arr *dJ[3] = {&g->dJx, &g->dJy, &g->dJz};
    int c0 = 0, c1 = 2, c;
    if (g->dims == 2) {
        if (g->mode == ORC_TMZ)
            c0 = c1 = 2;
        else {
            c0 = 0;
            c1 = 1;
        }
    } else if (g->dims == 1) {
        c0 = c1 = 0;
    }
    /* J_old = J (full grid), interactions_mod.f90:1067-1069 / 859-865 / 1D */
    for (c = c0; c <= c1; c++)
        memcpy(Jo[c]->p, J[c]->p, sizeof(double) * (size_t)arr_size(J[c]));
    for (e = 0; e < q->n; e++) {
        int i = q->cell[3 * e], j = q->cell[3 * e + 1], k = q->cell[3 * e + 2];
        int jj0 = (g->dims >= 2) ? j : 0, kk0 = (g->dims == 3) ? k : 0;
        const double *P = &q->dPt_dt[3 * e];
        if (q->group_type == ORC_Q_MATERIAL) { /* :1181-1190 */
            for (c = c0; c <= c1; c++)
                AT(*J[c], i, jj0, kk0) = q->density * P[c];
        } else { /* :1194-1212, order k, j, i */
            int nk = q->n_ker, side = 2 * nk + 1, a, b, d;
            for (d = (g->dims == 3 ? -nk : 0); d <= (g->dims == 3 ? nk : 0); d++)
                for (b = (g->dims >= 2 ? -nk : 0); b <= (g->dims >= 2 ? nk : 0); b++)
                    for (a = -nk; a <= nk; a++) {
                        int p = (a + nk) + side * ((g->dims >= 2 ? b + nk : 0) + side * (g->dims == 3 ? d + nk : 0));
                        int ii = i + a, jj = (g->dims >= 2) ? j + b : 0, kk = (g->dims == 3) ? k + d : 0;
                        for (c = c0; c <= c1; c++)
                            AT(*J[c], ii, jj, kk) = q->density * q->mat_kernel[p] * P[c];
                    }
        }
    }
    /* dJ = (J - J_old)/dt (:1216-1218) */
    for (c = c0; c <= c1; c++) {
        long s = arr_size(J[c]), t;
        for (t = 0; t < s; t++)
            dJ[c]->p[t] = (J[c]->p[t] - Jo[c]->p[t]) / q->dt;
    }
}

void orc_qgroup_read(const orc_qgroup *q, double *dipole, double *dPt_dt, double *efield, double *rho)
{
    if (dipole)
        memcpy(dipole, q->dipole, sizeof(double) * (size_t)q->n * 3);
    if (dPt_dt)
        memcpy(dPt_dt, q->dPt_dt, sizeof(double) * (size_t)q->n * 3);
    if (efield)
        memcpy(efield, q->E, sizeof(double) * (size_t)q->n * 3);
    if (rho)
        memcpy(rho, q->rho, sizeof(double) * (size_t)q->n * q->nst);
}

/* ======================================================================================= */
/* Detector sampling stencils (write_fields_subs_mod.f90:88-193, 279-628, 751-1509)          */
/* ======================================================================================= */

void orc_sample(const orc_grid *g, int type, int field, int nd, const int32_t *idx, double *out)
{
    int n;
    for (n = 0; n < nd; n++) {
        if (g->dims == 1) {
            int k = idx[n];
            out[n] = (field == ORC_EX) ? AT(g->Ex, k, 0, 0)
                                       : 0.5 * (AT(g->Hy, k - 1, 0, 0) + AT(g->Hy, k, 0, 0));
        } else if (g->dims == 2) {
            int i = idx[n], j = idx[nd + n];
            switch (field) {
            case ORC_EX: out[n] = 0.5 * (AT(g->Ex, i - 1, j, 0) + AT(g->Ex, i, j, 0)); break;
            case ORC_EY: out[n] = 0.5 * (AT(g->Ey, i, j - 1, 0) + AT(g->Ey, i, j, 0)); break;
            case ORC_EZ: out[n] = AT(g->Ez, i, j, 0); break;
            case ORC_HX: out[n] = 0.5 * (AT(g->Hx, i, j, 0) + AT(g->Hx, i, j - 1, 0)); break;
            case ORC_HY: out[n] = 0.5 * (AT(g->Hy, i, j, 0) + AT(g->Hy, i - 1, j, 0)); break;
            default:
                out[n] = 0.25 * (AT(g->Hz, i, j, 0) + AT(g->Hz, i - 1, j - 1, 0) + AT(g->Hz, i - 1, j, 0) +
                                 AT(g->Hz, i, j - 1, 0));
            }
        } else {
            int i = idx[n], j = idx[nd + n], k = idx[2 * nd + n];
            switch (field) {
            case ORC_EX: out[n] = 0.5 * (AT(g->Ex, i - 1, j, k) + AT(g->Ex, i, j, k)); break;
            case ORC_EY: out[n] = 0.5 * (AT(g->Ey, i, j - 1, k) + AT(g->Ey, i, j, k)); break;
            case ORC_EZ:
                /* point: raw Ez (:831); lines/planes/volumes: 2-point average (:892) */
                out[n] = (type == ORC_POINT) ? AT(g->Ez, i, j, k)
                                             : 0.5 * (AT(g->Ez, i, j, k - 1) + AT(g->Ez, i, j, k));
                break;
            case ORC_HX:
                out[n] = 0.25 * (AT(g->Hx, i, j - 1, k) + AT(g->Hx, i, j, k) + AT(g->Hx, i, j, k - 1) +
                                 AT(g->Hx, i, j - 1, k - 1));
                break;
            case ORC_HY:
                out[n] = 0.25 * (AT(g->Hy, i - 1, j, k) + AT(g->Hy, i, j, k) + AT(g->Hy, i, j, k - 1) +
                                 AT(g->Hy, i - 1, j, k - 1));
                break;
            default:
                out[n] = 0.25 * (AT(g->Hz, i, j, k) + AT(g->Hz, i - 1, j, k) + AT(g->Hz, i, j - 1, k) +
                                 AT(g->Hz, i - 1, j - 1, k));
            }
        }
    }
}

/* ======================================================================================= */
/* Time loop (mxim_mxll.f90:92-132)                                                          */
/* ======================================================================================= */

void orc_run(orc_scene *s, int tt0, int nsteps)
{
    orc_grid *g = s->grid;
    const int tt_0 = (s->n_skip_steps == 1) ? 1 : 0;
    int tt, i, rec_off = 0, total_pts = 0;
    for (i = 0; i < s->n_det; i++)
        total_pts += s->det_nd[i];
    for (tt = tt0; tt < tt0 + nsteps; tt++) {
        double time = g->dt * ((double)tt - 0.5);
        int tq_step = 1 + (tt - tt_0) / s->n_skip_steps;
        int move = 0;
        if (tq_step > s->tq_step_old) {
            s->t_skip = time;
            s->tq_step_old = tq_step;
            move = (s->n_groups > 0);
        }
        orc_grid_set_time(g, time, s->t_skip);
        orc_propagate_H(g);
        for (i = 0; i < s->n_src; i++)
            orc_source_update(s->src[i], time);
        orc_source_interactions(g, s->src, s->n_src);
        for (i = 0; i < s->n_plane; i++)
            orc_plane_source_apply(g, &s->plane[i], time);
        orc_propagate_E(g);
        if (move)
            for (i = 0; i < s->n_groups; i++) {
                orc_send_E_to_J(g, s->groups[i]);
                orc_td_propagate_q_group(s->groups[i], tq_step);
                orc_send_J_to_E(g, s->groups[i]);
            }
        if (s->n_det > 0 && s->t_det_print > 0 && tt % s->t_det_print == 0 && s->det_out) {
            int off = 0;
            for (i = 0; i < s->n_det; i++) {
                orc_sample(g, s->det_type[i], s->det_field[i], s->det_nd[i], s->det_idx[i],
                           s->det_out + (size_t)s->record * total_pts + off);
                off += s->det_nd[i];
            }
            s->record++;
        }
    }
    (void)rec_off;
}
