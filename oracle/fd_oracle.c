/*
 * fd_oracle.c -- FP64 CPU restatement of the reference's frequency-domain operator and its
 * BiCGStab(L) solver (test infrastructure: only tests and bench.py's CPU legs use it).
 *
 * Follows src/freq_domain_inverse_design/ of the reference:
 *   operator_mod.f90:41-232   init_operator (derivative coefficients, PML stretch factors)
 *   operator_mod.f90:293-361  apply_operator_1D (components pl_x, pl_y, mi_x, mi_y)
 *   operator_mod.f90:364-514  apply_operator_2D
 *   operator_mod.f90:518-710  apply_operator_3D (periodic ghost copies, curl of the
 *                             Riemann-Silberstein vectors, medium term)
 *   bicgstab_mod.f90:76-243   BICGStab_L
 *   rs_operations_subs_mod.f90 (vector operations; dot products conj(v1).v2 over the interior,
 *                             components in the order pl_x, pl_y, pl_z, mi_x, mi_y, mi_z)
 * Units are the program's own (constants_mod.f90:16-21: c0 = eps0 = mu0 = 1).
 * Parity against the reference itself is unpinned (no Fortran compiler); pinned by the
 * manufactured-solution and residual checks of tests/test_fd_oracle.py.
 *
 * Complex numbers are (re, im) pairs and every product is written out as the reference's
 * complex(dp) arithmetic computes it, so that the GPU kernels can match it bit for bit.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct { double re, im; } cplx;

static cplx cadd(cplx a, cplx b) { cplx r = {a.re + b.re, a.im + b.im}; return r; }
static cplx csub(cplx a, cplx b) { cplx r = {a.re - b.re, a.im - b.im}; return r; }
static cplx cmul(cplx a, cplx b) { cplx r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; return r; }
static cplx cscale(cplx a, double s) { cplx r = {a.re * s, a.im * s}; return r; }
/* complex division by Smith's method (R. L. Smith, CACM 5:435, 1962), the range-reduced form
 * gfortran uses for complex(dp) division under its default Fortran rules */
static cplx cdiv(cplx a, cplx b)
{
    cplx r;
    if (fabs(b.re) < fabs(b.im)) {
        const double t = b.re / b.im, d = b.re * t + b.im;
        r.re = (a.re * t + a.im) / d;
        r.im = (a.im * t - a.re) / d;
    } else {
        const double t = b.im / b.re, d = b.im * t + b.re;
        r.re = (a.im * t + a.re) / d;
        r.im = (a.im - a.re * t) / d;
    }
    return r;
}

/* operator state: padded component arrays are (nx+2g) x (ny+2gy) x (nz+2gz), x fastest, with
 * ghosts only along the active axes (ny = nz = 1 in 1D, nz = 1 in 2D); 4 components in 1D
 * (pl_x, pl_y, mi_x, mi_y), 6 otherwise (pl_x, pl_y, pl_z, mi_x, mi_y, mi_z) */
typedef struct {
    int dims, ncomp, nx, ny, nz, g, gy, gz, n_der, boundaries[3];
    double dr, w0;
    double coef[9];            /* coef_der(-n..n) / dr at coef[n + ii] */
    cplx *sx, *sy, *sz;        /* s_inv per interior index (0-based) */
    cplx *eps;                 /* nx x ny x nz */
} fd_op;

static long long fd_idx(const fd_op *A, int i, int j, int k)   /* 1-based interior indices */
{
    const long long px = A->nx + 2 * A->g, py = A->ny + 2 * A->gy;
    return (long long)(i - 1 + A->g) + px * ((long long)(j - 1 + A->gy) + py * (long long)(k - 1 + A->gz));
}

/* padded length of one component */
long long fd_vec_len(int dims, int nx, int ny, int nz, int n_der)
{
    const int gy = dims >= 2 ? n_der : 0, gz = dims == 3 ? n_der : 0;
    return (long long)(nx + 2 * n_der) * (ny + 2 * gy) * (nz + 2 * gz);
}
static long long fd_len(const fd_op *A) { return fd_vec_len(A->dims, A->nx, A->ny, A->nz, A->g); }

/* operator_mod.f90:97-140 (coefficients) and :185-232 (stretch factors) */
fd_op *fd_create(int dims, int nx, int ny, int nz, int n_pml, int n_der, const int boundaries[3], double dr,
                 double w0, const double *eps_re_im)
{
    static const double C1[3] = {-0.5, 0.0, 0.5};
    fd_op *A = (fd_op *)calloc(1, sizeof(fd_op));
    int i, q;
    if (dims < 3) nz = 1;
    if (dims < 2) ny = 1;
    A->dims = dims; A->ncomp = dims == 1 ? 4 : 6;
    A->nx = nx; A->ny = ny; A->nz = nz; A->g = n_der; A->n_der = n_der;
    A->gy = dims >= 2 ? n_der : 0; A->gz = dims == 3 ? n_der : 0;
    for (q = 0; q < 3; ++q) A->boundaries[q] = boundaries[q];
    A->dr = dr; A->w0 = w0;
    {
        double c[9] = {0};
        if (n_der == 1) { c[0] = C1[0]; c[1] = C1[1]; c[2] = C1[2]; }
        else if (n_der == 2) { c[0] = 1.0 / 12.0; c[1] = -2.0 / 3.0; c[2] = 0.0; c[3] = 2.0 / 3.0; c[4] = -1.0 / 12.0; }
        else if (n_der == 3) {
            c[0] = -1.0 / 60.0; c[1] = 3.0 / 20.0; c[2] = -3.0 / 4.0; c[3] = 0.0;
            c[4] = 3.0 / 4.0; c[5] = -3.0 / 20.0; c[6] = 1.0 / 60.0;
        } else {
            c[0] = 1.0 / 280.0; c[1] = -4.0 / 105.0; c[2] = 1.0 / 5.0; c[3] = -4.0 / 5.0; c[4] = 0.0;
            c[5] = 4.0 / 5.0; c[6] = -1.0 / 5.0; c[7] = 4.0 / 105.0; c[8] = -1.0 / 280.0;
        }
        for (q = 0; q <= 2 * n_der; ++q) A->coef[q] = c[q] / dr;      /* coef_der = coef_der / dr */
    }
    A->sx = (cplx *)malloc(sizeof(cplx) * nx);
    A->sy = (cplx *)malloc(sizeof(cplx) * ny);
    A->sz = (cplx *)malloc(sizeof(cplx) * nz);
    for (i = 0; i < nx; ++i) { A->sx[i].re = 1.0; A->sx[i].im = 0.0; }
    for (i = 0; i < ny; ++i) { A->sy[i].re = 1.0; A->sy[i].im = 0.0; }
    for (i = 0; i < nz; ++i) { A->sz[i].re = 1.0; A->sz[i].im = 0.0; }
    {
        /* sig_max = 0.8 (m+1) / (dr sqrt(mu0/eps0)), m = 3, kappa_max = 5, eps0 = mu0 = 1 */
        const double m = 3.0, kmax = 5.0;
        const double sig_max = 0.8 * (m + 1.0) / (dr * sqrt(1.0 / 1.0));
        cplx *s[3] = {A->sx, A->sy, A->sz};
        const int n[3] = {nx, ny, nz};
        int a;
        for (a = 0; a < dims; ++a) {
            if (boundaries[a] != 3) continue;
            for (i = 1; i <= n_pml; ++i) {
                const double r = (double)(n_pml - i + 1) / (double)n_pml;
                const double sig = sig_max * pow(r, m);
                const double kap = 1.0 + (kmax - 1.0) * pow(r, m);
                /* s_i = kappa + sig / (i w0 eps0) = kappa - i sig / w0 */
                const cplx si = {kap, -(sig / w0)};
                const cplx one = {1.0, 0.0};
                s[a][i - 1] = cdiv(one, si);                       /* low face, i = 1 .. n_pml */
                s[a][n[a] - n_pml + (n_pml - i)] = cdiv(one, si);   /* high face, mirrored */
            }
        }
    }
    A->eps = (cplx *)malloc(sizeof(cplx) * (size_t)nx * ny * nz);
    memcpy(A->eps, eps_re_im, sizeof(cplx) * (size_t)nx * ny * nz);
    return A;
}

void fd_destroy(fd_op *A)
{
    if (!A) return;
    free(A->sx); free(A->sy); free(A->sz); free(A->eps); free(A);
}

/* periodic ghost copies (non-MPI branches), in the reference's order.  1D (operator_mod.f90:
 * 316-329): the four components along x.  2D (:389-452): all six components, x ghosts over the
 * interior rows, then y ghosts over the interior columns.  3D (:549-621): x ghosts over interior
 * y, z; y ghosts over interior x, z; z ghosts over interior x, y -- and the 3D y block copies
 * mi_x only into the low ghosts and mi_y only into the high ghosts (as written in the
 * reference), so the other two stay zero. */
static void fd_ghosts(const fd_op *A, cplx **f)
{
    const int nx = A->nx, ny = A->ny, nz = A->nz, g = A->g;
    int c, i, j, k, t;
    if (A->boundaries[0] == 2)
        for (c = 0; c < A->ncomp; ++c)
            for (k = 1; k <= nz; ++k)
                for (j = 1; j <= ny; ++j)
                    for (t = 1; t <= g; ++t) {
                        f[c][fd_idx(A, 1 - t, j, k)] = f[c][fd_idx(A, nx + 1 - t, j, k)];
                        f[c][fd_idx(A, nx + t, j, k)] = f[c][fd_idx(A, t, j, k)];
                    }
    if (A->dims >= 2 && A->boundaries[1] == 2)
        for (c = 0; c < 6; ++c) {
            const int lo = A->dims == 2 || c != 4, hi = A->dims == 2 || c != 3;   /* the 3D quirk */
            for (k = 1; k <= nz; ++k)
                for (t = 1; t <= g; ++t)
                    for (i = 1; i <= nx; ++i) {
                        if (lo) f[c][fd_idx(A, i, 1 - t, k)] = f[c][fd_idx(A, i, ny + 1 - t, k)];
                        if (hi) f[c][fd_idx(A, i, ny + t, k)] = f[c][fd_idx(A, i, t, k)];
                    }
        }
    if (A->dims == 3 && A->boundaries[2] == 2)
        for (c = 0; c < 6; ++c)
            for (t = 1; t <= g; ++t)
                for (j = 1; j <= ny; ++j)
                    for (i = 1; i <= nx; ++i) {
                        f[c][fd_idx(A, i, j, 1 - t)] = f[c][fd_idx(A, i, j, nz + 1 - t)];
                        f[c][fd_idx(A, i, j, nz + t)] = f[c][fd_idx(A, i, j, t)];
                    }
}

/* apply_operator_1D (operator_mod.f90:293-361): the derivative runs along the grid's one axis
 * (named z there); the products keep the reference's left-to-right order, C1 * d * s_inv, and
 * the y components carry no medium term (as written in the reference) */
static void fd_apply1(const fd_op *A, cplx **f, cplx **Af, cplx C1, cplx C2, cplx C3, cplx C4)
{
    const int n = A->n_der;
    int i, q;
    for (i = 1; i <= A->nx; ++i) {
        cplx dpxdz = {0, 0}, dpydz = {0, 0}, dmxdz = {0, 0}, dmydz = {0, 0};
        const long long p = fd_idx(A, i, 1, 1);
        for (q = -n; q <= n; ++q) {
            const double a = A->coef[n + q];
            dpxdz = cadd(dpxdz, cscale(f[0][p + q], a));
            dpydz = cadd(dpydz, cscale(f[1][p + q], a));
            dmxdz = cadd(dmxdz, cscale(f[2][p + q], a));
            dmydz = cadd(dmydz, cscale(f[3][p + q], a));
        }
        {
            const cplx Ex = cadd(f[0][p], f[2][p]);
            const cplx s = A->sx[i - 1], e = A->eps[i - 1];
            const cplx m3 = cmul(C3, csub(e, C4));
            const cplx mC1 = {-C1.re, -C1.im};
            Af[0][p] = cadd(cadd(cmul(cmul(mC1, dpydz), s), cmul(C2, f[0][p])), cmul(m3, Ex));
            Af[1][p] = cadd(cmul(cmul(C1, dpxdz), s), cmul(C2, f[1][p]));
            Af[2][p] = cadd(cadd(cmul(cmul(C1, dmydz), s), cmul(C2, f[2][p])), cmul(m3, Ex));
            Af[3][p] = cadd(cmul(cmul(mC1, dmxdz), s), cmul(C2, f[3][p]));
        }
    }
}

/* apply_operator_2D (operator_mod.f90:364-514): its curl terms carry the opposite sign of the 3D
 * operator's (pl_x = -C1 dpz/dy ..., as written in the reference) */
static void fd_apply2(const fd_op *A, cplx **f, cplx **Af, cplx C1, cplx C2, cplx C3, cplx C4)
{
    const int n = A->n_der;
    const long long sy = A->nx + 2 * A->g;
    int i, j, q;
    for (j = 1; j <= A->ny; ++j)
        for (i = 1; i <= A->nx; ++i) {
            cplx dpxdy = {0, 0}, dpydx = {0, 0}, dpzdx = {0, 0}, dpzdy = {0, 0};
            cplx dmxdy = {0, 0}, dmydx = {0, 0}, dmzdx = {0, 0}, dmzdy = {0, 0};
            const long long p = fd_idx(A, i, j, 1);
            for (q = -n; q <= n; ++q) {
                const double a = A->coef[n + q];
                dpydx = cadd(dpydx, cscale(f[1][p + q], a));
                dpzdx = cadd(dpzdx, cscale(f[2][p + q], a));
                dmydx = cadd(dmydx, cscale(f[4][p + q], a));
                dmzdx = cadd(dmzdx, cscale(f[5][p + q], a));
            }
            for (q = -n; q <= n; ++q) {
                const double a = A->coef[n + q];
                dpxdy = cadd(dpxdy, cscale(f[0][p + q * sy], a));
                dpzdy = cadd(dpzdy, cscale(f[2][p + q * sy], a));
                dmxdy = cadd(dmxdy, cscale(f[3][p + q * sy], a));
                dmzdy = cadd(dmzdy, cscale(f[5][p + q * sy], a));
            }
            {
                const cplx Ex = cadd(f[0][p], f[3][p]), Ey = cadd(f[1][p], f[4][p]), Ez = cadd(f[2][p], f[5][p]);
                const cplx sxi = A->sx[i - 1], syj = A->sy[j - 1];
                const cplx e = A->eps[(size_t)(i - 1) + (size_t)A->nx * (j - 1)];
                const cplx m3 = cmul(C3, csub(e, C4));
                const cplx mC1 = {-C1.re, -C1.im};
                dpxdy = cmul(dpxdy, syj); dpydx = cmul(dpydx, sxi);
                dpzdx = cmul(dpzdx, sxi); dpzdy = cmul(dpzdy, syj);
                dmxdy = cmul(dmxdy, syj); dmydx = cmul(dmydx, sxi);
                dmzdx = cmul(dmzdx, sxi); dmzdy = cmul(dmzdy, syj);
                Af[0][p] = cadd(cadd(cmul(mC1, dpzdy), cmul(C2, f[0][p])), cmul(m3, Ex));
                Af[1][p] = cadd(cadd(cmul(C1, dpzdx), cmul(C2, f[1][p])), cmul(m3, Ey));
                Af[2][p] = cadd(cadd(cmul(mC1, csub(dpydx, dpxdy)), cmul(C2, f[2][p])), cmul(m3, Ez));
                Af[3][p] = cadd(cadd(cmul(C1, dmzdy), cmul(C2, f[3][p])), cmul(m3, Ex));
                Af[4][p] = cadd(cadd(cmul(mC1, dmzdx), cmul(C2, f[4][p])), cmul(m3, Ey));
                Af[5][p] = cadd(cadd(cmul(C1, csub(dmydx, dmxdy)), cmul(C2, f[5][p])), cmul(m3, Ez));
            }
        }
}

/* apply_operator (operator_mod.f90:261-289) for 1D / 2D / 3D; f and Af are ncomp padded complex
 * arrays; the ghosts of f are refreshed first */
void fd_apply(const fd_op *A, double *f_flat, double *Af_flat, int transpose)
{
    const long long len = fd_len(A);
    cplx *f[6], *Af[6];
    int c, i, j, k, q;
    const double sign = transpose ? -1.0 : 1.0;
    /* C1 = sign c0 i, C2 = -w0 i, C3 = -w0 i / (2 eps0), C4 = eps0 */
    const cplx C1 = {0.0, sign}, C2 = {0.0, -A->w0}, C3 = {0.0, -A->w0 / 2.0}, C4 = {1.0, 0.0};
    const int n = A->n_der;
    for (c = 0; c < A->ncomp; ++c) {
        f[c] = (cplx *)f_flat + c * len;
        Af[c] = (cplx *)Af_flat + c * len;
    }
    fd_ghosts(A, f);
    if (A->dims == 1) {
        fd_apply1(A, f, Af, C1, C2, C3, C4);
        return;
    }
    if (A->dims == 2) {
        fd_apply2(A, f, Af, C1, C2, C3, C4);
        return;
    }
    for (k = 1; k <= A->nz; ++k)
        for (j = 1; j <= A->ny; ++j)
            for (i = 1; i <= A->nx; ++i) {
                cplx dpydx = {0, 0}, dpzdx = {0, 0}, dmydx = {0, 0}, dmzdx = {0, 0};
                cplx dpxdy = {0, 0}, dpzdy = {0, 0}, dmxdy = {0, 0}, dmzdy = {0, 0};
                cplx dpxdz = {0, 0}, dpydz = {0, 0}, dmxdz = {0, 0}, dmydz = {0, 0};
                const long long p = fd_idx(A, i, j, k);
                const long long sy = A->nx + 2 * A->g, sz = sy * (A->ny + 2 * A->gy);
                for (q = -n; q <= n; ++q) {
                    const double a = A->coef[n + q];
                    dpydx = cadd(dpydx, cscale(f[1][p + q], a));
                    dpzdx = cadd(dpzdx, cscale(f[2][p + q], a));
                    dmydx = cadd(dmydx, cscale(f[4][p + q], a));
                    dmzdx = cadd(dmzdx, cscale(f[5][p + q], a));
                }
                for (q = -n; q <= n; ++q) {
                    const double a = A->coef[n + q];
                    dpxdy = cadd(dpxdy, cscale(f[0][p + q * sy], a));
                    dpzdy = cadd(dpzdy, cscale(f[2][p + q * sy], a));
                    dmxdy = cadd(dmxdy, cscale(f[3][p + q * sy], a));
                    dmzdy = cadd(dmzdy, cscale(f[5][p + q * sy], a));
                }
                for (q = -n; q <= n; ++q) {
                    const double a = A->coef[n + q];
                    dpxdz = cadd(dpxdz, cscale(f[0][p + q * sz], a));
                    dpydz = cadd(dpydz, cscale(f[1][p + q * sz], a));
                    dmxdz = cadd(dmxdz, cscale(f[3][p + q * sz], a));
                    dmydz = cadd(dmydz, cscale(f[4][p + q * sz], a));
                }
                {
                    const cplx Ex = cadd(f[0][p], f[3][p]), Ey = cadd(f[1][p], f[4][p]), Ez = cadd(f[2][p], f[5][p]);
                    const cplx sxi = A->sx[i - 1], syj = A->sy[j - 1], szk = A->sz[k - 1];
                    const cplx e = A->eps[(size_t)(i - 1) + (size_t)A->nx * ((size_t)(j - 1) + (size_t)A->ny * (k - 1))];
                    cplx m3;
                    dpxdy = cmul(dpxdy, syj); dpxdz = cmul(dpxdz, szk);
                    dpydx = cmul(dpydx, sxi); dpydz = cmul(dpydz, szk);
                    dpzdx = cmul(dpzdx, sxi); dpzdy = cmul(dpzdy, syj);
                    dmxdy = cmul(dmxdy, syj); dmxdz = cmul(dmxdz, szk);
                    dmydz = cmul(dmydz, szk); dmydx = cmul(dmydx, sxi);
                    dmzdx = cmul(dmzdx, sxi); dmzdy = cmul(dmzdy, syj);
                    m3 = cmul(C3, csub(e, C4));
                    {
                        const cplx mC1 = {-C1.re, -C1.im};
                        Af[0][p] = cadd(cadd(cmul(C1, csub(dpzdy, dpydz)), cmul(C2, f[0][p])), cmul(m3, Ex));
                        Af[1][p] = cadd(cadd(cmul(C1, csub(dpxdz, dpzdx)), cmul(C2, f[1][p])), cmul(m3, Ey));
                        Af[2][p] = cadd(cadd(cmul(C1, csub(dpydx, dpxdy)), cmul(C2, f[2][p])), cmul(m3, Ez));
                        Af[3][p] = cadd(cadd(cmul(mC1, csub(dmzdy, dmydz)), cmul(C2, f[3][p])), cmul(m3, Ex));
                        Af[4][p] = cadd(cadd(cmul(mC1, csub(dmxdz, dmzdx)), cmul(C2, f[4][p])), cmul(m3, Ey));
                        Af[5][p] = cadd(cadd(cmul(mC1, csub(dmydx, dmxdy)), cmul(C2, f[5][p])), cmul(m3, Ez));
                    }
                }
            }
}

/* ---- BiCGStab(L), bicgstab_mod.f90:76-243 ------------------------------------------------- */
static cplx fd_dot(const fd_op *A, const double *v1, const double *v2)
{
    const long long len = fd_len(A);
    cplx s = {0, 0};
    int c, i, j, k;
    for (c = 0; c < A->ncomp; ++c) {
        cplx sc = {0, 0};
        for (k = 1; k <= A->nz; ++k)
            for (j = 1; j <= A->ny; ++j)
                for (i = 1; i <= A->nx; ++i) {
                    const long long p = c * len + fd_idx(A, i, j, k);
                    const cplx a = {v1[2 * p], -v1[2 * p + 1]}, b = {v2[2 * p], v2[2 * p + 1]};
                    sc = cadd(sc, cmul(a, b));
                }
        s = cadd(s, sc);
    }
    return s;
}
/* v1 = v1 + a v2 (interior) */
static void fd_axpy(const fd_op *A, double *v1, const double *v2, cplx a)
{
    const long long len = fd_len(A);
    int c, i, j, k;
    for (c = 0; c < A->ncomp; ++c)
        for (k = 1; k <= A->nz; ++k)
            for (j = 1; j <= A->ny; ++j)
                for (i = 1; i <= A->nx; ++i) {
                    const long long p = c * len + fd_idx(A, i, j, k);
                    const cplx x = {v1[2 * p], v1[2 * p + 1]}, y = {v2[2 * p], v2[2 * p + 1]};
                    const cplx r = cadd(x, cmul(a, y));
                    v1[2 * p] = r.re; v1[2 * p + 1] = r.im;
                }
}
/* v1 = a v1 (interior) */
static void fd_scale(const fd_op *A, double *v1, cplx a)
{
    const long long len = fd_len(A);
    int c, i, j, k;
    for (c = 0; c < A->ncomp; ++c)
        for (k = 1; k <= A->nz; ++k)
            for (j = 1; j <= A->ny; ++j)
                for (i = 1; i <= A->nx; ++i) {
                    const long long p = c * len + fd_idx(A, i, j, k);
                    const cplx x = {v1[2 * p], v1[2 * p + 1]};
                    const cplx r = cmul(a, x);
                    v1[2 * p] = r.re; v1[2 * p + 1] = r.im;
                }
}
/* v1 = a v1 + v2 (interior) */
static void fd_xpay(const fd_op *A, double *v1, const double *v2, cplx a)
{
    const long long len = fd_len(A);
    int c, i, j, k;
    for (c = 0; c < A->ncomp; ++c)
        for (k = 1; k <= A->nz; ++k)
            for (j = 1; j <= A->ny; ++j)
                for (i = 1; i <= A->nx; ++i) {
                    const long long p = c * len + fd_idx(A, i, j, k);
                    const cplx x = {v1[2 * p], v1[2 * p + 1]}, y = {v2[2 * p], v2[2 * p + 1]};
                    const cplx r = cadd(cmul(a, x), y);
                    v1[2 * p] = r.re; v1[2 * p + 1] = r.im;
                }
}

/* f_out: initial guess in, solution out; returns the number of outer iterations */
int fd_bicgstab_l(const fd_op *A, const double *j_vec, double *f_out, int transpose, double tol, int n_max, int L,
                  int *converged, double *abs_err)
{
    const long long len2 = 2LL * A->ncomp * fd_len(A);   /* doubles per vector */
    double *r0 = (double *)calloc(len2, sizeof(double));
    double *r = (double *)calloc(len2 * (L + 1), sizeof(double));
    double *u = (double *)calloc(len2 * (L + 1), sizeof(double));
    double *f = (double *)calloc(len2, sizeof(double));
    double *Af = (double *)calloc(len2, sizeof(double));
    cplx tau[9][9], gam[9], gam_p[9], gam_pp[9], sig[9];
    cplx rho0 = {1, 0}, rho1 = {1, 0}, alpha = {1, 0}, omega = {1, 0}, beta, dot;
    const cplx mone = {-1, 0};
    double norm_t, err_r = 1.0;
    int n = 0, l, i, conv = 0;
    memset(tau, 0, sizeof tau); memset(gam, 0, sizeof gam); memset(gam_p, 0, sizeof gam_p);
    memset(gam_pp, 0, sizeof gam_pp); memset(sig, 0, sizeof sig);
    memcpy(f, f_out, len2 * sizeof(double));                         /* copy_V2_on_V1(f_vec_out, f_vec) */
    fd_apply(A, f, Af, transpose);
    memcpy(r0, j_vec, len2 * sizeof(double));                        /* r0 = j - A f */
    fd_axpy(A, r0, Af, mone);
    memcpy(r, r0, len2 * sizeof(double));                            /* r(0) = r0 */
    dot = fd_dot(A, r0, r0);
    norm_t = sqrt(dot.re);
    fd_scale(A, r0, (cplx){1.0 / norm_t, 0.0});      /* self_product_aV1(r0, Z_ONE * norm_inv) */
    dot = fd_dot(A, j_vec, j_vec);
    norm_t = sqrt(dot.re);
    while (n <= n_max && !conv) {
        rho0 = cmul(cscale(omega, -1.0), rho0);
        for (l = 0; l <= L - 1; ++l) {
            dot = fd_dot(A, r0, r + l * len2);
            rho1 = dot;
            beta = cdiv(cmul(alpha, rho1), rho0);
            rho0 = rho1;
            for (i = 0; i <= l; ++i) fd_xpay(A, u + i * len2, r + i * len2, cscale(beta, -1.0));
            fd_apply(A, u + l * len2, u + (l + 1) * len2, transpose);
            dot = fd_dot(A, r0, u + (l + 1) * len2);
            alpha = cdiv(rho0, dot);
            for (i = 0; i <= l; ++i) fd_axpy(A, r + i * len2, u + (i + 1) * len2, cscale(alpha, -1.0));
            fd_apply(A, r + l * len2, r + (l + 1) * len2, transpose);
            dot = fd_dot(A, r + (l + 1) * len2, r + (l + 1) * len2);
            fd_axpy(A, f_out, u, alpha);
        }
        for (l = 1; l <= L; ++l) {
            for (i = 1; i <= l - 1; ++i) {
                dot = fd_dot(A, r + i * len2, r + l * len2);
                tau[i][l] = cdiv(dot, sig[i]);
                fd_axpy(A, r + l * len2, r + i * len2, cscale(tau[i][l], -1.0));
            }
            sig[l] = fd_dot(A, r + l * len2, r + l * len2);
            dot = fd_dot(A, r + l * len2, r);
            gam_p[l] = cdiv(dot, sig[l]);
        }
        gam[L] = gam_p[L];
        omega = gam[L];
        for (l = L - 1; l >= 1; --l) {
            gam[l] = gam_p[l];
            for (i = l + 1; i <= L; ++i) gam[l] = csub(gam[l], cmul(tau[l][i], gam[i]));
        }
        for (l = 1; l <= L - 1; ++l) {
            gam_pp[l] = gam[l + 1];
            for (i = l + 1; i <= L - 1; ++i) gam_pp[l] = cadd(gam_pp[l], cmul(tau[l][i], gam[i + 1]));
        }
        fd_axpy(A, f_out, r, gam[1]);
        fd_axpy(A, r, r + L * len2, cscale(gam_p[L], -1.0));
        fd_axpy(A, u, u + L * len2, cscale(gam[L], -1.0));
        for (l = 1; l <= L - 1; ++l) {
            fd_axpy(A, u, u + l * len2, cscale(gam[l], -1.0));
            fd_axpy(A, f_out, r + l * len2, gam_pp[l]);
            fd_axpy(A, r, r + l * len2, cscale(gam_p[l], -1.0));
        }
        dot = fd_dot(A, r, r);
        err_r = sqrt(dot.re);
        n = n + 1;
        if (err_r <= tol * norm_t) conv = 1;
    }
    *converged = conv;
    *abs_err = err_r / norm_t;
    free(r0); free(r); free(u); free(f); free(Af);
    return n;
}
