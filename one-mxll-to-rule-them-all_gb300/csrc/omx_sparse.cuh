// omx_sparse.cuh -- the small kernels around the stencil: source injection, emitter
// gather / density-matrix step / current scatter, the emitter-current term of the E update,
// and detector sampling.  All arithmetic here is FP64 (also on the FP32 field path) and is
// compiled without FMA contraction so that it reproduces the FP64 CPU oracle bit for bit.
#pragma once
#include "omx_internal.h"
#include "omx_emitter.cuh"
#include "omx_post.cuh"

namespace omx {

// ---- source_interactions (interactions_mod.f90:21-163) ----------------------------------------
// J_mat = amp*ker (amp = j_amp*envelope*cos, computed on the host with the reference's libm
// calls); J_av = 0.5*(J_mat(p) + J_mat(p+1 along dir)); E += c_src*J_av.
template <class R>
__device__ __forceinline__ void src_point(const FieldPtrs<R> &F, const SrcArgs &S, const StepParam &amp_p, int q)
{
    const double amp = sp_get(amp_p);
    const double ja = amp * S.ka[q];
    double jav;
    if (S.avg) {
        const double jb = amp * S.kb[q];
        jav = 0.5 * (ja + jb);
    } else {
        jav = ja;
    }
    R *E = F.f[S.comp];
    const long long e = S.eidx[q];
    E[e] = (R)((double)E[e] + S.c_src * jav);
}
template <class R>
__global__ void k_src(FieldPtrs<R> F, SrcArgs S, StepParam amp_p)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < S.n) src_point<R>(F, S, amp_p, q);
}

// Plane-wave soft source (extension): E_comp += c_src*amp on one plane of cells.
template <class R>
__global__ void k_plane(FieldPtrs<R> F, Lay L, PlaneArgs P, StepParam amp_p)
{
    const double amp = sp_get(amp_p);
    if (amp == 0.0) return;
    plane_point<R>(F, L, P, amp, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y);
}

// ---- emitter current in the E update (mxll_3D_mod.f90:756-761 and 2D/1D analogues) --------
// E -= dt_eps0 * Jav with Jav = 0.5*(J_old(i) + tt*dJ(i) + J_old(i+1) + tt*dJ(i+1)), tt =
// time - t_skip, evaluated only at E components next to an emitter current point and
// outside dispersive media (where the reference ignores J).
template <class R>
__global__ void k_inject(FieldPtrs<R> F, JState J, InjArgs I, StepParam time_p, StepParam tskip_p, double dt_eps0)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= I.n) return;
    inject_point<R>(F, J, I, sp_get(time_p) - sp_get(tskip_p), dt_eps0, q);
}

// send_E_to_J_ranks (interactions_mod.f90:656-691, 2D :486-526, 1D :329-346) fused with
// td_propagate_q_group (q_group_mod.f90:813-816): gather E at the emitter cell, advance the
// density matrix, dipole = Tr(rho V) along u, dPt_dt = (dipole - dip_old)/dt.
template <class R>
__global__ void k_emit(FieldPtrs<R> F, Lay L, EmitArgs A, StepParam move_p)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= A.n) return;
    if (sp_get(move_p) == 0.0) return;
    if (A.only_if && *A.only_if == 0) return;
    const int i = A.ci[n], j = A.cj[n], k = A.ck[n];
    const long long c = L.off + i + (long long)L.px * j + L.pz * k;
    double E[3] = {0.0, 0.0, 0.0};
    if (A.dims == 3) {
        E[0] = 0.5 * ((double)F.f[0][c - 1] + (double)F.f[0][c]);
        E[1] = 0.5 * ((double)F.f[1][c - L.px] + (double)F.f[1][c]);
        E[2] = 0.5 * ((double)F.f[2][c - L.pz] + (double)F.f[2][c]);
    } else if (A.dims == 2) {
        if (A.mode2d == 2) {
            E[0] = 0.5 * ((double)F.f[0][c - 1] + (double)F.f[0][c]);
            E[1] = 0.5 * ((double)F.f[1][c - L.px] + (double)F.f[1][c]);
        } else {
            E[2] = (double)F.f[2][c];
        }
    } else {
        E[0] = (double)F.f[0][c];
    }
    const double *pr = A.par + (long long)n * A.npar;
    const double *u = pr + (A.npar - 3);
    const double E_u = u[0] * E[0] + u[1] * E[1] + u[2] * E[2];
    double rho[8];
    double *st = A.rho + (long long)n * A.nst;
    double d;
    const double g1 = A.rates[2 * n], g2 = A.rates[2 * n + 1];
    if (A.model == 1) {
#pragma unroll
        for (int q = 0; q < 3; ++q) rho[q] = st[q];
        rk4r<3>(1, pr, rho, E_u, A.dt, A.h2, A.h6, g1, g2);
#pragma unroll
        for (int q = 0; q < 3; ++q) st[q] = rho[q];
        d = 2.0 * pr[1] * rho[1];
    } else {
#pragma unroll
        for (int q = 0; q < 8; ++q) rho[q] = st[q];
        rk4r<8>(2, pr, rho, E_u, A.dt, A.h2, A.h6, g1, g2);
#pragma unroll
        for (int q = 0; q < 8; ++q) st[q] = rho[q];
        d = 2.0 * pr[2] * rho[2] + 2.0 * pr[3] * rho[4];
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double old = A.dipole[3 * n + a];
        const double nw = d * u[a];
        A.dipole[3 * n + a] = nw;
        A.dPdt[3 * n + a] = A.inv_dt != 0.0 ? (nw - old) * A.inv_dt : (nw - old) / A.dt;
        A.E[3 * n + a] = E[a];
    }
}

// send_J_to_E_ranks (interactions_mod.f90:1046-1220): J_old = J; J(point) = wk*dPt_dt of the
// last emitter writing the point (assignment); dJ = (J - J_old)/dt (times 1/dt with FP32 fields,
// as dPt_dt in k_emit).  Points this group does not write keep J, so their dJ becomes zero, as
// with the reference's full-grid passes.
__global__ void k_scatter(JState J, ScatArgs S, StepParam move_p)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= S.np) return;
    if (sp_get(move_p) == 0.0) return;
    const int w = S.win[p];
    for (int c = S.c0; c <= S.c1; ++c) {
        const double jo = J.J[c][p];
        const double jn = (w >= 0) ? S.wk[p] * S.dPdt[3 * w + c] : jo;
        J.Jo[c][p] = jo;
        J.J[c][p] = jn;
        J.dJ[c][p] = S.inv_dt != 0.0 ? (jn - jo) * S.inv_dt : (jn - jo) / S.dt;
    }
}

// ---- detector sampling (write_fields_subs_mod.f90 stencils) -------------------------------
template <class R>
__device__ __forceinline__ void sample_point(const FieldPtrs<R> &F, const DetArgs &D, const StepParam &slot_p,
                                             const StepParam &time_p, int s)
{
    const int slot = (int)sp_get(slot_p);
    if (slot < 0) return;
    if (s == 0) D.times[slot] = sp_get(time_p);
    if (s >= D.n) return;
    const R *a = F.f[D.field[s]];
    const int nt = D.nt[s];
    double v = (double)a[D.t0[s]];
    if (nt >= 2) {
        v = v + (double)a[D.t1[s]];
        if (nt == 4) {
            v = v + (double)a[D.t2[s]];
            v = v + (double)a[D.t3[s]];
        }
        v = D.w[s] * v;
    }
    D.rec[(long long)slot * D.n + s] = v;
    if (D.n_freq > 0) {
        const double t = sp_get(time_p);
        for (int k = 0; k < D.n_freq; ++k) {
            double sn, cs;
            sincos(D.omega[k] * t, &sn, &cs);
            D.dft_re[(long long)k * D.n + s] += D.dft_w * v * cs;
            D.dft_im[(long long)k * D.n + s] -= D.dft_w * v * sn;
        }
    }
}
template <class R>
__global__ void k_sample(FieldPtrs<R> F, DetArgs D, StepParam slot_p, StepParam time_p)
{
    sample_point<R>(F, D, slot_p, time_p, blockIdx.x * blockDim.x + threadIdx.x);
}

__global__ void k_step_advance(int *step)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) *step = *step + 1;
}

__global__ void k_flush(float *buf, long long n)
{
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
        buf[q] = buf[q] * 0.5f + 1.0f;
}

// ---- batched forms for several grids (one launch for the sources / detectors of all grids) ----
// entry of point q in a list of entries with ascending first points p0
template <class E> __device__ __forceinline__ int batch_entry(const E *e, int n, long long q)
{
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (e[mid].p0 <= q) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <class R> __global__ void k_src_batch(const BatchSrc<R> *__restrict__ e, int n, long long total)
{
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= total) return;
    const int k = batch_entry(e, n, q);
    src_point<R>(e[k].F, e[k].S, e[k].amp, (int)(q - e[k].p0));
}

template <class R> __global__ void k_sample_batch(const BatchDet<R> *__restrict__ e, int n, long long total)
{
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= total) return;
    const int k = batch_entry(e, n, q);
    sample_point<R>(e[k].F, e[k].D, e[k].slot, e[k].time, (int)(q - e[k].p0));
}

// ---- closure training data: the plain propagator under band-limited drives -------------------
__global__ void k_cl_trajectories(ClTrajArgs A)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= A.n) return;
    const double *pr = A.params + (long long)q * A.npar;
    const double *dv = A.drive + (long long)q * (1 + 3 * A.K);
    const int m = A.model == 1 ? 2 : 4;
    const double g1 = 1.0 / pr[m], g2 = 1.0 / pr[m + 1], h2 = 0.5 * A.dt, h6 = A.dt / 6.0;
    double rho[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int s = 0; s < A.T; ++s) {
        const double t = A.dt * s;
        double E = 0.0;
        for (int k = 0; k < A.K; ++k) E += dv[1 + 3 * k] * cos(dv[2 + 3 * k] * t + dv[3 + 3 * k]);
        E = dv[0] * E;
        double d;
        if (A.model == 1) {
            rk4r<3>(1, pr, rho, E, A.dt, h2, h6, g1, g2);
            d = 2.0 * pr[1] * rho[1];
        } else {
            rk4r<8>(2, pr, rho, E, A.dt, h2, h6, g1, g2);
            d = 2.0 * pr[2] * rho[2] + 2.0 * pr[3] * rho[4];
        }
        A.e[(long long)q * A.T + s] = (float)(E / A.e_scale);
        A.d[(long long)q * A.T + s] = (float)(d / A.d_scale);
    }
}

// ---- closure deployment: the plain-arithmetic parts ---------------------------------------------
// E at the emitter cell (the k_emit stencils), kept in A.E; its component on the dipole axis
// goes into the window ring while the network runs
template <class R>
__global__ void k_cl_gather(FieldPtrs<R> F, Lay L, EmitArgs A, ClDeploy D, StepParam move_p)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    const bool move = sp_get(move_p) != 0.0;
    const int use_plain = D.st->use_plain;
    if (n == 0) {
        D.st->skip_nn = (!move || use_plain) ? 1 : 0;
        D.st->plain_now = use_plain;
    }
    if (n >= A.n || !move) return;
    const int i = A.ci[n], j = A.cj[n], k = A.ck[n];
    const long long c = L.off + i + (long long)L.px * j + L.pz * k;
    double E[3] = {0.0, 0.0, 0.0};
    if (A.dims == 3) {
        E[0] = 0.5 * ((double)F.f[0][c - 1] + (double)F.f[0][c]);
        E[1] = 0.5 * ((double)F.f[1][c - L.px] + (double)F.f[1][c]);
        E[2] = 0.5 * ((double)F.f[2][c - L.pz] + (double)F.f[2][c]);
    } else if (A.dims == 2) {
        if (A.mode2d == 2) {
            E[0] = 0.5 * ((double)F.f[0][c - 1] + (double)F.f[0][c]);
            E[1] = 0.5 * ((double)F.f[1][c - L.px] + (double)F.f[1][c]);
        } else {
            E[2] = (double)F.f[2][c];
        }
    } else {
        E[0] = (double)F.f[0][c];
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) A.E[3 * n + a] = E[a];
    if (!use_plain) {
        const double *u = A.par + (long long)n * A.npar + (A.npar - 3);
        const double E_u = u[0] * E[0] + u[1] * E[1] + u[2] * E[2];
        D.win[(long long)n * CL_WIN + (D.st->cl_step % CL_WIN)] = (float)(E_u / D.e_scale);
    }
}

__device__ __forceinline__ double cl_axis_dipole(const EmitArgs &A, const double *rho, const double *pr)
{
    return A.model == 1 ? 2.0 * pr[1] * rho[1] : 2.0 * pr[2] * rho[2] + 2.0 * pr[3] * rho[4];
}

// spot-check subset: the plain propagator on the sampled emitters with the gathered field; the
// difference to the network's dipole (already in A.dipole) feeds the running maxima
__global__ void k_cl_subset(EmitArgs A, ClDeploy D)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= D.n_sub || D.st->skip_nn) return;
    const int n = D.sub[s];
    const double *pr = A.par + (long long)n * A.npar;
    const double *u = pr + (A.npar - 3);
    const double E_u = u[0] * A.E[3 * n] + u[1] * A.E[3 * n + 1] + u[2] * A.E[3 * n + 2];
    double *rho = D.sub_rho + (long long)s * A.nst;
    double r[8];
    for (int q = 0; q < A.nst; ++q) r[q] = rho[q];
    const double g1 = A.rates[2 * n], g2 = A.rates[2 * n + 1];
    if (A.model == 1) rk4r<3>(1, pr, r, E_u, A.dt, A.h2, A.h6, g1, g2);
    else rk4r<8>(2, pr, r, E_u, A.dt, A.h2, A.h6, g1, g2);
    for (int q = 0; q < A.nst; ++q) rho[q] = r[q];
    const double dp = cl_axis_dipole(A, r, pr);
    const double dn = u[0] * A.dipole[3 * n] + u[1] * A.dipole[3 * n + 1] + u[2] * A.dipole[3 * n + 2];
    atomicMax(&D.st->err_bits, (unsigned long long)__double_as_longlong(fabs(dn - dp)));
    atomicMax(&D.st->scale_bits, (unsigned long long)__double_as_longlong(fabs(dp)));
}

// every check_every network steps: error = max |closure - plain| / max |plain| over the window;
// above tol the plain propagator takes over (and the density matrices are re-seeded)
__global__ void k_cl_check(ClDeploy D)
{
    ClDevState *st = D.st;
    st->reseed = 0;
    if (st->skip_nn) return;
    if (++st->steps_since_check < D.check_every) return;
    const double err = __longlong_as_double((long long)st->err_bits);
    const double sc = __longlong_as_double((long long)st->scale_bits);
    const double rel = sc > 0.0 ? err / sc : (err > 0.0 ? 1e300 : 0.0);
    st->last_err = rel;
    st->checks += 1;
    st->steps_since_check = 0;
    st->err_bits = 0ull;
    st->scale_bits = 0ull;
    if (rel > D.tol) {
        st->use_plain = 1;
        st->reseed = 1;
        st->fallback_step = st->cl_step;
    }
}

// on the fallback step: every emitter's density matrix restarts from the ground state and is
// replayed through its stored field window with the plain propagator (the sampled emitters take
// their exact plain state); the network's last dipole stays as the previous-step dipole
__global__ void k_cl_reseed(EmitArgs A, ClDeploy D)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= A.n || !D.st->reseed) return;
    double *rho = A.rho + (long long)n * A.nst;
    const int s = D.sub_of[n];
    if (s >= 0) {
        for (int q = 0; q < A.nst; ++q) rho[q] = D.sub_rho[(long long)s * A.nst + q];
        return;
    }
    const double *pr = A.par + (long long)n * A.npar;
    const double g1 = A.rates[2 * n], g2 = A.rates[2 * n + 1];
    double r[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const int head = D.st->cl_step % CL_WIN;        // the newest sample sits at head - 1
    for (int c = 0; c < CL_WIN; ++c) {
        const double E_u = (double)D.win[(long long)n * CL_WIN + (head + c) % CL_WIN] * D.e_scale;
        if (A.model == 1) rk4r<3>(1, pr, r, E_u, A.dt, A.h2, A.h6, g1, g2);
        else rk4r<8>(2, pr, r, E_u, A.dt, A.h2, A.h6, g1, g2);
    }
    for (int q = 0; q < A.nst; ++q) rho[q] = r[q];
}

// ---- field energy (FP64 reduction, one partial per block, summed in a fixed order) ----------------
template <class R>
__global__ void k_field_energy(FieldPtrs<R> F, Lay L, int c, double coef, double *part)
{
    __shared__ double sh[256];
    const long long nx = L.nx, ny = L.dims >= 2 ? L.ny : 1, nz = L.dims == 3 ? L.nz : 1;
    const long long total = nx * ny * nz;
    double acc = 0.0;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        const long long i = 1 + q % nx, j = (L.dims >= 2 ? 1 + (q / nx) % ny : 0), k = (L.dims == 3 ? 1 + q / (nx * ny) : 0);
        const double v = (double)F.f[c][L.off + i + (long long)L.px * j + L.pz * k];
        acc += v * v;
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] += coef * sh[0];
}

__global__ void k_sum_parts(const double *part, int n, double *out)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double s = 0.0;
        for (int q = 0; q < n; ++q) s += part[q];
        *out = s;
    }
}

}  // namespace omx
