// omx_capi.cpp -- the C-ABI entry points of include/omx_gpu.h: context creation (init_*Dgrid),
// media / source / q-group / detector set-up, per-call stepping and the whole-loop runner with
// optional CUDA-graph capture.  All device memory is owned here; kernels live in
// omx_kernels_{exact,fast}.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <functional>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <type_traits>
#include <unordered_map>
#include <vector>

#include "../../include/omx_gpu.h"
#include "omx_host.h"
#include "omx_internal.h"

namespace omx {
void set_global_error(const std::string &msg);
bool closure_infer(omx_closure *c, const ClDeploy &D, const EmitArgs &A, cudaStream_t s, std::string &err);
double closure_e_scale(const omx_closure *c);
double closure_d_scale(const omx_closure *c);
}

using namespace omx;

namespace {

thread_local std::string g_last_error = "";

struct Fail {
    int code;
    std::string msg;
};

inline void ck(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) throw Fail{OMX_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e)};
}
inline void req(bool ok, const std::string &msg, int code = OMX_ERR_ARG)
{
    if (!ok) throw Fail{code, msg};
}

// Host-to-device copy that has landed when it returns: cudaMemcpy from pageable memory may
// return before its DMA ends, and the legacy stream it uses does not order the library's
// non-blocking streams.
void h2d(void *dst, const void *src, size_t bytes, const char *what)
{
    ck(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice), what);
    ck(cudaStreamSynchronize(0), what);
}

template <class T> struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    void alloc(size_t count, bool zero = true)
    {
        release();
        if (count == 0) return;
        cudaError_t e = cudaMalloc(&p, count * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            throw Fail{OMX_ERR_NOMEM, std::string("cudaMalloc failed: ") + cudaGetErrorString(e)};
        }
        n = count;
        if (zero) {
            // the legacy stream does not order the library's non-blocking streams: wait for it
            ck(cudaMemset(p, 0, count * sizeof(T)), "cudaMemset");
            ck(cudaStreamSynchronize(0), "cudaMemset");
        }
    }
    void upload(const std::vector<T> &v)
    {
        alloc(v.size(), false);
        if (!v.empty()) h2d(p, v.data(), v.size() * sizeof(T), "upload");
    }
};

int field_code_to_index(int field) { return field - 1; }

}  // namespace

// ----------------------------------------------------------------------------------------------
struct SourceRec {
    int kind;            // 0 kernel source, 1 plane source
    omx_source_desc d;
    omx_plane_source_desc pd;
    int comp;            // 0..2
    int avg;
    double c_src;
    DevBuf<long long> eidx;
    DevBuf<double> ka, kb;
    int n;
    std::vector<int4> cells;   // (i, j, k, component) of every point
};

struct GroupRec {
    omx_qgroup_desc d;
    int npar, nst;
    // the device arrays hold the emitters sorted by cell (neighbouring threads gather neighbouring
    // field words, and the current's points, sorted by cell too, read neighbouring dPt_dt rows):
    // emitter order[d] of the caller's list is device row d, and device row inv[e] is emitter e
    std::vector<int> order, inv;
    DevBuf<int> ci, cj, ck;
    DevBuf<double> par, rates, rho, E, dipole, dPdt;
    DevBuf<int> win;
    DevBuf<double> wk;
    std::vector<std::pair<long long, double>> pts;   // (cell key, wk) in write order
    std::vector<int> pts_owner;                       // emitter index per point
    // learned closure deployed on this group (omx_qgroup_attach_closure)
    omx_closure *cl = nullptr;
    omx::ClDeploy dep{};
    DevBuf<float> cwin, hst, cG, cY;
    DevBuf<uint16_t> xh, chb, ca1, ca2, ca3;
    DevBuf<int> sub, sub_of;
    DevBuf<double> sub_rho;
    DevBuf<unsigned char> cl_state;
};

struct omx_ctx {
    omx_grid_desc desc{};
    int dims = 3;
    int n[3] = {1, 1, 1};
    bool fp32 = false;
    cudaStream_t stream = nullptr;
    Lay L{};
    size_t felems = 0;
    DevBuf<float> ff[6];
    DevBuf<double> fd[6];
    bool field_used[6] = {false, false, false, false, false, false};
    // host tables
    CpmlTables T;
    std::vector<double> den_e[3], den_h[3];
    bool cpml_axis[3] = {false, false, false};
    int per[3] = {0, 0, 0};
    // device tables (one of the two precisions used)
    DevBuf<float> tf[3][6];   // den_e, den_h, bE, cE, bH, cH per axis
    DevBuf<double> td[3][6];
    DevBuf<short> tl[3][2];   // lE, lH per axis
    DevBuf<float> psif[3][2][2];
    DevBuf<double> psid[3][2][2];
    int L2 = 0;
    // media
    int n_media = 0;
    std::vector<omx_medium> media;
    int bb0[3] = {1, 1, 1}, bb1[3] = {0, 0, 0};
    long long bbV = 0;
    DevBuf<uint8_t> mat[3];
    DevBuf<unsigned char> clsbuf, medbuf;
    DevBuf<float> adef;
    DevBuf<double> aded;
    int P = 1;
    bool has_ade = false;
    DevBuf<int4> ade_ent;   // dispersive component-cells (i, j, k, component)
    DevBuf<int> ade_b;      // their media-box index
    int ade_n = 0;
    std::vector<int4> ade_host;
    std::vector<uint8_t> host_mat[3];   // class per component over the box (for injection checks)
    std::vector<int> cls_type;          // per class id
    // sources
    std::vector<std::unique_ptr<SourceRec>> sources;
    // emitters and J points
    std::vector<std::unique_ptr<GroupRec>> groups;
    std::vector<long long> jkeys;                  // cell keys of J points (sorted)
    std::unordered_map<long long, int> jslot;
    DevBuf<double> jbuf;                           // 9 * np: J[3], Jo[3], dJ[3]
    DevBuf<long long> inj_e;
    DevBuf<int> inj_c, inj_a, inj_b;
    int inj_n = 0;
    std::vector<int4> inj_host;    // (i, j, k, component) of every emitter-current point
    bool j_dirty = false;
    // detectors
    struct Det {
        int type, field, nd;
        int first;              // first tap (sample point) of this detector
        std::vector<int> idx;   // indx_list, nd x dims (column-major, as passed)
    };
    std::vector<Det> dets;
    int print_det_step = 0;     // records written by omx_detectors_write_text (file numbering)
    // running Fourier transforms of the detector samples
    int n_freq = 0;
    double dft_w = 0.0;
    DevBuf<double> d_omega, dft_re, dft_im;
    DevBuf<double> energy_buf;
    std::vector<int> tap_field, tap_nt;
    std::vector<double> tap_w;
    std::vector<long long> tap[4];
    DevBuf<int> d_tap_field, d_tap_nt;
    DevBuf<double> d_tap_w;
    DevBuf<long long> d_tap[4];
    DevBuf<double> rec, rec_times;
    int rec_capacity = 0, rec_count = 0;
    bool det_dirty = false;
    // stepping state (mxim_mxll.f90:96-104)
    bool started = false;
    bool fields_written = false;   // omx_write_field was called (the fields may be non-zero)
    // launch shapes (omx_autotune): planes / rows per thread of the unfused kernels (0 = default)
    // and the fused-kernel form (-1 = default)
    int march = 0;
    int fused_form = -1;
    int march_two_pass = 0;   // autotune: the two-pass candidate of a 3D FP32 fused-eligible grid is selected
    int tq_step_old = 0;
    double t_skip = 0.0;
    // run tables
    DevBuf<double> tab;
    DevBuf<int> d_step;
    // overlapped schedule of the fused path (graphs only): a side stream runs step s's detector
    // sampling and emitter work while the main stream runs step s+1's fused pass; the side
    // stream's kernels read their step's scalars through their own counter
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // the fused 3D pass's general runs (latency-bound) run on f3aux beside the lean runs
    // (bandwidth-bound) of the same step; ev_f3a / ev_f3b fork and join them
    cudaStream_t f3aux = nullptr;
    cudaEvent_t ev_f3a = nullptr, ev_f3b = nullptr;
    DevBuf<int> d_step2;
    // a one-step omx_run leaves its side-stream work running (ev_join marks its end) so that the
    // next call's fused pass overlaps it; every other entry point first orders the main stream
    // after it (join_side)
    bool side_pending = false;
    // an asynchronous drain behind pending side work queues its copies on the side stream and
    // marks their end with ev_drain: the next one-step call orders its emitter current after the
    // side kernels only (ev_join), every other entry point after the copies as well
    cudaEvent_t ev_drain = nullptr;
    bool drain_pending = false;
    // the reference's per-call sequence on the fused FP32 TMz path: omx_step_H is deferred and
    // fused with the next omx_step_E (sources requested in between are added after the fused
    // pass, as omx_run does); any other entry point first runs the deferred work unfused
    bool h_pending = false, src_pending = false;
    double src_time = 0.0;
    // asynchronous detector drains: a ring of pinned slots, each filled by copies on the stream
    // and marked by an event; omx_detectors_collect hands a slot's records to the caller
    struct DrainSlot {
        double *h = nullptr;   // times then values
        size_t cap = 0;        // doubles
        int *err = nullptr;    // copy of the kernel error word taken with the records
        int n = 0;
        long long ticket = -1;  // -1: free
        cudaEvent_t ev = nullptr;
    } drain_slots[OMX_DRAIN_SLOTS];
    long long next_ticket = 0;
    DevBuf<float> rowc;    // packed per-row y coefficients of the fused FP32 TMz kernel
    DevBuf<int> d_err;     // kernel error word (bit 0: a bulk-copy wait of the fused kernel ran out)
    DevBuf<int> d_done;    // finished blocks of the fused 3D pass in the device loop (zero between launches)
    int *h_err = nullptr;  // pinned host copy of it, read at every synchronisation
    // pinned staging of the per-step table, two halves used alternately (an event per half
    // marks when its last copy has been consumed)
    struct HostStage {
        double *p = nullptr;
        size_t cap = 0;
        cudaEvent_t ev = nullptr;
    } tab_stage[2];
    int tab_flip = 0;
    // captured step graphs, valid while the configuration epoch is unchanged (kernel arguments
    // hold device pointers and sizes that any configuration call may replace)
    unsigned long long epoch = 1;
    struct GraphRec {
        unsigned long long epoch;
        int steps, cur, W, has_det, fused, cur_after;
        long long launches;
        cudaGraphExec_t exec;
    };
    std::vector<GraphRec> graphs;
    // profiling
    bool prof = false;
    struct Ev { int cls; cudaEvent_t a, b; };
    std::vector<Ev> evs;
    double prof_ms[KC_N] = {0, 0, 0, 0, 0};
    long long prof_n[KC_N] = {0, 0, 0, 0, 0};
    long long launches = 0;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    DevBuf<float> flushbuf;
    // FP32 fused 2D TMz step (ping-pong): second field / H-psi buffer set and the parity
    DevBuf<float> ff2[6];
    DevBuf<float> psiH2[3][2];
    int cur = 0;
    bool fused_ok = false;
    bool fused_dirty = true;    // media or sources changed since the last eligibility check
    bool post_ok = false;       // the work after the fused pass goes in one launch (post_eligible)
    bool plane_fold = false;    // the 3D bulk E pass adds the plane source (plane_fold_eligible)
    bool fold3 = false;         // the fused 3D pass adds the single plane source (fold3_of)
    F3tMaps f3maps[2][2];       // tensor maps of the fused 3D pass: [in set][tile rows 8 / 16]
    const void *f3key[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};   // Ex buffer they were made for
    // runs {bx, by, k0, k1} of the fused 3D pass (general runs first, then lean ones), one list per
    // tile rows / planes per block / plane-source setting (kept: the autotuner switches between
    // them without uploading again); f3cur is the list of the current shape
    struct F3Plan {
        DevBuf<int4> items;
        int n_gen = 0, n_lean = 0;
    };
    std::map<long long, std::unique_ptr<F3Plan>> f3plans;
    F3Plan *f3cur = nullptr;
    std::vector<short> hl[3][2];   // host copies of the CPML layer tables (lE, lH per axis)
    int step_form = OMX_STEP_DEFAULT;   // omx_set_step_form; a batch sets TWO_PASS on its members
    int *run_step = nullptr;    // device step counter while omx_run issues a step sequence
    std::string err;
};

namespace {

void join_side(omx_ctx *c);

int set_err(omx_ctx *ctx, const Fail &f)
{
    g_last_error = f.msg;
    if (ctx) ctx->err = f.msg;
    return f.code;
}

#define OMX_API_BEGIN try {
#define OMX_API_END(ctx)                                                                          \
    }                                                                                             \
    catch (const Fail &f) { return set_err(ctx, f); }                                             \
    catch (const std::exception &e) { return set_err(ctx, Fail{OMX_ERR_ARG, e.what()}); }         \
    return OMX_OK;

long long cell_key(const omx_ctx *c, int i, int j, int k)
{
    return (long long)i + (long long)(c->n[0] + 2) * ((long long)j + (long long)(c->n[1] + 2) * (long long)k);
}

long long eindex(const omx_ctx *c, int i, int j, int k)
{
    return c->L.off + i + (long long)c->L.px * j + c->L.pz * k;
}

// ---- profiling helpers ------------------------------------------------------------------------
struct ProfScope {
    omx_ctx *c;
    int cls;
    cudaEvent_t a = nullptr, b = nullptr;
    ProfScope(omx_ctx *ctx, int k) : c(ctx), cls(k)
    {
        if (c->prof) {
            cudaEventCreate(&a);
            cudaEventCreate(&b);
            cudaEventRecord(a, c->stream);
        }
    }
    ~ProfScope()
    {
        if (c->prof) {
            cudaEventRecord(b, c->stream);
            c->evs.push_back({cls, a, b});
        }
    }
};

void prof_collect(omx_ctx *c)
{
    if (c->evs.empty()) return;
    ck(cudaStreamSynchronize(c->stream), "sync");
    for (auto &e : c->evs) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e.a, e.b);
        c->prof_ms[e.cls] += ms;
        c->prof_n[e.cls] += 1;
        cudaEventDestroy(e.a);
        cudaEventDestroy(e.b);
    }
    c->evs.clear();
}

// ---- field bounds (reference arrays) -----------------------------------------------------------
bool bounds_of(const omx_ctx *c, int field, int lo[3], int hi[3])
{
    const int nx = c->n[0], ny = c->n[1], nz = c->n[2];
    for (int a = 0; a < 3; ++a) lo[a] = hi[a] = 0;
    if (c->dims == 3) {
        switch (field) {
        case OMX_EX_FIELD: lo[0] = 0; hi[0] = nx; lo[1] = 1; hi[1] = ny + 1; lo[2] = 1; hi[2] = nz + 1; return true;
        case OMX_EY_FIELD: lo[0] = 1; hi[0] = nx + 1; lo[1] = 0; hi[1] = ny; lo[2] = 1; hi[2] = nz + 1; return true;
        case OMX_EZ_FIELD: lo[0] = 1; hi[0] = nx + 1; lo[1] = 1; hi[1] = ny + 1; lo[2] = 0; hi[2] = nz; return true;
        case OMX_HX_FIELD: lo[0] = 1; hi[0] = nx; lo[1] = 0; hi[1] = ny; lo[2] = 0; hi[2] = nz; return true;
        case OMX_HY_FIELD: lo[0] = 0; hi[0] = nx; lo[1] = 1; hi[1] = ny; lo[2] = 0; hi[2] = nz; return true;
        case OMX_HZ_FIELD: lo[0] = 0; hi[0] = nx; lo[1] = 0; hi[1] = ny; lo[2] = 1; hi[2] = nz; return true;
        }
        return false;
    }
    if (c->dims == 2) {
        if (c->desc.mode == OMX_TMZ_2D_MODE) {
            switch (field) {
            case OMX_EZ_FIELD: lo[0] = 1; hi[0] = nx + 1; lo[1] = 1; hi[1] = ny + 1; return true;
            case OMX_HX_FIELD: lo[0] = 1; hi[0] = nx; lo[1] = 0; hi[1] = ny; return true;
            case OMX_HY_FIELD: lo[0] = 0; hi[0] = nx; lo[1] = 1; hi[1] = ny; return true;
            }
        } else {
            switch (field) {
            case OMX_EX_FIELD: lo[0] = 0; hi[0] = nx; lo[1] = 1; hi[1] = ny + 1; return true;
            case OMX_EY_FIELD: lo[0] = 1; hi[0] = nx + 1; lo[1] = 0; hi[1] = ny; return true;
            case OMX_HZ_FIELD: lo[0] = 0; hi[0] = nx; lo[1] = 0; hi[1] = ny; return true;
            }
        }
        return false;
    }
    switch (field) {
    case OMX_EX_FIELD: lo[0] = 1; hi[0] = nx; return true;
    case OMX_HY_FIELD: lo[0] = 1; hi[0] = nx - 1; return true;
    }
    return false;
}

// ---- device tables ------------------------------------------------------------------------------
template <class R> DevBuf<R> (&tables(omx_ctx *c))[3][6];
template <> DevBuf<float> (&tables<float>(omx_ctx *c))[3][6] { return c->tf; }
template <> DevBuf<double> (&tables<double>(omx_ctx *c))[3][6] { return c->td; }
template <class R> DevBuf<R> (&psis(omx_ctx *c))[3][2][2];
template <> DevBuf<float> (&psis<float>(omx_ctx *c))[3][2][2] { return c->psif; }
template <> DevBuf<double> (&psis<double>(omx_ctx *c))[3][2][2] { return c->psid; }
template <class R> DevBuf<R> (&fields(omx_ctx *c))[6];
template <> DevBuf<float> (&fields<float>(omx_ctx *c))[6] { return c->ff; }
template <> DevBuf<double> (&fields<double>(omx_ctx *c))[6] { return c->fd; }
template <class R> DevBuf<R> &adebuf(omx_ctx *c);
template <> DevBuf<float> &adebuf<float>(omx_ctx *c) { return c->adef; }
template <> DevBuf<double> &adebuf<double>(omx_ctx *c) { return c->aded; }

template <class R> void upload_axis_tables(omx_ctx *c)
{
    const bool exact = std::is_same<R, double>::value;
    const int npml = c->desc.npml;
    for (int a = 0; a < 3; ++a) {
        const int na = c->n[a];
        std::vector<R> de(na + 2), dh(na + 2), bE(na + 2, R(0)), cE(na + 2, R(0)), bH(na + 2, R(0)), cH(na + 2, R(0));
        std::vector<short> lE(na + 2, -1), lH(na + 2, -1);
        for (int p = 0; p < na + 2; ++p) {
            de[p] = (R)c->den_e[a][p];
            dh[p] = (R)c->den_h[a][p];
        }
        if (c->cpml_axis[a]) {
            const double dr = c->desc.dr;
            auto cf = [&](double v) { return exact ? (R)v : (R)(v / dr); };
            // E: low face i = 2..npml (be(i)), high face i = n+1-npml..n-1 (be(n+1-i))
            for (int p = 2; p <= npml; ++p) {
                lE[p] = (short)(p - 2);
                bE[p] = (R)c->T.be[p - 1];
                cE[p] = cf(c->T.ce[p - 1]);
            }
            for (int p = na + 1 - npml; p <= na - 1; ++p) {
                lE[p] = (short)((npml - 1) + (p - (na + 1 - npml)));
                bE[p] = (R)c->T.be[na + 1 - p - 1];
                cE[p] = cf(c->T.ce[na + 1 - p - 1]);
            }
            // H: low face i = 1..npml-1 (bh(i)), high face i = n+1-npml..n-1 (bh(n-i))
            for (int p = 1; p <= npml - 1; ++p) {
                lH[p] = (short)(p - 1);
                bH[p] = (R)c->T.bh[p - 1];
                cH[p] = cf(c->T.ch[p - 1]);
            }
            for (int p = na + 1 - npml; p <= na - 1; ++p) {
                lH[p] = (short)((npml - 1) + (p - (na + 1 - npml)));
                bH[p] = (R)c->T.bh[na - p - 1];
                cH[p] = cf(c->T.ch[na - p - 1]);
            }
        }
        auto &tb = tables<R>(c)[a];
        tb[0].upload(de);
        tb[1].upload(dh);
        tb[2].upload(bE);
        tb[3].upload(cE);
        tb[4].upload(bH);
        tb[5].upload(cH);
        c->tl[a][0].upload(lE);
        c->tl[a][1].upload(lH);
        c->hl[a][0] = lE;
        c->hl[a][1] = lH;
        if (!exact && a == 1) {
            // packed y coefficients of the fused FP32 TMz kernel: (den_h, den_e, bH, cH) and
            // (bE, cE, H layer, E layer) per row, the layers as int bit patterns
            std::vector<float> rc((size_t)8 * (na + 2));
            for (int p = 0; p < na + 2; ++p) {
                const int lh = lH[p], le = lE[p];
                float *o = &rc[(size_t)8 * p];
                o[0] = (float)dh[p];
                o[1] = (float)de[p];
                o[2] = (float)bH[p];
                o[3] = (float)cH[p];
                o[4] = (float)bE[p];
                o[5] = (float)cE[p];
                std::memcpy(&o[6], &lh, sizeof(int));
                std::memcpy(&o[7], &le, sizeof(int));
            }
            c->rowc.upload(rc);
        }
    }
}

template <class R> void alloc_psi(omx_ctx *c)
{
    const int npml = c->desc.npml;
    c->L2 = 2 * (npml - 1);
    auto &ps = psis<R>(c);
    for (int a = 0; a < 3; ++a)
        for (int f = 0; f < 2; ++f)
            for (int q = 0; q < 2; ++q) ps[a][f][q].release();
    for (int a = 0; a < c->dims; ++a) {
        if (!c->cpml_axis[a]) continue;
        long long tr = 1;
        for (int b = 0; b < c->dims; ++b)
            if (b != a) tr *= c->n[b];
        const long long cnt = (long long)c->L2 * tr;
        const int ncomp = (c->dims == 3) ? 2 : 1;
        for (int f = 0; f < 2; ++f)
            for (int q = 0; q < ncomp; ++q) ps[a][f][q].alloc((size_t)cnt);
    }
}

template <class R> FieldPtrs<R> field_ptrs(omx_ctx *c, int parity = -1)
{
    // the current buffer set (the FP32 fused path alternates between two sets)
    const int p = parity < 0 ? c->cur : parity;
    FieldPtrs<R> F;
    for (int q = 0; q < 6; ++q) F.f[q] = fields<R>(c)[q].p;
    if (p == 1 && std::is_same<R, float>::value)
        for (int q = 0; q < 6; ++q) F.f[q] = reinterpret_cast<R *>(c->ff2[q].p);
    return F;
}

template <class R> GridArgs<R> grid_args(omx_ctx *c)
{
    GridArgs<R> G;
    std::memset(&G, 0, sizeof(G));
    G.L = c->L;
    const omx::Consts &K = omx::consts();
    (void)K;
    const double dt_eps0 = c->desc.dt / omx::consts().eps0, dt_mu0 = c->desc.dt / omx::consts().mu0;
    G.dt_mu0 = (R)dt_mu0;
    G.dt_eps0 = (R)dt_eps0;
    G.dr = (R)c->desc.dr;
    for (int a = 0; a < 3; ++a) G.per[a] = c->per[a];
    G.npml = c->desc.npml;
    G.L2 = c->L2;
    auto &tb = tables<R>(c);
    auto &ps = psis<R>(c);
    for (int a = 0; a < 3; ++a) {
        G.den_e[a] = tb[a][0].p;
        G.den_h[a] = tb[a][1].p;
        G.bE[a] = tb[a][2].p;
        G.cE[a] = tb[a][3].p;
        G.bH[a] = tb[a][4].p;
        G.cH[a] = tb[a][5].p;
        G.lE[a] = c->tl[a][0].p;
        G.lH[a] = c->tl[a][1].p;
        for (int q = 0; q < 2; ++q) {
            G.psiE[a][q] = ps[a][0][q].p;
            G.psiH[a][q] = ps[a][1][q].p;
            if (c->cur == 1 && std::is_same<R, float>::value) G.psiH[a][q] = reinterpret_cast<R *>(c->psiH2[a][q].p);
        }
        G.bb0[a] = c->bb0[a];
        G.bb1[a] = c->bb1[a];
        G.bbd[a] = std::max(0, c->bb1[a] - c->bb0[a] + 1);
        G.mat[a] = c->mat[a].p;
    }
    G.bbV = c->bbV;
    G.cls = reinterpret_cast<const ClsR<R> *>(c->clsbuf.p);
    G.med = reinterpret_cast<const MedR<R> *>(c->medbuf.p);
    G.ade = adebuf<R>(c).p;
    G.P = c->P;
    G.mode2d = c->desc.mode;
    G.ade_n = c->ade_n;
    G.ade_ent = c->ade_ent.p;
    G.ade_b = c->ade_b.p;
    G.step_inc = c->run_step;
    G.step_done = c->d_done.p;
    G.march = c->march;
    return G;
}

// ---- media ----------------------------------------------------------------------------------------
template <class R>
void build_media(omx_ctx *c, const int32_t *map, const double *eps[3])
{
    const int dims = c->dims;
    const int nx = c->n[0], ny = c->n[1], nz = c->n[2];
    const long long N = (long long)nx * ny * nz;
    const int comps = dims == 1 ? 1 : 3;
    const double dt_eps0 = c->desc.dt / omx::consts().eps0;
    auto mm = [&](long long cell, int comp) -> int32_t { return map ? map[cell + N * (comps == 1 ? 0 : comp)] : 0; };
    auto is_ade = [&](int32_t m) {
        return m > 0 && m <= c->n_media &&
               (c->media[m - 1].medium_type == OMX_DRUDE_MEDIUM || c->media[m - 1].medium_type == OMX_DL_MEDIUM);
    };
    // effective inverse permittivity of component `comp` at a cell (reference rule or arrays)
    auto eps_inv = [&](long long cell, int comp) -> double {
        if (eps[0] || eps[1] || eps[2]) {
            const double *e = eps[comp];
            return e ? e[cell] : 1.0;
        }
        int32_t m;
        if (dims == 3) m = mm(cell, comp);
        else if (dims == 2) m = mm(cell, 0);   // classical_medium_mod.f90:526-538 keys on component 1
        else m = mm(cell, 0);
        if (m > 0 && m <= c->n_media && c->media[m - 1].medium_type == OMX_DIELECTRIC_MEDIUM)
            return 1.0 / c->media[m - 1].eps_r;
        return 1.0;
    };
    const int act[3] = {dims == 3 || dims == 1 || (dims == 2 && c->desc.mode == OMX_TEZ_2D_MODE),
                        dims == 3 || (dims == 2 && c->desc.mode == OMX_TEZ_2D_MODE),
                        dims == 3 || (dims == 2 && c->desc.mode == OMX_TMZ_2D_MODE)};
    // bounding box of non-vacuum component cells
    int b0[3] = {1 << 30, 1 << 30, 1 << 30}, b1[3] = {-1, -1, -1};
    const bool all_vacuum = !map && !eps[0] && !eps[1] && !eps[2];
    for (long long cell = 0; cell < (all_vacuum ? 0 : N); ++cell) {
        bool nv = false;
        for (int q = 0; q < 3 && !nv; ++q) {
            if (!act[q]) continue;
            if (dims == 1 && q > 0) break;
            const int32_t m = (dims == 1) ? mm(cell, 0) : mm(cell, q);
            if (is_ade(m) || eps_inv(cell, q) != 1.0) nv = true;
        }
        if (!nv) continue;
        const int i = 1 + (int)(cell % nx), j = 1 + (int)((cell / nx) % ny), k = 1 + (int)(cell / ((long long)nx * ny));
        const int ijk[3] = {i, j, k};
        for (int a = 0; a < 3; ++a) {
            b0[a] = std::min(b0[a], ijk[a]);
            b1[a] = std::max(b1[a], ijk[a]);
        }
    }
    if (b1[0] < 0) {
        for (int a = 0; a < 3; ++a) { b0[a] = 1; b1[a] = 0; }
    }
    for (int a = 0; a < 3; ++a) { c->bb0[a] = b0[a]; c->bb1[a] = b1[a]; }
    const int bd[3] = {std::max(0, b1[0] - b0[0] + 1), std::max(0, b1[1] - b0[1] + 1), std::max(0, b1[2] - b0[2] + 1)};
    c->bbV = (long long)bd[0] * bd[1] * bd[2];
    // classes
    std::map<std::tuple<int, int, double>, int> ids;
    std::vector<ClsR<R>> cls;
    cls.push_back(ClsR<R>{CLS_PLAIN, 0, (R)dt_eps0, (R)0});
    c->cls_type.assign(1, CLS_PLAIN);
    ids[std::make_tuple((int)CLS_PLAIN, 0, 1.0)] = 0;
    int maxP = 1;
    for (int m = 0; m < c->n_media; ++m)
        if (c->media[m].medium_type == OMX_DL_MEDIUM) maxP = std::max(maxP, c->media[m].n_poles);
    c->P = maxP;
    bool any_ade = false;
    for (int q = 0; q < 3; ++q) c->host_mat[q].assign((size_t)c->bbV, 0);
    for (int k = b0[2]; k <= b1[2]; ++k)
        for (int j = b0[1]; j <= b1[1]; ++j)
            for (int i = b0[0]; i <= b1[0]; ++i) {
                const long long cell = (i - 1) + (long long)nx * ((j - 1) + (long long)ny * (k - 1));
                const long long b = (i - b0[0]) + (long long)bd[0] * ((j - b0[1]) + (long long)bd[1] * (k - b0[2]));
                for (int q = 0; q < comps; ++q) {
                    if (!act[q]) continue;
                    const int32_t m = mm(cell, q);
                    std::tuple<int, int, double> key;
                    if (is_ade(m)) {
                        key = std::make_tuple(c->media[m - 1].medium_type == OMX_DRUDE_MEDIUM ? (int)CLS_DRUDE : (int)CLS_DL,
                                              (int)m, 0.0);
                        any_ade = true;
                    } else {
                        key = std::make_tuple((int)CLS_PLAIN, 0, eps_inv(cell, q));
                    }
                    auto it = ids.find(key);
                    int id;
                    if (it == ids.end()) {
                        id = (int)cls.size();
                        req(id < 255, "more than 254 distinct material classes");
                        ids[key] = id;
                        ClsR<R> cr{};
                        cr.type = std::get<0>(key);
                        cr.medium = std::get<1>(key) > 0 ? std::get<1>(key) - 1 : 0;
                        cr.coef = (R)(dt_eps0 * std::get<2>(key));
                        cls.push_back(cr);
                        c->cls_type.push_back(cr.type);
                    } else {
                        id = it->second;
                    }
                    c->host_mat[q][(size_t)b] = (uint8_t)id;
                }
            }
    for (int q = 0; q < 3; ++q) {
        if (c->bbV > 0 && act[q]) {
            c->mat[q].alloc((size_t)c->bbV, false);
            h2d(c->mat[q].p, c->host_mat[q].data(), (size_t)c->bbV, "mat");
        } else {
            c->mat[q].release();
        }
    }
    std::vector<unsigned char> cb(cls.size() * sizeof(ClsR<R>));
    std::memcpy(cb.data(), cls.data(), cb.size());
    c->clsbuf.upload(cb);
    std::vector<MedR<R>> med((size_t)std::max(1, c->n_media));
    for (int m = 0; m < c->n_media; ++m) {
        const omx_medium &s = c->media[m];
        MedR<R> &d = med[(size_t)m];
        std::memset(&d, 0, sizeof(d));
        d.A1 = (R)s.A1; d.A2 = (R)s.A2; d.C1 = (R)s.C1; d.C2 = (R)s.C2; d.C3 = (R)s.C3; d.C4 = (R)s.C4;
        d.np = s.medium_type == OMX_DL_MEDIUM ? s.n_poles : 0;
        for (int p = 0; p < d.np; ++p) {
            d.al[p] = (R)s.alpha_k[p]; d.be[p] = (R)s.beta_k[p]; d.ga[p] = (R)s.gamma_k[p];
            d.B1[p] = (R)s.B1_k[p]; d.B2[p] = (R)s.B2_k[p];
        }
    }
    std::vector<unsigned char> mb(med.size() * sizeof(MedR<R>));
    std::memcpy(mb.data(), med.data(), mb.size());
    c->medbuf.upload(mb);
    c->has_ade = any_ade;
    if (any_ade) adebuf<R>(c).alloc((size_t)(3LL * (2 + 2 * c->P) * c->bbV));
    else adebuf<R>(c).release();
    // compact list of dispersive component-cells inside the E-update range
    std::vector<int4> ent;
    std::vector<int> eb;
    if (any_ade) {
        for (int k = b0[2]; k <= b1[2]; ++k)
            for (int j = b0[1]; j <= b1[1]; ++j)
                for (int i = b0[0]; i <= b1[0]; ++i) {
                    if (dims == 1 && (i < 2 || i > nx - 1)) continue;   // mxll_1D_mod.f90:320
                    const long long b = (i - b0[0]) + (long long)bd[0] * ((j - b0[1]) + (long long)bd[1] * (k - b0[2]));
                    for (int q = 0; q < comps; ++q) {
                        if (!act[q]) continue;
                        if (c->cls_type[c->host_mat[q][(size_t)b]] == CLS_PLAIN) continue;
                        ent.push_back(make_int4(i, dims >= 2 ? j : 0, dims == 3 ? k : 0, q));
                        eb.push_back((int)b);
                    }
                }
    }
    c->ade_n = (int)ent.size();
    c->ade_host = ent;
    c->ade_ent.upload(ent);
    c->ade_b.upload(eb);
}

int comp_axis_active(const omx_ctx *c, int q)
{
    if (c->dims == 3) return 1;
    if (c->dims == 1) return q == 0;
    return c->desc.mode == OMX_TMZ_2D_MODE ? q == 2 : q < 2;
}

// Injection list for the emitter current term of the E update.
void rebuild_injection(omx_ctx *c)
{
    const int np = (int)c->jkeys.size();
    const int avg = (c->dims == 3 || (c->dims == 2 && c->desc.mode == OMX_TEZ_2D_MODE)) ? 1 : 0;
    struct Ent { long long e; int comp, a, b; int4 cell; };
    std::map<std::pair<int, long long>, Ent> ents;
    const int nxx = c->n[0] + 2, nyy = c->n[1] + 2;
    for (int p = 0; p < np; ++p) {
        const long long key = c->jkeys[p];
        const int i = (int)(key % nxx), j = (int)((key / nxx) % nyy), k = (int)(key / ((long long)nxx * nyy));
        for (int q = 0; q < 3; ++q) {
            if (!comp_axis_active(c, q)) continue;
            int cand[2][3] = {{i, j, k}, {i, j, k}};
            int ncand = 1;
            if (avg) {
                cand[1][q] -= 1;   // E cell whose i+1 neighbour is this J point
                ncand = 2;
            }
            for (int t = 0; t < ncand; ++t) {
                const int ci = cand[t][0], cj = cand[t][1], cz = cand[t][2];
                // E update ranges: 3D/2D i,j,k in 1..n; 1D i in 2..n-1
                if (c->dims == 1) {
                    if (ci < 2 || ci > c->n[0] - 1) continue;
                } else {
                    if (ci < 1 || ci > c->n[0] || cj < 1 || cj > c->n[1]) continue;
                    if (c->dims == 3 && (cz < 1 || cz > c->n[2])) continue;
                }
                // skip dispersive components (the reference ignores J there); the media box
                // carries j == k == 1 on the axes a 1D/2D grid does not have
                const int bj = c->dims >= 2 ? cj : 1, bk = c->dims == 3 ? cz : 1;
                if (ci >= c->bb0[0] && ci <= c->bb1[0] && bj >= c->bb0[1] && bj <= c->bb1[1] &&
                    bk >= c->bb0[2] && bk <= c->bb1[2] && c->bbV > 0) {
                    const int bd0 = c->bb1[0] - c->bb0[0] + 1, bd1 = c->bb1[1] - c->bb0[1] + 1;
                    const long long b = (ci - c->bb0[0]) + (long long)bd0 * ((bj - c->bb0[1]) + (long long)bd1 * (bk - c->bb0[2]));
                    if (!c->host_mat[q].empty() && c->cls_type[c->host_mat[q][(size_t)b]] != CLS_PLAIN) continue;
                }
                const long long ck_ = cell_key(c, ci, cj, cz);
                auto kk = std::make_pair(q, ck_);
                if (ents.count(kk)) continue;
                Ent en;
                en.e = eindex(c, ci, cj, cz);
                en.comp = q;
                en.cell = make_int4(ci, cj, cz, q);
                auto fa = c->jslot.find(ck_);
                en.a = fa == c->jslot.end() ? -1 : fa->second;
                en.b = -1;
                if (avg) {
                    int nb[3] = {ci, cj, cz};
                    nb[q] += 1;
                    auto fb = c->jslot.find(cell_key(c, nb[0], nb[1], nb[2]));
                    en.b = fb == c->jslot.end() ? -1 : fb->second;
                }
                ents[kk] = en;
            }
        }
    }
    std::vector<long long> e;
    std::vector<int> comp, a, b;
    c->inj_host.clear();
    for (auto &kv : ents) {
        c->inj_host.push_back(kv.second.cell);
        e.push_back(kv.second.e);
        comp.push_back(kv.second.comp);
        a.push_back(kv.second.a);
        b.push_back(kv.second.b);
    }
    c->inj_n = (int)e.size();
    c->inj_e.upload(e);
    c->inj_c.upload(comp);
    c->inj_a.upload(a);
    c->inj_b.upload(b);
}

void rebuild_jpoints(omx_ctx *c)
{
    std::vector<long long> keys;
    for (auto &g : c->groups)
        for (auto &pt : g->pts) keys.push_back(pt.first);
    std::sort(keys.begin(), keys.end());
    keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
    c->jkeys = keys;
    c->jslot.clear();
    for (size_t p = 0; p < keys.size(); ++p) c->jslot[keys[p]] = (int)p;
    const int np = (int)keys.size();
    c->jbuf.alloc((size_t)9 * std::max(np, 1));
    for (auto &g : c->groups) {
        std::vector<int> win((size_t)std::max(np, 1), -1);
        std::vector<double> wk((size_t)std::max(np, 1), 0.0);
        for (size_t t = 0; t < g->pts.size(); ++t) {   // assignment: the last writer wins
            const int s = c->jslot[g->pts[t].first];
            win[(size_t)s] = g->pts_owner[t];
            wk[(size_t)s] = g->pts[t].second;
        }
        g->win.upload(win);
        g->wk.upload(wk);
    }
    rebuild_injection(c);
    c->j_dirty = false;
}

JState jstate(omx_ctx *c)
{
    JState J;
    J.np = (int)c->jkeys.size();
    const size_t np = (size_t)std::max(J.np, 1);
    for (int q = 0; q < 3; ++q) {
        J.J[q] = c->jbuf.p + np * q;
        J.Jo[q] = c->jbuf.p + np * (3 + q);
        J.dJ[q] = c->jbuf.p + np * (6 + q);
    }
    return J;
}

void rebuild_detectors(omx_ctx *c)
{
    c->d_tap_field.upload(c->tap_field);
    c->d_tap_nt.upload(c->tap_nt);
    c->d_tap_w.upload(c->tap_w);
    for (int t = 0; t < 4; ++t) c->d_tap[t].upload(c->tap[t]);
    c->det_dirty = false;
}

void ensure_rec_capacity(omx_ctx *c, int need)
{
    const int npts = (int)c->tap_field.size();
    if (need <= c->rec_capacity) return;
    join_side(c);   // records of a pending side sequence are copied below
    c->epoch++;
    int cap = std::max(need, c->rec_capacity * 2);
    DevBuf<double> nrec, ntim;
    nrec.alloc((size_t)cap * std::max(npts, 1));
    ntim.alloc((size_t)cap);
    if (c->rec_count > 0 && c->rec.p) {
        ck(cudaMemcpyAsync(nrec.p, c->rec.p, sizeof(double) * (size_t)c->rec_count * std::max(npts, 1),
                           cudaMemcpyDeviceToDevice, c->stream), "rec copy");
        ck(cudaMemcpyAsync(ntim.p, c->rec_times.p, sizeof(double) * (size_t)c->rec_count, cudaMemcpyDeviceToDevice,
                           c->stream), "rec copy");
        ck(cudaStreamSynchronize(c->stream), "sync");
    }
    std::swap(c->rec.p, nrec.p);
    std::swap(c->rec.n, nrec.n);
    std::swap(c->rec_times.p, ntim.p);
    std::swap(c->rec_times.n, ntim.n);
    c->rec_capacity = cap;
}

DetArgs det_args(omx_ctx *c)
{
    DetArgs D;
    D.n = (int)c->tap_field.size();
    D.field = c->d_tap_field.p;
    D.nt = c->d_tap_nt.p;
    D.w = c->d_tap_w.p;
    D.t0 = c->d_tap[0].p;
    D.t1 = c->d_tap[1].p;
    D.t2 = c->d_tap[2].p;
    D.t3 = c->d_tap[3].p;
    D.rec = c->rec.p;
    D.times = c->rec_times.p;
    D.n_freq = c->n_freq;
    D.omega = c->d_omega.p;
    D.dft_re = c->dft_re.p;
    D.dft_im = c->dft_im.p;
    D.dft_w = c->dft_w;
    return D;
}

// The FP32 fused TMz pass (k_fused_tmz_*) applies the dispersive cells, the sources and the
// emitter current after the bulk update; that commutes with the reference's order only with no
// dispersive cell in a CPML slab (its psi term would be lost) and no source point in a
// dispersive cell.  The 3D pass (k_fused3_tma) updates the dispersive cells inside the pass,
// before their CPML terms, as the reference does, and adds a single plane source to E_old before
// the update (fold3); other sources follow the pass and must avoid dispersive cells.  x and y
// must not be periodic (its staged halo holds the PEC ghosts there).
bool fold3_of(const omx_ctx *c)
{
    return c->dims == 3 && c->sources.size() == 1 && c->sources[0]->kind == 1;
}

bool fused_eligible(const omx_ctx *c)
{
    if (!c->fp32 || c->step_form == OMX_STEP_TWO_PASS) return false;
    if (c->dims == 2) {
        if (c->desc.mode != OMX_TMZ_2D_MODE || c->n[0] % 4 != 0) return false;
        const int npml = c->desc.npml;
        for (const int4 &e : c->ade_host) {
            for (int a = 0; a < c->dims; ++a) {
                const int p = a == 0 ? e.x : (a == 1 ? e.y : e.z);
                if (c->cpml_axis[a] && (p <= npml || p >= c->n[a] + 1 - npml)) return false;
            }
        }
    } else if (c->dims == 3) {
        if (c->per[0] || c->per[1]) return false;
    } else {
        return false;
    }
    if (!c->ade_host.empty() && !fold3_of(c)) {
        const bool d3 = c->dims == 3;
        std::unordered_map<long long, int> disp;
        for (const int4 &e : c->ade_host) disp[cell_key(c, e.x, e.y, d3 ? e.z : 0) * 4 + e.w] = 1;
        for (const auto &S : c->sources) {
            if (S->kind == 0) {
                for (const int4 &p : S->cells)
                    if (disp.count(cell_key(c, p.x, p.y, d3 ? p.z : 0) * 4 + p.w)) return false;
            } else {
                for (const int4 &e : c->ade_host) {
                    const int at = S->pd.plane_axis == 1 ? e.x : (S->pd.plane_axis == 2 ? e.y : e.z);
                    if (e.w == S->pd.comp - 1 && at == S->pd.plane_index) return false;
                }
            }
        }
    }
    return true;
}

// The dispersive cells, the sources and the emitter current after a fused pass can share one
// launch when they write disjoint E words: at most one source, a plane (the plane holds no
// dispersive cell on the fused path, and the emitter current skips dispersive cells), and no
// emitter-current point on the plane.
bool post_eligible(const omx_ctx *c)
{
    if (!c->fused_ok || c->sources.size() > 1) return false;
    if (c->sources.empty() || fold3_of(c)) return true;
    const SourceRec &S = *c->sources[0];
    if (S.kind != 1) return false;
    const int ax = S.pd.plane_axis - 1, comp = S.pd.comp - 1;
    for (const int4 &p : c->inj_host) {
        const int at = ax == 0 ? p.x : (ax == 1 ? p.y : p.z);
        if (p.w == comp && at == S.pd.plane_index) return false;
    }
    return true;
}

// The two-pass 3D step can add its single plane source inside the bulk E pass (to E_old, before
// the update, as the separate launch before the pass does) when no dispersive component-cell lies
// on the plane: those are updated before the bulk pass from the E that already holds the source.
bool plane_fold_eligible(const omx_ctx *c)
{
    if (c->dims != 3 || c->fused_ok || c->sources.size() != 1 || c->sources[0]->kind != 1) return false;
    const SourceRec &S = *c->sources[0];
    for (const int4 &e : c->ade_host) {
        const int at = S.pd.plane_axis == 1 ? e.x : (S.pd.plane_axis == 2 ? e.y : e.z);
        if (e.w == S.pd.comp - 1 && at == S.pd.plane_index) return false;
    }
    return true;
}

void f3t_plan(omx_ctx *c);

void prepare(omx_ctx *c)
{
    const bool recheck = c->j_dirty || c->fused_dirty;
    if (c->j_dirty || c->det_dirty || c->fused_dirty) c->epoch++;
    if (c->j_dirty) rebuild_jpoints(c);
    if (c->det_dirty) rebuild_detectors(c);
    c->started = true;
    if (c->fused_dirty) {
        c->fused_ok = fused_eligible(c);
        c->fused_dirty = false;
    }
    if (recheck) {
        c->post_ok = post_eligible(c);
        c->plane_fold = plane_fold_eligible(c);
        c->fold3 = c->fused_ok && fold3_of(c);
    }
    if (c->fused_ok && c->fp32 && c->dims == 3) f3t_plan(c);
    if (c->fused_ok && !c->ff2[2].p) {
        for (int q = 0; q < 6; ++q)
            if (c->field_used[q]) c->ff2[q].alloc(c->felems);
        for (int a = 0; a < 3; ++a)
            for (int q = 0; q < 2; ++q)
                if (c->psif[a][1][q].p) c->psiH2[a][q].alloc(c->psif[a][1][q].n);
        c->epoch++;
    }
}

StepParam imm(double v) { return StepParam{v, nullptr, nullptr, 0}; }

// ---- launch sequences (templated on the field precision) --------------------------------------
template <class R> void do_H(omx_ctx *c)
{
    ProfScope ps(c, KC_H);
    launch_h<R>(field_ptrs<R>(c), grid_args<R>(c), c->stream);
    c->launches++;
}

SrcArgs src_args(const SourceRec &S)
{
    SrcArgs a;
    a.n = S.n;
    a.eidx = S.eidx.p;
    a.ka = S.ka.p;
    a.kb = S.kb.p;
    a.comp = S.comp;
    a.avg = S.avg;
    a.c_src = S.c_src;
    return a;
}

template <class R> void launch_one_source(omx_ctx *c, size_t s, StepParam amp)
{
    const FieldPtrs<R> F = field_ptrs<R>(c);
    SourceRec &S = *c->sources[s];
    if (S.kind == 0) {
        launch_src<R>(F, src_args(S), amp, c->stream);
    } else {
        PlaneArgs p;
        p.comp = S.pd.comp - 1;
        p.axis = S.pd.plane_axis - 1;
        p.index = S.pd.plane_index;
        p.c_src = S.c_src;
        launch_plane<R>(F, c->L, p, amp, c->stream);
    }
    c->launches++;
}

template <class R> void do_sources(omx_ctx *c, const std::vector<StepParam> &amps)
{
    ProfScope ps(c, KC_SRC);
    for (size_t s = 0; s < c->sources.size(); ++s) launch_one_source<R>(c, s, amps[s]);
}

template <class R> void do_inject(omx_ctx *c, StepParam time, StepParam t_skip);

// plane: the amplitude of the context's single plane source when the 3D bulk E pass adds it
// (plane_fold holds), in place of a k_plane launch before the pass; nullptr otherwise
template <class R> void do_E(omx_ctx *c, StepParam time, StepParam t_skip, const StepParam *plane = nullptr)
{
    {
        ProfScope ps(c, KC_E);
        GridArgs<R> G = grid_args<R>(c);
        if (plane) {
            const SourceRec &S = *c->sources[0];
            G.pl_on = 1;
            G.pl_comp = S.pd.comp - 1;
            G.pl_axis = S.pd.plane_axis - 1;
            G.pl_index = S.pd.plane_index;
            G.pl_c_src = S.c_src;
            G.pl_amp = *plane;
        }
        launch_e<R>(field_ptrs<R>(c), G, c->stream);
        c->launches += 1 + (c->ade_n > 0 ? 1 : 0);
    }
    do_inject<R>(c, time, t_skip);
}

template <class R> void do_inject(omx_ctx *c, StepParam time, StepParam t_skip)
{
    if (c->inj_n > 0) {
        InjArgs I;
        I.n = c->inj_n;
        I.eidx = c->inj_e.p;
        I.comp = c->inj_c.p;
        I.sa = c->inj_a.p;
        I.sb = c->inj_b.p;
        I.avg = (c->dims == 3 || (c->dims == 2 && c->desc.mode == OMX_TEZ_2D_MODE)) ? 1 : 0;
        ProfScope ps(c, KC_EMIT);
        launch_inject<R>(field_ptrs<R>(c), jstate(c), I, time, t_skip, c->desc.dt / omx::consts().eps0, c->stream);
        c->launches++;
    }
}

template <class R> void do_group(omx_ctx *c, GroupRec &g, StepParam move)
{
    ProfScope ps(c, KC_EMIT);
    EmitArgs A;
    A.n = g.d.n_systems;
    A.model = g.d.model;
    A.npar = g.npar;
    A.nst = g.nst;
    A.dims = c->dims;
    A.mode2d = c->desc.mode;
    A.ci = g.ci.p;
    A.cj = g.cj.p;
    A.ck = g.ck.p;
    A.par = g.par.p;
    A.rates = g.rates.p;
    A.rho = g.rho.p;
    A.E = g.E.p;
    A.dipole = g.dipole.p;
    A.dPdt = g.dPdt.p;
    A.dt = g.d.dt;
    A.h2 = 0.5 * g.d.dt;
    A.h6 = g.d.dt / 6.0;
    A.inv_dt = c->fp32 ? 1.0 / g.d.dt : 0.0;
    A.only_if = nullptr;
    if (g.cl) {
        // network step, spot-check subset, check / fallback; the plain propagator below runs only
        // once the fallback flag is set
        launch_cl_gather<R>(field_ptrs<R>(c), c->L, A, g.dep, move, c->stream);
        std::string err;
        if (!closure_infer(g.cl, g.dep, A, c->stream, err)) throw Fail{OMX_ERR_CUDA, err};
        launch_cl_subset_check_reseed(A, g.dep, c->stream);
        c->launches += 1 + 9 + (g.dep.n_sub > 0 ? 1 : 0) + 2;
        A.only_if = &g.dep.st->plain_now;    // not on the step the fallback happens
    }
    launch_emit<R>(field_ptrs<R>(c), c->L, A, move, c->stream);
    ScatArgs S;
    S.np = (int)c->jkeys.size();
    if (c->dims == 3) { S.c0 = 0; S.c1 = 2; }
    else if (c->dims == 1) { S.c0 = 0; S.c1 = 0; }
    else if (c->desc.mode == OMX_TMZ_2D_MODE) { S.c0 = 2; S.c1 = 2; }
    else { S.c0 = 0; S.c1 = 1; }
    S.win = g.win.p;
    S.wk = g.wk.p;
    S.dPdt = g.dPdt.p;
    S.dt = g.d.dt;
    S.inv_dt = c->fp32 ? 1.0 / g.d.dt : 0.0;
    launch_scatter(jstate(c), S, move, c->stream);
    c->launches += 2;
}

template <class R> void do_sample(omx_ctx *c, StepParam slot, StepParam time)
{
    ProfScope ps(c, KC_DET);
    launch_sample<R>(field_ptrs<R>(c), det_args(c), slot, time, c->stream);
    c->launches++;
}

// The runs of the fused 3D pass.  Lean tiles (32 x ty columns, i0 = 1 mod 32) cover the columns
// and rows away from the x / y CPML slabs (own and halo cells);
// each of them is split along k where the plane form changes (the device's test, restated: a z
// slab at the plane, a media-box cell of the tile's part of the plane, the folded plane source)
// into lean and general runs of at most kch / F3T_GEN_KCH planes.  The columns and rows left at
// the edges (the slabs and what the alignment leaves beside them) are general on every plane, in
// pieces of at most 32 x ty columns.  General runs come first in the list; a general run packs
// its width and height as {i0 | w << 20, j0 | h << 20, k0, k1}, a lean run is {i0, j0, k0, k1}.
void f3t_runs(const omx_ctx *c, int ty, int kch, std::vector<int4> &gen, std::vector<int4> &lean)
{
    const bool pl = c->fold3 && !c->sources.empty();
    const int nx = c->n[0], ny = c->n[1], nz = c->n[2];
    int pl_axis = -1, pl_index = -1;
    if (pl) {
        const SourceRec &S = *c->sources[0];
        pl_axis = S.pd.plane_axis - 1;
        pl_index = S.pd.plane_index;
    }
    auto slab = [&](int a, int p) { return c->hl[a][0][p] >= 0 || c->hl[a][1][p] >= 0; };
    // clear(a, p0, p1): no slab of axis a at cells p0..p1 (clipped to the grid)
    auto clear = [&](int a, int p0, int p1) {
        for (int p = std::max(1, p0); p <= std::min(c->n[a], p1); ++p)
            if (slab(a, p)) return false;
        return true;
    };
    // lean tile origins along one axis: width w, origins = 1 mod align, own and halo cells clear
    auto lean_origins = [&](int a, int w, int align) {
        std::vector<int> o;
        int p = 1;
        while (p <= c->n[a]) {
            if ((p - 1) % align == 0 && clear(a, p - 1, p + w - 1)) {
                o.push_back(p);
                p += w;
            } else {
                ++p;
            }
        }
        return o;
    };
    // x origins at 1 mod 32: the new fields' rows then go out in whole 128-byte lines (a tile
    // shifted off them writes partial 32-byte sectors, which measured 30 % slower at 512^3)
    const std::vector<int> ox = lean_origins(0, 32, 32), oy = lean_origins(1, ty, 1);
    // the other cells of an axis as pieces of at most w: [start, length]
    auto rest = [&](const std::vector<int> &o, int n, int w) {
        std::vector<std::pair<int, int>> r;
        int p = 1;
        size_t t = 0;
        while (p <= n) {
            if (t < o.size() && o[t] == p) {
                p += w;
                ++t;
                continue;
            }
            const int end = t < o.size() ? o[t] - 1 : n;
            for (int q = p; q <= end; q += w) r.push_back({q, std::min(w, end - q + 1)});
            p = end + 1;
        }
        return r;
    };
    const auto rx = rest(ox, nx, 32), ry = rest(oy, ny, ty);
    const bool box = c->bb1[0] >= c->bb0[0] && c->bb1[1] >= c->bb0[1] && c->bb1[2] >= c->bb0[2];
    const int gk = std::min(kch, F3T_GEN_KCH);
    // planes of the media box in a grid with dispersive cells: general runs of at most
    // F3T_MEDIA_KCH planes there (a dispersive cell's ADE waits on its pole state plane by plane,
    // so shorter marches put more threads on the few columns that hold them)
    const bool disp = box && c->ade_n > 0;
    auto media_k = [&](int k) { return disp && k >= c->bb0[2] && k <= c->bb1[2]; };
    const int mkch = std::min(gk, F3T_MEDIA_KCH);
    auto general_column = [&](int i0, int w, int j0, int h) {
        const bool mxy = disp && c->bb0[0] <= i0 + w - 1 && c->bb1[0] >= i0 && c->bb0[1] <= j0 + h - 1 && c->bb1[1] >= j0;
        for (int k = 1; k <= nz;) {
            const bool m = mxy && media_k(k);
            int e = k;
            while (e < nz && e - k + 1 < (m ? mkch : gk) && (mxy && media_k(e + 1)) == m) ++e;
            gen.push_back(make_int4(i0 | (w << 20), j0 | (h << 20), k, e));
            k = e + 1;
        }
    };
    std::vector<char> lk(nz + 1);
    for (int j0 : oy)
        for (int i0 : ox) {
            const int h = std::min(ty, ny - j0 + 1), w = std::min(32, nx - i0 + 1);
            const bool mb = box && c->bb0[0] <= i0 + 31 && c->bb1[0] >= i0 && c->bb0[1] <= j0 + ty - 1 &&
                            c->bb1[1] >= j0;
            const bool plxy = (pl_axis == 0 && pl_index >= i0 && pl_index <= i0 + 31) ||
                              (pl_axis == 1 && pl_index >= j0 && pl_index <= j0 + ty - 1);
            for (int k = 1; k <= nz; ++k)
                lk[k] = !plxy && !slab(2, k) && !(pl_axis == 2 && k == pl_index) &&
                        !(mb && k >= c->bb0[2] && k <= c->bb1[2]);
            for (int k = 1; k <= nz;) {
                // general runs in short pieces: their plain kernels march a thread per column,
                // so more pieces are more threads in flight
                const bool m = !lk[k] && mb && media_k(k);
                const int cap = lk[k] ? kch : (m ? mkch : gk);
                int e = k;
                while (e < nz && lk[e + 1] == lk[k] && e - k + 1 < cap && (!lk[k] && mb && media_k(e + 1)) == m) ++e;
                if (lk[k]) lean.push_back(make_int4(i0, j0, k, e));
                else gen.push_back(make_int4(i0 | (w << 20), j0 | (h << 20), k, e));
                k = e + 1;
            }
        }
    // the edges: every (x piece, y piece) pair with at least one piece outside the lean tiles
    std::vector<std::pair<int, int>> px, py;
    for (int i0 : ox) px.push_back({i0, std::min(32, nx - i0 + 1)});
    for (int j0 : oy) py.push_back({j0, std::min(ty, ny - j0 + 1)});
    for (const auto &x : rx)
        for (const auto &y : py) general_column(x.first, x.second, y.first, y.second);
    for (const auto &y : ry) {
        for (const auto &x : px) general_column(x.first, x.second, y.first, y.second);
        for (const auto &x : rx) general_column(x.first, x.second, y.first, y.second);
    }
}

// The run list of the current launch shape, uploaded once per shape (f3cur).
void f3t_plan(omx_ctx *c)
{
    const int ty = f3t_rows(c->fused_form);
    const int kch = c->march > 0 ? std::min(c->march, F3T_KMAX) : 64;
    const bool pl = c->fold3 && !c->sources.empty();
    const long long key = ((long long)ty * 1000 + kch) * 2 + (pl ? 1 : 0);
    auto hit = c->f3plans.find(key);
    if (hit != c->f3plans.end()) {
        c->f3cur = hit->second.get();
        return;
    }
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    ck(cudaStreamIsCapturing(c->stream, &cs), "capture status");
    if (cs != cudaStreamCaptureStatusNone)
        throw Fail{OMX_ERR_STATE, "fused 3D pass: its run list changed during a stream capture"};
    std::vector<int4> gen, lean;
    f3t_runs(c, ty, kch, gen, lean);
    std::vector<int4> all(gen);
    all.insert(all.end(), lean.begin(), lean.end());
    std::unique_ptr<omx_ctx::F3Plan> P(new omx_ctx::F3Plan);
    P->items.upload(all);
    P->n_gen = (int)gen.size();
    P->n_lean = (int)lean.size();
    c->f3cur = P.get();
    c->f3plans[key] = std::move(P);
}

// One FP32 fused step: the H+E pass from the current buffer set into the other.  2D TMz: then
// the dispersive cells (ade); 3D: the dispersive cells are inside the pass, and so is the single
// plane source when fold3 holds (`plane`: its amplitude).  The caller adds the other sources and
// the emitter current to the new set.
template <class R> void fused_step(omx_ctx *c, bool ade = true, const StepParam *plane = nullptr);
template <> void fused_step<double>(omx_ctx *, bool, const StepParam *) {}
template <> void fused_step<float>(omx_ctx *c, bool ade, const StepParam *plane)
{
    ProfScope ps(c, KC_E);
    const int in = c->cur, out = 1 - c->cur;
    const FieldPtrs<float> Fin = field_ptrs<float>(c, in), Fout = field_ptrs<float>(c, out);
    GridArgs<float> G = grid_args<float>(c);
    if (c->dims == 3) {
        Fused3Args A;
        A.in = Fin;
        A.out = Fout;
        for (int a = 0; a < 3; ++a)
            for (int q = 0; q < 2; ++q) A.psiH_out[a][q] = in == 0 ? c->psiH2[a][q].p : c->psif[a][1][q].p;
        if (c->fold3 && plane) {
            const SourceRec &S = *c->sources[0];
            G.pl_on = 1;
            G.pl_comp = S.pd.comp - 1;
            G.pl_axis = S.pd.plane_axis - 1;
            G.pl_index = S.pd.plane_index;
            G.pl_c_src = S.c_src;
            G.pl_amp = *plane;
            // in the device loop this pass advances the step counter when it ends, so it reads
            // its step's row while the counter still holds the previous step
            if (G.pl_amp.tab && G.step_inc) G.pl_amp.tab += G.pl_amp.stride;
        }
        if (G.step_inc && !c->d_done.p) throw Fail{OMX_ERR_STATE, "fused 3D pass: block counter missing"};
        const int ty = f3t_rows(c->fused_form);
        const int t = ty == 16 ? 1 : 0;
        if (c->f3key[in][t] != Fin.f[0]) {
            if (!encode_f3t_maps(&c->f3maps[in][t], Fin, c->L, ty))
                throw Fail{OMX_ERR_CUDA, "cuTensorMapEncodeTiled failed for the fused 3D pass"};
            c->f3key[in][t] = Fin.f[0];
        }
        f3t_plan(c);
        const int4 *items = c->f3cur->items.p;
        // general runs (CPML, media, plane source): new H on f3aux beside the lean runs' fused
        // launch on the stream, then new E on the stream once both have written their new H; the E
        // launch (the pass's only reader of the step's scalars) advances the device-loop step
        // counter, or the lean launch when there are no general runs
        const int ng = c->f3cur->n_gen, nl = c->f3cur->n_lean;
        GridArgs<float> Gq = G;
        Gq.step_inc = nullptr;
        Gq.step_done = nullptr;
        if (ng > 0) {
            ck(cudaEventRecord(c->ev_f3a, c->stream), "fork");
            ck(cudaStreamWaitEvent(c->f3aux, c->ev_f3a, 0), "fork");
            ck(launch_fused3t_general(A, Gq, c->fused_form, items, ng, false, c->f3aux), "fused 3D launch");
            ck(cudaEventRecord(c->ev_f3b, c->f3aux), "join");
        }
        ck(launch_fused3t_lean(c->f3maps[in][t], A, ng > 0 ? Gq : G, c->fused_form, items + ng, nl, c->d_err.p,
                               c->stream),
           "fused 3D launch");
        if (ng > 0) {
            ck(cudaStreamWaitEvent(c->stream, c->ev_f3b, 0), "join");
            ck(launch_fused3t_general(A, G, c->fused_form, items, ng, true, c->stream), "fused 3D launch");
        }
        c->launches += (ng > 0 ? 2 : 0) + (nl > 0 ? 1 : 0);
        c->cur = out;
        return;
    }
    Fused2Args A;
    A.ez_in = Fin.f[2];
    A.hx_in = Fin.f[3];
    A.hy_in = Fin.f[4];
    A.ez_out = Fout.f[2];
    A.hx_out = Fout.f[3];
    A.hy_out = Fout.f[4];
    A.psi_hyx_in = G.psiH[0][0];
    A.psi_hxy_in = G.psiH[1][0];
    A.psi_hyx_out = in == 0 ? c->psiH2[0][0].p : c->psif[0][1][0].p;
    A.psi_hxy_out = in == 0 ? c->psiH2[1][0].p : c->psif[1][1][0].p;
    A.psi_ezx = G.psiE[0][0];
    A.psi_ezy = G.psiE[1][0];
    A.err = c->d_err.p;
    A.rowc = reinterpret_cast<const float4 *>(c->rowc.p);
    launch_fused_tmz(A, G, c->fused_form, c->stream);
    if (ade) launch_ade_post(Fin, Fout, G, c->stream);
    c->launches += 1 + (ade && c->ade_n > 0 ? 1 : 0);
    c->cur = out;
}

// After fused_step(c, false): the dispersive cells, the source (a plane, or none) and the
// emitter current in one launch (post_eligible holds).
template <class R> void do_post(omx_ctx *c, StepParam amp, StepParam time, StepParam t_skip);
template <> void do_post<double>(omx_ctx *, StepParam, StepParam, StepParam) {}
template <> void do_post<float>(omx_ctx *c, StepParam amp, StepParam time, StepParam t_skip)
{
    ProfScope ps(c, KC_SRC);
    const FieldPtrs<float> Fin = field_ptrs<float>(c, 1 - c->cur), Fout = field_ptrs<float>(c, c->cur);
    const GridArgs<float> G = grid_args<float>(c);
    PostArgs Q{};
    Q.nb_ade = c->dims == 3 ? 0 : (c->ade_n + 127) / 128;   // the 3D pass updates them itself
    if (!c->sources.empty() && !c->fold3) {
        const SourceRec &S = *c->sources[0];
        Q.P.comp = S.pd.comp - 1;
        Q.P.axis = S.pd.plane_axis - 1;
        Q.P.index = S.pd.plane_index;
        Q.P.c_src = S.c_src;
        const int ax0 = Q.P.axis == 0 ? 1 : 0, ax1 = c->dims == 2 ? -1 : (Q.P.axis == 2 ? 1 : 2);
        Q.plane_n0 = c->n[ax0];
        Q.plane_cells = c->n[ax0] * (ax1 >= 0 ? c->n[ax1] : 1);
        Q.nb_plane = (Q.plane_cells + 127) / 128;
        Q.amp = amp;
    }
    if (c->inj_n > 0) {
        Q.I.n = c->inj_n;
        Q.I.eidx = c->inj_e.p;
        Q.I.comp = c->inj_c.p;
        Q.I.sa = c->inj_a.p;
        Q.I.sb = c->inj_b.p;
        Q.I.avg = (c->dims == 3 || (c->dims == 2 && c->desc.mode == OMX_TEZ_2D_MODE)) ? 1 : 0;
        Q.nb_inj = (c->inj_n + 127) / 128;
        Q.J = jstate(c);
        Q.time = time;
        Q.tskip = t_skip;
        Q.dt_eps0 = c->desc.dt / omx::consts().eps0;
    }
    if (Q.nb_ade + Q.nb_plane + Q.nb_inj == 0) return;
    launch_post_fused(Fin, Fout, G, Q, c->stream);
    c->launches++;
}

// Order the main stream after the side-stream work a one-step omx_run left running.
// Order the main stream after the side stream's kernels (not after the detector copies an
// asynchronous drain queued behind them: the next side sequence follows those on the side
// stream anyway).
void join_side_kernels(omx_ctx *c)
{
    if (c && c->side_pending) {
        ck(cudaStreamWaitEvent(c->stream, c->ev_join, 0), "join");
        c->side_pending = false;
    }
}

void join_stream(omx_ctx *c)
{
    if (!c) return;
    join_side_kernels(c);
    if (c->drain_pending) {
        ck(cudaStreamWaitEvent(c->stream, c->ev_drain, 0), "join");
        c->drain_pending = false;
    }
}

double source_amp(const SourceRec &S, double time);

// Bring the context to a settled state before an entry point touches it: the side-stream work
// is joined and a deferred omx_step_H (with the sources requested after it) runs unfused.
void join_side(omx_ctx *c)
{
    join_stream(c);
    if (c && c->h_pending) {
        c->h_pending = false;
        if (c->fp32) do_H<float>(c);
        else do_H<double>(c);
        if (c->src_pending) {
            c->src_pending = false;
            std::vector<StepParam> amps;
            for (auto &s : c->sources) amps.push_back(imm(source_amp(*s, c->src_time)));
            if (c->fp32) do_sources<float>(c, amps);
            else do_sources<double>(c, amps);
        }
    }
}

// Synchronise the stream and report a failure that a kernel recorded in the error word.
void sync_checked(omx_ctx *c, const char *what)
{
    join_side(c);
    ck(cudaMemcpyAsync(c->h_err, c->d_err.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream), what);
    ck(cudaStreamSynchronize(c->stream), what);
    if (*c->h_err) {
        const int e = *c->h_err;
        *c->h_err = 0;
        ck(cudaMemsetAsync(c->d_err.p, 0, sizeof(int), c->stream), what);
        if (e & 4)
            throw Fail{OMX_ERR_CUDA, "fused 3D pass: a plane planned as lean needed CPML, media or a source; the "
                                     "fields of that step are invalid"};
        throw Fail{OMX_ERR_CUDA, "fused kernel: a bulk-copy wait ran out; the fields of that step are invalid"};
    }
}

double source_amp(const SourceRec &S, double time)
{
    // update_source (source_mod.f90:114-130): j_amp * exp(-((t-t0)/tau)^2) * cos(w0 (t-t0) + phase)
    const double j_amp = S.kind == 0 ? S.d.j_amp : S.pd.j_amp;
    const double t0 = S.kind == 0 ? S.d.t0 : S.pd.t0;
    const double tau = S.kind == 0 ? S.d.tau : S.pd.tau;
    const double w0 = S.kind == 0 ? S.d.w0 : S.pd.w0;
    const double ph0 = S.kind == 0 ? S.d.phase : S.pd.phase;
    const double chirp = S.kind == 0 ? S.d.chirp : S.pd.chirp;
    const double ti = S.kind == 0 ? S.d.t_init : S.pd.t_init;
    const double tf = S.kind == 0 ? S.d.t_final : S.pd.t_final;
    if (!(time >= ti && time <= tf)) return 0.0;
    const double a = (time - t0) / tau;
    const double envelope = std::exp(-(a * a));
    double ph = w0 * (time - t0) + ph0;
    if (chirp != 0.0) ph = ph + 0.5 * chirp * ((time - t0) * (time - t0));
    const double cos_t = std::cos(ph);
    return j_amp * envelope * cos_t;
}

// Per-step table of a device-loop run (step-major: time, t_skip, move, slot, amps...), copied
// from pinned staging to the device, and the step counter reset; the stepping state advances as
// the reference's loop does (mxim_mxll.f90:92-104).  Sets run_step; the caller clears it.
struct RunPlan {
    int W = 0;
    bool has_det = false;
    int nrec = 0;
    size_t need = 0;
    omx_ctx::HostStage *stage = nullptr;
};
// The device side of the staging: the table copy and the step counters.  first_counted: the
// step's first kernel already ran without a counter, so the main counter starts at step 0.
// The device table and the step counters exist with room for the plan (a larger table is a new
// allocation, which invalidates the captured graphs).
void stage_reserve(omx_ctx *c, const RunPlan &plan)
{
    if (plan.need > c->tab.n) {
        c->tab.alloc(std::max(plan.need, 2 * c->tab.n), false);
        c->epoch++;
    }
    if (!c->d_step.p) c->d_step.alloc(1, false);
    if (!c->d_step2.p) c->d_step2.alloc(1, false);
}
void stage_upload(omx_ctx *c, const RunPlan &plan, bool first_counted)
{
    stage_reserve(c, plan);
    ck(cudaMemcpyAsync(c->tab.p, plan.stage->p, plan.need * sizeof(double), cudaMemcpyHostToDevice, c->stream),
       "tab");
    ck(cudaEventRecord(plan.stage->ev, c->stream), "staging");
    // the first kernel of every step advances the counter, so it starts one below step 0
    ck(cudaMemsetAsync(c->d_step.p, first_counted ? 0x00 : 0xff, sizeof(int), c->stream), "step");
    ck(cudaMemsetAsync(c->d_step2.p, 0xff, sizeof(int), c->stream), "step");
    c->run_step = c->d_step.p;
}
RunPlan stage_run(omx_ctx *c, int tt0, int nsteps, int n_skip, int t_det_print, bool upload = true)
{
    prepare(c);
    const int nsrc = (int)c->sources.size();
    const bool has_det = !c->tap_field.empty() && t_det_print > 0;
    // per-step scalars, step-major: time, t_skip, move, slot, amps...
    const int W = 4 + nsrc;
    const size_t need = (size_t)W * nsteps;
    omx_ctx::HostStage &hs = c->tab_stage[c->tab_flip];
    c->tab_flip ^= 1;
    if (hs.ev) ck(cudaEventSynchronize(hs.ev), "staging");   // its previous copy has been consumed
    else ck(cudaEventCreateWithFlags(&hs.ev, cudaEventDisableTiming), "event");
    if (hs.cap < need) {
        if (hs.p) cudaFreeHost(hs.p);
        hs.p = nullptr;
        hs.cap = 0;
        ck(cudaMallocHost(&hs.p, need * sizeof(double)), "pinned staging");
        hs.cap = need;
    }
    double *tab = hs.p;
    const int tt_0 = (n_skip == 1) ? 1 : 0;
    int nrec = 0;
    for (int s = 0; s < nsteps; ++s) {
        const int tt = tt0 + s;
        const double time = c->desc.dt * ((double)tt - 0.5);
        const int tq_step = 1 + (tt - tt_0) / n_skip;
        bool move = false;
        if (tq_step > c->tq_step_old) {
            c->t_skip = time;
            c->tq_step_old = tq_step;
            move = !c->groups.empty();
        }
        int slot = -1;
        if (has_det && tt % t_det_print == 0) slot = c->rec_count + nrec++;
        double *row = tab + (size_t)s * W;
        row[0] = time;
        row[1] = c->t_skip;
        row[2] = move ? 1.0 : 0.0;
        row[3] = (double)slot;
        for (int q = 0; q < nsrc; ++q) row[4 + q] = source_amp(*c->sources[q], time);
    }
    if (has_det) ensure_rec_capacity(c, c->rec_count + nrec);
    RunPlan plan;
    plan.W = W;
    plan.has_det = has_det;
    plan.nrec = nrec;
    plan.need = need;
    plan.stage = &hs;
    if (upload) stage_upload(c, plan, false);
    return plan;
}

StepParam plan_param(omx_ctx *c, const RunPlan &plan, int row) { return StepParam{0.0, c->tab.p + row, c->d_step.p, plan.W}; }

// prepare_only: capture and instantiate the step graphs that the same call without it launches,
// with the device table and the record buffer sized for it, and run nothing (the stepping state
// and the record count stay as they are).
template <class R> void run_impl(omx_ctx *c, int tt0, int nsteps, int n_skip, int t_det_print, int use_graph,
                                 bool prepare_only = false)
{
    if (c->h_pending) join_side(c);
    // a configuration change, or anything but a one-step graph call, first waits for the side
    // sequence a previous one-step call left running
    if (c->j_dirty || c->det_dirty || c->fused_dirty || !c->started || nsteps != 1 || !use_graph || c->prof ||
        prepare_only)
        join_side(c);
    const double t_skip0 = c->t_skip;
    const int tq_old0 = c->tq_step_old;
    const RunPlan plan = stage_run(c, tt0, nsteps, n_skip, t_det_print, false);
    if (prepare_only) {
        c->t_skip = t_skip0;
        c->tq_step_old = tq_old0;
    }
    struct Reset {
        omx_ctx *c;
        ~Reset() { c->run_step = nullptr; }
    } reset{c};
    const int W = plan.W;
    const bool has_det = plan.has_det;
    const int nrec = plan.nrec;
    const int nsrc = (int)c->sources.size();
    auto P = [&](int row) { return StepParam{0.0, c->tab.p + row, c->d_step.p, W}; };
    auto P2 = [&](int row) { return StepParam{0.0, c->tab.p + row, c->d_step2.p, W}; };
    const bool fused = std::is_same<R, float>::value && c->fused_ok;
    // One step per call on the fused path (a host that drives the loop step by step): the step's
    // scalars go to the kernels as arguments (no table upload), the fused pass reads only the
    // field buffers, so it is launched before the wait on the previous call's side sequence and
    // overlaps it; the sources, the emitter current and this step's own side sequence follow,
    // and the side sequence is left running for the next call (every other entry point joins it
    // first; an asynchronous drain queues its copies behind it).  Same operations on the same
    // values as the graph schedule.
    // The two-pass path does the same with its H pass in place of the fused pass (when the
    // side work reads E only: every detector samples an E component).
    bool taps_e = true;
    for (int f : c->tap_field) taps_e = taps_e && f < 3;
    const bool split = !fused && c->dims >= 2 && (has_det || !c->groups.empty()) && (taps_e || !has_det);
    if (!prepare_only && (fused || split) && nsteps == 1 && use_graph && !c->prof && (has_det || !c->groups.empty())) {
        const double *row = plan.stage->p;    // this step's table row, on the host
        std::vector<StepParam> amps;
        for (int q = 0; q < nsrc; ++q) amps.push_back(imm(row[4 + q]));
        if (fused) {
            const bool post = c->post_ok;
            fused_step<R>(c, !post, c->fold3 ? &amps[0] : nullptr);
            join_side_kernels(c);
            if (post) {
                do_post<R>(c, nsrc ? amps[0] : imm(0.0), imm(row[0]), imm(row[1]));
            } else {
                do_sources<R>(c, amps);
                do_inject<R>(c, imm(row[0]), imm(row[1]));
            }
        } else {
            do_H<R>(c);
            join_side_kernels(c);
            if (c->plane_fold) {
                do_E<R>(c, imm(row[0]), imm(row[1]), &amps[0]);
            } else {
                do_sources<R>(c, amps);
                do_E<R>(c, imm(row[0]), imm(row[1]));
            }
        }
        ck(cudaEventRecord(c->ev_fork, c->stream), "fork");
        ck(cudaStreamWaitEvent(c->side, c->ev_fork, 0), "fork");
        std::swap(c->stream, c->side);
        if (has_det) do_sample<R>(c, imm(row[3]), imm(row[0]));
        for (auto &g : c->groups) do_group<R>(c, *g, imm(row[2]));
        std::swap(c->stream, c->side);
        ck(cudaEventRecord(c->ev_join, c->side), "join");
        c->side_pending = true;
        ck(cudaPeekAtLastError(), "launch");
        c->rec_count += nrec;
        return;
    }
    join_side(c);
    if (prepare_only) stage_reserve(c, plan);
    else stage_upload(c, plan, false);
    std::vector<StepParam> amps;
    for (int q = 0; q < nsrc; ++q) amps.push_back(P(4 + q));
    auto tail = [&]() {
        for (auto &g : c->groups) do_group<R>(c, *g, P(2));
        if (has_det) do_sample<R>(c, P(3), P(0));
    };
    const bool post = fused && c->post_ok;
    const StepParam *pl3 = (fused && c->fold3) ? &amps[0] : nullptr;   // the plane source inside the 3D pass
    auto one_step = [&]() {
        if (post) {
            fused_step<R>(c, false, pl3);
            do_post<R>(c, nsrc ? amps[0] : imm(0.0), P(0), P(1));
        } else if (fused) {
            fused_step<R>(c);
            do_sources<R>(c, amps);
            do_inject<R>(c, P(0), P(1));
        } else if (c->plane_fold) {
            do_H<R>(c);
            do_E<R>(c, P(0), P(1), &amps[0]);
        } else {
            do_H<R>(c);
            do_sources<R>(c, amps);
            do_E<R>(c, P(0), P(1));
        }
        tail();
    };
    // Fused path inside a graph: step s's detector sampling, emitter step and current scatter
    // run on the side stream, concurrently with step s+1's fused pass (which reads step s's
    // buffer set and writes the other one, and touches no emitter state); the emitter current
    // of step s+1 waits for step s's scatter.  Sampling goes first on the side stream, so that
    // the wait on the scatter also orders it before the pass that overwrites its buffer set.
    // Same operations on the same values as one_step: results are identical.
    auto overlapped_step = [&](bool wait_prev) {
        if (post) {
            fused_step<R>(c, false, pl3);
            if (wait_prev) ck(cudaStreamWaitEvent(c->stream, c->ev_join, 0), "wait");
            do_post<R>(c, nsrc ? amps[0] : imm(0.0), P(0), P(1));
        } else {
            fused_step<R>(c);
            do_sources<R>(c, amps);
            if (wait_prev) ck(cudaStreamWaitEvent(c->stream, c->ev_join, 0), "wait");
            do_inject<R>(c, P(0), P(1));
        }
        ck(cudaEventRecord(c->ev_fork, c->stream), "fork");
        ck(cudaStreamWaitEvent(c->side, c->ev_fork, 0), "fork");
        std::swap(c->stream, c->side);
        launch_step_advance(c->d_step2.p, c->stream);
        c->launches++;
        if (has_det) do_sample<R>(c, P2(3), P2(0));
        for (auto &g : c->groups) do_group<R>(c, *g, P2(2));
        std::swap(c->stream, c->side);
        ck(cudaEventRecord(c->ev_join, c->side), "join");
    };
    // Two-pass path inside a graph: step s's emitter work and detector sampling (which read E
    // only) run on the side stream next to step s+1's H pass (which writes H only); step s+1's
    // sources and E pass, which write E and take the emitter current, wait for them.  Same
    // operations on the same values as one_step.
    auto split_step = [&](bool wait_prev) {
        do_H<R>(c);
        if (wait_prev) ck(cudaStreamWaitEvent(c->stream, c->ev_join, 0), "wait");
        if (c->plane_fold) {
            do_E<R>(c, P(0), P(1), &amps[0]);
        } else {
            do_sources<R>(c, amps);
            do_E<R>(c, P(0), P(1));
        }
        ck(cudaEventRecord(c->ev_fork, c->stream), "fork");
        ck(cudaStreamWaitEvent(c->side, c->ev_fork, 0), "fork");
        std::swap(c->stream, c->side);
        launch_step_advance(c->d_step2.p, c->stream);
        c->launches++;
        for (auto &g : c->groups) do_group<R>(c, *g, P2(2));
        if (has_det) do_sample<R>(c, P2(3), P2(0));
        std::swap(c->stream, c->side);
        ck(cudaEventRecord(c->ev_join, c->side), "join");
    };
    // a captured graph of `steps` steps starting from the current buffer set, from the cache
    // when the configuration is unchanged
    auto launch_graph = [&](int steps, int times) {
        omx_ctx::GraphRec *hit = nullptr;
        for (auto &g : c->graphs)
            if (g.epoch == c->epoch && g.steps == steps && g.cur == c->cur && g.W == W && g.has_det == (int)has_det &&
                g.fused == (int)fused)
                hit = &g;
        if (!hit) {
            for (auto &g : c->graphs)
                if (g.epoch != c->epoch) cudaGraphExecDestroy(g.exec);
            c->graphs.erase(std::remove_if(c->graphs.begin(), c->graphs.end(),
                                           [&](const omx_ctx::GraphRec &g) { return g.epoch != c->epoch; }),
                            c->graphs.end());
            omx_ctx::GraphRec g{};
            g.epoch = c->epoch;
            g.steps = steps;
            g.cur = c->cur;
            g.W = W;
            g.has_det = has_det;
            g.fused = fused;
            cudaGraph_t graph;
            const long long before = c->launches;
            ck(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "capture");
            if (fused && (has_det || !c->groups.empty())) {
                for (int q = 0; q < steps; ++q) overlapped_step(q > 0);
                ck(cudaStreamWaitEvent(c->stream, c->ev_join, 0), "join");   // the last side sequence
            } else if (split && steps > 1) {
                for (int q = 0; q < steps; ++q) split_step(q > 0);
                ck(cudaStreamWaitEvent(c->stream, c->ev_join, 0), "join");
            } else {
                for (int q = 0; q < steps; ++q) one_step();
            }
            ck(cudaStreamEndCapture(c->stream, &graph), "end capture");
            g.launches = c->launches - before;
            c->launches = before;
            g.cur_after = c->cur;
            c->cur = g.cur;
            const cudaError_t e = cudaGraphInstantiate(&g.exec, graph, 0);
            cudaGraphDestroy(graph);
            ck(e, "instantiate");
            c->graphs.push_back(g);
            hit = &c->graphs.back();
        }
        for (int s = 0; s < times; ++s) ck(cudaGraphLaunch(hit->exec, c->stream), "graph launch");
        c->launches += hit->launches * times;
        // after an even number of fused steps this is the starting set; a graph only captured
        // (times == 0) leaves the set as it is
        if (times > 0) c->cur = hit->cur_after;
    };
    // the fused path alternates buffer sets, so its graphs cover an even number of steps; long
    // graphs keep the side stream's work overlapped across all but one step boundary per graph.
    // A run of 8 steps or more starts with a two-step graph, which the host submits quickly and
    // the device runs while the host submits the long one (a long graph's submission takes tens
    // of microseconds, during which the device would otherwise wait); then up to 64 steps are one
    // graph (an odd fused run: one graph of the even part and a one-step graph), a longer run
    // repeats a 16-step graph.
    if (use_graph && !c->prof) {
        const int k = prepare_only ? 0 : 1;
        int left = nsteps;
        if ((fused || split) && left >= 8) {
            launch_graph(2, k);
            left -= 2;
        }
        const int per_graph = (fused || split) ? (left > 64 ? 16 : (fused ? (left & ~1) : left)) : 1;
        const int ngraph = per_graph > 0 ? left / per_graph : 0;
        if (ngraph > 0) launch_graph(per_graph, k * ngraph);
        left -= ngraph * per_graph;
        if (left >= 2) launch_graph(2, k * (left / 2));
        if (left % 2) launch_graph(1, k);
    } else if (!prepare_only) {
        for (int s = 0; s < nsteps; ++s) one_step();
    }
    ck(cudaPeekAtLastError(), "launch");
    if (!prepare_only) c->rec_count += nrec;
}

// A launch shape as omx_autotune reports it: fused 3D pass: (ring depth x 100 + tile rows) x 1000
// + planes per block;
// fused TMz pass: the kernel form; unfused kernels: planes (3D) or rows (2D) per thread.
void apply_shape(omx_ctx *c, int v)
{
    const bool fused = c->fp32 && fused_eligible(c);
    c->march_two_pass = 0;
    if (v >= 1000) {
        c->fused_form = v / 1000;
        c->march = v % 1000;
    } else if (fused && c->dims == 3) {
        c->march = v;                 // the two half-step passes, v planes per thread
        c->march_two_pass = 1;
    } else if (fused) {
        c->fused_form = v;
    } else {
        c->march = v;
    }
}

constexpr int AUTOTUNE_STEPS = 4;   // steps timed back to back per candidate and round

// Time each candidate launch shape on the device and keep the fastest.  Runs on fields that are
// still all zero: every kernel maps zero fields, zero psi and zero ADE state to zero, so the
// candidates leave no trace in the simulation state.
template <class R> int autotune_impl(omx_ctx *c, int reps)
{
    const bool fused = std::is_same<R, float>::value && c->fused_ok;
    // 3D FP32 with the fused pass eligible: the two half-step passes compete too (shapes below
    // 1000: planes marched per thread); where their in-place buffers fit in L2 (small grids) they
    // can beat the single pass, whose ping-pong sets take twice the room
    const bool both = fused && c->dims == 3 && c->step_form == OMX_STEP_DEFAULT;
    std::vector<int> cand;
    if (fused && c->dims == 3) {
        // fused 3D pass: (ring depth x 100 + tile rows) x 1000 + planes per block
        int dev = 0, optin = 0;
        ck(cudaGetDevice(&dev), "device");
        ck(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev), "device");
        for (int ring : {0, 3, 6})
            for (int ty : {8, 16})
                for (int kch : {8, 16, 32, 64, 128})
                    if (kch <= c->n[2] * 2 && f3t_smem_bytes(ring * 100 + ty) <= optin)
                        cand.push_back((ring * 100 + ty) * 1000 + kch);
        if (both)
            for (int m : {1, 2, 4, 8, 16, 32}) cand.push_back(m);
    } else if (fused) {
        cand = {0, 4, 5, 6, 8, 14, 15, 16, 24, 25, 34, 36, 44, 45};
    } else if (c->dims == 3) {
        cand = {1, 2, 4, 8, 16, 32};
    } else if (c->dims == 2) {
        cand = {8, 16, 32, 64};
    } else {
        return 0;
    }
    auto select = [&](int v) { apply_shape(c, v); };
    auto once = [&]() {
        if (fused && c->march_two_pass == 0) {
            fused_step<R>(c);
        } else {
            do_H<R>(c);
            do_E<R>(c, imm(0.0), imm(0.0));
        }
    };
    // first use of every form sets its kernel attributes; then `reps` rounds, each timing
    // AUTOTUNE_STEPS steps of every candidate in turn (interleaved, so that clock or thermal drift
    // affects all candidates alike; several steps back to back, so that the host's launch gaps
    // hide behind the device's work as in a run); a candidate's time is its fastest round
    for (int v : cand) {
        select(v);
        once();
    }
    std::vector<float> best(cand.size(), 1e30f);
    for (int r = 0; r < reps; ++r)
        for (size_t k = 0; k < cand.size(); ++k) {
            select(cand[k]);
            ck(cudaEventRecord(c->t0, c->stream), "autotune");
            for (int s = 0; s < AUTOTUNE_STEPS; ++s) once();
            ck(cudaEventRecord(c->t1, c->stream), "autotune");
            ck(cudaEventSynchronize(c->t1), "autotune");
            float ms = 0.f;
            ck(cudaEventElapsedTime(&ms, c->t0, c->t1), "autotune");
            best[k] = std::min(best[k], ms);
        }
    int pick = cand[0];
    float bt = best[0];
    for (size_t k = 1; k < cand.size(); ++k)
        if (best[k] < bt) {
            bt = best[k];
            pick = cand[k];
        }
    if (fused && c->dims == 3) {
        // 3D: among the shapes within 1.5 % of the fastest, the one with the least shared memory
        // per block (the zero-field timing leaves out the emitter and sampling kernels that share
        // the SMs with the pass in a run; a smaller footprint leaves them more room)
        auto footprint = [](int v) { return v >= 1000 ? f3t_smem_bytes(v / 1000) : 0; };
        float pt = bt;
        for (size_t k = 0; k < cand.size(); ++k)
            if (best[k] <= bt * 1.015f &&
                (footprint(cand[k]) < footprint(pick) || (footprint(cand[k]) == footprint(pick) && best[k] < pt))) {
                pick = cand[k];
                pt = best[k];
            }
    }
    select(pick);
    ck(cudaPeekAtLastError(), "autotune");
    if (both && pick < 1000) {
        // the two half-step passes won: the grid steps with them from now on
        c->step_form = OMX_STEP_TWO_PASS;
        c->fused_dirty = true;
        c->march_two_pass = 0;
        c->march = pick;
        prepare(c);
    }
    return pick;
}

template <class R> void read_field_impl(omx_ctx *c, int field, double *host)
{
    int lo[3], hi[3];
    req(bounds_of(c, field, lo, hi), "field not present in this grid/mode");
    const int q = field_code_to_index(field);
    std::vector<R> tmp(c->felems);
    sync_checked(c, "sync");
    ck(cudaMemcpy(tmp.data(), field_ptrs<R>(c).f[q], c->felems * sizeof(R), cudaMemcpyDeviceToHost), "read field");
    long long o = 0;
    for (int k = lo[2]; k <= hi[2]; ++k)
        for (int j = lo[1]; j <= hi[1]; ++j)
            for (int i = lo[0]; i <= hi[0]; ++i) {
                // E ghost planes n+1 of periodic axes are closed by index remapping on the device
                // (not stored); H ghost planes 0 hold the wrapped values as in the reference
                bool ghost_periodic = false;
                const int ijk[3] = {i, j, k};
                for (int a = 0; a < c->dims; ++a)
                    if (field <= OMX_EZ_FIELD && c->per[a] && ijk[a] == c->n[a] + 1) ghost_periodic = true;
                host[o++] = ghost_periodic ? 0.0 : (double)tmp[(size_t)eindex(c, i, j, k)];
            }
}

template <class R> void write_field_impl(omx_ctx *c, int field, const double *host)
{
    int lo[3], hi[3];
    req(bounds_of(c, field, lo, hi), "field not present in this grid/mode");
    const int q = field_code_to_index(field);
    std::vector<R> tmp(c->felems);
    sync_checked(c, "sync");
    ck(cudaMemcpy(tmp.data(), field_ptrs<R>(c).f[q], c->felems * sizeof(R), cudaMemcpyDeviceToHost), "read field");
    long long o = 0;
    for (int k = lo[2]; k <= hi[2]; ++k)
        for (int j = lo[1]; j <= hi[1]; ++j)
            for (int i = lo[0]; i <= hi[0]; ++i) tmp[(size_t)eindex(c, i, j, k)] = (R)host[o++];
    h2d(field_ptrs<R>(c).f[q], tmp.data(), c->felems * sizeof(R), "write field");
}

}  // namespace

// message for calls without a context (omx_last_error(NULL))
void omx::set_global_error(const std::string &msg) { g_last_error = msg; }

// =================================================================================================
extern "C" {

const char *omx_last_error(const omx_ctx *ctx)
{
    if (ctx && !ctx->err.empty()) return ctx->err.c_str();
    return g_last_error.c_str();
}

int omx_select_device(int device)
{
    OMX_API_BEGIN
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        throw Fail{OMX_ERR_NODEV, "no CUDA device available (the library has no CPU path)"};
    }
    req(device >= 0 && device < ndev, "device index out of range");
    ck(cudaSetDevice(device), "cudaSetDevice");
    OMX_API_END(nullptr)
}

int omx_device_count(int *count)
{
    OMX_API_BEGIN
    req(count, "null argument");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess) {
        cudaGetLastError();
        ndev = 0;
    }
    *count = ndev;
    OMX_API_END(nullptr)
}

int omx_create(const omx_grid_desc *d, omx_ctx **out)
{
    omx_ctx *c = nullptr;
    try {
        req(d && out, "null argument");
        *out = nullptr;
        req(d->dimensions >= 1 && d->dimensions <= 3, "dimensions must be 1, 2 or 3");
        req(d->precision == OMX_PREC_FP64 || d->precision == OMX_PREC_FP32, "precision");
        req(d->dt > 0 && d->dr > 0, "dt and dr must be positive");
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
            cudaGetLastError();
            throw Fail{OMX_ERR_NODEV, "no CUDA device available (the library has no CPU path)"};
        }
        std::unique_ptr<omx_ctx> C(new omx_ctx);
        c = C.get();
        c->desc = *d;
        c->dims = d->dimensions;
        c->fp32 = d->precision == OMX_PREC_FP32;
        for (int a = 0; a < 3; ++a) c->n[a] = 1;
        for (int a = 0; a < c->dims; ++a) {
            req(d->grid_Ndims[a] >= 3, "grid_Ndims must be >= 3 on every active axis");
            c->n[a] = d->grid_Ndims[a];
        }
        if (c->dims == 2) req(d->mode == OMX_TMZ_2D_MODE || d->mode == OMX_TEZ_2D_MODE,
                              "2D mode must be TMz or TEz (the reference's 'full' mode allocates TEz only)");
        bool any_cpml = false;
        const int naxes = c->dims;
        for (int a = 0; a < naxes; ++a) {
            const int b = d->boundaries[a];
            req(b == OMX_CLOSE_BOUNDARIES || b == OMX_PERIODIC_BOUNDARIES || b == OMX_CPML_BOUNDARIES,
                "boundaries must be close, periodic or cpml");
            c->cpml_axis[a] = b == OMX_CPML_BOUNDARIES;
            c->per[a] = b == OMX_PERIODIC_BOUNDARIES;
            any_cpml |= c->cpml_axis[a];
        }
        req(!(c->dims == 1 && c->per[0]), "1D periodic boundaries write out of bounds in the reference (unsupported)");
        if (any_cpml) {
            req(d->npml >= 2, "npml must be >= 2 with CPML boundaries");
            for (int a = 0; a < naxes; ++a)
                if (c->cpml_axis[a]) req(c->n[a] >= 2 * d->npml, "grid too small for two CPML slabs");
        }
        ck(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "stream");
        ck(cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking), "stream");
        ck(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming), "event");
        ck(cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming), "event");
        ck(cudaStreamCreateWithFlags(&c->f3aux, cudaStreamNonBlocking), "stream");
        ck(cudaEventCreateWithFlags(&c->ev_f3a, cudaEventDisableTiming), "event");
        ck(cudaEventCreateWithFlags(&c->ev_f3b, cudaEventDisableTiming), "event");
        // layout
        const int align = c->fp32 ? 32 : 16;
        Lay &L = c->L;
        L.dims = c->dims;
        L.nx = c->n[0];
        L.ny = c->n[1];
        L.nz = c->n[2];
        L.off = align - 1;
        if (c->dims == 1) {
            L.px = 0;
            L.pz = 0;
            c->felems = (size_t)(L.off + L.nx + 2 + align);
        } else {
            // FP32 3D: the fused pass's tensor maps view each row from 3 elements before cell 0
            // (its tiles' boxes start on 16-byte boundaries) and must reach the ghost cell nx+1,
            // so the row holds nx + 5 elements at least
            const int row = (c->dims == 3 && c->fp32) ? L.nx + 5 : L.nx + 2;
            L.px = ((row + align - 1) / align) * align;
            L.pz = (c->dims == 3) ? (long long)L.px * (L.ny + 2) : 0;
            const long long rows = (long long)(L.ny + 2) * (c->dims == 3 ? (L.nz + 2) : 1);
            c->felems = (size_t)(L.off + (long long)L.px * rows + align);
        }
        bool used[6] = {false, false, false, false, false, false};
        if (c->dims == 3) for (int q = 0; q < 6; ++q) used[q] = true;
        else if (c->dims == 1) used[0] = used[4] = true;
        else if (d->mode == OMX_TMZ_2D_MODE) used[2] = used[3] = used[4] = true;
        else used[0] = used[1] = used[5] = true;
        for (int q = 0; q < 6; ++q) {
            c->field_used[q] = used[q];
            if (!used[q]) continue;
            if (c->fp32) c->ff[q].alloc(c->felems);
            else c->fd[q].alloc(c->felems);
        }
        // CPML tables and den arrays (init_*Dgrid)
        if (any_cpml) c->T = cpml_tables(d->npml, d->dr, d->dt);
        int b3[3] = {d->boundaries[0], c->dims >= 2 ? d->boundaries[1] : 0, c->dims == 3 ? d->boundaries[2] : 0};
        den_arrays(c->dims, c->n, d->npml, b3, d->dr, c->T, c->den_e, c->den_h);
        if (c->fp32) {
            upload_axis_tables<float>(c);
            alloc_psi<float>(c);
        } else {
            upload_axis_tables<double>(c);
            alloc_psi<double>(c);
        }
        // vacuum media
        const double *noeps[3] = {nullptr, nullptr, nullptr};
        if (c->fp32) build_media<float>(c, nullptr, noeps);
        else build_media<double>(c, nullptr, noeps);
        c->jbuf.alloc(9);
        c->d_err.alloc(1);
        c->d_done.alloc(1);
        ck(cudaMallocHost(&c->h_err, sizeof(int)), "pinned error word");
        *c->h_err = 0;
        ck(cudaEventCreate(&c->t0), "event");
        ck(cudaEventCreate(&c->t1), "event");
        *out = C.release();
        return OMX_OK;
    } catch (const Fail &f) {
        g_last_error = f.msg;
        return f.code;
    } catch (const std::exception &e) {
        g_last_error = e.what();
        return OMX_ERR_ARG;
    }
}

int omx_destroy(omx_ctx *c)
{
    if (!c) return OMX_OK;
    if (c->side) cudaStreamSynchronize(c->side);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto &e : c->evs) {
        cudaEventDestroy(e.a);
        cudaEventDestroy(e.b);
    }
    for (auto &g : c->graphs) cudaGraphExecDestroy(g.exec);
    for (auto &h : c->tab_stage) {
        if (h.p) cudaFreeHost(h.p);
        if (h.ev) cudaEventDestroy(h.ev);
    }
    if (c->t0) cudaEventDestroy(c->t0);
    if (c->t1) cudaEventDestroy(c->t1);
    if (c->h_err) cudaFreeHost(c->h_err);
    if (c->side) {
        cudaStreamSynchronize(c->side);
        cudaStreamDestroy(c->side);
    }
    if (c->f3aux) {
        cudaStreamSynchronize(c->f3aux);
        cudaStreamDestroy(c->f3aux);
    }
    if (c->ev_f3a) cudaEventDestroy(c->ev_f3a);
    if (c->ev_f3b) cudaEventDestroy(c->ev_f3b);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->ev_drain) cudaEventDestroy(c->ev_drain);
    for (auto &d : c->drain_slots) {
        if (d.h) cudaFreeHost(d.h);
        if (d.err) cudaFreeHost(d.err);
        if (d.ev) cudaEventDestroy(d.ev);
    }
    cudaStream_t s = c->stream;
    delete c;
    if (s) cudaStreamDestroy(s);
    return OMX_OK;
}

int omx_synchronize(omx_ctx *c)
{
    OMX_API_BEGIN
    join_side(c);
    req(c, "null context");
    sync_checked(c, "synchronize");
    OMX_API_END(c)
}

int omx_get_cpml_tables(const omx_ctx *c, double *be, double *ce, double *bh, double *ch)
{
    OMX_API_BEGIN
    req(c, "null context");
    req(!c->T.be.empty(), "no CPML axis in this grid");
    if (be) std::copy(c->T.be.begin(), c->T.be.end(), be);
    if (ce) std::copy(c->T.ce.begin(), c->T.ce.end(), ce);
    if (bh) std::copy(c->T.bh.begin(), c->T.bh.end(), bh);
    if (ch) std::copy(c->T.ch.begin(), c->T.ch.end(), ch);
    OMX_API_END(const_cast<omx_ctx *>(c))
}

int omx_get_den(const omx_ctx *c, int axis, double *den_e, double *den_h)
{
    OMX_API_BEGIN
    req(c && axis >= 1 && axis <= 3, "bad axis");
    const int a = axis - 1;
    for (int k = 1; k <= c->n[a]; ++k) {
        if (den_e) den_e[k - 1] = c->den_e[a][k];
        if (den_h) den_h[k - 1] = c->den_h[a][k];
    }
    OMX_API_END(const_cast<omx_ctx *>(c))
}

int omx_compute_cpml_tables(int npml, double dr, double dt, double *be, double *ce, double *bh, double *ch,
                            double *kappae, double *kappah)
{
    OMX_API_BEGIN
    req(npml >= 2 && dr > 0 && dt > 0, "bad argument");
    CpmlTables T = cpml_tables(npml, dr, dt);
    if (be) std::copy(T.be.begin(), T.be.end(), be);
    if (ce) std::copy(T.ce.begin(), T.ce.end(), ce);
    if (bh) std::copy(T.bh.begin(), T.bh.end(), bh);
    if (ch) std::copy(T.ch.begin(), T.ch.end(), ch);
    if (kappae) std::copy(T.kappae.begin(), T.kappae.end(), kappae);
    if (kappah) std::copy(T.kappah.begin(), T.kappah.end(), kappah);
    OMX_API_END(nullptr)
}

int omx_set_cpml_tables(omx_ctx *c, const double *be, const double *ce, const double *bh, const double *ch,
                        const double *dex, const double *dey, const double *dez, const double *dhx,
                        const double *dhy, const double *dhz)
{
    OMX_API_BEGIN
    join_side(c);
    req(c, "null context");
    c->epoch++;
    req(!c->started, "tables must be set before the first step", OMX_ERR_STATE);
    const int npml = c->desc.npml;
    if (be && ce && bh && ch && npml >= 2) {
        c->T.be.assign(be, be + npml);
        c->T.ce.assign(ce, ce + npml);
        c->T.bh.assign(bh, bh + npml - 1);
        c->T.ch.assign(ch, ch + npml - 1);
    }
    const double *de[3] = {dex, dey, dez}, *dh[3] = {dhx, dhy, dhz};
    for (int a = 0; a < 3; ++a)
        for (int k = 1; k <= c->n[a]; ++k) {
            if (de[a]) c->den_e[a][k] = de[a][k - 1];
            if (dh[a]) c->den_h[a][k] = dh[a][k - 1];
        }
    if (c->fp32) upload_axis_tables<float>(c);
    else upload_axis_tables<double>(c);
    OMX_API_END(c)
}

int omx_set_media(omx_ctx *c, int n_media, const omx_medium *media, const int32_t *media_map, const double *ex,
                  const double *ey, const double *ez)
{
    OMX_API_BEGIN
    join_side(c);
    req(c, "null context");
    c->epoch++;
    req(!c->started, "media must be set before the first step", OMX_ERR_STATE);
    req(n_media >= 0 && n_media < 255, "n_media out of range");
    req(n_media == 0 || media, "media descriptors missing");
    c->n_media = n_media;
    c->media.assign(media, media + n_media);
    for (auto &m : c->media) {
        req(m.medium_type >= OMX_NONE_MEDIUM && m.medium_type <= OMX_DL_MEDIUM, "medium_type");
        if (m.medium_type == OMX_DL_MEDIUM) req(m.n_poles >= 1 && m.n_poles <= OMX_MAX_POLES, "n_poles");
        if (m.medium_type == OMX_DIELECTRIC_MEDIUM) req(m.eps_r > 0, "dielectric eps_r must be positive");
    }
    const double *eps[3] = {ex, ey, ez};
    if (c->fp32) build_media<float>(c, media_map, eps);
    else build_media<double>(c, media_map, eps);
    c->j_dirty = true;
    c->fused_dirty = true;
    OMX_API_END(c)
}

int omx_medium_dielectric(double eps_r, omx_medium *m)
{
    OMX_API_BEGIN
    req(m, "null medium");
    medium_dielectric(eps_r, m);
    OMX_API_END(nullptr)
}

int omx_medium_drude(double omegaD, double GammaD, double eps_r, double dt, omx_medium *m)
{
    OMX_API_BEGIN
    req(m && dt > 0, "bad argument");
    medium_drude(omegaD, GammaD, eps_r, dt, m);
    OMX_API_END(nullptr)
}

int omx_medium_dl_library(const char *material, double eps_r, double dt, omx_medium *m)
{
    OMX_API_BEGIN
    req(material && m && dt > 0, "bad argument");
    req(medium_dl_library(material, eps_r, dt, m), std::string("unknown Drude-Lorentz material ") + material);
    OMX_API_END(nullptr)
}

int omx_medium_dl_custom(double eps_inf, double wp_ev, double gamma_ev, int n_poles, const double *pole_ev,
                         const double *strength, const double *width_ev, double dt, omx_medium *m)
{
    OMX_API_BEGIN
    req(m && dt > 0 && n_poles >= 1 && n_poles <= OMX_MAX_POLES && pole_ev && strength && width_ev, "bad argument");
    medium_dl_custom(eps_inf, wp_ev, gamma_ev, n_poles, pole_ev, strength, width_ev, dt, m);
    OMX_API_END(nullptr)
}

int omx_media_map_from_voxels(int dims, const int grid_Ndims[3], double dr, int n_media, const int *n_vox,
                              const double *vox_nm, int32_t *media_map)
{
    OMX_API_BEGIN
    req(dims >= 1 && dims <= 3 && grid_Ndims && media_map && dr > 0, "bad argument");
    int n[3] = {grid_Ndims[0], dims >= 2 ? grid_Ndims[1] : 1, dims == 3 ? grid_Ndims[2] : 1};
    media_map_from_voxels(dims, n, dr, n_media, n_vox, vox_nm, media_map);
    OMX_API_END(nullptr)
}

// The reference's per-call sequence keeps the overlap of the step graphs: q-group steps and
// detector records that read E only run on the side stream, next to the next step's first pass
// (the fused pass writes the other buffer set; the two-pass H pass writes H only).  Entry points
// that write E wait for the side kernels first; every other entry point joins fully (join_side).
bool side_capable(const omx_ctx *c, bool reads_h)
{
    if (c->prof) return false;
    if (c->fp32 && c->fused_ok) return true;
    return c->dims >= 2 && !reads_h;
}

void on_side(omx_ctx *c, const std::function<void()> &launch)
{
    ck(cudaEventRecord(c->ev_fork, c->stream), "fork");
    ck(cudaStreamWaitEvent(c->side, c->ev_fork, 0), "fork");
    std::swap(c->stream, c->side);
    try {
        launch();
    } catch (...) {
        std::swap(c->stream, c->side);
        throw;
    }
    std::swap(c->stream, c->side);
    ck(cudaEventRecord(c->ev_join, c->side), "join");
    c->side_pending = true;
}

// Before an entry point that reads E only, or writes H only: the deferred H half and a pending
// configuration change still join fully.
void settle_for_side(omx_ctx *c)
{
    if (c->h_pending || c->j_dirty || c->det_dirty || c->fused_dirty) join_side(c);
}

int omx_step_H(omx_ctx *c)
{
    OMX_API_BEGIN
    req(c, "null context");
    settle_for_side(c);
    prepare(c);
    if (c->fp32 && c->fused_ok && !c->prof) {
        c->h_pending = true;                 // runs with the next omx_step_E as one fused pass
        return OMX_OK;
    }
    // the H pass writes H only: side work left pending reads E only (side_capable)
    if (c->fp32) do_H<float>(c);
    else do_H<double>(c);
    ck(cudaPeekAtLastError(), "H launch");
    OMX_API_END(c)
}

int omx_step_E(omx_ctx *c, double time, double t_skip)
{
    OMX_API_BEGIN
    req(c, "null context");
    if (c->h_pending) {
        // the deferred H half and this E half in one pass, then the sources requested between
        // them and the emitter current: the order of omx_run's fused step.  The pass reads one
        // buffer set and writes the other, so it goes before the wait for the side kernels.
        c->h_pending = false;
        if (c->fold3) {
            // the single plane source goes inside the 3D pass (when it was requested)
            const StepParam amp = imm(c->src_pending ? source_amp(*c->sources[0], c->src_time) : 0.0);
            fused_step<float>(c, true, &amp);
            c->src_pending = false;
        } else {
            fused_step<float>(c);
        }
        join_side_kernels(c);
        if (c->src_pending) {
            c->src_pending = false;
            std::vector<StepParam> amps;
            for (auto &s : c->sources) amps.push_back(imm(source_amp(*s, c->src_time)));
            do_sources<float>(c, amps);
        }
        do_inject<float>(c, imm(time), imm(t_skip));
        ck(cudaPeekAtLastError(), "E launch");
        return OMX_OK;
    }
    settle_for_side(c);
    join_side_kernels(c);        // the E pass writes what the side work reads
    prepare(c);
    if (c->fp32) do_E<float>(c, imm(time), imm(t_skip));
    else do_E<double>(c, imm(time), imm(t_skip));
    ck(cudaPeekAtLastError(), "E launch");
    OMX_API_END(c)
}

int omx_source_add(omx_ctx *c, const omx_source_desc *d, int *id)
{
    OMX_API_BEGIN
    join_side(c);
    req(c && d, "null argument");
    c->epoch++;
    req(d->dir == 'x' || d->dir == 'y' || d->dir == 'z', "source direction must be x, y or z");
    if (c->dims == 1) req(d->dir == 'x', "1D sources must be along x (interactions_mod.f90:43-53)");
    if (c->dims == 2) {
        if (c->desc.mode == OMX_TMZ_2D_MODE) req(d->dir == 'z', "TMz sources drive Ez");
        else req(d->dir != 'z', "TEz sources drive Ex or Ey");
    }
    std::unique_ptr<SourceRec> S(new SourceRec);
    S->kind = 0;
    S->d = *d;
    const double dr = c->desc.dr;
    const int n_ker = (int)(d->radius / dr);   // source_mod.f90:71
    const int side = 2 * n_ker + 1;
    const int dims = c->dims;
    std::vector<double> ker = source_kernel(dims, n_ker, dr);
    const int npts = (int)ker.size();
    S->comp = d->dir == 'x' ? 0 : (d->dir == 'y' ? 1 : 2);
    S->avg = (dims == 1 || (dims == 2 && d->dir == 'z')) ? 0 : 1;
    S->c_src = c->desc.dt / omx::consts().eps0 / dr / omx::consts().c0 / 2.0;   // interactions_mod.f90:32
    // the next point along the source direction in the reference's column-major J_mat; the
    // reference reads one element past the kernel array at its last point (taken as zero)
    const int stride = d->dir == 'x' ? 1 : (d->dir == 'y' ? side : side * side);
    int N[3] = {c->n[0], c->n[1], c->n[2]};
    std::vector<long long> e;
    std::vector<double> ka, kb;
    const int kl = dims == 3 ? n_ker : 0, jl = dims >= 2 ? n_ker : 0;
    int q = 0;
    for (int k = -kl; k <= kl; ++k)
        for (int j = -jl; j <= jl; ++j)
            for (int i = -n_ker; i <= n_ker; ++i, ++q) {
                // determine_indx_and_ranks (source_mod.f90:345-367)
                const int ii = i + (int)(d->r0[0] / dr) + N[0] / 2;
                const int jj = dims >= 2 ? j + (int)(d->r0[1] / dr) + N[1] / 2 : 0;
                const int kk = dims == 3 ? k + (int)(d->r0[2] / dr) + N[2] / 2 : 0;
                req(ii >= 0 && ii <= N[0] + 1 && jj >= 0 && jj <= N[1] + 1 && kk >= 0 && kk <= N[2] + 1,
                    "source kernel extends outside the grid");
                e.push_back(eindex(c, ii, jj, kk));
                S->cells.push_back(make_int4(ii, jj, kk, d->dir == 'x' ? 0 : (d->dir == 'y' ? 1 : 2)));
                ka.push_back(ker[(size_t)q]);
                kb.push_back(S->avg ? (q + stride < npts ? ker[(size_t)(q + stride)] : 0.0) : 0.0);
            }
    S->n = (int)e.size();
    S->eidx.upload(e);
    S->ka.upload(ka);
    S->kb.upload(kb);
    c->sources.push_back(std::move(S));
    c->fused_dirty = true;
    if (id) *id = (int)c->sources.size() - 1;
    OMX_API_END(c)
}

int omx_plane_source_add(omx_ctx *c, const omx_plane_source_desc *d, int *id)
{
    OMX_API_BEGIN
    join_side(c);
    req(c && d, "null argument");
    c->epoch++;
    req(d->comp >= 1 && d->comp <= 3 && d->plane_axis >= 1 && d->plane_axis <= c->dims, "plane source axis/comp");
    req(c->field_used[d->comp - 1], "plane source component not present in this grid/mode");
    req(d->plane_index >= 1 && d->plane_index <= c->n[d->plane_axis - 1], "plane index");
    std::unique_ptr<SourceRec> S(new SourceRec);
    S->kind = 1;
    S->pd = *d;
    S->comp = d->comp - 1;
    S->avg = 0;
    S->n = 0;
    S->c_src = c->desc.dt / omx::consts().eps0 / c->desc.dr / omx::consts().c0 / 2.0;
    c->sources.push_back(std::move(S));
    c->fused_dirty = true;
    if (id) *id = (int)c->sources.size() - 1;
    OMX_API_END(c)
}

int omx_source_interactions(omx_ctx *c, double time)
{
    OMX_API_BEGIN
    req(c, "null context");
    if (c->h_pending && !c->src_pending && !c->j_dirty && !c->det_dirty && !c->fused_dirty) {
        c->src_pending = true;               // added after the fused pass of the next omx_step_E
        c->src_time = time;
        return OMX_OK;
    }
    settle_for_side(c);
    join_side_kernels(c);        // the sources write what the side work reads
    prepare(c);
    std::vector<StepParam> amps;
    for (auto &s : c->sources) amps.push_back(imm(source_amp(*s, time)));
    if (c->fp32) do_sources<float>(c, amps);
    else do_sources<double>(c, amps);
    ck(cudaPeekAtLastError(), "source launch");
    OMX_API_END(c)
}

int omx_qgroup_state_size(int model) { return model == OMX_EMITTER_TWO_LEVEL ? 3 : (model == OMX_EMITTER_THREE_LEVEL ? 8 : -1); }

int omx_qgroup_create(omx_ctx *c, const omx_qgroup_desc *d, const int32_t *cell, const double *params, int *gid)
{
    OMX_API_BEGIN
    join_side(c);
    req(c && d && cell && params, "null argument");
    c->epoch++;
    req(!c->started, "q-groups must be created before the first step", OMX_ERR_STATE);
    req(d->model == OMX_EMITTER_TWO_LEVEL || d->model == OMX_EMITTER_THREE_LEVEL, "emitter model");
    req(d->group_type == OMX_Q_MATERIAL || d->group_type == OMX_Q_SINGLE, "group type");
    req(d->n_systems >= 1 && d->dt > 0, "n_systems and dt must be positive");
    std::unique_ptr<GroupRec> G(new GroupRec);
    G->d = *d;
    G->npar = d->model == OMX_EMITTER_TWO_LEVEL ? 7 : 9;
    G->nst = omx_qgroup_state_size(d->model);
    const int n = d->n_systems, dims = c->dims;
    std::vector<int> ci(n), cj(n), ckk(n);
    for (int e = 0; e < n; ++e) {
        int ijk[3] = {cell[dims * e], dims >= 2 ? cell[dims * e + 1] : 0, dims == 3 ? cell[dims * e + 2] : 0};
        for (int a = 0; a < dims; ++a) req(ijk[a] >= 1 && ijk[a] <= c->n[a], "emitter cell outside the grid");
        ci[e] = ijk[0];
        cj[e] = ijk[1];
        ckk[e] = ijk[2];
    }
    // device rows sorted by cell (stable: emitters of one cell keep their order); every emitter's
    // arithmetic is its own, so the order changes no result
    G->order.resize(n);
    G->inv.resize(n);
    for (int e = 0; e < n; ++e) G->order[e] = e;
    std::stable_sort(G->order.begin(), G->order.end(), [&](int a, int b) {
        return cell_key(c, ci[a], cj[a], ckk[a]) < cell_key(c, ci[b], cj[b], ckk[b]);
    });
    for (int r = 0; r < n; ++r) G->inv[G->order[r]] = r;
    std::vector<int> di(n), dj(n), dk(n);
    std::vector<double> par((size_t)n * G->npar);
    for (int r = 0; r < n; ++r) {
        const int e = G->order[r];
        di[r] = ci[e];
        dj[r] = cj[e];
        dk[r] = ckk[e];
        std::copy(params + (size_t)e * G->npar, params + (size_t)(e + 1) * G->npar, par.begin() + (size_t)r * G->npar);
    }
    G->ci.upload(di);
    G->cj.upload(dj);
    G->ck.upload(dk);
    G->par.upload(par);
    // decay rates 1/T1, 1/T2 (IEEE quotients, the same values the oracle forms every step)
    std::vector<double> rates((size_t)2 * n);
    const int it1 = d->model == OMX_EMITTER_TWO_LEVEL ? 2 : 4;
    for (int r = 0; r < n; ++r) {
        rates[2 * r] = 1.0 / par[(size_t)r * G->npar + it1];
        rates[2 * r + 1] = 1.0 / par[(size_t)r * G->npar + it1 + 1];
    }
    G->rates.upload(rates);
    G->rho.alloc((size_t)n * G->nst);
    G->E.alloc((size_t)n * 3);
    G->dipole.alloc((size_t)n * 3);
    G->dPdt.alloc((size_t)n * 3);
    // J points written by this group, in the reference's write order
    if (d->group_type == OMX_Q_MATERIAL) {
        for (int e = 0; e < n; ++e) {
            G->pts.push_back({cell_key(c, ci[e], cj[e], ckk[e]), d->density});
            G->pts_owner.push_back(G->inv[e]);
        }
    } else {
        const int nk = 3;   // q_group_mod.f90:19
        std::vector<double> mk = qgroup_kernel(dims, nk);
        const int side = 2 * nk + 1;
        const int kl = dims == 3 ? nk : 0, jl = dims >= 2 ? nk : 0;
        for (int e = 0; e < n; ++e)
            for (int kk = -kl; kk <= kl; ++kk)
                for (int jj = -jl; jj <= jl; ++jj)
                    for (int ii = -nk; ii <= nk; ++ii) {
                        const int p = (ii + nk) + side * ((jj + jl) + side * (kk + kl));
                        const int pi = ci[e] + ii, pj = dims >= 2 ? cj[e] + jj : 0, pk = dims == 3 ? ckk[e] + kk : 0;
                        if (pi < 1 || pi > c->n[0] + 1 || (dims >= 2 && (pj < 1 || pj > c->n[1] + 1)) ||
                            (dims == 3 && (pk < 1 || pk > c->n[2] + 1)))
                            continue;   // outside the reference's J arrays
                        G->pts.push_back({cell_key(c, pi, pj, pk), d->density * mk[(size_t)p]});
                        G->pts_owner.push_back(G->inv[e]);
                    }
    }
    c->groups.push_back(std::move(G));
    c->j_dirty = true;
    if (gid) *gid = (int)c->groups.size() - 1;
    OMX_API_END(c)
}

int omx_qgroup_step(omx_ctx *c, int gid, int tq_step)
{
    OMX_API_BEGIN
    (void)tq_step;
    req(c && gid >= 0 && gid < (int)c->groups.size(), "bad group id");
    // reads E, writes the group's own state and the current the next E half takes
    if (side_capable(c, false)) {
        settle_for_side(c);
        prepare(c);
        if (side_capable(c, false)) {
            on_side(c, [&]() {
                if (c->fp32) do_group<float>(c, *c->groups[gid], imm(1.0));
                else do_group<double>(c, *c->groups[gid], imm(1.0));
            });
            ck(cudaPeekAtLastError(), "emitter launch");
            return OMX_OK;
        }
    }
    join_side(c);
    prepare(c);
    if (c->fp32) do_group<float>(c, *c->groups[gid], imm(1.0));
    else do_group<double>(c, *c->groups[gid], imm(1.0));
    ck(cudaPeekAtLastError(), "emitter launch");
    OMX_API_END(c)
}

int omx_qgroup_attach_closure(omx_ctx *c, int gid, omx_closure *cl, double check_fraction, double tol,
                              int check_every)
{
    OMX_API_BEGIN
    join_side(c);
    req(c && cl, "null argument");
    c->epoch++;
    req(gid >= 0 && gid < (int)c->groups.size(), "unknown q-group");
    req(!c->started, "attach the closure before the first step", OMX_ERR_STATE);
    req(check_fraction > 0.0 && check_fraction <= 1.0 && tol > 0.0 && check_every >= 1, "bad spot-check settings");
    GroupRec &g = *c->groups[gid];
    req(!g.cl, "the q-group already has a closure");
    const int n = g.d.n_systems;
    const int ns = std::max(1, (int)std::floor(check_fraction * n));
    std::vector<int> sub(ns), sub_of(n, -1);
    for (int s = 0; s < ns; ++s) {
        sub[s] = g.inv[(size_t)(((long long)s * n) / ns)];   // spread evenly over the caller's list
        sub_of[sub[s]] = s;
    }
    g.sub.upload(sub);
    g.sub_of.upload(sub_of);
    g.sub_rho.alloc((size_t)ns * g.nst);             // ground state, as the group's own state
    g.cwin.alloc((size_t)n * omx::CL_WIN);
    g.hst.alloc((size_t)n * 128);
    g.xh.alloc((size_t)n * 160, false);
    g.cY.alloc((size_t)n * 16, false);
    g.chb.alloc((size_t)n * 128, false);
    g.ca1.alloc((size_t)n * 256, false);
    g.ca2.alloc((size_t)n * 256, false);
    g.ca3.alloc((size_t)n * 256, false);
    g.cl_state.alloc(sizeof(omx::ClDevState));
    omx::ClDeploy &D = g.dep;
    D.n = n;
    D.n_sub = ns;
    D.check_every = check_every;
    D.e_scale = omx::closure_e_scale(cl);
    D.d_scale = omx::closure_d_scale(cl);
    D.tol = tol;
    D.win = g.cwin.p;
    D.hst = g.hst.p;
    D.xh = g.xh.p;
    D.G = nullptr;          // the gate pre-activations stay in tensor memory (fused GRU epilogue)
    D.Y = g.cY.p;
    D.hb = g.chb.p;
    D.a1 = g.ca1.p;
    D.a2 = g.ca2.p;
    D.a3 = g.ca3.p;
    D.sub = g.sub.p;
    D.sub_of = g.sub_of.p;
    D.sub_rho = g.sub_rho.p;
    D.st = reinterpret_cast<omx::ClDevState *>(g.cl_state.p);
    D.err = c->d_err.p;
    g.cl = cl;
    OMX_API_END(c)
}

int omx_qgroup_closure_status(omx_ctx *c, int gid, double *last_error, int *fallback, int *fallback_step,
                              int *checks)
{
    OMX_API_BEGIN
    join_side(c);
    req(c, "null context");
    req(gid >= 0 && gid < (int)c->groups.size() && c->groups[gid]->cl, "q-group without a closure");
    sync_checked(c, "closure status");
    omx::ClDevState st;
    ck(cudaMemcpy(&st, c->groups[gid]->dep.st, sizeof(st), cudaMemcpyDeviceToHost), "closure status");
    if (last_error) *last_error = st.last_err;
    if (fallback) *fallback = st.use_plain;
    if (fallback_step) *fallback_step = st.use_plain ? st.fallback_step : -1;
    if (checks) *checks = st.checks;
    OMX_API_END(c)
}

int omx_qgroup_read(omx_ctx *c, int gid, double *dipole, double *dPdt, double *efield, double *rho)
{
    OMX_API_BEGIN
    join_side(c);
    req(c && gid >= 0 && gid < (int)c->groups.size(), "bad group id");
    GroupRec &g = *c->groups[gid];
    ck(cudaStreamSynchronize(c->stream), "sync");
    const size_t n = (size_t)g.d.n_systems;
    // device rows back into the caller's emitter order
    std::vector<double> tmp;
    auto get = [&](double *out, const double *dev, int w) {
        if (!out) return;
        tmp.resize(n * w);
        ck(cudaMemcpy(tmp.data(), dev, n * w * sizeof(double), cudaMemcpyDeviceToHost), "read");
        for (size_t r = 0; r < n; ++r)
            std::copy(tmp.begin() + r * w, tmp.begin() + (r + 1) * w, out + (size_t)g.order[r] * w);
    };
    get(dipole, g.dipole.p, 3);
    get(dPdt, g.dPdt.p, 3);
    get(efield, g.E.p, 3);
    get(rho, g.rho.p, g.nst);
    OMX_API_END(c)
}

int omx_detector_add(omx_ctx *c, int type, int field, int nd, const int32_t *idx, int *did)
{
    OMX_API_BEGIN
    join_side(c);
    req(c && idx && nd >= 1, "bad argument");
    c->epoch++;
    req(type >= OMX_POINT_DETECTOR && type <= OMX_VOLUME_DETECTOR, "detector type");
    req(c->n_freq == 0, "add detectors before omx_detectors_dft_setup");
    req(field >= OMX_EX_FIELD && field <= OMX_HZ_FIELD, "field");
    req(c->field_used[field - 1], "detector field not present in this grid/mode");
    const int dims = c->dims;
    for (int s = 0; s < nd; ++s) {
        const int i = idx[s], j = dims >= 2 ? idx[nd + s] : 0, k = dims == 3 ? idx[2 * nd + s] : 0;
        req(i >= 1 && i <= c->n[0] && (dims < 2 || (j >= 1 && j <= c->n[1])) && (dims < 3 || (k >= 1 && k <= c->n[2])),
            "detector index outside the grid");
        long long t[4] = {0, 0, 0, 0};
        int nt = 1;
        double w = 1.0;
        auto E = [&](int a, int b, int cc) { return eindex(c, a, b, cc); };
        // write_fields_subs_mod.f90 stencils
        if (dims == 1) {
            if (field == OMX_EX_FIELD) { t[0] = E(i, 0, 0); }
            else { nt = 2; w = 0.5; t[0] = E(i - 1, 0, 0); t[1] = E(i, 0, 0); }   // :145
        } else if (dims == 2) {
            switch (field) {   // :346-369
            case OMX_EX_FIELD: nt = 2; w = 0.5; t[0] = E(i - 1, j, 0); t[1] = E(i, j, 0); break;
            case OMX_EY_FIELD: nt = 2; w = 0.5; t[0] = E(i, j - 1, 0); t[1] = E(i, j, 0); break;
            case OMX_EZ_FIELD: t[0] = E(i, j, 0); break;
            case OMX_HX_FIELD: nt = 2; w = 0.5; t[0] = E(i, j, 0); t[1] = E(i, j - 1, 0); break;
            case OMX_HY_FIELD: nt = 2; w = 0.5; t[0] = E(i, j, 0); t[1] = E(i - 1, j, 0); break;
            default: nt = 4; w = 0.25; t[0] = E(i, j, 0); t[1] = E(i - 1, j - 1, 0); t[2] = E(i - 1, j, 0); t[3] = E(i, j - 1, 0);
            }
        } else {
            switch (field) {   // :821-846 (points), :865-929 (lines, planes, volumes)
            case OMX_EX_FIELD: nt = 2; w = 0.5; t[0] = E(i - 1, j, k); t[1] = E(i, j, k); break;
            case OMX_EY_FIELD: nt = 2; w = 0.5; t[0] = E(i, j - 1, k); t[1] = E(i, j, k); break;
            case OMX_EZ_FIELD:
                if (type == OMX_POINT_DETECTOR) { t[0] = E(i, j, k); }
                else { nt = 2; w = 0.5; t[0] = E(i, j, k - 1); t[1] = E(i, j, k); }
                break;
            case OMX_HX_FIELD: nt = 4; w = 0.25; t[0] = E(i, j - 1, k); t[1] = E(i, j, k); t[2] = E(i, j, k - 1); t[3] = E(i, j - 1, k - 1); break;
            case OMX_HY_FIELD: nt = 4; w = 0.25; t[0] = E(i - 1, j, k); t[1] = E(i, j, k); t[2] = E(i, j, k - 1); t[3] = E(i - 1, j, k - 1); break;
            default: nt = 4; w = 0.25; t[0] = E(i, j, k); t[1] = E(i - 1, j, k); t[2] = E(i, j - 1, k); t[3] = E(i - 1, j - 1, k);
            }
        }
        c->tap_field.push_back(field - 1);
        c->tap_nt.push_back(nt);
        c->tap_w.push_back(w);
        for (int q = 0; q < 4; ++q) c->tap[q].push_back(t[q]);
    }
    {
        omx_ctx::Det dd;
        dd.type = type;
        dd.field = field;
        dd.nd = nd;
        dd.first = (int)c->tap_field.size() - nd;
        dd.idx.assign(idx, idx + (size_t)nd * dims);
        c->dets.push_back(std::move(dd));
    }
    c->det_dirty = true;
    if (did) *did = (int)c->dets.size() - 1;
    OMX_API_END(c)
}

int omx_detectors_total_points(const omx_ctx *c) { return c ? (int)c->tap_field.size() : 0; }

int omx_detectors_set_capacity(omx_ctx *c, int records)
{
    OMX_API_BEGIN
    join_side(c);
    req(c && records >= 1, "bad argument");
    c->epoch++;
    prepare(c);
    ensure_rec_capacity(c, records);
    OMX_API_END(c)
}

int omx_detectors_record(omx_ctx *c, double time)
{
    OMX_API_BEGIN
    req(c, "null context");
    req(!c->tap_field.empty(), "no detectors");
    bool reads_h = false;
    for (int f : c->tap_field) reads_h = reads_h || f >= 3;
    const bool side = side_capable(c, reads_h);
    if (side) settle_for_side(c);
    else join_side(c);
    prepare(c);
    ensure_rec_capacity(c, c->rec_count + 1);   // joins fully when it moves the records
    if (side && side_capable(c, reads_h)) {
        // the records are written on the side stream, behind any copies queued there
        on_side(c, [&]() {
            if (c->fp32) do_sample<float>(c, imm((double)c->rec_count), imm(time));
            else do_sample<double>(c, imm((double)c->rec_count), imm(time));
        });
    } else {
        join_side(c);
        if (c->fp32) do_sample<float>(c, imm((double)c->rec_count), imm(time));
        else do_sample<double>(c, imm((double)c->rec_count), imm(time));
    }
    ck(cudaPeekAtLastError(), "sample launch");
    c->rec_count++;
    OMX_API_END(c)
}

int omx_detectors_drain(omx_ctx *c, double *times, double *values, int max_records, int *n_records)
{
    OMX_API_BEGIN
    join_side(c);
    req(c && n_records, "null argument");
    sync_checked(c, "sync");
    const int npts = (int)c->tap_field.size();
    const int n = std::min(c->rec_count, max_records);
    if (n > 0) {
        if (times) ck(cudaMemcpy(times, c->rec_times.p, sizeof(double) * n, cudaMemcpyDeviceToHost), "drain");
        if (values) ck(cudaMemcpy(values, c->rec.p, sizeof(double) * (size_t)n * npts, cudaMemcpyDeviceToHost), "drain");
    }
    // keep records beyond max_records (moved to the front through host memory)
    if (n < c->rec_count) {
        const size_t rest = (size_t)(c->rec_count - n);
        std::vector<double> tv(rest), vv(rest * (size_t)npts);
        ck(cudaMemcpy(tv.data(), c->rec_times.p + n, sizeof(double) * rest, cudaMemcpyDeviceToHost), "drain");
        ck(cudaMemcpy(vv.data(), c->rec.p + (size_t)n * npts, sizeof(double) * vv.size(), cudaMemcpyDeviceToHost), "drain");
        h2d(c->rec_times.p, tv.data(), sizeof(double) * rest, "drain");
        h2d(c->rec.p, vv.data(), sizeof(double) * vv.size(), "drain");
    }
    c->rec_count -= n;
    *n_records = n;
    OMX_API_END(c)
}

int omx_detectors_drain_async(omx_ctx *c, long long *ticket)
{
    OMX_API_BEGIN
    req(c && ticket, "null argument");
    // behind a pending side sequence (which wrote the records) the copies go on the side stream,
    // so the main stream's next step does not wait for them
    const cudaStream_t st = c->side_pending ? c->side : c->stream;
    omx_ctx::DrainSlot *d = nullptr;
    for (auto &q : c->drain_slots)
        if (q.ticket < 0) {
            d = &q;
            break;
        }
    if (!d) throw Fail{OMX_ERR_STATE, "every drain slot holds an uncollected ticket"};
    const int npts = (int)c->tap_field.size();
    const int n = c->rec_count;
    const size_t need = (size_t)n * (1 + npts);
    if (!d->ev) ck(cudaEventCreateWithFlags(&d->ev, cudaEventDisableTiming), "event");
    if (!d->err) ck(cudaMallocHost(&d->err, sizeof(int)), "pinned drain");
    if (d->cap < need) {
        if (d->h) cudaFreeHost(d->h);
        d->h = nullptr;
        d->cap = 0;
        ck(cudaMallocHost(&d->h, std::max<size_t>(need, 64) * sizeof(double)), "pinned drain");
        d->cap = std::max<size_t>(need, 64);
    }
    if (n > 0) {
        ck(cudaMemcpyAsync(d->h, c->rec_times.p, sizeof(double) * n, cudaMemcpyDeviceToHost, st), "drain");
        ck(cudaMemcpyAsync(d->h + n, c->rec.p, sizeof(double) * (size_t)n * npts, cudaMemcpyDeviceToHost, st),
           "drain");
    }
    ck(cudaMemcpyAsync(d->err, c->d_err.p, sizeof(int), cudaMemcpyDeviceToHost, st), "drain");
    ck(cudaEventRecord(d->ev, st), "drain");
    if (c->side_pending) {
        // the copies end the side stream's queue: entry points that write the records or the
        // error word on the main stream wait for them (join_stream)
        if (!c->ev_drain) ck(cudaEventCreateWithFlags(&c->ev_drain, cudaEventDisableTiming), "event");
        ck(cudaEventRecord(c->ev_drain, c->side), "drain");
        c->drain_pending = true;
    }
    // the records are taken: later steps write from slot 0 again (stream order keeps the copy first)
    c->rec_count = 0;
    d->n = n;
    d->ticket = c->next_ticket++;
    *ticket = d->ticket;
    OMX_API_END(c)
}

int omx_detectors_collect(omx_ctx *c, long long ticket, double *times, double *values, int max_records,
                          int *n_records)
{
    OMX_API_BEGIN
    // waits on the ticket's own event only: no join, so a pending side sequence keeps running
    // next to the main stream's next step
    req(c && n_records, "null argument");
    omx_ctx::DrainSlot *d = nullptr;
    for (auto &q : c->drain_slots)
        if (q.ticket == ticket && ticket >= 0) d = &q;
    req(d != nullptr, "unknown or already collected ticket");
    ck(cudaEventSynchronize(d->ev), "collect");
    const int n = d->n;
    const int err = *d->err;
    d->ticket = -1;
    if (err) {
        join_side(c);
        ck(cudaMemsetAsync(c->d_err.p, 0, sizeof(int), c->stream), "collect");
        throw Fail{OMX_ERR_CUDA, "fused TMz kernel: a bulk-copy wait ran out; the fields of that step are invalid"};
    }
    req(max_records >= n, "max_records is smaller than the ticket's record count");
    const int npts = (int)c->tap_field.size();
    if (n > 0) {
        if (times) std::memcpy(times, d->h, sizeof(double) * n);
        if (values) std::memcpy(values, d->h + n, sizeof(double) * (size_t)n * npts);
    }
    *n_records = n;
    OMX_API_END(c)
}

int omx_detectors_dft_setup(omx_ctx *c, int n_freq, const double *omega, double weight)
{
    OMX_API_BEGIN
    join_side(c);
    req(c && n_freq >= 1 && omega, "bad argument");
    req(!c->tap_field.empty(), "no detectors");
    c->epoch++;
    const size_t n = (size_t)n_freq * c->tap_field.size();
    c->d_omega.upload(std::vector<double>(omega, omega + n_freq));
    c->dft_re.alloc(n);
    c->dft_im.alloc(n);
    c->n_freq = n_freq;
    c->dft_w = weight;
    OMX_API_END(c)
}

int omx_detectors_dft_read(omx_ctx *c, double *re, double *im)
{
    OMX_API_BEGIN
    join_side(c);
    req(c && re && im, "null argument");
    req(c->n_freq > 0, "no Fourier transforms set up");
    sync_checked(c, "dft read");
    const size_t n = (size_t)c->n_freq * c->tap_field.size();
    ck(cudaMemcpy(re, c->dft_re.p, n * sizeof(double), cudaMemcpyDeviceToHost), "dft read");
    ck(cudaMemcpy(im, c->dft_im.p, n * sizeof(double), cudaMemcpyDeviceToHost), "dft read");
    OMX_API_END(c)
}

int omx_field_energy(omx_ctx *c, double *energy)
{
    OMX_API_BEGIN
    join_side(c);
    req(c && energy, "null argument");
    if (!c->energy_buf.p) c->energy_buf.alloc(305);
    int used[6];
    for (int q = 0; q < 6; ++q) used[q] = c->field_used[q] ? 1 : 0;
    const omx::Consts &K = omx::consts();
    const double dV = std::pow(c->desc.dr, (double)c->dims);
    if (c->fp32) launch_field_energy<float>(field_ptrs<float>(c), c->L, used, K.eps0, K.mu0, dV, c->energy_buf.p, c->stream);
    else launch_field_energy<double>(field_ptrs<double>(c), c->L, used, K.eps0, K.mu0, dV, c->energy_buf.p, c->stream);
    ck(cudaPeekAtLastError(), "energy");
    sync_checked(c, "energy");
    ck(cudaMemcpy(energy, c->energy_buf.p + 304, sizeof(double), cudaMemcpyDeviceToHost), "energy");
    OMX_API_END(c)
}

namespace {
const char *field_name(int f)
{
    static const char *n[6] = {"Ex", "Ey", "Ez", "Hx", "Hy", "Hz"};
    return n[f - 1];
}
// cell index -> position in nm, as the reference's writers place a detector cell
// (write_fields_subs_mod.f90:672-690: i*dr - int(N/2)*dr)
double cell_nm(const omx_ctx *c, int axis, int i)
{
    return ((double)i * c->desc.dr - (double)(c->n[axis] / 2) * c->desc.dr) * omx::consts().au_to_nm;
}
}  // namespace

int omx_detectors_write_text(omx_ctx *c, const char *dir, int *n_records)
{
    OMX_API_BEGIN
    join_side(c);
    req(c && dir, "null argument");
    sync_checked(c, "write detectors");
    const int npts = (int)c->tap_field.size();
    const int n = c->rec_count;
    std::vector<double> times((size_t)n), vals((size_t)n * std::max(npts, 1));
    if (n > 0) {
        ck(cudaMemcpy(times.data(), c->rec_times.p, sizeof(double) * n, cudaMemcpyDeviceToHost), "write detectors");
        ck(cudaMemcpy(vals.data(), c->rec.p, sizeof(double) * vals.size(), cudaMemcpyDeviceToHost), "write detectors");
    }
    namespace fs = std::filesystem;
    const int dims = c->dims;
    for (size_t d = 0; d < c->dets.size(); ++d) {
        const omx_ctx::Det &D = c->dets[d];
        char sub[64];
        std::snprintf(sub, sizeof sub, "output_detector_%07d", (int)d + 1);
        const fs::path dp = fs::path(dir) / sub;
        std::error_code ec;
        fs::create_directories(dp, ec);
        req(!ec, "cannot create " + dp.string());
        auto idx = [&](int s, int a) { return a < dims ? D.idx[(size_t)a * D.nd + s] : 0; };
        if (D.type == OMX_POINT_DETECTOR) {
            // one file, one "time value" line per record (appended)
            const fs::path fp = dp / "point.dat";
            FILE *f = std::fopen(fp.string().c_str(), c->print_det_step == 0 ? "w" : "a");
            req(f != nullptr, "cannot open " + fp.string());
            for (int r = 0; r < n; ++r)
                std::fprintf(f, " %24.16E %24.16E\n", times[r], vals[(size_t)r * npts + D.first]);
            std::fclose(f);
            continue;
        }
        // lines, planes, volumes: one file per record with the reference's header lines
        const char *kind = D.type <= OMX_LINE_Z_DETECTOR ? "line" : (D.type <= OMX_PLANE_ZX_DETECTOR ? "plane" : "volume");
        for (int r = 0; r < n; ++r) {
            char name[64];
            std::snprintf(name, sizeof name, "%s_%s_%09d.dat", field_name(D.field), kind, c->print_det_step + r);
            const fs::path fp = dp / name;
            FILE *f = std::fopen(fp.string().c_str(), "w");
            req(f != nullptr, "cannot open " + fp.string());
            std::fprintf(f, "# Time = %18.8E (a.u.)\n", times[r]);
            for (int s = 0; s < D.nd; ++s) {
                for (int a = 0; a < dims; ++a) std::fprintf(f, " %24.16E", cell_nm(c, a, idx(s, a)));
                std::fprintf(f, " %24.16E\n", vals[(size_t)r * npts + D.first + s]);
            }
            std::fclose(f);
        }
    }
    c->print_det_step += n;
    c->rec_count = 0;
    if (n_records) *n_records = n;
    OMX_API_END(c)
}

int omx_qgroup_write_text(omx_ctx *c, int gid, const char *dir, double time, int append)
{
    OMX_API_BEGIN
    join_side(c);
    req(c && dir, "null argument");
    req(gid >= 0 && gid < (int)c->groups.size(), "unknown q-group");
    GroupRec &g = *c->groups[gid];
    sync_checked(c, "write q-group");
    const int n = g.d.n_systems;
    std::vector<double> rho((size_t)n * g.nst), dip((size_t)n * 3), par((size_t)n * g.npar);
    ck(cudaMemcpy(rho.data(), g.rho.p, rho.size() * sizeof(double), cudaMemcpyDeviceToHost), "write q-group");
    ck(cudaMemcpy(dip.data(), g.dipole.p, dip.size() * sizeof(double), cudaMemcpyDeviceToHost), "write q-group");
    ck(cudaMemcpy(par.data(), g.par.p, par.size() * sizeof(double), cudaMemcpyDeviceToHost), "write q-group");
    namespace fs = std::filesystem;
    char sub[64];
    std::snprintf(sub, sizeof sub, "output_q_group_%04d", gid + 1);
    const fs::path dp = fs::path(dir) / sub;
    std::error_code ec;
    fs::create_directories(dp, ec);
    req(!ec, "cannot create " + dp.string());
    const fs::path fp = dp / "energy_and_dipole.dat";
    FILE *f = std::fopen(fp.string().c_str(), append ? "a" : "w");
    req(f != nullptr, "cannot open " + fp.string());
    // the reference's block (output_mod.f90:324-331): time header, column header, one line per
    // emitter; the energy of a few-level emitter is Tr(rho H0) = sum over excited levels
    std::fprintf(f, "# Time = %18.8E (a.u.)\n", time);
    std::fprintf(f, "# N_mol        Energy (eV)                   Dipole_x (a.u.)             "
                    "Dipole_y (a.u.)             Dipole_z (a.u.)\n");
    const double au_to_ev = (double)27.2114f;
    for (int e = 0; e < n; ++e) {
        const size_t q = (size_t)g.inv[e];   // the emitter's device row
        const double *p = &par[q * g.npar], *r = &rho[q * g.nst];
        const double en = g.d.model == OMX_EMITTER_TWO_LEVEL ? p[0] * r[0] : p[0] * r[0] + p[1] * r[1];
        std::fprintf(f, "%8d %24.16E %24.16E %24.16E %24.16E\n", e + 1, en * au_to_ev, dip[3 * q], dip[3 * q + 1],
                     dip[3 * q + 2]);
    }
    std::fclose(f);
    OMX_API_END(c)
}

int omx_run(omx_ctx *c, int tt0, int nsteps, int n_skip_steps, int t_det_print, int use_graph)
{
    OMX_API_BEGIN
    req(c && nsteps >= 0 && n_skip_steps >= 1 && tt0 >= 1, "bad argument");
    if (nsteps == 0) return OMX_OK;
    if (c->fp32) run_impl<float>(c, tt0, nsteps, n_skip_steps, t_det_print, use_graph);
    else run_impl<double>(c, tt0, nsteps, n_skip_steps, t_det_print, use_graph);
    OMX_API_END(c)
}

int omx_run_prepare(omx_ctx *c, int tt0, int nsteps, int n_skip_steps, int t_det_print)
{
    OMX_API_BEGIN
    req(c && nsteps >= 0 && n_skip_steps >= 1 && tt0 >= 1, "bad argument");
    req(!c->prof, "profiling is on: runs launch kernels one by one", OMX_ERR_STATE);
    if (nsteps == 0) return OMX_OK;
    if (c->fp32) run_impl<float>(c, tt0, nsteps, n_skip_steps, t_det_print, 1, true);
    else run_impl<double>(c, tt0, nsteps, n_skip_steps, t_det_print, 1, true);
    sync_checked(c, "prepare");
    OMX_API_END(c)
}

int omx_set_step_form(omx_ctx *c, int form)
{
    OMX_API_BEGIN
    join_side(c);
    req(c, "null context");
    req(form == OMX_STEP_DEFAULT || form == OMX_STEP_TWO_PASS || form == OMX_STEP_SINGLE_PASS, "unknown step form");
    c->step_form = form;
    c->fused_dirty = true;
    c->epoch++;
    OMX_API_END(c)
}

int omx_set_launch_shape(omx_ctx *c, int shape)
{
    OMX_API_BEGIN
    join_side(c);
    req(c && shape >= 1, "bad argument");
    if (c->dims == 3 && c->fp32 && fused_eligible(c) && shape < 1000) {
        // 3D FP32: a shape below 1000 selects the two half-step passes (v planes per thread)
        c->step_form = OMX_STEP_TWO_PASS;
        c->fused_dirty = true;
        c->march = shape;
    } else if (c->dims == 3 && c->fp32 && fused_eligible(c)) {
        const int form = shape / 1000, rows = form % 100, ring = form / 100;
        req((rows == 8 || rows == 16) && (ring == 0 || (ring >= 2 && ring <= F3T_RING_MAX)) && shape % 1000 >= 1 &&
                shape % 1000 <= F3T_KMAX,
            "fused 3D shape: ring depth (0 or 2..16) * 100000 + (8 | 16) * 1000 + planes (1..128)");
        int dev = 0, optin = 0;
        ck(cudaGetDevice(&dev), "device");
        ck(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev), "device");
        req(f3t_smem_bytes(form) <= optin, "fused 3D shape: the ring does not fit in a block's shared memory");
    } else
        req(shape < 1000, "fused 3D shape for a grid that steps with two passes");
    apply_shape(c, shape);
    c->epoch++;
    OMX_API_END(c)
}

int omx_autotune(omx_ctx *c, int reps, int *choice)
{
    OMX_API_BEGIN
    join_side(c);
    req(c && reps >= 1, "bad argument");
    req(!c->started && !c->fields_written,
        "omx_autotune times kernels on the initial zero fields: call it after the grid is configured and "
        "before the first step or field write", OMX_ERR_STATE);
    req(!c->prof, "profiling is on");
    prepare(c);
    c->epoch++;
    const int pick = c->fp32 ? autotune_impl<float>(c, reps) : autotune_impl<double>(c, reps);
    sync_checked(c, "autotune");
    if (choice) *choice = pick;
    OMX_API_END(c)
}

}  // extern "C"

// ---- batched multi-grid runs ------------------------------------------------------------------
// Device tables of one batched run: the grids' tile list, the radial sources in rounds (round r
// holds source r of every grid, so one grid's sources keep their order) and the detectors.
template <class R> struct BatchTables {
    const BatchGrid<R> *grids = nullptr;
    long long tiles = 0;
    // grids large enough to fill the GPU on their own: they keep their own H / E launches (in the
    // same graph) and add no tiles to the batched passes
    std::vector<char> own;
    std::vector<const BatchSrc<R> *> src;
    std::vector<int> nsrc;
    std::vector<long long> src_pts;
    std::vector<std::vector<std::pair<int, int>>> planes;   // (grid, source) launched on their own
    const BatchDet<R> *dets = nullptr;
    int ndet = 0;
    long long det_pts = 0;
    // fused path: the grids of the batched pass (largest first); the first nsplit of them step with
    // the split pass (its runs: general runs, then lean runs, each with its grid's table index),
    // the others in one k_fused3_batch launch of f3_blocks blocks over their tiles
    const F3tBatchGrid *f3 = nullptr;
    int nsplit = 0, nmixed = 0;
    long long f3_blocks = 0;
    const int4 *f3gen = nullptr, *f3lean = nullptr;
    int nf3gen = 0, nf3lean = 0;
};

struct omx_batch {
    std::vector<omx_ctx *> ctx;
    bool fp32 = false;
    cudaStream_t stream = nullptr;
    int kch = 0;            // z planes per tile of the batched passes (0 = the default)
    int blocks = 0;         // persistent grid of the batched passes
    int own_launch_tiles_per_sm = 8;   // grids with at least this many tiles per SM launch alone (0: none)
    long long launches = 0;
    // device tables, one per step parity (the fused path alternates the members' buffer sets)
    DevBuf<unsigned char> dgrid[2], dsrc[2], ddet[2], df3[2];
    DevBuf<int4> df3runs[2];
    cudaEvent_t done = nullptr;   // recorded after a batched call; member streams wait on it
    // 1: every member steps with one fused pass and the batch runs the batched fused pass; 0: the
    // two half-step passes (k_batch3); -1: not decided yet
    int fused = -1;
    int f3form = 8, f3kch = 64;   // tile rows and planes per block of the fused batched pass
    // the f3nsplit largest grids step with the fused pass split by plane form (their general runs'
    // H on `aux` beside their lean runs, then their E), the others in one k_fused3_batch launch
    // (on `aux` after that H)
    int f3nsplit = 0;
    cudaStream_t aux = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_mixed = nullptr;
    // tables and captured step graphs, kept while the key (each member's configuration epoch,
    // buffer set, step table and the launch shapes) is unchanged
    std::vector<long long> key;
    BatchTables<float> Tf[2];
    BatchTables<double> Td[2];
    struct Graph {
        int steps;
        long long per;
        cudaGraphExec_t exec;
    };
    std::vector<Graph> graphs;
    void drop_graphs()
    {
        for (auto &g : graphs) cudaGraphExecDestroy(g.exec);
        graphs.clear();
    }
};
template <class R> BatchTables<R> (&batch_cache(omx_batch *b))[2];
template <> BatchTables<float> (&batch_cache<float>(omx_batch *b))[2] { return b->Tf; }
template <> BatchTables<double> (&batch_cache<double>(omx_batch *b))[2] { return b->Td; }

namespace {

constexpr int BATCH_DEFAULT_KCH = 16;

template <class T> size_t pad16(size_t n) { return (n * sizeof(T) + 15) / 16 * 16; }

// Tables of one batched step.  Two-pass path: q = 0.  Fused path: the step of parity q, whose
// pass reads each member's buffer set cur ^ q and whose sources and detectors work on the set the
// pass writes.
template <class R>
BatchTables<R> batch_tables(omx_batch *b, const std::vector<RunPlan> *plans, int kch, int q = 0)
{
    const int n = (int)b->ctx.size();
    const bool f3 = b->fused == 1;
    std::vector<int> cur0;
    for (auto *c : b->ctx) cur0.push_back(c->cur);
    struct RestoreCur {
        omx_batch *b;
        const std::vector<int> &cur0;
        ~RestoreCur()
        {
            for (size_t i = 0; i < b->ctx.size(); ++i) b->ctx[i]->cur = cur0[i];
        }
    } restore{b, cur0};
    if (f3)
        for (int i = 0; i < n; ++i) b->ctx[i]->cur = cur0[i] ^ q ^ 1;
    BatchTables<R> T;
    std::vector<BatchGrid<R>> grids(n);
    long long t0 = 0;
    size_t rounds = 0;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    T.own.assign(n, 0);
    for (int i = 0; i < n; ++i) {
        omx_ctx *c = b->ctx[i];
        std::memset(&grids[i], 0, sizeof(BatchGrid<R>));
        grids[i].G = grid_args<R>(c);
        grids[i].F = field_ptrs<R>(c);
        grids[i].tx = (c->L.nx + 31) / 32;
        grids[i].ty = (c->L.ny + 3) / 4;
        grids[i].tile0 = t0;
        const long long tiles = (long long)grids[i].tx * grids[i].ty * ((c->L.nz + kch - 1) / kch);
        // a grid of at least 8 tiles per SM fills the GPU by itself: its own launches beat the
        // persistent pass's per-tile lookup (an empty tile range is skipped by the lookup)
        if (b->own_launch_tiles_per_sm > 0 && tiles >= (long long)b->own_launch_tiles_per_sm * (sms > 0 ? sms : 152))
            T.own[i] = 1;
        else
            t0 += tiles;
        rounds = std::max(rounds, c->sources.size());
    }
    T.tiles = t0;
    std::vector<std::vector<BatchSrc<R>>> rs(rounds);
    T.planes.resize(rounds);
    std::vector<BatchDet<R>> dets;
    if (plans) {
        for (int i = 0; i < n; ++i) {
            omx_ctx *c = b->ctx[i];
            const RunPlan &P = (*plans)[i];
            for (size_t r = 0; r < c->sources.size(); ++r) {
                const SourceRec &S = *c->sources[r];
                if (f3 && c->fold3) continue;          // the single plane source is inside the pass
                if (S.kind != 0) {
                    T.planes[r].push_back({i, (int)r});
                    continue;
                }
                BatchSrc<R> e;
                std::memset(&e, 0, sizeof(e));
                e.F = field_ptrs<R>(c);
                e.S = src_args(S);
                e.amp = plan_param(c, P, 4 + (int)r);
                rs[r].push_back(e);
            }
            if (P.has_det) {
                BatchDet<R> e;
                std::memset(&e, 0, sizeof(e));
                e.F = field_ptrs<R>(c);
                e.D = det_args(c);
                e.slot = plan_param(c, P, 3);
                e.time = plan_param(c, P, 0);
                dets.push_back(e);
            }
        }
    }
    // points: a source entry covers its S.n points, a detector entry max(n, 1) (the first thread
    // also writes the record time)
    for (auto &r : rs) {
        long long p = 0;
        for (auto &e : r) {
            e.p0 = p;
            p += e.S.n;
        }
        T.src_pts.push_back(p);
        T.nsrc.push_back((int)r.size());
    }
    long long dp = 0;
    for (auto &e : dets) {
        e.p0 = dp;
        dp += std::max(e.D.n, 1);
    }
    T.det_pts = dp;
    T.ndet = (int)dets.size();
    // one upload per table
    size_t gbytes = pad16<BatchGrid<R>>(n);
    b->dgrid[q].alloc(gbytes, false);
    ck(cudaMemcpyAsync(b->dgrid[q].p, grids.data(), sizeof(BatchGrid<R>) * n, cudaMemcpyHostToDevice, b->stream),
       "batch");
    T.grids = reinterpret_cast<const BatchGrid<R> *>(b->dgrid[q].p);
    size_t sbytes = 0;
    std::vector<size_t> soff;
    for (auto &r : rs) {
        soff.push_back(sbytes);
        sbytes += pad16<BatchSrc<R>>(r.size());
    }
    if (sbytes) {
        b->dsrc[q].alloc(sbytes, false);
        for (size_t r = 0; r < rs.size(); ++r)
            if (!rs[r].empty())
                ck(cudaMemcpyAsync(b->dsrc[q].p + soff[r], rs[r].data(), sizeof(BatchSrc<R>) * rs[r].size(),
                                   cudaMemcpyHostToDevice, b->stream), "batch");
    }
    for (size_t r = 0; r < rs.size(); ++r)
        T.src.push_back(rs[r].empty() ? nullptr : reinterpret_cast<const BatchSrc<R> *>(b->dsrc[q].p + soff[r]));
    if (!dets.empty()) {
        b->ddet[q].alloc(pad16<BatchDet<R>>(dets.size()), false);
        ck(cudaMemcpyAsync(b->ddet[q].p, dets.data(), sizeof(BatchDet<R>) * dets.size(), cudaMemcpyHostToDevice,
                           b->stream), "batch");
        T.dets = reinterpret_cast<const BatchDet<R> *>(b->ddet[q].p);
    }
    std::vector<F3tBatchGrid> f3g;
    std::vector<int4> runs_gen, runs_lean;
    if constexpr (std::is_same<R, float>::value) {
        if (f3) {
            // the fused pass of every member in one launch, largest grid first
            std::vector<int> order(n);
            for (int i = 0; i < n; ++i) order[i] = i;
            std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
                const omx_ctx *x = b->ctx[a], *y = b->ctx[c];
                return (long long)x->n[0] * x->n[1] * x->n[2] > (long long)y->n[0] * y->n[1] * y->n[2];
            });
            const int TY = f3t_rows(b->f3form);
            const int ns = std::min(std::max(b->f3nsplit, 0), n);
            long long item = 0;
            for (int i : order) {
                omx_ctx *c = b->ctx[i];
                const int in = cur0[i] ^ q;
                c->cur = in;
                F3tBatchGrid e;
                std::memset(&e, 0, sizeof(e));
                e.G = grid_args<float>(c);
                e.A.in = field_ptrs<float>(c, in);
                e.A.out = field_ptrs<float>(c, 1 - in);
                for (int a = 0; a < 3; ++a)
                    for (int k = 0; k < 2; ++k) e.A.psiH_out[a][k] = in == 0 ? c->psiH2[a][k].p : c->psif[a][1][k].p;
                if (c->fold3 && plans) {
                    const SourceRec &S = *c->sources[0];
                    e.G.pl_on = 1;
                    e.G.pl_comp = S.pd.comp - 1;
                    e.G.pl_axis = S.pd.plane_axis - 1;
                    e.G.pl_index = S.pd.plane_index;
                    e.G.pl_c_src = S.c_src;
                    e.G.pl_amp = plan_param(c, (*plans)[i], 4);
                    // the pass advances the step counter when it ends: its reads are one row ahead
                    if (e.G.step_inc) e.G.pl_amp.tab += e.G.pl_amp.stride;
                }
                if (!encode_f3t_maps(reinterpret_cast<F3tMaps *>(e.m), e.A.in, c->L, TY))
                    throw Fail{OMX_ERR_CUDA, "cuTensorMapEncodeTiled failed for the batched fused pass"};
                e.kch = std::min(std::max(b->f3kch, 1), F3T_KMAX);
                e.tx = (c->L.nx + 31) / 32;
                e.ty = (c->L.ny + TY - 1) / TY;
                e.tz = (c->L.nz + e.kch - 1) / e.kch;
                const int gi = (int)f3g.size();
                if (gi >= ns) {
                    // one launch over the tiles of the grids from ns on
                    e.item0 = item;
                    item += (long long)e.tx * e.ty * e.tz;
                } else {
                    // the grid's runs for the split pass, tagged with its place in the table
                    std::vector<int4> g0, l0;
                    f3t_runs(c, TY, e.kch, g0, l0);
                    for (int4 &r : g0) r.w |= gi << 20;
                    for (int4 &r : l0) r.w |= gi << 20;
                    e.n_gen = (int)g0.size();
                    e.n_lean = (int)l0.size();
                    runs_gen.insert(runs_gen.end(), g0.begin(), g0.end());
                    runs_lean.insert(runs_lean.end(), l0.begin(), l0.end());
                }
                f3g.push_back(e);
            }
            b->df3[q].alloc(sizeof(F3tBatchGrid) * f3g.size(), false);
            ck(cudaMemcpyAsync(b->df3[q].p, f3g.data(), sizeof(F3tBatchGrid) * f3g.size(), cudaMemcpyHostToDevice,
                               b->stream),
               "batch");
            T.f3 = reinterpret_cast<const F3tBatchGrid *>(b->df3[q].p);
            T.nsplit = ns;
            T.nmixed = n - ns;
            T.f3_blocks = item;
            std::vector<int4> runs(runs_gen);
            runs.insert(runs.end(), runs_lean.begin(), runs_lean.end());
            b->df3runs[q].upload(runs);
            T.f3gen = b->df3runs[q].p;
            T.f3lean = b->df3runs[q].p + runs_gen.size();
            T.nf3gen = (int)runs_gen.size();
            T.nf3lean = (int)runs_lean.size();
        }
    }
    // the host vectors die here: wait for the copies that read them
    ck(cudaStreamSynchronize(b->stream), "batch");
    return T;
}

// Route every member's launches to the batch stream for the duration of a batched call (their
// own streams are drained first), and restore streams and run state afterwards; work a member
// stream receives later waits for the batched work (an event, no host synchronisation).
struct BatchStreams {
    omx_batch *b;
    std::vector<cudaStream_t> saved;
    explicit BatchStreams(omx_batch *bb) : b(bb)
    {
        for (auto *c : b->ctx) join_side(c);
        for (auto *c : b->ctx) ck(cudaStreamSynchronize(c->stream), "sync");
        for (auto *c : b->ctx) {
            saved.push_back(c->stream);
            c->stream = b->stream;
        }
    }
    ~BatchStreams()
    {
        const bool ev = b->done && cudaEventRecord(b->done, b->stream) == cudaSuccess;
        for (size_t i = 0; i < saved.size(); ++i) {
            b->ctx[i]->stream = saved[i];
            b->ctx[i]->run_step = nullptr;
            if (ev) cudaStreamWaitEvent(saved[i], b->done, 0);
            else cudaStreamSynchronize(b->stream);
        }
    }
};

// The fused pass of every member: the split pass for the T.nsplit largest grids (their general
// runs' new H on the auxiliary stream while their lean runs go on the batch's stream, then their
// general runs' new E) and one k_fused3_batch launch for the others (on the auxiliary stream after
// that H, so beside the lean runs too); every grid's pass writes only that grid.  Returns the
// kernels launched.
template <class R> long long batch_fused_pass(omx_batch *b, const BatchTables<R> &T, int form)
{
    int *err = b->ctx[0]->d_err.p;
    if (T.nsplit == 0) {
        ck(launch_fused3t_batch(T.f3, T.nmixed, T.f3_blocks, form, err, b->stream), "batched fused pass");
        return 1;
    }
    long long k = 0;
    const bool side = T.nf3gen > 0 || T.nmixed > 0;
    if (side) {
        ck(cudaEventRecord(b->ev_fork, b->stream), "event");
        ck(cudaStreamWaitEvent(b->aux, b->ev_fork, 0), "event");
        if (T.nf3gen > 0) {
            ck(launch_fused3t_batch_split(T.f3, T.f3gen, T.nf3gen, T.f3lean, T.nf3lean, form, 1, err, b->aux),
               "batched fused pass (general runs, H)");
            ++k;
        }
        ck(cudaEventRecord(b->ev_join, b->aux), "event");
        if (T.nmixed > 0) {
            ck(launch_fused3t_batch(T.f3 + T.nsplit, T.nmixed, T.f3_blocks, form, err, b->aux),
               "batched fused pass (one launch)");
            ++k;
        }
        ck(cudaEventRecord(b->ev_mixed, b->aux), "event");
    }
    if (T.nf3lean > 0) {
        ck(launch_fused3t_batch_split(T.f3, T.f3gen, T.nf3gen, T.f3lean, T.nf3lean, form, 2, err, b->stream),
           "batched fused pass (lean runs)");
        ++k;
    }
    if (side) {
        ck(cudaStreamWaitEvent(b->stream, b->ev_join, 0), "event");
        if (T.nf3gen > 0) {
            ck(launch_fused3t_batch_split(T.f3, T.f3gen, T.nf3gen, T.f3lean, T.nf3lean, form, 4, err, b->stream),
               "batched fused pass (general runs, E)");
            ++k;
        }
        ck(cudaStreamWaitEvent(b->stream, b->ev_mixed, 0), "event");
    }
    return k;
}

// One batched step: H of every grid in one launch, the sources, the dispersive cells and the
// bulk E of every grid in one launch, the per-grid emitter work, the detectors in one launch.
template <class R> long long batch_step(omx_batch *b, const BatchTables<R> &T, const std::vector<RunPlan> &plans,
                                        int kch)
{
    const int n = (int)b->ctx.size();
    long long k = 0;
    if (b->fused == 1) {
        // the fused pass of every member (dispersive cells and folded plane sources inside), then
        // the work on the sets it wrote: the other sources, the emitter current and q-groups,
        // the detectors
        k += batch_fused_pass(b, T, b->f3form);
        for (auto *c : b->ctx) c->cur ^= 1;
        for (size_t r = 0; r < T.src.size(); ++r) {
            if (T.nsrc[r] > 0) {
                launch_src_batch<R>(T.src[r], T.nsrc[r], T.src_pts[r], b->stream);
                ++k;
            }
            for (auto &gp : T.planes[r]) {
                omx_ctx *c = b->ctx[gp.first];
                launch_one_source<R>(c, (size_t)gp.second, plan_param(c, plans[gp.first], 4 + gp.second));
                ++k;
            }
        }
        for (int i = 0; i < n; ++i) {
            omx_ctx *c = b->ctx[i];
            const long long before = c->launches;
            do_inject<R>(c, plan_param(c, plans[i], 0), plan_param(c, plans[i], 1));
            for (auto &g : c->groups) do_group<R>(c, *g, plan_param(c, plans[i], 2));
            k += c->launches - before;
        }
        if (T.ndet > 0) {
            launch_sample_batch<R>(T.dets, T.ndet, T.det_pts, b->stream);
            ++k;
        }
        return k;
    }
    launch_batch3<R>(0, T.grids, n, T.tiles, kch, b->blocks, b->stream);
    ++k;
    for (int i = 0; i < n; ++i)
        if (T.own[i]) {
            omx_ctx *c = b->ctx[i];
            launch_h<R>(field_ptrs<R>(c), grid_args<R>(c), b->stream);
            ++k;
        }
    for (size_t r = 0; r < T.src.size(); ++r) {
        if (T.nsrc[r] > 0) {
            launch_src_batch<R>(T.src[r], T.nsrc[r], T.src_pts[r], b->stream);
            ++k;
        }
        for (auto &gp : T.planes[r]) {
            omx_ctx *c = b->ctx[gp.first];
            launch_one_source<R>(c, (size_t)gp.second, plan_param(c, plans[gp.first], 4 + gp.second));
            ++k;
        }
    }
    for (auto *c : b->ctx)
        if (c->ade_n > 0) {
            launch_ade<R>(field_ptrs<R>(c), grid_args<R>(c), b->stream);
            ++k;
        }
    launch_batch3<R>(1, T.grids, n, T.tiles, kch, b->blocks, b->stream);
    ++k;
    for (int i = 0; i < n; ++i)
        if (T.own[i]) {
            omx_ctx *c = b->ctx[i];
            GridArgs<R> G = grid_args<R>(c);
            G.ade_n = 0;   // the dispersive cells ran above with every grid's
            launch_e<R>(field_ptrs<R>(c), G, b->stream);
            ++k;
        }
    for (int i = 0; i < n; ++i) {
        omx_ctx *c = b->ctx[i];
        const long long before = c->launches;
        do_inject<R>(c, plan_param(c, plans[i], 0), plan_param(c, plans[i], 1));
        for (auto &g : c->groups) do_group<R>(c, *g, plan_param(c, plans[i], 2));
        k += c->launches - before;
    }
    if (T.ndet > 0) {
        launch_sample_batch<R>(T.dets, T.ndet, T.det_pts, b->stream);
        ++k;
    }
    return k;
}

// prepare_only: build the tables and capture the step graphs that the same call without it
// launches, and run nothing (the members' stepping state and records are unchanged).
template <class R> void batch_run_impl(omx_batch *b, int tt0, int nsteps, int n_skip, int t_det_print, int use_graph,
                                       bool prepare_only = false)
{
    BatchStreams streams(b);
    std::vector<RunPlan> plans;
    for (auto *c : b->ctx) {
        const double t_skip0 = c->t_skip;
        const int tq_old0 = c->tq_step_old;
        plans.push_back(stage_run(c, tt0, nsteps, n_skip, t_det_print, !prepare_only));
        if (prepare_only) {
            c->t_skip = t_skip0;
            c->tq_step_old = tq_old0;
            stage_reserve(c, plans.back());
            c->run_step = c->d_step.p;   // as stage_upload leaves it: the tables hold the counter
        }
    }
    const int kch = b->kch > 0 ? b->kch : BATCH_DEFAULT_KCH;
    if (b->blocks == 0) b->blocks = batch3_blocks<R>();
    // the fused path alternates the members' buffer sets: step s of this call uses T[s & 1]
    const bool f3 = b->fused == 1;
    std::vector<long long> key = {b->fused, kch, b->f3form, b->f3kch, b->f3nsplit, b->blocks};
    for (size_t i = 0; i < b->ctx.size(); ++i) {
        const omx_ctx *c = b->ctx[i];
        key.insert(key.end(), {(long long)c->epoch, c->cur, (long long)(uintptr_t)c->tab.p, plans[i].W,
                               plans[i].has_det ? 1 : 0});
    }
    BatchTables<R>(&T)[2] = batch_cache<R>(b);
    if (key != b->key) {
        b->drop_graphs();
        b->key.clear();
        T[0] = batch_tables<R>(b, &plans, kch, 0);
        T[1] = f3 ? batch_tables<R>(b, &plans, kch, 1) : BatchTables<R>();
        b->key = key;
    }
    if (use_graph) {
        // graphs of up to 8 steps (the step counters advance on the device, so every replay
        // runs the next steps; on the fused path a replayed graph covers an even number of
        // steps, so it starts from the same buffer sets); the remainder in one shorter graph.
        // A graph of an odd number of fused steps leaves the members on the other buffer sets,
        // which changes the key: it is never replayed from the wrong sets.
        auto run_graph = [&](int steps, int times) {
            omx_batch::Graph *hit = nullptr;
            for (auto &g : b->graphs)
                if (g.steps == steps) hit = &g;
            if (!hit) {
                std::vector<int> cur0;
                for (auto *c : b->ctx) cur0.push_back(c->cur);
                cudaGraph_t graph;
                ck(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "capture");
                long long per = 0;
                for (int q = 0; q < steps; ++q) per += batch_step<R>(b, T[f3 ? (q & 1) : 0], plans, kch);
                ck(cudaStreamEndCapture(b->stream, &graph), "end capture");
                for (size_t i = 0; i < b->ctx.size(); ++i) b->ctx[i]->cur = cur0[i];
                cudaGraphExec_t exec = nullptr;
                const cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
                cudaGraphDestroy(graph);
                ck(e, "instantiate");
                b->graphs.push_back({steps, per, exec});
                hit = &b->graphs.back();
            }
            for (int s = 0; s < times; ++s) ck(cudaGraphLaunch(hit->exec, b->stream), "graph launch");
            b->launches += hit->per * times;
            if (f3 && (steps * times) % 2)
                for (auto *c : b->ctx) c->cur ^= 1;
        };
        const int per_graph = f3 ? std::min(nsteps & ~1, 8) : std::min(nsteps, 8);
        const int k = prepare_only ? 0 : 1;
        if (per_graph > 0) run_graph(per_graph, k * (nsteps / per_graph));
        const int left = per_graph > 0 ? nsteps % per_graph : nsteps;
        if (left) run_graph(left, k);
    } else if (!prepare_only) {
        for (int s = 0; s < nsteps; ++s) b->launches += batch_step<R>(b, T[f3 ? (s & 1) : 0], plans, kch);
    }
    ck(cudaPeekAtLastError(), "launch");
    if (!prepare_only)
        for (size_t i = 0; i < b->ctx.size(); ++i) b->ctx[i]->rec_count += plans[i].nrec;
}

// Tile depth of the batched passes, timed on the zero initial fields (which every pass maps to
// zero, so nothing of the simulation state changes).
template <class R> int batch_autotune_impl(omx_batch *b, int reps)
{
    BatchStreams streams(b);
    if (b->blocks == 0) b->blocks = batch3_blocks<R>();
    const int n = (int)b->ctx.size();
    if (b->fused == 1) {
        // fused batched pass: s x 1000000 + (ring depth x 100 + tile rows) x 1000 + planes per
        // block (the s largest grids in the pass split by plane form, the others in one
        // k_fused3_batch launch; s among 0, n/4, n/2, n), each candidate timed over `reps` passes
        // on the zero initial fields (the pass maps them to zero)
        cudaEvent_t e0, e1;
        ck(cudaEventCreate(&e0), "event");
        ck(cudaEventCreate(&e1), "event");
        float best = 0.f;
        int pick = 8064;
        bool first = true;
        int dev = 0, optin = 0;
        ck(cudaGetDevice(&dev), "device");
        ck(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev), "device");
        std::vector<int> splits = {0, std::max(1, n / 4), std::max(1, n / 2), n};
        splits.erase(std::unique(splits.begin(), splits.end()), splits.end());
        for (int split : splits)
            for (int ring : {0, 6, 8})
                for (int ty : {8, 16})
                    for (int kch : {16, 32, 64, 128}) {
                        const int form = ring * 100 + ty;
                        if (f3t_smem_bytes(form) > optin) continue;
                        b->f3form = form;
                        b->f3kch = kch;
                        b->f3nsplit = split;
                        const BatchTables<R> T = batch_tables<R>(b, nullptr, kch, 0);
                        auto once = [&]() { batch_fused_pass(b, T, form); };
                        once();
                        ck(cudaEventRecord(e0, b->stream), "event");
                        for (int r = 0; r < reps; ++r) once();
                        ck(cudaEventRecord(e1, b->stream), "event");
                        ck(cudaEventSynchronize(e1), "batch autotune");
                        float ms = 0.f;
                        ck(cudaEventElapsedTime(&ms, e0, e1), "batch autotune");
                        if (first || ms < best) {
                            best = ms;
                            pick = split * 1000000 + form * 1000 + kch;
                            first = false;
                        }
                    }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        b->f3nsplit = pick / 1000000;
        b->f3form = pick / 1000 % 1000;
        b->f3kch = pick % 1000;
        return pick;
    }
    cudaEvent_t e0, e1;
    ck(cudaEventCreate(&e0), "event");
    ck(cudaEventCreate(&e1), "event");
    float best = 0.f;
    int pick = BATCH_DEFAULT_KCH;
    const int cand[4] = {4, 8, 16, 32};
    for (int k = 0; k < 4; ++k) {
        const BatchTables<R> T = batch_tables<R>(b, nullptr, cand[k]);
        auto once = [&]() {
            launch_batch3<R>(0, T.grids, n, T.tiles, cand[k], b->blocks, b->stream);
            for (auto *c : b->ctx)
                if (c->ade_n > 0) launch_ade<R>(field_ptrs<R>(c), grid_args<R>(c), b->stream);
            launch_batch3<R>(1, T.grids, n, T.tiles, cand[k], b->blocks, b->stream);
        };
        once();
        cudaEventRecord(e0, b->stream);
        for (int r = 0; r < reps; ++r) once();
        cudaEventRecord(e1, b->stream);
        const cudaError_t err = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (err == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
        if (err != cudaSuccess) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            ck(err, "batch autotune");
        }
        if (k == 0 || ms < best) {
            best = ms;
            pick = cand[k];
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->kch = pick;
    return pick;
}

// The batch's arithmetic, fixed at its first autotune or run: when every member steps with one
// fused FP32 pass, the batched fused pass (one launch, or split by plane form for the largest
// grids); otherwise the two half-step passes (k_batch3), which every member then keeps when used
// on its own.
void batch_decide(omx_batch *b)
{
    if (b->fused >= 0) return;
    bool all = b->fp32;
    for (auto *c : b->ctx) all = all && fused_eligible(c);
    b->fused = all ? 1 : 0;
    if (!all)
        for (auto *c : b->ctx) {
            c->step_form = OMX_STEP_TWO_PASS;
            c->fused_dirty = true;
            c->fused_ok = false;
            c->epoch++;
        }
}

}  // namespace

extern "C" {

int omx_batch_create(omx_ctx *const *ctxs, int n, omx_batch **out)
{
    OMX_API_BEGIN
    req(ctxs && out && n >= 1, "bad argument");
    *out = nullptr;
    std::unique_ptr<omx_batch> b(new omx_batch);
    for (int i = 0; i < n; ++i) {
        omx_ctx *c = ctxs[i];
        req(c != nullptr, "null context in the batch");
        req(c->dims == 3, "batched runs take 3D grids");
        req(c->fp32 == ctxs[0]->fp32, "the grids of a batch share one precision");
        req(!c->prof, "profiling is on for a member of the batch");
        for (int k = 0; k < i; ++k) req(ctxs[k] != c, "a context appears twice in the batch");
        b->ctx.push_back(c);
    }
    for (auto *c : b->ctx) join_side(c);
    b->fp32 = ctxs[0]->fp32;
    ck(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "stream");
    ck(cudaStreamCreateWithFlags(&b->aux, cudaStreamNonBlocking), "stream");
    ck(cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming), "event");
    ck(cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming), "event");
    ck(cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming), "event");
    ck(cudaEventCreateWithFlags(&b->ev_mixed, cudaEventDisableTiming), "event");
    *out = b.release();
    OMX_API_END(nullptr)
}

int omx_batch_autotune(omx_batch *b, int reps, int *choice)
{
    OMX_API_BEGIN
    req(b && reps >= 1, "bad argument");
    batch_decide(b);
    for (auto *c : b->ctx)
        req(!c->started && !c->fields_written,
            "omx_batch_autotune times the passes on the initial zero fields: call it after the grids are "
            "configured and before their first step or field write", OMX_ERR_STATE);
    for (auto *c : b->ctx) {
        prepare(c);
        c->epoch++;
    }
    b->drop_graphs();
    b->key.clear();
    const int pick = b->fp32 ? batch_autotune_impl<float>(b, reps) : batch_autotune_impl<double>(b, reps);
    if (choice) *choice = pick;
    OMX_API_END(nullptr)
}

int omx_batch_set_launch_shape(omx_batch *b, int shape)
{
    OMX_API_BEGIN
    req(b && shape >= 1, "bad argument");
    batch_decide(b);
    if (b->fused == 1) {
        const int form = shape / 1000 % 1000, rows = form % 100, ring = form / 100, kch = shape % 1000;
        req(shape / 1000000 <= (int)b->ctx.size() && (rows == 8 || rows == 16) &&
                (ring == 0 || (ring >= 2 && ring <= F3T_RING_MAX)) && kch >= 1 && kch <= F3T_KMAX,
            "fused batched shape: split grids (0..n) * 1000000 + ring depth (0 or 2..16) * 100000 + (8 | 16) * 1000 + "
            "planes (1..128)");
        int dev = 0, optin = 0;
        ck(cudaGetDevice(&dev), "device");
        ck(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev), "device");
        req(f3t_smem_bytes(form) <= optin, "fused batched shape: the ring does not fit in a block's shared memory");
        b->f3nsplit = shape / 1000000;
        b->f3form = form;
        b->f3kch = kch;
    } else {
        req(shape == 4 || shape == 8 || shape == 16 || shape == 32, "batched two-pass shape: tile depth 4, 8, 16 or 32");
        b->kch = shape;
    }
    OMX_API_END(nullptr)
}

int omx_batch_run(omx_batch *b, int tt0, int nsteps, int n_skip_steps, int t_det_print, int use_graph)
{
    OMX_API_BEGIN
    req(b && nsteps >= 0 && n_skip_steps >= 1 && tt0 >= 1, "bad argument");
    for (auto *c : b->ctx) req(!c->prof, "profiling is on for a member of the batch");
    if (nsteps == 0) return OMX_OK;
    batch_decide(b);
    if (b->fp32) batch_run_impl<float>(b, tt0, nsteps, n_skip_steps, t_det_print, use_graph);
    else batch_run_impl<double>(b, tt0, nsteps, n_skip_steps, t_det_print, use_graph);
    OMX_API_END(nullptr)
}

int omx_batch_run_prepare(omx_batch *b, int tt0, int nsteps, int n_skip_steps, int t_det_print)
{
    OMX_API_BEGIN
    req(b && nsteps >= 0 && n_skip_steps >= 1 && tt0 >= 1, "bad argument");
    for (auto *c : b->ctx) req(!c->prof, "profiling is on for a member of the batch");
    if (nsteps == 0) return OMX_OK;
    batch_decide(b);
    if (b->fp32) batch_run_impl<float>(b, tt0, nsteps, n_skip_steps, t_det_print, 1, true);
    else batch_run_impl<double>(b, tt0, nsteps, n_skip_steps, t_det_print, 1, true);
    ck(cudaStreamSynchronize(b->stream), "prepare");
    OMX_API_END(nullptr)
}

long long omx_batch_launch_count(const omx_batch *b) { return b ? b->launches : 0; }

int omx_batch_synchronize(omx_batch *b)
{
    OMX_API_BEGIN
    req(b, "null batch");
    ck(cudaStreamSynchronize(b->stream), "synchronize");
    for (auto *c : b->ctx) sync_checked(c, "synchronize");
    OMX_API_END(nullptr)
}

int omx_batch_destroy(omx_batch *b)
{
    if (!b) return OMX_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->aux) cudaStreamSynchronize(b->aux);
    b->drop_graphs();
    if (b->done) cudaEventDestroy(b->done);
    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    if (b->ev_join) cudaEventDestroy(b->ev_join);
    if (b->ev_mixed) cudaEventDestroy(b->ev_mixed);
    cudaStream_t s = b->stream, a = b->aux;
    delete b;
    if (s) cudaStreamDestroy(s);
    if (a) cudaStreamDestroy(a);
    return OMX_OK;
}

int omx_field_bounds(const omx_ctx *c, int field, int lo[3], int hi[3])
{
    OMX_API_BEGIN
    req(c && lo && hi, "null argument");
    req(bounds_of(c, field, lo, hi), "field not present in this grid/mode");
    OMX_API_END(const_cast<omx_ctx *>(c))
}

int omx_read_field(omx_ctx *c, int field, double *host)
{
    OMX_API_BEGIN
    join_side(c);
    req(c && host, "null argument");
    if (c->fp32) read_field_impl<float>(c, field, host);
    else read_field_impl<double>(c, field, host);
    OMX_API_END(c)
}

int omx_write_field(omx_ctx *c, int field, const double *host)
{
    OMX_API_BEGIN
    join_side(c);
    req(c && host, "null argument");
    c->fields_written = true;
    if (c->fp32) write_field_impl<float>(c, field, host);
    else write_field_impl<double>(c, field, host);
    OMX_API_END(c)
}

int omx_profile_enable(omx_ctx *c, int on)
{
    OMX_API_BEGIN
    join_side(c);
    req(c, "null context");
    c->epoch++;
    prof_collect(c);
    c->prof = on != 0;
    for (int k = 0; k < KC_N; ++k) {
        c->prof_ms[k] = 0;
        c->prof_n[k] = 0;
    }
    OMX_API_END(c)
}

int omx_profile_query(omx_ctx *c, int kc, double *total_ms, long long *launches)
{
    OMX_API_BEGIN
    join_side(c);
    req(c && kc >= 0 && kc < KC_N, "bad argument");
    prof_collect(c);
    if (total_ms) *total_ms = c->prof_ms[kc];
    if (launches) *launches = c->prof_n[kc];
    OMX_API_END(c)
}

int omx_algorithmic_bytes(const omx_ctx *c, int kc, double *bytes)
{
    OMX_API_BEGIN
    req(c && bytes, "null argument");
    const double w = c->fp32 ? 4.0 : 8.0;
    const double cells = (double)c->n[0] * c->n[1] * c->n[2];
    // per-cell words: 3D H reads 6 / writes 3, E reads 6 / writes 3; 2D TMz/TEz H 5, E 4;
    // 1D H 3, E 3.  CPML cells add psi read+write per component; media-box cells add the
    // 1-byte material id per component and ADE cells their state.
    double b = 0.0;
    int ncomp_e = c->dims == 3 ? 3 : (c->dims == 1 ? 1 : (c->desc.mode == OMX_TMZ_2D_MODE ? 1 : 2));
    int ncomp_h = c->dims == 3 ? 3 : (c->dims == 1 ? 1 : (c->desc.mode == OMX_TMZ_2D_MODE ? 2 : 1));
    double psi_cells_h = 0.0, psi_cells_e = 0.0;   // component-cells carrying a psi term
    for (int a = 0; a < c->dims; ++a) {
        if (!c->cpml_axis[a]) continue;
        double tr = 1.0;
        for (int q = 0; q < c->dims; ++q)
            if (q != a) tr *= c->n[q];
        const double layers = 2.0 * (c->desc.npml - 1);
        const int pc = c->dims == 3 ? 2 : 1;
        psi_cells_h += layers * tr * pc;
        psi_cells_e += layers * tr * pc;
    }
    double ade_bytes = 0.0;
    if (c->has_ade) {
        // dispersive component-cells and their state words
        long long drude = 0, dl = 0;
        for (int q = 0; q < 3; ++q)
            for (size_t t = 0; t < c->host_mat[q].size(); ++t) {
                const int ty = c->cls_type[c->host_mat[q][t]];
                if (ty == CLS_DRUDE) drude++;
                else if (ty == CLS_DL) dl++;
            }
        ade_bytes = (double)drude * 2.0 * w + (double)dl * (2.0 + 2.0 + 4.0 * c->P) * w;
    }
    const bool fused = c->fused_ok;   // FP32 fused (2D TMz, 3D): one pass per step (class KC_E)
    if (kc == KC_H) {
        b = fused ? 0.0 : cells * w * (ncomp_e + 2.0 * ncomp_h) + psi_cells_h * 2.0 * w;
    } else if (kc == KC_E) {
        if (fused)   // each field word read once and written once
            b = cells * w * 2.0 * (ncomp_e + ncomp_h) + (psi_cells_h + psi_cells_e) * 2.0 * w +
                (double)c->bbV * ncomp_e + ade_bytes;
        else
            b = cells * w * (ncomp_h + 2.0 * ncomp_e) + psi_cells_e * 2.0 * w + (double)c->bbV * ncomp_e + ade_bytes;
    } else {
        b = 0.0;
    }
    *bytes = b;
    OMX_API_END(const_cast<omx_ctx *>(c))
}

long long omx_launch_count(const omx_ctx *c) { return c ? c->launches : 0; }

int omx_timer_start(omx_ctx *c)
{
    OMX_API_BEGIN
    join_side(c);
    req(c, "null context");
    ck(cudaEventRecord(c->t0, c->stream), "event");
    OMX_API_END(c)
}

int omx_timer_stop(omx_ctx *c, float *ms)
{
    OMX_API_BEGIN
    join_side(c);
    req(c && ms, "null argument");
    ck(cudaEventRecord(c->t1, c->stream), "event");
    ck(cudaEventSynchronize(c->t1), "event sync");
    ck(cudaEventElapsedTime(ms, c->t0, c->t1), "elapsed");
    OMX_API_END(c)
}

int omx_flush_l2(omx_ctx *c)
{
    OMX_API_BEGIN
    join_side(c);
    req(c, "null context");
    const long long n = 64LL << 20;   // 256 MB of floats, twice the L2
    if (!c->flushbuf.p) c->flushbuf.alloc((size_t)n);
    launch_flush(c->flushbuf.p, n, c->stream);
    ck(cudaPeekAtLastError(), "flush");
    OMX_API_END(c)
}

}  // extern "C"
