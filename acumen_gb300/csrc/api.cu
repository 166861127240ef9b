// C ABI of libacumen_gpu.so: contexts, the Radon operators and the batched /
// per-slice split-Bregman TV solvers (tomography/tv_hpc.F90:1-390).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "ctx.h"
#include "tables.h"

using namespace acu;

namespace acu {
thread_local std::string g_last_error;

int set_err(acu_ctx* ctx, int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (ctx) ctx->err = buf;
    g_last_error = buf;
    return code;
}
}  // namespace acu

namespace {

template <typename Real>
GeomSet<Real>& geomset(acu_ctx* c);
template <>
GeomSet<float>& geomset<float>(acu_ctx* c) { return c->g32; }
template <>
GeomSet<double>& geomset<double>(acu_ctx* c) { return c->g64; }

template <typename Real>
int ensure_geom(acu_ctx* c)
{
    GeomSet<Real>& gs = geomset<Real>(c);
    if (gs.ready) return ACU_OK;
    if (c->N <= 0) return set_err(c, ACU_ERR_INVALID, "context has no reconstruction grid (nimage = 0)");
    HostTables<Real> h;
    make_tables<Real>(c->N, c->T, c->theta.data(), c->wpu, h);
    CK(c, gs.sc_bp.ensure(sizeof(Real) * h.sc_bp.size()));
    CK(c, gs.sc_fp.ensure(sizeof(Real) * h.sc_fp.size()));
    CK(c, gs.filt.ensure(sizeof(Real) * (h.filt.size() + 8)));
    CK(c, gs.cmask.ensure(sizeof(Real) * h.cmask.size()));
    CK(c, gs.fft_h.ensure(sizeof(Real) * h.fft_h.size()));
    CK(c, gs.fft_h_x.ensure(sizeof(Real) * h.fft_h_x.size()));
    std::vector<float> tw32(h.fft_tw.begin(), h.fft_tw.end());
    CK(c, gs.fft_tw.ensure(sizeof(double) * h.fft_tw.size()));
    CK(c, cudaMemcpy(gs.sc_bp.p, h.sc_bp.data(), sizeof(Real) * h.sc_bp.size(), cudaMemcpyHostToDevice));
    CK(c, cudaMemcpy(gs.sc_fp.p, h.sc_fp.data(), sizeof(Real) * h.sc_fp.size(), cudaMemcpyHostToDevice));
    CK(c, gs.xsc_bp.ensure(sizeof(float) * h.xsc_bp.size()));
    CK(c, gs.xsc_fp.ensure(sizeof(float) * h.xsc_fp.size()));
    CK(c, cudaMemcpy(gs.xsc_bp.p, h.xsc_bp.data(), sizeof(float) * h.xsc_bp.size(), cudaMemcpyHostToDevice));
    CK(c, cudaMemcpy(gs.xsc_fp.p, h.xsc_fp.data(), sizeof(float) * h.xsc_fp.size(), cudaMemcpyHostToDevice));
    CK(c, cudaMemset(gs.filt.p, 0, sizeof(Real) * (h.filt.size() + 8)));
    CK(c, cudaMemcpy(gs.filt.p, h.filt.data(), sizeof(Real) * h.filt.size(), cudaMemcpyHostToDevice));
    CK(c, cudaMemcpy(gs.cmask.p, h.cmask.data(), sizeof(Real) * h.cmask.size(), cudaMemcpyHostToDevice));
    CK(c, cudaMemcpy(gs.fft_h.p, h.fft_h.data(), sizeof(Real) * h.fft_h.size(), cudaMemcpyHostToDevice));
    CK(c, cudaMemcpy(gs.fft_h_x.p, h.fft_h_x.data(), sizeof(Real) * h.fft_h_x.size(), cudaMemcpyHostToDevice));
    if (sizeof(Real) == 4)
        CK(c, cudaMemcpy(gs.fft_tw.p, tw32.data(), sizeof(float) * tw32.size(), cudaMemcpyHostToDevice));
    else
        CK(c, cudaMemcpy(gs.fft_tw.p, h.fft_tw.data(), sizeof(double) * h.fft_tw.size(), cudaMemcpyHostToDevice));
    gs.d.N = c->N;
    gs.d.T = c->T;
    gs.d.mid = h.mid;
    gs.d.sc_bp = gs.sc_bp.template as<Real>();
    gs.d.sc_fp = gs.sc_fp.template as<Real>();
    gs.d.filt = gs.filt.template as<Real>();
    gs.d.cmask = gs.cmask.template as<Real>();
    gs.d.fft_h = gs.fft_h.template as<Real>();
    gs.d.fft_h_x = gs.fft_h_x.template as<Real>();
    if (sizeof(Real) == 4 && !h.fft_tw16.empty()) {
        const std::vector<float> t16(h.fft_tw16.begin(), h.fft_tw16.end());
        CK(c, gs.fft_tw16.ensure(sizeof(float) * t16.size()));
        CK(c, cudaMemcpy(gs.fft_tw16.p, t16.data(), sizeof(float) * t16.size(), cudaMemcpyHostToDevice));
        gs.d.fft_tw16 = gs.fft_tw16.template as<float2>();
    }
    gs.d.fft_tw = gs.fft_tw.template as<float2>();
    gs.d.fft_tw64 = gs.fft_tw.template as<double2>();
    {
        // angle order of the pair projector: angles read through the x-pair
        // image (|sin| >= |cos|) first, then the transposed ones
        std::vector<int> ord;
        for (int pass = 0; pass < 2; ++pass)
            for (int t = 0; t < c->T; ++t) {
                const bool tr = std::fabs((double)h.sc_fp[2 * t + 1]) > std::fabs((double)h.sc_fp[2 * t]);
                if (tr == (pass == 1)) ord.push_back(t);
            }
        CK(c, gs.fp_order.ensure(sizeof(int) * ord.size()));
        CK(c, cudaMemcpy(gs.fp_order.p, ord.data(), sizeof(int) * ord.size(), cudaMemcpyHostToDevice));
        gs.d.fp_order = gs.fp_order.template as<int>();
        // projector variant 6: chunks of neighbouring angles, longest blocks first
        const std::vector<float> s32(h.sc_fp.begin(), h.sc_fp.end());
        ord = lines_angle_order(s32.data(), c->T);
        CK(c, gs.lines_order.ensure(sizeof(int) * ord.size()));
        CK(c, cudaMemcpy(gs.lines_order.p, ord.data(), sizeof(int) * ord.size(), cudaMemcpyHostToDevice));
        gs.d.lines_order = gs.lines_order.template as<int>();
    }
    gs.d.xsc_bp = gs.xsc_bp.template as<float4>();
    gs.hx_bp.resize(c->T);
    std::memcpy(gs.hx_bp.data(), h.xsc_bp.data(), sizeof(float4) * c->T);
    gs.d.h_xsc_bp = gs.hx_bp.data();
    if (sizeof(Real) == 4) {
        gs.hs_bp.resize(c->T);
        for (int t = 0; t < c->T; ++t)
            gs.hs_bp[t] = make_float4((float)h.sc_bp[2 * t], (float)h.sc_bp[2 * t + 1], 0.f, 0.f);
        gs.d.h_sc_bp = gs.hs_bp.data();
    }
    gs.d.xsc_fp = gs.xsc_fp.template as<float4>();
    gs.d.exact = (sizeof(Real) == 4) ? c->opt_positions : 0;
    gs.d.fft_L = h.fft_L;
    gs.d.fft_log2L = h.fft_log2L;
    gs.ready = true;
    return ACU_OK;
}

int check_ctx(acu_ctx* c, int nslices)
{
    if (!c) return set_err(nullptr, ACU_ERR_INVALID, "null context");
    if (c->N <= 0) return set_err(c, ACU_ERR_INVALID, "context has no reconstruction grid (nimage = 0)");
    if (nslices < 0) return set_err(c, ACU_ERR_INVALID, "nslices must be >= 0 (got %d)", nslices);
    return ACU_OK;
}

// Slices per thread of the batched kernels.
int pick_lanes(const acu_ctx* c, int S, bool is_double)
{
    if (is_double) return 1;
    if (c->opt_lanes == 1 || c->opt_lanes == 4) return c->opt_lanes;
    return S >= 4 ? 4 : 1;
}

// ---- operators in lane layout ---------------------------------------------
template <typename Real, int V>
void lanes_filter(acu_ctx* c, const DevGeom<Real>& g, int G, const Real* in, Real* out)
{
    if (c->opt_filter == 0 && g.fft_L > 0 && fft_fits<Real>(g.fft_L))
        launch_filter_fft<Real, V>(g, G, in, out, c->stream);
    else
        launch_filter_direct<Real, V>(g, G, in, out, c->stream);
}

template <typename Real, int V>
void lanes_iradon(acu_ctx* c, const DevGeom<Real>& g, int G, const Real* sino, Real* q, Real* img)
{
    lanes_filter<Real, V>(c, g, G, sino, q);
    launch_backproject<Real, V>(g, G, q, img, c->stream);
}

enum OpKind { OP_IRADON, OP_RADON, OP_RADON_ADJ, OP_FILTER, OP_BACKPROJECT };

// Runs one operator on plain-layout device arrays of S slices.
// The single-precision 4-slice projector variant for G slice groups:
// ACU_OPT_PROJECTOR, where 7 (automatic) takes the pixel-line projector (6)
// when the groups fill their 8-group lines to 8/9 or more (its cost follows
// the lines, the others' the groups), else variant 5.
int projector_variant(const acu_ctx* c, int G)
{
    if (c->opt_projector != 7) return c->opt_projector;
    return 8 * ((G + 7) / 8) <= G + G / 8 ? 6 : 5;
}

// Work buffers of the single-precision 4-slice projector that
// ACU_OPT_PROJECTOR selects, for G slice groups (grow-only).
int ensure_projector_buffers(acu_ctx* c, int G)
{
    const size_t nimg = (size_t)c->N * c->N * G * 4;
    const int v = projector_variant(c, G);
    if (v == 0) {
        CK(c, c->pairP.ensure(sizeof(float) * 2 * nimg));
        CK(c, c->pairPT.ensure(sizeof(float) * 2 * nimg));
    } else if (v == 6) {
        CK(c, c->lineL.ensure(sizeof(float) * lines_image_floats(c->N, G)));
        CK(c, c->lineA.ensure(sizeof(float) * lines_sums_floats(c->N, c->T, G)));
    } else {
        CK(c, c->pairPT.ensure(sizeof(float) * nimg));
    }
    return ACU_OK;
}

// The single-precision 4-slice projector that ACU_OPT_PROJECTOR selects
// (buffers from ensure_projector_buffers).
void radon_quads(acu_ctx* c, const DevGeom<float>& g, int G, const float* img, float* sino)
{
    const int v = projector_variant(c, G);
    if (v == 6)
        launch_radon_lines(g, G, img, c->lineL.as<float>(), c->lineA.as<float>(), sino, c->stream);
    else if (v >= 1)
        launch_radon_quads(g, G, img, c->pairPT.as<float>(), sino, c->stream, v == 2, v >= 3, v >= 4, v == 5);
    else
        launch_radon_pairs(g, G, img, c->pairP.as<float>(), c->pairPT.as<float>(), sino, c->stream);
}

template <typename Real, int V>
int run_op_v(acu_ctx* c, OpKind op, int S, const Real* in, Real* out)
{
    CKRET(ensure_geom<Real>(c));
    const DevGeom<Real>& g = geomset<Real>(c).d;
    const int N = c->N, T = c->T;
    const int G = (S + V - 1) / V;
    const size_t nsino = (size_t)T * N, nimg = (size_t)N * N;
    const bool in_sino = (op != OP_RADON);
    const bool out_sino = (op == OP_RADON || op == OP_FILTER);
    const size_t nin = in_sino ? nsino : nimg, nout = out_sino ? nsino : nimg;
    const Real* lin = in;
    Real* lout = out;
    if constexpr (V > 1) {
        CK(c, c->w_in.ensure(sizeof(Real) * nin * G * V));
        CK(c, c->w_out.ensure(sizeof(Real) * nout * G * V));
        launch_to_lanes<Real, V>(in, c->w_in.template as<Real>(), S, nin, c->stream);
        lin = c->w_in.template as<Real>();
        lout = c->w_out.template as<Real>();
    }
    switch (op) {
    case OP_IRADON:
        CK(c, c->w_q.ensure(sizeof(Real) * nsino * G * V));
        lanes_iradon<Real, V>(c, g, G, lin, c->w_q.template as<Real>(), lout);
        break;
    case OP_RADON:
        if constexpr (V == 4 && sizeof(Real) == 4) {
            CKRET(ensure_projector_buffers(c, G));
            radon_quads(c, g, G, lin, lout);
        } else if constexpr (V == 1 && sizeof(Real) == 4) {
            CK(c, c->pairPT.ensure(sizeof(float) * nimg * G));
            launch_radon_v1_fast(g, G, lin, c->pairPT.template as<float>(), lout, c->stream);
        } else {
            launch_radon<Real, V>(g, G, lin, lout, c->stream);
        }
        break;
    case OP_RADON_ADJ: launch_radon_adjoint<Real, V>(g, G, lin, lout, c->stream); break;
    case OP_FILTER: lanes_filter<Real, V>(c, g, G, lin, lout); break;
    case OP_BACKPROJECT: launch_backproject<Real, V>(g, G, lin, lout, c->stream); break;
    }
    CKLAUNCH(c);
    if constexpr (V > 1) {
        launch_from_lanes<Real, V>(lout, out, S, nout, c->stream);
        CKLAUNCH(c);
    }
    return ACU_OK;
}

template <typename Real>
int run_op(acu_ctx* c, OpKind op, int S, const Real* in, Real* out)
{
    CKRET(check_ctx(c, S));
    if (S == 0) return ACU_OK;
    if (!in || !out) return set_err(c, ACU_ERR_INVALID, "null array");
    if constexpr (sizeof(Real) == 4) {
        if (pick_lanes(c, S, false) == 4) return run_op_v<Real, 4>(c, op, S, in, out);
    }
    return run_op_v<Real, 1>(c, op, S, in, out);
}

// Host-buffer wrapper: copy in, run on the device, copy out, synchronise.
int run_op_host(acu_ctx* c, OpKind op, int S, const float* in, float* out)
{
    CKRET(check_ctx(c, S));
    if (S == 0) return ACU_OK;
    if (!in || !out) return set_err(c, ACU_ERR_INVALID, "null array");
    const size_t nsino = (size_t)c->T * c->N, nimg = (size_t)c->N * c->N;
    const size_t nin = (op == OP_RADON ? nimg : nsino) * S;
    const size_t nout = (op == OP_RADON || op == OP_FILTER ? nsino : nimg) * S;
    CK(c, c->w_host_in.ensure(sizeof(float) * nin));
    CK(c, c->w_host_out.ensure(sizeof(float) * nout));
    CK(c, cudaMemcpyAsync(c->w_host_in.p, in, sizeof(float) * nin, cudaMemcpyHostToDevice, c->stream));
    CKRET(run_op<float>(c, op, S, c->w_host_in.template as<float>(), c->w_host_out.template as<float>()));
    CK(c, cudaMemcpyAsync(out, c->w_host_out.p, sizeof(float) * nout, cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    return ACU_OK;
}

// ---- batched split-Bregman TV (tomography/tv_hpc.F90:162-363) --------------
template <typename Real>
TvState<Real>& tvstate(acu_ctx* c);
template <>
TvState<float>& tvstate<float>(acu_ctx* c) { return c->tv32; }
template <>
TvState<double>& tvstate<double>(acu_ctx* c) { return c->tv64; }

template <typename Real, int V>
struct TvRun {
    acu_ctx* c;
    const DevGeom<Real>* g;
    TvState<Real>* s;
    int N, T, G, S, ninner, ncg;
    Real lambda, mu;
    bool verbose;
    TvScalars sc;
    size_t nimg() const { return (size_t)N * N * G * V; }
    size_t nsino() const { return (size_t)T * N * G * V; }
    Real* B(DevBuf& b) const { return b.template as<Real>(); }

    void iradon(const Real* sino, Real* img) { lanes_iradon<Real, V>(c, *g, G, sino, B(s->q), img); }
    void radon(const Real* img, Real* sino)
    {
        if constexpr (V == 1 && sizeof(Real) == 4) {
            launch_radon_v1_fast(*g, G, img, c->pairPT.template as<float>(), sino, c->stream);
        } else if constexpr (V == 4 && sizeof(Real) == 4) {
            radon_quads(c, *g, G, img, sino);
        }
        else
            launch_radon<Real, V>(*g, G, img, sino, c->stream);
    }

    // One Bregman outer iteration (tv_hpc.F90:206-346).  On entry ruk holds
    // radon(uk) for the current uk, which the first inner iteration reuses.
    bool merged = true;   // initial residual with one backprojection (ACU_OPT_RESIDUAL)
    bool carried = false; // initial residual from carried backprojections (ACU_OPT_RESIDUAL = 2)
    int refresh = 1;      // radon(uk) recomputed every refresh-th outer iteration (ACU_OPT_RADON_REFRESH)
    // full: end with radon(uk) recomputed (always when refresh == 1);
    // otherwise radon(uk) is carried by ruk += alpha radon(p) in the CG loop.
    void outer_body(bool full = true)
    {
        const bool carry = refresh != 1;
        // ACU_OPT_RESIDUAL = 2 with radon(uk) carried: the initial residual's
        // backprojection is carried too, refreshed with radon(uk) every
        // `refresh` outer iterations (two backprojections then)
        cudaStream_t st = c->stream;
        using E = TvEw<Real, V>;
        for (int jinner = 1; jinner <= ninner; ++jinner) {
            if (verbose) cudaMemcpyAsync(s->ukp.p, s->uk.p, sizeof(Real) * nimg(), cudaMemcpyDeviceToDevice, st);
            if (carried) {
                // iradon(fk - radon(uk)) = bd + dacc, both carried: no backprojection
                E::rhs(N, G, mu, lambda, B(s->bd), B(s->dx), B(s->bx), B(s->dy), B(s->by), B(s->rhs), st, B(s->dacc));
                E::resid(N, G, mu, lambda, B(s->rhs), nullptr, B(s->uk), B(s->r), B(s->p), sc, st);
            } else if (merged) {
                // mu*iradon(fk) - mu*iradon(radon(uk)) as one backprojection of
                // the data residual fk - radon(uk) (iradon is linear)
                if (jinner > 1 && !carry) radon(B(s->uk), B(s->ruk));
                E::diff(nsino(), B(s->fk), B(s->ruk), B(s->rp), st);
                iradon(B(s->rp), B(s->tmp));
                E::rhs(N, G, mu, lambda, B(s->tmp), B(s->dx), B(s->bx), B(s->dy), B(s->by), B(s->rhs), st);
                E::resid(N, G, mu, lambda, B(s->rhs), nullptr, B(s->uk), B(s->r), B(s->p), sc, st);
            } else {
                iradon(B(s->fk), B(s->tmp));                               // ifkt
                E::rhs(N, G, mu, lambda, B(s->tmp), B(s->dx), B(s->bx), B(s->dy), B(s->by), B(s->rhs), st);
                if (jinner > 1 && !carry) radon(B(s->uk), B(s->ruk));
                iradon(B(s->ruk), B(s->tmp));                              // iukt
                E::resid(N, G, mu, lambda, B(s->rhs), B(s->tmp), B(s->uk), B(s->r), B(s->p), sc, st);
            }
            launch_cg_finalize(0, G * V, sc, st);
            for (int k = 0; k < ncg; ++k) {
                radon(B(s->p), B(s->rp));
                iradon(B(s->rp), B(s->tmp));                               // irpt
                E::apply(N, G, mu, lambda, B(s->tmp), B(s->p), B(s->Ap), sc, st);
                launch_cg_finalize(1, G * V, sc, st);
                if (carried)
                    E::update(N, G, B(s->p), B(s->Ap), B(s->uk), B(s->r), sc, st, B(s->tmp), B(s->bd));
                else
                    E::update(N, G, B(s->p), B(s->Ap), B(s->uk), B(s->r), sc, st);
                if (carry) E::sino_axpy(T, N, G, B(s->rp), B(s->ruk), sc, st);
                launch_cg_finalize(2, G * V, sc, st);
                E::pupdate(N, G, B(s->r), B(s->p), sc, st);
            }
            E::shrink(N, G, lambda, B(s->uk), B(s->dx), B(s->bx), B(s->dy), B(s->by),
                      verbose ? B(s->ukp) : nullptr, sc, st);
            if (verbose) launch_cg_finalize(3, G * V, sc, st);
        }
        if (full || !carry) radon(B(s->uk), B(s->ruk));
        E::fk_update(nsino(), B(s->fk), B(s->f), B(s->ruk), st);
        if (carried) {
            if (full) {
                carried_refresh();
            } else {
                // fk - f gains f - radon(uk): dacc gains bd
                E::add(nimg(), B(s->bd), B(s->dacc), st);
            }
        }
    }

    // bd = iradon(f - radon(uk)) and dacc = iradon(fk - f) from the current
    // fk and radon(uk) (two backprojections)
    void carried_refresh()
    {
        using E = TvEw<Real, V>;
        cudaStream_t st = c->stream;
        E::diff(nsino(), B(s->f), B(s->ruk), B(s->rp), st);
        iradon(B(s->rp), B(s->bd));
        E::diff(nsino(), B(s->fk), B(s->f), B(s->rp), st);
        iradon(B(s->rp), B(s->dacc));
    }
};

template <typename Real, int V>
TvRun<Real, V> make_run(acu_ctx* c, TvState<Real>& s)
{
    TvRun<Real, V> run;
    run.c = c;
    run.g = &geomset<Real>(c).d;
    run.s = &s;
    run.N = c->N; run.T = c->T; run.G = s.G; run.S = s.S;
    run.ninner = s.ninner; run.ncg = s.ncg; run.lambda = (Real)s.lambda; run.mu = (Real)s.mu;
    run.verbose = c->opt_verbose != 0;
    run.merged = c->opt_residual != 0;
    run.refresh = c->opt_refresh;
    run.carried = c->opt_residual == 2 && c->opt_refresh != 1;
    run.sc = TvScalars{s.rsold.template as<double>(), s.alpha.template as<double>(), s.beta.template as<double>(),
                       s.delta.template as<double>(), s.part.template as<double>(), s.nblk};
    return run;
}

// Allocates the solver state for S slices, copies f in, and runs the warm
// start and initialisation of tv_hpc.F90:172-202 (FBP, d = b = 0, fk = f),
// plus radon(uk) for the first inner iteration.
template <typename Real, int V>
int tv_begin_v(acu_ctx* c, int S, const Real* d_f, int ninner, int ncg, double lambda, double mu, Real* d_fbp)
{
    CKRET(ensure_geom<Real>(c));
    TvState<Real>& s = tvstate<Real>(c);
    const int N = c->N, T = c->T, G = (S + V - 1) / V;
    const size_t nimg = (size_t)N * N * G * V, nsino = (size_t)T * N * G * V;
    for (DevBuf* b : {&s.f, &s.fk, &s.ruk, &s.rp, &s.q}) CK(c, b->ensure(sizeof(Real) * nsino));
    for (DevBuf* b : {&s.uk, &s.dx, &s.dy, &s.bx, &s.by, &s.rhs, &s.r, &s.p, &s.Ap, &s.tmp})
        CK(c, b->ensure(sizeof(Real) * nimg));
    if (c->opt_verbose) CK(c, s.ukp.ensure(sizeof(Real) * nimg));
    if constexpr (V == 4 && sizeof(Real) == 4) {
        CKRET(ensure_projector_buffers(c, G));
    } else if constexpr (sizeof(Real) == 4) {
        CK(c, c->pairPT.ensure(sizeof(float) * nimg));
    }
    const int Sp = G * V;
    s.nblk = (int)std::min<size_t>(((size_t)N * N + 255) / 256, 512);
    for (DevBuf* b : {&s.rsold, &s.alpha, &s.beta, &s.delta}) CK(c, b->ensure(sizeof(double) * Sp));
    CK(c, s.part.ensure(sizeof(double) * (size_t)s.nblk * Sp));
    s.S = S; s.G = G; s.V = V; s.ninner = ninner; s.ncg = ncg; s.lambda = lambda; s.mu = mu;
    s.outer_done = 0;
    s.active = true;
    TvRun<Real, V> run = make_run<Real, V>(c, s);
    cudaStream_t st = c->stream;
    if constexpr (V > 1)
        launch_to_lanes<Real, V>(d_f, s.f.template as<Real>(), S, (size_t)T * N, st);
    else
        CK(c, cudaMemcpyAsync(s.f.p, d_f, sizeof(Real) * nsino, cudaMemcpyDeviceToDevice, st));
    run.iradon(s.f.template as<Real>(), s.uk.template as<Real>());
    if (d_fbp) {
        if constexpr (V > 1)
            launch_from_lanes<Real, V>(s.uk.template as<Real>(), d_fbp, S, (size_t)N * N, st);
        else
            CK(c, cudaMemcpyAsync(d_fbp, s.uk.p, sizeof(Real) * nimg, cudaMemcpyDeviceToDevice, st));
    }
    for (DevBuf* b : {&s.dx, &s.dy, &s.bx, &s.by}) CK(c, cudaMemsetAsync(b->p, 0, sizeof(Real) * nimg, st));
    CK(c, cudaMemcpyAsync(s.fk.p, s.f.p, sizeof(Real) * nsino, cudaMemcpyDeviceToDevice, st));
    run.radon(s.uk.template as<Real>(), s.ruk.template as<Real>());
    s.carried_valid = false;
    if (run.carried) {
        // fk = f: bd = iradon(f - radon(uk)), dacc = iradon(fk - f) = 0
        for (DevBuf* b : {&s.bd, &s.dacc}) CK(c, b->ensure(sizeof(Real) * nimg));
        TvEw<Real, V>::diff(nsino, s.f.template as<Real>(), s.ruk.template as<Real>(), s.rp.template as<Real>(), st);
        run.iradon(s.rp.template as<Real>(), s.bd.template as<Real>());
        CK(c, cudaMemsetAsync(s.dacc.p, 0, sizeof(Real) * nimg, st));
        s.carried_valid = true;
    }
    CKLAUNCH(c);
    return ACU_OK;
}

// nouter Bregman outer iterations (tv_hpc.F90:205-353) of the active problem.
template <typename Real, int V>
int tv_iterate_v(acu_ctx* c, int nouter)
{
    TvState<Real>& s = tvstate<Real>(c);
    TvRun<Real, V> run = make_run<Real, V>(c, s);
    cudaStream_t st = c->stream;
    const int S = s.S, Sp = s.G * V;
    const bool use_graph = c->opt_graph != 0 && !run.verbose;
    // the projector option may have changed since acu_tv_begin
    if constexpr (V == 4 && sizeof(Real) == 4) CKRET(ensure_projector_buffers(c, s.G));
    // the residual options may have changed too: the carried backprojections
    // start from the current iterate, and lapse when not carried
    if (run.carried && !s.carried_valid) {
        const size_t nimg = (size_t)c->N * c->N * s.G * V;
        for (DevBuf* b : {&s.bd, &s.dacc}) CK(c, b->ensure(sizeof(Real) * nimg));
        run.carried_refresh();
        s.carried_valid = true;
    }
    if (!run.carried) s.carried_valid = false;
    if (use_graph) {
        // the key holds every device address the captured iteration uses
        // outside the solver state, so a work buffer that has grown since
        // (another call on a larger batch) forces a new capture
        char key[400];
        snprintf(key, sizeof key, "%d/%d/%d/%d/%d/%.17g/%.17g/%d/%d/%d/%d/%d/%p/%p/%p/%p/%p/%p", (int)sizeof(Real), V,
                 s.G, s.ninner, s.ncg, s.lambda, s.mu, c->opt_filter, c->opt_projector, c->opt_positions,
                 c->opt_residual, c->g32.d.bp_tma * 100 + c->g32.d.bp_groups * 10 + c->g32.d.bp_param, s.uk.p, s.part.p, c->pairP.p,
                 c->pairPT.p, c->lineL.p, c->lineA.p);
        char key2[440];
        snprintf(key2, sizeof key2, "%s/%d", key, c->opt_refresh);
        if (!s.graph || s.graph_key != key2) {
            for (cudaGraphExec_t* gx : {&s.graph, &s.graph_inc})
                if (*gx) {
                    cudaGraphExecDestroy(*gx);
                    *gx = nullptr;
                }
            // Capture on the context's private stream (the legacy stream
            // cannot be captured); the graphs are then launched on `st`.
            // graph: radon(uk) recomputed at the end; graph_inc: carried.
            for (int which = 0; which < (run.refresh == 1 ? 1 : 2); ++which) {
                cudaGraph_t graph;
                CK(c, cudaStreamBeginCapture(c->own_stream, cudaStreamCaptureModeThreadLocal));
                c->stream = c->own_stream;
                run.outer_body(which == 0);
                c->stream = st;
                cudaError_t e = cudaStreamEndCapture(c->own_stream, &graph);
                if (e != cudaSuccess) return set_err(c, ACU_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
                cudaGraphExec_t* gx = which == 0 ? &s.graph : &s.graph_inc;
                e = cudaGraphInstantiate(gx, graph, 0);
                cudaGraphDestroy(graph);
                if (e != cudaSuccess) {
                    *gx = nullptr;
                    return set_err(c, ACU_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(e));
                }
            }
            s.graph_key = key2;
        }
        for (int jo = 0; jo < nouter; ++jo) {
            const int n = s.outer_done + jo + 1;
            const bool full = run.refresh == 1 || (run.refresh > 1 && n % run.refresh == 0);
            CK(c, cudaGraphLaunch(full ? s.graph : s.graph_inc, st));
        }
        s.outer_done += nouter;
        return ACU_OK;
    }
    if ((int)c->last_delta.size() != S) c->last_delta.assign(S, 0.0);
    for (int k = 1; k <= nouter; ++k) {
        const int n = s.outer_done + 1;
        run.outer_body(run.refresh == 1 || (run.refresh > 1 && n % run.refresh == 0));
        CKLAUNCH(c);
        const int jo = ++s.outer_done;
        if (run.verbose && (jo % c->opt_print_every == 0 || k == nouter)) {
            std::vector<double> dl(Sp);
            CK(c, cudaMemcpyAsync(dl.data(), s.delta.p, sizeof(double) * Sp, cudaMemcpyDeviceToHost, st));
            CK(c, cudaStreamSynchronize(st));
            for (int i = 0; i < S; ++i) c->last_delta[i] = dl[i];
            if (jo % c->opt_print_every == 0) {
                for (int i = 0; i < S; ++i)
                    printf(" Slice: %12d Loop: %12d delta: %15.8E\n", c->opt_slice_base + i, jo, dl[i]);
                fflush(stdout);
            }
        }
    }
    return ACU_OK;
}

template <typename Real, int V>
int tv_end_v(acu_ctx* c, Real* d_tv)
{
    TvState<Real>& s = tvstate<Real>(c);
    const size_t nimg = (size_t)c->N * c->N * s.G * V;
    if constexpr (V > 1)
        launch_from_lanes<Real, V>(s.uk.template as<Real>(), d_tv, s.S, (size_t)c->N * c->N, c->stream);
    else
        CK(c, cudaMemcpyAsync(d_tv, s.uk.p, sizeof(Real) * nimg, cudaMemcpyDeviceToDevice, c->stream));
    CKLAUNCH(c);
    return ACU_OK;
}

template <typename Real>
int tv_begin(acu_ctx* c, int S, const Real* d_f, int ninner, int ncg, double lambda, double mu, Real* d_fbp)
{
    CKRET(check_ctx(c, S));
    if (S < 1) return set_err(c, ACU_ERR_INVALID, "nslices must be >= 1");
    if (!d_f) return set_err(c, ACU_ERR_INVALID, "null array");
    if (ninner < 0 || ncg < 0) return set_err(c, ACU_ERR_INVALID, "iteration counts must be >= 0");
    if (lambda == 0.0) return set_err(c, ACU_ERR_INVALID, "lambda must be non-zero (shrink threshold 1/lambda)");
    if constexpr (sizeof(Real) == 4) {
        if (pick_lanes(c, S, false) == 4) return tv_begin_v<Real, 4>(c, S, d_f, ninner, ncg, lambda, mu, d_fbp);
    }
    return tv_begin_v<Real, 1>(c, S, d_f, ninner, ncg, lambda, mu, d_fbp);
}

template <typename Real>
int tv_iterate(acu_ctx* c, int nouter)
{
    if (!c) return set_err(nullptr, ACU_ERR_INVALID, "null context");
    TvState<Real>& s = tvstate<Real>(c);
    if (!s.active) return set_err(c, ACU_ERR_INVALID, "no active TV problem: call acu_tv_begin first");
    if (nouter < 0) return set_err(c, ACU_ERR_INVALID, "nouter must be >= 0");
    if (nouter == 0) return ACU_OK;
    if (s.V == 4) {
        if constexpr (sizeof(Real) == 4) return tv_iterate_v<Real, 4>(c, nouter);
    }
    return tv_iterate_v<Real, 1>(c, nouter);
}

template <typename Real>
int tv_end(acu_ctx* c, Real* d_tv)
{
    if (!c) return set_err(nullptr, ACU_ERR_INVALID, "null context");
    TvState<Real>& s = tvstate<Real>(c);
    if (!s.active) return set_err(c, ACU_ERR_INVALID, "no active TV problem: call acu_tv_begin first");
    if (!d_tv) return set_err(c, ACU_ERR_INVALID, "null array");
    if (s.V == 4) {
        if constexpr (sizeof(Real) == 4) return tv_end_v<Real, 4>(c, d_tv);
    }
    return tv_end_v<Real, 1>(c, d_tv);
}

// Slices per device batch of the TV solver: all of S when they fit in the
// device memory that is free (plus what the context already holds for the
// solver), else the largest multiple of 4 that does, capped by
// ACU_OPT_MAX_BATCH.  Slices are independent, so a batch solved in chunks
// gives each slice what one batch gives it.
template <typename Real>
int tv_chunk(acu_ctx* c, int S, bool host_io)
{
    const size_t N = c->N, T = c->T;
    // per slice: 5 sinogram-sized and 10 image-sized solver arrays, the
    // projector's work buffers (transposed copy; pair images for variant 0;
    // line image and ray sums for variant 6), and the host-buffer entry
    // point's device copies of f, tv and fbp
    // the automatic projector choice can differ between the call and a
    // chunk of it: count the larger (pixel-line) buffers then
    const int proj = c->opt_projector == 7 ? 6 : c->opt_projector;
    size_t per = sizeof(Real) * (5 * T * N + 10 * N * N);
    if (c->opt_residual == 2 && c->opt_refresh != 1) per += sizeof(Real) * 2 * N * N;   // bd, dacc
    if (sizeof(Real) == 4)
        per += sizeof(float) * (proj == 0 ? 4 * N * N : proj == 6 ? N * N + T * N : N * N);
    if (host_io) per += sizeof(float) * (T * N + 2 * N * N);
    size_t freeb = 0, totalb = 0;
    if (cudaMemGetInfo(&freeb, &totalb) != cudaSuccess) freeb = 0;
    TvState<Real>& st = tvstate<Real>(c);
    size_t held = c->pairP.n + c->pairPT.n + c->lineL.n + c->lineA.n + c->w_host_in.n + c->w_host_out.n;
    for (const DevBuf* b : {&st.f, &st.fk, &st.ruk, &st.rp, &st.q, &st.uk, &st.ukp, &st.dx, &st.dy, &st.bx, &st.by,
                            &st.rhs, &st.r, &st.p, &st.Ap, &st.tmp, &st.bd, &st.dacc})
        held += b->n;
    const size_t reserve = ((size_t)1 << 30) + totalb / 50;
    const size_t avail = freeb + held > reserve ? freeb + held - reserve : 0;
    long long smax = (long long)(avail / per);
    if (smax >= 4) smax -= smax % 4;
    if (c->opt_max_batch > 0) smax = std::min<long long>(smax, c->opt_max_batch);
    return (int)std::max<long long>(1, std::min<long long>(S, smax));
}

template <typename Real>
int tv_solve(acu_ctx* c, int S, const Real* d_f, int ninner, int nouter, int ncg, Real lambda, Real mu,
             Real* d_tv, Real* d_fbp)
{
    CKRET(check_ctx(c, S));
    if (S == 0) return ACU_OK;
    if (!d_f || !d_tv) return set_err(c, ACU_ERR_INVALID, "null array");
    if (nouter < 0) return set_err(c, ACU_ERR_INVALID, "iteration counts must be >= 0");
    const int chunk = tv_chunk<Real>(c, S, false);
    const size_t nsino = (size_t)c->T * c->N, nimg = (size_t)c->N * c->N;
    for (int s0 = 0; s0 < S; s0 += chunk) {
        const int Sc = std::min(chunk, S - s0);
        CKRET(tv_begin<Real>(c, Sc, d_f + s0 * nsino, ninner, ncg, (double)lambda, (double)mu,
                             d_fbp ? d_fbp + s0 * nimg : nullptr));
        CKRET(tv_iterate<Real>(c, nouter));
        CKRET(tv_end<Real>(c, d_tv + s0 * nimg));
    }
    return ACU_OK;
}

// ---- per-slice comparator: the reference's loop structure on the GPU ---------
// One slice at a time, one kernel per OpenACC region of tv_hpc.F90:162-363,
// direct filter, radon(uk) recomputed where the reference recomputes it, and
// the CG reductions read back to the host every step (the reference computes
// alpha and beta on the host).
int tv_plain(acu_ctx* c, int S, const float* d_f, int ninner, int nouter, int ncg, float lambda, float mu,
             float* d_tv, float* d_fbp)
{
    CKRET(check_ctx(c, S));
    if (S == 0) return ACU_OK;
    if (!d_f || !d_tv) return set_err(c, ACU_ERR_INVALID, "null array");
    if (lambda == 0.0f) return set_err(c, ACU_ERR_INVALID, "lambda must be non-zero (shrink threshold 1/lambda)");
    CKRET(ensure_geom<float>(c));
    const DevGeom<float>& g = c->g32.d;
    TvState<float>& s = c->tv32;
    const int N = c->N, T = c->T;
    const size_t nimg = (size_t)N * N, nsino = (size_t)T * N;
    for (DevBuf* b : {&s.fk, &s.ruk, &s.rp, &s.q}) CK(c, b->ensure(sizeof(float) * nsino));
    for (DevBuf* b : {&s.uk, &s.ukp, &s.dx, &s.dy, &s.bx, &s.by, &s.rhs, &s.r, &s.p, &s.Ap, &s.tmp})
        CK(c, b->ensure(sizeof(float) * nimg));
    const int nblk = (int)std::min<size_t>((nimg + 255) / 256, 512);
    for (DevBuf* b : {&s.rsold, &s.alpha, &s.beta, &s.delta}) CK(c, b->ensure(sizeof(double) * 1));
    CK(c, s.part.ensure(sizeof(double) * (size_t)nblk));
    TvScalars sc{s.rsold.template as<double>(), s.alpha.template as<double>(), s.beta.template as<double>(), s.delta.template as<double>(),
                 s.part.template as<double>(), nblk};
    cudaStream_t st = c->stream;
    using E = TvEw<float, 1>;
    auto F = [](DevBuf& b) { return b.template as<float>(); };
    auto iradon = [&](const float* in, float* out) {
        launch_filter_direct<float, 1>(g, 1, in, F(s.q), st);
        launch_backproject<float, 1>(g, 1, F(s.q), out, st);
    };
    auto radon = [&](const float* in, float* out) { launch_radon<float, 1>(g, 1, in, out, st); };
    double host_scalar;
    c->last_delta.assign(S, 0.0);
    for (int sl = 0; sl < S; ++sl) {
        const float* f = d_f + (size_t)sl * nsino;
        iradon(f, F(s.uk));
        if (d_fbp) CK(c, cudaMemcpyAsync(d_fbp + (size_t)sl * nimg, s.uk.p, sizeof(float) * nimg,
                                         cudaMemcpyDeviceToDevice, st));
        for (DevBuf* b : {&s.dx, &s.dy, &s.bx, &s.by}) CK(c, cudaMemsetAsync(b->p, 0, sizeof(float) * nimg, st));
        CK(c, cudaMemcpyAsync(s.fk.p, f, sizeof(float) * nsino, cudaMemcpyDeviceToDevice, st));
        for (int jo = 1; jo <= nouter; ++jo) {
            for (int ji = 1; ji <= ninner; ++ji) {
                CK(c, cudaMemcpyAsync(s.ukp.p, s.uk.p, sizeof(float) * nimg, cudaMemcpyDeviceToDevice, st));
                iradon(F(s.fk), F(s.tmp));
                E::rhs(N, 1, mu, lambda, F(s.tmp), F(s.dx), F(s.bx), F(s.dy), F(s.by), F(s.rhs), st);
                radon(F(s.uk), F(s.ruk));
                iradon(F(s.ruk), F(s.tmp));
                E::resid(N, 1, mu, lambda, F(s.rhs), F(s.tmp), F(s.uk), F(s.r), F(s.p), sc, st);
                launch_cg_finalize(0, 1, sc, st);
                CK(c, cudaMemcpyAsync(&host_scalar, s.rsold.p, sizeof(double), cudaMemcpyDeviceToHost, st));
                CK(c, cudaStreamSynchronize(st));
                for (int k = 0; k < ncg; ++k) {
                    radon(F(s.p), F(s.rp));
                    iradon(F(s.rp), F(s.tmp));
                    E::apply(N, 1, mu, lambda, F(s.tmp), F(s.p), F(s.Ap), sc, st);
                    launch_cg_finalize(1, 1, sc, st);
                    CK(c, cudaMemcpyAsync(&host_scalar, s.alpha.p, sizeof(double), cudaMemcpyDeviceToHost, st));
                    CK(c, cudaStreamSynchronize(st));
                    E::update(N, 1, F(s.p), F(s.Ap), F(s.uk), F(s.r), sc, st);
                    launch_cg_finalize(2, 1, sc, st);
                    CK(c, cudaMemcpyAsync(&host_scalar, s.beta.p, sizeof(double), cudaMemcpyDeviceToHost, st));
                    CK(c, cudaStreamSynchronize(st));
                    E::pupdate(N, 1, F(s.r), F(s.p), sc, st);
                }
                E::shrink(N, 1, lambda, F(s.uk), F(s.dx), F(s.bx), F(s.dy), F(s.by), F(s.ukp), sc, st);
                launch_cg_finalize(3, 1, sc, st);
            }
            radon(F(s.uk), F(s.ruk));
            E::fk_update(nsino, F(s.fk), f, F(s.ruk), st);
            CKLAUNCH(c);
            if (c->opt_verbose && jo % c->opt_print_every == 0) {
                CK(c, cudaMemcpyAsync(&host_scalar, s.delta.p, sizeof(double), cudaMemcpyDeviceToHost, st));
                CK(c, cudaStreamSynchronize(st));
                printf(" Slice: %12d Loop: %12d delta: %15.8E\n", c->opt_slice_base + sl, jo, host_scalar);
                fflush(stdout);
            }
        }
        CK(c, cudaMemcpyAsync(d_tv + (size_t)sl * nimg, s.uk.p, sizeof(float) * nimg, cudaMemcpyDeviceToDevice, st));
        CK(c, cudaMemcpyAsync(&host_scalar, s.delta.p, sizeof(double), cudaMemcpyDeviceToHost, st));
        CK(c, cudaStreamSynchronize(st));
        c->last_delta[sl] = host_scalar;
    }
    return ACU_OK;
}

int tv_host(acu_ctx* c, bool plain, int S, const float* f, int ninner, int nouter, int ncg, float lambda,
            float mu, float* tv, float* fbp)
{
    CKRET(check_ctx(c, S));
    if (S == 0) return ACU_OK;
    if (!f || !tv) return set_err(c, ACU_ERR_INVALID, "null array");
    // chunks of slices that fit on the device (the per-slice path holds one
    // slice at a time, so only its copies count)
    const int chunk = plain ? std::max(1, std::min(S, c->opt_max_batch > 0 ? c->opt_max_batch : S))
                            : tv_chunk<float>(c, S, true);
    const size_t sino1 = (size_t)c->T * c->N, img1 = (size_t)c->N * c->N;
    for (int s0 = 0; s0 < S; s0 += chunk) {
        const int Sc = std::min(chunk, S - s0);
        const size_t nsino = sino1 * Sc, nimg = img1 * Sc;
        CK(c, c->w_host_in.ensure(sizeof(float) * nsino));
        CK(c, c->w_host_out.ensure(sizeof(float) * nimg * (fbp ? 2 : 1)));
        float* d_tv = c->w_host_out.template as<float>();
        float* d_fbp = fbp ? d_tv + nimg : nullptr;
        CK(c, cudaMemcpyAsync(c->w_host_in.p, f + s0 * sino1, sizeof(float) * nsino, cudaMemcpyHostToDevice,
                              c->stream));
        if (plain)
            CKRET(tv_plain(c, Sc, c->w_host_in.template as<float>(), ninner, nouter, ncg, lambda, mu, d_tv, d_fbp));
        else
            CKRET(tv_solve<float>(c, Sc, c->w_host_in.template as<float>(), ninner, nouter, ncg, lambda, mu, d_tv,
                                  d_fbp));
        CK(c, cudaMemcpyAsync(tv + s0 * img1, d_tv, sizeof(float) * nimg, cudaMemcpyDeviceToHost, c->stream));
        if (fbp)
            CK(c, cudaMemcpyAsync(fbp + s0 * img1, d_fbp, sizeof(float) * nimg, cudaMemcpyDeviceToHost, c->stream));
        CK(c, cudaStreamSynchronize(c->stream));
    }
    return ACU_OK;
}

}  // namespace

// ---- registration-aware TV objective and its gradient (new) -------------------
template <typename Real>
int tv_loss_grad(acu_ctx* c, int S, const Real* d_u, const Real* d_off, const Real* d_y, double lambda, double eps,
                 double* loss_out, Real* d_grad_u, Real* d_grad_off)
{
    CKRET(check_ctx(c, S));
    if (S == 0) return ACU_OK;
    if (!d_u || !d_y || !loss_out) return set_err(c, ACU_ERR_INVALID, "null array");
    if (!(eps > 0.0)) return set_err(c, ACU_ERR_INVALID, "eps must be > 0 (smoothed total variation)");
    CKRET(ensure_geom<Real>(c));
    const DevGeom<Real>& g = geomset<Real>(c).d;
    const int N = c->N, T = c->T;
    const size_t nsino = (size_t)T * N, nimg = (size_t)N * N;
    const int nblk = (int)std::min<size_t>((nimg + 255) / 256, 512);
    CK(c, c->w_in.ensure(sizeof(Real) * nsino * S));      // residual
    CK(c, c->w_out.ensure(sizeof(Real) * nsino * S));     // offset derivative of the projector
    CK(c, c->w_part.ensure(sizeof(double) * ((size_t)2 * nblk * S + 2 * S)));
    Real* r = c->w_in.template as<Real>();
    Real* D = c->w_out.template as<Real>();
    double* part = c->w_part.template as<double>();
    double* sums = part + (size_t)2 * nblk * S;
    cudaStream_t st = c->stream;
    launch_radon_off<Real>(g, S, d_u, d_off, r, st);
    GradEw<Real>::residual(nsino, S, r, d_y, part, nblk, st);
    launch_sum_rows(part, S, nblk, sums, st);
    Real* gu = d_grad_u;
    if (!gu) {
        // loss only: the TV term's kernel still needs a gradient buffer to add
        // into, but the adjoint of the data term is not needed
        CK(c, c->w_q.ensure(sizeof(Real) * nimg * S));
        gu = c->w_q.template as<Real>();
        CK(c, cudaMemsetAsync(gu, 0, sizeof(Real) * nimg * S, st));
    } else {
        launch_radon_adjoint_off<Real>(g, S, r, d_off, gu, st);
    }
    GradEw<Real>::tv_grad(N, S, (Real)lambda, (Real)eps, d_u, gu, part + (size_t)nblk * S, nblk, st);
    launch_sum_rows(part + (size_t)nblk * S, S, nblk, sums + S, st);
    if (d_grad_off) {
        launch_radon_doff<Real>(g, S, d_u, d_off, D, st);
        GradEw<Real>::off_grad(N, T, S, r, D, d_grad_off, st);
    }
    CKLAUNCH(c);
    std::vector<double> h(2 * (size_t)S);
    CK(c, cudaMemcpyAsync(h.data(), sums, sizeof(double) * 2 * S, cudaMemcpyDeviceToHost, st));
    CK(c, cudaStreamSynchronize(st));
    for (int k = 0; k < S; ++k) loss_out[k] = h[k] + h[S + k];
    return ACU_OK;
}

// =============================================================================
// exported C ABI
// =============================================================================
extern "C" {

int acu_ctx_create(acu_ctx** out, int nimage, int ntheta, const float* theta_deg, int wpu)
{
    if (!out) return set_err(nullptr, ACU_ERR_INVALID, "null output pointer");
    *out = nullptr;
    if (nimage < 0 || (nimage > 0 && (nimage < 3 || ntheta < 1 || !theta_deg)))
        return set_err(nullptr, ACU_ERR_INVALID, "invalid geometry: nimage=%d ntheta=%d theta=%p", nimage,
                       ntheta, (const void*)theta_deg);
    if (nimage > 46340)
        return set_err(nullptr, ACU_ERR_INVALID, "nimage=%d exceeds the supported maximum 46340", nimage);
    std::unique_ptr<acu_ctx> c(new (std::nothrow) acu_ctx());
    if (!c) return set_err(nullptr, ACU_ERR_NOMEM, "host allocation failed");
    c->N = nimage;
    c->T = nimage > 0 ? ntheta : 0;
    c->wpu = wpu;
    if (nimage > 0) c->theta.assign(theta_deg, theta_deg + ntheta);
    cudaError_t e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess)
        return set_err(nullptr, ACU_ERR_CUDA, "cudaStreamCreate failed: %s", cudaGetErrorString(e));
    c->stream = nullptr;  // the legacy default stream until acu_set_stream
    *out = c.release();
    return ACU_OK;
}

int acu_ctx_destroy(acu_ctx* c)
{
    if (!c) return ACU_OK;
    cudaStreamSynchronize(c->stream);
    cudaStream_t own = c->own_stream;
    delete c;
    if (own) cudaStreamDestroy(own);
    return ACU_OK;
}

const char* acu_last_error(const acu_ctx* c)
{
    if (c) return c->err.c_str();
    return g_last_error.c_str();
}

int acu_set_stream(acu_ctx* c, void* stream)
{
    if (!c) return set_err(nullptr, ACU_ERR_INVALID, "null context");
    c->stream = (cudaStream_t)stream;  // NULL: the legacy default stream
    return ACU_OK;
}

int acu_set_option(acu_ctx* c, int option, int value)
{
    if (!c) return set_err(nullptr, ACU_ERR_INVALID, "null context");
    switch (option) {
    case ACU_OPT_FILTER:
        if (value != 0 && value != 1) return set_err(c, ACU_ERR_INVALID, "ACU_OPT_FILTER must be 0 or 1");
        c->opt_filter = value;
        return ACU_OK;
    case ACU_OPT_LANES:
        if (value != 0 && value != 1 && value != 4)
            return set_err(c, ACU_ERR_INVALID, "ACU_OPT_LANES must be 0, 1 or 4");
        c->opt_lanes = value;
        return ACU_OK;
    case ACU_OPT_GRAPH: c->opt_graph = value != 0; return ACU_OK;
    case ACU_OPT_VERBOSE: c->opt_verbose = value != 0; return ACU_OK;
    case ACU_OPT_PRINT_EVERY:
        if (value < 1) return set_err(c, ACU_ERR_INVALID, "ACU_OPT_PRINT_EVERY must be >= 1");
        c->opt_print_every = value;
        return ACU_OK;
    case 6: c->opt_slice_base = value; return ACU_OK;
    case 7:
        if (value < 0 || value > 7) return set_err(c, ACU_ERR_INVALID, "ACU_OPT_PROJECTOR must be 0 to 7");
        c->opt_projector = value;
        return ACU_OK;
    case 8:
        if (value != 0 && value != 1) return set_err(c, ACU_ERR_INVALID, "ACU_OPT_POSITIONS must be 0 or 1");
        c->opt_positions = value;
        c->g32.d.exact = value;
        return ACU_OK;
    case 9:
        if (value < 0 || value > 2) return set_err(c, ACU_ERR_INVALID, "ACU_OPT_RESIDUAL must be 0, 1 or 2");
        c->opt_residual = value;
        return ACU_OK;
    case 11:
        if (value < 0) return set_err(c, ACU_ERR_INVALID, "ACU_OPT_RADON_REFRESH must be >= 0");
        c->opt_refresh = value;
        return ACU_OK;
    case 13:
        if (value < 0) return set_err(c, ACU_ERR_INVALID, "ACU_OPT_MAX_BATCH must be >= 0");
        c->opt_max_batch = value;
        return ACU_OK;
    case 10:
        if (value != 0 && value != 1 && value != 2 && value != 4)
            return set_err(c, ACU_ERR_INVALID, "ACU_OPT_BP_GROUPS must be 0, 1, 2 or 4");
        c->g32.d.bp_groups = value;
        return ACU_OK;
    case 12:
        if (value != 0 && value != 1) return set_err(c, ACU_ERR_INVALID, "ACU_OPT_BP_PARAM_TABLE must be 0 or 1");
        c->g32.d.bp_param = value;
        return ACU_OK;
    case 14:
        if (value != 0 && value != 1) return set_err(c, ACU_ERR_INVALID, "ACU_OPT_BP_STAGED must be 0 or 1");
        c->g32.d.bp_tma = value;
        return ACU_OK;

    }
    return set_err(c, ACU_ERR_INVALID, "unknown option %d", option);
}

int acu_get_option(const acu_ctx* c, int option, int* value)
{
    if (!c || !value) return set_err(nullptr, ACU_ERR_INVALID, "null argument");
    switch (option) {
    case ACU_OPT_FILTER: *value = c->opt_filter; return ACU_OK;
    case ACU_OPT_LANES: *value = c->opt_lanes; return ACU_OK;
    case ACU_OPT_GRAPH: *value = c->opt_graph; return ACU_OK;
    case ACU_OPT_VERBOSE: *value = c->opt_verbose; return ACU_OK;
    case ACU_OPT_PRINT_EVERY: *value = c->opt_print_every; return ACU_OK;
    case 6: *value = c->opt_slice_base; return ACU_OK;
    case 7: *value = c->opt_projector; return ACU_OK;
    case 8: *value = c->opt_positions; return ACU_OK;
    case 9: *value = c->opt_residual; return ACU_OK;
    case 11: *value = c->opt_refresh; return ACU_OK;
    case 13: *value = c->opt_max_batch; return ACU_OK;
    case 10: *value = c->g32.d.bp_groups; return ACU_OK;
    case 12: *value = c->g32.d.bp_param; return ACU_OK;
    case 14: *value = c->g32.d.bp_tma; return ACU_OK;
    }
    return set_err(nullptr, ACU_ERR_INVALID, "unknown option %d", option);
}

int acu_iradon(acu_ctx* c, int S, const float* sino, float* img) { return run_op_host(c, OP_IRADON, S, sino, img); }
int acu_radon(acu_ctx* c, int S, const float* img, float* sino) { return run_op_host(c, OP_RADON, S, img, sino); }
int acu_radon_adjoint(acu_ctx* c, int S, const float* sino, float* img)
{
    return run_op_host(c, OP_RADON_ADJ, S, sino, img);
}
int acu_iradon_dev(acu_ctx* c, int S, const float* s, float* i) { return run_op<float>(c, OP_IRADON, S, s, i); }
int acu_radon_dev(acu_ctx* c, int S, const float* i, float* s) { return run_op<float>(c, OP_RADON, S, i, s); }
int acu_radon_adjoint_dev(acu_ctx* c, int S, const float* s, float* i)
{
    return run_op<float>(c, OP_RADON_ADJ, S, s, i);
}
int acu_filter_dev(acu_ctx* c, int S, const float* s, float* o) { return run_op<float>(c, OP_FILTER, S, s, o); }
int acu_backproject_dev(acu_ctx* c, int S, const float* q, float* i)
{
    return run_op<float>(c, OP_BACKPROJECT, S, q, i);
}
int acu_iradon_dev_f64(acu_ctx* c, int S, const double* s, double* i) { return run_op<double>(c, OP_IRADON, S, s, i); }
int acu_radon_dev_f64(acu_ctx* c, int S, const double* i, double* s) { return run_op<double>(c, OP_RADON, S, i, s); }
int acu_radon_adjoint_dev_f64(acu_ctx* c, int S, const double* s, double* i)
{
    return run_op<double>(c, OP_RADON_ADJ, S, s, i);
}
int acu_filter_dev_f64(acu_ctx* c, int S, const double* s, double* o) { return run_op<double>(c, OP_FILTER, S, s, o); }
int acu_backproject_dev_f64(acu_ctx* c, int S, const double* q, double* i)
{
    return run_op<double>(c, OP_BACKPROJECT, S, q, i);
}

int acu_tvopt(acu_ctx* c, int S, const float* f, int ninner, int nouter, int ncg, float lambda, float mu,
              float* tv, float* fbp)
{
    return tv_host(c, false, S, f, ninner, nouter, ncg, lambda, mu, tv, fbp);
}
int acu_tvopt_dev(acu_ctx* c, int S, const float* f, int ninner, int nouter, int ncg, float lambda, float mu,
                  float* tv, float* fbp)
{
    return tv_solve<float>(c, S, f, ninner, nouter, ncg, lambda, mu, tv, fbp);
}
int acu_tvopt_plain(acu_ctx* c, int S, const float* f, int ninner, int nouter, int ncg, float lambda, float mu,
                    float* tv, float* fbp)
{
    return tv_host(c, true, S, f, ninner, nouter, ncg, lambda, mu, tv, fbp);
}
int acu_tvopt_plain_dev(acu_ctx* c, int S, const float* f, int ninner, int nouter, int ncg, float lambda,
                        float mu, float* tv, float* fbp)
{
    return tv_plain(c, S, f, ninner, nouter, ncg, lambda, mu, tv, fbp);
}
int acu_tvopt_dev_f64(acu_ctx* c, int S, const double* f, int ninner, int nouter, int ncg, double lambda,
                      double mu, double* tv, double* fbp)
{
    return tv_solve<double>(c, S, f, ninner, nouter, ncg, lambda, mu, tv, fbp);
}

int acu_tv_begin(acu_ctx* c, int S, const float* d_f, int ninner, int ncg, float lambda, float mu, float* d_fbp)
{
    return tv_begin<float>(c, S, d_f, ninner, ncg, lambda, mu, d_fbp);
}
int acu_tv_iterate(acu_ctx* c, int nouter) { return tv_iterate<float>(c, nouter); }
int acu_tv_end(acu_ctx* c, float* d_tv) { return tv_end<float>(c, d_tv); }

int acu_tv_loss_grad_dev(acu_ctx* c, int S, const float* d_u, const float* d_off, const float* d_y, float lambda,
                         float eps, double* loss, float* d_grad_u, float* d_grad_off)
{
    return tv_loss_grad<float>(c, S, d_u, d_off, d_y, lambda, eps, loss, d_grad_u, d_grad_off);
}
int acu_tv_loss_grad_dev_f64(acu_ctx* c, int S, const double* d_u, const double* d_off, const double* d_y,
                             double lambda, double eps, double* loss, double* d_grad_u, double* d_grad_off)
{
    return tv_loss_grad<double>(c, S, d_u, d_off, d_y, lambda, eps, loss, d_grad_u, d_grad_off);
}

int acu_tv_last_delta(const acu_ctx* c, int S, double* delta)
{
    if (!c || !delta) return set_err(nullptr, ACU_ERR_INVALID, "null argument");
    for (int k = 0; k < S; ++k) delta[k] = k < (int)c->last_delta.size() ? c->last_delta[k] : 0.0;
    return ACU_OK;
}

}  // extern "C"
