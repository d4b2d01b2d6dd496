// solver_common.h -- host-side set-up shared by the single-domain solver (solver.cu) and the
// batch (batch.cu): support checks, launch geometry and the fused pass's argument block.
#pragma once

#include <algorithm>
#include <cmath>
#include <string>

#include "armon_gb300.h"
#include "host_common.h"
#include "sweep.cuh"

namespace armon {

// Cells the fused pass reads beyond the real ones along its axis: the reference's flux domain
// (src/ranges.cpp:14-30) reaches one cell further than min_ghosts except for GAD + second order.
inline int stencil_reach(const armon_params* p)
{
    return 2 + (p->scheme == ARMON_GAD) + (p->projection == ARMON_EULER_2ND);
}

inline bool is_pow2(double x)
{
    int e;
    double m = std::frexp(x, &e);
    return x > 0 && m == 0.5;
}

// Lines per block for an axis of nlines lines: the whole block when there are that many lines,
// else the lines rounded up to a multiple of 32 that divides the block, which then holds
// block / lpb segments of the same lines.
inline int lines_per_block(int nlines, int block)
{
    int l = std::max(32, (nlines + 31) / 32 * 32);
    if (l >= block) return block;
    while (block % l != 0) l += 32;
    return l;
}

// The blocks of one axis for a given segment length.
struct AxisTiling {
    int seg_len, nseg, nlb, lpb, spb, blocks;
};

inline AxisTiling axis_tiling(int n, int nlines, int block, int seg_len)
{
    AxisTiling t;
    t.lpb = lines_per_block(nlines, block);
    t.spb = block / t.lpb;
    t.nlb = std::max(1, (nlines + t.lpb - 1) / t.lpb);
    t.seg_len = std::max(1, std::min(seg_len, n));
    t.nseg = (n + t.seg_len - 1) / t.seg_len;
    t.blocks = t.nlb * ((t.nseg + t.spb - 1) / t.spb);
    return t;
}

// Segments along the axis of one domain that has the GPU to itself: minimise (most threads on one
// SM, in units of 128) x (cells a thread walks, halo included) over the segment count, with
// segments of at least 16 cells.  forced > 0 imposes the segment length.
inline AxisTiling choose_segments(int n, int nlines, int block, int halo, int sms, int forced)
{
    if (forced > 0) return axis_tiling(n, nlines, block, forced);
    double best = 1e300;
    int best_seg = n;
    for (int ns = 1; ns <= std::max(1, n / 16); ns++) {
        int sl = (n + ns - 1) / ns;
        if ((int64_t)sl * (ns - 1) >= n) continue;
        AxisTiling t = axis_tiling(n, nlines, block, sl);
        double per_sm = std::ceil(double(t.blocks) * block / (128.0 * sms));
        double cost = per_sm * (sl + 1.2 * halo);
        if (cost < best - 1e-9) { best = cost; best_seg = sl; }
    }
    return axis_tiling(n, nlines, block, best_seg);
}

inline int check_supported(const armon_params* p)
{
    if (!armon_params_check(p)) { set_error("invalid parameters (Params::check)"); return ARMON_ERR_PARAMS; }
    if (p->test == ARMON_BIZARRIUM) {
        set_error("the fused solver implements the perfect-gas EOS only (Bizarrium is served by the stage kernels)");
        return ARMON_ERR_UNSUPPORTED;
    }
    if (p->projection == ARMON_PROJ_NONE) { set_error("projection None is not supported"); return ARMON_ERR_UNSUPPORTED; }
    const int halo = stencil_reach(p);
    if (p->nb_ghosts < halo) {
        set_error("the fused solver needs nb_ghosts >= " + std::to_string(halo) + " for this scheme");
        return ARMON_ERR_UNSUPPORTED;
    }
    if (p->nx < p->stencil_width || p->ny < p->stencil_width) {
        set_error("the fused solver needs nx, ny >= stencil_width (mirrored bands may not overlap)");
        return ARMON_ERR_UNSUPPORTED;
    }
    return ARMON_OK;
}

inline StepConfig make_step_config(const armon_params& p)
{
    StepConfig c{};
    c.cfl = p.cfl;
    c.Dt = p.Dt;
    c.max_time = p.max_time;
    c.dt_dx = p.domain_size[0] / double(p.nx);
    c.dt_dy = p.domain_size[1] / double(p.ny);
    c.cst_dt = p.cst_dt;
    c.dt_on_even_cycles = p.dt_on_even_cycles;
    c.max_cycles = p.max_cycles;
    c.splitting = p.axis_splitting;
    return c;
}

// The state buffers of one domain: set 0 and set 1 of (rho, umat, vmat, Emat), and p, c, g.
template <class T>
struct DomainBuffers {
    T* set[2][4];
    T *pmat, *cmat, *gmat;
};

// Fills the argument block of the fused pass for one domain; returns the blocks it needs (the
// larger of its two axes).  forced_seg[axis] > 0 imposes that axis's segment length.
template <class T>
int make_sweep_args(const armon_params& p, int npass, int block, int sms, const int forced_seg[2],
                    const DomainBuffers<T>& b, StepState* state, double* partials, int write_eos, int reuse,
                    SweepArgs<T>& a)
{
    const int halo = stencil_reach(&p);
    for (int axis = 0; axis < 2; axis++) {
        AxisGeom<T>& g = a.geom[axis];
        g.n = axis == 0 ? p.nx : p.ny;
        g.nlines = axis == 0 ? p.ny : p.nx;
        g.s = axis == 0 ? 1 : p.row_length;
        g.lstride = axis == 0 ? p.row_length : 1;
        const AxisTiling t = choose_segments(g.n, g.nlines, block, halo, sms, forced_seg[axis]);
        g.seg_len = t.seg_len;
        g.nseg = t.nseg;
        g.nlb = t.nlb;
        g.lpb = t.lpb;
        g.spb = t.spb;
        g.blocks = t.blocks;
        // BC sign factors: X pass low = Left, high = Right; Y pass low = Bottom (y = -1), high = Top.
        double lo_u, lo_v, hi_u, hi_v;
        armon_boundary_factors(p.test, axis == 0 ? ARMON_LEFT : ARMON_BOTTOM, &lo_u, &lo_v);
        armon_boundary_factors(p.test, axis == 0 ? ARMON_RIGHT : ARMON_TOP, &hi_u, &hi_v);
        // axis velocity: umat in X, vmat in Y
        g.fa_lo = T(axis == 0 ? lo_u : lo_v);
        g.fo_lo = T(axis == 0 ? lo_v : lo_u);
        g.fa_hi = T(axis == 0 ? hi_u : hi_v);
        g.fo_hi = T(axis == 0 ? hi_v : hi_u);
        const double f[4] = {double(g.fa_lo), double(g.fo_lo), double(g.fa_hi), double(g.fo_hi)};
        g.fneg = 0;
        g.f_unit = 1;
        for (int k = 0; k < 4; k++) {
            if (f[k] == -1.0) g.fneg |= 1u << k;
            else if (f[k] != 1.0) g.f_unit = 0;
        }
        double dx = (axis == 0 ? p.domain_size[0] / double(p.nx) : p.domain_size[1] / double(p.ny));
        g.dx = T(dx);
        g.dx_pow2 = is_pow2(double(g.dx)) ? 1 : 0;
        g.inv_dx = g.dx_pow2 ? T(1.0 / double(g.dx)) : T(0);
        g.dx_log2 = g.dx_pow2 ? std::ilogb(double(g.dx)) : 0;
        g.order = nullptr;
        g.cost = nullptr;
        g.face_order = nullptr;
        g.face_cost = nullptr;
    }
    a.origin = (int64_t)p.nb_ghosts * p.row_length + p.nb_ghosts;
    a.sw = p.stencil_width;
    a.limiter = p.limiter;
    a.npass = npass;
    a.pass = 0;
    a.write_eos = write_eos;
    a.reuse = reuse;
    a.gamma = T(1.4);   // update_EOS hard-codes gamma = 1.4 (src/armon_2D.cpp:94)
    for (int k = 0; k < 4; k++) { a.buf[0][k] = b.set[0][k]; a.buf[1][k] = b.set[1][k]; }
    a.pmat = b.pmat;
    a.cmat = b.cmat;
    a.gmat = b.gmat;
    a.state = state;
    a.cfg = make_step_config(p);
    a.partials = partials;
    a.faces = nullptr;
    a.face_stride = 0;
    return std::max(a.geom[0].blocks, a.geom[1].blocks);
}

}  // namespace armon
