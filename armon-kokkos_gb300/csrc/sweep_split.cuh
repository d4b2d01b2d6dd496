// sweep_split.cuh -- one axis pass as two launches: the face half (EOS, Godunov and GAD fluxes)
// stores u*, p* and p* u* of every face in a face buffer, and the cell half (Lagrange update,
// advection, projection, dt_CFL, cycle commit) reads them back.
//
// Same stage functions, same expression order and same operands as the fused pass (sweep.cuh),
// so the results are the same bits; only where the flux values live between the stages changes.
// Each half keeps far fewer values alive than the fused pipeline, so more warps fit on an SM.
//
// Face buffer: three arrays (u*, p*, p* u*) of face_stride values; face f of line l (f in [-2, n+2])
// at (f + 2) * nlines + l, so that the 32 lines of a warp touch 32 consecutive values in either
// pass.  The cell half of segment [a0, b0) reads faces [a0 - r, b0 + r], r = 2 for the second-order
// projection and 1 for the first; the face half of the segment writes the faces it owns, [a0, b0)
// plus [-r, 0) for the first segment and [n, n + r] for the last.  A face's flux reads cells f - 2
// to f + 1 (GAD) or f - 1 to f (Godunov), so the face half reads positions -(r + 2) to n + r + 1
// (GAD) or -(r + 1) to n + r: never more than the 2 + GAD + second-order ghosts the solver
// requires.
#pragma once

#include "sweep.cuh"

namespace armon {

template <class T>
__device__ __forceinline__ int64_t face_index(const AxisGeom<T>& g, int f, int line)
{
    return (int64_t)(f + 2) * g.nlines + line;
}

// Which line and segment a thread of block `blk` works on (the unit order of `order`, if any).
struct UnitPos {
    int u, line, seg;
    bool has_unit, active;
};

template <class T>
__device__ __forceinline__ UnitPos unit_position(const AxisGeom<T>& g, const uint32_t* order, int blk)
{
    UnitPos p;
    p.has_unit = blk < g.blocks;
    p.u = (order != nullptr && p.has_unit) ? (int)__ldg(&order[blk]) : blk;
    const int lb = p.u % max(g.nlb, 1);
    const int sb = p.u / max(g.nlb, 1);
    const int sub = (int)threadIdx.x / g.lpb;
    p.seg = sb * g.spb + sub;
    p.line = lb * g.lpb + (int)threadIdx.x % g.lpb;
    p.active = p.has_unit && p.line < g.nlines && p.seg < g.nseg && sub < g.spb;
    return p;
}

// The cell of the line that position tt reads: itself, or the real cell it mirrors.
template <class T>
__device__ __forceinline__ int position_source(const AxisGeom<T>&, int n, int sw, int tt)
{
    if (tt < 0 && tt >= -sw) return -1 - tt;
    if (tt >= n && tt < n + sw) return 2 * n - 1 - tt;
    return tt;
}

// The cell at position tt of a line: the real cell itself, a mirror of a real cell (side 1: low
// side, 2: high side) with the boundary's sign factors, or an untouched ghost (stale: true).
template <class T>
__device__ __forceinline__ bool load_position(const AxisGeom<T>& g, int n, int sw, int64_t base, int tt,
                                              const T* __restrict__ rho_in, const T* __restrict__ ua_in,
                                              const T* __restrict__ uo_in, const T* __restrict__ E_in,
                                              CellIn<T>& c, int& m, int64_t& idx)
{
    m = tt;
    int side = 0;
    bool stale = false;
    if (tt < 0) {
        if (tt >= -sw) { m = -1 - tt; side = 1; } else stale = true;
    } else if (tt >= n) {
        if (tt < n + sw) { m = 2 * n - 1 - tt; side = 2; } else stale = true;
    }
    idx = base + (int64_t)m * g.s;
    c.rho = rho_in[idx];
    c.ua = ua_in[idx];
    c.uo = uo_in[idx];
    c.E = E_in[idx];
    if (side) {
        // boundary_conditions: umat * u_factor, vmat * v_factor (+-1: a sign flip)
        if (g.f_unit) {
            const uint32_t sh = side == 1 ? 0 : 2;
            c.ua = qneg_if(c.ua, (g.fneg >> sh) & 1u);
            c.uo = qneg_if(c.uo, (g.fneg >> (sh + 1)) & 1u);
        } else {
            c.ua = c.ua * (side == 1 ? g.fa_lo : g.fa_hi);
            c.uo = c.uo * (side == 1 ? g.fo_lo : g.fo_hi);
        }
    }
    return stale;
}

// ---- the face half: EOS of the cells, Godunov state of each face, GAD (or Godunov) flux ----
template <class T, int SCHEME, int PROJ, bool LAST, int MULS = ARMON_SOFT_MUL, int ADDS = 0>
__device__ __forceinline__ void sweep_faces(const SweepArgs<T>& A, const int blk, const int pass)
{
    constexpr bool kGAD = SCHEME == 1;
    constexpr int R = PROJ == 2 ? 2 : 1;   // the cell half reads faces a0 - R .. b0 + R
    const StepState st = *A.state;
    const CycleDt cd = cycle_time_step(st, A.cfg);
    if (!cd.run || cd.invalid) return;   // the cell half reports an invalid dt

    int axis;
    double factor;
    split_axis(A.cfg.splitting, st.cycle, pass, &axis, &factor);
    const AxisGeom<T>& g = A.geom[axis];
    const T dt = T(cd.current * factor);
    const int src = (int)(((int64_t)st.cycle * A.npass + pass + st.buf_base) & 1);
    T* const* in = A.buf[src];
    const T* __restrict__ rho_in = in[0];
    const T* __restrict__ ua_in = in[axis == 0 ? 1 : 2];
    const T* __restrict__ uo_in = in[axis == 0 ? 2 : 1];
    const T* __restrict__ E_in = in[3];
    const T gamma_m1 = A.gamma - 1;

    const UnitPos P = unit_position(g, g.face_order, blk);
    const long long clock_start = clock64();
    if (P.active) {
        const int n = g.n, sw = A.sw;
        const int a0 = P.seg * g.seg_len;
        const int b0 = min(n, a0 + g.seg_len);
        const int fs = a0 == 0 ? -R : a0, fe = b0 == n ? n + R + 1 : b0;   // faces [fs, fe) are this segment's
        const int64_t base = A.origin + (int64_t)P.line * g.lstride;
        const int t0 = kGAD ? fs - 2 : fs - 1, t1 = kGAD ? fe : fe - 1;
        T* const us_out = A.faces;
        T* const ps_out = A.faces + A.face_stride;
        T* const psus_out = A.faces + 2 * A.face_stride;

        CellIn<T> C0{}, C1{}, C2{};
        God<T> G1{}, G2{};
        GadDiff<T> D0{}, D1{}, D2{};
        constexpr int LAGF = kGAD ? 1 : 0;          // step t stores face t - LAGF
        const auto prepare = [&](CellIn<T>& c) {
            eos(c, A.gamma, gamma_m1);
            c.rc = qmul<1>(c.rho, c.c);
            c.rcu = qmul<1>(c.rc, c.ua);
            c.dm = mul_dx(c.rho, g);
        };
        const auto flux = [&](const God<T>& Gc, const GadDiff<T>& Dm1, const GadDiff<T>& D0_, const GadDiff<T>& Dp1,
                              T dm_l, T dm_r, const God<T>& Gr, T (&o)[3]) {
            Flux<T> f;
            if (kGAD) {
                f = gad<T, MULS, ADDS>(Gc, Dm1, D0_, Dp1, dm_l, dm_r, A.limiter, dt);
            } else {
                f.us = Gr.us; f.ps = Gr.ps;
            }
            o[0] = f.us;
            o[1] = f.ps;
            o[2] = qmul<4>(f.ps, f.us);
        };
        const auto store_face = [&](int f, const T (&o)[3]) {
            const int64_t fi = face_index(g, f, P.line);
            us_out[fi] = o[0];
            ps_out[fi] = o[1];
            psus_out[fi] = o[2];
        };
        // the registers after a step whose window held only cells equal to u (sweep.cuh: exact reuse)
        const auto uniform_march = [&](const CellIn<T>& c) {
            C0 = c; C1 = c; C2 = c;
            G2 = godunov<T, ADDS>(c, c); G1 = G2;
            if (kGAD) { D2 = gad_diff<T, ADDS>(G2, c, c); D1 = D2; D0 = D2; }
        };
        const auto pcg = [&](int tt, const CellIn<T>& c) {
            if (tt >= a0 && tt < b0 && writes_eos<LAST>(A)) {   // owned real cell: what update_EOS stores
                const int64_t idx = base + (int64_t)tt * g.s;
                A.pmat[idx] = c.p;
                A.cmat[idx] = c.c;
                A.gmat[idx] = (1 + A.gamma) / 2;
            }
        };

        // Exact reuse (sweep.cuh): a face whose flux window (cells f - 2 .. f + 1 with GAD, f - 1 .. f
        // with Godunov) lies in a run of cells equal to u gets the run's uniform flux; such positions
        // are streamed, kReuseBatch at a time, and the march restarts from uniform_march(u).
        const bool reuse = A.reuse != 0;
        constexpr int kEnter = kGAD ? 3 : 1;
        constexpr int kReuseBatch = reuse_batch<T>();
        // the run's state (rho, ua, uo, E, p, c) and uniform face (u*, p*, p* u*), kept in this
        // thread's slot of shared memory while the march computes
        __shared__ T run_slot[9][128];
        const int tid = threadIdx.x;
        const auto keep_run = [&](const CellIn<T>& c, const T (&o)[3]) {
            run_slot[0][tid] = c.rho; run_slot[1][tid] = c.ua; run_slot[2][tid] = c.uo; run_slot[3][tid] = c.E;
            run_slot[4][tid] = c.p; run_slot[5][tid] = c.c;
            run_slot[6][tid] = o[0]; run_slot[7][tid] = o[1]; run_slot[8][tid] = o[2];
        };
        const auto run_cell = [&]() {
            CellIn<T> u;
            u.rho = run_slot[0][tid]; u.ua = run_slot[1][tid]; u.uo = run_slot[2][tid]; u.E = run_slot[3][tid];
            u.p = run_slot[4][tid]; u.c = run_slot[5][tid];
            return u;
        };
        // streams the positions from t on whose cell equals the run's; returns the first that differs
        const auto stream = [&](int t) -> int {
            const CellIn<T> u = run_cell();
            const T u_out[3] = {run_slot[6][tid], run_slot[7][tid], run_slot[8][tid]};
            const bool pcg_out = writes_eos<LAST>(A);
            while (t <= t1) {
                const int nb = min(kReuseBatch, t1 - t + 1);
                bool same[kReuseBatch];
                if (nb == kReuseBatch && t >= a0 && t + kReuseBatch <= b0 && t >= t0 + 1 + 2 * LAGF) {
                    // a batch of real cells the segment owns, each ending a face to store: no mirror,
                    // no ghost, and the stores need no per-position test
#pragma unroll
                    for (int q = 0; q < kReuseBatch; q++) {
                        const int64_t idx = base + (int64_t)(t + q) * g.s;
                        CellIn<T> c;
                        c.rho = rho_in[idx]; c.ua = ua_in[idx]; c.uo = uo_in[idx]; c.E = E_in[idx];
                        same[q] = same_state(c, u);
                    }
                    bool all = true;
#pragma unroll
                    for (int q = 0; q < kReuseBatch; q++) all = all && same[q];
                    if (all) {
#pragma unroll
                        for (int q = 0; q < kReuseBatch; q++) {
                            if (pcg_out) {
                                const int64_t idx = base + (int64_t)(t + q) * g.s;
                                A.pmat[idx] = u.p;
                                A.cmat[idx] = u.c;
                                A.gmat[idx] = (1 + A.gamma) / 2;
                            }
                            store_face(t + q - LAGF, u_out);
                        }
                        t += kReuseBatch;
                        continue;
                    }
                } else {
#pragma unroll
                    for (int q = 0; q < kReuseBatch; q++) {
                        same[q] = false;
                        if (q < nb) {
                            CellIn<T> c;
                            int m;
                            int64_t idx;
                            const bool stale = load_position(g, n, sw, base, t + q, rho_in, ua_in, uo_in, E_in, c, m, idx);
                            same[q] = !stale && same_state(c, u);
                        }
                    }
                }
                // the lines of the batches that follow, positions the march reads (at most t1)
#pragma unroll
                for (int q = 0; q < kReusePrefetch * kReuseBatch; q++) {
                    const int tp = t + nb + q;
                    if (tp <= t1) {
                        const int64_t idx = base + (int64_t)position_source(g, n, sw, tp) * g.s;
                        prefetch_l2(rho_in + idx); prefetch_l2(ua_in + idx); prefetch_l2(uo_in + idx); prefetch_l2(E_in + idx);
                    }
                }
                int k = 0;
#pragma unroll
                for (int q = 0; q < kReuseBatch; q++) k += (k == q && same[q]) ? 1 : 0;
                for (int q = 0; q < k; q++) {
                    pcg(t + q, u);
                    if (t + q >= t0 + 1 + 2 * LAGF) store_face(t + q - LAGF, u_out);
                }
                t += k;
                if (k < nb) break;
            }
            return t;
        };
        const auto restart = [&]() {
            CellIn<T> u = run_cell();
            prepare(u);
            uniform_march(u);
        };

        // the segment opens a run only when cells t0 .. t0 + kEnter, the first face's window, are
        // equal (loaded together and compared before the run's evaluation is spent)
        const auto opens_run = [&](const CellIn<T>& c) {
            bool same[kEnter];
#pragma unroll
            for (int q = 0; q < kEnter; q++) {
                CellIn<T> cq;
                int mq;
                int64_t iq;
                const bool stale = load_position(g, n, sw, base, t0 + 1 + q, rho_in, ua_in, uo_in, E_in, cq, mq, iq);
                same[q] = !stale && same_state(cq, c);
            }
            bool all = true;
#pragma unroll
            for (int q = 0; q < kEnter; q++) all = all && same[q];
            return all;
        };
        int t = t0;
        int run = 0;
        if (reuse) {
            CellIn<T> c;
            int m;
            int64_t idx;
            if (!load_position(g, n, sw, base, t0, rho_in, ua_in, uo_in, E_in, c, m, idx) && opens_run(c)) {
                prepare(c);
                uniform_march(c);
                T o[3];
                flux(G1, D0, D1, D2, C0.dm, C1.dm, G2, o);
                keep_run(c, o);
                t = stream(t0 + 1);
                if (t <= t1) restart();
            }
        }
#pragma unroll 1
        for (; t <= t1; ++t) {
            {
                CellIn<T> c;
                int m;
                int64_t idx;
                const bool stale = load_position(g, n, sw, base, t, rho_in, ua_in, uo_in, E_in, c, m, idx);
                if (reuse) run = stale ? -1 : (t > t0 && same_state(c, C2)) ? run + 1 : 0;
                C0 = C1; C1 = C2;
                if (stale) {
                    c.p = A.pmat[idx];
                    c.c = A.cmat[idx];
                    c.rc = qmul<1>(c.rho, c.c);
                    c.rcu = qmul<1>(c.rc, c.ua);
                    c.dm = mul_dx(c.rho, g);
                } else {
                    prepare(c);
                    if (m == t) pcg(t, c);
                }
                C2 = c;
            }
            if (t >= t0 + 1) {
                G1 = G2;
                G2 = godunov<T, ADDS>(C1, C2);
                if (kGAD) { D0 = D1; D1 = D2; D2 = gad_diff<T, ADDS>(G2, C1, C2); }
            }
            if (t >= t0 + 1 + 2 * LAGF) {
                T o[3];
                flux(G1, D0, D1, D2, C0.dm, C1.dm, G2, o);
                store_face(t - LAGF, o);
                if (reuse && run >= kEnter) {
                    // the window of this face lies in a run of equal cells: stream the run
                    keep_run(C2, o);
                    const int tn = stream(t + 1);
                    if (tn > t1) break;
                    restart();
                    run = 0;
                    t = tn - 1;          // the loop's increment brings it to tn
                }
            }
        }
    }
    if (g.face_cost != nullptr) {
        __syncthreads();
        if (threadIdx.x == 0 && P.has_unit)
            g.face_cost[P.u] = (uint32_t)min(clock64() - clock_start, (long long)0xFFFFFFFFu);
    }
}

// ---- the cell half: Lagrange update, advection, projection; on the last pass dt_CFL + commit ----
template <class T, int SCHEME, int PROJ, bool LAST>
__device__ __forceinline__ void sweep_cells(const SweepArgs<T>& A, const int blk, const int nblk, const int pass)
{
    constexpr bool kE2 = PROJ == 2;
    constexpr int LAG_A = kE2 ? 2 : 1;   // at iteration t: face t read, Lagrange cell t - 1, advection face t - LAG_A

    const StepState st = *A.state;
    const CycleDt cd = cycle_time_step(st, A.cfg);
    if (!cd.run) return;
    if (cd.invalid) {
        if (LAST && blk == 0 && threadIdx.x == 0) A.state->status = STATUS_INVALID_DT;
        return;
    }

    int axis;
    double factor;
    split_axis(A.cfg.splitting, st.cycle, pass, &axis, &factor);
    const AxisGeom<T>& g = A.geom[axis];
    const T dt = T(cd.current * factor);
    const T dx = g.dx;
    const int src = (int)(((int64_t)st.cycle * A.npass + pass + st.buf_base) & 1);
    T* const* in = A.buf[src];
    T* const* out = A.buf[src ^ 1];
    const T* __restrict__ rho_in = in[0];
    const T* __restrict__ ua_in = in[axis == 0 ? 1 : 2];
    const T* __restrict__ uo_in = in[axis == 0 ? 2 : 1];
    const T* __restrict__ E_in = in[3];

    DtAcc acc;
    acc.init();

    const UnitPos P = unit_position(g, g.order, blk);
    const long long clock_start = clock64();
    if (P.active) {
        const int n = g.n, sw = A.sw;
        const int a0 = P.seg * g.seg_len;
        const int b0 = min(n, a0 + g.seg_len);
        const int64_t base = A.origin + (int64_t)P.line * g.lstride;
        const int64_t s = g.s;
        const int t0 = a0 - LAG_A, t1 = b0 + LAG_A;
        const T* __restrict__ us_in = A.faces;
        const T* __restrict__ ps_in = A.faces + A.face_stride;
        const T* __restrict__ psus_in = A.faces + 2 * A.face_stride;

        Flux<T> F1{}, F2{}, F3{}, F4{};
        Lag<T> L1{}, L2{}, L3{};
        Adv<T> d01{}, d12{}, d23{};
        T s01{}, s12{}, s23{};
        Adv<T> A0{}, A1{};

        // The inputs of step t ("unit" t): face t and the state of cell t - 1.
        struct Unit { Flux<T> f; CellIn<T> c; };
        const auto load_face = [&](int tt, Flux<T>& f) {
            const int64_t fi = face_index(g, tt, P.line);
            f.us = us_in[fi];
            f.ps = ps_in[fi];
            f.psus = psus_in[fi];
        };
        const auto load_cell = [&](int tt, CellIn<T>& c) {
            int m;
            int64_t idx;
            load_position(g, n, sw, base, tt, rho_in, ua_in, uo_in, E_in, c, m, idx);
        };
        const auto same_unit = [&](const Flux<T>& f, const CellIn<T>& c, const Unit& v) {
            return same_bits(f.us, v.f.us) & same_bits(f.ps, v.f.ps) & same_bits(f.psus, v.f.psus) & same_state(c, v.c);
        };
        const auto lagrange_of = [&](CellIn<T> c, const Flux<T>& fl, const Flux<T>& fr) {
            c.dm = mul_dx(c.rho, g);
            c.c = T(0);
            return lagrange(c, fl, fr, dt, dx);
        };
        // src/kernels/euler_projection.cpp:36-46 for a cell Lc between advection fluxes a0 and a1
        const auto project = [&](const Lag<T>& Lc, const Adv<T>& a0_, const Adv<T>& a1_, T (&o)[4]) {
            T dXr = qmul<7>(Lc.W, Lc.rho);
            o[0] = div_dx(dXr - (a1_.r - a0_.r), g);
            T tmp_ra = div_dx(qmul<7>(dXr, Lc.ua) - (a1_.ra - a0_.ra), g);
            T tmp_ro = div_dx(qmul<7>(dXr, Lc.uo) - (a1_.ro - a0_.ro), g);
            T tmp_rE = div_dx(qmul<7>(dXr, Lc.E) - (a1_.rE - a0_.rE), g);
            const auto inv_rho = qrecip_at<8>(o[0]);
            o[1] = qdiv_at<8>(tmp_ra, inv_rho);
            o[2] = qdiv_at<8>(tmp_ro, inv_rho);
            o[3] = qdiv_at<8>(tmp_rE, inv_rho);
        };
        const auto store_out = [&](int mm, const T (&o)[4]) {
            const int64_t idx = base + (int64_t)mm * s;
            out[0][idx] = o[0];
            out[axis == 0 ? 1 : 2][idx] = o[1];
            out[axis == 0 ? 2 : 1][idx] = o[2];
            out[3][idx] = o[3];
        };
        // dt_CFL of the state after this pass, with c from this pass's EOS (the face half stored it
        // for every real cell)
        const auto add_dt = [&](int mm, const T (&o)[4]) {
            const T c = A.cmat[base + (int64_t)mm * s];
            if (axis == 0) acc.add(o[1], o[2], c);
            else acc.add(o[2], o[1], c);
        };
        // the registers after a step whose window held only units equal to v (sweep.cuh: exact reuse)
        const auto uniform_march = [&](const Unit& v) {
            Flux<T> f = v.f;
            f.dtus = qmul<4>(dt, f.us);
            F1 = f; F2 = f; F3 = f; F4 = f;
            L3 = lagrange_of(v.c, f, f); L2 = L3; L1 = L3;
            if (kE2) {
                d23 = lag_diff(L3, L3); d12 = d23; d01 = d23;
                s23 = L3.W + L3.W; s12 = s23; s01 = s23;
            }
            A1 = kE2 ? advect2(f, f, f, L3, L3, d23, d23, d23, s23, s23, s23, dx) : advect1(f, L3, L3);
            A0 = A1;
        };

        // Exact reuse (sweep.cuh): the projection of cell t - LAG_A - 1 depends on units
        // t - 2 LAG_A - 1 .. t; positions whose window lies in a run of units equal to v are
        // streamed, kReuseBatch at a time, and the march restarts from uniform_march(v).  The
        // segment's run starts at unit t0 + 1 (face t0 + 1, cell t0) when face t0 equals face t0 + 1
        // (the march's first Lagrange cell is t0, which reads faces t0 and t0 + 1).
        const bool reuse = A.reuse != 0;
        constexpr int kEnter = 2 * LAG_A + 1;
        constexpr int kReuseBatch = reuse_batch<T>();
        // the run's unit (u*, p*, p* u*, rho, ua, uo, E) and uniform results (rho, ua, uo, E) in this
        // thread's slot of shared memory while the march computes; slots 11..14 hold the cell of the
        // previous step, which the next step compares with its own
        __shared__ T run_slot[15][128];
        const int tid = threadIdx.x;
        const auto keep_run = [&](const Flux<T>& f, const T (&o)[4]) {
            run_slot[0][tid] = f.us; run_slot[1][tid] = f.ps; run_slot[2][tid] = f.psus;
            for (int q = 0; q < 4; q++) run_slot[3 + q][tid] = run_slot[11 + q][tid];
            for (int q = 0; q < 4; q++) run_slot[7 + q][tid] = o[q];
        };
        const auto run_unit = [&]() {
            Unit v;
            v.f.us = run_slot[0][tid]; v.f.ps = run_slot[1][tid]; v.f.psus = run_slot[2][tid];
            v.c.rho = run_slot[3][tid]; v.c.ua = run_slot[4][tid]; v.c.uo = run_slot[5][tid]; v.c.E = run_slot[6][tid];
            return v;
        };
        bool counted = false;
        // streams the positions from t on whose unit equals the run's; returns the first that differs
        const auto stream = [&](int t) -> int {
            const Unit v = run_unit();
            const T v_out[4] = {run_slot[7][tid], run_slot[8][tid], run_slot[9][tid], run_slot[10][tid]};
            while (t <= t1) {
                const int nb = min(kReuseBatch, t1 - t + 1);
                bool same[kReuseBatch];
                if (nb == kReuseBatch && t - 1 >= 0 && t + kReuseBatch - 1 <= n && t - LAG_A - 1 >= a0) {
                    // units of real cells, each with a result to store: no mirror, no per-position test
#pragma unroll
                    for (int q = 0; q < kReuseBatch; q++) {
                        Flux<T> f;
                        CellIn<T> c;
                        load_face(t + q, f);
                        const int64_t idx = base + (int64_t)(t + q - 1) * s;
                        c.rho = rho_in[idx]; c.ua = ua_in[idx]; c.uo = uo_in[idx]; c.E = E_in[idx];
                        same[q] = same_unit(f, c, v);
                    }
                    bool all = true;
#pragma unroll
                    for (int q = 0; q < kReuseBatch; q++) all = all && same[q];
                    if (all) {
#pragma unroll
                        for (int q = 0; q < kReuseBatch; q++) store_out(t + q - LAG_A - 1, v_out);
                        if (LAST && !counted) { add_dt(t - LAG_A - 1, v_out); counted = true; }
                        t += kReuseBatch;
                        continue;
                    }
                } else {
#pragma unroll
                    for (int q = 0; q < kReuseBatch; q++) {
                        same[q] = false;
                        if (q < nb) {
                            Flux<T> f;
                            CellIn<T> c;
                            load_face(t + q, f);
                            load_cell(t + q - 1, c);
                            same[q] = same_unit(f, c, v);
                        }
                    }
                }
                // the lines of the batches that follow, positions the march reads (at most t1)
#pragma unroll
                for (int q = 0; q < kReusePrefetch * kReuseBatch; q++) {
                    const int tp = t + nb + q;
                    if (tp <= t1) {
                        const int64_t fi = face_index(g, tp, P.line);
                        prefetch_l2(us_in + fi); prefetch_l2(ps_in + fi); prefetch_l2(psus_in + fi);
                        const int64_t idx = base + (int64_t)position_source(g, n, sw, tp - 1) * g.s;
                        prefetch_l2(rho_in + idx); prefetch_l2(ua_in + idx); prefetch_l2(uo_in + idx); prefetch_l2(E_in + idx);
                    }
                }
                int k = 0;
#pragma unroll
                for (int q = 0; q < kReuseBatch; q++) k += (k == q && same[q]) ? 1 : 0;
                for (int q = 0; q < k; q++) {
                    const int mm = t + q - LAG_A - 1;
                    if (mm >= a0) {
                        store_out(mm, v_out);
                        if (LAST && !counted) { add_dt(mm, v_out); counted = true; }
                    }
                }
                t += k;
                if (k < nb) break;
            }
            return t;
        };

        int t = t0;
        int run = 0;
        // units t0 + 2 .. t0 + 1 + kEnter must equal it too (loaded together) before the run's
        // evaluation is spent; they lie in the segment's range (faces up to t1) when
        // t1 - t0 = b0 - a0 + 2 LAG_A >= kEnter + 1, i.e. for segments of two cells or more
        if (reuse && t1 - t0 >= kEnter + 1) {
            Flux<T> f0, f1;
            CellIn<T> c;
            load_face(t0, f0);
            load_face(t0 + 1, f1);
            load_cell(t0, c);
            const Unit v{f1, c};
            bool same[kEnter];
#pragma unroll
            for (int q = 0; q < kEnter; q++) {
                Flux<T> fq;
                CellIn<T> cq;
                load_face(t0 + 2 + q, fq);
                load_cell(t0 + 1 + q, cq);
                same[q] = same_unit(fq, cq, v);
            }
            bool all = same_bits(f0.us, f1.us) & same_bits(f0.ps, f1.ps) & same_bits(f0.psus, f1.psus);
#pragma unroll
            for (int q = 0; q < kEnter; q++) all = all && same[q];
            if (all) {
                uniform_march(v);
                T o[4];
                project(kE2 ? L1 : L2, A0, A1, o);
                run_slot[11][tid] = c.rho; run_slot[12][tid] = c.ua; run_slot[13][tid] = c.uo; run_slot[14][tid] = c.E;
                keep_run(f1, o);
                t = stream(t0 + 2);
                if (t <= t1) uniform_march(run_unit());
            }
        }
#pragma unroll 1
        for (; t <= t1; ++t) {
            // ---- flux of face t, state of cell t - 1 ----
            Flux<T> f;
            load_face(t, f);
            CellIn<T> c{};
            if (t >= t0 + 1) load_cell(t - 1, c);
            if (reuse) {
                run = (t >= t0 + 2 && same_bits(f.us, F4.us) && same_bits(f.ps, F4.ps) && same_bits(f.psus, F4.psus) &&
                       same_bits(c.rho, run_slot[11][tid]) && same_bits(c.ua, run_slot[12][tid]) &&
                       same_bits(c.uo, run_slot[13][tid]) && same_bits(c.E, run_slot[14][tid])) ? run + 1 : 0;
                run_slot[11][tid] = c.rho; run_slot[12][tid] = c.ua; run_slot[13][tid] = c.uo; run_slot[14][tid] = c.E;
            }
            F1 = F2; F2 = F3; F3 = F4;
            f.dtus = qmul<4>(dt, f.us);
            F4 = f;
            // ---- Lagrange update of cell j = t - 1 ----
            if (t >= t0 + 1) {
                L1 = L2; L2 = L3;
                L3 = lagrange_of(c, F3, F4);
                if (kE2) {
                    d01 = d12; d12 = d23; d23 = lag_diff(L2, L3);
                    s01 = s12; s12 = s23; s23 = L2.W + L3.W;
                }
            }
            // ---- advection flux at face k = t - LAG_A ----
            const int k = t - LAG_A;
            if (k >= a0) {
                A0 = A1;
                A1 = kE2 ? advect2(F1, F2, F3, L1, L2, d01, d12, d23, s01, s12, s23, dx) : advect1(F3, L2, L3);
            }
            // ---- projection of cell mm = k - 1 ----
            const int mm = k - 1;
            if (mm >= a0) {
                T o[4];
                project(kE2 ? L1 : L2, A0, A1, o);
                store_out(mm, o);
                if (LAST) add_dt(mm, o);
                if (reuse && run >= kEnter) {
                    // units t - 2 LAG_A - 1 .. t are equal: the following positions of the run are streamed
                    keep_run(F4, o);
                    counted = true;
                    const int tn = stream(t + 1);
                    if (tn > t1) break;
                    uniform_march(run_unit());
                    // the cell compared with the next step's: the run's
                    for (int q = 0; q < 4; q++) run_slot[11 + q][tid] = run_slot[3 + q][tid];
                    run = 0;
                    t = tn - 1;          // the loop's increment brings it to tn
                }
            }
        }
    }
    if (g.cost != nullptr) {
        __syncthreads();
        if (threadIdx.x == 0 && P.has_unit)
            g.cost[P.u] = (uint32_t)min(clock64() - clock_start, (long long)0xFFFFFFFFu);
    }
    if constexpr (LAST) {
        acc.finish();
        commit_cycle(A, acc, st, cd, blk, nblk);
    }
}

template <class T, int SCHEME, int PROJ, bool LAST>
__global__ void __launch_bounds__(128, sweep_faces_min_blocks<T>()) sweep_faces_kernel(const SweepArgs<T> A)
{
    sweep_faces<T, SCHEME, PROJ, LAST, ARMON_FACES_SOFT_MUL, ARMON_FACES_SOFT_ADD>(A, blockIdx.x, A.pass);
}

template <class T, int SCHEME, int PROJ, bool LAST>
__global__ void __launch_bounds__(128, sweep_cells_min_blocks<T>()) sweep_cells_kernel(const SweepArgs<T> A)
{
    sweep_cells<T, SCHEME, PROJ, LAST>(A, blockIdx.x, gridDim.x, A.pass);
}

// Many domains in one launch (sweep_batch_kernel's layout), each half on its own.
template <class T, int SCHEME, int PROJ, bool LAST>
__global__ void __launch_bounds__(128, sweep_faces_min_blocks<T>())
    sweep_batch_faces_kernel(const SweepArgs<T>* __restrict__ doms, const int* __restrict__ offsets, int ndom, int pass,
                             BatchOrder ord)
{
    const int b = ord.order != nullptr ? (int)__ldg(&ord.order[blockIdx.x]) : (int)blockIdx.x;
    const long long clock_start = clock64();
    __shared__ __align__(16) SweepArgs<T> sA;
    const int lo = batch_domain(doms, offsets, ndom, b, sA);
    sweep_faces<T, SCHEME, PROJ, LAST>(sA, b - offsets[lo], pass);
    record_cost(ord, b, clock_start);
}

template <class T, int SCHEME, int PROJ, bool LAST>
__global__ void __launch_bounds__(128, sweep_batch_cells_min_blocks<T>())
    sweep_batch_cells_kernel(const SweepArgs<T>* __restrict__ doms, const int* __restrict__ offsets, int ndom, int pass,
                             BatchOrder ord)
{
    const int b = ord.order != nullptr ? (int)__ldg(&ord.order[blockIdx.x]) : (int)blockIdx.x;
    const long long clock_start = clock64();
    __shared__ __align__(16) SweepArgs<T> sA;
    const int lo = batch_domain(doms, offsets, ndom, b, sA);
    sweep_cells<T, SCHEME, PROJ, LAST>(sA, b - offsets[lo], offsets[lo + 1] - offsets[lo], pass);
    record_cost(ord, b, clock_start);
}

}  // namespace armon
