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
        // the last face stored, for positions that reuse it (sweep.cuh: exact reuse)
        __shared__ T reuse_f[3][128];
        const int tid = threadIdx.x;
        const bool reuse = A.reuse != 0;
        int run = 0;
#pragma unroll 1
        for (int t = t0; t <= t1; ++t) {
            {
                CellIn<T> c;
                int m;
                int64_t idx;
                const bool stale = load_position(g, n, sw, base, t, rho_in, ua_in, uo_in, E_in, c, m, idx);
                if (reuse) {
                    run = stale ? -1 : (t > t0 && same_state(c, C2)) ? run + 1 : 0;
                    if (run >= kReuseFaces) {
                        if (m == t && t >= a0 && t < b0 && (LAST || A.write_eos)) {
                            A.pmat[idx] = C2.p;
                            A.cmat[idx] = C2.c;
                            A.gmat[idx] = (1 + A.gamma) / 2;
                        }
                        const int64_t fi = face_index(g, kGAD ? t - 1 : t, P.line);
                        us_out[fi] = reuse_f[0][tid];
                        ps_out[fi] = reuse_f[1][tid];
                        psus_out[fi] = reuse_f[2][tid];
                        continue;
                    }
                }
                C0 = C1; C1 = C2;
                if (stale) {
                    c.p = A.pmat[idx];
                    c.c = A.cmat[idx];
                } else {
                    eos(c, A.gamma, gamma_m1);
                    if (m == t && t >= a0 && t < b0 && (LAST || A.write_eos)) {   // owned real cell: what update_EOS stores
                        A.pmat[idx] = c.p;
                        A.cmat[idx] = c.c;
                        A.gmat[idx] = (1 + A.gamma) / 2;
                    }
                }
                c.rc = qmul<1>(c.rho, c.c);
                c.rcu = qmul<1>(c.rc, c.ua);
                c.dm = mul_dx(c.rho, g);
                C2 = c;
            }
            if (t >= t0 + 1) {
                G1 = G2;
                G2 = godunov<T, ADDS>(C1, C2);
                if (kGAD) { D0 = D1; D1 = D2; D2 = gad_diff<T, ADDS>(G2, C1, C2); }
            }
            if (kGAD ? (t >= t0 + 3) : (t >= t0 + 1)) {
                Flux<T> f;
                if (kGAD) {
                    f = gad<T, MULS, ADDS>(G1, D0, D1, D2, C0.dm, C1.dm, A.limiter, dt);
                } else {
                    f.us = G2.us; f.ps = G2.ps;
                }
                const int64_t fi = face_index(g, kGAD ? t - 1 : t, P.line);
                const T psus = qmul<4>(f.ps, f.us);
                us_out[fi] = f.us;
                ps_out[fi] = f.ps;
                psus_out[fi] = psus;
                if (reuse) {
                    reuse_f[0][tid] = f.us;
                    reuse_f[1][tid] = f.ps;
                    reuse_f[2][tid] = psus;
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
        // face t and cell t - 1 of the next iteration, loaded one iteration ahead (ARMON_CELLS_PREFETCH)
        constexpr bool kPrefetch = cells_prefetch<T>();
        Flux<T> next_f{};
        CellIn<T> next_c{};
        if constexpr (kPrefetch) {
            const int64_t fi = face_index(g, t0, P.line);
            next_f.us = us_in[fi];
            next_f.ps = ps_in[fi];
            next_f.psus = psus_in[fi];
        }

        // the last projection's results, and the state of the cell read one step earlier, for
        // positions that reuse them (sweep.cuh: exact reuse; a step's inputs are face t and cell t - 1)
        __shared__ T reuse_out[4][128];
        __shared__ T prev_cell[4][128];
        const int tid = threadIdx.x;
        const bool reuse = A.reuse != 0;
        int run = 0;

#pragma unroll 1
        for (int t = t0; t <= t1; ++t) {
            // ---- flux of face t, state of cell t - 1 ----
            Flux<T> f;
            if constexpr (kPrefetch) {
                f = next_f;
                const int64_t fi = face_index(g, min(t + 1, t1), P.line);
                next_f.us = us_in[fi];
                next_f.ps = ps_in[fi];
                next_f.psus = psus_in[fi];
            } else {
                const int64_t fi = face_index(g, t, P.line);
                f.us = us_in[fi];
                f.ps = ps_in[fi];
                f.psus = psus_in[fi];
            }
            CellIn<T> c = next_c;
            if constexpr (kPrefetch) {
                // positions up to t1 - 1, the last cell the segment updates, stay inside the ghost band
                int m;
                int64_t idx;
                load_position(g, n, sw, base, min(t, t1 - 1), rho_in, ua_in, uo_in, E_in, next_c, m, idx);
            } else if (t >= t0 + 1) {
                int m;
                int64_t idx;
                load_position(g, n, sw, base, t - 1, rho_in, ua_in, uo_in, E_in, c, m, idx);
            }
            if (reuse && t >= t0 + 1) {
                const bool same = t >= t0 + 2 && same_bits(f.us, F4.us) && same_bits(f.ps, F4.ps) &&
                                  same_bits(f.psus, F4.psus) && same_bits(c.rho, prev_cell[0][tid]) &&
                                  same_bits(c.ua, prev_cell[1][tid]) && same_bits(c.uo, prev_cell[2][tid]) &&
                                  same_bits(c.E, prev_cell[3][tid]);
                run = same ? run + 1 : 0;
                if (run >= kReuseCells) {
                    const int64_t o = base + (int64_t)(t - LAG_A - 1) * s;
                    out[0][o] = reuse_out[0][tid];
                    out[axis == 0 ? 1 : 2][o] = reuse_out[1][tid];
                    out[axis == 0 ? 2 : 1][o] = reuse_out[2][tid];
                    out[3][o] = reuse_out[3][tid];
                    continue;
                }
                prev_cell[0][tid] = c.rho;
                prev_cell[1][tid] = c.ua;
                prev_cell[2][tid] = c.uo;
                prev_cell[3][tid] = c.E;
            }
            F1 = F2; F2 = F3; F3 = F4;
            f.dtus = qmul<4>(dt, f.us);
            F4 = f;
            // ---- Lagrange update of cell j = t - 1 ----
            if (t >= t0 + 1) {
                c.dm = mul_dx(c.rho, g);
                c.c = T(0);
                L1 = L2; L2 = L3;
                L3 = lagrange(c, F3, F4, dt, dx);
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
                const Lag<T>& Lc = kE2 ? L1 : L2;
                // src/kernels/euler_projection.cpp:36-46
                T dXr = qmul<7>(Lc.W, Lc.rho);
                T tmp_rho = div_dx(dXr - (A1.r - A0.r), g);
                T tmp_ra = div_dx(qmul<7>(dXr, Lc.ua) - (A1.ra - A0.ra), g);
                T tmp_ro = div_dx(qmul<7>(dXr, Lc.uo) - (A1.ro - A0.ro), g);
                T tmp_rE = div_dx(qmul<7>(dXr, Lc.E) - (A1.rE - A0.rE), g);
                const auto inv_rho = qrecip_at<8>(tmp_rho);
                T ua = qdiv_at<8>(tmp_ra, inv_rho), uo = qdiv_at<8>(tmp_ro, inv_rho), E = qdiv_at<8>(tmp_rE, inv_rho);
                const int64_t idx = base + (int64_t)mm * s;
                out[0][idx] = tmp_rho;
                out[axis == 0 ? 1 : 2][idx] = ua;
                out[axis == 0 ? 2 : 1][idx] = uo;
                out[3][idx] = E;
                if (reuse) {
                    reuse_out[0][tid] = tmp_rho;
                    reuse_out[1][tid] = ua;
                    reuse_out[2][tid] = uo;
                    reuse_out[3][tid] = E;
                }
                if (LAST) {
                    // dt_CFL of the state after this pass, with c from this pass's EOS (the face half
                    // stored it for every real cell; a reused position would add the same speeds again)
                    const T c = A.cmat[idx];
                    if (axis == 0) acc.add(ua, uo, c);
                    else acc.add(uo, ua, c);
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
