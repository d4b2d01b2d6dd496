// sweep.cuh -- the fused axis pass: one kernel does the whole per-axis stage sequence of
// solver_cycle (src/armon_2D.cpp:304-324) for every real cell:
//
//   perfect_gas_EOS     src/kernels/fluid_eos.cpp:9-23
//   boundary_conditions src/kernels/halo_exchange.cpp:9-36     (ghosts made on the fly)
//   acoustic / _GAD     src/kernels/acoustic.cpp:10-108
//   cell_update         src/kernels/euler_projection.cpp:9-22
//   advection 1st / 2nd src/kernels/euler_projection.cpp:51-120
//   euler_projection    src/kernels/euler_projection.cpp:25-48
//   dt_CFL (last pass)  src/kernels/reductions.cpp:8-24
//
// Mapping.  A thread owns one line (a row for the X pass, a column for the Y pass) and a segment
// [a, b) of its real cells, and marches t = a - H .. b - 1 + H along the line (H = the stencil
// reach: 4 for GAD + second-order remap).  Each step loads one cell and advances a register
// pipeline by one position: EOS(t), Godunov face t, GAD face t-1, Lagrange cell t-2, advection face
// t-3, projection cell t-4.  Every intermediate (face flux, Lagrangian cell, product rho*u, the
// Lagrangian width dx + dt*(u*[i+1] - u*[i])) is computed once and reused from the window, so the
// FP64 work per cell is the reference's minus its recomputation.  Threads of a warp own adjacent
// lines, so the Y pass reads coalesced rows.
//
// Exactness.  Every value is computed with the reference's expression tree; the file is compiled
// with --fmad=false, so results are bit-identical to the reference's strict build.  Reuse only
// replaces a recomputation of the same expression on the same inputs (differences of adjacent
// cells or faces, rho c, rho dx, width sums, which IEEE addition's commutativity makes shareable).
// Division by dx becomes a multiplication only when dx is a power of two (then both are exact
// scalings); exact scalings by powers of two move the exponent field on the integer pipes.
//
// Ghosts.  Positions -sw..-1 and n..n+sw-1 are the mirror images of real cells with the sign
// factors of the side (what boundary_conditions writes); EOS of a mirrored state equals the copied
// EOS of its source since (-u)^2 == u^2.  Positions beyond the stencil width keep the values in
// memory, as in the reference, where boundary_conditions never writes them.  Ghost memory is never
// written here.
//
// State.  Each pass reads one buffer set and writes the other (in-place updates would race across
// segment halos); the current set is (cycles_done * passes_per_cycle) % 2.  The pass also writes
// p, c, g of its input (what update_EOS leaves in memory) for the real cells when asked.
//
// This file holds the stage functions, the fused kernels (the FP32 pass, and the FP64 pass on
// request) and the batch kernel; sweep_split.cuh runs the same stages as two launches per pass (the
// FP64 default), and order.cuh orders each launch's units longest first.
#pragma once

#include "device_common.cuh"
#include "softfp.cuh"

#ifndef ARMON_SOFT_FP64
#define ARMON_SOFT_FP64 1
#endif

// Stages whose FP64 products run on the integer pipes (sfp::mul), one bit per stage: 0 EOS,
// 1 rho c and rho c u, 2 Godunov, 3 GAD, 4 face products, 5 Lagrange, 6 advection, 7 projection.
// The FP64 pipe and the integer pipes then share the products; results are the same either way.
// The mask applies to every kernel; the solver's split face half adds ARMON_FACES_SOFT_MUL: it
// keeps the FP64 pipe ~82 % busy with 16 warps per SM to hide the longer integer chains, and
// taking the GAD products off the pipe pays there (+2 %), while the batch and fused kernels,
// with fewer registers to spare, measured slower with it.
#ifndef ARMON_SOFT_MUL
#define ARMON_SOFT_MUL 0
#endif
#ifndef ARMON_FACES_SOFT_MUL
#define ARMON_FACES_SOFT_MUL 0x08
#endif
// The same for additions and subtractions (sfp::add), by stage: 2 Godunov, 3 GAD.  Only the
// solver's split face half takes them (ARMON_FACES_SOFT_ADD).
#ifndef ARMON_FACES_SOFT_ADD
#define ARMON_FACES_SOFT_ADD 0
#endif

// Division sites that use the FP64 pipe's IEEE division instead of the integer-pipe one, one bit
// per site: 0 EOS gamma p / rho, 1 Godunov, 2 GAD ratios, 3 GAD dt / Dm, 4 Lagrange dm / W,
// 5 Lagrange dt / dm, 6 advection ratios, 7 advection length factor, 8 projection, 9 EOS sqrt.
// Both give the same results.
#ifndef ARMON_HW_DIV
#define ARMON_HW_DIV 0
#endif

// Unrolling of the march along a line (the pipeline windows then rotate by register renaming
// instead of copies).
#ifndef ARMON_SWEEP_UNROLL
#define ARMON_SWEEP_UNROLL 1
#endif
constexpr int kSweepUnroll = ARMON_SWEEP_UNROLL;

// Blocks of 128 threads the compiler must fit on one SM (it caps registers accordingly): the FP64
// pass keeps its ~250 registers (two blocks), the FP32 pass fits three (four spill, and measured
// slower).
#ifndef ARMON_SWEEP_MIN_BLOCKS
#define ARMON_SWEEP_MIN_BLOCKS 2
#endif
#ifndef ARMON_SWEEP_MIN_BLOCKS_F32
#define ARMON_SWEEP_MIN_BLOCKS_F32 3
#endif
template <class T> constexpr int sweep_min_blocks() { return sizeof(T) == 4 ? ARMON_SWEEP_MIN_BLOCKS_F32 : ARMON_SWEEP_MIN_BLOCKS; }

// Blocks per SM the two halves of a split pass (sweep_split.cuh) must fit.
#ifndef ARMON_FACES_MIN_BLOCKS
#define ARMON_FACES_MIN_BLOCKS 3
#endif
#ifndef ARMON_CELLS_MIN_BLOCKS
#define ARMON_CELLS_MIN_BLOCKS 3
#endif
template <class T> constexpr int sweep_faces_min_blocks() { return sizeof(T) == 4 ? ARMON_SWEEP_MIN_BLOCKS_F32 : ARMON_FACES_MIN_BLOCKS; }
template <class T> constexpr int sweep_cells_min_blocks() { return sizeof(T) == 4 ? ARMON_SWEEP_MIN_BLOCKS_F32 : ARMON_CELLS_MIN_BLOCKS; }
// the batch's cell half reads its arguments from shared memory and needs more registers for them
#ifndef ARMON_BATCH_CELLS_MIN_BLOCKS
#define ARMON_BATCH_CELLS_MIN_BLOCKS ARMON_CELLS_MIN_BLOCKS
#endif
template <class T> constexpr int sweep_batch_cells_min_blocks() { return sizeof(T) == 4 ? ARMON_SWEEP_MIN_BLOCKS_F32 : ARMON_BATCH_CELLS_MIN_BLOCKS; }

// Load each cell's state one iteration ahead of its use: bit 0 for the FP64 pass, bit 1 for FP32.
// The FP32 pass gains from it; the FP64 pass has no registers to spare for it (with reuse, 4096²:
// 7.41-7.52 against 7.48-7.57 G over cycles 180-200, 6.10-6.32 against 7.52 G over the whole run).
#ifndef ARMON_SWEEP_PREFETCH
#define ARMON_SWEEP_PREFETCH 2
#endif
template <class T> __host__ __device__ constexpr bool sweep_prefetch() { return ((ARMON_SWEEP_PREFETCH >> (sizeof(T) == 4 ? 1 : 0)) & 1) != 0; }

// Positions a run streams per iteration (loads issued together, then compared and stored), FP64
// and FP32, and how many batches ahead the streaming loop asks L2 for the lines it will load next
// (prefetch.global.L2: no registers, no data returned; 0 = none).  Measured at 4096² FP64 / 8192²
// FP32, cycles 180-200 / 80-100 (G cell-updates/s), with the general streaming loop: no prefetch
// 6.78 / 13.84, one batch ahead 6.47 / 12.77, two 5.85 / 10.32; FP32 batches of 8: 12.72 (one
// ahead); FP64 batches of 8 or 16 (no prefetch): 6.41, 6.15.  With the straight-line path and
// pair accesses, FP32 batches of 8 against 4: 24.88 against 24.26-24.31 and 24.00 against
// 23.78-23.80 (two runs), the X pass holding four pair loads per array in flight instead of two;
// FP64 batches of 2, 6, 8 against 4: 7.51, 6.84, 6.84 against 7.54.
#ifndef ARMON_REUSE_BATCH
#define ARMON_REUSE_BATCH 4
#endif
#ifndef ARMON_REUSE_BATCH_F32
#define ARMON_REUSE_BATCH_F32 8
#endif
#ifndef ARMON_REUSE_PREFETCH
#define ARMON_REUSE_PREFETCH 0
#endif
// Whether the straight-line streaming path takes the following batches in a loop of its own, with
// the pair alignment of the run's positions taken once (bit 0 FP64, bit 1 FP32), instead of one
// batch per iteration of the general loop, each testing its alignment.  FP32 gains 1.3 % from it
// (25.35 against 25.03 G at 8192²); FP64 loses 6.5 % (7.00 against 7.49 G at 4096²), and 1 % with
// the alignment alone taken once (7.38-7.43 against 7.49-7.55 G).
#ifndef ARMON_REUSE_INNER
#define ARMON_REUSE_INNER 2
#endif
template <class T> __host__ __device__ constexpr int reuse_batch() { return sizeof(T) == 8 ? ARMON_REUSE_BATCH : ARMON_REUSE_BATCH_F32; }
template <class T> __host__ __device__ constexpr bool reuse_inner() { return ((ARMON_REUSE_INNER >> (sizeof(T) == 4 ? 1 : 0)) & 1) != 0; }
constexpr int kReusePrefetch = ARMON_REUSE_PREFETCH;

// Two consecutive values with one 8-byte (float) or 16-byte (double) access; p must be aligned to
// two values.
__device__ __forceinline__ void load2(const float* p, float& a, float& b)
{
    const float2 v = *reinterpret_cast<const float2*>(p);
    a = v.x;
    b = v.y;
}
__device__ __forceinline__ void load2(const double* p, double& a, double& b)
{
    const double2 v = *reinterpret_cast<const double2*>(p);
    a = v.x;
    b = v.y;
}
__device__ __forceinline__ void store2(float* p, float v) { *reinterpret_cast<float2*>(p) = make_float2(v, v); }
__device__ __forceinline__ void store2(double* p, double v) { *reinterpret_cast<double2*>(p) = make_double2(v, v); }

// A hint that the line holding p will be read soon: L2 fetches it; nothing comes back to the thread.
__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

namespace armon {

template <class T>
struct AxisGeom {
    int32_t n;          // real cells along the axis
    int32_t nlines;     // lines (rows for X, columns for Y)
    int32_t seg_len;    // real cells per thread
    int32_t nseg;       // segments per line
    int32_t nlb;        // blocks of lines (ceil(nlines / lpb))
    int32_t blocks;     // nlb * ceil(nseg / spb)
    int64_t s;          // stride along the axis
    int64_t lstride;    // stride between lines
    T fa_lo, fo_lo, fa_hi, fo_hi;   // sign factors of the axis / other velocity, low / high side
    T dx, inv_dx;       // p.dx of the axis; 1/dx when dx is a power of two
    int32_t dx_pow2;
    uint32_t fneg;      // bit k set: factor k (fa_lo, fo_lo, fa_hi, fo_hi) is -1
    int32_t f_unit;     // every factor is +1 or -1: apply them as sign flips
    int32_t dx_log2;    // dx == 2^dx_log2 when dx_pow2
    int32_t lpb;        // lines per block: a multiple of 32 dividing blockDim.x
    int32_t spb;        // segments per block: blockDim.x / lpb (narrow domains fill a block with segments)
    // Longest-first dispatch (optional, both NULL when unused): block b of the launch works on unit
    // order[b] of the axis, and records the SM cycles that unit took in cost[unit].
    const uint32_t* order;
    uint32_t* cost;
    const uint32_t* face_order;   // the same for the face half of a split pass (sweep_split.cuh)
    uint32_t* face_cost;
};

template <class T>
struct SweepArgs {
    AxisGeom<T> geom[2];              // X, Y
    int64_t origin;                   // linear index of real cell (0, 0)
    int32_t sw;                       // stencil width (depth of the mirrored band)
    int32_t limiter;                  // 0 None, 1 Minmod, 2 Superbee
    int32_t pass;                     // pass index within the cycle
    int32_t npass;                    // passes per cycle
    int32_t write_eos;                // p, c, g of the real cells: 1 on every pass, 0 on the last pass of a
                                      // cycle, -1 never (the solver computes them when they are read)
    int32_t reuse;                    // reuse a predecessor's results over runs of identical inputs (exact)
    T gamma;
    T* buf[2][4];                     // two state sets: rho, umat, vmat, Emat
    T *pmat, *cmat, *gmat;
    StepState* state;
    StepConfig cfg;
    double* partials;                 // 2 doubles per block (dt reduction)
    T* faces;                         // split passes: u*, p*, p* u* per face (sweep_split.cuh)
    int64_t face_stride;              // values per face array
};

// ---- Exact reuse over runs of identical inputs (SweepArgs::reuse) ----
// A pass is a pure function of the cells it reads: the results at a position of the march depend
// on a window of positions around it, through the same operations in the same order at every
// position.  So where a line holds a run of cells equal bit for bit (fluid at rest, or any uniform
// state), every position whose window lies inside the run has the same results, the run's
// "uniform" results.  Each march evaluates those once (its stage functions on operands that are
// all the run's state), streams the run's positions -- loads compared with the run's state, then
// stores of the uniform results -- several at a time with its pipeline registers dead, and at the
// first position that differs restarts the pipeline from the registers a march over the run would
// hold (the same single evaluation).  Loads and stores still happen for every cell.
__device__ __forceinline__ bool same_bits(double a, double b) { return __double_as_longlong(a) == __double_as_longlong(b); }
__device__ __forceinline__ bool same_bits(float a, float b) { return __float_as_uint(a) == __float_as_uint(b); }

// Whether a pass stores p, c, g of the cells it owns (SweepArgs::write_eos).
template <bool LAST, class A_t> __device__ __forceinline__ bool writes_eos(const A_t& A)
{
    return A.write_eos > 0 || (LAST && A.write_eos == 0);
}

// rc = rho c, rcu = rc ua, dm = rho dx: the products that the two faces of a cell both use
template <class T> struct CellIn { T rho, ua, uo, E, p, c, rc, rcu, dm; };
template <class T>
__device__ __forceinline__ bool same_state(const CellIn<T>& a, const CellIn<T>& b)
{
    return same_bits(a.rho, b.rho) & same_bits(a.ua, b.ua) & same_bits(a.uo, b.uo) & same_bits(a.E, b.E);
}
template <class T> struct God { T us, ps, rcs; };            // rcs = rho_l c_l + rho_r c_r
template <class T> struct Flux { T us, ps, psus, dtus; };    // psus = p* u*, dtus = dt u*
template <class T> struct Lag { T rho, ua, uo, E, rua, ruo, rE, W, c; };
template <class T> struct Adv { T r, ra, ro, rE; };
// Differences of the Godunov state across a face g (between cells g-1 and g), each used by the
// GAD fluxes of two faces: a = u*_g - u_{g-1}, b = u_g - u*_g, and the same for p.
template <class T> struct GadDiff { T au, bu, ap, bp; };

// Operations that the FP64 pass routes to the integer pipes (softfp.cuh: GB300's FP64 pipe is the
// bottleneck, its integer and FP32 pipes are idle) and the FP32 pass keeps on the FP32 pipe.  Both
// give the IEEE results of the plain operators (for non-NaN operands where noted there).
__device__ __forceinline__ double qdiv(double a, double b) { return ARMON_SOFT_FP64 ? sfp::div(a, b) : a / b; }
__device__ __forceinline__ float qdiv(float a, float b) { return a / b; }
// several quotients by one divisor share the divisor's reciprocal estimate
struct QRecipD { sfp::Recip r; double b; };
struct QRecipF { float b; };
__device__ __forceinline__ QRecipD qrecip(double b) { return QRecipD{ARMON_SOFT_FP64 ? sfp::recip(b) : sfp::Recip{}, b}; }
__device__ __forceinline__ QRecipF qrecip(float b) { return QRecipF{b}; }
__device__ __forceinline__ double qdiv(double a, const QRecipD& R) { return ARMON_SOFT_FP64 ? sfp::div(a, R.r, R.b) : a / R.b; }
__device__ __forceinline__ float qdiv(float a, const QRecipF& R) { return a / R.b; }
// the same per division site S (ARMON_HW_DIV)
template <int S> __device__ __forceinline__ double qdiv_at(double a, double b) { return ((ARMON_HW_DIV >> S) & 1) ? a / b : qdiv(a, b); }
template <int S> __device__ __forceinline__ float qdiv_at(float a, float b) { return a / b; }
template <int S> __device__ __forceinline__ QRecipD qrecip_at(double b) { return ((ARMON_HW_DIV >> S) & 1) ? QRecipD{sfp::Recip{}, b} : qrecip(b); }
template <int S> __device__ __forceinline__ QRecipF qrecip_at(float b) { return qrecip(b); }
template <int S> __device__ __forceinline__ double qdiv_at(double a, const QRecipD& R) { return ((ARMON_HW_DIV >> S) & 1) ? a / R.b : qdiv(a, R); }
template <int S> __device__ __forceinline__ float qdiv_at(float a, const QRecipF& R) { return a / R.b; }
__device__ __forceinline__ bool qlt(double a, double b) { return ARMON_SOFT_FP64 ? sfp::lt(a, b) : a < b; }
__device__ __forceinline__ bool qlt(float a, float b) { return a < b; }
__device__ __forceinline__ bool qgt0(double a) { return ARMON_SOFT_FP64 ? sfp::gt0(a) : a > 0.0; }
__device__ __forceinline__ bool qgt0(float a) { return a > 0.0f; }
__device__ __forceinline__ double qneg_if(double x, bool c) { return ARMON_SOFT_FP64 ? sfp::neg_if(x, c) : (c ? -x : x); }
__device__ __forceinline__ float qneg_if(float x, bool c) { return c ? -x : x; }
__device__ __forceinline__ bool qsignbit(double x) { return (int64_t)sfp::bits(x) < 0; }
__device__ __forceinline__ bool qsignbit(float x) { return (int32_t)__float_as_uint(x) < 0; }
// exact scalings: x * 0.5, x * 2, x * 2^k (p2 == 2^k)
__device__ __forceinline__ double qhalf(double x) { return ARMON_SOFT_FP64 ? sfp::half(x) : x * 0.5; }
__device__ __forceinline__ float qhalf(float x) { return x * 0.5f; }
__device__ __forceinline__ double qtwice(double x) { return ARMON_SOFT_FP64 ? sfp::twice(x) : x * 2.0; }
__device__ __forceinline__ float qtwice(float x) { return x * 2.0f; }
__device__ __forceinline__ double qscale(double x, int k, double p2) { return ARMON_SOFT_FP64 ? sfp::scale(x, k, p2) : x * p2; }
__device__ __forceinline__ float qscale(float x, int, float p2) { return x * p2; }
__device__ __forceinline__ double qsqrt(double x) { return ARMON_SOFT_FP64 ? sfp::sqrt(x) : ::sqrt(x); }
__device__ __forceinline__ float qsqrt(float x) { return sqrtf(x); }
template <int G, int MASK = ARMON_SOFT_MUL> __device__ __forceinline__ double qmul(double a, double b)
{
    return (ARMON_SOFT_FP64 && (((ARMON_SOFT_MUL | MASK) >> G) & 1)) ? sfp::mul(a, b) : a * b;
}
template <int G, int MASK = ARMON_SOFT_MUL> __device__ __forceinline__ float qmul(float a, float b) { return a * b; }
// a + b and a - b (== a + (-b) for non-NaN b), on the integer pipes for the stages in MASK
template <int G, int MASK> __device__ __forceinline__ double qadd(double a, double b)
{
    return (ARMON_SOFT_FP64 && ((MASK >> G) & 1)) ? sfp::add(a, b) : a + b;
}
template <int G, int MASK> __device__ __forceinline__ float qadd(float a, float b) { return a + b; }
template <int G, int MASK> __device__ __forceinline__ double qsub(double a, double b)
{
    return (ARMON_SOFT_FP64 && ((MASK >> G) & 1)) ? sfp::add(a, sfp::neg_if(b, true)) : a - b;
}
template <int G, int MASK> __device__ __forceinline__ float qsub(float a, float b) { return a - b; }
// Kokkos::min / Kokkos::max: (b < a) ? b : a and (a < b) ? b : a
template <class T> __device__ __forceinline__ T qmin(T a, T b) { return qlt(b, a) ? b : a; }
template <class T> __device__ __forceinline__ T qmax(T a, T b) { return qlt(a, b) ? b : a; }
// the same with a constant operand: max(0, x) and min(c, x) for c = 1 or 2
template <class T> __device__ __forceinline__ T qmax0(T x) { return qgt0(x) ? x : T(0); }
__device__ __forceinline__ double qmin_c(double c, uint64_t cbits, double x) { return ARMON_SOFT_FP64 ? (sfp::lt_pos(x, cbits) ? x : c) : (x < c ? x : c); }
__device__ __forceinline__ float qmin_c(float c, uint64_t, float x) { return x < c ? x : c; }
constexpr uint64_t kOneBits = 0x3FF0000000000000ull, kTwoBits = 0x4000000000000000ull;

template <class T>
__device__ __forceinline__ T limiter_fn(int L, T r)
{
    // src/kernels/limiters.h:15-34
    if (L == 1) return qmax0(qmin_c(T(1), kOneBits, r));
    if (L == 2) return qmax(qmax0(qmin_c(T(1), kOneBits, qtwice(r))), qmin_c(T(2), kTwoBits, r));
    return T(1);
}

// limiter_fn(L, num / den) for the GAD ratios.  With the minmod limiter, max(0, min(1, num / den))
// is +0 when num is zero or of the other sign than den, and 1 when |num| >= |den| with the same
// sign (the rounded quotient is then >= 1), whatever the quotient's rounding; only a ratio inside
// (0, 1) needs the division.  Zero and non-finite operands take the general path.
__device__ __forceinline__ double limited_ratio(int L, double num, double den)
{
    if (L == 1 && ARMON_SOFT_FP64) {
        const uint64_t un = sfp::bits(num), ud = sfp::bits(den);
        const uint64_t an = un & sfp::kAbs, ad = ud & sfp::kAbs;
        if (an < sfp::kInf && ad < sfp::kInf && ad != 0) {
            if (an == 0 || ((un ^ ud) >> 63)) return 0.0;
            if (an >= ad) return 1.0;
            return qdiv_at<2>(num, den);     // in (0, 1]: min(1, .) and max(0, .) keep it
        }
    }
    return limiter_fn(L, qdiv_at<2>(num, den));
}
__device__ __forceinline__ float limited_ratio(int L, float num, float den) { return limiter_fn(L, num / den); }

template <class T>
__device__ __forceinline__ T slope_minmod(T d_m, T d_p, T r_m, T r_p)
{
    // src/kernels/euler_projection.cpp:73-79 with d_p = u_ip - u_i and d_m = u_i - u_im (the
    // differences of adjacent cells, shared by neighbouring faces).  s = copysign(1, D_u_p) is
    // +-1, so s * v is v with its sign flipped when D_u_p's sign bit is set (bit-identical to the
    // multiply for non-NaN v).
    T D_u_p = qmul<6>(r_p, d_p);
    T D_u_m = qmul<6>(r_m, d_m);
    const bool neg = qsignbit(D_u_p);
    return qneg_if(qmax0(qmin(qneg_if(D_u_p, neg), qneg_if(D_u_m, neg))), neg);
}

template <class T>
__device__ __forceinline__ T div_dx(T x, const AxisGeom<T>& g)
{
    return g.dx_pow2 ? qscale(x, -g.dx_log2, g.inv_dx) : qdiv(x, g.dx);
}

template <class T>
__device__ __forceinline__ T mul_dx(T x, const AxisGeom<T>& g)
{
    return g.dx_pow2 ? qscale(x, g.dx_log2, g.dx) : x * g.dx;
}

template <class T>
__device__ __forceinline__ void eos(CellIn<T>& c, T gamma, T gamma_m1)
{
    // src/kernels/fluid_eos.cpp:18-21 (gamma_m1 = gamma - 1, computed once)
    T e = c.E - qhalf(qmul<0>(c.ua, c.ua) + qmul<0>(c.uo, c.uo));
    c.p = qmul<0>(qmul<0>(gamma_m1, c.rho), e);
    const T q = qdiv_at<0>(qmul<0>(gamma, c.p), c.rho);
    c.c = ((ARMON_HW_DIV >> 9) & 1) ? sqrt(q) : qsqrt(q);
}

template <class T, int ADDS = 0>
__device__ __forceinline__ God<T> godunov(const CellIn<T>& L, const CellIn<T>& R)
{
    // src/kernels/acoustic.cpp:10-19 (face between L = i-s and R = i); rc_l * L.ua == L.rcu
    God<T> g;
    g.rcs = qadd<2, ADDS>(L.rc, R.rc);
    const auto inv = qrecip_at<1>(g.rcs);
    g.us = qdiv_at<1>(qadd<2, ADDS>(qadd<2, ADDS>(L.rcu, R.rcu), qsub<2, ADDS>(L.p, R.p)), inv);
    g.ps = qdiv_at<1>(qadd<2, ADDS>(qadd<2, ADDS>(qmul<2>(R.rc, L.p), qmul<2>(L.rc, R.p)),
                                    qmul<2>(qmul<2>(L.rc, R.rc), qsub<2, ADDS>(L.ua, R.ua))), inv);
    return g;
}

template <class T, int ADDS = 0>
__device__ __forceinline__ GadDiff<T> gad_diff(const God<T>& G, const CellIn<T>& Cl, const CellIn<T>& Cr)
{
    GadDiff<T> d;
    d.au = qsub<3, ADDS>(G.us, Cl.ua);
    d.bu = qsub<3, ADDS>(Cr.ua, G.us);
    d.ap = qsub<3, ADDS>(G.ps, Cl.p);
    d.bp = qsub<3, ADDS>(Cr.p, G.ps);
    return d;
}

template <class T, int MULS = ARMON_SOFT_MUL, int ADDS = 0>
__device__ __forceinline__ Flux<T> gad(const God<T>& Gc, const GadDiff<T>& Dm1, const GadDiff<T>& D0,
                                       const GadDiff<T>& Dp1, T dm_l, T dm_r, int L, T dt)
{
    // src/kernels/acoustic.cpp:40-88 for face i (between cells i-s and i), with the differences
    // of faces i-s (Dm1), i (D0), i+s (Dp1):  Gp.us - Cr.ua == Dp1.au, Gc.us - Cl.ua == D0.au,
    // Cl.ua - Gm.us == Dm1.bu, Cr.ua - Gc.us == D0.bu (the same for p).
    const T r_um = limited_ratio(L, Dp1.au, qadd<3, ADDS>(D0.au, T(1e-6)));
    const T r_pm = limited_ratio(L, Dp1.ap, qadd<3, ADDS>(D0.ap, T(1e-6)));
    const T r_up = limited_ratio(L, Dm1.bu, qadd<3, ADDS>(D0.bu, T(1e-6)));
    const T r_pp = limited_ratio(L, Dm1.bp, qadd<3, ADDS>(D0.bp, T(1e-6)));
    T Dm = qhalf(qadd<3, ADDS>(dm_l, dm_r));              // (dm_l + dm_r) / 2
    T theta = qhalf(qsub<3, ADDS>(T(1), qmul<3, MULS>(qhalf(Gc.rcs), qdiv_at<3>(dt, Dm))));   // 0.5 (1 - (rc_l + rc_r) / 2 dt / Dm)
    Flux<T> f;
    f.us = qadd<3, ADDS>(Gc.us, qmul<3, MULS>(theta, qsub<3, ADDS>(qmul<3, MULS>(r_up, D0.bu), qmul<3, MULS>(r_um, D0.au))));
    f.ps = qadd<3, ADDS>(Gc.ps, qmul<3, MULS>(theta, qsub<3, ADDS>(qmul<3, MULS>(r_pp, D0.bp), qmul<3, MULS>(r_pm, D0.ap))));
    return f;
}

template <class T>
__device__ __forceinline__ Lag<T> lagrange(const CellIn<T>& C, const Flux<T>& F0, const Flux<T>& F1, T dt, T dx)
{
    // src/kernels/euler_projection.cpp:9-22 for cell i (F0 = face i, F1 = face i+s)
    Lag<T> l;
    const T dm = C.dm;
    l.W = dx + qmul<5>(dt, F1.us - F0.us);
    l.rho = qdiv_at<4>(dm, l.W);
    T dtdm = qdiv_at<5>(dt, dm);
    l.ua = C.ua + qmul<5>(dtdm, F0.ps - F1.ps);
    l.E = C.E + qmul<5>(dtdm, F0.psus - F1.psus);
    l.uo = C.uo;
    l.rua = qmul<5>(l.rho, l.ua);
    l.ruo = qmul<5>(l.rho, l.uo);
    l.rE = qmul<5>(l.rho, l.E);
    l.c = C.c;
    return l;
}

// The advected quantities of a Lagrangian cell, and differences of adjacent cells' ones.
template <class T>
__device__ __forceinline__ Adv<T> lag_diff(const Lag<T>& lo, const Lag<T>& hi)
{
    return Adv<T>{hi.rho - lo.rho, hi.rua - lo.rua, hi.ruo - lo.ruo, hi.rE - lo.rE};
}

// When is a face's minmod slope a signed zero fixed by the signs alone?  slope_minmod(d_m, d_p)
// is +-0 (the sign of d_p) whenever one difference is zero or the two have opposite signs, for any
// finite positive r_m, r_p; the slope times a finite length factor is then the zero with the sign
// of d_p XOR the factor's.  These tests decide it on the bit patterns; infinities and NaNs, and
// quotients that could overflow or underflow to zero, take the general path.
__device__ __forceinline__ bool slope_is_zero(double d_m, double d_p)
{
    const uint64_t um = sfp::bits(d_m), up = sfp::bits(d_p);
    const uint64_t am = um & sfp::kAbs, ap = up & sfp::kAbs;
    if (am >= sfp::kInf || ap >= sfp::kInf) return false;
    return am == 0 || ap == 0 || ((um ^ up) >> 63) != 0;
}

// num / den is finite for a positive normal den and a finite num whose exponent is not far above
__device__ __forceinline__ bool quotient_finite(double num, double den)
{
    const uint64_t un = sfp::bits(num), ud = sfp::bits(den);
    const int en = (int)((un >> 52) & 0x7FF), ed = (int)((ud >> 52) & 0x7FF);
    return (int64_t)ud > 0 && (unsigned)(ed - 1) < 2046u && en < 2047 && en - ed < 1000;
}

// num / den is positive, finite and not zero: both positive normal, exponents close
__device__ __forceinline__ bool quotient_positive(double num, double den)
{
    const uint64_t un = sfp::bits(num);
    const int en = (int)((un >> 52) & 0x7FF), ed = (int)((sfp::bits(den) >> 52) & 0x7FF);
    return (int64_t)un > 0 && (unsigned)(en - 1) < 2046u && quotient_finite(num, den) && ed - en < 1000;
}

template <class T>
__device__ __forceinline__ Adv<T> advect2(const Flux<T>& Fm, const Flux<T>& Fk, const Flux<T>& Fp,
                                          const Lag<T>& L1, const Lag<T>& L2, const Adv<T>& d01,
                                          const Adv<T>& d12, const Adv<T>& d23, T s01, T s12, T s23, T dx)
{
    // src/kernels/euler_projection.cpp:82-120 for face k, from cells L1 = k-1 and L2 = k and the
    // differences d01 = L(k-1) - L(k-2), d12 = L(k) - L(k-1), d23 = L(k+1) - L(k), and the width
    // sums s01 = W(k-2) + W(k-1), s12, s23, which neighbouring faces share.  Upwind (disp > 0) the
    // cells are (k-2, k-1, k), else (k-1, k, k+1).  x + y == y + x exactly, and
    // -(dx - y) == -(dx + (-y)), so the face's Dx costs one addition.
    T disp = Fk.dtus;
    bool up = qgt0(disp);
    T Dx = qneg_if(dx + (up ? qneg_if(Fm.dtus, true) : Fp.dtus), up);
    const T Dx_l = up ? L1.W : L2.W;
    const T two_Dx_l = qtwice(Dx_l);
    if constexpr (sizeof(T) == 8) {
        // every slope a signed zero: the three quotients are not needed (exactly the same result)
        const Adv<T> dm = up ? d01 : d12, dp = up ? d12 : d23;
        if (ARMON_SOFT_FP64 && slope_is_zero(dm.r, dp.r) && slope_is_zero(dm.ra, dp.ra) &&
            slope_is_zero(dm.ro, dp.ro) && slope_is_zero(dm.rE, dp.rE) &&
            quotient_positive(two_Dx_l, up ? s01 : s12) && quotient_positive(two_Dx_l, up ? s12 : s23) &&
            quotient_finite(Dx, two_Dx_l)) {
            const uint64_t sx = sfp::bits(Dx) >> 63;
            const auto prod = [&](T d_p) { return sfp::from_bits(((sfp::bits(d_p) >> 63) ^ sx) << 63); };
            Adv<T> a;
            a.r = qmul<6>(disp, (up ? L1.rho : L2.rho) - prod(dp.r));
            a.ra = qmul<6>(disp, (up ? L1.rua : L2.rua) - prod(dp.ra));
            a.ro = qmul<6>(disp, (up ? L1.ruo : L2.ruo) - prod(dp.ro));
            a.rE = qmul<6>(disp, (up ? L1.rE : L2.rE) - prod(dp.rE));
            return a;
        }
    }
    T r_m = qdiv_at<6>(two_Dx_l, up ? s01 : s12);    // 2 Dx_l / (Dx_l + Dx_lm)
    T r_p = qdiv_at<6>(two_Dx_l, up ? s12 : s23);    // 2 Dx_l / (Dx_l + Dx_lp)
    T slope_r = slope_minmod(up ? d01.r : d12.r, up ? d12.r : d23.r, r_m, r_p);
    T slope_ra = slope_minmod(up ? d01.ra : d12.ra, up ? d12.ra : d23.ra, r_m, r_p);
    T slope_ro = slope_minmod(up ? d01.ro : d12.ro, up ? d12.ro : d23.ro, r_m, r_p);
    T slope_rE = slope_minmod(up ? d01.rE : d12.rE, up ? d12.rE : d23.rE, r_m, r_p);
    T length_factor = qdiv_at<7>(Dx, two_Dx_l);
    Adv<T> a;
    a.r = qmul<6>(disp, (up ? L1.rho : L2.rho) - qmul<6>(slope_r, length_factor));
    a.ra = qmul<6>(disp, (up ? L1.rua : L2.rua) - qmul<6>(slope_ra, length_factor));
    a.ro = qmul<6>(disp, (up ? L1.ruo : L2.ruo) - qmul<6>(slope_ro, length_factor));
    a.rE = qmul<6>(disp, (up ? L1.rE : L2.rE) - qmul<6>(slope_rE, length_factor));
    return a;
}

template <class T>
__device__ __forceinline__ Adv<T> advect1(const Flux<T>& Fk, const Lag<T>& Lm, const Lag<T>& Lk)
{
    // src/kernels/euler_projection.cpp:51-70 for face k (Lm = cell k-s, Lk = cell k)
    T disp = Fk.dtus;
    bool up = qgt0(disp);
    Adv<T> a;
    a.r = qmul<6>(disp, up ? Lm.rho : Lk.rho);
    a.ra = qmul<6>(disp, up ? Lm.rua : Lk.rua);
    a.ro = qmul<6>(disp, up ? Lm.ruo : Lk.ruo);
    a.rE = qmul<6>(disp, up ? Lm.rE : Lk.rE);
    return a;
}

// The end of the last pass of a cycle: the block reduction of the dt maxima, then the last block to
// finish commits dt_CFL, time and cycle to the step state.
template <class T>
__device__ __forceinline__ void commit_cycle(const SweepArgs<T>& A, DtAcc acc, const StepState& st,
                                             const CycleDt& cd, const int blk, const int nblk)
{
    __shared__ double red[2][4];
    __shared__ int is_last_block;
    for (int o = 16; o > 0; o >>= 1) {
        acc.merge(__shfl_xor_sync(0xffffffffu, acc.ax, o), __shfl_xor_sync(0xffffffffu, acc.ay, o));
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { red[0][warp] = acc.ax; red[1][warp] = acc.ay; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ax = red[0][0], ay = red[1][0];
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) { ax = kmax(ax, red[0][w]); ay = kmax(ay, red[1][w]); }
        A.partials[2 * blk] = ax;
        A.partials[2 * blk + 1] = ay;
        __threadfence();
        unsigned prev = atomicAdd(&A.state->counter, 1u);
        is_last_block = (prev == (unsigned)nblk - 1);
    }
    __syncthreads();
    if (!is_last_block) return;
    __threadfence();
    DtAcc tot;
    tot.init();
    for (int b = threadIdx.x; b < nblk; b += blockDim.x)
        tot.merge(__ldcg(&A.partials[2 * b]), __ldcg(&A.partials[2 * b + 1]));
    for (int o = 16; o > 0; o >>= 1)
        tot.merge(__shfl_xor_sync(0xffffffffu, tot.ax, o), __shfl_xor_sync(0xffffffffu, tot.ay, o));
    __syncthreads();
    if (lane == 0) { red[0][warp] = tot.ax; red[1][warp] = tot.ay; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ax = red[0][0], ay = red[1][0];
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) { ax = kmax(ax, red[0][w]); ay = kmax(ay, red[1][w]); }
        StepState ns = st;
        ns.raw_dt = dt_from_maxima(ax, ay, A.cfg.dt_dx, A.cfg.dt_dy);
        ns.current_dt = cd.current;
        ns.next_dt = cd.next;
        ns.time = st.time + cd.current;
        ns.cycle = st.cycle + 1;
        ns.counter = 0;
        *A.state = ns;
    }
}

// One axis pass of one domain, as block `blk` of the `nblk` blocks given to that domain.
// Scheme 0 Godunov / 1 GAD; Proj 1 first order / 2 second order; LAST: the pass that ends a cycle.
template <class T, int SCHEME, int PROJ, bool LAST>
__device__ __forceinline__ void sweep_domain(const SweepArgs<T>& A, const int blk, const int nblk, const int pass)
{
    constexpr bool kGAD = SCHEME == 1;
    constexpr bool kE2 = PROJ == 2;
    constexpr int LAG_F = kGAD ? 1 : 0;             // flux face = t - LAG_F
    constexpr int LAG_L = LAG_F + 1;                // Lagrange cell
    constexpr int LAG_A = kE2 ? LAG_F + 2 : LAG_L;  // advection face
    constexpr int H = LAG_A + 1;                    // projection lag == stencil reach

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
    // X pass: the axis velocity is umat (1), Y pass: vmat (2)
    const T* __restrict__ rho_in = in[0];
    const T* __restrict__ ua_in = in[axis == 0 ? 1 : 2];
    const T* __restrict__ uo_in = in[axis == 0 ? 2 : 1];
    const T* __restrict__ E_in = in[3];

    DtAcc acc;
    acc.init();
    const T gamma_m1 = A.gamma - 1;

    // unit u = (line block lb, segment block sb); warp-aligned groups of lpb threads take spb
    // consecutive segments of the same lpb lines.  Units are independent, so which block takes which
    // unit changes nothing in the results; with an order, the units that took longest in the
    // previous cycle start first and the cheap ones fill the tail of the launch.
    const bool has_unit = blk < g.blocks;
    const int u = (g.order != nullptr && has_unit) ? (int)__ldg(&g.order[blk]) : blk;
    const long long clock_start = clock64();
    const int lb = u % max(g.nlb, 1);
    const int sb = u / max(g.nlb, 1);
    const int sub = (int)threadIdx.x / g.lpb;
    const int seg = sb * g.spb + sub;
    const int line = lb * g.lpb + (int)threadIdx.x % g.lpb;
    const bool active = has_unit && line < g.nlines && seg < g.nseg && sub < g.spb;

    if (active) {
        const int n = g.n, sw = A.sw;
        const int a0 = seg * g.seg_len;
        const int b0 = min(n, a0 + g.seg_len);
        const int64_t base = A.origin + (int64_t)line * g.lstride;
        const int64_t s = g.s;
        const int t0 = a0 - H, t1 = b0 - 1 + H;
        const int firstF = kGAD ? t0 + 2 : t0 + 1;

        CellIn<T> C0{}, C1{}, C2{};
        God<T> G1{}, G2{};
        GadDiff<T> D0{}, D1{}, D2{};         // faces t-2, t-1, t
        Flux<T> F0{}, F1{}, F2{}, F3{}, F4{};
        Lag<T> L1{}, L2{}, L3{};
        Adv<T> d01{}, d12{}, d23{};          // L(j+1) - L(j) for the Lagrangian cells
        T s01{}, s12{}, s23{};               // W(j) + W(j+1)
        Adv<T> A0{}, A1{};

        // position tt of the line -> the cell read there: itself (real, or an untouched ghost past the
        // mirrored band: stale), or the mirror of a real cell (side 1: low side, 2: high side)
        const auto source = [&](int tt, int& m, int& side) {
            m = tt;
            side = 0;
            bool stale = false;
            if (tt < 0) {
                if (tt >= -sw) { m = -1 - tt; side = 1; } else stale = true;
            } else if (tt >= n) {
                if (tt < n + sw) { m = 2 * n - 1 - tt; side = 2; } else stale = true;
            }
            return stale;
        };
        // boundary_conditions: umat * u_factor, vmat * v_factor (+-1: a sign flip)
        const auto mirror = [&](CellIn<T>& c, int side) {
            if (side) {
                if (g.f_unit) {
                    const uint32_t sh = side == 1 ? 0 : 2;
                    c.ua = qneg_if(c.ua, (g.fneg >> sh) & 1u);
                    c.uo = qneg_if(c.uo, (g.fneg >> (sh + 1)) & 1u);
                } else {
                    c.ua = c.ua * (side == 1 ? g.fa_lo : g.fa_hi);
                    c.uo = c.uo * (side == 1 ? g.fo_lo : g.fo_hi);
                }
            }
        };
        // EOS and the products the faces share, of a loaded (non-stale) cell
        const auto prepare = [&](CellIn<T>& c) {
            eos(c, A.gamma, gamma_m1);
            c.rc = qmul<1>(c.rho, c.c);
            c.rcu = qmul<1>(c.rc, c.ua);
            c.dm = mul_dx(c.rho, g);
        };
        // src/kernels/euler_projection.cpp:36-46 for a cell Lc between advection fluxes a0 and a1
        const auto project = [&](const Lag<T>& Lc, const Adv<T>& a0, const Adv<T>& a1, T (&o)[4]) {
            T dXr = qmul<7>(Lc.W, Lc.rho);
            o[0] = div_dx(dXr - (a1.r - a0.r), g);
            T tmp_ra = div_dx(qmul<7>(dXr, Lc.ua) - (a1.ra - a0.ra), g);
            T tmp_ro = div_dx(qmul<7>(dXr, Lc.uo) - (a1.ro - a0.ro), g);
            T tmp_rE = div_dx(qmul<7>(dXr, Lc.E) - (a1.rE - a0.rE), g);
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
        const auto add_dt = [&](const T (&o)[4], T c) {
            // dt_CFL of the state after this pass, with c from this pass's EOS
            if (axis == 0) acc.add(o[1], o[2], c);
            else acc.add(o[2], o[1], c);
        };
        // Every register of the march as it stands after a step whose window held only cells equal
        // to u (u prepared): the same stage functions on the same operands, each evaluated once.
        // Registers whose window would reach before the segment's first position are never read
        // into a result (results start at a0, whose window starts at t0), so this also stands for
        // the march's start.
        const auto uniform_march = [&](const CellIn<T>& c) {
            C0 = c; C1 = c; C2 = c;
            G2 = godunov(c, c); G1 = G2;
            if (kGAD) { D2 = gad_diff(G2, c, c); D1 = D2; D0 = D2; }
            Flux<T> f;
            if (kGAD) {
                f = gad(G2, D2, D2, D2, c.dm, c.dm, A.limiter, dt);
            } else {
                f.us = G2.us; f.ps = G2.ps;
            }
            f.psus = qmul<4>(f.ps, f.us);
            f.dtus = qmul<4>(dt, f.us);
            F0 = f; F1 = f; F2 = f; F3 = f; F4 = f;
            L3 = lagrange(c, f, f, dt, dx); L2 = L3; L1 = L3;
            if (kE2) {
                d23 = lag_diff(L3, L3); d12 = d23; d01 = d23;
                s23 = L3.W + L3.W; s12 = s23; s01 = s23;
            }
            A1 = kE2 ? advect2(f, f, f, L3, L3, d23, d23, d23, s23, s23, s23, dx) : advect1(f, L3, L3);
            A0 = A1;
        };

        // the state of the next position, loaded one iteration ahead so that the loads' latency
        // overlaps an iteration's arithmetic (ARMON_SWEEP_PREFETCH), else at the top of its iteration
        constexpr bool kPrefetch = sweep_prefetch<T>();
        T next_rho{}, next_ua{}, next_uo{}, next_E{};
        const auto prime = [&](int tt) {
            if constexpr (kPrefetch) {
                int m, side;
                source(tt, m, side);
                const int64_t i = base + (int64_t)m * s;
                next_rho = rho_in[i]; next_ua = ua_in[i]; next_uo = uo_in[i]; next_E = E_in[i];
            }
        };

        // Exact reuse: in a run of positions whose cells equal u (bit for bit, after the mirror), a
        // position's results equal the run's uniform results once the window of its projection
        // (cells t - 2 H .. t) lies inside the run; such positions are streamed, kReuseBatch at a time,
        // with the march's registers dead, and the march restarts from uniform_march(u) at the first
        // cell that differs.  The segment's first position opens a run.
        // The run's state (rho, ua, uo, E, p, c) and uniform results (rho, ua, uo, E) live in this
        // thread's slot of shared memory while the march computes, so that they take no registers
        // from the pipeline.
        const bool reuse = A.reuse != 0;
        constexpr int kEnter = 2 * H;        // equal pairs that put a projection's window inside a run
        constexpr int kReuseBatch = reuse_batch<T>();
        __shared__ T run_slot[10][128];
        const int tid = threadIdx.x;
        const auto keep_run = [&](const CellIn<T>& c, const T (&o)[4]) {
            run_slot[0][tid] = c.rho; run_slot[1][tid] = c.ua; run_slot[2][tid] = c.uo; run_slot[3][tid] = c.E;
            run_slot[4][tid] = c.p; run_slot[5][tid] = c.c;
            run_slot[6][tid] = o[0]; run_slot[7][tid] = o[1]; run_slot[8][tid] = o[2]; run_slot[9][tid] = o[3];
        };
        int run = 0;                         // equal consecutive cells ending at t (-1 after a stale one)
        bool counted = false;                // the run's speeds are in the dt maxima
        // Streams the positions from t on whose cell equals the run's; returns the first that
        // differs (t1 + 1 at the end of the segment).
        const auto stream = [&](int t) -> int {
            CellIn<T> u;
            u.rho = run_slot[0][tid]; u.ua = run_slot[1][tid]; u.uo = run_slot[2][tid]; u.E = run_slot[3][tid];
            const T up = run_slot[4][tid], uc = run_slot[5][tid];
            const T u_out[4] = {run_slot[6][tid], run_slot[7][tid], run_slot[8][tid], run_slot[9][tid]};
            const bool pcg_out = writes_eos<LAST>(A);
            const T g_out = (1 + A.gamma) / 2;
            // Along a row (s == 1) the cells of a batch are consecutive in memory: when every array's
            // address of the batch's first cell (and of its first result) is aligned to two values, the
            // batch moves pairs of cells with one access each, half the requests of a warp whose 32
            // threads each walk their own row.  With an even row length every thread of the warp has
            // the same alignment, so no thread waits for another.
            const auto pair_aligned = [&](int tt) {
                constexpr uintptr_t mask = 2 * sizeof(T) - 1;
                const int64_t i = base + tt, o = base + tt - H;
                uintptr_t a = (uintptr_t)(rho_in + i) | (uintptr_t)(ua_in + i) | (uintptr_t)(uo_in + i) |
                              (uintptr_t)(E_in + i) | (uintptr_t)(out[0] + o) | (uintptr_t)(out[1] + o) |
                              (uintptr_t)(out[2] + o) | (uintptr_t)(out[3] + o);
                if (pcg_out) a |= (uintptr_t)(A.pmat + i) | (uintptr_t)(A.cmat + i) | (uintptr_t)(A.gmat + i);
                return (a & mask) == 0;
            };
            // every address moves by two values from position tt to tt + 2, so the alignment of a
            // position is that of the first or the second position of the run, by parity (taken
            // once with reuse_inner; the FP64 pass measured faster testing each batch)
            const int ts = t;
            const bool hoist = reuse_inner<T>() && s == 1 && kReuseBatch % 2 == 0;
            const bool even_aligned = hoist && pair_aligned(ts);
            const bool odd_aligned = hoist && pair_aligned(ts + 1);
            while (t <= t1) {
                int nb = min(kReuseBatch, t1 - t + 1);
                bool same[kReuseBatch];
                bool fast = nb == kReuseBatch && t >= a0 && t + kReuseBatch <= b0 && t - H >= a0;
                bool pairs = false;
                if (fast && s == 1 && kReuseBatch % 2 == 0) {
                    bool next;   // whether the next position is aligned
                    if (reuse_inner<T>()) {
                        const bool odd = ((t - ts) & 1) != 0;
                        pairs = odd ? odd_aligned : even_aligned;
                        next = odd ? even_aligned : odd_aligned;
                    } else {
                        pairs = pair_aligned(t);
                        next = !pairs && pair_aligned(t + 1);
                    }
                    if (!pairs && next) { fast = false; nb = 1; }   // one position to the alignment
                }
                if (fast) {
                    // batches of real cells the segment owns, each with a result to store: no mirror,
                    // no ghost, and the stores need no per-position test.  Every batch up to tf is
                    // such a batch, with the same alignment (the batch is an even number of cells);
                    // with reuse_inner they are taken here, else one per iteration of the loop.
                    const int tf = min(b0, t1 + 1) - kReuseBatch;
                    bool all;
                    for (;;) {
                        if (pairs) {
#pragma unroll
                            for (int q = 0; q < kReuseBatch; q += 2) {
                                const int64_t idx = base + t + q;
                                CellIn<T> c0, c1;
                                load2(rho_in + idx, c0.rho, c1.rho);
                                load2(ua_in + idx, c0.ua, c1.ua);
                                load2(uo_in + idx, c0.uo, c1.uo);
                                load2(E_in + idx, c0.E, c1.E);
                                same[q] = same_state(c0, u);
                                same[q + 1] = same_state(c1, u);
                            }
                        } else {
#pragma unroll
                            for (int q = 0; q < kReuseBatch; q++) {
                                const int64_t idx = base + (int64_t)(t + q) * s;
                                CellIn<T> c;
                                c.rho = rho_in[idx]; c.ua = ua_in[idx]; c.uo = uo_in[idx]; c.E = E_in[idx];
                                same[q] = same_state(c, u);
                            }
                        }
                        all = true;
#pragma unroll
                        for (int q = 0; q < kReuseBatch; q++) all = all && same[q];
                        if (!all) break;     // same[] of this batch: the positions up to the first that differs are stored below
                        if (pairs) {
#pragma unroll
                            for (int q = 0; q < kReuseBatch; q += 2) {
                                const int64_t i = base + t + q, o = i - H;
                                if (pcg_out) { store2(A.pmat + i, up); store2(A.cmat + i, uc); store2(A.gmat + i, g_out); }
                                store2(out[0] + o, u_out[0]);
                                store2(out[axis == 0 ? 1 : 2] + o, u_out[1]);
                                store2(out[axis == 0 ? 2 : 1] + o, u_out[2]);
                                store2(out[3] + o, u_out[3]);
                            }
                        } else {
#pragma unroll
                            for (int q = 0; q < kReuseBatch; q++) {
                                if (pcg_out) {
                                    const int64_t idx = base + (int64_t)(t + q) * s;
                                    A.pmat[idx] = up;
                                    A.cmat[idx] = uc;
                                    A.gmat[idx] = g_out;
                                }
                                store_out(t + q - H, u_out);
                            }
                        }
                        if (LAST && !counted) { add_dt(u_out, uc); counted = true; }
                        t += kReuseBatch;
                        if (!reuse_inner<T>() || t > tf) break;
                    }
                    if (all) continue;       // past tf (or one batch taken): the general loop goes on
                } else {
#pragma unroll
                    for (int q = 0; q < kReuseBatch; q++) {
                        same[q] = false;
                        if (q < nb) {
                            int m, side;
                            const bool stale = source(t + q, m, side);
                            const int64_t idx = base + (int64_t)m * s;
                            CellIn<T> c;
                            c.rho = rho_in[idx]; c.ua = ua_in[idx]; c.uo = uo_in[idx]; c.E = E_in[idx];
                            mirror(c, side);
                            same[q] = !stale && same_state(c, u);
                        }
                    }
                }
                // the lines of the batches that follow, positions the march reads (at most t1)
#pragma unroll
                for (int q = 0; q < kReusePrefetch * kReuseBatch; q++) {
                    const int tp = t + nb + q;
                    if (tp <= t1) {
                        int m, side;
                        source(tp, m, side);
                        const int64_t idx = base + (int64_t)m * s;
                        prefetch_l2(rho_in + idx); prefetch_l2(ua_in + idx); prefetch_l2(uo_in + idx); prefetch_l2(E_in + idx);
                    }
                }
                int k = 0;
#pragma unroll
                for (int q = 0; q < kReuseBatch; q++) k += (k == q && same[q]) ? 1 : 0;
                for (int q = 0; q < k; q++) {
                    const int tt = t + q;
                    if (tt >= a0 && tt < b0 && pcg_out) {   // owned real cell
                        const int64_t idx = base + (int64_t)tt * s;
                        A.pmat[idx] = up;
                        A.cmat[idx] = uc;
                        A.gmat[idx] = (1 + A.gamma) / 2;
                    }
                    if (tt - H >= a0) {
                        store_out(tt - H, u_out);
                        if (LAST && !counted) { add_dt(u_out, uc); counted = true; }
                    }
                }
                t += k;
                if (k < nb) break;
            }
            return t;
        };
        // the march resumes as if every cell before the current position were the run's
        const auto restart = [&]() {
            CellIn<T> u;
            u.rho = run_slot[0][tid]; u.ua = run_slot[1][tid]; u.uo = run_slot[2][tid]; u.E = run_slot[3][tid];
            prepare(u);
            uniform_march(u);
        };

        // The segment opens a run only when its first positions t0 .. t0 + 2H, the first
        // projection's window, hold equal cells: loaded together, compared, and only then is the
        // run's evaluation spent (a segment that starts in a front computes from t0 at once).
        const auto opens_run = [&](const CellIn<T>& c) {
            bool same[kEnter];
#pragma unroll
            for (int q = 0; q < kEnter; q++) {
                int m, side;
                const bool stale = source(t0 + 1 + q, m, side);
                const int64_t idx = base + (int64_t)m * s;
                CellIn<T> cq;
                cq.rho = rho_in[idx]; cq.ua = ua_in[idx]; cq.uo = uo_in[idx]; cq.E = E_in[idx];
                mirror(cq, side);
                same[q] = !stale && same_state(cq, c);
            }
            bool all = true;
#pragma unroll
            for (int q = 0; q < kEnter; q++) all = all && same[q];
            return all;
        };
        int t = t0;
        if (reuse) {
            int m, side;
            const bool stale = source(t0, m, side);
            const int64_t idx = base + (int64_t)m * s;
            CellIn<T> c;
            c.rho = rho_in[idx]; c.ua = ua_in[idx]; c.uo = uo_in[idx]; c.E = E_in[idx];
            mirror(c, side);
            if (!stale && opens_run(c)) {
                prepare(c);
                uniform_march(c);
                T o[4];
                project(kE2 ? L1 : L2, A0, A1, o);
                keep_run(c, o);
                t = stream(t0 + 1);
                if (t <= t1) restart();
            }
        }
        prime(t);
#pragma unroll kSweepUnroll
        for (; t <= t1; ++t) {
            // ---- load cell t (real, mirrored ghost, or untouched ghost) + EOS ----
            {
                CellIn<T> c;
                int m, side;
                const bool stale = source(t, m, side);
                const int64_t idx = base + (int64_t)m * s;
                if constexpr (kPrefetch) {
                    c.rho = next_rho;
                    c.ua = next_ua;
                    c.uo = next_uo;
                    c.E = next_E;
                    prime(min(t + 1, t1));
                } else {
                    c.rho = rho_in[idx];
                    c.ua = ua_in[idx];
                    c.uo = uo_in[idx];
                    c.E = E_in[idx];
                }
                mirror(c, side);
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
                    if (m == t && t >= a0 && t < b0 && writes_eos<LAST>(A)) {   // owned real cell: what update_EOS stores
                        A.pmat[idx] = c.p;
                        A.cmat[idx] = c.c;
                        A.gmat[idx] = (1 + A.gamma) / 2;
                    }
                }
                C2 = c;
            }
            // ---- Godunov face t ----
            if (t >= t0 + 1) {
                G1 = G2;
                G2 = godunov(C1, C2);
                if (kGAD) { D0 = D1; D1 = D2; D2 = gad_diff(G2, C1, C2); }
            }
            // ---- numerical flux at face f = t - LAG_F ----
            if (kGAD ? (t >= t0 + 3) : (t >= t0 + 1)) {
                F0 = F1; F1 = F2; F2 = F3; F3 = F4;
                Flux<T> f;
                if (kGAD) {
                    f = gad(G1, D0, D1, D2, C0.dm, C1.dm, A.limiter, dt);
                } else {
                    f.us = G2.us; f.ps = G2.ps;
                }
                f.psus = qmul<4>(f.ps, f.us);
                f.dtus = qmul<4>(dt, f.us);
                F4 = f;
            }
            // ---- Lagrange update of cell j = t - LAG_L ----
            const int j = t - LAG_L;
            if (j >= firstF) {
                L1 = L2; L2 = L3;
                L3 = lagrange(kGAD ? C0 : C1, F3, F4, dt, dx);
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
                T o[4];
                project(Lc, A0, A1, o);
                store_out(mm, o);
                if (LAST) add_dt(o, Lc.c);
                if (reuse && run >= kEnter) {
                    // cells t - 2 H .. t are equal: the following positions of the run are streamed
                    keep_run(C2, o);
                    counted = true;
                    const int tn = stream(t + 1);
                    if (tn > t1) break;
                    restart();
                    prime(tn);
                    run = 0;
                    t = tn - 1;          // the loop's increment brings it to tn
                }
            }
        }
    }

    if (g.cost != nullptr) {
        __syncthreads();
        if (threadIdx.x == 0 && has_unit)
            g.cost[u] = (uint32_t)min(clock64() - clock_start, (long long)0xFFFFFFFFu);
    }
    if constexpr (LAST) {
        acc.finish();
        commit_cycle(A, acc, st, cd, blk, nblk);
    }
}

// One domain: the whole grid works on it.
template <class T, int SCHEME, int PROJ, bool LAST>
__global__ void __launch_bounds__(128, sweep_min_blocks<T>()) sweep_kernel(const SweepArgs<T> A)
{
    sweep_domain<T, SCHEME, PROJ, LAST>(A, blockIdx.x, gridDim.x, A.pass);
}

// Many independent domains in one launch.  Domain d owns blocks [offsets[d], offsets[d+1]) of the
// grid (enough for its larger axis); each domain keeps its own step state, so dt, time and cycle
// advance per domain and a finished domain's blocks return at once.
// Longest-first dispatch across the domains of a batch (both NULL when unused): block k of the
// launch takes the launch's block order[k] and records the SM cycles it took in cost[order[k]].
struct BatchOrder {
    const uint32_t* order;
    uint32_t* cost;
    const uint32_t* face_order;   // the same for the face half of a split pass (sweep_split.cuh)
    uint32_t* face_cost;
};

// The domain of launch block b: domain d owns blocks [offsets[d], offsets[d+1]).
__device__ __forceinline__ int batch_domain_index(const int* __restrict__ offsets, int ndom, int b)
{
    int lo = 0, hi = ndom;
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (offsets[mid] <= b) lo = mid; else hi = mid;
    }
    return lo;
}

// The same, with the domain's arguments copied into shared memory: read once, and not aliased by
// the stores.
template <class T>
__device__ __forceinline__ int batch_domain(const SweepArgs<T>* __restrict__ doms, const int* __restrict__ offsets,
                                            int ndom, int b, SweepArgs<T>& sA)
{
    const int lo = batch_domain_index(offsets, ndom, b);
    static_assert(sizeof(SweepArgs<T>) % 4 == 0, "word copy");
    const int* src = reinterpret_cast<const int*>(&doms[lo]);
    int* dst = reinterpret_cast<int*>(&sA);
    for (int w = threadIdx.x; w < (int)(sizeof(SweepArgs<T>) / 4); w += blockDim.x) dst[w] = src[w];
    __syncthreads();
    return lo;
}

__device__ __forceinline__ void record_cost(const BatchOrder& ord, int b, long long clock_start)
{
    if (ord.cost != nullptr) {
        __syncthreads();
        if (threadIdx.x == 0) ord.cost[b] = (uint32_t)min(clock64() - clock_start, (long long)0xFFFFFFFFu);
    }
}

template <class T, int SCHEME, int PROJ, bool LAST>
__global__ void __launch_bounds__(128, sweep_min_blocks<T>()) sweep_batch_kernel(const SweepArgs<T>* __restrict__ doms,
                                                          const int* __restrict__ offsets, int ndom, int pass,
                                                          BatchOrder ord)
{
    const int b = ord.order != nullptr ? (int)__ldg(&ord.order[blockIdx.x]) : (int)blockIdx.x;
    const long long clock_start = clock64();
    __shared__ __align__(16) SweepArgs<T> sA;
    const int lo = batch_domain(doms, offsets, ndom, b, sA);
    sweep_domain<T, SCHEME, PROJ, LAST>(sA, b - offsets[lo], offsets[lo + 1] - offsets[lo], pass);
    record_cost(ord, b, clock_start);
}

}  // namespace armon
