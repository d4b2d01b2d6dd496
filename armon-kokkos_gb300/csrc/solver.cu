// solver.cu -- the native solver: device-resident state, the fused time loop and its C ABI
// (include/armon_gb300.h).
//
// One cycle = passes_per_cycle(splitting) axis passes, each one fused launch or a face and a cell
// launch (the tiling measurement picks the form); the last one also reduces dt_CFL of the new
// state and commits the cycle (time, cycle, dts) into the device StepState, so the host never
// waits inside the loop.  Cycles are issued in batches captured in a CUDA graph;
// after each batch the host reads the 48-byte state back to test the reference's loop condition
// (time < max_time && cycle < max_cycles).  Cycles issued past the end are no-ops on the device.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "armon_gb300.h"
#include "host_common.h"
#include "launch.h"
#include "order.cuh"
#include "solver_common.h"

using namespace armon;

struct armon_solver {
    armon_params p{};
    armon_solver_opts o{};
    int device = 0;
    int sm_count = 152;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    bool fp32 = false;
    size_t elem = 8;
    void* arr[16] = {};
    bool owns_arrays = false;
    StepState* d_state = nullptr;
    StepState* h_state = nullptr;   // pinned
    double* d_partials = nullptr;
    double* d_cons = nullptr;       // conservation partials + 2 results
    int cons_grid = 0;
    StepConfig cfg{};
    SweepArgs<double> a64{};
    SweepArgs<float> a32{};
    int grid = 0, block = 128, npass = 2;
    cudaGraphExec_t graph = nullptr;
    int graph_cycles = 0;
    int64_t launches = 0;
    bool begun = false;
    int64_t partials_cap = 0;       // blocks the dt partials have room for
    int tuned_seg[2] = {0, 0};      // measured segment lengths per axis (0: the model's)
    bool tuned = false;             // the tiling measurement has been set up for this time loop
    struct Tune {                   // the tiling measurement in progress (see start_tuning)
        bool active = false;
        int delay = 0;              // cycles left before the first candidate runs
        std::vector<std::array<int, 4>> cand;   // seg X, seg Y, block, split form
        std::vector<float> ms;      // timed cycle of each entry of seq
        std::vector<size_t> seq;    // candidate of each measured entry: the list forwards, then the best backwards
        bool second = false;        // the backward entries have been appended
        size_t pos = 0;             // next entry of seq
        bool warm = true;           // the entry's unit-cost cycle comes next, then its timed cycle
        std::vector<cudaEvent_t> ev;
        std::array<int, 9> key{};
    } tune;
    int64_t issued = 0;             // cycles issued since begin_loop
    int64_t cycle0 = 0;             // the cycle count at begin_loop
    int64_t measure_cycles = 0;     // cycles run with a candidate tiling, over the solver's loops
    bool eos_stale = false;         // p, c, g of the last pass's input are not in memory yet
    double* stage = nullptr;        // FP32 solvers: FP64 staging array for uploads and downloads
    bool ordered = true;            // longest-first dispatch of each pass's units
    uint32_t* d_order = nullptr;    // per axis: order_cap unit indices, then order_cap costs
    uint32_t* d_cost = nullptr;
    int order_cap = 0;
    bool split = false;             // each pass as a face launch and a cell launch (sweep_split.cuh)
    bool default_split = false;     // the form before any measurement
    void* d_faces = nullptr;        // 3 * face_stride values
    int64_t face_stride = 0;
};

namespace {

int cuda_fail(cudaError_t e, const char* what)
{
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    return ARMON_ERR_CUDA;
}

#define CUDA_TRY(expr)                                            \
    do {                                                          \
        cudaError_t e_ = (expr);                                  \
        if (e_ != cudaSuccess) return cuda_fail(e_, #expr);       \
    } while (0)

template <class T>
void fill_geom(armon_solver* s, SweepArgs<T>& a)
{
    T* const* arr = reinterpret_cast<T* const*>(s->arr);
    // set 0: rho umat vmat Emat; set 1: the four work arrays (free in the fused path)
    DomainBuffers<T> b{{{arr[2], arr[3], arr[4], arr[5]}, {arr[11], arr[12], arr[13], arr[14]}}, arr[6], arr[7], arr[8]};
    const int forced[2] = {s->o.seg_len > 0 ? s->o.seg_len : s->tuned_seg[0],
                           s->o.seg_len > 0 ? s->o.seg_len : s->tuned_seg[1]};
    // the split form's cell half reads c of the last pass's cells (dt_CFL), so its face half writes
    // p, c, g on the last pass at least
    const int eos = s->split ? std::max(0, s->o.materialize_eos) : s->o.materialize_eos;
    s->grid = make_sweep_args<T>(s->p, s->npass, s->block, s->sm_count, forced, b, s->d_state, s->d_partials,
                                 eos, s->o.reuse >= 0 ? 1 : 0, a);
    if (s->split) {
        a.faces = static_cast<T*>(s->d_faces);
        a.face_stride = s->face_stride;
    }
}

int sync_state(armon_solver* s)
{
    CUDA_TRY(cudaMemcpyAsync(s->h_state, s->d_state, sizeof(StepState), cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    return ARMON_OK;
}

int axis_blocks(const armon_solver* s, int axis)
{
    return s->fp32 ? s->a32.geom[axis].blocks : s->a64.geom[axis].blocks;
}

// cost / order arrays: per axis for the (cell) pass, and per axis for the face half of split passes;
// a solver that holds a face buffer can switch forms, so it keeps room for both
int order_arrays(const armon_solver* s) { return s->split ? 4 : 2; }
int order_arrays_held(const armon_solver* s) { return s->d_faces ? 4 : 2; }

// The next passes' unit order from the costs the last passes recorded.
int launch_order(armon_solver* s)
{
    if (!s->ordered) return ARMON_OK;
    UnitCounts n{{axis_blocks(s, 0), axis_blocks(s, 1), axis_blocks(s, 0), axis_blocks(s, 1)}};
    order_units_kernel<<<order_arrays(s), 1024, 0, s->stream>>>(s->d_cost, s->d_order, s->order_cap, n);
    CUDA_TRY(cudaGetLastError());
    s->launches++;
    return ARMON_OK;
}

// (Re)sizes the order and cost arrays for the current tiling, points the sweep arguments at them
// and starts from index order.
int prepare_order(armon_solver* s)
{
    if (!s->ordered) return ARMON_OK;
    const int need = std::max(axis_blocks(s, 0), axis_blocks(s, 1));
    if (need > s->order_cap) {
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        cudaFree(s->d_order);
        cudaFree(s->d_cost);
        s->d_order = s->d_cost = nullptr;
        s->order_cap = 0;
        cudaError_t e = cudaMalloc(&s->d_order, sizeof(uint32_t) * order_arrays_held(s) * (size_t)need);
        if (e == cudaSuccess) e = cudaMalloc(&s->d_cost, sizeof(uint32_t) * order_arrays_held(s) * (size_t)need);
        if (e != cudaSuccess) {
            set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
            return ARMON_ERR_NOMEM;
        }
        s->order_cap = need;
    }
    for (int axis = 0; axis < 2; axis++) {
        uint32_t* o = s->d_order + (size_t)axis * s->order_cap;
        uint32_t* c = s->d_cost + (size_t)axis * s->order_cap;
        uint32_t* fo = s->split ? s->d_order + (size_t)(2 + axis) * s->order_cap : nullptr;
        uint32_t* fc = s->split ? s->d_cost + (size_t)(2 + axis) * s->order_cap : nullptr;
        if (s->fp32) {
            s->a32.geom[axis].order = o; s->a32.geom[axis].cost = c;
            s->a32.geom[axis].face_order = fo; s->a32.geom[axis].face_cost = fc;
        } else {
            s->a64.geom[axis].order = o; s->a64.geom[axis].cost = c;
            s->a64.geom[axis].face_order = fo; s->a64.geom[axis].face_cost = fc;
        }
    }
    const int total = order_arrays(s) * s->order_cap;
    reset_order_kernel<<<std::max(1, std::min(s->sm_count * 4, (total + 255) / 256)), 256, 0, s->stream>>>(
        s->d_order, s->d_cost, s->order_cap, order_arrays(s));
    CUDA_TRY(cudaGetLastError());
    s->launches++;
    return ARMON_OK;
}

cudaError_t launch_pass(armon_solver* s, int k, bool last)
{
    if (s->fp32) {
        s->a32.pass = k;
        return s->split ? launch_sweep_split(s->a32, s->p.scheme, s->p.projection, last, s->grid, s->block, s->stream)
                        : launch_sweep(s->a32, s->p.scheme, s->p.projection, last, s->grid, s->block, s->stream);
    }
    s->a64.pass = k;
    return s->split ? launch_sweep_split(s->a64, s->p.scheme, s->p.projection, last, s->grid, s->block, s->stream)
                    : launch_sweep(s->a64, s->p.scheme, s->p.projection, last, s->grid, s->block, s->stream);
}

int enqueue_direct(armon_solver* s, int n_cycles)
{
    if (n_cycles > 0) s->eos_stale = !s->split && s->o.materialize_eos < 0;
    for (int c = 0; c < n_cycles; c++) {
        for (int k = 0; k < s->npass; k++) {
            bool last = k == s->npass - 1;
            cudaError_t e;
            e = launch_pass(s, k, last);
            if (e != cudaSuccess) return cuda_fail(e, "sweep launch");
            s->launches += s->split ? 2 : 1;
        }
        int rc = launch_order(s);
        if (rc != ARMON_OK) return rc;
    }
    return ARMON_OK;
}

int build_graph(armon_solver* s)
{
    if (s->graph || s->graph_cycles <= 0) return ARMON_OK;
    cudaGraph_t g = nullptr;
    int64_t saved = s->launches;
    CUDA_TRY(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue_direct(s, s->graph_cycles);
    cudaError_t e = cudaStreamEndCapture(s->stream, &g);
    s->launches = saved;
    if (rc != ARMON_OK) { if (g) cudaGraphDestroy(g); return rc; }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&s->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { s->graph = nullptr; return cuda_fail(e, "cudaGraphInstantiate"); }
    return ARMON_OK;
}

int enqueue_steady(armon_solver* s, int n_cycles)
{
    s->issued += n_cycles;
    if (n_cycles > 0) s->eos_stale = !s->split && s->o.materialize_eos < 0;
    if (s->graph_cycles > 0 && n_cycles >= s->graph_cycles) {
        int rc = build_graph(s);
        if (rc != ARMON_OK) return rc;
        while (n_cycles >= s->graph_cycles) {
            CUDA_TRY(cudaGraphLaunch(s->graph, s->stream));
            s->launches += (int64_t)s->graph_cycles * (s->npass * (s->split ? 2 : 1) + (s->ordered ? 1 : 0));
            n_cycles -= s->graph_cycles;
        }
    }
    return enqueue_direct(s, n_cycles);
}

// FP64 <-> FP32 conversion of a staged array on the device (round to nearest, as the host's cast;
// widening is exact).
__global__ void narrow_kernel(const double* __restrict__ in, float* __restrict__ out, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = __double2float_rn(in[i]);
}

__global__ void widen_kernel(const float* __restrict__ in, double* __restrict__ out, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (double)in[i];
}

int ensure_stage(armon_solver* s)
{
    if (s->stage) return ARMON_OK;
    cudaError_t e = cudaMalloc(&s->stage, (size_t)s->p.nb_cells * sizeof(double));
    if (e != cudaSuccess) {
        s->stage = nullptr;
        set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
        return ARMON_ERR_NOMEM;
    }
    return ARMON_OK;
}

// Tiling of a lone domain, measured on the caller's own cycles.  With the GPU to itself, the best
// segment length depends on more than the cells a thread walks (how full the last wave of blocks
// is, how many blocks share an SM, how unevenly the units cost -- fronts against fluid at rest --,
// cache traffic), and so does the pass form (split passes keep the FP64 pipe busier where cells are
// computed, fused ones move half the bytes where runs are streamed), so the time loop times a few
// candidates -- the model's segments and segments aiming at 1, 2, 3, 4, 6 and 8 waves of resident
// blocks (FP32 also 12 and 16), for each form the solver can run (a solver holding a face buffer runs both) and for
// blocks of 128 lines (also of 32 when the caller fixed it) -- keeps the fastest and caches it per
// geometry for the process.  Results never depend on the tiling or the form, so the candidates run
// the loop's real cycles: after kTuneDelay cycles with the model's tiling (the fronts form), each
// candidate runs one cycle that records its units' costs (for longest-first dispatch) and one timed
// cycle, the list forwards, then the four fastest again backwards, so that a cost drifting with the
// flow weighs alike on the finalists.  The loop pays only the difference between the candidates and
// the best, a few cycles' worth.  A loop that ends before the measurement does keeps the model's
// tiling and caches nothing.  Domains under 2^20 cells, single-pass splittings and a caller-fixed
// seg_len are left to the model.
using Tiling = std::array<int, 4>;   // segment length X, segment length Y, block lines, split form
std::map<std::array<int, 9>, Tiling> g_tilings;
std::mutex g_tilings_mu;
constexpr int kTuneDelay = 16;
constexpr size_t kTuneFinalists = 4;

int refill(armon_solver* s)
{
    if (s->fp32) fill_geom(s, s->a32); else fill_geom(s, s->a64);
    if (s->graph) {
        cudaGraphExecDestroy(s->graph);
        s->graph = nullptr;
    }
    return prepare_order(s);
}

int ensure_partials(armon_solver* s)
{
    if (s->grid <= s->partials_cap) return ARMON_OK;
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    CUDA_TRY(cudaFree(s->d_partials));
    s->d_partials = nullptr;
    CUDA_TRY(cudaMalloc(&s->d_partials, sizeof(double) * 2 * (size_t)s->grid));
    s->partials_cap = s->grid;
    if (s->fp32) s->a32.partials = s->d_partials; else s->a64.partials = s->d_partials;
    return ARMON_OK;
}

int apply_tiling(armon_solver* s, const Tiling& t)
{
    s->tuned_seg[0] = t[0];
    s->tuned_seg[1] = t[1];
    s->block = t[2];
    s->split = t[3] != 0 && s->d_faces != nullptr;
    int rc = refill(s);
    return rc != ARMON_OK ? rc : ensure_partials(s);
}

std::array<int, 9> tiling_key(const armon_solver* s)
{
    const armon_params& p = s->p;
    return {p.nx, p.ny, s->fp32 ? 32 : 64, p.scheme, p.projection, p.axis_splitting, s->o.block_lines,
            (s->o.split_pass + 1) | (s->d_faces ? 4 : 0) | (s->o.reuse >= 0 ? 8 : 0), s->ordered ? 1 : 0};
}

// the cost model's tiling in the solver's default form
Tiling model_tiling(const armon_solver* s)
{
    return Tiling{0, 0, s->o.block_lines > 0 ? s->o.block_lines : 128, s->default_split ? 1 : 0};
}

void end_tuning(armon_solver* s)
{
    for (cudaEvent_t e : s->tune.ev) cudaEventDestroy(e);
    s->tune = armon_solver::Tune{};
}

// Called by begin_loop: the cached tiling of this geometry, or the measurement's set-up.
int start_tuning(armon_solver* s)
{
    end_tuning(s);
    if (s->tuned || s->o.seg_len > 0 || s->npass < 2) return ARMON_OK;
    const armon_params& p = s->p;
    if ((int64_t)p.nx * p.ny < (1 << 20)) return ARMON_OK;
    const std::array<int, 9> key = tiling_key(s);
    {
        std::lock_guard<std::mutex> lk(g_tilings_mu);
        auto it = g_tilings.find(key);
        if (it != g_tilings.end()) {
            s->tuned = true;
            return apply_tiling(s, it->second);
        }
    }
    // candidates per form and block size: the model's tiling, then segments aiming at w waves of
    // resident blocks per axis
    const int halo = stencil_reach(&p);
    const int block = s->o.block_lines > 0 ? s->o.block_lines : 128;
    std::vector<int> forms;
    if (s->d_faces && s->o.split_pass == 0) forms = {1, 0}; else forms = {s->split ? 1 : 0};
    auto& T = s->tune;
    for (int form : forms) {
        const int per_sm = form ? sweep_split_blocks_per_sm(s->fp32, p.scheme, p.projection, block)
                                : sweep_blocks_per_sm(s->fp32, p.scheme, p.projection, block);
        const int slots = s->sm_count * per_sm;
        Tiling model{0, 0, block, form};
        for (int axis = 0; axis < 2; axis++) {
            const int n = axis == 0 ? p.nx : p.ny, nl = axis == 0 ? p.ny : p.nx;
            model[axis] = choose_segments(n, nl, block, halo, s->sm_count, 0).seg_len;
        }
        T.cand.push_back(model);
        // FP32 also tries shorter segments (12 and 16 waves): 96-cell segments ran the 8192² run 3 %
        // faster than 144 throughout, whereas FP64's 36-cell segments, which win the cycles the
        // measurement runs on (thin fronts), lost 9 % on the late cycles of the 4096² run
        for (int w : {1, 2, 3, 4, 6, 8, 12, 16}) {
            if (w > 8 && !s->fp32) continue;
            Tiling c{0, 0, block, form};
            for (int axis = 0; axis < 2; axis++) {
                const int n = axis == 0 ? p.nx : p.ny, nl = axis == 0 ? p.ny : p.nx;
                const AxisTiling t = axis_tiling(n, nl, block, n);   // one segment: nlb, spb
                const int per_line = std::max(1, (int)std::lround(double(w) * slots * t.spb / t.nlb));
                c[axis] = std::max(16, (n + per_line - 1) / per_line);
            }
            if (std::find(T.cand.begin(), T.cand.end(), c) == T.cand.end()) T.cand.push_back(c);
        }
    }
    for (size_t i = 0; i < T.cand.size(); i++) T.seq.push_back(i);
    const size_t entries = T.cand.size() + std::min(kTuneFinalists, T.cand.size());
    T.ev.assign(2 * entries, nullptr);
    for (auto& e : T.ev) CUDA_TRY(cudaEventCreate(&e));
    T.key = key;
    T.delay = kTuneDelay;
    T.pos = 0;
    T.warm = true;
    T.active = true;
    return ARMON_OK;
}

// The forward list has run: the finalists go again, backwards.  Returns true when it appended them.
bool add_finalists(armon_solver* s)
{
    auto& T = s->tune;
    if (T.second) return false;
    T.second = true;
    if (cudaEventSynchronize(T.ev[2 * T.seq.size() - 1]) != cudaSuccess) return false;
    std::vector<std::pair<float, size_t>> fwd;
    for (size_t q = 0; q < T.seq.size(); q++) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, T.ev[2 * q], T.ev[2 * q + 1]) != cudaSuccess) return false;
        fwd.emplace_back(ms, T.seq[q]);
    }
    std::sort(fwd.begin(), fwd.end());
    const size_t nf = std::min(kTuneFinalists, fwd.size());
    std::vector<size_t> fin;
    for (size_t k = 0; k < nf; k++) fin.push_back(fwd[k].second);
    std::sort(fin.begin(), fin.end());
    for (size_t k = nf; k-- > 0;) T.seq.push_back(fin[k]);   // backwards in list order
    return true;
}

// The finalists have run again: keep the fastest over both visits if every measured cycle ran, else
// the model's tiling.
int finish_tuning(armon_solver* s)
{
    auto& T = s->tune;
    const size_t nc = T.cand.size();
    std::vector<float> total(nc, 0.f);
    std::vector<int> visits(nc, 0);
    CUDA_TRY(cudaEventSynchronize(T.ev[2 * T.seq.size() - 1]));
    for (size_t q = 0; q < T.seq.size(); q++) {
        float ms = 0;
        CUDA_TRY(cudaEventElapsedTime(&ms, T.ev[2 * q], T.ev[2 * q + 1]));
        total[T.seq[q]] += ms;
        visits[T.seq[q]]++;
    }
    int rc = sync_state(s);
    if (rc != ARMON_OK) return rc;
    const StepState& st = *s->h_state;
    const bool ran = st.status == STATUS_RUNNING && st.cycle == s->cycle0 + s->issued;
    size_t best = 0;
    float best_t = 0.f;
    bool have = false;
    for (size_t i = 0; i < nc; i++) {
        if (visits[i] < 2) continue;
        if (!have || total[i] < best_t) { best = i; best_t = total[i]; have = true; }
    }
    const Tiling choice = ran && have ? T.cand[best] : model_tiling(s);
    const std::array<int, 9> key = T.key;
    end_tuning(s);
    s->tuned = ran;
    rc = apply_tiling(s, choice);
    if (rc == ARMON_OK && ran) {
        std::lock_guard<std::mutex> lk(g_tilings_mu);
        g_tilings[key] = choice;
    }
    return rc;
}

// n cycles of the time loop, the first ones measuring candidate tilings while a measurement runs.
int enqueue(armon_solver* s, int n_cycles)
{
    auto& T = s->tune;
    while (n_cycles > 0 && T.active) {
        int rc = ARMON_OK;
        if (s->cycle0 + s->issued + 1 > s->cfg.max_cycles) {   // the loop ends first: keep the model's tiling
            end_tuning(s);
            rc = apply_tiling(s, model_tiling(s));
            if (rc != ARMON_OK) return rc;
            break;
        }
        if (T.delay > 0) {
            rc = enqueue_direct(s, 1);
            T.delay--;
        } else if (T.warm) {
            // the candidate's first cycle records its units' costs for longest-first dispatch
            rc = apply_tiling(s, T.cand[T.seq[T.pos]]);
            if (rc == ARMON_OK) rc = enqueue_direct(s, 1);
            T.warm = false;
            s->measure_cycles++;
        } else {
            s->measure_cycles++;
            CUDA_TRY(cudaEventRecord(T.ev[2 * T.pos], s->stream));
            rc = enqueue_direct(s, 1);
            if (rc == ARMON_OK) CUDA_TRY(cudaEventRecord(T.ev[2 * T.pos + 1], s->stream));
            T.pos++;
            T.warm = true;
        }
        if (rc != ARMON_OK) return rc;
        s->issued++;
        n_cycles--;
        if (T.pos == T.seq.size() && !add_finalists(s)) {
            rc = finish_tuning(s);
            if (rc != ARMON_OK) return rc;
        }
    }
    return enqueue_steady(s, n_cycles);
}

// p, c, g as update_EOS left them: the EOS of the last pass's input, which the set the current
// state is not in still holds (every pass reads one set and writes the other).  Passes that do not
// store them (materialize_eos < 0) leave this to the moment they are read, the loop ends, or the
// state is settled.
int materialize_eos(armon_solver* s)
{
    if (!s->eos_stale) return ARMON_OK;
    CUDA_TRY(cudaMemcpyAsync(s->h_state, s->d_state, sizeof(StepState), cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    const StepState& st = *s->h_state;
    const int cur = (int)(((int64_t)st.cycle * s->npass + st.buf_base) & 1);
    const int in = cur ^ 1;                      // the set the last pass read
    BeginArgs b{};
    b.nx = s->p.nx; b.ny = s->p.ny;
    b.origin = (int64_t)s->p.nb_ghosts * s->p.row_length + s->p.nb_ghosts;
    b.row_length = s->p.row_length;
    b.gamma = 1.4;
    b.rho = s->arr[in ? 11 : 2]; b.umat = s->arr[in ? 12 : 3]; b.vmat = s->arr[in ? 13 : 4]; b.Emat = s->arr[in ? 14 : 5];
    b.pmat = s->arr[6]; b.cmat = s->arr[7]; b.gmat = s->arr[8];
    b.eos_only = 1;
    CUDA_TRY(launch_begin(b, s->fp32, s->sm_count * 4, s->stream));
    s->launches++;
    s->eos_stale = false;
    return ARMON_OK;
}

// Puts the current state back into set 0 (rho, umat, vmat, Emat) so that the reference's
// arrays hold it, as after the reference's time loop.
int settle(armon_solver* s)
{
    int rc = materialize_eos(s);
    if (rc != ARMON_OK) return rc;
    const StepState& st = *s->h_state;
    int cur = (int)(((int64_t)st.cycle * s->npass + st.buf_base) & 1);
    if (cur == 0) return ARMON_OK;
    size_t bytes = (size_t)s->p.nb_cells * s->elem;
    for (int k = 0; k < 4; k++)
        CUDA_TRY(cudaMemcpyAsync(s->arr[2 + k], s->arr[11 + k], bytes, cudaMemcpyDeviceToDevice, s->stream));
    s->h_state->buf_base = (int)(((int64_t)st.cycle * s->npass) & 1);
    CUDA_TRY(cudaMemcpyAsync(&s->d_state->buf_base, &s->h_state->buf_base, sizeof(int32_t),
                             cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    return ARMON_OK;
}

}  // namespace

extern "C" {

void armon_solver_opts_default(armon_solver_opts* o)
{
    std::memset(o, 0, sizeof(*o));
    o->precision = 64;
    o->cycles_per_graph = 16;
    o->materialize_eos = -1;
}

static int solver_create(const armon_params* p, const armon_solver_opts* opts, double* const* borrowed, void* stream,
                         armon_solver** out)
{
    *out = nullptr;
    int rc = check_supported(p);
    if (rc != ARMON_OK) return rc;
    armon_solver* s = new armon_solver();
    s->p = *p;
    if (opts) s->o = *opts; else armon_solver_opts_default(&s->o);
    if (s->o.precision != 32 && s->o.precision != 64) { delete s; set_error("precision must be 32 or 64"); return ARMON_ERR_PARAMS; }
    s->fp32 = s->o.precision == 32;
    s->elem = s->fp32 ? 4 : 8;
    s->block = s->o.block_lines > 0 ? s->o.block_lines : 128;
    s->ordered = s->o.unit_order >= 0;
    s->split = s->o.split_pass > 0 || (s->o.split_pass == 0 && !s->fp32);
    if (s->block % 32 != 0 || s->block > 128) { delete s; set_error("block_lines must be a multiple of 32, at most 128"); return ARMON_ERR_PARAMS; }
    s->graph_cycles = s->o.cycles_per_graph;
    s->npass = passes_per_cycle(p->axis_splitting);
    cudaError_t e = cudaGetDevice(&s->device);
    if (e != cudaSuccess) { delete s; return cuda_fail(e, "cudaGetDevice"); }
    cudaDeviceGetAttribute(&s->sm_count, cudaDevAttrMultiProcessorCount, s->device);
    if (stream) {
        s->stream = (cudaStream_t)stream;
    } else {
        e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) { delete s; return cuda_fail(e, "cudaStreamCreate"); }
        s->own_stream = true;
    }
    size_t bytes = (size_t)p->nb_cells * s->elem;
    if (borrowed) {
        if (s->fp32) { armon_solver_destroy(s); set_error("borrowed arrays are FP64"); return ARMON_ERR_PARAMS; }
        for (int k = 0; k < 16; k++) {
            if (!borrowed[k]) { armon_solver_destroy(s); set_error("a borrowed array is NULL"); return ARMON_ERR_PARAMS; }
            s->arr[k] = borrowed[k];
        }
        s->owns_arrays = false;
    } else {
        s->owns_arrays = true;
        for (int k = 0; k < 16; k++) {
            e = cudaMalloc(&s->arr[k], bytes);
            if (e != cudaSuccess) {
                armon_solver_destroy(s);
                set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
                return ARMON_ERR_NOMEM;
            }
        }
    }
    e = cudaMalloc(&s->d_state, sizeof(StepState));
    if (e == cudaSuccess) e = cudaMallocHost(&s->h_state, sizeof(StepState));
    // the partial buffers are sized after the geometry is known
    s->cfg = make_step_config(*p);
    if (s->fp32) fill_geom(s, s->a32); else fill_geom(s, s->a64);
    int pblocks = std::max(s->grid, s->sm_count * 8);
    s->cons_grid = s->sm_count * 4;
    if (e == cudaSuccess) e = cudaMalloc(&s->d_partials, sizeof(double) * 2 * (size_t)pblocks);
    s->partials_cap = pblocks;
    if (e == cudaSuccess) e = cudaMalloc(&s->d_cons, sizeof(double) * (2 * (size_t)s->cons_grid + 2));
    if (e == cudaSuccess && s->split) {
        s->face_stride = std::max((int64_t)(p->nx + 5) * p->ny, (int64_t)(p->ny + 5) * p->nx);
        e = cudaMalloc(&s->d_faces, 3 * (size_t)s->face_stride * s->elem);
        if (e == cudaErrorMemoryAllocation && s->o.split_pass == 0) {
            // the split pass is only the default here: run fused passes, which need no face buffer
            cudaGetLastError();
            s->d_faces = nullptr;
            s->face_stride = 0;
            s->split = false;
            e = cudaSuccess;
        }
    }
    s->default_split = s->split;
    if (e == cudaSuccess) e = cudaMemsetAsync(s->d_state, 0, sizeof(StepState), s->stream);
    if (e != cudaSuccess) { armon_solver_destroy(s); return cuda_fail(e, "solver allocation"); }
    std::memset(s->h_state, 0, sizeof(StepState));
    if (s->fp32) fill_geom(s, s->a32); else fill_geom(s, s->a64);
    rc = prepare_order(s);
    if (rc != ARMON_OK) { armon_solver_destroy(s); return rc; }
    *out = s;
    return ARMON_OK;
}

int armon_solver_create(const armon_params* p, const armon_solver_opts* opts, void* stream, armon_solver** out)
{
    return solver_create(p, opts, nullptr, stream, out);
}

int armon_solver_create_with_arrays(const armon_params* p, const armon_solver_opts* opts, double* const arrays[16],
                                    void* stream, armon_solver** out)
{
    return solver_create(p, opts, arrays, stream, out);
}

void armon_solver_destroy(armon_solver* s)
{
    if (!s) return;
    if (s->stream) cudaStreamSynchronize(s->stream);
    end_tuning(s);
    if (s->graph) cudaGraphExecDestroy(s->graph);
    if (s->owns_arrays)
        for (auto& a : s->arr) if (a) cudaFree(a);
    if (s->d_state) cudaFree(s->d_state);
    if (s->h_state) cudaFreeHost(s->h_state);
    if (s->d_partials) cudaFree(s->d_partials);
    if (s->d_cons) cudaFree(s->d_cons);
    if (s->stage) cudaFree(s->stage);
    if (s->d_faces) cudaFree(s->d_faces);
    if (s->d_order) cudaFree(s->d_order);
    if (s->d_cost) cudaFree(s->d_cost);
    if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

int armon_solver_begin_loop(armon_solver* s)
{
    // time_loop's start (src/armon_2D.cpp:327-346): cycle = 0, time = 0, dts = 0, update_axis(X),
    // update_EOS, and here also the cycle-0 dt_CFL.  The shadow set starts as a copy of the state
    // so that its untouched ghost cells hold the same values.
    if (s->begun) {
        int rc = sync_state(s);
        if (rc == ARMON_OK) rc = settle(s);
        if (rc != ARMON_OK) return rc;
    }
    size_t bytes = (size_t)s->p.nb_cells * s->elem;
    for (int k = 0; k < 4; k++)
        CUDA_TRY(cudaMemcpyAsync(s->arr[11 + k], s->arr[2 + k], bytes, cudaMemcpyDeviceToDevice, s->stream));
    BeginArgs b{};
    b.nx = s->p.nx; b.ny = s->p.ny;
    b.origin = (int64_t)s->p.nb_ghosts * s->p.row_length + s->p.nb_ghosts;
    b.row_length = s->p.row_length;
    b.gamma = 1.4;
    b.rho = s->arr[2]; b.umat = s->arr[3]; b.vmat = s->arr[4]; b.Emat = s->arr[5];
    b.pmat = s->arr[6]; b.cmat = s->arr[7]; b.gmat = s->arr[8];
    b.state = s->d_state;
    b.cfg = s->cfg;
    b.partials = s->d_partials;
    b.buf_base = 0;
    CUDA_TRY(cudaMemsetAsync(&s->d_state->counter, 0, sizeof(uint32_t), s->stream));
    CUDA_TRY(launch_begin(b, s->fp32, s->sm_count * 4, s->stream));
    s->launches++;
    s->begun = true;
    s->eos_stale = false;
    s->issued = 0;
    int rc = sync_state(s);
    s->cycle0 = s->h_state->cycle;
    if (rc == ARMON_OK) rc = start_tuning(s);
    return rc;
}

int armon_solver_init_test(armon_solver* s)
{
    const armon_params& p = s->p;
    InitArgs a{};
    a.row_length = p.row_length; a.nb_ghosts = p.nb_ghosts; a.nx = p.nx; a.ny = p.ny;
    a.pos_x = 0; a.pos_y = 0; a.g_nx = p.nx; a.g_ny = p.ny;
    a.sx = p.domain_size[0]; a.sy = p.domain_size[1]; a.ox = p.domain_origin[0]; a.oy = p.domain_origin[1];
    double dx = p.domain_size[0] / double(p.nx), dy = p.domain_size[1] / double(p.ny);
    a.test_option = armon_test_option(&p, dx, dy);
    a.test = p.test;
    a.debug_indexes = 0;
    a.tp = make_test_params(p.test, a.test_option);
    InitPtrs ptr{s->arr[0], s->arr[1], s->arr[2], s->arr[5], s->arr[3], s->arr[4], s->arr[15],
                 s->arr[6], s->arr[7], s->arr[8], s->arr[9], s->arr[10]};
    CUDA_TRY(launch_init(a, p.nb_cells, ptr, s->fp32, s->stream));
    s->launches++;
    return armon_solver_begin_loop(s);
}

int armon_solver_enqueue_cycles(armon_solver* s, int n_cycles)
{
    if (!s->begun) { set_error("the time loop has not been started (init_test / begin_loop)"); return ARMON_ERR_STATE; }
    return enqueue(s, n_cycles);
}

int armon_solver_run(armon_solver* s, int cycle_limit)
{
    if (!s->begun) { set_error("the time loop has not been started (init_test / begin_loop)"); return ARMON_ERR_STATE; }
    int rc = sync_state(s);
    if (rc != ARMON_OK) return rc;
    int issued = 0;
    for (;;) {
        const StepState& st = *s->h_state;
        if (st.status == STATUS_INVALID_DT) {
            set_error("invalid dt at cycle " + std::to_string(st.cycle));
            return ARMON_ERR_INVALID_DT;
        }
        bool running = st.time < s->cfg.max_time && st.cycle < s->cfg.max_cycles;
        if (!running && s->tune.active) {
            // the loop ended while measuring: the model's tiling, nothing cached
            end_tuning(s);
            rc = apply_tiling(s, model_tiling(s));
            if (rc != ARMON_OK) return rc;
        }
        if (!running || (cycle_limit > 0 && issued >= cycle_limit)) break;
        // at most the cycles left before max_cycles; when time decides, one graph batch at a time
        int left = s->cfg.max_cycles - st.cycle;
        int n = std::min(left, s->graph_cycles > 0 ? s->graph_cycles : 16);
        if (cycle_limit > 0) n = std::min(n, cycle_limit - issued);
        rc = enqueue(s, n);
        if (rc != ARMON_OK) return rc;
        issued += n;
        rc = sync_state(s);
        if (rc != ARMON_OK) return rc;
    }
    return settle(s);
}

int armon_solver_sync_params(armon_solver* s, armon_params* p, int32_t* status)
{
    int rc = sync_state(s);
    if (rc != ARMON_OK) return rc;
    const StepState& st = *s->h_state;
    *p = s->p;
    p->cycle = st.cycle;
    p->time = st.time;
    p->current_cycle_dt = st.current_dt;
    p->next_cycle_dt = st.next_dt;
    if (status) *status = st.status;
    return ARMON_OK;
}

static int current_index(armon_solver* s, int which)
{
    // rho, umat, vmat, Emat live in the set the last pass wrote
    if (which < 2 || which > 5) return which;
    const StepState& st = *s->h_state;
    int cur = (int)(((int64_t)st.cycle * s->npass + st.buf_base) & 1);
    return cur ? which + 9 : which;
}

int armon_solver_download(armon_solver* s, int which, double* host)
{
    if (which < 0 || which > 15) { set_error("array index out of range"); return ARMON_ERR_PARAMS; }
    int rc = (which >= 6 && which <= 8) ? materialize_eos(s) : ARMON_OK;
    if (rc == ARMON_OK) rc = sync_state(s);
    if (rc != ARMON_OK) return rc;
    int k = current_index(s, which);
    size_t n = (size_t)s->p.nb_cells;
    if (!s->fp32) {
        CUDA_TRY(cudaMemcpyAsync(host, s->arr[k], n * 8, cudaMemcpyDeviceToHost, s->stream));
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        return ARMON_OK;
    }
    rc = ensure_stage(s);
    if (rc != ARMON_OK) return rc;
    widen_kernel<<<s->sm_count * 8, 256, 0, s->stream>>>((const float*)s->arr[k], s->stage, (int64_t)n);
    CUDA_TRY(cudaGetLastError());
    s->launches++;
    CUDA_TRY(cudaMemcpyAsync(host, s->stage, n * 8, cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    return ARMON_OK;
}

int armon_solver_upload(armon_solver* s, int which, const double* host)
{
    if (which < 0 || which > 15) { set_error("array index out of range"); return ARMON_ERR_PARAMS; }
    int rc = (which >= 6 && which <= 8) ? materialize_eos(s) : ARMON_OK;
    if (rc == ARMON_OK) rc = sync_state(s);
    if (rc != ARMON_OK) return rc;
    int k = current_index(s, which);
    size_t n = (size_t)s->p.nb_cells;
    if (!s->fp32) {
        CUDA_TRY(cudaMemcpyAsync(s->arr[k], host, n * 8, cudaMemcpyHostToDevice, s->stream));
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        return ARMON_OK;
    }
    rc = ensure_stage(s);
    if (rc != ARMON_OK) return rc;
    CUDA_TRY(cudaMemcpyAsync(s->stage, host, n * 8, cudaMemcpyHostToDevice, s->stream));
    narrow_kernel<<<s->sm_count * 8, 256, 0, s->stream>>>(s->stage, (float*)s->arr[k], (int64_t)n);
    CUDA_TRY(cudaGetLastError());
    s->launches++;
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    return ARMON_OK;
}

double* armon_solver_device_array(armon_solver* s, int which)
{
    if (s->fp32 || which < 0 || which > 15) return nullptr;
    if (which >= 6 && which <= 8 && materialize_eos(s) != ARMON_OK) return nullptr;
    if (sync_state(s) != ARMON_OK) return nullptr;
    return (double*)s->arr[current_index(s, which)];
}

int armon_solver_conservation(armon_solver* s, double* mass, double* energy)
{
    int rc = sync_state(s);
    if (rc != ARMON_OK) return rc;
    ConsArgs a{};
    a.nx = s->p.nx; a.ny = s->p.ny;
    a.origin = (int64_t)s->p.nb_ghosts * s->p.row_length + s->p.nb_ghosts;
    a.row_length = s->p.row_length;
    // conservation_vars uses p.dx of the current axis (src/armon_2D.cpp:293): after a full loop
    // the driver's current axis is the last pass's axis.
    int axis = 0;
    if (s->h_state->cycle > 0) {
        double f;
        split_axis(s->p.axis_splitting, s->h_state->cycle - 1, s->npass - 1, &axis, &f);
    }
    double dx = axis == 0 ? s->p.domain_size[0] / double(s->p.nx) : s->p.domain_size[1] / double(s->p.ny);
    a.ds = dx * dx;
    a.rho = s->arr[current_index(s, 2)];
    a.Emat = s->arr[current_index(s, 5)];
    a.partials = s->d_cons;
    a.out = s->d_cons + 2 * s->cons_grid;
    CUDA_TRY(launch_conservation(a, s->fp32, s->cons_grid, s->stream));
    double out[2];
    CUDA_TRY(cudaMemcpyAsync(out, a.out, sizeof(out), cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    *mass = out[0];
    *energy = out[1];
    return ARMON_OK;
}

int64_t armon_solver_kernel_launches(armon_solver* s) { return s->launches; }

int armon_solver_tiling(armon_solver* s, int32_t seg_len[2], int32_t blocks[2])
{
    for (int axis = 0; axis < 2; axis++) {
        const int sl = s->fp32 ? s->a32.geom[axis].seg_len : s->a64.geom[axis].seg_len;
        const int nb = s->fp32 ? s->a32.geom[axis].blocks : s->a64.geom[axis].blocks;
        if (seg_len) seg_len[axis] = sl;
        if (blocks) blocks[axis] = nb;
    }
    return ARMON_OK;
}

int armon_solver_block_lines(const armon_solver* s) { return s->block; }

int armon_solver_tuning(const armon_solver* s) { return s->tune.active ? 1 : 0; }

int64_t armon_solver_measurement_cycles(const armon_solver* s) { return s->measure_cycles; }

int armon_solver_split_pass(const armon_solver* s) { return s->split ? 1 : 0; }

void armon_tiling_cache_clear(void)
{
    std::lock_guard<std::mutex> lk(g_tilings_mu);
    g_tilings.clear();
}

int armon_solve_host(const armon_params* p, const armon_solver_opts* opts, const double* const in[4],
                     double* const out[5], armon_params* final_state)
{
    armon_solver* s = nullptr;
    int rc = armon_solver_create(p, opts, nullptr, &s);
    if (rc != ARMON_OK) return rc;
    rc = armon_solver_init_test(s);                 // geometry, mask and the ghosts of init_test
    static const int which_in[4] = {2, 3, 4, 5};
    for (int k = 0; k < 4 && rc == ARMON_OK; k++)
        if (in && in[k]) rc = armon_solver_upload(s, which_in[k], in[k]);
    if (rc == ARMON_OK && in) rc = armon_solver_begin_loop(s);
    if (rc == ARMON_OK) rc = armon_solver_run(s, 0);
    static const int which_out[5] = {2, 3, 4, 5, 6};
    for (int k = 0; k < 5 && rc == ARMON_OK; k++)
        if (out && out[k]) rc = armon_solver_download(s, which_out[k], out[k]);
    if (rc == ARMON_OK && final_state) rc = armon_solver_sync_params(s, final_state, nullptr);
    armon_solver_destroy(s);
    return rc;
}

}  // extern "C"
