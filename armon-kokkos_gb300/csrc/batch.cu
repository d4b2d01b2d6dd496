// batch.cu -- many independent domains advanced together (include/armon_gb300.h, armon_batch_*).
//
// Every domain keeps its own state (two buffer sets, p/c/g, dt partials) in one allocation from
// the batch's stream-ordered memory pool, and its own 48-byte step state in a slot of a device
// array.  A pass over the batch is one launch of sweep_batch_kernel: the launch table lists the
// running domains and the first grid block of each (enough blocks for its larger axis), so one
// launch covers every domain, each with its own dt, time and cycle.  The table is rebuilt when
// domains join or finish; cycles are captured in a CUDA graph per table.  The host reads all
// step states back with one copy per graph batch.
#include <algorithm>
#include <array>
#include <cstring>
#include <queue>
#include <string>
#include <vector>

#include "armon_gb300.h"
#include "host_common.h"
#include "launch.h"
#include "order.cuh"
#include "solver_common.h"

using namespace armon;

namespace {

constexpr int kMaxDomains = 8192;

// Candidates of the autotuned schedule (block waves per launch), and the least running cells for
// which tuning is worth a graph batch per candidate.
constexpr int kWaves[] = {2, 4, 8, 16, 64};
constexpr int kNumWaves = sizeof(kWaves) / sizeof(kWaves[0]);
constexpr int64_t kTuneMinCells = 1 << 21;

struct Tuner {
    int phase = 0;              // 0 never tuned, 1 timing candidates, 2 tuned
    int cand = 0;
    bool launched = false;      // the current candidate's graph batch is on the stream
    double work = 0;            // its cell-updates
    double rate[kNumWaves] = {};
    int64_t tuned_cells = 0;    // running cells when tuning started
};

size_t align256(size_t n) { return (n + 255) & ~size_t(255); }

struct Dom {
    bool used = false;
    bool done = false;
    armon_params p{};
    void* chunk = nullptr;
    int64_t bytes = 0;
    void* arr[11] = {};           // set 0 (rho umat vmat Emat), set 1 (same), pmat cmat gmat
    double* partials = nullptr;
    int64_t npartials = 0;        // pairs
    void* faces = nullptr;        // split passes: 3 face arrays of face_values(p) values
    int seg_len = 0;
};

// values per face array of a split pass (sweep_split.cuh): the larger axis's (n + 5) * nlines
int64_t face_values(const armon_params& p)
{
    return std::max((int64_t)(p.nx + 5) * p.ny, (int64_t)(p.ny + 5) * p.nx);
}

// FP64 batches run split passes (face launch, cell launch) unless told otherwise
bool split_default(int32_t precision) { return precision != 32; }



int64_t partial_pairs(const armon_params& p, int block)
{
    // an upper bound of the blocks either axis may use (segments of at least 16 cells), and the
    // grid of the EOS + first dt kernel
    int64_t bx = (int64_t)std::max(1, (p.ny + block - 1) / block) * std::max(1, p.nx / 16 + 1);
    int64_t by = (int64_t)std::max(1, (p.nx + block - 1) / block) * std::max(1, p.ny / 16 + 1);
    return std::max<int64_t>(std::max(bx, by), 152 * 4);
}

int64_t domain_bytes(const armon_params& p, size_t elem, bool split)
{
    return (int64_t)(11 * align256((size_t)p.nb_cells * elem) + align256(16 * (size_t)partial_pairs(p, 32)) +
                     (split ? 3 * align256((size_t)face_values(p) * elem) : 0));
}

}  // namespace

struct armon_batch {
    armon_batch_opts o{};
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    cudaMemPool_t pool = nullptr;
    int sm_count = 152;
    bool fp32 = false;
    size_t elem = 8;
    int scheme = -1, proj = -1, splitting = -1, npass = 2;
    std::vector<Dom> doms;
    StepState* d_states = nullptr;
    StepState* h_states = nullptr;
    void* d_args = nullptr;
    int* d_offsets = nullptr;
    std::vector<int> table;
    int total_blocks = 0;
    int blocks_per_sm = 0;        // of the batch kernel (0: not yet known)
    int waves = 8;                // block waves per launch the schedule aims for
    Tuner tune;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    bool dirty = true;
    cudaGraphExec_t graph = nullptr;
    int64_t bytes = 0;
    int64_t launches = 0;
    bool split = true;            // passes as a face launch and a cell launch (sweep_split.cuh)
    bool ordered = true;          // longest-first dispatch of each pass's blocks
    uint32_t* d_order = nullptr;  // per pass (and per half of a split pass) order_cap block indices
    uint32_t* d_cost = nullptr;   // the same for the costs
    int order_cap = 0;
};

namespace {

int cuda_fail(cudaError_t e, const char* what)
{
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? ARMON_ERR_NOMEM : ARMON_ERR_CUDA;
}

#define CUDA_TRY(expr)                                            \
    do {                                                          \
        cudaError_t e_ = (expr);                                  \
        if (e_ != cudaSuccess) return cuda_fail(e_, #expr);       \
    } while (0)

// FP64 <-> FP32 conversion of staged arrays on the device (round to nearest, as the host's cast;
// widening is exact); the staging array comes from the batch's pool for the one transfer.
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

template <class T>
DomainBuffers<T> buffers(const Dom& d)
{
    T* const* a = reinterpret_cast<T* const*>(d.arr);
    return DomainBuffers<T>{{{a[0], a[1], a[2], a[3]}, {a[4], a[5], a[6], a[7]}}, a[8], a[9], a[10]};
}

// Segment lengths of the running domains, both axes, for one launch over all of them.  Each axis
// starts as whole lines (one segment per line); then the longest segments are split while they
// are longer than 1 / waves of the average load of a resident block slot, and never below 16
// cells.  A launch lasts at least as long as its longest block and at least as long as its total
// work over the slots; a block's work is seg_len + 1.2 * halo thread-steps (the halo is recomputed
// per segment).  Few waves keep the recomputation low, more waves shorten the tail of the launch
// where the last blocks run alone; the batch autotunes the number.
std::vector<std::array<int, 2>> schedule_segments(const armon_batch* b)
{
    const int block = b->o.block_lines;
    const double slots = double(b->sm_count) * std::max(1, b->blocks_per_sm);
    const size_t nd = b->table.size();
    std::vector<std::array<int, 2>> seg(nd, {0, 0});
    struct Item {
        int n, nlines, nseg;
        double halo, len, blocks;
    };
    for (int axis = 0; axis < 2; axis++) {
        std::vector<Item> it(nd);
        std::priority_queue<std::pair<double, int>> heap;   // (block length, item)
        double total = 0;
        for (size_t k = 0; k < nd; k++) {
            const armon_params& p = b->doms[b->table[k]].p;
            Item& x = it[k];
            x.n = axis == 0 ? p.nx : p.ny;
            x.nlines = axis == 0 ? p.ny : p.nx;
            x.nseg = 1;
            x.halo = 1.2 * stencil_reach(&p);
            const AxisTiling t = axis_tiling(x.n, x.nlines, block, x.n);
            x.len = t.seg_len + x.halo;
            x.blocks = t.blocks;
            total += x.blocks * x.len;
            heap.push({x.len, (int)k});
        }
        while (!heap.empty()) {
            const int k = heap.top().second;
            Item& x = it[k];
            if (x.len <= total / (slots * b->waves)) break;
            const int nseg = std::max(x.nseg + 1, x.nseg * 5 / 4);
            const int sl = (x.n + nseg - 1) / nseg;
            if (sl < 16) break;                   // the longest block cannot get shorter
            heap.pop();
            const AxisTiling t = axis_tiling(x.n, x.nlines, block, sl);
            total -= x.blocks * x.len;
            x.nseg = t.nseg;
            x.len = t.seg_len + x.halo;
            x.blocks = t.blocks;
            total += x.blocks * x.len;
            heap.push({x.len, k});
        }
        for (size_t k = 0; k < nd; k++) seg[k][axis] = (it[k].n + it[k].nseg - 1) / it[k].nseg;
    }
    return seg;
}

// order / cost arrays: one per pass of a cycle, and one more per pass for the face halves
int order_arrays(const armon_batch* b) { return b->npass * (b->split ? 2 : 1); }

template <class T>
int rebuild_t(armon_batch* b)
{
    b->table.clear();
    for (int i = 0; i < (int)b->doms.size(); i++)
        if (b->doms[i].used && !b->doms[i].done) b->table.push_back(i);
    if (b->blocks_per_sm == 0 && !b->table.empty())
        b->blocks_per_sm = b->split ? sweep_batch_split_blocks_per_sm(b->fp32, b->scheme, b->proj, b->o.block_lines)
                                    : sweep_batch_blocks_per_sm(b->fp32, b->scheme, b->proj, b->o.block_lines);
    const std::vector<std::array<int, 2>> sched = schedule_segments(b);
    std::vector<SweepArgs<T>> args(b->table.size());
    std::vector<int> offsets(b->table.size() + 1, 0);
    for (size_t k = 0; k < b->table.size(); k++) {
        Dom& d = b->doms[b->table[k]];
        const int fixed = d.seg_len > 0 ? d.seg_len : b->o.seg_len;
        const int forced[2] = {fixed > 0 ? fixed : sched[k][0], fixed > 0 ? fixed : sched[k][1]};
        int nb = make_sweep_args<T>(d.p, b->npass, b->o.block_lines, b->sm_count, forced, buffers<T>(d),
                                    b->d_states + b->table[k], d.partials, 0, b->o.reuse >= 0 ? 1 : 0, args[k]);
        if (b->split) {
            args[k].faces = static_cast<T*>(d.faces);
            args[k].face_stride = face_values(d.p);
        }
        if (nb > d.npartials) { set_error("domain needs more partial slots than allotted"); return ARMON_ERR_STATE; }
        offsets[k + 1] = offsets[k] + nb;
    }
    b->total_blocks = offsets.back();
    if (b->ordered && !b->table.empty()) {
        // a new table: index order until its blocks have costs
        if (b->total_blocks > b->order_cap) {
            CUDA_TRY(cudaStreamSynchronize(b->stream));
            cudaFree(b->d_order);
            cudaFree(b->d_cost);
            b->d_order = b->d_cost = nullptr;
            b->order_cap = 0;
            const int cap = b->total_blocks + b->total_blocks / 4;
            CUDA_TRY(cudaMalloc(&b->d_order, sizeof(uint32_t) * kMaxOrderArrays * (size_t)cap));
            CUDA_TRY(cudaMalloc(&b->d_cost, sizeof(uint32_t) * kMaxOrderArrays * (size_t)cap));
            b->order_cap = cap;
        }
        const int total = b->order_cap * order_arrays(b);
        reset_order_kernel<<<std::max(1, std::min(b->sm_count * 4, (total + 255) / 256)), 256, 0, b->stream>>>(
            b->d_order, b->d_cost, b->order_cap, order_arrays(b));
        CUDA_TRY(cudaGetLastError());
        b->launches++;
    }
    if (!b->table.empty()) {
        CUDA_TRY(cudaMemcpyAsync(b->d_args, args.data(), args.size() * sizeof(SweepArgs<T>), cudaMemcpyHostToDevice,
                                 b->stream));
        CUDA_TRY(cudaMemcpyAsync(b->d_offsets, offsets.data(), offsets.size() * sizeof(int), cudaMemcpyHostToDevice,
                                 b->stream));
        CUDA_TRY(cudaStreamSynchronize(b->stream));   // the host vectors go out of scope
    }
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    b->dirty = false;
    return ARMON_OK;
}

int rebuild(armon_batch* b) { return b->fp32 ? rebuild_t<float>(b) : rebuild_t<double>(b); }

int64_t table_cells(const armon_batch* b)
{
    int64_t c = 0;
    for (int i : b->table) c += (int64_t)b->doms[i].p.nx * b->doms[i].p.ny;
    return c;
}

bool schedule_fixed(const armon_batch* b) { return b->o.waves > 0 || b->o.seg_len > 0; }

// Online autotuning of the schedule: each candidate number of waves is timed with CUDA events over
// one graph batch of real cycles (results do not depend on the segments, so nothing is wasted);
// the fastest is kept until the running cells change by a factor of two.
int tune_collect(armon_batch* b)
{
    Tuner& t = b->tune;
    if (t.phase != 1 || !t.launched) return ARMON_OK;
    CUDA_TRY(cudaEventSynchronize(b->ev1));
    float ms = 0;
    CUDA_TRY(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    t.rate[t.cand] = ms > 0 ? t.work / ms : 0;
    t.launched = false;
    if (++t.cand < kNumWaves) {
        b->waves = kWaves[t.cand];
    } else {
        int best = 0;
        for (int k = 1; k < kNumWaves; k++)
            if (t.rate[k] > t.rate[best]) best = k;
        b->waves = kWaves[best];
        t.phase = 2;
    }
    b->dirty = true;
    return ARMON_OK;
}

bool tune_start(armon_batch* b)
{
    Tuner& t = b->tune;
    if (schedule_fixed(b) || t.phase == 1) return false;
    const int64_t cells = table_cells(b);
    if (cells < kTuneMinCells) return false;
    if (t.phase == 2 && cells * 2 > t.tuned_cells && cells < t.tuned_cells * 2) return false;
    t.phase = 1;
    t.cand = 0;
    t.launched = false;
    t.tuned_cells = cells;
    b->waves = kWaves[0];
    b->dirty = true;
    return true;
}

int enqueue_direct(armon_batch* b, int n)
{
    const int nd = (int)b->table.size();
    for (int c = 0; c < n; c++) {
        for (int k = 0; k < b->npass; k++) {
            bool last = k == b->npass - 1;
            BatchOrder ord{nullptr, nullptr}, ford{nullptr, nullptr};
            if (b->ordered) {
                ord.order = b->d_order + (size_t)k * b->order_cap;
                ord.cost = b->d_cost + (size_t)k * b->order_cap;
                if (b->split) {
                    ford.order = b->d_order + (size_t)(b->npass + k) * b->order_cap;
                    ford.cost = b->d_cost + (size_t)(b->npass + k) * b->order_cap;
                }
            }
            cudaError_t e;
            if (b->split)
                e = b->fp32 ? launch_sweep_batch_split((const SweepArgs<float>*)b->d_args, b->d_offsets, nd, b->total_blocks,
                                                       k, ford, ord, b->scheme, b->proj, last, b->o.block_lines, b->stream)
                            : launch_sweep_batch_split((const SweepArgs<double>*)b->d_args, b->d_offsets, nd, b->total_blocks,
                                                       k, ford, ord, b->scheme, b->proj, last, b->o.block_lines, b->stream);
            else
                e = b->fp32 ? launch_sweep_batch((const SweepArgs<float>*)b->d_args, b->d_offsets, nd, b->total_blocks, k,
                                                 ord, b->scheme, b->proj, last, b->o.block_lines, b->stream)
                            : launch_sweep_batch((const SweepArgs<double>*)b->d_args, b->d_offsets, nd, b->total_blocks, k,
                                                 ord, b->scheme, b->proj, last, b->o.block_lines, b->stream);
            if (e != cudaSuccess) return cuda_fail(e, "batch sweep launch");
            b->launches += b->split ? 2 : 1;
        }
        if (b->ordered) {
            UnitCounts counts;
            for (int a = 0; a < kMaxOrderArrays; a++) counts.n[a] = b->total_blocks;
            order_units_kernel<<<order_arrays(b), 1024, 0, b->stream>>>(b->d_cost, b->d_order, b->order_cap, counts);
            CUDA_TRY(cudaGetLastError());
            b->launches++;
        }
    }
    return ARMON_OK;
}

int enqueue(armon_batch* b, int n)
{
    int rc = tune_collect(b);
    if (rc != ARMON_OK) return rc;
    if (b->dirty) {
        rc = rebuild(b);
        if (rc != ARMON_OK) return rc;
    }
    if (tune_start(b)) {
        rc = rebuild(b);
        if (rc != ARMON_OK) return rc;
    }
    if (b->table.empty() || n <= 0) return ARMON_OK;
    const int gc = b->o.cycles_per_graph;
    if (gc > 0 && n >= gc) {
        if (!b->graph) {
            cudaGraph_t g = nullptr;
            int64_t saved = b->launches;
            CUDA_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
            int rc = enqueue_direct(b, gc);
            cudaError_t e = cudaStreamEndCapture(b->stream, &g);
            b->launches = saved;
            if (rc != ARMON_OK) { if (g) cudaGraphDestroy(g); return rc; }
            if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
            e = cudaGraphInstantiate(&b->graph, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) { b->graph = nullptr; return cuda_fail(e, "cudaGraphInstantiate"); }
        }
        while (n >= gc) {
            const bool timed = b->tune.phase == 1 && !b->tune.launched;
            if (timed) CUDA_TRY(cudaEventRecord(b->ev0, b->stream));
            CUDA_TRY(cudaGraphLaunch(b->graph, b->stream));
            if (timed) {
                CUDA_TRY(cudaEventRecord(b->ev1, b->stream));
                b->tune.launched = true;
                b->tune.work = double(table_cells(b)) * gc;
            }
            b->launches += (int64_t)gc * (b->npass * (b->split ? 2 : 1) + (b->ordered ? 1 : 0));
            n -= gc;
        }
    }
    return enqueue_direct(b, n);
}

int max_slot(const armon_batch* b)
{
    int m = 0;
    for (int i = 0; i < (int)b->doms.size(); i++)
        if (b->doms[i].used) m = i + 1;
    return m;
}

bool loop_running(const Dom& d, const StepState& st)
{
    return st.status == STATUS_RUNNING && st.time < d.p.max_time && st.cycle < d.p.max_cycles;
}

int current_set(const armon_batch* b, int id)
{
    const StepState& st = b->h_states[id];
    return (int)(((int64_t)st.cycle * b->npass + st.buf_base) & 1);
}

}  // namespace

extern "C" {

void armon_batch_opts_default(armon_batch_opts* o)
{
    std::memset(o, 0, sizeof(*o));
    o->precision = 64;
    o->cycles_per_graph = 8;
    o->block_lines = 128;
    o->waves = 0;
}

int64_t armon_batch_domain_bytes(const armon_params* p, int32_t precision)
{
    return domain_bytes(*p, precision == 32 ? 4 : 8, split_default(precision));
}

int armon_batch_create(const armon_batch_opts* opts, void* stream, armon_batch** out)
{
    *out = nullptr;
    armon_batch* b = new armon_batch();
    if (opts) b->o = *opts; else armon_batch_opts_default(&b->o);
    if (b->o.precision != 32 && b->o.precision != 64) { delete b; set_error("precision must be 32 or 64"); return ARMON_ERR_PARAMS; }
    if (b->o.block_lines <= 0) b->o.block_lines = 128;
    if (b->o.block_lines % 32 != 0 || b->o.block_lines > 128) {
        delete b;
        set_error("block_lines must be a multiple of 32, at most 128");
        return ARMON_ERR_PARAMS;
    }
    b->fp32 = b->o.precision == 32;
    b->elem = b->fp32 ? 4 : 8;
    b->ordered = b->o.unit_order >= 0;
    b->split = b->o.split_pass > 0 || (b->o.split_pass == 0 && split_default(b->o.precision));
    if (b->o.waves > 0) b->waves = b->o.waves;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = cudaSuccess;
    if (stream) {
        b->stream = (cudaStream_t)stream;
    } else {
        e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
        b->own_stream = e == cudaSuccess;
    }
    if (e == cudaSuccess) {
        // a pool of its own that keeps freed memory for the next domain
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        e = cudaMemPoolCreate(&b->pool, &props);
        if (e == cudaSuccess) {
            uint64_t keep = UINT64_MAX;
            e = cudaMemPoolSetAttribute(b->pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
    }
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev1);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_states, sizeof(StepState) * kMaxDomains);
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_states, sizeof(StepState) * kMaxDomains);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_args, sizeof(SweepArgs<double>) * kMaxDomains);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_offsets, sizeof(int) * (kMaxDomains + 1));
    if (e != cudaSuccess) {
        armon_batch_destroy(b);
        return cuda_fail(e, "batch allocation");
    }
    std::memset(b->h_states, 0, sizeof(StepState) * kMaxDomains);
    *out = b;
    return ARMON_OK;
}

void armon_batch_destroy(armon_batch* b)
{
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (auto& d : b->doms)
        if (d.used && d.chunk) cudaFreeAsync(d.chunk, b->stream);
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->pool) cudaMemPoolDestroy(b->pool);
    if (b->d_states) cudaFree(b->d_states);
    if (b->h_states) cudaFreeHost(b->h_states);
    if (b->d_args) cudaFree(b->d_args);
    if (b->d_offsets) cudaFree(b->d_offsets);
    if (b->d_order) cudaFree(b->d_order);
    if (b->d_cost) cudaFree(b->d_cost);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

}  // extern "C"

namespace {

// armon_batch_add / armon_batch_add_sod: the initial state from init_test, then from the host
// arrays `init` or the interface `sod` when given.
int add_domain(armon_batch* b, const armon_params* p, const double* const init[4], const armon_sod_interface* sod,
               int32_t* id)
{
    *id = -1;
    int rc = check_supported(p);
    if (rc != ARMON_OK) return rc;
    if (b->scheme < 0) {
        b->scheme = p->scheme;
        b->proj = p->projection;
        b->splitting = p->axis_splitting;
        b->npass = passes_per_cycle(p->axis_splitting);
    } else if (b->scheme != p->scheme || b->proj != p->projection || b->splitting != p->axis_splitting) {
        set_error("all domains of a batch share scheme, projection and axis splitting");
        return ARMON_ERR_PARAMS;
    }
    int64_t need = domain_bytes(*p, b->elem, b->split);
    if (b->o.memory_budget > 0 && b->bytes + need > b->o.memory_budget) {
        set_error("the batch's memory budget would be exceeded");
        return ARMON_ERR_NOMEM;
    }
    int slot = -1;
    for (int i = 0; i < (int)b->doms.size(); i++)
        if (!b->doms[i].used) { slot = i; break; }
    if (slot < 0) {
        if ((int)b->doms.size() >= kMaxDomains) { set_error("too many domains in one batch"); return ARMON_ERR_PARAMS; }
        b->doms.emplace_back();
        slot = (int)b->doms.size() - 1;
    }
    Dom d;
    d.p = *p;
    d.bytes = need;
    cudaError_t e = cudaMallocFromPoolAsync(&d.chunk, (size_t)need, b->pool, b->stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMallocFromPoolAsync");
    char* base = (char*)d.chunk;
    size_t arr_bytes = align256((size_t)p->nb_cells * b->elem);
    for (int k = 0; k < 11; k++) d.arr[k] = base + k * arr_bytes;
    d.partials = (double*)(base + 11 * arr_bytes);
    d.npartials = partial_pairs(*p, 32);
    if (b->split) d.faces = base + 11 * arr_bytes + align256(16 * (size_t)d.npartials);
    b->doms[slot] = d;
    b->doms[slot].used = true;
    b->bytes += need;
    Dom& dd = b->doms[slot];

    // init_test on the device (ghosts, p = 0, c = 1 where the pass never writes), then the host state
    InitArgs a{};
    a.row_length = p->row_length; a.nb_ghosts = p->nb_ghosts; a.nx = p->nx; a.ny = p->ny;
    a.pos_x = 0; a.pos_y = 0; a.g_nx = p->nx; a.g_ny = p->ny;
    a.sx = p->domain_size[0]; a.sy = p->domain_size[1]; a.ox = p->domain_origin[0]; a.oy = p->domain_origin[1];
    double dx = p->domain_size[0] / double(p->nx), dy = p->domain_size[1] / double(p->ny);
    a.test_option = armon_test_option(p, dx, dy);
    a.test = p->test;
    a.tp = make_test_params(p->test, a.test_option);
    InitPtrs ip{nullptr, nullptr, dd.arr[0], dd.arr[3], dd.arr[1], dd.arr[2], nullptr, dd.arr[8], dd.arr[9], dd.arr[10],
                nullptr, nullptr};
    CUDA_TRY(launch_init(a, p->nb_cells, ip, b->fp32, b->stream));
    b->launches++;
    if (sod) {
        SodInit si{};
        si.row_length = p->row_length; si.nb_ghosts = p->nb_ghosts; si.nx = p->nx; si.ny = p->ny;
        si.sx = p->domain_size[0]; si.sy = p->domain_size[1]; si.ox = p->domain_origin[0]; si.oy = p->domain_origin[1];
        si.shape = sod->shape;
        si.cx = sod->cx; si.cy = sod->cy; si.nxv = sod->nx; si.nyv = sod->ny; si.offset = sod->offset; si.r2 = sod->r2;
        const double gm1 = 1.4 - 1.0;
        si.rho_high = sod->rho_high; si.E_high = sod->p_high / (gm1 * sod->rho_high);
        si.rho_low = sod->rho_low; si.E_low = sod->p_low / (gm1 * sod->rho_low);
        CUDA_TRY(launch_init_sod(si, p->nb_cells, dd.arr[0], dd.arr[1], dd.arr[2], dd.arr[3], b->fp32, b->stream));
        b->launches++;
    } else if (init) {
        // rho umat vmat Emat of set 0
        for (int k = 0; k < 4; k++) {
            if (!init[k]) continue;
            if (!b->fp32) {
                CUDA_TRY(cudaMemcpyAsync(dd.arr[k], init[k], (size_t)p->nb_cells * 8, cudaMemcpyHostToDevice, b->stream));
            } else {
                void* stage = nullptr;
                CUDA_TRY(cudaMallocFromPoolAsync(&stage, (size_t)p->nb_cells * 8, b->pool, b->stream));
                CUDA_TRY(cudaMemcpyAsync(stage, init[k], (size_t)p->nb_cells * 8, cudaMemcpyHostToDevice, b->stream));
                narrow_kernel<<<b->sm_count * 8, 256, 0, b->stream>>>((const double*)stage, (float*)dd.arr[k],
                                                                      (int64_t)p->nb_cells);
                CUDA_TRY(cudaGetLastError());
                b->launches++;
                CUDA_TRY(cudaFreeAsync(stage, b->stream));
                CUDA_TRY(cudaStreamSynchronize(b->stream));   // the caller's host array may go away
            }
        }
    }
    for (int k = 0; k < 4; k++)
        CUDA_TRY(cudaMemcpyAsync(dd.arr[4 + k], dd.arr[k], arr_bytes, cudaMemcpyDeviceToDevice, b->stream));
    CUDA_TRY(cudaMemsetAsync(b->d_states + slot, 0, sizeof(StepState), b->stream));
    BeginArgs ba{};
    ba.nx = p->nx; ba.ny = p->ny;
    ba.origin = (int64_t)p->nb_ghosts * p->row_length + p->nb_ghosts;
    ba.row_length = p->row_length;
    ba.gamma = 1.4;
    ba.rho = dd.arr[0]; ba.umat = dd.arr[1]; ba.vmat = dd.arr[2]; ba.Emat = dd.arr[3];
    ba.pmat = dd.arr[8]; ba.cmat = dd.arr[9]; ba.gmat = dd.arr[10];
    ba.state = b->d_states + slot;
    ba.cfg = make_step_config(*p);
    ba.partials = dd.partials;
    ba.buf_base = 0;
    CUDA_TRY(launch_begin(ba, b->fp32, 152 * 4, b->stream));
    b->launches++;
    std::memset(&b->h_states[slot], 0, sizeof(StepState));
    b->dirty = true;
    *id = slot;
    return ARMON_OK;
}

}  // namespace

extern "C" {

int armon_batch_add(armon_batch* b, const armon_params* p, const double* const init[4], int32_t* id)
{
    return add_domain(b, p, init, nullptr, id);
}

int armon_batch_add_sod(armon_batch* b, const armon_params* p, const armon_sod_interface* sod, int32_t* id)
{
    if (!sod) { *id = -1; set_error("no interface given"); return ARMON_ERR_PARAMS; }
    if (sod->shape != 0 && sod->shape != 1) { *id = -1; set_error("interface shape must be 0 or 1"); return ARMON_ERR_PARAMS; }
    return add_domain(b, p, nullptr, sod, id);
}

int armon_batch_set_seg_len(armon_batch* b, int32_t id, int32_t seg_len)
{
    if (id < 0 || id >= (int)b->doms.size() || !b->doms[id].used) { set_error("unknown domain"); return ARMON_ERR_PARAMS; }
    b->doms[id].seg_len = seg_len;
    b->dirty = true;
    return ARMON_OK;
}

int armon_batch_enqueue_cycles(armon_batch* b, int32_t n) { return enqueue(b, n); }

int armon_batch_poll(armon_batch* b, int32_t* running)
{
    int m = max_slot(b);
    if (m > 0) {
        CUDA_TRY(cudaMemcpyAsync(b->h_states, b->d_states, sizeof(StepState) * m, cudaMemcpyDeviceToHost, b->stream));
    }
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    int run = 0;
    for (int i = 0; i < m; i++) {
        Dom& d = b->doms[i];
        if (!d.used) continue;
        bool r = loop_running(d, b->h_states[i]);
        if (r) run++;
        if (!r && !d.done) {
            d.done = true;
            b->dirty = true;   // drop it from the launch table
        }
    }
    if (running) *running = run;
    return ARMON_OK;
}

int armon_batch_ready(armon_batch* b)
{
    return cudaStreamQuery(b->stream) == cudaSuccess ? 1 : 0;
}

int armon_batch_run(armon_batch* b, int32_t cycle_limit, int32_t* running)
{
    int issued = 0, run = 0;
    for (;;) {
        int rc = armon_batch_poll(b, &run);
        if (rc != ARMON_OK) return rc;
        if (run == 0 || (cycle_limit > 0 && issued >= cycle_limit)) break;
        int n = b->o.cycles_per_graph > 0 ? b->o.cycles_per_graph : 8;
        if (cycle_limit > 0) n = std::min(n, cycle_limit - issued);
        rc = enqueue(b, n);
        if (rc != ARMON_OK) return rc;
        issued += n;
    }
    if (running) *running = run;
    return ARMON_OK;
}

int armon_batch_domain_state(armon_batch* b, int32_t id, armon_params* p, int32_t* status)
{
    if (id < 0 || id >= (int)b->doms.size() || !b->doms[id].used) { set_error("unknown domain"); return ARMON_ERR_PARAMS; }
    const StepState& st = b->h_states[id];
    *p = b->doms[id].p;
    p->cycle = st.cycle;
    p->time = st.time;
    p->current_cycle_dt = st.current_dt;
    p->next_cycle_dt = st.next_dt;
    if (status) *status = st.status;
    return ARMON_OK;
}

int armon_batch_domain_done(armon_batch* b, int32_t id)
{
    if (id < 0 || id >= (int)b->doms.size() || !b->doms[id].used) return -1;
    return b->doms[id].done ? 1 : 0;
}

int armon_batch_download(armon_batch* b, int32_t id, int which, double* host)
{
    if (id < 0 || id >= (int)b->doms.size() || !b->doms[id].used) { set_error("unknown domain"); return ARMON_ERR_PARAMS; }
    if (which < 2 || which > 8) { set_error("a batch holds rho, umat, vmat, Emat, pmat, cmat, gmat only"); return ARMON_ERR_PARAMS; }
    CUDA_TRY(cudaMemcpyAsync(&b->h_states[id], b->d_states + id, sizeof(StepState), cudaMemcpyDeviceToHost, b->stream));
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    Dom& d = b->doms[id];
    int k = which <= 5 ? current_set(b, id) * 4 + (which - 2) : 8 + (which - 6);
    size_t n = (size_t)d.p.nb_cells;
    if (!b->fp32) {
        CUDA_TRY(cudaMemcpyAsync(host, d.arr[k], n * 8, cudaMemcpyDeviceToHost, b->stream));
        CUDA_TRY(cudaStreamSynchronize(b->stream));
        return ARMON_OK;
    }
    void* stage = nullptr;
    CUDA_TRY(cudaMallocFromPoolAsync(&stage, n * 8, b->pool, b->stream));
    widen_kernel<<<b->sm_count * 8, 256, 0, b->stream>>>((const float*)d.arr[k], (double*)stage, (int64_t)n);
    CUDA_TRY(cudaGetLastError());
    b->launches++;
    CUDA_TRY(cudaMemcpyAsync(host, stage, n * 8, cudaMemcpyDeviceToHost, b->stream));
    CUDA_TRY(cudaFreeAsync(stage, b->stream));
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    return ARMON_OK;
}

int armon_batch_remove(armon_batch* b, int32_t id)
{
    if (id < 0 || id >= (int)b->doms.size() || !b->doms[id].used) { set_error("unknown domain"); return ARMON_ERR_PARAMS; }
    Dom& d = b->doms[id];
    CUDA_TRY(cudaFreeAsync(d.chunk, b->stream));
    b->bytes -= d.bytes;
    d = Dom();
    b->dirty = true;
    return ARMON_OK;
}

int armon_batch_schedule(armon_batch* b, int32_t* waves, int32_t* blocks)
{
    if (waves) *waves = b->o.waves > 0 ? b->o.waves : b->waves;
    if (blocks) *blocks = b->total_blocks;
    return ARMON_OK;
}

int32_t armon_batch_size(armon_batch* b)
{
    int n = 0;
    for (auto& d : b->doms) n += d.used;
    return n;
}

int64_t armon_batch_bytes_in_use(armon_batch* b) { return b->bytes; }
int64_t armon_batch_kernel_launches(armon_batch* b) { return b->launches; }

}  // extern "C"
