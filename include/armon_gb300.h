/*
 * armon_gb300.h -- native C ABI of the GB300 Armon time step (libarmon_gb300.so).
 *
 * Plain C: POD structs, raw pointers, sizes, int status codes.  No CUDA or C++ types cross
 * this boundary (streams are passed as void*).  The parameter block mirrors the reference's
 * Params (src/parameters.h:34-108) field for field, so a caller configures a solve with the
 * reference's own vocabulary; the solver object plays the part of the reference's DataHolder
 * (src/data.h:15-43) plus its time loop (src/armon_2D.cpp:327-386), with the state resident in
 * HBM and the per-cycle dt kept on the device.
 *
 * Error behaviour: every call returns ARMON_OK (0) or an ARMON_ERR_* code; armon_last_error()
 * gives a message.  The reference instead prints and exits on an invalid time step
 * (src/armon_2D.cpp:238-242); here the solver stops and reports ARMON_ERR_INVALID_DT.
 */
#ifndef ARMON_GB300_H
#define ARMON_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* src/kernels/test_cases.h:8-14 */
enum { ARMON_SOD = 0, ARMON_SOD_Y = 1, ARMON_SOD_CIRC = 2, ARMON_BIZARRIUM = 3, ARMON_SEDOV = 4 };
/* src/parameters.h:17-31, src/kernels/limiters.h:8-12, src/kernels/common.h:30-40 */
enum { ARMON_GODUNOV = 0, ARMON_GAD = 1 };
enum { ARMON_PROJ_NONE = 0, ARMON_EULER = 1, ARMON_EULER_2ND = 2 };
enum { ARMON_LIM_NONE = 0, ARMON_MINMOD = 1, ARMON_SUPERBEE = 2 };
enum { ARMON_SEQUENTIAL = 0, ARMON_SEQUENTIAL_SYM = 1, ARMON_STRANG = 2, ARMON_X_ONLY = 3, ARMON_Y_ONLY = 4 };
enum { ARMON_AXIS_X = 0, ARMON_AXIS_Y = 1 };
enum { ARMON_LEFT = 0, ARMON_RIGHT = 1, ARMON_TOP = 2, ARMON_BOTTOM = 3 };

/* Status codes */
enum {
    ARMON_OK = 0,
    ARMON_ERR_INVALID_DT = 1,   /* a non-finite or non-positive time step (the reference exits) */
    ARMON_ERR_PARAMS = 2,       /* Params::check failed, or an argument is out of range */
    ARMON_ERR_CUDA = 3,         /* a CUDA call failed; see armon_last_error() */
    ARMON_ERR_UNSUPPORTED = 4,  /* a combination the library does not implement */
    ARMON_ERR_NOMEM = 5,        /* device allocation failed or would exceed the budget */
    ARMON_ERR_STATE = 6         /* the device step state is inconsistent (e.g. a skipped cycle) */
};

/* Field list of src/parameters.h:34-108.  Integer fields first, then doubles, so that the
 * layout has no padding.  `test_option` extends the reference: for Sod_circ it is the squared
 * radius of the high-pressure disc (0 = the reference's 0.09), for Sedov the blast radius
 * (0 = derived from dx, dy as the reference does).  The output file name of the reference
 * (a const char*) is not part of this block. */
typedef struct armon_params {
    int32_t test, scheme, riemann, projection, limiter, current_axis, axis_splitting;
    int32_t nb_ghosts, nx, ny, stencil_width;
    int32_t cst_dt, dt_on_even_cycles;
    int32_t row_length, col_length, nb_cells, ideb, ifin, index_start, idx_row, idx_col, s;
    int32_t cycle, max_cycles;
    int32_t write_output, write_ghosts, write_throughput, output_precision, verbose, compare;
    double dx, cfl, Dt;
    double domain_size[2], domain_origin[2];
    double cycle_dt, current_cycle_dt, next_cycle_dt, time;
    double max_time, comparison_tolerance, test_option;
} armon_params;

/* ---- parameters (src/parameters.cpp) ---- */
void armon_params_defaults(armon_params* p);          /* member initialisers, src/parameters.h:36-97 */
void armon_params_init(armon_params* p);              /* Params::init, src/parameters.cpp:21-34 */
int armon_params_check(const armon_params* p);        /* Params::check: 1 = valid, src/parameters.cpp:70-109 */
int armon_min_ghosts(const armon_params* p);          /* src/parameters.cpp:11-18 */
int armon_params_sizeof(void);
/* BC_* sign factors (u_factor, v_factor) of a test case on one side, src/kernels/test_cases.h:36-121 */
void armon_boundary_factors(int test, int side, double* u_factor, double* v_factor);
/* TestCase::test_option as the driver passes it to init_test (src/armon_2D.cpp:116-118), with a
 * non-zero armon_params.test_option taking precedence */
double armon_test_option(const armon_params* p, double dx, double dy);
const char* armon_last_error(void);
int armon_device_count(void);

/* ---- the solver: device-resident state and the fused time loop ---- */
typedef struct armon_solver armon_solver;

/* Solver options beyond the reference's Params. */
typedef struct armon_solver_opts {
    int32_t precision;        /* 64: FP64 state and arithmetic (bit-exact with the reference);
                                 32: FP32 state and arithmetic, FP64 dt and conservation sums */
    int32_t cycles_per_graph; /* cycles captured per CUDA graph launch (0 = default, 16) */
    int32_t seg_len;          /* cells per thread along the sweep axis (0 = automatic) */
    int32_t block_lines;      /* lines (threads) per block (0 = automatic, 128) */
    int32_t materialize_eos;  /* p, c, g of the real cells: written by every pass (1), by the last
                                 pass of each cycle (0), or (-1, default) computed from the last
                                 pass's input, which the other state set still holds, when the loop
                                 ends, when p, c or g is downloaded, uploaded or its device pointer
                                 taken, or at the next begin_loop.  The values are the same in every
                                 mode (each pass's EOS overwrites the previous one); with -1 the
                                 arrays hold older values while cycles are still being issued
                                 (armon_solver_enqueue_cycles).  Split passes write them on the last
                                 pass in modes -1 and 0 (their cell half reads c). */
    int32_t unit_order;       /* 0 (default): each pass launches its blocks longest first, by the time
                                 each took in the previous cycle (results do not depend on it);
                                 -1: in index order */
    int32_t split_pass;       /* 0 (default): an FP64 solver holds a face buffer (3 x max((nx+5) ny,
                                 (ny+5) nx) values) and runs each axis pass as two launches (face
                                 fluxes, then the cell update: fewer values per thread, more warps
                                 per SM) or as one fused launch (half the bytes), whichever its
                                 tiling measurement finds faster (domains under 2^20 cells: split;
                                 fused when the face buffer cannot be allocated); FP32 passes stay
                                 fused.  1: split for either precision; -1: fused.  Results are the
                                 same bits either way. */
    int32_t reuse;            /* 0 (default): along each line, a position whose whole input window
                                 (the cells, and faces, its results depend on) repeats the previous
                                 position's bit for bit stores the previous position's results
                                 instead of recomputing them (fluid at rest); -1: every position is
                                 computed.  Results are the same bits either way. */
} armon_solver_opts;

void armon_solver_opts_default(armon_solver_opts* o);

/* Allocates the state of one domain in HBM.  `stream` is a cudaStream_t (NULL = a stream the
 * solver creates).  The solver keeps a copy of `p`. */
int armon_solver_create(const armon_params* p, const armon_solver_opts* opts, void* stream,
                        armon_solver** out);
/* The same on 16 caller-owned FP64 device arrays of nb_cells values (the reference's DataHolder
 * order: x y rho umat vmat Emat pmat cmat gmat ustar pstar work_array_1..4 domain_mask).  The
 * fused path uses the four work arrays as its second state buffer; after armon_solver_run returns,
 * rho/umat/vmat/Emat/pmat/cmat/gmat hold the state as the reference's time loop leaves them.
 * The arrays are not freed by armon_solver_destroy. */
int armon_solver_create_with_arrays(const armon_params* p, const armon_solver_opts* opts, double* const arrays[16],
                                    void* stream, armon_solver** out);
void armon_solver_destroy(armon_solver* s);

/* Restarts the time loop on the current arrays (the start of time_loop, src/armon_2D.cpp:327-346:
 * cycle = 0, time = 0, update_EOS, and the first dt_CFL).  Call after uploading a new state. */
int armon_solver_begin_loop(armon_solver* s);

/* init_test on the device (src/armon_2D.cpp:112-127) followed by the EOS and the first dt
 * reduction of time_loop (src/armon_2D.cpp:327-346). */
int armon_solver_init_test(armon_solver* s);

/* Runs cycles until the reference's loop condition (time < max_time && cycle < max_cycles)
 * fails, or until `cycle_limit` more cycles have been issued (cycle_limit <= 0: no limit).
 * Asynchronous inputs, synchronous outcome: returns once the device state has been read back. */
int armon_solver_run(armon_solver* s, int cycle_limit);

/* Enqueues exactly `n_cycles` cycles (no-ops after the loop condition fails) on the solver's
 * stream without reading anything back; for timing and graph capture by the caller. */
int armon_solver_enqueue_cycles(armon_solver* s, int n_cycles);

/* Copies the device step state (cycle, time, dts, status) to `p` (blocking). */
int armon_solver_sync_params(armon_solver* s, armon_params* p, int32_t* status);

/* Host <-> device copies of whole arrays (nb_cells values each, in the reference's layout).
 * `which` names an array: 0 x, 1 y, 2 rho, 3 umat, 4 vmat, 5 Emat, 6 pmat, 7 cmat, 8 gmat,
 * 9 ustar, 10 pstar, 11..14 work arrays, 15 domain_mask.  FP32 solvers convert on the device,
 * through an FP64 staging array of nb_cells values allocated on the first such call. */
int armon_solver_download(armon_solver* s, int which, double* host);
int armon_solver_upload(armon_solver* s, int which, const double* host);
/* Device pointer of an FP64 array (NULL for an FP32 solver) */
double* armon_solver_device_array(armon_solver* s, int which);

/* Mass and energy sums over the real cells (src/armon_2D.cpp:287-298), FP64, blocking. */
int armon_solver_conservation(armon_solver* s, double* mass, double* energy);

/* Number of kernels the solver launched so far (diagnostics). */
int64_t armon_solver_kernel_launches(armon_solver* s);

/* The tiling of the axis pass per axis (X, Y): cells per thread along the axis and blocks per
 * launch.  Unless opts.seg_len fixes it, a domain of 2^20 cells or more gets the fastest of a few
 * candidate tilings, each timed on real cycles of its first time loop (after 16 cycles with the
 * model's tiling, two cycles per candidate forwards and two backwards: results never depend on
 * the tiling), and cached per geometry for the process; smaller domains use the cost model. */
int armon_solver_tiling(armon_solver* s, int32_t seg_len[2], int32_t blocks[2]);
/* Lines (threads) per block of the fused pass: the caller's block_lines, or the measured choice. */
int armon_solver_block_lines(const armon_solver* s);
/* 1 while the time loop is still measuring candidate tilings on its cycles (domains of 2^20 cells
 * or more whose geometry this process has not measured yet; results never depend on the tiling). */
int armon_solver_tuning(const armon_solver* s);
/* Cycles this solver has run with a candidate tiling of the tiling measurement so far (a cost cycle
 * and a timed cycle per candidate and visit). */
int64_t armon_solver_measurement_cycles(const armon_solver* s);
/* 1 when the axis passes run split (a face launch and a cell launch), 0 when fused: the caller's
 * split_pass, or the measured form when split_pass is 0 and the solver holds a face buffer. */
int armon_solver_split_pass(const armon_solver* s);
/* Forgets the tilings measured so far in this process (the next time loop of each geometry
 * measures again). */
void armon_tiling_cache_clear(void);

/* ---- batches: many independent domains advanced together (no counterpart in the reference;
 *      each domain follows time_loop, src/armon_2D.cpp:327-386, on its own) ---- */
typedef struct armon_batch armon_batch;

typedef struct armon_batch_opts {
    int32_t precision;        /* 64 or 32: every domain of a batch has this precision */
    int32_t cycles_per_graph; /* cycles captured per CUDA graph launch (default 8) */
    int32_t block_lines;      /* lines (threads) per block: a multiple of 32, at most 128 (default 128) */
    int32_t seg_len;          /* cells per thread along the sweep axis for every domain (0 = scheduled) */
    int64_t memory_budget;    /* bytes of domain state the batch may hold (0 = no limit) */
    int32_t waves;            /* scheduled segments: block waves per launch to aim for (0 = autotuned) */
    int32_t unit_order;       /* 0 (default): each pass launches the blocks of all domains longest
                                 first, by the time each took in the previous cycle; -1: in index order */
    int32_t split_pass;       /* as armon_solver_opts.split_pass: 0 (default) split FP64 passes into a
                                 face launch and a cell launch (each domain then holds a face buffer,
                                 counted by armon_batch_domain_bytes); 1: split; -1: fused */
    int32_t reuse;            /* as armon_solver_opts.reuse: 0 (default) on, -1 off */
} armon_batch_opts;

void armon_batch_opts_default(armon_batch_opts* o);
int armon_batch_create(const armon_batch_opts* opts, void* stream, armon_batch** out);
void armon_batch_destroy(armon_batch* b);

/* Device bytes a domain with these parameters holds in a batch of the given precision. */
int64_t armon_batch_domain_bytes(const armon_params* p, int32_t precision);

/* Adds a domain and starts its time loop: allocates its state from the stream-ordered pool
 * (ARMON_ERR_NOMEM when the batch's budget would be exceeded), initialises it with init_test or,
 * when `init` is not NULL, with the host FP64 arrays rho, umat, vmat, Emat (nb_cells values each,
 * the reference's layout), then runs the EOS and the first dt.  All domains of a batch share
 * scheme, projection and axis splitting.  *id receives the domain's handle. */
int armon_batch_add(armon_batch* b, const armon_params* p, const double* const init[4], int32_t* id);

/* A Sod-type initial state made on the device (no counterpart in the reference, whose tests have
 * axis-aligned or fixed-radius interfaces).  Cell centres follow init_test
 * (src/kernels/init_test.cpp:65-93): x = ix / nx * sx + ox + sx / (2 nx), the same for y.  The high
 * state (rho_high, p_high) holds where
 *   shape 0 (planar):   (x - cx) * nx + (y - cy) * ny <= offset
 *   shape 1 (circular): (x - cx) * (x - cx) + (y - cy) * (y - cy) <= r2
 * and the low state elsewhere, with u = v = 0 and E = p / ((1.4 - 1) rho), over all nb_cells
 * cells (ghosts included); every operation is one IEEE-rounded FP64 operation in that order. */
typedef struct armon_sod_interface {
    int32_t shape;
    int32_t reserved;
    double cx, cy;
    double nx, ny, offset;    /* planar */
    double r2;                /* circular */
    double rho_high, p_high, rho_low, p_low;
} armon_sod_interface;

/* armon_batch_add with the initial state of `sod` instead of host arrays. */
int armon_batch_add_sod(armon_batch* b, const armon_params* p, const armon_sod_interface* sod, int32_t* id);

/* Cells per thread along the sweep axis for one domain (0 = automatic); takes effect at the next
 * launch.  Results do not depend on it. */
int armon_batch_set_seg_len(armon_batch* b, int32_t id, int32_t seg_len);

/* Enqueues n cycles of every domain whose loop is still running (no host synchronisation). */
int armon_batch_enqueue_cycles(armon_batch* b, int32_t n);

/* Runs until no domain's loop condition holds (or cycle_limit cycles were issued, if > 0), reading
 * the domain states back once per graph batch.  *running receives the domains still running. */
int armon_batch_run(armon_batch* b, int32_t cycle_limit, int32_t* running);

/* Reads back all domain states; *running receives how many loops are still running. */
int armon_batch_poll(armon_batch* b, int32_t* running);

/* 1 when everything enqueued on the batch's stream has finished (a poll would not wait), else 0. */
int armon_batch_ready(armon_batch* b);

/* State of one domain as of the last poll / run (cycle, time, dts in p; status 0 running or done,
 * 1 invalid dt). */
int armon_batch_domain_state(armon_batch* b, int32_t id, armon_params* p, int32_t* status);
int armon_batch_domain_done(armon_batch* b, int32_t id);

/* Downloads one array of a domain (which: 2 rho, 3 umat, 4 vmat, 5 Emat, 6 pmat, 7 cmat, 8 gmat). */
int armon_batch_download(armon_batch* b, int32_t id, int which, double* host);

/* Frees a domain's state (stream-ordered) and its handle. */
int armon_batch_remove(armon_batch* b, int32_t id);

/* The batch schedule in use: block waves per launch the segments aim for (autotuned unless fixed
 * by armon_batch_opts.waves or seg_len) and the blocks of the current launch table. */
int armon_batch_schedule(armon_batch* b, int32_t* waves, int32_t* blocks);

int32_t armon_batch_size(armon_batch* b);                /* domains held */
int64_t armon_batch_bytes_in_use(armon_batch* b);
int64_t armon_batch_kernel_launches(armon_batch* b);

/* ---- serving: a request loop over batches (no counterpart in the reference) ----
 * Solves are submitted as requests and wait in a first-come-first-served queue.  Each round
 * admits waiting requests while their state fits in the memory budget (and their batch is under
 * its cell limit: a request whose batch is full waits, without holding back requests for other
 * batches, and is never overtaken by a later request for the same batch), then advances every
 * admitted solve by a few cycles: solves of one precision and scheme share a batch (one fused
 * launch per pass for all of them), different batches run on their own streams and overlap on the
 * device.  A solve's state stays on the device from admission until the caller releases it;
 * finished solves leave the launch tables at once, and released memory admits the next requests.
 * A request gives the same result as the same solve run alone. */
typedef struct armon_server armon_server;

typedef struct armon_server_opts {
    int64_t memory_budget;     /* device bytes of solve state held at once (default 150e9) */
    int32_t cycles_per_step;   /* cycles of every running solve per round (default 8) */
    int32_t block_lines;       /* as armon_batch_opts (default 128) */
    int64_t max_inflight_cells;/* real cells running at once in one batch (0 = no limit): beyond
                                  what saturates the GPU, more solves at once only share it, and
                                  every one of them finishes later */
    int32_t waves;             /* as armon_batch_opts.waves for every batch (0 = autotuned) */
    int32_t reserved;
} armon_server_opts;

enum { ARMON_REQ_QUEUED = 0, ARMON_REQ_RUNNING = 1, ARMON_REQ_DONE = 2, ARMON_REQ_FAILED = 3 };

typedef struct armon_server_request {
    int32_t status;            /* ARMON_REQ_* (FAILED: the solve stopped on an invalid dt) */
    int32_t precision;
    int32_t cycle;             /* cycles done when it finished */
    int32_t nx, ny;
    int32_t pad;
    double time;               /* simulated time reached */
    double t_submit, t_admit, t_done;   /* seconds since the server was created (-1: not yet) */
    int64_t bytes;             /* device bytes of its state */
} armon_server_request;

void armon_server_opts_default(armon_server_opts* o);
int armon_server_create(const armon_server_opts* opts, armon_server** out);
void armon_server_destroy(armon_server* s);

/* Queues a solve (p as for armon_batch_add; max_time and max_cycles end it) in precision 64 or 32,
 * initialised from `sod`, or by init_test when it is NULL.  *req receives its id. */
int armon_server_submit(armon_server* s, const armon_params* p, int32_t precision, const armon_sod_interface* sod,
                        int64_t* req);

/* One round: admission; every batch with running solves and no cycles in progress gets
 * cycles_per_step more; then waits until at least one batch in progress has finished its cycles,
 * and retires the solves of the finished batches whose loop ended.  Batches proceed independently
 * (a fast batch is not held back by a slow one).  *in_flight / *queued (may be NULL) receive the
 * running / waiting requests. */
int armon_server_step(armon_server* s, int32_t* in_flight, int32_t* queued);

/* Pops the next finished (done or failed) request not yet reported: returns 1 and sets *req, or 0. */
int armon_server_next_done(armon_server* s, int64_t* req);

int armon_server_request_info(armon_server* s, int64_t req, armon_server_request* info);

/* Downloads one array of a finished request (which as armon_batch_download). */
int armon_server_download(armon_server* s, int64_t req, int which, double* host);

/* Frees a finished request's device state. */
int armon_server_release(armon_server* s, int64_t req);

int64_t armon_server_bytes_in_use(armon_server* s);
int64_t armon_server_kernel_launches(armon_server* s);

/* One full solve with host buffers, the reference-facing end-to-end call: uploads rho, umat,
 * vmat, Emat (and the rest of the initial state made by init_test on the device), runs the time
 * loop and downloads rho, umat, vmat, Emat, pmat.  Arrays have nb_cells values in the
 * reference's layout; `in[k]`/`out[k]` may be NULL to skip one. */
int armon_solve_host(const armon_params* p, const armon_solver_opts* opts,
                     const double* const in[4], double* const out[5], armon_params* final_state);

#ifdef __cplusplus
}
#endif
#endif
