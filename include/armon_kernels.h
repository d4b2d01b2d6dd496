/*
 * armon_kernels.h -- the reference's kernel ABI (src/kernels/kernels.h of Armon-Kokkos),
 * re-implemented as hand-written CUDA for sm_103a in libarmon_gb300.so.
 *
 * Same symbol names, argument order and meaning as the reference, so an FFI binding written for
 * the reference's libarmon_kernels (Armon.jl through Kokkos.jl `ccall`s these names) binds this
 * library.  At the machine level the reference passes `const Range&`, `const InnerRange2D&` and
 * `view&` as pointers; here they are pointers to the C structs below.  A Kokkos::View becomes an
 * `armon_view` {device pointer, length, label}.  The label is optional (NULL skips the check);
 * when given, it is checked like the reference's CHECK_VIEW_LABELS (src/kernels/utils.h:74-96).
 *
 * All array pointers are DEVICE pointers (the reference's CUDA build passes CudaSpace views).
 * Launches are asynchronous on the stream set by armon_kernels_set_stream (default: the legacy
 * default stream); dt_CFL and conservation_vars return host values and therefore synchronise,
 * as the reference's parallel_reduce into a host scalar does.
 *
 * Errors (bad enum, label mismatch, CUDA failure) call *raise_exception_handler(kernel, msg),
 * whose default prints and calls exit(1), as in the reference (src/kernels/utils.cpp:8-55).
 * flt_t is double (flt_size() == 8); Idx is int64_t and UIdx uint64_t (idx_size() == 8,
 * is_uidx_signed() == false).
 */
#ifndef ARMON_GB300_KERNELS_H
#define ARMON_GB300_KERNELS_H

#include <stdbool.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef double flt_t;
typedef int64_t Idx;
typedef uint64_t UIdx;
#ifdef __cplusplus
}
/* C++ callers get the reference's scoped enums (same 32-bit representation as the C typedefs). */
enum class Limiter : int32_t { None = 0, Minmod = 1, Superbee = 2 };                          /* src/kernels/limiters.h:8-12 */
enum class Test : int32_t { Sod = 0, Sod_y = 1, Sod_circ = 2, Bizarrium = 3, Sedov = 4 };   /* src/kernels/test_cases.h:8-14 */
extern "C" {
#else
typedef int32_t Limiter;   /* src/kernels/limiters.h:8-12: None 0, Minmod 1, Superbee 2 */
typedef int32_t Test;      /* src/kernels/test_cases.h:8-14: Sod 0 .. Sedov 4 */
#endif

/* src/kernels/indexing.h:28-33 */
typedef struct Range { Idx start; Idx end; } Range;
/* src/kernels/indexing.h:39-45: index = start + k * step */
typedef struct InnerRange1D { Idx start; Idx step; } InnerRange1D;
/* src/kernels/indexing.h:60-73: index = row_range_start + k % len + main_range_start + (k / len) * main_range_step */
typedef struct InnerRange2D {
    Idx main_range_start;
    Idx main_range_step;
    Idx row_range_start;
    UIdx row_range_length;
} InnerRange2D;

/* Replaces Kokkos::View<flt_t*> (src/kernels/common.h:24-27) */
typedef struct armon_view {
    flt_t* data;        /* device pointer */
    int64_t size;       /* number of elements */
    const char* label;  /* optional; checked by suffix against the parameter name */
} armon_view;
typedef armon_view view;
typedef armon_view mask_view;

/* src/kernels/kernels.h:10-13 */
void acoustic(const Range* range, const InnerRange2D* inner_range, Idx s,
              view* ustar, view* pstar,
              const view* rho, const view* u, const view* pmat, const view* cmat);

/* src/kernels/kernels.h:15-19 */
void acoustic_GAD(const Range* range, const InnerRange2D* inner_range, Idx s, flt_t dt, flt_t dx,
                  view* ustar, view* pstar,
                  const view* rho, const view* u, const view* pmat, const view* cmat,
                  Limiter limiter);

/* src/kernels/kernels.h:21-24 */
void perfect_gas_EOS(const Range* range, const InnerRange2D* inner_range, flt_t gamma,
                     const view* rho, const view* Emat, const view* umat, const view* vmat,
                     view* pmat, view* cmat, view* gmat);

/* src/kernels/kernels.h:26-29 (the Bizarrium equation of state) */
void bizarrium_EOS(const Range* range, const InnerRange2D* inner_range,
                   const view* rho, const view* umat, const view* vmat, const view* Emat,
                   view* pmat, view* cmat, view* gmat);

/* src/kernels/kernels.h:31-33 */
void cell_update(const Range* range, const InnerRange2D* inner_range, Idx s, flt_t dx, flt_t dt,
                 const view* ustar, const view* pstar, view* rho, view* u, view* Emat);

/* src/kernels/kernels.h:35-39 */
void euler_projection(const Range* range, const InnerRange2D* inner_range, Idx s, flt_t dx, flt_t dt,
                      const view* ustar, view* rho, view* umat, view* vmat, view* Emat,
                      const view* advection_rho, const view* advection_urho,
                      const view* advection_vrho, const view* advection_Erho);

/* src/kernels/kernels.h:41-44 */
void advection_first_order(const Range* range, const InnerRange2D* inner_range, Idx s, flt_t dt,
                           const view* ustar, const view* rho, const view* umat, const view* vmat,
                           const view* Emat,
                           view* advection_rho, view* advection_urho, view* advection_vrho,
                           view* advection_Erho);

/* src/kernels/kernels.h:46-49 */
void advection_second_order(const Range* range, const InnerRange2D* inner_range, Idx s, flt_t dx, flt_t dt,
                            const view* ustar, const view* rho, const view* umat, const view* vmat,
                            const view* Emat,
                            view* advection_rho, view* advection_urho, view* advection_vrho,
                            view* advection_Erho);

/* src/kernels/kernels.h:51-55 */
void boundary_conditions(const Range* range, const InnerRange1D* inner_range,
                         Idx stencil_width, Idx disp,
                         flt_t u_factor, flt_t v_factor,
                         view* rho, view* umat, view* vmat, view* pmat, view* cmat, view* gmat,
                         view* Emat);

/* src/kernels/kernels.h:57-62 */
void read_border_array(const Range* range, const InnerRange2D* inner_range,
                       Idx side_length, Idx nghost,
                       const view* rho, const view* umat, const view* vmat, const view* pmat,
                       const view* cmat, const view* gmat, const view* Emat,
                       view* value_array);

/* src/kernels/kernels.h:64-69 */
void write_border_array(const Range* range, const InnerRange2D* inner_range,
                        Idx side_length, Idx nghost,
                        view* rho, view* umat, view* vmat, view* pmat,
                        view* cmat, view* gmat, view* Emat,
                        const view* value_array);

/* src/kernels/kernels.h:71-77 */
void init_test(const Range* range, const InnerRange2D* inner_range,
               Idx row_length, Idx nb_ghosts, Idx nx, Idx ny, flt_t sx,
               flt_t sy, flt_t ox, flt_t oy, Idx pos_x, Idx pos_y, Idx g_nx, Idx g_ny,
               view* x, view* y, view* rho, view* Emat, view* umat, view* vmat, mask_view* domain_mask,
               view* pmat, view* cmat, view* gmat, view* ustar, view* pstar,
               Test test, bool debug_indexes, flt_t test_option);

/* src/kernels/kernels.h:79-81 (blocking; returns a host value) */
flt_t dt_CFL(const Range* range, const InnerRange1D* inner_range, flt_t dx, flt_t dy,
             const view* umat, const view* vmat, const view* cmat, const mask_view* domain_mask);

/* No counterpart in the reference.  dt_CFL for callers that may not allocate device memory after
 * start-up: hosts that hand the whole device to their own memory pool (a Julia or Kokkos runtime
 * that reserved it), or time-critical loops that cannot afford cudaMalloc's device-wide
 * synchronisation.  Same arguments and result as dt_CFL, which allocates its reduction scratch on
 * first use; this variant keeps its scratch in a fixed 256 KB array inside the library's device
 * module instead, so it calls no cudaMalloc, cudaFree or allocating routine.
 *  - Limit: ranges of at most 134,217,728 indices (32768 tiles of 4096); a longer range goes to
 *    raise_exception_handler with an out_of_range message.
 *  - The first call on each device resolves the array's device address (cudaGetSymbolAddress with
 *    that device current); make that first call before any stream capture.  With CUDA's lazy
 *    module loading (the default), that call may also be what loads the library's device module
 *    and reserves the array, so make it, or any earlier call into the library, before the host
 *    hands the device's free memory to its own pool.
 *  - Every call shares the one array (it keeps the last call's partials; each call overwrites all
 *    it reads), so calls that overlap on the GPU race: issue them on one stream.
 *  - Every GPU that loads the library holds the array until the process exits. */
flt_t dt_CFL_no_alloc(const Range* range, const InnerRange1D* inner_range, flt_t dx, flt_t dy,
                      const view* umat, const view* vmat, const view* cmat, const mask_view* domain_mask);

/* src/kernels/kernels.h:83-86 (blocking; the sums are written to host memory) */
void conservation_vars(const Range* range, const InnerRange1D* inner_range, flt_t dx,
                       const view* rho, const view* Emat, const mask_view* domain_mask,
                       flt_t* total_mass, flt_t* total_energy);

/* src/kernels/utils.cpp:16-27 */
extern void (*raise_exception_handler)(const char* kernel, const char* msg);
int idx_size(void);
bool is_uidx_signed(void);
int flt_size(void);

/* Extension: the stream the entry points above launch on (a cudaStream_t; NULL = legacy default). */
void armon_kernels_set_stream(void* stream);

#ifdef __cplusplus
}
#endif
#endif
