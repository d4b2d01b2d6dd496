// abi_kernels.cu -- the reference's kernel ABI (src/kernels/kernels.h:10-86) as per-stage CUDA
// kernels for sm_103a, declared in include/armon_kernels.h.
//
// Each entry point walks the same flat index range as the reference's Kokkos RangePolicy
// (k in [range.start, range.end), cell = inner_range.scale_index(k)) with one thread per index and
// the reference's expression tree; the file is built with --fmad=false so every stage is bit-exact
// with the reference's strict FP64 build.  These are the drop-in stages and the step-level checks;
// the fused solver (sweep.cuh) is the fast path.
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>

#include <cuda_runtime.h>

#include "armon_kernels.h"
#include "device_common.cuh"
#include "init.cuh"

using armon::kmax;
using armon::kmin;

namespace {

cudaStream_t g_stream = nullptr;

[[noreturn]] void default_exception_handler(const char* kernel, const char* msg)
{
    std::printf("Exception in kernel %s: %s\n", kernel, msg);
    std::exit(1);
}

__host__ __device__ inline int64_t scale2d(const InnerRange2D& r, uint64_t i)
{
    int64_t ix = (int64_t)(i / r.row_range_length);
    int64_t iy = (int64_t)(i % r.row_range_length);
    int64_t j = r.main_range_start + ix * r.main_range_step;
    return r.row_range_start + iy + j;
}

__host__ __device__ inline int64_t scale1d(const InnerRange1D& r, uint64_t i) { return (int64_t)i * r.step + r.start; }

template <class F>
__global__ void range_kernel(int64_t start, int64_t end, F f)
{
    for (int64_t k = start + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < end; k += (int64_t)gridDim.x * blockDim.x)
        f(k);
}

void check_cuda(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

template <class F>
void launch_range(const Range* r, F f)
{
    int64_t n = r->end - r->start;
    if (n <= 0) return;
    int64_t blocks = (n + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    range_kernel<<<(int)blocks, 256, 0, g_stream>>>(r->start, r->end, f);
    check_cuda(cudaGetLastError(), "kernel launch");
}

// The entry point being run, for the label check's message (the checks run inside the lambda that
// guarded() calls, where __func__ would name the lambda).
thread_local const char* g_kernel = "";

// CHECK_VIEW_LABELS (src/kernels/utils.h:74-96): a labelled view must end with the parameter name.
void check_label(const view* v, const char* name, const char* func)
{
    if (!v || !v->label) return;
    size_t a = std::strlen(v->label), b = std::strlen(name);
    if (a >= b && std::strcmp(v->label + a - b, name) == 0) return;
    throw std::invalid_argument(std::string("Wrong view order in ") + func + ": expected " + name + ", got: " +
                                v->label + "\n");
}
#define CHECK_LABEL(v) check_label(v, #v, g_kernel)

// KERNEL_TRY / KERNEL_CATCH -> raise_exception (src/kernels/utils.h:103-114, utils.cpp:49-54)
template <class Body>
void guarded(const char* kernel, Body body)
{
    g_kernel = kernel;
    try {
        body();
    } catch (const std::invalid_argument& e) {
        raise_exception_handler(kernel, (std::string("(std::invalid_argument) ") + e.what()).c_str());
    } catch (const std::out_of_range& e) {
        raise_exception_handler(kernel, (std::string("(std::out_of_range) ") + e.what()).c_str());
    } catch (const std::exception& e) {
        raise_exception_handler(kernel, (std::string("(std::runtime_error) ") + e.what()).c_str());
    }
}

// Device scratch for the two reductions: one pair of doubles per block, kept between calls, one
// buffer per device (a buffer is only valid on the device that allocated it).  Host threads that
// call the reductions at the same time on one device share the buffer and race on it, as they
// share the library's stream; the lock only protects the allocation itself.
double* scratch(size_t doubles)
{
    static std::mutex mu;
    static double* buf[64] = {};
    static size_t cap[64] = {};
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= 64) throw std::runtime_error("device index out of range for the scratch table");
    std::lock_guard<std::mutex> lk(mu);
    if (doubles > cap[dev]) {
        if (buf[dev]) {
            check_cuda(cudaStreamSynchronize(g_stream), "cudaStreamSynchronize");
            cudaFree(buf[dev]);
        }
        buf[dev] = nullptr;
        cap[dev] = 0;
        check_cuda(cudaMalloc(&buf[dev], doubles * sizeof(double)), "cudaMalloc");
        cap[dev] = doubles;
    }
    return buf[dev];
}

__device__ __forceinline__ void godunov(double rho_i, double rho_im, double c_i, double c_im, double u_i, double u_im,
                                        double p_i, double p_im, double& us, double& ps)
{
    // src/kernels/acoustic.cpp:10-19
    double rc_l = rho_im * c_im;
    double rc_r = rho_i * c_i;
    us = (rc_l * u_im + rc_r * u_i + (p_im - p_i)) / (rc_l + rc_r);
    ps = (rc_r * p_im + rc_l * p_i + rc_l * rc_r * (u_im - u_i)) / (rc_l + rc_r);
}

__device__ __forceinline__ double limiter(int L, double r)
{
    // src/kernels/limiters.h:15-34
    if (L == 1) return kmax(0.0, kmin(1.0, r));
    if (L == 2) return kmax(kmax(0.0, kmin(1.0, 2 * r)), kmin(2.0, r));
    return 1.0;
}

__device__ __forceinline__ double slope_minmod(double u_im, double u_i, double u_ip, double r_m, double r_p)
{
    // src/kernels/euler_projection.cpp:73-79
    double D_u_p = r_p * (u_ip - u_i);
    double D_u_m = r_m * (u_i - u_im);
    double s = copysign(1.0, D_u_p);
    return s * kmax(0.0, kmin(s * D_u_p, s * D_u_m));
}

__global__ void dt_partial_kernel(int64_t start, int64_t end, InnerRange1D ir, double dx, double dy, const double* umat,
                                  const double* vmat, const double* cmat, const double* mask, double* partials)
{
    // src/kernels/reductions.cpp:16-20 per index; partials start at DBL_MAX like Kokkos::Min
    __shared__ double red[256];
    double acc = DBL_MAX;
    for (int64_t k = start + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < end; k += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = scale1d(ir, (uint64_t)k);
        double max_cx = kmax(fabs(umat[i] + cmat[i]), fabs(umat[i] - cmat[i])) * mask[i];
        double max_cy = kmax(fabs(vmat[i] + cmat[i]), fabs(vmat[i] - cmat[i])) * mask[i];
        acc = kmin(acc, kmin(dx / max_cx, dy / max_cy));
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) { double o = red[threadIdx.x + w]; if (o < red[threadIdx.x]) red[threadIdx.x] = o; }
        __syncthreads();
    }
    if (threadIdx.x == 0) partials[blockIdx.x] = red[0];
}

__global__ void min_final_kernel(const double* partials, int n, double* out)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double acc = DBL_MAX;
        for (int b = 0; b < n; b++) if (partials[b] < acc) acc = partials[b];
        out[0] = acc;
    }
}

__global__ void cons_partial_kernel(int64_t start, int64_t end, InnerRange1D ir, double ds, const double* rho,
                                    const double* E, const double* mask, double* partials)
{
    // src/kernels/reductions.cpp:40-48 per index, summed in a fixed tree
    __shared__ double sm[2][256];
    double m = 0, e = 0;
    for (int64_t k = start + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < end; k += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = scale1d(ir, (uint64_t)k);
        double cell_mass = rho[i] * mask[i] * ds;
        double cell_energy = cell_mass * E[i];
        m += cell_mass;
        e += cell_energy;
    }
    sm[0][threadIdx.x] = m;
    sm[1][threadIdx.x] = e;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) { sm[0][threadIdx.x] += sm[0][threadIdx.x + w]; sm[1][threadIdx.x] += sm[1][threadIdx.x + w]; }
        __syncthreads();
    }
    if (threadIdx.x == 0) { partials[2 * blockIdx.x] = sm[0][0]; partials[2 * blockIdx.x + 1] = sm[1][0]; }
}

__global__ void sum2_final_kernel(const double* partials, int n, double* out)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double m = 0, e = 0;
        for (int b = 0; b < n; b++) { m += partials[2 * b]; e += partials[2 * b + 1]; }
        out[0] = m;
        out[1] = e;
    }
}

constexpr int kReduceBlocks = 152 * 4;

// ---- dt_CFL without device allocation --------------------------------------------------------
// One partial minimum per tile of kNoAllocTile indices, in a fixed array that lives in the module
// (every GPU that loads the library holds it until the process exits), plus one slot for the
// result.  256 KB: ranges of up to kNoAllocMaxTiles * kNoAllocTile = 134,217,728 indices.
constexpr int kNoAllocTile = 4096;
constexpr int kNoAllocMaxTiles = 32768;
static __device__ __align__(256) double g_dt_no_alloc_scratch[kNoAllocMaxTiles + 1];

__global__ void dt_tile_kernel(int64_t start, int64_t end, InnerRange1D ir, double dx, double dy, const double* umat,
                               const double* vmat, const double* cmat, const double* mask, double* partials)
{
    // the same per-index formula as dt_partial_kernel, one tile of kNoAllocTile indices per block
    __shared__ double red[256];
    double acc = DBL_MAX;
    const int64_t t0 = start + (int64_t)blockIdx.x * kNoAllocTile;
    const int64_t t1 = min(end, t0 + kNoAllocTile);
    for (int64_t k = t0 + threadIdx.x; k < t1; k += blockDim.x) {
        int64_t i = scale1d(ir, (uint64_t)k);
        double max_cx = kmax(fabs(umat[i] + cmat[i]), fabs(umat[i] - cmat[i])) * mask[i];
        double max_cy = kmax(fabs(vmat[i] + cmat[i]), fabs(vmat[i] - cmat[i])) * mask[i];
        acc = kmin(acc, kmin(dx / max_cx, dy / max_cy));
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) { double o = red[threadIdx.x + w]; if (o < red[threadIdx.x]) red[threadIdx.x] = o; }
        __syncthreads();
    }
    if (threadIdx.x == 0) partials[blockIdx.x] = red[0];
}

__global__ void min_tiles_kernel(const double* partials, int n, double* out)
{
    __shared__ double red[1024];
    double acc = DBL_MAX;
    for (int b = threadIdx.x; b < n; b += blockDim.x)
        if (partials[b] < acc) acc = partials[b];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) { double o = red[threadIdx.x + w]; if (o < red[threadIdx.x]) red[threadIdx.x] = o; }
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = red[0];
}

// Device address of g_dt_no_alloc_scratch, resolved once per device with that device current.
// In host code the symbol itself is only a host-side stand-in for the array.
double* no_alloc_scratch_address()
{
    static std::mutex mu;
    static double* addr[64] = {};
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= 64) throw std::runtime_error("device index out of range for the static scratch table");
    std::lock_guard<std::mutex> lk(mu);
    if (!addr[dev]) {
        void* p = nullptr;
        check_cuda(cudaGetSymbolAddress(&p, g_dt_no_alloc_scratch), "cudaGetSymbolAddress");
        addr[dev] = static_cast<double*>(p);
    }
    return addr[dev];
}

}  // namespace

extern "C" {

void (*raise_exception_handler)(const char* kernel, const char* msg) = default_exception_handler;

int idx_size(void) { return (int)sizeof(Idx); }
bool is_uidx_signed(void) { return false; }
int flt_size(void) { return (int)sizeof(flt_t); }

void armon_kernels_set_stream(void* stream) { g_stream = (cudaStream_t)stream; }

void acoustic(const Range* range, const InnerRange2D* inner_range, Idx s, view* ustar, view* pstar,
              const view* rho, const view* u, const view* pmat, const view* cmat)
{
    guarded("acoustic", [&] {
        CHECK_LABEL(ustar); CHECK_LABEL(pstar); CHECK_LABEL(rho); CHECK_LABEL(pmat); CHECK_LABEL(cmat);
        const InnerRange2D ir = *inner_range;
        double *us = ustar->data, *ps = pstar->data;
        const double *r = rho->data, *uu = u->data, *p = pmat->data, *c = cmat->data;
        launch_range(range, [=] __device__(int64_t k) {
            int64_t i = scale2d(ir, (uint64_t)k);
            double a, b;
            godunov(r[i], r[i - s], c[i], c[i - s], uu[i], uu[i - s], p[i], p[i - s], a, b);
            us[i] = a;
            ps[i] = b;
        });
    });
}

void acoustic_GAD(const Range* range, const InnerRange2D* inner_range, Idx s, flt_t dt, flt_t dx, view* ustar,
                  view* pstar, const view* rho, const view* u, const view* pmat, const view* cmat, Limiter lim)
{
    guarded("acoustic_GAD", [&] {
        const int L = static_cast<int>(lim);
        if (L < 0 || L > 2)
            throw std::out_of_range("Invalid limiter index: " + std::to_string(L) + ", expected a value between 0 and 2");
        CHECK_LABEL(ustar); CHECK_LABEL(pstar); CHECK_LABEL(rho); CHECK_LABEL(pmat); CHECK_LABEL(cmat);
        const InnerRange2D ir = *inner_range;
        double *ust = ustar->data, *pst = pstar->data;
        const double *rh = rho->data, *uu = u->data, *p = pmat->data, *c = cmat->data;
        launch_range(range, [=] __device__(int64_t k) {
            // src/kernels/acoustic.cpp:40-88
            int64_t i = scale2d(ir, (uint64_t)k);
            double ustar_im, pstar_im, ustar_i, pstar_i, ustar_ip, pstar_ip;
            godunov(rh[i - s], rh[i - 2 * s], c[i - s], c[i - 2 * s], uu[i - s], uu[i - 2 * s], p[i - s], p[i - 2 * s],
                    ustar_im, pstar_im);
            godunov(rh[i], rh[i - s], c[i], c[i - s], uu[i], uu[i - s], p[i], p[i - s], ustar_i, pstar_i);
            godunov(rh[i + s], rh[i], c[i + s], c[i], uu[i + s], uu[i], p[i + s], p[i], ustar_ip, pstar_ip);
            double r_um = (ustar_ip - uu[i]) / (ustar_i - uu[i - s] + 1e-6);
            double r_pm = (pstar_ip - p[i]) / (pstar_i - p[i - s] + 1e-6);
            double r_up = (uu[i - s] - ustar_im) / (uu[i] - ustar_i + 1e-6);
            double r_pp = (p[i - s] - pstar_im) / (p[i] - pstar_i + 1e-6);
            r_um = limiter(L, r_um);
            r_pm = limiter(L, r_pm);
            r_up = limiter(L, r_up);
            r_pp = limiter(L, r_pp);
            double dm_l = rh[i - s] * dx;
            double dm_r = rh[i] * dx;
            double Dm = (dm_l + dm_r) / 2;
            double rc_l = rh[i - s] * c[i - s];
            double rc_r = rh[i] * c[i];
            double theta = 0.5 * (1 - (rc_l + rc_r) / 2 * (dt / Dm));
            ust[i] = ustar_i + theta * (r_up * (uu[i] - ustar_i) - r_um * (ustar_i - uu[i - s]));
            pst[i] = pstar_i + theta * (r_pp * (p[i] - pstar_i) - r_pm * (pstar_i - p[i - s]));
        });
    });
}

void perfect_gas_EOS(const Range* range, const InnerRange2D* inner_range, flt_t gamma, const view* rho,
                     const view* Emat, const view* umat, const view* vmat, view* pmat, view* cmat, view* gmat)
{
    guarded("perfect_gas_EOS", [&] {
        CHECK_LABEL(rho); CHECK_LABEL(umat); CHECK_LABEL(vmat); CHECK_LABEL(Emat);
        CHECK_LABEL(cmat); CHECK_LABEL(pmat); CHECK_LABEL(gmat);
        const InnerRange2D ir = *inner_range;
        const double *r = rho->data, *E = Emat->data, *u = umat->data, *v = vmat->data;
        double *p = pmat->data, *c = cmat->data, *g = gmat->data;
        launch_range(range, [=] __device__(int64_t k) {
            // src/kernels/fluid_eos.cpp:17-21 (Kokkos::pow(x, 2) == x * x)
            int64_t i = scale2d(ir, (uint64_t)k);
            double e = E[i] - 0.5 * (u[i] * u[i] + v[i] * v[i]);
            p[i] = (gamma - 1) * r[i] * e;
            c[i] = sqrt(gamma * p[i] / r[i]);
            g[i] = (1 + gamma) / 2;
        });
    });
}

void bizarrium_EOS(const Range* range, const InnerRange2D* inner_range, const view* rho, const view* umat,
                   const view* vmat, const view* Emat, view* pmat, view* cmat, view* gmat)
{
    guarded("bizarrium_EOS", [&] {
        CHECK_LABEL(rho); CHECK_LABEL(umat); CHECK_LABEL(vmat); CHECK_LABEL(Emat);
        CHECK_LABEL(cmat); CHECK_LABEL(pmat); CHECK_LABEL(gmat);
        const InnerRange2D ir = *inner_range;
        const double *rh = rho->data, *E = Emat->data, *u = umat->data, *v = vmat->data;
        double *pm = pmat->data, *cm = cmat->data, *gm = gmat->data;
        launch_range(range, [=] __device__(int64_t k) {
            // src/kernels/fluid_eos.cpp:31-60.  pow(., 3), pow(., 4) are CUDA's pow here, so this
            // stage agrees with the host build to rounding, not bit for bit.
            const double rho0 = 1e4, K0 = 1e11, Cv0 = 1e3, T0 = 300, eps0 = 0;
            const double G0 = 1.5, s = 1.5, q = -42080895. / 14941154., r = 727668333. / 149411540.;
            int64_t i = scale2d(ir, (uint64_t)k);
            double x = rh[i] / rho0 - 1;
            double g = G0 * (1 - rho0 / rh[i]);
            double f0 = (1 + (s / 3 - 2) * x + q * (x * x) + r * (x * x * x)) / (1 - s * x);
            double f1 = (s / 3 - 2 + 2 * q * x + 3 * r * (x * x) + s * f0) / (1 - s * x);
            double f2 = (2 * q + 6 * r * x + 2 * s * f1) / (1 - s * x);
            double f3 = (6 * r + 3 * s * f2) / (1 - s * x);
            double eps_k0 = eps0 - Cv0 * T0 * (1 + g) + 0.5 * (K0 / rho0) * (x * x) * f0;
            double pk0 = -Cv0 * T0 * G0 * rho0 + (0.5 * K0 * x * (1 + x) * (1 + x) * (2 * f0 + x * f1));
            double pk0prime = -0.5 * K0 * pow(1 + x, 3.0) * rho0 *
                              (2 * (1 + 3 * x) * f0 + 2 * x * (2 + 3 * x) * f1 + (x * x) * (1 + x) * f2);
            double pk0second = 0.5 * K0 * pow(1 + x, 4.0) * (rho0 * rho0) *
                               (12 * (1 + 2 * x) * f0 + 6 * (1 + 6 * x + 6 * (x * x)) * f1 +
                                6 * x * (1 + x) * (1 + 2 * x) * f2 + (x * (1 + x)) * (x * (1 + x)) * f3);
            double e = E[i] - 0.5 * (u[i] * u[i] + v[i] * v[i]);
            pm[i] = pk0 + G0 * rho0 * (e - eps_k0);
            cm[i] = sqrt(G0 * rho0 * (pm[i] - pk0) - pk0prime) / rh[i];
            gm[i] = 0.5 / (pow(rh[i], 3.0) * (cm[i] * cm[i])) * (pk0second + (G0 * rho0) * (G0 * rho0) * (pm[i] - pk0));
        });
    });
}

void cell_update(const Range* range, const InnerRange2D* inner_range, Idx s, flt_t dx, flt_t dt, const view* ustar,
                 const view* pstar, view* rho, view* u, view* Emat)
{
    guarded("cell_update", [&] {
        CHECK_LABEL(ustar); CHECK_LABEL(pstar); CHECK_LABEL(Emat); CHECK_LABEL(rho);
        const InnerRange2D ir = *inner_range;
        const double *us = ustar->data, *ps = pstar->data;
        double *r = rho->data, *uu = u->data, *E = Emat->data;
        launch_range(range, [=] __device__(int64_t k) {
            // src/kernels/euler_projection.cpp:16-20
            int64_t i = scale2d(ir, (uint64_t)k);
            double dm = r[i] * dx;
            r[i] = dm / (dx + dt * (us[i + s] - us[i]));
            uu[i] += dt / dm * (ps[i] - ps[i + s]);
            E[i] += dt / dm * (ps[i] * us[i] - ps[i + s] * us[i + s]);
        });
    });
}

void euler_projection(const Range* range, const InnerRange2D* inner_range, Idx s, flt_t dx, flt_t dt,
                      const view* ustar, view* rho, view* umat, view* vmat, view* Emat, const view* advection_rho,
                      const view* advection_urho, const view* advection_vrho, const view* advection_Erho)
{
    guarded("euler_projection", [&] {
        CHECK_LABEL(ustar); CHECK_LABEL(rho); CHECK_LABEL(umat); CHECK_LABEL(vmat); CHECK_LABEL(Emat);
        const InnerRange2D ir = *inner_range;
        const double* us = ustar->data;
        double *r = rho->data, *u = umat->data, *v = vmat->data, *E = Emat->data;
        const double *ar = advection_rho->data, *au = advection_urho->data, *av = advection_vrho->data,
                     *aE = advection_Erho->data;
        launch_range(range, [=] __device__(int64_t k) {
            // src/kernels/euler_projection.cpp:34-46
            int64_t i = scale2d(ir, (uint64_t)k);
            double dX = dx + dt * (us[i + s] - us[i]);
            double tmp_rho = (dX * r[i] - (ar[i + s] - ar[i])) / dx;
            double tmp_urho = (dX * r[i] * u[i] - (au[i + s] - au[i])) / dx;
            double tmp_vrho = (dX * r[i] * v[i] - (av[i + s] - av[i])) / dx;
            double tmp_Erho = (dX * r[i] * E[i] - (aE[i + s] - aE[i])) / dx;
            r[i] = tmp_rho;
            u[i] = tmp_urho / tmp_rho;
            v[i] = tmp_vrho / tmp_rho;
            E[i] = tmp_Erho / tmp_rho;
        });
    });
}

void advection_first_order(const Range* range, const InnerRange2D* inner_range, Idx s, flt_t dt, const view* ustar,
                           const view* rho, const view* umat, const view* vmat, const view* Emat, view* advection_rho,
                           view* advection_urho, view* advection_vrho, view* advection_Erho)
{
    guarded("advection_first_order", [&] {
        CHECK_LABEL(ustar); CHECK_LABEL(rho); CHECK_LABEL(umat); CHECK_LABEL(vmat); CHECK_LABEL(Emat);
        const InnerRange2D ir = *inner_range;
        const double *us = ustar->data, *r = rho->data, *u = umat->data, *v = vmat->data, *E = Emat->data;
        double *ar = advection_rho->data, *au = advection_urho->data, *av = advection_vrho->data,
               *aE = advection_Erho->data;
        launch_range(range, [=] __device__(int64_t k) {
            // src/kernels/euler_projection.cpp:59-68
            int64_t i = scale2d(ir, (uint64_t)k);
            double disp = dt * us[i];
            int64_t is = i;
            i -= (int64_t)(disp > 0) * s;
            ar[is] = disp * (r[i]);
            au[is] = disp * (r[i] * u[i]);
            av[is] = disp * (r[i] * v[i]);
            aE[is] = disp * (r[i] * E[i]);
        });
    });
}

void advection_second_order(const Range* range, const InnerRange2D* inner_range, Idx s, flt_t dx, flt_t dt,
                            const view* ustar, const view* rho, const view* umat, const view* vmat, const view* Emat,
                            view* advection_rho, view* advection_urho, view* advection_vrho, view* advection_Erho)
{
    guarded("advection_second_order", [&] {
        CHECK_LABEL(ustar); CHECK_LABEL(rho); CHECK_LABEL(umat); CHECK_LABEL(vmat); CHECK_LABEL(Emat);
        const InnerRange2D ir = *inner_range;
        const double *us = ustar->data, *r = rho->data, *u = umat->data, *v = vmat->data, *E = Emat->data;
        double *ar = advection_rho->data, *au = advection_urho->data, *av = advection_vrho->data,
               *aE = advection_Erho->data;
        launch_range(range, [=] __device__(int64_t k) {
            // src/kernels/euler_projection.cpp:90-118
            int64_t i = scale2d(ir, (uint64_t)k);
            int64_t is = i;
            double disp = dt * us[i];
            double Dx;
            if (disp > 0) {
                Dx = -(dx - dt * us[i - s]);
                i = i - s;
            } else {
                Dx = dx + dt * us[i + s];
            }
            double Dx_lm = dx + dt * (us[i] - us[i - s]);
            double Dx_l = dx + dt * (us[i + s] - us[i]);
            double Dx_lp = dx + dt * (us[i + 2 * s] - us[i + s]);
            double r_m = (2 * Dx_l) / (Dx_l + Dx_lm);
            double r_p = (2 * Dx_l) / (Dx_l + Dx_lp);
            double slope_r = slope_minmod(r[i - s], r[i], r[i + s], r_m, r_p);
            double slope_ur = slope_minmod(r[i - s] * u[i - s], r[i] * u[i], r[i + s] * u[i + s], r_m, r_p);
            double slope_vr = slope_minmod(r[i - s] * v[i - s], r[i] * v[i], r[i + s] * v[i + s], r_m, r_p);
            double slope_Er = slope_minmod(r[i - s] * E[i - s], r[i] * E[i], r[i + s] * E[i + s], r_m, r_p);
            double length_factor = Dx / (2 * Dx_l);
            ar[is] = disp * (r[i] - slope_r * length_factor);
            au[is] = disp * (r[i] * u[i] - slope_ur * length_factor);
            av[is] = disp * (r[i] * v[i] - slope_vr * length_factor);
            aE[is] = disp * (r[i] * E[i] - slope_Er * length_factor);
        });
    });
}

void boundary_conditions(const Range* range, const InnerRange1D* inner_range, Idx stencil_width, Idx disp,
                         flt_t u_factor, flt_t v_factor, view* rho, view* umat, view* vmat, view* pmat, view* cmat,
                         view* gmat, view* Emat)
{
    guarded("boundary_conditions", [&] {
        CHECK_LABEL(rho); CHECK_LABEL(umat); CHECK_LABEL(vmat); CHECK_LABEL(pmat);
        CHECK_LABEL(cmat); CHECK_LABEL(gmat); CHECK_LABEL(Emat);
        const InnerRange1D ir = *inner_range;
        double *r = rho->data, *u = umat->data, *v = vmat->data, *p = pmat->data, *c = cmat->data, *g = gmat->data,
               *E = Emat->data;
        launch_range(range, [=] __device__(int64_t k) {
            // src/kernels/halo_exchange.cpp:17-34
            int64_t i = scale1d(ir, (uint64_t)k);
            int64_t ip = i + disp;
            for (int64_t w = 0; w < stencil_width; w++) {
                r[i] = r[ip];
                u[i] = u[ip] * u_factor;
                v[i] = v[ip] * v_factor;
                p[i] = p[ip];
                c[i] = c[ip];
                g[i] = g[ip];
                E[i] = E[ip];
                i -= disp;
                ip += disp;
            }
        });
    });
}

void read_border_array(const Range* range, const InnerRange2D* inner_range, Idx side_length, Idx nghost,
                       const view* rho, const view* umat, const view* vmat, const view* pmat, const view* cmat,
                       const view* gmat, const view* Emat, view* value_array)
{
    guarded("read_border_array", [&] {
        CHECK_LABEL(rho); CHECK_LABEL(umat); CHECK_LABEL(vmat); CHECK_LABEL(pmat);
        CHECK_LABEL(cmat); CHECK_LABEL(gmat); CHECK_LABEL(Emat);
        const InnerRange2D ir = *inner_range;
        const double *r = rho->data, *u = umat->data, *v = vmat->data, *p = pmat->data, *c = cmat->data,
                     *g = gmat->data, *E = Emat->data;
        double* va = value_array->data;
        launch_range(range, [=] __device__(int64_t k) {
            // src/kernels/halo_exchange.cpp:47-63
            int64_t idx = scale2d(ir, (uint64_t)k);
            int64_t itr = k;
            int64_t i = itr / nghost;
            int64_t i_g = itr % nghost;
            int64_t i_arr = (i_g * side_length + i) * 7;
            va[i_arr + 0] = r[idx];
            va[i_arr + 1] = u[idx];
            va[i_arr + 2] = v[idx];
            va[i_arr + 3] = p[idx];
            va[i_arr + 4] = c[idx];
            va[i_arr + 5] = g[idx];
            va[i_arr + 6] = E[idx];
        });
    });
}

void write_border_array(const Range* range, const InnerRange2D* inner_range, Idx side_length, Idx nghost, view* rho,
                        view* umat, view* vmat, view* pmat, view* cmat, view* gmat, view* Emat,
                        const view* value_array)
{
    guarded("write_border_array", [&] {
        CHECK_LABEL(rho); CHECK_LABEL(umat); CHECK_LABEL(vmat); CHECK_LABEL(pmat);
        CHECK_LABEL(cmat); CHECK_LABEL(gmat); CHECK_LABEL(Emat);
        const InnerRange2D ir = *inner_range;
        double *r = rho->data, *u = umat->data, *v = vmat->data, *p = pmat->data, *c = cmat->data, *g = gmat->data,
               *E = Emat->data;
        const double* va = value_array->data;
        launch_range(range, [=] __device__(int64_t k) {
            // src/kernels/halo_exchange.cpp:75-91
            int64_t idx = scale2d(ir, (uint64_t)k);
            int64_t itr = k;
            int64_t i = itr / nghost;
            int64_t i_g = itr % nghost;
            int64_t i_arr = (i_g * side_length + i) * 7;
            r[idx] = va[i_arr + 0];
            u[idx] = va[i_arr + 1];
            v[idx] = va[i_arr + 2];
            p[idx] = va[i_arr + 3];
            c[idx] = va[i_arr + 4];
            g[idx] = va[i_arr + 5];
            E[idx] = va[i_arr + 6];
        });
    });
}

void init_test(const Range* range, const InnerRange2D* inner_range, Idx row_length, Idx nb_ghosts, Idx nx, Idx ny,
               flt_t sx, flt_t sy, flt_t ox, flt_t oy, Idx pos_x, Idx pos_y, Idx g_nx, Idx g_ny, view* x, view* y,
               view* rho, view* Emat, view* umat, view* vmat, mask_view* domain_mask, view* pmat, view* cmat,
               view* gmat, view* ustar, view* pstar, Test test, bool debug_indexes, flt_t test_option)
{
    guarded("init_test", [&] {
        const int test_i = static_cast<int>(test);
        if (test_i < 0 || test_i > 4)
            throw std::out_of_range("Invalid test case index: " + std::to_string(test_i) +
                                    ", expected a value between 0 and 4");
        CHECK_LABEL(x); CHECK_LABEL(y); CHECK_LABEL(rho); CHECK_LABEL(Emat); CHECK_LABEL(umat); CHECK_LABEL(vmat);
        CHECK_LABEL(domain_mask); CHECK_LABEL(pmat); CHECK_LABEL(cmat); CHECK_LABEL(gmat); CHECK_LABEL(ustar);
        CHECK_LABEL(pstar);
        armon::InitArgs a{};
        a.row_length = row_length; a.nb_ghosts = nb_ghosts; a.nx = nx; a.ny = ny;
        a.pos_x = pos_x; a.pos_y = pos_y; a.g_nx = g_nx; a.g_ny = g_ny;
        a.sx = sx; a.sy = sy; a.ox = ox; a.oy = oy;
        a.test_option = test_option;
        a.test = test_i;
        a.debug_indexes = debug_indexes ? 1 : 0;
        a.tp = armon::make_test_params(test_i, test_option);
        const InnerRange2D ir = *inner_range;
        double *px = x->data, *py = y->data, *r = rho->data, *E = Emat->data, *u = umat->data, *v = vmat->data,
               *m = domain_mask->data, *p = pmat->data, *c = cmat->data, *g = gmat->data, *us = ustar->data,
               *ps = pstar->data;
        launch_range(range, [=] __device__(int64_t k) {
            int64_t i = scale2d(ir, (uint64_t)k);
            armon::init_cell<double>(a, i, px, py, r, E, u, v, m, p, c, g, us, ps);
        });
    });
}

flt_t dt_CFL(const Range* range, const InnerRange1D* inner_range, flt_t dx, flt_t dy, const view* umat,
             const view* vmat, const view* cmat, const mask_view* domain_mask)
{
    double result = DBL_MAX;
    guarded("dt_CFL", [&] {
        CHECK_LABEL(umat); CHECK_LABEL(vmat); CHECK_LABEL(cmat); CHECK_LABEL(domain_mask);
        double* buf = scratch(kReduceBlocks + 1);
        int64_t n = range->end - range->start;
        if (n <= 0) { result = DBL_MAX; return; }
        dt_partial_kernel<<<kReduceBlocks, 256, 0, g_stream>>>(range->start, range->end, *inner_range, dx, dy, umat->data,
                                                               vmat->data, cmat->data, domain_mask->data, buf);
        min_final_kernel<<<1, 32, 0, g_stream>>>(buf, kReduceBlocks, buf + kReduceBlocks);
        check_cuda(cudaGetLastError(), "dt_CFL launch");
        check_cuda(cudaMemcpyAsync(&result, buf + kReduceBlocks, sizeof(double), cudaMemcpyDeviceToHost, g_stream),
                   "dt_CFL copy");
        check_cuda(cudaStreamSynchronize(g_stream), "dt_CFL sync");
    });
    return result;
}

flt_t dt_CFL_no_alloc(const Range* range, const InnerRange1D* inner_range, flt_t dx, flt_t dy, const view* umat,
                      const view* vmat, const view* cmat, const mask_view* domain_mask)
{
    // dt_CFL for callers that may not allocate device memory: the per-tile partial minima go to
    // g_dt_no_alloc_scratch instead of a cudaMalloc'd buffer.  Nothing here allocates.
    double result = DBL_MAX;
    guarded("dt_CFL_no_alloc", [&] {
        CHECK_LABEL(umat); CHECK_LABEL(vmat); CHECK_LABEL(cmat); CHECK_LABEL(domain_mask);
        int64_t n = range->end - range->start;
        if (n <= 0) { result = DBL_MAX; return; }
        int64_t tiles = (n + kNoAllocTile - 1) / kNoAllocTile;
        if (tiles > kNoAllocMaxTiles)
            throw std::out_of_range("range of " + std::to_string(n) + " indices exceeds the static scratch limit of " +
                                    std::to_string((int64_t)kNoAllocMaxTiles * kNoAllocTile) +
                                    " indices; use dt_CFL");
        double* scratch_dev = no_alloc_scratch_address();
        dt_tile_kernel<<<(int)tiles, 256, 0, g_stream>>>(range->start, range->end, *inner_range, dx, dy, umat->data,
                                                         vmat->data, cmat->data, domain_mask->data, scratch_dev);
        min_tiles_kernel<<<1, 1024, 0, g_stream>>>(scratch_dev, (int)tiles, scratch_dev + kNoAllocMaxTiles);
        check_cuda(cudaGetLastError(), "dt_CFL_no_alloc launch");
        check_cuda(cudaMemcpyAsync(&result, scratch_dev + kNoAllocMaxTiles, sizeof(double), cudaMemcpyDeviceToHost,
                                   g_stream), "dt_CFL_no_alloc copy");
        check_cuda(cudaStreamSynchronize(g_stream), "dt_CFL_no_alloc sync");
    });
    return result;
}

void conservation_vars(const Range* range, const InnerRange1D* inner_range, flt_t dx, const view* rho,
                       const view* Emat, const mask_view* domain_mask, flt_t* total_mass, flt_t* total_energy)
{
    guarded("conservation_vars", [&] {
        CHECK_LABEL(rho); CHECK_LABEL(Emat); CHECK_LABEL(domain_mask);
        double* buf = scratch(2 * kReduceBlocks + 2);
        double ds = dx * dx;
        cons_partial_kernel<<<kReduceBlocks, 256, 0, g_stream>>>(range->start, range->end, *inner_range, ds, rho->data,
                                                                 Emat->data, domain_mask->data, buf);
        sum2_final_kernel<<<1, 32, 0, g_stream>>>(buf, kReduceBlocks, buf + 2 * kReduceBlocks);
        check_cuda(cudaGetLastError(), "conservation_vars launch");
        double out[2];
        check_cuda(cudaMemcpyAsync(out, buf + 2 * kReduceBlocks, sizeof(out), cudaMemcpyDeviceToHost, g_stream),
                   "conservation_vars copy");
        check_cuda(cudaStreamSynchronize(g_stream), "conservation_vars sync");
        *total_mass = out[0];
        *total_energy = out[1];
    });
}

}  // extern "C"
