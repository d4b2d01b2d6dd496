// selftest.cu -- checks of the integer-pipe FP64 operations (softfp.cuh) against the FP64
// instructions, on generated operands.  Exposed as armon_selftest_softfp for the test suite.
#include <cstdint>
#include <cstring>

#include <cuda_runtime.h>

#include "softfp.cuh"

namespace {

__host__ __device__ __forceinline__ uint64_t mix(uint64_t x)
{
    // splitmix64 finaliser
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

__device__ __forceinline__ double normal_double(uint64_t r, int exp_span)
{
    // random sign and significand, exponent uniform in [1023 - span, 1023 + span]
    uint64_t e = 1023 - exp_span + (uint64_t)((r >> 53) % (uint64_t)(2 * exp_span + 1));
    return armon::sfp::from_bits((r & 0x8000000000000000ull) | (e << 52) | (r & armon::sfp::kMant));
}

__device__ void operands(int mode, uint64_t seed, uint64_t i, double& a, double& b)
{
    using namespace armon::sfp;
    uint64_t r1 = mix(seed ^ (2 * i)), r2 = mix(seed ^ (2 * i + 1)), r3 = mix(r1 ^ r2);
    switch (mode) {
    case 0:   // random normal operands
        a = normal_double(r1, 40);
        b = normal_double(r2, 40);
        break;
    case 1:   // random bit patterns: zeros, subnormals, infinities, NaN
        a = from_bits(r1);
        b = from_bits(r2);
        if ((r3 & 7) == 0) a = from_bits(r1 & 0x800FFFFFFFFFFFFFull);   // subnormal or zero
        if ((r3 & 7) == 1) b = from_bits(r2 & 0x800FFFFFFFFFFFFFull);
        if ((r3 & 15) == 2) a = from_bits((r1 & 0x8000000000000000ull) | 0x7FF0000000000000ull);
        break;
    case 2: {  // quotients near the midpoint between two doubles
        b = normal_double(r2, 20);
        double q = normal_double(r1, 20);
        uint64_t uq = bits(q);
        double half_ulp = from_bits((uq & 0x7FF0000000000000ull) - (53ull << 52));   // 2^(e_q - 53)
        a = fma(b, q, b * half_ulp * ((r3 & 1) ? 1.0 : -1.0));
        break;
    }
    case 3: {  // exact quotients: short significands
        uint64_t qm = (r1 >> 38) | 1, bm = (r2 >> 38) | 1;    // 26-bit odd integers
        double q = (double)qm * ((r3 & 1) ? 1.0 : -1.0), bb = (double)bm;
        b = ldexp(bb, (int)(r3 >> 8) % 64 - 32);
        a = q * b;
        break;
    }
    case 4:   // power-of-two divisors
        a = normal_double(r1, 60);
        b = from_bits((r2 & 0x8000000000000000ull) | ((uint64_t)(1023 - 60 + (r2 >> 53) % 121) << 52));
        break;
    case 5:   // zero dividends and large exponent differences
        a = (r3 & 1) ? normal_double(r1, 1000) : from_bits(r1 & 0x8000000000000000ull);
        b = normal_double(r2, 1000);
        break;
    default:  // the operand ranges of the solver: O(1e-6 .. 1e3), both signs
        a = normal_double(r1, 10) * 1e-3;
        b = normal_double(r2, 10);
        break;
    }
}

__global__ void div_check(int mode, uint64_t seed, int64_t n, unsigned long long* out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double a, b;
        operands(mode, seed, (uint64_t)i, a, b);
        double s = armon::sfp::div(a, b);
        double h = a / b;
        bool same = armon::sfp::bits(s) == armon::sfp::bits(h) || (s != s && h != h);
        if (!same) {
            if (atomicAdd(&out[0], 1ull) == 0) {
                out[2] = armon::sfp::bits(a);
                out[3] = armon::sfp::bits(b);
            }
        }
        // operands the fast path takes (normal or zero dividend, normal divisor, quotient in range)
        uint64_t ua = armon::sfp::bits(a), ub = armon::sfp::bits(b);
        uint32_t ea = (uint32_t)(ua >> 52) & 0x7FF, eb = (uint32_t)(ub >> 52) & 0x7FF;
        int e0 = (int)ea - (int)eb;
        bool fast = (eb - 1u) < 2046u && ((ua << 1) == 0 || ((ea - 1u) < 2046u && e0 >= -1021 && e0 <= 1022));
        if (fast) atomicAdd(&out[1], 1ull);
    }
}

__global__ void cmp_check(uint64_t seed, int64_t n, unsigned long long* out)
{
    using namespace armon::sfp;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t r1 = mix(seed ^ (2 * i)), r2 = mix(seed ^ (2 * i + 1)), r3 = mix(r1 ^ r2);
        double x = from_bits(r1), y = (r3 & 3) == 0 ? from_bits(r1 ^ (r3 & 0x8000000000000000ull)) : from_bits(r2);
        if ((r3 & 12) == 4) y = from_bits(r1 + (r3 >> 60) - 8);     // neighbours
        if ((r3 & 48) == 16) x = from_bits(r3 & 0x8000000000000000ull);   // +-0
        if ((r3 & 192) == 64) x = from_bits(0x3FF0000000000000ull + (r3 >> 61) - 4);   // around 1
        // neg_if is the multiply by -1 for non-NaN x (a NaN's sign and payload are not portable)
        bool ok = lt(x, y) == (x < y) && gt0(x) == (x > 0.0) &&
                  (x != x || bits(neg_if(x, (r3 >> 7) & 1)) == bits((r3 >> 7) & 1 ? -x : x)) &&
                  lt_pos(x, 0x3FF0000000000000ull) == (x < 1.0) && lt_pos(x, 0x4000000000000000ull) == (x < 2.0) &&
                  lt_pos(y, 0x3FF0000000000000ull) == (y < 1.0);
        if (!ok && atomicAdd(&out[0], 1ull) == 0) {
            out[2] = bits(x);
            out[3] = bits(y);
        }
    }
}

__global__ void scale_check(uint64_t seed, int64_t n, unsigned long long* out)
{
    using namespace armon::sfp;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t r1 = mix(seed ^ (2 * i)), r2 = mix(seed ^ (2 * i + 1));
        double x = from_bits(r1);                                   // every class of operand
        if ((r2 & 3) == 0) x = normal_double(r1, 1023);             // normal, all exponents
        if ((r2 & 12) == 4) x = from_bits(r1 & 0x801FFFFFFFFFFFFFull);   // near the subnormal range
        if ((r2 & 48) == 16) x = from_bits(r1 | 0x7FE0000000000000ull);  // near overflow
        if ((r2 & 192) == 64) x = from_bits(r1 & 0x8000000000000000ull); // +-0
        const int k = (int)((r2 >> 8) % 121) - 60;
        const double p2 = ldexp(1.0, k);
        const double s = scale(x, k, p2), h = x * p2;
        bool ok = bits(s) == bits(h) || (s != s && h != h);
        ok = ok && (bits(half(x)) == bits(x * 0.5) || x != x) && (bits(twice(x)) == bits(x * 2.0) || x != x);
        if (!ok && atomicAdd(&out[0], 1ull) == 0) {
            out[2] = bits(x);
            out[3] = (uint64_t)(int64_t)k;
        }
    }
}

__global__ void sqrt_check(uint64_t seed, int64_t n, unsigned long long* out)
{
    using namespace armon::sfp;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t r1 = mix(seed ^ (2 * i)), r2 = mix(seed ^ (2 * i + 1));
        double x;
        switch (r2 & 7) {
        case 0: x = from_bits(r1); break;                                  // every class
        case 1: {                                                          // exact squares
            double q = (double)((r1 >> 38) | 1) * ldexp(1.0, (int)(r2 >> 8) % 200 - 100);
            x = q * q;
            break;
        }
        case 2: case 3: {                                                  // root near a midpoint
            double q = normal_double(r1, 500);
            q = fabs(q);
            double h = q + from_bits((bits(q) & 0x7FF0000000000000ull) - (53ull << 52));   // q + ulp/2
            x = h * h;
            if (r2 & 8) x = from_bits(bits(x) + ((r2 >> 4) & 3) - 1);
            break;
        }
        default: x = fabs(normal_double(r1, 1022)); break;                 // positive normals
        }
        const double s = armon::sfp::sqrt(x), h = ::sqrt(x);
        const bool ok = bits(s) == bits(h) || (s != s && h != h);
        const bool abs_ok = x != x || bits(absval(x)) == bits(fabs(x));
        if (!(ok && abs_ok) && atomicAdd(&out[0], 1ull) == 0) {
            out[2] = bits(x);
            out[3] = bits(s);
        }
        // operands of the integer path: positive normals
        if ((uint32_t)(bits(x) >> 52) - 1u < 2046u) atomicAdd(&out[1], 1ull);
    }
}

__global__ void mul_check(uint64_t seed, int64_t n, unsigned long long* out)
{
    using namespace armon::sfp;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t r1 = mix(seed ^ (2 * i)), r2 = mix(seed ^ (2 * i + 1)), r3 = mix(r1 ^ r2);
        double a, b;
        switch (r3 & 7) {
        case 0: a = from_bits(r1); b = from_bits(r2); break;                       // every class
        case 1: {                                                                  // exact ties
            const double qa = (double)((r1 >> 37) | 1), qb = (double)((r2 >> 37) | 1);   // 27-bit odd
            a = ldexp(qa, (int)((r3 >> 8) % 200) - 100) * ((r3 & 8) ? -1.0 : 1.0);
            b = ldexp(qb, (int)((r3 >> 16) % 200) - 100);
            break;
        }
        case 2: a = normal_double(r1, 1023); b = normal_double(r2, 1023); break;   // overflow, underflow
        case 3: a = normal_double(r1, 1023); b = from_bits(r2 & 0x800FFFFFFFFFFFFFull); break;   // subnormal, 0
        default: a = normal_double(r1, 300); b = normal_double(r2, 300); break;    // normal products
        }
        const double s = mul(a, b), h = a * b;
        if (!(bits(s) == bits(h) || (s != s && h != h)) && atomicAdd(&out[0], 1ull) == 0) {
            out[2] = bits(a);
            out[3] = bits(b);
        }
        // operands of the integer path: both normal
        if ((uint32_t)((bits(a) >> 52) & 0x7FF) - 1u < 2046u && (uint32_t)((bits(b) >> 52) & 0x7FF) - 1u < 2046u)
            atomicAdd(&out[1], 1ull);
    }
}

// The division's quotient estimate against exact 128-bit arithmetic: the remainder
// ma 2^52 - q mb must lie in [0, 2 mb) (one correction step then gives the quotient).
__global__ void quot_check(uint64_t seed, int64_t n, unsigned long long* out)
{
    using namespace armon::sfp;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t r1 = mix(seed ^ (2 * i)), r2 = mix(seed ^ (2 * i + 1)), r3 = mix(r1 ^ r2);
        uint64_t mb = (r2 & kMant) | kHidden;
        if ((r3 & 15) == 0) mb = kHidden + 1;                       // just above a power of two
        if ((r3 & 15) == 1) mb = (kHidden << 1) - 1;                // just below the next
        if (mb == kHidden) mb += 1;
        uint64_t ma = (r1 & kMant) | kHidden;
        if ((r3 >> 4) & 1) ma <<= 1;                                // the doubled dividend
        if ((r3 & 0xE0) == 0x20) ma = (r3 >> 8) & 1 ? (kHidden << 2) - 1 : kHidden;
        const uint64_t q = quot_estimate(ma, recip_v(mb));
        const unsigned __int128 num = (unsigned __int128)ma << 52;
        const unsigned __int128 qm = (unsigned __int128)q * mb;
        const bool ok = qm <= num && num - qm < 2 * (unsigned __int128)mb;
        if (!ok && atomicAdd(&out[0], 1ull) == 0) {
            out[2] = ma;
            out[3] = mb;
        }
    }
}


// Operands for the addition check: every bit class, cancellations (|a| close to |b|, opposite
// signs), exact ties (y's dropped part exactly half a unit), large exponent differences, overflow
// and underflow ranges, zeros, and the solver's ranges.
__host__ __device__ void add_operands(uint64_t seed, uint64_t i, uint64_t& ua, uint64_t& ub)
{
    using namespace armon::sfp;
    const uint64_t r1 = mix(seed ^ (2 * i)), r2 = mix(seed ^ (2 * i + 1)), r3 = mix(r1 ^ r2);
    const auto normal = [](uint64_t r, uint32_t lo, uint32_t span) {
        return (r & ~kAbs) | ((uint64_t)(lo + (uint32_t)((r >> 53) % span)) << 52) | (r & kMant);
    };
    switch (r3 & 7) {
    case 0: ua = r1; ub = r2; break;                                              // every class
    case 1: {                                                                      // cancellation
        ua = normal(r1, 1000, 48);
        const uint64_t delta = (r2 >> ((r3 >> 8) % 64)) & 0xFFFFFull;
        ub = (((ua & kAbs) + ((r3 & 16) ? delta : (uint64_t)0 - delta)) & kAbs) | (~ua & ~kAbs);
        break;
    }
    case 2: {                                                                      // ties and near ties
        ua = normal(r1, 900, 200);
        const uint32_t d = 1 + (uint32_t)((r3 >> 8) % 60);
        const uint64_t ea = (ua >> 52) & 0x7FF;
        const uint64_t m = (r2 & kMant & ~((1ull << (d < 52 ? d : 52)) - 1)) | ((r3 >> 20) & 1 ? (1ull << (d - 1 < 52 ? d - 1 : 51)) : 0);
        ub = (r2 & ~kAbs) | ((ea > d ? ea - d : 1) << 52) | (m & kMant);
        break;
    }
    case 3: ua = normal(r1, 1, 2046); ub = normal(r2, 1, 2046); break;            // every exponent
    case 4: ua = normal(r1, 2000, 46); ub = normal(r2, 2000, 46); break;          // overflow
    case 5: ua = normal(r1, 1, 60); ub = normal(r2, 1, 60); break;                // underflow
    case 6: ua = normal(r1, 1000, 48); ub = (r3 & 32) ? (r2 & ~kAbs) : normal(r2, 1000, 48); break;   // zeros
    default: ua = normal(r1, 1003, 40); ub = normal(r2, 1003, 40); break;         // the solver's ranges
    }
}

__global__ void add_check(uint64_t seed, int64_t n, unsigned long long* out)
{
    using namespace armon::sfp;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t ua, ub;
        add_operands(seed, (uint64_t)i, ua, ub);
        const double a = from_bits(ua), b = from_bits(ub);
        const double s = add(a, b), h = a + b;
        if (!(bits(s) == bits(h) || (s != s && h != h)) && atomicAdd(&out[0], 1ull) == 0) {
            out[2] = ua;
            out[3] = ub;
        }
        bool ok;
        add_bits(ua, ub, ok);
        if (ok) atomicAdd(&out[1], 1ull);
    }
}

}  // namespace

extern "C" {

// add_bits on the host against the host's IEEE addition, on the operands of add_check:
// out[0] = mismatches, out[1] = operand pairs on the integer path, out[2..3] = the first mismatch.
int armon_selftest_add_host(uint64_t seed, int64_t n, uint64_t* out)
{
    out[0] = out[1] = out[2] = out[3] = 0;
    for (int64_t i = 0; i < n; i++) {
        uint64_t ua, ub;
        add_operands(seed, (uint64_t)i, ua, ub);
        bool ok;
        const uint64_t r = armon::sfp::add_bits(ua, ub, ok);
        if (!ok) continue;
        out[1]++;
        double a, b, h;
        std::memcpy(&a, &ua, 8);
        std::memcpy(&b, &ub, 8);
        h = a + b;
        uint64_t uh;
        std::memcpy(&uh, &h, 8);
        if (uh != r && out[0]++ == 0) {
            out[2] = ua;
            out[3] = ub;
        }
    }
    return 0;
}

// mode 0..6 (see operands) checks sfp::div against the hardware quotient; mode 100 checks lt,
// gt0 and neg_if against the IEEE comparisons; mode 101 checks scale, half and twice against the
// FP64 multiply by the power of two (out[3] = the exponent k of the first mismatch); mode 102
// checks sqrt and absval against the hardware square root and fabs (out[3] = the soft root);
// mode 103 checks mul against the FP64 multiply; mode 105 checks add against the FP64 addition;
// mode 104 checks the division's quotient
// estimate against 128-bit arithmetic (out[2..3] = ma, mb of the first miss).  out[0] = mismatches, out[1] = fast-path operand
// pairs, out[2..3] = the bits of the first mismatching operands.  Returns a cudaError_t.
int armon_selftest_softfp(uint64_t seed, int64_t n, int32_t mode, uint64_t* out_host)
{
    unsigned long long* out = nullptr;
    cudaError_t e = cudaMalloc(&out, 4 * sizeof(unsigned long long));
    if (e != cudaSuccess) return (int)e;
    cudaMemset(out, 0, 4 * sizeof(unsigned long long));
    if (mode == 100) cmp_check<<<152 * 16, 256>>>(seed, n, out);
    else if (mode == 101) scale_check<<<152 * 16, 256>>>(seed, n, out);
    else if (mode == 102) sqrt_check<<<152 * 16, 256>>>(seed, n, out);
    else if (mode == 103) mul_check<<<152 * 16, 256>>>(seed, n, out);
    else if (mode == 104) quot_check<<<152 * 16, 256>>>(seed, n, out);
    else if (mode == 105) add_check<<<152 * 16, 256>>>(seed, n, out);
    else div_check<<<152 * 16, 256>>>(mode, seed, n, out);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(out_host, out, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
    cudaFree(out);
    return (int)e;
}

}  // extern "C"
